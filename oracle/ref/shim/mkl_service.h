// Stand-in for <mkl_service.h>: the two service calls Puck makes are no-ops.
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
void mkl_set_dynamic(int flag);
int mkl_enable_instructions(int isa);
#ifdef __cplusplus
}
#endif
