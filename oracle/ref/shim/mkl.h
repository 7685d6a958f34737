// Stand-in for <mkl.h>: the CBLAS subset plus the two service calls Puck makes.
#pragma once
#include "mkl_cblas.h"
#include "mkl_service.h"
