// extern "C" entry points of the learned probe predictor (pgpu_probe_*).
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "pgpu_internal.h"

struct pgpu_probe {
    int device = 0;
    pgpu::ProbeNet net, grad, m, v;
    float* block = nullptr;  // 4 parameter-sized blocks: weights, gradients, Adam m, Adam v
    uint16_t* bf16 = nullptr;  // BF16 copies of W1, W2, W3
    pgpu::ProbeWork work;
    float* loss = nullptr;   // device scalar
    int* err = nullptr;      // device flag of the tensor-core waits
    uint64_t step = 0;
    cudaStream_t stream = nullptr;
    std::mutex mu;
};

namespace pgpu {
const ProbeNet* probe_net(const pgpu_probe* p) { return &p->net; }
int probe_device(const pgpu_probe* p) { return p->device; }
}  // namespace pgpu

namespace {

int cuda_fail(cudaError_t e, const char* what) {
    return pgpu::set_last_error(e == cudaErrorMemoryAllocation ? PGPU_E_NOMEM : PGPU_E_CUDA,
                                std::string(what) + ": " + cudaGetErrorString(e));
}

void free_work(pgpu::ProbeWork* w) {
    float* ptrs[] = {w->H1, w->Z1, w->H2, w->Z2, w->Z, w->dZ, w->dH2, w->dH1};
    for (float* p : ptrs)
        if (p) cudaFree(p);
    *w = pgpu::ProbeWork();
}

cudaError_t ensure_work(pgpu_probe* p, uint32_t n) {
    if (p->work.cap >= n) return cudaSuccess;
    free_work(&p->work);
    const uint64_t h = p->net.h, C = p->net.C;
    pgpu::ProbeWork& w = p->work;
    cudaError_t e = cudaSuccess;
    float** hs[] = {&w.H1, &w.Z1, &w.H2, &w.Z2, &w.dH2, &w.dH1};
    for (float** q : hs)
        if (e == cudaSuccess) e = cudaMalloc((void**)q, sizeof(float) * n * h);
    if (e == cudaSuccess) e = cudaMalloc((void**)&w.Z, sizeof(float) * n * C);
    if (e == cudaSuccess) e = cudaMalloc((void**)&w.dZ, sizeof(float) * n * C);
    if (e != cudaSuccess) {
        free_work(&w);
        return e;
    }
    w.cap = n;
    return cudaSuccess;
}

// One forward + backward pass on the probe's stream; the loss lands in p->loss.
int run_backward(pgpu_probe* p, const float* x, const uint32_t* labels, uint32_t n, uint32_t L) {
    cudaError_t e = ensure_work(p, n);
    if (e != cudaSuccess) return cuda_fail(e, "probe work buffers");
    cudaMemsetAsync(p->loss, 0, sizeof(float), p->stream);
    cudaMemsetAsync(p->err, 0, sizeof(int), p->stream);
    e = pgpu::probe_backward(p->net, x, n, labels, L, p->work, p->grad, p->loss, p->err, p->stream);
    if (e != cudaSuccess) return cuda_fail(e, "probe backward");
    return PGPU_OK;
}

int finish(pgpu_probe* p, float* loss) {
    float l = 0.0f;
    int flag = 0;
    cudaError_t e = cudaMemcpyAsync(&l, p->loss, sizeof(float), cudaMemcpyDeviceToHost, p->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&flag, p->err, sizeof(int), cudaMemcpyDeviceToHost, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) return cuda_fail(e, "probe step");
    if (flag) return pgpu::set_last_error(PGPU_E_TIMEOUT, "tensor-core wait expired");
    if (loss) *loss = l;
    return PGPU_OK;
}

}  // namespace

extern "C" {

int pgpu_probe_create(uint32_t dim, uint32_t hidden, uint32_t clusters, uint64_t seed,
                      int32_t device, pgpu_probe** out) {
    if (out == nullptr || dim == 0 || hidden == 0 || clusters == 0)
        return pgpu::set_last_error(PGPU_E_INVALID, "invalid argument");
    *out = nullptr;
    if (dim > pgpu::kMaxDim || hidden > 4096 || clusters > pgpu::kMaxClusters)
        return pgpu::set_last_error(PGPU_E_LIMIT, "probe size beyond the supported limits");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return pgpu::set_last_error(PGPU_E_CUDA, "no CUDA device available");
    if (device < 0 || device >= ndev)
        return pgpu::set_last_error(PGPU_E_INVALID, "device ordinal out of range");
    cudaSetDevice(device);
    auto* p = new pgpu_probe();
    p->device = device;
    for (pgpu::ProbeNet* n : {&p->net, &p->grad, &p->m, &p->v}) {
        n->d = dim;
        n->h = hidden;
        n->C = clusters;
    }
    const uint64_t np = p->net.param_count();
    cudaError_t e = cudaMalloc((void**)&p->block, sizeof(float) * np * 4);
    const uint64_t nw = (uint64_t)hidden * dim + (uint64_t)hidden * hidden + (uint64_t)clusters * hidden;
    if (e == cudaSuccess) e = cudaMalloc((void**)&p->bf16, sizeof(uint16_t) * nw);
    if (e == cudaSuccess) e = cudaMalloc((void**)&p->loss, sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&p->err, sizeof(int));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
        p->net.bind(p->block);
        p->grad.bind(p->block + np);
        p->m.bind(p->block + 2 * np);
        p->v.bind(p->block + 3 * np);
        p->net.W1b = p->bf16;
        p->net.W2b = p->net.W1b + (uint64_t)hidden * dim;
        p->net.W3b = p->net.W2b + (uint64_t)hidden * hidden;
        e = cudaMemsetAsync(p->block + np, 0, sizeof(float) * np * 3, p->stream);
    }
    if (e == cudaSuccess) e = pgpu::probe_init(p->net, seed, p->stream);
    if (e == cudaSuccess) e = pgpu::probe_sync_bf16(p->net, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) {
        int rc = cuda_fail(e, "probe create");
        if (p->block) cudaFree(p->block);
        if (p->bf16) cudaFree(p->bf16);
        if (p->loss) cudaFree(p->loss);
        if (p->err) cudaFree(p->err);
        if (p->stream) cudaStreamDestroy(p->stream);
        delete p;
        return rc;
    }
    *out = p;
    return PGPU_OK;
}

int pgpu_probe_destroy(pgpu_probe* p) {
    if (p == nullptr) return PGPU_OK;
    cudaSetDevice(p->device);
    cudaStreamSynchronize(p->stream);
    free_work(&p->work);
    cudaFree(p->block);
    cudaFree(p->bf16);
    cudaFree(p->loss);
    cudaFree(p->err);
    cudaStreamDestroy(p->stream);
    delete p;
    return PGPU_OK;
}

int pgpu_probe_info(const pgpu_probe* p, uint32_t* dim, uint32_t* hidden, uint32_t* clusters,
                    uint64_t* params) {
    if (p == nullptr) return pgpu::set_last_error(PGPU_E_INVALID, "null probe");
    if (dim) *dim = p->net.d;
    if (hidden) *hidden = p->net.h;
    if (clusters) *clusters = p->net.C;
    if (params) *params = p->net.param_count();
    return PGPU_OK;
}

int pgpu_probe_train_step(pgpu_probe* p, const float* queries, const uint32_t* labels, uint32_t n,
                          uint32_t L, float lr, float* loss) {
    if (p == nullptr || queries == nullptr || labels == nullptr || n == 0 || L == 0)
        return pgpu::set_last_error(PGPU_E_INVALID, "invalid argument");
    std::lock_guard<std::mutex> g(p->mu);
    cudaSetDevice(p->device);
    if (int rc = run_backward(p, queries, labels, n, L)) return rc;
    p->step += 1;
    cudaError_t e = pgpu::probe_adam(p->net, p->grad, p->m, p->v, lr, p->step, p->stream);
    if (e == cudaSuccess) e = pgpu::probe_sync_bf16(p->net, p->stream);
    if (e != cudaSuccess) return cuda_fail(e, "probe update");
    return finish(p, loss);
}

int pgpu_probe_gradients(pgpu_probe* p, const float* queries, const uint32_t* labels, uint32_t n,
                         uint32_t L, float* loss, float* grads) {
    if (p == nullptr || queries == nullptr || labels == nullptr || n == 0 || L == 0 ||
        grads == nullptr)
        return pgpu::set_last_error(PGPU_E_INVALID, "invalid argument");
    std::lock_guard<std::mutex> g(p->mu);
    cudaSetDevice(p->device);
    if (int rc = run_backward(p, queries, labels, n, L)) return rc;
    cudaError_t e = cudaMemcpyAsync(grads, p->grad.W1, sizeof(float) * p->net.param_count(),
                                    cudaMemcpyDeviceToHost, p->stream);
    if (e != cudaSuccess) return cuda_fail(e, "probe gradients");
    return finish(p, loss);
}

int pgpu_probe_forward(pgpu_probe* p, const float* queries, uint32_t n, float* scores) {
    if (p == nullptr || queries == nullptr || scores == nullptr)
        return pgpu::set_last_error(PGPU_E_INVALID, "invalid argument");
    if (n == 0) return PGPU_OK;
    std::lock_guard<std::mutex> g(p->mu);
    cudaSetDevice(p->device);
    cudaError_t e = ensure_work(p, n);
    if (e != cudaSuccess) return cuda_fail(e, "probe work buffers");
    cudaMemsetAsync(p->err, 0, sizeof(int), p->stream);
    // the search's own inference path: BF16 weights and activations
    e = pgpu::probe_infer(p->net, queries, nullptr, n, reinterpret_cast<uint16_t*>(p->work.H1),
                          reinterpret_cast<uint16_t*>(p->work.H2), scores, p->err, p->stream);
    if (e != cudaSuccess) return cuda_fail(e, "probe forward");
    return finish(p, nullptr);
}

int pgpu_probe_get_params(const pgpu_probe* p, float* params, uint64_t count) {
    if (p == nullptr || params == nullptr || count != p->net.param_count())
        return pgpu::set_last_error(PGPU_E_INVALID, "invalid argument");
    cudaSetDevice(p->device);
    cudaError_t e = cudaMemcpy(params, p->net.W1, sizeof(float) * count, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "probe params");
    return PGPU_OK;
}

int pgpu_probe_set_params(pgpu_probe* p, const float* params, uint64_t count) {
    if (p == nullptr || params == nullptr || count != p->net.param_count())
        return pgpu::set_last_error(PGPU_E_INVALID, "invalid argument");
    std::lock_guard<std::mutex> g(p->mu);
    cudaSetDevice(p->device);
    cudaStreamSynchronize(p->stream);
    cudaError_t e = cudaMemcpy(p->net.W1, params, sizeof(float) * count, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = pgpu::probe_sync_bf16(p->net, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) return cuda_fail(e, "probe params");
    return PGPU_OK;
}

}  // extern "C"
