// sw_run_device_noalloc: the swept run on a device-resident state for callers
// that cannot allocate device memory.  Its scratch -- the half-tile edge
// slots of the swept kernel and the work row of the classic remainder steps --
// lives in one file-scope device array of SW_NOALLOC_SCRATCH_BYTES, so the
// call itself allocates nothing (no cudaMalloc / cudaFree, no context, no
// events, no allocating library routine).
#include <cuda_runtime.h>

#include <mutex>

#include "ctx.h"
#include "sw_internal.h"

using namespace sw;

// Shared by every call on a device and held by every device that loads the
// library until the process exits.  Nothing in it has to start at zero: each
// run writes every slot before reading it.
static __device__ __align__(256) unsigned char sw_noalloc_scratch[SW_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_lock;
void *g_scratch[kMaxDevices] = {};

// Device address of the scratch array on the current device.  In host code
// the array's name is only a host-side stand-in, so the address is asked from
// the runtime.  It is asked again on every call made outside stream capture
// (a cheap lookup once the module is loaded), so a context that the host
// application destroyed and re-created (cudaDeviceReset) is never left with
// a stale address; inside a capture the address of the last call outside one
// is used, which is why the first call on a device must come before any
// capture.
cudaError_t scratch_address(cudaStream_t s, void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(s, &cap);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(g_setup_lock);
    if (cap == cudaStreamCaptureStatusNone || !g_scratch[dev]) {
        if (cap != cudaStreamCaptureStatusNone) return cudaErrorStreamCaptureUnsupported;
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, sw_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch[dev] = p;
    }
    *out = g_scratch[dev];
    return cudaSuccess;
}

// The state must be device memory of the current device: the scratch array
// used is the current device's, and a kernel must not read another GPU's
// memory through it.
bool on_current_device(const void *state) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, state) != cudaSuccess) {
        cudaGetLastError();  // an unregistered host pointer may leave an error behind
        return false;
    }
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

// Scratch bytes a run needs: the slots (two cells per cell) and one work row.
size_t scratch_need(const Ops *ops, int64_t nx) { return ops->cell * (size_t)nx * 3; }

template <typename T>
int run(const sw_config &c, void *state, cudaStream_t s) {
    const Ops *ops = ops_for(c.problem, c.precision, c.flags);
    const int W = c.tpb;
    const int64_t nx = c.nx;
    const size_t slot_bytes = ops->cell * (size_t)nx * 2;
    void *scratch = nullptr;
    if (scratch_address(s, &scratch) != cudaSuccess) return SW_ERR_CUDA;
    void *slots = scratch;
    void *work = static_cast<char *>(scratch) + slot_bytes;

    sw_constants k;
    sw_constants_of(&c, &k);
    const Params<T> p = make_params<T>(c, k);
    const int64_t q = W / (2 * ops->R * ops->S);
    const int64_t full = c.n_steps / q, rem = c.n_steps - full * q;
    if (full >= 1) {
        if (ops->swept(&p, MODE_UP, 0, state, slots, nx, W, c.threads, s) != cudaSuccess) return SW_ERR_CUDA;
        for (int64_t d = 1; d < full; ++d)
            if (ops->swept(&p, MODE_DIAMOND, (int)(d & 1), state, slots, nx, W, c.threads, s) != cudaSuccess) return SW_ERR_CUDA;
        if (ops->swept(&p, MODE_DOWN, (int)(full & 1), state, slots, nx, W, c.threads, s) != cudaSuccess) return SW_ERR_CUDA;
    }
    void *cur = state, *alt = work;
    for (int64_t i = 0; i < rem; ++i) {
        if (ops->classic(&p, cur, alt, 0, nx, W, s) != cudaSuccess) return SW_ERR_CUDA;
        if (ops->S == 1) {
            void *t = cur;
            cur = alt;
            alt = t;
        } else if (ops->classic(&p, alt, cur, 1, nx, W, s) != cudaSuccess) {
            return SW_ERR_CUDA;
        }
    }
    if (cur != state && cudaMemcpyAsync(state, cur, ops->cell * (size_t)nx, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return SW_ERR_CUDA;
    return SW_OK;
}

}  // namespace

extern "C" int sw_run_device_noalloc(const sw_config *cfg, void *state_dev, void *stream) {
    if (!cfg || !state_dev) return SW_ERR_ARG;
    int rc = sw_validate(cfg);
    if (rc) return rc;
    if (cfg->alg != SW_ALG_SWEPT || cfg->time_mode != SW_TIME_STEPS || (cfg->flags & SW_FLAG_HOST_TILE))
        return SW_ERR_UNSUPPORTED;
    if (scratch_need(ops_for(cfg->problem, cfg->precision, cfg->flags), cfg->nx) > (size_t)SW_NOALLOC_SCRATCH_BYTES)
        return SW_ERR_SIZE;
    if (!on_current_device(state_dev)) return SW_ERR_ARG;
    if (cfg->precision == 4) return run<float>(*cfg, state_dev, (cudaStream_t)stream);
    return run<double>(*cfg, state_dev, (cudaStream_t)stream);
}
