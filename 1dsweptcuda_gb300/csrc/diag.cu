// sw_wait_probe: the persistent kernels' bounded wait, run on a flag that
// nothing sets, so that the timeout path (status word -> SW_ERR_TIMEOUT) is
// exercised without starving a real run.  The wait is the production
// wait_slots with a caller-chosen limit.
#include <cuda_runtime.h>

#include "ctx.h"
#include "persistent.cuh"

namespace sw {
namespace {
__global__ void k_wait_probe(const unsigned *flags, int *status, uint64_t limit_ns) {
    wait_slots(flags, 0, 1, 1u, status, limit_ns);  // flags stay 0: the wait must run out
}
}  // namespace
}  // namespace sw

using namespace sw;

extern "C" int sw_wait_probe(sw_ctx *ctx, int64_t limit_ns, double *waited_ms) {
    if (!ctx || limit_ns < 1000000 || limit_ns > 10000000000LL) return SW_ERR_ARG;
    SW_CUDA(ctx, cudaSetDevice(ctx->device));
    SW_CUDA(ctx, grow_dev((void **)&ctx->d_flags, &ctx->n_flags, 2 * sizeof(unsigned)));
    if (!ctx->d_status) SW_CUDA(ctx, cudaMalloc(&ctx->d_status, sizeof(int)));
    cudaStream_t s = ctx->stream;
    SW_CUDA(ctx, cudaMemsetAsync(ctx->d_flags, 0, 2 * sizeof(unsigned), s));
    SW_CUDA(ctx, cudaMemsetAsync(ctx->d_status, 0, sizeof(int), s));
    SW_CUDA(ctx, cudaEventRecord(ctx->k0, s));
    k_wait_probe<<<1, 32, 0, s>>>(ctx->d_flags, ctx->d_status, (uint64_t)limit_ns);
    SW_CUDA(ctx, cudaGetLastError());
    SW_CUDA(ctx, cudaEventRecord(ctx->k1, s));
    SW_CUDA(ctx, cudaEventSynchronize(ctx->k1));
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->k0, ctx->k1);
    if (waited_ms) *waited_ms = ms;
    int status = 0;
    SW_CUDA(ctx, cudaMemcpy(&status, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    return status ? fail(ctx, SW_ERR_TIMEOUT, "bounded wait ran out (as the probe intends)") : SW_OK;
}

// sw_fp64_rates: the FP64 pipe's issue rates on this GPU, measured.  Every
// thread of a full grid (eight 256-thread blocks per SM) runs eight
// independent chains of one operation -- fma(a, x, y), a + y or a * x with x, y
// passed at run time -- so the pipe, not a dependence, sets the pace.  The
// stencils' FP64 roofs are built from these three rates and their operation
// counts.
namespace sw {
namespace {
constexpr int kProbeChains = 8;

template <int OP>
__global__ void __launch_bounds__(256) k_fp64_rate(double *sink, double x, double y, int iters) {
    double a[kProbeChains];
#pragma unroll
    for (int i = 0; i < kProbeChains; ++i) a[i] = 1.0 + (double)(threadIdx.x * kProbeChains + i) * 1e-9;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < kProbeChains; ++i) {
            if (OP == 0) a[i] = __fma_rn(a[i], x, y);
            else if (OP == 1) a[i] = __dadd_rn(a[i], y);
            else a[i] = __dmul_rn(a[i], x);
        }
    }
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < kProbeChains; ++i) s = __dadd_rn(s, a[i]);
    if (s == -1.0) sink[blockIdx.x] = s;  // never true: keeps the chains live
}
}  // namespace
}  // namespace sw

extern "C" int sw_fp64_rates(sw_ctx *ctx, double *fma_per_s, double *add_per_s, double *mul_per_s) {
    if (!ctx || !fma_per_s || !add_per_s || !mul_per_s) return SW_ERR_ARG;
    SW_CUDA(ctx, cudaSetDevice(ctx->device));
    int sms = 0;
    SW_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    const int blocks = sms * 8, threads = 256, iters = 8192;
    SW_CUDA(ctx, grow_dev(&ctx->d_io, &ctx->n_io, sizeof(double) * (size_t)blocks));
    double *sink = static_cast<double *>(ctx->d_io);
    cudaStream_t s = ctx->stream;
    const double ops = (double)blocks * threads * kProbeChains * iters;
    double *outs[3] = {fma_per_s, add_per_s, mul_per_s};
    for (int op = 0; op < 3; ++op) {
        float best = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {  // the first run also loads the module
            SW_CUDA(ctx, cudaEventRecord(ctx->k0, s));
            if (op == 0) k_fp64_rate<0><<<blocks, threads, 0, s>>>(sink, 1.0 - 0x1p-30, 0x1p-30, iters);
            else if (op == 1) k_fp64_rate<1><<<blocks, threads, 0, s>>>(sink, 1.0, 0x1p-40, iters);
            else k_fp64_rate<2><<<blocks, threads, 0, s>>>(sink, 1.0 - 0x1p-40, 0.0, iters);
            SW_CUDA(ctx, cudaGetLastError());
            SW_CUDA(ctx, cudaEventRecord(ctx->k1, s));
            SW_CUDA(ctx, cudaEventSynchronize(ctx->k1));
            float ms = 0;
            SW_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->k0, ctx->k1));
            if (rep > 0 && ms < best) best = ms;
        }
        *outs[op] = ops / (best * 1e-3);
    }
    return SW_OK;
}
