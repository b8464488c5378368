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
