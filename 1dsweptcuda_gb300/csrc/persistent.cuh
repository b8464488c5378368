// Persistent swept variant (alg 2): the up-triangle, every diamond and the
// down-triangle of one output segment in a single cooperative launch.
//
// Stages q = 0 (up-triangle, phase 0), q = 1..n_diamonds (diamond, phase q&1)
// and q = n_diamonds+1 (down-triangle).  Block b handles tiles b, b+grid, ...
// of every stage, stage by stage.  flags[h] counts the stages that have
// written half-tile slot h: a tile of stage q waits until both of its slots
// show q (stage q-1 wrote them), works, writes them back and publishes q+1.
// Only the one tile that owns a slot in a stage touches it, so the in-place
// slot scheme of the launch-per-pass kernels carries over unchanged.
//
// Waits are bounded: a block that spins past SW_WAIT_NS (or sees another block
// give up) records the failure in *status and returns; the host turns that
// into SW_ERR_TIMEOUT.  Co-residency of all blocks is guaranteed by the
// cooperative launch, so in a healthy run every wait ends.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "engine.cuh"

#ifndef SW_WAIT_NS
#define SW_WAIT_NS 4000000000ull  // 4 s per wait
#endif

namespace sw {

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Thread 0 waits for both slot flags to reach `need`; returns false (and sets
// *status) if the wait runs out or another block already failed.
__device__ __forceinline__ bool wait_slots(const unsigned *flags, int64_t hl, int64_t hr, unsigned need,
                                           volatile int *status) {
    __shared__ int ok;
    if (threadIdx.x == 0) {
        int good = 1;
        const uint64_t t0 = global_ns();
        while (ld_acquire_u32(flags + hl) < need || ld_acquire_u32(flags + hr) < need) {
            if (*status != 0) { good = 0; break; }
            if (global_ns() - t0 > SW_WAIT_NS) {
                atomicCAS((int *)status, 0, 1);
                good = 0;
                break;
            }
            __nanosleep(64);
        }
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// L2-only loads (ld.global.cg) of a slot cell
__device__ __forceinline__ double ldcg(const double *p) { return __ldcg(p); }
__device__ __forceinline__ float ldcg(const float *p) { return __ldcg(p); }
__device__ __forceinline__ V4<double> ldcg(const V4<double> *p) {
    const double2 a = __ldcg(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldcg(reinterpret_cast<const double2 *>(p) + 1);
    return V4<double>{a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ V4<float> ldcg(const V4<float> *p) {
    const float4 a = __ldcg(reinterpret_cast<const float4 *>(p));
    return V4<float>{a.x, a.y, a.z, a.w};
}

template <int P, typename T>
__device__ __forceinline__ void tile_import_cg(T *rows, int L, int W, const typename Scheme<P, T>::G *sl,
                                               const typename Scheme<P, T>::G *sr) {
    // slots were written by other SMs: read through L2 (ld.global.cg), never a stale L1 line
    constexpr int R = Scheme<P, T>::R;
    const int h = W >> 1;
    for (int i = threadIdx.x; i < W; i += blockDim.x) {
        if (i < h) {
            tile_put<P, T>(rows, L, 0, i, ldcg(sl + i));
            tile_put<P, T>(rows, L, 1, i - R, ldcg(sl + h + i));
        } else {
            const int j = i - h;
            tile_put<P, T>(rows, L, 0, h + j, ldcg(sr + j));
            tile_put<P, T>(rows, L, 1, h + R + j, ldcg(sr + h + j));
        }
    }
}

template <int P, typename T>
__global__ void __launch_bounds__(Scheme<P, T>::MAXT)
    k_persistent(const Params<T> p, typename Scheme<P, T>::G *__restrict__ state,
                 typename Scheme<P, T>::G *__restrict__ slots, unsigned *__restrict__ flags, int *status, const int W,
                 const int64_t n_diamonds) {
    constexpr int R = Scheme<P, T>::R;
    extern __shared__ __align__(16) unsigned char sw_smem[];
    T *rows = reinterpret_cast<T *>(sw_smem);
    const int L = W + 2 * R, h = W >> 1;
    const int64_t nx = p.nx, nhalf = nx / h, ntile = nx / W;
    const int64_t last = n_diamonds + 1;

    for (int64_t q = 0; q <= last; ++q) {
        const int phase = (int)(q & 1);
        for (int64_t t = blockIdx.x; t < ntile; t += gridDim.x) {
            const int64_t base = t * W + (int64_t)phase * h;
            const int64_t hl = (2 * t + phase) % nhalf;
            const int64_t hr = (hl + 1 == nhalf) ? 0 : hl + 1;
            if (q == 0) {
                for (int x = threadIdx.x; x < W; x += blockDim.x) tile_put<P, T>(rows, L, 0, x, state[base + x]);
            } else {
                if (!wait_slots(flags, hl, hr, (unsigned)q, status)) return;
                tile_import_cg<P, T>(rows, L, W, slots + hl * W, slots + hr * W);
            }
            if constexpr (P == SW_EULER) {
                __syncthreads();
                tile_fix_bc<P, T>(p, rows, L, base);
            }
            __syncthreads();
            if (q > 0) tile_down<P, T>(p, rows, L, W, base);
            if (q == last) {
                for (int x = threadIdx.x; x < W; x += blockDim.x)
                    state[wrap_pos(base + x, nx)] = tile_get<P, T>(rows, L, 0, x);
                __syncthreads();
            } else {
                tile_up<P, T>(p, rows, L, W, base);
                tile_export<P, T>(rows, L, W, slots + hl * W, slots + hr * W);
                __threadfence();
                __syncthreads();
                if (threadIdx.x == 0) {
                    st_release_u32(flags + hl, (unsigned)(q + 1));
                    st_release_u32(flags + hr, (unsigned)(q + 1));
                }
            }
        }
    }
}

template <int P, typename T>
cudaError_t launch_persistent(const void *vp, void *state, void *slots, unsigned *flags, int *status, int64_t nx,
                              int W, int64_t n_diamonds, cudaStream_t s) {
    using G = typename Scheme<P, T>::G;
    static bool configured = false;
    auto kern = k_persistent<P, T>;
    const size_t smem = swept_smem_bytes<P, T>(W);
    if (!configured) {
        allow_big_smem(kern);
        configured = true;
    }
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int threads = W < Scheme<P, T>::MAXT ? W : Scheme<P, T>::MAXT;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int64_t ntile = nx / W;
    int64_t grid = (int64_t)per_sm * sms;
    if (grid > ntile) grid = ntile;
    const int64_t nhalf = nx / (W >> 1);
    e = cudaMemsetAsync(flags, 0, sizeof(unsigned) * nhalf, s);
    if (e != cudaSuccess) return e;
    Params<T> p = *static_cast<const Params<T> *>(vp);
    G *st = static_cast<G *>(state), *sl = static_cast<G *>(slots);
    int Wv = W;
    int64_t nd = n_diamonds;
    void *args[] = {&p, &st, &sl, &flags, &status, &Wv, &nd};
    return cudaLaunchCooperativeKernel((const void *)kern, dim3((unsigned)grid), dim3(threads), args, smem, s);
}

}  // namespace sw
