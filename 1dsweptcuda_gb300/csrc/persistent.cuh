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

SW_KERNELS_BEGIN

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Thread 0 waits for both slot flags to reach `need`; returns false (and sets
// *status) if the wait runs out or another block already failed.  The wait
// ends after limit_ns of %globaltimer, or after limit_ns / 16 polls (each
// sleeps >= 64 ns, so >= 4 x limit_ns) should the timer ever stand still.
__device__ __forceinline__ bool wait_slots(const unsigned *flags, int64_t hl, int64_t hr, unsigned need,
                                           volatile int *status, uint64_t limit_ns = SW_WAIT_NS) {
    __shared__ int ok;
    if (threadIdx.x == 0) {
        int good = 1;
        const uint64_t t0 = global_ns(), max_polls = limit_ns / 16;
        uint64_t polls = 0;
        while (ld_acquire_u32(flags + hl) < need || ld_acquire_u32(flags + hr) < need) {
            if (*status != 0) { good = 0; break; }
            if (global_ns() - t0 > limit_ns || ++polls > max_polls) {
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

// Stage q of tile t of one domain (state / slots / flags at the domain's
// base).  Returns false if a wait gave up.
template <int P, typename T, int PATH>
__device__ __forceinline__ bool persistent_tile(const Params<T> &p, typename Scheme<P, T>::G *__restrict__ state,
                                                typename Scheme<P, T>::G *__restrict__ slots, unsigned *flags,
                                                int *status, T *rows, const int W, const int64_t q,
                                                const int64_t last, const int64_t t) {
    const int L = row_stride(W), h = W >> 1;
    const int64_t nx = p.nx, nhalf = nx / h;
    const int phase = (int)(q & 1);
    const int64_t base = t * W + (int64_t)phase * h;
    const int64_t hl = (2 * t + phase) % nhalf;
    const int64_t hr = (hl + 1 == nhalf) ? 0 : hl + 1;
    if (q == 0) {
        for (int x = threadIdx.x; x < W; x += blockDim.x) tile_put<P, T>(rows, L, 0, x, state[base + x]);
    } else {
        if (!wait_slots(flags, hl, hr, (unsigned)q, status)) return false;
        tile_import_cg<P, T>(rows, L, W, slots + hl * W, slots + hr * W);
    }
    if constexpr (P == SW_EULER) {
        __syncthreads();
        tile_fix_bc<P, T>(p, rows, L, base);
    }
    __syncthreads();
    if (q > 0) tile_down<P, T, PATH>(p, rows, L, W, base);
    if (q == last) {
        for (int x = threadIdx.x; x < W; x += blockDim.x)
            state[wrap_pos(base + x, nx)] = tile_get<P, T>(rows, L, 0, x);
        __syncthreads();
    } else {
        tile_up<P, T, PATH>(p, rows, L, W, base);
        tile_export<P, T>(rows, L, W, slots + hl * W, slots + hr * W);
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) {
            st_release_u32(flags + hl, (unsigned)(q + 1));
            st_release_u32(flags + hr, (unsigned)(q + 1));
        }
    }
    return true;
}

template <int P, typename T, int PATH>
__global__ void __launch_bounds__(Scheme<P, T>::MAXT)
    k_persistent(const Params<T> p, typename Scheme<P, T>::G *__restrict__ state,
                 typename Scheme<P, T>::G *__restrict__ slots, unsigned *__restrict__ flags, int *status, const int W,
                 const int64_t n_diamonds) {
    extern __shared__ __align__(16) unsigned char sw_smem[];
    T *rows = reinterpret_cast<T *>(sw_smem);
    const int64_t ntile = p.nx / W, last = n_diamonds + 1;
    for (int64_t q = 0; q <= last; ++q)
        for (int64_t t = blockIdx.x; t < ntile; t += gridDim.x)
            if (!persistent_tile<P, T, PATH>(p, state, slots, flags, status, rows, W, q, last, t)) return;
}

// ---------------------------------------------------------- KS 32-cell nodes
// KS alg 2 (the reference's register path, KS1D_SweptShared.cu:396-592) runs
// 32-cell nodes, one warp each, eight per block.  Each warp has its own tile
// rows in shared memory and runs persistent_tile's steps with warp barriers
// only, using the block's shared tile code (tile_put / tile_point / tile_get),
// so the results are those of persistent_tile bit for bit.  Eight nodes per
// block lift the per-SM warp count above the 32 that one-warp blocks allow.

// Lane 0 waits as wait_slots does; the warp learns the outcome by a shuffle.
__device__ __forceinline__ bool wait_slots_warp(const unsigned *flags, int64_t hl, int64_t hr, unsigned need,
                                                volatile int *status, uint64_t limit_ns = SW_WAIT_NS) {
    int good = 1;
    if ((threadIdx.x & 31) == 0) {
        const uint64_t t0 = global_ns(), max_polls = limit_ns / 16;
        uint64_t polls = 0;
        while (ld_acquire_u32(flags + hl) < need || ld_acquire_u32(flags + hr) < need) {
            if (*status != 0) { good = 0; break; }
            if (global_ns() - t0 > limit_ns || ++polls > max_polls) {
                atomicCAS((int *)status, 0, 1);
                good = 0;
                break;
            }
            __nanosleep(64);
        }
    }
    good = __shfl_sync(0xffffffffu, good, 0);
    __syncwarp();
    return good != 0;
}

constexpr int kKsWarpNodesPerBlock = 8;

// The warp barrier that ends a level of a one-warp node: level_barrier's warp
// form (a flagged lane computes its cell again on the FP64 pipe first).
template <typename T, typename Fix>
__device__ __forceinline__ void warp_level_barrier(uint32_t flagged, Fix &&fix) {
    if constexpr (int_products<SW_KS, T>()) {
        if (__any_sync(0xffffffffu, flagged != 0) && flagged) fix();
    }
    __syncwarp();
}

template <typename T>
__device__ __forceinline__ bool ks_smem_node_tile(const Params<T> &p, T *__restrict__ state, T *__restrict__ slots,
                                                  unsigned *flags, int *status, T *rows, const int64_t q,
                                                  const int64_t last, const int64_t t) {
    constexpr int W = 32, h = 16, R = 2, H = W / (2 * R);
    const int L = row_stride(W), x = threadIdx.x & 31;
    const int64_t nx = p.nx, nhalf = nx / h;
    const int phase = (int)(q & 1);
    const int64_t base = t * W + (int64_t)phase * h;
    const int64_t hl = (2 * t + phase) % nhalf;
    const int64_t hr = (hl + 1 == nhalf) ? 0 : hl + 1;
    T *sl = slots + hl * W, *sr = slots + hr * W;
    if (q == 0) {
        tile_put<SW_KS, T>(rows, L, 0, x, state[base + x]);
    } else {
        if (!wait_slots_warp(flags, hl, hr, (unsigned)q, status)) return false;
        if (x < h) {  // as tile_import_cg, one cell per lane
            tile_put<SW_KS, T>(rows, L, 0, x, ldcg(sl + x));
            tile_put<SW_KS, T>(rows, L, 1, x - R, ldcg(sl + h + x));
        } else {
            const int j = x - h;
            tile_put<SW_KS, T>(rows, L, 0, h + j, ldcg(sr + j));
            tile_put<SW_KS, T>(rows, L, 1, h + R + j, ldcg(sr + h + j));
        }
    }
    __syncwarp();
    const Ends e{INT32_MIN / 2, INT32_MIN / 2};  // KS is periodic: no end cells
    if (q > 0) {
        for (int jl = 1; jl <= H; ++jl) {
            uint32_t flagged = 0;
            if (x >= h - jl * R && x < h + jl * R) flagged = tile_point<SW_KS, T>(p, rows, L, jl & 1, x, e);
            warp_level_barrier<T>(flagged, [&] { tile_point_pipe<SW_KS, T>(p, rows, L, jl & 1, x, e); });
        }
    }
    if (q == last) {
        state[wrap_pos(base + x, nx)] = tile_get<SW_KS, T>(rows, L, 0, x);
        return true;
    }
    for (int u = 1; u < H; ++u) {
        uint32_t flagged = 0;
        if (x >= u * R && x < W - u * R) flagged = tile_point<SW_KS, T>(p, rows, L, u & 1, x, e);
        warp_level_barrier<T>(flagged, [&] { tile_point_pipe<SW_KS, T>(p, rows, L, u & 1, x, e); });
    }
    if (x < h) {  // as tile_export
        sl[x] = tile_get<SW_KS, T>(rows, L, 0, x);
        sl[h + x] = tile_get<SW_KS, T>(rows, L, 1, R + x);
    } else {
        const int j = x - h;
        sr[j] = tile_get<SW_KS, T>(rows, L, 0, h + j);
        sr[h + j] = tile_get<SW_KS, T>(rows, L, 1, h - R + j);
    }
    __threadfence();
    __syncwarp();
    if (x == 0) {
        st_release_u32(flags + hl, (unsigned)(q + 1));
        st_release_u32(flags + hr, (unsigned)(q + 1));
    }
    __syncwarp();  // the next stage's import overwrites this warp's rows
    return true;
}

template <typename T>
__global__ void __launch_bounds__(32 * kKsWarpNodesPerBlock)
    k_persistent_ks_smem_nodes(const Params<T> p, T *__restrict__ state, T *__restrict__ slots,
                               unsigned *__restrict__ flags, int *status, const int64_t n_diamonds) {
    extern __shared__ __align__(16) unsigned char sw_smem[];
    T *rows = reinterpret_cast<T *>(sw_smem) + (threadIdx.x >> 5) * (tile_rows<SW_KS>() * row_stride(32));
    const int64_t ntile = p.nx / 32, last = n_diamonds + 1;
    const int64_t w0 = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t q = 0; q <= last; ++q)
        for (int64_t t = w0; t < ntile; t += nw)
            if (!ks_smem_node_tile<T>(p, state, slots, flags, status, rows, q, last, t)) return;
}

template <typename T>
cudaError_t launch_persistent_ks_smem_nodes(const Params<T> &p, T *st, T *sl, unsigned *flags, int *status,
                                            int64_t nx, int64_t n_diamonds, cudaStream_t s) {
    auto kern = k_persistent_ks_smem_nodes<T>;
    const int threads = 32 * kKsWarpNodesPerBlock;
    const size_t smem = kKsWarpNodesPerBlock * swept_smem_bytes<SW_KS, T>(32);
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int64_t ntile = nx / 32;
    int64_t grid = (int64_t)per_sm * sms;
    const int64_t need = (ntile + kKsWarpNodesPerBlock - 1) / kKsWarpNodesPerBlock;
    if (grid > need) grid = need;
    e = cudaMemsetAsync(flags, 0, sizeof(unsigned) * (nx / 16), s);
    if (e != cudaSuccess) return e;
    Params<T> pv = p;
    int64_t nd = n_diamonds;
    void *args[] = {&pv, &st, &sl, &flags, &status, &nd};
    return cudaLaunchCooperativeKernel((const void *)kern, dim3((unsigned)grid), dim3(threads), args, smem, s);
}

// ------------------------------------------------------------ ensembles
// Many independent domains of uneven length in one launch (BatchDev, in
// sw_internal.h, maps a global tile to its domain).

template <int P, typename T, int MODE, int PATH>
__global__ void __launch_bounds__(Scheme<P, T>::MAXT, (swept_min_blocks<P, T, PATH>()))
    k_swept_batch(const Params<T> p, typename Scheme<P, T>::G *__restrict__ state,
                  typename Scheme<P, T>::G *__restrict__ slots, const BatchDev b, const int W, const int phase) {
    extern __shared__ __align__(16) unsigned char sw_smem[];
    const int64_t g = blockIdx.x;
    const int d = b.tile_dom[g];
    const int64_t off = b.off[d];
    Params<T> q = p;
    q.nx = b.off[d + 1] - off;
    swept_tile<P, T, MODE, PATH>(q, state + off, slots + 2 * off, reinterpret_cast<T *>(sw_smem), W, phase,
                           g - b.tile0[d]);
}

// G consecutive tiles of one domain per block (one cell per thread), as
// k_swept_group runs a single domain: the batch's tile counts are all
// multiples of G (BatchDev::group), so a block's tiles never straddle domains.
template <int P, typename T, int MODE, int G, int PATH>
__global__ void __launch_bounds__(1024, 2)
    k_swept_batch_group(const Params<T> p, T *__restrict__ state, T *__restrict__ slots, const BatchDev b, const int W,
                        const int phase) {
    extern __shared__ __align__(16) unsigned char sw_smem[];
    const int64_t g0 = G * (int64_t)blockIdx.x;
    const int d = b.tile_dom[g0];
    const int64_t off = b.off[d];
    Params<T> q = p;
    q.nx = b.off[d + 1] - off;
    swept_tile_group<P, T, MODE, G, PATH>(q, state + off, slots + 2 * off, reinterpret_cast<T *>(sw_smem), W, phase,
                                          g0 - b.tile0[d]);
}

// Classic step of an ensemble, one cell per thread, kClassicBlock threads per
// block.  The table gives the domain of the block's first cell; each thread
// walks forward from it, which is one compare when domains are longer than a
// block.
template <int P, typename T>
__global__ void __launch_bounds__(kClassicBlock)
    k_classic_batch(const Params<T> p, const typename Scheme<P, T>::G *__restrict__ in,
                    typename Scheme<P, T>::G *__restrict__ out, const BatchDev b, const int sub) {
    const int64_t g = (int64_t)blockIdx.x * kClassicBlock + threadIdx.x;
    if (g >= b.n_cells) return;
    int d = b.blk_dom[blockIdx.x];
    while (b.off[d + 1] <= g) ++d;
    const int64_t off = b.off[d];
    Params<T> q = p;
    q.nx = b.off[d + 1] - off;
    classic_cell<P, T>(q, in + off, out + off, sub, g - off);
}

template <int P, typename T, int PATH>
__global__ void __launch_bounds__(Scheme<P, T>::MAXT)
    k_persistent_batch(const Params<T> p, typename Scheme<P, T>::G *__restrict__ state,
                       typename Scheme<P, T>::G *__restrict__ slots, const BatchDev b, unsigned *__restrict__ flags,
                       int *status, const int W, const int64_t n_diamonds) {
    extern __shared__ __align__(16) unsigned char sw_smem[];
    T *rows = reinterpret_cast<T *>(sw_smem);
    const int64_t last = n_diamonds + 1;
    for (int64_t q = 0; q <= last; ++q) {
        for (int64_t g = blockIdx.x; g < b.n_tiles; g += gridDim.x) {
            const int d = b.tile_dom[g];
            const int64_t off = b.off[d];
            Params<T> pp = p;
            pp.nx = b.off[d + 1] - off;
            if (!persistent_tile<P, T, PATH>(pp, state + off, slots + 2 * off, flags + 2 * b.tile0[d], status, rows, W, q,
                                       last, g - b.tile0[d]))
                return;
        }
    }
}

// The cell path a launch runs: 4 cells per thread when threads * 4 == W (not Euler).
template <int P, typename T>
inline bool span4_launch(int W, int threads) {
    return P != SW_EULER && threads * 4 == W;
}

template <int P, typename T, int PATH>
cudaError_t launch_persistent_path(const Params<T> &p, typename Scheme<P, T>::G *st, typename Scheme<P, T>::G *sl,
                                   unsigned *flags, int *status, int64_t nx, int W, int threads, int64_t n_diamonds,
                                   cudaStream_t s) {
    static SmemOnce once;
    auto kern = k_persistent<P, T, PATH>;
    const size_t smem = swept_smem_bytes<P, T>(W);
    cudaError_t e = once.ensure(kern);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int64_t ntile = nx / W;
    int64_t grid = (int64_t)per_sm * sms;
    if (grid > ntile) grid = ntile;
    const int64_t nhalf = nx / (W >> 1);
    e = cudaMemsetAsync(flags, 0, sizeof(unsigned) * nhalf, s);
    if (e != cudaSuccess) return e;
    Params<T> pv = p;
    int Wv = W;
    int64_t nd = n_diamonds;
    void *args[] = {&pv, &st, &sl, &flags, &status, &Wv, &nd};
    return cudaLaunchCooperativeKernel((const void *)kern, dim3((unsigned)grid), dim3(threads), args, smem, s);
}

template <int P, typename T>
cudaError_t launch_persistent(const void *vp, void *state, void *slots, unsigned *flags, int *status, int64_t nx,
                              int W, int threads_req, int64_t n_diamonds, cudaStream_t s) {
    using G = typename Scheme<P, T>::G;
    const Params<T> &p = *static_cast<const Params<T> *>(vp);
    const int threads = swept_threads_for<P, T>(W, threads_req);
    G *st = static_cast<G *>(state), *sl = static_cast<G *>(slots);
    if constexpr (P == SW_KS) {
        if (W == 32) return launch_persistent_ks_smem_nodes<T>(p, st, sl, flags, status, nx, n_diamonds, s);
    }
    if (span4_launch<P, T>(W, threads))
        return launch_persistent_path<P, T, PATH_SPAN4>(p, st, sl, flags, status, nx, W, threads, n_diamonds, s);
    if constexpr (int_products<P, T>()) {
        if (few_tiles(nx / W))
            return launch_persistent_path<P, T, PATH_CELL_FP>(p, st, sl, flags, status, nx, W, threads, n_diamonds, s);
    }
    return launch_persistent_path<P, T, PATH_CELL>(p, st, sl, flags, status, nx, W, threads, n_diamonds, s);
}

template <int P, typename T, int PATH>
cudaError_t launch_swept_batch_path(const Params<T> &p, int mode, int phase, typename Scheme<P, T>::G *st,
                                    typename Scheme<P, T>::G *sl, const BatchDev &b, int W, int threads,
                                    cudaStream_t s) {
    static SmemOnce once;
    cudaError_t e = once.ensure(k_swept_batch<P, T, MODE_UP, PATH>, k_swept_batch<P, T, MODE_DIAMOND, PATH>,
                                k_swept_batch<P, T, MODE_DOWN, PATH>);
    if (e != cudaSuccess) return e;
    const size_t smem = swept_smem_bytes<P, T>(W);
    const unsigned grid = (unsigned)b.n_tiles;
    switch (mode) {
    case MODE_UP: k_swept_batch<P, T, MODE_UP, PATH><<<grid, threads, smem, s>>>(p, st, sl, b, W, phase); break;
    case MODE_DIAMOND:
        k_swept_batch<P, T, MODE_DIAMOND, PATH><<<grid, threads, smem, s>>>(p, st, sl, b, W, phase);
        break;
    default: k_swept_batch<P, T, MODE_DOWN, PATH><<<grid, threads, smem, s>>>(p, st, sl, b, W, phase); break;
    }
    return cudaGetLastError();
}

template <int P, typename T, int G>
cudaError_t launch_swept_batch_group(const Params<T> &p, int mode, int phase, T *st, T *sl, const BatchDev &b, int W,
                                     cudaStream_t s) {
    static SmemOnce once;
    cudaError_t e = once.ensure(k_swept_batch_group<P, T, MODE_UP, G, PATH_CELL>,
                                k_swept_batch_group<P, T, MODE_DIAMOND, G, PATH_CELL>,
                                k_swept_batch_group<P, T, MODE_DOWN, G, PATH_CELL>);
    if (e != cudaSuccess) return e;
    const size_t smem = G * swept_smem_bytes<P, T>(W);
    const unsigned grid = (unsigned)(b.n_tiles / G);
    const int block = G * W;
    switch (mode) {
    case MODE_UP:
        k_swept_batch_group<P, T, MODE_UP, G, PATH_CELL><<<grid, block, smem, s>>>(p, st, sl, b, W, phase);
        break;
    case MODE_DIAMOND:
        k_swept_batch_group<P, T, MODE_DIAMOND, G, PATH_CELL><<<grid, block, smem, s>>>(p, st, sl, b, W, phase);
        break;
    default: k_swept_batch_group<P, T, MODE_DOWN, G, PATH_CELL><<<grid, block, smem, s>>>(p, st, sl, b, W, phase); break;
    }
    return cudaGetLastError();
}

template <int P, typename T>
cudaError_t launch_swept_batch(const void *vp, int mode, int phase, void *state, void *slots, const void *bt, int W,
                               int threads, cudaStream_t s) {
    using G = typename Scheme<P, T>::G;
    const Params<T> &p = *static_cast<const Params<T> *>(vp);
    const BatchDev &b = *static_cast<const BatchDev *>(bt);
    threads = swept_threads_for<P, T>(W, threads);
    G *st = static_cast<G *>(state), *sl = static_cast<G *>(slots);
    if constexpr (P != SW_EULER) {
        // one cell per thread: G tiles of a domain per block, as the single-domain
        // launcher groups them (KS four up to 1024 threads, Heat two up to 512),
        // where blocks are plentiful
        constexpr int kMaxThreads = (P == SW_KS) ? 1024 : 512;
        if (threads == W && !span4_launch<P, T>(W, threads) && b.n_tiles >= kGroupMinTiles) {
            if (P == SW_KS && 4 * W <= kMaxThreads && b.group % 4 == 0)
                return launch_swept_batch_group<P, T, 4>(p, mode, phase, st, sl, b, W, s);
            if (2 * W <= kMaxThreads && b.group % 2 == 0)
                return launch_swept_batch_group<P, T, 2>(p, mode, phase, st, sl, b, W, s);
        }
    }
    if (span4_launch<P, T>(W, threads))
        return launch_swept_batch_path<P, T, PATH_SPAN4>(p, mode, phase, st, sl, b, W, threads, s);
    if constexpr (int_products<P, T>()) {  // few tiles: the FP64 products (PATH_CELL_FP)
        if (few_tiles(b.n_tiles))
            return launch_swept_batch_path<P, T, PATH_CELL_FP>(p, mode, phase, st, sl, b, W, threads, s);
    }
    return launch_swept_batch_path<P, T, PATH_CELL>(p, mode, phase, st, sl, b, W, threads, s);
}

template <int P, typename T>
cudaError_t launch_classic_batch(const void *vp, const void *in, void *out, int sub, const void *bt, int block,
                                 cudaStream_t s) {
    using G = typename Scheme<P, T>::G;
    const Params<T> &p = *static_cast<const Params<T> *>(vp);
    const BatchDev &b = *static_cast<const BatchDev *>(bt);
    (void)block;  // the block is fixed by the domain table's granularity
    const int64_t grid = (b.n_cells + kClassicBlock - 1) / kClassicBlock;
    k_classic_batch<P, T><<<(unsigned)grid, kClassicBlock, 0, s>>>(p, static_cast<const G *>(in), static_cast<G *>(out),
                                                                    b, sub);
    return cudaGetLastError();
}

// Cooperative launch through cudaLaunchKernelEx so that it can be captured
// into a CUDA graph.
template <int P, typename T, int PATH>
cudaError_t launch_persistent_batch_path(const Params<T> &p, typename Scheme<P, T>::G *st,
                                         typename Scheme<P, T>::G *sl, const BatchDev &b, unsigned *flags,
                                         int *status, int W, int threads, int64_t n_diamonds, cudaStream_t s) {
    static SmemOnce once;
    auto kern = k_persistent_batch<P, T, PATH>;
    const size_t smem = swept_smem_bytes<P, T>(W);
    cudaError_t e = once.ensure(kern);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int64_t grid = (int64_t)per_sm * sms;
    if (grid > b.n_tiles) grid = b.n_tiles;
    e = cudaMemsetAsync(flags, 0, sizeof(unsigned) * 2 * b.n_tiles, s);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, p, st, sl, b, flags, status, W, n_diamonds);
}

template <int P, typename T>
cudaError_t launch_persistent_batch(const void *vp, void *state, void *slots, const void *bt, unsigned *flags,
                                    int *status, int W, int threads, int64_t n_diamonds, cudaStream_t s) {
    using G = typename Scheme<P, T>::G;
    const Params<T> &p = *static_cast<const Params<T> *>(vp);
    const BatchDev &b = *static_cast<const BatchDev *>(bt);
    threads = swept_threads_for<P, T>(W, threads);
    G *st = static_cast<G *>(state), *sl = static_cast<G *>(slots);
    if (span4_launch<P, T>(W, threads))
        return launch_persistent_batch_path<P, T, PATH_SPAN4>(p, st, sl, b, flags, status, W, threads, n_diamonds, s);
    return launch_persistent_batch_path<P, T, PATH_CELL>(p, st, sl, b, flags, status, W, threads, n_diamonds, s);
}

SW_KERNELS_END
