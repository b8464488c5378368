// Kernels of the swept and classic schemes, generic over the problem P
// (SW_HEAT / SW_KS / SW_EULER) and the precision T.  Each k_*.cu includes this
// file and instantiates one problem for float and double.
//
// Swept decomposition (the reference's upTriangle / wholeDiamond /
// splitDiamond / downTriangle, Heat1D_SweptShared.cu:147-408,
// KS1D_SweptShared.cu:209-394, Euler1D_SweptShared.cu:437-746), laid out for
// GB300:
//  * a tile of W cells keeps two rows in shared memory; sub-step m reads row
//    (m-1)&1 and writes row m&1 (Heat: the two time-parity rows; KS/Euler: row
//    0 = u, row 1 = predictor u*, the corrector adds into row 0).  Each row has
//    R margin cells on both sides;
//  * the up part computes sub-steps u = 1..H-1 (H = W/(2R)) on [uR, W-uR); the
//    down part of a tile shifted by W/2 computes j = 1..H on [W/2-jR, W/2+jR);
//  * the edge exchange goes through one slot of W cells per half-tile
//    (2*nx cells in all): row 0 of the half, then row 1 of the half moved R
//    cells toward the tile centre.  A diamond reads the slots of its two halves
//    and overwrites the same two slots with its own exports, so one buffer
//    serves every pass (no ping-pong) and each access is a contiguous,
//    coalesced run of W/2 cells;
//  * phase 0 tiles start at t*W, phase 1 tiles at t*W + W/2 (mod nx), so the
//    reference's "split" diamond is simply the last phase-1 tile, whose
//    positions wrap; boundary conditions are applied per cell from its global
//    position.
// Every (cell, sub-step) value is computed once with the classic arithmetic,
// so swept, variant and classic agree bit for bit.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <climits>
#include <cstdint>
#include <type_traits>

#include "stencils.cuh"
#include "sw_internal.h"

SW_KERNELS_BEGIN

template <typename T>
struct alignas(4 * sizeof(T)) V4 {
    T x, y, z, w;
};

template <int P, typename T>
struct Scheme {
    static constexpr int R = (P == SW_HEAT) ? 1 : 2;
    static constexpr int S = (P == SW_HEAT) ? 1 : 2;
    static constexpr int C = (P == SW_EULER) ? 3 : 1;
    // largest swept block: 512 threads for Heat/KS (a 1024-thread bound would
    // cap the FP64 kernels at 32 registers and spill), 256 for Euler so its
    // long stencil keeps its registers
    static constexpr int MAXT = (P == SW_EULER) ? 256 : 512;
    // largest classic block (one cell per thread, any block size gives the same result)
    static constexpr int CMAXT = (P == SW_EULER) ? 256 : 1024;
    using G = typename std::conditional<P == SW_EULER, V4<T>, T>::type;
};

// ---- shared-memory tile access: layout [row][component][L], cell x of a row at
// index R + x.  L = W + 8 (>= W + 2R): every row starts 16-byte aligned and the
// 8-value windows of the 4-cells-per-thread path never leave their row.  KS
// also keeps rows 2 and 3, the squares of rows 0 and 1, for the
// one-cell-per-thread path: every write of a value there writes its square.
__host__ __device__ constexpr int row_stride(int W) { return W + 8; }
template <int P>
__host__ __device__ constexpr int tile_rows() { return P == SW_KS ? 4 : 2; }
template <int P, typename T>
__device__ __forceinline__ void tile_put(T *rows, int L, int row, int x, const typename Scheme<P, T>::G &v) {
    constexpr int R = Scheme<P, T>::R;
    if constexpr (P == SW_EULER) {
        T *b = rows + row * 3 * L + R + x;
        b[0] = v.x;
        b[L] = v.y;
        b[2 * L] = v.z;
    } else {
        rows[row * L + R + x] = v;
        if constexpr (P == SW_KS) rows[(2 + row) * L + R + x] = ml(v, v);
    }
}
template <int P, typename T>
__device__ __forceinline__ typename Scheme<P, T>::G tile_get(const T *rows, int L, int row, int x) {
    constexpr int R = Scheme<P, T>::R;
    if constexpr (P == SW_EULER) {
        const T *b = rows + row * 3 * L + R + x;
        return V4<T>{b[0], b[L], b[2 * L], T(0)};
    } else {
        return rows[row * L + R + x];
    }
}

// Tile coordinates of the domain's first and last cell (global 0 and nx-1),
// or a sentinel outside [-R, W+R) when the tile does not hold them.  Boundary
// conditions then cost two integer compares per cell instead of a wrapped
// 64-bit position.
struct Ends {
    int first, last;
};
__device__ __forceinline__ int tile_coord_of(int64_t g, int64_t base, int64_t nx, int lo, int hi) {
    int64_t x = (g - base) % nx;
    if (x < 0) x += nx;
    if (x < hi) return (int)x;
    if (x - nx >= lo) return (int)(x - nx);
    return INT32_MIN / 2;
}
__device__ __forceinline__ Ends tile_ends(int64_t base, int64_t nx, int W, int R) {
    return Ends{tile_coord_of(0, base, nx, -R, W + R), tile_coord_of(nx - 1, base, nx, -R, W + R)};
}

// One Heat / KS sub-step of parity `par` (1: predictor / odd Heat step; 0:
// corrector / even Heat step) at tile cell x.  (Euler levels run euler_level_tile / _warp.)
//
// FP64 Heat and KS form their general products on the integer pipe (mlq):
// Heat both of its two, KS the sub-step's two (by dt, and the new value's
// square).  A cell where one of them meets an operand or a product that path
// does not take (a zero, a subnormal, an infinity, a NaN, a product near the
// ends of the range) stores nothing and returns 1; the level's barrier
// (level_barrier) then has the flagged cells computed on the FP64 pipe
// (tile_point_pipe), from the same source rows, before any cell reads them.
// The results are the same bits either way, and in the common case no FP64
// instruction of that fallback is issued.
//
// Which cell mapping a kernel carries: PATH_ANY picks at run time (blockDim.x
// * 4 == W: 4 cells per thread), PATH_CELL and PATH_SPAN4 hold only one, so a
// kernel does not pay the registers of a path it never runs.  PATH_CELL_FP is
// PATH_CELL with every product on the FP64 pipe: for domains of few tiles, where
// each SM holds one or two tiles and a level's dependent chain is not hidden by
// other tiles' work, the integer products' longer chain costs more than the
// FP64 pipe time they free (Heat FP64 periodic, 32 tiles of 128 cells: 6.0e9
// cell-updates/s with them, 8.4e9 without).  Euler always runs
// euler_level_tile (FP64) or euler_level_warp (FP32).
enum TilePath { PATH_ANY = 0, PATH_CELL = 1, PATH_SPAN4 = 2, PATH_CELL_FP = 3 };

template <int P, typename T, int PATH = PATH_ANY>
__host__ __device__ constexpr bool int_products() {
    return P != SW_EULER && sizeof(T) == 8 && PATH != PATH_CELL_FP;
}

template <int P, typename T, int PATH = PATH_ANY>
__device__ __forceinline__ uint32_t tile_point(const Params<T> &p, T *rows, int L, int par, int x, Ends e) {
    static_assert(P != SW_EULER, "Euler tile levels run euler_level_tile / euler_level_warp");
    constexpr int R = Scheme<P, T>::R;
    const T *src = rows + (par ^ 1) * L + R;
    T *dst = rows + par * L + R;
    if constexpr (P == SW_HEAT) {
        int l = x - 1, r = x + 1;
        if (p.bc != SW_BC_PERIODIC) {  // insulated ends, Heat1D_SweptShared.cu:140-142,352-353
            if (x == e.first) l = x + 1;
            if (x == e.last) r = x - 1;
        }
        if constexpr (int_products<P, T, PATH>()) {
            uint32_t bad = 0;
            const T v = heat_step_q(p, src[l], src[x], src[r], bad);
            if (!bad) dst[x] = v;
            return bad;
        } else {
            dst[x] = heat_step(p, src[l], src[x], src[r]);
            return 0;
        }
    } else if constexpr (!int_products<P, T, PATH>()) {
        const T *sq = rows + (2 + (par ^ 1)) * L + R;  // squares of the source row
        const T v = par ? ks_predict_sq(p, src[x - 2], src[x - 1], src[x], src[x + 1], src[x + 2], sq[x - 1], sq[x + 1])
                        : ks_correct_sq(p, dst[x], src[x - 2], src[x - 1], src[x], src[x + 1], src[x + 2], sq[x - 1],
                                        sq[x + 1]);
        dst[x] = v;
        rows[(2 + par) * L + R + x] = ml(v, v);
        return 0;
    } else {
        const T *sq = rows + (2 + (par ^ 1)) * L + R;  // squares of the source row
        uint32_t bad = 0;
        const T v = par ? ks_predict_q(p, src[x - 2], src[x - 1], src[x], src[x + 1], src[x + 2], sq[x - 1], sq[x + 1],
                                       bad)
                        : ks_correct_q(p, dst[x], src[x - 2], src[x - 1], src[x], src[x + 1], src[x + 2], sq[x - 1],
                                       sq[x + 1], bad);
        const T v2 = mlq(v, v, bad);
        if (!bad) {
            dst[x] = v;
            rows[(2 + par) * L + R + x] = v2;
        }
        return bad;
    }
}
// Cell x of a level on the FP64 pipe alone (the cells tile_point flagged).
template <int P, typename T>
__device__ __noinline__ void tile_point_pipe(const Params<T> &p, T *rows, int L, int par, int x, Ends e) {
    constexpr int R = Scheme<P, T>::R;
    if constexpr (P == SW_HEAT && int_products<P, T>()) {
        const T *src = rows + (par ^ 1) * L + R;
        int l = x - 1, r = x + 1;
        if (p.bc != SW_BC_PERIODIC) {
            if (x == e.first) l = x + 1;
            if (x == e.last) r = x - 1;
        }
        rows[par * L + R + x] = heat_step(p, src[l], src[x], src[r]);
    } else if constexpr (int_products<P, T>()) {
        const T *src = rows + (par ^ 1) * L + R, *sq = rows + (2 + (par ^ 1)) * L + R;
        T *dst = rows + par * L + R;
        const T v = par ? ks_predict_sq(p, src[x - 2], src[x - 1], src[x], src[x + 1], src[x + 2], sq[x - 1], sq[x + 1])
                        : ks_correct_sq(p, dst[x], src[x - 2], src[x - 1], src[x], src[x + 1], src[x + 2], sq[x - 1],
                                        sq[x + 1]);
        dst[x] = v;
        rows[(2 + par) * L + R + x] = ml(v, v);
    }
}
// The barrier that ends a level.  With integer-pipe products it also tells
// whether any thread of the block flagged a cell; if one did, fix() computes
// the flagged cells on the FP64 pipe and a second barrier follows.
template <int P, typename T, int PATH, typename Fix>
__device__ __forceinline__ void level_barrier(uint32_t flagged, Fix &&fix) {
    if constexpr (int_products<P, T, PATH>()) {
        if (__syncthreads_or(flagged != 0)) {
            fix();
            __syncthreads();
        }
    } else {
        __syncthreads();
    }
}

// FP64 Euler tiles also keep, per level, the interface terms of
// euler_level_tile: the pressure differences D and the flux F and dissipation
// S (3 components each) of every interface, 7 values per row position.
constexpr int kEulerIfaceArrays = 7;
template <int P, typename T>
__host__ __device__ constexpr size_t swept_smem_bytes(int W) {
    return sizeof(T) *
           ((size_t)tile_rows<P>() * Scheme<P, T>::C + (P == SW_EULER && sizeof(T) == 8 ? kEulerIfaceArrays : 0)) *
           (size_t)row_stride(W);
}

__device__ __forceinline__ int64_t wrap_pos(int64_t q, int64_t nx) {
    if (q >= nx) q -= nx;
    if (q < 0) q += nx;
    return q;
}

// Euler: both rows of the Dirichlet cells hold the boundary states
// (splitDiamond, Euler1D_SweptShared.cu:684-694).
template <int P, typename T>
__device__ __forceinline__ void tile_fix_bc(const Params<T> &p, T *rows, int L, int64_t base) {
    if constexpr (P == SW_EULER) {
        constexpr int R = Scheme<P, T>::R;
        for (int i = threadIdx.x; i < L; i += blockDim.x) {
            const int x = i - R;
            const int64_t gp = wrap_pos(base + x, p.nx);
            if (gp == 0 || gp == p.nx - 1) {
                const int side = (gp == 0) ? 0 : 1;
                V4<T> b{p.bd[3 * side], p.bd[3 * side + 1], p.bd[3 * side + 2], T(0)};
                tile_put<P, T>(rows, L, 0, x, b);
                tile_put<P, T>(rows, L, 1, x, b);
            }
        }
    }
}

// Slot layout of half-tile h: cells [h*W, h*W + W/2) = row 0, [h*W + W/2, (h+1)*W) = row 1.
// Element i (0 <= i < W) of a tile's import / export: two values, one per row.
template <int P, typename T>
__device__ __forceinline__ void tile_import_at(T *rows, int L, int W, const typename Scheme<P, T>::G *sl,
                                               const typename Scheme<P, T>::G *sr, int i) {
    constexpr int R = Scheme<P, T>::R;
    const int h = W >> 1;
    if (i < h) {
        tile_put<P, T>(rows, L, 0, i, sl[i]);
        tile_put<P, T>(rows, L, 1, i - R, sl[h + i]);
    } else {
        const int j = i - h;
        tile_put<P, T>(rows, L, 0, h + j, sr[j]);
        tile_put<P, T>(rows, L, 1, h + R + j, sr[h + j]);
    }
}
template <int P, typename T>
__device__ __forceinline__ void tile_export_at(const T *rows, int L, int W, typename Scheme<P, T>::G *sl,
                                               typename Scheme<P, T>::G *sr, int i) {
    constexpr int R = Scheme<P, T>::R;
    const int h = W >> 1;
    if (i < h) {
        sl[i] = tile_get<P, T>(rows, L, 0, i);
        sl[h + i] = tile_get<P, T>(rows, L, 1, R + i);
    } else {
        const int j = i - h;
        sr[j] = tile_get<P, T>(rows, L, 0, h + j);
        sr[h + j] = tile_get<P, T>(rows, L, 1, h - R + j);
    }
}
template <int P, typename T>
__device__ __forceinline__ void tile_import(T *rows, int L, int W, const typename Scheme<P, T>::G *sl,
                                            const typename Scheme<P, T>::G *sr) {
    for (int i = threadIdx.x; i < W; i += blockDim.x) tile_import_at<P, T>(rows, L, W, sl, sr, i);
}
template <int P, typename T>
__device__ __forceinline__ void tile_export(const T *rows, int L, int W, typename Scheme<P, T>::G *sl,
                                            typename Scheme<P, T>::G *sr) {
    for (int i = threadIdx.x; i < W; i += blockDim.x) tile_export_at<P, T>(rows, L, W, sl, sr, i);
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---- bulk copies between global and shared memory (cp.async.bulk, the
// copy engine's 1D form), completion of loads tracked by an mbarrier.
// Addresses and sizes must be multiples of 16 bytes.
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_load(void *dst_smem, const void *src_global, unsigned bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst_smem)),
                 "l"(src_global), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void bulk_store(void *dst_global, const void *src_smem, unsigned bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst_global),
                 "r"(smem_addr(src_smem)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_store_commit_and_wait() {
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}
// Shared-memory writes of this thread made visible to the copy engine.
__device__ __forceinline__ void fence_smem_for_bulk() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Every thread waits for phase 0 of `bar`, up to kBulkWaitNs of %globaltimer
// (or kBulkWaitNs / 16 polls, should the timer stand still); the block's
// outcome is uniform.  A wait that runs out sets *status to 2 (when given)
// and the block returns false, so that its caller returns without touching
// the tile.  Bulk loads of valid global memory complete in microseconds: the
// limit only bounds a wait that something else went wrong with.
constexpr uint64_t kBulkWaitNs = 2000000000ull;
__device__ __forceinline__ bool bulk_wait(uint64_t *bar, int *status) {
    const uint64_t t0 = global_ns();
    uint64_t polls = 0;
    bool ok = true;
    while (!mbar_try_wait(bar, 0)) {
        if (global_ns() - t0 > kBulkWaitNs || ++polls > kBulkWaitNs / 16) {
            ok = false;
            break;
        }
    }
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0 && status) atomicCAS(status, 0, 2);
        const uint64_t t1 = global_ns();  // the copies in flight write this block's shared memory: wait
        polls = 0;                        // for them once more, again bounded, before the block leaves
        while (!mbar_try_wait(bar, 0) && global_ns() - t1 < kBulkWaitNs && ++polls < kBulkWaitNs / 16) {
        }
        return false;
    }
    return true;
}

// Aligned 4-value shared-memory loads.
__device__ __forceinline__ void load4(const float *p, float *w) {
    const float4 v = *reinterpret_cast<const float4 *>(p);
    w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w;
}
__device__ __forceinline__ void load4(const double *p, double *w) {
    const double2 a = *reinterpret_cast<const double2 *>(p);
    const double2 b = *reinterpret_cast<const double2 *>(p + 2);
    w[0] = a.x; w[1] = a.y; w[2] = b.x; w[3] = b.y;
}
// Four values as two aligned pairs (8-byte aligned float, 16-byte aligned double).
__device__ __forceinline__ void load_pairs(const float *p, float *w) {
    const float2 a = *reinterpret_cast<const float2 *>(p);
    const float2 b = *reinterpret_cast<const float2 *>(p + 2);
    w[0] = a.x; w[1] = a.y; w[2] = b.x; w[3] = b.y;
}
__device__ __forceinline__ void load_pairs(const double *p, double *w) { load4(p, w); }
__device__ __forceinline__ void store_pairs(float *p, const float *w) {
    *reinterpret_cast<float2 *>(p) = make_float2(w[0], w[1]);
    *reinterpret_cast<float2 *>(p + 2) = make_float2(w[2], w[3]);
}
__device__ __forceinline__ void store_pairs(double *p, const double *w) {
    *reinterpret_cast<double2 *>(p) = make_double2(w[0], w[1]);
    *reinterpret_cast<double2 *>(p + 2) = make_double2(w[2], w[3]);
}

// Heat / KS with 4 consecutive cells per thread (blockDim.x == W / 4, 0 <= lo <
// hi <= W).  The live range [lo, hi) is packed onto the lowest threads from the
// 4-aligned cell below lo, so that as a triangle narrows whole warps fall idle
// instead of every warp running part-empty.  The thread reads the 8-value
// window of source cells x0 - R .. x0 + 7 - R with two aligned vector loads and
// updates those of its cells x0 .. x0 + 3 that lie in [lo, hi).  Same
// arithmetic as tile_point, cell for cell.
// (tid: the thread's index among the tile's threads)
template <int P, typename T>
__device__ __forceinline__ void tile_span4(const Params<T> &p, T *rows, int L, int par, int lo, int hi, Ends e,
                                           const int tid) {
    constexpr int R = Scheme<P, T>::R;
    const int x0 = (lo & ~3) + tid * 4;
    if (x0 >= hi) return;
    const T *src = rows + (par ^ 1) * L;
    T *dst = rows + par * L + R;
    T w[8];
    load4(src + x0, w);  // cell x0 - R + k at src[R + x0 - R + k] = src[x0 + k]
    load4(src + x0 + 4, w + 4);
    // All four cells are computed (their windows lie inside the row; values of
    // cells outside [lo, hi) are never stored), so the warps at a triangle's
    // edge run the same instructions as the rest; only the stores branch.
    T o[4];
    if constexpr (P == SW_HEAT && std::is_same<T, float>::value) {
        // FP32 Heat: cells (x0, x0+1) and (x0+2, x0+3) as pairs (heat_step2).  Insulated
        // ends change a neighbour of cells first and last: those threads stay scalar.
        // (Paired KS measured slower than scalar KS: 4.96e11 against 5.62e11 at tile 1024.)
        if (p.bc == SW_BC_PERIODIC || ((unsigned)(e.first - x0) > 3u && (unsigned)(e.last - x0) > 3u)) {
            const float2 a = heat_step2(p, make_float2(w[0], w[1]), make_float2(w[1], w[2]), make_float2(w[2], w[3]));
            const float2 b = heat_step2(p, make_float2(w[2], w[3]), make_float2(w[3], w[4]), make_float2(w[4], w[5]));
            const float ov[4] = {a.x, a.y, b.x, b.y};
#pragma unroll
            for (int i = 0; i < 4; ++i)  // scalar stores: Heat rows are 4-byte aligned at x0 (R = 1)
                if (x0 + i >= lo && x0 + i < hi) dst[x0 + i] = ov[i];
            return;
        }
    }
    if constexpr (P == SW_KS) {
        if (par) {
#pragma unroll
            for (int i = 0; i < 4; ++i) o[i] = ks_predict(p, w[i], w[i + 1], w[i + 2], w[i + 3], w[i + 4]);
        } else {
            T d[4];
            load_pairs(dst + x0, d);  // dst + x0 = row + 2 + x0: 8-byte aligned for float, 16 for double
#pragma unroll
            for (int i = 0; i < 4; ++i) o[i] = ks_correct(p, d[i], w[i], w[i + 1], w[i + 2], w[i + 3], w[i + 4]);
        }
        if (x0 >= lo && x0 + 4 <= hi) {
            store_pairs(dst + x0, o);
            return;
        }
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            T l = w[i], c = w[i + 1], r = w[i + 2];
            if (p.bc != SW_BC_PERIODIC) {  // insulated ends, Heat1D_SweptShared.cu:140-142,352-353
                if (x0 + i == e.first) l = r;
                if (x0 + i == e.last) r = l;
            }
            o[i] = heat_step(p, l, c, r);
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
        if (x0 + i >= lo && x0 + i < hi) dst[x0 + i] = o[i];
}

// The classic Euler kernel's warp scheme (k_classic_euler): a warp takes 29
// cells at a time; lane l (cell b = s0 + l) loads cells b-2..b+1, forms
// D(b-2, b-1) and the interface (b-1, b) -- taking D(b-1, b) and D(b, b+1)
// from lanes l+1 and l+2 -- and adds its own interface minus the one of lane
// l+1.  Lanes 29..31 only feed lanes below them.
constexpr int kEulerCellsPerWarp = 29;

template <typename T>
__device__ __forceinline__ Q3<T> shfl_down3(Q3<T> v, int d) {
    return q3(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d),
              __shfl_down_sync(0xffffffffu, v.z, d));
}

// FP32 Euler levels keep the warp scheme: an FP32 tile is bound by instruction
// issue, where three passes with a barrier after each cost more than the 3 lanes
// of 32 they save (0.95x against 1.01x of classic, nx = 2^22).  Values read
// past W + R - 1 (clamped) only reach lanes whose cells are not stored.
template <typename T>
__device__ __forceinline__ void euler_level_warp(const Params<T> &p, T *rows, int L, int W, int par, int lo, int hi,
                                                 Ends e) {
    constexpr int R = Scheme<SW_EULER, T>::R;
    const T *src = rows + (par ^ 1) * 3 * L + R;
    T *dst = rows + par * 3 * L + R;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const T scale = par ? ml(T(0.25), p.dtdx) : ml(T(0.5), p.dtdx);
    for (int s0 = lo + warp * kEulerCellsPerWarp; s0 < hi; s0 += nwarp * kEulerCellsPerWarp) {
        const int b = s0 + lane;
        Q3<T> c[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int x = min(b - 2 + k, W + R - 1);
            c[k] = q3(src[x], src[L + x], src[2 * L + x]);
        }
        // zero across the domain's ends (the reference's edge flags, Euler1D_SweptShared.cu:311-335)
        const T D = (b - 1 == e.first || b - 2 == e.last) ? T(0) : eu_pdiff(c[0], c[1]);
        const T D1 = __shfl_down_sync(0xffffffffu, D, 1), D2 = __shfl_down_sync(0xffffffffu, D, 2);
        Q3<T> F, S;
        eu_iface(p, c[0], c[1], c[2], c[3], D, D1, D2, F, S);
        const Q3<T> Fr = shfl_down3(F, 1), Sr = shfl_down3(S, 1);
        if (lane < kEulerCellsPerWarp && b < hi && b != e.first && b != e.last) {
            const Q3<T> base = par ? c[2] : q3(dst[b], dst[L + b], dst[2 * L + b]);
            const Q3<T> o = qadd(base, qscale(scale, eu_combine(F, S, Fr, Sr)));
            dst[b] = o.x;
            dst[L + b] = o.y;
            dst[2 * L + b] = o.z;
        }
    }
}

// Euler sub-step over tile cells [lo, hi) of a swept tile, every interface
// computed once, in three passes of the whole block through shared memory
// (xs: kEulerIfaceArrays rows of L values after the tile rows):
//   A. the pressure-difference numerator D_k of each neighbour pair (k-1, k),
//      k in [lo-1, hi+2) -- zero across the domain's ends (the reference's
//      edge flags, Euler1D_SweptShared.cu:311-335);
//   B. the flux F_b and dissipation S_b of each interface (b-1, b), b in
//      [lo, hi+1), from the four cells around it and D_{b-1}, D_b, D_{b+1};
//   C. each cell's update from its two interfaces (eu_combine).
// Same operations on the same values as the classic kernel's warp scheme
// (and so as the reference's per-cell form), but every lane of pass B
// computes an interface that is used, where 29-cell warps spend 3 lanes of 32
// on terms only their neighbours need.  The cells read lie in [lo-2, hi+1],
// inside the row and its margins: the down part's widest level reads row 1's
// imported cells -2 .. W+1.
template <typename T>
__device__ __forceinline__ void euler_level_tile(const Params<T> &p, T *rows, int L, int par, int lo, int hi, Ends e) {
    constexpr int R = Scheme<SW_EULER, T>::R;
    const T *src = rows + (par ^ 1) * 3 * L + R;
    T *dst = rows + par * 3 * L + R;
    T *D = rows + 6 * L + R;  // D[k], F[c * L + b], S[c * L + b] at tile position k, b
    T *F = D + L, *S = D + 4 * L;
    const int t0 = (int)threadIdx.x, nt = (int)blockDim.x;
    for (int k = lo - 1 + t0; k < hi + 2; k += nt) {
        const Q3<T> a = q3(src[k - 1], src[L + k - 1], src[2 * L + k - 1]);
        const Q3<T> b = q3(src[k], src[L + k], src[2 * L + k]);
        D[k] = (k == e.first || k - 1 == e.last) ? T(0) : eu_pdiff(a, b);
    }
    __syncthreads();
    for (int b = lo + t0; b < hi + 1; b += nt) {
        Q3<T> c[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) c[k] = q3(src[b - 2 + k], src[L + b - 2 + k], src[2 * L + b - 2 + k]);
        Q3<T> f, g;
        eu_iface(p, c[0], c[1], c[2], c[3], D[b - 1], D[b], D[b + 1], f, g);
        F[b] = f.x;
        F[L + b] = f.y;
        F[2 * L + b] = f.z;
        S[b] = g.x;
        S[L + b] = g.y;
        S[2 * L + b] = g.z;
    }
    __syncthreads();
    const T scale = par ? ml(T(0.25), p.dtdx) : ml(T(0.5), p.dtdx);
    for (int b = lo + t0; b < hi; b += nt) {
        if (b == e.first || b == e.last) continue;
        const Q3<T> fl = q3(F[b], F[L + b], F[2 * L + b]), sl = q3(S[b], S[L + b], S[2 * L + b]);
        const Q3<T> fr = q3(F[b + 1], F[L + b + 1], F[2 * L + b + 1]), sr = q3(S[b + 1], S[L + b + 1], S[2 * L + b + 1]);
        const Q3<T> base = par ? q3(src[b], src[L + b], src[2 * L + b]) : q3(dst[b], dst[L + b], dst[2 * L + b]);
        const Q3<T> o = qadd(base, qscale(scale, eu_combine(fl, sl, fr, sr)));
        dst[b] = o.x;
        dst[L + b] = o.y;
        dst[2 * L + b] = o.z;
    }
}

// Heat / KS cells [lo, hi) of one level, one per thread from the lowest thread,
// so the live cells start at thread 0: whole warps idle, not part-empty ones.
// A block with a thread for every tile cell needs one pass (hi - lo <= W).
// Returns the thread's flagged cells (tile_point), bit i for its i-th cell (a
// thread has at most W / 32 <= 32 of them).
template <int P, typename T, int PATH>
__device__ __forceinline__ uint32_t tile_cells(const Params<T> &p, T *rows, int L, int W, int par, int lo, int hi,
                                               Ends e) {
    uint32_t flagged = 0;
    if ((int)blockDim.x >= W) {
        const int x = lo + (int)threadIdx.x;
        if (x < hi) flagged = tile_point<P, T, PATH>(p, rows, L, par, x, e);
    } else {
        int i = 0;
        for (int x = lo + (int)threadIdx.x; x < hi; x += blockDim.x, ++i)
            flagged |= tile_point<P, T, PATH>(p, rows, L, par, x, e) << i;
    }
    return flagged;
}
template <int P, typename T, int PATH>
__device__ __forceinline__ void tile_cells_fix(const Params<T> &p, T *rows, int L, int par, int lo, int hi, Ends e,
                                               uint32_t flagged) {
    if constexpr (int_products<P, T, PATH>()) {
        for (int x = lo + (int)threadIdx.x; x < hi && flagged; x += blockDim.x, flagged >>= 1)
            if (flagged & 1u) tile_point_pipe<P, T>(p, rows, L, par, x, e);
    }
}

// One sub-step of parity `par` on tile cells [lo, hi).
// Returns the thread's flagged cells (tile_cells).
template <int P, typename T, int PATH>
__device__ __forceinline__ uint32_t tile_level(const Params<T> &p, T *rows, int L, int W, int par, int lo, int hi,
                                               Ends e) {
    if constexpr (P == SW_EULER) {
        if constexpr (sizeof(T) == 8) euler_level_tile<T>(p, rows, L, par, lo, hi, e);
        else euler_level_warp<T>(p, rows, L, W, par, lo, hi, e);
    } else if constexpr (PATH == PATH_SPAN4) {
        tile_span4<P, T>(p, rows, L, par, lo, hi, e, (int)threadIdx.x);
    } else if constexpr (PATH == PATH_CELL || PATH == PATH_CELL_FP) {
        return tile_cells<P, T, PATH>(p, rows, L, W, par, lo, hi, e);
    } else {
        if ((int)blockDim.x * 4 == W) {
            tile_span4<P, T>(p, rows, L, par, lo, hi, e, (int)threadIdx.x);
        } else {
            return tile_cells<P, T, PATH>(p, rows, L, W, par, lo, hi, e);
        }
    }
    return 0;
}
// A Heat / KS level and the barrier after it.
template <int P, typename T, int PATH>
__device__ __forceinline__ void tile_level_sync(const Params<T> &p, T *rows, int L, int W, int par, int lo, int hi,
                                                Ends e) {
    const uint32_t flagged = tile_level<P, T, PATH>(p, rows, L, W, par, lo, hi, e);
    level_barrier<P, T, PATH>(flagged, [&] { tile_cells_fix<P, T, PATH>(p, rows, L, par, lo, hi, e, flagged); });
}

// Heat and KS take the level loops two levels at a time, so each level's
// parity (which row it reads and which it writes) is a constant; H = W / 2R is
// even, W being a multiple of 32.  Euler's long levels gain nothing from it and
// its persistent kernels would spill, so it keeps one level per iteration.
// Down part: sub-steps j = 1..H on the growing centre [W/2 - jR, W/2 + jR).
template <int P, typename T, int PATH = PATH_ANY>
__device__ __forceinline__ void tile_down(const Params<T> &p, T *rows, int L, int W, int64_t base) {
    constexpr int R = Scheme<P, T>::R;
    const int h = W >> 1, H = W / (2 * R);
    const Ends e = tile_ends(base, p.nx, W, R);
    if constexpr (P == SW_EULER) {
        for (int j = 1; j <= H; ++j) {
            tile_level<P, T, PATH>(p, rows, L, W, j & 1, h - j * R, h + j * R, e);
            __syncthreads();
        }
        return;
    }
    for (int j = 1; j < H; j += 2) {
        tile_level_sync<P, T, PATH>(p, rows, L, W, 1, h - j * R, h + j * R, e);
        tile_level_sync<P, T, PATH>(p, rows, L, W, 0, h - (j + 1) * R, h + (j + 1) * R, e);
    }
}
// Up part: sub-steps u = 1..H-1 on the shrinking [uR, W - uR).
template <int P, typename T, int PATH = PATH_ANY>
__device__ __forceinline__ void tile_up(const Params<T> &p, T *rows, int L, int W, int64_t base) {
    constexpr int R = Scheme<P, T>::R;
    const int H = W / (2 * R);
    const Ends e = tile_ends(base, p.nx, W, R);
    if constexpr (P == SW_EULER) {
        for (int u = 1; u < H; ++u) {
            tile_level<P, T, PATH>(p, rows, L, W, u & 1, u * R, W - u * R, e);
            __syncthreads();
        }
        return;
    }
    int u = 1;
    for (; u + 1 < H; u += 2) {
        tile_level_sync<P, T, PATH>(p, rows, L, W, 1, u * R, W - u * R, e);
        tile_level_sync<P, T, PATH>(p, rows, L, W, 0, (u + 1) * R, W - (u + 1) * R, e);
    }
    tile_level_sync<P, T, PATH>(p, rows, L, W, 1, u * R, W - u * R, e);  // u = H - 1, odd
}

// Default threads per swept block.  FP32 Heat / KS run 4 contiguous cells per
// thread from 128-cell tiles up (the vector path), FP64 one cell per thread
// (two on 1024-cell tiles): the FP64 pipe, not shared memory, bounds FP64 and
// it wants the warps.  Euler walks W / 256 cells.
template <int P, typename T>
__host__ __device__ constexpr int swept_threads(int W) {
    if (P == SW_EULER) return W < Scheme<P, T>::MAXT ? W : Scheme<P, T>::MAXT;
    if (sizeof(T) == 4) return W >= 128 ? W / 4 : W;
    return W <= Scheme<P, T>::MAXT ? W : Scheme<P, T>::MAXT;
}

// threads per swept block for a request (0 or out of range = the default)
template <int P, typename T>
inline int swept_threads_for(int W, int threads) {
    if (threads < 32 || threads > Scheme<P, T>::MAXT || threads > W || (threads & 31)) return swept_threads<P, T>(W);
    return threads;
}

// One swept pass of tile t of a periodic / bounded domain of p.nx cells whose
// state and slots start at `state` and `slots`.  MODE_UP: state ->
// up-triangle -> slots (phase 0 only).  MODE_DIAMOND: slots -> down + up ->
// slots.  MODE_DOWN: slots -> down-triangle -> state.
template <int P, typename T, int MODE, int PATH = PATH_ANY>
__device__ __forceinline__ void swept_tile(const Params<T> &p, typename Scheme<P, T>::G *__restrict__ state,
                                           typename Scheme<P, T>::G *__restrict__ slots, T *rows, const int W,
                                           const int phase, const int64_t t) {
    const int L = row_stride(W), h = W >> 1;
    const int64_t nx = p.nx, nhalf = nx / h;
    const int64_t base = t * W + (int64_t)phase * h;
    const int64_t hl = (2 * t + phase) % nhalf;
    const int64_t hr = (hl + 1 == nhalf) ? 0 : hl + 1;

    if constexpr (MODE == MODE_UP) {
        for (int x = threadIdx.x; x < W; x += blockDim.x) tile_put<P, T>(rows, L, 0, x, state[base + x]);
    } else {
        tile_import<P, T>(rows, L, W, slots + hl * W, slots + hr * W);
    }
    if constexpr (P == SW_EULER) {
        __syncthreads();
        tile_fix_bc<P, T>(p, rows, L, base);
    }
    __syncthreads();
    if constexpr (MODE != MODE_UP) tile_down<P, T, PATH>(p, rows, L, W, base);
    if constexpr (MODE == MODE_DOWN) {
        for (int x = threadIdx.x; x < W; x += blockDim.x) state[wrap_pos(base + x, nx)] = tile_get<P, T>(rows, L, 0, x);
    } else {
        tile_up<P, T, PATH>(p, rows, L, W, base);
        tile_export<P, T>(rows, L, W, slots + hl * W, slots + hr * W);
    }
}

// One swept pass over all tiles of one domain; block = one tile.
// FP32 four-cells-per-thread blocks ask for 2048 resident threads per SM (32 registers).
// FP64 Euler tiles (256 threads) ask for SW_EULER_MIN_BLOCKS blocks per SM: an
// Euler level is three passes with a barrier after each, and other blocks'
// warps keep the FP64 pipe busy through them.
#ifndef SW_EULER_MIN_BLOCKS
#define SW_EULER_MIN_BLOCKS 3
#endif
template <int P, typename T, int PATH>
constexpr int swept_min_blocks() {
    if (P == SW_EULER) return sizeof(T) == 8 ? SW_EULER_MIN_BLOCKS : 1;
    return (PATH == PATH_SPAN4 && sizeof(T) == 4) ? 2048 / Scheme<P, T>::MAXT : 1;
}
template <int P, typename T, int MODE, int PATH>
__global__ void __launch_bounds__(Scheme<P, T>::MAXT, (swept_min_blocks<P, T, PATH>()))
    k_swept(const Params<T> p, typename Scheme<P, T>::G *__restrict__ state,
                                                typename Scheme<P, T>::G *__restrict__ slots, const int W,
                                                const int phase) {
    extern __shared__ __align__(16) unsigned char sw_smem[];
    swept_tile<P, T, MODE, PATH>(p, state, slots, reinterpret_cast<T *>(sw_smem), W, phase, (int64_t)blockIdx.x);
}

// One classic sub-step at cell g of a domain of p.nx cells: classicHeat
// (Heat1D_SweptShared.cu:132-145), classicKS (KS1D_SweptShared.cu:189-207),
// classicEuler (Euler1D_SweptShared.cu:400-426).
// A KS cell of the classic step on the FP64 pipe alone (a cell whose
// integer-pipe products were flagged, as in tile_point).
template <typename T>
__device__ __noinline__ void classic_ks_pipe(const Params<T> &p, const T *__restrict__ in, T *__restrict__ out,
                                             const int sub, const int64_t g) {
    const int64_t nx = p.nx;
    T v[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) v[k] = in[wrap_pos(g - 2 + k, nx)];
    out[g] = sub == 0 ? ks_predict(p, v[0], v[1], v[2], v[3], v[4]) : ks_correct(p, out[g], v[0], v[1], v[2], v[3], v[4]);
}
template <typename T>
__device__ __noinline__ void classic_heat_pipe(const Params<T> &p, const T *__restrict__ in, T *__restrict__ out,
                                               const int64_t l, const int64_t g, const int64_t r) {
    out[g] = heat_step(p, in[l], in[g], in[r]);
}
template <int P, typename T>
__device__ __forceinline__ void classic_cell(const Params<T> &p, const typename Scheme<P, T>::G *__restrict__ in,
                                             typename Scheme<P, T>::G *__restrict__ out, const int sub,
                                             const int64_t g) {
    const int64_t nx = p.nx;
    if constexpr (P == SW_HEAT) {
        int64_t l = g - 1, r = g + 1;
        if (p.bc == SW_BC_PERIODIC) {
            if (l < 0) l = nx - 1;
            if (r == nx) r = 0;
        } else {
            if (g == 0) l = 1;
            if (g == nx - 1) r = nx - 2;
        }
        if constexpr (int_products<P, T>()) {  // both products on the integer pipe (tile_point)
            uint32_t bad = 0;
            const T o = heat_step_q(p, in[l], in[g], in[r], bad);
            if (__any_sync(__activemask(), bad != 0) && bad) classic_heat_pipe(p, in, out, l, g, r);
            else out[g] = o;
        } else {
            out[g] = heat_step(p, in[l], in[g], in[r]);
        }
    } else if constexpr (P == SW_KS) {
        T v[5];
        if (g >= 2 && g < nx - 2) {  // interior: no wrap
#pragma unroll
            for (int k = 0; k < 5; ++k) v[k] = in[g - 2 + k];
        } else {
#pragma unroll
            for (int k = 0; k < 5; ++k) v[k] = in[wrap_pos(g - 2 + k, nx)];
        }
        if constexpr (int_products<P, T>()) {  // the three products on the integer pipe (tile_point)
            uint32_t bad = 0;
            const T l2 = mlq(v[1], v[1], bad), r2 = mlq(v[3], v[3], bad);
            const T o = sub == 0 ? ks_predict_q(p, v[0], v[1], v[2], v[3], v[4], l2, r2, bad)
                                 : ks_correct_q(p, out[g], v[0], v[1], v[2], v[3], v[4], l2, r2, bad);
            if (__any_sync(__activemask(), bad != 0) && bad) classic_ks_pipe(p, in, out, sub, g);
            else out[g] = o;
        } else if (sub == 0) {
            out[g] = ks_predict(p, v[0], v[1], v[2], v[3], v[4]);
        } else {
            out[g] = ks_correct(p, out[g], v[0], v[1], v[2], v[3], v[4]);
        }
    } else {
        if (g == 0 || g == nx - 1) {
            const int side = (g == 0) ? 0 : 1;
            out[g] = V4<T>{p.bd[3 * side], p.bd[3 * side + 1], p.bd[3 * side + 2], T(0)};
            return;
        }
        Q3<T> s[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            int64_t q = g - 2 + k;
            q = q < 0 ? 0 : (q >= nx ? nx - 1 : q);  // only read when the edge flags let them matter
            const V4<T> v = in[q];
            s[k] = q3(v.x, v.y, v.z);
        }
        const bool fl = (g == 1), fr = (g == nx - 2);
        Q3<T> o;
        if (sub == 0) {
            o = eu_predict(p, s, fl, fr);
        } else {
            const V4<T> u = out[g];
            o = eu_correct(p, q3(u.x, u.y, u.z), s, fl, fr);
        }
        out[g] = V4<T>{o.x, o.y, o.z, T(0)};
    }
}

template <int P, typename T>
__global__ void __launch_bounds__(Scheme<P, T>::CMAXT) k_classic(const Params<T> p, const typename Scheme<P, T>::G *__restrict__ in,
                                                  typename Scheme<P, T>::G *__restrict__ out, const int sub) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g < p.nx) classic_cell<P, T>(p, in, out, sub, g);
}

// Classic Euler sub-step with shared interfaces (the warp scheme above over
// the whole domain, 29 cells per warp).  Cells 0 and nx-1
// hold the Dirichlet states (classicEuler, Euler1D_SweptShared.cu:400-426).
template <typename T>
__global__ void __launch_bounds__(256) k_classic_euler(const Params<T> p, const V4<T> *__restrict__ in,
                                                       V4<T> *__restrict__ out, const int sub) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t b = warp * kEulerCellsPerWarp + lane, nx = p.nx;
    Q3<T> c[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int64_t q = b - 2 + k;
        q = q < 0 ? 0 : (q >= nx ? nx - 1 : q);  // clamped values only reach cells that are not stored
        const V4<T> v = in[q];
        c[k] = q3(v.x, v.y, v.z);
    }
    const T D = (b - 1 == 0 || b - 2 == nx - 1) ? T(0) : eu_pdiff(c[0], c[1]);
    const T D1 = __shfl_down_sync(0xffffffffu, D, 1), D2 = __shfl_down_sync(0xffffffffu, D, 2);
    Q3<T> F, S;
    eu_iface(p, c[0], c[1], c[2], c[3], D, D1, D2, F, S);
    const Q3<T> Fr = shfl_down3(F, 1), Sr = shfl_down3(S, 1);
    if (lane >= kEulerCellsPerWarp || b >= nx) return;
    if (b == 0 || b == nx - 1) {
        const int side = (b == 0) ? 0 : 1;
        out[b] = V4<T>{p.bd[3 * side], p.bd[3 * side + 1], p.bd[3 * side + 2], T(0)};
        return;
    }
    Q3<T> base = c[2];
    T scale = ml(T(0.25), p.dtdx);
    if (sub) {
        const V4<T> u = out[b];
        base = q3(u.x, u.y, u.z);
        scale = ml(T(0.5), p.dtdx);
    }
    const Q3<T> o = qadd(base, qscale(scale, eu_combine(F, S, Fr, Sr)));
    out[b] = V4<T>{o.x, o.y, o.z, T(0)};
}

// Euler host layout (rho, rho u, E) <-> device layout (rho, rho u, E, 0).
template <typename T>
__global__ void k_pack3(const T *__restrict__ in3, V4<T> *__restrict__ out4, int64_t nx) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g < nx) out4[g] = V4<T>{in3[3 * g], in3[3 * g + 1], in3[3 * g + 2], T(0)};
}
template <typename T>
__global__ void k_unpack3(const V4<T> *__restrict__ in4, T *__restrict__ out3, int64_t nx) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g < nx) {
        const V4<T> v = in4[g];
        out3[3 * g] = v.x;
        out3[3 * g + 1] = v.y;
        out3[3 * g + 2] = v.z;
    }
}

// ------------------------------------------------ G tiles per block (Heat, KS)
// An FP64 warp instruction holds its SM sub-partition's FP64 pipe for the same
// time whatever number of its lanes are active (a probe measured 64 cycles per
// DADD for 1 to 32 lanes), so the part-empty top warp of every level costs a
// full warp of FP64 time (and an issue slot in FP32).  A block holds tiles
// t0 .. t0 + G - 1 and packs the G tiles' live cells of a level, the same
// count for each, onto its lowest threads: one part-empty warp per level
// instead of G.  PATH_CELL: one cell per thread (G*W threads); PATH_SPAN4: four
// cells per thread (G*W/4 threads).  Same cells, same arithmetic as swept_tile.
template <int G>
__device__ __forceinline__ int group_slot(int t, int n) {
    int k = 0;
#pragma unroll
    for (int q = 1; q < G; ++q) k += (t >= q * n) ? 1 : 0;
    return k;
}
template <int P, typename T, int G, int PATH>
__device__ __forceinline__ uint32_t group_level(const Params<T> &p, T *rows, int TS, int L, int par, int lo, int hi,
                                                const Ends (&e)[G]) {
    // threads per tile at this level
    const int n = (PATH == PATH_SPAN4) ? ((hi - (lo & ~3) + 3) >> 2) : (hi - lo);
    const int t = (int)threadIdx.x;
    if (t < G * n) {
        const int k = group_slot<G>(t, n);
        Ends ek = e[0];
#pragma unroll
        for (int q = 1; q < G; ++q)
            if (k == q) ek = e[q];
        if constexpr (PATH == PATH_SPAN4) tile_span4<P, T>(p, rows + k * TS, L, par, lo, hi, ek, t - k * n);
        else return tile_point<P, T, PATH>(p, rows + k * TS, L, par, lo + t - k * n, ek);
    }
    return 0;
}
// A grouped level and the barrier after it (level_barrier); the extra() of the
// last level (the fence before the bulk export) runs before that barrier.
template <int P, typename T, int G, int PATH, typename Extra>
__device__ __forceinline__ void group_level_sync(const Params<T> &p, T *rows, int TS, int L, int par, int lo, int hi,
                                                 const Ends (&e)[G], Extra &&extra) {
    const uint32_t flagged = group_level<P, T, G, PATH>(p, rows, TS, L, par, lo, hi, e);
    extra();
    level_barrier<P, T, PATH>(flagged, [&] {
        if (flagged) {
            const int n = hi - lo, t = (int)threadIdx.x, k = group_slot<G>(t, n);
            Ends ek = e[0];
#pragma unroll
            for (int q = 1; q < G; ++q)
                if (k == q) ek = e[q];
            tile_point_pipe<P, T>(p, rows + k * TS, L, par, lo + t - k * n, ek);
        }
        extra();
    });
}
template <int P, typename T, int G, int PATH>
__device__ __forceinline__ void group_level_sync(const Params<T> &p, T *rows, int TS, int L, int par, int lo, int hi,
                                                 const Ends (&e)[G]) {
    group_level_sync<P, T, G, PATH>(p, rows, TS, L, par, lo, hi, e, [] {});
}

// FP64 KS tiles move their slots (and the up-triangle its state) by bulk
// copy: with R = 2 cells of 8 bytes, every piece of a tile's import and
// export starts on a 16-byte boundary in both memories.  One thread issues
// the copies (4 per tile, or 1 per tile from the state) on one mbarrier; the
// squares rows that the one-cell path reads are then formed from the
// imported values, as tile_put forms them.
#ifndef SW_GROUP_BULK
#define SW_GROUP_BULK 1  // 0: the per-thread import and export instead (a build for comparison)
#endif
template <int P, typename T, int PATH>
__host__ __device__ constexpr bool group_bulk() {
    return SW_GROUP_BULK && P == SW_KS && sizeof(T) == 8 && PATH == PATH_CELL;
}

template <int P, typename T, int MODE, int G>
__device__ __forceinline__ bool group_bulk_import(const Params<T> &p, const T *state, const T *slots, T *rows, int TS,
                                                  int L, int W, const int64_t (&base)[G], const int64_t (&hl)[G],
                                                  const int64_t (&hr)[G]) {
    constexpr int R = Scheme<P, T>::R;
    const int h = W >> 1;
    __shared__ alignas(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned piece = (unsigned)(h * sizeof(T));
        mbar_expect_tx(&bar, (unsigned)(G * W * (MODE == MODE_UP ? 1 : 2) * sizeof(T)));
#pragma unroll
        for (int k = 0; k < G; ++k) {
            T *rk = rows + k * TS;
            if constexpr (MODE == MODE_UP) {
                bulk_load(rk + R, state + base[k], 2 * piece, &bar);  // row 0, cells 0 .. W-1
            } else {
                const T *sl = slots + hl[k] * W, *sr = slots + hr[k] * W;
                bulk_load(rk + R, sl, piece, &bar);                  // row 0, cells 0 .. h-1
                bulk_load(rk + L, sl + h, piece, &bar);              // row 1, cells -R .. h-R-1
                bulk_load(rk + R + h, sr, piece, &bar);              // row 0, cells h .. W-1
                bulk_load(rk + L + h + 2 * R, sr + h, piece, &bar);  // row 1, cells h+R .. W+R-1
            }
        }
    }
    if (!bulk_wait(&bar, p.status)) return false;
    // squares of the imported cells (rows 2 and 3)
    for (int i = threadIdx.x; i < G * W; i += blockDim.x) {
        const int k = i / W, x = i - k * W;
        T *rk = rows + k * TS;
        const T v0 = rk[R + x];
        rk[2 * L + R + x] = ml(v0, v0);
        if constexpr (MODE != MODE_UP) {
            const int c = x < h ? x - R : x + R;  // row 1's imported cells
            const T v1 = rk[L + R + c];
            rk[3 * L + R + c] = ml(v1, v1);
        }
    }
    return true;
}

template <int P, typename T, int G>
__device__ __forceinline__ void group_bulk_export(T *slots, T *rows, int TS, int L, int W, const int64_t (&hl)[G],
                                                  const int64_t (&hr)[G]) {
    constexpr int R = Scheme<P, T>::R;
    const int h = W >> 1;
    // the caller's last level fenced every thread's row writes and synchronised
    if (threadIdx.x == 0) {
        const unsigned piece = (unsigned)(h * sizeof(T));
#pragma unroll
        for (int k = 0; k < G; ++k) {
            const T *rk = rows + k * TS;
            T *sl = slots + hl[k] * W, *sr = slots + hr[k] * W;
            bulk_store(sl, rk + R, piece);                  // row 0, cells 0 .. h-1
            bulk_store(sl + h, rk + L + 2 * R, piece);      // row 1, cells R .. h+R-1
            bulk_store(sr, rk + R + h, piece);              // row 0, cells h .. W-1
            bulk_store(sr + h, rk + L + h, piece);          // row 1, cells h-R .. W-R-1
        }
        bulk_store_commit_and_wait();  // complete before the block's shared memory goes
    }
}

template <int P, typename T, int MODE, int G, int PATH>
__device__ __forceinline__ void swept_tile_group(const Params<T> &p, T *__restrict__ state, T *__restrict__ slots,
                                                 T *rows, const int W, const int phase, const int64_t t0) {
    static_assert(P != SW_EULER, "Euler tiles are not grouped");
    constexpr int R = Scheme<P, T>::R;
    const int L = row_stride(W), h = W >> 1, H = W / (2 * R), TS = tile_rows<P>() * L;
    const int64_t nx = p.nx, nhalf = nx / h;
    int64_t base[G], hl[G], hr[G];
    Ends e[G];
#pragma unroll
    for (int k = 0; k < G; ++k) {
        base[k] = (t0 + k) * W + (int64_t)phase * h;
        hl[k] = (2 * (t0 + k) + phase) % nhalf;
        hr[k] = (hl[k] + 1 == nhalf) ? 0 : hl[k] + 1;
        e[k] = tile_ends(base[k], nx, W, R);
    }
    // import / export: element i of the block is element i % W of tile i / W
    if constexpr (group_bulk<P, T, PATH>()) {
        if (!group_bulk_import<P, T, MODE, G>(p, state, slots, rows, TS, L, W, base, hl, hr)) return;
    } else {
        for (int i = threadIdx.x; i < G * W; i += blockDim.x) {
            const int k = i / W, x = i - k * W;
            if constexpr (MODE == MODE_UP) tile_put<P, T>(rows + k * TS, L, 0, x, state[base[k] + x]);
            else tile_import_at<P, T>(rows + k * TS, L, W, slots + hl[k] * W, slots + hr[k] * W, x);
        }
    }
    __syncthreads();
    if constexpr (MODE != MODE_UP) {  // down part, two levels per iteration (H is even)
        for (int j = 1; j < H; j += 2) {
            group_level_sync<P, T, G, PATH>(p, rows, TS, L, 1, h - j * R, h + j * R, e);
            group_level_sync<P, T, G, PATH>(p, rows, TS, L, 0, h - (j + 1) * R, h + (j + 1) * R, e);
        }
    }
    if constexpr (MODE == MODE_DOWN) {
        for (int i = threadIdx.x; i < G * W; i += blockDim.x) {
            const int k = i / W, x = i - k * W;
            state[wrap_pos(base[k] + x, nx)] = tile_get<P, T>(rows + k * TS, L, 0, x);
        }
    } else {
        int u = 1;
        for (; u + 1 < H; u += 2) {
            group_level_sync<P, T, G, PATH>(p, rows, TS, L, 1, u * R, W - u * R, e);
            group_level_sync<P, T, G, PATH>(p, rows, TS, L, 0, (u + 1) * R, W - (u + 1) * R, e);
        }
        if constexpr (group_bulk<P, T, PATH>()) {
            // u = H - 1; each thread's row writes made visible to the copy engine before the barrier
            group_level_sync<P, T, G, PATH>(p, rows, TS, L, 1, u * R, W - u * R, e, [] { fence_smem_for_bulk(); });
            group_bulk_export<P, T, G>(slots, rows, TS, L, W, hl, hr);
        } else {
            group_level_sync<P, T, G, PATH>(p, rows, TS, L, 1, u * R, W - u * R, e);  // u = H - 1
            for (int i = threadIdx.x; i < G * W; i += blockDim.x) {
                const int k = i / W, x = i - k * W;
                tile_export_at<P, T>(rows + k * TS, L, W, slots + hl[k] * W, slots + hr[k] * W, x);
            }
        }
    }
}

// Two 1024-thread blocks per SM (32 registers): the FP64 levels need the
// warps of both to keep the FP64 pipe fed across each level's barrier.
template <int P, typename T, int MODE, int G, int PATH>
__global__ void __launch_bounds__(1024, 2) k_swept_group(const Params<T> p, T *__restrict__ state,
                                                      T *__restrict__ slots, const int W, const int phase) {
    extern __shared__ __align__(16) unsigned char sw_smem[];
    swept_tile_group<P, T, MODE, G, PATH>(p, state, slots, reinterpret_cast<T *>(sw_smem), W, phase,
                                          G * (int64_t)blockIdx.x);
}

// Grouped tiles pay where blocks are plentiful: a domain of at least this many tiles.
constexpr int64_t kGroupMinTiles = 1024;

// ------------------------------------------------------------- launchers
// The dynamic shared-memory limit above the 48 KB default, set once per
// (launcher, device): the attribute belongs to the device that is current when
// it is set, so the record is a bit per device (devices 0..63; a higher index
// sets it on every call).  Setting it twice is harmless, so threads may race.
struct SmemOnce {
    std::atomic<uint64_t> done{0};
    template <typename... K>
    cudaError_t ensure(K... kernels) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        const uint64_t bit = (dev >= 0 && dev < 64) ? (uint64_t(1) << dev) : 0;
        if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
        for (auto k : {(const void *)kernels...}) {
            e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
            if (e != cudaSuccess) return e;
        }
        done.fetch_or(bit, std::memory_order_release);
        return cudaSuccess;
    }
};

template <int P, typename T>
cudaError_t launch_classic(const void *vp, const void *in, void *out, int sub, int64_t nx, int block,
                           cudaStream_t s) {
    using G = typename Scheme<P, T>::G;
    const Params<T> &p = *static_cast<const Params<T> *>(vp);
    if constexpr (P == SW_EULER) {
        const int64_t warps = (nx + kEulerCellsPerWarp - 1) / kEulerCellsPerWarp;
        k_classic_euler<T><<<(unsigned)((warps + 7) / 8), 256, 0, s>>>(p, static_cast<const G *>(in),
                                                                       static_cast<G *>(out), sub);
        return cudaGetLastError();
    }
    if (block <= 0 || block > Scheme<P, T>::CMAXT) block = block <= 0 ? 256 : Scheme<P, T>::CMAXT;
    const int64_t grid = (nx + block - 1) / block;
    k_classic<P, T><<<(unsigned)grid, block, 0, s>>>(p, static_cast<const G *>(in), static_cast<G *>(out), sub);
    return cudaGetLastError();
}

template <int P, typename T, int PATH>
cudaError_t launch_swept_path(const Params<T> &p, int mode, int phase, typename Scheme<P, T>::G *st,
                              typename Scheme<P, T>::G *sl, int64_t nx, int W, int threads, cudaStream_t s) {
    static SmemOnce once;
    cudaError_t e = once.ensure(k_swept<P, T, MODE_UP, PATH>, k_swept<P, T, MODE_DIAMOND, PATH>,
                                k_swept<P, T, MODE_DOWN, PATH>);
    if (e != cudaSuccess) return e;
    const size_t smem = swept_smem_bytes<P, T>(W);
    const unsigned grid = (unsigned)(nx / W);
    switch (mode) {
    case MODE_UP: k_swept<P, T, MODE_UP, PATH><<<grid, threads, smem, s>>>(p, st, sl, W, phase); break;
    case MODE_DIAMOND: k_swept<P, T, MODE_DIAMOND, PATH><<<grid, threads, smem, s>>>(p, st, sl, W, phase); break;
    default: k_swept<P, T, MODE_DOWN, PATH><<<grid, threads, smem, s>>>(p, st, sl, W, phase); break;
    }
    return cudaGetLastError();
}

// ------------------------------------------------ KS 128-cell tiles in one warp
// FP32 KS swept with W = 128: one warp per tile, 8 tiles per block, the tile's
// rows in registers -- lane l holds cells 4l .. 4l + 3 of row 0 (u) and row 1
// (the predictor u*) and their squares, and row-1 cells -2, -1, 128, 129 (read
// only by the last down level) sit in four more registers of every lane.  A
// cell's neighbours are the lane's own registers or the next lane's, by
// shuffles, so a level needs no barrier.  Slots, modes, level ranges and
// arithmetic (ks_*_sq) are those of swept_tile with W = 128: the results are
// the same bit for bit.
constexpr int kKsWarpTile = 128;
constexpr int kKsWarpTilesPerBlock = 8;

// One sub-step of parity `par` on tile cells [lo, hi).
template <typename T>
__device__ __forceinline__ void ks_warp4_level(const Params<T> &p, int par, int lo, int hi, T (&u0)[4], T (&u1)[4],
                                               T (&s0)[4], T (&s1)[4], const T (&m)[4], const T (&ms)[4]) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, c0 = 4 * lane;
    const T *src = par ? u0 : u1, *sq = par ? s0 : s1;
    // the previous lane's cells 2, 3 and square 3; the next lane's cells 0, 1 and square 0
    T pm2 = __shfl_up_sync(full, src[2], 1), pm1 = __shfl_up_sync(full, src[3], 1);
    T pq1 = __shfl_up_sync(full, sq[3], 1);
    T np0 = __shfl_down_sync(full, src[0], 1), np1 = __shfl_down_sync(full, src[1], 1);
    T nq0 = __shfl_down_sync(full, sq[0], 1);
    if (!par) {  // row-1 cells -2, -1 and 128, 129
        if (lane == 0) { pm2 = m[0]; pm1 = m[1]; pq1 = ms[1]; }
        if (lane == 31) { np0 = m[2]; np1 = m[3]; nq0 = ms[2]; }
    }
    const T w[8] = {pm2, pm1, src[0], src[1], src[2], src[3], np0, np1};  // cells c0 - 2 .. c0 + 5
    const T q[6] = {pq1, sq[0], sq[1], sq[2], sq[3], nq0};                // squares of cells c0 - 1 .. c0 + 4
    T v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
        v[k] = par ? ks_predict_sq(p, w[k], w[k + 1], w[k + 2], w[k + 3], w[k + 4], q[k], q[k + 2])
                   : ks_correct_sq(p, u0[k], w[k], w[k + 1], w[k + 2], w[k + 3], w[k + 4], q[k], q[k + 2]);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (c0 + k >= lo && c0 + k < hi) {
            if (par) { u1[k] = v[k]; s1[k] = ml(v[k], v[k]); }
            else { u0[k] = v[k]; s0[k] = ml(v[k], v[k]); }
        }
    }
}

template <typename T, int MODE>
__global__ void __launch_bounds__(32 * kKsWarpTilesPerBlock)
    k_swept_ks_warp(const Params<T> p, T *__restrict__ state, T *__restrict__ slots, const int phase,
                    const int64_t ntile) {
    constexpr int W = kKsWarpTile, h = W / 2, R = 2, H = W / (2 * R);
    const int lane = threadIdx.x & 31, c0 = 4 * lane;
    const int64_t nx = p.nx, nhalf = nx / h;  // ntile: the tiles launched (all, or all but the wrapping one)
    const int64_t t = (int64_t)blockIdx.x * kKsWarpTilesPerBlock + (threadIdx.x >> 5);
    if (t >= ntile) return;  // whole warps: t is the same for the 32 lanes
    const int64_t base = t * W + (int64_t)phase * h;
    const int64_t hl = (2 * t + phase) % nhalf;
    const int64_t hr = (hl + 1 == nhalf) ? 0 : hl + 1;
    T *sl = slots + hl * W, *sr = slots + hr * W;
    T u0[4], u1[4] = {T(0), T(0), T(0), T(0)}, m[4] = {T(0), T(0), T(0), T(0)};
    if constexpr (MODE == MODE_UP) {
#pragma unroll
        for (int k = 0; k < 4; ++k) u0[k] = state[base + c0 + k];
    } else {
        // slot layout as tile_import: sl = [row 0, cells 0..63][row 1, cells -2..61],
        // sr = [row 0, cells 64..127][row 1, cells 66..129]
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int c = c0 + k;
            u0[k] = c < h ? sl[c] : sr[c - h];
            if (c < h - R) u1[k] = sl[h + c + R];
            else if (c >= h + R) u1[k] = sr[c - R];
        }
        m[0] = sl[h];
        m[1] = sl[h + 1];
        m[2] = sr[W - 2];
        m[3] = sr[W - 1];
    }
    T s0[4], s1[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        s0[k] = ml(u0[k], u0[k]);
        s1[k] = ml(u1[k], u1[k]);
    }
    const T ms[4] = {ml(m[0], m[0]), ml(m[1], m[1]), ml(m[2], m[2]), ml(m[3], m[3])};
    if constexpr (MODE != MODE_UP) {
        for (int j = 1; j <= H; ++j) ks_warp4_level(p, j & 1, h - j * R, h + j * R, u0, u1, s0, s1, m, ms);
    }
    if constexpr (MODE == MODE_DOWN) {
#pragma unroll
        for (int k = 0; k < 4; ++k) state[wrap_pos(base + c0 + k, nx)] = u0[k];
    } else {
        for (int u = 1; u < H; ++u) ks_warp4_level(p, u & 1, u * R, W - u * R, u0, u1, s0, s1, m, ms);
        // as tile_export: sl[i] = row 0 cell i, sl[h + i] = row 1 cell R + i,
        // sr[j] = row 0 cell h + j, sr[h + j] = row 1 cell h - R + j
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int c = c0 + k;
            if (c < h) sl[c] = u0[k]; else sr[c - h] = u0[k];
            if (c >= R && c < h + R) sl[h + c - R] = u1[k];
            if (c >= h - R && c < W - R) sr[h + c - (h - R)] = u1[k];
        }
    }
}

template <int P, typename T, int G, int PATH>
cudaError_t launch_swept_group(const Params<T> &p, int mode, int phase, T *st, T *sl, int64_t nx, int W,
                               int threads, cudaStream_t s) {
    static SmemOnce once;
    cudaError_t e = once.ensure(k_swept_group<P, T, MODE_UP, G, PATH>, k_swept_group<P, T, MODE_DIAMOND, G, PATH>,
                                k_swept_group<P, T, MODE_DOWN, G, PATH>);
    if (e != cudaSuccess) return e;
    const size_t smem = G * swept_smem_bytes<P, T>(W);
    const unsigned grid = (unsigned)(nx / W / G);
    const int block = G * threads;
    switch (mode) {
    case MODE_UP: k_swept_group<P, T, MODE_UP, G, PATH><<<grid, block, smem, s>>>(p, st, sl, W, phase); break;
    case MODE_DIAMOND:
        k_swept_group<P, T, MODE_DIAMOND, G, PATH><<<grid, block, smem, s>>>(p, st, sl, W, phase);
        break;
    default: k_swept_group<P, T, MODE_DOWN, G, PATH><<<grid, block, smem, s>>>(p, st, sl, W, phase); break;
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_swept_ks_warp(const Params<T> &p, int mode, int phase, T *st, T *sl, int64_t nx, cudaStream_t s) {
    const int64_t ntile = nx / kKsWarpTile;
    const unsigned grid = (unsigned)((ntile + kKsWarpTilesPerBlock - 1) / kKsWarpTilesPerBlock);
    const int threads = 32 * kKsWarpTilesPerBlock;
    switch (mode) {
    case MODE_UP: k_swept_ks_warp<T, MODE_UP><<<grid, threads, 0, s>>>(p, st, sl, phase, ntile); break;
    case MODE_DIAMOND: k_swept_ks_warp<T, MODE_DIAMOND><<<grid, threads, 0, s>>>(p, st, sl, phase, ntile); break;
    default: k_swept_ks_warp<T, MODE_DOWN><<<grid, threads, 0, s>>>(p, st, sl, phase, ntile); break;
    }
    return cudaGetLastError();
}

// A domain of fewer tiles than two per SM of the current device: its levels'
// dependent chains are not hidden by other tiles' work (PATH_CELL_FP).
inline bool few_tiles(int64_t ntiles) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return false;
    return ntiles < 2 * (int64_t)sms;
}

template <int P, typename T>
cudaError_t launch_swept(const void *vp, int mode, int phase, void *state, void *slots, int64_t nx, int W,
                         int threads_req, cudaStream_t s) {
    using G = typename Scheme<P, T>::G;
    const Params<T> &p = *static_cast<const Params<T> *>(vp);
    const int threads = swept_threads_for<P, T>(W, threads_req);
    G *st = static_cast<G *>(state), *sl = static_cast<G *>(slots);
    if constexpr (P == SW_KS && sizeof(T) == 4) {  // 128-cell tiles: one warp each, rows in registers
        if (W == kKsWarpTile && threads == 32) return launch_swept_ks_warp<T>(p, mode, phase, st, sl, nx, s);
    }
    if constexpr (P != SW_EULER) {
        // The default shapes on a large domain: G tiles per block.  One cell per thread:
        // KS up to four tiles and 1024 threads; Heat, whose levels are four FP64
        // operations, two tiles and 512 threads (four measured 3 % slower than two).
        // Four cells per thread: tiles up to 256 cells only (KS four, Heat two; +6 % at
        // 256 cells), since at 1024 cells grouping measured 7 % (Heat) and 25 % (KS) slower.
        const int64_t ntiles = nx / W;
        const bool group = threads_req == 0 && ntiles >= kGroupMinTiles;
        if (threads * 4 == W) {
            if constexpr (sizeof(T) == 4) {  // FP64 defaults to a cell per thread: no grouped 4-cell kernels
                if (group && W <= 256 && P == SW_KS && ntiles % 4 == 0)
                    return launch_swept_group<P, T, 4, PATH_SPAN4>(p, mode, phase, st, sl, nx, W, threads, s);
                if (group && W <= 256 && ntiles % 2 == 0)
                    return launch_swept_group<P, T, 2, PATH_SPAN4>(p, mode, phase, st, sl, nx, W, threads, s);
            }
            return launch_swept_path<P, T, PATH_SPAN4>(p, mode, phase, st, sl, nx, W, threads, s);
        }
        constexpr int kMaxThreads = (P == SW_KS) ? 1024 : 512;
        if (group && threads == W) {
            if (P == SW_KS && 4 * W <= kMaxThreads && ntiles % 4 == 0)
                return launch_swept_group<P, T, 4, PATH_CELL>(p, mode, phase, st, sl, nx, W, threads, s);
            if (2 * W <= kMaxThreads && ntiles % 2 == 0)
                return launch_swept_group<P, T, 2, PATH_CELL>(p, mode, phase, st, sl, nx, W, threads, s);
        }
    }
    if constexpr (int_products<P, T>()) {
        if (few_tiles(nx / W)) return launch_swept_path<P, T, PATH_CELL_FP>(p, mode, phase, st, sl, nx, W, threads, s);
    }
    return launch_swept_path<P, T, PATH_CELL>(p, mode, phase, st, sl, nx, W, threads, s);
}

template <typename T>
cudaError_t launch_pack(const void *in3, void *out4, int64_t nx, cudaStream_t s) {
    k_pack3<T><<<(unsigned)((nx + 255) / 256), 256, 0, s>>>(static_cast<const T *>(in3), static_cast<V4<T> *>(out4),
                                                               nx);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_unpack(const void *in4, void *out3, int64_t nx, cudaStream_t s) {
    k_unpack3<T><<<(unsigned)((nx + 255) / 256), 256, 0, s>>>(static_cast<const V4<T> *>(in4), static_cast<T *>(out3),
                                                                 nx);
    return cudaGetLastError();
}

template <int P, typename T>
size_t smem_of(int W) {
    return swept_smem_bytes<P, T>(W);
}

SW_KERNELS_END
