// Internal interface between the C ABI (api.cu) and the per-problem kernel
// translation units (k_heat.cu, k_ks.cu, k_euler.cu).  Not installed.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/swept1d.h"

namespace sw {

// Kernel parameters: every constant of every scheme, in the run's precision.
// Passed by value (constant bank), so a launch never reads a __constant__
// symbol that another context might be rewriting.
template <typename T>
struct Params {
    T fo, fo2;                 // Heat: fourier, 1 - 2 fourier
    T c4, d2, d4, dt, dth;     // KS: 1/(4dx), 1/dx^2, 1/dx^4, dt, dt/2
    T gam, mgam, dtdx;         // Euler
    T bd[6];                   // Euler boundary states (rho, rho u, E) left, right
    int64_t nx;
    int bc;                    // SW_BC_MIRROR / PERIODIC / DIRICHLET
    int ks_form;               // KS: how c4, d2, d4 enter the right-hand side (enum KsForm)
    int d2_e;                  // KS_POW2: d2 = 2^d2_e
    T nz;                      // -0.0, the addend that makes an fma a plain product (paired FP32 path)
    int *status;               // device word a kernel sets when a bounded wait runs out (may be null)
};

// KS right-hand-side forms.  KS_POW2: c4, d2, d4 are exact powers of two, so
// their products fold into fused multiply-adds without changing a bit;
// KS_DIVIDE: c4, d2, d4 are the divisors 4dx, dx^2, dx^4 (SW_FLAG_KS_DIVIDE).
enum KsForm { KS_MULTIPLY = 0, KS_POW2 = 1, KS_DIVIDE = 2 };

// Device tables of an ensemble (see sw_run_batch): domain d holds cells
// [off[d], off[d+1]), its slots are the same range times two, its flags
// [2*tile0[d], ...); tile_dom maps a global tile of width W to its domain.
struct BatchDev {
    const int32_t *tile_dom;
    const int64_t *off;      // n_dom + 1 cell offsets
    const int64_t *tile0;    // first global tile of each domain
    const int32_t *blk_dom;  // domain of the first cell of each kClassicBlock-cell classic block
    int64_t n_tiles;
    int64_t n_cells;
    int32_t n_dom;
    int32_t group;  // the largest of 1, 2, 4 that divides every domain's tile count
};
constexpr int kClassicBlock = 256;  // threads (= cells) per block of the ensemble classic kernel

// Swept launch modes.
enum SweptMode { MODE_UP = 0, MODE_DIAMOND = 1, MODE_DOWN = 2 };

// Per (problem, precision) kernel table.  `params` points at a Params<T>
// of the table's precision.
struct Ops {
    int problem;
    int prec;        // 4 or 8
    int R;           // stencil radius per sub-step
    int S;           // sub-steps per time step
    int C;           // state components per cell on the host (1 or 3)
    size_t cell;     // bytes per cell in device layout
    int max_threads; // largest threads per block a swept kernel is built for
    // one classic sub-step (sub 0: predictor / heat step, 1: corrector)
    cudaError_t (*classic)(const void *params, const void *in, void *out, int sub, int64_t nx, int block,
                           cudaStream_t s);
    // one swept launch over all tiles of width W at `phase` (0 aligned, 1 shifted by W/2);
    // `threads` per block, 0 (or out of range) = the default for W
    cudaError_t (*swept)(const void *params, int mode, int phase, void *state, void *slots, int64_t nx, int W,
                         int threads, cudaStream_t s);
    // persistent swept variant: up-triangle, n_diamonds diamonds and the down-triangle in
    // one cooperative launch with per-half-tile phase flags; *status set non-zero on timeout.
    cudaError_t (*persistent)(const void *params, void *state, void *slots, unsigned *flags, int *status,
                              int64_t nx, int W, int threads, int64_t n_diamonds, cudaStream_t s);
    // Euler host layout (3 per cell) <-> device layout (4 per cell); null for Heat/KS
    cudaError_t (*pack)(const void *in3, void *out4, int64_t nx, cudaStream_t s);
    cudaError_t (*unpack)(const void *in4, void *out3, int64_t nx, cudaStream_t s);
    // dynamic shared memory a swept block of width W needs
    size_t (*swept_smem)(int W);
    // ensembles: `batch` points at a BatchDev (device tables), `threads` per block (0 = the default for W)
    cudaError_t (*batch_swept)(const void *params, int mode, int phase, void *state, void *slots, const void *batch,
                               int W, int threads, cudaStream_t s);
    cudaError_t (*batch_classic)(const void *params, const void *in, void *out, int sub, const void *batch, int block,
                                 cudaStream_t s);
    cudaError_t (*batch_persistent)(const void *params, void *state, void *slots, const void *batch, unsigned *flags,
                                    int *status, int W, int threads, int64_t n_diamonds, cudaStream_t s);
};

// The hybrid variant's host tile (host_tile.cu): the wrapping phase-1 tile of
// a domain computed on the CPU from its two slots (sl: the last half-tile's,
// sr: the first's); MODE_DIAMOND writes the slots back, MODE_DOWN the state's
// first and last half-tiles.  params: a Params<float or double>.
int host_tile_run(int problem, int prec, const void *params, int mode, void *sl, void *sr, void *state_first,
                  void *state_last, int W);

const Ops *heat_ops(int prec);
const Ops *ks_ops(int prec);
const Ops *ks_divide_ops(int prec);  // SW_FLAG_KS_DIVIDE (k_ks_div.cu)
const Ops *euler_ops(int prec);

inline const Ops *ops_for(int problem, int prec, int flags) {
    switch (problem) {
    case SW_HEAT: return heat_ops(prec);
    case SW_KS: return (flags & SW_FLAG_KS_DIVIDE) ? ks_divide_ops(prec) : ks_ops(prec);
    case SW_EULER: return euler_ops(prec);
    default: return nullptr;
    }
}

}  // namespace sw
