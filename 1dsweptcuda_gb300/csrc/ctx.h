// Context state shared by the C ABI translation units (api.cu, batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "sw_internal.h"

namespace sw {

struct BatchTables {          // device domain tables of the last ensemble shape
    std::vector<int64_t> nx;
    int W = -1;
    BatchDev dev{};
    void *d_tables = nullptr;
    size_t n_tables = 0;
};
struct GraphKey {             // what a captured ensemble graph was built for (compared bytewise)
    int problem, prec, alg, W, threads;
    int64_t n_steps;
    void *state, *slots, *tables, *work, *flags, *status;
    int64_t cells;
    unsigned char params[256];
};
struct GraphCache {
    cudaGraphExec_t exec = nullptr;
    GraphKey key;
    int64_t launches = 0;
};
struct TuneCache {
    bool valid = false;
    int problem = 0, prec = 0, alg = 0;
    std::vector<int64_t> nx;
    sw_tuning result;
};

inline cudaError_t grow_dev(void **p, size_t *cap, size_t need) {
    if (need <= *cap && *p) return cudaSuccess;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc(p, need);
    if (e == cudaSuccess) *cap = need;
    return e;
}
inline cudaError_t grow_pinned(void **p, size_t *cap, size_t need) {
    if (need <= *cap && *p) return cudaSuccess;
    if (*p) cudaFreeHost(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMallocHost(p, need);
    if (e == cudaSuccess) *cap = need;
    return e;
}

inline int resolved_bc(const sw_config &c) {
    if (c.bc != SW_BC_DEFAULT) return c.bc;
    return c.problem == SW_HEAT ? SW_BC_MIRROR : (c.problem == SW_KS ? SW_BC_PERIODIC : SW_BC_DIRICHLET);
}

template <typename T>
inline Params<T> make_params(const sw_config &c, const sw_constants &k) {
    Params<T> p{};
    p.fo = (T)k.fourier;
    p.fo2 = (T)k.fourier_two;
    p.c4 = (T)k.dx_times4;
    p.d2 = (T)k.dx2;
    p.d4 = (T)k.dx4;
    p.dt = (T)k.dt;
    p.dth = (T)k.dt_half;
    p.gam = (T)k.gam;
    p.mgam = (T)k.mgam;
    p.dtdx = (T)k.dt_dx;
    for (int i = 0; i < 6; ++i) p.bd[i] = (T)k.bd[i];
    p.nx = c.nx;
    p.bc = resolved_bc(c);
    p.nz = -T(0);
    auto is_pow2 = [](T v) {
        int e = 0;
        return v > T(0) && std::isfinite((double)v) && std::frexp((double)v, &e) == 0.5;
    };
    if (c.problem == SW_KS && (c.flags & SW_FLAG_KS_DIVIDE)) p.ks_form = KS_DIVIDE;
    else if (c.problem == SW_KS && is_pow2(p.c4) && is_pow2(p.d2) && is_pow2(p.d4)) p.ks_form = KS_POW2;
    else p.ks_form = KS_MULTIPLY;
    if (p.ks_form == KS_POW2) {
        int e = 0;
        std::frexp((double)p.d2, &e);  // d2 = 0.5 * 2^e
        p.d2_e = e - 1;
    }
    return p;
}

}  // namespace sw

struct sw_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr, k0 = nullptr, k1 = nullptr;
    void *d_state = nullptr;
    size_t n_state = 0;
    void *d_work = nullptr;
    size_t n_work = 0;
    void *d_slots = nullptr;
    size_t n_slots = 0;
    void *d_io = nullptr;
    size_t n_io = 0;
    unsigned *d_flags = nullptr;
    size_t n_flags = 0;
    int *d_status = nullptr;
    void *d_w2p = nullptr;  // closure layer-2 weights, BF16, in the kernels' shared-memory layout
    void *d_judge = nullptr;  // sw_closure_adaptive: the sample's rows, errors (run context) or fine shadow (judge)
    size_t n_judge = 0;
    void *h_pin = nullptr;
    size_t n_pin = 0;
    void *h_tile = nullptr;         // the hybrid variant's host tile: its two slots and two state pieces
    size_t n_tile = 0;
    cudaEvent_t tile_ready = nullptr;  // the host tile's slots have arrived in h_tile
    sw::BatchTables batch;
    sw::GraphCache graph;
    sw::TuneCache tune;
    std::string err;
};

inline int fail(sw_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->err = msg;
    return code;
}
inline int cuda_fail(sw_ctx *ctx, cudaError_t e, const char *where) {
    return fail(ctx, e == cudaErrorMemoryAllocation ? SW_ERR_NOMEM : SW_ERR_CUDA,
                std::string(where) + ": " + cudaGetErrorString(e));
}
#define SW_CUDA(ctx, call)                                         \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return cuda_fail((ctx), e_, #call); \
    } while (0)
