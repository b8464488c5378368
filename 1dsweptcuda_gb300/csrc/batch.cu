// Ensembles: many independent domains of uneven length advanced together
// (sw_run_batch, sw_run_batch_device), the launch sequence captured in a CUDA
// graph and replayed while its shape is unchanged, and the autotuner
// (sw_query_tuning) over tile width and threads per block.  No counterpart in
// the reference, which solves one domain per program run.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"
#include "sw_internal.h"

using namespace sw;

namespace {

constexpr int64_t kTuneCells = (int64_t)1 << 22;

bool valid_tile(int W, int32_t n, const int64_t *nx) {
    if (W < 32 || W > 1024 || (W & 31)) return false;
    for (int32_t d = 0; d < n; ++d)
        if (nx[d] < W || nx[d] % W) return false;
    return true;
}

// The checks sw_validate makes of one run, made for every domain: the
// problem's boundary condition and flags, and for Euler its stability limit.
// Every domain shares one set of constants (the kernels take one Params), so
// an Euler ensemble of uneven lengths must give dx: the reference's default
// dx = 1/(nx-2) would differ from domain to domain.
int check_batch(const sw_config *c, int32_t n, const int64_t *nx) {
    if (!c || !nx || n < 1) return SW_ERR_ARG;
    if (c->problem < SW_HEAT || c->problem > SW_EULER || (c->precision != 4 && c->precision != 8)) return SW_ERR_ARG;
    if (c->alg < SW_ALG_CLASSIC || c->alg > SW_ALG_VARIANT) return SW_ERR_ARG;
    if (c->time_mode != SW_TIME_STEPS || c->n_steps < 0 || !(c->dt > 0) || !std::isfinite(c->dt)) return SW_ERR_ARG;
    if ((c->flags & ~SW_FLAG_KS_DIVIDE) != 0) return SW_ERR_ARG;
    if ((c->flags & SW_FLAG_KS_DIVIDE) && c->problem != SW_KS) return SW_ERR_ARG;
    const int bc = resolved_bc(*c);
    if (c->problem == SW_HEAT && bc != SW_BC_MIRROR && bc != SW_BC_PERIODIC) return SW_ERR_ARG;
    if (c->problem == SW_KS && bc != SW_BC_PERIODIC) return SW_ERR_ARG;
    if (c->problem == SW_EULER && bc != SW_BC_DIRICHLET) return SW_ERR_ARG;
    for (int32_t d = 0; d < n; ++d)
        if (nx[d] < 32 || nx[d] > ((int64_t)1 << 34)) return SW_ERR_SIZE;
    if (c->tpb != 0 && c->alg != SW_ALG_CLASSIC && !valid_tile(c->tpb, n, nx)) return SW_ERR_SIZE;
    if (c->problem == SW_EULER) {
        if (c->dx == 0)
            for (int32_t d = 1; d < n; ++d)
                if (nx[d] != nx[0]) return SW_ERR_ARG;
        sw_config one = *c;
        one.nx = nx[0];
        sw_constants k;
        sw_constants_of(&one, &k);
        if (k.dt_dx > 0.21) return SW_ERR_UNSTABLE;  // Euler1D_SweptShared.cu:1168-1172
    }
    return SW_OK;
}

// Upload the domain tables for tile width W (kept while nx[] and W repeat).
int ensure_tables(sw_ctx *ctx, int32_t n, const int64_t *nx, int W) {
    BatchTables &bt = ctx->batch;
    if (bt.W == W && (int32_t)bt.nx.size() == n && std::equal(bt.nx.begin(), bt.nx.end(), nx)) return SW_OK;
    std::vector<int64_t> off(n + 1), tile0(n);
    std::vector<int32_t> dom;
    int64_t cells = 0, tiles = 0;
    for (int32_t d = 0; d < n; ++d) {
        off[d] = cells;
        tile0[d] = tiles;
        const int64_t nt = W ? nx[d] / W : 0;
        for (int64_t i = 0; i < nt; ++i) dom.push_back(d);
        cells += nx[d];
        tiles += nt;
    }
    off[n] = cells;
    // first domain of each classic block (empty domains are skipped by the kernel's forward walk)
    std::vector<int32_t> blk((size_t)((cells + sw::kClassicBlock - 1) / sw::kClassicBlock));
    for (int32_t d = 0, k = 0; k < (int32_t)blk.size(); ++k) {
        const int64_t first = (int64_t)k * sw::kClassicBlock;
        while (d + 1 < n && off[d + 1] <= first) ++d;
        blk[k] = d;
    }
    const size_t bytes = sizeof(int64_t) * (size_t)(2 * n + 1) + sizeof(int32_t) * (dom.size() + blk.size()) + 16;
    SW_CUDA(ctx, sw::grow_dev(&bt.d_tables, &bt.n_tables, bytes));
    char *base = static_cast<char *>(bt.d_tables);
    int64_t *d_off = reinterpret_cast<int64_t *>(base);
    int64_t *d_tile0 = d_off + (n + 1);
    int32_t *d_dom = reinterpret_cast<int32_t *>(d_tile0 + n);
    SW_CUDA(ctx, cudaMemcpy(d_off, off.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice));
    SW_CUDA(ctx, cudaMemcpy(d_tile0, tile0.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice));
    if (!dom.empty()) SW_CUDA(ctx, cudaMemcpy(d_dom, dom.data(), sizeof(int32_t) * dom.size(), cudaMemcpyHostToDevice));
    int32_t *d_blk = d_dom + dom.size();
    if (!blk.empty()) SW_CUDA(ctx, cudaMemcpy(d_blk, blk.data(), sizeof(int32_t) * blk.size(), cudaMemcpyHostToDevice));
    int32_t group = 4;  // grouped swept blocks (G tiles of one domain each) where every domain allows them
    for (int32_t d = 0; d < n && W; ++d)
        while (group > 1 && (nx[d] / W) % group != 0) group >>= 1;
    bt.dev = BatchDev{d_dom, d_off, d_tile0, d_blk, tiles, cells, n, W ? group : 1};
    bt.nx.assign(nx, nx + n);
    bt.W = W;
    if (ctx->graph.exec) {  // the tables moved: a cached graph may point at the old ones
        cudaGraphExecDestroy(ctx->graph.exec);
        ctx->graph.exec = nullptr;
    }
    return SW_OK;
}

template <typename T>
int enqueue(sw_ctx *ctx, const Ops *ops, const Params<T> &p, const sw_config &c, int W, int threads, void *state,
            cudaStream_t s, int64_t *launches) {
    const BatchDev *b = &ctx->batch.dev;
    const int64_t n = c.n_steps;
    if (c.alg == SW_ALG_CLASSIC) {
        void *cur = state, *alt = ctx->d_work;
        for (int64_t i = 0; i < n; ++i) {
            if (ops->S == 1) {
                SW_CUDA(ctx, ops->batch_classic(&p, cur, alt, 0, b, 256, s));
                std::swap(cur, alt);
                *launches += 1;
            } else {
                SW_CUDA(ctx, ops->batch_classic(&p, cur, alt, 0, b, 256, s));
                SW_CUDA(ctx, ops->batch_classic(&p, alt, cur, 1, b, 256, s));
                *launches += 2;
            }
        }
        if (cur != state) SW_CUDA(ctx, cudaMemcpyAsync(state, cur, ops->cell * b->n_cells, cudaMemcpyDeviceToDevice, s));
        return SW_OK;
    }
    const int64_t q = W / (2 * ops->R * ops->S);
    const int64_t full = n / q, rem = n - full * q;
    if (full >= 1) {
        if (c.alg == SW_ALG_VARIANT) {
            SW_CUDA(ctx, ops->batch_persistent(&p, state, ctx->d_slots, b, ctx->d_flags, ctx->d_status, W, threads,
                                               full - 1, s));
            *launches += 1;
        } else {
            SW_CUDA(ctx, ops->batch_swept(&p, MODE_UP, 0, state, ctx->d_slots, b, W, threads, s));
            for (int64_t d = 1; d < full; ++d)
                SW_CUDA(ctx, ops->batch_swept(&p, MODE_DIAMOND, (int)(d & 1), state, ctx->d_slots, b, W, threads, s));
            SW_CUDA(ctx, ops->batch_swept(&p, MODE_DOWN, (int)(full & 1), state, ctx->d_slots, b, W, threads, s));
            *launches += full + 1;
        }
    }
    void *cur = state, *alt = ctx->d_work;
    for (int64_t i = 0; i < rem; ++i) {
        SW_CUDA(ctx, ops->batch_classic(&p, cur, alt, 0, b, 256, s));
        if (ops->S == 1) {
            std::swap(cur, alt);
        } else {
            SW_CUDA(ctx, ops->batch_classic(&p, alt, cur, 1, b, 256, s));
        }
        *launches += ops->S;
    }
    if (cur != state) SW_CUDA(ctx, cudaMemcpyAsync(state, cur, ops->cell * b->n_cells, cudaMemcpyDeviceToDevice, s));
    return SW_OK;
}

bool same_key(const GraphKey &a, const GraphKey &b) { return std::memcmp(&a, &b, sizeof(GraphKey)) == 0; }

template <typename T>
int run_batch_device(sw_ctx *ctx, const sw_config &c0, int32_t n, const int64_t *nx, void *state, cudaStream_t user,
                     sw_result *out, bool tuning_pass, double *ms_out) {
    const Ops *ops = ops_for(c0.problem, c0.precision, c0.flags);
    sw_config c = c0;
    if (c.alg != SW_ALG_CLASSIC && c.tpb == 0) {
        sw_tuning t;
        int rc = sw_query_tuning(ctx, &c0, n, nx, &t);
        if (rc) return rc;
        c.tpb = t.tile;
        if (c.threads == 0) c.threads = t.threads;
    }
    const int W = (c.alg == SW_ALG_CLASSIC) ? 0 : c.tpb;
    int threads = c.threads;
    int64_t cells = 0;
    for (int32_t d = 0; d < n; ++d) cells += nx[d];
    // device buffers: slots 2 cells each, classic work, flags 2 per tile (>= 32-wide tiles)
    SW_CUDA(ctx, sw::grow_dev(&ctx->d_slots, &ctx->n_slots, ops->cell * (size_t)cells * 2));
    SW_CUDA(ctx, sw::grow_dev(&ctx->d_work, &ctx->n_work, ops->cell * (size_t)cells));
    SW_CUDA(ctx, sw::grow_dev((void **)&ctx->d_flags, &ctx->n_flags, sizeof(unsigned) * (size_t)(cells / 16 + 2)));
    if (!ctx->d_status) SW_CUDA(ctx, cudaMalloc(&ctx->d_status, sizeof(int)));
    int rc = ensure_tables(ctx, n, nx, W);
    if (rc) return rc;

    sw_constants k;
    sw_config cd = c;
    cd.nx = nx[0];
    sw_constants_of(&cd, &k);
    Params<T> p = sw::make_params<T>(cd, k);
    p.status = ctx->d_status;  // bounded waits (grouped blocks' bulk copies) report here

    cudaStream_t s = ctx->stream;
    SW_CUDA(ctx, cudaEventRecord(ctx->e0, user));
    SW_CUDA(ctx, cudaStreamWaitEvent(s, ctx->e0, 0));
    SW_CUDA(ctx, cudaMemsetAsync(ctx->d_status, 0, sizeof(int), s));
    int64_t launches = 0;
    if (tuning_pass || c.alg == SW_ALG_CLASSIC) {
        SW_CUDA(ctx, cudaEventRecord(ctx->k0, s));
        rc = enqueue<T>(ctx, ops, p, c, W, threads, state, s, &launches);
        if (rc) return rc;
    } else {
        GraphKey key;
        std::memset(&key, 0, sizeof(key));
        key.problem = c.problem;
        key.prec = c.precision;
        key.alg = c.alg;
        key.W = W;
        key.threads = threads;
        key.n_steps = c.n_steps;
        key.state = state;
        key.slots = ctx->d_slots;
        key.tables = ctx->batch.d_tables;
        key.work = ctx->d_work;
        key.flags = ctx->d_flags;
        key.status = ctx->d_status;
        key.cells = cells;
        std::memcpy(key.params, &p, sizeof(p) <= sizeof(key.params) ? sizeof(p) : sizeof(key.params));
        if (!ctx->graph.exec || !same_key(ctx->graph.key, key)) {
            if (ctx->graph.exec) cudaGraphExecDestroy(ctx->graph.exec);
            ctx->graph.exec = nullptr;
            SW_CUDA(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
            rc = enqueue<T>(ctx, ops, p, c, W, threads, state, s, &launches);
            cudaGraph_t g = nullptr;
            cudaError_t ec = cudaStreamEndCapture(s, &g);
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            if (ec != cudaSuccess) return cuda_fail(ctx, ec, "cudaStreamEndCapture");
            ec = cudaGraphInstantiate(&ctx->graph.exec, g, 0);
            cudaGraphDestroy(g);
            if (ec != cudaSuccess) return cuda_fail(ctx, ec, "cudaGraphInstantiate");
            ctx->graph.key = key;
            ctx->graph.launches = launches;
        }
        launches = ctx->graph.launches;
        // timed from here: a first call's capture and instantiation are host work, not stepping
        SW_CUDA(ctx, cudaEventRecord(ctx->k0, s));
        SW_CUDA(ctx, cudaGraphLaunch(ctx->graph.exec, s));
    }
    SW_CUDA(ctx, cudaEventRecord(ctx->k1, s));
    SW_CUDA(ctx, cudaStreamWaitEvent(user, ctx->k1, 0));
    SW_CUDA(ctx, cudaEventSynchronize(ctx->k1));
    SW_CUDA(ctx, cudaGetLastError());
    int st = 0;
    SW_CUDA(ctx, cudaMemcpy(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st == 2) return fail(ctx, SW_ERR_TIMEOUT, "ensemble swept kernel: a bulk copy's wait ran out");
    if (st) return fail(ctx, SW_ERR_TIMEOUT, "persistent ensemble kernel: an inter-block wait expired");
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->k0, ctx->k1);
    if (ms_out) *ms_out = ms;
    if (out) {
        std::memset(out, 0, sizeof(*out));
        out->t_final = (double)c.n_steps * c.dt;
        out->n_steps = c.n_steps;
        out->elapsed_ms = ms;
        out->kernel_ms = ms;
        out->us_per_step = c.n_steps ? ms * 1e3 / (double)c.n_steps : 0.0;
        out->launches = launches;
        out->tile = W;
    }
    return SW_OK;
}

int run_batch_dispatch(sw_ctx *ctx, const sw_config &c, int32_t n, const int64_t *nx, void *state, cudaStream_t user,
                       sw_result *out, bool tuning_pass, double *ms) {
    SW_CUDA(ctx, cudaSetDevice(ctx->device));
    if (c.precision == 4) return run_batch_device<float>(ctx, c, n, nx, state, user, out, tuning_pass, ms);
    return run_batch_device<double>(ctx, c, n, nx, state, user, out, tuning_pass, ms);
}

}  // namespace

extern "C" {

int sw_run_batch_device(sw_ctx *ctx, const sw_config *cfg, int32_t n, const int64_t *nx, void *state_dev, void *stream,
                        sw_result *out) {
    if (!ctx) return SW_ERR_ARG;
    int rc = check_batch(cfg, n, nx);
    if (rc) return fail(ctx, rc, std::string("invalid ensemble: ") + sw_strerror(rc));
    if (!state_dev) return fail(ctx, SW_ERR_ARG, "null device state");
    return run_batch_dispatch(ctx, *cfg, n, nx, state_dev, (cudaStream_t)stream, out, false, nullptr);
}

int sw_run_batch(sw_ctx *ctx, const sw_config *cfg, int32_t n, const int64_t *nx, const void *ic_host,
                 void *final_host, sw_result *out) {
    if (!ctx) return SW_ERR_ARG;
    int rc = check_batch(cfg, n, nx);
    if (rc) return fail(ctx, rc, std::string("invalid ensemble: ") + sw_strerror(rc));
    if (!ic_host || !final_host) return fail(ctx, SW_ERR_ARG, "sw_run_batch needs ic_host and final_host");
    const Ops *ops = ops_for(cfg->problem, cfg->precision, cfg->flags);
    int64_t cells = 0;
    for (int32_t d = 0; d < n; ++d) cells += nx[d];
    SW_CUDA(ctx, cudaSetDevice(ctx->device));
    SW_CUDA(ctx, sw::grow_dev(&ctx->d_state, &ctx->n_state, ops->cell * (size_t)cells));
    const size_t host_bytes = (size_t)ops->prec * ops->C * cells;
    cudaStream_t s = ctx->stream;
    if (ops->C == 3) {
        SW_CUDA(ctx, sw::grow_dev(&ctx->d_io, &ctx->n_io, host_bytes));
        SW_CUDA(ctx, cudaMemcpyAsync(ctx->d_io, ic_host, host_bytes, cudaMemcpyHostToDevice, s));
        SW_CUDA(ctx, ops->pack(ctx->d_io, ctx->d_state, cells, s));
    } else {
        SW_CUDA(ctx, cudaMemcpyAsync(ctx->d_state, ic_host, host_bytes, cudaMemcpyHostToDevice, s));
    }
    rc = run_batch_dispatch(ctx, *cfg, n, nx, ctx->d_state, s, out, false, nullptr);
    if (rc) return rc;
    if (ops->C == 3) {
        SW_CUDA(ctx, ops->unpack(ctx->d_state, ctx->d_io, cells, s));
        SW_CUDA(ctx, cudaMemcpyAsync(final_host, ctx->d_io, host_bytes, cudaMemcpyDeviceToHost, s));
    } else {
        SW_CUDA(ctx, cudaMemcpyAsync(final_host, ctx->d_state, host_bytes, cudaMemcpyDeviceToHost, s));
    }
    SW_CUDA(ctx, cudaStreamSynchronize(s));
    return SW_OK;
}

int sw_query_tuning(sw_ctx *ctx, const sw_config *cfg, int32_t n, const int64_t *nx, sw_tuning *out) {
    if (!ctx || !out) return SW_ERR_ARG;
    sw_config c = *cfg;
    c.tpb = 0;
    int rc = check_batch(&c, n, nx);
    if (rc) return fail(ctx, rc, std::string("invalid ensemble: ") + sw_strerror(rc));
    TuneCache &tc = ctx->tune;
    if (tc.valid && tc.problem == c.problem && tc.prec == c.precision && tc.alg == c.alg &&
        (int32_t)tc.nx.size() == n && std::equal(tc.nx.begin(), tc.nx.end(), nx)) {
        *out = tc.result;
        return SW_OK;
    }
    std::memset(out, 0, sizeof(*out));
    if (c.alg == SW_ALG_CLASSIC) return SW_OK;
    const Ops *ops = ops_for(c.problem, c.precision, c.flags);
    // sample: every k-th domain, at least kTuneCells cells where the ensemble has that many
    int64_t total = 0;
    for (int32_t d = 0; d < n; ++d) total += nx[d];
    const int32_t stride = (int32_t)std::max<int64_t>(1, total / kTuneCells);
    std::vector<int64_t> sample;
    for (int32_t d = 0; d < n; d += stride) sample.push_back(nx[d]);
    int64_t scells = 0;
    for (int64_t v : sample) scells += v;
    // time steps common to every candidate: two diamonds of the widest tile
    const int64_t steps = 2 * (1024 / (2 * ops->R * ops->S));
    // sample state: each sampled domain's reference initial condition, device layout
    const int comps = ops->C;
    std::vector<char> host((size_t)ops->prec * comps * scells);
    {
        size_t at = 0;
        for (int64_t v : sample) {
            sw_config ic = c;
            ic.nx = v;
            sw_initial_condition(&ic, host.data() + at);
            at += (size_t)ops->prec * comps * v;
        }
    }
    void *tune_state = nullptr;
    SW_CUDA(ctx, cudaSetDevice(ctx->device));
    SW_CUDA(ctx, cudaMalloc(&tune_state, ops->cell * (size_t)scells + (size_t)ops->prec * comps * scells));
    void *tune_io = static_cast<char *>(tune_state) + ops->cell * (size_t)scells;
    auto reset = [&]() -> cudaError_t {
        if (comps == 3) {
            cudaError_t e = cudaMemcpy(tune_io, host.data(), host.size(), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return e;
            e = ops->pack(tune_io, tune_state, scells, ctx->stream);
            if (e != cudaSuccess) return e;
            return cudaStreamSynchronize(ctx->stream);
        }
        return cudaMemcpy(tune_state, host.data(), host.size(), cudaMemcpyHostToDevice);
    };
    const int maxt = ops->max_threads;
    int best = -1;
    for (int W = 32; W <= 1024; W *= 2) {
        if (!valid_tile(W, n, nx)) continue;
        for (int div = 1; div <= 4; div *= 2) {
            const int threads = W / div;
            if (threads < 32 || threads > maxt || out->n_candidates >= 48) continue;
            sw_config t = c;
            t.tpb = W;
            t.threads = threads;
            t.n_steps = steps;
            double ms_best = 1e300;
            for (int rep = 0; rep < 2; ++rep) {
                cudaError_t e = reset();
                if (e != cudaSuccess) {
                    cudaFree(tune_state);
                    return cuda_fail(ctx, e, "tuning reset");
                }
                double ms = 0;
                rc = run_batch_dispatch(ctx, t, (int32_t)sample.size(), sample.data(), tune_state, ctx->stream, nullptr,
                                        true, &ms);
                if (rc) {
                    cudaFree(tune_state);
                    return rc;
                }
                ms_best = std::min(ms_best, ms);
            }
            const int i = out->n_candidates++;
            out->cand_tile[i] = W;
            out->cand_threads[i] = threads;
            out->cand_rate[i] = (double)scells * steps / (ms_best * 1e-3);
            if (best < 0 || out->cand_rate[i] > out->cand_rate[best]) best = i;
        }
    }
    cudaFree(tune_state);
    if (best < 0) return fail(ctx, SW_ERR_SIZE, "no tile width divides every domain");
    out->tile = out->cand_tile[best];
    out->threads = out->cand_threads[best];
    out->cell_updates_per_s = out->cand_rate[best];
    tc.valid = true;
    tc.problem = c.problem;
    tc.prec = c.precision;
    tc.alg = c.alg;
    tc.nx.assign(nx, nx + n);
    tc.result = *out;
    return SW_OK;
}

}  // extern "C"
