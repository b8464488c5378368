// C ABI of libswept1d: contexts, configuration, the reference's constants and
// initial conditions, and the run loop that replaces classicWrapper /
// sweptWrapper of the reference programs.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "ctx.h"
#include "sw_internal.h"

using namespace sw;

namespace {


// Tile width of the swept / variant path.  KS alg 2 keeps the reference's
// register path node of 32 cells (KS1D_SweptShared.cu:62-65,755-759).
int tile_width(const sw_config &c) {
    if (c.problem == SW_KS && (c.alg == SW_ALG_VARIANT || c.alg == SW_ALG_SELFTEST)) return 32;
    return c.tpb;
}

// ---- constants, rounded through REAL like the reference's main()
template <typename R>
void derive(const sw_config &c, sw_constants &k) {
    std::memset(&k, 0, sizeof(k));
    const int64_t nx = c.nx;
    if (c.problem == SW_HEAT) {
        // Heat1D_SweptShared.cu:56-58,719-728
        const R th = (R)(c.alpha != 0 ? c.alpha : 8.418e-5);
        const R ds = (R)(c.dx != 0 ? c.dx : 0.001);
        const double fou = (double)th * c.dt / (double)(ds * ds);
        k.fourier = (R)fou;
        k.fourier_two = (R)(1.0 - 2.0 * fou);
        k.lx = (double)ds * ((double)nx - 1.0);
        k.dx = (double)ds;
    } else if (c.problem == SW_KS) {
        // KS1D_SweptShared.cu:45,887,917-926
        const R dx = (R)(c.dx != 0 ? c.dx : 0.5);
        if (c.flags & SW_FLAG_KS_DIVIDE) {
            // the DIVISE build's divisors, KS1D_SweptShared.cu:904-914
            k.dx_times4 = R(4) * dx;
            k.dx2 = dx * dx;
            k.dx4 = dx * dx * dx * dx;
        } else {
            k.dx_times4 = R(1) / (R(4) * dx);
            k.dx2 = R(1) / (dx * dx);
            k.dx4 = R(1) / (dx * dx * dx * dx);
        }
        k.dt = (R)c.dt;
        k.dt_half = (R)(c.dt * 0.5);
        k.lx = (double)((R)nx * dx);
        k.dx = (double)dx;
    } else {
        // Euler1D_SweptShared.cu:69,1127-1149
        R gam, mgam;
        if (c.gamma == 0) {
            gam = (R)1.4;
            mgam = (R)0.4;
        } else {
            gam = (R)c.gamma;
            mgam = (R)(c.gamma - 1.0);
        }
        const R lx = R(1);
        const double dx = c.dx != 0 ? c.dx : (double)(lx / ((R)nx - R(2)));
        k.gam = gam;
        k.mgam = mgam;
        k.dt_dx = (R)(c.dt / dx);
        bool sod = true;
        for (int i = 0; i < 3; ++i) sod = sod && c.left[i] == 0 && c.right[i] == 0;
        if (sod) {
            k.bd[0] = R(1);
            k.bd[1] = R(0);
            k.bd[2] = R(1) / mgam;
            k.bd[3] = (R)0.125;
            k.bd[4] = R(0);
            k.bd[5] = (R)(0.1 / (double)mgam);
        } else {
            const double *st[2] = {c.left, c.right};
            for (int s = 0; s < 2; ++s) {
                const double rho = st[s][0], u = st[s][1], p = st[s][2];
                k.bd[3 * s] = (R)rho;
                k.bd[3 * s + 1] = (R)(rho * u);
                k.bd[3 * s + 2] = (R)(p / (double)mgam + 0.5 * rho * u * u);
            }
        }
        k.lx = (double)lx;
        k.dx = dx;
    }
}


// ---- run plans: the sequence of work the reference wrappers perform
struct Segment {
    int64_t count;   // classic: time steps; swept: diamonds between up- and down-triangle
    double t_snap;   // t_eq written with the snapshot (< 0: final segment)
};
struct Plan {
    bool swept = false;
    std::vector<Segment> segs;
    int64_t remainder = 0;  // SW_TIME_STEPS swept: classic steps after the last segment
    int down_phase = 0;     // swept, SW_TIME_STEPS: phase of the final down-triangle
    double t_final = 0;
    int64_t steps = 0;
};

// dt the wrapper receives: KS passes dsc.dt, i.e. dt rounded to REAL (KS1D_SweptShared.cu:975,979)
double wrapper_dt(const sw_config &c) {
    if (c.problem == SW_KS && c.precision == 4) return (double)(float)c.dt;
    return c.dt;
}

Plan plan_reference(const sw_config &c, int W, int R, int S) {
    Plan pl;
    const double dt = wrapper_dt(c);
    const double t_end = c.tf - 0.25 * c.dt;  // main(): tf = atof(argv[4]) - 0.25*dt
    const bool outputs = c.freq > 0;
    double twrite = c.freq - 0.25 * dt;
    if (c.alg == SW_ALG_CLASSIC) {
        if (c.problem == SW_HEAT) {
            // classicWrapper, Heat1D_SweptShared.cu:483-510: two steps per pass; after a
            // snapshot t_eq advances one more pass without stepping.
            const double tfs = dt + dt;
            int64_t n = 2;
            double t_eq = tfs;
            while (t_eq < t_end) {
                n += 2;
                t_eq += tfs;
                if (outputs && t_eq > twrite) {
                    pl.segs.push_back({n, t_eq});
                    pl.steps += n;
                    n = 0;
                    t_eq += tfs;
                    twrite += c.freq;
                }
            }
            pl.segs.push_back({n, -1});
            pl.steps += n;
            pl.t_final = t_eq;
        } else {
            // KS1D_SweptShared.cu:609-631 (t_eq <= t_end), Euler1D_SweptShared.cu:855-888 (<)
            const bool le = (c.problem == SW_KS);
            int64_t n = 0;
            double t_eq = 0.0;
            while (le ? (t_eq <= t_end) : (t_eq < t_end)) {
                ++n;
                t_eq += dt;
                if (outputs && t_eq > twrite) {
                    pl.segs.push_back({n, t_eq});
                    pl.steps += n;
                    n = 0;
                    twrite += c.freq;
                }
            }
            pl.segs.push_back({n, -1});
            pl.steps += n;
            pl.t_final = t_eq;
        }
        return pl;
    }
    // sweptWrapper (Heat1D_SweptShared.cu:541-682, KS1D_SweptShared.cu:676-851,
    // Euler1D_SweptShared.cu:924-1100): up, split diamond, then pairs of
    // diamonds; a snapshot is down-triangle, up-triangle, split diamond.
    pl.swept = true;
    const double tfs = dt * (double)W / (double)(R * S);  // Heat: tpb dt; KS/Euler: tpb dt / 4
    const int64_t per_seg_steps = (int64_t)(W / (2 * R * S));
    int64_t nd = 1;
    double t_eq = tfs;
    while (t_eq < t_end) {
        nd += 2;
        t_eq += tfs;
        if (outputs && t_eq > twrite) {
            pl.segs.push_back({nd, t_eq});
            pl.steps += (nd + 1) * per_seg_steps;
            nd = 1;
            t_eq += tfs;
            twrite += c.freq;
        }
    }
    pl.segs.push_back({nd, -1});
    pl.steps += (nd + 1) * per_seg_steps;
    pl.t_final = t_eq;
    return pl;
}

Plan plan_steps(const sw_config &c, int W, int R, int S) {
    Plan pl;
    const int64_t n = c.n_steps;
    pl.t_final = (double)n * c.dt;
    pl.steps = n;
    if (c.alg == SW_ALG_CLASSIC) {
        pl.segs.push_back({n, -1});
        return pl;
    }
    const int64_t q = W / (2 * R * S);  // time steps per diamond
    const int64_t full = n / q;
    pl.swept = true;
    if (full >= 1) {
        pl.segs.push_back({full - 1, -1});
        pl.down_phase = (int)(full & 1);
    }
    pl.remainder = n - full * q;
    return pl;
}

template <typename T>
struct Runner {
    sw_ctx *ctx;
    const Ops *ops;
    const sw_config &cfg;
    Params<T> p;
    int W;
    cudaStream_t s;
    void *cur;  // device state (device layout)
    void *alt;  // classic work buffer
    int64_t launches = 0;
    bool persistent;
    bool host_tile = false;  // SW_FLAG_HOST_TILE: phase-1 passes leave their wrapping tile to the host

    // One launch-per-pass pass.  With the host tile, a phase-1 pass launches every
    // tile but the last (the one that wraps from cell nx-1 to 0: the launch covers
    // nx - W cells while Params::nx stays the domain's) and the host computes that
    // tile meanwhile from its two slots, copied down before the launch and back
    // after it on the same stream.
    int pass(int mode, int phase) {
        const int64_t nx = cfg.nx;
        if (!host_tile || phase == 0) {
            SW_CUDA(ctx, ops->swept(&p, mode, phase, cur, ctx->d_slots, nx, W, cfg.threads, s));
            return SW_OK;
        }
        const size_t wb = ops->cell * (size_t)W, hb = wb / 2;
        char *slots = static_cast<char *>(ctx->d_slots), *state = static_cast<char *>(cur);
        char *dl = slots + (size_t)(nx / (W / 2) - 1) * wb, *dr = slots;
        char *h = static_cast<char *>(ctx->h_tile);  // [slot l: W][slot r: W][state first: W/2][state last: W/2]
        SW_CUDA(ctx, cudaMemcpyAsync(h, dl, wb, cudaMemcpyDeviceToHost, s));
        SW_CUDA(ctx, cudaMemcpyAsync(h + wb, dr, wb, cudaMemcpyDeviceToHost, s));
        SW_CUDA(ctx, cudaEventRecord(ctx->tile_ready, s));
        if (nx > W) SW_CUDA(ctx, ops->swept(&p, mode, 1, cur, ctx->d_slots, nx - W, W, cfg.threads, s));
        SW_CUDA(ctx, cudaEventSynchronize(ctx->tile_ready));
        host_tile_run(cfg.problem, cfg.precision, &p, mode, h, h + wb, h + 2 * wb, h + 2 * wb + hb, W);
        if (mode == MODE_DIAMOND) {
            SW_CUDA(ctx, cudaMemcpyAsync(dl, h, wb, cudaMemcpyHostToDevice, s));
            SW_CUDA(ctx, cudaMemcpyAsync(dr, h + wb, wb, cudaMemcpyHostToDevice, s));
        } else {
            SW_CUDA(ctx, cudaMemcpyAsync(state, h + 2 * wb, hb, cudaMemcpyHostToDevice, s));
            SW_CUDA(ctx, cudaMemcpyAsync(state + (size_t)(nx - W / 2) * ops->cell, h + 2 * wb + hb, hb,
                                         cudaMemcpyHostToDevice, s));
        }
        return SW_OK;
    }

    int classic_steps(int64_t n) {
        const int64_t nx = cfg.nx;
        const int block = cfg.tpb;
        for (int64_t i = 0; i < n; ++i) {
            if (ops->S == 1) {
                SW_CUDA(ctx, ops->classic(&p, cur, alt, 0, nx, block, s));
                std::swap(cur, alt);
                ++launches;
            } else {
                SW_CUDA(ctx, ops->classic(&p, cur, alt, 0, nx, block, s));
                SW_CUDA(ctx, ops->classic(&p, alt, cur, 1, nx, block, s));
                launches += 2;
            }
        }
        return SW_OK;
    }

    // up-triangle, nd diamonds (phases 1, 0, 1, ...), down-triangle at down_phase
    int swept_segment(int64_t nd, int down_phase) {
        const int64_t nx = cfg.nx;
        if (persistent && ((nd + 1) & 1) == down_phase) {
            SW_CUDA(ctx, ops->persistent(&p, cur, ctx->d_slots, ctx->d_flags, ctx->d_status, nx, W, cfg.threads, nd, s));
            ++launches;
            return SW_OK;
        }
        int rc = pass(MODE_UP, 0);
        for (int64_t d = 1; d <= nd && rc == SW_OK; ++d) rc = pass(MODE_DIAMOND, (int)(d & 1));
        if (rc == SW_OK) rc = pass(MODE_DOWN, down_phase);
        launches += nd + 2;
        return rc;
    }

    // cur back into the primary state buffer (Heat classic leaves it in alt after odd counts)
    int settle(void *primary) {
        if (cur != primary) {
            SW_CUDA(ctx, cudaMemcpyAsync(primary, cur, ops->cell * cfg.nx, cudaMemcpyDeviceToDevice, s));
            std::swap(cur, alt);
        }
        return SW_OK;
    }
};

template <typename T>
int check_status(sw_ctx *ctx, cudaStream_t s) {
    int st = 0;
    cudaError_t e = cudaMemcpyAsync(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "status readback");
    if (st == 2) return fail(ctx, SW_ERR_TIMEOUT, "swept kernel: a bulk copy's wait ran out");
    if (st) return fail(ctx, SW_ERR_TIMEOUT, "persistent swept kernel: an inter-block wait expired");
    return SW_OK;
}

// Deliver the device state to the host buffer `dst` (host layout).
int to_host(sw_ctx *ctx, const Ops *ops, const void *state, void *dst, int64_t nx, cudaStream_t s) {
    if (ops->C == 3) {
        SW_CUDA(ctx, ops->unpack(state, ctx->d_io, nx, s));
        SW_CUDA(ctx, cudaMemcpyAsync(dst, ctx->d_io, (size_t)ops->prec * 3 * nx, cudaMemcpyDeviceToHost, s));
    } else {
        SW_CUDA(ctx, cudaMemcpyAsync(dst, state, (size_t)ops->prec * nx, cudaMemcpyDeviceToHost, s));
    }
    SW_CUDA(ctx, cudaStreamSynchronize(s));
    return SW_OK;
}

int ensure_buffers(sw_ctx *ctx, const sw_config &c, const Ops *ops, bool need_io, bool need_pin) {
    const size_t cells = (size_t)c.nx;
    SW_CUDA(ctx, grow_dev(&ctx->d_state, &ctx->n_state, ops->cell * cells));
    SW_CUDA(ctx, grow_dev(&ctx->d_work, &ctx->n_work, ops->cell * cells));
    SW_CUDA(ctx, grow_dev(&ctx->d_slots, &ctx->n_slots, ops->cell * cells * 2));
    const size_t nhalf = (size_t)(c.nx / 16) + 2;  // smallest tile is 32 wide
    SW_CUDA(ctx, grow_dev((void **)&ctx->d_flags, &ctx->n_flags, sizeof(unsigned) * nhalf));
    if (!ctx->d_status) SW_CUDA(ctx, cudaMalloc(&ctx->d_status, sizeof(int)));
    if (need_io && ops->C == 3) SW_CUDA(ctx, grow_dev(&ctx->d_io, &ctx->n_io, (size_t)ops->prec * 3 * cells));
    if (need_pin) SW_CUDA(ctx, grow_pinned(&ctx->h_pin, &ctx->n_pin, (size_t)ops->prec * ops->C * cells));
    return SW_OK;
}

template <typename T>
int run_impl(sw_ctx *ctx, const sw_config &c, const void *ic_host, void *final_host, void *state_dev,
             cudaStream_t stream, sw_snapshot_fn cb, void *user, sw_result *out) {
    const Ops *ops = ops_for(c.problem, c.precision, c.flags);
    if (!ops) return fail(ctx, SW_ERR_ARG, "unknown problem/precision");
    sw_constants k;
    derive<T>(c, k);
    const int W = tile_width(c);
    const bool device_mode = (state_dev != nullptr);
    cudaStream_t s = stream ? stream : ctx->stream;
    const int64_t nx = c.nx;

    SW_CUDA(ctx, cudaEventRecord(ctx->e0, s));
    int rc = ensure_buffers(ctx, c, ops, !device_mode || cb, !device_mode);
    if (rc) return rc;
    SW_CUDA(ctx, cudaMemsetAsync(ctx->d_status, 0, sizeof(int), s));

    void *primary = device_mode ? state_dev : ctx->d_state;
    if (!device_mode) {
        if (ops->C == 3) {
            SW_CUDA(ctx, cudaMemcpyAsync(ctx->d_io, ic_host, (size_t)ops->prec * 3 * nx, cudaMemcpyHostToDevice, s));
            SW_CUDA(ctx, ops->pack(ctx->d_io, primary, nx, s));
        } else {
            SW_CUDA(ctx, cudaMemcpyAsync(primary, ic_host, (size_t)ops->prec * nx, cudaMemcpyHostToDevice, s));
        }
    }

    Plan pl = (c.time_mode == SW_TIME_STEPS) ? plan_steps(c, W, ops->R, ops->S) : plan_reference(c, W, ops->R, ops->S);
    const bool host_tile = (c.flags & SW_FLAG_HOST_TILE) != 0;
    if (host_tile) {
        SW_CUDA(ctx, grow_pinned(&ctx->h_tile, &ctx->n_tile, ops->cell * (size_t)W * 3));
        if (!ctx->tile_ready) SW_CUDA(ctx, cudaEventCreateWithFlags(&ctx->tile_ready, cudaEventDisableTiming));
    }
    Runner<T> r{ctx, ops, c, make_params<T>(c, k), W, s, primary, ctx->d_work, 0,
                c.alg == SW_ALG_VARIANT && !host_tile};
    r.host_tile = host_tile;
    r.p.status = ctx->d_status;  // bounded waits report here (checked after the run and at snapshots)
    int snaps = 0;
    SW_CUDA(ctx, cudaEventRecord(ctx->k0, s));
    for (size_t i = 0; i < pl.segs.size(); ++i) {
        const Segment &g = pl.segs[i];
        if (pl.swept) {
            const int dphase = (c.time_mode == SW_TIME_STEPS) ? pl.down_phase : 0;
            rc = r.swept_segment(g.count, dphase);
        } else {
            rc = r.classic_steps(g.count);
        }
        if (rc) return rc;
        if (g.t_snap >= 0 && cb) {
            rc = r.settle(primary);
            if (rc) return rc;
            rc = check_status<T>(ctx, s);
            if (rc) return rc;
            rc = to_host(ctx, ops, primary, ctx->h_pin, nx, s);
            if (rc) return rc;
            ++snaps;
            if (cb(user, g.t_snap, ctx->h_pin, nx)) return fail(ctx, SW_ERR_CALLBACK, "snapshot callback stopped the run");
        }
    }
    if (pl.remainder) {
        rc = r.classic_steps(pl.remainder);
        if (rc) return rc;
    }
    rc = r.settle(primary);
    if (rc) return rc;
    SW_CUDA(ctx, cudaEventRecord(ctx->k1, s));
    rc = check_status<T>(ctx, s);
    if (rc) return rc;
    if (!device_mode) {
        if (ops->C == 3) {
            SW_CUDA(ctx, ops->unpack(primary, ctx->d_io, nx, s));
            SW_CUDA(ctx, cudaMemcpyAsync(final_host, ctx->d_io, (size_t)ops->prec * 3 * nx, cudaMemcpyDeviceToHost, s));
        } else {
            SW_CUDA(ctx, cudaMemcpyAsync(final_host, primary, (size_t)ops->prec * nx, cudaMemcpyDeviceToHost, s));
        }
    }
    SW_CUDA(ctx, cudaEventRecord(ctx->e1, s));
    SW_CUDA(ctx, cudaEventSynchronize(ctx->e1));
    SW_CUDA(ctx, cudaGetLastError());
    float ms = 0, kms = 0;
    cudaEventElapsedTime(&ms, ctx->e0, ctx->e1);
    cudaEventElapsedTime(&kms, ctx->k0, ctx->k1);
    if (out) {
        out->t_final = pl.t_final;
        out->n_steps = pl.steps;
        out->elapsed_ms = ms;
        out->kernel_ms = kms;
        // main(): us per step = elapsed / (tfm/dt); KS truncates to int (KS1D_SweptShared.cu:997)
        double nts = pl.t_final / c.dt;
        if (c.problem == SW_KS) nts = (double)(int64_t)nts;
        out->us_per_step = nts > 0 ? (double)ms * 1e3 / nts : 0.0;
        out->launches = r.launches;
        out->snapshots = snaps;
        out->tile = (c.alg == SW_ALG_CLASSIC) ? 0 : W;
    }
    return SW_OK;
}

int run_any(sw_ctx *ctx, const sw_config *cfg, const void *ic, void *fin, void *dev, void *stream, sw_snapshot_fn cb,
            void *user, sw_result *out) {
    if (!ctx || !cfg) return SW_ERR_ARG;
    int rc = sw_validate(cfg);
    if (rc) return fail(ctx, rc, std::string("invalid configuration: ") + sw_strerror(rc));
    if (!dev && (!ic || !fin)) return fail(ctx, SW_ERR_ARG, "host run needs ic_host and final_host");
    if (cfg->alg == SW_ALG_SELFTEST) return fail(ctx, SW_ERR_UNSUPPORTED, "alg 3 is a CLI self-test");
    SW_CUDA(ctx, cudaSetDevice(ctx->device));
    if (cfg->precision == 4)
        return run_impl<float>(ctx, *cfg, ic, fin, dev, (cudaStream_t)stream, cb, user, out);
    return run_impl<double>(ctx, *cfg, ic, fin, dev, (cudaStream_t)stream, cb, user, out);
}

}  // namespace

// =================================================================== C ABI
extern "C" {

int sw_abi_version(void) { return SW_ABI_VERSION; }

const char *sw_strerror(int code) {
    switch (code) {
    case SW_OK: return "ok";
    case SW_ERR_ARG: return "invalid argument";
    case SW_ERR_SIZE: return "nx must be divisible by tpb and tpb a multiple of 32 (32..1024)";
    case SW_ERR_UNSTABLE: return "dt/dx too large for stability (Euler: must be <= 0.21)";
    case SW_ERR_CUDA: return "CUDA error";
    case SW_ERR_NOMEM: return "out of memory";
    case SW_ERR_IO: return "file I/O error";
    case SW_ERR_TIMEOUT: return "bounded inter-block wait expired";
    case SW_ERR_UNSUPPORTED: return "unsupported request";
    case SW_ERR_CALLBACK: return "stopped by snapshot callback";
    case SW_ERR_USAGE: return "usage: nx tpb dt tf freq alg solution.dat [timing.txt]";
    default: return "unknown error";
    }
}

int sw_ctx_create(int device, sw_ctx **out) {
    if (!out) return SW_ERR_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return SW_ERR_CUDA;
    if (device < 0 || device >= n) return SW_ERR_ARG;
    sw_ctx *c = new (std::nothrow) sw_ctx();
    if (!c) return SW_ERR_NOMEM;
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&c->e0) != cudaSuccess || cudaEventCreate(&c->e1) != cudaSuccess ||
        cudaEventCreate(&c->k0) != cudaSuccess || cudaEventCreate(&c->k1) != cudaSuccess) {
        sw_ctx_destroy(c);
        return SW_ERR_CUDA;
    }
    *out = c;
    return SW_OK;
}

int sw_ctx_destroy(sw_ctx *c) {
    if (!c) return SW_ERR_ARG;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    void *bufs[] = {c->d_state, c->d_work, c->d_slots, c->d_io, c->d_flags, c->d_status, c->d_w2p, c->d_judge};
    for (void *b : bufs)
        if (b) cudaFree(b);
    if (c->h_pin) cudaFreeHost(c->h_pin);
    if (c->h_tile) cudaFreeHost(c->h_tile);
    if (c->tile_ready) cudaEventDestroy(c->tile_ready);
    if (c->batch.d_tables) cudaFree(c->batch.d_tables);
    if (c->graph.exec) cudaGraphExecDestroy(c->graph.exec);
    cudaEvent_t evs[] = {c->e0, c->e1, c->k0, c->k1};
    for (cudaEvent_t e : evs)
        if (e) cudaEventDestroy(e);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return SW_OK;
}

const char *sw_ctx_last_error(const sw_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int sw_config_init(sw_config *c, int problem, int precision) {
    if (!c) return SW_ERR_ARG;
    std::memset(c, 0, sizeof(*c));
    if (problem < SW_HEAT || problem > SW_EULER || (precision != 4 && precision != 8)) return SW_ERR_ARG;
    c->problem = problem;
    c->precision = precision;
    c->alg = SW_ALG_SWEPT;
    c->bc = SW_BC_DEFAULT;
    c->nx = 1024;
    c->tpb = 64;
    c->time_mode = SW_TIME_REFERENCE;
    c->dt = (problem == SW_EULER) ? 1e-5 : 1e-3;
    c->tf = (problem == SW_EULER) ? 0.01 : 1.0;
    c->freq = 0;
    return SW_OK;
}

int sw_validate(const sw_config *c) {
    if (!c) return SW_ERR_ARG;
    if (c->problem < SW_HEAT || c->problem > SW_EULER) return SW_ERR_ARG;
    if (c->precision != 4 && c->precision != 8) return SW_ERR_ARG;
    if (c->alg < SW_ALG_CLASSIC || c->alg > SW_ALG_SELFTEST) return SW_ERR_ARG;
    if (c->alg == SW_ALG_SELFTEST && c->problem != SW_KS) return SW_ERR_ARG;
    if (c->time_mode != SW_TIME_REFERENCE && c->time_mode != SW_TIME_STEPS) return SW_ERR_ARG;
    if ((c->flags & ~(SW_FLAG_KS_DIVIDE | SW_FLAG_HOST_TILE)) != 0) return SW_ERR_ARG;
    if ((c->flags & SW_FLAG_KS_DIVIDE) && c->problem != SW_KS) return SW_ERR_ARG;
    if (c->flags & SW_FLAG_HOST_TILE) {  // the hybrid variant: swept passes, not with the dividing KS build
        const bool alg_ok = c->alg == SW_ALG_SWEPT || (c->alg == SW_ALG_VARIANT && c->problem != SW_KS);
        if (!alg_ok || (c->flags & SW_FLAG_KS_DIVIDE)) return SW_ERR_ARG;
    }
    const int bc = resolved_bc(*c);
    if (c->problem == SW_HEAT && bc != SW_BC_MIRROR && bc != SW_BC_PERIODIC) return SW_ERR_ARG;
    if (c->problem == SW_KS && bc != SW_BC_PERIODIC) return SW_ERR_ARG;
    if (c->problem == SW_EULER && bc != SW_BC_DIRICHLET) return SW_ERR_ARG;
    if (!(c->dt > 0) || !std::isfinite(c->dt)) return SW_ERR_ARG;
    if (c->time_mode == SW_TIME_STEPS && c->n_steps < 0) return SW_ERR_ARG;
    if (c->time_mode == SW_TIME_REFERENCE && !std::isfinite(c->tf)) return SW_ERR_ARG;
    // Heat1D_SweptShared.cu:735-740 (nx divisible by tpb, tpb a multiple of 32)
    if (c->tpb < 32 || c->tpb > 1024 || (c->tpb & 31) != 0) return SW_ERR_SIZE;
    if (c->nx < c->tpb || c->nx % c->tpb != 0 || c->nx > ((int64_t)1 << 34)) return SW_ERR_SIZE;
    if (c->problem == SW_EULER && c->nx < 8) return SW_ERR_SIZE;
    if (c->problem == SW_EULER) {
        sw_constants k;
        if (c->precision == 4) derive<float>(*c, k);
        else derive<double>(*c, k);
        if (k.dt_dx > 0.21) return SW_ERR_UNSTABLE;  // Euler1D_SweptShared.cu:1168-1172
    }
    return SW_OK;
}

int sw_constants_of(const sw_config *c, sw_constants *out) {
    if (!c || !out) return SW_ERR_ARG;
    if (c->problem < SW_HEAT || c->problem > SW_EULER || (c->precision != 4 && c->precision != 8)) return SW_ERR_ARG;
    if (c->precision == 4) derive<float>(*c, *out);
    else derive<double>(*c, *out);
    return SW_OK;
}

int sw_initial_condition(const sw_config *c, void *ic) {
    if (!c || !ic) return SW_ERR_ARG;
    if (c->problem < SW_HEAT || c->problem > SW_EULER || (c->precision != 4 && c->precision != 8) || c->nx < 1)
        return SW_ERR_ARG;
    const int64_t nx = c->nx;
    if (c->problem == SW_HEAT) {
        // initFun, Heat1D_SweptShared.cu:60-66, lx = ds*(nx-1) (:719)
        if (c->precision == 4) {
            const float ds = (float)(c->dx != 0 ? c->dx : 0.001);
            const float lx = (float)((double)ds * ((double)nx - 1.0));
            float *u = (float *)ic;
            for (int64_t i = 0; i < nx; ++i) {
                const float a = (float)i * ds;
                u[i] = 100.f * a * (1.f - a / lx);
            }
        } else {
            const double ds = c->dx != 0 ? c->dx : 0.001;
            const double lx = ds * ((double)nx - 1.0);
            double *u = (double *)ic;
            for (int64_t i = 0; i < nx; ++i) {
                const double a = (double)i * ds;
                u[i] = 100.f * a * (1.0 - a / lx);
            }
        }
    } else if (c->problem == SW_KS) {
        // initFun, KS1D_SweptShared.cu:67-72 at x = (REAL)k*(REAL)dx (:945)
        if (c->precision == 4) {
            const float dx = (float)(c->dx != 0 ? c->dx : 0.5);
            float *u = (float *)ic;
            for (int64_t i = 0; i < nx; ++i) {
                const float x = (float)i * dx;
                u[i] = (float)(2.0f * std::cos(19.0 * x * M_PI / 128.0));
            }
        } else {
            const double dx = c->dx != 0 ? c->dx : 0.5;
            double *u = (double *)ic;
            for (int64_t i = 0; i < nx; ++i) {
                const double x = (double)i * dx;
                u[i] = 2.0 * std::cos(19.0 * x * M_PI / 128.0);
            }
        }
    } else {
        // Euler1D_SweptShared.cu:1179: left state for k < nx/2
        sw_constants k;
        sw_constants_of(c, &k);
        for (int64_t i = 0; i < nx; ++i) {
            const double *b = (i < nx / 2) ? k.bd : k.bd + 3;
            for (int j = 0; j < 3; ++j) {
                if (c->precision == 4) ((float *)ic)[3 * i + j] = (float)b[j];
                else ((double *)ic)[3 * i + j] = b[j];
            }
        }
    }
    return SW_OK;
}

int sw_plan(const sw_config *cfg, sw_plan_info *out, double *snap_t, int64_t *snap_steps, int32_t cap) {
    if (!cfg || !out) return SW_ERR_ARG;
    int rc = sw_validate(cfg);
    if (rc) return rc;
    if (cfg->alg == SW_ALG_SELFTEST) return SW_ERR_UNSUPPORTED;
    const Ops *ops = ops_for(cfg->problem, cfg->precision, cfg->flags);
    if (!ops) return SW_ERR_ARG;
    const int W = tile_width(*cfg);
    Plan pl = (cfg->time_mode == SW_TIME_STEPS) ? plan_steps(*cfg, W, ops->R, ops->S)
                                                : plan_reference(*cfg, W, ops->R, ops->S);
    std::memset(out, 0, sizeof(*out));
    out->t_final = pl.t_final;
    out->n_steps = pl.steps;
    out->tile = pl.swept ? W : 0;
    const int64_t per_seg = (int64_t)(W / (2 * ops->R * ops->S));
    int64_t done = 0, launches = 0;
    int32_t k = 0;
    for (const Segment &g : pl.segs) {
        if (pl.swept) {
            done += (g.count + 1) * per_seg;
            launches += (cfg->alg == SW_ALG_VARIANT) ? 1 : g.count + 2;
        } else {
            done += g.count;
            launches += g.count * ops->S;
        }
        if (g.t_snap >= 0) {
            if (k < cap) {
                if (snap_t) snap_t[k] = g.t_snap;
                if (snap_steps) snap_steps[k] = done;
            }
            ++k;
        }
    }
    launches += pl.remainder * ops->S;
    out->n_snapshots = k;
    out->launches = launches;
    return SW_OK;
}

int sw_run(sw_ctx *ctx, const sw_config *cfg, const void *ic_host, void *final_host, sw_snapshot_fn cb, void *user,
           sw_result *out) {
    return run_any(ctx, cfg, ic_host, final_host, nullptr, nullptr, cb, user, out);
}

int sw_run_device(sw_ctx *ctx, const sw_config *cfg, void *state_dev, void *stream, sw_result *out) {
    if (!state_dev) return fail(ctx, SW_ERR_ARG, "null device state");
    return run_any(ctx, cfg, nullptr, nullptr, state_dev, stream, nullptr, nullptr, out);
}

int sw_swept_pass(sw_ctx *ctx, const sw_config *cfg, int32_t mode, int32_t phase, void *state_dev, void *slots_dev,
                  void *stream) {
    if (!ctx || !cfg) return SW_ERR_ARG;
    int rc = sw_validate(cfg);
    if (rc) return fail(ctx, rc, std::string("invalid configuration: ") + sw_strerror(rc));
    if (cfg->alg != SW_ALG_SWEPT) return fail(ctx, SW_ERR_UNSUPPORTED, "a swept pass needs alg 1");
    if (cfg->flags & SW_FLAG_HOST_TILE) return fail(ctx, SW_ERR_UNSUPPORTED, "the host tile is a run's, not a pass's");
    if (mode < MODE_UP || mode > MODE_DOWN || (phase != 0 && phase != 1) || (mode == MODE_UP && phase != 0))
        return fail(ctx, SW_ERR_ARG, "mode must be 0 (up, phase 0), 1 (diamond) or 2 (down); phase 0 or 1");
    if (!state_dev || !slots_dev) return fail(ctx, SW_ERR_ARG, "null device state or slots");
    const Ops *ops = ops_for(cfg->problem, cfg->precision, cfg->flags);
    SW_CUDA(ctx, cudaSetDevice(ctx->device));
    sw_constants k;
    sw_constants_of(cfg, &k);
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    if (cfg->precision == 4) {
        const Params<float> p = make_params<float>(*cfg, k);
        SW_CUDA(ctx, ops->swept(&p, mode, phase, state_dev, slots_dev, cfg->nx, cfg->tpb, cfg->threads, s));
    } else {
        const Params<double> p = make_params<double>(*cfg, k);
        SW_CUDA(ctx, ops->swept(&p, mode, phase, state_dev, slots_dev, cfg->nx, cfg->tpb, cfg->threads, s));
    }
    return SW_OK;
}

}  // extern "C"
