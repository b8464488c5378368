// sw_cli_main: the reference programs' main() over the C ABI.
//
// argv, banners, the .dat solution file and the appended timing row follow
// Heat1D_SweptShared.cu:697-836, KS1D_SweptShared.cu:866-1029 and
// Euler1D_SweptShared.cu:1112-1287: the same row names and leading spaces,
// ostream precision 10 for the solution (values printed in the run's
// precision), default precision for the timing row.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/swept1d.h"

namespace {

template <typename R>
struct Writer {
    std::ofstream &f;
    int problem;
    int alg;
    const sw_constants &k;
    int64_t nx;

    // pressure / energy as the .dat writer computes them, in REAL (Euler1D_SweptShared.cu:183-193,752-759)
    R pressure(const R *q) const { return (R)k.mgam * (q[2] - ((R)0.5 * q[1] * q[1] / q[0])); }
    R energy(const R *q) const {
        R u = q[1] / q[0];
        return q[2] / q[0] - (R)0.5 * u * u;
    }

    // one snapshot / final block of rows; `lead` is the reference's leading space
    void rows(const R *u, double t, bool lead, bool trailing_endl) {
        if (problem == SW_EULER) {
            const char *names[4] = {"Density ", "Velocity ", "Energy ", "Pressure "};
            for (int v = 0; v < 4; ++v) {
                f << names[v] << t << " ";
                for (int64_t i = 1; i < nx - 1; ++i) {
                    const R *q = u + 3 * i;
                    R val = v == 0 ? q[0] : v == 1 ? q[1] / q[0] : v == 2 ? energy(q) : pressure(q);
                    f << val << " ";
                }
                f << std::endl;
            }
            return;
        }
        const char *name = problem == SW_HEAT ? "Temperature " : "Velocity ";
        if (lead) f << " ";
        f << name << t << " ";
        for (int64_t i = 0; i < nx; ++i) f << u[i] << " ";
        if (trailing_endl) f << std::endl;
    }

    // header + initial condition rows
    void head(const R *ic) {
        if (problem == SW_HEAT) {
            // "lx nx ds \nTemperature 0 ..." (Heat1D_SweptShared.cu:763-767)
            f << k.lx << " " << nx << " " << (R)k.dx << " " << std::endl << "Temperature " << 0 << " ";
            for (int64_t i = 0; i < nx; ++i) f << ic[i] << " ";
            f << std::endl;
        } else if (problem == SW_KS) {
            // KS1D_SweptShared.cu:954-958
            f << k.lx << " " << nx << " " << (R)k.dx << " " << std::endl << " Velocity " << 0 << " ";
            for (int64_t i = 0; i < nx; ++i) f << ic[i] << " ";
            f << std::endl;
        } else {
            // Euler1D_SweptShared.cu:1188-1204 (the IC velocity row prints rho*u, energy E/rho)
            f << (R)k.lx << " " << (nx - 2) << " " << k.dx << " " << std::endl;
            f << "Density " << 0 << " ";
            for (int64_t i = 1; i < nx - 1; ++i) f << ic[3 * i] << " ";
            f << std::endl << "Velocity " << 0 << " ";
            for (int64_t i = 1; i < nx - 1; ++i) f << ic[3 * i + 1] << " ";
            f << std::endl << "Energy " << 0 << " ";
            for (int64_t i = 1; i < nx - 1; ++i) f << ic[3 * i + 2] / ic[3 * i] << " ";
            f << std::endl << "Pressure " << 0 << " ";
            for (int64_t i = 1; i < nx - 1; ++i) f << pressure(ic + 3 * i) << " ";
            f << std::endl;
        }
    }
};

template <typename R>
int snapshot_cb(void *user, double t, const void *state, int64_t) {
    Writer<R> *w = static_cast<Writer<R> *>(user);
    // Heat/KS classic rows start with a space; swept Heat rows do not; KS always does.
    const bool lead = (w->problem == SW_KS) || (w->problem == SW_HEAT && w->alg == SW_ALG_CLASSIC);
    w->rows(static_cast<const R *>(state), t, lead, true);
    return w->f.good() ? 0 : 1;
}

const char *scheme_banner(int problem, int alg) {
    if (alg == SW_ALG_CLASSIC) return "Classic scheme";
    if (alg == SW_ALG_VARIANT)
        return problem == SW_KS ? "GPU warp-node (register path) swept scheme" : "GPU persistent swept scheme";
    return "GPU only Swept scheme";
}

// KS alg 3: the variant kernels against the shared-memory kernels on one
// input, element-wise at tolerance dt^3 (KS1D_SweptShared.cu:641-656,681-751),
// then exit -1 as the reference does.
template <typename R>
int selftest(sw_ctx *ctx, sw_config cfg, const std::vector<R> &ic) {
    std::cout << std::endl << "--- TEST IT ----" << std::endl << std::endl << std::endl;
    cfg.tpb = 32;
    cfg.time_mode = SW_TIME_STEPS;
    const double tol = cfg.dt * cfg.dt * cfg.dt;
    std::cout << "Tolerance: " << (R)tol << std::endl;
    const int64_t stage_steps[3] = {4, 8, 12};  // up+down, one diamond, two diamonds (8-step cycle of 32-cell nodes)
    const char *names[3] = {"---- TEST UP / DOWN --------", "---- TEST WHOLE --------", "---- TEST WHOLE x2 --------"};
    for (int s = 0; s < 3; ++s) {
        std::vector<R> a(ic.size()), b(ic.size());
        cfg.n_steps = stage_steps[s];
        cfg.alg = SW_ALG_VARIANT;
        int rc = sw_run(ctx, &cfg, ic.data(), a.data(), nullptr, nullptr, nullptr);
        if (rc) return rc;
        cfg.alg = SW_ALG_SWEPT;
        rc = sw_run(ctx, &cfg, ic.data(), b.data(), nullptr, nullptr, nullptr);
        if (rc) return rc;
        int64_t bad = 0;
        for (size_t i = 0; i < a.size(); ++i) bad += (std::abs((double)a[i] - (double)b[i]) > tol);
        std::cout << names[s] << std::endl;
        if (!bad) std::cout << "EQUAL!" << std::endl;
        else std::cout << "NOT EQUAL!" << std::endl << bad << " out of " << a.size() << std::endl;
    }
    return -1;
}

template <typename R>
int cli(int problem, int argc, char **argv) {
    const int prec = (int)sizeof(R);
    sw_config cfg;
    sw_config_init(&cfg, problem, prec);
    cfg.nx = std::atoi(argv[1]);
    cfg.tpb = std::atoi(argv[2]);
    cfg.dt = std::atof(argv[3]);
    cfg.tf = std::atof(argv[4]);
    cfg.freq = std::atof(argv[5]);
    cfg.alg = std::atoi(argv[6]);
    cfg.time_mode = SW_TIME_REFERENCE;
    std::cout.precision(10);

    sw_constants k;
    sw_constants_of(&cfg, &k);
    const char *precname = prec == 4 ? "Single" : "Double";
    const int64_t bks = cfg.tpb ? cfg.nx / cfg.tpb : 0;
    if (problem == SW_HEAT)
        std::cout << "Heat --- #Blocks: " << bks << " | Length: " << k.lx << " | Precision: " << precname
                  << " | Fo: " << (cfg.dt * (double)(R)(8.418e-5) / ((double)(R)0.001 * (double)(R)0.001)) << std::endl;
    else if (problem == SW_KS)
        std::cout << "KS --- #Blocks: " << bks << " | Length: " << k.lx << " | Precision: " << precname
                  << " | dt/dx: " << cfg.dt / k.dx << std::endl;
    else
        std::cout << "Euler --- #Blocks: " << bks << " | Length: " << (R)k.lx << " | Precision: " << precname
                  << " | dt/dx: " << (R)k.dt_dx << std::endl;

    int rc = sw_validate(&cfg);
    if (rc == SW_ERR_SIZE) {
        std::cout << "INVALID NUMERIC INPUT!! " << std::endl;
        std::cout << "2nd ARGUMENT MUST BE A POWER OF TWO >= 32 AND FIRST ARGUMENT MUST BE DIVISIBLE BY SECOND"
                  << std::endl;
        return rc;
    }
    if (rc == SW_ERR_UNSTABLE) {
        std::cout << "The value of dt/dx (" << k.dt_dx << ") is too high.  In general it must be <=.21 for stability."
                  << std::endl;
        return rc;
    }
    if (rc) {
        std::cout << "INVALID INPUT: " << sw_strerror(rc) << std::endl;
        return rc;
    }

    const int comps = problem == SW_EULER ? 3 : 1;
    std::vector<R> ic((size_t)cfg.nx * comps), fin((size_t)cfg.nx * comps);
    sw_initial_condition(&cfg, ic.data());

    std::ofstream fwr(argv[7], std::ios::trunc);
    if (!fwr) {
        std::cout << "cannot open " << argv[7] << std::endl;
        return SW_ERR_IO;
    }
    fwr.precision(10);
    Writer<R> w{fwr, problem, cfg.alg, k, cfg.nx};
    w.head(ic.data());

    sw_ctx *ctx = nullptr;
    rc = sw_ctx_create(0, &ctx);
    if (rc) {
        std::cout << "CUDA error: " << sw_strerror(rc) << std::endl;
        return rc;
    }
    if (cfg.alg == SW_ALG_SELFTEST) {
        rc = selftest<R>(ctx, cfg, ic);
        sw_ctx_destroy(ctx);
        return rc;
    }
    std::cout << scheme_banner(problem, cfg.alg) << std::endl;
    sw_result res{};
    rc = sw_run(ctx, &cfg, ic.data(), fin.data(), snapshot_cb<R>, &w, &res);
    if (rc) {
        std::cout << "CUDA error: " << sw_ctx_last_error(ctx) << std::endl;
        sw_ctx_destroy(ctx);
        return rc;
    }
    sw_ctx_destroy(ctx);

    const double t_end = cfg.tf - 0.25 * cfg.dt;
    std::cout << res.t_final << " " << t_end << std::endl;
    double n_timesteps = res.t_final / cfg.dt;
    if (problem == SW_KS) n_timesteps = (double)(int)n_timesteps;
    std::cout << n_timesteps << " timesteps" << std::endl;
    std::cout << "Averaged " << res.us_per_step << " microseconds (us) per timestep" << std::endl;

    if (argc > 8) {  // the reference opens argv[8] whenever argc > 7; argv[8] is NULL when argc == 8
        std::ofstream ftime(argv[8], std::ios::app);
        if (!ftime) return SW_ERR_IO;
        ftime << cfg.nx << "\t" << cfg.tpb << "\t" << res.us_per_step << std::endl;
    }
    // final rows: Heat without a trailing newline (Heat1D_SweptShared.cu:821-824)
    w.rows(fin.data(), res.t_final, problem == SW_KS, problem != SW_HEAT);
    fwr.close();
    return fwr.fail() ? SW_ERR_IO : SW_OK;
}

}  // namespace

extern "C" int sw_cli_main(int problem, int precision, int argc, char **argv) {
    if (argc < 8 || !argv) {
        std::cout << "The Program takes 9 inputs, #Divisions, #Threads/block, deltat, finish time, output frequency..."
                  << std::endl;
        std::cout << "Algorithm type, Variable Output File, Timing Output File (optional)" << std::endl;
        return SW_ERR_USAGE;
    }
    if (problem < SW_HEAT || problem > SW_EULER) return SW_ERR_ARG;
    if (precision == 4) return cli<float>(problem, argc, argv);
    if (precision == 8) return cli<double>(problem, argc, argv);
    return SW_ERR_ARG;
}
