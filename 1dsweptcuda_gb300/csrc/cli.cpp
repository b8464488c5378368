// sw_cli_main: the reference programs' main() over the C ABI.
//
// argv, banners, the .dat solution file and the appended timing row follow
// Heat1D_SweptShared.cu:697-836, KS1D_SweptShared.cu:866-1029 and
// Euler1D_SweptShared.cu:1112-1287: the same row names and leading spaces,
// ostream precision 10 for the solution (values printed in the run's
// precision), default precision for the timing row.
//
// A solution path ending in ".npy" gets the same rows in binary instead: a
// NumPy structured array of records (var int32, t float64, v REAL[n]), n = nx
// (Euler nx - 2), rows in the .dat order with the .dat's values unrounded.
// Record 0 is the header: var = -1, t = lx, v[0] = n, v[1] = dx, v[2] = the
// problem (0 Heat, 1 KS, 2 Euler).  The var index is the row name's position
// in Temperature | Velocity | Density, Velocity, Energy, Pressure.
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

// The .npy form of Writer: same rows, same values, unrounded binary records.
template <typename R>
struct NpyWriter {
    std::FILE *f = nullptr;
    int problem;
    int alg;
    const sw_constants &k;
    int64_t nx;
    int64_t n_rows = 0;
    long shape_at = 0;
    bool ok = true;
    std::vector<R> buf;
    static constexpr int kShapeWidth = 20;

    int64_t n() const { return problem == SW_EULER ? nx - 2 : nx; }
    R pressure(const R *q) const { return (R)k.mgam * (q[2] - ((R)0.5 * q[1] * q[1] / q[0])); }
    R energy(const R *q) const {
        R u = q[1] / q[0];
        return q[2] / q[0] - (R)0.5 * u * u;
    }

    // NPY 1.0 header; the row count is patched in by finish()
    bool open(const char *path) {
        f = std::fopen(path, "wb");
        if (!f) return false;
        const char *real = sizeof(R) == 4 ? "<f4" : "<f8";
        std::string h = "{'descr': [('var', '<i4'), ('t', '<f8'), ('v', '" + std::string(real) + "', (" +
                        std::to_string(n()) + ",))], 'fortran_order': False, 'shape': (";
        const size_t shape_off = h.size();
        h += std::string(kShapeWidth, ' ') + ",), }";
        while ((10 + h.size() + 1) % 64) h += ' ';
        h += '\n';
        const unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
        const uint16_t len = (uint16_t)h.size();
        const unsigned char lenb[2] = {(unsigned char)(len & 0xff), (unsigned char)(len >> 8)};
        ok = std::fwrite(magic, 1, 8, f) == 8 && std::fwrite(lenb, 1, 2, f) == 2 &&
             std::fwrite(h.data(), 1, h.size(), f) == h.size();
        shape_at = (long)(10 + shape_off);
        buf.assign((size_t)n(), R(0));
        return ok;
    }
    void record(int32_t var, double t, const R *v) {
        unsigned char hdr[12];
        std::memcpy(hdr, &var, 4);
        std::memcpy(hdr + 4, &t, 8);
        ok = ok && std::fwrite(hdr, 1, 12, f) == 12 && std::fwrite(v, sizeof(R), (size_t)n(), f) == (size_t)n();
        ++n_rows;
    }
    // one Euler row of derived values from the device-layout-free host state (3 per cell)
    void euler_row(int var, double t, const R *u, bool ic) {
        for (int64_t i = 1; i < nx - 1; ++i) {
            const R *q = u + 3 * i;
            R val;
            if (var == 0) val = q[0];
            else if (var == 1) val = ic ? q[1] : q[1] / q[0];  // the IC row holds rho*u (as the .dat)
            else if (var == 2) val = ic ? q[2] / q[0] : energy(q);
            else val = pressure(q);
            buf[(size_t)(i - 1)] = val;
        }
        record(var, t, buf.data());
    }
    void head(const R *ic) {
        std::fill(buf.begin(), buf.end(), R(0));
        buf[0] = (R)n();
        buf[1] = (R)k.dx;
        buf[2] = (R)problem;
        record(-1, problem == SW_EULER ? (double)(R)k.lx : k.lx, buf.data());
        rows_of(ic, 0.0, true);
    }
    void rows_of(const R *u, double t, bool ic) {
        if (problem == SW_EULER) {
            for (int v = 0; v < 4; ++v) euler_row(v, t, u, ic);
        } else {
            record(0, t, u);
        }
    }
    void rows(const R *u, double t, bool, bool) { rows_of(u, t, false); }
    bool good() const { return ok; }
    bool finish() {
        if (!f) return false;
        std::string num = std::to_string(n_rows);
        num = std::string(kShapeWidth - num.size(), ' ') + num;
        ok = ok && std::fseek(f, shape_at, SEEK_SET) == 0 && std::fwrite(num.data(), 1, num.size(), f) == num.size();
        ok = (std::fclose(f) == 0) && ok;
        f = nullptr;
        return ok;
    }
};

template <typename R>
bool writer_good(const Writer<R> &w) { return w.f.good(); }
template <typename R>
bool writer_good(const NpyWriter<R> &w) { return w.good(); }

template <typename R, typename W>
int snapshot_cb(void *user, double t, const void *state, int64_t) {
    W *w = static_cast<W *>(user);
    // Heat/KS classic rows start with a space; swept Heat rows do not; KS always does.
    const bool lead = (w->problem == SW_KS) || (w->problem == SW_HEAT && w->alg == SW_ALG_CLASSIC);
    w->rows(static_cast<const R *>(state), t, lead, true);
    return writer_good(*w) ? 0 : 1;
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

template <typename R, typename W>
int run_and_write(W &w, sw_config cfg, const std::vector<R> &ic, std::vector<R> &fin, int argc, char **argv) {
    const int problem = cfg.problem;
    sw_ctx *ctx = nullptr;
    int rc = sw_ctx_create(0, &ctx);
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
    rc = sw_run(ctx, &cfg, ic.data(), fin.data(), snapshot_cb<R, W>, &w, &res);
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
    return writer_good(w) ? SW_OK : SW_ERR_IO;
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
    // The reference chooses its KS division form when it is compiled (-DDIVISE,
    // KS1D_SweptShared.cu:111,904); these programs take it from the environment.
    if (problem == SW_KS) {
        const char *d = std::getenv("SWEPT1D_KS_DIVIDE");
        if (d && *d && std::strcmp(d, "0") != 0) cfg.flags |= SW_FLAG_KS_DIVIDE;
    }
    // The reference's alg 2 for Heat and Euler is its hybrid variant (the split
    // node on the CPU); here alg 2 is the GPU-only persistent kernel unless
    // SWEPT1D_HOST_TILE asks for the host tile (alg 1 or 2).
    {
        const char *t = std::getenv("SWEPT1D_HOST_TILE");
        if (t && *t && std::strcmp(t, "0") != 0) cfg.flags |= SW_FLAG_HOST_TILE;
    }
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

    const std::string out_path = argv[7];
    const bool npy = out_path.size() >= 4 && out_path.compare(out_path.size() - 4, 4, ".npy") == 0;
    if (npy) {
        NpyWriter<R> w{nullptr, problem, cfg.alg, k, cfg.nx};
        if (!w.open(argv[7])) {
            std::cout << "cannot open " << argv[7] << std::endl;
            return SW_ERR_IO;
        }
        w.head(ic.data());
        rc = run_and_write<R>(w, cfg, ic, fin, argc, argv);
        const bool written = w.finish();
        return rc ? rc : (written ? SW_OK : SW_ERR_IO);
    }
    std::ofstream fwr(argv[7], std::ios::trunc);
    if (!fwr) {
        std::cout << "cannot open " << argv[7] << std::endl;
        return SW_ERR_IO;
    }
    fwr.precision(10);
    Writer<R> w{fwr, problem, cfg.alg, k, cfg.nx};
    w.head(ic.data());
    rc = run_and_write<R>(w, cfg, ic, fin, argc, argv);
    fwr.close();
    return rc ? rc : (fwr.fail() ? SW_ERR_IO : SW_OK);
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
