/*
 * Reference harness -- TEST INFRASTRUCTURE ONLY (builds oracle/_ref/).
 *
 * Compiles one of the reference programs, unmodified, from where it lies
 * (REF_SRC = .../SweptSource/<Problem>1D_SweptShared.cu, passed by
 * oracle/build.py) and exposes its own host-callable stencil code through a
 * small C ABI, so the oracle can be checked against the reference's arithmetic
 * bit for bit.  Nothing here is product code and nothing is copied: the
 * reference file is #included at build time.
 *
 * Shims (preprocessor only, no source edits):
 *  - `main` is renamed so the harness can provide the entry points;
 *  - KS: its stencil functions are __device__ only (KS1D_SweptShared.cu:111-187),
 *    so __device__ is widened to __host__ __device__, and the pre-CUDA-9
 *    __shfl_up/__shfl_down used by its register kernels are mapped to the
 *    _sync forms (the kernels are compiled, never launched here).
 * The classic loops below restate classicHeat / classicKS / classicEuler
 * (Heat1D_SweptShared.cu:132-145, KS1D_SweptShared.cu:189-207,
 * Euler1D_SweptShared.cu:400-426) around the reference's own functions.
 */
#include <cuda_runtime.h>
#include <cstdint>
#include <cstring>
#include <vector>

#if REF_PROBLEM == 1
#undef __device__
#define __device__ __location__(host) __location__(device)
#define __shfl_up(v, d) __shfl_up_sync(0xffffffffu, v, d)
#define __shfl_down(v, d) __shfl_down_sync(0xffffffffu, v, d)
#ifdef REF_KS_DIVIDE
/* The DIVISE build (KS1D_SweptShared.cu:111-132): its main() does not compile
 * as shipped (a missing brace at :905), so DIVISE is defined for the stencil
 * functions only.  It is saved undefined, defined, and restored to undefined
 * by the first expansion of classicKS (the kernel after the stencil functions,
 * :189), before main's own #ifdef DIVISE. */
#pragma push_macro("DIVISE")
#define DIVISE 1
#define classicKS _Pragma("pop_macro(\"DIVISE\")") classicKS
#endif
#endif

#define main reference_program_main
#include REF_SRC
#undef main
#ifdef REF_KS_DIVIDE
#undef classicKS
#endif

extern "C" int ref_real_size(void) { return (int)sizeof(REAL); }

#if REF_PROBLEM == 0 /* ---------------------------------------------- Heat */
extern "C" void ref_ic(int64_t nx, REAL *out)
{
    const double lx = ds * ((double)nx - 1.0);
    for (int64_t k = 0; k < nx; ++k) out[k] = initFun((int)k, ds, lx);
}
extern "C" void ref_classic(REAL *u, int64_t nx, double fourier, double fourier_two, int64_t nsteps)
{
    hostC.fourier = (REAL)fourier;
    hostC.fourierTwo = (REAL)fourier_two;
    hostC.idxend = (int)nx - 1;
    std::vector<REAL> w(nx);
    REAL *in = u, *out = w.data();
    for (int64_t n = 0; n < nsteps; ++n) {
        for (int gid = 0; gid < (int)nx; ++gid) {
            int gidz[3];
            gidz[0] = (gid == 0) ? (gid + 1) : (gid - 1);
            gidz[1] = gid;
            gidz[2] = (gid == hostC.idxend) ? (gid - 1) : (gid + 1);
            out[gid] = execFunc(in, gidz);
        }
        REAL *t = in; in = out; out = t;
    }
    if (in != u) std::memcpy(u, in, sizeof(REAL) * nx);
}
#elif REF_PROBLEM == 1 /* ------------------------------------------------- KS */
extern "C" void ref_ic(int64_t nx, REAL *out)
{
    for (int64_t k = 0; k < nx; ++k) out[k] = initFun((REAL)k * (REAL)dx);
}
extern "C" void ref_classic(REAL *u, int64_t nx, double c4, double d2, double d4, double dt_, double dth,
                            int64_t nsteps)
{
    disc.dxTimes4 = (REAL)c4;
    disc.dx2 = (REAL)d2;
    disc.dx4 = (REAL)d4;
    disc.dt = (REAL)dt_;
    disc.dt_half = (REAL)dth;
    disc.idxend = (int)nx - 1;
    std::vector<REAL> w(nx);
    const int lastidx = (int)nx - 1;
    for (int64_t n = 0; n < nsteps; ++n) {
        for (int pass = 0; pass < 2; ++pass) {
            const REAL *in = pass ? w.data() : u;
            REAL *out = pass ? u : w.data();
            for (int gid = 0; gid < (int)nx; ++gid) {
                int gidz[5];
                for (int k = -2; k < 3; k++) gidz[k + 2] = (gid + k) & lastidx;
                if (pass) out[gid] += finalStep(in, gidz);
                else out[gid] = stutterStep(in, gidz);
            }
        }
    }
}
#else /* --------------------------------------------------------------- Euler */
extern "C" void ref_set(int64_t nx, double gam, double mgam, double dt_dx, const double *b6)
{
    dimz.gam = (REAL)gam;
    dimz.mgam = (REAL)mgam;
    dimz.dt_dx = (REAL)dt_dx;
    dimz.idxend = (int)nx - 1;
    dimz.idxend_1 = (int)nx - 2;
    bd[0].x = (REAL)b6[0]; bd[0].y = (REAL)b6[1]; bd[0].z = (REAL)b6[2];
    bd[1].x = (REAL)b6[3]; bd[1].y = (REAL)b6[4]; bd[1].z = (REAL)b6[5];
}
extern "C" void ref_classic(REAL *q, int64_t nx, int64_t nsteps)
{
    REALthree *u = (REALthree *)q;
    std::vector<REALthree> w(nx);
    for (int64_t n = 0; n < nsteps; ++n) {
        for (int pass = 0; pass < 2; ++pass) {
            REALthree *in = pass ? w.data() : u;
            REALthree *out = pass ? u : w.data();
            for (int gid = 0; gid < (int)nx; ++gid) {
                const bool tx = gid == 0, ty = gid == 1, tz = gid == dimz.idxend_1, tw = gid == dimz.idxend;
                if (tx) { out[gid] = bd[0]; continue; }
                if (tw) { out[gid] = bd[1]; continue; }
                if (pass) out[gid] += eulerFinalStep(in, gid, ty, tz);
                else out[gid] = eulerStutterStep(in, gid, ty, tz);
            }
        }
    }
}
/* pressure() and energy() as the .dat writer uses them (Euler1D_SweptShared.cu:183-193,752-759) */
extern "C" void ref_derived(const REAL *q, int64_t nx, REAL *p, REAL *e)
{
    const REALthree *u = (const REALthree *)q;
    for (int64_t k = 0; k < nx; ++k) {
        p[k] = pressure(u[k]);
        e[k] = energy(u[k]);
    }
}
#endif
