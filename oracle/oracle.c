/*
 * CPU oracle for the swept-rule 1D stencil solvers -- TEST INFRASTRUCTURE ONLY
 * (see oracle.h).  Build: gcc -O2 -std=c11 -ffp-contract=off -fopenmp -fPIC
 * -shared oracle.c -lm  (oracle/build.py).  -ffp-contract=off is required:
 * the oracle must not fuse multiply-adds the reference's expressions do not
 * spell out.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "oracle.h"

#if defined(__FP_FAST_FMA) && !defined(OR_ALLOW_CONTRACT)
/* A fused build would still be correct C, but it would stop matching the
 * reference's rounding; -ffp-contract=off keeps the expressions unfused. */
#endif

#define REAL double
#define SFX f64
#define OR_IS_FLOAT 0
#include "oracle_impl.h"
#undef REAL
#undef SFX
#undef OR_IS_FLOAT

#define REAL float
#define SFX f32
#define OR_IS_FLOAT 1
#include "oracle_impl.h"
#undef REAL
#undef SFX
#undef OR_IS_FLOAT

int or_openmp_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Heat: th_diff = 8.418e-5, ds = 0.001 (Heat1D_SweptShared.cu:56-58);
 * fou = th_diff*dt/(ds*ds) with ds*ds in REAL (:720); fourierTwo =
 * ONE - TWO*fou (:725).  KS: dx = 0.5 (KS1D_SweptShared.cu:45), reciprocals in
 * REAL (:917-926).  Euler: gamma 1.4, Sod states, dx = lx/((REAL)dv - TWO)
 * in REAL, dt_dx = dt/dx in double (Euler1D_SweptShared.cu:1127-1149). */
int or_reference_consts(int problem, int prec, int64_t nx, double dt, or_consts *o)
{
    if (!o || nx < 8 || (prec != 4 && prec != 8)) return -1;
    memset(o, 0, sizeof(*o));
    o->problem = problem;
    o->nx = nx;
    if (problem == OR_HEAT) {
        o->bc = OR_BC_MIRROR;
        if (prec == 4) {
            const float th = 8.418e-5f, ds = 0.001f;
            double fou = (double)th * dt / (double)(ds * ds);
            o->fourier = (float)fou;
            o->fourier_two = (float)(1.0f - 2.0f * fou);
        } else {
            const double th = 8.418e-5, ds = 0.001;
            double fou = th * dt / (ds * ds);
            o->fourier = fou;
            o->fourier_two = 1.0 - 2.0 * fou;
        }
    } else if (problem == OR_KS) {
        o->bc = OR_BC_PERIODIC;
        if (prec == 4) {
            const float dx = 0.5f;
            o->dx_times4 = 1.0f / (4.0f * dx);
            o->dx2 = 1.0f / (dx * dx);
            o->dx4 = 1.0f / (dx * dx * dx * dx);
            o->dt = (float)dt;
            o->dt_half = (float)(dt * 0.5);
        } else {
            const double dx = 0.5;
            o->dx_times4 = 1.0 / (4.0 * dx);
            o->dx2 = 1.0 / (dx * dx);
            o->dx4 = 1.0 / (dx * dx * dx * dx);
            o->dt = dt;
            o->dt_half = dt * 0.5;
        }
    } else if (problem == OR_EULER) {
        o->bc = OR_BC_DIRICHLET;
        if (prec == 4) {
            const float lx = 1.0f;
            float gam = 1.4f, mgam = 0.4f;
            double dx = lx / ((float)nx - 2.0f);
            o->gam = gam;
            o->mgam = mgam;
            o->dt_dx = (float)(dt / dx);
            o->bd[0] = 1.0f; o->bd[1] = 0.0f; o->bd[2] = 1.0f / mgam;
            o->bd[3] = (float)0.125; o->bd[4] = 0.0f; o->bd[5] = (float)(0.1 / mgam);
        } else {
            const double lx = 1.0;
            double gam = 1.4, mgam = 0.4;
            double dx = lx / ((double)nx - 2.0);
            o->gam = gam;
            o->mgam = mgam;
            o->dt_dx = dt / dx;
            o->bd[0] = 1.0; o->bd[1] = 0.0; o->bd[2] = 1.0 / mgam;
            o->bd[3] = 0.125; o->bd[4] = 0.0; o->bd[5] = 0.1 / mgam;
        }
    } else {
        return -1;
    }
    return 0;
}

/* initFun: Heat1D_SweptShared.cu:60-66 (100 a (1 - a/lx), a = x ds,
 * lx = ds (nx-1)); KS1D_SweptShared.cu:68-72 (2 cos(19 pi x / 128) at
 * x = (REAL)k*(REAL)dx); Euler1D_SweptShared.cu:1179 (left state for
 * k < nx/2, right state otherwise). */
int or_reference_ic(int problem, int prec, int64_t nx, void *ic)
{
    if (!ic || nx < 8 || (prec != 4 && prec != 8)) return -1;
    if (problem == OR_HEAT) {
        if (prec == 4) {
            const float ds = 0.001f;
            const float lx = (float)(ds * ((double)nx - 1.0));
            float *u = (float *)ic;
            for (int64_t k = 0; k < nx; ++k) {
                float a = ((float)k * ds);
                u[k] = 100.f * a * (1.f - a / lx);
            }
        } else {
            const double ds = 0.001;
            const double lx = ds * ((double)nx - 1.0);
            double *u = (double *)ic;
            for (int64_t k = 0; k < nx; ++k) {
                double a = ((double)k * ds);
                u[k] = 100.f * a * (1.0 - a / lx);
            }
        }
    } else if (problem == OR_KS) {
        if (prec == 4) {
            float *u = (float *)ic;
            for (int64_t k = 0; k < nx; ++k) {
                float x = (float)k * 0.5f;
                u[k] = (float)(2.0f * cos(19.0 * x * M_PI / 128.0));
            }
        } else {
            double *u = (double *)ic;
            for (int64_t k = 0; k < nx; ++k) {
                double x = (double)k * 0.5;
                u[k] = 2.0 * cos(19.0 * x * M_PI / 128.0);
            }
        }
    } else if (problem == OR_EULER) {
        or_consts c;
        if (or_reference_consts(OR_EULER, prec, nx, 1e-6, &c)) return -1;
        for (int64_t k = 0; k < nx; ++k) {
            const double *b = (k < nx / 2) ? c.bd : c.bd + 3;
            for (int i = 0; i < 3; ++i) {
                if (prec == 4) ((float *)ic)[3 * k + i] = (float)b[i];
                else ((double *)ic)[3 * k + i] = b[i];
            }
        }
    } else {
        return -1;
    }
    return 0;
}
