/*
 * CPU oracle for the swept-rule 1D stencil solvers -- TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and the cpu_baseline / reference legs of
 * bench.py load this library, to check results and to time the CPU baseline.  The product path (the
 * CUDA library under 1dsweptcuda_gb300/) never links, loads or calls it.
 *
 * It restates, in plain C, the arithmetic of the reference programs
 * (Niemeyer-Research-Group/1DSweptCUDA):
 *   Heat  : execFunc + classicHeat          SweptSource/Heat1D_SweptShared.cu:121-145
 *   KS    : convect/secondDer/fourthDer,
 *           stutterStep/finalStep/classicKS SweptSource/KS1D_SweptShared.cu:136-207
 *           (and the DIVISE build's forms,  :111-132, with or_consts.divide)
 *   Euler : pressure ... eulerFinalStep,
 *           classicEuler                    SweptSource/Euler1D_SweptShared.cu:183-426
 * in the reference's own operation order, compiled with -ffp-contract=off so
 * that nothing is fused.  The result is bit-identical to the reference's
 * host-compiled stencil functions (pinned by tests/golden, made from the
 * reference sources by oracle/ref_harness.cu).
 *
 * It also holds a CPU model of the swept decomposition used on the GPU
 * (up-triangle / diamonds / down-triangle over half-tile edge slots), so the
 * tile logic can be checked against the classic loop on the CPU.
 *
 * State layout: Heat and KS use REAL[nx]; Euler uses REAL[3*nx] holding
 * (rho, rho*u, E) per cell, the layout of the reference's REALthree arrays.
 */
#ifndef SWEPT1D_ORACLE_H
#define SWEPT1D_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { OR_HEAT = 0, OR_KS = 1, OR_EULER = 2 };
enum { OR_BC_MIRROR = 1, OR_BC_PERIODIC = 2, OR_BC_DIRICHLET = 3 };

/* Problem constants, stored in the precision of the run (float fields are
 * rounded the way the reference's main() rounds them). */
typedef struct or_consts {
    int problem;
    int bc;
    int64_t nx;
    /* Heat (heatConstants, Heat1D_SweptShared.cu:43-54) */
    double fourier, fourier_two;
    /* KS (discConstants, KS1D_SweptShared.cu:47-59) */
    double dx_times4, dx2, dx4, dt, dt_half;
    /* Euler (dimensions + dbd, Euler1D_SweptShared.cu:73-93) */
    double gam, mgam, dt_dx;
    double bd[6]; /* left (rho, rho u, E), right (rho, rho u, E) */
    /* KS: 1 = the DIVISE build (KS1D_SweptShared.cu:111-132, 904-914):
     * dx_times4, dx2, dx4 hold 4dx, dx^2, dx^4 and the terms are divided */
    int divide;
} or_consts;

/* Advance `nsteps` full time steps of the classic scheme in place.
 * Heat: one FTCS step per time step.  KS/Euler: predictor + corrector. */
int or_classic_f64(const or_consts *c, double *u, int64_t nsteps);
int or_classic_f32(const or_consts *c, float *u, int64_t nsteps);

/* Same loop with OpenMP over cells (CPU baseline); nthreads<=0 = all. */
int or_classic_omp_f64(const or_consts *c, double *u, int64_t nsteps, int nthreads);
int or_classic_omp_f32(const or_consts *c, float *u, int64_t nsteps, int nthreads);

/* Swept decomposition on the CPU: tiles of width `tpb`, `n_diamonds` diamond
 * passes between the up-triangle and the down-triangle.  Advances
 * (n_diamonds + 1) * tpb / (2 * R * S) time steps, R = stencil radius per
 * sub-step (1 Heat, 2 KS/Euler), S = sub-steps per step (1 Heat, 2 KS/Euler).
 * Returns the number of time steps advanced, or a negative error. */
int64_t or_swept_f64(const or_consts *c, double *u, int tpb, int64_t n_diamonds);
int64_t or_swept_f32(const or_consts *c, float *u, int tpb, int64_t n_diamonds);

/* Pressure and energy for the .dat writer (Euler1D_SweptShared.cu:183-193,752-759). */
double or_euler_pressure_f64(const or_consts *c, const double *q3);
double or_euler_pressure_f32(const or_consts *c, const float *q3);

int or_openmp_max_threads(void);

/* The constants and initial condition the reference's main() builds for a
 * CLI run (Heat1D_SweptShared.cu:712-754, KS1D_SweptShared.cu:880-945,
 * Euler1D_SweptShared.cu:1127-1179), rounded through REAL as it does.
 * prec is 4 (float build) or 8 (double build).  The IC buffer holds nx
 * (Heat, KS) or 3*nx (Euler) values of that precision.  Heat keeps the
 * reference's insulated (mirror) ends, KS is periodic, Euler holds cells 0
 * and nx-1 at the Sod states.  Returns 0, or -1 on bad arguments. */
int or_reference_consts(int problem, int prec, int64_t nx, double dt, or_consts *out);
int or_reference_ic(int problem, int prec, int64_t nx, void *ic);

#ifdef __cplusplus
}
#endif
#endif
