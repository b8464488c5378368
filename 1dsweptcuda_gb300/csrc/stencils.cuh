// Stencil arithmetic of the three schemes, device side.
//
// Each function keeps the operation order of the reference's expression it
// restates and spells every operation with a round-to-nearest intrinsic, so
// the compiler can neither fuse nor reorder: the results are bit-identical to
// the reference's host-compiled stencil code and to the oracle, whatever
// -fmad setting a build uses.
#pragma once

#include <cuda_runtime.h>

#include <cmath>

#include "exact_int.h"
#include "sw_internal.h"

// k_ks_div.cu compiles the kernel headers (this file, engine.cuh,
// persistent.cuh) a second time with SW_KS_DIVIDE_TU defined: the KS
// right-hand side then divides (SW_FLAG_KS_DIVIDE), and every template
// instance of that build lands in the inline namespace sw::ks_divide, apart
// from the default build's.  The default build's kernels never carry the
// divisions, so its register allocation is the same as without them.
#ifdef SW_KS_DIVIDE_TU
#define SW_KERNELS_BEGIN namespace sw { inline namespace ks_divide {
#define SW_KERNELS_END } }
#else
#define SW_KERNELS_BEGIN namespace sw {
#define SW_KERNELS_END }
#endif

SW_KERNELS_BEGIN

// ---- correctly rounded scalar operations, both precisions.  Host builds of
// these functions (the host tile of the hybrid variant, csrc/host_tile.cu) use
// the IEEE operation itself; that translation unit is compiled with
// -ffp-contract=off, so nothing is fused there either.
#ifdef __CUDA_ARCH__
#define SW_OP(dev, host) dev
#else
#define SW_OP(dev, host) host
#endif
SW_HD double ad(double a, double b) { return SW_OP(__dadd_rn(a, b), a + b); }
SW_HD float ad(float a, float b) { return SW_OP(__fadd_rn(a, b), a + b); }
SW_HD double sb(double a, double b) { return SW_OP(__dsub_rn(a, b), a - b); }
SW_HD float sb(float a, float b) { return SW_OP(__fsub_rn(a, b), a - b); }
SW_HD double ml(double a, double b) { return SW_OP(__dmul_rn(a, b), a * b); }
SW_HD float ml(float a, float b) { return SW_OP(__fmul_rn(a, b), a * b); }
SW_HD double dv(double a, double b) { return SW_OP(__ddiv_rn(a, b), a / b); }
SW_HD float dv(float a, float b) { return SW_OP(__fdiv_rn(a, b), a / b); }
SW_HD double sq(double a) { return SW_OP(__dsqrt_rn(a), ::sqrt(a)); }
SW_HD float sq(float a) { return SW_OP(__fsqrt_rn(a), ::sqrtf(a)); }
SW_HD double mn(double a, double b) { return ::fmin(a, b); }
SW_HD float mn(float a, float b) { return ::fminf(a, b); }
SW_HD double ab(double a) { return ::fabs(a); }
SW_HD float ab(float a) { return ::fabsf(a); }

SW_HD double fm(double a, double b, double c) { return SW_OP(__fma_rn(a, b, c), ::fma(a, b, c)); }
SW_HD float fm(float a, float b, float c) { return SW_OP(__fmaf_rn(a, b, c), ::fmaf(a, b, c)); }

// Products whose FP64 form runs on the integer pipe (exact_int.h), with the
// bits of the FP64 multiply: 6 * c, and x * f with f = 2^k.  FP32 keeps its
// multiply: the FP32 kernels are bound by instruction issue, not by a pipe.
SW_HD double ml6(double c) { return mul6(c); }
SW_HD float ml6(float c) { return ml(6.0f, c); }
SW_HD double mlp2(double x, double f, int k) { return mul_pow2(x, f, k); }
SW_HD float mlp2(float x, float f, int) { return ml(x, f); }
// A general FP64 product on the integer pipe (mul_int_fast): bad is set where
// the value must be recomputed with ml.  FP32 multiplies.
SW_HD double mlq(double a, double b, uint32_t &bad) { return mul_int_fast(a, b, bad); }
SW_HD float mlq(float a, float b, uint32_t &) { return ml(a, b); }

// ---------------------------------------------------------------- Heat
// execFunc, Heat1D_SweptShared.cu:121-130: fourier*(T[l] + T[r]) + fourierTwo*T[c]
template <typename T>
SW_HD T heat_step(const Params<T> &p, T l, T c, T r) {
    return ad(ml(p.fo, ad(l, r)), ml(p.fo2, c));
}
// The same with both products on the integer pipe (mlq): in FP64 two FP64-pipe
// operations per cell-update instead of four.
template <typename T>
SW_HD T heat_step_q(const Params<T> &p, T l, T c, T r, uint32_t &bad) {
    return ad(mlq(p.fo, ad(l, r), bad), mlq(p.fo2, c, bad));
}

// ------------------------------------------------------------------ KS
// convect + secondDer + fourthDer (reciprocal build), KS1D_SweptShared.cu:136-155:
//   ((r*r - l*l)*c4 + (l + r - 2c)*d2) + (ll - 4l + 6c - 4r + rr)*d4
// A product by an exact power of two is exact, so folding it into the
// following add as one fused multiply-add rounds exactly as the separate
// multiply and add do.  That holds for the literal 2 and 4 always, and for the
// reciprocals c4, d2, d4 when they are powers of two (KS_POW2, set by the host:
// 0.5, 4, 16 at the reference's dx = 0.5).  Results stay bit-identical to the
// reference's expression while the FP64 pipe does 15 operations instead of 20
// (barring overflow or underflow of the scaled terms, ~1e+-300).
// KS_DIVIDE is the DIVISE build (KS1D_SweptShared.cu:111-132): each term divided
// by 4dx, dx^2, dx^4, summed in the same order.
// In FP64 two of the products run on the integer pipe with the same bits: 6c
// (ml6) and, under KS_POW2, sec * d2 (mlp2, d2 = 2^d2_e): 12 FP64-pipe
// operations per sub-step where the cell's square is supplied.
template <typename T>
SW_HD T ks_rhs_sq(const Params<T> &p, T ll, T l, T c, T r, T rr, T l2, T r2) {
    const T conv = sb(r2, l2);  // l2 = l*l, r2 = r*r
    const T sec = fm(T(-2), c, ad(l, r));                        // (l + r) - 2c
    const T fourth = ad(fm(T(-4), r, ad(fm(T(-4), l, ll), ml6(c))), rr);  // ((ll - 4l) + 6c) - 4r + rr
#ifdef SW_KS_DIVIDE_TU
    return ad(ad(dv(conv, p.c4), dv(sec, p.d2)), dv(fourth, p.d4));
#else
    if (p.ks_form == KS_POW2) return fm(fourth, p.d4, fm(conv, p.c4, mlp2(sec, p.d2, p.d2_e)));
    return ad(ad(ml(conv, p.c4), ml(sec, p.d2)), ml(fourth, p.d4));
#endif
}
template <typename T>
SW_HD T ks_rhs(const Params<T> &p, T ll, T l, T c, T r, T rr) {
    return ks_rhs_sq(p, ll, l, c, r, rr, ml(l, l), ml(r, r));
}
// stutterStep, KS1D_SweptShared.cu:159-164: u - dt/2 * rhs
template <typename T>
SW_HD T ks_predict(const Params<T> &p, T ll, T l, T c, T r, T rr) {
    return sb(c, ml(p.dth, ks_rhs(p, ll, l, c, r, rr)));
}
// finalStep, KS1D_SweptShared.cu:166-171 added to u (classicKS :201-202): u + (-dt * rhs)
template <typename T>
SW_HD T ks_correct(const Params<T> &p, T u, T ll, T l, T c, T r, T rr) {
    return ad(u, ml(-p.dt, ks_rhs(p, ll, l, c, r, rr)));
}
// The same with the squares l*l and r*r of the neighbours supplied (each cell's
// square is then formed once, by the thread that produced the value, instead
// of by both of its neighbours; the product is the same __dmul_rn either way).
template <typename T>
SW_HD T ks_predict_sq(const Params<T> &p, T ll, T l, T c, T r, T rr, T l2, T r2) {
    return sb(c, ml(p.dth, ks_rhs_sq(p, ll, l, c, r, rr, l2, r2)));
}
template <typename T>
SW_HD T ks_correct_sq(const Params<T> &p, T u, T ll, T l, T c, T r, T rr, T l2, T r2) {
    return ad(u, ml(-p.dt, ks_rhs_sq(p, ll, l, c, r, rr, l2, r2)));
}
// The same with the product by dt/2 or -dt on the integer pipe (mlq): in FP64
// 10 FP64-pipe operations per sub-step instead of 11, the cell's square being
// the other product a sub-step needs (engine.cuh forms it with mlq as well).
template <typename T>
SW_HD T ks_predict_q(const Params<T> &p, T ll, T l, T c, T r, T rr, T l2, T r2, uint32_t &bad) {
    return sb(c, mlq(p.dth, ks_rhs_sq(p, ll, l, c, r, rr, l2, r2), bad));
}
template <typename T>
SW_HD T ks_correct_q(const Params<T> &p, T u, T ll, T l, T c, T r, T rr, T l2, T r2, uint32_t &bad) {
    return ad(u, mlq(-p.dt, ks_rhs_sq(p, ll, l, c, r, rr, l2, r2), bad));
}

// ------------------------------------------------- paired FP32 (sm_100+)
// Two cells per instruction with the f32x2 add and fma (__fadd2_rn,
// __ffma2_rn).  Each component rounds as its scalar counterpart does, so a
// pair gives the same bits as two scalar evaluations -- provided no multiply
// is merged with a following add into one fma, which the compiler was found to
// do with the f32x2 multiply even with -fmad=false.  So a product is always
// formed as fma(a, b, nz) with nz = -0.0 passed at run time (Params::nz): the
// same single rounding of a * b, and an fma is never merged again.
__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 ad2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 ml2(const Params<float> &p, float2 a, float2 b) { return __ffma2_rn(a, b, dup2(p.nz)); }

// heat_step on a pair of cells
__device__ __forceinline__ float2 heat_step2(const Params<float> &p, float2 l, float2 c, float2 r) {
    return ad2(ml2(p, dup2(p.fo), ad2(l, r)), ml2(p, dup2(p.fo2), c));
}

// --------------------------------------------------------------- Euler
template <typename T>
struct Q3 {
    T x, y, z;
};
template <typename T>
SW_HD Q3<T> q3(T x, T y, T z) { return Q3<T>{x, y, z}; }
template <typename T>
SW_HD Q3<T> qadd(Q3<T> a, Q3<T> b) { return q3(ad(a.x, b.x), ad(a.y, b.y), ad(a.z, b.z)); }
template <typename T>
SW_HD Q3<T> qsub(Q3<T> a, Q3<T> b) { return q3(sb(a.x, b.x), sb(a.y, b.y), sb(a.z, b.z)); }
template <typename T>
SW_HD Q3<T> qscale(T s, Q3<T> a) { return q3(ml(s, a.x), ml(s, a.y), ml(s, a.z)); }

// pressure, Euler1D_SweptShared.cu:183-193: mgam*(E - (0.5*m*m/rho))
// (The products by 0.5 and 2 below are exact scalings: mlp2 forms them on the
// integer pipe in FP64, with the multiply's bits.)
template <typename T>
SW_HD T eu_pressure(const Params<T> &p, Q3<T> q) {
    return ml(p.mgam, sb(q.z, dv(ml(mlp2(q.y, T(0.5), -1), q.y), q.x)));
}
// pressureHalf, :202-212: mgam*(z - 0.5*y*y)
template <typename T>
SW_HD T eu_pressure_half(const Params<T> &p, Q3<T> q) {
    return ml(p.mgam, sb(q.z, ml(mlp2(q.y, T(0.5), -1), q.y)));
}
// limitor, :222-228: cur + 0.5*min(ratio,1)*(oth - cur)
template <typename T>
SW_HD Q3<T> eu_limit(Q3<T> cur, Q3<T> oth, T ratio) {
    return qadd(cur, qscale(mlp2(mn(ratio, T(1)), T(0.5), -1), qsub(oth, cur)));
}
// eulerFlux, :237-257
template <typename T>
SW_HD Q3<T> eu_flux(const Params<T> &p, Q3<T> L, Q3<T> R) {
    T uL = dv(L.y, L.x);
    T uR = dv(R.y, R.x);
    T pL = eu_pressure(p, L);
    T pR = eu_pressure(p, R);
    Q3<T> f;
    f.x = ad(L.y, R.y);
    f.y = ad(ad(ad(ml(L.y, uL), ml(R.y, uR)), pL), pR);
    f.z = ad(ad(ad(ml(L.z, uL), ml(R.z, uR)), ml(uL, pL)), ml(uR, pR));
    return f;
}
// eulerSpectral, :266-292
template <typename T>
SW_HD Q3<T> eu_spectral(const Params<T> &p, Q3<T> L, Q3<T> R) {
    T rl = sq(L.x), rr = sq(R.x);
    Q3<T> h;
    h.x = ml(rl, rr);
    T hd = dv(T(1), ml(h.x, ad(rl, rr)));
    h.y = ml(ad(ml(rl, R.y), ml(rr, L.y)), hd);
    h.z = ml(ad(ml(rl, R.z), ml(rr, L.z)), hd);
    T pH = eu_pressure_half(p, h);
    return qscale(ad(sq(ml(pH, p.gam)), ab(h.y)), qsub(L, R));
}
// The flux sum shared by eulerStutterStep / eulerFinalStep (:308-341, :354-380),
// on five cells s[0..4] around s[2].
template <typename T>
SW_HD Q3<T> eu_flux_sum(const Params<T> &p, const Q3<T> (&s)[5], bool fl, bool fr) {
    const T Z = T(0);
    // Written as in the reference: P1-P0 = 2*s1.x*s0.x*(s1.z - s0.z) + (s0.y*s0.y*s1.x - s1.y*s1.y*s0.x)
    T pLL = fl ? Z : ad(ml(ml(mlp2(s[1].x, T(2), 1), s[0].x), sb(s[1].z, s[0].z)),
                        sb(ml(ml(s[0].y, s[0].y), s[1].x), ml(ml(s[1].y, s[1].y), s[0].x)));
    T pL = ad(ml(ml(mlp2(s[2].x, T(2), 1), s[1].x), sb(s[2].z, s[1].z)),
              sb(ml(ml(s[1].y, s[1].y), s[2].x), ml(ml(s[2].y, s[2].y), s[1].x)));
    T pR = ad(ml(ml(mlp2(s[2].x, T(2), 1), s[3].x), sb(s[3].z, s[2].z)),
              sb(ml(ml(s[2].y, s[2].y), s[3].x), ml(ml(s[3].y, s[3].y), s[2].x)));
    T pRR = fr ? Z : ad(ml(ml(mlp2(s[3].x, T(2), 1), s[4].x), sb(s[4].z, s[3].z)),
                        sb(ml(ml(s[3].y, s[3].y), s[4].x), ml(ml(s[4].y, s[4].y), s[3].x)));

    const bool skipL = (pLL == Z) || (pL == Z) || ((pLL < Z) != (pL < Z));
    const bool skipM = (pL == Z) || (pR == Z) || ((pL < Z) != (pR < Z));
    const bool skipR = (pRR == Z) || (pR == Z) || ((pRR < Z) != (pR < Z));

    Q3<T> tL = skipL ? s[1] : eu_limit(s[1], s[2], dv(ml(s[0].x, pL), ml(s[2].x, pLL)));
    Q3<T> tR = skipM ? s[2] : eu_limit(s[2], s[1], dv(ml(s[3].x, pL), ml(s[1].x, pR)));
    Q3<T> flux = eu_flux(p, tL, tR);
    flux = qadd(flux, eu_spectral(p, tL, tR));

    tL = skipM ? s[2] : eu_limit(s[2], s[3], dv(ml(s[1].x, pR), ml(s[3].x, pL)));
    tR = skipR ? s[3] : eu_limit(s[3], s[2], dv(ml(s[4].x, pR), ml(s[2].x, pRR)));
    flux = qsub(flux, eu_flux(p, tL, tR));
    flux = qsub(flux, eu_spectral(p, tL, tR));
    return flux;
}
// Interface form of eu_flux_sum.  Each interface's terms are the same in the
// two cells that share it, so one lane computes them once:
//  * eu_pdiff(a, b): the pressure-difference numerator between neighbours a
//    (left) and b (right).  The reference spells the product 2*b.x*a.x for a
//    cell's left interfaces and 2*a.x*b.x for its right ones; the doubling is
//    exact, so both round to the same value;
//  * eu_iface: the limited states of the interface between a and b (outer
//    neighbours am, bp; Da = D(am, a), Db = D(a, b), Dbp = D(b, bp)) and its
//    flux F and dissipation S, as eulerStutterStep / eulerFinalStep form them
//    (:336-341 for a cell's left interface, :375-380 for its right one);
//  * eu_combine: the cell's sum ((F_left + S_left) - F_right) - S_right, in
//    the reference's order.
template <typename T>
SW_HD T eu_pdiff(Q3<T> a, Q3<T> b) {
    return ad(ml(ml(mlp2(b.x, T(2), 1), a.x), sb(b.z, a.z)), sb(ml(ml(a.y, a.y), b.x), ml(ml(b.y, b.y), a.x)));
}
template <typename T>
SW_HD void eu_iface(const Params<T> &p, Q3<T> am, Q3<T> a, Q3<T> b, Q3<T> bp, T Da, T Db, T Dbp,
                                         Q3<T> &F, Q3<T> &S) {
    const T Z = T(0);
    const bool skipA = (Da == Z) || (Db == Z) || ((Da < Z) != (Db < Z));
    const bool skipB = (Db == Z) || (Dbp == Z) || ((Db < Z) != (Dbp < Z));
    const Q3<T> tL = skipA ? a : eu_limit(a, b, dv(ml(am.x, Db), ml(b.x, Da)));
    const Q3<T> tR = skipB ? b : eu_limit(b, a, dv(ml(bp.x, Db), ml(a.x, Dbp)));
    F = eu_flux(p, tL, tR);
    S = eu_spectral(p, tL, tR);
}
template <typename T>
SW_HD Q3<T> eu_combine(Q3<T> Fl, Q3<T> Sl, Q3<T> Fr, Q3<T> Sr) {
    return qsub(qsub(qadd(Fl, Sl), Fr), Sr);
}

// eulerStutterStep result, :345: s2 + (0.25*dt_dx)*flux
template <typename T>
SW_HD Q3<T> eu_predict(const Params<T> &p, const Q3<T> (&s)[5], bool fl, bool fr) {
    Q3<T> f = eu_flux_sum(p, s, fl, fr);
    return qadd(s[2], qscale(ml(T(0.25), p.dtdx), f));
}
// eulerFinalStep result added to the cell, :384 and classicEuler :420
template <typename T>
SW_HD Q3<T> eu_correct(const Params<T> &p, Q3<T> u, const Q3<T> (&s)[5], bool fl, bool fr) {
    Q3<T> f = eu_flux_sum(p, s, fl, fr);
    return qadd(u, qscale(ml(T(0.5), p.dtdx), f));
}

SW_KERNELS_END
