/*
 * Precision-generic body of the oracle (TEST INFRASTRUCTURE ONLY).
 * Included twice by oracle.c, with REAL = double / float and SFX = f64 / f32.
 * Every expression keeps the reference's operation order; the file is
 * compiled with -ffp-contract=off so no multiply-add is fused.
 */
#define CAT2(a, b) a##_##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, SFX)
#define V3 FN(or_v3)

typedef struct { REAL x, y, z; } V3;

/* ------------------------------------------------------------------ Heat */
/* execFunc, Heat1D_SweptShared.cu:121-130:
 *   fourier*(T[l] + T[r]) + fourierTwo*T[c] */
static inline REAL FN(heat_exec)(REAL fo, REAL fo2, REAL l, REAL c, REAL r)
{
    return fo * (l + r) + fo2 * c;
}

/* ------------------------------------------------------------------- KS */
/* convect / secondDer / fourthDer: multiply-by-reciprocal build,
 * KS1D_SweptShared.cu:136-155, or the DIVISE build, :111-132 (k->divide) */
static inline REAL FN(ks_sum)(const or_consts *k, REAL ll, REAL l, REAL c, REAL r, REAL rr)
{
    const REAL c4 = (REAL)k->dx_times4, d2 = (REAL)k->dx2, d4 = (REAL)k->dx4;
    REAL conv, sec, four;
    if (k->divide) {
        conv = (r * r - l * l) / c4;
        sec = (l + r - (REAL)2 * c) / d2;
        four = (ll - (REAL)4 * l + (REAL)6 * c - (REAL)4 * r + rr) / d4;
    } else {
        conv = (r * r - l * l) * c4;
        sec = (l + r - (REAL)2 * c) * d2;
        four = (ll - (REAL)4 * l + (REAL)6 * c - (REAL)4 * r + rr) * d4;
    }
    return conv + sec + four;
}
/* stutterStep, KS1D_SweptShared.cu:159-164 */
static inline REAL FN(ks_stutter)(const or_consts *k, const REAL *u, int64_t i2, int64_t i1, int64_t i0,
                                  int64_t j1, int64_t j2)
{
    return u[i0] - (REAL)k->dt_half * FN(ks_sum)(k, u[i2], u[i1], u[i0], u[j1], u[j2]);
}
/* finalStep, KS1D_SweptShared.cu:166-171 (returned increment; caller adds) */
static inline REAL FN(ks_final)(const or_consts *k, const REAL *u, int64_t i2, int64_t i1, int64_t i0,
                                int64_t j1, int64_t j2)
{
    return (-(REAL)k->dt * FN(ks_sum)(k, u[i2], u[i1], u[i0], u[j1], u[j2]));
}

/* ---------------------------------------------------------------- Euler */
static inline V3 FN(v3)(REAL x, REAL y, REAL z) { V3 v; v.x = x; v.y = y; v.z = z; return v; }
static inline V3 FN(v3_add)(V3 a, V3 b) { return FN(v3)(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 FN(v3_sub)(V3 a, V3 b) { return FN(v3)(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 FN(v3_scale)(REAL s, V3 a) { return FN(v3)(s * a.x, s * a.y, s * a.z); }

/* pressure, Euler1D_SweptShared.cu:183-193 */
static inline REAL FN(eu_pressure)(const or_consts *k, V3 q)
{
    return (REAL)k->mgam * (q.z - ((REAL)0.5 * q.y * q.y / q.x));
}
/* pressureHalf, Euler1D_SweptShared.cu:202-212 */
static inline REAL FN(eu_pressure_half)(const or_consts *k, V3 q)
{
    return (REAL)k->mgam * (q.z - (REAL)0.5 * q.y * q.y);
}
/* limitor, Euler1D_SweptShared.cu:222-228 */
static inline V3 FN(eu_limitor)(V3 cur, V3 oth, REAL ratio)
{
#if OR_IS_FLOAT
    REAL m = fminf(ratio, (REAL)1);
#else
    REAL m = fmin(ratio, (REAL)1);
#endif
    return FN(v3_add)(cur, FN(v3_scale)((REAL)0.5 * m, FN(v3_sub)(oth, cur)));
}
/* eulerFlux, Euler1D_SweptShared.cu:237-257 */
static inline V3 FN(eu_flux)(const or_consts *k, V3 L, V3 R)
{
    REAL uL = L.y / L.x;
    REAL uR = R.y / R.x;
    REAL pL = FN(eu_pressure)(k, L);
    REAL pR = FN(eu_pressure)(k, R);
    V3 f;
    f.x = (L.y + R.y);
    f.y = (L.y * uL + R.y * uR + pL + pR);
    f.z = (L.z * uL + R.z * uR + uL * pL + uR * pR);
    return f;
}
/* eulerSpectral, Euler1D_SweptShared.cu:266-292 */
static inline V3 FN(eu_spectral)(const or_consts *k, V3 L, V3 R)
{
#if OR_IS_FLOAT
    REAL rl = sqrtf(L.x), rr = sqrtf(R.x);
#else
    REAL rl = sqrt(L.x), rr = sqrt(R.x);
#endif
    V3 h;
    h.x = rl * rr;
    REAL hd = (REAL)1 / (h.x * (rl + rr));
    h.y = (rl * R.y + rr * L.y) * hd;
    h.z = (rl * R.z + rr * L.z) * hd;
    REAL pH = FN(eu_pressure_half)(k, h);
#if OR_IS_FLOAT
    REAL s = sqrtf(pH * (REAL)k->gam) + fabsf(h.y);
#else
    REAL s = sqrt(pH * (REAL)k->gam) + fabs(h.y);
#endif
    return FN(v3_scale)(s, FN(v3_sub)(L, R));
}
/* The shared body of eulerStutterStep / eulerFinalStep,
 * Euler1D_SweptShared.cu:308-341 and 354-380: the four pressure-difference
 * numerators, the limited states at both interfaces and the summed flux. */
static inline V3 FN(eu_flux_sum)(const or_consts *k, const V3 *s, int64_t tr, int flagL, int flagR)
{
    const REAL Z = (REAL)0, T2 = (REAL)2;
    REAL pLL = (flagL) ? Z : (T2 * s[tr - 1].x * s[tr - 2].x * (s[tr - 1].z - s[tr - 2].z) +
                              (s[tr - 2].y * s[tr - 2].y * s[tr - 1].x - s[tr - 1].y * s[tr - 1].y * s[tr - 2].x));
    REAL pL = (T2 * s[tr].x * s[tr - 1].x * (s[tr].z - s[tr - 1].z) +
               (s[tr - 1].y * s[tr - 1].y * s[tr].x - s[tr].y * s[tr].y * s[tr - 1].x));
    REAL pR = (T2 * s[tr].x * s[tr + 1].x * (s[tr + 1].z - s[tr].z) +
               (s[tr].y * s[tr].y * s[tr + 1].x - s[tr + 1].y * s[tr + 1].y * s[tr].x));
    REAL pRR = (flagR) ? Z : (T2 * s[tr + 1].x * s[tr + 2].x * (s[tr + 2].z - s[tr + 1].z) +
                              (s[tr + 1].y * s[tr + 1].y * s[tr + 2].x - s[tr + 2].y * s[tr + 2].y * s[tr + 1].x));

    V3 tL = (!pLL || !pL || ((pLL < 0) != (pL < 0)))
                ? s[tr - 1]
                : FN(eu_limitor)(s[tr - 1], s[tr], (s[tr - 2].x * pL / (s[tr].x * pLL)));
    V3 tR = (!pL || !pR || ((pL < 0) != (pR < 0)))
                ? s[tr]
                : FN(eu_limitor)(s[tr], s[tr - 1], (s[tr + 1].x * pL / (s[tr - 1].x * pR)));

    V3 flux = FN(eu_flux)(k, tL, tR);
    flux = FN(v3_add)(flux, FN(eu_spectral)(k, tL, tR));

    tL = (!pL || !pR || ((pL < 0) != (pR < 0)))
             ? s[tr]
             : FN(eu_limitor)(s[tr], s[tr + 1], (s[tr - 1].x * pR / (s[tr + 1].x * pL)));
    tR = (!pRR || !pR || ((pRR < 0) != (pR < 0)))
             ? s[tr + 1]
             : FN(eu_limitor)(s[tr + 1], s[tr], (s[tr + 2].x * pR / (s[tr].x * pRR)));

    flux = FN(v3_sub)(flux, FN(eu_flux)(k, tL, tR));
    flux = FN(v3_sub)(flux, FN(eu_spectral)(k, tL, tR));
    return flux;
}
/* eulerStutterStep return, Euler1D_SweptShared.cu:345 */
static inline V3 FN(eu_stutter)(const or_consts *k, const V3 *s, int64_t tr, int fl, int fr)
{
    V3 f = FN(eu_flux_sum)(k, s, tr, fl, fr);
    return FN(v3_add)(s[tr], FN(v3_scale)((REAL)0.25 * (REAL)k->dt_dx, f));
}
/* eulerFinalStep return, Euler1D_SweptShared.cu:384 (increment; caller adds) */
static inline V3 FN(eu_final)(const or_consts *k, const V3 *s, int64_t tr, int fl, int fr)
{
    V3 f = FN(eu_flux_sum)(k, s, tr, fl, fr);
    return FN(v3_scale)((REAL)0.5 * (REAL)k->dt_dx, f);
}

static inline V3 FN(eu_bd)(const or_consts *k, int side)
{
    return FN(v3)((REAL)k->bd[3 * side], (REAL)k->bd[3 * side + 1], (REAL)k->bd[3 * side + 2]);
}

double FN(or_euler_pressure)(const or_consts *c, const REAL *q3)
{
    return (double)FN(eu_pressure)(c, FN(v3)(q3[0], q3[1], q3[2]));
}

/* ------------------------------------------------------ classic stepping */
/* One classic sub-step over cells [lo, hi).  `sub` 0 = predictor / the Heat
 * step (dst = F(src)), 1 = corrector (dst += G(src)).
 * classicHeat Heat1D_SweptShared.cu:132-145 (mirror ends), classicKS
 * KS1D_SweptShared.cu:189-207 (periodic), classicEuler
 * Euler1D_SweptShared.cu:400-426 (cells 0 and nx-1 held at dbd). */
static void FN(classic_range)(const or_consts *k, const REAL *src, REAL *dst, int sub, int64_t lo, int64_t hi)
{
    const int64_t nx = k->nx;
    if (k->problem == OR_HEAT) {
        const REAL fo = (REAL)k->fourier, fo2 = (REAL)k->fourier_two;
        for (int64_t g = lo; g < hi; ++g) {
            int64_t l, r;
            if (k->bc == OR_BC_PERIODIC) {
                l = (g == 0) ? nx - 1 : g - 1;
                r = (g == nx - 1) ? 0 : g + 1;
            } else {
                l = (g == 0) ? (g + 1) : (g - 1);
                r = (g == nx - 1) ? (g - 1) : (g + 1);
            }
            dst[g] = FN(heat_exec)(fo, fo2, src[l], src[g], src[r]);
        }
    } else if (k->problem == OR_KS) {
        for (int64_t g = lo; g < hi; ++g) {
            int64_t i2 = (g - 2 + nx) % nx, i1 = (g - 1 + nx) % nx, j1 = (g + 1) % nx, j2 = (g + 2) % nx;
            if (sub == 0)
                dst[g] = FN(ks_stutter)(k, src, i2, i1, g, j1, j2);
            else
                dst[g] += FN(ks_final)(k, src, i2, i1, g, j1, j2);
        }
    } else {
        const V3 *s = (const V3 *)src;
        V3 *d = (V3 *)dst;
        for (int64_t g = lo; g < hi; ++g) {
            if (g == 0) { d[g] = FN(eu_bd)(k, 0); continue; }
            if (g == nx - 1) { d[g] = FN(eu_bd)(k, 1); continue; }
            int fl = (g == 1), fr = (g == nx - 2);
            if (sub == 0)
                d[g] = FN(eu_stutter)(k, s, g, fl, fr);
            else
                d[g] = FN(v3_add)(d[g], FN(eu_final)(k, s, g, fl, fr));
        }
    }
}

static int FN(check)(const or_consts *c)
{
    if (!c || c->nx < 8) return -1;
    if (c->problem < 0 || c->problem > 2) return -1;
    return 0;
}

static int FN(classic_impl)(const or_consts *c, REAL *u, int64_t nsteps, int nthreads, int use_omp)
{
    if (FN(check)(c)) return -1;
    const int64_t nx = c->nx;
    const int comps = (c->problem == OR_EULER) ? 3 : 1;
    REAL *w = (REAL *)malloc(sizeof(REAL) * (size_t)nx * comps);
    if (!w) return -2;
    memcpy(w, u, sizeof(REAL) * (size_t)nx * comps);
#ifdef _OPENMP
    if (use_omp && nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    if (c->problem == OR_HEAT) {
        REAL *a = u, *b = w;
        for (int64_t n = 0; n < nsteps; ++n) {
            if (use_omp) {
#pragma omp parallel for schedule(static)
                for (int64_t blk = 0; blk < (nx + 4095) / 4096; ++blk) {
                    int64_t lo = blk * 4096, hi = lo + 4096 < nx ? lo + 4096 : nx;
                    FN(classic_range)(c, a, b, 0, lo, hi);
                }
            } else {
                FN(classic_range)(c, a, b, 0, 0, nx);
            }
            REAL *t = a; a = b; b = t;
        }
        if (a != u) memcpy(u, a, sizeof(REAL) * (size_t)nx);
    } else {
        /* u holds the state, w the predictor (classicKS(in,out,false); classicKS(out,in,true)) */
        for (int64_t n = 0; n < nsteps; ++n) {
            for (int sub = 0; sub < 2; ++sub) {
                const REAL *src = sub ? w : u;
                REAL *dst = sub ? u : w;
                if (use_omp) {
#pragma omp parallel for schedule(static)
                    for (int64_t blk = 0; blk < (nx + 4095) / 4096; ++blk) {
                        int64_t lo = blk * 4096, hi = lo + 4096 < nx ? lo + 4096 : nx;
                        FN(classic_range)(c, src, dst, sub, lo, hi);
                    }
                } else {
                    FN(classic_range)(c, src, dst, sub, 0, nx);
                }
            }
        }
    }
    free(w);
    return 0;
}

int FN(or_classic)(const or_consts *c, REAL *u, int64_t nsteps) { return FN(classic_impl)(c, u, nsteps, 0, 0); }
int FN(or_classic_omp)(const or_consts *c, REAL *u, int64_t nsteps, int nthreads)
{
    return FN(classic_impl)(c, u, nsteps, nthreads, 1);
}

/* ------------------------------------------------------- swept (CPU model)
 * The decomposition of the swept rule (docs/Swept_1_D_Scheme_Description.pdf;
 * kernels upTriangle / wholeDiamond / splitDiamond / downTriangle in
 * Heat1D_SweptShared.cu:147-408, KS1D_SweptShared.cu:209-394,
 * Euler1D_SweptShared.cu:437-746) written over half-tile edge slots:
 *
 *  - a tile of W points keeps two rows; sub-step m reads row (m-1)&1 and
 *    writes row m&1 (Heat: the two time-parity rows; KS/Euler: row 0 = u,
 *    row 1 = predictor u*, the corrector adds into row 0);
 *  - the up part of a tile computes sub-steps u = 1..H-1 (H = W/(2R)) on
 *    [uR, W-uR); the down part of a tile shifted by W/2 computes j = 1..H on
 *    [W/2-jR, W/2+jR);
 *  - a tile exports, per side, row 0 on its half [0,W/2) or [W/2,W) and row 1
 *    on that half moved R cells inward: [R, W/2+R) or [W/2-R, W-R).  Each
 *    half-tile h owns one slot of W values (row 0 then row 1); a diamond
 *    reads the two slots of its halves and overwrites them with its own
 *    exports.
 * Every (cell, sub-step) value is computed exactly once, with the same
 * arithmetic as the classic loop, so the result is bit-identical to it.
 */
typedef struct {
    const or_consts *k;
    int W, R, H;
    int64_t nx;
    V3 *row[2]; /* each W + 2R long, index x + R */
} FN(tile_t);

static inline int64_t FN(wrap)(int64_t p, int64_t nx)
{
    p %= nx;
    return p < 0 ? p + nx : p;
}

/* Compute sub-step parity `par` (1 = predictor / odd Heat step) at tile cell x. */
static void FN(tile_point)(FN(tile_t) *t, int par, int x, int64_t base)
{
    const or_consts *k = t->k;
    const int64_t p = FN(wrap)(base + x, t->nx);
    V3 *src = t->row[par ^ 1] + t->R; /* row (m-1)&1 */
    V3 *dst = t->row[par] + t->R;     /* row m&1 */
    if (k->problem == OR_HEAT) {
        int l = x - 1, r = x + 1;
        if (k->bc != OR_BC_PERIODIC) {
            if (p == 0) l = x + 1;
            if (p == t->nx - 1) r = x - 1;
        }
        dst[x].x = FN(heat_exec)((REAL)k->fourier, (REAL)k->fourier_two, src[l].x, src[x].x, src[r].x);
    } else if (k->problem == OR_KS) {
        REAL buf[5];
        for (int i = 0; i < 5; ++i) buf[i] = src[x - 2 + i].x;
        if (par)
            dst[x].x = FN(ks_stutter)(k, buf, 0, 1, 2, 3, 4);
        else
            dst[x].x += FN(ks_final)(k, buf, 0, 1, 2, 3, 4);
    } else {
        if (p == 0 || p == t->nx - 1) return;
        int fl = (p == 1), fr = (p == t->nx - 2);
        if (par)
            dst[x] = FN(eu_stutter)(k, src, x, fl, fr);
        else
            dst[x] = FN(v3_add)(dst[x], FN(eu_final)(k, src, x, fl, fr));
    }
}

static void FN(tile_fix_bc)(FN(tile_t) *t, int64_t base)
{
    if (t->k->problem != OR_EULER) return;
    for (int x = -t->R; x < t->W + t->R; ++x) {
        int64_t p = FN(wrap)(base + x, t->nx);
        if (p == 0 || p == t->nx - 1) {
            V3 b = FN(eu_bd)(t->k, p == 0 ? 0 : 1);
            t->row[0][x + t->R] = b;
            t->row[1][x + t->R] = b;
        }
    }
}

static void FN(tile_down)(FN(tile_t) *t, int64_t base)
{
    for (int j = 1; j <= t->H; ++j)
        for (int x = t->W / 2 - j * t->R; x < t->W / 2 + j * t->R; ++x) FN(tile_point)(t, j & 1, x, base);
}
static void FN(tile_up)(FN(tile_t) *t, int64_t base)
{
    for (int u = 1; u < t->H; ++u)
        for (int x = u * t->R; x < t->W - u * t->R; ++x) FN(tile_point)(t, u & 1, x, base);
}

/* slot layout: [row0: W/2][row1: W/2] */
static void FN(tile_import)(FN(tile_t) *t, const V3 *slotL, const V3 *slotR)
{
    const int h = t->W / 2, R = t->R;
    for (int i = 0; i < h; ++i) {
        t->row[0][R + i] = slotL[i];
        t->row[1][R + (i - R)] = slotL[h + i];
        t->row[0][R + h + i] = slotR[i];
        t->row[1][R + h + R + i] = slotR[h + i];
    }
}
static void FN(tile_export)(const FN(tile_t) *t, V3 *slotL, V3 *slotR)
{
    const int h = t->W / 2, R = t->R;
    for (int i = 0; i < h; ++i) {
        slotL[i] = t->row[0][R + i];
        slotL[h + i] = t->row[1][R + R + i];
        slotR[i] = t->row[0][R + h + i];
        slotR[h + i] = t->row[1][R + h - R + i];
    }
}

int64_t FN(or_swept)(const or_consts *c, REAL *u, int tpb, int64_t n_diamonds)
{
    if (FN(check)(c)) return -1;
    const int64_t nx = c->nx;
    const int R = (c->problem == OR_HEAT) ? 1 : 2;
    const int S = (c->problem == OR_HEAT) ? 1 : 2;
    if (tpb < 4 * R || (tpb % (4 * R)) || nx % tpb || n_diamonds < 0) return -3;
    FN(tile_t) t;
    t.k = c; t.W = tpb; t.R = R; t.H = tpb / (2 * R); t.nx = nx;
    const int L = tpb + 2 * R;
    V3 *rows = (V3 *)calloc((size_t)2 * L, sizeof(V3));
    const int64_t nhalf = nx / (tpb / 2), ntile = nx / tpb;
    V3 *slots = (V3 *)calloc((size_t)nhalf * tpb, sizeof(V3));
    if (!rows || !slots) { free(rows); free(slots); return -2; }
    t.row[0] = rows; t.row[1] = rows + L;
    V3 *st = NULL;
    REAL *uu = u;
    if (c->problem == OR_EULER) st = (V3 *)u;

#define OR_GET(p) (st ? st[p] : FN(v3)(uu[p], 0, 0))
#define OR_PUT(p, v) do { if (st) st[p] = (v); else uu[p] = (v).x; } while (0)
    const REAL qnan = (REAL)NAN;
    /* up-triangle on aligned tiles */
    for (int64_t ti = 0; ti < ntile; ++ti) {
        int64_t base = ti * tpb;
        for (int x = 0; x < 2 * L; ++x) rows[x] = FN(v3)(qnan, qnan, qnan);
        for (int x = 0; x < tpb; ++x) t.row[0][R + x] = OR_GET(base + x);
        FN(tile_fix_bc)(&t, base);
        FN(tile_up)(&t, base);
        FN(tile_export)(&t, slots + (2 * ti) * tpb, slots + (2 * ti + 1) * tpb);
    }
    /* diamonds, alternating shifted (odd phase) and aligned (even phase) */
    int64_t phase = 0;
    for (int64_t d = 0; d <= n_diamonds; ++d) {
        phase ^= 1;
        const int last = (d == n_diamonds);
        for (int64_t ti = 0; ti < ntile; ++ti) {
            int64_t hl = (2 * ti + phase) % nhalf, hr = (2 * ti + 1 + phase) % nhalf;
            int64_t base = ti * tpb + phase * (tpb / 2);
            for (int x = 0; x < 2 * L; ++x) rows[x] = FN(v3)(qnan, qnan, qnan);
            FN(tile_import)(&t, slots + hl * tpb, slots + hr * tpb);
            FN(tile_fix_bc)(&t, base);
            FN(tile_down)(&t, base);
            if (last) {
                for (int x = 0; x < tpb; ++x) OR_PUT(FN(wrap)(base + x, nx), t.row[0][R + x]);
            } else {
                FN(tile_up)(&t, base);
                FN(tile_export)(&t, slots + hl * tpb, slots + hr * tpb);
            }
        }
    }
#undef OR_GET
#undef OR_PUT
    free(rows);
    free(slots);
    return (n_diamonds + 1) * (int64_t)(tpb / (2 * R)) / S;
}

#undef V3
#undef FN
#undef CAT
#undef CAT2
