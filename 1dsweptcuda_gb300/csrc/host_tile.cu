// The host tile of the hybrid variant (SW_FLAG_HOST_TILE): the reference's
// alg 2 for Heat and Euler computes the split diamond -- the tile that
// straddles the domain's ends -- on the CPU while the GPU computes every other
// tile of the pass (CPU_diamond, Heat1D_SweptShared.cu:410-468, and its use in
// sweptWrapper :550-644; Euler1D_SweptShared.cu:761-835, :935-1050).  Here the
// GPU launch of a phase-1 pass simply leaves out its last tile (the one whose
// cells wrap from nx - 1 to 0) and host_tile computes it from that tile's two
// half-tile slots: the same import, levels, boundary cells and export as
// swept_tile in engine.cuh, with the stencils of stencils.cuh built for the
// host (each operation the IEEE operation itself; this file is compiled with
// -ffp-contract=off, so nothing is fused).  The results are those of the GPU
// tile bit for bit.
#include <cstdint>
#include <cstring>
#include <vector>

#include "engine.cuh"

namespace sw {
namespace {

template <int P, typename T>
struct HostRow {  // one tile row with R margin cells: value of cell x at v[R + x]
    using C = typename std::conditional<P == SW_EULER, Q3<T>, T>::type;
    std::vector<C> v;
};

template <typename T>
inline Q3<T> from_dev(const V4<T> &c) { return q3(c.x, c.y, c.z); }
template <typename T>
inline V4<T> to_dev(const Q3<T> &c) { return V4<T>{c.x, c.y, c.z, T(0)}; }

// The wrapping phase-1 tile of a domain of p.nx cells, tile width W: its cells
// x in [0, W/2) are the domain's last half-tile, x in [W/2, W) its first.
// mode MODE_DIAMOND: slots sl (half-tile nx/(W/2) - 1) and sr (half-tile 0) in,
// the same slots out.  MODE_DOWN: the slots in, the state's first half-tile
// (state_first) and last half-tile (state_last) out.
template <int P, typename T>
void tile_on_host(const Params<T> &p, int mode, typename Scheme<P, T>::G *sl, typename Scheme<P, T>::G *sr,
                  typename Scheme<P, T>::G *state_first, typename Scheme<P, T>::G *state_last, int W) {
    using G = typename Scheme<P, T>::G;
    constexpr int R = Scheme<P, T>::R;
    const int h = W / 2, H = W / (2 * R);
    const int first = h, last = h - 1;  // tile coordinates of global cells 0 and nx - 1
    HostRow<P, T> row[2];
    row[0].v.assign(W + 2 * R, {});
    row[1].v.assign(W + 2 * R, {});
    auto at = [&](int r, int x) -> typename HostRow<P, T>::C & { return row[r].v[R + x]; };
    auto get = [&](const G &g) {
        if constexpr (P == SW_EULER) return from_dev(g);
        else return g;
    };
    // import, as tile_import_at
    for (int i = 0; i < h; ++i) {
        at(0, i) = get(sl[i]);
        at(1, i - R) = get(sl[h + i]);
        at(0, h + i) = get(sr[i]);
        at(1, h + R + i) = get(sr[h + i]);
    }
    if constexpr (P == SW_EULER) {  // Dirichlet cells hold the boundary states in both rows (tile_fix_bc)
        const Q3<T> left = q3(p.bd[0], p.bd[1], p.bd[2]), right = q3(p.bd[3], p.bd[4], p.bd[5]);
        at(0, first) = at(1, first) = left;
        at(0, last) = at(1, last) = right;
    }
    // one sub-step of parity par on cells [lo, hi): read row par ^ 1, write row par
    auto level = [&](int par, int lo, int hi) {
        for (int b = lo; b < hi; ++b) {
            if constexpr (P == SW_HEAT) {
                int l = b - 1, r = b + 1;
                if (p.bc != SW_BC_PERIODIC) {  // insulated ends, Heat1D_SweptShared.cu:140-142,352-353
                    if (b == first) l = b + 1;
                    if (b == last) r = b - 1;
                }
                at(par, b) = heat_step(p, at(par ^ 1, l), at(par ^ 1, b), at(par ^ 1, r));
            } else if constexpr (P == SW_KS) {
                const int s = par ^ 1;
                if (par)
                    at(1, b) = ks_predict(p, at(s, b - 2), at(s, b - 1), at(s, b), at(s, b + 1), at(s, b + 2));
                else
                    at(0, b) = ks_correct(p, at(0, b), at(s, b - 2), at(s, b - 1), at(s, b), at(s, b + 1),
                                          at(s, b + 2));
            } else {
                if (b == first || b == last) continue;
                const Q3<T> st[5] = {at(par ^ 1, b - 2), at(par ^ 1, b - 1), at(par ^ 1, b), at(par ^ 1, b + 1),
                                     at(par ^ 1, b + 2)};
                const bool fl = (b - 1 == first), fr = (b + 1 == last);  // the reference's edge flags
                at(par, b) = par ? eu_predict(p, st, fl, fr) : eu_correct(p, at(0, b), st, fl, fr);
            }
        }
    };
    for (int j = 1; j <= H; ++j) level(j & 1, h - j * R, h + j * R);
    auto put = [&](const typename HostRow<P, T>::C &c) {
        if constexpr (P == SW_EULER) return to_dev(c);
        else return c;
    };
    if (mode == MODE_DOWN) {
        for (int x = 0; x < h; ++x) {
            state_last[x] = put(at(0, x));
            state_first[x] = put(at(0, h + x));
        }
        return;
    }
    for (int u = 1; u < H; ++u) level(u & 1, u * R, W - u * R);
    for (int i = 0; i < h; ++i) {  // export, as tile_export_at
        sl[i] = put(at(0, i));
        sl[h + i] = put(at(1, R + i));
        sr[i] = put(at(0, h + i));
        sr[h + i] = put(at(1, h - R + i));
    }
}

}  // namespace

// Entry from the run loop (api.cu): params is a Params<float or double>.
int host_tile_run(int problem, int prec, const void *params, int mode, void *sl, void *sr, void *state_first,
                  void *state_last, int W) {
    if (prec == 4) {
        const Params<float> &p = *static_cast<const Params<float> *>(params);
        switch (problem) {
        case SW_HEAT:
            tile_on_host<SW_HEAT, float>(p, mode, (float *)sl, (float *)sr, (float *)state_first, (float *)state_last, W);
            return 0;
        case SW_KS:
            tile_on_host<SW_KS, float>(p, mode, (float *)sl, (float *)sr, (float *)state_first, (float *)state_last, W);
            return 0;
        default:
            tile_on_host<SW_EULER, float>(p, mode, (V4<float> *)sl, (V4<float> *)sr, (V4<float> *)state_first,
                                          (V4<float> *)state_last, W);
            return 0;
        }
    }
    const Params<double> &p = *static_cast<const Params<double> *>(params);
    switch (problem) {
    case SW_HEAT:
        tile_on_host<SW_HEAT, double>(p, mode, (double *)sl, (double *)sr, (double *)state_first, (double *)state_last, W);
        return 0;
    case SW_KS:
        tile_on_host<SW_KS, double>(p, mode, (double *)sl, (double *)sr, (double *)state_first, (double *)state_last, W);
        return 0;
    default:
        tile_on_host<SW_EULER, double>(p, mode, (V4<double> *)sl, (V4<double> *)sr, (V4<double> *)state_first,
                                       (V4<double> *)state_last, W);
        return 0;
    }
}

}  // namespace sw
