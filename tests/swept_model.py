"""A NumPy model of one swept pass (test infrastructure): the kernels' tile
and half-tile slot scheme (csrc/engine.cuh swept_tile: import / export of the
slots, the down part's growing and the up part's shrinking levels, the wrap of
the last phase-1 tile) over a periodic KS or Heat domain, with the stencils
in the reference's operation order (KS1D_SweptShared.cu:134-171,
Heat1D_SweptShared.cu:121-130), each operation rounded in the state's own
precision.  It stands in for sw_swept_pass where no GPU is present, so that
the split-domain exchange (1dsweptcuda_gb300/split.py) runs on CPU ranks; its
results equal the oracle's classic scheme bit for bit."""
from __future__ import annotations

import numpy as np


def _ks_rhs(c, ll, l, m, r, rr):
    R = ll.dtype.type
    conv = r * r - l * l
    sec = (l + r) - R(2) * m
    fourth = (((ll - R(4) * l) + R(6) * m) - R(4) * r) + rr
    return (conv * R(c.dx_times4) + sec * R(c.dx2)) + fourth * R(c.dx4)


def _level(problem, c, rows, par, lo, hi, off):
    """Sub-step of parity `par` on tile cells [lo, hi) (row index = cell + off)."""
    x = np.arange(lo, hi) + off
    src, dst = rows[par ^ 1], rows[par]
    R = rows.dtype.type
    if problem == 0:
        dst[x] = R(c.fourier) * (src[x - 1] + src[x + 1]) + R(c.fourier_two) * src[x]
    elif par:  # predictor: u - dt/2 * rhs(u)
        dst[x] = src[x] - R(c.dt_half) * _ks_rhs(c, src[x - 2], src[x - 1], src[x], src[x + 1], src[x + 2])
    else:      # corrector: u + (-dt) * rhs(u*)
        dst[x] = dst[x] + (-R(c.dt)) * _ks_rhs(c, src[x - 2], src[x - 1], src[x], src[x + 1], src[x + 2])


def swept_pass(problem: int, c, mode: int, phase: int, state: np.ndarray, slots: np.ndarray, W: int) -> None:
    """One pass over every tile of the periodic domain `state` (nx cells),
    slots: 2 nx cells, half-tile h's slot at [h W, (h + 1) W)."""
    Rr = 1 if problem == 0 else 2
    nx, h = state.size, W // 2
    nhalf, H = nx // h, W // (2 * Rr)
    for t in range(nx // W):
        base = t * W + phase * h
        hl = (2 * t + phase) % nhalf
        hr = 0 if hl + 1 == nhalf else hl + 1
        sl, sr = slots[hl * W:(hl + 1) * W], slots[hr * W:(hr + 1) * W]
        rows = np.zeros((2, W + 2 * Rr), dtype=state.dtype)
        o = Rr  # row index of tile cell 0
        if mode == 0:
            rows[0, o:o + W] = state[base:base + W]
        else:
            rows[0, o:o + h] = sl[:h]
            rows[1, o - Rr:o - Rr + h] = sl[h:]
            rows[0, o + h:o + W] = sr[:h]
            rows[1, o + h + Rr:o + W + Rr] = sr[h:]
            for j in range(1, H + 1):
                _level(problem, c, rows, j & 1, h - j * Rr, h + j * Rr, o)
        if mode == 2:
            state[(base + np.arange(W)) % nx] = rows[0, o:o + W]
            continue
        for u in range(1, H):
            _level(problem, c, rows, u & 1, u * Rr, W - u * Rr, o)
        sl[:h] = rows[0, o:o + h]
        sl[h:] = rows[1, o + Rr:o + Rr + h]
        sr[:h] = rows[0, o + h:o + W]
        sr[h:] = rows[1, o + h - Rr:o + W - Rr]
