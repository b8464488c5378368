"""Ensembles of independent periodic KS domains (the batched workload).

``make_ensemble`` draws the benchmark's ensemble: n domains, nx = 2^e with e
uniform on {lo..hi} (log-uniform lengths), dx = 0.5, and per domain the
initial condition u(x,0) = sum_{k=1..8} (N(0,1)/k) cos(2 pi k x / L + phi_k),
phi_k uniform on [0, 2 pi), L = nx dx, all from one seeded generator.
``split`` / ``concat`` convert between the concatenated state the C ABI takes
and per-domain arrays.
"""
from __future__ import annotations

import numpy as np

SEED = 20261203


def make_ensemble(n_domains: int = 4096, lo: int = 10, hi: int = 16, dx: float = 0.5, modes: int = 8,
                  seed: int = SEED, dtype=np.float64) -> tuple[np.ndarray, np.ndarray]:
    rng = np.random.default_rng(seed)
    nx = (1 << rng.integers(lo, hi + 1, size=n_domains)).astype(np.int64)
    k = np.arange(1, modes + 1, dtype=np.float64)
    amps = rng.standard_normal((n_domains, modes)) / k
    phases = rng.uniform(0.0, 2.0 * np.pi, size=(n_domains, modes))
    # cos(2 pi k x/L + phi) = cos(2 pi k x/L) cos(phi) - sin(2 pi k x/L) sin(phi): one matrix
    # product per distinct length instead of 8 cosines per cell
    a = amps * np.cos(phases)
    b = amps * np.sin(phases)
    starts = np.concatenate([[0], np.cumsum(nx)[:-1]])
    out = np.empty(int(nx.sum()), dtype=dtype)
    for n in np.unique(nx):
        idx = np.nonzero(nx == n)[0]
        theta = 2.0 * np.pi * np.outer(np.arange(int(n), dtype=np.float64) / float(n), k)  # (n, modes), 2 pi k x / L
        block = np.cos(theta) @ a[idx].T - np.sin(theta) @ b[idx].T                         # (n, domains)
        for j, d in enumerate(idx):
            out[starts[d]:starts[d] + int(n)] = block[:, j]
    return nx, out


def split(state: np.ndarray, nx, comps: int = 1) -> list[np.ndarray]:
    parts, at = [], 0
    for n in nx:
        parts.append(state[at:at + comps * int(n)])
        at += comps * int(n)
    return parts


def concat(parts) -> np.ndarray:
    return np.concatenate([np.asarray(p) for p in parts])
