"""Host-side pieces of the closure's fallback: the conservative spectral
prolongation (torch on the CPU, no GPU needed)."""
import importlib
import math

import pytest

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def cl():
    return importlib.import_module("1dsweptcuda_gb300.closure")


def _cell_averages(a, ph, ks, x0, w, L):
    kap = 2 * math.pi * ks / L
    return ((a[None] * (torch.sin(kap[None] * (x0[:, None] + w) + ph) - torch.sin(kap[None] * x0[:, None] + ph)))
            / (kap[None] * w)).sum(1)


def test_prolong_reproduces_band_limited_fields(cl):
    """Coarse cell averages of a band-limited field -> the fine cell averages
    of the same field, to rounding."""
    n, f, H = 1024, 4, 2.0
    g = torch.Generator().manual_seed(0)
    ks = torch.arange(1, 300, dtype=torch.float64)
    a = torch.randn(len(ks), generator=g, dtype=torch.float64) / ks
    ph = torch.rand(len(ks), generator=g, dtype=torch.float64) * 2 * math.pi
    L = n * H
    c = _cell_averages(a, ph, ks, torch.arange(n, dtype=torch.float64) * H, H, L)[None]
    want = _cell_averages(a, ph, ks, torch.arange(n * f, dtype=torch.float64) * (H / f), H / f, L)[None]
    got = cl.prolong(c)
    assert float((got - want).abs().max()) < 1e-10


def test_prolong_is_conservative(cl):
    """Averaging each 4 fine cells gives the coarse state back, including its
    Nyquist mode; a constant stays exactly constant."""
    g = torch.Generator().manual_seed(1)
    r = torch.randn(3, 1024, generator=g, dtype=torch.float64)
    r[1] += 0.7 * (1 - 2 * (torch.arange(1024) % 2))
    back = cl.prolong(r).reshape(3, 1024, 4).mean(-1)
    assert float((back - r).abs().max()) < 1e-13
    one = torch.full((2, 1024), 1.5)
    assert torch.equal(cl.prolong(one), torch.full((2, 4096), 1.5, dtype=torch.float64))
