"""The hybrid variant (SW_FLAG_HOST_TILE, the reference's alg 2 for Heat and
Euler): in every phase-1 pass the tile that straddles the domain's ends is
computed on the host CPU while the GPU computes the others.  Its results must
equal the oracle bit for bit, as the reference's consistency.out shows its
hybrid equal to its classic and swept runs (RMSE 0)."""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HEAT, KS, EULER = 0, 1, 2
ROOT = Path(__file__).resolve().parent.parent


def _oracle_case(oracle, problem, prec, nx, dt, bc=None):
    c = oracle.reference_consts(problem, prec, nx, dt)
    if bc is not None:
        c.bc = bc
    return c


@pytest.mark.parametrize("problem,prec,alg,nx,tpb,dt,bc", [
    (HEAT, 8, 2, 1024, 64, 0.004, 0),        # the reference's hybrid: Heat, insulated ends, alg 2
    (HEAT, 4, 2, 512, 32, 0.004, 0),
    (HEAT, 8, 1, 1024, 128, 0.004, 2),       # periodic ends
    (EULER, 8, 2, 1024, 64, 0.1 / 1022, 0),  # Sod tube, Dirichlet cells at the split tile
    (EULER, 4, 2, 512, 128, 0.1 / 510, 0),
    (KS, 8, 1, 4096, 256, 0.005, 0),
    (KS, 4, 1, 4096, 128, 0.005, 0),         # FP32 KS 128-cell tiles run one warp per tile
    (KS, 8, 1, 1 << 18, 256, 0.005, 0),      # 1024 tiles: the launch of 1023 runs ungrouped
    (HEAT, 8, 2, 64, 64, 0.004, 0),          # a single tile: every phase-1 pass is the host's alone
])
def test_host_tile_equals_the_oracle(sw, solver, oracle, problem, prec, alg, nx, tpb, dt, bc):
    q = tpb // (2 * oracle.RADIUS[problem] * oracle.SUBSTEPS[problem])
    ic = oracle.reference_ic(problem, prec, nx)
    c = _oracle_case(oracle, problem, prec, nx, dt, oracle.BC_PERIODIC if bc == 2 else None)
    for nsteps in (q, 2 * q + 3, 5 * q):   # down-triangles of phase 0 and 1, a classic remainder
        cfg = sw.make_config(problem, prec, alg=alg, nx=nx, tpb=tpb, dt=dt, bc=bc, time_mode=sw.TIME_STEPS,
                             n_steps=nsteps, flags=sw.FLAG_HOST_TILE)
        got, res, _ = solver.run(cfg, ic)
        assert res.n_steps == nsteps
        np.testing.assert_array_equal(got, oracle.classic(c, ic, nsteps), err_msg="steps %d" % nsteps)


def test_host_tile_snapshots_equal_swept(sw, solver):
    """The reference's time bookkeeping with snapshots: the hybrid run's rows
    equal the swept run's."""
    out = {}
    for flags in (0, sw.FLAG_HOST_TILE):
        cfg = sw.make_config(HEAT, 8, alg=2, nx=2048, tpb=128, dt=0.004, tf=3.0, freq=1.0, flags=flags)
        fin, res, snaps = solver.run(cfg)
        out[flags] = (fin, [t for t, _ in snaps], [s for _, s in snaps])
    assert out[0][1] == out[sw.FLAG_HOST_TILE][1] and len(out[0][1]) >= 2
    np.testing.assert_array_equal(out[0][0], out[sw.FLAG_HOST_TILE][0])
    for a, b in zip(out[0][2], out[sw.FLAG_HOST_TILE][2]):
        np.testing.assert_array_equal(a, b)


def test_cli_alg2_host_tile_rows_equal_alg1(sw, tmp_path):
    """bin/HeatDoubleOut with alg 2 and SWEPT1D_HOST_TILE=1 (the reference's
    hybrid invocation) writes the same .dat rows as alg 1."""
    exe = ROOT / "bin" / "HeatDoubleOut"
    rows = {}
    for alg, env in ((1, {}), (2, {"SWEPT1D_HOST_TILE": "1"})):
        dat = tmp_path / ("h%d.dat" % alg)
        r = subprocess.run([str(exe), "1024", "64", "0.004", "2", "0.5", str(alg), str(dat)],
                           env=dict(os.environ, **env), capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
        rows[alg] = dat.read_text()
    assert rows[1] == rows[2]
