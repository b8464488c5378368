"""Time bookkeeping of the reference's wrappers -- TEST INFRASTRUCTURE ONLY.

A direct Python restatement of the host loops that decide how far each
reference program steps and when it writes a snapshot:

* Heat classicWrapper, SweptSource/Heat1D_SweptShared.cu:483-510 (two steps per
  pass; one extra t_fullstep after each snapshot without stepping);
* KS classicWrapper, SweptSource/KS1D_SweptShared.cu:609-631 (``t_eq <= t_end``);
* Euler classicWrapper, SweptSource/Euler1D_SweptShared.cu:855-888 (``<``);
* sweptWrapper of all three (Heat :541-682, KS :676-851, Euler :924-1100):
  up-triangle + split diamond, then pairs of diamonds; a snapshot is
  down-triangle, up-triangle, split diamond and one more t_fullstep.

Returns (t_final, time steps advanced, [(t_snapshot, steps so far)]).
"""
from __future__ import annotations

import numpy as np

HEAT, KS, EULER = 0, 1, 2


def reference_schedule(problem: int, prec: int, alg: int, tpb: int, dt: float, tf: float, freq: float):
    t_end = tf - 0.25 * dt                      # main(): tf = atof(argv[4]) - 0.25*dt
    wdt = float(np.float32(dt)) if (problem == KS and prec == 4) else dt  # KS passes dsc.dt (REAL)
    twrite = freq - 0.25 * wdt
    snaps = []
    if alg == 0:
        if problem == HEAT:
            tfs = wdt + wdt
            steps = 2
            t_eq = tfs
            while t_eq < t_end:
                steps += 2
                t_eq += tfs
                if t_eq > twrite:
                    snaps.append((t_eq, steps))
                    t_eq += tfs
                    twrite += freq
            return t_eq, steps, snaps
        t_eq, steps = 0.0, 0
        while (t_eq <= t_end) if problem == KS else (t_eq < t_end):
            steps += 1
            t_eq += wdt
            if t_eq > twrite:
                snaps.append((t_eq, steps))
                twrite += freq
        return t_eq, steps, snaps
    node = 32 if (problem == KS and alg == 2) else tpb       # KS register path: 32-cell nodes
    if problem == HEAT:
        tfs = wdt * float(node)
        per = node // 2                                       # steps per diamond
    else:
        tfs = 0.25 * wdt * float(node)
        per = node // 8
    t_eq = tfs
    steps = 2 * per                                           # up-triangle + split diamond + final down
    while t_eq < t_end:
        steps += 2 * per
        t_eq += tfs
        if t_eq > twrite:
            snaps.append((t_eq, steps))
            steps += 2 * per
            t_eq += tfs
            twrite += freq
    return t_eq, steps, snaps
