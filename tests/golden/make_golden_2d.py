"""Generate the 2D golden vectors (tests/golden/c1_2d_128.npz) from the oracle.

The reference has no 2D mode (its multigrid assumes 3D octants,
src/mg/solver.h:73-181), so this fixture is made by the CPU restatement in
oracle/restated/ on a grid with nz == 1, where every operator is the
reference's own 3D row with the one-cell z extent folded into the diagonal
(src/mg/laplacian.h:62-73, src/ns/helmholtz.h:77-88). The 2D mode is pinned
to the 3D restatement by tests/test_oracle_2d.py (a z-invariant 3D run on
four planes equals the 2D run).

    python tests/golden/make_golden_2d.py

Workload: periodic unit square on a 128 x 128 MAC grid, rho = 1, mu = 0.01,
dt = 1e-4, 200 IB steps from rest; a closed membrane of 512 markers equally
spaced in angle on the ellipse centred at (0.5, 0.5) with semi-axes 0.25 and
0.20, linear springs of stiffness 1 between ring neighbours; projection and
Helmholtz solves to 1e-12.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle as po  # noqa: E402
from afmibins_gb300 import markers as mk  # noqa: E402

N, M, STEPS = 128, 512, 200
MU, RHO, DT, TOL, K = 0.01, 1.0, 1e-4, 1e-12, 1.0


def run(steps=STEPS):
    g = po.Grid(N, N, 1, N, channel=False)
    zero = np.zeros(g.ncell)
    X0, nstart, nidx = mk.ellipse(M, z=0.5 / N)
    s = po.NSSolver(g, MU, RHO, DT, TOL, zero, zero, zero)
    X = X0.copy()
    for _ in range(steps):
        X, st = s.ib_step(X, nstart, nidx, K)
        assert st == 0, st
    u, v, w, p = s.get()
    return dict(X0=X0, nstart=nstart, nidx=nidx, X=X, u=u, v=v, p=p, w_max=np.float64(np.abs(w).max()),
                steps=np.int64(steps), mu=np.float64(MU), rho=np.float64(RHO), dt=np.float64(DT),
                tol=np.float64(TOL), k=np.float64(K))


def main():
    t = time.time()
    d = run()
    assert d["w_max"] == 0.0
    path = os.path.join(HERE, "c1_2d_128.npz")
    np.savez_compressed(path, **d)
    print("wrote", os.path.relpath(path, ROOT), f"in {time.time() - t:.1f} s")


if __name__ == "__main__":
    main()
