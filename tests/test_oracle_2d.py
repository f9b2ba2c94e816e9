"""The oracle's 2D mode (nz == 1) against its 3D mode, which the reference
pins: 2D operators are the 3D rows with the one-cell z extent folded into the
diagonal (src/mg/laplacian.h:62-73), so a z-invariant 3D problem must give
the 2D answer. The reference itself has no 2D mode."""
import numpy as np
import pytest

from oracle import pyoracle as po
from afmibins_gb300 import markers as mk


def test_laplacian_2d_is_five_point():
    n = 32
    g = po.Grid(n, n, 1, n)
    x = np.random.default_rng(1).standard_normal(g.ncell)
    X = x.reshape(n, n)
    ref = n * n * (np.roll(X, 1, 0) + np.roll(X, -1, 0) + np.roll(X, 1, 1) + np.roll(X, -1, 1) - 4 * X)
    np.testing.assert_allclose(po.lap_apply(g, x).reshape(n, n), ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def test_transfers_2d_match_z_invariant_3d():
    n = 16
    g2, g3 = po.Grid(n, n, 1, n), po.Grid(n, n, 4, n)
    rng = np.random.default_rng(2)
    x = rng.standard_normal(n * n)
    c2 = po.restrict(g2, x)
    c3 = po.restrict(g3, np.tile(x, 4)).reshape(2, -1)
    np.testing.assert_allclose(c3[0], c2, rtol=1e-14, atol=1e-14)
    np.testing.assert_allclose(c3[1], c2, rtol=1e-14, atol=1e-14)
    y = rng.standard_normal(n * n // 4)
    f2 = po.prolong(g2, y)
    f3 = po.prolong(g3, np.tile(y, 2)).reshape(4, -1)
    for k in range(4):
        np.testing.assert_allclose(f3[k], f2, rtol=1e-14, atol=1e-14)


def test_mg_2d_converges():
    n = 64
    g = po.Grid(n, n, 1, n)
    b = np.random.default_rng(3).standard_normal(g.ncell)
    x, cycles, st = po.mg_solve(g, b.copy(), 1e-11)
    assert st == 0 and 0 < cycles < 40
    r = (b - b.mean()) - po.lap_apply(g, x)
    assert np.sqrt(np.mean(r ** 2)) <= 1e-11


def test_ib_steps_2d_match_z_invariant_3d():
    """Five IB steps of a ring in 2D against the same ring replicated on the
    four planes of a z-periodic 3D grid (the replicas' z kernels sum to one
    on every plane). The 2D kernel is phi^2 against phi^3 in 3D, so the 3D
    springs carry k / n."""
    n, m, k, steps = 32, 96, 1.0, 5
    mu, rho, dt, tol = 0.01, 1.0, 1e-4, 1e-12
    X, ns, ni = mk.ellipse(m, axes=(0.25, 0.2), z=0.3 / n)
    g2 = po.Grid(n, n, 1, n)
    z2 = np.zeros(g2.ncell)
    s2 = po.NSSolver(g2, mu, rho, dt, tol, z2, z2, z2)
    X2 = X.copy()
    for _ in range(steps):
        X2, st = s2.ib_step(X2, ns, ni, k)
        assert st == 0
    u2, v2, w2, p2 = s2.get()
    assert np.abs(w2).max() == 0.0

    g3 = po.Grid(n, n, 4, n)
    z3 = np.zeros(g3.ncell)
    X3 = np.concatenate([X + [0, 0, j / n] for j in range(4)])
    ns3 = np.concatenate([ns[:-1] + j * len(ni) for j in range(4)] + [[4 * len(ni)]]).astype(np.int32)
    ni3 = np.concatenate([ni + j * m for j in range(4)]).astype(np.int32)
    s3 = po.NSSolver(g3, mu, rho, dt, tol, z3, z3, z3)
    for _ in range(steps):
        X3, st = s3.ib_step(X3, ns3, ni3, k / n)
        assert st == 0
    u3, v3, w3, p3 = s3.get()
    # the two runs take different multigrid iterates (the 3D smoother sweeps
    # plane by plane), so they agree to the solver tolerance, not to round-off:
    # velocity within 10 tol, marker motion within 10 tol dt per step
    assert np.abs(u2).max() > 1e-6
    for j in range(4):
        assert np.abs(u3.reshape(4, -1)[j] - u2).max() <= 10 * tol
        assert np.abs(v3.reshape(4, -1)[j] - v2).max() <= 10 * tol
    assert np.abs(w3).max() <= 10 * tol
    disp2 = X2 - X
    disp3 = X3[:m] - X
    assert np.abs(disp2).max() > 1e-9
    assert np.abs(disp3[:, :2] - disp2[:, :2]).max() <= 10 * tol * dt * steps


def test_golden_c1_fixture_is_2d(golden):
    d = golden("c1_2d_128")
    assert d["u"].size == 128 * 128 and float(d["w_max"]) == 0.0
    assert np.abs(d["X"] - d["X0"]).max() > 0
