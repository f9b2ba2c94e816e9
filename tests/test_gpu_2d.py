"""2D grids (nz == 1, periodic) on the GPU against the oracle's 2D mode: the
operators, a converged multigrid solve, and the 128 x 128 membrane workload
(512 markers on an ellipse, 200 IB steps) against its golden fixture."""
import numpy as np
import pytest

from afmibins_gb300 import capi
from afmibins_gb300 import markers as mk
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

OPS_TOL = 1e-13


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def demean(p):
    return p - p.mean()


def test_2d_operators():
    n = 32
    g = po.Grid(n, n, 1, n)
    rng = np.random.default_rng(11)
    u, v, w, p = (rng.standard_normal(g.ncell) for _ in range(4))
    w0 = np.zeros(g.ncell)
    with capi.Solver(n, n, 1) as sv:
        assert rel(sv.lap_apply(p), po.lap_apply(g, p)) < OPS_TOL
        for comp in range(3):
            assert rel(sv.helm_apply(comp, 0.3, p), po.helm_apply(g, comp, 0.3, p)) < OPS_TOL
        assert rel(sv.restrict(p), po.restrict(g, p)) < OPS_TOL
        c = rng.standard_normal(g.ncell // 4)
        assert rel(sv.prolong(c), po.prolong(g, c)) < OPS_TOL
        assert rel(sv.div(u, v, w0), po.div(g, u, v, w0)) < OPS_TOL
        for a, b in zip(sv.grad(p), po.grad(g, p)):
            assert rel(a, b) < OPS_TOL
        for a, b in zip(sv.advection(u, v, w0), po.advection(g, u, v, w0)):
            assert np.max(np.abs(a - b)) <= OPS_TOL * max(np.max(np.abs(b)), 1.0)
        X, _, _ = mk.ellipse(96, z=0.3 / n)
        F = rng.standard_normal((3, 96))
        F[2] = 0.0
        fx, fy, fz = sv.spread(X, F)
        for comp, f in enumerate((fx, fy)):
            assert rel(f, po.spread(g, comp, X, F[comp])) < OPS_TOL
        assert np.all(fz == 0)
        U = sv.interp(X, u, v, w0)
        for comp in range(2):
            assert rel(U[comp], po.interp(g, comp, X, (u, v)[comp])) < OPS_TOL
        assert np.all(U[2] == 0)


def test_2d_mg_solve():
    n = 64
    g = po.Grid(n, n, 1, n)
    b = np.random.default_rng(12).standard_normal(g.ncell)
    tol = 1e-11
    with capi.Solver(n, n, 1, tol=tol) as sv:
        x, cycles = sv.mg_solve(b)
    r = (b - b.mean()) - po.lap_apply(g, x)
    assert np.sqrt(np.mean(r ** 2)) <= tol
    xo, _, _ = po.mg_solve(g, b.copy(), tol)
    assert np.max(np.abs(demean(x) - demean(xo))) <= 1e-9 * np.max(np.abs(demean(xo)))


def _c1(d, precision):
    n = 128
    with capi.Solver(n, n, 1, precision=precision, mu=float(d["mu"]), rho=float(d["rho"]), dt=float(d["dt"]),
                     tol=float(d["tol"]), k_spring=float(d["k"])) as sv:
        z = np.zeros(n * n)
        sv.set_velocity(z, z, z)
        sv.project()
        sv.set_markers(d["X0"], d["nstart"], d["nidx"])
        sv.ib_step(int(d["steps"]))
        u, v, w = sv.get_velocity()
        return u, v, w, sv.get_pressure(), sv.get_markers()


def test_2d_membrane_fp64_matches_oracle(golden):
    """FP64 form after 200 IB steps: velocity, pressure (up to its constant) and
    marker displacement within 1e-10 of the oracle (both solve to 1e-12)."""
    d = golden("c1_2d_128")
    u, v, w, p, X = _c1(d, capi.FP64)
    assert np.all(w == 0)
    assert rel(u, d["u"]) < 1e-10 and rel(v, d["v"]) < 1e-10
    assert rel(demean(p), demean(d["p"])) < 1e-10
    # positions to 1e-10 relative; the displacement (about 3e-6 after 200
    # steps) carries the positions' last-place rounding, hence the looser bound
    assert rel(X, d["X"]) < 1e-10
    assert rel(X - d["X0"], d["X"] - d["X0"]) < 1e-9


def test_2d_membrane_mixed(golden):
    """Mixed form after 200 IB steps: velocity within 1e-8 of the oracle."""
    d = golden("c1_2d_128")
    u, v, w, p, X = _c1(d, capi.MIXED)
    assert rel(u, d["u"]) < 1e-8 and rel(v, d["v"]) < 1e-8
    assert rel(X, d["X"]) < 1e-10
    assert rel(X - d["X0"], d["X"] - d["X0"]) < 1e-8
