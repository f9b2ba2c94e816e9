"""Snapshots on the GPU: a run saved after some IB steps and continued from
the file in a new solver matches the uninterrupted run bit for bit
(velocity, pressure, markers), in both forms and both domains."""
import numpy as np
import pytest

from afmibins_gb300 import capi, markers as mk, snapshot
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _case(n, channel, seed=31):
    rng = np.random.default_rng(seed)
    g = po.Grid(n, n, n, n, channel=channel)
    u, v, w = 0.1 * rng.standard_normal(g.ncell), 0.1 * rng.standard_normal(g.nv), 0.1 * rng.standard_normal(g.ncell)
    P = mk.fibonacci_sphere(400)
    lists = [l[:6] for l in mk.knn_lists(P, 6)]
    X, _ = mk.shell(P, lists, (0.47, 0.5, 0.52), 0.2, 0.02, 0)
    nstart, nidx = mk._csr_from_lists(lists)
    vol = 1.0 + 0.1 * rng.random(len(X))
    return u, v, w, X, nstart, nidx, vol


def _state(sv):
    u, v, w = sv.get_velocity()
    return u, v, w, sv.get_pressure(), sv.get_markers()


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_restart_continues_bit_for_bit(tmp_path, bc, precision):
    n = 32
    u, v, w, X, nstart, nidx, vol = _case(n, bc == capi.BC_CHANNEL)
    path = str(tmp_path / "run.snap")
    kw = dict(bc=bc, precision=precision, mu=0.01, rho=1.0, dt=1e-4, tol=1e-11, k_spring=0.5)
    with capi.Solver(n, **kw) as a:
        a.set_velocity(u, v, w)
        a.project()
        a.set_markers(X, nstart, nidx, vol)
        a.ib_step(2)
        a.ns_step(None, None, None)  # leave the sub-step phase mid-step (BE done, CN next)
        a.save(path)
        a.ib_step(2)
        want = _state(a)
    with capi.Solver(n, **kw) as b:
        b.load(path)
        assert b.M == len(X)
        b.ib_step(2)
        got = _state(b)
    for x, y in zip(want, got):
        assert np.array_equal(x, y)
    sec = snapshot.read(path)
    assert sec["header"]["half"] == 1 and sec["header"]["nx"] == n
    np.testing.assert_array_equal(sec["vol"], vol)


def test_load_rejects_another_grid(tmp_path):
    path = str(tmp_path / "a.snap")
    with capi.Solver(16) as a:
        a.set_velocity(*(np.zeros(16 ** 3) for _ in range(3)))
        a.save(path)
    with capi.Solver(32) as b:
        with pytest.raises(capi.AfmibError) as e:
            b.load(path)
        assert e.value.status == capi.AFMIB_ERR_ARG
    with capi.Solver(16, bc=capi.BC_CHANNEL) as c:
        with pytest.raises(capi.AfmibError):
            c.load(path)
