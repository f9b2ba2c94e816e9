"""The oracle's threaded passes and its direct interior rows give the same
bits as one thread and the generic row builder.

The oracle runs on one thread in every parity test; the CPU baseline of the
benchmark runs it on all host cores at the full 256^3 size. These cases are
large enough (48^3) that every threaded path engages: element-wise passes,
the plane-pipelined lexicographic Gauss-Seidel sweep (src/alg/smooth.h:35-51),
the z-slab spreading and the per-operator cache of face rows.
"""
import hashlib

import numpy as np
import pytest

from oracle import pyoracle as po


def _digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def _ib_run(channel, threads, fast):
    from afmibins_gb300 import markers as mk
    po.set_threads(threads)
    po.set_fast_rows(fast)
    try:
        n = 48
        g = po.Grid(n, n, n, n, channel=channel)
        rng = np.random.default_rng(5)
        u, v, w = (0.05 * rng.standard_normal(s) for s in g.sizes())
        P = mk.fibonacci_sphere(600)
        lists = [l[:6] for l in mk.knn_lists(P, 6)]
        X, _ = mk.shell(P, lists, (0.5, 0.5, 0.5), 0.22, 0.02, 0)
        nstart, nidx = mk._csr_from_lists(lists)
        s = po.NSSolver(g, 0.01, 1.0, 1e-3, 1e-11, u, v, w)
        X, st = s.ib_step(X, nstart, nidx, 0.5)
        assert st == 0
        out = s.get()
        return _digest(*out, X), s.counters()
    finally:
        po.set_threads(1)
        po.set_fast_rows(True)


@pytest.mark.parametrize("channel", [False, True])
def test_ib_step_bits_do_not_depend_on_threads(channel):
    ref = _ib_run(channel, 1, False)
    assert _ib_run(channel, 1, True) == ref
    assert _ib_run(channel, 4, True) == ref
    assert _ib_run(channel, 3, True) == ref


def test_operator_passes_bits_do_not_depend_on_threads():
    n = 48
    rng = np.random.default_rng(9)
    for channel in (False, True):
        g = po.Grid(n, n, n, n, channel=channel)
        x, b = rng.standard_normal(g.ncell), rng.standard_normal(g.ncell)
        Xm = 0.2 + 0.6 * rng.random((500, 3))
        Fm = rng.standard_normal(500)
        runs = []
        for threads, fast in ((1, False), (1, True), (4, True)):
            po.set_threads(threads)
            po.set_fast_rows(fast)
            try:
                xs, it, st = po.cg(g, 0, -0.02, x, b, 1e-9)
                mg, cyc, st2 = po.mg_solve(g, b - b.mean(), 1e-10)
                runs.append(_digest(po.gs_sweep(g, x, b), po.lap_apply(g, x), po.helm_apply(g, 0, -0.02, x),
                                    po.restrict(g, x), po.prolong(g, x[:g.ncell // 8].copy()),
                                    po.spread(g, 0, Xm, Fm), po.spread(g, 1, Xm, Fm),
                                    po.interp(g, 2, Xm, x),
                                    xs, mg) + f"{it},{cyc},{st},{st2}")
            finally:
                po.set_threads(1)
                po.set_fast_rows(True)
        assert runs[0] == runs[1] == runs[2]
