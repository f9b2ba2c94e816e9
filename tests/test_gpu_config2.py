"""FP64 parity at the 128^3 icosphere configuration (20,480 markers).

* Periodic cube, 100 IB steps, against the oracle's digest
  (tests/golden/c2_periodic_128_digest.npz): velocity at 4096 seeded cells
  per component and by its sums, pressure at the same cells after fitting the
  null-space constant, all marker positions. Bar 1e-10 relative to each
  field's largest magnitude (displacements for the markers). The mixed form is
  checked against the same digest at the mixed form's bar, 1e-8.
* The reference's own channel domain, 4 IB steps, against the digest of the
  reference compiled unchanged (tests/golden/c2_channel_128_ref_digest.npz),
  same bar.

The inputs are regenerated from the seed by the fixture script's own
generator and checked against the fixture's input checksums first.
"""
import importlib.util
import os

import numpy as np
import pytest

from afmibins_gb300 import capi

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIX_P = os.path.join(HERE, "golden", "c2_periodic_128_digest.npz")
FIX_C = os.path.join(HERE, "golden", "c2_channel_128_ref_digest.npz")


def _gen():
    spec = importlib.util.spec_from_file_location("make_golden_c2", os.path.join(HERE, "golden", "make_golden_c2.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def _check_inputs(d, X, u, v, w):
    for name, a in (("u", u), ("v", v), ("w", w)):
        ref = float(d[f"in_{name}_sumsq"])
        assert abs(float((a * a).sum()) - ref) <= 1e-12 * ref, name
    assert abs(float(X.sum()) - float(d["in_X_sum"])) <= 1e-12 * abs(float(d["in_X_sum"]))


def _run(d, X0, nstart, nidx, u, v, w, bc, precision):
    n = int(d["n"])
    mu, rho, dt = float(d["mu"]), float(d["rho"]), float(d["dt"])
    with capi.Solver(n, bc=bc, precision=precision, mu=mu, rho=rho, dt=dt, tol=float(d["tol"]),
                     k_spring=float(d["k"]), max_cg_iters=20000, max_mg_cycles=2000) as sv:
        sv.set_velocity(u, v, w)
        sv.project()
        sv.set_markers(X0, nstart, nidx)
        sv.ib_step(int(d["steps"]))
        gu, gv, gw = sv.get_velocity()
        gp = sv.get_pressure()
        X = sv.get_markers()
        h1 = sv.helm_apply(0, -mu * dt / (2 * rho), np.ones(n ** 3))
    return gu, gv, gw, gp, X, h1


def _errors(d, X0, gu, gv, gw, gp, X, h1):
    err = {}
    for name, a in (("u", gu), ("v", gv), ("w", gw)):
        scale = float(d[name + "_max"])
        err[name] = float(np.max(np.abs(a[d[name + "_idx"]] - d[name + "_val"])) / scale)
        err[name + "_sum"] = abs(float(a.sum()) - float(d[name + "_sum"])) / (scale * a.size ** 0.5)
    idx = d["p_idx"]
    dlt = gp[idx] - d["p_val"]
    c = float(dlt @ h1[idx] / (h1[idx] @ h1[idx]))
    err["p"] = float(np.max(np.abs(gp[idx] - c * h1[idx] - d["p_val"])) / float(d["p_max"]))
    disp = d["X"] - X0
    err["X"] = float(np.max(np.abs(X - d["X"])) / np.max(np.abs(disp)))
    return err


@pytest.mark.skipif(not os.path.exists(FIX_P), reason="no 128^3 periodic digest fixture")
@pytest.mark.parametrize("precision,bar", [(capi.FP64, 1e-10), (capi.MIXED, 1e-8)])
def test_config2_periodic_100_steps_against_oracle_digest(precision, bar):
    d = np.load(FIX_P)
    X0, nstart, nidx, u, v, w = _gen().inputs(int(d["n"]))
    _check_inputs(d, X0, u, v, w)
    err = _errors(d, X0, *_run(d, X0, nstart, nidx, u, v, w, capi.BC_PERIODIC, precision))
    assert max(err.values()) < bar, err


@pytest.mark.skipif(not os.path.exists(FIX_C), reason="no 128^3 channel digest fixture")
def test_config2_channel_ib_steps_against_reference_digest():
    d = np.load(FIX_C)
    g = _gen()
    n = int(d["n"])
    X0, nstart, nidx, u, vp, w = g.inputs(n)
    v = g.channel_v(vp, n)
    _check_inputs(d, X0, u, v, w)
    err = _errors(d, X0, *_run(d, X0, nstart, nidx, u, v, w, capi.BC_CHANNEL, capi.FP64))
    assert max(err.values()) < 1e-10, err
