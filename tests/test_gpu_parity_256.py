"""FP64 parity with the compiled reference at 256^3 (channel): one BE/CN pair
of NS sub-steps from seeded fields against the digest of the reference's run
(tests/golden/make_golden_256.py). The inputs are regenerated from the seed;
velocity and wall velocities are compared at 4096 seeded cells each and by
their sums, the pressure at the same cells after fitting the null-space
constant on them. Bar: 1e-10 relative to each field's largest magnitude."""
import os

import numpy as np
import pytest

from afmibins_gb300 import capi

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "ns_channel_256_digest.npz")


def _inputs(seed, n=256):
    N, NV = n ** 3, n * (n - 1) * n
    rng = np.random.default_rng(seed)
    u, v, w = 0.1 * rng.standard_normal(N), 0.1 * rng.standard_normal(NV), 0.1 * rng.standard_normal(N)
    fx, fy, fz = rng.standard_normal(N), rng.standard_normal(NV), rng.standard_normal(N)
    return u, v, w, fx, fy, fz


@pytest.mark.skipif(not os.path.exists(FIXTURE), reason="no 256^3 digest fixture")
def test_ns_substeps_channel_256_against_reference_digest():
    d = np.load(FIXTURE)
    n = 256
    u, v, w, fx, fy, fz = _inputs(int(d["seed"]), n)
    mu, rho, dt, tol = float(d["mu"]), float(d["rho"]), float(d["dt"]), float(d["tol"])
    with capi.Solver(n, bc=capi.BC_CHANNEL, mu=mu, rho=rho, dt=dt, tol=tol, max_cg_iters=5000,
                     max_mg_cycles=500) as sv:
        sv.set_velocity(u, v, w)
        sv.project()
        for _ in range(int(d["substeps"])):
            sv.ns_step(fx, fy, fz)
        gu, gv, gw = sv.get_velocity()
        gp = sv.get_pressure()
        walls = np.concatenate(sv.get_walls())
        h1 = sv.helm_apply(0, -mu * dt / (2 * rho), np.ones(n ** 3))
    for name, a in (("u", gu), ("v", gv), ("w", gw), ("walls", walls)):
        scale = float(d[name + "_max"])
        err = np.max(np.abs(a[d[name + "_idx"]] - d[name + "_val"])) / scale
        assert err < 1e-10, (name, err)
        assert abs(a.sum() - float(d[name + "_sum"])) < 1e-10 * scale * a.size ** 0.5, name
    idx = d["p_idx"]
    dlt = gp[idx] - d["p_val"]
    c = float(dlt @ h1[idx] / (h1[idx] @ h1[idx]))
    assert np.max(np.abs(gp[idx] - c * h1[idx] - d["p_val"])) / float(d["p_max"]) < 1e-10


FIXTURE_C3 = os.path.join(HERE, "golden", "c3_periodic_256_digest.npz")


def _c3_inputs():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden_c3", os.path.join(HERE, "golden", "make_golden_c3.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m.inputs(256)


@pytest.mark.skipif(not os.path.exists(FIXTURE_C3), reason="no 256^3 periodic digest fixture")
def test_ib_steps_periodic_256_against_oracle_digest():
    """The FP64 form on the benchmark's own workload (256^3, 200,000 markers,
    2 IB steps, tolerance 1e-12) against the oracle's digest: the yardstick the
    benchmark measures the mixed form's error against is itself pinned at
    full size. Bar 1e-10 of each field's largest magnitude (marker
    displacement for the positions)."""
    d = np.load(FIXTURE_C3)
    X0, nstart, nidx, u, v, w = _c3_inputs()
    for name, a in (("u", u), ("v", v), ("w", w)):
        assert abs(float((a * a).sum()) - float(d[f"in_{name}_sumsq"])) <= 1e-12 * float(d[f"in_{name}_sumsq"])
    n = int(d["n"])
    mu, rho, dt = float(d["mu"]), float(d["rho"]), float(d["dt"])
    with capi.Solver(n, mu=mu, rho=rho, dt=dt, tol=float(d["tol"]), k_spring=float(d["k"]), max_cg_iters=20000,
                     max_mg_cycles=2000) as sv:
        sv.set_velocity(u, v, w)
        sv.project()
        sv.set_markers(X0, nstart, nidx)
        sv.ib_step(int(d["steps"]))
        gu, gv, gw = sv.get_velocity()
        gp = sv.get_pressure()
        X = sv.get_markers()
    err = {}
    for name, a in (("u", gu), ("v", gv), ("w", gw)):
        scale = float(d[name + "_max"])
        err[name] = float(np.max(np.abs(a[d[name + "_idx"]] - d[name + "_val"])) / scale)
        err[name + "_sum"] = abs(float(a.sum()) - float(d[name + "_sum"])) / (scale * a.size ** 0.5)
    idx = d["p_idx"]
    dlt = gp[idx] - d["p_val"]
    err["p"] = float(np.max(np.abs(dlt - dlt.mean())) / float(d["p_max"]))
    midx = d["X_idx"]
    disp = d["X_val"] - d["X0_val"]
    err["X"] = float(np.max(np.abs(X[midx] - d["X_val"])) / np.max(np.abs(disp)))
    assert max(err.values()) < 1e-10, err


FIXTURE_WALLS = os.path.join(HERE, "golden", "ib_channel_256_digest.npz")


@pytest.mark.skipif(not os.path.exists(FIXTURE_WALLS), reason="no 256^3 channel IB digest fixture")
@pytest.mark.parametrize("precision,bar", [(capi.FP64, 1e-10), (capi.MIXED, 1e-8)])
def test_ib_steps_channel_moving_walls_256_against_reference_digest(precision, bar):
    """The reference's own channel domain at 256^3 with moving walls and a
    5,120-marker shell: two IB steps of the FP64 form against the digest of
    the compiled reference (tests/golden/make_golden_walls.py). Velocity at
    4096 seeded cells per component and by its sums, pressure after fitting
    the null-space constant, the updated walls and every marker position.
    Bar 1e-10 of each field's largest magnitude (marker displacement for the
    positions); the mixed form at its bar, 1e-8 (pressure 1e-6, as in the
    other mixed tests)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden_walls",
                                                  os.path.join(HERE, "golden", "make_golden_walls.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    d = np.load(FIXTURE_WALLS)
    n = int(d["n"])
    X0, nstart, nidx, u, v, w, walls0 = gen.inputs_256(n)
    for name, a in (("u", u), ("v", v), ("w", w)):
        assert abs(float((a * a).sum()) - float(d[f"in_{name}_sumsq"])) <= 1e-12 * float(d[f"in_{name}_sumsq"])
    nxz = n * n
    mu, rho, dt = float(d["mu"]), float(d["rho"]), float(d["dt"])
    with capi.Solver(n, bc=capi.BC_CHANNEL, precision=precision, mu=mu, rho=rho, dt=dt, tol=float(d["tol"]),
                     k_spring=float(d["k"]), max_cg_iters=20000, max_mg_cycles=2000) as sv:
        sv.set_velocity(u, v, w)
        sv.set_walls(walls0[:nxz], walls0[nxz:2 * nxz], walls0[2 * nxz:3 * nxz], walls0[3 * nxz:])
        sv.project()
        sv.set_markers(X0, nstart, nidx)
        sv.ib_step(int(d["steps"]))
        gu, gv, gw = sv.get_velocity()
        gp = sv.get_pressure()
        X = sv.get_markers()
        walls = np.concatenate(sv.get_walls())
        h1 = sv.helm_apply(0, -mu * dt / (2 * rho), np.ones(n ** 3))
    err = {}
    for name, a in (("u", gu), ("v", gv), ("w", gw)):
        scale = float(d[name + "_max"])
        err[name] = float(np.max(np.abs(a[d[name + "_idx"]] - d[name + "_val"])) / scale)
        err[name + "_sum"] = abs(float(a.sum()) - float(d[name + "_sum"])) / (scale * a.size ** 0.5)
    idx = d["p_idx"]
    dlt = gp[idx] - d["p_val"]
    c = float(dlt @ h1[idx] / (h1[idx] @ h1[idx]))
    err["p"] = float(np.max(np.abs(gp[idx] - c * h1[idx] - d["p_val"])) / float(d["p_max"]))
    err["walls"] = float(np.max(np.abs(walls - d["walls"])) / np.max(np.abs(d["walls"])))
    err["X"] = float(np.max(np.abs(X - d["X"])) / np.max(np.abs(d["X"] - X0)))
    if precision == capi.MIXED:
        assert err.pop("p") < 1e-6, err
    assert max(err.values()) < bar, err
