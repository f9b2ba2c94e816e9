"""FP64 parity of the CUDA path (through the C ABI) with the reference.

Channel mode (the reference's own domain) is checked against the golden
vectors of the compiled reference (tests/golden/); periodic mode against the
CPU restatement (oracle/), run live on the same seeded inputs. The bar is the
FP64 drop-in tolerance: 1e-10 relative (max-norm) for fields and markers
after the stated steps; single stencils agree to ~1e-13 (FMA contraction);
pressure is compared after removing its mean (the singular Neumann/periodic
Poisson problem fixes phi only up to a constant)."""
import numpy as np
import pytest

from afmibins_gb300 import capi, markers as mk
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

TOL = 1e-10
OPS_TOL = 1e-13


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def demean(p):
    return p - p.mean()


def pressure_rel(p, pref, g, mu, rho, dt):
    """Pressure p = (I - s Delta) phi is fixed only up to phi -> phi + c. In the
    channel the one-sided wall closure of (I - s Delta) (src/ns/helmholtz.h:94-103)
    does not annihilate constants, so the null-space constant shows up as
    c * (I - s Delta) 1 rather than as a plain shift: fit c, then compare."""
    h1 = po.helm_apply(g, 0, -mu * dt / (2 * rho), np.ones(g.ncell))
    dlt = p - pref
    c = float(dlt @ h1 / (h1 @ h1))
    return rel(p - c * h1, pref)


def test_single_operators_channel(golden):
    d = golden("ops_8")
    s = float(d["s"])
    with capi.Solver(8, bc=capi.BC_CHANNEL, tol=1e-12) as sv:
        assert rel(sv.lap_apply(d["x"]), d["lap"]) < OPS_TOL
        assert rel(sv.restrict(d["x"]), d["restrict"]) < OPS_TOL
        assert rel(sv.prolong(d["c"]), d["prolong"]) < OPS_TOL
        assert rel(sv.div(d["u"], d["v"], d["w"], d["top"], d["bottom"]), d["div"]) < OPS_TOL
        assert rel(np.concatenate(sv.grad(d["x"])), d["grad"]) < OPS_TOL
        assert rel(np.concatenate(sv.advection(d["u"], d["v"], d["w"])), d["advect"]) < OPS_TOL
        h = np.concatenate([sv.helm_apply(0, s, d["u"]), sv.helm_apply(1, s, d["v"]), sv.helm_apply(2, s, d["w"])])
        assert rel(h, d["helm"][: h.size]) < OPS_TOL
        x, it = sv.helmholtz_cg(0, s, d["x0"], d["b"])
        assert rel(x, d["cg_x"]) < TOL


@pytest.mark.parametrize("channel", [False, True])
def test_rb_smoother_one_sweep_against_oracle(channel):
    """One FP64 red-black Gauss-Seidel sweep of the multigrid smoother
    (afmib_smooth) against the oracle's red-black restatement with the
    reference's row update (src/alg/smooth.h:35-51), 16^3."""
    n = 16
    g = po.Grid(n, n, n, n, channel=channel)
    rng = np.random.default_rng(21)
    x0, b = rng.standard_normal(g.ncell), rng.standard_normal(g.ncell)
    ref = po.rb_sweep(g, x0, b)
    with capi.Solver(n, bc=capi.BC_CHANNEL if channel else capi.BC_PERIODIC, tol=1e-12) as sv:
        out = sv.smooth(x0, b)
    assert rel(out, ref) < OPS_TOL


def test_restriction_known_answer(golden):
    d = golden("restr_test")
    with capi.Solver(2, bc=capi.BC_CHANNEL) as sv:
        np.testing.assert_allclose(sv.restrict(d["fine"]), d["coarse"], rtol=1e-15, atol=1e-40)


@pytest.mark.parametrize("name", ["mg_test_16", "mg_test3_16"])
def test_mg_reference_rhs(golden, name):
    d = golden(name)
    b, tol = d["rhs"], float(d["tol"])
    g = po.Grid(16, 16, 16, 16, channel=True)
    with capi.Solver(16, bc=capi.BC_CHANNEL, tol=tol) as sv:
        x, cycles = sv.mg_solve(b)
    r = (b - b.mean()) - po.lap_apply(g, x)
    assert np.sqrt(np.mean(r ** 2)) <= tol
    scale = max(np.max(np.abs(demean(d["x"]))), 1e-300)
    assert np.max(np.abs(demean(x) - demean(d["x"]))) <= max(TOL * scale, 1e-12 / 256)


def test_mg_box_mean_removal(golden):
    # test/mg_test2.cc: geometry<1,8,8,8>, an 8^3 coarsest level, L x = b - mean(b)
    d = golden("mg_test2_box")
    with capi.Solver(16, bc=capi.BC_CHANNEL, n=2, mg_levels=1, tol=float(d["tol"])) as sv:
        x, cycles = sv.mg_solve(d["rhs"])
        lx = sv.lap_apply(x)
    b = d["rhs"]
    np.testing.assert_allclose(lx, b - b.mean(), atol=1e-9)
    assert rel(demean(x), demean(d["x"])) < 1e-9


def test_ns_substeps_channel(golden):
    d = golden("ns_16")
    with capi.Solver(16, bc=capi.BC_CHANNEL, mu=float(d["mu"]), rho=float(d["rho"]), dt=float(d["dt"]),
                     tol=float(d["tol"])) as sv:
        sv.set_velocity(d["u0"], d["v0"], d["w0"])
        sv.project()
        for _ in range(int(d["substeps"])):
            sv.ns_step(d["fx"], d["fy"], d["fz"])
        u, v, w = sv.get_velocity()
        p = sv.get_pressure()
        walls = np.concatenate(sv.get_walls())
    assert rel(u, d["u"]) < TOL
    assert rel(v, d["v"]) < TOL
    assert rel(w, d["w"]) < TOL
    g = po.Grid(16, 16, 16, 16, channel=True)
    assert pressure_rel(p, d["p"], g, float(d["mu"]), float(d["rho"]), float(d["dt"])) < TOL
    assert rel(walls, d["walls"]) < TOL


def test_ns_substeps_channel_warm_start(golden):
    """FP64 form with warm-started projections (AFMIB_START_WARM): each
    projection starts from the previous pressure of its sub-step kind instead
    of the reference's nested iteration from zero, so the pressure converges
    to another point inside the same RMS tolerance. Velocity stays within
    1e-10 of the reference; pressure within 1e-9 (ten times the solver's
    tolerance, relative)."""
    d = golden("ns_16")
    with capi.Solver(16, bc=capi.BC_CHANNEL, mu=float(d["mu"]), rho=float(d["rho"]), dt=float(d["dt"]),
                     tol=float(d["tol"]), proj_start=capi.START_WARM) as sv:
        sv.set_velocity(d["u0"], d["v0"], d["w0"])
        sv.project()
        for _ in range(int(d["substeps"])):
            sv.ns_step(d["fx"], d["fy"], d["fz"])
        u, v, w = sv.get_velocity()
        p = sv.get_pressure()
    assert rel(u, d["u"]) < TOL and rel(v, d["v"]) < TOL and rel(w, d["w"]) < TOL
    g = po.Grid(16, 16, 16, 16, channel=True)
    assert pressure_rel(p, d["p"], g, float(d["mu"]), float(d["rho"]), float(d["dt"])) < 1e-9


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_ns_substeps_channel_extrapolated_start(golden, monkeypatch, precision):
    """Warm start extrapolated from the two previous potentials of the same
    sub-step kind (AFMIB_WARM_EXTRAP=1, phi0 = 2 phi_{n-1} - phi_{n-2}): the
    same fixed point inside the same RMS tolerance, so the bars are those of
    the plain warm start (mixed form: the mixed-form bars, 1e-8 on velocity
    and 1e-6 on pressure, as in the mixed sub-step test below)."""
    monkeypatch.setenv("AFMIB_WARM_EXTRAP", "1")
    d = golden("ns_16")
    with capi.Solver(16, bc=capi.BC_CHANNEL, mu=float(d["mu"]), rho=float(d["rho"]), dt=float(d["dt"]),
                     tol=float(d["tol"]), precision=precision, proj_start=capi.START_WARM) as sv:
        sv.set_velocity(d["u0"], d["v0"], d["w0"])
        sv.project()
        for _ in range(int(d["substeps"])):
            sv.ns_step(d["fx"], d["fy"], d["fz"])
        u, v, w = sv.get_velocity()
        p = sv.get_pressure()
    vt = TOL if precision == capi.FP64 else 1e-8
    assert rel(u, d["u"]) < vt and rel(v, d["v"]) < vt and rel(w, d["w"]) < vt
    g = po.Grid(16, 16, 16, 16, channel=True)
    pt = 1e-9 if precision == capi.FP64 else 1e-6
    assert pressure_rel(p, d["p"], g, float(d["mu"]), float(d["rho"]), float(d["dt"])) < pt


def test_proj_start_rejected():
    with pytest.raises(capi.AfmibError):
        capi.Solver(8, proj_start=3)


def test_spread_interp_channel(golden):
    d = golden("ib_16")
    with capi.Solver(16, bc=capi.BC_CHANNEL) as sv:
        fx, fy, fz = sv.spread(d["X"], d["F"], d["vol"])
        U = sv.interp(d["X"], d["ue"], d["ve"], d["we"])
    assert rel(np.concatenate([fx, fy, fz]), d["spread"]) < OPS_TOL
    assert rel(U.ravel(), d["interp"]) < OPS_TOL


def test_ib_steps_channel(golden):
    d = golden("ib_16")
    with capi.Solver(16, bc=capi.BC_CHANNEL, mu=float(d["mu"]), rho=float(d["rho"]), dt=float(d["dt"]),
                     tol=float(d["tol"]), k_spring=float(d["k"])) as sv:
        sv.set_velocity(d["u0"], d["v0"], d["w0"])
        sv.project()
        sv.set_markers(d["X"], d["nstart"], d["nidx"])
        sv.ib_step(int(d["steps"]))
        u, v, w = sv.get_velocity()
        p = sv.get_pressure()
        X = sv.get_markers()
    assert rel(u, d["u"]) < TOL and rel(v, d["v"]) < TOL and rel(w, d["w"]) < TOL
    g = po.Grid(16, 16, 16, 16, channel=True)
    assert pressure_rel(p, d["p"], g, float(d["mu"]), float(d["rho"]), float(d["dt"])) < TOL
    assert rel(X, d["Xout"]) < TOL


def _periodic_case(n, M=600, seed=7):
    rng = np.random.default_rng(seed)
    g = po.Grid(n, n, n, n, channel=False)
    u, v, w = (0.1 * rng.standard_normal(g.ncell) for _ in range(3))
    P = mk.fibonacci_sphere(M)
    lists = [l[:6] for l in mk.knn_lists(P, 6)]
    X, _ = mk.shell(P, lists, (0.45, 0.52, 0.5), 0.22, 0.02, 0)
    nstart, nidx = mk._csr_from_lists(lists)
    return g, u, v, w, X, nstart, nidx


@pytest.mark.parametrize("n", [16, 32])
def test_ns_substeps_periodic(n):
    g, u, v, w, _, _, _ = _periodic_case(n)
    rng = np.random.default_rng(11)
    f = [rng.standard_normal(g.ncell) for _ in range(3)]
    mu, rho, dt, tol = 0.01, 1.0, 1e-3, 1e-12
    ref = po.NSSolver(g, mu, rho, dt, tol, u, v, w)
    for _ in range(4):
        assert ref.step(*f) == 0
    ru, rv, rw, rp = ref.get()
    with capi.Solver(n, mu=mu, rho=rho, dt=dt, tol=tol) as sv:
        sv.set_velocity(u, v, w)
        sv.project()
        for _ in range(4):
            sv.ns_step(*f)
        gu, gv, gw = sv.get_velocity()
        gp = sv.get_pressure()
    assert rel(gu, ru) < TOL and rel(gv, rv) < TOL and rel(gw, rw) < TOL
    assert rel(demean(gp), demean(rp)) < TOL


def test_ib_steps_periodic():
    n = 32
    g, u, v, w, X, nstart, nidx = _periodic_case(n, M=2000)
    mu, rho, dt, tol, k = 0.01, 1.0, 5e-4, 1e-12, 0.5
    ref = po.NSSolver(g, mu, rho, dt, tol, u, v, w)
    Xr = X.copy()
    for _ in range(3):
        Xr, st = ref.ib_step(Xr, nstart, nidx, k)
        assert st == 0
    ru, rv, rw, _ = ref.get()
    with capi.Solver(n, mu=mu, rho=rho, dt=dt, tol=tol, k_spring=k) as sv:
        sv.set_velocity(u, v, w)
        sv.project()
        sv.set_markers(X, nstart, nidx)
        sv.ib_step(3)
        gu, gv, gw = sv.get_velocity()
        Xg = sv.get_markers()
    assert rel(gu, ru) < TOL and rel(gv, rv) < TOL and rel(gw, rw) < TOL
    assert rel(Xg - X, Xr - X) < 1e-8          # displacement, the sensitive part
    assert np.max(np.abs(Xg - Xr)) < 1e-12


def test_spread_periodic_wraps_images():
    n = 16
    g = po.Grid(n, n, n, n, channel=False)
    rng = np.random.default_rng(3)
    M = 500
    X = rng.uniform(0.0, 1.0, (M, 3))   # markers everywhere, including next to the faces
    F = rng.standard_normal((3, M))
    with capi.Solver(n) as sv:
        fx, fy, fz = sv.spread(X, F)
        U = sv.interp(X, fx, fy, fz)
    ref = [po.spread(g, c, X, F[c].copy()) for c in range(3)]
    assert rel(np.concatenate([fx, fy, fz]), np.concatenate(ref)) < OPS_TOL
    refU = np.stack([po.interp(g, c, X, r) for c, r in enumerate(ref)])
    assert rel(U, refU) < OPS_TOL
    # total force is conserved: sum f h^3 = sum F
    np.testing.assert_allclose(np.array([fx.sum(), fy.sum(), fz.sum()]) / n ** 3, F.sum(1), rtol=1e-12, atol=1e-12)


def test_spread_bitwise_repeatable():
    n = 32
    _, _, _, _, X, _, _ = _periodic_case(n, M=3000)
    F = np.random.default_rng(4).standard_normal((3, X.shape[0]))
    with capi.Solver(n) as sv:
        a = sv.spread(X, F)
        b = sv.spread(X, F)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_failure_statuses_are_reported():
    n = 16
    # a marker next to a channel wall: refused with a status, no fault
    with capi.Solver(n, bc=capi.BC_CHANNEL) as sv:
        X = np.array([[0.5, 0.05, 0.5]])
        with pytest.raises(capi.AfmibError) as e:
            sv.interp(X, np.zeros(sv.ncell), np.zeros(sv.nv), np.zeros(sv.ncell))
        assert e.value.status == capi.AFMIB_ERR_BOUNDS
    # a CG cap that is too small: bounded, reported
    with capi.Solver(n, tol=1e-14, max_cg_iters=1) as sv:
        b = np.random.default_rng(0).standard_normal(sv.ncell)
        with pytest.raises(capi.AfmibError) as e:
            sv.helmholtz_cg(0, -0.3, np.zeros(sv.ncell), b)
        assert e.value.status == capi.AFMIB_ERR_NOCONV
    # NaN in the input: the residual check reports it
    with capi.Solver(n, tol=1e-10) as sv:
        b = np.zeros(sv.ncell)
        b[5] = np.nan
        with pytest.raises(capi.AfmibError) as e:
            sv.mg_solve(b)
        assert e.value.status == capi.AFMIB_ERR_NAN
    # bad configuration
    with pytest.raises(capi.AfmibError) as e:
        capi.Solver(16, mu=0.01, rho=-1.0)
    assert e.value.status == capi.AFMIB_ERR_ARG


# ---------------------------------------------------------------------------
# Mixed precision: FP32 inner solves, spreading and interpolation inside FP64
# defect correction. Bar: relative error <= 1e-8 against the FP64 oracle.
# ---------------------------------------------------------------------------
MIXED_TOL = 1e-8


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
def test_mixed_ns_substeps(bc):
    n = 32
    channel = bc == capi.BC_CHANNEL
    g = po.Grid(n, n, n, n, channel=channel)
    rng = np.random.default_rng(21)
    u, v, w = 0.1 * rng.standard_normal(g.ncell), 0.1 * rng.standard_normal(g.nv), 0.1 * rng.standard_normal(g.ncell)
    f = [rng.standard_normal(g.ncell), rng.standard_normal(g.nv), rng.standard_normal(g.ncell)]
    mu, rho, dt, tol = 0.01, 1.0, 1e-3, 1e-12
    ref = po.NSSolver(g, mu, rho, dt, tol, u, v, w)
    for _ in range(4):
        assert ref.step(*f) == 0
    ru, rv, rw, rp = ref.get()
    with capi.Solver(n, bc=bc, precision=capi.MIXED, mu=mu, rho=rho, dt=dt, tol=tol) as sv:
        sv.set_velocity(u, v, w)
        sv.project()
        for _ in range(4):
            sv.ns_step(*f)
        gu, gv, gw = sv.get_velocity()
        gp = sv.get_pressure()
        st = sv.stats()
    assert st["outer_iters"] > 0
    assert rel(gu, ru) < MIXED_TOL and rel(gv, rv) < MIXED_TOL and rel(gw, rw) < MIXED_TOL
    # The pressure is fed by the small divergent part of the provisional
    # velocity, where the FP32 advection's rounding is not small: its error is
    # stated (bench.py reports it), bounded here at 1e-6.
    assert pressure_rel(gp, rp, g, mu, rho, dt) < 1e-6


def test_mixed_ib_steps_periodic():
    # dt of the 256^3 benchmark configuration: the FP32 spreading error enters
    # the velocity as dt * (FP32 rounding of the force density)
    n = 32
    g, u, v, w, X, nstart, nidx = _periodic_case(n, M=2000)
    mu, rho, dt, tol, k = 0.005, 1.0, 2e-5, 1e-12, 0.5
    ref = po.NSSolver(g, mu, rho, dt, tol, u, v, w)
    Xr = X.copy()
    for _ in range(3):
        Xr, st = ref.ib_step(Xr, nstart, nidx, k)
    ru, rv, rw, _ = ref.get()
    with capi.Solver(n, precision=capi.MIXED, mu=mu, rho=rho, dt=dt, tol=tol, k_spring=k) as sv:
        sv.set_velocity(u, v, w)
        sv.project()
        sv.set_markers(X, nstart, nidx)
        sv.ib_step(3)
        gu, gv, gw = sv.get_velocity()
        Xg = sv.get_markers()
    assert rel(gu, ru) < MIXED_TOL and rel(gv, rv) < MIXED_TOL and rel(gw, rw) < MIXED_TOL
    assert rel(Xg - X, Xr - X) < 1e-6
    assert np.max(np.abs(Xg - Xr)) < 1e-12


def test_mixed_fp32_transfers_run():
    """FP32 spreading and interpolation inside the mixed form (ib_fp32=3) run
    and stay within 1e-6 of the FP64 oracle; the default FP64 transfers are
    the ones held to 1e-8 above."""
    n = 32
    g, u, v, w, X, nstart, nidx = _periodic_case(n, M=2000)
    mu, rho, dt, tol, k = 0.005, 1.0, 2e-5, 1e-12, 0.5
    ref = po.NSSolver(g, mu, rho, dt, tol, u, v, w)
    Xr = X.copy()
    for _ in range(2):
        Xr, st = ref.ib_step(Xr, nstart, nidx, k)
    ru, rv, rw, _ = ref.get()
    with capi.Solver(n, precision=capi.MIXED, mu=mu, rho=rho, dt=dt, tol=tol, k_spring=k, ib_fp32=3) as sv:
        sv.set_velocity(u, v, w)
        sv.project()
        sv.set_markers(X, nstart, nidx)
        sv.ib_step(2)
        gu, gv, gw = sv.get_velocity()
    assert rel(gu, ru) < 1e-6 and rel(gv, rv) < 1e-6 and rel(gw, rw) < 1e-6


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
@pytest.mark.parametrize("shape", [(64, 64, 64), (32, 16, 8), (128, 64, 32)])
def test_pipelined_smoother_equals_per_colour(monkeypatch, bc, shape):
    """The pipelined sweep (bulk-copy row ring, z-marching blocks) performs
    the per-colour kernels' arithmetic in the same order: one sweep and a
    whole multigrid solve agree bit for bit."""
    nx, ny, nz = shape
    rng = np.random.default_rng(21)
    x0 = rng.standard_normal(nx * ny * nz)
    b = rng.standard_normal(nx * ny * nz)
    out = {}
    monkeypatch.setenv("AFMIB_PIPE_MIN_NX", "32")
    for mode in ("percolour", "pipe"):
        monkeypatch.setenv("AFMIB_SMOOTHER", mode)
        with capi.Solver(nx, ny, nz, n=nx, bc=bc, tol=1e-10) as sv:
            out[mode] = (sv.smooth(x0, b), sv.mg_solve(b)[0])
    assert np.array_equal(out["percolour"][0], out["pipe"][0])
    assert np.array_equal(out["percolour"][1], out["pipe"][1])


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
def test_block_arithmetic_defects_match_fp64_defects(monkeypatch, bc):
    """The mixed form's FP64-state defects from int64 block arithmetic (no FP64
    instruction) against the FP64 defect kernels: both stop on the same
    residual tests, so four NS sub-steps agree to the solver tolerance."""
    n = 32
    channel = bc == capi.BC_CHANNEL
    g = po.Grid(n, n, n, n, channel=channel)
    rng = np.random.default_rng(22)
    u, v, w = 0.1 * rng.standard_normal(g.ncell), 0.1 * rng.standard_normal(g.nv), 0.1 * rng.standard_normal(g.ncell)
    f = [rng.standard_normal(g.ncell), rng.standard_normal(g.nv), rng.standard_normal(g.ncell)]
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("AFMIB_BFP", mode)
        with capi.Solver(n, bc=bc, precision=capi.MIXED, mu=0.01, rho=1.0, dt=1e-3, tol=1e-12) as sv:
            sv.set_velocity(u, v, w)
            sv.project()
            for _ in range(4):
                sv.ns_step(*f)
            out[mode] = sv.get_velocity()
    for a, b in zip(out["0"], out["1"]):
        assert rel(b, a) < 1e-10


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
@pytest.mark.parametrize("n", [16, 32, 64])
def test_multigrid_tail_equals_level_launches(monkeypatch, bc, precision, n):
    """The V-cycle tail (in one block from 16^3, or on a thread-block cluster
    from 32^3 with AFMIB_MG_TAIL_CLUSTER=16) runs the per-cell functions of the
    level kernels and the same coarsest-level CG: multigrid solves agree bit
    for bit with the launch-by-launch V-cycle, and repeat bit for bit, with
    the one-block tail on 256, 512 (the default) or 1024 threads."""
    b = np.random.default_rng(23).standard_normal(n ** 3)
    out = {}
    for mode, tail, cluster, threads in (("levels", "0", None, None), ("cluster", "1", "16", None),
                                         ("cluster2", "1", "16", None), ("block", "1", None, None),
                                         ("block256", "1", None, "256"), ("block1024", "1", None, "1024")):
        monkeypatch.setenv("AFMIB_MG_TAIL", tail)
        if cluster:
            monkeypatch.setenv("AFMIB_MG_TAIL_CLUSTER", cluster)
        else:
            monkeypatch.delenv("AFMIB_MG_TAIL_CLUSTER", raising=False)
        if threads:
            monkeypatch.setenv("AFMIB_TAIL_THREADS", threads)
        else:
            monkeypatch.delenv("AFMIB_TAIL_THREADS", raising=False)
        with capi.Solver(n, bc=bc, precision=precision, tol=1e-10) as sv:
            out[mode] = sv.mg_solve(b)
    for mode in ("cluster", "cluster2", "block", "block256", "block1024"):
        assert out[mode][1] == out["levels"][1]
        assert np.array_equal(out[mode][0], out["levels"][0])


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
def test_inner_jacobi_matches_inner_cg(monkeypatch, bc):
    """Mixed form: the FP32 inner Helmholtz solves by a fixed number of Jacobi
    sweeps (bounded by the operator's diagonal dominance), of red-black
    Gauss-Seidel sweeps, or by CG; the FP64 outer loop stops on the same
    residual test, so the sub-steps agree to the solver tolerance."""
    n = 32
    channel = bc == capi.BC_CHANNEL
    g = po.Grid(n, n, n, n, channel=channel)
    rng = np.random.default_rng(24)
    u, v, w = 0.1 * rng.standard_normal(g.ncell), 0.1 * rng.standard_normal(g.nv), 0.1 * rng.standard_normal(g.ncell)
    f = [rng.standard_normal(g.ncell), rng.standard_normal(g.nv), rng.standard_normal(g.ncell)]
    out = {}
    for mode in ("cg", "jacobi", "gs"):
        monkeypatch.setenv("AFMIB_INNER_SOLVER", mode)
        with capi.Solver(n, bc=bc, precision=capi.MIXED, mu=0.01, rho=1.0, dt=1e-3, tol=1e-12) as sv:
            sv.set_velocity(u, v, w)
            sv.project()
            for _ in range(4):
                sv.ns_step(*f)
            out[mode] = sv.get_velocity()
    for mode in ("jacobi", "gs"):
        for a, b in zip(out["cg"], out[mode]):
            assert rel(b, a) < 1e-10


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
def test_power_of_two_kernels_match_general_kernels(monkeypatch, bc):
    """The power-of-two kernels (32-bit shift-composed indices, several planes
    per thread: smoother, residual, transfers, Jacobi sweeps) evaluate the
    same terms in the same order as the general kernels (AFMIB_IX2=0): an
    FP64 multigrid solve agrees bit for bit, mixed-form sub-steps to the
    solver tolerance."""
    n = 64
    channel = bc == capi.BC_CHANNEL
    g = po.Grid(n, n, n, n, channel=channel)
    rng = np.random.default_rng(25)
    b = rng.standard_normal(g.ncell)
    u, v, w = 0.1 * rng.standard_normal(g.ncell), 0.1 * rng.standard_normal(g.nv), 0.1 * rng.standard_normal(g.ncell)
    f = [rng.standard_normal(g.ncell), rng.standard_normal(g.nv), rng.standard_normal(g.ncell)]
    mg, ns = {}, {}
    for mode in ("0", "1"):
        monkeypatch.setenv("AFMIB_IX2", mode)
        with capi.Solver(n, bc=bc, precision=capi.FP64, tol=1e-10) as sv:
            mg[mode] = sv.mg_solve(b)
        with capi.Solver(n, bc=bc, precision=capi.MIXED, mu=0.01, rho=1.0, dt=1e-3, tol=1e-12) as sv:
            sv.set_velocity(u, v, w)
            sv.project()
            for _ in range(2):
                sv.ns_step(*f)
            ns[mode] = sv.get_velocity()
    assert mg["0"][1] == mg["1"][1]
    assert np.array_equal(mg["0"][0], mg["1"][0])
    for a, c in zip(ns["0"], ns["1"]):
        assert rel(c, a) < 1e-10


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
def test_inner_cycle_schedule_matches_plain_gauss_seidel(monkeypatch, bc):
    """Mixed form: the FP32 inner V-cycles' own schedule (V(2,1), red-black
    over-relaxation 1.25 on levels >= 64) against V(2,2) plain Gauss-Seidel
    (AFMIB_INNER_OMEGA=1, AFMIB_INNER_NU=2,2): both are preconditioners of the
    same FP64 defect correction and stop on the same residual test, so the
    sub-steps agree to the solver tolerance: RMS(r) <= 1e-12 leaves the
    velocities 1e-10 to 1e-9 apart (max-norm, relative), and each solve's own
    residual is checked against the oracle's Laplacian."""
    n = 64
    channel = bc == capi.BC_CHANNEL
    g = po.Grid(n, n, n, n, channel=channel)
    rng = np.random.default_rng(26)
    u, v, w = 0.1 * rng.standard_normal(g.ncell), 0.1 * rng.standard_normal(g.nv), 0.1 * rng.standard_normal(g.ncell)
    f = [rng.standard_normal(g.ncell), rng.standard_normal(g.nv), rng.standard_normal(g.ncell)]
    out = {}
    for mode, env in (("plain", ("1", "2,2")), ("default", None)):
        if env:
            monkeypatch.setenv("AFMIB_INNER_OMEGA", env[0])
            monkeypatch.setenv("AFMIB_INNER_NU", env[1])
        else:
            monkeypatch.delenv("AFMIB_INNER_OMEGA", raising=False)
            monkeypatch.delenv("AFMIB_INNER_NU", raising=False)
        with capi.Solver(n, bc=bc, precision=capi.MIXED, mu=0.01, rho=1.0, dt=1e-3, tol=1e-12) as sv:
            sv.set_velocity(u, v, w)
            sv.project()
            for _ in range(2):
                sv.ns_step(*f)
            out[mode] = sv.get_velocity()
            b = rng.standard_normal(g.ncell)
            x, cycles = sv.mg_solve(b)
        r = (b - b.mean()) - po.lap_apply(g, x)
        assert np.sqrt(np.mean(r ** 2)) <= 2e-12
    for a, c in zip(out["plain"], out["default"]):
        assert rel(c, a) < 1e-9


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_alternating_block_order_keeps_bits(monkeypatch, precision):
    """Passes over fields larger than L2 (256^3) alternate their block order;
    the kernels that take it are pointwise or update one red-black colour, so
    a multigrid solve is bit for bit the one in index order
    (AFMIB_ALTERNATE=0)."""
    n = 256
    b = np.random.default_rng(27).standard_normal(n ** 3)
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("AFMIB_ALTERNATE", mode)
        with capi.Solver(n, precision=precision, tol=1e-8) as sv:
            out[mode] = sv.mg_solve(b)
    assert out["0"][1] == out["1"][1]
    assert np.array_equal(out["0"][0], out["1"][0])


@pytest.mark.parametrize("n,bc", [(128, capi.BC_PERIODIC), (128, capi.BC_CHANNEL), (256, capi.BC_PERIODIC),
                                  (256, capi.BC_CHANNEL), ((256, 128, 64), capi.BC_PERIODIC),
                                  ((256, 128, 64), capi.BC_CHANNEL)])
def test_column_transfers_keep_bits(monkeypatch, n, bc):
    """Mixed form: the FP32 column-marching restriction and prolongation (fine
    tiles staged in shared memory by asynchronous copies, 16 bytes per lane
    with the neighbouring cells from adjacent lanes, a block walking 1, 2, 4
    or 8 coarse planes) evaluate the one-cell kernels' expressions in their
    order (AFMIB_TRANSFER_COLS=0): a multigrid solve agrees bit for bit, with
    the same cycle count, whatever the planes per block; at 256^3 the passes
    alternate their block order too."""
    precision = capi.MIXED
    channel = bc == capi.BC_CHANNEL
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    g = po.Grid(nx, ny, nz, nx, channel=channel)
    b = np.random.default_rng(29).standard_normal(g.ncell)
    out = {}
    for mode, min_blocks, max_planes in (("0", None, None), ("1", None, None), ("1", "1", "8"), ("1", "256", "2"),
                                         ("1", "100000000", "1")):
        monkeypatch.setenv("AFMIB_TRANSFER_COLS", mode)
        for key, val in (("AFMIB_TRANSFER_MIN_BLOCKS", min_blocks), ("AFMIB_PROLONG_MAX_PLANES", max_planes)):
            if val:
                monkeypatch.setenv(key, val)
            else:
                monkeypatch.delenv(key, raising=False)
        with capi.Solver(nx, ny, nz, n=nx, bc=bc, precision=precision, tol=1e-9) as sv:
            out[(mode, min_blocks)] = sv.mg_solve(b)
    ref = out[("0", None)]
    for key, (x, cycles) in out.items():
        assert cycles == ref[1], key
        assert np.array_equal(x, ref[0]), key


@pytest.mark.parametrize("n,bc,markers", [(64, capi.BC_PERIODIC, True), (64, capi.BC_CHANNEL, False),
                                          (256, capi.BC_PERIODIC, False)])
def test_interleaved_viscous_solves_keep_bits(monkeypatch, n, bc, markers):
    """Mixed form: the three viscous solves of a sub-step interleaved on two
    streams (one component's FP32 correction beside the next component's FP64
    defect, the defects on a persistent grid of 3 or 8 blocks per SM; FP64
    defects throughout, AFMIB_HELM_DF=0) go through the same defects,
    corrections and stopping tests as the solves one after another
    (AFMIB_HELM_OVERLAP=0): the same velocity, pressure and markers bit for
    bit, and the same number of defect-correction steps."""
    channel = bc == capi.BC_CHANNEL
    g = po.Grid(n, n, n, n, channel=channel)
    rng = np.random.default_rng(28)
    u, v, w = 0.1 * rng.standard_normal(g.ncell), 0.1 * rng.standard_normal(g.nv), 0.1 * rng.standard_normal(g.ncell)
    f = [rng.standard_normal(g.ncell), rng.standard_normal(g.nv), rng.standard_normal(g.ncell)]
    monkeypatch.setenv("AFMIB_HELM_DF", "0")
    out = {}
    for mode, blocks in (("0", None), ("1", None), ("1", "8")):
        monkeypatch.setenv("AFMIB_HELM_OVERLAP", mode)
        if blocks:
            monkeypatch.setenv("AFMIB_HELM_WALK_BLOCKS", blocks)
        else:
            monkeypatch.delenv("AFMIB_HELM_WALK_BLOCKS", raising=False)
        with capi.Solver(n, bc=bc, precision=capi.MIXED, mu=0.01, rho=1.0, dt=1e-3, tol=1e-10,
                         k_spring=0.5) as sv:
            sv.set_velocity(u, v, w)
            sv.project()
            if markers:
                _, _, _, _, X, nstart, nidx = _periodic_case(n, M=2000, seed=29)
                sv.set_markers(X, nstart, nidx)
                sv.ib_step(3)
                gX = sv.get_markers()
            else:
                for _ in range(4):
                    sv.ns_step(*f)
                gX = None
            out[(mode, blocks)] = (sv.get_velocity(), sv.get_pressure(), gX, sv.stats()["outer_iters"])
    ref = out[("0", None)]
    for key in (("1", None), ("1", "8")):
        got = out[key]
        for a, b in zip(ref[0], got[0]):
            assert np.array_equal(a, b)
        assert np.array_equal(ref[1], got[1])
        if markers:
            assert np.array_equal(ref[2], got[2])
        assert ref[3] == got[3]


@pytest.mark.parametrize("n,bc,markers", [(64, capi.BC_PERIODIC, True), (64, capi.BC_CHANNEL, False),
                                          (32, capi.BC_CHANNEL, True), (256, capi.BC_PERIODIC, False)])
def test_double_float_outer_residual(monkeypatch, n, bc, markers):
    """Mixed form: after the first FP64 defect of each viscous and pressure
    solve, the outer residual is kept as a double-float pair and updated by
    r -= H e (r -= L e) with the FP32 correction's rows in double-float
    (2^-46) instead of re-evaluating b - H x (b - L x) with the FP64 stencil.
    The FP64 state x takes the same += e, the stopping tests the same norms,
    so the sub-steps agree with the FP64-defect solves to the solver
    tolerance (1e-10 relative, as the inner-solver variants; 1e-9 at 256^3)
    and with the FP64 form to the mixed form's 1e-8 bar. The IB cases also spread their
    forces with double-float products and sums (2^-44) against FP64
    spreading (AFMIB_SPREAD_DF)."""
    channel = bc == capi.BC_CHANNEL
    g = po.Grid(n, n, n, n, channel=channel)
    rng = np.random.default_rng(32)
    u, v, w = 0.1 * rng.standard_normal(g.ncell), 0.1 * rng.standard_normal(g.nv), 0.1 * rng.standard_normal(g.ncell)
    f = [rng.standard_normal(g.ncell), rng.standard_normal(g.nv), rng.standard_normal(g.ncell)]
    _, _, _, _, X, nstart, nidx = _periodic_case(n, M=2000, seed=33)
    out = {}
    for key, prec, df in (("fp64", capi.FP64, "1"), ("defects", capi.MIXED, "0"), ("df", capi.MIXED, "1")):
        monkeypatch.setenv("AFMIB_HELM_DF", df)
        monkeypatch.setenv("AFMIB_LAP_DF", df)
        monkeypatch.setenv("AFMIB_SPREAD_DF", df)
        with capi.Solver(n, bc=bc, precision=prec, mu=0.01, rho=1.0, dt=1e-3, tol=1e-11, k_spring=0.5) as sv:
            sv.set_velocity(u, v, w)
            sv.project()
            if markers:
                sv.set_markers(X, nstart, nidx)
                sv.ib_step(3)
            else:
                for _ in range(4):
                    sv.ns_step(*f)
            out[key] = sv.get_velocity()
    # both pressure solves stop at RMS(r) <= tol: at 256^3 the 2-norm of
    # what each leaves is 4096 times that, and their velocities differ by
    # more than at 32^3-64^3 (measured 1.7e-10 after 4 sub-steps)
    bar = 1e-10 if n <= 64 else 1e-9
    for a, b in zip(out["defects"], out["df"]):
        assert rel(b, a) < bar
    for a, b in zip(out["fp64"], out["df"]):
        assert rel(b, a) < 1e-8


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
@pytest.mark.parametrize("n", [32, 128])
def test_pressure_double_float_residual(monkeypatch, bc, n):
    """Mixed pressure solves with the double-float recursive residual reach
    the reference's stopping rule on the true FP64 residual: RMS(b - mean(b)
    - L x) <= tol, L applied in FP64 through the C ABI, and agree with the
    FP64-defect solves to that tolerance."""
    b = np.random.default_rng(35).standard_normal(n ** 3)
    tol = 1e-9
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("AFMIB_LAP_DF", mode)
        with capi.Solver(n, bc=bc, precision=capi.MIXED, tol=tol) as sv:
            x, cycles = sv.mg_solve(b)
            r = (b - b.mean()) - sv.lap_apply(x)
            out[mode] = x
        assert np.sqrt(np.mean(r ** 2)) <= tol * (1 + 1e-6)
    # both residuals within tol: the potentials differ by L^-1 of at most
    # 2 tol, and L's smallest nonzero eigenvalue is pi^2 or more
    d0, d1 = demean(out["0"]), demean(out["1"])
    assert np.max(np.abs(d1 - d0)) <= 10 * tol


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
def test_double_float_update_kernels_agree(monkeypatch, bc):
    """The residual update's power-of-two kernel (eight z cells per thread,
    the column reused from registers) and its general kernel
    (AFMIB_UPDATE_DF_GENERIC=1) evaluate the same double-float rows: the same
    velocity bit for bit."""
    n = 64
    channel = bc == capi.BC_CHANNEL
    g = po.Grid(n, n, n, n, channel=channel)
    rng = np.random.default_rng(34)
    u, v, w = 0.1 * rng.standard_normal(g.ncell), 0.1 * rng.standard_normal(g.nv), 0.1 * rng.standard_normal(g.ncell)
    f = [rng.standard_normal(g.ncell), rng.standard_normal(g.nv), rng.standard_normal(g.ncell)]
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("AFMIB_UPDATE_DF_GENERIC", mode)
        with capi.Solver(n, bc=bc, precision=capi.MIXED, mu=0.01, rho=1.0, dt=1e-3, tol=1e-11) as sv:
            sv.set_velocity(u, v, w)
            sv.project()
            for _ in range(4):
                sv.ns_step(*f)
            out[mode] = (sv.get_velocity(), sv.stats()["outer_iters"])
    for a, b in zip(out["0"][0], out["1"][0]):
        assert np.array_equal(a, b)
    assert out["0"][1] == out["1"][1]


@pytest.mark.parametrize("m", [1200, 5000, 20000])
def test_spread_dense_cluster_takes_large_capacity_pass(m):
    """m markers inside two cells: 1,200 exceed the first pass's capacity and
    are spread by the large-capacity pass; 5,000 and 20,000 exceed that one
    too and are spread in chunks of its capacity. Same result as the oracle
    in every case, and the same bits on a repeat."""
    n = 32
    g = po.Grid(n, n, n, n, channel=False)
    rng = np.random.default_rng(25)
    X = 0.5 + rng.uniform(-1.0, 1.0, (m, 3)) / n
    F = rng.standard_normal((3, m))
    with capi.Solver(n) as sv:
        fx, fy, fz = sv.spread(X, F)
        again = sv.spread(X, F)
    for comp, f in enumerate((fx, fy, fz)):
        assert rel(f, po.spread(g, comp, X, F[comp])) < OPS_TOL
        assert np.array_equal(f, again[comp])


@pytest.mark.parametrize("dims", [(16, 8, 16), (16, 16, 8)])
@pytest.mark.parametrize("corrected", [0, 1])
def test_channel_walls_noncubic(dims, corrected):
    """Channel sub-steps on non-cubic grids, the wall-velocity update in the
    reference's form (its loop over nx*ny entries; only grids with ny <= nz,
    where that loop stays inside the arrays) or corrected (every nx*nz entry,
    w rows from the z-gradient), against the oracle in the same mode."""
    nx, ny, nz = dims
    if not corrected and ny > nz:
        pytest.skip("the reference's loop reads past the gradient arrays when ny > nz")
    g = po.Grid(nx, ny, nz, nx, channel=True)
    rng = np.random.default_rng(42)
    u, v, w = 0.1 * rng.standard_normal(g.ncell), 0.1 * rng.standard_normal(g.nv), 0.1 * rng.standard_normal(g.ncell)
    f = [rng.standard_normal(g.ncell), rng.standard_normal(g.nv), rng.standard_normal(g.ncell)]
    mu, rho, dt, tol = 0.01, 1.0, 1e-3, 1e-12
    ref = po.NSSolver(g, mu, rho, dt, tol, u, v, w, walls_corrected=bool(corrected))
    for _ in range(4):
        assert ref.step(*f) == 0
    ru, rv, rw, _ = ref.get()
    with capi.Solver(nx, ny, nz, n=nx, bc=capi.BC_CHANNEL, mu=mu, rho=rho, dt=dt, tol=tol,
                     walls_corrected=corrected) as sv:
        sv.set_velocity(u, v, w)
        sv.project()
        for _ in range(4):
            sv.ns_step(*f)
        gu, gv, gw = sv.get_velocity()
        walls = np.concatenate(sv.get_walls())
    assert rel(gu, ru) < TOL and rel(gv, rv) < TOL and rel(gw, rw) < TOL
    assert rel(walls, ref.walls) < TOL


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_ib_steps_with_bending_periodic(precision):
    """IB steps with membrane bending (k_bend: force -k_bend L (L X)) against
    the oracle: FP64 to 1e-10, the mixed form to its 1e-8 bar."""
    n = 16
    g, u, v, w, X, nstart, nidx = _periodic_case(n, M=400, seed=23)
    mu, rho, dt, tol, k, kb = 0.01, 1.0, 1e-3, 1e-12, 0.5, 0.05
    ref = po.NSSolver(g, mu, rho, dt, tol, u, v, w)
    Xr = X.copy()
    for _ in range(3):
        Xr, st = ref.ib_step(Xr, nstart, nidx, k, kb)
        assert st == 0
    ru, rv, rw, _ = ref.get()
    with capi.Solver(n, precision=precision, mu=mu, rho=rho, dt=dt, tol=tol, k_spring=k, k_bend=kb) as sv:
        sv.set_velocity(u, v, w)
        sv.project()
        sv.set_markers(X, nstart, nidx)
        sv.ib_step(3)
        gu, gv, gw = sv.get_velocity()
        gX = sv.get_markers()
    bar = TOL if precision == capi.FP64 else MIXED_TOL
    assert rel(gu, ru) < bar and rel(gv, rv) < bar and rel(gw, rw) < bar
    assert rel(gX, Xr) < bar


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
def test_double_float_interpolation_matches_fp64(monkeypatch, bc):
    """The mixed form's interpolation in double-float on the FP32 pipe
    (k_interp_dfl, axis-by-axis sums) against the FP64 kernel: two mixed IB
    steps with each, velocities and marker displacements agree far below the
    mixed form's 1e-8 bar (the marker velocities differ by a few units of
    2^-46, the steps' solver tolerance is 1e-12)."""
    g, u, v, w, X, nstart, nidx = _periodic_case(32, M=800, seed=13)
    if bc == capi.BC_CHANNEL:
        v = v[: g.nx * (g.ny - 1) * g.nz]
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("AFMIB_INTERP_DF", mode)
        with capi.Solver(32, bc=bc, precision=capi.MIXED, mu=0.01, dt=1e-3, tol=1e-12, k_spring=0.5) as sv:
            sv.set_velocity(u, v, w)
            sv.project()
            sv.set_markers(X, nstart, nidx)
            sv.ib_step(2)
            out[mode] = (sv.get_velocity(), sv.get_markers())
    for a, b in zip(out["1"][0], out["0"][0]):
        assert rel(a, b) < 1e-10
    assert rel(out["1"][1] - X, out["0"][1] - X) < 1e-10


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
def test_double_float_marker_weights(monkeypatch, bc):
    """The mixed form's marker weights from double-float sines and cosines
    (df_sincospi on the FP32 pipe, within 2^-45 of the FP64 sincospi weights)
    against the FP64 weights (AFMIB_PREP_DF=0): two IB steps, velocities and
    marker displacements agree to 1e-11."""
    g, u, v, w, X, nstart, nidx = _periodic_case(32, M=800, seed=15)
    if bc == capi.BC_CHANNEL:
        v = v[: g.nx * (g.ny - 1) * g.nz]
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("AFMIB_PREP_DF", mode)
        with capi.Solver(32, bc=bc, precision=capi.MIXED, mu=0.01, dt=1e-3, tol=1e-12, k_spring=0.5) as sv:
            sv.set_velocity(u, v, w)
            sv.project()
            sv.set_markers(X, nstart, nidx)
            sv.ib_step(2)
            out[mode] = (sv.get_velocity(), sv.get_markers())
    for a, b in zip(out["1"][0], out["0"][0]):
        assert rel(a, b) < 1e-11
    assert rel(out["1"][1] - X, out["0"][1] - X) < 1e-11


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
def test_interpolation_from_velocity_pairs(monkeypatch, bc):
    """The mixed form's double-float interpolation reading the velocity's
    float pairs, which the projection writes (hi + lo = u to 2^-46), against
    splitting the FP64 values itself (AFMIB_INTERP_PAIRS=0): two IB steps,
    velocities and marker displacements agree to 1e-12 (the two represent
    each face value to 2^-46 and differ only in how the bits are parted)."""
    g, u, v, w, X, nstart, nidx = _periodic_case(32, M=800, seed=14)
    if bc == capi.BC_CHANNEL:
        v = v[: g.nx * (g.ny - 1) * g.nz]
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("AFMIB_INTERP_PAIRS", mode)
        with capi.Solver(32, bc=bc, precision=capi.MIXED, mu=0.01, dt=1e-3, tol=1e-12, k_spring=0.5) as sv:
            sv.set_velocity(u, v, w)
            sv.project()
            sv.set_markers(X, nstart, nidx)
            sv.ib_step(2)
            out[mode] = (sv.get_velocity(), sv.get_markers())
    for a, b in zip(out["1"][0], out["0"][0]):
        assert rel(a, b) < 1e-12
    assert rel(out["1"][1] - X, out["0"][1] - X) < 1e-12


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
def test_double_float_projection_matches_fp64_passes(monkeypatch, bc):
    """The mixed form's projection passes in double-float (divergence with the
    sum of b, the first pressure defect with the mean removal folded in)
    against their FP64 kernels (AFMIB_PROJ_DF=0): two IB steps at 64^3 with
    seeded moving walls in the channel, velocity, pressure and markers far
    below the mixed form's 1e-8 bar (the passes differ by a few units of
    2^-46 of their terms; the solver tolerance is 1e-12 absolute). A
    pressure solve through the C ABI
    (the sum taken by its own pass, the mean folded into the defect) meets
    its tolerance on the FP64 residual."""
    n = 64
    g, u, v, w, X, nstart, nidx = _periodic_case(n, M=2000, seed=31)
    channel = bc == capi.BC_CHANNEL
    if channel:
        v = v[: g.nx * (g.ny - 1) * g.nz]
    walls = np.random.default_rng(33).standard_normal(4 * n * n) * 0.05 if channel else None
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("AFMIB_PROJ_DF", mode)
        with capi.Solver(n, bc=bc, precision=capi.MIXED, mu=0.01, dt=1e-3, tol=1e-12, k_spring=0.5) as sv:
            sv.set_velocity(u, v, w)
            if walls is not None:
                sv.set_walls(*np.split(walls, 4))
            sv.project()
            sv.set_markers(X, nstart, nidx)
            sv.ib_step(2)
            out[mode] = (sv.get_velocity(), sv.get_pressure(), sv.get_markers())
            b = np.random.default_rng(32).standard_normal(g.ncell)
            x, _ = sv.mg_solve(b)
        gp = po.Grid(n, n, n, n, channel=channel)
        r = (b - b.mean()) - po.lap_apply(gp, x)
        assert np.sqrt(np.mean(r ** 2)) <= 2e-12
    for a, b_ in zip(out["1"][0], out["0"][0]):
        assert rel(a, b_) < 1e-10
    gp = po.Grid(n, n, n, n, channel=channel)
    assert pressure_rel(out["1"][1], out["0"][1], gp, 0.01, 1.0, 1e-3) < 1e-8
    assert rel(out["1"][2] - X, out["0"][2] - X) < 1e-10


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_fused_residual_restriction_keeps_bits(monkeypatch, bc, precision):
    """The fine-level residual fused with the restriction (k_resid_restrict2,
    the residual kept in shared memory) against the residual and restriction
    kernels: the same terms in the same order, so multigrid solves and IB
    steps agree bit for bit (the fused kernel taken from 32-cell levels here,
    both of its z chunkings: 256^3 takes 8 coarse planes per block)."""
    monkeypatch.setenv("AFMIB_RESID_RESTRICT_MIN_NX", "32")
    for shape in ((64, 64, 64), (128, 64, 32), (256, 256, 256)):
        nx, ny, nz = shape
        rng = np.random.default_rng(5)
        b = rng.standard_normal(nx * ny * nz)
        b -= b.mean()
        out = {}
        for mode in ("0", "1"):
            monkeypatch.setenv("AFMIB_RESID_RESTRICT", mode)
            with capi.Solver(nx, ny, nz, n=nx, bc=bc, precision=precision, tol=1e-10) as sv:
                out[mode] = sv.mg_solve(b)
        assert np.array_equal(out["0"][0], out["1"][0]) and out["0"][1] == out["1"][1], shape
    g, u, v, w, X, nstart, nidx = _periodic_case(64, M=800, seed=3)
    if bc == capi.BC_CHANNEL:
        v = v[: g.nx * (g.ny - 1) * g.nz]
    res = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("AFMIB_RESID_RESTRICT", mode)
        with capi.Solver(64, bc=bc, precision=precision, mu=0.01, dt=1e-3, tol=1e-10, k_spring=0.5) as sv:
            sv.set_velocity(u, v, w)
            sv.project()
            sv.set_markers(X, nstart, nidx)
            sv.ib_step(2)
            res[mode] = (*sv.get_velocity(), sv.get_pressure(), sv.get_markers())
    for a, c in zip(res["0"], res["1"]):
        assert np.array_equal(a, c)


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
def test_column_residual_restriction_keeps_bits(monkeypatch, bc):
    """Mixed form: the FP32 fine-level residual fused with the column
    restriction (k_resid_restrict_cols: x and b planes staged by asynchronous
    copies, the residual plane kept in shared memory; the default on levels of
    256 cells and up, taken here from 128) against the residual and
    restriction kernels (AFMIB_RESID_RESTRICT=0): multigrid solves agree bit
    for bit with 8, 4 or 1 coarse planes per block, and so do IB steps."""
    monkeypatch.setenv("AFMIB_RR_COLS_MIN_NX", "128")
    for shape in ((128, 128, 128), (256, 256, 256), (256, 128, 64)):
        nx, ny, nz = shape
        b = np.random.default_rng(6).standard_normal(nx * ny * nz)
        b -= b.mean()
        out = {}
        for mode, min_blocks in (("0", None), ("2", None), ("2", "1"), ("2", "100000000")):
            monkeypatch.setenv("AFMIB_RESID_RESTRICT", mode)
            if min_blocks:
                monkeypatch.setenv("AFMIB_RR_MIN_BLOCKS", min_blocks)
            else:
                monkeypatch.delenv("AFMIB_RR_MIN_BLOCKS", raising=False)
            with capi.Solver(nx, ny, nz, n=nx, bc=bc, precision=capi.MIXED, tol=1e-10) as sv:
                out[(mode, min_blocks)] = sv.mg_solve(b)
        ref = out[("0", None)]
        for key, (x, cycles) in out.items():
            assert cycles == ref[1] and np.array_equal(x, ref[0]), (shape, key)
    monkeypatch.delenv("AFMIB_RR_MIN_BLOCKS", raising=False)
    g, u, v, w, X, nstart, nidx = _periodic_case(128, M=2000, seed=4)
    if bc == capi.BC_CHANNEL:
        v = v[: g.nx * (g.ny - 1) * g.nz]
    res = {}
    for mode in ("0", "2"):
        monkeypatch.setenv("AFMIB_RESID_RESTRICT", mode)
        with capi.Solver(128, bc=bc, precision=capi.MIXED, mu=0.01, dt=1e-3, tol=1e-10, k_spring=0.5) as sv:
            sv.set_velocity(u, v, w)
            sv.project()
            sv.set_markers(X, nstart, nidx)
            sv.ib_step(2)
            res[mode] = (*sv.get_velocity(), sv.get_pressure(), sv.get_markers())
    for a, c in zip(res["0"], res["2"]):
        assert np.array_equal(a, c)


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
def test_sweep_from_zero_keeps_bits(monkeypatch, bc):
    """Mixed form: each block of FP32 inner V-cycles starts its correction
    with a red colour that assumes x = 0 and writes both colours
    (k_rbgs_z2b_init) instead of clearing x and running the red colour
    (AFMIB_INIT_SWEEP=0): the same bits in multigrid solves at 256^3 and 128^3
    and in IB steps at 64^3."""
    for n in (256, 128):
        g = po.Grid(n, n, n, n, channel=bc == capi.BC_CHANNEL)
        b = np.random.default_rng(8).standard_normal(g.ncell)
        out = {}
        for mode in ("0", "1"):
            monkeypatch.setenv("AFMIB_INIT_SWEEP", mode)
            with capi.Solver(n, bc=bc, precision=capi.MIXED, tol=1e-10) as sv:
                out[mode] = sv.mg_solve(b)
        assert out["0"][1] == out["1"][1] and np.array_equal(out["0"][0], out["1"][0]), n
    g, u, v, w, X, nstart, nidx = _periodic_case(64, M=800, seed=9)
    if bc == capi.BC_CHANNEL:
        v = v[: g.nx * (g.ny - 1) * g.nz]
    res = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("AFMIB_INIT_SWEEP", mode)
        with capi.Solver(64, bc=bc, precision=capi.MIXED, mu=0.01, dt=1e-3, tol=1e-10, k_spring=0.5) as sv:
            sv.set_velocity(u, v, w)
            sv.project()
            sv.set_markers(X, nstart, nidx)
            sv.ib_step(2)
            res[mode] = (*sv.get_velocity(), sv.get_pressure(), sv.get_markers())
    for a, c in zip(res["0"], res["1"]):
        assert np.array_equal(a, c)


@pytest.mark.parametrize("precision,bar", [(capi.FP64, TOL), (capi.MIXED, 1e-8)])
def test_ns_substeps_moving_walls(golden, precision, bar):
    """Four channel sub-steps with seeded nonzero wall velocities (ut, ub, wt,
    wb: the wall terms of the Helmholtz right-hand sides and the reference's
    wall update, src/ns/helmholtz.h:177-196, src/ns/projection.h:75-122)
    against the compiled reference: fields, pressure and updated walls."""
    d = golden("ns_walls_16")
    n, nxz = 16, 16 * 16
    w0 = d["walls0"]
    with capi.Solver(n, bc=capi.BC_CHANNEL, precision=precision, mu=float(d["mu"]), rho=float(d["rho"]),
                     dt=float(d["dt"]), tol=float(d["tol"])) as sv:
        sv.set_velocity(d["u0"], d["v0"], d["w0"])
        sv.set_walls(w0[:nxz], w0[nxz:2 * nxz], w0[2 * nxz:3 * nxz], w0[3 * nxz:])
        sv.project()
        for _ in range(int(d["substeps"])):
            sv.ns_step(d["fx"], d["fy"], d["fz"])
        u, v, w = sv.get_velocity()
        p = sv.get_pressure()
        walls = np.concatenate(sv.get_walls())
    assert rel(u, d["u"]) < bar and rel(v, d["v"]) < bar and rel(w, d["w"]) < bar
    g = po.Grid(n, n, n, n, channel=True)
    # the mixed form's pressure is bounded at 1e-6, as in the other mixed
    # tests (it carries the FP32 rounding of the provisional velocity's
    # small divergent part)
    pbar = bar if precision == capi.FP64 else 1e-6
    assert pressure_rel(p, d["p"], g, float(d["mu"]), float(d["rho"]), float(d["dt"])) < pbar
    assert rel(walls, d["walls"]) < bar


@pytest.mark.parametrize("precision,bar", [(capi.FP64, TOL), (capi.MIXED, 1e-8)])
def test_ib_steps_moving_walls(golden, precision, bar):
    """Two channel IB steps of a 320-marker shell with moving walls against the
    compiled reference (fields, markers, walls)."""
    d = golden("ib_walls_16")
    n, nxz = 16, 16 * 16
    w0 = d["walls0"]
    with capi.Solver(n, bc=capi.BC_CHANNEL, precision=precision, mu=float(d["mu"]), rho=float(d["rho"]),
                     dt=float(d["dt"]), tol=float(d["tol"]), k_spring=float(d["k"])) as sv:
        sv.set_velocity(d["u0"], d["v0"], d["w0"])
        sv.set_walls(w0[:nxz], w0[nxz:2 * nxz], w0[2 * nxz:3 * nxz], w0[3 * nxz:])
        sv.project()
        sv.set_markers(d["X"], d["nstart"], d["nidx"])
        sv.ib_step(int(d["steps"]))
        u, v, w = sv.get_velocity()
        X = sv.get_markers()
        walls = np.concatenate(sv.get_walls())
    assert rel(u, d["u"]) < bar and rel(v, d["v"]) < bar and rel(w, d["w"]) < bar
    assert rel(X - d["X"], d["Xout"] - d["X"]) < bar
    assert rel(walls, d["walls"]) < bar


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
def test_double_float_first_residuals_match_fp64(monkeypatch, golden, bc):
    """The mixed form's first viscous residuals (the BE pass with Q(uold), the
    CN residual from Q) in double-float on the FP32 pipe against the FP64
    passes: two IB steps (the channel with moving walls) agree to 1e-10; the
    two differ by a few units of 2^-46 of the residuals' terms, so only the
    solves' stopping tests can tell them apart."""
    g, u, v, w, X, nstart, nidx = _periodic_case(32, M=800, seed=17)
    walls = None
    if bc == capi.BC_CHANNEL:
        v = v[: g.nx * (g.ny - 1) * g.nz]
        walls = np.random.default_rng(4).standard_normal(4 * 32 * 32) * 0.05
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("AFMIB_FIRST_DF", mode)
        with capi.Solver(32, bc=bc, precision=capi.MIXED, mu=0.01, dt=1e-3, tol=1e-12, k_spring=0.5) as sv:
            sv.set_velocity(u, v, w)
            if walls is not None:
                sv.set_walls(*np.split(walls, 4))
            sv.project()
            sv.set_markers(X, nstart, nidx)
            sv.ib_step(2)
            out[mode] = (sv.get_velocity(), sv.get_markers())
    for a, b in zip(out["1"][0], out["0"][0]):
        assert rel(a, b) < 1e-10
    assert rel(out["1"][1] - X, out["0"][1] - X) < 1e-10


@pytest.mark.parametrize("bc", [capi.BC_PERIODIC, capi.BC_CHANNEL])
def test_pair_smoother_keeps_bits(monkeypatch, bc):
    """The FP32 red-black colour on float pairs (k_rbgs_pair: the z
    neighbours from the thread's own column registers, the x neighbour across
    the pair boundary by a shuffle) performs the scalar kernel's arithmetic in
    the same order: mixed multigrid solves (128^3, 256 x 128 x 64) and mixed
    IB steps (128^3) agree bit for bit."""
    for shape in ((128, 128, 128), (256, 128, 64)):
        nx, ny, nz = shape
        b = np.random.default_rng(8).standard_normal(nx * ny * nz)
        b -= b.mean()
        out = {}
        for mode in ("0", "1"):
            monkeypatch.setenv("AFMIB_RBGS_PAIR", mode)
            with capi.Solver(nx, ny, nz, n=nx, bc=bc, precision=capi.MIXED, tol=1e-10) as sv:
                out[mode] = sv.mg_solve(b)
        assert out["0"][1] == out["1"][1] and np.array_equal(out["0"][0], out["1"][0]), shape
    g, u, v, w, X, nstart, nidx = _periodic_case(128, M=2000, seed=6)
    if bc == capi.BC_CHANNEL:
        v = v[: g.nx * (g.ny - 1) * g.nz]
    res = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("AFMIB_RBGS_PAIR", mode)
        with capi.Solver(128, bc=bc, precision=capi.MIXED, mu=0.01, dt=1e-3, tol=1e-10, k_spring=0.5) as sv:
            sv.set_velocity(u, v, w)
            sv.project()
            sv.set_markers(X, nstart, nidx)
            sv.ib_step(2)
            res[mode] = (*sv.get_velocity(), sv.get_pressure(), sv.get_markers())
    for a, c in zip(res["0"], res["1"]):
        assert np.array_equal(a, c)
