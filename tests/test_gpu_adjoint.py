"""Adjoint gradient of the IB trajectory (dL/dk, dL/dX0) through the
torch.autograd.Function, checked against central finite differences of the
GPU forward on 16 seeded random directions (h = 1e-6, FP64) and, for dL/dk,
against central differences of the CPU oracle (the FP64 reference gradient).
Bar: 1e-6 relative."""
import numpy as np
import pytest

from afmibins_gb300 import capi, markers as mk

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _case(n=16, M=240, seed=5):
    rng = np.random.default_rng(seed)
    P = mk.fibonacci_sphere(M)
    lists = mk.knn_lists(P, 6)
    X, _ = mk.shell(P, lists, (0.5, 0.5, 0.5), 0.25, 0.02, 0)
    nstart, nidx = mk._csr_from_lists(lists)
    u, v, w = mk.random_solenoidal_velocity(n, n, n, rms=0.05, k_peak=2.0, seed=seed)
    return X, nstart, nidx, (u, v, w)


def _setup(n, X, nstart, nidx, vel, precision=capi.FP64):
    sv = capi.Solver(n, mu=0.01, rho=1.0, dt=2e-3, tol=1e-13, k_spring=0.5, precision=precision, max_cg_iters=2000)
    sv.set_velocity(*vel)
    sv.project()
    u, v, w = sv.get_velocity()
    sv.set_markers(X, nstart, nidx)
    return sv, (u, v, w)


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_adjoint_matches_finite_differences(precision):
    """The adjoint gradient from the FP64 or the mixed-precision forward, against
    central differences of the FP64 forward (FP32 rounding of the mixed forward
    would dominate a 1e-6 difference quotient)."""
    from afmibins_gb300.autograd import ib_trajectory, membrane_loss
    n, nsteps, every = 16, 4, 2
    X, nstart, nidx, vel = _case(n)
    sv, vel0 = _setup(n, X, nstart, nidx, vel, precision)
    fd_sv = sv if precision == capi.FP64 else _setup(n, X, nstart, nidx, vel, capi.FP64)[0]
    dev = torch.device("cuda")
    h3 = 1.0 / n ** 3
    X0 = torch.tensor(X, device=dev, requires_grad=True)
    k = torch.tensor(0.5, dtype=torch.float64, device=dev, requires_grad=True)
    uN, XN = ib_trajectory(k, X0, sv, vel0, nsteps, every)
    L = membrane_loss(uN, XN, X0, h3)
    L.backward()
    gk, gX = float(k.grad), X0.grad.cpu().numpy()

    def loss(kv, Xv):
        with torch.no_grad():
            Xt = torch.tensor(Xv, device=dev)
            uN, XN = ib_trajectory(torch.tensor(kv, dtype=torch.float64), Xt, fd_sv, vel0, nsteps, every)
            return float(membrane_loss(uN, XN, Xt, h3))

    rng = np.random.default_rng(17)
    h = 1e-6
    worst = 0.0
    for _ in range(16):
        dX = rng.standard_normal(X.shape)
        dX /= np.linalg.norm(dX)
        dk = rng.standard_normal()
        fd = (loss(0.5 + h * dk, X + h * dX) - loss(0.5 - h * dk, X - h * dX)) / (2 * h)
        ad = gk * dk + float((gX * dX).sum())
        worst = max(worst, abs(fd - ad) / max(abs(fd), 1e-30))
    sv.close()
    fd_sv.close()
    assert worst < 1e-6, worst


def test_dk_against_oracle_reference():
    from afmibins_gb300.autograd import ib_trajectory, membrane_loss
    from oracle import pyoracle as po
    n, nsteps, every = 16, 3, 3
    X, nstart, nidx, vel = _case(n, M=160, seed=9)
    sv, vel0 = _setup(n, X, nstart, nidx, vel)
    dev = torch.device("cuda")
    h3 = 1.0 / n ** 3
    X0 = torch.tensor(X, device=dev)
    k = torch.tensor(0.5, dtype=torch.float64, device=dev, requires_grad=True)
    uN, XN = ib_trajectory(k, X0, sv, vel0, nsteps, every)
    membrane_loss(uN, XN, X0, h3).backward()
    gk = float(k.grad)
    sv.close()
    g = po.Grid(n, n, n, n, channel=False)

    def oracle_loss(kv):
        s = po.NSSolver(g, 0.01, 1.0, 2e-3, 1e-13, *vel0)
        Xo = X.copy()
        for _ in range(nsteps):
            Xo, st = s.ib_step(Xo, nstart, nidx, kv)
        u, v, w, _ = s.get()
        e = (Xo - Xo.mean(0)) - (X - X.mean(0))
        return float((e * e).sum() + 0.5 * h3 * ((u * u).sum() + (v * v).sum() + (w * w).sum()))

    h = 1e-6
    ref = (oracle_loss(0.5 + h) - oracle_loss(0.5 - h)) / (2 * h)
    assert abs(gk - ref) / abs(ref) < 1e-6, (gk, ref)


def test_adjoint_with_bending_matches_finite_differences():
    """With membrane bending (k_bend = 0.05: force -k_bend L (L X)) the
    adjoint carries the bending term's transpose; the gradient agrees with
    central differences of the forward, 1e-6 relative."""
    from afmibins_gb300.autograd import ib_trajectory, membrane_loss
    n, nsteps, every = 16, 4, 2
    X, nstart, nidx, vel = _case(n, M=200, seed=13)
    sv = capi.Solver(n, mu=0.01, rho=1.0, dt=2e-3, tol=1e-13, k_spring=0.5, k_bend=0.05, max_cg_iters=2000)
    sv.set_velocity(*vel)
    sv.project()
    vel0 = sv.get_velocity()
    sv.set_markers(X, nstart, nidx)
    dev = torch.device("cuda")
    h3 = 1.0 / n ** 3
    X0 = torch.tensor(X, device=dev, requires_grad=True)
    k = torch.tensor(0.5, dtype=torch.float64, device=dev, requires_grad=True)
    uN, XN = ib_trajectory(k, X0, sv, vel0, nsteps, every)
    membrane_loss(uN, XN, X0, h3).backward()
    gk, gX = float(k.grad), X0.grad.cpu().numpy()

    def loss(kv, Xv):
        with torch.no_grad():
            Xt = torch.tensor(Xv, device=dev)
            uN, XN = ib_trajectory(torch.tensor(kv, dtype=torch.float64), Xt, sv, vel0, nsteps, every)
            return float(membrane_loss(uN, XN, Xt, h3))

    rng = np.random.default_rng(19)
    h, worst = 1e-6, 0.0
    for _ in range(8):
        dX = rng.standard_normal(X.shape)
        dX /= np.linalg.norm(dX)
        dk = rng.standard_normal()
        fd = (loss(0.5 + h * dk, X + h * dX) - loss(0.5 - h * dk, X - h * dX)) / (2 * h)
        ad = gk * dk + float((gX * dX).sum())
        worst = max(worst, abs(fd - ad) / max(abs(fd), 1e-30))
    sv.close()
    assert worst < 1e-6, worst


def test_backward_of_a_superseded_trajectory_raises():
    """A solver keeps only its latest forward trajectory's checkpoints: the
    backward pass of an earlier one raises instead of returning the gradient
    of the later trajectory."""
    from afmibins_gb300.autograd import ib_trajectory, membrane_loss
    n = 16
    X, nstart, nidx, vel = _case(n)
    sv, vel0 = _setup(n, X, nstart, nidx, vel)
    dev = torch.device("cuda")
    X0 = torch.tensor(X, device=dev, requires_grad=True)
    k = torch.tensor(0.5, dtype=torch.float64, device=dev, requires_grad=True)
    uN, XN = ib_trajectory(k, X0, sv, vel0, 2, 1)
    L1 = membrane_loss(uN, XN, X0, 1.0 / n ** 3)
    uN2, XN2 = ib_trajectory(k, X0, sv, vel0, 2, 1)
    with pytest.raises(RuntimeError, match="another forward trajectory"):
        L1.backward()
    membrane_loss(uN2, XN2, X0, 1.0 / n ** 3).backward()  # the latest one still differentiates
    assert torch.isfinite(k.grad)
    sv.close()


def test_adjoint_repeats_bit_for_bit():
    """The same trajectory differentiated three times in one process gives the
    same gradients bit for bit: the wrapper waits for torch's kernels (the
    cotangents, the zeroed gradient buffer) before the solver, on its own
    stream, reads them."""
    from afmibins_gb300.autograd import ib_trajectory, membrane_loss
    n = 32
    X, nstart, nidx, vel = _case(n, M=600)
    dev = torch.device("cuda")
    out = []
    for _ in range(3):
        sv, vel0 = _setup(n, X, nstart, nidx, vel, capi.MIXED)
        X0 = torch.tensor(X, device=dev, requires_grad=True)
        k = torch.tensor(0.5, dtype=torch.float64, device=dev, requires_grad=True)
        uN, XN = ib_trajectory(k, X0, sv, vel0, 4, 2)
        membrane_loss(uN, XN, X0, 1.0 / n ** 3).backward()
        out.append((float(k.grad), X0.grad.cpu().numpy()))
        sv.close()
    for gk, gX in out[1:]:
        assert gk == out[0][0] and np.array_equal(gX, out[0][1])
