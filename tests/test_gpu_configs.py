"""The adjoint and the 512^3 configurations at their full sizes.

* Adjoint (128^3 periodic, 20,480-marker icosphere shell, mu 0.01, dt 5e-5,
  50 IB steps, checkpoints every 10): the gradient of the membrane loss in k
  and the 61,440 initial marker coordinates, from the FP64 and from the
  mixed forward, against central differences (h = 1e-6) of the FP64 forward
  on 16 seeded directions. Bar: 1e-6 relative.
* 512^3 (1,000,000 markers on 40 shells of radius 0.05, mu 0.002, dt 1e-5):
  the mixed form against the FP64 form from the same state (10 IB steps;
  the configuration's 50 are timed by bench.py --case large), and the
  adjoint of the mixed trajectory with checkpoints every 5 steps, whose
  dL/dk is checked against a central difference of the mixed forward.

Inputs are the seeded generators of the benchmark (afmibins_gb300.markers).
"""
import numpy as np
import pytest

from afmibins_gb300 import capi, markers as mk

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_adjoint_configuration_128_finite_differences():
    from afmibins_gb300.autograd import ib_trajectory, membrane_loss
    n, steps, every = 128, 50, 10
    dev = torch.device("cuda")
    X, nstart, nidx = mk.icoshell(5, (0.5, 0.5, 0.5), 0.2, 0.02)
    vel = mk.random_solenoidal_velocity(n, n, n, rms=0.1, k_peak=4.0, seed=mk.SEED + 4)
    h3 = 1.0 / n ** 3

    def solver(prec):
        sv = capi.Solver(n, mu=0.01, rho=1.0, dt=5e-5, tol=1e-12, k_spring=0.5, precision=prec, max_cg_iters=5000,
                         max_mg_cycles=500)
        sv.set_velocity(*vel)
        sv.project()
        v0 = tuple(torch.from_numpy(a).to(dev) for a in sv.get_velocity())
        sv.set_markers(X, nstart, nidx)
        return sv, v0

    fd_sv, vel0 = solver(capi.FP64)
    grads = {}
    for name, prec in (("fp64", capi.FP64), ("mixed", capi.MIXED)):
        sv, v0 = (fd_sv, vel0) if prec == capi.FP64 else solver(prec)
        X0 = torch.tensor(X, device=dev, requires_grad=True)
        k = torch.tensor(0.5, dtype=torch.float64, device=dev, requires_grad=True)
        uN, XN = ib_trajectory(k, X0, sv, v0, steps, every)
        membrane_loss(uN, XN, X0, h3).backward()
        grads[name] = (float(k.grad), X0.grad.cpu().numpy())
        if prec != capi.FP64:
            sv.close()

    def loss(kv, Xv):
        with torch.no_grad():
            Xt = torch.tensor(Xv, device=dev)
            uN, XN = ib_trajectory(torch.tensor(kv, dtype=torch.float64, device=dev), Xt, fd_sv, vel0, steps, every)
            return float(membrane_loss(uN, XN, Xt, h3))

    rng = np.random.default_rng(17)
    h = 1e-6
    worst = {"fp64": 0.0, "mixed": 0.0}
    for _ in range(16):
        dX = rng.standard_normal(X.shape)
        dX /= np.linalg.norm(dX)
        dk = rng.standard_normal()
        fd = (loss(0.5 + h * dk, X + h * dX) - loss(0.5 - h * dk, X - h * dX)) / (2 * h)
        for name, (gk, gX) in grads.items():
            ad = gk * dk + float((gX * dX).sum())
            worst[name] = max(worst[name], abs(fd - ad) / max(abs(fd), 1e-30))
    fd_sv.close()
    assert worst["fp64"] < 1e-6 and worst["mixed"] < 1e-6, worst


def test_large_configuration_512_mixed_and_adjoint():
    from afmibins_gb300.autograd import ib_trajectory, membrane_loss
    n, steps = 512, 10
    dev = torch.device("cuda")
    X, nstart, nidx = mk.multi_shell(40, 25000, 0.05, 0.12, 0.01, seed=mk.SEED + 5)
    vel = mk.random_solenoidal_velocity(n, n, n, rms=0.1, k_peak=4.0, seed=mk.SEED + 5)
    ends = {}
    for name, prec in (("fp64", capi.FP64), ("mixed", capi.MIXED)):
        with capi.Solver(n, mu=0.002, rho=1.0, dt=1e-5, tol=1e-10, k_spring=0.5, precision=prec) as sv:
            sv.set_velocity(*vel)
            sv.project()
            sv.set_markers(X, nstart, nidx)
            sv.ib_step(steps)
            ends[name] = (sv.get_velocity(), sv.get_markers())
    (um, Xm), (uf, Xf) = ends["mixed"], ends["fp64"]
    assert max(_rel(a, b) for a, b in zip(um, uf)) < 1e-8
    assert _rel(Xm - X, Xf - X) < 1e-8
    del ends, um, uf
    with capi.Solver(n, mu=0.002, rho=1.0, dt=1e-5, tol=1e-10, k_spring=0.5, precision=capi.MIXED) as sv:
        sv.set_velocity(*vel)
        sv.project()
        v0 = tuple(torch.from_numpy(a).to(dev) for a in sv.get_velocity())
        sv.set_markers(X, nstart, nidx)
        X0 = torch.tensor(X, device=dev, requires_grad=True)
        k = torch.tensor(0.5, dtype=torch.float64, device=dev, requires_grad=True)
        uN, XN = ib_trajectory(k, X0, sv, v0, steps, 5)
        membrane_loss(uN, XN, X0, 1.0 / n ** 3).backward()
        gk = float(k.grad)
        assert np.isfinite(gk) and bool(torch.isfinite(X0.grad).all())

        def loss(kv):
            with torch.no_grad():
                Xt = torch.tensor(X, device=dev)
                u_, X_ = ib_trajectory(torch.tensor(kv, dtype=torch.float64, device=dev), Xt, sv, v0, steps, 5)
                return float(membrane_loss(u_, X_, Xt, 1.0 / n ** 3))

        h = 1e-4
        fd = (loss(0.5 + h) - loss(0.5 - h)) / (2 * h)
    assert abs(fd - gk) <= 1e-5 * abs(fd), (fd, gk)
