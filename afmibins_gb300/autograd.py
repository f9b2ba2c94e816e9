"""torch.autograd.Function over the C ABI's trajectory and adjoint entry points.

This is the only PyTorch code of the package: a thin wrapper that lets a
torch loss on the final state of an immersed-boundary run be differentiated
with respect to the membrane stiffness k and the initial marker positions X0.
The forward pass runs `nsteps` IB steps on the GPU (afmib_trajectory_forward,
state checkpointed every `every` steps); the backward pass is the hand-written
adjoint (afmib_trajectory_adjoint), which recomputes each segment from its
checkpoint. The initial velocity is an input constant.

The solver runs on its own CUDA stream, which does not wait for torch's: the
tensors handed to it (X0, the cotangents, the gradient buffer torch fills
with zeros) are produced by torch kernels that may still be running, so each
pass synchronises torch's current stream before it calls the C ABI. The C ABI
calls return once their results are written.

A solver keeps the checkpoints of its latest forward pass only: each forward
pass stamps the solver and its autograd node with a trajectory number, and a
backward pass whose number is no longer the solver's raises instead of
returning the gradient of a different trajectory.
"""
from __future__ import annotations

import torch

from . import capi


def _torch_done(dev):
    """Wait for the work torch has queued on its current stream of `dev`."""
    if dev.type == "cuda":
        torch.cuda.current_stream(dev).synchronize()


class IBTrajectory(torch.autograd.Function):
    @staticmethod
    def forward(ctx, k, X0, solver, vel0, nsteps, every):
        dev = X0.device
        X0c = X0.detach().to(torch.float64).contiguous()
        _torch_done(dev)
        solver.set_spring(float(k))
        solver.set_velocity(*vel0)
        solver.set_marker_positions(X0c)
        solver.trajectory_forward(int(nsteps), int(every))
        solver._trajectory_id = getattr(solver, "_trajectory_id", 0) + 1
        ctx.trajectory_id = solver._trajectory_id
        n = solver.ncell
        uN = torch.empty((3, n), dtype=torch.float64, device=dev)
        solver.get_velocity((uN[0], uN[1], uN[2]))
        XN = torch.empty((solver.M, 3), dtype=torch.float64, device=dev)
        solver.get_markers(XN)
        ctx.solver = solver
        ctx.k_dtype = k.dtype if torch.is_tensor(k) else torch.float64
        return uN, XN

    @staticmethod
    def backward(ctx, g_u, g_X):
        s = ctx.solver
        if getattr(s, "_trajectory_id", None) != ctx.trajectory_id:
            raise RuntimeError("the solver ran another forward trajectory since this one; its checkpoints are gone "
                               "(run backward before the next forward on the same solver, or use two solvers)")
        dev = g_X.device if g_X is not None else g_u.device
        lam_u = g_u.contiguous() if g_u is not None else None
        lam_X = g_X.contiguous() if g_X is not None else None
        gX0 = torch.zeros((s.M, 3), dtype=torch.float64, device=dev)
        _torch_done(dev)  # the cotangents and the zeroed buffer are written before the solver reads them
        _, gk, _ = s.trajectory_adjoint(lam_u[0] if lam_u is not None else None,
                                        lam_u[1] if lam_u is not None else None,
                                        lam_u[2] if lam_u is not None else None,
                                        lam_X, out_X=gX0)
        return torch.tensor(gk, dtype=ctx.k_dtype, device=dev), gX0, None, None, None, None


def ib_trajectory(k, X0, solver: capi.Solver, vel0, nsteps: int, every: int):
    """Final (velocity [3, N], markers [M, 3]) after `nsteps` IB steps, differentiable in k and X0."""
    return IBTrajectory.apply(k, X0, solver, vel0, nsteps, every)


def membrane_loss(uN, XN, X0, h3):
    """Sum of squared marker displacements from the initial centroid-relative
    shape plus half the kinetic energy of the final velocity."""
    e = (XN - XN.mean(0)) - (X0 - X0.mean(0))
    return (e * e).sum() + 0.5 * h3 * (uN * uN).sum()
