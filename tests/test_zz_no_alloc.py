"""afmib_helmholtz_cg_noalloc — the Helmholtz CG entry point that allocates
nothing — against the solver-based afmib_helmholtz_cg, through the C ABI.

The no-allocation variant is for callers that may not call cudaMalloc where
they solve (memory pools or arenas that own the process's allocations, strict
memory budgets, inner loops that cannot take an allocation's synchronisation):
it keeps its working vectors in an array the library reserves on the GPU. The
test allocates its own x and b (the caller's buffers), calls the entry point
twice in a row on the same inputs, and compares with the solver path at the
tolerance of the other CG tests (1e-10 relative; both use the same kernels and
deterministic reductions, so they agree to round-off)."""
import ctypes

import numpy as np
import pytest

from afmibins_gb300 import capi

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _noalloc(lib, n, bc, comp, scale, tol, xd, bd):
    it = ctypes.c_int(-1)
    torch.cuda.synchronize()
    st = lib.afmib_helmholtz_cg_noalloc(n, n, n, n, bc, comp, scale, tol, 1000, xd.data_ptr(), bd.data_ptr(),
                                        ctypes.byref(it), None)
    torch.cuda.synchronize()
    return st, it.value


@pytest.mark.parametrize("bc,comp", [(capi.BC_PERIODIC, 0), (capi.BC_PERIODIC, 1), (capi.BC_CHANNEL, 2)])
def test_noalloc_cg_matches_solver_cg_twice(bc, comp):
    lib = capi.load()
    n, scale, tol = 32, -0.05, 1e-12
    rng = np.random.default_rng(40 + comp)
    b = rng.standard_normal(n ** 3)
    x0 = rng.standard_normal(n ** 3)
    with capi.Solver(n, bc=bc, tol=tol) as sv:
        x_ref, it_ref = sv.helmholtz_cg(comp, scale, x0, b)
    dev = torch.device("cuda")
    bd = torch.tensor(b, dtype=torch.float64, device=dev)
    for _ in range(2):
        xd = torch.tensor(x0, dtype=torch.float64, device=dev)
        st, it = _noalloc(lib, n, bc, comp, scale, tol, xd, bd)
        assert st == capi.AFMIB_OK
        assert it == it_ref
        x = xd.cpu().numpy()
        assert np.max(np.abs(x - x_ref)) <= 1e-10 * np.max(np.abs(x_ref))


def test_noalloc_capacity_edge_allocates_nothing_after_first_call():
    """At the largest grid the array holds (64^3) the solve still matches the
    solver path, and once the first call has loaded the array, later calls
    leave the device's free memory unchanged."""
    lib = capi.load()
    n, scale, tol = 64, -0.05, 1e-12
    rng = np.random.default_rng(64)
    b = rng.standard_normal(n ** 3)
    x0 = np.zeros(n ** 3)
    with capi.Solver(n, tol=tol) as sv:
        x_ref, it_ref = sv.helmholtz_cg(0, scale, x0, b)
    dev = torch.device("cuda")
    bd = torch.tensor(b, dtype=torch.float64, device=dev)
    xs = [torch.zeros(n ** 3, dtype=torch.float64, device=dev) for _ in range(2)]
    st, _ = _noalloc(lib, n, capi.BC_PERIODIC, 0, scale, tol, xs[0], bd)  # warm-up: loads the array
    assert st == capi.AFMIB_OK
    xs[0].zero_()
    for xd in xs:
        free0, _ = torch.cuda.mem_get_info()
        st, it = _noalloc(lib, n, capi.BC_PERIODIC, 0, scale, tol, xd, bd)
        free1, _ = torch.cuda.mem_get_info()
        assert st == capi.AFMIB_OK and it == it_ref
        assert free1 == free0
        x = xd.cpu().numpy()
        assert np.max(np.abs(x - x_ref)) <= 1e-10 * np.max(np.abs(x_ref))


def test_noalloc_rejects_oversize_and_channel_v():
    lib = capi.load()
    dev = torch.device("cuda")
    xd = torch.zeros(8, dtype=torch.float64, device=dev)
    st, _ = _noalloc(lib, 128, capi.BC_PERIODIC, 0, -0.05, 1e-12, xd, xd)
    assert st == capi.AFMIB_ERR_CAPACITY
    st, _ = _noalloc(lib, 16, capi.BC_CHANNEL, 1, -0.05, 1e-12, xd, xd)
    assert st == capi.AFMIB_ERR_ARG
    it = ctypes.c_int(-1)  # a 2D grid (nz = 1) is rejected
    st = lib.afmib_helmholtz_cg_noalloc(16, 16, 1, 16, capi.BC_PERIODIC, 0, -0.05, 1e-12, 100, xd.data_ptr(),
                                        xd.data_ptr(), ctypes.byref(it), None)
    assert st == capi.AFMIB_ERR_ARG
