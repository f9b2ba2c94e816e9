"""TEST INFRASTRUCTURE — the checker, never the product.

ctypes access to the CPU restatement (oracle/restated/oracle.cc, built into
oracle/_build/liborc.so) and a runner for the reference driver binaries
(oracle/ref_driver.cc compiled from the reference headers into oracle/_ref/).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.

Array conventions: FP64, x-fastest (i = x + nx*(y + ny*z)); in channel mode v
has nx*(ny-1)*nz entries (interior y faces), in periodic mode nx*ny*nz.
Markers are X[M, 3].
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liborc.so")
REF_DIR = os.path.join(HERE, "_ref")


def _make_default_reference() -> str:
    """The reference source tree named by the oracle's Makefile (REF ?= ...)."""
    try:
        with open(os.path.join(HERE, "Makefile")) as f:
            for line in f:
                if line.startswith("REF ?="):
                    return line.split("?=", 1)[1].strip()
    except OSError:
        pass
    return ""


# AFMIB_REFERENCE overrides the Makefile's default location of the reference sources.
REFERENCE_SRC = os.environ.get("AFMIB_REFERENCE") or _make_default_reference()

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lib = None


def build(force: bool = False) -> str:
    """Compile the restatement with make (gcc, -ffp-contract=off)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
        os.path.join(HERE, "restated", "oracle.cc")
    ):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_ns_create.restype = ctypes.c_void_p
        L.orc_ns_create.argtypes = [_ip, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_int, _dp, _dp, _dp]
        L.orc_ns_destroy.argtypes = [ctypes.c_void_p]
        L.orc_ns_set_walls_corrected.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_ns_set_bending.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.orc_membrane_forces.argtypes = [ctypes.c_long, _dp, _ip, _ip, ctypes.c_double, ctypes.c_double, _dp]
        L.orc_ns_step.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_ns_get.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp]
        L.orc_ns_set.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.orc_ns_counters.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_long),
                                      ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_int)]
        L.orc_ib_step.argtypes = [ctypes.c_void_p, ctypes.c_long, _dp, _ip, _ip, ctypes.c_double, _dp]
        L.orc_spread.argtypes = [_ip, ctypes.c_int, _dp, ctypes.c_long, _dp, _dp, _dp]
        L.orc_interp.argtypes = [_ip, ctypes.c_int, _dp, ctypes.c_long, _dp, _dp]
        L.orc_springs.argtypes = [ctypes.c_long, _dp, _ip, _ip, ctypes.c_double, _dp]
        L.orc_cg.argtypes = [_ip, ctypes.c_int, ctypes.c_double, _dp, _dp, ctypes.c_double, ctypes.c_int, _ip]
        L.orc_mg_solve.argtypes = [_ip, ctypes.c_int, _dp, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, _ip]
        L.orc_helm_apply.argtypes = [_ip, ctypes.c_int, ctypes.c_double, _dp, _dp]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_set_fast_rows.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    """Threads of the oracle's parallel passes; the results do not depend on it."""
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return int(lib().orc_get_threads())


def set_fast_rows(on: bool) -> None:
    """False routes every operator row through the generic row builder."""
    lib().orc_set_fast_rows(1 if on else 0)


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _pi(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


class Grid:
    """Grid of nx x ny x nz cells with n cells per unit length."""

    def __init__(self, nx, ny, nz, n=None, channel=False):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.n = n if n is not None else nx
        self.channel = bool(channel)

    @property
    def dims(self):
        return (ctypes.c_int * 5)(self.nx, self.ny, self.nz, self.n, int(self.channel))

    @property
    def ncell(self):
        return self.nx * self.ny * self.nz

    @property
    def nv(self):
        return self.nx * (self.ny - 1) * self.nz if self.channel else self.ncell

    def sizes(self):
        return (self.ncell, self.nv, self.ncell)

    def levels(self):
        """Coarsening depth down to one cell along the shortest axis (src/mg/solver.h:239-271)."""
        m = min(self.nx, self.ny) if self.nz == 1 else min(self.nx, self.ny, self.nz)
        return int(np.log2(m))


def div(g, u, v, w, top=None, bottom=None):
    d = np.zeros(g.ncell)
    lib().orc_div(g.dims, _p(d), _p(u), _p(v), _p(w), _p(top), _p(bottom))
    return d


def grad(g, p):
    px, py, pz = np.zeros(g.ncell), np.zeros(g.nv), np.zeros(g.ncell)
    lib().orc_grad(g.dims, _p(px), _p(py), _p(pz), _p(p))
    return px, py, pz


def advection(g, u, v, w):
    ua, va, wa = np.zeros(g.ncell), np.zeros(g.nv), np.zeros(g.ncell)
    lib().orc_advection(g.dims, _p(ua), _p(va), _p(wa), _p(u), _p(v), _p(w))
    return ua, va, wa


def lap_apply(g, x):
    y = np.zeros(g.ncell)
    lib().orc_lap_apply(g.dims, _p(y), _p(np.ascontiguousarray(x)))
    return y


def helm_apply(g, comp, s, x):
    y = np.zeros_like(x)
    lib().orc_helm_apply(g.dims, comp, s, _p(y), _p(np.ascontiguousarray(x)))
    return y


def gs_sweep(g, x, b):
    x = x.copy()
    lib().orc_gs_sweep(g.dims, _p(x), _p(b))
    return x


def rb_sweep(g, x, b):
    """One red-black Gauss-Seidel sweep of the pressure Laplacian (red: x+y+z even, first)."""
    x = x.copy()
    lib().orc_rb_sweep(g.dims, _p(x), _p(b))
    return x


def restrict(g, fine):
    c = np.zeros(g.ncell // (4 if g.nz == 1 else 8))
    lib().orc_restrict(g.dims, _p(c), _p(fine))
    return c


def prolong(g, coarse):
    f = np.zeros(g.ncell)
    lib().orc_prolong(g.dims, _p(f), _p(coarse))
    return f


def cg(g, comp, s, x0, b, tol, maxit=10000):
    x = x0.copy()
    it = ctypes.c_int(0)
    st = lib().orc_cg(g.dims, comp, s, _p(x), _p(b), tol, maxit, ctypes.byref(it))
    return x, it.value, st


def mg_solve(g, rhs, tol, nu1=2, nu2=2, maxit=1000, levels=None):
    x = rhs.copy()
    cyc = ctypes.c_int(0)
    lv = g.levels() if levels is None else levels
    st = lib().orc_mg_solve(g.dims, lv, _p(x), tol, nu1, nu2, maxit, ctypes.byref(cyc))
    return x, cyc.value, st


class NSSolver:
    """ns::solver restated (src/ns/solver.h:61-140); projects the initial field on construction."""

    def __init__(self, g, mu, rho, dt, tol, u0, v0, w0, maxit=10000, levels=None, walls_corrected=False):
        self.g = g
        self.dt = dt
        lv = g.levels() if levels is None else levels
        self.h = lib().orc_ns_create(g.dims, lv, mu, rho, dt, tol, maxit,
                                     _p(np.ascontiguousarray(u0, dtype=np.float64)),
                                     _p(np.ascontiguousarray(v0, dtype=np.float64)),
                                     _p(np.ascontiguousarray(w0, dtype=np.float64)))
        nxz = g.nx * g.nz
        self.walls = np.zeros(4 * nxz)
        lib().orc_ns_set_walls_corrected(self.h, 1 if walls_corrected else 0)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_ns_destroy(self.h)
            self.h = None

    def step(self, fx, fy, fz, walls=None):
        w = self.walls if walls is None else walls
        nxz = self.g.nx * self.g.nz
        base = w.ctypes.data
        ptr = [ctypes.cast(base + k * nxz * 8, _dp) for k in range(4)]
        return lib().orc_ns_step(self.h, ptr[0], ptr[1], ptr[2], ptr[3], _p(fx), _p(fy), _p(fz))

    def get(self):
        u, v, w, p = np.zeros(self.g.ncell), np.zeros(self.g.nv), np.zeros(self.g.ncell), np.zeros(self.g.ncell)
        lib().orc_ns_get(self.h, _p(u), _p(v), _p(w), _p(p))
        return u, v, w, p

    def counters(self):
        a, b, c = ctypes.c_long(), ctypes.c_long(), ctypes.c_int()
        lib().orc_ns_counters(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return a.value, b.value, c.value

    def ib_step(self, X, nstart, nidx, k, kb=0.0):
        X = np.ascontiguousarray(X, dtype=np.float64)
        lib().orc_ns_set_bending(self.h, kb)
        st = lib().orc_ib_step(self.h, X.shape[0], _p(X), _pi(nstart), _pi(nidx), k, _p(self.walls))
        return X, st


def spread(g, comp, X, F, vol=None):
    nf = g.nv if comp == 1 else g.ncell
    f = np.zeros(nf)
    X = np.ascontiguousarray(X, dtype=np.float64)
    lib().orc_spread(g.dims, comp, _p(f), X.shape[0], _p(X), _p(np.ascontiguousarray(F)), _p(vol))
    return f


def interp(g, comp, X, u):
    X = np.ascontiguousarray(X, dtype=np.float64)
    U = np.zeros(X.shape[0])
    lib().orc_interp(g.dims, comp, _p(U), X.shape[0], _p(X), _p(np.ascontiguousarray(u)))
    return U


def springs(X, nstart, nidx, k):
    X = np.ascontiguousarray(X, dtype=np.float64)
    M = X.shape[0]
    G = np.zeros(3 * M)
    lib().orc_springs(M, _p(X), _pi(nstart), _pi(nidx), k, _p(G))
    return G.reshape(3, M)


# ---------------------------------------------------------------------------
# reference driver
# ---------------------------------------------------------------------------

def reference_available() -> bool:
    return os.path.isdir(os.path.join(REFERENCE_SRC, "src", "ns"))


def ref_binary(L, M=256, W=1, H=1, D=1) -> str:
    path = os.path.join(REF_DIR, f"ref_L{L}_W{W}H{H}D{D}_M{M}")
    if not os.path.exists(path):
        if not reference_available():
            raise FileNotFoundError("reference sources not present; cannot build " + path)
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"L={L}", f"M={M}", f"W={W}", f"H={H}", f"D={D}",
                        f"REF={REFERENCE_SRC}"], check=True)
    return path


def run_ref(cmd, arrays, L, M=256, W=1, H=1, D=1, timeout=3600):
    """Run one reference-driver command; returns the flat float64 output."""
    exe = ref_binary(L, M, W, H, D)
    flat = np.concatenate([np.atleast_1d(np.asarray(a, dtype=np.float64)).ravel() for a in arrays])
    with tempfile.TemporaryDirectory() as td:
        fi, fo = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        flat.tofile(fi)
        subprocess.run([exe, cmd, fi, fo], check=True, timeout=timeout)
        return np.fromfile(fo, dtype=np.float64)


def membrane_forces(X, nstart, nidx, k, kb):
    """G (3, M): springs k L X plus bending -kb L (L X)."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    M = X.shape[0]
    G = np.zeros(3 * M)
    lib().orc_membrane_forces(M, _p(X), _pi(nstart), _pi(nidx), k, kb, _p(G))
    return G.reshape(3, M)
