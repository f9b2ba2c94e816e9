"""ctypes binding of the afmib C ABI (include/afmib.h).

This is the Python-side caller of the same entry points a C or C++ caller
links against. Arrays may be numpy (host) or torch CUDA tensors (device):
only their data pointers cross the boundary. The library must have been
built (afmibins_gb300.build); there is no fallback — a missing library raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

AFMIB_OK = 0
AFMIB_ERR_ARG = 1
AFMIB_ERR_CUDA = 2
AFMIB_ERR_NOCONV = 3
AFMIB_ERR_BOUNDS = 4
AFMIB_ERR_NAN = 5
AFMIB_ERR_STATE = 6
AFMIB_ERR_CAPACITY = 7

BC_PERIODIC = 0
BC_CHANNEL = 1
FP64 = 0
MIXED = 1
START_DEFAULT = 0
START_ZERO = 1
START_WARM = 2


class AfmibError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"afmib status {status}: {msg}")
        self.status = status


class Config(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("n", ctypes.c_int),
                ("bc", ctypes.c_int), ("precision", ctypes.c_int), ("mg_levels", ctypes.c_int),
                ("nu1", ctypes.c_int), ("nu2", ctypes.c_int), ("mu", ctypes.c_double), ("rho", ctypes.c_double),
                ("dt", ctypes.c_double), ("tol", ctypes.c_double), ("max_cg_iters", ctypes.c_int),
                ("max_mg_cycles", ctypes.c_int), ("k_spring", ctypes.c_double), ("inner_tol", ctypes.c_double),
                ("ib_fp32", ctypes.c_int), ("proj_start", ctypes.c_int), ("walls_corrected", ctypes.c_int),
                ("k_bend", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [("substeps", ctypes.c_longlong), ("ib_steps", ctypes.c_longlong), ("cg_iters", ctypes.c_longlong),
                ("mg_cycles", ctypes.c_longlong), ("outer_iters", ctypes.c_longlong),
                ("last_mg_rms", ctypes.c_double), ("last_cg_norm", ctypes.c_double), ("half", ctypes.c_int),
                ("spread_tiles", ctypes.c_int), ("kernel_launches", ctypes.c_longlong)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_vp = ctypes.c_void_p
_SIGS = {
    "afmib_create": ([ctypes.POINTER(Config), _vp, ctypes.POINTER(_vp)], ctypes.c_int),
    "afmib_destroy": ([_vp], ctypes.c_int),
    "afmib_error_string": ([ctypes.c_int], ctypes.c_char_p),
    "afmib_last_error": ([_vp], ctypes.c_char_p),
    "afmib_get_stats": ([_vp, ctypes.POINTER(Stats)], ctypes.c_int),
    "afmib_synchronize": ([_vp], ctypes.c_int),
    "afmib_set_velocity": ([_vp, _vp, _vp, _vp], ctypes.c_int),
    "afmib_get_velocity": ([_vp, _vp, _vp, _vp], ctypes.c_int),
    "afmib_get_pressure": ([_vp, _vp], ctypes.c_int),
    "afmib_set_walls": ([_vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "afmib_get_walls": ([_vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "afmib_project": ([_vp], ctypes.c_int),
    "afmib_ns_step": ([_vp, _vp, _vp, _vp], ctypes.c_int),
    "afmib_set_markers": ([_vp, ctypes.c_int, _vp, _vp, _vp, _vp], ctypes.c_int),
    "afmib_get_markers": ([_vp, _vp], ctypes.c_int),
    "afmib_save": ([_vp, ctypes.c_char_p], ctypes.c_int),
    "afmib_reset_warm_start": ([_vp], ctypes.c_int),
    "afmib_load": ([_vp, ctypes.c_char_p], ctypes.c_int),
    "afmib_set_marker_positions": ([_vp, _vp], ctypes.c_int),
    "afmib_ib_step": ([_vp, ctypes.c_int], ctypes.c_int),
    "afmib_div": ([_vp, _vp, _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "afmib_grad": ([_vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "afmib_advection": ([_vp, _vp, _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "afmib_mg_solve": ([_vp, _vp, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "afmib_lap_apply": ([_vp, _vp, _vp], ctypes.c_int),
    "afmib_helm_apply": ([_vp, ctypes.c_int, ctypes.c_double, _vp, _vp], ctypes.c_int),
    "afmib_helmholtz_cg": ([_vp, ctypes.c_int, ctypes.c_double, _vp, _vp, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "afmib_restrict": ([_vp, _vp, _vp], ctypes.c_int),
    "afmib_prolong": ([_vp, _vp, _vp], ctypes.c_int),
    "afmib_spread": ([_vp, ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "afmib_interp": ([_vp, ctypes.c_int, _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "afmib_set_spring": ([_vp, ctypes.c_double], ctypes.c_int),
    "afmib_set_bending": ([_vp, ctypes.c_double], ctypes.c_int),
    "afmib_set_tolerance": ([_vp, ctypes.c_double], ctypes.c_int),
    "afmib_smooth": ([_vp, _vp, _vp], ctypes.c_int),
    "afmib_helmholtz_cg_noalloc": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_int, _vp, _vp,
                                    ctypes.POINTER(ctypes.c_int), _vp], ctypes.c_int),
    "afmib_trajectory_forward": ([_vp, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "afmib_trajectory_adjoint": ([_vp, _vp, _vp, _vp, _vp, _vp, ctypes.POINTER(ctypes.c_double), _vp, _vp, _vp],
                                 ctypes.c_int),
    "afmib_profile_enable": ([_vp, ctypes.c_int], ctypes.c_int),
    "afmib_profile_reset": ([_vp], ctypes.c_int),
    "afmib_profile_count": ([_vp], ctypes.c_int),
    "afmib_profile_get": ([_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_longlong),
                           ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
}

_lib = None


def library_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load libafmib.so (building it first if requested). Raises if unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise FileNotFoundError(f"{path} missing: run `python -m afmibins_gb300.build`")
        _build.build()
    L = ctypes.CDLL(path)
    for name, (args, res) in _SIGS.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def ptr(a):
    """Data pointer of a numpy array or torch tensor (None passes through)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags.c_contiguous:
            raise ValueError("array must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return a.data_ptr()
    if isinstance(a, int):
        return a
    raise TypeError(f"unsupported buffer type {type(a)}")


def _f64(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return np.ascontiguousarray(a, dtype=np.float64)
    return a


def _i32(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return np.ascontiguousarray(a, dtype=np.int32)
    return a


class Solver:
    """One device-resident simulation behind the C ABI."""

    def __init__(self, nx, ny=None, nz=None, *, n=None, bc=BC_PERIODIC, precision=FP64, mu=0.01, rho=1.0, dt=1e-4,
                 tol=1e-10, mg_levels=0, nu1=2, nu2=2, max_cg_iters=1000, max_mg_cycles=200, k_spring=0.0,
                 inner_tol=0.0, ib_fp32=0, proj_start=0, walls_corrected=0, k_bend=0.0, stream=None):
        self.lib = load()
        ny = nx if ny is None else ny
        nz = nx if nz is None else nz
        self.cfg = Config(nx, ny, nz, n or nx, bc, precision, mg_levels, nu1, nu2, mu, rho, dt, tol, max_cg_iters,
                          max_mg_cycles, k_spring, inner_tol, ib_fp32, proj_start, walls_corrected, k_bend)
        self.nx, self.ny, self.nz = nx, ny, nz
        self.channel = bc == BC_CHANNEL
        h = _vp()
        st = self.lib.afmib_create(ctypes.byref(self.cfg), stream, ctypes.byref(h))
        self.h = h
        if st != AFMIB_OK:
            msg = self.last_error()
            self.lib.afmib_destroy(self.h)
            self.h = None
            raise AfmibError(st, msg)

    # sizes
    @property
    def ncell(self):
        return self.nx * self.ny * self.nz

    @property
    def nv(self):
        return self.nx * (self.ny - 1) * self.nz if self.channel else self.ncell

    def last_error(self):
        return (self.lib.afmib_last_error(self.h) or b"").decode()

    def _ck(self, st):
        if st != AFMIB_OK:
            raise AfmibError(st, self.last_error())
        return st

    def close(self):
        if getattr(self, "h", None):
            self.lib.afmib_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def stats(self):
        s = Stats()
        self._ck(self.lib.afmib_get_stats(self.h, ctypes.byref(s)))
        return s.as_dict()

    def synchronize(self):
        self._ck(self.lib.afmib_synchronize(self.h))

    # state
    def set_velocity(self, u, v, w):
        u, v, w = _f64(u), _f64(v), _f64(w)
        self._ck(self.lib.afmib_set_velocity(self.h, ptr(u), ptr(v), ptr(w)))

    def get_velocity(self, out=None):
        if out is None:
            out = (np.zeros(self.ncell), np.zeros(self.nv), np.zeros(self.ncell))
        self._ck(self.lib.afmib_get_velocity(self.h, *(ptr(a) for a in out)))
        return out

    def get_pressure(self, out=None):
        p = np.zeros(self.ncell) if out is None else out
        self._ck(self.lib.afmib_get_pressure(self.h, ptr(p)))
        return p

    def set_walls(self, ut=None, ub=None, wt=None, wb=None):
        self._ck(self.lib.afmib_set_walls(self.h, *(ptr(_f64(a)) for a in (ut, ub, wt, wb))))

    def get_walls(self):
        n = self.nx * self.nz
        out = [np.zeros(n) for _ in range(4)]
        self._ck(self.lib.afmib_get_walls(self.h, *(ptr(a) for a in out)))
        return out

    def project(self):
        self._ck(self.lib.afmib_project(self.h))

    def ns_step(self, fx=None, fy=None, fz=None):
        fx, fy, fz = _f64(fx), _f64(fy), _f64(fz)
        self._ck(self.lib.afmib_ns_step(self.h, ptr(fx), ptr(fy), ptr(fz)))

    def set_markers(self, X, nstart=None, nidx=None, vol=None):
        X = _f64(X)
        M = X.shape[0] if hasattr(X, "shape") and len(X.shape) == 2 else len(X) // 3
        self._ck(self.lib.afmib_set_markers(self.h, M, ptr(X), ptr(_i32(nstart)), ptr(_i32(nidx)), ptr(_f64(vol))))
        self.M = M

    def set_marker_positions(self, X):
        self._ck(self.lib.afmib_set_marker_positions(self.h, ptr(_f64(X))))

    def get_markers(self, out=None):
        X = np.zeros((self.M, 3)) if out is None else out
        self._ck(self.lib.afmib_get_markers(self.h, ptr(X)))
        return X

    def ib_step(self, nsteps=1):
        self._ck(self.lib.afmib_ib_step(self.h, nsteps))

    # snapshots (afmibins_gb300/snapshot.py reads the files without a GPU)
    def reset_warm_start(self):
        self._ck(self.lib.afmib_reset_warm_start(self.h))

    def save(self, path):
        self._ck(self.lib.afmib_save(self.h, os.fsencode(path)))

    def load(self, path):
        from . import snapshot
        self._ck(self.lib.afmib_load(self.h, os.fsencode(path)))
        counts = snapshot.sections(path)
        self.M = counts["X"][1] // 3 if "X" in counts else 0

    # adjoint
    def set_spring(self, k):
        self._ck(self.lib.afmib_set_spring(self.h, float(k)))

    def set_bending(self, kb):
        self._ck(self.lib.afmib_set_bending(self.h, float(kb)))

    def trajectory_forward(self, nsteps, ckpt_every):
        self._ck(self.lib.afmib_trajectory_forward(self.h, nsteps, ckpt_every))

    def trajectory_adjoint(self, lam_u=None, lam_v=None, lam_w=None, lam_X=None, want_u0=False, out_X=None):
        """Gradients (dX0 [M,3], dk, (du0, dv0, dw0) or None) of a loss with the given final-state adjoints."""
        gX = np.zeros((self.M, 3)) if out_X is None else out_X
        gk = ctypes.c_double(0.0)
        gu = [np.zeros(self.ncell) for _ in range(3)] if want_u0 else [None] * 3
        self._ck(self.lib.afmib_trajectory_adjoint(self.h, ptr(_f64(lam_u)), ptr(_f64(lam_v)), ptr(_f64(lam_w)),
                                                   ptr(_f64(lam_X)), ptr(gX), ctypes.byref(gk),
                                                   *(ptr(a) for a in gu)))
        return gX, gk.value, (gu if want_u0 else None)

    # per-kernel timing
    def profile(self, on=True):
        self._ck(self.lib.afmib_profile_enable(self.h, 1 if on else 0))

    def profile_reset(self):
        self._ck(self.lib.afmib_profile_reset(self.h))

    def profile_table(self):
        """{kernel: (launches, total_ms, algorithmic_bytes)} since the last reset."""
        out = {}
        for i in range(self.lib.afmib_profile_count(self.h)):
            name, n, ms, by = ctypes.c_char_p(), ctypes.c_longlong(), ctypes.c_double(), ctypes.c_double()
            self._ck(self.lib.afmib_profile_get(self.h, i, ctypes.byref(name), ctypes.byref(n), ctypes.byref(ms),
                                                ctypes.byref(by)))
            if n.value:
                out[name.value.decode()] = (n.value, ms.value, by.value)
        return out

    # single operators
    def div(self, u, v, w, top=None, bottom=None):
        d = np.zeros(self.ncell)
        self._ck(self.lib.afmib_div(self.h, ptr(d), ptr(_f64(u)), ptr(_f64(v)), ptr(_f64(w)), ptr(_f64(top)),
                                    ptr(_f64(bottom))))
        return d

    def grad(self, p):
        px, py, pz = np.zeros(self.ncell), np.zeros(self.nv), np.zeros(self.ncell)
        self._ck(self.lib.afmib_grad(self.h, ptr(px), ptr(py), ptr(pz), ptr(_f64(p))))
        return px, py, pz

    def advection(self, u, v, w):
        ua, va, wa = np.zeros(self.ncell), np.zeros(self.nv), np.zeros(self.ncell)
        self._ck(self.lib.afmib_advection(self.h, ptr(ua), ptr(va), ptr(wa), ptr(_f64(u)), ptr(_f64(v)), ptr(_f64(w))))
        return ua, va, wa

    def mg_solve(self, rhs):
        x = np.array(rhs, dtype=np.float64, copy=True)
        c = ctypes.c_int(0)
        self._ck(self.lib.afmib_mg_solve(self.h, ptr(x), ctypes.byref(c)))
        return x, c.value

    def smooth(self, x, b):
        """One red-black Gauss-Seidel sweep on L x = b (alg::smooth)."""
        x = np.array(x, dtype=np.float64, copy=True)
        self._ck(self.lib.afmib_smooth(self.h, ptr(x), ptr(_f64(b))))
        return x

    def mg_solve_device(self, x):
        """mg_solve in place on a device (or host) array; returns (x, cycles)."""
        c = ctypes.c_int(0)
        self._ck(self.lib.afmib_mg_solve(self.h, ptr(x), ctypes.byref(c)))
        return x, c.value

    def lap_apply(self, x):
        y = np.zeros(self.ncell)
        self._ck(self.lib.afmib_lap_apply(self.h, ptr(y), ptr(_f64(x))))
        return y

    def helm_apply(self, comp, scale, x):
        x = _f64(x)
        y = np.zeros_like(x)
        self._ck(self.lib.afmib_helm_apply(self.h, comp, scale, ptr(y), ptr(x)))
        return y

    def helmholtz_cg(self, comp, scale, x0, b):
        x = np.array(x0, dtype=np.float64, copy=True)
        it = ctypes.c_int(0)
        self._ck(self.lib.afmib_helmholtz_cg(self.h, comp, scale, ptr(x), ptr(_f64(b)), ctypes.byref(it)))
        return x, it.value

    def restrict(self, fine):
        c = np.zeros(self.ncell // (4 if self.nz == 1 else 8))
        self._ck(self.lib.afmib_restrict(self.h, ptr(c), ptr(_f64(fine))))
        return c

    def prolong(self, coarse):
        f = np.zeros(self.ncell)
        self._ck(self.lib.afmib_prolong(self.h, ptr(f), ptr(_f64(coarse))))
        return f

    def spread(self, X, F, vol=None):
        X = _f64(X)
        M = X.shape[0]
        fx, fy, fz = np.zeros(self.ncell), np.zeros(self.nv), np.zeros(self.ncell)
        self._ck(self.lib.afmib_spread(self.h, M, ptr(X), ptr(_f64(F)), ptr(_f64(vol)), ptr(fx), ptr(fy), ptr(fz)))
        return fx, fy, fz

    def interp(self, X, u, v, w):
        X = _f64(X)
        M = X.shape[0]
        U = np.zeros((3, M))
        self._ck(self.lib.afmib_interp(self.h, M, ptr(X), ptr(_f64(u)), ptr(_f64(v)), ptr(_f64(w)), ptr(U)))
        return U


def declared_symbols(header=None):
    """Entry points declared in include/afmib.h."""
    import re
    header = header or os.path.join(_build.INCLUDE, "afmib.h")
    text = open(header).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(afmib_\w+)\s*\(", text, re.M)))
