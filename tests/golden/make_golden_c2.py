"""Digest fixtures of the 128^3 icosphere configuration (FP64, 20,480 markers).

Two fixtures:

* c2_periodic_128_digest.npz — the periodic unit cube of the configuration:
  128^3, mu 0.01, rho 1, dt 5e-5, an icosphere face-centroid shell (level 5:
  20,480 markers, face-adjacency springs, radius 0.2 at the centre, radial
  perturbation 0.02 Y_2^0), k 0.5, a seeded solenoidal initial velocity (RMS
  0.1, spectrum peaked at wavenumber 4), 100 IB steps, solver tolerance
  1e-12. Made by the CPU oracle (the reference has no periodic mode), run on
  all host cores: its threaded passes give the one-thread bits.
* c2_channel_128_ref_digest.npz — the same shell and viscosity in the
  reference's own channel domain (walls in y), 4 IB steps, made by the
  reference compiled unchanged (oracle/_ref, the "ib" command of
  oracle/ref_driver.cc). The shell stays 0.08 from every wall and periodic
  face, clear of the kd-tree's periodic miss and the wall search bound.

Run in a container that has the reference sources (the channel fixture needs
them; default location in oracle/Makefile, override with AFMIB_REFERENCE):

    python tests/golden/make_golden_c2.py [periodic] [channel]

The fields are 16.8 MB each, so a fixture keeps, per field, its sum, sum of
squares, largest magnitude and values at 4096 seeded indices, plus checksums
of the regenerated inputs; marker positions are kept in full.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from afmibins_gb300 import markers as mk  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

N_PROBES = 4096
SEED = mk.SEED + 2
PARAMS = dict(n=128, mu=0.01, rho=1.0, dt=5e-5, k=0.5, tol=1e-12)


def inputs(n=128):
    """Markers (X, nstart, nidx) and the periodic initial velocity (u, v, w)."""
    X, nstart, nidx = mk.icoshell(5, (0.5, 0.5, 0.5), 0.2, 0.02)
    u, v, w = mk.random_solenoidal_velocity(n, n, n, rms=0.1, k_peak=4.0, seed=SEED)
    return X, nstart, nidx, u, v, w


def channel_v(v, n):
    """The periodic v without its y = 0 plane: the reference's interior faces."""
    return np.ascontiguousarray(v.reshape(n, n, n)[:, 1:, :]).ravel()


def probes(size, which):
    return np.random.default_rng(SEED + 1 + which).integers(0, size, N_PROBES)


def digest(prefix, a, which):
    idx = probes(a.size, which)
    return {f"{prefix}_sum": np.float64(a.sum()), f"{prefix}_sumsq": np.float64((a * a).sum()),
            f"{prefix}_max": np.float64(np.abs(a).max()), f"{prefix}_idx": idx, f"{prefix}_val": a[idx]}


def input_sums(X, u, v, w):
    return {"in_u_sumsq": np.float64((u * u).sum()), "in_v_sumsq": np.float64((v * v).sum()),
            "in_w_sumsq": np.float64((w * w).sum()), "in_X_sum": np.float64(X.sum())}


def periodic(steps=100):
    n = PARAMS["n"]
    X0, nstart, nidx, u, v, w = inputs(n)
    po.set_threads(os.cpu_count() or 1)
    g = po.Grid(n, n, n, n, channel=False)
    t0 = time.perf_counter()
    s = po.NSSolver(g, PARAMS["mu"], PARAMS["rho"], PARAMS["dt"], PARAMS["tol"], u, v, w, maxit=100000)
    X = X0.copy()
    for k in range(steps):
        X, st = s.ib_step(X, nstart, nidx, PARAMS["k"])
        assert st == 0, (k, st)
    ru, rv, rw, rp = s.get()
    cg, mg, _ = s.counters()
    out = {k: np.float64(v_) for k, v_ in PARAMS.items()}
    out.update(steps=np.int64(steps), seed=np.int64(SEED), cg_iters=np.int64(cg), mg_cycles=np.int64(mg),
               X=X, **input_sums(X0, u, v, w))
    for k, (name, a) in enumerate((("u", ru), ("v", rv), ("w", rw), ("p", rp))):
        out.update(digest(name, a, k))
    path = os.path.join(HERE, "c2_periodic_128_digest.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {os.path.relpath(path, ROOT)} ({time.perf_counter() - t0:.0f} s, {cg} CG iterations, "
          f"{mg} V-cycles)")


def channel(steps=4):
    assert po.reference_available(), "reference sources not found at " + po.REFERENCE_SRC
    n = PARAMS["n"]
    X0, nstart, nidx, u, vp, w = inputs(n)
    v = channel_v(vp, n)
    M = X0.shape[0]
    deg = np.diff(nstart).astype(np.float64)
    nbr = -np.ones((M, 6))
    for i in range(M):
        nbr[i, : deg.astype(int)[i]] = nidx[nstart[i]:nstart[i + 1]]
    N, NV = n ** 3, n * (n - 1) * n
    t0 = time.perf_counter()
    r = po.run_ref("ib", [PARAMS["mu"], PARAMS["rho"], PARAMS["dt"], PARAMS["tol"], PARAMS["k"], steps, u, v, w,
                          X0.ravel(), deg, nbr.ravel()], L=7, M=M, timeout=7200)
    o = np.cumsum([0, N, NV, N, N, 3 * M])
    out = {k: np.float64(v_) for k, v_ in PARAMS.items()}
    out.update(steps=np.int64(steps), seed=np.int64(SEED), X=r[o[4]:o[5]].reshape(M, 3),
               **input_sums(X0, u, v, w))
    for k, name in enumerate(("u", "v", "w", "p")):
        out.update(digest(name, r[o[k]:o[k + 1]], k))
    path = os.path.join(HERE, "c2_channel_128_ref_digest.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {os.path.relpath(path, ROOT)} ({time.perf_counter() - t0:.0f} s)")


if __name__ == "__main__":
    which = sys.argv[1:] or ["periodic", "channel"]
    if "periodic" in which:
        periodic()
    if "channel" in which:
        channel()
