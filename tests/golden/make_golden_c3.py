"""Digest fixture of the 256^3 benchmark workload in FP64 (the oracle).

The periodic unit cube on a 256^3 MAC grid, mu 0.005, rho 1, dt 2e-5, 200,000
markers on 10 spherical shells of radius 0.08 (spherical Fibonacci lattice,
6-nearest-neighbour springs, k 0.5, centres drawn from a seed with minimum
separation 0.2, radial perturbation 0.01 Y_2^m with seeded m), a seeded
solenoidal initial velocity (RMS 0.1, spectrum peaked at wavenumber 4): the
inputs of the benchmark's headline configuration. Two IB steps at solver
tolerance 1e-12, run by the CPU oracle on all host cores (its threaded
passes give the one-thread bits):

    python tests/golden/make_golden_c3.py

The fields are 134 MB each, so the fixture keeps, per field, its sum, sum of
squares, largest magnitude and values at 4096 seeded indices, checksums of
the regenerated inputs, and the positions of 4096 seeded markers.
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
SEED = mk.SEED + 3
PARAMS = dict(n=256, mu=0.005, rho=1.0, dt=2e-5, k=0.5, tol=1e-12)


def inputs(n=256):
    """The benchmark's markers (X, nstart, nidx) and initial velocity (u, v, w)."""
    X, nstart, nidx = mk.multi_shell(10, 20000, 0.08, 0.2, 0.01, seed=SEED)
    u, v, w = mk.random_solenoidal_velocity(n, n, n, rms=0.1, k_peak=4.0, seed=SEED)
    return X, nstart, nidx, u, v, w


def probes(size, which):
    return np.random.default_rng(SEED + 1 + which).integers(0, size, N_PROBES)


def digest(prefix, a, which):
    idx = probes(a.size, which)
    return {f"{prefix}_sum": np.float64(a.sum()), f"{prefix}_sumsq": np.float64((a * a).sum()),
            f"{prefix}_max": np.float64(np.abs(a).max()), f"{prefix}_idx": idx, f"{prefix}_val": a[idx]}


def main(steps=2):
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
               in_u_sumsq=np.float64((u * u).sum()), in_v_sumsq=np.float64((v * v).sum()),
               in_w_sumsq=np.float64((w * w).sum()), in_X_sum=np.float64(X0.sum()))
    for k, (name, a) in enumerate((("u", ru), ("v", rv), ("w", rw), ("p", rp))):
        out.update(digest(name, a, k))
    midx = probes(X.shape[0], 9)
    out.update(X_idx=midx, X_val=X[midx], X0_val=X0[midx])
    path = os.path.join(HERE, "c3_periodic_256_digest.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {os.path.relpath(path, ROOT)} ({time.perf_counter() - t0:.0f} s, {cg} CG iterations, "
          f"{mg} V-cycles)")


if __name__ == "__main__":
    main()
