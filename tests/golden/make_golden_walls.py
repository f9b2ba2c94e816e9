"""Golden vectors of the compiled reference with moving channel walls.

The reference's sub-step takes the wall velocities ut, ub, wt, wb (u and w at
the top and bottom walls, nx*nz each, x fastest) into the Helmholtz
right-hand sides (src/ns/helmholtz.h:177-196, 321-337) and updates them in its
projection (src/ns/projection.h:75-122); the other fixtures start from zero
walls. Three fixtures, all from the reference compiled unchanged
(oracle/ref_driver.cc) with seeded smooth, nonzero wall velocities:

* ns_walls_16.npz — 16^3 channel, 4 NS sub-steps with seeded forces;
* ib_walls_16.npz — 16^3 channel, 2 IB steps of a 320-marker shell;
* ib_channel_256_digest.npz — 256^3 channel, 2 IB steps of a 5,120-marker
  icosphere shell (level 4, radius 0.2 at the centre, 0.02 Y_2^0: 0.28 from
  every wall and periodic face), mu 0.01, dt 2e-5, tol 1e-12, a seeded
  solenoidal initial velocity (RMS 0.1); kept as a digest (per field its sum,
  sum of squares, largest magnitude and values at 4096 seeded indices; the
  walls and marker positions in full).

Run in a container that has the reference sources (default location in
oracle/Makefile, override with AFMIB_REFERENCE); the 256^3 case builds
oracle/_ref/ref_L8_* and needs about 12 GB of memory and several minutes:

    python tests/golden/make_golden_walls.py [small] [large]
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

SEED = mk.SEED + 7
N_PROBES = 4096


def wall_velocities(n, seed=SEED):
    """ut, ub, wt, wb (nx*nz each, x fastest): a seeded mean plus one smooth mode each."""
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    Z, X = np.meshgrid(x, x, indexing="ij")  # [z, x]: ravel is x fastest
    out = []
    for _ in range(4):
        a0, a1 = 0.05 * rng.standard_normal(), 0.02 * rng.standard_normal()
        p1, p2 = rng.random(2)
        out.append((a0 + a1 * np.sin(2 * np.pi * (X + p1)) * np.cos(2 * np.pi * (Z + p2))).ravel())
    return np.concatenate(out)


def _save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    print("wrote", os.path.relpath(path, ROOT))


def _nbr(nstart, nidx, M):
    deg = np.diff(nstart).astype(np.float64)
    nbr = -np.ones((M, 6))
    for i in range(M):
        nbr[i, : int(deg[i])] = nidx[nstart[i]:nstart[i + 1]]
    return deg, nbr


def small():
    assert po.reference_available(), "reference sources not found at " + po.REFERENCE_SRC
    tol = 1e-12
    rng = np.random.default_rng(SEED)
    n = 16
    N, NV, NXZ = n ** 3, n * (n - 1) * n, n * n
    u, v, w = 0.1 * rng.standard_normal(N), 0.1 * rng.standard_normal(NV), 0.1 * rng.standard_normal(N)
    fx, fy, fz = rng.standard_normal(N), rng.standard_normal(NV), rng.standard_normal(N)
    walls = wall_velocities(n)
    mu, rho, dt = 0.01, 1.0, 1e-3
    r = po.run_ref("ns", [mu, rho, dt, tol, 4, u, v, w, walls, fx, fy, fz], L=4)
    o = np.cumsum([0, N, NV, N, N, 4 * NXZ])
    _save("ns_walls_16", u0=u, v0=v, w0=w, fx=fx, fy=fy, fz=fz, walls0=walls, mu=np.float64(mu),
          rho=np.float64(rho), dt=np.float64(dt), tol=np.float64(tol), substeps=np.int64(4),
          u=r[o[0]:o[1]], v=r[o[1]:o[2]], w=r[o[2]:o[3]], p=r[o[3]:o[4]], walls=r[o[4]:o[5]])

    M = 320
    P = mk.fibonacci_sphere(M)
    lists = [l[:6] for l in mk.knn_lists(P, 6)]
    X, _ = mk.shell(P, lists, (0.5, 0.5, 0.5), 0.2, 0.02, 0)
    nstart, nidx = mk._csr_from_lists(lists)
    deg, nbr = _nbr(nstart, nidx, M)
    k = 0.5
    r = po.run_ref("ibw", [mu, rho, dt, tol, k, 2, u, v, w, X.ravel(), deg, nbr.ravel(), walls], L=4, M=M)
    o = np.cumsum([0, N, NV, N, N, 3 * M, 4 * NXZ])
    _save("ib_walls_16", X=X, nstart=nstart, nidx=nidx, u0=u, v0=v, w0=w, walls0=walls, mu=np.float64(mu),
          rho=np.float64(rho), dt=np.float64(dt), tol=np.float64(tol), k=np.float64(k), steps=np.int64(2),
          u=r[o[0]:o[1]], v=r[o[1]:o[2]], w=r[o[2]:o[3]], p=r[o[3]:o[4]], Xout=r[o[4]:o[5]].reshape(M, 3),
          walls=r[o[5]:o[6]])


PARAMS_256 = dict(n=256, mu=0.01, rho=1.0, dt=2e-5, k=0.5, tol=1e-12)


def inputs_256(n=256):
    """Markers, the channel initial velocity (v without its y = 0 plane) and the walls."""
    X, nstart, nidx = mk.icoshell(4, (0.5, 0.5, 0.5), 0.2, 0.02)
    u, v, w = mk.random_solenoidal_velocity(n, n, n, rms=0.1, k_peak=4.0, seed=SEED)
    v = np.ascontiguousarray(v.reshape(n, n, n)[:, 1:, :]).ravel()
    return X, nstart, nidx, u, v, w, wall_velocities(n)


def probes(size, which):
    return np.random.default_rng(SEED + 1 + which).integers(0, size, N_PROBES)


def digest(prefix, a, which):
    idx = probes(a.size, which)
    return {f"{prefix}_sum": np.float64(a.sum()), f"{prefix}_sumsq": np.float64((a * a).sum()),
            f"{prefix}_max": np.float64(np.abs(a).max()), f"{prefix}_idx": idx, f"{prefix}_val": a[idx]}


def large(steps=2):
    assert po.reference_available(), "reference sources not found at " + po.REFERENCE_SRC
    n = PARAMS_256["n"]
    X0, nstart, nidx, u, v, w, walls = inputs_256(n)
    M = X0.shape[0]
    deg, nbr = _nbr(nstart, nidx, M)
    N, NV, NXZ = n ** 3, n * (n - 1) * n, n * n
    t0 = time.perf_counter()
    p = PARAMS_256
    r = po.run_ref("ibw", [p["mu"], p["rho"], p["dt"], p["tol"], p["k"], steps, u, v, w, X0.ravel(), deg,
                           nbr.ravel(), walls], L=8, M=M, timeout=4 * 3600)
    o = np.cumsum([0, N, NV, N, N, 3 * M, 4 * NXZ])
    out = {k: np.float64(v_) for k, v_ in p.items()}
    out.update(steps=np.int64(steps), seed=np.int64(SEED), X=r[o[4]:o[5]].reshape(M, 3), walls=r[o[5]:o[6]],
               in_u_sumsq=np.float64((u * u).sum()), in_v_sumsq=np.float64((v * v).sum()),
               in_w_sumsq=np.float64((w * w).sum()), in_X_sum=np.float64(X0.sum()))
    for k, name in enumerate(("u", "v", "w", "p")):
        out.update(digest(name, r[o[k]:o[k + 1]], k))
    _save("ib_channel_256_digest", **out)
    print(f"{time.perf_counter() - t0:.0f} s")


if __name__ == "__main__":
    which = sys.argv[1:] or ["small", "large"]
    if "small" in which:
        small()
    if "large" in which:
        large()
