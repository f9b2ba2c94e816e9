"""Digest fixture of the compiled reference at 256^3 (channel): two NS
sub-steps (one BE/CN pair) from seeded fields, tol 1e-12.

Run in a container that has the reference sources (default /root/reference,
override with AFMIB_REFERENCE); it builds oracle/_ref/ref_L8_* (about 10 GB of
memory while it runs, a few minutes):

    python tests/golden/make_golden_256.py

The fields at 256^3 are 134 MB each, so the fixture keeps the seed that
regenerates the inputs (numpy PCG64, identical on every platform) and, per
output field, its sum, its sum of squares, its largest magnitude and its
values at 4096 seeded indices.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle as po  # noqa: E402

SEED = 20261203 + 256
N_PROBES = 4096


def inputs(n=256):
    """The seeded inputs: velocity (RMS 0.1) and forces in the reference's layout."""
    N, NV = n ** 3, n * (n - 1) * n
    rng = np.random.default_rng(SEED)
    u, v, w = 0.1 * rng.standard_normal(N), 0.1 * rng.standard_normal(NV), 0.1 * rng.standard_normal(N)
    fx, fy, fz = rng.standard_normal(N), rng.standard_normal(NV), rng.standard_normal(N)
    return u, v, w, fx, fy, fz


def probes(size, which):
    return np.random.default_rng(SEED + 1 + which).integers(0, size, N_PROBES)


def digest(prefix, a, which):
    idx = probes(a.size, which)
    return {f"{prefix}_sum": np.float64(a.sum()), f"{prefix}_sumsq": np.float64((a * a).sum()),
            f"{prefix}_max": np.float64(np.abs(a).max()), f"{prefix}_idx": idx, f"{prefix}_val": a[idx]}


def main():
    assert po.reference_available(), "reference sources not found at " + po.REFERENCE_SRC
    n = 256
    N, NV, NXZ = n ** 3, n * (n - 1) * n, n * n
    u, v, w, fx, fy, fz = inputs(n)
    mu, rho, dt, tol, substeps = 0.01, 1.0, 1e-4, 1e-12, 2
    walls = np.zeros(4 * NXZ)
    r = po.run_ref("ns", [mu, rho, dt, tol, substeps, u, v, w, walls, fx, fy, fz], L=8, timeout=7200)
    o = np.cumsum([0, N, NV, N, N, 4 * NXZ])
    out = dict(mu=np.float64(mu), rho=np.float64(rho), dt=np.float64(dt), tol=np.float64(tol),
               substeps=np.int64(substeps), seed=np.int64(SEED))
    for k, name in enumerate(("u", "v", "w", "p", "walls")):
        out.update(digest(name, r[o[k]:o[k + 1]], k))
    path = os.path.join(HERE, "ns_channel_256_digest.npz")
    np.savez_compressed(path, **out)
    print("wrote", os.path.relpath(path, ROOT))


if __name__ == "__main__":
    main()
