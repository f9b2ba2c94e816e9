"""Seeded generators for Lagrangian marker sets and initial velocity fields.

The reference ships no marker generators or membrane forces (its only IB
coupling is commented out in test/ib_ns_test.cc:73-96, and markers are built
by the caller as `ib::lagrangian_grid` subclasses, test/ib_test.cc:46-73).
These functions produce the benchmark inputs on the host, once, with numpy;
the same arrays feed the CUDA path and the CPU oracle.

Conventions: positions X[M, 3] in the unit box (x, y, z); neighbour lists in
CSR form (nstart[M+1], nidx[nnz], int32) for the zero-rest-length springs
G_i = k * sum_j (X_j - X_i).
"""
from __future__ import annotations

import numpy as np

SEED = 20261203


def _csr_from_lists(lists):
    nstart = np.zeros(len(lists) + 1, dtype=np.int32)
    nstart[1:] = np.cumsum([len(l) for l in lists])
    nidx = np.concatenate([np.asarray(l, dtype=np.int32) for l in lists]) if lists else np.zeros(0, np.int32)
    return nstart, nidx.astype(np.int32)


def ellipse(m=512, center=(0.5, 0.5), axes=(0.25, 0.20), z=0.5):
    """m markers equally spaced in angle on an ellipse (2-D membrane), ring springs."""
    t = 2 * np.pi * np.arange(m) / m
    X = np.stack([center[0] + axes[0] * np.cos(t), center[1] + axes[1] * np.sin(t), np.full(m, z)], 1)
    lists = [[(i - 1) % m, (i + 1) % m] for i in range(m)]
    return X, *_csr_from_lists(lists)


def _icosahedron():
    p = (1 + 5 ** 0.5) / 2
    v = np.array([[-1, p, 0], [1, p, 0], [-1, -p, 0], [1, -p, 0], [0, -1, p], [0, 1, p], [0, -1, -p], [0, 1, -p],
                  [p, 0, -1], [p, 0, 1], [-p, 0, -1], [-p, 0, 1]], dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    return v / np.linalg.norm(v, axis=1, keepdims=True), f


def _subdivide(v, f):
    cache = {}
    verts = list(v)

    def mid(a, b):
        key = (min(a, b), max(a, b))
        if key not in cache:
            m = (verts[a] + verts[b]) / 2
            verts.append(m / np.linalg.norm(m))
            cache[key] = len(verts) - 1
        return cache[key]

    out = []
    for a, b, c in f:
        ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
        out += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
    return np.array(verts), np.array(out, dtype=np.int64)


def icosphere_faces(level=5):
    """Unit-sphere face centroids of a level-`level` icosphere (20*4^level faces)
    and the face-adjacency lists (three neighbours per face)."""
    v, f = _icosahedron()
    for _ in range(level):
        v, f = _subdivide(v, f)
    c = v[f].mean(axis=1)
    c /= np.linalg.norm(c, axis=1, keepdims=True)
    edge_faces = {}
    for i, (a, b, cc) in enumerate(f):
        for e in ((a, b), (b, cc), (cc, a)):
            edge_faces.setdefault((min(e), max(e)), []).append(i)
    lists = [[] for _ in range(len(f))]
    for fs in edge_faces.values():
        if len(fs) == 2:
            lists[fs[0]].append(fs[1])
            lists[fs[1]].append(fs[0])
    return c, lists


def fibonacci_sphere(m):
    """m points of the spherical Fibonacci lattice on the unit sphere."""
    i = np.arange(m) + 0.5
    th = np.arccos(1 - 2 * i / m)
    ph = np.pi * (1 + 5 ** 0.5) * i
    return np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], 1)


def knn_lists(P, k=6):
    """k nearest neighbours on the unit sphere, symmetrised (j in N(i) <=> i in N(j))."""
    m = len(P)
    # bucket by a coarse 3-D grid to avoid an m^2 distance matrix
    cell = max(2.0 * np.sqrt(4 * np.pi / m) * 2.0, 1e-3)
    keys = np.floor((P + 1.0) / cell).astype(np.int64)
    buckets = {}
    for i, kk in enumerate(map(tuple, keys)):
        buckets.setdefault(kk, []).append(i)
    lists = [set() for _ in range(m)]
    offs = [(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)]
    for i in range(m):
        kx, ky, kz = keys[i]
        cand = []
        for a, b, c in offs:
            cand += buckets.get((kx + a, ky + b, kz + c), [])
        cand = np.array([j for j in cand if j != i])
        d = np.linalg.norm(P[cand] - P[i], axis=1)
        for j in cand[np.argsort(d, kind="stable")[:k]]:
            lists[i].add(int(j))
            lists[int(j)].add(i)
    return [sorted(s) for s in lists]


def y2(m_order, P):
    """Real spherical harmonic Y_2^m (unnormalised) on unit vectors P."""
    x, y, z = P[:, 0], P[:, 1], P[:, 2]
    return {0: 0.5 * (3 * z * z - 1), 1: x * z, -1: y * z, 2: 0.5 * (x * x - y * y), -2: x * y}[m_order]


def shell(P_unit, lists, center, radius, amp=0.0, m_order=0):
    """Place a unit-sphere marker set as a shell of `radius` around `center`,
    perturbed radially by amp * Y_2^m."""
    r = radius * (1.0 + (amp / radius) * y2(m_order, P_unit)) if amp else np.full(len(P_unit), radius)
    X = np.asarray(center)[None, :] + r[:, None] * P_unit
    return X, lists


def place_centres(count, radius, min_sep, rng, lo=None, hi=None, tries=100000):
    """Uniform centres with rejection at min_sep; centres kept in [lo, hi]^3."""
    lo = radius + 0.02 if lo is None else lo
    hi = 1.0 - radius - 0.02 if hi is None else hi
    out = []
    for _ in range(tries):
        c = rng.uniform(lo, hi, size=3)
        if all(np.linalg.norm(c - o) >= min_sep for o in out):
            out.append(c)
            if len(out) == count:
                return np.array(out)
    raise RuntimeError("could not place shells with the requested separation")


def multi_shell(nshell, per_shell, radius, min_sep, amp, seed=SEED, lo=None, hi=None, k=6):
    """`nshell` perturbed Fibonacci shells of `per_shell` markers each."""
    rng = np.random.default_rng(seed)
    centres = place_centres(nshell, radius, min_sep, rng, lo, hi)
    P = fibonacci_sphere(per_shell)
    base_lists = knn_lists(P, k)
    Xs, lists = [], []
    for s, c in enumerate(centres):
        m_order = int(rng.integers(-2, 3))
        X, _ = shell(P, base_lists, c, radius, amp, m_order)
        Xs.append(X)
        off = s * per_shell
        lists += [[j + off for j in l] for l in base_lists]
    X = np.concatenate(Xs)
    return X, *_csr_from_lists(lists)


def icoshell(level, center, radius, amp):
    """Icosphere face-centroid shell perturbed by amp * Y_2^0 (face-adjacency springs)."""
    P, lists = icosphere_faces(level)
    X, _ = shell(P, lists, center, radius, amp, 0)
    return X, *_csr_from_lists(lists)


def random_solenoidal_velocity(nx, ny, nz, rms=0.1, k_peak=4.0, seed=SEED):
    """Random periodic velocity on the MAC grid with energy spectrum
    E(k) ~ k^4 exp(-2 (k/k_peak)^2); made divergence-free in Fourier space
    (the NS constructor projects it again on the discrete grid) and scaled
    to the requested RMS. Returns u, v, w each of nx*ny*nz (x fastest)."""
    rng = np.random.default_rng(seed)
    kx = np.fft.fftfreq(nx, 1.0 / nx)
    ky = np.fft.fftfreq(ny, 1.0 / ny)
    kz = np.fft.rfftfreq(nz, 1.0 / nz)
    KX, KY, KZ = np.meshgrid(kx, ky, kz, indexing="ij")
    kk = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
    amp = np.where(kk > 0, kk ** 2 * np.exp(-(kk / k_peak) ** 2) / np.maximum(kk, 1e-12), 0.0)
    comps = []
    for _ in range(3):
        ph = rng.uniform(0, 2 * np.pi, KX.shape)
        comps.append(amp * (rng.standard_normal(KX.shape) + 0j) * np.exp(1j * ph))
    A = np.stack(comps)
    K = np.stack([KX, KY, KZ])
    kdot = (A * K).sum(0) / np.maximum(kk ** 2, 1e-12)
    A = A - K * kdot
    fields = [np.fft.irfftn(a, s=(nx, ny, nz), axes=(0, 1, 2)) for a in A]
    r = np.sqrt(sum((f ** 2).mean() for f in fields) / 3.0)
    # indexing='ij' gives [x, y, z]; flatten x-fastest -> transpose to [z, y, x]
    return [np.ascontiguousarray((f * (rms / r)).transpose(2, 1, 0)).ravel() for f in fields]
