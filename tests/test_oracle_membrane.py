"""Membrane forces of the oracle (springs plus bending): the force is minus
the gradient of the energy k/4 sum_i sum_{j in N(i)} |X_j - X_i|^2 +
kb/2 sum_i |(L X)_i|^2 (central differences), it sums to zero over the
markers, and it does not change under a translation."""
import numpy as np

from afmibins_gb300 import markers as mk
from oracle import pyoracle as po


def _graph(m=40, k=5, seed=3):
    P = mk.fibonacci_sphere(m) * 0.2 + 0.5
    lists = [l[:k] for l in mk.knn_lists(P, k)]
    # symmetrise: j in N(i) <=> i in N(j)
    sets = [set(l) for l in lists]
    for i, l in enumerate(lists):
        for j in l:
            sets[j].add(i)
    lists = [sorted(s) for s in sets]
    nstart, nidx = mk._csr_from_lists(lists)
    rng = np.random.default_rng(seed)
    return P + 0.01 * rng.standard_normal(P.shape), np.asarray(nstart), np.asarray(nidx), lists


def _energy(X, lists, k, kb):
    e = 0.0
    Y = np.zeros_like(X)
    for i, l in enumerate(lists):
        d = X[l] - X[i]
        e += 0.25 * k * np.sum(d * d)
        Y[i] = d.sum(axis=0)
    return e + 0.5 * kb * np.sum(Y * Y)


def test_forces_are_minus_the_energy_gradient():
    X, nstart, nidx, lists = _graph()
    k, kb = 0.7, 0.3
    G = po.membrane_forces(X, nstart, nidx, k, kb)
    h = 1e-6
    rng = np.random.default_rng(5)
    for _ in range(12):
        i, a = int(rng.integers(len(X))), int(rng.integers(3))
        Xp, Xm = X.copy(), X.copy()
        Xp[i, a] += h
        Xm[i, a] -= h
        fd = -(_energy(Xp, lists, k, kb) - _energy(Xm, lists, k, kb)) / (2 * h)
        assert abs(G[a, i] - fd) <= 1e-6 * max(1.0, abs(fd))


def test_forces_sum_to_zero_and_are_translation_invariant():
    X, nstart, nidx, _ = _graph()
    G = po.membrane_forces(X, nstart, nidx, 0.7, 0.3)
    assert np.abs(G.sum(axis=1)).max() < 1e-12
    G2 = po.membrane_forces(X + np.array([0.1, -0.2, 0.05]), nstart, nidx, 0.7, 0.3)
    np.testing.assert_allclose(G2, G, atol=1e-13)
    # kb = 0: the springs alone, bit for bit
    assert np.array_equal(po.membrane_forces(X, nstart, nidx, 0.7, 0.0), po.springs(X, nstart, nidx, 0.7))
