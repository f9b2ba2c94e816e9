"""Generate the golden vectors in tests/golden/ from the compiled reference.

Run in a container that has the reference sources (default /root/reference,
override with AFMIB_REFERENCE):

    python tests/golden/make_golden.py

Each fixture is an .npz holding the inputs and the reference's outputs of one
driver command (oracle/ref_driver.cc, built from the reference headers by
oracle/Makefile). The multigrid right-hand sides of the reference's own
tests are parsed from test/mg_test.cc, test/mg_test3.cc and
test/restr_test.cc; test/mg_test3.cc asks for tol 1e-16, which never
converges (src/mg/solver.h:228 spins), so these fixtures use 1e-12.
All other inputs are seeded (numpy PCG64).
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle as po  # noqa: E402
from afmibins_gb300 import markers as mk  # noqa: E402

REF = po.REFERENCE_SRC


def parse_array(path, count):
    """The numbers of the first brace-initialised dt::vector in a reference test file."""
    text = open(path).read()
    body = text[text.index("{", text.index("dt::vector<")) + 1:]
    body = body[: body.index("}")]
    nums = [float(t) for t in re.findall(r"[-+]?\d+\.?\d*(?:[eE][-+]?\d+)?", body)]
    assert len(nums) == count, (path, len(nums))
    return np.array(nums)


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    print("wrote", os.path.relpath(path, ROOT), sum(a.nbytes for a in map(np.asarray, arrays.values())), "bytes")


def main():
    assert po.reference_available(), "reference sources not found at " + REF
    tol = 1e-12

    # --- multigrid on the reference's own right-hand sides (16^3 channel) ---
    for name, fname in (("mg_test", "mg_test.cc"), ("mg_test3", "mg_test3.cc")):
        b = parse_array(os.path.join(REF, "test", fname), 4096)
        r = po.run_ref("mg", [tol, 2, 2, b], L=4)
        save(f"{name}_16", rhs=b, tol=np.float64(tol), cycles=np.int64(r[0]), x=r[1:])

    # --- restriction of test/restr_test.cc (2^3 -> 1) ---
    fine = parse_array(os.path.join(REF, "test", "restr_test.cc"), 8)
    r = po.run_ref("restrict", [fine], L=1)
    save("restr_test", fine=fine, coarse=r)

    # --- test/mg_test2.cc: an 8x8x8-cell coarsest level, b = 1 with b[0] = 2 ---
    b = np.ones(4096)
    b[0] = 2.0
    r = po.run_ref("mg", [tol, 2, 2, b], L=1, W=8, H=8, D=8)
    x = r[1:]
    lx = po.run_ref("lap", [x], L=1, W=8, H=8, D=8)
    save("mg_test2_box", rhs=b, tol=np.float64(tol), cycles=np.int64(r[0]), x=x, lap_x=lx)

    # --- single operators on seeded inputs (8^3 channel) ---
    rng = np.random.default_rng(mk.SEED + 1)
    n = 8
    N, NV, NXZ = n ** 3, n * (n - 1) * n, n * n
    x, b = rng.standard_normal(N), rng.standard_normal(N)
    c = rng.standard_normal(N // 8)
    u, v, w = rng.standard_normal(N), rng.standard_normal(NV), rng.standard_normal(N)
    top, bot = rng.standard_normal(NXZ), rng.standard_normal(NXZ)
    s = -0.013
    x0 = rng.standard_normal(N)
    out = dict(x=x, b=b, c=c, u=u, v=v, w=w, top=top, bottom=bot, s=np.float64(s), x0=x0)
    out["lap"] = po.run_ref("lap", [x], L=3)
    out["gs"] = po.run_ref("gs", [x, b], L=3)
    out["restrict"] = po.run_ref("restrict", [x], L=3)
    out["prolong"] = po.run_ref("prolong", [c], L=3)
    out["div"] = po.run_ref("div", [u, v, w, top, bot], L=3)
    out["grad"] = po.run_ref("grad", [x], L=3)
    out["advect"] = po.run_ref("advect", [u, v, w], L=3)
    out["helm"] = po.run_ref("helm", [s, u, v, w], L=3)
    r = po.run_ref("cg", [s, tol, x0, b], L=3)
    out["cg_iters"], out["cg_x"] = np.int64(r[0]), r[1:]
    save("ops_8", **out)

    # --- Navier-Stokes: 4 sub-steps (2 BE/CN pairs) at 16^3 channel ---
    rng = np.random.default_rng(mk.SEED + 2)
    n = 16
    N, NV, NXZ = n ** 3, n * (n - 1) * n, n * n
    u, v, w = 0.1 * rng.standard_normal(N), 0.1 * rng.standard_normal(NV), 0.1 * rng.standard_normal(N)
    fx, fy, fz = rng.standard_normal(N), rng.standard_normal(NV), rng.standard_normal(N)
    walls = np.zeros(4 * NXZ)
    mu, rho, dt = 0.01, 1.0, 1e-3
    r = po.run_ref("ns", [mu, rho, dt, tol, 4, u, v, w, walls, fx, fy, fz], L=4)
    o = np.cumsum([0, N, NV, N, N, 4 * NXZ])
    save("ns_16", u0=u, v0=v, w0=w, fx=fx, fy=fy, fz=fz, mu=np.float64(mu), rho=np.float64(rho),
         dt=np.float64(dt), tol=np.float64(tol), substeps=np.int64(4),
         u=r[o[0]:o[1]], v=r[o[1]:o[2]], w=r[o[2]:o[3]], p=r[o[3]:o[4]], walls=r[o[4]:o[5]])

    # --- spreading, interpolation and two IB steps at 16^3 channel, 320 markers ---
    M = 320
    P = mk.fibonacci_sphere(M)
    lists = [l[:6] for l in mk.knn_lists(P, 6)]
    X, _ = mk.shell(P, lists, (0.5, 0.5, 0.5), 0.2, 0.02, 0)
    nstart, nidx = mk._csr_from_lists(lists)
    deg = np.diff(nstart).astype(np.float64)
    nbr = -np.ones((M, 6))
    for i, l in enumerate(lists):
        nbr[i, : len(l)] = l
    vol = 0.5 + rng.random(M)
    F = rng.standard_normal((3, M))
    sp = po.run_ref("spread", [X.ravel(), vol, F[0], F[1], F[2]], L=4, M=M)
    ue, ve, we = rng.standard_normal(N), rng.standard_normal(NV), rng.standard_normal(N)
    ip = po.run_ref("interp", [X.ravel(), ue, ve, we], L=4, M=M)
    k = 0.5
    r = po.run_ref("ib", [mu, rho, dt, tol, k, 2, u, v, w, X.ravel(), deg, nbr.ravel()], L=4, M=M)
    o = np.cumsum([0, N, NV, N, N, 3 * M])
    save("ib_16", X=X, nstart=nstart, nidx=nidx, vol=vol, F=F, spread=sp, ue=ue, ve=ve, we=we, interp=ip,
         u0=u, v0=v, w0=w, mu=np.float64(mu), rho=np.float64(rho), dt=np.float64(dt), tol=np.float64(tol),
         k=np.float64(k), steps=np.int64(2),
         u=r[o[0]:o[1]], v=r[o[1]:o[2]], w=r[o[2]:o[3]], p=r[o[3]:o[4]], Xout=r[o[4]:o[5]].reshape(M, 3))


if __name__ == "__main__":
    main()
