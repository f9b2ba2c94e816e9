"""The oracle's corrected channel wall update (walls_corrected): every nx*nz
wall entry is updated and the w rows use the z-gradient, where the
reference's update (src/ns/projection.h:86-104) covers nx*ny entries and
reads the x-gradient for w. Checked on the oracle alone, on a grid with
ny < nz so that the two loops differ."""
import numpy as np

from oracle import pyoracle as po


def _run(corrected, nx=8, ny=4, nz=8, steps=2):
    g = po.Grid(nx, ny, nz, nx, channel=True)
    rng = np.random.default_rng(41)
    u, v, w = 0.1 * rng.standard_normal(g.ncell), 0.1 * rng.standard_normal(g.nv), 0.1 * rng.standard_normal(g.ncell)
    f = [rng.standard_normal(g.ncell), rng.standard_normal(g.nv), rng.standard_normal(g.ncell)]
    ns = po.NSSolver(g, 0.01, 1.0, 1e-3, 1e-12, u, v, w, walls_corrected=corrected)
    for _ in range(steps):
        assert ns.step(*f) == 0
    return g, ns.walls.reshape(4, nx * nz).copy(), ns.get()


def test_corrected_walls_cover_every_entry_and_use_the_z_gradient():
    g, ref, _ = _run(False)
    _, cor, _ = _run(True)
    nxny = g.nx * g.ny
    # the reference's loop leaves the entries past nx*ny untouched (zero)
    assert np.all(ref[:, nxny:] == 0.0)
    assert np.all(np.abs(cor[:, nxny:]).max(axis=1) > 0)
    # u walls: same update over the entries both loops cover (first sub-step);
    # w walls: the corrected rows read the z-gradient
    assert not np.allclose(ref[2, :nxny], cor[2, :nxny])
