// alg::grad<nx, ny, nz, n>(px, py, pz, p): MAC gradient of a cell-centred
// scalar, py on the interior y faces only (src/alg/grad.h:29-44), on the GPU.
#ifndef ALG_GRAD_H
#define ALG_GRAD_H

#include "afmib_shim.h"
#include "dt/vector.h"

namespace alg {

template <unsigned nx, unsigned ny, unsigned nz, unsigned n>
void grad(dt::vector<nx * ny * nz>& px, dt::vector<nx * (ny - 1) * nz>& py, dt::vector<nx * ny * nz>& pz,
          dt::vector<nx * ny * nz>& p) {
    static afmib_solver* s = afmib_shim::make_solver(nx, ny, nz, n, 1, 1e-12);
    afmib_shim::check(afmib_grad(s, px.data(), py.data(), pz.data(), p.data()), s, "alg::grad");
}

}  // namespace alg

#endif
