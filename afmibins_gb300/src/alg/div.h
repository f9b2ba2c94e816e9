// alg::div<nx, ny, nz, n>(d, u, v, w, top, bottom): MAC divergence
// n*(du + dv + dw) with x, z periodic and the wall fluxes top/bottom in y
// (src/alg/div.h:29-60), evaluated by the GPU (afmib_div).
#ifndef ALG_DIV_H
#define ALG_DIV_H

#include "afmib_shim.h"
#include "dt/vector.h"

namespace alg {

template <unsigned int nx, unsigned int ny, unsigned int nz, unsigned int n>
void div(dt::vector<nx * ny * nz>& d, dt::vector<nx * ny * nz>& u, dt::vector<nx * (ny - 1) * nz>& v,
         dt::vector<nx * ny * nz>& w, dt::vector<nx * nz>& top, dt::vector<nx * nz>& bottom) {
    static afmib_solver* s = afmib_shim::make_solver(nx, ny, nz, n, 1, 1e-12);
    afmib_shim::check(afmib_div(s, d.data(), u.data(), v.data(), w.data(), top.data(), bottom.data()), s, "alg::div");
}

}  // namespace alg

#endif
