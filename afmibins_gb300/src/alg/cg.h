// alg::conjugate_gradient(x, A, b, tol): CG from the warm start x until the
// absolute 2-norm of the residual is at most tol; returns the iteration count
// (src/alg/cg.h:32-56). Runs matrix-free on the GPU for the Helmholtz
// operators; bounded (the reference loops forever when tol is below round-off).
#ifndef ALG_CG_H
#define ALG_CG_H

#include "dt/matrix.h"
#include "dt/vector.h"

namespace alg {

template <unsigned int Size>
unsigned int conjugate_gradient(dt::vector<Size>& x, const dt::matrix<Size>& A, const dt::vector<Size>& b, double tol) {
    return A.solve_cg(x.data(), b.data(), tol);
}

}  // namespace alg

#endif
