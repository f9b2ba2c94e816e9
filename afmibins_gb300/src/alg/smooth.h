// alg::smooth(x, A, b): one Gauss-Seidel sweep on A x = b
// (src/alg/smooth.h:35-51). The GPU sweeps red cells then black cells; the
// reference sweeps lexicographically. Both are the same relaxation family and
// converge to the same solution; single sweeps differ in their iterates.
#ifndef ALG_SMOOTH_H
#define ALG_SMOOTH_H

#include "dt/matrix.h"
#include "dt/vector.h"

namespace alg {

template <unsigned int Size>
void smooth(dt::vector<Size>& x, const dt::matrix<Size>& A, const dt::vector<Size>& b) {
    A.relax(x.data(), b.data());
}

}  // namespace alg

#endif
