// dt::matrix<Size>: the reference's operator type (src/dt/matrix.h:35-94). The
// reference stores CSR and multiplies row by row; here every operator is
// matrix-free on the GPU, so a matrix is an object that can apply itself
// (y = A x), relax (one Gauss-Seidel sweep) and solve with CG. operator*
// keeps the reference's calling form A * x.
#ifndef DT_MATRIX_H
#define DT_MATRIX_H

#include <cstddef>

#include "vector.h"

namespace dt {

template <unsigned int Size>
class matrix {
  public:
    typedef double value_type;
    typedef std::size_t size_type;
    virtual ~matrix() {}
    // y = A x on host arrays of Size doubles
    virtual void apply(const double* x, double* y) const = 0;
    // one Gauss-Seidel sweep on A x = b (red-black on the GPU)
    virtual void relax(double* x, const double* b) const = 0;
    // CG on A x = b from the warm start x to ||r||_2 <= tol; returns the iterations
    virtual unsigned solve_cg(double* x, const double* b, double tol) const = 0;

    template <template <unsigned int> class V>
    V<Size> operator*(const V<Size>& right) const {
        V<Size> result;
        apply(right.data(), result.data());
        return result;
    }
    size_type size() const { return Size; }
};

}  // namespace dt

#endif
