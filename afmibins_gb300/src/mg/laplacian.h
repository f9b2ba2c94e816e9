// mg::laplacian<G>: the pressure Laplacian n^2 * Delta of the channel
// (x, z periodic, Neumann walls in y), src/mg/laplacian.h:31-153, applied
// matrix-free on the GPU.
#ifndef MG_LAPLACIAN_H
#define MG_LAPLACIAN_H

#include <cmath>
#include <vector>

#include "afmib_shim.h"
#include "dt/matrix.h"
#include "dt/vector.h"

namespace mg {

template <class Geometry>
class laplacian : public dt::matrix<Geometry::nx * Geometry::ny * Geometry::nz> {
  public:
    static constexpr unsigned int nx = Geometry::nx;
    static constexpr unsigned int ny = Geometry::ny;
    static constexpr unsigned int nz = Geometry::nz;
    static constexpr unsigned int n = Geometry::n;
    static constexpr unsigned int N = nx * ny * nz;

    void apply(const double* x, double* y) const override {
        afmib_solver* s = afmib_shim::context<Geometry>();
        afmib_shim::check(afmib_lap_apply(s, y, x), s, "mg::laplacian");
    }
    void relax(double* x, const double* b) const override {
        afmib_solver* s = afmib_shim::context<Geometry>();
        afmib_shim::check(afmib_smooth(s, x, b), s, "alg::smooth");
    }
    // CG on the (semi-definite) Laplacian, as the reference's coarsest level
    // does (src/mg/solver.h:264-271); matrix-vector products on the GPU.
    unsigned solve_cg(double* x, const double* b, double tol) const override {
        std::vector<double> r(N), p(N), q(N);
        apply(x, q.data());
        double n0 = 0.0;
        for (unsigned i = 0; i < N; ++i) { r[i] = b[i] - q[i]; p[i] = r[i]; n0 += r[i] * r[i]; }
        unsigned count = 0;
        while (std::sqrt(n0) > tol && count < 100000u) {
            apply(p.data(), q.data());
            double pq = 0.0;
            for (unsigned i = 0; i < N; ++i) pq += p[i] * q[i];
            const double a = n0 / pq;
            double n1 = 0.0;
            for (unsigned i = 0; i < N; ++i) { x[i] += a * p[i]; r[i] -= a * q[i]; n1 += r[i] * r[i]; }
            const double beta = n1 / n0;
            n0 = n1;
            for (unsigned i = 0; i < N; ++i) p[i] = p[i] * beta + r[i];
            ++count;
        }
        return count;
    }
};

}  // namespace mg

#endif
