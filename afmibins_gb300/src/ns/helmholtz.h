// ns::helmholtz_periodic<G>(s) and ns::helmholtz_dirichlet<G>(s): the
// viscous operators I + s * Delta of the cell-centred-in-y components (u, w)
// with the one-sided wall closure, and of v between the walls
// (src/ns/helmholtz.h:41-337), applied matrix-free on the GPU; boundary()
// returns the wall right-hand side exactly as the reference forms it.
#ifndef HELMHOLTZ_H
#define HELMHOLTZ_H

#include "afmib_shim.h"
#include "dt/matrix.h"
#include "dt/vector.h"

namespace ns {

template <class Geometry, unsigned int Size, int Comp>
class helmholtz : public dt::matrix<Size> {
  protected:
    double scale;

  public:
    explicit helmholtz(double k) : scale(k) {}
    void apply(const double* x, double* y) const override {
        afmib_solver* s = afmib_shim::context<Geometry>();
        afmib_shim::check(afmib_helm_apply(s, Comp, scale, y, x), s, "ns::helmholtz");
    }
    void relax(double*, const double*) const override {
        throw afmib_shim::error(AFMIB_ERR_ARG, "Gauss-Seidel on the Helmholtz operator is not provided");
    }
    unsigned solve_cg(double* x, const double* b, double tol) const override {
        afmib_solver* s = afmib_shim::context<Geometry>();
        afmib_shim::check(afmib_set_tolerance(s, tol), s, "conjugate_gradient");
        int it = 0;
        afmib_shim::check(afmib_helmholtz_cg(s, Comp, scale, x, b, &it), s, "conjugate_gradient");
        return (unsigned)it;
    }
};

template <class Geometry>
class helmholtz_periodic : public helmholtz<Geometry, Geometry::nx * Geometry::ny * Geometry::nz, 0> {
  public:
    static constexpr unsigned int nx = Geometry::nx;
    static constexpr unsigned int ny = Geometry::ny;
    static constexpr unsigned int nz = Geometry::nz;
    static constexpr unsigned int n = Geometry::n;
    explicit helmholtz_periodic(double k) : helmholtz<Geometry, nx * ny * nz, 0>(k) {}
    // wall right-hand side of the u/w rows, src/ns/helmholtz.h:177-196
    dt::vector<nx * ny * nz> boundary(dt::vector<nx * nz>& top, dt::vector<nx * nz>& bottom) {
        dt::vector<nx * ny * nz> b;
        for (unsigned i = 0; i < nx * nz; ++i) {
            const unsigned x = i % nx, z = i / nx;
            if (ny > 1) {
                b[x + nx * ny * z] = 8. / 3. * this->scale * n * n * bottom[i];
                b[x + nx * (ny - 1 + ny * z)] = 8. / 3. * this->scale * n * n * top[i];
            } else {
                b[x + nx * ny * z] = 3. * n * n * bottom[i];
                b[x + nx * (ny - 1 + ny * z)] = 3. * n * n * top[i];
            }
        }
        return b;
    }
};

template <class Geometry>
class helmholtz_dirichlet : public helmholtz<Geometry, Geometry::nx * (Geometry::ny - 1) * Geometry::nz, 1> {
  public:
    static constexpr unsigned int nx = Geometry::nx;
    static constexpr unsigned int ny = Geometry::ny;
    static constexpr unsigned int nz = Geometry::nz;
    static constexpr unsigned int n = Geometry::n;
    explicit helmholtz_dirichlet(double k) : helmholtz<Geometry, nx * (ny - 1) * nz, 1>(k) {}
    // src/ns/helmholtz.h:321-337
    dt::vector<nx * (ny - 1) * nz> boundary(dt::vector<nx * nz>& top, dt::vector<nx * nz>& bottom) {
        dt::vector<nx * (ny - 1) * nz> b;
        for (unsigned i = 0; i < nx * nz; ++i) {
            const unsigned x = i % nx, z = i / nx;
            b[x + nx * (ny - 1) * z] = this->scale * n * n * bottom[i];
            b[x + nx * (ny - 2 + (ny - 1) * z)] = this->scale * n * n * top[i];
        }
        return b;
    }
};

}  // namespace ns

#endif
