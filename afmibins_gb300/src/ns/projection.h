// ns::projection<G>(tol): pressure projection u -= grad(phi), L phi = div u
// (src/ns/projection.h:32-73), on the GPU. get_phidt() returns the last phi.
#ifndef NS_PROJECTION_H
#define NS_PROJECTION_H

#include "afmib_shim.h"
#include "dt/vector.h"
#include "mg/solver.h"

namespace ns {

template <class Geometry>
class projection {
  private:
    static constexpr unsigned n = Geometry::n;
    static constexpr unsigned nx = Geometry::nx;
    static constexpr unsigned ny = Geometry::ny;
    static constexpr unsigned nz = Geometry::nz;
    afmib_solver* s;
    dt::vector<nx * ny * nz> phidt;

  public:
    explicit projection(double tol) : s(afmib_shim::make_solver(nx, ny, nz, n, Geometry::level, tol)) {}
    projection(const projection&) = delete;
    projection& operator=(const projection&) = delete;
    ~projection() { afmib_destroy(s); }

    void project(dt::vector<nx * ny * nz>& u, dt::vector<nx * (ny - 1) * nz>& v, dt::vector<nx * ny * nz>& w) {
        afmib_shim::check(afmib_set_velocity(s, u.data(), v.data(), w.data()), s, "projection");
        afmib_shim::check(afmib_project(s), s, "projection");
        afmib_shim::check(afmib_get_velocity(s, u.data(), v.data(), w.data()), s, "projection");
        // phi from the (I - s Delta) phi pressure with s = 0: the solver was made with mu = 0
        afmib_shim::check(afmib_get_pressure(s, phidt.data()), s, "projection");
    }
    dt::vector<nx * ny * nz>& get_phidt() { return phidt; }
};

}  // namespace ns

#endif
