// ns::solver<G>(mu, rho, k, tol, u0, v0, w0): the incompressible Navier–Stokes
// stepper of the reference (src/ns/solver.h:37-140). Like the reference it
// keeps references to the caller's u0, v0, w0, projects them on construction,
// and each step(ut, ub, wt, wb, fx, fy, fz) advances them in place — the BE
// half step and the CN step alternately — and updates the caller's wall
// vectors. The whole step (advection, three Helmholtz CG solves, the multigrid
// projection) runs on the GPU; the fields are copied back after every call.
#ifndef NAVIERSTOKES_H
#define NAVIERSTOKES_H

#include "afmib_shim.h"
#include "dt/geometry.h"
#include "dt/vector.h"
#include "helmholtz.h"
#include "projection.h"

namespace ns {

template <class Geometry>
class solver {
  private:
    static constexpr unsigned n = Geometry::n;
    static constexpr unsigned nx = Geometry::nx;
    static constexpr unsigned ny = Geometry::ny;
    static constexpr unsigned nz = Geometry::nz;
    afmib_solver* s;
    dt::vector<nx * ny * nz>& u_curr;
    dt::vector<nx * (ny - 1) * nz>& v_curr;
    dt::vector<nx * ny * nz>& w_curr;

  public:
    solver(double mu, double rho, double k, double tol, dt::vector<nx * ny * nz>& u0,
           dt::vector<nx * (ny - 1) * nz>& v0, dt::vector<nx * ny * nz>& w0)
        : s(afmib_shim::make_solver(nx, ny, nz, n, Geometry::level, tol, 2, 2, mu, rho, k)),
          u_curr(u0), v_curr(v0), w_curr(w0) {
        afmib_shim::check(afmib_set_velocity(s, u0.data(), v0.data(), w0.data()), s, "ns::solver");
        afmib_shim::check(afmib_project(s), s, "ns::solver");
        afmib_shim::check(afmib_get_velocity(s, u0.data(), v0.data(), w0.data()), s, "ns::solver");
    }
    solver(const solver&) = delete;
    solver& operator=(const solver&) = delete;
    ~solver() { afmib_destroy(s); }

    void step(dt::vector<nx * nz>& ut, dt::vector<nx * nz>& ub, dt::vector<nx * nz>& wt, dt::vector<nx * nz>& wb,
              dt::vector<nx * ny * nz>& fx, dt::vector<nx * (ny - 1) * nz>& fy, dt::vector<nx * ny * nz>& fz) {
        afmib_shim::check(afmib_set_walls(s, ut.data(), ub.data(), wt.data(), wb.data()), s, "ns::solver::step");
        afmib_shim::check(afmib_ns_step(s, fx.data(), fy.data(), fz.data()), s, "ns::solver::step");
        afmib_shim::check(afmib_get_walls(s, ut.data(), ub.data(), wt.data(), wb.data()), s, "ns::solver::step");
        afmib_shim::check(afmib_get_velocity(s, u_curr.data(), v_curr.data(), w_curr.data()), s, "ns::solver::step");
    }

    const dt::vector<nx * ny * nz>& get_u() { return u_curr; }
    const dt::vector<nx * (ny - 1) * nz>& get_v() { return v_curr; }
    const dt::vector<nx * ny * nz>& get_w() { return w_curr; }
    const dt::vector<nx * ny * nz> get_p() {
        dt::vector<nx * ny * nz> p;
        afmib_shim::check(afmib_get_pressure(s, p.data()), s, "ns::solver::get_p");
        return p;
    }
};

}  // namespace ns

#endif
