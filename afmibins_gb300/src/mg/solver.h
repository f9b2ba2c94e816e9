// mg::solver<G>(tol, nu1, nu2): geometric multigrid for the pressure Poisson
// problem, src/mg/solver.h:35-271. solve(rhs) removes the mean of rhs, cycles
// V(nu1, nu2) until the RMS residual is at most tol and overwrites rhs with
// the solution, returning the cycle count — on the GPU (afmib_mg_solve) with
// red-black smoothing and the reference's restriction and prolongation. The
// static members L, restriction and interpolation keep the reference's names.
#ifndef MG_MULTIGRID_H
#define MG_MULTIGRID_H

#include "afmib_shim.h"
#include "dt/geometry.h"
#include "dt/vector.h"
#include "laplacian.h"

namespace mg {

template <class Geometry, unsigned Level = Geometry::level>
class solver {
  public:
    static constexpr unsigned n = Geometry::n;
    static constexpr unsigned nx = Geometry::nx;
    static constexpr unsigned ny = Geometry::ny;
    static constexpr unsigned nz = Geometry::nz;
    typedef Geometry geometry_type;
    typedef laplacian<geometry_type> laplacian_type;

  private:
    afmib_solver* s;

  protected:
    static laplacian_type L;
    static void interpolation(dt::vector<nx * ny * nz>& fine, dt::vector<nx * ny * nz / 8>& coarse) {
        afmib_solver* c = afmib_shim::context<Geometry>();
        afmib_shim::check(afmib_prolong(c, fine.data(), coarse.data()), c, "mg::solver::interpolation");
    }
    static void restriction(dt::vector<nx * ny * nz / 8>& coarse, dt::vector<nx * ny * nz>& fine) {
        afmib_solver* c = afmib_shim::context<Geometry>();
        afmib_shim::check(afmib_restrict(c, coarse.data(), fine.data()), c, "mg::solver::restriction");
    }

  public:
    solver(double tol, unsigned int nu1, unsigned int nu2)
        : s(afmib_shim::make_solver(nx, ny, nz, n, Level, tol, (int)nu1, (int)nu2)) {}
    solver(const solver&) = delete;
    solver& operator=(const solver&) = delete;
    ~solver() { afmib_destroy(s); }

    unsigned int solve(dt::vector<nx * ny * nz>& rhs) {
        int cycles = 0;
        afmib_shim::check(afmib_mg_solve(s, rhs.data(), &cycles), s, "mg::solver::solve");
        return (unsigned)cycles;
    }
};

template <class Geometry, unsigned Level>
laplacian<Geometry> solver<Geometry, Level>::L;

}  // namespace mg

#endif
