// Internal support of the C++ header shim: the reference's template API
// (dt::, alg::, mg::, ns::, ib::) rebuilt on the afmib C ABI. A caller keeps
// its #include lines ("dt/geometry.h", "ns/solver.h", ...) and adds
//   -I<repo>/afmibins_gb300/src -I<repo>/include -L<repo>/afmibins_gb300/_lib -lafmib
// Errors the reference never reports (it loops or reads out of range) are
// raised as afmib_shim::error exceptions.
#ifndef AFMIB_SHIM_H
#define AFMIB_SHIM_H

#include <stdexcept>
#include <string>

#include "afmib.h"

namespace afmib_shim {

struct error : std::runtime_error {
    int status;
    error(int st, const std::string& what) : std::runtime_error(what), status(st) {}
};

inline void check(int status, afmib_solver* s, const char* where) {
    if (status != AFMIB_OK) {
        std::string msg = std::string(where) + ": " + afmib_error_string(status);
        if (s) msg += std::string(" (") + afmib_last_error(s) + ")";
        throw error(status, msg);
    }
}

// A solver over the channel grid of a geometry (x, z periodic, walls in y,
// the reference's domain), multigrid depth = the geometry's level.
inline afmib_solver* make_solver(int nx, int ny, int nz, int n, int levels, double tol, int nu1 = 2, int nu2 = 2,
                                 double mu = 0.0, double rho = 1.0, double dt = 1.0) {
    afmib_config c{};
    c.nx = nx;
    c.ny = ny;
    c.nz = nz;
    c.n = n;
    c.bc = AFMIB_BC_CHANNEL;
    c.precision = AFMIB_FP64;
    c.mg_levels = levels;
    c.nu1 = nu1;
    c.nu2 = nu2;
    c.mu = mu;
    c.rho = rho;
    c.dt = dt;
    c.tol = tol;
    c.max_cg_iters = 100000;
    c.max_mg_cycles = 10000;
    afmib_solver* s = nullptr;
    const int st = afmib_create(&c, nullptr, &s);
    if (st != AFMIB_OK) {
        std::string msg = std::string("afmib_create: ") + afmib_error_string(st) + " (" + afmib_last_error(s) + ")";
        afmib_destroy(s);
        throw error(st, msg);
    }
    return s;
}

// One shared solver per geometry for the stateless operators (div, grad,
// Laplacian, Helmholtz apply, transfers, spreading, interpolation). It lives
// until the process exits.
template <class G>
afmib_solver* context() {
    static afmib_solver* s = make_solver(G::nx, G::ny, G::nz, G::n, G::level, 1e-12);
    return s;
}

}  // namespace afmib_shim

#endif
