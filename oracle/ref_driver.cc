// TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
//
// Drives the reference headers (best-of-both/afmibins src/, included
// unchanged through -I<reference>/src) on inputs read from a binary file and
// writes the results to another, so that the CPU restatement in
// oracle/restated/ and the golden vectors in tests/golden/ can be pinned to
// the reference itself. Grid sizes are compile-time in the reference
// (src/dt/geometry.h:29-44), so one binary is built per (level, W, H, D, M):
//   -DAFMIB_L=<level> -DAFMIB_W=.. -DAFMIB_H=.. -DAFMIB_D=.. -DAFMIB_M=<markers>
//
// Usage: ref_driver <command> <input.bin> <output.bin>
// Every input file is a flat array of float64; layouts are listed per command.
//
// The reference keeps several members private/protected (the restriction,
// the level Laplacian, the advection term); the driver opens them with the
// preprocessor before the includes so that they can be exercised one by one.

#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <iterator>
#include <memory>
#include <ostream>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

// standard headers first, so that only the reference's own classes are opened
#define private public
#define protected public
#include "dt/geometry.h"
#include "dt/vector.h"
#include "dt/point.h"
#include "alg/div.h"
#include "alg/grad.h"
#include "alg/cg.h"
#include "mg/solver.h"
#include "ns/solver.h"
#include "ns/helmholtz.h"
#include "ib/eulerian_grid.h"
#include "ib/mac_grid.h"
#include "ib/lagrangian_grid.h"
#undef private
#undef protected

#ifndef AFMIB_L
#define AFMIB_L 4
#endif
#ifndef AFMIB_W
#define AFMIB_W 1
#endif
#ifndef AFMIB_H
#define AFMIB_H 1
#endif
#ifndef AFMIB_D
#define AFMIB_D 1
#endif
#ifndef AFMIB_M
#define AFMIB_M 256
#endif

typedef dt::geometry<AFMIB_L, AFMIB_W, AFMIB_H, AFMIB_D> G;
constexpr unsigned NX = G::nx, NY = G::ny, NZ = G::nz, NN = G::n;
constexpr unsigned NC = NX * NY * NZ, NV = NX * (NY - 1) * NZ, NXZ = NX * NZ;
constexpr unsigned NM = AFMIB_M;

static std::vector<double> in;
static size_t cursor = 0;
static std::vector<double> out;

static double take() {
    if (cursor >= in.size()) { std::fprintf(stderr, "input too short\n"); std::exit(2); }
    return in[cursor++];
}
template <unsigned S> static void take(dt::vector<S>& v) { for (unsigned i = 0; i < S; ++i) v[i] = take(); }
template <unsigned S> static void put(const dt::vector<S>& v) { for (unsigned i = 0; i < S; ++i) out.push_back(v[i]); }
static void put(double x) { out.push_back(x); }

// Lagrangian markers with per-marker volume (the reference leaves volume()
// to the user, src/ib/lagrangian_grid.h:33-56, test/ib_test.cc:33-58).
class markers : public ib::lagrangian_grid<G, NM> {
  public:
    std::vector<double> vol;
    markers(std::vector<dt::point> p, std::vector<double> v) : ib::lagrangian_grid<G, NM>(p), vol(v) {}
    double volume(unsigned i) const { return vol[i]; }
    markers& operator=(double v) { for (auto& e : *this) e = v; return *this; }
};

static std::vector<dt::point> read_points(unsigned m) {
    std::vector<dt::point> p;
    for (unsigned i = 0; i < NM; ++i) {
        double x = take(), y = take(), z = take();
        p.push_back(dt::point(x, y, z, i));
    }
    (void)m;
    return p;
}

int main(int argc, char** argv) {
    if (argc != 4) { std::fprintf(stderr, "usage: %s cmd in out\n", argv[0]); return 2; }
    const std::string cmd = argv[1];
    {
        FILE* f = std::fopen(argv[2], "rb");
        if (!f) { std::perror("input"); return 2; }
        std::fseek(f, 0, SEEK_END);
        long bytes = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        in.resize(bytes / sizeof(double));
        if (std::fread(in.data(), sizeof(double), in.size(), f) != in.size()) return 2;
        std::fclose(f);
    }

    if (cmd == "info") {
        put(NX); put(NY); put(NZ); put(NN); put(NM);
    } else if (cmd == "mg") {
        // in: tol, nu1, nu2, rhs[NC]   out: cycles, x[NC]
        double tol = take();
        unsigned nu1 = (unsigned)take(), nu2 = (unsigned)take();
        dt::vector<NC> b;
        take(b);
        mg::solver<G> s(tol, nu1, nu2);
        unsigned c = s.solve(b);
        put(c); put(b);
    } else if (cmd == "restrict") {
        // in: fine[NC]  out: coarse[NC/8]
        dt::vector<NC> f;
        take(f);
        dt::vector<NC / 8> c;
        mg::solver<G>::restriction(c, f);
        put(c);
    } else if (cmd == "prolong") {
        // in: coarse[NC/8]  out: fine[NC]
        dt::vector<NC / 8> c;
        take(c);
        dt::vector<NC> f;
        mg::solver<G>::interpolation(f, c);
        put(f);
    } else if (cmd == "lap") {
        // in: x[NC]  out: L x
        dt::vector<NC> x;
        take(x);
        put(mg::solver<G>::L * x);
    } else if (cmd == "gs") {
        // in: x[NC], b[NC]  out: x after one sweep
        dt::vector<NC> x, b;
        take(x); take(b);
        alg::smooth(x, mg::solver<G>::L, b);
        put(x);
    } else if (cmd == "helm") {
        // in: s, u[NC], v[NV], w[NC]  out: Hu, Hv, Hw, bdy_u(top=1,bottom=2)
        double s = take();
        dt::vector<NC> u, w;
        dt::vector<NV> v;
        take(u); take(v); take(w);
        ns::helmholtz_periodic<G> hp(s);
        ns::helmholtz_dirichlet<G> hd(s);
        put(hp * u); put(hd * v); put(hp * w);
        dt::vector<NXZ> top(1.0), bot(2.0);
        put(hp.boundary(top, bot));
    } else if (cmd == "cg") {
        // in: s, tol, x0[NC], b[NC]   out: iters, x[NC]
        double s = take(), tol = take();
        dt::vector<NC> x, b;
        take(x); take(b);
        ns::helmholtz_periodic<G> hp(s);
        unsigned it = alg::conjugate_gradient(x, hp, b, tol);
        put(it); put(x);
    } else if (cmd == "div") {
        // in: u[NC], v[NV], w[NC], top[NXZ], bottom[NXZ]  out: d[NC]
        dt::vector<NC> u, w, d;
        dt::vector<NV> v;
        dt::vector<NXZ> t, b;
        take(u); take(v); take(w); take(t); take(b);
        alg::div<NX, NY, NZ, NN>(d, u, v, w, t, b);
        put(d);
    } else if (cmd == "grad") {
        // in: p[NC]  out: px[NC], py[NV], pz[NC]
        dt::vector<NC> p, px, pz;
        dt::vector<NV> py;
        take(p);
        alg::grad<NX, NY, NZ, NN>(px, py, pz, p);
        put(px); put(py); put(pz);
    } else if (cmd == "ns") {
        // in: mu, rho, dt, tol, substeps, u0[NC], v0[NV], w0[NC],
        //     ut, ub, wt, wb [NXZ each], fx[NC], fy[NV], fz[NC]
        // out: u, v, w, p, ut, ub, wt, wb
        double mu = take(), rho = take(), dt_ = take(), tol = take();
        unsigned sub = (unsigned)take();
        dt::vector<NC> u0, w0, fx, fz;
        dt::vector<NV> v0, fy;
        dt::vector<NXZ> ut, ub, wt, wb;
        take(u0); take(v0); take(w0);
        take(ut); take(ub); take(wt); take(wb);
        take(fx); take(fy); take(fz);
        ns::solver<G> s(mu, rho, dt_, tol, u0, v0, w0);
        for (unsigned k = 0; k < sub; ++k) s.step(ut, ub, wt, wb, fx, fy, fz);
        put(u0); put(v0); put(w0); put(s.get_p());
        put(ut); put(ub); put(wt); put(wb);
    } else if (cmd == "advect") {
        // in: u[NC], v[NV], w[NC]  out: ua, va, wa
        dt::vector<NC> u, w;
        dt::vector<NV> v;
        take(u); take(v); take(w);
        dt::vector<NC> zu, zw;
        dt::vector<NV> zv;
        ns::solver<G> s(1.0, 1.0, 1.0, 1e-8, zu, zv, zw);
        s.advection(u, v, w);
        put(s.u_adv); put(s.v_adv); put(s.w_adv);
    } else if (cmd == "spread") {
        // in: X[NM*3], vol[NM], Fx[NM], Fy[NM], Fz[NM]  out: fx[NC], fy[NV], fz[NC]
        auto pts = read_points(NM);
        std::vector<double> vol(NM);
        for (auto& e : vol) e = take();
        markers lx(pts, vol), ly(pts, vol), lz(pts, vol);
        for (unsigned i = 0; i < NM; ++i) lx[i] = take();
        for (unsigned i = 0; i < NM; ++i) ly[i] = take();
        for (unsigned i = 0; i < NM; ++i) lz[i] = take();
        ib::mac_grid<G, ib::mac::x> fx;
        ib::mac_grid<G, ib::mac::y> fy;
        ib::mac_grid<G, ib::mac::z> fz;
        fx.interpolate(lx); fy.interpolate(ly); fz.interpolate(lz);
        put(fx); put(fy); put(fz);
    } else if (cmd == "interp") {
        // in: X[NM*3], u[NC], v[NV], w[NC]  out: U[NM], V[NM], W[NM]
        auto pts = read_points(NM);
        std::vector<double> vol(NM, 1.0);
        ib::mac_grid<G, ib::mac::x> u;
        ib::mac_grid<G, ib::mac::y> v;
        ib::mac_grid<G, ib::mac::z> w;
        take(u); take(v); take(w);
        markers lx(pts, vol), ly(pts, vol), lz(pts, vol);
        lx.interpolate(u); ly.interpolate(v); lz.interpolate(w);
        for (unsigned i = 0; i < NM; ++i) put(lx[i]);
        for (unsigned i = 0; i < NM; ++i) put(ly[i]);
        for (unsigned i = 0; i < NM; ++i) put(lz[i]);
    } else if (cmd == "ib" || cmd == "ibw") {
        // The immersed-boundary step the reference leaves as comments in
        // test/ib_ns_test.cc:73-96, assembled from the reference pieces
        // (ns::solver::step, ib::grid::interpolate) plus linear springs.
        // in: mu, rho, dt, tol, k, nsteps, u0[NC], v0[NV], w0[NC], X[NM*3],
        //     deg[NM], nbr[NM*6] (unused slots -1)
        //     ibw: then the wall velocities ut, ub, wt, wb [NXZ each]
        // out: u, v, w, p, X[NM*3]; ibw: then ut, ub, wt, wb
        double mu = take(), rho = take(), dt_ = take(), tol = take(), k = take();
        unsigned nsteps = (unsigned)take();
        dt::vector<NC> u0, w0;
        dt::vector<NV> v0;
        take(u0); take(v0); take(w0);
        std::vector<double> X(3 * NM);
        for (auto& e : X) e = take();
        std::vector<int> deg(NM), nbr(6 * NM);
        for (auto& e : deg) e = (int)take();
        for (auto& e : nbr) e = (int)take();
        dt::vector<NXZ> ut, ub, wt, wb;
        if (cmd == "ibw") { take(ut); take(ub); take(wt); take(wb); }
        ns::solver<G> s(mu, rho, dt_, tol, u0, v0, w0);
        std::vector<double> ones(NM, 1.0);
        auto points = [&](const std::vector<double>& P) {
            std::vector<dt::point> p;
            for (unsigned i = 0; i < NM; ++i) p.push_back(dt::point(P[3 * i], P[3 * i + 1], P[3 * i + 2], i));
            return p;
        };
        auto spread_forces = [&](const std::vector<double>& P, ib::mac_grid<G, ib::mac::x>& fx,
                                 ib::mac_grid<G, ib::mac::y>& fy, ib::mac_grid<G, ib::mac::z>& fz) {
            auto pts = points(P);
            markers lx(pts, ones), ly(pts, ones), lz(pts, ones);
            for (unsigned i = 0; i < NM; ++i) {
                double g[3] = {0, 0, 0};
                for (int e = 0; e < deg[i]; ++e) {
                    int j = nbr[6 * i + e];
                    for (int a = 0; a < 3; ++a) g[a] += P[3 * j + a] - P[3 * i + a];
                }
                lx[i] = k * g[0]; ly[i] = k * g[1]; lz[i] = k * g[2];
            }
            fx.interpolate(lx); fy.interpolate(ly); fz.interpolate(lz);
        };
        auto velocity = [&](const std::vector<double>& P, std::vector<double>& U) {
            auto pts = points(P);
            markers lx(pts, ones), ly(pts, ones), lz(pts, ones);
            ib::mac_grid<G, ib::mac::x> eu; ib::mac_grid<G, ib::mac::y> ev; ib::mac_grid<G, ib::mac::z> ew;
            for (unsigned i = 0; i < NC; ++i) eu[i] = u0[i];
            for (unsigned i = 0; i < NV; ++i) ev[i] = v0[i];
            for (unsigned i = 0; i < NC; ++i) ew[i] = w0[i];
            lx.interpolate(eu); ly.interpolate(ev); lz.interpolate(ew);
            for (unsigned i = 0; i < NM; ++i) { U[3 * i] = lx[i]; U[3 * i + 1] = ly[i]; U[3 * i + 2] = lz[i]; }
        };
        std::vector<double> U1(3 * NM), U2(3 * NM), Xh(3 * NM);
        for (unsigned st = 0; st < nsteps; ++st) {
            {
                ib::mac_grid<G, ib::mac::x> fx; ib::mac_grid<G, ib::mac::y> fy; ib::mac_grid<G, ib::mac::z> fz;
                spread_forces(X, fx, fy, fz);
                s.step(ut, ub, wt, wb, fx, fy, fz);
            }
            velocity(X, U1);
            for (unsigned i = 0; i < 3 * NM; ++i) Xh[i] = X[i] + dt_ / 2 * U1[i];
            velocity(Xh, U2);
            {
                ib::mac_grid<G, ib::mac::x> fx; ib::mac_grid<G, ib::mac::y> fy; ib::mac_grid<G, ib::mac::z> fz;
                spread_forces(Xh, fx, fy, fz);
                s.step(ut, ub, wt, wb, fx, fy, fz);
            }
            for (unsigned i = 0; i < 3 * NM; ++i) X[i] = X[i] + dt_ * U2[i];
        }
        put(u0); put(v0); put(w0); put(s.get_p());
        for (double e : X) put(e);
        if (cmd == "ibw") { put(ut); put(ub); put(wt); put(wb); }
    } else {
        std::fprintf(stderr, "unknown command %s\n", cmd.c_str());
        return 2;
    }

    FILE* f = std::fopen(argv[3], "wb");
    if (!f) { std::perror("output"); return 2; }
    std::fwrite(out.data(), sizeof(double), out.size(), f);
    std::fclose(f);
    return 0;
}
