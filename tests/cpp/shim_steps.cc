// Drives the C++ header shim the way the reference's own test programs drive
// the reference (test/ns_test.cc, test/ib_test.cc, test/mg_test2.cc): reads a
// binary case, runs it through the reference's template API on the GPU and
// writes the results for the Python test to compare with the golden vectors.
//   shim_steps ns  <in.bin> <out.bin>   16^3 channel: 4 NS sub-steps
//   shim_steps mg  <in.bin> <out.bin>   16^3 channel: mg::solver::solve
//   shim_steps ib  <in.bin> <out.bin>   16^3 channel: spread + interp, 320 markers
#include <cstdio>
#include <string>
#include <vector>

#include "alg/cg.h"
#include "alg/div.h"
#include "alg/grad.h"
#include "dt/geometry.h"
#include "ib/lagrangian_grid.h"
#include "ib/mac_grid.h"
#include "mg/solver.h"
#include "ns/solver.h"

typedef dt::geometry<4u, 1u, 1u, 1u> G;
constexpr unsigned NC = G::nx * G::ny * G::nz, NV = G::nx * (G::ny - 1) * G::nz, NXZ = G::nx * G::nz, NM = 320;

static std::vector<double> in, out;
static size_t cur = 0;
static double take() { return in.at(cur++); }
template <unsigned S>
static void take(dt::vector<S>& v) { for (unsigned i = 0; i < S; ++i) v[i] = take(); }
template <unsigned S>
static void put(const dt::vector<S>& v) { for (unsigned i = 0; i < S; ++i) out.push_back(v[i]); }

class markers : public ib::lagrangian_grid<G, NM> {
  public:
    std::vector<double> vol;
    markers(std::vector<dt::point> p, std::vector<double> v) : ib::lagrangian_grid<G, NM>(p), vol(v) {}
    double volume(unsigned i) const override { return vol[i]; }
};

int main(int argc, char** argv) {
    if (argc != 4) return 2;
    {
        FILE* f = std::fopen(argv[2], "rb");
        if (!f) return 2;
        std::fseek(f, 0, SEEK_END);
        long b = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        in.resize(b / 8);
        if (std::fread(in.data(), 8, in.size(), f) != in.size()) return 2;
        std::fclose(f);
    }
    const std::string cmd = argv[1];
    try {
        if (cmd == "ns") {
            double mu = take(), rho = take(), dt = take(), tol = take();
            unsigned sub = (unsigned)take();
            dt::vector<NC> u0, w0, fx, fz;
            dt::vector<NV> v0, fy;
            dt::vector<NXZ> ut, ub, wt, wb;
            take(u0); take(v0); take(w0);
            take(fx); take(fy); take(fz);
            ns::solver<G> s(mu, rho, dt, tol, u0, v0, w0);
            for (unsigned k = 0; k < sub; ++k) s.step(ut, ub, wt, wb, fx, fy, fz);
            put(u0); put(v0); put(w0); put(s.get_p());
            put(ut); put(ub); put(wt); put(wb);
        } else if (cmd == "mg") {
            double tol = take();
            dt::vector<NC> b;
            take(b);
            mg::solver<G> s(tol, 2, 2);
            unsigned c = s.solve(b);
            out.push_back(c);
            put(b);
        } else if (cmd == "ib") {
            std::vector<dt::point> pts;
            for (unsigned i = 0; i < NM; ++i) {
                double x = take(), y = take(), z = take();
                pts.push_back(dt::point(x, y, z, i));
            }
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
            ib::mac_grid<G, ib::mac::x> ue;
            ib::mac_grid<G, ib::mac::y> ve;
            ib::mac_grid<G, ib::mac::z> we;
            take(ue); take(ve); take(we);
            lx.interpolate(ue); ly.interpolate(ve); lz.interpolate(we);
            put(lx); put(ly); put(lz);
        } else {
            return 2;
        }
    } catch (const afmib_shim::error& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 3;
    }
    FILE* f = std::fopen(argv[3], "wb");
    if (!f) return 2;
    std::fwrite(out.data(), 8, out.size(), f);
    std::fclose(f);
    return 0;
}
