// ib::grid<G, Size>: a field on a set of points with the immersed-boundary
// transfer target.interpolate(source) (src/ib/grid.h:35-84): spreading when
// the target is a MAC grid and the source Lagrangian markers, interpolation
// in the other direction, both with the cosine 4-point kernel
// phi(r) = n/4 (1 + cos(pi r n / 2)) (src/ib/grid.h:51-55). Here both run on
// the GPU (afmib_spread / afmib_interp) with markers binned by a radix sort;
// spreading includes the periodic images that the reference's kd-tree search
// misses near the x and z faces (src/dt/kdtree.h:82-100).
#ifndef IB_GRID_H
#define IB_GRID_H

#include <cmath>
#include <type_traits>
#include <vector>

#include "afmib_shim.h"
#include "dt/point.h"
#include "dt/vector.h"

// the reference exports this macro from ib/grid.h and its callers use it
#define pi 3.141592653589793238462643383279502884L

namespace ib {

namespace kind {
// what a grid's points are: the three MAC face families, Lagrangian markers,
// or grid nodes
enum { mac_x = 0, mac_y = 1, mac_z = 2, lagrangian = 3, node = 4 };
}

template <class Geometry, unsigned int Size>
class grid : public dt::vector<Size> {
  public:
    static constexpr unsigned int n = Geometry::n;
    static constexpr unsigned int nx = Geometry::nx;
    static constexpr unsigned int ny = Geometry::ny;
    static constexpr unsigned int nz = Geometry::nz;
    typedef Geometry geometry_type;
    typedef dt::point point_type;
    typedef typename point_type::value_type coordinate_type;
    using typename dt::vector<Size>::value_type;

    virtual point_type coordinates(unsigned int) = 0;
    virtual double volume(unsigned int) const = 0;
    virtual int point_kind() const = 0;
    virtual double delta_function(coordinate_type r) {
        if (std::fabs(n * r) > 2.) return 0;
        return 0.25 * n * (1 + std::cos((double)(pi * r * n / 2)));
    }

    template <unsigned int R>
    void interpolate(grid<Geometry, R>& source);

    grid(const grid& g) : dt::vector<Size>(g) {}
    grid(dt::vector<Size>& v) : dt::vector<Size>(v) {}
    grid(value_type v = 0.0) : dt::vector<Size>(v) {}
    grid(std::initializer_list<value_type> v) : dt::vector<Size>(v) {}
    using dt::vector<Size>::operator[];
    using dt::vector<Size>::operator=;

    template <class, unsigned int>
    friend class grid;
};

template <class Geometry, unsigned int Size>
template <unsigned int R>
void grid<Geometry, Size>::interpolate(grid<Geometry, R>& source) {
    afmib_solver* s = afmib_shim::context<Geometry>();
    const int tk = point_kind(), sk = source.point_kind();
    constexpr unsigned NC = Geometry::nx * Geometry::ny * Geometry::nz;
    constexpr unsigned NV = Geometry::nx * (Geometry::ny - 1) * Geometry::nz;
    if (tk <= kind::mac_z && sk == kind::lagrangian) {
        // spreading: f = sum_k phi^3 vol_k F_k onto this face family
        std::vector<double> X(3 * R), F(3 * R, 0.0), vol(R);
        for (unsigned k = 0; k < R; ++k) {
            const point_type p = source.coordinates(k);
            X[3 * k] = p[0];
            X[3 * k + 1] = p[1];
            X[3 * k + 2] = p[2];
            vol[k] = source.volume(k);
            F[(size_t)tk * R + k] = source[k];
        }
        std::vector<double> fx(NC), fy(NV), fz(NC);
        afmib_shim::check(afmib_spread(s, (int)R, X.data(), F.data(), vol.data(), fx.data(), fy.data(), fz.data()), s,
                          "ib::grid::interpolate (spread)");
        const std::vector<double>& out = tk == kind::mac_x ? fx : (tk == kind::mac_y ? fy : fz);
        for (unsigned i = 0; i < Size; ++i) (*this)[i] = out[i];
        return;
    }
    if (tk == kind::lagrangian && sk <= kind::mac_z) {
        // interpolation: U_k = sum phi^3 h^3 u(face) from this face family
        std::vector<double> X(3 * Size), f[3] = {std::vector<double>(NC, 0.0), std::vector<double>(NV, 0.0),
                                                 std::vector<double>(NC, 0.0)};
        for (unsigned k = 0; k < Size; ++k) {
            const point_type p = coordinates(k);
            X[3 * k] = p[0];
            X[3 * k + 1] = p[1];
            X[3 * k + 2] = p[2];
        }
        for (unsigned i = 0; i < R; ++i) f[sk][i] = source[i];
        std::vector<double> U(3 * (size_t)Size);
        afmib_shim::check(afmib_interp(s, (int)Size, X.data(), f[0].data(), f[1].data(), f[2].data(), U.data()), s,
                          "ib::grid::interpolate (interp)");
        for (unsigned k = 0; k < Size; ++k) (*this)[k] = U[(size_t)sk * Size + k];
        return;
    }
    throw afmib_shim::error(AFMIB_ERR_ARG, "ib::grid::interpolate: the GPU transfers run between MAC grids and "
                                           "Lagrangian markers");
}

}  // namespace ib

#endif
