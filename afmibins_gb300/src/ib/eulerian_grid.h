// ib::eulerian_grid<G, Size>: a field on the grid nodes (i/n, j/n, k/n) with
// cell volume h^3 (src/ib/eulerian_grid.h:30-62). Used by the reference's
// callers as plain field storage; IB transfers run on the MAC grids.
#ifndef IB_EULERIAN_GRID_H
#define IB_EULERIAN_GRID_H

#include "grid.h"

namespace ib {

template <class Geometry, unsigned int Size = Geometry::nx * Geometry::ny * Geometry::nz>
class eulerian_grid : public grid<Geometry, Size> {
  public:
    using grid<Geometry, Size>::n;
    using grid<Geometry, Size>::nx;
    using grid<Geometry, Size>::ny;
    using grid<Geometry, Size>::nz;
    using typename grid<Geometry, Size>::point_type;
    using typename grid<Geometry, Size>::value_type;
    using grid<Geometry, Size>::operator=;

  protected:
    static constexpr unsigned int width = Geometry::width;
    static constexpr unsigned int height = Geometry::height;
    static constexpr unsigned int depth = Geometry::depth;

  public:
    double volume(unsigned int) const override { return 1. / ((double)n * n * n); }
    int point_kind() const override { return kind::node; }
    point_type coordinates(unsigned int index) override {
        return point_type(((double)(index % nx)) / n, ((double)(index % (nx * ny) / nx)) / n,
                          ((double)(index / (nx * ny))) / n, index);
    }
    eulerian_grid(value_type v = value_type()) : grid<Geometry, Size>(v) {}
    eulerian_grid(grid<Geometry, Size>& v) : grid<Geometry, Size>(v) {}
    eulerian_grid(const eulerian_grid& v) : grid<Geometry, Size>(v) {}
    eulerian_grid(std::initializer_list<value_type> v) : grid<Geometry, Size>(v) {}
};

}  // namespace ib

#endif
