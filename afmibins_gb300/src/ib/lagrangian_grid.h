// ib::lagrangian_grid<G, np>: np markers at fixed positions carrying one
// value each; the caller derives from it and supplies volume(i) (the marker's
// area or length element), as with the reference (src/ib/lagrangian_grid.h:33-67).
// No kd-tree is built: the GPU bins markers by a radix sort when they are used.
#ifndef IB_LAGRANGIAN_GRID_H
#define IB_LAGRANGIAN_GRID_H

#include <ostream>
#include <vector>

#include "dt/vector.h"
#include "grid.h"

namespace ib {

template <class Geometry, unsigned int Size>
class lagrangian_grid : public grid<Geometry, Size> {
  public:
    using grid<Geometry, Size>::n;
    static constexpr unsigned int width = Geometry::width;
    static constexpr unsigned int height = Geometry::height;
    static constexpr unsigned int depth = Geometry::depth;
    using typename grid<Geometry, Size>::point_type;
    using typename grid<Geometry, Size>::value_type;
    using grid<Geometry, Size>::operator=;

  private:
    std::vector<point_type> positions;

  public:
    point_type coordinates(unsigned int index) override { return positions[index]; }
    int point_kind() const override { return kind::lagrangian; }

    lagrangian_grid(std::vector<point_type> p, value_type v = value_type()) : grid<Geometry, Size>(v), positions(p) {}
    lagrangian_grid(const lagrangian_grid& g) : grid<Geometry, Size>(g), positions(g.positions) {}
    lagrangian_grid(std::vector<point_type> p, std::initializer_list<value_type> v)
        : grid<Geometry, Size>(v), positions(p) {}
};

}  // namespace ib

#endif
