// ib::mac_grid<G, ib::mac::x/y/z>: a velocity or force component on its MAC
// faces — the component's own axis on integer positions, the other two on
// half-integers; v on the ny-1 interior y faces (src/ib/mac_grid.h:30-136).
#ifndef IB_MAC_GRID_H
#define IB_MAC_GRID_H

#include "eulerian_grid.h"

namespace ib {

namespace mac {
enum component { x, y, z };
}

template <class Geometry, mac::component Component>
class mac_grid : public eulerian_grid<Geometry, Geometry::nx * Geometry::ny * Geometry::nz> {
  private:
    static constexpr unsigned int Size = Geometry::nx * Geometry::ny * Geometry::nz;

  public:
    using eulerian_grid<Geometry, Size>::n;
    using typename eulerian_grid<Geometry, Size>::point_type;
    using typename eulerian_grid<Geometry, Size>::value_type;
    using eulerian_grid<Geometry, Size>::operator=;
    int point_kind() const override { return (int)Component; }
    point_type coordinates(unsigned int i) override {
        point_type p = eulerian_grid<Geometry, Size>::coordinates(i);
        p[(Component + 1) % 3] += 0.5 / n;
        p[(Component + 2) % 3] += 0.5 / n;
        return p;
    }
    mac_grid(value_type v = value_type()) : eulerian_grid<Geometry, Size>(v) {}
    mac_grid(std::initializer_list<value_type> v) : eulerian_grid<Geometry, Size>(v) {}
};

template <class Geometry>
class mac_grid<Geometry, mac::y> : public eulerian_grid<Geometry, Geometry::nx * (Geometry::ny - 1) * Geometry::nz> {
  private:
    static constexpr unsigned int Size = Geometry::nx * (Geometry::ny - 1) * Geometry::nz;

  public:
    using eulerian_grid<Geometry, Size>::nx;
    using eulerian_grid<Geometry, Size>::ny;
    using eulerian_grid<Geometry, Size>::n;
    using typename eulerian_grid<Geometry, Size>::point_type;
    using typename eulerian_grid<Geometry, Size>::value_type;
    using eulerian_grid<Geometry, Size>::operator=;
    int point_kind() const override { return (int)mac::y; }
    point_type coordinates(unsigned int i) override {
        return point_type(((double)(i % nx) + 0.5) / n, ((double)(i / nx % (ny - 1)) + 1.0) / n,
                          ((double)(i / (nx * (ny - 1))) + 0.5) / n, i);
    }
    mac_grid(value_type v = value_type()) : eulerian_grid<Geometry, Size>(v) {}
    mac_grid(std::initializer_list<value_type> v) : eulerian_grid<Geometry, Size>(v) {}
};

}  // namespace ib

#endif
