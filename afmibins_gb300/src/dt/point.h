// dt::point: a position (x, y, z) with an index, the reference's marker and
// node coordinate type (src/dt/point.h:29-54).
#ifndef DT_POINT_H
#define DT_POINT_H

#include <cstddef>
#include <ostream>

namespace dt {

class point {
  public:
    typedef double value_type;
    typedef value_type& reference;
    typedef const value_type& const_reference;
    typedef std::size_t size_type;

  private:
    value_type values[3];
    size_type idx;

  public:
    point(value_type x, value_type y, value_type z, const size_type index) : values{x, y, z}, idx(index) {}
    point() : values{0.0, 0.0, 0.0}, idx(0) {}
    reference operator[](size_type i) { return values[i]; }
    const_reference operator[](size_type i) const { return values[i]; }
    size_type get_index() const { return idx; }
};

inline std::ostream& operator<<(std::ostream& out, const point& p) {
    return out << p.get_index() << " (" << p[0] << ", " << p[1] << ", " << p[2] << ")";
}

}  // namespace dt

#endif
