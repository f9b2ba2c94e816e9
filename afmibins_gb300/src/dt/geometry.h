// dt::geometry<Level, Width, Height, Depth>: the compile-time grid hierarchy of
// the reference (src/dt/geometry.h:29-60) — n = 2^Level cells per unit length,
// nx = Width*n, ny = Height*n, nz = Depth*n; coarse/fine drive the multigrid
// depth. The same names and values, so that geometry-templated callers compile
// unchanged against the GPU shim.
#ifndef DT_GEOMETRY_H
#define DT_GEOMETRY_H

#include "vector.h"

namespace dt {

template <unsigned Level, unsigned Width, unsigned Height, unsigned Depth>
class geometry {
  public:
    typedef geometry<Level - 1, Width, Height, Depth> coarse;
    typedef geometry<Level + 1, Width, Height, Depth> fine;
    static constexpr unsigned factor = 2;
    static constexpr unsigned n = coarse::n * factor;
    static constexpr unsigned nx = Width * n;
    static constexpr unsigned ny = Height * n;
    static constexpr unsigned nz = Depth * n;
    static constexpr unsigned size = nx * ny * nz;
    static constexpr unsigned width = Width;
    static constexpr unsigned height = Height;
    static constexpr unsigned depth = Depth;
    static constexpr unsigned level = Level;
};

template <unsigned Width, unsigned Height, unsigned Depth>
class geometry<0u, Width, Height, Depth> {
  public:
    typedef geometry<1u, Width, Height, Depth> fine;
    static constexpr unsigned factor = 2;
    static constexpr unsigned n = 1;
    static constexpr unsigned nx = Width;
    static constexpr unsigned ny = Height;
    static constexpr unsigned nz = Depth;
    static constexpr unsigned size = nx * ny * nz;
    static constexpr unsigned width = Width;
    static constexpr unsigned height = Height;
    static constexpr unsigned depth = Depth;
    static constexpr unsigned level = 0u;
};

}  // namespace dt

#endif
