// kernels3d_s84.cu -- the 3D sweep kernels of tile shape 8x4x32 (kernels3d_tiles.cuh), compiled
// beside kernels3d.cu (shape 4x8x32).

#include "kernels3d_tiles.cuh"

namespace pfast {

template struct ShapeLaunchers<Shape84>;

}  // namespace pfast
