// hd_ecl_d3.cu -- instantiates the ECL kernels for 3-dimensional phase space
// (dim_x + dim_v = 3), degrees 1..5, FP64 and FP32.  One file per dimension
// keeps the translation units small enough to compile in parallel.
#include "hd_ecl.cuh"

namespace hd {

EclLaunchers ecl_launchers_d3(int N) {
  switch (N) {
    case 2: return make_launchers<3, 2>();
    case 3: return make_launchers<3, 3>();
    case 4: return make_launchers<3, 4>();
    case 5: return make_launchers<3, 5>();
    case 6: return make_launchers<3, 6>();
    default: return EclLaunchers{nullptr, nullptr, 0, 0, 0, 0, 0, 0, false, false};
  }
}

}  // namespace hd
