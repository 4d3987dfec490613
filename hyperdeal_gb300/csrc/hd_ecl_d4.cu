// hd_ecl_d4.cu -- instantiates the ECL kernels for 4-dimensional phase space
// (dim_x + dim_v = 4), degrees 1..5, FP64 and FP32.  One file per dimension
// keeps the translation units small enough to compile in parallel.
#include "hd_ecl.cuh"

namespace hd {

EclLaunchers ecl_launchers_d4(int N) {
  switch (N) {
    case 2: return make_launchers<4, 2>();
    case 3: return make_launchers<4, 3>();
    case 4: return make_launchers<4, 4>();
    case 5: return make_launchers<4, 5>();
    case 6: return make_launchers<4, 6>();
    default: return EclLaunchers{nullptr, nullptr, 0, 0, 0, 0, 0, 0, false, false};
  }
}

}  // namespace hd
