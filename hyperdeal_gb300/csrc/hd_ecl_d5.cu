// hd_ecl_d5.cu -- instantiates the ECL kernels for 5-dimensional phase space
// (dim_x + dim_v = 5), degrees 1..5, FP64 and FP32.  One file per dimension
// keeps the translation units small enough to compile in parallel.
#include "hd_ecl.cuh"

namespace hd {

EclLaunchers ecl_launchers_d5(int N) {
  switch (N) {
    case 2: return make_launchers<5, 2>();
    case 3: return make_launchers<5, 3>();
    case 4: return make_launchers<5, 4>();
    case 5: return make_launchers<5, 5>();
    case 6: return make_launchers<5, 6>();
    default: return EclLaunchers{nullptr, nullptr, 0, 0, 0, 0, 0, 0, false, false};
  }
}

}  // namespace hd
