// hd_dispatch.cu -- (dimension, nodes per direction) -> kernel launchers.
//
// Every (D, N) pair is instantiated in its own small translation unit,
// generated at build time by hyperdeal_gb300/build.py (ecl_<D>_<N>.cu for
// the single-instance kernels of hd_ecl.cuh, batch_<D>_<N>.cu for the batch
// kernels of hd_batch.cuh, gauss_<D>_<N>.cu for the Gauss-quadrature kernels
// of hd_gauss.cuh), so that the units compile in parallel.
#include "hd_batch.cuh"
#include "hd_ecl.cuh"
#include "hd_gauss.cuh"

#define HD_FOR_N(X, D) X(D, 2) X(D, 3) X(D, 4) X(D, 5) X(D, 6)
#define HD_DECL_ECL(D, N) EclLaunchers ecl_launchers_##D##_##N();
#define HD_CASE_ECL(D, N) \
  case N: return ecl_launchers_##D##_##N();
#define HD_DECL_BATCH(D, N) BatchLaunchers batch_launchers_##D##_##N();
#define HD_CASE_BATCH(D, N) \
  case N: return batch_launchers_##D##_##N();

namespace hd {

HD_FOR_N(HD_DECL_ECL, 2)
HD_FOR_N(HD_DECL_ECL, 3)
HD_FOR_N(HD_DECL_ECL, 4)
HD_FOR_N(HD_DECL_ECL, 5)
HD_FOR_N(HD_DECL_ECL, 6)
HD_DECL_BATCH(4, 3) HD_DECL_BATCH(4, 4) HD_DECL_BATCH(4, 5) HD_DECL_BATCH(4, 6)
HD_DECL_BATCH(5, 3) HD_DECL_BATCH(5, 4) HD_DECL_BATCH(5, 5) HD_DECL_BATCH(5, 6)
#define HD_FOR_NG(X, D) X(D, 2) X(D, 3) X(D, 4) X(D, 5)
#define HD_DECL_GAUSS(D, N) GaussLaunchers gauss_launchers_##D##_##N();
#define HD_CASE_GAUSS(D, N) \
  case N: return gauss_launchers_##D##_##N();
HD_FOR_NG(HD_DECL_GAUSS, 2)
HD_FOR_NG(HD_DECL_GAUSS, 3)
HD_FOR_NG(HD_DECL_GAUSS, 4)
HD_FOR_NG(HD_DECL_GAUSS, 5)
HD_FOR_NG(HD_DECL_GAUSS, 6)

static const EclLaunchers kNoEcl{nullptr, nullptr, 0, 0, 0, 0, 0, 0, false, false};

EclLaunchers ecl_launchers_d2(int N) {
  switch (N) { HD_FOR_N(HD_CASE_ECL, 2) default: return kNoEcl; }
}
EclLaunchers ecl_launchers_d3(int N) {
  switch (N) { HD_FOR_N(HD_CASE_ECL, 3) default: return kNoEcl; }
}
EclLaunchers ecl_launchers_d4(int N) {
  switch (N) { HD_FOR_N(HD_CASE_ECL, 4) default: return kNoEcl; }
}
EclLaunchers ecl_launchers_d5(int N) {
  switch (N) { HD_FOR_N(HD_CASE_ECL, 5) default: return kNoEcl; }
}
EclLaunchers ecl_launchers_d6(int N) {
  switch (N) { HD_FOR_N(HD_CASE_ECL, 6) default: return kNoEcl; }
}

BatchLaunchers batch_launchers_d4(int N) {
  switch (N) {
    HD_CASE_BATCH(4, 3) HD_CASE_BATCH(4, 4) HD_CASE_BATCH(4, 5) HD_CASE_BATCH(4, 6)
    default: return BatchLaunchers{nullptr, nullptr, 0, 0, 0, 0, false};
  }
}
BatchLaunchers batch_launchers_d5(int N) {
  switch (N) {
    HD_CASE_BATCH(5, 3) HD_CASE_BATCH(5, 4) HD_CASE_BATCH(5, 5) HD_CASE_BATCH(5, 6)
    default: return BatchLaunchers{nullptr, nullptr, 0, 0, 0, 0, false};
  }
}

// Gauss quadrature: degrees 1..4 (N = 2..5)
GaussLaunchers gauss_launchers(int D, int N) {
  const GaussLaunchers none{nullptr, nullptr, false, false};
  switch (D) {
    case 2: switch (N) { HD_FOR_NG(HD_CASE_GAUSS, 2) default: return none; }
    case 3: switch (N) { HD_FOR_NG(HD_CASE_GAUSS, 3) default: return none; }
    case 4: switch (N) { HD_FOR_NG(HD_CASE_GAUSS, 4) default: return none; }
    case 5: switch (N) { HD_FOR_NG(HD_CASE_GAUSS, 5) default: return none; }
    case 6: switch (N) { HD_FOR_NG(HD_CASE_GAUSS, 6) default: return none; }
    default: return none;
  }
}

}  // namespace hd
