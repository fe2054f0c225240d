// ref_shim.cpp -- C entry points over the KSpaceJet reference's own numerics,
// compiled together with the reference sources into oracle/_ref/ by
// oracle/build.py.  TEST INFRASTRUCTURE ONLY: it is the checker that pins the
// C restatement in ksj_oracle.c, and nothing in the product links it.
//
// Each wrapper calls the reference's public function unchanged and turns a
// thrown exception into the return value -1.
#include "kspacejet/base/types.hpp"
#include "kspacejet/nufft/direct_nudft.hpp"
#include "kspacejet/nufft/radial_gridding.hpp"

#include <complex>
#include <cstdint>
#include <vector>

#define KSJR_EXPORT extern "C" __attribute__((visibility("default")))

namespace {

template <typename T>
int linear_gridding(std::int64_t rows, std::int64_t cols, double row_origin, double col_origin, const T* samples,
                    const T* traj, const T* dcf, std::int64_t m, T* image) {
  try {
    using C = std::complex<T>;
    const auto r = static_cast<std::size_t>(rows);
    const auto c = static_cast<std::size_t>(cols);
    const auto line = r > c ? r : c;
    std::vector<C> inter(r * c), src(line), dst(line);
    const auto grid = ksj::nufft::Grid2D{r, c, row_origin, col_origin};
    const auto workspace = ksj::nufft::RadialGridding2Workspace<T>{
      ksj::array::MatrixView<C>{inter.data(), r, c},
      ksj::array::VectorView<C>{src.data(), line},
      ksj::array::VectorView<C>{dst.data(), line},
    };
    ksj::nufft::radial_linear_gridding2_adjoint(
      grid, ksj::array::VectorView<const C>{reinterpret_cast<const C*>(samples), static_cast<std::size_t>(m)},
      ksj::array::MatrixView<const T>{traj, static_cast<std::size_t>(m), 2U},
      ksj::array::VectorView<const T>{dcf, static_cast<std::size_t>(m)},
      ksj::array::MatrixView<C>{reinterpret_cast<C*>(image), r, c}, workspace);
    return 0;
  } catch (...) {
    return -1;
  }
}

template <typename T> int ramp(const T* traj, std::int64_t m, T* dcf) {
  try {
    ksj::nufft::radial_analytic_ramp_dcf2(ksj::array::MatrixView<const T>{traj, static_cast<std::size_t>(m), 2U},
                                          ksj::array::VectorView<T>{dcf, static_cast<std::size_t>(m)});
    return 0;
  } catch (...) {
    return -1;
  }
}

template <typename T>
int direct_adjoint(std::int64_t rows, std::int64_t cols, double row_origin, double col_origin, const T* samples,
                   const T* traj, std::int64_t m, T* image) {
  try {
    using C = std::complex<T>;
    const auto grid =
      ksj::nufft::Grid2D{static_cast<std::size_t>(rows), static_cast<std::size_t>(cols), row_origin, col_origin};
    ksj::nufft::direct_nudft2_adjoint(
      grid, ksj::array::VectorView<const C>{reinterpret_cast<const C*>(samples), static_cast<std::size_t>(m)},
      ksj::array::MatrixView<const T>{traj, static_cast<std::size_t>(m), 2U},
      ksj::array::MatrixView<C>{reinterpret_cast<C*>(image), static_cast<std::size_t>(rows),
                                static_cast<std::size_t>(cols)});
    return 0;
  } catch (...) {
    return -1;
  }
}

} // namespace

KSJR_EXPORT int ksjr_ramp_dcf2_f32(const float* traj, std::int64_t m, float* dcf) { return ramp(traj, m, dcf); }
KSJR_EXPORT int ksjr_ramp_dcf2_f64(const double* traj, std::int64_t m, double* dcf) { return ramp(traj, m, dcf); }

KSJR_EXPORT int ksjr_linear_gridding2_adjoint_f32(std::int64_t rows, std::int64_t cols, double ro, double co,
                                                  const float* samples, const float* traj, const float* dcf,
                                                  std::int64_t m, float* image) {
  return linear_gridding(rows, cols, ro, co, samples, traj, dcf, m, image);
}

KSJR_EXPORT int ksjr_linear_gridding2_adjoint_f64(std::int64_t rows, std::int64_t cols, double ro, double co,
                                                  const double* samples, const double* traj, const double* dcf,
                                                  std::int64_t m, double* image) {
  return linear_gridding(rows, cols, ro, co, samples, traj, dcf, m, image);
}

KSJR_EXPORT int ksjr_direct_nudft2_adjoint_f32(std::int64_t rows, std::int64_t cols, double ro, double co,
                                               const float* samples, const float* traj, std::int64_t m,
                                               float* image) {
  return direct_adjoint(rows, cols, ro, co, samples, traj, m, image);
}

KSJR_EXPORT int ksjr_direct_nudft2_adjoint_f64(std::int64_t rows, std::int64_t cols, double ro, double co,
                                               const double* samples, const double* traj, std::int64_t m,
                                               double* image) {
  return direct_adjoint(rows, cols, ro, co, samples, traj, m, image);
}
