// Scalar stand-in for Kokkos::Experimental::native_simd (width 1), matching
// the Kokkos CUDA backend where native_simd<double> is scalar.  Only the
// width is used by the default (non-OMEGA_KOKKOS_SIMD) reference build.
#pragma once
namespace Kokkos {
namespace Experimental {
struct element_aligned_tag {};
template <class T> struct native_simd {
  static constexpr int size() { return 1; }
};
} // namespace Experimental
} // namespace Kokkos
