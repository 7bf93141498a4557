// Accuracy of the kernels' reciprocal rcp_nr (swg_device.cuh) against CUDA's
// IEEE division 1.0 / x on the device, in units in the last place of the
// correctly rounded quotient.  rcp_nr refines the hardware estimate
// rcp.approx.ftz.f64 with two Newton-Raphson steps.  The sweep covers
// log-spaced magnitudes from 1e-6 to 1e6 (both signs), random mantissas in
// every binade of [2^-40, 2^40], and thicknesses near the frozen / dry
// levels a layer can reach (1e-3 .. 1e1 m).  Prints the maximum ulp error
// and the count of results that differ from the division at all.
#include "../../omega_playground_gb300/csrc/swg_device.cuh"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

__global__ void k_rcp(const double *x, double *nr, double *div, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    nr[i] = swg::rcp_nr(x[i]);
    div[i] = 1.0 / x[i];
  }
}

static int64_t ordered(double d) {
  int64_t b;
  std::memcpy(&b, &d, sizeof b);
  return b < 0 ? INT64_MIN - b : b;
}

int main() {
  std::vector<double> x;
  for (int i = 0; i <= 120000; ++i) { // 1e-6 .. 1e6, log-spaced
    const double v = std::pow(10.0, -6.0 + 12.0 * i / 120000.0);
    x.push_back(v);
    x.push_back(-v);
  }
  uint64_t z = 0x9E3779B97F4A7C15ull;
  auto next = [&z]() {
    z ^= z << 13;
    z ^= z >> 7;
    z ^= z << 17;
    return z;
  };
  for (int e = -40; e <= 40; ++e) // random mantissas in every binade
    for (int j = 0; j < 4000; ++j)
      x.push_back(std::ldexp(1.0 + double(next() >> 12) * 0x1.0p-52, e));
  for (int j = 0; j < 200000; ++j) // thin layers: 1e-3 .. 1e1 m
    x.push_back(1e-3 * std::pow(1e4, double(next() >> 11) * 0x1.0p-53));
  const int n = int(x.size());
  double *dx, *dnr, *ddiv;
  if (cudaMalloc(&dx, n * 8) != cudaSuccess ||
      cudaMalloc(&dnr, n * 8) != cudaSuccess ||
      cudaMalloc(&ddiv, n * 8) != cudaSuccess)
    return 2;
  cudaMemcpy(dx, x.data(), n * 8, cudaMemcpyHostToDevice);
  k_rcp<<<(n + 255) / 256, 256>>>(dx, dnr, ddiv, n);
  std::vector<double> nr(n), dv(n);
  cudaMemcpy(nr.data(), dnr, n * 8, cudaMemcpyDeviceToHost);
  if (cudaMemcpy(dv.data(), ddiv, n * 8, cudaMemcpyDeviceToHost) !=
      cudaSuccess)
    return 2;
  int64_t worst = 0, differ = 0;
  double worst_x = 0;
  for (int i = 0; i < n; ++i) {
    const int64_t d = std::llabs(ordered(nr[i]) - ordered(dv[i]));
    differ += d != 0;
    if (d > worst) {
      worst = d;
      worst_x = x[i];
    }
  }
  std::printf("samples %d max_ulp %lld at x=%.17g differing %lld\n", n,
              (long long)worst, worst_x, (long long)differ);
  cudaFree(dx);
  cudaFree(dnr);
  cudaFree(ddiv);
  return 0;
}
