// FP64 issue-rate measurement (swg_fp64_issue_rate): the roof the solver's
// kernels are bound by on GB300, measured on the GPU that runs them.
//
// Every thread runs kChains independent dependency chains of one FP64
// operation (DFMA, DADD or DMUL) for `iters` iterations, so the pipe, not
// the latency of one chain, limits the rate.  The grid fills every SM with
// the resident maximum of 256-thread blocks.  Operands come from device
// memory (not compile-time constants), the chains stay at a fixed point
// (FMA converges to 1, ADD adds a tiny value that rounds away, MUL
// multiplies by 1), so no value overflows or goes subnormal, and each
// thread stores its sum so nothing is eliminated.
#include "swg_internal.h"

namespace swg {
namespace {

constexpr int kChains = 4;

// a, b are read from device memory into registers: operands taken straight
// from the kernel's parameters measured about 12 % slower, and so did
// chains with operands of their own (8 or 16 chains, three distinct
// registers per instruction), while 4 chains sharing a and b reached 2
// thread-instructions per SM per clock on GB300.
template <int OP>
__global__ void __launch_bounds__(256)
    k_fp64_issue(double *out, const double *ab, int iters) {
  const double a = ab[0], b = ab[1];
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c)
    x[c] = 1.0 + c * 1e-3 + threadIdx.x * 1e-9;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) {
      if (OP == 0)
        x[c] = fma(x[c], a, b);
      else if (OP == 1)
        x[c] = x[c] + ((c & 1) ? b : -b);
      else
        x[c] = x[c] * a;
    }
  }
  double s = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c)
    s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

} // namespace
} // namespace swg

using namespace swg;

extern "C" int swg_fp64_issue_rate(int op, int iters, double *inst_per_s,
                                   double *ms, void *stream) try {
  if (op < 0 || op > 2 || iters < 1 || !inst_per_s)
    return fail(SWG_ERR_ARG, "swg_fp64_issue_rate: bad argument");
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err == cudaSuccess)
    err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (err == cudaSuccess)
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, k_fp64_issue<0>, 256, 0);
  if (err != cudaSuccess)
    return cuda_fail(err, "swg_fp64_issue_rate: device query");
  const int blocks = sms * (per_sm > 0 ? per_sm : 1);
  double *out = nullptr, *ab = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  err = cudaMalloc(&out, (size_t(blocks) * 256 + 2) * sizeof(double));
  ab = out + size_t(blocks) * 256;
  // fixed points: fma(x, 0.5, 0.5) -> 1, x * 1 = x, x +- 1e-300 = x
  const double hab[2] = {op == 0 ? 0.5 : 1.0, op == 0 ? 0.5 : 1e-300};
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(ab, hab, sizeof hab, cudaMemcpyHostToDevice, st);
  if (err == cudaSuccess)
    err = cudaEventCreate(&e0);
  if (err == cudaSuccess)
    err = cudaEventCreate(&e1);
  float t = 0.f;
  auto launch = [&](int n) {
    if (op == 0)
      k_fp64_issue<0><<<blocks, 256, 0, st>>>(out, ab, n);
    else if (op == 1)
      k_fp64_issue<1><<<blocks, 256, 0, st>>>(out, ab, n);
    else
      k_fp64_issue<2><<<blocks, 256, 0, st>>>(out, ab, n);
  };
  if (err == cudaSuccess) {
    launch(iters / 10 + 1); // warm-up
    cudaEventRecord(e0, st);
    launch(iters);
    cudaEventRecord(e1, st);
    err = cudaEventSynchronize(e1);
  }
  if (err == cudaSuccess)
    err = cudaEventElapsedTime(&t, e0, e1);
  g_launches += 2;
  if (e0)
    cudaEventDestroy(e0);
  if (e1)
    cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess)
    return cuda_fail(err, "swg_fp64_issue_rate");
  *inst_per_s = double(blocks) * 256.0 * kChains * double(iters) /
                (double(t) * 1e-3);
  if (ms)
    *ms = t;
  return SWG_OK;
} SWG_ABI_CATCH("swg_fp64_issue_rate")
