// Tendency, stage-update and diagnostic kernels of the GB300 shallow-water
// path (sm_103a, FP64).
//
// GB300 issues FP64 at 1/64 of its FP32 rate (about 0.6 T DFMA/s), so one
// tendency evaluation is bound by FP64 instructions, not by HBM.  The
// kernels are arranged to issue as few FP64 instructions per cell-level as
// possible:
//  - every intermediate is computed exactly once per stage and kept in
//    HBM/L2 for its consumers (no halo recomputation);
//  - all K-independent factors are folded into per-entity coefficient tables
//    (loaded as warp-broadcasts) and zero TRiSK weights are dropped;
//  - tracer terms are rewritten as weighted sums over neighbour values whose
//    weights are shared by all tracers of a cell;
//  - reciprocals use Newton-Raphson from the hardware approximation (5 FP64
//    slots instead of about 9 for IEEE division);
//  - the RK stage update is fused into the last two kernels.
// One thread handles one (entity, level); k is the fastest index, so a warp
// reads 32 consecutive levels (256 contiguous bytes) of one entity.
//
// Reference functors restated (omega_playground src/model/...):
//   k_vertex    vorticity_aux.hpp:294-325        (rvort, PV at vertices)
//   k_cell1     kinetic_aux.hpp:50-79, tracer_aux.hpp:181-201
//   k_edge1     thickness_aux.hpp:123-142, vorticity_aux.hpp:327-341,
//               vel_hyperdiff_edge.hpp:237-261 / vel_diff_edge.hpp:72-81
//   k_aux2      kinetic_aux.hpp:59-71 (ke), vel_hyperdiff_edge.hpp:263-307,
//               tracer_hyperdiff_cell.hpp:301-336
//   k_edge_final pv_flux_edge.hpp:149-177, ke_grad_edge.hpp:223-237,
//               ssh_grad_edge.hpp:281-294, vel_diff_edge.hpp:61-86,
//               vel_hyperdiff_edge.hpp:309-334, rk4.cpp:94-138, lsrk.cpp:47-86
//   k_cell_final thickness_hadv_cell.hpp:59-83, tracer_hadv_cell.hpp:60-90,
//               tracer_diff_cell.hpp:162-193, tracer_hyperdiff_cell.hpp:338-368
#include "swg_internal.h"

#include <algorithm>
#include <cstring>

namespace swg {
namespace {

constexpr int TPB = 256;

// 1/x: hardware estimate refined by two Newton-Raphson steps
// r <- r + r (1 - x r); each step squares the relative error of the estimate.
__device__ __forceinline__ double rcp_nr(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}

__device__ __forceinline__ void epilogue(const Epilogue &ep, const FieldIO &f,
                                         size_t i, double x) {
  switch (ep.mode) {
  case EPI_REPLACE:
    f.tend[i] = x;
    break;
  case EPI_INCREMENT:
    f.tend[i] += x;
    break;
  case EPI_LSRK: {
    const double t = fma(ep.a, f.tend[i], x);
    f.tend[i] = t;
    f.out[i] = fma(ep.dtb, t, f.out[i]);
  } break;
  case EPI_RK4_FIRST: {
    const double s = f.old[i];
    f.acc[i] = fma(ep.dtb, x, s);
    f.out[i] = fma(ep.dta, x, s);
  } break;
  case EPI_RK4_MID:
    f.acc[i] = fma(ep.dtb, x, f.acc[i]);
    f.out[i] = fma(ep.dta, x, f.old[i]);
    break;
  default: // EPI_RK4_LAST
    f.out[i] = fma(ep.dtb, x, f.acc[i]);
    break;
  }
}

// Vertex pass: relative vorticity and (rvort + f) / h_vertex.
__global__ void __launch_bounds__(TPB)
    k_vertex(MeshView m, ModelView p, AuxView a, const double *__restrict__ h,
             const double *__restrict__ vn) {
  const int K = m.nlayers;
  const unsigned i = blockIdx.x * TPB + threadIdx.x;
  if (i >= unsigned(m.nvertices) * unsigned(K))
    return;
  const int v = int(i / unsigned(K)), k = int(i - unsigned(v) * unsigned(K));
  double z, hv;
  {
    const int e = __ldg(m.ev + 3 * v), c = __ldg(m.cv + 3 * v);
    z = __ldg(m.cvr + 3 * v) * vn[size_t(e) * K + k];
    hv = __ldg(m.kvh + 3 * v) * h[size_t(c) * K + k];
  }
#pragma unroll
  for (int j = 1; j < 3; ++j) {
    const int e = __ldg(m.ev + 3 * v + j), c = __ldg(m.cv + 3 * v + j);
    z = fma(__ldg(m.cvr + 3 * v + j), vn[size_t(e) * K + k], z);
    hv = fma(__ldg(m.kvh + 3 * v + j), h[size_t(c) * K + k], hv);
  }
  a.q[i] = (z + __ldg(p.f_vertex + v)) * rcp_nr(hv);
  if (p.vel_del2 | p.vel_del4)
    a.zeta[i] = z;
}

// Cell pass 1: velocity divergence (for the dissipation terms) and the
// normalised tracers tr / h.
__global__ void __launch_bounds__(TPB)
    k_cell1(MeshView m, ModelView p, AuxView a, const double *__restrict__ h,
            const double *__restrict__ vn, const double *__restrict__ tr) {
  const int K = m.nlayers;
  const unsigned i = blockIdx.x * TPB + threadIdx.x;
  const unsigned CK = unsigned(m.ncells) * unsigned(K);
  if (i >= CK)
    return;
  const int c = int(i / unsigned(K)), k = int(i - unsigned(c) * unsigned(K));
  if (p.do_vn && (p.vel_del2 | p.vel_del4)) {
    double dv = __ldg(m.ccd + 6 * c) * vn[size_t(__ldg(m.ec + 6 * c)) * K + k];
#pragma unroll
    for (int j = 1; j < MAXE; ++j)
      dv = fma(__ldg(m.ccd + 6 * c + j),
               vn[size_t(__ldg(m.ec + 6 * c + j)) * K + k], dv);
    a.div[i] = dv;
  }
  if (p.ntracers > 0) {
    const double r = rcp_nr(h[i]);
    for (int l = 0; l < p.ntracers; ++l) {
      const size_t t = size_t(l) * CK + i;
      a.ntr[t] = tr[t] * r;
    }
  }
}

// Edge pass 1: mean thickness, thickness flux F = mean_h vn, vn^2, edge PV
// sum Q = q(v0) + q(v1), G = F Q, and the edge Laplacian of the velocity.
__global__ void __launch_bounds__(TPB)
    k_edge1(MeshView m, ModelView p, AuxView a, const double *__restrict__ h,
            const double *__restrict__ vn) {
  const int K = m.nlayers;
  const unsigned i = blockIdx.x * TPB + threadIdx.x;
  if (i >= unsigned(m.nedges) * unsigned(K))
    return;
  const int e = int(i / unsigned(K)), k = int(i - unsigned(e) * unsigned(K));
  const int c0 = __ldg(m.ce + 2 * e), c1 = __ldg(m.ce + 2 * e + 1);
  const double mh = 0.5 * (h[size_t(c0) * K + k] + h[size_t(c1) * K + k]);
  const double u = vn[i];
  const double F = mh * u;
  a.F[i] = F;
  if (p.ntracers > 0 && (p.tr_del2 | p.tr_del4))
    a.mh[i] = mh;
  if (p.do_vn) {
    const int v0 = __ldg(m.ve + 2 * e), v1 = __ldg(m.ve + 2 * e + 1);
    const double Q = a.q[size_t(v0) * K + k] + a.q[size_t(v1) * K + k];
    a.Q[i] = Q;
    a.G[i] = F * Q;
    a.u2[i] = u * u;
    if (p.vel_del2 | p.vel_del4) {
      const double dd = a.div[size_t(c1) * K + k] - a.div[size_t(c0) * K + k];
      const double dz = a.zeta[size_t(v1) * K + k] - a.zeta[size_t(v0) * K + k];
      const double idc = __ldg(m.inv_dc + e);
      a.d2u[i] = fma(dd, idc, -(dz * __ldg(m.inv_dv + e)));
      if (p.vel_del4 && m.dv4_differs)
        a.d2u4[i] = fma(dd, idc, -(dz * __ldg(m.inv_dv4 + e)));
    }
  }
}

// Second auxiliary pass: kinetic energy (cells), curl (vertices) and
// divergence (cells) of the edge Laplacian, and the thickness-weighted
// tracer Laplacian L (cells).  The first V*K threads take vertices, the
// rest cells.
__global__ void __launch_bounds__(TPB)
    k_aux2(MeshView m, ModelView p, AuxView a, unsigned base) {
  const int K = m.nlayers;
  unsigned i = base + blockIdx.x * TPB + threadIdx.x;
  const unsigned VK = unsigned(m.nvertices) * unsigned(K);
  const unsigned CK = unsigned(m.ncells) * unsigned(K);
  const bool vel = p.do_vn && p.vel_del4;
  if (i < VK) {
    if (!vel)
      return;
    const int v = int(i / unsigned(K)), k = int(i - unsigned(v) * unsigned(K));
    double z = __ldg(m.cvr + 3 * v) * a.d2u4[size_t(__ldg(m.ev + 3 * v)) * K + k];
#pragma unroll
    for (int j = 1; j < 3; ++j)
      z = fma(__ldg(m.cvr + 3 * v + j),
              a.d2u4[size_t(__ldg(m.ev + 3 * v + j)) * K + k], z);
    a.z4[i] = z;
    return;
  }
  i -= VK;
  if (i >= CK)
    return;
  const int c = int(i / unsigned(K)), k = int(i - unsigned(c) * unsigned(K));
  if (p.do_vn) {
    // ke = sum_j dv dc / (4 area) vn_j^2
    double ke = __ldg(m.cke + 6 * c) * a.u2[size_t(__ldg(m.ec + 6 * c)) * K + k];
#pragma unroll
    for (int j = 1; j < MAXE; ++j)
      ke = fma(__ldg(m.cke + 6 * c + j),
               a.u2[size_t(__ldg(m.ec + 6 * c + j)) * K + k], ke);
    a.ke[i] = ke;
  }
  if (vel) {
    double d = __ldg(m.ccd + 6 * c) * a.d2u4[size_t(__ldg(m.ec + 6 * c)) * K + k];
#pragma unroll
    for (int j = 1; j < MAXE; ++j)
      d = fma(__ldg(m.ccd + 6 * c + j),
              a.d2u4[size_t(__ldg(m.ec + 6 * c + j)) * K + k], d);
    a.d4[i] = d;
  }
  if (p.ntracers > 0 && p.tr_del4) {
    // L = sum_j w_j (n_nb - n_c), w_j = ckq_j mean_h_j
    double w[MAXE], M;
    int nb[MAXE];
#pragma unroll
    for (int j = 0; j < MAXE; ++j) {
      w[j] = __ldg(m.ckq + 6 * c + j) * a.mh[size_t(__ldg(m.ec + 6 * c + j)) * K + k];
      nb[j] = __ldg(m.nbc + 6 * c + j);
    }
    M = w[0] + w[1];
#pragma unroll
    for (int j = 2; j < MAXE; ++j)
      M += w[j];
    for (int l = 0; l < p.ntracers; ++l) {
      const double *n = a.ntr + size_t(l) * CK;
      double acc = w[0] * n[size_t(nb[0]) * K + k];
#pragma unroll
      for (int j = 1; j < MAXE; ++j)
        acc = fma(w[j], n[size_t(nb[j]) * K + k], acc);
      a.lap[size_t(l) * CK + i] = fma(-M, n[i], acc);
    }
  }
}

// Edge final pass: normal-velocity tendency (PV flux, Bernoulli gradient,
// del2 and del4 dissipation) and its stage update.
template <int NE>
__global__ void __launch_bounds__(TPB)
    k_edge_final(MeshView m, ModelView p, AuxView a, StageArgs s) {
  const int K = m.nlayers;
  const unsigned i = blockIdx.x * TPB + threadIdx.x;
  if (i >= unsigned(m.nedges) * unsigned(K))
    return;
  const int e = int(i / unsigned(K)), k = int(i - unsigned(e) * unsigned(K));
  // potential-vorticity flux: sum_j w_j F_j (Q_e + Q_j) / 4 with w/4 in woe
  double S1, S2;
  {
    const int je = __ldg(m.eoe + NE * e);
    const double w = __ldg(m.woe + NE * e);
    S1 = w * a.F[size_t(je) * K + k];
    S2 = w * a.G[size_t(je) * K + k];
  }
#pragma unroll
  for (int j = 1; j < NE; ++j) {
    const int je = __ldg(m.eoe + NE * e + j);
    const double w = __ldg(m.woe + NE * e + j);
    S1 = fma(w, a.F[size_t(je) * K + k], S1);
    S2 = fma(w, a.G[size_t(je) * K + k], S2);
  }
  double t = fma(a.Q[i], S1, S2);
  const int c0 = __ldg(m.ce + 2 * e), c1 = __ldg(m.ce + 2 * e + 1);
  const double idc = __ldg(m.inv_dc + e);
  // kinetic-energy and sea-surface-height gradients (the differences are
  // taken before scaling, as in the reference, so g h ~ 1e4 never rounds)
  t = fma(-idc, a.ke[size_t(c1) * K + k] - a.ke[size_t(c0) * K + k], t);
  t = fma(-__ldg(p.gidc + e), s.h[size_t(c1) * K + k] - s.h[size_t(c0) * K + k],
          t);
  const double mk = m.mask ? m.mask[i] : 1.0;
  if (p.vel_del2)
    t = fma(m.mask ? __ldg(p.c2e + e) * mk : __ldg(p.c2e + e), a.d2u[i], t);
  if (p.vel_del4) {
    const int v0 = __ldg(m.ve + 2 * e), v1 = __ldg(m.ve + 2 * e + 1);
    const double dd = a.d4[size_t(c1) * K + k] - a.d4[size_t(c0) * K + k];
    const double dz = a.z4[size_t(v1) * K + k] - a.z4[size_t(v0) * K + k];
    const double l = fma(dd, idc, -(dz * __ldg(m.inv_dv + e)));
    t = fma(m.mask ? __ldg(p.c4e + e) * mk : __ldg(p.c4e + e), l, t);
  }
  epilogue(s.ep, s.fvn, i, t);
}

// Cell final pass: thickness tendency and tracer tendencies (advection,
// del2, del4) with their stage updates.
__global__ void __launch_bounds__(TPB)
    k_cell_final(MeshView m, ModelView p, AuxView a, StageArgs s) {
  const int K = m.nlayers;
  const unsigned i = blockIdx.x * TPB + threadIdx.x;
  const unsigned CK = unsigned(m.ncells) * unsigned(K);
  if (i >= CK)
    return;
  const int c = int(i / unsigned(K)), k = int(i - unsigned(c) * unsigned(K));
  // a_j = -F_j ccd_j / 2: half the flux divergence weight of edge j
  double w[MAXE], Sa;
  int ej[MAXE];
#pragma unroll
  for (int j = 0; j < MAXE; ++j) {
    ej[j] = __ldg(m.ec + 6 * c + j);
    w[j] = __ldg(m.ccdh + 6 * c + j) * a.F[size_t(ej[j]) * K + k];
  }
  Sa = w[0] + w[1];
#pragma unroll
  for (int j = 2; j < MAXE; ++j)
    Sa += w[j];
  if (p.do_h)
    epilogue(s.ep, s.fh, i, 2.0 * Sa); // -sum_j ccd_j F_j
  if (p.ntracers == 0)
    return;
  // advection + del2: sum_j a_j (n_c + n_j) + b_j (n_j - n_c)
  double wc = Sa;
  if (p.tr_del2) {
    double b[MAXE], Sb;
#pragma unroll
    for (int j = 0; j < MAXE; ++j) {
      b[j] = __ldg(p.kd2 + 6 * c + j) * a.mh[size_t(ej[j]) * K + k];
      w[j] += b[j];
    }
    Sb = b[0] + b[1];
#pragma unroll
    for (int j = 2; j < MAXE; ++j)
      Sb += b[j];
    wc = Sa - Sb;
  }
  int nb[MAXE];
#pragma unroll
  for (int j = 0; j < MAXE; ++j)
    nb[j] = __ldg(m.nbc + 6 * c + j);
  for (int l = 0; l < p.ntracers; ++l) {
    const size_t base = size_t(l) * CK;
    const double *n = a.ntr + base;
    double acc = wc * n[i];
#pragma unroll
    for (int j = 0; j < MAXE; ++j)
      acc = fma(w[j], n[size_t(nb[j]) * K + k], acc);
    if (p.tr_del4) {
      const double *L = a.lap + base;
      acc = fma(-__ldg(p.r4sum + c), L[i], acc);
#pragma unroll
      for (int j = 0; j < MAXE; ++j)
        acc = fma(__ldg(p.r4 + 6 * c + j), L[size_t(nb[j]) * K + k], acc);
    }
    epilogue(s.ep, s.ftr, base + i, acc);
  }
}

// Elementwise helpers for the unfused stepper path (forcing hook set).
__global__ void k_axpby(double *__restrict__ y, const double *__restrict__ x,
                        const double *__restrict__ z, double alpha,
                        double beta, long long n, int kind) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  switch (kind) {
  case 0: y[i] *= alpha; break;                    // tend *= a
  case 1: y[i] = fma(alpha, x[i], y[i]); break;    // state += dtb * tend
  case 2: y[i] = fma(alpha, x[i], z[i]); break;    // provis = old + dta * tend
  default: y[i] = alpha; break;                    // fill
  }
  (void)beta;
}

// Diagnostics: one partial sum per block, summed on the host in block order.
template <int WHICH>
__global__ void __launch_bounds__(TPB)
    k_diag(MeshView m, ModelView p, const double *__restrict__ h,
           const double *__restrict__ vn, double *partials) {
  __shared__ double red[TPB];
  const int K = m.nlayers;
  const long long n = (WHICH == 2 ? (long long)m.nvertices : m.ncells) * K;
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)TPB + threadIdx.x; i < n;
       i += (long long)gridDim.x * TPB) {
    const int ent = int(i / K), k = int(i - (long long)ent * K);
    if (WHICH == 0) { // mass: area_cell h
      s += m.area_cell_d[ent] * h[i];
    } else if (WHICH == 1) { // energy: area (g h^2/2 + h ke)
      double ke = 0.0;
      for (int j = 0; j < MAXE; ++j) {
        const double u = vn[size_t(m.ec[6 * ent + j]) * K + k];
        ke += m.cke[6 * ent + j] * u * u;
      }
      const double hc = h[i];
      s += m.area_cell_d[ent] * (p.grav * hc * hc / 2 + hc * ke);
    } else { // circulation: sum_j dc s vn + f area_triangle
      double cir = 0.0;
      for (int j = 0; j < 3; ++j)
        cir += m.dcs_v[3 * ent + j] * vn[size_t(m.ev[3 * ent + j]) * K + k];
      s += cir + p.f_vertex[ent] * m.area_tri_d[ent];
    }
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = TPB / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    partials[blockIdx.x] = red[0];
}

unsigned nblocks(long long n) { return unsigned((n + TPB - 1) / TPB); }

// ---- opt-in per-kernel timing: an event pair around every tendency kernel
struct Timed {
  const char *name;
  cudaEvent_t start, stop;
};
std::vector<Timed> g_timed;
bool g_profile = false;

struct Scope {
  const char *name;
  cudaStream_t st;
  cudaEvent_t a = nullptr, b = nullptr;
  Scope(const char *n, cudaStream_t s) : name(n), st(s) {
    if (g_profile && cudaEventCreate(&a) == cudaSuccess &&
        cudaEventCreate(&b) == cudaSuccess)
      cudaEventRecord(a, st);
  }
  ~Scope() {
    if (a && b) {
      cudaEventRecord(b, st);
      g_timed.push_back({name, a, b});
    }
    ++g_launches;
  }
};

} // namespace

bool profiling_enabled() { return g_profile; }

int profile_enable(int on) {
  g_profile = on != 0;
  return SWG_OK;
}

int profile_read(int max_kernels, char *names, double *total_ms,
                 long long *launches, int *count) {
  std::vector<std::string> keys;
  std::vector<double> ms;
  std::vector<long long> n;
  for (auto &t : g_timed) {
    float x = 0.f;
    cudaError_t err = cudaEventSynchronize(t.stop);
    if (err == cudaSuccess)
      err = cudaEventElapsedTime(&x, t.start, t.stop);
    cudaEventDestroy(t.start);
    cudaEventDestroy(t.stop);
    if (err != cudaSuccess) {
      g_timed.clear();
      return cuda_fail(err, "swg_profile_read");
    }
    size_t j = 0;
    while (j < keys.size() && keys[j] != t.name)
      ++j;
    if (j == keys.size()) {
      keys.push_back(t.name);
      ms.push_back(0.0);
      n.push_back(0);
    }
    ms[j] += x;
    n[j] += 1;
  }
  g_timed.clear();
  const int m = std::min<int>(max_kernels, int(keys.size()));
  for (int j = 0; j < m; ++j) {
    std::strncpy(names + 32 * j, keys[j].c_str(), 31);
    names[32 * j + 31] = 0;
    total_ms[j] = ms[j];
    launches[j] = n[j];
  }
  *count = m;
  return SWG_OK;
}

void launch_tendency(const MeshView &m, const ModelView &p, const AuxView &a,
                     const StageArgs &s, cudaStream_t st) {
  const long long K = m.nlayers;
  const long long VK = m.nvertices * K, CK = m.ncells * K, EK = m.nedges * K;
  if (p.do_vn) {
    Scope sc("k_vertex", st);
    k_vertex<<<nblocks(VK), TPB, 0, st>>>(m, p, a, s.h, s.vn);
  }
  if ((p.do_vn && (p.vel_del2 || p.vel_del4)) || p.ntracers > 0) {
    Scope sc("k_cell1", st);
    k_cell1<<<nblocks(CK), TPB, 0, st>>>(m, p, a, s.h, s.vn, s.tr);
  }
  if (p.do_vn || p.do_h || p.ntracers > 0) {
    Scope sc("k_edge1", st);
    k_edge1<<<nblocks(EK), TPB, 0, st>>>(m, p, a, s.h, s.vn);
  }
  const bool tr4 = p.ntracers > 0 && p.tr_del4;
  if (p.do_vn || tr4) {
    Scope sc("k_aux2", st);
    // vertex threads only when the velocity del4 curl is needed
    const unsigned base = (p.do_vn && p.vel_del4) ? 0u : unsigned(VK);
    k_aux2<<<nblocks(VK + CK - base), TPB, 0, st>>>(m, p, a, base);
  }
  if (p.do_vn) {
    Scope sc("k_edge_final", st);
    if (m.ne == 8)
      k_edge_final<8><<<nblocks(EK), TPB, 0, st>>>(m, p, a, s);
    else
      k_edge_final<10><<<nblocks(EK), TPB, 0, st>>>(m, p, a, s);
  }
  if (p.do_h || p.ntracers > 0) {
    Scope sc("k_cell_final", st);
    k_cell_final<<<nblocks(CK), TPB, 0, st>>>(m, p, a, s);
  }
}

void launch_axpby(double *y, const double *x, const double *z, double alpha,
                  double beta, long long n, int kind, cudaStream_t st) {
  if (n <= 0)
    return;
  k_axpby<<<nblocks(n), TPB, 0, st>>>(y, x, z, alpha, beta, n, kind);
  ++g_launches;
}

int reduce_diag(int which, const MeshView &m, const ModelView &p,
                const double *h, const double *vn, double *partials,
                int npart, double *out, cudaStream_t st) {
  if (which == 0)
    k_diag<0><<<npart, TPB, 0, st>>>(m, p, h, vn, partials);
  else if (which == 1)
    k_diag<1><<<npart, TPB, 0, st>>>(m, p, h, vn, partials);
  else
    k_diag<2><<<npart, TPB, 0, st>>>(m, p, h, vn, partials);
  ++g_launches;
  std::vector<double> hp(npart);
  cudaError_t err = cudaMemcpyAsync(hp.data(), partials, npart * sizeof(double),
                                    cudaMemcpyDeviceToHost, st);
  if (err == cudaSuccess)
    err = cudaStreamSynchronize(st);
  if (err != cudaSuccess)
    return cuda_fail(err, "diagnostic reduction");
  double s = 0.0;
  for (double x : hp)
    s += x;
  *out = s;
  return SWG_OK;
}

} // namespace swg
