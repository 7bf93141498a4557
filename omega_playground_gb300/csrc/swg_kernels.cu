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
#include "swg_device.cuh"

#include <algorithm>
#include <type_traits>
#include <cstring>

namespace swg {
namespace {

constexpr int TPB = 256;

// Single-instance kernels: one launch per pass over (entity, level),
// templated on the value type (double, or Dual for the tangent-linear model).
template <class T>
__global__ void __launch_bounds__(TPB)
    k_vertex(MeshView m, ModelView p, AuxViewT<T> a, const T *__restrict__ h,
             const T *__restrict__ vn) {
  const unsigned i = blockIdx.x * TPB + threadIdx.x;
  if (i < unsigned(m.nvertices) * unsigned(m.nlayers))
    pt_vertex<T>(m, p, a, h, vn, i);
}

template <class T>
__global__ void __launch_bounds__(TPB)
    k_cell1(MeshView m, ModelView p, AuxViewT<T> a, const T *__restrict__ h,
            const T *__restrict__ vn, const T *__restrict__ tr) {
  const unsigned i = blockIdx.x * TPB + threadIdx.x;
  if (i < unsigned(m.ncells) * unsigned(m.nlayers))
    pt_cell1<T>(m, p, a, h, vn, tr, i);
}

template <class T>
__global__ void __launch_bounds__(TPB)
    k_edge1(MeshView m, ModelView p, AuxViewT<T> a, const T *__restrict__ h,
            const T *__restrict__ vn) {
  const unsigned i = blockIdx.x * TPB + threadIdx.x;
  if (i < unsigned(m.nedges) * unsigned(m.nlayers))
    pt_edge1<T>(m, p, a, h, vn, i);
}

template <class T>
__global__ void __launch_bounds__(TPB)
    k_aux2(MeshView m, ModelView p, AuxViewT<T> a, unsigned base) {
  const unsigned i = base + blockIdx.x * TPB + threadIdx.x;
  if (i < unsigned(m.nvertices + m.ncells) * unsigned(m.nlayers))
    pt_aux2<T>(m, p, a, i);
}

template <int NE, class T>
__global__ void __launch_bounds__(TPB)
    k_edge_final(MeshView m, ModelView p, AuxViewT<T> a, StageArgsT<T> s) {
  const unsigned i = blockIdx.x * TPB + threadIdx.x;
  if (i < unsigned(m.nedges) * unsigned(m.nlayers))
    pt_edge_final<NE, T>(m, p, a, s, i);
}

template <class T>
__global__ void __launch_bounds__(TPB)
    k_cell_final(MeshView m, ModelView p, AuxViewT<T> a, StageArgsT<T> s) {
  const unsigned i = blockIdx.x * TPB + threadIdx.x;
  if (i < unsigned(m.ncells) * unsigned(m.nlayers))
    pt_cell_final<T, std::is_same<T, double>::value>(m, p, a, s, i);
}

template <int NE, class T>
__global__ void __launch_bounds__(TPB)
    k_lin_edge(MeshView m, ModelView p, StageArgsT<T> s) {
  const unsigned i = blockIdx.x * TPB + threadIdx.x;
  if (i < unsigned(m.nedges) * unsigned(m.nlayers))
    pt_lin_edge<NE, T>(m, p, s, i);
}

template <class T>
__global__ void __launch_bounds__(TPB)
    k_lin_cell(MeshView m, ModelView p, StageArgsT<T> s) {
  const unsigned i = blockIdx.x * TPB + threadIdx.x;
  if (i < unsigned(m.ncells) * unsigned(m.nlayers))
    pt_lin_cell<T>(m, p, s, i);
}

// Thickness flux of a per-field tendency call (compute_h/vn/tr_tendency):
// F = mean_h vn from the last auxiliary state's mean thickness and the
// caller's normal velocity (pv_flux_edge.hpp and thickness_hadv_cell.hpp
// multiply the two per edge), and with G also F Q for the PV flux; the
// same expressions as pt_edge1, so equal inputs give equal fluxes.
template <bool G>
__global__ void __launch_bounds__(TPB)
    k_field_flux(MeshView m, AuxView a, const double *__restrict__ vn) {
  const unsigned i = blockIdx.x * TPB + threadIdx.x;
  if (i >= unsigned(m.nedges) * unsigned(m.nlayers))
    return;
  const double F = a.mh[i] * vn[i];
  a.F[i] = F;
  if (G)
    a.G[i] = F * a.Q[i];
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
    const int *maxlev = WHICH == 2 ? m.maxlev_v : m.maxlev_c;
    if (maxlev && k >= maxlev[ent])
      continue;
    if (WHICH == 0) { // mass: area_cell h
      s += m.area_cell_d[ent] * h[i];
    } else if (WHICH == 1) { // energy: area (g h^2/2 + h ke)
      double ke = 0.0;
      for (int j = 0; j < MAXE; ++j) {
        const double u = vn[size_t(m.ec[6 * ent + j]) * K + k];
        ke += m.cke[6 * ent + j] * u * u;
      }
      const double hc = h[i];
      // the linear model's kinetic energy is weighted by h0
      // (shallow_water_hierarchical.cpp:743-771)
      s += m.area_cell_d[ent] *
           (p.grav * hc * hc / 2 + (p.linear ? p.h0 : hc) * ke);
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
// > 0 while a ProfileOff guard is alive on this thread: launches not timed
thread_local int t_profile_off = 0;

struct Scope {
  const char *name;
  cudaStream_t st;
  cudaEvent_t a = nullptr, b = nullptr;
  Scope(const char *n, cudaStream_t s) : name(n), st(s) {
    if (g_profile && !t_profile_off && cudaEventCreate(&a) == cudaSuccess &&
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

ProfileOff::ProfileOff() { ++t_profile_off; }
ProfileOff::~ProfileOff() { --t_profile_off; }

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

namespace {

template <class T>
void launch_aux_t(const MeshView &m, const ModelView &p, const AuxViewT<T> &a,
                  const T *h, const T *vn, const T *tr, cudaStream_t st,
                  const Fork *fk) {
  const long long K = m.nlayers;
  const long long VK = m.nvertices * K, CK = m.ncells * K, EK = m.nedges * K;
  if (p.linear) // the linear model has no intermediates
    return;
  NvtxRange range("auxstate");
  // vertex and cell passes read only the state: independent
  const bool vert = p.do_vn;
  const bool cell1 = (p.do_vn && (p.vel_del2 || p.vel_del4)) || p.ntracers > 0;
  auto run_vertex = [&](cudaStream_t s) {
    Scope sc("k_vertex", s);
    k_vertex<T><<<nblocks(VK), TPB, 0, s>>>(m, p, a, h, vn);
  };
  auto run_cell1 = [&](cudaStream_t s) {
    Scope sc("k_cell1", s);
    k_cell1<T><<<nblocks(CK), TPB, 0, s>>>(m, p, a, h, vn, tr);
  };
  // per-kernel timing (profiling on) runs the passes one after another so
  // that each event pair times its own kernel alone
  if (g_profile)
    fk = nullptr;
  if (vert && cell1)
    fork_join(fk, st, run_vertex, run_cell1);
  else if (vert)
    run_vertex(st);
  else if (cell1)
    run_cell1(st);
  if (p.do_vn || p.do_h || p.ntracers > 0) {
    Scope sc("k_edge1", st);
    k_edge1<T><<<nblocks(EK), TPB, 0, st>>>(m, p, a, h, vn);
  }
  const bool tr4 = p.ntracers > 0 && p.tr_del4;
  if (p.do_vn || tr4) {
    Scope sc("k_aux2", st);
    // vertex threads only when the velocity del4 curl is needed
    const unsigned base = (p.do_vn && p.vel_del4) ? 0u : unsigned(VK);
    k_aux2<T><<<nblocks(VK + CK - base), TPB, 0, st>>>(m, p, a, base);
  }
}

template <class T>
void launch_tendency_t(const MeshView &m, const ModelView &p,
                       const AuxViewT<T> &a, const StageArgsT<T> &s,
                       cudaStream_t st, const Fork *fk) {
  const long long K = m.nlayers;
  const long long CK = m.ncells * K, EK = m.nedges * K;
  NvtxRange range("tendencies");
  if (p.linear) {
    // The linear passes read neighbouring h and vn of the stage input
    // directly, so an in-place (LSRK) stage first forms the tendency and
    // then updates the state.
    StageArgsT<T> ls = s;
    const bool in_place = s.ep.mode == EPI_LSRK;
    if (in_place)
      ls.ep.mode = EPI_LSRK_TEND;
    if (p.do_vn) {
      Scope sc("k_lin_edge", st);
      if (m.ne == 8)
        k_lin_edge<8, T><<<nblocks(EK), TPB, 0, st>>>(m, p, ls);
      else
        k_lin_edge<10, T><<<nblocks(EK), TPB, 0, st>>>(m, p, ls);
    }
    if (p.do_h) {
      Scope sc("k_lin_cell", st);
      k_lin_cell<T><<<nblocks(CK), TPB, 0, st>>>(m, p, ls);
    }
    if constexpr (std::is_same<T, double>::value) {
      if (in_place && p.do_vn) {
        Scope sc("k_axpby", st);
        k_axpby<<<nblocks(EK), TPB, 0, st>>>(s.fvn.out, s.fvn.tend, nullptr,
                                             s.ep.dtb, 0.0, EK, 1);
      }
      if (in_place && p.do_h) {
        Scope sc("k_axpby", st);
        k_axpby<<<nblocks(CK), TPB, 0, st>>>(s.fh.out, s.fh.tend, nullptr,
                                             s.ep.dtb, 0.0, CK, 1);
      }
    }
    return;
  }
  launch_aux_t<T>(m, p, a, s.h, s.vn, s.tr, st, fk);
  const bool edge = p.do_vn, cell = p.do_h || p.ntracers > 0;
  auto run_edge = [&](cudaStream_t q) {
    NvtxRange r("vn_tendency");
    Scope sc("k_edge_final", q);
    if (m.ne == 8)
      k_edge_final<8, T><<<nblocks(EK), TPB, 0, q>>>(m, p, a, s);
    else
      k_edge_final<10, T><<<nblocks(EK), TPB, 0, q>>>(m, p, a, s);
  };
  auto run_cell = [&](cudaStream_t q) {
    NvtxRange r("h_tendency+tr_tendency");
    Scope sc("k_cell_final", q);
    k_cell_final<T><<<nblocks(CK), TPB, 0, q>>>(m, p, a, s);
  };
  // The final passes are independent unless the stage updates the state in
  // place (LSRK): there the edge pass reads h, which the cell pass rewrites,
  // so the edge pass goes first.
  if (edge && cell)
    fork_join(s.ep.mode == EPI_LSRK || g_profile ? nullptr : fk, st, run_edge,
              run_cell);
  else if (edge)
    run_edge(st);
  else if (cell)
    run_cell(st);
}

} // namespace

void launch_tendency(const MeshView &m, const ModelView &p, const AuxView &a,
                     const StageArgs &s, cudaStream_t st, const Fork *fk) {
  launch_tendency_t<double>(m, p, a, s, st, fk);
}

void launch_tendency_dual(const MeshView &m, const ModelView &p,
                          const AuxViewT<Dual> &a, const StageArgsT<Dual> &s,
                          cudaStream_t st) {
  launch_tendency_t<Dual>(m, p, a, s, st, nullptr);
}

void launch_aux(const MeshView &m, const ModelView &p, const AuxView &a,
                const double *h, const double *vn, const double *tr,
                cudaStream_t st, const Fork *fk) {
  launch_aux_t<double>(m, p, a, h, vn, tr, st, fk);
}

void launch_field_tendency(const MeshView &m, const ModelView &p,
                           const AuxView &a, int field, const double *h,
                           const double *vn, double *tend, int mode,
                           cudaStream_t st) {
  const long long K = m.nlayers, CK = m.ncells * K, EK = m.nedges * K;
  StageArgs s{};
  s.h = h;
  s.vn = vn;
  s.ep.mode = mode;
  ModelView q = p;
  if (p.linear) { // the linear terms read h and vn themselves
    if (field == 0) {
      s.fh.tend = tend;
      Scope sc("k_lin_cell", st);
      k_lin_cell<double><<<nblocks(CK), TPB, 0, st>>>(m, q, s);
    } else {
      s.fvn.tend = tend;
      Scope sc("k_lin_edge", st);
      if (m.ne == 8)
        k_lin_edge<8, double><<<nblocks(EK), TPB, 0, st>>>(m, q, s);
      else
        k_lin_edge<10, double><<<nblocks(EK), TPB, 0, st>>>(m, q, s);
    }
    return;
  }
  {
    Scope sc("k_field_flux", st);
    if (field == 1)
      k_field_flux<true><<<nblocks(EK), TPB, 0, st>>>(m, a, vn);
    else
      k_field_flux<false><<<nblocks(EK), TPB, 0, st>>>(m, a, vn);
  }
  if (field == 1) {
    s.fvn.tend = tend;
    NvtxRange r("vn_tendency");
    Scope sc("k_edge_final", st);
    if (m.ne == 8)
      k_edge_final<8, double><<<nblocks(EK), TPB, 0, st>>>(m, q, a, s);
    else
      k_edge_final<10, double><<<nblocks(EK), TPB, 0, st>>>(m, q, a, s);
    return;
  }
  // the cell pass writes h when do_h is set and the tracers when ntracers
  // > 0: one of the two per call
  q.do_h = field == 0;
  if (field == 0) {
    q.ntracers = 0;
    s.fh.tend = tend;
  } else {
    s.ftr.tend = tend;
  }
  NvtxRange r(field == 0 ? "h_tendency" : "tr_tendency");
  Scope sc("k_cell_final", st);
  k_cell_final<double><<<nblocks(CK), TPB, 0, st>>>(m, q, a, s);
}

int fork_create(Fork &f) {
  cudaError_t err = cudaStreamCreateWithFlags(&f.side, cudaStreamNonBlocking);
  if (err == cudaSuccess)
    err = cudaEventCreateWithFlags(&f.go, cudaEventDisableTiming);
  if (err == cudaSuccess)
    err = cudaEventCreateWithFlags(&f.done, cudaEventDisableTiming);
  if (err != cudaSuccess) {
    fork_destroy(f);
    return cuda_fail(err, "fork stream");
  }
  return SWG_OK;
}

void fork_destroy(Fork &f) {
  if (f.go)
    cudaEventDestroy(f.go);
  if (f.done)
    cudaEventDestroy(f.done);
  if (f.side)
    cudaStreamDestroy(f.side);
  f = Fork{};
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
