// Tendency evaluation that allocates nothing (swg_compute_tendency_noalloc).
//
// Some callers cannot allocate device memory while they run: a host
// framework that owns the whole device pool and forbids libraries from
// calling cudaMalloc after start-up, or code that must not trigger the
// implicit synchronisation an allocation can cause.  swg_model_create
// allocates the parameter tables and the intermediate fields of a tendency
// evaluation, so it is out of reach for them.  This entry point instead
// keeps both in one fixed device array compiled into the library, and takes
// the state and tendency arrays as device pointers from the caller.
//
// The array holds SWG_NOALLOC_SCRATCH_BYTES (64 MiB).  Its device memory is
// committed when the library's device code is loaded into a context: at
// context creation with eager module loading, or under CUDA's default lazy
// loading at the first launch of one of this library's kernels in that
// context.  It is held until the context is destroyed (normally process
// exit).  In host code the array's name is only a host-side stand-in, never
// a device address.  The address belongs to the CUDA context, not to the
// device: it is looked up with cudaGetSymbolAddress, with the device
// current, the first time a call runs in a context, and cached under that
// context's unique ID (cuCtxGetId, never reused in a process).  A call in
// another context (a non-primary one, or the primary context re-created
// after cudaDeviceReset) therefore looks the address up again instead of
// using a stale one.  All calls share the array: each call rewrites every
// scratch element it later reads, so nothing has to start at zero, but
// calls that overlap on the GPU (different streams, no ordering between
// them) race on it.
#include "swg_internal.h"

#include <cuda.h> // driver types only; the entry points are looked up

#include <algorithm>
#include <cstdio>
#include <mutex>

namespace swg {
namespace {

constexpr size_t kScratchBytes = size_t(64) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Scratch address per device, valid for the context whose ID is ctx_id.
struct ScratchAddr {
  unsigned long long ctx_id = 0;
  unsigned char *addr = nullptr;
};
ScratchAddr g_scratch_addr[kMaxDevices];
std::mutex g_scratch_mu;

// cuCtxGetCurrent / cuCtxGetId through the runtime's driver entry points,
// so the library does not link libcuda itself.
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

// The unique ID of the calling thread's current context (making the
// device's primary context current if none is), or 0 when the driver does
// not offer cuCtxGetId.
int current_context_id(int dev, unsigned long long *id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000,
                                         cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000,
                                         cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
    (void)cudaGetLastError();
  });
  *id = 0;
  if (!get_current || !get_id)
    return SWG_OK;
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS)
    return fail(SWG_ERR_CUDA, "swg_compute_tendency_noalloc: cuCtxGetCurrent");
  if (!ctx) { // no context bound to this thread yet: bind the primary one
    cudaError_t err = cudaSetDevice(dev);
    if (err != cudaSuccess)
      return cuda_fail(err, "swg_compute_tendency_noalloc: cudaSetDevice");
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx)
      return fail(SWG_ERR_CUDA,
                  "swg_compute_tendency_noalloc: no current context");
  }
  if (get_id(ctx, id) != CUDA_SUCCESS)
    return fail(SWG_ERR_CUDA, "swg_compute_tendency_noalloc: cuCtxGetId");
  return SWG_OK;
}

// The scratch array's device address in the current context: cached per
// (device, context ID); looked up again in a context not seen before.
int scratch_address(int dev, unsigned char **out) {
  unsigned long long id = 0;
  TRY(current_context_id(dev, &id));
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  ScratchAddr &c = g_scratch_addr[dev];
  if (id == 0 || c.ctx_id != id || !c.addr) {
    void *ptr = nullptr;
    cudaError_t err = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (err != cudaSuccess || !ptr)
      return cuda_fail(err != cudaSuccess ? err : cudaErrorInvalidSymbol,
                       "swg_compute_tendency_noalloc: cudaGetSymbolAddress");
    c.addr = static_cast<unsigned char *>(ptr);
    c.ctx_id = id; // 0 (no cuCtxGetId): never matches, looked up every call
  }
  *out = c.addr;
  return SWG_OK;
}

// Parameter-scaled tables of a model, the same expressions swg_model_create
// evaluates on the host (shallow_water_model.cpp:5-41 enables the terms).
__global__ void k_noalloc_tables(MeshView m, double f0, double grav,
                                 double visc2, double visc4, double kappa2,
                                 double kappa4, double *f_vertex, double *gidc,
                                 double *c2e, double *c4e, double *kd2,
                                 double *r4, double *r4sum, double *r4f,
                                 double *c4i, double *c4v) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < m.nvertices)
    f_vertex[i] = f0;
  if (i < m.nedges) {
    gidc[i] = grav * m.inv_dc[i];
    c2e[i] = visc2 * m.scale2[i];
    const double c4 = -(visc4 * m.scale4[i]);
    c4e[i] = c4;
    c4i[i] = c4 * m.inv_dc[i];
    c4v[i] = -(c4 * m.inv_dv[i]);
  }
  if (i < m.ncells) {
    double s = 0;
    for (int j = 0; j < MAXE; ++j) {
      const int e = m.ec[6 * i + j];
      kd2[6 * i + j] = kappa2 * m.scale2[e] * m.ckq[6 * i + j];
      const double r = -(kappa4 * m.scale4[e] * m.ckq[6 * i + j]);
      r4[6 * i + j] = r;
      s += r;
    }
    r4sum[i] = s;
    if (r4f) // uniform del2 scaling: the tracer del2 folded into del4
      r4f[i] = kappa2 * m.scale2[0] - s;
  }
}

// Bump allocator over the scratch array: offsets only, 256-byte aligned.
struct Carve {
  unsigned char *base;
  size_t used = 0;
  double *take(size_t words) {
    used = (used + 255) & ~size_t(255);
    double *p = base ? reinterpret_cast<double *>(base + used) : nullptr;
    used += words * sizeof(double);
    return p;
  }
};

// Lays out the model tables and the intermediates the enabled terms need;
// with base == nullptr it only measures.
size_t layout(const swg_mesh_s *mesh, const ModelView &pv, unsigned char *base,
              double *tab[10], AuxView &a) {
  const size_t C = mesh->ncells, E = mesh->nedges, V = mesh->nvertices,
               K = mesh->nlayers, T = pv.ntracers;
  Carve cv{base};
  tab[0] = cv.take(V);     // f_vertex
  tab[1] = cv.take(E);     // gidc
  tab[2] = cv.take(E);     // c2e
  tab[3] = cv.take(E);     // c4e
  tab[4] = cv.take(6 * C); // kd2
  tab[5] = cv.take(6 * C); // r4
  tab[6] = cv.take(C);     // r4sum
  tab[7] = cv.take(C);     // r4f
  tab[8] = cv.take(E);     // c4i
  tab[9] = cv.take(E);     // c4v
  const bool vn = pv.do_vn;
  const bool vdiss = vn && (pv.vel_del2 || pv.vel_del4);
  const bool v4 = vn && pv.vel_del4;
  const bool trd = T > 0 && (pv.tr_del2 || pv.tr_del4);
  a = AuxView{};
  if (vn) a.q = cv.take(V * K);
  if (vdiss) a.zeta = cv.take(V * K);
  if (v4) a.z4 = cv.take(V * K);
  if (vdiss) a.div = cv.take(C * K);
  if (vn) a.ke = cv.take(C * K);
  if (v4) a.d4 = cv.take(C * K);
  if (T > 0) a.ntr = cv.take(T * C * K);
  if (T > 0 && pv.tr_del4) a.lap = cv.take(T * C * K);
  a.F = cv.take(E * K);
  if (vn) a.G = cv.take(E * K);
  if (vn) a.Q = cv.take(E * K);
  if (trd) a.mh = cv.take(E * K);
  if (vn) a.u2 = cv.take(E * K);
  if (vdiss) a.d2u = cv.take(E * K);
  a.d2u4 = (v4 && mesh->view.dv4_differs) ? cv.take(E * K) : a.d2u;
  return cv.used;
}

} // namespace
} // namespace swg

using namespace swg;

extern "C" int swg_compute_tendency_noalloc(swg_mesh mesh,
                                            const swg_params *params,
                                            const double *h, const double *vn,
                                            const double *tr, double *h_tend,
                                            double *vn_tend, double *tr_tend,
                                            int add_mode, void *stream) try {
  if (!mesh || !params || !h || !vn || !h_tend || !vn_tend ||
      params->ntracers < 0 || (params->ntracers > 0 && (!tr || !tr_tend)))
    return fail(SWG_ERR_ARG, "swg_compute_tendency_noalloc: bad argument");
  if (add_mode != SWG_ADD_REPLACE && add_mode != SWG_ADD_INCREMENT)
    return fail(SWG_ERR_ARG, "swg_compute_tendency_noalloc: bad add_mode");
  ModelView pv{};
  pv.grav = params->grav;
  pv.ntracers = params->ntracers;
  pv.vel_del2 = params->visc_del2 > 0;
  pv.vel_del4 = params->visc_del4 > 0;
  pv.tr_del2 = params->eddy_diff2 > 0;
  pv.tr_del4 = params->eddy_diff4 > 0;
  pv.do_h = !params->disable_h_tendency;
  pv.do_vn = !params->disable_vn_tendency;
  double *tab[10];
  AuxView a;
  const size_t need = layout(mesh, pv, nullptr, tab, a);
  if (need > kScratchBytes) {
    char msg[200];
    std::snprintf(msg, sizeof msg,
                  "swg_compute_tendency_noalloc: this mesh and parameter set "
                  "need %zu bytes of scratch; the static maximum is %zu bytes "
                  "(64 MiB)", need, kScratchBytes);
    return fail(SWG_ERR_ARG, msg);
  }
  // the array's device address in the current context, with the device
  // current (looked up once per context)
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess)
    return cuda_fail(err, "swg_compute_tendency_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices)
    return fail(SWG_ERR_ARG, "swg_compute_tendency_noalloc: device ordinal "
                             "above 63");
  unsigned char *base = nullptr;
  TRY(scratch_address(dev, &base));
  layout(mesh, pv, base, tab, a);
  pv.f_vertex = tab[0];
  pv.gidc = tab[1];
  pv.c2e = tab[2];
  pv.c4e = tab[3];
  pv.kd2 = tab[4];
  pv.r4 = tab[5];
  pv.r4sum = tab[6];
  const bool fold = mesh->scale2_uniform && pv.ntracers > 0 && pv.tr_del2 &&
                    pv.tr_del4;
  pv.r4f = fold ? tab[7] : nullptr;
  pv.c4i = tab[8];
  pv.c4v = tab[9];
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const MeshView &m = mesh->view;
  const long long n = std::max<long long>(
      std::max<long long>(m.nvertices, m.nedges), m.ncells);
  k_noalloc_tables<<<unsigned((n + 255) / 256), 256, 0, st>>>(
      m, params->f0, params->grav, params->visc_del2, params->visc_del4,
      params->eddy_diff2, params->eddy_diff4, tab[0], tab[1], tab[2], tab[3],
      tab[4], tab[5], tab[6], fold ? tab[7] : nullptr, tab[8], tab[9]);
  ++g_launches;
  StageArgs s{};
  s.h = h;
  s.vn = vn;
  s.tr = tr;
  s.fh.tend = h_tend;
  s.fvn.tend = vn_tend;
  s.ftr.tend = tr_tend;
  s.ep.mode = add_mode == SWG_ADD_REPLACE ? EPI_REPLACE : EPI_INCREMENT;
  {
    // the per-kernel profiler (swg_profile_enable) creates an event pair per
    // launch; this path creates no driver objects, so it is never timed
    ProfileOff no_timing;
    launch_tendency(m, pv, a, s, st);
  }
  err = cudaGetLastError();
  return err == cudaSuccess
             ? SWG_OK
             : cuda_fail(err, "swg_compute_tendency_noalloc: launch");
} SWG_ABI_CATCH("swg_compute_tendency_noalloc")
