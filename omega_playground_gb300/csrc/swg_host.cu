// Stepping a host-resident state in level chunks (swg_host_stepper_*).
//
// Every tendency term of the model reads and writes one vertical level at a
// time (the functors of shallow_water_model.cpp:43-311 index [entity][k]
// with the same k on both sides), so a state's levels [k0, k0 + kc) evolve
// independently of the others.  The one term tied to a level's position,
// the opt-in bottom drag, is given its level in each slice.  The host stepper cuts the levels into
// chunks and gives each chunk a level slice of the caller's model: a mesh
// that shares the caller's device tables but has kc levels (and its own
// slice of the per-level edge mask), a model whose view is the caller's,
// a device state of kc levels and an ordinary stepper with its graph.
// A call copies chunk c in on one stream, steps it on another (two compute
// streams take the chunks in turn) and copies it out on a fourth, so with
// page-locked host arrays the copies of one chunk overlap the compute of its
// neighbours.  Each level sees the same kernels
// and operands as in the unsliced model, so the results are bitwise equal.
//
// With page-locked mapped host arrays and a few steps per call, the whole
// call (copies in, the chunks' steps, copies out, across the three streams)
// is captured once into one CUDA graph and replayed: the host then makes one
// launch per call instead of a hundred-odd API calls, so a host thread that
// is held up while it issues them (by another process's driver calls, say)
// no longer leaves the copy engines and the SMs idle mid-call.
#include "swg_internal.h"

#include <algorithm>
#include <cstddef>
#include <new>
#include <vector>

using namespace swg;

namespace {

struct Chunk {
  int k0 = 0, kc = 0;
  swg_mesh mesh = nullptr;
  swg_model model = nullptr;
  swg_state state = nullptr;
  swg_stepper stepper = nullptr;
  cudaEvent_t in = nullptr, out = nullptr;
};

// Levels [k0, k0 + kc) of `src`: the K-independent device tables are
// shared (not owned: the slice frees only its own edge-mask copy), the
// per-level edge mask is copied, and the per-column maximum levels of the
// diagnostics are dropped (slices run no diagnostics).
int mesh_slice(swg_mesh src, int k0, int kc, swg_mesh *out) {
  swg_mesh m = new (std::nothrow) swg_mesh_s(*src);
  if (!m)
    return fail(SWG_ERR_OOM, "swg_host_stepper_create: host allocation");
  m->allocs.clear();
  m->nlayers = kc;
  m->view.nlayers = kc;
  m->view.maxlev_c = m->view.maxlev_v = nullptr;
  if (src->view.mask) {
    const size_t E = src->nedges, K = src->nlayers;
    void *d = nullptr;
    cudaError_t err = cudaMalloc(&d, E * kc * sizeof(double));
    if (err == cudaSuccess) {
      m->allocs.push_back(d);
      err = cudaMemcpy2D(d, kc * sizeof(double), src->view.mask + k0,
                         K * sizeof(double), kc * sizeof(double), E,
                         cudaMemcpyDeviceToDevice);
    }
    if (err != cudaSuccess) {
      swg_mesh_destroy(m);
      return cuda_fail(err, "swg_host_stepper_create: edge mask slice");
    }
    m->view.mask = static_cast<const double *>(d);
  }
  *out = m;
  return SWG_OK;
}

// Copy levels [k0, k0 + kc) of `rows` rows of K levels between the host
// array and a dense [rows][kc] device array.
cudaError_t copy_levels(double *dst, size_t dpitch, const double *src,
                        size_t spitch, int kc, size_t rows,
                        cudaMemcpyKind kind, cudaStream_t st) {
  if (rows == 0)
    return cudaSuccess;
  return cudaMemcpy2DAsync(dst, dpitch * sizeof(double), src,
                           spitch * sizeof(double), kc * sizeof(double), rows,
                           kind, st);
}

// Levels [k0, k0 + kc) of `rows` rows of K levels between host memory
// mapped into the device address space and a dense [rows][kc] device array,
// moved by the SMs.  The copy engines move rows of a few levels at a
// fraction of the link rate (64-byte rows at about half of it); a grid of
// threads issuing the rows together runs near the full rate.  Every index
// stays inside its array: r*K + k0 + j < rows*K because k0 + kc <= K.
__global__ void k_levels_in(double *__restrict__ dst,
                            const double *__restrict__ host, long long rows,
                            int K, int k0, int kc) {
  const long long n = rows * kc;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / kc;
    dst[i] = host[r * K + k0 + (i - r * kc)];
  }
}

__global__ void k_levels_out(double *__restrict__ host,
                             const double *__restrict__ src, long long rows,
                             int K, int k0, int kc) {
  const long long n = rows * kc;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / kc;
    host[r * K + k0 + (i - r * kc)] = src[i];
  }
}

// The device address of a host array of n doubles when the whole array is
// page-locked memory mapped into the device address space (cudaHostAlloc,
// or cudaHostRegister with mapping): both ends are mapped host memory at the
// same offset.  nullptr otherwise (pageable or managed memory), which keeps
// those arrays on the copy engines.
double *mapped(double *p, size_t n) {
  if (!p || n == 0)
    return nullptr;
  cudaPointerAttributes a{}, b{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess ||
      cudaPointerGetAttributes(&b, p + (n - 1)) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || b.type != cudaMemoryTypeHost ||
      !a.devicePointer || !b.devicePointer ||
      static_cast<double *>(b.devicePointer) -
              static_cast<double *>(a.devicePointer) !=
          std::ptrdiff_t(n - 1))
    return nullptr;
  return static_cast<double *>(a.devicePointer);
}

} // namespace

// One captured call: valid for the same host arrays (and their device
// mappings), dt, step count and model term version.
struct CallGraph {
  cudaGraphExec_t exec = nullptr;
  const double *h = nullptr, *vn = nullptr, *tr = nullptr;
  const double *mh = nullptr, *mv = nullptr, *mt = nullptr;
  double dt = 0;
  int nsteps = 0;
  unsigned long long version = 0;
  long long launches = 0;       // kernels one replay runs
  unsigned long long used = 0;  // last use (least recently used is replaced)
};
constexpr int kCallGraphs = 4;     // cached captured calls per stepper
constexpr int kCallGraphSteps = 4; // calls of more steps launch directly

struct swg_host_stepper_s {
  swg_model model = nullptr;
  int K = 0, T = 0;
  int copy_grid = 0; // blocks of the SM copies (8 per SM)
  std::vector<Chunk> chunks;
  // copies in, compute (even chunks on comp, odd ones on comp2, so a
  // chunk's last passes overlap the next chunk's first ones), copies out
  cudaStream_t h2d = nullptr, comp = nullptr, comp2 = nullptr, d2h = nullptr;
  cudaStream_t cap = nullptr; // origin of the call captures
  cudaEvent_t go = nullptr, done = nullptr;
  CallGraph graphs[kCallGraphs];
  unsigned long long uses = 0;
};

extern "C" int swg_host_stepper_destroy(swg_host_stepper hs) try {
  if (!hs)
    return SWG_OK;
  for (Chunk &c : hs->chunks) {
    swg_stepper_destroy(c.stepper);
    swg_state_destroy(c.state);
    swg_model_destroy(c.model);
    swg_mesh_destroy(c.mesh);
    if (c.in)
      cudaEventDestroy(c.in);
    if (c.out)
      cudaEventDestroy(c.out);
  }
  for (CallGraph &g : hs->graphs)
    if (g.exec)
      cudaGraphExecDestroy(g.exec);
  for (cudaStream_t s : {hs->h2d, hs->comp, hs->comp2, hs->d2h, hs->cap})
    if (s)
      cudaStreamDestroy(s);
  for (cudaEvent_t e : {hs->go, hs->done})
    if (e)
      cudaEventDestroy(e);
  delete hs;
  return SWG_OK;
} SWG_ABI_CATCH("swg_host_stepper_destroy")

static int make_chunk(swg_host_stepper hs, int kind, int nstages, Chunk &c) {
  swg_model src = hs->model;
  TRY(mesh_slice(src->mesh, c.k0, c.kc, &c.mesh));
  swg_model_options o{};
  o.linear = src->view.linear;
  o.h0 = src->view.h0;
  o.apply_drag = src->view.drag;
  TRY(swg_model_create_ex(c.mesh, &src->params, &o, &c.model));
  TRY(swg_state_create(c.mesh, hs->T, &c.state));
  TRY(swg_stepper_create(c.model, kind, nstages, &c.stepper));
  cudaError_t err = cudaEventCreateWithFlags(&c.in, cudaEventDisableTiming);
  if (err == cudaSuccess)
    err = cudaEventCreateWithFlags(&c.out, cudaEventDisableTiming);
  return err == cudaSuccess ? SWG_OK
                            : cuda_fail(err, "swg_host_stepper_create: events");
}

extern "C" int swg_host_stepper_create_levels(swg_model model, int kind,
                                              int nstages, int nchunks,
                                              const int *levels,
                                              swg_host_stepper *out) try {
  if (!model || !out || nchunks < 1 || !levels)
    return fail(SWG_ERR_ARG, "swg_host_stepper_create: bad argument");
  *out = nullptr;
  if (model->forcing)
    return fail(SWG_ERR_ARG, "swg_host_stepper_create: the model has a "
                             "forcing hook (it would see level slices)");
  long long sum = 0;
  for (int i = 0; i < nchunks; ++i) {
    if (levels[i] < 1)
      return fail(SWG_ERR_ARG, "swg_host_stepper_create: a chunk needs at "
                               "least one level");
    sum += levels[i];
  }
  if (sum != model->mesh->nlayers)
    return fail(SWG_ERR_ARG, "swg_host_stepper_create: the chunks' levels "
                             "must add up to the model's level count");
  swg_host_stepper hs = new (std::nothrow) swg_host_stepper_s();
  if (!hs)
    return fail(SWG_ERR_OOM, "swg_host_stepper_create: host allocation");
  hs->model = model;
  hs->K = model->mesh->nlayers;
  hs->T = model->params.ntracers;
  for (int i = 0, k0 = 0; i < nchunks; k0 += levels[i++]) {
    Chunk c;
    c.k0 = k0;
    c.kc = levels[i];
    hs->chunks.push_back(c);
  }
  int rc = SWG_OK;
  for (Chunk &c : hs->chunks)
    if ((rc = make_chunk(hs, kind, nstages, c)) != SWG_OK) {
      swg_host_stepper_destroy(hs);
      return rc;
    }
  cudaError_t err = cudaSuccess;
  int dev = 0, sms = 0;
  if ((err = cudaGetDevice(&dev)) == cudaSuccess)
    err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  hs->copy_grid = 8 * std::max(sms, 1);
  for (cudaStream_t *s : {&hs->h2d, &hs->comp, &hs->comp2, &hs->d2h, &hs->cap})
    if (err == cudaSuccess)
      err = cudaStreamCreateWithFlags(s, cudaStreamNonBlocking);
  for (cudaEvent_t *e : {&hs->go, &hs->done})
    if (err == cudaSuccess)
      err = cudaEventCreateWithFlags(e, cudaEventDisableTiming);
  if (err != cudaSuccess) {
    swg_host_stepper_destroy(hs);
    return cuda_fail(err, "swg_host_stepper_create: streams");
  }
  *out = hs;
  return SWG_OK;
} SWG_ABI_CATCH("swg_host_stepper_create_levels")

extern "C" int swg_host_stepper_create(swg_model model, int kind, int nstages,
                                       int level_chunk,
                                       swg_host_stepper *out) try {
  if (!model || !out)
    return fail(SWG_ERR_ARG, "swg_host_stepper_create: NULL argument");
  const int K = model->mesh->nlayers;
  const int kc = level_chunk <= 0 || level_chunk > K ? K : level_chunk;
  std::vector<int> levels;
  for (int k0 = 0; k0 < K; k0 += kc)
    levels.push_back(std::min(kc, K - k0));
  return swg_host_stepper_create_levels(model, kind, nstages,
                                        int(levels.size()), levels.data(), out);
} SWG_ABI_CATCH("swg_host_stepper_create")

extern "C" int swg_host_stepper_chunks(swg_host_stepper hs, int *levels,
                                       int *n) try {
  if (!hs || !n)
    return fail(SWG_ERR_ARG, "swg_host_stepper_chunks: NULL argument");
  if (levels)
    for (int i = 0; i < *n && i < int(hs->chunks.size()); ++i)
      levels[i] = hs->chunks[i].kc;
  *n = int(hs->chunks.size());
  return SWG_OK;
} SWG_ABI_CATCH("swg_host_stepper_chunks")

// Everything one call does, ordered after `origin` and before it again:
// copies in, each chunk's steps (its step graph when use_graph, else direct
// launches, as inside a capture), copies out.  mh, mv, mt: the device
// addresses of the mapped host arrays, or all nullptr (copy engines only).
static int enqueue_call(swg_host_stepper hs, double *h, double *vn, double *tr,
                        double *mh, double *mv, double *mt, double t0,
                        double dt, int nsteps, int use_graph,
                        cudaStream_t origin) {
  swg_model src = hs->model;
  const size_t K = hs->K, C = src->mesh->ncells, E = src->mesh->nedges,
               TC = size_t(hs->T) * C;
  // The first chunk's copy-in precedes all compute and the last chunk's
  // copy-out follows it, so the SMs are idle then: those two go through the
  // SM copies when the arrays are mapped page-locked memory.  The other
  // chunks' copies overlap compute and stay on the copy engines.
  const bool sm_copies = mh && mv && (mt || !TC);
  auto levels_in = [&](double *dst, const double *host, size_t rows, int k0,
                       int kc) {
    if (rows == 0)
      return cudaSuccess;
    k_levels_in<<<hs->copy_grid, 256, 0, hs->h2d>>>(dst, host, (long long)rows,
                                                    int(K), k0, kc);
    ++g_launches;
    return cudaGetLastError();
  };
  auto levels_out = [&](double *host, const double *src, size_t rows, int k0,
                        int kc) {
    if (rows == 0)
      return cudaSuccess;
    k_levels_out<<<hs->copy_grid, 256, 0, hs->d2h>>>(host, src,
                                                     (long long)rows, int(K),
                                                     k0, kc);
    ++g_launches;
    return cudaGetLastError();
  };
  cudaError_t err = cudaEventRecord(hs->go, origin);
  for (cudaStream_t s : {hs->h2d, hs->comp, hs->comp2, hs->d2h})
    if (err == cudaSuccess)
      err = cudaStreamWaitEvent(s, hs->go, 0);
  // copies in, back to back on the copy-in stream
  for (Chunk &c : hs->chunks) {
    const int kc = c.kc;
    if (sm_copies && &c == &hs->chunks.front()) {
      if (err == cudaSuccess)
        err = levels_in(c.state->h, mh, C, c.k0, kc);
      if (err == cudaSuccess)
        err = levels_in(c.state->vn, mv, E, c.k0, kc);
      if (err == cudaSuccess && TC)
        err = levels_in(c.state->tr, mt, TC, c.k0, kc);
    } else {
      if (err == cudaSuccess)
        err = copy_levels(c.state->h, kc, h + c.k0, K, kc, C,
                          cudaMemcpyHostToDevice, hs->h2d);
      if (err == cudaSuccess)
        err = copy_levels(c.state->vn, kc, vn + c.k0, K, kc, E,
                          cudaMemcpyHostToDevice, hs->h2d);
      if (err == cudaSuccess && TC)
        err = copy_levels(c.state->tr, kc, tr + c.k0, K, kc, TC,
                          cudaMemcpyHostToDevice, hs->h2d);
    }
    if (err == cudaSuccess)
      err = cudaEventRecord(c.in, hs->h2d);
  }
  if (err != cudaSuccess)
    return cuda_fail(err, "swg_host_step: copy in");
  // each chunk's steps once its levels are in, alternating between two
  // compute streams (chunks own their models and intermediates, so two can
  // run at once); the slice model takes the caller's current view (term
  // switches, f_vertex) and its version, so a switch recaptures the chunk's
  // step graph
  int ci = 0;
  for (Chunk &c : hs->chunks) {
    cudaStream_t cs = (ci++ % 2) ? hs->comp2 : hs->comp;
    err = cudaStreamWaitEvent(cs, c.in, 0);
    if (err != cudaSuccess)
      return cuda_fail(err, "swg_host_step: stream order");
    c.model->view = src->view;
    // the bottom drag acts on the caller's lowest level only: in the slice
    // holding it that is level drag_level - k0, in the others no level
    c.model->view.drag_level = src->view.drag_level - c.k0;
    c.model->version = src->version;
    c.model->terms_switched = src->terms_switched;
    TRY(swg_step(c.stepper, c.state, t0, dt, nsteps, use_graph, cs));
    err = cudaEventRecord(c.out, cs);
    if (err != cudaSuccess)
      return cuda_fail(err, "swg_host_step: stream order");
  }
  // copies out as each chunk finishes
  for (Chunk &c : hs->chunks) {
    const int kc = c.kc;
    if (err == cudaSuccess)
      err = cudaStreamWaitEvent(hs->d2h, c.out, 0);
    if (sm_copies && &c == &hs->chunks.back()) {
      if (err == cudaSuccess)
        err = levels_out(mh, c.state->h, C, c.k0, kc);
      if (err == cudaSuccess)
        err = levels_out(mv, c.state->vn, E, c.k0, kc);
      if (err == cudaSuccess && TC)
        err = levels_out(mt, c.state->tr, TC, c.k0, kc);
      continue;
    }
    if (err == cudaSuccess)
      err = copy_levels(h + c.k0, K, c.state->h, kc, kc, C,
                        cudaMemcpyDeviceToHost, hs->d2h);
    if (err == cudaSuccess)
      err = copy_levels(vn + c.k0, K, c.state->vn, kc, kc, E,
                        cudaMemcpyDeviceToHost, hs->d2h);
    if (err == cudaSuccess && TC)
      err = copy_levels(tr + c.k0, K, c.state->tr, kc, kc, TC,
                        cudaMemcpyDeviceToHost, hs->d2h);
  }
  if (err == cudaSuccess)
    err = cudaEventRecord(hs->done, hs->d2h);
  if (err == cudaSuccess)
    err = cudaStreamWaitEvent(origin, hs->done, 0);
  return err == cudaSuccess ? SWG_OK : cuda_fail(err, "swg_host_step");
}

// The captured call for these arrays, dt, step count and term version,
// captured now if no cached one matches; nullptr when the capture fails
// (the caller then launches the call directly).
static CallGraph *call_graph(swg_host_stepper hs, double *h, double *vn,
                             double *tr, double *mh, double *mv, double *mt,
                             double t0, double dt, int nsteps) {
  const unsigned long long version = hs->model->version;
  for (CallGraph &g : hs->graphs)
    if (g.exec && g.h == h && g.vn == vn && g.tr == tr && g.mh == mh &&
        g.mv == mv && g.mt == mt && g.dt == dt && g.nsteps == nsteps &&
        g.version == version) {
      g.used = ++hs->uses;
      return &g;
    }
  CallGraph *slot = &hs->graphs[0];
  for (CallGraph &g : hs->graphs)
    if (!g.exec || g.used < slot->used)
      slot = &g;
  if (slot->exec) {
    cudaGraphExecDestroy(slot->exec);
    slot->exec = nullptr;
  }
  const long long before = g_launches.load();
  cudaError_t err =
      cudaStreamBeginCapture(hs->cap, cudaStreamCaptureModeThreadLocal);
  int rc = SWG_OK;
  if (err == cudaSuccess)
    rc = enqueue_call(hs, h, vn, tr, mh, mv, mt, t0, dt, nsteps, 0, hs->cap);
  cudaGraph_t g = nullptr;
  const cudaError_t err2 =
      err == cudaSuccess ? cudaStreamEndCapture(hs->cap, &g) : err;
  const long long launches = g_launches.load() - before;
  g_launches -= launches; // captured, not launched
  cudaGraphExec_t exec = nullptr;
  if (err == cudaSuccess && err2 == cudaSuccess && rc == SWG_OK && g)
    err = cudaGraphInstantiate(&exec, g, 0);
  if (g)
    cudaGraphDestroy(g);
  if (err != cudaSuccess || err2 != cudaSuccess || rc != SWG_OK || !exec) {
    (void)cudaGetLastError();
    if (exec)
      cudaGraphExecDestroy(exec);
    return nullptr;
  }
  slot->exec = exec;
  slot->h = h;
  slot->vn = vn;
  slot->tr = tr;
  slot->mh = mh;
  slot->mv = mv;
  slot->mt = mt;
  slot->dt = dt;
  slot->nsteps = nsteps;
  slot->version = version;
  slot->launches = launches;
  slot->used = ++hs->uses;
  return slot;
}

static int host_step(swg_host_stepper hs, double *h, double *vn, double *tr,
                     double t0, double dt, int nsteps, void *stream) {
  swg_model src = hs->model;
  if (src->forcing)
    return fail(SWG_ERR_ARG, "swg_host_step: the model has a forcing hook "
                             "(it would see level slices)");
  const size_t K = hs->K, C = src->mesh->ncells, E = src->mesh->nedges,
               TC = size_t(hs->T) * C;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  NvtxRange range("host_step");
  double *mh = mapped(h, C * K), *mv = mapped(vn, E * K),
         *mt = TC ? mapped(tr, TC * K) : nullptr;
  if (!(mh && mv && (mt || !TC)))
    mh = mv = mt = nullptr;
  cudaError_t err = cudaSuccess;
  // the steps carry no time (the model has no forcing hook), so t0 does not
  // enter the captured call
  CallGraph *g = mh && nsteps > 0 && nsteps <= kCallGraphSteps &&
                         !profiling_enabled()
                     ? call_graph(hs, h, vn, tr, mh, mv, mt, t0, dt, nsteps)
                     : nullptr;
  if (g) {
    err = cudaGraphLaunch(g->exec, st);
    if (err == cudaSuccess)
      g_launches += g->launches;
  } else {
    TRY(enqueue_call(hs, h, vn, tr, mh, mv, mt, t0, dt, nsteps, 1, st));
  }
  if (err == cudaSuccess)
    err = cudaStreamSynchronize(st);
  return err == cudaSuccess ? SWG_OK : cuda_fail(err, "swg_host_step");
}

extern "C" int swg_host_step(swg_host_stepper hs, double *h, double *vn,
                             double *tr, double t0, double dt, int nsteps,
                             void *stream) try {
  if (!hs || !h || !vn || (hs->T > 0 && !tr) || nsteps < 0)
    return fail(SWG_ERR_ARG, "swg_host_step: bad argument");
  const int rc = host_step(hs, h, vn, tr, t0, dt, nsteps, stream);
  if (rc != SWG_OK) // no copy queued before the failure outlives the call
    for (cudaStream_t s : {hs->h2d, hs->comp, hs->comp2, hs->d2h})
      cudaStreamSynchronize(s);
  return rc;
} SWG_ABI_CATCH("swg_host_step")

extern "C" int swg_host_alloc(unsigned long long bytes, void **out) try {
  if (!out)
    return fail(SWG_ERR_ARG, "swg_host_alloc: NULL argument");
  *out = nullptr;
  cudaError_t err = cudaHostAlloc(out, bytes ? bytes : 1,
                                  cudaHostAllocMapped | cudaHostAllocPortable);
  if (err != cudaSuccess) {
    *out = nullptr;
    return cuda_fail(err, "swg_host_alloc");
  }
  return SWG_OK;
} SWG_ABI_CATCH("swg_host_alloc")

extern "C" int swg_host_free(void *p) try {
  if (!p)
    return SWG_OK;
  cudaError_t err = cudaFreeHost(p);
  return err == cudaSuccess ? SWG_OK : cuda_fail(err, "swg_host_free");
} SWG_ABI_CATCH("swg_host_free")
