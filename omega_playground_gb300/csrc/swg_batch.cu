// Batched ensembles: many independent instances (uneven mesh size, level
// count and tracer count) advanced together.
//
// One RK stage of every member is one persistent cooperative kernel that
// runs the six passes of the tendency (swg_device.cuh) over all members,
// with a grid barrier between passes.  Work is cut into virtual blocks of
// blockDim*ITEMS (entity, level) elements; a per-pass prefix table over the
// members maps a virtual block to its member, and resident blocks stride
// over the virtual blocks.  The arithmetic per element is exactly the
// single-instance kernels', so a member advanced in a batch is bitwise equal
// to the same member advanced alone.
//
// The grid barrier spins on a generation counter with a clock64 limit; if it
// expires (which needs the co-residency that the cooperative launch
// guarantees to fail) the block records SWG_ERR_TIMEOUT in the batch's
// status word and the kernel returns; swg_batch_check reports it.
//
// An autotuner times the launch configurations (persistent vs one launch
// per pass, block size, elements per thread) on the batch itself and keeps
// the fastest.
#include "swg_device.cuh"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <new>

namespace swg {

struct BatchSync {
  unsigned count;
  unsigned gen;
  int status;
  int pad;
};

// Bounded grid barrier for a cooperative launch.  Thread 0 of each block
// arrives on `count`; the last arriver resets it and bumps `gen`; the others
// spin on `gen` for at most `limit` clock64 ticks.  Returns false when the
// barrier failed here or elsewhere (status set).
__device__ bool grid_barrier(BatchSync *bs, long long limit) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *vgen = &bs->gen;
    volatile int *vstatus = &bs->status;
    const unsigned g = *vgen;
    __threadfence();
    const unsigned arrived = atomicAdd(&bs->count, 1u) + 1u;
    ok = 1;
    if (arrived == gridDim.x) {
      atomicExch(&bs->count, 0u);
      __threadfence();
      atomicAdd(&bs->gen, 1u);
    } else {
      const long long t0 = clock64();
      while (*vgen == g) {
        if (*vstatus != 0 || clock64() - t0 > limit) {
          atomicCAS(&bs->status, 0, SWG_ERR_TIMEOUT);
          ok = 0;
          break;
        }
        __nanosleep(100);
      }
    }
    __threadfence();
    if (*vstatus != 0)
      ok = 0;
  }
  __syncthreads();
  return ok != 0;
}

template <int NE>
__device__ __forceinline__ void run_pass(int pass, const Member &M, int stage,
                                         unsigned i) {
  const StageArgs &s = M.stage[stage];
  switch (pass) {
  case P_VERTEX: pt_vertex(M.m, M.p, M.a, s.h, s.vn, i); break;
  case P_CELL1: pt_cell1(M.m, M.p, M.a, s.h, s.vn, s.tr, i); break;
  case P_EDGE1: pt_edge1(M.m, M.p, M.a, s.h, s.vn, i); break;
  case P_AUX2: pt_aux2(M.m, M.p, M.a, M.aux2_base + i); break;
  case P_EDGE_FINAL: pt_edge_final<NE, double>(M.m, M.p, M.a, s, i); break;
  default: pt_cell_final(M.m, M.p, M.a, s, i); break;
  }
}

// Passes [pass0, pass1] of stage `stage` for all members.  prefix[pass] has
// nmem+1 entries: virtual-block offsets of the members in that pass.
template <int NE, int ITEMS>
__global__ void __launch_bounds__(512)
    k_batch(const Member *__restrict__ mem, int nmem,
            const unsigned *__restrict__ prefix, int stage, int pass0,
            int pass1, BatchSync *bs, long long limit) {
  const unsigned vbsize = blockDim.x * ITEMS;
  for (int pass = pass0; pass <= pass1; ++pass) {
    const unsigned *pre = prefix + pass * (nmem + 1);
    const unsigned nvb = pre[nmem];
    for (unsigned vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
      int lo = 0, hi = nmem;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (pre[mid] <= vb)
          lo = mid;
        else
          hi = mid;
      }
      const Member &M = mem[lo];
      const unsigned n = M.units[pass];
      const unsigned first = (vb - pre[lo]) * vbsize + threadIdx.x;
#pragma unroll
      for (int it = 0; it < ITEMS; ++it) {
        const unsigned i = first + it * blockDim.x;
        if (i < n)
          run_pass<NE>(pass, M, stage, i);
      }
    }
    if (pass < pass1 && !grid_barrier(bs, limit))
      return;
  }
}

// One pass of one stage for all members (the per-pass launch shape), with
// the pass fixed at compile time: each pass kernel is compiled on its own,
// so a light pass does not carry the registers of the heaviest one and
// keeps the occupancy of the single-instance kernels.
template <int NE, int ITEMS, int PASS>
__global__ void __launch_bounds__(512)
    k_batch_pass(const Member *__restrict__ mem, int nmem,
                 const unsigned *__restrict__ prefix, int stage) {
  const unsigned vbsize = blockDim.x * ITEMS;
  const unsigned *pre = prefix + PASS * (nmem + 1);
  const unsigned nvb = pre[nmem];
  for (unsigned vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
    int lo = 0, hi = nmem;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (pre[mid] <= vb)
        lo = mid;
      else
        hi = mid;
    }
    const Member &M = mem[lo];
    const unsigned n = M.units[PASS];
    const unsigned first = (vb - pre[lo]) * vbsize + threadIdx.x;
#pragma unroll
    for (int it = 0; it < ITEMS; ++it) {
      const unsigned i = first + it * blockDim.x;
      if (i < n)
        run_pass<NE>(PASS, M, stage, i);
    }
  }
}

template <int NE, int ITEMS> void *pass_kernel(int pass) {
  switch (pass) {
  case P_VERTEX:
    return reinterpret_cast<void *>(&k_batch_pass<NE, ITEMS, P_VERTEX>);
  case P_CELL1:
    return reinterpret_cast<void *>(&k_batch_pass<NE, ITEMS, P_CELL1>);
  case P_EDGE1:
    return reinterpret_cast<void *>(&k_batch_pass<NE, ITEMS, P_EDGE1>);
  case P_AUX2:
    return reinterpret_cast<void *>(&k_batch_pass<NE, ITEMS, P_AUX2>);
  case P_EDGE_FINAL:
    return reinterpret_cast<void *>(&k_batch_pass<NE, ITEMS, P_EDGE_FINAL>);
  default:
    return reinterpret_cast<void *>(&k_batch_pass<NE, ITEMS, P_CELL_FINAL>);
  }
}

int batch_launch_passes(const Member *mem, int nmem, const unsigned *prefix,
                        const unsigned *prefix_h, int ne, int items,
                        int pass0, int pass1, int stage, cudaStream_t st) {
  for (int pass = pass0; pass <= pass1; ++pass) {
    const unsigned nvb = prefix_h[pass * (nmem + 1) + nmem];
    if (nvb == 0)
      continue;
    void *args[] = {&mem, &nmem, &prefix, &stage};
    void *fn = items == 2 ? (ne == 8 ? pass_kernel<8, 2>(pass)
                                     : pass_kernel<10, 2>(pass))
                          : (ne == 8 ? pass_kernel<8, 1>(pass)
                                     : pass_kernel<10, 1>(pass));
    cudaError_t err =
        cudaLaunchKernel(fn, dim3(nvb), dim3(256), args, 0, st);
    if (err != cudaSuccess)
      return cuda_fail(err, "batched passes: launch");
    ++g_launches;
  }
  return SWG_OK;
}

// A wait that nothing releases, for testing the barrier's time limit: every
// block but block 0 waits at a barrier block 0 never reaches.
__global__ void k_barrier_selftest(BatchSync *bs, long long limit) {
  if (blockIdx.x == 0)
    return;
  grid_barrier(bs, limit);
}

} // namespace swg

using namespace swg;

struct LaunchConfig {
  int persistent; // 1: one cooperative kernel per stage; 0: one launch per pass
  int block;      // threads per block
  int items;      // elements per thread per virtual block
};

static const LaunchConfig kConfigs[] = {
    {1, 256, 1}, {1, 128, 1}, {1, 512, 1}, {1, 256, 2}, {1, 128, 2},
    {0, 256, 1}, {0, 128, 1}, {0, 512, 1}, {0, 256, 2},
};
static const int kNumConfigs = sizeof(kConfigs) / sizeof(kConfigs[0]);

struct swg_batch_s {
  int nmem, kind, nstages, ne;
  std::vector<swg_model> models;
  std::vector<swg_state> states, tend, acc, p0, p1;
  std::vector<double> rka, rkb, rkc;
  Member *d_mem = nullptr;
  unsigned *d_prefix = nullptr;
  BatchSync *d_sync = nullptr;
  std::vector<unsigned> prefix_h; // host copy of the prefix tables
  std::vector<Member> mem_h;
  std::vector<unsigned long long> versions; // members' model versions built
  double dt_built = -1.0;
  int config = 0;
  int sms = 0;
  long long limit = 0;
  cudaGraphExec_t graph = nullptr;
  double graph_dt = 0;
  int graph_config = -1;
  long long graph_launches = 0;
};

void swg::batch_pass_units(const swg_model_s *md, unsigned units[NPASS],
                           unsigned &base) {
  const ModelView &p = md->view;
  const long long K = md->mesh->nlayers, C = md->mesh->ncells,
                  E = md->mesh->nedges, V = md->mesh->nvertices;
  const bool tr4 = p.ntracers > 0 && p.tr_del4;
  units[P_VERTEX] = p.do_vn ? unsigned(V * K) : 0;
  units[P_CELL1] = ((p.do_vn && (p.vel_del2 || p.vel_del4)) || p.ntracers > 0)
                       ? unsigned(C * K) : 0;
  units[P_EDGE1] = (p.do_vn || p.do_h || p.ntracers > 0) ? unsigned(E * K) : 0;
  base = (p.do_vn && p.vel_del4) ? 0u : unsigned(V * K);
  units[P_AUX2] = (p.do_vn || tr4) ? unsigned((V + C) * K) - base : 0;
  units[P_EDGE_FINAL] = p.do_vn ? unsigned(E * K) : 0;
  units[P_CELL_FINAL] = (p.do_h || p.ntracers > 0) ? unsigned(C * K) : 0;
}

namespace {

// Stage inputs/outputs of one member (same buffer rotation as the
// single-instance fused stepper).
StageArgs member_stage(const swg_batch_s *b, int m, int stage, double dt) {
  const ModelView &pv = b->models[m]->view;
  swg_state S = b->states[m];
  StageArgs a{};
  if (b->kind == SWG_STEPPER_LSRK) {
    swg_state T = b->tend[m];
    a.h = S->h;
    a.vn = S->vn;
    a.tr = S->tr;
    a.fh = {T->h, nullptr, nullptr, S->h};
    a.fvn = {T->vn, nullptr, nullptr, S->vn};
    a.ftr = {T->tr, nullptr, nullptr, S->tr};
    a.ep = {EPI_LSRK, b->rka[stage], dt * b->rkb[stage], 0.0};
    return a;
  }
  swg_state P[2] = {b->p0[m], b->p1[m]};
  swg_state in = stage == 0 ? S : P[(stage - 1) % 2];
  swg_state outp = stage < 3 ? P[stage % 2] : S;
  swg_state A = b->acc[m];
  a.h = pv.do_h ? in->h : S->h;
  a.vn = pv.do_vn ? in->vn : S->vn;
  a.tr = in->tr;
  a.fh = {nullptr, S->h, A->h, outp->h};
  a.fvn = {nullptr, S->vn, A->vn, outp->vn};
  a.ftr = {nullptr, S->tr, A->tr, outp->tr};
  const int mode =
      stage == 0 ? EPI_RK4_FIRST : (stage < 3 ? EPI_RK4_MID : EPI_RK4_LAST);
  a.ep = {mode, 0.0, dt * b->rkb[stage], stage < 3 ? dt * b->rka[stage] : 0.0};
  return a;
}

int upload_prefix(swg_batch b, unsigned vbsize);

// A member's model switched a tendency term since its descriptor was built:
// take its current view and pass sizes, and rebuild the prefix tables and
// the step graph (both hold the pass sizes).
int refresh_members(swg_batch b) {
  bool changed = false;
  for (int m = 0; m < b->nmem; ++m)
    if (b->versions[m] != b->models[m]->version) {
      Member &M = b->mem_h[m];
      M.p = b->models[m]->view;
      batch_pass_units(b->models[m], M.units, M.aux2_base);
      b->versions[m] = b->models[m]->version;
      changed = true;
    }
  if (!changed)
    return SWG_OK;
  b->dt_built = -1.0;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  const LaunchConfig &c = kConfigs[b->config];
  return upload_prefix(b, unsigned(c.block * c.items));
}

int upload_members(swg_batch b, double dt) {
  TRY(refresh_members(b));
  if (b->dt_built == dt)
    return SWG_OK;
  for (int m = 0; m < b->nmem; ++m)
    for (int s = 0; s < b->nstages; ++s)
      b->mem_h[m].stage[s] = member_stage(b, m, s, dt);
  cudaError_t err = cudaMemcpy(b->d_mem, b->mem_h.data(),
                               sizeof(Member) * b->nmem, cudaMemcpyHostToDevice);
  if (err != cudaSuccess)
    return cuda_fail(err, "swg_batch: member upload");
  b->dt_built = dt;
  return SWG_OK;
}

template <int NE, int ITEMS> void *kernel_ptr() {
  return reinterpret_cast<void *>(&k_batch<NE, ITEMS>);
}

void *pick_kernel(int ne, int items) {
  if (ne == 8)
    return items == 1 ? kernel_ptr<8, 1>() : kernel_ptr<8, 2>();
  return items == 1 ? kernel_ptr<10, 1>() : kernel_ptr<10, 2>();
}

template <int NE, int ITEMS> void *pass_kernel_ptr(int pass) {
  switch (pass) {
  case P_VERTEX: return reinterpret_cast<void *>(&k_batch_pass<NE, ITEMS, P_VERTEX>);
  case P_CELL1: return reinterpret_cast<void *>(&k_batch_pass<NE, ITEMS, P_CELL1>);
  case P_EDGE1: return reinterpret_cast<void *>(&k_batch_pass<NE, ITEMS, P_EDGE1>);
  case P_AUX2: return reinterpret_cast<void *>(&k_batch_pass<NE, ITEMS, P_AUX2>);
  case P_EDGE_FINAL:
    return reinterpret_cast<void *>(&k_batch_pass<NE, ITEMS, P_EDGE_FINAL>);
  default: return reinterpret_cast<void *>(&k_batch_pass<NE, ITEMS, P_CELL_FINAL>);
  }
}

void *pick_pass_kernel(int ne, int items, int pass) {
  if (ne == 8)
    return items == 1 ? pass_kernel_ptr<8, 1>(pass) : pass_kernel_ptr<8, 2>(pass);
  return items == 1 ? pass_kernel_ptr<10, 1>(pass) : pass_kernel_ptr<10, 2>(pass);
}

// prefix tables for one virtual-block size: [NPASS][nmem+1]
int upload_prefix(swg_batch b, unsigned vbsize) {
  std::vector<unsigned> pre(size_t(NPASS) * (b->nmem + 1));
  for (int pass = 0; pass < NPASS; ++pass) {
    unsigned acc = 0;
    for (int m = 0; m < b->nmem; ++m) {
      pre[pass * (b->nmem + 1) + m] = acc;
      acc += (b->mem_h[m].units[pass] + vbsize - 1) / vbsize;
    }
    pre[pass * (b->nmem + 1) + b->nmem] = acc;
  }
  cudaError_t err = cudaMemcpy(b->d_prefix, pre.data(),
                               pre.size() * sizeof(unsigned),
                               cudaMemcpyHostToDevice);
  if (err != cudaSuccess)
    return cuda_fail(err, "swg_batch: prefix upload");
  b->prefix_h = pre;
  return SWG_OK;
}

int launch_stage(swg_batch b, int stage, cudaStream_t st) {
  const LaunchConfig &c = kConfigs[b->config];
  void *fn = pick_kernel(b->ne, c.items);
  int nmem = b->nmem;
  const Member *mem = b->d_mem;
  const unsigned *pre = b->d_prefix;
  BatchSync *bs = b->d_sync;
  long long limit = b->limit;
  const unsigned vbsize = unsigned(c.block * c.items);
  if (c.persistent) {
    int per_sm = 0;
    cudaError_t err =
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, c.block, 0);
    if (err != cudaSuccess || per_sm < 1)
      return cuda_fail(err != cudaSuccess ? err : cudaErrorInvalidConfiguration,
                       "swg_batch: occupancy");
    // no more resident blocks than the largest pass has virtual blocks
    unsigned maxvb = 1;
    for (int pass = 0; pass < NPASS; ++pass)
      maxvb = std::max(maxvb, b->prefix_h[pass * (nmem + 1) + nmem]);
    const unsigned grid = std::min<unsigned>(unsigned(per_sm * b->sms), maxvb);
    int p0 = 0, p1 = NPASS - 1;
    void *args[] = {&mem, &nmem, &pre, &stage, &p0, &p1, &bs, &limit};
    err = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(c.block), args, 0, st);
    if (err != cudaSuccess)
      return cuda_fail(err, "swg_batch: cooperative launch");
    ++g_launches;
    return SWG_OK;
  }
  for (int pass = 0; pass < NPASS; ++pass) {
    const unsigned nvb = b->prefix_h[pass * (nmem + 1) + nmem];
    if (nvb == 0)
      continue;
    void *args[] = {&mem, &nmem, &pre, &stage};
    cudaError_t err = cudaLaunchKernel(pick_pass_kernel(b->ne, c.items, pass),
                                       dim3(nvb), dim3(c.block), args, 0, st);
    if (err != cudaSuccess)
      return cuda_fail(err, "swg_batch: pass launch");
    ++g_launches;
  }
  (void)vbsize;
  return SWG_OK;
}

int enqueue_step(swg_batch b, cudaStream_t st) {
  cudaError_t err = cudaMemsetAsync(b->d_sync, 0, 2 * sizeof(unsigned), st);
  if (err != cudaSuccess)
    return cuda_fail(err, "swg_batch: barrier reset");
  for (int s = 0; s < b->nstages; ++s)
    TRY(launch_stage(b, s, st));
  return SWG_OK;
}

int set_config(swg_batch b, int config) {
  if (config < 0 || config >= kNumConfigs)
    return fail(SWG_ERR_ARG, "swg_batch: unknown launch configuration");
  b->config = config;
  const LaunchConfig &c = kConfigs[config];
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  return upload_prefix(b, unsigned(c.block * c.items));
}

} // namespace

extern "C" int swg_batch_create(int nmembers, const swg_model *models,
                                const swg_state *states, int kind, int nstages,
                                swg_batch *out) try {
  if (!out || !models || !states || nmembers < 1)
    return fail(SWG_ERR_ARG, "swg_batch_create: bad argument");
  *out = nullptr;
  if (kind != SWG_STEPPER_RK4 && !(kind == SWG_STEPPER_LSRK &&
                                   (nstages == 5 || nstages == 1)))
    return fail(SWG_ERR_ARG, "swg_batch_create: RK4 or LSRK with 5/1 stages");
  int ne = 0;
  for (int m = 0; m < nmembers; ++m) {
    swg_model md = models[m];
    if (!md || !states[m] || states[m]->mesh != md->mesh ||
        states[m]->ntracers != md->params.ntracers)
      return fail(SWG_ERR_ARG, "swg_batch_create: member model/state mismatch");
    if (md->forcing)
      return fail(SWG_ERR_ARG, "swg_batch_create: members cannot have an "
                               "additional_tendency hook");
    if (md->view.linear)
      return fail(SWG_ERR_ARG, "swg_batch_create: linear models are not "
                               "batched");
    for (int j = 0; j < m; ++j)
      if (models[j] == md || states[j] == states[m])
        return fail(SWG_ERR_ARG, "swg_batch_create: a model or state appears "
                                 "in two members (their passes would write "
                                 "the same arrays concurrently)");
    if (ne && md->mesh->view.ne != ne)
      return fail(SWG_ERR_ARG, "swg_batch_create: members must share the "
                               "edges-on-edge width (8 or 10)");
    ne = md->mesh->view.ne;
  }
  swg_batch b = new (std::nothrow) swg_batch_s();
  if (!b)
    return fail(SWG_ERR_OOM, "swg_batch_create: host allocation");
  b->nmem = nmembers;
  b->kind = kind;
  b->ne = ne;
  b->models.assign(models, models + nmembers);
  b->states.assign(states, states + nmembers);
  if (kind == SWG_STEPPER_RK4) {
    b->nstages = 4;
    b->rka = {1. / 2, 1. / 2, 1};
    b->rkb = {1. / 6, 1. / 3, 1. / 3, 1. / 6};
    b->rkc = {1. / 2, 1. / 2, 1};
  } else if (nstages == 5) {
    b->nstages = 5;
    b->rka = {0., -567301805773. / 1357537059087.,
              -2404267990393. / 2016746695238.,
              -3550918686646. / 2091501179385.,
              -1275806237668. / 842570457699.};
    b->rkb = {1432997174477. / 9575080441755.,
              5161836677717. / 13612068292357.,
              1720146321549. / 2090206949498.,
              3134564353537. / 4481467310338.,
              2277821191437. / 14882151754819.};
    b->rkc = {0., 1432997174477. / 9575080441755.,
              2526269341429. / 6820363962896.,
              2006345519317. / 3224310063776.,
              2802321613138. / 2924317926251.};
  } else {
    b->nstages = 1;
    b->rka = {0};
    b->rkb = {1};
    b->rkc = {0};
  }
  int rc = SWG_OK;
  for (int m = 0; m < nmembers && rc == SWG_OK; ++m) {
    swg_model md = models[m];
    const int T = md->params.ntracers;
    swg_state t = nullptr, a = nullptr, q0 = nullptr, q1 = nullptr;
    if (kind == SWG_STEPPER_LSRK)
      rc = swg_state_create(md->mesh, T, &t);
    else if ((rc = swg_state_create(md->mesh, T, &a)) == SWG_OK &&
             (rc = swg_state_create(md->mesh, T, &q0)) == SWG_OK)
      rc = swg_state_create(md->mesh, T, &q1);
    b->tend.push_back(t);
    b->acc.push_back(a);
    b->p0.push_back(q0);
    b->p1.push_back(q1);
  }
  b->mem_h.resize(nmembers);
  for (int m = 0; m < nmembers; ++m) {
    Member &M = b->mem_h[m];
    std::memset(&M, 0, sizeof(M));
    M.m = models[m]->mesh->view;
    M.p = models[m]->view;
    M.a = models[m]->aux;
    batch_pass_units(models[m], M.units, M.aux2_base);
    b->versions.push_back(models[m]->version);
  }
  cudaError_t err = cudaSuccess;
  if (rc == SWG_OK) {
    err = cudaMalloc(&b->d_mem, sizeof(Member) * nmembers);
    if (err == cudaSuccess)
      err = cudaMalloc(&b->d_prefix, sizeof(unsigned) * NPASS * (nmembers + 1));
    if (err == cudaSuccess)
      err = cudaMalloc(&b->d_sync, sizeof(BatchSync));
    if (err == cudaSuccess)
      err = cudaMemset(b->d_sync, 0, sizeof(BatchSync));
    int dev = 0;
    if (err == cudaSuccess)
      err = cudaGetDevice(&dev);
    if (err == cudaSuccess)
      err = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    int khz = 0;
    if (err == cudaSuccess)
      err = cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev);
    // barrier wait limit: about one second of SM clock
    b->limit = (long long)std::max(khz, 1000000) * 1000LL;
    if (err != cudaSuccess)
      rc = cuda_fail(err, "swg_batch_create: device setup");
  }
  if (rc == SWG_OK)
    rc = set_config(b, 0);
  if (rc != SWG_OK) {
    swg_batch_destroy(b);
    return rc;
  }
  *out = b;
  return SWG_OK;
} SWG_ABI_CATCH("swg_batch_create")

extern "C" int swg_batch_destroy(swg_batch b) try {
  if (!b)
    return SWG_OK;
  if (b->graph)
    cudaGraphExecDestroy(b->graph);
  for (auto *v : {&b->tend, &b->acc, &b->p0, &b->p1})
    for (swg_state s : *v)
      swg_state_destroy(s);
  cudaFree(b->d_mem);
  cudaFree(b->d_prefix);
  cudaFree(b->d_sync);
  delete b;
  return SWG_OK;
} SWG_ABI_CATCH("swg_batch_destroy")

extern "C" int swg_batch_step(swg_batch b, double t0, double dt, int nsteps,
                              int use_graph, void *stream) try {
  (void)t0; // stage times only matter to forcing hooks, which batches exclude
  if (!b || nsteps < 0)
    return fail(SWG_ERR_ARG, "swg_batch_step: bad argument");
  NvtxRange range("time_integration");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  TRY(upload_members(b, dt));
  if (!use_graph) {
    for (int s = 0; s < nsteps; ++s)
      TRY(enqueue_step(b, st));
    return SWG_OK;
  }
  if (!b->graph || b->graph_dt != dt || b->graph_config != b->config) {
    if (b->graph) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
    cudaStream_t cs;
    cudaError_t err = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (err != cudaSuccess)
      return cuda_fail(err, "swg_batch_step: capture stream");
    const long long before = g_launches.load();
    err = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int rc = err == cudaSuccess ? enqueue_step(b, cs) : SWG_OK;
    cudaGraph_t g = nullptr;
    cudaError_t err2 = cudaStreamEndCapture(cs, &g);
    b->graph_launches = g_launches.load() - before;
    g_launches -= b->graph_launches;
    cudaStreamDestroy(cs);
    if (err != cudaSuccess || err2 != cudaSuccess || rc != SWG_OK) {
      if (g)
        cudaGraphDestroy(g);
      (void)cudaGetLastError();
      // graph capture of this launch shape is unavailable: direct launches
      for (int s = 0; s < nsteps; ++s)
        TRY(enqueue_step(b, st));
      return SWG_OK;
    }
    err = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (err != cudaSuccess) {
      b->graph = nullptr;
      return cuda_fail(err, "swg_batch_step: graph instantiate");
    }
    b->graph_dt = dt;
    b->graph_config = b->config;
  }
  for (int s = 0; s < nsteps; ++s) {
    cudaError_t err = cudaGraphLaunch(b->graph, st);
    if (err != cudaSuccess)
      return cuda_fail(err, "swg_batch_step: graph launch");
    g_launches += b->graph_launches;
  }
  return SWG_OK;
} SWG_ABI_CATCH("swg_batch_step")

extern "C" int swg_batch_check(swg_batch b, void *stream) try {
  if (!b)
    return fail(SWG_ERR_ARG, "swg_batch_check: NULL batch");
  BatchSync h{};
  cudaError_t err = cudaMemcpyAsync(&h, b->d_sync, sizeof(h),
                                    cudaMemcpyDeviceToHost,
                                    static_cast<cudaStream_t>(stream));
  if (err == cudaSuccess)
    err = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
  if (err != cudaSuccess)
    return cuda_fail(err, "swg_batch_check");
  if (h.status != 0) {
    cudaMemset(b->d_sync, 0, sizeof(BatchSync));
    return fail(SWG_ERR_TIMEOUT, "swg_batch: a grid barrier wait expired");
  }
  return SWG_OK;
} SWG_ABI_CATCH("swg_batch_check")

extern "C" int swg_batch_set_config(swg_batch b, int config) try {
  if (!b)
    return fail(SWG_ERR_ARG, "swg_batch_set_config: NULL batch");
  return set_config(b, config);
} SWG_ABI_CATCH("swg_batch_set_config")

extern "C" int swg_batch_config_count(void) { return kNumConfigs; }

extern "C" int swg_batch_autotune(swg_batch b, double dt, int reps,
                                  void *stream, int *best,
                                  double *best_ms) try {
  if (!b || !best || reps < 1)
    return fail(SWG_ERR_ARG, "swg_batch_autotune: bad argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  TRY(upload_members(b, dt));
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return fail(SWG_ERR_CUDA, "swg_batch_autotune: events");
  int arg_best = -1;
  float t_best = 0.f;
  int rc = SWG_OK;
  for (int c = 0; c < kNumConfigs && rc == SWG_OK; ++c) {
    if ((rc = set_config(b, c)) != SWG_OK)
      break;
    // warm-up step, then `reps` timed steps (direct launches)
    if ((rc = enqueue_step(b, st)) != SWG_OK) {
      // a shape this device cannot launch is skipped, not an error
      (void)cudaGetLastError();
      rc = SWG_OK;
      continue;
    }
    cudaEventRecord(e0, st);
    for (int r = 0; r < reps && rc == SWG_OK; ++r)
      rc = enqueue_step(b, st);
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = cuda_fail(cudaGetLastError(), "swg_batch_autotune");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rc == SWG_OK && (arg_best < 0 || ms < t_best)) {
      arg_best = c;
      t_best = ms;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  TRY(rc);
  if (arg_best < 0)
    return fail(SWG_ERR_CUDA, "swg_batch_autotune: no launch shape ran");
  TRY(set_config(b, arg_best));
  *best = arg_best;
  if (best_ms)
    *best_ms = t_best / reps;
  // the tuning steps advanced the members; callers re-upload their state
  return swg_batch_check(b, stream);
} SWG_ABI_CATCH("swg_batch_autotune")

extern "C" int swg_batch_selftest_timeout(swg_batch b, double limit_ms,
                                          void *stream) try {
  if (!b || !(limit_ms > 0) || limit_ms > 2000)
    return fail(SWG_ERR_ARG, "swg_batch_selftest_timeout: 0 < limit_ms <= 2000");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int dev = 0, khz = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev);
  long long limit = (long long)(std::max(khz, 1000000) * limit_ms);
  cudaError_t err = cudaMemsetAsync(b->d_sync, 0, sizeof(BatchSync), st);
  if (err != cudaSuccess)
    return cuda_fail(err, "swg_batch_selftest_timeout: reset");
  BatchSync *bs = b->d_sync;
  void *args[] = {&bs, &limit};
  // two co-resident blocks: block 1 waits for block 0, which never arrives
  err = cudaLaunchCooperativeKernel(reinterpret_cast<void *>(&k_barrier_selftest),
                                    dim3(2), dim3(32), args, 0, st);
  if (err != cudaSuccess)
    return cuda_fail(err, "swg_batch_selftest_timeout: launch");
  ++g_launches;
  return swg_batch_check(b, stream);
} SWG_ABI_CATCH("swg_batch_selftest_timeout")
