// Batched adjoint ensemble (swg_adj_ensemble_*): the checkpointed adjoints
// of many independent members advanced together, each schedule action one
// batched launch per pass over the members.
//
// Members whose schedules are identical (the same step count, snapshot
// budget and stepper) and whose adjoint kernels take the same compile-time
// switches (edges-on-edge width, tracer diffusion) form a group.  A group
// runs its members in lockstep: every action of the shared schedule is
// executed for all of them at once.
//  - Plain advances: a batch (swg_batch_*) of the members' current states.
//  - Taped advances and tapes: the batched tendency passes (swg_batch.cu)
//    over member tables of each (tape, stage), whose intermediates go to
//    the members' tapes and whose stage updates write the stage inputs.
//  - The adjoint of a step: batched adjoint passes (kb_adj) over member
//    tables of each (tape, stage), a virtual-block prefix table mapping
//    blocks to members as in the forward batch.
// Checkpoints stay per member (each member's own snapshots and budget).
// Groups with different schedules run on streams of their own, interleaved
// one action at a time.  A member's arithmetic is the single-instance
// adjoint's (the same device functions of swg_adjoint.cuh and
// swg_device.cuh), so its results are bitwise those of swg_adj_forward /
// swg_adj_backward on the member alone.
#include "swg_adjoint.cuh"

#include <algorithm>
#include <cstring>
#include <map>
#include <new>
#include <tuple>

namespace swg {
namespace {

// One member of a batched adjoint pass: everything one tendency-evaluation
// transpose reads, and the element range of each pass.
struct AdjMember {
  MeshView m;
  ModelView p;
  AuxView a;
  AdjView v;
  AdjWork w;
  AdjIO io;
  unsigned units[NAPASS], base[NAPASS];
};

// The block's member descriptor is copied to shared memory once per
// virtual block: the pass reads its tables and arrays through it many times
// per thread, and shared loads are cheaper than the global ones a
// reference into the member table would issue.
template <int PASS, int NE, bool D2, bool D4, bool TRD>
__global__ void __launch_bounds__(ATPB)
    kb_adj(const AdjMember *__restrict__ mem, int nmem,
           const unsigned *__restrict__ prefix) {
  __shared__ AdjMember M;
  constexpr int kWords = sizeof(AdjMember) / sizeof(unsigned long long);
  static_assert(sizeof(AdjMember) % sizeof(unsigned long long) == 0,
                "member descriptor copied in 8-byte words");
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
    __syncthreads(); // the previous virtual block is done with M
    const unsigned long long *src =
        reinterpret_cast<const unsigned long long *>(mem + lo);
    unsigned long long *dst = reinterpret_cast<unsigned long long *>(&M);
    for (int k = threadIdx.x; k < kWords; k += ATPB)
      dst[k] = src[k];
    __syncthreads();
    const unsigned j = (vb - pre[lo]) * ATPB + threadIdx.x;
    if (j < M.units[PASS])
      adj_pass<PASS, NE, D2, D4, TRD>(M.m, M.p, M.a, M.v, M.w, M.io,
                                      M.base[PASS] + j);
  }
}

using KbFn = void (*)(const AdjMember *, int, const unsigned *);

// Batched state copies: every member's state (h, vn and the tracers are one
// block of words) in one launch of kCopyChunk-word chunks, instead of a
// copy-engine transfer per member.  first[s] is the first chunk of segment
// s and first[nseg] the chunk count, so no chunk spans two segments.
struct CopySeg {
  double *dst;
  const double *src;
  unsigned long long n;
};
constexpr unsigned kCopyChunk = 4096;

__global__ void __launch_bounds__(256)
    kb_copy(const CopySeg *__restrict__ segs,
            const unsigned *__restrict__ first, int nseg) {
  const unsigned c = blockIdx.x;
  int lo = 0, hi = nseg;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (first[mid] <= c)
      lo = mid;
    else
      hi = mid;
  }
  const CopySeg sg = segs[lo];
  const unsigned long long base =
      (unsigned long long)(c - first[lo]) * kCopyChunk;
  for (unsigned j = threadIdx.x; j < kCopyChunk; j += 256) {
    const unsigned long long w = base + j;
    if (w < sg.n)
      sg.dst[w] = sg.src[w];
  }
}

// the kernel of a pass for a group's switches (the single-instance launcher
// in swg_adjoint.cu picks the same instantiations)
KbFn kb_fn(int pass, int ne, bool d2, bool d4, bool trd) {
  switch (pass) {
  case AP_VEL:
    return kb_adj<AP_VEL, 8, false, false, false>;
  case AP_TR1:
    if (d2)
      return d4 ? kb_adj<AP_TR1, 8, true, true, false>
                : kb_adj<AP_TR1, 8, true, false, false>;
    return d4 ? kb_adj<AP_TR1, 8, false, true, false>
              : kb_adj<AP_TR1, 8, false, false, false>;
  case AP_TR2:
    return d4 ? kb_adj<AP_TR2, 8, false, true, false>
              : kb_adj<AP_TR2, 8, false, false, false>;
  case AP_EDGE:
    if (ne == 8)
      return trd ? kb_adj<AP_EDGE, 8, false, false, true>
                 : kb_adj<AP_EDGE, 8, false, false, false>;
    return trd ? kb_adj<AP_EDGE, 10, false, false, true>
               : kb_adj<AP_EDGE, 10, false, false, false>;
  case AP_VERTEX:
    return kb_adj<AP_VERTEX, 8, false, false, false>;
  case AP_CELL:
    return kb_adj<AP_CELL, 8, false, false, false>;
  default:
    return kb_adj<AP_VN, 8, false, false, false>;
  }
}

struct Group {
  std::vector<swg_adjoint> adjs; // the members, in the ensemble's order
  int ns = 4, kind = SWG_STEPPER_RK4, nsnap = 1, ne = 8;
  bool d2 = false, d4 = false, trd = false;
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;
  Fork fork; // second stream for the independent passes
  // backward sweep: restores, stores, plain and taped advances run on
  // `adv`, tapes and adjoints on `st`, as in the single adjoint; `ready`
  // hands the advanced state to `st`, `freed` gives `cur` back once its tape
  // input is copied, free_ev[b] marks tape b read by its adjoint
  cudaStream_t adv = nullptr;
  cudaEvent_t ready = nullptr, freed = nullptr, free_ev[kTapes] = {};
  swg_batch plain = nullptr; // the members' current states, plain steps
  // forward tables [kTapes][ns][n] and their prefix [NPASS][n + 1]
  Member *d_fwd = nullptr;
  unsigned *d_fpre = nullptr;
  std::vector<unsigned> fpre;
  // adjoint tables [kTapes][ns][n] and their prefix [NAPASS][n + 1]
  AdjMember *d_adj = nullptr;
  unsigned *d_apre = nullptr;
  std::vector<unsigned> apre;
  double built_dt = -1.0;
  std::vector<unsigned long long> built_version;
  std::vector<AdjAction> acts;
  size_t pos = 0;
  AdjGraph g_tadv[kTapes], g_tape_adj[kTapes], g_adj[kTapes];
  // batched state copies: tables [copy][n] of (dst, src, words) and their
  // chunk offsets [copy][n + 1]; copy = snapshot k stored (k), restored
  // (nsnap + k), `cur` to tape b's step input (2 nsnap + b)
  CopySeg *d_copy = nullptr;
  unsigned *d_cfirst = nullptr;
  std::vector<unsigned> cchunks; // chunk count per copy
  int n() const { return int(adjs.size()); }
};

enum { COPY_STORE = 0, COPY_RESTORE = 1, COPY_X0 = 2 };

// one launch: copy `kind` (slot or tape `idx`) for every member of g
int group_copy(const Group &g, int kind, int idx, cudaStream_t st) {
  const int n = g.n();
  const int t = kind == COPY_STORE     ? idx
                : kind == COPY_RESTORE ? g.nsnap + idx
                                       : 2 * g.nsnap + idx;
  kb_copy<<<g.cchunks[t], 256, 0, st>>>(g.d_copy + size_t(t) * n,
                                        g.d_cfirst + size_t(t) * (n + 1), n);
  ++g_launches;
  const cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? SWG_OK
                            : cuda_fail(err, "swg_adj_ensemble: state copy");
}


void drop_graphs(Group &g) {
  for (int b = 0; b < kTapes; ++b)
    for (AdjGraph *gr : {&g.g_tadv[b], &g.g_tape_adj[b], &g.g_adj[b]})
      if (gr->exec) {
        cudaGraphExecDestroy(gr->exec);
        gr->exec = nullptr;
      }
}

template <class T>
int upload_table(const std::vector<T> &h, T **d) {
  if (!*d) {
    cudaError_t err = cudaMalloc(d, std::max<size_t>(h.size(), 1) * sizeof(T));
    if (err != cudaSuccess)
      return cuda_fail(err, "swg_adj_ensemble: table allocation");
  }
  cudaError_t err = cudaMemcpy(*d, h.data(), h.size() * sizeof(T),
                               cudaMemcpyHostToDevice);
  return err == cudaSuccess ? SWG_OK
                            : cuda_fail(err, "swg_adj_ensemble: table upload");
}

int build_copies(Group &g) {
  const int n = g.n(), ncopy = 2 * g.nsnap + kTapes;
  std::vector<CopySeg> segs(size_t(ncopy) * n);
  std::vector<unsigned> first(size_t(ncopy) * (n + 1));
  g.cchunks.assign(ncopy, 0);
  for (int t = 0; t < ncopy; ++t) {
    unsigned acc = 0;
    for (int m = 0; m < n; ++m) {
      swg_adjoint ad = g.adjs[m];
      auto blk = [](swg_state s) { return static_cast<double *>(s->block); };
      double *cur = blk(ad->cur);
      CopySeg &c = segs[size_t(t) * n + m];
      if (t < g.nsnap) {
        c = {blk(ad->snaps[t]), cur, words(ad->model)};
      } else if (t < 2 * g.nsnap) {
        c = {cur, blk(ad->snaps[t - g.nsnap]), words(ad->model)};
      } else {
        c = {blk(ad->tp[t - 2 * g.nsnap].X[0]), cur, words(ad->model)};
      }
      first[size_t(t) * (n + 1) + m] = acc;
      acc += unsigned((c.n + kCopyChunk - 1) / kCopyChunk);
    }
    first[size_t(t) * (n + 1) + n] = acc;
    g.cchunks[t] = acc;
  }
  TRY(upload_table(segs, &g.d_copy));
  return upload_table(first, &g.d_cfirst);
}

template <class U>
std::vector<unsigned> prefix_of(const std::vector<U> &first, int npass, int n,
                                unsigned vbsize) {
  // first[m] holds member m's units[] (its first (tape, stage) entry: the
  // pass sizes do not depend on the tape or the stage)
  std::vector<unsigned> pre(size_t(npass) * (n + 1));
  for (int q = 0; q < npass; ++q) {
    unsigned acc = 0;
    for (int m = 0; m < n; ++m) {
      pre[size_t(q) * (n + 1) + m] = acc;
      acc += (first[m].units[q] + vbsize - 1) / vbsize;
    }
    pre[size_t(q) * (n + 1) + n] = acc;
  }
  return pre;
}

// The member tables of every (tape, stage) for time step dt, rebuilt when dt
// or a member's term switches change (the tables hold the model views).
int build_tables(Group &g, double dt) {
  const int n = g.n(), ns = g.ns;
  bool same = g.built_dt == dt && int(g.built_version.size()) == n;
  for (int m = 0; same && m < n; ++m)
    same = g.built_version[m] == g.adjs[m]->model->version;
  if (same)
    return SWG_OK;
  std::vector<Member> fwd(size_t(kTapes) * ns * n);
  std::vector<AdjMember> adj(size_t(kTapes) * ns * n);
  for (int b = 0; b < kTapes; ++b)
    for (int s = 0; s < ns; ++s)
      for (int m = 0; m < n; ++m) {
        swg_adjoint ad = g.adjs[m];
        const swg_model_s *md = ad->model;
        const size_t k = (size_t(b) * ns + s) * n + m;
        Member &F = fwd[k];
        std::memset(&F, 0, sizeof(F));
        F.m = md->mesh->view;
        F.p = md->view;
        F.a = ad->tp[b].taux[s];
        F.stage[0] = tape_stage_args(ad, ad->tp[b], s, dt, ad->cur);
        batch_pass_units(md, F.units, F.aux2_base);
        AdjMember &A = adj[k];
        std::memset(&A, 0, sizeof(A));
        A.m = md->mesh->view;
        A.p = md->view;
        A.a = ad->tp[b].taux[s];
        // the last stage's PV sum is taped only by a taped advance; the
        // batched reversals share one table for both kinds of tape and
        // recompute it
        if (s == ns - 1)
          A.a.S1 = nullptr;
        A.v = ad->av;
        A.w = ad->aw;
        A.io = stage_io(ad, ad->tp[b], s, dt);
        adj_units(md, A.units, A.base);
      }
  // the taped passes take 2 elements per thread, the shape of the plain
  // batched steps (512-element virtual blocks)
  g.fpre = prefix_of(std::vector<Member>(fwd.begin(), fwd.begin() + n),
                     NPASS, n, 512);
  g.apre = prefix_of(std::vector<AdjMember>(adj.begin(), adj.begin() + n),
                     NAPASS, n, ATPB);
  TRY(upload_table(fwd, &g.d_fwd));
  TRY(upload_table(adj, &g.d_adj));
  TRY(upload_table(g.fpre, &g.d_fpre));
  TRY(upload_table(g.apre, &g.d_apre));
  drop_graphs(g);
  g.built_dt = dt;
  g.built_version.resize(n);
  for (int m = 0; m < n; ++m)
    g.built_version[m] = g.adjs[m]->model->version;
  return SWG_OK;
}

// Captures `record` once (while the tables stay the same) and replays it.
template <class Fn>
int g_replay(AdjGraph &gr, cudaStream_t st, Fn record) {
  if (!gr.exec) {
    cudaStream_t cs;
    cudaError_t err = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (err != cudaSuccess)
      return cuda_fail(err, "swg_adj_ensemble: capture stream");
    const long long before = g_launches.load();
    err = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int rc = SWG_OK;
    if (err == cudaSuccess)
      rc = record(cs);
    cudaGraph_t graph = nullptr;
    cudaError_t err2 = cudaStreamEndCapture(cs, &graph);
    gr.launches = g_launches.load() - before;
    g_launches -= gr.launches;
    cudaStreamDestroy(cs);
    if (err != cudaSuccess || err2 != cudaSuccess || rc != SWG_OK) {
      if (graph)
        cudaGraphDestroy(graph);
      (void)cudaGetLastError();
      return record(st); // direct launches
    }
    err = cudaGraphInstantiate(&gr.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (err != cudaSuccess) {
      gr.exec = nullptr;
      return cuda_fail(err, "swg_adj_ensemble: graph instantiate");
    }
  }
  cudaError_t err = cudaGraphLaunch(gr.exec, st);
  if (err != cudaSuccess)
    return cuda_fail(err, "swg_adj_ensemble: graph launch");
  g_launches += gr.launches;
  return SWG_OK;
}

// The taped step of every member into tape b: out_cur = the result replaces
// `cur` (a taped advance); otherwise the last stage records only its
// intermediates (a tape from a state).  copy_in: copy `cur` to the tape's
// step input first (else the caller did).
int batched_tape(Group &g, int b, bool out_cur, bool copy_in,
                 cudaStream_t st) {
  const int n = g.n(), ns = g.ns;
  if (copy_in)
    TRY(group_copy(g, COPY_X0, b, st));
  for (swg_adjoint ad : g.adjs)
    TRY(tape_prologue(ad, ad->tp[b], out_cur ? ad->cur : nullptr, st));
  for (int s = 0; s < ns; ++s) {
    const bool aux_only = s == ns - 1 && !out_cur;
    if (!aux_only)
      for (swg_adjoint ad : g.adjs)
        TRY(tape_stage_copy(ad, ad->tp[b], s, ad->cur, st));
    TRY(batch_launch_passes(g.d_fwd + (size_t(b) * ns + s) * n, n, g.d_fpre,
                            g.fpre.data(), g.ne, 2, P_VERTEX,
                            aux_only ? P_AUX2 : P_CELL_FINAL, 0, st));
  }
  return SWG_OK;
}

// The adjoint of the step taped in tape b, for every member.
int batched_adjoint(Group &g, int b, cudaStream_t st) {
  const int n = g.n(), ns = g.ns;
  if (ns % 2 != 0) // odd stage counts form the step's first mu here
    for (swg_adjoint ad : g.adjs)
      adj_lincomb(ad->mu, ad->lam, ad->dt * step_rkb(ad)[ns - 1],
                  (long long)words(ad->model), st);
  for (int s = ns - 1; s >= 0; --s) {
    const AdjMember *tab = g.d_adj + (size_t(b) * ns + s) * n;
    auto pass = [&](int q) {
      return [&, q](cudaStream_t qs) {
        const unsigned nvb = g.apre[size_t(q) * (n + 1) + n];
        if (nvb == 0)
          return;
        kb_fn(q, g.ne, g.d2, g.d4, g.trd)<<<nvb, ATPB, 0, qs>>>(tab, n,
                                                               g.d_apre);
        ++g_launches;
      };
    };
    // the independent pairs run as fork/join branches, as in the single
    // adjoint: velocity and tracer transposes, edge and tracer output,
    // cell and normal-velocity output
    fork_join(&g.fork, st, pass(AP_VEL), pass(AP_TR1));
    fork_join(&g.fork, st, pass(AP_EDGE), pass(AP_TR2));
    pass(AP_VERTEX)(st);
    fork_join(&g.fork, st, pass(AP_VN), pass(AP_CELL));
  }
  cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? SWG_OK
                            : cuda_fail(err, "swg_adj_ensemble: adjoint step");
}

cudaError_t hand_over(cudaEvent_t ev, cudaStream_t from, cudaStream_t to) {
  cudaError_t e = cudaEventRecord(ev, from);
  return e == cudaSuccess ? cudaStreamWaitEvent(to, ev, 0) : e;
}

// One schedule action for every member of the group.  two: the backward
// sweep's two streams (advances on g.adv, tapes and adjoints on g.st).
int group_action(Group &g, const AdjAction &a, bool two) {
  cudaStream_t st = g.st, q = two ? g.adv : g.st;
  cudaError_t e = cudaSuccess;
  switch (a.type) {
  case A_ADV: {
    swg_adjoint ad0 = g.adjs[0];
    for (swg_adjoint ad : g.adjs)
      ad->plain_steps += a.b;
    return swg_batch_step(g.plain, ad0->t0 + a.a * ad0->dt, ad0->dt, a.b, 1,
                          q);
  }
  case A_STORE:
    return group_copy(g, COPY_STORE, a.a, q);
  case A_RESTORE:
    return group_copy(g, COPY_RESTORE, a.a, q);
  case A_TADV:
    for (swg_adjoint ad : g.adjs) {
      ++ad->taped_steps;
      ++ad->taped_advances;
    }
    if (two && (e = cudaStreamWaitEvent(q, g.free_ev[a.b], 0)) != cudaSuccess)
      return cuda_fail(e, "swg_adj_ensemble: stream handshake");
    return g_replay(g.g_tadv[a.b], q, [&](cudaStream_t cs) {
      return batched_tape(g, a.b, true, true, cs);
    });
  case A_TAPE_ADJ:
  case A_ADJ:
    break;
  default:
    return SWG_OK;
  }
  // the state (and a taped advance's tape) from the advance stream
  if (two && (e = hand_over(g.ready, g.adv, st)) != cudaSuccess)
    return cuda_fail(e, "swg_adj_ensemble: stream handshake");
  int rc;
  if (a.type == A_TAPE_ADJ) {
    for (swg_adjoint ad : g.adjs)
      ++ad->taped_steps;
    TRY(group_copy(g, COPY_X0, a.b, st));
    // `cur` may be advanced again once its copy is taken
    if (two && (e = hand_over(g.freed, st, g.adv)) != cudaSuccess)
      return cuda_fail(e, "swg_adj_ensemble: stream handshake");
    rc = g_replay(g.g_tape_adj[a.b], st, [&](cudaStream_t cs) {
      TRY(batched_tape(g, a.b, false, false, cs));
      return batched_adjoint(g, a.b, cs);
    });
  } else {
    rc = g_replay(g.g_adj[a.b], st, [&](cudaStream_t cs) {
      return batched_adjoint(g, a.b, cs);
    });
  }
  if (rc == SWG_OK && two &&
      (e = cudaEventRecord(g.free_ev[a.b], st)) != cudaSuccess)
    return cuda_fail(e, "swg_adj_ensemble: stream handshake");
  return rc;
}

// the caller's stream (st) before the groups' streams, or after them
int streams_follow(const std::vector<Group> &gs, cudaStream_t st,
                   cudaEvent_t ev) {
  cudaError_t err = cudaEventRecord(ev, st);
  for (const Group &g : gs)
    for (cudaStream_t s : {g.st, g.adv})
      if (err == cudaSuccess)
        err = cudaStreamWaitEvent(s, ev, 0);
  return err == cudaSuccess ? SWG_OK
                            : cuda_fail(err, "swg_adj_ensemble: streams");
}
int caller_follows(const std::vector<Group> &gs, cudaStream_t st) {
  cudaError_t err = cudaSuccess;
  for (const Group &g : gs) {
    if (err == cudaSuccess)
      err = cudaEventRecord(g.done, g.st);
    if (err == cudaSuccess)
      err = cudaStreamWaitEvent(st, g.done, 0);
  }
  return err == cudaSuccess ? SWG_OK
                            : cuda_fail(err, "swg_adj_ensemble: streams");
}

bool same_layout(const swg_adjoint_s *ad, const swg_state_s *s) {
  return s && s->mesh == ad->model->mesh &&
         s->ntracers == ad->model->params.ntracers;
}

} // namespace
} // namespace swg

using namespace swg;

struct swg_adj_ensemble_s {
  std::vector<swg_adjoint> adjs;
  std::vector<Group> groups;
  std::vector<std::pair<int, int>> where; // member -> (group, index)
  cudaEvent_t go = nullptr;
  int state = 0; // 1: forward sweep done
};

extern "C" int swg_adj_ensemble_destroy(swg_adj_ensemble e) try {
  if (!e)
    return SWG_OK;
  for (Group &g : e->groups) {
    drop_graphs(g);
    swg_batch_destroy(g.plain);
    cudaFree(g.d_fwd);
    cudaFree(g.d_fpre);
    cudaFree(g.d_adj);
    cudaFree(g.d_apre);
    cudaFree(g.d_copy);
    cudaFree(g.d_cfirst);
    for (cudaEvent_t ev : {g.done, g.ready, g.freed})
      if (ev)
        cudaEventDestroy(ev);
    for (cudaEvent_t ev : g.free_ev)
      if (ev)
        cudaEventDestroy(ev);
    fork_destroy(g.fork);
    for (cudaStream_t s : {g.st, g.adv})
      if (s)
        cudaStreamDestroy(s);
  }
  if (e->go)
    cudaEventDestroy(e->go);
  delete e;
  return SWG_OK;
} SWG_ABI_CATCH("swg_adj_ensemble_destroy")

extern "C" int swg_adj_ensemble_create(int n, const swg_adjoint *adjs,
                                       swg_adj_ensemble *out) try {
  if (n < 1 || !adjs || !out)
    return fail(SWG_ERR_ARG, "swg_adj_ensemble_create: bad argument");
  *out = nullptr;
  for (int a = 0; a < n; ++a) {
    if (!adjs[a])
      return fail(SWG_ERR_ARG, "swg_adj_ensemble_create: NULL member");
    for (int b = 0; b < a; ++b)
      if (adjs[a] == adjs[b] || adjs[a]->model == adjs[b]->model)
        return fail(SWG_ERR_ARG, "swg_adj_ensemble_create: members must have "
                                 "distinct adjoints and models (their passes "
                                 "run in the same launches)");
  }
  swg_adj_ensemble e = new (std::nothrow) swg_adj_ensemble_s();
  if (!e)
    return fail(SWG_ERR_OOM, "swg_adj_ensemble_create: host allocation");
  e->adjs.assign(adjs, adjs + n);
  // groups: identical schedule and kernel switches
  std::map<std::tuple<int, int, int, int, int, int, int>, int> key_to_group;
  for (int a = 0; a < n; ++a) {
    swg_adjoint ad = adjs[a];
    const ModelView &p = ad->model->view;
    const bool trd = p.ntracers > 0 && (p.tr_del2 || p.tr_del4);
    const auto key = std::make_tuple(ad->nsnap, ad->kind, ad->ns,
                                     ad->model->mesh->view.ne, int(p.tr_del2),
                                     int(p.tr_del4), int(trd));
    auto it = key_to_group.find(key);
    if (it == key_to_group.end()) {
      it = key_to_group.emplace(key, int(e->groups.size())).first;
      Group g;
      g.nsnap = ad->nsnap;
      g.kind = ad->kind;
      g.ns = ad->ns;
      g.ne = ad->model->mesh->view.ne;
      g.d2 = p.tr_del2;
      g.d4 = p.tr_del4;
      g.trd = trd;
      e->groups.push_back(g);
    }
    Group &g = e->groups[it->second];
    e->where.push_back({it->second, g.n()});
    g.adjs.push_back(ad);
  }
  int rc = SWG_OK;
  cudaError_t err = cudaEventCreateWithFlags(&e->go, cudaEventDisableTiming);
  for (Group &g : e->groups) {
    for (cudaStream_t *s : {&g.st, &g.adv})
      if (err == cudaSuccess)
        err = cudaStreamCreateWithFlags(s, cudaStreamNonBlocking);
    for (cudaEvent_t *ev : {&g.done, &g.ready, &g.freed})
      if (err == cudaSuccess)
        err = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    for (cudaEvent_t &ev : g.free_ev)
      if (err == cudaSuccess)
        err = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (err == cudaSuccess && fork_create(g.fork) != SWG_OK)
      err = cudaErrorMemoryAllocation;
    if (err != cudaSuccess)
      break;
    std::vector<swg_model> models;
    std::vector<swg_state> curs;
    for (swg_adjoint ad : g.adjs) {
      models.push_back(ad->model);
      curs.push_back(ad->cur);
    }
    rc = swg_batch_create(g.n(), models.data(), curs.data(), g.kind, g.ns,
                          &g.plain);
    if (rc == SWG_OK)
      rc = build_copies(g);
    // one launch per pass, 256 threads x 2 elements (the ensemble's usual
    // fastest shape)
    if (rc == SWG_OK)
      rc = swg_batch_set_config(g.plain, swg_batch_config_count() - 1);
    if (rc != SWG_OK)
      break;
  }
  if (err != cudaSuccess)
    rc = cuda_fail(err, "swg_adj_ensemble_create: streams");
  if (rc != SWG_OK) {
    swg_adj_ensemble_destroy(e);
    return rc;
  }
  *out = e;
  return SWG_OK;
} SWG_ABI_CATCH("swg_adj_ensemble_create")

extern "C" int swg_adj_ensemble_forward(swg_adj_ensemble e,
                                        const swg_state *states0, double t0,
                                        double dt, int nsteps,
                                        const swg_state *finals,
                                        void *stream) try {
  if (!e || !states0 || !finals || nsteps < 1)
    return fail(SWG_ERR_ARG, "swg_adj_ensemble_forward: bad argument");
  if (nsteps > 10000)
    return fail(SWG_ERR_ARG, "swg_adj_ensemble_forward: more steps than the "
                             "schedule planner takes (10000)");
  const int n = int(e->adjs.size());
  for (int a = 0; a < n; ++a)
    if (!same_layout(e->adjs[a], states0[a]) ||
        !same_layout(e->adjs[a], finals[a]))
      return fail(SWG_ERR_ARG, "swg_adj_ensemble_forward: member mismatch");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  NvtxRange range("adjoint_forward_sweep");
  for (Group &g : e->groups) {
    g.acts = plan_schedule(nsteps, g.nsnap, g.ns);
    long long plain = 0;
    for (const AdjAction &a : g.acts)
      plain += a.type == A_ADV ? a.b : 0;
    if (plain > 32LL * nsteps)
      return fail(SWG_ERR_BUDGET, "swg_adj_ensemble_forward: too few "
                                  "snapshots for a member: the schedule would "
                                  "re-run more than 32 plain steps per step");
    g.pos = 0;
  }
  for (int a = 0; a < n; ++a) {
    swg_adjoint ad = e->adjs[a];
    ad->t0 = t0;
    ad->dt = dt;
    ad->nsteps = nsteps;
    ad->plain_steps = ad->taped_steps = ad->taped_advances = 0;
    ad->fwd_terms = term_set(ad->model);
    ad->state = 0;
    TRY(swg_state_copy(ad->cur, states0[a], st));
  }
  for (Group &g : e->groups)
    TRY(build_tables(g, dt));
  TRY(streams_follow(e->groups, st, e->go));
  // the groups' forward sweeps, one action per group in turn
  for (size_t left = e->groups.size(); left > 0;) {
    left = 0;
    for (Group &g : e->groups) {
      if (g.pos >= g.acts.size() || g.acts[g.pos].type == A_FWD_END)
        continue;
      TRY(group_action(g, g.acts[g.pos++], false));
      ++left;
    }
  }
  for (int a = 0; a < n; ++a) {
    const Group &g = e->groups[e->where[a].first];
    TRY(swg_state_copy(finals[a], e->adjs[a]->cur, g.st));
    e->adjs[a]->state = 1;
  }
  for (Group &g : e->groups)
    ++g.pos; // past the end-of-forward marker
  e->state = 1;
  return caller_follows(e->groups, st);
} SWG_ABI_CATCH("swg_adj_ensemble_forward")

extern "C" int swg_adj_ensemble_backward(swg_adj_ensemble e,
                                         const swg_state *lambdas,
                                         void *stream) try {
  if (!e || !lambdas)
    return fail(SWG_ERR_ARG, "swg_adj_ensemble_backward: bad argument");
  if (e->state != 1)
    return fail(SWG_ERR_STATE, "swg_adj_ensemble_backward: call "
                               "swg_adj_ensemble_forward first");
  const int n = int(e->adjs.size());
  for (int a = 0; a < n; ++a) {
    swg_adjoint ad = e->adjs[a];
    if (!same_layout(ad, lambdas[a]))
      return fail(SWG_ERR_ARG, "swg_adj_ensemble_backward: member mismatch");
    if (ad->state != 1)
      return fail(SWG_ERR_STATE, "swg_adj_ensemble_backward: a member's "
                                 "adjoint ran another forward sweep since");
    if (term_set(ad->model) != ad->fwd_terms)
      return fail(SWG_ERR_STATE, "swg_adj_ensemble_backward: a tendency term "
                                 "of a member's model was switched after the "
                                 "forward sweep");
  }
  for (Group &g : e->groups)
    TRY(build_tables(g, g.adjs[0]->dt)); // the same tables unless switched
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  NvtxRange range("adjoint_backward_sweep");
  TRY(streams_follow(e->groups, st, e->go));
  for (int a = 0; a < n; ++a) {
    swg_adjoint ad = e->adjs[a];
    cudaStream_t gs = e->groups[e->where[a].first].st;
    TRY(swg_state_copy(ad->lam, lambdas[a], gs));
    if (ad->ns % 2 == 0) // the first step's first mu
      adj_lincomb(ad->mu, ad->lam, ad->dt * step_rkb(ad)[ad->ns - 1],
                  (long long)words(ad->model), gs);
    if (ad->aw.gc2e) {
      cudaError_t err = cudaMemsetAsync(
          ad->aw.gc2e, 0,
          sizeof(double) * ad->model->mesh->nedges * ad->model->mesh->nlayers,
          gs);
      if (err != cudaSuccess)
        return cuda_fail(err, "swg_adj_ensemble_backward: gradient reset");
    }
  }
  for (size_t left = e->groups.size(); left > 0;) {
    left = 0;
    for (Group &g : e->groups) {
      if (g.pos >= g.acts.size())
        continue;
      TRY(group_action(g, g.acts[g.pos++], true));
      ++left;
    }
  }
  for (Group &g : e->groups) { // the advance stream's last work before st's
    cudaError_t err = hand_over(g.ready, g.adv, g.st);
    if (err != cudaSuccess)
      return cuda_fail(err, "swg_adj_ensemble_backward: streams");
  }
  for (int a = 0; a < n; ++a) {
    swg_adjoint ad = e->adjs[a];
    TRY(swg_state_copy(lambdas[a], ad->lam, e->groups[e->where[a].first].st));
    ad->state = 0;
    ad->grad_ready = true;
  }
  e->state = 0;
  return caller_follows(e->groups, st);
} SWG_ABI_CATCH("swg_adj_ensemble_backward")

extern "C" int swg_adj_ensemble_groups(swg_adj_ensemble e, int *ngroups,
                                       int *group_of) try {
  if (!e || !ngroups)
    return fail(SWG_ERR_ARG, "swg_adj_ensemble_groups: bad argument");
  *ngroups = int(e->groups.size());
  if (group_of)
    for (size_t a = 0; a < e->where.size(); ++a)
      group_of[a] = e->where[a].first;
  return SWG_OK;
} SWG_ABI_CATCH("swg_adj_ensemble_groups")
