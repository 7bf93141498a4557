// Adjoint (reverse mode) and tangent-linear (forward mode) models of the
// RK4 shallow-water step, with binomial checkpointing.
//
// Tangent-linear model: the tendency passes of swg_device.cuh instantiated
// on dual numbers (value, tangent); their value part is the forward's exact
// operation sequence, so the TLM is the exact derivative of the discrete
// forward.  Used by swg_tlm_tendency / swg_tlm_apply and to check the
// adjoint with dot-product tests.
//
// Adjoint of one tendency evaluation F at a state X: given mu (adjoint of the
// tendency), lambda = J(X)^T mu.  Hand-written, seven gather-only passes (no
// atomics): every transposed stencil reads its neighbours' coefficients from
// transposed tables built on the host (the neighbour's coefficient for a
// shared edge, per-edge copies of the two cells' / vertices' coefficients,
// and the transposed edges-on-edge list).  Intermediates of F at X come from
// the forward auxiliary passes (launch_aux).  Reference terms transposed:
// thickness_hadv_cell.hpp:59-83, pv_flux_edge.hpp:149-177,
// ke_grad_edge.hpp:223-237, ssh_grad_edge.hpp:281-294,
// vel_diff_edge.hpp:61-86, vel_hyperdiff_edge.hpp:237-334,
// tracer_hadv_cell.hpp:60-90, tracer_diff_cell.hpp:162-193,
// tracer_hyperdiff_cell.hpp:301-368, and the auxiliary variables
// (vorticity_aux.hpp, kinetic_aux.hpp, thickness_aux.hpp, tracer_aux.hpp).
//
// RK4 step adjoint (rk4.cpp:28-104): with stage inputs X0..X3 recorded by a
// taped forward step, mu_3 = dt b3 lam, mu_s = dt b_s lam + dt a_s lamX_{s+1},
// lamX_s = J(X_s)^T mu_s, and lam_i = lam_{i+1} + sum_s lamX_s.
//
// Checkpointing: a binomial schedule (Griewank-Walther) for n steps and s
// snapshots with two tapes, computed by dynamic programming over (n, s):
// the forward sweep stores the schedule's checkpoints and tapes the last
// steps; the backward sweep restores, re-advances and reverses each step
// once, in reverse order, taping the last step of a re-advance on the way
// when the planner finds that cheaper (see Planner).
#include "swg_adjoint.cuh"

#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>

namespace swg {
namespace {

// Single-instance launches of the passes (swg_adjoint.cuh): one thread per
// element of the pass's domain, starting at `base`.
__global__ void __launch_bounds__(ATPB)
    ka_vel(MeshView m, ModelView p, AuxView a, AdjView v, AdjWork w,
           AdjIO io, unsigned base) {
  pa_vel(m, p, a, v, w, io, base + blockIdx.x * ATPB + threadIdx.x);
}
template <bool D2, bool D4>
__global__ void __launch_bounds__(ATPB)
    ka_tr1(MeshView m, ModelView p, AuxView a, AdjView v, AdjWork w,
           AdjIO io) {
  pa_tr1<D2, D4>(m, p, a, v, w, io, blockIdx.x * ATPB + threadIdx.x);
}
template <bool D4>
__global__ void __launch_bounds__(ATPB)
    ka_tr2(MeshView m, ModelView p, AuxView a, AdjView v, AdjWork w,
           AdjIO io) {
  pa_tr2<D4>(m, p, a, v, w, io, blockIdx.x * ATPB + threadIdx.x);
}
template <int NE, bool TRD>
__global__ void __launch_bounds__(ATPB)
    ka_edge(MeshView m, ModelView p, AuxView a, AdjView v, AdjWork w,
            AdjIO io) {
  pa_edge<NE, TRD>(m, p, a, v, w, io, blockIdx.x * ATPB + threadIdx.x);
}
__global__ void __launch_bounds__(ATPB)
    ka_vertex(MeshView m, ModelView p, AuxView a, AdjView v, AdjWork w,
              AdjIO io) {
  pa_vertex(m, p, a, v, w, io, blockIdx.x * ATPB + threadIdx.x);
}
__global__ void __launch_bounds__(ATPB)
    ka_cell(MeshView m, ModelView p, AuxView a, AdjView v, AdjWork w,
            AdjIO io) {
  pa_cell(m, p, a, v, w, io, blockIdx.x * ATPB + threadIdx.x);
}
__global__ void __launch_bounds__(ATPB)
    ka_vn(MeshView m, ModelView p, AuxView a, AdjView v, AdjWork w,
          AdjIO io) {
  pa_vn(m, p, a, v, w, io, blockIdx.x * ATPB + threadIdx.x);
}

// y = alpha x1 + beta x2 (x2 may be null); dual pack / unpack
__global__ void ka_lincomb(double *y, const double *x1, const double *x2,
                           double alpha, double beta, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n)
    y[i] = x2 ? fma(alpha, x1[i], beta * x2[i]) : alpha * x1[i];
}
// y = x over n words, by the SMs: a state copy on the adjoint's critical
// path (the tape input of a step) finishes sooner than on a copy engine
__global__ void ka_copy(double *__restrict__ y, const double *__restrict__ x,
                        long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = x[i];
}
// a whole state copied by the SMs (ka_copy): the schedule's stores,
// restores and tape inputs sit on the two streams' dependency chains, where
// a copy-engine transfer of the same bytes takes about twice as long
int sm_copy(swg_state dst, swg_state src, const swg_model_s *md,
            cudaStream_t st) {
  const long long n = (long long)words(md);
  ka_copy<<<unsigned(std::min<long long>((n + 255) / 256, 1024)), 256, 0,
            st>>>(static_cast<double *>(dst->block),
                  static_cast<const double *>(src->block), n);
  ++g_launches;
  const cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? SWG_OK
                            : cuda_fail(err, "swg_adjoint: state copy");
}
__global__ void ka_sum_levels(const double *x, double *out, int n, int K) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  double s = 0;
  for (int k = 0; k < K; ++k)
    s += x[size_t(i) * K + k];
  out[i] = s;
}
__global__ void ka_pack(Dual *y, const double *v, const double *d,
                        long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n)
    y[i] = Dual{v[i], d ? d[i] : 0.0};
}
__global__ void ka_unpack(double *v, double *d, const Dual *x, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) {
    if (v)
      v[i] = x[i].v;
    if (d)
      d[i] = x[i].d;
  }
}

unsigned nb(long long n) { return unsigned((n + ATPB - 1) / ATPB); }

} // namespace
} // namespace swg

using namespace swg;

namespace {

template <class T>
int up(std::vector<void *> &allocs, const std::vector<T> &h, const T **d) {
  void *p = nullptr;
  cudaError_t err = cudaMalloc(&p, std::max<size_t>(h.size(), 1) * sizeof(T));
  if (err != cudaSuccess)
    return cuda_fail(err, "swg_adjoint: cudaMalloc");
  allocs.push_back(p);
  if (!h.empty() && (err = cudaMemcpy(p, h.data(), h.size() * sizeof(T),
                                      cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_fail(err, "swg_adjoint: cudaMemcpy");
  *d = static_cast<const T *>(p);
  return SWG_OK;
}

template <class T> int zal(std::vector<void *> &allocs, size_t n, T **d) {
  void *p = nullptr;
  cudaError_t err = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
  if (err == cudaSuccess)
    err = cudaMemset(p, 0, std::max<size_t>(n, 1) * sizeof(T));
  if (err != cudaSuccess)
    return cuda_fail(err, "swg_adjoint: work allocation");
  allocs.push_back(p);
  *d = static_cast<T *>(p);
  return SWG_OK;
}

// The o-th slot j < n of list[base...] holding x (o = 0: the first), or -1.
int slot_of(const std::vector<int> &list, int base, int n, int x, int o = 0) {
  for (int j = 0; j < n; ++j)
    if (list[base + j] == x && o-- == 0)
      return j;
  return -1;
}

// How many of the slots before j hold the same entry as slot j.
int occurrence(const std::vector<int> &list, int base, int j) {
  int o = 0;
  for (int i = 0; i < j; ++i)
    o += list[base + i] == list[base + j];
  return o;
}

// The o-th side s of edge e with pair[2e+s] == x, or -1.
int side_of(const std::vector<int> &pair, int e, int x, int o) {
  for (int s = 0; s < 2; ++s)
    if (pair[2 * e + s] == x && o-- == 0)
      return s;
  return -1;
}

int build_tables(swg_adjoint ad) {
  swg_model md = ad->model;
  swg_mesh me = md->mesh;
  const swg_params &P = md->params;
  const int C = me->ncells, E = me->nedges, V = me->nvertices;
  std::vector<double> ccdh_nb(6 * C, 0), ckq_nb(6 * C, 0), kd2_nb(6 * C, 0),
      r4_nb(6 * C, 0), keadj(6 * C, 0), d4adj(6 * C, 0),
      divadj(6 * C, 0), ckvh(6 * C, 0);
  std::vector<int> cvtx(6 * C, 0);
  std::vector<double> zetaadj4(3 * V);
  std::vector<double> ccd_e2(2 * E), ccdh_e2(2 * E), cke_e2(2 * E),
      ckq_e2(2 * E), kd2_e2(2 * E), cvr_e2(2 * E), z4adj(3 * V), zetaadj(3 * V),
      ccdh2_e2(2 * E), cke2_e2(2 * E), hm_c(6 * C, 0);
  auto kd2 = [&](int c, int j) {
    return P.eddy_diff2 * me->scale2_h[me->ec_h[6 * c + j]] * me->ckq_h[6 * c + j];
  };
  auto r4 = [&](int c, int j) {
    return -(P.eddy_diff4 * me->scale4_h[me->ec_h[6 * c + j]] * me->ckq_h[6 * c + j]);
  };
  for (int c = 0; c < C; ++c)
    for (int j = 0; j < MAXE; ++j) {
      if (me->ccd_h[6 * c + j] != 0.0)
        hm_c[6 * c + j] = 0.5;
      if (me->ccd_h[6 * c + j] == 0.0 && me->ckq_h[6 * c + j] == 0.0)
        continue; // padding slot
      // On a mesh one cell wide an edge can have the same cell on both
      // sides; it then fills two slots of that cell, and the o-th of them
      // stands for the o-th side, so each (edge, side) pair is transposed
      // once.  Padding slots (zero coefficients) repeat the first edge and
      // are not counted; real slots come first.
      const int e = me->ec_h[6 * c + j], n = me->nbc_h[6 * c + j];
      const int nreal = me->nec_h[c];
      const int o = occurrence(me->ec_h, 6 * c, j);
      const int side = side_of(me->ce_h, e, c, o);
      const int jn = slot_of(me->ec_h, 6 * n, me->nec_h[n], e, n == c ? o : 0);
      if (j >= nreal || jn < 0 || side < 0)
        return fail(SWG_ERR_ARG, "swg_adjoint: edge missing from its neighbour");
      ccdh_nb[6 * c + j] = me->ccdh_h[6 * n + jn];
      ckq_nb[6 * c + j] = me->ckq_h[6 * n + jn];
      kd2_nb[6 * c + j] = kd2(n, jn);
      r4_nb[6 * c + j] = r4(n, jn);
      const double sg = side == 0 ? 1.0 : -1.0;
      keadj[6 * c + j] = sg * me->inv_dc_h[e];
      d4adj[6 * c + j] = -(sg * (-(P.visc_del4 * me->scale4_h[e])) * me->inv_dc_h[e]);
      divadj[6 * c + j] = -(sg * me->inv_dc_h[e]);
    }
  // cells' vertices and kite weights (inverse of cells_on_vertex)
  std::vector<int> cnt(C, 0);
  for (int v = 0; v < V; ++v)
    for (int j = 0; j < 3; ++j) {
      const int c = me->cv_h[3 * v + j];
      if (me->kvh_h[3 * v + j] == 0.0)
        continue;
      if (cnt[c] >= MAXE)
        return fail(SWG_ERR_ARG, "swg_adjoint: a cell is on more than 6 vertices");
      cvtx[6 * c + cnt[c]] = v;
      ckvh[6 * c + cnt[c]] = me->kvh_h[3 * v + j];
      ++cnt[c];
    }
  for (int e = 0; e < E; ++e)
    for (int s = 0; s < 2; ++s) {
      const int c = me->ce_h[2 * e + s];
      const int j = slot_of(me->ec_h, 6 * c, me->nec_h[c], e,
                            s == 1 && me->ce_h[2 * e] == c);
      const int v = me->ve_h[2 * e + s];
      const int jv = slot_of(me->ev_h, 3 * v, 3, e,
                             s == 1 && me->ve_h[2 * e] == v);
      if (j < 0 || jv < 0)
        return fail(SWG_ERR_ARG, "swg_adjoint: inconsistent edge tables");
      ccd_e2[2 * e + s] = me->ccd_h[6 * c + j];
      ccdh_e2[2 * e + s] = me->ccdh_h[6 * c + j];
      cke_e2[2 * e + s] = me->cke_h[6 * c + j];
      cke2_e2[2 * e + s] = 2.0 * me->cke_h[6 * c + j];
      ccdh2_e2[2 * e + s] = 2.0 * me->ccdh_h[6 * c + j];
      ckq_e2[2 * e + s] = me->ckq_h[6 * c + j];
      kd2_e2[2 * e + s] = kd2(c, j);
      cvr_e2[2 * e + s] = me->cvr_h[3 * v + jv];
    }
  for (int v = 0; v < V; ++v)
    for (int j = 0; j < 3; ++j) {
      const int e = me->ev_h[3 * v + j];
      const int side = side_of(me->ve_h, e, v, occurrence(me->ev_h, 3 * v, j));
      if (side < 0)
        return fail(SWG_ERR_ARG, "swg_adjoint: inconsistent vertex tables");
      const double sg = side == 0 ? -1.0 : 1.0;
      z4adj[3 * v + j] = -(sg * (-(P.visc_del4 * me->scale4_h[e])) * me->inv_dv_h[e]);
      zetaadj[3 * v + j] = -(sg * me->inv_dv_h[e]);
      zetaadj4[3 * v + j] = -(sg * me->inv_dv4_h[e]);
    }
  // transposed edges-on-edge
  const int NE = me->view.ne;
  std::vector<int> tc(E, 0);
  for (int e = 0; e < E; ++e)
    for (int j = 0; j < NE; ++j)
      if (me->woe_h[NE * e + j] != 0.0)
        ++tc[me->eoe_h[NE * e + j]];
  int nt = 1;
  for (int e = 0; e < E; ++e)
    nt = std::max(nt, tc[e]);
  std::vector<int> eoeT(size_t(nt) * E);
  std::vector<double> woeT(size_t(nt) * E, 0.0);
  std::fill(tc.begin(), tc.end(), 0);
  for (int e = 0; e < E; ++e)
    for (int t = 0; t < nt; ++t)
      eoeT[size_t(nt) * e + t] = e;
  for (int e = 0; e < E; ++e)
    for (int j = 0; j < NE; ++j) {
      const double w = me->woe_h[NE * e + j];
      if (w == 0.0)
        continue;
      const int t = me->eoe_h[NE * e + j];
      eoeT[size_t(nt) * t + tc[t]] = e;
      woeT[size_t(nt) * t + tc[t]] = w;
      ++tc[t];
    }
  AdjView &a = ad->av;
  auto &A = ad->allocs;
  int rc;
  if ((rc = up(A, ccdh_nb, &a.ccdh_nb)) || (rc = up(A, ckq_nb, &a.ckq_nb)) ||
      (rc = up(A, kd2_nb, &a.kd2_nb)) || (rc = up(A, r4_nb, &a.r4_nb)) ||
      (rc = up(A, keadj, &a.keadj)) || (rc = up(A, d4adj, &a.d4adj)) ||
      (rc = up(A, divadj, &a.divadj)) ||
      (rc = up(A, cvtx, &a.cvtx)) || (rc = up(A, ckvh, &a.ckvh)) ||
      (rc = up(A, ccd_e2, &a.ccd_e2)) || (rc = up(A, ccdh_e2, &a.ccdh_e2)) ||
      (rc = up(A, cke_e2, &a.cke_e2)) || (rc = up(A, ckq_e2, &a.ckq_e2)) ||
      (rc = up(A, kd2_e2, &a.kd2_e2)) || (rc = up(A, cvr_e2, &a.cvr_e2)) ||
      (rc = up(A, eoeT, &a.eoeT)) || (rc = up(A, woeT, &a.woeT)) ||
      (rc = up(A, z4adj, &a.z4adj)) || (rc = up(A, zetaadj, &a.zetaadj)) ||
      (rc = up(A, hm_c, &a.hm_c)) || (rc = up(A, ccdh2_e2, &a.ccdh2_e2)) ||
      (rc = up(A, cke2_e2, &a.cke2_e2)) ||
      (me->view.dv4_differs && (rc = up(A, zetaadj4, &a.zetaadj4))))
    return rc;
  a.nt = nt;
  return SWG_OK;
}

// aux arrays of the same set as the model's, of value type T
template <class T> int alloc_aux_like(swg_adjoint ad, AuxViewT<T> &d) {
  swg_model md = ad->model;
  const AuxView &a = md->aux;
  const size_t C = md->mesh->ncells, E = md->mesh->nedges,
               V = md->mesh->nvertices, K = md->mesh->nlayers,
               T_ = md->params.ntracers;
  auto &A = ad->allocs;
  struct {
    const double *on;
    size_t n;
    T **p;
  } t[] = {{a.q, V * K, &d.q},       {a.zeta, V * K, &d.zeta},
           {a.z4, V * K, &d.z4},     {a.div, C * K, &d.div},
           {a.ke, C * K, &d.ke},     {a.d4, C * K, &d.d4},
           {a.ntr, T_ * C * K, &d.ntr}, {a.lap, T_ * C * K, &d.lap},
           {a.F, E * K, &d.F},       {a.G, E * K, &d.G},
           {a.Q, E * K, &d.Q},       {a.mh, E * K, &d.mh},
           {a.u2, E * K, &d.u2},     {a.d2u, E * K, &d.d2u}};
  for (auto &x : t)
    if (x.on)
      TRY(zal(A, x.n, x.p));
  d.d2u4 = d.d2u;
  if (a.d2u4 && a.d2u4 != a.d2u) // 1/max(dv, dc/4) differs from 1/dv
    TRY(zal(A, E * K, &d.d2u4));
  return SWG_OK;
}

// stage s of tape slot b: the model's intermediates plus what the adjoint
// passes would otherwise recompute (1/h_vertex, 1/h, mean thickness, and for
// the stages whose final passes run in the taped step, the PV sum S1)
int alloc_tape(swg_adjoint ad, int b, int s) {
  swg_model md = ad->model;
  const size_t C = md->mesh->ncells, E = md->mesh->nedges,
               V = md->mesh->nvertices, K = md->mesh->nlayers;
  AuxView &t = ad->tp[b].taux[s];
  auto &A = ad->allocs;
  TRY(alloc_aux_like(ad, t));
  if (md->view.do_vn) {
    TRY(zal(A, V * K, &t.rhv));
    // the last stage's PV sum is written only when the step's final
    // passes run (a taped advance); the adjoint of a tape from a state
    // recomputes it (adjoint_step's last_s1)
    TRY(zal(A, E * K, &t.S1));
  }
  if (md->params.ntracers > 0)
    TRY(zal(A, C * K, &t.rh));
  if (!t.mh)
    TRY(zal(A, E * K, &t.mh));
  return SWG_OK;
}

// lambda = J(X)^T mu with the intermediates of X already in `aux`
void adj_passes(swg_adjoint ad, const AuxView &aux, const AdjIO &io,
                cudaStream_t st) {
  swg_model md = ad->model;
  const MeshView &m = md->mesh->view;
  const ModelView &p = md->view;
  const long long K = m.nlayers, CK = m.ncells * K, EK = m.nedges * K,
                  VK = m.nvertices * K;
  const AdjView &v = ad->av;
  const AdjWork &w = ad->aw;
  const Fork *fk = &md->fork;
  const bool trd = p.ntracers > 0 && (p.tr_del2 | p.tr_del4);
  auto vel = [&](cudaStream_t q) {
    const long long base = p.vel_del4 ? 0 : VK; // vertex part: del4 only
    ka_vel<<<nb(VK + CK + EK - base), ATPB, 0, q>>>(m, p, aux, v, w, io,
                                                    unsigned(base));
    ++g_launches;
  };
  auto tr1 = [&](cudaStream_t q) {
    if (p.tr_del2 && p.tr_del4)
      ka_tr1<true, true><<<nb(CK), ATPB, 0, q>>>(m, p, aux, v, w, io);
    else if (p.tr_del2)
      ka_tr1<true, false><<<nb(CK), ATPB, 0, q>>>(m, p, aux, v, w, io);
    else if (p.tr_del4)
      ka_tr1<false, true><<<nb(CK), ATPB, 0, q>>>(m, p, aux, v, w, io);
    else
      ka_tr1<false, false><<<nb(CK), ATPB, 0, q>>>(m, p, aux, v, w, io);
    ++g_launches;
  };
  auto tr2 = [&](cudaStream_t q) {
    if (p.tr_del4)
      ka_tr2<true><<<nb(CK), ATPB, 0, q>>>(m, p, aux, v, w, io);
    else
      ka_tr2<false><<<nb(CK), ATPB, 0, q>>>(m, p, aux, v, w, io);
    ++g_launches;
  };
  auto edge = [&](cudaStream_t q) {
    if (m.ne == 8 && !trd)
      ka_edge<8, false><<<nb(EK), ATPB, 0, q>>>(m, p, aux, v, w, io);
    else if (m.ne == 8)
      ka_edge<8, true><<<nb(EK), ATPB, 0, q>>>(m, p, aux, v, w, io);
    else if (!trd)
      ka_edge<10, false><<<nb(EK), ATPB, 0, q>>>(m, p, aux, v, w, io);
    else
      ka_edge<10, true><<<nb(EK), ATPB, 0, q>>>(m, p, aux, v, w, io);
    ++g_launches;
  };
  // ka_vel and ka_tr1 are independent, and so are ka_edge and ka_tr2 (the
  // tracer pass writes only the tracer adjoint and the h part of tr / h)
  if (p.do_vn && p.ntracers > 0) {
    fork_join(fk, st, vel, tr1);
    fork_join(fk, st, edge, tr2);
  } else {
    if (p.do_vn)
      vel(st);
    if (p.ntracers > 0) {
      tr1(st);
      tr2(st);
    }
    edge(st);
  }
  if (p.do_vn) { // vertices, then (velocity dissipation) the cells' ldiv
    const bool vdiss = p.vel_del2 | p.vel_del4;
    ka_vertex<<<nb(VK + (vdiss ? CK : 0)), ATPB, 0, st>>>(m, p, aux, v, w,
                                                          io);
    ++g_launches;
  }
  // the two output passes read disjoint work arrays and write disjoint
  // outputs (h: lh and its stage bookkeeping; vn: the same for vn)
  fork_join(
      fk, st,
      [&](cudaStream_t q) {
        ka_vn<<<nb(EK), ATPB, 0, q>>>(m, p, aux, v, w, io);
      },
      [&](cudaStream_t q) {
        ka_cell<<<nb(CK), ATPB, 0, q>>>(m, p, aux, v, w, io);
      });
  g_launches += 2;
}

void adj_tendency(swg_adjoint ad, const double *h, const double *vn,
                  const double *tr, swg_state mu, swg_state out,
                  cudaStream_t st) {
  swg_model md = ad->model;
  launch_aux(md->mesh->view, md->view, md->aux, h, vn, tr, st, &md->fork);
  AdjIO io{};
  io.h = h;
  io.vn = vn;
  io.tr = tr;
  io.mh_ = mu->h;
  io.mvn = mu->vn;
  io.mtr = mu->tr;
  io.lh = out->h;
  io.lvn = out->vn;
  io.ltr = out->tr;
  adj_passes(ad, md->aux, io, st);
}

void lincomb(swg_state y, swg_state x1, swg_state x2, double a, double b,
             long long n, cudaStream_t st) {
  ka_lincomb<<<nb(n), ATPB, 0, st>>>(y->h, x1->h, x2 ? x2->h : nullptr, a, b, n);
  ++g_launches;
}

// Taped low-storage RK step (lsrk.cpp:36-89) from tp.X[0]: stage s forms
// T = a_s T + F(X_s) in tp.acc and X_{s+1} = X_s + dt b_s T in a separate
// buffer (a copy of X_s updated by the same epilogue as the in-place
// stepper, so the values are the stepper's bit for bit).  The last stage
// only records its intermediates unless `out` takes the step's result.
//
// Taped RK4 step from tp.X[0] (the caller copies the step's start state
// there): X1..X3 the stage inputs, and (when `out` is given) the step's
// result.
int tape_step(swg_adjoint ad, TapeSlot &tp, double dt, swg_state out,
              cudaStream_t st) {
  swg_model md = ad->model;
  const ModelView &pv = md->view;
  const int ns = ad->ns;
  TRY(tape_prologue(ad, tp, out, st));
  for (int s = 0; s < ns; ++s) {
    if (s == ns - 1 && !out) { // intermediates of the last stage input
      const double *h, *vn, *tr;
      stage_ptrs(ad, tp, s, &h, &vn, &tr);
      launch_aux(md->mesh->view, pv, tp.taux[s], h, vn, tr, st, &md->fork);
      continue;
    }
    TRY(tape_stage_copy(ad, tp, s, out, st));
    launch_tendency(md->mesh->view, pv, tp.taux[s],
                    tape_stage_args(ad, tp, s, dt, out), st, &md->fork);
  }
  cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? SWG_OK : cuda_fail(err, "swg_adjoint: taped step");
}

// lam <- adjoint of the step taped in tp, applied to lam.  The output passes
// of stage s accumulate lamX_s and form mu_{s-1} directly (ping-pong mu
// buffers: the passes of stage s still read mu_s).  The first reversed
// stage adds to lam and writes lacc, the last adds to lacc and writes lam,
// so no copy between them is needed.  With an even stage count (RK4) the
// last stage also forms the next step's first mu, dt b_{ns-1} lam, in the
// buffer that step reads first (bwd_begin forms the first one); with an
// odd count a separate pass forms it at the start of every step.
//
// Low-storage RK (ns stages): with lamX_s the adjoint of the stage input X_s
// and mu_s that of T_s, mu_{ns-1} = dt b_{ns-1} lam,
// lamX_s = lamX_{s+1} + J(X_s)^T mu_s and
// mu_{s-1} = dt b_{s-1} lamX_s + a_s mu_s; the step's adjoint is lamX_0.
// The output passes accumulate lamX in lacc and form mu_{s-1} from it.
// last_s1: the tape was written by a taped advance, whose last stage ran
// its final passes and taped that stage's PV sum too
int adjoint_step(swg_adjoint ad, const TapeSlot &tp, double dt, bool last_s1,
                 cudaStream_t st) {
  const int ns = ad->ns;
  if (ns % 2 != 0)
    lincomb(ad->mu, ad->lam, nullptr, dt * step_rkb(ad)[ns - 1], 0.0,
            (long long)words(ad->model), st);
  for (int s = ns - 1; s >= 0; --s) {
    AuxView aux = tp.taux[s];
    if (s == ns - 1 && !last_s1)
      aux.S1 = nullptr;
    adj_passes(ad, aux, stage_io(ad, tp, s, dt), st);
  }
  cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? SWG_OK : cuda_fail(err, "swg_adjoint: adjoint step");
}

// ---- checkpoint schedule
// The planner's dynamic programs cost O(nsteps^2 * snapshots) host work
// (seconds at the step limit); a schedule that re-runs more than
// kMaxReadvance plain steps per step is refused as a too small budget.
constexpr int kMaxAdjointSteps = 10000;
constexpr long long kMaxReadvance = 32;

// The classic optimal binomial schedule (Griewank-Walther) with one tape:
// plain advances cost(n, s) = min_m [m + cost(n - m, s - 1) + cost(m, s)],
// cost(n, 0) = n (n - 1) / 2.  Reported by swg_checkpoint_cost as the
// count the planner below improves on.
long long classic_binomial_cost(int N, int S) {
  std::vector<long long> c(size_t(N + 1) * (S + 1), 0);
  auto C = [&](int n, int s) -> long long & { return c[size_t(n) * (S + 1) + s]; };
  for (int n = 1; n <= N; ++n) {
    C(n, 0) = (long long)n * (n - 1) / 2;
    for (int s = 1; s <= S; ++s) {
      if (n == 1)
        continue;
      long long best = -1;
      for (int m = 1; m < n; ++m) {
        const long long x = m + C(n - m, s - 1) + C(m, s);
        if (best < 0 || x < best)
          best = x;
      }
      C(n, s) = best;
    }
  }
  return C(N, S);
}

// Checkpoint schedule with two tapes.  Reversing a step needs its tape
// (stage inputs and intermediates).  The classic schedule restores a
// checkpoint, re-advances to x_i and tapes step i from it; but the last
// step of that re-advance is step i - 1, the very next step to reverse.
// Here it can run as a taped advance into the second tape, at about the
// cost of a plain step, so the next reversal needs no restore, no
// re-advance and no tape.  A dynamic program picks, for every range of
// steps and snapshot budget, between that pair (advance to x_{i-1}, taped
// advance of step i-1, tape of step i, both adjoints) and the binomial
// split (advance m steps, store a checkpoint, reverse the right part with
// one snapshot fewer, then the left part).  Costs are in hundredths of a
// plain step: a taped advance 104 (the plain step plus the tape's extra
// writes), a tape from a state (all but the last stage, plus the last
// stage's intermediates, about 40 per cent of a stage) (100 (ns - 1) + 40)
// / ns.  The adjoints cost the same under every schedule and are left out.
//
//   f(n, s): reverse steps [i0, i0 + n) with x_{i0} available (in `cur` or
//            a snapshot) and s free snapshots;
//   h(n, s): the same, starting the forward sweep: it also produces
//            x_{i0+n}, whose last step is taped on the way (taped advances).
struct Planner {
  int N, S;
  long long cADV = 100, cTADV = 104, cTAPE = 85;
  std::vector<long long> f, h;
  std::vector<int> fm, hm; // 0: the taped pair; m > 0: split after m steps
  // one row of n per snapshot count: the split search walks f(m, s) and
  // f(n - m, s - 1) through contiguous memory
  size_t at(int n, int s) const { return size_t(s) * (N + 1) + n; }
  Planner(int n, int s, int ns)
      : N(n), S(std::max(0, std::min(s, n - 1))) {
    cTAPE = (100LL * (ns - 1) + 40) / ns;
    const size_t sz = size_t(N + 1) * (S + 1);
    f.assign(sz, 0);
    h.assign(sz, 0);
    fm.assign(sz, 0);
    hm.assign(sz, 0);
    for (int nn = 1; nn <= N; ++nn)
      for (int ss = 0; ss <= S; ++ss) {
        if (nn == 1) {
          f[at(1, ss)] = cTAPE;
          h[at(1, ss)] = cTADV;
          continue;
        }
        const long long rest = f[at(nn - 2, ss)] + (nn - 2) * cADV + cTADV;
        long long bf = rest + cTAPE, bh = rest + cTADV;
        int mf = 0, mh = 0;
        if (ss > 0)
          for (int m = 1; m < nn; ++m) {
            const long long base = m * cADV + f[at(m, ss)];
            const long long cf = base + f[at(nn - m, ss - 1)];
            const long long ch = base + h[at(nn - m, ss - 1)];
            if (cf < bf) {
              bf = cf;
              mf = m;
            }
            if (ch < bh) {
              bh = ch;
              mh = m;
            }
          }
        f[at(nn, ss)] = bf;
        fm[at(nn, ss)] = mf;
        h[at(nn, ss)] = bh;
        hm[at(nn, ss)] = mh;
      }
  }
  // The two tapes alternate.  A taped advance runs on the advance stream
  // into the tape whose adjoint ran first in the previous pair (1 -
  // recent_), so it can overlap the adjoint still reading the other tape;
  // tapes from a state run on the adjoints' stream into the tape its last
  // adjoint read (recent_).  With fixed roles the taped advance of most
  // pairs (those with no plain advance before it) had to wait for the
  // previous pair's last adjoint, and ran alone.
  mutable int recent_ = 0;
  // reverse [i0, i0 + n): x_{i0} in `cur` (cur_ok) or in snapshot `slot`;
  // slots slot+1 ... slot+s are free
  void gen_f(std::vector<AdjAction> &out, int i0, int n, int s, int slot,
             bool cur_ok) const {
    while (n > 0) {
      if (!cur_ok)
        out.push_back({A_RESTORE, slot, 0});
      if (n == 1) {
        out.push_back({A_TAPE_ADJ, i0, recent_});
        return;
      }
      const int m = fm[at(n, s)];
      if (m == 0) {
        const int tadv = 1 - recent_, tape = recent_;
        if (n > 2)
          out.push_back({A_ADV, i0, n - 2});
        out.push_back({A_TADV, i0 + n - 2, tadv});
        out.push_back({A_TAPE_ADJ, i0 + n - 1, tape});
        out.push_back({A_ADJ, i0 + n - 2, tadv});
        recent_ = tadv;
        n -= 2;
      } else {
        out.push_back({A_ADV, i0, m});
        out.push_back({A_STORE, slot + 1, 0});
        gen_f(out, i0 + m, n - m, s - 1, slot + 1, true);
        n = m;
      }
      cur_ok = false;
    }
  }
  // the whole schedule from x_{i0} in `cur` and snapshot `slot`: the
  // forward sweep up to A_FWD_END (x_{i0+n} in `cur`, the last steps
  // taped), then the reversal
  void gen_h(std::vector<AdjAction> &out, int i0, int n, int s,
             int slot) const {
    if (n == 1) {
      out.push_back({A_TADV, i0, 0});
      out.push_back({A_FWD_END, 0, 0});
      out.push_back({A_ADJ, i0, 0});
      recent_ = 0;
      return;
    }
    const int m = hm[at(n, s)];
    if (m == 0) {
      if (n > 2)
        out.push_back({A_ADV, i0, n - 2});
      out.push_back({A_TADV, i0 + n - 2, 1});
      out.push_back({A_TADV, i0 + n - 1, 0});
      out.push_back({A_FWD_END, 0, 0});
      out.push_back({A_ADJ, i0 + n - 1, 0});
      out.push_back({A_ADJ, i0 + n - 2, 1});
      recent_ = 1;
      gen_f(out, i0, n - 2, s, slot, false);
      return;
    }
    out.push_back({A_ADV, i0, m});
    out.push_back({A_STORE, slot + 1, 0});
    gen_h(out, i0 + m, n - m, s - 1, slot + 1);
    gen_f(out, i0, m, s, slot, false);
  }
  // the schedule of nsteps steps (the planner's N), snapshot 0 holding x_0
  std::vector<AdjAction> schedule() const {
    std::vector<AdjAction> out;
    out.push_back({A_STORE, 0, 0});
    gen_h(out, 0, N, S, 0);
    return out;
  }
};

void count_actions(const std::vector<AdjAction> &acts, long long *plain,
                   long long *tadv) {
  *plain = *tadv = 0;
  for (const AdjAction &a : acts) {
    if (a.type == A_ADV)
      *plain += a.b;
    else if (a.type == A_TADV)
      ++*tadv;
  }
}

// Captures `record` once (per dt) into g on a private stream and replays
// it on st; when capture fails the launches run directly on st.
template <class Fn>
int replay(swg_adjoint ad, AdjGraph &g, cudaStream_t st, Fn record) {
  if (!g.exec || g.dt != ad->dt || g.version != ad->model->version) {
    if (g.exec) {
      cudaGraphExecDestroy(g.exec);
      g.exec = nullptr;
    }
    cudaStream_t cs;
    cudaError_t err = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (err != cudaSuccess)
      return cuda_fail(err, "swg_adjoint: capture stream");
    const long long before = g_launches.load();
    err = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int rc = SWG_OK;
    if (err == cudaSuccess)
      rc = record(cs);
    cudaGraph_t gr = nullptr;
    cudaError_t err2 = cudaStreamEndCapture(cs, &gr);
    g.launches = g_launches.load() - before;
    g_launches -= g.launches;
    cudaStreamDestroy(cs);
    if (err != cudaSuccess || err2 != cudaSuccess || rc != SWG_OK) {
      if (gr)
        cudaGraphDestroy(gr);
      (void)cudaGetLastError();
      return record(st); // direct launches
    }
    err = cudaGraphInstantiate(&g.exec, gr, 0);
    cudaGraphDestroy(gr);
    if (err != cudaSuccess) {
      g.exec = nullptr;
      return cuda_fail(err, "swg_adjoint: graph instantiate");
    }
    g.dt = ad->dt;
    g.version = ad->model->version;
  }
  cudaError_t err = cudaGraphLaunch(g.exec, st);
  if (err != cudaSuccess)
    return cuda_fail(err, "swg_adjoint: graph launch");
  g_launches += g.launches;
  return SWG_OK;
}

// One schedule action on stream st.  With `two` (backward sweep) the
// restores, stores and plain and taped advances go to ad->adv instead; the
// adjoints run on st after the advance stream's work queued so far (event
// `ready`), a tape from `cur` hands `cur` back through `freed`, and a taped
// advance into a tape waits until the adjoint that last read that tape is
// done (the tape's free_ev).
int run_action(swg_adjoint ad, const AdjAction &a, cudaStream_t st, bool two) {
  cudaStream_t q = two ? ad->adv : st;
  cudaError_t e = cudaSuccess;
  switch (a.type) {
  case A_ADV:
    ad->plain_steps += a.b;
    return swg_step(ad->stepper, ad->cur, ad->t0 + a.a * ad->dt, ad->dt, a.b,
                    1, q);
  case A_STORE:
    return sm_copy(ad->snaps[a.a], ad->cur, ad->model, q);
  case A_RESTORE:
    return sm_copy(ad->cur, ad->snaps[a.a], ad->model, q);
  case A_TADV: {
    TapeSlot &tp = ad->tp[a.b];
    if (two && (e = cudaStreamWaitEvent(q, tp.free_ev, 0)) != cudaSuccess)
      return cuda_fail(e, "swg_adjoint: stream handshake");
    ++ad->taped_steps;
    ++ad->taped_advances;
    return replay(ad, tp.tadv, q, [&](cudaStream_t cs) {
      TRY(sm_copy(tp.X[0], ad->cur, ad->model, cs));
      return tape_step(ad, tp, ad->dt, ad->cur, cs);
    });
  }
  case A_TAPE_ADJ:
  case A_ADJ:
    break;
  default:
    return SWG_OK;
  }
  TapeSlot &tp = ad->tp[a.b];
  if (two && ((e = cudaEventRecord(ad->ready, ad->adv)) != cudaSuccess ||
              (e = cudaStreamWaitEvent(st, ad->ready, 0)) != cudaSuccess))
    return cuda_fail(e, "swg_adjoint: stream handshake");
  int rc;
  if (a.type == A_TAPE_ADJ) {
    TRY(sm_copy(tp.X[0], ad->cur, ad->model, st));
    if (two && ((e = cudaEventRecord(ad->freed, st)) != cudaSuccess ||
                (e = cudaStreamWaitEvent(ad->adv, ad->freed, 0)) != cudaSuccess))
      return cuda_fail(e, "swg_adjoint: stream handshake");
    ++ad->taped_steps;
    // tape + adjoint of one step: the same launches every time (no
    // forcing), replayed from a graph captured on first use
    rc = replay(ad, tp.tape_adj, st, [&](cudaStream_t cs) {
      TRY(tape_step(ad, tp, ad->dt, nullptr, cs));
      return adjoint_step(ad, tp, ad->dt, false, cs);
    });
  } else {
    // a reversal without its own tape follows a taped advance into tp
    rc = replay(ad, tp.adj, st, [&](cudaStream_t cs) {
      return adjoint_step(ad, tp, ad->dt, true, cs);
    });
  }
  if (rc == SWG_OK && two && (e = cudaEventRecord(tp.free_ev, st)) != cudaSuccess)
    return cuda_fail(e, "swg_adjoint: stream handshake");
  return rc;
}

int check_model(swg_model md) {
  if (!md)
    return fail(SWG_ERR_ARG, "swg_adjoint: NULL model");
  if (md->forcing)
    return fail(SWG_ERR_ARG, "swg_adjoint: models with an additional_tendency "
                             "hook are not differentiated");
  if (md->view.linear || md->view.drag)
    return fail(SWG_ERR_ARG, "swg_adjoint: the linear model and the bottom "
                             "drag are not differentiated");
  return SWG_OK;
}

} // namespace

namespace swg {

AdjIO stage_io(const swg_adjoint_s *ad, const TapeSlot &tp, int s,
               double dt) {
  const bool lsrk = ad->kind != SWG_STEPPER_RK4;
  const int ns = ad->ns;
  const bool even = ns % 2 == 0;
  const double *rka = step_rka(ad), *rkb = step_rkb(ad);
  swg_state mus[2] = {ad->mu, ad->mu2};
  swg_state mu = mus[(ns - 1 - s) % 2], nmu = mus[(ns - s) % 2];
  AdjIO io{};
  stage_ptrs(ad, tp, s, &io.h, &io.vn, &io.tr);
  io.mh_ = mu->h;
  io.mvn = mu->vn;
  io.mtr = mu->tr;
  swg_state in = s == ns - 1 ? ad->lam : ad->lacc;
  swg_state out = s == 0 ? ad->lam : ad->lacc;
  io.acc_in_h = in->h;
  io.acc_in_vn = in->vn;
  io.acc_in_tr = in->tr;
  io.acc_h = out->h;
  io.acc_vn = out->vn;
  io.acc_tr = out->tr;
  if (s > 0 || even) {
    io.nmu_h = nmu->h;
    io.nmu_vn = nmu->vn;
    io.nmu_tr = nmu->tr;
  }
  if (s > 0) {
    io.lam_h = ad->lam->h;
    io.lam_vn = ad->lam->vn;
    io.lam_tr = ad->lam->tr;
    io.alpha = dt * rkb[s - 1];
    io.beta = lsrk ? 0.0 : dt * rka[s - 1];
    io.gamma = lsrk ? rka[s] : 0.0;
    io.mode = lsrk ? 1 : 0;
  } else if (even) { // the next step's first mu (its stage ns-1 reads mus[0])
    io.alpha = dt * rkb[ns - 1];
    io.mode = 2;
  }
  return io;
}

StageArgs tape_stage_args(const swg_adjoint_s *ad, const TapeSlot &tp, int s,
                          double dt, swg_state out) {
  const int ns = ad->ns;
  StageArgs a{};
  stage_ptrs(ad, tp, s, &a.h, &a.vn, &a.tr);
  swg_state o = s < ns - 1 ? tp.X[s + 1] : out;
  if (ad->kind != SWG_STEPPER_RK4) { // in place on the copy o of X_s
    a.fh = {tp.acc->h, nullptr, nullptr, o->h};
    a.fvn = {tp.acc->vn, nullptr, nullptr, o->vn};
    a.ftr = {tp.acc->tr, nullptr, nullptr, o->tr};
    a.ep = {EPI_LSRK, ad->rka[s], dt * ad->rkb[s], 0.0};
    return a;
  }
  const double *rka = step_rka(ad), *rkb = step_rkb(ad);
  swg_state S = tp.X[0];
  a.fh = {nullptr, S->h, tp.acc->h, o->h};
  a.fvn = {nullptr, S->vn, tp.acc->vn, o->vn};
  a.ftr = {nullptr, S->tr, tp.acc->tr, o->tr};
  const int mode = s == 0 ? EPI_RK4_FIRST : (s < 3 ? EPI_RK4_MID : EPI_RK4_LAST);
  a.ep = {mode, 0.0, dt * rkb[s], s < 3 ? dt * rka[s] : 0.0};
  return a;
}

int tape_prologue(const swg_adjoint_s *ad, const TapeSlot &tp, swg_state out,
                  cudaStream_t st) {
  if (!out || ad->kind != SWG_STEPPER_RK4)
    return SWG_OK;
  // a field whose tendency is disabled ends the step as it began; the
  // stage epilogues write only the enabled fields of `out`
  const swg_model_s *md = ad->model;
  const size_t CK = size_t(md->mesh->ncells) * md->mesh->nlayers,
               EK = size_t(md->mesh->nedges) * md->mesh->nlayers;
  cudaError_t e = cudaSuccess;
  if (!md->view.do_h)
    e = cudaMemcpyAsync(out->h, tp.X[0]->h, CK * sizeof(double),
                        cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && !md->view.do_vn)
    e = cudaMemcpyAsync(out->vn, tp.X[0]->vn, EK * sizeof(double),
                        cudaMemcpyDeviceToDevice, st);
  return e == cudaSuccess ? SWG_OK : cuda_fail(e, "swg_adjoint: taped step");
}

int tape_stage_copy(const swg_adjoint_s *ad, const TapeSlot &tp, int s,
                    swg_state out, cudaStream_t st) {
  if (ad->kind == SWG_STEPPER_RK4)
    return SWG_OK;
  swg_state o = s < ad->ns - 1 ? tp.X[s + 1] : out;
  return swg_state_copy(o, tp.X[s], st);
}

// The schedule of (steps, snapshots, stages), planned once per process and
// kept: the dynamic program is O(steps^2 snapshots) on the host (tens of ms
// at 1000 steps and 32 snapshots), which a forward sweep would otherwise
// spend before its first launch every time.
std::vector<AdjAction> plan_schedule(int nsteps, int nsnapshots, int nstages) {
  struct Entry {
    int n, s, ns;
    std::vector<AdjAction> acts;
  };
  static std::mutex mu;
  static std::vector<Entry> cache; // most recently used last
  {
    std::lock_guard<std::mutex> lock(mu);
    for (size_t i = 0; i < cache.size(); ++i)
      if (cache[i].n == nsteps && cache[i].s == nsnapshots &&
          cache[i].ns == nstages) {
        Entry e = std::move(cache[i]);
        cache.erase(cache.begin() + i);
        cache.push_back(std::move(e));
        return cache.back().acts;
      }
  }
  std::vector<AdjAction> acts =
      Planner(nsteps, nsnapshots - 1, nstages).schedule();
  std::lock_guard<std::mutex> lock(mu);
  for (const Entry &c : cache) // another thread planned it meanwhile
    if (c.n == nsteps && c.s == nsnapshots && c.ns == nstages)
      return acts;
  if (cache.size() >= 16)
    cache.erase(cache.begin());
  cache.push_back({nsteps, nsnapshots, nstages, acts});
  return acts;
}

void adj_lincomb(swg_state y, swg_state x, double a, long long n,
                 cudaStream_t st) {
  lincomb(y, x, nullptr, a, 0.0, n, st);
}

} // namespace swg

extern "C" int swg_adjoint_destroy(swg_adjoint ad);

extern "C" int swg_adjoint_create(swg_model md, int nsnapshots,
                                  swg_adjoint *out) try {
  return swg_adjoint_create_stepper(md, nsnapshots, SWG_STEPPER_RK4, 4, out);
} SWG_ABI_CATCH("swg_adjoint_create")

extern "C" int swg_adjoint_create_stepper(swg_model md, int nsnapshots,
                                          int kind, int nstages,
                                          swg_adjoint *out) try {
  if (!out || nsnapshots < 1)
    return fail(SWG_ERR_ARG, "swg_adjoint_create: bad argument");
  *out = nullptr;
  if (!(kind == SWG_STEPPER_RK4 ||
        (kind == SWG_STEPPER_LSRK && (nstages == 5 || nstages == 1))))
    return fail(SWG_ERR_ARG, "swg_adjoint_create: RK4, or LSRK with 5 or 1 "
                             "stages");
  TRY(check_model(md));
  swg_adjoint ad = new (std::nothrow) swg_adjoint_s();
  if (!ad)
    return fail(SWG_ERR_OOM, "swg_adjoint_create: host allocation");
  ad->model = md;
  ad->nsnap = nsnapshots;
  ad->kind = kind;
  ad->ns = kind == SWG_STEPPER_RK4 ? 4 : nstages;
  const int T = md->params.ntracers;
  const size_t C = md->mesh->ncells, E = md->mesh->nedges,
               V = md->mesh->nvertices, K = md->mesh->nlayers;
  int rc = build_tables(ad);
  auto &A = ad->allocs;
  AdjWork &w = ad->aw;
  if (rc == SWG_OK &&
      ((rc = zal(A, T * C * K, &w.lL)) || (rc = zal(A, T * C * K, &w.ln)) ||
       (rc = zal(A, C * K, &w.lke)) || (rc = zal(A, C * K, &w.ld4)) ||
       (rc = zal(A, C * K, &w.lhtr)) ||
       (rc = zal(A, C * K, &w.ldiv)) || (rc = zal(A, V * K, &w.lz4)) ||
       (rc = zal(A, V * K, &w.lzeta)) || (rc = zal(A, V * K, &w.lhv)) ||
       (rc = zal(A, E * K, &w.lQ)) || (rc = zal(A, E * K, &w.lmh)) ||
       (rc = zal(A, E * K, &w.lvnp)) || (rc = zal(A, E * K, &w.ld2u)) ||
       (rc = zal(A, E * K, &w.Qmu)) ||
       (md->view.vel_del2 && (rc = zal(A, E * K, &w.gc2e))) ||
       (md->view.vel_del4 && md->mesh->view.dv4_differs &&
        (rc = zal(A, E * K, &w.ld2u4)))))
    ;
  swg_state *st[] = {&ad->cur, &ad->lam, &ad->lacc, &ad->mu, &ad->mu2};
  for (auto *p : st)
    if (rc == SWG_OK)
      rc = swg_state_create(md->mesh, T, p);
  for (int b = 0; b < kTapes; ++b) { // stage inputs and accumulator of a tape
    for (int s = 0; s < ad->ns && rc == SWG_OK; ++s)
      rc = swg_state_create(md->mesh, T, &ad->tp[b].X[s]);
    if (rc == SWG_OK)
      rc = swg_state_create(md->mesh, T, &ad->tp[b].acc);
  }
  for (int s = 0; s < nsnapshots && rc == SWG_OK; ++s) {
    swg_state x = nullptr;
    rc = swg_state_create(md->mesh, T, &x);
    ad->snaps.push_back(x);
  }
  if (rc == SWG_OK)
    rc = swg_stepper_create(md, kind, ad->ns, &ad->stepper);
  if (rc == SWG_OK) { // the stepper's coefficients (lsrk.cpp:16-33)
    ad->rka = ad->stepper->rka;
    ad->rkb = ad->stepper->rkb;
  }
  if (rc == SWG_OK) {
    cudaError_t e = cudaStreamCreateWithFlags(&ad->adv, cudaStreamNonBlocking);
    for (cudaEvent_t *ev : {&ad->go, &ad->ready, &ad->freed,
                            &ad->tp[0].free_ev, &ad->tp[1].free_ev})
      if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    if (e != cudaSuccess)
      rc = cuda_fail(e, "swg_adjoint_create: advance stream");
  }
  const size_t n = words(md);
  if (rc == SWG_OK && ((rc = alloc_aux_like(ad, ad->daux)) ||
                       (rc = zal(A, n, &ad->dS)) ||
                       (rc = zal(A, n, &ad->dacc)) || (rc = zal(A, n, &ad->dP0)) ||
                       (rc = zal(A, n, &ad->dP1)) || (rc = zal(A, n, &ad->dT))))
    ;
  for (int b = 0; b < kTapes; ++b)
    for (int s = 0; s < ad->ns && rc == SWG_OK; ++s)
      rc = alloc_tape(ad, b, s);
  if (rc != SWG_OK) {
    swg_adjoint_destroy(ad);
    return rc;
  }
  *out = ad;
  return SWG_OK;
} SWG_ABI_CATCH("swg_adjoint_create_stepper")

extern "C" int swg_adjoint_destroy(swg_adjoint ad) try {
  if (!ad)
    return SWG_OK;
  swg_stepper_destroy(ad->stepper);
  for (TapeSlot &tp : ad->tp) {
    for (AdjGraph *g : {&tp.tape_adj, &tp.tadv, &tp.adj})
      if (g->exec)
        cudaGraphExecDestroy(g->exec);
    if (tp.free_ev)
      cudaEventDestroy(tp.free_ev);
    for (swg_state x : tp.X)
      swg_state_destroy(x);
    swg_state_destroy(tp.acc);
  }
  for (cudaEvent_t e : {ad->go, ad->ready, ad->freed})
    if (e)
      cudaEventDestroy(e);
  if (ad->adv)
    cudaStreamDestroy(ad->adv);
  swg_state st[] = {ad->cur, ad->lam, ad->lacc, ad->mu, ad->mu2};
  for (auto s : st)
    swg_state_destroy(s);
  for (auto s : ad->snaps)
    swg_state_destroy(s);
  for (void *p : ad->allocs)
    cudaFree(p);
  delete ad;
  return SWG_OK;
} SWG_ABI_CATCH("swg_adjoint_destroy")

// no adjoint or model appears twice (members run concurrently)
static bool distinct_members(int n, const swg_adjoint *adjs) {
  for (int a = 0; a < n; ++a)
    for (int b = a + 1; b < n; ++b)
      if (adjs[a] == adjs[b] || adjs[a]->model == adjs[b]->model)
        return false;
  return true;
}

static bool same_layout(swg_adjoint ad, swg_state s) {
  return s && s->mesh == ad->model->mesh &&
         s->ntracers == ad->model->params.ntracers;
}

extern "C" int swg_adj_tendency(swg_adjoint ad, swg_state x, swg_state mu,
                                swg_state lambda_out, void *stream) try {
  if (!ad || !same_layout(ad, x) || !same_layout(ad, mu) ||
      !same_layout(ad, lambda_out))
    return fail(SWG_ERR_ARG, "swg_adj_tendency: bad argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  adj_tendency(ad, x->h, x->vn, x->tr, mu, lambda_out, st);
  cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? SWG_OK : cuda_fail(err, "swg_adj_tendency");
} SWG_ABI_CATCH("swg_adj_tendency")

extern "C" int swg_tlm_tendency(swg_adjoint ad, swg_state x, swg_state dx,
                                swg_state dtend_out, void *stream) try {
  if (!ad || !same_layout(ad, x) || !same_layout(ad, dx) ||
      !same_layout(ad, dtend_out))
    return fail(SWG_ERR_ARG, "swg_tlm_tendency: bad argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  swg_model md = ad->model;
  const long long n = (long long)words(md);
  ka_pack<<<nb(n), ATPB, 0, st>>>(ad->dS, x->h, dx->h, n);
  ++g_launches;
  const size_t CKn = size_t(md->mesh->ncells) * md->mesh->nlayers;
  const size_t EKn = size_t(md->mesh->nedges) * md->mesh->nlayers;
  StageArgsT<Dual> a{};
  a.h = ad->dS;
  a.vn = ad->dS + CKn;
  a.tr = ad->dS + CKn + EKn;
  a.fh.tend = ad->dT;
  a.fvn.tend = ad->dT + CKn;
  a.ftr.tend = ad->dT + CKn + EKn;
  a.ep.mode = EPI_REPLACE;
  // fields whose tendency is disabled stay untouched: start from zero
  cudaMemsetAsync(ad->dT, 0, n * sizeof(Dual), st);
  launch_tendency_dual(md->mesh->view, md->view, ad->daux, a, st);
  ka_unpack<<<nb(n), ATPB, 0, st>>>(nullptr, dtend_out->h, ad->dT, n);
  g_launches += 2;
  cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? SWG_OK : cuda_fail(err, "swg_tlm_tendency");
} SWG_ABI_CATCH("swg_tlm_tendency")

extern "C" int swg_tlm_apply(swg_adjoint ad, swg_state x0, swg_state dx,
                             double t0, double dt, int nsteps,
                             void *stream) try {
  (void)t0;
  if (!ad || !same_layout(ad, x0) || !same_layout(ad, dx) || nsteps < 0)
    return fail(SWG_ERR_ARG, "swg_tlm_apply: bad argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  swg_model md = ad->model;
  const ModelView &pv = md->view;
  const long long n = (long long)words(md);
  const size_t CKn = size_t(md->mesh->ncells) * md->mesh->nlayers;
  const size_t EKn = size_t(md->mesh->nedges) * md->mesh->nlayers;
  ka_pack<<<nb(n), ATPB, 0, st>>>(ad->dS, x0->h, dx->h, n);
  ++g_launches;
  static const double rka[3] = {1. / 2, 1. / 2, 1};
  static const double rkb[4] = {1. / 6, 1. / 3, 1. / 3, 1. / 6};
  Dual *S = ad->dS, *A = ad->dacc, *P[2] = {ad->dP0, ad->dP1};
  auto fio = [&](Dual *base, size_t off) { return base ? base + off : nullptr; };
  if (ad->kind != SWG_STEPPER_RK4) {
    // low-storage RK on dual numbers, in place like the stepper
    // (lsrk.cpp:36-89): tend = a_s tend + F, state += dt b_s tend
    cudaError_t e = cudaMemsetAsync(ad->dT, 0, sizeof(Dual) * n, st);
    if (e != cudaSuccess)
      return cuda_fail(e, "swg_tlm_apply: tendency reset");
    Dual *Tn = ad->dT;
    for (int step = 0; step < nsteps; ++step)
      for (int s = 0; s < ad->ns; ++s) {
        StageArgsT<Dual> a{};
        a.h = S;
        a.vn = S + CKn;
        a.tr = S + CKn + EKn;
        a.fh = {Tn, nullptr, nullptr, S};
        a.fvn = {Tn + CKn, nullptr, nullptr, S + CKn};
        a.ftr = {Tn + CKn + EKn, nullptr, nullptr, S + CKn + EKn};
        a.ep = {EPI_LSRK, ad->rka[s], dt * ad->rkb[s], 0.0};
        launch_tendency_dual(md->mesh->view, pv, ad->daux, a, st);
      }
    nsteps = 0;
  }
  for (int step = 0; step < nsteps; ++step) {
    Dual *in = S;
    for (int s = 0; s < 4; ++s) {
      Dual *o = s < 3 ? P[s % 2] : S;
      StageArgsT<Dual> a{};
      a.h = pv.do_h ? in : S;
      a.vn = (pv.do_vn ? in : S) + CKn;
      a.tr = in + CKn + EKn;
      a.fh = {nullptr, S, A, o};
      a.fvn = {nullptr, fio(S, CKn), fio(A, CKn), fio(o, CKn)};
      a.ftr = {nullptr, fio(S, CKn + EKn), fio(A, CKn + EKn), fio(o, CKn + EKn)};
      const int mode = s == 0 ? EPI_RK4_FIRST : (s < 3 ? EPI_RK4_MID : EPI_RK4_LAST);
      a.ep = {mode, 0.0, dt * rkb[s], s < 3 ? dt * rka[s] : 0.0};
      launch_tendency_dual(md->mesh->view, pv, ad->daux, a, st);
      in = o;
    }
  }
  ka_unpack<<<nb(n), ATPB, 0, st>>>(nullptr, dx->h, S, n);
  ++g_launches;
  cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? SWG_OK : cuda_fail(err, "swg_tlm_apply");
} SWG_ABI_CATCH("swg_tlm_apply")

namespace {

// Resumable sweeps: one schedule action per call, so several members'
// schedules can be interleaved on their own streams.
int fwd_begin(swg_adjoint ad, swg_state state0, double t0, double dt,
              int nsteps, cudaStream_t st) {
  if (nsteps > kMaxAdjointSteps)
    return fail(SWG_ERR_ARG, "swg_adj_forward: more steps than the schedule "
                             "planner takes (10000); split the trajectory");
  std::vector<AdjAction> acts = plan_schedule(nsteps, ad->nsnap, ad->ns);
  long long plain, tadv;
  count_actions(acts, &plain, &tadv);
  if (plain > kMaxReadvance * (long long)nsteps)
    return fail(SWG_ERR_BUDGET, "swg_adj_forward: too few snapshots: the "
                                "schedule would re-run more than 32 plain "
                                "steps per step; give the adjoint more "
                                "snapshots");
  ad->t0 = t0;
  ad->dt = dt;
  ad->nsteps = nsteps;
  ad->fwd_terms = term_set(ad->model);
  ad->plain_steps = ad->taped_steps = ad->taped_advances = 0;
  ad->actions.swap(acts);
  ad->pos = 0;
  ad->state = 0;
  return swg_state_copy(ad->cur, state0, st);
}

// the forward sweep runs the schedule up to its end marker: x_N is then in
// `cur` and the last steps are taped
int fwd_next(swg_adjoint ad, swg_state final_out, cudaStream_t st, bool *done) {
  const AdjAction &a = ad->actions[ad->pos++];
  if (a.type != A_FWD_END) {
    *done = false;
    return run_action(ad, a, st, false);
  }
  TRY(swg_state_copy(final_out, ad->cur, st));
  ad->state = 1;
  *done = true;
  return SWG_OK;
}

int bwd_begin(swg_adjoint ad, swg_state lambda, cudaStream_t st) {
  // the advance stream starts after everything already queued on st
  cudaError_t e = cudaEventRecord(ad->go, st);
  if (e == cudaSuccess)
    e = cudaStreamWaitEvent(ad->adv, ad->go, 0);
  if (e != cudaSuccess)
    return cuda_fail(e, "swg_adj_backward: stream handshake");
  TRY(swg_state_copy(ad->lam, lambda, st));
  if (ad->ns % 2 == 0) // the first step's first mu (later steps form theirs)
    lincomb(ad->mu, ad->lam, nullptr, ad->dt * step_rkb(ad)[ad->ns - 1], 0.0,
            (long long)words(ad->model), st);
  if (ad->aw.gc2e) {
    cudaError_t err = cudaMemsetAsync(
        ad->aw.gc2e, 0,
        sizeof(double) * ad->model->mesh->nedges * ad->model->mesh->nlayers, st);
    if (err != cudaSuccess)
      return cuda_fail(err, "swg_adj_backward: reset parameter gradient");
  }
  return SWG_OK;
}

int bwd_next(swg_adjoint ad, swg_state lambda, cudaStream_t st, bool *done) {
  if (ad->pos < ad->actions.size()) {
    *done = false;
    return run_action(ad, ad->actions[ad->pos++], st, true);
  }
  cudaError_t e = cudaEventRecord(ad->ready, ad->adv);
  if (e == cudaSuccess)
    e = cudaStreamWaitEvent(st, ad->ready, 0);
  if (e != cudaSuccess)
    return cuda_fail(e, "swg_adj_backward: stream handshake");
  TRY(swg_state_copy(lambda, ad->lam, st));
  ad->state = 0;
  ad->grad_ready = true;
  *done = true;
  return SWG_OK;
}

} // namespace

extern "C" int swg_adj_forward(swg_adjoint ad, swg_state state0, double t0,
                               double dt, int nsteps, swg_state final_out,
                               void *stream) try {
  if (!ad || !same_layout(ad, state0) || !same_layout(ad, final_out) ||
      nsteps < 1)
    return fail(SWG_ERR_ARG, "swg_adj_forward: bad argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  NvtxRange range("adjoint_forward_sweep");
  TRY(fwd_begin(ad, state0, t0, dt, nsteps, st));
  for (bool done = false; !done;)
    TRY(fwd_next(ad, final_out, st, &done));
  return SWG_OK;
} SWG_ABI_CATCH("swg_adj_forward")

extern "C" int swg_adj_backward(swg_adjoint ad, swg_state lambda,
                                void *stream) try {
  if (!ad || !same_layout(ad, lambda))
    return fail(SWG_ERR_ARG, "swg_adj_backward: bad argument");
  if (ad->state != 1)
    return fail(SWG_ERR_STATE, "swg_adj_backward: call swg_adj_forward first");
  if (term_set(ad->model) != ad->fwd_terms) // re-advances would differ
    return fail(SWG_ERR_STATE, "swg_adj_backward: a tendency term of the "
                               "model was switched after swg_adj_forward");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  NvtxRange range("adjoint_backward_sweep");
  TRY(bwd_begin(ad, lambda, st));
  for (bool done = false; !done;)
    TRY(bwd_next(ad, lambda, st, &done));
  return SWG_OK;
} SWG_ABI_CATCH("swg_adj_backward")

extern "C" int swg_adj_batch_forward(int n, const swg_adjoint *adjs,
                                     const swg_state *states0, double t0,
                                     double dt, int nsteps,
                                     const swg_state *finals,
                                     void *const *streams) try {
  if (n < 1 || !adjs || !states0 || !finals || nsteps < 1)
    return fail(SWG_ERR_ARG, "swg_adj_batch_forward: bad argument");
  for (int m = 0; m < n; ++m)
    if (!adjs[m] || !same_layout(adjs[m], states0[m]) ||
        !same_layout(adjs[m], finals[m]))
      return fail(SWG_ERR_ARG, "swg_adj_batch_forward: member mismatch");
  if (!distinct_members(n, adjs))
    return fail(SWG_ERR_ARG, "swg_adj_batch_forward: members must have "
                             "distinct adjoints and models (a shared model's "
                             "intermediates would be written concurrently)");
  auto S = [&](int m) {
    return streams ? static_cast<cudaStream_t>(streams[m]) : cudaStream_t(0);
  };
  for (int m = 0; m < n; ++m)
    TRY(fwd_begin(adjs[m], states0[m], t0, dt, nsteps, S(m)));
  std::vector<char> done(n, 0);
  for (int left = n; left > 0;)
    for (int m = 0; m < n; ++m) {
      if (done[m])
        continue;
      bool d = false;
      TRY(fwd_next(adjs[m], finals[m], S(m), &d));
      if (d) {
        done[m] = 1;
        --left;
      }
    }
  return SWG_OK;
} SWG_ABI_CATCH("swg_adj_batch_forward")

extern "C" int swg_adj_batch_backward(int n, const swg_adjoint *adjs,
                                      const swg_state *lambdas,
                                      void *const *streams) try {
  if (n < 1 || !adjs || !lambdas)
    return fail(SWG_ERR_ARG, "swg_adj_batch_backward: bad argument");
  for (int m = 0; m < n; ++m)
    if (!adjs[m] || !same_layout(adjs[m], lambdas[m]) || adjs[m]->state != 1)
      return fail(SWG_ERR_ARG, "swg_adj_batch_backward: member not ready");
    else if (term_set(adjs[m]->model) != adjs[m]->fwd_terms)
      return fail(SWG_ERR_STATE, "swg_adj_batch_backward: a tendency term of "
                                 "a member's model was switched after the "
                                 "forward sweep");
  if (!distinct_members(n, adjs))
    return fail(SWG_ERR_ARG, "swg_adj_batch_backward: members must have "
                             "distinct adjoints and models");
  auto S = [&](int m) {
    return streams ? static_cast<cudaStream_t>(streams[m]) : cudaStream_t(0);
  };
  for (int m = 0; m < n; ++m)
    TRY(bwd_begin(adjs[m], lambdas[m], S(m)));
  std::vector<char> done(n, 0);
  for (int left = n; left > 0;)
    for (int m = 0; m < n; ++m) {
      if (done[m])
        continue;
      bool d = false;
      TRY(bwd_next(adjs[m], lambdas[m], S(m), &d));
      if (d) {
        done[m] = 1;
        --left;
      }
    }
  return SWG_OK;
} SWG_ABI_CATCH("swg_adj_batch_backward")

extern "C" int swg_adj_info(swg_adjoint ad, long long *plain_steps,
                            long long *taped_steps) try {
  if (!ad)
    return fail(SWG_ERR_ARG, "swg_adj_info: NULL");
  if (plain_steps)
    *plain_steps = ad->plain_steps;
  if (taped_steps)
    *taped_steps = ad->taped_steps;
  return SWG_OK;
} SWG_ABI_CATCH("swg_adj_info")

extern "C" int swg_adj_info_ex(swg_adjoint ad, long long *plain_steps,
                               long long *taped_steps,
                               long long *taped_advances) try {
  if (!ad)
    return fail(SWG_ERR_ARG, "swg_adj_info_ex: NULL");
  TRY(swg_adj_info(ad, plain_steps, taped_steps));
  if (taped_advances)
    *taped_advances = ad->taped_advances;
  return SWG_OK;
} SWG_ABI_CATCH("swg_adj_info_ex")

// bytes of the arrays of an intermediate set (null members not counted)
size_t aux_bytes(const AuxView &a, size_t C, size_t E, size_t V, size_t K,
                 size_t T) {
  size_t w = 0;
  for (const double *p : {a.q, a.zeta, a.z4, a.rhv})
    w += p ? V * K : 0;
  for (const double *p : {a.div, a.ke, a.d4, a.rh})
    w += p ? C * K : 0;
  for (const double *p : {a.ntr, a.lap})
    w += p ? T * C * K : 0;
  for (const double *p : {a.F, a.G, a.Q, a.mh, a.u2, a.d2u, a.S1})
    w += p ? E * K : 0;
  if (a.d2u4 && a.d2u4 != a.d2u)
    w += E * K;
  return w * sizeof(double);
}

extern "C" int swg_adj_memory(swg_adjoint ad, long long *snapshot_bytes,
                              long long *tape_bytes,
                              long long *total_bytes) try {
  if (!ad)
    return fail(SWG_ERR_ARG, "swg_adj_memory: NULL");
  swg_model md = ad->model;
  const size_t C = md->mesh->ncells, E = md->mesh->nedges,
               V = md->mesh->nvertices, K = md->mesh->nlayers,
               T = md->params.ntracers;
  const size_t state = words(md) * sizeof(double);
  size_t tape = 0;
  for (int s = 0; s < ad->ns; ++s)
    tape += aux_bytes(ad->tp[0].taux[s], C, E, V, K, T);
  tape += size_t(ad->ns + 1) * state; // stage inputs and accumulator
  if (snapshot_bytes)
    *snapshot_bytes = (long long)state;
  if (tape_bytes)
    *tape_bytes = (long long)tape;
  if (total_bytes) // snapshots, both tapes, the sweep's own states (cur,
                   // lam, lacc, mu, mu2) and the adjoint work arrays
    *total_bytes = (long long)(size_t(ad->nsnap + 5) * state + kTapes * tape +
                               (2 * T * C + 4 * C + 3 * V + 5 * E) * K *
                                   sizeof(double) +
                               (ad->aw.gc2e ? E * K * sizeof(double) : 0));
  return SWG_OK;
} SWG_ABI_CATCH("swg_adj_memory")

extern "C" int swg_adj_grad_visc(swg_adjoint ad, double *grad_edge,
                                 double *grad_cell, void *stream) try {
  if (!ad)
    return fail(SWG_ERR_ARG, "swg_adj_grad_visc: NULL");
  if (!ad->aw.gc2e)
    return fail(SWG_ERR_STATE, "swg_adj_grad_visc: the model has no del2 "
                               "viscosity term");
  if (!ad->grad_ready)
    return fail(SWG_ERR_STATE, "swg_adj_grad_visc: no backward sweep has "
                               "completed");
  swg_mesh me = ad->model->mesh;
  const int E = me->nedges, C = me->ncells, K = me->nlayers;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // reuse the edge work array lQ as the per-edge sum
  ka_sum_levels<<<(E + 255) / 256, 256, 0, st>>>(ad->aw.gc2e, ad->aw.lQ, E, K);
  ++g_launches;
  std::vector<double> ge(E);
  cudaError_t err = cudaMemcpyAsync(ge.data(), ad->aw.lQ, E * sizeof(double),
                                    cudaMemcpyDeviceToHost, st);
  if (err == cudaSuccess)
    err = cudaStreamSynchronize(st);
  if (err != cudaSuccess)
    return cuda_fail(err, "swg_adj_grad_visc");
  // dL/d visc_edge = dL/dc2e (c2e = visc_del2 * scale2 = visc_edge); a
  // per-cell field maps to edges as visc_e = (visc_c0 + visc_c1) / 2
  if (grad_edge)
    std::memcpy(grad_edge, ge.data(), E * sizeof(double));
  if (grad_cell) {
    std::fill(grad_cell, grad_cell + C, 0.0);
    for (int e = 0; e < E; ++e) {
      grad_cell[me->ce_h[2 * e]] += 0.5 * ge[e];
      grad_cell[me->ce_h[2 * e + 1]] += 0.5 * ge[e];
    }
  }
  return SWG_OK;
} SWG_ABI_CATCH("swg_adj_grad_visc")

extern "C" long long swg_checkpoint_cost(int nsteps, int nsnapshots) try {
  if (nsteps < 1 || nsnapshots < 1 || nsteps > kMaxAdjointSteps)
    return -1;
  return classic_binomial_cost(nsteps, nsnapshots - 1);
} catch (...) {
  abi_exception("swg_checkpoint_cost");
  return -1;
}

extern "C" int swg_adj_plan(int nsteps, int nsnapshots, int nstages,
                            long long *plain_steps,
                            long long *taped_advances) try {
  if (nsteps < 1 || nsnapshots < 1 || nsteps > kMaxAdjointSteps ||
      !(nstages == 4 || nstages == 5 || nstages == 1))
    return fail(SWG_ERR_ARG, "swg_adj_plan: bad argument");
  long long p = 0, t = 0;
  count_actions(plan_schedule(nsteps, nsnapshots, nstages), &p, &t);
  if (plain_steps)
    *plain_steps = p;
  if (taped_advances)
    *taped_advances = t;
  return SWG_OK;
} SWG_ABI_CATCH("swg_adj_plan")

extern "C" int swg_adj_schedule(int nsteps, int nsnapshots, int nstages,
                                int max_actions, int *actions, int *count) try {
  if (nsteps < 1 || nsnapshots < 1 || nsteps > kMaxAdjointSteps ||
      !(nstages == 4 || nstages == 5 || nstages == 1) || !count ||
      max_actions < 0 || (max_actions > 0 && !actions))
    return fail(SWG_ERR_ARG, "swg_adj_schedule: bad argument");
  const std::vector<AdjAction> acts =
      plan_schedule(nsteps, nsnapshots, nstages);
  *count = int(acts.size());
  const int n = std::min<int>(max_actions, int(acts.size()));
  for (int i = 0; i < n; ++i) {
    actions[3 * i] = acts[i].type;
    actions[3 * i + 1] = acts[i].a;
    actions[3 * i + 2] = acts[i].b;
  }
  return SWG_OK;
} SWG_ABI_CATCH("swg_adj_schedule")
