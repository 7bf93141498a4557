// Device code and handle of the adjoint (reverse mode) of the shallow-water
// step, shared by the single-instance adjoint (swg_adjoint.cu) and the
// batched member ensemble (swg_ensemble.cu).
//
// Each pass of the adjoint of one tendency evaluation is a device function
// of one flat index i of its domain ((entity, level), level fastest), as
// the forward passes of swg_device.cuh are: the single-instance kernels
// call it with i = block * 256 + thread, the ensemble's kernels with i
// inside a member's virtual blocks, so a member's adjoint is computed by
// exactly the same arithmetic in both.
#pragma once

#include "swg_device.cuh"

#include <vector>

namespace swg {

constexpr int ATPB = 256;

struct AdjView {
  // cells [C][6]
  const double *ccdh_nb, *ckq_nb, *kd2_nb, *r4_nb; // neighbour's coefficient
  const double *keadj, *d4adj, *divadj;    // transposed edge terms
  const int *cvtx;                                 // vertices of the cell
  const double *ckvh;                              // their kite weight for c
  const double *hm_c;                              // 0.5 on edges, 0 on padding
  // edges [E][2]: coefficients of cells (c0, c1) / vertices (v0, v1) for e
  const double *ccd_e2, *ccdh_e2, *cke_e2, *ckq_e2, *kd2_e2, *cvr_e2;
  const double *ccdh2_e2, *cke2_e2;                // 2 ccdh_e2, 2 cke_e2
  // transposed edges-on-edge [E][nt] with weights / 4
  const int *eoeT;
  const double *woeT;
  int nt;
  // vertices [V][3]
  const double *z4adj, *zetaadj;
  const double *zetaadj4; // with 1/max(dv, dc/4) (meshes where it differs)
};

struct AdjWork {
  double *lL, *ln;                      // [T][C][K]
  double *lke, *ld4, *lhtr, *ldiv; // [C][K]
  double *lz4, *lzeta, *lhv;            // [V][K]
  double *lQ, *lmh, *lvnp, *ld2u;       // [E][K]
  double *Qmu;                          // [E][K] Q mu_vn of the stage
  // [E][K] adjoint of the del4 chain's first Laplacian, kept apart from the
  // del2 one (ld2u) where 1/max(dv, dc/4) differs from 1/dv; else null
  double *ld2u4;
  double *gc2e; // [E][K] accumulated dL/d(visc_del2 * mesh_scaling_del2), or null
};

struct AdjIO {
  const double *h, *vn, *tr;    // state X
  const double *mh_, *mvn, *mtr; // mu (adjoint of the tendency)
  double *lh, *lvn, *ltr;        // lambda = J^T mu (written unless null)
  // fused stage bookkeeping (each may be null): acc = acc_in + lambda, and
  // the next stage's mu (mode): 0 RK4  mu_next = alpha * lam + beta * lambda;
  //                             1 LSRK mu_next = alpha * acc + gamma * mu;
  //                             2 next step: mu_next = alpha * acc
  // (acc after the update).  acc_in is acc itself except where a step's
  // first stage reads lam and its last stage writes lam, which saves the
  // copies between the two.
  const double *acc_in_h, *acc_in_vn, *acc_in_tr;
  double *acc_h, *acc_vn, *acc_tr;
  double *nmu_h, *nmu_vn, *nmu_tr;
  const double *lam_h, *lam_vn, *lam_tr;
  double alpha, beta, gamma;
  int mode;
};

// The adds here and in the passes that take a product (x is often one) are
// written as __dadd_rn: the compiler may not fuse them into a multiply-add,
// which it could otherwise do differently in the single-instance and the
// batched kernels that inline the same pass, and the two must agree bit for
// bit.
__device__ __forceinline__ void emit(const AdjIO &io, double *out,
                                     const double *acc_in, double *acc,
                                     double *nmu, const double *lam,
                                     const double *mu, size_t i, double x) {
  if (out)
    out[i] = x;
  double a = 0;
  if (acc) {
    a = __dadd_rn(acc_in[i], x);
    acc[i] = a;
  }
  if (nmu) {
    // the mode picks operands, not operations: one multiply and one
    // multiply-add in every mode (a chain per mode was if-converted, and
    // each element issued all three with two of them predicated off)
    double u = a, c = 0.0, y = 0.0;
    if (io.mode == 0) {
      u = lam[i];
      c = io.beta;
      y = x;
    } else if (io.mode == 1) {
      c = io.gamma;
      y = mu[i];
    }
    nmu[i] = fma(io.alpha, u, c * y);
  }
}

// the del4 transpose's cell part: sum_j d4adj_j (mask mu)_j
static __device__ __noinline__ double d4_transpose(const MeshView &m,
                                                   const AdjView &v,
                                                   const AdjIO &io, int c,
                                                   int k) {
  const int K = m.nlayers;
  double d4 = 0;
  for (int j = 0; j < MAXE; ++j) {
    const size_t ie = size_t(__ldg(m.ec + 6 * c + j)) * K + k;
    const double mu = io.mvn[ie];
    d4 = fma(__ldg(v.d4adj + 6 * c + j), m.mask ? mu * m.mask[ie] : mu, d4);
  }
  return d4;
}

// --- pass 1: transposed edge stencils of the velocity tendency (cells and
// vertices), and Q mu_vn per edge for the transposed PV flux; the first V*K
// threads take vertices, the next C*K cells, the last E*K edges (launches
// start at V*K when the vertex part, velocity del4, is off).
__device__ __forceinline__ void
pa_vel(const MeshView &m, const ModelView &p, const AuxView &a,
         const AdjView &v, const AdjWork &w, const AdjIO &io, unsigned i) {
  const int K = m.nlayers;
  const unsigned VK = unsigned(m.nvertices) * K, CK = unsigned(m.ncells) * K;
  if (i >= VK + CK) {
    i -= VK + CK;
    if (i < unsigned(m.nedges) * K && !p.off_pv)
      w.Qmu[i] = a.Q[i] * io.mvn[i];
    return;
  }
  // the del4 term is masked per edge and level (mask * c4e): its
  // transposes gather mask * mu
  if (i < VK) {
    if (!p.vel_del4)
      return;
    const int vx = int(i / unsigned(K)), k = int(i - unsigned(vx) * K);
    double z = 0;
    for (int j = 0; j < 3; ++j) {
      const size_t ie = size_t(__ldg(m.ev + 3 * vx + j)) * K + k;
      const double mu = m.mask ? io.mvn[ie] * m.mask[ie] : io.mvn[ie];
      z = fma(__ldg(v.z4adj + 3 * vx + j), mu, z);
    }
    w.lz4[i] = z;
    return;
  }
  i -= VK;
  const int c = int(i / unsigned(K)), k = int(i - unsigned(c) * K);
  // the SSH gradient's transpose is g times the kinetic-energy gradient's
  // (both are -(x_1 - x_0)/dc per edge), applied where lke is read: lke
  // serves either term
  if (!p.off_ke || !p.off_ssh) {
    double ke = 0;
    for (int j = 0; j < MAXE; ++j)
      ke = fma(__ldg(v.keadj + 6 * c + j),
               io.mvn[size_t(__ldg(m.ec + 6 * c + j)) * K + k], ke);
    w.lke[i] = ke;
  }
  if (p.vel_del4) // a loop of its own: no predicated-off FMAs without del4
    w.ld4[i] = d4_transpose(m, v, io, c, k);
}

// What the passes recompute when the intermediates are not taped (the
// adjoint of a single tendency, and the PV sum of a tape's last stage) sits
// in out-of-line functions: inlined, the compiler if-converted these short
// branches, and the taped path then issued their FP64 instructions with
// the predicate off, occupying the FP64 pipe for nothing.

// the forward's Newton reciprocal of x
__device__ __forceinline__ double fwd_rcp(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}

static __device__ __noinline__ double mean_h_of(const MeshView &m, const double *h,
                                         int e, int k) {
  const int K = m.nlayers;
  return 0.5 * (h[size_t(__ldg(m.ce + 2 * e)) * K + k] +
                h[size_t(__ldg(m.ce + 2 * e + 1)) * K + k]);
}

// mean thickness of edge e (the forward's value: taped, or recomputed)
__device__ __forceinline__ double mean_h(const MeshView &m, const AuxView &a,
                                         const double *h, int e, int k) {
  if (a.mh)
    return a.mh[size_t(e) * m.nlayers + k];
  return mean_h_of(m, h, e, k);
}

// 1/h of cell-level i, as the forward's cell pass forms it
static __device__ __noinline__ double cell_rcp(const double *h, unsigned i) {
  return fwd_rcp(h[i]);
}

// 1/h_vertex of vertex vx, level k, as the forward's vertex pass forms it
static __device__ __noinline__ double vertex_rcp(const MeshView &m, const double *h,
                                          int vx, int k) {
  const int K = m.nlayers;
  double hv = __ldg(m.kvh + 3 * vx) * h[size_t(__ldg(m.cv + 3 * vx)) * K + k];
  for (int j = 1; j < 3; ++j)
    hv = fma(__ldg(m.kvh + 3 * vx + j),
             h[size_t(__ldg(m.cv + 3 * vx + j)) * K + k], hv);
  return fwd_rcp(hv);
}

// the PV flux sum S1 = sum_j w_j F_j of edge e, level k
template <int NE>
__device__ __noinline__ double s1_of(const MeshView &m, const AuxView &a,
                                     int e, int k) {
  const int K = m.nlayers;
  double S1 = 0;
  for (int j = 0; j < NE; ++j)
    S1 = fma(__ldg(m.woe + NE * e + j),
             a.F[size_t(__ldg(m.eoe + NE * e + j)) * K + k], S1);
  return S1;
}

// --- pass 2: tracer tendency transposed to the normalised tracers (partial)
// and to the tracer Laplacian.  D2, D4: tracer del2 / del4 on, as
// compile-time switches (with runtime flags the diffusion arrays stayed in
// registers and lowered the occupancy of the diffusion-free case).
template <bool D2, bool D4>
__device__ __forceinline__ void
pa_tr1(const MeshView &m, const ModelView &p, const AuxView &a,
         const AdjView &v, const AdjWork &w, const AdjIO &io, unsigned i) {
  const int K = m.nlayers;
  const unsigned CK = unsigned(m.ncells) * K;
  if (i >= CK)
    return;
  const int c = int(i / unsigned(K)), k = int(i - unsigned(c) * K);
  double wnb[MAXE], wc = 0;
  int nb[MAXE];
  const bool adv = !p.off_tr_hadv; // tracer advection switched on
  for (int j = 0; j < MAXE; ++j) {
    const int e = __ldg(m.ec + 6 * c + j);
    nb[j] = __ldg(m.nbc + 6 * c + j);
    double x = 0;
    if (adv) {
      const double F = a.F[size_t(e) * K + k];
      x = __ldg(v.ccdh_nb + 6 * c + j) * F;
      wc = fma(__ldg(m.ccdh + 6 * c + j), F, wc);
    }
    if (D2) {
      const double mh = mean_h(m, a, io.h, e, k);
      x = fma(__ldg(v.kd2_nb + 6 * c + j), mh, x);
      wc = fma(-__ldg(p.kd2 + 6 * c + j), mh, wc);
    }
    wnb[j] = x;
  }
  for (int l = 0; l < p.ntracers; ++l) {
    const double *mu = io.mtr + size_t(l) * CK;
    double acc = wc * mu[i];
    for (int j = 0; j < MAXE; ++j)
      acc = fma(wnb[j], mu[size_t(nb[j]) * K + k], acc);
    w.ln[size_t(l) * CK + i] = acc;
    if (D4) {
      double L = -__ldg(p.r4sum + c) * mu[i];
      for (int j = 0; j < MAXE; ++j)
        L = fma(__ldg(v.r4_nb + 6 * c + j), mu[size_t(nb[j]) * K + k], L);
      w.lL[size_t(l) * CK + i] = L;
    }
  }
}

// --- pass 3: through the tracer Laplacian and n = tr / h to the tracers;
// the h part of n = tr / h is kept for pass 6.  D4: tracer del4 on.
template <bool D4>
__device__ __forceinline__ void
pa_tr2(const MeshView &m, const ModelView &p, const AuxView &a,
         const AdjView &v, const AdjWork &w, const AdjIO &io, unsigned i) {
  const int K = m.nlayers;
  const unsigned CK = unsigned(m.ncells) * K;
  if (i >= CK)
    return;
  const int c = int(i / unsigned(K)), k = int(i - unsigned(c) * K);
  double mnb[MAXE], M = 0;
  int nb[MAXE];
  if (D4)
    for (int j = 0; j < MAXE; ++j) {
      const int e = __ldg(m.ec + 6 * c + j);
      const double mh = mean_h(m, a, io.h, e, k);
      nb[j] = __ldg(m.nbc + 6 * c + j);
      mnb[j] = __ldg(v.ckq_nb + 6 * c + j) * mh;
      M = fma(__ldg(m.ckq + 6 * c + j), mh, M);
    }
  // 1/h: the forward's own reciprocal (taped, or recomputed)
  const double r = a.rh ? a.rh[i] : cell_rcp(io.h, i);
  double hsum = 0;
  for (int l = 0; l < p.ntracers; ++l) {
    const size_t t = size_t(l) * CK + i;
    double ln = w.ln[t];
    if (D4) {
      const double *lL = w.lL + size_t(l) * CK;
      ln = fma(-M, lL[i], ln);
      for (int j = 0; j < MAXE; ++j)
        ln = fma(mnb[j], lL[size_t(nb[j]) * K + k], ln);
    }
    emit(io, io.ltr, io.acc_in_tr, io.acc_tr, io.nmu_tr, io.lam_tr, io.mtr, t,
         ln * r);
    hsum = fma(ln, a.ntr[t], hsum);
  }
  w.lhtr[i] = -(r * hsum);
}

// mu times the edge mask of element i
static __device__ __noinline__ double masked(double mu, const double *mask,
                                            size_t i) {
  return mu * mask[i];
}

// --- pass 4: edges: PV flux (transposed edges-on-edge), thickness flux,
// mean thickness, kinetic energy, edge Laplacian.  TRD: tracer diffusion
// on (a compile-time switch: with a runtime flag the compiler evaluated the
// diffusion products speculatively, 9 wasted FP64 instructions per edge).
template <int NE, bool TRD>
__device__ __forceinline__ void
pa_edge(const MeshView &m, const ModelView &p, const AuxView &a,
         const AdjView &v, const AdjWork &w, const AdjIO &io, unsigned i) {
  const int K = m.nlayers;
  if (i >= unsigned(m.nedges) * K)
    return;
  const unsigned CK = unsigned(m.ncells) * K;
  const int e = int(i / unsigned(K)), k = int(i - unsigned(e) * K);
  const int c0 = __ldg(m.ce + 2 * e), c1 = __ldg(m.ce + 2 * e + 1);
  const size_t i0 = size_t(c0) * K + k, i1 = size_t(c1) * K + k;
  const double F = a.F[i], u = io.vn[i];
  double lF = 0, lmh = 0;
  if (p.do_vn) {
    const double mu = io.mvn[i];
    if (!p.off_pv) {
      // PV flux: t_e = Q_e S1_e + S2_e, S1 = sum w F_j, S2 = sum w G_j
      double lG = 0, lFq = 0;
      for (int t = 0; t < v.nt; ++t) {
        const size_t is = size_t(__ldg(v.eoeT + v.nt * e + t)) * K + k;
        const double ws = __ldg(v.woeT + v.nt * e + t);
        lG = fma(ws, io.mvn[is], lG);
        lFq = fma(ws, w.Qmu[is], lFq);
      }
      const double S1 = a.S1 ? a.S1[i] : s1_of<NE>(m, a, e, k);
      w.lQ[i] = fma(S1, mu, F * lG);
      lF = fma(a.Q[i], lG, lFq);
    } else {
      w.lQ[i] = 0.0;
    }
    // kinetic energy from vn^2 (the factor 2 of d(vn^2) is in cke2_e2)
    if (!p.off_ke) {
      const double lu2 = fma(__ldg(v.cke2_e2 + 2 * e), w.lke[i0],
                             __ldg(v.cke2_e2 + 2 * e + 1) * w.lke[i1]);
      w.lvnp[i] = u * lu2; // mean-h term added below
    } else {
      w.lvnp[i] = 0.0;
    }
    if (p.vel_del2 | p.vel_del4) {
      // the dissipation terms are masked per edge and level (no multiply
      // without a mask)
      const double mum = m.mask ? masked(mu, m.mask, i) : mu;
      const double d = p.vel_del2 ? __ldg(p.c2e + e) * mum : 0.0;
      if (p.vel_del2 && w.gc2e) // parameter gradient of the del2 coefficient
        w.gc2e[i] = fma(mum, a.d2u[i], w.gc2e[i]);
      if (p.vel_del4) {
        // the del4 chain's first Laplacian: accumulated onto the del2 part,
        // or kept apart (ld2u4) where 1/max(dv, dc/4) differs from 1/dv
        // (inline: out of line the pass needed 48 registers instead of 40,
        // which cost more than the predicated-off block does without del4)
        const int v0 = __ldg(m.ve + 2 * e), v1 = __ldg(m.ve + 2 * e + 1);
        double d4 = w.ld2u4 ? 0.0 : d;
        d4 = fma(__ldg(v.cvr_e2 + 2 * e), w.lz4[size_t(v0) * K + k], d4);
        d4 = fma(__ldg(v.cvr_e2 + 2 * e + 1), w.lz4[size_t(v1) * K + k], d4);
        d4 = fma(__ldg(v.ccd_e2 + 2 * e), w.ld4[i0], d4);
        d4 = fma(__ldg(v.ccd_e2 + 2 * e + 1), w.ld4[i1], d4);
        if (w.ld2u4) {
          w.ld2u[i] = d;
          w.ld2u4[i] = d4;
        } else {
          w.ld2u[i] = d4;
        }
      } else {
        w.ld2u[i] = d;
      }
    }
  } else {
    w.lvnp[i] = 0.0;
  }
  const double g0 = __ldg(v.ccdh_e2 + 2 * e), g1 = __ldg(v.ccdh_e2 + 2 * e + 1);
  if (p.do_h && !p.off_hadv)
    lF = fma(__ldg(v.ccdh2_e2 + 2 * e), io.mh_[i0],
             fma(__ldg(v.ccdh2_e2 + 2 * e + 1), io.mh_[i1], lF));
  const bool adv = !p.off_tr_hadv;
  for (int l = 0; l < p.ntracers; ++l) {
    const size_t b = size_t(l) * CK;
    const double n0 = a.ntr[b + i0], n1 = a.ntr[b + i1];
    const double m0 = io.mtr[b + i0], m1 = io.mtr[b + i1];
    if (adv)
      lF = fma(n0 + n1, fma(g0, m0, g1 * m1), lF);
    if (TRD) {
      const double dn = n1 - n0;
      if (p.tr_del2)
        lmh = fma(dn, fma(__ldg(v.kd2_e2 + 2 * e), m0,
                          -(__ldg(v.kd2_e2 + 2 * e + 1) * m1)), lmh);
      if (p.tr_del4)
        lmh = fma(dn, fma(__ldg(v.ckq_e2 + 2 * e), w.lL[b + i0],
                          -(__ldg(v.ckq_e2 + 2 * e + 1) * w.lL[b + i1])), lmh);
    }
  }
  const double mh = mean_h(m, a, io.h, e, k);
  lmh = fma(u, lF, lmh);
  w.lmh[i] = lmh;
  w.lvnp[i] = fma(mh, lF, w.lvnp[i]);
}

// The del4 chain's parts kept apart where 1/max(dv, dc/4) differs from 1/dv
// (out of line, like the recompute fallbacks above): the cells' divergence
// transpose of the two edge Laplacians, and the vertex part of the second.
static __device__ __noinline__ double ldiv_split(const MeshView &m,
                                                 const AdjView &v,
                                                 const AdjWork &w, int c,
                                                 int k) {
  const int K = m.nlayers;
  double ld = 0;
  for (int j = 0; j < MAXE; ++j) {
    const size_t ie = size_t(__ldg(m.ec + 6 * c + j)) * K + k;
    ld = fma(__ldg(v.divadj + 6 * c + j), __dadd_rn(w.ld2u[ie], w.ld2u4[ie]),
             ld);
  }
  return ld;
}
static __device__ __noinline__ double lz_split(const MeshView &m,
                                               const AdjView &v,
                                               const AdjWork &w, int vx,
                                               int k, double lz) {
  const int K = m.nlayers;
  for (int j = 0; j < 3; ++j)
    lz = fma(__ldg(v.zetaadj4 + 3 * vx + j),
             w.ld2u4[size_t(__ldg(m.ev + 3 * vx + j)) * K + k], lz);
  return lz;
}

// --- pass 5: vertices: PV q = (zeta + f) / h_v, vorticity; and, in the
// C*K threads after the V*K vertex threads (launched with velocity
// dissipation on), the cells' velocity-divergence adjoint, which reads only
// the edge pass's output.  Splitting it from the cell pass lets the cell
// and edge output passes run concurrently.
__device__ __forceinline__ void
pa_vertex(const MeshView &m, const ModelView &p, const AuxView &a,
         const AdjView &v, const AdjWork &w, const AdjIO &io, unsigned i) {
  const int K = m.nlayers;
  const unsigned VK = unsigned(m.nvertices) * K;
  if (i >= VK) {
    i -= VK;
    if (i >= unsigned(m.ncells) * K)
      return;
    const int c = int(i / unsigned(K)), k = int(i - unsigned(c) * K);
    if (w.ld2u4) { // a loop per case: no predicated-off adds without it
      w.ldiv[i] = ldiv_split(m, v, w, c, k);
      return;
    }
    double ld = 0;
    for (int j = 0; j < MAXE; ++j)
      ld = fma(__ldg(v.divadj + 6 * c + j),
               w.ld2u[size_t(__ldg(m.ec + 6 * c + j)) * K + k], ld);
    w.ldiv[i] = ld;
    return;
  }
  const int vx = int(i / unsigned(K)), k = int(i - unsigned(vx) * K);
  const int e0 = __ldg(m.ev + 3 * vx), e1 = __ldg(m.ev + 3 * vx + 1),
            e2 = __ldg(m.ev + 3 * vx + 2);
  const double lq = w.lQ[size_t(e0) * K + k] + w.lQ[size_t(e1) * K + k] +
                    w.lQ[size_t(e2) * K + k];
  double lz = 0;
  if (p.vel_del2 | p.vel_del4) {
    lz = __ldg(v.zetaadj + 3 * vx) * w.ld2u[size_t(e0) * K + k];
    lz = fma(__ldg(v.zetaadj + 3 * vx + 1), w.ld2u[size_t(e1) * K + k], lz);
    lz = fma(__ldg(v.zetaadj + 3 * vx + 2), w.ld2u[size_t(e2) * K + k], lz);
    if (w.ld2u4) // the del4 chain's part, with 1/max(dv, dc/4)
      lz = lz_split(m, v, w, vx, k, lz);
  }
  // 1/h_vertex: the forward's value (taped, or recomputed)
  const double r = a.rhv ? a.rhv[i] : vertex_rcp(m, io.h, vx, k);
  w.lzeta[i] = fma(r, lq, lz);
  w.lhv[i] = -(a.q[i] * r * lq);
}

// --- pass 6: cells: thickness adjoint.
__device__ __forceinline__ void
pa_cell(const MeshView &m, const ModelView &p, const AuxView &a,
         const AdjView &v, const AdjWork &w, const AdjIO &io, unsigned i) {
  const int K = m.nlayers;
  if (i >= unsigned(m.ncells) * K)
    return;
  const int c = int(i / unsigned(K)), k = int(i - unsigned(c) * K);
  double lh = 0;
  for (int j = 0; j < MAXE; ++j) {
    const int e = __ldg(m.ec + 6 * c + j);
    lh = fma(__ldg(v.hm_c + 6 * c + j), w.lmh[size_t(e) * K + k], lh);
    if (p.do_vn)
      lh = fma(__ldg(v.ckvh + 6 * c + j),
               w.lhv[size_t(__ldg(v.cvtx + 6 * c + j)) * K + k], lh);
  }
  if (p.do_vn && !p.off_ssh)
    lh = fma(p.grav, w.lke[i], lh); // SSH gradient: g times the KE term
  if (p.ntracers > 0)
    lh = __dadd_rn(lh, w.lhtr[i]);
  emit(io, io.lh, io.acc_in_h, io.acc_h, io.nmu_h, io.lam_h, io.mh_, i, lh);
}

// --- pass 7: edges: normal velocity adjoint.
__device__ __forceinline__ void
pa_vn(const MeshView &m, const ModelView &p, const AuxView &a,
         const AdjView &v, const AdjWork &w, const AdjIO &io, unsigned i) {
  const int K = m.nlayers;
  if (i >= unsigned(m.nedges) * K)
    return;
  const int e = int(i / unsigned(K)), k = int(i - unsigned(e) * K);
  double l = w.lvnp[i];
  if (p.do_vn) {
    const int v0 = __ldg(m.ve + 2 * e), v1 = __ldg(m.ve + 2 * e + 1);
    l = fma(__ldg(v.cvr_e2 + 2 * e), w.lzeta[size_t(v0) * K + k], l);
    l = fma(__ldg(v.cvr_e2 + 2 * e + 1), w.lzeta[size_t(v1) * K + k], l);
    if (p.vel_del2 | p.vel_del4) {
      const int c0 = __ldg(m.ce + 2 * e), c1 = __ldg(m.ce + 2 * e + 1);
      l = fma(__ldg(v.ccd_e2 + 2 * e), w.ldiv[size_t(c0) * K + k], l);
      l = fma(__ldg(v.ccd_e2 + 2 * e + 1), w.ldiv[size_t(c1) * K + k], l);
    }
  }
  emit(io, io.lvn, io.acc_in_vn, io.acc_vn, io.nmu_vn, io.lam_vn, io.mvn, i,
       l);
}

// The passes of one adjoint stage, in launch order (pa_vel and pa_tr1, then
// pa_edge and pa_tr2, are independent pairs).
enum AdjPass { AP_VEL = 0, AP_TR1, AP_TR2, AP_EDGE, AP_VERTEX, AP_CELL, AP_VN,
               NAPASS };

// One pass by number; D2 / D4 tracer del2 / del4 (pa_tr1, pa_tr2), TRD
// tracer diffusion of either kind and NE the edges-on-edge width (pa_edge).
template <int PASS, int NE, bool D2, bool D4, bool TRD>
__device__ __forceinline__ void
adj_pass(const MeshView &m, const ModelView &p, const AuxView &a,
         const AdjView &v, const AdjWork &w, const AdjIO &io, unsigned i) {
  if (PASS == AP_VEL)
    pa_vel(m, p, a, v, w, io, i);
  else if (PASS == AP_TR1)
    pa_tr1<D2, D4>(m, p, a, v, w, io, i);
  else if (PASS == AP_TR2)
    pa_tr2<D4>(m, p, a, v, w, io, i);
  else if (PASS == AP_EDGE)
    pa_edge<NE, TRD>(m, p, a, v, w, io, i);
  else if (PASS == AP_VERTEX)
    pa_vertex(m, p, a, v, w, io, i);
  else if (PASS == AP_CELL)
    pa_cell(m, p, a, v, w, io, i);
  else
    pa_vn(m, p, a, v, w, io, i);
}

// Schedule actions.  ADV (a = first step, b = count) advances `cur` with
// plain steps; STORE / RESTORE (a = slot) copy `cur` to / from a snapshot;
// TAPE_ADJ (a = step, b = tape) tapes the step from `cur` into tape b and
// runs its adjoint; TADV (a = step, b = tape) is a taped advance: the step
// is taped into tape b and its result replaces `cur`; ADJ (a = step,
// b = tape) runs the adjoint of a step taped earlier; FWD_END ends the
// forward sweep (x_N is in `cur`).
enum ActType { A_ADV = 0, A_STORE, A_RESTORE, A_TAPE_ADJ, A_TADV, A_ADJ,
               A_FWD_END };
struct AdjAction {
  int type;
  int a, b;
};

// A captured graph replayed while dt stays the same.
struct AdjGraph {
  cudaGraphExec_t exec = nullptr;
  double dt = 0;
  unsigned long long version = 0; // the model's term version captured
  long long launches = 0;         // kernels per replay
};

// One step's tape: the stage inputs, the taped step's accumulator and the
// intermediates of every stage, with the graphs that write and read it.
struct TapeSlot {
  swg_state X[5] = {}; // stage inputs; X[0] is the step's start state
  swg_state acc = nullptr;
  AuxView taux[5]{};
  AdjGraph tape_adj; // tape without the step's result, then its adjoint
  AdjGraph tadv;     // taped advance: X[0] <- cur, tape, result into cur
  AdjGraph adj;      // adjoint of the taped step
  // recorded on the caller's stream after each use of the tape by an
  // adjoint, so that a taped advance on the advance stream waits for it
  cudaEvent_t free_ev = nullptr;
};
constexpr int kTapes = 2;

} // namespace swg

struct swg_adjoint_s {
  swg_model model;
  int nsnap;
  swg::AdjView av{};
  swg::AdjWork aw{};
  std::vector<void *> allocs;
  swg_stepper stepper = nullptr; // plain advances (graph replay)
  std::vector<swg_state> snaps;
  // stepper differentiated: RK4 (4 stages) or LSRK with 5 or 1 stages;
  // rka / rkb are its coefficients (as in swg_stepper_create)
  int kind = SWG_STEPPER_RK4, ns = 4;
  std::vector<double> rka, rkb;
  swg_state cur = nullptr, lam = nullptr, lacc = nullptr, mu = nullptr,
            mu2 = nullptr;
  swg::TapeSlot tp[swg::kTapes];
  // tangent-linear model buffers
  swg::AuxViewT<swg::Dual> daux{};
  swg::Dual *dS = nullptr, *dacc = nullptr, *dP0 = nullptr, *dP1 = nullptr,
            *dT = nullptr;
  // schedule
  std::vector<swg::AdjAction> actions;
  size_t pos = 0;
  int nsteps = 0;
  double t0 = 0, dt = 0;
  long long plain_steps = 0, taped_steps = 0, taped_advances = 0;
  unsigned fwd_terms = 0; // the model's term set at the last forward sweep
  int state = 0; // 0 idle, 1 forward done (the last steps taped)
  bool grad_ready = false; // a backward sweep has completed
  // backward sweep: restores, stores, plain and taped advances run on
  // `adv`, concurrently with the caller's stream, which tapes and reverses
  // the steps; `ready` = the advance stream's work so far is done (x_i in
  // cur, taped advances written), `freed` = cur was copied to a tape
  cudaStream_t adv = nullptr;
  cudaEvent_t go = nullptr, ready = nullptr, freed = nullptr;
};

namespace swg {

// Domain of each pass for a model: threads run the indices
// [base, base + units) (0 units: the pass is not launched).
inline void adj_units(const swg_model_s *md, unsigned units[NAPASS],
                      unsigned base[NAPASS]) {
  const ModelView &p = md->view;
  const unsigned K = md->mesh->nlayers, C = md->mesh->ncells,
                 E = md->mesh->nedges, V = md->mesh->nvertices;
  for (int q = 0; q < NAPASS; ++q)
    base[q] = 0;
  base[AP_VEL] = p.vel_del4 ? 0u : V * K; // vertex part: velocity del4 only
  units[AP_VEL] = p.do_vn ? (V + C + E) * K - base[AP_VEL] : 0u;
  units[AP_TR1] = units[AP_TR2] = p.ntracers > 0 ? C * K : 0u;
  units[AP_EDGE] = E * K;
  units[AP_VERTEX] = p.do_vn ? (V + ((p.vel_del2 | p.vel_del4) ? C : 0u)) * K
                             : 0u;
  units[AP_CELL] = C * K;
  units[AP_VN] = E * K;
}

// host helpers shared by the single-instance adjoint and the ensemble
inline size_t words(const swg_model_s *md) {
  return (size_t(md->mesh->ncells) + md->mesh->nedges +
          size_t(md->params.ntracers) * md->mesh->ncells) *
         md->mesh->nlayers;
}

// stage input of a tape: a disabled field keeps its start-of-step value
inline void stage_ptrs(const swg_adjoint_s *ad, const TapeSlot &tp, int s,
                       const double **h, const double **vn,
                       const double **tr) {
  const ModelView &p = ad->model->view;
  *h = p.do_h ? tp.X[s]->h : tp.X[0]->h;
  *vn = p.do_vn ? tp.X[s]->vn : tp.X[0]->vn;
  *tr = tp.X[s]->tr;
}

// the b coefficients of the stepper the adjoint differentiates
inline const double *step_rkb(const swg_adjoint_s *ad) {
  static const double rk4b[4] = {1. / 6, 1. / 3, 1. / 3, 1. / 6};
  return ad->kind != SWG_STEPPER_RK4 ? ad->rkb.data() : rk4b;
}
inline const double *step_rka(const swg_adjoint_s *ad) {
  static const double rk4a[3] = {1. / 2, 1. / 2, 1};
  return ad->kind != SWG_STEPPER_RK4 ? ad->rka.data() : rk4a;
}

// The model's tendency-term switches as a bit set: a backward sweep must
// see the set its forward sweep ran with (its re-advances and tapes would
// differ otherwise).
inline unsigned term_set(const swg_model_s *md) {
  const ModelView &p = md->view;
  const int f[] = {p.off_hadv, p.off_pv, p.off_ke, p.off_ssh, p.off_tr_hadv,
                   p.vel_del2, p.vel_del4, p.tr_del2, p.tr_del4};
  unsigned s = 0;
  for (int i = 0; i < 9; ++i)
    s |= unsigned(f[i] != 0) << i;
  return s;
}

// The checkpoint schedule of nsteps steps, nsnapshots snapshots and a
// stepper of nstages stages (swg_adjoint.cu, Planner).
std::vector<AdjAction> plan_schedule(int nsteps, int nsnapshots, int nstages);

// The stage passes' inputs and outputs (AdjIO) for stage s of the adjoint
// of the step taped in tp: the state X_s, mu_s, the accumulation of lambda
// and the next stage's mu (swg_adjoint.cu, adjoint_step).
AdjIO stage_io(const swg_adjoint_s *ad, const TapeSlot &tp, int s, double dt);
// The taped step (swg_adjoint.cu, tape_step): stage s's arguments (inputs
// X_s, epilogue into X_{s+1}, or into `out` for the last stage), what must
// precede the first stage (RK4 with `out`: frozen fields copied), and what
// must precede stage s (LSRK: X_s copied to the buffer the stage updates).
StageArgs tape_stage_args(const swg_adjoint_s *ad, const TapeSlot &tp, int s,
                          double dt, swg_state out);
int tape_prologue(const swg_adjoint_s *ad, const TapeSlot &tp, swg_state out,
                  cudaStream_t st);
int tape_stage_copy(const swg_adjoint_s *ad, const TapeSlot &tp, int s,
                    swg_state out, cudaStream_t st);
// y = a x over n words of the state arrays (swg_adjoint.cu)
void adj_lincomb(swg_state y, swg_state x, double a, long long n,
                 cudaStream_t st);

} // namespace swg
