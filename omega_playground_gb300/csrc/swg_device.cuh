// Per-element passes of one tendency evaluation + stage update, shared by
// the single-instance kernels (swg_kernels.cu) and the batched persistent
// kernel (swg_batch.cu).  Each function handles one flat index i of its pass
// domain: (entity, level) with the level fastest.  Callers guarantee i is in
// range (pt_aux2: i < (V + C) K, vertices first).
#pragma once

#include "swg_internal.h"

namespace swg {

// Forward-mode dual number (value, tangent): the pass functions instantiated
// with it are the exact tangent-linear model of the double instantiation
// (the value part runs the identical operation sequence).
using ::fma; // keep the double overload visible beside the Dual ones
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator+(Dual a, double b) { return {a.v + b, a.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator-(Dual a) { return {-a.v, -a.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) {
  return {a.v * b.v, fma(a.d, b.v, a.v * b.d)};
}
__device__ __forceinline__ Dual operator*(double a, Dual b) { return {a * b.v, a * b.d}; }
__device__ __forceinline__ Dual operator*(Dual a, double b) { return {a.v * b, a.d * b}; }
__device__ __forceinline__ Dual &operator+=(Dual &a, Dual b) { a = a + b; return a; }
__device__ __forceinline__ Dual fma(double a, Dual b, Dual c) {
  return {::fma(a, b.v, c.v), ::fma(a, b.d, c.d)};
}
__device__ __forceinline__ Dual fma(Dual a, double b, Dual c) {
  return {::fma(a.v, b, c.v), ::fma(a.d, b, c.d)};
}
__device__ __forceinline__ Dual fma(Dual a, Dual b, Dual c) {
  return {::fma(a.v, b.v, c.v), ::fma(a.d, b.v, ::fma(a.v, b.d, c.d))};
}

// 1/x: hardware estimate refined by two Newton-Raphson steps
// r <- r + r (1 - x r); each step squares the relative error of the estimate.
// The estimate is the .ftz form: a subnormal input (|x| < 2^-1022) counts as
// zero (result infinite) and a result below 2^-1022 flushes to zero, so the
// function is for |x| in [2^-1022, 2^1022], far beyond any thickness.  On
// the GPU it is within 1 ulp of the correctly rounded 1.0 / x over 1e-6 ..
// 1e6 and random mantissas in [2^-40, 2^40] (tests/cpp/rcp_accuracy.cu).
__device__ __forceinline__ double rcp_nr(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}
__device__ __forceinline__ Dual rcp_nr(Dual x) {
  const double r = rcp_nr(x.v);
  return {r, -(r * r) * x.d};
}
using ::sqrt;
__device__ __forceinline__ Dual sqrt(Dual x) {
  const double s = ::sqrt(x.v);
  return {s, x.d * (0.5 / s)};
}

template <class T>
__device__ __forceinline__ void epilogue(const Epilogue &ep,
                                         const FieldIOT<T> &f, size_t i, T x) {
  switch (ep.mode) {
  case EPI_REPLACE:
    f.tend[i] = x;
    break;
  case EPI_INCREMENT:
    f.tend[i] += x;
    break;
  case EPI_LSRK: {
    const T t = fma(ep.a, f.tend[i], x);
    f.tend[i] = t;
    f.out[i] = fma(ep.dtb, t, f.out[i]);
  } break;
  case EPI_LSRK_TEND:
    f.tend[i] = fma(ep.a, f.tend[i], x);
    break;
  case EPI_RK4_FIRST: {
    const T s = f.old[i];
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
template <class T>
__device__ __forceinline__ void
pt_vertex(const MeshView &m, const ModelView &p, const AuxViewT<T> &a,
          const T *__restrict__ h, const T *__restrict__ vn, unsigned i) {
  const int K = m.nlayers;
  const int v = int(i / unsigned(K)), k = int(i - unsigned(v) * unsigned(K));
  T z, hv;
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
  const T r = rcp_nr(hv);
  a.q[i] = (z + __ldg(p.f_vertex + v)) * r;
  if (a.rhv)
    a.rhv[i] = r;
  if (p.vel_del2 | p.vel_del4)
    a.zeta[i] = z;
}

// Cell pass 1: velocity divergence (for the dissipation terms) and the
// normalised tracers tr / h.
template <class T>
__device__ __forceinline__ void
pt_cell1(const MeshView &m, const ModelView &p, const AuxViewT<T> &a,
         const T *__restrict__ h, const T *__restrict__ vn,
         const T *__restrict__ tr, unsigned i) {
  const int K = m.nlayers;
  const unsigned CK = unsigned(m.ncells) * unsigned(K);
  const int c = int(i / unsigned(K)), k = int(i - unsigned(c) * unsigned(K));
  if (p.do_vn && (p.vel_del2 | p.vel_del4)) {
    T dv = __ldg(m.ccd + 6 * c) * vn[size_t(__ldg(m.ec + 6 * c)) * K + k];
#pragma unroll
    for (int j = 1; j < MAXE; ++j)
      dv = fma(__ldg(m.ccd + 6 * c + j),
               vn[size_t(__ldg(m.ec + 6 * c + j)) * K + k], dv);
    a.div[i] = dv;
  }
  if (p.ntracers > 0) {
    const T r = rcp_nr(h[i]);
    if (a.rh)
      a.rh[i] = r;
    for (int l = 0; l < p.ntracers; ++l) {
      const size_t t = size_t(l) * CK + i;
      a.ntr[t] = tr[t] * r;
    }
  }
}

// Edge pass 1: mean thickness, thickness flux F = mean_h vn, vn^2, edge PV
// sum Q = q(v0) + q(v1), G = F Q, and the edge Laplacian of the velocity.
template <class T>
__device__ __forceinline__ void
pt_edge1(const MeshView &m, const ModelView &p, const AuxViewT<T> &a,
         const T *__restrict__ h, const T *__restrict__ vn, unsigned i) {
  const int K = m.nlayers;
  const int e = int(i / unsigned(K)), k = int(i - unsigned(e) * unsigned(K));
  const int c0 = __ldg(m.ce + 2 * e), c1 = __ldg(m.ce + 2 * e + 1);
  const T mh = 0.5 * (h[size_t(c0) * K + k] + h[size_t(c1) * K + k]);
  const T u = vn[i];
  const T F = mh * u;
  a.F[i] = F;
  if (a.mh) // kept by every nonlinear model and in the adjoint's tape
    a.mh[i] = mh;
  if (p.do_vn) {
    const int v0 = __ldg(m.ve + 2 * e), v1 = __ldg(m.ve + 2 * e + 1);
    const T Q = a.q[size_t(v0) * K + k] + a.q[size_t(v1) * K + k];
    a.Q[i] = Q;
    a.G[i] = F * Q;
    a.u2[i] = u * u;
    if (p.vel_del2 | p.vel_del4) {
      const T dd = a.div[size_t(c1) * K + k] - a.div[size_t(c0) * K + k];
      const T dz = a.zeta[size_t(v1) * K + k] - a.zeta[size_t(v0) * K + k];
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
template <class T>
__device__ __forceinline__ void pt_aux2(const MeshView &m, const ModelView &p,
                                        const AuxViewT<T> &a, unsigned i) {
  const int K = m.nlayers;
  const unsigned VK = unsigned(m.nvertices) * unsigned(K);
  const unsigned CK = unsigned(m.ncells) * unsigned(K);
  const bool vel = p.do_vn && p.vel_del4;
  if (i < VK) {
    if (!vel)
      return;
    const int v = int(i / unsigned(K)), k = int(i - unsigned(v) * unsigned(K));
    T z = __ldg(m.cvr + 3 * v) * a.d2u4[size_t(__ldg(m.ev + 3 * v)) * K + k];
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
    T ke = __ldg(m.cke + 6 * c) * a.u2[size_t(__ldg(m.ec + 6 * c)) * K + k];
#pragma unroll
    for (int j = 1; j < MAXE; ++j)
      ke = fma(__ldg(m.cke + 6 * c + j),
               a.u2[size_t(__ldg(m.ec + 6 * c + j)) * K + k], ke);
    a.ke[i] = ke;
  }
  if (vel) {
    T d = __ldg(m.ccd + 6 * c) * a.d2u4[size_t(__ldg(m.ec + 6 * c)) * K + k];
#pragma unroll
    for (int j = 1; j < MAXE; ++j)
      d = fma(__ldg(m.ccd + 6 * c + j),
              a.d2u4[size_t(__ldg(m.ec + 6 * c + j)) * K + k], d);
    a.d4[i] = d;
  }
  if (p.ntracers > 0 && p.tr_del4) {
    // L = sum_j w_j (n_nb - n_c), w_j = ckq_j mean_h_j
    T w[MAXE], M;
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
      const T *n = a.ntr + size_t(l) * CK;
      T acc = w[0] * n[size_t(nb[0]) * K + k];
#pragma unroll
      for (int j = 1; j < MAXE; ++j)
        acc = fma(w[j], n[size_t(nb[j]) * K + k], acc);
      a.lap[size_t(l) * CK + i] = fma(-M, n[i], acc);
    }
  }
}

// Bottom drag -c_d sqrt(ke_0 + ke_1) vn / mean_h added to t on the lowest
// level (the term commented out at shallow_water_hierarchical.cpp:479-486),
// with the auxiliary state's mean thickness (h_drag_edge = h_mean).  Out of
// line: inlined, the short branch was if-converted, and every edge of every
// model without drag issued its FP64 instructions with the predicate off.
template <class T>
__device__ __noinline__ T drag_add(const MeshView &m, const ModelView &p,
                                   const AuxViewT<T> &a,
                                   const StageArgsT<T> &s, int c0, int c1,
                                   size_t i, int k, T t) {
  const int K = m.nlayers;
  const T hm = a.mh ? a.mh[i]
                    : 0.5 * (s.h[size_t(c0) * K + k] + s.h[size_t(c1) * K + k]);
  const T ks = a.ke[size_t(c0) * K + k] + a.ke[size_t(c1) * K + k];
  return t + (-p.drag_coeff * sqrt(ks)) * s.vn[i] * rcp_nr(hm);
}

// The del2 and del4 velocity dissipation of edge element i with a per-level
// edge mask (mask * coefficient).  Out of line: inlined, the compiler
// if-converted the masked and unmasked forms, and every edge of an unmasked
// model issued the masked form's multiplies with the predicate off.
template <class T>
__device__ __noinline__ T masked_dissipation(const MeshView &m,
                                             const ModelView &p,
                                             const AuxViewT<T> &a,
                                             const StageArgsT<T> &s, int c0,
                                             int c1, size_t i, int k,
                                             double idc, T t) {
  const int K = m.nlayers;
  const int e = int(i / unsigned(K));
  const double mk = m.mask[i];
  if (p.vel_del2)
    t = fma(__ldg(p.c2e + e) * mk, a.d2u[i], t);
  if (p.vel_del4) {
    const int v0 = __ldg(m.ve + 2 * e), v1 = __ldg(m.ve + 2 * e + 1);
    const T dd = a.d4[size_t(c1) * K + k] - a.d4[size_t(c0) * K + k];
    const T dz = a.z4[size_t(v1) * K + k] - a.z4[size_t(v0) * K + k];
    const T l = fma(dd, idc, -(dz * __ldg(m.inv_dv + e)));
    t = fma(__ldg(p.c4e + e) * mk, l, t);
  }
  (void)s;
  return t;
}

// Edge final pass: normal-velocity tendency (PV flux, Bernoulli gradient,
// del2 and del4 dissipation) and its stage update.
template <int NE, class T>
__device__ __forceinline__ void pt_edge_final(const MeshView &m,
                                              const ModelView &p,
                                              const AuxViewT<T> &a,
                                              const StageArgsT<T> &s,
                                              unsigned i) {
  const int K = m.nlayers;
  const int e = int(i / unsigned(K)), k = int(i - unsigned(e) * unsigned(K));
  // potential-vorticity flux: sum_j w_j F_j (Q_e + Q_j) / 4 with w/4 in woe
  T t{};
  if (!p.off_pv) {
    T S1, S2;
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
    if (a.S1)
      a.S1[i] = S1;
    t = fma(a.Q[i], S1, S2);
  }
  const int c0 = __ldg(m.ce + 2 * e), c1 = __ldg(m.ce + 2 * e + 1);
  const double idc = __ldg(m.inv_dc + e);
  // kinetic-energy and sea-surface-height gradients (the differences are
  // taken before scaling, as in the reference, so g h ~ 1e4 never rounds)
  if (!p.off_ke)
    t = fma(-idc, a.ke[size_t(c1) * K + k] - a.ke[size_t(c0) * K + k], t);
  if (!p.off_ssh)
    t = fma(-__ldg(p.gidc + e),
            s.h[size_t(c1) * K + k] - s.h[size_t(c0) * K + k], t);
  if (p.drag && k == p.drag_level)
    t = drag_add(m, p, a, s, c0, c1, i, k, t);
  if (m.mask) { // masked dissipation: out of line (see masked_dissipation)
    t = masked_dissipation(m, p, a, s, c0, c1, i, k, idc, t);
  } else {
    if (p.vel_del2)
      t = fma(__ldg(p.c2e + e), a.d2u[i], t);
    if (p.vel_del4) { // the coefficient folded into c4e/dc and -c4e/dv
      const int v0 = __ldg(m.ve + 2 * e), v1 = __ldg(m.ve + 2 * e + 1);
      const T dd = a.d4[size_t(c1) * K + k] - a.d4[size_t(c0) * K + k];
      const T dz = a.z4[size_t(v1) * K + k] - a.z4[size_t(v0) * K + k];
      t = fma(__ldg(p.c4i + e), dd, t);
      t = fma(__ldg(p.c4v + e), dz, t);
    }
  }
  epilogue(s.ep, s.fvn, i, t);
}

// Cell final pass: thickness tendency and tracer tendencies (advection,
// del2, del4) with their stage updates.  PAIRS: tracers two at a time (the
// single-instance kernel; the batched kernels, which already give each
// thread several elements, keep one at a time and their registers).
template <class T, bool PAIRS = false>
__device__ __forceinline__ void pt_cell_final(const MeshView &m,
                                              const ModelView &p,
                                              const AuxViewT<T> &a,
                                              const StageArgsT<T> &s,
                                              unsigned i) {
  const int K = m.nlayers;
  const unsigned CK = unsigned(m.ncells) * unsigned(K);
  const int c = int(i / unsigned(K)), k = int(i - unsigned(c) * unsigned(K));
  // a_j = -F_j ccd_j / 2: half the flux divergence weight of edge j
  T w[MAXE], Sa{};
  int ej[MAXE];
#pragma unroll
  for (int j = 0; j < MAXE; ++j) {
    ej[j] = __ldg(m.ec + 6 * c + j);
    w[j] = T{};
  }
  if (!p.off_hadv || !p.off_tr_hadv) {
#pragma unroll
    for (int j = 0; j < MAXE; ++j)
      w[j] = __ldg(m.ccdh + 6 * c + j) * a.F[size_t(ej[j]) * K + k];
    Sa = w[0] + w[1];
#pragma unroll
    for (int j = 2; j < MAXE; ++j)
      Sa += w[j];
  }
  if (p.do_h) // -sum_j ccd_j F_j, or nothing with thickness advection off
    epilogue(s.ep, s.fh, i, p.off_hadv ? T{} : 2.0 * Sa);
  if (p.ntracers == 0)
    return;
  if (p.off_tr_hadv) { // tracer advection off: only diffusion weights
    Sa = T{};
#pragma unroll
    for (int j = 0; j < MAXE; ++j)
      w[j] = T{};
  }
  // advection + del2: sum_j a_j (n_c + n_j) + b_j (n_j - n_c); with a
  // uniform del2 scaling the del2 part is eddy_diff2 s L_c instead, taken
  // with the del4 stencil's centre weight (r4f)
  const bool fold = p.tr_del2 && p.tr_del4 && p.r4f;
  T wc = Sa;
  if (p.tr_del2 && !fold) {
    T b[MAXE], Sb;
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
  // del4 centre weight: -sum r4, plus eddy_diff2 s when del2 is folded in
  const double rc = !p.tr_del4 ? 0.0 : fold ? __ldg(p.r4f + c)
                                            : -__ldg(p.r4sum + c);
  // tracers in pairs: two independent FMA chains per thread keep more
  // loads and FP64 operations in flight (each tracer's operation sequence
  // is the same as alone, so the results are too)
  int l = 0;
  for (; PAIRS && l + 1 < p.ntracers; l += 2) {
    const size_t b0 = size_t(l) * CK, b1 = b0 + CK;
    const T *n0 = a.ntr + b0, *n1 = a.ntr + b1;
    T acc0 = wc * n0[i], acc1 = wc * n1[i];
#pragma unroll
    for (int j = 0; j < MAXE; ++j) {
      acc0 = fma(w[j], n0[size_t(nb[j]) * K + k], acc0);
      acc1 = fma(w[j], n1[size_t(nb[j]) * K + k], acc1);
    }
    if (p.tr_del4) {
      const T *L0 = a.lap + b0, *L1 = a.lap + b1;
      acc0 = fma(rc, L0[i], acc0);
      acc1 = fma(rc, L1[i], acc1);
#pragma unroll
      for (int j = 0; j < MAXE; ++j) {
        const double r = __ldg(p.r4 + 6 * c + j);
        acc0 = fma(r, L0[size_t(nb[j]) * K + k], acc0);
        acc1 = fma(r, L1[size_t(nb[j]) * K + k], acc1);
      }
    }
    epilogue(s.ep, s.ftr, b0 + i, acc0);
    epilogue(s.ep, s.ftr, b1 + i, acc1);
  }
  for (; l < p.ntracers; ++l) {
    const size_t base = size_t(l) * CK;
    const T *n = a.ntr + base;
    T acc = wc * n[i];
#pragma unroll
    for (int j = 0; j < MAXE; ++j)
      acc = fma(w[j], n[size_t(nb[j]) * K + k], acc);
    if (p.tr_del4) {
      const T *L = a.lap + base;
      acc = fma(rc, L[i], acc);
#pragma unroll
      for (int j = 0; j < MAXE; ++j)
        acc = fma(__ldg(p.r4 + 6 * c + j), L[size_t(nb[j]) * K + k], acc);
    }
    epilogue(s.ep, s.ftr, base + i, acc);
  }
}


// Pass domain sizes (threads) of pass `pass` for one instance.
enum Pass { P_VERTEX = 0, P_CELL1, P_EDGE1, P_AUX2, P_EDGE_FINAL,
            P_CELL_FINAL, NPASS };

// One member of a batched launch (swg_batch.cu, swg_ensemble.cu): its mesh,
// model, intermediates, stage arguments and the element count of each pass.
struct Member {
  MeshView m;
  ModelView p;
  AuxView a;
  StageArgs stage[5];
  unsigned units[NPASS]; // elements of each pass (0 = pass not needed)
  unsigned aux2_base;    // first element of the aux2 pass domain
};
// (swg_batch.cu) element counts of a model's passes
void batch_pass_units(const swg_model_s *md, unsigned units[NPASS],
                      unsigned &aux2_base);
// (swg_batch.cu) passes [pass0, pass1] of stage `stage` over the nmem
// members of the device table `mem`, one 256-thread block per virtual block
// of 256 x items elements (items 1 or 2 per thread); prefix: [NPASS][nmem +
// 1] virtual-block offsets of the members for that block size (device) and
// prefix_h its host copy (grid sizes).
int batch_launch_passes(const Member *mem, int nmem, const unsigned *prefix,
                        const unsigned *prefix_h, int ne, int items,
                        int pass0, int pass1, int stage, cudaStream_t st);

// LinearShallowWaterModel (shallow_water_hierarchical.cpp:680-740):
// vn_t = f sum_j w_j vn_j - g (h_1 - h_0) / dc and h_t = -h0 div(vn), each
// with its stage update.
template <int NE, class T>
__device__ __forceinline__ void pt_lin_edge(const MeshView &m,
                                            const ModelView &p,
                                            const StageArgsT<T> &s,
                                            unsigned i) {
  const int K = m.nlayers;
  const int e = int(i / unsigned(K)), k = int(i - unsigned(e) * unsigned(K));
  T vt = __ldg(m.woe + NE * e) * s.vn[size_t(__ldg(m.eoe + NE * e)) * K + k];
#pragma unroll
  for (int j = 1; j < NE; ++j)
    vt = fma(__ldg(m.woe + NE * e + j),
             s.vn[size_t(__ldg(m.eoe + NE * e + j)) * K + k], vt);
  const int c0 = __ldg(m.ce + 2 * e), c1 = __ldg(m.ce + 2 * e + 1);
  const T t = fma(-__ldg(p.gidc + e),
                  s.h[size_t(c1) * K + k] - s.h[size_t(c0) * K + k],
                  p.f4 * vt);
  epilogue(s.ep, s.fvn, i, t);
}

template <class T>
__device__ __forceinline__ void pt_lin_cell(const MeshView &m,
                                            const ModelView &p,
                                            const StageArgsT<T> &s,
                                            unsigned i) {
  const int K = m.nlayers;
  const int c = int(i / unsigned(K)), k = int(i - unsigned(c) * unsigned(K));
  T d = __ldg(m.ccd + 6 * c) * s.vn[size_t(__ldg(m.ec + 6 * c)) * K + k];
#pragma unroll
  for (int j = 1; j < MAXE; ++j)
    d = fma(__ldg(m.ccd + 6 * c + j),
            s.vn[size_t(__ldg(m.ec + 6 * c + j)) * K + k], d);
  epilogue(s.ep, s.fh, i, -p.h0 * d);
}

} // namespace swg
