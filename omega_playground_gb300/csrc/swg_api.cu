// C ABI of the GB300 shallow-water library: handles, host-side table
// derivation, stepper orchestration and CUDA-graph replay.  See
// include/swgpu.h for the contract of every entry point.
#include "swg_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <stdexcept>

namespace swg {

std::atomic<long long> g_launches{0};
static thread_local std::string t_last_error;

int fail(int code, const std::string &msg) {
  t_last_error = msg;
  return code;
}

int abi_exception(const char *entry) noexcept {
  int code = SWG_ERR_ARG;
  const char *what = "unexpected host exception";
  try {
    throw;
  } catch (const std::bad_alloc &) {
    code = SWG_ERR_OOM;
    what = "host allocation failed";
  } catch (const std::length_error &) {
    code = SWG_ERR_OOM;
    what = "host allocation too large";
  } catch (...) {
  }
  try { // the message needs memory too; the status is returned without it
    fail(code, std::string(entry) + ": " + what);
  } catch (...) {
  }
  return code;
}

int cuda_fail(cudaError_t err, const char *what) {
  (void)cudaGetLastError(); // clear sticky-free errors
  const int code =
      err == cudaErrorMemoryAllocation ? SWG_ERR_OOM : SWG_ERR_CUDA;
  return fail(code, std::string(what) + ": " + cudaGetErrorString(err));
}

namespace {

template <class T>
int upload(std::vector<void *> &allocs, const T *host, size_t n,
           const T **dev) {
  void *p = nullptr;
  cudaError_t err = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
  if (err != cudaSuccess)
    return cuda_fail(err, "cudaMalloc (mesh table)");
  allocs.push_back(p);
  if (n) {
    err = cudaMemcpy(p, host, n * sizeof(T), cudaMemcpyHostToDevice);
    if (err != cudaSuccess)
      return cuda_fail(err, "cudaMemcpy (mesh table)");
  }
  *dev = static_cast<const T *>(p);
  return SWG_OK;
}

int dalloc(std::vector<void *> &allocs, size_t n, double **dev) {
  void *p = nullptr;
  cudaError_t err = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(double));
  if (err != cudaSuccess)
    return cuda_fail(err, "cudaMalloc (work array)");
  allocs.push_back(p);
  err = cudaMemset(p, 0, std::max<size_t>(n, 1) * sizeof(double));
  if (err != cudaSuccess)
    return cuda_fail(err, "cudaMemset (work array)");
  *dev = static_cast<double *>(p);
  return SWG_OK;
}

void free_all(std::vector<void *> &allocs) {
  for (void *p : allocs)
    cudaFree(p);
  allocs.clear();
}

bool in_range(const int *a, size_t n, int lo, int hi) {
  for (size_t i = 0; i < n; ++i)
    if (a[i] < lo || a[i] >= hi)
      return false;
  return true;
}

// true when a is NULL or every entry equals x
bool all_equal(const int *a, size_t n, int x) {
  for (size_t i = 0; a && i < n; ++i)
    if (a[i] != x)
      return false;
  return true;
}

cudaStream_t as_stream(void *s) { return static_cast<cudaStream_t>(s); }

int check_launch(const char *what) {
  cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? SWG_OK : cuda_fail(err, what);
}

} // namespace
} // namespace swg

using namespace swg;

extern "C" const char *swg_last_error(void) { return t_last_error.c_str(); }
extern "C" const char *swg_version(void) { return "omega_playground_gb300 0.1 sm_103a fp64"; }
extern "C" long long swg_kernel_launches(void) { return g_launches.load(); }

// ------------------------------------------------------------------ mesh ---

extern "C" int swg_mesh_create(const swg_mesh_desc *d, swg_mesh *out) try {
  if (!d || !out)
    return fail(SWG_ERR_ARG, "swg_mesh_create: NULL argument");
  *out = nullptr;
  const long long C = d->ncells, E = d->nedges, V = d->nvertices,
                  K = d->nlayers;
  if (C <= 0 || E <= 0 || V <= 0 || K <= 0)
    return fail(SWG_ERR_ARG, "swg_mesh_create: sizes must be positive");
  if (E * K >= (1LL << 31) || (V + C) * K >= (1LL << 31))
    return fail(SWG_ERR_ARG,
                "swg_mesh_create: entity*level count exceeds 32-bit indexing");
  if (!d->nedges_on_cell || !d->edges_on_cell || !d->nedges_on_edge ||
      !d->edges_on_edge || !d->cells_on_edge || !d->vertices_on_edge ||
      !d->edges_on_vertex || !d->cells_on_vertex || !d->area_cell ||
      !d->edge_sign_on_cell || !d->dc_edge || !d->dv_edge ||
      !d->weights_on_edge || !d->area_triangle || !d->kiteareas_on_vertex ||
      !d->edge_sign_on_vertex)
    return fail(SWG_ERR_ARG, "swg_mesh_create: a required table is NULL");
  // ---- validate every index a kernel will dereference
  for (long long c = 0; c < C; ++c) {
    const int n = d->nedges_on_cell[c];
    if (n < 1 || n > MAXE)
      return fail(SWG_ERR_ARG, "swg_mesh_create: nedges_on_cell out of [1,6]");
    if (!in_range(d->edges_on_cell + 6 * c, n, 0, int(E)))
      return fail(SWG_ERR_ARG, "swg_mesh_create: edges_on_cell out of range");
    if (!(d->area_cell[c] > 0))
      return fail(SWG_ERR_ARG, "swg_mesh_create: area_cell must be > 0");
  }
  if (!in_range(d->cells_on_edge, 2 * E, 0, int(C)) ||
      !in_range(d->vertices_on_edge, 2 * E, 0, int(V)) ||
      !in_range(d->edges_on_vertex, 3 * V, 0, int(E)) ||
      !in_range(d->cells_on_vertex, 3 * V, 0, int(C)))
    return fail(SWG_ERR_ARG, "swg_mesh_create: connectivity out of range");
  for (long long e = 0; e < E; ++e) {
    const int n = d->nedges_on_edge[e];
    if (n < 0 || n > 12)
      return fail(SWG_ERR_ARG, "swg_mesh_create: nedges_on_edge out of [0,12]");
    if (!in_range(d->edges_on_edge + 12 * e, n, 0, int(E)))
      return fail(SWG_ERR_ARG, "swg_mesh_create: edges_on_edge out of range");
    if (!(d->dc_edge[e] > 0) || !(d->dv_edge[e] > 0))
      return fail(SWG_ERR_ARG, "swg_mesh_create: dc_edge/dv_edge must be > 0");
  }
  for (long long v = 0; v < V; ++v)
    if (!(d->area_triangle[v] > 0))
      return fail(SWG_ERR_ARG, "swg_mesh_create: area_triangle must be > 0");
  if ((d->max_level_cell && !in_range(d->max_level_cell, C, 0, int(K) + 1)) ||
      (d->max_level_vertex_bot &&
       !in_range(d->max_level_vertex_bot, V, 0, int(K) + 1)))
    return fail(SWG_ERR_ARG, "swg_mesh_create: max level out of [0, nlayers]");

  swg_mesh m = new (std::nothrow) swg_mesh_s();
  if (!m)
    return fail(SWG_ERR_OOM, "swg_mesh_create: host allocation");
  m->ncells = int(C);
  m->nedges = int(E);
  m->nvertices = int(V);
  m->nlayers = int(K);
  MeshView &mv = m->view;
  std::memset(&mv, 0, sizeof(mv));
  mv.ncells = int(C);
  mv.nedges = int(E);
  mv.nvertices = int(V);
  mv.nlayers = int(K);

  // ---- vertex tables
  std::vector<double> cvr(3 * V), kvh(3 * V), dcs(3 * V);
  for (long long v = 0; v < V; ++v) {
    const double inv_at = 1. / d->area_triangle[v];
    for (int j = 0; j < 3; ++j) {
      const int e = d->edges_on_vertex[3 * v + j];
      cvr[3 * v + j] = d->dc_edge[e] * inv_at * d->edge_sign_on_vertex[3 * v + j];
      kvh[3 * v + j] = d->kiteareas_on_vertex[3 * v + j] * inv_at;
      dcs[3 * v + j] = d->dc_edge[e] * d->edge_sign_on_vertex[3 * v + j];
    }
  }
  // ---- cell tables (padded to 6 slots)
  std::vector<int> ec(6 * C), nbc(6 * C);
  std::vector<double> ccd(6 * C), cke(6 * C), ckq(6 * C), ccdh(6 * C);
  for (long long c = 0; c < C; ++c) {
    const double inv_ac = 1. / d->area_cell[c];
    const int n = d->nedges_on_cell[c];
    for (int j = 0; j < MAXE; ++j) {
      if (j < n) {
        const int e = d->edges_on_cell[6 * c + j];
        const int c0 = d->cells_on_edge[2 * e], c1 = d->cells_on_edge[2 * e + 1];
        ec[6 * c + j] = e;
        nbc[6 * c + j] = c0 == c ? c1 : c0;
        ccd[6 * c + j] = inv_ac * d->dv_edge[e] * d->edge_sign_on_cell[6 * c + j];
        cke[6 * c + j] = inv_ac * (d->dv_edge[e] * d->dc_edge[e]) * 0.25;
        ckq[6 * c + j] = inv_ac * d->dv_edge[e] * (1. / d->dc_edge[e]);
        ccdh[6 * c + j] = -0.5 * ccd[6 * c + j];
      } else {
        ec[6 * c + j] = d->edges_on_cell[6 * c];
        nbc[6 * c + j] = int(c);
        ccd[6 * c + j] = cke[6 * c + j] = ckq[6 * c + j] = ccdh[6 * c + j] = 0.0;
      }
    }
  }
  // ---- edge tables
  std::vector<double> inv_dc(E), inv_dv(E), inv_dv4(E);
  int dv4_differs = 0, ne_max = 0;
  for (long long e = 0; e < E; ++e) {
    inv_dc[e] = 1. / d->dc_edge[e];
    inv_dv[e] = 1. / d->dv_edge[e];
    const double dvm = std::max(d->dv_edge[e], 0.25 * d->dc_edge[e]);
    inv_dv4[e] = 1. / dvm;
    dv4_differs |= inv_dv4[e] != inv_dv[e];
    int cnt = 0;
    for (int j = 0; j < d->nedges_on_edge[e]; ++j)
      cnt += d->weights_on_edge[12 * e + j] != 0.0;
    ne_max = std::max(ne_max, cnt);
  }
  const int NE = ne_max <= 8 ? 8 : 10;
  if (ne_max > 10)
    return swg_mesh_destroy(m),
           fail(SWG_ERR_ARG,
                "swg_mesh_create: more than 10 nonzero TRiSK weights per edge");
  std::vector<int> eoe(size_t(NE) * E);
  std::vector<double> woe(size_t(NE) * E);
  for (long long e = 0; e < E; ++e) {
    int s = 0;
    for (int j = 0; j < d->nedges_on_edge[e]; ++j) {
      const double w = d->weights_on_edge[12 * e + j];
      if (w != 0.0) {
        eoe[NE * e + s] = d->edges_on_edge[12 * e + j];
        woe[NE * e + s] = 0.25 * w;
        ++s;
      }
    }
    for (; s < NE; ++s) {
      eoe[NE * e + s] = int(e);
      woe[NE * e + s] = 0.0;
    }
  }
  m->scale2_h.assign(E, 1.0);
  m->scale4_h.assign(E, 1.0);
  if (d->mesh_scaling_del2)
    m->scale2_h.assign(d->mesh_scaling_del2, d->mesh_scaling_del2 + E);
  if (d->mesh_scaling_del4)
    m->scale4_h.assign(d->mesh_scaling_del4, d->mesh_scaling_del4 + E);
  m->scale2_uniform = E > 0;
  for (size_t e = 1; e < size_t(E) && m->scale2_uniform; ++e)
    m->scale2_uniform = m->scale2_h[e] == m->scale2_h[0];
  m->ckq_h = ckq;
  m->ec_h = ec;
  m->nec_h.assign(d->nedges_on_cell, d->nedges_on_cell + C);
  m->inv_dc_h = inv_dc;
  m->ev_h.assign(d->edges_on_vertex, d->edges_on_vertex + 3 * V);
  m->cv_h.assign(d->cells_on_vertex, d->cells_on_vertex + 3 * V);
  m->ce_h.assign(d->cells_on_edge, d->cells_on_edge + 2 * E);
  m->ve_h.assign(d->vertices_on_edge, d->vertices_on_edge + 2 * E);
  m->nbc_h = nbc;
  m->eoe_h = eoe;
  m->cvr_h = cvr;
  m->kvh_h = kvh;
  m->ccd_h = ccd;
  m->cke_h = cke;
  m->ccdh_h = ccdh;
  m->inv_dv_h = inv_dv;
  m->inv_dv4_h = inv_dv4;
  m->woe_h = woe;
  bool mask_ones = true;
  if (d->edge_mask)
    for (long long i = 0; i < E * K && mask_ones; ++i)
      mask_ones = d->edge_mask[i] == 1.0;

  int rc = SWG_OK;
  auto &A = m->allocs;
  if ((rc = upload(A, d->edges_on_vertex, 3 * V, &mv.ev)) ||
      (rc = upload(A, d->cells_on_vertex, 3 * V, &mv.cv)) ||
      (rc = upload(A, cvr.data(), 3 * V, &mv.cvr)) ||
      (rc = upload(A, kvh.data(), 3 * V, &mv.kvh)) ||
      (rc = upload(A, dcs.data(), 3 * V, &mv.dcs_v)) ||
      (rc = upload(A, ec.data(), 6 * C, &mv.ec)) ||
      (rc = upload(A, nbc.data(), 6 * C, &mv.nbc)) ||
      (rc = upload(A, ccd.data(), 6 * C, &mv.ccd)) ||
      (rc = upload(A, cke.data(), 6 * C, &mv.cke)) ||
      (rc = upload(A, ckq.data(), 6 * C, &mv.ckq)) ||
      (rc = upload(A, ccdh.data(), 6 * C, &mv.ccdh)) ||
      (rc = upload(A, d->cells_on_edge, 2 * E, &mv.ce)) ||
      (rc = upload(A, d->vertices_on_edge, 2 * E, &mv.ve)) ||
      (rc = upload(A, inv_dc.data(), E, &mv.inv_dc)) ||
      (rc = upload(A, inv_dv.data(), E, &mv.inv_dv)) ||
      (rc = upload(A, inv_dv4.data(), E, &mv.inv_dv4)) ||
      (rc = upload(A, eoe.data(), size_t(NE) * E, &mv.eoe)) ||
      (rc = upload(A, woe.data(), size_t(NE) * E, &mv.woe)) ||
      (rc = upload(A, m->scale2_h.data(), E, &mv.scale2)) ||
      (rc = upload(A, m->scale4_h.data(), E, &mv.scale4)) ||
      (rc = upload(A, d->area_cell, C, &mv.area_cell_d)) ||
      (rc = upload(A, d->area_triangle, V, &mv.area_tri_d)) ||
      (!mask_ones && (rc = upload(A, d->edge_mask, E * K, &mv.mask))) ||
      (!all_equal(d->max_level_cell, C, int(K)) &&
       (rc = upload(A, d->max_level_cell, C, &mv.maxlev_c))) ||
      (!all_equal(d->max_level_vertex_bot, V, int(K)) &&
       (rc = upload(A, d->max_level_vertex_bot, V, &mv.maxlev_v)))) {
    swg_mesh_destroy(m);
    return rc;
  }
  mv.ne = NE;
  mv.dv4_differs = dv4_differs;
  *out = m;
  return SWG_OK;
} SWG_ABI_CATCH("swg_mesh_create")

extern "C" int swg_mesh_destroy(swg_mesh m) try {
  if (!m)
    return SWG_OK;
  free_all(m->allocs);
  delete m;
  return SWG_OK;
} SWG_ABI_CATCH("swg_mesh_destroy")

// ----------------------------------------------------------------- state ---

static size_t state_words(swg_mesh m, int ntr) {
  return (size_t(m->ncells) + m->nedges + size_t(ntr) * m->ncells) * m->nlayers;
}

extern "C" int swg_state_create(swg_mesh m, int ntracers, swg_state *out) try {
  if (!m || !out || ntracers < 0)
    return fail(SWG_ERR_ARG, "swg_state_create: bad argument");
  *out = nullptr;
  swg_state s = new (std::nothrow) swg_state_s();
  if (!s)
    return fail(SWG_ERR_OOM, "swg_state_create: host allocation");
  static std::atomic<unsigned long long> next_serial{1};
  s->serial = next_serial++;
  s->mesh = m;
  s->ntracers = ntracers;
  const size_t n = state_words(m, ntracers);
  cudaError_t err = cudaMalloc(&s->block, n * sizeof(double));
  if (err != cudaSuccess) {
    delete s;
    return cuda_fail(err, "swg_state_create: cudaMalloc");
  }
  err = cudaMemset(s->block, 0, n * sizeof(double));
  if (err != cudaSuccess) {
    cudaFree(s->block);
    delete s;
    return cuda_fail(err, "swg_state_create: cudaMemset");
  }
  s->h = static_cast<double *>(s->block);
  s->vn = s->h + size_t(m->ncells) * m->nlayers;
  s->tr = s->vn + size_t(m->nedges) * m->nlayers;
  *out = s;
  return SWG_OK;
} SWG_ABI_CATCH("swg_state_create")

extern "C" int swg_state_destroy(swg_state s) try {
  if (!s)
    return SWG_OK;
  cudaFree(s->block);
  delete s;
  return SWG_OK;
} SWG_ABI_CATCH("swg_state_destroy")

extern "C" int swg_state_upload(swg_state s, const double *h, const double *vn,
                                const double *tr, void *stream) try {
  if (!s || !h || !vn || (s->ntracers > 0 && !tr))
    return fail(SWG_ERR_ARG, "swg_state_upload: NULL argument");
  const size_t K = s->mesh->nlayers;
  const size_t nh = s->mesh->ncells * K, nv = s->mesh->nedges * K,
               nt = size_t(s->ntracers) * nh;
  cudaStream_t st = as_stream(stream);
  cudaError_t err =
      cudaMemcpyAsync(s->h, h, nh * 8, cudaMemcpyHostToDevice, st);
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(s->vn, vn, nv * 8, cudaMemcpyHostToDevice, st);
  if (err == cudaSuccess && nt)
    err = cudaMemcpyAsync(s->tr, tr, nt * 8, cudaMemcpyHostToDevice, st);
  return err == cudaSuccess ? SWG_OK : cuda_fail(err, "swg_state_upload");
} SWG_ABI_CATCH("swg_state_upload")

extern "C" int swg_state_download(swg_state s, double *h, double *vn,
                                  double *tr, void *stream) try {
  if (!s)
    return fail(SWG_ERR_ARG, "swg_state_download: NULL state");
  const size_t K = s->mesh->nlayers;
  const size_t nh = s->mesh->ncells * K, nv = s->mesh->nedges * K,
               nt = size_t(s->ntracers) * nh;
  cudaStream_t st = as_stream(stream);
  cudaError_t err = cudaSuccess;
  if (h)
    err = cudaMemcpyAsync(h, s->h, nh * 8, cudaMemcpyDeviceToHost, st);
  if (err == cudaSuccess && vn)
    err = cudaMemcpyAsync(vn, s->vn, nv * 8, cudaMemcpyDeviceToHost, st);
  if (err == cudaSuccess && tr && nt)
    err = cudaMemcpyAsync(tr, s->tr, nt * 8, cudaMemcpyDeviceToHost, st);
  if (err == cudaSuccess)
    err = cudaStreamSynchronize(st);
  return err == cudaSuccess ? SWG_OK : cuda_fail(err, "swg_state_download");
} SWG_ABI_CATCH("swg_state_download")

extern "C" int swg_state_device_ptrs(swg_state s, double **h, double **vn,
                                     double **tr) try {
  if (!s)
    return fail(SWG_ERR_ARG, "swg_state_device_ptrs: NULL state");
  if (h)
    *h = s->h;
  if (vn)
    *vn = s->vn;
  if (tr)
    *tr = s->tr;
  return SWG_OK;
} SWG_ABI_CATCH("swg_state_device_ptrs")

extern "C" int swg_state_copy(swg_state dst, swg_state src, void *stream) try {
  if (!dst || !src || dst->mesh != src->mesh ||
      dst->ntracers != src->ntracers)
    return fail(SWG_ERR_ARG, "swg_state_copy: incompatible states");
  cudaError_t err = cudaMemcpyAsync(
      dst->block, src->block, state_words(dst->mesh, dst->ntracers) * 8,
      cudaMemcpyDeviceToDevice, as_stream(stream));
  return err == cudaSuccess ? SWG_OK : cuda_fail(err, "swg_state_copy");
} SWG_ABI_CATCH("swg_state_copy")

extern "C" int swg_state_fill(swg_state s, double value, void *stream) try {
  if (!s)
    return fail(SWG_ERR_ARG, "swg_state_fill: NULL state");
  const long long n = (long long)state_words(s->mesh, s->ntracers);
  launch_axpby(s->h, nullptr, nullptr, value, 0.0, n, 3, as_stream(stream));
  return check_launch("swg_state_fill");
} SWG_ABI_CATCH("swg_state_fill")

// ----------------------------------------------------------------- model ---

extern "C" int swg_model_create(swg_mesh mesh, const swg_params *p,
                                swg_model *out) try {
  return swg_model_create_ex(mesh, p, nullptr, out);
} SWG_ABI_CATCH("swg_model_create")

extern "C" int swg_linear_model_create(swg_mesh mesh, const swg_params *p,
                                       double h0, swg_model *out) try {
  swg_model_options o{};
  o.linear = 1;
  o.h0 = h0;
  return swg_model_create_ex(mesh, p, &o, out);
} SWG_ABI_CATCH("swg_linear_model_create")

extern "C" int swg_model_create_ex(swg_mesh mesh, const swg_params *p,
                                   const swg_model_options *opts,
                                   swg_model *out) try {
  if (!mesh || !p || !out || p->ntracers < 0)
    return fail(SWG_ERR_ARG, "swg_model_create: bad argument");
  *out = nullptr;
  const swg_model_options o = opts ? *opts : swg_model_options{};
  if (o.linear && (p->ntracers != 0 || !std::isfinite(o.h0)))
    return fail(SWG_ERR_ARG, "swg_model_create: the linear model takes no "
                             "tracers and a finite h0");
  if (o.apply_drag && !(p->drag_coeff >= 0))
    return fail(SWG_ERR_ARG, "swg_model_create: drag_coeff must be >= 0");
  swg_model md = new (std::nothrow) swg_model_s();
  if (!md)
    return fail(SWG_ERR_OOM, "swg_model_create: host allocation");
  md->mesh = mesh;
  md->params = *p;
  ModelView &pv = md->view;
  std::memset(&pv, 0, sizeof(pv));
  AuxView &a = md->aux;
  std::memset(&a, 0, sizeof(a));
  const size_t C = mesh->ncells, E = mesh->nedges, V = mesh->nvertices,
               K = mesh->nlayers, T = p->ntracers;
  // term enabling: shallow_water_model.cpp:17-35
  pv.grav = p->grav;
  pv.ntracers = p->ntracers;
  pv.vel_del2 = p->visc_del2 > 0;
  pv.vel_del4 = p->visc_del4 > 0;
  pv.tr_del2 = p->eddy_diff2 > 0;
  pv.tr_del4 = p->eddy_diff4 > 0;
  pv.do_h = !p->disable_h_tendency;
  pv.do_vn = !p->disable_vn_tendency;
  if (o.linear) { // shallow_water_hierarchical.cpp:676-740: no dissipation
    pv.linear = 1;
    pv.h0 = o.h0;
    pv.f4 = 4.0 * p->f0;
    pv.vel_del2 = pv.vel_del4 = pv.tr_del2 = pv.tr_del4 = 0;
  }
  pv.drag = !o.linear && o.apply_drag && p->drag_coeff > 0 && pv.do_vn;
  pv.drag_coeff = p->drag_coeff;
  pv.drag_level = int(K) - 1; // the lowest level

  std::vector<double> f(V, p->f0), c2(E), c4(E), kd2(6 * C), r4(6 * C),
      r4s(C), gidc(E), r4f, c4i(E), c4v(E);
  for (size_t e = 0; e < E; ++e) {
    gidc[e] = p->grav * mesh->inv_dc_h[e];
    c2[e] = p->visc_del2 * mesh->scale2_h[e];
    c4[e] = -(p->visc_del4 * mesh->scale4_h[e]);
    c4i[e] = c4[e] * mesh->inv_dc_h[e];
    c4v[e] = -(c4[e] * mesh->inv_dv_h[e]);
  }
  for (size_t c = 0; c < C; ++c) {
    double s = 0;
    for (int j = 0; j < MAXE; ++j) {
      const int e = mesh->ec_h[6 * c + j];
      kd2[6 * c + j] = p->eddy_diff2 * mesh->scale2_h[e] * mesh->ckq_h[6 * c + j];
      r4[6 * c + j] = -(p->eddy_diff4 * mesh->scale4_h[e] * mesh->ckq_h[6 * c + j]);
      s += r4[6 * c + j];
    }
    r4s[c] = s;
  }
  // the tracer del2 term folded into the del4 stencil (ModelView::r4f)
  if (mesh->scale2_uniform && T > 0 && pv.tr_del2 && pv.tr_del4) {
    const double k2 = p->eddy_diff2 * mesh->scale2_h[0];
    r4f.resize(C);
    for (size_t c = 0; c < C; ++c)
      r4f[c] = k2 - r4s[c];
  }
  auto &A = md->allocs;
  int rc = SWG_OK;
  if ((rc = upload(A, f.data(), V, &pv.f_vertex)) ||
      (rc = upload(A, gidc.data(), E, &pv.gidc)) ||
      (rc = upload(A, c2.data(), E, &pv.c2e)) ||
      (rc = upload(A, c4.data(), E, &pv.c4e)) ||
      (pv.vel_del4 && (rc = upload(A, c4i.data(), E, &pv.c4i))) ||
      (pv.vel_del4 && (rc = upload(A, c4v.data(), E, &pv.c4v))) ||
      (rc = upload(A, kd2.data(), 6 * C, &pv.kd2)) ||
      (rc = upload(A, r4.data(), 6 * C, &pv.r4)) ||
      (rc = upload(A, r4s.data(), C, &pv.r4sum)) ||
      (!r4f.empty() && (rc = upload(A, r4f.data(), C, &pv.r4f)))) {
    swg_model_destroy(md);
    return rc;
  }
  // work arrays: only what the enabled terms read
  const bool vn = pv.do_vn;
  const bool vdiss = vn && (pv.vel_del2 || pv.vel_del4);
  const bool v4 = vn && pv.vel_del4;
  struct Need {
    bool on;
    size_t n;
    double **p;
  } need[] = {
      {vn, V * K, &a.q},        {vdiss, V * K, &a.zeta},
      {v4, V * K, &a.z4},       {vdiss, C * K, &a.div},
      {vn, C * K, &a.ke},       {v4, C * K, &a.d4},
      {vn, E * K, &a.u2},
      {T > 0, T * C * K, &a.ntr},
      {T > 0 && pv.tr_del4, T * C * K, &a.lap},
      {true, E * K, &a.F},      {vn, E * K, &a.G},
      // the mean thickness is kept always: the per-field tendency calls
      // read the last auxiliary state's (the reference's m_mean_h_edge)
      {vn, E * K, &a.Q},        {true, E * K, &a.mh},
      {vdiss, E * K, &a.d2u},
      {v4 && mesh->view.dv4_differs, E * K, &a.d2u4},
  };
  for (auto &nd : need)
    if (!pv.linear && nd.on && (rc = dalloc(A, nd.n, nd.p))) {
      swg_model_destroy(md);
      return rc;
    }
  if (!a.d2u4)
    a.d2u4 = a.d2u;
  if ((rc = dalloc(A, 1024, &md->partials)) || (rc = fork_create(md->fork))) {
    swg_model_destroy(md);
    return rc;
  }
  *out = md;
  return SWG_OK;
} SWG_ABI_CATCH("swg_model_create_ex")

extern "C" int swg_model_destroy(swg_model md) try {
  if (!md)
    return SWG_OK;
  fork_destroy(md->fork);
  free_all(md->allocs);
  delete md;
  return SWG_OK;
} SWG_ABI_CATCH("swg_model_destroy")

// The reference's per-term m_enabled switches (shallow_water_model.hpp:19-29,
// read by compute_*_tendency in shallow_water_model.cpp:43-311).
static int *term_flag(swg_model md, int term, bool *off) {
  ModelView &p = md->view;
  *off = true;
  switch (term) {
  case SWG_TERM_THICKNESS_HADV: return &p.off_hadv;
  case SWG_TERM_PV_FLUX: return &p.off_pv;
  case SWG_TERM_KE_GRAD: return &p.off_ke;
  case SWG_TERM_SSH_GRAD: return &p.off_ssh;
  case SWG_TERM_TRACER_HADV: return &p.off_tr_hadv;
  default: break;
  }
  *off = false; // the dissipation terms: their enable flags
  switch (term) {
  case SWG_TERM_VEL_DIFF: return &p.vel_del2;
  case SWG_TERM_VEL_HYPERDIFF: return &p.vel_del4;
  case SWG_TERM_TRACER_DIFF: return &p.tr_del2;
  case SWG_TERM_TRACER_HYPERDIFF: return &p.tr_del4;
  default: return nullptr;
  }
}

// what swg_model_create enabled (shallow_water_model.cpp:17-35)
static bool created_on(swg_model md, int term) {
  const swg_params &q = md->params;
  switch (term) {
  case SWG_TERM_VEL_DIFF: return q.visc_del2 > 0;
  case SWG_TERM_VEL_HYPERDIFF: return q.visc_del4 > 0;
  case SWG_TERM_TRACER_DIFF: return q.eddy_diff2 > 0;
  case SWG_TERM_TRACER_HYPERDIFF: return q.eddy_diff4 > 0;
  default: return true;
  }
}

extern "C" int swg_model_set_term_enabled(swg_model md, int term,
                                          int enabled) try {
  if (!md)
    return fail(SWG_ERR_ARG, "swg_model_set_term_enabled: NULL model");
  if (md->view.linear)
    return fail(SWG_ERR_ARG, "swg_model_set_term_enabled: the linear model "
                             "has no switchable terms");
  bool off;
  int *f = term_flag(md, term, &off);
  if (!f)
    return fail(SWG_ERR_ARG, "swg_model_set_term_enabled: unknown term");
  if (enabled && !created_on(md, term))
    return fail(SWG_ERR_ARG, "swg_model_set_term_enabled: a dissipation term "
                             "whose coefficient is 0 has nothing to add");
  const int v = off ? !enabled : (enabled != 0);
  if (*f != v) {
    *f = v;
    ++md->version;
  }
  bool changed = false;
  for (int t = 0; t < SWG_NTERMS; ++t) {
    bool o;
    const int *g = term_flag(md, t, &o);
    changed |= (o ? *g != 0 : (*g != 0) != created_on(md, t));
  }
  md->terms_switched = changed;
  return SWG_OK;
} SWG_ABI_CATCH("swg_model_set_term_enabled")

extern "C" int swg_model_term_enabled(swg_model md, int term,
                                      int *enabled) try {
  bool off;
  int *f = md ? term_flag(md, term, &off) : nullptr;
  if (!f || !enabled)
    return fail(SWG_ERR_ARG, "swg_model_term_enabled: bad argument");
  *enabled = off ? !*f : *f != 0;
  return SWG_OK;
} SWG_ABI_CATCH("swg_model_term_enabled")

extern "C" int swg_model_set_forcing(swg_model md, swg_forcing_fn fn,
                                     void *user) try {
  if (!md)
    return fail(SWG_ERR_ARG, "swg_model_set_forcing: NULL model");
  md->forcing = fn;
  md->forcing_user = user;
  return SWG_OK;
} SWG_ABI_CATCH("swg_model_set_forcing")

extern "C" int swg_model_aux(swg_model md, const char *name,
                             const double **ptr, long long *count) try {
  if (!md || !name || !ptr || !count)
    return fail(SWG_ERR_ARG, "swg_model_aux: NULL argument");
  const long long C = md->mesh->ncells, E = md->mesh->nedges,
                  V = md->mesh->nvertices, K = md->mesh->nlayers,
                  T = md->params.ntracers;
  const AuxView &a = md->aux;
  struct {
    const char *n;
    const double *p;
    long long c;
  } tab[] = {
      {"q_vertex", a.q, V * K},
      {"rvort_vertex", a.zeta, V * K},
      {"vel_div_cell", a.div, C * K},
      {"ke_cell", a.ke, C * K},
      {"norm_tr_cell", a.ntr, T * C * K},
      {"thick_flux_edge", a.F, E * K},
      {"mean_h_edge", a.mh, E * K},
      {"pv_edge", a.Q, E * K},
      {"vel_del2_edge", a.d2u4, E * K},
      {"vel_del2_rvort_vertex", a.z4, V * K},
      {"vel_del2_div_cell", a.d4, C * K},
      {"tracer_del2_cell", a.lap, T * C * K},
      // the model's m_f_vertex (writable; read by every later evaluation)
      {"f_vertex", md->view.f_vertex, V},
  };
  for (auto &t : tab)
    if (std::strcmp(t.n, name) == 0) {
      if (!t.p)
        return fail(SWG_ERR_STATE,
                    std::string("swg_model_aux: '") + name +
                        "' is not computed by this configuration");
      *ptr = t.p;
      *count = t.c;
      return SWG_OK;
    }
  return fail(SWG_ERR_ARG, std::string("swg_model_aux: unknown field ") + name);
} SWG_ABI_CATCH("swg_model_aux")

namespace {

bool compatible(swg_model md, swg_state s) {
  return s && s->mesh == md->mesh && s->ntracers == md->params.ntracers;
}

StageArgs tendency_args(swg_state tend, swg_state state, int mode) {
  StageArgs s{};
  s.h = state->h;
  s.vn = state->vn;
  s.tr = state->tr;
  s.fh.tend = tend->h;
  s.fvn.tend = tend->vn;
  s.ftr.tend = tend->tr;
  s.ep.mode = mode;
  return s;
}

int run_tendency(swg_model md, const StageArgs &s, swg_state tend_for_hook,
                 const double *h, const double *vn, double t,
                 cudaStream_t st) {
  launch_tendency(md->mesh->view, md->view, md->aux, s, st, &md->fork);
  TRY(check_launch("tendency kernels"));
  if (md->forcing && tend_for_hook) {
    md->forcing(md->forcing_user, tend_for_hook->h, tend_for_hook->vn, h, vn,
                t, st);
    TRY(check_launch("additional_tendency hook"));
  }
  return SWG_OK;
}

} // namespace

extern "C" int swg_compute_tendency(swg_model md, swg_state tend,
                                    swg_state state, double t, int add_mode,
                                    void *stream) try {
  if (!md || !compatible(md, tend) || !compatible(md, state))
    return fail(SWG_ERR_ARG, "swg_compute_tendency: incompatible handles");
  if (add_mode != SWG_ADD_REPLACE && add_mode != SWG_ADD_INCREMENT)
    return fail(SWG_ERR_ARG, "swg_compute_tendency: bad add_mode");
  if (tend == state)
    return fail(SWG_ERR_ARG, "swg_compute_tendency: tend aliases state");
  const StageArgs s = tendency_args(
      tend, state, add_mode == SWG_ADD_REPLACE ? EPI_REPLACE : EPI_INCREMENT);
  return run_tendency(md, s, tend, state->h, state->vn, t, as_stream(stream));
} SWG_ABI_CATCH("swg_compute_tendency")

// ------------------------------------------- auxiliary state, per field ---
// The reference's model computes its auxiliary state (ShallowWaterAuxiliary-
// State::compute, shallow_water_auxstate.cpp:12-50) and then each field's
// tendency from it (compute_h_tendency / compute_vn_tendency /
// compute_tr_tendency, shallow_water_model.cpp:43-311).  These entry points
// expose the same split: the per-field calls read the intermediates of the
// last auxiliary computation (by swg_model_compute_aux or by any tendency
// evaluation or step on the model) together with their own h / vn
// arguments, as the reference's do.

extern "C" int swg_model_compute_aux(swg_model md, const double *h,
                                     const double *vn, const double *tr,
                                     void *stream) try {
  if (!md || !h || !vn || (md->params.ntracers > 0 && !tr))
    return fail(SWG_ERR_ARG, "swg_model_compute_aux: bad argument");
  if (md->view.linear)
    return fail(SWG_ERR_ARG, "swg_model_compute_aux: the linear model keeps "
                             "no auxiliary state");
  NvtxRange range("auxstate");
  launch_aux(md->mesh->view, md->view, md->aux, h, vn, tr, as_stream(stream),
             &md->fork);
  return check_launch("auxiliary state kernels");
} SWG_ABI_CATCH("swg_model_compute_aux")

static int field_tendency(swg_model md, int field, double *tend,
                          const double *h, const double *vn, int add_mode,
                          void *stream, const char *who) {
  // h is read by the velocity tendency only (the SSH gradient)
  if (!md || !tend || !vn || (field == 1 && !h))
    return fail(SWG_ERR_ARG, std::string(who) + ": bad argument");
  if (add_mode != SWG_ADD_REPLACE && add_mode != SWG_ADD_INCREMENT)
    return fail(SWG_ERR_ARG, std::string(who) + ": bad add_mode");
  if (field == 2 && md->view.linear)
    return fail(SWG_ERR_ARG, std::string(who) + ": the linear model has no "
                                                "tracers");
  if (field == 1 && !md->view.do_vn && !md->view.linear)
    return fail(SWG_ERR_STATE, std::string(who) +
                                   ": the model was created with the "
                                   "velocity tendency disabled, so it keeps "
                                   "no velocity intermediates");
  if (field == 2 && md->params.ntracers == 0)
    return SWG_OK; // no tracers: nothing to compute
  launch_field_tendency(md->mesh->view, md->view, md->aux, field, h, vn, tend,
                        add_mode == SWG_ADD_REPLACE ? EPI_REPLACE
                                                    : EPI_INCREMENT,
                        as_stream(stream));
  return check_launch(who);
}

extern "C" int swg_compute_h_tendency(swg_model md, double *h_tend,
                                      const double *h, const double *vn,
                                      int add_mode, void *stream) try {
  return field_tendency(md, 0, h_tend, h, vn, add_mode, stream,
                        "swg_compute_h_tendency");
} SWG_ABI_CATCH("swg_compute_h_tendency")

extern "C" int swg_compute_vn_tendency(swg_model md, double *vn_tend,
                                       const double *h, const double *vn,
                                       int add_mode, void *stream) try {
  return field_tendency(md, 1, vn_tend, h, vn, add_mode, stream,
                        "swg_compute_vn_tendency");
} SWG_ABI_CATCH("swg_compute_vn_tendency")

extern "C" int swg_compute_tr_tendency(swg_model md, double *tr_tend,
                                       const double *tr, const double *vn,
                                       int add_mode, void *stream) try {
  (void)tr; // the reference reads the normalised tracers of the aux state
  return field_tendency(md, 2, tr_tend, nullptr, vn, add_mode, stream,
                        "swg_compute_tr_tendency");
} SWG_ABI_CATCH("swg_compute_tr_tendency")

// -------------------------------------------------------------- steppers ---

extern "C" int swg_stepper_create(swg_model md, int kind, int nstages,
                                  swg_stepper *out) try {
  if (!md || !out)
    return fail(SWG_ERR_ARG, "swg_stepper_create: NULL argument");
  *out = nullptr;
  if (kind != SWG_STEPPER_RK4 && kind != SWG_STEPPER_LSRK)
    return fail(SWG_ERR_ARG, "swg_stepper_create: unknown kind");
  if (kind == SWG_STEPPER_LSRK && nstages != 5 && nstages != 1)
    return fail(SWG_ERR_ARG, "swg_stepper_create: LSRK supports 5 or 1 stages");
  swg_stepper sp = new (std::nothrow) swg_stepper_s();
  if (!sp)
    return fail(SWG_ERR_OOM, "swg_stepper_create: host allocation");
  sp->model = md;
  sp->kind = kind;
  if (kind == SWG_STEPPER_RK4) {
    // rk4.cpp:14-25
    sp->nstages = 4;
    sp->rka = {1. / 2, 1. / 2, 1};
    sp->rkb = {1. / 6, 1. / 3, 1. / 3, 1. / 6};
    sp->rkc = {1. / 2, 1. / 2, 1};
  } else if (nstages == 5) {
    // Carpenter-Kennedy 5-stage low-storage RK, lsrk.cpp:16-28
    sp->nstages = 5;
    sp->rka = {0., -567301805773. / 1357537059087.,
               -2404267990393. / 2016746695238.,
               -3550918686646. / 2091501179385.,
               -1275806237668. / 842570457699.};
    sp->rkb = {1432997174477. / 9575080441755.,
               5161836677717. / 13612068292357.,
               1720146321549. / 2090206949498.,
               3134564353537. / 4481467310338.,
               2277821191437. / 14882151754819.};
    sp->rkc = {0., 1432997174477. / 9575080441755.,
               2526269341429. / 6820363962896.,
               2006345519317. / 3224310063776.,
               2802321613138. / 2924317926251.};
  } else {
    sp->nstages = 1; // lsrk.cpp:29-33
    sp->rka = {0};
    sp->rkb = {1};
    sp->rkc = {0};
  }
  const int T = md->params.ntracers;
  int rc = swg_state_create(md->mesh, T, &sp->tend);
  if (rc == SWG_OK && kind == SWG_STEPPER_RK4) {
    if ((rc = swg_state_create(md->mesh, T, &sp->acc)) == SWG_OK &&
        (rc = swg_state_create(md->mesh, T, &sp->p0)) == SWG_OK)
      rc = swg_state_create(md->mesh, T, &sp->p1);
  }
  if (rc != SWG_OK) {
    swg_stepper_destroy(sp);
    return rc;
  }
  *out = sp;
  return SWG_OK;
} SWG_ABI_CATCH("swg_stepper_create")

extern "C" int swg_stepper_destroy(swg_stepper sp) try {
  if (!sp)
    return SWG_OK;
  if (sp->graph)
    cudaGraphExecDestroy(sp->graph);
  swg_state_destroy(sp->tend);
  swg_state_destroy(sp->acc);
  swg_state_destroy(sp->p0);
  swg_state_destroy(sp->p1);
  swg_state_destroy(sp->old);
  delete sp;
  return SWG_OK;
} SWG_ABI_CATCH("swg_stepper_destroy")

namespace {

// One fused step (no forcing hook): the stage update runs in the epilogue of
// the last two tendency kernels.
int fused_step(swg_stepper sp, swg_state S, double dt, cudaStream_t st) {
  swg_model md = sp->model;
  const ModelView &pv = md->view;
  if (sp->kind == SWG_STEPPER_LSRK) {
    for (int stage = 0; stage < sp->nstages; ++stage) {
      StageArgs a{};
      a.h = S->h;
      a.vn = S->vn;
      a.tr = S->tr;
      a.fh = {sp->tend->h, nullptr, nullptr, S->h};
      a.fvn = {sp->tend->vn, nullptr, nullptr, S->vn};
      a.ftr = {sp->tend->tr, nullptr, nullptr, S->tr};
      a.ep = {EPI_LSRK, sp->rka[stage], dt * sp->rkb[stage], 0.0};
      launch_tendency(md->mesh->view, pv, md->aux, a, st, &md->fork);
    }
    return check_launch("LSRK step");
  }
  // RK4 with rotating buffers: S -> (A, P0) -> (A, P1) -> (A, P0) -> S.
  swg_state P[2] = {sp->p0, sp->p1};
  swg_state in = S;
  for (int stage = 0; stage < 4; ++stage) {
    StageArgs a{};
    // a field whose tendency is disabled keeps its start-of-step value
    a.h = pv.do_h ? in->h : S->h;
    a.vn = pv.do_vn ? in->vn : S->vn;
    a.tr = in->tr;
    swg_state outp = stage < 3 ? P[stage % 2] : S;
    a.fh = {nullptr, S->h, sp->acc->h, outp->h};
    a.fvn = {nullptr, S->vn, sp->acc->vn, outp->vn};
    a.ftr = {nullptr, S->tr, sp->acc->tr, outp->tr};
    const int mode =
        stage == 0 ? EPI_RK4_FIRST : (stage < 3 ? EPI_RK4_MID : EPI_RK4_LAST);
    a.ep = {mode, 0.0, dt * sp->rkb[stage],
            stage < 3 ? dt * sp->rka[stage] : 0.0};
    launch_tendency(md->mesh->view, pv, md->aux, a, st, &md->fork);
    in = outp;
  }
  return check_launch("RK4 step");
}

// Unfused step with the forcing hook, the reference's exact sequence
// (lsrk.cpp:36-89, rk4.cpp:28-104).
int hooked_step(swg_stepper sp, swg_state S, double t, double dt,
                cudaStream_t st) {
  swg_model md = sp->model;
  const long long K = md->mesh->nlayers;
  const long long nh = md->mesh->ncells * K, nv = md->mesh->nedges * K,
                  nt = (long long)md->params.ntracers * nh;
  swg_state Tn = sp->tend;
  auto axpy3 = [&](swg_state y, swg_state x, swg_state z, double a, int kind) {
    launch_axpby(y->h, x ? x->h : nullptr, z ? z->h : nullptr, a, 0, nh, kind, st);
    launch_axpby(y->vn, x ? x->vn : nullptr, z ? z->vn : nullptr, a, 0, nv, kind, st);
    if (nt)
      launch_axpby(y->tr, x ? x->tr : nullptr, z ? z->tr : nullptr, a, 0, nt,
                   kind, st);
  };
  if (sp->kind == SWG_STEPPER_LSRK) {
    for (int stage = 0; stage < sp->nstages; ++stage) {
      axpy3(Tn, nullptr, nullptr, sp->rka[stage], 0);
      StageArgs a = tendency_args(Tn, S, EPI_INCREMENT);
      TRY(run_tendency(md, a, Tn, S->h, S->vn, t + sp->rkc[stage] * dt, st));
      axpy3(S, Tn, nullptr, dt * sp->rkb[stage], 1);
    }
    return check_launch("LSRK step (hooked)");
  }
  if (!sp->old)
    TRY(swg_state_create(md->mesh, md->params.ntracers, &sp->old));
  swg_state O = sp->old, P = sp->p0;
  TRY(swg_state_copy(O, S, st));
  StageArgs a0 = tendency_args(Tn, S, EPI_REPLACE);
  TRY(run_tendency(md, a0, Tn, S->h, S->vn, t, st));
  for (int stage = 0; stage < 4; ++stage) {
    axpy3(S, Tn, nullptr, dt * sp->rkb[stage], 1);
    if (stage < 3) {
      axpy3(P, Tn, O, dt * sp->rka[stage], 2);
      StageArgs a = tendency_args(Tn, P, EPI_REPLACE);
      TRY(run_tendency(md, a, Tn, P->h, P->vn, t + sp->rkc[stage] * dt, st));
    }
  }
  return check_launch("RK4 step (hooked)");
}

} // namespace

extern "C" int swg_step(swg_stepper sp, swg_state S, double t0, double dt,
                        int nsteps, int use_graph, void *stream) try {
  if (!sp || !compatible(sp->model, S) || nsteps < 0)
    return fail(SWG_ERR_ARG, "swg_step: bad argument");
  NvtxRange range("time_integration");
  cudaStream_t st = as_stream(stream);
  if (sp->model->forcing) {
    for (int s = 0; s < nsteps; ++s)
      TRY(hooked_step(sp, S, t0 + s * dt, dt, st));
    return SWG_OK;
  }
  if (!use_graph || profiling_enabled()) {
    for (int s = 0; s < nsteps; ++s)
      TRY(fused_step(sp, S, dt, st));
    return SWG_OK;
  }
  if (!sp->graph || sp->graph_serial != S->serial || sp->graph_dt != dt ||
      sp->graph_version != sp->model->version) {
    if (sp->graph) {
      cudaGraphExecDestroy(sp->graph);
      sp->graph = nullptr;
    }
    cudaStream_t cs;
    cudaError_t err = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (err != cudaSuccess)
      return cuda_fail(err, "swg_step: capture stream");
    const long long before = g_launches.load();
    err = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int rc = SWG_OK;
    if (err == cudaSuccess)
      rc = fused_step(sp, S, dt, cs);
    cudaGraph_t g = nullptr;
    cudaError_t err2 = cudaStreamEndCapture(cs, &g);
    sp->graph_launches = g_launches.load() - before;
    g_launches -= sp->graph_launches; // captured, not launched
    cudaStreamDestroy(cs);
    if (err != cudaSuccess || err2 != cudaSuccess || rc != SWG_OK) {
      if (g)
        cudaGraphDestroy(g);
      return rc != SWG_OK ? rc
                          : cuda_fail(err != cudaSuccess ? err : err2,
                                      "swg_step: graph capture");
    }
    err = cudaGraphInstantiate(&sp->graph, g, 0);
    cudaGraphDestroy(g);
    if (err != cudaSuccess) {
      sp->graph = nullptr;
      return cuda_fail(err, "swg_step: graph instantiate");
    }
    sp->graph_serial = S->serial;
    sp->graph_version = sp->model->version;
    sp->graph_dt = dt;
  }
  for (int s = 0; s < nsteps; ++s) {
    cudaError_t err = cudaGraphLaunch(sp->graph, st);
    if (err != cudaSuccess)
      return cuda_fail(err, "swg_step: graph launch");
    g_launches += sp->graph_launches;
  }
  return SWG_OK;
} SWG_ABI_CATCH("swg_step")

// ----------------------------------------------------------- diagnostics ---

static int diag(int which, swg_model md, swg_state s, double *out,
                void *stream) {
  if (!md || !compatible(md, s) || !out)
    return fail(SWG_ERR_ARG, "swg_diag: bad argument");
  return reduce_diag(which, md->mesh->view, md->view, s->h, s->vn,
                     md->partials, 1024, out, as_stream(stream));
}

extern "C" int swg_diag_mass(swg_model md, swg_state s, double *out,
                             void *stream) try {
  return diag(0, md, s, out, stream);
} SWG_ABI_CATCH("swg_diag_mass")
extern "C" int swg_diag_energy(swg_model md, swg_state s, double *out,
                               void *stream) try {
  return diag(1, md, s, out, stream);
} SWG_ABI_CATCH("swg_diag_energy")
extern "C" int swg_diag_circulation(swg_model md, swg_state s, double *out,
                                    void *stream) try {
  return diag(2, md, s, out, stream);
} SWG_ABI_CATCH("swg_diag_circulation")

extern "C" int swg_profile_enable(int on) try {
  return profile_enable(on);
} SWG_ABI_CATCH("swg_profile_enable")

extern "C" int swg_profile_read(int max_kernels, char *names,
                                double *total_ms, long long *launches,
                                int *count) try {
  return profile_read(max_kernels, names, total_ms, launches, count);
} SWG_ABI_CATCH("swg_profile_read")

extern "C" int swg_sync(void *stream) try {
  cudaError_t err = cudaStreamSynchronize(as_stream(stream));
  if (err == cudaSuccess)
    err = cudaGetLastError();
  return err == cudaSuccess ? SWG_OK : cuda_fail(err, "swg_sync");
} SWG_ABI_CATCH("swg_sync")
