// gfe_host.cpp -- host-side set-up of libgfe: errors, device buffers, Cartesian model
// arrays, face labels, CLagrangian dof numbering and quadrature tables.
//
// This is the part of Gridap's FE-space construction that fixes the sparsity pattern
// (dof numbering runs once per mesh on the host); it produces exactly the arrays Gridap
// hands across the boundary, so callers without Gridap get identical numbering.
#include <cmath>
#include <cstring>

#include "gfe_internal.h"

namespace gfe {

// ---- errors -------------------------------------------------------------------------------
static thread_local std::string g_last_error;

int set_error(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

void clear_error() { g_last_error.clear(); }

const char* g_last_error_ptr() { return g_last_error.c_str(); }

// ---- device buffers -----------------------------------------------------------------------
DevBuf::~DevBuf() { release(); }

void DevBuf::release() {
  if (ptr) {
    if (owner && owner->pool)
      cudaFreeAsync(ptr, owner->stream);
    else
      cudaFree(ptr);
  }
  ptr = nullptr;
  bytes = 0;
}

int DevBuf::reserve(size_t nbytes) {
  if (nbytes <= bytes && ptr) return GFE_OK;
  release();
  size_t n = nbytes < 256 ? 256 : nbytes;
  cudaError_t e = (owner && owner->pool)
                      ? cudaMallocFromPoolAsync(&ptr, n, owner->pool, owner->stream)
                      : cudaMalloc(&ptr, n);
  if (e != cudaSuccess) {
    ptr = nullptr;
    (void)cudaGetLastError();
    return set_error(GFE_ERR_OUT_OF_MEMORY, "cudaMalloc(%zu bytes) failed: %s", n,
                     cudaGetErrorString(e));
  }
  bytes = n;
  return GFE_OK;
}

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int device_view(gfe_ctx* ctx, const void* p, size_t n, int slot, const void** out) {
  if (!p || n == 0) {
    *out = p;
    return GFE_OK;
  }
  if (is_device_ptr(p)) {
    *out = p;
    return GFE_OK;
  }
  GFE_TRY(ctx->scratch[slot].reserve(n));
  GFE_CUDA_TRY(cudaMemcpyAsync(ctx->scratch[slot].ptr, p, n, cudaMemcpyHostToDevice,
                               ctx->stream));
  *out = ctx->scratch[slot].ptr;
  return GFE_OK;
}

int copy_out(gfe_ctx* ctx, void* dst, const void* src, size_t n) {
  if (n == 0) return GFE_OK;
  GFE_CUDA_TRY(cudaMemcpyAsync(dst, src, n, cudaMemcpyDefault, ctx->stream));
  if (!is_device_ptr(dst)) GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return GFE_OK;
}

int ensure_values(gfe_ctx* ctx, gfe_matrix* A) {
  if (!A || !A->val_pending) return GFE_OK;
  if (A->nnz > 0)
    GFE_CUDA_TRY(cudaMemsetAsync(A->val.ptr, 0, sizeof(double) * (size_t)A->nnz, ctx->stream));
  A->val_pending = false;
  A->zf_values = false;
  return GFE_OK;
}

// the error of a device error word read on the host (resets the device word when set)
static int report_device_error(gfe_ctx* ctx, const DevError& h, const char* where) {
  if (h.code == GFE_OK) return GFE_OK;
  GFE_CUDA_TRY(cudaMemsetAsync(ctx->d_err, 0, sizeof(DevError), ctx->stream));
  const char* what = "device error";
  switch (h.code) {
    case GFE_ERR_DEGENERATE_CELL: what = "degenerate cell (det J <= 0 or not finite)"; break;
    case GFE_ERR_ROW_TOO_WIDE: what = "matrix row wider than supported"; break;
    case GFE_ERR_INVALID_ARGUMENT: what = "id out of range"; break;
    case GFE_ERR_NONFINITE: what = "non-finite value"; break;
    case GFE_ERR_TIMEOUT: what = "bounded wait ran out"; break;
    default: break;
  }
  return set_error(h.code, "%s: %s at index %lld", where, what, h.index);
}

int check_device_error(gfe_ctx* ctx, const char* where) {
  ctx->err_staged = false;
  DevError h;
  GFE_CUDA_TRY(cudaMemcpyAsync(&h, ctx->d_err, sizeof(DevError), cudaMemcpyDeviceToHost,
                               ctx->stream));
  GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return report_device_error(ctx, h, where);
}

int stage_device_error(gfe_ctx* ctx) {
  GFE_CUDA_TRY(cudaMemcpyAsync(static_cast<char*>(ctx->h_pinned) + kStagedErrorOffset,
                               ctx->d_err, sizeof(DevError), cudaMemcpyDeviceToHost,
                               ctx->stream));
  ctx->err_staged = true;
  return GFE_OK;
}

int check_staged_error(gfe_ctx* ctx, const char* where) {
  if (!ctx->err_staged) return check_device_error(ctx, where);
  ctx->err_staged = false;
  DevError h;
  std::memcpy(&h, static_cast<const char*>(ctx->h_pinned) + kStagedErrorOffset, sizeof(h));
  return report_device_error(ctx, h, where);
}

// ---- kernel timing ------------------------------------------------------------------------
void timer_begin(gfe_ctx* ctx, int kind) {
  KernelTimer& t = ctx->timer;
  if (!t.enabled) return;
  while (t.pool.size() < t.used + 2) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) {
      (void)cudaGetLastError();
      return;
    }
    t.pool.push_back(e);
  }
  t.kinds.push_back(kind);
  cudaEventRecord(t.pool[t.used++], ctx->stream);
}

void timer_end(gfe_ctx* ctx) {
  KernelTimer& t = ctx->timer;
  if (!t.enabled || t.used % 2 == 0) return;
  cudaEventRecord(t.pool[t.used++], ctx->stream);
}

void timer_drop_last(gfe_ctx* ctx, int n) {
  KernelTimer& t = ctx->timer;
  while (n-- > 0 && t.used >= 2) {
    t.used -= 2;
    t.kinds.pop_back();
  }
}

int timer_flush(gfe_ctx* ctx) {
  KernelTimer& t = ctx->timer;
  if (t.used == 0) return GFE_OK;
  GFE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  for (size_t i = 0; i + 1 < t.used; i += 2) {
    float ms = 0.f;
    GFE_CUDA_TRY(cudaEventElapsedTime(&ms, t.pool[i], t.pool[i + 1]));
    const int k = t.kinds[i / 2];
    t.total_ms[k] += ms;
    t.count[k] += 1;
  }
  t.used = 0;
  t.kinds.clear();
  return GFE_OK;
}

void timer_release(gfe_ctx* ctx) {
  for (auto e : ctx->timer.pool) cudaEventDestroy(e);
  ctx->timer.pool.clear();
  ctx->timer.used = 0;
}

// ---- quadrature ---------------------------------------------------------------------------
// Gauss-Legendre rule with n points: Newton's method on the Legendre three-term recurrence
// from the Tricomi initial guesses; nodes/weights mapped from [-1,1] to [0,1]. Tensor
// product over dimensions, first coordinate fastest, weight = product of 1-D weights.
static void gauss01(int n, double* x, double* w) {
  // extended precision for the iteration and the weight formula, rounded at the end
  typedef long double R;
  const R pi = 3.141592653589793238462643383279502884L;
  auto legendre = [n](R t, R* pn, R* pn1) {
    R pm = 1.0L, pc = t;
    for (int k = 1; k < n; ++k) {
      const R pk = ((2 * k + 1) * t * pc - k * pm) / (k + 1);
      pm = pc;
      pc = pk;
    }
    *pn = pc;
    *pn1 = pm;
  };
  for (int i = 1; i <= n; ++i) {
    R t = std::cos(pi * (4.0L * i - 1.0L) / (4.0L * n + 2.0L));
    for (int it = 0; it < 64; ++it) {
      R pn, pn1;
      legendre(t, &pn, &pn1);
      const R dpn = (n == 1) ? 1.0L : n * (pn1 - t * pn) / (1.0L - t * t);
      const R step = pn / dpn;
      t -= step;
      if (std::fabs(step) <= 1e-30L) break;
    }
    R pn, pn1;
    legendre(t, &pn, &pn1);
    const R dpn = (n == 1) ? 1.0L : n * (pn1 - t * pn) / (1.0L - t * t);
    const int j = n - i;  // ascending order
    x[j] = (double)(0.5L * (t + 1.0L));
    w[j] = (double)(1.0L / ((1.0L - t * t) * dpn * dpn));
  }
}

// Q1 shape values phi[q][a] and reference gradients dphi[q][a][k] at the points qx[q][D];
// vertex a has coordinate bit d = (a >> d) & 1.
void q1_shapes(int D, int nq, const double* qx, std::vector<double>& phi,
                      std::vector<double>& dphi) {
  const int nv = 1 << D;
  phi.assign((size_t)nq * nv, 0.0);
  dphi.assign((size_t)nq * nv * D, 0.0);
  for (int q = 0; q < nq; ++q)
    for (int a = 0; a < nv; ++a) {
      double f[3], g[3];
      for (int d = 0; d < D; ++d) {
        const bool hi = (a >> d) & 1;
        f[d] = hi ? qx[q * D + d] : 1.0 - qx[q * D + d];
        g[d] = hi ? 1.0 : -1.0;
      }
      double v = 1.0;
      for (int d = 0; d < D; ++d) v *= f[d];
      phi[(size_t)q * nv + a] = v;
      for (int k = 0; k < D; ++k) {
        double dv = 1.0;
        for (int d = 0; d < D; ++d) dv *= (d == k) ? g[d] : f[d];
        dphi[((size_t)q * nv + a) * D + k] = dv;
      }
    }
}

int tensor_quadrature(int D, int degree, std::vector<double>& x, std::vector<double>& w) {
  if (D < 1 || D > 3 || degree < 0 || degree > 60)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "quadrature: bad dim %d / degree %d", D, degree);
  int n = degree / 2 + 1;
  double x1[32], w1[32];
  gauss01(n, x1, w1);
  int np = 1;
  for (int d = 0; d < D; ++d) np *= n;
  x.assign((size_t)np * D, 0.0);
  w.assign(np, 1.0);
  for (int k = 0; k < np; ++k) {
    int r = k;
    for (int d = 0; d < D; ++d) {
      int i = r % n;
      r /= n;
      x[(size_t)k * D + d] = x1[i];
      w[k] *= w1[i];
    }
  }
  return GFE_OK;
}

}  // namespace gfe

using namespace gfe;

// ---- Cartesian model ----------------------------------------------------------------------
// Entity id of a point of the box [0,1]^D lying in the interior of the face with extrusion
// mask `e` (bit d set = the face spans direction d) and anchor mask `a` (bit d set = on the
// upper side of direction d). Faces are ranked by dimension, then by extrusion mask, then by
// anchor mask compressed to the non-extruded directions -- Gridap's n-cube face order
// (ReferenceFEs/ExtrusionPolytopes.jl:460-481).
static int32_t box_entity(int D, unsigned e, unsigned a) {
  int k = __builtin_popcount(e);
  static const int binom[4][4] = {{1, 0, 0, 0}, {1, 1, 0, 0}, {1, 2, 1, 0}, {1, 3, 3, 1}};
  int id = 0;
  for (int j = 0; j < k; ++j) id += binom[D][j] << (D - j);  // faces of lower dimension
  int rank_e = 0;
  for (unsigned m = 0; m < e; ++m)
    if (__builtin_popcount(m) == k) ++rank_e;
  int rank_a = 0, bit = 0;
  for (int d = 0; d < D; ++d) {
    if (e & (1u << d)) continue;
    if (a & (1u << d)) rank_a |= 1 << bit;
    ++bit;
  }
  return 1 + id + rank_e * (1 << (D - k)) + rank_a;
}

extern "C" int gfe_cartesian_model(int dim, const int64_t* partition, const double* domain,
                                   double* node_coords, int32_t* cell_node_ids,
                                   int32_t* node_entity) {
  clear_error();
  if (dim < 1 || dim > 3 || !partition)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_cartesian_model: bad dim or partition");
  int64_t n[3] = {1, 1, 1}, np[3] = {1, 1, 1};
  double x0[3] = {0, 0, 0}, h[3] = {1, 1, 1};
  for (int d = 0; d < dim; ++d) {
    if (partition[d] < 1)
      return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_cartesian_model: partition[%d] < 1", d);
    n[d] = partition[d];
    np[d] = n[d] + 1;
    if (domain) {
      x0[d] = domain[2 * d];
      h[d] = (domain[2 * d + 1] - domain[2 * d]) / (double)n[d];
    }
  }
  const int64_t nnodes = np[0] * np[1] * np[2];
  if (node_coords || node_entity) {
    for (int64_t id = 0; id < nnodes; ++id) {
      int64_t I[3] = {id % np[0], (id / np[0]) % np[1], id / (np[0] * np[1])};
      unsigned e = 0, a = 0;
      for (int d = 0; d < dim; ++d) {
        if (node_coords) node_coords[id * dim + d] = x0[d] + (double)I[d] * h[d];
        if (I[d] != 0 && I[d] != n[d]) e |= 1u << d;
        if (I[d] == n[d]) a |= 1u << d;
      }
      if (node_entity) node_entity[id] = box_entity(dim, e, a);
    }
  }
  if (cell_node_ids) {
    const int nv = 1 << dim;
    const int64_t ncells = n[0] * n[1] * n[2];
    for (int64_t c = 0; c < ncells; ++c) {
      int64_t i = c % n[0], j = (c / n[0]) % n[1], k = c / (n[0] * n[1]);
      int64_t base = i + np[0] * (j + np[1] * k);
      for (int l = 0; l < nv; ++l) {
        int64_t off = (l & 1) + ((l >> 1) & 1) * np[0] + ((l >> 2) & 1) * np[0] * np[1];
        cell_node_ids[c * nv + l] = (int32_t)(base + off + 1);
      }
    }
  }
  return GFE_OK;
}

extern "C" int gfe_clagrangian_dofs(int64_t nnodes, const int8_t* node_to_tag, int ncomp,
                                    const uint8_t* tag_masks, int64_t ncells, int nv,
                                    const int32_t* cell_node_ids,
                                    const int32_t* lnode_comp_to_ldof,
                                    int32_t* node_comp_to_dof, int32_t* cell_dof_ids,
                                    int32_t* nfree, int32_t* ndiri) {
  clear_error();
  if (nnodes < 0 || ncomp < 1 || !node_to_tag || !node_comp_to_dof || !nfree || !ndiri)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_clagrangian_dofs: bad arguments");
  int64_t f = 0, g = 0;
  for (int64_t node = 0; node < nnodes; ++node) {
    const int tag = node_to_tag[node];
    for (int c = 0; c < ncomp; ++c) {
      const bool diri = tag > 0 && tag_masks && tag_masks[(size_t)(tag - 1) * ncomp + c];
      node_comp_to_dof[node * ncomp + c] = diri ? (int32_t)-(++g) : (int32_t)(++f);
    }
  }
  if (f > INT32_MAX || g > INT32_MAX)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_clagrangian_dofs: too many dofs");
  *nfree = (int32_t)f;
  *ndiri = (int32_t)g;
  if (cell_dof_ids && cell_node_ids) {
    const int ndc = nv * ncomp;
    for (int64_t cell = 0; cell < ncells; ++cell)
      for (int l = 0; l < nv; ++l) {
        const int64_t node = cell_node_ids[cell * nv + l] - 1;
        if (node < 0 || node >= nnodes)
          return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_clagrangian_dofs: node id %lld",
                           (long long)(node + 1));
        for (int c = 0; c < ncomp; ++c) {
          const int ld = lnode_comp_to_ldof ? lnode_comp_to_ldof[l * ncomp + c]
                                            : c * nv + l + 1;  // component-major local
          cell_dof_ids[cell * ndc + ld - 1] = node_comp_to_dof[node * ncomp + c];
        }
      }
  }
  return GFE_OK;
}

// ---- conforming Q2 numbering on Cartesian grids -------------------------------------------
// Faces of the D-cube in Gridap's order: by dimension, extrusion mask, anchor mask.
static int ncube_faces(int D, unsigned* ext, unsigned* anc) {
  int n = 0;
  for (int k = 0; k <= D; ++k)
    for (unsigned e = 0; e < (1u << D); ++e) {
      if (__builtin_popcount(e) != k) continue;
      // anchors over the non-extruded directions, ascending as a compressed mask
      const int free_dims = D - k;
      for (unsigned m = 0; m < (1u << free_dims); ++m) {
        unsigned a = 0;
        int bit = 0;
        for (int d = 0; d < D; ++d) {
          if (e & (1u << d)) continue;
          if (m & (1u << bit)) a |= 1u << d;
          ++bit;
        }
        ext[n] = e;
        anc[n] = a;
        ++n;
      }
    }
  return n;
}

extern "C" int gfe_cartesian_conforming_dofs(int dim, int order, const int64_t* partition,
                                             int ncomp, const int8_t* entity_to_tag,
                                             const uint8_t* tag_masks, int32_t* cell_dof_ids,
                                             int32_t* nfree, int32_t* ndiri) {
  clear_error();
  if (dim < 2 || dim > 3 || order != 2 || !partition || ncomp < 1 || !entity_to_tag ||
      !cell_dof_ids || !nfree || !ndiri)
    return set_error(GFE_ERR_INVALID_ARGUMENT,
                     "gfe_cartesian_conforming_dofs: dim 2/3, order 2 and outputs required");
  int64_t n[3] = {1, 1, 1}, np[3] = {1, 1, 1};
  for (int d = 0; d < dim; ++d) {
    if (partition[d] < 1)
      return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_cartesian_conforming_dofs: partition");
    n[d] = partition[d];
    np[d] = n[d] + 1;
  }
  unsigned fe[27], fa[27];
  const int nlf = ncube_faces(dim, fe, fa);
  const int64_t nlat = np[0] * np[1] * np[2];
  const int64_t ncells = n[0] * n[1] * n[2];
  // first-touch ids of the faces of dimension 1..D-1, keyed by (extrusion mask, lattice pos)
  std::vector<int32_t> id((size_t)(1u << dim) * nlat, 0);
  std::vector<std::vector<int64_t>> faces_of_dim(dim + 1);  // key of each id (1-based order)
  auto key = [&](unsigned e, const int64_t* P) {
    return (int64_t)e * nlat + P[0] + np[0] * (P[1] + np[1] * P[2]);
  };
  std::vector<int32_t> cell_face((size_t)ncells * nlf);
  for (int64_t c = 0; c < ncells; ++c) {
    const int64_t B[3] = {c % n[0], (c / n[0]) % n[1], c / (n[0] * n[1])};
    for (int f = 0; f < nlf; ++f) {
      const int k = __builtin_popcount(fe[f]);
      int64_t P[3] = {B[0], B[1], B[2]};
      for (int d = 0; d < dim; ++d)
        if (fa[f] & (1u << d)) P[d] += 1;
      if (k == 0) {
        cell_face[c * nlf + f] = (int32_t)(P[0] + np[0] * (P[1] + np[1] * P[2]) + 1);
      } else if (k == dim) {
        cell_face[c * nlf + f] = (int32_t)(c + 1);
      } else {
        const int64_t kk = key(fe[f], P);
        if (id[kk] == 0) {
          faces_of_dim[k].push_back(kk);
          id[kk] = (int32_t)faces_of_dim[k].size();
        }
        cell_face[c * nlf + f] = id[kk];
      }
    }
  }
  // label of a face with extrusion e at lattice position P: box-face classification
  auto entity = [&](unsigned e, const int64_t* P) {
    unsigned ext = 0, anc = 0;
    for (int d = 0; d < dim; ++d) {
      if ((e & (1u << d)) || (P[d] > 0 && P[d] < n[d])) ext |= 1u << d;
      else if (P[d] == n[d]) anc |= 1u << d;
    }
    return box_entity(dim, ext, anc);
  };
  int64_t f = 0, g = 0;
  std::vector<std::vector<int32_t>> dof(dim + 1);
  auto assign = [&](int dd, int64_t count, auto pos_of) {
    dof[dd].resize((size_t)(count + 1) * ncomp);
    for (int64_t i = 1; i <= count; ++i) {
      unsigned e;
      int64_t P[3];
      pos_of(i, &e, P);
      const int tag = entity_to_tag[entity(e, P) - 1];
      for (int comp = 0; comp < ncomp; ++comp) {
        const bool diri = tag > 0 && tag_masks && tag_masks[(size_t)(tag - 1) * ncomp + comp];
        dof[dd][i * ncomp + comp] = diri ? (int32_t)-(++g) : (int32_t)(++f);
      }
    }
  };
  assign(0, nlat, [&](int64_t i, unsigned* e, int64_t* P) {
    *e = 0;
    const int64_t v = i - 1;
    P[0] = v % np[0];
    P[1] = (v / np[0]) % np[1];
    P[2] = v / (np[0] * np[1]);
  });
  for (int dd = 1; dd < dim; ++dd)
    assign(dd, (int64_t)faces_of_dim[dd].size(), [&](int64_t i, unsigned* e, int64_t* P) {
      const int64_t kk = faces_of_dim[dd][i - 1];
      *e = (unsigned)(kk / nlat);
      const int64_t v = kk % nlat;
      P[0] = v % np[0];
      P[1] = (v / np[0]) % np[1];
      P[2] = v / (np[0] * np[1]);
    });
  assign(dim, ncells, [&](int64_t i, unsigned* e, int64_t* P) {
    *e = (1u << dim) - 1;
    const int64_t c = i - 1;
    P[0] = c % n[0];
    P[1] = (c / n[0]) % n[1];
    P[2] = c / (n[0] * n[1]);
  });
  if (f > INT32_MAX || g > INT32_MAX)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_cartesian_conforming_dofs: too many dofs");
  const int ndc = nlf * ncomp;
  for (int64_t c = 0; c < ncells; ++c)
    for (int lf = 0; lf < nlf; ++lf) {
      const int dd = __builtin_popcount(fe[lf]);
      const int32_t fid = cell_face[c * nlf + lf];
      for (int comp = 0; comp < ncomp; ++comp)
        cell_dof_ids[c * ndc + comp * nlf + lf] = dof[dd][(size_t)fid * ncomp + comp];
    }
  *nfree = (int32_t)f;
  *ndiri = (int32_t)g;
  return GFE_OK;
}

namespace gfe {
// Position of each local Q2 node on the cell's 3^D node lattice, in Gridap's local order:
// idx[a*D + d] = 0 / 1 / 2 along direction d (2*anchor along fixed directions, 1 along
// spanned ones).
void q2_node_lattice(int D, int* idx) {
  unsigned fe[27], fa[27];
  const int nn = ncube_faces(D, fe, fa);
  for (int a = 0; a < nn; ++a)
    for (int d = 0; d < D; ++d) idx[a * D + d] = (fe[a] >> d) & 1 ? 1 : 2 * ((fa[a] >> d) & 1);
}

// Q2 Lagrange basis on the 3^D nodes of the n-cube in Gridap's local order (vertices, edges,
// faces, interior; one node per face at its centre): node lattice index 0 / 1 / 2 per
// direction (2*anchor along fixed directions, 1 along spanned ones), 1-D factors the
// quadratic Lagrange polynomials on {0, 1/2, 1}.
void q2_shapes(int D, int nq, const double* qx, std::vector<double>& phi,
               std::vector<double>& dphi) {
  unsigned fe[27], fa[27];
  const int nn = ncube_faces(D, fe, fa);
  phi.assign((size_t)nq * nn, 0.0);
  dphi.assign((size_t)nq * nn * D, 0.0);
  for (int q = 0; q < nq; ++q)
    for (int a = 0; a < nn; ++a) {
      double L[3], dL[3];
      for (int d = 0; d < D; ++d) {
        const int idx = (fe[a] >> d) & 1 ? 1 : 2 * ((fa[a] >> d) & 1);
        const double t = qx[(size_t)q * D + d];
        if (idx == 0) {
          L[d] = 2.0 * (t - 0.5) * (t - 1.0);
          dL[d] = 4.0 * t - 3.0;
        } else if (idx == 1) {
          L[d] = 4.0 * t * (1.0 - t);
          dL[d] = 4.0 - 8.0 * t;
        } else {
          L[d] = 2.0 * t * (t - 0.5);
          dL[d] = 4.0 * t - 1.0;
        }
      }
      double v = 1.0;
      for (int d = 0; d < D; ++d) v *= L[d];
      phi[(size_t)q * nn + a] = v;
      for (int k = 0; k < D; ++k) {
        double g = 1.0;
        for (int d = 0; d < D; ++d) g *= (d == k) ? dL[d] : L[d];
        dphi[((size_t)q * nn + a) * D + k] = g;
      }
    }
}
}  // namespace gfe
