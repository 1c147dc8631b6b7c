// gfe_simplex.cpp -- host set-up for P2 tetrahedra on simplexified Cartesian boxes: the tet
// connectivity, the conforming P2 dof numbering, the Witherden-Vincent quadrature and the
// reference tables of isotropic elasticity.
#include <array>
#include <cmath>
#include <cstring>
#include <vector>

#include "gfe_internal.h"

namespace gfe {

// Local tets of a hexahedron, 1-based local vertices (x fastest): the oriented
// simplexification of the 3-cube (ReferenceFEs/ExtrusionPolytopes.jl:290-299).
const int kHexTets[6][4] = {{1, 2, 3, 7}, {1, 2, 5, 7}, {2, 3, 4, 7},
                            {2, 4, 7, 8}, {2, 5, 6, 7}, {2, 6, 7, 8}};
// TET edges (vertex pairs) in Gridap's face order for the (TET, TET, TET) extrusion.
const int kTetEdges[6][2] = {{1, 2}, {1, 3}, {2, 3}, {1, 4}, {2, 4}, {3, 4}};

// P2 basis on the unit tet in Gridap's node order (vertices, then TET edge midpoints).
void p2tet_shapes(int nq, const double* qx, double* phi, double* dphi) {
  static const double G[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int q = 0; q < nq; ++q) {
    const double x = qx[3 * q], y = qx[3 * q + 1], z = qx[3 * q + 2];
    const double l[4] = {1.0 - x - y - z, x, y, z};
    for (int a = 0; a < 4; ++a) {
      if (phi) phi[q * 10 + a] = l[a] * (2.0 * l[a] - 1.0);
      if (dphi)
        for (int d = 0; d < 3; ++d) dphi[(q * 10 + a) * 3 + d] = (4.0 * l[a] - 1.0) * G[a][d];
    }
    for (int e = 0; e < 6; ++e) {
      const int a = kTetEdges[e][0] - 1, b = kTetEdges[e][1] - 1;
      if (phi) phi[q * 10 + 4 + e] = 4.0 * l[a] * l[b];
      if (dphi)
        for (int d = 0; d < 3; ++d)
          dphi[(q * 10 + 4 + e) * 3 + d] = 4.0 * (G[a][d] * l[b] + l[a] * G[b][d]);
    }
  }
}

// The symmetric 14-point rule of degree 5 on the unit tet (Witherden & Vincent 2015; Gridap
// uses it for degrees 4 and 5: ReferenceFEs/WitherdenVincentQuadratures.jl:367-520). The
// rule is determined by its orbit structure -- two S31 orbits (a,a,a,1-3a) and one S22 orbit
// (b,b,1/2-b,1/2-b) -- and the degree-5 moment equations, solved here by Gauss-Newton in
// extended precision. Points follow Gridap's orbit expansion order; weights sum to 1/6.
namespace {
void wv_expand(const long double* u, long double P[14][3], long double W[14],
               long double dP[14][3][6], long double dW[14][6]) {
  std::memset(dP, 0, sizeof(long double) * 14 * 3 * 6);
  std::memset(dW, 0, sizeof(long double) * 14 * 6);
  int r = 0;
  static const int p31[4][3] = {{0, 0, 1}, {0, 1, 0}, {1, 0, 0}, {0, 0, 0}};
  for (int o = 0; o < 2; ++o)
    for (int k = 0; k < 4; ++k, ++r) {
      for (int d = 0; d < 3; ++d) {
        P[r][d] = p31[k][d] ? 1.0L - 3.0L * u[o] : u[o];
        dP[r][d][o] = p31[k][d] ? -3.0L : 1.0L;
      }
      W[r] = u[3 + o];
      dW[r][3 + o] = 1.0L;
    }
  static const int p22[6][3] = {{0, 1, 1}, {1, 0, 1}, {0, 0, 1}, {0, 1, 0}, {1, 0, 0}, {1, 1, 0}};
  for (int k = 0; k < 6; ++k, ++r) {
    for (int d = 0; d < 3; ++d) {
      P[r][d] = p22[k][d] ? 0.5L - u[2] : u[2];
      dP[r][d][2] = p22[k][d] ? -1.0L : 1.0L;
    }
    W[r] = u[5];
    dW[r][5] = 1.0L;
  }
}

long double ipow(long double x, int n) {
  long double r = 1.0L;
  while (n-- > 0) r *= x;
  return r;
}
}  // namespace

int tet_quadrature(int degree, std::vector<double>& x, std::vector<double>& w) {
  if (degree != 4 && degree != 5)
    return set_error(GFE_ERR_UNSUPPORTED, "tet quadrature: degrees 4 and 5 are provided");
  long double u[6] = {0.31L, 0.09L, 0.045L, 0.0188L, 0.0122L, 0.0071L};
  long double P[14][3], W[14], dP[14][3][6], dW[14][6];
  long double fact[9] = {1, 1, 2, 6, 24, 120, 720, 5040, 40320};
  for (int it = 0; it < 60; ++it) {
    wv_expand(u, P, W, dP, dW);
    long double M[6][7] = {{0}};
    for (int p = 0; p <= 5; ++p)
      for (int q = 0; p + q <= 5; ++q)
        for (int s = 0; p + q + s <= 5; ++s) {
          long double f = -fact[p] * fact[q] * fact[s] / fact[p + q + s + 3], g[6] = {0};
          for (int k = 0; k < 14; ++k) {
            const long double m = ipow(P[k][0], p) * ipow(P[k][1], q) * ipow(P[k][2], s);
            const long double d0 = p ? p * ipow(P[k][0], p - 1) * ipow(P[k][1], q) * ipow(P[k][2], s) : 0;
            const long double d1 = q ? q * ipow(P[k][0], p) * ipow(P[k][1], q - 1) * ipow(P[k][2], s) : 0;
            const long double d2 = s ? s * ipow(P[k][0], p) * ipow(P[k][1], q) * ipow(P[k][2], s - 1) : 0;
            f += W[k] * m;
            for (int j = 0; j < 6; ++j)
              g[j] += dW[k][j] * m + W[k] * (d0 * dP[k][0][j] + d1 * dP[k][1][j] + d2 * dP[k][2][j]);
          }
          for (int i = 0; i < 6; ++i) {
            M[i][6] -= g[i] * f;
            for (int j = 0; j < 6; ++j) M[i][j] += g[i] * g[j];
          }
        }
    for (int c = 0; c < 6; ++c) {  // Gaussian elimination, partial pivoting
      int piv = c;
      for (int i = c + 1; i < 6; ++i)
        if (fabsl(M[i][c]) > fabsl(M[piv][c])) piv = i;
      for (int j = 0; j < 7; ++j) std::swap(M[c][j], M[piv][j]);
      for (int i = c + 1; i < 6; ++i) {
        const long double f = M[i][c] / M[c][c];
        for (int j = c; j < 7; ++j) M[i][j] -= f * M[c][j];
      }
    }
    long double d[6], dn = 0.0L;
    for (int i = 5; i >= 0; --i) {
      long double s = M[i][6];
      for (int j = i + 1; j < 6; ++j) s -= M[i][j] * d[j];
      d[i] = s / M[i][i];
    }
    for (int i = 0; i < 6; ++i) {
      u[i] += d[i];
      dn += fabsl(d[i]);
    }
    if (dn < 1e-30L) break;
  }
  wv_expand(u, P, W, dP, dW);
  x.resize(42);
  w.resize(14);
  for (int k = 0; k < 14; ++k) {
    for (int d = 0; d < 3; ++d) x[3 * k + d] = (double)P[k][d];
    w[k] = (double)W[k];
  }
  return GFE_OK;
}

// Elasticity tables of the 6 local tets of a Cartesian cell of size h (in long double, from
// Gridap's per-quadrature-point steps): for tet t, Kl[t][(k,i),(l,j)] = sum_q dV_q d_k phi_i
// d_l phi_j and Km[t][..] = sum_q dV_q (delta_kl grad phi_i . grad phi_j + d_l phi_i d_k phi_j),
// so that the cell matrix is lambda Kl + mu Km (eps(v) : (lambda tr eps(u) I + 2 mu eps(u))
// expanded for v = phi_i e_k, u = phi_j e_l; local dof k*10 + i, column-major 30 x 30);
// mv[t][i] = sum_q dV_q phi_i. Layout: Kl[6*900] | Km[6*900] | mv[6*10].
int elasticity_p2_tables(const double* h, int degree, std::vector<double>& tab) {
  std::vector<double> qx, qw;
  GFE_TRY(tet_quadrature(degree, qx, qw));
  const int nq = (int)qw.size();
  std::vector<double> phi(nq * 10), dphi(nq * 30);
  p2tet_shapes(nq, qx.data(), phi.data(), dphi.data());
  tab.assign(6 * 900 * 2 + 60, 0.0);
  static const long double G1[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int t = 0; t < 6; ++t) {
    long double X[4][3];
    for (int a = 0; a < 4; ++a) {
      const int v = kHexTets[t][a] - 1;
      for (int d = 0; d < 3; ++d) X[a][d] = ((v >> d) & 1) ? (long double)h[d] : 0.0L;
    }
    long double J[3][3] = {{0}};  // Jt_{kl} = sum_a dphi1_a[k] x_a[l]
    for (int a = 0; a < 4; ++a)
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) J[k][l] += G1[a][k] * X[a][l];
    const long double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                            J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                            J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    long double C[3][3];  // inverse of Jt
    C[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
    C[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    C[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    C[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
    C[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    C[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    C[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
    C[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    C[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    std::vector<long double> Kl(900, 0.0L), Km(900, 0.0L), mv(10, 0.0L);
    for (int q = 0; q < nq; ++q) {
      const long double dV = fabsl(det) * qw[q];
      long double g[10][3];
      for (int n = 0; n < 10; ++n)
        for (int k = 0; k < 3; ++k) {
          long double s = 0.0L;
          for (int l = 0; l < 3; ++l) s += C[k][l] * dphi[(q * 10 + n) * 3 + l];
          g[n][k] = s;
        }
      for (int n = 0; n < 10; ++n) mv[n] += dV * phi[q * 10 + n];
      for (int l = 0; l < 3; ++l)
        for (int j = 0; j < 10; ++j)
          for (int k = 0; k < 3; ++k)
            for (int i = 0; i < 10; ++i) {
              const int r = k * 10 + i, c = l * 10 + j;
              const long double gg = g[i][0] * g[j][0] + g[i][1] * g[j][1] + g[i][2] * g[j][2];
              Kl[r + 30 * c] += dV * g[i][k] * g[j][l];
              Km[r + 30 * c] += dV * ((k == l ? gg : 0.0L) + g[i][l] * g[j][k]);
            }
    }
    for (int e = 0; e < 900; ++e) {
      tab[t * 900 + e] = (double)Kl[e];
      tab[5400 + t * 900 + e] = (double)Km[e];
    }
    for (int n = 0; n < 10; ++n) tab[10800 + t * 10 + n] = (double)mv[n];
  }
  return GFE_OK;
}

// Reference integrals for general affine tets: G[(a*3+b)*100 + i*10 + j] = sum_q w_q
// d_a phi_i(xi_q) d_b phi_j(xi_q) and m[i] = sum_q w_q phi_i(xi_q) (unit tet), in long double.
int p2tet_reference_integrals(int degree, std::vector<double>& G, std::vector<double>& m) {
  std::vector<double> qx, qw;
  GFE_TRY(tet_quadrature(degree, qx, qw));
  const int nq = (int)qw.size();
  std::vector<double> phi(nq * 10), dphi(nq * 30);
  p2tet_shapes(nq, qx.data(), phi.data(), dphi.data());
  G.assign(900, 0.0);
  m.assign(10, 0.0);
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      for (int i = 0; i < 10; ++i)
        for (int j = 0; j < 10; ++j) {
          long double s = 0.0L;
          for (int q = 0; q < nq; ++q)
            s += (long double)qw[q] * dphi[(q * 10 + i) * 3 + a] * dphi[(q * 10 + j) * 3 + b];
          G[(a * 3 + b) * 100 + i * 10 + j] = (double)s;
        }
  for (int i = 0; i < 10; ++i) {
    long double s = 0.0L;
    for (int q = 0; q < nq; ++q) s += (long double)qw[q] * phi[q * 10 + i];
    m[i] = (double)s;
  }
  return GFE_OK;
}

}  // namespace gfe

using namespace gfe;

extern "C" int gfe_simplex_model(const int64_t* partition, int32_t* tet_vertex_ids) {
  clear_error();
  if (!partition || !tet_vertex_ids)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_simplex_model: NULL argument");
  const int64_t n0 = partition[0], n1 = partition[1], n2 = partition[2];
  if (n0 < 1 || n1 < 1 || n2 < 1)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_simplex_model: bad partition");
  int64_t c = 0;
  for (int64_t k = 0; k < n2; ++k)
    for (int64_t j = 0; j < n1; ++j)
      for (int64_t i = 0; i < n0; ++i, ++c)
        for (int t = 0; t < 6; ++t)
          for (int a = 0; a < 4; ++a) {
            const int v = kHexTets[t][a] - 1;
            const int64_t node = (i + (v & 1)) + (n0 + 1) * ((j + ((v >> 1) & 1)) +
                                                              (n1 + 1) * (k + ((v >> 2) & 1)));
            tet_vertex_ids[(c * 6 + t) * 4 + a] = (int32_t)(node + 1);
          }
  return GFE_OK;
}

// Conforming P2 numbering on simplexify(CartesianDiscreteModel): an edge's id is its rank in
// first-touch order over (tet, local edge) -- the order in which Gridap's grid topology
// numbers faces (Geometry/GridTopologies.jl:1184-1250). An edge is identified by its
// midpoint on the twice-refined lattice, so the first-touch pass is one array lookup per
// (tet, edge). Faces whose vertices all carry vertex_mask are Dirichlet for the components in
// comp_mask (face_labeling_from_vertex_filter, Geometry/FaceLabelings.jl:590-611); dofs are
// numbered vertices first, then edges, components of a face consecutive
// (FESpaces/ConformingFESpaces.jl:543-636).
extern "C" int gfe_simplex_p2_dofs(const int64_t* partition, int32_t ncomp,
                                   const uint8_t* vertex_mask, const uint8_t* comp_mask,
                                   int32_t* cell_dof_ids, int32_t* nfree, int32_t* ndiri) {
  clear_error();
  if (!partition || !vertex_mask || !comp_mask || !cell_dof_ids || ncomp < 1 || ncomp > 3)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_simplex_p2_dofs: bad arguments");
  const int64_t n0 = partition[0], n1 = partition[1], n2 = partition[2];
  if (n0 < 1 || n1 < 1 || n2 < 1)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_simplex_p2_dofs: bad partition");
  const int64_t r0 = 2 * n0 + 1, r1 = 2 * n1 + 1, r2 = 2 * n2 + 1;
  const int64_t nverts = (n0 + 1) * (n1 + 1) * (n2 + 1);
  if (r0 * r1 * r2 * ncomp >= INT32_MAX)
    return set_error(GFE_ERR_UNSUPPORTED, "gfe_simplex_p2_dofs: too many dofs");
  std::vector<int32_t> edge_at(r0 * r1 * r2, 0);  // refined lattice point -> edge id
  std::vector<int64_t> edge_mid;                   // edge id - 1 -> lattice point
  std::vector<int32_t> tv((size_t)n0 * n1 * n2 * 24);
  GFE_TRY(gfe_simplex_model(partition, tv.data()));
  const int64_t ntets = n0 * n1 * n2 * 6;
  std::vector<int64_t> vlat(4);
  auto lattice = [&](int32_t v1) {  // 1-based vertex -> refined lattice coordinates
    const int64_t v = v1 - 1;
    const int64_t i = v % (n0 + 1), r = v / (n0 + 1), j = r % (n1 + 1), k = r / (n1 + 1);
    return std::array<int64_t, 3>{2 * i, 2 * j, 2 * k};
  };
  std::vector<int32_t> tet_edges((size_t)ntets * 6);
  for (int64_t c = 0; c < ntets; ++c)
    for (int e = 0; e < 6; ++e) {
      const auto A = lattice(tv[c * 4 + kTetEdges[e][0] - 1]);
      const auto B = lattice(tv[c * 4 + kTetEdges[e][1] - 1]);
      const int64_t m = (A[0] + B[0]) / 2 + r0 * ((A[1] + B[1]) / 2 + r1 * ((A[2] + B[2]) / 2));
      if (!edge_at[m]) {
        edge_mid.push_back(c * 6 + e);
        edge_at[m] = (int32_t)edge_mid.size();
      }
      tet_edges[c * 6 + e] = edge_at[m];
    }
  const int64_t nedges = (int64_t)edge_mid.size();
  std::vector<int32_t> vdof(nverts * ncomp), edof(nedges * ncomp);
  int32_t nf = 0, nd = 0;
  for (int64_t v = 0; v < nverts; ++v)
    for (int k = 0; k < ncomp; ++k)
      vdof[v * ncomp + k] = (vertex_mask[v] && comp_mask[k]) ? -(++nd) : ++nf;
  for (int64_t e = 0; e < nedges; ++e) {
    const int64_t c = edge_mid[e] / 6;
    const int le = (int)(edge_mid[e] % 6);
    const bool tagged = vertex_mask[tv[c * 4 + kTetEdges[le][0] - 1] - 1] &&
                        vertex_mask[tv[c * 4 + kTetEdges[le][1] - 1] - 1];
    for (int k = 0; k < ncomp; ++k)
      edof[e * ncomp + k] = (tagged && comp_mask[k]) ? -(++nd) : ++nf;
  }
  const int ndc = 10 * ncomp;
  for (int64_t c = 0; c < ntets; ++c)
    for (int k = 0; k < ncomp; ++k) {
      for (int a = 0; a < 4; ++a)
        cell_dof_ids[c * ndc + k * 10 + a] = vdof[(int64_t)(tv[c * 4 + a] - 1) * ncomp + k];
      for (int e = 0; e < 6; ++e)
        cell_dof_ids[c * ndc + k * 10 + 4 + e] =
            edof[(int64_t)(tet_edges[c * 6 + e] - 1) * ncomp + k];
    }
  if (nfree) *nfree = nf;
  if (ndiri) *ndiri = nd;
  return GFE_OK;
}
