// Host precompute: OpenFOAM-style 2-D polyMesh -> the reference's host field bundle.
//
// This is the work the reference's solver object does with OpenFOAM before the first step:
//   geometry + field init       basicCUDAsolver.cpp:122-258 (initFieldInfo)
//   adjacency, stencils         basicCUDAsolver.cpp:269-417
//   Gauss quadrature            d2GaussQuadrature.C:23-150, 153-280, 333-547
//   RBF P matrix, SVD pinv      basicCUDAsolver.cpp:420-533
//   O3 face weights             basicCUDAsolver.cpp:538-619
//   128-cell block halo remap   basicCUDAsolver.cpp:697-850
// OpenFOAM is not used: geometry is computed from the polygons, SVDinv is a one-sided Jacobi
// SVD pseudo-inverse, and the edge-neighbour stencil walks cell vertices (the cells sharing an
// edge of the extruded prism are the cells sharing a vertex of the cross-section).
//
// Compiled with -ffp-contract=off so x86 and aarch64 hosts produce the same arrays.
#include "afar_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace afar {

namespace {

struct Pt {
  double x, y;
};

// Standard rules of d2GaussQuadrature.C (reference square (-1,1)^2, area 4; reference triangle
// (0,0),(1,0),(0,1), area 1/2; reference bar (-1,1)).
void rec_rule(int order, std::vector<Pt>& ps, std::vector<double>& ws) {
  ps.clear();
  ws.clear();
  if (order == 1) {  // d2GaussQuadrature.C:342-351
    ps.push_back({0.0, 0.0});
    ws.push_back(4.0);
  } else if (order > 1 && order <= 3) {  // :352-364; the reference leaves ws[1..3] unset, here 1
    const double a = 1.0 / std::sqrt(3.0);
    ps = {{-a, -a}, {-a, a}, {a, -a}, {a, a}};
    ws = {1.0, 1.0, 1.0, 1.0};
  } else if (order > 3 && order <= 5) {  // :365-382, 3x3 tensor Gauss-Legendre
    const double a = std::sqrt(0.6);
    const double g[3] = {-a, 0.0, a};
    const double w[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        ps.push_back({g[i], g[j]});
        ws.push_back(w[i] * w[j]);
      }
  } else if (order > 5 && order <= 7) {  // :383-410, 4x4 tensor Gauss-Legendre
    const double g[4] = {0.861136311594053, 0.339981043584856, -0.339981043584856, -0.861136311594053};
    const double w[4] = {0.347854845137454, 0.652145154862546, 0.652145154862546, 0.347854845137454};
    for (int j = 0; j < 4; ++j)
      for (int i = 0; i < 4; ++i) {
        ps.push_back({g[i], g[j]});
        ws.push_back(w[i] * w[j]);
      }
  }
}

void tri_rule(int order, std::vector<Pt>& ps, std::vector<double>& ws) {
  ps.clear();
  ws.clear();
  if (order == 1) {  // d2GaussQuadrature.C:430-439
    ps.push_back({1.0 / 3.0, 1.0 / 3.0});
    ws.push_back(0.5);
  } else if (order > 1 && order <= 3) {  // :440-451, edge midpoints
    ps = {{0.5, 0.5}, {0.5, 0.0}, {0.0, 0.5}};
    ws = {1.0 / 6.0, 1.0 / 6.0, 1.0 / 6.0};
  } else if (order > 3 && order <= 5) {  // :452-464
    ps = {{1.0 / 3.0, 1.0 / 3.0}, {3.0 / 5.0, 1.0 / 5.0}, {1.0 / 5.0, 1.0 / 5.0}, {1.0 / 5.0, 3.0 / 5.0}};
    ws = {21.0 / 96.0, 25.0 / 96.0, 25.0 / 96.0, 25.0 / 96.0};
  } else if (order > 5 && order <= 7) {  // :465-479, 6-point degree-4 rule
    const double a = 0.816847572980459, b = 0.091576213509771;
    const double c = 0.108103018168070, d = 0.445948490915965;
    const double wa = 0.109951743655322 * 0.5, wc = 0.223381589678011 * 0.5;
    ps = {{a, b}, {b, a}, {b, b}, {c, d}, {d, c}, {d, d}};
    ws = {wa, wa, wa, wc, wc, wc};
  }
}

void bar_rule(int order, std::vector<double>& ps, std::vector<double>& ws) {
  ps.clear();
  ws.clear();
  if (order == 1) {  // d2GaussQuadrature.C:495-504
    ps = {0.0};
    ws = {2.0};
  } else if (order > 1 && order <= 3) {  // :505-515
    const double a = 1.0 / std::sqrt(3.0);
    ps = {-a, a};
    ws = {1.0, 1.0};
  } else if (order > 3 && order <= 5) {  // :516-527
    const double a = std::sqrt(0.6);
    ps = {-a, 0.0, a};
    ws = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
  } else if (order > 5 && order <= 7) {  // :528-540
    ps = {0.861136311594053, 0.339981043584856, -0.339981043584856, -0.861136311594053};
    ws = {0.347854845137454, 0.652145154862546, 0.652145154862546, 0.347854845137454};
  }
}

// Orders the 4 corners of a quad by decreasing polar angle about their mean
// (d2GaussQuadrature.C:283-331: bubble sort, largest angle first).
void sort_quad(Pt* p) {
  double cx = 0.0, cy = 0.0;
  for (int i = 0; i < 4; ++i) {
    cx += p[i].x;
    cy += p[i].y;
  }
  cx /= 4.0;
  cy /= 4.0;
  double polar[4];
  int idx[4] = {0, 1, 2, 3};
  for (int i = 0; i < 4; ++i) {
    const double x = p[i].x - cx, y = p[i].y - cy;
    const double r = std::sqrt(x * x + y * y);
    polar[i] = y >= 0 ? std::acos(x / r) : -std::acos(x / r);
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3 - i; ++j)
      if (polar[j] < polar[j + 1]) {
        std::swap(polar[j], polar[j + 1]);
        std::swap(idx[j], idx[j + 1]);
      }
  Pt q[4];
  for (int i = 0; i < 4; ++i) q[i] = p[idx[i]];
  for (int i = 0; i < 4; ++i) p[i] = q[i];
}

// A coordinate difference taken to the nearest periodic image (L > 0), else unchanged.
inline double wrapd(const double d, const double L) { return L > 0.0 ? d - L * std::rint(d / L) : d; }
// The point that stands for all periodic images of point p (topology only).
inline int point_id(const afar_polyMesh* m, const int p) { return m->pointAlias ? m->pointAlias[p] : p; }

struct Geom {
  std::vector<double> cx, cy, area;        // cells
  std::vector<double> fx, fy, sfx, sfy, magsf;  // all faces
};

bool compute_geometry(const afar_polyMesh* m, Geom& g) {
  const int nc = m->nCells, nF = m->nFaces;
  g.cx.assign(nc, 0.0);
  g.cy.assign(nc, 0.0);
  g.area.assign(nc, 0.0);
  for (int c = 0; c < nc; ++c) {
    const int b = m->cellPointsOffset[c], e = m->cellPointsOffset[c + 1];
    const int n = e - b;
    if (n != 3 && n != 4) {
      set_error("cell %d has %d points; only triangles and quadrilaterals are 2-D cells here", c, n);
      return false;
    }
    double a2 = 0.0, sx = 0.0, sy = 0.0;
    for (int k = 0; k < n; ++k) {
      const int i = m->cellPoints[b + k], j = m->cellPoints[b + (k + 1) % n];
      const double xi = m->points[2 * i], yi = m->points[2 * i + 1];
      const double xj = m->points[2 * j], yj = m->points[2 * j + 1];
      const double cr = xi * yj - xj * yi;
      a2 += cr;
      sx += (xi + xj) * cr;
      sy += (yi + yj) * cr;
    }
    if (!(std::fabs(a2) > 0.0)) {
      set_error("cell %d has zero area", c);
      return false;
    }
    g.cx[c] = sx / (3.0 * a2);
    g.cy[c] = sy / (3.0 * a2);
    g.area[c] = std::fabs(0.5 * a2);
  }
  g.fx.resize(nF);
  g.fy.resize(nF);
  g.sfx.resize(nF);
  g.sfy.resize(nF);
  g.magsf.resize(nF);
  for (int f = 0; f < nF; ++f) {
    const int a = m->facePoints[2 * f], b = m->facePoints[2 * f + 1];
    const double xa = m->points[2 * a], ya = m->points[2 * a + 1];
    const double xb = m->points[2 * b], yb = m->points[2 * b + 1];
    g.fx[f] = 0.5 * (xa + xb);
    g.fy[f] = 0.5 * (ya + yb);
    const double dx = xb - xa, dy = yb - ya;
    g.sfx[f] = dy * m->depth;
    g.sfy[f] = -dx * m->depth;
    g.magsf[f] = std::sqrt(dx * dx + dy * dy) * m->depth;
    // the face normal must point out of the owner
    const int o = m->owner[f];
    const double dot = (g.fx[f] - g.cx[o]) * g.sfx[f] + (g.fy[f] - g.cy[o]) * g.sfy[f];
    if (!(dot > 0.0)) {
      set_error("face %d: normal does not point out of its owner cell %d", f, o);
      return false;
    }
  }
  return true;
}

// Cell Gauss points/weights, weights normalised by the cell area (d2GaussQuadrature.C:63-141).
void cell_gauss(const afar_polyMesh* m, const Geom& g, int c, int order, std::vector<Pt>& out_p,
                std::vector<double>& out_w) {
  std::vector<Pt> sp;
  std::vector<double> sw;
  const int b = m->cellPointsOffset[c];
  const int n = m->cellPointsOffset[c + 1] - b;
  Pt p[4];
  for (int k = 0; k < n; ++k) {
    const int i = m->cellPoints[b + k];
    p[k] = {m->points[2 * i], m->points[2 * i + 1]};
  }
  out_p.clear();
  out_w.clear();
  const double area = g.area[c];
  if (n == 3) {
    tri_rule(order, sp, sw);
    const double jac = std::fabs((p[1].x - p[0].x) * (p[2].y - p[0].y) - (p[2].x - p[0].x) * (p[1].y - p[0].y));
    for (size_t k = 0; k < sp.size(); ++k) {
      const double xi = sp[k].x, eta = sp[k].y;
      out_p.push_back({p[0].x + (p[1].x - p[0].x) * xi + (p[2].x - p[0].x) * eta,
                       p[0].y + (p[1].y - p[0].y) * xi + (p[2].y - p[0].y) * eta});
      out_w.push_back(sw[k] * jac / area);
    }
  } else {
    rec_rule(order, sp, sw);
    sort_quad(p);
    for (size_t k = 0; k < sp.size(); ++k) {
      const double xi = sp[k].x, eta = sp[k].y;
      const double b1 = 0.25 * (1.0 - xi) * (1.0 - eta);
      const double b2 = 0.25 * (1.0 - xi) * (1.0 + eta);
      const double b3 = 0.25 * (1.0 + xi) * (1.0 + eta);
      const double b4 = 0.25 * (1.0 + xi) * (1.0 - eta);
      out_p.push_back({p[0].x * b1 + p[1].x * b2 + p[2].x * b3 + p[3].x * b4,
                       p[0].y * b1 + p[1].y * b2 + p[2].y * b3 + p[3].y * b4});
      const double dxdxi = -0.25 * p[0].x * (1.0 - eta) - 0.25 * p[1].x * (1.0 + eta) + 0.25 * p[2].x * (1.0 + eta) + 0.25 * p[3].x * (1.0 - eta);
      const double dxdeta = -0.25 * p[0].x * (1.0 - xi) + 0.25 * p[1].x * (1.0 - xi) + 0.25 * p[2].x * (1.0 + xi) - 0.25 * p[3].x * (1.0 + xi);
      const double dydxi = -0.25 * p[0].y * (1.0 - eta) - 0.25 * p[1].y * (1.0 + eta) + 0.25 * p[2].y * (1.0 + eta) + 0.25 * p[3].y * (1.0 - eta);
      const double dydeta = -0.25 * p[0].y * (1.0 - xi) + 0.25 * p[1].y * (1.0 - xi) + 0.25 * p[2].y * (1.0 + xi) - 0.25 * p[3].y * (1.0 + xi);
      out_w.push_back(sw[k] * std::fabs(dxdxi * dydeta - dxdeta * dydxi) / area);
    }
  }
}

// Boundary-face Gauss points on the edge, weights as a line average: the reference's
// w_std*jacobi*height (d2GaussQuadrature.C:259-276) divided by |Sf| (basicCUDAsolver.cpp:452).
void face_gauss(const afar_polyMesh* m, int f, int order, std::vector<Pt>& out_p, std::vector<double>& out_w) {
  std::vector<double> sp, sw;
  bar_rule(order, sp, sw);
  const int a = m->facePoints[2 * f], b = m->facePoints[2 * f + 1];
  const double xa = m->points[2 * a], ya = m->points[2 * a + 1];
  const double xb = m->points[2 * b], yb = m->points[2 * b + 1];
  const double jac = std::sqrt((0.5 * (xa - xb)) * (0.5 * (xa - xb)) + (0.5 * (ya - yb)) * (0.5 * (ya - yb)));
  const double len = std::sqrt((xb - xa) * (xb - xa) + (yb - ya) * (yb - ya));
  out_p.clear();
  out_w.clear();
  for (size_t k = 0; k < sp.size(); ++k) {
    const double xi = sp[k];
    out_p.push_back({0.5 * xa * (1 - xi) + 0.5 * xb * (1 + xi), 0.5 * ya * (1 - xi) + 0.5 * yb * (1 + xi)});
    out_w.push_back(sw[k] * jac * m->depth / (len * m->depth));
  }
}

}  // namespace

// One-sided (Hestenes) Jacobi SVD pseudo-inverse of a square n x n matrix A (row-major), the
// role of Foam::SVDinv with minCondition 0 (basicCUDAsolver.cpp:509): singular values that are
// exactly zero are dropped, all others inverted.  G = V diag(1/s^2) (AV)^T.
void svd_pinv(int n, const double* A, double* G) {
  std::vector<double> U(A, A + n * n);  // columns rotated in place: U = A V
  std::vector<double> V(n * n, 0.0);
  for (int i = 0; i < n; ++i) V[i * n + i] = 1.0;
  const double tol = 1e-15;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n - 1; ++p) {
      for (int q = p + 1; q < n; ++q) {
        double alpha = 0.0, beta = 0.0, gamma = 0.0;
        for (int i = 0; i < n; ++i) {
          const double up = U[i * n + p], uq = U[i * n + q];
          alpha += up * up;
          beta += uq * uq;
          gamma += up * uq;
        }
        if (alpha == 0.0 || beta == 0.0) continue;
        const double c0 = std::fabs(gamma) / std::sqrt(alpha * beta);
        off = std::max(off, c0);
        if (c0 <= tol) continue;
        const double zeta = (beta - alpha) / (2.0 * gamma);
        const double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / std::sqrt(1.0 + t * t);
        const double s = c * t;
        for (int i = 0; i < n; ++i) {
          const double up = U[i * n + p], uq = U[i * n + q];
          U[i * n + p] = c * up - s * uq;
          U[i * n + q] = s * up + c * uq;
          const double vp = V[i * n + p], vq = V[i * n + q];
          V[i * n + p] = c * vp - s * vq;
          V[i * n + q] = s * vp + c * vq;
        }
      }
    }
    if (off <= tol) break;
  }
  std::vector<double> inv_s2(n, 0.0);
  for (int k = 0; k < n; ++k) {
    double s2 = 0.0;
    for (int i = 0; i < n; ++i) s2 += U[i * n + k] * U[i * n + k];
    inv_s2[k] = s2 > 0.0 ? 1.0 / s2 : 0.0;
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double acc = 0.0;
      for (int k = 0; k < n; ++k) acc += V[i * n + k] * inv_s2[k] * U[j * n + k];
      G[i * n + j] = acc;
    }
}

// Inverse of a row-major n x n matrix by LU factorisation with partial (row) pivoting, G = A^-1.
// Returns false (G untouched) when a pivot is exactly zero: the matrix is singular and the caller
// falls back to the SVD pseudo-inverse.  For a nonsingular matrix the inverse is the pseudo-inverse,
// equal to svd_pinv's up to rounding amplified by the condition number, at ~n^3 instead of
// ~(Jacobi sweeps) * n^3 operations.
bool lu_inverse(int n, const double* A, double* G) {
  double LU[(AFAR_MAX_VALID_STENCIL_SIZE + 1) * (AFAR_MAX_VALID_STENCIL_SIZE + 1)];
  int piv[AFAR_MAX_VALID_STENCIL_SIZE + 1];
  for (int i = 0; i < n * n; ++i) LU[i] = A[i];
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = std::fabs(LU[k * n + k]);
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(LU[i * n + k]) > best) {
        best = std::fabs(LU[i * n + k]);
        p = i;
      }
    if (!(best > 0.0)) return false;
    piv[k] = p;
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(LU[k * n + j], LU[p * n + j]);
    const double inv = 1.0 / LU[k * n + k];
    for (int i = k + 1; i < n; ++i) {
      const double l = LU[i * n + k] * inv;
      LU[i * n + k] = l;
      for (int j = k + 1; j < n; ++j) LU[i * n + j] -= l * LU[k * n + j];
    }
  }
  for (int col = 0; col < n; ++col) {  // solve LU x = P e_col
    double x[AFAR_MAX_VALID_STENCIL_SIZE + 1];
    for (int i = 0; i < n; ++i) x[i] = i == col ? 1.0 : 0.0;
    for (int k = 0; k < n; ++k)
      if (piv[k] != k) std::swap(x[k], x[piv[k]]);
    for (int i = 1; i < n; ++i)
      for (int j = 0; j < i; ++j) x[i] -= LU[i * n + j] * x[j];
    for (int i = n - 1; i >= 0; --i) {
      for (int j = i + 1; j < n; ++j) x[i] -= LU[i * n + j] * x[j];
      x[i] /= LU[i * n + i];
    }
    for (int i = 0; i < n; ++i) G[i * n + col] = x[i];
  }
  return true;
}

}  // namespace afar

using namespace afar;

extern "C" void afar_default_case_config(afar_caseConfig* cfg) {
  if (!cfg) return;
  cfg->R = 1.0 / 1.4;
  cfg->Cv = cfg->R / 0.4;
  cfg->CFL = 0.5;
  cfg->shapeFactor = 10.0;
  cfg->stencilType = AFAR_STENCIL_EDGE_NEIGHBOUR;
  cfg->cOrder = 5;
  cfg->fOrder = 4;
  cfg->nThreads = 0;
}

static bool check_mesh(const afar_polyMesh* m) {
  if (!m || !m->points || !m->cellPointsOffset || !m->cellPoints || !m->facePoints || !m->owner ||
      (m->nInternalFaces > 0 && !m->neighbour) || m->nCells <= 0 || m->nInternalFaces < 0 ||
      m->nFaces < m->nInternalFaces || m->nPatches < 0 || (m->nPatches > 0 && (!m->patchStart || !m->patchSize || !m->patchLabel)) ||
      !(m->depth > 0.0)) {
    set_error("afar_polyMesh: null array, negative size or non-positive depth");
    return false;
  }
  for (int f = 0; f < m->nFaces; ++f) {
    if (m->owner[f] < 0 || m->owner[f] >= m->nCells) {
      set_error("face %d: owner %d out of range", f, m->owner[f]);
      return false;
    }
    if (f < m->nInternalFaces) {
      const int nb = m->neighbour[f];
      if (nb < 0 || nb >= m->nCells || nb <= m->owner[f]) {
        set_error("internal face %d: neighbour %d must be in range and greater than owner %d", f, nb, m->owner[f]);
        return false;
      }
    }
    for (int k = 0; k < 2; ++k)
      if (m->facePoints[2 * f + k] < 0 || m->facePoints[2 * f + k] >= m->nPoints) {
        set_error("face %d: point index out of range", f);
        return false;
      }
  }
  if (m->pointAlias)
    for (int p = 0; p < m->nPoints; ++p)
      if (m->pointAlias[p] < 0 || m->pointAlias[p] >= m->nPoints) {
        set_error("point %d: alias %d out of range", p, m->pointAlias[p]);
        return false;
      }
  int expect = m->nInternalFaces;
  for (int p = 0; p < m->nPatches; ++p) {
    if (m->patchSize[p] < 0 || (m->patchSize[p] > 0 && m->patchStart[p] != expect)) {
      set_error("patch %d: faces must follow the internal faces patch by patch (start %d, expected %d)", p,
                m->patchStart[p], expect);
      return false;
    }
    if (m->patchSize[p] > 0 && (m->patchLabel[p] < 0 || m->patchLabel[p] > 255)) {
      set_error("patch %d: boundary label %d out of range", p, m->patchLabel[p]);
      return false;
    }
    expect += m->patchSize[p];
  }
  if (expect != m->nFaces) {
    set_error("patch sizes add up to %d faces, mesh has %d", expect, m->nFaces);
    return false;
  }
  for (int c = 0; c < m->nCells; ++c)
    if (m->cellPointsOffset[c + 1] < m->cellPointsOffset[c]) {
      set_error("cellPointsOffset not monotone at cell %d", c);
      return false;
    }
  return true;
}

// The face Gauss points of d2GaussQuadrature::calcFaceGaussQuadrature (d2GaussQuadrature.C:153-214,
// and :216-277 for the boundary patches) for every face in face order: the bar rule of fOrder mapped
// onto the edge from its first to its second point, x_k = (p0 (1 - xi_k) + p1 (1 + xi_k)) / 2, weight
// w_k * |p1 - p0| / 2 * depth (the face area included, as the reference keeps it for face fluxes).
extern "C" afar_status afar_face_gauss_quadrature(const afar_polyMesh* m, const afar_caseConfig* cfg,
                                                  int* pointsPerFace, double* pts, double* w) {
  if (!check_mesh(m) || !cfg || !pointsPerFace) {
    if (!cfg || !pointsPerFace) set_error("afar_face_gauss_quadrature: null argument");
    return AFAR_ERR_ARGUMENT;
  }
  std::vector<double> sp, sw;
  bar_rule(cfg->fOrder, sp, sw);
  if (sp.empty()) {
    set_error("no Gauss rule stored for fOrder=%d", cfg->fOrder);
    return AFAR_ERR_ARGUMENT;
  }
  const int ng = (int)sp.size();
  *pointsPerFace = ng;
  if (!pts || !w) return AFAR_OK;
  for (int f = 0; f < m->nFaces; ++f) {
    const int a = m->facePoints[2 * f], b = m->facePoints[2 * f + 1];
    const double xa = m->points[2 * a], ya = m->points[2 * a + 1];
    const double xb = m->points[2 * b], yb = m->points[2 * b + 1];
    const double jac = std::sqrt((0.5 * (xa - xb)) * (0.5 * (xa - xb)) + (0.5 * (ya - yb)) * (0.5 * (ya - yb)));
    for (int k = 0; k < ng; ++k) {
      const double xi = sp[k];
      pts[2 * ((size_t)f * ng + k)] = 0.5 * xa * (1 - xi) + 0.5 * xb * (1 + xi);
      pts[2 * ((size_t)f * ng + k) + 1] = 0.5 * ya * (1 - xi) + 0.5 * yb * (1 + xi);
      w[(size_t)f * ng + k] = sw[k] * jac * m->depth;
    }
  }
  return AFAR_OK;
}

extern "C" afar_status afar_gauss_quadrature(const afar_polyMesh* m, const afar_caseConfig* cfg, int* offsets,
                                             double* pts, double* w, int* total) {
  if (!check_mesh(m) || !cfg || !total) {
    if (!cfg || !total) set_error("afar_gauss_quadrature: null argument");
    return AFAR_ERR_ARGUMENT;
  }
  Geom g;
  if (!compute_geometry(m, g)) return AFAR_ERR_MESH;
  const int nc = m->nCells, nb = m->nFaces - m->nInternalFaces;
  std::vector<Pt> gp;
  std::vector<double> gw;
  int n = 0;
  for (int i = 0; i < nc + nb; ++i) {
    if (i < nc)
      cell_gauss(m, g, i, cfg->cOrder, gp, gw);
    else
      face_gauss(m, m->nInternalFaces + (i - nc), cfg->fOrder, gp, gw);
    if (gp.empty()) {
      set_error("no Gauss rule stored for cOrder=%d / fOrder=%d", cfg->cOrder, cfg->fOrder);
      return AFAR_ERR_ARGUMENT;
    }
    if (offsets) offsets[i] = n;
    if (pts && w)
      for (size_t k = 0; k < gp.size(); ++k) {
        pts[2 * (n + k)] = gp[k].x;
        pts[2 * (n + k) + 1] = gp[k].y;
        w[n + k] = gw[k];
      }
    n += (int)gp.size();
  }
  if (offsets) offsets[nc + nb] = n;
  *total = n;
  return AFAR_OK;
}

extern "C" void afar_free_host_fields(afar_fieldPointer* h) {
  if (!h) return;
  void** members[] = {(void**)&h->CELL, (void**)&h->FACE, (void**)&h->cellVolume, (void**)&h->FD, (void**)&h->limiter,
                      (void**)&h->shockIndicator, (void**)&h->cFD, (void**)&h->cFDold, (void**)&h->gradFD,
                      (void**)&h->Flux, (void**)&h->Res, (void**)&h->neighbour, (void**)&h->boundaryFacesNum,
                      (void**)&h->boundaryFaceNeiLabel, (void**)&h->boundaryFacesType, (void**)&h->stencilSize,
                      (void**)&h->compactStencilSize, (void**)&h->RBFbasis, (void**)&h->faceFD,
                      (void**)&h->extendStencil, (void**)&h->extendStencilSize,
                      (void**)&h->compactExtendStencilSize, (void**)&h->localStencil, (void**)&h->matrix,
                      (void**)&h->cellFaces, (void**)&h->minDeltaT};
  for (void** p : members) {
    std::free(*p);
    *p = nullptr;
  }
}

template <class T>
static T* xalloc(size_t n) {
  T* p = static_cast<T*>(std::calloc(n > 0 ? n : 1, sizeof(T)));
  return p;
}

// The whole precompute; the RBF stage runs on CUDA device `device` when it is >= 0, else on the host.
static afar_status precompute(const afar_polyMesh* m, const afar_caseConfig* cfg, const double* Wc, const double* Wb,
                              int device, afar_fieldPointer* h, afar_fieldSizes* sz, double** rbf64_out,
                              double** gauss_out = nullptr, int* gauss_n = nullptr) {
  if (rbf64_out) *rbf64_out = nullptr;
  if (gauss_out) *gauss_out = nullptr;
  if (!check_mesh(m)) return AFAR_ERR_ARGUMENT;
  if (!cfg || !Wc || !h || !sz) {
    set_error("afar_precompute_fields: null argument");
    return AFAR_ERR_ARGUMENT;
  }
  if (cfg->stencilType != AFAR_STENCIL_FACE_NEIGHBOUR && cfg->stencilType != AFAR_STENCIL_EDGE_NEIGHBOUR) {
    set_error("Invalid stencil type setting. Valid settings are: faceNeighbour, edgeNeighbour");
    return AFAR_ERR_ARGUMENT;
  }
  {
    std::vector<Pt> tp;
    std::vector<double> tw, bp, bw;
    tri_rule(cfg->cOrder, tp, tw);
    bar_rule(cfg->fOrder, bp, bw);
    if (tp.empty() || bp.empty()) {
      set_error("No stored information for cOrder = %d / fOrder = %d", cfg->cOrder, cfg->fOrder);
      return AFAR_ERR_ARGUMENT;
    }
  }
  std::memset(h, 0, sizeof(*h));
  std::memset(sz, 0, sizeof(*sz));
  Geom g;
  if (!compute_geometry(m, g)) return AFAR_ERR_MESH;

  const int nc = m->nCells, nf = m->nInternalFaces;
  int patches = 0, nb = 0;
  for (int p = 0; p < m->nPatches; ++p)
    if (m->patchSize[p] > 0) {
      patches++;
      nb += m->patchSize[p];
    }
  const double R = cfg->R, Cv = cfg->Cv;
  const double px = m->periodX > 0.0 ? m->periodX : 0.0, py = m->periodY > 0.0 ? m->periodY : 0.0;

  // ---- initFieldInfo (basicCUDAsolver.cpp:122-258)
  h->boundaryFacesNum = xalloc<int>(patches);
  h->boundaryFaceNeiLabel = xalloc<int>(nb);
  h->boundaryFacesType = xalloc<uint8_t>(nb);
  {
    int idx = 0, tf = 0;
    for (int p = 0; p < m->nPatches; ++p) {
      if (m->patchSize[p] == 0) continue;
      h->boundaryFacesNum[idx++] = m->patchSize[p];
      for (int i = 0; i < m->patchSize[p]; ++i, ++tf) {
        h->boundaryFaceNeiLabel[tf] = m->owner[m->patchStart[p] + i];
        h->boundaryFacesType[tf] = (uint8_t)m->patchLabel[p];
      }
    }
  }
  h->CELL = xalloc<afar_meshCellData>(nc + nb);
  h->cellVolume = xalloc<double>(nc);
  h->FD = xalloc<afar_basicFieldData>(nc + nb);
  h->cFD = xalloc<afar_conservedFieldData>(nc);
  for (int i = 0; i < nc; ++i) {
    h->CELL[i] = {g.cx[i], g.cy[i]};
    h->cellVolume[i] = g.area[i] * m->depth;
    const double p = Wc[4 * i], ux = Wc[4 * i + 1], uy = Wc[4 * i + 2], T = Wc[4 * i + 3];
    h->FD[i] = {p, ux, uy, T};
    const double rho = p / (R * T);
    h->cFD[i] = {rho, rho * ux, rho * uy, rho * (Cv * T + 0.5 * (ux * ux + uy * uy))};
  }
  for (int b = 0; b < nb; ++b) {
    const int f = nf + b;
    h->CELL[nc + b] = {g.fx[f], g.fy[f]};
    if (Wb)
      h->FD[nc + b] = {Wb[4 * b], Wb[4 * b + 1], Wb[4 * b + 2], Wb[4 * b + 3]};
    else
      h->FD[nc + b] = h->FD[h->boundaryFaceNeiLabel[b]];
  }
  h->FACE = xalloc<afar_meshFaceData>(nf + nb);
  for (int f = 0; f < nf + nb; ++f) h->FACE[f] = {g.fx[f], g.fy[f], g.magsf[f], g.sfx[f], g.sfy[f]};

  // ---- adjacency (basicCUDAsolver.cpp:269-299)
  h->neighbour = xalloc<int>(2 * (size_t)nf);
  std::vector<int> cf_off(nc + 1, 0);
  for (int f = 0; f < nf; ++f) {
    cf_off[m->owner[f] + 1]++;
    cf_off[m->neighbour[f] + 1]++;
  }
  for (int b = 0; b < nb; ++b) cf_off[h->boundaryFaceNeiLabel[b] + 1]++;
  for (int c = 0; c < nc; ++c) cf_off[c + 1] += cf_off[c];
  std::vector<int> cf(cf_off[nc]), cc(cf_off[nc]);
  {
    std::vector<int> fill(cf_off.begin(), cf_off.end() - 1);
    for (int f = 0; f < nf; ++f) {
      const int o = m->owner[f], n = m->neighbour[f];
      h->neighbour[2 * f] = o;
      h->neighbour[2 * f + 1] = n;
      cf[fill[o]] = f + 1;
      cc[fill[o]++] = n;
      cf[fill[n]] = -(f + 1);
      cc[fill[n]++] = o;
    }
    for (int b = 0; b < nb; ++b) {
      const int c = h->boundaryFaceNeiLabel[b];
      cf[fill[c]] = nf + b + 1;
      cc[fill[c]++] = nc + b;
    }
  }

  // point -> cells (for the edge-neighbour stencil)
  std::vector<int> pc_off, pc;
  if (cfg->stencilType == AFAR_STENCIL_EDGE_NEIGHBOUR) {
    pc_off.assign(m->nPoints + 1, 0);
    for (int c = 0; c < nc; ++c)
      for (int k = m->cellPointsOffset[c]; k < m->cellPointsOffset[c + 1]; ++k) pc_off[point_id(m, m->cellPoints[k]) + 1]++;
    for (int p = 0; p < m->nPoints; ++p) pc_off[p + 1] += pc_off[p];
    pc.resize(pc_off[m->nPoints]);
    std::vector<int> fill(pc_off.begin(), pc_off.end() - 1);
    for (int c = 0; c < nc; ++c)  // ascending cell order within each point
      for (int k = m->cellPointsOffset[c]; k < m->cellPointsOffset[c + 1]; ++k)
        pc[fill[point_id(m, m->cellPoints[k])]++] = c;
  }

#ifdef _OPENMP
  const int nthreads = cfg->nThreads > 0 ? cfg->nThreads : omp_get_max_threads();
#endif
  // ---- stencils (basicCUDAsolver.cpp:303-398); cells are independent
  const int MAXV = AFAR_MAX_VALID_STENCIL_SIZE;
  std::vector<int> sten((size_t)MAXV * nc, 0);
  h->stencilSize = xalloc<uint8_t>(nc);
  h->compactStencilSize = xalloc<uint8_t>(nc);
  int maxS = 0, maxM = 0;
  int too_large = nc, too_large_size = 0;  // the first cell over the limit, as a serial walk reports it
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4096) num_threads(nthreads) reduction(max : maxS, maxM)
#endif
  for (int c = 0; c < nc; ++c) {
    int tmp[64];
    int idx = 0;
    auto added = [&](int id) {
      if (id == c) return true;
      for (int k = 0; k < idx; ++k)
        if (tmp[k] == id) return true;
      return false;
    };
    auto push = [&](int id) -> bool {
      if (idx >= 64) return false;
      tmp[idx++] = id;
      return true;
    };
    const int m0 = cf_off[c + 1] - cf_off[c];
    for (int k = cf_off[c]; k < cf_off[c + 1]; ++k) push(cc[k]);
    if (cfg->stencilType == AFAR_STENCIL_FACE_NEIGHBOUR) {
      for (int k = cf_off[c]; k < cf_off[c + 1]; ++k) {
        const int fn = cc[k];
        if (fn >= nc) continue;
        for (int l = cf_off[fn]; l < cf_off[fn + 1]; ++l)
          if (!added(cc[l])) push(cc[l]);
      }
    } else {
      for (int k = m->cellPointsOffset[c]; k < m->cellPointsOffset[c + 1]; ++k) {
        const int p = point_id(m, m->cellPoints[k]);
        for (int l = pc_off[p]; l < pc_off[p + 1]; ++l)
          if (!added(pc[l])) push(pc[l]);
      }
    }
    maxS = std::max(maxS, idx);
    maxM = std::max(maxM, m0);
    if (idx > MAXV) {
#ifdef _OPENMP
#pragma omp critical(afar_stencil_limit)
#endif
      if (c < too_large) {
        too_large = c;
        too_large_size = idx;
      }
      continue;
    }
    for (int k = 0; k < idx; ++k) sten[(size_t)MAXV * c + k] = tmp[k];
    h->stencilSize[c] = (uint8_t)idx;
    h->compactStencilSize[c] = (uint8_t)m0;
  }
  if (too_large < nc) {
    set_error("Too large stencil! maxStencilSize = %d (cell %d, limit %d)", too_large_size, too_large, MAXV);
    afar_free_host_fields(h);
    return AFAR_ERR_LIMIT;
  }
  h->cellFaces = xalloc<int>((size_t)maxM * nc);
  std::vector<int> gsten((size_t)maxS * nc, 0);
  for (int c = 0; c < nc; ++c) {
    for (int i = 0; i < h->compactStencilSize[c]; ++i) h->cellFaces[(size_t)maxM * c + i] = cf[cf_off[c] + i];
    for (int i = 0; i < h->stencilSize[c]; ++i) gsten[(size_t)maxS * c + i] = sten[(size_t)MAXV * c + i];
  }
  std::vector<int>().swap(sten);

  // ---- Gauss quadrature of cells and boundary faces (basicCUDAsolver.cpp:420-457)
  // (point counts from the rule sizes, then every member filled independently)
  std::vector<int> gq_off(nc + nb + 1, 0);
  std::vector<Pt> gq_p;
  std::vector<double> gq_w;
  {
    std::vector<Pt> rp;
    std::vector<double> rw;
    tri_rule(cfg->cOrder, rp, rw);
    const int ntri = (int)rp.size();
    rec_rule(cfg->cOrder, rp, rw);
    const int nquad = (int)rp.size();
    std::vector<double> bp;
    bar_rule(cfg->fOrder, bp, rw);
    const int nbar = (int)bp.size();
    for (int i = 0; i < nc + nb; ++i) {
      const int cnt = i < nc ? (m->cellPointsOffset[i + 1] - m->cellPointsOffset[i] == 3 ? ntri : nquad) : nbar;
      gq_off[i + 1] = gq_off[i] + cnt;
    }
    gq_p.resize(gq_off[nc + nb]);
    gq_w.resize(gq_off[nc + nb]);
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
      std::vector<Pt> tp;
      std::vector<double> tw;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4096)
#endif
      for (int i = 0; i < nc + nb; ++i) {
        if (i < nc)
          cell_gauss(m, g, i, cfg->cOrder, tp, tw);
        else
          face_gauss(m, nf + (i - nc), cfg->fOrder, tp, tw);
        for (size_t k = 0; k < tp.size() && gq_off[i] + (int)k < gq_off[i + 1]; ++k) {
          gq_p[gq_off[i] + k] = tp[k];
          gq_w[gq_off[i] + k] = tw[k];
        }
      }
    }
  }

  const int nmax = maxS + 1;
  const size_t rstride = 2 * (size_t)nmax;
  h->RBFbasis = xalloc<float>(rstride * nf);
  double* rbf64 = rbf64_out ? xalloc<double>(rstride * nf) : nullptr;
  if (device >= 0) {  // the RBF stage on the GPU, bit-identical to the host stage below
    const RbfInputs in{nc, nf, nb, maxS, h->stencilSize, gsten.data(), h->CELL, h->FACE, h->neighbour,
                       gq_off.data(), reinterpret_cast<const double*>(gq_p.data()), gq_w.data(), px, py,
                       cfg->shapeFactor};
    const afar_status st = rbf_stage_device(device, in, h->RBFbasis, rbf64);
    if (st != AFAR_OK) {
      afar_free_host_fields(h);
      std::free(rbf64);
      return st;
    }
  }
  // ---- RBF P matrices, pseudo-inverses, trouble flags (basicCUDAsolver.cpp:461-533): on the host
  // for the host stage, and for the face Gauss-point weights when they are asked for
  std::vector<double> refd;
  std::vector<double> Gall;
  std::vector<char> trouble;
  const double shape = cfg->shapeFactor;
  const afar_meshCellData* CELL = h->CELL;
  auto build_inverses = [&]() {
  refd.assign(nc, 0.0);
  Gall.assign((size_t)nc * nmax * nmax, 0.0);
  trouble.assign(nc, 0);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
#endif
  for (int c = 0; c < nc; ++c) {
    const int S = h->stencilSize[c];
    const int n = S + 1;
    const int* st = &gsten[(size_t)maxS * c];
    double rd = 0.0;
    for (int i = 0; i < S; ++i) {
      const double dx = wrapd(CELL[st[i]].x - CELL[c].x, px), dy = wrapd(CELL[st[i]].y - CELL[c].y, py);
      rd += std::sqrt(dx * dx + dy * dy);
    }
    rd /= double(S);
    refd[c] = rd;
    double P[(AFAR_MAX_VALID_STENCIL_SIZE + 1) * (AFAR_MAX_VALID_STENCIL_SIZE + 1)];
    for (int i = 0; i < n; ++i) {
      const int si = i == 0 ? c : st[i - 1];
      for (int j = 0; j < n; ++j) {
        const int sj = j == 0 ? c : st[j - 1];
        const double x0 = CELL[sj].x, y0 = CELL[sj].y;
        double acc = 0.0;
        for (int k = gq_off[si]; k < gq_off[si + 1]; ++k) {
          const double ex = wrapd(gq_p[k].x - x0, px) / rd, ey = wrapd(gq_p[k].y - y0, py) / rd;
          acc += gq_w[k] * std::sqrt(shape + (ex * ex + ey * ey));
        }
        P[i * n + j] = acc;
      }
    }
    double* G = &Gall[(size_t)c * nmax * nmax];
    if (!lu_inverse(n, P, G)) svd_pinv(n, P, G);  // the reference inverts with SVDinv
    for (int i = 0; i < n * n; ++i)
      if (!(std::fabs(G[i]) <= 1e10)) {
        trouble[c] = 1;
        break;
      }
  }
  };
  // The O3 weights of cell c at point (x, y): (G^T b) corrected to sum to one, b the multiquadric
  // basis of the stencil at the point (basicCUDAsolver.cpp:585-619); a troubled cell's weights
  // select the cell itself.  n = stencil size + 1 values into out.
  auto o3_weights = [&](const int c, const double x, const double y, double* out) {
    const int n = h->stencilSize[c] + 1;
    if (trouble[c]) {
      out[0] = 1.0;
      for (int i = 1; i < n; ++i) out[i] = 0.0;
      return;
    }
    const int* st = &gsten[(size_t)maxS * c];
    const double rd = refd[c];
    double bvec[AFAR_MAX_VALID_STENCIL_SIZE + 1];
    for (int i = 0; i < n; ++i) {
      const int si = i == 0 ? c : st[i - 1];
      const double ex = wrapd(x - CELL[si].x, px) / rd, ey = wrapd(y - CELL[si].y, py) / rd;
      bvec[i] = std::sqrt(shape + (ex * ex + ey * ey));
    }
    const double* G = &Gall[(size_t)c * nmax * nmax];
    double sum = 0.0;
    for (int i = 0; i < n; ++i) {  // (G^T b)_i = sum_j G(j,i) b_j
      double acc = 0.0;
      for (int j = 0; j < n; ++j) acc += G[j * n + i] * bvec[j];
      out[i] = acc;
      sum += acc;
    }
    for (int i = 0; i < n; ++i) out[i] = out[i] - sum / double(n) + 1.0 / double(n);
  };
  if (device < 0) {
  build_inverses();

  // ---- O3 face weights (basicCUDAsolver.cpp:538-619), stored as float
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads)
#endif
  for (int f = 0; f < nf; ++f) {
    const double x = h->FACE[f].x, y = h->FACE[f].y;
    for (int side = 0; side < 2; ++side) {
      const int c = h->neighbour[2 * f + side];
      const int n = h->stencilSize[c] + 1;
      float* out = &h->RBFbasis[rstride * f + side * nmax];
      double* out64 = rbf64 ? &rbf64[rstride * f + side * nmax] : nullptr;
      if (trouble[c]) {
        out[0] = 1.0f;
        for (int i = 1; i < n; ++i) out[i] = 0.0f;
        if (out64) {
          out64[0] = 1.0;
          for (int i = 1; i < n; ++i) out64[i] = 0.0;
        }
        continue;
      }
      const int* st = &gsten[(size_t)maxS * c];
      const double rd = refd[c];
      double bvec[AFAR_MAX_VALID_STENCIL_SIZE + 1], gtb[AFAR_MAX_VALID_STENCIL_SIZE + 1];
      for (int i = 0; i < n; ++i) {
        const int si = i == 0 ? c : st[i - 1];
        const double ex = wrapd(x - CELL[si].x, px) / rd, ey = wrapd(y - CELL[si].y, py) / rd;
        bvec[i] = std::sqrt(shape + (ex * ex + ey * ey));
      }
      const double* G = &Gall[(size_t)c * nmax * nmax];
      double sum = 0.0;
      for (int i = 0; i < n; ++i) {  // (G^T b)_i = sum_j G(j,i) b_j
        double acc = 0.0;
        for (int j = 0; j < n; ++j) acc += G[j * n + i] * bvec[j];
        gtb[i] = acc;
        sum += acc;
      }
      for (int i = 0; i < n; ++i) {
        const double wi = gtb[i] - sum / double(n) + 1.0 / double(n);
        out[i] = (float)wi;
        if (out64) out64[i] = wi;
      }
    }
  }
  }
  if (gauss_out) {
    // ---- O3 weights at the face Gauss points (the optional multi-point face flux): the fOrder
    // bar rule on each internal face (d2GaussQuadrature.C:153-214), the weights of both sides'
    // stencils at every point, [face][side][point][maxS+1]
    if (Gall.empty()) build_inverses();
    std::vector<double> bp, bw;
    bar_rule(cfg->fOrder, bp, bw);
    const int ng = (int)bp.size();
    double* gw = xalloc<double>((size_t)nf * 2 * ng * nmax);
    if (!gw) {
      set_error("out of host memory for the face Gauss-point weights");
      afar_free_host_fields(h);
      std::free(rbf64);
      return AFAR_ERR_LIMIT;
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1024) num_threads(nthreads)
#endif
    for (int f = 0; f < nf; ++f) {
      const int a = m->facePoints[2 * f], b = m->facePoints[2 * f + 1];
      const double xa = m->points[2 * a], ya = m->points[2 * a + 1];
      const double xb = m->points[2 * b], yb = m->points[2 * b + 1];
      for (int side = 0; side < 2; ++side)
        for (int k = 0; k < ng; ++k) {
          const double xi = bp[k];
          const double x = 0.5 * xa * (1 - xi) + 0.5 * xb * (1 + xi), y = 0.5 * ya * (1 - xi) + 0.5 * yb * (1 + xi);
          o3_weights(h->neighbour[2 * f + side], x, y, &gw[(((size_t)f * 2 + side) * ng + k) * nmax]);
        }
    }
    *gauss_out = gw;
    if (gauss_n) *gauss_n = ng;
  }
  std::vector<double>().swap(Gall);

  // ---- 128-cell block halo remap (basicCUDAsolver.cpp:697-850)
  const int BD = AFAR_BLOCKDIM;
  const int nblk = (nc + BD - 1) / BD;
  const int maxValidLB = (int)((AFAR_MAX_SHARED_MEMORY_SIZE - sizeof(double) * BD * 4 - sizeof(float) * BD * 2 -
                                sizeof(uint16_t) * BD * maxS - sizeof(uint8_t) * BD) /
                               sizeof(int8_t));
  h->extendStencilSize = xalloc<uint16_t>(nblk);
  h->compactExtendStencilSize = xalloc<uint16_t>(nblk);
  std::vector<std::vector<int>> ext(nblk);
  int maxLB = 0, maxCLB = 0;
  // membership of a cell id in the current block's halo list, in O(1): seen[id] == blk, at where[id]
  int max_id = nc;
  for (size_t k = 0; k < (size_t)maxS * nc; ++k) max_id = std::max(max_id, gsten[k] + 1);
  std::vector<int> seen(max_id, -1), where(max_id, 0);
  for (int blk = 0; blk < nblk; ++blk) {
    std::vector<int>& e = ext[blk];
    auto outside = [&](int id) { return id < blk * BD || id > BD - 1 + blk * BD || id >= nc; };
    auto add = [&](int id) {  // first occurrence order, as the reference's list
      if (seen[id] == blk) return;
      seen[id] = blk;
      where[id] = (int)e.size();
      e.push_back(id);
    };
    for (int t = 0; t < BD; ++t) {
      const int c = t + blk * BD;
      if (c >= nc) break;
      for (int i = 0; i < h->compactStencilSize[c]; ++i) {
        const int id = gsten[(size_t)maxS * c + i];
        if (outside(id)) add(id);
      }
    }
    h->compactExtendStencilSize[blk] = (uint16_t)e.size();
    maxCLB = std::max(maxCLB, (int)e.size() + BD);
    for (int t = 0; t < BD; ++t) {
      const int c = t + blk * BD;
      if (c >= nc) break;
      for (int i = h->compactStencilSize[c]; i < h->stencilSize[c]; ++i) {
        const int id = gsten[(size_t)maxS * c + i];
        if (outside(id)) add(id);
      }
    }
    h->extendStencilSize[blk] = (uint16_t)e.size();
    maxLB = std::max(maxLB, (int)e.size() + BD);
    if (maxLB > maxValidLB) {
      set_error("Too large local block stencil size. maxLocalBlockStencilSize = %d (limit %d); renumber the cells (RCM)",
                maxLB, maxValidLB);
      afar_free_host_fields(h);
      std::free(rbf64);
      return AFAR_ERR_LIMIT;
    }
  }
  h->localStencil = xalloc<uint16_t>((size_t)maxS * nc);
  h->extendStencil = xalloc<int>((size_t)(maxLB - BD) * nblk);
  for (int blk = 0; blk < nblk; ++blk) {
    const std::vector<int>& e = ext[blk];
    for (size_t i = 0; i < e.size(); ++i) {
      h->extendStencil[(size_t)(maxLB - BD) * blk + i] = e[i];
      where[e[i]] = (int)i;
    }
    for (int t = 0; t < BD; ++t) {
      const int c = t + blk * BD;
      if (c >= nc) break;
      for (int i = 0; i < h->stencilSize[c]; ++i) {
        const int sid = gsten[(size_t)maxS * c + i];
        const bool out = sid < blk * BD || sid > BD - 1 + blk * BD || sid >= nc;
        int loc;
        if (out) {
          loc = BD + where[sid];
        } else {
          loc = sid - blk * BD;
        }
        h->localStencil[(size_t)maxS * c + i] = (uint16_t)loc;
      }
    }
  }
  const size_t smem1 = sizeof(double) * maxCLB * 2 + sizeof(float) * maxLB * 4 + sizeof(uint16_t) * BD * maxS + sizeof(uint8_t) * BD * 2;
  const size_t smem2 = sizeof(double) * BD * 4 + sizeof(float) * BD * 2 + sizeof(uint16_t) * BD * maxS + sizeof(uint8_t) * BD + sizeof(int8_t) * maxLB;
  if (smem1 > AFAR_MAX_SHARED_MEMORY_SIZE || smem2 > AFAR_MAX_SHARED_MEMORY_SIZE) {
    set_error("Too large shared memory consumption! reconstruct %zu B, BVDindicator %zu B (limit %d)", smem1, smem2,
              AFAR_MAX_SHARED_MEMORY_SIZE);
    afar_free_host_fields(h);
    std::free(rbf64);
    return AFAR_ERR_LIMIT;
  }

  // the remaining members the reference allocates on the host
  h->shockIndicator = xalloc<int8_t>(2 * (size_t)(nc + nb));
  h->minDeltaT = xalloc<double>((nf + 1023) / 1024);

  sz->cellsNum = nc;
  sz->facesNum = nf;
  sz->patchesNum = patches;
  sz->totalBoundaryFacesNum = nb;
  sz->maxStencilSize = maxS;
  sz->maxCompactStencilSize = maxM;
  sz->maxLocalBlockStencilSize = maxLB;
  sz->maxCompactLocalBlockStencilSize = maxCLB;
  if (rbf64_out) *rbf64_out = rbf64;
  return AFAR_OK;
}

extern "C" afar_status afar_precompute_fields(const afar_polyMesh* m, const afar_caseConfig* cfg, const double* Wc,
                                              const double* Wb, afar_fieldPointer* h, afar_fieldSizes* sz,
                                              double** rbf64_out) {
  return precompute(m, cfg, Wc, Wb, -1, h, sz, rbf64_out);
}

extern "C" afar_status afar_precompute_fields_device(const afar_polyMesh* m, const afar_caseConfig* cfg,
                                                     const double* Wc, const double* Wb, int device,
                                                     afar_fieldPointer* h, afar_fieldSizes* sz, double** rbf64_out) {
  if (device < 0) {
    set_error("afar_precompute_fields_device: device %d", device);
    return AFAR_ERR_ARGUMENT;
  }
  return precompute(m, cfg, Wc, Wb, device, h, sz, rbf64_out);
}

extern "C" afar_status afar_precompute_fields_gauss(const afar_polyMesh* m, const afar_caseConfig* cfg,
                                                   const double* Wc, const double* Wb, int device,
                                                   afar_fieldPointer* h, afar_fieldSizes* sz, double** rbf64_out,
                                                   double** gaussWeights, int* pointsPerFace) {
  if (!gaussWeights || !pointsPerFace) {
    set_error("afar_precompute_fields_gauss: null output");
    return AFAR_ERR_ARGUMENT;
  }
  return precompute(m, cfg, Wc, Wb, device, h, sz, rbf64_out, gaussWeights, pointsPerFace);
}
