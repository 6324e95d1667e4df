/* afar_oracle.c - CPU restatement of the reference AFAR stage (test infrastructure only; see
 * afar_oracle.h for the file:line map).  The policy-dependent pieces live in
 * afar_oracle_stage.inc and are instantiated twice below. */
#include "afar_oracle.h"

#include <stdlib.h>
#include <string.h>
#include <tgmath.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* The reference kernels read stencil members through a per-block shared-memory table: local
 * index < 128 is cell blockIdx*128 + index, otherwise extendStencil[block][index - 128]
 * (cudaLimiter.h:91-133, basicCUDAsolver.cpp:697-830). */
void oracle_resolve_stencil(int Nc, int maxS, int maxLB, const uint8_t* S, const uint16_t* localStencil,
                            const int* extendStencil, int* gsten) {
  const int BD = AFAR_BLOCKDIM;
  for (int c = 0; c < Nc; ++c) {
    const int blk = c / BD;
    for (int i = 0; i < maxS; ++i) {
      int g = 0;
      if (i < S[c]) {
        const int loc = localStencil[(size_t)maxS * c + i];
        g = loc < BD ? blk * BD + loc : extendStencil[(size_t)(maxLB - BD) * blk + (loc - BD)];
      }
      gsten[(size_t)maxS * c + i] = g;
    }
  }
}

/* calcLeastSquareMatrix, cudaFieldOperation.h:91-120 */
void oracle_ls_matrix(const oracle_mesh* m, double* mat64, float* mat32) {
  const int Nc = m->Nc, maxS = m->maxS, maxM = m->maxM;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < Nc; ++c) {
    const int Mc = m->M[c];
    const double x0 = m->CELL[c].x, y0 = m->CELL[c].y;
    double Sxx = 0.0, Sxy = 0.0, Syy = 0.0;
    for (int i = 0; i < Mc; ++i) {
      const int j = m->gsten[(size_t)maxS * c + i];
      const double xj = m->CELL[j].x, yj = m->CELL[j].y;
      Sxx += (xj - x0) * (xj - x0);
      Sxy += (xj - x0) * (yj - y0);
      Syy += (yj - y0) * (yj - y0);
    }
    for (int i = 0; i < maxM; ++i) {
      double a = 0.0, b = 0.0;
      if (i < Mc) {
        const int j = m->gsten[(size_t)maxS * c + i];
        const double xj = m->CELL[j].x, yj = m->CELL[j].y;
        a = (Syy * (xj - x0) - Sxy * (yj - y0)) / (Sxx * Syy - Sxy * Sxy);
        b = (-Sxy * (xj - x0) + Sxx * (yj - y0)) / (Sxx * Syy - Sxy * Sxy);
      }
      if (mat64) {
        mat64[2 * (size_t)maxM * c + 2 * i] = a;
        mat64[2 * (size_t)maxM * c + 2 * i + 1] = b;
      }
      if (mat32) {
        mat32[2 * (size_t)maxM * c + 2 * i] = (float)a;
        mat32[2 * (size_t)maxM * c + 2 * i + 1] = (float)b;
      }
    }
  }
}

/* evaluateResidual, cudaFieldOperation.h:183-207: signed gather in cellFaces order. */
void oracle_residual(const oracle_mesh* m, const double* Flux, double* Res) {
  const int Nc = m->Nc, maxM = m->maxM;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < Nc; ++c) {
    double* r = Res + 4 * (size_t)c;
    for (int fi = 0; fi < m->M[c]; ++fi) {
      int f = m->cellFaces[(size_t)maxM * c + fi];
      const int dir = (f > 0) - (f < 0);
      f = abs(f) - 1;
      r[0] += dir * Flux[4 * (size_t)f + 0];
      r[1] += dir * Flux[4 * (size_t)f + 1];
      r[2] += dir * Flux[4 * (size_t)f + 2];
      r[3] += dir * Flux[4 * (size_t)f + 3];
    }
  }
}

/* updateFieldData, cudaFieldOperation.h:210-250 */
void oracle_update(const oracle_mesh* m, double* FD, double* cFD, const double* cFDold, double* Res, double R,
                   double gamma, double dt, double b1, double b2, double b3) {
  const int Nc = m->Nc;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < Nc; ++c) {
    const double* o = cFDold + 4 * (size_t)c;
    double* u = cFD + 4 * (size_t)c;
    double* r = Res + 4 * (size_t)c;
    const double V = m->V[c];
    const double rho = b1 * o[0] + b2 * u[0] + b3 * dt * (-r[0] / V);
    const double rux = b1 * o[1] + b2 * u[1] + b3 * dt * (-r[1] / V);
    const double ruy = b1 * o[2] + b2 * u[2] + b3 * dt * (-r[2] / V);
    const double rE = b1 * o[3] + b2 * u[3] + b3 * dt * (-r[3] / V);
    u[0] = rho;
    u[1] = rux;
    u[2] = ruy;
    u[3] = rE;
    double* W = FD + 4 * (size_t)c;
    W[0] = (gamma - 1.0) * (rE - 0.5 * (rux * rux + ruy * ruy) / rho);
    W[1] = rux / rho;
    W[2] = ruy / rho;
    W[3] = W[0] / (R * rho);
    r[0] = r[1] = r[2] = r[3] = 0.0;
  }
}

/* updateBoundaryFieldData + the BC table, cudaEulerBCs.h:45-95 and the six BCs/2D headers :4-10 */
void oracle_boundary(const oracle_mesh* m, double* FD, double R, double Cv) {
  const int Nc = m->Nc, Nf = m->Nf, Nb = m->Nb;
  (void)R;
  (void)Cv;
#pragma omp parallel for schedule(static)
  for (int b = 0; b < Nb; ++b) {
    const double* Wc = FD + 4 * (size_t)m->bnei[b];
    double* Wg = FD + 4 * (size_t)(Nc + b);
    const afar_meshFaceData* fc = &m->FACE[Nf + b];
    switch (m->btype[b]) {
      case 0: /* constantTemperatureWallBoundary */
        Wg[0] = Wc[0]; Wg[1] = 0.0; Wg[2] = 0.0; Wg[3] = 1.0;
        break;
      case 1: /* adiabaticWallBoundary */
        Wg[0] = Wc[0]; Wg[1] = 0.0; Wg[2] = 0.0; Wg[3] = Wc[3];
        break;
      case 2: { /* symmetryBoundary */
        const double nfx = fc->Sfx / fc->magSf, nfy = fc->Sfy / fc->magSf;
        Wg[0] = Wc[0];
        Wg[1] = Wc[1] - (Wc[1] * nfx + Wc[2] * nfy) * nfx;
        Wg[2] = Wc[2] - (Wc[1] * nfx + Wc[2] * nfy) * nfy;
        Wg[3] = Wc[3];
        break;
      }
      case 3: /* fixedValueBoundary */
        Wg[0] = 1.0; Wg[1] = 3.0; Wg[2] = 0.0; Wg[3] = 1.0;
        break;
      case 4: /* outletBoundary */
        Wg[0] = Wc[0]; Wg[1] = Wc[1]; Wg[2] = Wc[2]; Wg[3] = Wc[3];
        break;
      case 5: /* fixedValue2Boundary */
        Wg[0] = 30.05945; Wg[1] = 4.07795; Wg[2] = 0.0; Wg[3] = 5.97677;
        break;
      default: /* 6: the ghost keeps its initial state (a fixed value from the case's fields) */
        break;
    }
  }
}

/* setDeltaT kernel + host min of adjustTimeStep, cudaFieldOperation.h:140-179, GPUevolve.cu:197-203 */
double oracle_delta_t(const oracle_mesh* m, const double* FD, double R, double Cv, double CFL) {
  const int Nf = m->Nf;
  double best = 1e5;
#pragma omp parallel for schedule(static) reduction(min : best)
  for (int f = 0; f < Nf; ++f) {
    const int own = m->neighbour[2 * f], nei = m->neighbour[2 * f + 1];
    const double dR = hypot(m->CELL[nei].x - m->CELL[own].x, m->CELL[nei].y - m->CELL[own].y);
    const double frac = hypot(m->FACE[f].x - m->CELL[own].x, m->FACE[f].y - m->CELL[own].y) / dR;
    const double Sfx = m->FACE[f].Sfx, Sfy = m->FACE[f].Sfy, magSf = m->FACE[f].magSf;
    const double* Wo = FD + 4 * (size_t)own;
    const double* Wn = FD + 4 * (size_t)nei;
    const double dt = CFL * dR * magSf /
                      ((1.0 - frac) * fabs(Wo[1] * Sfx + Wo[2] * Sfy) + frac * fabs(Wn[1] * Sfx + Wn[2] * Sfy) +
                       sqrt((R / Cv + 1.0) * R * ((1.0 - frac) * Wo[3] + frac * Wn[3])) * magSf);
    if (dt < best) best = dt;
  }
  return best;
}

/* ---- policy instantiations ---- */
#define sT float
#define dT float
#define SFX(n) n##ref
#define K_(x) x##f
#define RBF m->rbf32
#define MAT m->mat32
#define PI_ 3.141593f
#include "afar_oracle_stage.inc"
#undef sT
#undef dT
#undef SFX
#undef K_
#undef RBF
#undef MAT
#undef PI_

#define sT double
#define dT double
#define SFX(n) n##fp64
#define K_(x) x
#define RBF m->rbf64
#define MAT m->mat64
#define PI_ 3.14159265358979323846
#include "afar_oracle_stage.inc"
#undef sT
#undef dT
#undef SFX
#undef K_
#undef RBF
#undef MAT
#undef PI_

/* ---- the multi-point face flux (fp64 policy of the library; see afar_oracle.h) ------------------ */
void oracle_reconstruct_gauss_fp64(const oracle_mesh* m, const double* FD, const double* grad, int ng,
                                   const double* rbfg, const double* gpts, double* faceFDg) {
  const int Nc = m->Nc, Nf = m->Nf, maxS = m->maxS, maxM = m->maxM;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < Nc; ++c) {
    const int S = m->S[c], Mc = m->M[c];
    const int* st = m->gsten + (size_t)maxS * c;
    const double* W = FD + 4 * (size_t)c;
    const double* g = grad + 8 * (size_t)c;
    /* the gradient of each variable (x, y): p (0, 1), Ux (2, 4), Uy (3, 5), T (6, 7) */
    const int gx[4] = {0, 2, 3, 6}, gy[4] = {1, 4, 5, 7};
    double vmax[4], vmin[4];
    for (int v = 0; v < 4; ++v) vmax[v] = vmin[v] = W[v];
    for (int i = 0; i < Mc; ++i)
      for (int v = 0; v < 4; ++v) {
        const double q = FD[4 * (size_t)st[i] + v];
        vmax[v] = fmax(q, vmax[v]);
        vmin[v] = fmin(q, vmin[v]);
      }
    const int flatT = fabs(vmax[3] - vmin[3]) < 1e-10;
    for (int fi = 0; fi < Mc; ++fi) {
      int f = m->cellFaces[(size_t)maxM * c + fi];
      const int isNei = f < 0;
      f = abs(f) - 1;
      if (f >= Nf) continue;
      for (int k = 0; k < ng; ++k) {
        const double dx = gpts[2 * ((size_t)f * ng + k)] - m->CELL[c].x;
        const double dy = gpts[2 * ((size_t)f * ng + k) + 1] - m->CELL[c].y;
        const double* w = rbfg + (((size_t)f * 2 + isNei) * ng + k) * (maxS + 1);
        double o3[4];
        for (int v = 0; v < 4; ++v) o3[v] = w[0] * W[v];
        for (int ci = 0; ci < S; ++ci)
          for (int v = 0; v < 4; ++v) o3[v] += w[ci + 1] * FD[4 * (size_t)st[ci] + v];
        double* o = faceFDg + ((2 * (size_t)f + isNei) * ng + k) * 4;
        for (int v = 0; v < 4; ++v) {
          const double lin = W[v] + g[gx[v]] * dx + g[gy[v]] * dy;
          o[v] = (!flatT && fabs(vmax[v] - vmin[v]) >= 1e-5) ? o3[v] : lin;
        }
      }
    }
  }
}

void oracle_flux_gauss_fp64(const oracle_mesh* m, const double* FD, const double* grad, const double* lim,
                            const double* faceFDg, const int8_t* si, int ng, const double* gpts, const double* gw,
                            double R, double Cv, double* Flux) {
  const int Nf = m->Nf;
  oracle_flux_fp64(m, FD, grad, lim, faceFDg, si, R, Cv, Flux); /* the boundary faces (internal ones rewritten) */
#pragma omp parallel for schedule(static)
  for (int f = 0; f < Nf; ++f) {
    const int cell[2] = {m->neighbour[2 * f], m->neighbour[2 * f + 1]};
    const int tvd[2] = {si[2 * (size_t)cell[0] + 1] != 0, si[2 * (size_t)cell[1] + 1] != 0};
    const int shock = si[2 * (size_t)cell[0] + 1] < 0 || si[2 * (size_t)cell[1] + 1] < 0;
    const double magSf = m->FACE[f].magSf, Sfx = m->FACE[f].Sfx, Sfy = m->FACE[f].Sfy;
    const int gx[4] = {0, 2, 3, 6}, gy[4] = {1, 4, 5, 7};
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int k = 0; k < ng; ++k) {
      double st[2][4], T[2][4], rho[2], rhoT[2];
      for (int s = 0; s < 2; ++s) {
        const int c = cell[s];
        const double dx = gpts[2 * ((size_t)f * ng + k)] - m->CELL[c].x;
        const double dy = gpts[2 * ((size_t)f * ng + k) + 1] - m->CELL[c].y;
        const double* W = FD + 4 * (size_t)c;
        const double* g = grad + 8 * (size_t)c;
        const double* L = lim + 4 * (size_t)c;
        const double* o3 = faceFDg + ((2 * (size_t)f + s) * ng + k) * 4;
        for (int v = 0; v < 4; ++v) {
          T[s][v] = W[v] + L[v] * (g[gx[v]] * dx + g[gy[v]] * dy);
          st[s][v] = tvd[s] ? T[s][v] : o3[v];
        }
        rho[s] = st[s][0] / (R * st[s][3]);
        rhoT[s] = T[s][0] / (R * T[s][3]);
      }
      const double dP = min_deltafp64(st[0][0], st[1][0], T[0][0], T[1][0]);
      const double dRho = min_deltafp64(rho[0], rho[1], rhoT[0], rhoT[1]);
      double F[4];
      F[0] = 0.5 * rho[0] * (st[0][1] * Sfx + st[0][2] * Sfy) + 0.5 * rho[1] * (st[1][1] * Sfx + st[1][2] * Sfy);
      F[1] = 0.5 * (F[0] * st[0][1] + st[0][0] * Sfx) + 0.5 * (F[0] * st[1][1] + st[1][0] * Sfx);
      F[2] = 0.5 * (F[0] * st[0][2] + st[0][0] * Sfy) + 0.5 * (F[0] * st[1][2] + st[1][0] * Sfy);
      F[3] = 0.5 * F[0] * (Cv * st[0][3] + 0.5 * (st[0][1] * st[0][1] + st[0][2] * st[0][2]) + st[0][0] / rho[0]) +
             0.5 * F[0] * (Cv * st[1][3] + 0.5 * (st[1][1] * st[1][1] + st[1][2] * st[1][2]) + st[1][0] / rho[1]);
      if (shock)
        kfvsfp64(F, rho[0], rho[1], st[0][0], st[1][0], st[0][1], st[1][1], st[0][2], st[1][2], st[0][3], st[1][3], R,
                 Cv, magSf, Sfx, Sfy);
      else
        roefp64(F, rho[0], rho[1], st[0][0], st[1][0], st[0][1], st[1][1], st[0][2], st[1][2], st[0][3], st[1][3], dP,
                dRho, R, Cv, magSf, Sfx, Sfy);
      for (int v = 0; v < 4; ++v) acc[v] += gw[k] * F[v];
    }
    for (int v = 0; v < 4; ++v) Flux[4 * (size_t)f + v] = acc[v];
  }
}

void oracle_evolve_gauss_fp64(const oracle_mesh* m, double* FD, double* cFD, double* cFDold, int8_t* si,
                              oracle_work* w, double R, double Cv, double dt, int ng, const double* rbfg,
                              const double* gpts, const double* gw, double* faceFDg) {
  const double gamma = R / Cv + 1.0;
  const double b1[3] = {1.0, 0.75, 0.333333};
  const double b2[3] = {0.0, 0.25, 0.666667};
  const double b3[3] = {1.0, 0.25, 0.666667};
  double* lim = (double*)w->lim;
  for (int k = 0; k < 3; ++k) {
    oracle_reconstruct_fp64(m, FD, w->grad, lim, w->faceFD, si);
    oracle_reconstruct_gauss_fp64(m, FD, w->grad, ng, rbfg, gpts, faceFDg);
    oracle_bvd_fp64(m, FD, w->grad, lim, w->faceFD, si);
    oracle_flux_gauss_fp64(m, FD, w->grad, lim, faceFDg, si, ng, gpts, gw, R, Cv, w->Flux);
    oracle_residual(m, w->Flux, w->Res);
    oracle_update(m, FD, cFD, cFDold, w->Res, R, gamma, dt, b1[k], b2[k], b3[k]);
    oracle_boundary(m, FD, R, Cv);
  }
  memcpy(cFDold, cFD, sizeof(double) * 4 * (size_t)m->Nc);
}
