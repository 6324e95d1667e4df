/*
 * afar_oracle.h - CPU restatement of the reference's per-stage AFAR residual + SSP-RK3 update.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU path is compared against; the product
 * (libafar) never calls it.  It consumes the reference's host field layout (include/afar.h
 * afar_fieldPointer) and follows the reference's device kernels statement by statement:
 *
 *   oracle_ls_matrix        cudaFieldOperation.h:51-121   (calcLeastSquareMatrix)
 *   oracle_reconstruct_*    cudaLimiter.h:35-50, 53-316   (limiterProcess, reconstruct)
 *   oracle_bvd_*            cudaLimiter.h:9-32, 319-464   (limiter maps, BVDindicator)
 *   oracle_flux_*           cudaRiemannSolver.h:7-271     (minimizeDeltaValue, KFVS, Roe, evaluateFlux)
 *   oracle_residual         cudaFieldOperation.h:183-207  (evaluateResidual)
 *   oracle_update           cudaFieldOperation.h:210-250  (updateFieldData)
 *   oracle_boundary         cudaEulerBCs.h:42-95, BCs/2D/<label>.h (updateBoundaryFieldData)
 *   oracle_delta_t          cudaFieldOperation.h:124-180 + GPUevolve.cu:177-204 (setDeltaT, adjustTimeStep)
 *   oracle_evolve_*         GPUevolve.cu:207-306          (GPUevolve)
 *
 * Two precision policies: _ref keeps the reference's float/double casts; _fp64 computes every
 * quantity in double (limiters, weights, dissipation with erfc/exp).  Loops over cells and faces
 * run under OpenMP; every output element is written by one iteration, so results do not depend
 * on the thread count.  Built with -ffp-contract=off.
 */
#ifndef AFAR_ORACLE_H
#define AFAR_ORACLE_H

#include <stdint.h>

#include "../include/afar.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Mesh and operator arrays of one case.  gsten holds global stencil indices (maxS per cell),
 * resolved from the block-local localStencil/extendStencil by oracle_resolve_stencil. */
typedef struct {
  int Nc, Nf, Nb, maxS, maxM;
  const afar_meshCellData* CELL;  /* Nc+Nb */
  const afar_meshFaceData* FACE;  /* Nf+Nb */
  const double* V;                /* Nc */
  const int* neighbour;           /* 2Nf */
  const int* bnei;                /* Nb  owner cell of each boundary face */
  const uint8_t* btype;           /* Nb  cudaEulerBCs label */
  const uint8_t* S;               /* Nc  stencil size */
  const uint8_t* M;               /* Nc  compact stencil size */
  const int* cellFaces;           /* maxM*Nc */
  const int* gsten;               /* maxS*Nc */
  const float* rbf32;             /* 2(maxS+1)Nf, _ref policy */
  const double* rbf64;            /* 2(maxS+1)Nf, _fp64 policy */
  const float* mat32;             /* 2 maxM Nc,   _ref policy */
  const double* mat64;            /* 2 maxM Nc,   _fp64 policy */
} oracle_mesh;

/* localStencil (block-local, 128-cell blocks) -> global indices. */
void oracle_resolve_stencil(int Nc, int maxS, int maxLB, const uint8_t* S, const uint16_t* localStencil,
                            const int* extendStencil, int* gsten);

/* calcLeastSquareMatrix in double; writes both the double and the float-rounded matrix. */
void oracle_ls_matrix(const oracle_mesh* m, double* mat64, float* mat32);

/* One stage piece each.  Limiter arrays: float[4Nc] for _ref, double[4Nc] for _fp64.
 * grad: 8 doubles per cell; faceFD: 4 doubles per face side (2Nf); si: shock indicator 2(Nc+Nb). */
void oracle_reconstruct_ref(const oracle_mesh* m, const double* FD, double* grad, float* lim, double* faceFD, int8_t* si);
void oracle_bvd_ref(const oracle_mesh* m, const double* FD, const double* grad, float* lim, const double* faceFD, int8_t* si);
void oracle_flux_ref(const oracle_mesh* m, const double* FD, const double* grad, const float* lim, const double* faceFD,
                     const int8_t* si, double R, double Cv, double* Flux);
void oracle_reconstruct_fp64(const oracle_mesh* m, const double* FD, double* grad, double* lim, double* faceFD, int8_t* si);
void oracle_bvd_fp64(const oracle_mesh* m, const double* FD, const double* grad, double* lim, const double* faceFD, int8_t* si);
void oracle_flux_fp64(const oracle_mesh* m, const double* FD, const double* grad, const double* lim, const double* faceFD,
                      const int8_t* si, double R, double Cv, double* Flux);

void oracle_residual(const oracle_mesh* m, const double* Flux, double* Res);
void oracle_update(const oracle_mesh* m, double* FD, double* cFD, const double* cFDold, double* Res, double R,
                   double gamma, double dt, double b1, double b2, double b3);
void oracle_boundary(const oracle_mesh* m, double* FD, double R, double Cv);
double oracle_delta_t(const oracle_mesh* m, const double* FD, double R, double Cv, double CFL);

/* Scratch for one evolve: sized by oracle_work_bytes. */
typedef struct {
  double* grad;    /* 8 Nc */
  void* lim;       /* 4 Nc floats (_ref) or doubles (_fp64) */
  double* faceFD;  /* 8 Nf */
  double* Flux;    /* 4 (Nf+Nb) */
  double* Res;     /* 4 Nc, zero on entry */
} oracle_work;

/* GPUevolve: three RK stages then cFDold <- cFD.  si: 2(Nc+Nb), ghosts stay 0.
 * exactRK != 0 uses exact 1/3, 2/3 instead of the reference's 0.333333/0.666667. */
void oracle_evolve_ref(const oracle_mesh* m, double* FD, double* cFD, double* cFDold, int8_t* si, oracle_work* w,
                       double R, double Cv, double dt, int exactRK);
void oracle_evolve_fp64(const oracle_mesh* m, double* FD, double* cFD, double* cFDold, int8_t* si, oracle_work* w,
                        double R, double Cv, double dt, int exactRK);

/* The optional multi-point face flux of the library (fp64 policy; no counterpart in the reference,
 * whose flux uses the face centre).  ng points per internal face: gpts [Nf][ng][2] their
 * coordinates, gw [ng] their weights normalised to sum to one, rbfg [Nf][2][ng][maxS+1] the O3
 * weights of each side's stencil at each point.  oracle_reconstruct_gauss_fp64 writes the face
 * values at the points, faceFDg [2Nf][ng][4], with the selection rules of the face-centre values
 * (O3 where a variable varies over the compact stencil, else its unlimited linear value; every
 * variable linear in a cell of flat temperature); oracle_flux_gauss_fp64 sums the flux of every
 * point times its weight, each with the switch of its cells (TVD states extrapolated to the point
 * with the cell's limited gradient); boundary faces as oracle_flux_fp64. */
void oracle_reconstruct_gauss_fp64(const oracle_mesh* m, const double* FD, const double* grad, int ng,
                                   const double* rbfg, const double* gpts, double* faceFDg);
void oracle_flux_gauss_fp64(const oracle_mesh* m, const double* FD, const double* grad, const double* lim,
                            const double* faceFDg, const int8_t* si, int ng, const double* gpts, const double* gw,
                            double R, double Cv, double* Flux);
/* oracle_evolve_fp64 with the multi-point face flux; faceFDg: scratch of 8*ng*Nf doubles. */
void oracle_evolve_gauss_fp64(const oracle_mesh* m, double* FD, double* cFD, double* cFDold, int8_t* si,
                              oracle_work* w, double R, double Cv, double dt, int ng, const double* rbfg,
                              const double* gpts, const double* gw, double* faceFDg);

int oracle_max_threads(void);
void oracle_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
