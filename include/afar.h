/*
 * afar.h - C ABI of the GB300-native AFAR per-stage residual + SSP-RK3 solver.
 *
 * Three groups of entry points:
 *
 *  1. The reference data layout (the structs of the reference's
 *     src/CUDA/cudaEuler2DmixO3RK3/basicDataStructure.h:10-160), kept byte-for-byte so that a
 *     caller that fills the reference's host `fieldPointer` can pass the same arrays here.
 *
 *  2. The host precompute that the reference's solver object performs with OpenFOAM
 *     (basicCUDAsolver.cpp:122-851 and src/gaussQuadrature/d2GaussQuadrature.C:3-547):
 *     OpenFOAM-style polyMesh arrays in, the reference's host field bundle out.
 *
 *  3. The drop-in replacement of the reference's host<->device boundary
 *     (src/CUDA/cudaEuler2DmixO3RK3/GPUevolve.h:6-59): same arguments and meaning, but an
 *     opaque solver handle in place of the device-side fieldPointer and a status code in place
 *     of printf + std::exit.  Plus native extensions: precision policy, device-resident
 *     CFL time step, CUDA-graph stepping, per-stage parity hooks.
 *
 * Every entry point returns an afar_status; afar_last_error() returns the message of the last
 * failure on the calling thread.  Calls on one solver handle must come from one host thread.
 */
#ifndef AFAR_H
#define AFAR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------------------------- */
/* status codes                                                                                 */
/* ------------------------------------------------------------------------------------------- */
typedef enum {
  AFAR_OK = 0,
  AFAR_ERR_ARGUMENT = 1,     /* a null pointer, a size out of range, an unknown option       */
  AFAR_ERR_MESH = 2,         /* malformed mesh: bad orientation, non-2-D cell, bad patch     */
  AFAR_ERR_LIMIT = 3,        /* a compile-time limit of the reference layout is exceeded     */
  AFAR_ERR_CUDA = 4,         /* a CUDA runtime call failed                                    */
  AFAR_ERR_STATE = 5,        /* call out of order (e.g. evolve before the stencil upload)    */
  AFAR_ERR_NOT_FINITE = 6,   /* a non-finite or non-positive state was detected              */
  AFAR_ERR_CANCELLED = 7     /* a served request was cancelled before it finished            */
} afar_status;

const char* afar_last_error(void);

/* ------------------------------------------------------------------------------------------- */
/* 1. reference data layout: basicDataStructure.h:6-160                                         */
/* ------------------------------------------------------------------------------------------- */
#define AFAR_BLOCKDIM 128                 /* basicDataStructure.h:6 */
#define AFAR_MAX_SHARED_MEMORY_SIZE 49152 /* basicDataStructure.h:7 */
#define AFAR_MAX_VALID_STENCIL_SIZE 20    /* basicDataStructure.h:8 */

typedef struct { double x, y; } afar_meshCellData;                          /* :10-14  */
typedef struct { double x, y, magSf, Sfx, Sfy; } afar_meshFaceData;         /* :16-23  */
typedef struct { double p, Ux, Uy, T; } afar_basicFieldData;                /* :25-31  */
typedef struct { double rho, rhoUx, rhoUy, rhoE; } afar_conservedFieldData; /* :33-39  */
typedef struct {                                                            /* :41-49  */
  double gradPx, gradPy;
  double gradUxx, gradUxy;
  double gradUyx, gradUyy;
  double gradTx, gradTy;
} afar_gradientFieldData;
typedef struct { double rhoFlux, rhoUxFlux, rhoUyFlux, rhoEFlux; } afar_basicFluxData; /* :51-57 */
typedef struct { double Rrho, RrhoUx, RrhoUy, RrhoE; } afar_residualFieldData;         /* :59-65 */
typedef struct { float pLimiter, UxLimiter, UyLimiter, TLimiter; } afar_limiterFieldData; /* :67-73 */

/* The reference's fieldPointer (basicDataStructure.h:75-160), host side.  Sizes:
 *   CELL, FD: cellsNum + totalBoundaryFacesNum     FACE, Flux: facesNum + totalBoundaryFacesNum
 *   cellVolume, cFD, cFDold, gradFD, Res, limiter, stencilSize, compactStencilSize: cellsNum
 *   shockIndicator: 2*(cellsNum + totalBoundaryFacesNum)   neighbour, faceFD: 2*facesNum
 *   boundaryFaceNeiLabel, boundaryFacesType: totalBoundaryFacesNum   boundaryFacesNum: patchesNum
 *   RBFbasis: 2*(maxStencilSize+1)*facesNum    localStencil: maxStencilSize*cellsNum
 *   matrix: 2*maxCompactStencilSize*cellsNum   cellFaces: maxCompactStencilSize*cellsNum
 *   extendStencilSize, compactExtendStencilSize: nBlocks = ceil(cellsNum/128)
 *   extendStencil: (maxLocalBlockStencilSize - 128)*nBlocks    minDeltaT: ceil(facesNum/1024) */
typedef struct {
  afar_meshCellData* CELL;
  afar_meshFaceData* FACE;
  double* cellVolume;
  afar_basicFieldData* FD;
  afar_limiterFieldData* limiter;
  int8_t* shockIndicator;
  afar_conservedFieldData* cFD;
  afar_conservedFieldData* cFDold;
  afar_gradientFieldData* gradFD;
  afar_basicFluxData* Flux;
  afar_residualFieldData* Res;
  int* neighbour;
  int* boundaryFacesNum;
  int* boundaryFaceNeiLabel;
  uint8_t* boundaryFacesType;
  uint8_t* stencilSize;
  uint8_t* compactStencilSize;
  float* RBFbasis;
  afar_basicFieldData* faceFD;
  int* extendStencil;
  uint16_t* extendStencilSize;
  uint16_t* compactExtendStencilSize;
  uint16_t* localStencil;
  float* matrix;
  int* cellFaces;
  double* minDeltaT;
} afar_fieldPointer;

/* The integer sizes that travel beside the fieldPointer in the reference
 * (basicCUDAsolver.h members cellsNum_ ... maxCompactLocalBlockStencilSize_). */
typedef struct {
  int cellsNum;
  int facesNum;
  int patchesNum;
  int totalBoundaryFacesNum;
  int maxStencilSize;
  int maxCompactStencilSize;
  int maxLocalBlockStencilSize;
  int maxCompactLocalBlockStencilSize;
} afar_fieldSizes;

/* ------------------------------------------------------------------------------------------- */
/* 2. host precompute (replaces basicCUDAsolver::initFieldInfo + initStencilData, which need    */
/*    OpenFOAM: basicCUDAsolver.cpp:122-851; d2GaussQuadrature.C:3-547)                          */
/* ------------------------------------------------------------------------------------------- */

/* OpenFOAM-style 2-D polyMesh: the x-y cross-section of a one-cell-deep mesh.  Face f joins
 * facePoints[2f] -> facePoints[2f+1]; its normal (Sf) points out of owner[f].  Internal faces
 * come first (owner < neighbour), then the boundary faces patch by patch. */
/* Boundary labels: the reference's cudaEulerBCs labels 0-5 (cudaEulerBCs.h:56-61: constant-
 * temperature wall, adiabatic wall, slip, fixed value (1, 3, 0, 1), outlet, fixed value of the
 * cornerFlow inlet), and one more with no counterpart in the reference: the ghost state stays at
 * the value given for it at upload (afar_fieldPointer FD[cellsNum + b]), a fixed-value patch whose
 * value comes from the case's initial fields, e.g. an inflow of any Mach number. */
#define AFAR_BC_FIXED_INITIAL 6

typedef struct {
  int nPoints;
  const double* points;           /* [2*nPoints] x, y */
  int nCells;
  const int* cellPointsOffset;    /* [nCells+1] CSR offsets */
  const int* cellPoints;          /* polygon vertices of each cell (3 or 4 per cell) */
  int nInternalFaces;
  int nFaces;                     /* internal + boundary */
  const int* facePoints;          /* [2*nFaces] */
  const int* owner;               /* [nFaces] */
  const int* neighbour;           /* [nInternalFaces] */
  int nPatches;
  const int* patchStart;          /* [nPatches] first face of each patch */
  const int* patchSize;           /* [nPatches] */
  const int* patchLabel;          /* [nPatches] cudaEulerBCs label (cudaEulerBCs.h:56-61) */
  double depth;                   /* extrusion depth (cell volume = area*depth) */
  /* Periodic meshes (no counterpart in the reference, which has no periodic patch type): faces
   * that join the two sides of a period are internal faces whose points are the owner's; seam
   * points are duplicated so that every polygon has its true coordinates.  periodX/periodY > 0
   * are the periods (0: not periodic in that direction); pointAlias (may be NULL) maps each point
   * to one representative of its periodic images, for the point-based (edge-neighbour) stencils. */
  double periodX, periodY;
  const int* pointAlias;          /* [nPoints] or NULL */
} afar_polyMesh;

#define AFAR_STENCIL_FACE_NEIGHBOUR 0  /* basicCUDAsolver.cpp:333-355 */
#define AFAR_STENCIL_EDGE_NEIGHBOUR 1  /* basicCUDAsolver.cpp:356-375 */

/* The case settings the reference reads from fvSchemes/controlDict
 * (basicCUDAsolver.cpp:55-68; d2GaussQuadrature.C:12-13). */
typedef struct {
  double R;            /* CUDA.R */
  double Cv;           /* CUDA.Cv */
  double CFL;          /* controlDict maxCo */
  double shapeFactor;  /* top-level shapeFactor, default 10 */
  int stencilType;     /* AFAR_STENCIL_* */
  int cOrder;          /* gaussQuadrature.cOrder, default 5 */
  int fOrder;          /* gaussQuadrature.fOrder, default 4 */
  int nThreads;        /* host threads for the precompute; <=0: all */
} afar_caseConfig;

void afar_default_case_config(afar_caseConfig* cfg);

/* Builds the reference's host field bundle.  W_cells: [4*nCells] (p,Ux,Uy,T) initial cell values;
 * W_boundary: [4*nBoundaryFaces] initial patch values (the reference takes OpenFOAM's patch values,
 * basicCUDAsolver.cpp:189-192,231-234), or NULL to copy the owner cell's values.
 * Arrays in *host are allocated by the library; release them with afar_free_host_fields.
 * RBFbasis64 (optional, may be NULL): receives a malloc'd double copy of the O3 weights before
 * their rounding to float (2*(maxStencilSize+1)*facesNum), for the FP64 policy; free() it. */
afar_status afar_precompute_fields(const afar_polyMesh* mesh, const afar_caseConfig* cfg,
                                   const double* W_cells, const double* W_boundary,
                                   afar_fieldPointer* host, afar_fieldSizes* sizes,
                                   double** RBFbasis64);
void afar_free_host_fields(afar_fieldPointer* host);

/* afar_precompute_fields with its heaviest stage -- the RBF P matrices, their inverses and the O3
 * face weights (basicCUDAsolver.cpp:461-619) -- on CUDA device `device` (one warp per cell); every
 * other stage stays on the host.  The arrays are bit-identical to afar_precompute_fields'.  Device
 * memory used and released within the call: about (maxStencilSize+1)^2 * 8 bytes per cell plus the
 * Gauss points and the weights.  AFAR_ERR_CUDA when the device is unusable. */
afar_status afar_precompute_fields_device(const afar_polyMesh* mesh, const afar_caseConfig* cfg,
                                          const double* W_cells, const double* W_boundary, int device,
                                          afar_fieldPointer* host, afar_fieldSizes* sizes,
                                          double** RBFbasis64);

/* afar_precompute_fields (device >= 0: afar_precompute_fields_device) plus the O3 weights at the
 * face Gauss points, for the optional multi-point face flux (afar_set_face_gauss_flux; no
 * counterpart in the reference, whose flux uses the face centre).  For every internal face, each
 * side and each point of the fOrder bar rule (the points of afar_face_gauss_quadrature), the
 * weights of that side's stencil (the cell itself first) formed like the face-centre weights
 * (basicCUDAsolver.cpp:585-619: the multiquadric basis at the point times the cell's RBF inverse,
 * corrected to sum to one; a troubled cell's select the cell).  *gaussWeights is malloc'd (free()
 * it): [face][side][point][maxStencilSize+1] doubles; *pointsPerFace receives the rule's size. */
afar_status afar_precompute_fields_gauss(const afar_polyMesh* mesh, const afar_caseConfig* cfg,
                                         const double* W_cells, const double* W_boundary, int device,
                                         afar_fieldPointer* host, afar_fieldSizes* sizes, double** RBFbasis64,
                                         double** gaussWeights, int* pointsPerFace);

/* The face Gauss points and weights of every face, internal then boundary in face order (the
 * d2GaussQuadrature faceGaussPoints/faceGaussWeights layout, d2GaussQuadrature.C:153-277 and the
 * getters of d2GaussQuadrature.H:75-83): the fOrder bar rule (1, 2, 3 or 4 points) on each edge from
 * its first to its second point; each weight is the rule's weight times half the edge length times
 * the mesh depth, so a face's weights sum to |Sf|.  *pointsPerFace receives the rule's size n;
 * pts: [2*n*nFaces] (x, y of point k of face f at 2*(f*n + k)), w: [n*nFaces].  Call with pts or w
 * NULL to get n alone. */
afar_status afar_face_gauss_quadrature(const afar_polyMesh* mesh, const afar_caseConfig* cfg, int* pointsPerFace,
                                       double* pts, double* w);

/* Cell and boundary-face Gauss points/weights (d2GaussQuadrature layout) as CSR lists over
 * nCells + nBoundaryFaces members; boundary-face weights are divided by |Sf| like
 * basicCUDAsolver.cpp:444-457.  offsets: [nCells+nBoundaryFaces+1]; pts: [2*total]; w: [total].
 * Call with pts == NULL to get the total in *total. */
afar_status afar_gauss_quadrature(const afar_polyMesh* mesh, const afar_caseConfig* cfg,
                                  int* offsets, double* pts, double* w, int* total);

/* ------------------------------------------------------------------------------------------- */
/* 3. host<->device boundary: GPUevolve.h:6-59                                                  */
/* ------------------------------------------------------------------------------------------- */
typedef struct afar_solver afar_solver;

#define AFAR_POLICY_REF 0    /* the reference's own casts: float stencils/weights/limiters/dissipation */
#define AFAR_POLICY_FP64 1   /* FP64 end to end                                                       */
#define AFAR_POLICY_MIXED 2  /* FP32 reconstruction + flux, FP64 conserved accumulation and update    */

/* Creates an empty solver on a CUDA device with a precision policy. */
afar_status afar_solver_create(afar_solver** solver, int policy, int device);

/* Replaces setDeviceFieldData(devicePtr, hostPtr, cellsNum, facesNum, totalBoundaryFacesNum)
 * (GPUevolve.h:8-14, GPUevolve.cu:13-64): uploads CELL, FACE, cellVolume, FD, cFD (cFDold = cFD)
 * and zeroes the shock indicator. */
afar_status afar_setDeviceFieldData(afar_solver* solver, const afar_fieldPointer* host,
                                    int cellsNum, int facesNum, int totalBoundaryFacesNum);

/* Replaces the 10-argument setDeviceFieldData (GPUevolve.h:16-27, GPUevolve.cu:67-148):
 * uploads the stencil/operator arrays and builds the least-squares matrix on the device.  Mixed
 * policy: also encodes the TMA tensor maps of the operator rows (cuTensorMapEncodeTiled through
 * the runtime's driver entry point; AFAR_ERR_CUDA if the driver lacks it). */
afar_status afar_setDeviceFieldDataStencil(afar_solver* solver, const afar_fieldPointer* host,
                                           int cellsNum, int facesNum, int patchesNum,
                                           int totalBoundaryFacesNum, int maxStencilSize,
                                           int maxCompactStencilSize, int maxLocalBlockStencilSize,
                                           int maxCompactLocalBlockStencilSize);

/* Replaces adjustTimeStep (GPUevolve.h:31-38, GPUevolve.cu:177-204): CFL time step from the
 * current state, min over internal faces (and 1e5).  Outside a batch it computes it as the first
 * part of the coming step (stage 1 through its flux, whose reduction is this minimum), which the
 * next afar_GPUevolve on the same solver then completes; any other call in between discards it. */
afar_status afar_adjustTimeStep(afar_solver* solver, int facesNum, double R, double Cv, double CFL,
                                double* deltaT);

/* Replaces GPUevolve (GPUevolve.h:40-53, GPUevolve.cu:207-306): one SSP-RK3 step of deltaT.
 * Right after afar_adjustTimeStep it enqueues the rest of the step begun there and returns without
 * waiting (results are stream-ordered for every later call; a device-side error of the step is
 * reported by the next call that waits); otherwise it runs and waits for the whole step. */
afar_status afar_GPUevolve(afar_solver* solver, double R, double Cv, double deltaT, int cellsNum,
                           int facesNum, int totalBoundaryFacesNum, int maxStencilSize,
                           int maxCompactStencilSize, int maxLocalBlockStencilSize,
                           int maxCompactLocalBlockStencilSize);

/* Replaces copyFieldDataDeviceToHost (GPUevolve.h:56-61, GPUevolve.cu:309-318): FD and the
 * shock indicator (2 entries per cell/ghost) to host->FD and host->shockIndicator. */
afar_status afar_copyFieldDataDeviceToHost(afar_fieldPointer* host, afar_solver* solver,
                                           int cellsNum, int totalBoundaryFacesNum);

/* Replaces freeFieldData (GPUevolve.h:29, GPUevolve.cu:151-174); frees every device array and
 * the handle. */
afar_status afar_freeFieldData(afar_solver* solver);

/* ---- native extensions ---------------------------------------------------------------------- */

/* Gas constants (fvSchemes CUDA.R, CUDA.Cv) for afar_run/afar_stage_debug; afar_GPUevolve sets
 * them from its own arguments like the reference. */
afar_status afar_set_gas(afar_solver* solver, double R, double Cv);

/* The FP64 policy reads the O3 weights in double when they are given here (same layout as
 * RBFbasis, from afar_precompute_fields' RBFbasis64) before afar_setDeviceFieldDataStencil;
 * otherwise it widens the float weights. */
afar_status afar_set_rbf_basis64(afar_solver* solver, const double* RBFbasis64, size_t count);

/* Runs nSteps SSP-RK3 steps as one replay of a captured CUDA graph per step.  deltaT > 0: fixed
 * step; deltaT <= 0: CFL step computed on the device each step from (R, Cv, CFL) (the
 * adjustTimeStep + GPUevolve pair of the reference's time loop, cudaEuler2DmixO3RK3solver.cpp:53-64,
 * with no host round trip).  tEnd > 0 clips the last step to land on tEnd; steps after that are
 * no-ops.  Waits for the steps to finish and reports device errors. */
afar_status afar_run(afar_solver* solver, int nSteps, double deltaT, double CFL, double tEnd);

/* Same as afar_run but only enqueues the steps on the solver's stream (no wait). */
afar_status afar_run_async(afar_solver* solver, int nSteps, double deltaT, double CFL, double tEnd);
afar_status afar_synchronize(afar_solver* solver);

/* The solver's CUDA stream (a cudaStream_t), for event timing by the caller. */
afar_status afar_get_stream(afar_solver* solver, void** stream);

/* afar_run with CUDA events recorded on the solver's stream around the steps; *ms receives the
 * device time of the nSteps steps. */
afar_status afar_run_timed(afar_solver* solver, int nSteps, double deltaT, double CFL, double tEnd, float* ms);

/* Runs one step kernel by kernel (not as a graph) with events between the kernels and returns
 * the device time of each kind summed over the three stages: ms[0] reconstruct, ms[1] BVD switch,
 * ms[2] face flux (with the CFL kernel where the policy runs one), ms[3] gather + RK update,
 * ms[4] step bookkeeping. */
afar_status afar_profile_step(afar_solver* solver, double deltaT, double CFL, float ms[5]);

/* Simulated time, last step size and number of steps taken on the device. */
afar_status afar_get_time(afar_solver* solver, double* t, double* lastDeltaT, long long* steps);
afar_status afar_set_time(afar_solver* solver, double t);

/* Runs RK stage k (0..2) of step size deltaT and copies every intermediate of that stage, in the
 * reference layout, into the non-NULL members of *out: faceFD, gradFD, limiter (after the BVD
 * transform), shockIndicator, Flux, Res (before the update zeroes it), FD, cFD.  The parity hook
 * for per-stage comparison with the reference kernels. */
afar_status afar_stage_debug(afar_solver* solver, int stage, double deltaT, afar_fieldPointer* out);

/* The current limiter (4 per cell) widened to double: the FP64 policy keeps double limiters. */
afar_status afar_debug_limiter64(afar_solver* solver, double* limiter);

/* Overwrites the state: FD (cells + ghosts), cFD and cFDold (cells); NULL members are skipped. */
afar_status afar_upload_state(afar_solver* solver, const afar_basicFieldData* FD,
                              const afar_conservedFieldData* cFD,
                              const afar_conservedFieldData* cFDold);
afar_status afar_download_state(afar_solver* solver, afar_basicFieldData* FD,
                                afar_conservedFieldData* cFD, int8_t* shockIndicator);

/* Step control of one solver for afar_run-style stepping inside a batch: fixed deltaT (> 0) or
 * the device CFL step, and an end time (<= 0: none). */
afar_status afar_set_step_params(afar_solver* solver, double deltaT, double CFL, double tEnd);

/* Write-time landing for graph-replayed steps (afar_run, afar_run_async, batches): with
 * writeInterval > 0 the step size of each step is spread over the steps left to the next multiple
 * of writeInterval, as OpenFOAM's Time does for writeControl adjustableRunTime after the reference
 * application's runTime.setDeltaT (cudaEuler2DmixO3RK3solver.cpp:44-48; the rule: with r the time
 * to the next write, n = floor(r/dt - 1e-15) + 1 steps of r/n, held within [dt/5, 2 dt]).  Run
 * with tEnd at the write time to stop there.  0 switches it off. */
afar_status afar_set_write_interval(afar_solver* solver, double writeInterval);

/* Periods of a periodic mesh (as in its afar_polyMesh), before afar_setDeviceFieldDataStencil: the
 * device geometry (least-squares rows, face offsets, Courant distances) then takes differences
 * between cell and face centres to the nearest periodic image.  Policies fp64 and mixed. */
afar_status afar_set_periodic(afar_solver* solver, double periodX, double periodY);

/* ---- batches: many independent solves stepped by the same kernel launches ------------------- */
/* A batch steps all of its member solvers with one launch per stage kernel (13 per RK3 step,
 * replayed as one CUDA graph): every block works on one member, so meshes of uneven size share the
 * GPU without padding.  Each member keeps its own device data, time step (fixed or CFL, with its
 * own step params), end time and step count.  A member's result does not depend on which other
 * solves share its batch (bitwise); it agrees with afar_run of the same solve to the policy's
 * rounding (the batched kernels read their arguments from a device table, afar_run's from kernel
 * parameters, and the compiler may fuse a multiply-add differently in the two).  Members join and
 * leave between runs without moving their data.  Policies fp64 and mixed; all members of a batch
 * share the batch's policy and device; a solver belongs to at most one batch at a time and must
 * not be stepped on its own while it belongs to one.  Not thread-safe: one host thread per batch. */
typedef struct afar_batch afar_batch;
afar_status afar_batch_create(afar_batch** batch, int policy, int device);
afar_status afar_batch_add(afar_batch* batch, afar_solver* solver);
afar_status afar_batch_remove(afar_batch* batch, afar_solver* solver);
afar_status afar_batch_size(afar_batch* batch, int* members);
/* nSteps RK3 steps of every member; *ms (may be NULL) receives the device time (CUDA events on
 * the batch stream).  Waits for completion. */
afar_status afar_batch_run(afar_batch* batch, int nSteps, float* ms);
afar_status afar_batch_destroy(afar_batch* batch);
/* The batch's launch schedule, picked by the batch autotuner (no counterpart in the reference,
 * whose kernels run in blocks of BLOCKDIM = 128, basicDataStructure.h:6) when the batch is built
 * (its first run after members join or leave): each mixed-policy member reconstructs with the
 * tile-staged kernel, or with the register pass where its solver forces it (afar_set_tuning; so a
 * member's result never depends on its batch-mates), and the BVD and flux kernels run in the block
 * size that timed fastest on the whole batch (BVD 64, 128 or 256 cells, flux 128 or 256 faces;
 * best of three launches each), cached per device, policy and batch shape (cells and members, each
 * to a factor of two).  Block sizes do not change results.  afar_batch_get_schedule reports the
 * members on each reconstruct, the block sizes and the launch times measured (ms: BVD at 64, 128,
 * 256, flux at 128, 256; zeros when the decision came from the cache or was forced);
 * afar_batch_set_schedule forces block sizes (0: autotune). */
afar_status afar_batch_get_schedule(afar_batch* batch, int* tileMembers, int* registerMembers, int* bvdBlock,
                                    int* fluxBlock, float ms[5]);
afar_status afar_batch_set_schedule(afar_batch* batch, int bvdBlock, int fluxBlock);

/* ---- serving: a queue of solve requests on one GPU under a device-memory budget --------------- */
/* No counterpart in the reference (it runs one case per process).  A server owns a worker thread
 * that admits queued requests while their estimated device memory fits the budget (at least one
 * at a time, whatever its size), builds a solver for each, steps all admitted solves together as
 * one batch (afar_batch_*) in chunks of chunkSteps RK3 steps, and retires each solve when it
 * reaches its end time or step count: its fields are copied into the request's output buffers and
 * its device memory is freed.  Policies fp64 and mixed. */
typedef struct afar_server afar_server;
typedef struct {
  const afar_fieldPointer* host; /* precomputed host fields (afar_precompute_fields); they and */
  afar_fieldSizes sizes;         /* the output buffers must stay valid until the request is done */
  const double* RBFbasis64;      /* fp64 policy: the FP64 O3 weights (may be NULL), count below */
  size_t RBFbasis64Count;
  double R, Cv, CFL;
  double tEnd;                   /* > 0: step to this simulated time */
  int nSteps;                    /* > 0: at most this many steps (both may be set) */
  afar_basicFieldData* outFD;    /* cellsNum + totalBoundaryFacesNum states, written when done */
  int8_t* outShockIndicator;     /* 2 (cellsNum + totalBoundaryFacesNum), may be NULL */
} afar_request;
typedef struct {
  long long submitted, completed, failed, queued, running;
  long long peakRunning;
  size_t bytesInUse, peakBytes, budgetBytes;
  long long batchSteps;          /* steps of the batch so far (each steps every running member) */
  long long cancelled;           /* requests cancelled (also counted in failed) */
} afar_server_stats;
afar_status afar_server_create(afar_server** server, int policy, int device, size_t hbmBudgetBytes,
                               int chunkSteps);
afar_status afar_server_submit(afar_server* server, const afar_request* request, long long* requestId);
/* Waits up to timeoutSeconds (< 0: no limit) for the request.  *done = 1 when it has finished;
 * then *requestStatus is its afar_status (AFAR_ERR_NOT_FINITE for a solve whose state broke down;
 * the message is available from afar_last_error on the calling thread), *latencyMs the time from
 * submit to completion and *steps the RK3 steps it took (any of the three may be NULL). */
afar_status afar_server_wait(afar_server* server, long long requestId, double timeoutSeconds, int* done,
                             int* requestStatus, double* latencyMs, long long* steps);
afar_status afar_server_get_stats(afar_server* server, afar_server_stats* stats);
/* Cancels a request: a queued one is dropped at once, a running one leaves the batch at the end of
 * the chunk being stepped and its device memory is freed; its output buffers are not written and
 * afar_server_wait reports AFAR_ERR_CANCELLED.  A request that has already finished is left as it
 * is (AFAR_ERR_STATE). */
afar_status afar_server_cancel(afar_server* server, long long requestId);
/* Finishes the running and queued requests, then stops the worker. */
afar_status afar_server_destroy(afar_server* server);

/* In-device checkpoint of the whole solver state (primitive + conserved fields, RK stage start,
 * time and step count): op 0 saves, op 1 restores (bit-exact resume).  The snapshot lives in
 * device memory next to the state; restore without a prior save is an error. */
#define AFAR_SNAPSHOT_SAVE 0
#define AFAR_SNAPSHOT_RESTORE 1
afar_status afar_state_snapshot(afar_solver* solver, int op);

/* The least-squares gradient matrix the device built (2*maxCompactStencilSize*cellsNum floats
 * in the reference layout; the FP64 policy keeps doubles internally and returns them rounded). */
afar_status afar_download_ls_matrix(afar_solver* solver, float* matrix);

/* The Courant time step of a state the caller already holds on the device, for callers that
 * cannot allocate device memory (an application that hands out all GPU memory from its own pool,
 * or has reserved its device memory budget up front, and forbids libraries to allocate).  It has
 * no counterpart in the reference; it computes the reference's setDeltaT in FP64 (min over
 * internal faces and 1e5), which is what afar_adjustTimeStep returns under the fp64 and ref
 * policies; the mixed policy's afar_adjustTimeStep returns an FP32 estimate of the same minimum,
 * which differs from this one by rounding.  It allocates nothing: no cudaMalloc, no cudaFree, no
 * allocating library call.
 *   FD, CELL, FACE, neighbour: device pointers to the reference-layout arrays (Nc+Nb, Nc+Nb,
 *     Nf+Nb and 2*Nf entries); deltaT: device pointer to one double, written in stream order;
 *   stream: a cudaStream_t, or NULL for the default stream.  Returns once the work is enqueued.
 * The owner and neighbour ids are read on the device and not checked: every entry of neighbour
 * must lie in [0, Nc+Nb), or the kernel reads out of bounds (checking them would need a copy to
 * the host, which this entry point exists to avoid).
 * Limit: facesNum <= 16,777,216 (a fixed scratch of 65,536 per-block minima, 512 KiB, in a static
 * device array that every GPU which loads the library holds until the process exits); larger
 * meshes get AFAR_ERR_LIMIT.  Each call overwrites the scratch entries it reads, so nothing needs
 * clearing; all calls share the scratch, so calls that overlap on the GPU race.  The first call on
 * a device resolves the scratch address on that device (cudaGetSymbolAddress) and keeps it for
 * the life of the process; make that first call before any stream capture.  A cudaDeviceReset
 * after that first call is not supported: the reset reloads the library's device code, the array
 * may move, and later calls would still use the address resolved before. */
afar_status afar_adjustTimeStep_noalloc(const afar_basicFieldData* FD, const afar_meshCellData* CELL,
                                        const afar_meshFaceData* FACE, const int* neighbour,
                                        int facesNum, double R, double Cv, double CFL,
                                        double* deltaT, void* stream);

/* Device memory held by the solver, in bytes. */
afar_status afar_device_bytes(afar_solver* solver, size_t* bytes);
/* The switch decisions of the last stage computed: counts[0] troubled cells, [1] cells on the
 * low-order (TVD) reconstruction, [2] shock cells (KFVS on their faces), [3] KFVS faces. */
afar_status afar_switch_counts(afar_solver* solver, long long counts[4]);

/* The autotuner (no counterpart in the reference).  The mixed policy's reconstruct has two
 * implementations, tile-staged (0) and register pass (1); at the stencil upload each is timed on
 * the solver's own data and the faster kept, the decision cached per device and mesh class (faces
 * per cell, stencil size, cell count to a factor of two).  afar_set_tuning picks one instead
 * (-1: autotune, the default); afar_get_tuning reports the choice and the measured launch times
 * (0 when the decision came from the cache). */
afar_status afar_set_tuning(afar_solver* solver, int reconVariant);
afar_status afar_get_tuning(afar_solver* solver, int* reconVariant, float* msTile, float* msRegister);

/* The device's FP64 multiply-add rate, measured (no counterpart in the reference): a kernel of
 * independent DFMA chains over every SM, timed with CUDA events (best of five ~70 ms launches);
 * *gflops counts two operations per DFMA, *ms (optional) is the timed launch.  The roofline of the
 * fp64 policy, whose flux and update are bound by the FP64 pipe rather than by memory. */
afar_status afar_measure_fp64_peak(int device, double* gflops, float* ms);

/* Test hook for the bounded device waits (no counterpart in the reference).  The mixed policy's
 * tile-staged reconstruct waits on mbarriers for its TMA loads; each wait gives up after a limit
 * of SM clocks (2^31, about a second), marks the solver's error word and lets the kernel return, so
 * that the call which waits next returns AFAR_ERR_CUDA ("... the state is not valid") and the CUDA
 * context stays usable.  extraBytes > 0 adds that many bytes to the transaction count the first
 * barrier of every tile expects (bytes never issued, so those waits run out); limitClocks > 0
 * replaces the limit (<= 0: the default).  afar_debug_wait_injection(device, 0, 0) restores normal
 * operation.  Affects every solver and batch on the device until then. */
afar_status afar_debug_wait_injection(int device, unsigned extraBytes, long long limitClocks);

/* The multi-point face flux (no counterpart in the reference, whose flux uses the face centre; off
 * by default since it changes results).  After afar_setDeviceFieldDataStencil, policies fp64 and
 * mixed: the flux of every internal face becomes the weighted sum of the fluxes at its nPoints (1-4)
 * Gauss points -- at each point the O3 value there (weights rbfGauss) or the TVD state
 * extrapolated there with the cell's limited gradient, as the cells' switches ask, then the same
 * Roe/KFVS choice and dissipation as at the face centre.  The troubled-cell and BVD decisions
 * stay those of the face-centre values; the Courant step is evaluated in FP64 by a kernel of its
 * own.  points: [2*nPoints*facesNum] the points of each internal face (afar_face_gauss_quadrature);
 * pointWeights: [nPoints] positive (normalised here to sum to one); rbfGauss:
 * [facesNum][2][nPoints][maxStencilSize+1] (afar_precompute_fields_gauss).  nPoints = 0 restores
 * the face-centre flux.  A solver with it cannot join a batch. */
afar_status afar_set_face_gauss_flux(afar_solver* solver, int nPoints, const double* points,
                                     const double* pointWeights, const double* rbfGauss);

/* Number of kernel launches one afar_run step issues on this solver (for accounting). */
int afar_launches_per_step(afar_solver* solver);

#ifdef __cplusplus
}
#endif
#endif /* AFAR_H */
