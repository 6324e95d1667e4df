// ref_harness.cpp - runs the reference's own CUDA kernels (oracle/_ref/ref_*.cubin, compiled from
// the reference sources by build_ref.sh) on the same host arrays the product consumes.
//
// TEST INFRASTRUCTURE ONLY (the GPU-side oracle).  The host sequence restates the reference's
// GPUevolve.cu: allocation and upload as setDeviceFieldData (GPUevolve.cu:13-148), the Courant
// step as adjustTimeStep (:177-204), one step as GPUevolve (:207-306), launch shapes and dynamic
// shared-memory sizes as there.  Kernels are looked up by their C++ names in the cubin with the
// CUDA driver API, so no reference host code is linked.
#include <cuda.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../include/afar.h"

namespace {

thread_local char g_err[512];

#define CU(call)                                                          \
  do {                                                                    \
    CUresult r_ = (call);                                                 \
    if (r_ != CUDA_SUCCESS) {                                             \
      const char* s_ = nullptr;                                           \
      cuGetErrorString(r_, &s_);                                          \
      std::snprintf(g_err, sizeof(g_err), "%s: %s", #call, s_ ? s_ : "?"); \
      return -1;                                                          \
    }                                                                     \
  } while (0)

const char* kKernels[] = {"reconstruct",     "BVDindicator",           "evaluateFlux",
                          "evaluateResidual", "updateFieldData",        "updateBoundaryFieldData",
                          "setDeltaT",        "storeConservedFieldData", "calcLeastSquareMatrix",
                          "initShockIndicator", "initResidual"};
enum { K_RECON, K_BVD, K_FLUX, K_RES, K_UPD, K_BC, K_DT, K_STORE, K_LSM, K_INITSI, K_INITRES, K_N };

struct Harness {
  CUcontext ctx = nullptr;
  CUmodule mod = nullptr;
  CUfunction fn[K_N] = {};
  int Nc, Nf, Nb, patches, maxS, maxM, maxLB, maxCLB;
  // device arrays in the reference layout (fieldPointer members)
  CUdeviceptr CELL, FACE, cellVolume, FD, limiter, shockIndicator, cFD, cFDold, gradFD, Flux, Res, neighbour,
      boundaryFacesNum, boundaryFaceNeiLabel, boundaryFacesType, stencilSize, compactStencilSize, RBFbasis, faceFD,
      extendStencil, extendStencilSize, compactExtendStencilSize, localStencil, matrix, cellFaces, minDeltaT;
  std::vector<CUdeviceptr> all;
};

int dmalloc(Harness* h, CUdeviceptr* p, size_t bytes) {
  CU(cuMemAlloc(p, bytes ? bytes : 16));
  h->all.push_back(*p);
  return 0;
}

int up(Harness* h, CUdeviceptr* p, const void* src, size_t bytes) {
  if (dmalloc(h, p, bytes)) return -1;
  if (bytes && src) CU(cuMemcpyHtoD(*p, src, bytes));
  return 0;
}

int launch(Harness* h, int k, unsigned grid, unsigned block, unsigned smem, void** args) {
  if (grid == 0) return 0;
  CU(cuLaunchKernel(h->fn[k], grid, 1, 1, block, 1, 1, smem, nullptr, args, nullptr));
  return 0;
}

}  // namespace

extern "C" const char* refh_last_error(void) { return g_err; }

extern "C" int refh_create(const char* cubin, const afar_fieldPointer* hp, const afar_fieldSizes* sz, void** out) {
  *out = nullptr;
  CU(cuInit(0));
  CUdevice dev;
  CU(cuDeviceGet(&dev, 0));
  Harness* h = new Harness();
  CU(cuDevicePrimaryCtxRetain(&h->ctx, dev));
  CU(cuCtxSetCurrent(h->ctx));
  CU(cuModuleLoad(&h->mod, cubin));
  unsigned count = 0;
  CU(cuModuleGetFunctionCount(&count, h->mod));
  std::vector<CUfunction> fs(count);
  CU(cuModuleEnumerateFunctions(fs.data(), count, h->mod));
  for (unsigned i = 0; i < count; ++i) {
    const char* name = nullptr;
    CU(cuFuncGetName(&name, fs[i]));
    for (int k = 0; k < K_N; ++k) {
      const std::string pre = "_Z" + std::to_string(std::strlen(kKernels[k])) + kKernels[k];
      if (name && std::strncmp(name, pre.c_str(), pre.size()) == 0) h->fn[k] = fs[i];
    }
  }
  for (int k = 0; k < K_N; ++k)
    if (!h->fn[k]) {
      std::snprintf(g_err, sizeof(g_err), "kernel %s not found in %s", kKernels[k], cubin);
      return -1;
    }
  h->Nc = sz->cellsNum;
  h->Nf = sz->facesNum;
  h->Nb = sz->totalBoundaryFacesNum;
  h->patches = sz->patchesNum;
  h->maxS = sz->maxStencilSize;
  h->maxM = sz->maxCompactStencilSize;
  h->maxLB = sz->maxLocalBlockStencilSize;
  h->maxCLB = sz->maxCompactLocalBlockStencilSize;
  const size_t Nc = h->Nc, Nf = h->Nf, Nb = h->Nb, maxS = h->maxS, maxM = h->maxM;
  const size_t nblk = (Nc + AFAR_BLOCKDIM - 1) / AFAR_BLOCKDIM;
  // setDeviceFieldData #1 (GPUevolve.cu:13-64)
  if (up(h, &h->CELL, hp->CELL, 16 * (Nc + Nb)) || up(h, &h->FACE, hp->FACE, 40 * (Nf + Nb)) ||
      up(h, &h->cellVolume, hp->cellVolume, 8 * Nc) || up(h, &h->FD, hp->FD, 32 * (Nc + Nb)) ||
      dmalloc(h, &h->limiter, 16 * Nc) || dmalloc(h, &h->shockIndicator, 2 * (Nc + Nb)) ||
      up(h, &h->cFD, hp->cFD, 32 * Nc) || up(h, &h->cFDold, hp->cFD, 32 * Nc) || dmalloc(h, &h->gradFD, 64 * Nc) ||
      dmalloc(h, &h->Flux, 32 * (Nf + Nb)) || dmalloc(h, &h->Res, 32 * Nc))
    return -1;
  int two = 2 * (int)(Nc + Nb), nc = (int)Nc, nb = (int)Nb, nf = (int)Nf;
  {
    void* a[] = {&h->shockIndicator, &nc, &nb};
    if (launch(h, K_INITSI, (two + 127) / 128, 128, 0, a)) return -1;
    void* b[] = {&h->Res, &nc};
    if (launch(h, K_INITRES, (nc + 127) / 128, 128, 0, b)) return -1;
  }
  // setDeviceFieldData #2 (GPUevolve.cu:67-148)
  if (up(h, &h->neighbour, hp->neighbour, 8 * Nf) || up(h, &h->boundaryFacesNum, hp->boundaryFacesNum, 4 * h->patches) ||
      up(h, &h->boundaryFaceNeiLabel, hp->boundaryFaceNeiLabel, 4 * Nb) ||
      up(h, &h->boundaryFacesType, hp->boundaryFacesType, Nb) || up(h, &h->stencilSize, hp->stencilSize, Nc) ||
      up(h, &h->compactStencilSize, hp->compactStencilSize, Nc) ||
      up(h, &h->RBFbasis, hp->RBFbasis, 4 * 2 * (maxS + 1) * Nf) || dmalloc(h, &h->faceFD, 32 * 2 * Nf) ||
      up(h, &h->extendStencilSize, hp->extendStencilSize, 2 * nblk) ||
      up(h, &h->compactExtendStencilSize, hp->compactExtendStencilSize, 2 * nblk) ||
      up(h, &h->extendStencil, hp->extendStencil, 4 * (size_t)(h->maxLB - AFAR_BLOCKDIM) * nblk) ||
      up(h, &h->localStencil, hp->localStencil, 2 * maxS * Nc) || dmalloc(h, &h->matrix, 4 * 2 * maxM * Nc) ||
      up(h, &h->cellFaces, hp->cellFaces, 4 * maxM * Nc) || dmalloc(h, &h->minDeltaT, 8 * ((Nf + 1023) / 1024)))
    return -1;
  CU(cuMemsetD8(h->matrix, 0, 4 * 2 * maxM * Nc));
  {
    int ms = h->maxS, mm = h->maxM, mclb = h->maxCLB, mlb = h->maxLB;
    void* a[] = {&h->matrix, &h->localStencil, &h->compactStencilSize, &h->CELL, &h->extendStencil,
                 &h->compactExtendStencilSize, &nc, &ms, &mm, &mclb, &mlb};
    if (launch(h, K_LSM, (nc + 127) / 128, 128, (unsigned)(8 * h->maxCLB * 2), a)) return -1;
  }
  CU(cuCtxSynchronize());
  *out = h;
  return 0;
}

// One RK stage k of GPUevolve (GPUevolve.cu:233-294); the residual is read back between
// evaluateResidual and updateFieldData.  Outputs may be NULL.
extern "C" int refh_stage(void* hv, int k, double R, double Cv, double dt, int store, afar_fieldPointer* out) {
  Harness* h = static_cast<Harness*>(hv);
  CU(cuCtxSetCurrent(h->ctx));
  const double beta1[3] = {1.0, 0.75, 0.333333};
  const double beta2[3] = {0.0, 0.25, 0.666667};
  const double beta3[3] = {1.0, 0.25, 0.666667};
  const double gamma = R / Cv + 1.0;
  int nc = h->Nc, nf = h->Nf, nb = h->Nb, ms = h->maxS, mm = h->maxM, mlb = h->maxLB, mclb = h->maxCLB;
  const unsigned gc = (nc + 127) / 128;
  {
    const unsigned smem = 8 * mclb * 2 + 4 * mlb * 4 + 2 * 128 * ms + 1 * 128 * 2;
    void* a[] = {&h->faceFD, &h->gradFD, &h->limiter, &h->shockIndicator, &h->FD, &h->matrix, &h->RBFbasis,
                 &h->CELL, &h->FACE, &h->cellFaces, &h->localStencil, &h->stencilSize, &h->compactStencilSize,
                 &h->extendStencil, &h->extendStencilSize, &h->compactExtendStencilSize, &nc, &nf, &ms, &mm, &mlb,
                 &mclb};
    if (launch(h, K_RECON, gc, 128, smem, a)) return -1;
  }
  {
    const unsigned smem = 8 * 128 * 4 + 4 * 128 * 2 + 2 * 128 * ms + 128 + mlb;
    void* a[] = {&h->faceFD, &h->gradFD, &h->shockIndicator, &h->limiter, &h->FD, &h->CELL, &h->FACE, &h->cellFaces,
                 &h->localStencil, &h->stencilSize, &h->compactStencilSize, &h->extendStencil, &h->extendStencilSize,
                 &nc, &nf, &ms, &mm, &mlb};
    if (launch(h, K_BVD, gc, 128, smem, a)) return -1;
  }
  {
    void* a[] = {&h->Flux, &h->FD, &h->gradFD, &h->limiter, &h->faceFD, &h->shockIndicator, &h->CELL, &h->FACE,
                 &h->neighbour, &nf, &nc, &nb, &R, &Cv};
    if (launch(h, K_FLUX, (nf + 127) / 128, 128, 0, a)) return -1;
  }
  {
    void* a[] = {&h->Res, &h->Flux, &h->cellFaces, &h->compactStencilSize, &nc, &mm};
    if (launch(h, K_RES, gc, 128, 0, a)) return -1;
  }
  if (out) {
    CU(cuCtxSynchronize());
    if (out->Res) CU(cuMemcpyDtoH(out->Res, h->Res, 32 * (size_t)nc));
    if (out->faceFD) CU(cuMemcpyDtoH(out->faceFD, h->faceFD, 64 * (size_t)nf));
    if (out->gradFD) CU(cuMemcpyDtoH(out->gradFD, h->gradFD, 64 * (size_t)nc));
    if (out->limiter) CU(cuMemcpyDtoH(out->limiter, h->limiter, 16 * (size_t)nc));
    if (out->Flux) CU(cuMemcpyDtoH(out->Flux, h->Flux, 32 * (size_t)(nf + nb)));
    if (out->shockIndicator) CU(cuMemcpyDtoH(out->shockIndicator, h->shockIndicator, 2 * (size_t)(nc + nb)));
  }
  {
    double b1 = beta1[k], b2 = beta2[k], b3 = beta3[k], g = gamma, d = dt, r = R;
    void* a[] = {&h->FD, &h->cFD, &h->cFDold, &h->Res, &h->cellVolume, &r, &g, &nc, &d, &b1, &b2, &b3};
    if (launch(h, K_UPD, gc, 128, 0, a)) return -1;
  }
  {
    void* a[] = {&h->FD, &h->CELL, &h->FACE, &h->boundaryFaceNeiLabel, &h->boundaryFacesType, &nc, &nf, &nb, &R, &Cv};
    if (launch(h, K_BC, (nb + 127) / 128, 128, 0, a)) return -1;
  }
  if (store) {
    void* a[] = {&h->cFDold, &h->cFD, &nc};
    if (launch(h, K_STORE, gc, 128, 0, a)) return -1;
  }
  if (out) {
    CU(cuCtxSynchronize());
    if (out->FD) CU(cuMemcpyDtoH(out->FD, h->FD, 32 * (size_t)(nc + nb)));
    if (out->cFD) CU(cuMemcpyDtoH(out->cFD, h->cFD, 32 * (size_t)nc));
  }
  return 0;
}

// GPUevolve (GPUevolve.cu:207-306), nsteps times with a fixed step; optional device time in ms.
extern "C" int refh_evolve(void* hv, int nsteps, double R, double Cv, double dt, float* ms) {
  Harness* h = static_cast<Harness*>(hv);
  CU(cuCtxSetCurrent(h->ctx));
  CUevent e0, e1;
  CU(cuEventCreate(&e0, CU_EVENT_DEFAULT));
  CU(cuEventCreate(&e1, CU_EVENT_DEFAULT));
  CU(cuEventRecord(e0, nullptr));
  for (int s = 0; s < nsteps; ++s)
    for (int k = 0; k < 3; ++k)
      if (refh_stage(hv, k, R, Cv, dt, k == 2, nullptr)) return -1;
  CU(cuEventRecord(e1, nullptr));
  CU(cuEventSynchronize(e1));
  if (ms) CU(cuEventElapsedTime(ms, e0, e1));
  cuEventDestroy(e0);
  cuEventDestroy(e1);
  return 0;
}

// adjustTimeStep (GPUevolve.cu:177-204): setDeltaT kernel, block minima to the host, host min.
extern "C" int refh_adjust_dt(void* hv, double R, double Cv, double CFL, double* dt) {
  Harness* h = static_cast<Harness*>(hv);
  CU(cuCtxSetCurrent(h->ctx));
  int nf = h->Nf;
  const unsigned g = (nf + 1023) / 1024;
  void* a[] = {&h->minDeltaT, &h->FD, &h->CELL, &h->FACE, &h->neighbour, &nf, &R, &Cv, &CFL};
  if (launch(h, K_DT, g, 1024, 0, a)) return -1;
  CU(cuCtxSynchronize());
  std::vector<double> m(g);
  if (g) CU(cuMemcpyDtoH(m.data(), h->minDeltaT, 8 * (size_t)g));
  double best = 1e5;
  for (unsigned i = 0; i < g; ++i) best = best > m[i] ? m[i] : best;
  *dt = best;
  return 0;
}

extern "C" int refh_download(void* hv, afar_fieldPointer* out) {
  Harness* h = static_cast<Harness*>(hv);
  CU(cuCtxSetCurrent(h->ctx));
  CU(cuCtxSynchronize());
  if (out->FD) CU(cuMemcpyDtoH(out->FD, h->FD, 32 * (size_t)(h->Nc + h->Nb)));
  if (out->cFD) CU(cuMemcpyDtoH(out->cFD, h->cFD, 32 * (size_t)h->Nc));
  if (out->shockIndicator) CU(cuMemcpyDtoH(out->shockIndicator, h->shockIndicator, 2 * (size_t)(h->Nc + h->Nb)));
  if (out->matrix) CU(cuMemcpyDtoH(out->matrix, h->matrix, 8 * (size_t)h->maxM * h->Nc));
  return 0;
}

extern "C" int refh_upload_state(void* hv, const void* FD, const void* cFD, const void* cFDold) {
  Harness* h = static_cast<Harness*>(hv);
  CU(cuCtxSetCurrent(h->ctx));
  if (FD) CU(cuMemcpyHtoD(h->FD, FD, 32 * (size_t)(h->Nc + h->Nb)));
  if (cFD) CU(cuMemcpyHtoD(h->cFD, cFD, 32 * (size_t)h->Nc));
  if (cFDold) CU(cuMemcpyHtoD(h->cFDold, cFDold, 32 * (size_t)h->Nc));
  return 0;
}

extern "C" void refh_destroy(void* hv) {
  Harness* h = static_cast<Harness*>(hv);
  if (!h) return;
  cuCtxSetCurrent(h->ctx);
  cuCtxSynchronize();
  for (CUdeviceptr p : h->all) cuMemFree(p);
  if (h->mod) cuModuleUnload(h->mod);
  CUdevice dev;
  if (cuCtxGetDevice(&dev) == CUDA_SUCCESS) cuDevicePrimaryCtxRelease(dev);
  delete h;
}
