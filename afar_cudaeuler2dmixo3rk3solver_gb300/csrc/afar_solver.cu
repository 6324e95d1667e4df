// libafar host<->device boundary: the drop-in replacement of the reference's GPUevolve.{h,cu}
// (setDeviceFieldData x2, adjustTimeStep, GPUevolve, copyFieldDataDeviceToHost, freeFieldData),
// plus graph-captured multi-step runs and per-stage parity hooks.
//
// The caller hands over the reference's host arrays (include/afar.h afar_fieldPointer); the
// library re-lays them out on the device (slot-major per-cell lists, per-face geometry constants,
// policy-typed intermediates; see afar_kernels.cuh) and owns all device memory.
#include <cuda_runtime.h>

#include <cstring>
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include <cudaTypedefs.h>  // PFN_cuTensorMapEncodeTiled
#include <nvtx3/nvToolsExt.h>

#include "afar_internal.h"
#include "afar_kernels.cuh"

namespace {
// A named NVTX range over an entry point (host-side tracing: it shows the library's calls on a
// profiler timeline beside their kernels; inert without a profiler attached).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};
}  // namespace

using namespace afar;

#define AFAR_CUDA(call)                                                                      \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) {                                                                 \
      set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return AFAR_ERR_CUDA;                                                                  \
    }                                                                                        \
  } while (0)

namespace {

constexpr int kCellBlock = 128;
constexpr size_t kMaxDynamicSmem = 227 * 1024;  // per CTA on sm_103a
constexpr int kFaceBlock = 256;
// GPUevolve.cu:223-225: the reference's truncated SSP-RK3 coefficients
constexpr double kBeta1[3] = {1.0, 0.75, 0.333333};
constexpr double kBeta2[3] = {0.0, 0.25, 0.666667};
constexpr double kBeta3[3] = {1.0, 0.25, 0.666667};

struct FaceRaw {
  double x, y, magSf, Sfx, Sfy;
};

// setup kernels that only move the reference arrays into the device layout
__global__ void k_setup_lists(int Nc, int ldc, int maxS, int maxM, int maxLB, const uint8_t* nS, const uint8_t* nM,
                              const uint16_t* localStencil, const int* extendStencil, const int* cellFaces, int* sten,
                              int* cf) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= Nc) return;
  const int blk = c / AFAR_BLOCKDIM;
  for (int i = 0; i < nS[c]; ++i) {
    const int loc = localStencil[(size_t)maxS * c + i];
    sten[(size_t)i * ldc + c] =
        loc < AFAR_BLOCKDIM ? blk * AFAR_BLOCKDIM + loc : extendStencil[(size_t)(maxLB - AFAR_BLOCKDIM) * blk + (loc - AFAR_BLOCKDIM)];
  }
  for (int i = 0; i < nM[c]; ++i) cf[(size_t)i * ldc + c] = cellFaces[(size_t)maxM * c + i];
}

__global__ void k_split_faces(int n, const FaceRaw* raw, V4<double>* xy, V4<double>* s) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= n) return;
  const FaceRaw r = raw[f];
  xy[f] = V4<double>{r.x, r.y, 0.0, 0.0};
  s[f] = V4<double>{r.Sfx, r.Sfy, r.magSf, 0.0};
}

template <class T, class Src>
__global__ void k_setup_wts(int Nc, int Nf, int ldc, int maxS, const uint8_t* nS, const uint8_t* nM, const int* cf,
                            const Src* rbf, T* wts) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= Nc) return;
  const size_t nmax = (size_t)maxS + 1;
  for (int fi = 0; fi < nM[c]; ++fi) {
    int f = cf[(size_t)fi * ldc + c];
    const int side = f < 0;
    f = abs(f) - 1;
    if (f >= Nf) continue;
    const Src* src = rbf + 2 * nmax * f + side * nmax;
    T* dst = wts + (size_t)fi * nmax * ldc + c;
    for (int j = 0; j <= nS[c]; ++j) dst[(size_t)j * ldc] = (T)src[j];
  }
}

__global__ void k_set_write_interval(StepCtl* ctl, double interval) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    ctl->write_interval = interval;
    ctl->write_index = interval > 0.0 ? (long long)floor(ctl->t / interval * (1.0 + 1e-12)) : 0;
  }
}

__global__ void k_set_ctl(StepCtl* ctl, double dt_fixed, double cfl, double t_end) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    ctl->dt_fixed = dt_fixed;
    ctl->cfl = cfl;
    ctl->t_end = t_end;
  }
}

__global__ void k_init_ctl(StepCtl* ctl) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    ctl->dt_bits = (unsigned long long)__double_as_longlong(1e5);
    ctl->t = 0.0;
    ctl->t_end = 0.0;
    ctl->dt_fixed = 0.0;
    ctl->cfl = 0.5;
    ctl->last_dt = 0.0;
    ctl->steps = 0;
    ctl->err = 0;
    ctl->write_interval = 0.0;
    ctl->write_index = 0;
  }
}

__global__ void k_reciprocal(int n, const double* in, double* out, float* outf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    out[i] = 1.0 / in[i];
    if (outf) outf[i] = (float)(1.0 / in[i]);
  }
}

// The mixed policy's conserved state: double -> float pair in place (each thread rewrites its own
// 32 bytes), and float pair -> double.
__global__ void k_df_from_double(int n, V4<double>* u) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const V4<double> v = u[i];
  DF4 d;
  d.hi = V4<float>{(float)v.x, (float)v.y, (float)v.z, (float)v.w};
  d.lo = V4<float>{(float)(v.x - (double)d.hi.x), (float)(v.y - (double)d.hi.y), (float)(v.z - (double)d.hi.z),
                   (float)(v.w - (double)d.hi.w)};
  reinterpret_cast<DF4*>(u)[i] = d;
}
__global__ void k_df_to_double(int n, const DF4* in, V4<double>* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const DF4 d = in[i];
  out[i] = V4<double>{(double)d.hi.x + (double)d.lo.x, (double)d.hi.y + (double)d.lo.y,
                      (double)d.hi.z + (double)d.lo.z, (double)d.hi.w + (double)d.lo.w};
}

template <class A, class B>
__global__ void k_convert2(int n, const V2<A>* in, V2<B>* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = V2<B>{(B)in[i].x, (B)in[i].y};
}

template <class A, class B>
__global__ void k_convert4(int n, const V4<A>* in, V4<B>* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = V4<B>{(B)in[i].x, (B)in[i].y, (B)in[i].z, (B)in[i].w};
}

inline int grid_for(long long n, int block) { return (int)((n + block - 1) / block); }

StageCoef stage_coef(int k) {
  StageCoef c;
  c.b1 = kBeta1[k];
  c.b2 = kBeta2[k];
  c.b3 = kBeta3[k];
  c.b1h = (float)c.b1;
  c.b1l = (float)(c.b1 - (double)c.b1h);
  c.b2h = (float)c.b2;
  c.b2l = (float)(c.b2 - (double)c.b2h);
  c.first = k == 0;
  c.last = k == 2;
  return c;
}

}  // namespace

struct afar_solver {
  int policy = AFAR_POLICY_REF;
  int device = 0;
  cudaStream_t stream = nullptr;
  // sizes
  int Nc = 0, Nf = 0, Nb = 0, patches = 0, maxS = 0, maxM = 0, maxLB = 0, maxCLB = 0, ldc = 0;
  bool have_fields = false, have_stencil = false;
  double R = 0.0, Cv = 0.0;  // of the captured graph
  // policy-independent device arrays
  V2<double>* cellC = nullptr;
  FaceRaw* faceRaw = nullptr;
  double* vol = nullptr;
  double* vinv = nullptr;
  float* vinvf = nullptr;  // mixed: 1/V as float
  V2<float>* dtgf = nullptr;  // mixed: Courant geometry as float
  double px = 0.0, py = 0.0;  // periods of a periodic mesh (afar_set_periodic)
  int recon_variant = 0;      // mixed reconstruct: 0 tile-staged, 1 register pass (autotuned)
  int recon_request = -1;     // afar_set_tuning: -1 autotune, else the variant to use
  // The step split for the reference-shaped loop: afar_adjustTimeStep runs the head (stage 1 up to
  // its flux, whose fused reduction is the Courant step) instead of a separate Courant pass, and the
  // afar_GPUevolve that follows runs the tail (the rest of the step) with the caller's step size.
  // head_pending: the head ran on the current state and nothing has touched the solver since.
  cudaGraphExec_t graph_head = nullptr, graph_tail = nullptr;
  bool head_pending = false;
  float tune_ms[2] = {0.f, 0.f};  // the autotuner's measured launch times (0: decision from the cache)
  void* xfer = nullptr;    // mixed: staging for double <-> device-format copies, 32 B x (Nc + Nb)
  int2* on = nullptr;
  int* bnei = nullptr;
  uint8_t* btype = nullptr;
  uint8_t* nS = nullptr;
  uint8_t* nM = nullptr;
  uint8_t* tileS = nullptr;  // per 128-cell tile: its largest stencil size
  TileMaps* tmaps = nullptr;  // mixed: tensor maps of the operator rows (device memory)
  int* sten = nullptr;
  int* cf = nullptr;
  V4<double>* U = nullptr;
  V4<double>* U0 = nullptr;
  int8_t* si = nullptr;
  V2<double>* dtg = nullptr;
  V2<double>* bn = nullptr;
  V4<double>* res_dbg = nullptr;
  afar_batch* batch = nullptr;  // the batch this solver belongs to, if any
  StepCtl* ctl = nullptr;
  unsigned long long* dt_bits = nullptr;
  // policy-typed device arrays (element size depends on the policy)
  void* W = nullptr;
  void* fd = nullptr;
  void* fs = nullptr;
  void* lsm = nullptr;
  void* sg = nullptr;
  void* sr = nullptr;
  void* wts = nullptr;
  void* grad = nullptr;
  void* lim = nullptr;
  void* fv = nullptr;
  void* flux = nullptr;
  void* snap = nullptr;       // device snapshot of W, U, U0, step control
  // the optional multi-point face flux (afar_set_face_gauss_flux): points per face (0: off)
  int ng = 0;
  void* wg = nullptr;
  void* sgk = nullptr;
  void* fgk = nullptr;
  void* fvg = nullptr;
  double gw[4] = {0.0, 0.0, 0.0, 0.0};
  std::vector<double> rbf64;  // optional FP64 weights awaiting the stencil upload
  cudaGraphExec_t graph = nullptr;
  size_t bytes = 0;
  std::vector<void*> allocs;
};

namespace {

afar_status dalloc(afar_solver* s, void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  AFAR_CUDA(cudaMalloc(p, bytes));
  s->allocs.push_back(*p);
  s->bytes += bytes;
  return AFAR_OK;
}
template <class T>
afar_status dalloc_t(afar_solver* s, T** p, size_t n) {
  return dalloc(s, reinterpret_cast<void**>(p), n * sizeof(T));
}

template <class P>
StageArgs<P> make_args(afar_solver* s) {
  StageArgs<P> a;
  using S = typename P::S;
  using G = typename P::G;
  a.Nc = s->Nc;
  a.Nf = s->Nf;
  a.Nb = s->Nb;
  a.ldc = s->ldc;
  a.maxS = s->maxS;
  a.maxM = s->maxM;
  a.cellC = s->cellC;
  a.on = s->on;
  a.fd = static_cast<const V4<G>*>(s->fd);
  a.fs = static_cast<const V4<G>*>(s->fs);
  a.dtg = s->dtg;
  a.bn = s->bn;
  a.btype = s->btype;
  a.vol = s->vol;
  a.nS = s->nS;
  a.tileS = s->tileS;
  a.nM = s->nM;
  a.sten = s->sten;
  a.cf = s->cf;
  a.lsm = static_cast<const V2<S>*>(s->lsm);
  a.sg = static_cast<const V2<G>*>(s->sg);
  a.sr = static_cast<const V2<S>*>(s->sr);
  a.wts = static_cast<const S*>(s->wts);
  a.tmaps = s->tmaps;
  a.W = static_cast<V4<typename P::W>*>(s->W);
  a.U = s->U;
  a.U0 = s->U0;
  a.grad = static_cast<V4<G>*>(s->grad);
  a.lim = static_cast<V4<S>*>(s->lim);
  a.si = s->si;
  a.fv = static_cast<V4<G>*>(s->fv);
  a.flux = static_cast<V4<typename P::F>*>(s->flux);
  a.vinv = s->vinv;
  a.ctl = s->ctl;
  a.res_dbg = nullptr;
  a.R = s->R;
  a.Cv = s->Cv;
  a.invR = s->R > 0.0 ? 1.0 / s->R : 0.0;
  a.gamma = s->Cv > 0.0 ? s->R / s->Cv + 1.0 : 0.0;
  a.gm1f = (float)(a.gamma - 1.0);
  a.invRf = (float)a.invR;
  a.vinvf = s->vinvf;
  a.Rf = (float)s->R;
  a.Cvf = (float)s->Cv;
  a.gRf = (float)(a.gamma * s->R);
  a.dtgf = s->dtgf;
  a.px = s->px;
  a.py = s->py;
  a.ng = s->ng;
  a.wg = static_cast<const S*>(s->wg);
  a.sgk = static_cast<const V2<G>*>(s->sgk);
  a.fgk = static_cast<const V2<G>*>(s->fgk);
  a.fvg = static_cast<V4<G>*>(s->fvg);
  for (int k = 0; k < 4; ++k) a.gw[k] = (G)s->gw[k];
  return a;
}

// cudaFuncAttributeMaxDynamicSharedMemorySize of a staged reconstruct kernel only grows (per
// device), so solvers and batches of different stencil sizes never lower one another's limit.
template <class K>
afar_status raise_smem_limit(K kernel, int device, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> done;
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = done[{reinterpret_cast<const void*>(kernel), device}];
  if (bytes > cur) {
    AFAR_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    cur = bytes;
  }
  return AFAR_OK;
}

// Dynamic shared memory of the reconstruct: the mixed policy stages a whole 128-cell tile of
// operator rows (recon_tile_layout); ref stages the stencil values, fp64 the compact stencil's.
template <class P>
size_t recon_smem(const afar_solver* s) {
  if constexpr (P::id == PolicyMixed::id) return recon_tile_layout(s->maxM, s->maxS).bytes;
  const int rows = P::id == PolicyFP64::id ? s->maxM : s->maxS;  // fp64 stages the compact stencil only
  return (size_t)(rows > 0 ? rows : 1) * kCellBlock * sizeof(V4<typename P::S>);
}

// One solve's stage launches, arguments by value.  The ref policy reconstructs in the staged
// kernel and runs the reference-layout flux; fp64 reconstructs staged, mixed in registers.
template <class P>
struct Stage {
  afar_solver* s;
  StageArgs<P> a;
  int gc() const { return grid_for(s->Nc, kCellBlock); }

  void reconstruct() const {
    if constexpr (P::id == PolicyMixed::id) {
      if (s->recon_variant == 1)
        k_reconstruct_reg<P><<<gc(), kCellBlock, 0, s->stream>>>(a);
      else if (s->maxM <= 3)
        k_reconstruct_tile<P, 3><<<gc(), kTile, recon_smem<P>(s), s->stream>>>(a);
      else
        k_reconstruct_tile<P, 4><<<gc(), kTile, recon_smem<P>(s), s->stream>>>(a);
    } else
      k_reconstruct_staged<P><<<gc(), kCellBlock, recon_smem<P>(s), s->stream>>>(a);
    if constexpr (P::id != PolicyRef::id) {
      if (s->ng > 0) k_reconstruct_gauss<P><<<gc(), kCellBlock, 0, s->stream>>>(a);
    }
  }
  void bvd() const { k_bvd<P><<<gc(), kCellBlock, 0, s->stream>>>(a); }
  // The face flux.  The ref policy computes the CFL step as a kernel of its own before the first
  // stage's flux, like the reference's setDeltaT; the other policies fuse it into that flux.
  void flux(bool dt_stage) const {
    const int gf = grid_for((long long)s->Nf + s->Nb, kFaceBlock);
    if constexpr (P::id == PolicyRef::id) {
      if (dt_stage && s->Nf > 0)
        k_delta_t<P><<<grid_for(s->Nf, kFaceBlock), kFaceBlock, 0, s->stream>>>(a, 0.0, &s->ctl->dt_bits, s->ctl);
      k_flux<P, false><<<gf, kFaceBlock, 0, s->stream>>>(a);
    } else if (s->ng > 0) {  // the multi-point face flux; the Courant step as a kernel of its own
      if (dt_stage && s->Nf > 0)
        k_delta_t<P><<<grid_for(s->Nf, kFaceBlock), kFaceBlock, 0, s->stream>>>(a, 0.0, &s->ctl->dt_bits, s->ctl);
      k_flux_gauss<P><<<gf, kFaceBlock, 0, s->stream>>>(a);
    } else {
      if (dt_stage)
        k_flux<P, true><<<gf, kFaceBlock, 0, s->stream>>>(a);
      else
        k_flux<P, false><<<gf, kFaceBlock, 0, s->stream>>>(a);
    }
  }
  void update(int k) const {
    k_update<P><<<gc(), kCellBlock, 0, s->stream>>>(a, stage_coef(k));
  }
};

// Stage launcher of a solver; debug = true also writes the residual copy (afar_stage_debug).
template <class P>
afar_status make_stage(afar_solver* s, bool debug, Stage<P>* out) {
  out->s = s;
  out->a = make_args<P>(s);
  if (debug) out->a.res_dbg = s->res_dbg;
  return AFAR_OK;
}

// A step is its head (stage 1 up to the flux, which also reduces the Courant step) and its tail.
template <class P>
void enqueue_head(const Stage<P>& st) {
  st.reconstruct();
  st.bvd();
  st.flux(true);
}
template <class P>
void enqueue_tail(const Stage<P>& st) {
  st.update(0);
  for (int k = 1; k < 3; ++k) {
    st.reconstruct();
    st.bvd();
    st.flux(false);
    st.update(k);
  }
  k_finish_step<<<1, 32, 0, st.s->stream>>>(st.s->ctl);
}
template <class P>
void enqueue_step(const Stage<P>& st) {
  enqueue_head(st);
  enqueue_tail(st);
}

template <class P>
afar_status setup_operators(afar_solver* s, const afar_fieldPointer* h) {
  using S = typename P::S;
  using G = typename P::G;
  const int Nc = s->Nc, Nf = s->Nf, Nb = s->Nb, ldc = s->ldc;
  afar_status st;
  if ((st = dalloc(s, &s->fd, sizeof(V4<G>) * (size_t)Nf))) return st;
  if ((st = dalloc(s, &s->fs, sizeof(V4<G>) * (size_t)(Nf + Nb)))) return st;
  if ((st = dalloc(s, &s->lsm, sizeof(V2<S>) * (size_t)s->maxM * ldc))) return st;
  if ((st = dalloc(s, &s->sg, sizeof(V2<G>) * (size_t)s->maxM * ldc))) return st;
  if ((st = dalloc(s, &s->sr, sizeof(V2<S>) * (size_t)s->maxM * ldc))) return st;
  if ((st = dalloc(s, &s->wts, sizeof(S) * (size_t)s->maxM * (s->maxS + 1) * ldc))) return st;
  AFAR_CUDA(cudaMemsetAsync(s->wts, 0, sizeof(S) * (size_t)s->maxM * (s->maxS + 1) * ldc, s->stream));
  AFAR_CUDA(cudaMemsetAsync(s->lsm, 0, sizeof(V2<S>) * (size_t)s->maxM * ldc, s->stream));

  // O3 weights: float reference layout (or the FP64 copy) -> slot-major
  const size_t nrbf = 2 * (size_t)(s->maxS + 1) * Nf;
  const int gc = grid_for(Nc, kCellBlock);
  if (std::is_same<S, double>::value && s->rbf64.size() == nrbf) {
    double* tmp = nullptr;
    AFAR_CUDA(cudaMalloc(&tmp, sizeof(double) * (nrbf ? nrbf : 1)));
    AFAR_CUDA(cudaMemcpyAsync(tmp, s->rbf64.data(), sizeof(double) * nrbf, cudaMemcpyHostToDevice, s->stream));
    k_setup_wts<S, double><<<gc, kCellBlock, 0, s->stream>>>(Nc, Nf, ldc, s->maxS, s->nS, s->nM, s->cf, tmp,
                                                             static_cast<S*>(s->wts));
    AFAR_CUDA(cudaStreamSynchronize(s->stream));
    AFAR_CUDA(cudaFree(tmp));
  } else {
    float* tmp = nullptr;
    AFAR_CUDA(cudaMalloc(&tmp, sizeof(float) * (nrbf ? nrbf : 1)));
    AFAR_CUDA(cudaMemcpyAsync(tmp, h->RBFbasis, sizeof(float) * nrbf, cudaMemcpyHostToDevice, s->stream));
    k_setup_wts<S, float><<<gc, kCellBlock, 0, s->stream>>>(Nc, Nf, ldc, s->maxS, s->nS, s->nM, s->cf, tmp,
                                                            static_cast<S*>(s->wts));
    AFAR_CUDA(cudaStreamSynchronize(s->stream));
    AFAR_CUDA(cudaFree(tmp));
  }
  s->rbf64.clear();
  s->rbf64.shrink_to_fit();

  V4<double>* fxy = nullptr;
  V4<double>* fsr = nullptr;
  AFAR_CUDA(cudaMalloc(&fxy, sizeof(V4<double>) * (size_t)(Nf + Nb + 1)));
  AFAR_CUDA(cudaMalloc(&fsr, sizeof(V4<double>) * (size_t)(Nf + Nb + 1)));
  const int gF = grid_for((long long)Nf + Nb, kFaceBlock);
  k_split_faces<<<gF, kFaceBlock, 0, s->stream>>>(Nf + Nb, s->faceRaw, fxy, fsr);
  StageArgs<P> a = make_args<P>(s);
  k_setup_lsm<P><<<gc, kCellBlock, 0, s->stream>>>(a, static_cast<V2<S>*>(s->lsm), nullptr, 0);
  k_setup_slot_geom<P><<<gc, kCellBlock, 0, s->stream>>>(a, fxy);
  k_setup_face_geom<P><<<gF, kFaceBlock, 0, s->stream>>>(a, fxy, fsr);
  if constexpr (P::id == PolicyMixed::id) {
    if ((st = dalloc_t(s, &s->dtgf, (size_t)Nf))) return st;
    if (Nf > 0) k_convert2<double, float><<<grid_for(Nf, 256), 256, 0, s->stream>>>(Nf, s->dtg, s->dtgf);
  }
  AFAR_CUDA(cudaGetLastError());
  AFAR_CUDA(cudaStreamSynchronize(s->stream));
  AFAR_CUDA(cudaFree(fxy));
  AFAR_CUDA(cudaFree(fsr));
  if constexpr (P::id != PolicyMixed::id) {
    return raise_smem_limit(k_reconstruct_staged<P>, s->device, recon_smem<P>(s));
  } else {
    if (recon_smem<P>(s) > kMaxDynamicSmem) {
      set_error("stencil too large for the reconstruct tile: %zu bytes of shared memory", recon_smem<P>(s));
      return AFAR_ERR_LIMIT;
    }
    if ((st = raise_smem_limit(k_reconstruct_tile<P, 3>, s->device, recon_smem<P>(s)))) return st;
    return raise_smem_limit(k_reconstruct_tile<P, 4>, s->device, recon_smem<P>(s));
  }
}

void destroy_graphs(afar_solver* s) {
  for (cudaGraphExec_t* g : {&s->graph, &s->graph_head, &s->graph_tail})
    if (*g) {
      cudaGraphExecDestroy(*g);
      *g = nullptr;
    }
  s->head_pending = false;
}

// The step graph, and its head and tail as graphs of their own (the same launches split in two).
afar_status capture_graph(afar_solver* s) {
  destroy_graphs(s);
  cudaGraph_t g[3] = {nullptr, nullptr, nullptr};
  auto capture = [&](auto tag) -> afar_status {
    using P = decltype(tag);
    Stage<P> st;
    afar_status r = make_stage<P>(s, false, &st);  // uploads the argument table before the capture
    if (r) return r;
    for (int i = 0; i < 3; ++i) {
      AFAR_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
      if (i == 0) enqueue_step<P>(st);
      if (i == 1) enqueue_head<P>(st);
      if (i == 2) enqueue_tail<P>(st);
      AFAR_CUDA(cudaStreamEndCapture(s->stream, &g[i]));
    }
    return AFAR_OK;
  };
  afar_status r;
  switch (s->policy) {
    case AFAR_POLICY_REF: r = capture(PolicyRef{}); break;
    case AFAR_POLICY_FP64: r = capture(PolicyFP64{}); break;
    default: r = capture(PolicyMixed{}); break;
  }
  cudaGraphExec_t* out[3] = {&s->graph, &s->graph_head, &s->graph_tail};
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 3; ++i) {
    if (!r && g[i] && e == cudaSuccess) e = cudaGraphInstantiate(out[i], g[i], 0);
    if (g[i]) cudaGraphDestroy(g[i]);
  }
  if (r) return r;
  if (e != cudaSuccess) {
    set_error("cudaGraphInstantiate failed: %s", cudaGetErrorString(e));
    destroy_graphs(s);
    return AFAR_ERR_CUDA;
  }
  return AFAR_OK;
}

afar_status check_ready(afar_solver* s) {
  if (!s) {
    set_error("null solver");
    return AFAR_ERR_ARGUMENT;
  }
  s->head_pending = false;  // every call that goes through here may change what the head computed
  if (!s->have_fields || !s->have_stencil) {
    set_error("call afar_setDeviceFieldData and afar_setDeviceFieldDataStencil first");
    return AFAR_ERR_STATE;
  }
  AFAR_CUDA(cudaSetDevice(s->device));
  return AFAR_OK;
}

// Stepping a batch member on its own would race with (and desynchronise) the batch.
afar_status check_not_batched(afar_solver* s) {
  if (s->batch) {
    set_error("the solver belongs to a batch: step it with afar_batch_run or remove it first");
    return AFAR_ERR_STATE;
  }
  return AFAR_OK;
}

// Reads (and clears) the device error word after a wait: a bounded device wait that gave up marks
// the step's results invalid.
afar_status check_device_error(afar_solver* s) {
  unsigned err = 0;
  AFAR_CUDA(cudaMemcpyAsync(&err, &s->ctl->err, sizeof(err), cudaMemcpyDeviceToHost, s->stream));
  AFAR_CUDA(cudaStreamSynchronize(s->stream));
  if (err) {
    AFAR_CUDA(cudaMemsetAsync(&s->ctl->err, 0, sizeof(err), s->stream));
    AFAR_CUDA(cudaStreamSynchronize(s->stream));
    set_error("a device-side wait for a bulk copy timed out (error word %u); the state is not valid", err);
    return AFAR_ERR_CUDA;
  }
  return AFAR_OK;
}

size_t w_size(int policy) { return policy == AFAR_POLICY_MIXED ? sizeof(V4<float>) : sizeof(V4<double>); }

}  // namespace

// ------------------------------------------------------------------------------------------------
extern "C" afar_status afar_solver_create(afar_solver** out, int policy, int device) {
  if (!out || policy < AFAR_POLICY_REF || policy > AFAR_POLICY_MIXED) {
    set_error("afar_solver_create: null output or unknown policy %d", policy);
    return AFAR_ERR_ARGUMENT;
  }
  *out = nullptr;
  int n = 0;
  AFAR_CUDA(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) {
    set_error("afar_solver_create: device %d not present (%d devices)", device, n);
    return AFAR_ERR_ARGUMENT;
  }
  AFAR_CUDA(cudaSetDevice(device));
  afar_solver* s = new afar_solver();
  s->policy = policy;
  s->device = device;
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
    set_error("cudaStreamCreate failed");
    delete s;
    return AFAR_ERR_CUDA;
  }
  *out = s;
  return AFAR_OK;
}

// Host <-> device state in the reference's double layout, ordered on the solver's stream.  The
// mixed policy keeps W as float and U, Un as float pairs: the doubles are staged in `xfer` and
// converted on the device.
static afar_status put_state(afar_solver* s, const afar_basicFieldData* FD, const afar_conservedFieldData* cFD,
                      const afar_conservedFieldData* cFDold) {
  const size_t Nc = s->Nc, Nb = s->Nb;
  const bool mixed = s->policy == AFAR_POLICY_MIXED;
  if (FD) {
    if (mixed) {
      AFAR_CUDA(cudaMemcpyAsync(s->xfer, FD, sizeof(V4<double>) * (Nc + Nb), cudaMemcpyHostToDevice, s->stream));
      k_convert4<double, float><<<grid_for(Nc + Nb, 256), 256, 0, s->stream>>>(
          (int)(Nc + Nb), static_cast<const V4<double>*>(s->xfer), static_cast<V4<float>*>(s->W));
    } else {
      AFAR_CUDA(cudaMemcpyAsync(s->W, FD, sizeof(V4<double>) * (Nc + Nb), cudaMemcpyHostToDevice, s->stream));
    }
  }
  const afar_conservedFieldData* src[2] = {cFD, cFDold};
  V4<double>* dst[2] = {s->U, s->U0};
  for (int i = 0; i < 2; ++i) {
    if (!src[i]) continue;
    if (i == 1 && cFDold == cFD) {  // the same host array twice: one upload, then a device copy
      AFAR_CUDA(cudaMemcpyAsync(s->U0, s->U, sizeof(V4<double>) * Nc, cudaMemcpyDeviceToDevice, s->stream));
      continue;
    }
    AFAR_CUDA(cudaMemcpyAsync(dst[i], src[i], sizeof(V4<double>) * Nc, cudaMemcpyHostToDevice, s->stream));
    if (mixed) k_df_from_double<<<grid_for(Nc, 256), 256, 0, s->stream>>>((int)Nc, dst[i]);
  }
  AFAR_CUDA(cudaGetLastError());
  AFAR_CUDA(cudaStreamSynchronize(s->stream));
  return AFAR_OK;
}

static afar_status get_state(afar_solver* s, afar_basicFieldData* FD, afar_conservedFieldData* cFD, int8_t* si) {
  const size_t Nc = s->Nc, Nb = s->Nb;
  const bool mixed = s->policy == AFAR_POLICY_MIXED;
  if (FD) {
    if (mixed) {
      k_convert4<float, double><<<grid_for(Nc + Nb, 256), 256, 0, s->stream>>>(
          (int)(Nc + Nb), static_cast<const V4<float>*>(s->W), static_cast<V4<double>*>(s->xfer));
      AFAR_CUDA(cudaMemcpyAsync(FD, s->xfer, sizeof(V4<double>) * (Nc + Nb), cudaMemcpyDeviceToHost, s->stream));
      AFAR_CUDA(cudaStreamSynchronize(s->stream));  // xfer is reused below
    } else {
      AFAR_CUDA(cudaMemcpyAsync(FD, s->W, sizeof(V4<double>) * (Nc + Nb), cudaMemcpyDeviceToHost, s->stream));
    }
  }
  if (cFD) {
    if (mixed) {
      k_df_to_double<<<grid_for(Nc, 256), 256, 0, s->stream>>>((int)Nc, reinterpret_cast<const DF4*>(s->U),
                                                               static_cast<V4<double>*>(s->xfer));
      AFAR_CUDA(cudaMemcpyAsync(cFD, s->xfer, sizeof(V4<double>) * Nc, cudaMemcpyDeviceToHost, s->stream));
    } else {
      AFAR_CUDA(cudaMemcpyAsync(cFD, s->U, sizeof(V4<double>) * Nc, cudaMemcpyDeviceToHost, s->stream));
    }
  }
  if (si) AFAR_CUDA(cudaMemcpyAsync(si, s->si, 2 * (Nc + Nb), cudaMemcpyDeviceToHost, s->stream));
  AFAR_CUDA(cudaGetLastError());
  AFAR_CUDA(cudaStreamSynchronize(s->stream));
  return AFAR_OK;
}

// The project autotuner: the mixed reconstruct has two implementations whose speed depends on the
// mesh (stencil size, faces per cell, size): the tile-staged kernel (TMA loads of each 128-cell
// tile's operator rows into shared memory) and the register pass (no shared memory, more tiles per
// SM).  At the stencil upload each is timed on the solver's own data (one warm-up, best of three
// launches, CUDA events on its stream; the launches only write the stage's intermediates) and the
// faster kept.  Decisions are cached per device and mesh class (faces per cell, stencil size, cell
// count to a factor of two), so later solvers of the same class skip the timing.
// cuTensorMapEncodeTiled, looked up once through the runtime (the library links no driver API).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// The tensor maps of the mixed tile-staged reconstruct (TileMaps): built on the host after the
// operator rows are in place and copied to the solver's device memory.  Each map describes one
// slot-major array as rows of ldc elements (ldc a multiple of 32, so every row stride is a multiple
// of 128 bytes), with boxes of 128 cells.
static afar_status build_tile_maps(afar_solver* s) {
  const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return (set_error("cuTensorMapEncodeTiled is not available from the driver"), AFAR_ERR_CUDA);
  TileMaps h;
  std::memset(&h, 0, sizeof(h));
  const cuuint64_t ldc = (cuuint64_t)s->ldc, M = (cuuint64_t)s->maxM, S = (cuuint64_t)s->maxS;
  const cuuint32_t one[3] = {1, 1, 1};
  auto encode = [&](CUtensorMap* m, CUtensorMapDataType dt, cuuint32_t rank, void* base, const cuuint64_t* dims,
                    const cuuint64_t* strides, const cuuint32_t* box) -> afar_status {
    const CUresult r = enc(m, dt, rank, base, dims, strides, box, one, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return (set_error("cuTensorMapEncodeTiled failed (%d)", (int)r), AFAR_ERR_CUDA);
    return AFAR_OK;
  };
  afar_status st;
  {
    const cuuint64_t dims[2] = {ldc, M}, strides[1] = {ldc * 4};
    const cuuint32_t box[2] = {(cuuint32_t)kTile, (cuuint32_t)M};
    if ((st = encode(&h.cf, CU_TENSOR_MAP_DATA_TYPE_INT32, 2, s->cf, dims, strides, box))) return st;
  }
  {
    const cuuint64_t dims[2] = {2 * ldc, M}, strides[1] = {ldc * 8};
    const cuuint32_t box[2] = {(cuuint32_t)(2 * kTile), (cuuint32_t)M};
    if ((st = encode(&h.lsm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, s->lsm, dims, strides, box))) return st;
    if ((st = encode(&h.sg, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, s->sg, dims, strides, box))) return st;
    if ((st = encode(&h.sr, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, s->sr, dims, strides, box))) return st;
  }
  for (cuuint32_t k = 1; k <= (cuuint32_t)S; ++k) {
    const cuuint64_t dims[2] = {ldc, S}, strides[1] = {ldc * 4};
    const cuuint32_t box[2] = {(cuuint32_t)kTile, k};
    if ((st = encode(&h.sten[k - 1], CU_TENSOR_MAP_DATA_TYPE_INT32, 2, s->sten, dims, strides, box))) return st;
    const cuuint64_t wdims[3] = {ldc, S + 1, M}, wstrides[2] = {ldc * 4, ldc * 4 * (S + 1)};
    const cuuint32_t wbox[3] = {(cuuint32_t)kTile, k, (cuuint32_t)M};
    if ((st = encode(&h.wts[k - 1], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, s->wts, wdims, wstrides, wbox))) return st;
  }
  if (!s->tmaps) {
    void* p = nullptr;
    if ((st = dalloc(s, &p, sizeof(TileMaps)))) return st;
    s->tmaps = static_cast<TileMaps*>(p);
  }
  AFAR_CUDA(cudaMemcpy(s->tmaps, &h, sizeof(TileMaps), cudaMemcpyHostToDevice));
  return AFAR_OK;
}

static afar_status tune_reconstruct(afar_solver* s) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int>, int> cache;
  if (s->recon_request >= 0) {
    s->recon_variant = s->recon_request;
    return AFAR_OK;
  }
  int lg = 0;
  while ((1 << (lg + 1)) <= s->Nc) ++lg;
  const auto key = std::make_tuple(s->device, s->maxM, s->maxS, lg);
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) {
      s->recon_variant = it->second;
      s->tune_ms[0] = s->tune_ms[1] = 0.f;
      return AFAR_OK;
    }
  }
  Stage<PolicyMixed> sg;
  afar_status st = make_stage<PolicyMixed>(s, false, &sg);
  if (st) return st;
  cudaEvent_t e0, e1;
  AFAR_CUDA(cudaEventCreate(&e0));
  AFAR_CUDA(cudaEventCreate(&e1));
  float best[2];
  for (int v = 0; v < 2; ++v) {
    s->recon_variant = v;
    sg.reconstruct();  // warm-up
    best[v] = 1e30f;
    for (int k = 0; k < 3; ++k) {
      AFAR_CUDA(cudaEventRecord(e0, s->stream));
      sg.reconstruct();
      AFAR_CUDA(cudaEventRecord(e1, s->stream));
      AFAR_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      AFAR_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      best[v] = std::min(best[v], ms);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  AFAR_CUDA(cudaGetLastError());
  if ((st = check_device_error(s))) return st;
  s->recon_variant = best[1] < best[0] ? 1 : 0;
  s->tune_ms[0] = best[0];
  s->tune_ms[1] = best[1];
  std::lock_guard<std::mutex> lock(mu);
  cache[key] = s->recon_variant;
  return AFAR_OK;
}

extern "C" afar_status afar_set_tuning(afar_solver* s, int reconVariant) {
  if (!s || reconVariant < -1 || reconVariant > 1) return (set_error("afar_set_tuning: variant -1, 0 or 1"), AFAR_ERR_ARGUMENT);
  s->recon_request = reconVariant;
  if (!s->have_stencil || s->policy != AFAR_POLICY_MIXED) return AFAR_OK;
  AFAR_CUDA(cudaSetDevice(s->device));
  afar_status st = tune_reconstruct(s);
  if (st) return st;
  return s->graph ? capture_graph(s) : AFAR_OK;
}

extern "C" afar_status afar_get_tuning(afar_solver* s, int* reconVariant, float* msTile, float* msRegister) {
  if (!s || !reconVariant) return (set_error("null argument"), AFAR_ERR_ARGUMENT);
  *reconVariant = s->recon_variant;
  if (msTile) *msTile = s->tune_ms[0];
  if (msRegister) *msRegister = s->tune_ms[1];
  return AFAR_OK;
}

extern "C" afar_status afar_setDeviceFieldData(afar_solver* s, const afar_fieldPointer* h, int cellsNum, int facesNum,
                                               int totalBoundaryFacesNum) {
  if (!s || !h || !h->CELL || !h->FACE || !h->cellVolume || !h->FD || !h->cFD || cellsNum <= 0 || facesNum < 0 ||
      totalBoundaryFacesNum < 0) {
    set_error("afar_setDeviceFieldData: null array or bad size");
    return AFAR_ERR_ARGUMENT;
  }
  if (s->have_fields) {
    set_error("afar_setDeviceFieldData: already called on this solver");
    return AFAR_ERR_STATE;
  }
  AFAR_CUDA(cudaSetDevice(s->device));
  s->Nc = cellsNum;
  s->Nf = facesNum;
  s->Nb = totalBoundaryFacesNum;
  s->ldc = (cellsNum + 31) / 32 * 32;
  const size_t Nc = cellsNum, Nf = facesNum, Nb = totalBoundaryFacesNum;
  afar_status st;
  if ((st = dalloc_t(s, &s->cellC, Nc + Nb))) return st;
  if ((st = dalloc_t(s, &s->faceRaw, Nf + Nb))) return st;
  if ((st = dalloc_t(s, &s->vol, Nc))) return st;
  if ((st = dalloc_t(s, &s->vinv, Nc))) return st;
  if (s->policy == AFAR_POLICY_MIXED) {
    if ((st = dalloc_t(s, &s->vinvf, Nc))) return st;
    if ((st = dalloc(s, &s->xfer, sizeof(V4<double>) * (Nc + Nb)))) return st;
  }
  if ((st = dalloc_t(s, &s->U, Nc))) return st;
  if ((st = dalloc_t(s, &s->U0, Nc))) return st;
  if ((st = dalloc_t(s, &s->si, 2 * (Nc + Nb)))) return st;
  if ((st = dalloc_t(s, &s->ctl, 1))) return st;
  if ((st = dalloc_t(s, &s->dt_bits, 1))) return st;
  if ((st = dalloc(s, &s->W, w_size(s->policy) * (Nc + Nb)))) return st;
  AFAR_CUDA(cudaMemcpyAsync(s->cellC, h->CELL, sizeof(V2<double>) * (Nc + Nb), cudaMemcpyHostToDevice, s->stream));
  AFAR_CUDA(cudaMemcpyAsync(s->faceRaw, h->FACE, sizeof(FaceRaw) * (Nf + Nb), cudaMemcpyHostToDevice, s->stream));
  AFAR_CUDA(cudaMemcpyAsync(s->vol, h->cellVolume, sizeof(double) * Nc, cudaMemcpyHostToDevice, s->stream));
  k_reciprocal<<<grid_for(Nc, 256), 256, 0, s->stream>>>((int)Nc, s->vol, s->vinv, s->vinvf);
  AFAR_CUDA(cudaMemsetAsync(s->si, 0, 2 * (Nc + Nb), s->stream));
  if ((st = put_state(s, reinterpret_cast<const afar_basicFieldData*>(h->FD),
                      reinterpret_cast<const afar_conservedFieldData*>(h->cFD),
                      reinterpret_cast<const afar_conservedFieldData*>(h->cFD))))
    return st;
  k_init_ctl<<<1, 32, 0, s->stream>>>(s->ctl);
  // intermediates
  const size_t g = s->policy == AFAR_POLICY_MIXED ? sizeof(V4<float>) : sizeof(V4<double>);
  const size_t l = s->policy == AFAR_POLICY_FP64 ? sizeof(V4<double>) : sizeof(V4<float>);
  if ((st = dalloc(s, &s->grad, g * 2 * Nc))) return st;
  if ((st = dalloc(s, &s->lim, l * Nc))) return st;
  if ((st = dalloc(s, &s->fv, g * 2 * Nf))) return st;
  if ((st = dalloc(s, &s->flux, g * (Nf + Nb)))) return st;
  if ((st = dalloc_t(s, &s->dtg, Nf))) return st;
  if ((st = dalloc_t(s, &s->bn, Nb))) return st;
  AFAR_CUDA(cudaMemsetAsync(s->fv, 0, g * 2 * Nf, s->stream));
  AFAR_CUDA(cudaStreamSynchronize(s->stream));
  AFAR_CUDA(cudaGetLastError());
  s->have_fields = true;
  return AFAR_OK;
}

extern "C" afar_status afar_set_rbf_basis64(afar_solver* s, const double* rbf, size_t count) {
  if (!s || (!rbf && count)) {
    set_error("afar_set_rbf_basis64: null argument");
    return AFAR_ERR_ARGUMENT;
  }
  s->head_pending = false;
  s->rbf64.assign(rbf, rbf + count);
  return AFAR_OK;
}

extern "C" afar_status afar_setDeviceFieldDataStencil(afar_solver* s, const afar_fieldPointer* h, int cellsNum,
                                                      int facesNum, int patchesNum, int totalBoundaryFacesNum,
                                                      int maxStencilSize, int maxCompactStencilSize,
                                                      int maxLocalBlockStencilSize,
                                                      int maxCompactLocalBlockStencilSize) {
  NvtxRange nvtx("afar_setDeviceFieldDataStencil");
  if (!s || !h) {
    set_error("afar_setDeviceFieldDataStencil: null argument");
    return AFAR_ERR_ARGUMENT;
  }
  if (!s->have_fields) {
    set_error("afar_setDeviceFieldDataStencil: call afar_setDeviceFieldData first");
    return AFAR_ERR_STATE;
  }
  if (s->have_stencil) {
    set_error("afar_setDeviceFieldDataStencil: already called on this solver");
    return AFAR_ERR_STATE;
  }
  if (cellsNum != s->Nc || facesNum != s->Nf || totalBoundaryFacesNum != s->Nb) {
    set_error("afar_setDeviceFieldDataStencil: sizes differ from afar_setDeviceFieldData");
    return AFAR_ERR_ARGUMENT;
  }
  if (maxStencilSize < 1 || maxStencilSize > AFAR_MAX_VALID_STENCIL_SIZE || maxCompactStencilSize < 1 ||
      maxCompactStencilSize > maxStencilSize || maxCompactStencilSize > kMaxFaces ||
      maxLocalBlockStencilSize < AFAR_BLOCKDIM ||
      maxCompactLocalBlockStencilSize < AFAR_BLOCKDIM || patchesNum < 0) {
    set_error("afar_setDeviceFieldDataStencil: stencil sizes out of range (maxS %d, maxM %d, maxLB %d)",
              maxStencilSize, maxCompactStencilSize, maxLocalBlockStencilSize);
    return AFAR_ERR_LIMIT;
  }
  if (!h->neighbour && facesNum > 0) return (set_error("neighbour is null"), AFAR_ERR_ARGUMENT);
  if (!h->stencilSize || !h->compactStencilSize || !h->localStencil || !h->cellFaces || !h->RBFbasis ||
      (totalBoundaryFacesNum > 0 && (!h->boundaryFaceNeiLabel || !h->boundaryFacesType)) ||
      (maxLocalBlockStencilSize > AFAR_BLOCKDIM && !h->extendStencil)) {
    set_error("afar_setDeviceFieldDataStencil: null stencil array");
    return AFAR_ERR_ARGUMENT;
  }
  AFAR_CUDA(cudaSetDevice(s->device));
  const int Nc = s->Nc, Nf = s->Nf, Nb = s->Nb;
  // host-side validation of everything a kernel indexes with
  for (int c = 0; c < Nc; ++c) {
    if (h->stencilSize[c] > maxStencilSize || h->compactStencilSize[c] > maxCompactStencilSize ||
        h->compactStencilSize[c] > h->stencilSize[c]) {
      set_error("cell %d: stencil sizes %d/%d exceed the declared maxima", c, h->stencilSize[c], h->compactStencilSize[c]);
      return AFAR_ERR_ARGUMENT;
    }
    for (int i = 0; i < h->compactStencilSize[c]; ++i) {
      const int fid = h->cellFaces[(size_t)maxCompactStencilSize * c + i];
      const int f = (fid < 0 ? -fid : fid) - 1;
      if (fid == 0 || f >= Nf + Nb || (f >= Nf && fid < 0)) {
        set_error("cell %d: cellFaces entry %d out of range", c, fid);
        return AFAR_ERR_ARGUMENT;
      }
    }
    const int blk = c / AFAR_BLOCKDIM;
    for (int i = 0; i < h->stencilSize[c]; ++i) {
      const int loc = h->localStencil[(size_t)maxStencilSize * c + i];
      if (loc >= maxLocalBlockStencilSize) {
        set_error("cell %d: localStencil entry %d out of range", c, loc);
        return AFAR_ERR_ARGUMENT;
      }
      const int g = loc < AFAR_BLOCKDIM ? blk * AFAR_BLOCKDIM + loc
                                        : h->extendStencil[(size_t)(maxLocalBlockStencilSize - AFAR_BLOCKDIM) * blk + (loc - AFAR_BLOCKDIM)];
      if (g < 0 || g >= Nc + Nb || (loc < AFAR_BLOCKDIM && g >= Nc)) {
        set_error("cell %d: stencil member %d out of range", c, g);
        return AFAR_ERR_ARGUMENT;
      }
    }
  }
  for (int f = 0; f < Nf; ++f) {
    const int o = h->neighbour[2 * f], n = h->neighbour[2 * f + 1];
    if (o < 0 || o >= Nc || n < 0 || n >= Nc) {
      set_error("face %d: owner/neighbour (%d, %d) out of range", f, o, n);
      return AFAR_ERR_ARGUMENT;
    }
  }
  for (int b = 0; b < Nb; ++b) {
    if (h->boundaryFaceNeiLabel[b] < 0 || h->boundaryFaceNeiLabel[b] >= Nc) {
      set_error("boundary face %d: owner out of range", b);
      return AFAR_ERR_ARGUMENT;
    }
    if (h->boundaryFacesType[b] > AFAR_BC_FIXED_INITIAL) {
      set_error("boundary face %d: unknown boundary label %d (cudaEulerBCs 0-5, or 6)", b, h->boundaryFacesType[b]);
      return AFAR_ERR_ARGUMENT;
    }
  }
  s->patches = patchesNum;
  s->maxS = maxStencilSize;
  s->maxM = maxCompactStencilSize;
  s->maxLB = maxLocalBlockStencilSize;
  s->maxCLB = maxCompactLocalBlockStencilSize;
  const size_t ldc = s->ldc;
  afar_status st;
  if ((st = dalloc_t(s, &s->on, (size_t)Nf))) return st;
  if ((st = dalloc_t(s, &s->bnei, (size_t)Nb))) return st;
  if ((st = dalloc_t(s, &s->btype, (size_t)Nb))) return st;
  if ((st = dalloc_t(s, &s->nS, (size_t)Nc))) return st;
  if ((st = dalloc_t(s, &s->nM, (size_t)Nc))) return st;
  if ((st = dalloc_t(s, &s->sten, (size_t)s->maxS * ldc))) return st;
  if ((st = dalloc_t(s, &s->cf, (size_t)s->maxM * ldc))) return st;
  AFAR_CUDA(cudaMemsetAsync(s->sten, 0, sizeof(int) * s->maxS * ldc, s->stream));
  AFAR_CUDA(cudaMemsetAsync(s->cf, 0, sizeof(int) * s->maxM * ldc, s->stream));
  if (Nf) AFAR_CUDA(cudaMemcpyAsync(s->on, h->neighbour, sizeof(int2) * Nf, cudaMemcpyHostToDevice, s->stream));
  if (Nb) {
    AFAR_CUDA(cudaMemcpyAsync(s->bnei, h->boundaryFaceNeiLabel, sizeof(int) * Nb, cudaMemcpyHostToDevice, s->stream));
    AFAR_CUDA(cudaMemcpyAsync(s->btype, h->boundaryFacesType, Nb, cudaMemcpyHostToDevice, s->stream));
  }
  AFAR_CUDA(cudaMemcpyAsync(s->nS, h->stencilSize, Nc, cudaMemcpyHostToDevice, s->stream));
  {
    const int ntile = (Nc + kTile - 1) / kTile;
    std::vector<uint8_t> ts(ntile, 0);
    for (int c = 0; c < Nc; ++c) ts[c / kTile] = std::max(ts[c / kTile], h->stencilSize[c]);
    for (auto& v : ts) v = std::max<uint8_t>(v, 1);  // the tile kernel loads the boxes of stencil size v
    if ((st = dalloc_t(s, &s->tileS, (size_t)ntile))) return st;
    AFAR_CUDA(cudaMemcpy(s->tileS, ts.data(), ntile, cudaMemcpyHostToDevice));
  }
  AFAR_CUDA(cudaMemcpyAsync(s->nM, h->compactStencilSize, Nc, cudaMemcpyHostToDevice, s->stream));
  {
    uint16_t* dls = nullptr;
    int* dext = nullptr;
    int* dcf = nullptr;
    const size_t nblk = (Nc + AFAR_BLOCKDIM - 1) / AFAR_BLOCKDIM;
    const size_t next = (size_t)(s->maxLB - AFAR_BLOCKDIM) * nblk;
    AFAR_CUDA(cudaMalloc(&dls, sizeof(uint16_t) * (size_t)s->maxS * Nc));
    AFAR_CUDA(cudaMalloc(&dext, sizeof(int) * (next ? next : 1)));
    AFAR_CUDA(cudaMalloc(&dcf, sizeof(int) * (size_t)s->maxM * Nc));
    AFAR_CUDA(cudaMemcpyAsync(dls, h->localStencil, sizeof(uint16_t) * (size_t)s->maxS * Nc, cudaMemcpyHostToDevice, s->stream));
    if (next) AFAR_CUDA(cudaMemcpyAsync(dext, h->extendStencil, sizeof(int) * next, cudaMemcpyHostToDevice, s->stream));
    AFAR_CUDA(cudaMemcpyAsync(dcf, h->cellFaces, sizeof(int) * (size_t)s->maxM * Nc, cudaMemcpyHostToDevice, s->stream));
    k_setup_lists<<<grid_for(Nc, kCellBlock), kCellBlock, 0, s->stream>>>(Nc, s->ldc, s->maxS, s->maxM, s->maxLB, s->nS,
                                                                           s->nM, dls, dext, dcf, s->sten, s->cf);
    AFAR_CUDA(cudaGetLastError());
    AFAR_CUDA(cudaStreamSynchronize(s->stream));
    cudaFree(dls);
    cudaFree(dext);
    cudaFree(dcf);
  }
  switch (s->policy) {
    case AFAR_POLICY_REF: st = setup_operators<PolicyRef>(s, h); break;
    case AFAR_POLICY_FP64: st = setup_operators<PolicyFP64>(s, h); break;
    default: st = setup_operators<PolicyMixed>(s, h); break;
  }
  if (st) return st;
  if ((st = dalloc_t(s, &s->res_dbg, (size_t)Nc))) return st;
  AFAR_CUDA(cudaStreamSynchronize(s->stream));
  if (s->policy == AFAR_POLICY_MIXED && (st = build_tile_maps(s))) return st;
  if (s->policy == AFAR_POLICY_MIXED && (st = tune_reconstruct(s))) return st;
  s->have_stencil = true;
  return AFAR_OK;
}

static afar_status ensure_graph(afar_solver* s, double R, double Cv) {
  if (!s->graph || s->R != R || s->Cv != Cv) {
    if (!s->have_stencil) {  // capture needs the operators; keep the constants for later
      s->R = R;
      s->Cv = Cv;
      return AFAR_OK;
    }
    s->R = R;
    s->Cv = Cv;
    return capture_graph(s);
  }
  return AFAR_OK;
}

extern "C" afar_status afar_adjustTimeStep(afar_solver* s, int facesNum, double R, double Cv, double CFL, double* dt) {
  NvtxRange nvtx("afar_adjustTimeStep");
  afar_status st = check_ready(s);
  if (st) return st;
  if (!dt || facesNum != s->Nf || !(R > 0.0) || !(Cv > 0.0) || !(CFL > 0.0)) {
    set_error("afar_adjustTimeStep: bad argument");
    return AFAR_ERR_ARGUMENT;
  }
  const unsigned long long init = 0x40F86A0000000000ull;  // bits of 1e5
  // Outside a batch the Courant step comes from the head of the coming step -- stage 1 up to its
  // flux, whose fused reduction is the same Courant minimum over the internal faces (the ref
  // policy's head runs the reference-shaped Courant kernel itself) -- so no separate pass runs and
  // the afar_GPUevolve that follows runs only the tail of the step.
  if (!s->batch && s->Nf > 0) {
    if ((st = ensure_graph(s, R, Cv))) return st;
    if (s->graph_head) {
      k_set_ctl<<<1, 32, 0, s->stream>>>(s->ctl, 0.0, CFL, 0.0);
      AFAR_CUDA(cudaMemcpyAsync(&s->ctl->dt_bits, &init, sizeof(init), cudaMemcpyHostToDevice, s->stream));
      AFAR_CUDA(cudaGraphLaunch(s->graph_head, s->stream));
      StepCtl c;
      AFAR_CUDA(cudaMemcpyAsync(&c, s->ctl, sizeof(c), cudaMemcpyDeviceToHost, s->stream));
      AFAR_CUDA(cudaStreamSynchronize(s->stream));
      AFAR_CUDA(cudaGetLastError());
      if (c.err) {  // a bounded device wait gave up, in this head or in the step before it
        AFAR_CUDA(cudaMemsetAsync(&s->ctl->err, 0, sizeof(c.err), s->stream));
        AFAR_CUDA(cudaStreamSynchronize(s->stream));
        set_error("a device-side wait for a bulk copy timed out (error word %u); the state is not valid", c.err);
        return AFAR_ERR_CUDA;
      }
      std::memcpy(dt, &c.dt_bits, sizeof(double));
      s->head_pending = true;
      return AFAR_OK;
    }
  }
  AFAR_CUDA(cudaMemcpyAsync(s->dt_bits, &init, sizeof(init), cudaMemcpyHostToDevice, s->stream));
  const int gf = grid_for(s->Nf, kFaceBlock);
  if (s->Nf > 0) {
    switch (s->policy) {
      case AFAR_POLICY_REF: {
        StageArgs<PolicyRef> a = make_args<PolicyRef>(s);
        a.R = R;
        a.Cv = Cv;
        k_delta_t<PolicyRef><<<gf, kFaceBlock, 0, s->stream>>>(a, CFL, s->dt_bits, nullptr);
        break;
      }
      case AFAR_POLICY_FP64: {
        StageArgs<PolicyFP64> a = make_args<PolicyFP64>(s);
        a.R = R;
        a.Cv = Cv;
        k_delta_t<PolicyFP64><<<gf, kFaceBlock, 0, s->stream>>>(a, CFL, s->dt_bits, nullptr);
        break;
      }
      default: {  // the mixed policy's FP32 Courant estimate, as in its fused stage-1 flux
        StageArgs<PolicyMixed> a = make_args<PolicyMixed>(s);
        a.gRf = (float)((R / Cv + 1.0) * R);
        k_delta_t_mixed<<<gf, kFaceBlock, 0, s->stream>>>(a, (float)CFL, s->dt_bits);
        break;
      }
    }
  }
  unsigned long long bits = 0;
  AFAR_CUDA(cudaMemcpyAsync(&bits, s->dt_bits, sizeof(bits), cudaMemcpyDeviceToHost, s->stream));
  AFAR_CUDA(cudaStreamSynchronize(s->stream));
  AFAR_CUDA(cudaGetLastError());
  double v;
  std::memcpy(&v, &bits, sizeof(v));
  *dt = v;
  return AFAR_OK;
}

static afar_status run_impl(afar_solver* s, int nSteps, double dt, double CFL, double tEnd, bool wait) {
  NvtxRange nvtx("afar_run");
  afar_status st = check_ready(s);
  if (st || (st = check_not_batched(s))) return st;
  if (nSteps < 0 || (!(dt > 0.0) && !(CFL > 0.0))) {
    set_error("afar_run: nSteps must be >= 0 and either deltaT > 0 or CFL > 0");
    return AFAR_ERR_ARGUMENT;
  }
  if (!(s->R > 0.0)) return (set_error("call afar_set_gas (or afar_GPUevolve) first"), AFAR_ERR_STATE);
  if ((st = ensure_graph(s, s->R, s->Cv))) return st;
  k_set_ctl<<<1, 32, 0, s->stream>>>(s->ctl, dt > 0.0 ? dt : 0.0, CFL, tEnd);
  for (int i = 0; i < nSteps; ++i) AFAR_CUDA(cudaGraphLaunch(s->graph, s->stream));
  AFAR_CUDA(cudaGetLastError());
  if (wait) return check_device_error(s);
  return AFAR_OK;
}

extern "C" afar_status afar_GPUevolve(afar_solver* s, double R, double Cv, double deltaT, int cellsNum, int facesNum,
                                      int totalBoundaryFacesNum, int maxStencilSize, int maxCompactStencilSize,
                                      int maxLocalBlockStencilSize, int maxCompactLocalBlockStencilSize) {
  NvtxRange nvtx("afar_GPUevolve");
  const bool head_done = s && s->head_pending;  // read before check_ready clears it
  afar_status st = check_ready(s);
  if (st) return st;
  if (cellsNum != s->Nc || facesNum != s->Nf || totalBoundaryFacesNum != s->Nb || maxStencilSize != s->maxS ||
      maxCompactStencilSize != s->maxM) {
    set_error("afar_GPUevolve: sizes differ from the uploaded fields");
    return AFAR_ERR_ARGUMENT;
  }
  (void)maxLocalBlockStencilSize;
  (void)maxCompactLocalBlockStencilSize;
  if (!(deltaT > 0.0) || !(R > 0.0) || !(Cv > 0.0)) {
    set_error("afar_GPUevolve: deltaT, R and Cv must be positive");
    return AFAR_ERR_ARGUMENT;
  }
  if (head_done && s->graph_tail && s->R == R && s->Cv == Cv) {
    // afar_adjustTimeStep ran this step's head on the current state: the tail with the caller's
    // step size completes it, the same kernels as the whole-step graph.  Enqueued, not waited
    // for: a device-side error of the step surfaces at the next call that waits.
    k_set_ctl<<<1, 32, 0, s->stream>>>(s->ctl, deltaT, 1.0, 0.0);
    AFAR_CUDA(cudaGraphLaunch(s->graph_tail, s->stream));
    AFAR_CUDA(cudaGetLastError());
    return AFAR_OK;
  }
  if ((st = ensure_graph(s, R, Cv))) return st;
  return run_impl(s, 1, deltaT, 1.0, 0.0, true);
}

extern "C" afar_status afar_set_gas(afar_solver* s, double R, double Cv) {
  if (!s || !(R > 0.0) || !(Cv > 0.0)) {
    set_error("afar_set_gas: bad argument");
    return AFAR_ERR_ARGUMENT;
  }
  s->head_pending = false;
  return ensure_graph(s, R, Cv);
}

extern "C" afar_status afar_run(afar_solver* s, int nSteps, double deltaT, double CFL, double tEnd) {
  return run_impl(s, nSteps, deltaT, CFL, tEnd, true);
}

extern "C" afar_status afar_run_async(afar_solver* s, int nSteps, double deltaT, double CFL, double tEnd) {
  return run_impl(s, nSteps, deltaT, CFL, tEnd, false);
}

extern "C" afar_status afar_run_timed(afar_solver* s, int nSteps, double dt, double CFL, double tEnd, float* ms) {
  afar_status st = check_ready(s);
  if (st || (st = check_not_batched(s))) return st;
  if (!ms) return (set_error("null output"), AFAR_ERR_ARGUMENT);
  if (!(s->R > 0.0)) return (set_error("call afar_set_gas (or afar_GPUevolve) first"), AFAR_ERR_STATE);
  if ((st = ensure_graph(s, s->R, s->Cv))) return st;
  cudaEvent_t e0, e1;
  AFAR_CUDA(cudaEventCreate(&e0));
  AFAR_CUDA(cudaEventCreate(&e1));
  k_set_ctl<<<1, 32, 0, s->stream>>>(s->ctl, dt > 0.0 ? dt : 0.0, CFL, tEnd);
  AFAR_CUDA(cudaEventRecord(e0, s->stream));
  for (int i = 0; i < nSteps; ++i) AFAR_CUDA(cudaGraphLaunch(s->graph, s->stream));
  AFAR_CUDA(cudaEventRecord(e1, s->stream));
  AFAR_CUDA(cudaEventSynchronize(e1));
  AFAR_CUDA(cudaEventElapsedTime(ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  AFAR_CUDA(cudaGetLastError());
  return check_device_error(s);
}

extern "C" afar_status afar_profile_step(afar_solver* s, double dt, double CFL, float ms[5]) {
  afar_status st = check_ready(s);
  if (st || (st = check_not_batched(s))) return st;
  if (!ms) return (set_error("null output"), AFAR_ERR_ARGUMENT);
  if (!(s->R > 0.0)) return (set_error("call afar_set_gas (or afar_GPUevolve) first"), AFAR_ERR_STATE);
  cudaEvent_t ev[32];
  for (int i = 0; i < 32; ++i) AFAR_CUDA(cudaEventCreate(&ev[i]));
  k_set_ctl<<<1, 32, 0, s->stream>>>(s->ctl, dt > 0.0 ? dt : 0.0, CFL, 0.0);
  int n = 0;
  int kind[32];
  auto mark = [&](int k) {
    cudaEventRecord(ev[n], s->stream);
    kind[n++] = k;
  };
  auto body = [&](auto tag) -> afar_status {
    using P = decltype(tag);
    Stage<P> sg;
    afar_status r = make_stage<P>(s, false, &sg);
    if (r) return r;
    mark(-1);
    for (int k = 0; k < 3; ++k) {
      sg.reconstruct();
      mark(0);
      sg.bvd();
      mark(1);
      sg.flux(k == 0);
      mark(2);
      sg.update(k);
      mark(3);
    }
    k_finish_step<<<1, 32, 0, s->stream>>>(s->ctl);
    mark(4);
    return AFAR_OK;
  };
  switch (s->policy) {
    case AFAR_POLICY_REF: st = body(PolicyRef{}); break;
    case AFAR_POLICY_FP64: st = body(PolicyFP64{}); break;
    default: st = body(PolicyMixed{}); break;
  }
  if (st) return st;
  AFAR_CUDA(cudaEventSynchronize(ev[n - 1]));
  for (int k = 0; k < 5; ++k) ms[k] = 0.f;
  for (int i = 1; i < n; ++i) {
    float t = 0.f;
    AFAR_CUDA(cudaEventElapsedTime(&t, ev[i - 1], ev[i]));
    ms[kind[i]] += t;
  }
  for (int i = 0; i < 32; ++i) cudaEventDestroy(ev[i]);
  AFAR_CUDA(cudaGetLastError());
  return check_device_error(s);
}

extern "C" afar_status afar_synchronize(afar_solver* s) {
  if (!s) return (set_error("null solver"), AFAR_ERR_ARGUMENT);
  AFAR_CUDA(cudaSetDevice(s->device));
  AFAR_CUDA(cudaStreamSynchronize(s->stream));
  AFAR_CUDA(cudaGetLastError());
  return AFAR_OK;
}

extern "C" afar_status afar_get_stream(afar_solver* s, void** stream) {
  if (!s || !stream) return (set_error("null argument"), AFAR_ERR_ARGUMENT);
  *stream = (void*)s->stream;
  return AFAR_OK;
}

extern "C" afar_status afar_get_time(afar_solver* s, double* t, double* lastDt, long long* steps) {
  if (!s || !s->have_fields) return (set_error("solver not initialised"), AFAR_ERR_STATE);
  AFAR_CUDA(cudaSetDevice(s->device));
  StepCtl c;
  AFAR_CUDA(cudaMemcpyAsync(&c, s->ctl, sizeof(c), cudaMemcpyDeviceToHost, s->stream));
  AFAR_CUDA(cudaStreamSynchronize(s->stream));
  if (t) *t = c.t;
  if (lastDt) *lastDt = c.last_dt;
  if (steps) *steps = c.steps;
  return AFAR_OK;
}

extern "C" afar_status afar_set_time(afar_solver* s, double t) {
  if (!s || !s->have_fields) return (set_error("solver not initialised"), AFAR_ERR_STATE);
  s->head_pending = false;
  AFAR_CUDA(cudaSetDevice(s->device));
  AFAR_CUDA(cudaMemcpyAsync(&s->ctl->t, &t, sizeof(double), cudaMemcpyHostToDevice, s->stream));
  AFAR_CUDA(cudaStreamSynchronize(s->stream));
  return AFAR_OK;
}

extern "C" afar_status afar_stage_debug(afar_solver* s, int stage, double deltaT, afar_fieldPointer* out) {
  afar_status st = check_ready(s);
  if (st || (st = check_not_batched(s))) return st;
  if (stage < 0 || stage > 2 || !(deltaT > 0.0) || !out) {
    set_error("afar_stage_debug: stage must be 0..2, deltaT > 0, out non-null");
    return AFAR_ERR_ARGUMENT;
  }
  if (!(s->R > 0.0)) return (set_error("call afar_set_gas (or afar_GPUevolve) first"), AFAR_ERR_STATE);
  k_set_ctl<<<1, 32, 0, s->stream>>>(s->ctl, deltaT, 1.0, 0.0);
  const size_t Nc = s->Nc, Nf = s->Nf, Nb = s->Nb;
  const bool mixed = s->policy == AFAR_POLICY_MIXED;
  const bool f64 = s->policy == AFAR_POLICY_FP64;
  auto run = [&](auto tag) -> afar_status {
    using P = decltype(tag);
    Stage<P> sg;
    afar_status r = make_stage<P>(s, true, &sg);
    if (r) return r;
    sg.reconstruct();
    sg.bvd();
    sg.flux(false);
    sg.update(stage);
    return AFAR_OK;
  };
  switch (s->policy) {
    case AFAR_POLICY_REF: st = run(PolicyRef{}); break;
    case AFAR_POLICY_FP64: st = run(PolicyFP64{}); break;
    default: st = run(PolicyMixed{}); break;
  }
  if (st) return st;
  AFAR_CUDA(cudaGetLastError());
  AFAR_CUDA(cudaStreamSynchronize(s->stream));
  // copy out in the reference layout
  auto get4 = [&](void* dst, const void* src, size_t n, bool is_float) -> afar_status {
    if (!is_float) {
      AFAR_CUDA(cudaMemcpy(dst, src, n * sizeof(V4<double>), cudaMemcpyDeviceToHost));
    } else {
      std::vector<V4<float>> tmp(n);
      AFAR_CUDA(cudaMemcpy(tmp.data(), src, n * sizeof(V4<float>), cudaMemcpyDeviceToHost));
      V4<double>* d = static_cast<V4<double>*>(dst);
      for (size_t i = 0; i < n; ++i) d[i] = V4<double>{tmp[i].x, tmp[i].y, tmp[i].z, tmp[i].w};
    }
    return AFAR_OK;
  };
  if (out->faceFD && (st = get4(out->faceFD, s->fv, 2 * Nf, mixed))) return st;
  if (out->gradFD && (st = get4(out->gradFD, s->grad, 2 * Nc, mixed))) return st;
  if (out->Flux && (st = get4(out->Flux, s->flux, Nf + Nb, mixed))) return st;
  if (out->FD && (st = get4(out->FD, s->W, Nc + Nb, mixed))) return st;
  if (out->cFD && (st = get_state(s, nullptr, reinterpret_cast<afar_conservedFieldData*>(out->cFD), nullptr)))
    return st;
  if (out->Res) AFAR_CUDA(cudaMemcpy(out->Res, s->res_dbg, Nc * sizeof(V4<double>), cudaMemcpyDeviceToHost));
  if (out->shockIndicator) AFAR_CUDA(cudaMemcpy(out->shockIndicator, s->si, 2 * (Nc + Nb), cudaMemcpyDeviceToHost));
  if (out->limiter) {
    if (f64) {
      std::vector<V4<double>> tmp(Nc);
      AFAR_CUDA(cudaMemcpy(tmp.data(), s->lim, Nc * sizeof(V4<double>), cudaMemcpyDeviceToHost));
      for (size_t i = 0; i < Nc; ++i)
        out->limiter[i] = afar_limiterFieldData{(float)tmp[i].x, (float)tmp[i].y, (float)tmp[i].z, (float)tmp[i].w};
    } else {
      AFAR_CUDA(cudaMemcpy(out->limiter, s->lim, Nc * sizeof(V4<float>), cudaMemcpyDeviceToHost));
    }
  }
  return AFAR_OK;
}

extern "C" afar_status afar_debug_limiter64(afar_solver* s, double* lim) {
  afar_status st = check_ready(s);
  if (st) return st;
  if (!lim) return (set_error("null output"), AFAR_ERR_ARGUMENT);
  const size_t Nc = s->Nc;
  if (s->policy == AFAR_POLICY_FP64) {
    AFAR_CUDA(cudaMemcpy(lim, s->lim, Nc * sizeof(V4<double>), cudaMemcpyDeviceToHost));
  } else {
    std::vector<float> tmp(4 * Nc);
    AFAR_CUDA(cudaMemcpy(tmp.data(), s->lim, Nc * sizeof(V4<float>), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < 4 * Nc; ++i) lim[i] = tmp[i];
  }
  return AFAR_OK;
}

extern "C" afar_status afar_upload_state(afar_solver* s, const afar_basicFieldData* FD, const afar_conservedFieldData* cFD,
                                         const afar_conservedFieldData* cFDold) {
  if (!s || !s->have_fields) return (set_error("solver not initialised"), AFAR_ERR_STATE);
  s->head_pending = false;
  AFAR_CUDA(cudaSetDevice(s->device));
  return put_state(s, FD, cFD, cFDold);
}

extern "C" afar_status afar_download_state(afar_solver* s, afar_basicFieldData* FD, afar_conservedFieldData* cFD,
                                           int8_t* shockIndicator) {
  if (!s || !s->have_fields) return (set_error("solver not initialised"), AFAR_ERR_STATE);
  AFAR_CUDA(cudaSetDevice(s->device));
  return get_state(s, FD, cFD, shockIndicator);
}

extern "C" afar_status afar_copyFieldDataDeviceToHost(afar_fieldPointer* h, afar_solver* s, int cellsNum,
                                                      int totalBoundaryFacesNum) {
  if (!h || !s) return (set_error("null argument"), AFAR_ERR_ARGUMENT);
  if (cellsNum != s->Nc || totalBoundaryFacesNum != s->Nb) {
    set_error("afar_copyFieldDataDeviceToHost: sizes differ from the uploaded fields");
    return AFAR_ERR_ARGUMENT;
  }
  return afar_download_state(s, h->FD, nullptr, h->shockIndicator);
}

extern "C" afar_status afar_state_snapshot(afar_solver* s, int op) {
  if (!s || !s->have_fields) return (set_error("solver not initialised"), AFAR_ERR_STATE);
  if (op != AFAR_SNAPSHOT_SAVE && op != AFAR_SNAPSHOT_RESTORE) return (set_error("unknown snapshot op %d", op), AFAR_ERR_ARGUMENT);
  if (op == AFAR_SNAPSHOT_RESTORE) s->head_pending = false;
  AFAR_CUDA(cudaSetDevice(s->device));
  const size_t wb = w_size(s->policy) * (size_t)(s->Nc + s->Nb);
  const size_t ub = sizeof(V4<double>) * (size_t)s->Nc;
  if (op == AFAR_SNAPSHOT_SAVE && !s->snap) {
    afar_status st = dalloc(s, &s->snap, wb + 2 * ub + sizeof(StepCtl));
    if (st) return st;
  }
  if (!s->snap) return (set_error("restore without a saved snapshot"), AFAR_ERR_STATE);
  char* p = static_cast<char*>(s->snap);
  void* dst[4] = {p, p + wb, p + wb + ub, p + wb + 2 * ub};
  void* src[4] = {s->W, s->U, s->U0, s->ctl};
  const size_t n[4] = {wb, ub, ub, sizeof(StepCtl)};
  for (int i = 0; i < 4; ++i) {
    if (op == AFAR_SNAPSHOT_SAVE)
      AFAR_CUDA(cudaMemcpyAsync(dst[i], src[i], n[i], cudaMemcpyDeviceToDevice, s->stream));
    else
      AFAR_CUDA(cudaMemcpyAsync(src[i], dst[i], n[i], cudaMemcpyDeviceToDevice, s->stream));
  }
  AFAR_CUDA(cudaStreamSynchronize(s->stream));
  return AFAR_OK;
}

extern "C" afar_status afar_download_ls_matrix(afar_solver* s, float* matrix) {
  afar_status st = check_ready(s);
  if (st) return st;
  if (!matrix) return (set_error("null output"), AFAR_ERR_ARGUMENT);
  float* d = nullptr;
  const size_t n = 2 * (size_t)s->maxM * s->Nc;
  AFAR_CUDA(cudaMalloc(&d, n * sizeof(float)));
  AFAR_CUDA(cudaMemsetAsync(d, 0, n * sizeof(float), s->stream));
  const int gc = grid_for(s->Nc, kCellBlock);
  void* scratch = nullptr;
  const size_t sl = (s->policy == AFAR_POLICY_FP64 ? sizeof(V2<double>) : sizeof(V2<float>)) * (size_t)s->maxM * s->ldc;
  AFAR_CUDA(cudaMalloc(&scratch, sl));
  switch (s->policy) {
    case AFAR_POLICY_REF:
      k_setup_lsm<PolicyRef><<<gc, kCellBlock, 0, s->stream>>>(make_args<PolicyRef>(s), static_cast<V2<float>*>(scratch), d, s->maxM);
      break;
    case AFAR_POLICY_FP64:
      k_setup_lsm<PolicyFP64><<<gc, kCellBlock, 0, s->stream>>>(make_args<PolicyFP64>(s), static_cast<V2<double>*>(scratch), d, s->maxM);
      break;
    default:
      k_setup_lsm<PolicyMixed><<<gc, kCellBlock, 0, s->stream>>>(make_args<PolicyMixed>(s), static_cast<V2<float>*>(scratch), d, s->maxM);
      break;
  }
  AFAR_CUDA(cudaGetLastError());
  AFAR_CUDA(cudaMemcpyAsync(matrix, d, n * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
  AFAR_CUDA(cudaStreamSynchronize(s->stream));
  cudaFree(d);
  cudaFree(scratch);
  return AFAR_OK;
}

namespace {
// Switch decisions of the last stage: troubled cells (si[2c] != 0), cells on the low-order TVD
// reconstruction (si[2c+1] == 1), shock cells (si[2c+1] < 0) and KFVS faces (a shock cell on either
// side).  Per-block counts in shared memory, one atomic per counter and block.
__global__ void k_switch_counts(int Nc, int Nf, const int8_t* si, const int2* on, unsigned long long* out) {
  __shared__ unsigned int cnt[4];
  if (threadIdx.x < 4) cnt[threadIdx.x] = 0;
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < Nc) {
    if (si[2 * i] != 0) atomicAdd(&cnt[0], 1u);
    const int8_t f = si[2 * i + 1];
    if (f == 1) atomicAdd(&cnt[1], 1u);
    if (f < 0) atomicAdd(&cnt[2], 1u);
  }
  if (i < Nf) {
    const int2 p = on[i];
    if (si[2 * p.x + 1] < 0 || si[2 * p.y + 1] < 0) atomicAdd(&cnt[3], 1u);
  }
  __syncthreads();
  if (threadIdx.x < 4 && cnt[threadIdx.x]) atomicAdd(&out[threadIdx.x], (unsigned long long)cnt[threadIdx.x]);
}
}  // namespace

extern "C" afar_status afar_switch_counts(afar_solver* s, long long counts[4]) {
  afar_status st = check_ready(s);
  if (st) return st;
  if (!counts) return (set_error("null output"), AFAR_ERR_ARGUMENT);
  unsigned long long* d = nullptr;
  AFAR_CUDA(cudaMalloc(&d, 4 * sizeof(unsigned long long)));
  AFAR_CUDA(cudaMemsetAsync(d, 0, 4 * sizeof(unsigned long long), s->stream));
  const int n = std::max(s->Nc, s->Nf);
  k_switch_counts<<<grid_for(n, 256), 256, 0, s->stream>>>(s->Nc, s->Nf, s->si, s->on, d);
  unsigned long long h[4];
  AFAR_CUDA(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
  AFAR_CUDA(cudaStreamSynchronize(s->stream));
  AFAR_CUDA(cudaFree(d));
  for (int k = 0; k < 4; ++k) counts[k] = (long long)h[k];
  return AFAR_OK;
}

extern "C" afar_status afar_device_bytes(afar_solver* s, size_t* bytes) {
  if (!s || !bytes) return (set_error("null argument"), AFAR_ERR_ARGUMENT);
  *bytes = s->bytes;
  return AFAR_OK;
}

extern "C" int afar_launches_per_step(afar_solver* s) {
  if (!s) return 13;  // the face-centre step of the fp64 and mixed policies
  if (s->policy == AFAR_POLICY_REF) return 14;
  return s->ng > 0 ? 17 : 13;  // the multi-point flux: a Gauss-point reconstruct per stage, the Courant kernel
}

extern "C" afar_status afar_freeFieldData(afar_solver* s) {
  if (!s) return AFAR_OK;
  if (s->batch) afar_batch_remove(s->batch, s);  // the batch forgets a freed member
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  destroy_graphs(s);
  for (void* p : s->allocs) cudaFree(p);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return AFAR_OK;
}

// ------------------------------------------------------------------------------------------------
// step parameters and batches

extern "C" afar_status afar_set_step_params(afar_solver* s, double dt, double CFL, double tEnd) {
  afar_status st = check_ready(s);
  if (st) return st;
  if (!(dt > 0.0) && !(CFL > 0.0)) return (set_error("afar_set_step_params: deltaT or CFL must be positive"), AFAR_ERR_ARGUMENT);
  k_set_ctl<<<1, 32, 0, s->stream>>>(s->ctl, dt > 0.0 ? dt : 0.0, CFL, tEnd);
  AFAR_CUDA(cudaStreamSynchronize(s->stream));
  AFAR_CUDA(cudaGetLastError());
  return AFAR_OK;
}

extern "C" afar_status afar_set_periodic(afar_solver* s, double px, double py) {
  if (!s) return (set_error("null solver"), AFAR_ERR_ARGUMENT);
  if (s->have_stencil) return (set_error("afar_set_periodic: call it before afar_setDeviceFieldDataStencil"), AFAR_ERR_STATE);
  if (!(px >= 0.0) || !(py >= 0.0)) return (set_error("afar_set_periodic: negative period"), AFAR_ERR_ARGUMENT);
  if (s->policy == AFAR_POLICY_REF && (px > 0.0 || py > 0.0))
    return (set_error("afar_set_periodic: the ref policy takes raw cell centres in its flux (no periodic meshes)"),
            AFAR_ERR_ARGUMENT);
  s->px = px;
  s->py = py;
  return AFAR_OK;
}

extern "C" afar_status afar_set_write_interval(afar_solver* s, double writeInterval) {
  if (!s || !s->have_fields) return (set_error("solver not initialised"), AFAR_ERR_STATE);
  if (!(writeInterval >= 0.0)) return (set_error("afar_set_write_interval: negative interval"), AFAR_ERR_ARGUMENT);
  s->head_pending = false;
  AFAR_CUDA(cudaSetDevice(s->device));
  k_set_write_interval<<<1, 32, 0, s->stream>>>(s->ctl, writeInterval);
  AFAR_CUDA(cudaStreamSynchronize(s->stream));
  AFAR_CUDA(cudaGetLastError());
  return AFAR_OK;
}

// The batch's launch schedule: which reconstruct each member runs (the tile-staged one unless its
// solver forces the register pass, so a member's result never depends on its batch-mates) and the
// BVD and flux block sizes (timed on the whole batch; the results do not depend on them, every
// reduction being an exact minimum).
struct BatchSchedule {
  int bvd_block = 128, flux_block = 256;
  int tile_members = 0, reg_members = 0;
  float ms[5] = {0.f, 0.f, 0.f, 0.f, 0.f};  // BVD at 64, 128, 256; flux at 128, 256 (0: from the cache)
};

struct afar_batch {
  int policy = AFAR_POLICY_MIXED;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<afar_solver*> members;
  void* tab = nullptr;  // StageArgs<P>[members]
  size_t tab_bytes = 0;
  // block maps, (member, block within the member) per block, one after another in one buffer:
  // 128-cell blocks of the tile-reconstruct members, of the register-reconstruct members, of every
  // member (update; the fp64 reconstruct), BVD blocks, face blocks
  int2* maps = nullptr;
  size_t maps_n = 0;
  int n_tile = 0, n_reg = 0, n_cell = 0, n_bvd = 0, n_face = 0;
  size_t smem = 0;  // dynamic shared memory of the staged reconstruct (largest member)
  BatchSchedule sched;
  int forced_bvd = 0, forced_flux = 0;  // afar_batch_set_schedule (0: autotune)
  cudaGraphExec_t graph = nullptr;
  bool dirty = true;
};

namespace {

// Blocks of `block` cells (or faces when faces) of each member in `which` (empty: all members).
void batch_map(const std::vector<afar_solver*>& members, int block, bool faces, const std::vector<int>* which,
               std::vector<int2>& out) {
  for (size_t i = 0; i < members.size(); ++i) {
    if (which && !(*which)[i]) continue;
    const afar_solver* s = members[i];
    const long long n = faces ? (long long)s->Nf + s->Nb : (long long)s->Nc;
    const int nb = grid_for(n, block);
    for (int k = 0; k < nb; ++k) out.push_back(int2{(int)i, k});
  }
}

template <class P>
void launch_bvd(int block, int nblocks, const StageArgs<P>* t, const int2* map, cudaStream_t st) {
  if (nblocks == 0) return;
  if (block == 64)
    kb_bvd<P, 64><<<nblocks, 64, 0, st>>>(t, map);
  else if (block == 256)
    kb_bvd<P, 256><<<nblocks, 256, 0, st>>>(t, map);
  else
    kb_bvd<P, 128><<<nblocks, 128, 0, st>>>(t, map);
}
template <class P, bool DT>
void launch_flux(int block, int nblocks, const StageArgs<P>* t, const int2* map, cudaStream_t st) {
  if (nblocks == 0) return;
  if (block == 128)
    kb_flux<P, DT, 128><<<nblocks, 128, 0, st>>>(t, map);
  else
    kb_flux<P, DT, 256><<<nblocks, 256, 0, st>>>(t, map);
}

// The batch autotuner's decisions, per device, policy and batch shape (cells and members, each to
// a factor of two): BVD and flux block sizes.
std::mutex g_batch_tune_mu;
std::map<std::tuple<int, int, int, int>, std::pair<int, int>> g_batch_tune;

template <class P>
afar_status batch_build(afar_batch* b) {
  std::vector<StageArgs<P>> tab;
  size_t smem = 0;
  afar_status st;
  long long cells = 0;
  std::vector<int> is_tile(b->members.size(), 1), is_reg(b->members.size(), 0);
  for (size_t i = 0; i < b->members.size(); ++i) {
    afar_solver* s = b->members[i];
    tab.push_back(make_args<P>(s));
    smem = std::max(smem, recon_smem<P>(s));
    cells += s->Nc;
    if constexpr (P::id == PolicyMixed::id) {
      // the tile-staged reconstruct unless the member's solver forces the register pass
      // (afar_set_tuning): a member's solo autotuner times its mesh alone, where small meshes leave
      // the GPU idle and favour the register pass; in a full batch the tile kernel is faster
      // (14.2M cells in 256 members: 11.2 against 11.5 ms a step)
      is_reg[i] = s->recon_request == 1;
      is_tile[i] = !is_reg[i];
    }
  }
  int lc = 0, lm = 0;
  while ((1ll << (lc + 1)) <= cells) ++lc;
  while ((1ll << (lm + 1)) <= (long long)b->members.size()) ++lm;
  const auto key = std::make_tuple(b->device, (int)P::id, lc, lm);
  BatchSchedule sc;
  for (size_t i = 0; i < b->members.size(); ++i) sc.tile_members += is_tile[i], sc.reg_members += is_reg[i];
  bool timed = true;
  if (b->forced_bvd || b->forced_flux) {
    sc.bvd_block = b->forced_bvd ? b->forced_bvd : 128;
    sc.flux_block = b->forced_flux ? b->forced_flux : 256;
    timed = false;
  } else {
    std::lock_guard<std::mutex> lock(g_batch_tune_mu);
    auto it = g_batch_tune.find(key);
    if (it != g_batch_tune.end()) {
      sc.bvd_block = it->second.first;
      sc.flux_block = it->second.second;
      timed = false;
    }
  }

  std::vector<int2> mp_tile, mp_reg, mp_cell;
  batch_map(b->members, kTile, false, &is_tile, mp_tile);
  batch_map(b->members, kTile, false, &is_reg, mp_reg);
  batch_map(b->members, kCellBlock, false, nullptr, mp_cell);
  // candidate maps for the timing: BVD in 64/128/256-cell blocks, flux in 128/256-face blocks
  const int bvd_sizes[3] = {64, 128, 256}, flux_sizes[2] = {128, 256};
  std::vector<int2> mp_bvd[3], mp_face[2];
  for (int k = 0; k < 3; ++k)
    if (timed || bvd_sizes[k] == sc.bvd_block) batch_map(b->members, bvd_sizes[k], false, nullptr, mp_bvd[k]);
  for (int k = 0; k < 2; ++k)
    if (timed || flux_sizes[k] == sc.flux_block) batch_map(b->members, flux_sizes[k], true, nullptr, mp_face[k]);
  std::vector<int2> all;
  auto append = [&](const std::vector<int2>& v) {
    const size_t o = all.size();
    all.insert(all.end(), v.begin(), v.end());
    return o;
  };
  const size_t o_tile = append(mp_tile), o_reg = append(mp_reg), o_cell = append(mp_cell);
  size_t o_bvd[3], o_face[2];
  for (int k = 0; k < 3; ++k) o_bvd[k] = append(mp_bvd[k]);
  for (int k = 0; k < 2; ++k) o_face[k] = append(mp_face[k]);

  auto grow = [&](void** p, size_t* cap, size_t need) -> afar_status {
    if (need > *cap) {
      if (*p) cudaFree(*p);
      *p = nullptr;
      AFAR_CUDA(cudaMalloc(p, need));
      *cap = need;
    }
    return AFAR_OK;
  };
  size_t cap_m = b->maps_n * sizeof(int2);
  if ((st = grow(&b->tab, &b->tab_bytes, std::max<size_t>(1, tab.size()) * sizeof(StageArgs<P>)))) return st;
  if ((st = grow(reinterpret_cast<void**>(&b->maps), &cap_m, std::max<size_t>(1, all.size()) * sizeof(int2)))) return st;
  b->maps_n = cap_m / sizeof(int2);
  if (!tab.empty()) {
    AFAR_CUDA(cudaMemcpyAsync(b->tab, tab.data(), tab.size() * sizeof(StageArgs<P>), cudaMemcpyHostToDevice, b->stream));
    AFAR_CUDA(cudaMemcpyAsync(b->maps, all.data(), all.size() * sizeof(int2), cudaMemcpyHostToDevice, b->stream));
  }
  AFAR_CUDA(cudaStreamSynchronize(b->stream));
  b->smem = smem;
  int nfmax = 3;
  for (afar_solver* s : b->members) nfmax = std::max(nfmax, s->maxM);
  if constexpr (P::id != PolicyMixed::id) {
    if ((st = raise_smem_limit(kb_reconstruct_staged<P>, b->device, smem))) return st;
  } else {
    if ((st = raise_smem_limit(kb_reconstruct_tile<P, 3>, b->device, smem))) return st;
    if ((st = raise_smem_limit(kb_reconstruct_tile<P, 4>, b->device, smem))) return st;
  }
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  b->n_tile = (int)mp_tile.size();
  b->n_reg = (int)mp_reg.size();
  b->n_cell = (int)mp_cell.size();
  if (tab.empty()) {
    b->sched = sc;
    b->dirty = false;
    return AFAR_OK;
  }
  const StageArgs<P>* t = static_cast<const StageArgs<P>*>(b->tab);
  auto reconstruct = [&]() {
    if constexpr (P::id == PolicyMixed::id) {
      if (b->n_tile) {
        if (nfmax <= 3)
          kb_reconstruct_tile<P, 3><<<b->n_tile, kTile, b->smem, b->stream>>>(t, b->maps + o_tile);
        else
          kb_reconstruct_tile<P, 4><<<b->n_tile, kTile, b->smem, b->stream>>>(t, b->maps + o_tile);
      }
      if (b->n_reg) kb_reconstruct_reg<P><<<b->n_reg, kCellBlock, 0, b->stream>>>(t, b->maps + o_reg);
    } else
      kb_reconstruct_staged<P><<<b->n_cell, kCellBlock, b->smem, b->stream>>>(t, b->maps + o_cell);
  };

  if (timed) {
    // reconstruct once so that the BVD and flux read this step's intermediates, then time each
    // candidate: a warm-up and the best of three launches (both kernels are functions of the state
    // and the stage's intermediates; they change neither the state nor the step control)
    reconstruct();
    cudaEvent_t e0, e1;
    AFAR_CUDA(cudaEventCreate(&e0));
    AFAR_CUDA(cudaEventCreate(&e1));
    auto best_of = [&](auto&& launch) -> float {
      launch();
      float best = 1e30f;
      for (int r = 0; r < 3; ++r) {
        cudaEventRecord(e0, b->stream);
        launch();
        cudaEventRecord(e1, b->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        best = std::min(best, ms);
      }
      return best;
    };
    for (int k = 0; k < 3; ++k)
      sc.ms[k] = best_of([&] { launch_bvd<P>(bvd_sizes[k], (int)mp_bvd[k].size(), t, b->maps + o_bvd[k], b->stream); });
    for (int k = 0; k < 2; ++k)
      sc.ms[3 + k] =
          best_of([&] { launch_flux<P, false>(flux_sizes[k], (int)mp_face[k].size(), t, b->maps + o_face[k], b->stream); });
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    AFAR_CUDA(cudaGetLastError());
    for (afar_solver* m : b->members)
      if ((st = check_device_error(m))) return st;
    sc.bvd_block = bvd_sizes[std::min_element(sc.ms, sc.ms + 3) - sc.ms];
    sc.flux_block = flux_sizes[std::min_element(sc.ms + 3, sc.ms + 5) - (sc.ms + 3)];
    std::lock_guard<std::mutex> lock(g_batch_tune_mu);
    g_batch_tune[key] = {sc.bvd_block, sc.flux_block};
  }
  const int kb = sc.bvd_block == 64 ? 0 : sc.bvd_block == 128 ? 1 : 2;
  const int kf = sc.flux_block == 128 ? 0 : 1;
  const int2* bmap = b->maps + o_bvd[kb];
  const int2* fmap = b->maps + o_face[kf];
  b->n_bvd = (int)mp_bvd[kb].size();
  b->n_face = (int)mp_face[kf].size();
  b->sched = sc;

  // capture one step of the whole batch
  cudaGraph_t g = nullptr;
  AFAR_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < 3; ++k) {
    reconstruct();
    launch_bvd<P>(sc.bvd_block, b->n_bvd, t, bmap, b->stream);
    if (k == 0)
      launch_flux<P, true>(sc.flux_block, b->n_face, t, fmap, b->stream);
    else
      launch_flux<P, false>(sc.flux_block, b->n_face, t, fmap, b->stream);
    kb_update<P><<<b->n_cell, kCellBlock, 0, b->stream>>>(t, b->maps + o_cell, stage_coef(k));
  }
  kb_finish_step<P><<<grid_for((long long)tab.size(), 128), 128, 0, b->stream>>>(t, (int)tab.size());
  AFAR_CUDA(cudaStreamEndCapture(b->stream, &g));
  const cudaError_t e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    b->graph = nullptr;
    set_error("batch graph instantiation failed: %s", cudaGetErrorString(e));
    return AFAR_ERR_CUDA;
  }
  b->dirty = false;
  return AFAR_OK;
}

}  // namespace

extern "C" afar_status afar_batch_create(afar_batch** out, int policy, int device) {
  if (!out || (policy != AFAR_POLICY_MIXED && policy != AFAR_POLICY_FP64)) {
    set_error("afar_batch_create: null output or policy other than fp64/mixed");
    return AFAR_ERR_ARGUMENT;
  }
  *out = nullptr;
  AFAR_CUDA(cudaSetDevice(device));
  afar_batch* b = new afar_batch();
  b->policy = policy;
  b->device = device;
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete b;
    set_error("cudaStreamCreate failed");
    return AFAR_ERR_CUDA;
  }
  *out = b;
  return AFAR_OK;
}

extern "C" afar_status afar_batch_add(afar_batch* b, afar_solver* s) {
  if (!b || !s) return (set_error("null argument"), AFAR_ERR_ARGUMENT);
  afar_status st = check_ready(s);
  if (st) return st;
  if (s->policy != b->policy || s->device != b->device)
    return (set_error("afar_batch_add: member policy/device differ from the batch's"), AFAR_ERR_ARGUMENT);
  if (!(s->R > 0.0)) return (set_error("afar_batch_add: call afar_set_gas on the member first"), AFAR_ERR_STATE);
  if (!s->have_stencil)
    return (set_error("afar_batch_add: upload the stencil (afar_setDeviceFieldDataStencil) first"), AFAR_ERR_STATE);
  if (s->batch) return (set_error("afar_batch_add: the solver already belongs to a batch"), AFAR_ERR_STATE);
  if (s->ng > 0)
    return (set_error("afar_batch_add: batches run the face-centre flux; the solver has the multi-point face flux"),
            AFAR_ERR_ARGUMENT);
  AFAR_CUDA(cudaStreamSynchronize(s->stream));  // no pending work of the member on its own stream
  b->members.push_back(s);
  s->batch = b;
  b->dirty = true;
  return AFAR_OK;
}

extern "C" afar_status afar_batch_remove(afar_batch* b, afar_solver* s) {
  if (!b || !s) return (set_error("null argument"), AFAR_ERR_ARGUMENT);
  for (size_t i = 0; i < b->members.size(); ++i)
    if (b->members[i] == s) {
      AFAR_CUDA(cudaSetDevice(b->device));
      AFAR_CUDA(cudaStreamSynchronize(b->stream));
      b->members.erase(b->members.begin() + i);
      s->batch = nullptr;
      b->dirty = true;
      return AFAR_OK;
    }
  set_error("afar_batch_remove: not a member");
  return AFAR_ERR_ARGUMENT;
}

extern "C" afar_status afar_batch_size(afar_batch* b, int* n) {
  if (!b || !n) return (set_error("null argument"), AFAR_ERR_ARGUMENT);
  *n = (int)b->members.size();
  return AFAR_OK;
}

extern "C" afar_status afar_batch_run(afar_batch* b, int nSteps, float* ms) {
  NvtxRange nvtx("afar_batch_run");
  if (!b || nSteps < 0) return (set_error("afar_batch_run: bad argument"), AFAR_ERR_ARGUMENT);
  AFAR_CUDA(cudaSetDevice(b->device));
  afar_status st;
  if (b->dirty) {
    st = b->policy == AFAR_POLICY_MIXED ? batch_build<PolicyMixed>(b) : batch_build<PolicyFP64>(b);
    if (st) return st;
  }
  if (ms) *ms = 0.f;
  if (b->members.empty() || nSteps == 0) return AFAR_OK;
  cudaEvent_t e0, e1;
  AFAR_CUDA(cudaEventCreate(&e0));
  AFAR_CUDA(cudaEventCreate(&e1));
  AFAR_CUDA(cudaEventRecord(e0, b->stream));
  for (int i = 0; i < nSteps; ++i) AFAR_CUDA(cudaGraphLaunch(b->graph, b->stream));
  AFAR_CUDA(cudaEventRecord(e1, b->stream));
  AFAR_CUDA(cudaEventSynchronize(e1));
  if (ms) AFAR_CUDA(cudaEventElapsedTime(ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  AFAR_CUDA(cudaGetLastError());
  for (afar_solver* m : b->members)
    if ((st = check_device_error(m))) return st;
  return AFAR_OK;
}

extern "C" afar_status afar_batch_destroy(afar_batch* b) {
  if (!b) return AFAR_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (afar_solver* m : b->members) m->batch = nullptr;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->tab) cudaFree(b->tab);
  if (b->maps) cudaFree(b->maps);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return AFAR_OK;
}

extern "C" afar_status afar_batch_set_schedule(afar_batch* b, int bvdBlock, int fluxBlock) {
  if (!b) return (set_error("null batch"), AFAR_ERR_ARGUMENT);
  if ((bvdBlock != 0 && bvdBlock != 64 && bvdBlock != 128 && bvdBlock != 256) ||
      (fluxBlock != 0 && fluxBlock != 128 && fluxBlock != 256))
    return (set_error("afar_batch_set_schedule: BVD block 0/64/128/256, flux block 0/128/256"), AFAR_ERR_ARGUMENT);
  b->forced_bvd = bvdBlock;
  b->forced_flux = fluxBlock;
  b->dirty = true;
  return AFAR_OK;
}

extern "C" afar_status afar_batch_get_schedule(afar_batch* b, int* tileMembers, int* registerMembers, int* bvdBlock,
                                               int* fluxBlock, float ms[5]) {
  if (!b) return (set_error("null batch"), AFAR_ERR_ARGUMENT);
  if (b->dirty) {
    AFAR_CUDA(cudaSetDevice(b->device));
    const afar_status st = b->policy == AFAR_POLICY_MIXED ? batch_build<PolicyMixed>(b) : batch_build<PolicyFP64>(b);
    if (st) return st;
  }
  if (tileMembers) *tileMembers = b->sched.tile_members;
  if (registerMembers) *registerMembers = b->sched.reg_members;
  if (bvdBlock) *bvdBlock = b->sched.bvd_block;
  if (fluxBlock) *fluxBlock = b->sched.flux_block;
  if (ms)
    for (int k = 0; k < 5; ++k) ms[k] = b->sched.ms[k];
  return AFAR_OK;
}

extern "C" afar_status afar_debug_wait_injection(int device, unsigned extraBytes, long long limitClocks) {
  AFAR_CUDA(cudaSetDevice(device));
  const long long lim = limitClocks > 0 ? limitClocks : (1ll << 31);
  AFAR_CUDA(cudaMemcpyToSymbol(g_tile_extra_tx, &extraBytes, sizeof(extraBytes)));
  AFAR_CUDA(cudaMemcpyToSymbol(g_tile_wait_limit, &lim, sizeof(lim)));
  AFAR_CUDA(cudaDeviceSynchronize());
  return AFAR_OK;
}

extern "C" afar_status afar_set_face_gauss_flux(afar_solver* s, int nPoints, const double* points,
                                                const double* pointWeights, const double* rbfGauss) {
  afar_status st = check_ready(s);
  if (st || (st = check_not_batched(s))) return st;
  if (nPoints == 0) {
    s->ng = 0;
    destroy_graphs(s);
    return AFAR_OK;
  }
  if (s->policy == AFAR_POLICY_REF)
    return (set_error("afar_set_face_gauss_flux: the ref policy keeps the reference's face-centre flux"),
            AFAR_ERR_ARGUMENT);
  if (nPoints < 1 || nPoints > 4 || !points || !pointWeights || !rbfGauss)
    return (set_error("afar_set_face_gauss_flux: 1 to 4 points per face and non-null arrays"), AFAR_ERR_ARGUMENT);
  double wsum = 0.0;
  for (int k = 0; k < nPoints; ++k) {
    if (!(pointWeights[k] > 0.0)) return (set_error("afar_set_face_gauss_flux: non-positive point weight"), AFAR_ERR_ARGUMENT);
    wsum += pointWeights[k];
  }
  const int Nf = s->Nf, ng = nPoints, nmax = s->maxS + 1;
  const bool mixed = s->policy == AFAR_POLICY_MIXED;
  const size_t wS = mixed ? sizeof(float) : sizeof(double), wG = mixed ? sizeof(float) : sizeof(double);
  if ((st = dalloc(s, &s->wg, wS * (size_t)s->maxM * ng * nmax * s->ldc))) return st;
  AFAR_CUDA(cudaMemsetAsync(s->wg, 0, wS * (size_t)s->maxM * ng * nmax * s->ldc, s->stream));
  if ((st = dalloc(s, &s->sgk, 2 * wG * (size_t)s->maxM * ng * s->ldc))) return st;
  AFAR_CUDA(cudaMemsetAsync(s->sgk, 0, 2 * wG * (size_t)s->maxM * ng * s->ldc, s->stream));
  if ((st = dalloc(s, &s->fgk, 2 * wG * (size_t)Nf * ng))) return st;
  if ((st = dalloc(s, &s->fvg, 4 * wG * 2 * (size_t)Nf * ng))) return st;
  double *d_w = nullptr, *d_p = nullptr;
  V4<double>* fxy = nullptr;
  auto cleanup = [&]() {
    if (d_w) cudaFree(d_w);
    if (d_p) cudaFree(d_p);
    if (fxy) cudaFree(fxy);
  };
  const size_t nw = (size_t)Nf * 2 * ng * nmax, np = (size_t)Nf * ng * 2;
  if (cudaMalloc(&d_w, sizeof(double) * (nw ? nw : 1)) != cudaSuccess ||
      cudaMalloc(&d_p, sizeof(double) * (np ? np : 1)) != cudaSuccess ||
      cudaMalloc(&fxy, sizeof(V4<double>) * (size_t)(Nf + s->Nb + 1)) != cudaSuccess) {
    cleanup();
    set_error("afar_set_face_gauss_flux: out of device memory for the set-up");
    return AFAR_ERR_CUDA;
  }
  cudaMemcpyAsync(d_w, rbfGauss, sizeof(double) * nw, cudaMemcpyHostToDevice, s->stream);
  cudaMemcpyAsync(d_p, points, sizeof(double) * np, cudaMemcpyHostToDevice, s->stream);
  V4<double>* fsr = nullptr;
  if (cudaMalloc(&fsr, sizeof(V4<double>) * (size_t)(Nf + s->Nb + 1)) != cudaSuccess) {
    cleanup();
    set_error("afar_set_face_gauss_flux: out of device memory for the set-up");
    return AFAR_ERR_CUDA;
  }
  const int gF = grid_for((long long)Nf + s->Nb, kFaceBlock);
  k_split_faces<<<gF, kFaceBlock, 0, s->stream>>>(Nf + s->Nb, s->faceRaw, fxy, fsr);
  s->ng = ng;
  for (int k = 0; k < 4; ++k) s->gw[k] = k < ng ? pointWeights[k] / wsum : 0.0;
  auto setup = [&](auto tag) {
    using P = decltype(tag);
    StageArgs<P> a = make_args<P>(s);
    k_setup_gauss<P><<<grid_for(s->Nc, kCellBlock), kCellBlock, 0, s->stream>>>(a, d_w, d_p);
    if (Nf > 0) k_setup_gauss_faces<P><<<grid_for((long long)Nf * ng, 256), 256, 0, s->stream>>>(a, d_p, fxy);
  };
  if (mixed)
    setup(PolicyMixed{});
  else
    setup(PolicyFP64{});
  const cudaError_t e = cudaGetLastError();
  const cudaError_t e2 = cudaStreamSynchronize(s->stream);
  cleanup();
  cudaFree(fsr);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    s->ng = 0;
    set_error("afar_set_face_gauss_flux: set-up failed: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
    return AFAR_ERR_CUDA;
  }
  destroy_graphs(s);  // the next run captures the step with the multi-point flux
  return AFAR_OK;
}
