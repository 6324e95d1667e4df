// The RBF stage of the host precompute on a CUDA device: per cell the multiquadric P matrix of its
// stencil (each entry Gauss-integrated over a stencil cell, basicCUDAsolver.cpp:461-505), its inverse
// (LU with partial pivoting; the host's Jacobi-SVD pseudo-inverse when a pivot is exactly zero, as
// SVDinv at basicCUDAsolver.cpp:509) and the trouble flag (:511-529); per internal face side the O3
// weights G^T b - 1 1^T G^T b / n + 1/n (:538-619).
//
// Every value is computed by the same operations in the same order as the host stage in
// afar_precompute.cpp, and this file is compiled without multiply-add contraction (-fmad=false,
// like the host's -ffp-contract=off); double division and square root are correctly rounded on
// both sides, so the arrays are bit-identical to the host's.  One warp per cell: lanes share the
// P entries, the elimination of each LU step and the columns of the inverse; the pivot search stays
// serial (lane 0) so ties and NaNs resolve exactly as in the host loop.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "afar_internal.h"

namespace afar {

namespace {

constexpr int kN = AFAR_MAX_VALID_STENCIL_SIZE + 1;  // largest P matrix order
constexpr int kWarps = 4;                            // cells per block of k_rbf_cell
constexpr unsigned kFull = 0xffffffffu;

enum : uint8_t { kCellOk = 0, kCellTrouble = 1, kCellSingular = 2 };

__device__ __forceinline__ double wrap_period(double d, double L) { return L > 0.0 ? d - L * rint(d / L) : d; }

// One warp per cell: P (n x n, n = stencil size + 1) into shared memory and into the cell's G slot
// (kept there for the host's SVD fallback), LU in place, then G = P^-1 column by column.
__global__ void __launch_bounds__(32 * kWarps) k_rbf_cell(int nc, int maxS, int nmax, const uint8_t* __restrict__ ssz,
                                                          const int* __restrict__ sten,
                                                          const double2* __restrict__ cell,
                                                          const int* __restrict__ gq_off,
                                                          const double2* __restrict__ gq_xy,
                                                          const double* __restrict__ gq_w, double px, double py,
                                                          double shape, double* __restrict__ refd,
                                                          double* __restrict__ Gall, uint8_t* __restrict__ status) {
  __shared__ double sP[kWarps][kN * kN];
  __shared__ double sX[kWarps][kN][32];
  __shared__ int sIdx[kWarps][kN];
  __shared__ int sPiv[kWarps][kN];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * kWarps + w;
  if (c >= nc) return;  // warp-uniform
  const int S = ssz[c], n = S + 1;
  const int* st = sten + (size_t)maxS * c;
  double* P = sP[w];
  int* idx = sIdx[w];
  if (lane < n) idx[lane] = lane == 0 ? c : st[lane - 1];
  double rd = 0.0;
  if (lane == 0) {  // reference distance: mean centre distance, summed in stencil order
    const double2 cc = cell[c];
    for (int i = 0; i < S; ++i) {
      const double2 q = cell[st[i]];
      const double dx = wrap_period(q.x - cc.x, px), dy = wrap_period(q.y - cc.y, py);
      rd += sqrt(dx * dx + dy * dy);
    }
    rd /= double(S);
    refd[c] = rd;
  }
  rd = __shfl_sync(kFull, rd, 0);
  __syncwarp();
  double* G = Gall + (size_t)c * nmax * nmax;
  for (int e = lane; e < n * n; e += 32) {
    const int i = e / n, j = e - i * n;
    const int si = idx[i];
    const double2 o = cell[idx[j]];
    double acc = 0.0;
    for (int k = gq_off[si]; k < gq_off[si + 1]; ++k) {
      const double2 g = gq_xy[k];
      const double ex = wrap_period(g.x - o.x, px) / rd, ey = wrap_period(g.y - o.y, py) / rd;
      acc += gq_w[k] * sqrt(shape + (ex * ex + ey * ey));
    }
    P[e] = acc;
    G[e] = acc;
  }
  __syncwarp();

  for (int k = 0; k < n; ++k) {
    int p = k, ok = 0;
    if (lane == 0) {
      double best = fabs(P[k * n + k]);
      for (int i = k + 1; i < n; ++i)
        if (fabs(P[i * n + k]) > best) {
          best = fabs(P[i * n + k]);
          p = i;
        }
      ok = best > 0.0;
      sPiv[w][k] = p;
    }
    p = __shfl_sync(kFull, p, 0);
    ok = __shfl_sync(kFull, ok, 0);
    if (!ok) {  // exactly singular: the host inverts the P left in the G slot by SVD
      if (lane == 0) status[c] = kCellSingular;
      return;
    }
    if (p != k)
      for (int j = lane; j < n; j += 32) {
        const double t = P[k * n + j];
        P[k * n + j] = P[p * n + j];
        P[p * n + j] = t;
      }
    __syncwarp();
    const double inv = 1.0 / P[k * n + k];
    for (int i = k + 1 + lane; i < n; i += 32) P[i * n + k] = P[i * n + k] * inv;
    __syncwarp();
    const int m = n - k - 1;
    for (int e = lane; e < m * m; e += 32) {
      const int i = k + 1 + e / m, j = k + 1 + e % m;
      P[i * n + j] -= P[i * n + k] * P[k * n + j];
    }
    __syncwarp();
  }

  bool bad = false;
  if (lane < n) {  // column `lane` of the inverse: L U x = (row swaps) e_lane
    double(*x)[32] = sX[w];
    const int* piv = sPiv[w];
    for (int i = 0; i < n; ++i) x[i][lane] = i == lane ? 1.0 : 0.0;
    for (int k = 0; k < n; ++k) {
      const int q = piv[k];
      if (q != k) {
        const double t = x[k][lane];
        x[k][lane] = x[q][lane];
        x[q][lane] = t;
      }
    }
    for (int i = 1; i < n; ++i) {
      double xi = x[i][lane];
      for (int j = 0; j < i; ++j) xi -= P[i * n + j] * x[j][lane];
      x[i][lane] = xi;
    }
    for (int i = n - 1; i >= 0; --i) {
      double xi = x[i][lane];
      for (int j = i + 1; j < n; ++j) xi -= P[i * n + j] * x[j][lane];
      xi /= P[i * n + i];
      x[i][lane] = xi;
    }
    for (int i = 0; i < n; ++i) {
      const double v = x[i][lane];
      G[i * n + lane] = v;
      if (!(fabs(v) <= 1e10)) bad = true;
    }
  }
  bad = __any_sync(kFull, bad);
  if (lane == 0) status[c] = bad ? kCellTrouble : kCellOk;
}

// One thread per internal face side: the multiquadric basis at the face centre, G^T b and the
// weights (a troubled cell gets the first-order weights 1, 0, ..., 0).
__global__ void __launch_bounds__(128) k_rbf_face(int nf, int maxS, int nmax, const uint8_t* __restrict__ ssz,
                                                  const int* __restrict__ sten, const double2* __restrict__ cell,
                                                  const double2* __restrict__ fxy, const int* __restrict__ neighbour,
                                                  const double* __restrict__ refd, const double* __restrict__ Gall,
                                                  const uint8_t* __restrict__ status, double px, double py,
                                                  double shape, float* __restrict__ out, double* __restrict__ out64) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2LL * nf) return;
  const int f = (int)(t >> 1), side = (int)(t & 1);
  const int c = neighbour[2 * f + side];
  const int n = ssz[c] + 1;
  const size_t base = 2 * (size_t)nmax * f + (size_t)side * nmax;
  if (status[c] == kCellTrouble) {
    for (int i = 0; i < n; ++i) {
      out[base + i] = i == 0 ? 1.0f : 0.0f;
      if (out64) out64[base + i] = i == 0 ? 1.0 : 0.0;
    }
    return;
  }
  const double2 x = fxy[f];
  const int* st = sten + (size_t)maxS * c;
  const double rd = refd[c];
  double b[kN];
#pragma unroll
  for (int i = 0; i < kN; ++i)
    if (i < n) {
      const double2 q = cell[i == 0 ? c : st[i - 1]];
      const double ex = wrap_period(x.x - q.x, px) / rd, ey = wrap_period(x.y - q.y, py) / rd;
      b[i] = sqrt(shape + (ex * ex + ey * ey));
    }
  const double* G = Gall + (size_t)c * nmax * nmax;
  double gtb[kN];
  double sum = 0.0;
#pragma unroll
  for (int i = 0; i < kN; ++i)
    if (i < n) {
      double acc = 0.0;
#pragma unroll
      for (int j = 0; j < kN; ++j)
        if (j < n) acc += G[j * n + i] * b[j];
      gtb[i] = acc;
      sum += acc;
    }
#pragma unroll
  for (int i = 0; i < kN; ++i)
    if (i < n) {
      const double wi = gtb[i] - sum / double(n) + 1.0 / double(n);
      out[base + i] = (float)wi;
      if (out64) out64[base + i] = wi;
    }
}

// Device buffers of one call, released on every path out.
struct DeviceBuffers {
  std::vector<void*> ptrs;
  ~DeviceBuffers() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  T* alloc(size_t n, cudaError_t& err) {
    void* p = nullptr;
    if (err == cudaSuccess) err = cudaMalloc(&p, (n > 0 ? n : 1) * sizeof(T));
    if (err == cudaSuccess) ptrs.push_back(p);
    return static_cast<T*>(p);
  }
};

}  // namespace

afar_status rbf_stage_device(int device, const RbfInputs& in, float* RBFbasis, double* rbf64) {
  int prev = -1;
  cudaGetDevice(&prev);
  cudaError_t err = cudaSetDevice(device);
  if (err != cudaSuccess) {
    set_error("precompute on device %d: %s", device, cudaGetErrorString(err));
    cudaGetLastError();  // a bad ordinal is not sticky: leave no error for the caller's next check
    return AFAR_ERR_CUDA;
  }
  afar_status st = AFAR_OK;
  {
    const int nc = in.nc, nf = in.nf, nmax = in.maxS + 1;
    const size_t ncb = (size_t)nc + in.nb, total = (size_t)in.gq_off[ncb];
    const size_t nG = (size_t)nc * nmax * nmax, nOut = 2 * (size_t)nmax * nf;
    std::vector<double> fxy(2 * (size_t)nf);
    for (int f = 0; f < nf; ++f) {
      fxy[2 * f] = in.FACE[f].x;
      fxy[2 * f + 1] = in.FACE[f].y;
    }
    cudaStream_t s = nullptr;
    err = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    DeviceBuffers B;
    uint8_t* d_ssz = B.alloc<uint8_t>(nc, err);
    int* d_sten = B.alloc<int>((size_t)in.maxS * nc, err);
    double2* d_cell = B.alloc<double2>(ncb, err);
    int* d_off = B.alloc<int>(ncb + 1, err);
    double2* d_gxy = B.alloc<double2>(total, err);
    double* d_gw = B.alloc<double>(total, err);
    double2* d_fxy = B.alloc<double2>(nf, err);
    int* d_nb = B.alloc<int>(2 * (size_t)nf, err);
    double* d_refd = B.alloc<double>(nc, err);
    double* d_G = B.alloc<double>(nG, err);
    uint8_t* d_status = B.alloc<uint8_t>(nc, err);
    float* d_out = B.alloc<float>(nOut, err);
    double* d_out64 = rbf64 ? B.alloc<double>(nOut, err) : nullptr;
    auto up = [&](void* dst, const void* src, size_t bytes) {
      if (err == cudaSuccess && bytes) err = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
    };
    auto down = [&](void* dst, const void* src, size_t bytes) {
      if (err == cudaSuccess && bytes) err = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
    };
    up(d_ssz, in.stencilSize, nc);
    up(d_sten, in.stencil, sizeof(int) * (size_t)in.maxS * nc);
    up(d_cell, in.CELL, sizeof(double2) * ncb);
    up(d_off, in.gq_off, sizeof(int) * (ncb + 1));
    up(d_gxy, in.gq_xy, sizeof(double2) * total);
    up(d_gw, in.gq_w, sizeof(double) * total);
    up(d_fxy, fxy.data(), sizeof(double2) * nf);
    up(d_nb, in.neighbour, sizeof(int) * 2 * (size_t)nf);
    if (err == cudaSuccess) err = cudaMemsetAsync(d_out, 0, sizeof(float) * nOut, s);
    if (err == cudaSuccess && d_out64) err = cudaMemsetAsync(d_out64, 0, sizeof(double) * nOut, s);
    if (err == cudaSuccess) {
      k_rbf_cell<<<(nc + kWarps - 1) / kWarps, 32 * kWarps, 0, s>>>(nc, in.maxS, nmax, d_ssz, d_sten, d_cell, d_off,
                                                                    d_gxy, d_gw, in.px, in.py, in.shape, d_refd,
                                                                    d_G, d_status);
      err = cudaGetLastError();
    }
    std::vector<uint8_t> status(nc);
    down(status.data(), d_status, nc);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    // exactly singular P matrices: the host's SVD pseudo-inverse, as the host stage falls back
    std::vector<double> P, G;
    for (int c = 0; c < nc && err == cudaSuccess; ++c) {
      if (status[c] != kCellSingular) continue;
      const int n = in.stencilSize[c] + 1;
      P.resize((size_t)n * n);
      G.resize((size_t)n * n);
      double* slot = d_G + (size_t)c * nmax * nmax;
      err = cudaMemcpy(P.data(), slot, sizeof(double) * n * n, cudaMemcpyDeviceToHost);
      if (err != cudaSuccess) break;
      svd_pinv(n, P.data(), G.data());
      uint8_t flag = kCellOk;
      for (int i = 0; i < n * n; ++i)
        if (!(std::fabs(G[i]) <= 1e10)) {
          flag = kCellTrouble;
          break;
        }
      err = cudaMemcpy(slot, G.data(), sizeof(double) * n * n, cudaMemcpyHostToDevice);
      if (err == cudaSuccess) err = cudaMemcpy(d_status + c, &flag, 1, cudaMemcpyHostToDevice);
    }
    if (err == cudaSuccess && nf > 0) {
      const long long threads = 2LL * nf;
      k_rbf_face<<<(unsigned)((threads + 127) / 128), 128, 0, s>>>(nf, in.maxS, nmax, d_ssz, d_sten, d_cell, d_fxy,
                                                                   d_nb, d_refd, d_G, d_status, in.px, in.py,
                                                                   in.shape, d_out, d_out64);
      err = cudaGetLastError();
    }
    down(RBFbasis, d_out, sizeof(float) * nOut);
    if (rbf64) down(rbf64, d_out64, sizeof(double) * nOut);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (s) cudaStreamDestroy(s);
    if (err != cudaSuccess) {
      set_error("precompute on device %d: %s", device, cudaGetErrorString(err));
      cudaGetLastError();
      st = AFAR_ERR_CUDA;
    }
  }
  if (prev >= 0) cudaSetDevice(prev);
  return st;
}

}  // namespace afar
