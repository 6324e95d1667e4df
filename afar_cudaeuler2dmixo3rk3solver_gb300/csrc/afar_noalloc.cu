// afar_adjustTimeStep_noalloc: the Courant time step of a state the caller already holds on the
// device, computed without allocating any device memory.
//
// Who needs it: callers that cannot call cudaMalloc, such as an application that hands out all of
// the GPU's memory from its own pool and forbids libraries to allocate, or one that has reserved its
// device memory budget up front.  They pass device pointers to the reference-layout arrays they
// already own and a device pointer for the result; the only scratch (one minimum per block of
// faces) lives in a file-scope device array that every GPU which loads this library holds until the
// process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "afar_internal.h"

namespace {

constexpr int kNoallocBlock = 256;
constexpr int kNoallocMaxBlocks = 65536;  // 512 KiB of scratch: up to 16,777,216 internal faces

// Per-block minima of one call.  Each call writes entries [0, nblocks) before reading them, so no
// entry needs clearing; every call shares the array, so calls that overlap on the GPU race.
static __device__ __align__(256) double g_noalloc_block_min[kNoallocMaxBlocks];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
// Device address of g_noalloc_block_min, per device, resolved by the first call on that device and
// kept for the life of the process (a cudaDeviceReset, which reloads this file's device code, is not
// supported after that first call).
double* g_scratch[kMaxDevices] = {};

// setDeltaT of the reference (cudaFieldOperation.h:124-180) on the reference layout; one minimum
// per block into the scratch array.
__global__ void __launch_bounds__(kNoallocBlock) k_noalloc_block_min(const afar_basicFieldData* __restrict__ FD,
                                                                     const afar_meshCellData* __restrict__ CELL,
                                                                     const afar_meshFaceData* __restrict__ FACE,
                                                                     const int* __restrict__ neighbour, int nf,
                                                                     double R, double Cv, double CFL,
                                                                     double* __restrict__ block_min) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  double dt = 1e5;
  if (f < nf) {
    const int own = neighbour[2 * f], nei = neighbour[2 * f + 1];  // in [0, Nc+Nb): the caller's guarantee
    const double deltaR = hypot(CELL[nei].x - CELL[own].x, CELL[nei].y - CELL[own].y);
    const double fraction = hypot(FACE[f].x - CELL[own].x, FACE[f].y - CELL[own].y) / deltaR;
    const double Sfx = FACE[f].Sfx, Sfy = FACE[f].Sfy, magSf = FACE[f].magSf;
    dt = CFL * deltaR * magSf /
         ((1.0 - fraction) * fabs(FD[own].Ux * Sfx + FD[own].Uy * Sfy) +
          fraction * fabs(FD[nei].Ux * Sfx + FD[nei].Uy * Sfy) +
          sqrt((R / Cv + 1.0) * R * ((1.0 - fraction) * FD[own].T + fraction * FD[nei].T)) * magSf);
    if (!(dt >= 0.0)) dt = 1e300;  // a NaN step never wins the minimum
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) dt = fmin(dt, __shfl_xor_sync(0xffffffffu, dt, o));
  __shared__ double wmin[kNoallocBlock / 32];
  if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = dt;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = wmin[0];
    for (int k = 1; k < kNoallocBlock / 32; ++k) m = fmin(m, wmin[k]);
    block_min[blockIdx.x] = m;
  }
}

// Min over the nblocks block minima and 1e5 (adjustTimeStep, GPUevolve.cu:197-203) into *out.
__global__ void __launch_bounds__(1024) k_noalloc_finish(const double* __restrict__ block_min, int nblocks,
                                                         double* __restrict__ out) {
  double m = 1e5;
  for (int i = threadIdx.x; i < nblocks; i += blockDim.x) m = fmin(m, block_min[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ double wmin[32];
  if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = wmin[0];
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) r = fmin(r, wmin[k]);
    *out = r;
  }
}

}  // namespace

using afar::set_error;

extern "C" afar_status afar_adjustTimeStep_noalloc(const afar_basicFieldData* FD, const afar_meshCellData* CELL,
                                                   const afar_meshFaceData* FACE, const int* neighbour, int facesNum,
                                                   double R, double Cv, double CFL, double* deltaT, void* stream) {
  if (facesNum < 0 || !deltaT || (facesNum > 0 && (!FD || !CELL || !FACE || !neighbour)) || !(R > 0.0) ||
      !(Cv > 0.0) || !(CFL > 0.0)) {
    set_error("afar_adjustTimeStep_noalloc: null pointer or non-positive R, Cv, CFL or negative facesNum");
    return AFAR_ERR_ARGUMENT;
  }
  const long long nblocks = ((long long)facesNum + kNoallocBlock - 1) / kNoallocBlock;
  if (nblocks > kNoallocMaxBlocks) {
    set_error("afar_adjustTimeStep_noalloc: facesNum %d exceeds the limit of %d internal faces (fixed scratch of "
              "%d block minima)",
              facesNum, kNoallocMaxBlocks * kNoallocBlock, kNoallocMaxBlocks);
    return AFAR_ERR_LIMIT;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    set_error("afar_adjustTimeStep_noalloc: no usable current device (%s)", cudaGetErrorString(e));
    return AFAR_ERR_CUDA;
  }
  double* scratch;
  {
    // first call on a device: resolve the device address of the scratch array with that device current
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_block_min);
      if (e != cudaSuccess || !p) {
        set_error("afar_adjustTimeStep_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev,
                  cudaGetErrorString(e));
        return AFAR_ERR_CUDA;
      }
      g_scratch[dev] = static_cast<double*>(p);
    }
    scratch = g_scratch[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (nblocks > 0)
    k_noalloc_block_min<<<(unsigned)nblocks, kNoallocBlock, 0, st>>>(FD, CELL, FACE, neighbour, facesNum, R, Cv, CFL,
                                                                      scratch);
  k_noalloc_finish<<<1, 1024, 0, st>>>(scratch, (int)nblocks, deltaT);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("afar_adjustTimeStep_noalloc: launch failed: %s", cudaGetErrorString(e));
    return AFAR_ERR_CUDA;
  }
  return AFAR_OK;
}
