// Internal helpers shared by the host translation units of libafar.
#pragma once

#include <cstdarg>
#include <cstdint>
#include <cstdio>

#include "../../include/afar.h"

namespace afar {

// Records the message returned by afar_last_error() on this thread.
void set_error(const char* fmt, ...)
#if defined(__GNUC__)
    __attribute__((format(printf, 1, 2)))
#endif
    ;

// Jacobi-SVD pseudo-inverse of a row-major n x n matrix (afar_precompute.cpp).
void svd_pinv(int n, const double* A, double* G);

// Inputs of the RBF stage of the precompute (P matrices, their inverses, O3 face weights).
struct RbfInputs {
  int nc, nf, nb, maxS;               // cells, internal faces, boundary faces, maximum stencil size
  const uint8_t* stencilSize;         // [nc] stencil size without the cell itself
  const int* stencil;                 // [maxS*nc] global stencil ids (cells, or nc + boundary face)
  const afar_meshCellData* CELL;      // [nc+nb] cell centres, then boundary face centres
  const afar_meshFaceData* FACE;      // [nf+...] face centres of the internal faces come first
  const int* neighbour;               // [2*nf] owner, neighbour of each internal face
  const int* gq_off;                  // [nc+nb+1] Gauss points of cells then boundary faces (CSR)
  const double* gq_xy;                // [2*total] point coordinates (x, y)
  const double* gq_w;                 // [total] weights
  double px, py;                      // periods of a periodic mesh (0: not periodic)
  double shape;                       // multiquadric shape factor
};

// The RBF stage on CUDA device `device` (afar_precompute_gpu.cu): writes RBFbasis [2*(maxS+1)*nf]
// and, when non-null, rbf64 (the same weights before rounding to float).  The arrays are
// bit-identical to the host stage's.  Returns AFAR_OK or AFAR_ERR_CUDA (message set).
afar_status rbf_stage_device(int device, const RbfInputs& in, float* RBFbasis, double* rbf64);

}  // namespace afar
