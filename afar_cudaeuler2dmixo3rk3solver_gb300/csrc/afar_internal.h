// Internal helpers shared by the host translation units of libafar.
#pragma once

#include <cstdarg>
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

}  // namespace afar
