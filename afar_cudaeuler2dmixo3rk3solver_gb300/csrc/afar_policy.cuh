// Precision policies and small math helpers shared by the AFAR kernels.
//
// A policy fixes the arithmetic type of each part of the stage:
//   W   stored primitive state (cells and ghosts)
//   S   staged stencil values, limiter arithmetic, least-squares and O3 weights
//   G   gradients, face values, TVD states, central flux
//   D   Riemann dissipation (Roe / KFVS)
//   RC  R and Cv as seen by the dissipation
//   F   stored face flux
// The conserved state, the residual gather and the RK update are FP64 under every policy.
//
// PolicyRef reproduces the reference's own mix (float stencils/weights/limiters/dissipation,
// double elsewhere; reference cudaLimiter.h:83-98, basicDataStructure.h:67-73,134,150,
// cudaRiemannSolver.h:16-136).  Under it every expression below is written with the same operand
// types and order as the reference kernel it restates, so nvcc makes the same rounding and
// FMA-contraction decisions; that is what makes the 1e-12 / identical-switch parity possible.
#pragma once

#include <cuda.h>  // CUtensorMap (the type only: the library does not link the driver API)
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace afar {

struct PolicyRef {
  static constexpr int id = 0;
  using W = double;
  using S = float;
  using G = double;
  using D = float;
  using RC = double;
  using F = double;
  static constexpr bool exact_blend = true;
};

struct PolicyFP64 {
  static constexpr int id = 1;
  using W = double;
  using S = double;
  using G = double;
  using D = double;
  using RC = double;
  using F = double;
  static constexpr bool exact_blend = false;
};

struct PolicyMixed {
  static constexpr int id = 2;
  using W = float;
  using S = float;
  using G = float;
  using D = float;
  using RC = float;
  using F = float;
  static constexpr bool exact_blend = false;
};

template <class T>
struct alignas(4 * sizeof(T)) V4 {
  T x, y, z, w;
};
template <class T>
struct alignas(2 * sizeof(T)) V2 {
  T x, y;
};

// A literal of type T that equals the reference's float literal when T is float (x##f) and the
// double literal otherwise.
#define AFAR_LIT(T, x) (std::is_same<T, float>::value ? (T)(x##f) : (T)(x))

// Overloads that resolve like the CUDA C++ math overloads the reference calls.
__device__ __forceinline__ float fmx(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ double fmx(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ float fmn(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ double fmn(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ float fab(float a) { return fabsf(a); }
__device__ __forceinline__ double fab(double a) { return fabs(a); }
__device__ __forceinline__ float sqr_(float a) { return sqrtf(a); }
__device__ __forceinline__ double sqr_(double a) { return sqrt(a); }
__device__ __forceinline__ float rsq_(float a) { return rsqrtf(a); }
__device__ __forceinline__ double rsq_(double a) { return rsqrt(a); }
__device__ __forceinline__ float erfc_(float a) { return erfcf(a); }
__device__ __forceinline__ double erfc_(double a) { return erfc(a); }
__device__ __forceinline__ float exp_(float a) { return expf(a); }
__device__ __forceinline__ double exp_(double a) { return exp(a); }

// Bulk global->shared copies (cp.async.bulk, the TMA unit's untiled form) completing on an
// mbarrier.  Both addresses 16-byte aligned, size a multiple of 16.
__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_to_smem(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for phase `parity` of the barrier for at most `limit` SM clocks (by default 2^31, about
// 1 s); false if it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  const long long limit = 1ll << 31) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}

// cond ? a : b.  The reference writes these selections as arithmetic blends
// (c1*a + c2*b with c1, c2 in {0,1}); the ref policy keeps the blend so that signed zeros and
// non-finite operands propagate the same way.
template <class P, class A, class B>
__device__ __forceinline__ auto pick(bool c1, bool c2, A a, B b) -> decltype(a * 1 + b * 1) {
  if constexpr (P::exact_blend) {
    return c1 * a + c2 * b;
  } else {
    using R = decltype(a * 1 + b * 1);
    return c1 ? (R)a : (R)b;
  }
}

// ---------------------------------------------------------------- float-pair ("double-float") values
// A value hi + lo with |lo| <= ulp(hi)/2 (about 48 significant bits) built from FP32 operations
// only, for the mixed policy's conserved state: GB300's FP64 pipe runs at 1/53 of FP32.  The
// error-free transformations are Knuth's two-sum, Dekker's fast two-sum (|a| >= |b|) and the
// FMA two-product; the explicitly rounded __fadd_rn/__fmul_rn keep the compiler from fusing a
// product into a later sum, which would break the transformations.
struct DF {
  float hi, lo;
};
// The conserved state of one cell as float pairs: 32 bytes, like V4<double>.
struct alignas(16) DF4 {
  V4<float> hi, lo;
};

__device__ __forceinline__ DF df_two_sum(const float a, const float b) {
  const float s = __fadd_rn(a, b);
  const float bp = __fadd_rn(s, -a);
  return DF{s, __fadd_rn(__fadd_rn(a, -__fadd_rn(s, -bp)), __fadd_rn(b, -bp))};
}
__device__ __forceinline__ DF df_fast_two_sum(const float a, const float b) {
  const float s = __fadd_rn(a, b);
  return DF{s, __fadd_rn(b, -__fadd_rn(s, -a))};
}
// a + b, both float pairs (the accurate sum: two-sums of both parts).
__device__ __forceinline__ DF df_add(const DF a, const DF b) {
  DF s = df_two_sum(a.hi, b.hi);
  const DF t = df_two_sum(a.lo, b.lo);
  s = df_fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return df_fast_two_sum(s.hi, __fadd_rn(s.lo, t.lo));
}
// a + b, b a float.
__device__ __forceinline__ DF df_add(const DF a, const float b) {
  const DF s = df_two_sum(a.hi, b);
  return df_fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}
// a * b.
__device__ __forceinline__ DF df_mul(const DF a, const DF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_fast_two_sum(p, e);
}
// a * a.
__device__ __forceinline__ DF df_sqr(const DF a) {
  const float p = __fmul_rn(a.hi, a.hi);
  const float e = __fmaf_rn(__fmul_rn(2.f, a.hi), a.lo, __fmaf_rn(a.hi, a.hi, -p));
  return df_fast_two_sum(p, e);
}
// a / b given r ~ 1/b.hi: one correction of the float quotient, q = q0 + (a - q0 b) r.
__device__ __forceinline__ DF df_div(const DF a, const DF b, const float r) {
  const float q0 = __fmul_rn(a.hi, r);
  const DF qb = df_mul(DF{q0, 0.f}, b);
  const DF rem = df_add(a, DF{-qb.hi, -qb.lo});
  return df_fast_two_sum(q0, __fmul_rn(__fadd_rn(rem.hi, rem.lo), r));
}

}  // namespace afar
