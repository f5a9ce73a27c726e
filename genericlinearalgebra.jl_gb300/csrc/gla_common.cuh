// Shared device helpers for the GB300 self-adjoint eigensolver kernels.
//
// GB300 facts that shape this file (measured on the target with CUDA events
// and clock64): an FP64 warp instruction (DFMA/DMUL/DADD/DSETP) occupies its
// SM sub-partition's FP64 unit for ~64-68 cycles whether 1 or 32 lanes are
// active; IEEE FP64 divide and sqrt have ~640-675 cycle latency; the MUFU
// reciprocal seed rcp.approx.ftz.f64 answers in ~19 cycles; FP32 FFMA has
// 4.5-cycle latency at ~73 TFLOP/s. Hence: FP64 work is kept lane-dense,
// scalar FP64 recurrences run one matrix per lane, FP64 comparisons in hot
// loops are done on the integer bit patterns, and reciprocals/rsqrts use a
// hardware seed refined by Newton-Raphson (the classical iteration
// y <- y + y(1 - x y) for 1/x and y <- y + y(1 - x y^2)/2 for 1/sqrt(x)).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define GLA_DEV __device__ __forceinline__

namespace gla {

// ---------------------------------------------------------------- precision
template <class T> struct prec;

template <> struct prec<double> {
  static constexpr double eps = 0x1p-52;          // Julia eps(Float64)
  static constexpr int mant = 52;
  static constexpr int expbias = 1023;
  typedef unsigned long long bits_t;
  GLA_DEV static bits_t bits(double x) { return (bits_t)__double_as_longlong(x); }
  GLA_DEV static int biased_exp(double x) { return (int)((bits(x) >> 52) & 0x7ff); }
  GLA_DEV static double sqrt_ieee(double x) { return __dsqrt_rn(x); }
  GLA_DEV static double div_ieee(double a, double b) { return __ddiv_rn(a, b); }
  // 1/x: rcp.approx.ftz.f64 seed (relative error below 2^-22) refined by two
  // Newton-Raphson steps to within ~1 ulp. Only for normal, finite x whose
  // reciprocal is normal (callers guard the range).
  GLA_DEV static double rcp(double x) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    return fma(y, e, y);
  }
  // 1/sqrt(x): rsqrt.approx.ftz.f64 seed refined by two Newton-Raphson steps.
  GLA_DEV static double rsqrt(double x) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double h = x * y;
    double r = fma(-h, y, 1.0);
    y = fma(0.5 * y, r, y);
    h = x * y;
    r = fma(-h, y, 1.0);
    return fma(0.5 * y, r, y);
  }
  // True when |x| lies in [2^-900, 2^900]: reciprocals and squares of such
  // values stay normal, so the seeded Newton paths above are safe.
  GLA_DEV static bool tame(double x) {
    int be = biased_exp(x);
    return be >= expbias - 900 && be <= expbias + 900;
  }
};

template <> struct prec<float> {
  static constexpr float eps = 0x1p-23f;           // Julia eps(Float32)
  static constexpr int mant = 23;
  static constexpr int expbias = 127;
  typedef unsigned int bits_t;
  GLA_DEV static bits_t bits(float x) { return (bits_t)__float_as_uint(x); }
  GLA_DEV static int biased_exp(float x) { return (int)((bits(x) >> 23) & 0xff); }
  GLA_DEV static float sqrt_ieee(float x) { return __fsqrt_rn(x); }
  GLA_DEV static float div_ieee(float a, float b) { return __fdiv_rn(a, b); }
  GLA_DEV static float rcp(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    float e = fmaf(-x, y, 1.0f);
    return fmaf(y, e, y);
  }
  GLA_DEV static float rsqrt(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    float h = x * y;
    float r = fmaf(-h, y, 1.0f);
    return fmaf(0.5f * y, r, y);
  }
  GLA_DEV static bool tame(float x) {
    int be = biased_exp(x);
    return be >= expbias - 60 && be <= expbias + 60;
  }
};

template <class T> GLA_DEV T tabs(T x) { return x < 0 ? -x : x; }
GLA_DEV double tabs(double x) { return fabs(x); }
GLA_DEV float tabs(float x) { return fabsf(x); }
GLA_DEV double tcopysign(double x, double y) { return copysign(x, y); }
GLA_DEV float tcopysign(float x, float y) { return copysignf(x, y); }
GLA_DEV bool tisfinite(double x) { return isfinite(x); }
GLA_DEV bool tisfinite(float x) { return isfinite(x); }

// |a| <= |b| on the integer bit patterns (valid for non-NaN a, b); runs on the
// integer pipe instead of the FP64 compare unit.
template <class T> GLA_DEV bool abs_le(T a, T b) {
  typedef typename prec<T>::bits_t B;
  const B mask = ~((B)1 << (sizeof(B) * 8 - 1));
  return (prec<T>::bits(a) & mask) <= (prec<T>::bits(b) & mask);
}

// hypot(x, y) following C. F. Borges, "An Improved Algorithm for hypot(a,b)",
// ACM TOMS 47 (2021) (fused-correction variant; the algorithm Julia's hypot
// uses). Called once per sweep, not per rotation.
template <class T> GLA_DEV T hypot_borges(T x, T y) {
  const T eps = prec<T>::eps;
  T ax = tabs(x), ay = tabs(y);
  if (isinf(ax) || isinf(ay)) return (T)INFINITY;
  if (ay > ax) { T t = ax; ax = ay; ay = t; }
  if (ay <= ax * prec<T>::sqrt_ieee(eps / 2)) return ax;
  const T fmin = sizeof(T) == 8 ? (T)0x1p-1022 : (T)0x1p-126f;
  const T fmax = sizeof(T) == 8 ? (T)1.7976931348623157e308 : (T)3.40282347e38f;
  T scale = eps * prec<T>::sqrt_ieee(fmin);
  if (ax > prec<T>::sqrt_ieee(fmax / 2)) {
    ax *= scale;
    ay *= scale;
    scale = 1 / scale;
  } else if (ay < prec<T>::sqrt_ieee(fmin)) {
    ax /= scale;
    ay /= scale;
  } else {
    scale = 1;
  }
  T h = prec<T>::sqrt_ieee(fma(ax, ax, ay * ay));
  T hsq = h * h;
  T axsq = ax * ax;
  h -= (fma(-ay, ay, hsq - axsq) + fma(h, h, -hsq) - fma(ax, ax, -axsq)) / (2 * h);
  return h * scale;
}

// ---------------------------------------------------------------- reductions
template <class T> GLA_DEV T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
GLA_DEV unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// Block-wide sum over all threads of the block; red must hold blockDim/32
// entries. Every thread gets the result.
template <class T> GLA_DEV T block_sum(T v, T* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  T s = 0;
  for (int i = 0; i < nw; i++) s += red[i];
  return s;
}

}  // namespace gla
