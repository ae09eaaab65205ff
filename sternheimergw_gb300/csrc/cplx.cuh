// Complex arithmetic for the Sternheimer kernels, in FP64 (plain drop-in) or
// FP32 (mixed-precision Krylov).  Layout: interleaved (re, im), identical to
// Fortran COMPLEX(dp) / COMPLEX(sp), C99 _Complex and the C-ABI's sgw_zcomplex.
#pragma once
#include <cuda_runtime.h>

#if defined(__CUDACC__)
#define SGW_HD __host__ __device__ __forceinline__
#else
#define SGW_HD inline
#endif

template <typename T>
struct alignas(2 * sizeof(T)) cplx {
  T re, im;
};

using zcd = cplx<double>;
using zcf = cplx<float>;

template <typename T> SGW_HD cplx<T> mk(T r, T i) { return cplx<T>{r, i}; }
template <typename T> SGW_HD cplx<T> operator+(cplx<T> a, cplx<T> b) { return {a.re + b.re, a.im + b.im}; }
template <typename T> SGW_HD cplx<T> operator-(cplx<T> a, cplx<T> b) { return {a.re - b.re, a.im - b.im}; }
template <typename T> SGW_HD cplx<T> operator-(cplx<T> a) { return {-a.re, -a.im}; }
template <typename T> SGW_HD cplx<T> operator*(cplx<T> a, cplx<T> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename T> SGW_HD cplx<T> operator*(T s, cplx<T> a) { return {s * a.re, s * a.im}; }
template <typename T> SGW_HD cplx<T> operator*(cplx<T> a, T s) { return {s * a.re, s * a.im}; }
template <typename T> SGW_HD cplx<T>& operator+=(cplx<T>& a, cplx<T> b) { a.re += b.re; a.im += b.im; return a; }
template <typename T> SGW_HD cplx<T>& operator-=(cplx<T>& a, cplx<T> b) { a.re -= b.re; a.im -= b.im; return a; }
template <typename T> SGW_HD cplx<T> conj(cplx<T> a) { return {a.re, -a.im}; }
// a * conj(b)... helpers used in dot products
template <typename T> SGW_HD cplx<T> cmul_conj_a(cplx<T> a, cplx<T> b) {  // conj(a) * b
  return {a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re};
}
// multiply by i*s (s = +1 or -1)
template <typename T> SGW_HD cplx<T> mul_si(cplx<T> a, int s) { return s > 0 ? cplx<T>{-a.im, a.re} : cplx<T>{a.im, -a.re}; }
// division a / b (Smith's algorithm is not needed: scalars here are well scaled)
template <typename T> SGW_HD cplx<T> operator/(cplx<T> a, cplx<T> b) {
  T d = b.re * b.re + b.im * b.im;
  return {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}
template <typename T> SGW_HD T abs2(cplx<T> a) { return a.re * a.re + a.im * a.im; }

template <typename To, typename From> SGW_HD cplx<To> ccast(cplx<From> a) { return {(To)a.re, (To)a.im}; }

#if defined(__CUDACC__)
__device__ __forceinline__ double fmad_(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fmad_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
// acc += a * b with four fused multiply-adds
template <typename T> __device__ __forceinline__ void cfma(cplx<T>& acc, cplx<T> a, cplx<T> b) {
  acc.re = fmad_(a.re, b.re, acc.re);
  acc.re = fmad_(-a.im, b.im, acc.re);
  acc.im = fmad_(a.re, b.im, acc.im);
  acc.im = fmad_(a.im, b.re, acc.im);
}
// acc += conj(a) * b
template <typename T> __device__ __forceinline__ void cfma_conj(cplx<T>& acc, cplx<T> a, cplx<T> b) {
  acc.re = fmad_(a.re, b.re, acc.re);
  acc.re = fmad_(a.im, b.im, acc.re);
  acc.im = fmad_(a.re, b.im, acc.im);
  acc.im = fmad_(-a.im, b.re, acc.im);
}
#endif
