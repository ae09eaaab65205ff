// Register-resident FFT of one line per thread.
//
// fft_reg<T, N, S>(v, tw) transforms the N complex values v[0..N) held in one
// thread's registers.  The mixed-radix Stockham schedule (radix 8, 5, 4, 3, 2)
// is resolved at compile time: every index, every twiddle offset and every
// butterfly is a constant, so the transform is straight-line code with no
// shared-memory traffic, no integer index arithmetic and no barriers.  The
// twiddle table tw[e] = exp(+2 pi i e / N) sits in shared memory; all threads
// read the same entry at the same time (a broadcast).  S = +1 is QE's invfft
// direction, S = -1 fwfft, unscaled.
#pragma once
#include <type_traits>

#include "fft.cuh"

namespace sgw {

// radix of stage `s` for length n (greedy 8, 5, 4, 3, 2), 0 past the last stage
__host__ __device__ constexpr int radix_at(int n, int s) {
  int m = n;
  for (int k = 0;; ++k) {
    int r = (m % 8 == 0) ? 8 : (m % 5 == 0) ? 5 : (m % 4 == 0) ? 4 : (m % 3 == 0) ? 3 : (m % 2 == 0) ? 2 : 0;
    if (m == 1 || r == 0) return 0;
    if (k == s) return r;
    m /= r;
  }
}

template <typename T, int S, int R>
__device__ __forceinline__ void dft_fixed(cplx<T>* v) {
  if constexpr (R == 2) dft2<T, S>(v);
  else if constexpr (R == 3) dft3<T, S>(v);
  else if constexpr (R == 4) dft4<T, S>(v);
  else if constexpr (R == 5) dft5<T, S>(v);
  else dft8<T, S>(v);
}

template <typename T, int N, int S, int STAGE, int NS>
struct FftRegStage {
  static __device__ __forceinline__ void run(cplx<T>* a, cplx<T>* b, const cplx<T>* tw) {
    constexpr int R = radix_at(N, STAGE);
    if constexpr (R == 0) {
#pragma unroll
      for (int i = 0; i < N; ++i) b[i] = a[i];
    } else {
      constexpr int M = N / R;
#pragma unroll
      for (int j = 0; j < M; ++j) {
        const int k = j % NS;
        cplx<T> w[R];
#pragma unroll
        for (int r = 0; r < R; ++r) w[r] = a[j + r * M];
        if (NS > 1) {
#pragma unroll
          for (int r = 1; r < R; ++r) w[r] = w[r] * twid<T, S>(tw, r * k * (N / (NS * R)));
        }
        dft_fixed<T, S, R>(w);
        const int idxD = (j / NS) * NS * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) b[idxD + r * NS] = w[r];
      }
      FftRegStage<T, N, S, STAGE + 1, NS * R>::run(b, a, tw);
    }
  }
};

// Stages alternate the two arrays and the terminal stage copies the last
// result into the other one, so v holds the transform on return either way
// (the compiler drops the dead copy).
template <typename T, int N, int S>
__device__ __forceinline__ void fft_reg(cplx<T>* v, const cplx<T>* tw) {
  cplx<T> b[N];
  FftRegStage<T, N, S, 0, 1>::run(v, b, tw);
}

// Lengths with a compiled register path (a line must fit in one thread's
// registers: up to 48 complex floats or 40 complex doubles).
template <typename T>
__host__ __device__ constexpr bool fft_reg_supported(int n) {
  return n == 16 || n == 18 || n == 20 || n == 24 || n == 25 || n == 27 || n == 30 || n == 32 || n == 36 ||
         n == 40 || (sizeof(T) == 4 && (n == 45 || n == 48));
}

// Call f(std::integral_constant<int, N>) for the supported runtime length n.
template <typename T, class F>
__device__ __forceinline__ void with_len(int n, F&& f) {
  switch (n) {
    case 16: f(std::integral_constant<int, 16>{}); break;
    case 18: f(std::integral_constant<int, 18>{}); break;
    case 20: f(std::integral_constant<int, 20>{}); break;
    case 24: f(std::integral_constant<int, 24>{}); break;
    case 25: f(std::integral_constant<int, 25>{}); break;
    case 27: f(std::integral_constant<int, 27>{}); break;
    case 30: f(std::integral_constant<int, 30>{}); break;
    case 32: f(std::integral_constant<int, 32>{}); break;
    case 36: f(std::integral_constant<int, 36>{}); break;
    case 40: f(std::integral_constant<int, 40>{}); break;
    case 45: if constexpr (sizeof(T) == 4) f(std::integral_constant<int, 45>{}); break;
    case 48: if constexpr (sizeof(T) == 4) f(std::integral_constant<int, 48>{}); break;
    default: break;
  }
}

}  // namespace sgw
