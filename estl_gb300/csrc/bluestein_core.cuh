// bluestein_core.cuh — transforms of any length N through power-of-two FFTs
// (Bluestein's chirp-z algorithm), shared by the CUDA kernels (api.cu) and
// the host emulator.
//
// The reference only runs powers of two: it rounds every length up with
// ceilog (SimpleMath.h:7-11, FFT_OpenCL_Contiguous.h:56), which is wrong for
// other lengths.  With nk = (n^2 + k^2 - (k - n)^2) / 2 the forward DFT is a
// convolution:
//   X_k = w_k * sum_n (x_n w_n) conj(w_{k-n}),   w_n = exp(-i pi n^2 / N),
// computed with M = 2^ceil(log2(2N - 1)) point FFTs:
//   a_m = x_m w_m (m < N, zero above)      A = FFT_M(a)
//   C = A * Bs,  Bs = FFT_M(b) / M,  b_m = conj(w_m) for |m| < N (circular)
//   c = IFFT_M(C) (unnormalised),          X_k = w_k c_k   (k < N).
// The chirp is generated from the exact integer n^2 mod 2N (so its argument
// stays in [-2, 0]) with an FP64 sine/cosine and rounded once to FP32.
// Backward transforms conjugate the input and the output, like every other
// plan here.
#pragma once
#include "fft_core.cuh"

#if !defined(__CUDA_ARCH__)
#include <cmath>
#endif

namespace estl {

constexpr int kBluesteinMaxLogM = 24;  // M <= 2^24, so N <= 2^23

ESTL_CX long long bluestein_m(long long n) {
  long long m = 1;
  while (m < 2 * n - 1) m <<= 1;
  return m;
}

// w_n = exp(-i pi n^2 / N) rounded to FP32.
ESTL_HD cf32 bluestein_chirp(long long n, long long N) {
  const unsigned long long q = ((unsigned long long)n * (unsigned long long)n) % (2ULL * (unsigned long long)N);
  const double x = -(double)q / (double)N;  // in (-2, 0]
#if defined(__CUDA_ARCH__)
  double s, c;
  sincospi(x, &s, &c);
  return cf32{(float)c, (float)s};
#else
  const long double pi = 3.14159265358979323846264338327950288L;
  return cf32{(float)cosl(pi * (long double)x), (float)sinl(pi * (long double)x)};
#endif
}

// a_m of transform b: the conjugated (backward) or plain input times the chirp,
// zero for m >= N.
ESTL_HD cf32 bluestein_pre(const cf32* x, const cf32* chirp, long long m, long long N, float sgn) {
  if (m >= N) return cf32{0.f, 0.f};
  return cmul(conj_if(x[m], sgn), chirp[m]);
}

// b_m = conj(w_{|m|}) on the circle of length M (before its FFT).
ESTL_HD cf32 bluestein_kernel_elem(const cf32* chirp, long long m, long long N, long long M) {
  if (m < N) return cf32{chirp[m].x, -chirp[m].y};
  if (m > M - N) return cf32{chirp[M - m].x, -chirp[M - m].y};
  return cf32{0.f, 0.f};
}

// X_k = w_k c_k, conjugated back for a backward transform.
ESTL_HD cf32 bluestein_post(const cf32* c, const cf32* chirp, long long k, float sgn) {
  return conj_if(cmul(c[k], chirp[k]), sgn);
}

}  // namespace estl
