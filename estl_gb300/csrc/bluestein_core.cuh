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
#include "conv_core.cuh"
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

// ---------------------------------------------------------------------------
// M <= 2^14: the whole algorithm in one tile kernel, C transforms per CTA:
//   v = a (pre-multiplied input, zero-padded to M)  -> FFT_M
//   v = conj(v * Bs)                                -> FFT_M  (= conj(c))
//   X_k = w_k conj(v_k)                             (k < N)
// One HBM read of the input and one write of the output per transform (the
// chirp and the kernel spectrum, N + M values shared by every transform,
// stay in L2), instead of five passes over M-element work buffers.
// ---------------------------------------------------------------------------
constexpr int kBlueFusedMaxLog = 14;

// Tile shapes of the fused kernel, one per M (X(log2 M, log2 elements a
// thread, log2 radix, log2 transforms a CTA)): 256 threads up to 2^12, 512 at
// 2^13 (radix 16, 148 bytes of register spill a thread) and 2^14 (radix 32,
// 744 bytes: with two transforms and the chirp and spectrum products a thread
// holds more than its 128 registers).
#define ESTL_BLUE_TILES(X) \
  X(3, 3, 4, 8)            \
  X(4, 4, 4, 8)            \
  X(5, 4, 4, 7)            \
  X(6, 4, 4, 6)            \
  X(7, 4, 4, 5)            \
  X(8, 4, 4, 4)            \
  X(9, 4, 4, 3)            \
  X(10, 4, 4, 2)           \
  X(11, 4, 4, 1)           \
  X(12, 4, 4, 0)           \
  X(13, 4, 4, 0)           \
  X(14, 5, 5, 0)
ESTL_CX bool bluestein_fused(long long m) { return m <= (1LL << kBlueFusedMaxLog); }

// A point the compiler does not move memory accesses across (no instruction).
ESTL_HD void compiler_order() {
#if defined(__CUDA_ARCH__)
  asm volatile("" ::: "memory");
#endif
}

struct BlueArgs {
  Ptr<const cf32> in;     // count transforms of N
  Ptr<cf32> out;          // count transforms of N
  Ptr<const cf32> chirp;  // w_n, N values
  Ptr<const cf32> spec;   // Bs = FFT_M(b) / M, M values (four-step: in the middle kernel's order)
  Ptr<const cf32> bank;
  long long n;
  long long count;
  float sgn;
  // four-step (M > 2^14): M = 2^logm, scratch s1 / s2 of count * M
  int logm = 0;
  Ptr<cf32> s1{nullptr, 0};
  Ptr<cf32> s2{nullptr, 0};
};

template <int LOGM, int LOGE, int LOGR, int LOGC>
struct BlueSingleKernel {
  using K = SingleKernel<LOGM, LOGE, LOGR, LOGC>;
  using TL = typename K::TL;
  static constexpr int C = K::C;
  static constexpr int NT = K::NT;
  static constexpr int SMEM_ELEMS = K::SMEM_ELEMS;
  // up to 128 registers a thread: the chirp and spectrum products beside the
  // tile's elements spill at the plain tiles' 64
  static constexpr int MIN_BLOCKS = NT <= 256 ? 2 : 1;

  ESTL_HD static void run(const BlueArgs& a, long long cta, int tid, cf32* smraw) {
    const int t = tid & (TL::T - 1);
    const int c = tid >> TL::LOGT;
    const long long f = cta * C + c;
    const bool valid = f < a.count;
    const int n = (int)a.n;
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, K::EXCH};
    const typename K::Sidx sidx{};
    const Ptr<const cf32> x = valid ? a.in.sub(f * a.n, a.n) : Ptr<const cf32>{a.in.p, 0};
    // The chirp and spectrum factors are loaded in groups of 8 slots with a
    // compiler ordering point between groups, so that they are not all
    // hoisted beside the tile's elements (measured without the groups:
    // N = 3000 660 -> 601 GB/s, N = 6000 561 -> 545, N = 1000 unchanged).
    cf32 v[TL::E];
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const int m = t + TL::T * j;
      v[j] = valid && m < n ? conj_if(ldcs(x, m), a.sgn) : cf32{0.f, 0.f};
    }
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const int m = t + TL::T * j;
      if (m < n) v[j] = cmul(v[j], ldg(a.chirp, m));
      if ((j & 7) == 7) compiler_order();
    }
    run_passes<TL, 0>(v, t, c, sm, tw, sidx);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const cf32 p = cmul(v[j], ldg(a.spec, t + TL::T * j));
      v[j] = cf32{p.x, -p.y};
      if ((j & 7) == 7) compiler_order();
    }
    run_passes<TL, 0>(v, t, c, sm, tw, sidx);
    if (valid) {
      const Ptr<cf32> y = a.out.sub(f * a.n, a.n);
#pragma unroll
      for (int j = 0; j < TL::E; ++j) {
        const int k = t + TL::T * j;
        if (k < n) stcs(y, k, conj_if(cmul(cf32{v[j].x, -v[j].y}, ldg(a.chirp, k)), a.sgn));
        if ((j & 7) == 7) compiler_order();
      }
    }
  }
};

// ---------------------------------------------------------------------------
// 2^14 < M <= 2^22: the convolution's three-launch four-step
// (conv_core.cuh: ConvColKernel, ConvMidKernel, ConvOutKernel), M = N1 * N2,
// with complex data and the chirps folded into its first load and last store:
//   A  column n1 of the pre-multiplied input a_{n1 + N1 n2} (zero for n >= N):
//      N2-point DFTs, times w_M^{n1 k2}            -> s1[f*M + k2*N1 + n1]
//   B  row k2: N1-point DFT, times Bs (stored as Bp[k2*N1 + k1] = Bs[k2 + N2 k1]),
//      conj, N1-point DFT, times w_M^{k2 n1}       -> s2[f*M + n1*N2 + k2]
//   C  row n1 of s2: N2-point DFT = conj(c_k), k = n1 + N1 n2,
//      X_k = w_k c_k (k < N)                        -> output
// Three HBM round trips over M-element rows (the input and output only over
// N) instead of five plus two per M-point FFT pass.
// ---------------------------------------------------------------------------
ESTL_CX bool bluestein_four_step(long long m) { return m > (1LL << kBlueFusedMaxLog) && m <= (1LL << 22); }
ESTL_CX int bluestein_logn2(int logm) { return logm / 2; }  // column DFT length N2 (the convolution's split)

template <int LOGM, int LOGE, int LOGR, int LOGC>
struct BlueColKernel {
  using B = ConvColKernel<LOGM, LOGE, LOGR, LOGC>;
  using TL = typename B::TL;
  // up to 128 registers a thread (the chirp products spill at the plain column tile's 64)
  static constexpr int C = B::C, NT = B::NT, SMEM_ELEMS = B::SMEM_ELEMS, MIN_BLOCKS = NT <= 256 ? 2 : 1;
  ESTL_HD static void run(const BlueArgs& a, long long cta, int tid, cf32* smraw) {
    const int c = tid & (C - 1);
    const int t = tid >> LOGC;
    const int logn1 = a.logm - LOGM;
    const int M = 1 << a.logm, N1 = 1 << logn1;
    const int nblk = N1 >> LOGC;
    const long long f = cta / nblk;
    const int n1 = (int)(cta - f * nblk) * C + c;
    const int n = (int)a.n;
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, B::EXCH};
    const Ptr<const cf32> x = a.in.sub(f * a.n, a.n);
    cf32 v[TL::E];
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const int m = n1 + ((t + TL::T * j) << logn1);
      v[j] = m < n ? cmul(conj_if(ldcs(x, m), a.sgn), ldg(a.chirp, m)) : cf32{0.f, 0.f};
    }
    run_passes<TL, 0>(v, t, c, sm, tw, typename B::Sidx{});
    const Ptr<cf32> o = a.s1.sub(f * M, M);
    fourstep_twiddle<TL>(v, n1, t, a.logm, a.bank);  // times w_M^{n1 k2}, k2 = t + T j
#pragma unroll
    for (int j = 0; j < TL::E; ++j) o[((t + TL::T * j) << logn1) + n1] = v[j];
  }
};

template <int LOGM, int LOGE, int LOGR, int LOGC>
struct BlueMidKernel {
  using B = ConvMidKernel<LOGM, LOGE, LOGR, LOGC>;
  using TL = typename B::TL;
  static constexpr int C = B::C, NT = B::NT, SMEM_ELEMS = B::SMEM_ELEMS, MIN_BLOCKS = B::MINB;
  ESTL_HD static void run(const BlueArgs& a, long long cta, int tid, cf32* smraw) {
    const int t = tid & (TL::T - 1);
    const int c = tid >> TL::LOGT;
    const int M = 1 << a.logm;
    const int logn2 = a.logm - LOGM;
    const int nblk = 1 << (logn2 - LOGC);
    const long long f = cta / nblk;
    const int k2_0 = (int)(cta - f * nblk) * C;
    const int k2 = k2_0 + c;
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, B::EXCH};
    const typename B::Sidx sidx{};
    const Ptr<cf32> s1 = a.s1.sub(f * M + (long long)k2 * TL::M, TL::M);
    cf32 v[TL::E];
#pragma unroll
    for (int j = 0; j < TL::E; ++j) v[j] = s1[t + TL::T * j];
    run_passes<TL, 0>(v, t, c, sm, tw, sidx);
    const Ptr<const cf32> h = a.spec.sub((long long)k2 * TL::M, TL::M);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) v[j] = cconj(cmul(v[j], ldg(h, t + TL::T * j)));
    run_passes<TL, 0>(v, t, c, sm, tw, sidx);
    fourstep_twiddle<TL>(v, k2, t, a.logm, a.bank);  // times w_M^{k2 n1}, n1 = t + T j
#pragma unroll
    for (int j = 0; j < TL::E; ++j) sm[sidx(c, t + TL::T * j)] = v[j];
    ESTL_SYNC();
    const int c2 = tid & (C - 1);
    const int t2 = tid >> LOGC;
    const Ptr<cf32> o = a.s2.sub(f * M, M);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const int n1 = t2 + TL::T * j;
      o[(n1 << logn2) + k2_0 + c2] = sm[sidx(c2, n1)];
    }
  }
};

template <int LOGM, int LOGE, int LOGR, int LOGC>
struct BlueOutKernel {
  using B = ConvOutKernel<LOGM, LOGE, LOGR, LOGC>;
  using TL = typename B::TL;
  static constexpr int C = B::C, NT = B::NT, SMEM_ELEMS = B::SMEM_ELEMS, MIN_BLOCKS = B::MINB;
  ESTL_HD static void run(const BlueArgs& a, long long cta, int tid, cf32* smraw) {
    const int t = tid & (TL::T - 1);
    const int c = tid >> TL::LOGT;
    const int M = 1 << a.logm;
    const int logn1 = a.logm - LOGM;
    const int nblk = 1 << (logn1 - LOGC);
    const long long f = cta / nblk;
    const int n1_0 = (int)(cta - f * nblk) * C;
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, B::EXCH};
    const typename B::Sidx sidx{};
    const Ptr<cf32> s2 = a.s2.sub(f * M + (long long)(n1_0 + c) * TL::M, TL::M);
    cf32 v[TL::E];
#pragma unroll
    for (int j = 0; j < TL::E; ++j) v[j] = s2[t + TL::T * j];
    run_passes<TL, 0>(v, t, c, sm, tw, sidx);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) sm[sidx(c, t + TL::T * j)] = v[j];
    ESTL_SYNC();
    const int c2 = tid & (C - 1);
    const int t2 = tid >> LOGC;
    const int n = (int)a.n;
    const Ptr<cf32> y = a.out.sub(f * a.n, a.n);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const int k = n1_0 + c2 + ((t2 + TL::T * j) << logn1);
      if (k < n) stcs(y, k, conj_if(cmul(cconj(sm[sidx(c2, t2 + TL::T * j)]), ldg(a.chirp, k)), a.sgn));
    }
  }
};

}  // namespace estl
