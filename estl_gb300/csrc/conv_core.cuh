// conv_core.cuh — FFT convolution tile kernels (real signal * real filter).
//
// Reference: Convolution2D_FFT::convolve (Convolution.h:95-154): zero-pad both
// operands to nextPowerOf2(W + K - 1) (:89-97), forward FFT of both (:122-123),
// pointwise product (or product with the conjugate for correlation,
// :125-137), inverse FFT (:139), scale 1/(W*H*K^[0]) and crop (:141-148).
// Restated here in 1D for a batch of independent requests, with
//  * the filter spectrum computed once per filter and pre-scaled by 1/N
//    (plain linear convolution) or 1/(N * sum h) with the kernel-centring
//    shift (reference-compatible mode), conjugated for correlation;
//  * the inverse transform taken as conj(FFT(conj(Y))) so that it reuses the
//    forward register layout, and the real part of conj(z) is Re(z), so the
//    final conjugation disappears;
//  * N <= 2^14: one kernel per tile of requests: load padded real signal,
//    forward FFT, multiply, second FFT, store real part — one HBM read of the
//    signal and of the spectrum, one HBM write of the output;
//  * N > 2^14: four-step with the spectrum kept in the row-pass order
//    Hp[k2*N1 + k1] = H[k2 + N2*k1] so that the multiply, the inverse row DFT
//    and the forward row DFT fuse into one kernel (3 kernels in total).
#pragma once
#include "fft_core.cuh"

#if !defined(__CUDA_ARCH__)
#include <cmath>
#endif

namespace estl {

// One request (or one filter) inside a launch.  Offsets are element offsets
// into the packed arrays of the launch.
struct ConvRow {
  long long sig_off;   // real input (signal, or filter for the spectrum kernels)
  long long spec_off;  // complex filter spectrum (read by conv kernels, written by spectrum kernels)
  long long out_off;   // real output
  int sig_len;         // valid input samples; the rest of the N-point row is zero
  int out_len;         // output samples written
  int out_shift;       // first sample of the circular result that is written; output m is
                       // sample (m + out_shift) mod N (the reference's cyclic kernel shift,
                       // Convolution.h:113-120, wraps when out_shift + out_len > N)
  float scale;         // spectrum kernels: multiplies the spectrum (1/N, or 1/(N*sum h))
  float conj;          // spectrum kernels: -1 stores conj(H) (correlation), +1 H
  int dc_norm;         // conv kernels: divide the output by N * spectrum[0] (= sum of the
                       // filter): the 1/K^[0] normalisation of Convolution.h:141-143
};

struct ConvArgs {
  Ptr<const ConvRow> rows;
  long long nrows;
  Ptr<const float> sig;
  Ptr<const cf32> spec;
  Ptr<cf32> spec_out;
  Ptr<float> out;
  Ptr<cf32> s1;        // four-step scratch: N per row
  Ptr<cf32> s2;        // four-step scratch: N per row
  Ptr<const cf32> bank;
  int logn;
  int split;   // tensor-core kernels: SplitKind of the radix-16 passes (tc_core.cuh)
  int shared;  // paired kernels: every request uses one filter spectrum H (not an A / B pair)
};

ESTL_HD cf32 cconj(cf32 v) { return {v.x, -v.y}; }

// w^j (0 <= j < 16) from w, w^2, w^4, w^8: at most three products.
ESTL_HD cf32 pow16(int j, cf32 w1, cf32 w2, cf32 w4, cf32 w8) {
  cf32 r{1.f, 0.f};
  bool one = true;
  const cf32 f[4] = {w1, w2, w4, w8};
#pragma unroll
  for (int b = 0; b < 4; ++b)
    if (j & (1 << b)) {
      r = one ? f[b] : cmul(r, f[b]);
      one = false;
    }
  return r;
}

// The real-input split twiddles w_N^{k2 + N2 k1} of a row tile's slots
// k1 = t + T j: the base w_N^{k2 + N2 t} and the step powers W^1, W^2, W^4,
// W^8 (W = w_N^{N2 T}) from the table, slot j's factor as base * W^j.
struct SplitTwiddles {
  cf32 base, w1, w2, w4, w8;
  ESTL_HD cf32 operator()(int j) const { return j ? cmul(base, pow16(j, w1, w2, w4, w8)) : base; }
};
ESTL_HD SplitTwiddles split_twiddles(const Ptr<const cf32>& bank, int logn_full, int k2, int t, int logn2, int T) {
  const int s = T << logn2;
  return SplitTwiddles{twiddle_n(bank, logn_full, k2 + (t << logn2)), twiddle_n(bank, logn_full, s),
                       twiddle_n(bank, logn_full, 2 * s), twiddle_n(bank, logn_full, 4 * s),
                       twiddle_n(bank, logn_full, 8 * s)};
}

// 1 / (N * spectrum DC) when the row asks for the reference's DC
// normalisation, else 1 (the stored spectrum already carries 1/N).
ESTL_HD float dc_factor(const ConvArgs& a, const ConvRow& r) {
  if (!r.dc_norm) return 1.f;
  const float dc = ldg(a.spec, r.spec_off).x;
  return 1.f / ((float)(1 << a.logn) * dc);
}

// ---------------------------------------------------------------------------
// N <= 2^14: whole requests in one CTA (C requests per CTA)
// ---------------------------------------------------------------------------
template <int LOGM, int LOGE, int LOGR, int LOGC, bool TC = false>
struct ConvSingleKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  static constexpr int CS = row_stride(TL::MP, TL::T >= 16 ? 16 : TL::T * C >= 16 ? 16 / TL::T : C);
  static constexpr int EXCH = (TL::P > 1) ? C * CS : 0;
  static constexpr int TC_OFF = (EXCH + 1) & ~1;  // 16-byte aligned tensor-core area
  static constexpr int SMEM_ELEMS = TC ? TC_OFF + (int)((tc_area_words(NT / 32) + 1) / 2) : EXCH;
  static_assert(NT <= 1024, "too many threads");
  static_assert(!TC || NT % 32 == 0, "tensor-core tiles run whole warps");
  static constexpr int MINB = TC ? (NT <= 256 ? 2 : 1) : min_blocks(NT, TL::E);
  struct Sidx {
    ESTL_HD int operator()(int c, int m) const { return c * CS + TL::pad(m); }
  };

  ESTL_HD static void load_real(cf32 (&v)[TL::E], const ConvArgs& a, const ConvRow& r, int t) {
    const Ptr<const float> s = a.sig.sub(r.sig_off, r.sig_len);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const int pos = t + TL::T * j;
      v[j] = cf32{pos < r.sig_len ? s[pos] : 0.f, 0.f};
    }
  }

  // mode 0: convolution (signal -> real output); mode 1: filter -> spectrum
  template <int MODE>
  ESTL_HD static void run_mode(const ConvArgs& a, long long cta, int tid, cf32* smraw) {
    const int t = tid & (TL::T - 1);
    const int c = tid >> TL::LOGT;
    const long long ri = cta * C + c;
    const bool valid = ri < a.nrows;
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, EXCH};
    if constexpr (TC) tc_init_atab(Ptr<uint32_t>{reinterpret_cast<uint32_t*>(smraw + TC_OFF), kTcAtabWords}, a.split, tid, NT);
    ConvRow r{};
    if (valid) r = a.rows[ri];
    cf32 v[TL::E];
    if (valid) {
      load_real(v, a, r, t);
    } else {
#pragma unroll
      for (int j = 0; j < TL::E; ++j) v[j] = cf32{0.f, 0.f};
    }
    any_passes<TC, TL>(v, t, c, sm, tw, Sidx{}, smraw + TC_OFF, a.split, tid);
    if constexpr (MODE == 1) {
      if (valid) {
        const Ptr<cf32> o = a.spec_out.sub(r.spec_off, TL::M);
#pragma unroll
        for (int j = 0; j < TL::E; ++j) o[t + TL::T * j] = cf32{v[j].x * r.scale, v[j].y * r.scale * r.conj};
      }
    } else {
      if (valid) {
        const Ptr<const cf32> h = a.spec.sub(r.spec_off, TL::M);
#pragma unroll
        for (int j = 0; j < TL::E; ++j) v[j] = cconj(cmul(v[j], ldg(h, t + TL::T * j)));
      }
      any_passes<TC, TL>(v, t, c, sm, tw, Sidx{}, smraw + TC_OFF, a.split, tid);
      if (valid) {
        const Ptr<float> o = a.out.sub(r.out_off, r.out_len);
        const float g = dc_factor(a, r);
#pragma unroll
        for (int j = 0; j < TL::E; ++j) {
          const int m = (t + TL::T * j - r.out_shift) & (TL::M - 1);
          if (m < r.out_len) o[m] = v[j].x * g;
        }
      }
    }
  }
  ESTL_HD static void run(const ConvArgs& a, long long cta, int tid, cf32* sm) { run_mode<0>(a, cta, tid, sm); }
};

template <int LOGM, int LOGE, int LOGR, int LOGC, bool TC = false>
struct SpecSingleKernel : ConvSingleKernel<LOGM, LOGE, LOGR, LOGC, TC> {
  using B = ConvSingleKernel<LOGM, LOGE, LOGR, LOGC, TC>;
  ESTL_HD static void run(const ConvArgs& a, long long cta, int tid, cf32* sm) {
    B::template run_mode<1>(a, cta, tid, sm);
  }
};

// ---------------------------------------------------------------------------
// N <= 2^14, two real requests per complex transform (the real-input
// specialisation).  Rows 2i and 2i+1 of a launch share one N-point complex
// FFT: z = x1 + i s x2, Z = FFT(z), and with Zm_k = Z_{(N-k) mod N}
//   X1_k = (Z_k + conj(Zm_k)) / 2,      s X2_k = (Z_k - conj(Zm_k)) / (2i).
// Both outputs are real, so one inverse transform carries both:
//   IFFT(X1 H1 + i s X2 H2) = y1 + i s y2.
// FP32 rounding in both transforms is relative to the larger of the two
// halves, so the halves are balanced with exact powers of two: s = 2^k from
// the two signals' energies (k = half the difference of their binary
// exponents), and each filter spectrum is stored normalised, H / 2^e with
// 2^(2e) ~ sum h^2; e is kept in Im H_0, which is zero for a real filter.
// The spectrum kernel makes both normalised spectra from one transform of
// h1 2^-e1 + i h2 2^-e2 (scaled by 1/N, conjugated for correlation) and stores
// them in the two rows' spectrum slots.  With one filter for every request
// (ConvArgs::shared) the spectrum is the plain H of SpecSingleKernel and
// Y = Z H.  An unpaired last row runs with x2 = 0.  Zm comes from one extra
// shared-memory exchange; the energies from a row reduction.
// ---------------------------------------------------------------------------

// Sums of (x, y) over the T consecutive threads of each row of the CTA; every
// thread gets its row's sums.  buf: shared scratch of 2 * NT floats (free).
template <int T, int NT>
ESTL_HD void row_sum2(float& x, float& y, int tid, float* buf) {
#if defined(__CUDA_ARCH__)
  constexpr int W = T < 32 ? T : 32;
#pragma unroll
  for (int o = 1; o < W; o <<= 1) {
    x += __shfl_xor_sync(0xffffffffu, x, o);
    y += __shfl_xor_sync(0xffffffffu, y, o);
  }
  if constexpr (T > 32) {
    const int warp = tid >> 5;
    if ((tid & 31) == 0) {
      buf[2 * warp] = x;
      buf[2 * warp + 1] = y;
    }
    __syncthreads();
    const int w0 = (tid / T) * (T / 32);
    x = 0.f;
    y = 0.f;
    for (int w = 0; w < T / 32; ++w) {
      x += buf[2 * (w0 + w)];
      y += buf[2 * (w0 + w) + 1];
    }
    __syncthreads();
  }
#else
  buf[2 * tid] = x;
  buf[2 * tid + 1] = y;
  ESTL_SYNC();
  const int r0 = (tid / T) * T;
  x = 0.f;
  y = 0.f;
  for (int i = 0; i < T; ++i) {
    x += buf[2 * (r0 + i)];
    y += buf[2 * (r0 + i) + 1];
  }
  ESTL_SYNC();
#endif
}

ESTL_HD int ilogb_f(float v) {
#if defined(__CUDA_ARCH__)
  return ilogbf(v);
#else
  return std::ilogb(v);
#endif
}
ESTL_HD float pow2_f(int k) {
#if defined(__CUDA_ARCH__)
  return ldexpf(1.f, k);
#else
  return std::ldexp(1.f, k);
#endif
}
// k with 2^k ~ sqrt(e1 / e2) (0 when either energy is zero), |k| <= 60
ESTL_HD int balance_exp(float e1, float e2) {
  if (!(e1 > 0.f) || !(e2 > 0.f)) return 0;
  int k = (ilogb_f(e1) - ilogb_f(e2)) / 2;
  return k > 60 ? 60 : (k < -60 ? -60 : k);
}
// e with 2^(2e) ~ energy (0 for a zero filter), |e| <= 60
ESTL_HD int norm_exp(float energy) {
  if (!(energy > 0.f)) return 0;
  int e = ilogb_f(energy) / 2;
  return e > 60 ? 60 : (e < -60 ? -60 : e);
}

template <int LOGM, int LOGE, int LOGR, int LOGC, bool TC = false>
struct ConvPairKernel : ConvSingleKernel<LOGM, LOGE, LOGR, LOGC, TC> {
  using B = ConvSingleKernel<LOGM, LOGE, LOGR, LOGC, TC>;
  using TL = typename B::TL;
  using Sidx = typename B::Sidx;
  static constexpr int C = B::C;
  // the mirror exchange needs the buffer even for single-pass tiles
  static constexpr int EXCH = C * B::CS;
  static constexpr int TC_OFF = (EXCH + 1) & ~1;
  static constexpr int SMEM_ELEMS = TC ? TC_OFF + (int)((tc_area_words(B::NT / 32) + 1) / 2) : EXCH;
  static_assert(EXCH >= B::NT, "row reduction scratch");
  // the mirror values double the live registers: allow 128 per thread
  static constexpr int MINB = B::NT <= 128 ? 4 : (B::NT <= 256 ? 2 : 1);

  // MODE 0: convolution of rows (2i, 2i+1); MODE 1: spectra of filter rows (2i, 2i+1)
  template <int MODE>
  ESTL_HD static void run_mode(const ConvArgs& a, long long cta, int tid, cf32* smraw) {
    const int t = tid & (TL::T - 1);
    const int c = tid >> TL::LOGT;
    const long long ri = 2 * (cta * C + c);
    const bool valid = ri < a.nrows;
    const bool has2 = ri + 1 < a.nrows;
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, EXCH};
    const Sidx sidx{};
    if constexpr (TC) tc_init_atab(Ptr<uint32_t>{reinterpret_cast<uint32_t*>(smraw + TC_OFF), kTcAtabWords}, a.split, tid, B::NT);
    ConvRow r1{}, r2{};
    if (valid) r1 = a.rows[ri];
    if (has2) r2 = a.rows[ri + 1];
    cf32 v[TL::E];
    float e1 = 0.f, e2 = 0.f;
    {
      const Ptr<const float> s1 = valid ? a.sig.sub(r1.sig_off, r1.sig_len) : Ptr<const float>{a.sig.p, 0};
      const Ptr<const float> s2 = has2 ? a.sig.sub(r2.sig_off, r2.sig_len) : Ptr<const float>{a.sig.p, 0};
#pragma unroll
      for (int j = 0; j < TL::E; ++j) {
        const int pos = t + TL::T * j;
        v[j] = cf32{valid && pos < r1.sig_len ? s1[pos] : 0.f, has2 && pos < r2.sig_len ? s2[pos] : 0.f};
        e1 += v[j].x * v[j].x;
        e2 += v[j].y * v[j].y;
      }
    }
    row_sum2<TL::T, B::NT>(e1, e2, tid, reinterpret_cast<float*>(smraw));
    // MODE 0: x2 scaled by 2^k to the energy of x1; MODE 1: each filter normalised
    const int k = MODE == 0 ? balance_exp(e1, e2) : 0;
    const int f1 = MODE == 1 ? norm_exp(e1) : 0, f2 = MODE == 1 ? norm_exp(e2) : 0;
    {
      const float g1 = MODE == 1 ? pow2_f(-f1) : 1.f, g2 = MODE == 1 ? pow2_f(-f2) : pow2_f(k);
#pragma unroll
      for (int j = 0; j < TL::E; ++j) v[j] = cf32{v[j].x * g1, v[j].y * g2};
    }
    any_passes<TC, TL>(v, t, c, sm, tw, sidx, smraw + TC_OFF, a.split, tid);
    const bool mirror = MODE == 1 || !a.shared;  // uniform over the launch
    cf32 zm[TL::E];
    if (mirror) {
      ESTL_SYNC();  // the last pass's exchange reads are done
#pragma unroll
      for (int j = 0; j < TL::E; ++j) sm[sidx(c, t + TL::T * j)] = v[j];
      ESTL_SYNC();
#pragma unroll
      for (int j = 0; j < TL::E; ++j) zm[j] = sm[sidx(c, (TL::M - (t + TL::T * j)) & (TL::M - 1))];
      ESTL_SYNC();  // before the next passes reuse the exchange buffer
    }
    if constexpr (MODE == 1) {
      if (valid) {
        const Ptr<cf32> oa = a.spec_out.sub(r1.spec_off, TL::M);
        const Ptr<cf32> ob = has2 ? a.spec_out.sub(r2.spec_off, TL::M) : Ptr<cf32>{a.spec_out.p, 0};
        const float sc = 0.5f * r1.scale;
#pragma unroll
        for (int j = 0; j < TL::E; ++j) {
          const int pos = t + TL::T * j;
          // H1 = (Z + conj Zm) / 2, H2 = (Z - conj Zm) / (2i), each conjugated for correlation;
          // Im H_0 carries the normalisation exponent
          oa[pos] = cf32{sc * (v[j].x + zm[j].x), pos ? sc * (v[j].y - zm[j].y) * r1.conj : (float)f1};
          if (has2) ob[pos] = cf32{sc * (v[j].y + zm[j].y), pos ? -sc * (v[j].x - zm[j].x) * r1.conj : (float)f2};
        }
      }
    } else {
      float g1 = 1.f, g2 = 1.f;
      if (valid) {
        const Ptr<const cf32> h1 = a.spec.sub(r1.spec_off, TL::M);
        const float N = (float)(1 << a.logn);
        if (a.shared) {
          // one plain spectrum: Y = Z H, y2 carries 2^k
#pragma unroll
          for (int j = 0; j < TL::E; ++j) v[j] = cconj(cmul(v[j], ldg(h1, t + TL::T * j)));
          const float dc = ldg(h1, 0).x;
          g1 = r1.dc_norm ? 1.f / (N * dc) : 1.f;
          g2 = (r2.dc_norm ? 1.f / (N * dc) : 1.f) * pow2_f(-k);
        } else {
          const Ptr<const cf32> h2 = has2 ? a.spec.sub(r2.spec_off, TL::M) : h1;
          const cf32 d1 = ldg(h1, 0), d2 = ldg(h2, 0);  // (DC / 2^e, e)
#pragma unroll
          for (int j = 0; j < TL::E; ++j) {
            const int pos = t + TL::T * j;
            cf32 a1 = ldg(h1, pos), a2 = ldg(h2, pos);
            if (pos == 0) {
              a1.y = 0.f;
              a2.y = 0.f;
            }
            const cf32 x1{0.5f * (v[j].x + zm[j].x), 0.5f * (v[j].y - zm[j].y)};
            const cf32 x2{0.5f * (v[j].y + zm[j].y), -0.5f * (v[j].x - zm[j].x)};  // s X2
            const cf32 q = cmul(x2, a2);
            const cf32 y = cadd(cmul(x1, a1), cf32{-q.y, q.x});  // X1 H1 + i s X2 H2
            v[j] = cconj(y);
          }
          // the reference DC normalisation cancels the stored 2^-e
          g1 = r1.dc_norm ? 1.f / (N * d1.x) : pow2_f((int)d1.y);
          g2 = (r2.dc_norm ? 1.f / (N * d2.x) : pow2_f((int)d2.y)) * pow2_f(-k);
        }
      } else {
#pragma unroll
        for (int j = 0; j < TL::E; ++j) v[j] = cf32{0.f, 0.f};
      }
      any_passes<TC, TL>(v, t, c, sm, tw, sidx, smraw + TC_OFF, a.split, tid);
      // FFT(conj(Y)) = conj(y1 + i s y2): y1 = re, s y2 = -im
      if (valid) {
        const Ptr<float> o1 = a.out.sub(r1.out_off, r1.out_len);
#pragma unroll
        for (int j = 0; j < TL::E; ++j) {
          const int m = (t + TL::T * j - r1.out_shift) & (TL::M - 1);
          if (m < r1.out_len) o1[m] = v[j].x * g1;
        }
      }
      if (has2) {
        const Ptr<float> o2 = a.out.sub(r2.out_off, r2.out_len);
#pragma unroll
        for (int j = 0; j < TL::E; ++j) {
          const int m = (t + TL::T * j - r2.out_shift) & (TL::M - 1);
          if (m < r2.out_len) o2[m] = -v[j].y * g2;
        }
      }
    }
  }
  ESTL_HD static void run(const ConvArgs& a, long long cta, int tid, cf32* sm) { run_mode<0>(a, cta, tid, sm); }
};

template <int LOGM, int LOGE, int LOGR, int LOGC, bool TC = false>
struct SpecPairKernel : ConvPairKernel<LOGM, LOGE, LOGR, LOGC, TC> {
  using P = ConvPairKernel<LOGM, LOGE, LOGR, LOGC, TC>;
  ESTL_HD static void run(const ConvArgs& a, long long cta, int tid, cf32* sm) { P::template run_mode<1>(a, cta, tid, sm); }
};

// ---------------------------------------------------------------------------
// N > 2^14: four-step, N = N1 * N2, x[n1 + N1 n2]
// ---------------------------------------------------------------------------
// A: column pass over the zero-padded real input of row f: C adjacent
// columns n1, N2-point DFTs, times w_N^{n1 k2}, to s1[f*N + k2*N1 + n1].
// HALF: the real-input form (below): the input is the N'-point complex
// sequence z_m = x_{2m} + i x_{2m+1} and a.logn = log2 N'.
template <int LOGM, int LOGE, int LOGR, int LOGC, bool TC = false, bool HALF = false>
struct ConvColKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  static constexpr int EXCH = (TL::P > 1) ? TL::MP * C : 0;
  static constexpr int TC_OFF = (EXCH + 1) & ~1;
  static constexpr int SMEM_ELEMS = TC ? TC_OFF + (int)((tc_area_words(NT / 32) + 1) / 2) : EXCH;
  static_assert(NT <= 1024, "too many threads");
  static_assert(!TC || NT % 32 == 0, "tensor-core tiles run whole warps");
  static constexpr int MINB = TC ? (NT <= 256 ? 2 : 1) : min_blocks(NT, TL::E);
  struct Sidx {
    ESTL_HD int operator()(int c, int m) const { return TL::pad(m) * C + c; }
  };
  ESTL_HD static void run(const ConvArgs& a, long long cta, int tid, cf32* smraw) {
    const int c = tid & (C - 1);
    const int t = tid >> LOGC;
    const int logn1 = a.logn - LOGM;
    const int N = 1 << a.logn, N1 = 1 << logn1;
    const int nblk = N1 >> LOGC;
    const long long f = cta / nblk;
    const int n1 = (int)(cta - f * nblk) * C + c;
    const ConvRow r = a.rows[f];
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, EXCH};
    if constexpr (TC) tc_init_atab(Ptr<uint32_t>{reinterpret_cast<uint32_t*>(smraw + TC_OFF), kTcAtabWords}, a.split, tid, NT);
    const Ptr<const float> s = a.sig.sub(r.sig_off, r.sig_len);
    cf32 v[TL::E];
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const int n = n1 + ((t + TL::T * j) << logn1);
      if constexpr (HALF)
        v[j] = cf32{2 * n < r.sig_len ? s[2 * n] : 0.f, 2 * n + 1 < r.sig_len ? s[2 * n + 1] : 0.f};
      else
        v[j] = cf32{n < r.sig_len ? s[n] : 0.f, 0.f};
    }
    any_passes<TC, TL>(v, t, c, sm, tw, Sidx{}, smraw + TC_OFF, a.split, tid);
    const Ptr<cf32> o = a.s1.sub(f * N, N);
    fourstep_twiddle<TL>(v, n1, t, a.logn, a.bank);  // times w_N^{n1 k2}, k2 = t + T j
#pragma unroll
    for (int j = 0; j < TL::E; ++j) o[((t + TL::T * j) << logn1) + n1] = v[j];
  }
};

// B (spectrum): row pass of the filter: row k2 of s1 -> N1-point DFT ->
// Hp[k2*N1 + k1] = scale * H[k2 + N2 k1] (conjugated for correlation), stored
// unit-stride in the permuted order the convolution kernels read.
template <int LOGM, int LOGE, int LOGR, int LOGC, bool TC = false>
struct SpecRowKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  static constexpr int CS = row_stride(TL::MP, TL::T >= 16 ? 16 : TL::T * C >= 16 ? 16 / TL::T : C);
  static constexpr int EXCH = (TL::P > 1) ? C * CS : 0;
  static constexpr int TC_OFF = (EXCH + 1) & ~1;  // 16-byte aligned tensor-core area
  static constexpr int SMEM_ELEMS = TC ? TC_OFF + (int)((tc_area_words(NT / 32) + 1) / 2) : EXCH;
  static_assert(NT <= 1024, "too many threads");
  static_assert(!TC || NT % 32 == 0, "tensor-core tiles run whole warps");
  static constexpr int MINB = TC ? (NT <= 256 ? 2 : 1) : min_blocks(NT, TL::E);
  struct Sidx {
    ESTL_HD int operator()(int c, int m) const { return c * CS + TL::pad(m); }
  };
  ESTL_HD static void run(const ConvArgs& a, long long cta, int tid, cf32* smraw) {
    const int t = tid & (TL::T - 1);
    const int c = tid >> TL::LOGT;
    const int N = 1 << a.logn;
    const int logn2 = a.logn - LOGM;
    const int nblk = 1 << (logn2 - LOGC);
    const long long f = cta / nblk;
    const int k2 = (int)(cta - f * nblk) * C + c;
    const ConvRow r = a.rows[f];
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, EXCH};
    if constexpr (TC) tc_init_atab(Ptr<uint32_t>{reinterpret_cast<uint32_t*>(smraw + TC_OFF), kTcAtabWords}, a.split, tid, NT);
    const Ptr<cf32> s1 = a.s1.sub(f * N + (long long)k2 * TL::M, TL::M);
    cf32 v[TL::E];
#pragma unroll
    for (int j = 0; j < TL::E; ++j) v[j] = s1[t + TL::T * j];
    any_passes<TC, TL>(v, t, c, sm, tw, Sidx{}, smraw + TC_OFF, a.split, tid);
    const Ptr<cf32> o = a.spec_out.sub(r.spec_off + (long long)k2 * TL::M, TL::M);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) o[t + TL::T * j] = cf32{v[j].x * r.scale, v[j].y * r.scale * r.conj};
  }
};

// B (convolution): row k2 of s1 -> N1-point DFT (X[k2 + N2 k1]) -> times
// Hp -> conj -> N1-point DFT over k1 (V[k2][n1]) -> times w_N^{k2 n1} ->
// s2[f*N + n1*N2 + k2], stored through shared memory in runs of C rows.
template <int LOGM, int LOGE, int LOGR, int LOGC, bool TC = false>
struct ConvMidKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  using XR = XposeRows<TL::T, C, TL::MP>;  // row-major passes, column-fastest stores
  static constexpr int EXCH = XR::ELEMS;
  static constexpr int TC_OFF = (EXCH + 1) & ~1;
  static constexpr int SMEM_ELEMS = TC ? TC_OFF + (int)((tc_area_words(NT / 32) + 1) / 2) : EXCH;
  static_assert(NT <= 1024, "too many threads");
  static_assert(!TC || NT % 32 == 0, "tensor-core tiles run whole warps");
  // two DFTs, the spectrum multiply and the twiddle epilogue: allow 128 registers
  static constexpr int MINB = 1;
  struct Sidx {
    ESTL_HD int operator()(int c, int m) const { return XR::row(c) + TL::pad(m); }
  };
  ESTL_HD static void run(const ConvArgs& a, long long cta, int tid, cf32* smraw) {
    const int t = tid & (TL::T - 1);
    const int c = tid >> TL::LOGT;
    const int N = 1 << a.logn;
    const int logn2 = a.logn - LOGM;
    const int nblk = 1 << (logn2 - LOGC);
    const long long f = cta / nblk;
    const int k2_0 = (int)(cta - f * nblk) * C;
    const int k2 = k2_0 + c;
    const ConvRow r = a.rows[f];
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, EXCH};
    if constexpr (TC) tc_init_atab(Ptr<uint32_t>{reinterpret_cast<uint32_t*>(smraw + TC_OFF), kTcAtabWords}, a.split, tid, NT);
    const Sidx sidx{};
    const Ptr<cf32> s1 = a.s1.sub(f * N + (long long)k2 * TL::M, TL::M);
    cf32 v[TL::E];
#pragma unroll
    for (int j = 0; j < TL::E; ++j) v[j] = s1[t + TL::T * j];
    any_passes<TC, TL>(v, t, c, sm, tw, sidx, smraw + TC_OFF, a.split, tid);
    const Ptr<const cf32> h = a.spec.sub(r.spec_off + (long long)k2 * TL::M, TL::M);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) v[j] = cconj(cmul(v[j], ldg(h, t + TL::T * j)));
    any_passes<TC, TL>(v, t, c, sm, tw, sidx, smraw + TC_OFF, a.split, tid);
    fourstep_twiddle<TL>(v, k2, t, a.logn, a.bank);  // times w_N^{k2 n1}, n1 = t + T j
#pragma unroll
    for (int j = 0; j < TL::E; ++j) sm[sidx(c, t + TL::T * j)] = v[j];
    ESTL_SYNC();
    const int c2 = tid & (C - 1);
    const int t2 = tid >> LOGC;
    const Ptr<cf32> o = a.s2.sub(f * N, N);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const int n1 = t2 + TL::T * j;
      o[(n1 << logn2) + k2_0 + c2] = sm[sidx(c2, n1)];
    }
  }
};

// C: row n1 of s2 (N2 contiguous values over k2) -> N2-point DFT over k2 ->
// conj(result)[n1 + N1 n2] -> real part, staged through shared memory and
// stored in runs of C columns, cropped to [out_shift, out_shift + out_len).
template <int LOGM, int LOGE, int LOGR, int LOGC, bool TC = false>
struct ConvOutKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  using XR = XposeRows<TL::T, C, TL::MP>;  // row-major passes, column-fastest stores
  static constexpr int EXCH = XR::ELEMS;
  static constexpr int TC_OFF = (EXCH + 1) & ~1;
  static constexpr int SMEM_ELEMS = TC ? TC_OFF + (int)((tc_area_words(NT / 32) + 1) / 2) : EXCH;
  static_assert(NT <= 1024, "too many threads");
  static_assert(!TC || NT % 32 == 0, "tensor-core tiles run whole warps");
  static constexpr int MINB = TC ? (NT <= 256 ? 2 : 1) : min_blocks(NT, TL::E);
  struct Sidx {
    ESTL_HD int operator()(int c, int m) const { return XR::row(c) + TL::pad(m); }
  };
  ESTL_HD static void run(const ConvArgs& a, long long cta, int tid, cf32* smraw) {
    const int t = tid & (TL::T - 1);
    const int c = tid >> TL::LOGT;
    const int N = 1 << a.logn;
    const int logn1 = a.logn - LOGM;
    const int nblk = 1 << (logn1 - LOGC);
    const long long f = cta / nblk;
    const int n1_0 = (int)(cta - f * nblk) * C;
    const ConvRow r = a.rows[f];
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, EXCH};
    if constexpr (TC) tc_init_atab(Ptr<uint32_t>{reinterpret_cast<uint32_t*>(smraw + TC_OFF), kTcAtabWords}, a.split, tid, NT);
    const Sidx sidx{};
    const Ptr<cf32> s2 = a.s2.sub(f * N + (long long)(n1_0 + c) * TL::M, TL::M);
    cf32 v[TL::E];
#pragma unroll
    for (int j = 0; j < TL::E; ++j) v[j] = s2[t + TL::T * j];
    any_passes<TC, TL>(v, t, c, sm, tw, sidx, smraw + TC_OFF, a.split, tid);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) sm[sidx(c, t + TL::T * j)] = v[j];
    ESTL_SYNC();
    const int c2 = tid & (C - 1);
    const int t2 = tid >> LOGC;
    const Ptr<float> o = a.out.sub(r.out_off, r.out_len);
    const float g = dc_factor(a, r);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const int n2 = t2 + TL::T * j;
      const int m = (n1_0 + c2 + (n2 << logn1) - r.out_shift) & ((1 << a.logn) - 1);
      const float val = sm[sidx(c2, n2)].x;
      if (m < r.out_len) o[m] = val * g;
    }
  }
};

// ---------------------------------------------------------------------------
// N > 2^14, real input (the real-input specialisation of the four-step path,
// after Convolution.h:106-120,146-148: real data in, real output).  A real
// request x of padded length N is transformed as the N' = N/2-point complex
// sequence z_m = x_{2m} + i x_{2m+1} (ConvColKernel<..., HALF>), so every
// pass moves half the bytes of the complex path.  With Z = FFT_N'(z) and
// Zm_k = conj(Z_{(N'-k) mod N'}):
//   E_k = (Z_k + Zm_k) / 2,  O_k = (Z_k - Zm_k) / (2i),
//   X_k = E_k + w_N^k O_k,   X_{N'-k} = conj(E_k - w_N^k O_k),
// the spectrum of x for k in [0, N'] (X_{N'} from k = 0).  The product
// Y = X H is Hermitian, and the real inverse is again a half-length complex
// transform: v = IFFT_N'(V) with
//   V_k = (Y_k + conj(Y_{N'-k})) + i conj(w_N^k) (Y_k - conj(Y_{N'-k})),
// y_{2m} = Re v_m, y_{2m+1} = Im v_m.
//
// In the four-step layout N' = N1 * N2 the row pass holds row k2 (all k1 of
// k = k2 + N2 k1), and the mirror N' - k lies in row (N2 - k2) mod N2 at k1'
// = N1 - 1 - k1 (row 0: k1' = (N1 - k1) mod N1).  A CTA of C rows therefore
// takes C/2 rows k2 = b C/2 + r and their mirror rows N2 - k2; row 0 and row
// N2/2 are their own mirrors and share CTA 0.  One shared-memory exchange
// brings each element's mirror into the thread.  The filter spectrum is kept
// for k < N' in the permuted order Hp[k2 N1 + k1] = H_k, with H_{N'} (real)
// in slot N'.
// ---------------------------------------------------------------------------

// Row k2 held by row c of CTA b (C = 2h rows per CTA) and the row of the CTA
// holding its mirror.
struct MirrorRows {
  int k2, partner;
};
ESTL_HD MirrorRows mirror_rows(int b, int c, int h, int n2) {
  const int r = c < h ? c : c - h;
  const int base = b * h + r;  // in [0, N2/2)
  if (c < h) return {base, base == 0 ? c : c + h};
  return {base == 0 ? n2 / 2 : n2 - base, base == 0 ? c : c - h};
}

// Position k1' of the mirror of (k2, k1) in its row.
ESTL_HD int mirror_k1(int k2, int k1, int n1) { return k2 == 0 ? (n1 - k1) & (n1 - 1) : n1 - 1 - k1; }

// E and O of X_k = E + w O from Z_k and the mirror Z_{N'-k}.
ESTL_HD void real_split(cf32 z, cf32 zmirror, cf32& e, cf32& o) {
  const cf32 zc = cconj(zmirror);
  e = cf32{0.5f * (z.x + zc.x), 0.5f * (z.y + zc.y)};
  const cf32 d = cf32{0.5f * (z.x - zc.x), 0.5f * (z.y - zc.y)};
  o = cf32{d.y, -d.x};  // d / i
}

// B (spectrum, real input): row DFTs of the filter's half-length transform,
// then H_k (and H_{N'}) from each element and its mirror, scaled by
// 1/N (conjugated for correlation), stored in the permuted order.
template <int LOGM, int LOGE, int LOGR, int LOGC>
struct SpecRowHalfKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  static constexpr int CS = row_stride(TL::MP, TL::T >= 16 ? 16 : TL::T * C >= 16 ? 16 / TL::T : C);
  static constexpr int EXCH = C * CS;
  static constexpr int SMEM_ELEMS = EXCH;
  static_assert(NT <= 1024, "too many threads");
  static_assert(C >= 2, "rows come in mirror pairs");
  static constexpr int MINB = min_blocks(NT, TL::E);
  struct Sidx {
    ESTL_HD int operator()(int c, int m) const { return c * CS + TL::pad(m); }
  };
  ESTL_HD static void run(const ConvArgs& a, long long cta, int tid, cf32* smraw) {
    const int t = tid & (TL::T - 1);
    const int c = tid >> TL::LOGT;
    const int NH = 1 << a.logn;  // N'
    const int logn2 = a.logn - LOGM, n2 = 1 << logn2;
    const int nblk = n2 >> LOGC;
    const long long f = cta / nblk;
    const int b = (int)(cta - f * nblk);
    const MirrorRows mr = mirror_rows(b, c, C / 2, n2);
    const ConvRow r = a.rows[f];
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, EXCH};
    const Sidx sidx{};
    const Ptr<cf32> s1 = a.s1.sub(f * NH + (long long)mr.k2 * TL::M, TL::M);
    cf32 v[TL::E];
#pragma unroll
    for (int j = 0; j < TL::E; ++j) v[j] = s1[t + TL::T * j];
    run_passes<TL, 0>(v, t, c, sm, tw, sidx);
    if constexpr (TL::P == 1) ESTL_SYNC();
#pragma unroll
    for (int j = 0; j < TL::E; ++j) sm[sidx(c, t + TL::T * j)] = v[j];
    ESTL_SYNC();
    const Ptr<cf32> o = a.spec_out.sub(r.spec_off, NH + 2);
    static_assert(TL::E == 16, "split twiddle powers for 16 slots");
    const SplitTwiddles stw = split_twiddles(a.bank, a.logn + 1, mr.k2, t, logn2, TL::T);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const int k1 = t + TL::T * j;
      const cf32 zm = sm[sidx(mr.partner, mirror_k1(mr.k2, k1, TL::M))];
      cf32 e, od;
      real_split(v[j], zm, e, od);
      const cf32 w = stw(j);  // w_N^{k2 + N2 k1}
      const cf32 wo = cmul(w, od);
      const cf32 h = cadd(e, wo);
      o[mr.k2 * TL::M + k1] = cf32{h.x * r.scale, h.y * r.scale * r.conj};
      if (mr.k2 == 0 && k1 == 0) {
        const cf32 hn = cconj(csub(e, wo));  // H_{N'} (real)
        o[NH] = cf32{hn.x * r.scale, hn.y * r.scale * r.conj};
      }
    }
  }
};

// B (convolution, real input): row DFT (Z), the spectrum of x from Z and
// its mirror, times H, the half-length inverse's input V, conj, row DFT over
// k1, times w_N'^{k2 n1}, stored to s2[f*N' + n1*N2 + k2] through shared
// memory.
template <int LOGM, int LOGE, int LOGR, int LOGC>
struct ConvMidHalfKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  using XR = XposeRows<TL::T, C, TL::MP>;  // row-major passes, column-fastest stores
  static constexpr int EXCH = XR::ELEMS;
  static constexpr int SMEM_ELEMS = EXCH;
  static_assert(NT <= 1024, "too many threads");
  static_assert(C >= 2, "rows come in mirror pairs");
  static constexpr int MINB = 1;  // two DFTs, the spectrum algebra and the twiddle epilogue
  struct Sidx {
    ESTL_HD int operator()(int c, int m) const { return XR::row(c) + TL::pad(m); }
  };
  ESTL_HD static void run(const ConvArgs& a, long long cta, int tid, cf32* smraw) {
    const int t = tid & (TL::T - 1);
    const int c = tid >> TL::LOGT;
    const int NH = 1 << a.logn;
    const int logn2 = a.logn - LOGM, n2 = 1 << logn2;
    const int nblk = n2 >> LOGC;
    const long long f = cta / nblk;
    const int b = (int)(cta - f * nblk);
    const MirrorRows mr = mirror_rows(b, c, C / 2, n2);
    const int k2p = mirror_rows(b, mr.partner, C / 2, n2).k2;
    const ConvRow r = a.rows[f];
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, EXCH};
    const Sidx sidx{};
    const Ptr<cf32> s1 = a.s1.sub(f * NH + (long long)mr.k2 * TL::M, TL::M);
    cf32 v[TL::E];
#pragma unroll
    for (int j = 0; j < TL::E; ++j) v[j] = s1[t + TL::T * j];
    run_passes<TL, 0>(v, t, c, sm, tw, sidx);
    if constexpr (TL::P == 1) ESTL_SYNC();
#pragma unroll
    for (int j = 0; j < TL::E; ++j) sm[sidx(c, t + TL::T * j)] = v[j];
    ESTL_SYNC();
    cf32 zm[TL::E];
#pragma unroll
    for (int j = 0; j < TL::E; ++j) zm[j] = sm[sidx(mr.partner, mirror_k1(mr.k2, t + TL::T * j, TL::M))];
    ESTL_SYNC();  // the buffer is the next passes' exchange space
    const Ptr<const cf32> h = a.spec.sub(r.spec_off, NH + 2);
    static_assert(TL::E == 16, "split twiddle powers for 16 slots");
    const SplitTwiddles stw = split_twiddles(a.bank, a.logn + 1, mr.k2, t, logn2, TL::T);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const int k1 = t + TL::T * j;
      const int k1p = mirror_k1(mr.k2, k1, TL::M);
      cf32 e, od;
      real_split(v[j], zm[j], e, od);
      const cf32 w = stw(j);  // w_N^{k2 + N2 k1}
      const cf32 wo = cmul(w, od);
      const cf32 xk = cadd(e, wo), xm = cconj(csub(e, wo));
      const cf32 hk = ldg(h, mr.k2 * TL::M + k1);
      const cf32 hm = (mr.k2 == 0 && k1 == 0) ? ldg(h, NH) : ldg(h, k2p * TL::M + k1p);
      const cf32 yk = cmul(xk, hk), ymc = cconj(cmul(xm, hm));
      const cf32 sum = cadd(yk, ymc), dif = csub(yk, ymc);
      const cf32 id = cmul(cconj(w), cf32{-dif.y, dif.x});  // i conj(w) (Yk - conj(Ym))
      v[j] = cconj(cadd(sum, id));
    }
    run_passes<TL, 0>(v, t, c, sm, tw, sidx);
    if constexpr (TL::P == 1) ESTL_SYNC();
    fourstep_twiddle<TL>(v, mr.k2, t, a.logn, a.bank);  // times w_N'^{k2 n1}, n1 = t + T j
#pragma unroll
    for (int j = 0; j < TL::E; ++j) sm[sidx(c, t + TL::T * j)] = v[j];
    ESTL_SYNC();
    const int c2 = tid & (C - 1);
    const int t2 = tid >> LOGC;
    const int k2o = mirror_rows(b, c2, C / 2, n2).k2;
    const Ptr<cf32> o = a.s2.sub(f * NH, NH);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const int n1 = t2 + TL::T * j;
      o[(n1 << logn2) + k2o] = sm[sidx(c2, n1)];
    }
  }
};

// C (real input): as ConvOutKernel over the half-length transform; the
// complex result v_m carries two real outputs, y_{2m} = Re v_m and
// y_{2m+1} = Im v_m.
template <int LOGM, int LOGE, int LOGR, int LOGC>
struct ConvOutHalfKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  using XR = XposeRows<TL::T, C, TL::MP>;  // row-major passes, column-fastest stores
  static constexpr int EXCH = XR::ELEMS;
  static constexpr int SMEM_ELEMS = EXCH;
  static_assert(NT <= 1024, "too many threads");
  static constexpr int MINB = min_blocks(NT, TL::E);
  struct Sidx {
    ESTL_HD int operator()(int c, int m) const { return XR::row(c) + TL::pad(m); }
  };
  ESTL_HD static void run(const ConvArgs& a, long long cta, int tid, cf32* smraw) {
    const int t = tid & (TL::T - 1);
    const int c = tid >> TL::LOGT;
    const int NH = 1 << a.logn;
    const int logn1 = a.logn - LOGM;
    const int nblk = 1 << (logn1 - LOGC);
    const long long f = cta / nblk;
    const int n1_0 = (int)(cta - f * nblk) * C;
    const ConvRow r = a.rows[f];
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, EXCH};
    const Sidx sidx{};
    const Ptr<cf32> s2 = a.s2.sub(f * NH + (long long)(n1_0 + c) * TL::M, TL::M);
    cf32 v[TL::E];
#pragma unroll
    for (int j = 0; j < TL::E; ++j) v[j] = s2[t + TL::T * j];
    run_passes<TL, 0>(v, t, c, sm, tw, sidx);
    if constexpr (TL::P == 1) ESTL_SYNC();
#pragma unroll
    for (int j = 0; j < TL::E; ++j) sm[sidx(c, t + TL::T * j)] = v[j];
    ESTL_SYNC();
    const int c2 = tid & (C - 1);
    const int t2 = tid >> LOGC;
    const Ptr<float> o = a.out.sub(r.out_off, r.out_len);
    // the reference's 1/K^[0] normalisation: 1 / (N * stored DC), N = 2 N'
    const float g = r.dc_norm ? 1.f / ((float)(2 * NH) * ldg(a.spec, r.spec_off).x) : 1.f;
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const int n2 = t2 + TL::T * j;
      const cf32 val = sm[sidx(c2, n2)];  // conj(v_m)
      const int pos = 2 * (n1_0 + c2 + (n2 << logn1));
      const int m0 = (pos - r.out_shift) & (2 * NH - 1), m1 = (pos + 1 - r.out_shift) & (2 * NH - 1);
      if (m0 < r.out_len) o[m0] = val.x * g;
      if (m1 < r.out_len) o[m1] = -val.y * g;
    }
  }
};

}  // namespace estl
