// tc_core.cuh — split-precision radix-16 stages on the tensor cores.
//
// The plain tile kernels run every radix-16 DFT of a Stockham pass as FP32
// register arithmetic (DFT<16> in fft_core.cuh; the reference's per-pass
// KomplexConstMultiplication network, KernelGenerator.h:100-142).  With a split
// precision the 32 butterflies a warp owns in a radix-16 pass become one GEMM:
//
//   [Yr; Yi] (32 x 32) = [[Fr, -Fi], [Fi, Fr]] (32 x 32) . [Xr; Xi] (32 x 32)
//
// F = the forward 16-point DFT matrix, X = the warp's twiddled butterfly inputs
// (one column per lane), run as 16 x 8 x 16 tensor-core products
// (mma.sync m16n8k16) with FP32 accumulation.  Both operands are split into a
// sum of 16-bit terms, x = x_0 + x_1 (+ x_2), x_q = round16(x - x_0 - .. - x_{q-1}),
// and the products with q_a + q_b < terms are accumulated:
//   SPLIT_FP16X2  fp16 hi + lo (22 significant bits); every butterfly is
//                 scaled by a power of two to max |x| < 1 before the split and
//                 back after the GEMM, so fp16's range is never the limit;
//   SPLIT_BF16X2  bf16 hi + lo (16 significant bits, ~1e-5 relative);
//   SPLIT_BF16X3  bf16 hi + mid + lo (24 significant bits, six products).
// Twiddles, radix-2/4/8 remainder passes and the four-step twiddle stay FP32.
//
// Data movement per radix-16 pass (per warp):
//   registers (FP32, twiddled) -> split terms, staged in shared memory as
//   [butterfly][k] 16-bit pairs (row stride 20 words: conflict-free for both
//   the 128-bit staging stores and the 32-bit fragment loads)
//   -> B fragments, A fragments from a per-CTA table of the split DFT matrix
//   -> mma -> each D fragment element Y[r][n] is written straight to the
//   Stockham exchange slot of output r of butterfly n, which another lane owns.
// The emulator (ESTL_EMU) computes the same D elements directly from the
// staged terms, so every shared-memory index of this file is bounds checked
// on the host; the fragment layouts (PTX ISA, mma.m16n8k16 for 16-bit types)
// are only exercised on the GPU.
//
// Included by fft_core.cuh between the tile machinery and the tile kernels.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#endif
#include <cmath>
#include <cstring>

#ifdef ESTL_EMU
#define ESTL_SYNCWARP() estl_emu_sync()
#else
#define ESTL_SYNCWARP() __syncwarp()
#endif

namespace estl {

enum SplitKind { SPLIT_NONE = 0, SPLIT_FP16X2 = 1, SPLIT_BF16X2 = 2, SPLIT_BF16X3 = 3 };
ESTL_CX int split_terms(int kind) { return kind == SPLIT_BF16X3 ? 3 : 2; }

// Shared-memory words of the tensor-core area: the split DFT matrix (three
// term tables of 32 rows x 20 words) and, per warp, three staging tables of
// the same shape plus 32 butterfly scale factors.
constexpr int kTcRowWords = 20;
constexpr int kTcTableWords = 32 * kTcRowWords;
constexpr int kTcAtabWords = 3 * kTcTableWords;
constexpr int kTcWarpWords = 3 * kTcTableWords + 32;
ESTL_CX long long tc_area_words(int nwarps) { return kTcAtabWords + (long long)nwarps * kTcWarpWords; }

// ---- 16-bit conversions (round to nearest even) ----------------------------
#if defined(__CUDA_ARCH__)
ESTL_HD uint32_t to16(float x, bool bf) {
  return bf ? (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(x)) : (uint32_t)__half_as_ushort(__float2half_rn(x));
}
ESTL_HD float from16(uint32_t h, bool bf) {
  return bf ? __bfloat162float(__ushort_as_bfloat16((unsigned short)h)) : __half2float(__ushort_as_half((unsigned short)h));
}
#else
inline uint32_t f32_bits(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return u;
}
inline float bits_f32(uint32_t u) {
  float x;
  std::memcpy(&x, &u, 4);
  return x;
}
// bfloat16: the upper 16 bits of the float, rounded to nearest even.
inline uint32_t to_bf16(float x) {
  uint32_t u = f32_bits(x);
  u += 0x7fffu + ((u >> 16) & 1u);
  return u >> 16;
}
// IEEE binary16 with subnormals, rounded to nearest even (finite inputs).
inline uint32_t to_f16(float x) {
  const uint32_t u = f32_bits(x);
  const uint32_t sign = (u >> 16) & 0x8000u;
  const float a = std::fabs(x);
  if (a >= 65520.f) return sign | 0x7c00u;  // rounds to infinity
  if (a < 6.103515625e-05f) {               // subnormal (or zero): multiples of 2^-24
    const float q = std::nearbyint(a * 16777216.f);  // round-half-even in the default mode
    return sign | (uint32_t)q;
  }
  const uint32_t au = f32_bits(a);
  uint32_t exp = ((au >> 23) & 0xff) - 127 + 15;
  uint32_t mant = au & 0x7fffffu;
  uint32_t h = (exp << 10) | (mant >> 13);
  const uint32_t rest = mant & 0x1fffu;
  if (rest > 0x1000u || (rest == 0x1000u && (h & 1u))) h += 1;  // carries into the exponent correctly
  return sign | h;
}
inline float from_f16(uint32_t h) {
  const uint32_t sign = (h & 0x8000u) << 16;
  const uint32_t e = (h >> 10) & 0x1f, m = h & 0x3ff;
  float v;
  if (e == 0)
    v = (float)m * 5.9604644775390625e-08f;  // m * 2^-24
  else if (e == 31)
    v = INFINITY;
  else
    v = bits_f32(((e - 15 + 127) << 23) | (m << 13));
  return bits_f32(f32_bits(v) | sign);
}
inline uint32_t to16(float x, bool bf) { return bf ? to_bf16(x) : to_f16(x); }
inline float from16(uint32_t h, bool bf) { return bf ? bits_f32(h << 16) : from_f16(h); }
#endif

// cos(2 pi m / 16), m = 0..15, exactly rounded FP32.
ESTL_HD float cos16(int m) {
  switch (m & 15) {
    case 0: return 1.f;
    case 1: case 15: return kC16;
    case 2: case 14: return kC8;
    case 3: case 13: return kS16;
    case 4: case 12: return 0.f;
    case 5: case 11: return -kS16;
    case 6: case 10: return -kC8;
    default: return -kC16;  // 7, 9
    case 8: return -1.f;
  }
}

// Real block form of the forward 16-point DFT: rows m < 16 give Re Y[m],
// rows m >= 16 give Im Y[m - 16]; columns k < 16 take Re x[k], k >= 16 Im x[k - 16].
//   Fr[r][s] = cos(2 pi r s / 16), Fi[r][s] = -sin(2 pi r s / 16) = -cos(2 pi (r s - 4) / 16).
ESTL_HD float dft16_real(int m, int k) {
  const int r = m & 15, s = k & 15;
  const float fr = cos16(r * s);
  const float fi = -cos16(r * s - 4);
  if (m < 16) return k < 16 ? fr : -fi;
  return k < 16 ? fi : fr;
}

// Fills the per-CTA table of the split DFT matrix: word (q, m, w) holds the
// term-q values of A[m][2w] (low half) and A[m][2w + 1] (high half).
ESTL_HD void tc_init_atab(const Ptr<uint32_t>& atab, int kind, int tid, int nt) {
  const bool bf = kind != SPLIT_FP16X2;
  const int terms = split_terms(kind);
  for (int i = tid; i < 32 * 16; i += nt) {
    const int m = i >> 4, w = i & 15;
    float r0 = dft16_real(m, 2 * w), r1 = dft16_real(m, 2 * w + 1);
    for (int q = 0; q < 3; ++q) {
      uint32_t h0 = 0, h1 = 0;
      if (q < terms) {
        h0 = to16(r0, bf);
        h1 = to16(r1, bf);
        r0 -= from16(h0, bf);
        r1 -= from16(h1, bf);
      }
      atab[q * kTcTableWords + m * kTcRowWords + w] = h0 | (h1 << 16);
    }
  }
}

// Per-warp view of the tensor-core area.
struct TcCtx {
  Ptr<uint32_t> atab;   // 3 term tables of the DFT matrix
  Ptr<uint32_t> stage;  // this warp's 3 staging tables
  Ptr<float> scale;     // this warp's 32 butterfly scale factors
  int kind;
  int lane;
  int tid0;  // thread index of lane 0 of this warp
};

ESTL_HD TcCtx tc_ctx(cf32* area, int kind, int tid) {
  uint32_t* w = reinterpret_cast<uint32_t*>(area);
  const int warp = tid >> 5;
  uint32_t* ws = w + kTcAtabWords + (long long)warp * kTcWarpWords;
  return TcCtx{Ptr<uint32_t>{w, kTcAtabWords}, Ptr<uint32_t>{ws, 3 * kTcTableWords},
               Ptr<float>{reinterpret_cast<float*>(ws + 3 * kTcTableWords), 32}, kind, tid & 31, tid & ~31};
}

// Lane `lane` stages its butterfly: the 32 real inputs (16 re, 16 im), scaled
// (fp16) and split into terms, as row `lane` of each staging table.
ESTL_HD void tc_stage(const cf32 (&x)[16], const TcCtx& ctx) {
  const bool bf = ctx.kind != SPLIT_FP16X2;
  const int terms = split_terms(ctx.kind);
  float s = 1.f;
  if (!bf) {
    float m = 0.f;
#pragma unroll
    for (int k = 0; k < 16; ++k) m = fmaxf(m, fmaxf(fabsf(x[k].x), fabsf(x[k].y)));
    int e = 0;
    if (m > 0.f) (void)frexpf(m, &e);  // m = f 2^e, 0.5 <= f < 1
    s = ldexpf(1.f, -e);
    ctx.scale[ctx.lane] = ldexpf(1.f, e);
  } else {
    ctx.scale[ctx.lane] = 1.f;
  }
#pragma unroll
  for (int w = 0; w < 16; ++w) {
    // word w holds k = 2w, 2w + 1: real parts for w < 8, imaginary parts after
    float r0 = (w < 8 ? x[2 * w].x : x[2 * w - 16].y) * s;
    float r1 = (w < 8 ? x[2 * w + 1].x : x[2 * w - 15].y) * s;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      if (q < terms) {
        const uint32_t h0 = to16(r0, bf), h1 = to16(r1, bf);
        r0 -= from16(h0, bf);
        r1 -= from16(h1, bf);
        ctx.stage[q * kTcTableWords + ctx.lane * kTcRowWords + w] = h0 | (h1 << 16);
      }
    }
  }
}

#if defined(__CUDA_ARCH__)
ESTL_HD void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1, bool bf) {
  if (bf)
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
  else
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
#endif

// The warp's 32 staged butterflies through the tensor cores; every output
// y_r of butterfly n (owned by lane n, thread tid0 + n) is written to the
// exchange slot sidx(c_n, out_pos<p>(t_n, r)), times the butterfly's scale.
// OWN(tid, t, c) gives a thread's (t, c) in the kernel's thread mapping.
template <class TL, int p, class SIDX, class OWN>
ESTL_HD void tc_dft16_scatter(const TcCtx& ctx, const Ptr<cf32>& sm, SIDX sidx, OWN own) {
  const bool bf = ctx.kind != SPLIT_FP16X2;
  const int terms = split_terms(ctx.kind);
  const int g = ctx.lane >> 2, tig = ctx.lane & 3;
#pragma unroll 1
  for (int nt = 0; nt < 4; ++nt) {
    float d[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#if defined(__CUDA_ARCH__)
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) {
      uint32_t b[3][2];
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        if (q < terms) {
          const int base = q * kTcTableWords + (8 * nt + g) * kTcRowWords + 8 * kt + tig;
          b[q][0] = ctx.stage[base];
          b[q][1] = ctx.stage[base + 4];
        }
      }
#pragma unroll
      for (int qa = 0; qa < 3; ++qa) {
        if (qa < terms) {
#pragma unroll
          for (int mt = 0; mt < 2; ++mt) {
            const int base = qa * kTcTableWords + (16 * mt + g) * kTcRowWords + 8 * kt + tig;
            const uint32_t a[4] = {ctx.atab[base], ctx.atab[base + 8 * kTcRowWords], ctx.atab[base + 4],
                                   ctx.atab[base + 8 * kTcRowWords + 4]};
#pragma unroll
            for (int qb = 0; qb < 3; ++qb)
              if (qa + qb < terms) mma16816(d[mt], a, b[qb][0], b[qb][1], bf);
          }
        }
      }
    }
#else
    // emulator: the same D elements from the staged terms
    for (int mt = 0; mt < 2; ++mt)
      for (int i = 0; i < 4; ++i) {
        const int m = 16 * mt + g + ((i & 2) ? 8 : 0);
        const int n = 8 * nt + 2 * tig + (i & 1);
        float acc = 0.f;
        for (int qa = 0; qa < terms; ++qa)
          for (int qb = 0; qa + qb < terms; ++qb)
            for (int k = 0; k < 32; ++k) {
              const uint32_t aw = ctx.atab[qa * kTcTableWords + m * kTcRowWords + (k >> 1)];
              const uint32_t bw = ctx.stage[qb * kTcTableWords + n * kTcRowWords + (k >> 1)];
              acc += from16((k & 1) ? aw >> 16 : aw & 0xffffu, bf) * from16((k & 1) ? bw >> 16 : bw & 0xffffu, bf);
            }
        d[mt][i] = acc;
      }
#endif
    // D element i of m-tile mt: row g (+8 for i >= 2), column 2 tig + (i & 1)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = g + ((i & 2) ? 8 : 0);
      const int n = 8 * nt + 2 * tig + (i & 1);
      const float s = ctx.scale[n];
      int tn, cn;
      own(ctx.tid0 + n, tn, cn);
      sm[sidx(cn, TL::template out_pos<p>(tn, r))] = cf32{d[0][i] * s, d[1][i] * s};
    }
  }
}

// run_passes with the radix-16 passes on the tensor cores (E = 16: one
// butterfly per thread).  Other passes are FP32 as in run_passes.  On exit
// v[j] holds position t + T*j of the transformed tile, as run_passes leaves it.
template <class TL, int p, class SIDX, class OWN>
ESTL_HD void run_passes_tc(cf32 (&v)[TL::E], int t, int c, const Ptr<cf32>& sm, const Ptr<const cf32>& tw,
                           SIDX sidx, OWN own, const TcCtx& ctx) {
  static_assert(TL::E == 16 && TL::LR_FULL == 4, "tensor-core passes need radix-16 tiles of 16 elements per thread");
  if constexpr (p < TL::P) {
    constexpr bool last = p + 1 == TL::P;
    if constexpr (TL::lr(p) == 4) {
      TL::template twiddle_only<p>(v, t, tw);
      tc_stage(v, ctx);
      ESTL_SYNCWARP();
      tc_dft16_scatter<TL, p>(ctx, sm, sidx, own);
      ESTL_SYNC();
#pragma unroll
      for (int j = 0; j < TL::E; ++j) v[j] = sm[sidx(c, t + TL::T * j)];
      if constexpr (!last) ESTL_SYNC();
    } else {
      TL::template compute<p>(v, t, tw);
      if constexpr (!last) {
#pragma unroll
        for (int j = 0; j < TL::E; ++j) sm[sidx(c, TL::template out_pos<p>(t, j))] = v[j];
        ESTL_SYNC();
#pragma unroll
        for (int j = 0; j < TL::E; ++j) v[j] = sm[sidx(c, t + TL::T * j)];
        ESTL_SYNC();
      }
    }
    run_passes_tc<TL, p + 1>(v, t, c, sm, tw, sidx, own, ctx);
  }
}

}  // namespace estl
