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
//   -> mma -> D staged as [butterfly][output] (18-element rows) -> each lane
//   reads back its own butterfly's 16 outputs and continues exactly like the
//   FP32 path after DFT<16> (Stockham exchange, next pass).
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
// the same shape (B operand terms; the first two then hold D).
constexpr int kTcRowWords = 20;
constexpr int kTcTableWords = 32 * kTcRowWords;
constexpr int kTcAtabWords = 3 * kTcTableWords;
constexpr int kTcWarpWords = 3 * kTcTableWords;
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
  Ptr<uint32_t> stage;  // this warp's staging words (B terms, then D)
  int kind;
  int lane;
};

ESTL_HD TcCtx tc_ctx(cf32* area, int kind, int tid) {
  uint32_t* w = reinterpret_cast<uint32_t*>(area);
  const int warp = tid >> 5;
  uint32_t* ws = w + kTcAtabWords + (long long)warp * kTcWarpWords;
  return TcCtx{Ptr<uint32_t>{w, kTcAtabWords}, Ptr<uint32_t>{ws, kTcWarpWords}, kind, tid & 31};
}

ESTL_HD uint32_t f32_bits_hd(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return u;
#endif
}
ESTL_HD float bits_f32_hd(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  std::memcpy(&x, &u, 4);
  return x;
#endif
}

#if defined(__CUDA_ARCH__)
// ldmatrix .x4: four 8 x 8 16-bit matrices; lane L supplies the address of
// row L & 7 of matrix L >> 3; register i receives matrix i, row lane / 4,
// elements 2 (lane % 4) and 2 (lane % 4) + 1.
ESTL_HD void ldmatrix_x4(uint32_t (&r)[4], const uint32_t* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}
#endif

// Two floats -> one word of two 16-bit values (a in the low half).
template <bool BF>
ESTL_HD uint32_t pack16(float a, float b) {
#if defined(__CUDA_ARCH__)
  if constexpr (BF) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
  } else {
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
  }
#else
  return to16(a, BF) | (to16(b, BF) << 16);
#endif
}
template <bool BF>
ESTL_HD void unpack16(uint32_t w, float& a, float& b) {
#if defined(__CUDA_ARCH__)
  if constexpr (BF) {
    const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w));
    a = f.x;
    b = f.y;
  } else {
    const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&w));
    a = f.x;
    b = f.y;
  }
#else
  a = from16(w & 0xffffu, BF);
  b = from16(w >> 16, BF);
#endif
}

// D staging: butterfly n's 16 outputs at complex index n * kTcDRow + r
// (18-element rows: conflict-free for the fragment stores and the 16-byte
// row reads).
constexpr int kTcDRow = 18;
static_assert(32 * kTcDRow * 2 <= 2 * kTcTableWords, "D staging must fit the first two B tables");

#if defined(__CUDA_ARCH__)
template <bool BF>
ESTL_HD void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  if constexpr (BF)
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

// The 16-point DFT of every lane's butterfly x (twiddled, FP32) through the
// tensor cores: split and stage, GEMM, stage D, read back.  On return x[r]
// holds output r of the lane's own butterfly, as DFT<16>::run leaves it.
// Warp-collective: all 32 lanes call it together.
template <int KIND>
ESTL_HD void tc_dft16(cf32 (&x)[16], const TcCtx& ctx) {
  constexpr bool BF = KIND != SPLIT_FP16X2;
  constexpr int TERMS = split_terms(KIND);
  // 1. scale (fp16) and split the 32 real inputs into TERMS 16-bit terms
  float sc = 1.f, inv = 1.f;
  if constexpr (!BF) {
    float m = 0.f;
#pragma unroll
    for (int k = 0; k < 16; ++k) m = fmaxf(m, fmaxf(fabsf(x[k].x), fabsf(x[k].y)));
    // 2^e with m < 2^e <= 2m from the exponent field of m (clamped so that
    // 2^e and 2^-e are normal floats; m = 0 leaves the butterfly unscaled)
    int be = (int)((f32_bits_hd(m) >> 23) & 0xff) - 126;  // m = f 2^be, 0.5 <= f < 1
    be = be < -125 ? -125 : (be > 126 ? 126 : be);
    if (m == 0.f) be = 0;
    sc = bits_f32_hd((uint32_t)(127 + be) << 23);
    inv = bits_f32_hd((uint32_t)(127 - be) << 23);
  }
#pragma unroll
  for (int w = 0; w < 16; ++w) {
    // word w: k = 2w, 2w + 1 (real parts for w < 8, imaginary parts after)
    float r0 = (w < 8 ? x[2 * w].x : x[2 * w - 16].y) * inv;
    float r1 = (w < 8 ? x[2 * w + 1].x : x[2 * w - 15].y) * inv;
#pragma unroll
    for (int q = 0; q < TERMS; ++q) {
      const uint32_t h = pack16<BF>(r0, r1);
      ctx.stage[q * kTcTableWords + ctx.lane * kTcRowWords + w] = h;
      if (q + 1 < TERMS) {
        float f0, f1;
        unpack16<BF>(h, f0, f1);
        r0 -= f0;
        r1 -= f1;
      }
    }
  }
  ESTL_SYNCWARP();
  // 2. D = A B: 2 m-tiles (Re, Im rows) x 4 n-tiles (8 butterflies) per lane
  const int g = ctx.lane >> 2, tig = ctx.lane & 3;
  float d[4][2][4];
#pragma unroll
  for (int nt = 0; nt < 4; ++nt)
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int i = 0; i < 4; ++i) d[nt][mt][i] = 0.f;
#if defined(__CUDA_ARCH__)
  // B fragments of butterfly columns 8 nt .. 8 nt + 7, all 32 k: one
  // ldmatrix.x4 per (n-tile, term): registers {b0, b1} of k-tile 0, then 1
  // (row address: butterfly 8 nt + (lane & 7), k = 8 (lane >> 3)).
  uint32_t b[4][TERMS][4];
  const int lrow = ctx.lane & 7, lblk = ctx.lane >> 3;
#pragma unroll
  for (int nt = 0; nt < 4; ++nt)
#pragma unroll
    for (int q = 0; q < TERMS; ++q)
      ldmatrix_x4(b[nt][q], ctx.stage.p + q * kTcTableWords + (8 * nt + lrow) * kTcRowWords + 4 * lblk);
  // The tensor cores accumulate with truncation relative to the largest
  // term: the small correction products (qa + qb >= 1) go first, into an
  // accumulator that is still small, and the large hi x hi products last, so
  // that the large partial sums are truncated only twice (once per k-tile).
#pragma unroll
  for (int phase = 0; phase < 2; ++phase) {
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) {
#pragma unroll
      for (int qa = 0; qa < TERMS; ++qa) {
        if (phase == 1 && qa > 0) continue;
        // A fragment of rows 16 mt .. +15, k = 16 kt .. +15: matrices
        // (rows 0-7, k 0-7), (rows 8-15, k 0-7), (rows 0-7, k 8-15), (rows 8-15, k 8-15)
        uint32_t a[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
          ldmatrix_x4(a[mt], ctx.atab.p + qa * kTcTableWords + (16 * mt + lrow + 8 * (lblk & 1)) * kTcRowWords +
                                 8 * kt + 4 * (lblk >> 1));
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
          for (int qb = 0; qa + qb < TERMS; ++qb) {
            if ((phase == 0) == (qa + qb == 0)) continue;  // phase 0: corrections, phase 1: hi x hi
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
              mma16816<BF>(d[nt][mt], a[mt], b[nt][qb][2 * kt], b[nt][qb][2 * kt + 1]);
          }
      }
    }
  }
#else
  // emulator: the same D elements from the staged terms
  for (int nt = 0; nt < 4; ++nt)
    for (int mt = 0; mt < 2; ++mt)
      for (int i = 0; i < 4; ++i) {
        const int m = 16 * mt + g + ((i & 2) ? 8 : 0);
        const int n = 8 * nt + 2 * tig + (i & 1);
        float acc = 0.f;
        for (int qa = 0; qa < TERMS; ++qa)
          for (int qb = 0; qa + qb < TERMS; ++qb)
            for (int k = 0; k < 32; ++k) {
              const uint32_t aw = ctx.atab[qa * kTcTableWords + m * kTcRowWords + (k >> 1)];
              const uint32_t bw = ctx.stage[qb * kTcTableWords + n * kTcRowWords + (k >> 1)];
              acc += from16((k & 1) ? aw >> 16 : aw & 0xffffu, BF) * from16((k & 1) ? bw >> 16 : bw & 0xffffu, BF);
            }
        d[nt][mt][i] = acc;
      }
#endif
  ESTL_SYNCWARP();  // every lane has its B fragments before D overwrites them
  // 3. D element i of m-tile mt: row g (+8 for i >= 2), butterfly 8 nt + 2 tig + (i & 1)
  const Ptr<cf32> dst{reinterpret_cast<cf32*>(ctx.stage.p), 32 * kTcDRow};
#pragma unroll
  for (int nt = 0; nt < 4; ++nt)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = g + ((i & 2) ? 8 : 0);
      const int n = 8 * nt + 2 * tig + (i & 1);
      dst[n * kTcDRow + r] = cf32{d[nt][0][i], d[nt][1][i]};
    }
  ESTL_SYNCWARP();
#if defined(__CUDA_ARCH__)
  const float4* row = reinterpret_cast<const float4*>(dst.p + ctx.lane * kTcDRow);  // 144-byte rows: 16-byte aligned
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const float4 y = row[r];
    x[2 * r] = cf32{y.x * sc, y.y * sc};
    x[2 * r + 1] = cf32{y.z * sc, y.w * sc};
  }
#else
  for (int r = 0; r < 16; ++r) {
    const cf32 y = dst[ctx.lane * kTcDRow + r];
    x[r] = cf32{y.x * sc, y.y * sc};
  }
#endif
  ESTL_SYNCWARP();  // D rows read before the next pass stages over them
}

// run_passes with the radix-16 DFTs on the tensor cores (E = 16: one
// butterfly per thread; the other radices stay FP32).  Same exchanges and
// the same register state on exit as run_passes.
template <int KIND, class TL, int p, class SIDX>
ESTL_HD void run_passes_tc_k(cf32 (&v)[TL::E], int t, int c, const Ptr<cf32>& sm, const Ptr<const cf32>& tw,
                             SIDX sidx, const TcCtx& ctx) {
  static_assert(TL::E == 16 && TL::LR_FULL == 4, "tensor-core passes need radix-16 tiles of 16 elements per thread");
  if constexpr (p < TL::P) {
    if constexpr (TL::lr(p) == 4) {
      TL::template twiddle_only<p>(v, t, tw);
      tc_dft16<KIND>(v, ctx);
    } else {
      TL::template compute<p>(v, t, tw);
    }
    if constexpr (p + 1 < TL::P) {
#pragma unroll
      for (int j = 0; j < TL::E; ++j) sm[sidx(c, TL::template out_pos<p>(t, j))] = v[j];
      ESTL_SYNC();
#pragma unroll
      for (int j = 0; j < TL::E; ++j) v[j] = sm[sidx(c, t + TL::T * j)];
      ESTL_SYNC();
    }
    run_passes_tc_k<KIND, TL, p + 1>(v, t, c, sm, tw, sidx, ctx);
  }
}

template <class TL, class SIDX>
ESTL_HD void run_passes_tc(cf32 (&v)[TL::E], int t, int c, const Ptr<cf32>& sm, const Ptr<const cf32>& tw,
                           SIDX sidx, const TcCtx& ctx);

// run_passes (FP32) or run_passes_tc (split precision, TC tiles).  The
// tensor-core table of the tile must be complete: the first call of a
// TC tile synchronises the CTA before its first pass.
template <bool TC, class TL, class SIDX>
ESTL_HD void any_passes(cf32 (&v)[TL::E], int t, int c, const Ptr<cf32>& sm, const Ptr<const cf32>& tw, SIDX sidx,
                        cf32* tc_area, int split, int tid) {
  if constexpr (TC) {
    ESTL_SYNC();
    run_passes_tc<TL>(v, t, c, sm, tw, sidx, tc_ctx(tc_area, split, tid));
  } else {
    run_passes<TL, 0>(v, t, c, sm, tw, sidx);
  }
}

template <class TL, class SIDX>
ESTL_HD void run_passes_tc(cf32 (&v)[TL::E], int t, int c, const Ptr<cf32>& sm, const Ptr<const cf32>& tw,
                           SIDX sidx, const TcCtx& ctx) {
  switch (ctx.kind) {
    case SPLIT_FP16X2: run_passes_tc_k<SPLIT_FP16X2, TL, 0>(v, t, c, sm, tw, sidx, ctx); break;
    case SPLIT_BF16X2: run_passes_tc_k<SPLIT_BF16X2, TL, 0>(v, t, c, sm, tw, sidx, ctx); break;
    default: run_passes_tc_k<SPLIT_BF16X3, TL, 0>(v, t, c, sm, tw, sidx, ctx); break;
  }
}

}  // namespace estl
