// fft_core.cuh — FFT tile machinery shared by the sm_103a kernels and the
// host-side index emulator.
//
// The reference computes one Stockham pass per OpenCL kernel
// (FFT_OpenCL_Contiguous.h:144-184): one work-item loads B_q points, applies
// the pass twiddle, runs an unrolled radix-2 B_q-point DFT in registers
// (OpenCLFFTAlgorithm.h:14-43) and stores them, with a full global-memory
// round trip per pass.  Here a CTA keeps a whole tile of transforms on chip
// and runs every pass of the tile in one launch:
//
//   global --(coalesced ld)--> registers --radix-R butterfly--> shared
//          --> registers --butterfly--> ... --> registers --(coalesced st)--> global
//
// Stockham pass p (radix R, Ns = product of earlier radices), butterfly b:
//   inputs   b + r*(M/R)                          r = 0..R-1
//   twiddle  x_r *= w_{Ns*R}^{r*k},  k = b mod Ns (w_M = exp(-2*pi*i/M))
//   outputs  (b div Ns)*Ns*R + k + r*Ns           (natural order after the last pass)
// Thread t of a row owns butterflies b = t + T*i, so every pass reads the
// thread's slots at positions t + T*j (j = i + r*E/R): the first-pass loads and
// the last-pass stores are both unit-stride across a warp.
//
// All index arithmetic lives in ESTL_HD functions so that the same code runs
// under the host emulator (ESTL_EMU: every global/shared access is bounds
// checked, barriers are std::barrier) before it ever runs on a GPU.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define ESTL_HD __device__ __forceinline__
#define ESTL_CX __host__ __device__ constexpr
#else
#define ESTL_HD inline
#define ESTL_CX constexpr
#endif

#ifdef ESTL_EMU
void estl_emu_sync();
[[noreturn]] void estl_emu_fail(const char* what, long long idx, long long n);
#define ESTL_SYNC() estl_emu_sync()
#define ESTL_CHECK(i, n, what)                                                       \
  do {                                                                               \
    if (!((long long)(i) >= 0 && (long long)(i) < (long long)(n)))                   \
      estl_emu_fail(what, (long long)(i), (long long)(n));                           \
  } while (0)
#else
#define ESTL_SYNC() __syncthreads()
#define ESTL_CHECK(i, n, what) ((void)0)
#endif

namespace estl {

// Interleaved complex64, the device image of Complex<float> in the
// SplitInterleavedDataInterface(n, false) layout (DataInterface.h:37-45,
// Complex.h:177-180): re at 2i, im at 2i+1.
struct alignas(8) cf32 {
  float x, y;
};

ESTL_HD cf32 cadd(cf32 a, cf32 b) { return {a.x + b.x, a.y + b.y}; }
ESTL_HD cf32 csub(cf32 a, cf32 b) { return {a.x - b.x, a.y - b.y}; }
ESTL_HD cf32 cmul(cf32 a, cf32 b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
ESTL_HD cf32 mul_mi(cf32 a) { return {a.y, -a.x}; }  // a * (-i)

// Pointer with an element count.  The count is only checked by the emulator.
template <class T>
struct Ptr {
  T* p;
  long long n;
  ESTL_HD T& operator[](long long i) const {
    ESTL_CHECK(i, n, "global/shared index");
    return p[i];
  }
  // Sub-range [off, off + len): lets the hot loops index with 32-bit offsets.
  ESTL_HD Ptr sub(long long off, long long len) const {
    ESTL_CHECK(off, n + 1, "sub-range start");
    ESTL_CHECK(off + len, n + 1, "sub-range end");
    return Ptr{p + off, len};
  }
};

// Read-only global load through the non-coherent path.
ESTL_HD cf32 ldg(const Ptr<const cf32>& q, long long i) {
  ESTL_CHECK(i, q.n, "global load");
#if defined(__CUDA_ARCH__)
  float2 v = __ldg(reinterpret_cast<const float2*>(q.p) + i);
  return {v.x, v.y};
#else
  return q.p[i];
#endif
}

// Streaming global load/store: the input of a transform is read once and its
// output written once, so they are marked evict-first in L1/L2.
ESTL_HD cf32 ldcs(const Ptr<const cf32>& q, long long i) {
  ESTL_CHECK(i, q.n, "global load");
#if defined(__CUDA_ARCH__)
  float2 v = __ldcs(reinterpret_cast<const float2*>(q.p) + i);
  return {v.x, v.y};
#else
  return q.p[i];
#endif
}
// Load that bypasses L1: data another CTA of the same launch may have
// written (four-step scratch in the persistent packed kernel).
ESTL_HD cf32 ldcg(const Ptr<cf32>& q, long long i) {
  ESTL_CHECK(i, q.n, "global load");
#if defined(__CUDA_ARCH__)
  float2 v = __ldcg(reinterpret_cast<const float2*>(q.p) + i);
  return {v.x, v.y};
#else
  return q.p[i];
#endif
}

ESTL_HD void stcs(const Ptr<cf32>& q, long long i, cf32 v) {
  ESTL_CHECK(i, q.n, "global store");
#if defined(__CUDA_ARCH__)
  __stcs(reinterpret_cast<float2*>(q.p) + i, make_float2(v.x, v.y));
#else
  q.p[i] = v;
#endif
}

// ---------------------------------------------------------------------------
// Register DFTs (forward, e^{-2 pi i / R}), natural-order in and out.
// The reference generates these as fully unrolled radix-2 networks with
// 6-significant-digit twiddle literals (KernelGenerator.h:53-69,100-142); here
// they are radix-4 based with exactly rounded FP32 constants.
// ---------------------------------------------------------------------------
constexpr float kC8 = 0.70710678118654752440f;   // cos(pi/4)
constexpr float kC16 = 0.92387953251128675613f;  // cos(pi/8)
constexpr float kS16 = 0.38268343236508977173f;  // sin(pi/8)

ESTL_HD cf32 cmulc(cf32 a, float c, float s) { return {a.x * c - a.y * s, a.x * s + a.y * c}; }

ESTL_HD void dft2(cf32& a, cf32& b) {
  cf32 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

ESTL_HD void dft4(cf32& x0, cf32& x1, cf32& x2, cf32& x3) {
  cf32 a = cadd(x0, x2), b = csub(x0, x2), c = cadd(x1, x3), d = mul_mi(csub(x1, x3));
  x0 = cadd(a, c);
  x2 = csub(a, c);
  x1 = cadd(b, d);
  x3 = csub(b, d);
}

// x * w8^1 = x * (c, -c)
ESTL_HD cf32 mul_w8_1(cf32 a) { return {kC8 * (a.x + a.y), kC8 * (a.y - a.x)}; }
// x * w8^3 = x * (-c, -c)
ESTL_HD cf32 mul_w8_3(cf32 a) { return {kC8 * (a.y - a.x), -kC8 * (a.x + a.y)}; }

template <int R>
struct DFT;

template <>
struct DFT<1> {
  ESTL_HD static void run(cf32*) {}
};
template <>
struct DFT<2> {
  ESTL_HD static void run(cf32* x) { dft2(x[0], x[1]); }
};
template <>
struct DFT<4> {
  ESTL_HD static void run(cf32* x) { dft4(x[0], x[1], x[2], x[3]); }
};
template <>
struct DFT<8> {
  // decimation in frequency: a_r = x_r + x_{r+4}, b_r = (x_r - x_{r+4}) w8^r,
  // X[2k] = DFT4(a)[k], X[2k+1] = DFT4(b)[k].
  ESTL_HD static void run(cf32* x) {
    cf32 a0 = cadd(x[0], x[4]), a1 = cadd(x[1], x[5]), a2 = cadd(x[2], x[6]), a3 = cadd(x[3], x[7]);
    cf32 b0 = csub(x[0], x[4]);
    cf32 b1 = mul_w8_1(csub(x[1], x[5]));
    cf32 b2 = mul_mi(csub(x[2], x[6]));
    cf32 b3 = mul_w8_3(csub(x[3], x[7]));
    dft4(a0, a1, a2, a3);
    dft4(b0, b1, b2, b3);
    x[0] = a0; x[2] = a1; x[4] = a2; x[6] = a3;
    x[1] = b0; x[3] = b1; x[5] = b2; x[7] = b3;
  }
};
template <>
struct DFT<16> {
  // 4 x 4: n = n2 + 4 n1, k = k1 + 4 k2.
  //   A[n2][k1] = DFT4_n1(x[n2 + 4 n1]) * w16^(n2 k1);  X[k1 + 4 k2] = DFT4_n2(A[n2][k1]).
  ESTL_HD static void run(cf32* x) {
    dft4(x[0], x[4], x[8], x[12]);
    dft4(x[1], x[5], x[9], x[13]);
    dft4(x[2], x[6], x[10], x[14]);
    dft4(x[3], x[7], x[11], x[15]);
    // now x[n2 + 4 k1] = A[n2][k1]
    x[5] = cmulc(x[5], kC16, -kS16);   // w^1
    x[9] = mul_w8_1(x[9]);             // w^2
    x[13] = cmulc(x[13], kS16, -kC16); // w^3
    x[6] = mul_w8_1(x[6]);             // w^2
    x[10] = mul_mi(x[10]);             // w^4
    x[14] = mul_w8_3(x[14]);           // w^6
    x[7] = cmulc(x[7], kS16, -kC16);   // w^3
    x[11] = mul_w8_3(x[11]);           // w^6
    x[15] = cmulc(x[15], -kC16, kS16); // w^9
    dft4(x[0], x[1], x[2], x[3]);      // k1 = 0 -> X[0], X[4], X[8], X[12]
    dft4(x[4], x[5], x[6], x[7]);      // k1 = 1
    dft4(x[8], x[9], x[10], x[11]);    // k1 = 2
    dft4(x[12], x[13], x[14], x[15]);  // k1 = 3
    // x[4 k1 + k2] = X[k1 + 4 k2]: transpose the 4x4 block in registers
    cf32 t;
    t = x[1]; x[1] = x[4]; x[4] = t;
    t = x[2]; x[2] = x[8]; x[8] = t;
    t = x[3]; x[3] = x[12]; x[12] = t;
    t = x[6]; x[6] = x[9]; x[9] = t;
    t = x[7]; x[7] = x[13]; x[13] = t;
    t = x[11]; x[11] = x[14]; x[14] = t;
  }
};

// w32^k = exp(-2 pi i k / 32) = cos(pi k / 16) - i sin(pi k / 16), k = 1..7
constexpr float kC32_1 = 0.98078528040323044913f;  // cos(pi/16)
constexpr float kS32_1 = 0.19509032201612826785f;  // sin(pi/16)
constexpr float kC32_3 = 0.83146961230254523708f;  // cos(3 pi/16)
constexpr float kS32_3 = 0.55557023301960222474f;  // sin(3 pi/16)

template <>
struct DFT<32> {
  // decimation in time: E = DFT16(x[2m]), O = DFT16(x[2m+1]),
  // X[k] = E[k] + w32^k O[k], X[k+16] = E[k] - w32^k O[k].
  ESTL_HD static void run(cf32* x) {
    cf32 e[16], o[16];
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      e[m] = x[2 * m];
      o[m] = x[2 * m + 1];
    }
    DFT<16>::run(e);
    DFT<16>::run(o);
    o[1] = cmulc(o[1], kC32_1, -kS32_1);
    o[2] = cmulc(o[2], kC16, -kS16);
    o[3] = cmulc(o[3], kC32_3, -kS32_3);
    o[4] = mul_w8_1(o[4]);
    o[5] = cmulc(o[5], kS32_3, -kC32_3);
    o[6] = cmulc(o[6], kS16, -kC16);
    o[7] = cmulc(o[7], kS32_1, -kC32_1);
    o[8] = mul_mi(o[8]);
    o[9] = cmulc(o[9], -kS32_1, -kC32_1);
    o[10] = cmulc(o[10], -kS16, -kC16);
    o[11] = cmulc(o[11], -kS32_3, -kC32_3);
    o[12] = mul_w8_3(o[12]);
    o[13] = cmulc(o[13], -kC32_3, -kS32_3);
    o[14] = cmulc(o[14], -kC16, -kS16);
    o[15] = cmulc(o[15], -kC32_1, -kS32_1);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      x[k] = cadd(e[k], o[k]);
      x[k + 16] = csub(e[k], o[k]);
    }
  }
};

// ---------------------------------------------------------------------------
// Twiddle bank: one device table holding w_{2^k}^j for every k <= kBankLog
// at index 2^k + j, followed by 4096-entry "low" tables for 2^(kBankLog+1)..2^kMaxLog
// so that w_N^a = lo_N[a mod 4096] * w_{N/4096}^{a div 4096} for large N.
// Generated on the device from FP64 sincospi and rounded once to FP32.
// ---------------------------------------------------------------------------
constexpr int kBankLog = 18;
constexpr int kMaxLog = 26;
constexpr int kLoLog = 12;
constexpr long long kBankDirect = 1LL << (kBankLog + 1);
constexpr long long kBankSize = kBankDirect + (long long)(kMaxLog - kBankLog) * (1LL << kLoLog);
ESTL_CX long long bank_lo_offset(int logn) { return kBankDirect + (long long)(logn - kBankLog - 1) * (1LL << kLoLog); }

// w_N^a for 0 <= a < N, N = 2^logn.
ESTL_HD cf32 twiddle_n(const Ptr<const cf32>& bank, int logn, int a) {
  if (logn <= kBankLog) return ldg(bank, (1 << logn) + a);
  cf32 lo = ldg(bank, (int)bank_lo_offset(logn) + (a & ((1 << kLoLog) - 1)));
  cf32 hi = ldg(bank, (1 << (logn - kLoLog)) + (a >> kLoLog));
  return cmul(lo, hi);
}

// x_r *= w^r for r = 1..15 given w, w^2, w^4 and w^8: every other power is
// a product of at most three of them.
ESTL_HD void apply_powers16(cf32* x, cf32 w1, cf32 w2, cf32 w4, cf32 w8) {
  cf32 w3 = cmul(w1, w2), w5 = cmul(w1, w4), w6 = cmul(w2, w4), w7 = cmul(w3, w4);
  x[1] = cmul(x[1], w1);
  x[2] = cmul(x[2], w2);
  x[3] = cmul(x[3], w3);
  x[4] = cmul(x[4], w4);
  x[5] = cmul(x[5], w5);
  x[6] = cmul(x[6], w6);
  x[7] = cmul(x[7], w7);
  x[8] = cmul(x[8], w8);
  x[9] = cmul(x[9], cmul(w1, w8));
  x[10] = cmul(x[10], cmul(w2, w8));
  x[11] = cmul(x[11], cmul(w3, w8));
  x[12] = cmul(x[12], cmul(w4, w8));
  x[13] = cmul(x[13], cmul(w5, w8));
  x[14] = cmul(x[14], cmul(w6, w8));
  x[15] = cmul(x[15], cmul(w7, w8));
}

// x_r *= w_M^{r u} for r = 1..R-1 with w_M^{u}, w_M^{2u}, w_M^{4u}, w_M^{8u}
// loaded from the table (tw points at w_M^0) and the other powers formed by at
// most three products.
template <int R>
ESTL_HD void twiddle_apply(cf32* x, const Ptr<const cf32>& tw, int u) {
  if constexpr (R == 2) {
    x[1] = cmul(x[1], ldg(tw, u));
  } else if constexpr (R == 4) {
    cf32 w1 = ldg(tw, u), w2 = ldg(tw, 2 * u);
    x[1] = cmul(x[1], w1);
    x[2] = cmul(x[2], w2);
    x[3] = cmul(x[3], cmul(w1, w2));
  } else if constexpr (R == 8) {
    cf32 w1 = ldg(tw, u), w2 = ldg(tw, 2 * u), w4 = ldg(tw, 4 * u);
    cf32 w3 = cmul(w1, w2);
    x[1] = cmul(x[1], w1);
    x[2] = cmul(x[2], w2);
    x[3] = cmul(x[3], w3);
    x[4] = cmul(x[4], w4);
    x[5] = cmul(x[5], cmul(w1, w4));
    x[6] = cmul(x[6], cmul(w2, w4));
    x[7] = cmul(x[7], cmul(w3, w4));
  } else if constexpr (R == 16) {
    apply_powers16(x, ldg(tw, u), ldg(tw, 2 * u), ldg(tw, 4 * u), ldg(tw, 8 * u));
  } else if constexpr (R == 32) {
    const cf32 w1 = ldg(tw, u), w2 = ldg(tw, 2 * u), w4 = ldg(tw, 4 * u), w8 = ldg(tw, 8 * u), w16 = ldg(tw, 16 * u);
    // x_r *= w^r: r < 16 directly, r >= 16 as w^16 * w^(r - 16)
#pragma unroll
    for (int r = 16; r < 32; ++r) x[r] = cmul(x[r], w16);
    apply_powers16(x, w1, w2, w4, w8);
    apply_powers16(x + 16, w1, w2, w4, w8);
  }
}

// ---------------------------------------------------------------------------
// Radix schedule of an M = 2^LOGM point tile FFT: full passes of radix
// 2^LOGR, then one remainder pass.  Mirrors the reference plan
// BGs = [16]*floor(log2 N / 4) (+ 2^(log2 N mod 4)) (FFT_OpenCL_Contiguous.h:54-61)
// with its prefix products A_q / N_q (OpenCLFFTAlgorithm.h:9-12).
// ---------------------------------------------------------------------------
template <int LOGM, int LOGE, int LOGR>
struct Tile {
  static_assert(LOGE >= LOGR || LOGE >= LOGM, "elements per thread must cover a radix");
  static constexpr int LM = LOGM, LE = LOGE;
  static constexpr int M = 1 << LOGM;
  static constexpr int LR_FULL = (LOGR < LOGM) ? LOGR : LOGM;
  static constexpr int E = 1 << LOGE;
  static constexpr int LOGT = LOGM - LOGE;
  static constexpr int T = 1 << LOGT;
  static constexpr int NFULL = LOGM / LR_FULL;
  static constexpr int LREM = LOGM % LR_FULL;
  static constexpr int P = NFULL + (LREM ? 1 : 0);
  static_assert(LOGM >= LOGE, "tile smaller than a thread's register block");

  ESTL_CX static int lr(int p) { return p < NFULL ? LR_FULL : LREM; }
  ESTL_CX static int lns(int p) { return p * LR_FULL; }

  // Compute pass p in registers: v[j] holds position t + T*j on entry and
  // output y_r of butterfly i (slot j = i + r*E/R) on exit.
  template <int p>
  ESTL_HD static void compute(cf32 (&v)[E], int t, const Ptr<const cf32>& tw) {
    constexpr int LR = lr(p), R = 1 << LR, LNS = lns(p), NS = 1 << LNS, G = E / R;
#pragma unroll
    for (int i = 0; i < G; ++i) {
      cf32 x[R];
#pragma unroll
      for (int r = 0; r < R; ++r) x[r] = v[i + r * G];
      if constexpr (NS > 1) {
        int b = t + T * i;
        int k = b & (NS - 1);
        int u = k << (LOGM - LNS - LR);  // k * M / (Ns * R)
        twiddle_apply<R>(x, tw, u);
      }
      DFT<R>::run(x);
#pragma unroll
      for (int r = 0; r < R; ++r) v[i + r * G] = x[r];
    }
  }

  // The twiddle step of pass p alone (the tensor-core passes run the DFT
  // elsewhere); only for one butterfly per thread (E == R).
  template <int p>
  ESTL_HD static void twiddle_only(cf32 (&v)[E], int t, const Ptr<const cf32>& tw) {
    constexpr int LR = lr(p), R = 1 << LR, LNS = lns(p), NS = 1 << LNS;
    static_assert(R == E, "one butterfly per thread");
    if constexpr (NS > 1) {
      const int k = t & (NS - 1);
      twiddle_apply<R>(v, tw, k << (LOGM - LNS - LR));
    }
  }

  // Output position of slot j after pass p.
  template <int p>
  ESTL_HD static int out_pos(int t, int j) {
    constexpr int LR = lr(p), R = 1 << LR, LNS = lns(p), NS = 1 << LNS, G = E / R;
    int i = j & (G - 1), r = j / G;
    int b = t + T * i;
    int k = b & (NS - 1);
    return ((b - k) << LR) + k + (r << LNS);
  }

  // Shared-memory row padding: one spare slot per R elements keeps the
  // scattered radix-R pass stores (a half-warp writing slots R apart) free of
  // bank conflicts: 16 for radix-16 tiles, 32 for radix-32 tiles.
  static constexpr int PADSH = (LOGR >= 5 && LOGM >= 5) ? 5 : 4;
  ESTL_CX static int pad(int m) { return m + (m >> PADSH); }
  static constexpr int MP = M + (M >> PADSH);
};

// Stride (in complex elements) between the shared-memory rows of a tile of
// C rows.  A half-warp of 8-byte accesses covers all 32 banks once when its
// 16 lanes hit distinct 16-element residues.  Row-major accesses by T >= 16
// lanes per row never span rows; the column-fastest store remap (lanes c
// fastest, then 16/C positions per row) needs stride = 16/C (mod 16).
ESTL_CX int row_stride(int mp, int c) { return c >= 16 ? (mp | 1) : ((mp + 15) / 16) * 16 + 16 / c; }

// Rows of an exchange that is accessed both row-major (T threads a row, the
// tile passes) and transposed (lanes over C rows at one position, the
// column-fastest stores).  For T >= 16 or C < 16 this is row_stride(MP, C).
// For T < 16 and C >= 16 a half-warp's row-major access spans 16/T rows: a
// stride of T (mod 16) puts those rows on disjoint bank pairs, and each group
// of 16/T rows is skewed by one more slot, so that 16 consecutive rows at one
// position also fall on 16 distinct bank pairs (8-byte elements: bank pair =
// index mod 16).  An odd stride alone doubles the row-major wavefronts there.
template <int T, int C, int MP>
struct XposeRows {
  static constexpr bool SKEW = T < 16 && C >= 16;
  static constexpr int LSK = T >= 16 ? 0 : T == 8 ? 1 : T == 4 ? 2 : T == 2 ? 3 : 4;  // log2(16 / T)
  static constexpr int CS = SKEW ? MP + (((T - MP) % 16) + 16) % 16 : row_stride(MP, C);
  static constexpr int ELEMS = C * CS + (SKEW ? (C >> LSK) : 0);
  ESTL_HD static int row(int c) { return c * CS + (SKEW ? (c >> LSK) : 0); }
};

// Runs passes p..P-1 over the tile.  Between passes each thread writes its
// outputs to shared memory at their Stockham positions and re-reads its next
// inputs at t + T*j.  SIDX maps (column c, position m) to a shared index.
template <class TL, int p, class SIDX>
ESTL_HD void run_passes(cf32 (&v)[TL::E], int t, int c, const Ptr<cf32>& sm, const Ptr<const cf32>& tw,
                        SIDX sidx) {
  if constexpr (p < TL::P) {
    TL::template compute<p>(v, t, tw);
    if constexpr (p + 1 < TL::P) {
#pragma unroll
      for (int j = 0; j < TL::E; ++j) sm[sidx(c, TL::template out_pos<p>(t, j))] = v[j];
      ESTL_SYNC();
#pragma unroll
      for (int j = 0; j < TL::E; ++j) v[j] = sm[sidx(c, t + TL::T * j)];
      ESTL_SYNC();
    }
    run_passes<TL, p + 1>(v, t, c, sm, tw, sidx);
  }
}

// ---------------------------------------------------------------------------
// Blocks per SM requested from the compiler: 16 elements per thread are built
// for 1024 resident threads per SM (64 registers), 32 elements per thread for
// 512 (128 registers).
ESTL_CX int min_blocks(int nt, int e) {
  return nt * e >= 16384 ? 1 : (16384 / (nt * e) < 2048 / nt ? 16384 / (nt * e) : 2048 / nt);
}

// Programmatic dependent launch (kernels launched with
// cudaLaunchAttributeProgrammaticStreamSerialization): wait until the
// previous kernel of the stream has completed and its writes are visible,
// then let the next kernel's CTAs be scheduled as soon as every CTA of this
// grid has started, so that its launch and prologue overlap this grid's last
// wave.  Without the launch attribute both instructions do nothing.
ESTL_HD void pdl_wait() {
#if defined(__CUDA_ARCH__)
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
#endif
}
ESTL_HD void pdl_trigger() {
#if defined(__CUDA_ARCH__)
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
#endif
}
ESTL_HD void pdl_enter() {
  pdl_wait();
  pdl_trigger();
}

// Kernels whose CTAs are all resident from the start (persistent tile loops)
// trigger their dependents when a CTA has issued its last tile instead.
template <class K, class = void>
struct is_persistent {
  static constexpr bool value = false;
};
template <class K>
struct is_persistent<K, decltype((void)K::PERSISTENT)> {
  static constexpr bool value = K::PERSISTENT;
};

// Cluster tiles (cluster_core.cuh): log2 of the CTAs per cluster and of the
// column DFT length; 0 for every other kernel.
template <class K, class = void>
struct cluster_of {
  static constexpr int log_cluster = 0, log_split = 0;
};
template <class K>
struct cluster_of<K, decltype((void)K::LOG_CLUSTER)> {
  static constexpr int log_cluster = K::LOG_CLUSTER, log_split = K::LOG_SPLIT;
};

// Keeps the compiler from hoisting every iteration's table loads to the top
// of an unrolled epilogue (which costs 2 registers per load in flight).
ESTL_HD void schedule_fence() {
#if defined(__CUDA_ARCH__)
  asm volatile("" ::: "memory");
#endif
}

}  // namespace estl

#include "tc_core.cuh"

namespace estl {

// Launch parameters shared by all tile kernels.
// ---------------------------------------------------------------------------
struct TileArgs {
  Ptr<const cf32> in;
  Ptr<cf32> out;
  Ptr<const cf32> bank;
  long long rows;  // single: number of transforms
  int logn;        // log2 of the full transform length
  int logn1;       // four-step: log2 N1 (N = N1 * N2)
  float sgn;       // +1 forward; -1 = backward via conj(FFT(conj(x)))
  long long grid;  // CTAs launched (persistent kernels loop over rows / tiles grid apart)
  int split;       // tensor-core kernels: SplitKind of the radix-16 passes (tc_core.cuh)
  long long* err;  // bulk-load kernels: 1 + the tile whose bounded wait gave up (0 = none)
  const void* tmap = nullptr;  // tensor-map kernels: the CUtensorMap kernel parameter of the input
  int ologr = 0;  // column tiles: interleaved output of a three-pass plan's middle pass (planner.h Step::ologr)
  // Uneven batches (bucketed packed plans): element offset of each transform
  // of the step in the caller's input (single, column and resident tiles) and
  // output (single, row and resident tiles) buffers; p == nullptr: transform
  // f at f * N.  The four-step scratch stays dense.
  Ptr<const long long> xoff{nullptr, 0};
};

// Element offset of transform f of a step in the caller's buffers.
ESTL_HD long long xbase(const TileArgs& a, long long f, long long n) { return a.xoff.p ? a.xoff[f] : f * n; }

ESTL_HD void atomic_max_ll(long long* p, long long v) {
#if defined(__CUDA_ARCH__)
  atomicMax(p, v);
#else
  if (*p < v) *p = v;
#endif
}

ESTL_HD cf32 conj_if(cf32 v, float sgn) { return {v.x, v.y * sgn}; }

// Whole transforms of length M = 2^LOGM, C transforms per CTA.  Thread
// (c, t) = (tid >> LOGT, tid & (T-1)): unit-stride rows for loads and stores.
// TC: radix-16 passes on the tensor cores with the split precision
// TileArgs::split (tc_core.cuh); the shared memory then also holds the
// tensor-core area after the exchange buffer.
template <int LOGM, int LOGE, int LOGR, int LOGC, bool TC = false>
struct SingleKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  static constexpr int CS = row_stride(TL::MP, TL::T >= 16 ? 16 : TL::T * C >= 16 ? 16 / TL::T : C);
  static constexpr int EXCH = (TL::P > 1 || TC) ? C * CS : 0;
  static constexpr int TC_OFF = (EXCH + 1) & ~1;  // 16-byte aligned tensor-core area
  static constexpr int SMEM_ELEMS = TC ? TC_OFF + (int)((tc_area_words(NT / 32) + 1) / 2) : EXCH;
  static constexpr int MIN_BLOCKS = TC ? (NT <= 256 ? 2 : 1) : min_blocks(NT, TL::E);
  static_assert(NT <= 1024, "too many threads");
  static_assert(!TC || NT % 32 == 0, "tensor-core tiles run whole warps");

  struct Sidx {
    ESTL_HD int operator()(int c, int m) const { return c * CS + TL::pad(m); }
  };

  // One tile: row c of the tile is transform `in` -> `out` (length M each);
  // rows with valid == false only take part in the barriers.
  ESTL_HD static void body(const Ptr<const cf32>& in, const Ptr<cf32>& out, bool valid, int tid, cf32* smraw,
                           const Ptr<const cf32>& bank, float sgn, int split = SPLIT_NONE) {
    const int t = tid & (TL::T - 1);
    const int c = tid >> TL::LOGT;
    const Ptr<const cf32> tw = bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, EXCH};
    if constexpr (TC) tc_init_atab(Ptr<uint32_t>{reinterpret_cast<uint32_t*>(smraw + TC_OFF), kTcAtabWords}, split, tid, NT);
    cf32 v[TL::E];
    if (valid) {
#pragma unroll
      for (int j = 0; j < TL::E; ++j) v[j] = conj_if(ldcs(in, t + TL::T * j), sgn);
    } else {
#pragma unroll
      for (int j = 0; j < TL::E; ++j) v[j] = cf32{0.f, 0.f};
    }
    if constexpr (TC) {
      ESTL_SYNC();  // the DFT matrix table is complete
      run_passes_tc<TL>(v, t, c, sm, tw, Sidx{}, tc_ctx(smraw + TC_OFF, split, tid));
    } else {
      run_passes<TL, 0>(v, t, c, sm, tw, Sidx{});
    }
    if (valid) {
#pragma unroll
      for (int j = 0; j < TL::E; ++j) stcs(out, t + TL::T * j, conj_if(v[j], sgn));
    }
  }

  ESTL_HD static void run(const TileArgs& a, long long cta, int tid, cf32* smraw) {
    const int c = tid >> TL::LOGT;
    const long long row = cta * C + c;
    const bool valid = row < a.rows;
    const long long base = valid ? xbase(a, row, TL::M) : 0;
    const Ptr<const cf32> in = valid ? a.in.sub(base, TL::M) : Ptr<const cf32>{a.in.p, 0};
    const Ptr<cf32> out = valid ? a.out.sub(base, TL::M) : Ptr<cf32>{a.out.p, 0};
    body(in, out, valid, tid, smraw, a.bank, a.sgn, a.split);
  }
};

// Four-step twiddle of a column tile's outputs: y[k2] *= w_N^{n1 k2} for the
// thread's outputs k2 = t + T*j (T = TL::T).  w_N^{n1 k2} = w_N^{n1 t} * W^j
// with W = w_N^{n1 T} = w_{E N1}^{n1}: one two-level table lookup for the
// base, four for W, W^2, W^4, W^8, and the other powers by products (instead
// of a scattered two-level lookup per element).
template <class TL>
ESTL_HD void fourstep_twiddle(cf32 (&v)[TL::E], int n1, int t, int logn, const Ptr<const cf32>& bank) {
  static_assert(TL::E == 16 || TL::E == 32, "column tiles hold 16 or 32 elements per thread");
  const int logw = TL::LE + logn - TL::LM;  // W = w_{E N1}^{n1}, N1 = N / M
  const cf32 base = twiddle_n(bank, logn, n1 * t);
  const cf32 w1 = twiddle_n(bank, logw, n1), w2 = twiddle_n(bank, logw, 2 * n1);
  const cf32 w4 = twiddle_n(bank, logw, 4 * n1), w8 = twiddle_n(bank, logw, 8 * n1);
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = cmul(v[j], base);
  apply_powers16(v, w1, w2, w4, w8);
  if constexpr (TL::E == 32) {
    const cf32 base16 = cmul(base, twiddle_n(bank, logw, 16 * n1));
#pragma unroll
    for (int j = 16; j < 32; ++j) v[j] = cmul(v[j], base16);
    apply_powers16(v + 16, w1, w2, w4, w8);
  }
}

// Four-step column pass: N = N1 * N2, x[n1 + N1 n2].  A CTA owns C adjacent
// columns n1 of one transform and runs their N2-point DFTs (M = N2), then
// multiplies by w_N^{n1 k2} and writes S[k2 * N1 + n1].  Thread mapping is
// column-fastest so both the loads and the stores move runs of C elements.
// TW = false: the plain strided column FFT of a 2D transform (no four-step
// twiddle, conjugated store of the inverse), in place on a [rows][N1] array.
template <int LOGM, int LOGE, int LOGR, int LOGC, bool TC = false, bool TW = true>
struct ColKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  static constexpr int EXCH = (TL::P > 1 || TC) ? TL::MP * C : 0;
  static constexpr int TC_OFF = (EXCH + 1) & ~1;
  static constexpr int SMEM_ELEMS = TC ? TC_OFF + (int)((tc_area_words(NT / 32) + 1) / 2) : EXCH;
  static constexpr int MIN_BLOCKS = TC ? (NT <= 256 ? 2 : 1) : min_blocks(NT, TL::E);
  static_assert(NT <= 1024, "too many threads");
  static_assert(!TC || NT % 32 == 0, "tensor-core tiles run whole warps");

  struct Sidx {
    ESTL_HD int operator()(int c, int m) const { return TL::pad(m) * C + c; }
  };

  // Columns n1_0 .. n1_0 + C - 1 of one transform: in = the transform
  // (N elements), out = its scratch (N elements, S[k2*N1 + n1]).
  ESTL_HD static void body(const Ptr<const cf32>& in, const Ptr<cf32>& out, int n1_0, int logn, int tid,
                           cf32* smraw, const Ptr<const cf32>& bank, float sgn, int split = SPLIT_NONE,
                           int ologr = 0) {
    const int c = tid & (C - 1);
    const int t = tid >> LOGC;
    const int logn1 = logn - LOGM;
    const int n1 = n1_0 + c;
    const Ptr<const cf32> tw = bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, EXCH};
    if constexpr (TC) tc_init_atab(Ptr<uint32_t>{reinterpret_cast<uint32_t*>(smraw + TC_OFF), kTcAtabWords}, split, tid, NT);
    cf32 v[TL::E];
    {
      const int step = TL::T << logn1;
      int off = n1 + (t << logn1);
#pragma unroll
      for (int j = 0; j < TL::E; ++j, off += step) v[j] = conj_if(ldcs(in, off), sgn);
    }
    if constexpr (TC) {
      ESTL_SYNC();  // the DFT matrix table is complete
      run_passes_tc<TL>(v, t, c, sm, tw, Sidx{}, tc_ctx(smraw + TC_OFF, split, tid));
    } else {
      run_passes<TL, 0>(v, t, c, sm, tw, Sidx{});
    }
    if constexpr (TW) {
      store_twiddled(v, out, n1, t, logn, bank, ologr);
    } else {
#pragma unroll
      for (int j = 0; j < TL::E; ++j) out[((t + TL::T * j) << logn1) + n1] = conj_if(v[j], sgn);
    }
  }

  // Four-step twiddle and store: S[k2 * N1 + n1] = y[k2] * w_N^{n1 k2} for
  // the thread's outputs k2 = t + T*j.  w_N^{n1 k2} = w_N^{n1 t} * W^j with
  // W = w_N^{n1 T} = w_{E N1}^{n1}: one two-level table lookup for the base,
  // four for W, W^2, W^4, W^8, and the other powers by products (instead of a
  // scattered two-level lookup per element).
  ESTL_HD static void store_twiddled(cf32 (&v)[TL::E], const Ptr<cf32>& out, int n1, int t, int logn,
                                     const Ptr<const cf32>& bank, int ologr = 0) {
    const int logn1 = logn - LOGM;
    fourstep_twiddle<TL>(v, n1, t, logn, bank);
    const int oshift = logn1 + ologr;  // output row pitch: N1, or 2^ologr N1 (three-pass middle pass)
#pragma unroll
    for (int j = 0; j < TL::E; ++j) out[((t + TL::T * j) << oshift) + n1] = v[j];
  }

  // Output of transform f of the step: its own N elements, or (three-pass
  // middle pass, ologr > 0) rows interleaved 2^ologr apart with transform
  // f = b 2^ologr + k3 starting at b N 2^ologr + k3 N1.
  ESTL_HD static Ptr<cf32> out_of(const Ptr<cf32>& out, long long f, int logn, int ologr) {
    const long long N = 1LL << logn;
    if (!ologr) return out.sub(f * N, N);
    const long long r = f & ((1LL << ologr) - 1);
    const long long off = ((f >> ologr) << (logn + ologr)) + (r << (logn - LOGM));
    return out.sub(off, (N << ologr) - (r << (logn - LOGM)));
  }

  ESTL_HD static void run(const TileArgs& a, long long cta, int tid, cf32* smraw) {
    const int logn1 = a.logn - LOGM;
    const int N = 1 << a.logn;
    const int nblk = (1 << logn1) >> LOGC;
    const long long f = cta / nblk;
    const int n1_0 = (int)(cta - f * nblk) * C;
    body(a.in.sub(xbase(a, f, N), N), out_of(a.out, f, a.logn, a.ologr), n1_0, a.logn, tid, smraw, a.bank, a.sgn, a.split,
         a.ologr);
  }
};

// Four-step row pass: reads S[k2 * N1 + n1] (C contiguous rows of N1 = M),
// runs the N1-point DFTs and writes X[k2 + N2 k1].  Threads are mapped
// column-fastest (c = tid mod C), as in the column pass: a warp loads C runs
// of 32/C consecutive row elements and stores runs of C consecutive outputs
// (X[k2_0 .. k2_0 + C - 1 + N2 k1]) straight from registers, with the tile
// exchanged through shared memory laid out [m][c].
template <int LOGM, int LOGE, int LOGR, int LOGC, bool TC = false>
struct RowKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  static constexpr int EXCH = (TL::P > 1 || TC) ? TL::MP * C : 0;
  static constexpr int TC_OFF = (EXCH + 1) & ~1;
  static constexpr int SMEM_ELEMS = TC ? TC_OFF + (int)((tc_area_words(NT / 32) + 1) / 2) : EXCH;
  static constexpr int MIN_BLOCKS = TC ? (NT <= 256 ? 2 : 1) : min_blocks(NT, TL::E);
  static_assert(NT <= 1024, "too many threads");
  static_assert(!TC || NT % 32 == 0, "tensor-core tiles run whole warps");

  struct Sidx {
    ESTL_HD int operator()(int c, int m) const { return TL::pad(m) * C + c; }
  };

  // Rows k2_0 .. k2_0 + C - 1 of one transform's scratch `in` (N elements)
  // -> the transform's output `out` (N elements, X[k2 + N2 k1]).
  ESTL_HD static void body(const Ptr<cf32>& in, const Ptr<cf32>& out, int k2_0, int logn, int tid, cf32* smraw,
                           const Ptr<const cf32>& bank, float sgn, int split = SPLIT_NONE) {
    const int c = tid & (C - 1);
    const int t = tid >> LOGC;
    const int logn2 = logn - LOGM;
    const Ptr<const cf32> tw = bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, EXCH};
    if constexpr (TC) tc_init_atab(Ptr<uint32_t>{reinterpret_cast<uint32_t*>(smraw + TC_OFF), kTcAtabWords}, split, tid, NT);
    cf32 v[TL::E];
    const Ptr<cf32> row = in.sub((long long)(k2_0 + c) * TL::M, TL::M);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) v[j] = ldcg(row, t + TL::T * j);
    if constexpr (TC) {
      ESTL_SYNC();  // the DFT matrix table is complete
      run_passes_tc<TL>(v, t, c, sm, tw, Sidx{}, tc_ctx(smraw + TC_OFF, split, tid));
    } else {
      run_passes<TL, 0>(v, t, c, sm, tw, Sidx{});
    }
#pragma unroll
    for (int j = 0; j < TL::E; ++j) stcs(out, k2_0 + c + ((t + TL::T * j) << logn2), conj_if(v[j], sgn));
  }

  ESTL_HD static void run(const TileArgs& a, long long cta, int tid, cf32* smraw) {
    const int N = 1 << a.logn;
    const int logn2 = a.logn - LOGM;
    const int nblk = 1 << (logn2 - LOGC);
    const long long f = cta / nblk;
    const int k2_0 = (int)(cta - f * nblk) * C;
    // the scratch written by the column pass is read-only here
    const Ptr<cf32> in{const_cast<cf32*>(a.in.p) + f * N, N};
    ESTL_CHECK(f * N + N, a.in.n + 1, "row pass input range");
    body(in, a.out.sub(xbase(a, f, N), N), k2_0, a.logn, tid, smraw, a.bank, a.sgn, a.split);
  }
};

// Four-step row pass for tiles of many rows (the persistent kernels, whose
// row and column tiles share one thread count): threads are mapped row-fastest
// (unit-stride loads of whole rows), and the results are staged in shared
// memory and stored column-fastest so that every store moves a run of C
// elements.  The C <= 8 tiles of the two-launch four-step use RowKernel.
template <int LOGM, int LOGE, int LOGR, int LOGC>
struct RemapRowKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  static constexpr int CS = row_stride(TL::MP, C);
  static constexpr int SMEM_ELEMS = C * CS;
  static constexpr int MIN_BLOCKS = min_blocks(NT, TL::E);
  static_assert(NT <= 1024, "too many threads");
  static_assert(NT % C == 0 && (NT / C) * TL::E >= TL::M, "store remap must cover the tile");

  struct Sidx {
    ESTL_HD int operator()(int c, int m) const { return c * CS + TL::pad(m); }
  };

  // Rows k2_0 .. k2_0 + C - 1 of one transform's scratch `in` (N elements)
  // -> the transform's output `out` (N elements, X[k2 + N2 k1]).
  ESTL_HD static void body(const Ptr<cf32>& in, const Ptr<cf32>& out, int k2_0, int logn, int tid, cf32* smraw,
                           const Ptr<const cf32>& bank, float sgn) {
    const int t = tid & (TL::T - 1);
    const int c = tid >> TL::LOGT;
    const int logn2 = logn - LOGM;
    const Ptr<const cf32> tw = bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, SMEM_ELEMS};
    const Sidx sidx{};
    cf32 v[TL::E];
    const Ptr<cf32> row = in.sub((long long)(k2_0 + c) * TL::M, TL::M);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) v[j] = ldcg(row, t + TL::T * j);
    run_passes<TL, 0>(v, t, c, sm, tw, sidx);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) sm[sidx(c, t + TL::T * j)] = v[j];
    ESTL_SYNC();
    const int c2 = tid & (C - 1);
    const int t2 = tid >> LOGC;
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const int k1 = t2 + TL::T * j;
      stcs(out, k2_0 + c2 + (k1 << logn2), conj_if(sm[sidx(c2, k1)], sgn));
    }
  }
};

}  // namespace estl
