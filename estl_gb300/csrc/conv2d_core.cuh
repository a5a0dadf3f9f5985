// conv2d_core.cuh — 2D FFT convolution of real images with one real filter,
// shared by the CUDA kernels (conv2d.cu) and the host emulator.
//
// Reference: Convolution2D_FFT::convolve (Convolution.h:95-148): both operands
// zero-padded to Pw x Ph = nextPowerOf2(W + Kw - 1) x nextPowerOf2(H + Kh - 1)
// (:96-97), the filter read cyclically from ((Kw+1)/2, (Kh+1)/2) so that it is
// centred (:113-120), forward FFT2D of both (:122-123), pointwise product (or
// product with the conjugate for correlation, :125-137), inverse FFT2D (:139),
// scaled by 1 / (Pw Ph K^[0]) (:141-143), the first H rows of W pixels kept
// (:146-148).  The reference runs one FFT object per row and per column with
// host copies in between; here a batch of images takes three launches:
//
//   1  row pass      rows y < H of each image: real pixels, zero-padded to
//                    Pw, forward Pw-point FFT -> complex work array [y][x]
//   2  column pass   C adjacent columns of one image: rows y < H (the rest
//                    is zero), forward Ph-point FFT, times the filter
//                    spectrum S (pre-scaled, conjugated for correlation),
//                    conjugate, forward FFT again (= the conjugated inverse
//                    column transform), rows y < out_h stored back in place
//   3  row pass      rows y < out_h: forward Pw-point FFT; the real part is the
//                    inverse 2D transform (Re conj z = Re z), cropped to out_w
//                    pixels and stored as float.
//
// The filter spectrum is made once per filter by passes 1 and 2 in spectrum
// mode.  Default output: the full linear convolution (H + Kh - 1) x
// (W + Kw - 1) scaled by 1 / (Pw Ph); the reference-compatible mode keeps the
// reference's centring, K^[0] normalisation and H x W crop.
#pragma once
#include "fft_core.cuh"

namespace estl {

struct Conv2dArgs {
  Ptr<const float> src;   // pass 1: real images (or the filter), h x w each, row-major
  Ptr<cf32> buf;          // count padded arrays of Ph x Pw complex, row-major (the spectrum in spectrum mode)
  Ptr<const cf32> spec;   // pass 2 (convolution): the filter spectrum, Ph x Pw
  Ptr<float> out;         // pass 3: count outputs of out_h x out_w floats
  Ptr<const cf32> bank;
  long long count;        // images (1 for the filter)
  int logw, logh;         // log2 Pw, log2 Ph
  int w, h;               // source width and height (pass 1)
  int xoff, yoff;         // pass 1: the source is read from ((x + xoff) mod Pw, (y + yoff) mod Ph)
  int in_rows;            // pass 1: rows of each padded array computed; pass 2: rows that may be nonzero
  int out_w, out_h;       // pass 2: rows stored; pass 3: output size
  float scale;            // pass 2, spectrum mode: multiplies the spectrum
  float conj;             // pass 2, spectrum mode: -1 stores conj(S) (correlation)
  int dc_norm;            // pass 3: divide by Pw Ph S[0] (= K^[0] with the stored 1 / (Pw Ph))
  int mode;               // pass 1 / 3 row kernel: 0 real rows in, 1 rows out; pass 2: 0 convolve, 1 spectrum
};

// Row passes: C rows of Pw = M points per CTA, the thread layout of
// SingleKernel (thread t of row c owns positions t + T*j).
template <int LOGM, int LOGE, int LOGR, int LOGC>
struct Conv2dRowKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  static constexpr int CS = row_stride(TL::MP, TL::T >= 16 ? 16 : TL::T * C >= 16 ? 16 / TL::T : C);
  static constexpr int EXCH = (TL::P > 1) ? C * CS : 0;
  static constexpr int SMEM_ELEMS = EXCH;
  static constexpr int MIN_BLOCKS = min_blocks(NT, TL::E);
  static_assert(NT <= 1024, "too many threads");
  struct Sidx {
    ESTL_HD int operator()(int c, int m) const { return c * CS + TL::pad(m); }
  };

  ESTL_HD static long long nrows(const Conv2dArgs& a) { return a.count * (a.mode == 0 ? a.in_rows : a.out_h); }

  ESTL_HD static void run(const Conv2dArgs& a, long long cta, int tid, cf32* smraw) {
    const int t = tid & (TL::T - 1);
    const int c = tid >> TL::LOGT;
    const long long g = cta * C + c;
    const bool valid = g < nrows(a);
    const int rpi = a.mode == 0 ? a.in_rows : a.out_h;  // rows per image
    const long long b = valid ? g / rpi : 0;
    const int y = valid ? (int)(g - b * rpi) : 0;
    const int ph = 1 << a.logh;
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, EXCH};
    const Ptr<cf32> row = valid ? a.buf.sub(((b << a.logh) + y) << LOGM, TL::M) : Ptr<cf32>{a.buf.p, 0};
    cf32 v[TL::E];
    if (a.mode == 0) {
      // padded real row y: source row (y + yoff) mod Ph, pixel (x + xoff) mod Pw
      const int sy = (y + a.yoff) & (ph - 1);
      const bool any = valid && sy < a.h;
      const Ptr<const float> s = any ? a.src.sub((b * a.h + sy) * a.w, a.w) : Ptr<const float>{a.src.p, 0};
#pragma unroll
      for (int j = 0; j < TL::E; ++j) {
        const int sx = (t + TL::T * j + a.xoff) & (TL::M - 1);
        v[j] = cf32{any && sx < a.w ? s[sx] : 0.f, 0.f};
      }
    } else {
#pragma unroll
      for (int j = 0; j < TL::E; ++j) v[j] = valid ? row[t + TL::T * j] : cf32{0.f, 0.f};
    }
    run_passes<TL, 0>(v, t, c, sm, tw, Sidx{});
    if (!valid) return;
    if (a.mode == 0) {
#pragma unroll
      for (int j = 0; j < TL::E; ++j) row[t + TL::T * j] = v[j];
    } else {
      const float gsc = a.dc_norm ? 1.f / ((float)(1 << (a.logw + a.logh)) * ldg(a.spec, 0).x) : 1.f;
      const Ptr<float> o = a.out.sub((b * a.out_h + y) * a.out_w, a.out_w);
#pragma unroll
      for (int j = 0; j < TL::E; ++j) {
        const int x = t + TL::T * j;
        if (x < a.out_w) o[x] = v[j].x * gsc;
      }
    }
  }
};

// Column pass: C adjacent columns of one padded array, column-fastest threads
// (the layout of ColKernel: loads and stores move runs of C elements), in
// place.  The tile reads every row it needs before it stores any.
template <int LOGM, int LOGE, int LOGR, int LOGC>
struct Conv2dColKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  static constexpr int EXCH = (TL::P > 1) ? TL::MP * C : 0;
  static constexpr int SMEM_ELEMS = EXCH;
  static constexpr int MIN_BLOCKS = min_blocks(NT, TL::E);
  static_assert(NT <= 1024, "too many threads");
  struct Sidx {
    ESTL_HD int operator()(int c, int m) const { return TL::pad(m) * C + c; }
  };

  ESTL_HD static long long ntiles(const Conv2dArgs& a) { return a.count << (a.logw - LOGC); }

  ESTL_HD static void run(const Conv2dArgs& a, long long cta, int tid, cf32* smraw) {
    const int c = tid & (C - 1);
    const int t = tid >> LOGC;
    const int nblk = 1 << (a.logw - LOGC);
    const long long b = cta / nblk;
    const int n1 = (int)(cta - b * nblk) * C + c;
    const Ptr<cf32> img = a.buf.sub(b << (a.logw + LOGM), 1LL << (a.logw + LOGM));
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, EXCH};
    cf32 v[TL::E];
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const int m = t + TL::T * j;
      v[j] = m < a.in_rows ? img[(m << a.logw) + n1] : cf32{0.f, 0.f};
    }
    run_passes<TL, 0>(v, t, c, sm, tw, Sidx{});
    if (a.mode == 1) {
#pragma unroll
      for (int j = 0; j < TL::E; ++j)
        img[((t + TL::T * j) << a.logw) + n1] = cf32{v[j].x * a.scale, v[j].y * a.scale * a.conj};
      return;
    }
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const cf32 s = ldg(a.spec, ((t + TL::T * j) << a.logw) + n1);
      const cf32 p = cmul(v[j], s);
      v[j] = cf32{p.x, -p.y};
    }
    run_passes<TL, 0>(v, t, c, sm, tw, Sidx{});
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const int m = t + TL::T * j;
      if (m < a.out_h) img[(m << a.logw) + n1] = v[j];
    }
  }
};

// Geometry of a 2D convolution (shared by the host code and the emulator).
struct Conv2dGeom {
  int logw = 0, logh = 0;  // padded size Pw x Ph
  int out_w = 0, out_h = 0;
  int xoff = 0, yoff = 0;  // filter read offsets (reference-compatible centring)
};

ESTL_CX int conv2d_ceil_log2(long long n) {
  int l = 0;
  while ((1LL << l) < n) ++l;
  return l;
}

// false if the sizes are out of range.
inline bool conv2d_geometry(long long w, long long h, long long kw, long long kh, bool compat, Conv2dGeom* g) {
  if (w < 1 || h < 1 || kw < 1 || kh < 1 || w > (1 << 20) || h > (1 << 20) || kw > (1 << 20) || kh > (1 << 20))
    return false;
  // at least 2 x 2 (the smallest tiles); more zero padding leaves the linear
  // (and the centred) convolution unchanged
  g->logw = conv2d_ceil_log2(w + kw - 1) > 1 ? conv2d_ceil_log2(w + kw - 1) : 1;
  g->logh = conv2d_ceil_log2(h + kh - 1) > 1 ? conv2d_ceil_log2(h + kh - 1) : 1;
  g->out_w = (int)(compat ? w : w + kw - 1);
  g->out_h = (int)(compat ? h : h + kh - 1);
  g->xoff = compat ? (int)((kw + 1) / 2) : 0;
  g->yoff = compat ? (int)((kh + 1) / 2) : 0;
  return true;
}

// Padded sizes the tiles cover: rows of at most 2^14 points (one row tile),
// columns of at most 2^12 (one column tile), at most 2^26 points.
inline bool conv2d_supported(const Conv2dGeom& g) { return g.logw <= 14 && g.logh <= 12 && g.logw + g.logh <= 26; }

// CTAs of a row (col = false) or column launch with 2^logc rows / columns per CTA.
inline long long conv2d_grid(bool col, int logc, const Conv2dArgs& a) {
  if (col) return a.count << (a.logw - logc);
  return (a.count * (a.mode == 0 ? a.in_rows : a.out_h) + (1LL << logc) - 1) >> logc;
}

// Arguments of the filter-spectrum passes: the row pass (mode 0) then the
// column pass (mode 1, in place on `spec`), spectrum scaled by 1 / (Pw Ph).
inline Conv2dArgs conv2d_filter_args(const Conv2dGeom& g, long long kw, long long kh, int compat, int correlate,
                                     const float* filt, cf32* spec, const cf32* bank, long long bank_n) {
  const long long pts = 1LL << (g.logw + g.logh);
  Conv2dArgs a{};
  a.src = Ptr<const float>{filt, kw * kh};
  a.buf = Ptr<cf32>{spec, pts};
  a.spec = Ptr<const cf32>{spec, pts};
  a.out = Ptr<float>{nullptr, 0};
  a.bank = Ptr<const cf32>{bank, bank_n};
  a.count = 1;
  a.logw = g.logw;
  a.logh = g.logh;
  a.w = (int)kw;
  a.h = (int)kh;
  a.xoff = g.xoff;
  a.yoff = g.yoff;
  // with a centring offset every padded row can hold filter taps
  a.in_rows = compat ? (1 << g.logh) : (int)kh;
  a.out_w = 1 << g.logw;
  a.out_h = 1 << g.logh;
  a.scale = 1.f / (float)pts;
  a.conj = correlate ? -1.f : 1.f;
  a.mode = 0;
  return a;
}

// Arguments of the convolution passes: row pass (mode 0), column pass
// (mode 0), row pass (mode 1).
inline Conv2dArgs conv2d_exec_args(const Conv2dGeom& g, long long w, long long h, long long count, int compat,
                                   const float* images, cf32* work, const cf32* spec, float* out, const cf32* bank,
                                   long long bank_n) {
  const long long pts = 1LL << (g.logw + g.logh);
  Conv2dArgs a{};
  a.src = Ptr<const float>{images, count * w * h};
  a.buf = Ptr<cf32>{work, count * pts};
  a.spec = Ptr<const cf32>{spec, pts};
  a.out = Ptr<float>{out, count * (long long)g.out_w * g.out_h};
  a.bank = Ptr<const cf32>{bank, bank_n};
  a.count = count;
  a.logw = g.logw;
  a.logh = g.logh;
  a.w = (int)w;
  a.h = (int)h;
  a.in_rows = (int)h;
  a.out_w = g.out_w;
  a.out_h = g.out_h;
  a.dc_norm = compat ? 1 : 0;
  a.mode = 0;
  return a;
}

}  // namespace estl
