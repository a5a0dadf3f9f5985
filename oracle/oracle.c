/* oracle.c — TEST INFRASTRUCTURE ONLY (the tests' reference results, never
 * the product).
 *
 * CPU FP64 restatement of the transform the reference's CPU backend computes:
 *   FFT_FFTW3.h:23-31  fftwf_plan_many_dft(rank 1, n = size, howmany = batch,
 *                      stride 1, dist = size, out-of-place, interleaved complex,
 *                      FFTW_FORWARD = exp(-2 pi i jk/N) / FFTW_BACKWARD = exp(+2 pi i jk/N),
 *                      unnormalised in both directions)
 *   FFT.h:32-33        flattened element index batch*size + index
 *   DataInterface.h:37-45 + Complex.h:177-180  interleaved (re, im) layout
 * FFTW 3 itself (the reference links -lfftw3f, ESTL.pro:10, version not pinned)
 * is not available here; its published definition of the DFT is restated.
 *
 * Pinned by: the known-answer test of tests/Test.cpp:60-77 (cosine -> two
 * spikes of M/2, forward sign), a long-double direct DFT (oracle_dft_ld) and
 * numpy.fft (tests/test_oracle.py).
 *
 * Also here: linear convolution by FFT and directly (Convolution.h:95-148
 * restated in 1D), used to check the CUDA convolution path.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

typedef struct {
  double re, im;
} c64;

/* ---- twiddle tables w_N^j = exp(-2 pi i j / N), j < N/2, cached per log2 N ---- */
static c64* g_tw[40];
static pthread_mutex_t g_tw_lock = PTHREAD_MUTEX_INITIALIZER;

static int ilog2_exact(int64_t n) {
  int l = 0;
  while (((int64_t)1 << l) < n) l++;
  return (((int64_t)1 << l) == n) ? l : -1;
}

/* cos/sin of 2 pi j / N from the first octant only, so every table entry
 * carries the error of one libm call on an argument in [0, pi/4]. */
static void octant_cs(int64_t j, int64_t n, double* c, double* s) {
  int64_t q = n / 8;
  if (n < 8) {
    double a = 2.0 * M_PI * (double)j / (double)n;
    *c = cos(a);
    *s = sin(a);
    if (4 * j == n) *c = 0.0;
    if (2 * j == n) *s = 0.0;
    return;
  }
  if (j <= q) {
    double a = 2.0 * M_PI * (double)j / (double)n;
    *c = cos(a);
    *s = sin(a);
  } else if (j <= 2 * q) {
    double a = 2.0 * M_PI * (double)(2 * q - j) / (double)n;
    *c = sin(a);
    *s = cos(a);
  } else if (j <= 3 * q) {
    double a = 2.0 * M_PI * (double)(j - 2 * q) / (double)n;
    *c = -sin(a);
    *s = cos(a);
  } else {
    double a = 2.0 * M_PI * (double)(4 * q - j) / (double)n;
    *c = -cos(a);
    *s = sin(a);
  }
}

static const c64* twiddles(int logn) {
  pthread_mutex_lock(&g_tw_lock);
  if (!g_tw[logn]) {
    int64_t n = (int64_t)1 << logn, h = n / 2 > 0 ? n / 2 : 1;
    c64* t = (c64*)malloc(sizeof(c64) * (size_t)h);
    for (int64_t j = 0; j < h; j++) {
      double c, s;
      octant_cs(j, n, &c, &s);
      t[j].re = c;
      t[j].im = -s;
    }
    g_tw[logn] = t;
  }
  const c64* r = g_tw[logn];
  pthread_mutex_unlock(&g_tw_lock);
  return r;
}

/* One radix-2 Stockham FFT (natural order in and out).  sign = -1 forward,
 * +1 backward.  x is overwritten with the result; w is work space of n. */
static void fft1(c64* x, c64* w, int logn, int sign) {
  int64_t n = (int64_t)1 << logn, h = n / 2;
  const c64* tw = twiddles(logn);
  c64 *src = x, *dst = w;
  for (int64_t ns = 1; ns < n; ns *= 2) {
    int64_t step = n / (2 * ns);
    for (int64_t j = 0; j < h; j++) {
      int64_t k = j & (ns - 1);
      c64 wk = tw[k * step];
      if (sign > 0) wk.im = -wk.im;
      c64 a = src[j], b = src[j + h];
      c64 bw = {b.re * wk.re - b.im * wk.im, b.re * wk.im + b.im * wk.re};
      int64_t o = (j - k) * 2 + k;
      dst[o].re = a.re + bw.re;
      dst[o].im = a.im + bw.im;
      dst[o + ns].re = a.re - bw.re;
      dst[o + ns].im = a.im - bw.im;
    }
    c64* t = src;
    src = dst;
    dst = t;
  }
  if (src != x) memcpy(x, src, sizeof(c64) * (size_t)n);
}

typedef struct {
  const double* in;
  double* out;
  int64_t n, b0, b1;
  int logn, sign;
} job_t;

static void* fft_worker(void* arg) {
  job_t* jb = (job_t*)arg;
  c64* w = (c64*)malloc(sizeof(c64) * (size_t)jb->n);
  for (int64_t b = jb->b0; b < jb->b1; b++) {
    c64* o = (c64*)(jb->out + 2 * b * jb->n);
    if ((const double*)o != jb->in + 2 * b * jb->n) memcpy(o, jb->in + 2 * b * jb->n, sizeof(c64) * (size_t)jb->n);
    fft1(o, w, jb->logn, jb->sign);
  }
  free(w);
  return NULL;
}

/* Batched FP64 FFT with the plan semantics of FFT_FFTW3.h:26-28.
 * in/out: interleaved complex128, batch*n elements.  Returns 0, or -1 when n
 * is not a power of two (the reference plan rounds every size up to 2^k,
 * SimpleMath.h:7-11, FFT_OpenCL_Contiguous.h:56). */
int oracle_fft(const double* in, double* out, int64_t n, int64_t batch, int sign, int nthreads) {
  int logn = ilog2_exact(n);
  if (logn < 0 || batch < 0) return -1;
  if (n == 1) {
    memmove(out, in, sizeof(double) * 2 * (size_t)batch);
    return 0;
  }
  if (nthreads < 1) nthreads = 1;
  if (nthreads > batch) nthreads = (int)(batch > 0 ? batch : 1);
  pthread_t th[256];
  job_t jobs[256];
  if (nthreads > 256) nthreads = 256;
  for (int t = 0; t < nthreads; t++) {
    jobs[t].in = in;
    jobs[t].out = out;
    jobs[t].n = n;
    jobs[t].b0 = batch * t / nthreads;
    jobs[t].b1 = batch * (t + 1) / nthreads;
    jobs[t].logn = logn;
    jobs[t].sign = sign;
  }
  if (nthreads == 1) {
    fft_worker(&jobs[0]);
    return 0;
  }
  for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, fft_worker, &jobs[t]);
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  return 0;
}

/* Long-double direct O(n^2) DFT of one transform (independent check of
 * oracle_fft for small n).  The phase index jk mod n is reduced exactly. */
void oracle_dft_ld(const double* in, double* out, int64_t n, int sign) {
  for (int64_t k = 0; k < n; k++) {
    long double sr = 0.0L, si = 0.0L;
    for (int64_t j = 0; j < n; j++) {
      int64_t m = (j * k) % n;
      long double a = 2.0L * 3.14159265358979323846264338327950288L * (long double)m / (long double)n;
      long double c = cosl(a), s = sign * sinl(a);
      long double xr = in[2 * j], xi = in[2 * j + 1];
      sr += xr * c - xi * s;
      si += xr * s + xi * c;
    }
    out[2 * k] = (double)sr;
    out[2 * k + 1] = (double)si;
  }
}

/* Selected bins of the direct DFT of one sequence of any length (the
 * definition FFT_FFTW3.h:26-28 computes, evaluated term by term):
 * out[b] = sum_j x_j exp(sign 2 pi i j k_b / n), O(n) per bin.  The root for
 * bin k is re-seeded every 256 terms from long-double cosl/sinl of the exact
 * integer angle (j k mod n) and stepped in double in between; the sums are
 * compensated (Kahan) doubles.  Error near 1e-14 relative for n up to 2^23,
 * far below the FP32 tolerances it checks, and fast on hosts whose long
 * double is a software type. */
static void kahan_add(double* s, double* c, double v) {
  const double y = v - *c, t = *s + y;
  *c = (t - *s) - y;
  *s = t;
}

void oracle_dft_bins(const double* in, double* out, int64_t n, const int64_t* bins, int64_t nbins, int sign) {
  const long double two_pi = 2.0L * 3.14159265358979323846264338327950288L;
  for (int64_t b = 0; b < nbins; b++) {
    const int64_t k = ((bins[b] % n) + n) % n;
    const long double a1 = two_pi * (long double)k / (long double)n;
    const double c1 = (double)cosl(a1), s1 = (double)(sign * sinl(a1));
    double sr = 0.0, si = 0.0, cr = 0.0, ci = 0.0, wr = 1.0, wi = 0.0;
    for (int64_t j = 0; j < n; j++) {
      if ((j & 255) == 0) {
        const int64_t m = (int64_t)(((__int128)j * k) % n);
        const long double a = two_pi * (long double)m / (long double)n;
        wr = (double)cosl(a);
        wi = (double)(sign * sinl(a));
      }
      const double xr = in[2 * j], xi = in[2 * j + 1];
      kahan_add(&sr, &cr, xr * wr - xi * wi);
      kahan_add(&si, &ci, xr * wi + xi * wr);
      const double t = wr * c1 - wi * s1;
      wi = wr * s1 + wi * c1;
      wr = t;
    }
    out[2 * b] = sr;
    out[2 * b + 1] = si;
  }
}

/* Direct linear convolution (and correlation) of real sequences in long
 * double: out[m] = sum_i a[i] b[m - i], length la + lb - 1. */
void oracle_conv_direct(const double* a, int64_t la, const double* b, int64_t lb, double* out) {
  for (int64_t m = 0; m < la + lb - 1; m++) {
    long double s = 0.0L;
    int64_t i0 = m - (lb - 1) > 0 ? m - (lb - 1) : 0;
    int64_t i1 = m < la - 1 ? m : la - 1;
    for (int64_t i = i0; i <= i1; i++) s += (long double)a[i] * (long double)b[m - i];
    out[m] = (double)s;
  }
}

/* FP64 FFT linear convolution of real sequences: zero-pad both to
 * n = nextPow2(la + lb - 1) (Convolution.h:89-97), forward FFT, pointwise
 * product (Convolution.h:132-136; conj(B) when correlate, :125-130), inverse
 * FFT, scale 1/n, keep the real part of the first la + lb - 1 samples. */
int oracle_conv_circular(const double* a, int64_t la, const double* b, int64_t lb, int64_t n, double* out,
                         int64_t keep, int correlate);

int oracle_conv_fft(const double* a, int64_t la, const double* b, int64_t lb, double* out, int correlate) {
  int64_t len = la + lb - 1, n = 1;
  while (n < len) n *= 2;
  return oracle_conv_circular(a, la, b, lb, n, out, len, correlate);
}

/* The first `keep` samples of the n-point circular convolution (correlation:
 * the product with the conjugate spectrum) of a and b, both zero-padded to n
 * (n >= la, lb), by FP64 FFTs. */
int oracle_conv_circular(const double* a, int64_t la, const double* b, int64_t lb, int64_t n, double* out,
                         int64_t keep, int correlate) {
  const int64_t len = keep;
  if (n < la || n < lb || keep > n) return 1;
  c64* A = (c64*)calloc((size_t)n, sizeof(c64));
  c64* B = (c64*)calloc((size_t)n, sizeof(c64));
  for (int64_t i = 0; i < la; i++) A[i].re = a[i];
  for (int64_t i = 0; i < lb; i++) B[i].re = b[i];
  oracle_fft((double*)A, (double*)A, n, 1, -1, 1);
  oracle_fft((double*)B, (double*)B, n, 1, -1, 1);
  for (int64_t i = 0; i < n; i++) {
    double br = B[i].re, bi = correlate ? -B[i].im : B[i].im;
    double r = A[i].re * br - A[i].im * bi, im = A[i].re * bi + A[i].im * br;
    A[i].re = r;
    A[i].im = im;
  }
  oracle_fft((double*)A, (double*)A, n, 1, +1, 1);
  for (int64_t i = 0; i < len; i++) out[i] = A[i].re / (double)n;
  free(A);
  free(B);
  return 0;
}

/* 2D FFT of an h x w complex array in place (rows, then columns), FP64. */
static void fft2d(c64* A, int64_t h, int64_t w, int sign) {
  oracle_fft((double*)A, (double*)A, w, h, sign, 1);
  c64* col = (c64*)malloc((size_t)h * sizeof(c64));
  for (int64_t x = 0; x < w; x++) {
    for (int64_t y = 0; y < h; y++) col[y] = A[y * w + x];
    oracle_fft((double*)col, (double*)col, h, 1, sign, 1);
    for (int64_t y = 0; y < h; y++) A[y * w + x] = col[y];
  }
  free(col);
}

/* 2D FFT convolution of a real h x w image with a real kh x kw kernel, after
 * Convolution2D_FFT::convolve (Convolution.h:95-148), in FP64.  Both padded to
 * W x H = nextPow2(w + kw - 1) x nextPow2(h + kh - 1) (:96-97), 2D FFTs,
 * product (with conj of the kernel spectrum when correlate, :125-137),
 * inverse 2D FFT.
 *   compat = 0: the kernel at the origin, result / (W H), the full linear
 *               convolution (h + kh - 1) x (w + kw - 1) kept;
 *   compat = 1: the reference's own steps: kernel read from
 *               ((x + (kw+1)/2) mod W, (y + (kh+1)/2) mod H) (:113-120),
 *               result / (W H K^[0]) (:141-143), h x w kept (:146-148). */
int oracle_conv2d_fft(const double* a, int64_t h, int64_t w, const double* k, int64_t kh, int64_t kw, double* out,
                      int correlate, int compat) {
  int64_t W = 1, H = 1;
  while (W < w + kw - 1) W *= 2;
  while (H < h + kh - 1) H *= 2;
  c64* A = (c64*)calloc((size_t)(W * H), sizeof(c64));
  c64* K = (c64*)calloc((size_t)(W * H), sizeof(c64));
  for (int64_t y = 0; y < h; y++)
    for (int64_t x = 0; x < w; x++) A[y * W + x].re = a[y * w + x];
  const int64_t xo = compat ? (kw + 1) / 2 : 0, yo = compat ? (kh + 1) / 2 : 0;
  for (int64_t y = 0; y < H; y++) {
    const int64_t sy = (y + yo) % H;
    for (int64_t x = 0; x < W; x++) {
      const int64_t sx = (x + xo) % W;
      if (sx < kw && sy < kh) K[y * W + x].re = k[sy * kw + sx];
    }
  }
  fft2d(A, H, W, -1);
  fft2d(K, H, W, -1);
  const double k0 = K[0].re;
  for (int64_t i = 0; i < W * H; i++) {
    double br = K[i].re, bi = correlate ? -K[i].im : K[i].im;
    double r = A[i].re * br - A[i].im * bi, im = A[i].re * bi + A[i].im * br;
    A[i].re = r;
    A[i].im = im;
  }
  fft2d(A, H, W, +1);
  const double scale = 1.0 / ((double)W * (double)H * (compat ? k0 : 1.0));
  const int64_t ow = compat ? w : w + kw - 1, oh = compat ? h : h + kh - 1;
  for (int64_t y = 0; y < oh; y++)
    for (int64_t x = 0; x < ow; x++) out[y * ow + x] = A[y * W + x].re * scale;
  free(A);
  free(K);
  return 0;
}

/* Direct 2D linear convolution in long double:
 * out[y][x] = sum_{r,q} a[y - r][x - q] k[r][q], (h + kh - 1) x (w + kw - 1). */
void oracle_conv2d_direct(const double* a, int64_t h, int64_t w, const double* k, int64_t kh, int64_t kw,
                          double* out) {
  const int64_t ow = w + kw - 1, oh = h + kh - 1;
  for (int64_t y = 0; y < oh; y++)
    for (int64_t x = 0; x < ow; x++) {
      long double s = 0.0L;
      for (int64_t r = 0; r < kh; r++) {
        const int64_t ya = y - r;
        if (ya < 0 || ya >= h) continue;
        for (int64_t q = 0; q < kw; q++) {
          const int64_t xa = x - q;
          if (xa < 0 || xa >= w) continue;
          s += (long double)a[ya * w + xa] * (long double)k[r * kw + q];
        }
      }
      out[y * ow + x] = (double)s;
    }
}
