// Driver for Convolution2D_FFT_CUDA<float> (include/Convolution2D_CUDA.h):
// images and kernels behind ESTL's Data2D<T> interface, convolve() and
// convolve(true), each pixel against the reference's steps (Convolution.h:
// 95-148) restated directly in double: zero padding to powers of two, the
// cyclically centred kernel, circular convolution (or correlation) as direct
// sums, division by K^[0] = the sum of the padded kernel, crop.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "Convolution2D_CUDA.h"

class Image : public Data2D<float> {
 public:
  Image(int w, int h) : w_(w), h_(h), px_((size_t)w * h, 0.f) {}
  int getWidth() { return w_; }
  int getHeight() { return h_; }
  float getPixel(int x, int y) { return px_[(size_t)y * w_ + x]; }
  void setPixel(int x, int y, float v) { px_[(size_t)y * w_ + x] = v; }

 private:
  int w_, h_;
  std::vector<float> px_;
};

static int next_pow2(int n) {
  int r = 1;
  while (r < n) r *= 2;
  return r;
}

// the reference's result by direct circular sums over the padded W x H arrays
static std::vector<double> reference(Image& a, Image& k, bool correlate) {
  const int w = a.getWidth(), h = a.getHeight(), kw = k.getWidth(), kh = k.getHeight();
  const int W = next_pow2(w + kw - 1), H = next_pow2(h + kh - 1);
  const int xo = (kw + 1) / 2, yo = (kh + 1) / 2;
  std::vector<double> K((size_t)W * H, 0.0);
  double k0 = 0.0;
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const int sx = (x + xo) % W, sy = (y + yo) % H;
      if (sx < kw && sy < kh) K[(size_t)y * W + x] = k.getPixel(sx, sy);
      k0 += K[(size_t)y * W + x];
    }
  std::vector<double> out((size_t)w * h, 0.0);
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      double s = 0.0;
      for (int my = 0; my < h; ++my)
        for (int mx = 0; mx < w; ++mx) {
          // convolution: K[(p - m) mod]; correlation (conj of the spectrum): K[(m - p) mod]
          const int dx = correlate ? ((mx - x) % W + W) % W : ((x - mx) % W + W) % W;
          const int dy = correlate ? ((my - y) % H + H) % H : ((y - my) % H + H) % H;
          s += (double)a.getPixel(mx, my) * K[(size_t)dy * W + dx];
        }
      out[(size_t)y * w + x] = s / k0;
    }
  return out;
}

static int check(int w, int h, int kw, int kh, bool correlate, unsigned seed) {
  Image a(w, h), k(kw, kh), r(w, h);
  srand(seed);
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) a.setPixel(x, y, (float)rand() / RAND_MAX - 0.5f);
  for (int y = 0; y < kh; ++y)
    for (int x = 0; x < kw; ++x) k.setPixel(x, y, 0.1f + (float)rand() / RAND_MAX);
  Convolution2D_FFT_CUDA<float> conv(&a, &k, &r);
  conv.convolve(correlate);
  std::vector<double> ref = reference(a, k, correlate);
  double num = 0.0, den = 0.0;
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const double d = r.getPixel(x, y) - ref[(size_t)y * w + x];
      num += d * d;
      den += ref[(size_t)y * w + x] * ref[(size_t)y * w + x];
    }
  const double rel = sqrt(num / den);
  printf("%dx%d * %dx%d %s: rel-L2 %.3g\n", w, h, kw, kh, correlate ? "correlate" : "convolve", rel);
  return rel < 1e-6 ? 0 : 1;
}

int main() {
  int failures = 0;
  try {
    failures += check(37, 29, 5, 4, false, 1);
    failures += check(37, 29, 5, 4, true, 2);
    failures += check(64, 20, 9, 9, false, 3);
    failures += check(13, 50, 1, 7, true, 4);
  } catch (std::exception& e) {
    printf("exception: %s\n", e.what());
    return 2;
  }
  printf("%s (%d failures)\n", failures ? "FAILED" : "PASSED", failures);
  return failures ? 1 : 0;
}
