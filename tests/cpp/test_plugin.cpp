// test_plugin.cpp — the reference's test driver semantics (tests/Test.cpp)
// run on the FFT_CUDA<float> plugin through ESTL's factory API.
//
//  * known-answer sweep (Test.cpp:45-110): batch B = 2^b, size M = 2^m, input
//    cos(2 pi effK q / M), expected M/2 spikes at effK and M - effK, failure if
//    |d|^2 > MAX_ERR * M; GFlop/s with the 5 M log2 M convention (:80) and the
//    per-kernel breakdown read through dynamic_cast<GpuAlgorithm*> (:86-99);
//  * FFT2D through the factory (Test.cpp:113-184) checked against a direct 2D
//    DFT with the cross-backend tolerance MAX_ERR * Mx * My (:147);
//  * backward transforms of every transform in a batch (the reference's
//    contiguous backend conjugates only batch 0, FFT_OpenCL_Contiguous.h:100-102).
//
// Build: g++ -std=c++17 -O2 -I include -I <ESTL headers> test_plugin.cpp -lestl_cuda
#include <math.h>
#include <stdio.h>

#include <chrono>
#include <exception>
#include <string>
#include <vector>

#include "FFT.h"
#include "FFT_CUDA.h"

#define MAX_ERR 1E-3

typedef float D;
typedef Complex<D> C;

static int failures = 0;

static void check_close(C a, C b, double factor, const char* what) {
  C d = a - b;
  if (d.getNormSquared() > MAX_ERR * factor) {
    if (failures < 10) printf("FAIL %s: %s != %s\n", what, a.toString().c_str(), b.toString().c_str());
    failures++;
  }
}

static double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static void known_answer_sweep(FFTFactory<D>* f, int max_b, int max_m) {
  for (int b = 0; b <= max_b; ++b) {
    int B = 1 << b;
    for (int m = 1; m <= max_m; ++m) {
      int M = 1 << m;
      if (B > f->getMaxBatchSize(M)) continue;
      FFT<D>* fft = f->newFFT(M, true, B);
      EstlHostTimer comp;
      GpuAlgorithm* gpu = dynamic_cast<GpuAlgorithm*>(fft);
      if (gpu) gpu->timerComputation = &comp;
      double t_total = 0;
      int runs = 0;
      for (int k = 1; 2 * k < M && k < 4; ++k) {
        for (int bIx = 0; bIx < B; ++bIx) {
          int effK = ((k + bIx) % (M / 2 - 1)) + 1;
          for (int q = 0; q < M; q++) fft->setData(q + bIx * M, (D)cos(2 * M_PI * ((1.0 * effK * q) / M)));
        }
        double t0 = now();
        fft->execute();
        t_total += now() - t0;
        runs++;
        for (int bIx = 0; bIx < B; ++bIx) {
          int effK = ((k + bIx) % (M / 2 - 1)) + 1;
          for (int q = 0; q < M; q++) {
            C c = ((q == effK) || (q == M - effK)) ? C((D)(M / 2.0)) : C((D)0.0);
            check_close(fft->getData(q + bIx * M), c, M, "known answer");
          }
        }
      }
      if (runs) {
        double flops = 5.0 * m * (1 << m) * B;
        printf("[%i] %s m == %i: %.2f Gfs (%.2f Gfs device)", b, f->getName().c_str(), m, 1e-9 * flops / (t_total / runs),
               comp.getRuns() ? 1e-9 * flops / comp.getAverageTime() : -1.0);
        if (gpu)
          for (size_t q = 0; q < gpu->kernelTimers.size(); ++q)
            printf("  [K%zu %s: %.2f Gfs]", q + 1, gpu->getKernelInfo((int)q).c_str(),
                   1e-9 * gpu->getTotalComputationFlops((int)q) / gpu->kernelTimers[q].getAverageTime());
        printf("\n");
      }
      delete fft;
    }
  }
}

static void fft2d_against_direct(FFTFactory<D>* f, int mx, int my) {
  int X = 1 << mx, Y = 1 << my;
  FFT2D<D>* tp = f ? new FFT2D<D>(X, Y, f) : new FFT2D_CUDA<D>(X, Y);
  FFT2D<D>& t = *tp;
  std::vector<C> in((size_t)X * Y);
  unsigned s = 12345;
  for (int q = 0; q < X * Y; ++q) {
    s = s * 1103515245u + 12345u;
    D re = (D)((s >> 8) & 0xffff) / 65536.0f - 0.5f;
    s = s * 1103515245u + 12345u;
    D im = (D)((s >> 8) & 0xffff) / 65536.0f - 0.5f;
    in[q] = C(re, im);
    t.data[q] = in[q];
  }
  t.execute();
  for (int ky = 0; ky < Y; ++ky)
    for (int kx = 0; kx < X; ++kx) {
      double sr = 0, si = 0;
      for (int y = 0; y < Y; ++y)
        for (int x = 0; x < X; ++x) {
          double a = -2 * M_PI * ((double)kx * x / X + (double)ky * y / Y);
          C v = in[(size_t)y * X + x];
          sr += v.getReal() * cos(a) - v.getImaginary() * sin(a);
          si += v.getReal() * sin(a) + v.getImaginary() * cos(a);
        }
      check_close(t.data[(size_t)ky * X + kx], C((D)sr, (D)si), (double)X * Y, "2D");
    }
  printf("%s %dx%d checked against a direct DFT\n", f ? "FFT2D" : "FFT2D_CUDA", X, Y);
  delete tp;
}

static void backward_every_batch(FFTFactory<D>* f, int m, int B) {
  int M = 1 << m;
  FFT<D>* fwd = f->newFFT(M, true, B);
  FFT<D>* bwd = f->newFFT(M, false, B);
  std::vector<C> x((size_t)M * B);
  for (int i = 0; i < M * B; ++i) x[i] = C((D)sin(0.37 * i), (D)cos(0.11 * i * i));
  for (int i = 0; i < M * B; ++i) fwd->setData(i, x[i]);
  fwd->execute();
  for (int i = 0; i < M * B; ++i) bwd->setData(i, fwd->getData(i));
  bwd->execute();
  for (int i = 0; i < M * B; ++i) {
    C r = bwd->getData(i);
    check_close(C(r.getReal() / M, r.getImaginary() / M), x[i], 1.0, "round trip");
  }
  printf("backward round trip M=%d B=%d checked for every transform\n", M, B);
  delete fwd;
  delete bwd;
}

int main(int argc, char** argv) {
  int max_b = argc > 1 ? atoi(argv[1]) : 4;
  int max_m = argc > 2 ? atoi(argv[2]) : 16;
  std::vector<FFTFactory<D>*> factories;
  factories.push_back(new FFTFactorySpecific<FFT_CUDA<D> >());
  // the FFT_OpenCL_Contiguous host layout (PlannarizedDataInterface, block-planar)
  factories.push_back(new FFTFactorySpecific<FFT_CUDA<D, PlannarizedDataInterface<D> > >());
  try {
    for (size_t i = 0; i < factories.size(); ++i) {
      known_answer_sweep(factories[i], max_b, max_m);
      fft2d_against_direct(factories[i], 3, 4);
      fft2d_against_direct(factories[i], 5, 2);
      backward_every_batch(factories[i], 10, 8);
      backward_every_batch(factories[i], 17, 3);
    }
    fft2d_against_direct(NULL, 3, 4);
    fft2d_against_direct(NULL, 6, 5);
  } catch (std::exception& e) {
    printf("exception: %s\n", e.what());
    return 2;
  }
  for (size_t i = 0; i < factories.size(); ++i) delete factories[i];
  printf("%s (%d failures)\n", failures ? "FAILED" : "PASSED", failures);
  return failures ? 1 : 0;
}
