/* Convolution2D_CUDA.h — ESTL's Convolution2D_FFT (Convolution.h:78-154) on
 * the GB300 engine.
 *
 * Convolution2D_FFT_CUDA<T> is a Convolution2D<T> with the constructor of
 * Convolution2D_FFT<T> (data, kernel, result as Data2D<T>*) and the same
 * result: the data zero-padded to powers of two, the kernel read cyclically
 * from ((kw + 1) / 2, (kh + 1) / 2) (:113-120), product of the 2D spectra (or
 * with the conjugate kernel spectrum for correlation, :125-137), divided by
 * W * H * K^[0] (:141-143), the data's width x height written back
 * (:146-148).  The reference runs FFT2D objects with per-row host copies; here
 * one blocking call (estl_conv2d_host) runs the three fused launches.
 *
 * Include after ESTL's Convolution.h (Data2D<T>, Convolution2D<T>).
 */
#ifndef CONVOLUTION2D_CUDA_H
#define CONVOLUTION2D_CUDA_H

#include <vector>

#include "Convolution.h"
#include "FFT_CUDA.h"
#include "estl_cuda.h"

template <class T>
class Convolution2D_FFT_CUDA : public Convolution2D<T> {
 private:
  Data2D<T>*dataToConvolve, *convolutionKernel, *result;

 public:
  bool cyclic[2];

  Convolution2D_FFT_CUDA(Data2D<T>* iDataToConvolve, Data2D<T>* iConvolutionKernel, Data2D<T>* iResult)
      : dataToConvolve(iDataToConvolve), convolutionKernel(iConvolutionKernel), result(iResult) {
    cyclic[0] = cyclic[1] = false;
  }

  virtual void convolve(bool correlate = false) {
    const int w = dataToConvolve->getWidth(), h = dataToConvolve->getHeight();
    const int kw = convolutionKernel->getWidth(), kh = convolutionKernel->getHeight();
    std::vector<float> img((size_t)w * h), ker((size_t)kw * kh), out((size_t)w * h);
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) img[(size_t)y * w + x] = (float)dataToConvolve->getPixel(x, y);
    for (int y = 0; y < kh; ++y)
      for (int x = 0; x < kw; ++x) ker[(size_t)y * kw + x] = (float)convolutionKernel->getPixel(x, y);
    estlCheck(estl_init(0, 0), "estl_init");
    estlCheck(estl_conv2d_host(w, h, kw, kh, ESTL_CONV_REFERENCE_COMPAT | (correlate ? ESTL_CONV_CORRELATE : 0),
                               img.data(), ker.data(), out.data()),
              "estl_conv2d_host");
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) result->setPixel(x, y, (T)out[(size_t)y * w + x]);
  }
};

#endif  // CONVOLUTION2D_CUDA_H
