// conv_exec.h — device execution of a convolution layout (conv.cu), shared
// with the serving loop.
#pragma once
#include <cuda_runtime.h>

#include "conv_plan.h"
#include "engine.h"

namespace estl {

// Device pointers of one convolution batch.
struct ConvBuffers {
  const float* sig;
  long long sig_elems;
  const float* filt;
  long long filt_elems;
  float* out;
  long long out_elems;
  const ConvRow* filt_rows;
  const ConvRow* sig_rows;
  cf32* spec;
  cf32* s1;
  cf32* s2;
};

// which: 1 = spectrum launches, 2 = convolution launches, 3 = both.
estl_status launch_conv(const ConvLayout& L, const ConvBuffers& b, int which, cudaStream_t stream);

// Buffers of a layout whose workspace starts at ws (rows must already be there).
ConvBuffers conv_buffers(const ConvLayout& L, void* ws, const float* sig, long long sig_elems, const float* filt,
                         long long filt_elems, float* out);

}  // namespace estl
