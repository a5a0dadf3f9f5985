// engine.h — internal state shared by the C-ABI translation units:
// device selection, the HBM budget accounting allocator, the twiddle bank,
// kernel lookup and the plan executor.
//
// Replaces the reference's OpenCL runtime wrapper (uOpenCL.h:275-348:
// context, queue, buffers, profiling) with the CUDA runtime: streams and
// events instead of a profiling queue, a budgeted device allocator instead of
// per-object clCreateBuffer.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <mutex>
#include <string>

#include "../../include/estl_cuda.h"
#include "fft_core.cuh"
#include "packed_plan.h"
#include "planner.h"

namespace estl {

struct Engine {
  std::mutex mu;
  bool inited = false;
  int device = -1;
  size_t budget = 0;
  std::atomic<size_t> used{0};
  cf32* bank = nullptr;  // twiddle bank, kBankSize entries
  long long* dev_err = nullptr;  // bulk-load kernels' wait-timeout word (TileArgs::err)
  int num_sms = 0;
};

Engine& engine();

// Sets the calling thread's last-error message and returns `s`.
estl_status fail(estl_status s, const char* fmt, ...);
estl_status ok();
estl_status check_cuda(cudaError_t e, const char* what);
estl_status require_init();

// Kernel launch with programmatic stream serialisation: the kernel (which
// starts with pdl_enter) may be scheduled while the previous kernel of the
// stream finishes its last wave.
// cluster > 0: launched in clusters of 2^cluster consecutive CTAs.
estl_status launch_pdl(const void* fn, long long grid, int threads, void** args, int smem, cudaStream_t stream,
                       const char* what, int cluster = 0);

// Budgeted device allocation (counted against Engine::budget).
estl_status dev_alloc(void** p, size_t bytes, const char* what);
void dev_free(void* p, size_t bytes);

// Kernel attributes of every step of a plan set now (before a stream capture).
estl_status prepare_steps(const Plan1D& plan);
// Reads and clears the bulk-load kernels' wait-timeout word (after a device
// synchronisation): ESTL_TIMEOUT if a wait gave up, ESTL_DEVICE_ERROR if its
// copies in flight did not drain either, else ESTL_OK.
estl_status take_bulk_wait_error();

// Launches one plan's steps on `stream`.  in/out/scratch are device
// pointers of interleaved complex64; sgn = +1 forward, -1 backward.  xoff
// (device, one element offset per transform of the plan) places transform f
// at in/out + xoff[f] instead of f * n, in buffers of `extent` elements
// (bucketed uneven batches; single, column, row and resident tiles; no
// tensor-copy tiles).
estl_status launch_steps(const Plan1D& plan, const cf32* in, cf32* out, cf32* scratch, float sgn,
                         cudaStream_t stream, const long long* xoff = nullptr, long long extent = 0);

}  // namespace estl
