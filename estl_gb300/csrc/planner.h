// planner.h — host-side FFT plan: which tile kernels run, on which buffers,
// in which order.  Pure C++ (no CUDA calls) so that the CPU index emulator
// executes exactly the launch list the GPU executor runs.
//
// Reference counterpart: the constructor of FFT_OpenCL_Contiguous
// (FFT_OpenCL_Contiguous.h:46-71), which fixes the radix list BGs and builds
// one kernel per radix-16 pass, and OpenCLFFTAlgorithm::computeParameters
// (OpenCLFFTAlgorithm.h:9-12).  Here the plan groups passes into tile kernels:
//   log2 N <= 14 : one launch (all passes of a transform in one CTA)
//   log2 N >  14 : four-step N = N1 * N2, a column launch then a row launch
//                  per chunk of transforms (two HBM round trips)
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace estl {

// STEP_COLUMN: the column pass of a 2D transform (strided column DFTs, no
// four-step twiddle), in place on the output.
// (kind 4 is unused: it named the streamed four-step, which was removed)
enum StepKind { STEP_SINGLE = 0, STEP_COL = 1, STEP_ROW = 2, STEP_COPY = 3, STEP_COLUMN = 5 };
constexpr int kStepKinds = 6;
enum BufId { BUF_IN = 0, BUF_OUT = 1, BUF_SCRATCH = 2 };

struct TileCfg {
  int kind;  // STEP_SINGLE / STEP_COL / STEP_ROW
  int logm, loge, logr, logc;
  int nthreads;
  int smem_bytes;
  int pipe;  // 0 plain; 2 bulk-load ring (bulk_core.cuh); 3 / 4 resident whole transforms (resident_core.cuh)
  int tc;    // radix-16 passes on the tensor cores (split precision)
  int cluster = 0;  // cluster tiles (cluster_core.cuh): log2 CTAs per cluster, 0 otherwise
  int csplit = 0;   // cluster tiles: log2 of the column DFT length N2
};

// All instantiated tile kernels (kernel_list.inc).
const std::vector<TileCfg>& tile_configs();
const TileCfg* find_tile(int kind, int logm, int loge, int logr, int logc, int pipe = 0, int tc = 0, int cluster = 0,
                         int csplit = 0);

struct Step {
  int kind;
  int logm, loge, logr, logc;
  long long grid;
  int src, dst;
  long long src_off, src_len;  // complex elements
  long long dst_off, dst_len;
  long long rows;  // STEP_SINGLE / STEP_COL / STEP_ROW: transforms; STEP_COPY: elements
  int logn;
  // persistent variant (pipe >= 2; grid = tiles, the launcher runs min(tiles, resident CTAs))
  int pipe = 0;
  // tensor-core variant (radix-16 passes as split-precision GEMMs)
  int tc = 0;
  // middle pass of a three-pass plan (STEP_COL): its input is already
  // conjugated for a backward transform (no conjugation on load), and inner
  // transform f = b * 2^ologr + k3 stores column output k2 at
  // b * N + k3 * N1 + k2 * 2^ologr * N1 (N1 = 2^(logn - logm)).
  int ologr = 0;
  // STEP_SINGLE on a cluster tile: log2 CTAs per transform (the grid is
  // rows * 2^cluster CTAs, launched in clusters of 2^cluster) and log2 of its
  // column DFT length
  int cluster = 0, csplit = 0;
};

// Tunable plan parameters (what the autotuner searches).  Zero / -1 fields
// mean "planner default".
struct PlanChoice {
  int mode = 0;  // 0 default, 1 single kernel, 2 four-step, 4 three-pass (3 is unused)
  int single_loge = -1, single_logc = -1;
  int logn2 = -1;  // four-step: log2 N2 (column DFT length); three-pass: log2 R (first column DFTs)
  int logn3 = -1;  // three-pass: log2 Q (second column DFTs); <= 0 = default
  int col_loge = -1, col_logc = -1;
  int row_loge = -1, row_logc = -1;
  long long chunk = 0;  // four-step: transforms per chunk (bounds the scratch)
  int pipe = 0;         // tile kernels: 0 plain, 2 bulk-load, 3 / 4 resident (where the variant exists)
  int split = 0;        // 0 FP32; else the SplitKind of tensor-core radix-16 passes (tc_core.cuh)
  // log2 of the largest radix of the single / column / row tiles (-1 = 4:
  // radix 16; 5: radix-32 passes, 32 elements per thread)
  int single_logr = -1, col_logr = -1, row_logr = -1;
  // single-kernel plans: log2 CTAs per transform of a cluster tile
  // (cluster_core.cuh; its column DFT length in logn2), 0 = one CTA per
  // transform, -1 = planner default
  int single_cluster = -1;
};

struct Plan1D {
  long long n = 0, batch = 0;
  int logn = 0;
  long long xdim = 0, ydim = 0;  // 2D plans (make_plan2d): n = xdim * ydim; 0 for 1D
  long long blue_m = 0;          // Bluestein plans (make_plan_bluestein): the FFT length M; 0 otherwise
  long long blue_chunk = 0;      // Bluestein: transforms per pass through the M-point FFTs
  PlanChoice choice;
  std::vector<Step> steps;
  long long scratch_elems = 0;
  int hbm_passes = 0;
  std::string describe() const;  // one-line JSON
};

constexpr int kSingleMaxLog = 14;
constexpr int kClusterMaxLog = 17;  // single-pass plans on cluster tiles: up to 2^17 points
constexpr int kTcSingleMaxLog = 13;  // split precision: larger n run four-step
constexpr int kMaxLogN = 24;
constexpr int kThreePassDefaultLog = 23;  // default plans of N >= 2^23 (FP32) run three passes
// At most 2^40 complex elements per plan (8 TiB, beyond any device memory;
// the planner's messages quote the number):
// keeps every 64-bit product of a length and a batch far from overflow.
constexpr int kMaxTotalLog = 40;

// Returns false (with *err set) when n is not a power of two in [1, 2^24] or
// the choice names no instantiated kernel.
bool make_plan(long long n, long long batch, const PlanChoice& choice, Plan1D* out, std::string* err);

// 2D transforms of ydim rows by xdim columns (row-major, x fastest), the
// layout of ESTL's FFT2D<D> (FFT.h:54-84): xdim-point row FFTs (any 1D plan),
// then ydim-point column FFTs in place (ydim <= 2^12, xdim * ydim <= 2^26).
constexpr int kColumnMaxLog = 12;
constexpr int kPlan2dMaxLog = 26;
bool make_plan2d(long long xdim, long long ydim, long long batch, const PlanChoice& choice, Plan1D* out,
                 std::string* err);

// Transforms of a length N that is not a power of two (2 < N <= 2^23):
// Bluestein's algorithm over M = 2^ceil(log2(2N - 1)) point FFT plans
// (bluestein_core.cuh).  The plan holds no steps; scratch_elems is the
// scratch of its M-point plan for blue_chunk transforms.
bool make_plan_bluestein(long long n, long long batch, Plan1D* out, std::string* err);

// The plan of the same transform (1D, 2D or Bluestein) for another batch count.
bool make_plan_like(const Plan1D& base, long long batch, Plan1D* out, std::string* err);

// Candidate choices for (n, batch), default first (autotuner search space).
std::vector<PlanChoice> plan_candidates(long long n, long long batch);

int ilog2_exact(long long n);

}  // namespace estl
