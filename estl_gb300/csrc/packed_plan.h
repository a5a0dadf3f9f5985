// packed_plan.h — uneven batches: many independent transforms of different
// power-of-two lengths, packed in one buffer with an offsets array, run as a
// list of work items by one persistent launch (or one launch per size class).
//
// The reference runs one FFT object per size (tests/Test.cpp:45-60 creates a
// plan per (M, B)); there is no uneven batch.  Work items reuse the tile
// bodies of fft_core.cuh with a fixed CTA of 256 threads:
//   n <= 2^12           one item = C whole transforms of one size
//   2^13 <= n <= 2^18   four-step: column items then row items per transform
// A mixed batch adds FFT convolutions (Convolution.h:95-154 in 1D): those of
// padded length <= 2^12 are work items of the same launch (one item = C whole
// convolutions), longer ones run the convolution engine's own launches.
#pragma once
#include <string>
#include <vector>

#include "conv_plan.h"
#include "planner.h"

namespace estl {

enum PackedItemKind { PK_SINGLE = 0, PK_COL = 1, PK_ROW = 2, PK_CONV = 3 };

// One convolution work item's request: real signal (sig_len floats at
// sig_off) * real filter (filt_len floats at filt_off), zero-padded to the
// item's length; output samples [out_shift, out_shift + out_len) of the
// circular result go to out_off.  correlate: the filter spectrum is
// conjugated (Convolution.h:125-137); dc_norm: the result is divided by the
// filter's sum, the spectrum DC (Convolution.h:141-143).
struct PackedConv {
  long long sig_off, filt_off, out_off;
  int sig_len, filt_len, out_len, out_shift;
  int correlate, dc_norm;
};

struct PackedItem {
  int kind;   // PackedItemKind
  int logn;   // transform length class
  int tf;     // PK_SINGLE: first position in class_list; PK_COL/PK_ROW: transform index
  int blk;    // PK_SINGLE: transforms in the item; PK_COL: first column n1; PK_ROW: first row k2
};

constexpr int kPackedThreads = 256;
constexpr int kPackedMinLog = 1;
constexpr int kPackedMaxLog = 18;
constexpr int kPackedSingleMaxLog = 12;

// Tile shape of a size class: log2 rows (single) or columns/rows (four-step) per item.
int packed_single_logc(int logn);
int packed_logn2(int logn);  // four-step column DFT length
int packed_col_logc(int logn);
int packed_row_logc(int logn);

struct PackedLayout {
  std::vector<PackedItem> items;
  std::vector<int> class_list;          // transform indices grouped by size class
  std::vector<long long> offsets;       // element offset of each transform (input and output)
  std::vector<int> lognv;               // log2 length of each transform
  std::vector<long long> scratch_off;   // four-step transforms: element offset in the scratch
  std::vector<int> ncol;                // four-step transforms: column items (row-item dependency)
  std::vector<int> launch_begin, launch_count;  // per-size mode: item ranges, one launch each
  long long scratch_elems = 0;
  long long total_elems = 0;  // max(offset + length)
  long long elements = 0;     // sum of lengths
  double flops = 0;           // sum of 5 n log2 n
  bool persistent = true;
  // mixed batches: convolutions run as work items (padded length <= 2^12) ...
  std::vector<PackedConv> convs;
  std::vector<int> conv_class_list;  // convs grouped by padded length
  // ... and the longer ones, run by the convolution engine
  std::vector<ConvReq> conv_engine;
  long long conv_sig_elems = 0, conv_filt_elems = 0, conv_out_elems = 0;  // float extents
  double conv_flops = 0;  // 2 x 5 n log2 n per in-kernel convolution
};

// offsets / sizes: count transforms (count may be 0 when nconv > 0).
// Returns false with *err on a size that is not a power of two in
// [2^1, 2^18], a negative offset, or overlapping transforms.  convs / nconv:
// the convolutions of a mixed batch, conv_flags the CONV_CORRELATE /
// CONV_REFERENCE_COMPAT semantics of all of them (CONV_NO_PAIRING and
// CONV_COMPLEX only shape the convolution engine's launches of the longer
// ones); a request needs lengths >= 1, offsets >= 0 and a padded length of
// at most 2^22.
bool build_packed_layout(const long long* offsets, const long long* sizes, long long count, bool persistent,
                         PackedLayout* out, std::string* err, const ConvReq* convs = nullptr, long long nconv = 0,
                         int conv_flags = 0);

// Bucketed uneven batches: one size class of the batch, run by the engine's
// own plan for (2^logn, count) over the class's transforms through their
// offsets (TileArgs::xoff), the four-step scratch dense per class.
struct PackedBucket {
  int logn = 0;
  Plan1D plan;                  // planned for the class's transform count
  std::vector<long long> xoff;  // element offset of each transform of the class, in class order
};

// Groups the batch by length and plans each class with choose(n, count)
// (the autotuner's cache on the device, the planner default in the
// emulator).  Column passes run their plain tiles (the tensor-copy variant
// needs a regular 2D view of the input), and a class with an odd offset runs
// no bulk-copy variant (16-byte aligned rows).  Validation as
// build_packed_layout.
bool build_packed_buckets(const long long* offsets, const long long* sizes, long long count,
                          PlanChoice (*choose)(long long n, long long count), std::vector<PackedBucket>* out,
                          long long* total_elems, std::string* err);

}  // namespace estl
