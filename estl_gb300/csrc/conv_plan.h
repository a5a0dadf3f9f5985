// conv_plan.h — host-side layout of a batch of FFT convolutions: size
// buckets, per-request descriptors, workspace offsets and the launch list.
// Pure C++ so that the host emulator runs the same launch list as the GPU.
//
// Reference: Convolution2D_FFT::convolve (Convolution.h:95-154), restated in
// 1D for many independent requests.
#pragma once
#include <string>
#include <vector>

#include "conv_core.cuh"

namespace estl {

// CONV_NO_PAIRING: padded lengths <= 2^14 run each request as its own
// complex transform (no two real requests per transform).  CONV_COMPLEX:
// every length runs complex transforms (neither pairing nor the real-input
// four-step form of longer requests).
enum ConvFlags { CONV_CORRELATE = 1, CONV_REFERENCE_COMPAT = 2, CONV_NO_PAIRING = 4, CONV_COMPLEX = 8 };
// Bits 8-9 of the flags: the split precision of the FFT stages (SplitKind;
// 0 = FP32), ESTL_CONV_PRECISION(p) in the C ABI.
constexpr int kConvSplitShift = 8;
constexpr int kConvFlagMask =
    CONV_CORRELATE | CONV_REFERENCE_COMPAT | CONV_NO_PAIRING | CONV_COMPLEX | (3 << kConvSplitShift);
inline int conv_split(int flags) { return (flags >> kConvSplitShift) & 3; }

// One convolution request: offsets (in floats) into the caller's packed
// signal / filter / output arrays.
struct ConvReq {
  long long signal_len, filter_len;
  long long sig_off, filt_off, out_off;
};

enum ConvLaunchKind {
  CK_SPEC_SINGLE = 0,  // filter -> spectrum, N <= 2^14
  CK_CONV_SINGLE = 1,  // signal -> output, N <= 2^14 (fused)
  CK_COL_FILTER = 2,   // four-step column pass of the filters
  CK_SPEC_ROW = 3,     // four-step row pass of the filters -> permuted spectrum
  CK_COL_SIGNAL = 4,   // four-step column pass of the signals
  CK_MID = 5,          // row DFT, multiply, row DFT, twiddle
  CK_OUT = 6,          // column DFT -> real output
  CK_SPEC_PAIR = 7,    // two filters per complex FFT -> the A / B spectra of a request pair, N <= 2^14
  CK_CONV_PAIR = 8,    // two signals per complex FFT -> two outputs, N <= 2^14 (fused)
  // N > 2^14, real input: every launch runs the N/2-point complex transform of
  // the request (ConvLaunch::logn = log2 N - 1)
  CK_COL_FILTER_H = 9,   // column pass of the filters (pairs of reals as complex)
  CK_SPEC_ROW_H = 10,    // row pass of the filters -> permuted half spectrum + Nyquist term
  CK_COL_SIGNAL_H = 11,  // column pass of the signals
  CK_MID_H = 12,         // row DFT, spectrum split, multiply, inverse's input, row DFT, twiddle
  CK_OUT_H = 13,         // column DFT -> two real outputs per complex value
};

// launches that read the filter rows (and write spectra)
inline bool ck_is_filter(int kind) {
  return kind == CK_SPEC_SINGLE || kind == CK_COL_FILTER || kind == CK_SPEC_ROW || kind == CK_SPEC_PAIR ||
         kind == CK_COL_FILTER_H || kind == CK_SPEC_ROW_H;
}
// single-tile launches (N <= 2^14)
inline bool ck_is_single(int kind) {
  return kind == CK_SPEC_SINGLE || kind == CK_CONV_SINGLE || kind == CK_SPEC_PAIR || kind == CK_CONV_PAIR;
}

struct ConvLaunch {
  int kind;
  int logm, loge, logr, logc;
  long long grid;
  int logn;
  long long row_begin, row_count;  // rows in the filter (CK_SPEC_*, CK_COL_FILTER) or signal row array
  long long s_off;                 // element offset of this bucket's scratch in s1 / s2
  int tc = 0;                      // split-precision (tensor-core) variant
};

struct ConvLayout {
  std::vector<ConvRow> filt_rows, sig_rows;
  std::vector<ConvLaunch> launches;
  long long spec_elems = 0;     // complex
  long long scratch_elems = 0;  // complex, each of s1 and s2
  long long out_elems = 0;      // floats written (max out_off + out_len)
  // workspace byte offsets (256-byte aligned regions)
  size_t off_filt_rows = 0, off_sig_rows = 0, off_spec = 0, off_s1 = 0, off_s2 = 0, workspace_bytes = 0;
  int buckets = 0;
  // launches that compute spectra come first in each bucket; these counts let
  // a caller run the spectrum launches once and the convolution launches often
  std::vector<char> is_spectrum_launch;
  int split = 0;  // SplitKind of the tensor-core launches
  int shared = 0;  // one filter for every request (ConvArgs::shared of the paired kernels)
};

constexpr int kConvMaxLogN = 22;
// Split-precision single-tile convolutions up to 2^13: a 2^14 tile with the
// tensor-core staging of its 32 warps exceeds the 227 KB of shared memory, so
// that bucket runs its FP32 tiles.
constexpr int kConvTcSingleMaxLog = 13;
constexpr long long kMaxConvSmemBytes = 227 * 1024;

// Output length of one request (signal_len + filter_len - 1, or signal_len
// in reference-compatible mode).
long long conv_out_len(long long signal_len, long long filter_len, int flags);
int conv_logn(long long signal_len, long long filter_len);
// First circular sample of the output in reference-compatible mode (0
// otherwise): output m is sample (m + shift) mod 2^logn of the result.
int conv_out_shift(long long filter_len, int logn, int flags);

// shared_filter: every request uses the filter of request 0 (one spectrum,
// computed once); all requests must then pad to the same N.
bool build_conv_layout(const ConvReq* reqs, int count, int flags, ConvLayout* out, std::string* err,
                       bool shared_filter = false);

// Extents (in floats) of the packed signal / filter arrays the requests use.
void conv_extents(const ConvReq* reqs, int count, long long* sig_elems, long long* filt_elems);

}  // namespace estl
