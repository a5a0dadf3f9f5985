// stream_core.cuh — streamed four-step FFT: one persistent launch runs the
// column and row tiles of a whole batch of equal-length transforms through a
// small scratch ring that stays in L2.
//
// The two-launch four-step (ColKernel then RowKernel per chunk) writes the
// full intermediate to scratch and reads it back: two HBM round trips per
// element.  Here the work queue interleaves the tiles of consecutive
// transforms,
//     col(0..Lg-1), [col(t), row(t - Lg)] for t = Lg .., row(B - Lg .. B - 1)
// so a row tile reads intermediate data that column tiles wrote moments
// earlier (an L2 hit), and transform t's intermediate lives in ring slot
// t mod R (R > Lg): the ring, a few transforms long, is rewritten in L2
// before its dirty lines are ever evicted.  HBM then sees one read of the
// input and one write of the output.
//
// Ordering: a row tile of t waits until all column tiles of t have finished
// (col_done[t]); a column tile of t >= R waits until all row tiles of t - R
// have finished reading slot t mod R (row_done[t - R]).  Both waits are on
// tiles that were taken from the queue earlier by running CTAs, so they end;
// they are bounded anyway (kStreamSpinLimit) and report *error instead of
// hanging.
#pragma once
#include "fft_core.cuh"
#include "packed_core.cuh"

namespace estl {

struct StreamArgs {
  Ptr<const PackedItem> items;  // kind PK_COL / PK_ROW, tf = transform, blk = first column / row
  long long nitems;
  Ptr<const cf32> in;
  Ptr<cf32> out;
  Ptr<cf32> scratch;  // ring * N elements
  Ptr<const cf32> bank;
  unsigned int* next;      // work counter
  unsigned int* col_done;  // per transform
  unsigned int* row_done;  // per transform
  int* error;
  float sgn;
  int logn;
  int ring;  // transforms held by the scratch ring
  int ncol, nrow;  // tiles per transform
};

constexpr unsigned long long kStreamSpinLimit = 1ULL << 24;

// Spins (thread 0 of the CTA) until *p >= need; returns false after the limit.
ESTL_HD bool wait_count(const unsigned int* p, unsigned int need, int* error) {
  unsigned long long spins = 0;
  while (load_acquire_u32(p) < need) {
    if (++spins > kStreamSpinLimit) {
      *error = 1;
      return false;
    }
    backoff();
  }
  return true;
}

template <class CK, class RK>
ESTL_HD void stream_run(const StreamArgs& a, long long cta, int tid, cf32* sm, int* slot) {
  (void)cta;
  static_assert(CK::NT == RK::NT, "column and row tiles share the CTA");
  const long long N = 1LL << a.logn;
  for (;;) {
    if (tid == 0) slot[0] = (int)atomic_add_u32(a.next, 1u);
    ESTL_SYNC();
    const long long idx = slot[0];
    ESTL_SYNC();
    if (idx >= a.nitems) return;
    const PackedItem it = a.items[idx];
    const long long tf = it.tf;
    const long long slot_off = (tf % a.ring) * N;
    if (tid == 0) {
      bool ok = true;
      if (it.kind == PK_ROW)
        ok = wait_count(a.col_done + tf, (unsigned int)a.ncol, a.error);
      else if (tf >= a.ring)
        ok = wait_count(a.row_done + (tf - a.ring), (unsigned int)a.nrow, a.error);
      slot[1] = ok ? 1 : 0;
    }
    ESTL_SYNC();
    const int ok = slot[1];
    ESTL_SYNC();
    if (ok) {
      if (it.kind == PK_COL)
        CK::body(a.in.sub(tf * N, N), a.scratch.sub(slot_off, N), it.blk, a.logn, tid, sm, a.bank, a.sgn);
      else
        RK::body(a.scratch.sub(slot_off, N), a.out.sub(tf * N, N), it.blk, a.logn, tid, sm, a.bank, a.sgn);
    }
    fence_gpu();  // this CTA's scratch stores / loads are ordered before the count
    ESTL_SYNC();
    if (tid == 0) atomic_add_u32(it.kind == PK_COL ? a.col_done + tf : a.row_done + tf, 1u);
  }
}

// Work list of a streamed four-step batch: per transform ncol column tiles of
// C_col columns and nrow row tiles of C_row rows; row tiles lag by `lag`
// transforms.
inline void stream_items(long long batch, int logn, int logn2, int col_logc, int row_logc, int lag,
                         PackedItem* out) {
  const int logn1 = logn - logn2;
  const int ncol = 1 << (logn1 - col_logc), nrow = 1 << (logn2 - row_logc);
  long long k = 0;
  for (long long s = 0; s < batch + lag; ++s) {
    if (s < batch)
      for (int b = 0; b < ncol; ++b) out[k++] = PackedItem{PK_COL, logn, (int)s, b << col_logc};
    if (s >= lag)
      for (int b = 0; b < nrow; ++b) out[k++] = PackedItem{PK_ROW, logn, (int)(s - lag), b << row_logc};
  }
}

}  // namespace estl
