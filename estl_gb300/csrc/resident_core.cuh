// resident_core.cuh — whole transforms of 2^12..2^14 points, one per tile,
// with the next transform's load overlapping the current one's compute.
//
// The reference runs one Stockham pass per kernel with a full HBM round trip
// per pass (FFT_OpenCL_Contiguous.h:55-61,107-124).  SingleKernel keeps every
// pass of a transform on chip, but a CTA loads its transform, computes, then
// stores: with one 2^14-point transform per CTA (128 KB) only one CTA fits on
// an SM and the SM idles on memory while it computes.  ResKernel is
// persistent and splits shared memory into
//   * a landing zone of one whole transform (M complex), filled by bulk
//     asynchronous copies (cp.async.bulk, completion counted in bytes on an
//     mbarrier), and
//   * the Stockham exchange buffer, either a whole padded tile (H = 1) or half
//     of one (H = 2), exchanged in two rounds.
// A tile: wait for the landing zone -> registers -> issue the next tile's
// copy into the landing zone -> radix passes (exchanges in the exchange
// buffer) -> stores from registers.  The next transform streams in while the
// current one is computed and stored.
//
// Two-round exchange (H = 2): after pass p, output slot j of thread t goes to
// position q = out_pos<p>(t, j); the next pass reads positions t + T*j, so
// reads j < E/2 are exactly the positions q < M/2.  The first half-exchange
// writes the values with q < M/2 and reads them into a temporary, the second
// writes the rest and reads v[E/2..E); the temporary then fills v[0..E/2).
//
// Waits are bounded as in bulk_core.cuh.
#pragma once
#include "bulk_core.cuh"

namespace estl {

template <class TL, int p, int H>
ESTL_HD void run_passes_halves(cf32 (&v)[TL::E], int t, const Ptr<cf32>& xb, const Ptr<const cf32>& tw) {
  if constexpr (p < TL::P) {
    TL::template compute<p>(v, t, tw);
    if constexpr (p + 1 < TL::P) {
      if constexpr (H == 1) {
#pragma unroll
        for (int j = 0; j < TL::E; ++j) xb[TL::pad(TL::template out_pos<p>(t, j))] = v[j];
        ESTL_SYNC();
#pragma unroll
        for (int j = 0; j < TL::E; ++j) v[j] = xb[TL::pad(t + TL::T * j)];
        ESTL_SYNC();
      } else {
        static_assert(H == 2, "one or two exchange rounds");
        constexpr int HM = TL::M / 2, HE = TL::E / 2;
        cf32 lo[HE];
#pragma unroll
        for (int j = 0; j < TL::E; ++j) {
          const int q = TL::template out_pos<p>(t, j);
          if (q < HM) xb[TL::pad(q)] = v[j];
        }
        ESTL_SYNC();
#pragma unroll
        for (int j = 0; j < HE; ++j) lo[j] = xb[TL::pad(t + TL::T * j)];
        ESTL_SYNC();
#pragma unroll
        for (int j = 0; j < TL::E; ++j) {
          const int q = TL::template out_pos<p>(t, j);
          if (q >= HM) xb[TL::pad(q - HM)] = v[j];
        }
        ESTL_SYNC();
#pragma unroll
        for (int j = HE; j < TL::E; ++j) v[j] = xb[TL::pad(t + TL::T * j - HM)];
        ESTL_SYNC();
#pragma unroll
        for (int j = 0; j < HE; ++j) v[j] = lo[j];
      }
    }
    run_passes_halves<TL, p + 1, H>(v, t, xb, tw);
  }
}

template <int LOGM, int LOGE, int LOGR, int H>
struct ResKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  static constexpr int NT = TL::T;
  static constexpr int M = TL::M;
  static constexpr int XB = ((H == 1 ? TL::MP : TL::pad(M / 2)) + 1) & ~1;  // exchange buffer, even
  static constexpr int SMEM_ELEMS = M + XB + 2;                            // landing, exchange, mbarrier
  static constexpr int SMEM_BLOCKS = (227 * 1024) / (SMEM_ELEMS * 8 + 1024);
  static constexpr int MIN_BLOCKS =
      SMEM_BLOCKS < 1 ? 1 : (SMEM_BLOCKS < min_blocks(NT, TL::E) ? SMEM_BLOCKS : min_blocks(NT, TL::E));
  static constexpr bool PERSISTENT = true;
  static constexpr int COPY = M < 2048 ? M : 2048;  // elements per bulk copy (16 KB)
  static_assert(TL::P > 1, "a transform of one pass needs no exchange buffer");
  static_assert(M % COPY == 0 && COPY % 2 == 0, "whole 16-byte bulk copies");
  static_assert(H == 1 || (TL::E % 2 == 0 && M % 2 == 0), "two exchange rounds split the slots in halves");

  // thread 0: transform `tile` into the landing zone
  ESTL_HD static void issue(const TileArgs& a, long long tile, const Ptr<cf32>& land, uint64_t* bar) {
    bulk_fence_proxy();
    mbar_expect_tx(bar, (uint32_t)(M * sizeof(cf32)));
    const long long base = xbase(a, tile, M);
    for (int c = 0; c < M; c += COPY) bulk_load(land, c, a.in, base + c, COPY, bar);
  }

  ESTL_HD static void run(const TileArgs& a, long long cta, int tid, cf32* smraw) {
    const long long nt = a.rows, grid = a.grid;
    const Ptr<cf32> land{smraw, M};
    const Ptr<cf32> xb{smraw + M, XB};
    uint64_t* bar = reinterpret_cast<uint64_t*>(smraw + M + XB);
    const int t = tid;
    const Ptr<const cf32> tw = a.bank.sub(M, M);
    if (tid == 0) {
      mbar_init(bar, 1);
      bulk_fence_init();
      if (cta < nt) issue(a, cta, land, bar);
    }
    ESTL_SYNC();
    long long k = 0;
    for (long long tile = cta; tile < nt; tile += grid, ++k) {
      if (tile + grid >= nt) pdl_trigger();  // last tile: let the next kernel's CTAs in as this one drains
      if (cta_any(!mbar_wait(bar, (uint32_t)(k & 1)))) {
        if (tid == 0) {
          // this tile's copies may still be in flight: drain them (bounded)
          long long e = tile + 1;
          if (!mbar_wait(bar, (uint32_t)(k & 1))) e |= kErrCopiesInFlight;
          if (a.err) atomic_max_ll(a.err, e);
        }
        return;
      }
      cf32 v[TL::E];
#pragma unroll
      for (int j = 0; j < TL::E; ++j) v[j] = conj_if(land[t + TL::T * j], a.sgn);
      ESTL_SYNC();  // every thread holds its elements: the landing zone is free
      if (tid == 0 && tile + grid < nt) issue(a, tile + grid, land, bar);
      run_passes_halves<TL, 0, H>(v, t, xb, tw);
      const Ptr<cf32> out = a.out.sub(xbase(a, tile, M), M);
#pragma unroll
      for (int j = 0; j < TL::E; ++j) stcs(out, t + TL::T * j, conj_if(v[j], a.sgn));
    }
  }
};

}  // namespace estl
