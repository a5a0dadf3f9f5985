// bulk_core.cuh — four-step row and column passes with bulk asynchronous
// tile loads.
//
// The plain tile kernels load their tile with per-thread global loads, then
// compute, then store; with 1-2 CTAs per SM the SM is idle on memory during
// compute.  BulkRowKernel is persistent: each CTA owns two shared-memory
// stages, and one thread issues the next tiles' rows as bulk asynchronous
// copies (cp.async.bulk, global -> shared, completion counted in bytes on an
// mbarrier) while the CTA computes the current tile.  A stage is first the
// landing zone of its tile's rows (row c at c * RS, RS = M + 16/C so that the
// column-fastest reads are conflict-free; RS = M for one row per tile, which
// also runs whole transforms: N2 = 1), then, once every thread holds its
// elements in registers, the Stockham exchange buffer of that tile.  The
// next load into the stage is issued after the tile's last exchange.
//
//   tile k:  wait(stage k%2) -> registers -> passes (exchange in the stage)
//            -> issue tile k+2 into stage k%2 -> stores (C-wide runs)
//
// BulkColKernel runs the column pass the same way; its tiles are strided
// column runs, fetched as 2D tensor copies (TMA boxes) through a tensor map.
//
// Both are launched with plain stream order; when a programmatically launched
// kernel precedes them they trigger their dependents at their last tile.
//
// Waits are bounded: after kBulkSpinLimit polls the kernel records the tile in
// an error word, waits (bounded again) for its copies in flight and returns.
// The emulator runs the same code with the copies as bounds-checked memcpys at
// issue time.
#pragma once
#include <stdint.h>

#include <cstring>

#include "fft_core.cuh"

namespace estl {

constexpr long long kBulkSpinLimit = 1LL << 22;

// Bit of the bulk-load kernels' error word (TileArgs::err) above the tile
// number: a CTA gave up on a wait and its bounded drain of the copies it had
// in flight also ran out, so those copies may still land in shared memory
// that a later launch owns.  estl_plan_check then marks the plan unusable.
constexpr long long kErrCopiesInFlight = 1LL << 62;

#if defined(__CUDA_ARCH__)
ESTL_HD uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
#endif

ESTL_HD void mbar_init(uint64_t* bar, int count) {
#if defined(__CUDA_ARCH__)
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
#else
  *bar = 0;
  (void)count;
#endif
}

ESTL_HD void bulk_fence_init() {
#if defined(__CUDA_ARCH__)
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
#endif
}

// Orders this thread's (and, after a barrier, the CTA's) generic-proxy accesses
// of shared memory before later async-proxy (bulk copy) writes.
ESTL_HD void bulk_fence_proxy() {
#if defined(__CUDA_ARCH__)
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
#endif
}

ESTL_HD void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
#if defined(__CUDA_ARCH__)
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
#else
  (void)bar;
  (void)bytes;
#endif
}

// Bulk copy of `n` complex elements from global `src` to shared `dst` (both
// 16-byte aligned, n even), counted on `bar`.
ESTL_HD void bulk_load(const Ptr<cf32>& dst, long long didx, const Ptr<const cf32>& src, long long sidx, int n,
                       uint64_t* bar) {
  ESTL_CHECK(didx + n - 1, dst.n, "bulk copy shared destination");
  ESTL_CHECK(sidx + n - 1, src.n, "bulk copy global source");
  ESTL_CHECK((long long)(((uintptr_t)(dst.p + didx)) & 15), 1, "bulk copy shared alignment (16 B)");
  ESTL_CHECK((long long)(((uintptr_t)(src.p + sidx)) & 15), 1, "bulk copy global alignment (16 B)");
#if defined(__CUDA_ARCH__)
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
          smem_u32(dst.p + didx)),
      "l"(src.p + sidx), "r"((uint32_t)(n * sizeof(cf32))), "r"(smem_u32(bar))
      : "memory");
#else
  std::memcpy(dst.p + didx, src.p + sidx, (size_t)n * sizeof(cf32));
  (void)bar;
#endif
}

// Bounded wait for phase `parity` of `bar`; false if the limit ran out.
ESTL_HD bool mbar_wait(uint64_t* bar, uint32_t parity) {
#if defined(__CUDA_ARCH__)
  for (long long it = 0; it < kBulkSpinLimit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
#else
  (void)bar;
  (void)parity;
  return true;  // the emulator's copies complete at issue
#endif
}

// CTA-wide OR (a barrier): every thread leaves a failed wait together.
ESTL_HD bool cta_any(bool x) {
#if defined(__CUDA_ARCH__)
  return __syncthreads_or(x ? 1 : 0) != 0;
#else
  ESTL_SYNC();
  return x;  // the emulator's waits never fail
#endif
}

// A bounded tile wait gave up: record the tile, then let the copies that may
// still be in flight (this stage's and the other stage's next tile) land
// before the CTA's shared memory is released, again with bounded waits.
ESTL_HD void bulk_give_up(const TileArgs& a, long long tile, int tid, uint64_t* bar, int s, long long k,
                          bool other_pending) {
  if (tid != 0) return;
  long long e = tile + 1;
  if (!mbar_wait(&bar[s], (uint32_t)((k >> 1) & 1))) e |= kErrCopiesInFlight;
  if (other_pending && !mbar_wait(&bar[s ^ 1], (uint32_t)(((k + 1) >> 1) & 1))) e |= kErrCopiesInFlight;
  if (a.err) atomic_max_ll(a.err, e);
}

// Row pass of the four-step (as RowKernel: C rows k2_0.. of one transform's
// scratch -> X[k2 + N2 k1], column-fastest threads), persistent over tiles.
template <int LOGM, int LOGE, int LOGR, int LOGC>
struct BulkRowKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  using Base = RowKernel<LOGM, LOGE, LOGR, LOGC>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  static_assert(C >= 1 && C <= 8, "landing rows 16-byte aligned and conflict-free for 1 <= C <= 8");
  // landing row stride (elements, even); one row per tile (a whole transform,
  // N2 = 1: the single-tile case) needs no padding
  static constexpr int RS = C == 1 ? TL::M : TL::M + 16 / C;
  static constexpr int EXCH = TL::MP * C;    // exchange layout of RowKernel (pad(m) * C + c)
  static constexpr int STAGE = ((EXCH > C * RS ? EXCH : C * RS) + 1) & ~1;
  static constexpr int SMEM_ELEMS = 2 * STAGE + 2;  // two stages, then two 8-byte mbarriers
  // CTAs per SM that shared memory allows: the registers are sized for those
  static constexpr int SMEM_BLOCKS = (227 * 1024) / (SMEM_ELEMS * 8 + 1024);
  static constexpr int MIN_BLOCKS =
      SMEM_BLOCKS < 1 ? 1 : (SMEM_BLOCKS < min_blocks(NT, TL::E) ? SMEM_BLOCKS : min_blocks(NT, TL::E));
  static_assert(TL::M % 2 == 0, "rows of an even number of elements (16-byte copies)");
  static constexpr bool PERSISTENT = true;

  ESTL_HD static long long ntiles(const TileArgs& a) { return a.rows << (a.logn - LOGM - LOGC); }

  // thread 0: the C rows of `tile` into stage `s`
  ESTL_HD static void issue(const TileArgs& a, long long tile, const Ptr<cf32>& stage, uint64_t* bar) {
    const int logn2 = a.logn - LOGM;
    const int nblk = 1 << (logn2 - LOGC);
    const long long f = tile / nblk;
    const int k2_0 = (int)(tile - f * nblk) * C;
    const long long N = 1LL << a.logn;
    bulk_fence_proxy();
    mbar_expect_tx(bar, (uint32_t)(C * TL::M * sizeof(cf32)));
    // N2 = 1 (whole transforms): the rows are the caller's transforms
    const long long base = logn2 == 0 ? xbase(a, f, N) : f * N;
    for (int c = 0; c < C; ++c) bulk_load(stage, (long long)c * RS, a.in, base + (long long)(k2_0 + c) * TL::M, TL::M, bar);
  }

  ESTL_HD static void run(const TileArgs& a, long long cta, int tid, cf32* smraw) {
    const long long nt = ntiles(a), grid = a.grid;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smraw + 2 * STAGE);
    const int c = tid & (C - 1);
    const int t = tid >> LOGC;
    const int logn2 = a.logn - LOGM;
    const int nblk = 1 << (logn2 - LOGC);
    const long long N = 1LL << a.logn;
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    if (tid == 0) {
      mbar_init(&bar[0], 1);
      mbar_init(&bar[1], 1);
      bulk_fence_init();
      if (cta < nt) issue(a, cta, Ptr<cf32>{smraw, STAGE}, &bar[0]);
      if (cta + grid < nt) issue(a, cta + grid, Ptr<cf32>{smraw + STAGE, STAGE}, &bar[1]);
    }
    ESTL_SYNC();
    long long k = 0;
    for (long long tile = cta; tile < nt; tile += grid, ++k) {
      if (tile + grid >= nt) pdl_trigger();  // last tile: let the next kernel's CTAs in as this one drains
      const int s = (int)(k & 1);
      const Ptr<cf32> stage{smraw + s * STAGE, STAGE};
      if (cta_any(!mbar_wait(&bar[s], (uint32_t)((k >> 1) & 1)))) {
        bulk_give_up(a, tile, tid, bar, s, k, tile + grid < nt);
        return;
      }
      cf32 v[TL::E];
      // a four-step row pass reads the column pass's (already conjugated)
      // scratch; a whole transform per tile (N2 = 1) reads the plan's input
      const float lsgn = logn2 == 0 ? a.sgn : 1.f;
#pragma unroll
      for (int j = 0; j < TL::E; ++j) v[j] = conj_if(stage[c * RS + t + TL::T * j], lsgn);
      ESTL_SYNC();  // the stage becomes the exchange buffer
      run_passes<TL, 0>(v, t, c, stage, tw, typename Base::Sidx{});
      ESTL_SYNC();  // every exchange read of this stage is done
      if (tid == 0 && tile + 2 * grid < nt) issue(a, tile + 2 * grid, stage, &bar[s]);
      const long long f = tile / nblk;
      const int k2_0 = (int)(tile - f * nblk) * C;
      const Ptr<cf32> out = a.out.sub(xbase(a, f, N), N);
#pragma unroll
      for (int j = 0; j < TL::E; ++j) stcs(out, k2_0 + c + ((t + TL::T * j) << logn2), conj_if(v[j], a.sgn));
    }
  }
};

// 2D tensor tile copy, global -> shared (TMA), counted on `bar`: the box of
// the tensor map `tmap` (a __grid_constant__ kernel parameter) at element
// coordinates (x, y) lands densely at `dst` (128-byte aligned).
ESTL_HD void tma_load_2d(cf32* dst, const void* tmap, int x, int y, uint64_t* bar) {
#if defined(__CUDA_ARCH__)
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
          smem_u32(dst)),
      "l"(tmap), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
#else
  (void)dst;
  (void)tmap;
  (void)x;
  (void)y;
  (void)bar;
#endif
}

// Column pass of the four-step (as ColKernel: columns n1_0 .. n1_0 + C - 1 of
// one transform -> its scratch S[k2 * N1 + n1] with the four-step twiddle),
// persistent over tiles, with each tile's strided columns fetched by 2D tensor
// copies.  The tensor map views the step's input as a matrix of rows * M rows
// of N1 complex (2 N1 floats, pitch N1 * 8 bytes); a tile is M / BH boxes of
// BH rows x C complex, which land as the dense [m][c] layout the threads read
// column-fastest.  Box x = 2 n1_0 floats: 8 n1_0 bytes, a multiple of 16 since
// C >= 2 divides n1_0.  Stages as in BulkRowKernel: landing zone, then the
// exchange buffer (pad(m) * C + c), reloaded after the tile's last exchange.
template <int LOGM, int LOGE, int LOGR, int LOGC>
struct BulkColKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  using Base = ColKernel<LOGM, LOGE, LOGR, LOGC>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  static_assert(C >= 2 && C <= 128, "box rows of 2C floats: 16-byte multiples, at most 256 elements");
  static_assert(TL::P > 1, "the exchange buffer doubles as the landing zone");
  static constexpr int BH = TL::M < 256 ? TL::M : 256;  // box height (rows of the tensor map)
  static constexpr int NBOX = TL::M / BH;
  static constexpr int EXCH = TL::MP * C;
  static constexpr int STAGE = (((EXCH > TL::M * C) ? EXCH : TL::M * C) + 15) & ~15;  // 128-byte multiple
  static constexpr int ALIGN = 16;                                                    // elements of slack
  static constexpr int SMEM_ELEMS = 2 * STAGE + ALIGN + 2;
  static constexpr int SMEM_BLOCKS = (227 * 1024) / (SMEM_ELEMS * 8 + 1024);
  static constexpr int MIN_BLOCKS =
      SMEM_BLOCKS < 1 ? 1 : (SMEM_BLOCKS < min_blocks(NT, TL::E) ? SMEM_BLOCKS : min_blocks(NT, TL::E));
  static_assert((BH * C * 8) % 128 == 0, "boxes keep the 128-byte alignment of the stage");
  static constexpr bool PERSISTENT = true;

  ESTL_HD static long long ntiles(const TileArgs& a) { return a.rows << (a.logn - LOGM - LOGC); }

  // thread 0: the C columns of `tile` into `stage`
  ESTL_HD static void issue(const TileArgs& a, long long tile, cf32* stage, uint64_t* bar) {
    const int logn1 = a.logn - LOGM;
    const int nblk = 1 << (logn1 - LOGC);
    const long long f = tile / nblk;
    const int n1_0 = (int)(tile - f * nblk) * C;
    bulk_fence_proxy();
    mbar_expect_tx(bar, (uint32_t)(TL::M * C * sizeof(cf32)));
    for (int b = 0; b < NBOX; ++b) {
      const long long y = f * TL::M + (long long)b * BH;
      cf32* dst = stage + b * BH * C;
#if defined(__CUDA_ARCH__)
      tma_load_2d(dst, a.tmap, 2 * n1_0, (int)y, bar);
#else
      // the emulated box: BH rows of C complex, rows N1 apart, bounds-checked
      ESTL_CHECK((long long)((n1_0 * 8) & 15), 1, "tensor copy x offset (16 B)");
      ESTL_CHECK((long long)(((uintptr_t)dst) & 127), 1, "tensor copy shared alignment (128 B)");
      for (int r = 0; r < BH; ++r) {
        const long long src = ((y + r) << logn1) + n1_0;
        ESTL_CHECK(src + C - 1, a.in.n, "tensor copy global source");
        std::memcpy(dst + r * C, a.in.p + src, (size_t)C * sizeof(cf32));
      }
      (void)bar;
#endif
    }
  }

  ESTL_HD static void run(const TileArgs& a, long long cta, int tid, cf32* smraw) {
    const long long nt = ntiles(a), grid = a.grid;
    // stages on a 128-byte boundary of the dynamic shared memory
#if defined(__CUDA_ARCH__)
    const int skew = (int)(((128u - (smem_u32(smraw) & 127u)) & 127u) >> 3);
#else
    const int skew = (int)(((128u - ((uintptr_t)smraw & 127u)) & 127u) >> 3);
#endif
    cf32* base = smraw + skew;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smraw + ALIGN + 2 * STAGE);
    const int c = tid & (C - 1);
    const int t = tid >> LOGC;
    const int logn1 = a.logn - LOGM;
    const int nblk = 1 << (logn1 - LOGC);
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    if (tid == 0) {
      mbar_init(&bar[0], 1);
      mbar_init(&bar[1], 1);
      bulk_fence_init();
      if (cta < nt) issue(a, cta, base, &bar[0]);
      if (cta + grid < nt) issue(a, cta + grid, base + STAGE, &bar[1]);
    }
    ESTL_SYNC();
    long long k = 0;
    for (long long tile = cta; tile < nt; tile += grid, ++k) {
      if (tile + grid >= nt) pdl_trigger();  // last tile: let the next kernel's CTAs in as this one drains
      const int s = (int)(k & 1);
      const Ptr<cf32> stage{base + s * STAGE, STAGE};
      if (cta_any(!mbar_wait(&bar[s], (uint32_t)((k >> 1) & 1)))) {
        bulk_give_up(a, tile, tid, bar, s, k, tile + grid < nt);
        return;
      }
      cf32 v[TL::E];
#pragma unroll
      for (int j = 0; j < TL::E; ++j) v[j] = conj_if(stage[(t + TL::T * j) * C + c], a.sgn);
      ESTL_SYNC();  // the stage becomes the exchange buffer
      run_passes<TL, 0>(v, t, c, stage, tw, typename Base::Sidx{});
      ESTL_SYNC();  // every exchange read of this stage is done
      if (tid == 0 && tile + 2 * grid < nt) issue(a, tile + 2 * grid, stage.p, &bar[s]);
      const long long f = tile / nblk;
      const int n1 = (int)(tile - f * nblk) * C + c;
      Base::store_twiddled(v, Base::out_of(a.out, f, a.logn, a.ologr), n1, t, a.logn, a.bank, a.ologr);
    }
  }
};

}  // namespace estl
