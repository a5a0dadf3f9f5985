// pipe_core.cuh — pipelined tile kernels: the tile bodies of fft_core.cuh run
// by grid-stride CTAs that prefetch the next tile while computing the
// current one.
//
// Each CTA owns two shared-memory tile buffers.  While it computes tile i in
// buffer k, cp.async (global -> shared, L2 only, no register staging) brings
// tile i + grid into buffer k^1, so the loads of the next tile are in flight
// during the whole compute of the current one and the SM never waits for
// HBM with nothing to do.  A tile buffer is also the padded exchange buffer
// of its tile: the unpadded input is read into registers, a barrier, and the
// Stockham passes then exchange through the same bytes (shared memory per CTA
// = 2 x max(tile, padded tile) instead of 3 x).
//
// cp.async moves 16 bytes (two complex64), so these kernels need 16-byte
// aligned transform data; the launcher uses the plain kernels otherwise.
#pragma once
#include <stdint.h>

#include <cstring>

#include "fft_core.cuh"

namespace estl {

// 16-byte async copy global -> shared.  Both addresses must be 16-byte
// aligned (the emulator checks bounds and alignment).
ESTL_HD void cp_async16(const Ptr<cf32>& sm, long long sidx, const Ptr<const cf32>& g, long long gidx) {
  ESTL_CHECK(sidx + 1, sm.n, "cp.async shared destination");
  ESTL_CHECK(gidx + 1, g.n, "cp.async global source");
  ESTL_CHECK(sidx, sm.n, "cp.async shared destination");
  ESTL_CHECK(gidx, g.n, "cp.async global source");
  ESTL_CHECK((long long)((uintptr_t)(sm.p + sidx) & 15), 1, "cp.async shared destination alignment (16 B)");
  ESTL_CHECK((long long)((uintptr_t)(g.p + gidx) & 15), 1, "cp.async global source alignment (16 B)");
#if defined(__CUDA_ARCH__)
  const unsigned s = (unsigned)__cvta_generic_to_shared(sm.p + sidx);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(g.p + gidx) : "memory");
#else
  std::memcpy(sm.p + sidx, g.p + gidx, 16);
#endif
}
ESTL_HD void cp_async_commit() {
#if defined(__CUDA_ARCH__)
  asm volatile("cp.async.commit_group;\n" ::: "memory");
#endif
}
// Waits until at most `pending` of this thread's committed groups are in flight.
template <int PENDING>
ESTL_HD void cp_async_wait() {
#if defined(__CUDA_ARCH__)
  asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory");
#endif
}

// Grid-stride driver: prefetch tile `first`, then for every tile prefetch the
// next one into the other buffer, wait for the current one and compute it.
// K provides: TILE_BUF (elements per buffer), ntiles(a), issue(a, tile, tid,
// buf), compute(a, tile, tid, buf).
template <class K>
ESTL_HD void pipe_loop(const TileArgs& a, long long cta, long long grid, int tid, cf32* smraw) {
  const long long ntiles = K::ntiles(a);
  const Ptr<cf32> buf[2] = {Ptr<cf32>{smraw, K::TILE_BUF}, Ptr<cf32>{smraw + K::TILE_BUF, K::TILE_BUF}};
  int k = 0;
  long long tile = cta;
  if (tile < ntiles) K::issue(a, tile, tid, buf[0]);
  cp_async_commit();
  for (; tile < ntiles; tile += grid, k ^= 1) {
    const long long next = tile + grid;
    if (next < ntiles) K::issue(a, next, tid, buf[k ^ 1]);
    cp_async_commit();
    cp_async_wait<1>();  // this thread's copies of `tile` have landed
    ESTL_SYNC();         // ... and every other thread's
    K::compute(a, tile, tid, buf[k]);
    ESTL_SYNC();  // buffer k is free before it is refilled two tiles later
  }
  cp_async_wait<0>();
}

// Whole transforms, C per tile (row mapping, as SingleKernel).
template <int LOGM, int LOGE, int LOGR, int LOGC>
struct PipeSingleKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  using Base = SingleKernel<LOGM, LOGE, LOGR, LOGC>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  static constexpr int TILE = C * TL::M;
  // each buffer a multiple of 16 bytes, so that the second one stays aligned
  static constexpr long long TILE_BUF = (((Base::SMEM_ELEMS > TILE) ? Base::SMEM_ELEMS : TILE) + 1) & ~1LL;
  static constexpr long long SMEM_ELEMS = 2 * TILE_BUF;
  static constexpr int MIN_BLOCKS = min_blocks(NT, TL::E);
  static_assert(TL::M >= 2 && (TILE / 2) % NT == 0, "16-byte chunks must split evenly");

  ESTL_HD static long long ntiles(const TileArgs& a) { return (a.rows + C - 1) / C; }

  ESTL_HD static void issue(const TileArgs& a, long long tile, int tid, const Ptr<cf32>& buf) {
    const long long valid = (a.rows - tile * C < C ? a.rows - tile * C : C) * TL::M;
    const Ptr<const cf32> src = a.in.sub(tile * TILE, valid);
#pragma unroll
    for (int i = 0; i < TILE / 2 / NT; ++i) {
      const int e = 2 * (tid + NT * i);
      if (e < valid) cp_async16(buf, e, src, e);
    }
  }

  ESTL_HD static void compute(const TileArgs& a, long long tile, int tid, const Ptr<cf32>& buf) {
    const int t = tid & (TL::T - 1);
    const int c = tid >> TL::LOGT;
    const long long row = tile * C + c;
    const bool valid = row < a.rows;
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    cf32 v[TL::E];
#pragma unroll
    for (int j = 0; j < TL::E; ++j) v[j] = conj_if(buf[c * TL::M + t + TL::T * j], a.sgn);
    ESTL_SYNC();  // the buffer becomes the exchange buffer
    run_passes<TL, 0>(v, t, c, buf, tw, typename Base::Sidx{});
    if (valid) {
      const Ptr<cf32> out = a.out.sub(row * TL::M, TL::M);
#pragma unroll
      for (int j = 0; j < TL::E; ++j) stcs(out, t + TL::T * j, conj_if(v[j], a.sgn));
    }
  }

  ESTL_HD static void run(const TileArgs& a, long long cta, int tid, cf32* sm) {
    pipe_loop<PipeSingleKernel>(a, cta, a.grid, tid, sm);
  }
};

// Four-step column pass: tile = C adjacent columns of one transform (column
// mapping, as ColKernel); the tile lands in shared memory as [n2][c].
template <int LOGM, int LOGE, int LOGR, int LOGC>
struct PipeColKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  using Base = ColKernel<LOGM, LOGE, LOGR, LOGC>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  static constexpr int TILE = C * TL::M;
  // each buffer a multiple of 16 bytes, so that the second one stays aligned
  static constexpr long long TILE_BUF = (((Base::SMEM_ELEMS > TILE) ? Base::SMEM_ELEMS : TILE) + 1) & ~1LL;
  static constexpr long long SMEM_ELEMS = 2 * TILE_BUF;
  static constexpr int MIN_BLOCKS = min_blocks(NT, TL::E);
  static_assert(C >= 2 && (TILE / 2) % NT == 0, "16-byte chunks must split evenly");

  ESTL_HD static long long ntiles(const TileArgs& a) { return a.rows << (a.logn - LOGM - LOGC); }

  ESTL_HD static void issue(const TileArgs& a, long long tile, int tid, const Ptr<cf32>& buf) {
    const int logn1 = a.logn - LOGM;
    const int N = 1 << a.logn;
    const int nblk = 1 << (logn1 - LOGC);
    const long long f = tile / nblk;
    const int n1_0 = (int)(tile - f * nblk) * C;
    const Ptr<const cf32> src = a.in.sub(f * N, N);
#pragma unroll
    for (int i = 0; i < TILE / 2 / NT; ++i) {
      const int q = tid + NT * i;     // 16-byte chunk of the tile
      const int n2 = q / (C / 2);     // row
      const int off = 2 * (q % (C / 2));
      cp_async16(buf, n2 * C + off, src, n1_0 + off + ((long long)n2 << logn1));
    }
  }

  ESTL_HD static void compute(const TileArgs& a, long long tile, int tid, const Ptr<cf32>& buf) {
    const int c = tid & (C - 1);
    const int t = tid >> LOGC;
    const int logn1 = a.logn - LOGM;
    const int N = 1 << a.logn;
    const int nblk = 1 << (logn1 - LOGC);
    const long long f = tile / nblk;
    const int n1 = (int)(tile - f * nblk) * C + c;
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    cf32 v[TL::E];
#pragma unroll
    for (int j = 0; j < TL::E; ++j) v[j] = conj_if(buf[(t + TL::T * j) * C + c], a.sgn);
    ESTL_SYNC();
    run_passes<TL, 0>(v, t, c, buf, tw, typename Base::Sidx{});
    Base::store_twiddled(v, a.out.sub(f * N, N), n1, t, a.logn, a.bank);
  }

  ESTL_HD static void run(const TileArgs& a, long long cta, int tid, cf32* sm) {
    pipe_loop<PipeColKernel>(a, cta, a.grid, tid, sm);
  }
};

// Four-step row pass: tile = C contiguous scratch rows (row mapping, as
// RowKernel), results stored column-fastest through the same buffer.
template <int LOGM, int LOGE, int LOGR, int LOGC>
struct PipeRowKernel {
  using TL = Tile<LOGM, LOGE, LOGR>;
  static constexpr int C = 1 << LOGC;
  static constexpr int NT = TL::T * C;
  static constexpr int TILE = C * TL::M;
  // row-major exchange layout (rows CS apart, conflict-free for the
  // column-fastest remap of the stores)
  static constexpr int CS = row_stride(TL::MP, C);
  struct Sidx {
    ESTL_HD int operator()(int c, int m) const { return c * CS + TL::pad(m); }
  };
  // each buffer a multiple of 16 bytes, so that the second one stays aligned
  static constexpr long long TILE_BUF = (((C * CS > TILE) ? C * CS : TILE) + 1) & ~1LL;
  static constexpr long long SMEM_ELEMS = 2 * TILE_BUF;
  static constexpr int MIN_BLOCKS = min_blocks(NT, TL::E);
  static_assert((TILE / 2) % NT == 0, "16-byte chunks must split evenly");

  ESTL_HD static long long ntiles(const TileArgs& a) { return a.rows << (a.logn - LOGM - LOGC); }

  ESTL_HD static void issue(const TileArgs& a, long long tile, int tid, const Ptr<cf32>& buf) {
    const Ptr<const cf32> src = a.in.sub(tile * TILE, TILE);  // C whole rows of the scratch
#pragma unroll
    for (int i = 0; i < TILE / 2 / NT; ++i) {
      const int e = 2 * (tid + NT * i);
      cp_async16(buf, e, src, e);
    }
  }

  ESTL_HD static void compute(const TileArgs& a, long long tile, int tid, const Ptr<cf32>& buf) {
    const int t = tid & (TL::T - 1);
    const int c = tid >> TL::LOGT;
    const int N = 1 << a.logn;
    const int logn2 = a.logn - LOGM;
    const int nblk = 1 << (logn2 - LOGC);
    const long long f = tile / nblk;
    const int k2_0 = (int)(tile - f * nblk) * C;
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    const Sidx sidx{};
    cf32 v[TL::E];
#pragma unroll
    for (int j = 0; j < TL::E; ++j) v[j] = buf[c * TL::M + t + TL::T * j];
    ESTL_SYNC();
    run_passes<TL, 0>(v, t, c, buf, tw, sidx);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) buf[sidx(c, t + TL::T * j)] = v[j];
    ESTL_SYNC();
    const int c2 = tid & (C - 1);
    const int t2 = tid >> LOGC;
    const Ptr<cf32> out = a.out.sub(f * N, N);
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const int k1 = t2 + TL::T * j;
      stcs(out, k2_0 + c2 + (k1 << logn2), conj_if(buf[sidx(c2, k1)], a.sgn));
    }
  }

  ESTL_HD static void run(const TileArgs& a, long long cta, int tid, cf32* sm) {
    pipe_loop<PipeRowKernel>(a, cta, a.grid, tid, sm);
  }
};

}  // namespace estl
