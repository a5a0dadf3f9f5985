// cluster_core.cuh — whole transforms of 2^13..2^17 points in one HBM pass,
// each transform split over a thread-block cluster of R CTAs.
//
// The reference runs one Stockham pass per kernel with a full HBM round trip
// per pass (FFT_OpenCL_Contiguous.h:55-61,107-124).  A single CTA can keep a
// whole transform on chip only up to 2^14 points (SingleKernel), and a 2^14-
// point tile fills half of an SM's registers: one CTA per SM, whose barriers
// then stall the whole SM.  Here each CTA holds 2^12..2^13 points, two or more
// CTAs share an SM, and the R CTAs of a cluster together run one N-point
// transform as a four-step N = N1 * N2 whose transpose goes through
// distributed shared memory instead of HBM:
//
//   phase A  CTA r owns the W = N1 / R adjacent columns n1 = r W + c: loads
//            x[n1 + N1 n2] (runs of W complex), N2-point column DFTs (radix
//            passes, exchanges in its own shared memory), twiddle
//            w_N^{n1 k2}, writes Z[c][k2] into its own shared memory
//   cluster barrier (arrive with release, then the gather of the columns
//            this CTA holds itself, then wait)
//            CTA r gathers rows k2 = r H + c' (H = N2 / R) of all N1 columns:
//            column n1 of row k2 lives in CTA n1 / W at Z[n1 mod W][k2]
//   phase B  first radix pass in registers (it consumes every gathered
//            value), cluster barrier (relaxed arrive: every read of a peer's
//            Z has delivered its value; Z may be reused), the other passes,
//            stores X[k2 + N2 k1] (runs of H complex)
//
// Remote traffic per element: (R - 1) / R of the data crosses CTAs once, 8 B
// per element read through distributed shared memory; HBM traffic is the
// compulsory 16 B per element.  A warp's gather reads 32 consecutive k2 of one
// column: one contiguous 256-byte run of the remote CTA's shared memory (the
// same gather with lanes 8 B apart in scattered rows ran 3x slower).  Z rows
// are padded to N2 + 1 elements so that phase A's writes (lanes = adjacent
// columns, one row apart) are free of bank conflicts.
#pragma once
#include "bulk_core.cuh"

// Cluster barrier, split into its arrive and its wait.  ESTL_CLUSTER_ARRIVE
// releases this thread's earlier writes to the cluster; the relaxed form
// orders nothing and is used only where every earlier read has delivered its
// value into a register that later work has already consumed.
#ifdef ESTL_EMU
void estl_emu_cluster_arrive();
void estl_emu_cluster_wait();
// Shared memory of CTA `rank` of the emulated cluster; *n = its elements.
estl::cf32* estl_emu_cluster_smem(int rank, long long* n);
#define ESTL_CLUSTER_ARRIVE() estl_emu_cluster_arrive()
#define ESTL_CLUSTER_ARRIVE_RELAXED() estl_emu_cluster_arrive()
#define ESTL_CLUSTER_WAIT() estl_emu_cluster_wait()
#else
#define ESTL_CLUSTER_ARRIVE() asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory")
#define ESTL_CLUSTER_ARRIVE_RELAXED() asm volatile("barrier.cluster.arrive.relaxed.aligned;\n" ::: "memory")
#define ESTL_CLUSTER_WAIT() asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory")
#endif

namespace estl {

// Read-only view of a buffer of another CTA of the cluster: the same offset
// in that CTA's shared memory as `local` has in this CTA's.
struct PeerBuf {
#if defined(__CUDA_ARCH__)
  uint32_t addr;  // shared::cluster address of element 0
#else
  const cf32* p;
#endif
  long long n;
  ESTL_HD cf32 operator[](int i) const {
    ESTL_CHECK(i, n, "distributed shared memory index");
#if defined(__CUDA_ARCH__)
    float x, y;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];\n"
                 : "=f"(x), "=f"(y)
                 : "r"(addr + 8u * (uint32_t)i)
                 : "memory");
    return {x, y};
#else
    return p[i];
#endif
  }
};

ESTL_HD PeerBuf peer_buf(const cf32* local, long long n, int self, int rank) {
#if defined(__CUDA_ARCH__)
  (void)self;
  uint32_t ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(ra) : "r"(smem_u32(local)), "r"(rank));
  return PeerBuf{ra, n};
#elif defined(ESTL_EMU)
  long long own_n = 0, peer_n = 0;
  const cf32* own = estl_emu_cluster_smem(self, &own_n);
  const cf32* peer = estl_emu_cluster_smem(rank, &peer_n);
  const long long off = local - own;
  ESTL_CHECK(off + n, peer_n + 1, "distributed shared memory buffer");
  return PeerBuf{peer + off, n};
#else
  (void)self;
  (void)rank;
  return PeerBuf{local, n};  // host compilation pass of nvcc: never executed
#endif
}

template <int LOGN, int LOGR, int LOGN2, int LOGE>
struct ClusterKernel {
  static constexpr int R = 1 << LOGR;
  static constexpr int LOGN1 = LOGN - LOGN2;
  static constexpr int N = 1 << LOGN;
  static constexpr int N2 = 1 << LOGN2;
  static constexpr int LOGW = LOGN1 - LOGR, W = 1 << LOGW;  // phase A: columns per CTA
  static constexpr int LOGH = LOGN2 - LOGR, H = 1 << LOGH;  // phase B: rows per CTA
  using TA = Tile<LOGN2, LOGE, 4>;                          // column DFTs (N2 points)
  using TB = Tile<LOGN1, LOGE, 4>;                          // row DFTs (N1 points)
  static constexpr int NT = TA::T * W;
  static constexpr int ZS = N2 + 1;  // Z row stride (one row per column c)
  static constexpr int XA = TA::MP * W, XB = TB::MP * H, ZE = W * ZS;
  static constexpr int SMEM_ELEMS = (((XA > XB ? XA : XB) > ZE ? (XA > XB ? XA : XB) : ZE) + 1) & ~1;
  static constexpr int MIN_BLOCKS = min_blocks(NT, TA::E);
  static constexpr int LOG_CLUSTER = LOGR;  // kernel tables: cluster of 2^LOG_CLUSTER CTAs
  static constexpr int LOG_SPLIT = LOGN2;   // kernel tables: column DFT length 2^LOG_SPLIT
  static_assert(NT == TB::T * H, "both phases run the same threads");
  static_assert(NT <= 1024, "too many threads");
  static_assert(R >= 2 && R <= 16, "clusters of 2..16 CTAs");
  static_assert(W >= 16 && H >= 16, "runs of at least 16 complex (128 B) in HBM");
  static_assert(W % TB::T == 0, "a row slot's source CTA is fixed per slot");
  static_assert(TA::E == 16 || TA::E == 32, "four-step twiddle of 16 or 32 elements per thread");

  struct SidxA {  // phase A exchange: [m][c]
    ESTL_HD int operator()(int c, int m) const { return TA::pad(m) * W + c; }
  };
  struct SidxB {  // phase B exchange: [m][c']
    ESTL_HD int operator()(int c, int m) const { return TB::pad(m) * H + c; }
  };

  ESTL_HD static void run(const TileArgs& a, long long cta, int tid, cf32* smraw) {
    const int rank = (int)(cta & (R - 1));
    const long long f = cta >> LOGR;  // the grid is exactly rows * R CTAs
    const Ptr<const cf32> in = a.in.sub(xbase(a, f, N), N);
    const Ptr<cf32> out = a.out.sub(xbase(a, f, N), N);
    const Ptr<cf32> sm{smraw, SMEM_ELEMS};
    cf32 v[TA::E];
    // phase A: column DFTs of this CTA's W columns
    {
      const int c = tid & (W - 1), t = tid >> LOGW;
      const int n1 = rank * W + c;
      int off = n1 + (t << LOGN1);
#pragma unroll
      for (int j = 0; j < TA::E; ++j, off += TA::T << LOGN1) v[j] = conj_if(ldcs(in, off), a.sgn);
      run_passes<TA, 0>(v, t, c, sm, a.bank.sub(N2, N2), SidxA{});
      fourstep_twiddle<TA>(v, n1, t, LOGN, a.bank);
      ESTL_SYNC();  // the last exchange's reads are done: Z overwrites the buffer
#pragma unroll
      for (int j = 0; j < TA::E; ++j) sm[c * ZS + t + TA::T * j] = v[j];
    }
    ESTL_CLUSTER_ARRIVE();  // release: this CTA's Z to the cluster
    ESTL_SYNC();            // ... and to this CTA
    const int c = tid & (H - 1), t = tid >> LOGH;
    const int k2 = rank * H + c;
    {
      constexpr int SPAN = W / TB::T;  // slots per source CTA
      // the columns this CTA holds first, while the other CTAs arrive
#pragma unroll
      for (int j = 0; j < TB::E; ++j)
        if (j / SPAN == rank) v[j] = sm[((t + TB::T * j) & (W - 1)) * ZS + k2];
      ESTL_CLUSTER_WAIT();  // every CTA's Z is complete and visible
      PeerBuf z[R];
#pragma unroll
      for (int q = 0; q < R; ++q) z[q] = peer_buf(smraw, ZE, rank, q);
#pragma unroll
      for (int j = 0; j < TB::E; ++j)
        if (j / SPAN != rank) v[j] = z[j / SPAN][((t + TB::T * j) & (W - 1)) * ZS + k2];
    }
    const Ptr<const cf32> twb = a.bank.sub(1 << LOGN1, 1 << LOGN1);
    TB::template compute<0>(v, t, twb);  // consumes every gathered value
    ESTL_CLUSTER_ARRIVE_RELAXED();       // this CTA's reads of the cluster's Z are done
    ESTL_CLUSTER_WAIT();                 // everyone's are: Z becomes exchange space again
    if constexpr (TB::P > 1) {
#pragma unroll
      for (int j = 0; j < TB::E; ++j) sm[SidxB{}(c, TB::template out_pos<0>(t, j))] = v[j];
      ESTL_SYNC();
#pragma unroll
      for (int j = 0; j < TB::E; ++j) v[j] = sm[SidxB{}(c, t + TB::T * j)];
      ESTL_SYNC();
    }
    run_passes<TB, 1>(v, t, c, sm, twb, SidxB{});
#pragma unroll
    for (int j = 0; j < TB::E; ++j) stcs(out, k2 + ((t + TB::T * j) << LOGN2), conj_if(v[j], a.sgn));
  }
};

}  // namespace estl
