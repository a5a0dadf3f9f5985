// packed_core.cuh — the persistent uneven-batch kernel body (device and host
// emulator).  One CTA of 256 threads takes work items from a queue and runs
// the tile body of the item's size class (fft_core.cuh), or a whole FFT
// convolution (PackedConvTile below).
#pragma once
#include "conv_core.cuh"
#include "fft_core.cuh"
#include "packed_plan.h"

namespace estl {

// Iterations of the dependency wait before it gives up (~2^24 x 128 ns, a few
// seconds): a row item whose column items never finish records the failure in
// *error and is skipped instead of spinning forever.
constexpr unsigned long long kPackedSpinLimit = 1ULL << 24;

struct PackedArgs {
  Ptr<const PackedItem> items;
  long long item_base;  // first item of this launch
  long long nitems;     // items of this launch
  Ptr<const int> class_list;
  Ptr<const long long> offsets;
  Ptr<const long long> scratch_off;
  Ptr<const int> ncol;
  Ptr<const cf32> in;
  Ptr<cf32> out;
  Ptr<cf32> scratch;
  Ptr<const cf32> bank;
  unsigned int* next;  // persistent mode: work counter (zero at launch)
  unsigned int* done;  // column items finished per transform (zero at launch)
  int* error;          // set to 1 when a dependency wait gives up
  float sgn;
  int persistent;
  // test hook (estl_packed_plan_set_test_hook): items of this kind are left
  // out (-1: none), and the dependency wait gives up after spin_limit polls
  int skip_kind = -1;
  unsigned long long spin_limit = kPackedSpinLimit;
  // mixed batches: convolution items (PackedConv, grouped by padded length)
  Ptr<const PackedConv> convs{nullptr, 0};
  Ptr<const int> conv_class_list{nullptr, 0};
  Ptr<const float> csig{nullptr, 0};
  Ptr<const float> cfilt{nullptr, 0};
  Ptr<float> cout{nullptr, 0};
};

// ---------------------------------------------------------------------------
// A convolution item: C requests of padded length M = 2^LOGM in one CTA, each
// from one complex transform of z = x + i 2^k h (the real signal and the real
// filter as the two halves; 2^k, an exact power of two, balances their
// energies so that FP32 rounding is relative to both), with Zm_m = Z_{-m mod M}
// from one shared-memory exchange:
//   X = (Z + conj Zm) / 2,   2^k H = (Z - conj Zm) / (2i),
//   Y = X * 2^k H  (X * conj(2^k H) for correlation),
//   y = Re(FFT(conj Y)) / M * 2^-k,  or / (M * 2^k H_0) with the DC
//   normalisation (2^k H_0 = Im Z_0, the filter's sum times 2^k).
// Two transforms per request and no spectrum in global memory: the signal
// and the filter are read once, the output written once.  The transforms run
// with the forward sign whatever the batch's direction.
// ---------------------------------------------------------------------------
template <int LOGM, int LOGE, int LOGC>
struct PackedConvTile {
  using B = ConvSingleKernel<LOGM, LOGE, 4, LOGC>;
  using TL = typename B::TL;
  using Sidx = typename B::Sidx;
  static constexpr int C = B::C;
  static constexpr int NT = B::NT;
  static constexpr int SMEM_ELEMS = C * B::CS;  // the mirror exchange, also for one-pass tiles
  static_assert(SMEM_ELEMS >= NT, "row reduction scratch");

  ESTL_HD static void body(const PackedArgs& a, const PackedItem& it, int tid, cf32* smraw) {
    const int t = tid & (TL::T - 1);
    const int c = tid >> TL::LOGT;
    const bool valid = c < it.blk;
    // the request's descriptor is read where it is used (here, then at the
    // store) rather than held in registers across the transforms
    const long long ri = valid ? a.conv_class_list[(long long)it.tf + c] : 0;
    const Ptr<const cf32> tw = a.bank.sub(TL::M, TL::M);
    const Ptr<cf32> sm{smraw, SMEM_ELEMS};
    const Sidx sidx{};
    cf32 v[TL::E];
    float ex = 0.f, eh = 0.f;
    {
      PackedConv r{};
      if (valid) r = a.convs[ri];
      const Ptr<const float> xs = valid ? a.csig.sub(r.sig_off, r.sig_len) : Ptr<const float>{a.csig.p, 0};
      const Ptr<const float> hs = valid ? a.cfilt.sub(r.filt_off, r.filt_len) : Ptr<const float>{a.cfilt.p, 0};
#pragma unroll
      for (int j = 0; j < TL::E; ++j) {
        const int pos = t + TL::T * j;
        v[j] = cf32{pos < r.sig_len ? xs[pos] : 0.f, pos < r.filt_len ? hs[pos] : 0.f};
        ex += v[j].x * v[j].x;
        eh += v[j].y * v[j].y;
      }
    }
    row_sum2<TL::T, NT>(ex, eh, tid, reinterpret_cast<float*>(smraw));
    const int k = balance_exp(ex, eh);  // 2^k ~ sqrt(ex / eh)
    {
      const float gk = pow2_f(k);
#pragma unroll
      for (int j = 0; j < TL::E; ++j) v[j].y *= gk;
    }
    run_passes<TL, 0>(v, t, c, sm, tw, sidx);
    ESTL_SYNC();
#pragma unroll
    for (int j = 0; j < TL::E; ++j) sm[sidx(c, t + TL::T * j)] = v[j];
    ESTL_SYNC();
    const float h0 = sm[sidx(c, 0)].y;  // Im Z_0 = 2^k * sum of the filter
    const float cj = valid && a.convs[ri].correlate ? -1.f : 1.f;
#pragma unroll
    for (int j = 0; j < TL::E; ++j) {
      const cf32 zm = sm[sidx(c, (TL::M - (t + TL::T * j)) & (TL::M - 1))];
      const cf32 x{0.5f * (v[j].x + zm.x), 0.5f * (v[j].y - zm.y)};
      const cf32 h{0.5f * (v[j].y + zm.y), -0.5f * (v[j].x - zm.x) * cj};
      v[j] = cconj(cmul(x, h));
    }
    ESTL_SYNC();  // before the passes reuse the exchange buffer
    run_passes<TL, 0>(v, t, c, sm, tw, sidx);
    if (valid) {
      const PackedConv r = a.convs[ri];
      const Ptr<float> o = a.cout.sub(r.out_off, r.out_len);
      const float g = r.dc_norm ? 1.f / ((float)TL::M * h0) : pow2_f(-k) / (float)TL::M;
#pragma unroll
      for (int j = 0; j < TL::E; ++j) {
        const int m = (t + TL::T * j - r.out_shift) & (TL::M - 1);  // the cyclic shift wraps
        if (m < r.out_len) o[m] = v[j].x * g;
      }
    }
  }
};

// Size-class tile bodies, all with 256 threads per CTA.
using PSingle1 = SingleKernel<1, 1, 4, 8>;
using PSingle2 = SingleKernel<2, 2, 4, 8>;
using PSingle3 = SingleKernel<3, 3, 4, 8>;
using PSingle4 = SingleKernel<4, 4, 4, 8>;
using PSingle5 = SingleKernel<5, 4, 4, 7>;
using PSingle6 = SingleKernel<6, 4, 4, 6>;
using PSingle7 = SingleKernel<7, 4, 4, 5>;
using PSingle8 = SingleKernel<8, 4, 4, 4>;
using PSingle9 = SingleKernel<9, 4, 4, 3>;
using PSingle10 = SingleKernel<10, 4, 4, 2>;
using PSingle11 = SingleKernel<11, 4, 4, 1>;
using PSingle12 = SingleKernel<12, 4, 4, 0>;
using PCol6 = ColKernel<6, 4, 4, 6>;
using PCol7 = ColKernel<7, 4, 4, 5>;
using PCol8 = ColKernel<8, 4, 4, 4>;
using PCol9 = ColKernel<9, 4, 4, 3>;
using PRow7 = RemapRowKernel<7, 4, 4, 5>;
using PRow8 = RemapRowKernel<8, 4, 4, 4>;
using PRow9 = RemapRowKernel<9, 4, 4, 3>;
// convolution items: the single tiles' shapes (256 threads)
using PConv1 = PackedConvTile<1, 1, 8>;
using PConv2 = PackedConvTile<2, 2, 8>;
using PConv3 = PackedConvTile<3, 3, 8>;
using PConv4 = PackedConvTile<4, 4, 8>;
using PConv5 = PackedConvTile<5, 4, 7>;
using PConv6 = PackedConvTile<6, 4, 6>;
using PConv7 = PackedConvTile<7, 4, 5>;
using PConv8 = PackedConvTile<8, 4, 4>;
using PConv9 = PackedConvTile<9, 4, 3>;
using PConv10 = PackedConvTile<10, 4, 2>;
using PConv11 = PackedConvTile<11, 4, 1>;
using PConv12 = PackedConvTile<12, 4, 0>;

ESTL_CX long long cmax(long long a, long long b) { return a > b ? a : b; }
// Dynamic shared memory of the packed kernel: the largest tile of every class.
constexpr long long kPackedTileSmemElems = cmax(
    cmax(cmax(cmax(PSingle1::SMEM_ELEMS, PSingle2::SMEM_ELEMS), cmax(PSingle3::SMEM_ELEMS, PSingle4::SMEM_ELEMS)),
         cmax(cmax(PSingle5::SMEM_ELEMS, PSingle6::SMEM_ELEMS), cmax(PSingle7::SMEM_ELEMS, PSingle8::SMEM_ELEMS))),
    cmax(cmax(cmax(PSingle9::SMEM_ELEMS, PSingle10::SMEM_ELEMS), cmax(PSingle11::SMEM_ELEMS, PSingle12::SMEM_ELEMS)),
         cmax(cmax(cmax(PCol6::SMEM_ELEMS, PCol7::SMEM_ELEMS), cmax(PCol8::SMEM_ELEMS, PCol9::SMEM_ELEMS)),
              cmax(PRow7::SMEM_ELEMS, cmax(PRow8::SMEM_ELEMS, PRow9::SMEM_ELEMS)))));
constexpr long long kPackedConvSmemElems = cmax(
    cmax(cmax(cmax(PConv1::SMEM_ELEMS, PConv2::SMEM_ELEMS), cmax(PConv3::SMEM_ELEMS, PConv4::SMEM_ELEMS)),
         cmax(cmax(PConv5::SMEM_ELEMS, PConv6::SMEM_ELEMS), cmax(PConv7::SMEM_ELEMS, PConv8::SMEM_ELEMS))),
    cmax(cmax(PConv9::SMEM_ELEMS, PConv10::SMEM_ELEMS), cmax(PConv11::SMEM_ELEMS, PConv12::SMEM_ELEMS)));
constexpr long long kPackedSmemElems = cmax(kPackedTileSmemElems, kPackedConvSmemElems);

// ---- synchronisation helpers (device: PTX memory model; emulator: builtins)
ESTL_HD unsigned int atomic_add_u32(unsigned int* p, unsigned int v) {
#if defined(__CUDA_ARCH__)
  return atomicAdd(p, v);
#else
  return __atomic_fetch_add(p, v, __ATOMIC_ACQ_REL);
#endif
}
ESTL_HD unsigned int load_acquire_u32(const unsigned int* p) {
#if defined(__CUDA_ARCH__)
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
#else
  return __atomic_load_n(p, __ATOMIC_ACQUIRE);
#endif
}
ESTL_HD void fence_gpu() {
#if defined(__CUDA_ARCH__)
  __threadfence();
#else
  __atomic_thread_fence(__ATOMIC_SEQ_CST);
#endif
}
ESTL_HD void backoff() {
#if defined(__CUDA_ARCH__)
  __nanosleep(128);
#endif
}

template <class K>
ESTL_HD void packed_single(const PackedArgs& a, const PackedItem& it, int tid, cf32* sm) {
  static_assert(K::SMEM_ELEMS <= kPackedSmemElems, "tile needs more shared memory than the packed kernel has");
  static_assert(K::NT == kPackedThreads, "packed tiles run with 256 threads");
  const int c = tid >> K::TL::LOGT;
  const bool valid = c < it.blk;
  const int n = 1 << it.logn;
  Ptr<const cf32> in{a.in.p, 0};
  Ptr<cf32> out{a.out.p, 0};
  if (valid) {
    const long long off = a.offsets[a.class_list[(long long)it.tf + c]];
    in = a.in.sub(off, n);
    out = a.out.sub(off, n);
  }
  K::body(in, out, valid, tid, sm, a.bank, a.sgn);
}

template <class K>
ESTL_HD void packed_col(const PackedArgs& a, const PackedItem& it, int tid, cf32* sm) {
  static_assert(K::SMEM_ELEMS <= kPackedSmemElems, "tile needs more shared memory than the packed kernel has");
  static_assert(K::NT == kPackedThreads, "packed tiles run with 256 threads");
  const int n = 1 << it.logn;
  const long long off = a.offsets[it.tf];
  K::body(a.in.sub(off, n), a.scratch.sub(a.scratch_off[it.tf], n), it.blk, it.logn, tid, sm, a.bank, a.sgn);
}

template <class K>
ESTL_HD void packed_row(const PackedArgs& a, const PackedItem& it, int tid, cf32* sm) {
  static_assert(K::SMEM_ELEMS <= kPackedSmemElems, "tile needs more shared memory than the packed kernel has");
  static_assert(K::NT == kPackedThreads, "packed tiles run with 256 threads");
  const int n = 1 << it.logn;
  const long long off = a.offsets[it.tf];
  K::body(a.scratch.sub(a.scratch_off[it.tf], n), a.out.sub(off, n), it.blk, it.logn, tid, sm, a.bank, a.sgn);
}

// Convolution items run as separate device functions: inlined beside every
// transform tile, their register demand made the whole kernel spill.
template <class K>
#if defined(__CUDA_ARCH__)
__device__ __noinline__
#else
inline
#endif
void packed_conv(const PackedArgs& a, const PackedItem& it, int tid, cf32* sm) {
  static_assert(K::NT == kPackedThreads, "packed tiles run with 256 threads");
  K::body(a, it, tid, sm);
}

ESTL_HD void packed_dispatch(const PackedArgs& a, const PackedItem& it, int tid, cf32* sm) {
  if (it.kind == PK_CONV) {
    switch (it.logn) {
      case 1: packed_conv<PConv1>(a, it, tid, sm); break;
      case 2: packed_conv<PConv2>(a, it, tid, sm); break;
      case 3: packed_conv<PConv3>(a, it, tid, sm); break;
      case 4: packed_conv<PConv4>(a, it, tid, sm); break;
      case 5: packed_conv<PConv5>(a, it, tid, sm); break;
      case 6: packed_conv<PConv6>(a, it, tid, sm); break;
      case 7: packed_conv<PConv7>(a, it, tid, sm); break;
      case 8: packed_conv<PConv8>(a, it, tid, sm); break;
      case 9: packed_conv<PConv9>(a, it, tid, sm); break;
      case 10: packed_conv<PConv10>(a, it, tid, sm); break;
      case 11: packed_conv<PConv11>(a, it, tid, sm); break;
      default: packed_conv<PConv12>(a, it, tid, sm); break;
    }
  } else if (it.kind == PK_SINGLE) {
    switch (it.logn) {
      case 1: packed_single<PSingle1>(a, it, tid, sm); break;
      case 2: packed_single<PSingle2>(a, it, tid, sm); break;
      case 3: packed_single<PSingle3>(a, it, tid, sm); break;
      case 4: packed_single<PSingle4>(a, it, tid, sm); break;
      case 5: packed_single<PSingle5>(a, it, tid, sm); break;
      case 6: packed_single<PSingle6>(a, it, tid, sm); break;
      case 7: packed_single<PSingle7>(a, it, tid, sm); break;
      case 8: packed_single<PSingle8>(a, it, tid, sm); break;
      case 9: packed_single<PSingle9>(a, it, tid, sm); break;
      case 10: packed_single<PSingle10>(a, it, tid, sm); break;
      case 11: packed_single<PSingle11>(a, it, tid, sm); break;
      default: packed_single<PSingle12>(a, it, tid, sm); break;
    }
  } else if (it.kind == PK_COL) {
    switch (it.logn >> 1) {  // column DFT length N2 = 2^floor(log2 n / 2) (packed_logn2)
      case 6: packed_col<PCol6>(a, it, tid, sm); break;
      case 7: packed_col<PCol7>(a, it, tid, sm); break;
      case 8: packed_col<PCol8>(a, it, tid, sm); break;
      default: packed_col<PCol9>(a, it, tid, sm); break;
    }
  } else {
    switch (it.logn - (it.logn >> 1)) {  // row DFT length N1
      case 7: packed_row<PRow7>(a, it, tid, sm); break;
      case 8: packed_row<PRow8>(a, it, tid, sm); break;
      default: packed_row<PRow9>(a, it, tid, sm); break;
    }
  }
}

// One CTA.  Persistent mode: loop over the launch's items through the work
// counter; otherwise run item `cta` of the launch.  `slot` is a CTA-shared
// int used to broadcast the item index and the dependency-wait result.
ESTL_HD void packed_run(const PackedArgs& a, long long cta, int tid, cf32* sm, int* slot) {
  for (;;) {
    long long idx;
    if (a.persistent) {
      if (tid == 0) slot[0] = (int)atomic_add_u32(a.next, 1u);
      ESTL_SYNC();
      idx = slot[0];
      ESTL_SYNC();
      if (idx >= a.nitems) return;
    } else {
      idx = cta;
      if (idx >= a.nitems) return;
    }
    const PackedItem it = a.items[a.item_base + idx];
    if (it.kind == a.skip_kind) {
      // test hook: the item is left out (a skipped column item is never counted)
    } else if (it.kind == PK_ROW) {
      // wait until every column item of this transform has been written
      if (tid == 0) {
        const unsigned int need = (unsigned int)a.ncol[it.tf];
        unsigned long long spins = 0;
        int ok = 1;
        while (load_acquire_u32(a.done + it.tf) < need) {
          if (++spins > a.spin_limit) {
            ok = 0;
            *a.error = 1;
            break;
          }
          backoff();
        }
        slot[1] = ok;
      }
      ESTL_SYNC();
      const int ok = slot[1];
      ESTL_SYNC();
      if (ok) packed_dispatch(a, it, tid, sm);
    } else {
      packed_dispatch(a, it, tid, sm);
    }
    if (it.kind == PK_COL && it.kind != a.skip_kind) {
      fence_gpu();  // this thread's scratch stores before the count
      ESTL_SYNC();
      if (tid == 0) atomic_add_u32(a.done + it.tf, 1u);
    }
    ESTL_SYNC();  // shared memory is reused by the next item
    if (!a.persistent) return;
  }
}

}  // namespace estl
