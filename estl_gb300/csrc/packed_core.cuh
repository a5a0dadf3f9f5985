// packed_core.cuh — the persistent uneven-batch kernel body (device and host
// emulator).  One CTA of 256 threads takes work items from a queue and runs
// the tile body of the item's size class (fft_core.cuh).
#pragma once
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

ESTL_CX long long cmax(long long a, long long b) { return a > b ? a : b; }
// Dynamic shared memory of the packed kernel: the largest tile of every class.
constexpr long long kPackedSmemElems = cmax(
    cmax(cmax(cmax(PSingle1::SMEM_ELEMS, PSingle2::SMEM_ELEMS), cmax(PSingle3::SMEM_ELEMS, PSingle4::SMEM_ELEMS)),
         cmax(cmax(PSingle5::SMEM_ELEMS, PSingle6::SMEM_ELEMS), cmax(PSingle7::SMEM_ELEMS, PSingle8::SMEM_ELEMS))),
    cmax(cmax(cmax(PSingle9::SMEM_ELEMS, PSingle10::SMEM_ELEMS), cmax(PSingle11::SMEM_ELEMS, PSingle12::SMEM_ELEMS)),
         cmax(cmax(cmax(PCol6::SMEM_ELEMS, PCol7::SMEM_ELEMS), cmax(PCol8::SMEM_ELEMS, PCol9::SMEM_ELEMS)),
              cmax(PRow7::SMEM_ELEMS, cmax(PRow8::SMEM_ELEMS, PRow9::SMEM_ELEMS)))));

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

ESTL_HD void packed_dispatch(const PackedArgs& a, const PackedItem& it, int tid, cf32* sm) {
  if (it.kind == PK_SINGLE) {
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
