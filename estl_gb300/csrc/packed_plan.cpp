// packed_plan.cpp — see packed_plan.h.
#include "packed_plan.h"
#include "planner.h"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace estl {

int packed_single_logc(int logn) {
  // 256 threads: 16 elements per thread for n >= 16, n elements (one thread) below
  static const int c[13] = {0, 8, 8, 8, 8, 7, 6, 5, 4, 3, 2, 1, 0};
  return c[logn];
}
int packed_logn2(int logn) { return logn / 2; }
static int logc_for_m(int logm) { return 12 - logm; }  // 256 threads = (2^logm / 16) * C
int packed_col_logc(int logn) { return logc_for_m(packed_logn2(logn)); }
int packed_row_logc(int logn) { return logc_for_m(logn - packed_logn2(logn)); }

bool build_packed_layout(const long long* offsets, const long long* sizes, long long count, bool persistent,
                         PackedLayout* out, std::string* err, const ConvReq* convs, long long nconv,
                         int conv_flags) {
  PackedLayout L;
  L.persistent = persistent;
  if (nconv < 0 || nconv > (1LL << 30) || (nconv > 0 && !convs)) {
    if (err) *err = "bad convolution list";
    return false;
  }
  if (count < 0 || (count > 0 && (!offsets || !sizes)) || (count == 0 && nconv == 0)) {
    if (err) *err = "need at least one transform or convolution";
    return false;
  }
  if (count > (1LL << 30)) {
    if (err) *err = "too many transforms";
    return false;
  }
  if (conv_flags & ~(CONV_CORRELATE | CONV_REFERENCE_COMPAT | CONV_NO_PAIRING | CONV_COMPLEX)) {
    if (err) *err = "convolution flags of a mixed batch: CORRELATE, REFERENCE_COMPAT, NO_PAIRING, COMPLEX (FP32)";
    return false;
  }
  L.offsets.assign(offsets, offsets + count);
  L.lognv.resize(count);
  L.scratch_off.assign(count, -1);
  L.ncol.assign(count, 0);
  for (long long i = 0; i < count; ++i) {
    const long long n = sizes[i];
    int l = 0;
    while ((1LL << l) < n) l++;
    if (n < 2 || (1LL << l) != n || l > kPackedMaxLog) {
      if (err) *err = "transform " + std::to_string(i) + ": length " + std::to_string(n) +
                      " is not a power of two in [2, 2^" + std::to_string(kPackedMaxLog) + "]";
      return false;
    }
    if (offsets[i] < 0 || offsets[i] > (1LL << kMaxTotalLog)) {
      if (err) *err = "transform " + std::to_string(i) + ": offset outside [0, 2^" + std::to_string(kMaxTotalLog) + "]";
      return false;
    }
    L.lognv[i] = l;
    L.total_elems = std::max(L.total_elems, offsets[i] + n);
    L.elements += n;
    L.flops += 5.0 * (double)n * l;
  }
  // overlapping transforms would write the same output elements
  std::vector<long long> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(), [&](long long a, long long b) { return offsets[a] < offsets[b]; });
  for (long long k = 1; k < count; ++k) {
    const long long a = order[k - 1], b = order[k];
    if (offsets[a] + sizes[a] > offsets[b]) {
      if (err) *err = "transforms " + std::to_string(a) + " and " + std::to_string(b) + " overlap";
      return false;
    }
  }
  // class lists, smallest class first
  std::vector<std::vector<int>> cls(kPackedMaxLog + 1);
  for (long long i = 0; i < count; ++i) cls[L.lognv[i]].push_back((int)i);
  std::vector<PackedItem> single_items, col_items, row_items, conv_items;
  std::vector<std::vector<PackedItem>> per_class(kPackedMaxLog + 1);
  std::vector<std::vector<PackedItem>> per_class_row(kPackedMaxLog + 1);
  std::vector<std::vector<PackedItem>> per_class_conv(kPackedSingleMaxLog + 1);
  // convolutions: padded lengths up to 2^12 are work items, C whole requests
  // of one length per item (the single tiles' C); longer ones go to the engine
  std::vector<std::vector<int>> ccls(kPackedSingleMaxLog + 1);
  for (long long i = 0; i < nconv; ++i) {
    const ConvReq& q = convs[i];
    if (q.signal_len < 1 || q.filter_len < 1 || q.sig_off < 0 || q.filt_off < 0 || q.out_off < 0 ||
        q.signal_len > (1LL << kConvMaxLogN) || q.filter_len > (1LL << kConvMaxLogN)) {
      if (err) *err = "convolution " + std::to_string(i) + ": lengths must be in [1, 2^22] and offsets >= 0";
      return false;
    }
    const long long lim = 1LL << kMaxTotalLog;  // no sum of a length and an offset can overflow
    if (q.sig_off > lim || q.filt_off > lim || q.out_off > lim) {
      if (err) *err = "convolution " + std::to_string(i) + ": offsets must be at most 2^" + std::to_string(kMaxTotalLog);
      return false;
    }
    const int l = conv_logn(q.signal_len, q.filter_len);
    if (l > kConvMaxLogN) {
      if (err) *err = "convolution " + std::to_string(i) + ": padded length exceeds 2^" + std::to_string(kConvMaxLogN);
      return false;
    }
    const long long olen = conv_out_len(q.signal_len, q.filter_len, conv_flags);
    L.conv_sig_elems = std::max(L.conv_sig_elems, q.sig_off + q.signal_len);
    L.conv_filt_elems = std::max(L.conv_filt_elems, q.filt_off + q.filter_len);
    L.conv_out_elems = std::max(L.conv_out_elems, q.out_off + olen);
    if (l > kPackedSingleMaxLog) {
      L.conv_engine.push_back(q);
      continue;
    }
    PackedConv pc;
    pc.sig_off = q.sig_off;
    pc.filt_off = q.filt_off;
    pc.out_off = q.out_off;
    pc.sig_len = (int)q.signal_len;
    pc.filt_len = (int)q.filter_len;
    pc.out_len = (int)olen;
    pc.out_shift = conv_out_shift(q.filter_len, l, conv_flags);
    pc.correlate = (conv_flags & CONV_CORRELATE) ? 1 : 0;
    pc.dc_norm = (conv_flags & CONV_REFERENCE_COMPAT) ? 1 : 0;
    ccls[l].push_back((int)L.convs.size());
    L.convs.push_back(pc);
    L.conv_flops += 10.0 * (double)(1LL << l) * l;
  }
  for (int l = 1; l <= kPackedSingleMaxLog; ++l) {
    const int per = 1 << packed_single_logc(l);
    const int base = (int)L.conv_class_list.size();
    L.conv_class_list.insert(L.conv_class_list.end(), ccls[l].begin(), ccls[l].end());
    for (int k = 0; k < (int)ccls[l].size(); k += per) {
      PackedItem it{PK_CONV, l, base + k, std::min(per, (int)ccls[l].size() - k)};
      conv_items.push_back(it);
      per_class_conv[l].push_back(it);
    }
  }
  for (int l = kPackedMinLog; l <= kPackedMaxLog; ++l) {
    if (cls[l].empty()) continue;
    if (l <= kPackedSingleMaxLog) {
      const int per = 1 << packed_single_logc(l);
      const int base = (int)L.class_list.size();
      L.class_list.insert(L.class_list.end(), cls[l].begin(), cls[l].end());
      for (int k = 0; k < (int)cls[l].size(); k += per) {
        PackedItem it{PK_SINGLE, l, base + k, std::min(per, (int)cls[l].size() - k)};
        single_items.push_back(it);
        per_class[l].push_back(it);
      }
    } else {
      const int l2 = packed_logn2(l), l1 = l - l2;
      const int cc = packed_col_logc(l), rc = packed_row_logc(l);
      for (int id : cls[l]) {
        L.scratch_off[id] = L.scratch_elems;
        L.scratch_elems += 1LL << l;
        L.ncol[id] = 1 << (l1 - cc);
        for (int b = 0; b < (1 << (l1 - cc)); ++b) {
          PackedItem it{PK_COL, l, id, b << cc};
          col_items.push_back(it);
          per_class[l].push_back(it);
        }
        for (int b = 0; b < (1 << (l2 - rc)); ++b) {
          PackedItem it{PK_ROW, l, id, b << rc};
          row_items.push_back(it);
          per_class_row[l].push_back(it);
        }
      }
    }
  }
  if (persistent) {
    // Column items of the largest transforms first, then convolutions and
    // whole small transforms (they keep the SMs busy while the column items
    // finish), then the row items in the same transform order: a row item is
    // only taken after every column item has been taken by a running CTA, so
    // its dependency wait ends.
    auto by_size_desc = [](const PackedItem& a, const PackedItem& b) { return a.logn > b.logn; };
    std::stable_sort(col_items.begin(), col_items.end(), by_size_desc);
    std::stable_sort(row_items.begin(), row_items.end(), by_size_desc);
    std::stable_sort(single_items.begin(), single_items.end(), by_size_desc);
    std::stable_sort(conv_items.begin(), conv_items.end(), by_size_desc);
    L.items = col_items;
    L.items.insert(L.items.end(), conv_items.begin(), conv_items.end());
    L.items.insert(L.items.end(), single_items.begin(), single_items.end());
    L.items.insert(L.items.end(), row_items.begin(), row_items.end());
    if (!L.items.empty()) {  // none when every convolution runs on the engine
      L.launch_begin.push_back(0);
      L.launch_count.push_back((int)L.items.size());
    }
  } else {
    // one launch per size class (two for four-step classes: columns, then rows)
    for (int l = kPackedMinLog; l <= kPackedMaxLog; ++l) {
      if (!per_class[l].empty()) {
        L.launch_begin.push_back((int)L.items.size());
        L.launch_count.push_back((int)per_class[l].size());
        L.items.insert(L.items.end(), per_class[l].begin(), per_class[l].end());
      }
      if (!per_class_row[l].empty()) {
        L.launch_begin.push_back((int)L.items.size());
        L.launch_count.push_back((int)per_class_row[l].size());
        L.items.insert(L.items.end(), per_class_row[l].begin(), per_class_row[l].end());
      }
    }
    for (int l = 1; l <= kPackedSingleMaxLog; ++l)
      if (!per_class_conv[l].empty()) {
        L.launch_begin.push_back((int)L.items.size());
        L.launch_count.push_back((int)per_class_conv[l].size());
        L.items.insert(L.items.end(), per_class_conv[l].begin(), per_class_conv[l].end());
      }
  }
  *out = std::move(L);
  return true;
}

bool build_packed_buckets(const long long* offsets, const long long* sizes, long long count,
                          PlanChoice (*choose)(long long n, long long count), std::vector<PackedBucket>* out,
                          long long* total_elems, std::string* err) {
  PackedLayout L;  // the validation of the persistent layout (lengths, offsets, overlaps)
  if (!build_packed_layout(offsets, sizes, count, false, &L, err)) return false;
  std::vector<PackedBucket> buckets;
  for (int l = kPackedMinLog; l <= kPackedMaxLog; ++l) {
    PackedBucket b;
    b.logn = l;
    bool odd = false;
    for (long long i = 0; i < count; ++i)
      if (L.lognv[i] == l) {
        b.xoff.push_back(offsets[i]);
        odd = odd || (offsets[i] & 1);
      }
    if (b.xoff.empty()) continue;
    const long long n = 1LL << l, c = (long long)b.xoff.size();
    PlanChoice ch = choose ? choose(n, c) : PlanChoice{};
    std::string e;
    if (!make_plan(n, c, ch, &b.plan, &e) && !make_plan(n, c, PlanChoice{}, &b.plan, &e)) {
      if (err) *err = e;
      return false;
    }
    bool dense_only = false;  // steps that read a transform's columns through a 2D view
    for (Step& st : b.plan.steps) {
      if (st.ologr || st.src == BUF_OUT) dense_only = true;
      if (st.kind == STEP_COL && st.pipe == 2) st.pipe = 0;  // plain column tile: loads through the offsets
      if (odd && st.pipe >= 2) st.pipe = 0;                   // bulk copies need 16-byte aligned rows
    }
    if (dense_only) {
      // plans of three passes: the default four-step instead
      PlanChoice four;
      four.mode = 2;
      if (!make_plan(n, c, four, &b.plan, &e)) {
        if (err) *err = e;
        return false;
      }
      for (Step& st : b.plan.steps)
        if (st.pipe && (st.kind == STEP_COL || odd)) st.pipe = 0;
    }
    buckets.push_back(std::move(b));
  }
  *total_elems = L.total_elems;
  *out = std::move(buckets);
  return true;
}

}  // namespace estl
