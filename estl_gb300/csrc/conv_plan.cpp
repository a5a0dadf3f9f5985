// conv_plan.cpp — see conv_plan.h.
#include "conv_plan.h"

#include "planner.h"

#include <algorithm>
#include <cstdio>
#include <map>

namespace estl {

namespace {

// Rows/columns per CTA of the instantiated convolution kernels (conv_list.inc).
int single_logc(int logm) {
  static const int c[15] = {0, 8, 8, 8, 8, 7, 6, 5, 4, 3, 2, 1, 0, 0, 0};
  return c[logm];
}
int four_step_logc(int logm) {
  switch (logm) {
    case 7: return 5;
    case 8: return 4;
    case 9: return 3;
    case 10: return 3;
    default: return 2;
  }
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace

int conv_logn(long long signal_len, long long filter_len) {
  long long len = signal_len + filter_len - 1;
  int l = 1;  // N >= 2 keeps every request on a tile kernel
  while ((1LL << l) < len) l++;
  return l;
}

int conv_out_shift(long long filter_len, int logn, int flags) {
  if (!(flags & CONV_REFERENCE_COMPAT)) return 0;
  const long long n = 1LL << logn, off = (filter_len + 1) / 2;
  // the kernel shifted by -off (Convolution.h:113-120) moves a convolution by
  // -off and a correlation, whose kernel spectrum is conjugated after the
  // shift (:125-137), by +off
  return (int)((flags & CONV_CORRELATE) ? (n - off % n) % n : off % n);
}

long long conv_out_len(long long signal_len, long long filter_len, int flags) {
  return (flags & CONV_REFERENCE_COMPAT) ? signal_len : signal_len + filter_len - 1;
}

void conv_extents(const ConvReq* reqs, int count, long long* sig_elems, long long* filt_elems) {
  long long s = 0, f = 0;
  for (int i = 0; i < count; ++i) {
    s = std::max(s, reqs[i].sig_off + reqs[i].signal_len);
    f = std::max(f, reqs[i].filt_off + reqs[i].filter_len);
  }
  *sig_elems = s;
  *filt_elems = f;
}

bool build_conv_layout(const ConvReq* reqs, int count, int flags, ConvLayout* out, std::string* err,
                       bool shared_filter) {
  ConvLayout L;
  if (count < 0 || (count > 0 && !reqs)) {
    if (err) *err = "invalid request array";
    return false;
  }
  std::map<int, std::vector<int>> buckets;  // log2 N -> request indices
  for (int i = 0; i < count; ++i) {
    const ConvReq& q = reqs[i];
    if (q.signal_len < 1 || q.filter_len < 1 || q.sig_off < 0 || q.filt_off < 0 || q.out_off < 0) {
      if (err) *err = "request " + std::to_string(i) + ": lengths must be >= 1 and offsets >= 0";
      return false;
    }
    const long long lim = 1LL << kMaxTotalLog;  // no sum of a length and an offset can overflow
    if (q.signal_len > lim || q.filter_len > lim || q.sig_off > lim || q.filt_off > lim || q.out_off > lim) {
      if (err) *err = "request " + std::to_string(i) + ": lengths and offsets must be at most 2^40";
      return false;
    }
    int logn = conv_logn(q.signal_len, q.filter_len);
    if (logn > kConvMaxLogN) {
      if (err) *err = "request " + std::to_string(i) + ": padded length exceeds 2^" + std::to_string(kConvMaxLogN);
      return false;
    }
    buckets[logn].push_back(i);
    if (shared_filter && (q.filter_len != reqs[0].filter_len || q.filt_off != reqs[0].filt_off ||
                          logn != conv_logn(reqs[0].signal_len, reqs[0].filter_len))) {
      if (err) *err = "shared-filter batch: every request must use filter 0 and pad to the same length";
      return false;
    }
    L.out_elems = std::max(L.out_elems, q.out_off + conv_out_len(q.signal_len, q.filter_len, flags));
  }
  long long spec = 0, scratch = 0;
  for (auto& kv : buckets) {
    const int logn = kv.first;
    const long long N = 1LL << logn;
    const long long rb = (long long)L.sig_rows.size();
    const long long cnt = (long long)kv.second.size();
    const long long fb = (long long)L.filt_rows.size();
    // four-step lengths run the real-input form (N/2-point complex transforms,
    // spectrum of N/2 + 1 values, kept in N/2 + 2 slots) unless the caller asks
    // for complex transforms or split precision
    const bool half = logn > kSingleMaxLog && !(flags & CONV_COMPLEX) && conv_split(flags) == 0;
    const long long spec_len = half ? N / 2 + 2 : N;
    for (int i : kv.second) {
      const ConvReq& q = reqs[i];
      const bool new_spectrum = !shared_filter || L.filt_rows.empty();
      ConvRow f{}, s{};
      f.sig_off = q.filt_off;
      f.sig_len = (int)q.filter_len;
      f.spec_off = spec;
      f.scale = 1.0f / (float)N;
      f.conj = (flags & CONV_CORRELATE) ? -1.f : 1.f;
      s.sig_off = q.sig_off;
      s.sig_len = (int)q.signal_len;
      s.spec_off = new_spectrum ? spec : L.filt_rows[0].spec_off;
      s.out_off = q.out_off;
      s.out_len = (int)conv_out_len(q.signal_len, q.filter_len, flags);
      s.out_shift = conv_out_shift(q.filter_len, logn, flags);
      s.dc_norm = (flags & CONV_REFERENCE_COMPAT) ? 1 : 0;
      s.scale = 1.f;
      s.conj = 1.f;
      if (new_spectrum) {
        L.filt_rows.push_back(f);
        spec += spec_len;
      }
      L.sig_rows.push_back(s);
    }
    const long long fcnt = (long long)L.filt_rows.size() - fb;
    if (logn <= kSingleMaxLog) {
      const int lc = single_logc(logn), le = std::min(4, logn);
      const long long grid = (cnt + (1LL << lc) - 1) >> lc;
      const long long fgrid = (fcnt + (1LL << lc) - 1) >> lc;
      if (flags & (CONV_NO_PAIRING | CONV_COMPLEX)) {
        if (fcnt) L.launches.push_back(ConvLaunch{CK_SPEC_SINGLE, logn, le, 4, lc, fgrid, logn, fb, fcnt, 0});
        L.launches.push_back(ConvLaunch{CK_CONV_SINGLE, logn, le, 4, lc, grid, logn, rb, cnt, 0});
      } else {
        // two real requests per complex transform (rows 2i, 2i+1 of the bucket); one
        // shared filter keeps its plain spectrum
        const long long pgrid = ((cnt + 1) / 2 + (1LL << lc) - 1) >> lc;
        const long long pfgrid = ((fcnt + 1) / 2 + (1LL << lc) - 1) >> lc;
        if (fcnt && shared_filter)
          L.launches.push_back(ConvLaunch{CK_SPEC_SINGLE, logn, le, 4, lc, fgrid, logn, fb, fcnt, 0});
        else if (fcnt)
          L.launches.push_back(ConvLaunch{CK_SPEC_PAIR, logn, le, 4, lc, pfgrid, logn, fb, fcnt, 0});
        L.launches.push_back(ConvLaunch{CK_CONV_PAIR, logn, le, 4, lc, pgrid, logn, rb, cnt, 0});
      }
    } else if (half) {
      const int lh = logn - 1, logn2 = lh / 2, logn1 = lh - logn2;
      const int cc = four_step_logc(logn2), cr = four_step_logc(logn1);
      const long long s_off = scratch;
      if (fcnt) {
        L.launches.push_back(ConvLaunch{CK_COL_FILTER_H, logn2, 4, 4, cc, fcnt << (logn1 - cc), lh, fb, fcnt, s_off});
        L.launches.push_back(ConvLaunch{CK_SPEC_ROW_H, logn1, 4, 4, cr, fcnt << (logn2 - cr), lh, fb, fcnt, s_off});
      }
      L.launches.push_back(ConvLaunch{CK_COL_SIGNAL_H, logn2, 4, 4, cc, cnt << (logn1 - cc), lh, rb, cnt, s_off});
      L.launches.push_back(ConvLaunch{CK_MID_H, logn1, 4, 4, cr, cnt << (logn2 - cr), lh, rb, cnt, s_off});
      L.launches.push_back(ConvLaunch{CK_OUT_H, logn2, 4, 4, cc, cnt << (logn1 - cc), lh, rb, cnt, s_off});
      scratch += cnt * (N / 2);
    } else {
      const int logn2 = logn / 2, logn1 = logn - logn2;
      const int cc = four_step_logc(logn2), cr = four_step_logc(logn1);
      const long long s_off = scratch;
      if (fcnt) {
        L.launches.push_back(ConvLaunch{CK_COL_FILTER, logn2, 4, 4, cc, fcnt << (logn1 - cc), logn, fb, fcnt, s_off});
        L.launches.push_back(ConvLaunch{CK_SPEC_ROW, logn1, 4, 4, cr, fcnt << (logn2 - cr), logn, fb, fcnt, s_off});
      }
      L.launches.push_back(ConvLaunch{CK_COL_SIGNAL, logn2, 4, 4, cc, cnt << (logn1 - cc), logn, rb, cnt, s_off});
      L.launches.push_back(ConvLaunch{CK_MID, logn1, 4, 4, cr, cnt << (logn2 - cr), logn, rb, cnt, s_off});
      L.launches.push_back(ConvLaunch{CK_OUT, logn2, 4, 4, cc, cnt << (logn1 - cc), logn, rb, cnt, s_off});
      scratch += cnt * N;
    }
  }
  L.buckets = (int)buckets.size();
  L.shared = shared_filter ? 1 : 0;
  L.split = conv_split(flags);
  // split precision: the tiles with radix-16 passes run their tensor-core variant
  for (ConvLaunch& l : L.launches) {
    const bool single = ck_is_single(l.kind);
    l.tc = (L.split != 0 && l.loge == 4 && l.logm >= 4 && (!single || l.logm <= kConvTcSingleMaxLog)) ? 1 : 0;
  }
  for (const ConvLaunch& l : L.launches)
    L.is_spectrum_launch.push_back(ck_is_filter(l.kind));
  L.spec_elems = spec;
  L.scratch_elems = scratch;
  size_t off = 0;
  L.off_filt_rows = off;
  off = align256(off + L.filt_rows.size() * sizeof(ConvRow));
  L.off_sig_rows = off;
  off = align256(off + L.sig_rows.size() * sizeof(ConvRow));
  L.off_spec = off;
  off = align256(off + (size_t)spec * sizeof(cf32));
  L.off_s1 = off;
  off = align256(off + (size_t)scratch * sizeof(cf32));
  L.off_s2 = off;
  off = align256(off + (size_t)scratch * sizeof(cf32));
  L.workspace_bytes = off;
  *out = std::move(L);
  return true;
}

}  // namespace estl
