// msc_graph.cuh -- the Morse-Smale complex as a mutable graph on the device,
// shared by the simplification (simplify.cu) and the piece merges (merge.cu).
//
// critical_point::asc / des (std::multiset<uint>, dmsc/include/discreteMorseDS.h:
// 90-126) are run-length encoded sorted arrays -- (value, count) runs, so equal
// elements stay consecutive exactly as std::multiset iterates them -- in one
// device pool, growing by reallocation inside it.  cancel / uncancel restate
// cancelPairs (dmsc/include/discreteMorseAlgorithm.h:348-585) and
// uncancel_pairs (:1006-1089).  Everything here runs on a single thread; the
// methods are __host__ __device__ only so that they have one definition.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "dmsc_common.cuh"

namespace dmsc {

// flags bits of a critical point (as exported by dmsc_msc_export)
constexpr uint8_t F_CANCELLED = 1, F_STRANG = 2, F_BCANCEL = 4;

struct Lists {  // list 2*cp = asc, 2*cp+1 = des
  uint32_t *off, *nrun, *cap;  // runs of list l live at pool[off[l] .. off[l]+nrun[l])
  uint32_t *total;             // multiset size (sum of counts)
  uint2 *pool;                 // .x = value, .y = count
  unsigned long long top, pool_cap;
};

// Moves n runs from src to dst (the ranges may overlap), eight at a time:
// the eight loads of a group are issued before its stores, so one thread
// waits for one memory round trip per group instead of one per run.
__host__ __device__ __forceinline__ void move_runs(uint2 *dst, const uint2 *src, unsigned long long n) {
  if (n == 0 || dst == src) return;
  if (dst < src) {  // forward
    unsigned long long i = 0;
    for (; i + 8 <= n; i += 8) {
      uint2 t[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) t[k] = src[i + k];
#pragma unroll
      for (int k = 0; k < 8; ++k) dst[i + k] = t[k];
    }
    for (; i < n; ++i) dst[i] = src[i];
  } else {  // backward
    unsigned long long i = n;
    for (; i >= 8; i -= 8) {
      uint2 t[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) t[k] = src[i - 8 + k];
#pragma unroll
      for (int k = 0; k < 8; ++k) dst[i - 8 + k] = t[k];
    }
    for (; i > 0; --i) dst[i - 1] = src[i - 1];
  }
}

struct Graph {
  uint32_t ncp;
  uint32_t *cellid;
  uint8_t *flags;
  uint32_t *pair_idx;
  Lists L;
  uint2 *tmp;                  // scratch runs
  unsigned long long tmp_cap;
  unsigned long long max_ops, ops = 0;
  bool fail = false;

  __host__ __device__ __forceinline__ int dim(uint32_t k) const {
    uint32_t c = cellid[k];
    return (int)(c & 1u) + (int)((c >> 16) & 1u);
  }
  __host__ __device__ __forceinline__ bool tick(unsigned long long n = 1) {
    ops += n;
    if (ops > max_ops) fail = true;
    return !fail;
  }

  // ---- run-length multisets ----
  __host__ __device__ __forceinline__ uint2 *runs(uint32_t l) const { return L.pool + L.off[l]; }
  __host__ __device__ uint32_t find_run(uint32_t l, uint32_t x) const {  // first run with value >= x
    const uint2 *p = runs(l);
    const uint32_t n = L.nrun[l];
    if (n <= 8) {  // short list: the runs below x counted from independent loads (one memory round trip)
      uint32_t i = 0;
#pragma unroll
      for (uint32_t k = 0; k < 8; ++k)
        if (k < n && p[k].x < x) ++i;
      return i;
    }
    uint32_t lo = 0, hi = n;
    while (lo < hi) { uint32_t m = (lo + hi) >> 1; if (p[m].x < x) lo = m + 1; else hi = m; }
    return lo;
  }
  __host__ __device__ uint32_t count(uint32_t l, uint32_t x) const {
    uint32_t i = find_run(l, x);
    return (i < L.nrun[l] && runs(l)[i].x == x) ? runs(l)[i].y : 0u;
  }
  __host__ __device__ bool contains(uint32_t l, uint32_t x) const { return count(l, x) != 0; }
  __host__ __device__ bool reserve(uint32_t l, uint32_t need) {
    if (need <= L.cap[l]) return true;
    uint32_t nc = L.cap[l] * 2 + 4;
    while (nc < need) nc *= 2;
    if (L.top + nc > L.pool_cap) { fail = true; return false; }
    uint2 *src = runs(l), *dst = L.pool + L.top;
    move_runs(dst, src, L.nrun[l]);
    L.off[l] = (uint32_t)L.top;
    L.cap[l] = nc;
    L.top += nc;
    return true;
  }
  __host__ __device__ void insert(uint32_t l, uint32_t x, uint32_t c = 1) {  // std::multiset::insert, c times
    uint32_t i = find_run(l, x), n = L.nrun[l];
    if (i < n && runs(l)[i].x == x) {
      uint2 &r = runs(l)[i];
      if (r.y > 0xffffffffu - c) { fail = true; return; }
      r.y += c;
    } else {
      if (!reserve(l, n + 1)) return;
      uint2 *p = runs(l);
      move_runs(p + i + 1, p + i, n - i);
      p[i] = make_uint2(x, c);
      L.nrun[l] = n + 1;
      tick(n - i);
    }
    if (L.total[l] > 0xffffffffu - c) { fail = true; return; }
    L.total[l] += c;
  }
  __host__ __device__ void erase(uint32_t l, uint32_t x) {  // std::multiset::erase(key): all copies
    uint32_t i = find_run(l, x), n = L.nrun[l];
    if (i >= n || runs(l)[i].x != x) return;
    uint2 *p = runs(l);
    L.total[l] -= p[i].y;
    move_runs(p + i, p + i + 1, n - i - 1);
    L.nrun[l] = n - 1;
    tick(n - i);
  }
  __host__ __device__ void clear(uint32_t l) { L.nrun[l] = 0; L.total[l] = 0; }

  // heap sort of tmp[0..n) by value (in place, O(n log n))
  __host__ __device__ void sort_tmp(unsigned long long n) {
    uint2 *t = tmp;
    for (unsigned long long s = n / 2; s-- > 0;) sift(s, n);
    for (unsigned long long e = n; e-- > 1;) { uint2 q = t[0]; t[0] = t[e]; t[e] = q; sift(0, e); }
  }
  __host__ __device__ void sift(unsigned long long root, unsigned long long end) {
    uint2 *t = tmp;
    while (2 * root + 1 < end) {
      unsigned long long c = 2 * root + 1;
      if (c + 1 < end && t[c].x < t[c + 1].x) ++c;
      if (t[root].x < t[c].x) { uint2 q = t[root]; t[root] = t[c]; t[c] = q; root = c; }
      else return;
    }
  }
  // list l := the multiset of the n (value, count) items in tmp (any order)
  __host__ __device__ bool set_list_from_tmp(uint32_t l, unsigned long long n) {
    if (!tick(n + 1)) return false;
    sort_tmp(n);
    unsigned long long m = 0, tot = 0;
    for (unsigned long long u = 0; u < n; ++u) {
      if (m > 0 && tmp[m - 1].x == tmp[u].x) {
        unsigned long long c = (unsigned long long)tmp[m - 1].y + tmp[u].y;
        if (c > 0xffffffffull) { fail = true; return false; }
        tmp[m - 1].y = (uint32_t)c;
      } else {
        tmp[m++] = tmp[u];
      }
      tot += tmp[u].y;
    }
    if (tot > 0xffffffffull || m > 0xffffffffull || !reserve(l, (uint32_t)m)) { fail = true; return false; }
    uint2 *p = runs(l);
    move_runs(p, tmp, m);
    L.nrun[l] = (uint32_t)m;
    L.total[l] = (uint32_t)tot;
    return true;
  }

  // cancelPairs (discreteMorseAlgorithm.h:348-585) without the new-edge list.
  // Orients the pair so that asc(cp0) holds cp1 and returns false when they are
  // not connected ("critical points are not connected": nothing changes).  The
  // new edges of the 4-argument form are (d, a) for every occurrence of a in
  // asc(cp0) \ {cp1} (ascending) times every occurrence of d in des(cp1) \ {cp0}
  // (ascending); both lists are left intact, so a caller can enumerate them.
  // The k runs tmp[0..k) (ascending, distinct values) inserted into list l
  // as k insert() calls in that order would leave it -- same multiset, same
  // operation count -- with one merge instead of k shifts of the list's tail;
  // each value whose count reaches 2 marks itself and `a` strangulated.
  __host__ __device__ void insert_sorted(uint32_t l, unsigned long long k, uint32_t a, bool mark = true) {
    const uint32_t n = L.nrun[l];
    const uint2 *R = runs(l);
    unsigned long long ticks = 0, nnew = 0, add = 0;
    for (unsigned long long q = 0, i = 0; q < k; ++q) {  // the shifts the k inserts would make
      const uint32_t x = tmp[q].x;
      while (i < n && R[i].x < x) ++i;
      if (!(i < n && R[i].x == x)) { ticks += n - i; ++nnew; }
      add += tmp[q].y;
    }
    if (!tick(ticks)) return;
    if (n + nnew > 0xffffffffull || L.total[l] + add > 0xffffffffull) { fail = true; return; }
    if (!reserve(l, (uint32_t)(n + nnew))) return;
    uint2 *P = runs(l);
    long long i = (long long)n - 1, w = (long long)(n + nnew) - 1;
    for (long long q = (long long)k - 1; q >= 0; --q) {  // merge from the back, in place
      const uint32_t x = tmp[q].x, c = tmp[q].y;
      while (i >= 0 && P[i].x > x) P[w--] = P[i--];
      if (i >= 0 && P[i].x == x) {
        uint2 r = P[i--];
        if (r.y > 0xffffffffu - c) { fail = true; return; }
        r.y += c;
        P[w--] = r;
        if (mark) { flags[a] |= F_STRANG; flags[x] |= F_STRANG; }
      } else {
        P[w--] = make_uint2(x, c);
        if (mark && c >= 2) { flags[a] |= F_STRANG; flags[x] |= F_STRANG; }
      }
    }
    L.nrun[l] = (uint32_t)(n + nnew);
    L.total[l] += (uint32_t)add;
  }

  __host__ __device__ bool cancel_pairs(uint32_t &cp0, uint32_t &cp1) {
    if (!contains(2 * cp0, cp1)) { uint32_t t = cp0; cp0 = cp1; cp1 = t; }
    if (!contains(2 * cp0, cp1)) return false;
    const uint32_t la0 = 2 * cp0, ld1 = 2 * cp1 + 1;
    // few d and many a (a minimum's saddles): the inserts into each asc(d)
    // become one merge per d after the loop instead of one shift each
    const bool batch_asc = L.nrun[ld1] < 8 && L.nrun[la0] >= 8 && L.nrun[la0] <= tmp_cap;
    for (uint32_t i = 0; i < L.nrun[la0] && !fail; ++i) {
      uint2 ra = runs(la0)[i];
      if (ra.x == cp1) continue;
      if (L.nrun[ld1] >= 8 && L.nrun[ld1] <= tmp_cap) {
        // many new edges into des(a): (d, a) for every d of des(cp1) but cp0,
        // ascending; asc(d) takes a one by one, des(a) takes all d at once
        unsigned long long k = 0, cs = 0;
        for (uint32_t j = 0; j < L.nrun[ld1] && !fail; ++j) {
          const uint2 rd = runs(ld1)[j];
          if (rd.x == cp0) continue;
          const unsigned long long c = (unsigned long long)ra.y * rd.y;
          if (c > 0xffffffffull) { fail = true; return true; }
          insert(2 * rd.x, ra.x, (uint32_t)c);
          tmp[k++] = make_uint2(rd.x, (uint32_t)c);
          cs += c;
        }
        if (fail) return true;
        insert_sorted(2 * ra.x + 1, k, ra.x);
        if (!tick(cs)) return true;
        continue;
      }
      if (batch_asc) {  // asc(d) takes every a at once below
        for (uint32_t j = 0; j < L.nrun[ld1] && !fail; ++j) {
          uint2 rd = runs(ld1)[j];
          if (rd.x == cp0) continue;
          unsigned long long c = (unsigned long long)ra.y * rd.y;
          if (c > 0xffffffffull) { fail = true; return true; }
          insert(2 * ra.x + 1, rd.x, (uint32_t)c);
          if (count(2 * ra.x + 1, rd.x) >= 2) {
            flags[ra.x] |= F_STRANG;
            flags[rd.x] |= F_STRANG;
          }
          if (!tick(c)) return true;
        }
        continue;
      }
      for (uint32_t j = 0; j < L.nrun[ld1] && !fail; ++j) {
        uint2 rd = runs(ld1)[j];
        if (rd.x == cp0) continue;
        unsigned long long c = (unsigned long long)ra.y * rd.y;
        if (c > 0xffffffffull) { fail = true; return true; }
        insert(2 * ra.x + 1, rd.x, (uint32_t)c);
        insert(2 * rd.x, ra.x, (uint32_t)c);
        if (count(2 * ra.x + 1, rd.x) >= 2) {
          flags[ra.x] |= F_STRANG;
          flags[rd.x] |= F_STRANG;
        }
        if (!tick(c)) return true;
      }
    }
    if (batch_asc) {
      // every d of des(cp1) but cp0 takes all a of asc(cp0) but cp1 (ascending,
      // distinct) with counts ra.y * rd.y in one merge: the same multiset the
      // inserts one by one leave (the strangulation marks were set above,
      // from des(a))
      for (uint32_t j = 0; j < L.nrun[ld1] && !fail; ++j) {
        const uint2 rd = runs(ld1)[j];
        if (rd.x == cp0) continue;
        unsigned long long k = 0;
        for (uint32_t i = 0; i < L.nrun[la0]; ++i) {
          const uint2 ra = runs(la0)[i];
          if (ra.x == cp1) continue;
          tmp[k++] = make_uint2(ra.x, (uint32_t)((unsigned long long)ra.y * rd.y));
        }
        insert_sorted(2 * rd.x, k, rd.x, false);
      }
    }
    for (uint32_t i = 0; i < L.nrun[la0]; ++i) {
      uint32_t a = runs(la0)[i].x;
      if (a == cp1) continue;
      erase(2 * a + 1, cp0);
    }
    for (uint32_t i = 0; i < L.nrun[2 * cp0 + 1]; ++i) erase(2 * runs(2 * cp0 + 1)[i].x, cp0);
    for (uint32_t i = 0; i < L.nrun[2 * cp1]; ++i) erase(2 * runs(2 * cp1)[i].x + 1, cp1);
    for (uint32_t i = 0; i < L.nrun[ld1]; ++i) {
      uint32_t d = runs(ld1)[i].x;
      if (d == cp0) continue;
      erase(2 * d, cp1);
    }
    flags[cp0] |= F_CANCELLED;
    clear(2 * cp0 + 1);
    flags[cp1] |= F_CANCELLED;
    clear(2 * cp1);
    return true;
  }

  // uncancel_pairs(msc, cp1, cp2) (discreteMorseAlgorithm.h:1006-1089).
  // Returns false on a reference logic_error condition.
  __host__ __device__ bool uncancel_pairs(uint32_t c1, uint32_t c2) {
    if (!contains(2 * c1, c2)) { uint32_t t = c1; c1 = c2; c2 = t; }
    const uint32_t lists[2] = {2 * c1, 2 * c2 + 1};
    const uint32_t ids[2] = {c1, c2};
    for (int i = 0; i < 2; ++i) {
      uint32_t l = lists[i], other = ids[(i + 1) % 2];
      if (!contains(l, other)) return false;  // "cancellable pair is not connected"
      unsigned long long n = 0;
      for (uint32_t k = 0; k < L.nrun[l]; ++k) {
        uint2 rx = runs(l)[k];
        if (rx.x == other) continue;
        if (!(flags[rx.x] & F_BCANCEL)) {
          if (n >= tmp_cap) { fail = true; return true; }
          tmp[n++] = rx;
          continue;
        }
        if (flags[rx.x] & F_CANCELLED) return false;
        uint32_t pidx = pair_idx[rx.x];
        if (pidx >= ncp || pair_idx[pidx] != rx.x) return false;
        uint32_t pl = 2 * pidx + i;
        for (uint32_t q = 0; q < L.nrun[pl]; ++q) {
          uint2 ry = runs(pl)[q];
          if (flags[ry.x] & F_BCANCEL) return false;
          unsigned long long c = (unsigned long long)rx.y * ry.y;
          if (c > 0xffffffffull || n >= tmp_cap) { fail = true; return true; }
          tmp[n++] = make_uint2(ry.x, (uint32_t)c);
        }
        if (!tick(1 + L.nrun[pl])) return true;
      }
      if (!set_list_from_tmp(l, n)) return true;
    }
    flags[c1] &= ~F_CANCELLED;
    flags[c2] &= ~F_CANCELLED;
    return true;
  }
};

}  // namespace dmsc
