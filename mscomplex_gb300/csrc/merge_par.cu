// merge_par.cu -- the piece merges of one tree level with the bulk of their
// work spread over the GPU: GridMSComplex::merge_up and merge_down
// (dmsc/src/grid_mscomplex.cpp:24-322) for complexes of millions of critical
// points, where one thread per merge (merge.cu) would walk every critical
// point and every arc in sequence.
//
// merge_up (:24-156) splits into
//   * the union of the critical points (:56-75): A's uncancelled points keep
//     their order, then B's uncancelled points whose cell A does not hold --
//     a scan over each input gives every point its index in the result;
//   * the boundary pairs (:84-92): each input's uncancelled boundary-cancelable
//     point takes its partner's index (B's assignment after A's, as the
//     reference's loop order leaves it);
//   * the connectivity (:77-122): the result's list of a point is the
//     multiset union of A's list and B's list (B's without arcs inside the
//     shared boundary when the point itself lies on it), restricted to
//     uncancelled points -- counts, a scan, a scatter, and a sort of each list
//     by index (the ascending order in which a std::multiset iterates);
//   * the cancellations along the shared boundary (:124-153), row-major and
//     order dependent: one thread per merge, on the mutable graph
//     (merge_up_cancel in merge_graph.cuh), all merges of the level in one
//     launch.
// merge_down (:158-322) splits into
//   * the uncancellations along the shared boundary (:172-201): one thread
//     per parent (merge_down_boundary), all merges of the level in one launch;
//   * the parent's boundary-cancelable points pushed into each child
//     (:207-281): the points it adds to the child are numbered by a scan over
//     the sequence of additions the reference's loop makes (down_child);
//   * every child point whose cell the parent holds takes the parent's
//     lists, restricted to points the child holds (:283-320): counts, a scan,
//     a scatter and a sort per list into the child's new CSR arrays.
// A step whose outcome only the one-thread restatement reproduces (a partner
// missing from the union, where the reference's std::map::operator[] would
// insert index 0; a boundary-cancelable point whose partner does not point
// back) reports ST_FALLBACK and the caller reruns the level with the
// one-thread merges.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "dmsc_common.cuh"
#include "dmsc_internal.h"
#include "grid_types.h"
#include "host_pool.h"
#include "merge_graph.cuh"

namespace dmsc {

namespace {

unsigned nblk(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (unsigned)(b < 1 ? 1 : b);
}

#define GRID_LOOP(i, n) for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)(n); i += (long long)gridDim.x * blockDim.x)

// Cell id -> critical-point index over a box of cell coordinates (the same
// table a merged graph keeps).  Entries are written and read in separate
// launches; each cell is written once.
struct CellTab {
  uint32_t *tab;
  int x0, y0, w, h;
  __device__ long long slot(uint32_t cid) const {
    const int x = (int)(cid & 0xffffu) - x0, y = (int)(cid >> 16) - y0;
    if (x < 0 || y < 0 || x >= w || y >= h) return -1;
    return (long long)y * w + x;
  }
  __device__ uint32_t find(uint32_t cid) const {
    const long long s = slot(cid);
    return s < 0 ? NO_CP : tab[s];
  }
  __device__ bool insert(uint32_t cid, uint32_t v) {
    const long long s = slot(cid);
    if (s < 0) return false;
    tab[s] = v;
    return true;
  }
};

__device__ __forceinline__ bool cancelled(const uint8_t *fl, uint32_t i) { return fl[i] & F_CANCELLED; }

// ---------------------------------------------------------------------------
// sorting every list of a CSR array by value
// ---------------------------------------------------------------------------
constexpr uint32_t SS_THREAD = 32, SS_BLOCK = 8192;

// Segments of up to SS_THREAD values: insertion sort by one thread; longer
// ones are queued (up to SS_BLOCK for one block each, beyond for the radix
// sort).  `need` (may be null) marks the segments that can be out of order.
__global__ void k_ss_small(long long nseg, const uint32_t *__restrict__ off, const uint8_t *__restrict__ need,
                           uint32_t *__restrict__ vals, uint32_t *__restrict__ q_block, uint32_t *__restrict__ n_block,
                           uint32_t *__restrict__ q_huge, uint32_t *__restrict__ n_huge) {
  GRID_LOOP(s, nseg) {
    if (need && !need[s]) continue;
    const uint32_t b = off[s], n = off[s + 1] - b;
    if (n <= 1) continue;
    if (n > SS_THREAD) {
      if (n > SS_BLOCK) q_huge[atomicAdd(n_huge, 1u)] = (uint32_t)s;
      else q_block[atomicAdd(n_block, 1u)] = (uint32_t)s;
      continue;
    }
    uint32_t v[SS_THREAD];
    for (uint32_t i = 0; i < n; ++i) v[i] = vals[b + i];
    for (uint32_t i = 1; i < n; ++i) {
      const uint32_t x = v[i];
      uint32_t j = i;
      while (j > 0 && v[j - 1] > x) { v[j] = v[j - 1]; --j; }
      v[j] = x;
    }
    for (uint32_t i = 0; i < n; ++i) vals[b + i] = v[i];
  }
}

// queued segments of up to SS_BLOCK values: one block each, bitonic sort in shared memory
__global__ void __launch_bounds__(512) k_ss_block(const uint32_t *__restrict__ off, uint32_t *__restrict__ vals,
                                                  const uint32_t *__restrict__ q, const uint32_t *__restrict__ nq) {
  __shared__ uint32_t sh[SS_BLOCK];
  const uint32_t count = *nq;
  for (uint32_t k = blockIdx.x; k < count; k += gridDim.x) {
    const uint32_t s = q[k], b = off[s], n = off[s + 1] - b;
    if (n <= 1024) {  // rank sort: each value's place is the count of values before it
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) sh[i] = vals[b + i];
      __syncthreads();
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint32_t v = sh[i];
        uint32_t r = 0;
        for (uint32_t j = 0; j < n; ++j) {
          const uint32_t u = sh[j];
          r += (u < v) || (u == v && j < i);
        }
        vals[b + r] = v;
      }
      __syncthreads();
      continue;
    }
    uint32_t p2 = 1;
    while (p2 < n) p2 <<= 1;
    for (uint32_t i = threadIdx.x; i < p2; i += blockDim.x) sh[i] = i < n ? vals[b + i] : 0xFFFFFFFFu;
    __syncthreads();
    for (uint32_t size = 2; size <= p2; size <<= 1)
      for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
        for (uint32_t i = threadIdx.x; i < p2; i += blockDim.x) {
          const uint32_t j = i ^ stride;
          if (j > i) {
            const bool up = (i & size) == 0;
            const uint32_t x = sh[i], y = sh[j];
            if ((x > y) == up) { sh[i] = y; sh[j] = x; }
          }
        }
        __syncthreads();
      }
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) vals[b + i] = sh[i];
    __syncthreads();
  }
}

// Sorts segments [off[s], off[s+1]) of vals for s < nseg where need[s] (all
// when need is null).  `off` is on the device; synchronises `st` once.
cudaError_t sort_segments(long long nseg, const uint32_t *off, uint32_t *vals, const uint8_t *need, cudaStream_t st) {
  if (nseg <= 0) return cudaSuccess;
  uint32_t *buf = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&buf, 4ull * (2 * nseg + 4), st);
  if (e != cudaSuccess) return e;
  uint32_t *q_block = buf, *q_huge = buf + nseg, *cnt = buf + 2 * nseg;
  e = cudaMemsetAsync(cnt, 0, 16, st);
  if (e == cudaSuccess) {
    k_ss_small<<<nblk(nseg), 256, 0, st>>>(nseg, off, need, vals, q_block, cnt, q_huge, cnt + 1);
    k_ss_block<<<152 * 2, 512, 0, st>>>(off, vals, q_block, cnt);
    DMSC_LAUNCHED(2);
    e = cudaGetLastError();
  }
  uint32_t nh = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&nh, cnt + 1, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess && nh) {  // rare: lists longer than SS_BLOCK, one radix sort each
    std::vector<uint32_t> segs(nh), o0(nh), o1(nh);
    e = cudaMemcpy(segs.data(), q_huge, 4ull * nh, cudaMemcpyDeviceToHost);
    for (uint32_t k = 0; k < nh && e == cudaSuccess; ++k) {
      e = cudaMemcpy(&o0[k], off + segs[k], 4, cudaMemcpyDeviceToHost);
      if (e == cudaSuccess) e = cudaMemcpy(&o1[k], off + segs[k] + 1, 4, cudaMemcpyDeviceToHost);
    }
    for (uint32_t k = 0; k < nh && e == cudaSuccess; ++k) {
      const long long n = (long long)o1[k] - o0[k];
      uint32_t *tmp = nullptr;
      e = cudaMallocAsync((void **)&tmp, 12ull * n, st);
      if (e != cudaSuccess) break;
      e = cudaMemsetAsync(tmp, 0, 4ull * n, st);
      if (e == cudaSuccess) e = radix_sort_pairs(vals + o0[k], tmp, tmp + n, tmp + 2 * n, n, 32, st);
      cudaFreeAsync(tmp, st);
    }
  }
  cudaFreeAsync(buf, st);
  return e;
}

// ---------------------------------------------------------------------------
// merge_up: union, boundary pairs, connectivity
// ---------------------------------------------------------------------------
struct CsrIn {  // a complex being read (device arrays)
  long long n;
  const uint32_t *cellid, *pair, *aoff, *asc, *doff, *des;
  const float *fn;
  const uint8_t *flags;
};
struct CsrOut {
  uint32_t *cellid, *pair, *aoff, *asc, *doff, *des;
  float *fn;
  uint8_t *flags;
};

CsrIn csr_in(const dmsc_msc &m) {
  return CsrIn{m.ncp, m.cellid.p, m.pair_idx.p, m.aoff.p, m.asc.p, m.doff.p, m.des.p, m.fn.p, m.flags.p};
}

__global__ void k_keep(CsrIn a, uint32_t *keep) {
  GRID_LOOP(j, a.n) keep[j] = cancelled(a.flags, (uint32_t)j) ? 0u : 1u;
}

// shallow_replicate_cp (grid_mscomplex.cpp:7-22): flags copied, partner unset
__device__ __forceinline__ void put_cp(const CsrIn &a, long long j, uint32_t d, CsrOut &o) {
  o.cellid[d] = a.cellid[j];
  o.fn[d] = a.fn[j];
  o.flags[d] = a.flags[j] & (F_CANCELLED | F_STRANG | F_BCANCEL);
  o.pair[d] = NO_CP;
}

// A's uncancelled points: index = scan of the keep flags
__global__ void k_up_a(CsrIn a, const uint32_t *idx, CellTab H, CsrOut o, uint32_t *status) {
  GRID_LOOP(j, a.n) {
    if (cancelled(a.flags, (uint32_t)j)) continue;
    if (!H.insert(a.cellid[j], idx[j])) { atomicOr(status, ST_SIMPLIFY_LIMIT); continue; }
    put_cp(a, j, idx[j], o);
  }
}

// B's uncancelled points: the index of A's copy, or new (counted by isnew)
__global__ void k_up_b_classify(CsrIn b, CellTab H, uint32_t *idx, uint32_t *isnew) {
  GRID_LOOP(j, b.n) {
    uint32_t d = NO_CP, nw = 0;
    if (!cancelled(b.flags, (uint32_t)j)) {
      d = H.find(b.cellid[j]);
      nw = d == NO_CP;
    }
    idx[j] = d;
    isnew[j] = nw;
  }
}

__global__ void k_up_b_new(CsrIn b, const uint32_t *isnew, const uint32_t *pos, const uint32_t *na, CellTab H, uint32_t *idx,
                           CsrOut o, uint32_t *status) {
  const uint32_t base = *na;
  GRID_LOOP(j, b.n) {
    if (!isnew[j]) continue;
    const uint32_t d = base + pos[j];
    idx[j] = d;
    if (!H.insert(b.cellid[j], d)) { atomicOr(status, ST_SIMPLIFY_LIMIT); continue; }
    put_cp(b, j, d, o);
  }
}

// boundary pairs (:84-92) of one input; idx = the result index of each point
__global__ void k_up_pairs(CsrIn a, const uint32_t *idx, CellTab H, uint32_t *opair, uint32_t *status) {
  GRID_LOOP(j, a.n) {
    const uint8_t fl = a.flags[j];
    if ((fl & F_CANCELLED) || !(fl & F_BCANCEL)) continue;
    const uint32_t p = a.pair[j];
    if (p >= (uint32_t)a.n) { atomicOr(status, ST_INVARIANT); continue; }
    const uint32_t t = H.find(a.cellid[p]);
    if (t == NO_CP) { atomicOr(status, ST_FALLBACK); continue; }
    opair[idx[j]] = t;
  }
}

// list lengths: A's stored, B's added (each result point has at most one
// source point in each input); mix marks the lists that B contributed to
__global__ void k_up_count(CsrIn a, const uint32_t *idx, bool second, CRect ixn, uint32_t *tot_a, uint32_t *tot_d,
                           uint8_t *mix, uint32_t *status) {
  GRID_LOOP(j, a.n) {
    if (cancelled(a.flags, (uint32_t)j)) continue;
    const uint32_t d = idx[j], cid = a.cellid[j];
    const bool cmn = second && ixn.contains(px_(cid), py_(cid));
    uint32_t c[2] = {0, 0};
    for (int w = 0; w < 2; ++w) {
      const uint32_t *o = w ? a.doff : a.aoff, *l = w ? a.des : a.asc;
      for (uint32_t q = o[j]; q < o[j + 1]; ++q) {
        const uint32_t r = l[q];
        if (r >= (uint32_t)a.n) { atomicOr(status, ST_INVARIANT); continue; }
        if (cancelled(a.flags, r)) continue;
        if (cmn && ixn.contains(px_(a.cellid[r]), py_(a.cellid[r]))) continue;
        ++c[w];
      }
    }
    if (second) {
      tot_a[d] += c[0];
      tot_d[d] += c[1];
      if (c[0] + c[1]) mix[d] = 1;
    } else {
      tot_a[d] = c[0];
      tot_d[d] = c[1];
    }
  }
}

// entries: A's from the front of each list (in order), B's from the back
__global__ void k_up_write(CsrIn a, const uint32_t *idx, bool second, CRect ixn, CsrOut o) {
  GRID_LOOP(j, a.n) {
    if (cancelled(a.flags, (uint32_t)j)) continue;
    const uint32_t d = idx[j], cid = a.cellid[j];
    const bool cmn = second && ixn.contains(px_(cid), py_(cid));
    for (int w = 0; w < 2; ++w) {
      const uint32_t *io = w ? a.doff : a.aoff, *l = w ? a.des : a.asc;
      uint32_t *oo = w ? o.doff : o.aoff, *ol = w ? o.des : o.asc;
      const uint32_t lo = oo[d], hi = oo[d + 1];
      uint32_t p = second ? hi : lo;
      for (uint32_t q = io[j]; q < io[j + 1]; ++q) {
        const uint32_t r = l[q];
        if (r >= (uint32_t)a.n || cancelled(a.flags, r)) continue;
        if (cmn && ixn.contains(px_(a.cellid[r]), py_(a.cellid[r]))) continue;
        if (second) { if (p > lo) ol[--p] = idx[r]; }
        else if (p < hi) ol[p++] = idx[r];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// merge_down: parent checks, its boundary-cancelable list, the child rewrite
// ---------------------------------------------------------------------------
// "all cps ought to be uncancelled" (:209) and the boundary-cancelable flags
__global__ void k_down_check(MGraph P, uint32_t *bflag, uint32_t *status) {
  GRID_LOOP(j, P.G.ncp) {
    const uint8_t fl = P.G.flags[j];
    if (fl & F_CANCELLED) atomicOr(status, ST_INVARIANT);
    bflag[j] = (fl & F_BCANCEL) ? 1u : 0u;
  }
}

// the boundary-cancelable points in index order, a bound on the points they
// can add to a child (themselves, their partners, their list entries) and
// the box of those points' cells (box: l, b, r, t)
__device__ __forceinline__ void box_add(int b[4], uint32_t cid) {
  const int x = (int)(cid & 0xffffu), y = (int)(cid >> 16);
  b[0] = min(b[0], x); b[1] = min(b[1], y); b[2] = max(b[2], x); b[3] = max(b[3], y);
}
__global__ void k_down_list(MGraph P, const uint32_t *bflag, const uint32_t *pos, uint32_t *jb,
                            unsigned long long *adds, int *box) {
  unsigned long long mine = 0;
  int b[4] = {1 << 30, 1 << 30, -1, -1};
  GRID_LOOP(j, P.G.ncp) {
    if (!bflag[j]) continue;
    jb[pos[j]] = (uint32_t)j;
    mine += 2ull + P.G.L.nrun[2 * j] + P.G.L.nrun[2 * j + 1];
    box_add(b, P.G.cellid[j]);
    const uint32_t sp = P.G.pair_idx[j];
    if (sp < P.G.ncp) box_add(b, P.G.cellid[sp]);
    for (int w = 0; w < 2; ++w) {
      const uint2 *r = P.G.runs(2 * j + w);
      for (uint32_t q = 0; q < P.G.L.nrun[2 * j + w]; ++q)
        if (r[q].x < P.G.ncp) box_add(b, P.G.cellid[r[q].x]);
    }
  }
  if (mine) atomicAdd(adds, mine);
  if (b[2] >= 0) {
    atomicMin(box, b[0]); atomicMin(box + 1, b[1]); atomicMax(box + 2, b[2]); atomicMax(box + 3, b[3]);
  }
}

// ---------------------------------------------------------------------------
// merge_down into one child (:207-320) without a mutable graph of the child.
// The parent's boundary-cancelable points j (in index order, the list jb)
// come in pairs (j, sp).  A pair whose two cells the child lacks is skipped;
// when it holds exactly one, the first of the pair (lower index) adds the
// other; the pair is then marked boundary-cancelable and paired in the child
// unless both cells were already there with the mark.  The first of each
// non-skipped point's list entries that the child lacks adds it, in the
// order the reference's loop meets them: so every addition is an event in
// one sequence (per point: its partner, then its asc, then its des entries),
// and a scan over that sequence numbers the added points.  Finally every
// child point whose cell the parent holds takes the parent's lists,
// restricted to the points the child holds (for boundary-cancelable points
// the child holds them all by then); the others keep their own.
// ---------------------------------------------------------------------------
enum : uint8_t { DC_SKIP = 1, DC_ADD = 2, DC_FIRST = 4, DC_S0 = 8, DC_P0 = 16 };

struct DcArgs {
  MGraph P;                 // the parent after its boundary uncancellations
  const uint32_t *jb;       // its boundary-cancelable points, ascending
  uint32_t njb;
  CsrIn c;                  // the child before the merge
  CellTab tab;              // child cell -> index (initial points, then the added ones)
  CellTab first;            // missing cell -> position of its first list event
  uint32_t *cnt, *base, *addsrc;
  uint8_t *kind;            // per boundary point
  uint32_t *addf, *rank;    // per event
  CsrOut o;                 // the child's point arrays after the merge
  uint32_t ncp0;
  uint32_t *status;
};

__global__ void k_dc_table(CsrIn c, CellTab tab, uint32_t *status) {
  GRID_LOOP(i, c.n) {
    if (!tab.insert(c.cellid[i], (uint32_t)i)) atomicOr(status, ST_INVARIANT);
  }
}

__global__ void k_dc_classify(DcArgs a) {
  GRID_LOOP(q, a.njb) {
    const uint32_t j = a.jb[q], sp = a.P.G.pair_idx[j];
    uint8_t kd = 0;
    uint32_t n = 0;
    if (sp >= a.P.G.ncp || sp == j || a.P.G.pair_idx[sp] != j || !(a.P.G.flags[sp] & F_BCANCEL)) {
      atomicOr(a.status, ST_FALLBACK);  // not a plain pair: the one-thread merge handles it
      kd = DC_SKIP;
    } else {
      const bool s0 = a.tab.find(a.P.G.cellid[j]) != NO_CP, p0 = a.tab.find(a.P.G.cellid[sp]) != NO_CP;
      if (s0) kd |= DC_S0;
      if (p0) kd |= DC_P0;
      if (j < sp) kd |= DC_FIRST;
      if (!s0 && !p0) kd |= DC_SKIP;
      else {
        if (j < sp && s0 != p0) { kd |= DC_ADD; a.addsrc[q] = s0 ? sp : j; ++n; }
        n += a.P.G.L.nrun[2 * j] + a.P.G.L.nrun[2 * j + 1];
      }
    }
    a.kind[q] = kd;
    a.cnt[q] = n;
  }
}

// the first list event of every cell the child lacks
__global__ void k_dc_first(DcArgs a) {
  GRID_LOOP(q, a.njb) {
    const uint8_t kd = a.kind[q];
    if (kd & DC_SKIP) continue;
    const uint32_t j = a.jb[q];
    uint32_t pos = a.base[q] + ((kd & DC_ADD) ? 1 : 0);
    for (int w = 0; w < 2; ++w) {
      const uint2 *r = a.P.G.runs(2 * j + w);
      for (uint32_t k = 0; k < a.P.G.L.nrun[2 * j + w]; ++k, ++pos) {
        const uint32_t x = r[k].x;
        if (x >= a.P.G.ncp || (a.P.G.flags[x] & F_BCANCEL)) { atomicOr(a.status, ST_INVARIANT); continue; }
        const uint32_t cc = a.P.G.cellid[x];
        if (a.tab.find(cc) != NO_CP) continue;
        const long long sl = a.first.slot(cc);
        if (sl < 0) atomicOr(a.status, ST_INVARIANT);
        else atomicMin(a.first.tab + sl, pos);
      }
    }
  }
}

__global__ void k_dc_addflags(DcArgs a) {
  GRID_LOOP(q, a.njb) {
    const uint8_t kd = a.kind[q];
    if (kd & DC_SKIP) continue;
    const uint32_t j = a.jb[q];
    uint32_t pos = a.base[q];
    if (kd & DC_ADD) a.addf[pos++] = 1;
    for (int w = 0; w < 2; ++w) {
      const uint2 *r = a.P.G.runs(2 * j + w);
      for (uint32_t k = 0; k < a.P.G.L.nrun[2 * j + w]; ++k, ++pos) {
        const uint32_t x = r[k].x;
        if (x >= a.P.G.ncp) continue;
        const uint32_t cc = a.P.G.cellid[x];
        const long long sl = a.first.slot(cc);
        a.addf[pos] = (a.tab.find(cc) == NO_CP && sl >= 0 && a.first.tab[sl] == pos) ? 1u : 0u;
      }
    }
  }
}

// shallow_replicate_cp of parent point x as child point d
__device__ __forceinline__ void dc_put(DcArgs &a, uint32_t x, uint32_t d) {
  const uint32_t cid = a.P.G.cellid[x];
  a.o.cellid[d] = cid;
  a.o.fn[d] = a.P.fn[x];
  a.o.flags[d] = a.P.G.flags[x] & (F_CANCELLED | F_STRANG | F_BCANCEL);
  a.o.pair[d] = NO_CP;
  if (!a.tab.insert(cid, d)) atomicOr(a.status, ST_INVARIANT);
}

__global__ void k_dc_add(DcArgs a) {
  GRID_LOOP(q, a.njb) {
    const uint8_t kd = a.kind[q];
    if (kd & DC_SKIP) continue;
    const uint32_t j = a.jb[q];
    uint32_t pos = a.base[q];
    if (kd & DC_ADD) { dc_put(a, a.addsrc[q], a.ncp0 + a.rank[pos]); ++pos; }
    for (int w = 0; w < 2; ++w) {
      const uint2 *r = a.P.G.runs(2 * j + w);
      for (uint32_t k = 0; k < a.P.G.L.nrun[2 * j + w]; ++k, ++pos)
        if (a.addf[pos]) dc_put(a, r[k].x, a.ncp0 + a.rank[pos]);
    }
  }
}

// the pairing of each non-skipped pair, once (by its first point)
__global__ void k_dc_pairing(DcArgs a) {
  GRID_LOOP(q, a.njb) {
    const uint8_t kd = a.kind[q];
    if ((kd & DC_SKIP) || !(kd & DC_FIRST)) continue;
    const uint32_t j = a.jb[q], sp = a.P.G.pair_idx[j];
    const uint32_t d1 = a.tab.find(a.P.G.cellid[j]), d2 = a.tab.find(a.P.G.cellid[sp]);
    if (d1 == NO_CP || d2 == NO_CP) { atomicOr(a.status, ST_INVARIANT); continue; }
    const bool set = (kd & DC_ADD) || !(a.o.flags[d1] & F_BCANCEL) || !(a.o.flags[d2] & F_BCANCEL);
    if (!set) continue;
    a.o.flags[d1] |= F_BCANCEL;
    a.o.flags[d2] |= F_BCANCEL;
    a.o.pair[d1] = d2;
    a.o.pair[d2] = d1;
  }
}

// the parent point (if any) whose lists each child point takes
__global__ void k_dc_src(DcArgs a, uint32_t n, uint32_t *src) {
  GRID_LOOP(d, n) src[d] = a.P.find(a.o.cellid[d]);
}

__global__ void k_dc_count(DcArgs a, uint32_t n, const uint32_t *src, uint32_t *tot_a, uint32_t *tot_d, uint8_t *need) {
  GRID_LOOP(d, n) {
    const uint32_t j = src[d];
    for (int w = 0; w < 2; ++w) {
      uint32_t c = 0;
      if (j == NO_CP) {
        const uint32_t *off = w ? a.c.doff : a.c.aoff;
        if (d < a.ncp0) c = off[d + 1] - off[d];
      } else {
        const uint2 *r = a.P.G.runs(2 * j + w);
        for (uint32_t k = 0; k < a.P.G.L.nrun[2 * j + w]; ++k)
          if (r[k].x < a.P.G.ncp && a.tab.find(a.P.G.cellid[r[k].x]) != NO_CP) c += r[k].y;
      }
      (w ? tot_d : tot_a)[d] = c;
    }
    need[d] = j != NO_CP;
  }
}

__global__ void k_dc_write(DcArgs a, uint32_t n, const uint32_t *src) {
  GRID_LOOP(d, n) {
    const uint32_t j = src[d];
    for (int w = 0; w < 2; ++w) {
      const uint32_t *oo = w ? a.o.doff : a.o.aoff;
      uint32_t p = oo[d];
      const uint32_t end = oo[d + 1];
      uint32_t *ol = w ? a.o.des : a.o.asc;
      if (j == NO_CP) {
        if (d >= a.ncp0) continue;
        const uint32_t *off = w ? a.c.doff : a.c.aoff, *l = w ? a.c.des : a.c.asc;
        for (uint32_t q = off[d]; q < off[d + 1] && p < end; ++q) ol[p++] = l[q];
      } else {
        const uint2 *r = a.P.G.runs(2 * j + w);
        for (uint32_t k = 0; k < a.P.G.L.nrun[2 * j + w]; ++k) {
          if (r[k].x >= a.P.G.ncp) continue;
          const uint32_t ci = a.tab.find(a.P.G.cellid[r[k].x]);
          if (ci == NO_CP) continue;
          for (uint32_t c = 0; c < r[k].y && p < end; ++c) ol[p++] = ci;
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// the one-thread steps of a level, one block per job
// ---------------------------------------------------------------------------
enum SeqKind : int { SEQ_UP_CANCEL = 0, SEQ_DOWN_BOUNDARY = 1 };
struct SeqJob {
  int kind, g0;
  CRect ixn;
  int win = 0, min_commits = 0;  // SEQ_UP_CANCEL: rounds window (0: one thread) and hand-off rate
};

// Loads, across the GPU, what the one-thread step of a job will read -- the
// boundary points, their partners, their lists and their neighbours' list
// descriptors -- so that the step finds it in L2 instead of DRAM.  Reads
// only; the sum is stored only under a condition that never holds, so the
// loads are kept.
__device__ __forceinline__ uint32_t touch_cp(const MGraph &M, uint32_t c) {
  if (c >= M.G.ncp) return 0;
  uint32_t acc = M.G.flags[c] ^ M.G.pair_idx[c] ^ M.G.cellid[c];
  for (int w = 0; w < 2; ++w) {
    const uint32_t l = 2 * c + w, n = M.G.L.nrun[l];
    const uint2 *r = M.G.L.pool + M.G.L.off[l];
    acc ^= M.G.L.cap[l] ^ M.G.L.total[l];
    for (uint32_t q = 0; q < n && q < 64; ++q) {
      const uint32_t v = r[q].x;
      if (v >= M.G.ncp) continue;
      acc ^= M.G.flags[v] ^ M.G.pair_idx[v] ^ M.G.cellid[v];
      for (int u = 0; u < 2; ++u) {
        const uint32_t lv = 2 * v + u;
        acc ^= M.G.L.nrun[lv] ^ M.G.L.cap[lv] ^ M.G.L.total[lv];
        if (M.G.L.nrun[lv]) acc ^= M.G.L.pool[M.G.L.off[lv]].x;
      }
    }
  }
  return acc;
}

__global__ void k_seq_prefetch(const MGraph *graphs, const SeqJob *jobs, uint32_t *sink) {
  const SeqJob jb = jobs[blockIdx.y];
  const MGraph &M = graphs[jb.g0];
  uint32_t acc = 0;
  const long long w = jb.ixn.r - jb.ixn.l + 1, h = jb.ixn.t - jb.ixn.b + 1;
  GRID_LOOP(t, w * h) {
    const uint32_t si = M.find(pack_cellid(jb.ixn.l + (int)(t % w), jb.ixn.b + (int)(t / w)));
    if (si == NO_CP || si >= M.G.ncp) continue;
    acc ^= touch_cp(M, si) ^ touch_cp(M, M.G.pair_idx[si]);
  }
  if (acc == 0x9E3779B9u && sink) *sink = acc;
}

// The graphs are worked on as local copies of their descriptors: the
// pointers and counters stay in registers instead of being reloaded from
// global memory after every store through a list pointer.
__global__ void k_merge_seq(MGraph *graphs, const SeqJob *jobs, int njobs, uint32_t *status) {
  const int b = blockIdx.x;
  if (b >= njobs || threadIdx.x != 0) return;
  const SeqJob jb = jobs[b];
  MGraph g0 = graphs[jb.g0];
  if (jb.kind == SEQ_UP_CANCEL) merge_up_cancel(g0, jb.ixn, status);
  else merge_down_boundary(g0, jb.ixn, status);
  if (g0.G.fail) set_status(status, ST_SIMPLIFY_LIMIT);
  graphs[jb.g0] = g0;
}

// ---------------------------------------------------------------------------
// merge_up's boundary cancellations in ordered-parallel rounds.  Task t is
// cell t of the shared boundary in row-major order.  Each round looks at a
// window: the first `win` cells from the first pending task on.  Every
// pending task of the window reserves its footprint -- the critical points
// whose lists or flags its cancellation reads or writes -- with the
// round-tagged key (round, t) in a per-point slot (atomicMin: the round's
// smallest task touching the point wins); tasks sharing a slot are joined in
// a union-find that hooks the larger root under the smaller; and the root of
// each group, its smallest task, runs.  Every pending task earlier than a
// window task is inside the window, so a root has no earlier pending task
// that overlaps it.  Edges are only added inside a running task's footprint,
// so groups cannot merge through growth and every task sees the graph the
// row-major loop would show it.  The first pending task is always a root, so
// every round commits at least one task.  One block per merge; the rounds are
// separated by barriers of the block.  Each thread allocates list room from
// its own slice of the pool's free part, so the graph code stays that of one
// thread.  Where groups stay large (one point in most footprints, as a large
// extremum on a smooth field), rounds commit few tasks each: after
// ROUND_PATIENCE rounds in a row below `min_commits`, or if a union-find
// guard runs out, thread 0 runs the remaining tasks in row-major order, which
// is exact at any round boundary (every task that ran commutes with every
// earlier one still pending), from a quarter of the free pool kept for it.
// ---------------------------------------------------------------------------
constexpr int ROUND_THREADS = 512, ROUND_TASKS = 32768, ROUND_PATIENCE = 8;
struct RoundSmem {
  uint32_t parent[ROUND_TASKS];
  uint32_t done[ROUND_TASKS / 32];
};

// Parents only point to smaller tasks of the window, so a chain is shorter
// than the window and the guard never ends a search early.
__device__ __forceinline__ uint32_t uf_root(uint32_t *parent, uint32_t a) {
  for (int guard = 0; guard < ROUND_TASKS; ++guard) {
    const uint32_t p = ((volatile uint32_t *)parent)[a];
    if (p == a) return a;
    a = p;
  }
  return a;
}
// False if the join did not happen within the guard (each failed CAS means
// another thread hooked a root meanwhile); the caller then stops the rounds.
__device__ __forceinline__ bool uf_join(uint32_t *parent, uint32_t a, uint32_t b) {
  for (int guard = 0; guard < 4 * ROUND_TASKS; ++guard) {
    a = uf_root(parent, a);
    b = uf_root(parent, b);
    if (a == b) return true;
    if (a > b) { const uint32_t t = a; a = b; b = t; }
    if (atomicCAS(&parent[b], b, a) == b) return true;
  }
  return false;
}

// The cell's point and, while it may still cancel, its partner and both
// points' neighbours.
template <class F>
__device__ void up_footprint(const MGraph &M, uint32_t si, F f) {
  f(si);
  const uint8_t fl = M.G.flags[si];
  if ((fl & F_CANCELLED) || !(fl & F_BCANCEL)) return;
  const uint32_t pi = M.G.pair_idx[si];
  if (pi >= M.G.ncp) return;
  f(pi);
  const uint32_t c2[2] = {si, pi};
  for (int k = 0; k < 2; ++k)
    for (int w = 0; w < 2; ++w) {
      const uint32_t l = 2 * c2[k] + w, n = M.G.L.nrun[l];
      const uint2 *r = M.G.L.pool + M.G.L.off[l];
      for (uint32_t q = 0; q < n; ++q) f(r[q].x);
    }
}

// Whether cell (x, y) can ever act: the rect / ext test of the loop on it and
// its partner (fixed for the whole loop; flags are not).
__device__ __forceinline__ bool up_cell_static(const MGraph &M, int x, int y, uint32_t si) {
  if (si >= M.G.ncp) return true;  // left to the loop body, which reports it
  const uint32_t pi = M.G.pair_idx[si];
  if (pi >= M.G.ncp) return true;
  const uint32_t p = M.G.cellid[pi];
  return (M.rect.interior(x, y) || M.ext.boundary(x, y)) && (M.rect.interior(px_(p), py_(p)) || M.ext.boundary(px_(p), py_(p)));
}

// The first task at or after `from` whose done bit is clear (n if none),
// into *lo (which the caller set to n); all threads take part.
__device__ __forceinline__ void first_pending(const RoundSmem &S, long long from, long long n, unsigned int *lo) {
  const long long nw = (n + 31) / 32;
  for (long long wi = from / 32 + threadIdx.x; wi < nw; wi += blockDim.x) {
    uint32_t open = ~S.done[wi];
    if (wi == from / 32) open &= ~0u << (from & 31);
    if (wi == nw - 1 && (n & 31)) open &= (1u << (n & 31)) - 1;
    if (open) atomicMin(lo, (unsigned int)(wi * 32 + __ffs(open) - 1));
  }
}

__global__ void __launch_bounds__(ROUND_THREADS, 1) k_merge_up_rounds(MGraph *graphs, const SeqJob *jobs, int njobs,
                                                                      unsigned long long *const *slots, uint32_t *status) {
  extern __shared__ __align__(16) unsigned char round_smem[];
  RoundSmem &S = *reinterpret_cast<RoundSmem *>(round_smem);
  __shared__ int abort_all, uf_bad;
  __shared__ unsigned int lo_s, commits;
  const int b = blockIdx.x;
  if (b >= njobs) return;
  const SeqJob jb = jobs[b];
  MGraph g = graphs[jb.g0];  // every thread's own descriptor copy, read before any write-back
  const long long w = jb.ixn.r - jb.ixn.l + 1, h = jb.ixn.t - jb.ixn.b + 1, n = w * h;
  unsigned long long *slot = slots[b];
  if (n > ROUND_TASKS || !slot || jb.win <= 0) {  // one thread, as k_merge_seq
    if (threadIdx.x == 0) {
      merge_up_cancel(g, jb.ixn, status);
      if (g.G.fail) set_status(status, ST_SIMPLIFY_LIMIT);
      graphs[jb.g0] = g;
    }
    return;
  }
  const long long win = jb.win < ROUND_TASKS ? jb.win : ROUND_TASKS;
  if (threadIdx.x == 0) { abort_all = 0; uf_bad = 0; lo_s = (unsigned int)n; }
  for (long long t = threadIdx.x; t < ROUND_TASKS / 32; t += blockDim.x) S.done[t] = 0;
  __syncthreads();
  const unsigned long long free_runs = g.G.L.pool_cap - g.G.L.top, pool_end = g.G.L.pool_cap;
  const unsigned long long room = (free_runs - free_runs / 4) / blockDim.x, fin_start = g.G.L.top + room * blockDim.x;
  const unsigned long long tmp_cap0 = g.G.tmp_cap;
  g.G.L.top += room * threadIdx.x;  // this thread's slice of the free pool
  g.G.L.pool_cap = g.G.L.top + room;
  g.G.tmp_cap = 0;  // no shared scratch: cancel_pairs takes its per-entry path (the same result)
  auto cell_of = [&](long long t, int &x, int &y) { x = jb.ixn.l + (int)(t % w); y = jb.ixn.b + (int)(t / w); };
  auto is_done = [&](long long t) { return (S.done[t >> 5] >> (t & 31)) & 1u; };
  // cells that can never act are done from the start
  for (long long t = threadIdx.x; t < n; t += blockDim.x) {
    int x, y;
    cell_of(t, x, y);
    const uint32_t si = g.find(pack_cellid(x, y));
    if (si != NO_CP && !up_cell_static(g, x, y, si)) atomicOr(&S.done[t >> 5], 1u << (t & 31));
  }
  __syncthreads();
  first_pending(S, 0, n, &lo_s);
  __syncthreads();
  int slow = 0;  // rounds in a row that committed fewer than min_commits tasks
  for (uint32_t round = 0; round < (uint32_t)n + 1; ++round) {
    const long long lo = lo_s;
    if (lo >= n || abort_all || uf_bad || slow >= ROUND_PATIENCE) break;
    const long long hi = lo + win < n ? lo + win : n;
    const unsigned long long tag = (unsigned long long)(0xFFFFFFFFu - round) << 32;
    __syncthreads();  // every thread has read lo_s and the flags
    if (threadIdx.x == 0) { commits = 0; lo_s = (unsigned int)n; }
    // reserve
    for (long long t = lo + threadIdx.x; t < hi; t += blockDim.x) {
      if (is_done(t)) continue;
      S.parent[t] = (uint32_t)t;
      int x, y;
      cell_of(t, x, y);
      const uint32_t si = g.find(pack_cellid(x, y));
      if (si >= g.G.ncp) continue;  // the loop body reports it when the task runs
      up_footprint(g, si, [&](uint32_t c) { if (c < g.G.ncp) atomicMin(&slot[c], tag | (unsigned long long)t); });
    }
    __syncthreads();
    // join the tasks that share a point
    for (long long t = lo + threadIdx.x; t < hi; t += blockDim.x) {
      if (is_done(t)) continue;
      int x, y;
      cell_of(t, x, y);
      const uint32_t si = g.find(pack_cellid(x, y));
      if (si >= g.G.ncp) continue;
      up_footprint(g, si, [&](uint32_t c) {
        if (c >= g.G.ncp) return;
        const unsigned long long v = slot[c];
        if ((v & 0xFFFFFFFF00000000ull) == tag && (v & 0xFFFFFFFFull) < (unsigned long long)n)
          if (!uf_join(S.parent, (uint32_t)t, (uint32_t)(v & 0xFFFFFFFFull))) uf_bad = 1;
      });
    }
    __syncthreads();
    // the smallest task of each group runs (none if a join was lost)
    if (!uf_bad)
      for (long long t = lo + threadIdx.x; t < hi; t += blockDim.x) {
        if (is_done(t) || uf_root(S.parent, (uint32_t)t) != (uint32_t)t) continue;
        int x, y;
        cell_of(t, x, y);
        if (!merge_up_cell(g, x, y, status) || g.G.fail) abort_all = 1;
        atomicOr(&S.done[t >> 5], 1u << (t & 31));
        atomicAdd(&commits, 1u);
      }
    __syncthreads();
    first_pending(S, lo, n, &lo_s);
    __syncthreads();
    slow = commits < (unsigned int)jb.min_commits ? slow + 1 : 0;
  }
  if (g.G.fail) set_status(status, ST_SIMPLIFY_LIMIT);
  __syncthreads();
  if (threadIdx.x == 0) {
    if (!abort_all) {  // tasks left to one thread, in row-major order
      MGraph f = g;
      f.G.L.top = fin_start;
      f.G.L.pool_cap = pool_end;
      f.G.tmp_cap = tmp_cap0;
      f.G.fail = false;
      for (long long t = 0; t < n && !f.G.fail; ++t) {
        if (is_done(t)) continue;
        int x, y;
        cell_of(t, x, y);
        if (!merge_up_cell(f, x, y, status)) break;
      }
      if (f.G.fail) set_status(status, ST_SIMPLIFY_LIMIT);
    }
    // the slices are used up: later allocations of this graph find no room
    g.G.L.top = pool_end;
    g.G.L.pool_cap = pool_end;
    g.G.tmp_cap = tmp_cap0;
    graphs[jb.g0] = g;
  }
}

MGraph &mg(MGraphHost &h) { return *reinterpret_cast<MGraph *>(h.raw); }

// List pool (runs) beyond the lists themselves for the one-thread steps
// along a shared boundary: lists there relocate to the pool top as they
// grow (the graphs start without slack); retries multiply it.
unsigned long long boundary_room(const int ixn[4]) {
  const unsigned long long cells = (unsigned long long)(ixn[2] - ixn[0] + 1) * (ixn[3] - ixn[1] + 1);
  return (1ull << 20) + 256ull * cells;
}

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Runs the jobs (one block each) and brings the graphs' counters back; adds
// its wall time to *ms.
cudaError_t run_seq(std::vector<MGraphHost *> &graphs, const std::vector<SeqJob> &jobs, uint32_t *status,
                    cudaStream_t st, double *ms) {
  if (jobs.empty()) return cudaSuccess;
  cudaStreamSynchronize(st);
  const double t0 = now_ms();
  struct Acc {
    double *ms, t0;
    ~Acc() { if (ms) *ms += now_ms() - t0; }
  } acc{ms, t0};
  const size_t ng = graphs.size();
  char *buf = nullptr;
  const size_t nj = jobs.size();
  const size_t gb = sizeof(MGraph) * ng, jbytes = sizeof(SeqJob) * nj;
  // merge_up's jobs run in rounds: per job a slot per critical point of its
  // graph (round-tagged keys, all ones = empty) and a pool top
  const bool rounds = jobs[0].kind == SEQ_UP_CANCEL;
  std::vector<size_t> soff(nj, 0);
  size_t sbytes = 0;
  if (rounds)
    for (size_t k = 0; k < nj; ++k) {
      soff[k] = sbytes;
      sbytes += 8ull * ((mg(*graphs[jobs[k].g0]).G.ncp + 1 + 31) / 32 * 32);
    }
  const size_t head = (gb + 15) / 16 * 16 + (jbytes + 15) / 16 * 16, pbytes = rounds ? (8ull * nj + 15) / 16 * 16 : 0;
  cudaError_t e = cudaMallocAsync((void **)&buf, head + pbytes + sbytes + 64, st);
  if (e != cudaSuccess) return e;
  MGraph *dg = (MGraph *)buf;
  SeqJob *dj = (SeqJob *)(buf + ((gb + 15) / 16) * 16);
  unsigned long long **dslot = (unsigned long long **)(buf + head);
  unsigned long long *slots = (unsigned long long *)(buf + head + pbytes);
  std::vector<MGraph> hg(ng);
  for (size_t i = 0; i < ng; ++i) hg[i] = mg(*graphs[i]);
  e = cudaMemcpyAsync(dg, hg.data(), gb, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dj, jobs.data(), jbytes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && rounds) {
    std::vector<unsigned long long *> hp(nj);
    for (size_t k = 0; k < nj; ++k) hp[k] = slots + soff[k] / 8;
    e = cudaMemcpyAsync(dslot, hp.data(), 8ull * nj, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(slots, 0xFF, sbytes, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // hp is read before it goes out of scope
  }
  if (e == cudaSuccess) {
    k_seq_prefetch<<<dim3(64, (unsigned)nj), 256, 0, st>>>(dg, dj, nullptr);
    if (rounds) {
      static const cudaError_t attr = cudaFuncSetAttribute(k_merge_up_rounds, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                           (int)sizeof(RoundSmem));
      e = attr;
      if (e == cudaSuccess)
        k_merge_up_rounds<<<(unsigned)nj, ROUND_THREADS, sizeof(RoundSmem), st>>>(dg, dj, (int)nj, dslot, status);
    } else {
      k_merge_seq<<<(unsigned)nj, 32, 0, st>>>(dg, dj, (int)nj, status);
    }
    DMSC_LAUNCHED(2);
    if (e == cudaSuccess) e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(hg.data(), dg, gb, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess)
    for (size_t i = 0; i < ng; ++i) mg(*graphs[i]) = hg[i];
  cudaFreeAsync(buf, st);
  return e;
}

struct Scratch {  // one device allocation carved into arrays
  char *buf = nullptr;
  std::vector<size_t> sz;
  std::vector<void *> ptr;
  cudaError_t alloc(cudaStream_t st) {
    size_t tot = 0;
    for (size_t s : sz) tot += (s + 255) / 256 * 256;
    cudaError_t e = cudaMallocAsync((void **)&buf, tot + 256, st);
    if (e != cudaSuccess) { buf = nullptr; return e; }
    char *p = buf;
    for (size_t s : sz) { ptr.push_back(p); p += (s + 255) / 256 * 256; }
    return cudaSuccess;
  }
  void free(cudaStream_t st) {
    if (buf) cudaFreeAsync(buf, st);
    buf = nullptr;
  }
};

CsrOut csr_out(dmsc_msc &m) {
  return CsrOut{m.cellid.p, m.pair_idx.p, m.aoff.p, m.asc.p, m.doff.p, m.des.p, m.fn.p, m.flags.p};
}

// merge_up of one pair into o's CSR arrays (before the boundary cancellations);
// *tab receives the cell table of the result over O.bbox (the caller owns it).
cudaError_t union_one(const dmsc_msc &A, const dmsc_msc &B, dmsc_msc &O, CRect ixn, uint32_t *status, uint32_t **tab,
                      cudaStream_t st) {
  const long long nA = A.ncp, nB = B.ncp, bound = nA + nB;
  if (bound >= (1ll << 30) || A.nasc + B.nasc >= (1ll << 32) - 1 || A.ndes + B.ndes >= (1ll << 32) - 1)
    return cudaErrorInvalidValue;  // 32-bit indices and offsets
  const int tw = O.bbox[2] - O.bbox[0] + 1, th = O.bbox[3] - O.bbox[1] + 1;
  if (tw <= 0 || th <= 0) return cudaErrorInvalidValue;
  const size_t tcells = (size_t)tw * th;
  cudaError_t e = cudaMallocAsync((void **)tab, sizeof(uint32_t) * tcells, st);
  if (e != cudaSuccess) { *tab = nullptr; return e; }
  e = cudaMemsetAsync(*tab, 0xFF, sizeof(uint32_t) * tcells, st);
  if (e == cudaSuccess) e = O.cellid.ensure(bound + 1, st);
  if (e == cudaSuccess) e = O.fn.ensure(bound + 1, st);
  if (e == cudaSuccess) e = O.pair_idx.ensure(bound + 1, st);
  if (e == cudaSuccess) e = O.flags.ensure(bound + 1, st);
  if (e == cudaSuccess) e = O.aoff.ensure(bound + 1, st);
  if (e == cudaSuccess) e = O.doff.ensure(bound + 1, st);
  if (e == cudaSuccess) e = O.asc.ensure(A.nasc + B.nasc + 1, st);
  if (e == cudaSuccess) e = O.des.ensure(A.ndes + B.ndes + 1, st);
  if (e != cudaSuccess) return e;
  Scratch s;
  // keepA, idxA, idxB, isnew, posB, tot_a, tot_d, mix, counters
  s.sz = {4ull * (nA + 1), 4ull * (nA + 1), 4ull * (nB + 1), 4ull * (nB + 1), 4ull * (nB + 1),
          4ull * (bound + 1), 4ull * (bound + 1), (size_t)bound + 1, 64};
  if (e == cudaSuccess) e = s.alloc(st);
  if (e != cudaSuccess) return e;
  uint32_t *keep = (uint32_t *)s.ptr[0], *idxA = (uint32_t *)s.ptr[1], *idxB = (uint32_t *)s.ptr[2];
  uint32_t *isnew = (uint32_t *)s.ptr[3], *posB = (uint32_t *)s.ptr[4];
  CellTab H{*tab, O.bbox[0], O.bbox[1], tw, th};
  uint32_t *tot_a = (uint32_t *)s.ptr[5], *tot_d = (uint32_t *)s.ptr[6];
  uint8_t *mix = (uint8_t *)s.ptr[7];
  uint32_t *cnt = (uint32_t *)s.ptr[8];  // [0] kept of A, [1] new of B
  const CsrIn a = csr_in(A), b = csr_in(B);
  CsrOut o = csr_out(O);
  if (e == cudaSuccess) e = cudaMemsetAsync(tot_a, 0, 4ull * (bound + 1), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(tot_d, 0, 4ull * (bound + 1), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(mix, 0, bound + 1, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, 64, st);
  // union (:56-75)
  if (e == cudaSuccess && nA) {
    k_keep<<<nblk(nA), 256, 0, st>>>(a, keep);
    DMSC_LAUNCHED(1);
    e = scan_exclusive_u32(keep, nA, idxA, cnt, st);
    if (e == cudaSuccess) {
      k_up_a<<<nblk(nA), 256, 0, st>>>(a, idxA, H, o, status);
      DMSC_LAUNCHED(1);
    }
  }
  if (e == cudaSuccess && nB) {
    k_up_b_classify<<<nblk(nB), 256, 0, st>>>(b, H, idxB, isnew);
    DMSC_LAUNCHED(1);
    e = scan_exclusive_u32(isnew, nB, posB, cnt + 1, st);
    if (e == cudaSuccess) {
      k_up_b_new<<<nblk(nB), 256, 0, st>>>(b, isnew, posB, cnt, H, idxB, o, status);
      DMSC_LAUNCHED(1);
    }
  }
  // boundary pairs (:84-92), A's then B's
  if (e == cudaSuccess && nA) { k_up_pairs<<<nblk(nA), 256, 0, st>>>(a, idxA, H, o.pair, status); DMSC_LAUNCHED(1); }
  if (e == cudaSuccess && nB) { k_up_pairs<<<nblk(nB), 256, 0, st>>>(b, idxB, H, o.pair, status); DMSC_LAUNCHED(1); }
  // connectivity (:94-121)
  if (e == cudaSuccess && nA) {
    k_up_count<<<nblk(nA), 256, 0, st>>>(a, idxA, false, ixn, tot_a, tot_d, mix, status);
    DMSC_LAUNCHED(1);
  }
  if (e == cudaSuccess && nB) {
    k_up_count<<<nblk(nB), 256, 0, st>>>(b, idxB, true, ixn, tot_a, tot_d, mix, status);
    DMSC_LAUNCHED(1);
  }
  if (e == cudaSuccess) e = scan_exclusive_u32(tot_a, bound, o.aoff, o.aoff + bound, st);
  if (e == cudaSuccess) e = scan_exclusive_u32(tot_d, bound, o.doff, o.doff + bound, st);
  if (e == cudaSuccess && nA) { k_up_write<<<nblk(nA), 256, 0, st>>>(a, idxA, false, ixn, o); DMSC_LAUNCHED(1); }
  if (e == cudaSuccess && nB) { k_up_write<<<nblk(nB), 256, 0, st>>>(b, idxB, true, ixn, o); DMSC_LAUNCHED(1); }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = sort_segments(bound, o.aoff, o.asc, mix, st);
  if (e == cudaSuccess) e = sort_segments(bound, o.doff, o.des, mix, st);
  uint32_t h[4] = {0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, cnt, 8, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h + 2, o.aoff + bound, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h + 3, o.doff + bound, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  s.free(st);
  if (e != cudaSuccess) return e;
  O.ncp = (long long)h[0] + h[1];
  O.nasc = h[2];
  O.ndes = h[3];
  O.any_bcancel = true;
  return cudaSuccess;
}

// A child's complex after merge_down, computed beside it (the child itself
// is replaced only once every merge of the level has succeeded).
struct ChildOut {
  DevBuf<uint32_t> cellid, pair_idx, aoff, asc, doff, des;
  DevBuf<float> fn;
  DevBuf<uint8_t> flags;
  long long ncp = 0, nasc = 0, ndes = 0;
};

template <typename T> void swap_buf(DevBuf<T> &a, DevBuf<T> &b) {
  std::swap(a.p, b.p);
  std::swap(a.n, b.n);
  std::swap(a.pooled, b.pooled);
}

void child_take(dmsc_msc &C, ChildOut &o, const int box[4]) {
  swap_buf(C.cellid, o.cellid); swap_buf(C.pair_idx, o.pair_idx); swap_buf(C.aoff, o.aoff); swap_buf(C.asc, o.asc);
  swap_buf(C.doff, o.doff); swap_buf(C.des, o.des); swap_buf(C.fn, o.fn); swap_buf(C.flags, o.flags);
  C.ncp = o.ncp; C.nasc = o.nasc; C.ndes = o.ndes;
  C.any_bcancel = true;
  for (int i = 0; i < 4; ++i) C.bbox[i] = box[i];
}

// merge_down of parent graph hp into child C (:207-320), into `out`.
// jb/njb: the parent's boundary-cancelable points; adds: a bound on the
// events (partners and list entries of those points); box: the child's box
// grown by the cells those points can add.
cudaError_t down_child(MGraphHost &hp, const uint32_t *jb, uint32_t njb, unsigned long long adds, const dmsc_msc &C,
                       const int box[4], ChildOut &out, uint32_t *status, cudaStream_t st) {
  const MGraph &P = mg(hp);
  const long long n0 = C.ncp, cap = n0 + (long long)adds + 1;
  if (cap >= (1ll << 31)) return cudaErrorInvalidValue;
  const int tw = box[2] - box[0] + 1, th = box[3] - box[1] + 1;
  if (tw <= 0 || th <= 0) return cudaErrorInvalidValue;
  const size_t cells = (size_t)tw * th;
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = out.cellid.ensure(cap, st);
  if (e == cudaSuccess) e = out.fn.ensure(cap, st);
  if (e == cudaSuccess) e = out.pair_idx.ensure(cap, st);
  if (e == cudaSuccess) e = out.flags.ensure(cap, st);
  if (e == cudaSuccess) e = out.aoff.ensure(cap, st);
  if (e == cudaSuccess) e = out.doff.ensure(cap, st);
  if (e != cudaSuccess) return e;
  Scratch s;
  // tab, first, cnt, base, addsrc, kind, addf, rank, src, tot_a, tot_d, need, counters
  s.sz = {4 * cells, 4 * cells, 4ull * (njb + 1), 4ull * (njb + 1), 4ull * (njb + 1), (size_t)njb + 1,
          4ull * (adds + 1), 4ull * (adds + 1), 4ull * cap, 4ull * cap, 4ull * cap, (size_t)cap, 64};
  if ((e = s.alloc(st)) != cudaSuccess) return e;
  DcArgs a;
  a.P = P;
  a.jb = jb;
  a.njb = njb;
  a.c = csr_in(C);
  a.tab = CellTab{(uint32_t *)s.ptr[0], box[0], box[1], tw, th};
  a.first = CellTab{(uint32_t *)s.ptr[1], box[0], box[1], tw, th};
  a.cnt = (uint32_t *)s.ptr[2];
  a.base = (uint32_t *)s.ptr[3];
  a.addsrc = (uint32_t *)s.ptr[4];
  a.kind = (uint8_t *)s.ptr[5];
  a.addf = (uint32_t *)s.ptr[6];
  a.rank = (uint32_t *)s.ptr[7];
  uint32_t *src = (uint32_t *)s.ptr[8], *tot_a = (uint32_t *)s.ptr[9], *tot_d = (uint32_t *)s.ptr[10];
  uint8_t *need = (uint8_t *)s.ptr[11];
  uint32_t *ctr = (uint32_t *)s.ptr[12];  // [0] events, [1] added points
  a.o = CsrOut{out.cellid.p, out.pair_idx.p, out.aoff.p, nullptr, out.doff.p, nullptr, out.fn.p, out.flags.p};
  a.ncp0 = (uint32_t)n0;
  a.status = status;
  e = cudaMemsetAsync(s.ptr[0], 0xFF, 4 * cells, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(s.ptr[1], 0xFF, 4 * cells, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctr, 0, 64, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(a.addf, 0, 4ull * (adds + 1), st);
  if (e == cudaSuccess && n0) {
    k_dc_table<<<nblk(n0), 256, 0, st>>>(a.c, a.tab, status);
    DMSC_LAUNCHED(1);
    e = cudaMemcpyAsync(out.cellid.p, C.cellid.p, 4ull * n0, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out.fn.p, C.fn.p, 4ull * n0, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out.pair_idx.p, C.pair_idx.p, 4ull * n0, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out.flags.p, C.flags.p, n0, cudaMemcpyDeviceToDevice, st);
  }
  if (e == cudaSuccess && njb) {
    k_dc_classify<<<nblk(njb), 256, 0, st>>>(a);
    DMSC_LAUNCHED(1);
    e = scan_exclusive_u32(a.cnt, njb, a.base, ctr, st);
    if (e == cudaSuccess) {
      k_dc_first<<<nblk(njb), 256, 0, st>>>(a);
      k_dc_addflags<<<nblk(njb), 256, 0, st>>>(a);
      DMSC_LAUNCHED(2);
      e = scan_exclusive_u32(a.addf, (long long)adds + 1, a.rank, ctr + 1, st);
    }
    if (e == cudaSuccess) {
      k_dc_add<<<nblk(njb), 256, 0, st>>>(a);
      k_dc_pairing<<<nblk(njb), 256, 0, st>>>(a);
      DMSC_LAUNCHED(2);
      e = cudaGetLastError();
    }
  }
  uint32_t hc[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(hc, ctr, 8, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  const long long n = n0 + hc[1];
  if (e == cudaSuccess && (unsigned long long)hc[0] > adds) e = cudaErrorInvalidValue;  // the event bound failed
  // the lists (:283-320): taken from the parent where it holds the cell
  if (e == cudaSuccess && n) {
    k_dc_src<<<nblk(n), 256, 0, st>>>(a, (uint32_t)n, src);
    k_dc_count<<<nblk(n), 256, 0, st>>>(a, (uint32_t)n, src, tot_a, tot_d, need);
    DMSC_LAUNCHED(2);
  }
  if (e == cudaSuccess) e = scan_exclusive_u32(tot_a, n, out.aoff.p, out.aoff.p + n, st);
  if (e == cudaSuccess) e = scan_exclusive_u32(tot_d, n, out.doff.p, out.doff.p + n, st);
  uint32_t tot[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(&tot[0], out.aoff.p + n, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&tot[1], out.doff.p + n, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = out.asc.ensure((size_t)tot[0] + 1, st);
  if (e == cudaSuccess) e = out.des.ensure((size_t)tot[1] + 1, st);
  if (e == cudaSuccess && n) {
    a.o.asc = out.asc.p;
    a.o.des = out.des.p;
    k_dc_write<<<nblk(n), 256, 0, st>>>(a, (uint32_t)n, src);
    DMSC_LAUNCHED(1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = sort_segments(n, out.aoff.p, out.asc.p, need, st);
  if (e == cudaSuccess) e = sort_segments(n, out.doff.p, out.des.p, need, st);
  s.free(st);
  if (e != cudaSuccess) return e;
  out.ncp = n;
  out.nasc = tot[0];
  out.ndes = tot[1];
  return cudaSuccess;
}

}  // namespace

namespace {
constexpr int MERGE_WORKERS = 8;

cudaError_t as_cuda(int rc) {
  return rc == 0 ? cudaSuccess : rc < 0 ? cudaErrorUnknown : (cudaError_t)rc;
}
int current_device() {
  int d = 0;
  cudaGetDevice(&d);
  return d;
}
}  // namespace

// The merges of a level run side by side on their own streams (several host
// threads); the one-thread steps of all of them run in one launch on `st`.
cudaError_t merge_up_level_par(const std::vector<MergeJob> &jobs, unsigned long long grow, uint32_t *status,
                               uint32_t *stw, cudaStream_t st, double *seq_ms, long long round_window,
                               long long round_min_commits) {
  *stw = 0;
  const int nj = (int)jobs.size(), dev = current_device();
  cudaError_t e = cudaMemsetAsync(status, 0, 4, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  // union and connectivity; each result's cell table passes to its graph
  std::vector<MGraphHost> g(nj);
  std::vector<uint32_t *> tabs(nj, nullptr);
  if (e == cudaSuccess)
    e = as_cuda(for_each_on_streams(dev, nj, MERGE_WORKERS, [&](int k, cudaStream_t s) {
      const MergeJob &J = jobs[k];
      return (int)union_one(*J.a, *J.b, *J.parent, CRect{J.ixn[0], J.ixn[1], J.ixn[2], J.ixn[3]}, status, &tabs[k], s);
    }));
  if (e == cudaSuccess) e = cudaMemcpy(stw, status, 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess || *stw) {
    for (uint32_t *t : tabs)
      if (t) cudaFreeAsync(t, st);
    cudaStreamSynchronize(st);
    return e;
  }
  // the boundary cancellations, one thread per merge, on mutable graphs
  std::vector<MGraphHost *> gp;
  std::vector<SeqJob> seq;
  for (int k = 0; k < nj; ++k) {
    const int *x = jobs[k].ixn;
    gp.push_back(&g[k]);
    SeqJob j{SEQ_UP_CANCEL, k, CRect{x[0], x[1], x[2], x[3]}};
    j.win = (int)std::min<long long>(std::max<long long>(round_window, 0), 1 << 30);
    j.min_commits = (int)std::min<long long>(std::max<long long>(round_min_commits, 0), 1 << 30);
    seq.push_back(j);
  }
  e = as_cuda(for_each_on_streams(dev, nj, MERGE_WORKERS, [&](int k, cudaStream_t s) {
    const dmsc_msc &O = *jobs[k].parent;
    g[k].status = status;
    const cudaError_t r =
        mgraph_alloc(g[k], O, (uint32_t)O.ncp, O.nasc + O.ndes + grow * boundary_room(jobs[k].ixn), s, 0, tabs[k]);
    if (g[k].tab) tabs[k] = nullptr;  // the graph owns it now
    return (int)r;
  }));
  for (uint32_t *t : tabs)
    if (t) cudaFreeAsync(t, st);
  if (e == cudaSuccess) e = run_seq(gp, seq, status, st, seq_ms);
  if (e == cudaSuccess) e = cudaMemcpy(stw, status, 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && !*stw)
    e = as_cuda(for_each_on_streams(dev, nj, MERGE_WORKERS,
                                    [&](int k, cudaStream_t s) { return (int)mgraph_to_csr(g[k], *jobs[k].parent, s); }));
  for (auto &h : g) mgraph_free(h, st);
  cudaStreamSynchronize(st);
  return e;
}

cudaError_t merge_down_level_par(const std::vector<MergeJob> &jobs, unsigned long long grow, uint32_t *status,
                                 uint32_t *stw, cudaStream_t st, double *seq_ms) {
  *stw = 0;
  const int nj = (int)jobs.size(), dev = current_device();
  cudaError_t e = cudaMemsetAsync(status, 0, 4, st);
  // the parents' graphs
  std::vector<MGraphHost> g(nj);
  std::vector<MGraphHost *> gp;
  for (auto &h : g) gp.push_back(&h);
  std::vector<SeqJob> seq;
  for (int k = 0; k < nj; ++k) {
    const int *x = jobs[k].ixn;
    seq.push_back(SeqJob{SEQ_DOWN_BOUNDARY, k, CRect{x[0], x[1], x[2], x[3]}});
  }
  // scratch: per job the boundary-cancelable flags, positions and list; counters
  Scratch s;
  for (int k = 0; k < nj; ++k) {
    const long long n = jobs[k].parent->ncp;
    for (int q = 0; q < 3; ++q) s.sz.push_back(4ull * (n + 1));
  }
  s.sz.push_back(16ull * (nj + 1));  // per job: count, adds
  s.sz.push_back(16ull * (nj + 1));  // per job: the box of the cells its boundary points can add
  if (e == cudaSuccess) e = s.alloc(st);
  unsigned long long *ctr = e == cudaSuccess ? (unsigned long long *)s.ptr[3 * nj] : nullptr;
  int *boxes = e == cudaSuccess ? (int *)s.ptr[3 * nj + 1] : nullptr;
  std::vector<int> hbox(4 * (nj + 1));
  for (int k = 0; k <= nj; ++k) {
    hbox[4 * k] = hbox[4 * k + 1] = 1 << 30;
    hbox[4 * k + 2] = hbox[4 * k + 3] = -1;
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(ctr, 0, 16ull * (nj + 1), st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(boxes, hbox.data(), 16ull * (nj + 1), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess)
    e = as_cuda(for_each_on_streams(dev, nj, MERGE_WORKERS, [&](int k, cudaStream_t q) {
      const dmsc_msc &P = *jobs[k].parent;
      g[k].status = status;
      return (int)mgraph_alloc(g[k], P, (uint32_t)P.ncp, P.nasc + P.ndes + grow * boundary_room(jobs[k].ixn), q, 0);
    }));
  // the uncancellations along each shared boundary (:172-201)
  if (e == cudaSuccess) e = run_seq(gp, seq, status, st, seq_ms);
  // checks, the boundary-cancelable lists and the bounds of the children's growth
  if (e == cudaSuccess)
    e = as_cuda(for_each_on_streams(dev, nj, MERGE_WORKERS, [&](int k, cudaStream_t q) {
      MGraph &P = mg(g[k]);
      uint32_t *bflag = (uint32_t *)s.ptr[3 * k], *pos = (uint32_t *)s.ptr[3 * k + 1], *jb = (uint32_t *)s.ptr[3 * k + 2];
      uint32_t *njb = (uint32_t *)(ctr + 2 * k);
      if (!P.G.ncp) return 0;
      k_down_check<<<nblk(P.G.ncp), 256, 0, q>>>(P, bflag, status);
      DMSC_LAUNCHED(1);
      cudaError_t r = scan_exclusive_u32(bflag, P.G.ncp, pos, njb, q);
      if (r == cudaSuccess) {
        k_down_list<<<nblk(P.G.ncp), 256, 0, q>>>(P, bflag, pos, jb, ctr + 2 * k + 1, boxes + 4 * k);
        DMSC_LAUNCHED(1);
        r = cudaGetLastError();
      }
      return (int)r;
    }));
  std::vector<unsigned long long> hc(2 * (nj + 1), 0);
  if (e == cudaSuccess) e = cudaMemcpy(hc.data(), ctr, 16ull * nj, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(hbox.data(), boxes, 16ull * nj, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(stw, status, 4, cudaMemcpyDeviceToHost);
  // each child's box grows by the cells its parent's boundary points can add
  std::vector<int> cbox(8 * nj);
  for (int k = 0; k < nj; ++k)
    for (int c = 0; c < 2; ++c) {
      const dmsc_msc &C = *(c ? jobs[k].b : jobs[k].a);
      int *o = &cbox[8 * k + 4 * c];
      const int *t = &hbox[4 * k];
      for (int i = 0; i < 4; ++i) o[i] = C.bbox[i];
      if (t[2] >= 0) {
        o[0] = std::min(o[0], t[0]); o[1] = std::min(o[1], t[1]);
        o[2] = std::max(o[2], t[2]); o[3] = std::max(o[3], t[3]);
      }
    }
  // the parent into each child (:207-320), beside the child
  std::vector<ChildOut> outs(2 * nj);
  if (e == cudaSuccess && !*stw)
    e = as_cuda(for_each_on_streams(dev, 2 * nj, MERGE_WORKERS, [&](int kc, cudaStream_t q) {
      const int k = kc / 2, c = kc % 2;
      const dmsc_msc &C = *(c ? jobs[k].b : jobs[k].a);
      return (int)down_child(g[k], (const uint32_t *)s.ptr[3 * k + 2], (uint32_t)hc[2 * k], hc[2 * k + 1], C,
                             &cbox[8 * k + 4 * c], outs[kc], status, q);
    }));
  if (e == cudaSuccess && !*stw) e = cudaMemcpy(stw, status, 4, cudaMemcpyDeviceToHost);
  // every merge of the level succeeded: the children take their new
  // complexes and the parents are written back
  if (e == cudaSuccess && !*stw) {
    for (int kc = 0; kc < 2 * nj; ++kc) child_take(*(kc % 2 ? jobs[kc / 2].b : jobs[kc / 2].a), outs[kc], &cbox[4 * kc]);
    e = as_cuda(for_each_on_streams(dev, nj, MERGE_WORKERS,
                                    [&](int k, cudaStream_t q) { return (int)mgraph_to_csr(g[k], *jobs[k].parent, q); }));
  }
  s.free(st);
  for (auto &h : g) mgraph_free(h, st);
  cudaStreamSynchronize(st);
  return e;
}

}  // namespace dmsc
