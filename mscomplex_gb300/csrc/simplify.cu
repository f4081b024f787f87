// simplify.cu -- persistence simplification of a Morse-Smale complex on the
// device: GridMSComplex::simplify + un_simplify (dmsc/src/grid_mscomplex.cpp:
// 384-526) with cancelPairs (dmsc/include/discreteMorseAlgorithm.h:466-585)
// and uncancel_pairs (:1006-1089).
//
// The reference pops a std::priority_queue whose comparator (grid_mscomplex.cpp:
// 331-379) reads c3/c4 from p1, so for equal persistence it returns false both
// ways: the order among ties is whatever the binary-heap algorithms produce.
// The result depends on that order (including the order produced by the
// strangulation resubmissions, :474-479, 503-508), so this pass replays the
// heap exactly: the standard bottom-up binary heap of push_heap / pop_heap
// (hole sifted down to a leaf choosing the right child unless the left one is
// strictly smaller, then the last element sifted up) -- the algorithm of the
// C++ standard library the reference is built with.  Persistence |f2 - f1| is
// precomputed per heap entry; the comparator is "d1 > d2" (a min-heap on d).
//
// The replay is sequential by nature and runs on one thread of one block.
// Multisets (critical_point::asc / des, std::multiset<uint>) are run-length
// encoded sorted arrays in a device pool; they grow by reallocation inside it.
// Every loop is bounded: the pass stops with ST_SIMPLIFY_LIMIT when the
// operation budget or a pool runs out, leaving the complex unmodified.
#include "dmsc_common.cuh"
#include "dmsc_internal.h"

namespace dmsc {

struct HeapEnt {
  float d;
  uint32_t a, b;
};

// IEEE single subtraction without contraction on either side of the compiler.
__host__ __device__ __forceinline__ float fsub_rn(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  volatile float r = a - b;
  return r;
#endif
}

// flags bits of a critical point (as exported by dmsc_msc_export)
constexpr uint8_t F_CANCELLED = 1, F_STRANG = 2, F_BCANCEL = 4;

// Multisets are run-length encoded: sorted (value, count) runs, so equal
// elements stay consecutive exactly as std::multiset iterates them, and a
// multiplicity of thousands costs one run.
struct Lists {  // list 2*cp = asc, 2*cp+1 = des
  uint32_t *off, *nrun, *cap;  // runs of list l live at pool[off[l] .. off[l]+nrun[l])
  uint32_t *total;             // multiset size (sum of counts)
  uint2 *pool;                 // .x = value, .y = count
  unsigned long long top, pool_cap;
};

struct SimpArgs {
  uint32_t ncp;
  const uint32_t *cellid;
  const float *fn;
  uint8_t *flags;
  uint32_t *pair_idx;
  Lists L;
  HeapEnt *heap;
  unsigned long long heap_cap;
  uint2 *resub;       // resubmit list (capacity heap_cap)
  uint2 *canc;        // cancellation list (capacity ncp)
  uint2 *tmp;         // new_edges (d, a) / uncancel runs (capacity tmp_cap)
  unsigned long long tmp_cap;
  int rx0, ry0, rx1, ry1;  // m_rect of the complex (cell coordinates)
  double tresh;
  unsigned long long max_ops;
  unsigned long long *stats;  // [0] pushes [1] pops [2] cancels [3] ops [4] status
};

struct Simp {
  SimpArgs A;
  unsigned long long nheap = 0, nres = 0, ncanc = 0, ops = 0;
  bool fail = false;

  __host__ __device__ __forceinline__ int dim(uint32_t k) const {
    uint32_t c = A.cellid[k];
    return (int)(c & 1u) + (int)((c >> 16) & 1u);
  }
  __host__ __device__ __forceinline__ bool on_boundary(uint32_t k) const {  // m_rect.isOnBoundry
    uint32_t c = A.cellid[k];
    int x = (int16_t)(c & 0xffff), y = (int16_t)(c >> 16);
    bool contains = x >= A.rx0 && y >= A.ry0 && x <= A.rx1 && y <= A.ry1;
    bool interior = x > A.rx0 && y > A.ry0 && x < A.rx1 && y < A.ry1;
    return contains && !interior;
  }
  __host__ __device__ __forceinline__ float pers(uint32_t a, uint32_t b) const {
    return fabsf(fsub_rn(A.fn[b], A.fn[a]));
  }
  __host__ __device__ __forceinline__ bool tick(unsigned long long n = 1) {
    ops += n;
    if (ops > A.max_ops) fail = true;
    return !fail;
  }

  // ---- run-length multisets ----
  __host__ __device__ __forceinline__ uint2 *runs(uint32_t l) const { return A.L.pool + A.L.off[l]; }
  __host__ __device__ uint32_t find_run(uint32_t l, uint32_t x) const {  // first run with value >= x
    const uint2 *p = runs(l);
    uint32_t lo = 0, hi = A.L.nrun[l];
    while (lo < hi) { uint32_t m = (lo + hi) >> 1; if (p[m].x < x) lo = m + 1; else hi = m; }
    return lo;
  }
  __host__ __device__ uint32_t count(uint32_t l, uint32_t x) const {
    uint32_t i = find_run(l, x);
    return (i < A.L.nrun[l] && runs(l)[i].x == x) ? runs(l)[i].y : 0u;
  }
  __host__ __device__ bool contains(uint32_t l, uint32_t x) const { return count(l, x) != 0; }
  __host__ __device__ bool reserve(uint32_t l, uint32_t need) {
    if (need <= A.L.cap[l]) return true;
    uint32_t nc = A.L.cap[l] * 2 + 4;
    while (nc < need) nc *= 2;
    if (A.L.top + nc > A.L.pool_cap) { fail = true; return false; }
    uint2 *src = runs(l), *dst = A.L.pool + A.L.top;
    for (uint32_t i = 0; i < A.L.nrun[l]; ++i) dst[i] = src[i];
    A.L.off[l] = (uint32_t)A.L.top;
    A.L.cap[l] = nc;
    A.L.top += nc;
    return true;
  }
  __host__ __device__ void insert(uint32_t l, uint32_t x, uint32_t c = 1) {  // std::multiset::insert, c times
    uint32_t i = find_run(l, x), n = A.L.nrun[l];
    if (i < n && runs(l)[i].x == x) {
      uint2 &r = runs(l)[i];
      if (r.y > 0xffffffffu - c) { fail = true; return; }
      r.y += c;
    } else {
      if (!reserve(l, n + 1)) return;
      uint2 *p = runs(l);
      for (uint32_t k = n; k > i; --k) p[k] = p[k - 1];
      p[i] = make_uint2(x, c);
      A.L.nrun[l] = n + 1;
      tick(n - i);
    }
    if (A.L.total[l] > 0xffffffffu - c) { fail = true; return; }
    A.L.total[l] += c;
  }
  __host__ __device__ void erase(uint32_t l, uint32_t x) {  // std::multiset::erase(key): all copies
    uint32_t i = find_run(l, x), n = A.L.nrun[l];
    if (i >= n || runs(l)[i].x != x) return;
    uint2 *p = runs(l);
    A.L.total[l] -= p[i].y;
    for (uint32_t k = i + 1; k < n; ++k) p[k - 1] = p[k];
    A.L.nrun[l] = n - 1;
    tick(n - i);
  }

  // ---- heap (binary heap of the standard library, comparator d1 > d2) ----
  __host__ __device__ __forceinline__ static bool comp(const HeapEnt &x, const HeapEnt &y) { return x.d > y.d; }
  __host__ __device__ void push_at(unsigned long long hole, unsigned long long topi, HeapEnt val) {
    HeapEnt *v = A.heap;
    unsigned long long parent = (hole - 1) / 2;
    while (hole > topi && comp(v[parent], val)) {
      v[hole] = v[parent];
      hole = parent;
      parent = (hole - 1) / 2;
    }
    v[hole] = val;
  }
  __host__ __device__ void push(uint32_t a, uint32_t b) {
    if (nheap >= A.heap_cap) { fail = true; return; }
    HeapEnt x{pers(a, b), a, b};
    A.heap[nheap] = x;
    push_at(nheap, 0, x);
    ++nheap;
    ++A.stats[0];
  }
  __host__ __device__ HeapEnt pop() {
    HeapEnt *v = A.heap;
    HeapEnt top = v[0];
    if (nheap > 1) {
      unsigned long long len = nheap - 1;
      HeapEnt val = v[len];
      v[len] = v[0];
      unsigned long long hole = 0, second = 0;
      while (second < (len - 1) / 2) {
        second = 2 * (second + 1);
        if (comp(v[second], v[second - 1])) second--;
        v[hole] = v[second];
        hole = second;
      }
      if ((len & 1) == 0 && second == (len - 2) / 2) {
        second = 2 * (second + 1);
        v[hole] = v[second - 1];
        hole = second - 1;
      }
      push_at(hole, 0, val);
    }
    --nheap;
    ++A.stats[1];
    return top;
  }

  // cancelPairs(msc, cp0, cp1, new_edges) (discreteMorseAlgorithm.h:466-585).
  // The new edges (d, a) are pushed onto the heap in the reference's order:
  // every occurrence of a (ascending) times every occurrence of d (ascending).
  __host__ __device__ void cancel_pairs(uint32_t cp0, uint32_t cp1) {
    if (!contains(2 * cp0, cp1)) { uint32_t t = cp0; cp0 = cp1; cp1 = t; }
    if (!contains(2 * cp0, cp1)) return;  // "critical points are not connected"
    const uint32_t la0 = 2 * cp0, ld1 = 2 * cp1 + 1;
    // 1. connections: collect (d, a) runs first (the iterated lists do not change)
    for (uint32_t i = 0; i < A.L.nrun[la0] && !fail; ++i) {
      uint2 ra = runs(la0)[i];
      if (ra.x == cp1) continue;
      for (uint32_t j = 0; j < A.L.nrun[ld1] && !fail; ++j) {
        uint2 rd = runs(ld1)[j];
        if (rd.x == cp0) continue;
        unsigned long long c = (unsigned long long)ra.y * rd.y;
        if (c > 0xffffffffull) { fail = true; return; }
        insert(2 * ra.x + 1, rd.x, (uint32_t)c);
        insert(2 * rd.x, ra.x, (uint32_t)c);
        if (count(2 * ra.x + 1, rd.x) >= 2) {
          A.flags[ra.x] |= F_STRANG;
          A.flags[rd.x] |= F_STRANG;
        }
        if (!tick(c)) return;
      }
    }
    // 2. heap pushes of the new edges, in the reference's order
    for (uint32_t i = 0; i < A.L.nrun[la0] && !fail; ++i) {
      uint2 ra = runs(la0)[i];
      if (ra.x == cp1) continue;
      for (uint32_t ca = 0; ca < ra.y && !fail; ++ca)
        for (uint32_t j = 0; j < A.L.nrun[ld1] && !fail; ++j) {
          uint2 rd = runs(ld1)[j];
          if (rd.x == cp0) continue;
          for (uint32_t cd = 0; cd < rd.y && !fail; ++cd) push(rd.x, ra.x);
        }
    }
    if (fail) return;
    // 3. remove the pair from its neighbours
    for (uint32_t i = 0; i < A.L.nrun[la0]; ++i) {
      uint32_t a = runs(la0)[i].x;
      if (a == cp1) continue;
      erase(2 * a + 1, cp0);
    }
    for (uint32_t i = 0; i < A.L.nrun[2 * cp0 + 1]; ++i) erase(2 * runs(2 * cp0 + 1)[i].x, cp0);
    for (uint32_t i = 0; i < A.L.nrun[2 * cp1]; ++i) erase(2 * runs(2 * cp1)[i].x + 1, cp1);
    for (uint32_t i = 0; i < A.L.nrun[ld1]; ++i) {
      uint32_t d = runs(ld1)[i].x;
      if (d == cp0) continue;
      erase(2 * d, cp1);
    }
    A.flags[cp0] |= F_CANCELLED;
    A.L.nrun[2 * cp0 + 1] = 0; A.L.total[2 * cp0 + 1] = 0;
    A.flags[cp1] |= F_CANCELLED;
    A.L.nrun[2 * cp1] = 0; A.L.total[2 * cp1] = 0;
  }

  // heap sort of tmp[0..n) by value (in place, O(n log n))
  __host__ __device__ void sort_runs(unsigned long long n) {
    uint2 *t = A.tmp;
    auto sift = [&](unsigned long long root, unsigned long long end) {
      while (2 * root + 1 < end) {
        unsigned long long c = 2 * root + 1;
        if (c + 1 < end && t[c].x < t[c + 1].x) ++c;
        if (t[root].x < t[c].x) { uint2 q = t[root]; t[root] = t[c]; t[c] = q; root = c; }
        else return;
      }
    };
    for (unsigned long long s = n / 2; s-- > 0;) sift(s, n);
    for (unsigned long long e = n; e-- > 1;) { uint2 q = t[0]; t[0] = t[e]; t[e] = q; sift(0, e); }
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
      for (uint32_t k = 0; k < A.L.nrun[l]; ++k) {
        uint2 rx = runs(l)[k];
        if (rx.x == other) continue;
        if (!(A.flags[rx.x] & F_BCANCEL)) {
          if (n >= A.tmp_cap) { fail = true; return true; }
          A.tmp[n++] = rx;
          continue;
        }
        if (A.flags[rx.x] & F_CANCELLED) return false;
        uint32_t pidx = A.pair_idx[rx.x];
        if (pidx >= A.ncp || A.pair_idx[pidx] != rx.x) return false;
        uint32_t pl = 2 * pidx + i;
        for (uint32_t q = 0; q < A.L.nrun[pl]; ++q) {
          uint2 ry = runs(pl)[q];
          if (A.flags[ry.x] & F_BCANCEL) return false;
          unsigned long long c = (unsigned long long)rx.y * ry.y;
          if (c > 0xffffffffull || n >= A.tmp_cap) { fail = true; return true; }
          A.tmp[n++] = make_uint2(ry.x, (uint32_t)c);
        }
        if (!tick(1 + A.L.nrun[pl])) return true;
      }
      if (!tick(n + 1)) return true;
      sort_runs(n);
      // merge equal values into runs
      unsigned long long m = 0, tot = 0;
      for (unsigned long long u = 0; u < n; ++u) {
        if (m > 0 && A.tmp[m - 1].x == A.tmp[u].x) {
          unsigned long long c = (unsigned long long)A.tmp[m - 1].y + A.tmp[u].y;
          if (c > 0xffffffffull) { fail = true; return true; }
          A.tmp[m - 1].y = (uint32_t)c;
        } else {
          A.tmp[m++] = A.tmp[u];
        }
        tot += A.tmp[u].y;
      }
      if (tot > 0xffffffffull || m > 0xffffffffull || !reserve(l, (uint32_t)m)) { fail = true; return true; }
      uint2 *p = runs(l);
      for (unsigned long long u = 0; u < m; ++u) p[u] = A.tmp[u];
      A.L.nrun[l] = (uint32_t)m;
      A.L.total[l] = (uint32_t)tot;
    }
    A.flags[c1] &= ~F_CANCELLED;
    A.flags[c2] &= ~F_CANCELLED;
    return true;
  }

  // simplify (grid_mscomplex.cpp:384-512) followed by un_simplify (:514-526)
  __host__ __device__ void run() {
    const uint32_t n = A.ncp;
    float max_val = 1.17549435e-38f;  // std::numeric_limits<float>::min(), as in the reference (:399)
    float min_val = 3.40282347e+38f;
    for (uint32_t i = 0; i < n && !fail; ++i) {
      if (dim(i) == 1) {
        for (int j = 0; j < 2; ++j) {
          uint32_t l = 2 * i + j;
          if (A.L.total[l] != 2) continue;
          if (runs(l)[0].y == 2) A.flags[i] |= F_STRANG;  // both elements equal
        }
      }
      float f = A.fn[i];
      max_val = (max_val < f) ? f : max_val;  // std::max
      min_val = (f < min_val) ? f : min_val;  // std::min
      const uint32_t ld = 2 * i + 1;
      for (uint32_t k = 0; k < A.L.nrun[ld] && !fail; ++k)
        for (uint32_t c = 0; c < runs(ld)[k].y && !fail; ++c) push(i, runs(ld)[k].x);
    }
    const float max_persistence = fsub_rn(max_val, min_val);
    while (nheap != 0 && !fail) {
      if (!tick()) break;
      HeapEnt e = pop();
      uint32_t v1 = e.a, v2 = e.b;
      if ((double)e.d / (double)max_persistence > A.tresh) break;
      if (dim(v2) == 1) { uint32_t t = v1; v1 = v2; v2 = t; }
      const int cp2_dim = dim(v2);
      if ((A.flags[v1] & F_CANCELLED) || (A.flags[v2] & F_CANCELLED)) continue;
      bool b1 = on_boundary(v1), b2 = on_boundary(v2);
      if (b1 && !b2) continue;
      if (!b1 && b2) continue;
      const bool strang = A.flags[v1] & F_STRANG;
      if (strang && A.L.total[2 * v2 + cp2_dim / 2] != 1) {
        if (nres >= A.heap_cap) { fail = true; break; }
        A.resub[nres++] = make_uint2(e.a, e.b);
        continue;
      }
      if (strang && b1) continue;
      cancel_pairs(v1, v2);
      if (fail) break;
      A.flags[v1] |= F_BCANCEL;
      A.flags[v2] |= F_BCANCEL;
      A.pair_idx[v1] = v2;
      A.pair_idx[v2] = v1;
      if (ncanc >= n) { fail = true; break; }
      A.canc[ncanc++] = make_uint2(e.a, e.b);
      for (unsigned long long i = 0; i < nres && !fail; ++i) push(A.resub[i].x, A.resub[i].y);
      nres = 0;
    }
    A.stats[2] = ncanc;
    if (fail) return;
    for (unsigned long long k = ncanc; k-- > 0;) {
      uint2 c = A.canc[k];
      if (!uncancel_pairs(c.x, c.y)) { A.stats[4] |= ST_INVARIANT; return; }
      if (fail) return;
    }
  }
};

__global__ void k_simplify(SimpArgs a) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  Simp s;
  s.A = a;
  s.run();
  a.stats[3] = s.ops;
  if (s.fail) a.stats[4] |= ST_SIMPLIFY_LIMIT;
}

// CSR (expanded, ascending) -> run-length lists.  Capacity of a list is its
// CSR length + 4 runs; asc lists first, des lists after them.
__global__ void k_lists_from_csr(uint32_t ncp, const uint32_t *aoff, const uint32_t *asc, const uint32_t *doff,
                                 const uint32_t *des, unsigned long long des_base, uint32_t *off, uint32_t *nrun,
                                 uint32_t *cap, uint32_t *total, uint2 *pool) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ncp; i += gridDim.x * blockDim.x) {
    for (int w = 0; w < 2; ++w) {
      const uint32_t *o = w ? doff : aoff, *src = w ? des : asc;
      uint32_t b = o[i], e = o[i + 1];
      uint32_t base = w ? (uint32_t)(des_base + (unsigned long long)b + 4ull * i) : (uint32_t)(b + 4u * i);
      uint32_t m = 0;
      for (uint32_t k = b; k < e; ++k) {
        if (m > 0 && pool[base + m - 1].x == src[k]) pool[base + m - 1].y += 1;
        else pool[base + m++] = make_uint2(src[k], 1u);
      }
      off[2 * i + w] = base; nrun[2 * i + w] = m; cap[2 * i + w] = (e - b) + 4; total[2 * i + w] = e - b;
    }
  }
}

// run-length lists -> expanded CSR (offsets from a scan of the totals)
__global__ void k_csr_from_lists(uint32_t ncp, const uint32_t *off, const uint32_t *nrun, const uint2 *pool, int which,
                                 const uint32_t *outoff, uint32_t *out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ncp; i += gridDim.x * blockDim.x) {
    uint32_t l = 2 * i + which, o = outoff[i];
    const uint2 *p = pool + off[l];
    for (uint32_t k = 0; k < nrun[l]; ++k)
      for (uint32_t c = 0; c < p[k].y; ++c) out[o++] = p[k].x;
  }
}
__global__ void k_pick_len(uint32_t ncp, const uint32_t *len, int which, uint32_t *out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ncp; i += gridDim.x * blockDim.x) out[i] = len[2 * i + which];
}

static unsigned blocks_for(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (unsigned)(b < 1 ? 1 : b);
}

// Work buffers of one simplification (one stream-ordered allocation).
struct SimplifyWork {
  SimpArgs a;
  char *buf = nullptr;
  uint8_t *flags_in = nullptr;     // caller's arrays, written back on success
  uint32_t *pair_in = nullptr;
  uint32_t *lens = nullptr;        // ncp words for the rebuilt offsets
};

cudaError_t simplify_run(SimplifyIO &io, cudaStream_t st) {
  const uint32_t ncp = (uint32_t)io.ncp;
  unsigned long long des_base = (unsigned long long)io.nasc + 4ull * ncp;
  unsigned long long base_top = des_base + (unsigned long long)io.ndes + 4ull * ncp;
  unsigned long long pool_cap = base_top + (io.pool_extra ? io.pool_extra : (2 * base_top + (1ull << 22)));
  unsigned long long heap_cap = io.heap_cap ? io.heap_cap : (4ull * io.ndes + (1ull << 20));
  unsigned long long tmp_cap = io.tmp_cap ? io.tmp_cap : (1ull << 22);
  if (pool_cap > 0xffffffffull) return cudaErrorInvalidValue;  // list offsets are 32-bit
  auto rnd = [](size_t n) { return (n + 255) / 256 * 256; };
  size_t sizes[] = {sizeof(uint32_t) * 2 * ncp, sizeof(uint32_t) * 2 * ncp, sizeof(uint32_t) * 2 * ncp,
                    sizeof(uint32_t) * 2 * ncp, sizeof(uint2) * pool_cap, sizeof(uint2) * tmp_cap, sizeof(HeapEnt) * heap_cap,
                    sizeof(uint2) * heap_cap, sizeof(uint2) * (ncp + 1), sizeof(unsigned long long) * 8,
                    sizeof(uint8_t) * (ncp + 1), sizeof(uint32_t) * (ncp + 1), sizeof(uint32_t) * (ncp + 1)};
  size_t bytes = 0;
  for (size_t z : sizes) bytes += rnd(z);
  SimplifyWork *w = new SimplifyWork;
  io.work = w;
  cudaError_t e = cudaMallocAsync((void **)&w->buf, bytes, st);
  if (e != cudaSuccess) { w->buf = nullptr; return e; }
  char *p = w->buf;
  int si = 0;
  auto take = [&]() { char *r = p; p += rnd(sizes[si++]); return r; };
  SimpArgs &a = w->a;
  a.ncp = ncp;
  a.cellid = io.cellid;
  a.fn = io.fn;
  a.L.off = (uint32_t *)take();
  a.L.nrun = (uint32_t *)take();
  a.L.cap = (uint32_t *)take();
  a.L.total = (uint32_t *)take();
  a.L.pool = (uint2 *)take();
  a.L.top = base_top;
  a.L.pool_cap = pool_cap;
  a.tmp = (uint2 *)take();
  a.tmp_cap = tmp_cap;
  a.heap = (HeapEnt *)take();
  a.heap_cap = heap_cap;
  a.resub = (uint2 *)take();
  a.canc = (uint2 *)take();
  a.stats = (unsigned long long *)take();
  a.flags = (uint8_t *)take();
  a.pair_idx = (uint32_t *)take();
  w->lens = (uint32_t *)take();
  w->flags_in = io.flags;
  w->pair_in = io.pair_idx;
  a.rx0 = io.rect[0]; a.ry0 = io.rect[1]; a.rx1 = io.rect[2]; a.ry1 = io.rect[3];
  a.tresh = io.tresh;
  a.max_ops = io.max_ops;
  e = cudaMemsetAsync(a.stats, 0, sizeof(unsigned long long) * 8, st);
  if (e == cudaSuccess && ncp) e = cudaMemcpyAsync(a.flags, io.flags, ncp, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && ncp) e = cudaMemcpyAsync(a.pair_idx, io.pair_idx, 4ull * ncp, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return e;
  if (ncp) {
    k_lists_from_csr<<<blocks_for(ncp), 256, 0, st>>>(ncp, io.aoff, io.asc, io.doff, io.des, des_base, a.L.off,
                                                       a.L.nrun, a.L.cap, a.L.total, a.L.pool);
    DMSC_LAUNCHED(1);
    k_simplify<<<1, 32, 0, st>>>(a);
    DMSC_LAUNCHED(1);
  }
  e = cudaMemcpyAsync(io.host_stats, a.stats, sizeof(unsigned long long) * 5, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess || io.host_stats[4] != 0 || !ncp) return e;
  // new CSR offsets (asc, then des) from the list lengths
  for (int which = 0; which < 2 && e == cudaSuccess; ++which) {
    uint32_t *offs = which ? io.doff : io.aoff;
    k_pick_len<<<blocks_for(ncp), 256, 0, st>>>(ncp, a.L.total, which, w->lens);
    DMSC_LAUNCHED(1);
    e = scan_exclusive_u32(w->lens, ncp, offs, offs + ncp, st);
  }
  uint32_t tot[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(&tot[0], io.aoff + ncp, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&tot[1], io.doff + ncp, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  io.nasc_out = tot[0];
  io.ndes_out = tot[1];
  return e;
}

cudaError_t simplify_emit(SimplifyIO &io, uint32_t *asc, uint32_t *des, cudaStream_t st) {
  SimplifyWork *w = (SimplifyWork *)io.work;
  const uint32_t ncp = (uint32_t)io.ncp;
  if (!w || !ncp) return cudaSuccess;
  k_csr_from_lists<<<blocks_for(ncp), 256, 0, st>>>(ncp, w->a.L.off, w->a.L.nrun, w->a.L.pool, 0, io.aoff, asc);
  DMSC_LAUNCHED(1);
  k_csr_from_lists<<<blocks_for(ncp), 256, 0, st>>>(ncp, w->a.L.off, w->a.L.nrun, w->a.L.pool, 1, io.doff, des);
  DMSC_LAUNCHED(1);
  cudaError_t e = cudaMemcpyAsync(w->flags_in, w->a.flags, ncp, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(w->pair_in, w->a.pair_idx, 4ull * ncp, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaGetLastError();
  return e;
}

void simplify_release(SimplifyIO &io, cudaStream_t st) {
  SimplifyWork *w = (SimplifyWork *)io.work;
  if (!w) return;
  if (w->buf) cudaFreeAsync(w->buf, st);
  delete w;
  io.work = nullptr;
}

}  // namespace dmsc
