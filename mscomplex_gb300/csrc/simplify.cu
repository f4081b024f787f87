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
#include "msc_graph.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

namespace dmsc {

// A heap entry: persistence and the pair (a, b).  The top three bits of a
// and of b carry that critical point's static facts (on rect's boundary, cell
// dimension), so that a popped pair is classified from the entry itself and
// a resubmitted pair goes back on the heap without a load.  Critical point
// indices are below 2^29.
struct HeapEnt {
  float d;
  uint32_t a, b;
};
constexpr uint32_t IDX_MASK = (1u << 29) - 1u, META_BOUNDARY = 1u << 31;
__host__ __device__ __forceinline__ uint32_t ent_idx(uint32_t x) { return x & IDX_MASK; }
__host__ __device__ __forceinline__ int ent_dim(uint32_t x) { return (int)((x >> 29) & 3u); }
__host__ __device__ __forceinline__ bool ent_boundary(uint32_t x) { return (x & META_BOUNDARY) != 0; }

// IEEE single subtraction without contraction on either side of the compiler.
__host__ __device__ __forceinline__ float fsub_rn(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  volatile float r = a - b;
  return r;
#endif
}

__host__ __device__ __forceinline__ float bits_float(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}
__host__ __device__ __forceinline__ uint32_t float_bits(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}
// The loop stops at the first pair with (double)d / (double)max_persistence >
// tresh (grid_mscomplex.cpp:446-447).  A correctly rounded division by a
// fixed divisor is monotone in d, so over the persistences (non-negative,
// finite floats, whose bit patterns order like their values) the test is
// true exactly from one bit pattern on.  That pattern is found once here, by
// bisection with the same double-precision test, and each pop compares bits:
// the same outcome for every d, without a double division per pop (double
// precision is slow on this part).  Returns 0x7F800001 if no finite d passes.
__host__ __device__ inline uint32_t stop_bits(float max_persistence, double tresh) {
  auto over = [&](uint32_t u) { return (double)bits_float(u) / (double)max_persistence > tresh; };
  uint32_t lo = 0, hi = 0x7F800001u;  // the first passing pattern lies in [lo, hi]
  while (lo < hi) {
    const uint32_t mid = lo + (hi - lo) / 2;
    if (over(mid)) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

struct SimpArgs {
  Graph G;            // the complex as a mutable graph (msc_graph.cuh)
  const float *fn;
  uint32_t *meta;     // per critical point: its index with the entry bits (k_simp_prep)
  HeapEnt *heap;
  unsigned long long heap_cap;
  HeapEnt *resub;     // resubmit list (capacity heap_cap), whole entries
  uint2 *canc;        // cancellation list (capacity ncp)
  int rx0, ry0, rx1, ry1;  // m_rect of the complex (cell coordinates)
  double tresh;
  unsigned long long *stats;  // [0] pushes [1] pops [2] cancels [3] ops [4] status
  // the complex's CSR lists (offsets may be based anywhere) and the entries of
  // its first pushes, one per des arc in that order (k_simp_prep)
  const uint32_t *aoff, *asc, *doff, *des;
  HeapEnt *init;
  unsigned long long ninit;
};

// The top HEAP_TOP entries of the heap (its first 14 levels, which every pop
// walks) live in shared memory; the rest in global memory.  Same layout and
// the same operations, only the storage of those indices differs.
constexpr unsigned long long HEAP_TOP = (1u << 14) - 1;
constexpr size_t HEAP_TOP_BYTES = sizeof(HeapEnt) * HEAP_TOP;

struct Simp {
  SimpArgs A;
  unsigned long long nheap = 0, nres = 0, ncanc = 0;
  unsigned long long n_push = 0, n_pop = 0;  // heap operations (stats[0], stats[1] at the end)
  HeapEnt *top = nullptr;         // shared-memory part of the heap (null: all in global memory)
  unsigned long long ntop = 0;    // indices below ntop are in `top`

  __host__ __device__ __forceinline__ HeapEnt &H(unsigned long long i) { return i < ntop ? top[i] : A.heap[i]; }
  // L1 prefetch of the global part of heap[lo..hi], one request per 128-byte line
  __host__ __device__ __forceinline__ void prefetch_heap(unsigned long long lo, unsigned long long hi) {
#ifdef __CUDA_ARCH__
    if (lo < ntop) lo = ntop;
    if (hi >= A.heap_cap) hi = A.heap_cap - 1;
    if (lo > hi) return;
    const char *p = reinterpret_cast<const char *>(A.heap + lo), *e = reinterpret_cast<const char *>(A.heap + hi + 1);
    for (p = reinterpret_cast<const char *>(reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)127); p < e; p += 128)
      asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
#else
    (void)lo; (void)hi;
#endif
  }
  // before a burst of m pushes at the end: the lines of the three ancestor
  // levels above the positions they take, and of the entries themselves
  __host__ __device__ __forceinline__ void prefetch_pushes(const HeapEnt *src, unsigned long long m) {
#ifdef __CUDA_ARCH__
    if (m == 0) return;
    const unsigned long long n0 = nheap, n1 = nheap + m;
    for (int k = 1; k <= 3; ++k) prefetch_heap(((n0 + 1) >> k) - 1, ((n1 + 1) >> k) - 1);
    const char *p = reinterpret_cast<const char *>(src), *e = reinterpret_cast<const char *>(src + m);
    for (p = reinterpret_cast<const char *>(reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)127); p < e; p += 128)
      asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
#else
    (void)src; (void)m;
#endif
  }

  // ---- heap (binary heap of the standard library, comparator d1 > d2) ----
  __host__ __device__ __forceinline__ static bool comp(const HeapEnt &x, const HeapEnt &y) { return x.d > y.d; }
  // __push_heap from position hole up to the root: the hole climbs while its
  // parent is larger (comparator d1 > d2) -- in global memory while the hole
  // is there, then in shared memory with 32-bit indices
  __host__ __device__ void push_at(unsigned long long hole, HeapEnt val) {
    while (hole >= ntop && hole > 0) {
      const unsigned long long parent = (hole - 1) / 2;
      const HeapEnt pe = H(parent);
      if (!comp(pe, val)) { H(hole) = val; return; }
      H(hole) = pe;
      hole = parent;
    }
    if (hole >= ntop) { H(hole) = val; return; }  // the root itself is in global memory (no shared part)
    uint32_t h = (uint32_t)hole;
    while (h > 0) {
      const uint32_t parent = (h - 1) >> 1;
      if (!(top[parent].d > val.d)) break;
      top[h] = top[parent];
      h = parent;
    }
    top[h] = val;
  }
  __host__ __device__ void push_ent(const HeapEnt &x) {
    if (nheap >= A.heap_cap) { A.G.fail = true; return; }
    push_at(nheap, x);
    ++nheap;
    ++n_push;
  }
  // a new pair: its two values and its two entry words from independent loads
  __host__ __device__ void push(uint32_t a, uint32_t b) {
    const float fa = A.fn[a], fb = A.fn[b];
    const uint32_t ma = A.meta[a], mb = A.meta[b];
    push_ent(HeapEnt{fabsf(fsub_rn(fb, fa)), ma, mb});
  }
  // pop_heap + pop_back: libstdc++'s __adjust_heap moves the hole from the
  // root to a leaf along the smaller children (the right one unless the left
  // is strictly smaller), then sifts the last element up from that leaf.  The
  // sift-up restores every path entry below the place where the last element
  // lands, so stopping the descent there -- at the first chosen child larger
  // than the last element -- leaves the same heap with fewer steps.
  //
  // The path does not depend on the last element, so the shared-memory part
  // is chosen first from the keys alone (while the last element, often in
  // global memory, is still on its way), then shifted up to the stop; in
  // global memory both children and all four grandchildren of the hole are
  // loaded together, two levels per round trip.
  __host__ __device__ HeapEnt pop() {
    ++n_pop;
    HeapEnt first = H(0);
    const unsigned long long len = nheap - 1;
    --nheap;
    if (len == 0) return first;
    const HeapEnt val = H(len);
    // the next pops' last elements are the entries below this one: keep
    // their lines on their way into L1
    if (len >= ntop + 16) prefetch_heap(len - 16, len - 16);
    unsigned long long hole = 0;
    // shared-memory levels: the path while both children are in `top`, two
    // levels per step (children and grandchildren keys loaded together),
    // kept in registers (fixed-size arrays indexed by unrolled constants)
    constexpr int PMAX = 14;  // HEAP_TOP holds 14 levels
    uint32_t path[PMAX];
    float pkey[PMAX];
    int np = 0;
    {
      // 32-bit indices: every index here is below ntop (at most HEAP_TOP); len
      // is clamped, which keeps each comparison with it exact
      const uint32_t nt = (uint32_t)ntop, ln = len > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)len;
      uint32_t h = 0;
#pragma unroll
      for (int q = 0; q < PMAX; q += 2) {
        const uint32_t l = 2 * h + 1;
        if (l >= ln || l + 1 >= nt) break;
        const uint32_t ll = 2 * l + 1, rl = ll + 2;  // first child of l and of l + 1
        const bool g_ok = rl + 1 < nt;              // all four grandchildren in `top`
        const float dl = top[l].d, dr = l + 1 < ln ? top[l + 1].d : 0.0f;
        float g0 = 0, g1 = 0, g2 = 0, g3 = 0;
        if (g_ok) { g0 = top[ll].d; g1 = top[ll + 1].d; g2 = top[rl].d; g3 = top[rl + 1].d; }
        const bool right = l + 1 < ln && !(dr > dl);
        const uint32_t c = right ? l + 1 : l;
        path[q] = c;
        pkey[q] = right ? dr : dl;
        np = q + 1;
        h = c;
        if (q + 1 >= PMAX || !g_ok) break;
        const uint32_t l2 = 2 * c + 1;
        if (l2 >= ln) break;
        const float el = right ? g2 : g0, er = right ? g3 : g1;
        const bool right2 = l2 + 1 < ln && !(er > el);
        const uint32_t c2 = right2 ? l2 + 1 : l2;
        path[q + 1] = c2;
        pkey[q + 1] = right2 ? er : el;
        np = q + 2;
        h = c2;
      }
    }
    int stop = np;
#pragma unroll
    for (int i = PMAX - 1; i >= 0; --i)
      if (i < np && pkey[i] > val.d) stop = i;
    {
      // the path's entries first (independent loads), then each one level up
      HeapEnt mv[PMAX];
#pragma unroll
      for (int i = 0; i < PMAX; ++i)
        if (i < stop) mv[i] = top[path[i]];
      uint32_t hs = 0;  // the hole while it is in shared memory (32-bit)
#pragma unroll
      for (int i = 0; i < PMAX; ++i) {
        if (i >= stop) break;
        top[hs] = mv[i];
        hs = path[i];
      }
      hole = hs;
    }
    if (stop < np) {  // the last element lands in shared memory
      top[hole] = val;
      return first;
    }
    // global levels (and the step from the last shared-memory node), two at a time
    for (;;) {
      const unsigned long long l = 2 * hole + 1;
      if (l >= len) break;
      const bool has_r = l + 1 < len;
      const unsigned long long ll = 2 * l + 1, rl = 2 * (l + 1) + 1;
      const HeapEnt L = H(l), R = has_r ? H(l + 1) : L;
      HeapEnt g[4];
      g[0] = ll < len ? H(ll) : L;
      g[1] = ll + 1 < len ? H(ll + 1) : L;
      g[2] = rl < len ? H(rl) : L;
      g[3] = rl + 1 < len ? H(rl + 1) : L;
      const bool right = has_r && !(R.d > L.d);
      const unsigned long long c = right ? l + 1 : l;
      const HeapEnt hc = right ? R : L;
      if (hc.d > val.d) break;
      H(hole) = hc;
      hole = c;
      // the next level from the loaded grandchildren
      const unsigned long long l2 = 2 * c + 1;
      if (l2 >= len) break;
      const HeapEnt L2 = right ? g[2] : g[0], R2 = right ? g[3] : g[1];
      const bool right2 = l2 + 1 < len && !(R2.d > L2.d);
      const HeapEnt hc2 = right2 ? R2 : L2;
      if (hc2.d > val.d) break;
      H(hole) = hc2;
      hole = right2 ? l2 + 1 : l2;
    }
    H(hole) = val;
    return first;
  }

  // simplify (grid_mscomplex.cpp:384-512) followed by un_simplify (:514-526)
  __host__ __device__ void run() {
    Graph &G = A.G;
    const uint32_t n = G.ncp;
    // (:396-428) the strangulation marks and the entries of the first pushes
    // come from k_simp_prep; the value range and the pushes, in the
    // reference's order, here
    float max_val = 1.17549435e-38f;  // std::numeric_limits<float>::min(), as in the reference (:399)
    float min_val = 3.40282347e+38f;
    for (uint32_t i = 0; i < n; ++i) {
      const float f = A.fn[i];
      max_val = (max_val < f) ? f : max_val;  // std::max
      min_val = (f < min_val) ? f : min_val;  // std::min
    }
    for (unsigned long long q = 0; q < A.ninit && !G.fail; ++q) push_ent(A.init[q]);
    const float max_persistence = fsub_rn(max_val, min_val);
    const uint32_t stop_at = stop_bits(max_persistence, A.tresh);
    while (nheap != 0 && !G.fail) {
      if (!G.tick()) break;
      // the entry on top and its pair's dynamic state (three independent
      // loads), issued before the pop's descent so that they arrive during it
      const HeapEnt top0 = H(0);
      uint32_t w1 = top0.a, w2 = top0.b;
      if (ent_dim(w2) == 1) { uint32_t t = w1; w1 = w2; w2 = t; }
      const uint32_t v1 = ent_idx(w1), v2 = ent_idx(w2);
      const bool inside = v1 < n && v2 < n;
      const int cp2_dim = ent_dim(w2);
      const uint8_t f1 = inside ? G.flags[v1] : 0, f2 = inside ? G.flags[v2] : 0;
      const uint32_t tot2 = inside ? G.L.total[2 * v2 + cp2_dim / 2] : 0;
      HeapEnt e = pop();
      if (float_bits(e.d) >= stop_at) break;  // (double)e.d / max_persistence > tresh
      if (!inside) { A.stats[4] |= ST_INVARIANT; continue; }  // a list entry outside the complex
      if ((f1 & F_CANCELLED) || (f2 & F_CANCELLED)) continue;
      const bool b1 = ent_boundary(w1), b2 = ent_boundary(w2);
      if (b1 && !b2) continue;
      if (!b1 && b2) continue;
      const bool strang = f1 & F_STRANG;
      if (strang && tot2 != 1) {
        if (nres >= A.heap_cap) { G.fail = true; break; }
        A.resub[nres++] = e;
        continue;
      }
      if (strang && b1) continue;
      uint32_t cp0 = v1, cp1 = v2;
      bool connected = G.cancel_pairs(cp0, cp1);
      if (G.fail) break;
      G.flags[v1] |= F_BCANCEL;
      G.flags[v2] |= F_BCANCEL;
      G.pair_idx[v1] = v2;
      G.pair_idx[v2] = v1;
      if (ncanc >= n) { G.fail = true; break; }
      A.canc[ncanc++] = make_uint2(ent_idx(e.a), ent_idx(e.b));
      if (connected) {  // new edges (d, a) in the reference's order
        const uint32_t la0 = 2 * cp0, ld1 = 2 * cp1 + 1;
        for (uint32_t i = 0; i < G.L.nrun[la0] && !G.fail; ++i) {
          uint2 ra = G.runs(la0)[i];
          if (ra.x == cp1) continue;
          for (uint32_t ca = 0; ca < ra.y && !G.fail; ++ca)
            for (uint32_t j = 0; j < G.L.nrun[ld1] && !G.fail; ++j) {
              uint2 rd = G.runs(ld1)[j];
              if (rd.x == cp0) continue;
              for (uint32_t cd = 0; cd < rd.y && !G.fail; ++cd) push(rd.x, ra.x);
            }
        }
      }
      prefetch_pushes(A.resub, nres);
      for (unsigned long long i = 0; i < nres && !G.fail; ++i) push_ent(A.resub[i]);
      nres = 0;
    }
    A.stats[0] = n_push;
    A.stats[1] = n_pop;
    A.stats[2] = ncanc;
    if (G.fail) return;
    for (unsigned long long k = ncanc; k-- > 0;) {
      uint2 c = A.canc[k];
      if (!G.uncancel_pairs(c.x, c.y)) { A.stats[4] |= ST_INVARIANT; return; }
      if (G.fail) return;
    }
  }
};

// In parallel, per critical point of args[blockIdx.y]: the strangulation
// mark of a saddle whose asc or des multiset holds one point twice (:404-417),
// and the heap entries of its des arcs, at their places in the push order.
// the entry word of critical point k: its index, dimension and boundary bit
__device__ __forceinline__ uint32_t meta_of(const SimpArgs &A, uint32_t k) {
  const uint32_t c = A.G.cellid[k];
  const int x = (int16_t)(c & 0xffff), y = (int16_t)(c >> 16);
  const bool contains = x >= A.rx0 && y >= A.ry0 && x <= A.rx1 && y <= A.ry1;
  const bool interior = x > A.rx0 && y > A.ry0 && x < A.rx1 && y < A.ry1;
  const uint32_t dim = (c & 1u) + ((c >> 16) & 1u);
  return k | (dim << 29) | (contains && !interior ? META_BOUNDARY : 0u);
}
__global__ void k_simp_meta(SimpArgs *args) {
  SimpArgs &A = args[blockIdx.y];
  const uint32_t n = A.G.ncp;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) A.meta[i] = meta_of(A, i);
}
__global__ void k_simp_prep(SimpArgs *args) {
  SimpArgs &A = args[blockIdx.y];
  const uint32_t n = A.G.ncp, base = A.doff[0];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (A.G.dim(i) == 1) {
      if ((A.aoff[i + 1] - A.aoff[i] == 2 && A.asc[A.aoff[i]] == A.asc[A.aoff[i] + 1]) ||
          (A.doff[i + 1] - A.doff[i] == 2 && A.des[A.doff[i]] == A.des[A.doff[i] + 1]))
        A.G.flags[i] |= F_STRANG;
    }
    const uint32_t mi = A.meta[i];
    for (uint32_t q = A.doff[i]; q < A.doff[i + 1]; ++q) {
      const uint32_t b = A.des[q];
      A.init[q - base] = b < n ? HeapEnt{fabsf(fsub_rn(A.fn[b], A.fn[i])), mi, A.meta[b]} : HeapEnt{0.0f, mi, b};
    }
  }
}

__global__ void k_simplify(SimpArgs a) {
  extern __shared__ HeapEnt heap_top[];
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  Simp s;
  s.A = a;
  s.top = heap_top;
  s.ntop = HEAP_TOP;
  s.run();
  a.stats[3] = s.A.G.ops;
  if (s.A.G.fail) a.stats[4] |= ST_SIMPLIFY_LIMIT;
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

// run-length lists -> expanded CSR (offsets from a scan of the totals; a
// list never writes past the next list's offset)
__global__ void k_csr_from_lists(uint32_t ncp, const uint32_t *off, const uint32_t *nrun, const uint2 *pool, int which,
                                 const uint32_t *outoff, uint32_t *out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ncp; i += gridDim.x * blockDim.x) {
    uint32_t l = 2 * i + which, o = outoff[i];
    const uint32_t end = outoff[i + 1];
    const uint2 *p = pool + off[l];
    for (uint32_t k = 0; k < nrun[l]; ++k)
      for (uint32_t c = 0; c < p[k].y && o < end; ++c) out[o++] = p[k].x;
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
  if (ncp > IDX_MASK) return cudaErrorInvalidValue;               // heap entries hold 29-bit indices
  auto rnd = [](size_t n) { return (n + 255) / 256 * 256; };
  size_t sizes[] = {sizeof(uint32_t) * 2 * ncp, sizeof(uint32_t) * 2 * ncp, sizeof(uint32_t) * 2 * ncp,
                    sizeof(uint32_t) * 2 * ncp, sizeof(uint2) * pool_cap, sizeof(uint2) * tmp_cap, sizeof(HeapEnt) * heap_cap,
                    sizeof(HeapEnt) * heap_cap, sizeof(uint2) * (ncp + 1), sizeof(unsigned long long) * 8,
                    sizeof(uint8_t) * (ncp + 1), sizeof(uint32_t) * (ncp + 1), sizeof(uint32_t) * (ncp + 1),
                    sizeof(HeapEnt) * ((size_t)io.ndes + 1), sizeof(SimpArgs), sizeof(uint32_t) * (ncp + 1)};
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
  Graph &G = a.G;
  G.ncp = ncp;
  G.cellid = const_cast<uint32_t *>(io.cellid);
  a.fn = io.fn;
  G.L.off = (uint32_t *)take();
  G.L.nrun = (uint32_t *)take();
  G.L.cap = (uint32_t *)take();
  G.L.total = (uint32_t *)take();
  G.L.pool = (uint2 *)take();
  G.L.top = base_top;
  G.L.pool_cap = pool_cap;
  G.tmp = (uint2 *)take();
  G.tmp_cap = tmp_cap;
  a.heap = (HeapEnt *)take();
  a.heap_cap = heap_cap;
  a.resub = (HeapEnt *)take();
  a.canc = (uint2 *)take();
  a.stats = (unsigned long long *)take();
  G.flags = (uint8_t *)take();
  G.pair_idx = (uint32_t *)take();
  w->lens = (uint32_t *)take();
  a.init = (HeapEnt *)take();
  a.ninit = (unsigned long long)io.ndes;
  a.aoff = io.aoff; a.asc = io.asc; a.doff = io.doff; a.des = io.des;
  SimpArgs *dargs = (SimpArgs *)take();
  a.meta = (uint32_t *)take();
  w->flags_in = io.flags;
  w->pair_in = io.pair_idx;
  a.rx0 = io.rect[0]; a.ry0 = io.rect[1]; a.rx1 = io.rect[2]; a.ry1 = io.rect[3];
  a.tresh = io.tresh;
  G.max_ops = io.max_ops;
  G.ops = 0;
  G.fail = false;
  e = cudaMemsetAsync(a.stats, 0, sizeof(unsigned long long) * 8, st);
  if (e == cudaSuccess && ncp) e = cudaMemcpyAsync(G.flags, io.flags, ncp, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && ncp) e = cudaMemcpyAsync(G.pair_idx, io.pair_idx, 4ull * ncp, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return e;
  if (ncp) {
    k_lists_from_csr<<<blocks_for(ncp), 256, 0, st>>>(ncp, io.aoff, io.asc, io.doff, io.des, des_base, G.L.off,
                                                       G.L.nrun, G.L.cap, G.L.total, G.L.pool);
    DMSC_LAUNCHED(1);
    e = cudaMemcpyAsync(dargs, &a, sizeof(SimpArgs), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    k_simp_meta<<<blocks_for(ncp), 256, 0, st>>>(dargs);
    k_simp_prep<<<blocks_for(ncp), 256, 0, st>>>(dargs);
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_simplify, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)HEAP_TOP_BYTES);
    if (attr != cudaSuccess) return attr;
    k_simplify<<<1, 32, HEAP_TOP_BYTES, st>>>(a);
    DMSC_LAUNCHED(3);
  }
  e = cudaMemcpyAsync(io.host_stats, a.stats, sizeof(unsigned long long) * 5, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess || io.host_stats[4] != 0 || !ncp) return e;
  // new CSR offsets (asc, then des) from the list lengths
  for (int which = 0; which < 2 && e == cudaSuccess; ++which) {
    uint32_t *offs = which ? io.doff : io.aoff;
    k_pick_len<<<blocks_for(ncp), 256, 0, st>>>(ncp, G.L.total, which, w->lens);
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
  k_csr_from_lists<<<blocks_for(ncp), 256, 0, st>>>(ncp, w->a.G.L.off, w->a.G.L.nrun, w->a.G.L.pool, 0, io.aoff, asc);
  DMSC_LAUNCHED(1);
  k_csr_from_lists<<<blocks_for(ncp), 256, 0, st>>>(ncp, w->a.G.L.off, w->a.G.L.nrun, w->a.G.L.pool, 1, io.doff, des);
  DMSC_LAUNCHED(1);
  cudaError_t e = cudaMemcpyAsync(w->flags_in, w->a.G.flags, ncp, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(w->pair_in, w->a.G.pair_idx, 4ull * ncp, cudaMemcpyDeviceToDevice, st);
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

// ---------------------------------------------------------------------------
// batches: one block per complex to simplify, all in one launch
// ---------------------------------------------------------------------------
__global__ void k_simplify_batch(SimpArgs *args, int n, unsigned ntop) {
  extern __shared__ HeapEnt heap_top[];
  if (threadIdx.x != 0 || blockIdx.x >= (unsigned)n) return;
  Simp s;
  s.A = args[blockIdx.x];
  s.top = heap_top;
  s.ntop = ntop;
  s.run();
  s.A.stats[3] = s.A.G.ops;
  if (s.A.G.fail) s.A.stats[4] |= ST_SIMPLIFY_LIMIT;
}

struct BatchSimplifyWork {
  char *buf = nullptr;
  uint32_t *off = nullptr, *nrun = nullptr, *lcap = nullptr, *total = nullptr, *lens = nullptr;
  uint2 *pool = nullptr;
  SimpArgs *dargs = nullptr;
  unsigned long long *dstats = nullptr;
  int nsimp = 0;
};

cudaError_t simplify_batch_run(BatchSimplifyIO &io, cudaStream_t st) {
  const uint32_t ncp = (uint32_t)io.ncp;
  const unsigned long long des_base = (unsigned long long)io.nasc + 4ull * ncp;
  const unsigned long long base_top = des_base + (unsigned long long)io.ndes + 4ull * ncp;
  // per simplified grid: pool growth region, heap, resubmits, cancellations, scratch runs
  std::vector<int> which;
  unsigned long long grow = 0, heap = 0, canc = 0, tmp = 0, init = 0;
  const unsigned long long sc = io.scale ? io.scale : 1;
  auto grow_of = [&](unsigned long long na, unsigned long long nd, unsigned long long n) {
    return sc * (4 * (na + nd + 8 * n) + 16384);
  };
  auto heap_of = [&](unsigned long long nd) { return sc * (8 * nd + 16384); };
  auto tmp_of = [&](unsigned long long na, unsigned long long nd) { return sc * (4 * (na + nd) + 16384); };
  for (int g = 0; g < io.ngrids; ++g) {
    const unsigned long long n = io.cpb[g + 1] - io.cpb[g];
    if (!(io.tresh[g] > 0.0) || n == 0) continue;
    const unsigned long long na = io.abase[g + 1] - io.abase[g], nd = io.dbase[g + 1] - io.dbase[g];
    which.push_back(g);
    grow += grow_of(na, nd, n);
    heap += heap_of(nd);
    canc += n + 1;
    tmp += tmp_of(na, nd);
    init += nd + 1;
  }
  const unsigned long long pool_cap = base_top + grow;
  if (pool_cap > 0xffffffffull) return cudaErrorInvalidValue;  // list offsets are 32-bit
  // Blocks start roughly in index order and more grids than fit at once wait
  // for a free slot, while the batch lasts as long as its longest replay: the
  // complexes with the most arcs (the longest replays, as a rule) take the
  // first blocks.
  std::stable_sort(which.begin(), which.end(), [&](int x, int y) {
    const unsigned long long ax = (io.abase[x + 1] - io.abase[x]) + (io.dbase[x + 1] - io.dbase[x]);
    const unsigned long long ay = (io.abase[y + 1] - io.abase[y]) + (io.dbase[y + 1] - io.dbase[y]);
    return ax > ay;
  });
  const int ns = (int)which.size();
  auto rnd = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t sizes[] = {4ull * 2 * ncp, 4ull * 2 * ncp, 4ull * 2 * ncp, 4ull * 2 * ncp, 4ull * (ncp + 1),
                          sizeof(uint2) * pool_cap, sizeof(uint2) * tmp, sizeof(HeapEnt) * heap, sizeof(HeapEnt) * heap,
                          sizeof(uint2) * canc, sizeof(unsigned long long) * 8 * (size_t)(ns + 1),
                          sizeof(SimpArgs) * (size_t)(ns + 1), sizeof(HeapEnt) * (init + 1), 4ull * (ncp + 1)};
  size_t bytes = 0;
  for (size_t z : sizes) bytes += rnd(z);
  BatchSimplifyWork *w = new BatchSimplifyWork;
  io.work = w;
  cudaError_t e = cudaMallocAsync((void **)&w->buf, bytes, st);
  if (e != cudaSuccess) { w->buf = nullptr; return e; }
  char *p = w->buf;
  int si = 0;
  auto take = [&]() { char *r = p; p += rnd(sizes[si++]); return r; };
  w->off = (uint32_t *)take(); w->nrun = (uint32_t *)take(); w->lcap = (uint32_t *)take(); w->total = (uint32_t *)take();
  w->lens = (uint32_t *)take();
  w->pool = (uint2 *)take();
  uint2 *dtmp = (uint2 *)take();
  HeapEnt *dheap = (HeapEnt *)take();
  HeapEnt *dres = (HeapEnt *)take();
  uint2 *dcanc = (uint2 *)take();
  w->dstats = (unsigned long long *)take();
  w->dargs = (SimpArgs *)take();
  HeapEnt *dinit = (HeapEnt *)take();
  uint32_t *dmeta = (uint32_t *)take();
  w->nsimp = ns;
  if (ncp) {
    k_lists_from_csr<<<blocks_for(ncp), 256, 0, st>>>(ncp, io.aoff, io.asc, io.doff, io.des, des_base, w->off, w->nrun,
                                                       w->lcap, w->total, w->pool);
    DMSC_LAUNCHED(1);
  }
  e = cudaMemsetAsync(w->dstats, 0, sizeof(unsigned long long) * 8 * (size_t)(ns + 1), st);
  std::vector<SimpArgs> args(ns);
  unsigned long long top = base_top, ho = 0, co = 0, to = 0, io2 = 0;
  for (int k = 0; k < ns && e == cudaSuccess; ++k) {
    const int g = which[k];
    const unsigned long long c0 = io.cpb[g], n = io.cpb[g + 1] - c0;
    const unsigned long long na = io.abase[g + 1] - io.abase[g], nd = io.dbase[g + 1] - io.dbase[g];
    SimpArgs &a = args[k];
    Graph &G = a.G;
    G = Graph();
    G.ncp = (uint32_t)n;
    G.cellid = const_cast<uint32_t *>(io.cellid) + c0;
    G.flags = io.flags + c0;
    G.pair_idx = io.pair_idx + c0;
    G.L.off = w->off + 2 * c0; G.L.nrun = w->nrun + 2 * c0; G.L.cap = w->lcap + 2 * c0; G.L.total = w->total + 2 * c0;
    G.L.pool = w->pool;
    G.L.top = top;
    top += grow_of(na, nd, n);
    G.L.pool_cap = top;
    G.tmp = dtmp + to;
    G.tmp_cap = tmp_of(na, nd);
    to += G.tmp_cap;
    G.max_ops = io.max_ops;
    G.ops = 0;
    G.fail = false;
    a.fn = io.fn + c0;
    a.meta = dmeta + c0;
    a.heap = dheap + ho;
    a.resub = dres + ho;
    a.heap_cap = heap_of(nd);
    ho += a.heap_cap;
    a.canc = dcanc + co;
    co += n + 1;
    a.aoff = io.aoff + c0; a.asc = io.asc; a.doff = io.doff + c0; a.des = io.des;
    a.init = dinit + io2;
    a.ninit = nd;
    io2 += nd + 1;
    a.rx0 = io.rect[4 * g]; a.ry0 = io.rect[4 * g + 1]; a.rx1 = io.rect[4 * g + 2]; a.ry1 = io.rect[4 * g + 3];
    a.tresh = io.tresh[g];
    a.stats = w->dstats + 8 * k;
  }
  if (e == cudaSuccess && ns) e = cudaMemcpyAsync(w->dargs, args.data(), sizeof(SimpArgs) * ns, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && ns) {
    static const cudaError_t attr =
        cudaFuncSetAttribute(k_simplify_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)HEAP_TOP_BYTES);
    if (attr != cudaSuccess) return attr;
    // one grid per SM can keep 14 heap levels in shared memory; more grids
    // than SMs keep 13, two per SM (measured on the 1000-grid workload: 13
    // levels 108.8 ms, 12 levels (four per SM) 113.8, 14 levels 122.4)
    const unsigned ntop = ns <= 152 ? (unsigned)HEAP_TOP : (1u << 13) - 1;
    k_simp_meta<<<dim3(64, (unsigned)ns), 256, 0, st>>>(w->dargs);
    k_simp_prep<<<dim3(64, (unsigned)ns), 256, 0, st>>>(w->dargs);
    k_simplify_batch<<<ns, 32, sizeof(HeapEnt) * ntop, st>>>(w->dargs, ns, ntop);
    DMSC_LAUNCHED(3);
    e = cudaGetLastError();
  }
  std::vector<unsigned long long> hs(8 * (size_t)(ns + 1), 0);
  if (e == cudaSuccess && ns) e = cudaMemcpyAsync(hs.data(), w->dstats, sizeof(unsigned long long) * 8 * ns, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  for (int g = 0; g < io.ngrids; ++g)
    for (int q = 0; q < 5; ++q) io.host_stats[5 * g + q] = 0;
  for (int k = 0; k < ns; ++k)
    for (int q = 0; q < 5; ++q) io.host_stats[5 * which[k] + q] = hs[8 * k + q];
  return cudaSuccess;  // the caller reads the per-grid status
}

// List offsets of the simplified batch; the grids in `dead` (whose
// simplification failed) keep their critical points but get empty lists.
cudaError_t simplify_batch_offsets(BatchSimplifyIO &io, const std::vector<int> &dead, cudaStream_t st) {
  BatchSimplifyWork *w = (BatchSimplifyWork *)io.work;
  const uint32_t ncp = (uint32_t)io.ncp;
  io.nasc_out = io.ndes_out = 0;
  if (!w || !ncp) return cudaSuccess;
  cudaError_t e = cudaSuccess;
  for (int g : dead) {  // no runs and no total: the emit writes nothing for them
    const unsigned long long c0 = io.cpb[g], n = io.cpb[g + 1] - c0;
    if (n && e == cudaSuccess) e = cudaMemsetAsync(w->total + 2 * c0, 0, 8ull * n, st);
    if (n && e == cudaSuccess) e = cudaMemsetAsync(w->nrun + 2 * c0, 0, 8ull * n, st);
  }
  for (int wch = 0; wch < 2 && e == cudaSuccess; ++wch) {
    uint32_t *offs = wch ? io.doff : io.aoff;
    k_pick_len<<<blocks_for(ncp), 256, 0, st>>>(ncp, w->total, wch, w->lens);
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

cudaError_t simplify_batch_emit(BatchSimplifyIO &io, uint32_t *asc, uint32_t *des, cudaStream_t st) {
  BatchSimplifyWork *w = (BatchSimplifyWork *)io.work;
  const uint32_t ncp = (uint32_t)io.ncp;
  if (!w || !ncp) return cudaSuccess;
  k_csr_from_lists<<<blocks_for(ncp), 256, 0, st>>>(ncp, w->off, w->nrun, w->pool, 0, io.aoff, asc);
  k_csr_from_lists<<<blocks_for(ncp), 256, 0, st>>>(ncp, w->off, w->nrun, w->pool, 1, io.doff, des);
  DMSC_LAUNCHED(2);
  return cudaGetLastError();
}

void simplify_batch_release(BatchSimplifyIO &io, cudaStream_t st) {
  BatchSimplifyWork *w = (BatchSimplifyWork *)io.work;
  if (!w) return;
  if (w->buf) cudaFreeAsync(w->buf, st);
  delete w;
  io.work = nullptr;
}

}  // namespace dmsc
