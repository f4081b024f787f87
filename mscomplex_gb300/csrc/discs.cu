// discs.cu -- manifold ("disc") collection on the device:
// GridDataset::postMergeFillDiscs (dmsc/src/grid_dataset.cpp:1044-1231).
//
// The reference walks the complex's critical points in index order:
//   * a cancelled saddle redirects the owner of itself and of its paired
//     extremum to the one surviving extremum it is connected to (:1062-1083);
//   * a cancelled maximum (minimum) appends its paired saddle to the asc (des)
//     disc of every saddle in its des (asc) multiset (:1084-1103);
//   * a surviving saddle seeds its discs with the pairs of its incident
//     non-critical cells (:1112-1133);
// then appends every rect vertex (face) to the asc (des) disc of its owner
// after one level of redirection (:1142-1187), and finally grows each
// surviving saddle's discs breadth-first along the gradient (:1190-1228).
// The device does the same in four passes: redirection per critical point,
// a stable sort of the vertices and faces by owner (row-major order is the
// append order), a stable sort of the cancelled-extremum seeds by saddle, and
// one thread per surviving saddle that first counts and then writes its
// breadth-first discs, using the output array as the queue.
#include "dmsc_common.cuh"
#include "dmsc_internal.h"
#include "grid_types.h"
#include <algorithm>

namespace dmsc {

constexpr uint8_t F_BCANCEL = 4;

struct DiscArgs {
  GridGeom g;                 // dataset geometry (rect relative to ext)
  const uint32_t *codes;      // dataset gradient codes
  const uint4 *labels;        // dataset owner labels (cp indices of the dataset)
  uint32_t ncp_ds;            // dataset critical points (label index space)
  uint32_t ncp;               // complex critical points
  const uint32_t *cellid;     // complex cp cell ids (packed x | y << 16, global)
  const uint8_t *flags;
  const uint32_t *pair_idx;
  const uint32_t *aoff, *asc, *doff, *des;
  uint32_t *status;
};

__device__ __forceinline__ int cdim(uint32_t c) { return (int)(c & 1u) + (int)((c >> 16) & 1u); }
__device__ __forceinline__ int cx(uint32_t c) { return (int16_t)(c & 0xffff); }
__device__ __forceinline__ int cy(uint32_t c) { return (int16_t)(c >> 16); }
// rect containment of a global cell
__device__ __forceinline__ bool rect_has(const GridGeom &g, int x, int y) {
  int rx = x - g.ex0, ry = y - g.ey0;
  return rx >= g.rx0 && rx <= g.rx1 && ry >= g.ry0 && ry <= g.ry1;
}
__device__ __forceinline__ bool ext_has(const GridGeom &g, int x, int y) {
  int rx = x - g.ex0, ry = y - g.ey0;
  return rx >= 0 && rx <= g.cx && ry >= 0 && ry <= g.cy;
}
// gradient code of a global cell inside ext
__device__ __forceinline__ uint32_t code_at(const DiscArgs &a, int x, int y) {
  int rx = x - a.g.ex0, ry = y - a.g.ey0;
  uint32_t q = a.codes[(long long)(ry >> 1) * a.g.vnx + (rx >> 1)];
  return (q >> (8 * ((rx & 1) | ((ry & 1) << 1)))) & 0xff;
}
__device__ __forceinline__ uint32_t pair_of(uint32_t code, int x, int y) {
  uint32_t d = code & 3;
  int px = x + (d == DIR_PX ? 1 : d == DIR_MX ? -1 : 0), py = y + (d == DIR_PY ? 1 : d == DIR_MY ? -1 : 0);
  return pack_cellid(px, py);
}

// 1a. redir[k] = k
__global__ void k_redir_init(uint32_t n, uint32_t *redir) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) redir[k] = k;
}
// 1b. cancelled saddles redirect themselves and their extremum (:1062-1083)
__global__ void k_redir_saddles(DiscArgs a, uint32_t *redir) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.ncp; i += gridDim.x * blockDim.x) {
    if (!(a.flags[i] & F_BCANCEL) || cdim(a.cellid[i]) != 1) continue;
    uint32_t p = a.pair_idx[i];
    if (p >= a.ncp) { atomicOr(a.status, ST_INVARIANT); continue; }
    bool to_min = cdim(a.cellid[p]) == 0;
    const uint32_t *off = to_min ? a.doff : a.aoff, *lst = to_min ? a.des : a.asc;
    if (off[i + 1] - off[i] != 1) { atomicOr(a.status, ST_INVARIANT); continue; }  // "connected to exactly one surv extrema"
    if (a.pair_idx[p] != i) { atomicOr(a.status, ST_INVARIANT); continue; }      // "My pair does not know ..."
    uint32_t ext = lst[off[i]];
    if (rect_has(a.g, cx(a.cellid[i]), cy(a.cellid[i]))) redir[i] = ext;
    if (rect_has(a.g, cx(a.cellid[p]), cy(a.cellid[p]))) redir[p] = ext;
  }
}

// 2. owner keys of the rect vertices (kind 0) or faces (kind 1), row-major
__global__ void k_disc_keys(DiscArgs a, const uint32_t *redir, int kind, uint32_t *key, uint32_t *val) {
  const GridGeom &g = a.g;
  int x0 = g.rx0 + kind, y0 = g.ry0 + kind;
  int nx = (g.rx1 - g.rx0) / 2 + 1 - kind, ny = (g.ry1 - g.ry0) / 2 + 1 - kind;
  long long n = (long long)nx * ny;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    int jj = (int)(t / nx), ii = (int)(t - (long long)jj * nx);
    int rx = x0 + 2 * ii, ry = y0 + 2 * jj;
    uint4 L = a.labels[(long long)(ry >> 1) * g.vnx + (rx >> 1)];
    uint32_t m = kind ? L.w : L.x, o = LABEL_NONE;
    if (m != LABEL_NONE) {
      if (m >= a.ncp_ds || m >= a.ncp) { atomicOr(a.status, ST_INVARIANT); m = LABEL_NONE; }
      else {
        uint32_t mc = a.cellid[m];
        o = rect_has(g, cx(mc), cy(mc)) ? redir[m] : m;
        // the owner must be a surviving extremum of the right dimension
        if (o >= a.ncp || (a.flags[o] & F_BCANCEL) || cdim(a.cellid[o]) != 2 * kind) {
          atomicOr(a.status, ST_INVARIANT);
          o = LABEL_NONE;
        }
      }
    }
    key[t] = o == LABEL_NONE ? a.ncp : o;
    val[t] = pack_cellid(g.ex0 + rx, g.ey0 + ry);
  }
}

// 3. seeds from cancelled extrema: counts, then (saddle, pusher) items in pusher order
__global__ void k_seed_count(DiscArgs a, int kind, uint32_t *cnt) {
  // kind 0: cancelled maxima -> asc discs (via des); kind 1: cancelled minima -> des discs (via asc)
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.ncp; i += gridDim.x * blockDim.x) {
    uint32_t c = 0;
    if ((a.flags[i] & F_BCANCEL) && cdim(a.cellid[i]) == (kind ? 0 : 2)) {
      uint32_t p = a.pair_idx[i];
      if (p < a.ncp && rect_has(a.g, cx(a.cellid[p]), cy(a.cellid[p])))
        c = kind ? a.aoff[i + 1] - a.aoff[i] : a.doff[i + 1] - a.doff[i];
    }
    cnt[i] = c;
  }
}
__global__ void k_seed_write(DiscArgs a, int kind, const uint32_t *off, uint32_t *key, uint32_t *val) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.ncp; i += gridDim.x * blockDim.x) {
    uint32_t o = off[i], e = off[i + 1];
    if (o == e) continue;
    const uint32_t *lst = kind ? a.asc + a.aoff[i] : a.des + a.doff[i];
    for (uint32_t k = 0; k < e - o; ++k) { key[o + k] = lst[k]; val[o + k] = i; }
  }
}

// 4. surviving saddles: own seeds, then breadth-first growth
struct SeedRuns {
  const uint32_t *val;     // sorted pushers
  const uint32_t *start;   // first sorted position of each saddle (valid when count > 0)
  const uint32_t *count;   // items per saddle
};

// Successors of one path cell (kind 0: asc, via cofacets; kind 1: des, via
// facets): up to 2, in the reference's order (:1204-1222).
__device__ __forceinline__ int next_cells(const DiscArgs &a, int kind, uint32_t pc, uint32_t out[2]) {
  int x = cx(pc), y = cy(pc), d0 = x & 1, d1 = y & 1, n = 0;
  int c[2][2];
  if (kind == 0) {  // getCellCofacets of an edge: (x+d1, y+d0), (x-d1, y-d0), filtered to ext
    c[0][0] = x + d1; c[0][1] = y + d0; c[1][0] = x - d1; c[1][1] = y - d0;
  } else {          // getCellFacets of an edge: (x+d0, y+d1), (x-d0, y-d1)
    c[0][0] = x + d0; c[0][1] = y + d1; c[1][0] = x - d0; c[1][1] = y - d1;
  }
  if (cdim(pc) != 1) return 0;
  for (int k = 0; k < 2; ++k) {
    int qx = c[k][0], qy = c[k][1];
    if (!ext_has(a.g, qx, qy)) continue;
    uint32_t qc = code_at(a, qx, qy);
    if (qc & CODE_CRIT) continue;
    if (!rect_has(a.g, qx, qy)) continue;
    uint32_t p = (qc & CODE_PAIRED) ? pair_of(qc, qx, qy) : pack_cellid(-1, -1);
    if (p == pc) continue;
    out[n++] = p;
  }
  return n;
}

// the saddle's own seeds (:1114-1130) for one disc kind, in the reference order
__device__ __forceinline__ int own_seeds(const DiscArgs &a, int kind, uint32_t sc, uint32_t out[4]) {
  int x = cx(sc), y = cy(sc), n = 0;
  const int inc[4][2] = {{x, y + 1}, {x, y - 1}, {x - 1, y}, {x + 1, y}};
  for (int k = 0; k < 4; ++k) {
    int qx = inc[k][0], qy = inc[k][1];
    if (!rect_has(a.g, qx, qy)) continue;
    uint32_t qc = code_at(a, qx, qy);
    if (!(qc & CODE_PAIRED) || (qc & CODE_CRIT)) continue;
    int qdim = (qx & 1) + (qy & 1);
    if ((qdim == 0) != (kind == 1)) continue;  // vertices feed des discs, faces asc discs
    out[n++] = pair_of(qc, qx, qy);
  }
  return n;
}

// Initial disc vector of saddle s: pushes from cancelled extrema with index
// < s, then its own seeds, then pushes with index > s.  Calls f(cell).
template <class F>
__device__ __forceinline__ void for_seeds(const DiscArgs &a, int kind, uint32_t s, const SeedRuns &sr, F f) {
  uint32_t cnt = sr.count[s], st = sr.start[s];
  uint32_t k = 0;
  for (; k < cnt && sr.val[st + k] < s; ++k) f(a.cellid[a.pair_idx[sr.val[st + k]]]);
  uint32_t own[4];
  int n = own_seeds(a, kind, a.cellid[s], own);
  for (int q = 0; q < n; ++q) f(own[q]);
  for (; k < cnt; ++k) f(a.cellid[a.pair_idx[sr.val[st + k]]]);
}

// pass 1: disc lengths.  Every non-critical path cell has at most one
// successor, so each seed expands into at most two chains.
__global__ void k_saddle_disc_count(DiscArgs a, int kind, SeedRuns sr, uint32_t *len, unsigned long long limit) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < a.ncp; s += gridDim.x * blockDim.x) {
    if ((a.flags[s] & F_BCANCEL) || cdim(a.cellid[s]) != 1) { len[s] = 0; continue; }
    unsigned long long total = 0;
    bool bad = false;
    for_seeds(a, kind, s, sr, [&](uint32_t seed) {
      ++total;
      uint32_t nx[2];
      int n = next_cells(a, kind, seed, nx);
      for (int b = 0; b < n; ++b) {
        uint32_t c = nx[b];
        // a gradient path is acyclic: a chain is never longer than `limit` (the cell count)
        for (unsigned long long steps = 0;; ++steps) {
          if (steps >= limit) { bad = true; break; }
          ++total;
          uint32_t nn[2];
          int m = next_cells(a, kind, c, nn);
          if (m == 0) break;
          if (m > 1) { atomicOr(a.status, ST_INVARIANT); break; }  // a chain cell never branches
          c = nn[0];
        }
      }
    });
    if (bad) { atomicOr(a.status, ST_CYCLE); total = 0; }
    if (total > 0xffffffffull) { atomicOr(a.status, ST_SIMPLIFY_LIMIT); total = 0; }
    len[s] = (uint32_t)total;
  }
}

// pass 2: the reference's breadth-first growth, the output span is the queue
__global__ void k_saddle_disc_write(DiscArgs a, int kind, SeedRuns sr, const uint32_t *off, uint32_t *out) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < a.ncp; s += gridDim.x * blockDim.x) {
    if ((a.flags[s] & F_BCANCEL) || cdim(a.cellid[s]) != 1) continue;
    uint32_t o = off[s], cap = off[s + 1] - o, tail = 0;
    uint32_t *q = out + o;
    for_seeds(a, kind, s, sr, [&](uint32_t seed) { if (tail < cap) q[tail++] = seed; });
    for (uint32_t head = 0; head < tail; ++head) {
      uint32_t nx[2];
      int n = next_cells(a, kind, q[head], nx);
      for (int b = 0; b < n; ++b) {
        if (tail < cap) q[tail++] = nx[b];
        else atomicOr(a.status, ST_INVARIANT);
      }
    }
  }
}

// 5. per-cp disc lengths of the extrema from the sorted owner keys
__global__ void k_group_counts(long long n, uint32_t ncp, const uint32_t *key, uint32_t *cnt) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    uint32_t k = key[p];
    if (k < ncp) atomicAdd(cnt + k, 1u);
  }
}
__global__ void k_add_counts(uint32_t n, const uint32_t *a, uint32_t *b) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] += a[i];
}
__global__ void k_seed_runs(long long n, uint32_t ncp, const uint32_t *key, uint32_t *start, uint32_t *count) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    uint32_t k = key[p];
    if (k >= ncp) continue;
    if (p == 0 || key[p - 1] != k) start[k] = (uint32_t)p;
    atomicAdd(count + k, 1u);
  }
}
__global__ void k_group_scatter(long long n, uint32_t ncp, const uint32_t *key, const uint32_t *val,
                                const uint32_t *start, const uint32_t *off, uint32_t *out) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    uint32_t k = key[p];
    if (k < ncp) out[off[k] + (uint32_t)p - start[k]] = val[p];
  }
}

static unsigned nb(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (unsigned)(b < 1 ? 1 : b);
}
static int nbits_for(long long n) {
  int b = 1;
  while ((1ll << b) <= n) ++b;
  return b;
}

cudaError_t fill_discs(DiscIO &io, cudaStream_t st) {
  DiscArgs a;
  a.g = io.g; a.codes = io.codes; a.labels = io.labels; a.ncp_ds = (uint32_t)io.ncp_ds; a.ncp = (uint32_t)io.ncp;
  a.cellid = io.cellid; a.flags = io.flags; a.pair_idx = io.pair_idx;
  a.aoff = io.aoff; a.asc = io.asc; a.doff = io.doff; a.des = io.des; a.status = io.status;
  const long long ncp = io.ncp;
  const GridGeom &g = io.g;
  const long long nV = (long long)((g.rx1 - g.rx0) / 2 + 1) * ((g.ry1 - g.ry0) / 2 + 1);
  const long long nF = (long long)((g.rx1 - g.rx0) / 2) * ((g.ry1 - g.ry0) / 2);
  const long long nmax = std::max(std::max(nV, nF), std::max(io.nasc, io.ndes)) + 1;
  size_t words = (size_t)ncp * 7 + 8 + (size_t)nmax * 4 + (size_t)(nV + nF) * 2 + 64;
  uint32_t *buf = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&buf, sizeof(uint32_t) * words, st);
  if (e != cudaSuccess) return e;
  uint32_t *redir = buf, *acnt = buf + ncp, *dcnt = buf + 2 * ncp, *slen = buf + 3 * ncp;
  uint32_t *sstart = buf + 4 * ncp, *scount = buf + 5 * ncp, *soff = buf + 6 * ncp;  // soff: ncp+1
  uint32_t *key = buf + 7 * ncp + 8, *val = key + nmax, *kt = val + nmax, *vt = kt + nmax;
  uint32_t *gkey[2] = {vt + nmax, vt + nmax + nV}, *gval[2] = {vt + nmax + nV + nF, vt + nmax + 2 * nV + nF};
  const long long gn[2] = {nV, nF};
  auto L = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };

  if (ncp) {
    k_redir_init<<<nb(ncp), 256, 0, st>>>((uint32_t)ncp, redir);
    DMSC_LAUNCHED(1);
    k_redir_saddles<<<nb(ncp), 256, 0, st>>>(a, redir);
    DMSC_LAUNCHED(1);
  }
  L(cudaMemsetAsync(acnt, 0, sizeof(uint32_t) * ncp * 2, st));
  // extremum discs: vertices -> minima (asc_disc), faces -> maxima (des_disc),
  // grouped by owner with a stable sort (row-major order is the append order)
  for (int kind = 0; kind < 2 && e == cudaSuccess; ++kind) {
    long long n = gn[kind];
    if (n <= 0) continue;
    k_disc_keys<<<nb(n), 256, 0, st>>>(a, redir, kind, gkey[kind], gval[kind]);
    DMSC_LAUNCHED(1);
    L(radix_sort_pairs(gkey[kind], gval[kind], kt, vt, n, nbits_for(ncp), st));
    k_group_counts<<<nb(n), 256, 0, st>>>(n, (uint32_t)ncp, gkey[kind], kind ? dcnt : acnt);
    DMSC_LAUNCHED(1);
  }
  // saddle discs
  for (int kind = 0; kind < 2 && e == cudaSuccess; ++kind) {
    // seeds pushed by cancelled extrema: asc from maxima (via des), des from minima (via asc)
    k_seed_count<<<nb(ncp), 256, 0, st>>>(a, kind, slen);
    DMSC_LAUNCHED(1);
    L(scan_exclusive_u32(slen, ncp, soff, soff + ncp, st));
    uint32_t ns = 0;
    L(cudaMemcpyAsync(&ns, soff + ncp, 4, cudaMemcpyDeviceToHost, st));
    L(cudaStreamSynchronize(st));
    if (e != cudaSuccess) break;
    if ((long long)ns > nmax) { e = cudaErrorInvalidValue; break; }
    if (ns) {
      k_seed_write<<<nb(ncp), 256, 0, st>>>(a, kind, soff, key, val);
      DMSC_LAUNCHED(1);
      L(radix_sort_pairs(key, val, kt, vt, ns, nbits_for(ncp), st));  // stable: pushers stay in index order
    }
    L(cudaMemsetAsync(scount, 0, sizeof(uint32_t) * ncp, st));
    if (ns) {
      k_seed_runs<<<nb(ns), 256, 0, st>>>(ns, (uint32_t)ncp, key, sstart, scount);
      DMSC_LAUNCHED(1);
    }
    SeedRuns sr{val, sstart, scount};
    k_saddle_disc_count<<<nb(ncp), 128, 0, st>>>(a, kind, sr, slen, io.limit);
    DMSC_LAUNCHED(1);
    k_add_counts<<<nb(ncp), 256, 0, st>>>((uint32_t)ncp, slen, kind ? dcnt : acnt);
    DMSC_LAUNCHED(1);
    uint32_t *offs = kind ? io.ddoff : io.adoff;
    L(scan_exclusive_u32(kind ? dcnt : acnt, ncp, offs, offs + ncp, st));
    uint32_t tot = 0;
    L(cudaMemcpyAsync(&tot, offs + ncp, 4, cudaMemcpyDeviceToHost, st));
    L(cudaStreamSynchronize(st));
    if (e != cudaSuccess) break;
    DevBuf<uint32_t> *ob = kind ? io.ddisc : io.adisc;
    L(ob->ensure((size_t)tot + 1));
    if (e != cudaSuccess) break;
    k_saddle_disc_write<<<nb(ncp), 128, 0, st>>>(a, kind, sr, offs, ob->p);
    DMSC_LAUNCHED(1);
    long long n = gn[kind];
    if (n > 0) {  // extremum groups of this kind
      k_seed_runs<<<nb(n), 256, 0, st>>>(n, (uint32_t)ncp, gkey[kind], sstart, scount);
      DMSC_LAUNCHED(1);
      k_group_scatter<<<nb(n), 256, 0, st>>>(n, (uint32_t)ncp, gkey[kind], gval[kind], sstart, offs, ob->p);
      DMSC_LAUNCHED(1);
    }
    (kind ? io.nddisc : io.nadisc) = tot;
  }
  cudaFreeAsync(buf, st);
  if (e == cudaSuccess) e = cudaGetLastError();
  return e;
}

}  // namespace dmsc
