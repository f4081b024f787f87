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
// The device does the same in four parts: redirection per critical point;
// the extremum discs from runs of one owner along the rows, stably sorted by
// owner (row-major order is the append order); a stable sort of the
// cancelled-extremum seeds by saddle; and the saddle discs as interleaved
// chains (section 4b below) placed window by window, with one thread per
// saddle that first counts and then writes its breadth-first discs (the
// output array as the queue) for the few saddles with more than KMAX chains.
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

// 2a. the disc owner of every critical point used as a label: one level of
// redirection (:1142-1187).  fo = owner | grid << 30 (grid 0: a minimum, for
// vertices; 1: a maximum, for faces); FO_BAD where a label would break the
// reference's invariants (the owner must be a surviving extremum of the
// label's dimension).
constexpr uint32_t FO_BAD = 0xFFFFFFFFu;
__global__ void k_owner_final(DiscArgs a, const uint32_t *redir, uint32_t *fo) {
  const uint32_t n = a.ncp_ds < a.ncp ? a.ncp_ds : a.ncp;
  for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
    const uint32_t mc = a.cellid[m];
    const int d = cdim(mc);
    uint32_t o = FO_BAD;
    if (d != 1) {
      const uint32_t r = rect_has(a.g, cx(mc), cy(mc)) ? redir[m] : m;
      if (r < a.ncp && !(a.flags[r] & F_BCANCEL) && cdim(a.cellid[r]) == d) o = r | ((uint32_t)(d >> 1) << 30);
    }
    fo[m] = o;
  }
}

// 2b. owner keys of the rect vertices (vertex grid) and faces (face grid),
// row-major, from one read of the labels
// one rect row of vertices per blockIdx.y, KEYS_ILP vertices per thread
// (KEYS_THREADS apart) with their label loads issued together
constexpr int KEYS_THREADS = 256, KEYS_ILP = 2, KEYS_SPAN = KEYS_THREADS * KEYS_ILP;
__global__ void __launch_bounds__(KEYS_THREADS) k_disc_keys(DiscArgs a, const uint32_t *__restrict__ fo,
                                                            uint32_t *__restrict__ key0, uint32_t *__restrict__ key1) {
  const GridGeom &g = a.g;
  const int nx = (g.rx1 - g.rx0) / 2 + 1, ny = (g.ry1 - g.ry0) / 2 + 1;
  const uint32_t n_ok = a.ncp_ds < a.ncp ? a.ncp_ds : a.ncp;
  const int jj = blockIdx.y, ry = g.ry0 + 2 * jj;
  const int i0 = blockIdx.x * KEYS_SPAN + threadIdx.x;
  uint4 L[KEYS_ILP];
#pragma unroll
  for (int q = 0; q < KEYS_ILP; ++q) {
    const int ii = i0 + q * KEYS_THREADS;
    L[q] = ii < nx ? a.labels[(long long)(ry >> 1) * g.vnx + ((g.rx0 >> 1) + ii)] : make_uint4(0, 0, 0, 0);
  }
  uint32_t bad = 0;
#pragma unroll
  for (int q = 0; q < KEYS_ILP; ++q) {
    const int ii = i0 + q * KEYS_THREADS;
    if (ii >= nx) continue;
    for (int kind = 0; kind < 2; ++kind) {
      if (kind && (ii == nx - 1 || jj == ny - 1)) continue;
      const uint32_t m = kind ? L[q].w : L[q].x;
      uint32_t o = a.ncp;
      if (m != LABEL_NONE) {
        const uint32_t v = m < n_ok ? fo[m] : FO_BAD;
        if (v == FO_BAD || (v >> 30) != (uint32_t)kind) bad = 1;
        else o = v & 0x3FFFFFFFu;
      }
      const long long fi = kind ? (long long)jj * (nx - 1) + ii : (long long)jj * nx + ii;
      (kind ? key1 : key0)[fi] = o;
    }
  }
  if (bad) atomicOr(a.status, ST_INVARIANT);
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

// Serial pass for saddles with more than KMAX chains.  1: disc lengths (every
// non-critical path cell has at most one successor, so each seed expands into
// at most two chains).
__global__ void k_saddle_disc_count(DiscArgs a, int kind, SeedRuns sr, const uint8_t *big, uint32_t *len,
                                    unsigned long long limit) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < a.ncp; s += gridDim.x * blockDim.x) {
    if (!big[s]) continue;
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

// 2: the reference's breadth-first growth, the output span is the queue
__global__ void k_saddle_disc_write(DiscArgs a, int kind, SeedRuns sr, const uint8_t *big, const uint32_t *off,
                                    uint32_t *out) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < a.ncp; s += gridDim.x * blockDim.x) {
    if (!big[s]) continue;
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

// ---------------------------------------------------------------------------
// 4b. Saddle discs as chains.  A disc's breadth-first queue starts with its
// level-0 items (the seeds above, m of them); each item has up to two
// successors, and every later cell exactly one or none (a chain cell is an
// edge paired with the face (asc) or vertex (des) it was reached from).  So
// the disc is m items followed by K chains c_1..c_K (successors of item 1 in
// order, then of item 2, ...) interleaved level by level: the cell at level
// t >= 1 of chain j sits at
//     m + sum_j' min(L_j', t - 1) + #{ j' < j : L_j' >= t }
// where L_j is the length of chain j.  Chains are followed in "hops": per
// 64x64 vertex tile, list ranking in shared memory gives every edge the
// number of cells to its tile exit, the edge after it and the edge SEG_MAX
// cells ahead, so a chain's length costs one step per tile crossed.  The
// lengths fix every cell's place before any cell is known: per saddle, the
// level ranges over which its set of alive chains is constant are regular
// interleaves (k_zip_blocks).  The chains are cut into pieces of at most
// SEG_MAX cells (also where the set of alive chains changes), each with the
// disc position of its first cell and its stride, and every block gathers the
// cells of one window of disc positions in shared memory, walking the pieces
// that reach it one lane each, and stores the window out (k_win_place).
// ---------------------------------------------------------------------------
constexpr int KMAX = 32;                 // saddles with more chains take the serial pass
constexpr uint32_t HOP_END = 0xFFFFFFFFu;
constexpr int HOP_SLOTS = 2 * TX * TY;   // H and Vt edge of every vertex of a tile
constexpr uint16_t SLOT_NIL = 0xFFFF;

// edge id over the ext window: 2 * vertex index + (0: H edge (2i+1, 2j), 1: Vt edge (2i, 2j+1))
__host__ __device__ __forceinline__ uint32_t edge_id(const GridGeom &g, int rx, int ry) {
  return (uint32_t)(((long long)(ry >> 1) * g.vnx + (rx >> 1)) * 2 + (ry & 1));
}
__host__ __device__ __forceinline__ void edge_cell(const GridGeom &g, uint32_t e, int &rx, int &ry) {
  uint32_t v = e >> 1;
  int vx = (int)(v % (uint32_t)g.vnx), vy = (int)(v / (uint32_t)g.vnx);
  rx = 2 * vx + ((e & 1) ? 0 : 1);
  ry = 2 * vy + (int)(e & 1);
}

// Index of edge (rx, ry) (ext-local) in the successor-word array, which is
// laid out in 8x8-vertex blocks of 128 words (two edges per vertex), so that a
// chain walked in any direction stays inside one block for several steps.
__host__ __device__ __forceinline__ uint32_t succ_idx(const GridGeom &g, int rx, int ry) {
  const uint32_t vx = (uint32_t)(rx >> 1), vy = (uint32_t)(ry >> 1), nbx = ((uint32_t)g.vnx + 7u) >> 3;
  return (((vy >> 3) * nbx + (vx >> 3)) << 7) | ((vy & 7u) << 4) | ((vx & 7u) << 1) | ((uint32_t)ry & 1u);
}
__host__ __device__ __forceinline__ size_t succ_words(const GridGeom &g) {
  return (size_t)(((uint32_t)g.vnx + 7u) >> 3) * (size_t)(((uint32_t)g.vny + 7u) >> 3) * 128u;
}

// Successor words.  A chain step from an edge goes to another edge of the
// face (asc) or vertex (des) it crosses: one of the four diagonal neighbours
// (dx, dy = +-1) or one of the two edges 2 cells away along one axis, which
// is y for an asc H edge or a des Vt edge and x otherwise.  So a step is a
// 3-bit code: 0-3 diagonal (dx = +1 if bit 0, dy = +1 if bit 1), 4 / 5 the
// +2 / -2 axis step, 7 no further step in this word.  Every edge keeps a
// 16-bit word of the next WORD_STEPS steps of its chain inside its tile
// (fewer where the chain leaves the tile or ends: the step out of the tile
// is the word's last), so a walk makes one dependent load per WORD_STEPS
// cells instead of one per cell.  A diagonal step changes the edge's
// orientation, an axis step keeps it.
constexpr int WORD_STEPS = 5;
constexpr uint32_t WORD_END = 7u;
__device__ __forceinline__ bool step_axis_y(int kind, int rx) { return ((rx & 1) != 0) == (kind == 0); }
// code of the step (dx, dy); WORD_END if it is no chain step
__device__ __forceinline__ uint32_t step_code(int dx, int dy) {
  if ((dx == 1 || dx == -1) && (dy == 1 || dy == -1)) return (uint32_t)(dx > 0) | ((uint32_t)(dy > 0) << 1);
  if ((dx == 0 && (dy == 2 || dy == -2)) || (dy == 0 && (dx == 2 || dx == -2))) return dx + dy > 0 ? 4u : 5u;
  return WORD_END;
}
__device__ __forceinline__ void step_apply(uint32_t q, bool axis_y, int &rx, int &ry) {
  if (q < 4u) {
    rx += (q & 1u) ? 1 : -1;
    ry += (q & 2u) ? 1 : -1;
  } else {
    const int s = q == 4u ? 2 : -2;
    if (axis_y) ry += s; else rx += s;
  }
}
// the same step as a packed cell id delta (x | y << 16)
__device__ __forceinline__ uint32_t step_delta(uint32_t q, bool axis_y) {
  if (q < 4u) return (uint32_t)(((q & 2u) ? 65536 : -65536) + ((q & 1u) ? 1 : -1));
  const int s = q == 4u ? 2 : -2;
  return (uint32_t)(axis_y ? s * 65536 : s);
}
static_assert(WORD_STEPS >= 1 && 3 * WORD_STEPS <= 16, "a word's steps fit its 16 bits");
// a loaded word with the bits above its steps set, so that a used-up word reads WORD_END
__device__ __forceinline__ uint32_t word_bits(uint16_t w) { return (uint32_t)w | (0xFFFFFFFFu << (3 * WORD_STEPS)); }
// an ext-local cell whose successor word may be loaded
__device__ __forceinline__ bool word_cell_ok(const GridGeom &g, int rx, int ry) {
  return rx >= 0 && ry >= 0 && rx <= g.cx && ry <= g.cy && ((rx ^ ry) & 1);
}

// next_cells in ext-local coordinates with a code accessor: up to two
// successors of edge (rx, ry); returns -1 on a non-critical unpaired rect cell.
template <class CodeFn>
__device__ __forceinline__ int succ_local(const GridGeom &g, int kind, int rx, int ry, CodeFn code, int ox[2], int oy[2]) {
  const int d0 = rx & 1, d1 = ry & 1;
  int c[2][2];
  if (kind == 0) { c[0][0] = rx + d1; c[0][1] = ry + d0; c[1][0] = rx - d1; c[1][1] = ry - d0; }
  else           { c[0][0] = rx + d0; c[0][1] = ry + d1; c[1][0] = rx - d0; c[1][1] = ry - d1; }
  int n = 0;
  for (int k = 0; k < 2; ++k) {
    const int qx = c[k][0], qy = c[k][1];
    if (qx < 0 || qy < 0 || qx > g.cx || qy > g.cy) continue;
    const uint32_t qc = code(qx, qy);
    if (qc & CODE_CRIT) continue;
    if (qx < g.rx0 || qx > g.rx1 || qy < g.ry0 || qy > g.ry1) continue;
    if (!(qc & CODE_PAIRED)) return -1;  // every rect cell is paired or critical
    const uint32_t d = qc & 3;
    const int px = qx + (d == DIR_PX ? 1 : d == DIR_MX ? -1 : 0), py = qy + (d == DIR_PY ? 1 : d == DIR_MY ? -1 : 0);
    if (px == rx && py == ry) continue;
    ox[n] = px; oy[n] = py; ++n;
  }
  return n;
}

// The chain kind of an edge: 0 if it is paired with a face (asc chains),
// 1 if paired with a vertex (des chains), -1 if critical or unpaired.
__device__ __forceinline__ int chain_kind(uint32_t code, int rx, int ry) {
  if ((code & CODE_CRIT) || !(code & CODE_PAIRED)) return -1;
  const uint32_t d = code & 3;
  const int px = rx + (d == DIR_PX ? 1 : d == DIR_MX ? -1 : 0), py = ry + (d == DIR_PY ? 1 : d == DIR_MY ? -1 : 0);
  return ((px & 1) + (py & 1)) == 2 ? 0 : 1;
}

constexpr int HOP_THREADS = 512;
// successor of an edge along its chain as a step code (0-5, as in the successor words)
constexpr uint8_t SUCC_NONE = 0xFF;
constexpr int SEG_LOG = 5, SEG_MAX = 1 << SEG_LOG;  // cells of a write piece: the jump pointer distance

constexpr uint8_t SUCC_TWO = 0xFE;  // a cell with two successors (it ends no chain)
struct HopSmem {
  uint32_t code[(TX + 2) * (TY + 2)];
  uint32_t nv[HOP_SLOTS];     // next slot << 16 | cells counted so far
  uint16_t tail[HOP_SLOTS];
  uint8_t sd[HOP_SLOTS];      // successor step code of every slot (SUCC_NONE / SUCC_TWO)
};

// Per edge, for the chains of its own kind: hop_to (the edge after its
// in-tile run, HOP_END if the chain ends in the tile), hop_len (cells of the
// run, 0 for a branching cell), jseg (the edge SEG_MAX cells ahead in the
// same run, HOP_END if the run is shorter) and its successor word (wcode, at
// succ_idx).  One block per tile.
__global__ void __launch_bounds__(HOP_THREADS, 3)
k_disc_hops(GridGeom g, const uint32_t *__restrict__ codes, uint32_t *__restrict__ to, uint16_t *__restrict__ len,
            uint32_t *__restrict__ jseg, uint16_t *__restrict__ wcode, uint32_t *status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  HopSmem &S = *reinterpret_cast<HopSmem *>(smem_raw);
  const int tx0 = blockIdx.x * TX, ty0 = blockIdx.y * TY;
  for (int e = threadIdx.x; e < (TX + 2) * (TY + 2); e += blockDim.x) {
    const int jj = e / (TX + 2), ii = e - jj * (TX + 2);
    const int vx = tx0 - 1 + ii, vy = ty0 - 1 + jj;
    S.code[e] = (vx >= 0 && vy >= 0 && vx < g.vnx && vy < g.vny) ? codes[(long long)vy * g.vnx + vx] : 0u;
  }
  __syncthreads();
  auto code = [&](int qx, int qy) -> uint32_t {
    const int ii = (qx >> 1) - tx0 + 1, jj = (qy >> 1) - ty0 + 1;
    return (S.code[jj * (TX + 2) + ii] >> (8 * ((qx & 1) | ((qy & 1) << 1)))) & 0xff;
  };
  auto slot_cell = [&](int sl, int &rx, int &ry) -> bool {  // false: no such edge
    const int t = sl & 1, v = sl >> 1, li = v % TX, lj = v / TX;
    const int vx = tx0 + li, vy = ty0 + lj;
    rx = 2 * vx + (t ? 0 : 1);
    ry = 2 * vy + t;
    return vx < g.vnx && vy < g.vny && rx <= g.cx && ry <= g.cy;
  };
  auto in_tile = [&](int ox, int oy) {
    const int vx = ox >> 1, vy = oy >> 1;
    return vx >= tx0 && vx < tx0 + TX && vy >= ty0 && vy < ty0 + TY;
  };
  uint32_t st = 0;
  int active = 0;
  for (int sl = threadIdx.x; sl < HOP_SLOTS; sl += blockDim.x) {
    int rx, ry, ox[2], oy[2];
    uint32_t nx = SLOT_NIL;
    if (slot_cell(sl, rx, ry)) {
      const int kind = chain_kind(code(rx, ry), rx, ry);
      uint8_t sd = SUCC_NONE;
      if (kind >= 0) {
        const int n = succ_local(g, kind, rx, ry, code, ox, oy);
        if (n < 0) st |= ST_INVARIANT;
        if (n == 1) {
          const int dx = ox[0] - rx, dy = oy[0] - ry;
          const uint32_t q = step_code(dx, dy);
          // the decoders take an axis step along the axis of the kind and orientation
          if (q == WORD_END || (q >= 4u && (dy != 0) != step_axis_y(kind, rx))) st |= ST_INVARIANT;
          else sd = (uint8_t)q;
        }
        if (n == 2) sd = SUCC_TWO;
        if (n == 1 && in_tile(ox[0], oy[0])) {
          nx = (uint32_t)((((oy[0] >> 1) - ty0) * TX + ((ox[0] >> 1) - tx0)) << 1) | (uint32_t)(oy[0] & 1);
          active = 1;
        }
      }
      S.sd[sl] = sd;
    } else {
      S.sd[sl] = SUCC_NONE;
    }
    S.nv[sl] = (nx << 16) | 1u;
    S.tail[sl] = (uint16_t)sl;
  }
  __syncthreads();
  // successor words: the next WORD_STEPS steps of each edge's chain inside the
  // tile, from the successor pointers before the ranking rounds replace them;
  // WORD_ILP slots per thread step together so that their loads overlap
  constexpr int WORD_ILP = 4;
  static_assert(HOP_SLOTS % (WORD_ILP * HOP_THREADS) == 0, "word pass covers the slots exactly");
  for (int base = threadIdx.x; base < HOP_SLOTS; base += WORD_ILP * HOP_THREADS) {
    int s[WORD_ILP], k[WORD_ILP];
    uint32_t w[WORD_ILP];
    bool on[WORD_ILP];
#pragma unroll
    for (int j = 0; j < WORD_ILP; ++j) { s[j] = base + j * HOP_THREADS; k[j] = 0; w[j] = 0; on[j] = true; }
#pragma unroll
    for (int t = 0; t < WORD_STEPS; ++t) {
#pragma unroll
      for (int j = 0; j < WORD_ILP; ++j) {
        if (!on[j]) continue;
        const uint32_t q = S.sd[s[j]];
        const uint32_t n = S.nv[s[j]] >> 16;
        if (q >= SUCC_TWO) { on[j] = false; continue; }
        w[j] |= q << (3 * k[j]);
        ++k[j];
        if (n == SLOT_NIL) on[j] = false;  // the step left the tile, or the chain ends after it
        else s[j] = (int)n;
      }
    }
#pragma unroll
    for (int j = 0; j < WORD_ILP; ++j) {
      int rx, ry;
      if (!slot_cell(base + j * HOP_THREADS, rx, ry)) continue;
      if (k[j] < WORD_STEPS) w[j] |= WORD_END << (3 * k[j]);
      wcode[succ_idx(g, rx, ry)] = (uint16_t)w[j];
    }
  }
  // list ranking: at most 13 rounds (2^13 = HOP_SLOTS cells); after round
  // SEG_LOG every pointer still inside the tile is exactly SEG_MAX cells ahead
  constexpr int PER = HOP_SLOTS / HOP_THREADS;
  int rounds = 0;
  for (int round = 0; round < 14 && __syncthreads_or(active); ++round) {
    rounds = round + 1;
    uint32_t nn[PER];
    uint16_t nt[PER];
    active = 0;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int sl = threadIdx.x + q * HOP_THREADS;
      const uint32_t v = S.nv[sl];
      nn[q] = v; nt[q] = S.tail[sl];
      const uint32_t n = v >> 16;
      if (n != SLOT_NIL) {
        const uint32_t w = S.nv[n];
        nn[q] = (w & 0xFFFF0000u) | ((v + w) & 0xFFFFu);
        nt[q] = S.tail[n];
        active |= (w >> 16) != SLOT_NIL;
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int sl = threadIdx.x + q * HOP_THREADS;
      S.nv[sl] = nn[q]; S.tail[sl] = nt[q];
      if (round == SEG_LOG - 1) {  // pointers now SEG_MAX cells ahead (or none)
        int rx, ry, jx, jy;
        if (slot_cell(sl, rx, ry)) {
          const uint32_t js = nn[q] >> 16;
          uint32_t jv = HOP_END;
          if (js != SLOT_NIL) { slot_cell((int)js, jx, jy); jv = edge_id(g, jx, jy); }
          jseg[edge_id(g, rx, ry)] = jv;
        }
      }
    }
  }
  __syncthreads();
  for (int sl = threadIdx.x; sl < HOP_SLOTS; sl += blockDim.x) {
    int rx, ry;
    if (!slot_cell(sl, rx, ry)) continue;
    const uint32_t e = edge_id(g, rx, ry);
    const uint32_t v = S.nv[sl];
    if ((v >> 16) != SLOT_NIL) { st |= ST_CYCLE; to[e] = HOP_END; len[e] = 0; continue; }
    const int tl = S.tail[sl];
    const uint8_t sd = S.sd[tl];
    uint32_t dst = HOP_END;
    if (sd < SUCC_TWO) {  // the run leaves the tile after its tail
      int tx, ty;
      slot_cell(tl, tx, ty);
      const int kind = chain_kind(code(tx, ty), tx, ty);
      step_apply(sd, step_axis_y(kind, tx), tx, ty);
      dst = edge_id(g, tx, ty);
    }
    to[e] = dst;
    // a cell with two successors ends no chain: length 0 marks it for the walkers
    len[e] = sd == SUCC_TWO ? 0 : (uint16_t)(v & 0xFFFFu);
    if (rounds < SEG_LOG) jseg[e] = HOP_END;  // every run in the tile is shorter than SEG_MAX + 1 cells
  }
  if (st) atomicOr(status, st);
}

struct ChainArgs {
  const uint32_t *hop_to;
  const uint16_t *hop_len;
  const uint32_t *jseg;
  const uint16_t *wcode;  // per edge (at succ_idx): its successor word
  int kind;               // the chains' kind (0 asc, 1 des)
  uint32_t *kc;         // per cp: chains of a saddle handled here (0 otherwise)
  uint32_t *mc;         // per cp: level-0 items
  uint8_t *big;         // per cp: surviving saddle with more than KMAX chains
  uint32_t *cbase;      // exclusive scan of kc
  uint32_t *cstart, *csaddle, *clen, *cnseg, *csegoff;  // per chain
  uint4 *segs;          // (first edge, first disc position, cells | alive << 8, chain)
  uint4 *blocks;        // per chain slot of a saddle, 2 uint4: an interleave record (k_zip_blocks)
  uint32_t cap;         // chain slots allocated
  unsigned long long limit;
};

__device__ __forceinline__ bool surviving_saddle(const DiscArgs &a, uint32_t s) {
  return !(a.flags[s] & F_BCANCEL) && cdim(a.cellid[s]) == 1;
}
// successors of a level-0 item (a global edge cell) as ext-local edge ids
__device__ __forceinline__ int item_children(const DiscArgs &a, int kind, uint32_t pc, uint32_t out[2]) {
  uint32_t nx[2];
  int n = next_cells(a, kind, pc, nx);
  for (int b = 0; b < n; ++b) out[b] = edge_id(a.g, cx(nx[b]) - a.g.ex0, cy(nx[b]) - a.g.ey0);
  return n;
}

__global__ void k_chain_count(DiscArgs a, int kind, SeedRuns sr, ChainArgs c) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < a.ncp; s += gridDim.x * blockDim.x) {
    uint32_t m = 0, K = 0;
    if (surviving_saddle(a, s)) {
      for_seeds(a, kind, s, sr, [&](uint32_t seed) {
        uint32_t ch[2];
        ++m;
        K += item_children(a, kind, seed, ch);
      });
    }
    const bool big = K > KMAX;
    c.kc[s] = big ? 0 : K;
    c.mc[s] = m;
    c.big[s] = big;
  }
}

// chain starts, lengths and piece counts; the disc length of every saddle
// handled here (0 for other critical points, big saddles untouched)
__global__ void k_chain_len(DiscArgs a, int kind, SeedRuns sr, ChainArgs c, uint32_t *slen) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < a.ncp; s += gridDim.x * blockDim.x) {
    if (c.big[s]) continue;
    if (!surviving_saddle(a, s)) { slen[s] = 0; continue; }
    unsigned long long total = c.mc[s];
    uint32_t j = c.cbase[s];
    bool bad = false;
    for_seeds(a, kind, s, sr, [&](uint32_t seed) {
      uint32_t ch[2];
      const int n = item_children(a, kind, seed, ch);
      for (int b = 0; b < n; ++b) {
        unsigned long long L = 0;
        uint32_t nseg = 0;
        for (uint32_t e = ch[b]; e != HOP_END; e = c.hop_to[e]) {
          const uint32_t l = c.hop_len[e];
          if (l == 0) { atomicOr(a.status, ST_INVARIANT); break; }  // a chain cell never branches
          L += l;
          nseg += (l + SEG_MAX - 1) / SEG_MAX;
          if (L > c.limit) { bad = true; break; }
        }
        // piece slots: one per SEG_MAX cells of each hop, and one more for each level
        // where another of the saddle's chains ends inside this one (at most K - 1)
        if (j < c.cap) { c.cstart[j] = ch[b]; c.csaddle[j] = s; c.clen[j] = (uint32_t)L; c.cnseg[j] = nseg + c.kc[s] - 1; }
        else atomicOr(a.status, ST_CAPACITY);
        ++j;
        total += L;
      }
    });
    if (bad) { atomicOr(a.status, ST_CYCLE); total = 0; }
    if (total > 0xffffffffull) { atomicOr(a.status, ST_SIMPLIFY_LIMIT); total = 0; }
    slen[s] = (uint32_t)total;
  }
}

// Pieces of every chain, each with the disc position of its first cell and
// the step between its cells: the chain's hops cut at every SEG_MAX cells
// and at the levels where the saddle's set of alive chains changes (the
// interleave records of k_zip_blocks), so that a piece's cells are
// `alive` apart in the disc.  A piece is (first edge, first position,
// cells | alive << 8, chain); the chain's unused slots get 0 cells.
__global__ void k_chain_segs(long long nchains, DiscArgs a, ChainArgs c) {
  const GridGeom &g = a.g;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nchains; k += (long long)gridDim.x * blockDim.x) {
    uint32_t o = c.csegoff[k], end = c.csegoff[k + 1];
    if (o == end) continue;  // an unused chain slot (slots counted by the two-per-saddle bound)
    const uint32_t s = c.csaddle[k];
    bool ok = s < a.ncp;
    const uint32_t cb = ok ? c.cbase[s] : 0, K = ok ? c.kc[s] : 0, j = (uint32_t)k - cb;
    ok = ok && j < K && K <= (uint32_t)KMAX && cb + K <= c.cap;
    uint32_t b = 0, first = 1, nlev = 0;
    uint4 r0 = make_uint4(0, 0, 0, 0);
    if (ok) {
      r0 = c.blocks[2 * cb];
      first = c.blocks[2 * cb + 1].x;
      ok = r0.z != 0 && r0.y != 0;
      nlev = ok ? r0.y / r0.z : 0;
    }
    uint32_t T = 1;
    for (uint32_t e = c.cstart[k]; ok && e != HOP_END && o < end; e = c.hop_to[e]) {
      const uint32_t l = c.hop_len[e];
      if (l == 0) break;
      uint32_t x = e, done = 0;
      while (ok && done < l && o < end) {
        const uint32_t t0 = T + done;
        while (t0 - first >= nlev) {  // the record holding level t0 (records ascend in level)
          if (++b >= K) { ok = false; break; }
          r0 = c.blocks[2 * (cb + b)];
          first = c.blocks[2 * (cb + b) + 1].x;
          if (!r0.z || !r0.y || t0 < first) { ok = false; break; }
          nlev = r0.y / r0.z;
        }
        if (!ok || !(r0.w & (1u << j))) { ok = false; break; }
        uint32_t w = l - done < (uint32_t)SEG_MAX ? l - done : (uint32_t)SEG_MAX;
        if (first + nlev - t0 < w) w = first + nlev - t0;
        const uint32_t pos = r0.x + (t0 - first) * r0.z + __popc(r0.w & ((1u << j) - 1u));
        c.segs[o++] = make_uint4(x, pos, w | (r0.z << 8), (uint32_t)k);
        done += w;
        if (done < l) {  // the next piece's first edge, w cells ahead in the run
          if (w == (uint32_t)SEG_MAX) {
            x = c.jseg[x];
          } else {  // w steps along the successor words
            int rx, ry;
            edge_cell(g, x, rx, ry);
            bool ax = step_axis_y(c.kind, rx);
            uint32_t word = WORD_END;
            for (uint32_t i = 0; i < w; ++i) {
              uint32_t q = word & 7u;
              if (q == WORD_END) {
                if (!word_cell_ok(g, rx, ry)) { ok = false; break; }
                word = word_bits(c.wcode[succ_idx(g, rx, ry)]);
                q = word & 7u;
                if (q > 5u) { ok = false; break; }
              }
              word >>= 3;
              step_apply(q, ax, rx, ry);
              ax ^= q < 4u;
            }
            x = edge_id(g, rx, ry);
          }
          if (x == HOP_END) ok = false;
        }
      }
      T += l;
    }
    if (!ok) atomicOr(a.status, ST_INVARIANT);
    for (; o < end; ++o) c.segs[o] = make_uint4(0, 0, 0, (uint32_t)k);
  }
}

// level-0 items of the saddles handled here
__global__ void k_level0(DiscArgs a, int kind, SeedRuns sr, ChainArgs c, const uint32_t *off, uint32_t *out) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < a.ncp; s += gridDim.x * blockDim.x) {
    if (c.big[s] || !surviving_saddle(a, s)) continue;
    uint32_t o = off[s], end = off[s + 1];
    for_seeds(a, kind, s, sr, [&](uint32_t seed) {
      if (o < end) out[o++] = seed;
      else atomicOr(a.status, ST_INVARIANT);
    });
  }
}

// Per saddle: the level ranges over which the set of alive chains is
// constant.  Between consecutive distinct chain lengths the disc is a
// regular interleave of the alive chains.  Each range becomes a record of
// two uint4: (first output position, cells, alive chains, alive mask) and
// (first level, 0, 0, 0); the saddle's unused record slots are zeroed.
__global__ void k_zip_blocks(DiscArgs a, ChainArgs c, const uint32_t *off) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < a.ncp; s += gridDim.x * blockDim.x) {
    const uint32_t K = c.kc[s], cb = c.cbase[s];
    if (!K) continue;
    if (cb + K > c.cap) { atomicOr(a.status, ST_CAPACITY); continue; }
    uint32_t L[KMAX];
    for (uint32_t q = 0; q < K; ++q) L[q] = c.clen[cb + q];
    const uint32_t base = off[s] + c.mc[s];
    uint32_t prev = 0, P = 0, nb = 0;
    for (;;) {
      uint32_t u = 0xFFFFFFFFu, mask = 0;
      for (uint32_t q = 0; q < K; ++q)
        if (L[q] > prev) { mask |= 1u << q; u = L[q] < u ? L[q] : u; }
      if (!mask) break;
      const uint32_t na = (uint32_t)__popc(mask), n = (u - prev) * na;
      c.blocks[2 * (cb + nb)] = make_uint4(base + P, n, na, mask);
      c.blocks[2 * (cb + nb) + 1] = make_uint4(prev + 1, 0, 0, 0);
      ++nb;
      P += n;
      prev = u;
    }
    for (; nb < K; ++nb) c.blocks[2 * (cb + nb)] = make_uint4(0, 0, 0, 0);
  }
}

// Placement of the pieces' cells, one window of WIN disc positions per block.
// A piece's cells are `alive` positions apart from its first position
// (k_chain_segs).  Stored straight from the walking threads, every cell is a
// separate 4-byte store to a different sector; instead, the block walks every
// piece that has a cell inside its window (following the successor words,
// one load per WORD_STEPS cells), puts the window's cells into shared memory
// and stores the window out with 16-byte stores.  Positions of the window
// that no piece fills (level-0 items, saddles with many chains, extremum
// discs: other kernels write them) are left alone.  Discs are laid out in
// critical-point order, so the pieces that reach a window are those of the
// critical points from the one whose disc holds the window's first position
// (k_win_first) to the one whose disc holds the next window's first position.
constexpr int WIN = 8192, WIN_THREADS = 256;
constexpr uint32_t WIN_EMPTY = 0xFFFFFFFFu;  // no packed cell id (coordinates are below 2^15)

// first[w]: the critical point whose disc holds position w * WIN
__global__ void k_win_first(uint32_t ncp, const uint32_t *__restrict__ off, uint32_t nwin, uint32_t *__restrict__ first) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < ncp; s += gridDim.x * blockDim.x) {
    const unsigned long long a = off[s], b = off[s + 1];
    if (b <= a) continue;
    const unsigned long long w1 = (b - 1) / WIN;
    for (unsigned long long w = (a + WIN - 1) / WIN; w <= w1 && w < nwin; ++w) first[w] = s;
  }
}

__global__ void __launch_bounds__(WIN_THREADS) k_win_place(DiscArgs a, ChainArgs c, const uint32_t *__restrict__ first,
                                                           uint32_t nwin, uint32_t *__restrict__ out,
                                                           unsigned long long out_len) {
  __shared__ __align__(16) uint32_t stage[WIN];
  __shared__ uint32_t range[2], next_piece;
  __shared__ int dtab[16];  // packed cell id delta of step code q: [8 * (axis y) + q]
  const GridGeom &g = a.g;
  if (threadIdx.x < 16) {
    const uint32_t q = threadIdx.x & 7u;
    dtab[threadIdx.x] = q <= 5u ? (int)step_delta(q, threadIdx.x >= 8) : 0;
  }
  uint32_t st = 0;
  for (uint32_t w = blockIdx.x; w < nwin; w += gridDim.x) {
    const unsigned long long P0 = (unsigned long long)w * WIN;
    const unsigned long long P1 = P0 + WIN < out_len ? P0 + WIN : out_len;
    for (int i = threadIdx.x; i < WIN / 4; i += blockDim.x)
      reinterpret_cast<uint4 *>(stage)[i] = make_uint4(WIN_EMPTY, WIN_EMPTY, WIN_EMPTY, WIN_EMPTY);
    if (threadIdx.x == 0) {
      const uint32_t sa = first[w], sb = w + 1 < nwin ? first[w + 1] : a.ncp - 1;
      uint32_t lo = 0, hi = 0;
      if (sa <= sb && sb < a.ncp) {
        lo = c.csegoff[c.cbase[sa]];
        hi = c.csegoff[c.cbase[sb + 1]];
      } else {
        st |= ST_INVARIANT;
      }
      range[0] = lo;
      range[1] = hi;
      next_piece = lo + blockDim.x;
    }
    __syncthreads();
    const uint32_t lo = range[0], hi = range[1];
    // each thread's first piece by its index, the rest taken in turn from a
    // shared counter, so that threads whose walks end early take more
    for (uint32_t k = lo + threadIdx.x; k < hi; k = atomicAdd(&next_piece, 1u)) {
      const uint4 sg = c.segs[k];
      const uint32_t wl = sg.z & 0xffu, na = sg.z >> 8;
      if (!wl) continue;  // an unused slot
      unsigned long long pos = sg.y;
      const unsigned long long last = pos + (unsigned long long)(wl - 1) * na;
      if (wl > (uint32_t)SEG_MAX || na == 0 || na > (uint32_t)KMAX || last >= out_len) {
        st |= ST_INVARIANT;
        continue;
      }
      if (pos >= P1 || last < P0) continue;  // no cell in this window
      int rx, ry;
      edge_cell(g, sg.x, rx, ry);
      if (!word_cell_ok(g, rx, ry)) {
        st |= ST_INVARIANT;
        continue;
      }
      uint32_t cell = pack_cellid(g.ex0 + rx, g.ey0 + ry);
      uint32_t axb = step_axis_y(c.kind, rx) ? 8u : 0u;
      uint32_t word = wl > 1 ? word_bits(__ldg(c.wcode + succ_idx(g, rx, ry))) : WORD_END;
      uint32_t left = wl - 1;  // steps after the current cell
      uint32_t p = (uint32_t)pos;
      const uint32_t p0 = (uint32_t)P0, p1 = (uint32_t)P1;
      auto advance = [&]() -> bool {  // one step along the successor words
        uint32_t q = word & 7u;
        if (q == WORD_END) {  // the word is used up (or ended at a tile exit): the current cell's word
          rx = (int)(cell & 0xffffu) - g.ex0;
          ry = (int)(cell >> 16) - g.ey0;
          if (!word_cell_ok(g, rx, ry)) return false;
          word = word_bits(__ldg(c.wcode + succ_idx(g, rx, ry)));
          q = word & 7u;
          if (q > 5u) return false;
        }
        word >>= 3;
        cell += (uint32_t)dtab[axb | q];
        axb ^= q < 4u ? 8u : 0u;
        p += na;
        --left;
        return true;
      };
      bool ok = true;
      while (ok && p < p0) ok = advance();  // cells before the window: walked, not stored
      while (ok) {
        stage[p - p0] = cell;
        if (left == 0 || p + na >= p1) break;
        ok = advance();
      }
      if (!ok) st |= ST_INVARIANT;
    }
    __syncthreads();
    // the window out: four positions per thread, one 16-byte store where all four are filled
    const int nw = (int)(P1 - P0);
    for (int i = 4 * threadIdx.x; i < nw; i += 4 * blockDim.x) {
      const uint4 v = *reinterpret_cast<const uint4 *>(stage + i);
      if (i + 4 <= nw && v.x != WIN_EMPTY && v.y != WIN_EMPTY && v.z != WIN_EMPTY && v.w != WIN_EMPTY) {
        __stcs(reinterpret_cast<uint4 *>(out + P0 + i), v);
      } else {
        const uint32_t e[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (i + q < nw && e[q] != WIN_EMPTY) __stcs(out + P0 + i + q, e[q]);
      }
    }
    __syncthreads();  // the stage is refilled for the next window
  }
  if (st) atomicOr(a.status, st);
}

// 5. runs of equal sorted keys: the last element of each run writes (or adds)
// its length, after k_seed_runs has recorded the run starts
__global__ void k_run_len(long long n, uint32_t ncp, const uint32_t *key, const uint32_t *start, uint32_t *cnt,
                          int accumulate) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    uint32_t k = key[p];
    if (k < ncp && (p + 1 == n || key[p + 1] != k)) {
      uint32_t len = (uint32_t)p + 1 - start[k];
      cnt[k] = accumulate ? cnt[k] + len : len;
    }
  }
}
__global__ void k_add_counts(uint32_t n, const uint32_t *a, uint32_t *b) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] += a[i];
}
// first position of each run of equal sorted keys
__global__ void k_seed_runs(long long n, uint32_t ncp, const uint32_t *key, uint32_t *start) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    uint32_t k = key[p];
    if (k < ncp && (p == 0 || key[p - 1] != k)) start[k] = (uint32_t)p;
  }
}

// ---- extremum discs from runs: a row of the vertex (face) grid splits into
// runs of one owner; the disc of an owner is its runs in row-major order, so
// a stable sort of the runs (far fewer than the cells) by owner gives every
// cell's place.
// The row-wise run kernels take one grid row per blockIdx.y and RUN_SPAN
// cells of it per block, RUN_ILP cells per thread (RUN_THREADS apart, so a
// warp's loads stay coalesced) with all of a thread's loads issued before
// any is used: one 4-byte load in flight per thread leaves these streaming
// kernels far below the memory bandwidth.
constexpr int RUN_THREADS = 256, RUN_ILP = 4, RUN_SPAN = RUN_THREADS * RUN_ILP;
static dim3 run_grid(long long n, int w) { return dim3((unsigned)((w + RUN_SPAN - 1) / RUN_SPAN), (unsigned)(n / w)); }

__global__ void __launch_bounds__(RUN_THREADS) k_run_flags(const uint32_t *__restrict__ key, int w, uint32_t *__restrict__ flag) {
  const uint32_t *kr = key + (long long)blockIdx.y * w;
  uint32_t *fr = flag + (long long)blockIdx.y * w;
  const int c0 = blockIdx.x * RUN_SPAN + threadIdx.x;
  uint32_t k[RUN_ILP], kp[RUN_ILP];
#pragma unroll
  for (int q = 0; q < RUN_ILP; ++q) {
    const int c = c0 + q * RUN_THREADS;
    k[q] = c < w ? kr[c] : 0u;
    kp[q] = c > 0 && c < w ? kr[c - 1] : ~k[q];
  }
#pragma unroll
  for (int q = 0; q < RUN_ILP; ++q) {
    const int c = c0 + q * RUN_THREADS;
    if (c < w) fr[c] = k[q] != kp[q] ? 1u : 0u;  // a run starts at a row start or a change of owner
  }
}
// rid: exclusive scan of the start flags (the run of a start cell)
__global__ void __launch_bounds__(RUN_THREADS) k_run_records(const uint32_t *__restrict__ key, int w,
                                                             const uint32_t *__restrict__ rid, uint32_t *__restrict__ rkey,
                                                             uint32_t *__restrict__ rstart, uint32_t *__restrict__ rend) {
  const long long r0 = (long long)blockIdx.y * w;
  const uint32_t *kr = key + r0, *ir = rid + r0;
  const int c0 = blockIdx.x * RUN_SPAN + threadIdx.x;
  uint32_t k[RUN_ILP], kp[RUN_ILP], kn[RUN_ILP], id[RUN_ILP];
#pragma unroll
  for (int q = 0; q < RUN_ILP; ++q) {
    const int c = c0 + q * RUN_THREADS;
    const bool in = c < w;
    k[q] = in ? kr[c] : 0u;
    kp[q] = in && c > 0 ? kr[c - 1] : ~k[q];
    kn[q] = in && c + 1 < w ? kr[c + 1] : ~k[q];
    id[q] = in ? ir[c] : 0u;
  }
#pragma unroll
  for (int q = 0; q < RUN_ILP; ++q) {
    const int c = c0 + q * RUN_THREADS;
    if (c >= w) continue;
    const bool st = k[q] != kp[q];
    const uint32_t r = st ? id[q] : id[q] - 1u;  // the run holding the cell
    if (st) { rkey[r] = k[q]; rstart[r] = (uint32_t)(r0 + c); }
    if (k[q] != kn[q]) rend[r] = (uint32_t)(r0 + c) + 1u;
  }
}
__global__ void k_runs_sorted_len(long long R, uint32_t ncp, const uint32_t *rkey_s, const uint32_t *ridx,
                                  const uint32_t *rstart, const uint32_t *rend, uint32_t *len_s) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < R; i += (long long)gridDim.x * blockDim.x)
    len_s[i] = rkey_s[i] < ncp ? rend[ridx[i]] - rstart[ridx[i]] : 0u;
}
// the first sorted position of each owner's runs (gbase), then each run's place
// in its owner's disc and the owner's count
__global__ void k_runs_group_base(long long R, uint32_t ncp, const uint32_t *rkey_s, const uint32_t *spos, uint32_t *gbase) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < R; i += (long long)gridDim.x * blockDim.x) {
    const uint32_t k = rkey_s[i];
    if (k < ncp && (i == 0 || rkey_s[i - 1] != k)) gbase[k] = spos[i];
  }
}
__global__ void k_runs_place(long long R, uint32_t ncp, const uint32_t *rkey_s, const uint32_t *ridx, const uint32_t *spos,
                             const uint32_t *len_s, const uint32_t *gbase, uint32_t *rpos, uint32_t *cnt) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < R; i += (long long)gridDim.x * blockDim.x) {
    const uint32_t k = rkey_s[i];
    if (k >= ncp) continue;
    rpos[ridx[i]] = spos[i] - gbase[k];
    if (i + 1 == R || rkey_s[i + 1] != k) cnt[k] += spos[i] + len_s[i] - gbase[k];
  }
}
// every owned cell to its owner's disc: off[owner] + its run's place + offset in the run
__global__ void __launch_bounds__(RUN_THREADS) k_runs_scatter(const GridGeom g, int kind, const uint32_t *__restrict__ key,
                                                              int w, uint32_t ncp, const uint32_t *__restrict__ rid,
                                                              const uint32_t *__restrict__ rpos,
                                                              const uint32_t *__restrict__ rstart,
                                                              const uint32_t *__restrict__ off, uint32_t *__restrict__ out) {
  const int jj = blockIdx.y;
  const long long r0 = (long long)jj * w;
  const uint32_t *kr = key + r0, *ir = rid + r0;
  const int c0 = blockIdx.x * RUN_SPAN + threadIdx.x;
  uint32_t k[RUN_ILP], kp[RUN_ILP], id[RUN_ILP];
#pragma unroll
  for (int q = 0; q < RUN_ILP; ++q) {
    const int c = c0 + q * RUN_THREADS;
    const bool in = c < w;
    k[q] = in ? kr[c] : ncp;
    kp[q] = in && c > 0 ? kr[c - 1] : ~k[q];
    id[q] = in ? ir[c] : 0u;
  }
#pragma unroll
  for (int q = 0; q < RUN_ILP; ++q) {
    const int c = c0 + q * RUN_THREADS;
    if (k[q] >= ncp) continue;  // out of the row, or a cell without a disc owner
    const uint32_t r = k[q] != kp[q] ? id[q] : id[q] - 1u;
    out[off[k[q]] + rpos[r] + ((uint32_t)(r0 + c) - rstart[r])] =
        pack_cellid(g.ex0 + g.rx0 + kind + 2 * c, g.ey0 + g.ry0 + kind + 2 * jj);
  }
}
__global__ void k_iota_u32(long long n, uint32_t *a) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] = (uint32_t)i;
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

static cudaError_t hops_attr() {
  static const cudaError_t attr =
      cudaFuncSetAttribute(k_disc_hops, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(HopSmem));
  return attr;
}

// Everything both disc kinds share: the hop structure, the redirections, the
// owner keys of the vertex and face grids.
struct DiscShared {
  DiscArgs a;
  const DiscIO *io;
  long long ncp, nmax, gn[2];
  int gw[2];
  uint32_t *redir, *hop_to, *jseg, *gkey[2], *gval[2];
  uint16_t *hop_len;
  uint16_t *wcode;
};

// One disc kind (0 asc, 1 des) as a sequence of stages on its own stream;
// a stage ends where the host needs a count back.  Two kinds interleave on
// one host thread: while it waits for one kind's count, the other kind's
// launches keep the GPU busy.
struct DiscKind {
  int kind = 0;
  cudaStream_t st = nullptr;
  const DiscShared *sh = nullptr;
  // per-kind scratch (device)
  uint32_t *cnt = nullptr, *slen = nullptr, *sstart = nullptr, *scount = nullptr, *soff = nullptr;
  uint32_t *key = nullptr, *val = nullptr, *kt = nullptr, *vt = nullptr, *kc = nullptr, *mc = nullptr, *cbase = nullptr;
  uint8_t *big = nullptr;
  uint32_t *hbuf = nullptr;  // pinned host counts: [0] runs, [1] seeds, [2] chains, [3..5] totals
  uint32_t *runbuf = nullptr, *chain_buf = nullptr, *wfirst_buf = nullptr;
  uint4 *segs = nullptr, *blocks = nullptr;
  uint32_t *rp = nullptr, *rstart = nullptr;
  uint32_t nrun = 0, ns = 0, nch = 0, tot[2] = {0, 0};
  ChainArgs c{};
  int stage = 0;
  cudaError_t e = cudaSuccess;

  void L(cudaError_t x) { if (e == cudaSuccess) e = x; }
  void release() {
    if (segs) cudaFreeAsync(segs, st);
    if (blocks) cudaFreeAsync(blocks, st);
    if (chain_buf) cudaFreeAsync(chain_buf, st);
    if (runbuf) cudaFreeAsync(runbuf, st);
    if (wfirst_buf) cudaFreeAsync(wfirst_buf, st);
    segs = nullptr; blocks = nullptr; chain_buf = nullptr; runbuf = nullptr; wfirst_buf = nullptr;
  }
  // Runs the next stage; returns true while more stages remain (the caller
  // synchronises the stream before the next one).
  bool step() {
    if (e != cudaSuccess) return false;
    const DiscShared &S = *sh;
    const DiscArgs &a = S.a;
    const DiscIO &io = *S.io;
    const long long ncp = S.ncp, n = S.gn[kind];
    switch (stage++) {
      case 0: {  // runs of one owner along the rows, numbered row-major (gval holds the run ids)
        if (n > 0 && ncp) {
          k_run_flags<<<run_grid(n, S.gw[kind]), RUN_THREADS, 0, st>>>(S.gkey[kind], S.gw[kind], S.gval[kind]);
          DMSC_LAUNCHED(1);
          L(scan_exclusive_u32(S.gval[kind], n, S.gval[kind], soff, st));
          const uint32_t *w[1] = {soff};
          L(read_words(&hbuf[0], w, 1, st));
        } else {
          hbuf[0] = 0;
        }
        return true;
      }
      case 1: {  // the runs in owner order (stable: row-major within an owner); seeds pushed by cancelled extrema
        nrun = hbuf[0];
        const size_t R = nrun;
        L(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * ncp, st));
        if (R) {
          // rkey ridx rstart rend len_s spos rpos + sort scratch (2 R); gbase (ncp)
          L(cudaMallocAsync((void **)&runbuf, sizeof(uint32_t) * (9 * R + (size_t)ncp + 16), st));
          if (e != cudaSuccess) return false;
          uint32_t *rkey = runbuf, *ridx = runbuf + R, *rend = runbuf + 3 * R, *len_s = runbuf + 4 * R;
          uint32_t *spos = runbuf + 5 * R, *tk = runbuf + 7 * R, *tv = runbuf + 8 * R, *gbase = runbuf + 9 * R;
          rstart = runbuf + 2 * R;
          rp = runbuf + 6 * R;
          k_run_records<<<run_grid(n, S.gw[kind]), RUN_THREADS, 0, st>>>(S.gkey[kind], S.gw[kind], S.gval[kind], rkey,
                                                                          rstart, rend);
          k_iota_u32<<<nb(R), 256, 0, st>>>(R, ridx);
          DMSC_LAUNCHED(2);
          L(radix_sort_pairs(rkey, ridx, tk, tv, R, nbits_for(ncp + 1), st));
          k_runs_sorted_len<<<nb(R), 256, 0, st>>>(R, (uint32_t)ncp, rkey, ridx, rstart, rend, len_s);
          DMSC_LAUNCHED(1);
          L(scan_exclusive_u32(len_s, R, spos, nullptr, st));
          k_runs_group_base<<<nb(R), 256, 0, st>>>(R, (uint32_t)ncp, rkey, spos, gbase);
          k_runs_place<<<nb(R), 256, 0, st>>>(R, (uint32_t)ncp, rkey, ridx, spos, len_s, gbase, rp, cnt);
          DMSC_LAUNCHED(2);
        }
        hbuf[1] = 0;
        if (!io.no_cancel) {  // a complex without boundary-cancelable points has no seeds
          k_seed_count<<<nb(ncp), 256, 0, st>>>(a, kind, slen);
          DMSC_LAUNCHED(1);
          L(scan_exclusive_u32(slen, ncp, soff, soff + ncp, st));
          const uint32_t *w[1] = {soff + ncp};
          L(read_words(&hbuf[1], w, 1, st));
          return true;
        }
        return step();  // nothing to wait for
      }
      case 2: {  // chains per saddle
        ns = hbuf[1];
        if ((long long)ns > S.nmax) { e = cudaErrorInvalidValue; return false; }
        if (ns) {
          k_seed_write<<<nb(ncp), 256, 0, st>>>(a, kind, soff, key, val);
          DMSC_LAUNCHED(1);
          L(radix_sort_pairs(key, val, kt, vt, ns, nbits_for(ncp), st));  // stable: pushers stay in index order
        }
        L(cudaMemsetAsync(scount, 0, sizeof(uint32_t) * ncp, st));
        if (ns) {
          k_seed_runs<<<nb(ns), 256, 0, st>>>(ns, (uint32_t)ncp, key, sstart);
          k_run_len<<<nb(ns), 256, 0, st>>>(ns, (uint32_t)ncp, key, sstart, scount, 0);
          DMSC_LAUNCHED(2);
        }
        c.hop_to = S.hop_to; c.hop_len = S.hop_len; c.jseg = S.jseg; c.wcode = S.wcode; c.kind = kind;
        c.kc = kc; c.mc = mc; c.big = big; c.cbase = cbase; c.limit = io.limit;
        k_chain_count<<<nb(ncp), 128, 0, st>>>(a, kind, SeedRuns{val, sstart, scount}, c);
        DMSC_LAUNCHED(1);
        L(scan_exclusive_u32(kc, ncp, cbase, cbase + ncp, st));
        // chain slots: the exact count, or without seeds from cancelled extrema the
        // bound of two chains per saddle (two own seeds, one successor each), with
        // the unused slots zeroed -- saving a synchronisation
        if (ns || !io.no_cancel) {
          const uint32_t *w[1] = {cbase + ncp};
          L(read_words(&hbuf[2], w, 1, st));
          return true;
        }
        hbuf[2] = (uint32_t)std::min<long long>(2 * ncp, 0xFFFFFFF0ll);
        return step();
      }
      case 3: {  // chain lengths, pieces, disc sizes
        nch = hbuf[2];
        c.cap = nch;
        // per chain: cstart csaddle clen cnseg | csegoff (nch + 1)
        L(cudaMallocAsync((void **)&chain_buf, sizeof(uint32_t) * (5ull * nch + 8), st));
        L(cudaMallocAsync((void **)&blocks, sizeof(uint4) * (2 * (size_t)nch + 2), st));
        if (e != cudaSuccess) return false;
        if (!ns && io.no_cancel) {
          L(cudaMemsetAsync(chain_buf, 0, sizeof(uint32_t) * 4ull * nch, st));
          L(cudaMemsetAsync(blocks, 0, sizeof(uint4) * 2ull * nch, st));
        }
        c.cstart = chain_buf; c.csaddle = chain_buf + nch; c.clen = chain_buf + 2 * nch; c.cnseg = chain_buf + 3 * nch;
        c.csegoff = chain_buf + 4 * nch;      // nch + 1
        c.blocks = blocks;
        const SeedRuns sr{val, sstart, scount};
        k_chain_len<<<nb(ncp), 128, 0, st>>>(a, kind, sr, c, slen);
        k_saddle_disc_count<<<nb(ncp), 128, 0, st>>>(a, kind, sr, big, slen, io.limit);
        k_add_counts<<<nb(ncp), 256, 0, st>>>((uint32_t)ncp, slen, cnt);
        DMSC_LAUNCHED(3);
        uint32_t *offs = kind ? io.ddoff : io.adoff;
        L(scan_exclusive_u32(cnt, ncp, offs, offs + ncp, st));
        L(scan_exclusive_u32(c.cnseg, nch, c.csegoff, c.csegoff + nch, st));
        const uint32_t *w[2] = {offs + ncp, c.csegoff + nch};
        L(read_words(&hbuf[3], w, 2, st));
        return true;
      }
      case 4: {  // the cells
        for (int q = 0; q < 2; ++q) tot[q] = hbuf[3 + q];
        uint32_t *offs = kind ? io.ddoff : io.adoff;
        DevBuf<uint32_t> *ob = kind ? io.ddisc : io.adisc;
        L(ob->ensure((size_t)tot[0] + 1, st));
        L(cudaMallocAsync((void **)&segs, sizeof(uint4) * ((size_t)tot[1] + 1), st));
        if (e != cudaSuccess) return false;
        c.segs = segs;
        const SeedRuns sr{val, sstart, scount};
        k_zip_blocks<<<nb(ncp), 128, 0, st>>>(a, c, offs);  // the records the pieces are placed by
        DMSC_LAUNCHED(1);
        if (nch) {
          k_chain_segs<<<nb(nch), 128, 0, st>>>(nch, a, c);
          DMSC_LAUNCHED(1);
        }
        if (S.io->ev_place[kind][0]) L(cudaEventRecord(S.io->ev_place[kind][0], st));
        if (tot[1] && tot[0]) {
          const uint32_t nwin = (uint32_t)(((unsigned long long)tot[0] + WIN - 1) / WIN);
          // the window starts reuse the per-saddle disc lengths (slen, ncp words, read
          // by no later kernel); a complex with fewer critical points than windows allocates
          uint32_t *wfirst = nwin <= (uint32_t)ncp ? slen : nullptr;
          if (!wfirst) L(cudaMallocAsync((void **)&wfirst_buf, sizeof(uint32_t) * nwin, st));
          if (e != cudaSuccess) return false;
          if (!wfirst) wfirst = wfirst_buf;
          k_win_first<<<nb(ncp), 256, 0, st>>>((uint32_t)ncp, offs, nwin, wfirst);
          k_win_place<<<std::min<uint32_t>(nwin, 152u * 8u), WIN_THREADS, 0, st>>>(a, c, wfirst, nwin, ob->p,
                                                                                  (unsigned long long)tot[0]);
          DMSC_LAUNCHED(2);
        }
        k_level0<<<nb(ncp), 128, 0, st>>>(a, kind, sr, c, offs, ob->p);
        k_saddle_disc_write<<<nb(ncp), 128, 0, st>>>(a, kind, sr, big, offs, ob->p);
        DMSC_LAUNCHED(2);
        // between the two events: every saddle disc cell of this kind is written once
        if (S.io->ev_place[kind][1]) L(cudaEventRecord(S.io->ev_place[kind][1], st));
        if (n > 0 && nrun) {  // extremum discs of this kind
          k_runs_scatter<<<run_grid(n, S.gw[kind]), RUN_THREADS, 0, st>>>(a.g, kind, S.gkey[kind], S.gw[kind], (uint32_t)ncp,
                                                                          S.gval[kind], rp, rstart, offs, ob->p);
          DMSC_LAUNCHED(1);
        }
        release();
        return false;
      }
    }
    return false;
  }
};

cudaError_t fill_discs(DiscIO &io, cudaStream_t st) {
  DiscShared S;
  DiscArgs &a = S.a;
  a.g = io.g; a.codes = io.codes; a.labels = io.labels; a.ncp_ds = (uint32_t)io.ncp_ds; a.ncp = (uint32_t)io.ncp;
  a.cellid = io.cellid; a.flags = io.flags; a.pair_idx = io.pair_idx;
  a.aoff = io.aoff; a.asc = io.asc; a.doff = io.doff; a.des = io.des; a.status = io.status;
  S.io = &io;
  const long long ncp = io.ncp;
  S.ncp = ncp;
  const GridGeom &g = io.g;
  const long long nV = (long long)((g.rx1 - g.rx0) / 2 + 1) * ((g.ry1 - g.ry0) / 2 + 1);
  const long long nF = (long long)((g.rx1 - g.rx0) / 2) * ((g.ry1 - g.ry0) / 2);
  const long long nmax = std::max(std::max(nV, nF), std::max(io.nasc, io.ndes)) + 1;
  S.nmax = nmax;
  S.gn[0] = nV; S.gn[1] = nF;
  S.gw[0] = (g.rx1 - g.rx0) / 2 + 1; S.gw[1] = (g.rx1 - g.rx0) / 2;
  const long long nE = 2ll * g.vnx * g.vny;  // edge ids of the ext window
  const bool seeds = !io.no_cancel;
  // shared words: redir (ncp) | owner keys and run ids 2 (nV + nF) | hops 3 nE
  // per kind: cnt slen sstart scount (4 ncp) soff (ncp + 8) kc mc cbase (3 ncp + 1) big (ncp / 4 + 1)
  //           seed sort 4 nmax (only with seeds) | pinned counts
  const size_t kwords = (size_t)ncp * 8 + 16 + (size_t)ncp / 4 + 1 + (seeds ? 4 * (size_t)nmax : 0);
  size_t words = (size_t)ncp + 8 + (size_t)(nV + nF) * 2 + 2 * (size_t)nE + (size_t)nE / 2 + succ_words(g) / 2 + 64 +
                 2 * kwords;
  uint32_t *buf = nullptr;
  cudaError_t e = hops_attr();
  if (e != cudaSuccess) return e;
  if (!io.aux || !io.ev[0] || !io.ev[1]) return cudaErrorInvalidValue;
  e = cudaMallocAsync((void **)&buf, sizeof(uint32_t) * words, st);
  if (e != cudaSuccess) return e;
  uint32_t *p = buf;
  S.redir = p; p += ncp + 8;
  S.gkey[0] = p; p += nV;
  S.gkey[1] = p; p += nF;
  S.gval[0] = p; p += nV;
  S.gval[1] = p; p += nF;
  S.hop_to = p; p += nE;
  S.jseg = p; p += nE;
  S.hop_len = (uint16_t *)p; p += nE / 2 + 1;
  S.wcode = (uint16_t *)p; p += succ_words(g) / 2 + 1;
  DiscKind K[2];
  for (int k = 0; k < 2; ++k) {
    DiscKind &D = K[k];
    D.kind = k;
    D.st = k ? io.aux : st;
    D.sh = &S;
    D.hbuf = io.hcounts + 8 * k;
    D.cnt = p; p += ncp;
    D.slen = p; p += ncp;
    D.sstart = p; p += ncp;
    D.scount = p; p += ncp;
    D.soff = p; p += ncp + 8;
    D.kc = p; p += ncp;
    D.mc = p; p += ncp;
    D.cbase = p; p += ncp + 1;
    D.big = (uint8_t *)p; p += ncp / 4 + 1;
    if (seeds) {
      D.key = p; p += nmax;
      D.val = p; p += nmax;
      D.kt = p; p += nmax;
      D.vt = p; p += nmax;
    }
  }
  auto L = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
  if (ncp) {
    k_redir_init<<<nb(ncp), 256, 0, st>>>((uint32_t)ncp, S.redir);
    DMSC_LAUNCHED(1);
    if (seeds) {
      k_redir_saddles<<<nb(ncp), 256, 0, st>>>(a, S.redir);
      DMSC_LAUNCHED(1);
    }
  }
  if (io.ev_hops[0]) L(cudaEventRecord(io.ev_hops[0], st));
  k_disc_hops<<<dim3(g.ntx, g.nty), HOP_THREADS, sizeof(HopSmem), st>>>(g, io.codes, S.hop_to, S.hop_len, S.jseg,
                                                                        S.wcode, io.status);
  DMSC_LAUNCHED(1);
  if (io.ev_hops[1]) L(cudaEventRecord(io.ev_hops[1], st));
  // extremum discs: vertices -> minima (asc_disc), faces -> maxima (des_disc),
  // grouped by owner with a stable sort (row-major order is the append order)
  if (ncp) {
    k_owner_final<<<nb(ncp), 256, 0, st>>>(a, S.redir, K[0].scount);  // free until the saddle passes
    const int knx = (a.g.rx1 - a.g.rx0) / 2 + 1, kny = (a.g.ry1 - a.g.ry0) / 2 + 1;
    k_disc_keys<<<dim3((unsigned)((knx + KEYS_SPAN - 1) / KEYS_SPAN), (unsigned)kny), KEYS_THREADS, 0, st>>>(
        a, K[0].scount, S.gkey[0], S.gkey[1]);
    DMSC_LAUNCHED(2);
  }
  // the des kind runs on the auxiliary stream once the shared part is done
  L(cudaEventRecord(io.ev[0], st));
  L(cudaStreamWaitEvent(io.aux, io.ev[0], 0));
  if (e == cudaSuccess) {
    bool more[2] = {true, true};
    while (more[0] || more[1])
      for (int k = 0; k < 2; ++k) {
        if (!more[k]) continue;
        more[k] = K[k].step();
        if (more[k] && K[k].e == cudaSuccess) K[k].L(cudaStreamSynchronize(K[k].st));
      }
    for (int k = 0; k < 2; ++k) {
      if (K[k].e != cudaSuccess && e == cudaSuccess) e = K[k].e;
      K[k].release();
    }
    io.nadisc = K[0].tot[0];
    io.nddisc = K[1].tot[0];
  }
  // the caller's stream waits for the auxiliary one
  cudaEventRecord(io.ev[1], io.aux);
  cudaStreamWaitEvent(st, io.ev[1], 0);
  cudaFreeAsync(buf, st);
  if (e == cudaSuccess) e = cudaGetLastError();
  return e;
}

}  // namespace dmsc
