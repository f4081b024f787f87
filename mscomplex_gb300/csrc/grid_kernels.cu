// grid_kernels.cu -- discrete gradient, critical-cell collation and owner
// labels for one piece of a 2D grid, hand-written for sm_103a.
//
// Restates, as data-parallel tile kernels, the reference CPU path
//   GridDataset::assignGradients        dmsc/src/grid_dataset.cpp:1743-1820
//   lowestPairableCoFacet               dmsc/src/grid_dataset.cpp:1314-1373
//   compareCells / ptLt                 grid_dataset.cpp:1519-1536, grid_dataset.h:158-167
//   GridDataset::collateCriticalPoints  grid_dataset.cpp:1822-1832
//   assignCellOwnerExtrema + BFS        grid_dataset.cpp:1376-1427, 1835-1856
//   writeout_connectivity (arcs, fns)   grid_dataset.cpp:1538-1552, 1858-1907
//
// Vertex order.  ptLt compares values, then cell ids lexicographically; a
// vertex key is (order-preserving value bits << 32 | x << 16 | y), so ptLt is
// a 64-bit integer compare.  compareCells sorts cell vertices ASCENDING and
// compares lexicographically; two closed forms replace the sorts:
//   * two faces sharing an edge differ in two vertices each, and ascending-
//     sorted lexicographic order puts first the face holding the smallest
//     vertex of the symmetric difference;
//   * edge e=(P,Q) is >= every edge of a face whose other corners are U
//     (adjacent to P) and W (adjacent to Q) iff U<Q, W<P and min(U,W) <
//     min(P,Q) ("usable" test of lowestPairableCoFacet, :1344-1351).
// The reference's OpenCL kernels (work_ocl) sort cell vertices DESCENDING
// instead (dmsc/resources/assigngradient.cl:40-87); GridGeom::desc selects
// their mirrored closed forms:
//   * two faces sharing an edge are ordered by the LARGEST vertex of their
//     symmetric difference: the face holding it is the larger one;
//   * e=(P,Q) is the largest edge of the face iff the face's largest vertex
//     is P or Q and the other end of e is that vertex's larger neighbour in
//     the face: max(P,Q) > max(U,W) and (P > Q ? Q > U : P > W).
// A vertex pairs with the edge to its lowest lower neighbour in both orders.
// With either order the other steps of work_ocl (complete_pairings, the two
// boundary-pair kernels, pointer-jumping owners, saddle incidences) give the
// cells and owners of the CPU path's steps.
//
// Exactness of the parallel gradient.  The reference pairs cells in row-major
// order and skips cells already marked.  A cell can only be chosen by its
// unique maximal facet, and a vertex v choosing edge e=(w,v) (w its lowest
// usable lower neighbour) makes e fail the usable test for both of its faces
// (the face edge (v,y) beats e), so no cell is both chosen and choosing and
// row-major order never matters: pair(v) = cand(v); pair(e) = its choosing
// vertex, else cand(e); pair(f) = its choosing edge.  ST_PAIR_CONFLICT flags
// the (impossible) mixed case.
//
// Owner labels.  own() of a non-critical vertex is own() of the far end of
// its paired edge; of a non-critical face, own() of the face across its
// paired edge; of a non-critical edge, own() of its pair.  Critical cells own
// themselves; non-critical exterior cells are never reached (LABEL_NONE).
// K1 follows the V-paths by pointer jumping in shared memory inside a tile
// and writes each cell's in-tile terminal; paths leaving the tile end at a
// border cell, and only the border table is resolved globally (K3).
#include <algorithm>

#include "dmsc_common.cuh"
#include "dmsc_internal.h"

namespace dmsc {

__device__ __forceinline__ bool in_rect(const GridGeom &g, int x, int y) {
  return x >= g.rx0 && x <= g.rx1 && y >= g.ry0 && y <= g.ry1;
}
// True if cell (x,y) (relative to ext) has a cofacet inside ext but outside
// rect.  Only meaningful for cells inside rect (isCellExterior, :1708-1711).
__device__ __forceinline__ bool has_ext_cofacet(const GridGeom &g, int x, int y) {
  int kind = (x & 1) | ((y & 1) << 1);
  bool up = (y == g.ry1 && y + 1 <= g.cy), dn = (y == g.ry0 && y >= 1);
  bool lf = (x == g.rx0 && x >= 1), rt = (x == g.rx1 && x + 1 <= g.cx);
  switch (kind) {
    case 0: return up || dn || lf || rt;  // vertex: four edges
    case 1: return up || dn;              // horizontal edge: faces above/below
    case 2: return lf || rt;              // vertical edge: faces left/right
    default: return false;                // face: no cofacets
  }
}
__device__ __forceinline__ int dir_dx(uint32_t d) { return d == DIR_PX ? 1 : (d == DIR_MX ? -1 : 0); }
__device__ __forceinline__ int dir_dy(uint32_t d) { return d == DIR_PY ? 1 : (d == DIR_MY ? -1 : 0); }

// Gradient code of a cell after the pairing (assignGradients steps 2 and 3):
// unmarked rect cells are critical; the boundary rule marks a paired rect
// cell with an exterior cofacet, and its pair, critical as well.
template <bool INTERIOR = false>
__device__ __forceinline__ uint32_t finish_code(const GridGeom &g, bool piece, int x, int y, uint32_t dir, bool paired) {
  bool inr = INTERIOR || in_rect(g, x, y);
  bool crit = inr && !paired;
  if (piece && paired) {
    if (inr && has_ext_cofacet(g, x, y)) crit = true;
    int px = x + dir_dx(dir), py = y + dir_dy(dir);
    if (in_rect(g, px, py) && has_ext_cofacet(g, px, py)) crit = true;
  }
  return (paired ? (CODE_PAIRED | dir) : 0u) | (crit ? CODE_CRIT : 0u);
}

// usable test of an edge (P,Q) for the face whose other corners are U (next
// to P) and W (next to Q)
__device__ __forceinline__ bool usable_face(uint64_t P, uint64_t Q, uint64_t U, uint64_t W) {
  return U < Q && W < P && min(U, W) < min(P, Q);
}
// the same test under the descending order of the OpenCL kernels
__device__ __forceinline__ bool usable_face_desc(uint64_t P, uint64_t Q, uint64_t U, uint64_t W) {
  return max(P, Q) > max(U, W) && (P > Q ? Q > U : P > W);
}
// the smaller of two usable faces of an edge, given each face's two corners
// off the edge: true if face b (the second) is the smaller
__device__ __forceinline__ bool second_face_smaller(bool desc, uint64_t Ua, uint64_t Wa, uint64_t Ub, uint64_t Wb) {
  return desc ? max(Ua, Wa) > max(Ub, Wb) : min(Ub, Wb) < min(Ua, Wa);
}

// pointer-jumping words (uint16): tag in bits 14-15, local cell index below
constexpr uint16_t PJ_PTR = 0x0000, PJ_ROOT = 0x4000, PJ_EXIT = 0x8000, PJ_INVALID = 0xC000;
constexpr uint16_t PJ_TAG = 0xC000, PJ_IDX = 0x0FFF;

// Jumps every pointer of pv[0..TX*TY) and pf[...] to its terminal.  Each
// thread (THREADS per block) keeps a bit mask of its still-active entries.
// Returns true if a path failed to terminate (a cycle).
template <int THREADS>
__device__ __forceinline__ bool pointer_jump(uint16_t *pv, uint16_t *pf) {
  constexpr int n = TX * TY;
  constexpr int PER = 2 * n / THREADS;  // 16 entries per thread with 512 threads, 32 with 256
  static_assert(PER <= 32 && PER * THREADS == 2 * n, "one bit of the mask per entry");
  uint32_t active = 0;
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    int e = threadIdx.x + k * THREADS;
    uint16_t v = e < n ? pv[e] : pf[e - n];
    if ((v & PJ_TAG) == PJ_PTR) active |= 1u << k;
  }
  for (int round = 0; round < 16; ++round) {  // log2(4096) + 4
    if (!__syncthreads_or(active != 0)) return false;
    uint32_t still = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      if (!(active & (1u << k))) continue;
      int e = threadIdx.x + k * THREADS;
      uint16_t *p = e < n ? pv : pf;
      int c = e < n ? e : e - n;
      uint16_t w = p[p[c] & PJ_IDX];
      p[c] = w;
      if ((w & PJ_TAG) == PJ_PTR) still |= 1u << k;
    }
    active = still;
  }
  bool bad = __syncthreads_or(active != 0);
  if (bad) {
#pragma unroll
    for (int k = 0; k < PER; ++k)
      if (active & (1u << k)) {
        int e = threadIdx.x + k * THREADS;
        if (e < n) pv[e] = PJ_INVALID; else pf[e - n] = PJ_INVALID;
      }
    __syncthreads();
  }
  return bad;
}

// Per-row ranks of critical cells inside the tile's row segments.
// rankA[j][i]: critical cells of cell row 2j before vertex i (V,H interleaved);
// rankB[j][i]: same for cell row 2j+1 (Vt,F).  Row totals in cntA/cntB.
__device__ __forceinline__ void row_ranks(const uint32_t (*code)[TX], uint8_t (*rankA)[TX], uint8_t (*rankB)[TX],
                                          uint8_t *cntA, uint8_t *cntB, int w, int h) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = warp; j < h; j += nw) {
    uint32_t c0 = lane < w ? code[j][lane] : 0u;
    uint32_t c1 = lane + 32 < w ? code[j][lane + 32] : 0u;
    uint32_t a0 = ((c0 >> 3) & 1) + ((c0 >> 11) & 1), a1 = ((c1 >> 3) & 1) + ((c1 >> 11) & 1);
    uint32_t b0 = ((c0 >> 19) & 1) + ((c0 >> 27) & 1), b1 = ((c1 >> 19) & 1) + ((c1 >> 27) & 1);
    uint32_t v0 = a0 | (b0 << 16), v1 = a1 | (b1 << 16);  // two 16-bit scans at once
    uint32_t sa0 = v0, sa1 = v1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t0 = __shfl_up_sync(0xffffffffu, sa0, o), t1 = __shfl_up_sync(0xffffffffu, sa1, o);
      if (lane >= o) { sa0 += t0; sa1 += t1; }
    }
    uint32_t t = __shfl_sync(0xffffffffu, sa0, 31);
    uint32_t x0 = sa0 - v0, x1 = t + sa1 - v1;
    rankA[j][lane] = (uint8_t)(x0 & 0xffff);
    rankB[j][lane] = (uint8_t)(x0 >> 16);
    rankA[j][lane + 32] = (uint8_t)(x1 & 0xffff);
    rankB[j][lane + 32] = (uint8_t)(x1 >> 16);
    if (lane == 31) {
      uint32_t tot = t + sa1;
      cntA[j] = (uint8_t)(tot & 0xffff);
      cntB[j] = (uint8_t)(tot >> 16);
    }
  }
}

// ---------------------------------------------------------------------------
// K1: gradient + in-tile tracing + critical counts + border table
// ---------------------------------------------------------------------------
struct GradPhase1 {
  uint64_t key[TY + 3][TX + 3];  // vertex (tx0-1+ii, ty0-1+jj)
  uint8_t candV[TY + 1][TX + 1];
  uint8_t candH[TY + 1][TX];
  uint8_t candVt[TY][TX + 1];
};
struct GradPhase2 {
  uint16_t pv[TY * TX];
  uint16_t pf[TY * TX];
  uint8_t rankA[TY][TX];
  uint8_t rankB[TY][TX];
  uint8_t cntA[TY], cntB[TY];
};
struct GradSmem {
  union {
    GradPhase1 a;
    GradPhase2 b;
  } u;
  uint32_t code[TY][TX];
};

// True if every cell of tile (bx, by), its one-vertex halo and the cells
// paired across its border lie strictly inside rect and away from the grid's
// border: the bounds tests, the grid-border rule of lowestPairableCoFacet and
// the exterior-cofacet rule then all have fixed outcomes.
__device__ __forceinline__ bool interior_tile(const GridGeom &g, int bx, int by) {
  const int tx0 = bx * TX, ty0 = by * TY;
  return tx0 >= 2 && ty0 >= 2 && tx0 + TX + 2 < g.vnx && ty0 + TY + 2 < g.vny && g.rx0 + 4 <= 2 * tx0 &&
         g.ry0 + 4 <= 2 * ty0 && 2 * (tx0 + TX) + 4 <= g.rx1 && 2 * (ty0 + TY) + 4 <= g.ry1;
}

// K1 on tile (bx, by) of one grid, THREADS threads per block; INTERIOR:
// the tile satisfies interior_tile (the same results with fewer tests).
template <int THREADS, bool INTERIOR>
__device__ __forceinline__ void gradient_tile_t(const float *__restrict__ hgt, const GridGeom &g, uint32_t *__restrict__ codes,
                                              uint32_t *__restrict__ terms, uint8_t *__restrict__ rowcnt,
                                              uint64_t *__restrict__ table, uint32_t *__restrict__ status, int bx, int by) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  GradSmem &s = *reinterpret_cast<GradSmem *>(smem_raw);
  GradPhase1 &A = s.u.a;
  const int tx0 = bx * TX, ty0 = by * TY;
  int w, h, wf, hf;
  tile_extent(g, bx, by, 0, w, h);
  tile_extent(g, bx, by, 1, wf, hf);
  if (INTERIOR) { w = h = wf = hf = TX; }
  const bool piece = !INTERIOR && !(g.rx0 == 0 && g.ry0 == 0 && g.rx1 == g.cx && g.ry1 == g.cy);
  auto inr = [&](int x, int y) { return INTERIOR || in_rect(g, x, y); };
  uint32_t st = 0;

  // 1. vertex keys with a 1-vertex halo below/left and 2 above/right
  for (int e = threadIdx.x; e < (TX + 3) * (TY + 3); e += blockDim.x) {
    int jj = e / (TX + 3), ii = e - jj * (TX + 3);
    int vi = tx0 - 1 + ii, vj = ty0 - 1 + jj;
    uint64_t k = 0;
    if (INTERIOR || (vi >= 0 && vi < g.vnx && vj >= 0 && vj < g.vny)) {
      float f = __ldg(hgt + (long long)vj * g.pitch + vi);
      if ((__float_as_uint(f) & 0x7fffffffu) > 0x7f800000u) st |= ST_NAN_INPUT;
      k = ((uint64_t)ord_key(f) << 32) | ((uint32_t)vi << 16) | (uint32_t)vj;
    }
    A.key[jj][ii] = k;
  }
  __syncthreads();
#define KEY(i, j) A.key[(j) + 1][(i) + 1]

  // 2. lowest pairable cofacet of vertices and edges (only rect cells choose)
  for (int e = threadIdx.x; e < (TX + 1) * (TY + 1); e += blockDim.x) {
    int j = e / (TX + 1), i = e - j * (TX + 1);
    int vi = tx0 + i, vj = ty0 + j;
    uint8_t best = CAND_NONE;
    if (INTERIOR || (vi < g.vnx && vj < g.vny && in_rect(g, 2 * vi, 2 * vj))) {
      uint64_t kv = KEY(i, j), bk = kv;
      bool tbv = !INTERIOR && (vi == 0 || vi == g.vnx - 1 || vj == 0 || vj == g.vny - 1);
      bool okv = !tbv || vi == 0 || vi == g.vnx - 1;  // vertical edges usable
      bool okh = !tbv || vj == 0 || vj == g.vny - 1;  // horizontal edges usable
      // cofacet order of getCellCofacets (:1626-1629): up, down, left, right;
      // minimum over lower neighbours (keys are distinct, order is irrelevant)
      if (okv && (INTERIOR || vj + 1 < g.vny)) { uint64_t k = KEY(i, j + 1); if (k < bk) { bk = k; best = DIR_PY; } }
      if (okv && (INTERIOR || vj >= 1)) { uint64_t k = KEY(i, j - 1); if (k < bk) { bk = k; best = DIR_MY; } }
      if (okh && (INTERIOR || vi >= 1)) { uint64_t k = KEY(i - 1, j); if (k < bk) { bk = k; best = DIR_MX; } }
      if (okh && (INTERIOR || vi + 1 < g.vnx)) { uint64_t k = KEY(i + 1, j); if (k < bk) { bk = k; best = DIR_PX; } }
    }
    A.candV[j][i] = best;
  }
  for (int e = threadIdx.x; e < TX * (TY + 1); e += blockDim.x) {
    int j = e / TX, i = e - j * TX;  // H(i,j): P = V(i,j), Q = V(i+1,j)
    int hi = tx0 + i, hj = ty0 + j;
    uint8_t best = CAND_NONE;
    if (INTERIOR || (hi + 1 < g.vnx && hj < g.vny && in_rect(g, 2 * hi + 1, 2 * hj) && hj != 0 && hj != g.vny - 1)) {
      uint64_t P = KEY(i, j), Q = KEY(i + 1, j);
      uint64_t Ua = KEY(i, j + 1), Wa = KEY(i + 1, j + 1), Ub = KEY(i, j - 1), Wb = KEY(i + 1, j - 1);
      bool u0 = g.desc ? usable_face_desc(P, Q, Ua, Wa) : usable_face(P, Q, Ua, Wa);  // cf[0] above
      bool u1 = g.desc ? usable_face_desc(P, Q, Ub, Wb) : usable_face(P, Q, Ub, Wb);  // cf[1] below
      if (u0 && u1) best = second_face_smaller(g.desc, Ua, Wa, Ub, Wb) ? DIR_MY : DIR_PY;
      else if (u0) best = DIR_PY;
      else if (u1) best = DIR_MY;
    }
    A.candH[j][i] = best;
  }
  for (int e = threadIdx.x; e < (TX + 1) * TY; e += blockDim.x) {
    int j = e / (TX + 1), i = e - j * (TX + 1);  // Vt(i,j): P = V(i,j), Q = V(i,j+1)
    int vi = tx0 + i, vj = ty0 + j;
    uint8_t best = CAND_NONE;
    if (INTERIOR || (vi < g.vnx && vj + 1 < g.vny && in_rect(g, 2 * vi, 2 * vj + 1) && vi != 0 && vi != g.vnx - 1)) {
      uint64_t P = KEY(i, j), Q = KEY(i, j + 1);
      uint64_t Ur = KEY(i + 1, j), Wr = KEY(i + 1, j + 1), Ul = KEY(i - 1, j), Wl = KEY(i - 1, j + 1);
      bool u0 = g.desc ? usable_face_desc(P, Q, Ur, Wr) : usable_face(P, Q, Ur, Wr);  // cf[0] right
      bool u1 = g.desc ? usable_face_desc(P, Q, Ul, Wl) : usable_face(P, Q, Ul, Wl);  // cf[1] left
      if (u0 && u1) best = second_face_smaller(g.desc, Ur, Wr, Ul, Wl) ? DIR_MX : DIR_PX;
      else if (u0) best = DIR_PX;
      else if (u1) best = DIR_MX;
    }
    A.candVt[j][i] = best;
  }
#undef KEY
  __syncthreads();

  // 3. final codes of the tile's own cells
  for (int e = threadIdx.x; e < TX * TY; e += blockDim.x) {
    int j = e / TX, i = e - j * TX;
    uint32_t packed = 0;
    if (i < w && j < h) {
      int vi = tx0 + i, vj = ty0 + j, x = 2 * vi, y = 2 * vj;
      uint8_t cv = A.candV[j][i];
      packed |= finish_code<INTERIOR>(g, piece, x, y, cv, cv != CAND_NONE);
      if (INTERIOR || vi + 1 < g.vnx) {  // H(i,j)
        uint32_t d = CAND_NONE;
        if (cv == DIR_PX) d = DIR_MX;
        if (A.candV[j][i + 1] == DIR_MX) d = DIR_PX;
        uint8_t ce = A.candH[j][i];
        if (ce != CAND_NONE) { if (d != CAND_NONE) st |= ST_PAIR_CONFLICT; else d = ce; }
        packed |= finish_code<INTERIOR>(g, piece, x + 1, y, d & 3, d != CAND_NONE) << 8;
      }
      if (INTERIOR || vj + 1 < g.vny) {  // Vt(i,j)
        uint32_t d = CAND_NONE;
        if (cv == DIR_PY) d = DIR_MY;
        if (A.candV[j + 1][i] == DIR_MY) d = DIR_PY;
        uint8_t ce = A.candVt[j][i];
        if (ce != CAND_NONE) { if (d != CAND_NONE) st |= ST_PAIR_CONFLICT; else d = ce; }
        packed |= finish_code<INTERIOR>(g, piece, x, y + 1, d & 3, d != CAND_NONE) << 16;
      }
      if (INTERIOR || (vi + 1 < g.vnx && vj + 1 < g.vny)) {  // F(i,j): chosen by at most one edge
        uint32_t d = CAND_NONE;
        if (A.candH[j][i] == DIR_PY) d = DIR_MY;
        if (A.candH[j + 1][i] == DIR_MY) d = DIR_PY;
        if (A.candVt[j][i] == DIR_PX) d = DIR_MX;
        if (A.candVt[j][i + 1] == DIR_MX) d = DIR_PX;
        packed |= finish_code<INTERIOR>(g, piece, x + 1, y + 1, d & 3, d != CAND_NONE) << 24;
      }
      codes[(long long)vj * g.vnx + vi] = packed;
    }
    s.code[j][i] = packed;
  }
  __syncthreads();  // phase-1 arrays are dead from here on (phase 2 aliases them)
  GradPhase2 &B = s.u.b;

  // 4. in-tile tracing: vertices follow their paired edge to the next vertex,
  //    faces follow their paired edge to the face across it.
  for (int e = threadIdx.x; e < TX * TY; e += blockDim.x) {
    int j = e / TX, i = e - j * TX;
    uint16_t pvv = PJ_INVALID, pff = PJ_INVALID;
    uint32_t c = s.code[j][i];
    if (i < w && j < h) {
      uint32_t cvv = c & 0xff;
      if (cvv & CODE_CRIT) pvv = PJ_ROOT | e;
      else if (inr(2 * (tx0 + i), 2 * (ty0 + j))) {
        uint32_t d = cvv & 3;
        int ni = i + dir_dx(d), nj = j + dir_dy(d);
        pvv = (ni >= 0 && ni < w && nj >= 0 && nj < h) ? (uint16_t)(PJ_PTR | (nj * TX + ni)) : (uint16_t)(PJ_EXIT | e);
      }
    }
    if (i < wf && j < hf) {
      uint32_t cf = c >> 24;
      if (cf & CODE_CRIT) pff = PJ_ROOT | e;
      else if (inr(2 * (tx0 + i) + 1, 2 * (ty0 + j) + 1)) {
        uint32_t d = cf & 3;
        int ni = i + dir_dx(d), nj = j + dir_dy(d);
        pff = (ni >= 0 && ni < wf && nj >= 0 && nj < hf) ? (uint16_t)(PJ_PTR | (nj * TX + ni)) : (uint16_t)(PJ_EXIT | e);
      }
    }
    B.pv[e] = pvv;
    B.pf[e] = pff;
  }
  row_ranks(s.code, B.rankA, B.rankB, B.cntA, B.cntB, w, h);
  if (pointer_jump<THREADS>(B.pv, B.pf)) st |= ST_CYCLE;  // (begins with a barrier)

  // 5. in-tile terminals of every vertex and face, per (cell row, tile) counts
  for (int e = threadIdx.x; e < TX * TY; e += blockDim.x) {
    int j = e / TX, i = e - j * TX;
    if (i < w && j < h) terms[(long long)(ty0 + j) * g.vnx + tx0 + i] = (uint32_t)B.pv[e] | ((uint32_t)B.pf[e] << 16);
  }
  for (int j = threadIdx.x; j < h; j += blockDim.x) {
    int y = 2 * (ty0 + j);
    rowcnt[(long long)y * g.ntx + bx] = B.cntA[j];
    if (y + 1 <= g.cy) rowcnt[(long long)(y + 1) * g.ntx + bx] = B.cntB[j];
  }

  // 6. border table: where each border cell's path ends inside this tile
  long long tile_base = ((long long)by * g.ntx + bx) * SLOTS_PER_TILE;
  for (int e = threadIdx.x; e < 2 * SLOTS_SIDE; e += blockDim.x) {
    int kind = e / SLOTS_SIDE, b = e - kind * SLOTS_SIDE;
    int W = kind ? wf : w, H = kind ? hf : h;
    int i, j;  // invert border_index
    if (b < TX) { i = b; j = 0; }
    else if (b < 2 * TX) { i = b - TX; j = H - 1; }
    else if (b < 2 * TX + TY) { i = 0; j = b - 2 * TX; }
    else { i = W - 1; j = b - 2 * TX - TY; }
    uint64_t entry = BT_INVALID;
    if (W > 0 && H > 0 && i >= 0 && i < W && j >= 0 && j < H && border_index(i, j, W, H) == b) {
      uint16_t p = kind ? B.pf[j * TX + i] : B.pv[j * TX + i];
      int k = p & PJ_IDX, ki = k % TX, kj = k / TX;
      if ((p & PJ_TAG) == PJ_ROOT) {
        int y = 2 * (ty0 + kj) + kind;
        uint32_t rank = kind ? (uint32_t)B.rankB[kj][ki] + ((s.code[kj][ki] >> 19) & 1) : B.rankA[kj][ki];
        entry = BT_ROOT | ((uint64_t)((long long)y * g.ntx + bx + g.gbase) << 8) | rank;
      } else if ((p & PJ_TAG) == PJ_EXIT) {
        uint32_t d = (kind ? (s.code[kj][ki] >> 24) : s.code[kj][ki]) & 3;
        int gi = tx0 + ki + dir_dx(d), gj = ty0 + kj + dir_dy(d);
        if (gi >= 0 && gj >= 0 && gi < g.vnx - kind && gj < g.vny - kind) entry = BT_EXIT | (uint64_t)(border_slot(g, kind, gi, gj) + g.sbase);
        else st |= ST_CYCLE;  // a path leaving the window: never expected
      }
    }
    table[tile_base + kind * SLOTS_SIDE + b] = entry;
  }
  if (st) atomicOr(status, st);
}
template <int THREADS>
__device__ __forceinline__ void gradient_tile(const float *__restrict__ hgt, const GridGeom &g, uint32_t *__restrict__ codes,
                                              uint32_t *__restrict__ terms, uint8_t *__restrict__ rowcnt,
                                              uint64_t *__restrict__ table, uint32_t *__restrict__ status, int bx, int by) {
  if (interior_tile(g, bx, by))
    gradient_tile_t<THREADS, true>(hgt, g, codes, terms, rowcnt, table, status, bx, by);
  else
    gradient_tile_t<THREADS, false>(hgt, g, codes, terms, rowcnt, table, status, bx, by);
}

__global__ void __launch_bounds__(GRAD_THREADS, 3)
k_gradient(const float *__restrict__ hgt, GridGeom g, uint32_t *__restrict__ codes, uint32_t *__restrict__ terms,
           uint8_t *__restrict__ rowcnt, uint64_t *__restrict__ table, uint32_t *__restrict__ status) {
  gradient_tile<GRAD_THREADS>(hgt, g, codes, terms, rowcnt, table, status, blockIdx.x, blockIdx.y);
}

// The grid of batch tile t (tiles numbered grid after grid).
__device__ __forceinline__ int batch_grid_of(const BatchGrid *G, int ngrids, long long t) {
  int lo = 0, hi = ngrids - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (G[mid].tile0 <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// K1 over a batch: a persistent grid of blocks takes (grid, tile) items in
// order; THREADS threads per block (the launch configurations of the batch's
// autotuner).
template <int THREADS>
__global__ void __launch_bounds__(THREADS, 3)
k_gradient_batch(const BatchGrid *__restrict__ G, int ngrids, long long ntiles, uint32_t *__restrict__ status) {
  for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const BatchGrid &B = G[batch_grid_of(G, ngrids, t)];
    const long long lt = t - B.tile0;
    gradient_tile<THREADS>(B.hgt, B.g, B.codes, B.terms, B.rowcnt, B.table, status, (int)(lt % B.g.ntx),
                           (int)(lt / B.g.ntx));
    __syncthreads();  // shared memory is reused by the next item
  }
}

// ---------------------------------------------------------------------------
// K3: resolve the border table.  Every EXIT chain is followed to its root;
// pointers are compressed in place (any value a reader sees is a valid
// pointer along the same chain), so no grid-wide barrier is needed.
// ---------------------------------------------------------------------------
__global__ void k_resolve(uint64_t *table, long long nslots, const uint32_t *__restrict__ offsets, long long nseg,
                          uint32_t *__restrict__ status) {
  for (long long sidx = blockIdx.x * (long long)blockDim.x + threadIdx.x; sidx < nslots;
       sidx += (long long)gridDim.x * blockDim.x) {
    volatile uint64_t *vt = table;
    uint64_t e = vt[sidx];
    long long iter = 0;
    while (bt_tag(e) == BT_EXIT) {
      if ((long long)bt_payload(e) >= nslots) { e = BT_INVALID; atomicOr(status, ST_RESOLVE_LIMIT); break; }
      uint64_t t = vt[bt_payload(e)];
      e = t;
      if (bt_tag(e) == BT_EXIT) vt[sidx] = e;
      if (++iter > nslots) { e = BT_INVALID; atomicOr(status, ST_RESOLVE_LIMIT); break; }
    }
    if (bt_tag(e) == BT_ROOT) {
      uint64_t pl = bt_payload(e);
      if ((long long)(pl >> 8) < nseg) e = BT_FINAL | (uint64_t)(offsets[pl >> 8] + (uint32_t)(pl & 0xff));
      else { e = BT_INVALID; atomicOr(status, ST_RESOLVE_LIMIT); }
    }
    vt[sidx] = e;
  }
}

// ---------------------------------------------------------------------------
// K4: owner labels, critical-point records and saddle arcs.
// ---------------------------------------------------------------------------
struct LabelSmem {
  uint32_t code[TY][TX];
  uint32_t labV[TY][TX];
  uint32_t labF[TY][TX];
  uint8_t rankA[TY][TX];
  uint8_t rankB[TY][TX];
  uint8_t cntA[TY], cntB[TY];
  uint32_t offA[TY], offB[TY];
};

__device__ __forceinline__ uint32_t slot_label(const uint64_t *table, const GridGeom &g, int kind, int gi, int gj) {
  uint64_t e = table[border_slot(g, kind, gi, gj)];
  return bt_tag(e) == BT_FINAL ? (uint32_t)bt_payload(e) : LABEL_NONE;
}
__device__ __forceinline__ float hat(const float *hgt, const GridGeom &g, int vi, int vj) {
  return __ldg(hgt + (long long)vj * g.pitch + vi);
}
// get_cell_fn (:1538-1552): float sum in getCellPoints order, then / count.
__device__ __forceinline__ float cell_fn(const float *hgt, const GridGeom &g, int kind, int vi, int vj) {
  float fn = 0.0f;
  switch (kind) {
    case 0: fn = __fadd_rn(fn, hat(hgt, g, vi, vj)); return __fdiv_rn(fn, 1.0f);
    case 1: fn = __fadd_rn(fn, hat(hgt, g, vi + 1, vj)); fn = __fadd_rn(fn, hat(hgt, g, vi, vj)); return __fdiv_rn(fn, 2.0f);
    case 2: fn = __fadd_rn(fn, hat(hgt, g, vi, vj + 1)); fn = __fadd_rn(fn, hat(hgt, g, vi, vj)); return __fdiv_rn(fn, 2.0f);
    default:
      fn = __fadd_rn(fn, hat(hgt, g, vi + 1, vj + 1));
      fn = __fadd_rn(fn, hat(hgt, g, vi + 1, vj));
      fn = __fadd_rn(fn, hat(hgt, g, vi, vj));
      fn = __fadd_rn(fn, hat(hgt, g, vi, vj + 1));
      return __fdiv_rn(fn, 4.0f);
  }
}

// K4 on tile (bx, by) of one grid.
__device__ __forceinline__ void labels_tile(const uint32_t *__restrict__ codes, const uint32_t *__restrict__ terms,
                                            const float *__restrict__ hgt, const GridGeom &g,
                                            const uint32_t *__restrict__ offsets, const uint64_t *__restrict__ table,
                                            uint4 *__restrict__ labels, const CpOut &cp, uint32_t *__restrict__ status,
                                            int bx, int by) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  LabelSmem &s = *reinterpret_cast<LabelSmem *>(smem_raw);
  const int tx0 = bx * TX, ty0 = by * TY;
  int w, h, wf, hf;
  tile_extent(g, bx, by, 0, w, h);
  tile_extent(g, bx, by, 1, wf, hf);
  uint32_t st = 0;

  for (int e = threadIdx.x; e < TX * TY; e += blockDim.x) {
    int j = e / TX, i = e - j * TX;
    s.code[j][i] = (i < w && j < h) ? codes[(long long)(ty0 + j) * g.vnx + tx0 + i] : 0u;
  }
  for (int j = threadIdx.x; j < h; j += blockDim.x) {
    int y = 2 * (ty0 + j);
    s.offA[j] = offsets[(long long)y * g.ntx + bx];
    s.offB[j] = (y + 1 <= g.cy) ? offsets[(long long)(y + 1) * g.ntx + bx] : 0u;
  }
  __syncthreads();
  row_ranks(s.code, s.rankA, s.rankB, s.cntA, s.cntB, w, h);
  __syncthreads();

  // vertex / face labels from the in-tile terminals written by K1
  for (int e = threadIdx.x; e < TX * TY; e += blockDim.x) {
    int j = e / TX, i = e - j * TX;
    uint32_t lv = LABEL_NONE, lf = LABEL_NONE;
    if (i < w && j < h) {
      uint32_t t2 = terms[(long long)(ty0 + j) * g.vnx + tx0 + i];
      uint16_t p = (uint16_t)(t2 & 0xffff);
      int k = p & PJ_IDX, ki = k % TX, kj = k / TX;
      if ((p & PJ_TAG) == PJ_ROOT) lv = s.offA[kj] + s.rankA[kj][ki];
      else if ((p & PJ_TAG) == PJ_EXIT) lv = slot_label(table, g, 0, tx0 + ki, ty0 + kj);
      if (i < wf && j < hf) {
        p = (uint16_t)(t2 >> 16);
        k = p & PJ_IDX; ki = k % TX; kj = k / TX;
        if ((p & PJ_TAG) == PJ_ROOT) lf = s.offB[kj] + s.rankB[kj][ki] + ((s.code[kj][ki] >> 19) & 1);
        else if ((p & PJ_TAG) == PJ_EXIT) lf = slot_label(table, g, 1, tx0 + ki, ty0 + kj);
      }
    }
    s.labV[j][i] = lv;
    s.labF[j][i] = lf;
  }
  __syncthreads();

  for (int e = threadIdx.x; e < TX * TY; e += blockDim.x) {
    int j = e / TX, i = e - j * TX;
    if (i >= w || j >= h) continue;
    const int vi = tx0 + i, vj = ty0 + j, x = 2 * vi, y = 2 * vj;
    const uint32_t c = s.code[j][i];
    // neighbour labels that may live in the next tile (that tile's border cells)
    auto labV_at = [&](int ii, int jj) -> uint32_t {
      if (ii >= 0 && ii < w && jj >= 0 && jj < h) return s.labV[jj][ii];
      return slot_label(table, g, 0, tx0 + ii, ty0 + jj);
    };
    auto labF_at = [&](int ii, int jj) -> uint32_t {
      if (ii >= 0 && ii < wf && jj >= 0 && jj < hf) return s.labF[jj][ii];
      return slot_label(table, g, 1, tx0 + ii, ty0 + jj);
    };
    uint32_t L[4];
    L[0] = s.labV[j][i];
    L[3] = s.labF[j][i];
    uint32_t idxH = s.offA[j] + s.rankA[j][i] + ((c >> 3) & 1);
    uint32_t idxVt = s.offB[j] + s.rankB[j][i];
    // H(i,j)
    L[1] = LABEL_NONE;
    uint32_t ch = (c >> 8) & 0xff;
    if (vi + 1 < g.vnx) {
      if (ch & CODE_CRIT) L[1] = idxH;
      else if ((ch & CODE_PAIRED) && in_rect(g, x + 1, y)) {
        switch (ch & 3) {
          case DIR_MX: L[1] = s.labV[j][i]; break;
          case DIR_PX: L[1] = labV_at(i + 1, j); break;
          case DIR_PY: L[1] = labF_at(i, j); break;
          default: L[1] = labF_at(i, j - 1); break;
        }
      }
    }
    // Vt(i,j)
    L[2] = LABEL_NONE;
    uint32_t cvt = (c >> 16) & 0xff;
    if (vj + 1 < g.vny) {
      if (cvt & CODE_CRIT) L[2] = idxVt;
      else if ((cvt & CODE_PAIRED) && in_rect(g, x, y + 1)) {
        switch (cvt & 3) {
          case DIR_MY: L[2] = s.labV[j][i]; break;
          case DIR_PY: L[2] = labV_at(i, j + 1); break;
          case DIR_PX: L[2] = labF_at(i, j); break;
          default: L[2] = labF_at(i - 1, j); break;
        }
      }
    }
    labels[(long long)vj * g.vnx + vi] = make_uint4(L[0], L[1], L[2], L[3]);

    // critical-point records
    if (!(c & 0x08080808u)) continue;
#pragma unroll
    for (int kind = 0; kind < 4; ++kind) {
      uint32_t cc = (c >> (8 * kind)) & 0xff;
      if (!(cc & CODE_CRIT)) continue;
      int cxr = x + (kind & 1), cyr = y + (kind >> 1);
      uint32_t k = kind == 0 ? L[0] : kind == 1 ? idxH : kind == 2 ? idxVt : L[3];
      if ((long long)k >= cp.cap) { st |= ST_CAPACITY; continue; }
      cp.cellid[k] = pack_cellid(g.ex0 + cxr, g.ey0 + cyr);
      cp.fn[k] = cell_fn(hgt, g, kind, vi, vj);
      cp.flags[k] = (cc & CODE_PAIRED) ? 1 : 0;
      if (cc & CODE_PAIRED) {
        uint32_t d = cc & 3;
        cp.pair_cell[k] = pack_cellid(g.ex0 + cxr + dir_dx(d), g.ey0 + cyr + dir_dy(d));
      }
      if (kind == 1 || kind == 2) {
        // facets f[0..1] and ext-filtered cofacets (writeout_connectivity, :1876-1898)
        uint32_t f0, f1, q0 = LABEL_NONE, q1 = LABEL_NONE;
        if (kind == 1) {
          f0 = labV_at(i + 1, j); f1 = L[0];
          if (vj + 1 < g.vny) q0 = labF_at(i, j);
          if (vj >= 1) q1 = labF_at(i, j - 1);
        } else {
          f0 = labV_at(i, j + 1); f1 = L[0];
          if (vi + 1 < g.vnx) q0 = labF_at(i, j);
          if (vi >= 1) q1 = labF_at(i - 1, j);
        }
        uint32_t dlo = min(f0, f1), dhi = max(f0, f1), alo = min(q0, q1), ahi = max(q0, q1);
        cp.des2[2 * k] = dlo; cp.des2[2 * k + 1] = dhi;
        cp.asc2[2 * k] = alo; cp.asc2[2 * k + 1] = ahi;
        cp.dcnt[k] = (dlo != LABEL_NONE) + (dhi != LABEL_NONE);
        cp.acnt[k] = (alo != LABEL_NONE) + (ahi != LABEL_NONE);
        if (dlo != LABEL_NONE && dlo < cp.cap) atomicAdd(cp.acnt + dlo, 1u);
        if (dhi != LABEL_NONE && dhi < cp.cap) atomicAdd(cp.acnt + dhi, 1u);
        if (alo != LABEL_NONE && alo < cp.cap) atomicAdd(cp.dcnt + alo, 1u);
        if (ahi != LABEL_NONE && ahi < cp.cap) atomicAdd(cp.dcnt + ahi, 1u);
      } else {
        cp.des2[2 * k] = cp.des2[2 * k + 1] = LABEL_NONE;
        cp.asc2[2 * k] = cp.asc2[2 * k + 1] = LABEL_NONE;
      }
    }
  }
  if (st) atomicOr(status, st);
}

__global__ void __launch_bounds__(GRAD_THREADS, 3)
k_labels(const uint32_t *__restrict__ codes, const uint32_t *__restrict__ terms, const float *__restrict__ hgt, GridGeom g,
         const uint32_t *__restrict__ offsets, const uint64_t *__restrict__ table, uint4 *__restrict__ labels,
         CpOut cp, uint32_t *__restrict__ status) {
  labels_tile(codes, terms, hgt, g, offsets, table, labels, cp, status, blockIdx.x, blockIdx.y);
}

// K4 over a batch; cp indices (and so labels) are batch-wide.
template <int THREADS>
__global__ void __launch_bounds__(THREADS, 3)
k_labels_batch(const BatchGrid *__restrict__ G, int ngrids, long long ntiles, CpOut cp, uint32_t *__restrict__ status) {
  for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const BatchGrid &B = G[batch_grid_of(G, ngrids, t)];
    const long long lt = t - B.tile0;
    labels_tile(B.codes, B.terms, B.hgt, B.g, B.offsets, B.table, B.labels, cp, status, (int)(lt % B.g.ntx),
                (int)(lt / B.g.ntx));
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
size_t grad_smem_bytes() { return sizeof(GradSmem); }
size_t label_smem_bytes() { return sizeof(LabelSmem); }

cudaError_t launch_gradient(const float *hgt, const GridGeom &g, uint32_t *codes, uint32_t *terms, uint8_t *rowcnt,
                            uint64_t *table, uint32_t *status, cudaStream_t st) {
  // once per process (thread-safe static initialisation)
  static const cudaError_t attr = cudaFuncSetAttribute(k_gradient, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(GradSmem));
  if (attr != cudaSuccess) return attr;
  dim3 grid(g.ntx, g.nty);
  k_gradient<<<grid, GRAD_THREADS, sizeof(GradSmem), st>>>(hgt, g, codes, terms, rowcnt, table, status);
  DMSC_LAUNCHED(1);
  return cudaGetLastError();
}

cudaError_t launch_resolve(uint64_t *table, long long nslots, const uint32_t *offsets, long long nseg, uint32_t *status,
                           cudaStream_t st) {
  int threads = 256;
  long long blocks = (nslots + threads - 1) / threads;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  k_resolve<<<(unsigned)blocks, threads, 0, st>>>(table, nslots, offsets, nseg, status);
  DMSC_LAUNCHED(1);
  return cudaGetLastError();
}

cudaError_t launch_labels(const uint32_t *codes, const uint32_t *terms, const float *hgt, const GridGeom &g,
                          const uint32_t *offsets, const uint64_t *table, uint4 *labels, const CpOut &cp,
                          uint32_t *status, cudaStream_t st) {
  // once per process (thread-safe static initialisation)
  static const cudaError_t attr = cudaFuncSetAttribute(k_labels, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(LabelSmem));
  if (attr != cudaSuccess) return attr;
  dim3 grid(g.ntx, g.nty);
  k_labels<<<grid, GRAD_THREADS, sizeof(LabelSmem), st>>>(codes, terms, hgt, g, offsets, table, labels, cp, status);
  DMSC_LAUNCHED(1);
  return cudaGetLastError();
}

// The persistent batch kernels' launch: `threads` per block (256 or 512) and
// blocks_per_sm resident blocks per SM (1 to 3; the shared memory of a 64x64
// tile allows 3) over the device's SMs.
static long long persistent_blocks(long long ntiles, int blocks_per_sm) {
  static const int sms = [] {
    int dev = 0, n = 152;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      n = 152;
    return n;
  }();
  const int bps = blocks_per_sm < 1 ? 1 : blocks_per_sm > 3 ? 3 : blocks_per_sm;
  return std::min<long long>(ntiles, (long long)sms * bps);
}

template <int THREADS>
static cudaError_t gradient_batch_t(const BatchGrid *grids, int ngrids, long long ntiles, int bps, uint32_t *status,
                                    cudaStream_t st) {
  static const cudaError_t attr =  // once per instantiation (thread-safe static initialisation)
      cudaFuncSetAttribute(k_gradient_batch<THREADS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(GradSmem));
  if (attr != cudaSuccess) return attr;
  k_gradient_batch<THREADS><<<(unsigned)persistent_blocks(ntiles, bps), THREADS, sizeof(GradSmem), st>>>(grids, ngrids,
                                                                                                      ntiles, status);
  DMSC_LAUNCHED(1);
  return cudaGetLastError();
}

template <int THREADS>
static cudaError_t labels_batch_t(const BatchGrid *grids, int ngrids, long long ntiles, const CpOut &cp, int bps,
                                  uint32_t *status, cudaStream_t st) {
  static const cudaError_t attr =
      cudaFuncSetAttribute(k_labels_batch<THREADS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(LabelSmem));
  if (attr != cudaSuccess) return attr;
  k_labels_batch<THREADS><<<(unsigned)persistent_blocks(ntiles, bps), THREADS, sizeof(LabelSmem), st>>>(grids, ngrids,
                                                                                                     ntiles, cp, status);
  DMSC_LAUNCHED(1);
  return cudaGetLastError();
}

cudaError_t launch_gradient_batch(const BatchGrid *grids, int ngrids, long long ntiles, uint32_t *status, cudaStream_t st,
                                  BatchLaunch cfg) {
  if (ntiles <= 0) return cudaSuccess;
  return cfg.threads == 256 ? gradient_batch_t<256>(grids, ngrids, ntiles, cfg.blocks_per_sm, status, st)
                            : gradient_batch_t<GRAD_THREADS>(grids, ngrids, ntiles, cfg.blocks_per_sm, status, st);
}

cudaError_t launch_labels_batch(const BatchGrid *grids, int ngrids, long long ntiles, const CpOut &cp, uint32_t *status,
                                cudaStream_t st, BatchLaunch cfg) {
  if (ntiles <= 0) return cudaSuccess;
  return cfg.threads == 256 ? labels_batch_t<256>(grids, ngrids, ntiles, cp, cfg.blocks_per_sm, status, st)
                            : labels_batch_t<GRAD_THREADS>(grids, ngrids, ntiles, cp, cfg.blocks_per_sm, status, st);
}

}  // namespace dmsc
