// merge_graph.cuh -- a complex being merged, as a mutable graph (msc_graph.cuh)
// plus a table from cell id to critical-point index over the box of its
// cells, standing in for m_id_cp_map (std::map), and the reference's two
// merges restated step by step on it: GridMSComplex::merge_up and merge_down
// (dmsc/src/grid_mscomplex.cpp:7-322), including its std::map::operator[]
// (a missing key is inserted with index 0).  Shared by the level-at-a-time
// merges (merge.cu) and the parallel merges (merge_par.cu), which run the
// parts that must stay sequential (the cancellations along the shared
// boundary) through these same functions.
#pragma once
#include "dmsc_common.cuh"
#include "msc_graph.cuh"

namespace dmsc {

constexpr uint32_t NO_CP = 0xFFFFFFFFu;

struct CRect {  // rect_t (dmsc/include/rectangle_complex.h:108-308), global cell coordinates
  int l, b, r, t;
  __host__ __device__ bool contains(int x, int y) const { return x >= l && y >= b && x <= r && y <= t; }
  __host__ __device__ bool interior(int x, int y) const { return x > l && y > b && x < r && y < t; }
  __host__ __device__ bool boundary(int x, int y) const { return contains(x, y) && !interior(x, y); }
};

struct MGraph {
  Graph G;           // G.ncp is the current number of critical points
  float *fn;
  uint32_t cap;      // capacity of the per-cp arrays
  // m_id_cp_map: critical-point index of every cell of the box
  // [tx0, tx0 + tw) x [ty0, ty0 + th) (cell coordinates), NO_CP where none
  uint32_t *tab;
  int tx0, ty0, tw, th;
  CRect rect, ext;

  __host__ __device__ long long slot(uint32_t cid) const {
    const int x = (int)(cid & 0xffffu) - tx0, y = (int)(cid >> 16) - ty0;
    if (x < 0 || y < 0 || x >= tw || y >= th) return -1;
    return (long long)y * tw + x;
  }
  __host__ __device__ uint32_t find(uint32_t cid) const {
    const long long s = slot(cid);
    return s < 0 ? NO_CP : tab[s];
  }
  __host__ __device__ bool put(uint32_t cid, uint32_t idx) {
    const long long s = slot(cid);
    if (s < 0) { G.fail = true; return false; }  // outside the box the complex was given
    tab[s] = idx;
    return true;
  }
  // std::map::operator[]: inserts index 0 for a missing key
  __host__ __device__ uint32_t at(uint32_t cid) {
    uint32_t i = find(cid);
    if (i != NO_CP) return i;
    put(cid, 0);
    return 0;
  }
  // shallow_replicate_cp (grid_mscomplex.cpp:7-22): flags copied, pair unset
  __host__ __device__ uint32_t add(uint32_t cid, uint8_t fl, float f) {
    if (G.ncp >= cap) { G.fail = true; return 0; }
    uint32_t k = G.ncp++;
    G.cellid[k] = cid;
    G.flags[k] = fl & (F_CANCELLED | F_STRANG | F_BCANCEL);
    G.pair_idx[k] = NO_CP;
    fn[k] = f;
    for (int w = 0; w < 2; ++w) {
      G.L.off[2 * k + w] = 0; G.L.nrun[2 * k + w] = 0; G.L.cap[2 * k + w] = 0; G.L.total[2 * k + w] = 0;
    }
    put(cid, k);
    return k;
  }
};

__host__ __device__ __forceinline__ void set_status(uint32_t *s, uint32_t v) {
#ifdef __CUDA_ARCH__
  atomicOr(s, v);
#else
  *s |= v;
#endif
}

__host__ __device__ __forceinline__ int px_(uint32_t c) { return (int16_t)(c & 0xffff); }
__host__ __device__ __forceinline__ int py_(uint32_t c) { return (int16_t)(c >> 16); }

inline __host__ __device__ void merge_up_cancel(MGraph &out, CRect ixn, uint32_t *status);

// merge_up (grid_mscomplex.cpp:24-156); out starts empty.
inline __host__ __device__ void merge_up_one(MGraph *in[2], MGraph &out, CRect ixn, uint32_t *status) {
  // union of the critical points (:56-75)
  for (int i = 0; i < 2; ++i) {
    MGraph &M = *in[i];
    for (uint32_t j = 0; j < M.G.ncp && !out.G.fail; ++j) {
      uint32_t cid = M.G.cellid[j];
      if (i == 1 && out.find(cid) != NO_CP) continue;
      if (M.G.flags[j] & F_CANCELLED) continue;
      out.add(cid, M.G.flags[j], M.fn[j]);
    }
  }
  // connectivity (:77-122)
  for (int i = 0; i < 2 && !out.G.fail; ++i) {
    MGraph &M = *in[i];
    for (uint32_t j = 0; j < M.G.ncp && !out.G.fail; ++j) {
      if (M.G.flags[j] & F_CANCELLED) continue;
      uint32_t cid = M.G.cellid[j];
      uint32_t d = out.find(cid);
      if (d == NO_CP) { set_status(status, ST_INVARIANT); return; }
      if (M.G.flags[j] & F_BCANCEL) {
        uint32_t p = M.G.pair_idx[j];
        if (p >= M.G.ncp) { set_status(status, ST_INVARIANT); return; }
        out.G.pair_idx[d] = out.at(M.G.cellid[p]);
      }
      bool cmn = ixn.contains(px_(cid), py_(cid)) && i == 1;
      for (int k = 0; k < 2; ++k) {
        uint32_t l = 2 * j + k;
        for (uint32_t q = 0; q < M.G.L.nrun[l]; ++q) {
          uint2 r = M.G.runs(l)[q];
          uint32_t cc = M.G.cellid[r.x];
          if (cmn && ixn.contains(px_(cc), py_(cc))) continue;
          if (M.G.flags[r.x] & F_CANCELLED) continue;
          out.G.insert(2 * d + k, out.at(cc), r.y);
        }
      }
    }
  }
  merge_up_cancel(out, ixn, status);
}

// One cell (x, y) of merge_up's boundary loop (:125-152); false where the
// loop stops on a reference logic_error condition (status set).
inline __host__ __device__ bool merge_up_cell(MGraph &out, int x, int y, uint32_t *status) {
  uint32_t si = out.find(pack_cellid(x, y));
  if (si == NO_CP) { set_status(status, ST_INVARIANT); return false; }  // "missing common bndry cp"
  if ((out.G.flags[si] & F_CANCELLED) || !(out.G.flags[si] & F_BCANCEL)) return true;
  uint32_t pi = out.G.pair_idx[si];
  if (pi >= out.G.ncp) { set_status(status, ST_INVARIANT); return false; }
  uint32_t p = out.G.cellid[pi];
  if (!out.rect.interior(x, y) && !out.ext.boundary(x, y)) return true;
  if (!out.rect.interior(px_(p), py_(p)) && !out.ext.boundary(px_(p), py_(p))) return true;
  uint32_t a = si, b = pi;
  out.G.cancel_pairs(a, b);
  return true;
}

// merge_up's cancellation along the shared boundary (:124-153), row-major
inline __host__ __device__ void merge_up_cancel(MGraph &out, CRect ixn, uint32_t *status) {
  for (int y = ixn.b; y <= ixn.t && !out.G.fail; ++y)
    for (int x = ixn.l; x <= ixn.r && !out.G.fail; ++x)
      if (!merge_up_cell(out, x, y, status)) return;
}

// merge_down (grid_mscomplex.cpp:158-322) of parent P into one child C; the
// boundary uncancellation on P is done once by the caller.
// The cancelable critical points of the parent (:207-281), in index order.
inline __host__ __device__ void merge_down_loop1(MGraph &P, MGraph &C, uint32_t *status) {
  Graph &G = C.G;
  for (uint32_t j = 0; j < P.G.ncp && !G.fail; ++j) {
    if (P.G.flags[j] & F_CANCELLED) { set_status(status, ST_INVARIANT); return; }  // "all cps ought to be uncancelled"
    if (!(P.G.flags[j] & F_BCANCEL)) continue;
    uint32_t sp = P.G.pair_idx[j];
    if (sp >= P.G.ncp) { set_status(status, ST_INVARIANT); return; }
    uint32_t scid = P.G.cellid[j], spcid = P.G.cellid[sp];
    bool s_in = C.find(scid) != NO_CP, sp_in = C.find(spcid) != NO_CP;
    if (!s_in && !sp_in) continue;
    if (!s_in) C.add(scid, P.G.flags[j], P.fn[j]);
    if (!sp_in) C.add(spcid, P.G.flags[sp], P.fn[sp]);
    uint32_t di = C.at(scid);
    if (!s_in || !sp_in || !(G.flags[di] & F_BCANCEL)) {
      uint32_t dpi = C.at(spcid);
      G.flags[di] |= F_BCANCEL;
      G.flags[dpi] |= F_BCANCEL;
      G.pair_idx[di] = dpi;
      G.pair_idx[dpi] = di;
    }
    for (int k = 0; k < 2 && !G.fail; ++k) {
      uint32_t l = 2 * j + k;
      unsigned long long n = 0;
      for (uint32_t q = 0; q < P.G.L.nrun[l]; ++q) {
        uint2 r = P.G.runs(l)[q];
        if (P.G.flags[r.x] & F_BCANCEL) { set_status(status, ST_INVARIANT); return; }  // "only non cancellable cps"
        uint32_t cc = P.G.cellid[r.x];
        if (C.find(cc) == NO_CP) C.add(cc, P.G.flags[r.x], P.fn[r.x]);
        if (n >= G.tmp_cap) { G.fail = true; return; }
        G.tmp[n++] = make_uint2(C.at(cc), r.y);
      }
      G.set_list_from_tmp(2 * di + k, n);
    }
  }
}

inline __host__ __device__ void merge_down_child(MGraph &P, MGraph &C, uint32_t *status) {
  merge_down_loop1(P, C, status);
  Graph &G = C.G;
  // the other critical points the child holds (:283-320)
  for (uint32_t j = 0; j < P.G.ncp && !G.fail; ++j) {
    if (P.G.flags[j] & F_BCANCEL) continue;
    uint32_t di = C.find(P.G.cellid[j]);
    if (di == NO_CP) continue;
    for (int k = 0; k < 2 && !G.fail; ++k) {
      uint32_t l = 2 * j + k;
      unsigned long long n = 0;
      for (uint32_t q = 0; q < P.G.L.nrun[l]; ++q) {
        uint2 r = P.G.runs(l)[q];
        uint32_t ci = C.find(P.G.cellid[r.x]);
        if (ci == NO_CP) continue;
        if (n >= G.tmp_cap) { G.fail = true; return; }
        G.tmp[n++] = make_uint2(ci, r.y);
      }
      G.set_list_from_tmp(2 * di + k, n);
    }
  }
}

// merge_down's uncancellation along the shared boundary of the children, in
// reverse row-major order (grid_mscomplex.cpp:172-201), done once on the parent.
inline __host__ __device__ void merge_down_boundary(MGraph &P, CRect ixn, uint32_t *status) {
  for (int y = ixn.t; y >= ixn.b && !P.G.fail; --y)
    for (int x = ixn.r; x >= ixn.l && !P.G.fail; --x) {
      uint32_t si = P.find(pack_cellid(x, y));
      if (si == NO_CP) { set_status(status, ST_INVARIANT); return; }
      if (!(P.G.flags[si] & F_CANCELLED)) continue;
      uint32_t pi = P.G.pair_idx[si];
      if (pi >= P.G.ncp) { set_status(status, ST_INVARIANT); return; }
      uint32_t p = P.G.cellid[pi];
      if (!P.rect.interior(x, y) && !P.ext.boundary(x, y)) continue;
      if (!P.rect.interior(px_(p), py_(p)) && !P.ext.boundary(px_(p), py_(p))) continue;
      if (!P.G.uncancel_pairs(si, pi)) { set_status(status, ST_INVARIANT); return; }
    }
}

}  // namespace dmsc
