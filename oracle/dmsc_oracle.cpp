// dmsc_oracle.cpp -- CPU ORACLE. TEST INFRASTRUCTURE ONLY.
//
// A plain C++ restatement of the reference's CPU path for the 2D grid
// Morse-Smale complex (nithins/mscomplex, dmsc/).  It exists to CHECK the CUDA
// implementation in mscomplex_gb300/ and to serve as the timed CPU baseline; it
// is never linked into, loaded by, or called from the product path.
//
// PARITY UNPINNED: the reference ships no tests, fixtures or golden vectors,
// and it cannot be compiled in this environment (it needs Boost, Qt4, OpenCL
// and the un-vendored glapp_framework submodule), so this restatement is not
// checked against reference outputs.  It follows the reference source line by
// line (citations below are path:line within the reference project) and keeps
// its data structures (std::map, std::multiset, std::queue BFS, std::sort in
// compareCells, std::priority_queue with the reference comparator) so that the
// result -- including heap tie order -- is the reference's, and so that its
// timing is representative of the reference's CPU path.
//
// Known reference quirks that are kept on purpose:
//   * compareCells sorts cell vertices ASCENDING (dmsc/src/grid_dataset.cpp:1530)
//   * persistence_comparator_t reads c3,c4 from p1 (dmsc/src/grid_mscomplex.cpp:358-359)
//   * simplify starts max_val at numeric_limits<float>::min() (grid_mscomplex.cpp:399)
//   * getCellPairId never throws (precedence bug, grid_dataset.cpp:1513)
//   * merge_up uses the lexicographic std::min/max of points (grid_mscomplex.cpp:43-49)
// Unpinned third-party semantics (glapp_framework two_tuple_t, not vendored):
//   operator< on cell ids is taken as lexicographic (x, then y).

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <queue>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

namespace orc {

typedef int16_t coord_t;
typedef unsigned int uint;

// two_tuple_t stand-in: rectangle_complex.h:57-106 (point_def), default (-1,-1) :69
struct cellid_t {
  coord_t v[2];
  cellid_t() { v[0] = -1; v[1] = -1; }
  cellid_t(int x, int y) { v[0] = (coord_t)x; v[1] = (coord_t)y; }
  coord_t &operator[](int i) { return v[i]; }
  const coord_t &operator[](int i) const { return v[i]; }
  bool operator<(const cellid_t &o) const { return v[0] < o.v[0] || (v[0] == o.v[0] && v[1] < o.v[1]); }
  bool operator>(const cellid_t &o) const { return o < *this; }
  bool operator==(const cellid_t &o) const { return v[0] == o.v[0] && v[1] == o.v[1]; }
  bool operator!=(const cellid_t &o) const { return !(*this == o); }
};

// rectangle_complex.h:108-308
struct rect_t {
  cellid_t bl, tr;
  rect_t() {}
  rect_t(int sx, int sy, int ex, int ey) {
    bl[0] = (coord_t)std::min(sx, ex); bl[1] = (coord_t)std::min(sy, ey);
    tr[0] = (coord_t)std::max(sx, ex); tr[1] = (coord_t)std::max(sy, ey);
  }
  rect_t(const cellid_t &p1, const cellid_t &p2) {
    bl[0] = std::min(p1[0], p2[0]); bl[1] = std::min(p1[1], p2[1]);
    tr[0] = std::max(p1[0], p2[0]); tr[1] = std::max(p1[1], p2[1]);
  }
  bool isInInterior(const cellid_t &p) const {
    return p[0] > bl[0] && p[1] > bl[1] && p[0] < tr[0] && p[1] < tr[1];
  }
  bool contains(const cellid_t &p) const {
    return p[0] >= bl[0] && p[1] >= bl[1] && p[0] <= tr[0] && p[1] <= tr[1];
  }
  bool isOnBoundry(const cellid_t &p) const { return contains(p) && !isInInterior(p); }
  bool intersects(const rect_t &r) const {
    return !((tr[0] < r.bl[0]) || (r.tr[0] < bl[0]) || (tr[1] < r.bl[1]) || (r.tr[1] < bl[1]));
  }
  bool intersection(const rect_t &r, rect_t &i) const {  // :208-220
    if (!intersects(r)) return false;
    int l = std::max(r.left(), left()), rr = std::min(r.right(), right());
    int b = std::max(r.bottom(), bottom()), t = std::min(r.top(), top());
    i = rect_t(l, b, rr, t);
    return true;
  }
  int left() const { return bl[0]; }
  int right() const { return tr[0]; }
  int bottom() const { return bl[1]; }
  int top() const { return tr[1]; }
  cellid_t bottom_left() const { return bl; }
  cellid_t top_right() const { return tr; }
  int size(int d) const { return tr[d] - bl[d]; }
};

enum eCellFlags { CELLFLAG_UNKNOWN = 0, CELLFLAG_PAIRED = 1, CELLFLAG_CRITCAL = 2 };  // grid_dataset.h:40-45
enum eGradDirection { GRADIENT_DIR_DOWNWARD, GRADIENT_DIR_UPWARD };                 // discreteMorseDS.h:32

// discreteMorseDS.h:90-126
struct critpt_t {
  cellid_t cellid;
  uint pair_idx = (uint)-1;
  bool isCancelled = false;
  bool isOnStrangulationPath = false;
  bool isBoundryCancelable = false;
  std::vector<cellid_t> asc_disc, des_disc;
  std::multiset<uint> asc, des;
};
typedef std::multiset<uint> conn_t;

// discreteMorseDS.h:78-143 + grid_mscomplex.h:48-84
struct GridMSComplex {
  rect_t m_rect, m_ext_rect;
  std::vector<float> m_cp_fns;
  std::vector<critpt_t *> m_cps;
  std::map<cellid_t, uint> m_id_cp_map;
  GridMSComplex() {}
  GridMSComplex(rect_t r, rect_t e) : m_rect(r), m_ext_rect(e) {}
  ~GridMSComplex() { for (auto *c : m_cps) delete c; }
};

static inline uint s_getCellDim(cellid_t c) { return (c[0] & 1) + (c[1] & 1); }  // grid_dataset.h:207-210

// ---------------------------------------------------------------------------
// GridDataset: dmsc/src/grid_dataset.cpp:1024-1907
// ---------------------------------------------------------------------------
struct GridDataset {
  rect_t m_rect, m_ext_rect;
  std::vector<float> verts;  // ext window, x fastest (fortran [x][y]), grid_dataset.cpp:1466
  int vnx = 0, vny = 0;      // vertex extents of the window
  int cnx = 0, cny = 0;      // cell extents (1+size)
  std::vector<int8_t> flags;
  std::vector<cellid_t> pairs, own;
  std::vector<cellid_t> m_critical_cells;
  int64_t pair_overwrites = 0;  // oracle-only assertion counter (pairCells overwriting a pair)
  // compareCells with the cell's vertices sorted DESCENDING, as the
  // reference's OpenCL kernels sort them (dmsc/resources/assigngradient.cl:
  // 40-87); false: the CPU path's ascending sort (grid_dataset.cpp:1530-1531)
  bool desc_cmp = false;
  // work_ocl's saddle incidences (grid_dataset.h:83-84)
  std::vector<uint> m_saddle_incidence_idx_offset, m_saddle_incidence_idx;

  GridDataset(rect_t r, rect_t e) : m_rect(r), m_ext_rect(e) {}

  // grid_dataset.cpp:1461-1484: C-order [x][y] cell arrays reindexed to ext.bl;
  // flags cleared to UNKNOWN, pairs/own default-constructed to (-1,-1).
  void init(const float *window) {
    cnx = 1 + m_ext_rect.size(0);
    cny = 1 + m_ext_rect.size(1);
    vnx = 1 + m_ext_rect.size(0) / 2;
    vny = 1 + m_ext_rect.size(1) / 2;
    if (window) verts.assign(window, window + (size_t)vnx * vny);
    flags.assign((size_t)cnx * cny, CELLFLAG_UNKNOWN);
    pairs.assign((size_t)cnx * cny, cellid_t());
    own.assign((size_t)cnx * cny, cellid_t());
  }
  size_t ci(cellid_t c) const {
    return (size_t)(c[0] - m_ext_rect.bl[0]) * cny + (size_t)(c[1] - m_ext_rect.bl[1]);
  }
  float vert(cellid_t c) const {  // vertex value at vertex-cell c (even coords)
    int x = (c[0] >> 1) - (m_ext_rect.bl[0] >> 1), y = (c[1] >> 1) - (m_ext_rect.bl[1] >> 1);
    return verts[(size_t)y * vnx + x];
  }

  // grid_dataset.h:158-167
  bool ptLt(cellid_t c1, cellid_t c2) const {
    double f1 = vert(c1), f2 = vert(c2);
    if (f1 != f2) return f1 < f2;
    return c1 < c2;
  }
  uint getCellDim(cellid_t c) const { return s_getCellDim(c); }

  uint getCellPoints(cellid_t c, cellid_t *p) const {  // :1566-1591
    switch (getCellDim(c)) {
      case 0: p[0] = c; return 1;
      case 1: {
        int d0 = c[0] & 1, d1 = c[1] & 1;
        p[0] = cellid_t(c[0] + d0, c[1] + d1);
        p[1] = cellid_t(c[0] - d0, c[1] - d1);
        return 2;
      }
      case 2:
        p[0] = cellid_t(c[0] + 1, c[1] + 1);
        p[1] = cellid_t(c[0] + 1, c[1] - 1);
        p[2] = cellid_t(c[0] - 1, c[1] - 1);
        p[3] = cellid_t(c[0] - 1, c[1] + 1);
        return 4;
    }
    throw std::logic_error("impossible dim");
  }
  uint getCellFacets(cellid_t c, cellid_t *f) const {  // :1593-1617
    switch (getCellDim(c)) {
      case 0: return 0;
      case 1: {
        int d0 = c[0] & 1, d1 = c[1] & 1;
        f[0] = cellid_t(c[0] + d0, c[1] + d1);
        f[1] = cellid_t(c[0] - d0, c[1] - d1);
        return 2;
      }
      case 2:
        f[0] = cellid_t(c[0], c[1] + 1);
        f[1] = cellid_t(c[0], c[1] - 1);
        f[2] = cellid_t(c[0] - 1, c[1]);
        f[3] = cellid_t(c[0] + 1, c[1]);
        return 4;
    }
    throw std::logic_error("impossible dim");
  }
  uint getCellCofacets(cellid_t c, cellid_t *cf) const {  // :1619-1657 (filtered to ext, order kept)
    uint cf_ct = 0;
    switch (getCellDim(c)) {
      case 0:
        cf[0] = cellid_t(c[0], c[1] + 1);
        cf[1] = cellid_t(c[0], c[1] - 1);
        cf[2] = cellid_t(c[0] - 1, c[1]);
        cf[3] = cellid_t(c[0] + 1, c[1]);
        cf_ct = 4;
        break;
      case 1: {
        int d0 = c[0] & 1, d1 = c[1] & 1;
        cf[0] = cellid_t(c[0] + d1, c[1] + d0);
        cf[1] = cellid_t(c[0] - d1, c[1] - d0);
        cf_ct = 2;
        break;
      }
      case 2: return 0;
    }
    uint nv = 0;
    for (uint i = 0; i < cf_ct; ++i)
      if (m_ext_rect.contains(cf[i])) cf[nv++] = cf[i];
    return nv;
  }
  uint getCellIncCells(cellid_t c, cellid_t *inc) const {  // :1035-1042
    inc[0] = cellid_t(c[0], c[1] + 1);
    inc[1] = cellid_t(c[0], c[1] - 1);
    inc[2] = cellid_t(c[0] - 1, c[1]);
    inc[3] = cellid_t(c[0] + 1, c[1]);
    return 4;
  }
  uint getcets(int dir, cellid_t c, cellid_t *out) const {  // :1029-1033
    return dir == 0 ? getCellFacets(c, out) : getCellCofacets(c, out);
  }

  // :1519-1536 (ascending vertex sort, then lexicographical_compare); with
  // desc_cmp the OpenCL kernels' compareCells (assigngradient.cl:62-87):
  // ins_sort_pts puts the largest vertex first (max_pt_idx, :40-60), then the
  // same lexicographic compare, a shorter list being the smaller
  bool compareCells(cellid_t c1, cellid_t c2) const {
    if (getCellDim(c1) == 0) return ptLt(c1, c2);
    cellid_t p1[4], p2[4];
    uint n1 = getCellPoints(c1, p1), n2 = getCellPoints(c2, p2);
    auto lt = [this](cellid_t a, cellid_t b) { return ptLt(a, b); };
    if (desc_cmp) {
      auto gt = [this](cellid_t a, cellid_t b) { return ptLt(b, a); };
      std::sort(p1, p1 + n1, gt);
      std::sort(p2, p2 + n2, gt);
    } else {
      std::sort(p1, p1 + n1, lt);
      std::sort(p2, p2 + n2, lt);
    }
    return std::lexicographical_compare(p1, p1 + n1, p2, p2 + n2, lt);
  }
  // :1538-1552
  float get_cell_fn(cellid_t c) const {
    float fn = 0.0f;
    cellid_t pts[4];
    uint n = getCellPoints(c, pts);
    for (uint j = 0; j < n; ++j) fn += vert(pts[j]);
    fn /= (float)n;
    return fn;
  }

  bool isCellMarked(cellid_t c) const { return flags[ci(c)] != CELLFLAG_UNKNOWN; }      // :1669
  bool isCellCritical(cellid_t c) const { return flags[ci(c)] & CELLFLAG_CRITCAL; }     // :1674
  bool isCellPaired(cellid_t c) const { return flags[ci(c)] & CELLFLAG_PAIRED; }        // :1679
  cellid_t getCellPairId(cellid_t c) const { return pairs[ci(c)]; }                     // :1511-1517
  void pairCells(cellid_t c, cellid_t p) {                                              // :1684-1691
    if ((flags[ci(c)] & CELLFLAG_PAIRED) || (flags[ci(p)] & CELLFLAG_PAIRED)) ++pair_overwrites;
    pairs[ci(c)] = p;
    pairs[ci(p)] = c;
    flags[ci(c)] |= CELLFLAG_PAIRED;
    flags[ci(p)] |= CELLFLAG_PAIRED;
  }
  void markCellCritical(cellid_t c) { flags[ci(c)] |= CELLFLAG_CRITCAL; }               // :1693
  bool isTrueBoundryCell(cellid_t c) const { return m_ext_rect.isOnBoundry(c); }        // :1698
  bool isCellExterior(cellid_t c) const { return !m_rect.contains(c) && m_ext_rect.contains(c); }  // :1708

  // :1314-1373
  bool lowestPairableCoFacet(cellid_t cellId, cellid_t &pairid) const {
    cellid_t cofacets[4];
    bool usable[4];
    uint cf_ct = getCellCofacets(cellId, cofacets);
    bool tb = isTrueBoundryCell(cellId);
    for (uint i = 0; i < cf_ct; ++i) {
      cellid_t facets[4];
      uint f_ct = getCellFacets(cofacets[i], facets);
      usable[i] = true;
      if (tb && !isTrueBoundryCell(cofacets[i])) { usable[i] = false; continue; }
      for (uint j = 0; j < f_ct; ++j)
        if (compareCells(cellId, facets[j])) { usable[i] = false; break; }
    }
    bool found = false;
    for (uint i = 0; i < cf_ct; ++i) {
      if (!usable[i]) continue;
      if (!found) { found = true; pairid = cofacets[i]; continue; }
      if (compareCells(cofacets[i], pairid)) pairid = cofacets[i];
    }
    return found;
  }

  // :1743-1820
  void assignGradients() {
    const rect_t &R = m_rect;
    for (int y = R.bottom(); y <= R.top(); ++y)
      for (int x = R.left(); x <= R.right(); ++x) {
        cellid_t c(x, y), p;
        if (isCellMarked(c)) continue;
        if (lowestPairableCoFacet(c, p)) pairCells(c, p);
      }
    for (int y = R.bottom(); y <= R.top(); ++y)
      for (int x = R.left(); x <= R.right(); ++x) {
        cellid_t c(x, y);
        if (!isCellMarked(c)) markCellCritical(c);
      }
    auto fix = [this](cellid_t c) {
      if (isCellCritical(c)) return;
      cellid_t cf[4];
      uint n = getCellCofacets(c, cf);
      for (uint j = 0; j < n; ++j)
        if (isCellExterior(cf[j])) {
          markCellCritical(c);
          markCellCritical(getCellPairId(c));
          break;
        }
    };
    for (int x = R.left(); x <= R.right(); ++x) {
      fix(cellid_t(x, R.bottom()));
      fix(cellid_t(x, R.top()));
    }
    for (int y = R.bottom() + 1; y < R.top(); ++y) {
      fix(cellid_t(R.left(), y));
      fix(cellid_t(R.right(), y));
    }
  }
  // :1822-1832
  void collateCriticalPoints() {
    const rect_t &E = m_ext_rect;
    for (int y = E.bottom(); y <= E.top(); ++y)
      for (int x = E.left(); x <= E.right(); ++x) {
        cellid_t c(x, y);
        if (isCellCritical(c)) m_critical_cells.push_back(c);
      }
  }
  // :1376-1427
  void track_gradient_tree_bfs(cellid_t start, int dir) {
    std::queue<cellid_t> q;
    q.push(start);
    while (!q.empty()) {
      cellid_t top = q.front();
      q.pop();
      own[ci(top)] = start;
      cellid_t cets[4];
      uint n = getcets(dir, top, cets);
      for (uint i = 0; i < n; ++i) {
        if (isCellCritical(cets[i])) continue;
        if (isCellExterior(cets[i])) continue;
        cellid_t next = getCellPairId(cets[i]);
        if (getCellDim(top) == getCellDim(next) && next != top) {
          own[ci(cets[i])] = start;
          q.push(next);
        }
      }
    }
  }
  // :1835-1856
  void assignCellOwnerExtrema() {
    for (size_t k = 0; k < m_critical_cells.size(); ++k) {
      cellid_t c = m_critical_cells[k];
      own[ci(c)] = c;
      switch (getCellDim(c)) {
        case 0: track_gradient_tree_bfs(c, GRADIENT_DIR_UPWARD); break;
        case 2: track_gradient_tree_bfs(c, GRADIENT_DIR_DOWNWARD); break;
        default: break;
      }
    }
  }
  // :1734-1741
  void work() {
    assignGradients();
    collateCriticalPoints();
    assignCellOwnerExtrema();
  }

  void writeout_connectivity(GridMSComplex *msc);
  int postMergeFillDiscs(GridMSComplex *msc);
  void work_ocl(bool collect_cps = true);
  void writeout_connectivity_ocl(GridMSComplex *msc);
};

// discreteMorseAlgorithm.h:244-268
static void addCriticalPointsToMSComplex(GridMSComplex *msc, const std::vector<cellid_t> &cl) {
  msc->m_cps.resize(cl.size());
  for (uint pos = 0; pos < cl.size(); ++pos) {
    critpt_t *cp = new critpt_t;
    msc->m_cps[pos] = cp;
    cp->cellid = cl[pos];
    msc->m_id_cp_map.insert(std::make_pair(cl[pos], pos));
  }
}

// grid_dataset.cpp:1285-1312
static void connectCps(GridMSComplex *msc, cellid_t c1, cellid_t c2) {
  if (s_getCellDim(c1) < s_getCellDim(c2)) std::swap(c1, c2);
  if (s_getCellDim(c1) != s_getCellDim(c2) + 1) throw std::logic_error("must connect i,i+1 cp (or vice versa)");
  if (msc->m_id_cp_map.find(c1) == msc->m_id_cp_map.end()) throw std::logic_error("cell not in id_cp_map c1");
  if (msc->m_id_cp_map.find(c2) == msc->m_id_cp_map.end()) throw std::logic_error("cell not in id_cp_map c2");
  uint i1 = msc->m_id_cp_map[c1], i2 = msc->m_id_cp_map[c2];
  msc->m_cps[i1]->des.insert(i2);
  msc->m_cps[i2]->asc.insert(i1);
}

// grid_dataset.cpp:1858-1907
void GridDataset::writeout_connectivity(GridMSComplex *msc) {
  addCriticalPointsToMSComplex(msc, m_critical_cells);
  msc->m_cp_fns.resize(m_critical_cells.size());
  for (size_t k = 0; k < m_critical_cells.size(); ++k) {
    cellid_t c = m_critical_cells[k];
    uint cp_idx = msc->m_id_cp_map[c];
    msc->m_cp_fns[cp_idx] = get_cell_fn(c);
    if (getCellDim(c) == 1) {
      cellid_t f[4], cf[4];
      uint f_ct = getCellFacets(c, f), cf_ct = getCellCofacets(c, cf);
      for (uint i = 0; i < f_ct; ++i) {
        cellid_t o = own[ci(f[i])];
        if (o != cellid_t(-1, -1)) connectCps(msc, c, o);
      }
      for (uint i = 0; i < cf_ct; ++i) {
        cellid_t o = own[ci(cf[i])];
        if (o != cellid_t(-1, -1)) connectCps(msc, c, o);
      }
    }
    if (!isCellPaired(c)) continue;
    msc->m_cps[cp_idx]->isBoundryCancelable = true;
    msc->m_cps[cp_idx]->pair_idx = msc->m_id_cp_map[getCellPairId(c)];
  }
}

// ---------------------------------------------------------------------------
// GridDataset::work_ocl (grid_dataset.cpp:353-399) restated on the CPU: the
// OpenCL kernels of assigngradient.cl, collate_critpts.cl and
// bfs_watershed.cl run one work-item at a time over ext-local coordinates,
// each reading the images as they were before the kernel (the host binds the
// same image as input and output, :476-479, 502-504, 529-531; the kernels'
// results do not depend on the order their work-items run in).  Images hold
// cells in the host arrays' [x][y] layout; pairs and owners in global
// coordinates, owners with a -1 coordinate stored as they are
// (common_funcs.cl:218-261).
// ---------------------------------------------------------------------------
namespace ocl {
struct L2 { int x, y; };
static inline bool eq(L2 a, L2 b) { return a.x == b.x && a.y == b.y; }
static inline int dim(L2 c) { return (c.x & 1) + (c.y & 1); }
static int facets(L2 c, L2 *f) {  // common_funcs.cl:15-49
  if (dim(c) == 1) { f[0] = {c.x + c.x % 2, c.y + c.y % 2}; f[1] = {c.x - c.x % 2, c.y - c.y % 2}; return 2; }
  if (dim(c) == 2) { f[0] = {c.x + 1, c.y}; f[1] = {c.x - 1, c.y}; f[2] = {c.x, c.y + 1}; f[3] = {c.x, c.y - 1}; return 4; }
  return 0;
}
static int cofacets(L2 c, L2 *cf) {  // :51-85
  if (dim(c) == 0) { cf[0] = {c.x + 1, c.y}; cf[1] = {c.x - 1, c.y}; cf[2] = {c.x, c.y + 1}; cf[3] = {c.x, c.y - 1}; return 4; }
  if (dim(c) == 1) { cf[0] = {c.x + c.y % 2, c.y + c.x % 2}; cf[1] = {c.x - c.y % 2, c.y - c.x % 2}; return 2; }
  return 0;
}
static bool on_tb(L2 c, L2 sz) { return c.x == 0 || c.y == 0 || c.x == sz.x || c.y == sz.y; }   // :134-142
static bool outside_tb(L2 c, L2 sz) { return c.x < 0 || c.y < 0 || c.x > sz.x || c.y > sz.y; }  // :144-152
}  // namespace ocl

void GridDataset::work_ocl(bool collect_cps) {
  using namespace ocl;
  const L2 sz{m_ext_rect.size(0), m_ext_rect.size(1)};
  const L2 eb{m_ext_rect.left(), m_ext_rect.bottom()};
  const L2 ib{m_rect.left() - eb.x, m_rect.bottom() - eb.y}, it{m_rect.right() - eb.x, m_rect.top() - eb.y};
  auto at = [&](L2 c) { return (size_t)c.x * cny + (size_t)c.y; };
  auto G = [&](L2 c) { return cellid_t(c.x + eb.x, c.y + eb.y); };
  auto Lc = [&](cellid_t c) { return L2{c[0] - eb.x, c[1] - eb.y}; };
  const bool saved = desc_cmp;
  desc_cmp = true;  // the kernels' compareCells (assigngradient.cl:62-87)
  // create_pair_flag_imgs_ocl (:248-279): images from the host arrays
  std::vector<uint8_t> fimg(flags.begin(), flags.end());
  std::vector<cellid_t> pimg(pairs);
  // assign_gradient (assigngradient.cl:89-183), over m_rect
  for (int gy = 0; gy <= it.y - ib.y; ++gy)
    for (int gx = 0; gx <= it.x - ib.x; ++gx) {
      const L2 c{gx + ib.x, gy + ib.y};
      L2 cf[4];
      const int cf_ct = cofacets(c, cf);
      int usable[4];
      const bool c_tb = on_tb(c, sz);
      for (int i = 0; i < 4; ++i) {
        usable[i] = i < cf_ct;
        if (!usable[i]) continue;
        if (outside_tb(cf[i], sz)) usable[i] = 0;
        if (c_tb && !on_tb(cf[i], sz)) usable[i] = 0;
        if (!usable[i]) continue;
        L2 f[4];
        const int f_ct = facets(cf[i], f);
        for (int j = 0; j < f_ct; ++j)
          if (compareCells(G(c), G(f[j]))) usable[i] = 0;
      }
      bool paired = false;
      L2 p{0, 0};
      for (int i = 0; i < 4; ++i) {
        if (!usable[i]) continue;
        if (!paired) { p = cf[i]; paired = true; }
        else if (compareCells(G(cf[i]), G(p))) p = cf[i];
      }
      if (paired) { pimg[at(c)] = G(p); fimg[at(c)] = 1; }
      else fimg[at(c)] = 2;
    }
  // complete_pairings (:184-238), over ext
  {
    const std::vector<uint8_t> fin(fimg);
    const std::vector<cellid_t> pin(pimg);
    for (int y = 0; y <= sz.y; ++y)
      for (int x = 0; x <= sz.x; ++x) {
        const L2 c{x, y};
        L2 f[4];
        const int f_ct = facets(c, f);
        for (int i = 0; i < f_ct; ++i) {
          if (outside_tb(f[i], sz)) continue;  // (a 2D image read out of range; never taken for ext cells)
          const L2 fp = Lc(pin[at(f[i])]);
          if (eq(fp, c) && (fin[at(f[i])] & 1)) { pimg[at(c)] = G(f[i]); fimg[at(c)] = 1; break; }
        }
      }
  }
  // mark_boundrypairs_critical_1 (:240-301) and _2 (:303-336), over ext
  {
    const std::vector<uint8_t> fin(fimg);
    for (int y = 0; y <= sz.y; ++y)
      for (int x = 0; x <= sz.x; ++x) {
        const L2 c{x, y};
        if (!(fin[at(c)] & 1)) continue;
        L2 cf[4];
        const int cf_ct = cofacets(c, cf);
        bool out = false;
        for (int i = 0; i < cf_ct; ++i) {
          if (outside_tb(cf[i], sz)) continue;
          out |= cf[i].x < ib.x || cf[i].y < ib.y || cf[i].x > it.x || cf[i].y > it.y;
        }
        if (out) fimg[at(c)] = 3;
      }
  }
  {
    const std::vector<uint8_t> fin(fimg);
    for (int y = 0; y <= sz.y; ++y)
      for (int x = 0; x <= sz.x; ++x) {
        const L2 c{x, y};
        if (!(fin[at(c)] & 1)) continue;
        const uint8_t pf = fin[at(Lc(pimg[at(c)]))];
        if ((pf & 2) && (pf & 1)) fimg[at(c)] = 3;
      }
  }
  desc_cmp = saved;
  // read_pair_img_ocl / read_flag_img_ocl (:372-373)
  pairs = pimg;
  for (size_t k = 0; k < flags.size(); ++k) flags[k] = (int8_t)fimg[k];
  // collateCritcalPoints_ocl (:550-657): row-major over ext
  m_critical_cells.clear();
  std::map<std::pair<int, int>, uint> crit_idx;  // the index collate_cps_writeids writes into the pair image
  for (int y = 0; y <= sz.y; ++y)
    for (int x = 0; x <= sz.x; ++x)
      if (fimg[at(L2{x, y})] & 2) {
        crit_idx[{x, y}] = (uint)m_critical_cells.size();
        m_critical_cells.push_back(G(L2{x, y}));
      }
  // assignCellOwnerExtrema_ocl (:763-890): dobfs_markowner_extrema_init, then
  // dobfs_markowner_extrema until nothing changes (bfs_watershed.cl:6-98)
  auto store = [&](L2 v) { return (v.x != -1 && v.y != -1) ? cellid_t(v.x + eb.x, v.y + eb.y) : cellid_t(v.x, v.y); };
  auto load = [&](cellid_t v) { return (v[0] != -1 && v[1] != -1) ? L2{v[0] - eb.x, v[1] - eb.y} : L2{v[0], v[1]}; };
  std::vector<cellid_t> oimg(flags.size());
  for (int y = 0; y <= sz.y; ++y)
    for (int x = 0; x <= sz.x; ++x) {
      const L2 c{x, y};
      L2 inf{-1, -1};
      const uint8_t fl = fimg[at(c)];
      if (fl & 2) inf = c;
      if (!(fl & 2) && (fl & 1)) {
        const L2 p = Lc(pimg[at(c)]);
        const int d = dim(c), pd = dim(p);
        if (d == 0 || d == 2) inf = p;
        else {
          L2 cets[4];
          if (pd == 0) facets(c, cets);
          else cofacets(c, cets);
          const int k = eq(cets[0], p) ? 1 : 0;
          if (cets[k].x <= sz.x && cets[k].y <= sz.y) inf = cets[k];
        }
      }
      oimg[at(c)] = store(inf);
    }
  for (int iter = 0;; ++iter) {
    if (iter > 64) throw std::logic_error("work_ocl: owner pointers did not converge");
    const std::vector<cellid_t> oin(oimg);
    bool changed = false;
    for (int y = 0; y <= sz.y; ++y)
      for (int x = 0; x <= sz.x; ++x) {
        const L2 c{x, y};
        const L2 o = load(oin[at(c)]);
        L2 oo = o;
        if (!outside_tb(o, sz)) oo = load(oin[at(o)]);
        oimg[at(c)] = store(oo);
        if (!eq(oo, o)) changed = true;
      }
    if (!changed) break;
  }
  // collect_saddle_conn_ocl (:907-1022): count_critpt_incidences and
  // write_critpt_incidences (collate_critpts.cl:101-195)
  m_saddle_incidence_idx_offset.assign(m_critical_cells.size() + 1, 0);
  m_saddle_incidence_idx.clear();
  if (collect_cps) {
    for (size_t k = 0; k < m_critical_cells.size(); ++k) {
      const L2 c = Lc(m_critical_cells[k]);
      if (dim(c) == 1) {
        L2 n[4];
        facets(c, n);
        cofacets(c, n + 2);
        for (int i = 0; i < 4; ++i) {
          if (outside_tb(n[i], sz)) continue;
          const L2 o = load(oimg[at(n[i])]);
          if (outside_tb(o, sz)) continue;
          auto f = crit_idx.find({o.x, o.y});
          if (f == crit_idx.end()) throw std::logic_error("work_ocl: an incidence owner is not critical");
          m_saddle_incidence_idx.push_back(f->second);
        }
      }
      m_saddle_incidence_idx_offset[k + 1] = (uint)m_saddle_incidence_idx.size();
    }
  }
  // read_own_img_ocl (:392)
  own = oimg;
}

// grid_dataset.cpp:1250-1283 with the index overload of connectCps (:1233-1248)
void GridDataset::writeout_connectivity_ocl(GridMSComplex *msc) {
  addCriticalPointsToMSComplex(msc, m_critical_cells);
  msc->m_cp_fns.resize(m_critical_cells.size());
  for (size_t k = 0; k < m_critical_cells.size(); ++k) {
    cellid_t c = m_critical_cells[k];
    uint cp_idx = msc->m_id_cp_map[c];
    msc->m_cp_fns[cp_idx] = get_cell_fn(c);
    if (!isCellPaired(c)) continue;
    msc->m_cps[cp_idx]->isBoundryCancelable = true;
    msc->m_cps[cp_idx]->pair_idx = msc->m_id_cp_map[getCellPairId(c)];
  }
  for (size_t i = 1; i < m_saddle_incidence_idx_offset.size(); ++i)
    for (uint j = m_saddle_incidence_idx_offset[i - 1]; j < m_saddle_incidence_idx_offset[i]; ++j) {
      uint a = m_saddle_incidence_idx[j], b = (uint)(i - 1);
      if (s_getCellDim(msc->m_cps[a]->cellid) < s_getCellDim(msc->m_cps[b]->cellid)) std::swap(a, b);
      msc->m_cps[a]->des.insert(b);
      msc->m_cps[b]->asc.insert(a);
    }
}

// grid_dataset.cpp:1044-1231
int GridDataset::postMergeFillDiscs(GridMSComplex *msc) {
  std::map<cellid_t, std::vector<cellid_t> *> surv_asc, surv_des;
  std::vector<uint> surv_saddle_idxs;
  for (uint i = 0; i < msc->m_cps.size(); ++i) {
    critpt_t *cp = msc->m_cps[i];
    int cp_dim = getCellDim(cp->cellid);
    if (cp->isBoundryCancelable) {
      critpt_t *pair_cp = msc->m_cps[cp->pair_idx];
      if (cp_dim == 1) {
        conn_t *cc = (getCellDim(pair_cp->cellid) == 0) ? &cp->des : &cp->asc;
        if (cc->size() != 1) throw std::logic_error("I should be connected to exactly one surv extrema");
        critpt_t *ext = msc->m_cps[*cc->begin()];
        if (pair_cp->pair_idx != i) throw std::logic_error("My pair does not know Im paired with him");
        if (m_rect.contains(cp->cellid)) own[ci(cp->cellid)] = ext->cellid;
        if (m_rect.contains(pair_cp->cellid)) own[ci(pair_cp->cellid)] = ext->cellid;
      } else if (cp_dim == 2) {
        for (auto it = cp->des.begin(); it != cp->des.end(); ++it)
          if (m_rect.contains(pair_cp->cellid)) msc->m_cps[*it]->asc_disc.push_back(pair_cp->cellid);
      } else if (cp_dim == 0) {
        for (auto it = cp->asc.begin(); it != cp->asc.end(); ++it)
          if (m_rect.contains(pair_cp->cellid)) msc->m_cps[*it]->des_disc.push_back(pair_cp->cellid);
      }
    } else {
      switch (cp_dim) {
        case 0: surv_asc.insert(std::make_pair(cp->cellid, &cp->asc_disc)); break;
        case 1: {
          cellid_t inc[4];
          getCellIncCells(cp->cellid, inc);
          for (uint j = 0; j < 4; ++j)
            if (m_rect.contains(inc[j]) && isCellPaired(inc[j]) && !isCellCritical(inc[j])) {
              auto *disc = (getCellDim(inc[j]) == 0) ? &cp->des_disc : &cp->asc_disc;
              disc->push_back(getCellPairId(inc[j]));
            }
          surv_saddle_idxs.push_back(i);
          break;
        }
        case 2: surv_des.insert(std::make_pair(cp->cellid, &cp->des_disc)); break;
      }
    }
  }
  auto lookup = [](std::map<cellid_t, std::vector<cellid_t> *> &m, cellid_t o) {
    // The reference uses operator[] here; a missing key would dereference NULL.
    auto it = m.find(o);
    if (it == m.end()) throw std::logic_error("owner is not a surviving extremum");
    return it->second;
  };
  for (int y = m_rect.bottom();; y += 2) {
    for (int x = m_rect.left();; x += 2) {
      cellid_t c(x, y), o = own[ci(c)];
      if (m_rect.contains(o)) o = own[ci(o)];
      if (o[0] != -1 && o[1] != -1) lookup(surv_asc, o)->push_back(c);
      if (x == m_rect.right()) break;
    }
    if (y == m_rect.top()) break;
  }
  for (int y = m_rect.bottom() + 1;; y += 2) {
    for (int x = m_rect.left() + 1;; x += 2) {
      cellid_t c(x, y), o = own[ci(c)];
      if (m_rect.contains(o)) o = own[ci(o)];
      if (o[0] != -1 && o[1] != -1) lookup(surv_des, o)->push_back(c);
      if (x + 1 == m_rect.right()) break;
    }
    if (y + 1 == m_rect.top()) break;
  }
  for (uint i = 0; i < surv_saddle_idxs.size(); ++i) {
    critpt_t *cp = msc->m_cps[surv_saddle_idxs[i]];
    std::vector<cellid_t> *disc[] = {&cp->asc_disc, &cp->des_disc};
    for (uint j = 0; j < 2; ++j) {
      size_t k = 0;
      while (k != disc[j]->size()) {
        cellid_t path_cell = (*disc[j])[k];
        cellid_t cets[4];
        uint n = getcets((j + 1) % 2, path_cell, cets);
        for (uint m = 0; m < n; ++m) {
          if (isCellCritical(cets[m])) continue;
          if (!m_rect.contains(cets[m])) continue;
          cellid_t p = getCellPairId(cets[m]);
          if (p == path_cell) continue;
          disc[j]->push_back(p);
        }
        ++k;
      }
    }
  }
  return 0;
}

// discreteMorseAlgorithm.h:348-464 (record==nullptr) and :466-585 (with new_edges)
static void cancelPairs(GridMSComplex *msc, uint cp0, uint cp1, std::vector<uint> *new_edges) {
  auto &C = msc->m_cps;
  if (C[cp0]->asc.find(cp1) == C[cp0]->asc.end()) std::swap(cp0, cp1);
  if (C[cp0]->asc.find(cp1) == C[cp0]->asc.end()) return;  // "critical points are not connected"
  for (auto a = C[cp0]->asc.begin(); a != C[cp0]->asc.end(); ++a)
    for (auto d = C[cp1]->des.begin(); d != C[cp1]->des.end(); ++d) {
      if (*a == cp1 || *d == cp0) continue;
      C[*a]->des.insert(*d);
      C[*d]->asc.insert(*a);
      if (new_edges) { new_edges->push_back(*d); new_edges->push_back(*a); }
      if (C[*a]->des.count(*d) >= 2) {
        C[*a]->isOnStrangulationPath = true;
        C[*d]->isOnStrangulationPath = true;
      }
    }
  for (auto a = C[cp0]->asc.begin(); a != C[cp0]->asc.end(); ++a) {
    if (*a == cp1) continue;
    C[*a]->des.erase(cp0);
  }
  for (auto d = C[cp0]->des.begin(); d != C[cp0]->des.end(); ++d) C[*d]->asc.erase(cp0);
  for (auto a = C[cp1]->asc.begin(); a != C[cp1]->asc.end(); ++a) C[*a]->des.erase(cp1);
  for (auto d = C[cp1]->des.begin(); d != C[cp1]->des.end(); ++d) {
    if (*d == cp0) continue;
    C[*d]->asc.erase(cp1);
  }
  C[cp0]->isCancelled = true;
  C[cp0]->des.clear();
  C[cp1]->isCancelled = true;
  C[cp1]->asc.clear();
}

// discreteMorseAlgorithm.h:1006-1089
static void uncancel_pairs(GridMSComplex *msc, uint cp1, uint cp2) {
  auto &C = msc->m_cps;
  if (C[cp1]->asc.find(cp2) == C[cp1]->asc.end()) std::swap(cp1, cp2);
  conn_t *acdc[] = {&C[cp1]->asc, &C[cp2]->des};
  uint *ids[] = {&cp1, &cp2};
  for (uint i = 0; i < 2; ++i) {
    uint other = *ids[(i + 1) % 2];
    if (acdc[i]->find(other) == acdc[i]->end()) throw std::logic_error("cancellable pair is not connected");
    conn_t nac;
    for (auto it = acdc[i]->begin(); it != acdc[i]->end(); ++it) {
      if (*it == other) continue;
      if (!C[*it]->isBoundryCancelable) { nac.insert(*it); continue; }
      if (C[*it]->isCancelled) throw std::logic_error("*acdc_conn_it should not have been cancelled yet");
      uint pidx = C[*it]->pair_idx;
      if (C[pidx]->pair_idx != *it) throw std::logic_error("*acdc_conn_it and its pair dont agree on pairing");
      conn_t *pc[] = {&C[pidx]->asc, &C[pidx]->des};
      for (auto jt = pc[i]->begin(); jt != pc[i]->end(); ++jt) {
        if (C[*jt]->isBoundryCancelable)
          throw std::logic_error("the connected cancelable cp shold not  contain a cancelable cp in its connections");
        nac.insert(*jt);
      }
    }
    acdc[i]->clear();
    acdc[i]->insert(nac.begin(), nac.end());
  }
  C[cp1]->isCancelled = false;
  C[cp2]->isCancelled = false;
}

// grid_mscomplex.cpp:7-22
static void shallow_replicate_cp(GridMSComplex &msc, const critpt_t &cp) {
  if (msc.m_id_cp_map.count(cp.cellid) != 0) throw std::logic_error("this cp is present in msc");
  critpt_t *d = new critpt_t;
  d->isCancelled = cp.isCancelled;
  d->isBoundryCancelable = cp.isBoundryCancelable;
  d->isOnStrangulationPath = cp.isOnStrangulationPath;
  d->cellid = cp.cellid;
  msc.m_id_cp_map[d->cellid] = (uint)msc.m_cps.size();
  msc.m_cps.push_back(d);
}

static void check_merge_ixn(const rect_t &ixn) {
  if ((ixn.left() != ixn.right()) && (ixn.top() != ixn.bottom())) throw std::logic_error("rects must merge along a 1 manifold");
  if (ixn.bottom_left() == ixn.top_right()) throw std::logic_error("rects cannot merge along a point alone");
}

// grid_mscomplex.cpp:24-156
static GridMSComplex *merge_up(const GridMSComplex &msc1, const GridMSComplex &msc2) {
  rect_t ixn;
  if (!msc2.m_rect.intersection(msc1.m_rect, ixn)) throw std::logic_error("rects should intersect for merge");
  check_merge_ixn(ixn);
  rect_t r(std::min(msc1.m_rect.bottom_left(), msc2.m_rect.bottom_left()),
           std::max(msc1.m_rect.top_right(), msc2.m_rect.top_right()));
  rect_t e(std::min(msc1.m_ext_rect.bottom_left(), msc2.m_ext_rect.bottom_left()),
           std::max(msc1.m_ext_rect.top_right(), msc2.m_ext_rect.top_right()));
  GridMSComplex *out = new GridMSComplex(r, e);
  const GridMSComplex *arr[] = {&msc1, &msc2};
  for (uint i = 0; i < 2; ++i) {
    const GridMSComplex *msc = arr[i];
    for (uint j = 0; j < msc->m_cps.size(); ++j) {
      const critpt_t *s = msc->m_cps[j];
      if (i == 1 && out->m_id_cp_map.count(s->cellid) == 1) continue;
      if (s->isCancelled) continue;
      shallow_replicate_cp(*out, *s);
      out->m_cp_fns.push_back(msc->m_cp_fns[j]);
    }
  }
  for (uint i = 0; i < 2; ++i) {
    const GridMSComplex *msc = arr[i];
    for (uint j = 0; j < msc->m_cps.size(); ++j) {
      const critpt_t *s = msc->m_cps[j];
      if (s->isCancelled) continue;
      critpt_t *d = out->m_cps[out->m_id_cp_map[s->cellid]];
      if (s->isBoundryCancelable) {
        const critpt_t *sp = msc->m_cps[s->pair_idx];
        d->pair_idx = out->m_id_cp_map[sp->cellid];
      }
      const conn_t *src[] = {&s->asc, &s->des};
      conn_t *dst[] = {&d->asc, &d->des};
      bool cmn = ixn.contains(s->cellid) && i == 1;
      for (uint k = 0; k < 2; ++k)
        for (auto it = src[k]->begin(); it != src[k]->end(); ++it) {
          const critpt_t *cc = msc->m_cps[*it];
          if (cmn && ixn.contains(cc->cellid)) continue;
          if (cc->isCancelled) continue;
          dst[k]->insert(out->m_id_cp_map[cc->cellid]);
        }
    }
  }
  for (int y = ixn.bottom(); y <= ixn.top(); ++y)
    for (int x = ixn.left(); x <= ixn.right(); ++x) {
      cellid_t c(x, y);
      if (out->m_id_cp_map.count(c) != 1) throw std::logic_error("missing common bndry cp");
      uint si = out->m_id_cp_map[c];
      critpt_t *s = out->m_cps[si];
      if (s->isCancelled || !s->isBoundryCancelable) continue;
      uint pi = s->pair_idx;
      cellid_t p = out->m_cps[pi]->cellid;
      if (!out->m_rect.isInInterior(c) && !out->m_ext_rect.isOnBoundry(c)) continue;
      if (!out->m_rect.isInInterior(p) && !out->m_ext_rect.isOnBoundry(p)) continue;
      cancelPairs(out, si, pi, nullptr);
    }
  return out;
}

// grid_mscomplex.cpp:158-322
static void merge_down(GridMSComplex &self, GridMSComplex &msc1, GridMSComplex &msc2) {
  rect_t ixn;
  if (!msc2.m_rect.intersection(msc1.m_rect, ixn)) throw std::logic_error("rects should intersect for merge");
  check_merge_ixn(ixn);
  for (int y = ixn.top(); y >= ixn.bottom(); --y)
    for (int x = ixn.right(); x >= ixn.left(); --x) {
      cellid_t c(x, y);
      if (self.m_id_cp_map.count(c) != 1) throw std::logic_error("missing common bndry cp");
      uint si = self.m_id_cp_map[c];
      critpt_t *s = self.m_cps[si];
      if (!s->isCancelled) continue;
      uint pi = s->pair_idx;
      cellid_t p = self.m_cps[pi]->cellid;
      if (!self.m_rect.isInInterior(c) && !self.m_ext_rect.isOnBoundry(c)) continue;
      if (!self.m_rect.isInInterior(p) && !self.m_ext_rect.isOnBoundry(p)) continue;
      uncancel_pairs(&self, si, pi);
    }
  GridMSComplex *arr[] = {&msc1, &msc2};
  auto &M = self.m_cps;
  for (uint i = 0; i < 2; ++i) {
    GridMSComplex *msc = arr[i];
    for (uint j = 0; j < M.size(); ++j) {
      critpt_t *s = M[j];
      if (s->isCancelled) throw std::logic_error("all cps ought to be uncancelled by now");
      if (!s->isBoundryCancelable) continue;
      critpt_t *sp = M[s->pair_idx];
      bool s_in = msc->m_id_cp_map.count(s->cellid) != 0;
      bool sp_in = msc->m_id_cp_map.count(sp->cellid) != 0;
      if (!s_in && !sp_in) continue;
      if (!s_in) { shallow_replicate_cp(*msc, *s); msc->m_cp_fns.push_back(self.m_cp_fns[j]); }
      if (!sp_in) { shallow_replicate_cp(*msc, *sp); msc->m_cp_fns.push_back(self.m_cp_fns[s->pair_idx]); }
      uint di = msc->m_id_cp_map[s->cellid];
      critpt_t *d = msc->m_cps[di];
      if (!s_in || !sp_in || !d->isBoundryCancelable) {
        uint dpi = msc->m_id_cp_map[sp->cellid];
        critpt_t *dp = msc->m_cps[dpi];
        d->isBoundryCancelable = true;
        dp->isBoundryCancelable = true;
        d->pair_idx = dpi;
        dp->pair_idx = di;
      }
      conn_t *src[] = {&s->asc, &s->des};
      conn_t *dst[] = {&d->asc, &d->des};
      for (uint k = 0; k < 2; ++k) {
        dst[k]->clear();
        for (auto it = src[k]->begin(); it != src[k]->end(); ++it) {
          critpt_t *sc = M[*it];
          if (sc->isBoundryCancelable) throw std::logic_error("only non cancellable cps must be remaining");
          if (msc->m_id_cp_map.count(sc->cellid) == 0) {
            shallow_replicate_cp(*msc, *sc);
            msc->m_cp_fns.push_back(self.m_cp_fns[*it]);
          }
          dst[k]->insert(msc->m_id_cp_map[sc->cellid]);
        }
      }
    }
    for (uint j = 0; j < M.size(); ++j) {
      critpt_t *s = M[j];
      if (s->isBoundryCancelable) continue;
      if (msc->m_id_cp_map.count(s->cellid) != 1) continue;
      critpt_t *d = msc->m_cps[msc->m_id_cp_map[s->cellid]];
      conn_t *src[] = {&s->asc, &s->des};
      conn_t *dst[] = {&d->asc, &d->des};
      for (uint k = 0; k < 2; ++k) {
        dst[k]->clear();
        for (auto it = src[k]->begin(); it != src[k]->end(); ++it) {
          critpt_t *sc = M[*it];
          if (msc->m_id_cp_map.count(sc->cellid) == 0) continue;
          dst[k]->insert(msc->m_id_cp_map[sc->cellid]);
        }
      }
    }
  }
}

// grid_mscomplex.cpp:331-379. c3/c4 are read from p1 (reference bug), so for
// equal persistence every remaining test compares a value with itself.
struct persistence_comparator_t {
  GridMSComplex *m_msc;
  explicit persistence_comparator_t(GridMSComplex *m) : m_msc(m) {}
  bool operator()(const std::pair<uint, uint> &p1, const std::pair<uint, uint> &p2) const {
    float f1 = m_msc->m_cp_fns[p1.first], f2 = m_msc->m_cp_fns[p1.second];
    float f3 = m_msc->m_cp_fns[p2.first], f4 = m_msc->m_cp_fns[p2.second];
    float d1 = std::abs(f2 - f1), d2 = std::abs(f4 - f3);
    if (d1 != d2) return d1 > d2;
    cellid_t c1 = m_msc->m_cps[p1.first]->cellid, c2 = m_msc->m_cps[p1.second]->cellid;
    cellid_t c3 = m_msc->m_cps[p1.first]->cellid, c4 = m_msc->m_cps[p1.second]->cellid;
    d1 = (float)((c1[0] - c2[0]) * (c1[0] - c2[0]) + (c1[1] - c2[1]) * (c1[1] - c2[1]));
    d2 = (float)((c3[0] - c4[0]) * (c3[0] - c4[0]) + (c3[1] - c4[1]) * (c3[1] - c4[1]));
    if (d1 != d2) return d1 > d2;
    if (c1 > c2) std::swap(c1, c2);
    if (c3 > c4) std::swap(c3, c4);
    if (c1 != c3) return c1 > c3;
    return c2 > c4;
  }
};

typedef std::vector<std::pair<uint, uint>> canc_list_t;

// Oracle-only counters of the simplification (sizes of the work, for design).
struct SimplifyStats {
  uint64_t pushes = 0, pops = 0, cancels = 0, new_edges = 0, resubmits = 0, max_heap = 0, erase_work = 0;
};
static thread_local SimplifyStats g_sstats;

// grid_mscomplex.cpp:384-512
static void simplify(GridMSComplex *self, canc_list_t &canc, double tresh, uint *n_cancel) {
  typedef std::priority_queue<std::pair<uint, uint>, canc_list_t, persistence_comparator_t> pq_t;
  persistence_comparator_t comp(self);
  pq_t pq(comp);
  float max_val = std::numeric_limits<float>::min();
  float min_val = std::numeric_limits<float>::max();
  auto &C = self->m_cps;
  for (uint i = 0; i < C.size(); ++i) {
    critpt_t *cp = C[i];
    if (s_getCellDim(cp->cellid) == 1) {
      conn_t *acdc[] = {&cp->asc, &cp->des};
      for (uint j = 0; j < 2; ++j) {
        if (acdc[j]->size() != 2) continue;
        if (*(acdc[j]->begin()) == *(++acdc[j]->begin())) cp->isOnStrangulationPath = true;
      }
    }
    max_val = std::max(max_val, self->m_cp_fns[i]);
    min_val = std::min(min_val, self->m_cp_fns[i]);
    for (auto it = cp->des.begin(); it != cp->des.end(); ++it) { pq.push(std::make_pair(i, *it)); ++g_sstats.pushes; }
  }
  canc_list_t resubmit;
  float max_persistence = max_val - min_val;
  uint ncanc = 0;
  while (pq.size() != 0) {
    std::pair<uint, uint> cpair = pq.top();
    if (pq.size() > g_sstats.max_heap) g_sstats.max_heap = pq.size();
    pq.pop();
    ++g_sstats.pops;
    uint v1 = cpair.first, v2 = cpair.second;
    critpt_t *cp1 = C[v1], *cp2 = C[v2];
    float persistence = std::abs(self->m_cp_fns[v1] - self->m_cp_fns[v2]);
    if ((double)persistence / (double)max_persistence > tresh) break;
    if (s_getCellDim(cp2->cellid) == 1) { std::swap(cp1, cp2); std::swap(v1, v2); }
    uint cp2_dim = s_getCellDim(cp2->cellid);
    if (cp1->isCancelled || cp2->isCancelled) continue;
    if (self->m_rect.isOnBoundry(cp1->cellid) && !self->m_rect.isOnBoundry(cp2->cellid)) continue;
    if (!self->m_rect.isOnBoundry(cp1->cellid) && self->m_rect.isOnBoundry(cp2->cellid)) continue;
    conn_t *cp2_acdc[] = {&cp2->asc, &cp2->des};
    if (cp1->isOnStrangulationPath && cp2_acdc[cp2_dim / 2]->size() != 1) { resubmit.push_back(cpair); continue; }
    if (cp1->isOnStrangulationPath && self->m_rect.isOnBoundry(cp1->cellid)) continue;
    std::vector<uint> new_edges;
    cancelPairs(self, v1, v2, &new_edges);
    ++ncanc;
    cp1->isBoundryCancelable = true;
    cp2->isBoundryCancelable = true;
    cp1->pair_idx = v2;
    cp2->pair_idx = v1;
    canc.push_back(cpair);
    for (size_t i = 0; i < new_edges.size(); i += 2) pq.push(std::make_pair(new_edges[i], new_edges[i + 1]));
    for (size_t i = 0; i < resubmit.size(); ++i) pq.push(resubmit[i]);
    g_sstats.pushes += new_edges.size() / 2 + resubmit.size();
    g_sstats.new_edges += new_edges.size() / 2;
    g_sstats.resubmits += resubmit.size();
    ++g_sstats.cancels;
    g_sstats.erase_work += cp1->des.size() + cp2->asc.size() + cp2->des.size() + cp1->asc.size();
    resubmit.clear();
  }
  if (n_cancel) *n_cancel = ncanc;
}

// grid_mscomplex.cpp:514-526
static void un_simplify(GridMSComplex *self, const canc_list_t &canc) {
  for (auto it = canc.rbegin(); it != canc.rend(); ++it) uncancel_pairs(self, it->first, it->second);
}

// ---------------------------------------------------------------------------
// Snapshot of a complex in flat arrays (the exchange format the tests use).
// ---------------------------------------------------------------------------
struct MscDump {
  int16_t rect[4], ext[4];
  std::vector<int16_t> cellid;  // 2 per cp (x, y)
  std::vector<float> fn;
  std::vector<uint32_t> pair_idx;
  std::vector<uint8_t> flags;   // bit0 cancelled, bit1 strangulation, bit2 boundary-cancelable
  std::vector<uint32_t> asc_off, asc, des_off, des;
  std::vector<uint32_t> adisc_off, ddisc_off;
  std::vector<int16_t> adisc, ddisc;  // 2 per cell
};

static void dump_msc(const GridMSComplex &m, MscDump &d) {
  d.rect[0] = m.m_rect.bl[0]; d.rect[1] = m.m_rect.bl[1]; d.rect[2] = m.m_rect.tr[0]; d.rect[3] = m.m_rect.tr[1];
  d.ext[0] = m.m_ext_rect.bl[0]; d.ext[1] = m.m_ext_rect.bl[1]; d.ext[2] = m.m_ext_rect.tr[0]; d.ext[3] = m.m_ext_rect.tr[1];
  size_t n = m.m_cps.size();
  d.cellid.resize(2 * n); d.fn.resize(n); d.pair_idx.resize(n); d.flags.resize(n);
  d.asc_off.assign(1, 0); d.des_off.assign(1, 0); d.adisc_off.assign(1, 0); d.ddisc_off.assign(1, 0);
  d.asc.clear(); d.des.clear(); d.adisc.clear(); d.ddisc.clear();
  for (size_t i = 0; i < n; ++i) {
    const critpt_t *c = m.m_cps[i];
    d.cellid[2 * i] = c->cellid[0]; d.cellid[2 * i + 1] = c->cellid[1];
    d.fn[i] = i < m.m_cp_fns.size() ? m.m_cp_fns[i] : 0.0f;
    d.pair_idx[i] = c->pair_idx;
    d.flags[i] = (c->isCancelled ? 1 : 0) | (c->isOnStrangulationPath ? 2 : 0) | (c->isBoundryCancelable ? 4 : 0);
    for (uint v : c->asc) d.asc.push_back(v);
    for (uint v : c->des) d.des.push_back(v);
    d.asc_off.push_back((uint32_t)d.asc.size());
    d.des_off.push_back((uint32_t)d.des.size());
    for (auto &q : c->asc_disc) { d.adisc.push_back(q[0]); d.adisc.push_back(q[1]); }
    for (auto &q : c->des_disc) { d.ddisc.push_back(q[0]); d.ddisc.push_back(q[1]); }
    d.adisc_off.push_back((uint32_t)(d.adisc.size() / 2));
    d.ddisc_off.push_back((uint32_t)(d.ddisc.size() / 2));
  }
}

// ---------------------------------------------------------------------------
// Pipeline: GridDataManager, dmsc/src/grid_datamanager.cpp:40-89, 121-140,
// 258-357, 359-490, 530-594, 596-662, run in its single-threaded order.
// split2d=0 is the reference (y-strips only, split_axes=1 at :50); split2d=1
// alternates y/x splits per level to form square blocks (an extension: the
// reference's merge_up accepts any shared 1-manifold, grid_mscomplex.cpp:35-39).
// ---------------------------------------------------------------------------
struct Piece {
  GridDataset *ds = nullptr;
  GridMSComplex *msc = nullptr;
  int level = 0;
};

struct Pipeline {
  int X = 0, Y = 0, levels = 0, split2d = 0;
  int ocl = 0;  // GridDataManager's ocl flag (-ocl): pieces through work_ocl (grid_datamanager.cpp:123-132, 221-222, 433-434)
  double tresh = 0;
  std::vector<Piece> pieces;
  size_t nleaves = 0;
  MscDump root_after_simplify;
  bool have_root_snapshot = false;
  canc_list_t canc;
  uint ncancel = 0;
  int64_t pair_overwrites = 0;
  // write_discs (grid_mscomplex.cpp:542-590): files keyed by (kind, cellid),
  // opened in append mode by every leaf in turn; kept in memory here.
  std::map<std::pair<int, cellid_t>, std::vector<cellid_t>> disc_files;
  double t_stage[5] = {0, 0, 0, 0, 0};
  ~Pipeline() {
    for (auto &p : pieces) { delete p.ds; delete p.msc; }
  }
};

static void create_pieces(Pipeline &P, rect_t r, rect_t e, int level, int depth) {
  if (level == 0) {
    Piece p;
    p.ds = new GridDataset(r, e);
    p.msc = new GridMSComplex(r, e);
    P.pieces.push_back(p);
    return;
  }
  int dim = P.split2d ? ((depth % 2 == 0) ? 1 : 0) : 1;  // :50-51 split_axes = 1
  int s = r.size(dim);
  cellid_t tr1 = r.top_right(), bl1 = r.bottom_left();
  tr1[dim] = (coord_t)(tr1[dim] - 2 * (s / 4));
  bl1[dim] = tr1[dim];
  rect_t r1(r.bottom_left(), tr1), r2(bl1, r.top_right());
  cellid_t tr2 = e.top_right(), bl2 = e.bottom_left();
  tr2[dim] = (coord_t)(tr1[dim] + 2);
  bl2[dim] = (coord_t)(bl1[dim] - 2);
  rect_t e1(e.bottom_left(), tr2), e2(bl2, e.top_right());
  create_pieces(P, r1, e1, level - 1, depth + 1);
  create_pieces(P, r2, e2, level - 1, depth + 1);
}

static void init_piece_data(const float *full, int X, GridDataset *ds) {
  // readDataAndInit (:530-577): the dataset wraps the rows of its ext rect; with
  // 2D blocks the window is copied out of the full field.
  const rect_t &e = ds->m_ext_rect;
  int x0 = e.left() / 2, y0 = e.bottom() / 2, nx = e.size(0) / 2 + 1, ny = e.size(1) / 2 + 1;
  std::vector<float> win((size_t)nx * ny);
  for (int y = 0; y < ny; ++y)
    std::memcpy(&win[(size_t)y * nx], full + (size_t)(y0 + y) * X + x0, sizeof(float) * nx);
  ds->init(win.data());
}

static double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static void run_pipeline(Pipeline &P, const float *full) {
  rect_t r(0, 0, 2 * (P.X - 1), 2 * (P.Y - 1));
  create_pieces(P, r, r, P.levels, 0);  // :40-48
  P.nleaves = P.pieces.size();
  double t0 = now_ms();
  // computeSubdomainMsgraphs / computeMsGraph (:121-140, :493-528)
  for (size_t i = 0; i < P.nleaves; ++i) {
    Piece &p = P.pieces[i];
    init_piece_data(full, P.X, p.ds);
    if (P.ocl) {
      p.ds->work_ocl();
      p.ds->writeout_connectivity_ocl(p.msc);
    } else {
      p.ds->work();
      p.ds->writeout_connectivity(p.msc);
    }
    P.pair_overwrites += p.ds->pair_overwrites;
  }
  double t1 = now_ms();
  // mergePiecesUp (:258-306): node N+k = merge_up(2k, 2k+1)
  size_t N = P.nleaves;
  for (size_t k = 0; k + 1 < N; ++k) {
    Piece np;
    np.level = P.pieces[2 * k].level + 1;
    np.msc = merge_up(*P.pieces[2 * k].msc, *P.pieces[2 * k + 1].msc);
    P.pieces.push_back(np);
  }
  double t2 = now_ms();
  // :651-652
  GridMSComplex *root = P.pieces.back().msc;
  if (P.tresh > 0.0) {
    simplify(root, P.canc, P.tresh, &P.ncancel);
    un_simplify(root, P.canc);
    dump_msc(*root, P.root_after_simplify);
    P.have_root_snapshot = true;
  }
  double t3 = now_ms();
  // mergePiecesDown + finalMergeDownPiecesInRange (:308-395): every internal
  // node, root first, pushes into its two children.
  for (size_t node = P.pieces.size(); node-- > N;) {
    size_t k = node - N;
    merge_down(*P.pieces[node].msc, *P.pieces[2 * k].msc, *P.pieces[2 * k + 1].msc);
  }
  double t4 = now_ms();
  // collectSubdomainManifolds / collectManifold (:397-490)
  for (size_t i = 0; i < N; ++i) {
    Piece &p = P.pieces[i];
    GridDataset *ds = new GridDataset(p.ds->m_rect, p.ds->m_ext_rect);
    init_piece_data(full, P.X, ds);
    if (P.ocl) ds->work_ocl(false);
    else ds->work();
    ds->postMergeFillDiscs(p.msc);
    delete ds;
    for (auto *cp : p.msc->m_cps) {
      if (cp->isBoundryCancelable) continue;
      if (!cp->asc_disc.empty()) {
        auto &f = P.disc_files[std::make_pair(0, cp->cellid)];
        f.insert(f.end(), cp->asc_disc.begin(), cp->asc_disc.end());
      }
      if (!cp->des_disc.empty()) {
        auto &f = P.disc_files[std::make_pair(1, cp->cellid)];
        f.insert(f.end(), cp->des_disc.begin(), cp->des_disc.end());
      }
    }
  }
  double t5 = now_ms();
  P.t_stage[0] = t1 - t0; P.t_stage[1] = t2 - t1; P.t_stage[2] = t3 - t2; P.t_stage[3] = t4 - t3; P.t_stage[4] = t5 - t4;
}

}  // namespace orc

// ---------------------------------------------------------------------------
// C API used by tests/ and bench.py (via oracle/oracle.py, ctypes).
// ---------------------------------------------------------------------------
using namespace orc;

struct orc_ds_h { GridDataset *ds; GridMSComplex *msc; };

extern "C" {

const char *orc_last_error();
static thread_local std::string g_err;
const char *orc_last_error() { return g_err.c_str(); }

// One GridDataset: init + work + writeout_connectivity (+ optional simplify
// and postMergeFillDiscs on its own complex, as with levels = 0).  mode 0:
// the CPU path; 1: the CPU path with the OpenCL kernels' compareCells
// (descending vertex sort); 2: work_ocl + writeout_connectivity_ocl.
void *orc_ds_run_mode(const float *window, const int16_t rect[4], const int16_t ext[4], double tresh, int fill_discs,
                      int mode) {
  try {
    orc_ds_h *h = new orc_ds_h;
    h->ds = new GridDataset(rect_t(rect[0], rect[1], rect[2], rect[3]), rect_t(ext[0], ext[1], ext[2], ext[3]));
    h->ds->init(window);
    h->msc = new GridMSComplex(h->ds->m_rect, h->ds->m_ext_rect);
    if (mode == 2) {
      h->ds->work_ocl();
      h->ds->writeout_connectivity_ocl(h->msc);
    } else {
      h->ds->desc_cmp = mode == 1;
      h->ds->work();
      h->ds->writeout_connectivity(h->msc);
    }
    if (tresh > 0.0) {
      canc_list_t canc;
      simplify(h->msc, canc, tresh, nullptr);
      un_simplify(h->msc, canc);
    }
    if (fill_discs) h->ds->postMergeFillDiscs(h->msc);
    return h;
  } catch (std::exception &e) {
    g_err = e.what();
    return nullptr;
  }
}
void *orc_ds_run(const float *window, const int16_t rect[4], const int16_t ext[4], double tresh, int fill_discs) {
  return orc_ds_run_mode(window, rect, ext, tresh, fill_discs, 0);
}
void orc_ds_free(void *p) {
  orc_ds_h *h = (orc_ds_h *)p;
  if (!h) return;
  delete h->ds; delete h->msc; delete h;
}
// Per-cell arrays in the reference layout: C order [x][y] over ext (y fastest).
int64_t orc_ds_ncells(void *p) { orc_ds_h *h = (orc_ds_h *)p; return (int64_t)h->ds->cnx * h->ds->cny; }
void orc_ds_cells(void *p, int8_t *flags, int16_t *pairs, int16_t *own) {
  orc_ds_h *h = (orc_ds_h *)p;
  size_t n = (size_t)h->ds->cnx * h->ds->cny;
  std::memcpy(flags, h->ds->flags.data(), n);
  for (size_t i = 0; i < n; ++i) {
    pairs[2 * i] = h->ds->pairs[i][0]; pairs[2 * i + 1] = h->ds->pairs[i][1];
    own[2 * i] = h->ds->own[i][0]; own[2 * i + 1] = h->ds->own[i][1];
  }
}
int64_t orc_ds_overwrites(void *p) { return ((orc_ds_h *)p)->ds->pair_overwrites; }

static void *new_dump(const GridMSComplex &m) { MscDump *d = new MscDump; dump_msc(m, *d); return d; }
void *orc_ds_msc_dump(void *p) { return new_dump(*((orc_ds_h *)p)->msc); }

// Dump accessors. sizes[0]=ncp, [1]=n_asc, [2]=n_des, [3]=n_adisc, [4]=n_ddisc
void orc_dump_sizes(void *p, int64_t *sizes) {
  MscDump *d = (MscDump *)p;
  sizes[0] = (int64_t)d->fn.size(); sizes[1] = (int64_t)d->asc.size(); sizes[2] = (int64_t)d->des.size();
  sizes[3] = (int64_t)d->adisc.size() / 2; sizes[4] = (int64_t)d->ddisc.size() / 2;
}
void orc_dump_fill(void *p, int16_t *rect_ext, int16_t *cellid, float *fn, uint32_t *pair_idx, uint8_t *flags,
                   uint32_t *asc_off, uint32_t *asc, uint32_t *des_off, uint32_t *des,
                   uint32_t *adisc_off, int16_t *adisc, uint32_t *ddisc_off, int16_t *ddisc) {
  MscDump *d = (MscDump *)p;
  std::memcpy(rect_ext, d->rect, 8); std::memcpy(rect_ext + 4, d->ext, 8);
  auto cp = [](void *dst, const void *src, size_t n) { if (n) std::memcpy(dst, src, n); };
  cp(cellid, d->cellid.data(), d->cellid.size() * 2);
  cp(fn, d->fn.data(), d->fn.size() * 4);
  cp(pair_idx, d->pair_idx.data(), d->pair_idx.size() * 4);
  cp(flags, d->flags.data(), d->flags.size());
  cp(asc_off, d->asc_off.data(), d->asc_off.size() * 4);
  cp(asc, d->asc.data(), d->asc.size() * 4);
  cp(des_off, d->des_off.data(), d->des_off.size() * 4);
  cp(des, d->des.data(), d->des.size() * 4);
  cp(adisc_off, d->adisc_off.data(), d->adisc_off.size() * 4);
  cp(adisc, d->adisc.data(), d->adisc.size() * 2);
  cp(ddisc_off, d->ddisc_off.data(), d->ddisc_off.size() * 4);
  cp(ddisc, d->ddisc.data(), d->ddisc.size() * 2);
}
void orc_dump_free(void *p) { delete (MscDump *)p; }

// Whole pipeline (GridDataManager ctor), full field x-fastest X*Y; ocl as
// the -ocl flag.
void *orc_pipeline_run_ocl(const float *full, int X, int Y, int levels, double tresh, int split2d, int ocl) {
  try {
    Pipeline *P = new Pipeline;
    P->X = X; P->Y = Y; P->levels = levels; P->tresh = tresh; P->split2d = split2d; P->ocl = ocl;
    run_pipeline(*P, full);
    return P;
  } catch (std::exception &e) {
    g_err = e.what();
    return nullptr;
  }
}
void *orc_pipeline_run(const float *full, int X, int Y, int levels, double tresh, int split2d) {
  return orc_pipeline_run_ocl(full, X, Y, levels, tresh, split2d, 0);
}
void orc_pipeline_free(void *p) { delete (Pipeline *)p; }
int64_t orc_pipeline_nleaves(void *p) { return (int64_t)((Pipeline *)p)->nleaves; }
int64_t orc_pipeline_npieces(void *p) { return (int64_t)((Pipeline *)p)->pieces.size(); }
void *orc_pipeline_piece_dump(void *p, int64_t i) { return new_dump(*((Pipeline *)p)->pieces[i].msc); }
void *orc_pipeline_root_simplified_dump(void *p) {
  Pipeline *P = (Pipeline *)p;
  if (!P->have_root_snapshot) return nullptr;
  return new MscDump(P->root_after_simplify);
}
int64_t orc_pipeline_ncancel(void *p) { return ((Pipeline *)p)->ncancel; }
// Simplification counters of the calling thread's last runs (reset on read).
void orc_simplify_stats(uint64_t *out) {
  out[0] = g_sstats.pushes; out[1] = g_sstats.pops; out[2] = g_sstats.cancels; out[3] = g_sstats.new_edges;
  out[4] = g_sstats.resubmits; out[5] = g_sstats.max_heap; out[6] = g_sstats.erase_work;
  g_sstats = SimplifyStats();
}
int64_t orc_pipeline_overwrites(void *p) { return ((Pipeline *)p)->pair_overwrites; }
void orc_pipeline_times(void *p, double *t) { std::memcpy(t, ((Pipeline *)p)->t_stage, sizeof(double) * 5); }
// Disc "files": count, then per file (kind, x, y, n) headers and concatenated cells.
int64_t orc_pipeline_ndisc_files(void *p) { return (int64_t)((Pipeline *)p)->disc_files.size(); }
int64_t orc_pipeline_disc_cells(void *p) {
  int64_t n = 0;
  for (auto &kv : ((Pipeline *)p)->disc_files) n += (int64_t)kv.second.size();
  return n;
}
void orc_pipeline_discs(void *p, int32_t *hdr, int16_t *cells) {
  size_t k = 0, c = 0;
  for (auto &kv : ((Pipeline *)p)->disc_files) {
    hdr[4 * k] = kv.first.first; hdr[4 * k + 1] = kv.first.second[0]; hdr[4 * k + 2] = kv.first.second[1];
    hdr[4 * k + 3] = (int32_t)kv.second.size();
    for (auto &q : kv.second) { cells[2 * c] = q[0]; cells[2 * c + 1] = q[1]; ++c; }
    ++k;
  }
}

}  // extern "C"
