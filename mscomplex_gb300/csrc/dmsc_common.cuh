// dmsc_common.cuh -- shared definitions of the grid Morse-Smale CUDA path (sm_103a).
//
// Cell model (as in dmsc/include/grid_dataset.h:207-210): a refined grid in
// which vertex (i,j) is cell (2i,2j); dim = (x&1)+(y&1).  On the device every
// vertex (i,j) of a piece's ext window owns four cells -- the vertex V, the
// edge to its right H=(2i+1,2j), the edge above it Vt=(2i,2j+1) and the face
// to its upper right F=(2i+1,2j+1) -- so per-cell arrays are "vertex-major
// quads": uchar4 gradient codes and uint4 owner labels per vertex.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace dmsc {

// Tile of vertices processed by one CTA of the gradient / label kernels.
constexpr int TX = 64;
constexpr int TY = 64;
constexpr int GRAD_THREADS = 512;
constexpr int SLOTS_SIDE = 2 * TX + 2 * TY;   // border slots per grid kind (vertex / face) per tile
constexpr int SLOTS_PER_TILE = 2 * SLOTS_SIDE;

// Gradient code, one byte per cell.  bits 0-1: direction of the paired cell,
// bit 2: PAIRED, bit 3: CRITICAL.  (code >> 2) & 3 is the reference's cell
// flag byte (CELLFLAG_PAIRED = 1, CELLFLAG_CRITCAL = 2, grid_dataset.h:40-45).
enum : uint32_t { DIR_PX = 0, DIR_MX = 1, DIR_PY = 2, DIR_MY = 3 };
enum : uint32_t { CODE_PAIRED = 4, CODE_CRIT = 8 };
constexpr uint8_t CAND_NONE = 0xFF;

// Device status word bits (OR-ed by kernels, read by the host after a stage).
enum : uint32_t {
  ST_NAN_INPUT = 1u << 0,      // a NaN height was seen (outside the supported input domain)
  ST_PAIR_CONFLICT = 1u << 1,  // a cell chosen by its facet also chose a cofacet (never expected)
  ST_CYCLE = 1u << 2,          // a gradient path did not terminate (never expected)
  ST_RESOLVE_LIMIT = 1u << 3,  // border-table resolution hit its iteration bound
  ST_BAD_LABEL = 1u << 4,      // a saddle's neighbour label did not resolve to a critical cell
  ST_SIMPLIFY_LIMIT = 1u << 5, // simplification pool / iteration bound exceeded
  ST_INVARIANT = 1u << 6,      // a reference logic_error condition (merge / disc invariants)
  ST_CAPACITY = 1u << 7,       // critical-point arrays too small (host grows them and reruns)
  ST_FALLBACK = 1u << 8,       // a parallel merge met a case only the one-thread restatement reproduces
};

constexpr uint32_t LABEL_NONE = 0xFFFFFFFFu;

// Border-table entries (uint64): tag in bits 62-63.
constexpr uint64_t BT_INVALID = 0;
constexpr uint64_t BT_ROOT = 1ull << 62;    // payload: seg << 8 | rank (critical cell in its row segment)
constexpr uint64_t BT_EXIT = 2ull << 62;    // payload: global slot of the next border cell
constexpr uint64_t BT_FINAL = 3ull << 62;   // payload: cp index
__host__ __device__ __forceinline__ uint64_t bt_tag(uint64_t e) { return e & (3ull << 62); }
__host__ __device__ __forceinline__ uint64_t bt_payload(uint64_t e) { return e & ((1ull << 62) - 1); }

// Geometry of one piece: the ext window (vertex extents, global bottom-left)
// and its rect, in cell coordinates RELATIVE to the ext bottom-left.
struct GridGeom {
  int ex0, ey0;           // ext bottom-left, global cell coordinates (even)
  int vnx, vny;           // vertices of the ext window
  int cx, cy;             // ext size in cells: 2(vnx-1), 2(vny-1)
  int rx0, ry0, rx1, ry1; // rect relative to ext (even)
  int ntx, nty;           // tiles of TX x TY vertices
  long long pitch;        // height row pitch in elements (>= vnx)
  // Offsets of this grid's border slots and row segments in tables shared by
  // a batch of grids (0 for a grid on its own): the border table's EXIT and
  // ROOT entries carry batch-wide indices.
  long long sbase = 0, gbase = 0;
  // compareCells sorts a cell's vertices descending (the reference's OpenCL
  // kernels, dmsc/resources/assigngradient.cl:40-87) instead of ascending
  // (its CPU path, dmsc/src/grid_dataset.cpp:1530-1531)
  int desc = 0;
};

__host__ __device__ __forceinline__ uint32_t pack_cellid(int x, int y) {
  return (uint32_t)(uint16_t)(int16_t)x | ((uint32_t)(uint16_t)(int16_t)y << 16);
}

// Order-preserving map of a float to uint32; -0.0 and +0.0 map to the same key
// because the reference compares values with != / < (grid_dataset.h:158-167).
__device__ __forceinline__ uint32_t ord_key(float f) {
  uint32_t b = __float_as_uint(f);
  if (b == 0x80000000u) b = 0u;
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// Border slot of a cell at local (i,j) of a tile with clipped extents (w,h).
__host__ __device__ __forceinline__ int border_index(int i, int j, int w, int h) {
  if (j == 0) return i;
  if (j == h - 1) return TX + i;
  if (i == 0) return 2 * TX + j;
  return 2 * TX + TY + j;  // i == w-1
}
__host__ __device__ __forceinline__ bool on_tile_border(int i, int j, int w, int h) {
  return i == 0 || j == 0 || i == w - 1 || j == h - 1;
}

// Clipped tile extents of the vertex grid (kind 0) or the face grid (kind 1).
__host__ __device__ __forceinline__ void tile_extent(const GridGeom &g, int bx, int by, int kind, int &w, int &h) {
  int nx = g.vnx - kind, ny = g.vny - kind;
  w = nx - bx * TX; if (w > TX) w = TX;
  h = ny - by * TY; if (h > TY) h = TY;
}

// Global border slot of the vertex (kind 0) or face (kind 1) with global
// vertex/face coordinates (gi, gj), which must lie on its tile's border.
__host__ __device__ __forceinline__ long long border_slot(const GridGeom &g, int kind, int gi, int gj) {
  int bx = gi / TX, by = gj / TY;
  int w, h;
  tile_extent(g, bx, by, kind, w, h);
  return ((long long)by * g.ntx + bx) * SLOTS_PER_TILE + kind * SLOTS_SIDE +
         border_index(gi - bx * TX, gj - by * TY, w, h);
}

}  // namespace dmsc
