// merge.cu -- piece merges of Morse-Smale complexes on the device, one merge
// per thread: GridMSComplex::merge_up and merge_down
// (dmsc/src/grid_mscomplex.cpp:7-322) as restated in merge_graph.cuh, the
// independent merges of one tree level in separate blocks of one launch; and
// the conversions between a CSR complex and the mutable graph.  This is the
// path for small pieces and the fallback of the parallel merges
// (merge_par.cu).
#include "dmsc_common.cuh"
#include "dmsc_internal.h"
#include "merge_graph.cuh"
#include "msc_graph.cuh"
#include "grid_types.h"

namespace dmsc {

// One block per merge of a tree level; thread 0 works, on local copies of
// the graph descriptors (kept in registers rather than reloaded from global
// memory after every store through a list pointer).
__global__ void k_merge_up(MGraph *graphs, const int3 *jobs, const CRect *ixns, int njobs, uint32_t *status) {
  int b = blockIdx.x;
  if (b >= njobs || threadIdx.x != 0) return;
  int3 jb = jobs[b];  // (left child, right child, output)
  MGraph ga = graphs[jb.x], gb = graphs[jb.y], go = graphs[jb.z];
  MGraph *in[2] = {&ga, &gb};
  merge_up_one(in, go, ixns[b], status);
  if (go.G.fail) set_status(status, ST_SIMPLIFY_LIMIT);
  graphs[jb.z] = go;
}

__global__ void k_merge_down(MGraph *graphs, const int3 *jobs, const CRect *ixns, int njobs, uint32_t *status) {
  int b = blockIdx.x;
  if (b >= njobs || threadIdx.x != 0) return;
  int3 jb = jobs[b];  // (parent, child 1, child 2)
  MGraph P = graphs[jb.x], C1 = graphs[jb.y], C2 = graphs[jb.z];
  merge_down_boundary(P, ixns[b], status);
  if (P.G.fail) set_status(status, ST_SIMPLIFY_LIMIT);
  if (!P.G.fail) merge_down_child(P, C1, status);
  if (C1.G.fail) set_status(status, ST_SIMPLIFY_LIMIT);
  if (!P.G.fail && !C1.G.fail) merge_down_child(P, C2, status);
  if (C2.G.fail) set_status(status, ST_SIMPLIFY_LIMIT);
  graphs[jb.x] = P;
  graphs[jb.y] = C1;
  graphs[jb.z] = C2;
}

// ---------------------------------------------------------------------------
// conversions between a CSR complex and an MGraph (parallel)
// ---------------------------------------------------------------------------
__global__ void k_mg_from_csr(MGraph m, uint32_t n, const uint32_t *cellid, const float *fn, const uint8_t *flags,
                              const uint32_t *pair_idx, const uint32_t *aoff, const uint32_t *asc, const uint32_t *doff,
                              const uint32_t *des, uint32_t slack, bool fill_tab, uint32_t *status) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    m.G.cellid[i] = cellid[i];
    m.fn[i] = fn[i];
    m.G.flags[i] = flags[i];
    m.G.pair_idx[i] = pair_idx[i];
    for (int w = 0; w < 2; ++w) {
      const uint32_t *o = w ? doff : aoff, *src = w ? des : asc;
      uint32_t b = o[i], e = o[i + 1];
      // initial lists: asc runs at aoff[i] + i*slack, des runs after all asc runs
      unsigned long long base = w ? (unsigned long long)aoff[n] + (unsigned long long)slack * n + doff[i] + (unsigned long long)slack * i
                                  : aoff[i] + (unsigned long long)slack * i;
      uint32_t r = 0;
      for (uint32_t k = b; k < e; ++k) {
        if (r > 0 && m.G.L.pool[base + r - 1].x == src[k]) m.G.L.pool[base + r - 1].y += 1;
        else m.G.L.pool[base + r++] = make_uint2(src[k], 1u);
      }
      m.G.L.off[2 * i + w] = (uint32_t)base; m.G.L.nrun[2 * i + w] = r; m.G.L.cap[2 * i + w] = (e - b) + slack;
      m.G.L.total[2 * i + w] = e - b;
    }
    // the cell -> index table (cell ids are unique within a complex)
    if (fill_tab) {
      const long long sl = m.slot(cellid[i]);
      if (sl >= 0) m.tab[sl] = i;
      else if (status) atomicOr(status, ST_INVARIANT);  // a critical cell outside the complex's box
    }
  }
}

__global__ void k_mg_totals(MGraph m, int which, uint32_t *out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m.G.ncp; i += gridDim.x * blockDim.x)
    out[i] = m.G.L.total[2 * i + which];
}
__global__ void k_mg_to_csr(MGraph m, int which, const uint32_t *off, uint32_t *out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m.G.ncp; i += gridDim.x * blockDim.x) {
    uint32_t l = 2 * i + which, o = off[i];
    const uint2 *p = m.G.L.pool + m.G.L.off[l];
    for (uint32_t k = 0; k < m.G.L.nrun[l]; ++k)
      for (uint32_t c = 0; c < p[k].y; ++c) out[o++] = p[k].x;
  }
}

static unsigned nblk(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (unsigned)(b < 1 ? 1 : b);
}

// Allocates an MGraph with room for `cap` critical points and a list pool of
// `pool` runs, and fills it from a CSR complex (n critical points, may be 0);
// each list starts with room for `slack` more runs than it holds.  The cell
// table covers src.bbox; `tab` (may be null) is a table over that box that
// already maps src's cells, which the graph then takes over; `box` (may be
// null) replaces src.bbox as the table's box.
cudaError_t mgraph_alloc(MGraphHost &h, const dmsc_msc &src, uint32_t cap, unsigned long long pool, cudaStream_t st,
                         uint32_t slack, uint32_t *tab, const int *box) {
  uint32_t n = (uint32_t)src.ncp;
  if (cap < n) cap = n;
  if (cap >= (1u << 30)) return cudaErrorInvalidValue;
  if (!box) box = src.bbox;
  const int tx0 = box[0], ty0 = box[1], tw = box[2] - box[0] + 1, th = box[3] - box[1] + 1;
  if (tw <= 0 || th <= 0) return cudaErrorInvalidValue;
  unsigned long long base = (unsigned long long)src.nasc + src.ndes + 2ull * slack * n;
  if (pool < base + 1024) pool = base + 1024;
  if (pool > 0xffffffffull) return cudaErrorInvalidValue;
  unsigned long long tmpc = 1ull << 20;
  size_t words = 4ull * cap + 8ull * cap + 2 * pool + 2 * tmpc + 64;
  cudaError_t e = cudaMallocAsync((void **)&h.buf, sizeof(uint32_t) * words, st);
  if (e != cudaSuccess) return e;
  const size_t tcells = (size_t)tw * th;
  const bool fill_tab = tab == nullptr;
  if (fill_tab) {
    e = cudaMallocAsync((void **)&tab, sizeof(uint32_t) * tcells, st);
    if (e != cudaSuccess) { cudaFreeAsync(h.buf, st); h.buf = nullptr; return e; }
    e = cudaMemsetAsync(tab, 0xFF, sizeof(uint32_t) * tcells, st);
  }
  h.tab = tab;
  uint32_t *p = h.buf;
  MGraph &m = *reinterpret_cast<MGraph *>(h.raw);
  static_assert(sizeof(MGraph) <= sizeof(h.raw), "MGraphHost storage");
  m = MGraph();
  m.G.cellid = p; p += cap;
  m.fn = (float *)p; p += cap;
  m.G.pair_idx = p; p += cap;
  m.G.flags = (uint8_t *)p; p += cap;  // (1 byte used per word)
  m.G.L.off = p; p += 2ull * cap;
  m.G.L.nrun = p; p += 2ull * cap;
  m.G.L.cap = p; p += 2ull * cap;
  m.G.L.total = p; p += 2ull * cap;
  m.G.L.pool = (uint2 *)p; p += 2 * pool;
  m.G.tmp = (uint2 *)p; p += 2 * tmpc;
  m.G.tmp_cap = tmpc;
  m.G.L.top = base;
  m.G.L.pool_cap = pool;
  m.G.ncp = n;
  m.G.max_ops = ~0ull;
  m.G.ops = 0;
  m.G.fail = false;
  m.cap = cap;
  m.tab = tab;
  m.tx0 = tx0; m.ty0 = ty0; m.tw = tw; m.th = th;
  m.rect = CRect{src.rect[0], src.rect[1], src.rect[2], src.rect[3]};
  m.ext = CRect{src.ext[0], src.ext[1], src.ext[2], src.ext[3]};
  if (e == cudaSuccess && n) {
    k_mg_from_csr<<<nblk(n), 256, 0, st>>>(m, n, src.cellid.p, src.fn.p, src.flags.p, src.pair_idx.p, src.aoff.p,
                                          src.asc.p, src.doff.p, src.des.p, slack, fill_tab, h.status);
    DMSC_LAUNCHED(1);
    e = cudaGetLastError();
  }
  return e;
}

__global__ void k_cell_box(long long n, const uint32_t *cellid, int *box) {
  int b[4] = {1 << 30, 1 << 30, -1, -1};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(cellid[i] & 0xffffu), y = (int)(cellid[i] >> 16);
    b[0] = min(b[0], x); b[1] = min(b[1], y); b[2] = max(b[2], x); b[3] = max(b[3], y);
  }
  for (int o = 16; o > 0; o >>= 1) {
    b[0] = min(b[0], __shfl_xor_sync(0xffffffffu, b[0], o)); b[1] = min(b[1], __shfl_xor_sync(0xffffffffu, b[1], o));
    b[2] = max(b[2], __shfl_xor_sync(0xffffffffu, b[2], o)); b[3] = max(b[3], __shfl_xor_sync(0xffffffffu, b[3], o));
  }
  if ((threadIdx.x & 31) == 0 && b[2] >= 0) {
    atomicMin(box, b[0]); atomicMin(box + 1, b[1]); atomicMax(box + 2, b[2]); atomicMax(box + 3, b[3]);
  }
}

// The box of a complex's critical cells (its ext rect when it has none).
cudaError_t cell_box(dmsc_msc &m, cudaStream_t st) {
  if (m.ncp <= 0) {
    for (int i = 0; i < 4; ++i) m.bbox[i] = m.ext[i];
    return cudaSuccess;
  }
  int *d = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&d, 16, st);
  if (e != cudaSuccess) return e;
  const int init[4] = {1 << 30, 1 << 30, -1, -1};
  int hb[4];
  e = cudaMemcpyAsync(d, init, 16, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    k_cell_box<<<nblk(m.ncp), 256, 0, st>>>(m.ncp, m.cellid.p, d);
    DMSC_LAUNCHED(1);
    e = cudaMemcpyAsync(hb, d, 16, cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFreeAsync(d, st);
  if (e == cudaSuccess)
    for (int i = 0; i < 4; ++i) m.bbox[i] = hb[i];
  return e;
}

void mgraph_free(MGraphHost &h, cudaStream_t st) {
  if (h.buf) cudaFreeAsync(h.buf, st);
  if (h.tab) cudaFreeAsync(h.tab, st);
  h.buf = nullptr;
  h.tab = nullptr;
}

// Runs one tree level of merges; graphs[] is a device array of MGraph.
cudaError_t merge_level(bool up, MGraphHost *hosts, int ngraphs, const int *jobs3, const int *ixn4, int njobs,
                        uint32_t *status, cudaStream_t st) {
  MGraph *dg = nullptr;
  int3 *dj = nullptr;
  CRect *dx = nullptr;
  size_t bytes = sizeof(MGraph) * ngraphs + sizeof(int3) * njobs + sizeof(CRect) * njobs + 64;
  char *buf = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&buf, bytes, st);
  if (e != cudaSuccess) return e;
  dg = (MGraph *)buf;
  dj = (int3 *)(buf + sizeof(MGraph) * ngraphs);
  dx = (CRect *)((char *)dj + sizeof(int3) * njobs);
  // host images
  MGraph *hg = new MGraph[ngraphs];
  for (int i = 0; i < ngraphs; ++i) hg[i] = *reinterpret_cast<MGraph *>(hosts[i].raw);
  e = cudaMemcpyAsync(dg, hg, sizeof(MGraph) * ngraphs, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dj, jobs3, sizeof(int3) * njobs, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, ixn4, sizeof(CRect) * njobs, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    if (up) k_merge_up<<<njobs, 32, 0, st>>>(dg, dj, dx, njobs, status);
    else k_merge_down<<<njobs, 32, 0, st>>>(dg, dj, dx, njobs, status);
    DMSC_LAUNCHED(1);
    e = cudaGetLastError();
  }
  // bring back the counts and pool tops the kernels changed
  if (e == cudaSuccess) e = cudaMemcpyAsync(hg, dg, sizeof(MGraph) * ngraphs, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess)
    for (int i = 0; i < ngraphs; ++i) *reinterpret_cast<MGraph *>(hosts[i].raw) = hg[i];
  delete[] hg;
  cudaFreeAsync(buf, st);
  return e;
}

uint32_t mgraph_ncp(const MGraphHost &h) { return reinterpret_cast<const MGraph *>(h.raw)->G.ncp; }
unsigned long long mgraph_pool_used(const MGraphHost &h) { return reinterpret_cast<const MGraph *>(h.raw)->G.L.top; }
bool mgraph_failed(const MGraphHost &h) { return reinterpret_cast<const MGraph *>(h.raw)->G.fail; }
void mgraph_set_rects(MGraphHost &h, const int rect[4], const int ext[4]) {
  MGraph &m = *reinterpret_cast<MGraph *>(h.raw);
  m.rect = CRect{rect[0], rect[1], rect[2], rect[3]};
  m.ext = CRect{ext[0], ext[1], ext[2], ext[3]};
}

// Writes an MGraph back into a CSR complex (rect/ext are the caller's).
cudaError_t mgraph_to_csr(const MGraphHost &h, dmsc_msc &out, cudaStream_t st) {
  const MGraph &m = *reinterpret_cast<const MGraph *>(h.raw);
  uint32_t n = m.G.ncp;
  out.any_bcancel = true;  // merged complexes carry the pieces' boundary pairs
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = out.cellid.ensure(n + 1, st);
  if (e == cudaSuccess) e = out.fn.ensure(n + 1, st);
  if (e == cudaSuccess) e = out.pair_idx.ensure(n + 1, st);
  if (e == cudaSuccess) e = out.flags.ensure(n + 1, st);
  if (e == cudaSuccess) e = out.aoff.ensure(n + 1, st);
  if (e == cudaSuccess) e = out.doff.ensure(n + 1, st);
  if (e != cudaSuccess) return e;
  out.ncp = n;
  if (n) {
    e = cudaMemcpyAsync(out.cellid.p, m.G.cellid, 4ull * n, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out.fn.p, m.fn, 4ull * n, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out.pair_idx.p, m.G.pair_idx, 4ull * n, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out.flags.p, m.G.flags, n, cudaMemcpyDeviceToDevice, st);
  }
  for (int w = 0; w < 2 && e == cudaSuccess; ++w) {
    uint32_t *tot = nullptr;
    e = cudaMallocAsync((void **)&tot, 4ull * (n + 1), st);
    if (e != cudaSuccess) break;
    uint32_t *off = w ? out.doff.p : out.aoff.p;
    if (n) {
      k_mg_totals<<<nblk(n), 256, 0, st>>>(m, w, tot);
      DMSC_LAUNCHED(1);
    }
    e = scan_exclusive_u32(tot, n, off, off + n, st);
    uint32_t total = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total, off + n, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    DevBuf<uint32_t> &lb = w ? out.des : out.asc;
    if (e == cudaSuccess) e = lb.ensure((size_t)total + 1, st);
    if (e == cudaSuccess && n) {
      k_mg_to_csr<<<nblk(n), 256, 0, st>>>(m, w, off, lb.p);
      DMSC_LAUNCHED(1);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) (w ? out.ndes : out.nasc) = total;
    cudaFreeAsync(tot, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e;
}

}  // namespace dmsc
