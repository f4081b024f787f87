// dmsc_capi.cu -- extern "C" boundary of libdmsc.so (declared in include/dmsc.h).
//
// Host-side objects mirror the reference's C++ classes: dmsc_dataset is a
// GridDataset (dmsc/include/grid_dataset.h:35-240) whose cell arrays live in
// device memory, dmsc_msc is a GridMSComplex (dmsc/include/grid_mscomplex.h)
// held as flat device arrays.  There is no CPU fallback: every computation
// here is a CUDA kernel launch.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "dmsc.h"
#include "dmsc_internal.h"
#include "grid_types.h"

using namespace dmsc;

namespace {
thread_local std::string g_err;

int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char *where) {
  cudaGetLastError();  // clear sticky-free errors
  std::string m = std::string(where) + ": " + cudaGetErrorString(e);
  return fail(e == cudaErrorMemoryAllocation ? DMSC_ERR_OOM : DMSC_ERR_CUDA, m);
}
}  // namespace

int dmsc::set_last_error(int code, const char *msg) { return fail(code, msg); }

#define CK(call)                                             \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);      \
  } while (0)

static cudaStream_t pick(dmsc_ctx *c, void *s) { return s ? (cudaStream_t)s : c->stream; }

// Maps the device status word to an error code.
static int status_to_error(uint32_t st) {
  if (!st) return DMSC_OK;
  if (st & ST_NAN_INPUT) return fail(DMSC_ERR_INPUT, "NaN height in input (outside the supported domain)");
  if (st & (ST_RESOLVE_LIMIT | ST_SIMPLIFY_LIMIT))
    return fail(DMSC_ERR_DEVICE_TIMEOUT, "a bounded device loop ran out of iterations (status " + std::to_string(st) + ")");
  return fail(DMSC_ERR_INVARIANT, "device invariant violated (status " + std::to_string(st) + ")");
}

namespace {
uint32_t *pin_take();  // pinned 16-word slots (below)
void pin_give(uint32_t *p);
}  // namespace

extern "C" {

const char *dmsc_last_error(void) { return g_err.c_str(); }

int dmsc_init(int device, dmsc_ctx **out) {
  if (!out) return fail(DMSC_ERR_BAD_ARG, "out is null");
  int n = 0;
  CK(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return fail(DMSC_ERR_BAD_ARG, "no such device");
  CK(cudaSetDevice(device));
  // Scratch comes from the device's default stream-ordered pool.  Its default
  // release threshold (0) hands freed memory back at every synchronisation,
  // so each call would map its scratch anew; keep it cached instead
  // (dmsc_shutdown trims the pool).
  cudaMemPool_t pool;
  CK(cudaDeviceGetDefaultMemPool(&pool, device));
  uint64_t keep = ~0ull;
  CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
  dmsc_ctx *c = new dmsc_ctx;
  c->device = device;
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete c; return cuda_fail(e, "cudaStreamCreate"); }
  *out = c;
  return DMSC_OK;
}

int dmsc_shutdown(dmsc_ctx *c) {
  if (!c) return fail(DMSC_ERR_BAD_ARG, "ctx is null");
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  cudaStreamDestroy(c->stream);
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, c->device) == cudaSuccess) cudaMemPoolTrimTo(pool, 0);
  delete c;
  return DMSC_OK;
}

// ---------------------------------------------------------------------------
// dataset
// ---------------------------------------------------------------------------
int dmsc_dataset_create(dmsc_ctx *ctx, const int16_t rect[4], const int16_t ext[4], dmsc_dataset **out) {
  if (!ctx || !rect || !ext || !out) return fail(DMSC_ERR_BAD_ARG, "null argument");
  for (int i = 0; i < 4; ++i) {
    if (rect[i] < 0 || ext[i] < 0) return fail(DMSC_ERR_BAD_ARG, "negative coordinate");
    if ((rect[i] & 1) || (ext[i] & 1)) return fail(DMSC_ERR_BAD_ARG, "rect and ext corners must be vertices (even coordinates)");
  }
  if (rect[0] > rect[2] || rect[1] > rect[3] || ext[0] > ext[2] || ext[1] > ext[3])
    return fail(DMSC_ERR_BAD_ARG, "rect corners out of order");
  if (rect[0] < ext[0] || rect[1] < ext[1] || rect[2] > ext[2] || rect[3] > ext[3])
    return fail(DMSC_ERR_BAD_ARG, "ext must contain rect");
  if (ext[2] - ext[0] < 2 || ext[3] - ext[1] < 2) return fail(DMSC_ERR_BAD_ARG, "ext needs at least 2x2 vertices");
  if (ext[2] > 32766 || ext[3] > 32766) return fail(DMSC_ERR_INT16_OVERFLOW, "cell ids exceed int16");
  dmsc_dataset *d = new dmsc_dataset;
  d->ctx = ctx;
  std::memcpy(d->rect, rect, 8);
  std::memcpy(d->ext, ext, 8);
  GridGeom &g = d->g;
  g.ex0 = ext[0]; g.ey0 = ext[1];
  g.vnx = (ext[2] - ext[0]) / 2 + 1; g.vny = (ext[3] - ext[1]) / 2 + 1;
  g.cx = 2 * (g.vnx - 1); g.cy = 2 * (g.vny - 1);
  g.rx0 = rect[0] - ext[0]; g.ry0 = rect[1] - ext[1]; g.rx1 = rect[2] - ext[0]; g.ry1 = rect[3] - ext[1];
  g.ntx = (g.vnx + TX - 1) / TX; g.nty = (g.vny + TY - 1) / TY;
  g.pitch = g.vnx;
  *out = d;
  return DMSC_OK;
}

int dmsc_dataset_destroy(dmsc_dataset *d) {
  if (!d) return fail(DMSC_ERR_BAD_ARG, "dataset is null");
  cudaSetDevice(d->ctx->device);
  cudaStreamSynchronize(d->ctx->stream);
  delete d;
  return DMSC_OK;
}

int dmsc_dataset_init(dmsc_dataset *d, const float *heights, int64_t pitch, int on_device, void *stream) {
  if (!d || !heights) return fail(DMSC_ERR_BAD_ARG, "null argument");
  GridGeom &g = d->g;
  if (pitch < g.vnx) return fail(DMSC_ERR_BAD_ARG, "pitch smaller than the ext window width");
  CK(cudaSetDevice(d->ctx->device));
  cudaStream_t st = pick(d->ctx, stream);
  if (on_device) {
    d->hgt = heights;
    g.pitch = pitch;
  } else {
    CK(d->hown.ensure((size_t)g.vnx * g.vny, st));
    CK(cudaMemcpy2DAsync(d->hown.p, sizeof(float) * g.vnx, heights, sizeof(float) * pitch, sizeof(float) * g.vnx,
                         g.vny, cudaMemcpyHostToDevice, st));
    d->hgt = d->hown.p;
    g.pitch = g.vnx;
  }
  d->worked = false;
  return DMSC_OK;
}

// Runs K1 (gradient) -> scan -> K3 (resolve) -> K4 (labels) on `st`.
// Returns after the device status is known.  desc: the OpenCL kernels'
// compareCells (work_ocl) instead of the CPU path's (work).
static int dataset_work(dmsc_dataset *d, void *stream, int desc) {
  if (!d) return fail(DMSC_ERR_BAD_ARG, "dataset is null");
  if (!d->hgt) return fail(DMSC_ERR_STATE, "dataset has no heights (call dmsc_dataset_init first)");
  d->g.desc = desc;
  CK(cudaSetDevice(d->ctx->device));
  cudaStream_t st = pick(d->ctx, stream);
  int rc = d->alloc_cells(st);
  if (rc) return rc;
  const GridGeom &g = d->g;
  const bool tm = d->ctx->timing;
  if (tm && !d->ev_ready) {
    for (auto &e : d->ev) CK(cudaEventCreate(&e));
    d->ev_ready = true;
  }
  CK(cudaMemsetAsync(d->scal.p, 0, sizeof(uint32_t) * 4, st));
  if (tm) CK(cudaEventRecord(d->ev[0], st));
  CK(launch_gradient(d->hgt, g, d->codes.p, d->terms.p, d->rowcnt.p, d->table.p, d->scal.p, st));
  if (tm) CK(cudaEventRecord(d->ev[1], st));
  CK(scan_exclusive_u8(d->rowcnt.p, (long long)(g.cy + 1) * g.ntx, d->offsets.p, d->scal.p + 1, st));
  if (tm) CK(cudaEventRecord(d->ev[2], st));
  CK(launch_resolve(d->table.p, d->nslots(), d->offsets.p, (long long)(g.cy + 1) * g.ntx, d->scal.p, st));
  if (tm) CK(cudaEventRecord(d->ev[3], st));
  if (d->cap <= 0) d->cap = (long long)g.vnx * g.vny / 16 + 4096;
  for (int attempt = 0; attempt < 2; ++attempt) {
    rc = d->alloc_cps(d->cap, st);
    if (rc) return rc;
    CK(cudaMemsetAsync(d->cp_acnt.p, 0, sizeof(uint32_t) * d->cap, st));
    CK(cudaMemsetAsync(d->cp_dcnt.p, 0, sizeof(uint32_t) * d->cap, st));
    CpOut cp{d->cp_cellid.p, d->cp_fn.p, d->cp_flags.p, d->cp_pair_cell.p, d->cp_des2.p,
             d->cp_asc2.p, d->cp_acnt.p, d->cp_dcnt.p, d->cap};
    if (tm) CK(cudaEventRecord(d->ev[3], st));
    CK(launch_labels(d->codes.p, d->terms.p, d->hgt, g, d->offsets.p, d->table.p, d->labels.p, cp, d->scal.p, st));
    if (tm) CK(cudaEventRecord(d->ev[4], st));
    {
      const uint32_t *w[4] = {d->scal.p, d->scal.p + 1, d->scal.p + 2, d->scal.p + 3};
      CK(read_words(d->host_scal, w, 4, st));
    }
    CK(cudaStreamSynchronize(st));
    d->ncp = d->host_scal[1];
    if (!(d->host_scal[0] & ST_CAPACITY)) break;
    d->cap = d->ncp + d->ncp / 8 + 1024;
    uint32_t clear = d->host_scal[0] & ~ST_CAPACITY;
    CK(cudaMemcpyAsync(d->scal.p, &clear, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  }
  if (d->host_scal[0] & ST_CAPACITY) return fail(DMSC_ERR_INVARIANT, "critical-point capacity could not be met");
  rc = status_to_error(d->host_scal[0]);
  if (rc) return rc;
  // pair_idx of critical cells that keep a pair (boundary rule; only with rect != ext)
  CK(d->cp_pair_idx.ensure(d->cap, st));
  if (d->rect_is_ext()) {
    if (d->ncp) CK(cudaMemsetAsync(d->cp_pair_idx.p, 0xFF, sizeof(uint32_t) * d->ncp, st));
  } else {
    CK(launch_pair_index(d->ncp, d->cp_cellid.p, d->cp_flags.p, d->cp_pair_cell.p, d->cp_pair_idx.p, d->scal.p, st));
    const uint32_t *w[1] = {d->scal.p};
    CK(read_words(d->host_scal, w, 1, st));
    CK(cudaStreamSynchronize(st));
    rc = status_to_error(d->host_scal[0]);
    if (rc) return rc;
  }
  d->worked = true;
  return DMSC_OK;
}

int dmsc_dataset_num_critical(dmsc_dataset *d, int64_t *n) {
  if (!d || !n) return fail(DMSC_ERR_BAD_ARG, "null argument");
  if (!d->worked) return fail(DMSC_ERR_STATE, "dataset_work has not run");
  *n = d->ncp;
  return DMSC_OK;
}

int dmsc_dataset_export_cells(dmsc_dataset *d, int8_t *flags, int16_t *pairs, int16_t *own, void *stream) {
  if (!d) return fail(DMSC_ERR_BAD_ARG, "dataset is null");
  if (!d->worked) return fail(DMSC_ERR_STATE, "dataset_work has not run");
  CK(cudaSetDevice(d->ctx->device));
  cudaStream_t st = pick(d->ctx, stream);
  const GridGeom &g = d->g;
  size_t n = (size_t)(g.cx + 1) * (g.cy + 1);
  DevBuf<int8_t> f;
  DevBuf<int16_t> p, o;
  if (flags) CK(f.ensure(n, st));
  if (pairs) CK(p.ensure(2 * n, st));
  if (own) CK(o.ensure(2 * n, st));
  CK(launch_export_cells(g, d->codes.p, d->labels.p, d->cp_cellid.p, d->ncp, f.p, p.p, o.p, st));
  if (flags) CK(cudaMemcpyAsync(flags, f.p, n, cudaMemcpyDeviceToHost, st));
  if (pairs) CK(cudaMemcpyAsync(pairs, p.p, 4 * n, cudaMemcpyDeviceToHost, st));
  if (own) CK(cudaMemcpyAsync(own, o.p, 4 * n, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return DMSC_OK;
}

int dmsc_dataset_export_critical(dmsc_dataset *d, int16_t *cellids, void *stream) {
  if (!d || !cellids) return fail(DMSC_ERR_BAD_ARG, "null argument");
  if (!d->worked) return fail(DMSC_ERR_STATE, "dataset_work has not run");
  CK(cudaSetDevice(d->ctx->device));
  cudaStream_t st = pick(d->ctx, stream);
  if (d->ncp) CK(cudaMemcpyAsync(cellids, d->cp_cellid.p, 4 * d->ncp, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return DMSC_OK;
}

int dmsc_dataset_work(dmsc_dataset *d, void *stream) { return dataset_work(d, stream, 0); }
int dmsc_dataset_work_ocl(dmsc_dataset *d, void *stream) { return dataset_work(d, stream, 1); }

// writeout_connectivity_ocl builds the same complex from the same cells: its
// saddle incidences (collect_saddle_conn_ocl) read the owners of a saddle's
// facets and cofacets inside ext, as writeout_connectivity reads them.
int dmsc_dataset_writeout_connectivity_ocl(dmsc_dataset *d, dmsc_msc **out, void *stream) {
  return dmsc_dataset_writeout_connectivity(d, out, stream);
}

int dmsc_dataset_writeout_connectivity(dmsc_dataset *d, dmsc_msc **out, void *stream) {
  if (!d || !out) return fail(DMSC_ERR_BAD_ARG, "null argument");
  if (!d->worked) return fail(DMSC_ERR_STATE, "dataset_work has not run");
  CK(cudaSetDevice(d->ctx->device));
  cudaStream_t st = pick(d->ctx, stream);
  // a complex passed in is overwritten in place (its device buffers are
  // reused, growing only when too small); otherwise a new one is made
  const bool fresh = *out == nullptr;
  if (!fresh && (*out)->ctx != d->ctx) return fail(DMSC_ERR_BAD_ARG, "complex belongs to another context");
  dmsc_msc *m = fresh ? new dmsc_msc : *out;
  m->ctx = d->ctx;
  std::memcpy(m->rect, d->rect, 8);
  std::memcpy(m->ext, d->ext, 8);
  for (int i = 0; i < 4; ++i) m->bbox[i] = d->ext[i];
  m->nadisc = m->nddisc = 0;
  for (auto &v : m->simp_stats) v = 0;
  if (d->ctx->timing && d->ev_ready) CK(cudaEventRecord(d->ev[5], st));
  int rc = m->writeout_from(*d, st);
  if (rc) {
    if (fresh) delete m;
    else m->ncp = m->nasc = m->ndes = 0;
    return rc;
  }
  if (d->ctx->timing && d->ev_ready) CK(cudaEventRecord(d->ev[6], st));
  *out = m;
  return DMSC_OK;
}

// ---------------------------------------------------------------------------
// complex
// ---------------------------------------------------------------------------
int dmsc_msc_destroy(dmsc_msc *m) {
  if (!m) return fail(DMSC_ERR_BAD_ARG, "complex is null");
  cudaSetDevice(m->ctx->device);
  cudaStreamSynchronize(m->ctx->stream);
  delete m;
  return DMSC_OK;
}

int dmsc_msc_sizes(dmsc_msc *m, int64_t sizes[5]) {
  if (!m || !sizes) return fail(DMSC_ERR_BAD_ARG, "null argument");
  sizes[0] = m->ncp; sizes[1] = m->nasc; sizes[2] = m->ndes; sizes[3] = m->nadisc; sizes[4] = m->nddisc;
  return DMSC_OK;
}

static int msc_export(dmsc_msc *m, int16_t rect_ext[8], int16_t *cellid, float *fn, uint32_t *pair_idx, uint8_t *flags,
                      uint32_t *asc_off, uint32_t *asc, uint32_t *des_off, uint32_t *des, uint32_t *adisc_off,
                      int16_t *adisc, uint32_t *ddisc_off, int16_t *ddisc, void *stream, bool sync) {
  if (!m) return fail(DMSC_ERR_BAD_ARG, "complex is null");
  CK(cudaSetDevice(m->ctx->device));
  cudaStream_t st = pick(m->ctx, stream);
  if (rect_ext) { std::memcpy(rect_ext, m->rect, 8); std::memcpy(rect_ext + 4, m->ext, 8); }
  size_t n = (size_t)m->ncp;
  auto cp = [&](void *dst, const void *src, size_t bytes) -> cudaError_t {
    if (!dst || !bytes) return cudaSuccess;
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st);
  };
  CK(cp(cellid, m->cellid.p, 4 * n));
  CK(cp(fn, m->fn.p, 4 * n));
  CK(cp(pair_idx, m->pair_idx.p, 4 * n));
  CK(cp(flags, m->flags.p, n));
  CK(cp(asc_off, m->aoff.p, 4 * (n + 1)));
  CK(cp(asc, m->asc.p, 4 * (size_t)m->nasc));
  CK(cp(des_off, m->doff.p, 4 * (n + 1)));
  CK(cp(des, m->des.p, 4 * (size_t)m->ndes));
  CK(cp(adisc_off, m->adoff.p, m->adoff.p ? 4 * (n + 1) : 0));
  CK(cp(adisc, m->adisc.p, 4 * (size_t)m->nadisc));
  CK(cp(ddisc_off, m->ddoff.p, m->ddoff.p ? 4 * (n + 1) : 0));
  CK(cp(ddisc, m->ddisc.p, 4 * (size_t)m->nddisc));
  if (sync) CK(cudaStreamSynchronize(st));
  // no discs: zero offsets (host buffers no copy writes)
  if (adisc_off && !m->adoff.p) std::memset(adisc_off, 0, 4 * (n + 1));
  if (ddisc_off && !m->ddoff.p) std::memset(ddisc_off, 0, 4 * (n + 1));
  return DMSC_OK;
}

int dmsc_msc_export(dmsc_msc *m, int16_t rect_ext[8], int16_t *cellid, float *fn, uint32_t *pair_idx, uint8_t *flags,
                    uint32_t *asc_off, uint32_t *asc, uint32_t *des_off, uint32_t *des, uint32_t *adisc_off,
                    int16_t *adisc, uint32_t *ddisc_off, int16_t *ddisc, void *stream) {
  return msc_export(m, rect_ext, cellid, fn, pair_idx, flags, asc_off, asc, des_off, des, adisc_off, adisc, ddisc_off,
                    ddisc, stream, true);
}

int dmsc_msc_export_async(dmsc_msc *m, int16_t rect_ext[8], int16_t *cellid, float *fn, uint32_t *pair_idx,
                          uint8_t *flags, uint32_t *asc_off, uint32_t *asc, uint32_t *des_off, uint32_t *des,
                          uint32_t *adisc_off, int16_t *adisc, uint32_t *ddisc_off, int16_t *ddisc, void *stream) {
  return msc_export(m, rect_ext, cellid, fn, pair_idx, flags, asc_off, asc, des_off, des, adisc_off, adisc, ddisc_off,
                    ddisc, stream, false);
}

int dmsc_set_timing(dmsc_ctx *ctx, int enable) {
  if (!ctx) return fail(DMSC_ERR_BAD_ARG, "ctx is null");
  ctx->timing = enable != 0;
  return DMSC_OK;
}

int dmsc_pool_stats(dmsc_ctx *ctx, int64_t stats[4]) {
  if (!ctx || !stats) return fail(DMSC_ERR_BAD_ARG, "null argument");
  cudaMemPool_t pool;
  CK(cudaDeviceGetDefaultMemPool(&pool, ctx->device));
  const cudaMemPoolAttr a[4] = {cudaMemPoolAttrReservedMemCurrent, cudaMemPoolAttrReservedMemHigh,
                                cudaMemPoolAttrUsedMemCurrent, cudaMemPoolAttrUsedMemHigh};
  for (int i = 0; i < 4; ++i) {
    uint64_t v = 0;
    CK(cudaMemPoolGetAttribute(pool, a[i], &v));
    stats[i] = (int64_t)v;
  }
  return DMSC_OK;
}

int dmsc_set_merge_parallel_min(dmsc_ctx *ctx, int64_t min_cps) {
  if (!ctx || min_cps < 0) return fail(DMSC_ERR_BAD_ARG, "ctx is null or min_cps negative");
  ctx->merge_parallel_min = min_cps;
  return DMSC_OK;
}

int dmsc_set_out_of_core(dmsc_ctx *ctx, const char *dir) {
  if (!ctx) return fail(DMSC_ERR_BAD_ARG, "ctx is null");
  ctx->ooc_dir = dir ? dir : "";
  return DMSC_OK;
}

int dmsc_set_use_ocl(dmsc_ctx *ctx, int use_ocl) {
  if (!ctx) return fail(DMSC_ERR_BAD_ARG, "ctx is null");
  ctx->use_ocl = use_ocl != 0;
  return DMSC_OK;
}

int dmsc_set_merge_rounds(dmsc_ctx *ctx, int64_t window, int64_t min_commits) {
  if (!ctx || window < 0 || min_commits < 0) return fail(DMSC_ERR_BAD_ARG, "ctx is null or a setting is negative");
  ctx->merge_round_window = window;
  ctx->merge_round_min_commits = min_commits;
  return DMSC_OK;
}

int dmsc_dataset_stage_times(dmsc_dataset *d, float *ms, int n) {
  if (!d || !ms) return fail(DMSC_ERR_BAD_ARG, "null argument");
  if (!d->ev_ready) return fail(DMSC_ERR_STATE, "timing was not enabled for the last run");
  CK(cudaSetDevice(d->ctx->device));
  // gradient, collate_scan, border_resolve, labels_arcs, connectivity, disc_hops, discs,
  // the placement kernel of the asc and of the des discs
  const int pairs[9][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 4}, {5, 6}, {7, 8}, {7, 9}, {10, 11}, {12, 13}};
  for (int i = 0; i < n && i < 9; ++i) {
    CK(cudaEventSynchronize(d->ev[pairs[i][1]]));
    float t = 0;
    if (cudaEventElapsedTime(&t, d->ev[pairs[i][0]], d->ev[pairs[i][1]]) != cudaSuccess) { cudaGetLastError(); t = -1; }
    ms[i] = t;
  }
  return DMSC_OK;
}

int dmsc_msc_simplify_un_simplify(dmsc_msc *m, double tresh, int64_t max_ops, void *stream) {
  if (!m) return fail(DMSC_ERR_BAD_ARG, "complex is null");
  if (!(tresh >= 0.0)) return fail(DMSC_ERR_BAD_ARG, "threshold must be >= 0");
  CK(cudaSetDevice(m->ctx->device));
  cudaStream_t st = pick(m->ctx, stream);
  unsigned long long *hs = nullptr;
  CK(cudaMallocHost((void **)&hs, sizeof(unsigned long long) * 5));
  SimplifyIO io;
  io.ncp = m->ncp; io.nasc = m->nasc; io.ndes = m->ndes;
  io.cellid = m->cellid.p; io.fn = m->fn.p; io.flags = m->flags.p; io.pair_idx = m->pair_idx.p;
  io.aoff = m->aoff.p; io.asc = m->asc.p; io.doff = m->doff.p; io.des = m->des.p;
  for (int i = 0; i < 4; ++i) io.rect[i] = m->rect[i];
  io.tresh = tresh;
  io.max_ops = max_ops > 0 ? (unsigned long long)max_ops : 2000000000ull;
  io.host_stats = hs;
  cudaError_t e = simplify_run(io, st);
  int rc = DMSC_OK;
  if (e != cudaSuccess) rc = cuda_fail(e, "simplify_run");
  else if (hs[4] != 0) rc = status_to_error((uint32_t)hs[4]);
  if (rc == DMSC_OK) {
    // grow the CSR arrays if needed, then write the new lists
    if ((size_t)io.nasc_out + 1 > m->asc.n) e = m->asc.ensure(io.nasc_out + io.nasc_out / 4 + 16, st);
    if (e == cudaSuccess && (size_t)io.ndes_out + 1 > m->des.n) e = m->des.ensure(io.ndes_out + io.ndes_out / 4 + 16, st);
    if (e == cudaSuccess) e = simplify_emit(io, m->asc.p, m->des.p, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_fail(e, "simplify_emit");
    else {
      m->nasc = io.nasc_out;
      m->ndes = io.ndes_out;
      if (hs[2]) m->any_bcancel = true;  // cancelled pairs are left boundary-cancelable
    }
  }
  for (int i = 0; i < 5; ++i) m->simp_stats[i] = hs[i];
  simplify_release(io, st);
  cudaStreamSynchronize(st);
  cudaFreeHost(hs);
  return rc;
}

int dmsc_msc_simplify_stats(dmsc_msc *m, uint64_t stats[5]) {
  if (!m || !stats) return fail(DMSC_ERR_BAD_ARG, "null argument");
  for (int i = 0; i < 5; ++i) stats[i] = m->simp_stats[i];
  return DMSC_OK;
}

int dmsc_dataset_fill_discs(dmsc_dataset *d, dmsc_msc *m, void *stream) {
  if (!d || !m) return fail(DMSC_ERR_BAD_ARG, "null argument");
  if (!d->worked) return fail(DMSC_ERR_STATE, "dataset_work has not run");
  if (m->ncp < d->ncp) return fail(DMSC_ERR_BAD_ARG, "complex does not hold the dataset's critical points");
  if (m->ncp >= (1ll << 30)) return fail(DMSC_ERR_BAD_ARG, "disc collection supports fewer than 2^30 critical points");
  CK(cudaSetDevice(d->ctx->device));
  cudaStream_t st = pick(d->ctx, stream);
  const size_t n = (size_t)m->ncp;
  CK(m->adoff.ensure(n + 1, st));
  CK(m->ddoff.ensure(n + 1, st));
  DiscIO io;
  io.g = d->g; io.codes = d->codes.p; io.labels = d->labels.p; io.ncp_ds = d->ncp;
  io.ncp = m->ncp; io.nasc = m->nasc; io.ndes = m->ndes;
  io.cellid = m->cellid.p; io.flags = m->flags.p; io.pair_idx = m->pair_idx.p;
  io.aoff = m->aoff.p; io.asc = m->asc.p; io.doff = m->doff.p; io.des = m->des.p;
  io.adoff = m->adoff.p; io.ddoff = m->ddoff.p; io.adisc = &m->adisc; io.ddisc = &m->ddisc;
  io.status = d->scal.p;
  // a gradient path visits each cell at most once: bounds every chain of a disc
  io.limit = (unsigned long long)(d->g.cx + 1) * (d->g.cy + 1) + 16;
  io.no_cancel = !m->any_bcancel;
  if (!d->disc_aux) CK(cudaStreamCreateWithFlags(&d->disc_aux, cudaStreamNonBlocking));
  for (auto &ev : d->disc_ev)
    if (!ev) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  if (!d->host_disc && !(d->host_disc = pin_take())) return fail(DMSC_ERR_OOM, "pinned count slot");
  io.aux = d->disc_aux;
  io.ev[0] = d->disc_ev[0];
  io.ev[1] = d->disc_ev[1];
  io.hcounts = d->host_disc;
  const bool tm = d->ctx->timing && d->ev_ready;
  if (tm) {
    io.ev_hops[0] = d->ev[7];
    io.ev_hops[1] = d->ev[8];
    io.ev_place[0][0] = d->ev[10];
    io.ev_place[0][1] = d->ev[11];
    io.ev_place[1][0] = d->ev[12];
    io.ev_place[1][1] = d->ev[13];
    CK(cudaEventRecord(d->ev[7], st));
  }
  CK(cudaMemsetAsync(d->scal.p, 0, sizeof(uint32_t), st));
  CK(fill_discs(io, st));
  if (tm) CK(cudaEventRecord(d->ev[9], st));
  const uint32_t *w[1] = {d->scal.p};
  CK(read_words(d->host_scal, w, 1, st));
  CK(cudaStreamSynchronize(st));
  if (const uint32_t stw = d->host_scal[0]) return status_to_error(stw);
  m->nadisc = io.nadisc;
  m->nddisc = io.nddisc;
  return DMSC_OK;
}

int dmsc_msc_write_discs(dmsc_msc *m, const char *prefix) {
  if (!m || !prefix) return fail(DMSC_ERR_BAD_ARG, "null argument");
  if (!m->adoff.p || !m->ddoff.p) return fail(DMSC_ERR_STATE, "the complex has no discs (fill_discs has not run)");
  CK(cudaSetDevice(m->ctx->device));
  size_t n = (size_t)m->ncp;
  std::vector<uint32_t> cell(n), ao(n + 1), dofs(n + 1), ad(m->nadisc), dd(m->nddisc);
  std::vector<uint8_t> fl(n);
  if (n) {
    CK(cudaMemcpy(cell.data(), m->cellid.p, 4 * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(fl.data(), m->flags.p, n, cudaMemcpyDeviceToHost));
  }
  CK(cudaMemcpy(ao.data(), m->adoff.p, 4 * (n + 1), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(dofs.data(), m->ddoff.p, 4 * (n + 1), cudaMemcpyDeviceToHost));
  if (m->nadisc) CK(cudaMemcpy(ad.data(), m->adisc.p, 4 * m->nadisc, cudaMemcpyDeviceToHost));
  if (m->nddisc) CK(cudaMemcpy(dd.data(), m->ddisc.p, 4 * m->nddisc, cudaMemcpyDeviceToHost));
  for (size_t i = 0; i < n; ++i) {
    if (fl[i] & 4) continue;
    const int16_t x = (int16_t)(cell[i] & 0xffff), y = (int16_t)(cell[i] >> 16);
    for (int k = 0; k < 2; ++k) {
      const std::vector<uint32_t> &off = k ? dofs : ao;
      const std::vector<uint32_t> &v = k ? dd : ad;
      if (off[i + 1] == off[i]) continue;
      std::string fn = std::string(prefix) + (k ? "des_" : "asc_") + "(" + std::to_string(x) + "," + std::to_string(y) + ")";
      FILE *f = fopen(fn.c_str(), "ab");
      if (!f) return fail(DMSC_ERR_BAD_ARG, "asc/des disc file not writeable: " + fn);
      // each packed cell id is (x, y) as two little-endian int16, the layout of cellid_t
      size_t cnt = off[i + 1] - off[i];
      size_t wrote = fwrite(v.data() + off[i], 4, cnt, f);
      fclose(f);
      if (wrote != cnt) return fail(DMSC_ERR_BAD_ARG, "short write to " + fn);
    }
  }
  return DMSC_OK;
}

int dmsc_prefix_scan(dmsc_ctx *ctx, uint32_t *d_out, const uint32_t *d_in, int64_t n, uint32_t *d_total,
                     void *stream) {
  if (!ctx || n < 0 || (n > 0 && (!d_out || !d_in))) return fail(DMSC_ERR_BAD_ARG, "bad argument");
  if (n > (int64_t)INT32_MAX * 32) return fail(DMSC_ERR_BAD_ARG, "n too large");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = pick(ctx, stream);
  CK(scan_exclusive_u32(d_in, n, d_out, d_total, st));
  CK(cudaStreamSynchronize(st));
  return DMSC_OK;
}

int dmsc_sort_pairs(dmsc_ctx *ctx, uint32_t *d_dst_key, uint32_t *d_dst_val, const uint32_t *d_src_key,
                    const uint32_t *d_src_val, uint32_t batch, uint32_t array_length, uint32_t dir, void *stream) {
  if (!ctx || !d_dst_key || !d_dst_val || !d_src_key || !d_src_val) return fail(DMSC_ERR_BAD_ARG, "null argument");
  if (dir > 1) return fail(DMSC_ERR_BAD_ARG, "dir must be 0 (descending) or 1 (ascending)");
  if ((uint64_t)batch * array_length > (1ull << 31)) return fail(DMSC_ERR_BAD_ARG, "batch * array_length too large");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = pick(ctx, stream);
  CK(sort_pairs_batched(d_dst_key, d_dst_val, d_src_key, d_src_val, batch, array_length, dir, st));
  CK(cudaStreamSynchronize(st));
  return DMSC_OK;
}

int dmsc_kernel_launches(uint64_t *count) {
  if (!count) return fail(DMSC_ERR_BAD_ARG, "null argument");
  *count = __atomic_load_n(&g_kernel_launches, __ATOMIC_RELAXED);
  return DMSC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// member functions of the handle types
// ---------------------------------------------------------------------------
// Pinned 64-byte slots for the status and count read-backs of datasets,
// carved from pinned blocks that live as long as the process (pinning a small
// buffer per dataset would serialise on the driver when many pieces start at
// once).
namespace {
std::mutex &pin_mu() {
  static std::mutex *m = new std::mutex;
  return *m;
}
std::vector<uint32_t *> &pin_free() {
  static std::vector<uint32_t *> *v = new std::vector<uint32_t *>;
  return *v;
}
uint32_t *pin_take() {
  std::lock_guard<std::mutex> lk(pin_mu());
  auto &f = pin_free();
  if (f.empty()) {
    constexpr int SLOTS = 1024, WORDS = 16;
    uint32_t *blk = nullptr;
    if (cudaMallocHost((void **)&blk, sizeof(uint32_t) * WORDS * SLOTS) != cudaSuccess) return nullptr;
    for (int i = SLOTS - 1; i >= 0; --i) f.push_back(blk + WORDS * i);
  }
  uint32_t *p = f.back();
  f.pop_back();
  return p;
}
void pin_give(uint32_t *p) {
  std::lock_guard<std::mutex> lk(pin_mu());
  pin_free().push_back(p);
}
}  // namespace

int dmsc_dataset::alloc_cells(cudaStream_t st) {
  size_t nv = (size_t)g.vnx * g.vny;
  CK(codes.ensure(nv, st));
  CK(terms.ensure(nv, st));
  CK(labels.ensure(nv, st));
  CK(rowcnt.ensure((size_t)(g.cy + 1) * g.ntx, st));
  CK(offsets.ensure((size_t)(g.cy + 1) * g.ntx, st));
  CK(table.ensure((size_t)nslots(), st));
  CK(scal.ensure(4, st));
  if (!host_scal && !(host_scal = pin_take())) return fail(DMSC_ERR_OOM, "pinned status slot");
  return DMSC_OK;
}

int dmsc_dataset::alloc_cps(long long n, cudaStream_t st) {
  CK(cp_cellid.ensure(n, st));
  CK(cp_fn.ensure(n, st));
  CK(cp_flags.ensure(n, st));
  CK(cp_pair_cell.ensure(n, st));
  CK(cp_des2.ensure(2 * n, st));
  CK(cp_asc2.ensure(2 * n, st));
  CK(cp_acnt.ensure(n, st));
  CK(cp_dcnt.ensure(n, st));
  return DMSC_OK;
}

dmsc_dataset::~dmsc_dataset() {
  if (host_scal) pin_give(host_scal);
  if (host_disc) pin_give(host_disc);
  if (disc_aux) cudaStreamDestroy(disc_aux);
  for (auto &e : disc_ev)
    if (e) cudaEventDestroy(e);
  if (ev_ready)
    for (auto &e : ev) cudaEventDestroy(e);
}

int dmsc_msc::writeout_from(const dmsc_dataset &d, cudaStream_t st) {
  ncp = d.ncp;
  any_bcancel = !d.rect_is_ext();  // only pieces hold paired critical cells
  size_t n = (size_t)ncp;
  CK(cellid.ensure(n + 1, st));
  CK(fn.ensure(n + 1, st));
  CK(pair_idx.ensure(n + 1, st));
  CK(flags.ensure(n + 1, st));
  CK(aoff.ensure(n + 1, st));
  CK(doff.ensure(n + 1, st));
  CK(asc.ensure(4 * n + 1, st));
  CK(des.ensure(4 * n + 1, st));
  if (n) {
    CK(copy_u32(cellid.p, d.cp_cellid.p, (long long)n, st));
    CK(copy_u32((uint32_t *)fn.p, (const uint32_t *)d.cp_fn.p, (long long)n, st));
    CK(copy_u32(pair_idx.p, d.cp_pair_idx.p, (long long)n, st));
    CK(launch_msc_flags(ncp, d.cp_flags.p, flags.p, st));
  }
  CK(scan_exclusive_u32(d.cp_acnt.p, ncp, aoff.p, aoff.p + n, st));
  CK(scan_exclusive_u32(d.cp_dcnt.p, ncp, doff.p, doff.p + n, st));
  CK(cudaMemsetAsync(d.scal.p, 0, sizeof(uint32_t), st));
  CK(build_csr(ncp, d.cp_cellid.p, d.cp_des2.p, d.cp_asc2.p, aoff.p, doff.p, asc.p, des.p, 4 * (long long)n + 1,
               d.scal.p, st));
  uint32_t *tot = d.host_scal;  // the dataset's pinned slot: [0] asc, [1] des entries, [2] status
  {
    const uint32_t *w[3] = {aoff.p + n, doff.p + n, d.scal.p};
    CK(read_words(tot, w, 3, st));
  }
  CK(cudaStreamSynchronize(st));
  if (tot[2] == ST_CAPACITY) {  // an extremum segment too long for the in-place sorts
    CK(cudaMemsetAsync(d.scal.p, 0, sizeof(uint32_t), st));
    CK(build_csr_radix(ncp, d.cp_cellid.p, d.cp_des2.p, d.cp_asc2.p, aoff.p, doff.p, asc.p, des.p,
                       4 * (long long)n + 1, d.scal.p, st));
    const uint32_t *w[1] = {d.scal.p};
    CK(read_words(tot + 2, w, 1, st));
    CK(cudaStreamSynchronize(st));
  }
  nasc = tot[0];
  ndes = tot[1];
  if (tot[2]) return status_to_error(tot[2]);
  if (nasc > 4 * (long long)n || ndes > 4 * (long long)n) return fail(DMSC_ERR_INVARIANT, "arc count exceeds its bound");
  return DMSC_OK;
}
