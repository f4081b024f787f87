// batch.cu -- many whole grids of different sizes in one pass.
//
// The reference builds one GridDataset at a time (GridDataManager,
// dmsc/src/grid_datamanager.cpp:121-140); here a batch packs the grids'
// heights and cell arrays back to back and runs every stage once for all of
// them: one persistent launch per tile kernel over (grid, tile) items, one
// scan over all row segments, one border-table resolve, one connectivity
// pass, and one launch that simplifies every grid with tresh > 0 (one block
// per grid).  Each grid's result is exactly what dmsc_dataset_work +
// writeout_connectivity + simplify_un_simplify give for it alone.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "dmsc.h"
#include "dmsc_internal.h"
#include "grid_types.h"

using namespace dmsc;

struct dmsc_batch {
  dmsc_ctx *ctx = nullptr;
  int ngrids = 0;
  std::vector<GridGeom> geo;
  std::vector<long long> vbase, rbase, sbase, tile0;  // ngrids + 1 each
  std::vector<double> tresh;
  std::vector<int> rect;                              // 4 per grid
  DevBuf<float> hgt;
  DevBuf<uint32_t> codes, terms, offsets, scal, cpb_dev, bases_dev;
  DevBuf<uint4> labels;
  DevBuf<uint8_t> rowcnt;
  DevBuf<uint64_t> table;
  DevBuf<BatchGrid> grids;
  // critical points of all grids (batch-wide indices)
  long long ncp = 0, nasc = 0, ndes = 0;
  DevBuf<uint32_t> cp_cellid, cp_pair_cell, cp_des2, cp_asc2, cp_acnt, cp_dcnt;
  DevBuf<float> cp_fn;
  DevBuf<uint8_t> cp_flags;
  // the complexes: shared arrays, list values local to each grid
  DevBuf<uint32_t> pair_idx, aoff, doff, asc, des;
  DevBuf<uint8_t> flags;
  std::vector<uint32_t> cpb, abase, dbase;            // ngrids + 1 each
  std::vector<unsigned long long> stats;              // 5 per grid
  std::vector<int> gstat;                             // per grid: DMSC_OK or the grid's own error
  std::vector<std::string> gerr;                      // its message
  int ndead = 0;
  // the grids regrouped by size class (per-class launches of a tuned context)
  DevBuf<BatchGrid> grids_cls;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};  // around the gradient and the labels launches
  ~dmsc_batch() {
    for (auto e : ev)
      if (e) cudaEventDestroy(e);
  }
};

namespace {

int berr(int code, const std::string &m) { return set_last_error(code, m.c_str()); }

#define BCK(call)                                                                                       \
  do {                                                                                                  \
    cudaError_t e_ = (call);                                                                            \
    if (e_ != cudaSuccess)                                                                              \
      return berr(e_ == cudaErrorMemoryAllocation ? DMSC_ERR_OOM : DMSC_ERR_CUDA,                       \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                                  \
  } while (0)

// Size class of a grid for the launch configurations: its larger side below
// 128, 256, 512, 1024, 2048 vertices, or above.
constexpr int NCLASS = 6;
int size_class(int nx, int ny) {
  const int s = nx > ny ? nx : ny;
  int c = 0;
  for (int lim = 128; c < NCLASS - 1 && s >= lim; lim *= 2) ++c;
  return c;
}

unsigned nblk(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (unsigned)(b < 1 ? 1 : b);
}

// cp base of every grid (the offsets value at its first row segment) and the total
__global__ void k_cp_bases(int n, const long long *rbase, const uint32_t *offsets, uint32_t *cpb) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g <= n; g += gridDim.x * blockDim.x) cpb[g] = offsets[rbase[g]];
}
// list bases of every grid: aoff / doff at its first critical point
__global__ void k_list_bases(int n, const uint32_t *cpb, const uint32_t *aoff, const uint32_t *doff, uint32_t *ab,
                             uint32_t *db) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g <= n; g += gridDim.x * blockDim.x) {
    ab[g] = aoff[cpb[g]];
    db[g] = doff[cpb[g]];
  }
}
// batch-wide list values -> indices local to the grid of the list's owner
__global__ void k_localize(long long ncp, int n, const uint32_t *cpb, const uint32_t *aoff, uint32_t *asc,
                           const uint32_t *doff, uint32_t *des, uint32_t *status) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ncp; i += (long long)gridDim.x * blockDim.x) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (cpb[mid] <= (uint32_t)i) lo = mid; else hi = mid - 1;
    }
    const uint32_t b = cpb[lo], e = cpb[lo + 1];
    for (int w = 0; w < 2; ++w) {
      const uint32_t *o = w ? doff : aoff;
      uint32_t *l = w ? des : asc;
      for (uint32_t k = o[i]; k < o[i + 1]; ++k) {
        const uint32_t v = l[k];
        if (v < b || v >= e) { atomicOr(status, ST_INVARIANT); continue; }  // arcs never cross grids
        l[k] = v - b;
      }
    }
  }
}

}  // namespace

extern "C" {

int dmsc_batch_run(dmsc_ctx *ctx, int ngrids, const int32_t *sizes, const float *heights, int on_device,
                   const double *tresh, int64_t max_ops, dmsc_batch **out, void *stream) {
  if (!ctx || !sizes || !heights || !tresh || !out) return berr(DMSC_ERR_BAD_ARG, "null argument");
  if (ngrids <= 0) return berr(DMSC_ERR_BAD_ARG, "a batch holds at least one grid");
  for (int g = 0; g < ngrids; ++g) {
    const int nx = sizes[2 * g], ny = sizes[2 * g + 1];
    if (nx < 2 || ny < 2) return berr(DMSC_ERR_BAD_ARG, "grid " + std::to_string(g) + " is smaller than 2x2");
    if (nx > 16384 || ny > 16384) return berr(DMSC_ERR_INT16_OVERFLOW, "grid " + std::to_string(g) + " exceeds int16 cell ids");
    if (!(tresh[g] >= 0.0)) return berr(DMSC_ERR_BAD_ARG, "negative or NaN threshold");
  }
  BCK(cudaSetDevice(ctx->device));
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  const bool fresh = *out == nullptr;
  dmsc_batch *B = fresh ? new dmsc_batch : *out;
  if (!fresh && B->ctx != ctx) return berr(DMSC_ERR_BAD_ARG, "batch belongs to another context");
  B->ctx = ctx;
  B->ngrids = ngrids;
  B->gstat.assign(ngrids, DMSC_OK);
  B->gerr.assign(ngrids, std::string());
  B->ndead = 0;
  auto fail = [&](int rc) {
    if (fresh) delete B;
    else { B->ncp = 0; B->cpb.clear(); B->abase.clear(); B->dbase.clear(); }
    return rc;
  };

  // geometry and packing
  B->geo.assign(ngrids, GridGeom());
  B->vbase.assign(ngrids + 1, 0); B->rbase.assign(ngrids + 1, 0); B->sbase.assign(ngrids + 1, 0);
  B->tile0.assign(ngrids + 1, 0);
  B->tresh.assign(tresh, tresh + ngrids);
  B->rect.assign(4 * ngrids, 0);
  for (int g = 0; g < ngrids; ++g) {
    GridGeom &G = B->geo[g];
    G.ex0 = 0; G.ey0 = 0;
    G.vnx = sizes[2 * g]; G.vny = sizes[2 * g + 1];
    G.cx = 2 * (G.vnx - 1); G.cy = 2 * (G.vny - 1);
    G.rx0 = 0; G.ry0 = 0; G.rx1 = G.cx; G.ry1 = G.cy;
    G.ntx = (G.vnx + TX - 1) / TX; G.nty = (G.vny + TY - 1) / TY;
    G.pitch = G.vnx;
    G.sbase = B->sbase[g];
    G.gbase = B->rbase[g];
    B->rect[4 * g + 2] = G.cx; B->rect[4 * g + 3] = G.cy;
    B->vbase[g + 1] = B->vbase[g] + (long long)G.vnx * G.vny;
    B->rbase[g + 1] = B->rbase[g] + (long long)(G.cy + 1) * G.ntx;
    B->sbase[g + 1] = B->sbase[g] + (long long)G.ntx * G.nty * SLOTS_PER_TILE;
    B->tile0[g + 1] = B->tile0[g] + (long long)G.ntx * G.nty;
  }
  const long long NV = B->vbase[ngrids], NR = B->rbase[ngrids], NS = B->sbase[ngrids], NT = B->tile0[ngrids];
  if (B->codes.ensure(NV, st) || B->terms.ensure(NV, st) || B->labels.ensure(NV, st) || B->rowcnt.ensure(NR, st) ||
      B->offsets.ensure(NR + 1, st) || B->table.ensure(NS, st) || B->scal.ensure(4, st) || B->grids.ensure(ngrids, st) ||
      B->cpb_dev.ensure(ngrids + 1, st) || B->bases_dev.ensure(2 * (ngrids + 1) + 2 * ngrids + 2, st))
    return fail(berr(DMSC_ERR_OOM, "batch buffers"));
  const float *hgt = heights;
  if (!on_device) {
    if (B->hgt.ensure(NV, st)) return fail(berr(DMSC_ERR_OOM, "batch heights"));
    if (cudaMemcpyAsync(B->hgt.p, heights, sizeof(float) * NV, cudaMemcpyHostToDevice, st) != cudaSuccess)
      return fail(berr(DMSC_ERR_CUDA, "heights copy"));
    hgt = B->hgt.p;
  }
  std::vector<BatchGrid> hg(ngrids);
  std::vector<long long> rb(B->rbase);
  for (int g = 0; g < ngrids; ++g) {
    BatchGrid &q = hg[g];
    q.g = B->geo[g];
    q.hgt = hgt + B->vbase[g];
    q.codes = B->codes.p + B->vbase[g];
    q.terms = B->terms.p + B->vbase[g];
    q.labels = B->labels.p + B->vbase[g];
    q.rowcnt = B->rowcnt.p + B->rbase[g];
    q.table = B->table.p + B->sbase[g];
    q.offsets = B->offsets.p + B->rbase[g];
    q.tile0 = B->tile0[g];
  }
  long long *rb_dev = (long long *)(B->bases_dev.p + 2 * (ngrids + 1));
  if (cudaMemcpyAsync(B->grids.p, hg.data(), sizeof(BatchGrid) * ngrids, cudaMemcpyHostToDevice, st) ||
      cudaMemcpyAsync(rb_dev, rb.data(), sizeof(long long) * (ngrids + 1), cudaMemcpyHostToDevice, st) ||
      cudaMemsetAsync(B->scal.p, 0, sizeof(uint32_t) * 4, st))
    return fail(berr(DMSC_ERR_CUDA, "batch descriptors"));

  // the tile kernels' launches: one over all grids, or with a tuned context
  // one per size class present, each with its class's configuration
  struct ClassLaunch { int off, n; long long ntiles; BatchLaunch cfg; };
  std::vector<ClassLaunch> cl;
  const BatchGrid *lgrids = B->grids.p;
  if (ctx->batch_tuned) {
    std::vector<BatchGrid> hc;
    for (int c = 0; c < NCLASS; ++c) {
      ClassLaunch L{(int)hc.size(), 0, 0, BatchLaunch{ctx->batch_cfg[c][0], ctx->batch_cfg[c][1]}};
      for (int g = 0; g < ngrids; ++g) {
        if (size_class(sizes[2 * g], sizes[2 * g + 1]) != c) continue;
        BatchGrid q = hg[g];
        q.tile0 = L.ntiles;  // class-local tile numbering
        L.ntiles += B->tile0[g + 1] - B->tile0[g];
        hc.push_back(q);
        ++L.n;
      }
      if (L.n) cl.push_back(L);
    }
    if (B->grids_cls.ensure(hc.size(), st) ||
        cudaMemcpyAsync(B->grids_cls.p, hc.data(), sizeof(BatchGrid) * hc.size(), cudaMemcpyHostToDevice, st) ||
        cudaStreamSynchronize(st))  // hc is read before it goes out of scope
      return fail(berr(DMSC_ERR_CUDA, "batch class descriptors"));
    lgrids = B->grids_cls.p;
  } else {
    cl.push_back(ClassLaunch{0, ngrids, NT, BatchLaunch()});
  }
  for (auto &e : B->ev)
    if (!e && cudaEventCreate(&e) != cudaSuccess) return fail(berr(DMSC_ERR_CUDA, "batch events"));
  // K1 -> scan -> K3 over all grids, then the cp bases
  bool ok = cudaEventRecord(B->ev[0], st) == cudaSuccess;
  for (const auto &L : cl)
    ok = ok && launch_gradient_batch(lgrids + L.off, L.n, L.ntiles, B->scal.p, st, L.cfg) == cudaSuccess;
  ok = ok && cudaEventRecord(B->ev[1], st) == cudaSuccess;
  if (!ok ||
      scan_exclusive_u8(B->rowcnt.p, NR, B->offsets.p, B->offsets.p + NR, st) != cudaSuccess ||
      launch_resolve(B->table.p, NS, B->offsets.p, NR, B->scal.p, st) != cudaSuccess)
    return fail(berr(DMSC_ERR_CUDA, std::string("batch gradient: ") + cudaGetErrorString(cudaGetLastError())));
  k_cp_bases<<<nblk(ngrids + 1), 256, 0, st>>>(ngrids, rb_dev, B->offsets.p, B->cpb_dev.p);
  DMSC_LAUNCHED(1);
  B->cpb.assign(ngrids + 1, 0);
  uint32_t stw = 0;
  if (cudaMemcpyAsync(B->cpb.data(), B->cpb_dev.p, 4ull * (ngrids + 1), cudaMemcpyDeviceToHost, st) ||
      cudaMemcpyAsync(&stw, B->scal.p, 4, cudaMemcpyDeviceToHost, st) || cudaStreamSynchronize(st))
    return fail(berr(DMSC_ERR_CUDA, "batch counts"));
  if (stw & ST_NAN_INPUT) return fail(berr(DMSC_ERR_INPUT, "NaN heights are outside the supported domain"));
  if (stw) return fail(berr(DMSC_ERR_INVARIANT, "batch gradient status " + std::to_string(stw)));
  const long long ncp = B->cpb[ngrids];
  B->ncp = ncp;
  const size_t n = (size_t)ncp;
  if (B->cp_cellid.ensure(n + 1, st) || B->cp_fn.ensure(n + 1, st) || B->cp_flags.ensure(n + 1, st) || B->cp_pair_cell.ensure(n + 1, st) ||
      B->cp_des2.ensure(2 * n + 2, st) || B->cp_asc2.ensure(2 * n + 2, st) || B->cp_acnt.ensure(n + 1, st) ||
      B->cp_dcnt.ensure(n + 1, st) || B->pair_idx.ensure(n + 1, st) || B->flags.ensure(n + 1, st) || B->aoff.ensure(n + 1, st) ||
      B->doff.ensure(n + 1, st) || B->asc.ensure(4 * n + 1, st) || B->des.ensure(4 * n + 1, st))
    return fail(berr(DMSC_ERR_OOM, "batch critical points"));
  CpOut cp{B->cp_cellid.p, B->cp_fn.p, B->cp_flags.p, B->cp_pair_cell.p, B->cp_des2.p, B->cp_asc2.p,
           B->cp_acnt.p, B->cp_dcnt.p, ncp};
  if (cudaMemsetAsync(B->cp_acnt.p, 0, 4 * (n + 1), st) || cudaMemsetAsync(B->cp_dcnt.p, 0, 4 * (n + 1), st) ||
      cudaEventRecord(B->ev[2], st))
    return fail(berr(DMSC_ERR_CUDA, "batch labels"));
  for (const auto &L : cl)
    if (launch_labels_batch(lgrids + L.off, L.n, L.ntiles, cp, B->scal.p, st, L.cfg) != cudaSuccess)
      return fail(berr(DMSC_ERR_CUDA, "batch labels"));
  if (cudaEventRecord(B->ev[3], st)) return fail(berr(DMSC_ERR_CUDA, "batch labels"));

  // writeout_connectivity of every grid: shared CSR, then local list values
  if (launch_msc_flags(ncp, B->cp_flags.p, B->flags.p, st) || cudaMemsetAsync(B->pair_idx.p, 0xFF, 4 * (n + 1), st) ||
      scan_exclusive_u32(B->cp_acnt.p, ncp, B->aoff.p, B->aoff.p + ncp, st) ||
      scan_exclusive_u32(B->cp_dcnt.p, ncp, B->doff.p, B->doff.p + ncp, st) ||
      build_csr(ncp, B->cp_cellid.p, B->cp_des2.p, B->cp_asc2.p, B->aoff.p, B->doff.p, B->asc.p, B->des.p,
                4 * (long long)n + 1, B->scal.p, st))
    return fail(berr(DMSC_ERR_CUDA, "batch connectivity"));
  if (cudaMemcpyAsync(&stw, B->scal.p, 4, cudaMemcpyDeviceToHost, st) || cudaStreamSynchronize(st))
    return fail(berr(DMSC_ERR_CUDA, "batch status"));
  if (stw == ST_CAPACITY) {  // an extremum segment too long for the in-place sorts
    if (cudaMemsetAsync(B->scal.p, 0, 4, st) ||
        build_csr_radix(ncp, B->cp_cellid.p, B->cp_des2.p, B->cp_asc2.p, B->aoff.p, B->doff.p, B->asc.p, B->des.p,
                        4 * (long long)n + 1, B->scal.p, st) ||
        cudaMemcpyAsync(&stw, B->scal.p, 4, cudaMemcpyDeviceToHost, st) || cudaStreamSynchronize(st))
      return fail(berr(DMSC_ERR_CUDA, "batch connectivity"));
  }
  if (stw) return fail(berr(DMSC_ERR_INVARIANT, "batch connectivity status " + std::to_string(stw)));
  uint32_t *ab_dev = B->bases_dev.p, *db_dev = B->bases_dev.p + (ngrids + 1);
  if (ncp) {
    k_localize<<<nblk(ncp), 256, 0, st>>>(ncp, ngrids, B->cpb_dev.p, B->aoff.p, B->asc.p, B->doff.p, B->des.p, B->scal.p);
    DMSC_LAUNCHED(1);
  }
  k_list_bases<<<nblk(ngrids + 1), 256, 0, st>>>(ngrids, B->cpb_dev.p, B->aoff.p, B->doff.p, ab_dev, db_dev);
  DMSC_LAUNCHED(1);
  B->abase.assign(ngrids + 1, 0);
  B->dbase.assign(ngrids + 1, 0);
  if (cudaMemcpyAsync(B->abase.data(), ab_dev, 4ull * (ngrids + 1), cudaMemcpyDeviceToHost, st) ||
      cudaMemcpyAsync(B->dbase.data(), db_dev, 4ull * (ngrids + 1), cudaMemcpyDeviceToHost, st) ||
      cudaMemcpyAsync(&stw, B->scal.p, 4, cudaMemcpyDeviceToHost, st) || cudaStreamSynchronize(st))
    return fail(berr(DMSC_ERR_CUDA, "batch list bases"));
  if (stw) return fail(berr(DMSC_ERR_INVARIANT, "batch connectivity status " + std::to_string(stw)));
  B->nasc = B->abase[ngrids];
  B->ndes = B->dbase[ngrids];

  // simplify_un_simplify of every grid with tresh > 0, one block each
  B->stats.assign(5 * (size_t)ngrids, 0);
  bool any = false;
  for (int g = 0; g < ngrids; ++g) any |= tresh[g] > 0.0 && B->cpb[g + 1] > B->cpb[g];
  if (any) {
    BatchSimplifyIO io;
    io.ncp = ncp; io.nasc = B->nasc; io.ndes = B->ndes;
    io.cellid = B->cp_cellid.p; io.fn = B->cp_fn.p; io.flags = B->flags.p; io.pair_idx = B->pair_idx.p;
    io.aoff = B->aoff.p; io.asc = B->asc.p; io.doff = B->doff.p; io.des = B->des.p;
    io.ngrids = ngrids; io.cpb = B->cpb.data(); io.abase = B->abase.data(); io.dbase = B->dbase.data();
    io.tresh = B->tresh.data(); io.rect = B->rect.data();
    io.max_ops = max_ops > 0 ? (unsigned long long)max_ops : 2000000000ull;
    io.host_stats = B->stats.data();
    int rc = DMSC_OK;
    std::vector<int> dead;
    // a grid that ran out of list pool, heap or scratch (not of its operation
    // budget) makes the whole simplification rerun with larger capacities;
    // whole grids start with no flags and no pairs, so the rerun starts clean.
    // A grid that exhausts its operation budget or breaks an invariant fails
    // alone: its lists are emptied and the other grids complete.
    for (int attempt = 0;; ++attempt) {
      cudaError_t e = simplify_batch_run(io, st);
      if (e != cudaSuccess) {
        rc = berr(e == cudaErrorMemoryAllocation ? DMSC_ERR_OOM : DMSC_ERR_CUDA,
                  std::string("batch simplify: ") + cudaGetErrorString(e));
        break;
      }
      bool capacity = false;
      dead.clear();
      for (int g = 0; g < ngrids; ++g) {
        const unsigned long long s = B->stats[5 * g + 4];
        if (!s) continue;
        if (s == ST_SIMPLIFY_LIMIT && B->stats[5 * g + 3] <= io.max_ops && attempt < 3) { capacity = true; continue; }
        dead.push_back(g);
        if (s == ST_SIMPLIFY_LIMIT && B->stats[5 * g + 3] <= io.max_ops) {
          B->gstat[g] = DMSC_ERR_DEVICE_TIMEOUT;
          B->gerr[g] = "grid " + std::to_string(g) + ": simplification ran out of list pool after retries";
        } else if (s & ST_SIMPLIFY_LIMIT) {
          B->gstat[g] = DMSC_ERR_DEVICE_TIMEOUT;
          B->gerr[g] = "grid " + std::to_string(g) + ": simplification ran out of its operation budget";
        } else {
          B->gstat[g] = DMSC_ERR_INVARIANT;
          B->gerr[g] = "grid " + std::to_string(g) + ": simplification status " + std::to_string(s);
        }
      }
      if (!capacity) break;
      for (int g : dead) { B->gstat[g] = DMSC_OK; B->gerr[g].clear(); }
      simplify_batch_release(io, st);
      io.scale *= 4;
      if (cudaMemsetAsync(B->flags.p, 0, n, st) || cudaMemsetAsync(B->pair_idx.p, 0xFF, 4 * n, st)) {
        rc = berr(DMSC_ERR_CUDA, "batch simplify reset");
        break;
      }
    }
    if (rc == DMSC_OK && simplify_batch_offsets(io, dead, st) != cudaSuccess)
      rc = berr(DMSC_ERR_CUDA, "batch simplify offsets");
    if (rc == DMSC_OK) {
      if (B->asc.ensure((size_t)io.nasc_out + 1, st) || B->des.ensure((size_t)io.ndes_out + 1, st) ||
          simplify_batch_emit(io, B->asc.p, B->des.p, st))
        rc = berr(DMSC_ERR_CUDA, "batch simplify output");
    }
    B->ndead = (int)dead.size();
    simplify_batch_release(io, st);
    if (rc) return fail(rc);
    B->nasc = io.nasc_out;
    B->ndes = io.ndes_out;
    k_list_bases<<<nblk(ngrids + 1), 256, 0, st>>>(ngrids, B->cpb_dev.p, B->aoff.p, B->doff.p, ab_dev, db_dev);
    DMSC_LAUNCHED(1);
    if (cudaMemcpyAsync(B->abase.data(), ab_dev, 4ull * (ngrids + 1), cudaMemcpyDeviceToHost, st) ||
        cudaMemcpyAsync(B->dbase.data(), db_dev, 4ull * (ngrids + 1), cudaMemcpyDeviceToHost, st) ||
        cudaStreamSynchronize(st))
      return fail(berr(DMSC_ERR_CUDA, "batch list bases"));
  }
  *out = B;
  if (B->ndead) {
    for (int g = 0; g < ngrids; ++g)
      if (B->gstat[g] != DMSC_OK)
        return berr(DMSC_ERR_PARTIAL, std::to_string(B->ndead) + " grid(s) failed; first: " + B->gerr[g]);
  }
  return DMSC_OK;
}

int dmsc_batch_destroy(dmsc_batch *b) {
  if (!b) return berr(DMSC_ERR_BAD_ARG, "batch is null");
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->ctx->stream);
  delete b;
  return DMSC_OK;
}

int dmsc_batch_tile_times(dmsc_batch *b, float ms[2]) {
  if (!b || !ms) return berr(DMSC_ERR_BAD_ARG, "null argument");
  if (!b->ev[3]) return berr(DMSC_ERR_STATE, "the batch has not run");
  BCK(cudaSetDevice(b->ctx->device));
  BCK(cudaEventSynchronize(b->ev[3]));
  BCK(cudaEventElapsedTime(&ms[0], b->ev[0], b->ev[1]));
  BCK(cudaEventElapsedTime(&ms[1], b->ev[2], b->ev[3]));
  return DMSC_OK;
}

// Per size class present in the sample: every launch configuration of the
// two tile kernels, `repeats` timed batch runs of the class's grids each
// (after one untimed), the median of the tile kernels' time; the fastest
// configuration becomes the class's.
int dmsc_batch_autotune(dmsc_ctx *ctx, int ngrids, const int32_t *sizes, const float *heights, int on_device,
                        int repeats, int32_t *table) {
  if (!ctx || !sizes || !heights || ngrids <= 0) return berr(DMSC_ERR_BAD_ARG, "null argument or empty sample");
  if (repeats < 1 || repeats > 50) return berr(DMSC_ERR_BAD_ARG, "repeats must be 1..50");
  for (int g = 0; g < ngrids; ++g)
    if (sizes[2 * g] < 2 || sizes[2 * g + 1] < 2 || sizes[2 * g] > 16384 || sizes[2 * g + 1] > 16384)
      return berr(DMSC_ERR_BAD_ARG, "sample grid " + std::to_string(g) + " has a bad size");
  BCK(cudaSetDevice(ctx->device));
  std::vector<long long> voff(ngrids + 1, 0);
  for (int g = 0; g < ngrids; ++g) voff[g + 1] = voff[g] + (long long)sizes[2 * g] * sizes[2 * g + 1];
  const BatchLaunch cand[] = {{512, 3}, {512, 2}, {512, 1}, {256, 3}, {256, 2}, {256, 1}};
  const bool was_tuned = ctx->batch_tuned;
  int saved[NCLASS][2], chosen[NCLASS][2];
  std::memcpy(saved, ctx->batch_cfg, sizeof saved);
  std::memcpy(chosen, ctx->batch_cfg, sizeof chosen);
  std::vector<int32_t> out(4 * NCLASS, 0);
  auto restore = [&](int rc) {
    std::memcpy(ctx->batch_cfg, saved, sizeof saved);
    ctx->batch_tuned = was_tuned;
    return rc;
  };
  for (int c = 0; c < NCLASS; ++c) {
    std::vector<int32_t> sz;
    std::vector<float> hh;
    float *dh = nullptr;
    long long nv = 0;
    std::vector<int> members;
    for (int g = 0; g < ngrids; ++g)
      if (size_class(sizes[2 * g], sizes[2 * g + 1]) == c) {
        members.push_back(g);
        sz.push_back(sizes[2 * g]);
        sz.push_back(sizes[2 * g + 1]);
        nv += voff[g + 1] - voff[g];
      }
    if (members.empty()) continue;
    const int nc = (int)members.size();
    if (on_device) {  // the class's grids packed into one device buffer
      if (cudaMalloc((void **)&dh, sizeof(float) * nv) != cudaSuccess) return restore(berr(DMSC_ERR_OOM, "autotune sample"));
      long long o = 0;
      for (int g : members) {
        const long long k = voff[g + 1] - voff[g];
        if (cudaMemcpy(dh + o, heights + voff[g], sizeof(float) * k, cudaMemcpyDeviceToDevice) != cudaSuccess) {
          cudaFree(dh);
          return restore(berr(DMSC_ERR_CUDA, "autotune sample copy"));
        }
        o += k;
      }
    } else {
      hh.reserve(nv);
      for (int g : members) hh.insert(hh.end(), heights + voff[g], heights + voff[g + 1]);
    }
    const std::vector<double> zero(nc, 0.0);
    dmsc_batch *b = nullptr;
    float best = 3.4e38f, def = 0;
    BatchLaunch pick;
    int rc = DMSC_OK;
    for (const BatchLaunch &cfg : cand) {
      ctx->batch_tuned = true;
      for (int k = 0; k < NCLASS; ++k) { ctx->batch_cfg[k][0] = cfg.threads; ctx->batch_cfg[k][1] = cfg.blocks_per_sm; }
      std::vector<float> t;
      for (int r = 0; r <= repeats && rc == DMSC_OK; ++r) {
        rc = dmsc_batch_run(ctx, nc, sz.data(), on_device ? dh : hh.data(), on_device, zero.data(), 0, &b, nullptr);
        float ms[2] = {0, 0};
        if (rc == DMSC_OK) rc = dmsc_batch_tile_times(b, ms);
        if (r) t.push_back(ms[0] + ms[1]);
      }
      if (rc != DMSC_OK) break;
      std::sort(t.begin(), t.end());
      const float med = t[t.size() / 2];
      if (cfg.threads == 512 && cfg.blocks_per_sm == 3) def = med;
      if (med < best) { best = med; pick = cfg; }
    }
    if (b) dmsc_batch_destroy(b);
    if (dh) cudaFree(dh);
    if (rc != DMSC_OK) return restore(rc);
    chosen[c][0] = pick.threads;
    chosen[c][1] = pick.blocks_per_sm;
    out[4 * c] = pick.threads;
    out[4 * c + 1] = pick.blocks_per_sm;
    out[4 * c + 2] = (int32_t)(best * 1000.0f + 0.5f);
    out[4 * c + 3] = (int32_t)(def * 1000.0f + 0.5f);
  }
  std::memcpy(ctx->batch_cfg, chosen, sizeof chosen);
  ctx->batch_tuned = true;
  if (table) std::memcpy(table, out.data(), sizeof(int32_t) * out.size());
  return DMSC_OK;
}

int dmsc_batch_set_launch(dmsc_ctx *ctx, int size_class, int threads, int blocks_per_sm) {
  if (!ctx || size_class < 0 || size_class >= NCLASS || (threads != 256 && threads != 512) || blocks_per_sm < 1 ||
      blocks_per_sm > 3)
    return berr(DMSC_ERR_BAD_ARG, "size class 0..5, threads 256 or 512, blocks per SM 1..3");
  ctx->batch_cfg[size_class][0] = threads;
  ctx->batch_cfg[size_class][1] = blocks_per_sm;
  ctx->batch_tuned = true;
  return DMSC_OK;
}

int dmsc_batch_autotune_reset(dmsc_ctx *ctx) {
  if (!ctx) return berr(DMSC_ERR_BAD_ARG, "ctx is null");
  ctx->batch_tuned = false;
  for (int c = 0; c < NCLASS; ++c) { ctx->batch_cfg[c][0] = 512; ctx->batch_cfg[c][1] = 3; }
  return DMSC_OK;
}

int dmsc_batch_num_grids(dmsc_batch *b, int64_t *n) {
  if (!b || !n) return berr(DMSC_ERR_BAD_ARG, "null argument");
  *n = b->ngrids;
  return DMSC_OK;
}

int dmsc_batch_sizes(dmsc_batch *b, int64_t i, int64_t sizes[3]) {
  if (!b || !sizes || i < 0 || i >= b->ngrids) return berr(DMSC_ERR_BAD_ARG, "no such grid");
  if (b->cpb.size() != (size_t)b->ngrids + 1) return berr(DMSC_ERR_STATE, "batch has not run");
  sizes[0] = b->cpb[i + 1] - b->cpb[i];
  sizes[1] = b->abase[i + 1] - b->abase[i];
  sizes[2] = b->dbase[i + 1] - b->dbase[i];
  return DMSC_OK;
}

int dmsc_batch_grid_status(dmsc_batch *b, int64_t i, int *status, char *error, int error_len) {
  if (!b || !status || i < 0 || i >= b->ngrids || b->gstat.size() != (size_t)b->ngrids)
    return berr(DMSC_ERR_BAD_ARG, "no such grid");
  *status = b->gstat[i];
  if (error && error_len > 0) {
    std::strncpy(error, b->gerr[i].c_str(), (size_t)error_len - 1);
    error[error_len - 1] = 0;
  }
  return DMSC_OK;
}

int dmsc_batch_simplify_stats(dmsc_batch *b, int64_t i, uint64_t stats[5]) {
  if (!b || !stats || i < 0 || i >= b->ngrids || b->stats.size() != 5 * (size_t)b->ngrids)
    return berr(DMSC_ERR_BAD_ARG, "no such grid");
  for (int q = 0; q < 5; ++q) stats[q] = b->stats[5 * i + q];
  return DMSC_OK;
}

int dmsc_batch_export(dmsc_batch *b, int64_t i, int16_t rect_ext[8], int16_t *cellid, float *fn, uint32_t *pair_idx,
                      uint8_t *flags, uint32_t *asc_off, uint32_t *asc, uint32_t *des_off, uint32_t *des, void *stream) {
  if (!b || i < 0 || i >= b->ngrids) return berr(DMSC_ERR_BAD_ARG, "no such grid");
  if (b->cpb.size() != (size_t)b->ngrids + 1) return berr(DMSC_ERR_STATE, "batch has not run");
  if (b->gstat[i] != DMSC_OK) return berr(b->gstat[i], b->gerr[i]);
  BCK(cudaSetDevice(b->ctx->device));
  cudaStream_t st = stream ? (cudaStream_t)stream : b->ctx->stream;
  const size_t c0 = b->cpb[i], n = b->cpb[i + 1] - c0;
  const size_t a0 = b->abase[i], na = b->abase[i + 1] - a0, d0 = b->dbase[i], nd = b->dbase[i + 1] - d0;
  if (rect_ext) {
    const GridGeom &G = b->geo[i];
    const int16_t r[8] = {0, 0, (int16_t)G.cx, (int16_t)G.cy, 0, 0, (int16_t)G.cx, (int16_t)G.cy};
    std::memcpy(rect_ext, r, sizeof(r));
  }
  if (cellid && n) BCK(cudaMemcpyAsync(cellid, b->cp_cellid.p + c0, 4 * n, cudaMemcpyDeviceToHost, st));
  if (fn && n) BCK(cudaMemcpyAsync(fn, b->cp_fn.p + c0, 4 * n, cudaMemcpyDeviceToHost, st));
  if (pair_idx && n) BCK(cudaMemcpyAsync(pair_idx, b->pair_idx.p + c0, 4 * n, cudaMemcpyDeviceToHost, st));
  if (flags && n) BCK(cudaMemcpyAsync(flags, b->flags.p + c0, n, cudaMemcpyDeviceToHost, st));
  if (asc_off) BCK(cudaMemcpyAsync(asc_off, b->aoff.p + c0, 4 * (n + 1), cudaMemcpyDeviceToHost, st));
  if (des_off) BCK(cudaMemcpyAsync(des_off, b->doff.p + c0, 4 * (n + 1), cudaMemcpyDeviceToHost, st));
  if (asc && na) BCK(cudaMemcpyAsync(asc, b->asc.p + a0, 4 * na, cudaMemcpyDeviceToHost, st));
  if (des && nd) BCK(cudaMemcpyAsync(des, b->des.p + d0, 4 * nd, cudaMemcpyDeviceToHost, st));
  BCK(cudaStreamSynchronize(st));
  if (asc_off)
    for (size_t k = 0; k <= n; ++k) asc_off[k] -= (uint32_t)a0;
  if (des_off)
    for (size_t k = 0; k <= n; ++k) des_off[k] -= (uint32_t)d0;
  return DMSC_OK;
}

int dmsc_batch_totals(dmsc_batch *b, int64_t totals[3]) {
  if (!b || !totals) return berr(DMSC_ERR_BAD_ARG, "null argument");
  totals[0] = b->ncp; totals[1] = b->nasc; totals[2] = b->ndes;
  return DMSC_OK;
}

int dmsc_batch_export_all(dmsc_batch *b, uint32_t *cp_base, uint32_t *asc_base, uint32_t *des_base, uint32_t *cellid,
                          float *fn, uint32_t *pair_idx, uint8_t *flags, uint32_t *asc_off, uint32_t *asc,
                          uint32_t *des_off, uint32_t *des, void *stream) {
  if (!b) return berr(DMSC_ERR_BAD_ARG, "batch is null");
  if (b->cpb.size() != (size_t)b->ngrids + 1) return berr(DMSC_ERR_STATE, "batch has not run");
  if (b->ndead) return berr(DMSC_ERR_STATE, "batch has failed grids; export the others one by one");
  BCK(cudaSetDevice(b->ctx->device));
  cudaStream_t st = stream ? (cudaStream_t)stream : b->ctx->stream;
  const size_t n = (size_t)b->ncp, g1 = (size_t)b->ngrids + 1;
  if (cp_base) std::memcpy(cp_base, b->cpb.data(), 4 * g1);
  if (asc_base) std::memcpy(asc_base, b->abase.data(), 4 * g1);
  if (des_base) std::memcpy(des_base, b->dbase.data(), 4 * g1);
  if (cellid && n) BCK(cudaMemcpyAsync(cellid, b->cp_cellid.p, 4 * n, cudaMemcpyDeviceToHost, st));
  if (fn && n) BCK(cudaMemcpyAsync(fn, b->cp_fn.p, 4 * n, cudaMemcpyDeviceToHost, st));
  if (pair_idx && n) BCK(cudaMemcpyAsync(pair_idx, b->pair_idx.p, 4 * n, cudaMemcpyDeviceToHost, st));
  if (flags && n) BCK(cudaMemcpyAsync(flags, b->flags.p, n, cudaMemcpyDeviceToHost, st));
  if (asc_off) BCK(cudaMemcpyAsync(asc_off, b->aoff.p, 4 * (n + 1), cudaMemcpyDeviceToHost, st));
  if (des_off) BCK(cudaMemcpyAsync(des_off, b->doff.p, 4 * (n + 1), cudaMemcpyDeviceToHost, st));
  if (asc && b->nasc) BCK(cudaMemcpyAsync(asc, b->asc.p, 4ull * b->nasc, cudaMemcpyDeviceToHost, st));
  if (des && b->ndes) BCK(cudaMemcpyAsync(des, b->des.p, 4ull * b->ndes, cudaMemcpyDeviceToHost, st));
  BCK(cudaStreamSynchronize(st));
  return DMSC_OK;
}

}  // extern "C"
