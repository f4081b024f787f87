// serve.cu -- a request server over the batch engine (no reference
// counterpart: the reference is a batch program over one grid).
//
// Requests (one whole grid each: heights, size, threshold) are queued on
// submit.  Each of `lanes` worker threads owns a CUDA stream, a pinned
// staging buffer and a dmsc_batch; whenever it is free it admits the queued
// requests in arrival order while their device footprint fits the arena
// budget (and the batch stays under max_batch grids), runs them as one batch,
// copies every complex back to host memory and completes the requests.  With
// two or more lanes a batch is admitted and copied while another computes, so
// requests that arrive while the GPU is busy join the next free lane
// (continuous batching).  A request's result is the complex of its grid
// alone: batching does not change any output.
//
// The exact simplification is sequential per grid and can be long on fields
// with many exact ties (its heap replays the reference's tie order), and a
// batch completes with its slowest grid.  So requests with tresh > 0 whose
// heights have more than 1% equal neighbour pairs are "heavy" and queue for
// the first half of the lanes (when there are two or more lanes: lanes / 2 of
// them); the other lanes never wait behind them, and a heavy request that
// arrives while a heavy batch runs starts on the next free heavy lane.  A request whose simplification exhausts the operation budget
// fails alone (DMSC_ERR_PARTIAL from the batch); its batch mates complete.
// Only a batch that fails as a whole (NaN heights, an allocation) is rerun
// one grid at a time.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "dmsc.h"
#include "dmsc_internal.h"
#include "grid_types.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t id = 0;
  int nx = 0, ny = 0;
  double tresh = 0;
  std::vector<float> heights;
  long long footprint = 0;
  double t_submit = 0, t_start = 0, t_done = 0;
  bool heavy = false;
  int status = -1;  // -1 pending, else DMSC_OK or an error code
  std::string error;
  int64_t sizes[3] = {0, 0, 0};
  std::vector<uint32_t> cellid, pair_idx, aoff, asc, doff, des;
  std::vector<float> fn;
  std::vector<uint8_t> flags;
};

// Device bytes one grid holds inside a batch: heights, codes, terms and
// labels per vertex, row counts / offsets and the border table per tile,
// and a bound on its critical points and arcs (a critical cell per 4
// vertices at most in practice; checked by the engine, which grows buffers
// when needed).  With a threshold, the simplification's first allocation for
// that many points and arcs (n = v/4 points, v arcs): list pool 4 (arcs +
// 8 n) runs of 8 B, heap and resubmit list 8 * (v/2) entries of 12 + 12 B,
// scratch runs 4 * arcs of 8 B, list descriptors and entry words 36 B per point.  A
// simplification that outgrows it retries with larger buffers, beyond this
// estimate.
long long footprint_of(int nx, int ny, bool simplify) {
  const long long v = (long long)nx * ny;
  const long long tiles = (long long)((nx + dmsc::TX - 1) / dmsc::TX) * ((ny + dmsc::TY - 1) / dmsc::TY);
  long long b = v * (4 + 4 + 4 + 16) + 2ll * ny * (long long)((nx + dmsc::TX - 1) / dmsc::TX) * 5 +
                tiles * dmsc::SLOTS_PER_TILE * 8 + (v / 4) * 64 + (1 << 16);
  if (simplify) {
    const long long n = v / 4, arcs = v;
    b += 8 * 4 * (arcs + 8 * n) + 24 * 8 * (v / 2) + 8 * 4 * arcs + 36 * n + (1 << 20);
  }
  return b;
}

}  // namespace

struct dmsc_server {
  dmsc_ctx *ctx = nullptr;
  long long arena = 0, in_use = 0;
  int max_batch = 0;
  long long max_ops = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Request>> queue, heavy;  // light and heavy requests
  int lanes = 1;
  std::unordered_map<int64_t, std::shared_ptr<Request>> all;
  int64_t next_id = 1;
  bool stop = false;
  Clock::time_point t0 = Clock::now();
  std::vector<std::thread> workers;
  long long batches = 0, grids_done = 0;

  double now_ms() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }
  void lane(int k);
};

void dmsc_server::lane(int k) {
  // the first lanes / 2 lanes take the heavy queue when there are other lanes;
  // a single lane takes both
  const int nheavy = lanes >= 2 ? lanes / 2 : 0;
  const bool heavy_lane = k < nheavy, light_lane = lanes == 1 || k >= nheavy;
  cudaSetDevice(ctx->device);
  cudaStream_t st = nullptr;
  cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  dmsc_batch *batch = nullptr;
  float *staging = nullptr;
  size_t staging_n = 0;
  uint32_t *ex = nullptr;  // pinned export buffer (words)
  size_t ex_n = 0, staging_n_prev = 0;
  // Pinned buffers outgrown while the server runs: freeing pinned memory
  // waits for the whole device (every lane's work), so they are kept until
  // the lane stops.
  std::vector<void *> retired;
  std::vector<std::shared_ptr<Request>> take;
  for (;;) {
    take.clear();
    long long fp = 0;
    {
      std::unique_lock<std::mutex> lk(mu);
      auto pick = [&]() -> std::deque<std::shared_ptr<Request>> * {
        if (light_lane && !queue.empty()) return &queue;
        if (heavy_lane && !heavy.empty()) return &heavy;
        if (lanes == 1 && !heavy.empty()) return &heavy;
        return nullptr;
      };
      auto ready = [&] {
        auto *q = pick();
        return q && (in_use + q->front()->footprint <= arena || in_use == 0);
      };
      cv_work.wait(lk, [&] { return stop || ready(); });
      auto *q = pick();
      if (stop && !q) break;
      if (!q) continue;
      // admit in arrival order while the footprint fits (a request larger than
      // the whole arena is admitted alone once the arena is empty)
      while (!q->empty() && (int)take.size() < max_batch) {
        const long long f = q->front()->footprint;
        if (in_use + fp + f > arena && !(take.empty() && in_use == 0)) break;
        take.push_back(q->front());
        q->pop_front();
        fp += f;
      }
      in_use += fp;
    }
    if (take.empty()) continue;
    const double t_start = now_ms();
    // pack heights into pinned staging memory
    size_t nv = 0;
    std::vector<int32_t> sizes;
    std::vector<double> tr;
    for (auto &r : take) {
      nv += (size_t)r->nx * r->ny;
      sizes.push_back(r->nx);
      sizes.push_back(r->ny);
      tr.push_back(r->tresh);
    }
    int rc = DMSC_OK;
    bool partial = false;
    std::string err;
    if (nv > staging_n) {  // grow (x2); the old buffer is freed when the lane stops
      if (staging) retired.push_back(staging);
      staging = nullptr;
      staging_n = 0;
      const size_t want = std::max(nv, 2 * staging_n_prev);
      if (cudaMallocHost((void **)&staging, sizeof(float) * want) == cudaSuccess) staging_n = staging_n_prev = want;
      else { rc = DMSC_ERR_OOM; err = "pinned staging"; }
    }
    if (rc == DMSC_OK) {
      size_t o = 0;
      for (auto &r : take) {
        std::memcpy(staging + o, r->heights.data(), sizeof(float) * r->heights.size());
        o += r->heights.size();
      }
      rc = dmsc_batch_run(ctx, (int)take.size(), sizes.data(), staging, 0, tr.data(), max_ops, &batch, st);
      if (rc == DMSC_ERR_PARTIAL) { rc = DMSC_OK; partial = true; }  // a failed grid's export returns its own error
      else if (rc) err = dmsc_last_error();
    }
    // a failed batch of several grids is rerun one grid at a time, so that
    // one bad request (NaN heights, an exhausted budget) fails alone
    std::vector<int> solo(take.size(), 0);
    if (rc != DMSC_OK && take.size() > 1) {
      size_t o = 0;
      for (size_t i = 0; i < take.size(); ++i) {
        Request &r = *take[i];
        const int32_t sz[2] = {r.nx, r.ny};
        solo[i] = dmsc_batch_run(ctx, 1, sz, staging + o, 0, &tr[i], max_ops, &batch, st);
        o += r.heights.size();
        if (solo[i] == DMSC_OK) solo[i] = 1000;  // done alone: export below, then mark
        else {
          r.error = dmsc_last_error();
          if (solo[i] == DMSC_ERR_PARTIAL) {  // the grid's own status and message
            char msg[512] = {0};
            dmsc_batch_grid_status(batch, 0, &solo[i], msg, (int)sizeof(msg));
            r.error = msg;
          }
          r.t_start = t_start;
          r.t_done = now_ms();
          std::lock_guard<std::mutex> lk(mu);
          r.status = solo[i];
          continue;
        }
        // export this grid now, before the batch object is reused
        int rrc = dmsc_batch_sizes(batch, 0, r.sizes);
        if (rrc == DMSC_OK) {
          const size_t n = (size_t)r.sizes[0];
          r.cellid.resize(n); r.fn.resize(n); r.pair_idx.resize(n); r.flags.resize(n);
          r.aoff.resize(n + 1); r.doff.resize(n + 1); r.asc.resize((size_t)r.sizes[1]); r.des.resize((size_t)r.sizes[2]);
          int16_t rect_ext[8];
          rrc = dmsc_batch_export(batch, 0, rect_ext, (int16_t *)r.cellid.data(), r.fn.data(), r.pair_idx.data(),
                                  r.flags.data(), r.aoff.data(), r.asc.data(), r.doff.data(), r.des.data(), st);
        }
        r.error = rrc ? dmsc_last_error() : std::string();
        r.t_start = t_start;
        r.t_done = now_ms();
        std::lock_guard<std::mutex> lk(mu);
        r.status = rrc;
      }
      for (auto &r : take) { r->heights.clear(); r->heights.shrink_to_fit(); }
    }
    // a batch without failed grids comes back in one set of copies into pinned
    // memory, split per request on the host
    bool bulk = false;
    if (rc == DMSC_OK && !partial && take.size() > 1) {
      int64_t tot[3] = {0, 0, 0};
      if (dmsc_batch_totals(batch, tot) == DMSC_OK) {
        const size_t g1 = take.size() + 1, ncp = (size_t)tot[0], na = (size_t)tot[1], nd = (size_t)tot[2];
        const size_t need = 3 * g1 + 4 * ncp + ncp + 2 * (ncp + 1) + na + nd + (ncp + 3) / 4 + 16;  // words
        if (need > ex_n) {  // grow (x2); the old buffer is freed when the lane stops
          if (ex) retired.push_back(ex);
          ex = nullptr;
          const size_t want = std::max(need, 2 * ex_n);
          ex_n = 0;
          if (cudaMallocHost((void **)&ex, sizeof(uint32_t) * want) == cudaSuccess) ex_n = want;
        }
        if (ex) {
          uint32_t *cpb = ex, *ab = cpb + g1, *db = ab + g1, *cell = db + g1, *fnb = cell + ncp, *pair = fnb + ncp;
          uint32_t *ao = pair + ncp, *asc = ao + ncp + 1, *dof = asc + na, *des = dof + ncp + 1;
          uint8_t *fl = (uint8_t *)(des + nd);
          bulk = dmsc_batch_export_all(batch, cpb, ab, db, cell, (float *)fnb, pair, fl, ao, asc, dof, des, st) == DMSC_OK;
          for (size_t i = 0; bulk && i < take.size(); ++i) {
            Request &r = *take[i];
            const size_t c0 = cpb[i], n = cpb[i + 1] - c0, a0 = ab[i], a1 = ab[i + 1], d0 = db[i], d1 = db[i + 1];
            r.t_start = t_start;
            r.sizes[0] = (int64_t)n; r.sizes[1] = (int64_t)(a1 - a0); r.sizes[2] = (int64_t)(d1 - d0);
            r.cellid.assign(cell + c0, cell + c0 + n);
            r.fn.assign((float *)fnb + c0, (float *)fnb + c0 + n);
            r.pair_idx.assign(pair + c0, pair + c0 + n);
            r.flags.assign(fl + c0, fl + c0 + n);
            r.asc.assign(asc + a0, asc + a1);
            r.des.assign(des + d0, des + d1);
            r.aoff.resize(n + 1);
            r.doff.resize(n + 1);
            for (size_t k = 0; k <= n; ++k) {
              r.aoff[k] = ao[c0 + k] - (uint32_t)a0;
              r.doff[k] = dof[c0 + k] - (uint32_t)d0;
            }
            r.heights.clear();
            r.heights.shrink_to_fit();
            r.error.clear();
            r.t_done = now_ms();
            std::lock_guard<std::mutex> lk(mu);
            r.status = DMSC_OK;
          }
        }
      }
    }
    for (size_t i = 0; !bulk && i < take.size() && !(rc != DMSC_OK && take.size() > 1); ++i) {
      Request &r = *take[i];
      r.t_start = t_start;
      int rrc = rc;
      if (rrc == DMSC_OK) rrc = dmsc_batch_sizes(batch, (int64_t)i, r.sizes);
      if (rrc == DMSC_OK) {
        const size_t n = (size_t)r.sizes[0];
        r.cellid.resize(n); r.fn.resize(n); r.pair_idx.resize(n); r.flags.resize(n);
        r.aoff.resize(n + 1); r.doff.resize(n + 1); r.asc.resize((size_t)r.sizes[1]); r.des.resize((size_t)r.sizes[2]);
        int16_t rect_ext[8];
        rrc = dmsc_batch_export(batch, (int64_t)i, rect_ext, (int16_t *)r.cellid.data(), r.fn.data(), r.pair_idx.data(),
                                r.flags.data(), r.aoff.data(), r.asc.data(), r.doff.data(), r.des.data(), st);
        if (rrc) err = dmsc_last_error();
      }
      r.heights.clear();
      r.heights.shrink_to_fit();
      r.error = rrc ? err : std::string();
      r.t_done = now_ms();
      std::lock_guard<std::mutex> lk(mu);
      r.status = rrc;
    }
    {
      std::lock_guard<std::mutex> lk(mu);
      in_use -= fp;
      ++batches;
      grids_done += (long long)take.size();
    }
    cv_done.notify_all();
    cv_work.notify_all();
  }
  if (batch) dmsc_batch_destroy(batch);
  if (staging) cudaFreeHost(staging);
  if (ex) cudaFreeHost(ex);
  for (void *p : retired) cudaFreeHost(p);
  cudaStreamDestroy(st);
}

extern "C" {

int dmsc_server_create(dmsc_ctx *ctx, int64_t arena_bytes, int lanes, int max_batch, int64_t max_ops, dmsc_server **out) {
  if (!ctx || !out) return dmsc::set_last_error(DMSC_ERR_BAD_ARG, "null argument");
  if (arena_bytes <= 0 || lanes < 1 || lanes > 16 || max_batch < 1)
    return dmsc::set_last_error(DMSC_ERR_BAD_ARG, "arena must be positive, lanes in [1, 16], max_batch >= 1");
  dmsc_server *s = new dmsc_server;
  s->ctx = ctx;
  s->arena = arena_bytes;
  s->max_batch = max_batch;
  s->max_ops = max_ops;
  s->lanes = lanes;
  for (int k = 0; k < lanes; ++k) s->workers.emplace_back([s, k] { s->lane(k); });
  *out = s;
  return DMSC_OK;
}

int dmsc_server_submit(dmsc_server *s, const float *heights, int nx, int ny, double tresh, int64_t *id) {
  if (!s || !heights || !id) return dmsc::set_last_error(DMSC_ERR_BAD_ARG, "null argument");
  if (nx < 2 || ny < 2 || nx > 16384 || ny > 16384 || !(tresh >= 0.0))
    return dmsc::set_last_error(DMSC_ERR_BAD_ARG, "grid must be 2..16384 vertices per side, tresh >= 0");
  auto r = std::make_shared<Request>();
  r->nx = nx; r->ny = ny; r->tresh = tresh;
  r->heights.assign(heights, heights + (size_t)nx * ny);
  r->footprint = footprint_of(nx, ny, tresh > 0.0);
  if (tresh > 0.0) {  // equal neighbour pairs along x and y
    size_t ties = 0;
    const float *h = r->heights.data();
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const size_t i = (size_t)y * nx + x;
        ties += (x + 1 < nx && h[i] == h[i + 1]) + (y + 1 < ny && h[i] == h[i + nx]);
      }
    r->heavy = ties * 100 > (size_t)nx * ny;
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->id = s->next_id++;
    r->t_submit = s->now_ms();
    (r->heavy ? s->heavy : s->queue).push_back(r);
    s->all[r->id] = r;
    *id = r->id;
  }
  s->cv_work.notify_one();
  return DMSC_OK;
}

// Waits up to timeout_ms (< 0: forever) for request id; *done = 1 once it has
// completed (its status is in *status).
int dmsc_server_wait(dmsc_server *s, int64_t id, int timeout_ms, int *done, int *status) {
  if (!s || !done) return dmsc::set_last_error(DMSC_ERR_BAD_ARG, "null argument");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return dmsc::set_last_error(DMSC_ERR_BAD_ARG, "no such request");
  auto r = it->second;
  auto ready = [&] { return r->status >= 0; };
  if (timeout_ms < 0) s->cv_done.wait(lk, ready);
  else s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready);
  *done = r->status >= 0;
  if (status) *status = r->status;
  return DMSC_OK;
}

int dmsc_server_result(dmsc_server *s, int64_t id, int64_t sizes[3], double times_ms[3], char *error, int error_len) {
  if (!s) return dmsc::set_last_error(DMSC_ERR_BAD_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return dmsc::set_last_error(DMSC_ERR_BAD_ARG, "no such request");
  const Request &r = *it->second;
  if (r.status < 0) return dmsc::set_last_error(DMSC_ERR_STATE, "request still pending");
  if (sizes) for (int q = 0; q < 3; ++q) sizes[q] = r.sizes[q];
  if (times_ms) { times_ms[0] = r.t_submit; times_ms[1] = r.t_start; times_ms[2] = r.t_done; }
  if (error && error_len > 0) {
    std::strncpy(error, r.error.c_str(), (size_t)error_len - 1);
    error[error_len - 1] = 0;
  }
  if (r.status != DMSC_OK) return dmsc::set_last_error(r.status, r.error.c_str());
  return DMSC_OK;
}

// The completed request's complex in the layout of dmsc_msc_export (no discs).
int dmsc_server_export(dmsc_server *s, int64_t id, int16_t *cellid, float *fn, uint32_t *pair_idx, uint8_t *flags,
                       uint32_t *asc_off, uint32_t *asc, uint32_t *des_off, uint32_t *des) {
  if (!s) return dmsc::set_last_error(DMSC_ERR_BAD_ARG, "null argument");
  std::shared_ptr<Request> rp;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return dmsc::set_last_error(DMSC_ERR_BAD_ARG, "no such request");
    rp = it->second;
    if (rp->status < 0) return dmsc::set_last_error(DMSC_ERR_STATE, "request still pending");
    if (rp->status != DMSC_OK) return dmsc::set_last_error(rp->status, rp->error.c_str());
  }
  const Request &r = *rp;
  const size_t n = r.cellid.size();
  if (cellid) std::memcpy(cellid, r.cellid.data(), 4 * n);
  if (fn) std::memcpy(fn, r.fn.data(), 4 * n);
  if (pair_idx) std::memcpy(pair_idx, r.pair_idx.data(), 4 * n);
  if (flags) std::memcpy(flags, r.flags.data(), n);
  if (asc_off) std::memcpy(asc_off, r.aoff.data(), 4 * (n + 1));
  if (des_off) std::memcpy(des_off, r.doff.data(), 4 * (n + 1));
  if (asc) std::memcpy(asc, r.asc.data(), 4 * r.asc.size());
  if (des) std::memcpy(des, r.des.data(), 4 * r.des.size());
  return DMSC_OK;
}

int dmsc_server_release(dmsc_server *s, int64_t id) {
  if (!s) return dmsc::set_last_error(DMSC_ERR_BAD_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return dmsc::set_last_error(DMSC_ERR_BAD_ARG, "no such request");
  if (it->second->status < 0) return dmsc::set_last_error(DMSC_ERR_STATE, "request still pending");
  s->all.erase(it);
  return DMSC_OK;
}

// [0] batches run, [1] grids completed, [2] queued, [3] arena bytes in use
int dmsc_server_stats(dmsc_server *s, int64_t stats[4]) {
  if (!s || !stats) return dmsc::set_last_error(DMSC_ERR_BAD_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  stats[0] = s->batches; stats[1] = s->grids_done; stats[2] = (int64_t)(s->queue.size() + s->heavy.size());
  stats[3] = s->in_use;
  return DMSC_OK;
}

int dmsc_server_destroy(dmsc_server *s) {
  if (!s) return dmsc::set_last_error(DMSC_ERR_BAD_ARG, "null argument");
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto &t : s->workers) t.join();
  delete s;
  return DMSC_OK;
}

}  // extern "C"
