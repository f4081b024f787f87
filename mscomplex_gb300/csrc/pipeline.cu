// pipeline.cu -- the whole grid pipeline of GridDataManager
// (dmsc/src/grid_datamanager.cpp:40-89, 121-140, 258-490, 596-662) on one GPU:
// pieces of the grid (binary splits with a one-vertex halo), one dataset and
// complex per piece, merge_up of the piece tree, simplify_un_simplify at the
// root, merge_down back to the pieces, and the manifold discs of every piece.
//
// The reference splits along y only (split_axes = 1, :50-51); split2d = 1
// alternates y and x splits per level to produce square blocks (merge_up and
// merge_down accept any shared 1-manifold, grid_mscomplex.cpp:35-39).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <unistd.h>

#include "dmsc.h"
#include "dmsc_internal.h"
#include "grid_types.h"
#include "host_pool.h"

using namespace dmsc;

namespace {
struct R4 {
  int l, b, r, t;
};
R4 rmake(int x0, int y0, int x1, int y1) { return R4{std::min(x0, x1), std::min(y0, y1), std::max(x0, x1), std::max(y0, y1)}; }

// createPieces_quadtree (:53-89)
void create_pieces(std::vector<std::pair<R4, R4>> &out, R4 r, R4 e, int level, int depth, bool split2d) {
  if (level == 0) { out.push_back({r, e}); return; }
  int dim = split2d ? ((depth % 2 == 0) ? 1 : 0) : 1;
  int s = dim ? (r.t - r.b) : (r.r - r.l);
  int tr1[2] = {r.r, r.t}, bl1[2] = {r.l, r.b};
  tr1[dim] -= 2 * (s / 4);
  bl1[dim] = tr1[dim];
  R4 r1 = rmake(r.l, r.b, tr1[0], tr1[1]), r2 = rmake(bl1[0], bl1[1], r.r, r.t);
  int tr2[2] = {e.r, e.t}, bl2[2] = {e.l, e.b};
  tr2[dim] = tr1[dim] + 2;
  bl2[dim] = bl1[dim] - 2;
  R4 e1 = rmake(e.l, e.b, tr2[0], tr2[1]), e2 = rmake(bl2[0], bl2[1], e.r, e.t);
  create_pieces(out, r1, e1, level - 1, depth + 1, split2d);
  create_pieces(out, r2, e2, level - 1, depth + 1, split2d);
}
// lexicographic std::min / std::max of two points (two_tuple_t order, x then y)
void pmin(int ax, int ay, int bx, int by, int &ox, int &oy) {
  bool a_lt = ax < bx || (ax == bx && ay < by);
  if (a_lt || (ax == bx && ay == by)) { ox = ax; oy = ay; } else { ox = bx; oy = by; }
}
void pmax(int ax, int ay, int bx, int by, int &ox, int &oy) {
  bool a_lt = ax < bx || (ax == bx && ay < by);
  if (a_lt) { ox = bx; oy = by; } else { ox = ax; oy = ay; }
}
double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

constexpr int PIECE_WORKERS = 8;
}  // namespace

struct dmsc_pipeline {
  dmsc_ctx *ctx = nullptr;
  int X = 0, Y = 0, levels = 0;
  bool split2d = false;
  double tresh = 0;
  std::vector<std::pair<R4, R4>> pieces;  // leaves (rect, ext)
  std::vector<dmsc_dataset *> ds;         // one per leaf
  std::vector<dmsc_msc *> msc;            // all 2N-1 tree nodes, leaves first
  DevBuf<float> field;                    // device copy when the input was on the host
  DevBuf<uint32_t> status;
  double ms[5] = {0, 0, 0, 0, 0};
  double seq_ms[2] = {0, 0};  // one-thread steps of the parallel merges: up, down
  unsigned long long simp[5] = {0, 0, 0, 0, 0};
  // out of core (GridDataManager's compute_out_of_core): the archive file
  // prefix of this run, and per tree node whether its archive exists
  std::string ooc;
  std::vector<char> archived;
  ~dmsc_pipeline() {
    for (auto *d : ds)
      if (d) dmsc_dataset_destroy(d);
    for (auto *m : msc)
      if (m) dmsc_msc_destroy(m);
    for (size_t i = 0; i < archived.size(); ++i)
      if (archived[i]) std::remove((ooc + std::to_string(i)).c_str());
  }
};

static int perr(int code, const std::string &m) { return set_last_error(code, m.c_str()); }
#define PCK(call)                                                                         \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) return perr(e_ == cudaErrorMemoryAllocation ? DMSC_ERR_OOM : DMSC_ERR_CUDA, \
                                       std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
#define PRC(call)              \
  do {                         \
    int r_ = (call);           \
    if (r_ != DMSC_OK) return r_; \
  } while (0)

// Out of core, as write_msgraph_to_archive / read_msgraph_from_archive
// (dmsc/src/grid_datamanager.cpp:91-119): a node's complex goes to its
// archive file and leaves the device; it is read back when a stage needs it.
static int archive_node(dmsc_pipeline *P, int node) {  // write, then free the device copy
  PRC(dmsc_msc_save(P->msc[node], (P->ooc + std::to_string(node)).c_str()));
  dmsc_msc_destroy(P->msc[node]);
  P->msc[node] = nullptr;
  P->archived[node] = 1;
  return DMSC_OK;
}
static int unarchive_node(dmsc_pipeline *P, int node) {
  if (P->msc[node]) return DMSC_OK;
  if (!P->archived[node]) return perr(DMSC_ERR_STATE, "piece " + std::to_string(node) + " has no complex");
  return dmsc_msc_load(P->ctx, (P->ooc + std::to_string(node)).c_str(), &P->msc[node]);
}
static void drop_node(dmsc_pipeline *P, int node) {  // its archive is current: free the device copy
  if (P->archived[node] && P->msc[node]) {
    dmsc_msc_destroy(P->msc[node]);
    P->msc[node] = nullptr;
  }
}

static dmsc_msc *new_msc(dmsc_ctx *c, const R4 &r, const R4 &e) {
  dmsc_msc *m = new dmsc_msc;
  m->ctx = c;
  m->rect[0] = r.l; m->rect[1] = r.b; m->rect[2] = r.r; m->rect[3] = r.t;
  m->ext[0] = e.l; m->ext[1] = e.b; m->ext[2] = e.r; m->ext[3] = e.t;
  return m;
}

// The shared 1-manifold of the children of `node` (rect_t::intersection,
// rectangle_complex.h); false when they do not share one.
static bool shared_edge(dmsc_pipeline *P, int node, int ixn[4]) {
  const int N = (int)P->pieces.size(), k = node - N;
  const dmsc_msc *ma = P->msc[2 * k], *mb = P->msc[2 * k + 1];
  const int x0 = std::max(ma->rect[0], mb->rect[0]), y0 = std::max(ma->rect[1], mb->rect[1]);
  const int x1 = std::min(ma->rect[2], mb->rect[2]), y1 = std::min(ma->rect[3], mb->rect[3]);
  ixn[0] = x0; ixn[1] = y0; ixn[2] = x1; ixn[3] = y1;
  return !(x0 > x1 || y0 > y1 || (x0 != x1 && y0 != y1) || (x0 == x1 && y0 == y1));
}

constexpr int LEVEL_FALLBACK = -1;

static void box_join(int *o, const int *a) {
  if (o[2] < o[0]) { for (int i = 0; i < 4; ++i) o[i] = a[i]; return; }
  o[0] = std::min(o[0], a[0]); o[1] = std::min(o[1], a[1]);
  o[2] = std::max(o[2], a[2]); o[3] = std::max(o[3], a[3]);
}

// One tree level through the parallel merges (merge_par.cu), with the same
// retries as below; LEVEL_FALLBACK when a merge needs the one-thread path.
static int run_level_par(dmsc_pipeline *P, bool up, const std::vector<int> &nodes, cudaStream_t st) {
  const int N = (int)P->pieces.size();
  std::vector<MergeJob> jobs;
  for (int node : nodes) {
    MergeJob J;
    const int k = node - N;
    J.a = P->msc[2 * k]; J.b = P->msc[2 * k + 1]; J.parent = P->msc[node];
    if (!shared_edge(P, node, J.ixn)) return perr(DMSC_ERR_INVARIANT, "pieces must share a 1-manifold");
    jobs.push_back(J);
  }
  for (int attempt = 0; attempt < 4; ++attempt) {
    const unsigned long long grow = 1ull << (2 * attempt);
    uint32_t stw = 0;
    cudaError_t e = up ? merge_up_level_par(jobs, grow, P->status.p, &stw, st, &P->seq_ms[0],
                                            P->ctx->merge_round_window, P->ctx->merge_round_min_commits)
                       : merge_down_level_par(jobs, grow, P->status.p, &stw, st, &P->seq_ms[1]);
    if (e != cudaSuccess)
      return perr(e == cudaErrorMemoryAllocation ? DMSC_ERR_OOM : DMSC_ERR_CUDA,
                  std::string("parallel merge level: ") + cudaGetErrorString(e));
    if (stw & ST_FALLBACK) {  // nothing was written back; the one-thread merge_up starts from an empty parent
      if (up)
        for (auto &J : jobs) J.parent->ncp = J.parent->nasc = J.parent->ndes = 0;
      return LEVEL_FALLBACK;
    }
    if (stw == ST_SIMPLIFY_LIMIT && attempt + 1 < 4) continue;
    if (stw & ST_SIMPLIFY_LIMIT) return perr(DMSC_ERR_DEVICE_TIMEOUT, "a merge ran out of list pool or table room");
    if (stw) return perr(DMSC_ERR_INVARIANT, "merge invariant violated (status " + std::to_string(stw) + ")");
    return DMSC_OK;
  }
  return perr(DMSC_ERR_DEVICE_TIMEOUT, "merge pools still too small after retries");
}

// One tree level of merges, with retries: a level that runs out of list pool
// is rerun from its unchanged inputs with larger pools.  Up: node N+k is built
// from nodes 2k and 2k+1.  Down: node N+k pushes into nodes 2k and 2k+1.
// Levels whose largest merge involves at least the context's
// merge_parallel_min critical points take the parallel merges.
static int run_level(dmsc_pipeline *P, bool up, const std::vector<int> &nodes, cudaStream_t st) {
  const int N = (int)P->pieces.size();
  // the box of cell coordinates holding a merged complex's critical cells:
  // its children's (a child's box after merge_down is measured afterwards)
  for (int node : nodes) {
    const int k = node - N;
    dmsc_msc *ma = P->msc[2 * k], *mb = P->msc[2 * k + 1], *mp = P->msc[node];
    if (up) { box_join(mp->bbox, ma->bbox); box_join(mp->bbox, mb->bbox); }
  }
  long long biggest = 0;
  for (int node : nodes) {
    const int k = node - N;
    long long n = P->msc[2 * k]->ncp + P->msc[2 * k + 1]->ncp + (up ? 0 : P->msc[node]->ncp);
    biggest = std::max(biggest, n);
  }
  if (biggest >= P->ctx->merge_parallel_min) {
    const int rc = run_level_par(P, up, nodes, st);
    if (rc != LEVEL_FALLBACK) return rc;
  }
  for (int attempt = 0; attempt < 4; ++attempt) {
    const unsigned long long grow = 1ull << (2 * attempt);
    std::vector<MGraphHost> g(3 * nodes.size());
    std::vector<int> jobs, ixn, gnode(3 * nodes.size(), -1);
    int rc = DMSC_OK;
    if (cudaMemsetAsync(P->status.p, 0, 4, st) != cudaSuccess) return perr(DMSC_ERR_CUDA, "merge status");
    for (auto &h : g) h.status = P->status.p;
    for (size_t j = 0; j < nodes.size() && rc == DMSC_OK; ++j) {
      const int node = nodes[j], k = node - N, a = 2 * k, b = 2 * k + 1;
      dmsc_msc *ma = P->msc[a], *mb = P->msc[b], *mp = P->msc[node];
      int x[4];
      if (!shared_edge(P, node, x)) return perr(DMSC_ERR_INVARIANT, "pieces must share a 1-manifold");
      const int x0 = x[0], y0 = x[1], x1 = x[2], y1 = x[3];
      const int ia = 3 * (int)j, ib = ia + 1, ip = ia + 2;
      gnode[ia] = a; gnode[ib] = b; gnode[ip] = node;
      const unsigned long long pa = ma->nasc + ma->ndes + 8ull * ma->ncp;
      const unsigned long long pb = mb->nasc + mb->ndes + 8ull * mb->ncp;
      const unsigned long long pp = mp->nasc + mp->ndes + 8ull * mp->ncp;
      cudaError_t e;
      if (up) {  // children read-only, parent starts empty
        e = mgraph_alloc(g[ia], *ma, (uint32_t)ma->ncp, pa + 1024, st);
        if (e == cudaSuccess) e = mgraph_alloc(g[ib], *mb, (uint32_t)mb->ncp, pb + 1024, st);
        if (e == cudaSuccess)
          e = mgraph_alloc(g[ip], *mp, (uint32_t)(ma->ncp + mb->ncp + 16), grow * 2 * (pa + pb) + 4096, st);
        jobs.insert(jobs.end(), {ia, ib, ip});
      } else {  // parent uncancels its boundary, children take the parent's cps (tables over both boxes)
        int boxa[4], boxb[4];
        for (int i = 0; i < 4; ++i) { boxa[i] = ma->bbox[i]; boxb[i] = mb->bbox[i]; }
        box_join(boxa, mp->bbox);
        box_join(boxb, mp->bbox);
        e = mgraph_alloc(g[ip], *mp, (uint32_t)mp->ncp, grow * 2 * pp + 4096, st);
        if (e == cudaSuccess)
          e = mgraph_alloc(g[ia], *ma, (uint32_t)(ma->ncp + mp->ncp + 16), grow * 2 * (pa + pp) + 4096, st, 4, nullptr,
                           boxa);
        if (e == cudaSuccess)
          e = mgraph_alloc(g[ib], *mb, (uint32_t)(mb->ncp + mp->ncp + 16), grow * 2 * (pb + pp) + 4096, st, 4, nullptr,
                           boxb);
        jobs.insert(jobs.end(), {ip, ia, ib});
      }
      ixn.insert(ixn.end(), {x0, y0, x1, y1});
      if (e != cudaSuccess) rc = perr(DMSC_ERR_OOM, std::string("merge graphs: ") + cudaGetErrorString(e));
    }
    uint32_t stw = 0;
    if (rc == DMSC_OK) {
      cudaError_t e =
          merge_level(up, g.data(), (int)g.size(), jobs.data(), ixn.data(), (int)nodes.size(), P->status.p, st);
      if (e == cudaSuccess) e = cudaMemcpy(&stw, P->status.p, 4, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) rc = perr(DMSC_ERR_CUDA, std::string("merge level: ") + cudaGetErrorString(e));
    }
    const bool retry = rc == DMSC_OK && stw == ST_SIMPLIFY_LIMIT && attempt + 1 < 4;
    if (rc == DMSC_OK && !retry) {
      if (stw & ST_SIMPLIFY_LIMIT) rc = perr(DMSC_ERR_DEVICE_TIMEOUT, "a merge ran out of list pool or table room");
      else if (stw) rc = perr(DMSC_ERR_INVARIANT, "merge invariant violated (status " + std::to_string(stw) + ")");
      // merge up changes the new nodes; merge down the parents and children
      for (size_t i = 0; i < g.size() && rc == DMSC_OK; ++i) {
        if (up && (i % 3) != 2) continue;
        cudaError_t e = mgraph_to_csr(g[i], *P->msc[gnode[i]], st);
        if (e == cudaSuccess && !up && (i % 3) != 2) e = cell_box(*P->msc[gnode[i]], st);  // a child
        if (e != cudaSuccess) rc = perr(DMSC_ERR_CUDA, std::string("merge writeback: ") + cudaGetErrorString(e));
      }
    }
    for (auto &h : g) mgraph_free(h, st);
    cudaStreamSynchronize(st);
    if (!retry) return rc;
  }
  return perr(DMSC_ERR_DEVICE_TIMEOUT, "merge pools still too small after retries");
}

extern "C" {

int dmsc_pipeline_run(dmsc_ctx *ctx, const float *heights, int64_t pitch, int on_device, int size_x, int size_y,
                      int levels, double tresh, int split2d, dmsc_pipeline **out, void *stream) {
  if (!ctx || !heights || !out) return perr(DMSC_ERR_BAD_ARG, "null argument");
  if (size_x < 2 || size_y < 2 || pitch < size_x || levels < 0 || levels > 16 || !(tresh >= 0))
    return perr(DMSC_ERR_BAD_ARG, "bad grid size, pitch, levels or threshold");
  if (size_x > 16384 || size_y > 16384) return perr(DMSC_ERR_INT16_OVERFLOW, "cell ids exceed int16");
  PCK(cudaSetDevice(ctx->device));
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  dmsc_pipeline *P = new dmsc_pipeline;
  P->ctx = ctx; P->X = size_x; P->Y = size_y; P->levels = levels; P->tresh = tresh; P->split2d = split2d != 0;
  auto fail = [&](int rc) { delete P; return rc; };
  const float *dev = heights;
  if (!on_device) {
    if (P->field.ensure((size_t)size_x * size_y) != cudaSuccess) return fail(perr(DMSC_ERR_OOM, "field"));
    if (cudaMemcpy2DAsync(P->field.p, 4ull * size_x, heights, 4ull * pitch, 4ull * size_x, size_y,
                          cudaMemcpyHostToDevice, st) != cudaSuccess)
      return fail(perr(DMSC_ERR_CUDA, "field copy"));
    dev = P->field.p;
    pitch = size_x;
  }
  if (P->status.ensure(4) != cudaSuccess) return fail(perr(DMSC_ERR_OOM, "status"));
  R4 whole{0, 0, 2 * (size_x - 1), 2 * (size_y - 1)};
  create_pieces(P->pieces, whole, whole, levels, 0, split2d != 0);
  const int N = (int)P->pieces.size();
  P->msc.assign(2 * N - 1, nullptr);
  P->archived.assign(2 * N - 1, 0);
  // out of core only with pieces to merge (grid_datamanager.cpp:640-641)
  const bool ooc = !ctx->ooc_dir.empty() && levels > 0;
  if (ooc) {
    static std::atomic<unsigned long long> serial{0};
    P->ooc = ctx->ooc_dir + "/dp_msgraph_" + std::to_string((long long)getpid()) + "_" + std::to_string(serial++) + "_";
  }
  // a leaf's dataset: its window of the field, the gradient (work or work_ocl)
  auto leaf_dataset = [&](int i, cudaStream_t s) {
    const R4 &r = P->pieces[i].first, &e = P->pieces[i].second;
    int16_t rr[4] = {(int16_t)r.l, (int16_t)r.b, (int16_t)r.r, (int16_t)r.t};
    int16_t ee[4] = {(int16_t)e.l, (int16_t)e.b, (int16_t)e.r, (int16_t)e.t};
    int q = dmsc_dataset_create(ctx, rr, ee, &P->ds[i]);
    if (!q) q = dmsc_dataset_init(P->ds[i], dev + (long long)(e.b / 2) * pitch + e.l / 2, pitch, 1, s);
    if (!q) q = P->ctx->use_ocl ? dmsc_dataset_work_ocl(P->ds[i], s) : dmsc_dataset_work(P->ds[i], s);
    return q;
  };
  // out of core: the leaf's complex to its archive, its dataset freed (dataset->clear())
  auto leaf_out = [&](int i, cudaStream_t s) {
    int q = cudaStreamSynchronize(s) == cudaSuccess ? DMSC_OK : perr(DMSC_ERR_CUDA, "leaf stream");
    if (!q) q = archive_node(P, i);
    dmsc_dataset_destroy(P->ds[i]);
    P->ds[i] = nullptr;
    return q;
  };
  double t0 = now_ms();
  // computeSubdomainMsgraphs (:493-528): every leaf independently, several at a time
  if (cudaStreamSynchronize(st) != cudaSuccess) return fail(perr(DMSC_ERR_CUDA, "field copy"));
  P->ds.assign(N, nullptr);
  {
    std::string msg;
    std::mutex mu;
    const int rc = for_each_on_streams(ctx->device, N, PIECE_WORKERS, [&](int i, cudaStream_t s) {
      int q = leaf_dataset(i, s);
      if (!q) q = dmsc_dataset_writeout_connectivity(P->ds[i], &P->msc[i], s);
      if (!q && ooc) q = leaf_out(i, s);
      if (q) { std::lock_guard<std::mutex> lk(mu); msg = dmsc_last_error(); }
      return q;
    });
    if (rc) return fail(perr(rc < 0 ? DMSC_ERR_CUDA : rc, rc < 0 ? "worker stream" : msg));
  }
  double t1 = now_ms();
  // mergePiecesUp (:258-306), one level at a time
  {
    int lo = 0, cnt = N;
    while (cnt > 1) {
      // node N+k merges 2k and 2k+1; this level's inputs are [lo, lo+cnt)
      std::vector<int> nodes;
      for (int j = lo; j < lo + cnt; j += 2) nodes.push_back(N + j / 2);
      if (ooc)  // the level's inputs back from their archives
        for (int node : nodes) {
          int rc = unarchive_node(P, 2 * (node - N));
          if (!rc) rc = unarchive_node(P, 2 * (node - N) + 1);
          if (rc) return fail(rc);
        }
      for (int node : nodes) {
        int k = node - N;
        dmsc_msc *a = P->msc[2 * k], *b = P->msc[2 * k + 1];
        // merged rects: lexicographic min of bottom-lefts, max of top-rights (grid_mscomplex.cpp:43-49)
        int rx0, ry0, rx1, ry1, ex0, ey0, ex1, ey1;
        pmin(a->rect[0], a->rect[1], b->rect[0], b->rect[1], rx0, ry0);
        pmax(a->rect[2], a->rect[3], b->rect[2], b->rect[3], rx1, ry1);
        pmin(a->ext[0], a->ext[1], b->ext[0], b->ext[1], ex0, ey0);
        pmax(a->ext[2], a->ext[3], b->ext[2], b->ext[3], ex1, ey1);
        P->msc[node] = new_msc(ctx, rmake(rx0, ry0, rx1, ry1), rmake(ex0, ey0, ex1, ey1));
      }
      int rc = run_level(P, true, nodes, st);
      if (rc) return fail(rc);
      if (ooc)  // inputs stay in their archives; new nodes but the root go to theirs
        for (int node : nodes) {
          drop_node(P, 2 * (node - N));
          drop_node(P, 2 * (node - N) + 1);
          if (cnt > 2 && (rc = archive_node(P, node))) return fail(rc);
        }
      lo += cnt;
      cnt /= 2;
    }
  }
  double t2 = now_ms();
  // simplify_un_simplify at the root (:651-652)
  if (tresh > 0.0) {
    int rc = dmsc_msc_simplify_un_simplify(P->msc[2 * N - 2], tresh, 0, st);
    for (int i = 0; i < 5; ++i) P->simp[i] = P->msc[2 * N - 2]->simp_stats[i];
    if (rc) return fail(rc);
  }
  double t3 = now_ms();
  // mergePiecesDown + finalMergeDownPiecesInRange (:308-395): root first
  {
    std::vector<std::pair<int, int>> lv;  // [first, last] node of each level, bottom up
    int lo = 0, cnt = N;
    while (cnt > 1) { lv.push_back({N + lo / 2, N + (lo + cnt) / 2 - 1}); lo += cnt; cnt /= 2; }
    for (size_t q = lv.size(); q-- > 0;) {
      std::vector<int> nodes;
      for (int n2 = lv[q].second; n2 >= lv[q].first; --n2) nodes.push_back(n2);
      int rc = DMSC_OK;
      if (ooc)
        for (int node : nodes)
          for (int x : {node, 2 * (node - N), 2 * (node - N) + 1})
            if ((rc = unarchive_node(P, x))) return fail(rc);
      rc = run_level(P, false, nodes, st);
      if (rc) return fail(rc);
      if (ooc)  // the parents and children changed: all back to their archives
        for (int node : nodes)
          for (int x : {node, 2 * (node - N), 2 * (node - N) + 1})
            if ((rc = archive_node(P, x))) return fail(rc);
    }
  }
  double t4 = now_ms();
  // collectSubdomainManifolds (:454-490): discs of every leaf, several at a time
  if (cudaStreamSynchronize(st) != cudaSuccess) return fail(perr(DMSC_ERR_CUDA, "merge down"));
  {
    std::string msg;
    std::mutex mu;
    const int rc = for_each_on_streams(ctx->device, N, PIECE_WORKERS, [&](int i, cudaStream_t s) {
      int q = DMSC_OK;
      if (ooc) {  // collectManifold (:397-422): the gradient again, the complex from its archive
        q = leaf_dataset(i, s);
        if (!q) q = unarchive_node(P, i);
      }
      if (!q) q = dmsc_dataset_fill_discs(P->ds[i], P->msc[i], s);
      if (!q && ooc) q = leaf_out(i, s);
      if (q) { std::lock_guard<std::mutex> lk(mu); msg = dmsc_last_error(); }
      return q;
    });
    if (rc) return fail(perr(rc < 0 ? DMSC_ERR_CUDA : rc, rc < 0 ? "worker stream" : msg));
  }
  double t5 = now_ms();
  P->ms[0] = t1 - t0; P->ms[1] = t2 - t1; P->ms[2] = t3 - t2; P->ms[3] = t4 - t3; P->ms[4] = t5 - t4;
  *out = P;
  return DMSC_OK;
}

int dmsc_pipeline_destroy(dmsc_pipeline *p) {
  if (!p) return perr(DMSC_ERR_BAD_ARG, "pipeline is null");
  const int device = p->ctx->device;
  cudaSetDevice(device);
  delete p;
  // A pipeline over a large field leaves tens of GB of differently sized
  // blocks in the stream-ordered pool, which the next one cannot always
  // reuse; keep a working set cached and hand the rest back.
  cudaMemPool_t pool;
  size_t total = 0, free_b = 0;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess && cudaMemGetInfo(&free_b, &total) == cudaSuccess)
    cudaMemPoolTrimTo(pool, total / 2);
  return DMSC_OK;
}

int dmsc_pipeline_num_pieces(dmsc_pipeline *p, int64_t *n) {
  if (!p || !n) return perr(DMSC_ERR_BAD_ARG, "null argument");
  *n = (int64_t)p->pieces.size();
  return DMSC_OK;
}

int dmsc_pipeline_piece(dmsc_pipeline *p, int64_t i, dmsc_msc **msc, dmsc_dataset **ds) {
  if (!p || i < 0 || i >= (int64_t)p->msc.size()) return perr(DMSC_ERR_BAD_ARG, "no such piece");
  if (msc) PRC(unarchive_node(p, (int)i));  // out of core: read back on first use
  if (msc) *msc = p->msc[i];
  if (ds) *ds = i < (int64_t)p->ds.size() ? p->ds[i] : nullptr;
  return DMSC_OK;
}

int dmsc_pipeline_write_discs(dmsc_pipeline *p, const char *prefix) {
  if (!p || !prefix) return perr(DMSC_ERR_BAD_ARG, "null argument");
  for (size_t i = 0; i < p->pieces.size(); ++i) {
    PRC(unarchive_node(p, (int)i));
    PRC(dmsc_msc_write_discs(p->msc[i], prefix));
  }
  return DMSC_OK;
}

int dmsc_pipeline_stage_times(dmsc_pipeline *p, double ms[5]) {
  if (!p || !ms) return perr(DMSC_ERR_BAD_ARG, "null argument");
  std::memcpy(ms, p->ms, sizeof(p->ms));
  return DMSC_OK;
}

int dmsc_pipeline_merge_times(dmsc_pipeline *p, double ms[2]) {
  if (!p || !ms) return perr(DMSC_ERR_BAD_ARG, "null argument");
  std::memcpy(ms, p->seq_ms, sizeof(p->seq_ms));
  return DMSC_OK;
}

}  // extern "C"
