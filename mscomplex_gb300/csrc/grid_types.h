// grid_types.h -- host-side handle types behind the C ABI (device-resident data).
#pragma once
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "dmsc.h"
#include "dmsc_common.cuh"

// Grow-only device buffer.  ensure(count) uses cudaMalloc / cudaFree (which
// synchronise the device); ensure(count, stream) uses the stream-ordered pool,
// so growing a buffer never waits for work on other streams.  A buffer that
// came from the pool is returned to it on release (ordered on the legacy
// stream: every use of it has completed by then, each call that fills one
// synchronises its own stream before returning).
template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  bool pooled = false;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  cudaError_t ensure(size_t count) {
    if (count <= n && p) return cudaSuccess;
    release();
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)&p, sizeof(T) * count);
    if (e != cudaSuccess) { p = nullptr; n = 0; return e; }
    n = count;
    return cudaSuccess;
  }
  cudaError_t ensure(size_t count, cudaStream_t st) {
    if (count <= n && p) return cudaSuccess;
    if (p) {
      if (pooled) cudaFreeAsync(p, st);
      else cudaFree(p);
    }
    p = nullptr;
    n = 0;
    if (count == 0) count = 1;
    cudaError_t e = cudaMallocAsync((void **)&p, sizeof(T) * count, st);
    if (e != cudaSuccess) { p = nullptr; return e; }
    n = count;
    pooled = true;
    return cudaSuccess;
  }
  void release() {
    if (p) {
      if (pooled) cudaFreeAsync(p, 0);
      else cudaFree(p);
    }
    p = nullptr;
    n = 0;
    pooled = false;
  }
};

// GridDataset (dmsc/include/grid_dataset.h:35-240) with device-resident cell arrays.
struct dmsc_dataset {
  dmsc_ctx *ctx = nullptr;
  int16_t rect[4], ext[4];
  dmsc::GridGeom g;
  const float *hgt = nullptr;  // heights on the device (owned copy or borrowed)
  DevBuf<float> hown;
  DevBuf<uint32_t> codes;      // uchar4 gradient codes per vertex
  DevBuf<uint32_t> terms;      // in-tile path terminals of the vertex and face of each vertex (2 x uint16)
  DevBuf<uint4> labels;        // owner labels (cp indices) of the 4 cells of each vertex
  DevBuf<uint8_t> rowcnt;      // critical cells per (cell row, tile column)
  DevBuf<uint32_t> offsets;    // exclusive scan of rowcnt: first cp index of each segment
  DevBuf<uint64_t> table;      // border table
  DevBuf<uint32_t> scal;       // [0] status word, [1] number of critical points
  uint32_t *host_scal = nullptr;
  uint32_t *host_disc = nullptr;  // pinned counts of fill_discs (16 words)
  cudaStream_t disc_aux = nullptr;  // fill_discs' second stream and its two ordering events
  cudaEvent_t disc_ev[2] = {nullptr, nullptr};
  long long cap = 0;           // capacity of the cp arrays
  long long ncp = 0;
  bool worked = false;
  DevBuf<uint32_t> cp_cellid, cp_pair_cell, cp_des2, cp_asc2, cp_acnt, cp_dcnt, cp_pair_idx;
  DevBuf<float> cp_fn;
  DevBuf<uint8_t> cp_flags;
  cudaEvent_t ev[14] = {};    // stage events (only when the context has timing enabled)
  bool ev_ready = false;

  long long nslots() const { return (long long)g.ntx * g.nty * dmsc::SLOTS_PER_TILE; }
  bool rect_is_ext() const {
    return rect[0] == ext[0] && rect[1] == ext[1] && rect[2] == ext[2] && rect[3] == ext[3];
  }
  int alloc_cells(cudaStream_t st);
  int alloc_cps(long long n, cudaStream_t st);
  ~dmsc_dataset();
};

// GridMSComplex (dmsc/include/grid_mscomplex.h:48-84) as flat device arrays.
struct dmsc_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool timing = false;
  long long merge_parallel_min = 2048;  // pipeline levels with merges this large take the parallel merges
  // merge_up's boundary cancellations in ordered-parallel rounds: each round
  // looks at the first merge_round_window pending boundary cells (0, the
  // default: one thread per merge, measured faster on noise); after 8 rounds
  // in a row that each commit fewer than merge_round_min_commits cells, one
  // thread finishes the rest in order
  long long merge_round_window = 0, merge_round_min_commits = 4;
  bool use_ocl = false;  // pipeline pieces through work_ocl (GridDataManager's ocl flag)
  std::string ooc_dir;   // pipelines spill their pieces' complexes to files here (empty: in memory)
  // batch launch configurations per size class (dmsc_batch_autotune): threads
  // per block and resident blocks per SM of the persistent tile kernels
  bool batch_tuned = false;
  int batch_cfg[6][2] = {{512, 3}, {512, 3}, {512, 3}, {512, 3}, {512, 3}, {512, 3}};
};

struct dmsc_msc {
  dmsc_ctx *ctx = nullptr;
  int16_t rect[4], ext[4];
  int bbox[4] = {0, 0, -1, -1};  // a box (l, b, r, t) of cell coordinates holding every critical cell
  long long ncp = 0, nasc = 0, ndes = 0, nadisc = 0, nddisc = 0;
  DevBuf<uint32_t> cellid, pair_idx, aoff, asc, doff, des, adoff, ddoff;
  DevBuf<uint32_t> adisc, ddisc;  // packed cell ids
  DevBuf<float> fn;
  DevBuf<uint8_t> flags;  // bit0 isCancelled, bit1 isOnStrangulationPath, bit2 isBoundryCancelable
  unsigned long long simp_stats[5] = {0, 0, 0, 0, 0};
  bool any_bcancel = true;  // false only when known to hold no boundary-cancelable point

  int writeout_from(const dmsc_dataset &d, cudaStream_t st);
};
