// dmsc_internal.h -- launchers shared between the CUDA translation units.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <vector>
#include "dmsc_common.cuh"

namespace dmsc {

// Number of kernels this library has launched (process-wide, all devices).
extern unsigned long long g_kernel_launches;
#define DMSC_LAUNCHED(n) __atomic_fetch_add(&::dmsc::g_kernel_launches, (unsigned long long)(n), __ATOMIC_RELAXED)

// Critical-point outputs of the label kernel (one entry per cp index).
struct CpOut {
  uint32_t *cellid;   // packed global (x | y<<16)
  float *fn;
  uint8_t *flags;     // bit0 PAIRED (isBoundryCancelable after writeout)
  uint32_t *pair_cell;// packed global cellid of the pair (paired critical cells only)
  uint32_t *des2;     // saddles: 2 facet (minimum) labels, ascending, LABEL_NONE padded
  uint32_t *asc2;     // saddles: 2 cofacet (maximum) labels
  uint32_t *acnt;     // per cp: |asc| (saddles written, minima counted atomically)
  uint32_t *dcnt;     // per cp: |des|
  long long cap;      // capacity of every array above (in critical points)
};

// One grid of a batch: its geometry (with batch-wide slot / segment bases)
// and its parts of the batch's packed arrays.
struct BatchGrid {
  GridGeom g;
  const float *hgt;
  uint32_t *codes, *terms;
  uint4 *labels;
  uint8_t *rowcnt;
  uint64_t *table;
  const uint32_t *offsets;  // the batch's cp offsets from this grid's first row segment on
  long long tile0;          // first tile of this grid in the batch's tile numbering
};
// Launch configuration of the batch's persistent tile kernels (chosen per
// size class by dmsc_batch_autotune): threads per block (256 or 512) and
// resident blocks per SM (1..3).
struct BatchLaunch {
  int threads = 512, blocks_per_sm = 3;
};
cudaError_t launch_gradient_batch(const BatchGrid *grids, int ngrids, long long ntiles, uint32_t *status, cudaStream_t st,
                                  BatchLaunch cfg = BatchLaunch());
cudaError_t launch_labels_batch(const BatchGrid *grids, int ngrids, long long ntiles, const CpOut &cp, uint32_t *status,
                                cudaStream_t st, BatchLaunch cfg = BatchLaunch());

size_t grad_smem_bytes();
size_t label_smem_bytes();
cudaError_t launch_gradient(const float *hgt, const GridGeom &g, uint32_t *codes, uint32_t *terms, uint8_t *rowcnt,
                            uint64_t *table, uint32_t *status, cudaStream_t st);
cudaError_t launch_resolve(uint64_t *table, long long nslots, const uint32_t *offsets, long long nseg, uint32_t *status,
                           cudaStream_t st);
cudaError_t launch_labels(const uint32_t *codes, const uint32_t *terms, const float *hgt, const GridGeom &g,
                          const uint32_t *offsets, const uint64_t *table, uint4 *labels, const CpOut &cp,
                          uint32_t *status, cudaStream_t st);

cudaError_t scan_exclusive_u8(const uint8_t *in, long long n, uint32_t *out, uint32_t *total, cudaStream_t st);
cudaError_t scan_exclusive_u32(const uint32_t *in, long long n, uint32_t *out, uint32_t *total, cudaStream_t st);
// dst[0..n) = src[0..n) on the device with a kernel (no copy engine: see
// read_words)
cudaError_t copy_u32(uint32_t *dst, const uint32_t *src, long long n, cudaStream_t st);
// Reads up to 8 device words src[0..n) into host[0..n) with a one-warp kernel
// that stores into the pinned host memory directly (memory from
// cudaMallocHost / cudaHostAlloc, which kernels address by the same pointer).
// A small read-back done this way does not use a copy engine, so it does not
// queue behind large device-to-host copies that other streams have in flight.
// host[] holds the words once `st` is synchronised.
cudaError_t read_words(uint32_t *host, const uint32_t *const *src, int n, cudaStream_t st);
long long scan_scratch_words(long long n);
cudaError_t scan_exclusive_u32_scratch(const uint32_t *in, long long n, uint32_t *out, uint32_t *total,
                                       uint32_t *scratch, cudaStream_t st);
// Records the calling thread's last error message (dmsc_last_error) and returns `code`.
int set_last_error(int code, const char *msg);
cudaError_t radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *ktmp, uint32_t *vtmp, long long n, int nbits,
                             cudaStream_t st);
cudaError_t sort_pairs_batched(uint32_t *dk, uint32_t *dv, const uint32_t *sk, const uint32_t *sv, uint32_t batch,
                               uint32_t len, uint32_t dir, cudaStream_t st);
cudaError_t build_csr(long long ncp, const uint32_t *cellid, const uint32_t *des2, const uint32_t *asc2,
                      const uint32_t *aoff, const uint32_t *doff, uint32_t *asc, uint32_t *des, long long out_cap,
                      uint32_t *status, cudaStream_t st);
cudaError_t build_csr_radix(long long ncp, const uint32_t *cellid, const uint32_t *des2, const uint32_t *asc2,
                      const uint32_t *aoff, const uint32_t *doff, uint32_t *asc, uint32_t *des, long long out_cap,
                      uint32_t *status, cudaStream_t st);
cudaError_t launch_pair_index(long long ncp, const uint32_t *cellid, const uint8_t *flags, const uint32_t *pair_cell,
                              uint32_t *pair_idx, uint32_t *status, cudaStream_t st);
cudaError_t launch_msc_flags(long long ncp, const uint8_t *cpflags, uint8_t *out, cudaStream_t st);
cudaError_t launch_export_cells(const GridGeom &g, const uint32_t *codes, const uint4 *labels, const uint32_t *cp_cellid,
                                long long ncp, int8_t *flags, int16_t *pairs, int16_t *own, cudaStream_t st);

// Persistence simplification (simplify.cu): run, then emit the new CSR into
// buffers of nasc_out / ndes_out entries, then release.
struct SimplifyIO {
  long long ncp = 0, nasc = 0, ndes = 0;
  const uint32_t *cellid = nullptr;
  const float *fn = nullptr;
  uint8_t *flags = nullptr;      // updated by simplify_emit
  uint32_t *pair_idx = nullptr;  // updated by simplify_emit
  uint32_t *aoff = nullptr, *asc = nullptr, *doff = nullptr, *des = nullptr;  // offsets rewritten by simplify_run
  int rect[4] = {0, 0, 0, 0};
  double tresh = 0;
  unsigned long long max_ops = 0;
  unsigned long long heap_cap = 0, tmp_cap = 0, pool_extra = 0;  // 0 = defaults
  unsigned long long *host_stats = nullptr;  // [0] pushes [1] pops [2] cancels [3] ops [4] status
  long long nasc_out = 0, ndes_out = 0;
  void *work = nullptr;
};
cudaError_t simplify_run(SimplifyIO &io, cudaStream_t st);

cudaError_t simplify_emit(SimplifyIO &io, uint32_t *asc, uint32_t *des, cudaStream_t st);
void simplify_release(SimplifyIO &io, cudaStream_t st);

// Simplification of many complexes held in shared arrays (a batch): critical
// points of grid g are [cpb[g], cpb[g+1]) with list values local to the grid;
// one block per grid with tresh > 0.  flags / pair_idx are edited in place.
struct BatchSimplifyIO {
  long long ncp = 0, nasc = 0, ndes = 0;  // batch totals
  const uint32_t *cellid = nullptr;
  const float *fn = nullptr;
  uint8_t *flags = nullptr;
  uint32_t *pair_idx = nullptr;
  uint32_t *aoff = nullptr, *asc = nullptr, *doff = nullptr, *des = nullptr;  // offsets rewritten by the run
  int ngrids = 0;
  const uint32_t *cpb = nullptr, *abase = nullptr, *dbase = nullptr;  // host, ngrids + 1 each
  const double *tresh = nullptr;  // host, per grid
  const int *rect = nullptr;      // host, 4 per grid
  unsigned long long max_ops = 0;
  unsigned long long scale = 1;              // multiplies every per-grid capacity
  unsigned long long *host_stats = nullptr;  // host, 5 per grid
  long long nasc_out = 0, ndes_out = 0;
  void *work = nullptr;
};
cudaError_t simplify_batch_run(BatchSimplifyIO &io, cudaStream_t st);
cudaError_t simplify_batch_offsets(BatchSimplifyIO &io, const std::vector<int> &dead, cudaStream_t st);
cudaError_t simplify_batch_emit(BatchSimplifyIO &io, uint32_t *asc, uint32_t *des, cudaStream_t st);
void simplify_batch_release(BatchSimplifyIO &io, cudaStream_t st);

}  // namespace dmsc
template <typename T> struct DevBuf;
namespace dmsc {
// Manifold discs (discs.cu): postMergeFillDiscs of one dataset into its complex.
struct DiscIO {
  GridGeom g;
  const uint32_t *codes = nullptr;
  const uint4 *labels = nullptr;
  long long ncp_ds = 0, ncp = 0, nasc = 0, ndes = 0;
  const uint32_t *cellid = nullptr;
  const uint8_t *flags = nullptr;
  const uint32_t *pair_idx = nullptr;
  const uint32_t *aoff = nullptr, *asc = nullptr, *doff = nullptr, *des = nullptr;
  uint32_t *adoff = nullptr, *ddoff = nullptr;  // ncp+1 each (outputs)
  DevBuf<uint32_t> *adisc = nullptr, *ddisc = nullptr;
  uint32_t *status = nullptr;
  unsigned long long limit = 1ull << 31;  // bound on one gradient chain (cells of the window)
  cudaEvent_t ev_hops[2] = {nullptr, nullptr};  // recorded around the hop kernel when set
  cudaEvent_t ev_place[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // around the saddle-disc placement, per kind, when set
  bool no_cancel = false;  // the complex has no boundary-cancelable critical point
  long long nadisc = 0, nddisc = 0;
  // the des discs run on `aux` beside the asc discs on the caller's stream;
  // ev[0]/ev[1] order the two streams; hcounts: 16 words of pinned host memory
  cudaStream_t aux = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  uint32_t *hcounts = nullptr;
};
cudaError_t fill_discs(DiscIO &io, cudaStream_t st);

// Piece merges (merge.cu).  MGraphHost is host-side storage of a device
// MGraph (a complex as a mutable graph with its cell table).
struct MGraphHost {
  uint32_t *buf = nullptr;
  uint32_t *tab = nullptr;     // its cell table (owned)
  uint32_t *status = nullptr;  // device status word for the fill (ST_INVARIANT: a cell outside the box)
  alignas(16) unsigned char raw[320];
};

}  // namespace dmsc

struct dmsc_msc;
namespace dmsc {
cudaError_t mgraph_alloc(MGraphHost &h, const dmsc_msc &src, uint32_t cap, unsigned long long pool, cudaStream_t st,
                         uint32_t slack = 4, uint32_t *tab = nullptr, const int *box = nullptr);
// Sets m.bbox to the box of its critical cells (synchronises st).
cudaError_t cell_box(dmsc_msc &m, cudaStream_t st);
void mgraph_free(MGraphHost &h, cudaStream_t st);
void mgraph_set_rects(MGraphHost &h, const int rect[4], const int ext[4]);
uint32_t mgraph_ncp(const MGraphHost &h);
unsigned long long mgraph_pool_used(const MGraphHost &h);
cudaError_t mgraph_to_csr(const MGraphHost &h, dmsc_msc &out, cudaStream_t st);
// One tree level: jobs are (a, b, c) graph indices -- merge up: out c = a + b;
// merge down: parent a into children b and c; ixn4: the shared 1-manifold (l,b,r,t).
cudaError_t merge_level(bool up, MGraphHost *hosts, int ngraphs, const int *jobs3, const int *ixn4, int njobs,
                        uint32_t *status, cudaStream_t st);
// Parallel merges of one tree level (merge_par.cu): up builds each parent
// from its children a, b; down pushes each parent into its children.  The
// shared 1-manifold is ixn (l, b, r, t).  grow scales the list pools; *stw
// is the OR of the device status words (ST_FALLBACK: rerun the level with
// merge_level; ST_SIMPLIFY_LIMIT: rerun with a larger grow).
struct MergeJob {
  dmsc_msc *a, *b, *parent;
  int ixn[4];
};
// seq_ms accumulates the host wall time of the one-thread steps.
cudaError_t merge_up_level_par(const std::vector<MergeJob> &jobs, unsigned long long grow, uint32_t *status,
                               uint32_t *stw, cudaStream_t st, double *seq_ms, long long round_window,
                               long long round_min_commits);
cudaError_t merge_down_level_par(const std::vector<MergeJob> &jobs, unsigned long long grow, uint32_t *status,
                                 uint32_t *stw, cudaStream_t st, double *seq_ms);
}  // namespace dmsc
