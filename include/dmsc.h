/* dmsc.h -- C ABI of the GB300 grid Morse-Smale complex library (libdmsc.so).
 *
 * The reference (nithins/mscomplex) has no plugin or FFI API: its hot path is
 * the C++ class GridDataset (dmsc/include/grid_dataset.h) driven by
 * GridDataManager (dmsc/src/grid_datamanager.cpp), with an OpenCL backend
 * selected by a bool.  Every entry point below replaces one of those calls;
 * the citation on each names the reference interface it stands in for.
 *
 * Conventions
 *  - Every function returns DMSC_OK (0) or a DMSC_ERR_* code; the message of
 *    the last error of the calling thread is dmsc_last_error().
 *  - Cell ids are (x, y) pairs of int16 in the reference's refined-grid
 *    coordinates: vertex (i, j) is cell (2i, 2j), cell dimension is
 *    (x & 1) + (y & 1).  A rect is {left, bottom, right, top} in cell coords.
 *  - `stream` is a cudaStream_t (NULL = the context's own stream, which is
 *    created non-blocking: it does not order with the legacy default
 *    stream, so a caller that produced device inputs on another stream
 *    passes that stream or synchronises first).  Export functions write
 *    HOST buffers and return after the copy completes.
 *  - Inputs containing NaN are outside the supported domain (the reference's
 *    vertex comparison is not a strict weak order on NaN) and are rejected
 *    with DMSC_ERR_INPUT.
 */
#ifndef DMSC_H_
#define DMSC_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dmsc_ctx dmsc_ctx;
typedef struct dmsc_dataset dmsc_dataset;
typedef struct dmsc_msc dmsc_msc;

enum {
  DMSC_OK = 0,
  DMSC_ERR_BAD_ARG = 1,        /* invalid argument (null pointer, bad rect) */
  DMSC_ERR_OOM = 2,            /* device allocation failed */
  DMSC_ERR_CUDA = 3,           /* CUDA runtime error */
  DMSC_ERR_INT16_OVERFLOW = 4, /* grid exceeds the int16 cell-id range (16384 vertices per side) */
  DMSC_ERR_DEVICE_TIMEOUT = 5, /* a bounded device loop ran out of iterations */
  DMSC_ERR_INVARIANT = 6,      /* a reference std::logic_error condition */
  DMSC_ERR_INPUT = 7,          /* input outside the supported domain (NaN heights) */
  DMSC_ERR_STATE = 8,          /* call out of order (e.g. export before work) */
  DMSC_ERR_PARTIAL = 9         /* a batch ran but some of its grids failed (dmsc_batch_grid_status) */
};

/* Message of the calling thread's last error ("" if none). */
const char *dmsc_last_error(void);

/* GridDataset::init_opencl() -- process-wide device setup
 * (dmsc/include/grid_dataset.h:236, dmsc/src/grid_dataset.cpp:186-226).
 * Scratch buffers come from the device's default stream-ordered memory
 * pool; dmsc_init sets that pool to keep freed memory cached (release
 * threshold = max) and dmsc_shutdown trims it. */
int dmsc_init(int device, dmsc_ctx **out);
/* GridDataset::stop_opencl() (dmsc/include/grid_dataset.h:238). */
int dmsc_shutdown(dmsc_ctx *ctx);

/* GridDataset::GridDataset(const rect_t &r, const rect_t &e)
 * (dmsc/src/grid_dataset.cpp:1429-1441). */
int dmsc_dataset_create(dmsc_ctx *ctx, const int16_t rect[4], const int16_t ext[4], dmsc_dataset **out);
/* GridDataset::clear() / ~GridDataset() (dmsc/src/grid_dataset.cpp:1456-1509). */
int dmsc_dataset_destroy(dmsc_dataset *ds);
/* GridDataset::init(cell_fn_t *) (dmsc/src/grid_dataset.cpp:1461-1484): the
 * heights of the ext window, x fastest, `pitch` elements between rows.
 * on_device = 0: host pointer (copied); 1: device pointer (borrowed, must stay
 * valid until the dataset is destroyed or re-initialised). */
int dmsc_dataset_init(dmsc_dataset *ds, const float *heights, int64_t pitch, int on_device, void *stream);
/* GridDataset::work() (dmsc/src/grid_dataset.cpp:1734-1741): gradient,
 * critical-cell collation and owner extrema of the reference's CPU path. */
int dmsc_dataset_work(dmsc_dataset *ds, void *stream);
/* GridDataset::work_ocl() (dmsc/src/grid_dataset.cpp:353-399): the gradient
 * of the reference's OpenCL kernels, whose compareCells sorts a cell's
 * vertices descending (dmsc/resources/assigngradient.cl:40-87; the CPU path
 * sorts them ascending), then collation and owner extrema as the OpenCL
 * kernels compute them (collate_critpts.cl, bfs_watershed.cl). */
int dmsc_dataset_work_ocl(dmsc_dataset *ds, void *stream);
/* m_critical_cells.size() (dmsc/include/grid_dataset.h:81). */
int dmsc_dataset_num_critical(dmsc_dataset *ds, int64_t *n);
/* m_cell_flags, m_cell_pairs, m_cell_own (dmsc/include/grid_dataset.h:78-80)
 * in the reference layout: C order [x][y] over ext (y fastest); flags int8,
 * pairs and own as (x, y) int16 pairs, (-1,-1) where unset.  Any output
 * pointer may be NULL. */
int dmsc_dataset_export_cells(dmsc_dataset *ds, int8_t *flags, int16_t *pairs, int16_t *own, void *stream);
/* m_critical_cells (dmsc/src/grid_dataset.cpp:1822-1832): (x, y) int16 pairs in
 * collation (row-major) order. */
int dmsc_dataset_export_critical(dmsc_dataset *ds, int16_t *cellids, void *stream);
/* GridDataset::writeout_connectivity(mscomplex_t *) (dmsc/src/grid_dataset.cpp:
 * 1858-1907).  *out == NULL: a new
 * complex is returned in *out.  *out != NULL: that complex (of the same
 * context) is overwritten in place, reusing its device buffers, as the
 * reference fills the mscomplex_t it is given. */
int dmsc_dataset_writeout_connectivity(dmsc_dataset *ds, dmsc_msc **out, void *stream);
/* GridDataset::writeout_connectivity_ocl(mscomplex_t *)
 * (dmsc/src/grid_dataset.cpp:1250-1283, with collect_saddle_conn_ocl :907-1022):
 * the complex from the saddle incidences of the dataset's last work_ocl.
 * These read the same owners as writeout_connectivity, so both calls give
 * the same complex for the same dataset. */
int dmsc_dataset_writeout_connectivity_ocl(dmsc_dataset *ds, dmsc_msc **msc, void *stream);

/* GridMSComplex::clear() (dmsc/src/grid_mscomplex.cpp:324-329). */
int dmsc_msc_destroy(dmsc_msc *msc);
/* GridMSComplex::serialize (dmsc/src/grid_mscomplex.cpp:604-695) as used by
 * write_msgraph_to_archive / read_msgraph_from_archive
 * (dmsc/src/grid_datamanager.cpp:91-119): the whole complex (points, values,
 * pairs, flags, lists, discs) to a file and back.  The file layout is this
 * library's own (documented in mscomplex_gb300/csrc/archive.cu): the
 * reference's Boost binary archive cannot be reproduced without Boost.  A
 * loaded complex is identical to the saved one. */
int dmsc_msc_save(dmsc_msc *msc, const char *path);
int dmsc_msc_load(dmsc_ctx *ctx, const char *path, dmsc_msc **out);
/* Sizes of a complex: [0] critical points, [1] asc entries, [2] des entries,
 * [3] asc_disc cells, [4] des_disc cells. */
int dmsc_msc_sizes(dmsc_msc *msc, int64_t sizes[5]);
/* MSComplex<cellid_t> (dmsc/include/discreteMorseDS.h:78-143) in flat form:
 * rect_ext = m_rect then m_ext_rect; per critical point its cell id, m_cp_fns
 * value, pair_idx, flags (bit0 isCancelled, bit1 isOnStrangulationPath,
 * bit2 isBoundryCancelable); the asc/des multisets as CSR (offsets have
 * ncp+1 entries, each segment ascending with multiplicity); asc_disc/des_disc
 * as CSR of (x, y) cell ids.  Any output pointer may be NULL. */
int dmsc_msc_export(dmsc_msc *msc, int16_t rect_ext[8], int16_t *cellid, float *fn, uint32_t *pair_idx,
                    uint8_t *flags, uint32_t *asc_off, uint32_t *asc, uint32_t *des_off, uint32_t *des,
                    uint32_t *adisc_off, int16_t *adisc, uint32_t *ddisc_off, int16_t *ddisc, void *stream);
/* dmsc_msc_export without waiting: the copies are queued on `stream`, behind
 * what is already queued there, and the host buffers (pinned, so that the
 * copies run asynchronously) hold the complex once the stream reaches that
 * point.  Until then the complex must not be changed or destroyed, and the
 * buffers must stay allocated.  No reference counterpart: it lets a caller
 * overlap one grid's device-to-host copies with the next grid's work. */
int dmsc_msc_export_async(dmsc_msc *msc, int16_t rect_ext[8], int16_t *cellid, float *fn, uint32_t *pair_idx,
                          uint8_t *flags, uint32_t *asc_off, uint32_t *asc, uint32_t *des_off, uint32_t *des,
                          uint32_t *adisc_off, int16_t *adisc, uint32_t *ddisc_off, int16_t *ddisc, void *stream);

/* GridMSComplex::simplify_un_simplify(tresh) (dmsc/src/grid_mscomplex.cpp:
 * 384-535): persistence cancellation in the reference's exact pop order,
 * then every cancellation undone, leaving isBoundryCancelable / pair_idx as
 * the record of the simplified complex.  The reference heap's order among
 * equal persistences is replayed exactly, so the pass is sequential: it stops
 * with DMSC_ERR_DEVICE_TIMEOUT (complex unchanged) after max_ops heap pops
 * and cross-connections (max_ops <= 0: 2,000,000,000). */
int dmsc_msc_simplify_un_simplify(dmsc_msc *msc, double tresh, int64_t max_ops, void *stream);
/* Counters of the last simplification: [0] heap pushes, [1] pops,
 * [2] cancellations, [3] operations, [4] device status. */
int dmsc_msc_simplify_stats(dmsc_msc *msc, uint64_t stats[5]);

/* GridDataset::postMergeFillDiscs(mscomplex_t *) (dmsc/src/grid_dataset.cpp:
 * 1044-1231): fills the asc/des manifold discs of the complex's surviving
 * critical points from the dataset's gradient and owners (dataset_work must
 * have run on the piece the complex belongs to).  The dataset's owner labels
 * of cancelled extrema are redirected as in the reference, on a copy: the
 * dataset itself is not modified. */
int dmsc_dataset_fill_discs(dmsc_dataset *ds, dmsc_msc *msc, void *stream);
/* GridMSComplex::write_discs(prefix) (dmsc/src/grid_mscomplex.cpp:542-590):
 * for every critical point that is not boundary-cancelable, appends its
 * non-empty asc / des disc (x, y int16 pairs) to the file prefix + "asc_" /
 * "des_" + "(x,y)" (binary, append mode, as the reference). */
int dmsc_msc_write_discs(dmsc_msc *msc, const char *prefix);

/* ---- the whole piece pipeline ----
 * GridDataManager (dmsc/src/grid_datamanager.cpp): createPieces_quadtree
 * (:40-89), computeSubdomainMsgraphs (:493-528), mergePiecesUp (:258-306),
 * simplify_un_simplify at the root (:651-652), mergePiecesDown +
 * finalMergeDownPiecesInRange (:308-395) and collectSubdomainManifolds
 * (:454-490) on one GPU.  The grid (size_x x size_y vertices, row pitch in
 * floats) is split `levels` times into 2^levels pieces with a one-vertex
 * halo; split2d = 0 splits along y as the reference (split_axes = 1,
 * :50-51), split2d = 1 alternates y and x.  tresh <= 0 skips simplification.
 * On success every piece holds its merged-down complex with manifold discs.
 * The pipeline owns the pieces' datasets and complexes. */
typedef struct dmsc_pipeline dmsc_pipeline;
int dmsc_pipeline_run(dmsc_ctx *ctx, const float *heights, int64_t pitch, int on_device, int size_x, int size_y,
                      int levels, double tresh, int split2d, dmsc_pipeline **out, void *stream);
int dmsc_pipeline_destroy(dmsc_pipeline *p);
int dmsc_pipeline_num_pieces(dmsc_pipeline *p, int64_t *n);
/* Node i of the piece tree: i < num_pieces is a leaf (order of
 * createPieces_quadtree), num_pieces <= i < 2 num_pieces - 1 is the merge of
 * nodes 2(i - num_pieces) and 2(i - num_pieces) + 1 (the last is the root),
 * in its state after merge_down.  Returns its complex and, for a leaf, its
 * dataset (NULL for inner nodes); either output pointer may be NULL.  Both
 * stay owned by the pipeline. */
int dmsc_pipeline_piece(dmsc_pipeline *p, int64_t i, dmsc_msc **msc, dmsc_dataset **ds);
/* write_discs of every piece in leaf order, as collectSubdomainManifolds. */
int dmsc_pipeline_write_discs(dmsc_pipeline *p, const char *prefix);
/* Host wall time (ms) of the last run's stages: pieces, merge up, simplify,
 * merge down, discs. */
int dmsc_pipeline_stage_times(dmsc_pipeline *p, double ms[5]);
/* Of merge up and merge down, the host wall time (ms) spent in the boundary
 * steps: merge up's cancellations (ordered-parallel rounds) and merge down's
 * uncancellations (one thread per merge). */
int dmsc_pipeline_merge_times(dmsc_pipeline *p, double ms[2]);
/* Tree levels whose largest merge involves at least min_cps critical points
 * (default 2048) run the parallel merges; smaller levels run every merge on
 * one thread (one block per merge).  Both give the same complexes. */
int dmsc_set_merge_parallel_min(dmsc_ctx *ctx, int64_t min_cps);
/* merge_up's cancellations along each shared boundary (the loop of
 * dmsc/src/grid_mscomplex.cpp:124-153) on the parallel merges: 0 (the
 * default) runs the loop on one thread per merge; window > 0 runs it in
 * ordered-parallel rounds over the first `window` pending boundary cells,
 * and after 8 rounds in a row that each commit fewer than `min_commits` cells
 * (default 4) one thread finishes the rest in order.  Every setting gives the
 * same complexes; on white noise the one-thread loop is the faster. */
int dmsc_set_merge_rounds(dmsc_ctx *ctx, int64_t window, int64_t min_commits);
/* GridDataManager's `ocl` argument (the -ocl flag, dmsc/src/main.cpp:527-530;
 * used at dmsc/src/grid_datamanager.cpp:123-132, 221-222, 433-434): pipelines
 * run with this context compute their pieces with work_ocl (1) or work (0,
 * the default). */
int dmsc_set_use_ocl(dmsc_ctx *ctx, int use_ocl);
/* GridDataManager's compute_out_of_core argument (--out-of-core,
 * dmsc/src/grid_datamanager.cpp:91-119, 134-139, 258-395, 397-422): pipelines
 * run with this context keep their pieces' complexes in archive files under
 * `dir` (NULL or "" turns it off, the default) instead of device memory: a
 * leaf's complex goes to its archive once computed and its dataset is freed;
 * each merge-up level reads its inputs back and archives its new nodes (all
 * but the root); each merge-down level reads its nodes and archives them
 * again; the discs stage recomputes each leaf's gradient and reads its
 * complex back.  A pipeline with levels == 0 stays in memory, as the
 * reference's does.  After the run the complexes stay archived and are read
 * back by dmsc_pipeline_piece and dmsc_pipeline_write_discs on first use;
 * leaf datasets are not kept (dmsc_pipeline_piece returns NULL for them).
 * The archive files are removed by dmsc_pipeline_destroy. */
int dmsc_set_out_of_core(dmsc_ctx *ctx, const char *dir);

/* ---- batches of whole grids ----
 * No counterpart in the reference, which builds one GridDataset at a time
 * (GridDataManager::computeMsGraph, dmsc/src/grid_datamanager.cpp:121-140):
 * ngrids whole grids (rect == ext) of sizes[2g] x sizes[2g+1] vertices, their
 * heights packed back to back (x fastest, grid after grid; host or device
 * pointer), each taken through work + writeout_connectivity +
 * simplify_un_simplify(tresh[g]) (skipped where tresh[g] == 0) in shared
 * launches.  Every grid's complex is identical to the one-grid path.
 * *out == NULL: a new batch; otherwise that batch is rerun in place (buffers
 * reused).  max_ops bounds each grid's simplification (<= 0: 2,000,000,000).
 * A grid whose simplification exhausts max_ops (or breaks an invariant) fails
 * alone: the run returns DMSC_ERR_PARTIAL, the batch is still *out, the
 * other grids export as usual, and dmsc_batch_export of a failed grid returns
 * its own error (dmsc_batch_export_all refuses a batch with failed grids). */
typedef struct dmsc_batch dmsc_batch;
int dmsc_batch_run(dmsc_ctx *ctx, int ngrids, const int32_t *sizes, const float *heights, int on_device,
                   const double *tresh, int64_t max_ops, dmsc_batch **out, void *stream);
int dmsc_batch_destroy(dmsc_batch *b);
int dmsc_batch_num_grids(dmsc_batch *b, int64_t *n);
/* [0] critical points, [1] asc entries, [2] des entries of grid i */
int dmsc_batch_sizes(dmsc_batch *b, int64_t i, int64_t sizes[3]);
/* grid i's own status (DMSC_OK or its error) and message (may be NULL) */
int dmsc_batch_grid_status(dmsc_batch *b, int64_t i, int *status, char *error, int error_len);
/* simplification counters of grid i, as dmsc_msc_simplify_stats */
int dmsc_batch_simplify_stats(dmsc_batch *b, int64_t i, uint64_t stats[5]);
/* grid i's complex in the layout of dmsc_msc_export (no discs) */
int dmsc_batch_export(dmsc_batch *b, int64_t i, int16_t rect_ext[8], int16_t *cellid, float *fn, uint32_t *pair_idx,
                      uint8_t *flags, uint32_t *asc_off, uint32_t *asc, uint32_t *des_off, uint32_t *des, void *stream);
/* [0] critical points, [1] asc entries, [2] des entries of the whole batch */
int dmsc_batch_totals(dmsc_batch *b, int64_t totals[3]);
/* every grid at once: per-grid bases (ngrids + 1 each) into the shared arrays;
 * asc_off / des_off are batch-wide (subtract asc_base[g] / des_base[g]); list
 * values and pair_idx are local to each grid.  Any pointer may be NULL. */
int dmsc_batch_export_all(dmsc_batch *b, uint32_t *cp_base, uint32_t *asc_base, uint32_t *des_base, uint32_t *cellid,
                          float *fn, uint32_t *pair_idx, uint8_t *flags, uint32_t *asc_off, uint32_t *asc,
                          uint32_t *des_off, uint32_t *des, void *stream);
/* Device times (ms) of the batch's last run: [0] the gradient tile kernel's
 * launches, [1] the owner-label tile kernel's launches. */
int dmsc_batch_tile_times(dmsc_batch *b, float ms[2]);
/* No counterpart in the reference: the launch autotuner of the batched path.
 * Grids are grouped into size classes by their larger side: below 128, 256,
 * 512, 1024, 2048 vertices, and from 2048 on.  For every class present in
 * the sample (ngrids grids packed as for dmsc_batch_run), each launch
 * configuration of the two persistent tile kernels -- 256 or 512 threads per
 * block, 1, 2 or 3 resident blocks per SM -- is timed over `repeats` batch
 * runs of the class's grids (after one untimed run), and the configuration
 * with the smallest median becomes the class's in the context.  From then on
 * dmsc_batch_run launches the tile kernels once per size class present, each
 * with its class's configuration.  Results never depend on the
 * configuration.  table (may be NULL) receives per class 4 int32: threads,
 * blocks per SM, the chosen configuration's median time and the default
 * configuration's (512 threads, 3 blocks per SM), in microseconds; zeros for
 * classes absent from the sample.  The tile shape (64 x 64 vertices) is not a
 * parameter: it fixes the border table's layout and the 12-bit in-tile cell
 * indices of the pointer jumping. */
int dmsc_batch_autotune(dmsc_ctx *ctx, int ngrids, const int32_t *sizes, const float *heights, int on_device,
                        int repeats, int32_t table[24]);
/* Sets one size class's configuration by hand (as the autotuner would);
 * later batches launch per size class. */
int dmsc_batch_set_launch(dmsc_ctx *ctx, int size_class, int threads, int blocks_per_sm);
/* Back to one launch over all grids with the default configuration. */
int dmsc_batch_autotune_reset(dmsc_ctx *ctx);

/* ---- request server (continuous batching) ----
 * No counterpart in the reference.  Requests (one whole grid each, heights
 * copied at submit) are admitted in arrival order by their device footprint
 * against arena_bytes and run as batches (dmsc_batch_run) by `lanes` worker
 * threads, each with its own stream, so one batch is admitted and copied
 * while another computes.  With two or more lanes, lanes / 2 of them take
 * the requests whose exact simplification is expected to be long (tresh > 0
 * and more than 1% equal neighbour pairs) and the others the rest.  A
 * request's result equals its grid's complex computed alone.  max_ops bounds
 * each grid's simplification (<= 0: the default of
 * dmsc_msc_simplify_un_simplify). */
typedef struct dmsc_server dmsc_server;
int dmsc_server_create(dmsc_ctx *ctx, int64_t arena_bytes, int lanes, int max_batch, int64_t max_ops, dmsc_server **out);
int dmsc_server_submit(dmsc_server *s, const float *heights, int nx, int ny, double tresh, int64_t *id);
/* waits up to timeout_ms (< 0: without limit); *done = 1 once the request
 * has completed, *status (may be NULL) is then its DMSC_* result */
int dmsc_server_wait(dmsc_server *s, int64_t id, int timeout_ms, int *done, int *status);
/* a completed request: sizes as dmsc_batch_sizes, times (ms since the server
 * started) of submit, batch start and completion; returns its status */
int dmsc_server_result(dmsc_server *s, int64_t id, int64_t sizes[3], double times_ms[3], char *error, int error_len);
/* a completed request's complex in the layout of dmsc_msc_export (no discs) */
int dmsc_server_export(dmsc_server *s, int64_t id, int16_t *cellid, float *fn, uint32_t *pair_idx, uint8_t *flags,
                       uint32_t *asc_off, uint32_t *asc, uint32_t *des_off, uint32_t *des);
/* forgets a completed request */
int dmsc_server_release(dmsc_server *s, int64_t id);
/* [0] batches run, [1] grids completed, [2] queued, [3] arena bytes in use */
int dmsc_server_stats(dmsc_server *s, int64_t stats[4]);
/* drains the queue, stops the workers */
int dmsc_server_destroy(dmsc_server *s);

/* PrefixScan::PreScanBuffer(out, in, n, queue) (dmsc/include/prefix_scan.h:105-109,
 * dmsc/src/prefix_scan.cpp:457-464): exclusive prefix sum of n uint32 values
 * in device memory, out[i] = in[0] + ... + in[i-1] (wrapping modulo 2^32).
 * d_total (device pointer, may be NULL) receives the sum of all n values.
 * Scratch for block partial sums comes from the stream-ordered allocator.
 * d_out may equal d_in. */
int dmsc_prefix_scan(dmsc_ctx *ctx, uint32_t *d_out, const uint32_t *d_in, int64_t n, uint32_t *d_total,
                     void *stream);
/* No counterpart in the reference.  The same exclusive scan as
 * dmsc_prefix_scan, for callers that cannot let a library allocate device
 * memory: a host runtime that has reserved the GPU's memory for its own pool,
 * or a latency-bound serving loop where cudaMalloc (it synchronises the
 * device) and cudaFree must not appear.  It calls no allocator; its scratch
 * is a fixed array of about 128 KiB compiled into libdmsc.so, held by every
 * GPU that loads the library until the process exits.
 *  - n may be at most 67,108,864 (2^26); larger n fails with
 *    DMSC_ERR_BAD_ARG and a message naming the limit.
 *  - The first call on a device looks up the scratch array's device address
 *    (cudaGetSymbolAddress) with that device current; make that first call
 *    before any stream capture.  After a device reset the next call looks it
 *    up again (the device's context has changed); make that call before any
 *    capture as well.
 *  - All calls share the one scratch array: calls that overlap on the GPU
 *    (concurrent streams, or threads) race and corrupt each other's result.
 *  - The call only enqueues work on `stream`; the result is ready once that
 *    stream reaches it. */
int dmsc_prefix_scan_noalloc(dmsc_ctx *ctx, uint32_t *d_out, const uint32_t *d_in, int64_t n, uint32_t *d_total,
                             void *stream);
/* BitonicSortProgram::bitonicSort(queue, dstKey, dstVal, srcKey, srcVal,
 * batch, arrayLength, dir) (dmsc/include/bitonic_sort.h:30-39): sorts `batch`
 * consecutive arrays of `array_length` (key, value) uint32 pairs each, in
 * device memory, ascending (dir = 1) or descending (dir = 0) by key.  Unlike
 * the bitonic network this sort is stable and takes any array length.  The
 * destination may alias the source. */
int dmsc_sort_pairs(dmsc_ctx *ctx, uint32_t *d_dst_key, uint32_t *d_dst_val, const uint32_t *d_src_key,
                    const uint32_t *d_src_val, uint32_t batch, uint32_t array_length, uint32_t dir, void *stream);

/* Tracing: the reference's compile-time _LOG_TIMINGS stage timers
 * (dmsc/src/grid_dataset.cpp:19-34, 357-390).  When enabled, CUDA events are
 * recorded on the launching stream around every stage of work and
 * writeout_connectivity. */
int dmsc_set_timing(dmsc_ctx *ctx, int enable);
/* Stage times in ms of the dataset's last work + writeout_connectivity:
 * [0] gradient, [1] collation scan, [2] border resolve, [3] owner labels and
 * arcs, [4] connectivity CSR; and of its last fill_discs: [5] the hop kernel,
 * [6] the whole pass, [7] / [8] the kernels that write the saddle discs of
 * the asc / des kind (the chain cells' placement, the level-0 items and the
 * discs of saddles with many chains).  Writes min(n, 9) floats. */
int dmsc_dataset_stage_times(dmsc_dataset *ds, float *ms, int n);
/* The device's stream-ordered memory pool, which holds the library's device
 * buffers: bytes [0] reserved now, [1] reserved at most, [2] in use now,
 * [3] in use at most. */
int dmsc_pool_stats(dmsc_ctx *ctx, int64_t stats[4]);
/* Kernels launched by this library so far in this process. */
int dmsc_kernel_launches(uint64_t *count);

#ifdef __cplusplus
}
#endif

#endif /* DMSC_H_ */
