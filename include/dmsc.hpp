// dmsc.hpp -- header-only C++ mirror of the reference's GridDataset,
// GridMSComplex and GridDataManager (dmsc/include/grid_dataset.h:35-240,
// dmsc/include/grid_mscomplex.h:48-86, dmsc/src/grid_datamanager.cpp:596-747)
// over the C ABI of dmsc.h.  Link with libdmsc.so.
//
// Errors follow the reference: a failed call throws dmsc_cxx::logic_error (a
// std::logic_error) where the reference throws std::logic_error, i.e. for a
// violated invariant (DMSC_ERR_INVARIANT), and dmsc_cxx::runtime_error (a
// std::runtime_error) otherwise, as the reference's _CHECKCL_ERR_CODE
// (dmsc/src/grid_dataset.cpp:14-15).  The message is dmsc_last_error(), and
// code() gives the DMSC_ERR_* value.
//
// Ownership: every class owns its handle (destroyed by its destructor, moved
// but not copied).  Complexes must come from the same Context as the dataset
// that fills them.  `stream` is a cudaStream_t as void* (nullptr: the
// context's own stream).
#ifndef DMSC_HPP_
#define DMSC_HPP_

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "dmsc.h"

namespace dmsc_cxx {

class runtime_error : public std::runtime_error {
 public:
  runtime_error(int code, const std::string &msg) : std::runtime_error(msg), code_(code) {}
  int code() const noexcept { return code_; }

 private:
  int code_;
};

class logic_error : public std::logic_error {
 public:
  logic_error(int code, const std::string &msg) : std::logic_error(msg), code_(code) {}
  int code() const noexcept { return code_; }

 private:
  int code_;
};

// Throws for a DMSC_ERR_* status, as described above.
inline void check(int rc) {
  if (rc == DMSC_OK) return;
  const std::string msg = dmsc_last_error();
  if (rc == DMSC_ERR_INVARIANT) throw logic_error(rc, msg);
  throw runtime_error(rc, msg);
}

// rect_t of the reference: {left, bottom, right, top} in refined-grid cell
// coordinates (vertex (i, j) is cell (2i, 2j)).
using rect_t = std::array<int16_t, 4>;

// GridDataset::init_opencl() / stop_opencl() (dmsc/include/grid_dataset.h:236-238):
// one per process and device.
class Context {
 public:
  explicit Context(int device = 0) { check(dmsc_init(device, &c_)); }
  ~Context() {
    if (c_) dmsc_shutdown(c_);
  }
  Context(const Context &) = delete;
  Context &operator=(const Context &) = delete;
  Context(Context &&o) noexcept : c_(std::exchange(o.c_, nullptr)) {}
  Context &operator=(Context &&o) noexcept {
    if (this != &o) {
      if (c_) dmsc_shutdown(c_);
      c_ = std::exchange(o.c_, nullptr);
    }
    return *this;
  }
  dmsc_ctx *get() const noexcept { return c_; }
  // GridDataManager's ocl argument (-ocl): pipelines of this context use work_ocl
  void set_use_ocl(bool use_ocl) { check(dmsc_set_use_ocl(c_, use_ocl ? 1 : 0)); }

 private:
  dmsc_ctx *c_ = nullptr;
};

// MSComplex<cellid_t> (dmsc/include/discreteMorseDS.h:78-143) in flat host
// form, the layout of dmsc_msc_export: per critical point its (x, y) cell id,
// m_cp_fns value, pair_idx and flags; asc/des multisets and discs as CSR.
struct MSComplexData {
  rect_t rect{}, ext{};
  std::vector<int16_t> cellid;  // 2 per critical point
  std::vector<float> fn;
  std::vector<uint32_t> pair_idx;
  std::vector<uint8_t> flags;  // bit0 isCancelled, bit1 isOnStrangulationPath, bit2 isBoundryCancelable
  std::vector<uint32_t> asc_off, asc, des_off, des;
  std::vector<uint32_t> adisc_off, ddisc_off;
  std::vector<int16_t> adisc, ddisc;  // 2 per cell
};

// The complex behind handle m in host memory (dmsc_msc_export).
inline MSComplexData export_complex(dmsc_msc *m, void *stream = nullptr) {
  std::array<int64_t, 5> s{};
  check(dmsc_msc_sizes(m, s.data()));
  const size_t n = (size_t)s[0];
  MSComplexData d;
  d.cellid.resize(2 * n);
  d.fn.resize(n);
  d.pair_idx.resize(n);
  d.flags.resize(n);
  d.asc_off.resize(n + 1);
  d.des_off.resize(n + 1);
  d.asc.resize((size_t)s[1]);
  d.des.resize((size_t)s[2]);
  d.adisc_off.resize(n + 1);
  d.ddisc_off.resize(n + 1);
  d.adisc.resize(2 * (size_t)s[3]);
  d.ddisc.resize(2 * (size_t)s[4]);
  int16_t re[8];
  check(dmsc_msc_export(m, re, d.cellid.data(), d.fn.data(), d.pair_idx.data(), d.flags.data(), d.asc_off.data(),
                        d.asc.data(), d.des_off.data(), d.des.data(), d.adisc_off.data(), d.adisc.data(),
                        d.ddisc_off.data(), d.ddisc.data(), stream));
  for (int i = 0; i < 4; ++i) {
    d.rect[i] = re[i];
    d.ext[i] = re[4 + i];
  }
  return d;
}

// GridMSComplex (dmsc/include/grid_mscomplex.h:48-86).  Empty until a
// GridDataset writes it out.
class GridMSComplex {
 public:
  GridMSComplex() = default;
  explicit GridMSComplex(dmsc_msc *m) noexcept : m_(m) {}  // takes ownership
  ~GridMSComplex() { clear(); }
  GridMSComplex(const GridMSComplex &) = delete;
  GridMSComplex &operator=(const GridMSComplex &) = delete;
  GridMSComplex(GridMSComplex &&o) noexcept : m_(std::exchange(o.m_, nullptr)) {}
  GridMSComplex &operator=(GridMSComplex &&o) noexcept {
    if (this != &o) {
      clear();
      m_ = std::exchange(o.m_, nullptr);
    }
    return *this;
  }

  // GridMSComplex::clear() (dmsc/src/grid_mscomplex.cpp:324-329)
  void clear() noexcept {
    if (m_) dmsc_msc_destroy(m_);
    m_ = nullptr;
  }
  // GridMSComplex::simplify_un_simplify (dmsc/src/grid_mscomplex.cpp:528-535);
  // max_ops <= 0: the library's default operation budget
  void simplify_un_simplify(double tresh, int64_t max_ops = 0, void *stream = nullptr) {
    check(dmsc_msc_simplify_un_simplify(m_, tresh, max_ops, stream));
  }
  // GridMSComplex::write_discs (dmsc/src/grid_mscomplex.cpp:542-590)
  void write_discs(const std::string &prefix) const { check(dmsc_msc_write_discs(m_, prefix.c_str())); }
  // [0] critical points, [1] asc entries, [2] des entries, [3] asc_disc cells, [4] des_disc cells
  std::array<int64_t, 5> sizes() const {
    std::array<int64_t, 5> s{};
    check(dmsc_msc_sizes(m_, s.data()));
    return s;
  }
  // the whole complex in host memory
  MSComplexData data(void *stream = nullptr) const { return export_complex(m_, stream); }
  dmsc_msc *get() const noexcept { return m_; }
  dmsc_msc **slot() noexcept { return &m_; }  // for writeout_connectivity
  bool empty() const noexcept { return m_ == nullptr; }

 private:
  dmsc_msc *m_ = nullptr;
};

// GridDataset (dmsc/include/grid_dataset.h:35-240): one piece of a grid,
// rect inside ext.
class GridDataset {
 public:
  GridDataset(const Context &ctx, const rect_t &rect, const rect_t &ext) : rect_(rect), ext_(ext) {
    check(dmsc_dataset_create(ctx.get(), rect.data(), ext.data(), &d_));
  }
  ~GridDataset() {
    if (d_) dmsc_dataset_destroy(d_);
  }
  GridDataset(const GridDataset &) = delete;
  GridDataset &operator=(const GridDataset &) = delete;
  GridDataset(GridDataset &&o) noexcept : d_(std::exchange(o.d_, nullptr)), rect_(o.rect_), ext_(o.ext_) {}
  GridDataset &operator=(GridDataset &&o) noexcept {
    if (this != &o) {
      if (d_) dmsc_dataset_destroy(d_);
      d_ = std::exchange(o.d_, nullptr);
      rect_ = o.rect_;
      ext_ = o.ext_;
    }
    return *this;
  }

  // GridDataset::init(cell_fn_t *) (dmsc/src/grid_dataset.cpp:1461-1484): the
  // ext window's heights, x fastest, `pitch` floats per row (0: the window
  // width).  A host pointer is copied; a device pointer is borrowed until the
  // next init or the dataset's end.
  void init(const float *heights, int64_t pitch = 0, bool on_device = false, void *stream = nullptr) {
    if (pitch == 0) pitch = (ext_[2] - ext_[0]) / 2 + 1;
    check(dmsc_dataset_init(d_, heights, pitch, on_device ? 1 : 0, stream));
  }
  // GridDataset::work() (dmsc/src/grid_dataset.cpp:1734-1741)
  void work(void *stream = nullptr) { check(dmsc_dataset_work(d_, stream)); }
  // GridDataset::work_ocl() (dmsc/src/grid_dataset.cpp:353-399): the OpenCL
  // kernels' gradient (compareCells with vertices sorted descending)
  void work_ocl(void *stream = nullptr) { check(dmsc_dataset_work_ocl(d_, stream)); }
  // m_critical_cells.size()
  int64_t num_critical() const {
    int64_t n = 0;
    check(dmsc_dataset_num_critical(d_, &n));
    return n;
  }
  // GridDataset::writeout_connectivity(mscomplex_t *) (dmsc/src/grid_dataset.cpp:
  // 1858-1907): fills msc, reusing its device buffers when it already holds a complex
  void writeout_connectivity(GridMSComplex &msc, void *stream = nullptr) {
    check(dmsc_dataset_writeout_connectivity(d_, msc.slot(), stream));
  }
  GridMSComplex writeout_connectivity(void *stream = nullptr) {
    GridMSComplex m;
    writeout_connectivity(m, stream);
    return m;
  }
  // GridDataset::writeout_connectivity_ocl(mscomplex_t *) (dmsc/src/grid_dataset.cpp:1250-1283)
  GridMSComplex writeout_connectivity_ocl(void *stream = nullptr) {
    GridMSComplex m;
    check(dmsc_dataset_writeout_connectivity_ocl(d_, m.slot(), stream));
    return m;
  }
  // GridDataset::postMergeFillDiscs(mscomplex_t *) (dmsc/src/grid_dataset.cpp:1044-1231)
  void postMergeFillDiscs(GridMSComplex &msc, void *stream = nullptr) {
    check(dmsc_dataset_fill_discs(d_, msc.get(), stream));
  }
  // m_cell_flags, m_cell_pairs, m_cell_own (dmsc/include/grid_dataset.h:78-80) in
  // the reference layout: C order [x][y] over ext, pairs and owners as (x, y)
  // int16 pairs, (-1, -1) where unset.  A null vector is skipped.
  void export_cells(std::vector<int8_t> *flags, std::vector<int16_t> *pairs, std::vector<int16_t> *own,
                    void *stream = nullptr) const {
    const size_t cells = (size_t)(ext_[2] - ext_[0] + 1) * (size_t)(ext_[3] - ext_[1] + 1);
    if (flags) flags->resize(cells);
    if (pairs) pairs->resize(2 * cells);
    if (own) own->resize(2 * cells);
    check(dmsc_dataset_export_cells(d_, flags ? flags->data() : nullptr, pairs ? pairs->data() : nullptr,
                                    own ? own->data() : nullptr, stream));
  }
  // m_critical_cells (dmsc/src/grid_dataset.cpp:1822-1832): (x, y) pairs in collation order
  std::vector<int16_t> critical_cells(void *stream = nullptr) const {
    std::vector<int16_t> c(2 * (size_t)num_critical());
    check(dmsc_dataset_export_critical(d_, c.data(), stream));
    return c;
  }
  const rect_t &rect() const noexcept { return rect_; }
  const rect_t &ext() const noexcept { return ext_; }
  dmsc_dataset *get() const noexcept { return d_; }

 private:
  dmsc_dataset *d_ = nullptr;
  rect_t rect_, ext_;
};

// GridDataManager's pipeline (dmsc/src/grid_datamanager.cpp:596-747): the grid
// split `levels` times into pieces (split2d: alternating y and x instead of
// the reference's y only), a complex per piece, merged up to the root,
// simplify_un_simplify(tresh) there (tresh <= 0: skipped), merged down, and the
// manifold discs of every piece.
class GridDataManager {
 public:
  GridDataManager(const Context &ctx, const float *heights, int size_x, int size_y, int levels, double tresh,
                  bool split2d = false, int64_t pitch = 0, bool on_device = false, void *stream = nullptr) {
    check(dmsc_pipeline_run(ctx.get(), heights, pitch ? pitch : size_x, on_device ? 1 : 0, size_x, size_y, levels,
                            tresh, split2d ? 1 : 0, &p_, stream));
  }
  ~GridDataManager() {
    if (p_) dmsc_pipeline_destroy(p_);
  }
  GridDataManager(const GridDataManager &) = delete;
  GridDataManager &operator=(const GridDataManager &) = delete;
  GridDataManager(GridDataManager &&o) noexcept : p_(std::exchange(o.p_, nullptr)) {}
  GridDataManager &operator=(GridDataManager &&o) noexcept {
    if (this != &o) {
      if (p_) dmsc_pipeline_destroy(p_);
      p_ = std::exchange(o.p_, nullptr);
    }
    return *this;
  }

  int64_t num_pieces() const {
    int64_t n = 0;
    check(dmsc_pipeline_num_pieces(p_, &n));
    return n;
  }
  // node i of the piece tree (leaves first, the root last) after merge down,
  // in host memory (the complex itself stays owned by the pipeline)
  MSComplexData piece(int64_t i, void *stream = nullptr) const {
    dmsc_msc *m = nullptr;
    check(dmsc_pipeline_piece(p_, i, &m, nullptr));
    return export_complex(m, stream);
  }
  // collectSubdomainManifolds: write_discs of every piece in leaf order
  void write_discs(const std::string &prefix) const { check(dmsc_pipeline_write_discs(p_, prefix.c_str())); }
  dmsc_pipeline *get() const noexcept { return p_; }

 private:
  dmsc_pipeline *p_ = nullptr;
};

}  // namespace dmsc_cxx

#endif  // DMSC_HPP_
