// archive.cu -- a complex to and from a file: the out-of-core archives of
// the piece pipeline.
//
// The reference writes a piece's complex with boost::serialization
// (GridMSComplex::serialize, dmsc/src/grid_mscomplex.cpp:604-695) into the
// archive "dp_msgraph_<piece>" (write_msgraph_to_archive /
// read_msgraph_from_archive, dmsc/src/grid_datamanager.cpp:91-119).  Boost's
// binary archive layout is not reproducible without Boost, so the files here
// use this library's own layout (host byte order):
//
//   char     magic[8]       "DMSCMSC" + NUL
//   uint32   version        1
//   uint32   bits           1: asc discs present, 2: des discs present,
//                           4: may hold boundary-cancelable points
//   int16    rect[4], ext[4]
//   int32    bbox[4]        a box of cell coordinates holding every critical cell
//   int64    ncp, nasc, ndes, nadisc, nddisc
//   uint64   simplify counters[5]
//   uint32   cellid[ncp]    packed (x, y) cell ids
//   float    fn[ncp]
//   uint32   pair_idx[ncp]
//   uint8    flags[ncp]
//   uint32   asc_off[ncp+1], asc[nasc], des_off[ncp+1], des[ndes]
//   uint32   asc_disc_off[ncp+1], asc_disc[nadisc]   (if bit 1)
//   uint32   des_disc_off[ncp+1], des_disc[nddisc]   (if bit 2)
//
// The arrays are the complex's device arrays as they are, so a loaded
// complex is the saved one.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "dmsc.h"
#include "dmsc_internal.h"
#include "grid_types.h"

namespace {

constexpr char kMagic[8] = {'D', 'M', 'S', 'C', 'M', 'S', 'C', 0};
constexpr uint32_t kVersion = 1;

struct Header {
  char magic[8];
  uint32_t version, bits;
  int16_t rect[4], ext[4];
  int32_t bbox[4];
  int64_t ncp, nasc, ndes, nadisc, nddisc;
  uint64_t simp[5];
};

int fail(int code, const std::string &m) { return dmsc::set_last_error(code, m.c_str()); }

struct File {
  FILE *f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

template <typename T>
cudaError_t to_host(std::vector<T> &h, const T *d, size_t n, cudaStream_t st) {
  h.resize(n);
  if (!n) return cudaSuccess;
  return cudaMemcpyAsync(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost, st);
}

}  // namespace

extern "C" {

int dmsc_msc_save(dmsc_msc *m, const char *path) {
  if (!m || !path) return fail(DMSC_ERR_BAD_ARG, "null argument");
  cudaError_t e = cudaSetDevice(m->ctx->device);
  cudaStream_t st = m->ctx->stream;
  const size_t n = (size_t)m->ncp;
  const bool ad = m->adoff.p != nullptr, dd = m->ddoff.p != nullptr;
  std::vector<uint32_t> cellid, pair_idx, aoff, asc, doff, des, adoff, adisc, ddoff, ddisc;
  std::vector<float> fn;
  std::vector<uint8_t> flags;
  if (e == cudaSuccess) e = to_host(cellid, m->cellid.p, n, st);
  if (e == cudaSuccess) e = to_host(fn, m->fn.p, n, st);
  if (e == cudaSuccess) e = to_host(pair_idx, m->pair_idx.p, n, st);
  if (e == cudaSuccess) e = to_host(flags, m->flags.p, n, st);
  if (e == cudaSuccess) e = to_host(aoff, m->aoff.p, m->aoff.p ? n + 1 : 0, st);
  if (e == cudaSuccess) e = to_host(asc, m->asc.p, (size_t)m->nasc, st);
  if (e == cudaSuccess) e = to_host(doff, m->doff.p, m->doff.p ? n + 1 : 0, st);
  if (e == cudaSuccess) e = to_host(des, m->des.p, (size_t)m->ndes, st);
  if (e == cudaSuccess && ad) e = to_host(adoff, m->adoff.p, n + 1, st);
  if (e == cudaSuccess && ad) e = to_host(adisc, m->adisc.p, (size_t)m->nadisc, st);
  if (e == cudaSuccess && dd) e = to_host(ddoff, m->ddoff.p, n + 1, st);
  if (e == cudaSuccess && dd) e = to_host(ddisc, m->ddisc.p, (size_t)m->nddisc, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(DMSC_ERR_CUDA, std::string("save: ") + cudaGetErrorString(e));
  aoff.resize(n + 1, 0);  // a complex without points has no offset arrays
  doff.resize(n + 1, 0);
  Header h{};
  std::memcpy(h.magic, kMagic, 8);
  h.version = kVersion;
  h.bits = (ad ? 1u : 0u) | (dd ? 2u : 0u) | (m->any_bcancel ? 4u : 0u);
  std::memcpy(h.rect, m->rect, 8);
  std::memcpy(h.ext, m->ext, 8);
  for (int i = 0; i < 4; ++i) h.bbox[i] = m->bbox[i];
  h.ncp = m->ncp; h.nasc = m->nasc; h.ndes = m->ndes;
  h.nadisc = ad ? m->nadisc : 0; h.nddisc = dd ? m->nddisc : 0;
  for (int i = 0; i < 5; ++i) h.simp[i] = m->simp_stats[i];
  File f;
  f.f = std::fopen(path, "wb");
  if (!f.f) return fail(DMSC_ERR_BAD_ARG, std::string("cannot write ") + path);
  bool ok = std::fwrite(&h, sizeof h, 1, f.f) == 1;
  auto put = [&](const void *p, size_t bytes) { if (ok && bytes) ok = std::fwrite(p, 1, bytes, f.f) == bytes; };
  put(cellid.data(), 4 * n); put(fn.data(), 4 * n); put(pair_idx.data(), 4 * n); put(flags.data(), n);
  put(aoff.data(), 4 * (n + 1)); put(asc.data(), 4 * asc.size());
  put(doff.data(), 4 * (n + 1)); put(des.data(), 4 * des.size());
  if (ad) { put(adoff.data(), 4 * (n + 1)); put(adisc.data(), 4 * adisc.size()); }
  if (dd) { put(ddoff.data(), 4 * (n + 1)); put(ddisc.data(), 4 * ddisc.size()); }
  if (ok) ok = std::fflush(f.f) == 0;
  if (!ok) return fail(DMSC_ERR_BAD_ARG, std::string("short write to ") + path);
  return DMSC_OK;
}

int dmsc_msc_load(dmsc_ctx *ctx, const char *path, dmsc_msc **out) {
  if (!ctx || !path || !out) return fail(DMSC_ERR_BAD_ARG, "null argument");
  File f;
  f.f = std::fopen(path, "rb");
  if (!f.f) return fail(DMSC_ERR_BAD_ARG, std::string("cannot read ") + path);
  Header h{};
  if (std::fread(&h, sizeof h, 1, f.f) != 1 || std::memcmp(h.magic, kMagic, 8) != 0 || h.version != kVersion)
    return fail(DMSC_ERR_INPUT, std::string(path) + " is not a complex archive of this library");
  if (h.ncp < 0 || h.nasc < 0 || h.ndes < 0 || h.nadisc < 0 || h.nddisc < 0 || h.ncp > (1ll << 32))
    return fail(DMSC_ERR_INPUT, std::string(path) + ": bad sizes");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return fail(DMSC_ERR_CUDA, cudaGetErrorString(e));
  cudaStream_t st = ctx->stream;
  const size_t n = (size_t)h.ncp;
  const bool ad = h.bits & 1u, dd = h.bits & 2u;
  dmsc_msc *m = new dmsc_msc;
  m->ctx = ctx;
  std::memcpy(m->rect, h.rect, 8);
  std::memcpy(m->ext, h.ext, 8);
  for (int i = 0; i < 4; ++i) m->bbox[i] = h.bbox[i];
  m->ncp = h.ncp; m->nasc = h.nasc; m->ndes = h.ndes;
  m->nadisc = h.nadisc; m->nddisc = h.nddisc;
  m->any_bcancel = (h.bits & 4u) != 0;
  for (int i = 0; i < 5; ++i) m->simp_stats[i] = h.simp[i];
  std::vector<char> buf;
  bool ok = true;
  // one array: read into the staging buffer, copy to a fresh device buffer
  auto get = [&](auto &dev, size_t count) {
    using T = typename std::remove_reference<decltype(*dev.p)>::type;
    if (!ok) return;
    const size_t bytes = sizeof(T) * count;
    buf.resize(bytes ? bytes : 1);
    if (bytes && std::fread(buf.data(), 1, bytes, f.f) != bytes) { ok = false; return; }
    if (dev.ensure(count ? count : 1, st) != cudaSuccess) { ok = false; e = cudaErrorMemoryAllocation; return; }
    if (bytes && cudaMemcpyAsync(dev.p, buf.data(), bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) ok = false;
    if (ok && cudaStreamSynchronize(st) != cudaSuccess) ok = false;  // buf is reused for the next array
  };
  get(m->cellid, n); get(m->fn, n); get(m->pair_idx, n); get(m->flags, n);
  get(m->aoff, n + 1); get(m->asc, (size_t)h.nasc);
  get(m->doff, n + 1); get(m->des, (size_t)h.ndes);
  if (ad) { get(m->adoff, n + 1); get(m->adisc, (size_t)h.nadisc); }
  if (dd) { get(m->ddoff, n + 1); get(m->ddisc, (size_t)h.nddisc); }
  if (!ok) {
    delete m;
    if (e == cudaErrorMemoryAllocation) return fail(DMSC_ERR_OOM, std::string("load: device allocation for ") + path);
    return fail(DMSC_ERR_INPUT, std::string(path) + ": truncated archive or copy failure");
  }
  *out = m;
  return DMSC_OK;
}

}  // extern "C"
