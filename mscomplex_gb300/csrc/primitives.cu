// primitives.cu -- device-wide exclusive scan, stable LSD radix sort and the
// kernels that assemble the Morse-Smale complex in CSR form.
//
// The reference's scan is the OpenCL PrefixScan (dmsc/src/prefix_scan.cpp:
// 340-465, kernels absent: dmsc/resources/scan_kernel.cl is empty) and its
// sort slot is an unused bitonic sort (dmsc/src/bitonic_sort.cpp).  Both are
// written here from scratch: the scan is a single pass with decoupled
// look-back out of place (bounded waits on earlier tiles) and reduce-then-scan
// in place, the radix sort is a stable 8-bit LSD sort (histogram, scan,
// match_any-ranked scatter).
#include "dmsc_common.cuh"
#include "dmsc_internal.h"

namespace dmsc {

unsigned long long g_kernel_launches = 0;

constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_CHUNK = SCAN_THREADS * SCAN_ITEMS;

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ __forceinline__ uint32_t block_exscan(uint32_t v, uint32_t &excl) {
  __shared__ uint32_t wsum[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t s = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, s, o);
    if (lane >= o) s += t;
  }
  if (lane == 31) wsum[warp] = s;
  __syncthreads();
  if (warp == 0) {
    uint32_t ws = lane < nw ? wsum[lane] : 0u;
    uint32_t ss = ws;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, ss, o);
      if (lane >= o) ss += t;
    }
    if (lane < nw) wsum[lane] = ss - ws;
    if (lane == 31) wsum[31] = ss;  // total (nw <= 32)
  }
  __syncthreads();
  excl = wsum[warp] + s - v;
  uint32_t total = wsum[31];
  __syncthreads();
  return total;
}

// A thread's SCAN_ITEMS consecutive items: one or two vector loads when the
// array is aligned for them and the items are all in range, else scalars.
template <typename T>
__device__ __forceinline__ void load_items(const T *__restrict__ in, long long base, long long n, bool vec,
                                           uint32_t v[SCAN_ITEMS]) {
  static_assert(SCAN_ITEMS == 8, "two 16-byte (u32) or one 8-byte (u8) vector per thread");
  if (vec && base + SCAN_ITEMS <= n) {
    if constexpr (sizeof(T) == 4) {
      const uint4 a = reinterpret_cast<const uint4 *>(in + base)[0], b = reinterpret_cast<const uint4 *>(in + base)[1];
      v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    } else {
      const uint2 a = *reinterpret_cast<const uint2 *>(in + base);
#pragma unroll
      for (int k = 0; k < 4; ++k) { v[k] = (a.x >> (8 * k)) & 0xffu; v[4 + k] = (a.y >> (8 * k)) & 0xffu; }
    }
    return;
  }
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) v[k] = (base + k < n) ? (uint32_t)in[base + k] : 0u;
}
template <typename T>
__host__ __forceinline__ bool items_aligned(const T *p) {
  return ((uintptr_t)p % (sizeof(T) == 4 ? 16 : 8)) == 0;
}

template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const T *__restrict__ in, long long n, bool vec,
                                                              uint32_t *partial) {
  long long base = (long long)blockIdx.x * SCAN_CHUNK + (long long)threadIdx.x * SCAN_ITEMS;
  uint32_t v[SCAN_ITEMS];
  load_items(in, base, n, vec, v);
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) s += v[k];
  uint32_t ex;
  uint32_t tot = block_exscan(s, ex);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

// (in and out may be the same array: a thread reads its items before it
// writes them, and no thread reads another's)
template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_down(const T *in, long long n, bool vec_in,
                                                            const uint32_t *__restrict__ block_off, uint32_t *out,
                                                            bool vec_out, uint32_t *total) {
  long long base = (long long)blockIdx.x * SCAN_CHUNK + (long long)threadIdx.x * SCAN_ITEMS;
  uint32_t v[SCAN_ITEMS];
  load_items(in, base, n, vec_in, v);
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) s += v[k];
  uint32_t ex;
  uint32_t tot = block_exscan(s, ex);
  uint32_t run = (block_off ? block_off[blockIdx.x] : 0u) + ex;
  uint32_t o[SCAN_ITEMS];
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) { o[k] = run; run += v[k]; }
  if (vec_out && base + SCAN_ITEMS <= n) {
    reinterpret_cast<uint4 *>(out + base)[0] = make_uint4(o[0], o[1], o[2], o[3]);
    reinterpret_cast<uint4 *>(out + base)[1] = make_uint4(o[4], o[5], o[6], o[7]);
  } else {
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
      if (base + k < n) out[base + k] = o[k];
  }
  if (total && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *total = (block_off ? block_off[blockIdx.x] : 0u) + tot;
}

// Single-pass scan (decoupled look-back): a block takes the next tile from
// an atomic counter, publishes its tile's sum, then warp 0 walks back over
// the earlier tiles' published words -- adding sums until it meets a tile
// that has published its inclusive prefix -- and publishes its own.  Tiles
// are taken in counter order, so a block only waits for blocks that already
// run.  A word is (flag << 32 | value) in one 64-bit store: 0 not yet, 1 the
// tile's sum, 2 its inclusive prefix.  The wait is bounded: past
// LOOKBACK_LIMIT polls the block sums the earlier tiles' inputs itself (the
// same prefix, slower), which is why the input must not be the output.
constexpr unsigned long long LOOKBACK_LIMIT = 1ull << 22;
__device__ __forceinline__ unsigned long long ld_word(const unsigned long long *p) {
  return *reinterpret_cast<const volatile unsigned long long *>(p);
}
__device__ __forceinline__ void st_word(unsigned long long *p, unsigned long long v) {
  *reinterpret_cast<volatile unsigned long long *>(p) = v;
}
template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_onepass(const T *__restrict__ in, long long n, bool vec_in,
                                                               uint32_t *__restrict__ out, bool vec_out,
                                                               unsigned long long *__restrict__ word,
                                                               uint32_t *__restrict__ counter, long long nb,
                                                               uint32_t *__restrict__ total) {
  __shared__ uint32_t tile_s, excl_s;
  if (threadIdx.x == 0) tile_s = atomicAdd(counter, 1u);
  __syncthreads();
  const long long tile = tile_s;
  if (tile >= nb) return;  // (block-uniform)
  const long long base = tile * SCAN_CHUNK + (long long)threadIdx.x * SCAN_ITEMS;
  uint32_t v[SCAN_ITEMS];
  load_items(in, base, n, vec_in, v);
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) s += v[k];
  uint32_t ex;
  const uint32_t tot = block_exscan(s, ex);
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    uint32_t excl = 0;
    bool fallback = false;
    if (tile == 0) {
      if (lane == 0) st_word(word, (2ull << 32) | tot);
    } else {
      if (lane == 0) st_word(word + tile, (1ull << 32) | tot);
      long long j = tile - 1;
      unsigned long long polls = 0;
      for (;;) {
        const long long idx = j - lane;  // lane 0: the nearest earlier tile
        const unsigned long long w = idx >= 0 ? ld_word(word + idx) : (2ull << 32);
        const uint32_t flag = (uint32_t)(w >> 32);
        const unsigned pm = __ballot_sync(0xffffffffu, flag == 2u), zm = __ballot_sync(0xffffffffu, flag == 0u);
        const int fp = pm ? __ffs(pm) - 1 : 32;  // the nearest tile with its prefix
        const unsigned need = fp >= 31 ? 0xffffffffu : ((2u << fp) - 1u);
        if (zm & need) {  // a tile before it has published nothing yet
          if (++polls > LOOKBACK_LIMIT) { fallback = true; break; }
          continue;
        }
        uint32_t c = lane <= fp ? (uint32_t)w : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        excl += c;
        if (fp < 32) break;
        j -= 32;
      }
      fallback = __any_sync(0xffffffffu, fallback);
      if (!fallback && lane == 0) st_word(word + tile, (2ull << 32) | (excl + tot));
    }
    if (lane == 0) excl_s = fallback ? 0xFFFFFFFFu : excl;
  }
  __syncthreads();
  uint32_t prefix = excl_s;
  if (prefix == 0xFFFFFFFFu && tile > 0) {  // bounded wait ran out: the earlier tiles' sum from their inputs
    __shared__ uint32_t red[32];
    const long long upto = tile * SCAN_CHUNK;
    uint32_t acc = 0;
    for (long long i = threadIdx.x; i < upto; i += blockDim.x) acc += (uint32_t)in[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
      uint32_t r = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0u;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
      if (threadIdx.x == 0) { excl_s = r; st_word(word + tile, (2ull << 32) | (r + tot)); }
    }
    __syncthreads();
    prefix = excl_s;
  }
  uint32_t run = prefix + ex;
  uint32_t o[SCAN_ITEMS];
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) { o[k] = run; run += v[k]; }
  if (vec_out && base + SCAN_ITEMS <= n) {
    reinterpret_cast<uint4 *>(out + base)[0] = make_uint4(o[0], o[1], o[2], o[3]);
    reinterpret_cast<uint4 *>(out + base)[1] = make_uint4(o[4], o[5], o[6], o[7]);
  } else {
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
      if (base + k < n) out[base + k] = o[k];
  }
  if (total && tile == nb - 1 && threadIdx.x == 0) *total = prefix + tot;
}

template <typename T>
cudaError_t scan_exclusive_t(const T *in, long long n, uint32_t *out, uint32_t *total, cudaStream_t st) {
  if (n <= 0) {
    if (total) return cudaMemsetAsync(total, 0, sizeof(uint32_t), st);
    return cudaSuccess;
  }
  long long nb = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
  if (nb == 1) {
    k_scan_down<T><<<1, SCAN_THREADS, 0, st>>>(in, n, items_aligned(in), nullptr, out, items_aligned(out), total);
    DMSC_LAUNCHED(1);
    return cudaGetLastError();
  }
  if ((const void *)in != (const void *)out) {  // one pass (the look-back's fallback reads the input)
    unsigned long long *word = nullptr;
    cudaError_t e = cudaMallocAsync((void **)&word, sizeof(unsigned long long) * (nb + 1), st);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(word, 0, sizeof(unsigned long long) * (nb + 1), st);
    if (e == cudaSuccess) {
      k_scan_onepass<T><<<(unsigned)nb, SCAN_THREADS, 0, st>>>(in, n, items_aligned(in), out, items_aligned(out), word,
                                                                reinterpret_cast<uint32_t *>(word + nb), nb, total);
      DMSC_LAUNCHED(1);
      e = cudaGetLastError();
    }
    cudaFreeAsync(word, st);
    return e;
  }
  uint32_t *part = nullptr, *poff = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&part, sizeof(uint32_t) * nb * 2, st);
  if (e != cudaSuccess) return e;
  poff = part + nb;
  k_scan_reduce<T><<<(unsigned)nb, SCAN_THREADS, 0, st>>>(in, n, items_aligned(in), part);
  DMSC_LAUNCHED(1);
  e = scan_exclusive_t<uint32_t>(part, nb, poff, nullptr, st);
  if (e == cudaSuccess) {
    k_scan_down<T><<<(unsigned)nb, SCAN_THREADS, 0, st>>>(in, n, items_aligned(in), poff, out, items_aligned(out), total);
    DMSC_LAUNCHED(1);
    e = cudaGetLastError();
  }
  cudaFreeAsync(part, st);
  return e;
}

cudaError_t scan_exclusive_u8(const uint8_t *in, long long n, uint32_t *out, uint32_t *total, cudaStream_t st) {
  return scan_exclusive_t<uint8_t>(in, n, out, total, st);
}
__global__ void k_copy_u32(long long n, const uint32_t *__restrict__ src, uint32_t *__restrict__ dst) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

cudaError_t copy_u32(uint32_t *dst, const uint32_t *src, long long n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  long long b = (n + 255) / 256;
  if (b > 152 * 8) b = 152 * 8;
  k_copy_u32<<<(unsigned)b, 256, 0, st>>>(n, src, dst);
  DMSC_LAUNCHED(1);
  return cudaGetLastError();
}

struct Words8 {
  const uint32_t *src[8];
};
__global__ void k_read_words(Words8 w, int n, uint32_t *host) {
  const int i = threadIdx.x;
  if (i < n) host[i] = *w.src[i];
}

cudaError_t read_words(uint32_t *host, const uint32_t *const *src, int n, cudaStream_t st) {
  if (n < 1 || n > 8 || !host) return cudaErrorInvalidValue;
  Words8 w{};
  for (int i = 0; i < n; ++i) w.src[i] = src[i];
  k_read_words<<<1, 32, 0, st>>>(w, n, host);
  DMSC_LAUNCHED(1);
  return cudaGetLastError();
}

cudaError_t scan_exclusive_u32(const uint32_t *in, long long n, uint32_t *out, uint32_t *total, cudaStream_t st) {
  return scan_exclusive_t<uint32_t>(in, n, out, total, st);
}

// Same scan with caller-provided scratch instead of the stream-ordered
// allocator: `scratch` must hold scan_scratch_words(n) uint32 words.
long long scan_scratch_words(long long n) {
  long long words = 0;
  for (long long nb = (n + SCAN_CHUNK - 1) / SCAN_CHUNK; nb > 1; nb = (nb + SCAN_CHUNK - 1) / SCAN_CHUNK)
    words += 2 * nb;
  return words;
}

cudaError_t scan_exclusive_u32_scratch(const uint32_t *in, long long n, uint32_t *out, uint32_t *total,
                                       uint32_t *scratch, cudaStream_t st) {
  if (n <= 0) {
    if (total) return cudaMemsetAsync(total, 0, sizeof(uint32_t), st);
    return cudaSuccess;
  }
  long long nb = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
  if (nb == 1) {
    k_scan_down<uint32_t><<<1, SCAN_THREADS, 0, st>>>(in, n, items_aligned(in), nullptr, out, items_aligned(out), total);
    DMSC_LAUNCHED(1);
    return cudaGetLastError();
  }
  uint32_t *part = scratch, *poff = scratch + nb;
  k_scan_reduce<uint32_t><<<(unsigned)nb, SCAN_THREADS, 0, st>>>(in, n, items_aligned(in), part);
  DMSC_LAUNCHED(1);
  cudaError_t e = scan_exclusive_u32_scratch(part, nb, poff, nullptr, scratch + 2 * nb, st);
  if (e != cudaSuccess) return e;
  k_scan_down<uint32_t><<<(unsigned)nb, SCAN_THREADS, 0, st>>>(in, n, items_aligned(in), poff, out,
                                                                items_aligned(out), total);
  DMSC_LAUNCHED(1);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// stable LSD radix sort of (key, value) pairs on key bits [0, nbits)
// ---------------------------------------------------------------------------
constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ROUNDS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;  // each warp owns a contiguous run of 256 items

__global__ void __launch_bounds__(RS_THREADS) k_radix_hist(const uint32_t *__restrict__ keys, long long n, int shift,
                                                           uint32_t *__restrict__ hist, long long nb) {
  __shared__ uint32_t cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  long long base = (long long)blockIdx.x * RS_TILE;
  for (int k = threadIdx.x; k < RS_TILE; k += RS_THREADS) {
    long long i = base + k;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(long long)threadIdx.x * nb + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(RS_THREADS) k_radix_scatter(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin,
                                                              long long n, int shift, const uint32_t *__restrict__ hoff,
                                                              long long nb, uint32_t *__restrict__ kout,
                                                              uint32_t *__restrict__ vout) {
  __shared__ uint32_t wcnt[RS_WARPS][256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = threadIdx.x; k < RS_WARPS * 256; k += RS_THREADS) (&wcnt[0][0])[k] = 0;
  __syncthreads();
  long long base = (long long)blockIdx.x * RS_TILE + warp * (32 * RS_ROUNDS);
  uint32_t key[RS_ROUNDS], val[RS_ROUNDS], rank[RS_ROUNDS];
  const uint32_t lt_mask = (1u << lane) - 1u;
#pragma unroll
  for (int r = 0; r < RS_ROUNDS; ++r) {
    long long i = base + r * 32 + lane;
    bool valid = i < n;
    key[r] = valid ? kin[i] : 0u;
    val[r] = valid ? vin[i] : 0u;
    uint32_t d = valid ? ((key[r] >> shift) & 255u) : 256u;
    uint32_t peers = __match_any_sync(0xffffffffu, d);
    uint32_t before = valid ? wcnt[warp][d] : 0u;
    rank[r] = before + __popc(peers & lt_mask);
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) wcnt[warp][d] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  {
    uint32_t d = threadIdx.x, run = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) { uint32_t t = wcnt[w][d]; wcnt[w][d] = run; run += t; }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < RS_ROUNDS; ++r) {
    long long i = base + r * 32 + lane;
    if (i < n) {
      uint32_t d = (key[r] >> shift) & 255u;
      uint32_t pos = hoff[(long long)d * nb + blockIdx.x] + wcnt[warp][d] + rank[r];
      kout[pos] = key[r];
      vout[pos] = val[r];
    }
  }
}

// Sorts in place (keys/vals) using caller scratch of the same size.
cudaError_t radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *ktmp, uint32_t *vtmp, long long n, int nbits,
                             cudaStream_t st) {
  if (n <= 1 || nbits <= 0) return cudaSuccess;
  long long nb = (n + RS_TILE - 1) / RS_TILE;
  uint32_t *hist = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&hist, sizeof(uint32_t) * 256 * nb * 2, st);
  if (e != cudaSuccess) return e;
  uint32_t *hoff = hist + 256 * nb;
  uint32_t *ka = keys, *va = vals, *kb = ktmp, *vb = vtmp;
  for (int shift = 0; shift < nbits; shift += 8) {
    k_radix_hist<<<(unsigned)nb, RS_THREADS, 0, st>>>(ka, n, shift, hist, nb);
    DMSC_LAUNCHED(1);
    e = scan_exclusive_u32(hist, 256 * nb, hoff, nullptr, st);
    if (e != cudaSuccess) break;
    k_radix_scatter<<<(unsigned)nb, RS_THREADS, 0, st>>>(ka, va, n, shift, hoff, nb, kb, vb);
    DMSC_LAUNCHED(1);
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (e == cudaSuccess && ka != keys) {
    e = copy_u32(keys, ka, n, st);
    if (e == cudaSuccess) e = copy_u32(vals, va, n, st);
  }
  cudaFreeAsync(hist, st);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

// Batched key/value sort (the BitonicSortProgram slot): arrays [b*len, (b+1)*len)
// sorted independently, ascending or descending, stably.  Implemented as one
// stable LSD sort on the (possibly inverted) key followed by a stable sort on
// the array index.
__global__ void k_sort_prepare(long long n, uint32_t len, uint32_t dir, const uint32_t *__restrict__ ks,
                               const uint32_t *__restrict__ vs, uint32_t *__restrict__ k, uint32_t *__restrict__ v,
                               uint32_t *__restrict__ seg) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    uint32_t key = ks[i];
    k[i] = dir ? key : ~key;
    v[i] = vs[i];
    seg[i] = (uint32_t)(i / len);
  }
}
__global__ void k_sort_finish(long long n, uint32_t dir, const uint32_t *__restrict__ k, uint32_t *__restrict__ kout) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    kout[i] = dir ? k[i] : ~k[i];
}
// (seg, key) pairs: after sorting by key, a stable sort by segment keeps the
// key order inside each segment.  Values travel through an index permutation.
__global__ void k_gather_u32(long long n, const uint32_t *__restrict__ idx, const uint32_t *__restrict__ src,
                             uint32_t *__restrict__ dst) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = src[idx[i]];
}
__global__ void k_iota(long long n, uint32_t *__restrict__ a) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] = (uint32_t)i;
}

static unsigned grid_for(long long n, int threads);

cudaError_t sort_pairs_batched(uint32_t *dk, uint32_t *dv, const uint32_t *sk, const uint32_t *sv, uint32_t batch,
                               uint32_t len, uint32_t dir, cudaStream_t st) {
  long long n = (long long)batch * len;
  if (n == 0) return cudaSuccess;
  uint32_t *buf = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&buf, sizeof(uint32_t) * n * 7, st);
  if (e != cudaSuccess) return e;
  uint32_t *k = buf, *v = buf + n, *seg = buf + 2 * n, *perm = buf + 3 * n, *t1 = buf + 4 * n, *t2 = buf + 5 * n,
           *t3 = buf + 6 * n;
  unsigned gb = grid_for(n, 256);
  k_sort_prepare<<<gb, 256, 0, st>>>(n, len, dir, sk, sv, k, v, seg);
  DMSC_LAUNCHED(1);
  k_iota<<<gb, 256, 0, st>>>(n, perm);
  DMSC_LAUNCHED(1);
  // 1) stable by key, carrying the original index
  e = radix_sort_pairs(k, perm, t1, t2, n, 32, st);
  if (e == cudaSuccess && batch > 1) {
    // 2) stable by segment of the original index: seg of perm[i]
    k_gather_u32<<<gb, 256, 0, st>>>(n, perm, seg, t3);
    DMSC_LAUNCHED(1);
    int sbits = 1;
    while ((1ll << sbits) < (long long)batch) ++sbits;
    // sort (segment, position-in-key-order) carrying the key-sorted position
    k_iota<<<gb, 256, 0, st>>>(n, t1);
    DMSC_LAUNCHED(1);
    e = radix_sort_pairs(t3, t1, seg, t2, n, sbits, st);
    if (e == cudaSuccess) {
      k_gather_u32<<<gb, 256, 0, st>>>(n, t1, k, t2);  // keys in final order
      DMSC_LAUNCHED(1);
      k_gather_u32<<<gb, 256, 0, st>>>(n, t1, perm, t3);  // original indices in final order
      DMSC_LAUNCHED(1);
      e = copy_u32(k, t2, n, st);
      if (e == cudaSuccess) e = copy_u32(perm, t3, n, st);
    }
  }
  if (e == cudaSuccess) {
    k_gather_u32<<<gb, 256, 0, st>>>(n, perm, v, t2);  // values (v holds the source values)
    DMSC_LAUNCHED(1);
    k_sort_finish<<<gb, 256, 0, st>>>(n, dir, k, dk);
    DMSC_LAUNCHED(1);
    e = copy_u32(dv, t2, n, st);
  }
  cudaFreeAsync(buf, st);
  return e;
}

// ---------------------------------------------------------------------------
// complex assembly (writeout_connectivity, dmsc/src/grid_dataset.cpp:1858-1907)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int cell_dim(uint32_t packed) {
  return (int)(packed & 1u) + (int)((packed >> 16) & 1u);
}

// Saddle segments come straight from the 2+2 staged labels; every staged
// (extremum label, saddle) arc also becomes a sort item for the extremum side.
__global__ void k_fill_saddles(long long ncp, const uint32_t *__restrict__ cellid, const uint32_t *__restrict__ des2,
                               const uint32_t *__restrict__ asc2, const uint32_t *__restrict__ aoff,
                               const uint32_t *__restrict__ doff, uint32_t *__restrict__ asc, uint32_t *__restrict__ des,
                               uint32_t *__restrict__ kmin, uint32_t *__restrict__ kmax, uint32_t *__restrict__ vidx) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < ncp; k += (long long)gridDim.x * blockDim.x) {
    bool sad = cell_dim(cellid[k]) == 1;
    uint32_t d0 = sad ? des2[2 * k] : LABEL_NONE, d1 = sad ? des2[2 * k + 1] : LABEL_NONE;
    uint32_t a0 = sad ? asc2[2 * k] : LABEL_NONE, a1 = sad ? asc2[2 * k + 1] : LABEL_NONE;
    if (sad) {
      uint32_t p = doff[k], pe = doff[k + 1];
      if (d0 != LABEL_NONE && p < pe) des[p++] = d0;
      if (d1 != LABEL_NONE && p < pe) des[p++] = d1;
      p = aoff[k]; pe = aoff[k + 1];
      if (a0 != LABEL_NONE && p < pe) asc[p++] = a0;
      if (a1 != LABEL_NONE && p < pe) asc[p++] = a1;
    }
    uint32_t none = (uint32_t)ncp;
    kmin[2 * k] = d0 == LABEL_NONE ? none : d0;
    kmin[2 * k + 1] = d1 == LABEL_NONE ? none : d1;
    kmax[2 * k] = a0 == LABEL_NONE ? none : a0;
    kmax[2 * k + 1] = a1 == LABEL_NONE ? none : a1;
    vidx[2 * k] = (uint32_t)k;
    vidx[2 * k + 1] = (uint32_t)k;
  }
}

__global__ void k_run_starts(long long n, long long ncp, const uint32_t *__restrict__ keys, uint32_t *__restrict__ start) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    uint32_t k = keys[p];
    if (k < (uint32_t)ncp && (p == 0 || keys[p - 1] != k)) start[k] = (uint32_t)p;
  }
}
__global__ void k_scatter_runs(long long n, long long ncp, const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals,
                               const uint32_t *__restrict__ start, const uint32_t *__restrict__ off,
                               uint32_t *__restrict__ out, long long out_cap, uint32_t *__restrict__ status) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    uint32_t k = keys[p];
    if (k >= (uint32_t)ncp) continue;
    uint32_t r = (uint32_t)p - start[k];
    long long pos = (long long)off[k] + r;
    if (r < off[k + 1] - off[k] && pos < out_cap) out[pos] = vals[p];
    else atomicOr(status, ST_INVARIANT);
  }
}

static unsigned grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b > 152 * 32) b = 152 * 32;
  return (unsigned)(b < 1 ? 1 : b);
}

// ---- extremum side by atomic scatter + per-segment sort ----
// Every staged (extremum, saddle) arc is placed into its extremum's CSR
// segment at an atomically claimed slot; each segment is then sorted by
// saddle index, which is the ascending iteration order of the reference's
// multiset (equal saddle indices are indistinguishable, so the result does
// not depend on the claim order).  Segments of up to SEG_THREAD items are
// sorted by one thread, up to SEG_BLOCK by one block in shared memory; a
// longer one sets ST_CAPACITY and the caller falls back to the radix path.
// Segments of up to SEG_WARP items are sorted by one warp, taken from a queue
// with an atomic counter, so that a few long segments do not hold the rest.
constexpr uint32_t SEG_THREAD = 32, SEG_WARP = 256, SEG_BLOCK = 8192;

__global__ void k_ext_scatter(long long ncp, const uint32_t *__restrict__ cellid, const uint32_t *__restrict__ des2,
                              const uint32_t *__restrict__ asc2, const uint32_t *__restrict__ aoff,
                              const uint32_t *__restrict__ doff, uint32_t *__restrict__ asc, uint32_t *__restrict__ des,
                              uint32_t *__restrict__ afill, uint32_t *__restrict__ dfill, uint32_t *__restrict__ status) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < ncp; k += (long long)gridDim.x * blockDim.x) {
    if (cell_dim(cellid[k]) != 1) continue;
    for (int q = 0; q < 2; ++q) {
      const uint32_t x = des2[2 * k + q];  // a minimum: the saddle joins its asc list
      if (x != LABEL_NONE) {
        if (x >= (uint32_t)ncp) { atomicOr(status, ST_INVARIANT); continue; }
        const uint32_t r = atomicAdd(afill + x, 1u);
        if (r < aoff[x + 1] - aoff[x]) asc[aoff[x] + r] = (uint32_t)k;
        else atomicOr(status, ST_INVARIANT);
      }
      const uint32_t y = asc2[2 * k + q];  // a maximum: the saddle joins its des list
      if (y != LABEL_NONE) {
        if (y >= (uint32_t)ncp) { atomicOr(status, ST_INVARIANT); continue; }
        const uint32_t r = atomicAdd(dfill + y, 1u);
        if (r < doff[y + 1] - doff[y]) des[doff[y] + r] = (uint32_t)k;
        else atomicOr(status, ST_INVARIANT);
      }
    }
  }
}

// the saddle's own lists straight from its 2+2 staged labels
__global__ void k_saddle_lists(long long ncp, const uint32_t *__restrict__ cellid, const uint32_t *__restrict__ des2,
                               const uint32_t *__restrict__ asc2, const uint32_t *__restrict__ aoff,
                               const uint32_t *__restrict__ doff, uint32_t *__restrict__ asc, uint32_t *__restrict__ des) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < ncp; k += (long long)gridDim.x * blockDim.x) {
    if (cell_dim(cellid[k]) != 1) continue;
    uint32_t p = doff[k], pe = doff[k + 1];
    for (int q = 0; q < 2; ++q)
      if (des2[2 * k + q] != LABEL_NONE && p < pe) des[p++] = des2[2 * k + q];
    p = aoff[k]; pe = aoff[k + 1];
    for (int q = 0; q < 2; ++q)
      if (asc2[2 * k + q] != LABEL_NONE && p < pe) asc[p++] = asc2[2 * k + q];
  }
}

// short extremum segments: insertion sort by one thread; longer ones queued,
// up to SEG_WARP items in midq, longer in longq
__global__ void k_seg_sort(long long ncp, const uint32_t *__restrict__ cellid, const uint32_t *__restrict__ aoff,
                           const uint32_t *__restrict__ doff, uint32_t *__restrict__ asc, uint32_t *__restrict__ des,
                           uint32_t *__restrict__ midq, uint32_t *__restrict__ nmid, uint32_t *__restrict__ longq,
                           uint32_t *__restrict__ nlong, uint32_t *__restrict__ status) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < ncp; k += (long long)gridDim.x * blockDim.x) {
    const int dim = cell_dim(cellid[k]);
    if (dim == 1) continue;
    uint32_t *seg = dim == 0 ? asc + aoff[k] : des + doff[k];
    const uint32_t n = dim == 0 ? aoff[k + 1] - aoff[k] : doff[k + 1] - doff[k];
    if (n <= 1) continue;
    if (n > SEG_THREAD) {
      if (n > SEG_BLOCK) { atomicOr(status, ST_CAPACITY); continue; }
      if (n <= SEG_WARP) midq[atomicAdd(nmid, 1u)] = (uint32_t)k;
      else longq[atomicAdd(nlong, 1u)] = (uint32_t)k;
      continue;
    }
    uint32_t v[SEG_THREAD];
    for (uint32_t i = 0; i < n; ++i) v[i] = seg[i];
    for (uint32_t i = 1; i < n; ++i) {
      const uint32_t x = v[i];
      uint32_t j = i;
      while (j > 0 && v[j - 1] > x) { v[j] = v[j - 1]; --j; }
      v[j] = x;
    }
    for (uint32_t i = 0; i < n; ++i) seg[i] = v[i];
  }
}

// queued segments of up to SEG_WARP items: one warp each, taken in turn from
// the queue; each item's place is the count of items before it (value, then
// position, so equal saddle indices keep distinct places)
constexpr int SEG_WARP_THREADS = 256;
__global__ void __launch_bounds__(SEG_WARP_THREADS) k_seg_sort_warp(const uint32_t *__restrict__ cellid,
                                                                    const uint32_t *__restrict__ aoff,
                                                                    const uint32_t *__restrict__ doff,
                                                                    uint32_t *__restrict__ asc, uint32_t *__restrict__ des,
                                                                    const uint32_t *__restrict__ midq,
                                                                    const uint32_t *__restrict__ nmid,
                                                                    uint32_t *__restrict__ taken) {
  __shared__ uint32_t sh[SEG_WARP_THREADS / 32][SEG_WARP];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t *buf = sh[wid];
  const uint32_t nq = *nmid;
  for (;;) {
    uint32_t q = 0;
    if (lane == 0) q = atomicAdd(taken, 1u);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= nq) break;
    const uint32_t k = midq[q];
    const int dim = cell_dim(cellid[k]);
    uint32_t *seg = dim == 0 ? asc + aoff[k] : des + doff[k];
    const uint32_t n = dim == 0 ? aoff[k + 1] - aoff[k] : doff[k + 1] - doff[k];
    if (n > SEG_WARP) continue;  // queued by size: cannot happen
    for (uint32_t i = lane; i < n; i += 32) buf[i] = seg[i];
    __syncwarp();
    for (uint32_t i = lane; i < n; i += 32) {
      const uint32_t v = buf[i];
      uint32_t r = 0;
      for (uint32_t j = 0; j < n; ++j) {
        const uint32_t u = buf[j];
        r += (u < v) || (u == v && j < i);
      }
      seg[r] = v;
    }
    __syncwarp();
  }
}

// queued segments: one block each, bitonic sort in shared memory
__global__ void __launch_bounds__(512) k_seg_sort_block(const uint32_t *__restrict__ cellid, const uint32_t *__restrict__ aoff,
                                                        const uint32_t *__restrict__ doff, uint32_t *__restrict__ asc,
                                                        uint32_t *__restrict__ des, const uint32_t *__restrict__ longq,
                                                        const uint32_t *__restrict__ nlong) {
  __shared__ uint32_t sh[SEG_BLOCK];
  const uint32_t nq = *nlong;
  for (uint32_t q = blockIdx.x; q < nq; q += gridDim.x) {
    const uint32_t k = longq[q];
    const int dim = cell_dim(cellid[k]);
    uint32_t *seg = dim == 0 ? asc + aoff[k] : des + doff[k];
    const uint32_t n = dim == 0 ? aoff[k + 1] - aoff[k] : doff[k + 1] - doff[k];
    if (n <= 1024) {  // rank sort: each value's place is the count of values before it
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) sh[i] = seg[i];
      __syncthreads();
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint32_t v = sh[i];
        uint32_t r = 0;
        for (uint32_t j = 0; j < n; ++j) {
          const uint32_t u = sh[j];
          r += (u < v) || (u == v && j < i);
        }
        seg[r] = v;
      }
      __syncthreads();
      continue;
    }
    uint32_t p2 = 1;
    while (p2 < n) p2 <<= 1;
    for (uint32_t i = threadIdx.x; i < p2; i += blockDim.x) sh[i] = i < n ? seg[i] : 0xFFFFFFFFu;
    __syncthreads();
    for (uint32_t size = 2; size <= p2; size <<= 1)
      for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
        for (uint32_t i = threadIdx.x; i < p2; i += blockDim.x) {
          const uint32_t j = i ^ stride;
          if (j > i) {
            const bool up = (i & size) == 0;
            const uint32_t a = sh[i], b = sh[j];
            if ((a > b) == up) { sh[i] = b; sh[j] = a; }
          }
        }
        __syncthreads();
      }
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) seg[i] = sh[i];
    __syncthreads();
  }
}

cudaError_t build_csr(long long ncp, const uint32_t *cellid, const uint32_t *des2, const uint32_t *asc2,
                      const uint32_t *aoff, const uint32_t *doff, uint32_t *asc, uint32_t *des, long long out_cap,
                      uint32_t *status, cudaStream_t st) {
  if (ncp <= 0) return cudaSuccess;
  uint32_t *buf = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&buf, sizeof(uint32_t) * (4 * ncp + 8), st);
  if (e != cudaSuccess) return e;
  // afill dfill (2 ncp) | nlong nmid taken (3) | longq midq (2 ncp)
  uint32_t *afill = buf, *dfill = buf + ncp, *nlong = buf + 2 * ncp, *nmid = nlong + 1, *taken = nlong + 2;
  uint32_t *longq = buf + 2 * ncp + 8, *midq = longq + ncp;
  e = cudaMemsetAsync(afill, 0, sizeof(uint32_t) * (2 * ncp + 8), st);
  if (e == cudaSuccess) {
    (void)out_cap;  // every write is bounded by its own segment of aoff/doff
    k_saddle_lists<<<grid_for(ncp, 256), 256, 0, st>>>(ncp, cellid, des2, asc2, aoff, doff, asc, des);
    k_ext_scatter<<<grid_for(ncp, 256), 256, 0, st>>>(ncp, cellid, des2, asc2, aoff, doff, asc, des, afill, dfill, status);
    k_seg_sort<<<grid_for(ncp, 128), 128, 0, st>>>(ncp, cellid, aoff, doff, asc, des, midq, nmid, longq, nlong, status);
    k_seg_sort_warp<<<152 * 4, SEG_WARP_THREADS, 0, st>>>(cellid, aoff, doff, asc, des, midq, nmid, taken);
    k_seg_sort_block<<<152 * 2, 512, 0, st>>>(cellid, aoff, doff, asc, des, longq, nlong);
    DMSC_LAUNCHED(5);
    e = cudaGetLastError();
  }
  cudaFreeAsync(buf, st);
  return e;
}

cudaError_t build_csr_radix(long long ncp, const uint32_t *cellid, const uint32_t *des2, const uint32_t *asc2,
                      const uint32_t *aoff, const uint32_t *doff, uint32_t *asc, uint32_t *des, long long out_cap,
                      uint32_t *status, cudaStream_t st) {
  if (ncp <= 0) return cudaSuccess;
  long long n = 2 * ncp;
  uint32_t *buf = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&buf, sizeof(uint32_t) * (n * 6 + ncp), st);
  if (e != cudaSuccess) return e;
  uint32_t *kmin = buf, *kmax = buf + n, *vmin = buf + 2 * n, *vmax = buf + 3 * n, *kt = buf + 4 * n, *vt = buf + 5 * n;
  uint32_t *start = buf + 6 * n;
  k_fill_saddles<<<grid_for(ncp, 256), 256, 0, st>>>(ncp, cellid, des2, asc2, aoff, doff, asc, des, kmin, kmax, vmin);
  DMSC_LAUNCHED(1);
  e = copy_u32(vmax, vmin, n, st);
  if (e != cudaSuccess) { cudaFreeAsync(buf, st); return e; }
  int nbits = 1;
  while ((1ll << nbits) <= ncp) ++nbits;
  // minima: asc side; maxima: des side -- ascending saddle index within each run (stable sort)
  e = radix_sort_pairs(kmin, vmin, kt, vt, n, nbits, st);
  if (e == cudaSuccess) {
    k_run_starts<<<grid_for(n, 256), 256, 0, st>>>(n, ncp, kmin, start);
    DMSC_LAUNCHED(1);
    k_scatter_runs<<<grid_for(n, 256), 256, 0, st>>>(n, ncp, kmin, vmin, start, aoff, asc, out_cap, status);
    DMSC_LAUNCHED(1);
    e = radix_sort_pairs(kmax, vmax, kt, vt, n, nbits, st);
  }
  if (e == cudaSuccess) {
    k_run_starts<<<grid_for(n, 256), 256, 0, st>>>(n, ncp, kmax, start);
    DMSC_LAUNCHED(1);
    k_scatter_runs<<<grid_for(n, 256), 256, 0, st>>>(n, ncp, kmax, vmax, start, doff, des, out_cap, status);
    DMSC_LAUNCHED(1);
    e = cudaGetLastError();
  }
  cudaFreeAsync(buf, st);
  return e;
}

// pair_idx of paired critical cells: binary search of the pair's cell id in
// the row-major (y, then x) sorted cp list.
__global__ void k_pair_index(long long ncp, const uint32_t *__restrict__ cellid, const uint8_t *__restrict__ flags,
                             const uint32_t *__restrict__ pair_cell, uint32_t *__restrict__ pair_idx,
                             uint32_t *__restrict__ status) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < ncp; k += (long long)gridDim.x * blockDim.x) {
    if (!(flags[k] & 1)) { pair_idx[k] = 0xFFFFFFFFu; continue; }
    uint32_t tk = pair_cell[k];  // packed x | y<<16 sorts in (y, x) order for non-negative coordinates
    long long lo = 0, hi = ncp;
    while (lo < hi) {
      long long mid = (lo + hi) >> 1;
      if (cellid[mid] < tk) lo = mid + 1; else hi = mid;
    }
    if (lo < ncp && cellid[lo] == tk) pair_idx[k] = (uint32_t)lo;
    else { pair_idx[k] = 0xFFFFFFFFu; atomicOr(status, ST_INVARIANT); }
  }
}

cudaError_t launch_pair_index(long long ncp, const uint32_t *cellid, const uint8_t *flags, const uint32_t *pair_cell,
                              uint32_t *pair_idx, uint32_t *status, cudaStream_t st) {
  if (ncp <= 0) return cudaSuccess;
  k_pair_index<<<grid_for(ncp, 256), 256, 0, st>>>(ncp, cellid, flags, pair_cell, pair_idx, status);
  DMSC_LAUNCHED(1);
  return cudaGetLastError();
}

// Complex flags after writeout: only isBoundryCancelable (bit 2) can be set.
__global__ void k_msc_flags(long long ncp, const uint8_t *__restrict__ cpflags, uint8_t *__restrict__ out) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < ncp; k += (long long)gridDim.x * blockDim.x)
    out[k] = (cpflags[k] & 1) ? 4 : 0;
}
cudaError_t launch_msc_flags(long long ncp, const uint8_t *cpflags, uint8_t *out, cudaStream_t st) {
  if (ncp <= 0) return cudaSuccess;
  k_msc_flags<<<grid_for(ncp, 256), 256, 0, st>>>(ncp, cpflags, out);
  DMSC_LAUNCHED(1);
  return cudaGetLastError();
}

// Reference-layout export of the per-cell arrays: C order [x][y] over ext
// (grid_dataset.cpp:1468-1483), flags int8, pairs/own as (x,y) int16 pairs.
__global__ void k_export_cells(GridGeom g, const uint32_t *__restrict__ codes, const uint4 *__restrict__ labels,
                               const uint32_t *__restrict__ cp_cellid, long long ncp, int8_t *__restrict__ flags,
                               int16_t *__restrict__ pairs, int16_t *__restrict__ own) {
  const long long cny = g.cy + 1, n = (long long)(g.cx + 1) * cny;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    int x = (int)(t / cny), y = (int)(t - (long long)x * cny);
    long long v = (long long)(y >> 1) * g.vnx + (x >> 1);
    int kind = (x & 1) | ((y & 1) << 1);
    uint32_t c = (codes[v] >> (8 * kind)) & 0xff;
    uint4 L4 = labels[v];
    uint32_t lab = kind == 0 ? L4.x : kind == 1 ? L4.y : kind == 2 ? L4.z : L4.w;
    if (flags) flags[t] = (int8_t)((c >> 2) & 3);
    if (pairs) {
      int16_t px = -1, py = -1;
      if (c & CODE_PAIRED) {
        uint32_t d = c & 3;
        px = (int16_t)(g.ex0 + x + (d == DIR_PX ? 1 : d == DIR_MX ? -1 : 0));
        py = (int16_t)(g.ey0 + y + (d == DIR_PY ? 1 : d == DIR_MY ? -1 : 0));
      }
      pairs[2 * t] = px;
      pairs[2 * t + 1] = py;
    }
    if (own) {
      int16_t ox = -1, oy = -1;
      if (lab < (uint32_t)ncp) { uint32_t cc = cp_cellid[lab]; ox = (int16_t)(cc & 0xffff); oy = (int16_t)(cc >> 16); }
      own[2 * t] = ox;
      own[2 * t + 1] = oy;
    }
  }
}

cudaError_t launch_export_cells(const GridGeom &g, const uint32_t *codes, const uint4 *labels, const uint32_t *cp_cellid,
                                long long ncp, int8_t *flags, int16_t *pairs, int16_t *own, cudaStream_t st) {
  long long n = (long long)(g.cx + 1) * (g.cy + 1);
  k_export_cells<<<grid_for(n, 256), 256, 0, st>>>(g, codes, labels, cp_cellid, ncp, flags, pairs, own);
  DMSC_LAUNCHED(1);
  return cudaGetLastError();
}

}  // namespace dmsc
