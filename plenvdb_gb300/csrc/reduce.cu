// Device-wide scan, stable LSD radix sort and the generic point backward
// (DensityVDB/ColorVDB backward, plenvdb.h:468-485, :557-573).
//
// Sizes may live on the device (n_dev != NULL): kernels are launched for the
// host-side maximum with a fixed, SM-count-sized grid and loop over the tiles
// that the device-side count actually needs, so the fused training step never
// synchronises with the host.
#include <algorithm>

#include <atomic>

#include "reduce.cuh"

namespace pvdb {

static int g_num_sms = 0;
int num_sms() {
  if (!g_num_sms) {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    g_num_sms = n > 0 ? n : 148;
  }
  return g_num_sms;
}

__device__ __forceinline__ int64_t eff_size(int64_t n_max, const uint32_t* n_dev) {
  return n_dev ? min(n_max, (int64_t)*n_dev) : n_max;
}

// ------------------------------------------------------------------- scan
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;  // 4096

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t warp_sums[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    uint32_t s = lane < nw ? warp_sums[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < nw) warp_sums[lane] = s;  // inclusive
  }
  __syncthreads();
  const uint32_t warp_excl = wid ? warp_sums[wid - 1] : 0u;
  if (total) *total = warp_sums[(blockDim.x >> 5) - 1];
  const uint32_t r = warp_excl + x - v;
  __syncthreads();
  return r;
}

__global__ void k_scan_reduce(const uint32_t* __restrict__ in, int64_t n_max,
                              const uint32_t* n_dev, uint32_t* partial) {
  grid_dep_sync();
  const int64_t n = eff_size(n_max, n_dev);
  const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t base = t * kScanTile + int64_t(threadIdx.x) * kScanItems;
    uint32_t s = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; ++q)
      if (base + q < n) s += in[base + q];
    uint32_t tot;
    block_exclusive_scan(s, &tot);
    if (threadIdx.x == 0) partial[t] = tot;
  }
}

__global__ void k_scan_partials(uint32_t* partial, int64_t n_max, const uint32_t* n_dev,
                                uint32_t* total) {
  grid_dep_sync();
  __shared__ uint32_t carry_s;
  const int64_t n = eff_size(n_max, n_dev);
  const int64_t nb = (n + kScanTile - 1) / kScanTile;
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  for (int64_t base = 0; base < nb; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    const uint32_t v = i < nb ? partial[i] : 0u;
    uint32_t tot;
    const uint32_t ex = block_exclusive_scan(v, &tot);
    const uint32_t c = carry_s;
    if (i < nb) partial[i] = c + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry_s = c + tot;
    __syncthreads();
  }
  if (threadIdx.x == 0 && total) *total = carry_s;
}

__global__ void k_scan_apply(const uint32_t* __restrict__ in, uint32_t* out, int64_t n_max,
                             const uint32_t* n_dev, const uint32_t* __restrict__ partial) {
  grid_dep_sync();
  const int64_t n = eff_size(n_max, n_dev);
  const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t base = t * kScanTile + int64_t(threadIdx.x) * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) {
      v[q] = base + q < n ? in[base + q] : 0u;
      s += v[q];
    }
    uint32_t run = block_exclusive_scan(s, nullptr) + partial[t];
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) {
      if (base + q < n) out[base + q] = run;
      run += v[q];
    }
  }
}

// Single-block scan for short inputs: 1024 threads walk the input in chunks
// of 8192 with a running carry (one launch instead of three). Each chunk goes
// through shared memory so that global loads and stores are coalesced; thread
// t scans elements 8t .. 8t+7 of the chunk (the padded index spreads them
// over the banks).
constexpr int kScan1Threads = 1024;
constexpr int kScan1Items = 8;
constexpr int64_t kScan1Max = 262144;  // inputs up to this length take the one-block path

__device__ __forceinline__ int scan1_pad(int i) { return i + (i >> 5); }

__global__ void __launch_bounds__(kScan1Threads)
    k_scan_single(const uint32_t* __restrict__ in, uint32_t* out, int64_t n_max,
                  const uint32_t* n_dev, uint32_t* total) {
  grid_dep_sync();
  constexpr int kChunk = kScan1Threads * kScan1Items;
  __shared__ uint32_t buf[kChunk + kChunk / 32];
  __shared__ uint32_t carry_s;
  const int64_t n = eff_size(n_max, n_dev);
  const int t = threadIdx.x;
  if (t == 0) carry_s = 0;
  __syncthreads();
  for (int64_t c0 = 0; c0 < n; c0 += kChunk) {
#pragma unroll
    for (int q = 0; q < kScan1Items; ++q) {
      const int e = q * kScan1Threads + t;
      buf[scan1_pad(e)] = c0 + e < n ? in[c0 + e] : 0u;
    }
    __syncthreads();
    uint32_t v[kScan1Items];
    uint32_t sum = 0;
#pragma unroll
    for (int q = 0; q < kScan1Items; ++q) {
      v[q] = buf[scan1_pad(t * kScan1Items + q)];
      sum += v[q];
    }
    uint32_t tot;
    uint32_t run = block_exclusive_scan(sum, &tot) + carry_s;
#pragma unroll
    for (int q = 0; q < kScan1Items; ++q) {
      buf[scan1_pad(t * kScan1Items + q)] = run;
      run += v[q];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kScan1Items; ++q) {
      const int e = q * kScan1Threads + t;
      if (c0 + e < n) out[c0 + e] = buf[scan1_pad(e)];
    }
    __syncthreads();
    if (t == 0) carry_s += tot;
    __syncthreads();
  }
  if (t == 0 && total) *total = carry_s;
}

int scan_exclusive_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* total,
                       uint32_t** partial, size_t* partial_cap, cudaStream_t st) {
  return scan_exclusive_u32_dev(in, out, n, nullptr, total, partial, partial_cap, st);
}

int scan_exclusive_u32_dev(const uint32_t* in, uint32_t* out, int64_t n_max,
                           const uint32_t* n_dev, uint32_t* total, uint32_t** partial,
                           size_t* partial_cap, cudaStream_t st) {
  if (n_max <= 0) {
    if (total) PVDB_CHECK_CUDA(cudaMemsetAsync(total, 0, 4, st));
    return PVDB_OK;
  }
  if (n_max <= kScan1Max) {
    launch_k(k_scan_single, 1, kScan1Threads, 0, st, in, out, n_max, n_dev, total);
    PVDB_CHECK_LAUNCH("k_scan_single");
    return PVDB_OK;
  }
  const int64_t nb = (n_max + kScanTile - 1) / kScanTile;
  int rc = dev_reserve((void**)partial, partial_cap, size_t(nb) * 4);
  if (rc) return rc;
  const int grid = int(std::min<int64_t>(nb, int64_t(num_sms()) * 8));
  launch_k(k_scan_reduce, grid, kScanThreads, 0, st, in, n_max, n_dev, *partial);
  launch_k(k_scan_partials, 1, 1024, 0, st, *partial, n_max, n_dev, total);
  launch_k(k_scan_apply, grid, kScanThreads, 0, st, in, out, n_max, n_dev, *partial);
  PVDB_CHECK_LAUNCHES("scan", 3);
  return PVDB_OK;
}

// ------------------------------------------------------------- radix sort
// Stable LSD radix sort, 8-bit digits, one kernel per digit pass ("onesweep"):
//   k_os_init     zeroes the per-pass tile status words, digit histograms and
//                 tile counters for the tiles the device-side count needs;
//   k_os_hist     builds the digit histograms of every pass in one read;
//   k_os_scatter  per pass: CTAs take 1024-key tiles in order from a counter,
//                 count the tile's digits, publish them, and find the tile's
//                 exclusive prefix per digit by looking back over the earlier
//                 tiles' published counts (decoupled look-back); then scatter
//                 stably (tile order, and (warp, round, lane) = index order
//                 inside a tile).
// A tile publishes its own count before it waits on anyone, and a tile only
// waits on tiles taken earlier (already running), so every wait ends; each is
// still bounded, and one that gives up sets an error flag.
constexpr int kRsWarps = kRsThreads / 32;
constexpr uint32_t kOsAgg = 0x40000000u;     // status: tile count published
constexpr uint32_t kOsPrefix = 0x80000000u;  // status: inclusive prefix published
constexpr uint32_t kOsValue = 0x3FFFFFFFu;
constexpr uint32_t kOsSpinMax = 1u << 24;

// Scratch words after the status array: ghist [npass][256], counters
// [npass], n, error flag.
struct OsLayout {
  int64_t ntiles_max;
  int npass;
  int64_t status, ghist, counters, n, err, words;
};
static OsLayout os_layout(int64_t n_max, int npass) {
  OsLayout L;
  L.ntiles_max = (n_max + kRsTile - 1) / kRsTile;
  L.npass = npass;
  L.status = 0;
  L.ghist = L.status + int64_t(npass) * L.ntiles_max * kRsBins;
  L.counters = L.ghist + int64_t(npass) * kRsBins;
  L.n = L.counters + npass;
  L.err = L.n + 1;
  L.words = L.err + 1;
  return L;
}

__global__ void k_os_init(int64_t n_max, const uint32_t* n_dev, int npass, int64_t ntiles_max,
                          uint32_t* scratch, OsLayout L) {
  grid_dep_sync();
  const int64_t n = eff_size(n_max, n_dev);
  const int64_t ntiles = (n + kRsTile - 1) / kRsTile;
  const int64_t per = ntiles * kRsBins;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < int64_t(npass) * per;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t p = i / per, r = i - p * per;
    scratch[L.status + p * ntiles_max * kRsBins + r] = 0u;
  }
  const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (t < int64_t(npass) * kRsBins) scratch[L.ghist + t] = 0u;
  if (t < npass) scratch[L.counters + t] = 0u;
  if (t == 0) {
    scratch[L.n] = uint32_t(n);
    scratch[L.err] = 0u;
  }
}

__global__ void __launch_bounds__(kRsThreads)
    k_os_hist(const uint32_t* __restrict__ keys, int npass, uint32_t* scratch, OsLayout L) {
  grid_dep_sync();
  __shared__ uint32_t h[4][kRsBins];
  const int64_t n = scratch[L.n];
  for (int q = threadIdx.x; q < 4 * kRsBins; q += blockDim.x) (&h[0][0])[q] = 0u;
  __syncthreads();
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const uint32_t k = keys[i];
    for (int p = 0; p < npass; ++p) atomicAdd(&h[p][(k >> (8 * p)) & 255u], 1u);
  }
  __syncthreads();
  for (int p = 0; p < npass; ++p) {
    const uint32_t c = h[p][threadIdx.x];
    if (c) atomicAdd(scratch + L.ghist + p * kRsBins + threadIdx.x, c);
  }
}

__global__ void __launch_bounds__(kRsThreads)
    k_os_scatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin, int pass,
                 uint32_t* scratch, OsLayout L, uint32_t* kout, uint32_t* vout, uint32_t* err,
                 uint32_t spin_max, int hold_first) {
  grid_dep_sync();
  // an earlier pass gave up: its order is wrong, so this one does nothing
  if (*(volatile uint32_t*)err) return;
  __shared__ uint32_t wh[kRsWarps][kRsBins];
  __shared__ uint32_t gbase[kRsBins];
  __shared__ uint32_t tile_s;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, d = threadIdx.x;
  const int shift = 8 * pass;
  const int64_t n = scratch[L.n];
  const int64_t ntiles = (n + kRsTile - 1) / kRsTile;
  volatile uint32_t* status = scratch + L.status + int64_t(pass) * L.ntiles_max * kRsBins;
  const unsigned lt = lanemask_lt();
  // bucket bases of this pass: exclusive scan of the digit histogram
  {
    uint32_t tot;
    gbase[d] = block_exclusive_scan(scratch[L.ghist + pass * kRsBins + d], &tot);
  }
  for (;;) {
    if (threadIdx.x == 0) tile_s = atomicAdd(scratch + L.counters + pass, 1u);
    for (int q = threadIdx.x; q < kRsWarps * kRsBins; q += kRsThreads) (&wh[0][0])[q] = 0;
    __syncthreads();
    const int64_t t = tile_s;
    if (t >= ntiles) break;
    const int64_t wbase = t * kRsTile + int64_t(w) * (kRsRounds * 32);
    uint32_t key[kRsRounds];
#pragma unroll
    for (int r = 0; r < kRsRounds; ++r) {
      const int64_t i = wbase + r * 32 + lane;
      key[r] = i < n ? kin[i] : 0u;
    }
    // per-warp digit histogram
#pragma unroll
    for (int r = 0; r < kRsRounds; ++r) {
      const bool valid = wbase + r * 32 + lane < n;
      const uint32_t dg = valid ? ((key[r] >> shift) & 255u) : 256u;
      const unsigned peers = __match_any_sync(0xffffffffu, dg);
      if (valid && lane == __ffs(peers) - 1) wh[w][dg] += __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    // thread d: tile count, publish, look back, publish the inclusive prefix
    {
      uint32_t cnt = 0;
#pragma unroll
      for (int q = 0; q < kRsWarps; ++q) cnt += wh[q][d];
      volatile uint32_t* my = status + t * kRsBins + d;
      if (t == 0) {
        if (!hold_first) *my = kOsPrefix | cnt;  // (the test hook withholds it)
      } else {
        *my = kOsAgg | cnt;
      }
      uint32_t acc = 0;
      for (int64_t tt = t - 1; tt >= 0; --tt) {
        uint32_t v = status[tt * kRsBins + d];
        for (uint32_t it = 0; v == 0u; ++it) {
          if (it >= spin_max) {
            atomicOr(err, 4u);
            v = kOsPrefix;  // give up: leave the positions wrong but finish
            break;
          }
          v = status[tt * kRsBins + d];
        }
        acc += v & kOsValue;
        if (v & kOsPrefix) break;
      }
      if (t > 0) *my = kOsPrefix | (acc + cnt);
      // per-warp exclusive offsets of this digit
      uint32_t run = gbase[d] + acc;
#pragma unroll
      for (int q = 0; q < kRsWarps; ++q) {
        const uint32_t c = wh[q][d];
        wh[q][d] = run;
        run += c;
      }
    }
    __syncthreads();
    // stable ranks and scatter
#pragma unroll
    for (int r = 0; r < kRsRounds; ++r) {
      const int64_t i = wbase + r * 32 + lane;
      const bool valid = i < n;
      const uint32_t dg = valid ? ((key[r] >> shift) & 255u) : 256u;
      const unsigned peers = __match_any_sync(0xffffffffu, dg);
      uint32_t pos = 0;
      if (valid) pos = wh[w][dg] + __popc(peers & lt);
      __syncwarp();
      if (valid && lane == __ffs(peers) - 1) wh[w][dg] += __popc(peers);
      __syncwarp();
      if (valid) {
        kout[pos] = key[r];
        vout[pos] = vin ? vin[i] : uint32_t(i);
      }
    }
    __syncthreads();
  }
}

int slot_key_bits(int64_t nslots) {
  int b = 1;
  while ((int64_t(1) << b) <= nslots) ++b;
  return b;
}

int radix_sort_pairs_dev(ReduceScratch& rs, int64_t n_max, const uint32_t* n_dev, int key_bits,
                         bool iota_vals, int* out_buf, cudaStream_t st, uint32_t** status) {
  *out_buf = 0;
  if (status) *status = nullptr;
  if (n_max <= 0) return PVDB_OK;
  const int npass = (key_bits + 7) / 8;
  if (npass < 1 || npass > 4) return set_error(PVDB_ERR_ARG, "radix sort takes 1..32 key bits");
  const OsLayout L = os_layout(n_max, npass);
  int rc = dev_reserve((void**)&rs.hist, &rs.hist_cap, size_t(L.words) * 4);
  if (rc) return rc;
  uint32_t* sc = rs.hist;
  uint32_t* errp = sc + L.err;
  if (status) *status = errp;
  const uint32_t spin = debug_spin_limit(kOsSpinMax);
  const int hold = debug_hold_first();
  const int g_init = int(std::min<int64_t>(
      std::max<int64_t>(ceil_div(int64_t(npass) * L.ntiles_max * kRsBins, 256), 1),
      int64_t(num_sms()) * 8));
  launch_k(k_os_init, g_init, 256, 0, st, n_max, n_dev, npass, L.ntiles_max, sc, L);
  PVDB_CHECK_LAUNCH("k_os_init");
  const int g_hist = int(std::min<int64_t>(ceil_div(n_max, kRsThreads), int64_t(num_sms()) * 4));
  launch_k(k_os_hist, g_hist, kRsThreads, 0, st, rs.keys[0], npass, sc, L);
  PVDB_CHECK_LAUNCH("k_os_hist");
  const int grid = int(std::min<int64_t>(L.ntiles_max, int64_t(num_sms()) * 4));
  int cur = 0;
  for (int p = 0; p < npass; ++p) {
    launch_k(k_os_scatter, grid, kRsThreads, 0, st, rs.keys[cur],
             (p == 0 && iota_vals) ? nullptr : rs.vals[cur], p, sc, L, rs.keys[cur ^ 1],
             rs.vals[cur ^ 1], errp, spin, hold);
    PVDB_CHECK_LAUNCH("k_os_scatter");
    cur ^= 1;
  }
  *out_buf = cur;
  return PVDB_OK;
}

int radix_sort_words(int64_t n_max, int key_bits) {
  return int(os_layout(n_max, (key_bits + 7) / 8).words);
}

int radix_sort_pairs(ReduceScratch& rs, int64_t n, int key_bits, bool iota_vals, int* out_buf,
                     cudaStream_t st, uint32_t** status) {
  return radix_sort_pairs_dev(rs, n, nullptr, key_bits, iota_vals, out_buf, st, status);
}

int scratch_reserve(ReduceScratch& rs, int64_t n) {
  if (rs.cap >= size_t(n) && rs.keys[0]) return PVDB_OK;
  for (int b = 0; b < 2; ++b) {
    dev_free(rs.keys[b]);
    dev_free(rs.vals[b]);
    rs.keys[b] = rs.vals[b] = nullptr;
  }
  rs.cap = 0;
  const size_t want = std::max<size_t>(size_t(n), 4096);
  int rc;
  for (int b = 0; b < 2; ++b) {
    if ((rc = dev_alloc((void**)&rs.keys[b], want * 4))) return rc;
    if ((rc = dev_alloc((void**)&rs.vals[b], want * 4))) return rc;
  }
  rs.cap = want;
  return PVDB_OK;
}

int reduce_reserve(pvdb_grid_s* g, int64_t n) { return scratch_reserve(g->red, n); }

void free_scratch(ReduceScratch& rs) {
  for (int b = 0; b < 2; ++b) {
    dev_free(rs.keys[b]);
    dev_free(rs.vals[b]);
    rs.keys[b] = rs.vals[b] = nullptr;
  }
  dev_free(rs.hist);
  dev_free(rs.partial);
  rs.hist = rs.partial = nullptr;
  rs.cap = rs.hist_cap = rs.partial_cap = 0;
}

// ------------------------------------------------- generic point backward
struct PointSrc {
  const float* xs;
  const float* ys;
  const float* zs;
  const float* g;
  int C;
  __device__ __forceinline__ void pos(int64_t s, float& x, float& y, float& z) const {
    x = xs[s]; y = ys[s]; z = zs[s];
  }
  __device__ __forceinline__ float gd(int64_t s) const { return g[s]; }
  __device__ __forceinline__ bool has_c(int64_t) const { return true; }
  __device__ __forceinline__ float gc(int64_t s, int ch) const { return g[s * C + ch]; }
};

namespace {
std::atomic<uint32_t> g_dbg_spin{0};
std::atomic<int> g_dbg_hold{0};
}  // namespace

uint32_t debug_spin_limit(uint32_t builtin) {
  const uint32_t v = g_dbg_spin.load();
  return v ? v : builtin;
}

int debug_hold_first() { return g_dbg_hold.load() == 1 ? 1 : 0; }
int debug_hold_staging() { return g_dbg_hold.load() == 2 ? 1 : 0; }

int read_wait_status(const uint32_t* status, cudaStream_t st, const char* what) {
  uint32_t h = 0;
  if (status) PVDB_CHECK_CUDA(cudaMemcpyAsync(&h, status, 4, cudaMemcpyDeviceToHost, st));
  PVDB_CHECK_CUDA(cudaStreamSynchronize(st));
  if (h) return set_error(PVDB_ERR_TIMEOUT, what);
  return PVDB_OK;
}

__global__ void k_point_keys(GridView gv, const float* __restrict__ xs, const float* __restrict__ ys,
                             const float* __restrict__ zs, int64_t n, uint32_t* keys) {
  grid_dep_sync();
  const int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= n) return;
  emit_corner_keys(gv, xs[p], ys[p], zs[p], keys, p);
}

}  // namespace pvdb

using namespace pvdb;

extern "C" int pvdb_debug_wait_limit(uint32_t spins, int32_t hold_first) {
  clear_error();
  g_dbg_spin.store(spins);
  g_dbg_hold.store(hold_first == 2 ? 2 : hold_first ? 1 : 0);
  return PVDB_OK;
}

extern "C" int pvdb_grid_sample_backward(pvdb_grid g, const float* xs, const float* ys,
                                         const float* zs, const float* grad_out, int64_t n,
                                         int32_t mem, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(g, "null grid");
  PVDB_REQUIRE(n >= 0, "negative size");
  if (n == 0) return PVDB_OK;
  PVDB_REQUIRE(xs && ys && zs && grad_out, "null argument");
  PVDB_REQUIRE(n * 8 < int64_t(0xFFFFFFF0u), "too many points for one backward call");
  cudaStream_t st = as_stream(s);
  const float *dx = xs, *dy = ys, *dz = zs, *dg = grad_out;
  if (mem == PVDB_MEM_HOST) {
    int rc = dev_reserve(&g->d_stage, &g->stage_cap, size_t(n) * 4 * (3 + g->C));
    if (rc) return rc;
    float* b = (float*)g->d_stage;
    PVDB_CHECK_CUDA(cudaMemcpyAsync(b, xs, n * 4, cudaMemcpyHostToDevice, st));
    PVDB_CHECK_CUDA(cudaMemcpyAsync(b + n, ys, n * 4, cudaMemcpyHostToDevice, st));
    PVDB_CHECK_CUDA(cudaMemcpyAsync(b + 2 * n, zs, n * 4, cudaMemcpyHostToDevice, st));
    PVDB_CHECK_CUDA(cudaMemcpyAsync(b + 3 * n, grad_out, n * 4 * g->C, cudaMemcpyHostToDevice, st));
    dx = b; dy = b + n; dz = b + 2 * n; dg = b + 3 * n;
  }
  const int64_t nc = n * 8;
  int rc = reduce_reserve(g, nc);
  if (rc) return rc;
  launch_k(k_point_keys, ceil_div(n, 256), 256, 0, st, g->view(), dx, dy, dz, n, g->red.keys[0]);
  PVDB_CHECK_LAUNCH("k_point_keys");
  int buf = 0;
  uint32_t* status = nullptr;
  rc = radix_sort_pairs(g->red, nc, slot_key_bits(g->nslots()), true, &buf, st, &status);
  if (rc) return rc;
  PointSrc src{dx, dy, dz, dg, g->C};
  const int grid = int(std::min<int64_t>(ceil_div(nc, 256), int64_t(num_sms()) * 16));
  launch_k(k_segment_reduce<PointSrc>, grid, 256, 0, st, g->red.keys[buf], g->red.vals[buf], nc,
           nullptr, src, g->C == 1 ? g->d_grad : nullptr, g->C == 1 ? nullptr : g->d_grad, g->C,
           g->d_touched, g->d_touched, status);
  PVDB_CHECK_LAUNCH("k_segment_reduce");
  g->tlist_valid = false;
  // the call waits for its stream (as the reference's backward does) so that a
  // sort wait that gave up is reported, with the gradient left unchanged
  return read_wait_status(status, st, "a radix-sort look-back wait of the grid backward timed out");
}
