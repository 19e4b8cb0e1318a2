// Allocation-free variant of the grid backward (pvdb_grid_sample_backward).
//
// Some callers cannot let a library call cudaMalloc: processes that reserve
// all device memory up front through their own pool (a serving process or an
// engine running under a fixed memory budget) must not see allocations they did
// not plan for, and cudaMalloc/cudaFree synchronise the device, which stalls
// the caller's streams. For them this entry point runs the same deterministic
// leaf-sorted reduction with its scratch (sort keys and payloads, radix
// histograms, scan partials) in one fixed file-scope device array, so the call
// itself allocates nothing. The caller still passes the points, the gradients
// and the grid (device memory). The array holds kNoAllocMaxPoints points'
// worth of scratch (about 5.3 MB) on every GPU where the library's module is
// loaded, until the process exits. With CUDA's lazy module loading (the
// default) the module, and so the array, is loaded on a device by the first
// call of this entry point there, which also looks up the array's address:
// make that first call before reserving a memory pool or capturing a stream.
#include <mutex>

#include "reduce.cuh"

namespace pvdb {

constexpr int64_t kNoAllocMaxPoints = 32768;
constexpr int64_t kNoAllocMaxPairs = kNoAllocMaxPoints * 8;
constexpr int64_t kNoAllocTiles = (kNoAllocMaxPairs + kRsTile - 1) / kRsTile;
// radix sort scratch: tile status words of up to 4 digit passes, the digit
// histograms, tile counters and a few scalars
constexpr int64_t kNoAllocHistWords = 4 * kNoAllocTiles * kRsBins + 4 * kRsBins + 16;
// scan partials of the histogram scan (one per 4096-entry tile)
constexpr int64_t kNoAllocPartialWords = 64;
constexpr int64_t kNoAllocWords = 4 * kNoAllocMaxPairs + kNoAllocHistWords + kNoAllocPartialWords;

// Shared by every call on a device. Within one call every word is written
// before it is read (keys and payloads for the call's pairs, histogram tiles,
// partials, size words, the sort's status word, which the sort clears first),
// so nothing needs clearing between calls; calls that overlap on the GPU
// (e.g. issued on two streams) race on it, so serialise them on one stream
// per device.
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocWords];

namespace {
std::mutex g_na_mu;
uint32_t* g_na_ptr[128] = {nullptr};

// Device address of the array for the current device, looked up once per
// device (with that device current) on the first call.
int noalloc_base(uint32_t** out) {
  int dev = 0;
  PVDB_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 128) return set_error(PVDB_ERR_STATE, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_na_mu);
  if (!g_na_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(no-alloc scratch)");
    g_na_ptr[dev] = static_cast<uint32_t*>(p);
  }
  *out = g_na_ptr[dev];
  return PVDB_OK;
}

struct NaPointSrc {
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

__global__ void k_noalloc_keys(GridView gv, const float* __restrict__ xs,
                               const float* __restrict__ ys, const float* __restrict__ zs,
                               int64_t n, uint32_t* keys) {
  const int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= n) return;
  emit_corner_keys(gv, xs[p], ys[p], zs[p], keys, p);
}
}  // namespace

}  // namespace pvdb

using namespace pvdb;

extern "C" int pvdb_grid_sample_backward_noalloc(pvdb_grid g, const float* xs, const float* ys,
                                                 const float* zs, const float* grad_out,
                                                 int64_t n, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(g, "null grid");
  PVDB_REQUIRE(n >= 0, "negative size");
  if (n > kNoAllocMaxPoints)
    return set_error(PVDB_ERR_ARG,
                     "pvdb_grid_sample_backward_noalloc: n exceeds the fixed scratch of 32768 "
                     "points; split the call or use pvdb_grid_sample_backward");
  if (n == 0) return PVDB_OK;
  PVDB_REQUIRE(xs && ys && zs && grad_out, "null argument");
  uint32_t* base = nullptr;
  int rc = noalloc_base(&base);
  if (rc) return rc;
  cudaStream_t st = as_stream(s);
  // views into the fixed array; the capacities make every reserve a no-op
  ReduceScratch rs;
  rs.keys[0] = base;
  rs.keys[1] = base + kNoAllocMaxPairs;
  rs.vals[0] = base + 2 * kNoAllocMaxPairs;
  rs.vals[1] = base + 3 * kNoAllocMaxPairs;
  rs.cap = size_t(kNoAllocMaxPairs);
  rs.hist = base + 4 * kNoAllocMaxPairs;
  rs.hist_cap = size_t(kNoAllocHistWords) * 4;
  rs.partial = rs.hist + kNoAllocHistWords;
  rs.partial_cap = size_t(kNoAllocPartialWords) * 4;
  const int64_t nc = n * 8;
  if (radix_sort_words(nc, slot_key_bits(g->nslots())) > kNoAllocHistWords)
    return set_error(PVDB_ERR_STATE, "no-alloc scratch too small for the sort");
  k_noalloc_keys<<<ceil_div(n, 256), 256, 0, st>>>(g->view(), xs, ys, zs, n, rs.keys[0]);
  PVDB_CHECK_LAUNCH("k_noalloc_keys");
  int buf = 0;
  uint32_t* status = nullptr;
  rc = radix_sort_pairs(rs, nc, slot_key_bits(g->nslots()), true, &buf, st, &status);
  if (rc) return rc;
  NaPointSrc src{xs, ys, zs, grad_out, g->C};
  const int grid = int(std::min<int64_t>(ceil_div(nc, 256), int64_t(num_sms()) * 16));
  k_segment_reduce<NaPointSrc><<<grid, 256, 0, st>>>(
      rs.keys[buf], rs.vals[buf], nc, nullptr, src, g->C == 1 ? g->d_grad : nullptr,
      g->C == 1 ? nullptr : g->d_grad, g->C, g->d_touched, g->d_touched, status);
  PVDB_CHECK_LAUNCH("k_segment_reduce(noalloc)");
  g->tlist_valid = false;  // new touched leaves
  // the status word is read into host stack memory (no allocation); the call
  // waits for its stream, as pvdb_grid_sample_backward does
  return read_wait_status(status, st,
                          "a radix-sort look-back wait of the no-alloc grid backward timed out");
}
