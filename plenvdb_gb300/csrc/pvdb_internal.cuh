// Internal declarations shared by the libpvdb translation units.
//
// Leaf store layout (device, HBM):
//   table  int32 [ldim0*ldim1*ldim2]   leaf id of each 8^3 block of [0, 8*ldim), -1 = none
//   origin int32 [nleaf*3]             voxel coordinate of each leaf's (0,0,0) corner
//   mask   uint64[nleaf*8]             active bits, bit n of the leaf = voxel offset n
//   data   f32   [nleaf*512*C]         values, voxel-major with the C channels innermost
//   grad   f32   [nleaf*512*C]         gradient, same layout
// A voxel's offset inside its leaf is ((x&7)<<6)|((y&7)<<3)|(z&7), the NanoVDB
// LeafNode::CoordToOffset order (nanovdb/NanoVDB.h:3893-3899), and its "slot" is
// leaf*512 + offset. Leaves are numbered in Morton order of their leaf
// coordinates so that leaves adjacent along a ray sit close together.
#pragma once
#include <utility>

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/pvdb.h"

namespace pvdb {

constexpr int kLeafVox = 512;
// BF16 values per voxel in a 12-channel grid's shadow (32 bytes: one sector)
constexpr int kHalfStride = 16;

// ------------------------------------------------------------- errors (host)
int set_error(int code, const std::string& msg);
int cuda_error(cudaError_t e, const char* what);
void clear_error();

#define PVDB_CHECK_CUDA(call)                                  \
  do {                                                          \
    cudaError_t _e = (call);                                    \
    if (_e != cudaSuccess) return ::pvdb::cuda_error(_e, #call); \
  } while (0)

// Every kernel launch is followed by exactly one PVDB_CHECK_LAUNCH (or
// PVDB_CHECK_LAUNCHES(n) after n launches); it also counts the launches.
void count_launches(int n);
#define PVDB_CHECK_LAUNCHES(what, n)                                \
  do {                                                               \
    ::pvdb::count_launches(n);                                       \
    cudaError_t _e = cudaGetLastError();                             \
    if (_e != cudaSuccess) return ::pvdb::cuda_error(_e, what);      \
  } while (0)
#define PVDB_CHECK_LAUNCH(what) PVDB_CHECK_LAUNCHES(what, 1)

// Opt a kernel into more than 48 KB of dynamic shared memory, once per
// process (so a stream capture never issues the call).
#define PVDB_SMEM_ATTR(kernel, bytes)                                                    \
  do {                                                                                  \
    static bool _done = false;                                                          \
    if (!_done) {                                                                       \
      PVDB_CHECK_CUDA(                                                                  \
          cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)); \
      _done = true;                                                                     \
    }                                                                                   \
  } while (0)

#define PVDB_REQUIRE(cond, msg)                                         \
  do {                                                                   \
    if (!(cond)) return ::pvdb::set_error(PVDB_ERR_ARG, msg);            \
  } while (0)

// Device allocation through the library (honours the failure-injection hook).
int dev_alloc(void** p, size_t bytes);
void dev_free(void* p);
// Grows *p to at least `bytes` (contents not preserved).
int dev_reserve(void** p, size_t* cap, size_t bytes);

inline cudaStream_t as_stream(pvdb_stream s) { return reinterpret_cast<cudaStream_t>(s); }

inline int ceil_div(int64_t a, int64_t b) { return int((a + b - 1) / b); }

// ------------------------------------------------------------ device view
struct GridView {
  int reso[3];
  int ldim[3];
  int C;
  int nleaf;
  float background;
  const int32_t* __restrict__ table;
  const int32_t* __restrict__ origin;
  const uint64_t* __restrict__ mask;
  float* data;
  float* grad;
  // per-brick upper bound of the values a trilinear sample can interpolate
  // (scalar grids that a march reads; NULL when not maintained)
  uint32_t* bmax;
  int bdim[3];
};

// Scratch of the deterministic gradient reduction (one per grid topology).
struct ReduceScratch {
  uint32_t* keys[2] = {nullptr, nullptr};
  uint32_t* vals[2] = {nullptr, nullptr};
  size_t cap = 0;              // elements per buffer
  uint32_t* hist = nullptr;    // radix histograms
  size_t hist_cap = 0;
  uint32_t* partial = nullptr; // scan partials
  size_t partial_cap = 0;
};

}  // namespace pvdb

// Opaque handles (declared in the global namespace to match pvdb.h).
struct pvdb_grid_s {
  int reso[3];
  int ldim[3];
  int C;
  int nleaf;
  float background;
  int64_t nactive;
  int32_t* d_table = nullptr;
  int32_t* d_origin = nullptr;
  uint64_t* d_mask = nullptr;
  float* d_data = nullptr;
  float* d_grad = nullptr;
  uint8_t* d_touched = nullptr;  // [nleaf] leaves whose gradient may be nonzero
  bool all_touched = true;       // every leaf must be treated as touched
  int32_t* d_tlist = nullptr;    // [nleaf] compacted ids of the touched leaves
  uint32_t* d_tcount = nullptr;  // number of entries in d_tlist (device)
  bool tlist_valid = false;      // d_tlist reflects d_touched
  // Brick bound: for each brick of 4^3 trilinear cells, the largest value of
  // the voxels [4b-1, 4b+5] per axis (every corner of those cells and of their
  // neighbours), as order-preserving uint32 keys. Kept an upper bound by the
  // voxel Adam (atomicMax when a value grows); any other write of the data
  // invalidates it.
  uint32_t* d_bmax = nullptr;
  int bdim[3] = {0, 0, 0};
  bool bmax_valid = false;
  // BF16 shadow of a 12-channel grid's values, [nleaf*512][kHalfStride]
  // (channels 0..11, then zeros; read by the BF16 train step): rebuilt from
  // the FP32 master values when invalid, kept current by the voxel Adam
  // (which writes both); any other write of the data invalidates it, as it
  // does the brick bound.
  __nv_bfloat16* d_half = nullptr;
  bool half_valid = false;
  // TV terms of the touched leaves' voxels, [nleaf*512][C] (the fused train
  // step's deferred sparse TV: written beside the gradient sums, added by the
  // voxel Adam); allocated at first use
  float* d_tv = nullptr;
  std::vector<int32_t> h_table;
  std::vector<int32_t> h_origin;
  std::vector<uint64_t> h_mask;
  pvdb::ReduceScratch red;
  // host staging for PVDB_MEM_HOST calls
  void* d_stage = nullptr;
  size_t stage_cap = 0;

  pvdb::GridView view() const {
    pvdb::GridView v;
    for (int a = 0; a < 3; ++a) { v.reso[a] = reso[a]; v.ldim[a] = ldim[a]; }
    v.C = C; v.nleaf = nleaf; v.background = background;
    v.table = d_table; v.origin = d_origin; v.mask = d_mask; v.data = d_data; v.grad = d_grad;
    v.bmax = bmax_valid ? d_bmax : nullptr;
    for (int a = 0; a < 3; ++a) v.bdim[a] = bdim[a];
    return v;
  }
  int64_t nslots() const { return int64_t(nleaf) * pvdb::kLeafVox; }
};

namespace pvdb {

// ------------------------------------------------------- device helpers
__device__ __forceinline__ int leaf_of(const GridView& g, int i, int j, int k) {
  if ((unsigned)i >= (unsigned)(g.ldim[0] << 3) || (unsigned)j >= (unsigned)(g.ldim[1] << 3) ||
      (unsigned)k >= (unsigned)(g.ldim[2] << 3))
    return -1;
  return __ldg(g.table + ((i >> 3) * g.ldim[1] + (j >> 3)) * g.ldim[2] + (k >> 3));
}

__device__ __forceinline__ int vox_offset(int i, int j, int k) {
  return ((i & 7) << 6) | ((j & 7) << 3) | (k & 7);
}

// Slot (leaf*512 + offset) of a voxel, or -1 when it lies in no allocated leaf.
__device__ __forceinline__ int slot_of(const GridView& g, int i, int j, int k) {
  int l = leaf_of(g, i, j, k);
  return l < 0 ? -1 : (l << 9) | vox_offset(i, j, k);
}

// Scalar (C == 1) value at a voxel.
__device__ __forceinline__ float value1(const GridView& g, int i, int j, int k) {
  int s = slot_of(g, i, j, k);
  return s < 0 ? g.background : __ldg(g.data + s);
}

// The 8 trilinear corners in the reference's visiting order
// (densityvdb.cu:116-123): 000,001,011,010,110,111,101,100.
__device__ __forceinline__ void corner_delta(int c, int& di, int& dj, int& dk) {
  switch (c) {
    case 0: di = 0; dj = 0; dk = 0; break;
    case 1: di = 0; dj = 0; dk = 1; break;
    case 2: di = 0; dj = 1; dk = 1; break;
    case 3: di = 0; dj = 1; dk = 0; break;
    case 4: di = 1; dj = 1; dk = 0; break;
    case 5: di = 1; dj = 1; dk = 1; break;
    case 6: di = 1; dj = 0; dk = 1; break;
    default: di = 1; dj = 0; dk = 0; break;
  }
}

// Floor to int as nanovdb::Vec3::floor (Floor(x) = int32(floorf(x))).
__device__ __forceinline__ int ifloor(float x) { return int(floorf(x)); }

// Slots of the 8 trilinear corners of cell (i,j,k) in the reference's corner
// order (see corner_delta), -1 where a corner lies in no allocated leaf. When
// the cell does not cross a leaf face ((i|j|k) & 7 < 7 per axis) all corners
// share one leaf: one table lookup, and the offsets follow from the voxel
// layout (+64 x, +8 y, +1 z).
__device__ __forceinline__ void corner_slots(const GridView& g, int i, int j, int k, int s[8]) {
  if ((i & 7) != 7 && (j & 7) != 7 && (k & 7) != 7) {
    const int l = leaf_of(g, i, j, k);
    const int b = l < 0 ? -1 : ((l << 9) | vox_offset(i, j, k));
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      int di, dj, dk;
      corner_delta(c, di, dj, dk);
      s[c] = b < 0 ? -1 : b + (di << 6) + (dj << 3) + dk;
    }
  } else {
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      int di, dj, dk;
      corner_delta(c, di, dj, dk);
      s[c] = slot_of(g, i + di, j + dj, k + dk);
    }
  }
}

// Density trilinear with the reference's association: for each corner in order,
// res += ((v*(1-u))*(1-v))*(1-w) (densityvdb.cu:115-123), from the 8 corner
// values in the order of corner_delta.
__device__ __forceinline__ float trilinear1_values(const float val[8], float u, float v, float w) {
  const float iu = 1.f - u, iv = 1.f - v, iw = 1.f - w;
  float r = 0.f;
  r = __fadd_rn(r, __fmul_rn(__fmul_rn(__fmul_rn(val[0], iu), iv), iw));
  r = __fadd_rn(r, __fmul_rn(__fmul_rn(__fmul_rn(val[1], iu), iv), w));
  r = __fadd_rn(r, __fmul_rn(__fmul_rn(__fmul_rn(val[2], iu), v), w));
  r = __fadd_rn(r, __fmul_rn(__fmul_rn(__fmul_rn(val[3], iu), v), iw));
  r = __fadd_rn(r, __fmul_rn(__fmul_rn(__fmul_rn(val[4], u), v), iw));
  r = __fadd_rn(r, __fmul_rn(__fmul_rn(__fmul_rn(val[5], u), v), w));
  r = __fadd_rn(r, __fmul_rn(__fmul_rn(__fmul_rn(val[6], u), iv), w));
  r = __fadd_rn(r, __fmul_rn(__fmul_rn(__fmul_rn(val[7], u), iv), iw));
  return r;
}

// Density trilinear at index-space position (x, y, z).
__device__ __forceinline__ float trilinear1(const GridView& g, float x, float y, float z) {
  const int i = ifloor(x), j = ifloor(y), k = ifloor(z);
  int s[8];
  corner_slots(g, i, j, k, s);
  float val[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) val[c] = s[c] < 0 ? g.background : __ldg(g.data + s[c]);
  return trilinear1_values(val, x - float(i), y - float(j), z - float(k));
}

// Trilinear corner weights for the multi-channel formula (colorvdb.cu:100-107):
// scale_c = ((a*b)*c) of the three 1-u / u factors, computed before the multiply.
__device__ __forceinline__ void corner_scales(float u, float v, float w, float s[8]) {
  const float iu = 1.f - u, iv = 1.f - v, iw = 1.f - w;
  s[0] = __fmul_rn(__fmul_rn(iu, iv), iw);
  s[1] = __fmul_rn(__fmul_rn(iu, iv), w);
  s[2] = __fmul_rn(__fmul_rn(iu, v), w);
  s[3] = __fmul_rn(__fmul_rn(iu, v), iw);
  s[4] = __fmul_rn(__fmul_rn(u, v), iw);
  s[5] = __fmul_rn(__fmul_rn(u, v), w);
  s[6] = __fmul_rn(__fmul_rn(u, iv), w);
  s[7] = __fmul_rn(__fmul_rn(u, iv), iw);
}

// Density-style corner weight of corner c for a gradient g:
// ((g*(1-u))*(1-v))*(1-w) pattern (densityvdb.cu:158-165).
__device__ __forceinline__ float density_corner_term(float g, float u, float v, float w, int c) {
  int di, dj, dk;
  corner_delta(c, di, dj, dk);
  const float a = di ? u : 1.f - u, b = dj ? v : 1.f - v, cc = dk ? w : 1.f - w;
  return __fmul_rn(__fmul_rn(__fmul_rn(g, a), b), cc);
}

// Order-preserving float <-> uint32 keys (for atomicMax on floats).
__device__ __forceinline__ uint32_t fkey(float f) {
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float fkey_inv(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

// Raises the brick bounds that cover voxel (x,y,z) to at least v: the bricks
// b with 4b-1 <= x <= 4b+5 per axis.
__device__ __forceinline__ void bmax_raise(const GridView& g, int x, int y, int z, float v) {
  const uint32_t key = fkey(v);
  const int x0 = max((x - 2) >> 2, 0), x1 = min((x + 1) >> 2, g.bdim[0] - 1);
  const int y0 = max((y - 2) >> 2, 0), y1 = min((y + 1) >> 2, g.bdim[1] - 1);
  const int z0 = max((z - 2) >> 2, 0), z1 = min((z + 1) >> 2, g.bdim[2] - 1);
  for (int bx = x0; bx <= x1; ++bx)
    for (int by = y0; by <= y1; ++by)
      for (int bz = z0; bz <= z1; ++bz)
        atomicMax(g.bmax + (int64_t(bx) * g.bdim[1] + by) * g.bdim[2] + bz, key);
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// ------------------------------------------------- shared host routines
// Device-wide exclusive scan of uint32 (n elements) into out; total (device
// scalar, may be NULL) receives the sum. Uses the grid's reduce scratch.
int scan_exclusive_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* total,
                       uint32_t** partial, size_t* partial_cap, cudaStream_t st);
// Same with the element count on the device (n_dev, clamped to n_max); the
// launch is sized from n_max, the work from *n_dev.
int scan_exclusive_u32_dev(const uint32_t* in, uint32_t* out, int64_t n_max,
                           const uint32_t* n_dev, uint32_t* total, uint32_t** partial,
                           size_t* partial_cap, cudaStream_t st);

// Stable LSD radix sort of (key,val) pairs, low `key_bits` bits of the keys,
// input in rs.keys[0] (and rs.vals[0] unless iota_vals, in which case the
// payload is the input index). Result ends in rs.keys[*out_buf], rs.vals[*out_buf].
// Both sorts clear a status word in rs.hist and point *status at it (when
// given): nonzero after the sort means a bounded look-back wait gave up, the
// order is wrong, and the kernels that take the status skip their work.
int radix_sort_pairs(ReduceScratch& rs, int64_t n, int key_bits, bool iota_vals, int* out_buf,
                     cudaStream_t st, uint32_t** status = nullptr);
int radix_sort_pairs_dev(ReduceScratch& rs, int64_t n_max, const uint32_t* n_dev, int key_bits,
                         bool iota_vals, int* out_buf, cudaStream_t st, uint32_t** status = nullptr);
// Test hooks of the bounded device waits (pvdb_debug_wait_limit): the spin
// limit of the look-back waits (0 = the built-in limit), whether the first
// publisher of a look-back chain withholds its count, and whether the first
// block of the staged density pass issues no leaf copies.
uint32_t debug_spin_limit(uint32_t builtin);
int debug_hold_first();
int debug_hold_staging();
// Reads a device status word back (the stream is synchronised) and maps a
// nonzero value to PVDB_ERR_TIMEOUT with the given message.
int read_wait_status(const uint32_t* status, cudaStream_t st, const char* what);
// Scratch words (rs.hist) the sort needs for n_max keys of key_bits bits.
int radix_sort_words(int64_t n_max, int key_bits);

int scratch_reserve(ReduceScratch& rs, int64_t n);
void free_scratch(ReduceScratch& rs);
int num_sms();
// rgbnet X tiles of the tensor-core path: per 128 rows one [128][48] BF16 tile
// in the canonical no-swizzle K-major layout, a row = [k0 | PE | 1 | 0].
constexpr int kRgbXK = 48;
constexpr uint32_t kRgbXTile = 128 * kRgbXK * 2;

// Ensure the reduce scratch of g can hold n contributions.
int reduce_reserve(pvdb_grid_s* g, int64_t n);

// Stage profiler (prof.cu): mark i records an event after stage i of a call.
constexpr int kProfMarks = 16;
void prof_begin_call();
void prof_mark(cudaStream_t st, int id);

// Launch helpers shared by the train step.
float adam_step_size(float lr, float beta_m, float beta_v, int step);
int adam_dense_launch(float* param, const float* grad, float* m, float* v, const float* perlr,
                      int64_t n, float stepsz, float b1, float b2, float eps, int mode,
                      cudaStream_t st, const float* stepsz_dev = nullptr);
// Launch-counter value (every library kernel launch adds one).
uint64_t launch_counter();

// Allocates (once) and rebuilds the brick bound of a scalar grid if invalid.
int bmax_ensure(pvdb_grid_s* g, cudaStream_t st);
// Allocates (once) and rebuilds the BF16 shadow of a grid's values if invalid.
int half_ensure(pvdb_grid_s* g, cudaStream_t st);
// The TV terms k_tv / k_tv_c12 would add in sparse mode, into g->d_tv, for the
// active voxels of the grid's touched leaves (the touched list must be
// current); weights as pvdb_grid_tv_add_grad's.
int tv_terms_launch(pvdb_grid_s* g, float wx, float wy, float wz, cudaStream_t st);
// Marks the grid's derived data (brick bound, BF16 shadow) stale after a
// write of its values that the library does not track.
inline void data_written(pvdb_grid_s* g) {
  g->bmax_valid = false;
  g->half_valid = false;
}

// Compacts the touched flags of g into g->d_tlist / d_tcount unless the list
// is still valid (device work on st, no host synchronisation).
int touched_list(pvdb_grid_s* g, cudaStream_t st);

// Fixed grid for grid-stride kernels whose work size lives on the device.
inline int stride_grid() { return num_sms() * 8; }

// Programmatic dependent launch. Kernels launched by launch_k on a stream
// that is not being captured may be scheduled while the kernel before them
// in the stream is still running, so that a dependent kernel's launch
// overlaps its predecessor's tail instead of following its completion (the
// eager steps are chains of dependent kernels). Every kernel of the library
// starts with grid_dep_sync(): it waits until the preceding kernel has
// completed and its writes are visible (a no-op for a kernel launched
// without the attribute), then allows the kernel after it to be scheduled.
// So nothing a kernel reads or writes overlaps its predecessor; only the
// launch does. Captured graphs keep plain edges: their kernel nodes launch
// back to back already, and early-scheduled blocks waiting on one branch
// measured slower beside the step's parallel branches.
__device__ __forceinline__ void grid_dep_sync() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
inline void launch_k(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                     cudaStream_t st, Args&&... args) {
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  (void)cudaStreamIsCapturing(st, &cap);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = cap == cudaStreamCaptureStatusNone ? 1 : 0;
  // an error is left for the PVDB_CHECK_LAUNCH that follows every launch
  (void)cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Number of key bits needed so that all slots and the invalid key sort apart.
int slot_key_bits(int64_t nslots);

}  // namespace pvdb
