// Leaf store: creation, dense copies, trilinear sampling, lookups, TV, zero_grad,
// save/load. Reference semantics: plenvdb/lib/vdb/plenvdb.h:89-303 (GridType),
// :389-602 (VDBType), densityvdb.cu / colorvdb.cu kernels, NanoVDB accessor
// rules (nanovdb/NanoVDB.h:2999-3010 background outside the tree, :4626-4674
// getValue/isActive, :3893-3899 CoordToOffset).
#include <algorithm>
#include <array>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>

#include "pvdb_internal.cuh"
#include "tc.cuh"

namespace pvdb {

// ------------------------------------------------------------------ errors
namespace {
thread_local int g_err_code = PVDB_OK;
thread_local std::string g_err_msg;
std::mutex g_fail_mu;
int g_fail_allocs = 0;
}  // namespace

int set_error(int code, const std::string& msg) {
  g_err_code = code;
  g_err_msg = msg;
  return code;
}
int cuda_error(cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return set_error(e == cudaErrorMemoryAllocation ? PVDB_ERR_NOMEM : PVDB_ERR_CUDA, m);
}
void clear_error() {
  g_err_code = PVDB_OK;
  g_err_msg.clear();
}

int dev_alloc(void** p, size_t bytes) {
  {
    std::lock_guard<std::mutex> lk(g_fail_mu);
    if (g_fail_allocs > 0) {
      --g_fail_allocs;
      *p = nullptr;
      return set_error(PVDB_ERR_NOMEM, "device allocation failed (injected)");
    }
  }
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_error(e, "cudaMalloc");
  }
  return PVDB_OK;
}
void dev_free(void* p) {
  if (p) cudaFree(p);
}
int dev_reserve(void** p, size_t* cap, size_t bytes) {
  if (*p && *cap >= bytes) return PVDB_OK;
  dev_free(*p);
  *p = nullptr;
  *cap = 0;
  size_t want = std::max<size_t>(bytes, 256);
  int rc = dev_alloc(p, want);
  if (rc) return rc;
  *cap = want;
  return PVDB_OK;
}

// ------------------------------------------------------------------ kernels
__global__ void k_fill(float* p, int64_t n, float v) {
  grid_dep_sync();
  int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i < n) p[i] = v;
}

__device__ __forceinline__ bool is_active(const GridView& g, int leaf, int vox) {
  return (__ldg(g.mask + leaf * 8 + (vox >> 6)) >> (vox & 63)) & 1ull;
}

__device__ __forceinline__ void slot_coord(const GridView& g, int leaf, int vox, int& x, int& y,
                                           int& z) {
  x = __ldg(g.origin + leaf * 3 + 0) + (vox >> 6);
  y = __ldg(g.origin + leaf * 3 + 1) + ((vox >> 3) & 7);
  z = __ldg(g.origin + leaf * 3 + 2) + (vox & 7);
}

// Slots of the 6 face neighbours of voxel (x, y, z) = (leaf, vox), in the order
// -z, +z, -y, +y, -x, +x: -2 outside [0, reso) (no TV term), -1 in no
// allocated leaf (background). A neighbour inside the voxel's own leaf follows
// from the offset layout (+64 x, +8 y, +1 z) without a table lookup.
__device__ __forceinline__ void face_neighbours(const GridView& g, int leaf, int vox, int x, int y,
                                                int z, int nb[6]) {
  const int base = leaf << 9;
  const int lx = vox >> 6, ly = (vox >> 3) & 7, lz = vox & 7;
  nb[0] = z == 0 ? -2 : lz > 0 ? base | (vox - 1) : slot_of(g, x, y, z - 1);
  nb[1] = z == g.reso[2] - 1 ? -2 : lz < 7 ? base | (vox + 1) : slot_of(g, x, y, z + 1);
  nb[2] = y == 0 ? -2 : ly > 0 ? base | (vox - 8) : slot_of(g, x, y - 1, z);
  nb[3] = y == g.reso[1] - 1 ? -2 : ly < 7 ? base | (vox + 8) : slot_of(g, x, y + 1, z);
  nb[4] = x == 0 ? -2 : lx > 0 ? base | (vox - 64) : slot_of(g, x - 1, y, z);
  nb[5] = x == g.reso[0] - 1 ? -2 : lx < 7 ? base | (vox + 64) : slot_of(g, x + 1, y, z);
}

// copyFromDense: active voxels only (densityvdb.cu:39-48, colorvdb.cu:52-62).
__global__ void k_copy_from_dense(GridView g, float* dst, const float* __restrict__ arr, int rx,
                                  int ry, int rz) {
  grid_dep_sync();
  int64_t n = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (n >= int64_t(g.nleaf) * kLeafVox) return;
  const int leaf = int(n >> 9), vox = int(n & 511);
  if (!is_active(g, leaf, vox)) return;
  int x, y, z;
  slot_coord(g, leaf, vox, x, y, z);
  if (x >= rx || y >= ry || z >= rz) return;
  const int64_t src = ((int64_t(x) * ry + y) * rz + z) * g.C;
  for (int c = 0; c < g.C; ++c) dst[n * g.C + c] = arr[src + c];
}

// copyToDense: every voxel of [0,reso) gets its stored or background value.
__global__ void k_copy_to_dense(GridView g, const float* __restrict__ src, float* out, int rx,
                                int ry, int rz, float bg) {
  grid_dep_sync();
  int64_t n = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (n >= int64_t(rx) * ry * rz) return;
  const int z = int(n % rz), y = int((n / rz) % ry), x = int(n / (int64_t(ry) * rz));
  const int s = slot_of(g, x, y, z);
  for (int c = 0; c < g.C; ++c) out[n * g.C + c] = s < 0 ? bg : src[int64_t(s) * g.C + c];
}

__global__ void k_set_by_mask(GridView g, const uint8_t* __restrict__ mask, float val, int rx,
                              int ry, int rz) {
  grid_dep_sync();
  int64_t n = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (n >= int64_t(g.nleaf) * kLeafVox) return;
  const int leaf = int(n >> 9), vox = int(n & 511);
  if (!is_active(g, leaf, vox)) return;
  int x, y, z;
  slot_coord(g, leaf, vox, x, y, z);
  if (x >= rx || y >= ry || z >= rz) return;
  if (mask[(int64_t(x) * ry + y) * rz + z])
    for (int c = 0; c < g.C; ++c) g.data[n * g.C + c] = val;
}

__global__ void k_sample1(GridView g, const float* __restrict__ xs, const float* __restrict__ ys,
                          const float* __restrict__ zs, int64_t n, float* out) {
  grid_dep_sync();
  int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= n) return;
  out[p] = trilinear1(g, xs[p], ys[p], zs[p]);
}

// Multi-channel trilinear (colorvdb.cu:81-111): per corner the scale is formed
// first, then out[c] += value[c]*scale in corner order.
__global__ void k_sampleC(GridView g, const float* __restrict__ xs, const float* __restrict__ ys,
                          const float* __restrict__ zs, int64_t n, float* out) {
  grid_dep_sync();
  int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= n) return;
  const float x = xs[p], y = ys[p], z = zs[p];
  const int i = ifloor(x), j = ifloor(y), k = ifloor(z);
  float sc[8];
  corner_scales(x - float(i), y - float(j), z - float(k), sc);
  int slots[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    int di, dj, dk;
    corner_delta(c, di, dj, dk);
    slots[c] = slot_of(g, i + di, j + dj, k + dk);
  }
  for (int ch = 0; ch < g.C; ++ch) {
    float r = 0.f;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const float v = slots[c] < 0 ? g.background : __ldg(g.data + int64_t(slots[c]) * g.C + ch);
      r = __fadd_rn(r, __fmul_rn(v, sc[c]));
    }
    out[p * g.C + ch] = r;
  }
}

__global__ void k_lookup(GridView g, const int32_t* __restrict__ is, const int32_t* __restrict__ js,
                         const int32_t* __restrict__ ks, int64_t n, float* out, uint8_t* act) {
  grid_dep_sync();
  int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= n) return;
  const int i = is[p], j = js[p], k = ks[p];
  const int l = leaf_of(g, i, j, k);
  const int vox = vox_offset(i, j, k);
  for (int c = 0; c < g.C; ++c)
    out[p * g.C + c] = l < 0 ? g.background : g.data[(int64_t(l) * kLeafVox + vox) * g.C + c];
  if (act) act[p] = l < 0 ? 0 : (uint8_t)is_active(g, l, vox);
}

__global__ void k_zero_grad(GridView g, const uint8_t* __restrict__ touched) {
  grid_dep_sync();
  int64_t n = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (n >= int64_t(g.nleaf) * kLeafVox) return;
  const int leaf = int(n >> 9), vox = int(n & 511);
  if (touched && !touched[leaf]) return;
  if (!is_active(g, leaf, vox)) return;
  for (int c = 0; c < g.C; ++c) g.grad[n * g.C + c] = 0.f;
}

__global__ void k_clear_touched(uint8_t* t, int n) {
  grid_dep_sync();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) t[i] = 0;
}

__device__ __forceinline__ float tv_clamp(float v) { return fminf(fmaxf(v, -1.f), 1.f); }

__device__ __forceinline__ float value_c(const GridView& g, int i, int j, int k, int ch) {
  const int s = slot_of(g, i, j, k);
  return s < 0 ? g.background : g.data[int64_t(s) * g.C + ch];
}

// TV gradient (total_variation_kernel.cu:13-35) on the leaf store, for the
// voxels of the listed leaves (list = NULL: all leaves). One thread per voxel:
// the six neighbour slots are looked up once and shared by the channels;
// neighbours inside [0,reso) only, values through the leaf table (background
// outside allocated leaves). Per channel the sum is formed in the reference's
// order z-, z+, y-, y+, x-, x+.
__global__ void k_tv(GridView g, float wx, float wy, float wz, int dense_mode,
                     const int32_t* __restrict__ list, const uint32_t* __restrict__ count) {
  grid_dep_sync();
  const int64_t nl = list ? int64_t(*count) : int64_t(g.nleaf);
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < nl * kLeafVox;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int leaf = list ? list[i >> 9] : int(i >> 9);
    const int vox = int(i & 511);
    if (!is_active(g, leaf, vox)) continue;
    int x, y, z;
    slot_coord(g, leaf, vox, x, y, z);
    if (x >= g.reso[0] || y >= g.reso[1] || z >= g.reso[2]) continue;
    int nb[6];
    face_neighbours(g, leaf, vox, x, y, z, nb);
    const float wt[6] = {wz, wz, wy, wy, wx, wx};
    const int64_t t0 = (int64_t(leaf) * kLeafVox + vox) * g.C;
    for (int ch = 0; ch < g.C; ++ch) {
      const float gcur = g.grad[t0 + ch];
      if (!dense_mode && gcur == 0.f) continue;
      const float p = g.data[t0 + ch];
      float add = 0.f;
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        if (nb[q] == -2) {
          add += 0.f;
        } else {
          const float vn = nb[q] < 0 ? g.background : g.data[int64_t(nb[q]) * g.C + ch];
          // each term rounded, then added (the reference's conditional terms
          // are not fused, total_variation_kernel.cu:27-32)
          add = __fadd_rn(add, __fmul_rn(wt[q], tv_clamp(p - vn)));
        }
      }
      g.grad[t0 + ch] = gcur + add;
    }
  }
}

// Brick bound from scratch: one thread per brick, the max over the 7^3
// voxels [4b-1, 4b+5] (background outside allocated leaves).
__global__ void k_bmax_init(GridView g, uint32_t* bmax) {
  grid_dep_sync();
  const int64_t nb = int64_t(g.bdim[0]) * g.bdim[1] * g.bdim[2];
  for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < nb;
       t += int64_t(gridDim.x) * blockDim.x) {
    const int bz = int(t % g.bdim[2]), by = int((t / g.bdim[2]) % g.bdim[1]),
              bx = int(t / (int64_t(g.bdim[2]) * g.bdim[1]));
    float m = -INFINITY;
    for (int x = 4 * bx - 1; x <= 4 * bx + 5; ++x)
      for (int y = 4 * by - 1; y <= 4 * by + 5; ++y)
        for (int z = 4 * bz - 1; z <= 4 * bz + 5; ++z) {
          const float v = value1(g, x, y, z);
          m = (v > m || v != v) ? v : m;
        }
    bmax[t] = fkey(m);
  }
}

// k_tv for 12-channel grids: the voxel's and its neighbours' channels in
// float4 loads; per-channel arithmetic and order as k_tv.
__global__ void k_tv_c12(GridView g, float wx, float wy, float wz, int dense_mode,
                         const int32_t* __restrict__ list, const uint32_t* __restrict__ count) {
  grid_dep_sync();
  const int64_t nl = list ? int64_t(*count) : int64_t(g.nleaf);
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < nl * kLeafVox;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int leaf = list ? list[i >> 9] : int(i >> 9);
    const int vox = int(i & 511);
    if (!is_active(g, leaf, vox)) continue;
    const int64_t t0 = (int64_t(leaf) * kLeafVox + vox) * 12;
    float4* g4 = reinterpret_cast<float4*>(g.grad + t0);
    float gc[12];
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const float4 x = g4[b];
      gc[4 * b] = x.x; gc[4 * b + 1] = x.y; gc[4 * b + 2] = x.z; gc[4 * b + 3] = x.w;
    }
    bool any = dense_mode != 0;
#pragma unroll
    for (int ch = 0; ch < 12; ++ch) any = any || gc[ch] != 0.f;
    if (!any) continue;
    int x, y, z;
    slot_coord(g, leaf, vox, x, y, z);
    if (x >= g.reso[0] || y >= g.reso[1] || z >= g.reso[2]) continue;
    int nb[6];
    face_neighbours(g, leaf, vox, x, y, z, nb);
    const float wt[6] = {wz, wz, wy, wy, wx, wx};
    float p[12], add[12];
    const float4* d4 = reinterpret_cast<const float4*>(g.data + t0);
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const float4 v = d4[b];
      p[4 * b] = v.x; p[4 * b + 1] = v.y; p[4 * b + 2] = v.z; p[4 * b + 3] = v.w;
    }
#pragma unroll
    for (int ch = 0; ch < 12; ++ch) add[ch] = 0.f;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      if (nb[q] == -2) continue;  // (adding 0.f leaves the sum as it is)
      float vn[12];
      if (nb[q] < 0) {
#pragma unroll
        for (int ch = 0; ch < 12; ++ch) vn[ch] = g.background;
      } else {
        const float4* n4 = reinterpret_cast<const float4*>(g.data + int64_t(nb[q]) * 12);
#pragma unroll
        for (int b = 0; b < 3; ++b) {
          const float4 v = n4[b];
          vn[4 * b] = v.x; vn[4 * b + 1] = v.y; vn[4 * b + 2] = v.z; vn[4 * b + 3] = v.w;
        }
      }
#pragma unroll
      for (int ch = 0; ch < 12; ++ch)
        add[ch] = __fadd_rn(add[ch], __fmul_rn(wt[q], tv_clamp(p[ch] - vn[ch])));
    }
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      float o[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int ch = 4 * b + e;
        o[e] = (!dense_mode && gc[ch] == 0.f) ? gc[ch] : gc[ch] + add[ch];
      }
      g4[b] = make_float4(o[0], o[1], o[2], o[3]);
    }
  }
}

// The TV sums of k_tv / k_tv_c12 (same neighbours, order and rounding)
// without the gradient: tv[slot*C + ch] for every active voxel of the listed
// leaves (0 outside [0, reso)). In sparse mode k_tv adds them to the channels
// whose gradient is nonzero; the fused step's voxel Adam does that addition
// instead, so this pass needs only the values and can run beside the
// gradient sums.
__global__ void k_tv_terms(GridView g, float wx, float wy, float wz,
                           const int32_t* __restrict__ list, const uint32_t* __restrict__ count,
                           float* __restrict__ tv) {
  grid_dep_sync();
  const int64_t nl = *count;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < nl * kLeafVox;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int leaf = list[i >> 9];
    const int vox = int(i & 511);
    if (!is_active(g, leaf, vox)) continue;
    const int64_t t0 = (int64_t(leaf) * kLeafVox + vox) * g.C;
    int x, y, z;
    slot_coord(g, leaf, vox, x, y, z);
    if (x >= g.reso[0] || y >= g.reso[1] || z >= g.reso[2]) {
      for (int ch = 0; ch < g.C; ++ch) tv[t0 + ch] = 0.f;
      continue;
    }
    int nb[6];
    face_neighbours(g, leaf, vox, x, y, z, nb);
    const float wt[6] = {wz, wz, wy, wy, wx, wx};
    for (int ch = 0; ch < g.C; ++ch) {
      const float p = g.data[t0 + ch];
      float add = 0.f;
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        if (nb[q] == -2) continue;
        const float vn = nb[q] < 0 ? g.background : g.data[int64_t(nb[q]) * g.C + ch];
        add = __fadd_rn(add, __fmul_rn(wt[q], tv_clamp(p - vn)));
      }
      tv[t0 + ch] = add;
    }
  }
}

__global__ void k_tv_terms_c12(GridView g, float wx, float wy, float wz,
                               const int32_t* __restrict__ list,
                               const uint32_t* __restrict__ count, float* __restrict__ tv) {
  grid_dep_sync();
  const int64_t nl = *count;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < nl * kLeafVox;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int leaf = list[i >> 9];
    const int vox = int(i & 511);
    if (!is_active(g, leaf, vox)) continue;
    const int64_t t0 = (int64_t(leaf) * kLeafVox + vox) * 12;
    float4* o4 = reinterpret_cast<float4*>(tv + t0);
    int x, y, z;
    slot_coord(g, leaf, vox, x, y, z);
    if (x >= g.reso[0] || y >= g.reso[1] || z >= g.reso[2]) {
#pragma unroll
      for (int b = 0; b < 3; ++b) o4[b] = make_float4(0.f, 0.f, 0.f, 0.f);
      continue;
    }
    int nb[6];
    face_neighbours(g, leaf, vox, x, y, z, nb);
    const float wt[6] = {wz, wz, wy, wy, wx, wx};
    float p[12], add[12];
    const float4* d4 = reinterpret_cast<const float4*>(g.data + t0);
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const float4 v = d4[b];
      p[4 * b] = v.x; p[4 * b + 1] = v.y; p[4 * b + 2] = v.z; p[4 * b + 3] = v.w;
    }
#pragma unroll
    for (int ch = 0; ch < 12; ++ch) add[ch] = 0.f;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      if (nb[q] == -2) continue;
      float vn[12];
      if (nb[q] < 0) {
#pragma unroll
        for (int ch = 0; ch < 12; ++ch) vn[ch] = g.background;
      } else {
        const float4* n4 = reinterpret_cast<const float4*>(g.data + int64_t(nb[q]) * 12);
#pragma unroll
        for (int b = 0; b < 3; ++b) {
          const float4 v = n4[b];
          vn[4 * b] = v.x; vn[4 * b + 1] = v.y; vn[4 * b + 2] = v.z; vn[4 * b + 3] = v.w;
        }
      }
#pragma unroll
      for (int ch = 0; ch < 12; ++ch)
        add[ch] = __fadd_rn(add[ch], __fmul_rn(wt[q], tv_clamp(p[ch] - vn[ch])));
    }
#pragma unroll
    for (int b = 0; b < 3; ++b)
      o4[b] = make_float4(add[4 * b], add[4 * b + 1], add[4 * b + 2], add[4 * b + 3]);
  }
}

__global__ void k_touched_compact(const uint8_t* __restrict__ touched, int nleaf, int32_t* list,
                                  uint32_t* count) {
  grid_dep_sync();
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l < nleaf && touched[l]) list[atomicAdd(count, 1u)] = l;
}

// ---------------------------------------------------------------- helpers
static uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
  auto spread = [](uint32_t v) {
    v &= 0x3ff;
    v = (v | (v << 16)) & 0x030000FF;
    v = (v | (v << 8)) & 0x0300F00F;
    v = (v | (v << 4)) & 0x030C30C3;
    v = (v | (v << 2)) & 0x09249249;
    return v;
  };
  return (spread(x) << 2) | (spread(y) << 1) | spread(z);
}

// Builds the topology of a grid from a per-leaf "allocated" list and active
// masks (host), uploads it, and fills values with the background.
static int build_grid(const int reso[3], int C, float bg,
                      const std::vector<std::array<int, 3>>& leaves,
                      const std::vector<std::array<uint64_t, 8>>& masks, pvdb_grid_s** out) {
  pvdb_grid_s* g = new pvdb_grid_s();
  for (int a = 0; a < 3; ++a) {
    g->reso[a] = reso[a];
    g->ldim[a] = (reso[a] + 7) / 8;
  }
  g->C = C;
  g->background = bg;
  g->nleaf = int(leaves.size());
  // Morton order of leaves.
  std::vector<int> order(leaves.size());
  std::iota(order.begin(), order.end(), 0);
  std::vector<uint32_t> codes(leaves.size());
  for (size_t i = 0; i < leaves.size(); ++i)
    codes[i] = morton3(leaves[i][0], leaves[i][1], leaves[i][2]);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return codes[a] < codes[b]; });
  const int64_t ntab = int64_t(g->ldim[0]) * g->ldim[1] * g->ldim[2];
  g->h_table.assign(ntab, -1);
  g->h_origin.resize(size_t(g->nleaf) * 3);
  g->h_mask.resize(size_t(g->nleaf) * 8);
  int64_t nact = 0;
  for (int id = 0; id < g->nleaf; ++id) {
    const auto& L = leaves[order[id]];
    g->h_table[(int64_t(L[0]) * g->ldim[1] + L[1]) * g->ldim[2] + L[2]] = id;
    for (int a = 0; a < 3; ++a) g->h_origin[id * 3 + a] = L[a] * 8;
    for (int w = 0; w < 8; ++w) {
      g->h_mask[id * 8 + w] = masks[order[id]][w];
      nact += __builtin_popcountll(masks[order[id]][w]);
    }
  }
  g->nactive = nact;
  int rc = PVDB_OK;
  const size_t nval = size_t(g->nleaf) * kLeafVox * C;
  if ((rc = dev_alloc((void**)&g->d_table, ntab * sizeof(int32_t))) ||
      (rc = dev_alloc((void**)&g->d_origin, std::max<size_t>(1, g->h_origin.size()) * 4)) ||
      (rc = dev_alloc((void**)&g->d_mask, std::max<size_t>(1, g->h_mask.size()) * 8)) ||
      (rc = dev_alloc((void**)&g->d_data, std::max<size_t>(1, nval) * 4)) ||
      (rc = dev_alloc((void**)&g->d_grad, std::max<size_t>(1, nval) * 4)) ||
      (rc = dev_alloc((void**)&g->d_touched, std::max(1, g->nleaf))) ||
      (rc = dev_alloc((void**)&g->d_tlist, std::max<size_t>(1, g->nleaf) * 4)) ||
      (rc = dev_alloc((void**)&g->d_tcount, 16))) {
    pvdb_grid_destroy(g);
    return rc;
  }
  cudaError_t e;
  if ((e = cudaMemcpy(g->d_table, g->h_table.data(), ntab * 4, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(g->d_origin, g->h_origin.data(), g->h_origin.size() * 4,
                      cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(g->d_mask, g->h_mask.data(), g->h_mask.size() * 8,
                      cudaMemcpyHostToDevice)) ||
      (e = cudaMemset(g->d_grad, 0, nval * 4)) ||
      (e = cudaMemset(g->d_touched, 0, std::max(1, g->nleaf)))) {
    pvdb_grid_destroy(g);
    return cuda_error(e, "grid upload");
  }
  if (nval) {
    launch_k(k_fill, ceil_div(nval, 256), 256, 0, 0, g->d_data, nval, bg);
    if ((e = cudaGetLastError()) || (e = cudaDeviceSynchronize())) {
      pvdb_grid_destroy(g);
      return cuda_error(e, "grid fill");
    }
  }
  g->all_touched = false;
  *out = g;
  return PVDB_OK;
}

// Host staging: copy `n` host bytes into the grid's device stage at `offset`.
static int stage_reserve(pvdb_grid_s* g, size_t bytes) {
  return dev_reserve(&g->d_stage, &g->stage_cap, bytes);
}

int touched_list(pvdb_grid_s* g, cudaStream_t st) {
  if (g->tlist_valid) return PVDB_OK;
  PVDB_CHECK_CUDA(cudaMemsetAsync(g->d_tcount, 0, 4, st));
  if (g->nleaf) {
    launch_k(k_touched_compact, ceil_div(g->nleaf, 256), 256, 0, st, g->d_touched, g->nleaf,
             g->d_tlist, g->d_tcount);
    PVDB_CHECK_LAUNCH("k_touched_compact");
  }
  g->tlist_valid = true;
  return PVDB_OK;
}

int bmax_ensure(pvdb_grid_s* g, cudaStream_t st) {
  if (g->C != 1) return set_error(PVDB_ERR_ARG, "brick bounds are for scalar grids");
  if (g->bmax_valid) return PVDB_OK;
  if (!g->d_bmax) {
    for (int a = 0; a < 3; ++a) g->bdim[a] = (g->reso[a] + 3) / 4;
    const size_t nb = size_t(g->bdim[0]) * g->bdim[1] * g->bdim[2];
    int rc = dev_alloc((void**)&g->d_bmax, std::max<size_t>(nb, 1) * 4);
    if (rc) return rc;
  }
  GridView v = g->view();
  launch_k(k_bmax_init, stride_grid(), 256, 0, st, v, g->d_bmax);
  PVDB_CHECK_LAUNCH("k_bmax_init");
  g->bmax_valid = true;
  return PVDB_OK;
}

// BF16 copy of a 12-channel grid's values (round to nearest even), one voxel a
// thread: 32 bytes per voxel, channels 0..11 then four zeros, so that a voxel
// is one aligned 32-byte sector and two 16-byte loads.
__global__ void k_half_build(const float* __restrict__ src, __nv_bfloat16* dst, int64_t nvox) {
  grid_dep_sync();
  const int64_t v = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (v >= nvox) return;
  const float4* s4 = reinterpret_cast<const float4*>(src + v * 12);
  const float4 a = __ldg(s4), b = __ldg(s4 + 1), c = __ldg(s4 + 2);
  uint4* d4 = reinterpret_cast<uint4*>(dst + v * kHalfStride);
  d4[0] = make_uint4(tc::pack_bf16(a.x, a.y), tc::pack_bf16(a.z, a.w), tc::pack_bf16(b.x, b.y),
                     tc::pack_bf16(b.z, b.w));
  d4[1] = make_uint4(tc::pack_bf16(c.x, c.y), tc::pack_bf16(c.z, c.w), 0u, 0u);
}

int tv_terms_launch(pvdb_grid_s* g, float wx, float wy, float wz, cudaStream_t st) {
  if (g->nslots() == 0) return PVDB_OK;
  if (!g->tlist_valid) return set_error(PVDB_ERR_STATE, "TV terms: the touched list is stale");
  if (!g->d_tv) {
    const int rc = dev_alloc((void**)&g->d_tv, size_t(g->nslots()) * g->C * 4);
    if (rc) return rc;
  }
  // the reference divides the weights by 6 on the host (total_variation_kernel.cu:45-47)
  wx /= 6.f;
  wy /= 6.f;
  wz /= 6.f;
  if (g->C == 12)
    launch_k(k_tv_terms_c12, stride_grid(), 256, 0, st, g->view(), wx, wy, wz, g->d_tlist,
             g->d_tcount, g->d_tv);
  else
    launch_k(k_tv_terms, stride_grid(), 256, 0, st, g->view(), wx, wy, wz, g->d_tlist, g->d_tcount,
             g->d_tv);
  PVDB_CHECK_LAUNCH("k_tv_terms");
  return PVDB_OK;
}

int half_ensure(pvdb_grid_s* g, cudaStream_t st) {
  if (g->C != 12) return set_error(PVDB_ERR_STATE, "the BF16 feature shadow is kept for 12 channels");
  const int64_t nvox = g->nslots();
  if (!g->d_half) {
    int rc = dev_alloc((void**)&g->d_half, size_t(std::max<int64_t>(nvox, 1)) * kHalfStride * 2);
    if (rc) return rc;
    g->half_valid = false;
  }
  if (g->half_valid) return PVDB_OK;
  if (nvox) {
    launch_k(k_half_build, ceil_div(nvox, 256), 256, 0, st, g->d_data, g->d_half, nvox);
    PVDB_CHECK_LAUNCH("k_half_build");
  }
  g->half_valid = true;
  return PVDB_OK;
}

}  // namespace pvdb

using namespace pvdb;

// ===================================================================== C ABI
extern "C" {

const char* pvdb_version(void) { return "plenvdb-gb300 0.1 (sm_103a)"; }

int pvdb_last_error(char* buf, size_t len) {
  if (buf && len) {
    size_t n = std::min(len - 1, g_err_msg.size());
    std::memcpy(buf, g_err_msg.data(), n);
    buf[n] = 0;
  }
  return g_err_code;
}

int pvdb_debug_fail_next_allocs(int count) {
  std::lock_guard<std::mutex> lk(g_fail_mu);
  g_fail_allocs = std::max(0, count);
  return PVDB_OK;
}

int pvdb_grid_create(const int32_t reso[3], int32_t channels, float background, pvdb_grid* out) {
  clear_error();
  PVDB_REQUIRE(reso && out, "null argument");
  PVDB_REQUIRE(channels == 1 || (channels > 0 && channels % 3 == 0),
               "channels must be 1 or a positive multiple of 3");
  for (int a = 0; a < 3; ++a) PVDB_REQUIRE(reso[a] > 0 && reso[a] <= 8192, "bad resolution");
  int ld[3];
  for (int a = 0; a < 3; ++a) ld[a] = (reso[a] + 7) / 8;
  std::vector<std::array<int, 3>> leaves;
  std::vector<std::array<uint64_t, 8>> masks;
  leaves.reserve(size_t(ld[0]) * ld[1] * ld[2]);
  for (int x = 0; x < ld[0]; ++x)
    for (int y = 0; y < ld[1]; ++y)
      for (int z = 0; z < ld[2]; ++z) {
        leaves.push_back({x, y, z});
        std::array<uint64_t, 8> m{};
        for (int v = 0; v < 512; ++v) {
          const int vx = x * 8 + (v >> 6), vy = y * 8 + ((v >> 3) & 7), vz = z * 8 + (v & 7);
          if (vx < reso[0] && vy < reso[1] && vz < reso[2]) m[v >> 6] |= 1ull << (v & 63);
        }
        masks.push_back(m);
      }
  pvdb_grid_s* g = nullptr;
  int rc = build_grid(reso, channels, background, leaves, masks, &g);
  if (rc) return rc;
  *out = g;
  return PVDB_OK;
}

int pvdb_grid_create_from_mask(const int32_t reso[3], int32_t channels, float background,
                               const uint8_t* active, int32_t mem, pvdb_grid* out) {
  clear_error();
  PVDB_REQUIRE(reso && out && active, "null argument");
  PVDB_REQUIRE(channels == 1 || (channels > 0 && channels % 3 == 0),
               "channels must be 1 or a positive multiple of 3");
  for (int a = 0; a < 3; ++a) PVDB_REQUIRE(reso[a] > 0 && reso[a] <= 8192, "bad resolution");
  const int64_t nvox = int64_t(reso[0]) * reso[1] * reso[2];
  std::vector<uint8_t> host;
  const uint8_t* act = active;
  if (mem == PVDB_MEM_DEVICE) {
    host.resize(nvox);
    PVDB_CHECK_CUDA(cudaMemcpy(host.data(), active, nvox, cudaMemcpyDeviceToHost));
    act = host.data();
  }
  int ld[3];
  for (int a = 0; a < 3; ++a) ld[a] = (reso[a] + 7) / 8;
  std::vector<std::array<uint64_t, 8>> lm(size_t(ld[0]) * ld[1] * ld[2]);
  std::vector<uint8_t> any(lm.size(), 0);
  for (int x = 0; x < reso[0]; ++x)
    for (int y = 0; y < reso[1]; ++y)
      for (int z = 0; z < reso[2]; ++z) {
        if (!act[(int64_t(x) * reso[1] + y) * reso[2] + z]) continue;
        const int64_t li = (int64_t(x >> 3) * ld[1] + (y >> 3)) * ld[2] + (z >> 3);
        const int v = ((x & 7) << 6) | ((y & 7) << 3) | (z & 7);
        lm[li][v >> 6] |= 1ull << (v & 63);
        any[li] = 1;
      }
  std::vector<std::array<int, 3>> leaves;
  std::vector<std::array<uint64_t, 8>> masks;
  for (int x = 0; x < ld[0]; ++x)
    for (int y = 0; y < ld[1]; ++y)
      for (int z = 0; z < ld[2]; ++z) {
        const int64_t li = (int64_t(x) * ld[1] + y) * ld[2] + z;
        if (!any[li]) continue;
        leaves.push_back({x, y, z});
        masks.push_back(lm[li]);
      }
  pvdb_grid_s* g = nullptr;
  int rc = build_grid(reso, channels, background, leaves, masks, &g);
  if (rc) return rc;
  *out = g;
  return PVDB_OK;
}

int pvdb_grid_create_like(pvdb_grid like, int32_t channels, float background, pvdb_grid* out) {
  clear_error();
  PVDB_REQUIRE(like && out, "null argument");
  PVDB_REQUIRE(channels == 1 || (channels > 0 && channels % 3 == 0),
               "channels must be 1 or a positive multiple of 3");
  std::vector<std::array<int, 3>> leaves(like->nleaf);
  std::vector<std::array<uint64_t, 8>> masks(like->nleaf);
  for (int id = 0; id < like->nleaf; ++id) {
    for (int a = 0; a < 3; ++a) leaves[id][a] = like->h_origin[id * 3 + a] / 8;
    for (int w = 0; w < 8; ++w) masks[id][w] = like->h_mask[id * 8 + w];
  }
  pvdb_grid_s* g = nullptr;
  int rc = build_grid(like->reso, channels, background, leaves, masks, &g);
  if (rc) return rc;
  *out = g;
  return PVDB_OK;
}

int pvdb_grid_destroy(pvdb_grid g) {
  if (!g) return PVDB_OK;
  dev_free(g->d_table);
  dev_free(g->d_origin);
  dev_free(g->d_mask);
  dev_free(g->d_data);
  dev_free(g->d_grad);
  dev_free(g->d_touched);
  dev_free(g->d_tlist);
  dev_free(g->d_tcount);
  dev_free(g->d_bmax);
  dev_free(g->d_half);
  dev_free(g->d_tv);
  dev_free(g->d_stage);
  free_scratch(g->red);
  delete g;
  return PVDB_OK;
}

int pvdb_grid_get_info(pvdb_grid g, int32_t reso[3], int32_t* channels, int32_t* nleaf,
                       int64_t* nactive, float* background) {
  clear_error();
  PVDB_REQUIRE(g, "null grid");
  if (reso)
    for (int a = 0; a < 3; ++a) reso[a] = g->reso[a];
  if (channels) *channels = g->C;
  if (nleaf) *nleaf = g->nleaf;
  if (nactive) *nactive = g->nactive;
  if (background) *background = g->background;
  return PVDB_OK;
}

int pvdb_grid_set_reso(pvdb_grid g, int32_t rx, int32_t ry, int32_t rz) {
  clear_error();
  PVDB_REQUIRE(g, "null grid");
  PVDB_REQUIRE(rx > 0 && ry > 0 && rz > 0, "bad resolution");
  g->reso[0] = rx;
  g->reso[1] = ry;
  g->reso[2] = rz;
  return PVDB_OK;
}

int pvdb_grid_copy_from_dense(pvdb_grid g, int32_t which, const float* arr, int64_t n,
                              int32_t mem, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(g && arr, "null argument");
  PVDB_REQUIRE(which == PVDB_WHICH_DATA || which == PVDB_WHICH_GRAD, "bad `which`");
  const int64_t want = int64_t(g->reso[0]) * g->reso[1] * g->reso[2] * g->C;
  PVDB_REQUIRE(n == want, "dense size must be reso[0]*reso[1]*reso[2]*channels");
  cudaStream_t st = as_stream(s);
  const float* src = arr;
  if (mem == PVDB_MEM_HOST) {
    int rc = stage_reserve(g, n * 4);
    if (rc) return rc;
    PVDB_CHECK_CUDA(cudaMemcpyAsync(g->d_stage, arr, n * 4, cudaMemcpyHostToDevice, st));
    src = (const float*)g->d_stage;
  }
  const int64_t ns = g->nslots();
  if (ns)
    launch_k(k_copy_from_dense, ceil_div(ns, 256), 256, 0, st, g->view(),
             which == PVDB_WHICH_DATA ? g->d_data : g->d_grad, src, g->reso[0], g->reso[1],
             g->reso[2]);
  PVDB_CHECK_LAUNCH("k_copy_from_dense");
  if (which == PVDB_WHICH_GRAD) g->all_touched = true;
  if (which == PVDB_WHICH_DATA) data_written(g);
  if (mem == PVDB_MEM_HOST) PVDB_CHECK_CUDA(cudaStreamSynchronize(st));
  return PVDB_OK;
}

int pvdb_grid_copy_to_dense(pvdb_grid g, int32_t which, float* out, int64_t n, int32_t mem,
                            pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(g && out, "null argument");
  PVDB_REQUIRE(which == PVDB_WHICH_DATA || which == PVDB_WHICH_GRAD, "bad `which`");
  const int64_t nvox = int64_t(g->reso[0]) * g->reso[1] * g->reso[2];
  PVDB_REQUIRE(n == nvox * g->C, "dense size must be reso[0]*reso[1]*reso[2]*channels");
  cudaStream_t st = as_stream(s);
  float* dst = out;
  if (mem == PVDB_MEM_HOST) {
    int rc = stage_reserve(g, n * 4);
    if (rc) return rc;
    dst = (float*)g->d_stage;
  }
  // the gradient of a voxel outside every leaf reads as 0, data as the background
  const float bg = which == PVDB_WHICH_DATA ? g->background : 0.f;
  if (nvox)
    launch_k(k_copy_to_dense, ceil_div(nvox, 256), 256, 0, st, g->view(),
             which == PVDB_WHICH_DATA ? g->d_data : g->d_grad, dst, g->reso[0], g->reso[1],
             g->reso[2], bg);
  PVDB_CHECK_LAUNCH("k_copy_to_dense");
  if (mem == PVDB_MEM_HOST) {
    PVDB_CHECK_CUDA(cudaMemcpyAsync(out, dst, n * 4, cudaMemcpyDeviceToHost, st));
    PVDB_CHECK_CUDA(cudaStreamSynchronize(st));
  }
  return PVDB_OK;
}

int pvdb_grid_set_values_by_mask(pvdb_grid g, const uint8_t* mask, int64_t n, float val,
                                 int32_t mem, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(g && mask, "null argument");
  PVDB_REQUIRE(n == int64_t(g->reso[0]) * g->reso[1] * g->reso[2],
               "mask size must be reso[0]*reso[1]*reso[2]");
  cudaStream_t st = as_stream(s);
  const uint8_t* m = mask;
  if (mem == PVDB_MEM_HOST) {
    int rc = stage_reserve(g, n);
    if (rc) return rc;
    PVDB_CHECK_CUDA(cudaMemcpyAsync(g->d_stage, mask, n, cudaMemcpyHostToDevice, st));
    m = (const uint8_t*)g->d_stage;
  }
  const int64_t ns = g->nslots();
  if (ns)
    launch_k(k_set_by_mask, ceil_div(ns, 256), 256, 0, st, g->view(), m, val, g->reso[0],
             g->reso[1], g->reso[2]);
  PVDB_CHECK_LAUNCH("k_set_by_mask");
  data_written(g);
  if (mem == PVDB_MEM_HOST) PVDB_CHECK_CUDA(cudaStreamSynchronize(st));
  return PVDB_OK;
}

int pvdb_grid_sample(pvdb_grid g, const float* xs, const float* ys, const float* zs, int64_t n,
                     float* out, int32_t mem, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(g, "null grid");
  PVDB_REQUIRE(n >= 0, "negative size");
  if (n == 0) return PVDB_OK;
  PVDB_REQUIRE(xs && ys && zs && out, "null argument");
  cudaStream_t st = as_stream(s);
  const float *dx = xs, *dy = ys, *dz = zs;
  float* dout = out;
  if (mem == PVDB_MEM_HOST) {
    int rc = stage_reserve(g, size_t(n) * 4 * (3 + g->C));
    if (rc) return rc;
    float* b = (float*)g->d_stage;
    PVDB_CHECK_CUDA(cudaMemcpyAsync(b, xs, n * 4, cudaMemcpyHostToDevice, st));
    PVDB_CHECK_CUDA(cudaMemcpyAsync(b + n, ys, n * 4, cudaMemcpyHostToDevice, st));
    PVDB_CHECK_CUDA(cudaMemcpyAsync(b + 2 * n, zs, n * 4, cudaMemcpyHostToDevice, st));
    dx = b; dy = b + n; dz = b + 2 * n; dout = b + 3 * n;
  }
  if (g->C == 1)
    launch_k(k_sample1, ceil_div(n, 256), 256, 0, st, g->view(), dx, dy, dz, n, dout);
  else
    launch_k(k_sampleC, ceil_div(n, 256), 256, 0, st, g->view(), dx, dy, dz, n, dout);
  PVDB_CHECK_LAUNCH("k_sample");
  if (mem == PVDB_MEM_HOST) {
    PVDB_CHECK_CUDA(cudaMemcpyAsync(out, dout, n * 4 * g->C, cudaMemcpyDeviceToHost, st));
    PVDB_CHECK_CUDA(cudaStreamSynchronize(st));
  }
  return PVDB_OK;
}

int pvdb_grid_lookup(pvdb_grid g, const int32_t* is, const int32_t* js, const int32_t* ks,
                     int64_t n, float* out, uint8_t* active_out, int32_t mem, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(g, "null grid");
  PVDB_REQUIRE(n >= 0, "negative size");
  if (n == 0) return PVDB_OK;
  PVDB_REQUIRE(is && js && ks && out, "null argument");
  cudaStream_t st = as_stream(s);
  const int32_t *di = is, *dj = js, *dk = ks;
  float* dout = out;
  uint8_t* dact = active_out;
  if (mem == PVDB_MEM_HOST) {
    int rc = stage_reserve(g, size_t(n) * (12 + 4 * g->C + 1) + 64);
    if (rc) return rc;
    int32_t* b = (int32_t*)g->d_stage;
    PVDB_CHECK_CUDA(cudaMemcpyAsync(b, is, n * 4, cudaMemcpyHostToDevice, st));
    PVDB_CHECK_CUDA(cudaMemcpyAsync(b + n, js, n * 4, cudaMemcpyHostToDevice, st));
    PVDB_CHECK_CUDA(cudaMemcpyAsync(b + 2 * n, ks, n * 4, cudaMemcpyHostToDevice, st));
    di = b; dj = b + n; dk = b + 2 * n;
    dout = (float*)(b + 3 * n);
    dact = active_out ? (uint8_t*)(dout + n * g->C) : nullptr;
  }
  launch_k(k_lookup, ceil_div(n, 256), 256, 0, st, g->view(), di, dj, dk, n, dout, dact);
  PVDB_CHECK_LAUNCH("k_lookup");
  if (mem == PVDB_MEM_HOST) {
    PVDB_CHECK_CUDA(cudaMemcpyAsync(out, dout, n * 4 * g->C, cudaMemcpyDeviceToHost, st));
    if (active_out)
      PVDB_CHECK_CUDA(cudaMemcpyAsync(active_out, dact, n, cudaMemcpyDeviceToHost, st));
    PVDB_CHECK_CUDA(cudaStreamSynchronize(st));
  }
  return PVDB_OK;
}

int pvdb_grid_tv_add_grad(pvdb_grid g, float wx, float wy, float wz, int32_t dense_mode,
                          int32_t mimic_axis_bug, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(g, "null grid");
  // the reference divides the weights by 6 on the host (total_variation_kernel.cu:45-47)
  wx /= 6.f;
  wy /= 6.f;
  wz /= 6.f;
  if (mimic_axis_bug) wx = wz;
  cudaStream_t st = as_stream(s);
  if (g->nslots() == 0) return PVDB_OK;
  // without dense mode only voxels with a nonzero gradient change: the touched leaves
  const bool use_list = !dense_mode && !g->all_touched;
  if (use_list) {
    int rc = touched_list(g, st);
    if (rc) return rc;
  }
  if (g->C == 12)
    launch_k(k_tv_c12, stride_grid(), 256, 0, st, g->view(), wx, wy, wz, dense_mode ? 1 : 0,
             use_list ? g->d_tlist : nullptr, g->d_tcount);
  else
    launch_k(k_tv, stride_grid(), 256, 0, st, g->view(), wx, wy, wz, dense_mode ? 1 : 0,
             use_list ? g->d_tlist : nullptr, g->d_tcount);
  PVDB_CHECK_LAUNCH("k_tv");
  if (dense_mode) g->all_touched = true;
  return PVDB_OK;
}



int pvdb_grid_touched_leaves(pvdb_grid g, int64_t* n, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(g && n, "null argument");
  *n = 0;
  if (!g->d_tcount) return PVDB_OK;
  uint32_t c = 0;
  cudaStream_t st = as_stream(s);
  PVDB_CHECK_CUDA(cudaMemcpyAsync(&c, g->d_tcount, 4, cudaMemcpyDeviceToHost, st));
  PVDB_CHECK_CUDA(cudaStreamSynchronize(st));
  *n = std::min<int64_t>(c, g->nleaf);
  return PVDB_OK;
}

int pvdb_grid_zero_grad(pvdb_grid g, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(g, "null grid");
  cudaStream_t st = as_stream(s);
  const int64_t ns = g->nslots();
  if (ns) {
    launch_k(k_zero_grad, ceil_div(ns, 256), 256, 0, st, g->view(),
             g->all_touched ? nullptr : g->d_touched);
    PVDB_CHECK_LAUNCH("k_zero_grad");
    launch_k(k_clear_touched, ceil_div(g->nleaf, 256), 256, 0, st, g->d_touched, g->nleaf);
    PVDB_CHECK_LAUNCH("k_clear_touched");
  }
  g->all_touched = false;
  g->tlist_valid = false;
  return PVDB_OK;
}

int pvdb_grid_mark_written(pvdb_grid g, int32_t which) {
  clear_error();
  PVDB_REQUIRE(g, "null grid");
  PVDB_REQUIRE(which == PVDB_WHICH_DATA || which == PVDB_WHICH_GRAD, "bad `which`");
  if (which == PVDB_WHICH_DATA) data_written(g);
  else g->all_touched = true;
  return PVDB_OK;
}

int pvdb_grid_device_views(pvdb_grid g, void** data, void** grad, void** mask, void** leaf_table,
                           void** leaf_origin, int32_t ldim[3]) {
  clear_error();
  PVDB_REQUIRE(g, "null grid");
  if (data) {
    *data = g->d_data;
    data_written(g);  // the caller may write values we cannot track
  }
  if (grad) {
    *grad = g->d_grad;
    g->all_touched = true;  // the caller may write gradients we cannot track
  }
  if (mask) *mask = g->d_mask;
  if (leaf_table) *leaf_table = g->d_table;
  if (leaf_origin) *leaf_origin = g->d_origin;
  if (ldim)
    for (int a = 0; a < 3; ++a) ldim[a] = g->ldim[a];
  return PVDB_OK;
}

// ------------------------------------------------------------- save / load
static uint64_t fnv1a(uint64_t h, const void* p, size_t n) {
  const uint8_t* b = (const uint8_t*)p;
  for (size_t i = 0; i < n; ++i) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}

int pvdb_grid_save(pvdb_grid g, const char* path) {
  clear_error();
  PVDB_REQUIRE(g && path, "null argument");
  const size_t nval = size_t(g->nleaf) * kLeafVox * g->C;
  std::vector<float> vals(nval);
  PVDB_CHECK_CUDA(cudaDeviceSynchronize());
  if (nval) PVDB_CHECK_CUDA(cudaMemcpy(vals.data(), g->d_data, nval * 4, cudaMemcpyDeviceToHost));
  FILE* f = std::fopen(path, "wb");
  if (!f) return set_error(PVDB_ERR_IO, std::string("cannot open for writing: ") + path);
  const char magic[8] = {'P', 'V', 'D', 'B', 'G', 'R', 'D', '1'};
  int32_t hdr[8] = {g->reso[0], g->reso[1], g->reso[2], g->C, g->nleaf, 0, 0, 0};
  float bg = g->background;
  uint64_t h = 14695981039346656037ull;
  auto put = [&](const void* p, size_t n) {
    h = fnv1a(h, p, n);
    return std::fwrite(p, 1, n, f) == n;
  };
  bool ok = put(magic, 8) && put(hdr, sizeof(hdr)) && put(&bg, 4) &&
            put(g->h_origin.data(), g->h_origin.size() * 4) &&
            put(g->h_mask.data(), g->h_mask.size() * 8) && put(vals.data(), nval * 4);
  ok = ok && std::fwrite(&h, 1, 8, f) == 8;
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return set_error(PVDB_ERR_IO, std::string("write failed: ") + path);
  return PVDB_OK;
}

int pvdb_grid_load(const char* path, pvdb_grid* out) {
  clear_error();
  PVDB_REQUIRE(path && out, "null argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_error(PVDB_ERR_IO, std::string("cannot open: ") + path);
  uint64_t h = 14695981039346656037ull;
  auto get = [&](void* p, size_t n) {
    if (std::fread(p, 1, n, f) != n) return false;
    h = fnv1a(h, p, n);
    return true;
  };
  char magic[8];
  int32_t hdr[8];
  float bg;
  bool ok = get(magic, 8) && std::memcmp(magic, "PVDBGRD1", 8) == 0 && get(hdr, sizeof(hdr)) &&
            get(&bg, 4);
  if (ok) ok = hdr[0] > 0 && hdr[1] > 0 && hdr[2] > 0 && hdr[0] <= 8192 && hdr[1] <= 8192 &&
               hdr[2] <= 8192 && hdr[3] > 0 && hdr[4] >= 0;
  if (ok) {
    const int64_t maxleaf = int64_t((hdr[0] + 7) / 8) * ((hdr[1] + 7) / 8) * ((hdr[2] + 7) / 8);
    ok = hdr[4] <= maxleaf;
  }
  std::vector<int32_t> origin;
  std::vector<uint64_t> mask;
  std::vector<float> vals;
  if (ok) {
    origin.resize(size_t(hdr[4]) * 3);
    mask.resize(size_t(hdr[4]) * 8);
    vals.resize(size_t(hdr[4]) * kLeafVox * hdr[3]);
    ok = get(origin.data(), origin.size() * 4) && get(mask.data(), mask.size() * 8) &&
         get(vals.data(), vals.size() * 4);
  }
  uint64_t stored = 0;
  const uint64_t computed = h;
  ok = ok && std::fread(&stored, 1, 8, f) == 8 && stored == computed;
  std::fclose(f);
  if (!ok) return set_error(PVDB_ERR_IO, std::string("corrupt or truncated grid file: ") + path);
  const int reso[3] = {hdr[0], hdr[1], hdr[2]};
  std::vector<std::array<int, 3>> leaves(hdr[4]);
  std::vector<std::array<uint64_t, 8>> masks(hdr[4]);
  for (int i = 0; i < hdr[4]; ++i) {
    for (int a = 0; a < 3; ++a) {
      if (origin[i * 3 + a] % 8 || origin[i * 3 + a] < 0 || origin[i * 3 + a] >= reso[a] + 7)
        return set_error(PVDB_ERR_IO, "corrupt leaf origin");
      leaves[i][a] = origin[i * 3 + a] / 8;
    }
    for (int w = 0; w < 8; ++w) masks[i][w] = mask[i * 8 + w];
  }
  pvdb_grid_s* g = nullptr;
  int rc = build_grid(reso, hdr[3], bg, leaves, masks, &g);
  if (rc) return rc;
  // build_grid keeps the file's leaf order only if it is already Morton sorted;
  // place the values through the table to be independent of the order.
  std::vector<float> placed(vals.size());
  for (int i = 0; i < hdr[4]; ++i) {
    const int64_t ti = (int64_t(leaves[i][0]) * g->ldim[1] + leaves[i][1]) * g->ldim[2] + leaves[i][2];
    const int id = g->h_table[ti];
    std::memcpy(&placed[size_t(id) * kLeafVox * hdr[3]], &vals[size_t(i) * kLeafVox * hdr[3]],
                size_t(kLeafVox) * hdr[3] * 4);
  }
  if (!placed.empty()) {
    cudaError_t e = cudaMemcpy(g->d_data, placed.data(), placed.size() * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      pvdb_grid_destroy(g);
      return cuda_error(e, "grid load upload");
    }
  }
  g->all_touched = true;
  *out = g;
  return PVDB_OK;
}

}  // extern "C"
