// Grid lifecycle around the training step:
//   * merged-row compression for the renderer (vdb_compression.py:19-59);
//   * trilinear rescaling of a grid for progressive scaling
//     (VDBGrid.scale_volume_grid, lib/grid.py:91-102);
//   * the occupancy (mask-cache) builds: update_occupancy_cache
//     (lib/dvgo.py:200-210), the rebuild after rescaling (lib/dvgo.py:186-197)
//     and MaskGrid from a checkpoint's density (lib/grid.py:210-221);
//   * maskout_near_cam_vox (lib/dvgo.py:163-175);
//   * voxel_count_views (lib/dvgo.py:212-243), the per-voxel lr counts.
// None of these run inside a training step; each is one or two HBM-bound
// passes over a grid or over the rays of a view.
#include <cuda_fp16.h>

#include <cmath>
#include <mutex>

#include "ray_ops.cuh"

namespace pvdb {

// ------------------------------------------------------------------ merge
// Row ids are given to the voxels with a nonzero mask byte in C order
// (x*ry*rz + y*rz + z), starting at 1; row 0 stays the empty row. A block
// covers 4096 mask bytes (16 per thread, one 16-byte load); pass 1 counts per
// block, a device scan turns the counts into block offsets, pass 2 recounts,
// ranks inside the block and writes the index and the rows.
constexpr int kMergeThreads = 256;
constexpr int kMergeVox = 16;
constexpr int64_t kMergeBlockVox = int64_t(kMergeThreads) * kMergeVox;

__device__ __forceinline__ uint32_t merge_flags(const uint8_t* mask, int64_t n, int64_t base,
                                                int vec) {
  uint32_t f = 0;
  if (vec && base + kMergeVox <= n) {
    const uint4 w = __ldg(reinterpret_cast<const uint4*>(mask + base));
    const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if ((ws[b] >> (8 * q)) & 0xffu) f |= 1u << (4 * b + q);
  } else {
    for (int q = 0; q < kMergeVox; ++q)
      if (base + q < n && mask[base + q]) f |= 1u << q;
  }
  return f;
}

__global__ void __launch_bounds__(kMergeThreads)
    k_merge_count(const uint8_t* __restrict__ mask, int64_t n, int vec, uint32_t* block_cnt) {
  const int64_t base = (int64_t(blockIdx.x) * kMergeThreads + threadIdx.x) * kMergeVox;
  const uint32_t c = __reduce_add_sync(0xffffffffu, __popc(merge_flags(mask, n, base, vec)));
  __shared__ uint32_t ws[kMergeThreads / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
#pragma unroll
    for (int w = 0; w < kMergeThreads / 32; ++w) t += ws[w];
    block_cnt[blockIdx.x] = t;
  }
}

struct MergeArgs {
  GridView den, col;
  int has_den, has_col;
  int reso[3];
  int32_t* index;
  void* den_rows;
  void* col_rows;
  int dtype;    // 0 FP32 rows, 1 FP16 rows
  int vec;      // mask and index are 16-byte aligned
  int col_vec;  // colour rows aligned for whole-row vector stores
};

__device__ __forceinline__ void put_row(void* rows, int64_t i, int dtype, float v) {
  if (dtype == 1) reinterpret_cast<__half*>(rows)[i] = __float2half_rn(v);
  else reinterpret_cast<float*>(rows)[i] = v;
}

// Row r of the colour rows: the voxel's C channels (background outside the
// leaves). C == 12 with aligned rows moves 16-byte loads and 16-/8-byte stores.
__device__ __forceinline__ void put_col_row(const MergeArgs& a, int64_t r, int x, int y, int z) {
  const int s = slot_of(a.col, x, y, z);
  const int C = a.col.C;
  if (C == 12 && a.col_vec) {
    float v[12];
    if (s < 0) {
#pragma unroll
      for (int c = 0; c < 12; ++c) v[c] = a.col.background;
    } else {
      const float4* src = reinterpret_cast<const float4*>(a.col.data + int64_t(s) * 12);
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const float4 w = __ldg(src + b);
        v[4 * b] = w.x;
        v[4 * b + 1] = w.y;
        v[4 * b + 2] = w.z;
        v[4 * b + 3] = w.w;
      }
    }
    if (a.dtype == 1) {
      uint2* dst = reinterpret_cast<uint2*>(reinterpret_cast<__half*>(a.col_rows) + r * 12);
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const __half2 lo = __floats2half2_rn(v[4 * b], v[4 * b + 1]);
        const __half2 hi = __floats2half2_rn(v[4 * b + 2], v[4 * b + 3]);
        dst[b] = make_uint2(*reinterpret_cast<const uint32_t*>(&lo),
                            *reinterpret_cast<const uint32_t*>(&hi));
      }
    } else {
      float4* dst = reinterpret_cast<float4*>(reinterpret_cast<float*>(a.col_rows) + r * 12);
#pragma unroll
      for (int b = 0; b < 3; ++b)
        dst[b] = make_float4(v[4 * b], v[4 * b + 1], v[4 * b + 2], v[4 * b + 3]);
    }
    return;
  }
  for (int ch = 0; ch < C; ++ch)
    put_row(a.col_rows, r * C + ch, a.dtype,
            s < 0 ? a.col.background : __ldg(a.col.data + int64_t(s) * C + ch));
}

// Rank of this thread's first flagged voxel among all flagged voxels (block
// offset from the scan plus the prefix inside the block).
__device__ __forceinline__ int64_t merge_rank(uint32_t c, const uint32_t* __restrict__ block_off) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t inc = c;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += y;
  }
  __shared__ uint32_t wsum[kMergeThreads / 32];
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  uint32_t wpre = 0;
  for (int w = 0; w < wid; ++w) wpre += wsum[w];
  return int64_t(block_off[blockIdx.x]) + wpre + (inc - c);
}

__global__ void __launch_bounds__(kMergeThreads)
    k_merge_write(const uint8_t* __restrict__ mask, int64_t n,
                  const uint32_t* __restrict__ block_off, MergeArgs a) {
  const int t = threadIdx.x;
  const int64_t base = (int64_t(blockIdx.x) * kMergeThreads + t) * kMergeVox;
  const uint32_t f = merge_flags(mask, n, base, a.vec);
  const int64_t row0 = 1 + merge_rank(__popc(f), block_off);

  int32_t idx[kMergeVox];
  int64_t r = row0;
#pragma unroll
  for (int q = 0; q < kMergeVox; ++q) idx[q] = ((f >> q) & 1u) ? int32_t(r++) : 0;
  if (a.vec && base + kMergeVox <= n) {
    int4* dst = reinterpret_cast<int4*>(a.index + base);
#pragma unroll
    for (int b = 0; b < 4; ++b)
      dst[b] = make_int4(idx[4 * b], idx[4 * b + 1], idx[4 * b + 2], idx[4 * b + 3]);
  } else {
    for (int q = 0; q < kMergeVox; ++q)
      if (base + q < n) a.index[base + q] = idx[q];
  }

  if (blockIdx.x == 0 && t == 0) {
    if (a.has_den) put_row(a.den_rows, 0, a.dtype, 0.f);
    if (a.has_col)
      for (int ch = 0; ch < a.col.C; ++ch) put_row(a.col_rows, ch, a.dtype, 0.f);
  }
  if (!f) return;
  // coordinates of the chunk's first voxel, then stepped along z (C order)
  const int64_t yz = int64_t(a.reso[1]) * a.reso[2];
  int x = int(base / yz);
  const int64_t rem = base - int64_t(x) * yz;
  int y = int(rem / a.reso[2]);
  int z = int(rem - int64_t(y) * a.reso[2]);
  r = row0;
  for (int q = 0; q < kMergeVox; ++q) {
    if ((f >> q) & 1u) {
      if (a.has_den) put_row(a.den_rows, r, a.dtype, value1(a.den, x, y, z));
      if (a.has_col) put_col_row(a, r, x, y, z);
      ++r;
    }
    if (++z == a.reso[2]) {
      z = 0;
      if (++y == a.reso[1]) {
        y = 0;
        ++x;
      }
    }
  }
}

// Order-preserving compaction of up to four [n,3] float arrays by a byte flag
// (the boolean indexing of get_training_rays_in_maskcache_sampling,
// lib/dvgo.py:607-613).
struct CompactArgs {
  const float* src[4];
  float* dst[4];
  int narr;
  int vec;
};

__global__ void __launch_bounds__(kMergeThreads)
    k_compact_rows(const uint8_t* __restrict__ keep, int64_t n,
                   const uint32_t* __restrict__ block_off, CompactArgs a) {
  const int64_t base = (int64_t(blockIdx.x) * kMergeThreads + threadIdx.x) * kMergeVox;
  const uint32_t f = merge_flags(keep, n, base, a.vec);
  int64_t r = merge_rank(__popc(f), block_off);
  for (int q = 0; q < kMergeVox; ++q) {
    if (!((f >> q) & 1u)) continue;
    const int64_t v = base + q;
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k < a.narr)
#pragma unroll
        for (int c = 0; c < 3; ++c) a.dst[k][3 * r + c] = __ldg(a.src[k] + 3 * v + c);
    ++r;
  }
}

// --------------------------------------------------------------- rescale
// F.interpolate(mode='trilinear', align_corners=True) on the dense values
// (grid.py:92, ATen upsample_trilinear3d, as its CPU build evaluates 1- and
// 3-channel volumes; some wider shapes take another ATen order, a few ulps
// apart): per axis src = scale*o with
// scale = (in-1)/(out-1), i0 = min(floor(src), in-1), i1 = i0 + (i0 < in-1),
// l1 = clamp(src - i0, 0, 1), l0 = 1 - l1; the value nests z inside y inside
// x: ((v[..z0]*l0z + v[..z1]*l1z)*l0y + (...)*l1y)*l0x + (...)*l1x, each
// a*w0 + b*w1 contracted to fma(a, w0, b*w1) as in ATen's CPU build.
struct AxisMap {
  float scale[3];
  int in[3];
};

__device__ __forceinline__ void axis_weights(float scale, int in, int o, int& i0, int& i1,
                                             float& l0, float& l1) {
  const float real = __fmul_rn(scale, float(o));
  i0 = min(int(floorf(real)), in - 1);
  l1 = fminf(fmaxf(real - float(i0), 0.f), 1.f);
  i1 = i0 + (i0 < in - 1 ? 1 : 0);
  l0 = 1.f - l1;
}

// a*wa + b*wb as ATen's kernel evaluates it on the CPU: fma(a, wa, b*wb).
__device__ __forceinline__ float lerp2(float a, float wa, float b, float wb) {
  return __fmaf_rn(a, wa, __fmul_rn(b, wb));
}

__global__ void k_resample(GridView src, GridView dst, AxisMap m) {
  const int64_t slot = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (slot >= int64_t(dst.nleaf) * kLeafVox) return;
  const int l = int(slot >> 9), off = int(slot & 511);
  const int x = __ldg(dst.origin + 3 * l) + (off >> 6);
  const int y = __ldg(dst.origin + 3 * l + 1) + ((off >> 3) & 7);
  const int z = __ldg(dst.origin + 3 * l + 2) + (off & 7);
  if (x >= dst.reso[0] || y >= dst.reso[1] || z >= dst.reso[2]) return;
  int xi[2], yi[2], zi[2];
  float xw[2], yw[2], zw[2];
  axis_weights(m.scale[0], m.in[0], x, xi[0], xi[1], xw[0], xw[1]);
  axis_weights(m.scale[1], m.in[1], y, yi[0], yi[1], yw[0], yw[1]);
  axis_weights(m.scale[2], m.in[2], z, zi[0], zi[1], zw[0], zw[1]);
  int s[8];
  if ((xi[0] >> 3) == (xi[1] >> 3) && (yi[0] >> 3) == (yi[1] >> 3) &&
      (zi[0] >> 3) == (zi[1] >> 3)) {
    // all 8 corners in the low corner's leaf: one table lookup
    const int l = leaf_of(src, xi[0], yi[0], zi[0]);
    const int b = l < 0 ? -1 : ((l << 9) | vox_offset(xi[0], yi[0], zi[0]));
    const int dx = (xi[1] - xi[0]) << 6, dy = (yi[1] - yi[0]) << 3, dz = zi[1] - zi[0];
#pragma unroll
    for (int c = 0; c < 8; ++c)
      s[c] = b < 0 ? -1 : b + ((c >> 2) ? dx : 0) + (((c >> 1) & 1) ? dy : 0) + ((c & 1) ? dz : 0);
  } else {
#pragma unroll
    for (int c = 0; c < 8; ++c) s[c] = slot_of(src, xi[c >> 2], yi[(c >> 1) & 1], zi[c & 1]);
  }
  const int C = dst.C;
  if ((C & 3) == 0) {
    float4* out = reinterpret_cast<float4*>(dst.data + slot * C);
    const float4 bg = make_float4(src.background, src.background, src.background, src.background);
    for (int q = 0; q < C / 4; ++q) {
      float4 v[8];
#pragma unroll
      for (int c = 0; c < 8; ++c)
        v[c] = s[c] < 0 ? bg : __ldg(reinterpret_cast<const float4*>(src.data + int64_t(s[c]) * C) + q);
      float r[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        float w[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) w[c] = e == 0 ? v[c].x : e == 1 ? v[c].y : e == 2 ? v[c].z : v[c].w;
        const float y0 = lerp2(lerp2(w[0], zw[0], w[1], zw[1]), yw[0],
                               lerp2(w[2], zw[0], w[3], zw[1]), yw[1]);
        const float y1 = lerp2(lerp2(w[4], zw[0], w[5], zw[1]), yw[0],
                               lerp2(w[6], zw[0], w[7], zw[1]), yw[1]);
        r[e] = lerp2(y0, xw[0], y1, xw[1]);
      }
      out[q] = make_float4(r[0], r[1], r[2], r[3]);
    }
    return;
  }
  float* out = dst.data + slot * C;
  for (int ch = 0; ch < C; ++ch) {
    float v[8];
#pragma unroll
    for (int c = 0; c < 8; ++c)
      v[c] = s[c] < 0 ? src.background : __ldg(src.data + int64_t(s[c]) * C + ch);
    const float y0 = lerp2(lerp2(v[0], zw[0], v[1], zw[1]), yw[0], lerp2(v[2], zw[0], v[3], zw[1]),
                           yw[1]);
    const float y1 = lerp2(lerp2(v[4], zw[0], v[5], zw[1]), yw[0], lerp2(v[6], zw[0], v[7], zw[1]),
                           yw[1]);
    out[ch] = lerp2(y0, xw[0], y1, xw[1]);
  }
}

// Scalar grids: one thread per 8-voxel z column of a destination leaf. The
// x/y weights and the table rows of the four (x, y) source corners are formed
// once per column; per z only the z weights, one table load per corner and
// the values remain.
__global__ void __launch_bounds__(256) k_resample_col(GridView src, GridView dst, AxisMap m) {
  const int64_t col = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (col >= int64_t(dst.nleaf) * 64) return;
  const int l = int(col >> 6), xy = int(col & 63);
  const int x = __ldg(dst.origin + 3 * l) + (xy >> 3);
  const int y = __ldg(dst.origin + 3 * l + 1) + (xy & 7);
  const int zb = __ldg(dst.origin + 3 * l + 2);
  if (x >= dst.reso[0] || y >= dst.reso[1]) return;
  int xi[2], yi[2];
  float xw[2], yw[2];
  axis_weights(m.scale[0], m.in[0], x, xi[0], xi[1], xw[0], xw[1]);
  axis_weights(m.scale[1], m.in[1], y, yi[0], yi[1], yw[0], yw[1]);
  // per (x, y) corner: the table row (-1 outside the table) and the in-leaf offset
  int trow[4], xyoff[4];
  const int lx = src.ldim[0] << 3, ly = src.ldim[1] << 3;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int i = xi[c >> 1], j = yi[c & 1];
    trow[c] = ((unsigned)i < (unsigned)lx && (unsigned)j < (unsigned)ly)
                  ? ((i >> 3) * src.ldim[1] + (j >> 3)) * src.ldim[2]
                  : -1;
    xyoff[c] = ((i & 7) << 6) | ((j & 7) << 3);
  }
  const int lz = src.ldim[2] << 3;
  float* out = dst.data + ((int64_t(l) << 9) | (xy << 3));
  for (int dz = 0; dz < 8; ++dz) {
    const int z = zb + dz;
    if (z >= dst.reso[2]) break;
    int zi[2];
    float zw[2];
    axis_weights(m.scale[2], m.in[2], z, zi[0], zi[1], zw[0], zw[1]);
    int sl[8];  // corner c = 4*xbit + 2*ybit + zbit
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int k = zi[e];
        int leaf = -1;
        if (trow[c] >= 0 && (unsigned)k < (unsigned)lz) leaf = __ldg(src.table + trow[c] + (k >> 3));
        sl[2 * c + e] = leaf < 0 ? -1 : ((leaf << 9) | xyoff[c] | (k & 7));
      }
    float v[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) v[c] = sl[c] < 0 ? src.background : __ldg(src.data + sl[c]);
    const float y0 = lerp2(lerp2(v[0], zw[0], v[1], zw[1]), yw[0],
                           lerp2(v[2], zw[0], v[3], zw[1]), yw[1]);
    const float y1 = lerp2(lerp2(v[4], zw[0], v[5], zw[1]), yw[0],
                           lerp2(v[6], zw[0], v[7], zw[1]), yw[1]);
    out[dz] = lerp2(y0, xw[0], y1, xw[1]);
  }
}

// ------------------------------------------------------------- occupancy
// One block per 8^3 tile of the output mask: the 10^3 values the 3x3x3 max
// pool of the tile reads are computed once into shared memory (-inf outside
// the grid, which is max_pool3d's padding), then every thread pools 27.
constexpr int kOccTile = 8;
constexpr int kOccHalo = kOccTile + 2;

struct OccArgs {
  GridView den;
  int mode;
  int shape[3];          // output mask shape
  float lin_start[3], lin_end[3], lin_step[3];  // linspace(min, max, shape)
  float ext[3], wsm1[3];  // wld2idx of the density grid (mode 0)
  const uint8_t* old_mask;  // mode 1 (may be NULL: all true)
  int old_shape[3];
  float old_scale[3], old_shift[3];
  float shift, interval, thres;
  uint8_t* out;
};

// torch.linspace(start, end, n)[i] by the two-sided formula of ATen's scalar
// path: start + step*i in the first half, end - step*(n-1-i) in the second
// (ATen RangeFactoriesKernel). ATen's vectorised path, which depends on the
// CPU, can round differently by up to one ulp of the range.
__device__ __forceinline__ float linspace_at(float start, float end, float step, int n, int i) {
  if (n == 1) return start;
  return i < n / 2 ? __fadd_rn(start, __fmul_rn(step, float(i)))
                   : __fsub_rn(end, __fmul_rn(step, float(n - 1 - i)));
}

// 1 - exp(-softplus(x) * interval), softplus as log1p(exp(x)) with torch's
// threshold 20 (torch's vectorised CPU kernel forms log(exp(x) + 1): within
// 2e-5 relative).
__device__ __forceinline__ float softplus_alpha(float x, float interval) {
  const float sp = x > 20.f ? x : log1pf(expf(x));
  return 1.f - expf(-__fmul_rn(sp, interval));
}

__global__ void __launch_bounds__(512) k_occupancy(OccArgs a) {
  __shared__ float val[kOccHalo * kOccHalo * kOccHalo];
  const int tiles_z = (a.shape[2] + kOccTile - 1) / kOccTile;
  const int tiles_y = (a.shape[1] + kOccTile - 1) / kOccTile;
  const int tz = blockIdx.x % tiles_z, ty = (blockIdx.x / tiles_z) % tiles_y,
            tx = blockIdx.x / (tiles_z * tiles_y);
  const int x0 = tx * kOccTile - 1, y0 = ty * kOccTile - 1, z0 = tz * kOccTile - 1;
  const int lx = threadIdx.x >> 6, ly = (threadIdx.x >> 3) & 7, lz = threadIdx.x & 7;
  const int i = x0 + 1 + lx, j = y0 + 1 + ly, k = z0 + 1 + lz;
  const bool inside = i < a.shape[0] && j < a.shape[1] && k < a.shape[2];
  const int64_t o = (int64_t(i) * a.shape[1] + j) * a.shape[2] + k;
  // the pooled value only matters where the other operand of the & is set:
  // mode 0 the mask itself, mode 1 the old mask at the grid point
  bool need = inside;
  if (inside && a.mode == 0) {
    need = a.out[o] != 0;
  } else if (inside && a.mode == 1 && a.old_mask) {
    const float p[3] = {linspace_at(a.lin_start[0], a.lin_end[0], a.lin_step[0], a.shape[0], i),
                        linspace_at(a.lin_start[1], a.lin_end[1], a.lin_step[1], a.shape[1], j),
                        linspace_at(a.lin_start[2], a.lin_end[2], a.lin_step[2], a.shape[2], k)};
    need = mask_lookup(a.old_mask, a.old_shape, p, a.old_scale, a.old_shift);
  }
  if (!__syncthreads_or(need)) {
    if (inside && a.mode == 1) a.out[o] = 0;  // mode 0 leaves the zeros as they are
    return;
  }
  for (int e = threadIdx.x; e < kOccHalo * kOccHalo * kOccHalo; e += blockDim.x) {
    const int hx = e / (kOccHalo * kOccHalo), hy = (e / kOccHalo) % kOccHalo, hz = e % kOccHalo;
    const int ii = x0 + hx, jj = y0 + hy, kk = z0 + hz;
    float v = -INFINITY;
    if (ii >= 0 && jj >= 0 && kk >= 0 && ii < a.shape[0] && jj < a.shape[1] && kk < a.shape[2]) {
      if (a.mode == 0) {
        const float p[3] = {
            linspace_at(a.lin_start[0], a.lin_end[0], a.lin_step[0], a.shape[0], ii),
            linspace_at(a.lin_start[1], a.lin_end[1], a.lin_step[1], a.shape[1], jj),
            linspace_at(a.lin_start[2], a.lin_end[2], a.lin_step[2], a.shape[2], kk)};
        float idx[3];
        world_to_index(p, a.lin_start, a.ext, a.wsm1, idx);
        float e_;
        v = raw2alpha(trilinear1(a.den, idx[0], idx[1], idx[2]), a.shift, a.interval, e_);
      } else if (a.mode == 1) {
        float e_;
        v = raw2alpha(value1(a.den, ii, jj, kk), a.shift, a.interval, e_);
      } else {
        v = value1(a.den, ii, jj, kk);
      }
    }
    val[e] = v;
  }
  __syncthreads();
  if (!inside) return;
  if (!need) {
    if (a.mode == 1) a.out[o] = 0;
    return;
  }
  float m = -INFINITY;
#pragma unroll
  for (int dx = 0; dx < 3; ++dx)
#pragma unroll
    for (int dy = 0; dy < 3; ++dy)
#pragma unroll
      for (int dz = 0; dz < 3; ++dz)
        m = fmaxf(m, val[((lx + dx) * kOccHalo + (ly + dy)) * kOccHalo + (lz + dz)]);
  uint8_t r;
  if (a.mode == 0 || a.mode == 1) r = m > a.thres;
  else r = softplus_alpha(m + a.shift, a.interval) >= a.thres;
  a.out[o] = r;
}

// ------------------------------------------------------ near-camera voxels
// Active voxels whose grid point lies within near_clip of a camera centre get
// `value` (maskout_near_cam_vox + setValuesOn_bymask, densityvdb.cu:64-97).
struct NearCamArgs {
  GridView g;
  const float* cams;
  int n_cams;
  float lin_start[3], lin_end[3], lin_step[3];
  float near_clip, value;
};

__global__ void k_near_cams(NearCamArgs a) {
  const int64_t slot = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (slot >= int64_t(a.g.nleaf) * kLeafVox) return;
  const int l = int(slot >> 9), off = int(slot & 511);
  if (!((__ldg(a.g.mask + l * 8 + (off >> 6)) >> (off & 63)) & 1ull)) return;
  const int x = __ldg(a.g.origin + 3 * l) + (off >> 6);
  const int y = __ldg(a.g.origin + 3 * l + 1) + ((off >> 3) & 7);
  const int z = __ldg(a.g.origin + 3 * l + 2) + (off & 7);
  const float p[3] = {linspace_at(a.lin_start[0], a.lin_end[0], a.lin_step[0], a.g.reso[0], x),
                      linspace_at(a.lin_start[1], a.lin_end[1], a.lin_step[1], a.g.reso[1], y),
                      linspace_at(a.lin_start[2], a.lin_end[2], a.lin_step[2], a.g.reso[2], z)};
  float best = INFINITY;
  for (int c = 0; c < a.n_cams; ++c) {
    const float dx = p[0] - __ldg(a.cams + 3 * c), dy = p[1] - __ldg(a.cams + 3 * c + 1),
                dz = p[2] - __ldg(a.cams + 3 * c + 2);
    best = fminf(best, sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)),
                                       __fmul_rn(dz, dz))));
  }
  if (best <= a.near_clip)
    for (int ch = 0; ch < a.g.C; ++ch) a.g.data[slot * a.g.C + ch] = a.value;
}

// ----------------------------------------------------------- view counts
// One view's rays: every ray takes n_samples points at
// t = t_min + stepdist*k/|d| (t_min from the slab test clamped to [near, 1e9]),
// and each point adds its 8 trilinear weights (grid_sample, align_corners,
// zero padding: corners outside the grid are dropped) to the voxels it
// touches. The sums are kept in 32.32 fixed point so that they are exact and
// independent of the order of the atomics; a voxel counts the view when its
// sum exceeds 1.
struct CountArgs {
  int reso[3];
  float xyz_min[3], xyz_max[3];
  float near_, stepdist;
  int n_samples;
};

__global__ void k_count_views_acc(const float* __restrict__ ro, const float* __restrict__ rd,
                                  int64_t n_rays, CountArgs a, unsigned long long* acc) {
  const int64_t total = n_rays * a.n_samples;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total;
       e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = e / a.n_samples;
    const int k = int(e - r * a.n_samples);
    const float o[3] = {__ldg(ro + 3 * r), __ldg(ro + 3 * r + 1), __ldg(ro + 3 * r + 2)};
    const float d[3] = {__ldg(rd + 3 * r), __ldg(rd + 3 * r + 1), __ldg(rd + 3 * r + 2)};
    float ta[3], tb[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const float vq = d[q] == 0.f ? 1e-6f : d[q];
      ta[q] = __fdiv_rn(a.xyz_max[q] - o[q], vq);
      tb[q] = __fdiv_rn(a.xyz_min[q] - o[q], vq);
    }
    const float t_min = fminf(fmaxf(fmaxf(fmaxf(fminf(ta[0], tb[0]), fminf(ta[1], tb[1])),
                                          fminf(ta[2], tb[2])),
                                    a.near_),
                              1e9f);
    const float dn = torch_norm3(d[0], d[1], d[2]);  // rays_d.norm(dim=-1)
    const float tk = __fadd_rn(t_min, __fdiv_rn(__fmul_rn(a.stepdist, float(k)), dn));
    float g[3];
    int g0[3];
    bool any = true;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const float p = __fadd_rn(o[q], __fmul_rn(d[q], tk));
      const float nrm = __fsub_rn(__fmul_rn(__fdiv_rn(p - a.xyz_min[q], a.xyz_max[q] - a.xyz_min[q]), 2.f), 1.f);
      g[q] = __fmul_rn(__fmul_rn(__fadd_rn(nrm, 1.f), 0.5f), float(a.reso[q] - 1));
      const float fl = floorf(g[q]);
      any &= fl >= -1.f && fl <= float(a.reso[q] - 1);
      g0[q] = any ? int(fl) : 0;
    }
    if (!any) continue;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int i = g0[0] + (c >> 2), j = g0[1] + ((c >> 1) & 1), kk = g0[2] + (c & 1);
      if (i < 0 || j < 0 || kk < 0 || i >= a.reso[0] || j >= a.reso[1] || kk >= a.reso[2])
        continue;
      // weight of a corner = product of the distances to the opposite corner
      const float wx = (c >> 2) ? g[0] - float(g0[0]) : float(g0[0] + 1) - g[0];
      const float wy = ((c >> 1) & 1) ? g[1] - float(g0[1]) : float(g0[1] + 1) - g[1];
      const float wz = (c & 1) ? g[2] - float(g0[2]) : float(g0[2] + 1) - g[2];
      const float w = __fmul_rn(__fmul_rn(wz, wy), wx);  // grid_sample's (W, H, D) order
      if (w > 0.f)
        atomicAdd(acc + (int64_t(i) * a.reso[1] + j) * a.reso[2] + kk,
                  (unsigned long long)__float2ull_rn(__fmul_rn(w, 4294967296.f)));
    }
  }
}

__global__ void k_count_views_apply(unsigned long long* acc, int64_t n, float* count) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const unsigned long long v = acc[i];
  if (v > (1ull << 32)) count[i] += 1.f;
  acc[i] = 0ull;
}

}  // namespace pvdb

using namespace pvdb;

namespace {

void linspace_params(const float mn[3], const float mx[3], const int shape[3], float start[3],
                     float end[3], float step[3]) {
  for (int a = 0; a < 3; ++a) {
    start[a] = mn[a];
    end[a] = mx[a];
    step[a] = shape[a] > 1 ? (mx[a] - mn[a]) / float(shape[a] - 1) : 0.f;
  }
}

// Scratch of the counting passes, kept for the process (grown, never shrunk):
// every call that uses it synchronises its stream before returning and holds
// the lock meanwhile, so calls from several threads take turns.
struct MergeScratch {
  std::mutex mu;
  int device = -1;
  uint32_t *cnt = nullptr, *off = nullptr, *total = nullptr, *partial = nullptr;
  size_t cnt_cap = 0, off_cap = 0, total_cap = 0, partial_cap = 0;
};

MergeScratch& merge_scratch() {
  static MergeScratch* s = new MergeScratch();
  return *s;
}

// Counts and block offsets of mask (device scalar total), in the scratch.
int merge_pass(MergeScratch& m, const uint8_t* mask, int64_t n, int vec, int64_t* nblocks,
               cudaStream_t st) {
  int dev = 0;
  PVDB_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev != m.device) {
    for (uint32_t** p : {&m.cnt, &m.off, &m.total, &m.partial}) {
      dev_free(*p);
      *p = nullptr;
    }
    m.cnt_cap = m.off_cap = m.total_cap = m.partial_cap = 0;
    m.device = dev;
  }
  *nblocks = (n + kMergeBlockVox - 1) / kMergeBlockVox;
  int rc = dev_reserve((void**)&m.cnt, &m.cnt_cap, size_t(*nblocks) * 4);
  if (!rc) rc = dev_reserve((void**)&m.off, &m.off_cap, size_t(*nblocks) * 4);
  if (!rc) rc = dev_reserve((void**)&m.total, &m.total_cap, 4);
  if (rc) return rc;
  k_merge_count<<<int(*nblocks), kMergeThreads, 0, st>>>(mask, n, vec, m.cnt);
  PVDB_CHECK_LAUNCH("k_merge_count");
  return scan_exclusive_u32(m.cnt, m.off, *nblocks, m.total, &m.partial, &m.partial_cap, st);
}

int merge_total(MergeScratch& m, cudaStream_t st, uint32_t* h) {
  PVDB_CHECK_CUDA(cudaMemcpyAsync(h, m.total, 4, cudaMemcpyDeviceToHost, st));
  PVDB_CHECK_CUDA(cudaStreamSynchronize(st));
  return PVDB_OK;
}

}  // namespace

extern "C" {

int pvdb_merge_count(const uint8_t* mask, int64_t n, int64_t* n_active, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(n >= 0 && n_active, "bad argument");
  *n_active = 0;
  if (!n) return PVDB_OK;
  PVDB_REQUIRE(mask, "null mask");
  cudaStream_t st = as_stream(s);
  MergeScratch& m = merge_scratch();
  std::lock_guard<std::mutex> lk(m.mu);
  int64_t nb = 0;
  const int vec = (reinterpret_cast<uintptr_t>(mask) & 15) == 0;
  int rc = merge_pass(m, mask, n, vec, &nb, st);
  uint32_t h = 0;
  if (!rc) rc = merge_total(m, st, &h);
  if (rc) return rc;
  *n_active = h;
  return PVDB_OK;
}

int pvdb_merge_build(pvdb_grid density, pvdb_grid color, const uint8_t* mask, int32_t* index,
                     void* den_rows, void* col_rows, int64_t n_rows, int32_t row_dtype,
                     pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(density || color, "no grid given");
  PVDB_REQUIRE(mask && index, "null mask or index");
  PVDB_REQUIRE(row_dtype == 0 || row_dtype == 1, "row_dtype must be 0 (f32) or 1 (f16)");
  PVDB_REQUIRE(!density || (density->C == 1 && den_rows), "density must be a 1-channel grid with rows");
  PVDB_REQUIRE(!color || col_rows, "color rows missing");
  const pvdb_grid_s* ref = density ? density : color;
  if (density && color)
    for (int q = 0; q < 3; ++q)
      PVDB_REQUIRE(density->reso[q] == color->reso[q], "density and color resolutions differ");
  const int64_t n = int64_t(ref->reso[0]) * ref->reso[1] * ref->reso[2];
  cudaStream_t st = as_stream(s);
  MergeScratch& m = merge_scratch();
  std::lock_guard<std::mutex> lk(m.mu);
  int64_t nb = 0;
  const int vec = (reinterpret_cast<uintptr_t>(mask) & 15) == 0 &&
                  (reinterpret_cast<uintptr_t>(index) & 15) == 0;
  int rc = merge_pass(m, mask, n, vec, &nb, st);
  uint32_t h = 0;
  if (!rc) rc = merge_total(m, st, &h);
  if (rc) return rc;
  // the row buffers are sized by the caller: check before anything is written
  PVDB_REQUIRE(n_rows == int64_t(h) + 1, "n_rows must be the number of masked voxels + 1");
  MergeArgs a;
  a.has_den = density != nullptr;
  a.has_col = color != nullptr;
  if (density) a.den = density->view();
  if (color) a.col = color->view();
  else a.col.C = 0;
  for (int q = 0; q < 3; ++q) a.reso[q] = ref->reso[q];
  a.index = index;
  a.den_rows = den_rows;
  a.col_rows = col_rows;
  a.dtype = row_dtype;
  a.vec = vec;
  a.col_vec = (reinterpret_cast<uintptr_t>(col_rows) & (row_dtype == 1 ? 7 : 15)) == 0;
  k_merge_write<<<int(nb), kMergeThreads, 0, st>>>(mask, n, m.off, a);
  PVDB_CHECK_LAUNCH("k_merge_write");
  PVDB_CHECK_CUDA(cudaStreamSynchronize(st));
  return PVDB_OK;
}

int pvdb_compact_rows(const uint8_t* keep, int64_t n, const float* const* src, float* const* dst,
                      int32_t n_arrays, int64_t cap, int64_t* n_kept, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(n >= 0 && n_kept, "bad argument");
  PVDB_REQUIRE(n_arrays >= 0 && n_arrays <= 4, "at most four arrays");
  *n_kept = 0;
  if (!n) return PVDB_OK;
  PVDB_REQUIRE(keep && (n_arrays == 0 || (src && dst)), "null argument");
  CompactArgs a;
  a.narr = n_arrays;
  for (int k = 0; k < n_arrays; ++k) {
    PVDB_REQUIRE(src[k] && dst[k], "null array");
    a.src[k] = src[k];
    a.dst[k] = dst[k];
  }
  a.vec = (reinterpret_cast<uintptr_t>(keep) & 15) == 0;
  cudaStream_t st = as_stream(s);
  MergeScratch& m = merge_scratch();
  std::lock_guard<std::mutex> lk(m.mu);
  int64_t nb = 0;
  int rc = merge_pass(m, keep, n, a.vec, &nb, st);
  uint32_t h = 0;
  if (!rc) rc = merge_total(m, st, &h);
  if (rc) return rc;
  // the destination rows are sized by the caller: check before anything is written
  PVDB_REQUIRE(int64_t(h) <= cap, "destination arrays hold fewer rows than the kept count");
  *n_kept = h;
  if (h && n_arrays) {
    k_compact_rows<<<int(nb), kMergeThreads, 0, st>>>(keep, n, m.off, a);
    PVDB_CHECK_LAUNCH("k_compact_rows");
    PVDB_CHECK_CUDA(cudaStreamSynchronize(st));
  }
  return PVDB_OK;
}

int pvdb_grid_resample(pvdb_grid src, pvdb_grid dst, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(src && dst, "null grid");
  PVDB_REQUIRE(src->C == dst->C, "channel counts differ");
  AxisMap m;
  for (int q = 0; q < 3; ++q) {
    m.in[q] = src->reso[q];
    m.scale[q] = dst->reso[q] > 1 ? float(src->reso[q] - 1) / float(dst->reso[q] - 1) : 0.f;
  }
  const int64_t n = dst->nslots();
  if (n) {
    const int64_t cols = int64_t(dst->nleaf) * 64;
    // one channel: a thread per z column; wider voxels: a thread per voxel
    // (per-thread columns of 48-byte rows lose memory parallelism)
    if (dst->C == 1) {
      k_resample_col<<<ceil_div(cols, 256), 256, 0, as_stream(s)>>>(src->view(), dst->view(), m);
    } else {
      k_resample<<<ceil_div(n, 256), 256, 0, as_stream(s)>>>(src->view(), dst->view(), m);
    }
    PVDB_CHECK_LAUNCH("k_resample");
  }
  data_written(dst);
  return PVDB_OK;
}

int pvdb_occupancy(pvdb_grid density, int32_t mode, uint8_t* mask, const int32_t shape[3],
                   const float xyz_min[3], const float xyz_max[3], float act_shift,
                   float interval, float thres, const uint8_t* old_mask,
                   const int32_t old_shape[3], pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(density && density->C == 1, "density must be a 1-channel grid");
  PVDB_REQUIRE(mode >= 0 && mode <= 2, "mode must be 0, 1 or 2");
  PVDB_REQUIRE(mask && shape && xyz_min && xyz_max, "null argument");
  for (int q = 0; q < 3; ++q) PVDB_REQUIRE(shape[q] > 0, "empty mask shape");
  if (mode != 0)
    for (int q = 0; q < 3; ++q)
      PVDB_REQUIRE(shape[q] == density->reso[q], "mask shape must equal the grid resolution");
  PVDB_REQUIRE(!old_mask || old_shape, "old mask without a shape");
  OccArgs a;
  a.den = density->view();
  a.mode = mode;
  int sh[3];
  for (int q = 0; q < 3; ++q) {
    sh[q] = shape[q];
    a.shape[q] = shape[q];
    a.ext[q] = xyz_max[q] - xyz_min[q];
    a.wsm1[q] = float(density->reso[q] - 1);
  }
  linspace_params(xyz_min, xyz_max, sh, a.lin_start, a.lin_end, a.lin_step);
  a.old_mask = mode == 1 ? old_mask : nullptr;
  for (int q = 0; q < 3; ++q) {
    a.old_shape[q] = a.old_mask ? old_shape[q] : 1;
    // MaskGrid buffers (grid.py:230-232): scale = (shape-1)/(max-min), shift = -min*scale
    a.old_scale[q] = a.old_mask ? float(a.old_shape[q] - 1) / (xyz_max[q] - xyz_min[q]) : 0.f;
    a.old_shift[q] = -xyz_min[q] * a.old_scale[q];
  }
  a.shift = act_shift;
  a.interval = interval;
  a.thres = thres;
  a.out = mask;
  const int64_t tiles = int64_t((sh[0] + kOccTile - 1) / kOccTile) *
                        ((sh[1] + kOccTile - 1) / kOccTile) * ((sh[2] + kOccTile - 1) / kOccTile);
  k_occupancy<<<int(tiles), 512, 0, as_stream(s)>>>(a);
  PVDB_CHECK_LAUNCH("k_occupancy");
  return PVDB_OK;
}

int pvdb_grid_maskout_near_cams(pvdb_grid g, const float* cam_o, int32_t n_cams,
                                const float xyz_min[3], const float xyz_max[3], float near_clip,
                                float value, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(g && xyz_min && xyz_max, "null argument");
  PVDB_REQUIRE(n_cams >= 0, "negative camera count");
  if (!n_cams) return PVDB_OK;
  PVDB_REQUIRE(cam_o, "null cameras");
  NearCamArgs a;
  a.g = g->view();
  a.cams = cam_o;
  a.n_cams = n_cams;
  linspace_params(xyz_min, xyz_max, g->reso, a.lin_start, a.lin_end, a.lin_step);
  a.near_clip = near_clip;
  a.value = value;
  const int64_t n = g->nslots();
  if (n) {
    k_near_cams<<<ceil_div(n, 256), 256, 0, as_stream(s)>>>(a);
    PVDB_CHECK_LAUNCH("k_near_cams");
  }
  data_written(g);
  return PVDB_OK;
}

int pvdb_count_views(const float* rays_o, const float* rays_d, int64_t n_rays,
                     const int32_t reso[3], const float xyz_min[3], const float xyz_max[3],
                     float near_, float stepdist, int32_t n_samples, uint64_t* acc, float* count,
                     pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(reso && xyz_min && xyz_max && acc && count, "null argument");
  PVDB_REQUIRE(n_rays >= 0 && n_samples > 0, "bad sizes");
  for (int q = 0; q < 3; ++q) PVDB_REQUIRE(reso[q] > 0, "bad resolution");
  const int64_t nvox = int64_t(reso[0]) * reso[1] * reso[2];
  cudaStream_t st = as_stream(s);
  if (n_rays) {
    PVDB_REQUIRE(rays_o && rays_d, "null rays");
    CountArgs a;
    for (int q = 0; q < 3; ++q) {
      a.reso[q] = reso[q];
      a.xyz_min[q] = xyz_min[q];
      a.xyz_max[q] = xyz_max[q];
    }
    a.near_ = near_;
    a.stepdist = stepdist;
    a.n_samples = n_samples;
    const int64_t total = n_rays * n_samples;
    const int grid = int(std::min<int64_t>((total + 255) / 256, int64_t(num_sms()) * 16));
    k_count_views_acc<<<grid, 256, 0, st>>>(rays_o, rays_d, n_rays, a,
                                             reinterpret_cast<unsigned long long*>(acc));
    PVDB_CHECK_LAUNCH("k_count_views_acc");
  }
  k_count_views_apply<<<ceil_div(nvox, 256), 256, 0, st>>>(
      reinterpret_cast<unsigned long long*>(acc), nvox, count);
  PVDB_CHECK_LAUNCH("k_count_views_apply");
  return PVDB_OK;
}

}  // extern "C"
