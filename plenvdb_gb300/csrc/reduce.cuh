// Deterministic leaf-sorted segmented reduction of trilinear gradient
// contributions into voxel gradients (replaces the float atomicAdd scatter of
// densityvdb.cu:16-27 / colorvdb.cu:28-37).
//
// A contribution is (sample s, corner c) with id = s*8 + c and key = the slot
// (leaf*512 + voxel offset) of that corner, or kInvalidKey when the corner lies
// in no allocated leaf (the reference drops those, densityvdb.cu:23). Keys are
// written at their canonical position (the id), stably radix-sorted by slot, so
// each slot's contributions form one contiguous segment in ascending id order;
// the segment head sums it sequentially in that order and adds the sum into the
// gradient. The result is bitwise reproducible run to run.
#pragma once
#include "pvdb_internal.cuh"

namespace pvdb {

constexpr uint32_t kInvalidKey = 0xFFFFFFFFu;

// Radix sort tiling (reduce.cu): keys per tile and bins per 8-bit digit. The
// sort keeps one histogram of kRsBins words per tile.
constexpr int kRsThreads = 256;
constexpr int kRsRounds = 4;                     // keys per lane
constexpr int kRsTile = kRsThreads * kRsRounds;  // 1024 keys per tile
constexpr int kRsBins = 256;

// Writes the 8 corner keys of one sample at keys[s*8 .. s*8+7].
__device__ __forceinline__ void emit_corner_keys(const GridView& g, float x, float y, float z,
                                                 uint32_t* keys, int64_t s) {
  const int i = ifloor(x), j = ifloor(y), k = ifloor(z);
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    int di, dj, dk;
    corner_delta(c, di, dj, dk);
    const int sl = slot_of(g, i + di, j + dj, k + dk);
    keys[s * 8 + c] = sl < 0 ? kInvalidKey : uint32_t(sl);
  }
}

// Leaf-major key of the trilinear cell (or voxel) (i,j,k) over the dense leaf
// lattice [0, 8*ldim): dense leaf index * 512 + NanoVDB voxel offset; defined
// whether or not the leaf is allocated. kInvalidKey outside the lattice.
__device__ __forceinline__ uint32_t cell_key(const int ld[3], int i, int j, int k) {
  if ((unsigned)i >= (unsigned)(ld[0] << 3) || (unsigned)j >= (unsigned)(ld[1] << 3) ||
      (unsigned)k >= (unsigned)(ld[2] << 3))
    return kInvalidKey;
  return (uint32_t(((i >> 3) * ld[1] + (j >> 3)) * ld[2] + (k >> 3)) << 9) | uint32_t(vox_offset(i, j, k));
}

// Source of contributions for the segmented reduce:
//   pos(s)       -> index-space position of sample s
//   gd(s)        -> density gradient of sample s (scalar grid)
//   gc(s, ch)    -> feature gradient of sample s, channel ch (multi-channel grid)
//   has_c(s)     -> whether sample s carries a feature gradient
template <class Src>
__device__ __forceinline__ void segment_reduce_one(const uint32_t* __restrict__ skeys,
                                                   const uint32_t* __restrict__ svals, int64_t n,
                                                   int64_t i, const Src& src, float* grad_d,
                                                   float* grad_c, int Cc, uint8_t* touched_d,
                                                   uint8_t* touched_c) {
  const uint32_t key = skeys[i];
  if (key == kInvalidKey) return;
  if (i > 0 && skeys[i - 1] == key) return;  // not a segment head
  int64_t end = i + 1;
  while (end < n && skeys[end] == key) ++end;
  if (grad_d) {
    // density pattern ((g*a)*b)*c, summed in ascending id order
    float sum = 0.f;
    bool any = false;
    for (int64_t j = i; j < end; ++j) {
      const uint32_t id = svals[j];
      const int64_t s = id >> 3;
      const float gd = src.gd(s);
      if (gd == 0.f) continue;
      float x, y, z;
      src.pos(s, x, y, z);
      const float u = x - float(ifloor(x)), v = y - float(ifloor(y)), w = z - float(ifloor(z));
      sum = __fadd_rn(sum, density_corner_term(gd, u, v, w, int(id & 7)));
      any = true;
    }
    if (any) {
      grad_d[key] = __fadd_rn(grad_d[key], sum);
      if (touched_d) touched_d[key >> 9] = 1;
    }
  }
  if (grad_c) {
    // feature pattern g[ch]*scale, channels in register chunks of 12
    for (int ch0 = 0; ch0 < Cc; ch0 += 12) {
      const int nch = min(12, Cc - ch0);
      float acc[12];
#pragma unroll
      for (int q = 0; q < 12; ++q) acc[q] = 0.f;
      bool any = false;
      for (int64_t j = i; j < end; ++j) {
        const uint32_t id = svals[j];
        const int64_t s = id >> 3;
        if (!src.has_c(s)) continue;
        float x, y, z;
        src.pos(s, x, y, z);
        float sc[8];
        corner_scales(x - float(ifloor(x)), y - float(ifloor(y)), z - float(ifloor(z)), sc);
        const float scale = sc[id & 7];
        any = true;
#pragma unroll
        for (int q = 0; q < 12; ++q)
          if (q < nch) acc[q] = __fadd_rn(acc[q], __fmul_rn(src.gc(s, ch0 + q), scale));
      }
      if (any) {
        float* dst = grad_c + int64_t(key) * Cc + ch0;
        for (int q = 0; q < nch; ++q) dst[q] = __fadd_rn(dst[q], acc[q]);
        if (touched_c) touched_c[key >> 9] = 1;
      }
    }
  }
}

// Grid-stride over the sorted contributions; the count may live on the device.
template <class Src>
__global__ void k_segment_reduce(const uint32_t* __restrict__ skeys,
                                 const uint32_t* __restrict__ svals, int64_t n_max,
                                 const uint32_t* n_dev, Src src, float* grad_d, float* grad_c,
                                 int Cc, uint8_t* touched_d, uint8_t* touched_c,
                                 const uint32_t* status = nullptr) {
  grid_dep_sync();
  if (status && *status) return;  // the sort gave up a wait: its order is wrong
  const int64_t n = n_dev ? min(n_max, (int64_t)*n_dev) : n_max;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x)
    segment_reduce_one(skeys, svals, n, i, src, grad_d, grad_c, Cc, touched_d, touched_c);
}

}  // namespace pvdb
