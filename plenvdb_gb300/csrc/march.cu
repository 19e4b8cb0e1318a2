// Fused training march over ragged per-ray sample counts.
//
// Forward (k_march_setup / k_march_alpha / k_march_chain) covers, per ray:
// sample_pts_on_rays (render_utils_kernel.cu:196-242), the bbox filter and
// MaskGrid lookup (dvgo.py:290-315), wld2idx (grid.py:77-78), DensityVDB
// trilinear (densityvdb.cu:101-125), raw2alpha (render_utils_kernel.cu:430-443),
// the alpha threshold (dvgo.py:319-325) and alpha2weight with its T < 1e-3
// early stop (render_utils_kernel.cu:576-605). Samples in bricks whose density
// bound keeps alpha below the threshold skip the trilinear (they would be
// dropped anyway). The transmittance chain is walked in sample order over the
// kept samples. Only per-ray alpha / weight / step lists are kept for the
// backward.
//
// k_march_chain also lays the colour samples (weight > thres,
// dvgo.py:329-335) out as dense rows, and k_march_k0 samples the k0 grid there
// (colorvdb.cu:81-111).
//
// Backward (k_march_bwd) recovers transmittance from the saved alphas and
// weights, runs alpha2weight_backward (:653-677) as a suffix scan and
// raw2alpha_backward (:506-517), and keys every kept sample by its trilinear
// cell; a counting placement groups the samples by cell in sample order and a
// per-voxel gather over the touched leaves then adds the density and k0
// gradients deterministically (see the reduction below).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>

#include "march.cuh"
#include "reduce.cuh"
#include "tc.cuh"

namespace pvdb {

constexpr int kMarchWarps = 8;
constexpr int kMarchThreads = kMarchWarps * 32;

__device__ __forceinline__ void load_ray(const float* __restrict__ ro, const float* __restrict__ rd,
                                         int r, float o[3], float d[3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    o[a] = __ldg(ro + r * 3 + a);
    d[a] = __ldg(rd + r * 3 + a);
  }
}

// Forward, in three passes:
//  k_march_setup (thread per ray): slab test, sample count, start point and
//    unit direction;
//  k_march_alpha (thread per (ray, sample)): position, brick-bound skip,
//    density trilinear and raw2alpha; writes alpha (0 for a sample that is not
//    kept) into the ray's slots — independent work, so the gathers of all
//    samples are in flight together;
//  k_march_chain (warp per ray): the transmittance chain over the kept
//    samples in order, the T < t_stop early stop, and the in-place compaction
//    of the kept samples (a kept sample moves to a slot at or before its own,
//    after the whole chunk has been read); then the ray's offsets among all
//    kept samples and colour rows, and its colour rows' records.
__global__ void __launch_bounds__(256)
    k_march_setup(const float* __restrict__ ro, const float* __restrict__ rd, int R, MarchP P,
                  MarchW W) {
  grid_dep_sync();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  float o[3], d[3];
  load_ray(ro, rd, r, o, d);
  RaySetup rs;
  ray_setup(o, d, P.mn, P.mx, P.near_, P.far_, P.stepdist, rs);
  int64_t ns = rs.n_steps;
  if (ns > P.cap) {
    atomicOr(W.totals + 3, 1u);
    ns = P.cap;
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    W.ray_sd[r * 6 + a] = rs.start[a];
    W.ray_sd[r * 6 + 3 + a] = rs.dir[a];
  }
  W.ray_ns[r] = int32_t(ns);
  atomicAdd(W.totals + 4, uint32_t(ns));
  W.chain_status[r] = 0ull;  // k_march_chain look-back status of this ray
}

// Sample k of a ray: its index-space position when the sample is evaluated
// (its brick bound does not rule it out, it lies in the bbox and, with a mask,
// in the mask); false otherwise (alpha 0).
__device__ __forceinline__ bool alpha_eval_index(const GridView& gd, const MarchP& P,
                                                 const RaySetup& rs, int k, float idx[3]) {
  float p[3];
  ray_point(rs, P.stepdist, k, p);
  if (gd.bmax) {
    // brick of the (approximate) cell; its bound covers the cells next to it
    int b[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
      b[a] = min(max(int(floorf((p[a] - P.mn[a]) * P.binv[a])), 0), gd.bdim[a] - 1);
    const uint32_t key = __ldg(gd.bmax + (b[0] * gd.bdim[1] + b[1]) * gd.bdim[2] + b[2]);
    if (fkey_inv(key) < P.sigma_skip) return false;
  }
  if (out_of_bbox(p, P.mn, P.mx) ||
      (P.mask && !mask_lookup(P.mask, P.mshape, p, P.mscale, P.mshift)))
    return false;
  world_to_index(p, P.mn, P.ext, P.wsm1, idx);
  return true;
}

__device__ __forceinline__ float alpha_of(const MarchP& P, float sigma) {
  float e;
  const float a = raw2alpha(sigma, P.shift, P.interval, e);
  return a > P.thr ? a : 0.f;
}

__device__ __forceinline__ void load_ray_setup(const MarchW& W, int r, RaySetup& rs) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    rs.start[a] = W.ray_sd[r * 6 + a];
    rs.dir[a] = W.ray_sd[r * 6 + 3 + a];
  }
}

// One block per ray, threads over the ray's samples.
__global__ void __launch_bounds__(256)
    k_march_alpha(GridView gd, MarchP P, MarchW W) {
  grid_dep_sync();
  const int r = blockIdx.x;
  const int ns = W.ray_ns[r];
  RaySetup rs;
  load_ray_setup(W, r, rs);
  const int64_t sbase = int64_t(r) * P.cap;
  for (int k = threadIdx.x; k < ns; k += blockDim.x) {
    float idx[3];
    float alpha = 0.f;
    if (alpha_eval_index(gd, P, rs, k, idx)) alpha = alpha_of(P, trilinear1(gd, idx[0], idx[1], idx[2]));
    W.k_alpha[sbase + k] = alpha;
  }
}

// The same pass with the density leaves staged in shared memory
// (pvdb_march_set_leaf_staging). A block first walks its ray's samples and
// collects, in an open-addressing table, the leaves of every corner of every
// evaluated sample; up to kStageSlots of them are copied into shared memory
// with one 1-D bulk copy each (cp.async.bulk, 2 KB, completion counted on one
// mbarrier); then it walks the samples again and interpolates, reading staged
// leaves from shared memory and the others (beyond the slots, or all of them
// after a copy wait that gave up: error bit 8) from global memory. The values
// and the arithmetic are those of k_march_alpha.
constexpr int kStageSlots = 24;                 // 48 KB of density leaves per block
constexpr int kStageHash = 128;                 // table entries (a power of two)
constexpr uint32_t kStageSpinMax = 1u << 22;
constexpr size_t kStageSmem = size_t(kStageSlots) * kLeafVox * 4;

__device__ __forceinline__ uint32_t stage_hash(int leaf) {
  return (uint32_t(leaf) * 2654435761u) >> 25;  // 7 bits: kStageHash entries
}

// Staging slot of a leaf, -1 when it is not staged.
__device__ __forceinline__ int stage_find(const int32_t* hkey, const int16_t* hslot, int leaf) {
  uint32_t h = stage_hash(leaf);
  for (int t = 0; t < kStageHash; ++t, h = (h + 1) & (kStageHash - 1)) {
    const int key = hkey[h];
    if (key == leaf) return hslot[h];
    if (key < 0) return -1;
  }
  return -1;
}

__device__ __forceinline__ void stage_insert(int32_t* hkey, int16_t* hslot, uint32_t* nslot,
                                             int leaf) {
  uint32_t h = stage_hash(leaf);
  for (int t = 0; t < kStageHash; ++t, h = (h + 1) & (kStageHash - 1)) {
    const int old = atomicCAS(hkey + h, -1, leaf);
    if (old == -1) {
      const uint32_t slot = atomicAdd(nslot, 1u);
      hslot[h] = int16_t(slot < uint32_t(kStageSlots) ? int(slot) : -1);
      return;
    }
    if (old == leaf) return;
  }
}

__global__ void __launch_bounds__(256)
    k_march_alpha_staged(GridView gd, MarchP P, MarchW W, uint32_t spin_max, int hold) {
  grid_dep_sync();
  extern __shared__ __align__(128) float st_vox[];  // [kStageSlots][512]
  __shared__ int32_t hkey[kStageHash];
  __shared__ int16_t hslot[kStageHash];
  __shared__ uint32_t nslot;
  __shared__ __align__(8) uint64_t bar;
  const int r = blockIdx.x;
  const int ns = W.ray_ns[r];
  RaySetup rs;
  load_ray_setup(W, r, rs);
  for (int h = threadIdx.x; h < kStageHash; h += blockDim.x) hkey[h] = -1;
  if (threadIdx.x == 0) {
    nslot = 0;
    tc::mbar_init(&bar, 1);
  }
  __syncthreads();
  // the leaves of the evaluated samples' corners
  for (int k = threadIdx.x; k < ns; k += blockDim.x) {
    float idx[3];
    if (!alpha_eval_index(gd, P, rs, k, idx)) continue;
    const int i = ifloor(idx[0]), j = ifloor(idx[1]), kk = ifloor(idx[2]);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      int di, dj, dk;
      corner_delta(c, di, dj, dk);
      // a corner in another leaf than corner 0 only where the cell crosses a leaf face
      if (c > 0 && !(((i & 7) == 7 && di) || ((j & 7) == 7 && dj) || ((kk & 7) == 7 && dk)))
        continue;
      const int l = leaf_of(gd, i + di, j + dj, kk + dk);
      if (l >= 0) stage_insert(hkey, hslot, &nslot, l);
    }
  }
  __syncthreads();
  const uint32_t nstaged = min(nslot, uint32_t(kStageSlots));
  bool staged = nstaged > 0;
  if (staged) {
    __shared__ int held;
    if (threadIdx.x == 0) {
      tc::mbar_expect_tx(&bar, nstaged * uint32_t(kLeafVox * 4));
      // test hook: the first block with leaves to stage issues no copies
      held = hold && atomicCAS(W.totals + 2, 0u, 1u) == 0u;
    }
    __syncthreads();  // the transaction count is set before any copy lands
    if (threadIdx.x < 32 && !held) {
      for (int h = threadIdx.x; h < kStageHash; h += 32) {
        const int l = hkey[h], sl = hslot[h];
        if (l >= 0 && sl >= 0)
          tc::bulk_g2s(st_vox + sl * kLeafVox, gd.data + int64_t(l) * kLeafVox,
                       uint32_t(kLeafVox * 4), &bar);
      }
    }
    if (!tc::mbar_wait(&bar, 0, spin_max)) {
      atomicOr(W.totals + 3, 8u);
      staged = false;
    }
  }
  const int64_t sbase = int64_t(r) * P.cap;
  for (int k = threadIdx.x; k < ns; k += blockDim.x) {
    float idx[3];
    float alpha = 0.f;
    if (alpha_eval_index(gd, P, rs, k, idx)) {
      const int i = ifloor(idx[0]), j = ifloor(idx[1]), kk = ifloor(idx[2]);
      const float u = idx[0] - float(i), v = idx[1] - float(j), w = idx[2] - float(kk);
      const bool inner = (i & 7) != 7 && (j & 7) != 7 && (kk & 7) != 7;
      const int l0 = leaf_of(gd, i, j, kk);
      const int s0 = staged && l0 >= 0 ? stage_find(hkey, hslot, l0) : -1;
      float val[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        int di, dj, dk;
        corner_delta(c, di, dj, dk);
        const int off = vox_offset(i + di, j + dj, kk + dk);
        int l = l0, sl = s0;
        if (!inner && c > 0) {
          l = leaf_of(gd, i + di, j + dj, kk + dk);
          sl = staged && l >= 0 ? stage_find(hkey, hslot, l) : -1;
        }
        val[c] = l < 0 ? gd.background
                 : sl >= 0 ? st_vox[sl * kLeafVox + off]
                           : __ldg(gd.data + (int64_t(l) << 9) + off);
      }
      alpha = alpha_of(P, trilinear1_values(val, u, v, w));
    }
    W.k_alpha[sbase + k] = alpha;
  }
  if (nstaged > 0 && !staged && threadIdx.x == 0)
    tc::mbar_wait(&bar, 0, spin_max);  // copies still in flight land before the block exits
}

constexpr int kChainBatch = 8;  // 32-sample chunks whose alphas are loaded together

// Ray offsets: warps take rays in order from a counter (totals[6]); a ray
// publishes its (colour, kept) counts, then sums the earlier rays' published
// counts back to the first inclusive prefix, 32 rays at a time (decoupled
// look-back). A ray publishes before it waits and only waits on rays taken
// earlier (running or done), so every wait ends; each is still bounded, and
// one that gives up sets error bit 4.
constexpr uint64_t kChainAgg = 1ull << 62;     // status: ray counts published
constexpr uint64_t kChainPrefix = 1ull << 63;  // status: inclusive prefix published
constexpr uint64_t kChainValue = kChainAgg - 1;
constexpr uint32_t kChainSpinMax = 1u << 24;

__global__ void __launch_bounds__(kMarchThreads)
    k_march_chain(int R, MarchP P, MarchW W, uint32_t spin_max, int hold_first) {
  grid_dep_sync();
  const int lane = threadIdx.x & 31;
  uint32_t ticket = 0;
  if (lane == 0) ticket = atomicAdd(W.totals + 6, 1u);
  const int r = int(__shfl_sync(0xffffffffu, ticket, 0));
  if (r >= R) return;
  const unsigned lt = lanemask_lt();
  const int64_t sbase = int64_t(r) * P.cap;
  int nk = 0, nc = 0;
  {
    const int ns = W.ray_ns[r];
    float T = 1.f;
    bool stop = false;
    for (int b0 = 0; b0 < ns && !stop; b0 += 32 * kChainBatch) {
      // the batch's alphas, loaded before any of them is used
      float al[kChainBatch];
#pragma unroll
      for (int j = 0; j < kChainBatch; ++j) {
        const int k = b0 + 32 * j + lane;
        al[j] = k < ns ? W.k_alpha[sbase + k] : 0.f;
      }
      __syncwarp();  // every lane has read its alphas before the compaction writes
#pragma unroll
      for (int j = 0; j < kChainBatch; ++j) {
        if (stop) continue;
        const int k = b0 + 32 * j + lane;
        unsigned km = __ballot_sync(0xffffffffu, al[j] > P.thr);
        // alpha2weight over the kept lanes, in sample order (uniform across the warp)
        float w = 0.f;
        unsigned rem = km;
        while (rem) {
          const int l = __ffs(rem) - 1;
          rem &= rem - 1;
          const float a = __shfl_sync(0xffffffffu, al[j], l);
          const float wl = T * a;
          if (lane == l) w = wl;
          T = trans_step(T, a);
          if (T < P.t_stop) {
            km &= (l == 31) ? 0xffffffffu : ((2u << l) - 1u);
            stop = true;
            break;
          }
        }
        const bool kept = (km >> lane) & 1u;
        const bool col = kept && (w > P.thr);
        const unsigned cm = __ballot_sync(0xffffffffu, col);
        if (kept) {
          const int64_t pos = sbase + nk + __popc(km & lt);
          W.k_alpha[pos] = al[j];
          W.k_w[pos] = w;
          W.k_step[pos] = int32_t(k) | (col ? int32_t(0x80000000) : 0);
          W.k_row[pos] = col ? nc + __popc(cm & lt) : -1;  // rank among the ray's colour rows
        }
        nk += __popc(km);
        nc += __popc(cm);
      }
    }
    if (lane == 0) {
      W.T_last[r] = T;
      W.n_kept[r] = nk;
      W.n_color[r] = nc;
    }
  }
  // publish, then look back 32 rays at a time
  const uint64_t agg = (uint64_t(nc) << 32) | uint64_t(uint32_t(nk));
  volatile uint64_t* status = W.chain_status;
  // (hold_first: the test hook of the bounded waits withholds ray 0's counts)
  if (lane == 0 && !(hold_first && r == 0)) status[r] = (r == 0 ? kChainPrefix : kChainAgg) | agg;
  uint32_t ex_k = 0, ex_c = 0;  // exclusive prefix (kept, colour)
  for (int t = r - 1; t >= 0; t -= 32) {
    const int j = t - lane;
    uint64_t v = j >= 0 ? uint64_t(status[j]) : uint64_t(kChainPrefix);
    for (uint32_t it = 0; __any_sync(0xffffffffu, v == 0ull); ++it) {
      if (it >= spin_max) {
        if (lane == 0) atomicOr(W.totals + 3, 4u);
        v = v ? v : uint64_t(kChainPrefix);  // give up: offsets wrong, but the kernel ends
        break;
      }
      if (v == 0ull) v = status[j];
    }
    const unsigned pm = __ballot_sync(0xffffffffu, (v & kChainPrefix) != 0ull);
    const int stop_lane = pm ? __ffs(pm) - 1 : 31;  // nearest ray with a prefix
    const uint64_t val = lane <= stop_lane && j >= 0 ? (v & kChainValue) : 0ull;
    ex_k += __reduce_add_sync(0xffffffffu, uint32_t(val));
    ex_c += __reduce_add_sync(0xffffffffu, uint32_t(val >> 32));
    if (pm) break;
  }
  const uint64_t excl = (uint64_t(ex_c) << 32) | ex_k;
  if (lane == 0) {
    if (r > 0) status[r] = kChainPrefix | (excl + agg);
    W.kept_off[r] = ex_k;
    W.color_off[r] = ex_c;
    if (r == R - 1) {
      W.totals[0] = uint32_t(excl + agg);
      W.totals[1] = uint32_t((excl + agg) >> 32);
    }
  }
  // colour rows: global row m = color_off + rank, the row record, k_row = m
  // (the kept records of four 32-sample chunks are loaded together)
  for (int i0 = lane; i0 < nk; i0 += 4 * 32) {
    int32_t rank[4], step[4];
    float wv[4], av[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + 32 * u;
      const int64_t t = sbase + i;
      rank[u] = i < nk ? W.k_row[t] : -1;
      wv[u] = i < nk ? W.k_w[t] : 0.f;
      av[u] = i < nk ? W.k_alpha[t] : 0.f;
      step[u] = i < nk ? W.k_step[t] : 0;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (rank[u] < 0) continue;
      const int64_t t = sbase + i0 + 32 * u;
      const int64_t m = int64_t(ex_c) + rank[u];
      W.r_w[m] = wv[u];
      W.r_alpha[m] = av[u];
      W.r_ray[m] = r;
      W.r_step[m] = step[u] & 0x7fffffff;
      W.k_row[t] = int32_t(m);
    }
  }
}

__device__ __forceinline__ void load_setup(const MarchW& W, int r, RaySetup& rs) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    rs.start[a] = W.ray_sd[r * 6 + a];
    rs.dir[a] = W.ray_sd[r * 6 + 3 + a];
  }
}

// Multi-channel trilinear of k0 at one point (colorvdb.cu:97-108 ordering).
// The 12-channel case: the channels in three 16-byte loads per corner.
__device__ __forceinline__ void k0_trilinear12(const GridView& g, const float idx[3], float* out) {
  const int i = ifloor(idx[0]), j = ifloor(idx[1]), k = ifloor(idx[2]);
  float sc[8];
  corner_scales(idx[0] - float(i), idx[1] - float(j), idx[2] - float(k), sc);
  int slots[8];
  corner_slots(g, i, j, k, slots);
  float acc[12];
#pragma unroll
  for (int q = 0; q < 12; ++q) acc[q] = 0.f;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    float v[12];
    if (slots[c] >= 0) {
      const float4* src = reinterpret_cast<const float4*>(g.data + int64_t(slots[c]) * 12);
      const float4 a = __ldg(src), b = __ldg(src + 1), cc = __ldg(src + 2);
      v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
      v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
      v[8] = cc.x; v[9] = cc.y; v[10] = cc.z; v[11] = cc.w;
    } else {
#pragma unroll
      for (int q = 0; q < 12; ++q) v[q] = g.background;
    }
#pragma unroll
    for (int q = 0; q < 12; ++q) acc[q] = __fadd_rn(acc[q], __fmul_rn(v[q], sc[c]));
  }
#pragma unroll
  for (int q = 0; q < 12; ++q) out[q] = acc[q];
}

__device__ __forceinline__ void k0_trilinear(const GridView& g, const float idx[3], float* out) {
  if (g.C == 12) {
    k0_trilinear12(g, idx, out);
    return;
  }
  const int i = ifloor(idx[0]), j = ifloor(idx[1]), k = ifloor(idx[2]);
  float sc[8];
  corner_scales(idx[0] - float(i), idx[1] - float(j), idx[2] - float(k), sc);
  int slots[8];
  corner_slots(g, i, j, k, slots);
  for (int ch = 0; ch < g.C; ++ch) {
    float acc = 0.f;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const float v = slots[c] < 0 ? g.background : __ldg(g.data + int64_t(slots[c]) * g.C + ch);
      acc = __fadd_rn(acc, __fmul_rn(v, sc[c]));
    }
    out[ch] = acc;
  }
}

// The 12-channel trilinear from the grid's BF16 shadow (the BF16 train step):
// one 32-byte record per corner in two 16-byte loads, FP32 interpolation in
// the order of k0_trilinear.
__device__ __forceinline__ void k0_trilinear_half(const GridView& g,
                                                  const __nv_bfloat16* __restrict__ half,
                                                  const float idx[3], float* out) {
  const int i = ifloor(idx[0]), j = ifloor(idx[1]), k = ifloor(idx[2]);
  float sc[8];
  corner_scales(idx[0] - float(i), idx[1] - float(j), idx[2] - float(k), sc);
  int slots[8];
  corner_slots(g, i, j, k, slots);
  uint4 lo[8];
  uint2 hi[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    if (slots[c] >= 0) {
      const uint4* src = reinterpret_cast<const uint4*>(half + int64_t(slots[c]) * kHalfStride);
      lo[c] = __ldg(src);
      const uint4 h = __ldg(src + 1);
      hi[c] = make_uint2(h.x, h.y);
    }
  }
  float acc[12];
#pragma unroll
  for (int q = 0; q < 12; ++q) acc[q] = 0.f;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    float v[12];
    if (slots[c] >= 0) {
      const uint32_t w[6] = {lo[c].x, lo[c].y, lo[c].z, lo[c].w, hi[c].x, hi[c].y};
#pragma unroll
      for (int b = 0; b < 6; ++b) {
        v[2 * b] = __uint_as_float(w[b] << 16);
        v[2 * b + 1] = __uint_as_float(w[b] & 0xFFFF0000u);
      }
    } else {
#pragma unroll
      for (int q = 0; q < 12; ++q) v[q] = g.background;
    }
#pragma unroll
    for (int q = 0; q < 12; ++q) acc[q] = __fadd_rn(acc[q], __fmul_rn(v[q], sc[c]));
  }
#pragma unroll
  for (int q = 0; q < 12; ++q) out[q] = acc[q];
}

// k_march_k0 (thread per colour row): the k0 trilinear at the row's position
// (colorvdb.cu:81-111).
__global__ void __launch_bounds__(256)
    k_march_k0(GridView gk, MarchP P, MarchW W) {
  grid_dep_sync();
  const int64_t M = W.totals[1];
  for (int64_t m = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; m < M;
       m += int64_t(gridDim.x) * blockDim.x) {
    const int r = W.r_ray[m];
    RaySetup rs;
    load_setup(W, r, rs);
    float p[3], idx[3];
    ray_point(rs, P.stepdist, W.r_step[m], p);
    world_to_index(p, P.mn, P.ext, P.wsm1, idx);
    k0_trilinear(gk, idx, W.r_k0 + m * gk.C);
  }
}

// BF16 tensor-core path of the train step: the k0 trilinear of each colour row
// goes straight into the row of its X tile ([k0 | PE | 1 | 0], BF16), so the
// FP32 k0 rows are never written. pe: per-ray PE (pe_stride floats per ray).
// The padding rows of the last tile are zero.
// MINB: resident blocks per SM the register budget is cut for (2: 128
// registers, no spills; 3: 80 registers with a few spilled values — faster
// once the rows fill several waves).
template <int CT, int MINB>
__global__ void __launch_bounds__(256, MINB)
    k_march_k0_x(GridView gk, MarchP P, MarchW W, const float* __restrict__ pe, int pe_stride,
                 int dpe, uint8_t* xt, const __nv_bfloat16* __restrict__ half) {
  grid_dep_sync();
  // CT = 12: the channel count is a compile-time constant, so the row's
  // features stay in registers; CT = 0: any count up to 16
  const int64_t M = W.totals[1];
  const int64_t Mpad = (M + 127) / 128 * 128;
  const int C = CT ? CT : gk.C, din = C + dpe;
  for (int64_t m = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; m < Mpad;
       m += int64_t(gridDim.x) * blockDim.x) {
    float k0v[16];
    int r = 0;
    if (m < M) {
      r = W.r_ray[m];
      RaySetup rs;
      load_setup(W, r, rs);
      float p[3], idx[3];
      ray_point(rs, P.stepdist, W.r_step[m], p);
      world_to_index(p, P.mn, P.ext, P.wsm1, idx);
      if (CT == 12) {
        if (half)
          k0_trilinear_half(gk, half, idx, k0v);
        else
          k0_trilinear12(gk, idx, k0v);
      } else {
        k0_trilinear(gk, idx, k0v);
      }
    }
    uint8_t* tile = xt + (m >> 7) * int64_t(kRgbXTile);
    const int row = int(m & 127);
#pragma unroll
    for (int cb = 0; cb < kRgbXK / 8; ++cb) {
      float v[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int q = 8 * cb + e;
        v[e] = m >= M ? 0.f
               : q < C ? k0v[q < 16 ? q : 15]
               : q < din ? __ldg(pe + int64_t(r) * pe_stride + (q - C))
               : q == din ? 1.f : 0.f;
      }
      const uint4 pk = make_uint4(tc::pack_bf16(v[0], v[1]), tc::pack_bf16(v[2], v[3]),
                                  tc::pack_bf16(v[4], v[5]), tc::pack_bf16(v[6], v[7]));
      *reinterpret_cast<uint4*>(tile + tc::kmaj(row, 8 * cb, kRgbXK)) = pk;
    }
  }
}

// Backward of the composite chain for one ray (warp per ray), chunks of 32
// kept samples from the last to the first. The transmittance before sample i
// is recovered from the saved forward weight, T_i = w_i / alpha_i (alpha_i >
// fast_color_thres > 0), so no per-sample transmittance is stored and no
// serial pass is needed. back_i = grad_last*T_last + sum_{j>i} gw_j*w_j
// (alpha2weight_backward, render_utils_kernel.cu:665-673) is an exclusive
// suffix sum: a warp shuffle scan inside the chunk plus the carry of the later
// chunks.
__global__ void __launch_bounds__(kMarchThreads)
    k_march_bwd(GridView gd, int R, MarchP P, MarchW W, const float* __restrict__ grad_w,
                const float* __restrict__ grad_last, uint32_t* keys, uint32_t* cnt,
                uint32_t* leaf_cnt, uint32_t* rank) {
  grid_dep_sync();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * kMarchWarps + warp;
  if (r >= R) return;
  const int nk = int(W.n_kept[r]);
  if (nk == 0) return;
  const int64_t sbase = int64_t(r) * P.cap;
  const int64_t kb = W.kept_off[r];
  const int nchunks = (nk + 31) >> 5;
  const unsigned lt = lanemask_lt();
  RaySetup rs;
  load_setup(W, r, rs);
  float carry = (grad_last ? grad_last[r] : 0.f) * W.T_last[r];
  for (int c = nchunks - 1; c >= 0; --c) {
    const int i = c * 32 + lane;
    const bool valid = i < nk;
    float a = 1.f, w = 0.f, gw = 0.f;
    int32_t st = 0, row = -1;
    uint32_t key = kInvalidKey;
    if (valid) {
      a = W.k_alpha[sbase + i];
      w = W.k_w[sbase + i];
      st = W.k_step[sbase + i];
      row = W.k_row[sbase + i];
      if (row >= 0 && grad_w) gw = grad_w[row];
    }
    // inclusive suffix sum of gw*w over lanes >= lane
    const float term = __fmul_rn(gw, w);
    float suf = term;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const float v = __shfl_down_sync(0xffffffffu, suf, o);
      if (lane + o < 32) suf += v;
    }
    const float back = carry + (suf - term);
    carry += __shfl_sync(0xffffffffu, suf, 0);
    if (valid) {
      const float Ti = __fdiv_rn(w, a);
      const float ga = alpha_grad(gw, Ti, back, a);
      const int32_t k = st & 0x7fffffff;
      float p[3], idx[3];
      ray_point(rs, P.stepdist, k, p);
      world_to_index(p, P.mn, P.ext, P.wsm1, idx);
      const float sigma = trilinear1(gd, idx[0], idx[1], idx[2]);
      float e;
      (void)raw2alpha(sigma, P.shift, P.interval, e);
      const float gs = raw2alpha_grad(e, P.interval, ga);
      const int64_t s = kb + i;
      W.b_rec[s] = make_float4(idx[0], idx[1], idx[2], gs);
      W.b_row[s] = row;
      key = cell_key(gd.ldim, ifloor(idx[0]), ifloor(idx[1]), ifloor(idx[2]));
      keys[s] = key;
    }
    // counts per cell and per leaf for the grouping: one atomic per distinct
    // cell (leaf) among the warp's samples; each sample gets a distinct rank
    // within its cell (in no particular order)
    const bool counted = valid && key != kInvalidKey;
    const unsigned same = __match_any_sync(0xffffffffu, counted ? key : kInvalidKey);
    const int lead = __ffs(same) - 1;
    uint32_t base = 0;
    if (counted && lane == lead) base = atomicAdd(cnt + key, uint32_t(__popc(same)));
    base = __shfl_sync(0xffffffffu, base, lead);
    if (counted) rank[kb + i] = base + uint32_t(__popc(same & lt));
    const uint32_t lkey = counted ? (key >> 9) : 0xFFFFFFFFu;
    const unsigned same_l = __match_any_sync(0xffffffffu, lkey);
    if (counted && lane == __ffs(same_l) - 1) atomicAdd(leaf_cnt + lkey, uint32_t(__popc(same_l)));
  }
}

// Deterministic reduction of the sample gradients into voxel gradients.
//
// Each kept sample s sits in the trilinear cell whose low corner is
// floor(idx); its 8 corners receive w_c * gs (density) and w_c * gk0[row]
// (k0). The cell key is a leaf-major code of the low corner (dense leaf index
// x 512 + NanoVDB offset). The samples are grouped by cell with a counting
// placement:
//   k_march_bwd    per sample: its rank among the samples of its cell (an
//                  atomic counter per distinct cell of a warp, so in no
//                  particular order) and the counts per cell and per leaf;
//   leaf scan      exclusive scan of the per-leaf counts (one block);
//   k_cell_offsets per leaf with samples: exclusive scan of its 512 cell
//                  counts, offset by the leaf's start; flags the leaves
//                  holding corners of its cells with samples as touched;
//   k_cell_place   per sample: position = cell offset + rank;
//   k_cell_heads   per cell: sorts its segment by sample index (so the
//                  placement equals a stable sort by key: each cell's samples
//                  contiguous, in ascending sample order);
//   k_group_records per grouped sample (once the rows' k0 gradients exist):
//                  its record and its row's k0 gradient, in grouped order.
// Then one thread per voxel of the touched leaves computes
//   grad += sum over c' = 0..7, in that order, of
//           (sum over the samples of cell v - delta(c'), in sample order,
//            of that sample's corner-c' contribution).
// Every sum has an order fixed by the data, so the result is bitwise
// reproducible without atomics on floats. Corners in no allocated leaf are
// dropped (densityvdb.cu:23).

// Warp per dense leaf with samples: lane t scans cells 16t .. 16t+15 (four
// 16-byte loads), the warp scans the lane totals. The warp also flags as
// touched the allocated leaves that hold a corner of one of the leaf's cells
// with samples: the leaf itself and, for cells on its +x / +y / +z faces,
// the neighbour leaves those corners fall in — in the density grid gd and
// (touched_c != NULL) the k0 grid gc (k0_same: gc has gd's leaves).
__global__ void __launch_bounds__(256)
    k_cell_offsets(const uint32_t* __restrict__ cnt, const uint32_t* __restrict__ leaf_cnt,
                   const uint32_t* __restrict__ leaf_off, int64_t nleaves, uint32_t* off,
                   GridView gd, GridView gc, uint8_t* touched_d, uint8_t* touched_c,
                   int k0_same) {
  grid_dep_sync();
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * int64_t(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nw = (int64_t(gridDim.x) * blockDim.x) >> 5;
  for (int64_t l = w0; l < nleaves; l += nw) {
    if (__ldg(leaf_cnt + l) == 0) continue;  // uniform over the warp
    const uint4* src = reinterpret_cast<const uint4*>(cnt + l * kLeafVox) + lane * 4;
    uint32_t v[16];
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const uint4 q = src[b];
      v[4 * b] = q.x; v[4 * b + 1] = q.y; v[4 * b + 2] = q.z; v[4 * b + 3] = q.w;
    }
    uint32_t sum = 0;
#pragma unroll
    for (int q = 0; q < 16; ++q) sum += v[q];
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    uint32_t run = __ldg(leaf_off + l) + x - sum;
    uint4* dst = reinterpret_cast<uint4*>(off + l * kLeafVox) + lane * 4;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      uint32_t o4[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        o4[e] = run;
        run += v[4 * b + e];
      }
      dst[b] = make_uint4(o4[0], o4[1], o4[2], o4[3]);
    }
    // bit (di, dj, dk) = 4 di + 2 dj + dk: some cell with samples has a
    // corner in the leaf at that offset (cells of lane t: x = t / 4,
    // y = 2 (t % 4) + q / 8, z = q % 8)
    uint32_t dm = 0;
    const bool fx = (lane >> 2) == 7;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      if (!v[q]) continue;
      const bool fy = ((lane & 3) == 3) && q >= 8, fz = (q & 7) == 7;
      dm |= 1u | (fz ? 2u : 0u) | (fy ? 4u : 0u) | (fy && fz ? 8u : 0u);
      if (fx) dm |= 16u | (fz ? 32u : 0u) | (fy ? 64u : 0u) | (fy && fz ? 128u : 0u);
    }
    dm = __reduce_or_sync(0xffffffffu, dm);
    if (lane < 8 && ((dm >> lane) & 1u)) {
      const int lk = int(l % gd.ldim[2]), lj = int((l / gd.ldim[2]) % gd.ldim[1]),
                li = int(l / (int64_t(gd.ldim[2]) * gd.ldim[1]));
      const int ni = li + (lane >> 2), nj = lj + ((lane >> 1) & 1), nk = lk + (lane & 1);
      const int al = leaf_of(gd, ni << 3, nj << 3, nk << 3);
      if (al >= 0) {
        touched_d[al] = 1;
        if (touched_c && k0_same) touched_c[al] = 1;
      }
      if (touched_c && !k0_same) {
        const int alc = leaf_of(gc, ni << 3, nj << 3, nk << 3);
        if (alc >= 0) touched_c[alc] = 1;
      }
    }
  }
}

__global__ void k_cell_place(const uint32_t* __restrict__ keys, const uint32_t* n_dev,
                             const uint32_t* __restrict__ off, const uint32_t* __restrict__ rank,
                             uint32_t* skeys, uint32_t* svals) {
  grid_dep_sync();
  const int64_t n = *n_dev;
  for (int64_t s = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; s < n;
       s += int64_t(gridDim.x) * blockDim.x) {
    const uint32_t key = keys[s];
    if (key == kInvalidKey) continue;
    const uint32_t pos = off[key] + rank[s];
    skeys[pos] = key;
    svals[pos] = uint32_t(s);
  }
}

// Ascending sort of a[0..len): insertion sort for short segments, heapsort
// (O(len log len), in place) for long ones.
__device__ void sort_segment(uint32_t* a, uint32_t len) {
  if (len <= 24) {
    for (uint32_t i = 1; i < len; ++i) {
      const uint32_t v = a[i];
      uint32_t j = i;
      while (j > 0 && a[j - 1] > v) {
        a[j] = a[j - 1];
        --j;
      }
      a[j] = v;
    }
    return;
  }
  auto sift = [&](uint32_t root, uint32_t end) {
    for (;;) {
      uint32_t child = 2 * root + 1;
      if (child >= end) return;
      if (child + 1 < end && a[child + 1] > a[child]) ++child;
      if (a[root] >= a[child]) return;
      const uint32_t t = a[root];
      a[root] = a[child];
      a[child] = t;
      root = child;
    }
  };
  for (uint32_t r = len / 2; r-- > 0;) sift(r, len);
  for (uint32_t end = len - 1; end > 0; --end) {
    const uint32_t t = a[0];
    a[0] = a[end];
    a[end] = t;
    sift(0, end);
  }
}

// Ascending sort of up to 8 indices in registers (odd-even transposition
// network; entries past len are padded with the largest value and stay last).
__device__ __forceinline__ void sort8(uint32_t v[8]) {
#pragma unroll
  for (int round = 0; round < 8; ++round) {
#pragma unroll
    for (int i = round & 1; i + 1 < 8; i += 2) {
      const uint32_t a = v[i], b = v[i + 1];
      v[i] = min(a, b);
      v[i + 1] = max(a, b);
    }
  }
}

// Thread per placed index; cell heads sort their segment (by sample index)
// and lay the segment's gradient records out in that order when rec_s is
// given (the density-only backward: the per-voxel sums then read each
// cell's records contiguously; with k0 rows, k_group_records does this once
// the rows' gradients exist).
__global__ void k_cell_heads(const uint32_t* __restrict__ skeys, const uint32_t* n_dev,
                             const uint32_t* __restrict__ cnt, uint32_t* svals,
                             const float4* __restrict__ rec, float4* rec_s) {
  grid_dep_sync();
  const int64_t n = *n_dev;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const uint32_t key = skeys[i];
    if (i > 0 && skeys[i - 1] == key) continue;
    const uint32_t len = cnt[key];
    if (len == 1) {
      if (rec_s) rec_s[i] = rec[svals[i]];
    } else if (len <= 8) {
      uint32_t v[8];
#pragma unroll
      for (uint32_t t = 0; t < 8; ++t) v[t] = t < len ? svals[i + t] : 0xFFFFFFFFu;
      sort8(v);
#pragma unroll
      for (uint32_t t = 0; t < 8; ++t)
        if (t < len) {
          svals[i + t] = v[t];
          if (rec_s) rec_s[i + t] = rec[v[t]];
        }
    } else {
      sort_segment(svals + i, len);
      if (rec_s)
        for (uint32_t t = 0; t < len; ++t) rec_s[i + t] = rec[svals[i + t]];
    }
  }
}

// Resets the counts of the cells and leaves that got samples.
__global__ void k_cell_clear(const uint32_t* __restrict__ keys, const uint32_t* n_dev,
                             uint32_t* cnt, uint32_t* leaf_cnt) {
  grid_dep_sync();
  const int64_t n = *n_dev;
  for (int64_t s = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; s < n;
       s += int64_t(gridDim.x) * blockDim.x) {
    const uint32_t key = keys[s];
    if (key == kInvalidKey) continue;
    cnt[key] = 0u;
    leaf_cnt[key >> 9] = 0u;
  }
}

// Corner weight c of the multi-channel formula, ((a*b)*c) (colorvdb.cu:100-107).
__device__ __forceinline__ float corner_scale(float u, float v, float w, int c) {
  int di, dj, dk;
  corner_delta(c, di, dj, dk);
  const float a = di ? u : 1.f - u, b = dj ? v : 1.f - v, cc = dk ? w : 1.f - w;
  return __fmul_rn(__fmul_rn(a, b), cc);
}

// A kept sample's k0-gradient row (NQ float4), zero when it has none.
template <int NQ>
__device__ __forceinline__ void gather_row(const float* __restrict__ gk0, int32_t row, int C,
                                           int vec, float4* q) {
#pragma unroll
  for (int b = 0; b < NQ; ++b) {
    if (row < 0) {
      q[b] = make_float4(0.f, 0.f, 0.f, 0.f);
      continue;
    }
    const float* gr = gk0 + int64_t(row) * C;
    if (vec) {
      q[b] = __ldg(reinterpret_cast<const float4*>(gr) + b);
    } else {
      q[b].x = __ldg(gr + 4 * b);
      q[b].y = 4 * b + 1 < C ? __ldg(gr + 4 * b + 1) : 0.f;
      q[b].z = 4 * b + 2 < C ? __ldg(gr + 4 * b + 2) : 0.f;
      q[b].w = 4 * b + 3 < C ? __ldg(gr + 4 * b + 3) : 0.f;
    }
  }
}

// Thread per grouped index j: the grouped record of sample svals[j] — its
// gradient record (index-space position, dL/dsigma) followed by its colour
// row's k0 gradient (NQ float4; zeros when the sample has no colour row) —
// as 1 + NQ consecutive float4. The per-voxel sums then read a cell's
// samples as one contiguous run, without the dependent row lookup (the rows
// are in ray order, the cells in key order). Runs once the rgbnet backward
// has written the rows' gradients.
template <int NQ>
__global__ void __launch_bounds__(256)
    k_group_records(const uint32_t* __restrict__ svals, const uint32_t* n_dev,
                    const float4* __restrict__ rec, const int32_t* __restrict__ brow,
                    const float* __restrict__ gk0, int C, int vec, float4* rec_g) {
  grid_dep_sync();
  constexpr int NB = NQ > 0 ? NQ : 1;
  const int64_t n = *n_dev;
  for (int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; j < n;
       j += int64_t(gridDim.x) * blockDim.x) {
    const uint32_t sv = __ldg(svals + j);
    const float4 p = __ldg(rec + sv);
    float4 q[NB];
    if (NQ) gather_row<NQ>(gk0, __ldg(brow + sv), C, vec, q);
    float4* dst = rec_g + j * (1 + NQ);
    dst[0] = p;
#pragma unroll
    for (int b = 0; b < NQ; ++b) dst[1 + b] = q[b];
  }
}

// Adds one sample's contribution to corner c of its cell: the density term
// (when the grid takes one and the sample's dL/dsigma is nonzero) and the
// k0 row scaled by the corner weight (want_c; a sample without a colour row
// carries a zero row, whose products leave the sums' bits unchanged: they
// start at +0 and adding a signed zero to a value other than -0 returns it).
template <int NQ>
__device__ __forceinline__ void gather_add(const float4 p, const float4* q, bool want_c,
                                           bool want_d, int c, float& pd, float4* pk) {
  const float u = p.x - float(ifloor(p.x)), v = p.y - float(ifloor(p.y)),
              w = p.z - float(ifloor(p.z));
  if (want_d && p.w != 0.f) pd = __fadd_rn(pd, density_corner_term(p.w, u, v, w, c));
  if (want_c) {
    const float sce = corner_scale(u, v, w, c);
#pragma unroll
    for (int b = 0; b < NQ; ++b) {
      pk[b].x = __fadd_rn(pk[b].x, __fmul_rn(q[b].x, sce));
      pk[b].y = __fadd_rn(pk[b].y, __fmul_rn(q[b].y, sce));
      pk[b].z = __fadd_rn(pk[b].z, __fmul_rn(q[b].z, sce));
      pk[b].w = __fadd_rn(pk[b].w, __fmul_rn(q[b].w, sce));
    }
  }
}

// Thread per voxel of the listed (touched) leaves of grid g; adds the density
// sum to grad_d and/or the k0 sums to grad_c (C channels). NQ = the number of
// float4 chunks of the k0 gradient in a grouped record (0 = density only).
template <int NQ>
__global__ void __launch_bounds__(256, 4)
    k_voxel_gather(GridView g, const int32_t* __restrict__ list, const uint32_t* __restrict__ count,
                   const uint32_t* __restrict__ cnt, const uint32_t* __restrict__ off,
                   const float4* __restrict__ rec_g, float* grad_d, float* grad_c, int C) {
  grid_dep_sync();
  constexpr int NB = NQ > 0 ? NQ : 1;
  const int64_t nv = int64_t(*count) * kLeafVox;
  const bool want_d = grad_d != nullptr, want_c = NQ && grad_c;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < nv;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int leaf = list[i >> 9];
    const int vox = int(i & 511);
    const int vi = g.origin[leaf * 3] + (vox >> 6), vj = g.origin[leaf * 3 + 1] + ((vox >> 3) & 7),
              vk = g.origin[leaf * 3 + 2] + (vox & 7);
    // the up to 8 cells that have this voxel as corner c, in corner order:
    // the counts are loaded together (a cell outside the lattice reads entry
    // 0 and counts as empty), so the loads of idle voxels overlap
    uint32_t len[8], key[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      int di, dj, dk;
      corner_delta(c, di, dj, dk);
      const uint32_t k = cell_key(g.ldim, vi - di, vj - dj, vk - dk);
      key[c] = k == kInvalidKey ? 0u : k;
      len[c] = __ldg(cnt + key[c]);
      if (k == kInvalidKey) len[c] = 0;
    }
    uint32_t any = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) any |= len[c];
    if (!any) continue;
    float sum_d = 0.f;
    float4 acc[NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) acc[b] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      if (!len[c]) continue;
      float pd = 0.f;
      float4 pk[NB];
#pragma unroll
      for (int b = 0; b < NB; ++b) pk[b] = make_float4(0.f, 0.f, 0.f, 0.f);
      const uint32_t h = __ldg(off + key[c]);
      for (uint32_t j = h; j < h + len[c]; ++j) {
        const float4* r = rec_g + int64_t(j) * (1 + NQ);
        const float4 p0 = __ldg(r);
        float4 q0[NB];
        if (want_c) {
#pragma unroll
          for (int b = 0; b < NQ; ++b) q0[b] = __ldg(r + 1 + b);
        }
        gather_add<NQ>(p0, q0, want_c, want_d, c, pd, pk);
      }
      sum_d = __fadd_rn(sum_d, pd);
#pragma unroll
      for (int b = 0; b < NQ; ++b) {
        acc[b].x = __fadd_rn(acc[b].x, pk[b].x);
        acc[b].y = __fadd_rn(acc[b].y, pk[b].y);
        acc[b].z = __fadd_rn(acc[b].z, pk[b].z);
        acc[b].w = __fadd_rn(acc[b].w, pk[b].w);
      }
    }
    const int64_t slot = int64_t(leaf) * kLeafVox + vox;
    if (want_d) grad_d[slot] = __fadd_rn(grad_d[slot], sum_d);
    if (want_c) {
      float* dst = grad_c + slot * C;
#pragma unroll
      for (int b = 0; b < NQ; ++b) {
        const float a4[4] = {acc[b].x, acc[b].y, acc[b].z, acc[b].w};
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (4 * b + q < C) dst[4 * b + q] = __fadd_rn(dst[4 * b + q], a4[q]);
      }
    }
  }
}

template <int NQ>
static int cell_reduce_launch(pvdb_march_s* m, pvdb_grid_s* density, pvdb_grid_s* k0,
                              const float* grad_k0, cudaStream_t st) {
  const int grid = stride_grid();
  const GridView gv = density->view();
  const GridView kv = NQ ? k0->view() : gv;
  int rc = touched_list(density, st);
  if (rc) return rc;
  const bool same = NQ && k0->h_table == density->h_table;
  const int C = NQ ? k0->C : 0;
  const int vec = NQ && C % 4 == 0 && (reinterpret_cast<uintptr_t>(grad_k0) & 15u) == 0;
  if (m->bwd_with_k0) {
    // the grouped records with their rows' k0 gradients (k_cell_heads wrote
    // the density-only records already when the keys ran without k0)
    PVDB_REQUIRE(m->b_rec_s_cap >= size_t(m->slots) * 16 * (1 + NQ),
                 "march backward: grouped-record buffer too small");
    const int sgrid = int(std::min<int64_t>(ceil_div(m->slots, 256), int64_t(grid)));
    launch_k(k_group_records<NQ>, sgrid, 256, 0, st, m->red.vals[0], m->w.totals + 5, m->w.b_rec,
             m->w.b_row, grad_k0, C, vec, m->b_rec_s);
    PVDB_CHECK_LAUNCH("k_group_records");
  }
  const float4* rec_g = m->b_rec_s;
  launch_k(k_voxel_gather<NQ>, grid, 256, 0, st, gv, density->d_tlist, density->d_tcount,
           m->cell_cnt, m->cell_off, rec_g, density->d_grad, same ? k0->d_grad : nullptr, C);
  PVDB_CHECK_LAUNCH("k_voxel_gather");
  if (NQ && !same) {
    if ((rc = touched_list(k0, st))) return rc;
    launch_k(k_voxel_gather<NQ>, grid, 256, 0, st, kv, k0->d_tlist, k0->d_tcount, m->cell_cnt,
             m->cell_off, rec_g, nullptr, k0->d_grad, C);
    PVDB_CHECK_LAUNCH("k_voxel_gather(k0)");
  }
  return PVDB_OK;
}

// --------------------------------------------------------------- composite
__global__ void __launch_bounds__(kMarchThreads)
    k_composite_fwd(MarchW W, const float* __restrict__ rgb, float bg, float* out, int R) {
  grid_dep_sync();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * kMarchWarps + warp;
  if (r >= R) return;
  const int n = rgb ? int(W.n_color[r]) : 0;  // NULL rgb: no colour rows
  const int64_t off = W.color_off[r];
  float s0 = 0.f, s1 = 0.f, s2 = 0.f;
  for (int j = lane; j < n; j += 32) {
    const int64_t m = off + j;
    const float w = W.r_w[m];
    s0 = __fadd_rn(s0, __fmul_rn(w, rgb[m * 3]));
    s1 = __fadd_rn(s1, __fmul_rn(w, rgb[m * 3 + 1]));
    s2 = __fadd_rn(s2, __fmul_rn(w, rgb[m * 3 + 2]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s0 = __fadd_rn(s0, __shfl_xor_sync(0xffffffffu, s0, o));
    s1 = __fadd_rn(s1, __shfl_xor_sync(0xffffffffu, s1, o));
    s2 = __fadd_rn(s2, __shfl_xor_sync(0xffffffffu, s2, o));
  }
  if (lane == 0) {
    const float tb = __fmul_rn(W.T_last[r], bg);
    out[r * 3] = __fadd_rn(s0, tb);
    out[r * 3 + 1] = __fadd_rn(s1, tb);
    out[r * 3 + 2] = __fadd_rn(s2, tb);
  }
}

__global__ void __launch_bounds__(kMarchThreads)
    k_composite_bwd(MarchW W, const float* __restrict__ rgb, const float* __restrict__ g, float bg,
                    float* grad_rgb, float* grad_w, float* grad_last, int R) {
  grid_dep_sync();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * kMarchWarps + warp;
  if (r >= R) return;
  const float g0 = g[r * 3], g1 = g[r * 3 + 1], g2 = g[r * 3 + 2];
  if (lane == 0 && grad_last)
    grad_last[r] = __fadd_rn(grad_last[r], __fadd_rn(__fadd_rn(__fmul_rn(g0, bg), __fmul_rn(g1, bg)),
                                                      __fmul_rn(g2, bg)));
  const int n = int(W.n_color[r]);
  const int64_t off = W.color_off[r];
  for (int j = lane; j < n; j += 32) {
    const int64_t m = off + j;
    const float w = W.r_w[m];
    if (grad_rgb) {
      grad_rgb[m * 3] = __fmul_rn(w, g0);
      grad_rgb[m * 3 + 1] = __fmul_rn(w, g1);
      grad_rgb[m * 3 + 2] = __fmul_rn(w, g2);
    }
    if (grad_w)
      grad_w[m] = __fadd_rn(__fadd_rn(__fmul_rn(g0, rgb[m * 3]), __fmul_rn(g1, rgb[m * 3 + 1])),
                            __fmul_rn(g2, rgb[m * 3 + 2]));
  }
}

// ------------------------------------------------------------------ host
static void fill_params(const pvdb_march_params* in, const pvdb_grid_s* gd, const uint8_t* mask,
                        const int32_t* mshape, int cap, MarchP& P) {
  for (int a = 0; a < 3; ++a) {
    P.mn[a] = in->xyz_min[a];
    P.mx[a] = in->xyz_max[a];
    P.ext[a] = in->xyz_max[a] - in->xyz_min[a];
    P.wsm1[a] = float(gd->reso[a] - 1);
  }
  P.near_ = in->near_;
  P.far_ = in->far_;
  P.stepdist = in->stepdist;
  P.shift = in->act_shift;
  P.interval = in->interval;
  P.thr = in->fast_color_thres;
  P.t_stop = in->t_stop;
  P.bg = in->bg;
  P.mask = mask;
  for (int a = 0; a < 3; ++a) {
    P.mshape[a] = mask ? mshape[a] : 0;
    // MaskGrid (grid.py:230-232): scale = (shape-1)/(max-min); shift = -min*scale
    P.mscale[a] = mask ? float(mshape[a] - 1) / P.ext[a] : 0.f;
    P.mshift[a] = mask ? (-P.mn[a]) * P.mscale[a] : 0.f;
  }
  P.cap = cap;
  // alpha > thr  <=>  sigma > log((1 - thr)^(-1/interval) - 1) - shift; the
  // margin covers the float evaluation of the trilinear and of raw2alpha
  P.sigma_skip = -INFINITY;
  if (in->fast_color_thres > 0.f && in->fast_color_thres < 1.f && in->interval > 0.f) {
    const double t = std::log(std::pow(1.0 - double(in->fast_color_thres),
                                       -1.0 / double(in->interval)) - 1.0) -
                     double(in->act_shift);
    P.sigma_skip = float(t - 1e-3 * (std::fabs(t) + 1.0));
  }
  for (int a = 0; a < 3; ++a) P.binv[a] = P.wsm1[a] / P.ext[a] * 0.25f;
}

int march_forward_impl(pvdb_march_s* m, pvdb_grid_s* density, pvdb_grid_s* k0, const float* ro,
                       const float* rd, int R, const pvdb_march_params* prm, const uint8_t* mask,
                       const int32_t* mshape, cudaStream_t st, bool skip_k0) {
  if (k0) {
    for (int a = 0; a < 3; ++a) {
      PVDB_REQUIRE(k0->reso[a] == density->reso[a], "k0 and density grids need the same resolution");
      PVDB_REQUIRE(k0->ldim[a] == density->ldim[a], "k0 and density grids need the same leaf lattice");
    }
    if (m->k0_channels < k0->C) {
      dev_free(m->w.r_k0);
      m->w.r_k0 = nullptr;
      int rc = dev_alloc((void**)&m->w.r_k0, size_t(m->slots) * k0->C * 4);
      if (rc) return rc;
      m->k0_channels = k0->C;
    }
  }
  if (density->C == 1) {
    int rc = bmax_ensure(density, st);
    if (rc) return rc;
  }
  fill_params(prm, density, mask, mshape, m->cap, m->p);
  m->n_rays = R;
  m->density = density;
  m->k0 = k0;
  PVDB_CHECK_CUDA(cudaMemsetAsync(m->w.totals, 0, 32, st));
  if (R > 0) {
    const int nb = ceil_div(R, kMarchWarps);
    launch_k(k_march_setup, ceil_div(R, 256), 256, 0, st, ro, rd, R, m->p, m->w);
    PVDB_CHECK_LAUNCH("k_march_setup");
    if (m->leaf_staging) {
      PVDB_SMEM_ATTR(k_march_alpha_staged, int(kStageSmem));
      launch_k(k_march_alpha_staged, R, 256, kStageSmem, st, density->view(), m->p, m->w,
               debug_spin_limit(kStageSpinMax), debug_hold_staging());
      PVDB_CHECK_LAUNCH("k_march_alpha_staged");
    } else {
      launch_k(k_march_alpha, R, 256, 0, st, density->view(), m->p, m->w);
      PVDB_CHECK_LAUNCH("k_march_alpha");
    }
    launch_k(k_march_chain, nb, kMarchThreads, 0, st, R, m->p, m->w,
             debug_spin_limit(kChainSpinMax), debug_hold_first());
    PVDB_CHECK_LAUNCH("k_march_chain");
    if (m->prof) prof_mark(st, 1);
    GridView gk{};
    if (k0) gk = k0->view();
    if (k0 && !skip_k0) {
      launch_k(k_march_k0, int(std::min<int64_t>(ceil_div(m->slots, 256), int64_t(num_sms()) * 16)),
               256, 0, st, gk, m->p, m->w);
      PVDB_CHECK_LAUNCH("k_march_k0");
    }
    if (m->prof) prof_mark(st, 2);
  }
  m->has_fwd = true;
  return PVDB_OK;
}

// Test hook: forces the k0 gather's blocks-per-SM variant (0: automatic).
static std::atomic<int> g_dbg_k0_blocks{0};

// Backward, first part: the density-path gradients of every kept sample
// (k_march_bwd) and the grouping of the kept samples by cell, which need only
// the gradients w.r.t. the weights and alphainv_last — so it can run while
// the rgbnet backward produces the k0-row gradients. with_k0: the k0 grid gets
// gradients (its touched leaves are flagged too).
// The fused k0 + X-tile pass (after a forward run with skip_k0); xt must hold
// ceil(slots / 128) tiles; half: the k0 grid's BF16 shadow to gather from
// (NULL: the FP32 values).
int march_k0_x(pvdb_march_s* m, const float* pe, int pe_stride, int dpe, uint8_t* xt,
               cudaStream_t st, const __nv_bfloat16* half) {
  if (m->n_rays == 0 || !m->k0) return PVDB_OK;
  PVDB_REQUIRE(!half || m->k0->C == 12, "the BF16 feature shadow is kept for 12 channels");
  PVDB_REQUIRE(m->k0->C <= 16 && m->k0->C + dpe + 1 <= kRgbXK,
               "the tensor-core rgbnet takes at most 16 k0 and 47 input channels");
  const int grid = int(std::min<int64_t>(ceil_div(m->slots, 256), int64_t(num_sms()) * 16));
  // The row count is on the device; the batch's ray count stands in for it:
  // 2 blocks per SM for batches up to 32768 rays (a few waves of rows), 3
  // beyond (65536 rays at 320^3: 384 against 402 us; 8192 rays at 160^3: 21.8
  // against 20.0 us).
  const int forced = g_dbg_k0_blocks.load();
  const bool many = forced ? forced == 3 : m->n_rays > 32768;
  if (m->k0->C == 12 && many)
    launch_k(k_march_k0_x<12, 3>, grid, 256, 0, st, m->k0->view(), m->p, m->w, pe, pe_stride, dpe,
             xt, half);
  else if (m->k0->C == 12)
    launch_k(k_march_k0_x<12, 2>, grid, 256, 0, st, m->k0->view(), m->p, m->w, pe, pe_stride, dpe,
             xt, half);
  else
    launch_k(k_march_k0_x<0, 2>, grid, 256, 0, st, m->k0->view(), m->p, m->w, pe, pe_stride, dpe,
             xt, nullptr);
  PVDB_CHECK_LAUNCH("k_march_k0_x");
  if (m->prof) prof_mark(st, 2);
  return PVDB_OK;
}

int march_backward_keys(pvdb_march_s* m, const float* grad_w, const float* grad_last,
                        bool with_k0, cudaStream_t st) {
  pvdb_grid_s* density = m->density;
  pvdb_grid_s* k0 = with_k0 ? m->k0 : nullptr;
  const int R = m->n_rays;
  if (R == 0) return PVDB_OK;
  const int64_t nmax = m->slots;
  int rc = scratch_reserve(m->red, nmax);
  if (rc) return rc;
  const int64_t ncells = int64_t(density->ldim[0]) * density->ldim[1] * density->ldim[2] * kLeafVox;
  const int64_t nleaves = ncells / kLeafVox;
  if (m->cell_cap < size_t(ncells)) {
    for (uint32_t** p : {&m->cell_cnt, &m->cell_off, &m->leaf_cnt, &m->leaf_off}) {
      dev_free(*p);
      *p = nullptr;
    }
    m->cell_cap = 0;
    if ((rc = dev_alloc((void**)&m->cell_cnt, size_t(ncells) * 4)) ||
        (rc = dev_alloc((void**)&m->cell_off, size_t(ncells) * 4)) ||
        (rc = dev_alloc((void**)&m->leaf_cnt, size_t(nleaves) * 4)) ||
        (rc = dev_alloc((void**)&m->leaf_off, size_t(nleaves) * 4)))
      return rc;
    PVDB_CHECK_CUDA(cudaMemsetAsync(m->cell_cnt, 0, size_t(ncells) * 4, st));
    PVDB_CHECK_CUDA(cudaMemsetAsync(m->leaf_cnt, 0, size_t(nleaves) * 4, st));
    m->cell_cap = size_t(ncells);
  }
  if ((rc = dev_reserve((void**)&m->w.b_rec, &m->b_rec_cap, size_t(nmax) * 16)) ||
      (rc = dev_reserve((void**)&m->w.b_row, &m->b_row_cap, size_t(nmax) * 4)) ||
      (rc = dev_reserve((void**)&m->b_rec_s, &m->b_rec_s_cap,
                        size_t(nmax) * 16 * (1 + (k0 ? (k0->C + 3) / 4 : 0)))))
    return rc;
  const int nb = ceil_div(R, kMarchWarps);
  // the kept samples' keys, with their per-cell ranks and the per-cell and
  // per-leaf counts of the grouping below
  const uint32_t* keys = m->red.keys[0];
  uint32_t* rank = m->red.vals[1];
  uint32_t* skeys = m->red.keys[1];
  uint32_t* svals = m->red.vals[0];
  launch_k(k_march_bwd, nb, kMarchThreads, 0, st, density->view(), R, m->p, m->w, grad_w, grad_last,
           m->red.keys[0], m->cell_cnt, m->leaf_cnt, rank);
  PVDB_CHECK_LAUNCH("k_march_bwd");
  if (m->prof) prof_mark(st, 6);
  // group the kept samples by cell (stable order, see above)
  const int sgrid = int(std::min<int64_t>(ceil_div(nmax, 256), int64_t(stride_grid())));
  rc = scan_exclusive_u32(m->leaf_cnt, m->leaf_off, nleaves, m->w.totals + 5, &m->scan_partial,
                          &m->scan_partial_cap, st);
  if (rc) return rc;
  const GridView gv = density->view();
  const GridView kv = k0 ? k0->view() : gv;
  launch_k(k_cell_offsets, int(std::min<int64_t>(ceil_div(nleaves, 8), int64_t(stride_grid()))),
           256, 0, st, m->cell_cnt, m->leaf_cnt, m->leaf_off, nleaves, m->cell_off, gv, kv,
           density->d_touched, k0 ? k0->d_touched : nullptr,
           k0 && k0->h_table == density->h_table ? 1 : 0);
  PVDB_CHECK_LAUNCH("k_cell_offsets");
  launch_k(k_cell_place, sgrid, 256, 0, st, keys, m->w.totals + 0, m->cell_off, rank, skeys, svals);
  PVDB_CHECK_LAUNCH("k_cell_place");
  launch_k(k_cell_heads, stride_grid(), 256, 0, st, skeys, m->w.totals + 5, m->cell_cnt, svals,
           m->w.b_rec, k0 ? nullptr : m->b_rec_s);
  PVDB_CHECK_LAUNCH("k_cell_heads");
  density->tlist_valid = false;
  if (k0) k0->tlist_valid = false;
  if (m->prof) prof_mark(st, 7);
  m->bwd_keys_ready = true;
  m->bwd_with_k0 = with_k0;
  return PVDB_OK;
}

// Backward, second part: the per-voxel sums into the density and k0 gradients
// (grad_k0 [M, C]: the k0-row gradients; ignored when the first part ran
// without k0), then the cell counts are reset.
// Resets the counts of the cells and leaves that got samples (needed before
// the next backward's grouping; a caller may run it on another stream once
// the per-voxel sums are done).
int march_backward_clear(pvdb_march_s* m, cudaStream_t st) {
  if (m->n_rays == 0) return PVDB_OK;
  const int sgrid = int(std::min<int64_t>(ceil_div(m->slots, 256), int64_t(stride_grid())));
  launch_k(k_cell_clear, sgrid, 256, 0, st, m->red.keys[0], m->w.totals + 0, m->cell_cnt,
           m->leaf_cnt);
  PVDB_CHECK_LAUNCH("k_cell_clear");
  return PVDB_OK;
}

// clear: also reset the cell counts here (else the caller runs
// march_backward_clear).
int march_backward_reduce(pvdb_march_s* m, const float* grad_k0, cudaStream_t st, bool clear) {
  if (m->n_rays == 0) return PVDB_OK;
  if (!m->bwd_keys_ready) return set_error(PVDB_ERR_STATE, "march backward: keys not grouped");
  m->bwd_keys_ready = false;
  pvdb_grid_s* density = m->density;
  pvdb_grid_s* k0 = m->k0;
  const int C = m->bwd_with_k0 && grad_k0 ? k0->C : 0;
  PVDB_REQUIRE(C <= 16, "the march backward takes at most 16 k0 channels");
  int rc;
  switch ((C + 3) / 4) {
    case 0: rc = cell_reduce_launch<0>(m, density, k0, grad_k0, st); break;
    case 1: rc = cell_reduce_launch<1>(m, density, k0, grad_k0, st); break;
    case 2: rc = cell_reduce_launch<2>(m, density, k0, grad_k0, st); break;
    case 3: rc = cell_reduce_launch<3>(m, density, k0, grad_k0, st); break;
    default: rc = cell_reduce_launch<4>(m, density, k0, grad_k0, st); break;
  }
  if (rc) return rc;
  if (clear && (rc = march_backward_clear(m, st))) return rc;
  if (m->prof) prof_mark(st, 8);
  return PVDB_OK;
}

int march_backward_impl(pvdb_march_s* m, const float* grad_w, const float* grad_last,
                        const float* grad_k0, cudaStream_t st) {
  const bool use_k0 = m->k0 && grad_k0;
  if (use_k0) PVDB_REQUIRE(m->k0->C <= 16, "the march backward takes at most 16 k0 channels");
  int rc = march_backward_keys(m, grad_w, grad_last, use_k0, st);
  if (rc) return rc;
  return march_backward_reduce(m, grad_k0, st, true);
}

int composite_forward_impl(pvdb_march_s* m, const float* rgb, float bg, float* out, int R,
                           cudaStream_t st) {
  if (R <= 0) return PVDB_OK;
  launch_k(k_composite_fwd, ceil_div(R, kMarchWarps), kMarchThreads, 0, st, m->w, rgb, bg, out, R);
  PVDB_CHECK_LAUNCH("k_composite_fwd");
  return PVDB_OK;
}

int composite_backward_impl(pvdb_march_s* m, const float* rgb, const float* g, float bg,
                            float* grad_rgb, float* grad_w, float* grad_last, int R,
                            cudaStream_t st) {
  if (R <= 0) return PVDB_OK;
  launch_k(k_composite_bwd, ceil_div(R, kMarchWarps), kMarchThreads, 0, st, m->w, rgb, g, bg,
           grad_rgb, grad_w, grad_last, R);
  PVDB_CHECK_LAUNCH("k_composite_bwd");
  return PVDB_OK;
}

}  // namespace pvdb

using namespace pvdb;

extern "C" {

int pvdb_debug_k0_blocks(int blocks) {
  clear_error();
  PVDB_REQUIRE(blocks == 0 || blocks == 2 || blocks == 3, "blocks must be 0, 2 or 3");
  g_dbg_k0_blocks.store(blocks);
  return PVDB_OK;
}

int32_t pvdb_march_samples_cap(const float xyz_min[3], const float xyz_max[3], float stepdist) {
  if (!xyz_min || !xyz_max || !(stepdist > 0.f)) return 0;
  double d2 = 0;
  for (int a = 0; a < 3; ++a) {
    const double e = double(xyz_max[a]) - double(xyz_min[a]);
    d2 += e * e;
  }
  // n_steps = ceil(chord*|d|/stepdist) <= ceil(diag/stepdist) (+ rounding slack)
  return int32_t(std::ceil(std::sqrt(d2) / stepdist * (1.0 + 1e-5))) + 2;
}

int pvdb_march_create(int32_t max_rays, int32_t samples_cap, pvdb_march* out) {
  clear_error();
  PVDB_REQUIRE(out, "null argument");
  PVDB_REQUIRE(max_rays > 0 && samples_cap > 0, "max_rays and samples_cap must be positive");
  PVDB_REQUIRE(int64_t(max_rays) * samples_cap * 8 < int64_t(0xFFFFFFF0u),
               "max_rays * samples_cap too large for 32-bit contribution ids");
  pvdb_march_s* m = new pvdb_march_s();
  m->max_rays = max_rays;
  m->cap = samples_cap;
  m->slots = int64_t(max_rays) * samples_cap;
  MarchW& w = m->w;
  const size_t R = max_rays, S = size_t(m->slots);
  int rc;
  if ((rc = dev_alloc((void**)&w.ray_sd, R * 24)) || (rc = dev_alloc((void**)&w.ray_ns, R * 4)) ||
      (rc = dev_alloc((void**)&w.chain_status, R * 8)) ||
      (rc = dev_alloc((void**)&w.T_last, R * 4)) || (rc = dev_alloc((void**)&w.n_kept, R * 4)) ||
      (rc = dev_alloc((void**)&w.n_color, R * 4)) ||
      (rc = dev_alloc((void**)&w.kept_off, R * 4)) ||
      (rc = dev_alloc((void**)&w.color_off, R * 4)) ||
      (rc = dev_alloc((void**)&w.k_alpha, S * 4)) || (rc = dev_alloc((void**)&w.k_w, S * 4)) ||
      (rc = dev_alloc((void**)&w.k_step, S * 4)) || (rc = dev_alloc((void**)&w.k_row, S * 4)) ||
      (rc = dev_alloc((void**)&w.r_w, S * 4)) || (rc = dev_alloc((void**)&w.r_alpha, S * 4)) ||
      (rc = dev_alloc((void**)&w.r_ray, S * 4)) || (rc = dev_alloc((void**)&w.r_step, S * 4)) ||
      (rc = dev_alloc((void**)&w.totals, 64))) {
    pvdb_march_destroy(m);
    return rc;
  }
  // totals, and the row records' ray and step indices: rows that a forward
  // does not write (after a look-back wait gave up) keep in-range values
  cudaError_t e = cudaMemset(w.totals, 0, 64);
  if (e == cudaSuccess) e = cudaMemset(w.r_ray, 0, S * 4);
  if (e == cudaSuccess) e = cudaMemset(w.r_step, 0, S * 4);
  if (e != cudaSuccess) {
    pvdb_march_destroy(m);
    return cuda_error(e, "cudaMemset");
  }
  *out = m;
  return PVDB_OK;
}

int pvdb_march_set_leaf_staging(pvdb_march m, int32_t on) {
  clear_error();
  if (!m) return set_error(PVDB_ERR_ARG, "pvdb_march_set_leaf_staging: null workspace");
  m->leaf_staging = on ? 1 : 0;
  return PVDB_OK;
}

int pvdb_march_destroy(pvdb_march m) {
  if (!m) return PVDB_OK;
  MarchW& w = m->w;
  void* ptrs[] = {w.ray_sd, w.ray_ns, w.chain_status, w.T_last, w.n_kept, w.n_color, w.kept_off, w.color_off, w.k_alpha, w.k_w,
                  w.k_step, w.k_row, w.r_k0, w.r_w, w.r_alpha, w.r_ray, w.r_step, w.b_rec, w.b_row,
                  m->b_rec_s, w.totals, m->scan_partial, m->hpe, m->wpart, m->mlp_packed, m->mlp_xt,
                  m->t_rgb, m->t_grad_rgb, m->t_grad_w, m->t_grad_k0, m->t_grad_last,
                  m->t_loss_part, m->t_rgb_marched};
  for (void* p : ptrs) dev_free(p);
  free_scratch(m->red);
  for (uint32_t* p : {m->cell_cnt, m->cell_off, m->leaf_cnt, m->leaf_off}) dev_free(p);
  dev_free(m->g_in);
  dev_free(m->g_scal);
  if (m->g_exec) cudaGraphExecDestroy(m->g_exec);
  if (m->g_graph) cudaGraphDestroy(m->g_graph);
  if (m->g_stream) cudaStreamDestroy(m->g_stream);
  for (cudaStream_t& x : m->side)
    if (x) cudaStreamDestroy(x);
  for (cudaEvent_t& e : m->side_ev)
    if (e) cudaEventDestroy(e);
  delete m;
  return PVDB_OK;
}

int pvdb_march_forward(pvdb_march m, pvdb_grid density, pvdb_grid k0, const float* rays_o,
                       const float* rays_d, int32_t n_rays, const pvdb_march_params* p,
                       const uint8_t* mask, const int32_t mask_shape[3], pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(m && density && p, "null argument");
  PVDB_REQUIRE(density->C == 1, "density grid must have 1 channel");
  PVDB_REQUIRE(n_rays >= 0 && n_rays <= m->max_rays, "n_rays exceeds the workspace");
  PVDB_REQUIRE(n_rays == 0 || (rays_o && rays_d), "null rays");
  PVDB_REQUIRE(!mask || mask_shape, "mask needs mask_shape");
  PVDB_REQUIRE(p->stepdist > 0.f, "stepdist must be positive");
  return march_forward_impl(m, density, k0, rays_o, rays_d, n_rays, p, mask, mask_shape,
                            as_stream(s), false);
}

int pvdb_march_views(pvdb_march m, pvdb_march_views_t* v) {
  clear_error();
  PVDB_REQUIRE(m && v, "null argument");
  v->alphainv_last = m->w.T_last;
  v->n_kept = (int32_t*)m->w.n_kept;
  v->n_color = (int32_t*)m->w.n_color;
  v->color_offset = (int32_t*)m->w.color_off;
  v->k0 = m->w.r_k0;
  v->weight = m->w.r_w;
  v->alpha = m->w.r_alpha;
  v->ray_id = m->w.r_ray;
  v->step_id = m->w.r_step;
  v->totals = (int32_t*)m->w.totals;
  v->rows_capacity = m->slots;
  return PVDB_OK;
}

int pvdb_march_totals(pvdb_march m, int64_t* total_kept, int64_t* total_rows, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(m, "null argument");
  uint32_t t[4];
  cudaStream_t st = as_stream(s);
  PVDB_CHECK_CUDA(cudaMemcpyAsync(t, m->w.totals, 16, cudaMemcpyDeviceToHost, st));
  PVDB_CHECK_CUDA(cudaStreamSynchronize(st));
  if (total_kept) *total_kept = t[0];
  if (total_rows) *total_rows = t[1];
  if (t[3] & 1u) return set_error(PVDB_ERR_STATE, "a ray had more samples than samples_cap");
  if (t[3] & 2u) return set_error(PVDB_ERR_TIMEOUT, "a tensor-core MMA wait timed out");
  if (t[3] & 4u) return set_error(PVDB_ERR_TIMEOUT, "a ray-offset look-back wait of the march timed out");
  if (t[3] & 8u)
    return set_error(PVDB_ERR_TIMEOUT, "a leaf-staging copy wait of the march timed out "
                                       "(those samples read global memory)");
  return PVDB_OK;
}

int pvdb_march_stats(pvdb_march m, int64_t* kept, int64_t* rows, int64_t* evaluated,
                     pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(m, "null argument");
  uint32_t t[8];
  cudaStream_t st = as_stream(s);
  PVDB_CHECK_CUDA(cudaMemcpyAsync(t, m->w.totals, 32, cudaMemcpyDeviceToHost, st));
  PVDB_CHECK_CUDA(cudaStreamSynchronize(st));
  if (kept) *kept = t[0];
  if (rows) *rows = t[1];
  if (evaluated) *evaluated = t[4];
  return PVDB_OK;
}

int pvdb_march_adam_counts(pvdb_march m, int64_t* out, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(m && out, "null argument");
  uint32_t t[4];
  cudaStream_t st = as_stream(s);
  PVDB_CHECK_CUDA(cudaMemcpyAsync(t, m->w.totals + 8, 16, cudaMemcpyDeviceToHost, st));
  PVDB_CHECK_CUDA(cudaStreamSynchronize(st));
  for (int i = 0; i < 4; ++i) out[i] = t[i];
  return PVDB_OK;
}

int pvdb_march_backward(pvdb_march m, pvdb_grid density, pvdb_grid k0, const float* grad_weight,
                        const float* grad_last, const float* grad_k0, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(m && density, "null argument");
  PVDB_REQUIRE(m->has_fwd, "backward before forward");
  PVDB_REQUIRE(density == m->density && k0 == m->k0, "grids differ from the forward's");
  PVDB_REQUIRE(!grad_k0 || k0, "grad_k0 given without a k0 grid");
  return march_backward_impl(m, grad_weight, grad_last, grad_k0, as_stream(s));
}

int pvdb_composite_forward(pvdb_march m, const float* rgb, float bg, float* rgb_marched,
                           int32_t n_rays, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(m && rgb_marched, "null argument");
  PVDB_REQUIRE(m->has_fwd && n_rays == m->n_rays, "n_rays differs from the forward's");
  return composite_forward_impl(m, rgb, bg, rgb_marched, n_rays, as_stream(s));
}

int pvdb_composite_backward(pvdb_march m, const float* rgb, const float* grad_rgb_marched,
                            float bg, float* grad_rgb, float* grad_weight, float* grad_last,
                            int32_t n_rays, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(m && grad_rgb_marched, "null argument");
  PVDB_REQUIRE(m->has_fwd && n_rays == m->n_rays, "n_rays differs from the forward's");
  PVDB_REQUIRE(!grad_weight || rgb, "grad_weight needs rgb");
  return composite_backward_impl(m, rgb, grad_rgb_marched, bg, grad_rgb, grad_weight, grad_last,
                                 n_rays, as_stream(s));
}

}  // extern "C"
