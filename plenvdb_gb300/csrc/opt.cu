// Per-voxel Adam over the active voxels of a leaf store (DensityOpt/ColorOpt,
// plenvdb.h:686-790; densityvdb.cu:185-349, colorvdb.cu:179-351) and the dense
// Adam used for the rgbnet (lib/cuda/adam_upd_kernel.cu:8-132).
#include <cmath>

#include "pvdb_internal.cuh"
#include "tc.cuh"

struct pvdb_opt_s {
  pvdb_grid_s* params = nullptr;  // borrowed (the caller keeps it alive, plenvdb.h:695)
  pvdb_grid_s* exp_avg = nullptr;
  pvdb_grid_s* exp_avg_sq = nullptr;
  pvdb_grid_s* per_lr = nullptr;  // optional ScaleGrid with the params' topology
  int step = 0;
  float lr, eps, beta0, beta1;
};

namespace pvdb {

// Bias-corrected step size, float arithmetic on the host exactly as
// plenvdb.h:753 / :776 and adam_upd_kernel.cu:72.
float adam_step_size(float lr, float beta_m, float beta_v, int step) {
  return lr * std::sqrt(1 - std::pow(beta_v, (float)step)) / (1 - std::pow(beta_m, (float)step));
}

// One thread per (slot, group); a group is 1 channel for scalar grids and a
// 3-channel Vec3 for multi-channel grids (the reference skips a Vec3 only when
// all three gradient components are zero, colorvdb.cu:318). With a leaf list
// only the listed leaves are visited (grid-stride; the count is on the device).
__global__ void k_vdb_adam(GridView g, float* __restrict__ m, float* __restrict__ v,
                           const float* __restrict__ perlr, float stepsz,
                           const float* __restrict__ stepsz_dev, float eps, float b0, float b1,
                           int mode, int zero_after, const int32_t* __restrict__ list,
                           const uint32_t* __restrict__ count, const float* __restrict__ tv) {
  grid_dep_sync();
  const int G = g.C == 1 ? 1 : 3;
  const int ngroups = g.C / G;
  const int64_t per = int64_t(kLeafVox) * ngroups;
  const int64_t nl = list ? int64_t(*count) : int64_t(g.nleaf);
  if (stepsz_dev) stepsz = *stepsz_dev;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < nl * per;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t li = i / per;
    const int leaf = list ? list[li] : int(li);
    const int64_t rem = i - li * per;
    const int vox = int(rem / ngroups);
    const int grp = int(rem % ngroups);
    const int64_t slot = int64_t(leaf) * kLeafVox + vox;
    if (!((__ldg(g.mask + leaf * 8 + (vox >> 6)) >> (vox & 63)) & 1ull)) continue;
    const int64_t base = slot * g.C + int64_t(grp) * G;
    float gr[3];
    bool allzero = true;
    for (int q = 0; q < G; ++q) {
      gr[q] = g.grad[base + q];
      // deferred sparse TV: its term joins the channels with a gradient
      if (tv && gr[q] != 0.f) gr[q] = gr[q] + tv[base + q];
      allzero = allzero && (gr[q] == 0.f);
    }
    if (mode == 1 && allzero) continue;
    const float lrf = mode == 2 ? perlr[slot] : 1.f;
    for (int q = 0; q < G; ++q) {
      const float mn = b0 * m[base + q] + (1 - b0) * gr[q];
      const float vn = b1 * v[base + q] + (1 - b1) * gr[q] * gr[q];
      m[base + q] = mn;
      v[base + q] = vn;
      const float num = mode == 2 ? lrf * stepsz * mn : stepsz * mn;
      const float old = g.data[base + q];
      const float nv = old - num / (eps + sqrtf(vn));
      g.data[base + q] = nv;
      if (zero_after) g.grad[base + q] = 0.f;
      // keep the march's brick bound an upper bound (scalar grids only)
      if (g.bmax && !(nv <= old))
        bmax_raise(g, g.origin[leaf * 3] + (vox >> 6), g.origin[leaf * 3 + 1] + ((vox >> 3) & 7),
                   g.origin[leaf * 3 + 2] + (vox & 7), nv);
    }
  }
}

// Adds a thread's two counts to counts[0..1], one atomic per warp (every lane
// of the warp calls it).
__device__ __forceinline__ void count_add(uint32_t* counts, uint32_t a, uint32_t b) {
  a = __reduce_add_sync(0xffffffffu, a);
  b = __reduce_add_sync(0xffffffffu, b);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(counts, a);
    atomicAdd(counts + 1, b);
  }
}

// The same update for scalar grids (density), one thread per voxel. A warp's
// 32 voxels are 32 consecutive offsets of one leaf (one x, four y, all z), so
// the brick bounds their growing values raise (bmax_raise) span at most
// 2 x 3 x 4 bricks: the warp raises every brick of that box to the largest
// grown value, one atomicMax per brick from its own lane, instead of up to 8
// atomics per voxel on the same few words. A bound may end above bmax_raise's
// (by a value from at most a few voxels away); it stays an upper bound, which
// is all the march's skip test needs (a skipped sample's alpha is below the
// threshold either way, so results do not depend on it). Per-voxel
// arithmetic is identical to k_vdb_adam.
__global__ void __launch_bounds__(256)
    k_vdb_adam1(GridView g, float* __restrict__ m, float* __restrict__ v,
                const float* __restrict__ perlr, float stepsz, const float* __restrict__ stepsz_dev,
                float eps, float b0, float b1, int mode, int zero_after,
                const int32_t* __restrict__ list, const uint32_t* __restrict__ count,
                const float* __restrict__ tv, uint32_t* counts) {
  grid_dep_sync();
  const int64_t nl = list ? int64_t(*count) : int64_t(g.nleaf);
  if (stepsz_dev) stepsz = *stepsz_dev;
  const int lane = threadIdx.x & 31;
  uint32_t n_act = 0, n_upd = 0;
  // whole leaves and whole warps: every lane of a warp takes the same trips
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < nl * kLeafVox;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int leaf = list ? list[i >> 9] : int(i >> 9);
    const int vox = int(i & 511);
    const int64_t slot = int64_t(leaf) * kLeafVox + vox;
    const bool active = (__ldg(g.mask + leaf * 8 + (vox >> 6)) >> (vox & 63)) & 1ull;
    // the voxel's gradient, TV term, moments and value are loaded together
    float gr = 0.f, tt = 0.f, ms = 0.f, vs = 0.f, old = 0.f;
    if (active) {
      gr = g.grad[slot];
      if (tv) tt = tv[slot];
      ms = m[slot];
      vs = v[slot];
      old = g.data[slot];
    }
    if (tv && gr != 0.f) gr = gr + tt;  // deferred sparse TV
    bool grew = false;
    float nv = 0.f;
    n_act += active;
    if (active && !(mode == 1 && gr == 0.f)) {
      ++n_upd;
      const float lrf = mode == 2 ? perlr[slot] : 1.f;
      const float mn = b0 * ms + (1 - b0) * gr;
      const float vn = b1 * vs + (1 - b1) * gr * gr;
      m[slot] = mn;
      v[slot] = vn;
      const float num = mode == 2 ? lrf * stepsz * mn : stepsz * mn;
      nv = old - num / (eps + sqrtf(vn));
      g.data[slot] = nv;
      if (zero_after) g.grad[slot] = 0.f;
      grew = !(nv <= old);
    }
    // keep the march's brick bound an upper bound
    if (!g.bmax || !__any_sync(0xffffffffu, grew)) continue;
    const int x = g.origin[leaf * 3] + (vox >> 6);
    const int y = g.origin[leaf * 3 + 1] + ((vox >> 3) & 7);
    const int z = g.origin[leaf * 3 + 2] + (vox & 7);
    const int x0 = max((x - 2) >> 2, 0), x1 = min((x + 1) >> 2, g.bdim[0] - 1);
    const int y0 = max((y - 2) >> 2, 0), y1 = min((y + 1) >> 2, g.bdim[1] - 1);
    const int z0 = max((z - 2) >> 2, 0), z1 = min((z + 1) >> 2, g.bdim[2] - 1);
    const int big = 1 << 30;
    const int ux0 = __reduce_min_sync(0xffffffffu, grew ? x0 : big);
    const int ux1 = __reduce_max_sync(0xffffffffu, grew ? x1 : -1);
    const int uy0 = __reduce_min_sync(0xffffffffu, grew ? y0 : big);
    const int uy1 = __reduce_max_sync(0xffffffffu, grew ? y1 : -1);
    const int uz0 = __reduce_min_sync(0xffffffffu, grew ? z0 : big);
    const int uz1 = __reduce_max_sync(0xffffffffu, grew ? z1 : -1);
    const uint32_t kmax = __reduce_max_sync(0xffffffffu, grew ? fkey(nv) : 0u);
    const int ny = uy1 - uy0 + 1, nz = uz1 - uz0 + 1;
    if (kmax && lane < (ux1 - ux0 + 1) * ny * nz) {  // at most 24 bricks: one per lane
      const int bx = ux0 + lane / (ny * nz), by = uy0 + (lane / nz) % ny, bz = uz0 + lane % nz;
      atomicMax(g.bmax + (int64_t(bx) * g.bdim[1] + by) * g.bdim[2] + bz, kmax);
    }
  }
  if (counts) count_add(counts, n_act, n_upd);
}

// The same update for 12-channel grids (k0), one thread per voxel with the
// channels in float4 loads; the four Vec3 groups keep their own skip rule.
// Per-channel arithmetic is identical to k_vdb_adam.
// half: the grid's BF16 shadow, written with every updated voxel (NULL: none).
__global__ void k_vdb_adam_c12(GridView g, float* __restrict__ m, float* __restrict__ v,
                               const float* __restrict__ perlr, float stepsz,
                               const float* __restrict__ stepsz_dev, float eps, float b0, float b1,
                               int mode, int zero_after, const int32_t* __restrict__ list,
                               const uint32_t* __restrict__ count, __nv_bfloat16* half,
                               const float* __restrict__ tv, uint32_t* counts) {
  grid_dep_sync();
  const int64_t nl = list ? int64_t(*count) : int64_t(g.nleaf);
  if (stepsz_dev) stepsz = *stepsz_dev;
  uint32_t n_act = 0, n_upd = 0;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < nl * kLeafVox;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int leaf = list ? list[i >> 9] : int(i >> 9);
    const int vox = int(i & 511);
    if (!((__ldg(g.mask + leaf * 8 + (vox >> 6)) >> (vox & 63)) & 1ull)) continue;
    ++n_act;
    const int64_t slot = int64_t(leaf) * kLeafVox + vox;
    float4* g4 = reinterpret_cast<float4*>(g.grad + slot * 12);
    float4* m4 = reinterpret_cast<float4*>(m + slot * 12);
    float4* v4 = reinterpret_cast<float4*>(v + slot * 12);
    float4* d4 = reinterpret_cast<float4*>(g.data + slot * 12);
    // the voxel's gradient, TV terms, moments and values are loaded together
    // (one round trip; most voxels of a touched leaf are updated)
    float gr[12], tt[12], mm[12], vv[12], dd[12];
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const float4 x = g4[b], t = tv ? reinterpret_cast<const float4*>(tv + slot * 12)[b]
                                     : make_float4(0.f, 0.f, 0.f, 0.f);
      const float4 a = m4[b], c = v4[b], d = d4[b];
      gr[4 * b] = x.x; gr[4 * b + 1] = x.y; gr[4 * b + 2] = x.z; gr[4 * b + 3] = x.w;
      tt[4 * b] = t.x; tt[4 * b + 1] = t.y; tt[4 * b + 2] = t.z; tt[4 * b + 3] = t.w;
      mm[4 * b] = a.x; mm[4 * b + 1] = a.y; mm[4 * b + 2] = a.z; mm[4 * b + 3] = a.w;
      vv[4 * b] = c.x; vv[4 * b + 1] = c.y; vv[4 * b + 2] = c.z; vv[4 * b + 3] = c.w;
      dd[4 * b] = d.x; dd[4 * b + 1] = d.y; dd[4 * b + 2] = d.z; dd[4 * b + 3] = d.w;
    }
    if (tv) {  // deferred sparse TV: its terms join the channels with a gradient
#pragma unroll
      for (int ch = 0; ch < 12; ++ch)
        if (gr[ch] != 0.f) gr[ch] = gr[ch] + tt[ch];
    }
    bool live[4];
    bool any = false;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      live[q] = mode != 1 || gr[3 * q] != 0.f || gr[3 * q + 1] != 0.f || gr[3 * q + 2] != 0.f;
      any = any || live[q];
    }
    if (!any) continue;
    ++n_upd;
    const float lrf = mode == 2 ? perlr[slot] : 1.f;
#pragma unroll
    for (int ch = 0; ch < 12; ++ch) {
      if (!live[ch / 3]) continue;
      const float mn = b0 * mm[ch] + (1 - b0) * gr[ch];
      const float vn = b1 * vv[ch] + (1 - b1) * gr[ch] * gr[ch];
      mm[ch] = mn;
      vv[ch] = vn;
      const float num = mode == 2 ? lrf * stepsz * mn : stepsz * mn;
      dd[ch] = dd[ch] - num / (eps + sqrtf(vn));
    }
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      m4[b] = make_float4(mm[4 * b], mm[4 * b + 1], mm[4 * b + 2], mm[4 * b + 3]);
      v4[b] = make_float4(vv[4 * b], vv[4 * b + 1], vv[4 * b + 2], vv[4 * b + 3]);
      d4[b] = make_float4(dd[4 * b], dd[4 * b + 1], dd[4 * b + 2], dd[4 * b + 3]);
      if (zero_after) g4[b] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (half) {  // the voxel's 32-byte shadow record: channels 0..11, then zeros
      uint4* h4 = reinterpret_cast<uint4*>(half + slot * kHalfStride);
      h4[0] = make_uint4(tc::pack_bf16(dd[0], dd[1]), tc::pack_bf16(dd[2], dd[3]),
                         tc::pack_bf16(dd[4], dd[5]), tc::pack_bf16(dd[6], dd[7]));
      h4[1] = make_uint4(tc::pack_bf16(dd[8], dd[9]), tc::pack_bf16(dd[10], dd[11]), 0u, 0u);
    }
  }
  if (counts) count_add(counts, n_act, n_upd);
}

// zero_after for voxels the Adam pass skipped (mode 1, all-zero gradient):
// nothing to do, their gradient is already zero.

__global__ void k_clear_u8(uint8_t* t, int n) {
  grid_dep_sync();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) t[i] = 0;
}

template <int MODE>
__global__ void k_adam_dense(float* __restrict__ p, const float* __restrict__ g,
                             float* __restrict__ m, float* __restrict__ v,
                             const float* __restrict__ perlr, int64_t n, float stepsz,
                             const float* __restrict__ stepsz_dev, float b1, float b2, float eps) {
  grid_dep_sync();
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  if (MODE == 1 && gi == 0.f) return;
  if (stepsz_dev) stepsz = *stepsz_dev;
  // the reference kernel's float arithmetic as nvcc contracts it
  // (adam_upd_kernel.cu:19-21): the decayed moment fused onto the rounded
  // gradient term, then a correctly rounded sqrt and divide
  const float mn = __fmaf_rn(b1, m[i], __fmul_rn(1.f - b1, gi));
  const float vn = __fmaf_rn(b2, v[i], __fmul_rn(__fmul_rn(1.f - b2, gi), gi));
  m[i] = mn;
  v[i] = vn;
  const float num = MODE == 2 ? __fmul_rn(__fmul_rn(stepsz, perlr[i]), mn) : __fmul_rn(stepsz, mn);
  p[i] = __fsub_rn(p[i], __fdiv_rn(num, __fadd_rn(__fsqrt_rn(vn), eps)));
}

int adam_dense_launch(float* param, const float* grad, float* m, float* v, const float* perlr,
                      int64_t n, float stepsz, float b1, float b2, float eps, int mode,
                      cudaStream_t st, const float* stepsz_dev) {
  if (n <= 0) return PVDB_OK;
  const int nb = ceil_div(n, 256);
  const float* sd = stepsz_dev;
  if (mode == 1)
    launch_k(k_adam_dense<1>, nb, 256, 0, st, param, grad, m, v, perlr, n, stepsz, sd, b1, b2, eps);
  else if (mode == 2)
    launch_k(k_adam_dense<2>, nb, 256, 0, st, param, grad, m, v, perlr, n, stepsz, sd, b1, b2, eps);
  else
    launch_k(k_adam_dense<0>, nb, 256, 0, st, param, grad, m, v, perlr, n, stepsz, sd, b1, b2, eps);
  PVDB_CHECK_LAUNCH("k_adam_dense");
  return PVDB_OK;
}

int opt_launch(pvdb_opt_s* o, int mode, int zero_after, float stepsz, const float* stepsz_dev,
               cudaStream_t st, const float* tv = nullptr, uint32_t* counts = nullptr);

// Advances the step counter and returns this step's Adam step size.
float opt_next_stepsz(pvdb_opt_s* o) {
  o->step++;
  return adam_step_size(o->lr, o->beta0, o->beta1, o->step);
}

// Runs one voxel-Adam step (used by the C ABI and the fused train step).
int opt_step_launch(pvdb_opt_s* o, int mode, int zero_after, cudaStream_t st) {
  return opt_launch(o, mode, zero_after, opt_next_stepsz(o), nullptr, st);
}

// The launches of one voxel-Adam step; the step size is stepsz, or
// *stepsz_dev when that is given (a captured graph reads it each replay).
// tv (optional): TV terms of the touched leaves' voxels (tv_terms_launch),
// added to the channels with a nonzero gradient before the update.
// counts (optional, 1- and 12-channel grids): two words that get the number
// of active voxels visited and of voxels updated (the stage profiler's byte
// model).
int opt_launch(pvdb_opt_s* o, int mode, int zero_after, float stepsz, const float* stepsz_dev,
               cudaStream_t st, const float* tv, uint32_t* counts) {
  pvdb_grid_s* g = o->params;
  // mode 1 skips voxels whose gradient is zero: only the touched leaves matter
  const bool use_list = mode == 1 && !g->all_touched;
  if (tv && !use_list) return set_error(PVDB_ERR_STATE, "deferred TV needs the touched leaves");
  if (g->nslots()) {
    if (use_list) {
      int rc = touched_list(g, st);
      if (rc) return rc;
    }
    if (g->C == 12)
      launch_k(k_vdb_adam_c12, stride_grid(), 256, 0, st, g->view(), o->exp_avg->d_data,
               o->exp_avg_sq->d_data, mode == 2 ? o->per_lr->d_data : nullptr, stepsz, stepsz_dev,
               o->eps, o->beta0, o->beta1, mode, zero_after, use_list ? g->d_tlist : nullptr,
               g->d_tcount, g->d_half, tv, counts);
    else if (g->C == 1)
      launch_k(k_vdb_adam1, stride_grid(), 256, 0, st, g->view(), o->exp_avg->d_data,
               o->exp_avg_sq->d_data, mode == 2 ? o->per_lr->d_data : nullptr, stepsz, stepsz_dev,
               o->eps, o->beta0, o->beta1, mode, zero_after, use_list ? g->d_tlist : nullptr,
               g->d_tcount, tv, counts);
    else
      launch_k(k_vdb_adam, stride_grid(), 256, 0, st, g->view(), o->exp_avg->d_data,
               o->exp_avg_sq->d_data, mode == 2 ? o->per_lr->d_data : nullptr, stepsz, stepsz_dev,
               o->eps, o->beta0, o->beta1, mode, zero_after, use_list ? g->d_tlist : nullptr,
               g->d_tcount, tv);
    PVDB_CHECK_LAUNCH("k_vdb_adam");
    if (g->C != 12) g->half_valid = false;  // only the 12-channel update writes the shadow
  }
  if (zero_after && g->nleaf) {
    launch_k(k_clear_u8, ceil_div(g->nleaf, 256), 256, 0, st, g->d_touched, g->nleaf);
    PVDB_CHECK_LAUNCH("k_clear_u8");
    g->all_touched = false;
    g->tlist_valid = false;
  }
  return PVDB_OK;
}

pvdb_grid_s* opt_params(pvdb_opt_s* o) { return o->params; }
pvdb_grid_s* opt_moment(pvdb_opt_s* o, int which) { return which ? o->exp_avg_sq : o->exp_avg; }
float opt_lr_scale(pvdb_opt_s* o, float factor) {
  o->lr *= factor;
  return o->lr;
}

}  // namespace pvdb

using namespace pvdb;

extern "C" {

int pvdb_opt_create(pvdb_grid g, float lr, float eps, float beta0, float beta1, pvdb_opt* out) {
  clear_error();
  PVDB_REQUIRE(g && out, "null argument");
  pvdb_opt_s* o = new pvdb_opt_s();
  o->params = g;
  o->lr = lr;
  o->eps = eps;
  o->beta0 = beta0;
  o->beta1 = beta1;
  int rc = pvdb_grid_create_like(g, g->C, 0.f, &o->exp_avg);
  if (!rc) rc = pvdb_grid_create_like(g, g->C, 0.f, &o->exp_avg_sq);
  if (rc) {
    pvdb_opt_destroy(o);
    return rc;
  }
  *out = o;
  return PVDB_OK;
}

int pvdb_opt_destroy(pvdb_opt o) {
  if (!o) return PVDB_OK;
  pvdb_grid_destroy(o->exp_avg);
  pvdb_grid_destroy(o->exp_avg_sq);
  pvdb_grid_destroy(o->per_lr);
  delete o;
  return PVDB_OK;
}

int pvdb_opt_step(pvdb_opt o, int32_t mode, int32_t zero_grad_after, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(o, "null optimiser");
  PVDB_REQUIRE(mode >= 0 && mode <= 2, "mode must be 0, 1 or 2");
  if (mode == 2 && !o->per_lr)
    return set_error(PVDB_ERR_STATE, "step(2) needs set_pervoxel_lr first");
  return opt_step_launch(o, mode, zero_grad_after, as_stream(s));
}

int pvdb_opt_zero_grad(pvdb_opt o, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(o, "null optimiser");
  return pvdb_grid_zero_grad(o->params, s);
}

int pvdb_opt_set_grad(pvdb_opt o, const float* arr, int64_t n, int32_t mem, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(o, "null optimiser");
  return pvdb_grid_copy_from_dense(o->params, PVDB_WHICH_GRAD, arr, n, mem, s);
}

int pvdb_opt_set_pervoxel_lr(pvdb_opt o, const float* count, int64_t n, int32_t mem,
                             pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(o && count, "null argument");
  pvdb_grid_s* g = o->params;
  PVDB_REQUIRE(n == int64_t(g->reso[0]) * g->reso[1] * g->reso[2],
               "per-voxel lr size must be reso[0]*reso[1]*reso[2]");
  if (!o->per_lr) {
    int rc = pvdb_grid_create_like(g, 1, 0.f, &o->per_lr);
    if (rc) return rc;
  }
  return pvdb_grid_copy_from_dense(o->per_lr, PVDB_WHICH_DATA, count, n, mem, s);
}

int pvdb_opt_update_lr(pvdb_opt o, float factor) {
  clear_error();
  PVDB_REQUIRE(o, "null optimiser");
  o->lr *= factor;
  return PVDB_OK;
}

int pvdb_opt_get_scalars(pvdb_opt o, int32_t* step, float* lr, float* eps, float* beta0,
                         float* beta1) {
  clear_error();
  PVDB_REQUIRE(o, "null optimiser");
  if (step) *step = o->step;
  if (lr) *lr = o->lr;
  if (eps) *eps = o->eps;
  if (beta0) *beta0 = o->beta0;
  if (beta1) *beta1 = o->beta1;
  return PVDB_OK;
}

int pvdb_opt_set_scalars(pvdb_opt o, int32_t step, float lr, float eps, float beta0,
                         float beta1) {
  clear_error();
  PVDB_REQUIRE(o, "null optimiser");
  o->step = step;
  o->lr = lr;
  o->eps = eps;
  o->beta0 = beta0;
  o->beta1 = beta1;
  return PVDB_OK;
}

int pvdb_opt_moments(pvdb_opt o, pvdb_grid* exp_avg, pvdb_grid* exp_avg_sq) {
  clear_error();
  PVDB_REQUIRE(o, "null optimiser");
  if (exp_avg) *exp_avg = o->exp_avg;
  if (exp_avg_sq) *exp_avg_sq = o->exp_avg_sq;
  return PVDB_OK;
}

int pvdb_adam_dense(float* param, const float* grad, float* exp_avg, float* exp_avg_sq,
                    const float* perlr, int64_t n, int32_t step, float beta1, float beta2,
                    float lr, float eps, int32_t mode, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(n >= 0, "negative size");
  if (n == 0) return PVDB_OK;
  PVDB_REQUIRE(param && grad && exp_avg && exp_avg_sq, "null argument");
  PVDB_REQUIRE(mode >= 0 && mode <= 2, "mode must be 0, 1 or 2");
  PVDB_REQUIRE(mode != 2 || perlr, "mode 2 needs perlr");
  PVDB_REQUIRE(step >= 1, "step must be >= 1");
  const float stepsz = adam_step_size(lr, beta1, beta2, step);
  return adam_dense_launch(param, grad, exp_avg, exp_avg_sq, perlr, n, stepsz, beta1, beta2, eps,
                           mode, as_stream(s));
}

}  // extern "C"
