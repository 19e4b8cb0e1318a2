// Fused training march over ragged per-ray sample counts, one ray per warp.
//
// Forward (k_march_fwd) fuses, per ray: sample_pts_on_rays
// (render_utils_kernel.cu:196-242), the bbox filter and MaskGrid lookup
// (dvgo.py:290-315), wld2idx (grid.py:77-78), DensityVDB trilinear
// (densityvdb.cu:101-125), raw2alpha (render_utils_kernel.cu:430-443), the
// alpha threshold (dvgo.py:319-325) and alpha2weight with its T < 1e-3 early
// stop (render_utils_kernel.cu:576-605). The transmittance chain is walked in
// sample order over the kept lanes of each 32-sample chunk with exactly the
// reference's rounding. Only per-ray alpha / step lists are kept for the
// backward.
//
// k_march_gather compacts the colour samples (weight > thres, dvgo.py:329-335)
// into dense rows and samples the k0 grid there (colorvdb.cu:81-111).
//
// Backward (k_march_bwd) recovers transmittance from the saved alphas and
// weights, runs alpha2weight_backward (:653-677) as a suffix scan and
// raw2alpha_backward (:506-517),
// and emits the 8 corner keys of every kept sample; a stable radix sort by
// voxel slot and a sequential per-slot sum (reduce.cuh) then add the density
// and k0 gradients deterministically.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "march.cuh"
#include "reduce.cuh"

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

__global__ void __launch_bounds__(kMarchThreads)
    k_march_fwd(GridView gd, const float* __restrict__ ro, const float* __restrict__ rd, int R,
                MarchP P, MarchW W) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * kMarchWarps + warp;
  if (r >= R) return;
  float o[3], d[3];
  load_ray(ro, rd, r, o, d);
  RaySetup rs;
  ray_setup(o, d, P.mn, P.mx, P.near_, P.far_, P.stepdist, rs);
  int64_t ns = rs.n_steps;
  if (ns > P.cap) {
    if (lane == 0) atomicOr(W.totals + 3, 1u);
    ns = P.cap;
  }
  if (lane < 3) {
    W.ray_sd[r * 6 + lane] = rs.start[lane];
    W.ray_sd[r * 6 + 3 + lane] = rs.dir[lane];
  }
  const unsigned lt = lanemask_lt();
  const int64_t sbase = int64_t(r) * P.cap;
  float T = 1.f;
  int nk = 0, nc = 0;
  for (int64_t base = 0; base < ns; base += 32) {
    const int64_t k = base + lane;
    float alpha = 0.f;
    bool keep = false;
    if (k < ns) {
      float p[3];
      ray_point(rs, P.stepdist, k, p);
      if (!out_of_bbox(p, P.mn, P.mx) &&
          (!P.mask || mask_lookup(P.mask, P.mshape, p, P.mscale, P.mshift))) {
        float idx[3];
        world_to_index(p, P.mn, P.ext, P.wsm1, idx);
        const float sigma = trilinear1(gd, idx[0], idx[1], idx[2]);
        float e;
        alpha = raw2alpha(sigma, P.shift, P.interval, e);
        keep = alpha > P.thr;
      }
    }
    unsigned km = __ballot_sync(0xffffffffu, keep);
    // alpha2weight over the kept lanes, in sample order (uniform across the warp)
    float w = 0.f;
    bool stop = false;
    unsigned rem = km;
    while (rem) {
      const int l = __ffs(rem) - 1;
      rem &= rem - 1;
      const float a = __shfl_sync(0xffffffffu, alpha, l);
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
      W.k_alpha[pos] = alpha;
      W.k_w[pos] = w;
      W.k_step[pos] = int32_t(k) | (col ? int32_t(0x80000000) : 0);
      W.k_row[pos] = -1;
    }
    nk += __popc(km);
    nc += __popc(cm);
    if (stop) break;
  }
  if (lane == 0) {
    W.T_last[r] = T;
    W.n_kept[r] = nk;
    W.n_color[r] = nc;
  }
}

__device__ __forceinline__ void load_setup(const MarchW& W, int r, RaySetup& rs) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    rs.start[a] = W.ray_sd[r * 6 + a];
    rs.dir[a] = W.ray_sd[r * 6 + 3 + a];
  }
}

__global__ void k_march_totals(MarchW W) {
  W.totals[2] = W.totals[0] * 8u;
}

// Multi-channel trilinear of k0 at one point (colorvdb.cu:97-108 ordering).
__device__ __forceinline__ void k0_trilinear(const GridView& g, const float idx[3], float* out) {
  const int i = ifloor(idx[0]), j = ifloor(idx[1]), k = ifloor(idx[2]);
  float sc[8];
  corner_scales(idx[0] - float(i), idx[1] - float(j), idx[2] - float(k), sc);
  int slots[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    int di, dj, dk;
    corner_delta(c, di, dj, dk);
    slots[c] = slot_of(g, i + di, j + dj, k + dk);
  }
  if (g.C == 12) {
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
  } else {
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
}

__global__ void __launch_bounds__(kMarchThreads)
    k_march_gather(GridView gk, int R, MarchP P, MarchW W) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * kMarchWarps + warp;
  if (r >= R) return;
  const int nk = int(W.n_kept[r]);
  if (nk == 0) return;
  RaySetup rs;
  load_setup(W, r, rs);
  const unsigned lt = lanemask_lt();
  const int64_t sbase = int64_t(r) * P.cap;
  int64_t row = W.color_off[r];
  for (int base = 0; base < nk; base += 32) {
    const int i = base + lane;
    int32_t st = 0;
    bool col = false;
    if (i < nk) {
      st = W.k_step[sbase + i];
      col = st < 0;
    }
    const unsigned cm = __ballot_sync(0xffffffffu, col);
    if (col) {
      const int64_t m = row + __popc(cm & lt);
      const int32_t k = st & 0x7fffffff;
      float p[3], idx[3];
      ray_point(rs, P.stepdist, k, p);
      world_to_index(p, P.mn, P.ext, P.wsm1, idx);
      if (gk.C > 0) k0_trilinear(gk, idx, W.r_k0 + m * gk.C);
      W.r_w[m] = W.k_w[sbase + i];
      W.r_alpha[m] = W.k_alpha[sbase + i];
      W.r_ray[m] = r;
      W.r_step[m] = k;
      W.k_row[sbase + i] = int32_t(m);
    }
    row += __popc(cm);
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
                const float* __restrict__ grad_last, uint32_t* keys) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * kMarchWarps + warp;
  if (r >= R) return;
  const int nk = int(W.n_kept[r]);
  if (nk == 0) return;
  const int64_t sbase = int64_t(r) * P.cap;
  const int64_t kb = W.kept_off[r];
  const int nchunks = (nk + 31) >> 5;
  RaySetup rs;
  load_setup(W, r, rs);
  float carry = (grad_last ? grad_last[r] : 0.f) * W.T_last[r];
  for (int c = nchunks - 1; c >= 0; --c) {
    const int i = c * 32 + lane;
    const bool valid = i < nk;
    float a = 1.f, w = 0.f, gw = 0.f;
    int32_t st = 0, row = -1;
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
      W.b_pos[s * 3 + 0] = idx[0];
      W.b_pos[s * 3 + 1] = idx[1];
      W.b_pos[s * 3 + 2] = idx[2];
      W.b_gsig[s] = gs;
      W.b_row[s] = row;
      emit_corner_keys(gd, idx[0], idx[1], idx[2], keys, s);
    }
  }
}

// Keys of the k0 grid (when its topology differs from the density grid's).
__global__ void k_march_keys_k0(GridView gk, MarchW W, uint32_t* keys) {
  const int64_t n = W.totals[0];
  for (int64_t s = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; s < n;
       s += int64_t(gridDim.x) * blockDim.x) {
    if (W.b_row[s] >= 0) {
      emit_corner_keys(gk, W.b_pos[s * 3], W.b_pos[s * 3 + 1], W.b_pos[s * 3 + 2], keys, s);
    } else {
#pragma unroll
      for (int c = 0; c < 8; ++c) keys[s * 8 + c] = kInvalidKey;
    }
  }
}

struct MarchSrc {
  const float* xyz;
  const float* gsig;
  const int32_t* row;
  const float* gk0;
  int C;
  __device__ __forceinline__ void pos(int64_t s, float& x, float& y, float& z) const {
    x = xyz[s * 3];
    y = xyz[s * 3 + 1];
    z = xyz[s * 3 + 2];
  }
  __device__ __forceinline__ float gd(int64_t s) const { return gsig ? gsig[s] : 0.f; }
  __device__ __forceinline__ bool has_c(int64_t s) const { return gk0 && row[s] >= 0; }
  __device__ __forceinline__ float gc(int64_t s, int ch) const {
    return gk0[int64_t(row[s]) * C + ch];
  }
};

// --------------------------------------------------------------- composite
__global__ void __launch_bounds__(kMarchThreads)
    k_composite_fwd(MarchW W, const float* __restrict__ rgb, float bg, float* out, int R) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * kMarchWarps + warp;
  if (r >= R) return;
  const int n = int(W.n_color[r]);
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
}

int march_forward_impl(pvdb_march_s* m, pvdb_grid_s* density, pvdb_grid_s* k0, const float* ro,
                       const float* rd, int R, const pvdb_march_params* prm, const uint8_t* mask,
                       const int32_t* mshape, cudaStream_t st) {
  if (k0) {
    for (int a = 0; a < 3; ++a)
      PVDB_REQUIRE(k0->reso[a] == density->reso[a], "k0 and density grids need the same resolution");
    if (m->k0_channels < k0->C) {
      dev_free(m->w.r_k0);
      m->w.r_k0 = nullptr;
      int rc = dev_alloc((void**)&m->w.r_k0, size_t(m->slots) * k0->C * 4);
      if (rc) return rc;
      m->k0_channels = k0->C;
    }
  }
  fill_params(prm, density, mask, mshape, m->cap, m->p);
  m->n_rays = R;
  m->density = density;
  m->k0 = k0;
  PVDB_CHECK_CUDA(cudaMemsetAsync(m->w.totals, 0, 16, st));
  if (R > 0) {
    const int nb = ceil_div(R, kMarchWarps);
    k_march_fwd<<<nb, kMarchThreads, 0, st>>>(density->view(), ro, rd, R, m->p, m->w);
    PVDB_CHECK_LAUNCH("k_march_fwd");
    int rc = scan_exclusive_u32(m->w.n_kept, m->w.kept_off, R, m->w.totals + 0, &m->scan_partial,
                                &m->scan_partial_cap, st);
    if (rc) return rc;
    rc = scan_exclusive_u32(m->w.n_color, m->w.color_off, R, m->w.totals + 1, &m->scan_partial,
                            &m->scan_partial_cap, st);
    if (rc) return rc;
    k_march_totals<<<1, 1, 0, st>>>(m->w);
    PVDB_CHECK_LAUNCH("k_march_totals");
    if (m->prof) prof_mark(st, 1);
    GridView gk{};
    if (k0) gk = k0->view();
    k_march_gather<<<nb, kMarchThreads, 0, st>>>(gk, R, m->p, m->w);
    PVDB_CHECK_LAUNCH("k_march_gather");
    if (m->prof) prof_mark(st, 2);
  }
  m->has_fwd = true;
  return PVDB_OK;
}

static bool same_topology(const pvdb_grid_s* a, const pvdb_grid_s* b) {
  if (a->nleaf != b->nleaf) return false;
  for (int q = 0; q < 3; ++q)
    if (a->ldim[q] != b->ldim[q]) return false;
  return a->h_table == b->h_table;
}

int march_backward_impl(pvdb_march_s* m, const float* grad_w, const float* grad_last,
                        const float* grad_k0, cudaStream_t st) {
  pvdb_grid_s* density = m->density;
  pvdb_grid_s* k0 = m->k0;
  const int R = m->n_rays;
  if (R == 0) return PVDB_OK;
  const int64_t nmax = m->slots * 8;
  int rc = scratch_reserve(m->red, nmax);
  if (rc) return rc;
  const int nb = ceil_div(R, kMarchWarps);
  k_march_bwd<<<nb, kMarchThreads, 0, st>>>(density->view(), R, m->p, m->w, grad_w, grad_last,
                                            m->red.keys[0]);
  PVDB_CHECK_LAUNCH("k_march_bwd");
  if (m->prof) prof_mark(st, 6);
  int buf = 0;
  rc = radix_sort_pairs_dev(m->red, nmax, m->w.totals + 2, slot_key_bits(density->nslots()), true,
                            &buf, st);
  if (rc) return rc;
  if (m->prof) prof_mark(st, 7);
  const bool use_k0 = k0 && grad_k0;
  const bool shared = use_k0 && same_topology(density, k0);
  MarchSrc src{m->w.b_pos, m->w.b_gsig, m->w.b_row, shared ? grad_k0 : nullptr,
               k0 ? k0->C : 0};
  const int grid = num_sms() * 16;
  k_segment_reduce<MarchSrc><<<grid, 256, 0, st>>>(
      m->red.keys[buf], m->red.vals[buf], nmax, m->w.totals + 2, src, density->d_grad,
      shared ? k0->d_grad : nullptr, k0 ? k0->C : 0, density->d_touched,
      shared ? k0->d_touched : nullptr);
  PVDB_CHECK_LAUNCH("k_segment_reduce(march)");
  if (use_k0 && !shared) {
    rc = scratch_reserve(m->red2, nmax);
    if (rc) return rc;
    k_march_keys_k0<<<grid, 256, 0, st>>>(k0->view(), m->w, m->red2.keys[0]);
    PVDB_CHECK_LAUNCH("k_march_keys_k0");
    rc = radix_sort_pairs_dev(m->red2, nmax, m->w.totals + 2, slot_key_bits(k0->nslots()), true,
                              &buf, st);
    if (rc) return rc;
    MarchSrc src2{m->w.b_pos, nullptr, m->w.b_row, grad_k0, k0->C};
    k_segment_reduce<MarchSrc><<<grid, 256, 0, st>>>(m->red2.keys[buf], m->red2.vals[buf], nmax,
                                                     m->w.totals + 2, src2, nullptr, k0->d_grad,
                                                     k0->C, nullptr, k0->d_touched);
    PVDB_CHECK_LAUNCH("k_segment_reduce(k0)");
  }
  if (m->prof) prof_mark(st, 8);
  return PVDB_OK;
}

int composite_forward_impl(pvdb_march_s* m, const float* rgb, float bg, float* out, int R,
                           cudaStream_t st) {
  if (R <= 0) return PVDB_OK;
  k_composite_fwd<<<ceil_div(R, kMarchWarps), kMarchThreads, 0, st>>>(m->w, rgb, bg, out, R);
  PVDB_CHECK_LAUNCH("k_composite_fwd");
  return PVDB_OK;
}

int composite_backward_impl(pvdb_march_s* m, const float* rgb, const float* g, float bg,
                            float* grad_rgb, float* grad_w, float* grad_last, int R,
                            cudaStream_t st) {
  if (R <= 0) return PVDB_OK;
  k_composite_bwd<<<ceil_div(R, kMarchWarps), kMarchThreads, 0, st>>>(m->w, rgb, g, bg, grad_rgb,
                                                                      grad_w, grad_last, R);
  PVDB_CHECK_LAUNCH("k_composite_bwd");
  return PVDB_OK;
}

}  // namespace pvdb

using namespace pvdb;

extern "C" {

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
  if ((rc = dev_alloc((void**)&w.ray_sd, R * 24)) ||
      (rc = dev_alloc((void**)&w.T_last, R * 4)) || (rc = dev_alloc((void**)&w.n_kept, R * 4)) ||
      (rc = dev_alloc((void**)&w.n_color, R * 4)) ||
      (rc = dev_alloc((void**)&w.kept_off, R * 4)) ||
      (rc = dev_alloc((void**)&w.color_off, R * 4)) ||
      (rc = dev_alloc((void**)&w.k_alpha, S * 4)) || (rc = dev_alloc((void**)&w.k_w, S * 4)) ||
      (rc = dev_alloc((void**)&w.k_step, S * 4)) || (rc = dev_alloc((void**)&w.k_row, S * 4)) ||
      (rc = dev_alloc((void**)&w.r_w, S * 4)) || (rc = dev_alloc((void**)&w.r_alpha, S * 4)) ||
      (rc = dev_alloc((void**)&w.r_ray, S * 4)) || (rc = dev_alloc((void**)&w.r_step, S * 4)) ||
      (rc = dev_alloc((void**)&w.b_pos, S * 12)) || (rc = dev_alloc((void**)&w.b_gsig, S * 4)) ||
      (rc = dev_alloc((void**)&w.b_row, S * 4)) || (rc = dev_alloc((void**)&w.totals, 64))) {
    pvdb_march_destroy(m);
    return rc;
  }
  cudaError_t e = cudaMemset(w.totals, 0, 64);
  if (e != cudaSuccess) {
    pvdb_march_destroy(m);
    return cuda_error(e, "cudaMemset");
  }
  *out = m;
  return PVDB_OK;
}

int pvdb_march_destroy(pvdb_march m) {
  if (!m) return PVDB_OK;
  MarchW& w = m->w;
  void* ptrs[] = {w.ray_sd, w.T_last, w.n_kept, w.n_color, w.kept_off, w.color_off, w.k_alpha, w.k_w,
                  w.k_step, w.k_row, w.r_k0, w.r_w, w.r_alpha, w.r_ray, w.r_step, w.b_pos,
                  w.b_gsig, w.b_row, w.totals, m->scan_partial, m->hpe, m->wpart, m->mlp_packed,
                  m->t_rgb, m->t_grad_rgb, m->t_grad_w, m->t_grad_k0, m->t_grad_last,
                  m->t_loss_part, m->t_rgb_marched};
  for (void* p : ptrs) dev_free(p);
  free_scratch(m->red);
  free_scratch(m->red2);
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
                            as_stream(s));
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
  PVDB_REQUIRE(rgb || n_rays == 0, "null rgb");
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
