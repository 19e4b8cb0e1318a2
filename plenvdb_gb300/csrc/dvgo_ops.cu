// Standalone DVGO compositing primitives (render_utils_cuda,
// lib/cuda/render_utils_kernel.cu). They keep the reference's flattened
// [ray_id, step_id] representation and one-thread-per-ray scans, and exist for
// drop-in parity of the unfused path; the training hot path is march.cu.
#include "ray_ops.cuh"

namespace pvdb {

__global__ void k_raw2alpha(const float* __restrict__ d, int64_t n, float shift, float interval,
                            float* exp_d, float* alpha) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  float e;
  alpha[i] = raw2alpha(d[i], shift, interval, e);
  exp_d[i] = e;
}

__global__ void k_raw2alpha_bwd(const float* __restrict__ e, const float* __restrict__ g,
                                int64_t n, float interval, float* out) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  out[i] = raw2alpha_grad(e[i], interval, g[i]);
}

// __set_i_for_segment_start_end (:607-617) plus the zero/one initialisation of
// alpha2weight_cuda (:624-628).
__global__ void k_a2w_init(const int64_t* __restrict__ ray_id, int64_t n, int n_rays, float* w,
                           float* T, float* last, int64_t* i_start, int64_t* i_end) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i < n) {
    w[i] = 0.f;
    T[i] = 1.f;
  }
  if (i < n_rays) {
    last[i] = 1.f;
    i_start[i] = 0;
    i_end[i] = 0;
  }
}
__global__ void k_a2w_bounds(const int64_t* __restrict__ ray_id, int64_t n, int64_t* i_start,
                             int64_t* i_end) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i > 0 && i < n && ray_id[i] != ray_id[i - 1]) {
    i_start[ray_id[i]] = i;
    i_end[ray_id[i - 1]] = i;
  }
  if (i == 0 && n > 0) i_end[ray_id[n - 1]] = n;
}

__global__ void k_a2w(const float* __restrict__ alpha, int n_rays, float* w, float* T,
                      float* last, const int64_t* __restrict__ i_start, int64_t* i_end) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rays) return;
  const int64_t is = i_start[r], ie = i_end[r];
  float Tc = 1.f;
  int64_t i;
  for (i = is; i < ie; ++i) {
    T[i] = Tc;
    w[i] = Tc * alpha[i];
    Tc = trans_step(Tc, alpha[i]);
    // Tc < 1e-3 (a double literal): no float lies in [1e-3, 1e-3f), so the
    // FP32 compare against 1e-3f is the same test
    if (Tc < 1e-3f) {
      ++i;
      break;
    }
  }
  i_end[r] = i;
  last[r] = Tc;
}

__global__ void k_a2w_bwd(const float* __restrict__ alpha, const float* __restrict__ w,
                          const float* __restrict__ T, const float* __restrict__ last,
                          const int64_t* __restrict__ i_start, const int64_t* __restrict__ i_end,
                          int n_rays, const float* __restrict__ gw, const float* __restrict__ gl,
                          float* grad) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rays) return;
  const int64_t is = i_start[r], ie = i_end[r];
  float back = gl[r] * last[r];
  for (int64_t i = ie - 1; i >= is; --i) {
    grad[i] = alpha_grad(gw[i], T[i], back, alpha[i]);
    back += gw[i] * w[i];
  }
}

__global__ void k_zero_f(float* p, int64_t n) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i < n) p[i] = 0.f;
}

struct Box {
  float mn[3], mx[3];
};

__global__ void k_ray_count(const float* __restrict__ ro, const float* __restrict__ rd, int n_rays,
                            Box b, float near_, float far_, float stepdist, float* tmin,
                            float* tmax, int64_t* nsteps) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rays) return;
  const float o[3] = {ro[r * 3], ro[r * 3 + 1], ro[r * 3 + 2]};
  const float d[3] = {rd[r * 3], rd[r * 3 + 1], rd[r * 3 + 2]};
  RaySetup s;
  ray_setup(o, d, b.mn, b.mx, near_, far_, stepdist, s);
  tmin[r] = s.t_min;
  tmax[r] = s.t_max;
  nsteps[r] = s.n_steps;
}

// One thread per ray writes its samples (the reference spreads them over
// threads with ray_id/step_id arrays; the values are identical).
__global__ void k_ray_points(const float* __restrict__ ro, const float* __restrict__ rd,
                             int n_rays, Box b, float stepdist, const float* __restrict__ tmin,
                             const int64_t* __restrict__ cum, float* pts, uint8_t* outbbox,
                             int64_t* ray_id, int64_t* step_id) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rays) return;
  const float o[3] = {ro[r * 3], ro[r * 3 + 1], ro[r * 3 + 2]};
  const float d[3] = {rd[r * 3], rd[r * 3 + 1], rd[r * 3 + 2]};
  RaySetup s;
  s.t_min = tmin[r];
  const float rn = ray_norm(d[0], d[1], d[2]);
  for (int a = 0; a < 3; ++a) {
    s.start[a] = __fmaf_rn(d[a], s.t_min, o[a]);
    s.dir[a] = __fdiv_rn(d[a], rn);
  }
  const int64_t beg = r ? cum[r - 1] : 0, end = cum[r];
  for (int64_t i = beg; i < end; ++i) {
    float p[3];
    ray_point(s, stepdist, i - beg, p);
    pts[i * 3] = p[0];
    pts[i * 3 + 1] = p[1];
    pts[i * 3 + 2] = p[2];
    outbbox[i] = out_of_bbox(p, b.mn, b.mx);
    ray_id[i] = r;
    step_id[i] = i - beg;
  }
}

struct MaskArgs {
  int shape[3];
  float scale[3], shift[3];
};

__global__ void k_maskcache(const uint8_t* __restrict__ world, MaskArgs a,
                            const float* __restrict__ xyz, int64_t n, uint8_t* out) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const float p[3] = {xyz[i * 3], xyz[i * 3 + 1], xyz[i * 3 + 2]};
  out[i] = mask_lookup(world, a.shape, p, a.scale, a.shift) ? 1 : 0;
}

}  // namespace pvdb

using namespace pvdb;

extern "C" {

int pvdb_raw2alpha(const float* density, int64_t n, float shift, float interval, float* exp_d,
                   float* alpha, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(n >= 0, "negative size");
  if (!n) return PVDB_OK;
  PVDB_REQUIRE(density && exp_d && alpha, "null argument");
  k_raw2alpha<<<ceil_div(n, 256), 256, 0, as_stream(s)>>>(density, n, shift, interval, exp_d,
                                                          alpha);
  PVDB_CHECK_LAUNCH("k_raw2alpha");
  return PVDB_OK;
}

int pvdb_raw2alpha_backward(const float* exp_d, const float* grad_back, int64_t n, float interval,
                            float* grad, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(n >= 0, "negative size");
  if (!n) return PVDB_OK;
  PVDB_REQUIRE(exp_d && grad_back && grad, "null argument");
  k_raw2alpha_bwd<<<ceil_div(n, 256), 256, 0, as_stream(s)>>>(exp_d, grad_back, n, interval, grad);
  PVDB_CHECK_LAUNCH("k_raw2alpha_bwd");
  return PVDB_OK;
}

int pvdb_alpha2weight(const float* alpha, const int64_t* ray_id, int64_t n, int32_t n_rays,
                      float* weight, float* T, float* alphainv_last, int64_t* i_start,
                      int64_t* i_end, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(n >= 0 && n_rays >= 0, "negative size");
  PVDB_REQUIRE(weight && T && alphainv_last && i_start && i_end, "null argument");
  PVDB_REQUIRE(n == 0 || (alpha && ray_id), "null argument");
  cudaStream_t st = as_stream(s);
  const int64_t m = std::max<int64_t>(n, n_rays);
  if (m) k_a2w_init<<<ceil_div(m, 256), 256, 0, st>>>(ray_id, n, n_rays, weight, T, alphainv_last,
                                                     i_start, i_end);
  PVDB_CHECK_LAUNCH("k_a2w_init");
  if (!n) return PVDB_OK;
  k_a2w_bounds<<<ceil_div(n, 256), 256, 0, st>>>(ray_id, n, i_start, i_end);
  PVDB_CHECK_LAUNCH("k_a2w_bounds");
  if (n_rays)
    k_a2w<<<ceil_div(n_rays, 256), 256, 0, st>>>(alpha, n_rays, weight, T, alphainv_last, i_start,
                                                 i_end);
  PVDB_CHECK_LAUNCH("k_a2w");
  return PVDB_OK;
}

int pvdb_alpha2weight_backward(const float* alpha, const float* weight, const float* T,
                               const float* alphainv_last, const int64_t* i_start,
                               const int64_t* i_end, int32_t n_rays, const float* grad_weights,
                               const float* grad_last, int64_t n, float* grad, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(n >= 0 && n_rays >= 0, "negative size");
  if (n) PVDB_REQUIRE(grad, "null argument");
  cudaStream_t st = as_stream(s);
  if (n) k_zero_f<<<ceil_div(n, 256), 256, 0, st>>>(grad, n);
  PVDB_CHECK_LAUNCH("k_zero_f");
  if (!n_rays || !n) return PVDB_OK;
  PVDB_REQUIRE(alpha && weight && T && alphainv_last && i_start && i_end && grad_weights &&
                   grad_last,
               "null argument");
  k_a2w_bwd<<<ceil_div(n_rays, 256), 256, 0, st>>>(alpha, weight, T, alphainv_last, i_start, i_end,
                                                   n_rays, grad_weights, grad_last, grad);
  PVDB_CHECK_LAUNCH("k_a2w_bwd");
  return PVDB_OK;
}

int pvdb_ray_count_samples(const float* rays_o, const float* rays_d, int32_t n_rays,
                           const float xyz_min[3], const float xyz_max[3], float near_,
                           float far_, float stepdist, float* t_min, float* t_max,
                           int64_t* n_steps, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(n_rays >= 0, "negative size");
  if (!n_rays) return PVDB_OK;
  PVDB_REQUIRE(rays_o && rays_d && xyz_min && xyz_max && t_min && t_max && n_steps,
               "null argument");
  PVDB_REQUIRE(stepdist > 0.f, "stepdist must be positive");
  Box b;
  for (int a = 0; a < 3; ++a) {
    b.mn[a] = xyz_min[a];
    b.mx[a] = xyz_max[a];
  }
  k_ray_count<<<ceil_div(n_rays, 256), 256, 0, as_stream(s)>>>(rays_o, rays_d, n_rays, b, near_,
                                                               far_, stepdist, t_min, t_max,
                                                               n_steps);
  PVDB_CHECK_LAUNCH("k_ray_count");
  return PVDB_OK;
}

int pvdb_ray_sample_points(const float* rays_o, const float* rays_d, int32_t n_rays,
                           const float xyz_min[3], const float xyz_max[3], float stepdist,
                           const float* t_min, const int64_t* n_steps_cumsum, int64_t total,
                           float* rays_pts, uint8_t* mask_outbbox, int64_t* ray_id,
                           int64_t* step_id, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(n_rays >= 0 && total >= 0, "negative size");
  if (!n_rays || !total) return PVDB_OK;
  PVDB_REQUIRE(rays_o && rays_d && xyz_min && xyz_max && t_min && n_steps_cumsum && rays_pts &&
                   mask_outbbox && ray_id && step_id,
               "null argument");
  Box b;
  for (int a = 0; a < 3; ++a) {
    b.mn[a] = xyz_min[a];
    b.mx[a] = xyz_max[a];
  }
  k_ray_points<<<ceil_div(n_rays, 128), 128, 0, as_stream(s)>>>(
      rays_o, rays_d, n_rays, b, stepdist, t_min, n_steps_cumsum, rays_pts, mask_outbbox, ray_id,
      step_id);
  PVDB_CHECK_LAUNCH("k_ray_points");
  return PVDB_OK;
}

int pvdb_maskcache_lookup(const uint8_t* world, const int32_t shape[3], const float* xyz,
                          int64_t n, const float scale[3], const float shift[3], uint8_t* out,
                          pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(n >= 0, "negative size");
  if (!n) return PVDB_OK;
  PVDB_REQUIRE(world && shape && xyz && scale && shift && out, "null argument");
  MaskArgs a;
  for (int q = 0; q < 3; ++q) {
    a.shape[q] = shape[q];
    a.scale[q] = scale[q];
    a.shift[q] = shift[q];
  }
  k_maskcache<<<ceil_div(n, 256), 256, 0, as_stream(s)>>>(world, a, xyz, n, out);
  PVDB_CHECK_LAUNCH("k_maskcache");
  return PVDB_OK;
}

}  // extern "C"
