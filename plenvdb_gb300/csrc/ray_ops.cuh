// Per-ray and per-sample arithmetic shared by the standalone DVGO primitives
// and the fused march, written to reproduce the reference's float/double
// promotions (lib/cuda/render_utils_kernel.cu). Multiply-adds that nvcc
// contracts in the reference build are written as explicit fmaf; every other
// product and sum is rounded separately.
#pragma once
#include "pvdb_internal.cuh"

namespace pvdb {

struct RaySetup {
  float t_min, t_max;
  float start[3];  // rays_o + rays_d * t_min
  float dir[3];    // rays_d / |rays_d|
  int64_t n_steps;
};

// |d| as sqrt(fma(dz,dz,fma(dx,dx,dy*dy))) (infer_n_samples_cuda_kernel :47-50):
// nvcc contracts `dx*dx + dy*dy + dz*dz` by fusing the left product of the
// first sum and the right product of the second, which the golden vectors of
// the reference's own kernel show bit for bit.
__device__ __forceinline__ float ray_norm(float dx, float dy, float dz) {
  return sqrtf(__fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy))));
}

// torch's CPU vector norm of a float[3] (rays_d.norm(dim=-1) in the Python
// steps around the path, dvgo.py:524, :236): sqrt(fma(z,z,fma(y,y,x*x))).
__device__ __forceinline__ float torch_norm3(float x, float y, float z) {
  return sqrtf(__fmaf_rn(z, z, __fmaf_rn(y, y, __fmul_rn(x, x))));
}

// infer_t_minmax_cuda_kernel (:12-35): slab test, clamped to [near, far].
__device__ __forceinline__ void ray_tminmax(const float o[3], const float d[3], const float mn[3],
                                            const float mx[3], float near_, float far_,
                                            float& t_min, float& t_max) {
  const float vx = d[0] == 0.f ? float(1e-6) : d[0];
  const float vy = d[1] == 0.f ? float(1e-6) : d[1];
  const float vz = d[2] == 0.f ? float(1e-6) : d[2];
  const float ax = __fdiv_rn(mx[0] - o[0], vx), ay = __fdiv_rn(mx[1] - o[1], vy),
              az = __fdiv_rn(mx[2] - o[2], vz);
  const float bx = __fdiv_rn(mn[0] - o[0], vx), by = __fdiv_rn(mn[1] - o[1], vy),
              bz = __fdiv_rn(mn[2] - o[2], vz);
  t_min = fmaxf(fminf(fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fminf(az, bz)), far_), near_);
  t_max = fmaxf(fminf(fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fmaxf(az, bz)), far_), near_);
}

__device__ __forceinline__ void ray_setup(const float o[3], const float d[3], const float mn[3],
                                          const float mx[3], float near_, float far_,
                                          float stepdist, RaySetup& r) {
  ray_tminmax(o, d, mn, mx, near_, far_, r.t_min, r.t_max);
  const float rn = ray_norm(d[0], d[1], d[2]);
  // n_samples = max(ceil((t_max-t_min)*|d|/stepdist), 1.)  (:52)
  const float q = __fdiv_rn(__fmul_rn(r.t_max - r.t_min, rn), stepdist);
  r.n_steps = (int64_t)fmaxf(ceilf(q), 1.f);
  for (int a = 0; a < 3; ++a) {
    r.start[a] = __fmaf_rn(d[a], r.t_min, o[a]);  // (:71-73)
    r.dir[a] = __fdiv_rn(d[a], rn);               // (:74-76)
  }
}

// Sample k of a ray (sample_pts_on_rays_cuda_kernel :164-170).
__device__ __forceinline__ void ray_point(const RaySetup& r, float stepdist, int64_t k,
                                          float p[3]) {
  const float dist = __fmul_rn(stepdist, (float)k);
  for (int a = 0; a < 3; ++a) p[a] = __fmaf_rn(r.dir[a], dist, r.start[a]);
}

__device__ __forceinline__ bool out_of_bbox(const float p[3], const float mn[3], const float mx[3]) {
  return (mn[0] > p[0]) | (mn[1] > p[1]) | (mn[2] > p[2]) | (mx[0] < p[0]) | (mx[1] < p[1]) |
         (mx[2] < p[2]);
}

// VDBGrid.wld2idx (grid.py:77-78): (p - min) / (max - min) * (ws - 1), each op
// rounded (three torch kernels).
__device__ __forceinline__ void world_to_index(const float p[3], const float mn[3],
                                               const float ext[3], const float wsm1[3],
                                               float idx[3]) {
  for (int a = 0; a < 3; ++a) idx[a] = __fmul_rn(__fdiv_rn(p[a] - mn[a], ext[a]), wsm1[a]);
}

// maskcache_lookup_cuda_kernel (:380-394).
__device__ __forceinline__ bool mask_lookup(const uint8_t* world, const int shape[3],
                                            const float p[3], const float scale[3],
                                            const float shift[3]) {
  const int i = (int)roundf(__fmaf_rn(p[0], scale[0], shift[0]));
  const int j = (int)roundf(__fmaf_rn(p[1], scale[1], shift[1]));
  const int k = (int)roundf(__fmaf_rn(p[2], scale[2], shift[2]));
  if (0 <= i && i < shape[0] && 0 <= j && j < shape[1] && 0 <= k && k < shape[2])
    return world[(int64_t(i) * shape[1] + j) * shape[2] + k] != 0;
  return false;
}

// raw2alpha (:439-441).
__device__ __forceinline__ float raw2alpha(float sigma, float shift, float interval, float& e) {
  e = expf(sigma + shift);
  return 1.f - powf(1.f + e, -interval);
}

// raw2alpha_backward (:514): min(e,1e10) * (1+e)^(-interval-1) * interval * g.
// The reference forms the product in double (min() of a double literal); here
// it is three FP32 products, within a few ulps of that.
__device__ __forceinline__ float raw2alpha_grad(float e, float interval, float g) {
  return __fmul_rn(__fmul_rn(__fmul_rn(fminf(e, 1e10f), powf(1.f + e, -interval - 1.f)), interval), g);
}

// T_cum *= (1. - alpha) (:593). The reference promotes to double because of
// the literal: it rounds the exact product T*(1-alpha) to double, then to
// float. One fmaf rounds the same exact product T - T*alpha straight to
// float; the two agree except when the double rounding lands on a float tie
// (about one step in 2^29), and no FP64 unit is used.
__device__ __forceinline__ float trans_step(float T, float alpha) {
  return __fmaf_rn(-T, alpha, T);
}

// grad = gw*T - back_cum / (1-alpha + 1e-10) (:671), in FP32 (the reference
// adds the double literal and divides in double).
__device__ __forceinline__ float alpha_grad(float gw, float T, float back_cum, float alpha) {
  return __fmul_rn(gw, T) - __fdiv_rn(back_cum, (1.f - alpha) + 1e-10f);
}

}  // namespace pvdb
