// Training-ray generation (lib/dvgo.py:471-635): the pinhole rays of a view
// with the reference's pixel grid, flips, inverse_y and optional NDC warp
// (get_rays / ndc_rays / get_rays_of_a_view), and hit_coarse_geo (does any
// sample of a ray land in an occupied mask-cache voxel), which
// get_training_rays_in_maskcache_sampling uses to keep only the rays that can
// see the scene. One thread per pixel / ray.
#include "ray_ops.cuh"

namespace pvdb {

struct GetRaysArgs {
  int H, W;
  float fx, fy, cx, cy;
  float R[9];   // c2w[:3,:3], row-major
  float t[3];   // c2w[:3,3]
  int inverse_y, flip_x, flip_y;
  int mode;     // 0 'center' (+0.5), 1 'lefttop', 2 'random' (+ jitter)
  const float* jitter;  // mode 2: [2][H*W] uniform offsets of i then j
  int ndc;
  float ndc_near;       // 1.0 in get_rays_of_a_view
  float ndc_ax, ndc_ay; // -1/(W/(2f)), -1/(H/(2f)), formed in double
};

__global__ void k_get_rays(GetRaysArgs a, float* rays_o, float* rays_d, float* viewdirs) {
  const int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= int64_t(a.H) * a.W) return;
  const int h = int(p / a.W), w = int(p - int64_t(h) * a.W);
  // meshgrid of linspace(0, W-1) x linspace(0, H-1) (exact integers), the
  // offset, then flip((1,)) / flip((0,)) of the offset grids
  const int wc = a.flip_x ? a.W - 1 - w : w;
  const int hr = a.flip_y ? a.H - 1 - h : h;
  float fi = float(wc), fj = float(hr);
  if (a.mode == 0) {
    fi = __fadd_rn(fi, 0.5f);
    fj = __fadd_rn(fj, 0.5f);
  } else if (a.mode == 2) {
    const int64_t n = int64_t(a.H) * a.W;
    fi = __fadd_rn(fi, __ldg(a.jitter + int64_t(h) * a.W + wc));
    fj = __fadd_rn(fj, __ldg(a.jitter + n + int64_t(hr) * a.W + w));
  }
  float dir[3];
  dir[0] = __fdiv_rn(fi - a.cx, a.fx);
  if (a.inverse_y) {
    dir[1] = __fdiv_rn(fj - a.cy, a.fy);
    dir[2] = 1.f;
  } else {
    dir[1] = -__fdiv_rn(fj - a.cy, a.fy);
    dir[2] = -1.f;
  }
  // sum(dirs[..., None, :] * c2w[:3,:3], -1)
  float d[3];
#pragma unroll
  for (int k = 0; k < 3; ++k)
    d[k] = __fadd_rn(__fadd_rn(__fmul_rn(dir[0], a.R[3 * k]), __fmul_rn(dir[1], a.R[3 * k + 1])),
                     __fmul_rn(dir[2], a.R[3 * k + 2]));
  // rays_d.norm(dim=-1): torch's CPU vector norm is sqrt(fma(z,z,fma(y,y,x*x)))
  const float nrm = torch_norm3(d[0], d[1], d[2]);
#pragma unroll
  for (int k = 0; k < 3; ++k) viewdirs[3 * p + k] = __fdiv_rn(d[k], nrm);
  float o[3] = {a.t[0], a.t[1], a.t[2]};
  if (a.ndc) {
    // ndc_rays (lib/dvgo.py:496-514)
    const float t = __fdiv_rn(-__fadd_rn(a.ndc_near, o[2]), d[2]);
#pragma unroll
    for (int k = 0; k < 3; ++k) o[k] = __fadd_rn(o[k], __fmul_rn(t, d[k]));
    const float qx = __fdiv_rn(o[0], o[2]), qy = __fdiv_rn(o[1], o[2]);
    const float o0 = __fdiv_rn(__fmul_rn(a.ndc_ax, o[0]), o[2]);
    const float o1 = __fdiv_rn(__fmul_rn(a.ndc_ay, o[1]), o[2]);
    const float o2 = __fadd_rn(1.f, __fdiv_rn(2.f * a.ndc_near, o[2]));
    const float d0 = __fmul_rn(a.ndc_ax, __fsub_rn(__fdiv_rn(d[0], d[2]), qx));
    const float d1 = __fmul_rn(a.ndc_ay, __fsub_rn(__fdiv_rn(d[1], d[2]), qy));
    const float d2 = __fdiv_rn(-2.f * a.ndc_near, o[2]);
    o[0] = o0;
    o[1] = o1;
    o[2] = o2;
    d[0] = d0;
    d[1] = d1;
    d[2] = d2;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    rays_o[3 * p + k] = o[k];
    rays_d[3 * p + k] = d[k];
  }
}

struct HitArgs {
  float mn[3], mx[3];
  float near_, stepdist;
  const uint8_t* mask;
  int shape[3];
  float scale[3], shift[3];
};

// hit_coarse_geo (lib/dvgo.py:258-270): the samples of sample_pts_on_rays
// (far = 1e9), in-bbox ones looked up in the mask cache.
__global__ void k_rays_hit(const float* __restrict__ ro, const float* __restrict__ rd, int64_t n,
                           HitArgs a, uint8_t* hit) {
  const int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (r >= n) return;
  const float o[3] = {ro[3 * r], ro[3 * r + 1], ro[3 * r + 2]};
  const float d[3] = {rd[3 * r], rd[3 * r + 1], rd[3 * r + 2]};
  RaySetup s;
  ray_setup(o, d, a.mn, a.mx, a.near_, 1e9f, a.stepdist, s);
  uint8_t h = 0;
  for (int64_t k = 0; k < s.n_steps; ++k) {
    float p[3];
    ray_point(s, a.stepdist, k, p);
    if (!out_of_bbox(p, a.mn, a.mx) && mask_lookup(a.mask, a.shape, p, a.scale, a.shift)) {
      h = 1;
      break;
    }
  }
  hit[r] = h;
}

}  // namespace pvdb

using namespace pvdb;

extern "C" {

int pvdb_get_rays(int32_t H, int32_t W, const double K[9], const float c2w[16], int32_t ndc,
                  int32_t inverse_y, int32_t flip_x, int32_t flip_y, int32_t mode,
                  const float* jitter, float* rays_o, float* rays_d, float* viewdirs,
                  pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(H >= 0 && W >= 0, "negative image size");
  PVDB_REQUIRE(K && c2w, "null K or c2w");
  PVDB_REQUIRE(mode >= 0 && mode <= 2, "mode must be 0 (center), 1 (lefttop) or 2 (random)");
  PVDB_REQUIRE(mode != 2 || jitter, "random mode needs the jitter array");
  const int64_t n = int64_t(H) * W;
  if (!n) return PVDB_OK;
  PVDB_REQUIRE(rays_o && rays_d && viewdirs, "null output");
  GetRaysArgs a;
  a.H = H;
  a.W = W;
  a.fx = float(K[0]);
  a.cx = float(K[2]);
  a.fy = float(K[4]);
  a.cy = float(K[5]);
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) a.R[3 * r + c] = c2w[4 * r + c];
    a.t[r] = c2w[4 * r + 3];
  }
  a.inverse_y = inverse_y != 0;
  a.flip_x = flip_x != 0;
  a.flip_y = flip_y != 0;
  a.mode = mode;
  a.jitter = jitter;
  a.ndc = ndc != 0;
  a.ndc_near = 1.f;
  // -1./(W/(2.*focal)) in double, focal = K[0][0] (lib/dvgo.py:502-509)
  a.ndc_ax = float(-1.0 / (double(W) / (2.0 * K[0])));
  a.ndc_ay = float(-1.0 / (double(H) / (2.0 * K[0])));
  k_get_rays<<<ceil_div(n, 256), 256, 0, as_stream(s)>>>(a, rays_o, rays_d, viewdirs);
  PVDB_CHECK_LAUNCH("k_get_rays");
  return PVDB_OK;
}

int pvdb_rays_hit_mask(const float* rays_o, const float* rays_d, int64_t n,
                       const float xyz_min[3], const float xyz_max[3], float near_,
                       float stepdist, const uint8_t* mask, const int32_t shape[3], uint8_t* hit,
                       pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(n >= 0, "negative size");
  if (!n) return PVDB_OK;
  PVDB_REQUIRE(rays_o && rays_d && xyz_min && xyz_max && mask && shape && hit, "null argument");
  PVDB_REQUIRE(stepdist > 0.f, "stepdist must be positive");
  HitArgs a;
  for (int q = 0; q < 3; ++q) {
    PVDB_REQUIRE(shape[q] > 0, "empty mask shape");
    a.mn[q] = xyz_min[q];
    a.mx[q] = xyz_max[q];
    a.shape[q] = shape[q];
    // MaskGrid buffers (lib/grid.py:230-232)
    a.scale[q] = float(shape[q] - 1) / (xyz_max[q] - xyz_min[q]);
    a.shift[q] = -xyz_min[q] * a.scale[q];
  }
  a.near_ = near_;
  a.stepdist = stepdist;
  a.mask = mask;
  k_rays_hit<<<ceil_div(n, 128), 128, 0, as_stream(s)>>>(rays_o, rays_d, n, a, hit);
  PVDB_CHECK_LAUNCH("k_rays_hit");
  return PVDB_OK;
}

}  // extern "C"
