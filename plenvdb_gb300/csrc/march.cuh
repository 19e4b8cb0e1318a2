// Fused training march: workspace layout shared by march.cu, mlp.cu and
// train.cu.
#pragma once
#include "pvdb_internal.cuh"
#include "ray_ops.cuh"

namespace pvdb {

// Per-launch constants of the march (device copy of pvdb_march_params plus
// derived values).
struct MarchP {
  float mn[3], mx[3];
  float ext[3];   // xyz_max - xyz_min (float, as torch computes it)
  float wsm1[3];  // world_size - 1 (as float)
  float near_, far_, stepdist, shift, interval, thr, t_stop, bg;
  const uint8_t* mask;
  int mshape[3];
  float mscale[3], mshift[3];
  int cap;
  // empty-space skipping: a sample whose brick bound is below sigma_skip has
  // alpha <= thr for certain (raw2alpha is increasing in sigma)
  float sigma_skip;
  float binv[3];  // approximate world -> brick scale: wsm1 / ext / 4
};

// Device pointers of the workspace, passed by value to kernels.
struct MarchW {
  // per ray
  float* ray_sd;  // [R*6] sample origin (rays_o + rays_d*t_min) and unit direction
  int32_t* ray_ns;  // [R] samples in the bbox (clamped to cap)
  uint64_t* chain_status;  // [R] k_march_chain ray counts / prefixes
  float* T_last;
  uint32_t* n_kept;
  uint32_t* n_color;
  uint32_t* kept_off;
  uint32_t* color_off;
  // per (ray, kept slot): index r*cap + i
  float* k_alpha;
  float* k_w;
  int32_t* k_step;  // sample index along the ray; bit 31 set for colour samples
  int32_t* k_row;   // colour row of the sample, -1 otherwise
  // per colour row
  float* r_k0;
  float* r_w;
  float* r_alpha;
  int32_t* r_ray;
  int32_t* r_step;
  // per kept sample (global kept index), backward: (x, y, z, dL/dsigma) and
  // the sample's colour row (-1: none), whose k0 gradient is read from the
  // rgbnet backward's output
  float4* b_rec;
  int32_t* b_row;
  // [0] total kept, [1] total colour rows, [2] block claimed by the
  // leaf-staging test hook, [3] error flags (1 samples_cap exceeded,
  // 2 tensor-core wait, 4 ray-offset look-back wait, 8 leaf-staging copy
  // wait), [4] samples evaluated, [5] samples grouped by cell (backward),
  // [6] k_march_chain ray counter, [7] unused,
  // [8..11] voxels visited / updated by the density and k0 Adam of the last
  // profiled train step
  uint32_t* totals;
};

}  // namespace pvdb

struct pvdb_march_s {
  int max_rays = 0;
  int cap = 0;
  int64_t slots = 0;  // max_rays * cap
  int k0_channels = 0;
  pvdb::MarchW w{};
  pvdb::ReduceScratch red;   // kept samples grouped by cell key
  // per cell of the leaf lattice (dense leaf-major keys): sample count (zero
  // between calls) and first grouped index; per dense leaf: count and start
  uint32_t* cell_cnt = nullptr;
  uint32_t* cell_off = nullptr;
  uint32_t* leaf_cnt = nullptr;
  uint32_t* leaf_off = nullptr;
  size_t cell_cap = 0;  // cells
  size_t b_rec_cap = 0;         // bytes of w.b_rec
  // grouped (cell, sample) order records: w.b_rec, followed (backward with
  // k0) by the sample's k0-row gradient, 1 + ceil(C/4) float4 per sample
  float4* b_rec_s = nullptr;
  size_t b_rec_s_cap = 0;
  size_t b_row_cap = 0;         // bytes of w.b_row
  bool bwd_keys_ready = false;  // march_backward_keys ran since the last reduce
  bool bwd_with_k0 = false;
  uint32_t* scan_partial = nullptr;
  size_t scan_partial_cap = 0;
  // state of the last forward
  pvdb::MarchP p{};
  int n_rays = 0;
  bool has_fwd = false;
  bool prof = false;  // record stage-profiler marks (set by the train step)
  int leaf_staging = 0;  // density leaves staged in shared memory (pvdb_march_set_leaf_staging)
  pvdb_grid_s* density = nullptr;
  pvdb_grid_s* k0 = nullptr;
  // rgbnet scratch (mlp.cu)
  float* hpe = nullptr;          // [max_rays, width] per-ray layer-0 PE part + bias
  size_t hpe_cap = 0;
  float* wpart = nullptr;        // per-CTA partial weight gradients
  size_t wpart_cap = 0;
  void* mlp_packed = nullptr;    // packed BF16 weights for the tensor-core path
  size_t mlp_packed_cap = 0;
  void* mlp_xt = nullptr;        // BF16 X tiles of the rows (tensor-core path)
  size_t mlp_xt_cap = 0;
  // train-step scratch (train.cu)
  float* t_rgb = nullptr;        // [M_max,3]
  float* t_grad_rgb = nullptr;   // [M_max,3]
  float* t_grad_w = nullptr;     // [M_max]
  float* t_grad_k0 = nullptr;    // [M_max, C]
  float* t_grad_last = nullptr;  // [max_rays]
  float* t_loss_part = nullptr;  // [max_rays]
  float* t_rgb_marched = nullptr;  // [max_rays,3]
  size_t t_cap_rows = 0;
  // CUDA graph of the fused train step (train.cu)
  cudaGraph_t g_graph = nullptr;
  cudaGraphExec_t g_exec = nullptr;
  cudaStream_t g_stream = nullptr;  // capture stream
  float* g_in = nullptr;            // staged rays_o, rays_d, viewdirs, target [4][R][3]
  size_t g_in_cap = 0;
  float* g_scal = nullptr;          // [0..2] Adam step sizes, [4] loss
  std::vector<uint8_t> g_key;       // what the graph was captured for
  std::vector<uint8_t> g_pending;   // key of the last eager step (capture on a repeat)
  cudaStream_t side[2] = {nullptr, nullptr};  // side streams of the train step
  cudaEvent_t side_ev[3] = {nullptr, nullptr, nullptr};
  uint64_t g_launches = 0;          // library launches per replay
};
