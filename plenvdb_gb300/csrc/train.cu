// One fine-stage training iteration on device-resident rays (run.py:516-598):
// march forward, rgbnet, composite, the reference losses (run.py:551-575),
// the full backward, TV on both grids (run.py:578-584), voxel Adam (mode 1,
// configs/default.py:76) on both grids, dense Adam on the rgbnet
// (masked_adam.py:128-158, mode 0) and the lr decay (run.py:592-598).
// Nothing synchronises with the host.
#include <cmath>

#include "march.cuh"

struct pvdb_opt_s;

namespace pvdb {

struct MlpArgs {
  const float* w0; const float* b0;
  const float* w1; const float* b1;
  const float* w2; const float* b2;
  int c0, dpe, din;
};
int mlp_prepare(pvdb_march_s* m, const MlpArgs& a, const float* viewdirs, int R, int precision,
                cudaStream_t st);
int mlp_forward_impl(pvdb_march_s* m, const MlpArgs& a, const float* k0rows,
                     const float* viewdirs, float* rgb, int precision, cudaStream_t st,
                     bool prepared, bool x_ready);
int mlp_backward_impl(pvdb_march_s* m, const MlpArgs& a, const float* k0rows, const float* rgb,
                      const float* grad_rgb, float* grad_k0, float* grad_flat, int precision,
                      cudaStream_t st, bool prepared);
int march_forward_impl(pvdb_march_s* m, pvdb_grid_s* density, pvdb_grid_s* k0, const float* ro,
                       const float* rd, int R, const pvdb_march_params* prm, const uint8_t* mask,
                       const int32_t* mshape, cudaStream_t st, bool skip_k0);
int march_k0_x(pvdb_march_s* m, const float* pe, int pe_stride, int dpe, uint8_t* xt,
               cudaStream_t st, const __nv_bfloat16* half);
const float* mlp_pe_buffer(pvdb_march_s* m, int* stride);
int mlp_reserve_x(pvdb_march_s* m);
int march_backward_keys(pvdb_march_s* m, const float* grad_w, const float* grad_last,
                        bool with_k0, cudaStream_t st);
int march_backward_reduce(pvdb_march_s* m, const float* grad_k0, cudaStream_t st, bool clear);
int march_backward_clear(pvdb_march_s* m, cudaStream_t st);
float opt_next_stepsz(pvdb_opt_s* o);
int opt_launch(pvdb_opt_s* o, int mode, int zero_after, float stepsz, const float* stepsz_dev,
               cudaStream_t st, const float* tv, uint32_t* counts);
pvdb_grid_s* opt_params(pvdb_opt_s* o);
pvdb_grid_s* opt_moment(pvdb_opt_s* o, int which);
float opt_lr_scale(pvdb_opt_s* o, float factor);

struct LossW {
  float main, ent, rgbper, bg;
};

// Per ray (warp per ray): the composite rgb_marched = sum_rows w*rgb + T*bg
// (the same arithmetic as k_composite_fwd), the losses and their gradients
// w.r.t. rgb_marched (folded into the per-row colour gradient), alphainv_last
// and the colour weights; each ray's loss partial (k_loss_sum adds them).
__global__ void __launch_bounds__(256)
    k_loss(MarchW W, const float* __restrict__ rgb, float* rgbm_out,
           const float* __restrict__ target, int R, LossW L, float* grad_rgb, float* grad_w,
           float* grad_last, float* loss_part) {
  grid_dep_sync();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * 8 + warp;
  if (r < R) {
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
    const float T = W.T_last[r];
    const float tb = __fmul_rn(T, L.bg);
    const float m0 = __fadd_rn(__shfl_sync(0xffffffffu, s0, 0), tb);
    const float m1 = __fadd_rn(__shfl_sync(0xffffffffu, s1, 0), tb);
    const float m2 = __fadd_rn(__shfl_sync(0xffffffffu, s2, 0), tb);
    if (lane == 0) {
      rgbm_out[r * 3] = m0;
      rgbm_out[r * 3 + 1] = m1;
      rgbm_out[r * 3 + 2] = m2;
    }
    const float t0 = target[r * 3], t1 = target[r * 3 + 1], t2 = target[r * 3 + 2];
    const float e0 = m0 - t0, e1 = m1 - t1, e2 = m2 - t2;
    // d/d rgb_marched of weight_main * mean((rgbm-target)^2) over R*3 entries
    const float cm = L.main * 2.f / (3.f * float(R));
    const float g0 = cm * e0, g1 = cm * e1, g2 = cm * e2;
    const float cp = L.rgbper * 2.f / float(R);
    float per = 0.f;
    for (int j = lane; j < n; j += 32) {
      const int64_t m = off + j;
      const float w = W.r_w[m];
      const float y0 = rgb[m * 3], y1 = rgb[m * 3 + 1], y2 = rgb[m * 3 + 2];
      const float d0 = y0 - t0, d1 = y1 - t1, d2 = y2 - t2;
      per += (d0 * d0 + d1 * d1 + d2 * d2) * w;
      grad_rgb[m * 3] = w * g0 + cp * w * d0;
      grad_rgb[m * 3 + 1] = w * g1 + cp * w * d1;
      grad_rgb[m * 3 + 2] = w * g2 + cp * w * d2;
      grad_w[m] = g0 * y0 + g1 * y1 + g2 * y2;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) per += __shfl_xor_sync(0xffffffffu, per, o);
    if (lane == 0) {
      const float p = fminf(fmaxf(T, 1e-6f), 1.f - 1e-6f);
      const float ent = -(p * logf(p) + (1.f - p) * logf(1.f - p));
      const float dent = (T > 1e-6f && T < 1.f - 1e-6f) ? logf((1.f - p) / p) : 0.f;
      grad_last[r] = L.bg * (g0 + g1 + g2) + L.ent / float(R) * dent;
      loss_part[r] = L.main * (e0 * e0 + e1 * e1 + e2 * e2) / (3.f * float(R)) +
                     L.ent * ent / float(R) + L.rgbper * per / float(R);
    }
  }
}

// One block sums the rays' loss partials: thread t sums partials t, t + 256,
// ... in that order (eight loads in flight at a time), then a fixed tree.
// It runs beside the backward (only the step's reported loss needs it).
__global__ void __launch_bounds__(256)
    k_loss_sum(const float* __restrict__ loss_part, int R, float* loss) {
  grid_dep_sync();
  __shared__ float red[256];
  float acc = 0.f;
  for (int i0 = threadIdx.x; i0 < R; i0 += 8 * blockDim.x) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int i = i0 + u * int(blockDim.x);
      v[u] = i < R ? __ldcg(loss_part + i) : 0.f;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (i0 + u * int(blockDim.x) < R) acc += v[u];
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss[0] = red[0];
}

static int train_reserve(pvdb_march_s* m, int C) {
  const size_t rows = size_t(m->slots);
  if (m->t_cap_rows >= rows && m->t_rgb) return PVDB_OK;
  void** ps[] = {(void**)&m->t_rgb, (void**)&m->t_grad_rgb, (void**)&m->t_grad_w,
                 (void**)&m->t_grad_k0, (void**)&m->t_grad_last, (void**)&m->t_loss_part,
                 (void**)&m->t_rgb_marched};
  for (void** p : ps) {
    dev_free(*p);
    *p = nullptr;
  }
  const size_t R = m->max_rays;
  int rc;
  if ((rc = dev_alloc((void**)&m->t_rgb, rows * 12)) ||
      (rc = dev_alloc((void**)&m->t_grad_rgb, rows * 12)) ||
      (rc = dev_alloc((void**)&m->t_grad_w, rows * 4)) ||
      (rc = dev_alloc((void**)&m->t_grad_k0, rows * 4 * size_t(C))) ||
      (rc = dev_alloc((void**)&m->t_grad_last, R * 4)) ||
      (rc = dev_alloc((void**)&m->t_loss_part, R * 4)) ||
      (rc = dev_alloc((void**)&m->t_rgb_marched, R * 12)))
    return rc;
  m->t_cap_rows = rows;
  return PVDB_OK;
}

// Before a graph replay: the step's rays, view directions and targets into the
// fixed input buffer the captured step reads (dst = [rays_o | rays_d |
// viewdirs | target], n3 floats each), and the step sizes it reads; one
// launch for what would be four copies and a scalar write.
__global__ void __launch_bounds__(256)
    k_step_inputs(float* __restrict__ dst, const float* __restrict__ ro,
                  const float* __restrict__ rd, const float* __restrict__ vd,
                  const float* __restrict__ tgt, int64_t n3, float* scal, float ss_d, float ss_k,
                  float ss_n) {
  grid_dep_sync();
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    scal[0] = ss_d;
    scal[1] = ss_k;
    scal[2] = ss_n;
  }
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < 4 * n3;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int q = int(i / n3);
    const int64_t e = i - int64_t(q) * n3;
    const float* src = q == 0 ? ro : q == 1 ? rd : q == 2 ? vd : tgt;
    dst[i] = __ldg(src + e);
  }
}

struct TrainArgs {
  pvdb_march_s* m;
  pvdb_opt_s* dopt;
  pvdb_opt_s* kopt;
  pvdb_rgbnet_state* net;
  const float *ro, *rd, *vd, *tgt;
  int R;
  const pvdb_train_config* cfg;
  float* loss;
  float ss[3];             // Adam step sizes (density, k0, rgbnet)
  const float* ss_dev;     // or read from the device ([0..2]) when captured
  bool prof;
};

// Side streams of the train step: independent branches (the rgbnet inputs
// beside the march, the two grids' TV and Adam, the rgbnet Adam) run
// concurrently. Fork: the side streams wait for st; join: st waits for them.
// Inside a stream capture the same calls make parallel graph branches.
static int side_streams(pvdb_march_s* m) {
  if (m->side[0]) return PVDB_OK;
  for (int i = 0; i < 2; ++i)
    PVDB_CHECK_CUDA(cudaStreamCreateWithFlags(&m->side[i], cudaStreamNonBlocking));
  for (int i = 0; i < 3; ++i)
    PVDB_CHECK_CUDA(cudaEventCreateWithFlags(&m->side_ev[i], cudaEventDisableTiming));
  return PVDB_OK;
}
static int fork_side(pvdb_march_s* m, cudaStream_t st, int n) {
  PVDB_CHECK_CUDA(cudaEventRecord(m->side_ev[0], st));
  for (int i = 0; i < n; ++i) PVDB_CHECK_CUDA(cudaStreamWaitEvent(m->side[i], m->side_ev[0], 0));
  return PVDB_OK;
}
static int join_side(pvdb_march_s* m, cudaStream_t st, int n) {
  for (int i = 0; i < n; ++i) {
    PVDB_CHECK_CUDA(cudaEventRecord(m->side_ev[1 + i], m->side[i]));
    PVDB_CHECK_CUDA(cudaStreamWaitEvent(st, m->side_ev[1 + i], 0));
  }
  return PVDB_OK;
}

// All device work of one train step: launches only, no host state changes
// (so it can be captured into a graph and replayed).
static int train_launches(const TrainArgs& t, cudaStream_t st) {
  pvdb_march_s* m = t.m;
  pvdb_rgbnet_state* net = t.net;
  const pvdb_train_config* cfg = t.cfg;
  pvdb_grid_s* dg = opt_params(t.dopt);
  pvdb_grid_s* kg = opt_params(t.kopt);
  const int n_rays = t.R;
  pvdb_stream s = reinterpret_cast<pvdb_stream>(st);
  // parameters in the flat layout [w0,b0,w1,b1,w2,b2]
  MlpArgs a;
  a.c0 = net->c0;
  a.dpe = 3 + 6 * net->pe;
  a.din = a.c0 + a.dpe;
  const int W = 128;
  a.w0 = net->params;
  a.b0 = a.w0 + W * a.din;
  a.w1 = a.b0 + W;
  a.b1 = a.w1 + W * W;
  a.w2 = a.b1 + W;
  a.b2 = a.w2 + 3 * W;
  const int64_t P = int64_t(W) * a.din + W + W * W + W + 3 * W + 3;

  if (t.prof) {
    prof_begin_call();
    prof_mark(st, 0);
  }
  struct ProfGuard {
    pvdb_march_s* m;
    ~ProfGuard() { m->prof = false; }
  } guard{m};
  m->prof = t.prof;
  int rc = side_streams(m);
  if (rc) return rc;
  // rgbnet inputs (PE, packed weights) beside the march
  if ((rc = fork_side(m, st, 1))) return rc;
  if ((rc = mlp_prepare(m, a, t.vd, n_rays, cfg->precision, m->side[0]))) return rc;
  // BF16: the k0 trilinear writes the rgbnet's X tiles directly (after the
  // join: the tiles hold the PE too)
  const bool fused_x = cfg->precision == 1;
  if (fused_x && (rc = mlp_reserve_x(m))) return rc;
  // BF16: 12-channel features are gathered from the grid's BF16 shadow (the
  // voxel Adam keeps it current; a replayed graph requires it valid)
  const bool use_half = fused_x && kg->C == 12;
  if (use_half && (rc = half_ensure(kg, st))) return rc;
  rc = march_forward_impl(m, dg, kg, t.ro, t.rd, n_rays, &cfg->march, nullptr, nullptr, st,
                          fused_x);
  if (rc) return rc;
  if ((rc = join_side(m, st, 1))) return rc;
  if (fused_x) {
    int pe_stride = 0;
    const float* pe = mlp_pe_buffer(m, &pe_stride);
    rc = march_k0_x(m, pe, pe_stride, a.dpe, static_cast<uint8_t*>(m->mlp_xt), st,
                    use_half ? kg->d_half : nullptr);
    if (rc) return rc;
  }
  rc = mlp_forward_impl(m, a, m->w.r_k0, t.vd, m->t_rgb, cfg->precision, st, true, fused_x);
  if (rc) return rc;
  if (t.prof) prof_mark(st, 3);
  LossW L{cfg->weight_main, cfg->weight_entropy_last, cfg->weight_rgbper, cfg->march.bg};
  launch_k(k_loss, ceil_div(n_rays, 8), 256, 0, st, m->w, m->t_rgb, m->t_rgb_marched, t.tgt, n_rays,
           L, m->t_grad_rgb, m->t_grad_w, m->t_grad_last, m->t_loss_part);
  PVDB_CHECK_LAUNCH("k_loss");
  // the loss sum beside the backward (side[1] is free until the Adam updates)
  cudaStream_t lst = st;
  if (!t.prof) {
    PVDB_CHECK_CUDA(cudaEventRecord(m->side_ev[0], st));
    PVDB_CHECK_CUDA(cudaStreamWaitEvent(m->side[1], m->side_ev[0], 0));
    lst = m->side[1];
  }
  launch_k(k_loss_sum, 1, 256, 0, lst, m->t_loss_part, n_rays, t.loss);
  PVDB_CHECK_LAUNCH("k_loss_sum");
  if (t.prof) prof_mark(st, 4);
  // The march backward's density path and the grouping of the kept samples by
  // cell need only the weight / alphainv_last gradients: they run beside the
  // rgbnet backward, whose k0-row gradients the per-voxel sums then read.
  // (The stage profiler keeps the stages in sequence.)
  const bool par = !t.prof;
  if (par && (rc = fork_side(m, st, 1))) return rc;
  if (par) {
    rc = march_backward_keys(m, m->t_grad_w, m->t_grad_last, true, m->side[0]);
    if (rc) return rc;
  }
  rc = mlp_backward_impl(m, a, m->w.r_k0, m->t_rgb, m->t_grad_rgb, m->t_grad_k0, net->grads,
                         cfg->precision, st, true);
  if (rc) return rc;
  if (t.prof) prof_mark(st, 5);
  if (par) {
    if ((rc = join_side(m, st, 1))) return rc;
  } else {
    rc = march_backward_keys(m, m->t_grad_w, m->t_grad_last, true, st);
    if (rc) return rc;
  }
  // TV (dvgo.py:245-251: w = weight * max(world_size) / 128; run.py:580 divides by len(rays)).
  // Sparse TV adds its terms only to voxels with a nonzero gradient, and the
  // terms depend on the values alone: they are computed beside the gradient
  // sums (for the touched leaves' voxels) and the voxel Adam adds them to the
  // channels with a gradient. Dense TV (every voxel) keeps the in-place pass.
  const int wsmax = std::max(dg->reso[0], std::max(dg->reso[1], dg->reso[2]));
  const float w_k = cfg->tv_weight_k0 / float(n_rays) * float(wsmax) / 128.f;
  const float w_d = cfg->tv_weight_density / float(n_rays) * float(wsmax) / 128.f;
  const bool defer = !cfg->tv_dense_mode && !cfg->tv_in_place;
  const bool defer_k = defer && cfg->tv_weight_k0 > 0.f && !kg->all_touched;
  const bool defer_d = defer && cfg->tv_weight_density > 0.f && !dg->all_touched;
  if (defer_k || defer_d) {
    // the touched leaves (flagged by the grouping) for the terms and for Adam
    if (defer_d && (rc = touched_list(dg, st))) return rc;
    if (defer_k && (rc = touched_list(kg, st))) return rc;
  }
  if (t.prof) {
    // stage profiler: every stage in sequence on the launching stream, with
    // a mark between the per-voxel sums, the TV terms and the Adam updates
    if ((rc = march_backward_reduce(m, m->t_grad_k0, st, true))) return rc;
    if (defer_k && (rc = tv_terms_launch(kg, w_k, w_k, w_k, st))) return rc;
    if (defer_d && (rc = tv_terms_launch(dg, w_d, w_d, w_d, st))) return rc;
    if (cfg->tv_weight_k0 > 0.f && !defer_k &&
        (rc = pvdb_grid_tv_add_grad(kg, w_k, w_k, w_k, cfg->tv_dense_mode, 0, s)))
      return rc;
    if (cfg->tv_weight_density > 0.f && !defer_d &&
        (rc = pvdb_grid_tv_add_grad(dg, w_d, w_d, w_d, cfg->tv_dense_mode, 0, s)))
      return rc;
    prof_mark(st, 9);
    // the Adam updates count the voxels they visit and update (totals[8..11])
    PVDB_CHECK_CUDA(cudaMemsetAsync(m->w.totals + 8, 0, 16, st));
    if ((rc = opt_launch(t.kopt, 1, 1, t.ss[1], t.ss_dev ? t.ss_dev + 1 : nullptr, st,
                         defer_k ? kg->d_tv : nullptr, m->w.totals + 10)) ||
        (rc = opt_launch(t.dopt, 1, 1, t.ss[0], t.ss_dev ? t.ss_dev + 0 : nullptr, st,
                         defer_d ? dg->d_tv : nullptr, m->w.totals + 8)))
      return rc;
    prof_mark(st, 10);
    rc = adam_dense_launch(net->params, net->grads, net->exp_avg, net->exp_avg_sq, nullptr, P,
                           t.ss[2], cfg->rgbnet_beta1, cfg->rgbnet_beta2, cfg->rgbnet_eps, 0, st,
                           t.ss_dev ? t.ss_dev + 2 : nullptr);
    if (rc) return rc;
    prof_mark(st, 11);
    return PVDB_OK;
  }
  if ((defer_k || defer_d) && (rc = fork_side(m, st, 1))) return rc;
  if (defer_k && (rc = tv_terms_launch(kg, w_k, w_k, w_k, m->side[0]))) return rc;
  if (defer_d && (rc = tv_terms_launch(dg, w_d, w_d, w_d, m->side[0]))) return rc;
  // the cell counts are reset beside Adam
  rc = march_backward_reduce(m, m->t_grad_k0, st, false);
  if (rc) return rc;
  if ((defer_k || defer_d) && (rc = join_side(m, st, 1))) return rc;
  // TV in place where it is not deferred (the two grids side by side, each
  // with its own touched list), then the three Adam updates side by side; the
  // rgbnet Adam needs only the rgbnet gradients, complete since the MLP
  // backward
  if ((rc = fork_side(m, st, 2))) return rc;
  if ((rc = march_backward_clear(m, m->side[1]))) return rc;
  rc = adam_dense_launch(net->params, net->grads, net->exp_avg, net->exp_avg_sq, nullptr, P,
                         t.ss[2], cfg->rgbnet_beta1, cfg->rgbnet_beta2, cfg->rgbnet_eps, 0,
                         m->side[1], t.ss_dev ? t.ss_dev + 2 : nullptr);
  if (rc) return rc;
  if (cfg->tv_weight_k0 > 0.f && !defer_k) {
    rc = pvdb_grid_tv_add_grad(kg, w_k, w_k, w_k, cfg->tv_dense_mode, 0,
                               reinterpret_cast<pvdb_stream>(m->side[0]));
    if (rc) return rc;
  }
  rc = opt_launch(t.kopt, 1, 1, t.ss[1], t.ss_dev ? t.ss_dev + 1 : nullptr, m->side[0],
                  defer_k ? kg->d_tv : nullptr, nullptr);
  if (rc) return rc;
  if (cfg->tv_weight_density > 0.f && !defer_d) {
    rc = pvdb_grid_tv_add_grad(dg, w_d, w_d, w_d, cfg->tv_dense_mode, 0, s);
    if (rc) return rc;
  }
  rc = opt_launch(t.dopt, 1, 1, t.ss[0], t.ss_dev ? t.ss_dev + 0 : nullptr, st,
                  defer_d ? dg->d_tv : nullptr, nullptr);
  if (rc) return rc;
  if ((rc = join_side(m, st, 2))) return rc;
  return PVDB_OK;
}

static void graph_reset(pvdb_march_s* m) {
  if (m->g_exec) cudaGraphExecDestroy(m->g_exec);
  if (m->g_graph) cudaGraphDestroy(m->g_graph);
  m->g_exec = nullptr;
  m->g_graph = nullptr;
  m->g_key.clear();
}

template <class T>
static void key_put(std::vector<uint8_t>& k, const T& v) {
  const uint8_t* p = reinterpret_cast<const uint8_t*>(&v);
  k.insert(k.end(), p, p + sizeof(T));
}

static void grid_key(std::vector<uint8_t>& k, const pvdb_grid_s* g) {
  key_put(k, g);
  key_put(k, g->d_data);
  key_put(k, g->d_grad);
  key_put(k, g->d_mask);
  key_put(k, g->d_table);
  key_put(k, g->d_touched);
  key_put(k, g->nleaf);
  key_put(k, g->d_bmax);
  key_put(k, g->bmax_valid);
  key_put(k, g->d_half);
  key_put(k, g->half_valid);
  key_put(k, g->d_tv);
  key_put(k, g->all_touched);
}

// Everything a captured step has baked in: sizes, configuration, and the
// device pointers of every buffer it touches.
static std::vector<uint8_t> graph_key(const TrainArgs& t) {
  std::vector<uint8_t> k;
  const pvdb_march_s* m = t.m;
  key_put(k, t.R);
  key_put(k, *t.cfg);
  key_put(k, t.dopt);
  key_put(k, t.kopt);
  for (pvdb_opt_s* o : {t.dopt, t.kopt}) {
    grid_key(k, opt_params(o));
    grid_key(k, opt_moment(o, 0));
    grid_key(k, opt_moment(o, 1));
  }
  key_put(k, t.net->params);
  key_put(k, t.net->grads);
  key_put(k, t.net->exp_avg);
  key_put(k, t.net->exp_avg_sq);
  key_put(k, t.net->c0);
  key_put(k, t.net->pe);
  key_put(k, m->w);
  key_put(k, m->hpe);
  key_put(k, m->wpart);
  key_put(k, m->mlp_packed);
  key_put(k, m->mlp_xt);
  key_put(k, m->red.keys[0]);
  key_put(k, m->red.keys[1]);
  key_put(k, m->red.vals[0]);
  key_put(k, m->red.vals[1]);
  key_put(k, m->b_rec_s);
  key_put(k, m->leaf_staging);
  key_put(k, m->red.hist);
  key_put(k, m->red.partial);
  key_put(k, m->scan_partial);
  key_put(k, m->cell_cnt);
  key_put(k, m->cell_off);
  key_put(k, m->leaf_cnt);
  key_put(k, m->leaf_off);
  key_put(k, m->t_rgb);
  key_put(k, m->t_grad_k0);
  key_put(k, m->g_in);
  key_put(k, m->g_scal);
  key_put(k, t.loss);  // the replay writes the loss straight to the caller's loss_out
  return k;
}

static int graph_capture(TrainArgs t, const std::vector<uint8_t>& key) {
  pvdb_march_s* m = t.m;
  graph_reset(m);
  if (!m->g_stream) PVDB_CHECK_CUDA(cudaStreamCreateWithFlags(&m->g_stream, cudaStreamNonBlocking));
  const size_t R3 = size_t(t.R) * 3;
  t.ro = m->g_in;
  t.rd = m->g_in + R3;
  t.vd = m->g_in + 2 * R3;
  t.tgt = m->g_in + 3 * R3;
  t.ss_dev = m->g_scal;
  t.prof = false;
  const uint64_t before = launch_counter();
  PVDB_CHECK_CUDA(cudaStreamBeginCapture(m->g_stream, cudaStreamCaptureModeThreadLocal));
  const int rc = train_launches(t, m->g_stream);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(m->g_stream, &g);
  const uint64_t n = launch_counter() - before;
  count_launches(-int(n));  // nothing ran yet; each replay counts them
  if (rc || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    if (rc) return rc;
    return cuda_error(e, "cudaStreamEndCapture");
  }
  m->g_graph = g;
  const cudaError_t ei = cudaGraphInstantiate(&m->g_exec, g, 0);
  if (ei != cudaSuccess) {
    graph_reset(m);
    return cuda_error(ei, "cudaGraphInstantiate");
  }
  m->g_launches = n;
  m->g_key = key;
  return PVDB_OK;
}

}  // namespace pvdb

using namespace pvdb;

extern "C" int pvdb_train_step(pvdb_march m, pvdb_opt density_opt, pvdb_opt k0_opt,
                               pvdb_rgbnet_state* net, const float* rays_o, const float* rays_d,
                               const float* viewdirs, const float* target, int32_t n_rays,
                               const pvdb_train_config* cfg, float* loss_out, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(m && density_opt && k0_opt && net && cfg && loss_out, "null argument");
  PVDB_REQUIRE(n_rays > 0 && n_rays <= m->max_rays, "n_rays must be in 1..max_rays");
  PVDB_REQUIRE(rays_o && rays_d && viewdirs && target, "null rays");
  PVDB_REQUIRE(net->params && net->grads && net->exp_avg && net->exp_avg_sq && net->step &&
                   net->lr,
               "null rgbnet state");
  PVDB_REQUIRE(net->width == 128 && net->c0 > 0 && net->c0 <= 16 && net->pe >= 0 && net->pe <= 4,
               "unsupported rgbnet shape");
  PVDB_REQUIRE(cfg->precision == 0 || cfg->precision == 1, "precision must be 0 or 1");
  pvdb_grid_s* dg = opt_params(density_opt);
  pvdb_grid_s* kg = opt_params(k0_opt);
  PVDB_REQUIRE(dg->C == 1 && kg->C == net->c0, "grid channels do not match the rgbnet");
  cudaStream_t st = as_stream(s);
  int rc = train_reserve(m, kg->C);
  if (rc) return rc;
  // a graph replays the step whose gradients start at zero on tracked leaves;
  // right after the grids were written from outside, step eagerly once
  // (and with the density grid's brick bound and, in BF16, the k0 grid's BF16
  // shadow current: a replay rebuilds neither)
  bool graph_ok = cfg->use_graph && !dg->all_touched && !kg->all_touched && dg->bmax_valid &&
                  (cfg->precision == 0 || kg->C != 12 || kg->half_valid);
  TrainArgs t{m, density_opt, k0_opt, net, rays_o, rays_d, viewdirs, target, n_rays, cfg,
              loss_out, {0.f, 0.f, 0.f}, nullptr, !graph_ok};
  if (graph_ok) {
    const size_t R3 = size_t(n_rays) * 3;
    if ((rc = dev_reserve((void**)&m->g_in, &m->g_in_cap, 4 * R3 * 4))) return rc;
    if (!m->g_scal && (rc = dev_alloc((void**)&m->g_scal, 64))) return rc;
    // capture once the same key was seen on the previous call, i.e. after an
    // eager step allocated every buffer the step needs
    std::vector<uint8_t> key = graph_key(t);
    if (!m->g_exec || key != m->g_key) {
      if (key == m->g_pending) {
        rc = graph_capture(t, key);
        if (rc) return rc;
      } else {
        graph_reset(m);
        m->g_pending = key;
        graph_ok = false;
        t.prof = true;
      }
    }
  }
  // host-side optimiser state (run.py:592-598 order: step, then lr decay)
  t.ss[0] = opt_next_stepsz(density_opt);
  t.ss[1] = opt_next_stepsz(k0_opt);
  *net->step += 1;
  t.ss[2] = adam_step_size(*net->lr, cfg->rgbnet_beta1, cfg->rgbnet_beta2, *net->step);
  if (graph_ok) {
    const int64_t R3 = int64_t(n_rays) * 3;
    launch_k(k_step_inputs, int(std::min<int64_t>(ceil_div(4 * R3, 256), int64_t(2 * num_sms()))),
             256, 0, st, m->g_in, rays_o, rays_d, viewdirs, target, R3, m->g_scal, t.ss[0], t.ss[1],
             t.ss[2]);
    PVDB_CHECK_LAUNCH("k_step_inputs");
    PVDB_CHECK_CUDA(cudaGraphLaunch(m->g_exec, st));
    count_launches(int(m->g_launches));
  } else {
    rc = train_launches(t, st);
    if (rc) return rc;
  }
  *net->lr *= cfg->lr_decay_factor;
  opt_lr_scale(density_opt, cfg->lr_decay_factor);
  opt_lr_scale(k0_opt, cfg->lr_decay_factor);
  return PVDB_OK;
}
