// ORACLE — test infrastructure only. A CPU restatement of PlenVDB's
// differentiable sparse-grid ray-marching path, used by tests/, by
// __graft_entry__.smoke() as the checker, and by bench.py's CPU baseline.
// Nothing in the product (plenvdb_gb300/) may call it.
//
// Every function states the reference code it follows (paths inside
// wolfball/PlenVDB). Two arithmetic modes:
//   fp64  — the truth: positions are formed in float exactly as the reference
//           forms them (they are float tensors there), everything after that in
//           double;
//   fp32  — mimics the reference's float/double promotions operation by
//           operation (the timed CPU baseline and bit-level checks).
// Build with -ffp-contract=off: every multiply-add that the reference's nvcc
// build contracts is written as an explicit std::fma.
//
// Grid representation: a dense padded array over [0, 8*ceil(reso/8))^3 with a
// per-leaf "allocated" flag and a per-voxel active flag. A coordinate outside
// that box or inside an unallocated leaf reads the background, otherwise the
// stored value — the NanoVDB ReadAccessor rules (nanovdb/NanoVDB.h:2999-3010,
// :4626-4674) for a tree whose leaves are the allocated 8^3 blocks.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

typedef struct {
  int reso[3];
  int pad[3];
  int C;
  float background;
  const uint8_t* alloc;   // [pad0/8 * pad1/8 * pad2/8]
  const uint8_t* active;  // [pad0*pad1*pad2]
  const double* values;   // [pad0*pad1*pad2*C]
} ogrid;

typedef struct {
  float xyz_min[3], xyz_max[3];
  float near_, far_, stepdist, act_shift, interval, fast_color_thres, t_stop, bg;
} omarch_params;

typedef struct {
  const double* w0; const double* b0;  // [128, din], [128]
  const double* w1; const double* b1;  // [128, 128], [128]
  const double* w2; const double* b2;  // [3, 128], [3]
  int c0, pe, width;
} omlp;

}  // extern "C"

namespace {

inline bool in_box(const ogrid& g, int i, int j, int k) {
  return i >= 0 && j >= 0 && k >= 0 && i < g.pad[0] && j < g.pad[1] && k < g.pad[2];
}
inline bool allocated(const ogrid& g, int i, int j, int k) {
  if (!in_box(g, i, j, k)) return false;
  const int L1 = g.pad[1] / 8, L2 = g.pad[2] / 8;
  return g.alloc[((i >> 3) * L1 + (j >> 3)) * L2 + (k >> 3)] != 0;
}
inline int64_t vidx(const ogrid& g, int i, int j, int k) {
  return (int64_t(i) * g.pad[1] + j) * g.pad[2] + k;
}
inline double value(const ogrid& g, int i, int j, int k, int ch) {
  return allocated(g, i, j, k) ? g.values[vidx(g, i, j, k) * g.C + ch] : double(g.background);
}

// corner order of densityvdb.cu:116-123
const int kCorner[8][3] = {{0, 0, 0}, {0, 0, 1}, {0, 1, 1}, {0, 1, 0},
                           {1, 1, 0}, {1, 1, 1}, {1, 0, 1}, {1, 0, 0}};

// ---------------------------------------------------------------- sampling
// density_forward_kernel (densityvdb.cu:101-125): res += ((v*(1-u))*(1-v))*(1-w)
template <class T>
T trilinear_density(const ogrid& g, float x, float y, float z) {
  const int i = int(std::floor(x)), j = int(std::floor(y)), k = int(std::floor(z));
  const float uf = x - float(i), vf = y - float(j), wf = z - float(k);
  const T u = T(uf), v = T(vf), w = T(wf);
  T r = 0;
  for (int c = 0; c < 8; ++c) {
    const int* d = kCorner[c];
    const T a = d[0] ? u : T(1) - u, b = d[1] ? v : T(1) - v, cc = d[2] ? w : T(1) - w;
    const T val = T(value(g, i + d[0], j + d[1], k + d[2], 0));
    r = r + ((val * a) * b) * cc;
  }
  return r;
}

// color_forward_kernel (colorvdb.cu:81-111): scale formed first, then v*scale.
template <class T>
void trilinear_color(const ogrid& g, float x, float y, float z, T* out) {
  const int i = int(std::floor(x)), j = int(std::floor(y)), k = int(std::floor(z));
  const T u = T(x - float(i)), v = T(y - float(j)), w = T(z - float(k));
  for (int ch = 0; ch < g.C; ++ch) out[ch] = 0;
  for (int c = 0; c < 8; ++c) {
    const int* d = kCorner[c];
    const T a = d[0] ? u : T(1) - u, b = d[1] ? v : T(1) - v, cc = d[2] ? w : T(1) - w;
    const T scale = (a * b) * cc;
    for (int ch = 0; ch < g.C; ++ch)
      out[ch] = out[ch] + T(value(g, i + d[0], j + d[1], k + d[2], ch)) * scale;
  }
}

// -------------------------------------------------------- ray arithmetic
struct Ray {
  float t_min, t_max, start[3], dir[3];
  int64_t n_steps;
};

// infer_t_minmax / infer_n_samples / infer_ray_start_dir
// (render_utils_kernel.cu:12-78); |d| = sqrt(fma(dz,dz,fma(dx,dx,dy*dy))),
// nvcc's contraction of dx*dx + dy*dy + dz*dz (pinned by the golden vectors
// of the reference's own kernel).
void ray_setup(const float* o, const float* d, const omarch_params& p, Ray& r) {
  const float vx = d[0] == 0.f ? float(1e-6) : d[0];
  const float vy = d[1] == 0.f ? float(1e-6) : d[1];
  const float vz = d[2] == 0.f ? float(1e-6) : d[2];
  const float ax = (p.xyz_max[0] - o[0]) / vx, ay = (p.xyz_max[1] - o[1]) / vy,
              az = (p.xyz_max[2] - o[2]) / vz;
  const float bx = (p.xyz_min[0] - o[0]) / vx, by = (p.xyz_min[1] - o[1]) / vy,
              bz = (p.xyz_min[2] - o[2]) / vz;
  r.t_min = std::max(std::min(std::max(std::max(std::min(ax, bx), std::min(ay, by)), std::min(az, bz)), p.far_), p.near_);
  r.t_max = std::max(std::min(std::min(std::min(std::max(ax, bx), std::max(ay, by)), std::max(az, bz)), p.far_), p.near_);
  const float rn = std::sqrt(std::fma(d[2], d[2], std::fma(d[0], d[0], d[1] * d[1])));
  const float q = ((r.t_max - r.t_min) * rn) / p.stepdist;
  r.n_steps = int64_t(std::max(double(std::ceil(q)), 1.0));
  for (int a = 0; a < 3; ++a) {
    r.start[a] = std::fma(d[a], r.t_min, o[a]);
    r.dir[a] = d[a] / rn;
  }
}

void ray_point(const Ray& r, float stepdist, int64_t k, float* pt) {
  const float dist = stepdist * float(k);
  for (int a = 0; a < 3; ++a) pt[a] = std::fma(r.dir[a], dist, r.start[a]);
}

bool out_of_bbox(const float* pt, const omarch_params& p) {
  for (int a = 0; a < 3; ++a)
    if (p.xyz_min[a] > pt[a] || p.xyz_max[a] < pt[a]) return true;
  return false;
}

// VDBGrid.wld2idx (grid.py:77-78)
void world_to_index(const float* pt, const omarch_params& p, const int* reso, float* idx) {
  for (int a = 0; a < 3; ++a) {
    const float ext = p.xyz_max[a] - p.xyz_min[a];
    idx[a] = ((pt[a] - p.xyz_min[a]) / ext) * float(reso[a] - 1);
  }
}

// raw2alpha (render_utils_kernel.cu:439-441)
template <class T>
T raw2alpha(T sigma, float shift, float interval, T& e) {
  if constexpr (sizeof(T) == 4) {
    e = std::exp(sigma + shift);
    return 1.f - std::pow(1.f + e, -interval);
  } else {
    e = std::exp(sigma + double(shift));
    return 1.0 - std::pow(1.0 + e, -double(interval));
  }
}

// raw2alpha_backward (:514)
template <class T>
T raw2alpha_grad(T e, float interval, T g) {
  if constexpr (sizeof(T) == 4) {
    const double a = std::min(double(e), 1e10);
    return float(a * double(std::pow(1.f + e, -interval - 1.f)) * double(interval) * double(g));
  } else {
    return std::min(e, 1e10) * std::pow(1.0 + e, -double(interval) - 1.0) * double(interval) * g;
  }
}

// T_cum *= (1. - alpha) (:593)
template <class T>
T trans_step(T t, T a) {
  if constexpr (sizeof(T) == 4)
    return float(double(t) * (1.0 - double(a)));
  else
    return t * (1.0 - a);
}

// grad = gw*T - back/(1-alpha+1e-10) (:671)
template <class T>
T alpha_grad(T gw, T t, T back, T a) {
  if constexpr (sizeof(T) == 4)
    return float(double(gw * t) - double(back) / (double(1.f - a) + 1e-10));
  else
    return gw * t - back / (1.0 - a + 1e-10);
}

// ------------------------------------------------------------------ MLP
template <class T>
struct MlpT {
  std::vector<T> w0, b0, w1, b1, w2, b2;
  int c0, pe, din, W;
  explicit MlpT(const omlp& m) : c0(m.c0), pe(m.pe), W(m.width) {
    din = c0 + 3 + 6 * pe;
    w0.assign(m.w0, m.w0 + W * din);
    b0.assign(m.b0, m.b0 + W);
    w1.assign(m.w1, m.w1 + W * W);
    b1.assign(m.b1, m.b1 + W);
    w2.assign(m.w2, m.w2 + 3 * W);
    b2.assign(m.b2, m.b2 + 3);
  }
};

// viewdirs PE (dvgo.py:354-355): [d, sin(d*2^i), cos(d*2^i)], i-major per axis.
template <class T>
void view_pe(const float* d, int npe, T* out) {
  out[0] = d[0]; out[1] = d[1]; out[2] = d[2];
  for (int a = 0; a < 3; ++a)
    for (int i = 0; i < npe; ++i) {
      const float x = d[a] * float(1 << i);
      out[3 + a * npe + i] = T(std::sin(T(x)));
      out[3 + 3 * npe + a * npe + i] = T(std::cos(T(x)));
    }
}

template <class T>
void mlp_forward(const MlpT<T>& m, const T* x, T* h0, T* h1, T* logit) {
  for (int n = 0; n < m.W; ++n) {
    T s = m.b0[n];
    for (int q = 0; q < m.din; ++q) s += m.w0[n * m.din + q] * x[q];
    h0[n] = s > 0 ? s : T(0);
  }
  for (int n = 0; n < m.W; ++n) {
    T s = m.b1[n];
    for (int q = 0; q < m.W; ++q) s += m.w1[n * m.W + q] * h0[q];
    h1[n] = s > 0 ? s : T(0);
  }
  for (int c = 0; c < 3; ++c) {
    T s = m.b2[c];
    for (int q = 0; q < m.W; ++q) s += m.w2[c * m.W + q] * h1[q];
    logit[c] = s;
  }
}

template <class T>
T sigmoid(T x) { return T(1) / (T(1) + std::exp(-x)); }

// ------------------------------------------------------------ the march
struct Row {
  int ray;
  int step;
  int kept_index;  // index within the ray's kept list
  float idx[3];
};

template <class T>
struct MarchOut {
  std::vector<T> T_last;
  std::vector<int> n_kept, n_color;
  std::vector<std::vector<T>> kept_alpha;   // per ray
  std::vector<std::vector<int>> kept_step;  // per ray
  std::vector<std::vector<int>> kept_row;   // per ray: colour row or -1
  std::vector<std::vector<float>> kept_idx; // per ray: index-space position (3 per sample)
  std::vector<std::vector<T>> kept_sigma;   // per ray: raw density
  std::vector<Row> rows;
  std::vector<T> row_w, row_alpha, row_k0;  // row_k0 [M*C]
};

// DirectVoxGO.forward up to the k0 query (dvgo.py:296-341) for one ray.
template <class T>
void march_ray(const ogrid& gd, const ogrid* gk, const float* o, const float* d,
               const omarch_params& p, int r, MarchOut<T>& out, std::vector<Row>& rows_r,
               std::vector<T>& w_r, std::vector<T>& a_r) {
  Ray ray;
  ray_setup(o, d, p, ray);
  T Tc = 1;
  auto& ka = out.kept_alpha[r];
  auto& ks = out.kept_step[r];
  auto& kx = out.kept_idx[r];
  auto& kg = out.kept_sigma[r];
  std::vector<T> kw;
  for (int64_t k = 0; k < ray.n_steps; ++k) {
    float pt[3];
    ray_point(ray, p.stepdist, k, pt);
    if (out_of_bbox(pt, p)) continue;
    float idx[3];
    world_to_index(pt, p, gd.reso, idx);
    const T sigma = trilinear_density<T>(gd, idx[0], idx[1], idx[2]);
    T e;
    const T alpha = raw2alpha<T>(sigma, p.act_shift, p.interval, e);
    if (!(alpha > T(p.fast_color_thres))) continue;
    const T w = Tc * alpha;
    ka.push_back(alpha);
    ks.push_back(int(k));
    kw.push_back(w);
    kx.insert(kx.end(), idx, idx + 3);
    kg.push_back(sigma);
    Tc = trans_step<T>(Tc, alpha);
    const bool stop = sizeof(T) == 4 ? (float(Tc) < p.t_stop) : (double(Tc) < double(p.t_stop));
    if (stop) break;
  }
  out.T_last[r] = Tc;
  out.n_kept[r] = int(ka.size());
  out.kept_row[r].assign(ka.size(), -1);
  int nc = 0;
  for (size_t i = 0; i < ka.size(); ++i) {
    if (!(kw[i] > T(p.fast_color_thres))) continue;
    Row row;
    row.ray = r;
    row.step = ks[i];
    row.kept_index = int(i);
    float pt[3];
    ray_point(ray, p.stepdist, ks[i], pt);
    world_to_index(pt, p, gd.reso, row.idx);
    rows_r.push_back(row);
    w_r.push_back(kw[i]);
    a_r.push_back(ka[i]);
    ++nc;
  }
  out.n_color[r] = nc;
  (void)gk;
}

template <class T>
void march_forward(const ogrid& gd, const ogrid* gk, const float* ro, const float* rd, int R,
                   const omarch_params& p, MarchOut<T>& out) {
  out.T_last.assign(R, 1);
  out.n_kept.assign(R, 0);
  out.n_color.assign(R, 0);
  out.kept_alpha.assign(R, {});
  out.kept_step.assign(R, {});
  out.kept_row.assign(R, {});
  out.kept_idx.assign(R, {});
  out.kept_sigma.assign(R, {});
  std::vector<std::vector<Row>> rows(R);
  std::vector<std::vector<T>> ws(R), as(R);
#pragma omp parallel for schedule(dynamic, 16)
  for (int r = 0; r < R; ++r) march_ray<T>(gd, gk, ro + 3 * r, rd + 3 * r, p, r, out, rows[r], ws[r], as[r]);
  out.rows.clear();
  out.row_w.clear();
  out.row_alpha.clear();
  for (int r = 0; r < R; ++r) {
    for (size_t j = 0; j < rows[r].size(); ++j) {
      out.kept_row[r][rows[r][j].kept_index] = int(out.rows.size());
      out.rows.push_back(rows[r][j]);
      out.row_w.push_back(ws[r][j]);
      out.row_alpha.push_back(as[r][j]);
    }
  }
  const int C = gk ? gk->C : 0;
  out.row_k0.assign(out.rows.size() * size_t(C), 0);
  if (gk) {
#pragma omp parallel for schedule(static)
    for (int64_t m = 0; m < int64_t(out.rows.size()); ++m)
      trilinear_color<T>(*gk, out.rows[m].idx[0], out.rows[m].idx[1], out.rows[m].idx[2],
                         &out.row_k0[m * C]);
  }
}

}  // namespace

// =================================================================== C API
extern "C" {

int oracle_version(void) { return 1; }

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// ReadAccessor::getValue / isActive at integer coordinates (forward_single,
// densityvdb.cu:376-403).
void oracle_lookup(const ogrid* g, const int32_t* ijk, int64_t n, double* out, uint8_t* act) {
  for (int64_t p = 0; p < n; ++p) {
    const int i = ijk[3 * p], j = ijk[3 * p + 1], k = ijk[3 * p + 2];
    for (int ch = 0; ch < g->C; ++ch) out[p * g->C + ch] = value(*g, i, j, k, ch);
    act[p] = allocated(*g, i, j, k) ? g->active[vidx(*g, i, j, k)] : 0;
  }
}

// forward (densityvdb.cu:101-125 for C == 1, colorvdb.cu:81-111 otherwise)
void oracle_sample(const ogrid* g, const float* xyz, int64_t n, int fp32, double* out) {
  for (int64_t p = 0; p < n; ++p) {
    const float x = xyz[3 * p], y = xyz[3 * p + 1], z = xyz[3 * p + 2];
    if (g->C == 1) {
      out[p] = fp32 ? double(trilinear_density<float>(*g, x, y, z))
                    : trilinear_density<double>(*g, x, y, z);
    } else if (fp32) {
      std::vector<float> tmp(g->C);
      trilinear_color<float>(*g, x, y, z, tmp.data());
      for (int ch = 0; ch < g->C; ++ch) out[p * g->C + ch] = tmp[ch];
    } else {
      trilinear_color<double>(*g, x, y, z, out + p * g->C);
    }
  }
}

// backward (densityvdb.cu:16-27 + :143-167; colorvdb.cu:28-37 + :130-160): the
// contribution of every corner inside an allocated leaf is added to grad
// (a dense padded array [pad^3 * C]); the sum runs in point order.
void oracle_sample_backward(const ogrid* g, const float* xyz, const double* grad_in, int64_t n,
                            double* grad) {
  for (int64_t p = 0; p < n; ++p) {
    const float x = xyz[3 * p], y = xyz[3 * p + 1], z = xyz[3 * p + 2];
    const int i = int(std::floor(x)), j = int(std::floor(y)), k = int(std::floor(z));
    const double u = x - float(i), v = y - float(j), w = z - float(k);
    for (int c = 0; c < 8; ++c) {
      const int* d = kCorner[c];
      const int ci = i + d[0], cj = j + d[1], ck = k + d[2];
      if (!allocated(*g, ci, cj, ck)) continue;
      const double a = d[0] ? u : 1 - u, b = d[1] ? v : 1 - v, cc = d[2] ? w : 1 - w;
      for (int ch = 0; ch < g->C; ++ch)
        grad[vidx(*g, ci, cj, ck) * g->C + ch] += grad_in[p * g->C + ch] * a * b * cc;
    }
  }
}

// Voxel Adam (densityvdb.cu:185-330, colorvdb.cu:179-331) on dense padded
// arrays; only active voxels of allocated leaves; mode 1 skips a group (1 or 3
// channels) whose gradient is all zero. stepsz is the host-side bias-corrected
// step (plenvdb.h:753). fp32 mimics float arithmetic.
void oracle_adam(const ogrid* g, double* data, const double* grad, double* m, double* v,
                 const double* perlr, float stepsz, float eps, float b0, float b1, int mode,
                 int fp32) {
  const int G = g->C == 1 ? 1 : 3;
  const int64_t nvox = int64_t(g->pad[0]) * g->pad[1] * g->pad[2];
  for (int64_t q = 0; q < nvox; ++q) {
    const int i = int(q / (int64_t(g->pad[1]) * g->pad[2]));
    const int j = int((q / g->pad[2]) % g->pad[1]);
    const int k = int(q % g->pad[2]);
    if (!allocated(*g, i, j, k) || !g->active[q]) continue;
    for (int gr = 0; gr < g->C / G; ++gr) {
      const int64_t base = q * g->C + gr * G;
      bool allzero = true;
      for (int t = 0; t < G; ++t) allzero = allzero && grad[base + t] == 0;
      if (mode == 1 && allzero) continue;
      for (int t = 0; t < G; ++t) {
        if (fp32) {
          const float gg = float(grad[base + t]);
          const float mn = b0 * float(m[base + t]) + (1 - b0) * gg;
          const float vn = b1 * float(v[base + t]) + (1 - b1) * gg * gg;
          m[base + t] = mn;
          v[base + t] = vn;
          const float num = mode == 2 ? float(perlr[q]) * stepsz * mn : stepsz * mn;
          data[base + t] = float(data[base + t]) - num / (eps + std::sqrt(vn));
        } else {
          const double gg = grad[base + t];
          const double mn = double(b0) * m[base + t] + (1 - double(b0)) * gg;
          const double vn = double(b1) * v[base + t] + (1 - double(b1)) * gg * gg;
          m[base + t] = mn;
          v[base + t] = vn;
          const double num = (mode == 2 ? perlr[q] : 1.0) * double(stepsz) * mn;
          data[base + t] = data[base + t] - num / (double(eps) + std::sqrt(vn));
        }
      }
    }
  }
}

// TV (total_variation_kernel.cu:13-35) with weights already divided by 6;
// neighbours inside [0, reso); values through the leaf rules; every active
// voxel (dense_mode) or those with a nonzero gradient. The six terms are taken
// in the reference's order (k-1, k+1, j-1, j+1, i-1, i+1). fp32 mimics the
// reference's float arithmetic: each term w * clamp(p - q) is rounded, then
// added to the running float sum (the conditional around each term keeps nvcc
// from fusing them), and the sum is added to the gradient last. The i axis is weighted by wx (the
// reference writes wz there, :31-32; its callers pass wx == wz, dvgo.py:245-251).
void oracle_tv(const ogrid* g, double* grad, float wx, float wy, float wz, int dense_mode,
               int fp32) {
  const int64_t nvox = int64_t(g->pad[0]) * g->pad[1] * g->pad[2];
  std::vector<double> add(size_t(nvox) * g->C, 0.0);
  std::vector<uint8_t> has(size_t(nvox) * g->C, 0);
  auto cl = [](double x) { return std::min(std::max(x, -1.0), 1.0); };
  auto clf = [](float x) { return std::min(std::max(x, -1.f), 1.f); };
  for (int i = 0; i < g->reso[0]; ++i)
    for (int j = 0; j < g->reso[1]; ++j)
      for (int k = 0; k < g->reso[2]; ++k) {
        const int64_t q = vidx(*g, i, j, k);
        if (!allocated(*g, i, j, k) || !g->active[q]) continue;
        for (int ch = 0; ch < g->C; ++ch) {
          if (!dense_mode && grad[q * g->C + ch] == 0) continue;
          const bool in[6] = {k > 0, k < g->reso[2] - 1, j > 0, j < g->reso[1] - 1, i > 0,
                              i < g->reso[0] - 1};
          const int nb[6][3] = {{i, j, k - 1}, {i, j, k + 1}, {i, j - 1, k},
                                {i, j + 1, k}, {i - 1, j, k}, {i + 1, j, k}};
          const float w[6] = {wz, wz, wy, wy, wx, wx};
          if (fp32) {
            const float p = float(value(*g, i, j, k, ch));
            float s = 0.f;
            for (int t = 0; t < 6; ++t)
              if (in[t]) {
                const float term = w[t] * clf(p - float(value(*g, nb[t][0], nb[t][1], nb[t][2], ch)));
                s = s + term;
              }
            add[q * g->C + ch] = s;
          } else {
            const double p = value(*g, i, j, k, ch);
            double s = 0;
            for (int t = 0; t < 6; ++t)
              if (in[t]) s += w[t] * cl(p - value(*g, nb[t][0], nb[t][1], nb[t][2], ch));
            add[q * g->C + ch] = s;
          }
          has[q * g->C + ch] = 1;
        }
      }
  for (int64_t q = 0; q < nvox * g->C; ++q) {
    if (!has[q]) continue;
    grad[q] = fp32 ? double(float(grad[q]) + float(add[q])) : grad[q] + add[q];
  }
}

// Dense Adam of MaskedAdam (masked_adam.py:105-158 -> adam_upd_kernel.cu):
// mode 0 adam_upd (:8-23), 1 masked_adam_upd (skip g == 0, :25-41), 2
// adam_upd_with_perlr (:43-58). The step size is the host's
// lr * sqrt(1 - beta2^step) / (1 - beta1^step) in float (:72). fp32 mimics
// the float kernel: each moment is one fused multiply-add of the decayed
// moment onto the rounded gradient term (nvcc's contraction of
// `beta * m + (1 - beta) * g`).
float oracle_adam_step_size(float lr, float beta1, float beta2, int step) {
  return lr * std::sqrt(1.f - std::pow(beta2, float(step))) / (1.f - std::pow(beta1, float(step)));
}

void oracle_adam_dense(double* p, const double* g, double* m, double* v, const double* perlr,
                       int64_t n, int step, float beta1, float beta2, float lr, float eps,
                       int mode, int fp32) {
  const float ss = oracle_adam_step_size(lr, beta1, beta2, step);
  for (int64_t i = 0; i < n; ++i) {
    if (mode == 1 && g[i] == 0) continue;
    if (fp32) {
      const float gi = float(g[i]);
      const float mn = std::fma(beta1, float(m[i]), (1.f - beta1) * gi);
      const float vn = std::fma(beta2, float(v[i]), (1.f - beta2) * gi * gi);
      m[i] = mn;
      v[i] = vn;
      const float num = mode == 2 ? ss * float(perlr[i]) * mn : ss * mn;
      p[i] = float(p[i]) - num / (std::sqrt(vn) + eps);
    } else {
      const double b1 = beta1, b2 = beta2;
      const double mn = b1 * m[i] + (1 - b1) * g[i];
      const double vn = b2 * v[i] + (1 - b2) * g[i] * g[i];
      m[i] = mn;
      v[i] = vn;
      const double num = double(ss) * (mode == 2 ? perlr[i] : 1.0) * mn;
      p[i] = p[i] - num / (std::sqrt(vn) + double(eps));
    }
  }
}

// raw2alpha / raw2alpha_backward (render_utils_kernel.cu:430-552)
void oracle_raw2alpha(const float* d, int64_t n, float shift, float interval, int fp32,
                      double* e_out, double* a_out) {
  for (int64_t i = 0; i < n; ++i) {
    if (fp32) {
      float e;
      const float a = raw2alpha<float>(d[i], shift, interval, e);
      e_out[i] = e;
      a_out[i] = a;
    } else {
      double e;
      a_out[i] = raw2alpha<double>(double(d[i]), shift, interval, e);
      e_out[i] = e;
    }
  }
}

void oracle_raw2alpha_backward(const double* e, const double* g, int64_t n, float interval,
                               int fp32, double* out) {
  for (int64_t i = 0; i < n; ++i)
    out[i] = fp32 ? double(raw2alpha_grad<float>(float(e[i]), interval, float(g[i])))
                  : raw2alpha_grad<double>(e[i], interval, g[i]);
}

// alpha2weight (:576-605) on sorted ray ids; returns i_end per ray.
void oracle_alpha2weight(const double* alpha, const int64_t* ray_id, int64_t n, int R, int fp32,
                         double* weight, double* T, double* last, int64_t* i_start,
                         int64_t* i_end) {
  for (int64_t i = 0; i < n; ++i) {
    weight[i] = 0;
    T[i] = 1;
  }
  for (int r = 0; r < R; ++r) {
    last[r] = 1;
    i_start[r] = 0;
    i_end[r] = 0;
  }
  for (int64_t i = 1; i < n; ++i)
    if (ray_id[i] != ray_id[i - 1]) {
      i_start[ray_id[i]] = i;
      i_end[ray_id[i - 1]] = i;
    }
  if (n) i_end[ray_id[n - 1]] = n;
  for (int r = 0; r < R; ++r) {
    int64_t i;
    if (fp32) {
      float Tc = 1.f;
      for (i = i_start[r]; i < i_end[r]; ++i) {
        T[i] = Tc;
        weight[i] = Tc * float(alpha[i]);
        Tc = trans_step<float>(Tc, float(alpha[i]));
        if (double(Tc) < 1e-3) {
          ++i;
          break;
        }
      }
      last[r] = Tc;
    } else {
      double Tc = 1.0;
      for (i = i_start[r]; i < i_end[r]; ++i) {
        T[i] = Tc;
        weight[i] = Tc * alpha[i];
        Tc = Tc * (1.0 - alpha[i]);
        if (Tc < 1e-3) {
          ++i;
          break;
        }
      }
      last[r] = Tc;
    }
    i_end[r] = i;
  }
}

void oracle_alpha2weight_backward(const double* alpha, const double* weight, const double* T,
                                  const double* last, const int64_t* i_start,
                                  const int64_t* i_end, int R, const double* gw, const double* gl,
                                  int64_t n, int fp32, double* grad) {
  for (int64_t i = 0; i < n; ++i) grad[i] = 0;
  for (int r = 0; r < R; ++r) {
    if (fp32) {
      float back = float(gl[r]) * float(last[r]);
      for (int64_t i = i_end[r] - 1; i >= i_start[r]; --i) {
        grad[i] = alpha_grad<float>(float(gw[i]), float(T[i]), back, float(alpha[i]));
        back = std::fma(float(gw[i]), float(weight[i]), back);
      }
    } else {
      double back = gl[r] * last[r];
      for (int64_t i = i_end[r] - 1; i >= i_start[r]; --i) {
        grad[i] = gw[i] * T[i] - back / (1.0 - alpha[i] + 1e-10);
        back += gw[i] * weight[i];
      }
    }
  }
}

// sample_pts_on_rays step 1 (:196-212)
void oracle_ray_count(const float* ro, const float* rd, int R, const omarch_params* p,
                      float* t_min, float* t_max, int64_t* n_steps) {
  for (int r = 0; r < R; ++r) {
    Ray ray;
    ray_setup(ro + 3 * r, rd + 3 * r, *p, ray);
    t_min[r] = ray.t_min;
    t_max[r] = ray.t_max;
    n_steps[r] = ray.n_steps;
  }
}

// sample_pts_on_rays step 2 (:213-242) into preallocated arrays of length total
void oracle_ray_points(const float* ro, const float* rd, int R, const omarch_params* p,
                       float* pts, uint8_t* outbbox, int64_t* ray_id, int64_t* step_id) {
  int64_t o = 0;
  for (int r = 0; r < R; ++r) {
    Ray ray;
    ray_setup(ro + 3 * r, rd + 3 * r, *p, ray);
    for (int64_t k = 0; k < ray.n_steps; ++k, ++o) {
      ray_point(ray, p->stepdist, k, pts + 3 * o);
      outbbox[o] = out_of_bbox(pts + 3 * o, *p) ? 1 : 0;
      ray_id[o] = r;
      step_id[o] = k;
    }
  }
}

// maskcache_lookup (:380-394)
void oracle_maskcache(const uint8_t* world, const int32_t* shape, const float* xyz, int64_t n,
                      const float* scale, const float* shift, uint8_t* out) {
  for (int64_t q = 0; q < n; ++q) {
    int ijk[3];
    for (int a = 0; a < 3; ++a) ijk[a] = int(std::round(std::fma(xyz[3 * q + a], scale[a], shift[a])));
    bool in = true;
    for (int a = 0; a < 3; ++a) in = in && ijk[a] >= 0 && ijk[a] < shape[a];
    out[q] = in ? world[(int64_t(ijk[0]) * shape[1] + ijk[1]) * shape[2] + ijk[2]] : 0;
  }
}

// -------------------------------------------------------- fused march
// Runs DirectVoxGO.forward (dvgo.py:296-370) without the mask cache and
// returns per-ray and per-colour-row results. The result object is kept in a
// handle so that the caller can size its arrays before copying.
struct OracleMarch {
  int fp32;
  MarchOut<double> d;
  MarchOut<float> f;
  int C;
  int R;
};

void* oracle_march_run(const ogrid* gd, const ogrid* gk, const float* ro, const float* rd, int R,
                       const omarch_params* p, int fp32) {
  OracleMarch* h = new OracleMarch();
  h->fp32 = fp32;
  h->C = gk ? gk->C : 0;
  h->R = R;
  if (fp32)
    march_forward<float>(*gd, gk, ro, rd, R, *p, h->f);
  else
    march_forward<double>(*gd, gk, ro, rd, R, *p, h->d);
  return h;
}

int64_t oracle_march_rows(void* hp) {
  OracleMarch* h = (OracleMarch*)hp;
  return h->fp32 ? int64_t(h->f.rows.size()) : int64_t(h->d.rows.size());
}

int64_t oracle_march_kept(void* hp) {
  OracleMarch* h = (OracleMarch*)hp;
  int64_t s = 0;
  for (int r = 0; r < h->R; ++r) s += h->fp32 ? h->f.n_kept[r] : h->d.n_kept[r];
  return s;
}

}  // extern "C"

template <class T>
static void march_copy(const MarchOut<T>& o, int R, int C, double* T_last, int32_t* n_kept,
                       int32_t* n_color, double* k0, double* w, double* alpha, int32_t* ray,
                       int32_t* step, double* kept_alpha, int32_t* kept_step) {
  int64_t kk = 0;
  for (int r = 0; r < R; ++r) {
    T_last[r] = o.T_last[r];
    n_kept[r] = o.n_kept[r];
    n_color[r] = o.n_color[r];
    for (size_t i = 0; i < o.kept_alpha[r].size(); ++i, ++kk) {
      if (kept_alpha) kept_alpha[kk] = o.kept_alpha[r][i];
      if (kept_step) kept_step[kk] = o.kept_step[r][i];
    }
  }
  for (size_t m = 0; m < o.rows.size(); ++m) {
    for (int c = 0; c < C; ++c) k0[m * C + c] = o.row_k0[m * C + c];
    w[m] = o.row_w[m];
    alpha[m] = o.row_alpha[m];
    ray[m] = o.rows[m].ray;
    step[m] = o.rows[m].step;
  }
}

extern "C" {

void oracle_march_fetch(void* hp, double* T_last, int32_t* n_kept, int32_t* n_color, double* k0,
                        double* w, double* alpha, int32_t* ray, int32_t* step,
                        double* kept_alpha, int32_t* kept_step) {
  OracleMarch* h = (OracleMarch*)hp;
  if (h->fp32)
    march_copy(h->f, h->R, h->C, T_last, n_kept, n_color, k0, w, alpha, ray, step, kept_alpha,
               kept_step);
  else
    march_copy(h->d, h->R, h->C, T_last, n_kept, n_color, k0, w, alpha, ray, step, kept_alpha,
               kept_step);
}

// rgbnet on the colour rows: rgb = sigmoid(MLP([k0, PE(viewdir[ray])])).
void oracle_march_rgb(void* hp, const omlp* mw, const float* viewdirs, double* rgb) {
  OracleMarch* h = (OracleMarch*)hp;
  MlpT<double> m(*mw);
  const int64_t M = oracle_march_rows(hp);
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < M; ++r) {
    std::vector<double> x(m.din), h0(m.W), h1(m.W);
    double lg[3];
    const int ray = h->fp32 ? h->f.rows[r].ray : h->d.rows[r].ray;
    for (int c = 0; c < m.c0; ++c) x[c] = h->fp32 ? h->f.row_k0[r * m.c0 + c] : h->d.row_k0[r * m.c0 + c];
    view_pe<double>(viewdirs + 3 * ray, m.pe, x.data() + m.c0);
    mlp_forward<double>(m, x.data(), h0.data(), h1.data(), lg);
    for (int c = 0; c < 3; ++c) rgb[r * 3 + c] = sigmoid(lg[c]);
  }
}

// Backward of the whole path in FP64 given the upstream gradients:
//   g_rgbm [R,3]  gradient of rgb_marched,
//   g_last [R]    extra gradient of alphainv_last (entropy loss),
//   g_rgb  [M,3]  extra gradient of the per-row rgb (per-point rgb loss).
// Writes the dense padded gradients of the density (C=1) and k0 grids and the
// rgbnet parameter gradients (same layouts as omlp). Only valid for fp64 runs.
void oracle_march_backward_sample(void* hp, const ogrid* gd, const ogrid* gk,
                                  const omarch_params* p, const double* g_w, const double* g_last,
                                  const double* g_k0, double* gdens, double* gk0);

void oracle_march_backward(void* hp, const ogrid* gd, const ogrid* gk, const omlp* mw,
                           const float* viewdirs, const omarch_params* p, const double* g_rgbm,
                           const double* g_last_extra, const double* g_rgb_extra,
                           double* gdens, double* gk0, double* gw0, double* gb0, double* gw1,
                           double* gb1, double* gw2, double* gb2) {
  OracleMarch* h = (OracleMarch*)hp;
  const MarchOut<double>& o = h->d;
  MlpT<double> m(*mw);
  const int64_t M = int64_t(o.rows.size());
  const int C = gk->C;
  std::vector<double> grad_w(M, 0.0), gk0_rows(M * size_t(C), 0.0);
  // composite + MLP backward per row
  for (int64_t r = 0; r < M; ++r) {
    const int ray = o.rows[r].ray;
    std::vector<double> x(m.din), h0(m.W), h1(m.W), dh1(m.W), dh0(m.W);
    double lg[3], rgb[3], dl[3];
    for (int c = 0; c < C; ++c) x[c] = o.row_k0[r * C + c];
    view_pe<double>(viewdirs + 3 * ray, m.pe, x.data() + m.c0);
    mlp_forward<double>(m, x.data(), h0.data(), h1.data(), lg);
    const double w = o.row_w[r];
    double gwr = 0;
    for (int c = 0; c < 3; ++c) {
      rgb[c] = sigmoid(lg[c]);
      gwr += g_rgbm[ray * 3 + c] * rgb[c];
      const double grgb = w * g_rgbm[ray * 3 + c] + (g_rgb_extra ? g_rgb_extra[r * 3 + c] : 0.0);
      dl[c] = grgb * rgb[c] * (1 - rgb[c]);
    }
    grad_w[r] = gwr;
    for (int c = 0; c < 3; ++c) {
      gb2[c] += dl[c];
      for (int q = 0; q < m.W; ++q) gw2[c * m.W + q] += dl[c] * h1[q];
    }
    for (int q = 0; q < m.W; ++q) {
      double s = 0;
      for (int c = 0; c < 3; ++c) s += dl[c] * m.w2[c * m.W + q];
      dh1[q] = h1[q] > 0 ? s : 0;
    }
    for (int n = 0; n < m.W; ++n) {
      gb1[n] += dh1[n];
      for (int q = 0; q < m.W; ++q) gw1[n * m.W + q] += dh1[n] * h0[q];
    }
    for (int q = 0; q < m.W; ++q) {
      double s = 0;
      for (int n = 0; n < m.W; ++n) s += dh1[n] * m.w1[n * m.W + q];
      dh0[q] = h0[q] > 0 ? s : 0;
    }
    for (int n = 0; n < m.W; ++n) {
      gb0[n] += dh0[n];
      for (int q = 0; q < m.din; ++q) gw0[n * m.din + q] += dh0[n] * x[q];
    }
    for (int c = 0; c < C; ++c) {
      double s = 0;
      for (int n = 0; n < m.W; ++n) s += dh0[n] * m.w0[n * m.din + c];
      gk0_rows[r * C + c] = s;
    }
  }
  std::vector<double> gl(h->R);
  for (int ray = 0; ray < h->R; ++ray) {
    gl[ray] = g_last_extra ? g_last_extra[ray] : 0.0;
    for (int c = 0; c < 3; ++c) gl[ray] += g_rgbm[ray * 3 + c] * double(p->bg);
  }
  oracle_march_backward_sample(hp, gd, gk, p, grad_w.data(), gl.data(), gk0_rows.data(), gdens,
                               gk0);
}

// Backward of the sample stage alone (FP64), given the gradient of every
// colour-row weight g_w [M], of alphainv_last g_last [R] and of the k0 rows
// g_k0 [M, C] (may be NULL): alpha2weight_backward (:653-677), raw2alpha_backward
// (:506-517) and the two grid scatters (densityvdb.cu:143-167,
// colorvdb.cu:130-160) into dense padded gradients.
void oracle_march_backward_sample(void* hp, const ogrid* gd, const ogrid* gk,
                                  const omarch_params* p, const double* g_w, const double* g_last,
                                  const double* g_k0, double* gdens, double* gk0) {
  OracleMarch* h = (OracleMarch*)hp;
  const MarchOut<double>& o = h->d;
  const int64_t M = int64_t(o.rows.size());
  if (g_k0 && gk)
    for (int64_t r = 0; r < M; ++r)
      oracle_sample_backward(gk, o.rows[r].idx, &g_k0[r * gk->C], 1, gk0);
  for (int ray = 0; ray < h->R; ++ray) {
    const auto& ka = o.kept_alpha[ray];
    const int nk = int(ka.size());
    if (!nk) continue;
    std::vector<double> Tv(nk), wv(nk), gwv(nk, 0.0);
    double Tc = 1;
    for (int i = 0; i < nk; ++i) {
      Tv[i] = Tc;
      wv[i] = Tc * ka[i];
      Tc *= (1 - ka[i]);
    }
    for (int i = 0; i < nk; ++i)
      if (o.kept_row[ray][i] >= 0) gwv[i] = g_w[o.kept_row[ray][i]];
    double back = g_last[ray] * o.T_last[ray];
    for (int i = nk - 1; i >= 0; --i) {
      const double ga = gwv[i] * Tv[i] - back / (1 - ka[i] + 1e-10);
      back += gwv[i] * wv[i];
      double e;
      (void)raw2alpha<double>(o.kept_sigma[ray][i], p->act_shift, p->interval, e);
      const double gs = raw2alpha_grad<double>(e, p->interval, ga);
      oracle_sample_backward(gd, &o.kept_idx[ray][3 * i], &gs, 1, gdens);
    }
  }
}

void oracle_march_free(void* hp) { delete (OracleMarch*)hp; }

// ------------------------------------------------ CPU training iteration
// One fine-stage iteration (run.py:516-598) in FP32 on the host cores: the
// reference's float arithmetic (march_forward<float>), rgbnet forward and
// backward in float, the three losses, alpha2weight/raw2alpha backward, the
// gradient scatter (float atomics as the reference's kernels do), TV with
// weight tv_w (already / 6), and voxel Adam mode 1 on both grids plus Adam on
// the rgbnet parameters (flat [w0,b0,w1,b1,w2,b2]). Grids are dense padded
// float arrays (values, grads, moments); `vals` are modified in place.
// Returns the loss.
typedef struct {
  int reso[3], pad[3];
  float background;
  const uint8_t* alloc;
  const uint8_t* active;
  float* dens;  // [pad^3]
  float* k0;    // [pad^3 * C]
  float* gdens;
  float* gk0;
  float* m_d; float* v_d; float* m_k; float* v_k;
  int C;
  int step;
  float lr_d, lr_k;
} otrain_grids;

typedef struct {
  float* params; float* grads; float* m; float* v;
  int c0, pe, width, step;
  float lr;
} otrain_net;

double oracle_train_step_fp32(otrain_grids* G, otrain_net* N, const float* ro, const float* rd,
                              const float* vd, const float* target, int R,
                              const omarch_params* p, float w_main, float w_ent, float w_per,
                              float tv_w) {
  // views of the grids as ogrid (values as double are not needed: build float accessors)
  const int P0 = G->pad[0], P1 = G->pad[1], P2 = G->pad[2];
  const int C = G->C;
  const int64_t nvox = int64_t(P0) * P1 * P2;
  auto alloc_at = [&](int i, int j, int k) {
    if (i < 0 || j < 0 || k < 0 || i >= P0 || j >= P1 || k >= P2) return false;
    return G->alloc[((i >> 3) * (P1 / 8) + (j >> 3)) * (P2 / 8) + (k >> 3)] != 0;
  };
  auto vid = [&](int i, int j, int k) { return (int64_t(i) * P1 + j) * P2 + k; };
  auto dval = [&](int i, int j, int k) { return alloc_at(i, j, k) ? G->dens[vid(i, j, k)] : G->background; };
  const int W = N->width, din = N->c0 + 3 + 6 * N->pe;
  float* w0 = N->params;
  float* b0 = w0 + W * din;
  float* w1 = b0 + W;
  float* b1 = w1 + W * W;
  float* w2 = b1 + W;
  float* b2 = w2 + 3 * W;
  const int64_t NP = int64_t(W) * din + W + W * W + W + 3 * W + 3;
  std::fill(N->grads, N->grads + NP, 0.f);
  double loss = 0;
  int nth = 1;
#ifdef _OPENMP
  nth = omp_get_max_threads();
#endif
  std::vector<std::vector<float>> tgrads(nth, std::vector<float>(NP, 0.f));
#pragma omp parallel for schedule(dynamic, 8) reduction(+ : loss)
  for (int r = 0; r < R; ++r) {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    float* tg = tgrads[tid].data();
    Ray ray;
    ray_setup(ro + 3 * r, rd + 3 * r, *p, ray);
    // forward march (density, alpha, composite) in the reference's float arithmetic
    std::vector<float> ka, kw, kT, ksig;
    std::vector<std::array<float, 3>> kidx;
    float Tc = 1.f;
    for (int64_t k = 0; k < ray.n_steps; ++k) {
      float pt[3], idx[3];
      ray_point(ray, p->stepdist, k, pt);
      if (out_of_bbox(pt, *p)) continue;
      world_to_index(pt, *p, G->reso, idx);
      const int i = int(std::floor(idx[0])), j = int(std::floor(idx[1])), kk = int(std::floor(idx[2]));
      const float u = idx[0] - float(i), v = idx[1] - float(j), w = idx[2] - float(kk);
      float sig = 0.f;
      for (int c = 0; c < 8; ++c) {
        const int* d = kCorner[c];
        const float a = d[0] ? u : 1.f - u, b = d[1] ? v : 1.f - v, cc = d[2] ? w : 1.f - w;
        sig = sig + ((dval(i + d[0], j + d[1], kk + d[2]) * a) * b) * cc;
      }
      float e;
      const float alpha = raw2alpha<float>(sig, p->act_shift, p->interval, e);
      if (!(alpha > p->fast_color_thres)) continue;
      ka.push_back(alpha);
      kw.push_back(Tc * alpha);
      kT.push_back(Tc);
      ksig.push_back(sig);
      kidx.push_back({idx[0], idx[1], idx[2]});
      Tc = trans_step<float>(Tc, alpha);
      if (Tc < p->t_stop) break;
    }
    const int nk = int(ka.size());
    // colour rows: k0 trilinear + MLP forward
    std::vector<int> rows;
    for (int q = 0; q < nk; ++q)
      if (kw[q] > p->fast_color_thres) rows.push_back(q);
    const int nr = int(rows.size());
    std::vector<float> x(size_t(nr) * din), h0(size_t(nr) * W), h1(size_t(nr) * W), rgb(size_t(nr) * 3);
    float pe[32];
    {
      const float* d = vd + 3 * r;
      pe[0] = d[0]; pe[1] = d[1]; pe[2] = d[2];
      for (int a = 0; a < 3; ++a)
        for (int q = 0; q < N->pe; ++q) {
          const float xx = d[a] * float(1 << q);
          pe[3 + a * N->pe + q] = std::sin(xx);
          pe[3 + 3 * N->pe + a * N->pe + q] = std::cos(xx);
        }
    }
    float rgbm[3] = {0.f, 0.f, 0.f};
    for (int m = 0; m < nr; ++m) {
      const auto& id3 = kidx[rows[m]];
      const int i = int(std::floor(id3[0])), j = int(std::floor(id3[1])), kk = int(std::floor(id3[2]));
      const float u = id3[0] - float(i), v = id3[1] - float(j), w = id3[2] - float(kk);
      float* xm = &x[size_t(m) * din];
      for (int c = 0; c < C; ++c) xm[c] = 0.f;
      for (int c = 0; c < 8; ++c) {
        const int* d = kCorner[c];
        const float a = d[0] ? u : 1.f - u, b = d[1] ? v : 1.f - v, cc = d[2] ? w : 1.f - w;
        const float sc = (a * b) * cc;
        const int ci = i + d[0], cj = j + d[1], ck = kk + d[2];
        if (!alloc_at(ci, cj, ck)) continue;
        const float* src = G->k0 + vid(ci, cj, ck) * C;
        for (int q = 0; q < C; ++q) xm[q] += src[q] * sc;
      }
      for (int q = 0; q < 3 + 6 * N->pe; ++q) xm[C + q] = pe[q];
      float* a0 = &h0[size_t(m) * W];
      float* a1 = &h1[size_t(m) * W];
      for (int n = 0; n < W; ++n) {
        float s = b0[n];
        for (int q = 0; q < din; ++q) s += w0[n * din + q] * xm[q];
        a0[n] = s > 0 ? s : 0.f;
      }
      for (int n = 0; n < W; ++n) {
        float s = b1[n];
        for (int q = 0; q < W; ++q) s += w1[n * W + q] * a0[q];
        a1[n] = s > 0 ? s : 0.f;
      }
      for (int c = 0; c < 3; ++c) {
        float s = b2[c];
        for (int q = 0; q < W; ++q) s += w2[c * W + q] * a1[q];
        rgb[m * 3 + c] = 1.f / (1.f + std::exp(-s));
        rgbm[c] += kw[rows[m]] * rgb[m * 3 + c];
      }
    }
    for (int c = 0; c < 3; ++c) rgbm[c] += Tc * p->bg;
    // losses and their gradients
    const float* t3 = target + 3 * r;
    float g3[3];
    for (int c = 0; c < 3; ++c) {
      const float e = rgbm[c] - t3[c];
      loss += double(w_main) * e * e / (3.0 * R);
      g3[c] = w_main * 2.f * e / (3.f * R);
    }
    const float pT = std::min(std::max(Tc, 1e-6f), 1.f - 1e-6f);
    loss += double(w_ent) * -(pT * std::log(pT) + (1 - pT) * std::log(1 - pT)) / R;
    float glast = p->bg * (g3[0] + g3[1] + g3[2]) +
                  ((Tc > 1e-6f && Tc < 1.f - 1e-6f) ? w_ent / R * std::log((1 - pT) / pT) : 0.f);
    std::vector<float> gw(nk, 0.f);
    std::vector<float> dh1(W), dh0(W);
    for (int m = 0; m < nr; ++m) {
      const int q = rows[m];
      float dl[3];
      float gwm = 0.f;
      for (int c = 0; c < 3; ++c) {
        const float y = rgb[m * 3 + c];
        gwm += g3[c] * y;
        const float dy = kw[q] * g3[c] + w_per * 2.f / R * kw[q] * (y - t3[c]);
        loss += double(w_per) * (y - t3[c]) * (y - t3[c]) * kw[q] / R;
        dl[c] = dy * y * (1 - y);
      }
      gw[q] = gwm;
      const float* a0 = &h0[size_t(m) * W];
      const float* a1 = &h1[size_t(m) * W];
      const float* xm = &x[size_t(m) * din];
      float* gw0 = tg;
      float* gb0 = gw0 + W * din;
      float* gw1 = gb0 + W;
      float* gb1 = gw1 + W * W;
      float* gw2 = gb1 + W;
      float* gb2 = gw2 + 3 * W;
      for (int c = 0; c < 3; ++c) {
        gb2[c] += dl[c];
        for (int n = 0; n < W; ++n) gw2[c * W + n] += dl[c] * a1[n];
      }
      for (int n = 0; n < W; ++n) {
        float s = 0;
        for (int c = 0; c < 3; ++c) s += dl[c] * w2[c * W + n];
        dh1[n] = a1[n] > 0 ? s : 0.f;
        gb1[n] += dh1[n];
      }
      for (int n = 0; n < W; ++n)
        if (dh1[n] != 0.f)
          for (int q2 = 0; q2 < W; ++q2) gw1[n * W + q2] += dh1[n] * a0[q2];
      for (int q2 = 0; q2 < W; ++q2) {
        float s = 0;
        for (int n = 0; n < W; ++n) s += dh1[n] * w1[n * W + q2];
        dh0[q2] = a0[q2] > 0 ? s : 0.f;
      }
      for (int n = 0; n < W; ++n) {
        gb0[n] += dh0[n];
        if (dh0[n] != 0.f)
          for (int q2 = 0; q2 < din; ++q2) gw0[n * din + q2] += dh0[n] * xm[q2];
      }
      // k0 gradient scatter
      float gk[16];
      for (int c = 0; c < C; ++c) {
        float s = 0;
        for (int n = 0; n < W; ++n) s += dh0[n] * w0[n * din + c];
        gk[c] = s;
      }
      const auto& id3 = kidx[q];
      const int i = int(std::floor(id3[0])), j = int(std::floor(id3[1])), kk = int(std::floor(id3[2]));
      const float u = id3[0] - float(i), v = id3[1] - float(j), w = id3[2] - float(kk);
      for (int c = 0; c < 8; ++c) {
        const int* d = kCorner[c];
        const int ci = i + d[0], cj = j + d[1], ck = kk + d[2];
        if (!alloc_at(ci, cj, ck)) continue;
        const float a = d[0] ? u : 1.f - u, b = d[1] ? v : 1.f - v, cc = d[2] ? w : 1.f - w;
        const float sc = (a * b) * cc;
        float* dst = G->gk0 + vid(ci, cj, ck) * C;
        for (int q2 = 0; q2 < C; ++q2) {
#pragma omp atomic
          dst[q2] += gk[q2] * sc;
        }
      }
    }
    // alpha2weight + raw2alpha backward and the density scatter
    float back = glast * Tc;
    for (int q = nk - 1; q >= 0; --q) {
      const float ga = alpha_grad<float>(gw[q], kT[q], back, ka[q]);
      back = std::fma(gw[q], kw[q], back);
      float e;
      (void)raw2alpha<float>(ksig[q], p->act_shift, p->interval, e);
      const float gs = raw2alpha_grad<float>(e, p->interval, ga);
      const auto& id3 = kidx[q];
      const int i = int(std::floor(id3[0])), j = int(std::floor(id3[1])), kk = int(std::floor(id3[2]));
      const float u = id3[0] - float(i), v = id3[1] - float(j), w = id3[2] - float(kk);
      for (int c = 0; c < 8; ++c) {
        const int* d = kCorner[c];
        const int ci = i + d[0], cj = j + d[1], ck = kk + d[2];
        if (!alloc_at(ci, cj, ck)) continue;
        const float a = d[0] ? u : 1.f - u, b = d[1] ? v : 1.f - v, cc = d[2] ? w : 1.f - w;
#pragma omp atomic
        G->gdens[vid(ci, cj, ck)] += ((gs * a) * b) * cc;
      }
    }
  }
  for (int t = 0; t < nth; ++t)
    for (int64_t q = 0; q < NP; ++q) N->grads[q] += tgrads[t][q];
  // TV (non-dense mode) on both grids
  if (tv_w > 0.f) {
    auto tv = [&](float* vals, float* grads, int ch, float bg) {
      std::vector<float> add(size_t(nvox) * ch, 0.f);
#pragma omp parallel for schedule(static)
      for (int64_t q = 0; q < nvox; ++q) {
        const int i = int(q / (int64_t(P1) * P2)), j = int((q / P2) % P1), k = int(q % P2);
        if (i >= G->reso[0] || j >= G->reso[1] || k >= G->reso[2]) continue;
        if (!alloc_at(i, j, k) || !G->active[q]) continue;
        for (int c = 0; c < ch; ++c) {
          if (grads[q * ch + c] == 0.f) continue;
          const float pv = vals[q * ch + c];
          auto nb = [&](int a, int b, int cc) {
            return alloc_at(a, b, cc) ? vals[vid(a, b, cc) * ch + c] : bg;
          };
          auto cl = [](float x) { return std::min(std::max(x, -1.f), 1.f); };
          float s = 0.f;
          if (k > 0) s += tv_w * cl(pv - nb(i, j, k - 1));
          if (k < G->reso[2] - 1) s += tv_w * cl(pv - nb(i, j, k + 1));
          if (j > 0) s += tv_w * cl(pv - nb(i, j - 1, k));
          if (j < G->reso[1] - 1) s += tv_w * cl(pv - nb(i, j + 1, k));
          if (i > 0) s += tv_w * cl(pv - nb(i - 1, j, k));
          if (i < G->reso[0] - 1) s += tv_w * cl(pv - nb(i + 1, j, k));
          add[q * ch + c] = s;
        }
      }
      for (int64_t q = 0; q < nvox * ch; ++q) grads[q] += add[q];
    };
    tv(G->dens, G->gdens, 1, G->background);
    tv(G->k0, G->gk0, C, 0.f);
  }
  // voxel Adam (mode 1) on both grids, zeroing the gradient afterwards
  G->step += 1;
  const float b0f = 0.9f, b1f = 0.99f, eps = 1e-8f;
  const float sd = G->lr_d * std::sqrt(1 - std::pow(b1f, (float)G->step)) / (1 - std::pow(b0f, (float)G->step));
  const float sk = G->lr_k * std::sqrt(1 - std::pow(b1f, (float)G->step)) / (1 - std::pow(b0f, (float)G->step));
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < nvox; ++q) {
    const int i = int(q / (int64_t(P1) * P2)), j = int((q / P2) % P1), k = int(q % P2);
    if (!alloc_at(i, j, k) || !G->active[q]) continue;
    const float g = G->gdens[q];
    if (g != 0.f) {
      G->m_d[q] = b0f * G->m_d[q] + (1 - b0f) * g;
      G->v_d[q] = b1f * G->v_d[q] + (1 - b1f) * g * g;
      G->dens[q] -= sd * G->m_d[q] / (eps + std::sqrt(G->v_d[q]));
      G->gdens[q] = 0.f;
    }
    for (int grp = 0; grp < C / 3; ++grp) {
      float* gg = G->gk0 + q * C + 3 * grp;
      if (gg[0] == 0.f && gg[1] == 0.f && gg[2] == 0.f) continue;
      for (int c = 0; c < 3; ++c) {
        const int64_t o = q * C + 3 * grp + c;
        G->m_k[o] = b0f * G->m_k[o] + (1 - b0f) * gg[c];
        G->v_k[o] = b1f * G->v_k[o] + (1 - b1f) * gg[c] * gg[c];
        G->k0[o] -= sk * G->m_k[o] / (eps + std::sqrt(G->v_k[o]));
        gg[c] = 0.f;
      }
    }
  }
  G->lr_d *= float(std::pow(0.1, 1.0 / 20000.0));
  G->lr_k *= float(std::pow(0.1, 1.0 / 20000.0));
  // rgbnet Adam (mode 0)
  N->step += 1;
  const float sn = N->lr * std::sqrt(1 - std::pow(0.99f, (float)N->step)) / (1 - std::pow(0.9f, (float)N->step));
  for (int64_t q = 0; q < NP; ++q) {
    const float g = N->grads[q];
    N->m[q] = 0.9f * N->m[q] + 0.1f * g;
    N->v[q] = 0.99f * N->v[q] + 0.01f * g * g;
    N->params[q] -= sn * N->m[q] / (std::sqrt(N->v[q]) + 1e-8f);
  }
  N->lr *= float(std::pow(0.1, 1.0 / 20000.0));
  return loss;
}

// Density-only forward + backward in FP32 on the host cores (the plain
// density-only configuration): the march of dvgo.py:296-335 without colour
// (density trilinear, raw2alpha, alpha2weight with the T < t_stop stop), the
// composited alpha 1 - alphainv_last, the loss mean((alpha - target)^2) over
// the rays, and its gradient through alpha2weight_backward (:653-677),
// raw2alpha_backward (:506-517) and the density scatter (densityvdb.cu:16-27,
// 143-167; float atomics as the reference's kernel) into G->gdens. No
// optimiser step. Returns the loss.
double oracle_density_step_fp32(otrain_grids* G, const float* ro, const float* rd,
                                const float* target_alpha, int R, const omarch_params* p) {
  const int P1 = G->pad[1], P2 = G->pad[2];
  auto alloc_at = [&](int i, int j, int k) {
    if (i < 0 || j < 0 || k < 0 || i >= G->pad[0] || j >= P1 || k >= P2) return false;
    return G->alloc[((i >> 3) * (P1 / 8) + (j >> 3)) * (P2 / 8) + (k >> 3)] != 0;
  };
  auto vid = [&](int i, int j, int k) { return (int64_t(i) * P1 + j) * P2 + k; };
  auto dval = [&](int i, int j, int k) { return alloc_at(i, j, k) ? G->dens[vid(i, j, k)] : G->background; };
  double loss = 0;
#pragma omp parallel for schedule(dynamic, 8) reduction(+ : loss)
  for (int r = 0; r < R; ++r) {
    Ray ray;
    ray_setup(ro + 3 * r, rd + 3 * r, *p, ray);
    std::vector<float> ka, kT, ksig;
    std::vector<std::array<float, 3>> kidx;
    float Tc = 1.f;
    for (int64_t k = 0; k < ray.n_steps; ++k) {
      float pt[3], idx[3];
      ray_point(ray, p->stepdist, k, pt);
      if (out_of_bbox(pt, *p)) continue;
      world_to_index(pt, *p, G->reso, idx);
      const int i = int(std::floor(idx[0])), j = int(std::floor(idx[1])), kk = int(std::floor(idx[2]));
      const float u = idx[0] - float(i), v = idx[1] - float(j), w = idx[2] - float(kk);
      float sig = 0.f;
      for (int c = 0; c < 8; ++c) {
        const int* d = kCorner[c];
        const float a = d[0] ? u : 1.f - u, b = d[1] ? v : 1.f - v, cc = d[2] ? w : 1.f - w;
        sig = sig + ((dval(i + d[0], j + d[1], kk + d[2]) * a) * b) * cc;
      }
      float e;
      const float alpha = raw2alpha<float>(sig, p->act_shift, p->interval, e);
      if (!(alpha > p->fast_color_thres)) continue;
      ka.push_back(alpha);
      kT.push_back(Tc);
      ksig.push_back(sig);
      kidx.push_back({idx[0], idx[1], idx[2]});
      Tc = trans_step<float>(Tc, alpha);
      if (Tc < p->t_stop) break;
    }
    const float err = (1.f - Tc) - target_alpha[r];
    loss += double(err) * err / R;
    // d loss / d alphainv_last; the weights carry no gradient
    float back = (-2.f * err / float(R)) * Tc;
    for (int q = int(ka.size()) - 1; q >= 0; --q) {
      const float ga = alpha_grad<float>(0.f, kT[q], back, ka[q]);
      float e;
      (void)raw2alpha<float>(ksig[q], p->act_shift, p->interval, e);
      const float gs = raw2alpha_grad<float>(e, p->interval, ga);
      const auto& id3 = kidx[q];
      const int i = int(std::floor(id3[0])), j = int(std::floor(id3[1])), kk = int(std::floor(id3[2]));
      const float u = id3[0] - float(i), v = id3[1] - float(j), w = id3[2] - float(kk);
      for (int c = 0; c < 8; ++c) {
        const int* d = kCorner[c];
        const int ci = i + d[0], cj = j + d[1], ck = kk + d[2];
        if (!alloc_at(ci, cj, ck)) continue;
        const float a = d[0] ? u : 1.f - u, b = d[1] ? v : 1.f - v, cc = d[2] ? w : 1.f - w;
#pragma omp atomic
        G->gdens[vid(ci, cj, ck)] += ((gs * a) * b) * cc;
      }
    }
  }
  return loss;
}

}  // extern "C"

// ------------------------------------------------ merged-index renderer
// MGRenderer::render_an_image (plenvdb.h:1010-1060 -> renderer.cu:370-412) for a
// list of pixels. The index grid is a dense row-id array (0 = empty row, the
// voxels with a row id are the active ones); rows beyond the grid read row 0.
//   get_rays / get_tminmax      renderer.cu:122-167, 50-64 (unit-cube frame,
//                               float arithmetic, contractions written as fma)
//   march                       renderer.cu:227-266 (t += steplen before each
//                               sample, isActive(Round(xyz)), thresholds on
//                               alpha and weight, stop once T < t_stop)
//   trigetDensity2/trigetColor  renderer.cu:271-317 (int() truncation, corner
//                               scales first, then the fma chain over corners)
//   cuda_rgbnet                 renderer.cu:83-110 ([k0 | PE(viewdir)] -> 128
//                               ReLU -> 128 ReLU -> 3)
//   final_render + last_rgb     renderer.cu:112-119, 360-362 (T*bg plus
//                               w/(1+exp(-logit)) in sample order; bg alone
//                               for a pixel without a colour sample, :325-329)
// The reference marches every pixel twice (count, then fill) and restarts the
// fill pass from t_first - steplen, which can shift the fill pass's sample
// positions by an ulp; this restatement uses one march for both, with the
// fill pass's density association. fp32 mirrors the float operations; fp64
// forms the positions in float as the reference does and evaluates density,
// alpha, transmittance, features, the MLP and the composite in double.
extern "C" {

typedef struct {
  int H, W, inverse_y;
  int reso[3];
  float K[9];
  float c2w[16];
  float xyz_min[3], xyz_max[3];
  float near_, stepdist, shift, interval, thr, bg, t_stop;
} orender_params;

}  // extern "C"

namespace {

// The merged index grid: row id of voxel (i,j,k), 0 outside the grid.
struct IndexGrid {
  int r0, r1, r2;
  const int32_t* index;
  int32_t row(int i, int j, int k) const {
    if (i < 0 || j < 0 || k < 0 || i >= r0 || j >= r1 || k >= r2) return 0;
    return index[(int64_t(i) * r1 + j) * r2 + k];
  }
  // isActive(Round(xyz)) (renderer.cu:253): the voxels with a row are active
  bool active_round(const float* xyz) const {
    return row(int(std::nearbyint(xyz[0])), int(std::nearbyint(xyz[1])),
               int(std::nearbyint(xyz[2]))) > 0;
  }
  // trigetDensity2 corner rows and scales (renderer.cu:271-300); returns the
  // density, fp32: scales first, then the fma chain over the corners
  template <class T>
  T density(const float* xyz, const float* den, int32_t id[8], T sc[8]) const {
    const int i = int(xyz[0]), j = int(xyz[1]), k = int(xyz[2]);
    const float u = xyz[0] - float(i), v = xyz[1] - float(j), w = xyz[2] - float(k);
    id[0] = row(i, j, k);         id[1] = row(i, j, k + 1);
    id[2] = row(i, j + 1, k + 1); id[3] = row(i, j + 1, k);
    id[4] = row(i + 1, j + 1, k); id[5] = row(i + 1, j + 1, k + 1);
    id[6] = row(i + 1, j, k + 1); id[7] = row(i + 1, j, k);
    const T U = u, V = v, Wt = w, iu = T(1) - U, iv = T(1) - V, iw = T(1) - Wt;
    sc[0] = (iu * iv) * iw; sc[1] = (iu * iv) * Wt; sc[2] = (iu * V) * Wt; sc[3] = (iu * V) * iw;
    sc[4] = (U * V) * iw;   sc[5] = (U * V) * Wt;   sc[6] = (U * iv) * Wt; sc[7] = (U * iv) * iw;
    T sig = T(den[id[0]]) * sc[0];
    for (int c = 1; c < 8; ++c) {
      if constexpr (sizeof(T) == 4) sig = std::fma(den[id[c]], sc[c], sig);
      else sig += T(den[id[c]]) * sc[c];
    }
    return sig;
  }
};

template <class T>
void render_pixel(const orender_params& P, const int32_t* index, const float* den,
                  const float* col, int dcol, const MlpT<T>& mlp, int64_t n, double* rgb_out,
                  int32_t* ncol_out, double* T_out) {
  const IndexGrid ig{P.reso[0], P.reso[1], P.reso[2], index};
  const int r0 = P.reso[0], r1 = P.reso[1], r2 = P.reso[2];
  const float pi = float(n % P.W) + 0.5f, pj = float(n / P.W) + 0.5f;
  float dir[3];
  dir[0] = (pi - P.K[2]) / P.K[0];
  if (P.inverse_y) {
    dir[1] = (pj - P.K[5]) / P.K[4];
    dir[2] = 1.f;
  } else {
    dir[1] = -((pj - P.K[5]) / P.K[4]);
    dir[2] = -1.f;
  }
  float rd[3];
  for (int a = 0; a < 3; ++a)
    rd[a] = std::fma(dir[2], P.c2w[4 * a + 2], std::fma(dir[1], P.c2w[4 * a + 1], dir[0] * P.c2w[4 * a]));
  const float len = std::sqrt(std::fma(rd[2], rd[2], std::fma(rd[1], rd[1], rd[0] * rd[0])));
  const float steplen = P.stepdist / len;
  float o[3], d[3], vd[3];
  for (int a = 0; a < 3; ++a) {
    const float ext = P.xyz_max[a] - P.xyz_min[a];
    o[a] = (P.c2w[4 * a + 3] - P.xyz_min[a]) / ext;
    d[a] = rd[a] / ext;
    vd[a] = rd[a] / len;
  }
  const float vx = d[0] == 0.f ? float(1e-6) : d[0];
  const float vy = d[1] == 0.f ? float(1e-6) : d[1];
  const float vz = d[2] == 0.f ? float(1e-6) : d[2];
  const float ax = (1.f - o[0]) / vx, ay = (1.f - o[1]) / vy, az = (1.f - o[2]) / vz;
  const float bx = (-o[0]) / vx, by = (-o[1]) / vy, bz = (-o[2]) / vz;
  const float far_ = 1e9f;
  const float tmin = std::max(std::min(std::max(std::max(std::min(ax, bx), std::min(ay, by)), std::min(az, bz)), far_), P.near_);
  const float tmax = std::max(std::min(std::min(std::min(std::max(ax, bx), std::max(ay, by)), std::max(az, bz)), far_), P.near_);
  const float wsm1[3] = {float(r0 - 1), float(r1 - 1), float(r2 - 1)};
  // PE of the view direction, shared by the pixel's colour samples
  const int npe = mlp.pe;
  std::vector<T> x(size_t(dcol) + 3 + 6 * npe), h0(mlp.W), h1(mlp.W);
  view_pe<T>(vd, npe, x.data() + dcol);
  T Tc = 1;
  std::vector<T> terms;  // w/(1+exp(-logit)) of each colour sample, 3 per sample
  int32_t cnt = 0;
  float t = tmin;
  const float nsteps_f = (tmax - tmin) / steplen;
  const int max_it = (nsteps_f > 0.f && nsteps_f < 1e6f) ? int(nsteps_f) + 4 : 0;
  for (int it = 0; t < tmax && it < max_it; ++it) {
    t = t + steplen;
    float p[3];
    for (int a = 0; a < 3; ++a) p[a] = std::fma(t, d[a], o[a]);
    if ((0.f > p[0]) | (0.f > p[1]) | (0.f > p[2]) | (1.f < p[0]) | (1.f < p[1]) | (1.f < p[2]))
      continue;
    float xyz[3];
    for (int a = 0; a < 3; ++a) xyz[a] = p[a] * wsm1[a];
    if (!ig.active_round(xyz)) continue;
    int32_t id[8];
    T sc[8];
    const T sig = ig.density<T>(xyz, den, id, sc);
    T alpha;
    if constexpr (sizeof(T) == 4) alpha = 1.f - std::pow(1.f + std::exp(sig + P.shift), -P.interval);
    else alpha = 1.0 - std::pow(1.0 + std::exp(sig + double(P.shift)), -double(P.interval));
    if (alpha <= T(P.thr)) continue;
    const T wt = Tc * alpha;
    Tc = Tc * (T(1) - alpha);
    if (wt <= T(P.thr)) continue;
    for (int q = 0; q < dcol; ++q) {
      T f = T(col[int64_t(id[0]) * dcol + q]) * sc[0];
      for (int c = 1; c < 8; ++c) {
        if constexpr (sizeof(T) == 4) f = std::fma(col[int64_t(id[c]) * dcol + q], sc[c], f);
        else f += T(col[int64_t(id[c]) * dcol + q]) * sc[c];
      }
      x[q] = f;
    }
    T logit[3];
    mlp_forward<T>(mlp, x.data(), h0.data(), h1.data(), logit);
    for (int c = 0; c < 3; ++c) terms.push_back(wt / (T(1) + std::exp(-logit[c])));
    ++cnt;
    const bool stop = sizeof(T) == 4 ? (float(Tc) < P.t_stop) : (double(Tc) < double(P.t_stop));
    if (stop) break;
  }
  ncol_out[0] = cnt;
  T_out[0] = double(Tc);
  for (int c = 0; c < 3; ++c) {
    if (cnt == 0) {
      rgb_out[c] = P.bg;
      continue;
    }
    T s = Tc * T(P.bg);
    for (int32_t q = 0; q < cnt; ++q) s += terms[size_t(q) * 3 + c];
    rgb_out[c] = double(s);
  }
}

}  // namespace

extern "C" {

// Index-grid density and isActive(Round(xyz)) at index-space points (the
// render march's per-sample lookups).
void oracle_index_density(const int32_t* reso, const int32_t* index, const float* den,
                          const float* xyz, int64_t n, int fp32, double* out, uint8_t* active) {
  const IndexGrid ig{reso[0], reso[1], reso[2], index};
  for (int64_t q = 0; q < n; ++q) {
    int32_t id[8];
    active[q] = ig.active_round(xyz + 3 * q) ? 1 : 0;
    if (fp32) {
      float sc[8];
      out[q] = ig.density<float>(xyz + 3 * q, den, id, sc);
    } else {
      double sc[8];
      out[q] = ig.density<double>(xyz + 3 * q, den, id, sc);
    }
  }
}

void oracle_render_pixels(const orender_params* P, const int32_t* index, const float* den,
                          const float* col, int dcol, const omlp* mw, const int64_t* pix,
                          int64_t npix, int fp32, double* rgb, int32_t* n_color, double* T_last) {
  if (fp32) {
    const MlpT<float> m(*mw);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t q = 0; q < npix; ++q)
      render_pixel<float>(*P, index, den, col, dcol, m, pix[q], rgb + 3 * q, n_color + q, T_last + q);
  } else {
    const MlpT<double> m(*mw);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t q = 0; q < npix; ++q)
      render_pixel<double>(*P, index, den, col, dcol, m, pix[q], rgb + 3 * q, n_color + q, T_last + q);
  }
}

}  // extern "C"
