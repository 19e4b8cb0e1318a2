// Merged-VDB renderer (MGRenderer, plenvdb.h:933-1068; renderer.cu:122-424).
//
// Data: an index leaf store (voxel -> row id, 0 = empty; the voxels with a row
// are the active ones) plus per-row density and k0 features (FP32, or BF16
// features with FP32 density).
//
// Per frame:
//   k_render_march<COUNT>  one thread per pixel: get_rays (renderer.cu:122-167)
//                          in the unit-cube frame, t += steplen before each
//                          sample, skip when isActive(rint(xyz)) is false,
//                          index-grid trilinear density (int() truncation,
//                          renderer.cu:271-300), raw2alpha, both thresholds,
//                          early stop at a colour sample once T < t_stop
//                          (renderer.cu:240-266); counts colour samples
//   device scan            per-pixel row offsets
//   k_render_march<FILL>   the same march, writing each colour sample's k0 row
//                          (renderer.cu:303-310) and weight
//   rgbnet                 the MLP on all rows (PE part once per pixel)
//   k_render_composite     per pixel: T*bg + sum_rows w/(1+exp(-logit)) in
//                          sample order (final_render renderer.cu:112-119,
//                          deterministic instead of atomics); bg alone when the
//                          pixel has no colour sample (renderer.cu:325-329).
// The reference runs the march twice with slightly different float
// associations in the two passes; here both passes share one code path, so the
// fill pass reproduces the count pass exactly.
#include <cmath>
#include <cstring>
#include <vector>

#include "pvdb_internal.cuh"
#include "tc.cuh"

namespace pvdb {

struct MlpArgs {
  const float* w0; const float* b0;
  const float* w1; const float* b1;
  const float* w2; const float* b2;
  int c0, dpe, din;
};
int mlp_forward_rows(const MlpArgs& a, const float* k0rows, const int32_t* ray,
                     const float* viewdirs, int R, const uint32_t* totals, int64_t max_rows,
                     float* out, int out_logits, float* hpe_buf, int precision, void** blob,
                     size_t* blob_cap, void** xt, size_t* xt_cap, uint32_t* err,
                     cudaStream_t st, int x_ready);
int mlp_pe_rows(const MlpArgs& a, const float* viewdirs, int R, float* hpe_buf, int* pe_stride,
                cudaStream_t st);

struct RenderP {
  int H, W, inverse_y;
  float K[9];
  float c2w[16];
  float mn[3], mx[3];
  float wsm1[3];
  float near_, far_, stepdist, shift, interval, thr, bg, t_stop;
  int dcol;
  // index store
  GridView idx;            // topology; values unused
  const int32_t* rows;     // [nleaf*512] row id of every in-leaf voxel
  const float* den;        // [N]
  const float* col;        // [N*dcol] (storage 0)
  const __nv_bfloat16* colh;  // [N*dcol] (storage 1)
  int storage;
};

struct RenderW {
  uint32_t* n;       // [HW] colour samples per pixel
  uint32_t* off;     // [HW]
  float* T;          // [HW]
  float* viewdirs;   // [HW*3]
  float* rk0;        // [cap*dcol]
  float* rw;         // [cap]
  int32_t* rpix;     // [cap]
  uint32_t* totals;  // [0] unused, [1] total rows
  int64_t cap;
  // BF16 rgbnet: the fill pass writes each colour sample's rgbnet input row
  // ([k0 | PE | 1 | 0], BF16) into the X tiles instead of the FP32 k0 row
  uint8_t* xt;       // [ceil(cap/128)] tiles, or NULL
  const float* pe;   // [HW][pe_stride] per-pixel PE
  int pe_stride, dpe;
};

__device__ __forceinline__ int32_t row_at(const RenderP& P, int i, int j, int k) {
  const int s = slot_of(P.idx, i, j, k);
  return s < 0 ? 0 : __ldg(P.rows + s);
}

__device__ __forceinline__ bool index_active(const RenderP& P, int i, int j, int k) {
  const int l = leaf_of(P.idx, i, j, k);
  if (l < 0) return false;
  const int v = vox_offset(i, j, k);
  return (__ldg(P.idx.mask + l * 8 + (v >> 6)) >> (v & 63)) & 1ull;
}

// 12-channel rows (the reference's k0): three float4, or three 8-byte BF16
// quads per corner.
__device__ __forceinline__ void fill_features12(const RenderP& P, const int32_t id[8],
                                                const float sc[8], float acc[12]) {
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    float v[12];
    if (P.storage == 0) {
      const float4* src = reinterpret_cast<const float4*>(P.col + int64_t(id[c]) * 12);
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const float4 f = __ldg(src + b);
        v[4 * b] = f.x; v[4 * b + 1] = f.y; v[4 * b + 2] = f.z; v[4 * b + 3] = f.w;
      }
    } else {
      const uint2* src = reinterpret_cast<const uint2*>(P.colh + int64_t(id[c]) * 12);
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const uint2 h = __ldg(src + b);
        v[4 * b] = __uint_as_float(h.x << 16);
        v[4 * b + 1] = __uint_as_float(h.x & 0xFFFF0000u);
        v[4 * b + 2] = __uint_as_float(h.y << 16);
        v[4 * b + 3] = __uint_as_float(h.y & 0xFFFF0000u);
      }
    }
#pragma unroll
    for (int q = 0; q < 12; ++q)
      acc[q] = c == 0 ? __fmul_rn(v[q], sc[0]) : __fmaf_rn(v[q], sc[c], acc[q]);
  }
}

// Trilinear features of a colour sample (trigetColor, renderer.cu:303-310):
// per channel c0*s0, then the fma chain over corners 1..7. 12-channel rows are
// read with vector loads (three float4, or three 8-byte BF16 quads).
__device__ __forceinline__ void fill_features(const RenderP& P, const int32_t id[8],
                                              const float sc[8], float acc[16]) {
  if (P.dcol == 12) {
    fill_features12(P, id, sc, acc);
    return;
  }
  for (int q = 0; q < P.dcol; ++q) {
    float a;
    if (P.storage == 0) {
      a = __fmul_rn(__ldg(P.col + int64_t(id[0]) * P.dcol + q), sc[0]);
      for (int c = 1; c < 8; ++c) a = __fmaf_rn(__ldg(P.col + int64_t(id[c]) * P.dcol + q), sc[c], a);
    } else {
      a = __fmul_rn(__bfloat162float(P.colh[int64_t(id[0]) * P.dcol + q]), sc[0]);
      for (int c = 1; c < 8; ++c)
        a = __fmaf_rn(__bfloat162float(P.colh[int64_t(id[c]) * P.dcol + q]), sc[c], a);
    }
    acc[q] = a;
  }
}

// 12 k0 channels and 27 PE values (the rgbnet of the reference): the row is
// 2 k0 chunks, the first of which carries PE 0..3, then pixel-constant chunks.
__device__ __forceinline__ void write_x_row12(const RenderW& Wk, int64_t m, const float* k0v,
                                              const uint4* pe_chunks) {
  uint8_t* tile = Wk.xt + (m >> 7) * int64_t(kRgbXTile);
  const int row = int(m & 127);
  const uint4 c0 = make_uint4(tc::pack_bf16(k0v[0], k0v[1]), tc::pack_bf16(k0v[2], k0v[3]),
                              tc::pack_bf16(k0v[4], k0v[5]), tc::pack_bf16(k0v[6], k0v[7]));
  const uint4 c1 = make_uint4(tc::pack_bf16(k0v[8], k0v[9]), tc::pack_bf16(k0v[10], k0v[11]),
                              pe_chunks[0].z, pe_chunks[0].w);
  *reinterpret_cast<uint4*>(tile + tc::kmaj(row, 0, kRgbXK)) = c0;
  *reinterpret_cast<uint4*>(tile + tc::kmaj(row, 8, kRgbXK)) = c1;
#pragma unroll
  for (int cb = 2; cb < 6; ++cb)
    *reinterpret_cast<uint4*>(tile + tc::kmaj(row, 8 * cb, kRgbXK)) = pe_chunks[cb - 1];
}

// The BF16 X row m of pixel n: [k0 (dcol) | PE (dpe) | 1 | 0 ...] in the
// canonical K-major tile layout; pe_bits holds the pixel's PE as BF16 pairs.
__device__ __forceinline__ void write_x_row(const RenderW& Wk, int64_t m, int n,
                                            const float* k0v, int dcol, const uint32_t* pe_bits) {
  uint8_t* tile = Wk.xt + (m >> 7) * int64_t(kRgbXTile);
  const int row = int(m & 127);
  const int din = dcol + Wk.dpe;
#pragma unroll
  for (int cb = 0; cb < kRgbXK / 8; ++cb) {
    uint32_t w4[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      float v2[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int q = 8 * cb + 2 * e + h;
        v2[h] = q < dcol ? k0v[q < 16 ? q : 15] : q == din ? 1.f : 0.f;
      }
      uint32_t bits = tc::pack_bf16(v2[0], v2[1]);
      // PE columns come pre-rounded from pe_bits
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int q = 8 * cb + 2 * e + h;
        if (q >= dcol && q < din) {
          const int pq = q - dcol;
          const uint32_t pb = (pe_bits[pq >> 1] >> (16 * (pq & 1))) & 0xFFFFu;
          bits = h == 0 ? ((bits & 0xFFFF0000u) | pb) : ((bits & 0x0000FFFFu) | (pb << 16));
        }
      }
      w4[e] = bits;
    }
    *reinterpret_cast<uint4*>(tile + tc::kmaj(row, 8 * cb, kRgbXK)) =
        make_uint4(w4[0], w4[1], w4[2], w4[3]);
  }
  (void)n;
}

template <bool FILL>
__global__ void __launch_bounds__(128)
    k_render_march(RenderP P, RenderW Wk) {
  const int HW = P.H * P.W;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= HW) return;
  // get_rays (renderer.cu:134-151)
  const float pi = float(n % P.W) + 0.5f, pj = float(n / P.W) + 0.5f;
  float dir[3];
  dir[0] = __fdiv_rn(pi - P.K[2], P.K[0]);
  if (P.inverse_y) {
    dir[1] = __fdiv_rn(pj - P.K[5], P.K[4]);
    dir[2] = 1.f;
  } else {
    dir[1] = -__fdiv_rn(pj - P.K[5], P.K[4]);
    dir[2] = -1.f;
  }
  float rd[3];
  for (int a = 0; a < 3; ++a)
    rd[a] = __fmaf_rn(dir[2], P.c2w[4 * a + 2], __fmaf_rn(dir[1], P.c2w[4 * a + 1],
                                                          __fmul_rn(dir[0], P.c2w[4 * a])));
  const float len = sqrtf(__fmaf_rn(rd[2], rd[2], __fmaf_rn(rd[1], rd[1], __fmul_rn(rd[0], rd[0]))));
  const float steplen = __fdiv_rn(P.stepdist, len);
  float o[3], d[3];
  for (int a = 0; a < 3; ++a) {
    const float ext = P.mx[a] - P.mn[a];
    o[a] = __fdiv_rn(P.c2w[4 * a + 3] - P.mn[a], ext);
    d[a] = __fdiv_rn(rd[a], ext);
  }
  if (!FILL) {
    for (int a = 0; a < 3; ++a) Wk.viewdirs[n * 3 + a] = __fdiv_rn(rd[a], len);
  }
  // get_tminmax against the unit cube (renderer.cu:50-64)
  const float vx = d[0] == 0.f ? float(1e-6) : d[0];
  const float vy = d[1] == 0.f ? float(1e-6) : d[1];
  const float vz = d[2] == 0.f ? float(1e-6) : d[2];
  const float ax = __fdiv_rn(1.f - o[0], vx), ay = __fdiv_rn(1.f - o[1], vy), az = __fdiv_rn(1.f - o[2], vz);
  const float bx = __fdiv_rn(-o[0], vx), by = __fdiv_rn(-o[1], vy), bz = __fdiv_rn(-o[2], vz);
  const float tmin = fmaxf(fminf(fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fminf(az, bz)), P.far_), P.near_);
  const float tmax = fmaxf(fminf(fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fmaxf(az, bz)), P.far_), P.near_);
  float T = 1.f;
  uint32_t cnt = 0;
  const int64_t base = FILL ? int64_t(Wk.off[n]) : 0;
  // BF16 fill: the pixel's PE, rounded to BF16 once — for 12 k0 channels and
  // 27 PE values as the pixel-constant part of its X rows (pe_chunks[0].zw =
  // PE 0..3, pe_chunks[1..4] = columns 16..47), else as BF16 pairs
  const bool fast12 = FILL && Wk.xt && P.dcol == 12 && Wk.dpe == 27;
  uint4 pe_chunks[5];
  uint32_t pe_bits[16];
  if (fast12) {
    const float* pp = Wk.pe + int64_t(n) * Wk.pe_stride;
    float pv[27];
#pragma unroll
    for (int q = 0; q < 27; ++q) pv[q] = pp[q];
    pe_chunks[0] = make_uint4(0u, 0u, tc::pack_bf16(pv[0], pv[1]), tc::pack_bf16(pv[2], pv[3]));
#pragma unroll
    for (int cb = 2; cb < 5; ++cb) {  // columns 8cb .. 8cb+7 = PE 8cb-12 ..
      uint32_t w4[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int p0 = 8 * cb - 12 + 2 * e, p1 = p0 + 1;
        const float a0 = p0 < 27 ? pv[p0 < 27 ? p0 : 0] : (p0 == 27 ? 1.f : 0.f);
        const float a1 = p1 < 27 ? pv[p1 < 27 ? p1 : 0] : (p1 == 27 ? 1.f : 0.f);
        w4[e] = tc::pack_bf16(a0, a1);
      }
      pe_chunks[cb - 1] = make_uint4(w4[0], w4[1], w4[2], w4[3]);
    }
    pe_chunks[4] = make_uint4(0u, 0u, 0u, 0u);
  } else if (FILL && Wk.xt) {
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int q0 = 2 * i, q1 = 2 * i + 1;
      const float a0 = q0 < Wk.dpe ? Wk.pe[int64_t(n) * Wk.pe_stride + q0] : 0.f;
      const float a1 = q1 < Wk.dpe ? Wk.pe[int64_t(n) * Wk.pe_stride + q1] : 0.f;
      pe_bits[i] = tc::pack_bf16(a0, a1);
    }
  }
  if (FILL && Wk.xt) {
    // the padding rows of the last tile are zero (block 0 writes them)
    if (blockIdx.x == 0) {
      const int64_t M = Wk.totals[1], Mpad = (M + 127) / 128 * 128;
      const int64_t mz = M + threadIdx.x;
      if (mz < Mpad) {  // Mpad <= the tiles reserved for cap rows
        uint8_t* tile = Wk.xt + (mz >> 7) * int64_t(kRgbXTile);
        for (int cb = 0; cb < kRgbXK / 8; ++cb)
          *reinterpret_cast<uint4*>(tile + tc::kmaj(int(mz & 127), 8 * cb, kRgbXK)) =
              make_uint4(0u, 0u, 0u, 0u);
      }
    }
  }
  float t = tmin;
  // the reference loops while t < tmax; the iteration bound (the sample count
  // of the [tmin,tmax] chord plus slack) only guards against a step that no
  // longer advances t (non-finite or vanishing steplen)
  const float nsteps_f = (tmax - tmin) / steplen;
  const int max_it = (nsteps_f > 0.f && nsteps_f < 1e6f) ? int(nsteps_f) + 4 : 0;
  for (int it = 0; t < tmax && it < max_it; ++it) {
    t = __fadd_rn(t, steplen);
    float p[3];
    for (int a = 0; a < 3; ++a) p[a] = __fmaf_rn(t, d[a], o[a]);
    if ((0.f > p[0]) | (0.f > p[1]) | (0.f > p[2]) | (1.f < p[0]) | (1.f < p[1]) | (1.f < p[2]))
      continue;
    float xyz[3];
    for (int a = 0; a < 3; ++a) xyz[a] = __fmul_rn(p[a], P.wsm1[a]);
    if (!index_active(P, __float2int_rn(xyz[0]), __float2int_rn(xyz[1]), __float2int_rn(xyz[2])))
      continue;
    // trigetDensity2 (renderer.cu:271-300): int() truncation, scales then sum
    const int i = int(xyz[0]), j = int(xyz[1]), k = int(xyz[2]);
    const float u = xyz[0] - float(i), v = xyz[1] - float(j), w = xyz[2] - float(k);
    int32_t id[8];
    id[0] = row_at(P, i, j, k);
    id[1] = row_at(P, i, j, k + 1);
    id[2] = row_at(P, i, j + 1, k + 1);
    id[3] = row_at(P, i, j + 1, k);
    id[4] = row_at(P, i + 1, j + 1, k);
    id[5] = row_at(P, i + 1, j + 1, k + 1);
    id[6] = row_at(P, i + 1, j, k + 1);
    id[7] = row_at(P, i + 1, j, k);
    float sc[8];
    corner_scales(u, v, w, sc);
    float sig = __fmul_rn(__ldg(P.den + id[0]), sc[0]);
    for (int c = 1; c < 8; ++c) sig = __fmaf_rn(__ldg(P.den + id[c]), sc[c], sig);
    const float alpha = 1.f - powf(1.f + expf(sig + P.shift), -P.interval);
    if (alpha <= P.thr) continue;
    const float wt = T * alpha;
    T = T * (1.f - alpha);
    if (wt <= P.thr) continue;
    if (FILL) {
      const int64_t m = base + cnt;
      if (m < Wk.cap) {
        if (Wk.xt && fast12) {
          float acc[12];
          fill_features12(P, id, sc, acc);
          write_x_row12(Wk, m, acc, pe_chunks);
        } else if (Wk.xt) {
          float acc[16];
          fill_features(P, id, sc, acc);
          write_x_row(Wk, m, n, acc, P.dcol, pe_bits);
        } else if (P.dcol == 12) {
          float acc[12];
          fill_features12(P, id, sc, acc);
          float4* dst = reinterpret_cast<float4*>(Wk.rk0 + m * 12);
#pragma unroll
          for (int b = 0; b < 3; ++b)
            dst[b] = make_float4(acc[4 * b], acc[4 * b + 1], acc[4 * b + 2], acc[4 * b + 3]);
        } else {
          float* dst = Wk.rk0 + m * P.dcol;
          float acc[16];
          fill_features(P, id, sc, acc);
          for (int q = 0; q < P.dcol; ++q) dst[q] = acc[q];
        }
        Wk.rw[m] = wt;
        Wk.rpix[m] = n;
      }
    }
    ++cnt;
    if (T < P.t_stop) break;
  }
  if (!FILL) {
    Wk.n[n] = cnt;
    Wk.T[n] = T;
  }
}

__global__ void k_render_composite(RenderP P, RenderW Wk, const float* __restrict__ logits,
                                   float* image) {
  const int HW = P.H * P.W;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= HW) return;
  const uint32_t cnt = Wk.n[n];
  if (cnt == 0) {
    image[n * 3] = image[n * 3 + 1] = image[n * 3 + 2] = P.bg;
    return;
  }
  const float tb = __fmul_rn(Wk.T[n], P.bg);
  float acc[3] = {tb, tb, tb};
  const int64_t off = Wk.off[n];
  for (uint32_t j = 0; j < cnt; ++j) {
    const int64_t m = off + j;
    if (m >= Wk.cap) break;
    const float w = Wk.rw[m];
    for (int c = 0; c < 3; ++c)
      acc[c] = __fadd_rn(acc[c], __fdiv_rn(w, 1.f + expf(-logits[m * 3 + c])));
  }
  for (int c = 0; c < 3; ++c) image[n * 3 + c] = acc[c];
}

__global__ void k_fill_rows(GridView g, int32_t* rows, const int32_t* __restrict__ dense, int rx,
                            int ry, int rz) {
  const int64_t s = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (s >= int64_t(g.nleaf) * kLeafVox) return;
  const int leaf = int(s >> 9), v = int(s & 511);
  const int x = g.origin[leaf * 3] + (v >> 6), y = g.origin[leaf * 3 + 1] + ((v >> 3) & 7),
            z = g.origin[leaf * 3 + 2] + (v & 7);
  rows[s] = (x < rx && y < ry && z < rz) ? dense[(int64_t(x) * ry + y) * rz + z] : 0;
}

}  // namespace pvdb

using namespace pvdb;

struct pvdb_renderer_s {
  int dcol, dpe, dhid, dout;
  bool flags[5] = {false, false, false, false, false};
  pvdb_grid_s* topo = nullptr;
  int32_t* d_rows = nullptr;
  float* d_den = nullptr;
  float* d_col = nullptr;
  __nv_bfloat16* d_colh = nullptr;
  int64_t nrows = 0;
  int storage = 0;
  float* d_params = nullptr;  // [w0 (dhid x din), b0, w1, b1, w2 (3 x dhid), b2]
  int reso[3] = {0, 0, 0};
  float K[9], xyz_min[3], xyz_max[3];
  float near_ = 0, far_ = 1e9f, stepdist = 0, shift = 0, interval = 0, thr = 0, bg = 0, t_stop = 1e-3f;
  int inverse_y = 0, H = 0, W = 0;
  float c2w[16];
  // frame buffers
  uint32_t* d_n = nullptr;
  uint32_t* d_off = nullptr;
  float* d_T = nullptr;
  float* d_viewdirs = nullptr;
  float* d_hpe = nullptr;
  float* d_image = nullptr;
  uint32_t* d_totals = nullptr;
  uint32_t* scan_partial = nullptr;
  size_t scan_partial_cap = 0;
  float* d_rk0 = nullptr;
  float* d_rw = nullptr;
  int32_t* d_rpix = nullptr;
  float* d_logits = nullptr;
  int64_t rows_cap = 0;
  void* d_packed = nullptr;  // BF16 weight tiles of the tensor-core rgbnet
  size_t packed_cap = 0;
  void* d_xt = nullptr;      // BF16 X tiles of the rows (tensor-core rgbnet)
  size_t xt_cap = 0;
};

static int renderer_grow_rows(pvdb_renderer_s* r, int64_t need) {
  if (need <= r->rows_cap) return PVDB_OK;
  const int64_t cap = std::max<int64_t>(need + need / 4, 1 << 20);
  void* ptrs[] = {r->d_rk0, r->d_rw, r->d_rpix, r->d_logits};
  for (void* p : ptrs) dev_free(p);
  r->d_rk0 = r->d_rw = r->d_logits = nullptr;
  r->d_rpix = nullptr;
  r->rows_cap = 0;
  int rc;
  if ((rc = dev_alloc((void**)&r->d_rk0, size_t(cap) * r->dcol * 4)) ||
      (rc = dev_alloc((void**)&r->d_rw, size_t(cap) * 4)) ||
      (rc = dev_alloc((void**)&r->d_rpix, size_t(cap) * 4)) ||
      (rc = dev_alloc((void**)&r->d_logits, size_t(cap) * 12)))
    return rc;
  r->rows_cap = cap;
  return PVDB_OK;
}

extern "C" {

int pvdb_renderer_create(int32_t dcol, int32_t dpe, int32_t dhid, int32_t dout,
                         pvdb_renderer* out) {
  clear_error();
  PVDB_REQUIRE(out, "null argument");
  PVDB_REQUIRE(dcol > 0 && dcol <= 16, "dcol must be in 1..16");
  PVDB_REQUIRE(dpe == 3 || dpe == 9 || dpe == 15 || dpe == 21 || dpe == 27,
               "dpe must be 3*(1+2*pe) with pe in 0..4");
  PVDB_REQUIRE(dhid == 128, "dhid must be 128");
  PVDB_REQUIRE(dout == 3, "dout must be 3");
  pvdb_renderer_s* r = new pvdb_renderer_s();
  r->dcol = dcol;
  r->dpe = dpe;
  r->dhid = dhid;
  r->dout = dout;
  const size_t P = size_t(dhid) * (dcol + dpe) + dhid + size_t(dhid) * dhid + dhid + 3 * dhid + 3;
  int rc = dev_alloc((void**)&r->d_params, P * 4);
  if (!rc) rc = dev_alloc((void**)&r->d_totals, 64);
  if (rc) {
    pvdb_renderer_destroy(r);
    return rc;
  }
  *out = r;
  return PVDB_OK;
}

int pvdb_renderer_destroy(pvdb_renderer r) {
  if (!r) return PVDB_OK;
  pvdb_grid_destroy(r->topo);
  void* ptrs[] = {r->d_rows, r->d_den, r->d_col, r->d_colh, r->d_params, r->d_n, r->d_off,
                  r->d_T, r->d_viewdirs, r->d_hpe, r->d_image, r->d_totals, r->scan_partial,
                  r->d_rk0, r->d_rw, r->d_rpix, r->d_logits, r->d_packed, r->d_xt};
  for (void* p : ptrs) dev_free(p);
  delete r;
  return PVDB_OK;
}

int pvdb_renderer_load_data(pvdb_renderer r, const int32_t reso[3], const int32_t* index,
                            const float* density, const float* features, int64_t n_rows,
                            int32_t storage, int32_t mem) {
  clear_error();
  PVDB_REQUIRE(r && reso && index && density && features, "null argument");
  PVDB_REQUIRE(n_rows >= 1, "n_rows must be >= 1 (row 0 is the empty row)");
  PVDB_REQUIRE(storage == 0 || storage == 1, "storage must be 0 (FP32) or 1 (BF16 features)");
  const int64_t nvox = int64_t(reso[0]) * reso[1] * reso[2];
  std::vector<int32_t> idx_host;
  const int32_t* idx = index;
  if (mem == PVDB_MEM_DEVICE) {
    idx_host.resize(nvox);
    PVDB_CHECK_CUDA(cudaMemcpy(idx_host.data(), index, nvox * 4, cudaMemcpyDeviceToHost));
    idx = idx_host.data();
  }
  std::vector<uint8_t> active(nvox);
  for (int64_t q = 0; q < nvox; ++q) {
    PVDB_REQUIRE(idx[q] >= 0 && idx[q] < n_rows, "index row out of range");
    active[q] = idx[q] > 0;
  }
  pvdb_grid_destroy(r->topo);
  r->topo = nullptr;
  int rc = pvdb_grid_create_from_mask(reso, 1, 0.f, active.data(), PVDB_MEM_HOST, &r->topo);
  if (rc) return rc;
  dev_free(r->d_rows);
  dev_free(r->d_den);
  dev_free(r->d_col);
  dev_free(r->d_colh);
  r->d_rows = nullptr;
  r->d_den = r->d_col = nullptr;
  r->d_colh = nullptr;
  const int64_t ns = r->topo->nslots();
  int32_t* d_dense = nullptr;
  if ((rc = dev_alloc((void**)&r->d_rows, std::max<int64_t>(ns, 1) * 4)) ||
      (rc = dev_alloc((void**)&d_dense, nvox * 4)) ||
      (rc = dev_alloc((void**)&r->d_den, n_rows * 4))) {
    dev_free(d_dense);
    return rc;
  }
  const cudaMemcpyKind kind = mem == PVDB_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  PVDB_CHECK_CUDA(cudaMemcpy(d_dense, index, nvox * 4, kind));
  if (ns) k_fill_rows<<<ceil_div(ns, 256), 256>>>(r->topo->view(), r->d_rows, d_dense, reso[0], reso[1], reso[2]);
  PVDB_CHECK_LAUNCH("k_fill_rows");
  PVDB_CHECK_CUDA(cudaDeviceSynchronize());
  dev_free(d_dense);
  PVDB_CHECK_CUDA(cudaMemcpy(r->d_den, density, n_rows * 4, kind));
  const size_t nf = size_t(n_rows) * r->dcol;
  if (storage == 0) {
    if ((rc = dev_alloc((void**)&r->d_col, nf * 4))) return rc;
    PVDB_CHECK_CUDA(cudaMemcpy(r->d_col, features, nf * 4, kind));
  } else {
    std::vector<float> hf;
    const float* f = features;
    if (mem == PVDB_MEM_DEVICE) {
      hf.resize(nf);
      PVDB_CHECK_CUDA(cudaMemcpy(hf.data(), features, nf * 4, cudaMemcpyDeviceToHost));
      f = hf.data();
    }
    std::vector<__nv_bfloat16> hb(nf);
    for (size_t q = 0; q < nf; ++q) hb[q] = __float2bfloat16_rn(f[q]);
    if ((rc = dev_alloc((void**)&r->d_colh, nf * 2))) return rc;
    PVDB_CHECK_CUDA(cudaMemcpy(r->d_colh, hb.data(), nf * 2, cudaMemcpyHostToDevice));
  }
  r->nrows = n_rows;
  r->storage = storage;
  for (int a = 0; a < 3; ++a) r->reso[a] = reso[a];
  r->flags[0] = true;
  return PVDB_OK;
}

int pvdb_renderer_load_params(pvdb_renderer r, const float* w0, const float* b0, const float* w1,
                              const float* b1, const float* w2, const float* b2) {
  clear_error();
  PVDB_REQUIRE(r && w0 && b0 && w1 && b1 && w2 && b2, "null argument");
  const int din = r->dcol + r->dpe, H = r->dhid;
  // the reference takes [in,out] row-major (run.py:98-104); store nn.Linear [out,in]
  std::vector<float> flat;
  flat.reserve(size_t(H) * din + H + size_t(H) * H + H + 3 * H + 3);
  for (int o = 0; o < H; ++o)
    for (int i = 0; i < din; ++i) flat.push_back(w0[size_t(i) * H + o]);
  flat.insert(flat.end(), b0, b0 + H);
  for (int o = 0; o < H; ++o)
    for (int i = 0; i < H; ++i) flat.push_back(w1[size_t(i) * H + o]);
  flat.insert(flat.end(), b1, b1 + H);
  for (int o = 0; o < 3; ++o)
    for (int i = 0; i < H; ++i) flat.push_back(w2[size_t(i) * 3 + o]);
  flat.insert(flat.end(), b2, b2 + 3);
  PVDB_CHECK_CUDA(cudaMemcpy(r->d_params, flat.data(), flat.size() * 4, cudaMemcpyHostToDevice));
  r->flags[1] = true;
  return PVDB_OK;
}

int pvdb_renderer_set_scene(pvdb_renderer r, const int32_t reso[3], const float K[9],
                            const float xyz_min[3], const float xyz_max[3]) {
  clear_error();
  PVDB_REQUIRE(r && reso && K && xyz_min && xyz_max, "null argument");
  for (int a = 0; a < 3; ++a) {
    r->reso[a] = reso[a];
    r->xyz_min[a] = xyz_min[a];
    r->xyz_max[a] = xyz_max[a];
  }
  std::memcpy(r->K, K, sizeof(r->K));
  r->flags[2] = true;
  return PVDB_OK;
}

int pvdb_renderer_set_kwargs(pvdb_renderer r, float near_, float far_, float stepdist,
                             float act_shift, float interval, float fast_color_thres, float bg,
                             int32_t inverse_y, int32_t h, int32_t w, float t_stop) {
  clear_error();
  PVDB_REQUIRE(r, "null renderer");
  PVDB_REQUIRE(h > 0 && w > 0 && int64_t(h) * w < (int64_t(1) << 31), "bad image size");
  PVDB_REQUIRE(stepdist > 0.f, "stepdist must be positive");
  (void)far_;
  r->near_ = near_;
  r->far_ = 1e9f;  // plenvdb.h:1008
  r->stepdist = stepdist;
  r->shift = act_shift;
  r->interval = interval;
  r->thr = fast_color_thres;
  r->bg = bg;
  r->inverse_y = inverse_y;
  r->t_stop = t_stop;
  if (h != r->H || w != r->W || !r->d_n) {
    const size_t HW = size_t(h) * w;
    void* ptrs[] = {r->d_n, r->d_off, r->d_T, r->d_viewdirs, r->d_hpe, r->d_image};
    for (void* p : ptrs) dev_free(p);
    r->d_n = r->d_off = nullptr;
    r->d_T = r->d_viewdirs = r->d_hpe = r->d_image = nullptr;
    int rc;
    if ((rc = dev_alloc((void**)&r->d_n, HW * 4)) || (rc = dev_alloc((void**)&r->d_off, HW * 4)) ||
        (rc = dev_alloc((void**)&r->d_T, HW * 4)) ||
        (rc = dev_alloc((void**)&r->d_viewdirs, HW * 12)) ||
        (rc = dev_alloc((void**)&r->d_hpe, HW * (128 + 32) * 4)) ||
        (rc = dev_alloc((void**)&r->d_image, HW * 12)))
      return rc;
    r->H = h;
    r->W = w;
  }
  r->flags[3] = true;
  return PVDB_OK;
}

int pvdb_renderer_input_c2w(pvdb_renderer r, const float* c2w, int32_t mem, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(r && c2w, "null argument");
  if (mem == PVDB_MEM_DEVICE) {
    PVDB_CHECK_CUDA(cudaMemcpyAsync(r->c2w, c2w, 64, cudaMemcpyDeviceToHost, as_stream(s)));
    PVDB_CHECK_CUDA(cudaStreamSynchronize(as_stream(s)));
  } else {
    std::memcpy(r->c2w, c2w, 64);
  }
  r->flags[4] = true;
  return PVDB_OK;
}

int pvdb_renderer_render(pvdb_renderer r, int32_t precision, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(r, "null renderer");
  for (int q = 0; q < 5; ++q)
    if (!r->flags[q])
      return set_error(PVDB_ERR_STATE,
                       "render needs load_data, load_params, setScene, setKwargs and input_a_c2w");
  PVDB_REQUIRE(precision == 0 || precision == 1, "precision must be 0 (FP32) or 1 (BF16 rgbnet)");
  cudaStream_t st = as_stream(s);
  RenderP P{};
  P.H = r->H;
  P.W = r->W;
  P.inverse_y = r->inverse_y;
  std::memcpy(P.K, r->K, sizeof(P.K));
  std::memcpy(P.c2w, r->c2w, sizeof(P.c2w));
  for (int a = 0; a < 3; ++a) {
    P.mn[a] = r->xyz_min[a];
    P.mx[a] = r->xyz_max[a];
    P.wsm1[a] = float(r->reso[a] - 1);
  }
  P.near_ = r->near_;
  P.far_ = r->far_;
  P.stepdist = r->stepdist;
  P.shift = r->shift;
  P.interval = r->interval;
  P.thr = r->thr;
  P.bg = r->bg;
  P.t_stop = r->t_stop;
  P.dcol = r->dcol;
  P.idx = r->topo->view();
  P.rows = r->d_rows;
  P.den = r->d_den;
  P.col = r->d_col;
  P.colh = r->d_colh;
  P.storage = r->storage;
  RenderW Wk{};
  Wk.n = r->d_n;
  Wk.off = r->d_off;
  Wk.T = r->d_T;
  Wk.viewdirs = r->d_viewdirs;
  Wk.totals = r->d_totals;
  const int HW = r->H * r->W;
  prof_begin_call();
  prof_mark(st, 0);
  k_render_march<false><<<ceil_div(HW, 128), 128, 0, st>>>(P, Wk);
  PVDB_CHECK_LAUNCH("k_render_march<count>");
  prof_mark(st, 1);
  int rc = scan_exclusive_u32(r->d_n, r->d_off, HW, r->d_totals + 1, &r->scan_partial,
                              &r->scan_partial_cap, st);
  if (rc) return rc;
  prof_mark(st, 2);
  uint32_t total = 0;
  PVDB_CHECK_CUDA(cudaMemcpyAsync(&total, r->d_totals + 1, 4, cudaMemcpyDeviceToHost, st));
  PVDB_CHECK_CUDA(cudaStreamSynchronize(st));
  rc = renderer_grow_rows(r, int64_t(total) + 1);
  if (rc) return rc;
  Wk.rk0 = r->d_rk0;
  Wk.rw = r->d_rw;
  Wk.rpix = r->d_rpix;
  Wk.cap = r->rows_cap;
  MlpArgs a;
  const int din = r->dcol + r->dpe, H = r->dhid;
  a.w0 = r->d_params;
  a.b0 = a.w0 + size_t(H) * din;
  a.w1 = a.b0 + H;
  a.b1 = a.w1 + size_t(H) * H;
  a.w2 = a.b1 + H;
  a.b2 = a.w2 + 3 * H;
  a.c0 = r->dcol;
  a.dpe = r->dpe;
  a.din = din;
  // BF16 rgbnet: the fill pass writes the X tiles (with the PE computed first)
  const bool x_direct = precision == 1 && total > 0 && din + 1 <= kRgbXK;
  if (x_direct) {
    const int64_t ntiles = (r->rows_cap + 127) / 128;
    if ((rc = dev_reserve(&r->d_xt, &r->xt_cap, size_t(ntiles) * kRgbXTile))) return rc;
    int pe_stride = 0;
    if ((rc = mlp_pe_rows(a, r->d_viewdirs, HW, r->d_hpe, &pe_stride, st))) return rc;
    Wk.xt = static_cast<uint8_t*>(r->d_xt);
    Wk.pe = r->d_hpe + size_t(HW) * H;
    Wk.pe_stride = pe_stride;
    Wk.dpe = r->dpe;
  }
  k_render_march<true><<<ceil_div(HW, 128), 128, 0, st>>>(P, Wk);
  PVDB_CHECK_LAUNCH("k_render_march<fill>");
  prof_mark(st, 3);
  if (total) {
    rc = mlp_forward_rows(a, r->d_rk0, r->d_rpix, r->d_viewdirs, HW, r->d_totals, r->rows_cap,
                          r->d_logits, 1, r->d_hpe, precision, &r->d_packed, &r->packed_cap,
                          &r->d_xt, &r->xt_cap, r->d_totals + 3, st, x_direct ? 1 : 0);
    if (rc) return rc;
  }
  prof_mark(st, 4);
  k_render_composite<<<ceil_div(HW, 256), 256, 0, st>>>(P, Wk, r->d_logits, r->d_image);
  PVDB_CHECK_LAUNCH("k_render_composite");
  prof_mark(st, 5);
  return PVDB_OK;
}

int pvdb_renderer_output(pvdb_renderer r, float* out, int32_t mem, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(r && out, "null argument");
  PVDB_REQUIRE(r->d_image, "no image rendered");
  const size_t bytes = size_t(r->H) * r->W * 12;
  cudaStream_t st = as_stream(s);
  PVDB_CHECK_CUDA(cudaMemcpyAsync(out, r->d_image, bytes,
                                  mem == PVDB_MEM_DEVICE ? cudaMemcpyDeviceToDevice
                                                         : cudaMemcpyDeviceToHost,
                                  st));
  if (mem == PVDB_MEM_HOST) PVDB_CHECK_CUDA(cudaStreamSynchronize(st));
  return PVDB_OK;
}

int pvdb_renderer_views(pvdb_renderer r, float** image, int32_t** n_samples_total) {
  clear_error();
  PVDB_REQUIRE(r, "null renderer");
  if (image) *image = r->d_image;
  if (n_samples_total) *n_samples_total = (int32_t*)(r->d_totals + 1);
  return PVDB_OK;
}

}  // extern "C"
