// rgbnet: Linear(C0+Dpe -> 128) ReLU Linear(128 -> 128) ReLU Linear(128 -> 3),
// then sigmoid (dvgo.py:91-107, :354-362), evaluated on the colour rows of a
// march workspace. Layer 0 is split into the per-row k0 part and a per-ray
// part W0[:,C0:]·PE(viewdir) + b0 computed once per ray (the reference
// renderer hoists it the same way, renderer.cu:100-101).
//
// FP32 SIMT kernels: persistent CTAs over 64-row tiles; every thread owns a
// 4-row x 8-column block (columns strided by 16 so the padded weight rows are
// read without bank conflicts). The backward recomputes the activations of its
// tile, and accumulates the weight gradients of all tiles it visits in
// registers; per-CTA partials are summed in CTA order by k_wgrad_reduce, so the
// weight gradients are deterministic for a given grid size.
#include <algorithm>

#include "march.cuh"

namespace pvdb {

constexpr int kW = 128;       // hidden width
constexpr int kTile = 64;     // rows per tile
constexpr int kMaxC0 = 16;    // k0 channels
constexpr int kMaxPe = 32;    // PE dims
constexpr int kW1S = kW + 1;  // padded row stride of W1 in shared memory
constexpr int kAS = kTile + 4;  // row stride of transposed activation tiles
constexpr int kMlpThreads = 256;

struct MlpArgs {
  const float* w0; const float* b0;
  const float* w1; const float* b1;
  const float* w2; const float* b2;
  int c0, dpe, din;  // din = c0 + dpe
};

// Flat parameter layout shared with the train step and the Python side:
// [w0 (128 x din), b0 (128), w1 (128 x 128), b1 (128), w2 (3 x 128), b2 (3)].
__host__ __device__ inline int64_t mlp_param_count(int din) { return int64_t(kW) * din + kW + kW * kW + kW + 3 * kW + 3; }

// PE of a unit view direction (dvgo.py:354-355): [d, sin(d*2^i), cos(d*2^i)]
// with the frequencies innermost per axis: sin at 3 + a*npe + i, cos at
// 3 + 3*npe + a*npe + i.
// Per ray: pe[r][0:dpe] and hpe[r][n] = b0[n] + sum_q w0[n][c0+q] * pe[r][q].
// A 128-thread block takes kPeRays rays: the PE part of W0 is staged
// transposed in shared memory (coalesced), each PE component is evaluated
// once, then thread n forms hpe[r][n] for the block's rays.
constexpr int kPeRays = 32;
__global__ void __launch_bounds__(128)
    k_pe_hpe(const float* __restrict__ viewdirs, int R, int npe, MlpArgs a, float* pe_out,
             float* hpe) {
  grid_dep_sync();  // hpe == NULL: the PE only
  __shared__ float wt[kMaxPe][kW];       // wt[q][n] = w0[n][c0+q]
  __shared__ float pe_s[kPeRays][kMaxPe];
  const int n = threadIdx.x;
  const int r0 = blockIdx.x * kPeRays;
  for (int q = 0; q < a.dpe; ++q) wt[q][n] = a.w0[n * a.din + a.c0 + q];
  for (int e = n; e < kPeRays * a.dpe; e += kW) {
    const int rr = e / a.dpe, q = e % a.dpe, r = r0 + rr;
    if (r >= R) continue;
    float v;
    if (q < 3) {
      v = viewdirs[r * 3 + q];
    } else {
      const int qq = q - 3, sc = qq / (3 * npe), rem = qq % (3 * npe), ax = rem / npe,
                i = rem % npe;
      const float x = viewdirs[r * 3 + ax] * float(1 << i);
      v = sc ? cosf(x) : sinf(x);
    }
    pe_s[rr][q] = v;
    pe_out[int64_t(r) * kMaxPe + q] = v;
  }
  __syncthreads();
  if (!hpe) return;
  const float b = a.b0[n];
  for (int rr = 0; rr < kPeRays && r0 + rr < R; ++rr) {
    float s = 0.f;
    for (int q = 0; q < a.dpe; ++q) s = fmaf(wt[q][n], pe_s[rr][q], s);
    hpe[int64_t(r0 + rr) * kW + n] = b + s;
  }
}

struct MlpSmem {
  float w1[kW * kW1S];
  float w0k[kW * (kMaxC0 + 1)];
  float w2[3 * kW];
  float b1[kW];
  float b2[4];
  float x[kTile * kMaxC0];  // k0 rows of the tile
  float h0t[kW * kAS];      // relu(layer 0), transposed [n][row]
};

__device__ void mlp_load_weights(MlpSmem& S, const MlpArgs& a) {
  for (int i = threadIdx.x; i < kW * kW; i += blockDim.x) S.w1[(i / kW) * kW1S + (i % kW)] = a.w1[i];
  for (int i = threadIdx.x; i < kW * a.c0; i += blockDim.x)
    S.w0k[(i / a.c0) * (kMaxC0 + 1) + (i % a.c0)] = a.w0[(i / a.c0) * a.din + (i % a.c0)];
  for (int i = threadIdx.x; i < 3 * kW; i += blockDim.x) S.w2[i] = a.w2[i];
  for (int i = threadIdx.x; i < kW; i += blockDim.x) S.b1[i] = a.b1[i];
  if (threadIdx.x < 3) S.b2[threadIdx.x] = a.b2[threadIdx.x];
}

// Layer 0 and layer 1 of one tile; returns relu(layer 1) in h1[4][8] for rows
// ty*4+i and columns tx+16*j. Leaves relu(layer 0) in S.h0t.
__device__ __forceinline__ void mlp_tile_forward(MlpSmem& S, const MlpArgs& a,
                                                 const float* __restrict__ k0,
                                                 const int32_t* __restrict__ ray,
                                                 const float* __restrict__ hpe, int64_t row0,
                                                 int64_t M, float h1[4][8]) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int i = threadIdx.x; i < kTile * a.c0; i += blockDim.x) {
    const int rr = i / a.c0, q = i % a.c0;
    const int64_t m = row0 + rr;
    S.x[rr * kMaxC0 + q] = m < M ? k0[m * a.c0 + q] : 0.f;
  }
  __syncthreads();
  // layer 0
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int rr = ty * 4 + i;
    const int64_t m = row0 + rr;
    const int r = m < M ? ray[m] : -1;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int n = tx + 16 * j;
      float z = r >= 0 ? hpe[int64_t(r) * kW + n] : 0.f;
      for (int q = 0; q < a.c0; ++q) z = fmaf(S.w0k[n * (kMaxC0 + 1) + q], S.x[rr * kMaxC0 + q], z);
      S.h0t[n * kAS + rr] = fmaxf(z, 0.f);
    }
  }
  __syncthreads();
  // layer 1
  float acc[4][8];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
#pragma unroll 4
  for (int k = 0; k < kW; ++k) {
    const float4 av = *reinterpret_cast<const float4*>(&S.h0t[k * kAS + ty * 4]);
    const float aa[4] = {av.x, av.y, av.z, av.w};
    float bb[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) bb[j] = S.w1[(tx + 16 * j) * kW1S + k];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(aa[i], bb[j], acc[i][j]);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) h1[i][j] = fmaxf(acc[i][j] + S.b1[tx + 16 * j], 0.f);
}

// Layer 2 logits for rows ty*4+i: partial dot products over this thread's
// columns, reduced over the 16 threads of the row group (xor within 16 lanes).
__device__ __forceinline__ void mlp_logits(const MlpSmem& S, const float h1[4][8], float lg[4][3]) {
  const int tx = threadIdx.x & 15;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float s = 0.f;
#pragma unroll
      for (int j = 0; j < 8; ++j) s = fmaf(S.w2[c * kW + tx + 16 * j], h1[i][j], s);
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      lg[i][c] = s + S.b2[c];
    }
}

__global__ void __launch_bounds__(kMlpThreads, 1)
    k_mlp_fwd_f32(MlpArgs a, const float* __restrict__ k0, const int32_t* __restrict__ ray,
                  const float* __restrict__ hpe, const uint32_t* __restrict__ totals,
                  float* rgb, int out_logits) {
  grid_dep_sync();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MlpSmem& S = *reinterpret_cast<MlpSmem*>(smem_raw);
  const int64_t M = totals[1];
  const int64_t ntiles = (M + kTile - 1) / kTile;
  if (blockIdx.x >= ntiles) return;
  mlp_load_weights(S, a);
  __syncthreads();
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t row0 = t * kTile;
    float h1[4][8];
    mlp_tile_forward(S, a, k0, ray, hpe, row0, M, h1);
    float lg[4][3];
    mlp_logits(S, h1, lg);
    if (tx == 0) {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int64_t m = row0 + ty * 4 + i;
        if (m < M)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            rgb[m * 3 + c] = out_logits ? lg[i][c] : 1.f / (1.f + expf(-lg[i][c]));
      }
    }
    __syncthreads();
  }
}

struct MlpBwdSmem {
  MlpSmem f;
  float dl[kTile * 4];       // d logits [row][c]
  float dz1t[kW * kAS];      // d(layer-1 pre-activation), transposed [n][row]
  float dz0t[kW * kAS];      // d(layer-0 pre-activation), transposed [n][row]
  float pe[kTile * kMaxPe];  // PE rows of the tile
};

// Per-CTA partial gradient layout (same as the flat parameter layout).
__global__ void __launch_bounds__(kMlpThreads, 1)
    k_mlp_bwd_f32(MlpArgs a, const float* __restrict__ k0, const int32_t* __restrict__ ray,
                  const float* __restrict__ hpe, const float* __restrict__ pe_buf,
                  const uint32_t* __restrict__ totals, const float* __restrict__ rgb,
                  const float* __restrict__ grad_rgb, float* grad_k0, float* wpart) {
  grid_dep_sync();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MlpBwdSmem& B = *reinterpret_cast<MlpBwdSmem*>(smem_raw);
  MlpSmem& S = B.f;
  const int64_t M = totals[1];
  const int64_t ntiles = (M + kTile - 1) / kTile;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int64_t P = mlp_param_count(a.din);
  float* part = wpart + int64_t(blockIdx.x) * P;
  float* pw0 = part;
  float* pb0 = pw0 + kW * a.din;
  float* pw1 = pb0 + kW;
  float* pb1 = pw1 + kW * kW;
  float* pw2 = pb1 + kW;
  float* pb2 = pw2 + 3 * kW;
  // accumulators: dW1 block (n = ty+16i, k = tx+16j), dW0 row n = tid>>1 half q,
  // db0/db1 for n = tid>>1 (even threads), dW2/db2 entries tid, tid+256
  float aw1[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) aw1[i][j] = 0.f;
  const int n0 = tid >> 1, qh = tid & 1;
  const int qbeg = qh ? (a.din + 1) / 2 : 0, qend = qh ? a.din : (a.din + 1) / 2;
  float aw0[24];
#pragma unroll
  for (int q = 0; q < 24; ++q) aw0[q] = 0.f;
  float ab0 = 0.f, ab1 = 0.f;
  float aw2[2] = {0.f, 0.f};
  float ab2 = 0.f;
  if (blockIdx.x < ntiles) {
    mlp_load_weights(S, a);
    __syncthreads();
  }
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t row0 = t * kTile;
    // PE rows
    for (int i = tid; i < kTile * a.dpe; i += blockDim.x) {
      const int rr = i / a.dpe, q = i % a.dpe;
      const int64_t m = row0 + rr;
      B.pe[rr * kMaxPe + q] = m < M ? pe_buf[int64_t(ray[m]) * kMaxPe + q] : 0.f;
    }
    float h1[4][8];
    mlp_tile_forward(S, a, k0, ray, hpe, row0, M, h1);
    // d logits: sigmoid backward
    if (tid < kTile * 3) {
      const int rr = tid / 3, c = tid % 3;
      const int64_t m = row0 + rr;
      float d = 0.f;
      if (m < M) {
        const float y = rgb[m * 3 + c];
        d = grad_rgb[m * 3 + c] * (1.f - y) * y;
      }
      B.dl[rr * 4 + c] = d;
    }
    __syncthreads();
    // dz1 = (dl . W2) * relu'(h1); also dW2 needs h1: write h1 into dz0t scratch
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int rr = ty * 4 + i;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int n = tx + 16 * j;
        float g = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) g = fmaf(B.dl[rr * 4 + c], S.w2[c * kW + n], g);
        B.dz1t[n * kAS + rr] = h1[i][j] > 0.f ? g : 0.f;
        B.dz0t[n * kAS + rr] = h1[i][j];
      }
    }
    __syncthreads();
    // dW2, db2 (entries e = c*128+n for c<3) and db2
    for (int e = tid, s = 0; e < 3 * kW; e += blockDim.x, ++s) {
      const int c = e / kW, n = e % kW;
      float acc = 0.f;
      for (int rr = 0; rr < kTile; ++rr) acc = fmaf(B.dl[rr * 4 + c], B.dz0t[n * kAS + rr], acc);
      aw2[s] += acc;
    }
    if (tid < 3) {
      float acc = 0.f;
      for (int rr = 0; rr < kTile; ++rr) acc += B.dl[rr * 4 + tid];
      ab2 += acc;
    }
    // dW1[n][k] += sum_row dz1[row][n] * h0[row][k]   (n = ty+16i, k = tx+16j)
    for (int rr = 0; rr < kTile; ++rr) {
      float av[8], bv[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) av[i] = B.dz1t[(ty + 16 * i) * kAS + rr];
#pragma unroll
      for (int j = 0; j < 8; ++j) bv[j] = S.h0t[(tx + 16 * j) * kAS + rr];
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) aw1[i][j] = fmaf(av[i], bv[j], aw1[i][j]);
    }
    if (!qh) {
      float acc = 0.f;
      for (int rr = 0; rr < kTile; ++rr) acc += B.dz1t[n0 * kAS + rr];
      ab1 += acc;
    }
    __syncthreads();  // dz0t scratch (h1) no longer needed
    // dh0[row][k] = sum_n dz1[row][n] * W1[n][k]; dz0 = dh0 * relu'(h0)
    {
      float acc[4][8];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
#pragma unroll 4
      for (int n = 0; n < kW; ++n) {
        const float4 av = *reinterpret_cast<const float4*>(&B.dz1t[n * kAS + ty * 4]);
        const float aa[4] = {av.x, av.y, av.z, av.w};
        float bb[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) bb[j] = S.w1[n * kW1S + tx + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(aa[i], bb[j], acc[i][j]);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int k = tx + 16 * j, rr = ty * 4 + i;
          B.dz0t[k * kAS + rr] = S.h0t[k * kAS + rr] > 0.f ? acc[i][j] : 0.f;
        }
    }
    __syncthreads();
    // dW0[n][q] += sum_row dz0[row][n] * x[row][q]  (x = [k0, pe]); db0
    for (int rr = 0; rr < kTile; ++rr) {
      const float g = B.dz0t[n0 * kAS + rr];
#pragma unroll
      for (int q = 0; q < 24; ++q) {
        const int qq = qbeg + q;
        if (qq < qend) {
          const float xv = qq < a.c0 ? S.x[rr * kMaxC0 + qq] : B.pe[rr * kMaxPe + qq - a.c0];
          aw0[q] = fmaf(g, xv, aw0[q]);
        }
      }
      if (!qh) ab0 += g;
    }
    // grad_k0[row][q] = sum_n dz0[row][n] * W0[n][q]
    for (int e = tid; e < kTile * a.c0; e += blockDim.x) {
      const int rr = e / a.c0, q = e % a.c0;
      const int64_t m = row0 + rr;
      float acc = 0.f;
      for (int n = 0; n < kW; ++n) acc = fmaf(B.dz0t[n * kAS + rr], S.w0k[n * (kMaxC0 + 1) + q], acc);
      if (m < M) grad_k0[m * a.c0 + q] = acc;
    }
    __syncthreads();
  }
  // write this CTA's partials (zeros if it had no tile)
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) pw1[(ty + 16 * i) * kW + tx + 16 * j] = aw1[i][j];
  for (int q = 0; q < 24; ++q)
    if (qbeg + q < qend) pw0[n0 * a.din + qbeg + q] = aw0[q];
  if (!qh) {
    pb0[n0] = ab0;
    pb1[n0] = ab1;
  }
  for (int e = tid, s = 0; e < 3 * kW; e += blockDim.x, ++s) pw2[e] = aw2[s];
  if (tid < 3) pb2[tid] = ab2;
}

// Sum of the per-CTA partials: eight interleaved running sums (partials c,
// c+8, ...) combined in a fixed order, so the loads of eight partials are in
// flight together and the result is the same on every run.
// 256 threads per 32 parameters: warp u sums the partials c = u, u+8, ... in
// increasing c, then the 8 warp sums combine as ((s0+s1)+(s2+s3))+((s4+s5)+(s6+s7)).
__global__ void __launch_bounds__(256)
    k_wgrad_reduce(const float* __restrict__ wpart, int nparts, int64_t P, float* out) {
  grid_dep_sync();
  __shared__ float part[8][33];
  const int u = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t i = blockIdx.x * 32ll + lane;
  float acc = 0.f;
  if (i < P)
    for (int c = u; c < nparts; c += 8) acc += __ldg(wpart + int64_t(c) * P + i);
  part[u][lane] = acc;
  __syncthreads();
  if (u == 0 && i < P)
    out[i] = ((part[0][lane] + part[1][lane]) + (part[2][lane] + part[3][lane])) +
             ((part[4][lane] + part[5][lane]) + (part[6][lane] + part[7][lane]));
}

__global__ void k_scatter_grads(const float* __restrict__ flat, int din, float* w0, float* b0,
                                float* w1, float* b1, float* w2, float* b2) {
  grid_dep_sync();
  const int64_t P = mlp_param_count(din);
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= P) return;
  int64_t o = i;
  const int64_t s0 = int64_t(kW) * din, s1 = kW, s2 = int64_t(kW) * kW, s3 = kW, s4 = 3 * kW;
  if (o < s0) { if (w0) w0[o] = flat[i]; return; }
  o -= s0;
  if (o < s1) { if (b0) b0[o] = flat[i]; return; }
  o -= s1;
  if (o < s2) { if (w1) w1[o] = flat[i]; return; }
  o -= s2;
  if (o < s3) { if (b1) b1[o] = flat[i]; return; }
  o -= s3;
  if (o < s4) { if (w2) w2[o] = flat[i]; return; }
  o -= s4;
  if (b2) b2[o] = flat[i];
}

// ------------------------------------------------------------------ host
static int mlp_grid() { return num_sms(); }

static int mlp_reserve(pvdb_march_s* m, int din) {
  int rc = dev_reserve((void**)&m->hpe, &m->hpe_cap,
                       size_t(m->max_rays) * (kW + kMaxPe) * 4);
  if (rc) return rc;
  const size_t P = size_t(mlp_param_count(din));
  return dev_reserve((void**)&m->wpart, &m->wpart_cap, (size_t(mlp_grid()) + 1) * P * 4);
}

int mlp_tc_pack(const float* w0, const float* b0, const float* w1, const float* b1,
                const float* w2, const float* b2, int c0, int dpe, void** blob,
                size_t* blob_cap, cudaStream_t st);
int mlp_tc_forward_rows(const float* w0, const float* b0, const float* w1, const float* b1,
                        const float* w2, const float* b2, int c0, int dpe, const float* k0rows,
                        const int32_t* ray, const float* pe, int pe_stride, const uint32_t* totals,
                        int64_t max_rows, float* out, int out_logits, void** blob,
                        size_t* blob_cap, void** xt, size_t* xt_cap, uint32_t* err,
                        cudaStream_t st, int packed, int x_ready);

// Inputs of the rgbnet that depend only on the rays and the weights: the
// per-ray PE (FP32 path: and hpe) and, BF16 path, the packed BF16 weight
// tiles of the forward and the backward. The train step runs this on a side
// stream while the march runs.
int mlp_prepare(pvdb_march_s* m, const MlpArgs& a, const float* viewdirs, int R, int precision,
                cudaStream_t st) {
  if (R <= 0) return PVDB_OK;
  int rc = mlp_reserve(m, a.din);
  if (rc) return rc;
  float* pe = m->hpe + size_t(m->max_rays) * kW;
  launch_k(k_pe_hpe, ceil_div(R, kPeRays), kW, 0, st, viewdirs, R, (a.dpe - 3) / 6, a, pe,
           precision == 1 ? nullptr : m->hpe);
  PVDB_CHECK_LAUNCH("k_pe_hpe");
  if (precision == 1)
    return mlp_tc_pack(a.w0, a.b0, a.w1, a.b1, a.w2, a.b2, a.c0, a.dpe, &m->mlp_packed,
                       &m->mlp_packed_cap, st);
  return PVDB_OK;
}

// The per-ray PE that mlp_prepare writes (stride floats per ray), and the X
// tiles of the tensor-core path reserved for the workspace's rows.
const float* mlp_pe_buffer(pvdb_march_s* m, int* stride) {
  *stride = kMaxPe;
  return m->hpe ? m->hpe + size_t(m->max_rays) * kW : nullptr;
}
int mlp_reserve_x(pvdb_march_s* m) {
  const int64_t ntiles = (m->slots + 127) / 128;
  return dev_reserve(&m->mlp_xt, &m->mlp_xt_cap, size_t(std::max<int64_t>(ntiles, 1)) * kRgbXTile);
}

// prepared: mlp_prepare already ran for these rays and weights; x_ready: the
// BF16 X tiles are already built (march_k0_x).
int mlp_forward_impl(pvdb_march_s* m, const MlpArgs& a, const float* k0rows,
                     const float* viewdirs, float* rgb, int precision, cudaStream_t st,
                     bool prepared, bool x_ready) {
  const int R = m->n_rays;
  if (R <= 0) return PVDB_OK;
  int rc = mlp_reserve(m, a.din);
  if (rc) return rc;
  float* hpe = m->hpe;
  float* pe = m->hpe + size_t(m->max_rays) * kW;
  if (!prepared) {
    launch_k(k_pe_hpe, ceil_div(R, kPeRays), kW, 0, st, viewdirs, R, (a.dpe - 3) / 6, a, pe, hpe);
    PVDB_CHECK_LAUNCH("k_pe_hpe");
  }
  if (precision == 1)
    return mlp_tc_forward_rows(a.w0, a.b0, a.w1, a.b1, a.w2, a.b2, a.c0, a.dpe, k0rows,
                               m->w.r_ray, pe, kMaxPe, m->w.totals, m->slots, rgb, 0,
                               &m->mlp_packed, &m->mlp_packed_cap, &m->mlp_xt, &m->mlp_xt_cap,
                               m->w.totals + 3, st, prepared ? 1 : 0, x_ready ? 1 : 0);
  PVDB_SMEM_ATTR(k_mlp_fwd_f32, int(sizeof(MlpSmem)));
  launch_k(k_mlp_fwd_f32, mlp_grid(), kMlpThreads, sizeof(MlpSmem), st, a, k0rows, m->w.r_ray, hpe,
           m->w.totals, rgb, 0);
  PVDB_CHECK_LAUNCH("k_mlp_fwd_f32");
  return PVDB_OK;
}

// Rows from any producer (the merged renderer): k0rows [M, c0], ray [M] ->
// viewdirs [R,3]; M = totals[1]. hpe_buf holds R*(128+32) floats.
// The per-ray PE alone into hpe_buf + R * 128 (stride kMaxPe floats): the
// input of rgbnet X tiles that a caller builds itself.
int mlp_pe_rows(const MlpArgs& a, const float* viewdirs, int R, float* hpe_buf, int* pe_stride,
                cudaStream_t st) {
  *pe_stride = kMaxPe;
  if (R <= 0) return PVDB_OK;
  launch_k(k_pe_hpe, ceil_div(R, kPeRays), kW, 0, st, viewdirs, R, (a.dpe - 3) / 6, a,
           hpe_buf + size_t(R) * kW, nullptr);
  PVDB_CHECK_LAUNCH("k_pe_hpe");
  return PVDB_OK;
}

// x_ready (BF16 only): the X tiles in *xt are already built from the rows and
// the PE (mlp_pe_rows), so neither is recomputed here.
int mlp_forward_rows(const MlpArgs& a, const float* k0rows, const int32_t* ray,
                     const float* viewdirs, int R, const uint32_t* totals, int64_t max_rows,
                     float* out, int out_logits, float* hpe_buf, int precision, void** blob,
                     size_t* blob_cap, void** xt, size_t* xt_cap, uint32_t* err,
                     cudaStream_t st, int x_ready) {
  if (R <= 0) return PVDB_OK;
  float* hpe = hpe_buf;
  float* pe = hpe_buf + size_t(R) * kW;
  if (precision == 1 && x_ready)
    return mlp_tc_forward_rows(a.w0, a.b0, a.w1, a.b1, a.w2, a.b2, a.c0, a.dpe, k0rows, ray, pe,
                               kMaxPe, totals, max_rows, out, out_logits, blob, blob_cap, xt,
                               xt_cap, err, st, 0, 1);
  launch_k(k_pe_hpe, ceil_div(R, kPeRays), kW, 0, st, viewdirs, R, (a.dpe - 3) / 6, a, pe, hpe);
  PVDB_CHECK_LAUNCH("k_pe_hpe");
  if (precision == 1)
    return mlp_tc_forward_rows(a.w0, a.b0, a.w1, a.b1, a.w2, a.b2, a.c0, a.dpe, k0rows, ray, pe,
                               kMaxPe, totals, max_rows, out, out_logits, blob, blob_cap, xt,
                               xt_cap, err, st, 0, 0);
  PVDB_SMEM_ATTR(k_mlp_fwd_f32, int(sizeof(MlpSmem)));
  launch_k(k_mlp_fwd_f32, mlp_grid(), kMlpThreads, sizeof(MlpSmem), st, a, k0rows, ray, hpe, totals,
           out, out_logits);
  PVDB_CHECK_LAUNCH("k_mlp_fwd_f32(rows)");
  return PVDB_OK;
}

int mlp_tc_backward_rows(const float* w0, const float* b0, const float* w1, const float* b1,
                         const float* w2, const float* b2, int c0, int dpe, const float* k0rows,
                         const int32_t* ray, const float* pe, int pe_stride,
                         const uint32_t* totals, int64_t max_rows, const float* rgb,
                         const float* grad_rgb, float* grad_k0, float* wpart, int grid,
                         void** blob, size_t* blob_cap, void** xt, size_t* xt_cap, uint32_t* err,
                         cudaStream_t st, int packed, int x_ready);

// hpe/pe of the current forward must still be in the workspace; prepared: the
// BF16 backward tiles were packed by mlp_prepare.
int mlp_backward_impl(pvdb_march_s* m, const MlpArgs& a, const float* k0rows, const float* rgb,
                      const float* grad_rgb, float* grad_k0, float* grad_flat, int precision,
                      cudaStream_t st, bool prepared) {
  const int R = m->n_rays;
  const int64_t P = mlp_param_count(a.din);
  if (R <= 0) {
    PVDB_CHECK_CUDA(cudaMemsetAsync(grad_flat, 0, P * 4, st));
    return PVDB_OK;
  }
  int rc = mlp_reserve(m, a.din);
  if (rc) return rc;
  const int G = mlp_grid();
  if (precision == 1) {
    rc = mlp_tc_backward_rows(a.w0, a.b0, a.w1, a.b1, a.w2, a.b2, a.c0, a.dpe, k0rows, m->w.r_ray,
                              m->hpe + size_t(m->max_rays) * kW, kMaxPe, m->w.totals, m->slots,
                              rgb, grad_rgb, grad_k0, m->wpart, G, &m->mlp_packed,
                              &m->mlp_packed_cap, &m->mlp_xt, &m->mlp_xt_cap, m->w.totals + 3, st,
                              prepared ? 1 : 0, prepared ? 1 : 0);
    if (rc) return rc;
    launch_k(k_wgrad_reduce, ceil_div(P, 32), 256, 0, st, m->wpart, G, P, grad_flat);
    PVDB_CHECK_LAUNCH("k_wgrad_reduce");
    return PVDB_OK;
  }
  PVDB_SMEM_ATTR(k_mlp_bwd_f32, int(sizeof(MlpBwdSmem)));
  launch_k(k_mlp_bwd_f32, G, kMlpThreads, sizeof(MlpBwdSmem), st, a, k0rows, m->w.r_ray, m->hpe,
           m->hpe + size_t(m->max_rays) * kW, m->w.totals, rgb, grad_rgb, grad_k0, m->wpart);
  PVDB_CHECK_LAUNCH("k_mlp_bwd_f32");
  launch_k(k_wgrad_reduce, ceil_div(P, 32), 256, 0, st, m->wpart, G, P, grad_flat);
  PVDB_CHECK_LAUNCH("k_wgrad_reduce");
  return PVDB_OK;
}

int mlp_args_from(const pvdb_mlp_weights* w, MlpArgs& a) {
  PVDB_REQUIRE(w && w->w0 && w->b0 && w->w1 && w->b1 && w->w2 && w->b2, "null MLP weight");
  PVDB_REQUIRE(w->width == kW, "rgbnet width must be 128");
  PVDB_REQUIRE(w->c0 > 0 && w->c0 <= kMaxC0, "k0 channels must be in 1..16");
  PVDB_REQUIRE(w->pe >= 0 && w->pe <= 4, "viewbase_pe must be in 0..4");
  a.w0 = w->w0; a.b0 = w->b0; a.w1 = w->w1; a.b1 = w->b1; a.w2 = w->w2; a.b2 = w->b2;
  a.c0 = w->c0;
  a.dpe = 3 + 6 * w->pe;
  a.din = a.c0 + a.dpe;
  return PVDB_OK;
}

}  // namespace pvdb

using namespace pvdb;

extern "C" {

int pvdb_mlp_forward(pvdb_march m, const pvdb_mlp_weights* w, const float* k0,
                     const float* viewdirs, float* rgb, int32_t precision, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(m && viewdirs && rgb, "null argument");
  PVDB_REQUIRE(m->has_fwd, "mlp before march forward");
  PVDB_REQUIRE(m->k0 && m->k0->C == w->c0, "k0 channels differ from the march's k0 grid");
  PVDB_REQUIRE(precision == 0 || precision == 1, "precision must be 0 or 1");
  MlpArgs a;
  int rc = mlp_args_from(w, a);
  if (rc) return rc;
  return mlp_forward_impl(m, a, k0 ? k0 : m->w.r_k0, viewdirs, rgb, precision, as_stream(s), false,
                          false);
}

int pvdb_mlp_backward(pvdb_march m, const pvdb_mlp_weights* w, const float* k0,
                      const float* viewdirs, const float* rgb, const float* grad_rgb,
                      pvdb_mlp_grads* g, float* grad_k0, int32_t precision, pvdb_stream s) {
  clear_error();
  PVDB_REQUIRE(m && viewdirs && rgb && grad_rgb && g && grad_k0, "null argument");
  PVDB_REQUIRE(m->has_fwd, "mlp before march forward");
  PVDB_REQUIRE(m->k0 && m->k0->C == w->c0, "k0 channels differ from the march's k0 grid");
  MlpArgs a;
  int rc = mlp_args_from(w, a);
  if (rc) return rc;
  PVDB_REQUIRE(precision == 0 || precision == 1, "precision must be 0 (fp32) or 1 (bf16)");
  cudaStream_t st = as_stream(s);
  // hpe/pe depend only on the weights and viewdirs: recompute them so the
  // backward does not rely on a preceding forward call of the same weights.
  rc = mlp_reserve(m, a.din);
  if (rc) return rc;
  launch_k(k_pe_hpe, ceil_div(m->n_rays, kPeRays), kW, 0, st, viewdirs, m->n_rays, (a.dpe - 3) / 6,
           a, m->hpe + size_t(m->max_rays) * kW, m->hpe);
  PVDB_CHECK_LAUNCH("k_pe_hpe");
  const int64_t P = mlp_param_count(a.din);
  float* flat = m->wpart + int64_t(mlp_grid()) * P;  // spare slot after the partials
  rc = mlp_backward_impl(m, a, k0 ? k0 : m->w.r_k0, rgb, grad_rgb, grad_k0, flat, precision, st,
                         false);
  if (rc) return rc;
  launch_k(k_scatter_grads, ceil_div(P, 256), 256, 0, st, flat, a.din, g->w0, g->b0, g->w1, g->b1,
           g->w2, g->b2);
  PVDB_CHECK_LAUNCH("k_scatter_grads");
  return PVDB_OK;
}

}  // extern "C"
