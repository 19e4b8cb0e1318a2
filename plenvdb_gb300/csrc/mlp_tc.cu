// rgbnet on the 5th-generation tensor cores (tcgen05), BF16 operands with FP32
// accumulation in TMEM — the BF16 path of the colour MLP (dvgo.py:99-107,
// :354-362; renderer.cu:83-119).
//
// Rows are processed in tiles of 128 (TMEM lane = tile row). Each row's input
// is X = [k0 (c0) | PE (dpe) | 1 | 0...], 48 BF16 columns, so layer 0 is one
// K=48 GEMM against W0f = [W0 | b0 | 0] (the bias rides on the ones column).
//
// Forward (k_mlp_fwd_tc: persistent CTAs, 8 warps, 2 CTAs per SM, 256 TMEM
// columns each):
//   L0  Z0 = X . W0f^T            3 MMAs (K=48)        H0 = relu(Z0)
//   L1  Z1 = H0 . W1^T            8 MMAs (K=128)       H1 = relu(Z1 + b1)
//   L2  Z2 = H1 . W2p^T           8 MMAs, N=16         rgb = sigmoid(Z2 + b2)
// X tiles are built once per step (k_build_x) and each CTA fetches the next
// tile's with a bulk copy while the current tile computes. One thread issues
// the MMAs; completion is signalled through an
// mbarrier (tcgen05.commit). Epilogues read TMEM with tcgen05.ld (warp w reads
// lanes 32*(w%4).., columns 64*(w/4)..), apply bias/activation in FP32 and
// store BF16 into shared memory in the canonical layout the next MMA reads.
#include <algorithm>

#include "march.cuh"
#include "tc.cuh"

namespace pvdb {

namespace {

constexpr int kW = 128;
constexpr int kTcThreads = 256;
constexpr int kXK = kRgbXK;  // input columns of a row: k0 | PE | 1 | 0
// packed weight blob (bytes, canonical K-major BF16 tiles)
constexpr uint32_t kOffW0 = 0;                             // W0f  [128 n][48 q]
constexpr uint32_t kOffW1 = kOffW0 + 128 * kXK * 2;        // W1   [128 n][128 k]   12288
constexpr uint32_t kOffW2 = kOffW1 + 128 * 128 * 2;        // W2p  [16 c][128 k]    45056
constexpr uint32_t kPackFwdBytes = kOffW2 + 16 * 128 * 2;  // 49152
// shared-memory layout of the forward kernel
constexpr uint32_t kXTile = kRgbXTile;                // 12288 B: one X tile
constexpr uint32_t kSmX = kPackFwdBytes;              // two X tiles [128 x 48] bf16
constexpr uint32_t kSmH = kSmX + 2 * kXTile;          // H tile [128 x 128] bf16
constexpr uint32_t kSmB1 = kSmH + 128 * 128 * 2;      // b1 f32[128]
constexpr uint32_t kSmB2 = kSmB1 + 128 * 4;           // b2 f32[16]
constexpr uint32_t kSmBar = kSmB2 + 16 * 4;           // mbarriers: MMA, X0, X1, weights (32 B)
constexpr uint32_t kSmTmem = kSmBar + 32;             // TMEM base address (4 B)
constexpr uint32_t kSmFlag = kSmTmem + 4;             // timeout flag (4 B)
constexpr uint32_t kSmFwdBytes = kSmFlag + 16;
static_assert(2 * kSmFwdBytes <= 228 * 1024, "two forward CTAs must fit on an SM");
constexpr uint32_t kTmemCols = 256;
constexpr uint32_t kWaitIters = 1u << 22;

struct MlpArgsTc {
  const float* w0; const float* b0;
  const float* w1; const float* b1;
  const float* w2; const float* b2;
  int c0, dpe, din;
};

// FP32 nn.Linear weights -> BF16 canonical K-major tiles (one thread per
// element). The backward reads the same tiles, transposed through MN-major
// descriptors.
__global__ void k_pack(MlpArgsTc a, uint8_t* blob) {
  grid_dep_sync();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  __nv_bfloat16* w0 = reinterpret_cast<__nv_bfloat16*>(blob + kOffW0);
  __nv_bfloat16* w1 = reinterpret_cast<__nv_bfloat16*>(blob + kOffW1);
  __nv_bfloat16* w2 = reinterpret_cast<__nv_bfloat16*>(blob + kOffW2);
  if (t < 128 * kXK) {  // W0f[n][q] = w0[n][q] (q < din), b0[n] (q == din), 0
    const int n = t / kXK, q = t % kXK;
    const float v = q < a.din ? a.w0[n * a.din + q] : q == a.din ? a.b0[n] : 0.f;
    w0[tc::kmaj(n, q, kXK) / 2] = __float2bfloat16_rn(v);
  }
  if (t < 128 * 128) {
    const int n = t / 128, k = t % 128;
    w1[tc::kmaj(n, k, 128) / 2] = __float2bfloat16_rn(a.w1[n * 128 + k]);
  }
  if (t < 16 * 128) {
    const int n = t / 128, k = t % 128;
    w2[tc::kmaj(n, k, 128) / 2] = __float2bfloat16_rn(n < 3 ? a.w2[n * 128 + k] : 0.f);
  }
}

__device__ __forceinline__ bool wait_or_flag(uint64_t* bar, uint32_t parity, uint32_t* flag,
                                             uint32_t* err) {
  if (!tc::mbar_wait(bar, parity, kWaitIters)) {
    atomicOr(flag, 1u);
    if (err) atomicOr(err, 2u);
  }
  __syncthreads();
  return *((volatile uint32_t*)flag) == 0;
}

// The rows' X tiles in global memory, tile after tile in the canonical BF16
// K-major layout the MMAs read (one 16-byte chunk per thread): the MLP
// kernels fetch a tile with one bulk copy.
__global__ void __launch_bounds__(256)
    k_build_x(MlpArgsTc a, const float* __restrict__ k0, const int32_t* __restrict__ ray,
              const float* __restrict__ pe, int pe_stride, const uint32_t* __restrict__ totals,
              uint8_t* xt) {
  grid_dep_sync();
  const int64_t M = totals[1];
  const int64_t nchunks = (M + 127) / 128 * (128 * 6);
  for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < nchunks;
       c += int64_t(gridDim.x) * blockDim.x) {
    const int64_t tile = c / (128 * 6);
    const int w = int(c - tile * (128 * 6));
    const int r = w / 6, qb = (w % 6) * 8;
    const int64_t m = tile * 128 + r;
    float v[8];
    if (m < M) {
      const int64_t rr = __ldg(ray + m);
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int qq = qb + e;
        v[e] = qq < a.c0 ? __ldg(k0 + m * a.c0 + qq)
               : qq < a.din ? __ldg(pe + rr * pe_stride + (qq - a.c0))
               : qq == a.din ? 1.f : 0.f;
      }
    } else {
#pragma unroll
      for (int e = 0; e < 8; ++e) v[e] = 0.f;
    }
    uint4 pk;
    pk.x = tc::pack_bf16(v[0], v[1]);
    pk.y = tc::pack_bf16(v[2], v[3]);
    pk.z = tc::pack_bf16(v[4], v[5]);
    pk.w = tc::pack_bf16(v[6], v[7]);
    *reinterpret_cast<uint4*>(xt + tile * kXTile + tc::kmaj(r, qb, kXK)) = pk;
  }
}

// Thread 0 starts the bulk copy of X tile `t` into shared buffer `b`.
__device__ __forceinline__ void x_fetch(uint8_t* sm_x, const uint8_t* xt, int64_t t,
                                        uint64_t* xbar) {
  tc::mbar_expect_tx(xbar, kXTile);
  tc::bulk_g2s(sm_x, xt + t * kXTile, kXTile, xbar);
}

// BF16 pair (lo, hi) of FP32 values, rounded to nearest even and clamped below
// at zero: relu and rounding in one instruction (the values of relu before
// rounding, up to the sign of a zero).
__device__ __forceinline__ uint32_t pack_relu_bf16(float lo, float hi) {
  uint32_t r;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}

// relu(v + bias) of 8 consecutive columns as 8 BF16.
__device__ __forceinline__ uint4 relu_pack8(const float* v, const float* bias, int col) {
  float h[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) h[e] = bias ? v[e] + bias[col + e] : v[e];
  return make_uint4(pack_relu_bf16(h[0], h[1]), pack_relu_bf16(h[2], h[3]),
                    pack_relu_bf16(h[4], h[5]), pack_relu_bf16(h[6], h[7]));
}

// 32 FP32 values (+ bias, relu) -> 4 x 8 BF16 into a K-major tile (ktot columns).
__device__ __forceinline__ void store_relu32(uint8_t* tile, int row, int col0, int ktot,
                                             const float* v, const float* bias) {
#pragma unroll
  for (int c = 0; c < 4; ++c)
    *reinterpret_cast<uint4*>(tile + tc::kmaj(row, col0 + 8 * c, ktot)) =
        relu_pack8(v + 8 * c, bias, col0 + 8 * c);
}

__global__ void __launch_bounds__(kTcThreads, 2)
    k_mlp_fwd_tc(MlpArgsTc a, const uint8_t* __restrict__ blob, const uint8_t* __restrict__ xt,
                 const uint32_t* __restrict__ totals, float* out, int out_logits, uint32_t* err) {
  grid_dep_sync();
  extern __shared__ __align__(1024) uint8_t sm[];
  const int64_t M = totals[1];
  const int64_t ntiles = (M + 127) / 128;
  if (blockIdx.x >= ntiles) return;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + kSmBar);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + kSmTmem);
  uint32_t* flag = reinterpret_cast<uint32_t*>(sm + kSmFlag);
  float* b1s = reinterpret_cast<float*>(sm + kSmB1);
  float* b2s = reinterpret_cast<float*>(sm + kSmB2);
  if (tid < 128) b1s[tid] = a.b1[tid];
  if (tid < 16) b2s[tid] = tid < 3 ? a.b2[tid] : 0.f;
  uint64_t* xbar = bar + 1;  // X tile barriers, one per buffer
  uint64_t* wbar = bar + 3;  // the weight tiles
  if (tid == 0) {
    *flag = 0;
    tc::mbar_init(bar, 1);
    tc::mbar_init(xbar, 1);
    tc::mbar_init(xbar + 1, 1);
    tc::mbar_init(wbar, 1);
    // the packed weights (48 KB) in one bulk copy, beside the first X tile's
    tc::mbar_expect_tx(wbar, kPackFwdBytes);
    tc::bulk_g2s(sm, blob, kPackFwdBytes, wbar);
    x_fetch(sm + kSmX, xt, blockIdx.x, xbar);
  }
  if (warp == 0) {
    tc::tmem_alloc(tmem_slot, kTmemCols);
    tc::tmem_relinquish();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t sbase = tc::smem_addr(sm);
  const uint32_t id_n128 = tc::idesc_bf16(128, 128);
  const uint32_t id_n16 = tc::idesc_bf16(128, 16);
  const int q = warp & 3, half = warp >> 2;
  const int row = 32 * q + lane;  // TMEM lane = tile row of this thread
  const uint32_t t_lane = tmem + (uint32_t(32 * q) << 16);
  uint32_t phase = 0, xph[2] = {0u, 0u};
  bool ok = true;
  int it = 0;
  for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++it) {
    const int64_t row0 = t * 128;
    const int b = it & 1;
    // the next tile's X travels while this tile computes (its buffer was last
    // read by the previous tile's layer-0 MMA, complete)
    if (tid == 0 && t + gridDim.x < ntiles) x_fetch(sm + kSmX + (b ^ 1) * kXTile, xt, t + gridDim.x, xbar + (b ^ 1));
    ok = wait_or_flag(xbar + b, xph[b], flag, err);
    if (!ok) break;
    xph[b] ^= 1u;
    if (it == 0 && !(ok = wait_or_flag(wbar, 0, flag, err))) break;
    if (tid == 0) {
      tc::fence_after();
#pragma unroll
      for (int s = 0; s < 3; ++s)
        tc::mma_bf16(tmem, tc::make_desc(sbase + kSmX + b * kXTile + 256 * s, 128, 768),
                     tc::make_desc(sbase + kOffW0 + 256 * s, 128, 768), id_n128, s > 0);
      tc::mma_commit(bar);
    }
    ok = wait_or_flag(bar, phase, flag, err);
    phase ^= 1;
    if (!ok) break;
    tc::fence_after();
    // ---- H0 = relu(Z0)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      float v[32];
      tc::tmem_ld32(t_lane + uint32_t(64 * half + 32 * j), v);
      store_relu32(sm + kSmH, row, 64 * half + 32 * j, 128, v, nullptr);
    }
    tc::fence_before();
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
#pragma unroll
      for (int s = 0; s < 8; ++s)
        tc::mma_bf16(tmem + 128, tc::make_desc(sbase + kSmH + 256 * s, 128, 2048),
                     tc::make_desc(sbase + kOffW1 + 256 * s, 128, 2048), id_n128, s > 0);
      tc::mma_commit(bar);
    }
    ok = wait_or_flag(bar, phase, flag, err);
    phase ^= 1;
    if (!ok) break;
    tc::fence_after();
    // ---- H1 = relu(Z1 + b1), over H0
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      float v[32];
      tc::tmem_ld32(t_lane + 128u + uint32_t(64 * half + 32 * j), v);
      store_relu32(sm + kSmH, row, 64 * half + 32 * j, 128, v, b1s);
    }
    tc::fence_before();
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
#pragma unroll
      for (int s = 0; s < 8; ++s)
        tc::mma_bf16(tmem, tc::make_desc(sbase + kSmH + 256 * s, 128, 2048),
                     tc::make_desc(sbase + kOffW2 + 256 * s, 128, 2048), id_n16, s > 0);
      tc::mma_commit(bar);
    }
    ok = wait_or_flag(bar, phase, flag, err);
    phase ^= 1;
    if (!ok) break;
    tc::fence_after();
    // ---- logits (warps 0-3 hold all 16 columns of their rows)
    if (half == 0) {
      float v[16];
      tc::tmem_ld16(t_lane, v);
      const int64_t m = row0 + row;
      if (m < M) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float lg = v[c] + b2s[c];
          out[m * 3 + c] = out_logits ? lg : 1.f / (1.f + expf(-lg));
        }
      }
    }
    tc::fence_before();
    __syncthreads();
  }
  if (!ok) {
    // a wait gave up: give the MMAs and X copies in flight one more bounded
    // wait before their TMEM and shared memory are released
    tc::mbar_wait(bar, phase ^ 1u, kWaitIters);
    tc::mbar_wait(xbar, xph[0], kWaitIters);
    tc::mbar_wait(xbar + 1, xph[1], kWaitIters);
    tc::mbar_wait(wbar, 0, kWaitIters);
  }
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

// ---------------------------------------------------------------- backward
// Per 128-row tile:
//   recompute  Z0 = X.W0f^T -> H0 = relu(Z0);  Z1 = H0.W1^T -> H1 = relu(Z1 + b1)
//   dl   = grad_rgb * y (1 - y)                       [128 x 3] (sigmoid backward)
//   dZ1  = (dl . W2) * [H1 > 0]
//   dZ0  = (dZ1 . W1) * [H0 > 0]
//   gk0  = dZ0 . W0k
//   dW2 += H1^T . dl      dW1|db1 += dZ1^T . [H0|1]   dW0|db0 += dZ0^T . X
// One persistent CTA per SM keeps two tiles in flight, in two slots with their
// own shared-memory tiles and TMEM columns: while the eight epilogue warps of
// one slot drain TMEM and write the next operand, the tensor cores run the
// other slot's MMAs. One elected thread of a seventeenth warp issues every
// MMA, in a fixed order (stage k of slot 0, then stage k of slot 1, tile pair
// after tile pair), so the weight-gradient accumulators, resident in TMEM
// across all the CTA's tiles, sum in an order fixed by the data: bitwise
// reproducible.
//   stage  MMAs (issuer)                                   epilogue (the slot's warps)
//   S0     Z0 = X.W0f^T                -> A                E0  H0 = relu(Z0)
//   S1     Z1 = H0.W1^T                -> A                E1  H1 = relu(Z1 + b1), dl
//   S2     dZ1' = dl.W2 -> A;  dW2 += H1^T.dl             E2  dZ1 = dZ1'*[H1 > 0], over H1
//   S3     dH0 = dZ1.W1 -> A;  dW1|db1 += dZ1^T.[H0|1]     E3  dZ0 = dH0*[H0 > 0], over dZ1
//   S4     gk0 = dZ0.W0k -> G; dW0|db0 += dZ0^T.X          E4  gk0 -> global
// dl has three nonzero columns of the MMA's 16; dZ1' is one K = 16 MMA whose
// B operand is W2's first 8 rows (rows 3..7 zero) followed, as the second
// 8 of K, by finite weights that meet dl's zero columns. E2 masks it with the
// relu of H1, which E1 keeps in registers. A ones column in H0 and in X turns
// the bias sums into one more MMA column. W1 and
// W0k are the forward's K-major weight tiles read through MN-major
// descriptors (no transposed copies). An epilogue signals the issuer through
// its slot's mbarrier (256 arrivals) after a proxy fence (its shared-memory
// writes feed the next MMAs) and a tcgen05 fence (its TMEM reads precede the
// next MMA into those columns). The X tiles rotate through three buffers
// (tile j in buffer j % 3): E4 of tile j, after S4 has read the buffer for the
// last time, starts the bulk copy of tile j + 3's X, so a copy has two tiles'
// time to land before S0 needs it. At the end the CTA writes its partial
// weight gradients in the flat parameter layout; the partials are summed over
// CTAs in a fixed order.
constexpr int kBwdEpiWarps = 8;             // per slot: 4 lane quarters x 2 column halves
constexpr int kBwdThreads = (2 * kBwdEpiWarps + 1) * 32;  // + the issuer warp: 544
constexpr int kBwdIssuer = 2 * kBwdEpiWarps;  // warp index of the issuer
constexpr int kBwdXBufs = 3;                // X tiles in flight: tile j uses buffer j % 3
constexpr uint32_t kSlH0 = 0;               // H0 [128 r][144 k], col 128 = 1
constexpr uint32_t kSlH1 = kSlH0 + 128 * 144 * 2;  // H1, then dZ1, then dZ0 [128 r][128 n]
constexpr uint32_t kSlDl = kSlH1 + 128 * 128 * 2;  // dl [128 r][16 c]
constexpr uint32_t kSlot = kSlDl + 128 * 16 * 2;   // 73728 B per slot
constexpr uint32_t kBX = 2 * kSlot;                // X x 3 [128 r][48 q]: k0 | PE | 1 | 0
// W2p rows 0..7 [8 c][128 k] (K-major, as in the blob): the B operand of
// dZ1 = dl . W2, read MN-major; its K = 16 reaches 2 KB past the rows, into
// W0f (finite values that meet dl's zero columns 8..15)
constexpr uint32_t kBW2 = kBX + kBwdXBufs * kXTile;
constexpr uint32_t kBW0f = kBW2 + 8 * 128 * 2;     // W0f [128 n][48 q]
constexpr uint32_t kBW1 = kBW0f + 128 * kXK * 2;   // W1  [128 n][128 k]
constexpr uint32_t kBB1 = kBW1 + 128 * 128 * 2;    // b1 f32[128]
constexpr uint32_t kBBar = kBB1 + 128 * 4;         // mma[2], epi[2], x[3], drain, weights
constexpr uint32_t kBTmem = kBBar + 80;
constexpr uint32_t kBFlag = kBTmem + 4;
constexpr uint32_t kBXIssued = kBFlag + 4;         // X copies started, per buffer
constexpr uint32_t kSmBwdBytes = kBXIssued + 12;
constexpr uint32_t kBwdWBytes = kOffW2;            // W0f and W1 of the blob (45056 B)
constexpr uint32_t kBwdW2Bytes = 8 * 128 * 2;      // W2p rows 0..7 of the blob
static_assert(kSlot % 1024 == 0, "slot tiles keep their alignment");
static_assert(kBW1 - kBW0f == kOffW1 - kOffW0 && kBwdWBytes % 16 == 0, "W0f, W1 as in the blob");
static_assert(kSmBwdBytes <= 232448, "backward CTA exceeds 227 KB of shared memory");
// TMEM columns: per slot A (128) and G (16); the resident weight-gradient sums
constexpr uint32_t kTA0 = 0;     // slot s: kTA0 + 128*s  (Z0, Z1, dH0)
constexpr uint32_t kTG0 = 256;   // slot s: kTG0 + 16*s   (grad k0)
constexpr uint32_t kTW2 = 288;   // dW2 [128 n x 16 c]
constexpr uint32_t kTW0 = 304;   // dW0|db0 [128 n x 48 q]
constexpr uint32_t kTW1 = 352;   // dW1|db1 [128 n x 144 k]
constexpr uint32_t kTmemBwdCols = 512;
static_assert(kTW1 + 144 <= kTmemBwdCols, "TMEM columns");

// 0xFFFF in each 16-bit half of a BF16 pair whose magnitude is nonzero: bit 15
// (bit 31) of (w & 0x7FFF7FFF) + 0x7FFF7FFF is set exactly when the low (high)
// half is nonzero, and a byte permute replicates those sign bits over their
// halves.
__device__ __forceinline__ uint32_t nonzero_mask_bf16x2(uint32_t w) {
  const uint32_t t = (w & 0x7FFF7FFFu) + 0x7FFF7FFFu;
  uint32_t m;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(m) : "r"(t), "r"(0u), "r"(0xBB99u));
  return m;
}

// relu mask of 8 BF16 activations (a uint4: a relu output is positive exactly
// when its magnitude is nonzero) applied to 8 FP32 values, as 8 BF16.
__device__ __forceinline__ uint4 mask_pack(const float* v, uint4 h) {
  return make_uint4(tc::pack_bf16(v[0], v[1]) & nonzero_mask_bf16x2(h.x),
                    tc::pack_bf16(v[2], v[3]) & nonzero_mask_bf16x2(h.y),
                    tc::pack_bf16(v[4], v[5]) & nonzero_mask_bf16x2(h.z),
                    tc::pack_bf16(v[6], v[7]) & nonzero_mask_bf16x2(h.w));
}

// Bounded wait that also gives up as soon as another role has (flag set).
__device__ __forceinline__ bool bwait(uint64_t* bar, uint32_t parity, uint32_t* flag,
                                      uint32_t* err, uint32_t spin_max) {
  for (uint32_t i = 0; i < spin_max; ++i) {
    if (tc::mbar_try(bar, parity)) return true;
    if ((i & 31u) == 31u && *((volatile uint32_t*)flag)) return false;
  }
  atomicOr(flag, 1u);
  if (err) atomicOr(err, 2u);
  return false;
}

// The slot's epilogue threads: results written to shared memory are made
// visible to the tensor cores, TMEM reads are ordered before the next MMA,
// then the thread arrives on the slot's epilogue barrier.
__device__ __forceinline__ void epi_done(uint64_t* bar) {
  tc::fence_async_smem();
  tc::fence_before();
  tc::mbar_arrive(bar);
}

__global__ void __launch_bounds__(kBwdThreads, 1)
    k_mlp_bwd_tc(MlpArgsTc a, const uint8_t* __restrict__ blob, const uint8_t* __restrict__ xt,
                 const uint32_t* __restrict__ totals, const float* __restrict__ rgb,
                 const float* __restrict__ grad_rgb, float* grad_k0, float* wpart, uint32_t* err,
                 uint32_t spin_max, int hold) {
  grid_dep_sync();
  extern __shared__ __align__(1024) uint8_t sm[];
  const int64_t M = totals[1];
  const int64_t ntiles = (M + 127) / 128;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t P = int64_t(kW) * a.din + kW + kW * kW + kW + 3 * kW + 3;
  float* pw0 = wpart + int64_t(blockIdx.x) * P;
  float* pb0 = pw0 + kW * a.din;
  float* pw1 = pb0 + kW;
  float* pb1 = pw1 + kW * kW;
  float* pw2 = pb1 + kW;
  float* pb2 = pw2 + 3 * kW;
  if (blockIdx.x >= ntiles) {
    for (int64_t i = tid; i < P; i += kBwdThreads) pw0[i] = 0.f;
    return;
  }
  // this CTA's tiles: t_j = blockIdx.x + j * gridDim.x, j < nj; tile j goes to slot j & 1
  const int nj = int((ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + kBBar);  // [2] MMA stage done
  uint64_t* ebar = mbar + 2;                                  // [2] epilogue done
  uint64_t* xbar = mbar + 4;                                  // [3] X buffer landed
  uint64_t* dbar = mbar + 7;                                  // drain
  uint64_t* wbar = mbar + 8;                                  // weight tiles landed
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + kBTmem);
  uint32_t* flag = reinterpret_cast<uint32_t*>(sm + kBFlag);
  uint32_t* xissued = reinterpret_cast<uint32_t*>(sm + kBXIssued);
  float* b1s = reinterpret_cast<float*>(sm + kBB1);
  if (tid < 128) b1s[tid] = a.b1[tid];
  if (tid < 256) {
    // H0 columns 128..143 of both slots: [1, 0 x 15] for every row
    const int s = tid >> 7, r = tid & 127;
    uint8_t* h0 = sm + s * kSlot + kSlH0;
    *reinterpret_cast<uint4*>(h0 + tc::kmaj(r, 128, 144)) =
        make_uint4(tc::pack_bf16(1.f, 0.f), 0u, 0u, 0u);
    *reinterpret_cast<uint4*>(h0 + tc::kmaj(r, 136, 144)) = make_uint4(0u, 0u, 0u, 0u);
  }
  if (tid == kBwdIssuer * 32) {
    *flag = 0;
    tc::mbar_init(mbar, 1);
    tc::mbar_init(mbar + 1, 1);
    tc::mbar_init(ebar, 32 * kBwdEpiWarps);
    tc::mbar_init(ebar + 1, 32 * kBwdEpiWarps);
    for (int b = 0; b < kBwdXBufs; ++b) tc::mbar_init(xbar + b, 1);
    tc::mbar_init(dbar, 1);
    tc::mbar_init(wbar, 1);
    // W0f and W1 of the forward's blob in one bulk copy
    tc::mbar_expect_tx(wbar, kBwdWBytes + kBwdW2Bytes);
    tc::bulk_g2s(sm + kBW0f, blob, kBwdWBytes, wbar);
    tc::bulk_g2s(sm + kBW2, blob + kOffW2, kBwdW2Bytes, wbar);
    // the X tiles of the first three tiles
    for (int b = 0; b < kBwdXBufs; ++b) {
      xissued[b] = b < nj ? 1u : 0u;
      if (b < nj) x_fetch(sm + kBX + b * kXTile, xt, blockIdx.x + int64_t(b) * gridDim.x, xbar + b);
    }
  }
  if (warp == kBwdIssuer) {
    tc::tmem_alloc(tmem_slot, kTmemBwdCols);
    tc::tmem_relinquish();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t sb = tc::smem_addr(sm);
  float db2[3] = {0.f, 0.f, 0.f};
  uint32_t xwaits[kBwdXBufs] = {0u, 0u, 0u};  // X arrivals the issuer consumed, per buffer
  bool wdone = false;             // the issuer saw the weight copy land

  if (warp == kBwdIssuer) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0 && !hold) {
      const uint32_t id_kk = tc::idesc_bf16(128, 128);               // A, B K-major
      const uint32_t id_kn = tc::idesc_bf16(128, 128, false, true);  // B MN-major
      const uint32_t id_g = tc::idesc_bf16(128, 16, false, true);    // grad k0
      const uint32_t id_w2 = tc::idesc_bf16(128, 16, true, true);    // H1^T . dl
      const uint32_t id_w1 = tc::idesc_bf16(128, 144, true, true);   // dZ1^T . [H0|1]
      const uint32_t id_w0 = tc::idesc_bf16(128, 48, true, true);    // dZ0^T . X
      uint32_t eph[2] = {0u, 0u};
      bool w2_on = false, w1_on = false, w0_on = false;
      bool ok = wdone = bwait(wbar, 0, flag, err, spin_max);
      for (int pair = 0; ok && 2 * pair < nj; ++pair) {
        for (int k = 0; ok && k < 5; ++k) {
          for (int s = 0; ok && s < 2; ++s) {
            const int j = 2 * pair + s;
            if (j >= nj) continue;
            const int xb = j % kBwdXBufs;
            if (k == 0) {
              ok = bwait(xbar + xb, xwaits[xb] & 1u, flag, err, spin_max);
              if (ok) xwaits[xb]++;
            } else {
              ok = bwait(ebar + s, eph[s], flag, err, spin_max);
              eph[s] ^= 1u;
            }
            if (!ok) break;
            tc::fence_after();
            // descriptors advance by (byte step >> 4) in their address field;
            // the loops stay rolled so the single issuing thread keeps few
            // registers live
            const uint32_t sl = sb + uint32_t(s) * kSlot;
            const uint32_t sx = sb + kBX + uint32_t(xb) * kXTile;
            const uint32_t tA = tmem + kTA0 + 128u * uint32_t(s);
            if (k == 0) {  // Z0 = X . W0f^T
              uint64_t da = tc::make_desc(sx, 128, 768);
              uint64_t db = tc::make_desc(sb + kBW0f, 128, 768);
#pragma unroll 1
              for (int q = 0; q < 3; ++q, da += 256 >> 4, db += 256 >> 4)
                tc::mma_bf16(tA, da, db, id_kk, q > 0);
            } else if (k == 1) {  // Z1 = H0 . W1^T
              uint64_t da = tc::make_desc(sl + kSlH0, 128, 2304);
              uint64_t db = tc::make_desc(sb + kBW1, 128, 2048);
#pragma unroll 1
              for (int q = 0; q < 8; ++q, da += 256 >> 4, db += 256 >> 4)
                tc::mma_bf16(tA, da, db, id_kk, q > 0);
            } else if (k == 2) {  // dZ1' = dl . W2 -> A;  dW2 += H1^T . dl
              tc::mma_bf16(tA, tc::make_desc(sl + kSlDl, 128, 256),
                           tc::make_desc(sb + kBW2, 2048, 128), id_kn, 0u);
              uint64_t da = tc::make_desc(sl + kSlH1, 2048, 128);
              uint64_t db = tc::make_desc(sl + kSlDl, 256, 128);
#pragma unroll 1
              for (int q = 0; q < 8; ++q, da += 4096 >> 4, db += 512 >> 4)
                tc::mma_bf16(tmem + kTW2, da, db, id_w2, (w2_on || q > 0) ? 1u : 0u);
              w2_on = true;
            } else if (k == 3) {  // dH0 = dZ1 . W1;  dW1|db1 += dZ1^T . [H0|1]
              uint64_t da = tc::make_desc(sl + kSlH1, 128, 2048);
              uint64_t db = tc::make_desc(sb + kBW1, 2048, 128);
#pragma unroll 1
              for (int q = 0; q < 8; ++q, da += 256 >> 4, db += 4096 >> 4)
                tc::mma_bf16(tA, da, db, id_kn, q > 0);
              da = tc::make_desc(sl + kSlH1, 2048, 128);
              db = tc::make_desc(sl + kSlH0, 2304, 128);
#pragma unroll 1
              for (int q = 0; q < 8; ++q, da += 4096 >> 4, db += 4608 >> 4)
                tc::mma_bf16(tmem + kTW1, da, db, id_w1, (w1_on || q > 0) ? 1u : 0u);
              w1_on = true;
            } else {  // grad k0 = dZ0 . W0k;  dW0|db0 += dZ0^T . X
              const uint32_t tG = tmem + kTG0 + 16u * uint32_t(s);
              uint64_t da = tc::make_desc(sl + kSlH1, 128, 2048);
              uint64_t db = tc::make_desc(sb + kBW0f, 768, 128);
#pragma unroll 1
              for (int q = 0; q < 8; ++q, da += 256 >> 4, db += 1536 >> 4)
                tc::mma_bf16(tG, da, db, id_g, q > 0);
              da = tc::make_desc(sl + kSlH1, 2048, 128);
              db = tc::make_desc(sx, 768, 128);
#pragma unroll 1
              for (int q = 0; q < 8; ++q, da += 4096 >> 4, db += 1536 >> 4)
                tc::mma_bf16(tmem + kTW0, da, db, id_w0, (w0_on || q > 0) ? 1u : 0u);
              w0_on = true;
            }
            tc::mma_commit(mbar + s);
          }
        }
      }
    }
    __syncwarp();
  } else {
    // ------------------------------------------------- epilogues of slot s
    // warp (s, q4, half): TMEM lanes / tile rows 32*q4.., columns 64*half..
    const int s = warp / kBwdEpiWarps, w8 = warp % kBwdEpiWarps;
    const int q4 = w8 & 3, half = w8 >> 2;
    const int row = 32 * q4 + lane;
    const int c0 = 64 * half;
    const uint32_t tl = tmem + (uint32_t(32 * q4) << 16);
    const uint32_t tA = tl + kTA0 + 128u * uint32_t(s) + uint32_t(c0);
    const uint32_t tG = tl + kTG0 + 16u * uint32_t(s);
    uint8_t* h0 = sm + s * kSlot + kSlH0;
    uint8_t* h1 = sm + s * kSlot + kSlH1;
    uint8_t* dl = sm + s * kSlot + kSlDl;
    // 16-byte row stores only when every row starts on a 16-byte boundary
    const bool vec_k0 = (a.c0 & 3) == 0 && (reinterpret_cast<uintptr_t>(grad_k0) & 15u) == 0;
    uint32_t mph = 0;
    bool ok = true;
    for (int j = s; ok && j < nj; j += 2) {
      const int64_t mrow = (int64_t(blockIdx.x) + int64_t(j) * gridDim.x) * 128 + row;
      // sigmoid inputs of this row, read before the first wait
      float yv[3] = {0.f, 0.f, 0.f}, gv[3] = {0.f, 0.f, 0.f};
      if (mrow < M) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          yv[c] = __ldg(rgb + mrow * 3 + c);
          gv[c] = __ldg(grad_rgb + mrow * 3 + c);
        }
      }
      // ---- E0: H0 = relu(Z0) (the thread's 64 columns in one TMEM round trip)
      if (!(ok = bwait(mbar + s, mph, flag, err, spin_max))) break;
      mph ^= 1u;
      tc::fence_after();
      {
        uint32_t r[64];
#pragma unroll
        for (int q = 0; q < 4; ++q) tc::tmem_ld16_issue(tA + uint32_t(16 * q), r + 16 * q);
        tc::tmem_wait_ld();
#pragma unroll
        for (int g = 0; g < 8; ++g) {
          float v[8];
#pragma unroll
          for (int e = 0; e < 8; ++e) v[e] = __uint_as_float(r[8 * g + e]);
          *reinterpret_cast<uint4*>(h0 + tc::kmaj(row, c0 + 8 * g, 144)) =
              relu_pack8(v, nullptr, 0);
        }
      }
      epi_done(ebar + s);
      // ---- E1: H1 = relu(Z1 + b1); dl = grad_rgb * y * (1 - y)
      if (!(ok = bwait(mbar + s, mph, flag, err, spin_max))) break;
      mph ^= 1u;
      tc::fence_after();
      uint4 hp[8];  // this thread's 64 H1 values, then its dZ1 values, as BF16
#pragma unroll
      for (int cb = 0; cb < 64; cb += 32) {
        float v[32];
        tc::tmem_ld32(tA + uint32_t(cb), v);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          hp[cb / 8 + c] = relu_pack8(v + 8 * c, b1s, c0 + cb + 8 * c);
          *reinterpret_cast<uint4*>(h1 + tc::kmaj(row, c0 + cb + 8 * c, 128)) = hp[cb / 8 + c];
        }
      }
      // dl, in BF16 the A operand of dZ1' = dl . W2 and the B operand of dW2
      {
        float d[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) d[c] = gv[c] * (1.f - yv[c]) * yv[c];
        if (half == 0) {
#pragma unroll
          for (int c = 0; c < 3; ++c) db2[c] += d[c];
          *reinterpret_cast<uint4*>(dl + tc::kmaj(row, 0, 16)) =
              make_uint4(tc::pack_bf16(d[0], d[1]), tc::pack_bf16(d[2], 0.f), 0u, 0u);
          *reinterpret_cast<uint4*>(dl + tc::kmaj(row, 8, 16)) = make_uint4(0u, 0u, 0u, 0u);
        }
      }
      epi_done(ebar + s);
      // ---- E2: dZ1 = dZ1' * [H1 > 0] over H1 once the dW2 MMA has read it
      if (!(ok = bwait(mbar + s, mph, flag, err, spin_max))) break;
      mph ^= 1u;
      tc::fence_after();
#pragma unroll
      for (int cb = 0; cb < 64; cb += 32) {
        float v[32];
        tc::tmem_ld32(tA + uint32_t(cb), v);
#pragma unroll
        for (int c = 0; c < 4; ++c)
          *reinterpret_cast<uint4*>(h1 + tc::kmaj(row, c0 + cb + 8 * c, 128)) =
              mask_pack(v + 8 * c, hp[cb / 8 + c]);
      }
      epi_done(ebar + s);
      // ---- E3: dZ0 = dH0 * [H0 > 0], over dZ1 (the thread's own H0 columns,
      // written by its E0, are read before the wait)
      uint4 hm[8];
#pragma unroll
      for (int g = 0; g < 8; ++g)
        hm[g] = *reinterpret_cast<const uint4*>(h0 + tc::kmaj(row, c0 + 8 * g, 144));
      if (!(ok = bwait(mbar + s, mph, flag, err, spin_max))) break;
      mph ^= 1u;
      tc::fence_after();
#pragma unroll
      for (int cb = 0; cb < 64; cb += 32) {
        float v[32];
        tc::tmem_ld32(tA + uint32_t(cb), v);
#pragma unroll
        for (int c = 0; c < 4; ++c)
          *reinterpret_cast<uint4*>(h1 + tc::kmaj(row, c0 + cb + 8 * c, 128)) =
              mask_pack(v + 8 * c, hm[cb / 8 + c]);
      }
      epi_done(ebar + s);
      // ---- E4: grad k0; the tile's X buffer is free again (S4 is done): it
      // takes the X tile of tile j + 3
      if (!(ok = bwait(mbar + s, mph, flag, err, spin_max))) break;
      mph ^= 1u;
      tc::fence_after();
      if (w8 == 0 && lane == 0 && j + kBwdXBufs < nj) {
        const int xb = j % kBwdXBufs;
        xissued[xb] += 1u;
        x_fetch(sm + kBX + xb * kXTile, xt, blockIdx.x + int64_t(j + kBwdXBufs) * gridDim.x,
                xbar + xb);
      }
      if (half == 0) {
        float v[16];
        tc::tmem_ld16(tG, v);
        if (mrow < M) {
          float* dst = grad_k0 + mrow * a.c0;
          if (vec_k0) {
#pragma unroll
            for (int b = 0; b < 4; ++b)
              if (4 * b < a.c0)
                reinterpret_cast<float4*>(dst)[b] =
                    make_float4(v[4 * b], v[4 * b + 1], v[4 * b + 2], v[4 * b + 3]);
          } else {
#pragma unroll
            for (int qq = 0; qq < 16; ++qq)
              if (qq < a.c0) dst[qq] = v[qq];
          }
        }
      }
      tc::fence_before();
    }
  }
  // ---------------------------------------------------------------- teardown
  __syncthreads();
  const bool failed = *((volatile uint32_t*)flag) != 0;
  if (warp == kBwdIssuer && lane == 0) {
    // every MMA this thread issued completes before TMEM is released; copies
    // still in flight (a wait gave up) land before shared memory is released
    if (!hold) {
      tc::mma_commit(dbar);
      tc::mbar_wait(dbar, 0, spin_max);
    }
    if (!wdone) tc::mbar_wait(wbar, 0, spin_max);
    for (int b = 0; b < kBwdXBufs; ++b)  // at most one copy per buffer is outstanding
      if (xissued[b] > xwaits[b]) tc::mbar_wait(xbar + b, xwaits[b] & 1u, spin_max);
  }
  __syncthreads();
  // The dW1 and dW0|db0 rows are staged in shared memory (the slots' space,
  // free now) with odd row strides, so that thread n's row writes hit
  // distinct banks, and then written out row-major by consecutive threads:
  // coalesced stores, not one 32-byte sector per thread and store.
  constexpr int kS1 = kW + 1;   // dW1 row stride (floats)
  constexpr int kS0 = kXK + 1;  // dW0|db0 row stride
  float* s1 = reinterpret_cast<float*>(sm);
  float* s0 = s1 + kW * kS1;
  static_assert((kW * kS1 + kW * kS0) * 4 <= kBX, "staging fits in the slots");
  if (failed) {
    for (int64_t i = tid; i < P; i += kBwdThreads) pw0[i] = 0.f;
  } else if (warp < 8) {
    tc::fence_after();
    // partial gradients of this CTA: thread (q4, lane) holds row n = 32*q4 + lane
    const int q4 = warp & 3, half = warp >> 2;
    const int n = 32 * q4 + lane;
    const uint32_t tl = tmem + (uint32_t(32 * q4) << 16);
    float v[16];
    float* s1row = s1 + n * kS1;
    float* s0row = s0 + n * kS0;
    if (half == 0) {
      tc::tmem_ld16(tl + kTW2, v);
#pragma unroll
      for (int c = 0; c < 3; ++c) pw2[c * kW + n] = v[c];
#pragma unroll
      for (int j = 0; j < 2; ++j) {  // dW0|db0 columns 0..31
        tc::tmem_ld16(tl + kTW0 + 16 * j, v);
#pragma unroll
        for (int i = 0; i < 16; ++i) s0row[16 * j + i] = v[i];
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {  // dW1 columns 0..63
        tc::tmem_ld16(tl + kTW1 + 16 * j, v);
#pragma unroll
        for (int i = 0; i < 16; ++i) s1row[16 * j + i] = v[i];
      }
      tc::tmem_ld16(tl + kTW1 + 128, v);  // db1
      pb1[n] = v[0];
    } else {
      tc::tmem_ld16(tl + kTW0 + 32, v);  // dW0|db0 columns 32..47
#pragma unroll
      for (int i = 0; i < 16; ++i) s0row[32 + i] = v[i];
#pragma unroll
      for (int j = 4; j < 8; ++j) {  // dW1 columns 64..127
        tc::tmem_ld16(tl + kTW1 + 16 * j, v);
#pragma unroll
        for (int i = 0; i < 16; ++i) s1row[16 * j + i] = v[i];
      }
    }
  }
  __syncthreads();
  if (!failed) {
    for (int i = tid; i < kW * kW; i += kBwdThreads) pw1[i] = s1[(i >> 7) * kS1 + (i & 127)];
    for (int i = tid; i < kW * a.din; i += kBwdThreads) {
      const int n = i / a.din;
      pw0[i] = s0[n * kS0 + (i - n * a.din)];
    }
    if (tid < kW) pb0[tid] = s0[tid * kS0 + a.din];
  }

  if (!failed) {
    // db2: fixed-order sum of the per-row partials of both slots (the first X
    // buffer as scratch: no copy or MMA touches it any more)
    float* red = reinterpret_cast<float*>(sm + kBX);
    if (warp < 2 * kBwdEpiWarps && ((warp % kBwdEpiWarps) >> 2) == 0) {
      const int idx = (warp / kBwdEpiWarps) * 128 + 32 * (warp & 3) + lane;
      for (int c = 0; c < 3; ++c) red[c * 256 + idx] = db2[c];
    }
    __syncthreads();
    if (tid < 3) {
      float acc = 0.f;
      for (int i = 0; i < 256; ++i) acc += red[tid * 256 + i];
      pb2[tid] = acc;
    }
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (warp == kBwdIssuer) tc::tmem_dealloc(tmem, kTmemBwdCols);
}

}  // namespace

// Packs the FP32 weights into the BF16 tile blob (read by the forward and,
// transposed, by the backward).
int mlp_tc_pack(const float* w0, const float* b0, const float* w1, const float* b1,
                const float* w2, const float* b2, int c0, int dpe, void** blob,
                size_t* blob_cap, cudaStream_t st) {
  if (c0 > 16 || c0 + dpe + 1 > kXK)
    return set_error(PVDB_ERR_ARG, "the tensor-core rgbnet takes at most 16 k0 and 47 input channels");
  int rc = dev_reserve(blob, blob_cap, kPackFwdBytes);
  if (rc) return rc;
  MlpArgsTc a{w0, b0, w1, b1, w2, b2, c0, dpe, c0 + dpe};
  launch_k(k_pack, ceil_div(128 * 128, 256), 256, 0, st, a, static_cast<uint8_t*>(*blob));
  PVDB_CHECK_LAUNCH("k_pack");
  return PVDB_OK;
}

// The X tiles of rows k0rows [M, c0] (M = totals[1]) with the PE of each
// row's ray (pe [rays, pe_stride]); room for max_rows rows is reserved.
int mlp_tc_build_x(int c0, int dpe, const float* k0rows, const int32_t* ray, const float* pe,
                   int pe_stride, const uint32_t* totals, int64_t max_rows, void** xt,
                   size_t* xt_cap, cudaStream_t st) {
  if (c0 > 16 || c0 + dpe + 1 > kXK)
    return set_error(PVDB_ERR_ARG, "the tensor-core rgbnet takes at most 16 k0 and 47 input channels");
  const int64_t ntiles = (max_rows + 127) / 128;
  int rc = dev_reserve(xt, xt_cap, size_t(std::max<int64_t>(ntiles, 1)) * kXTile);
  if (rc) return rc;
  MlpArgsTc a{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, c0, dpe, c0 + dpe};
  const int grid = int(std::min<int64_t>(ceil_div(ntiles * 128 * 6, 256), int64_t(num_sms()) * 16));
  launch_k(k_build_x, std::max(grid, 1), 256, 0, st, a, k0rows, ray, pe, pe_stride, totals,
           static_cast<uint8_t*>(*xt));
  PVDB_CHECK_LAUNCH("k_build_x");
  return PVDB_OK;
}

// Forward over the rows (see mlp_tc_build_x for the inputs). packed: the blob
// already holds this call's weights; x_ready: the X tiles are already built.
int mlp_tc_forward_rows(const float* w0, const float* b0, const float* w1, const float* b1,
                        const float* w2, const float* b2, int c0, int dpe, const float* k0rows,
                        const int32_t* ray, const float* pe, int pe_stride, const uint32_t* totals,
                        int64_t max_rows, float* out, int out_logits, void** blob,
                        size_t* blob_cap, void** xt, size_t* xt_cap, uint32_t* err,
                        cudaStream_t st, int packed, int x_ready) {
  int rc = PVDB_OK;
  if (!packed && (rc = mlp_tc_pack(w0, b0, w1, b1, w2, b2, c0, dpe, blob, blob_cap, st)))
    return rc;
  if (!x_ready && (rc = mlp_tc_build_x(c0, dpe, k0rows, ray, pe, pe_stride, totals, max_rows, xt,
                                       xt_cap, st)))
    return rc;
  MlpArgsTc a{w0, b0, w1, b1, w2, b2, c0, dpe, c0 + dpe};
  PVDB_SMEM_ATTR(k_mlp_fwd_tc, int(kSmFwdBytes));
  launch_k(k_mlp_fwd_tc, 2 * num_sms(), kTcThreads, kSmFwdBytes, st, a,
           static_cast<const uint8_t*>(*blob), static_cast<const uint8_t*>(*xt), totals, out,
           out_logits, err);
  PVDB_CHECK_LAUNCH("k_mlp_fwd_tc");
  return PVDB_OK;
}

// Weight and k0 gradients of the rows; per-CTA partials go to wpart (grid x P
// floats), the caller sums them.
int mlp_tc_backward_rows(const float* w0, const float* b0, const float* w1, const float* b1,
                         const float* w2, const float* b2, int c0, int dpe, const float* k0rows,
                         const int32_t* ray, const float* pe, int pe_stride,
                         const uint32_t* totals, int64_t max_rows, const float* rgb,
                         const float* grad_rgb, float* grad_k0, float* wpart, int grid,
                         void** blob, size_t* blob_cap, void** xt, size_t* xt_cap, uint32_t* err,
                         cudaStream_t st, int packed, int x_ready) {
  int rc = PVDB_OK;
  if (!packed && (rc = mlp_tc_pack(w0, b0, w1, b1, w2, b2, c0, dpe, blob, blob_cap, st)))
    return rc;
  if (!x_ready && (rc = mlp_tc_build_x(c0, dpe, k0rows, ray, pe, pe_stride, totals, max_rows, xt,
                                       xt_cap, st)))
    return rc;
  MlpArgsTc a{w0, b0, w1, b1, w2, b2, c0, dpe, c0 + dpe};
  PVDB_SMEM_ATTR(k_mlp_bwd_tc, int(kSmBwdBytes));
  launch_k(k_mlp_bwd_tc, grid, kBwdThreads, kSmBwdBytes, st, a, static_cast<const uint8_t*>(*blob),
           static_cast<const uint8_t*>(*xt), totals, rgb, grad_rgb, grad_k0, wpart, err,
           debug_spin_limit(kWaitIters), debug_hold_first());
  PVDB_CHECK_LAUNCH("k_mlp_bwd_tc");
  return PVDB_OK;
}

}  // namespace pvdb
