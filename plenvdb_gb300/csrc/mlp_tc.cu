// rgbnet on the 5th-generation tensor cores (tcgen05), BF16 operands with FP32
// accumulation in TMEM — the BF16 path of the colour MLP (dvgo.py:99-107,
// :354-362; renderer.cu:83-119).
//
// Forward, per 128-row tile (one CTA, 8 warps, persistent over tiles, 2 CTAs
// per SM, 256 TMEM columns each):
//   L0  Z0 = X[128x16] . W0k^T          one MMA (K=16; k0's 12 channels padded)
//       H0 = relu(Z0 + hpe[ray])         epilogue (hpe = W0[:,k0:]·PE + b0 per ray)
//   L1  Z1 = H0[128x128] . W1^T          8 MMAs (K=128 in steps of 16)
//       H1 = relu(Z1 + b1)               epilogue, written over H0
//   L2  Z2 = H1 . W2p^T                  8 MMAs, N=16 (3 outputs padded)
//       rgb = sigmoid(Z2 + b2)           epilogue (or the raw logits)
// One thread issues the MMAs; completion is signalled through an mbarrier
// (tcgen05.commit). Epilogues read TMEM with tcgen05.ld (warp w reads lanes
// 32*(w%4).., columns 64*(w/4)..), apply bias/activation in FP32 and store
// BF16 into shared memory in the canonical layout the next MMA reads.
#include <algorithm>

#include "march.cuh"
#include "tc.cuh"

namespace pvdb {

namespace {

constexpr int kW = 128;
constexpr int kTcThreads = 256;
// packed weight blob (bytes): W0k [128x16] | W1 [128x128] | W2p [16x128]
constexpr uint32_t kOffW0 = 0;
constexpr uint32_t kOffW1 = kOffW0 + 128 * 16 * 2;    // 4096
constexpr uint32_t kOffW2 = kOffW1 + 128 * 128 * 2;   // 36864
constexpr uint32_t kPackFwdBytes = kOffW2 + 16 * 128 * 2;  // 40960
// shared-memory layout of the forward kernel
constexpr uint32_t kSmX = kPackFwdBytes;              // X tile [128x16] bf16
constexpr uint32_t kSmH = kSmX + 128 * 16 * 2;        // H tile [128x128] bf16
constexpr uint32_t kSmB1 = kSmH + 128 * 128 * 2;      // b1 f32[128]
constexpr uint32_t kSmB2 = kSmB1 + 128 * 4;           // b2 f32[16]
constexpr uint32_t kSmBar = kSmB2 + 16 * 4;           // mbarrier (8 B)
constexpr uint32_t kSmTmem = kSmBar + 8;              // TMEM base address (4 B)
constexpr uint32_t kSmFlag = kSmTmem + 4;             // timeout flag (4 B)
constexpr uint32_t kSmFwdBytes = kSmFlag + 16;
constexpr uint32_t kTmemCols = 256;
constexpr uint32_t kWaitIters = 1u << 22;

struct MlpArgsTc {
  const float* w0; const float* b0;
  const float* w1; const float* b1;
  const float* w2; const float* b2;
  int c0, dpe, din;
};

// FP32 nn.Linear weights -> BF16 canonical K-major tiles (one thread per element).
__global__ void k_pack_fwd(MlpArgsTc a, uint8_t* blob) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  __nv_bfloat16* w0 = reinterpret_cast<__nv_bfloat16*>(blob + kOffW0);
  __nv_bfloat16* w1 = reinterpret_cast<__nv_bfloat16*>(blob + kOffW1);
  __nv_bfloat16* w2 = reinterpret_cast<__nv_bfloat16*>(blob + kOffW2);
  if (t < 128 * 16) {  // W0k[n][k] = w0[n][k] for k < c0, 0 otherwise
    const int n = t / 16, k = t % 16;
    w0[tc::kmaj(n, k, 16) / 2] = __float2bfloat16_rn(k < a.c0 ? a.w0[n * a.din + k] : 0.f);
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

__global__ void __launch_bounds__(kTcThreads, 2)
    k_mlp_fwd_tc(MlpArgsTc a, const uint8_t* __restrict__ blob, const float* __restrict__ k0,
                 const int32_t* __restrict__ ray, const float* __restrict__ hpe,
                 const uint32_t* __restrict__ totals, float* out, int out_logits, uint32_t* err) {
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
  // weights: 16-byte copies of the packed blob
  {
    const int4* src = reinterpret_cast<const int4*>(blob);
    int4* dst = reinterpret_cast<int4*>(sm);
    for (int i = tid; i < int(kPackFwdBytes / 16); i += kTcThreads) dst[i] = __ldg(src + i);
  }
  if (tid < 128) b1s[tid] = a.b1[tid];
  if (tid < 16) b2s[tid] = tid < 3 ? a.b2[tid] : 0.f;
  if (tid == 0) {
    *flag = 0;
    tc::mbar_init(bar, 1);
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
  uint32_t phase = 0;
  bool ok = true;
  for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
    const int64_t row0 = t * 128;
    // ---- X tile: row = tid/2, k = 8*(tid&1) .. +7
    {
      const int r = tid >> 1, kb = (tid & 1) * 8;
      const int64_t m = row0 + r;
      float v[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = (m < M && kb + i < a.c0) ? k0[m * a.c0 + kb + i] : 0.f;
      uint4 pk;
      pk.x = tc::pack_bf16(v[0], v[1]);
      pk.y = tc::pack_bf16(v[2], v[3]);
      pk.z = tc::pack_bf16(v[4], v[5]);
      pk.w = tc::pack_bf16(v[6], v[7]);
      *reinterpret_cast<uint4*>(sm + kSmX + tc::kmaj(r, kb, 16)) = pk;
    }
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
      tc::mma_bf16(tmem, tc::make_desc(sbase + kSmX, 128, 256), tc::make_desc(sbase + kOffW0, 128, 256),
                   id_n128, 0);
      tc::mma_commit(bar);
    }
    ok = wait_or_flag(bar, phase, flag, err);
    phase ^= 1;
    if (!ok) break;
    tc::fence_after();
    // ---- epilogue 0: H0 = relu(Z0 + hpe[ray])
    {
      const int64_t m = row0 + row;
      const bool valid = m < M;
      const float* hp = hpe + int64_t(valid ? ray[m] : 0) * kW + 64 * half;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        float v[16];
        tc::tmem_ld16(t_lane + uint32_t(64 * half + 16 * j), v);
        float hv[16];
#pragma unroll
        for (int i = 0; i < 16; i += 4) {
          const float4 h4 = valid ? __ldg(reinterpret_cast<const float4*>(hp + 16 * j + i))
                                  : make_float4(0.f, 0.f, 0.f, 0.f);
          hv[i] = h4.x; hv[i + 1] = h4.y; hv[i + 2] = h4.z; hv[i + 3] = h4.w;
        }
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          uint4 pk;
          const int o = 8 * c;
          pk.x = tc::pack_bf16(fmaxf(v[o] + hv[o], 0.f), fmaxf(v[o + 1] + hv[o + 1], 0.f));
          pk.y = tc::pack_bf16(fmaxf(v[o + 2] + hv[o + 2], 0.f), fmaxf(v[o + 3] + hv[o + 3], 0.f));
          pk.z = tc::pack_bf16(fmaxf(v[o + 4] + hv[o + 4], 0.f), fmaxf(v[o + 5] + hv[o + 5], 0.f));
          pk.w = tc::pack_bf16(fmaxf(v[o + 6] + hv[o + 6], 0.f), fmaxf(v[o + 7] + hv[o + 7], 0.f));
          *reinterpret_cast<uint4*>(sm + kSmH + tc::kmaj(row, 64 * half + 16 * j + o, 128)) = pk;
        }
      }
    }
    tc::fence_before();
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
#pragma unroll
      for (int s = 0; s < 8; ++s)
        tc::mma_bf16(tmem, tc::make_desc(sbase + kSmH + 256 * s, 128, 2048),
                     tc::make_desc(sbase + kOffW1 + 256 * s, 128, 2048), id_n128, s > 0);
      tc::mma_commit(bar);
    }
    ok = wait_or_flag(bar, phase, flag, err);
    phase ^= 1;
    if (!ok) break;
    tc::fence_after();
    // ---- epilogue 1: H1 = relu(Z1 + b1), over H0
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      float v[16];
      tc::tmem_ld16(t_lane + uint32_t(64 * half + 16 * j), v);
      const int cb = 64 * half + 16 * j;
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        uint4 pk;
        const int o = 8 * c;
        pk.x = tc::pack_bf16(fmaxf(v[o] + b1s[cb + o], 0.f), fmaxf(v[o + 1] + b1s[cb + o + 1], 0.f));
        pk.y = tc::pack_bf16(fmaxf(v[o + 2] + b1s[cb + o + 2], 0.f), fmaxf(v[o + 3] + b1s[cb + o + 3], 0.f));
        pk.z = tc::pack_bf16(fmaxf(v[o + 4] + b1s[cb + o + 4], 0.f), fmaxf(v[o + 5] + b1s[cb + o + 5], 0.f));
        pk.w = tc::pack_bf16(fmaxf(v[o + 6] + b1s[cb + o + 6], 0.f), fmaxf(v[o + 7] + b1s[cb + o + 7], 0.f));
        *reinterpret_cast<uint4*>(sm + kSmH + tc::kmaj(row, cb + o, 128)) = pk;
      }
    }
    tc::fence_before();
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
#pragma unroll
      for (int s = 0; s < 8; ++s)
        tc::mma_bf16(tmem + 128, tc::make_desc(sbase + kSmH + 256 * s, 128, 2048),
                     tc::make_desc(sbase + kOffW2 + 256 * s, 128, 2048), id_n16, s > 0);
      tc::mma_commit(bar);
    }
    ok = wait_or_flag(bar, phase, flag, err);
    phase ^= 1;
    if (!ok) break;
    tc::fence_after();
    // ---- epilogue 2: logits (warps 0-3 hold all 16 columns of their rows)
    if (half == 0) {
      float v[16];
      tc::tmem_ld16(t_lane + 128u, v);
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
    // a wait gave up: give the MMAs in flight one more bounded wait before the
    // TMEM they write is released
    tc::mbar_wait(bar, phase ^ 1u, kWaitIters);
  }
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

}  // namespace

// Packs the weights and runs the forward over rows k0rows [M, c0] (M = totals[1]).
int mlp_tc_forward_rows(const float* w0, const float* b0, const float* w1, const float* b1,
                        const float* w2, const float* b2, int c0, int dpe, const float* k0rows,
                        const int32_t* ray, const float* hpe, const uint32_t* totals, float* out,
                        int out_logits, void** blob, size_t* blob_cap, uint32_t* err,
                        cudaStream_t st) {
  if (c0 > 16) return set_error(PVDB_ERR_ARG, "the tensor-core rgbnet takes at most 16 k0 channels");
  int rc = dev_reserve(blob, blob_cap, kPackFwdBytes);
  if (rc) return rc;
  MlpArgsTc a{w0, b0, w1, b1, w2, b2, c0, dpe, c0 + dpe};
  k_pack_fwd<<<ceil_div(128 * 128, 256), 256, 0, st>>>(a, static_cast<uint8_t*>(*blob));
  PVDB_CHECK_LAUNCH("k_pack_fwd");
  PVDB_CHECK_CUDA(cudaFuncSetAttribute(k_mlp_fwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(kSmFwdBytes)));
  k_mlp_fwd_tc<<<2 * num_sms(), kTcThreads, kSmFwdBytes, st>>>(
      a, static_cast<const uint8_t*>(*blob), k0rows, ray, hpe, totals, out, out_logits, err);
  PVDB_CHECK_LAUNCH("k_mlp_fwd_tc");
  return PVDB_OK;
}

}  // namespace pvdb
