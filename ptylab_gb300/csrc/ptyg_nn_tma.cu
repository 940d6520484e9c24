// 3x3 'same' convolution (the warm-start network's forward and data-gradient
// GEMMs) with TMA operand loads and tcgen05 MMAs.
//
// Y[m, co] = sum_{tap, c} X[pixel(m) + tap, c] W[co, tap * Ct + c]: an
// implicit GEMM with M = pixels, N = Co, K = 9 Ct.  A CTA computes a tile of
// 128 pixels, a BW x BH block of one image (BW = min(W, 128)), against BN
// output channels.  Per K block (one tap, BK channels of one input tensor):
//   A tile: one 4-D TMA box (BK channels, BW, BH, 1 image) of the NHWC
//           activations at (c, x0 + dx, y0 + dy, b); the rows and columns the
//           tap shifts outside the image arrive as zeros (out-of-bounds fill),
//           which is the convolution's zero padding;
//   B tile: one 2-D TMA box (BK, BN) of the K-major weights.
// Both land in the canonical K-major layout with the swizzle of their row
// width (BK * 2 bytes: 128, 64 or 32), which is how the tensor map writes
// them and how the MMA descriptors read them.
//
// Roles (128 threads): thread 0 issues the TMA loads into a 4-stage ring,
// thread 32 issues the MMAs (accumulator in tensor memory) and commits each
// stage back to the producer, and all four warps read the accumulator out
// (warp w owns tensor-memory lanes 32w..32w+31 = tile rows) for the bias /
// ReLU / bf16 or f32 epilogue.  Every wait is bounded; a wait that gives up
// sets *status, stops issuing work, and the CTA still waits (bounded) for
// the copies and MMAs it issued before it frees tensor memory and exits.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "ptyg_nn_tma.cuh"

namespace ptyg {
namespace nn {

namespace {

typedef __nv_bfloat16 bf16;
#define TMA_DEV __device__ __forceinline__

constexpr int TBM = 128, TSTAGES = 4;

TMA_DEV uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

TMA_DEV bool wait_parity(uint32_t bar, uint32_t phase, long long limit) {
  uint32_t done = 0;
  for (long long i = 0; i < limit && !done; ++i) {
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
  }
  return done != 0;
}

TMA_DEV void expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

TMA_DEV void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];\n" ::"r"(dst),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}

TMA_DEV void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::
          "r"(dst),
      "l"(map), "r"(c0), "r"(c1), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor for a K-major operand whose rows are
// `row_bytes` (= the swizzle width: 32, 64 or 128) apart: start >> 4, leading
// offset 16 bytes (unused by swizzled K-major layouts), stride between
// 8-row groups = 8 * row_bytes, version 1, swizzle mode in bits 61-63
// (6 = 32 B, 4 = 64 B, 2 = 128 B).
TMA_DEV uint64_t sw_desc(uint32_t addr, uint32_t row_bytes) {
  const uint64_t mode = row_bytes == 128 ? 2 : row_bytes == 64 ? 4 : 6;
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)(((8 * row_bytes) >> 4) & 0x3FFF) << 32) |
         ((uint64_t)1 << 46) | (mode << 61);
}

// kind::f16 instruction descriptor: f32 D, bf16 A and B, both K-major.
__host__ __device__ constexpr uint32_t idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

template <int BN>
__global__ void __launch_bounds__(128, 1)
    conv3_tma_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmA1,
                     const __grid_constant__ CUtensorMap tmB, const ConvTmaArgs g) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = su32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;  // swizzle atoms need 1024-byte alignment
  const int BK = g.BK;
  const uint32_t A_BYTES = (uint32_t)(TBM * BK * 2), B_BYTES = (uint32_t)(BN * BK * 2);
  const uint32_t STAGE = A_BYTES + B_BYTES;
  const uint32_t bars = base + TSTAGES * STAGE;  // full[4], empty[4], done
  auto full = [&](int s) { return bars + 8u * (uint32_t)s; };
  auto empty = [&](int s) { return bars + 8u * (uint32_t)(TSTAGES + s); };
  const uint32_t done = bars + 8u * (2 * TSTAGES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem_raw + (done + 8u - raw));

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tile = blockIdx.x;
  const int tx = tile % g.tilesX, ty = (tile / g.tilesX) % g.tilesY, b = tile / (g.tilesX * g.tilesY);
  const int x0 = tx * g.BW, y0 = ty * g.BH, n0 = blockIdx.y * BN;
  const int Ct = g.C0 + g.C1;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(su32(tmem_slot)),
                 "r"(BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  if (tid == 0) {
    for (int s = 0; s < 2 * TSTAGES + 1; ++s) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bars + 8u * s));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    asm volatile("prefetch.tensormap [%0];\n" ::"l"(&tmA) : "memory");
    asm volatile("prefetch.tensormap [%0];\n" ::"l"(&tmB) : "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n");
  const uint32_t tmem = *tmem_slot;
  bool ok = true;

  if (tid == 0) {
    // ---- producer
    int issued = 0;
    // fault injection (failure-detection tests): wait on stage 0's empty
    // barrier before any copy is issued; nothing arrives there, the bounded
    // wait runs out and nothing is issued (the MMA thread's first wait then
    // runs out too)
    if (g.stall && !wait_parity(empty(0), 0u, g.waitLimit)) ok = false;
    for (int kb = 0; ok && kb < g.nkb; ++kb) {
      const int s = kb % TSTAGES;
      if (kb >= TSTAGES && !wait_parity(empty(s), (uint32_t)((kb / TSTAGES - 1) & 1), g.waitLimit)) {
        ok = false;
        break;
      }
      const int tap = kb / g.kbPerTap, c = (kb - tap * g.kbPerTap) * BK;
      const int dy = tap / 3 - 1, dx = tap - (tap / 3) * 3 - 1;
      const uint32_t sA = base + (uint32_t)s * STAGE, sB = sA + A_BYTES;
      expect_tx(full(s), STAGE);
      if (c < g.C0)
        tma_load_4d(sA, &tmA, c, x0 + dx, y0 + dy, b, full(s));
      else
        tma_load_4d(sA, &tmA1, c - g.C0, x0 + dx, y0 + dy, b, full(s));
      tma_load_2d(sB, &tmB, tap * Ct + c, n0, full(s));
      ++issued;
    }
    // every issued copy lands before the CTA may exit (on the normal path the
    // MMA thread has consumed them all; these waits then return at once)
    for (int kb = issued > TSTAGES ? issued - TSTAGES : 0; kb < issued; ++kb)
      if (!wait_parity(full(kb % TSTAGES), (uint32_t)((kb / TSTAGES) & 1), g.waitLimit)) ok = false;
  } else if (tid == 32) {
    // ---- MMA issuer
    constexpr uint32_t id = idesc(TBM, BN);
    const uint32_t rowb = (uint32_t)(BK * 2);
    for (int kb = 0; kb < g.nkb; ++kb) {
      const int s = kb % TSTAGES;
      if (!wait_parity(full(s), (uint32_t)((kb / TSTAGES) & 1), g.waitLimit)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n");
      const uint32_t sA = base + (uint32_t)s * STAGE, sB = sA + A_BYTES;
      for (int kk = 0; kk < BK / 16; ++kk) {
        // K = 16 elements = 32 bytes further along each swizzled row
        const uint64_t ad = sw_desc(sA + 32u * kk, rowb), bd = sw_desc(sB + 32u * kk, rowb);
        const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(id), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(empty(s)));
    }
    // completes once every MMA issued above has (also after a failed wait)
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(done));
  }
  if (!wait_parity(done, 0, g.waitLimit)) ok = false;
  asm volatile("tcgen05.fence::after_thread_sync;\n");
  ok = __syncthreads_and(ok);
  if (!ok) {
    if (tid == 0 && g.status) atomicExch(g.status, 1);
  } else {
    // tensor-memory lane = tile row r = pixel (b, y0 + r / BW, x0 + r % BW)
    const int r = warp * 32 + lane;
    const int y = y0 + r / g.BW, x = x0 + r % g.BW;
    const size_t gm = ((size_t)b * g.H + y) * g.W + x;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 32) {
      if (n0 + c0 >= g.N) break;
      uint32_t v32[32];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
          : "=r"(v32[0]), "=r"(v32[1]), "=r"(v32[2]), "=r"(v32[3]), "=r"(v32[4]), "=r"(v32[5]), "=r"(v32[6]),
            "=r"(v32[7]), "=r"(v32[8]), "=r"(v32[9]), "=r"(v32[10]), "=r"(v32[11]), "=r"(v32[12]), "=r"(v32[13]),
            "=r"(v32[14]), "=r"(v32[15]), "=r"(v32[16]), "=r"(v32[17]), "=r"(v32[18]), "=r"(v32[19]), "=r"(v32[20]),
            "=r"(v32[21]), "=r"(v32[22]), "=r"(v32[23]), "=r"(v32[24]), "=r"(v32[25]), "=r"(v32[26]), "=r"(v32[27]),
            "=r"(v32[28]), "=r"(v32[29]), "=r"(v32[30]), "=r"(v32[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      const int nb = n0 + c0;
      float v[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        v[j] = __uint_as_float(v32[j]);
        if (g.bias && nb + j < g.N) v[j] += g.bias[nb + j];
        if (g.out && g.relu) v[j] = fmaxf(v[j], 0.f);
      }
      const bool full_row = nb + 32 <= g.N && (g.N & 7) == 0;
      if (!g.out) {
        float* crow = g.C + gm * g.N + nb;
        if (full_row) {
#pragma unroll
          for (int j = 0; j < 32; j += 4)
            *reinterpret_cast<float4*>(crow + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
        } else {
          for (int j = 0; j < 32 && nb + j < g.N; ++j) crow[j] = v[j];
        }
      } else {
        bf16* orow = g.out + gm * g.N + nb;
        if (full_row) {
#pragma unroll
          for (int j = 0; j < 32; j += 8) {
            uint4 q;
            __nv_bfloat162 h0 = __floats2bfloat162_rn(v[j], v[j + 1]), h1 = __floats2bfloat162_rn(v[j + 2], v[j + 3]);
            __nv_bfloat162 h2 = __floats2bfloat162_rn(v[j + 4], v[j + 5]), h3 = __floats2bfloat162_rn(v[j + 6], v[j + 7]);
            q.x = *reinterpret_cast<uint32_t*>(&h0);
            q.y = *reinterpret_cast<uint32_t*>(&h1);
            q.z = *reinterpret_cast<uint32_t*>(&h2);
            q.w = *reinterpret_cast<uint32_t*>(&h3);
            *reinterpret_cast<uint4*>(orow + j) = q;
          }
        } else {
          for (int j = 0; j < 32 && nb + j < g.N; ++j) orow[j] = __float2bfloat16(v[j]);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(BN));
}

// ---------------------------------------------------------------- host side
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

CUtensorMapSwizzle swizzle_for(int BK) {
  return BK == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : BK == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B;
}

// NHWC activations [Bn][H][W][C] as a 4-D map (C innermost), box BK x BW x BH x 1
bool encode_act(CUtensorMap* m, const void* X, int C, int Bn, int H, int W, int BK, int BW, int BH) {
  const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)Bn};
  const cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
  const cuuint32_t box[4] = {(cuuint32_t)BK, (cuuint32_t)BW, (cuuint32_t)BH, 1};
  const cuuint32_t es[4] = {1, 1, 1, 1};
  return encode_fn()(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(X), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(BK), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// K-major weights [Co][K] as a 2-D map, box BK x BN
bool encode_wts(CUtensorMap* m, const void* Wt, int K, int Co, int BK, int BN) {
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)Co};
  const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  const cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)BN};
  const cuuint32_t es[2] = {1, 1};
  return encode_fn()(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(Wt), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(BK), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
cudaError_t launch_bn(const CUtensorMap& a, const CUtensorMap& a1, const CUtensorMap& w, const ConvTmaArgs& g,
                      int tiles, cudaStream_t st) {
  const size_t smem = (size_t)TSTAGES * (TBM * g.BK * 2 + BN * g.BK * 2) + 1024 + 8 * (2 * TSTAGES + 2);
  cudaError_t e = cudaFuncSetAttribute(conv3_tma_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid(tiles, (g.N + BN - 1) / BN);
  conv3_tma_kernel<BN><<<grid, 128, smem, st>>>(a, a1, w, g);
  return cudaGetLastError();
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace

cudaError_t conv3_tma(const void* X, const void* X1, int C0, int C1, int Bn, int H, int W, const void* Wt, int Co,
                      float* C, void* out, const float* bias, int relu, int* status, cudaStream_t st) {
  // eligibility: one K block never straddles the two inputs, the pixel tile
  // is a whole block of one image, the maps' addresses and strides are
  // 16-byte multiples
  int BK = C0 < 64 ? C0 : 64;
  if (C1 > 0 && C1 < BK) BK = C1;
  if (BK != 16 && BK != 32 && BK != 64) return cudaErrorNotSupported;
  if (C0 % BK || (C1 % BK) || Co < 1 || Co > 256) return cudaErrorNotSupported;
  const int BW = W < TBM ? W : TBM;
  if (TBM % BW || W % BW) return cudaErrorNotSupported;
  const int BH = TBM / BW;
  if (H % BH) return cudaErrorNotSupported;
  if (!aligned16(X) || (C1 && !aligned16(X1)) || !aligned16(Wt) || !encode_fn()) return cudaErrorNotSupported;
  const int K = 9 * (C0 + C1);
  const int BN = Co <= 32 ? 32 : Co <= 64 ? 64 : Co <= 128 ? 128 : 256;
  CUtensorMap ma, ma1, mw;
  if (!encode_act(&ma, X, C0, Bn, H, W, BK, BW, BH)) return cudaErrorNotSupported;
  if (!encode_act(&ma1, C1 ? X1 : X, C1 ? C1 : C0, Bn, H, W, BK, BW, BH)) return cudaErrorNotSupported;
  if (!encode_wts(&mw, Wt, K, Co, BK, BN)) return cudaErrorNotSupported;
  ConvTmaArgs g = {};
  g.C0 = C0;
  g.C1 = C1;
  g.BK = BK;
  g.H = H;
  g.W = W;
  g.BW = BW;
  g.BH = BH;
  g.tilesX = W / BW;
  g.tilesY = H / BH;
  g.N = Co;
  g.kbPerTap = (C0 + C1) / BK;
  g.nkb = 9 * g.kbPerTap;
  g.C = C;
  g.out = (bf16*)out;
  g.bias = bias;
  g.relu = relu;
  g.status = status;
  wait_policy(&g.waitLimit, &g.stall);
  const int tiles = Bn * g.tilesX * g.tilesY;
  switch (BN) {
    case 32: return launch_bn<32>(ma, ma1, mw, g, tiles, st);
    case 64: return launch_bn<64>(ma, ma1, mw, g, tiles, st);
    case 128: return launch_bn<128>(ma, ma1, mw, g, tiles, st);
    default: return launch_bn<256>(ma, ma1, mw, g, tiles, st);
  }
}

}  // namespace nn
}  // namespace ptyg
