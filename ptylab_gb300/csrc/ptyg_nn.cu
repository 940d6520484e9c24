// Kernels of the learned warm start: a small convolutional encoder-decoder
// trained and evaluated on the GPU.  No counterpart in PtyLab.
//
// Convolutions are implicit GEMMs on the 5th-generation tensor cores:
// tcgen05.mma (kind::f16, BF16 operands, FP32 accumulator in tensor memory),
// issued by one thread per CTA, operands staged in shared memory in the
// canonical K-major layout without swizzle (8-row x 16-byte core matrices),
// two pipeline stages so the next tile loads while the tensor core works on
// the current one.  The A-operand loader either reads a dense K-major matrix
// or gathers 3x3 'same' convolution patches straight from NHWC activations
// (optionally the channel concatenation of two tensors, the decoder's skip
// connections), 8 channels (16 bytes) per load.
//
//   forward            Y[m, co]  = sum_k Xpatch[m, k] W[co, k]         (conv A-loader)
//   backward, data     dX[m, ci] = sum_k dYpatch[m, k] W'[ci, k]       (conv A-loader on dY,
//                      W' = W with the taps flipped and in/out channels swapped)
//   backward, weights  dW^T[k, co] = sum_m XcolT[k, m] dYT[co, m]      (dense, split over m)
//
// Every wait on a tensor-core completion is bounded: after the limit the
// kernel records an error and skips its remaining MMAs, so a fault can never
// hang the device.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdio>

#include "ptyg.h"
#include "ptyg_nn_tma.cuh"
#include "ptyg_ops.cuh"

namespace ptyg {
namespace nn {

// Bounded-wait policy of every network launch (ptyg_nn_set_wait_policy): the
// poll limit, and how many of the next launches start with the injected wait.
static std::atomic<long long> g_wait_limit{1LL << 26};
static std::atomic<int> g_stall_launches{0};

void wait_policy(long long* limit, int* stall) {
  *limit = g_wait_limit.load();
  int n = g_stall_launches.load();
  while (n > 0 && !g_stall_launches.compare_exchange_weak(n, n - 1)) {
  }
  *stall = n > 0 ? 1 : 0;
}

typedef __nv_bfloat16 bf16;

#define NN_DEV __device__ __forceinline__

NN_DEV uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// tcgen05 shared-memory matrix descriptor: start >> 4 in [0,14), leading
// (K-direction) byte offset >> 4 in [16,30), stride (M/N-direction) byte
// offset >> 4 in [32,46), descriptor version 1 in [46,48), no swizzle.
NN_DEV uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor, kind::f16: FP32 D (bits 4-5 = 1), BF16 A and B
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 in bits 17-22, M >> 4 in 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

constexpr int BM = 128, BK = 64, STAGES = 4;

enum AMode { A_DENSE = 0, A_CONV3 = 1 };
enum Epilogue { EPI_F32 = 0, EPI_BF16 = 1 };

struct GemmArgs {
  // A: dense [M, K] bf16 (lda = K), or NHWC activations for the 3x3 gather
  const bf16* A;
  const bf16* A1;    // conv: second input of a channel concatenation (or null)
  int C0, C1;        // conv: channels of A and A1 (both multiples of 8)
  int H, W;          // conv: image size (M = batch * H * W)
  const bf16* B;     // [N, K] bf16
  int M, N, K;       // K: a multiple of 8
  int kSplit;        // K range per blockIdx.z (multiple of BK); gridDim.z partials
  int epi;           // EPI_F32: C[z][M][N] f32 partials; EPI_BF16: out bf16 [M, N]
  float* C;
  bf16* out;
  const float* bias; // + bias[n] (single K split only)
  int relu;          // EPI_BF16: max(0, .)
  int* status;       // set to 1 when a wait gives up
  long long waitLimit;  // try_wait polls before a wait is declared lost
  int stall;         // fault injection: first wait on a barrier nothing arrives at
};

NN_DEV bool mbar_wait(uint32_t bar, uint32_t phase, long long limit) {
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

// 16-byte asynchronous copy global -> shared; src_bytes = 0 writes zeros
NN_DEV void cp16(uint32_t dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
NN_DEV void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
NN_DEV void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Thread t of the 128 stages, for every K block, the 16-byte chunks of tile
// rows t/8 + 16 i (A: i < 8; B: i < BN/16), K chunk t % 8.  The pixel
// coordinates of its A rows are fixed for the whole tile, so the conv gather
// costs one division per K block, not per chunk.
struct RowInfo {
  int y[8], x[8];   // conv: pixel row/column (y = -1e6 for rows past M)
  size_t base[8];   // conv: pixel index of (b, 0, 0); dense: row offset m * K
};

template <int BN, int AMODE>
NN_DEV void load_stage(const GemmArgs& g, const RowInfo& ri, uint32_t sA, uint32_t sB, int k0, int kEnd, int n0,
                       int tid) {
  const int kc = tid & 7, rb = tid >> 3;
  const int k = k0 + kc * 8;
  const uint32_t coff = (uint32_t)(kc * 128);
  if (AMODE == A_DENSE) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = rb + 16 * i;
      const bool ok = ri.y[i] >= 0 && k < g.K;
      const bf16* src = ok ? g.A + ri.base[i] + k : g.A;
      cp16(sA + (uint32_t)((r >> 3) * (BK / 8) * 128) + coff + (uint32_t)((r & 7) * 16), src, ok ? 16u : 0u);
    }
  } else {
    const int Ct = g.C0 + g.C1;
    const int tap = k / Ct, c = k - tap * Ct;
    const int dy = tap / 3 - 1, dx = tap - (tap / 3) * 3 - 1;
    const bool kin = k < g.K;
    const bool first = c < g.C0;
    const bf16* X = first ? g.A : g.A1;
    const int Cx = first ? g.C0 : g.C1;
    const int cx = first ? c : c - g.C0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = rb + 16 * i;
      const int yy = ri.y[i] + dy, xx = ri.x[i] + dx;
      const bool ok = kin && yy >= 0 && yy < g.H && xx >= 0 && xx < g.W;
      const bf16* src = ok ? X + (ri.base[i] + (size_t)yy * g.W + xx) * Cx + cx : g.A;
      cp16(sA + (uint32_t)((r >> 3) * (BK / 8) * 128) + coff + (uint32_t)((r & 7) * 16), src, ok ? 16u : 0u);
    }
  }
#pragma unroll
  for (int i = 0; i < BN / 16; ++i) {
    const int r = rb + 16 * i;
    const int gn = n0 + r;
    const bool ok = gn < g.N && k < kEnd;
    const bf16* src = ok ? g.B + (size_t)gn * g.K + k : g.B;
    cp16(sB + (uint32_t)((r >> 3) * (BK / 8) * 128) + coff + (uint32_t)((r & 7) * 16), src, ok ? 16u : 0u);
  }
}

template <int BN, int AMODE>
__global__ void __launch_bounds__(128, 1) gemm_kernel(const GemmArgs g) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // stage s: A tile (BM x BK) then B tile (BN x BK), K-major no-swizzle core matrices
  constexpr int A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2, STAGE_BYTES = A_BYTES + B_BYTES;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem_raw + STAGES * STAGE_BYTES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar + STAGES);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int kBegin = blockIdx.z * g.kSplit;
  const int kEnd = min(g.K, kBegin + g.kSplit);
  const int nkb = (kEnd - kBegin + BK - 1) / BK;
  const uint32_t smem0 = smem_u32(smem_raw);

  RowInfo ri;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int m = m0 + (tid >> 3) + 16 * i;
    if (m >= g.M) {
      ri.y[i] = -(1 << 20);
      ri.x[i] = 0;
      ri.base[i] = 0;
    } else if (AMODE == A_DENSE) {
      ri.y[i] = 0;
      ri.x[i] = 0;
      ri.base[i] = (size_t)m * g.K;
    } else {
      const int hw = g.H * g.W;
      const int b = m / hw, rem = m - b * hw;
      ri.y[i] = rem / g.W;
      ri.x[i] = rem - ri.y[i] * g.W;
      ri.base[i] = (size_t)b * hw;
    }
  }

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                 "r"(BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(mbar + s)));
    asm volatile("fence.mbarrier_init.release.cluster;\n");
  }
  // prologue: stages 0 .. STAGES-2 in flight
#pragma unroll
  for (int s = 0; s < STAGES - 1; ++s) {
    if (s < nkb)
      load_stage<BN, AMODE>(g, ri, smem0 + s * STAGE_BYTES, smem0 + s * STAGE_BYTES + A_BYTES, kBegin + s * BK, kEnd, n0,
                            tid);
    cp_commit();
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n");
  const uint32_t tmem = *tmem_slot;
  constexpr uint32_t idesc = idesc_bf16(BM, BN);
  bool ok = true;
  // fault injection (failure-detection tests): wait on stage 0's barrier
  // before any MMA is committed to it; nothing arrives, the bounded wait runs
  // out and the launch reports it, with no copy or MMA of its own in flight
  // but the prologue's cp.async groups, which are waited for below
  if (g.stall) ok = __syncthreads_and(mbar_wait(smem_u32(mbar), 0u, g.waitLimit));
  for (int kb = 0; kb < nkb; ++kb) {
    const int s = kb % STAGES;
    // refill the stage the MMAs of kb - 1 read, once they are done
    const int kn = kb + STAGES - 1;
    if (kn < nkb) {
      const int sn = kn % STAGES;
      if (kb >= 1 && !mbar_wait(smem_u32(mbar + sn), (uint32_t)(((kb - 1) / STAGES) & 1), g.waitLimit)) ok = false;
      if (ok)
        load_stage<BN, AMODE>(g, ri, smem0 + sn * STAGE_BYTES, smem0 + sn * STAGE_BYTES + A_BYTES, kBegin + kn * BK,
                              kEnd, n0, tid);
    }
    cp_commit();
    cp_wait<STAGES - 1>();  // this thread's copies for stage s have landed
    // generic-proxy writes -> visible to the tensor core (async proxy)
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n");
      const uint32_t sA = smem0 + s * STAGE_BYTES, sB = sA + A_BYTES;
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk) {
        // K = 16 per MMA: two core-matrix columns, 128 bytes apart
        const uint64_t ad = smem_desc(sA + kk * 256, 128, (BK / 8) * 128);
        const uint64_t bd = smem_desc(sB + kk * 256, 128, (BK / 8) * 128);
        const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
          smem_u32(mbar + s)));
    }
  }
  cp_wait<0>();
  // drain: the last MMAs (each stage's last commit not yet waited for)
  if (ok) {
    // the loop waited for commit j exactly when j + STAGES < nkb (before refilling its stage)
    for (int j = max(0, nkb - STAGES); j < nkb; ++j)
      if (!mbar_wait(smem_u32(mbar + (j % STAGES)), (uint32_t)((j / STAGES) & 1), g.waitLimit)) ok = false;
  }
  asm volatile("tcgen05.fence::after_thread_sync;\n");
  ok = __syncthreads_and(ok);
  if (!ok) {
    if (tid == 0 && g.status) atomicExch(g.status, 1);
  } else if (nkb > 0) {
    // accumulator: TMEM lane = tile row (warp w owns lanes 32w..32w+31), column = n
    const int gm = m0 + warp * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 32) {
      uint32_t r[32];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
            "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (gm >= g.M) continue;
      const int nb = n0 + c0;
      float v[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        v[j] = __uint_as_float(r[j]);
        if (g.bias && nb + j < g.N) v[j] += g.bias[nb + j];
        if (g.epi == EPI_BF16 && g.relu) v[j] = fmaxf(v[j], 0.f);
      }
      const bool full = nb + 32 <= g.N && (g.N & 7) == 0;
      if (g.epi == EPI_F32) {
        float* crow = g.C + ((size_t)blockIdx.z * g.M + gm) * g.N + nb;
        if (full) {
#pragma unroll
          for (int j = 0; j < 32; j += 4) *reinterpret_cast<float4*>(crow + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
        } else {
          for (int j = 0; j < 32 && nb + j < g.N; ++j) crow[j] = v[j];
        }
      } else {
        bf16* orow = g.out + (size_t)gm * g.N + nb;
        if (full) {
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

// ------------------------------------------------------------------ weight gradients
// dW[co][k] = sum_pixels dY[pixel][co] P[pixel][k], P the 3x3 patch matrix of X
// (or a dense [pixels][K] matrix): a GEMM whose contraction runs over pixels,
// with both operands staged MN-major (the 16 contiguous bytes run along co,
// resp. k), so dY and X are read in their NHWC order with no transposes and no
// materialised patch matrix.  MN-major no-swizzle core matrices: 8 K rows
// (pixels) x 16 bytes (8 co, resp. 8 k); core (mn, kc) at (kc * R/8 + mn) * 128
// bytes; the descriptor's leading offset is the K-direction stride (R/8 * 128),
// the stride offset the MN-direction one (128 bytes).  Every MMA reads within
// its stage: largest offset (2 kk + 1) * R/8 * 128 + (R/8 - 1) * 128 + 127 =
// R * 128 - 1 at kk = 3, the size of an R x 64 tile.
struct DwArgs {
  const bf16* dY;    // [P][Co] (row stride Co)
  int Co;
  const bf16* X;     // conv: NHWC [P][C0] (+ X1 [P][C1]); dense: [P][K]
  const bf16* X1;
  int C0, C1;
  int lgW, lgHW, H, W;  // conv: log2 of the width and of the image size (powers of two)
  int K;             // columns of dW (9 (C0 + C1) for conv)
  int P;             // pixels (the contraction)
  int pSplit;        // pixels per blockIdx.z (multiple of BK)
  float* C;          // [splits][Co][K]
  int* status;
  long long waitLimit;  // try_wait polls before a wait is declared lost
  int stall;         // fault injection: first wait on a barrier nothing arrives at
};

// The B-operand column a thread loads is the same for every pixel block
// (its 8 k values at n0 + (t % (BN/8)) * 8): tap, channel and source tensor
// are worked out once.
struct DwCol {
  bool kin;
  int dy, dx, Cx, cx;
  const bf16* X;
};

template <int BN, bool CONV>
NN_DEV DwCol dw_column(const DwArgs& g, int k0, int tid) {
  DwCol d;
  const int k = k0 + (tid % (BN / 8)) * 8;
  d.kin = k < g.K;
  if (!CONV) {
    d.dy = d.dx = 0;
    d.Cx = g.K;
    d.cx = k;
    d.X = g.X;
  } else {
    const int Ct = g.C0 + g.C1;
    const int tap = d.kin ? k / Ct : 0, c = d.kin ? k - tap * Ct : 0;
    d.dy = tap / 3 - 1;
    d.dx = tap - (tap / 3) * 3 - 1;
    const bool first = c < g.C0;
    d.X = first ? g.X : g.X1;
    d.Cx = first ? g.C0 : g.C1;
    d.cx = first ? c : c - g.C0;
  }
  return d;
}

template <int BN, bool CONV>
NN_DEV void dw_load_stage(const DwArgs& g, const DwCol& col, uint32_t sA, uint32_t sB, int p0, int pEnd, int co0,
                          int tid) {
  // A: 64 pixels x 128 co, chunk (pixel p, co chunk mc): thread t -> mc = t % 16, p = t / 16 + 8 i
  {
    const int mc = tid & 15;
    const int co = co0 + mc * 8;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int p = (tid >> 4) + 8 * i;
      const int pix = p0 + p;
      const bool ok = pix < pEnd && co < g.Co;
      const bf16* src = ok ? g.dY + (size_t)pix * g.Co + co : g.dY;
      cp16(sA + (uint32_t)(((p >> 3) * (BM / 8) + mc) * 128 + (p & 7) * 16), src, ok ? 16u : 0u);
    }
  }
  // B: 64 pixels x BN k, chunk (pixel p, k chunk nc): thread t -> nc = t % (BN/8), p = t / (BN/8) + (128/(BN/8)) i
  {
    constexpr int NCH = BN / 8, PSTEP = 128 / NCH, NI = 64 / PSTEP;
    const int nc = tid % NCH;
#pragma unroll
    for (int i = 0; i < NI; ++i) {
      const int p = tid / NCH + PSTEP * i;
      const int pix = p0 + p;
      bool ok = col.kin && pix < pEnd;
      const bf16* src = g.X;
      if (ok) {
        if (!CONV) {
          src = col.X + (size_t)pix * col.Cx + col.cx;
        } else {
          const int b = pix >> g.lgHW, rem = pix & ((1 << g.lgHW) - 1);
          const int y = (rem >> g.lgW) + col.dy, x = (rem & ((1 << g.lgW) - 1)) + col.dx;
          ok = y >= 0 && y < g.H && x >= 0 && x < g.W;
          const size_t q = ((size_t)b << g.lgHW) + ((size_t)y << g.lgW) + x;
          src = ok ? col.X + q * col.Cx + col.cx : g.X;
        }
      }
      cp16(sB + (uint32_t)(((p >> 3) * NCH + nc) * 128 + (p & 7) * 16), src, ok ? 16u : 0u);
    }
  }
}

template <int BN, bool CONV>
__global__ void __launch_bounds__(128, 1) dw_kernel(const DwArgs g) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  constexpr int A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2, STAGE_BYTES = A_BYTES + B_BYTES;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem_raw + STAGES * STAGE_BYTES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar + STAGES);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int co0 = blockIdx.x * BM, k0 = blockIdx.y * BN;
  const int pBegin = blockIdx.z * g.pSplit;
  const int pEnd = min(g.P, pBegin + g.pSplit);
  const int nkb = (pEnd - pBegin + BK - 1) / BK;
  const uint32_t smem0 = smem_u32(smem_raw);
  const DwCol col = dw_column<BN, CONV>(g, k0, tid);

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                 "r"(BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(mbar + s)));
    asm volatile("fence.mbarrier_init.release.cluster;\n");
  }
#pragma unroll
  for (int s = 0; s < STAGES - 1; ++s) {
    if (s < nkb)
      dw_load_stage<BN, CONV>(g, col, smem0 + s * STAGE_BYTES, smem0 + s * STAGE_BYTES + A_BYTES, pBegin + s * BK, pEnd,
                              co0, tid);
    cp_commit();
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n");
  const uint32_t tmem = *tmem_slot;
  // MN-major A (bit 15) and B (bit 16)
  constexpr uint32_t idesc = idesc_bf16(BM, BN) | (1u << 15) | (1u << 16);
  constexpr uint32_t LBO_A = (BM / 8) * 128, LBO_B = (BN / 8) * 128;
  bool ok = true;
  // fault injection (failure-detection tests): wait on stage 0's barrier
  // before any MMA is committed to it; nothing arrives, the bounded wait runs
  // out and the launch reports it, with no copy or MMA of its own in flight
  // but the prologue's cp.async groups, which are waited for below
  if (g.stall) ok = __syncthreads_and(mbar_wait(smem_u32(mbar), 0u, g.waitLimit));
  for (int kb = 0; kb < nkb; ++kb) {
    const int s = kb % STAGES;
    const int kn = kb + STAGES - 1;
    if (kn < nkb) {
      const int sn = kn % STAGES;
      if (kb >= 1 && !mbar_wait(smem_u32(mbar + sn), (uint32_t)(((kb - 1) / STAGES) & 1), g.waitLimit)) ok = false;
      if (ok)
        dw_load_stage<BN, CONV>(g, col, smem0 + sn * STAGE_BYTES, smem0 + sn * STAGE_BYTES + A_BYTES,
                                pBegin + kn * BK, pEnd, co0, tid);
    }
    cp_commit();
    cp_wait<STAGES - 1>();
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n");
      const uint32_t sA = smem0 + s * STAGE_BYTES, sB = sA + A_BYTES;
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk) {
        const uint64_t ad = smem_desc(sA + kk * 2 * LBO_A, LBO_A, 128);
        const uint64_t bd = smem_desc(sB + kk * 2 * LBO_B, LBO_B, 128);
        const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
          smem_u32(mbar + s)));
    }
  }
  cp_wait<0>();
  if (ok) {
    for (int j = max(0, nkb - STAGES); j < nkb; ++j)
      if (!mbar_wait(smem_u32(mbar + (j % STAGES)), (uint32_t)((j / STAGES) & 1), g.waitLimit)) ok = false;
  }
  asm volatile("tcgen05.fence::after_thread_sync;\n");
  ok = __syncthreads_and(ok);
  if (!ok) {
    if (tid == 0 && g.status) atomicExch(g.status, 1);
  } else {
    const int co = co0 + warp * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 32) {
      uint32_t r[32];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
            "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (co < g.Co) {
        float* crow = g.C + ((size_t)blockIdx.z * g.Co + co) * g.K + k0 + c0;
        const bool full = k0 + c0 + 32 <= g.K && (g.K & 3) == 0;
        if (full) {
#pragma unroll
          for (int j = 0; j < 32; j += 4)
            *reinterpret_cast<float4*>(crow + j) = make_float4(__uint_as_float(r[j]), __uint_as_float(r[j + 1]),
                                                               __uint_as_float(r[j + 2]), __uint_as_float(r[j + 3]));
        } else {
          for (int j = 0; j < 32 && k0 + c0 + j < g.K; ++j) crow[j] = __uint_as_float(r[j]);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(BN));
}

template <int BN, bool CONV>
static cudaError_t launch_dw_t(const DwArgs& g, int splits, cudaStream_t st) {
  const size_t smem = (size_t)STAGES * (BM * BK * 2 + BN * BK * 2) + STAGES * 8 + 16;
  cudaError_t e = cudaFuncSetAttribute(dw_kernel<BN, CONV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid((g.Co + BM - 1) / BM, (g.K + BN - 1) / BN, splits);
  dw_kernel<BN, CONV><<<grid, 128, smem, st>>>(g);
  return cudaGetLastError();
}

static cudaError_t launch_dw(const DwArgs& g, bool conv, int splits, cudaStream_t st) {
  const int bn = g.K <= 32 ? 32 : g.K <= 64 ? 64 : g.K <= 128 ? 128 : 256;
#define NN_CASE(b)                                                                                          \
  if (bn == b) return conv ? launch_dw_t<b, true>(g, splits, st) : launch_dw_t<b, false>(g, splits, st);
  NN_CASE(32)
  NN_CASE(64)
  NN_CASE(128)
  NN_CASE(256)
#undef NN_CASE
  return cudaErrorInvalidValue;
}

template <int BN, int AMODE>
static cudaError_t launch_gemm_t(const GemmArgs& g, int splits, cudaStream_t st) {
  const size_t smem = (size_t)STAGES * (BM * BK * 2 + BN * BK * 2) + STAGES * 8 + 16;
  cudaError_t e = cudaFuncSetAttribute(gemm_kernel<BN, AMODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid((g.M + BM - 1) / BM, (g.N + BN - 1) / BN, splits);
  gemm_kernel<BN, AMODE><<<grid, 128, smem, st>>>(g);
  return cudaGetLastError();
}

static cudaError_t launch_gemm(const GemmArgs& g, int amode, int splits, cudaStream_t st) {
  const int bn = g.N <= 32 ? 32 : g.N <= 64 ? 64 : g.N <= 128 ? 128 : 256;
#define NN_CASE(b)                                                                         \
  if (bn == b) return amode == A_CONV3 ? launch_gemm_t<b, A_CONV3>(g, splits, st)         \
                                       : launch_gemm_t<b, A_DENSE>(g, splits, st);
  NN_CASE(32)
  NN_CASE(64)
  NN_CASE(128)
  NN_CASE(256)
#undef NN_CASE
  return cudaErrorInvalidValue;
}

// ------------------------------------------------------------------ helpers
// partials [splits][M][N] -> out[M][N] (fixed order)
__global__ void reduce_splits_kernel(const float* part, float* out, size_t n, int splits) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (4 * i + 3 < n && (n & 3) == 0) {
    // four outputs per thread, every split's load issued before the sums
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int z = 0; z < splits; ++z) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(part + (size_t)z * n) + i);
      s.x += v.x;
      s.y += v.y;
      s.z += v.z;
      s.w += v.w;
    }
    reinterpret_cast<float4*>(out)[i] = s;
    return;
  }
  if ((n & 3) == 0 || i >= n) return;
  float s = 0.f;
  for (int z = 0; z < splits; ++z) s += part[(size_t)z * n + i];
  out[i] = s;
}

// im2col of a 3x3 'same' patch, transposed: colT[k][m], k = tap * Ct + c
// (channels of X then X1), m = pixel; rows k >= 9 Ct (padding to Kpad) are zero
__global__ void im2col_t_kernel(const bf16* X, const bf16* X1, int C0, int C1, int Bn, int H, int W, int Kpad,
                                bf16* colT) {
  const size_t M = (size_t)Bn * H * W;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M * Kpad) return;
  const int k = (int)(i / M);
  const size_t m = i - (size_t)k * M;
  const int Ct = C0 + C1;
  bf16 v = __float2bfloat16(0.f);
  if (k < 9 * Ct) {
    const int tap = k / Ct, c = k - tap * Ct;
    const int hw = H * W;
    const int b = (int)(m / hw), rem = (int)(m - (size_t)b * hw), y = rem / W, x = rem % W;
    const int yy = y + tap / 3 - 1, xx = x + tap % 3 - 1;
    if (yy >= 0 && yy < H && xx >= 0 && xx < W) {
      const size_t pix = ((size_t)b * H + yy) * W + xx;
      v = c < C0 ? X[pix * C0 + c] : X1[pix * C1 + (c - C0)];
    }
  }
  colT[i] = v;
}

// im2col of a one-channel image into a dense [M][Kpad] matrix (the first layer)
__global__ void im2col1_kernel(const bf16* X, int Bn, int H, int W, int Kpad, bf16* col) {
  const size_t M = (size_t)Bn * H * W;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M * Kpad) return;
  const size_t m = i / Kpad;
  const int k = (int)(i - m * Kpad);
  bf16 v = __float2bfloat16(0.f);
  if (k < 9) {
    const int hw = H * W;
    const int b = (int)(m / hw), rem = (int)(m - (size_t)b * hw), y = rem / W, x = rem % W;
    const int yy = y + k / 3 - 1, xx = x + k % 3 - 1;
    if (yy >= 0 && yy < H && xx >= 0 && xx < W) v = X[((size_t)b * H + yy) * W + xx];
  }
  col[i] = v;
}

__global__ void transpose_kernel(const bf16* in, bf16* out, int R, int Cc) {
  __shared__ bf16 t[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = r0 + j, c = c0 + threadIdx.x;
    if (r < R && c < Cc) t[j][threadIdx.x] = in[(size_t)r * Cc + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int c = c0 + j, r = r0 + threadIdx.x;
    if (c < Cc && r < R) out[(size_t)c * R + r] = t[threadIdx.x][j];
  }
}

// W [Co][9][Ci] -> W' [Ci][9][Co] with the taps flipped: the weights of the
// backward-data convolution
__global__ void flip_weights_kernel(const bf16* w, bf16* wf, int Co, int Ci) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Co * 9 * Ci) return;
  const int co = i / (9 * Ci), rem = i - co * 9 * Ci, tap = rem / Ci, ci = rem - (rem / Ci) * Ci;
  wf[((size_t)ci * 9 + (8 - tap)) * Co + co] = w[i];
}

// dPre = dY * (Y > 0) (ReLU backward, Y the bf16 forward output), cast to bf16
__global__ void relu_bwd_kernel(const float* dy, const bf16* y, bf16* dpre, float* dpre_f32, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = __bfloat162float(y[i]) > 0.f ? dy[i] : 0.f;
  dpre[i] = __float2bfloat16(g);
  if (dpre_f32) dpre_f32[i] = g;
}

// db[n] = sum_m d[m][n] in two fixed-order passes: block b sums rows
// [b R, (b+1) R) column-wise with coalesced reads (consecutive threads read
// consecutive columns of a row; N divides 256), then one pass over the blocks.
constexpr int COLSUM_ROWS = 256;
__global__ void col_sum_part_kernel(const float* d, float* part, int M, int N) {
  __shared__ float red[256];
  const int rpp = 256 / N;  // rows per pass
  const int c = threadIdx.x % N, r0 = threadIdx.x / N;
  const int m0 = blockIdx.x * COLSUM_ROWS, m1 = min(M, m0 + COLSUM_ROWS);
  // four independent running sums keep four loads in flight per thread
  float s4[4] = {0.f, 0.f, 0.f, 0.f};
  int m = m0 + r0;
  for (; m + 3 * rpp < m1; m += 4 * rpp) {
#pragma unroll
    for (int u = 0; u < 4; ++u) s4[u] += d[(size_t)(m + u * rpp) * N + c];
  }
  for (int u = 0; m < m1; m += rpp, ++u) s4[u & 3] += d[(size_t)m * N + c];
  const float s = (s4[0] + s4[1]) + (s4[2] + s4[3]);
  red[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x < N) {
    float t = 0.f;
    for (int j = 0; j < rpp; ++j) t += red[j * N + threadIdx.x];
    part[(size_t)blockIdx.x * N + threadIdx.x] = t;
  }
}

// one block per column: strided partial sums, then a fixed tree (FP64)
__global__ void col_sum_final_kernel(const float* part, float* out, int nb, int N) {
  __shared__ double red[256];
  const int n = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) s += (double)part[(size_t)b * N + n];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = (float)red[0];
}

// 2x2 average pooling, NHWC
__global__ void pool2_kernel(const bf16* x, bf16* y, int Bn, int H, int W, int C) {
  const size_t n = (size_t)Bn * (H / 2) * (W / 2) * C;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = (int)(i % C);
  size_t p = i / C;
  const int xo = (int)(p % (W / 2));
  p /= (W / 2);
  const int yo = (int)(p % (H / 2));
  const int b = (int)(p / (H / 2));
  float s = 0.f;
  for (int dy = 0; dy < 2; ++dy)
    for (int dx = 0; dx < 2; ++dx) s += __bfloat162float(x[(((size_t)b * H + 2 * yo + dy) * W + 2 * xo + dx) * C + c]);
  y[i] = __float2bfloat16(0.25f * s);
}

__global__ void pool2_bwd_kernel(const float* dy, float* dx, int Bn, int H, int W, int C) {
  const size_t n = (size_t)Bn * H * W * C;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = (int)(i % C);
  size_t p = i / C;
  const int x = (int)(p % W);
  p /= W;
  const int y = (int)(p % H);
  const int b = (int)(p / H);
  dx[i] += 0.25f * dy[(((size_t)b * (H / 2) + y / 2) * (W / 2) + x / 2) * C + c];
}

// nearest 2x upsampling, NHWC (H, W: the input size)
__global__ void up2_kernel(const bf16* in, bf16* out, int Bn, int H, int W, int C) {
  const size_t n = (size_t)Bn * 2 * H * 2 * W * C;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = (int)(i % C);
  size_t p = i / C;
  const int x = (int)(p % (2 * W));
  p /= (2 * W);
  const int y = (int)(p % (2 * H));
  const int b = (int)(p / (2 * H));
  out[i] = in[(((size_t)b * H + y / 2) * W + x / 2) * C + c];
}

__global__ void up2_bwd_kernel(const float* dy, float* dx, int Bn, int H, int W, int C, int ldy, int coff) {
  // dy: [Bn, 2H, 2W, ldy] with this tensor's channels at [coff, coff + C)
  const size_t n = (size_t)Bn * H * W * C;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = (int)(i % C);
  size_t p = i / C;
  const int x = (int)(p % W);
  p /= W;
  const int y = (int)(p % H);
  const int b = (int)(p / H);
  float s = 0.f;
  for (int dyy = 0; dyy < 2; ++dyy)
    for (int dxx = 0; dxx < 2; ++dxx)
      s += dy[(((size_t)b * 2 * H + 2 * y + dyy) * 2 * W + 2 * x + dxx) * ldy + coff + c];
  dx[i] = s;
}

// dst[m][c] (+)= src[m][coff + c], c < C: a channel slice of a concatenation's gradient
__global__ void slice_add_kernel(const float* src, int ldsrc, int coff, float* dst, int C, size_t M, int accumulate) {
  const size_t n = M * C;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const size_t m = i / C;
  const int c = (int)(i - m * C);
  const float v = src[m * ldsrc + coff + c];
  dst[i] = accumulate ? dst[i] + v : v;
}

__global__ void cast_kernel(const float* x, bf16* y, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16(x[i]);
}

// Adam on FP32 master weights, BF16 copy for the tensor cores
__global__ void adam_kernel(float* p, const float* g, float* m, float* v, bf16* p16, size_t n, float lr, float b1,
                            float b2, float eps, float c1, float c2, float wd) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i] + wd * p[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  p[i] = pi;
  if (p16) p16[i] = __float2bfloat16(pi);
}

static unsigned blocks(size_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace nn
}  // namespace ptyg

using namespace ptyg::nn;

static int nn_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return PTYG_OK;
  char msg[256];
  snprintf(msg, sizeof msg, "%s: %s", what, cudaGetErrorString(e));
  return ptyg::set_last_error(PTYG_ERR_CUDA, msg);
}

extern "C" int ptyg_nn_gemm(const void* A, const void* B, int M, int N, int K, int splits, float* C, void* out,
                            const float* bias, int relu, int* status, void* stream) {
  if (!A || !B || M < 1 || N < 1 || K < 1 || (K % 8) || splits < 1 || (!C && !out))
    return ptyg::set_last_error(PTYG_ERR_INVALID, "ptyg_nn_gemm: bad arguments (K must be a multiple of 8)");
  if (((uintptr_t)A | (uintptr_t)B) % 16) return ptyg::set_last_error(PTYG_ERR_INVALID, "ptyg_nn_gemm: A, B not 16-byte aligned");
  GemmArgs g = {};
  g.A = (const bf16*)A;
  g.B = (const bf16*)B;
  g.M = M;
  g.N = N;
  g.K = K;
  const int kb = (K + BK - 1) / BK;
  if (splits > kb) splits = kb;
  g.kSplit = ((kb + splits - 1) / splits) * BK;
  splits = (K + g.kSplit - 1) / g.kSplit;
  g.epi = out ? EPI_BF16 : EPI_F32;
  if ((out || bias) && splits > 1)
    return ptyg::set_last_error(PTYG_ERR_INVALID, "ptyg_nn_gemm: bf16 output and bias need splits = 1");
  g.C = C;
  g.out = (bf16*)out;
  g.bias = bias;
  g.relu = relu;
  g.status = status;
  ptyg::nn::wait_policy(&g.waitLimit, &g.stall);
  return nn_check(launch_gemm(g, A_DENSE, splits, (cudaStream_t)stream), "ptyg_nn_gemm");
}

static int g_conv_tma = 1;  // ptyg_nn_conv3_path

extern "C" int ptyg_nn_conv3_path(int tma) {
  g_conv_tma = tma != 0;
  return PTYG_OK;
}

extern "C" int ptyg_nn_conv3(const void* X, const void* X1, int C0, int C1, int Bn, int H, int W, const void* Wt,
                             int Co, float* C, void* out, const float* bias, int relu, int* status, void* stream) {
  if (!X || !Wt || C0 < 8 || (C0 % 8) || (C1 % 8) || (C1 && !X1) || Bn < 1 || H < 1 || W < 1 || Co < 1 ||
      (!C && !out))
    return ptyg::set_last_error(PTYG_ERR_INVALID, "ptyg_nn_conv3: bad arguments (channels: multiples of 8)");
  if (g_conv_tma) {
    const cudaError_t e = ptyg::nn::conv3_tma(X, C1 ? X1 : nullptr, C0, C1, Bn, H, W, Wt, Co, C, out, bias, relu,
                                              status, (cudaStream_t)stream);
    if (e != cudaErrorNotSupported) return nn_check(e, "ptyg_nn_conv3 (TMA)");
    cudaGetLastError();
  }
  GemmArgs g = {};
  g.A = (const bf16*)X;
  g.A1 = (const bf16*)X1;
  g.C0 = C0;
  g.C1 = C1;
  g.H = H;
  g.W = W;
  g.B = (const bf16*)Wt;
  g.M = Bn * H * W;
  g.N = Co;
  g.K = 9 * (C0 + C1);
  g.kSplit = ((g.K + BK - 1) / BK) * BK;
  g.epi = out ? EPI_BF16 : EPI_F32;
  g.C = C;
  g.out = (bf16*)out;
  g.bias = bias;
  g.relu = relu;
  g.status = status;
  ptyg::nn::wait_policy(&g.waitLimit, &g.stall);
  return nn_check(launch_gemm(g, A_CONV3, 1, (cudaStream_t)stream), "ptyg_nn_conv3");
}

extern "C" int ptyg_nn_reduce_splits(const float* part, float* out, int64_t n, int splits, void* stream) {
  reduce_splits_kernel<<<blocks(n % 4 == 0 ? n / 4 : n), 256, 0, (cudaStream_t)stream>>>(part, out, (size_t)n, splits);
  return nn_check(cudaGetLastError(), "ptyg_nn_reduce_splits");
}

extern "C" int ptyg_nn_im2col_t(const void* X, const void* X1, int C0, int C1, int Bn, int H, int W, int Kpad,
                                void* colT, void* stream) {
  const size_t n = (size_t)Bn * H * W * Kpad;
  im2col_t_kernel<<<blocks(n), 256, 0, (cudaStream_t)stream>>>((const bf16*)X, (const bf16*)X1, C0, C1, Bn, H, W,
                                                               Kpad, (bf16*)colT);
  return nn_check(cudaGetLastError(), "ptyg_nn_im2col_t");
}

extern "C" int ptyg_nn_im2col1(const void* X, int Bn, int H, int W, int Kpad, void* col, void* stream) {
  const size_t n = (size_t)Bn * H * W * Kpad;
  im2col1_kernel<<<blocks(n), 256, 0, (cudaStream_t)stream>>>((const bf16*)X, Bn, H, W, Kpad, (bf16*)col);
  return nn_check(cudaGetLastError(), "ptyg_nn_im2col1");
}

extern "C" int ptyg_nn_transpose(const void* in, void* out, int R, int Cc, void* stream) {
  dim3 grid((Cc + 31) / 32, (R + 31) / 32), block(32, 8);
  transpose_kernel<<<grid, block, 0, (cudaStream_t)stream>>>((const bf16*)in, (bf16*)out, R, Cc);
  return nn_check(cudaGetLastError(), "ptyg_nn_transpose");
}

extern "C" int ptyg_nn_flip_weights(const void* w, void* wf, int Co, int Ci, void* stream) {
  flip_weights_kernel<<<blocks((size_t)Co * 9 * Ci), 256, 0, (cudaStream_t)stream>>>((const bf16*)w, (bf16*)wf, Co, Ci);
  return nn_check(cudaGetLastError(), "ptyg_nn_flip_weights");
}

extern "C" int ptyg_nn_relu_bwd(const float* dy, const void* y, void* dpre, float* dpre_f32, int64_t n, void* stream) {
  relu_bwd_kernel<<<blocks(n), 256, 0, (cudaStream_t)stream>>>(dy, (const bf16*)y, (bf16*)dpre, dpre_f32, (size_t)n);
  return nn_check(cudaGetLastError(), "ptyg_nn_relu_bwd");
}

extern "C" int ptyg_nn_col_sum(const float* d, float* part, float* out, int M, int N, void* stream) {
  if (!d || !part || !out || N < 1 || N > 256 || (256 % N))
    return ptyg::set_last_error(PTYG_ERR_INVALID, "ptyg_nn_col_sum: N must divide 256");
  cudaStream_t st = (cudaStream_t)stream;
  const int nb = (M + COLSUM_ROWS - 1) / COLSUM_ROWS;
  col_sum_part_kernel<<<nb, 256, 0, st>>>(d, part, M, N);
  col_sum_final_kernel<<<N, 256, 0, st>>>(part, out, nb, N);
  return nn_check(cudaGetLastError(), "ptyg_nn_col_sum");
}

extern "C" int ptyg_nn_pool2(const void* x, void* y, int Bn, int H, int W, int C, void* stream) {
  pool2_kernel<<<blocks((size_t)Bn * H * W * C / 4), 256, 0, (cudaStream_t)stream>>>((const bf16*)x, (bf16*)y, Bn, H,
                                                                                     W, C);
  return nn_check(cudaGetLastError(), "ptyg_nn_pool2");
}

extern "C" int ptyg_nn_pool2_bwd(const float* dy, float* dx, int Bn, int H, int W, int C, void* stream) {
  pool2_bwd_kernel<<<blocks((size_t)Bn * H * W * C), 256, 0, (cudaStream_t)stream>>>(dy, dx, Bn, H, W, C);
  return nn_check(cudaGetLastError(), "ptyg_nn_pool2_bwd");
}

extern "C" int ptyg_nn_up2(const void* x, void* y, int Bn, int H, int W, int C, void* stream) {
  up2_kernel<<<blocks((size_t)Bn * H * W * C * 4), 256, 0, (cudaStream_t)stream>>>((const bf16*)x, (bf16*)y, Bn, H, W,
                                                                                   C);
  return nn_check(cudaGetLastError(), "ptyg_nn_up2");
}

extern "C" int ptyg_nn_up2_bwd(const float* dy, float* dx, int Bn, int H, int W, int C, int ldy, int coff,
                               void* stream) {
  up2_bwd_kernel<<<blocks((size_t)Bn * H * W * C), 256, 0, (cudaStream_t)stream>>>(dy, dx, Bn, H, W, C, ldy, coff);
  return nn_check(cudaGetLastError(), "ptyg_nn_up2_bwd");
}

extern "C" int ptyg_nn_slice_add(const float* src, int ldsrc, int coff, float* dst, int C, int64_t M, int accumulate,
                                 void* stream) {
  slice_add_kernel<<<blocks((size_t)M * C), 256, 0, (cudaStream_t)stream>>>(src, ldsrc, coff, dst, C, (size_t)M,
                                                                            accumulate);
  return nn_check(cudaGetLastError(), "ptyg_nn_slice_add");
}

extern "C" int ptyg_nn_cast_bf16(const float* x, void* y, int64_t n, void* stream) {
  cast_kernel<<<blocks(n), 256, 0, (cudaStream_t)stream>>>(x, (bf16*)y, (size_t)n);
  return nn_check(cudaGetLastError(), "ptyg_nn_cast_bf16");
}

extern "C" int ptyg_nn_adam(float* p, const float* g, float* m, float* v, void* p16, int64_t n, float lr, float b1,
                            float b2, float eps, int step, float weight_decay, void* stream) {
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  adam_kernel<<<blocks(n), 256, 0, (cudaStream_t)stream>>>(p, g, m, v, (bf16*)p16, (size_t)n, lr, b1, b2, eps, c1, c2,
                                                           weight_decay);
  return nn_check(cudaGetLastError(), "ptyg_nn_adam");
}

// Phase-aligned windowed stitching of n complex patches (Np x Np) into an
// No x No object, in order: each patch is rotated by the unit phase of its
// windowed overlap with what is stitched so far, then added with the window.
// Patch j depends on patches < j, so one CTA walks them: a block reduction
// (FP64) for the overlap, then the windowed update of the patch's rows.
__global__ void __launch_bounds__(1024) stitch_kernel(const float2* __restrict__ patches, const int* __restrict__ pos,
                                                      int n, int Np, int No, const float* __restrict__ w, float2* acc,
                                                      float* wsum) {
  __shared__ double red[2][32];
  __shared__ float2 rot_s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int NN = Np * Np;
  for (int j = 0; j < n; ++j) {
    const int r = pos[2 * j], c = pos[2 * j + 1];
    if (r < 0 || c < 0 || r > No - Np || c > No - Np) continue;  // uniform over the block
    const float2* p = patches + (size_t)j * NN;
    double ox = 0.0, oy = 0.0;
    for (int i = tid; i < NN; i += blockDim.x) {
      const int y = i / Np, x = i - (i / Np) * Np;
      const float2 pv = p[i], a = acc[(size_t)(r + y) * No + c + x];
      const double wv = w[i];
      ox += wv * ((double)pv.x * a.x + (double)pv.y * a.y);  // conj(p) a w
      oy += wv * ((double)pv.x * a.y - (double)pv.y * a.x);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ox += __shfl_xor_sync(0xffffffffu, ox, o);
      oy += __shfl_xor_sync(0xffffffffu, oy, o);
    }
    if (lane == 0) {
      red[0][warp] = ox;
      red[1][warp] = oy;
    }
    __syncthreads();
    if (tid == 0) {
      double sx = 0.0, sy = 0.0;
      for (int k = 0; k < nw; ++k) {
        sx += red[0][k];
        sy += red[1][k];
      }
      const double mag = sqrt(sx * sx + sy * sy);
      rot_s = mag > 0.0 ? make_float2((float)(sx / mag), (float)(sy / mag)) : make_float2(1.f, 0.f);
    }
    __syncthreads();
    const float2 rot = rot_s;
    for (int i = tid; i < NN; i += blockDim.x) {
      const int y = i / Np, x = i - (i / Np) * Np;
      const size_t oi = (size_t)(r + y) * No + c + x;
      const float2 pv = p[i];
      const float wv = w[i];
      const float2 q = make_float2(rot.x * pv.x - rot.y * pv.y, rot.x * pv.y + rot.y * pv.x);
      acc[oi] = make_float2(acc[oi].x + q.x * wv, acc[oi].y + q.y * wv);
      wsum[oi] += wv;
    }
    __syncthreads();  // this patch's writes before the next patch's overlap
  }
}

extern "C" int ptyg_stitch(const void* patches, const int32_t* positions, int n, int Np, int No, const float* window,
                           void* acc, float* wsum, void* stream) {
  if (!patches || !positions || !window || !acc || !wsum || n < 0 || Np < 1 || No < Np)
    return ptyg::set_last_error(PTYG_ERR_INVALID, "ptyg_stitch: bad arguments");
  if (n == 0) return PTYG_OK;
  stitch_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>((const float2*)patches, positions, n, Np, No, window,
                                                      (float2*)acc, wsum);
  return nn_check(cudaGetLastError(), "ptyg_stitch");
}

static int ilog2_exact(int v) {
  int l = 0;
  while ((1 << l) < v) ++l;
  return (1 << l) == v ? l : -1;
}

extern "C" int ptyg_nn_conv3_wgrad(const void* dY, int Co, const void* X, const void* X1, int C0, int C1, int Bn, int H,
                                   int W, int splits, float* C, void* status, void* stream) {
  const int lgW = ilog2_exact(W), lgHW = ilog2_exact(H * W);
  if (!dY || !X || !C || Co < 8 || (Co % 8) || C0 < 8 || (C0 % 8) || (C1 % 8) || (C1 && !X1) || Bn < 1 || lgW < 0 ||
      lgHW < 0 || splits < 1)
    return ptyg::set_last_error(PTYG_ERR_INVALID,
                                "ptyg_nn_conv3_wgrad: bad arguments (channels multiples of 8, H and W powers of two)");
  DwArgs g = {};
  g.dY = (const bf16*)dY;
  g.Co = Co;
  g.X = (const bf16*)X;
  g.X1 = (const bf16*)X1;
  g.C0 = C0;
  g.C1 = C1;
  g.lgW = lgW;
  g.lgHW = lgHW;
  g.H = H;
  g.W = W;
  g.K = 9 * (C0 + C1);
  g.P = Bn * H * W;
  const int pb = (g.P + BK - 1) / BK;
  if (splits > pb) splits = pb;
  g.pSplit = ((pb + splits - 1) / splits) * BK;
  splits = (g.P + g.pSplit - 1) / g.pSplit;
  g.C = C;
  g.status = (int*)status;
  ptyg::nn::wait_policy(&g.waitLimit, &g.stall);
  return nn_check(launch_dw(g, true, splits, (cudaStream_t)stream), "ptyg_nn_conv3_wgrad");
}

extern "C" int ptyg_nn_dense_wgrad(const void* dY, int Co, const void* X, int K, int P, int splits, float* C,
                                   void* status, void* stream) {
  if (!dY || !X || !C || Co < 8 || (Co % 8) || K < 8 || (K % 8) || P < 1 || splits < 1)
    return ptyg::set_last_error(PTYG_ERR_INVALID, "ptyg_nn_dense_wgrad: bad arguments (Co, K multiples of 8)");
  DwArgs g = {};
  g.dY = (const bf16*)dY;
  g.Co = Co;
  g.X = (const bf16*)X;
  g.K = K;
  g.P = P;
  const int pb = (P + BK - 1) / BK;
  if (splits > pb) splits = pb;
  g.pSplit = ((pb + splits - 1) / splits) * BK;
  splits = (P + g.pSplit - 1) / g.pSplit;
  g.C = C;
  g.status = (int*)status;
  ptyg::nn::wait_policy(&g.waitLimit, &g.stall);
  return nn_check(launch_dw(g, false, splits, (cudaStream_t)stream), "ptyg_nn_dense_wgrad");
}

extern "C" int ptyg_nn_set_wait_policy(long long polls, int stall_launches) {
  if (polls < 1 || stall_launches < 0)
    return ptyg::set_last_error(PTYG_ERR_INVALID, "ptyg_nn_set_wait_policy: polls >= 1, stall_launches >= 0");
  ptyg::nn::g_wait_limit.store(polls);
  ptyg::nn::g_stall_launches.store(stall_launches);
  return PTYG_OK;
}
