// Device helpers shared by the position-loop kernels (ptyg_engine.cu,
// ptyg_e3pie.cu): cluster barrier and distributed shared memory, cp.async,
// warp/CTA reductions into cluster slots, the DSMEM row/column transposes
// and the transfer-function column pass.
#pragma once

#include <cooperative_groups.h>

#include "ptyg_common.cuh"
#include "ptyg_engine.cuh"

namespace cg = cooperative_groups;

namespace ptyg {

// Address of `local` in the shared memory of cluster rank `rank`.
template <class T>
PTYG_DEV T* dsmem(T* local, int rank) {
  return cg::this_cluster().map_shared_rank(local, (unsigned)rank);
}

PTYG_DEV void cp_async16(void* smem_dst, const void* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc) : "memory");
}
PTYG_DEV void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
PTYG_DEV void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
PTYG_DEV void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// The two halves of cluster_sync, for work that may overlap the barrier:
// arrive (release: this CTA's earlier writes, local and remote, become
// visible to the cluster), then wait (acquire) before reading what the other
// CTAs wrote.  For C == 1 the wait is a CTA barrier.
PTYG_DEV void cluster_arrive(int C) {
  if (C > 1) asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
}
PTYG_DEV void cluster_wait(int C) {
  if (C > 1)
    asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
  else
    __syncthreads();
}

PTYG_DEV void cluster_sync(int C) {
  if (C > 1) {
    asm volatile(
        "barrier.cluster.arrive.release.aligned;\n\t"
        "barrier.cluster.wait.acquire.aligned;\n" ::
            : "memory");
  } else {
    __syncthreads();
  }
}

PTYG_DEV float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

PTYG_DEV double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over the warp as the balanced binary tree over lane order (pairs of
// neighbouring lanes first); every lane receives the same bits.
PTYG_DEV double warp_tree_sum(double v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
PTYG_DEV float warp_tree_sumf(float v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) v = __fadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Sum of v[0, n), n a power of two of at most 128, as the balanced binary tree
// over index order, on every lane.  The tree is fixed by n alone, so n values
// split across CTAs in power-of-two blocks and summed block by block, then
// over the blocks in the same tree, round exactly as one sum over all values.
PTYG_DEV double tree_sum(const double* v, int n, unsigned lane) {
  double s;
  if (n <= 32)
    s = (int)lane < n ? v[lane] : 0.0;  // the zero leaves add exactly
  else if (n == 64)
    s = v[2 * lane] + v[2 * lane + 1];
  else
    s = (v[4 * lane] + v[4 * lane + 1]) + (v[4 * lane + 2] + v[4 * lane + 3]);
  return warp_tree_sum(s);
}

// Max-reduce NV values over the CTA and fold them into the cluster slots (rank
// 0's shared memory) with one cluster-scope atomicMax per value per CTA
// (non-negative floats order like their bits).
template <int NV>
PTYG_DEV void block_max_to_slots(float (&v)[NV], float* scratch, unsigned* slots, const int* idx) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const float m = warp_max(v[i]);
    if (lane == 0) scratch[i * 32 + warp] = m;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    float m = 0.f;
    for (int w = 0; w < nw; ++w) m = fmaxf(m, scratch[threadIdx.x * 32 + w]);
    atomicMax(slots + idx[threadIdx.x], __float_as_uint(m));
  }
}

// Sum NV values over the CTA (scratch: NV * 32 doubles); thread 0 receives
// the results in v.  Fixed order, so every run gives the same bits.
template <int NV>
PTYG_DEV void block_sum_n(double (&v)[NV], double* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const double w = warp_sum(v[i]);
    if (lane == 0) scratch[i * 32 + warp] = w;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      double t = 0.0;
      for (int w = 0; w < nw; ++w) t += scratch[i * 32 + w];
      v[i] = t;
    }
  }
}

// Sum NV values over the whole cluster: CTA totals go to rank 0's `part`
// ([value][CTA], NV * C doubles), one cluster barrier, then every thread of
// every CTA adds the C totals in the same order (an xor butterfly over C
// lanes), so all CTAs hold bitwise the same sums.  scratch: NV * 32 doubles.
template <int NV, int C>
PTYG_DEV void cluster_sum_n(double (&v)[NV], double* part, double* scratch, int crank) {
  __syncthreads();  // scratch may still be read by an earlier block reduction
  block_sum_n<NV>(v, scratch);
  if (threadIdx.x == 0) {
    double* dst = dsmem(part, 0);
#pragma unroll
    for (int k = 0; k < NV; ++k) dst[k * C + crank] = v[k];
  }
  cluster_sync(C);
  const int lane = threadIdx.x & 31;
  const double* src = dsmem(part, 0);
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double t = lane < C ? src[k * C + lane] : 0.0;
#pragma unroll
    for (int off = 1; off < C; off <<= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    v[k] = __shfl_sync(0xffffffffu, t, 0);
  }
}

// Sum over the CTA; thread 0 receives the result.
PTYG_DEV double block_sum(double v, double* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < nw; ++w) t += scratch[w];
  return t;
}

PTYG_DEV float slot_value(const unsigned* slots, int i) {
  return __uint_as_float(*reinterpret_cast<const volatile unsigned*>(slots + i));
}

// Column block (tile) layout: row (k * NP + y) holds the CTA's L columns,
// unpadded, column c stored at c ^ swz(row).  The swizzle spreads the 16
// consecutive rows of a 64-bit half-warp access (a column task: lanes step
// through y) over 16 distinct bank pairs: swz = row & 15 for L >= 16 and
// (row >> 1) & 7 for L = 8 (where a row pair shares one 16-element span).
// A row write (lanes step through c) stays one permuted contiguous span.
template <int L>
PTYG_DEV int tix_swz(int row) {
  static_assert(L == 8 || L == 16 || L == 32 || L == 64, "tile swizzle defined for 8 to 64 columns");
  return L == 8 ? (row >> 1) & 7 : row & 15;
}
template <int L>
PTYG_DEV int tix(int row, int c) {
  return row * L + (c ^ tix_swz<L>(row));
}

// Store into the shared memory of cluster rank `rank` at the address `local`
// has in this CTA (mapa on the 32-bit shared-window address).
PTYG_DEV void st_cluster(const float2* local, int rank, float2 v) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(local);
  unsigned r;
  asm("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(a), "r"(rank));
  asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};\n" ::"r"(r), "f"(v.x), "f"(v.y));
}
PTYG_DEV void st_cluster4(const float4* local, int rank, float4 v) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(local);
  unsigned r;
  asm("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(a), "r"(rank));
  asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};\n" ::"r"(r), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w));
}

// Element lo + hi (a Fourier slot; lo the thread's part, hi a compile-time
// offset) of the transformed row y of mode k goes to the column block of the
// CTA owning that slot.
template <int NP, int L>
PTYG_DEV void scatter_row(float2* tile, int k, int y, int lo, int hi, float2 v) {
  const unsigned s = (unsigned)(lo + hi);
  st_cluster(&tile[tix<L>(k * NP + y, (int)(s % L))], (int)(s / L), v);
}

// Row buffers (K * L rows of NP, Fourier layout along x) are written by the
// column owners and read along rows, so the slot is swizzled by the row: row
// task t = k * L + l keeps slot s at t * NP + (s ^ (l mod 16)) (rsw).  The XOR
// touches bits 0..3 only, so it permutes slots within aligned groups of 16
// (a column block of L >= 16 stays one contiguous span of every row) and
// commutes with adding a multiple of 16: rsw(t, lo + hi) = rsw(t, lo) + hi.
template <int L>
PTYG_DEV int rsw(int t, int s) {
  return s ^ (t & ((L < 16 ? L : 16) - 1));
}

// A column task stores its result (natural order along y) in its own column of
// the CTA's tile, row k * NP + y; once every column task of the CTA is done
// (a CTA barrier), flush_columns sends the tile to the row owners' row
// buffers.  Each thread moves two neighbouring columns of one row (16 bytes),
// and the L / 2 threads of a row write its whole column block, L * 8
// contiguous bytes of the owner's buffer: one remote line per row instead of
// one 8-byte remote store per column and row.
template <int NP, int L>
PTYG_DEV void flush_columns(const float2* tile, float2* rows, int K, int sx0) {
  constexpr int PAIRS = L / 2;
  const int n = K * NP * PAIRS;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int r = i / PAIRS, c = 2 * (i - (i / PAIRS) * PAIRS);  // tile row k * NP + y, even column c
    const int k = r / NP, y = r - (r / NP) * NP;
    const int sw = tix_swz<L>(r);
    // columns c, c + 1 sit at (c ^ sw) and (c ^ sw) ^ 1: one aligned pair, swapped when sw is odd
    const float4 f = *reinterpret_cast<const float4*>(tile + r * L + ((c ^ sw) & ~1));
    const int owner = y / L, ly = y - (y / L) * L;
    // in the owner's row, slots sx0 + c and sx0 + c + 1 sit at rsw(sx0 + c) and that ^ 1
    const int t = k * L + ly;
    const int pos = t * NP + (rsw<L>(t, sx0 + c) & ~1);
    const float4 o = ((sw ^ t) & 1) ? make_float4(f.z, f.w, f.x, f.y) : f;
    st_cluster4(reinterpret_cast<const float4*>(rows + pos), owner, o);
  }
}

// The column task's store into its own tile column (natural order along y).
template <int E, int L>
PTYG_DEV void store_column(float2* tile, const float2 (&v)[E], int k, int c) {
  constexpr int NP = 32 * E;
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < E; ++j) tile[tix<L>(k * NP + lane + 32 * j, c)] = v[j];
}

// Copy nblk blocks of `bytes` bytes (block b from src + b * srcStride, 16-byte
// aligned, bytes a multiple of 16) to consecutive shared memory at dst with
// the bulk-copy engine (cp.async.bulk, completion on the mbarrier `bar`), and
// wait in every thread of the CTA, polling at most BULK_WAIT_POLLS times.
// Returns false when the wait gave up (the caller raises its status word).
constexpr long long BULK_WAIT_POLLS = 1ll << 22;
PTYG_DEV bool bulk_copy_wait(float2* dst, const float2* src, unsigned bytes, int nblk, size_t srcStride,
                             unsigned long long* bar) {
  const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
  const unsigned d0 = (unsigned)__cvta_generic_to_shared(dst);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(b) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(b), "r"(bytes * (unsigned)nblk)
                 : "memory");
    for (int k = 0; k < nblk; ++k)
      asm volatile(
          "{\n.reg .u64 g;\ncvta.to.global.u64 g, %1;\n"
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [g], %2, [%3];\n}\n" ::"r"(
              d0 + (unsigned)k * bytes),
          "l"(src + (size_t)k * srcStride), "r"(bytes), "r"(b)
          : "memory");
  }
  __syncthreads();  // the barrier is initialised before anyone polls it
  unsigned done = 0;
  for (long long i = 0; i < BULK_WAIT_POLLS && !done; ++i)
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(b)
        : "memory");
  return done != 0;
}

// Column pass that multiplies the spectrum by H (or conj H) / Np^2 between a
// forward and an inverse column transform (ASP, Operators.py:155-230); the
// result goes to the row owners' row buffers (visible after a cluster barrier).
// Column task t = k * L + c is transformed in place in the tile.  H: the
// table in global memory (Fourier layout [sx][sy], tables Hset apart), or
// with hsm the CTA's own columns of it in shared memory (column c at c * NP).
template <int E, int L, bool SETS = false>
PTYG_DEV void column_filter(float2* tile, float2* rows, const WarpFFT<E>& F, const float2* H, size_t Hset, bool hsm,
                            bool conjH, int crank, int K, int kPerSet) {
  constexpr int NP = 32 * E;
  const int sx0 = crank * L;
  const float inv2 = 1.f / (float)(NP * NP);
  auto col = [&](int t, int i) -> float2& { return tile[tix<L>((t / L) * NP + i, t % L)]; };
  fft_tasks<E, false>(
      F, K * L, [&](int t, int lo, int hi) { return col(t, lo + hi); },
      [&](int t, int lo, int hi, float2 v) {
        const int k = t / L, c = t % L;
        // SETS: one table per wavelength, modes k of wavelength k / kPerSet
        const float2* h = H + (SETS ? (size_t)(k / kPerSet) * Hset : 0) + (size_t)((hsm ? 0 : sx0) + c) * NP;
        float2 hv = hsm ? h[lo + hi] : __ldg(h + lo + hi);
        if (conjH) hv.y = -hv.y;
        col(t, lo + hi) = cscale(cmul(v, hv), inv2);
      });
  __syncthreads();
  fft_tasks<E, true>(
      F, K * L, [&](int t, int lo, int hi) { return col(t, lo + hi); },
      [&](int t, int lo, int hi, float2 v) { col(t, lo + hi) = v; });
  __syncthreads();
  flush_columns<NP, L>(tile, rows, K, sx0);
}

// The intensity projection of a CTA's LN = L * NP detector pixels
// (BaseEngine.py:881-1009): getRMSD on the estimate (plus the background),
// adaptive denoising (:1805-1822, a frame mean: one cluster sum), the
// standard / poission / exponential / fluctuation constraint (fluctuation:
// two more frame sums), the intensity mask, the background update.  Iest(i)
// is the estimate of pixel i; the factor goes to io.fr[i] times outScale.
// Tables and the background are in the data layout, this CTA's block at
// blk0 * NP.  Returns this thread's (FourierMask-weighted) error sum.
// COLS: warp w handles the NP / 32 pixels of its own column w (pixel
// w * NP + 32 r + lane gets Iest(r)), else every thread strides over the
// CTA's LN pixels (pixel i gets Iest(i)); the column form serves only
// single-pass projections.  FAST: the standard projection without
// background, masks or denoising, folded at compile time.  INTERF: the
// interferometric constraint compiled in (the raw factor goes to fr, applied
// with the reference field after the projection: no intensity mask there,
// BaseEngine.py:975-982).
struct ProjectionIO {
  float* fr;         // L * NP factors (between the passes of a two-pass projection: the estimates)
  const float* dat;  // L * NP measured intensities
  double* part;      // cluster-sum partials, rank 0's read by all (64 doubles)
  double* redD;      // CTA scratch (64 doubles)
};
template <int NP, int L, bool FAST, bool INTERF, bool COLS, class IestF>
PTYG_DEV double project_intensities(const EngineArgs& a, const ScanDev& s, int frame, int blk0, int crank,
                                    const ProjectionIO& io, IestF&& Iest, float outScale) {
  constexpr int C = NP / L, LN = L * NP, E = NP / 32;
  const unsigned lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const bool interf = INTERF && a.iconstraint == IC_INTERFEROMETRIC;
  const int icon = FAST ? (int)IC_STANDARD : a.iconstraint;
  const bool denoise = !FAST && a.denoise;
  float* fr = io.fr;
  const float* dat = io.dat;
  const bool det = a.writeDetErr && s.detErr;
  const size_t tb = (size_t)blk0 * NP;
  float* bg = (!FAST && a.bgMode) ? s.background + tb : nullptr;
  const float* Wt = (!FAST && a.fmask) ? a.W + tb : nullptr;
  const float* Mt = (!FAST && a.imask) ? a.imaskTab + tb : nullptr;
  float e = 0.f, noise = 0.f, aleph = 0.f;
  auto denoised = [&](float im) {
    if (!denoise) return im;
    const float am = fmaxf(sqrtf(im) - noise, 0.f);
    return am * am;
  };
  auto finish = [&](int i, float ie, float im, float d) {
    const float q = denoised(im) / (ie + 1e-10f);
    float frac;
    if (icon == IC_POISSON) {
      frac = q;
    } else if (icon == IC_EXPONENTIAL) {
      const float w = expf(-0.05f * (d / (ie + 1e-10f)));
      frac = w * sqrtf(q) + (1.f - w);
    } else if (icon == IC_FLUCTUATION) {
      frac = (1.f + aleph) * 0.5f * q;
    } else {  // standard and interferometric (BaseEngine.py:955-962)
      frac = sqrtf(q);
    }
    fr[i] = interf ? frac : (Mt ? frac * Mt[i] + (Mt[i] - 1.f) : frac) * outScale;
    if (bg) {
      const float u = 1.f + a.invFrames * (sqrtf(frac) - 1.f);
      float b = bg[i] * (u * u);
      if (Wt) b *= Wt[i];
      bg[i] = b;
    }
  };
  const bool twoPass = !COLS && (denoise || icon == IC_FLUCTUATION);
  double dn = 0.0;
  auto pixel = [&](int i, float ie) {
    if (bg) ie += bg[i];
    const float im = dat[i];
    const float d = fabsf(im - ie);
    e += Wt ? d * Wt[i] : d;
    if (det) s.detErr[((size_t)frame * NP + blk0) * NP + i] = d;
    if (twoPass) {
      fr[i] = ie;  // kept for the second pass (same thread)
      if (denoise) dn += (double)(sqrtf(im) - sqrtf(fabsf(ie)));
    } else {
      finish(i, ie, im, d);
    }
  };
  if constexpr (COLS) {
#pragma unroll
    for (int r = 0; r < E; ++r) pixel(warp * NP + 32 * r + (int)lane, Iest(r));
  } else {
    for (int i = threadIdx.x; i < LN; i += blockDim.x) pixel(i, Iest(i));
  }
  if (twoPass) {
    if (denoise) {
      double v[1] = {dn};
      cluster_sum_n<1, C>(v, io.part, io.redD, crank);
      noise = fabsf((float)(v[0] / (double)(NP * NP)));
    }
    if (icon == IC_FLUCTUATION) {
      double v[2] = {0.0, 0.0};
      for (int i = threadIdx.x; i < LN; i += blockDim.x) {
        const float ie = fr[i], imd = denoised(dat[i]), w = Wt ? Wt[i] : 1.f;
        v[0] += (double)(imd * ie * w);
        v[1] += (double)(imd * imd * w);
      }
      cluster_sum_n<2, C>(v, io.part + 32, io.redD, crank);
      aleph = (float)(v[0] / v[1]);
      if (crank == 0 && threadIdx.x == 0 && s.iscale) s.iscale[frame] = (double)aleph;
    }
    for (int i = threadIdx.x; i < LN; i += blockDim.x) {
      const float ie = fr[i], im = dat[i];
      finish(i, ie, im, fabsf(im - ie));
    }
  }
  return (double)e;
}

// Prefetch the measured intensities of order slot `it` (if it exists and is a
// valid frame) into dat[it & 1]: the CTA's L*NP block is contiguous in both
// layouts (Fourier [frame][sx][sy] columns sx0.., or natural rows line0..).
// DOUBLE: dat[it & 1] of a double buffer, else the one buffer.
template <int NP, int L, bool DOUBLE = true>
PTYG_DEV void prefetch_data(const EngineArgs& a, const ScanDev& s, float* datBuf, int it, int blk0) {
  if (it < a.count) {
    const int frame = s.order[a.start + it];
    if (frame >= 0 && frame < a.numFrames) {
      const float* src = s.data + ((size_t)frame * NP + blk0) * NP;
      float* dst = datBuf + (DOUBLE ? (it & 1) * L * NP : 0);
      for (int i = threadIdx.x; i < L * NP / 4; i += blockDim.x) cp_async16(dst + 4 * i, src + 4 * i);
    }
  }
  cp_async_commit();
}

}  // namespace ptyg
