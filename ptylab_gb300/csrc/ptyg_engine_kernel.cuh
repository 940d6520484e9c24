// Persistent position-loop kernel for ePIE / mPIE / qNewton / mqNewton (CPM and
// FPM) with the Fraunhofer, Fresnel and ASP propagators.
//
// One thread-block cluster of C CTAs reconstructs one scan; a grid of G
// clusters reconstructs G independent scans.  The cluster walks the positions
// of one iteration in the order the host drew (PtyLab/Engines/BaseEngine.py:637-665)
// and, for each position, runs the body of ePIE.py:84-105 / mPIE.py:119-172 /
// qNewton.py:69-90 / mqNewton.py:95-126 as passes separated by cluster barriers.  CTA c owns rows
// [c*L, (c+1)*L) of every row pass and Fourier-layout columns [c*L, (c+1)*L)
// of every column pass (L = Np/C), so it always updates the same probe rows
// and keeps them in shared memory for the whole launch.
//
// Data moves between the passes through distributed shared memory: a row
// pass writes each transformed row straight into the shared-memory column
// block of the CTA that owns those columns, and a column pass writes back into
// the row owners' row buffers, so the 2D transpose never touches L2.  The
// norm maxima are reduced with cluster-scope atomics into rank 0's shared
// memory, and each position's measured intensities are prefetched with
// cp.async into their buffer as soon as the previous position's projection
// has read it.
//
// Work is split into warp tasks, one 1D transform of one mode each, so a CTA
// runs K*L independent transforms per pass (K = nosm*npsm); everything that
// couples modes (the estimated intensity, the object step's sum over probe
// modes, the probe step's sum over object modes) is done afterwards by a
// pixel loop over shared memory in a fixed order, so results are deterministic.
//
//   A  stage the object patch rows; maxima of the update norms; tasks: exit
//      wave O_o*P_p [*chirp][*sign], forward row FFT -> work buffer
//   B  stage the CTA's column block; tasks: forward column FFT; pixels:
//      I_est, FP64 error partial, frac = sqrt(I_meas/(I_est+1e-10)); tasks:
//      * frac / Np^2, inverse column FFT; write back.  With one warp per
//      column of the CTA (and a single-pass projection) the warp does all of
//      this for its column, the intensities summed in registers
//   C  tasks: inverse row FFT, [sign], [conj chirp], DELTA = eswUpdate - esw;
//      pixels: object and probe steps (qNewton: whole-object max first)
//   M  mqNewton: gradient norms; adaptive-momentum step over the whole object
//      (tiles spread over the cluster) and the CTA's probe rows
// ASP replaces B by transfer-function column passes around a real-space
// projection row pass (Operators.py:155-230).
//
// This header holds the kernel template and its launch helpers; the
// instantiations are split over ptyg_engine.cu (ePIE / mPIE / qNewton) and
// ptyg_engine_mq.cu (mqNewton) so they compile in parallel.
#pragma once

#include <type_traits>

#include "ptyg_engine_dev.cuh"

namespace ptyg {

// max over one TILE x TILE object tile of sum_o |O_o|, this lane's share
// (8 pixels per lane; the caller reduces across the warp).
PTYG_DEV float tile_max(const ScanDev& s, int ty, int tx, int nosm, int No, size_t No2, int lane) {
  float m = 0.f;
#pragma unroll
  for (int q = 0; q < TILE * TILE / 32; ++q) {
    const int idx = q * 32 + lane;
    const int y = ty * TILE + idx / TILE, x = tx * TILE + idx % TILE;
    if (y < No && x < No) {
      float sum = 0.f;
      for (int o = 0; o < nosm; ++o) sum += cabs(ld_cg(s.object + o * No2 + (size_t)y * No + x));
      m = fmaxf(m, sum);
    }
  }
  return m;
}

// One mqNewton momentum step of one real component (mqNewton.py:142-182):
// updates the first moment m in place and returns X - beta_m * update, in the
// reference's float32 rounding order.  rb1 = 1/(1-beta1^itr) and rd =
// 1/(sqrt(v/(1-beta2^itr)) + 1e-8) are correctly rounded reciprocals: NumPy
// divides complex64 by a real-valued complex as a product with them.
struct MomStep {
  float b1, omb1, rb1, friction, rd, beta_m;
};

template <int METHOD>
PTYG_DEV float mom_step(const MomStep& p, float X, float g, float& m) {
  float u;
  if (METHOD == MOM_PLAIN) {
    m = __fadd_rn(g, __fmul_rn(p.friction, m));
    u = m;
  } else {
    m = __fadd_rn(__fmul_rn(p.b1, m), __fmul_rn(p.omb1, g));
    const float mh = __fmul_rn(m, p.rb1);
    if (METHOD == MOM_ADAM)
      u = __fmul_rn(mh, p.rd);
    else  // NADAM
      u = __fmul_rn(__fadd_rn(__fmul_rn(p.b1, mh), __fmul_rn(__fmul_rn(g, p.omb1), p.rb1)), p.rd);
  }
  return __fsub_rn(X, __fmul_rn(p.beta_m, u));
}

#ifndef PTYG_MQ_TILES_IN_FLIGHT
#define PTYG_MQ_TILES_IN_FLIGHT 1
#endif

// Loads the compiler may not move: the momentum pass issues every load of its
// tiles before the arithmetic that consumes them, so they overlap in flight.
PTYG_DEV float2 ld_cg_early(const float2* p) {
  float2 v;
  asm volatile("ld.global.cg.v2.f32 {%0, %1}, [%2];\n" : "=f"(v.x), "=f"(v.y) : "l"(p));
  return v;
}
PTYG_DEV float4 ld_cg_early4(const float2* p) {  // two complex64, 16-byte aligned
  float4 v;
  asm volatile("ld.global.cg.v4.f32 {%0, %1, %2, %3}, [%4];\n" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
  return v;
}
PTYG_DEV float2 ld_early(const float2* p) {  // generic address (shared or distributed shared memory)
  float2 v;
  asm volatile("ld.v2.f32 {%0, %1}, [%2];\n" : "=f"(v.x), "=f"(v.y) : "l"(p));
  return v;
}

// mqNewton's momentum step over the whole object (mqNewton.py:184-203):
// TILE x TILE tiles spread over the cluster's warps.  The gradient
// objectBuffer - object is zero outside the patch; inside it is read from the
// row owners' shared memory (gradO, nosm x L x NP per CTA).  The tile maxima
// of sum_o |O_o| are refreshed for the next position's probe step.  Each lane
// issues all loads of its tiles in flight (8 pixels x object, moment and
// gradient per tile) before using any: 4 KB of L2 traffic per warp and tile.
template <int NP, int L, int METHOD>
__device__ __forceinline__ void object_momentum_tiles(float2* object, float2* moment, float* tileMax, float2* gradO,
                                                      int No, int tilesPerRow, int nosm, int row0, int col0,
                                                      int crank, const MomStep st) {
  constexpr int C = NP / L, LN = L * NP;
  constexpr int PPL = TILE * TILE / 32;  // pixels per lane per tile: rows 2q + lane/16, column lane%16
  constexpr int TB = PTYG_MQ_TILES_IN_FLIGHT;  // tiles per warp in flight
  const unsigned lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const size_t No2 = (size_t)No * No;
  const int nt = tilesPerRow * tilesPerRow;
  const int stride = C * nw;
  const int ly = (int)(lane >> 4), lx = (int)(lane & 15);
  for (int t0 = crank * nw + warp; t0 < nt; t0 += TB * stride) {
    int y0[TB], x[TB];
    float sum[TB][PPL];
#pragma unroll
    for (int b = 0; b < TB; ++b) {
      const int t = t0 + b * stride;
      const int ty = t / tilesPerRow;
      y0[b] = t < nt ? ty * TILE + ly : No;  // rows of a tile past the end fail the bound
      x[b] = (t - ty * tilesPerRow) * TILE + lx;
#pragma unroll
      for (int q = 0; q < PPL; ++q) sum[b][q] = 0.f;
    }
    for (int o = 0; o < nosm; ++o) {
      float2 X[TB][PPL], M[TB][PPL], G[TB][PPL];
#pragma unroll
      for (int b = 0; b < TB; ++b) {
        const size_t base = (size_t)o * No2 + (size_t)y0[b] * No + x[b];
        const int c = x[b] - col0;
#pragma unroll
        for (int q = 0; q < PPL; ++q) {
          const int y = y0[b] + 2 * q;
          const bool ok = y < No && x[b] < No;
          const size_t gi = ok ? base + (size_t)(2 * q) * No : 0;  // pixel 0 stands in outside the object
          X[b][q] = ld_cg_early(object + gi);
          M[b][q] = ld_cg_early(moment + gi);
          // the patch gradient lives in the row owner's shared memory; other
          // pixels read this CTA's first entry and discard it
          const int r = y - row0;
          const bool in = ok && (unsigned)r < (unsigned)NP && (unsigned)c < (unsigned)NP;
          G[b][q] = ld_early(in ? dsmem(gradO, r / L) + o * LN + (r % L) * NP + c : gradO);
        }
      }
#pragma unroll
      for (int b = 0; b < TB; ++b) {
        const size_t base = (size_t)o * No2 + (size_t)y0[b] * No + x[b];
        const int c = x[b] - col0;
#pragma unroll
        for (int q = 0; q < PPL; ++q) {
          const int y = y0[b] + 2 * q;
          if (y < No && x[b] < No) {
            const size_t gi = base + (size_t)(2 * q) * No;
            const int r = y - row0;
            const bool in = (unsigned)r < (unsigned)NP && (unsigned)c < (unsigned)NP;
            const float2 g = in ? G[b][q] : make_float2(0.f, 0.f);
            const float2 Xn =
                make_float2(mom_step<METHOD>(st, X[b][q].x, g.x, M[b][q].x), mom_step<METHOD>(st, X[b][q].y, g.y, M[b][q].y));
            st_cg(moment + gi, M[b][q]);
            st_cg(object + gi, Xn);
            sum[b][q] += cabs(Xn);
          }
        }
      }
    }
#pragma unroll
    for (int b = 0; b < TB; ++b) {
      float mx = 0.f;
#pragma unroll
      for (int q = 0; q < PPL; ++q) mx = fmaxf(mx, sum[b][q]);
      mx = warp_max(mx);
      const int t = t0 + b * stride;
      if (lane == 0 && t < nt) tileMax[t] = mx;
    }
  }
}

// max over the pixels of one TILE x TILE object tile that lie outside the
// Np x Np patch at (row0, col0), of sum_o |O_o|, this lane's share.
PTYG_DEV float tile_max_outside(const ScanDev& s, int ty, int tx, int row0, int col0, int NP, int nosm, int No,
                                size_t No2, int lane) {
  float m = 0.f;
#pragma unroll
  for (int q = 0; q < TILE * TILE / 32; ++q) {
    const int idx = q * 32 + lane;
    const int y = ty * TILE + idx / TILE, x = tx * TILE + idx % TILE;
    const bool inPatch = (unsigned)(y - row0) < (unsigned)NP && (unsigned)(x - col0) < (unsigned)NP;
    if (y < No && x < No && !inPatch) {
      float sum = 0.f;
      for (int o = 0; o < nosm; ++o) sum += cabs(ld_cg(s.object + o * No2 + (size_t)y * No + x));
      m = fmaxf(m, sum);
    }
  }
  return m;
}

// The same step with 16-byte accesses (two pixels per lane and load), for an
// even object size and 16-byte aligned object and moment: strips of TILE rows
// x 2 TILE columns (two tiles) per warp; float4 f = q * 32 + lane of a strip
// covers strip row 2q + lane/16 and pixel columns 2 (lane % 16) + {0, 1}, so
// lanes 0-7 and 16-23 hold the left tile, 8-15 and 24-31 the right one.
template <int NP, int L, int METHOD>
__device__ __forceinline__ void object_momentum_strips(float2* object, float2* moment, float* tileMax, float2* gradO,
                                                       int No, int tilesPerRow, int nosm, int row0, int col0,
                                                       int crank, const MomStep st) {
  constexpr int C = NP / L, LN = L * NP;
  constexpr int QN = 2 * TILE * TILE / 64;  // float4 per lane per strip
  const unsigned lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const size_t No2 = (size_t)No * No;
  const int spr = (tilesPerRow + 1) / 2;  // strips per row of tiles
  const int ns = tilesPerRow * spr;
  const int lx = 2 * (int)(lane & 15), ly = (int)(lane >> 4);
  for (int si = crank * nw + warp; si < ns; si += C * nw) {
    const int ty = si / spr, sx = si - ty * spr;
    const int x = sx * 2 * TILE + lx, y0 = ty * TILE + ly;
    float mx = 0.f;
    float sum[QN][2];
#pragma unroll
    for (int q = 0; q < QN; ++q) sum[q][0] = sum[q][1] = 0.f;
    for (int o = 0; o < nosm; ++o) {
      float4 X[QN], M[QN];
      float2 G[QN][2];
#pragma unroll
      for (int q = 0; q < QN; ++q) {
        const int y = y0 + 2 * q;
        const bool ok = y < No && x < No;
        const size_t gi = ok ? (size_t)o * No2 + (size_t)y * No + x : 0;
        X[q] = ld_cg_early4(object + gi);
        M[q] = ld_cg_early4(moment + gi);
        const int r = y - row0;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          const int c = x + k - col0;
          const bool in = ok && (unsigned)r < (unsigned)NP && (unsigned)c < (unsigned)NP;
          G[q][k] = ld_early(in ? dsmem(gradO, r / L) + o * LN + (r % L) * NP + c : gradO);
        }
      }
#pragma unroll
      for (int q = 0; q < QN; ++q) {
        const int y = y0 + 2 * q;
        if (y < No && x < No) {
          const size_t gi = (size_t)o * No2 + (size_t)y * No + x;
          const int r = y - row0;
          float2 g[2];
#pragma unroll
          for (int k = 0; k < 2; ++k) {
            const int c = x + k - col0;
            g[k] = ((unsigned)r < (unsigned)NP && (unsigned)c < (unsigned)NP) ? G[q][k] : make_float2(0.f, 0.f);
          }
          float4 Xn;
          Xn.x = mom_step<METHOD>(st, X[q].x, g[0].x, M[q].x);
          Xn.y = mom_step<METHOD>(st, X[q].y, g[0].y, M[q].y);
          Xn.z = mom_step<METHOD>(st, X[q].z, g[1].x, M[q].z);
          Xn.w = mom_step<METHOD>(st, X[q].w, g[1].y, M[q].w);
          __stcg(reinterpret_cast<float4*>(moment + gi), M[q]);
          __stcg(reinterpret_cast<float4*>(object + gi), Xn);
          sum[q][0] += cabs(make_float2(Xn.x, Xn.y));
          sum[q][1] += cabs(make_float2(Xn.z, Xn.w));
        }
      }
    }
#pragma unroll
    for (int q = 0; q < QN; ++q) mx = fmaxf(mx, fmaxf(sum[q][0], sum[q][1]));
    // max within each tile's 16 lanes (xor offsets that keep bit 3 of the lane)
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 2));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 4));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 16));
    const int tx = 2 * sx + (int)((lane >> 3) & 1);
    if ((lane == 0 || lane == 8) && tx < tilesPerRow) tileMax[ty * tilesPerRow + tx] = mx;
  }
}

// Shared-memory layout of one CTA, in complex64 units.
struct Smem {
  float2* probe;    // npsm * L * NP, the CTA's probe rows (resident all launch)
  float2* obj;      // nosm * L * NP, this position's object patch rows
  float2* tile;     // K * NP * L: the CTA's column block (written by every CTA; swizzled, tix)
  float2* rows;     // K * L * NP: the CTA's rows, Fourier layout along x
  float2* U;        // qNewton probe numerators, npsm * L * NP
  float2* H;        // ASP (hInSmem): the CTA's L columns of the transfer function, one block per wavelength
  float* fr;        // L * NP projection factors
  float* dat;       // L * NP measured intensities: this position's, then (once the
                    // projection has read them) the next position's, in flight
  unsigned* slots;  // 2 * RED_BANK norm slots (used on rank 0)
  double* redD;     // 4 * 32
  float* redF;      // 4 * 32
  double* part;     // 4 * 16: mqNewton gradient-norm partials [value][CTA] (rank 0)
  unsigned long long* bar;  // the transfer function copy's mbarrier
};

__host__ __device__ inline size_t smem_complex_elems(int NP, int L, int K, int nosm, int npsm, bool qn,
                                                     bool probe_in_smem, int hBlocks) {
  const size_t LN = (size_t)L * NP;
  return (probe_in_smem ? (size_t)npsm * LN : 0) + (size_t)nosm * LN + (size_t)K * NP * L + (size_t)K * LN +
         (qn ? npsm * LN : 0) + (size_t)hBlocks * LN;
}

// ------------------------------------------------------------------ kernel
// E: Np / 32 points per lane; L: rows (and Fourier columns) per CTA, so the
// cluster has C = Np / L CTAs.  Both compile-time so index arithmetic is shifts.
// VAR: VAR_MQ is the mqNewton instantiation (engine == ENG_MQNEWTON), VAR_POLY
// ePIE / mPIE / qNewton over several wavelengths, VAR_STD ePIE / mPIE /
// qNewton at one, VAR_MQ_POLY mqNewton over several wavelengths.  VAR_FAST is
// VAR_STD with the common case's switches made compile-time constants (one
// wavelength, one object mode, Fraunhofer or Fresnel, the standard
// projection without background, masks or denoising), so its index
// arithmetic and mode loops fold away; the host picks it whenever they hold
// (launch_engine).  It computes exactly what VAR_STD computes.
enum { VAR_STD = 0, VAR_MQ = 1, VAR_POLY = 2, VAR_MQ_POLY = 3, VAR_FAST = 4 };
template <int E, int L, int VAR>
__global__ void __launch_bounds__((VAR == VAR_MQ || VAR == VAR_MQ_POLY) ? 256 : 512, 1)
    engine_kernel(const EngineArgs a) {
  constexpr bool MQ = VAR == VAR_MQ || VAR == VAR_MQ_POLY;
  constexpr bool POLY = VAR == VAR_POLY || VAR == VAR_MQ_POLY;
  constexpr bool FAST = VAR == VAR_FAST;
  // (512 threads x 128 registers: one CTA of 16 warps, or two of 8 warps, per
  // SM; mqNewton: at most 256 threads, so its momentum pass keeps all of a
  // tile's loads in registers)
  constexpr int NP = 32 * E;
  constexpr int C = NP / L;
  constexpr int LN = L * NP;
  const int crank = (int)(blockIdx.x % (unsigned)C);
  const ScanDev s = a.scans[blockIdx.x / C];
  const int line0 = crank * L, sx0 = crank * L;
  const unsigned lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // object and probe modes of every wavelength (wavelength-major); an exit
  // wave k = (l * nosmW + o) * npsmW + p pairs object mode l * nosmW + o with
  // probe mode l * npsmW + p of the same wavelength l
  const int nl = POLY ? a.nlambda : 1;  // a compile-time 1 outside the several-wavelength instantiations
  const int nosmW = FAST ? 1 : a.nosm, npsmW = a.npsm;
  const int nosm = nl * nosmW, npsm = nl * npsmW, K = nl * nosmW * npsmW, No = a.No;
  const bool centred = a.centred != 0;
  const bool fresnel = a.prop == PROP_FRESNEL;
  const bool asp = !FAST && a.prop == PROP_ASP;
  const int eng = a.engine;
  // mqNewton is its own instantiation (MQ): its momentum pass costs registers
  // the other engines' passes do not need
  const bool qn = MQ || eng == ENG_QNEWTON;
  constexpr bool mq = MQ;
  const size_t No2 = (size_t)No * No;
  const int blk0 = asp ? line0 : sx0;

  extern __shared__ float4 smem_f4[];
  Smem sm;
  // the CTA's probe rows: in shared memory when the layout fits (probeInSmem),
  // else in place in global memory (only this CTA touches them)
  const bool psm = a.probeInSmem != 0;
  const int pst = psm ? LN : NP * NP;  // stride between probe modes
  sm.probe = psm ? reinterpret_cast<float2*>(smem_f4) : s.probe + (size_t)line0 * NP;
  sm.obj = reinterpret_cast<float2*>(smem_f4) + (psm ? npsm * LN : 0);
  sm.tile = sm.obj + nosm * LN;
  sm.rows = sm.tile + K * NP * L;
  sm.U = sm.rows + K * LN;
  const bool hsm = asp && a.hInSmem;
  sm.H = sm.U + (qn ? npsm * LN : 0);
  sm.fr = reinterpret_cast<float*>(sm.H + (hsm ? nl * LN : 0));
  sm.dat = sm.fr + LN;
  sm.slots = reinterpret_cast<unsigned*>(sm.dat + LN);
  sm.redD = reinterpret_cast<double*>(sm.slots + 2 * RED_BANK);
  sm.redF = reinterpret_cast<float*>(sm.redD + 4 * 32);
  sm.part = reinterpret_cast<double*>(sm.redF + 4 * 32);
  sm.bar = reinterpret_cast<unsigned long long*>(sm.part + 4 * 16);
  unsigned* slots0 = dsmem(sm.slots, 0);
  // ASP: the CTA's columns sx0 .. sx0 + L of each wavelength's transfer
  // function are contiguous in the Fourier layout [sx][sy]: one bulk copy
  // per wavelength, read by the column filters of every position
  const float2* Htab = hsm ? sm.H : a.aspH;
  const size_t Hset = hsm ? (size_t)LN : (size_t)NP * NP;
  if (hsm) {
    if (!bulk_copy_wait(sm.H, a.aspH + (size_t)sx0 * NP, (unsigned)(LN * sizeof(float2)), nl, (size_t)NP * NP,
                        sm.bar) &&
        threadIdx.x == 0)
      atomicCAS(s.status, 0, 3);
  }

  if (psm) {
    for (int i = threadIdx.x; i < npsm * LN; i += blockDim.x) {
      const int p = i / LN, rem = i - (i / LN) * LN;
      sm.probe[i] = s.probe[(size_t)p * a.nslice * NP * NP + (size_t)line0 * NP + rem];
    }
  }
  if (threadIdx.x < 2 * RED_BANK) sm.slots[threadIdx.x] = 0u;
  prefetch_data<NP, L, false>(a, s, sm.dat, 0, blk0);
  WarpFFT<E> F;  // the column transforms (rows: row_tasks)
  F.init(a.twiddle, lane);
  // mqNewton second moments: every CTA of the cluster carries the same values
  float vO = 0.f, vP = 0.f;
  if (mq && s.moment2) {
    vO = s.moment2[0];
    vP = s.moment2[1];
  }
  if (qn) {
    // all tile maxima once per launch
    const int nt = a.tilesPerRow * a.tilesPerRow;
    for (int t = crank * nw + warp; t < nt; t += C * nw) {
      const float v = warp_max(tile_max(s, t / a.tilesPerRow, t % a.tilesPerRow, nosm, No, No2, lane));
      if (lane == 0) s.tileMax[t] = v;
    }
  }
  __syncthreads();
  cluster_sync(C);

  const float inv2 = 1.f / (float)(NP * NP);

  for (int it = 0; it < a.count; ++it) {
    const int frame = s.order[a.start + it];
    const int row0 = (frame >= 0 && frame < a.numFrames) ? s.positions[2 * frame] : -1;
    const int col0 = (frame >= 0 && frame < a.numFrames) ? s.positions[2 * frame + 1] : -1;
    if (row0 < 0 || col0 < 0 || row0 > No - NP || col0 > No - NP) {
      if (crank == 0 && threadIdx.x == 0) atomicCAS(s.status, 0, 2);
      prefetch_data<NP, L, false>(a, s, sm.dat, it + 1, blk0);  // nothing reads dat here
      continue;  // uniform across the cluster
    }
    unsigned* red = slots0 + (it & 1) * RED_BANK;
    const float* dat = sm.dat;

    // ---------------- A: stage the patch rows, norms, exit waves, row FFT
    {
      // stage the patch and take, in the same pass over the CTA's pixels, the
      // max of sum_p|P|^2, sum_o|O|^2 (patch), sum_p|P| (qNewton), and for
      // qNewton the max of sum_o|O| over the object outside the patch, which
      // this position leaves unchanged until its momentum step
      float mx[4] = {0.f, 0.f, 0.f, 0.f};
      auto norms = [&](int i, float so2) {
        float sp2 = 0.f, sp1 = 0.f;
        for (int p = 0; p < npsm; ++p) {
          const float q = cabs2(sm.probe[p * pst + i]);
          sp2 += q;
          if (qn) sp1 += sqrtf(q);
        }
        mx[0] = fmaxf(mx[0], sp2);
        mx[1] = fmaxf(mx[1], so2);
        mx[2] = fmaxf(mx[2], sp1);
      };
      if constexpr (FAST) {
        // one object mode: a thread's loads of up to four pixels are all in
        // flight before the first is used
        constexpr int U = 4;
        for (int i0 = threadIdx.x; i0 < LN; i0 += U * (int)blockDim.x) {
          float2 v[U];
#pragma unroll
          for (int q = 0; q < U; ++q) {
            const int i = i0 + q * (int)blockDim.x;
            const int ic = i < LN ? i : i0;
            const int l = ic / NP, x = ic - (ic / NP) * NP;
            v[q] = ld_cg(s.object + (size_t)(row0 + line0 + l) * No + col0 + x);
          }
#pragma unroll
          for (int q = 0; q < U; ++q) {
            const int i = i0 + q * (int)blockDim.x;
            if (i < LN) {
              sm.obj[i] = v[q];
              norms(i, cabs2(v[q]));
            }
          }
        }
      } else {
        for (int i = threadIdx.x; i < LN; i += blockDim.x) {
          const int l = i / NP, x = i - (i / NP) * NP;
          const float2* src = s.object + (size_t)(row0 + line0 + l) * No + col0 + x;
          float so2 = 0.f;
          for (int o = 0; o < nosm; ++o) {
            const float2 v = ld_cg(src + o * No2);
            sm.obj[o * LN + i] = v;
            so2 += cabs2(v);
          }
          norms(i, so2);
        }
      }
      if (qn) {
        // qNewton.py:130 takes the max over the whole object after the patch
        // step: kept exactly from per-tile maxima.  Tiles away from the patch
        // are read back; for the tiles the patch touches, the pixels outside
        // it are recomputed here (and stored as the tile's max, which pass C
        // raises with the new patch pixels).
        const int tpr = a.tilesPerRow;
        const int ty0 = row0 / TILE, ty1 = (row0 + NP - 1) / TILE;
        const int tx0 = col0 / TILE, tx1 = (col0 + NP - 1) / TILE;
        const int tw = tx1 - tx0 + 1, nPatchTiles = (ty1 - ty0 + 1) * tw;
        for (int t = crank * nw + warp; t < nPatchTiles; t += C * nw) {
          const int ty = ty0 + t / tw, tx = tx0 + t % tw;
          const float v = warp_max(tile_max_outside(s, ty, tx, row0, col0, NP, nosm, No, No2, lane));
          mx[3] = fmaxf(mx[3], v);
          if (lane == 0) s.tileMax[ty * tpr + tx] = v;
        }
        const int nt = tpr * tpr;
        for (int t = crank * blockDim.x + threadIdx.x; t < nt; t += C * blockDim.x) {
          const int ty = t / tpr, tx = t - ty * tpr;
          if (ty < ty0 || ty > ty1 || tx < tx0 || tx > tx1) mx[3] = fmaxf(mx[3], __ldcg(s.tileMax + t));
        }
      }
      const int idx[4] = {RED_PMAX2, RED_OMAX2, RED_PMAX1, RED_OMAXW};
      block_max_to_slots<4>(mx, sm.redF, red, idx);
    }
    // (the row buffers are free until pass B writes them: exchange buffers)
    row_tasks<E, false>(
        a.twiddle, K * L,
        [&](int t, int lo, int hi) {
          const int k = t / L, l = t % L;
          const int o = nosm == 1 ? 0 : k / npsmW, p = (nl == 1 ? 0 : (o / nosmW) * npsmW) + (k - o * npsmW);
          const int y = line0 + l;
          float2 e = cmul(sm.obj[(o * L + l) * NP + lo + hi], sm.probe[p * pst + l * NP + lo + hi]);
          if (fresnel) e = cmul(e, __ldg(a.fresnelQ + y * NP + lo + hi));
          return cscale(e, (centred && !asp && ((y + lo) & 1)) ? -1.f : 1.f);  // hi is even
        },
        [&](int t, int lo, int hi, float2 v) { scatter_row<NP, L>(sm.tile, t / L, line0 + t % L, lo, hi, v); },
        [&](int t) { return reinterpret_cast<float4*>(sm.rows + t * NP); });
    cp_async_wait_all();  // this position's intensities (the one group in flight)
    cluster_sync(C);

    // The intensity projection of this CTA's pixels (project_intensities):
    // cols (a compile-time tag) picks the warp-per-column form of the fused
    // pass B.  The interferometric constraint is compiled into the
    // several-wavelength instantiation only (which serves ePIE, mPIE and
    // qNewton for any nlambda), so the standard kernel's registers stay as
    // they are.
    const bool interf = VAR == VAR_POLY && a.iconstraint == IC_INTERFEROMETRIC;
    const int icon = FAST ? (int)IC_STANDARD : a.iconstraint;
    const bool denoise = !FAST && a.denoise;
    auto project = [&](auto Iest, float outScale, auto colsTag) -> double {
      return project_intensities<NP, L, FAST, VAR == VAR_POLY, decltype(colsTag)::value>(
          a, s, frame, blk0, crank, ProjectionIO{sm.fr, dat, sm.part, sm.redD}, Iest, outScale);
    };

    double err = 0.0;
    if (!asp && nw == L && !(denoise || icon == IC_FLUCTUATION || interf)) {
      // ---------------- B, fused: warp w owns column w of every mode, so it
      // transforms the column's K modes, sums their intensities in
      // registers, projects its own pixels and transforms back, with no
      // block-wide barrier in between (the tile column and its factors are
      // written and read by this warp only)
      const int c = warp;
      float ie[E];
#pragma unroll
      for (int r = 0; r < E; ++r) ie[r] = 0.f;
      auto colLoad = [&](int k, float2(&v)[E]) {
#pragma unroll
        for (int j = 0; j < E; ++j) v[j] = sm.tile[tix<L>(k * NP + lane + 32 * j, c)];
      };
      auto colStore = [&](int k, const float2(&v)[E]) {
#pragma unroll
        for (int r = 0; r < E; ++r) {
          sm.tile[tix<L>(k * NP + 32 * r + lane, c)] = v[r];
          ie[r] += cabs2(v[r]);
        }
      };
      int k = 0;
      for (; k + 1 < K; k += 2) {
        float2 v[2][E];
        colLoad(k, v[0]);
        colLoad(k + 1, v[1]);
        F.fwd2(v);
        __syncwarp();
        colStore(k, v[0]);
        colStore(k + 1, v[1]);
      }
      if (k < K) {
        float2 v[E];
        colLoad(k, v);
        F.fwd(v);
        __syncwarp();
        colStore(k, v);
      }
      err = project([&](int r) { return __fmul_rn(ie[r], inv2); }, inv2, std::true_type{});
      __syncwarp();
      auto invLoad = [&](int kk, float2(&v)[E]) {
#pragma unroll
        for (int r = 0; r < E; ++r)
          v[r] = cscale(sm.tile[tix<L>(kk * NP + 32 * r + lane, c)], sm.fr[c * NP + 32 * r + lane]);
      };
      for (k = 0; k + 1 < K; k += 2) {
        float2 v[2][E];
        invLoad(k, v[0]);
        invLoad(k + 1, v[1]);
        F.inv2(v);
        __syncwarp();  // the column is stored in place of what the warp loaded
        store_column<E, L>(sm.tile, v[0], k, c);
        store_column<E, L>(sm.tile, v[1], k + 1, c);
      }
      if (k < K) {
        float2 v[E];
        invLoad(k, v);
        F.inv(v);
        __syncwarp();
        store_column<E, L>(sm.tile, v, k, c);
      }
      __syncthreads();
      flush_columns<NP, L>(sm.tile, sm.rows, K, sx0);
    } else if (!asp) {
      // ---------------- B: Fourier-plane intensity projection (BaseEngine.py:870-1012)
      auto col = [&](int t, int i) -> float2& { return sm.tile[tix<L>((t / L) * NP + i, t % L)]; };
      fft_tasks<E, false>(
          F, K * L, [&](int t, int lo, int hi) { return col(t, lo + hi); },
          [&](int t, int lo, int hi, float2 v) { col(t, lo + hi) = v; });
      __syncthreads();
      // interferometric: the reference field of this CTA's pixels, plane k at
      // + k * NP * NP, held as N M R in the tile's scale and sign
      float2* refb = interf ? s.reference + (size_t)blk0 * NP : nullptr;
      err = project(
          [&](int i) {
            const int c = i / NP, sy = i - (i / NP) * NP;
            float ie = 0.f;
            if (interf) {  // BaseEngine.py:883-888: sum |Psi + R|^2
              for (int k = 0; k < K; ++k) {
                const float2 v = sm.tile[tix<L>(k * NP + sy, c)], r = refb[(size_t)k * NP * NP + i];
                ie += cabs2(make_float2(v.x + r.x, v.y + r.y));
              }
            } else {
              for (int k = 0; k < K; ++k) ie += cabs2(sm.tile[tix<L>(k * NP + sy, c)]);
            }
            return __fmul_rn(ie, inv2);  // explicit rounding: every column path rounds alike
          },
          inv2, std::false_type{});
      if (interf) {
        // BaseEngine.py:975-982: Psi' = (Psi + R) frac - R, R' = (Psi + R) frac - Psi
        __syncthreads();
        for (int i = threadIdx.x; i < LN; i += blockDim.x) {
          const int c = i / NP, sy = i - (i / NP) * NP;
          const float f = sm.fr[i];
          for (int k = 0; k < K; ++k) {
            float2& v = sm.tile[tix<L>(k * NP + sy, c)];
            float2* rp = refb + (size_t)k * NP * NP + i;
            const float2 r = *rp, psi = v;
            const float2 sf = make_float2((psi.x + r.x) * f, (psi.y + r.y) * f);
            *rp = make_float2(sf.x - psi.x, sf.y - psi.y);
            v = make_float2(sf.x - r.x, sf.y - r.y);
          }
          sm.fr[i] = inv2;
        }
      }
      __syncthreads();
      fft_tasks<E, true>(
          F, K * L, [&](int t, int lo, int hi) { return cscale(col(t, lo + hi), sm.fr[(t % L) * NP + lo + hi]); },
          [&](int t, int lo, int hi, float2 v) { col(t, lo + hi) = v; });
      __syncthreads();
      flush_columns<NP, L>(sm.tile, sm.rows, K, sx0);
    } else {
      // ---------------- ASP: x H, real-space projection, x conj(H)
      column_filter<E, L, POLY>(sm.tile, sm.rows, F, Htab, Hset, hsm, false, crank, K, nosmW * npsmW);
      cluster_sync(C);
      auto row = [&](int t, int i) -> float2& { return sm.rows[t * NP + i]; };
      auto pairs = [&](int t) { return reinterpret_cast<float4*>(sm.rows + t * NP); };
      row_tasks<E, true>(
          a.twiddle, K * L, [&](int t, int lo, int hi) { return row(t, rsw<L>(t, lo) + hi); },
          [&](int t, int lo, int hi, float2 v) { row(t, lo + hi) = v; }, pairs);
      __syncthreads();
      err = project(
          [&](int i) {
            float ie = 0.f;
            for (int k = 0; k < K; ++k) ie += cabs2(sm.rows[k * LN + i]);
            return ie;
          },
          1.f, std::false_type{});
      __syncthreads();
      row_tasks<E, false>(
          a.twiddle, K * L, [&](int t, int lo, int hi) { return cscale(row(t, lo + hi), sm.fr[(t % L) * NP + lo + hi]); },
          [&](int t, int lo, int hi, float2 v) { scatter_row<NP, L>(sm.tile, t / L, line0 + t % L, lo, hi, v); }, pairs);
      cluster_sync(C);
      column_filter<E, L, POLY>(sm.tile, sm.rows, F, Htab, Hset, hsm, true, crank, K, nosmW * npsmW);
    }
    // every read of dat (the projection) and of redD (its cluster sums) is
    // behind this barrier: fetch the next position's intensities into dat
    // while C and A run
    __syncthreads();
    prefetch_data<NP, L, false>(a, s, sm.dat, it + 1, blk0);
    if (crank == 0 && threadIdx.x < RED_BANK) sm.slots[((it & 1) ^ 1) * RED_BANK + threadIdx.x] = 0u;
    // this CTA's column results are in the row owners' buffers: arrive, and
    // reduce the error partial while the other CTAs finish pass B
    cluster_arrive(C);
    {
      const double t = block_sum(err, sm.redD);
      if (threadIdx.x == 0) s.errPart[(size_t)frame * C + crank] = t;
    }
    cluster_wait(C);

    // ---------------- C: inverse row FFT and DELTA per mode
    row_tasks<E, true>(
        a.twiddle, K * L, [&](int t, int lo, int hi) { return sm.rows[t * NP + rsw<L>(t, lo) + hi]; },
        [&](int t, int lo, int hi, float2 v) {
          const int k = t / L, l = t % L;
          const int o = nosm == 1 ? 0 : k / npsmW, p = (nl == 1 ? 0 : (o / nosmW) * npsmW) + (k - o * npsmW);
          const int y = line0 + l;
          const int x = lo + hi;
          float2 u = cscale(v, (centred && !asp && ((y + lo) & 1)) ? -1.f : 1.f);  // hi is even
          if (fresnel) u = cmulc(__ldg(a.fresnelQ + y * NP + x), u);
          const float2 esw = cmul(sm.obj[(o * L + l) * NP + x], sm.probe[p * pst + l * NP + x]);
          sm.rows[t * NP + x] = csub(u, esw);
        },
        [&](int t) { return reinterpret_cast<float4*>(sm.rows + t * NP); });
    __syncthreads();

    // ---------------- C: object and probe steps, pixel by pixel
    float omaxPatch = 0.f;  // qNewton: max over the new patch of sum_o |O_o|
    // mqNewton sums over the patch: |objectBuffer - object|^2, and with
    // d = probeBuffer - probe and the probe numerator U: |d|^2, Re(conj(d) U),
    // |U|^2, from which |probeBuffer - (probe + U/Omax)|^2 follows once Omax is
    // known.  A pixel's terms are FP32 with explicit rounding, summed over
    // the modes in order; a warp sums its 32-pixel row segment in a fixed
    // FP32 tree, and the segment sums (FP64, in sm.tile, free in this pass)
    // in the balanced tree over segment order, per CTA here and over the
    // cluster in pass M: the same tree for every CTA shape, so a batched
    // launch gives a single-scan launch's bits.  (FP64 per pixel would cost
    // more than the rest of the pass on this GPU's FP64 rate.)
    const int nseg = LN / 32;
    double* segSum = reinterpret_cast<double*>(sm.tile);  // [4][nseg]
    {
      const float pmax2 = slot_value(red, RED_PMAX2);
      const float omax2 = slot_value(red, RED_OMAX2);
      const float pmax1 = slot_value(red, RED_PMAX1);
      const float invPmax2 = 1.f / pmax2, invOmax2 = 1.f / omax2, invPmax1 = 1.f / pmax1;
      const float stepP = a.betaP * a.weightP;
      if constexpr (FAST) {
        // one object mode, one wavelength, no mqNewton: each thread takes up
        // to PPT pixels at once and runs the probe modes outermost, so the
        // pixels' independent chains interleave; per pixel the arithmetic and
        // its order are those of the general loop below
        constexpr int PPT = LN >= 2048 ? 4 : (LN >= 512 ? LN / 512 : 1);
        auto gObjF = [&](float qp) {
          if (eng == ENG_EPIE) return invPmax2;
          if (eng == ENG_MPIE) {
            float g = 1.f / (a.alphaO * pmax2 + (1.f - a.alphaO) * qp);
            if (a.fpm) g *= sqrtf(qp) * invPmax2;
            return g;
          }
          return sqrtf(qp) * invPmax1 / (qp + a.regO);
        };
        for (int base = 0; base < LN; base += PPT * (int)blockDim.x) {
          int idx[PPT];
          float2 O[PPT], accO[PPT];
          float gP[PPT];
#pragma unroll
          for (int q = 0; q < PPT; ++q) {
            idx[q] = base + (int)threadIdx.x + q * (int)blockDim.x;  // warp-uniform validity
            O[q] = sm.obj[idx[q] < LN ? idx[q] : 0];
            accO[q] = make_float2(0.f, 0.f);
            const float qq = cabs2(O[q]);
            if (eng == ENG_EPIE)
              gP[q] = invOmax2;
            else if (eng == ENG_MPIE)
              gP[q] = 1.f / (a.alphaP * omax2 + (1.f - a.alphaP) * qq);
            else
              gP[q] = sqrtf(qq) / (qq + a.regP);
          }
          for (int p = 0; p < npsm; ++p) {
#pragma unroll
            for (int q = 0; q < PPT; ++q) {
              if (idx[q] < LN) {
                const int i = idx[q];
                const float2 P = sm.probe[p * pst + i];
                const float2 d = sm.rows[p * LN + i];
                accO[q] = cadd(accO[q], cscale(cmulc(P, d), gObjF(cabs2(P))));
                const float2 accP = cadd(make_float2(0.f, 0.f), cscale(cmulc(O[q], d), gP[q]));
                if (qn)
                  sm.U[p * LN + i] = accP;
                else
                  sm.probe[p * pst + i] = cadd(P, cscale(accP, stepP));
              }
            }
          }
#pragma unroll
          for (int q = 0; q < PPT; ++q) {
            if (idx[q] < LN) {
              const int i = idx[q];
              const int l = i / NP, x = i - (i / NP) * NP;
              const float2 On = cadd(O[q], cscale(accO[q], a.betaO));
              st_cg(s.object + (size_t)(row0 + line0 + l) * No + col0 + x, On);
              if (qn) {
                const float onew = cabs(On);
                omaxPatch = fmaxf(omaxPatch, onew);
                const int tx = (col0 + x) / TILE;
                const unsigned grp = __match_any_sync(0xffffffffu, tx);
                const unsigned m = __reduce_max_sync(grp, __float_as_uint(onew));
                if ((int)lane == __ffs(grp) - 1)
                  atomicMax(reinterpret_cast<unsigned*>(s.tileMax) + ((row0 + line0 + l) / TILE) * a.tilesPerRow + tx, m);
              }
            }
          }
        }
      } else
      for (int i = threadIdx.x; i < LN; i += blockDim.x) {
        float2 O[MAX_OBJECT_MODES], accO[MAX_OBJECT_MODES];
        float gP[MAX_OBJECT_MODES];
        float tgO = 0.f, tdd = 0.f, tdu = 0.f, tuu = 0.f;
#pragma unroll
        for (int o = 0; o < MAX_OBJECT_MODES; ++o) {
          if (o < nosm) {
            O[o] = sm.obj[o * LN + i];
            accO[o] = make_float2(0.f, 0.f);
            const float q = cabs2(O[o]);
            if (eng == ENG_EPIE)
              gP[o] = invOmax2;  // ePIE.py:154-156
            else if (eng == ENG_MPIE)
              gP[o] = 1.f / (a.alphaP * omax2 + (1.f - a.alphaP) * q);  // mPIE.py:262-264
            else
              gP[o] = sqrtf(q) / (q + a.regP);  // qNewton.py:131-136 (1/Omax applied later)
          }
        }
        // per-wavelength probe mode p; with several wavelengths object mode
        // o pairs with the probe of wavelength o / nosmW.  ePIE and qNewton
        // sum their steps over the wavelengths (ePIE.py:128-160, qNewton.py
        // :108-140: axes 0, 2, 3 and 0, 1, 3) and give every wavelength's
        // copy the same step; mPIE sums over the probe modes (object) and
        // the object modes (probe) of each wavelength only (mPIE.py:226-270:
        // axis 2 and axis 1).
        auto gObj = [&](float qp) {  // the object step's weight for a probe mode of intensity qp
          if (eng == ENG_EPIE) return invPmax2;  // ePIE.py:138-140
          if (eng == ENG_MPIE) {
            float g = 1.f / (a.alphaO * pmax2 + (1.f - a.alphaO) * qp);  // mPIE.py:246-248
            if (a.fpm) g *= sqrtf(qp) * invPmax2;                         // mPIE.py:237-243
            return g;
          }
          return sqrtf(qp) * invPmax1 / (qp + a.regO);  // qNewton.py:113-119
        };
        const bool perLambda = nl > 1 && eng == ENG_MPIE;
        for (int p = 0; p < npsmW; ++p) {
          const float2 P = sm.probe[p * pst + i];
          const float gO = gObj(cabs2(P));
          float2 accP = make_float2(0.f, 0.f);
#pragma unroll
          for (int o = 0; o < MAX_OBJECT_MODES; ++o) {
            if (o < nosm) {
              float2 Po = P;
              float gOo = gO;
              if (nl > 1) {
                Po = sm.probe[((o / nosmW) * npsmW + p) * pst + i];
                gOo = gObj(cabs2(Po));
              }
              const float2 d = sm.rows[(o * npsmW + p) * LN + i];
              accO[o] = cadd(accO[o], cscale(cmulc(Po, d), gOo));
              accP = cadd(accP, cscale(cmulc(O[o], d), gP[o]));
              if (perLambda && o % nosmW == nosmW - 1) {
                // the last object mode of wavelength o / nosmW: its probe step
                sm.probe[((o / nosmW) * npsmW + p) * pst + i] = cadd(Po, cscale(accP, stepP));
                accP = make_float2(0.f, 0.f);
              }
            }
          }
          if (qn) {
            sm.U[p * LN + i] = accP;  // several wavelengths: summed over them
          } else if (nl == 1) {
            sm.probe[p * pst + i] = cadd(P, cscale(accP, stepP));
          } else if (!perLambda) {
            for (int w = 0; w < nl; ++w) {
              float2* Pw = sm.probe + (w * npsmW + p) * pst + i;
              *Pw = cadd(*Pw, cscale(accP, stepP));
            }
          }
          if (mq) {
            // the probe gradient's norm covers every wavelength's copy: each
            // takes the same numerator U (mqNewton.py:205-215 on the whole probe)
            for (int w = 0; w < nl; ++w) {
              const int pw = w * npsmW + p;
              const float2 Pw = nl == 1 ? P : sm.probe[pw * pst + i];
              const float2 d = csub(s.probeBuffer[(size_t)pw * NP * NP + (size_t)line0 * NP + i], Pw);
              tdd = __fadd_rn(tdd, __fmaf_rn(d.x, d.x, __fmul_rn(d.y, d.y)));
              tdu = __fadd_rn(tdu, __fmaf_rn(d.x, accP.x, __fmul_rn(d.y, accP.y)));
              tuu = __fadd_rn(tuu, __fmaf_rn(accP.x, accP.x, __fmul_rn(accP.y, accP.y)));
            }
          }
        }
        const int l = i / NP, x = i - (i / NP) * NP;
        float onew = 0.f;
#pragma unroll
        for (int o = 0; o < MAX_OBJECT_MODES; ++o) {
          if (o < nosm) {
            float2 u = accO[o];
            if (nl > 1 && !perLambda) {
              u = make_float2(0.f, 0.f);
#pragma unroll
              for (int o2 = 0; o2 < MAX_OBJECT_MODES; ++o2)
                if (o2 < nosm && o2 % nosmW == o % nosmW) u = cadd(u, accO[o2]);
            }
            const float2 On = cadd(O[o], cscale(u, a.betaO));
            st_cg(s.object + o * No2 + (size_t)(row0 + line0 + l) * No + col0 + x, On);
            onew += cabs(On);
            if (mq) {
              // gradient = objectBuffer - object (mqNewton.py:190): the buffer
              // equals the object after every momentum step (nothing between
              // positions or iterations touches one without the other), so
              // it is the patch as it was before this step; kept for pass M
              const float2 g = csub(O[o], On);
              sm.obj[o * LN + i] = g;
              tgO = __fadd_rn(tgO, __fmaf_rn(g.x, g.x, __fmul_rn(g.y, g.y)));
            }
          }
        }
        if (mq) {
          // warp-uniform: LN and blockDim are multiples of 32
          tgO = warp_tree_sumf(tgO);
          tdd = warp_tree_sumf(tdd);
          tdu = warp_tree_sumf(tdu);
          tuu = warp_tree_sumf(tuu);
          if (lane < 4)
            segSum[lane * nseg + (i >> 5)] = (double)(lane == 0 ? tgO : lane == 1 ? tdd : lane == 2 ? tdu : tuu);
        }
        if (qn) {
          omaxPatch = fmaxf(omaxPatch, onew);
          if (!mq) {
            // raise the maxima of the tiles this row segment touches (a warp
            // covers 32 consecutive pixels of one row: two or three tiles)
            const int tx = (col0 + x) / TILE;
            const unsigned grp = __match_any_sync(0xffffffffu, tx);
            const unsigned m = __reduce_max_sync(grp, __float_as_uint(onew));
            if ((int)lane == __ffs(grp) - 1)
              atomicMax(reinterpret_cast<unsigned*>(s.tileMax) + ((row0 + line0 + l) / TILE) * a.tilesPerRow + tx, m);
          }
        }
      }
      if (qn) {
        float m[1] = {omaxPatch};
        const int idx[1] = {RED_OMAXW};
        block_max_to_slots<1>(m, sm.redF, red, idx);
      }
      if (mq) {
        __syncthreads();
        if (warp < 4) {
          const double v = tree_sum(segSum + warp * nseg, nseg, lane);
          if (lane == 0) dsmem(sm.part, 0)[warp * C + crank] = v;
        }
      }
    }

    if (qn) {
      cluster_sync(C);  // every contribution to the whole-object max (and mqNewton's partial sums) is in
      const float scale = a.betaP / slot_value(red, RED_OMAXW);
      if (!mq) {
        // several wavelengths: every wavelength's probe mode p takes the
        // numerator summed over the wavelengths, U[p % npsmW]
        for (int i = threadIdx.x; i < npsm * LN; i += blockDim.x) {
          const int p = i / LN, rem = i - (i / LN) * LN;
          const int pu = nl == 1 ? p : p % npsmW;
          sm.probe[p * pst + rem] = cadd(sm.probe[p * pst + rem], cscale(sm.U[pu * LN + rem], scale));
        }
      } else {
        // ---------------- M: adaptive momentum (mqNewton.py:142-224) after every
        // position, on the whole object and probe, in the reference's complex64
        // rounding order: NumPy divides complex64 by a real-valued complex as a
        // product with the correctly rounded reciprocal, hence __frcp_rn.
        double t0, t1;
        {
          // lanes [0,2C) read [|gO|^2 | |d|^2] and then [Re conj(d)U | |U|^2]
          // partials; the xor butterfly from offset 1 up sums each group of C
          // lanes in the balanced tree over CTA order, in every warp and CTA
          const double* src = dsmem(sm.part, 0);
          t0 = (int)lane < 2 * C ? src[lane] : 0.0;
          t1 = (int)lane < 2 * C ? src[2 * C + lane] : 0.0;
#pragma unroll
          for (int off = 1; off < C; off <<= 1) {
            t0 += __shfl_xor_sync(0xffffffffu, t0, off);
            t1 += __shfl_xor_sync(0xffffffffu, t1, off);
          }
        }
        const double nsqO = __shfl_sync(0xffffffffu, t0, 0), dd = __shfl_sync(0xffffffffu, t0, C);
        const double du = __shfl_sync(0xffffffffu, t1, 0), uu = __shfl_sync(0xffffffffu, t1, C);
        const double sc = (double)scale;
        const double nsqP = fmax(dd - 2.0 * sc * du + sc * sc * uu, 0.0);
        const int method = a.momentum;
        const float rb1 = __frcp_rn(a.b1s);
        float rdO = 1.f, rdP = 1.f;
        if (method != MOM_PLAIN) {
          // vt = beta2*vt + (1-beta2)*||grad||^2 ; 1/(sqrt(vt/(1-beta2^itr)) + 1e-8)
          const float rb2 = __frcp_rn(a.b2s);
          const float nO = __fsqrt_rn((float)nsqO), nP = __fsqrt_rn((float)nsqP);
          vO = __fadd_rn(__fmul_rn(a.b2, vO), __fmul_rn(a.omb2, __fmul_rn(nO, nO)));
          vP = __fadd_rn(__fmul_rn(a.b2, vP), __fmul_rn(a.omb2, __fmul_rn(nP, nP)));
          rdO = __frcp_rn(__fadd_rn(__fsqrt_rn(__fmul_rn(vO, rb2)), 1e-8f));
          rdP = __frcp_rn(__fadd_rn(__fsqrt_rn(__fmul_rn(vP, rb2)), 1e-8f));
        }
        const MomStep stO{a.b1, a.omb1, rb1, a.frictionM, rdO, a.betaOm};
        const MomStep stP{a.b1, a.omb1, rb1, a.frictionM, rdP, a.betaPm};
        // probe: qNewton step, then the momentum step, on the CTA's own rows;
        // gradient probeBuffer - probe (mqNewton.py:211), the buffer read, not
        // assumed: the probe constraints between iterations move the probe
        // but not its buffer
        for (int i = threadIdx.x; i < npsm * LN; i += blockDim.x) {
          const int p = i / LN, rem = i - (i / LN) * LN;
          const size_t gi = (size_t)p * NP * NP + (size_t)line0 * NP + rem;
          const int pu = nl == 1 ? p : p % npsmW;  // every wavelength takes U summed over them
          const float2 P = cadd(sm.probe[p * pst + rem], cscale(sm.U[pu * LN + rem], scale));
          const float2 g = csub(s.probeBuffer[gi], P);
          float2 M = s.probeMomentum[gi];
          float2 Pn;
          if (method == MOM_ADAM)
            Pn = make_float2(mom_step<MOM_ADAM>(stP, P.x, g.x, M.x), mom_step<MOM_ADAM>(stP, P.y, g.y, M.y));
          else if (method == MOM_NADAM)
            Pn = make_float2(mom_step<MOM_NADAM>(stP, P.x, g.x, M.x), mom_step<MOM_NADAM>(stP, P.y, g.y, M.y));
          else
            Pn = make_float2(mom_step<MOM_PLAIN>(stP, P.x, g.x, M.x), mom_step<MOM_PLAIN>(stP, P.y, g.y, M.y));
          s.probeMomentum[gi] = M;
          s.probeBuffer[gi] = Pn;
          sm.probe[p * pst + rem] = Pn;
        }
#define PTYG_TILES(m)                                                                                           \
  if (s.vec4)                                                                                                   \
    object_momentum_strips<NP, L, m>(s.object, s.objectMomentum, s.tileMax, sm.obj, No, a.tilesPerRow, nosm,    \
                                     row0, col0, crank, stO);                                                   \
  else                                                                                                          \
    object_momentum_tiles<NP, L, m>(s.object, s.objectMomentum, s.tileMax, sm.obj, No, a.tilesPerRow, nosm, row0, \
                                    col0, crank, stO)
        if (method == MOM_ADAM) {
          PTYG_TILES(MOM_ADAM);
        } else if (method == MOM_NADAM) {
          PTYG_TILES(MOM_NADAM);
        } else {
          PTYG_TILES(MOM_PLAIN);
        }
#undef PTYG_TILES
      }
    }

    if (eng == ENG_MPIE && s.momentum && s.momentum[a.start + it]) {
      // momentum step on the whole object and probe (mPIE.py:196-224), in the
      // reference's complex64 arithmetic and rounding order (no fused multiply-add):
      //   M <- (buffer - X) + friction*M ;  X <- X - feedback*M ;  buffer <- X
      cluster_sync(C);
      const float eta = a.frictionM, nu = a.feedbackM;
      auto step = [&](float2 X, float2 B, float2 M, float2& Xn, float2& Mn) {
        Mn = make_float2(__fadd_rn(__fsub_rn(B.x, X.x), __fmul_rn(eta, M.x)),
                         __fadd_rn(__fsub_rn(B.y, X.y), __fmul_rn(eta, M.y)));
        Xn = make_float2(__fsub_rn(X.x, __fmul_rn(nu, Mn.x)), __fsub_rn(X.y, __fmul_rn(nu, Mn.y)));
      };
      const size_t nobj = (size_t)nosm * No2;
      const size_t stride = (size_t)C * blockDim.x;
      if (s.vec4 && ((reinterpret_cast<uintptr_t>(s.objectBuffer) & 15) == 0)) {
        // 16-byte accesses (two pixels), MU of them per array in flight per
        // thread before any is used: the pass streams three arrays, so it
        // runs at what L2 delivers rather than one load latency per pixel
        constexpr int MU = 4;
        const size_t n4 = nobj / 2;  // No even: whole float4s
        for (size_t i0 = (size_t)crank * blockDim.x + threadIdx.x; i0 < n4; i0 += MU * stride) {
          float4 X[MU], B[MU], M[MU];
#pragma unroll
          for (int u = 0; u < MU; ++u) {
            const size_t i = i0 + u * stride;
            const size_t j = 2 * (i < n4 ? i : 0);  // pixel 0 stands in past the end
            X[u] = ld_cg_early4(s.object + j);
            B[u] = ld_cg_early4(s.objectBuffer + j);
            M[u] = ld_cg_early4(s.objectMomentum + j);
          }
#pragma unroll
          for (int u = 0; u < MU; ++u) {
            const size_t i = i0 + u * stride;
            if (i < n4) {
              float2 X0, M0, X1, M1;
              step(make_float2(X[u].x, X[u].y), make_float2(B[u].x, B[u].y), make_float2(M[u].x, M[u].y), X0, M0);
              step(make_float2(X[u].z, X[u].w), make_float2(B[u].z, B[u].w), make_float2(M[u].z, M[u].w), X1, M1);
              const float4 Xn = make_float4(X0.x, X0.y, X1.x, X1.y), Mn = make_float4(M0.x, M0.y, M1.x, M1.y);
              __stcg(reinterpret_cast<float4*>(s.objectMomentum) + i, Mn);
              __stcg(reinterpret_cast<float4*>(s.object) + i, Xn);
              __stcg(reinterpret_cast<float4*>(s.objectBuffer) + i, Xn);
            }
          }
        }
      } else {
        for (size_t i = (size_t)crank * blockDim.x + threadIdx.x; i < nobj; i += stride) {
          float2 Xn, Mn;
          step(ld_cg(s.object + i), ld_cg(s.objectBuffer + i), ld_cg(s.objectMomentum + i), Xn, Mn);
          st_cg(s.objectMomentum + i, Mn);
          st_cg(s.object + i, Xn);
          st_cg(s.objectBuffer + i, Xn);
        }
      }
      // the probe rows: PU elements' buffer and momentum loads in flight per
      // thread before the first step
      constexpr int PU = 4;
      const int np = npsm * LN;
      for (int i0 = threadIdx.x; i0 < np; i0 += PU * (int)blockDim.x) {
        float2 B[PU], M[PU];
#pragma unroll
        for (int q = 0; q < PU; ++q) {
          const int i = i0 + q * (int)blockDim.x, ic = i < np ? i : i0;
          const size_t gi = (size_t)(ic / LN) * NP * NP + (size_t)line0 * NP + (ic - (ic / LN) * LN);
          B[q] = s.probeBuffer[gi];
          M[q] = s.probeMomentum[gi];
        }
#pragma unroll
        for (int q = 0; q < PU; ++q) {
          const int i = i0 + q * (int)blockDim.x;
          if (i < np) {
            const int p = i / LN, rem = i - (i / LN) * LN;
            const size_t gi = (size_t)p * NP * NP + (size_t)line0 * NP + rem;
            float2 Xn, Mn;
            step(sm.probe[p * pst + rem], B[q], M[q], Xn, Mn);
            s.probeMomentum[gi] = Mn;
            s.probeBuffer[gi] = Xn;
            sm.probe[p * pst + rem] = Xn;
          }
        }
      }
    }
    // qNewton's last cluster barrier (after pass C) already orders this
    // position's object writes before the next position's reads; the other
    // engines (and mqNewton's momentum step) need one here
    if (!qn || mq) {
      __syncthreads();
      cluster_sync(C);
    }
  }
  cp_async_wait_all();
  __syncthreads();
  if (mq && s.moment2 && crank == 0 && threadIdx.x == 0) {
    s.moment2[0] = vO;
    s.moment2[1] = vP;
  }

  if (psm) {
    for (int i = threadIdx.x; i < npsm * LN; i += blockDim.x) {
      const int p = i / LN, rem = i - (i / LN) * LN;
      s.probe[(size_t)p * a.nslice * NP * NP + (size_t)line0 * NP + rem] = sm.probe[i];
    }
  }
  // no CTA may exit while another can still write into its shared memory
  cluster_sync(C);
}

// ------------------------------------------------------------------ launch helpers
inline cudaLaunchConfig_t launch_config(int cluster, int grid, int threads, size_t smem, cudaStream_t st,
                                        cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

template <int E, int L, int VAR>
cudaError_t prepare_t(size_t smem) {
  auto kern = engine_kernel<E, L, VAR>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (32 * E / L > 8) e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  return e;
}

template <int E, int L, int VAR>
cudaError_t launch_t(const EngineArgs& a, int nscans, int threads, size_t smem, cudaStream_t st) {
  cudaError_t e = prepare_t<E, L, VAR>(smem);
  if (e != cudaSuccess) return e;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = launch_config(a.cluster, nscans * a.cluster, threads, smem, st, attr);
  return cudaLaunchKernelEx(&cfg, engine_kernel<E, L, VAR>, a);
}

template <int E, int L, int VAR>
cudaError_t clusters_t(int threads, size_t smem, int* out) {
  cudaError_t e = prepare_t<E, L, VAR>(smem);
  if (e != cudaSuccess) return e;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = launch_config(32 * E / L, 32 * E / L, threads, smem, 0, attr);
  return cudaOccupancyMaxActiveClusters(out, (void*)engine_kernel<E, L, VAR>, &cfg);
}

// Instantiated shapes: 8 or 16 rows per CTA, at most 16 CTAs per cluster;
// and at Np = 64 the whole patch in one CTA (a cluster of one: its barriers
// are CTA barriers and its transposes stay in its own shared memory).
#define PTYG_ENGINE_SHAPES(X) X(1, 8) X(1, 16) X(2, 8) X(2, 16) X(2, 64) X(4, 8) X(4, 16) X(8, 16)


// Launch / occupancy over the instantiated shapes for one variant; each
// translation unit instantiates one (ptyg_engine.cu: VAR_STD,
// ptyg_engine_mq.cu: VAR_MQ, ptyg_engine_poly.cu: VAR_POLY,
// ptyg_engine_mq_poly.cu: VAR_MQ_POLY).
template <int VAR>
cudaError_t engine_max_clusters_t(int Np, int cluster, int threads, size_t smem, int* out) {
  *out = 0;
  const int E = Np / 32, L = Np / cluster;
#define PTYG_CALL(e, l) \
  if (E == e && L == l) return clusters_t<e, l, VAR>(threads, smem, out);
  PTYG_ENGINE_SHAPES(PTYG_CALL)
#undef PTYG_CALL
  return cudaErrorNotSupported;
}

template <int VAR>
cudaError_t launch_engine_t(const EngineArgs& a, int nscans, int threads, size_t smem, cudaStream_t st) {
  const int E = a.Np / 32, L = a.Np / a.cluster;
#define PTYG_CALL(e, l) \
  if (E == e && L == l) return launch_t<e, l, VAR>(a, nscans, threads, smem, st);
  PTYG_ENGINE_SHAPES(PTYG_CALL)
#undef PTYG_CALL
  return cudaErrorNotSupported;
}

}  // namespace ptyg
