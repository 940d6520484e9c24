// Persistent position-loop kernel for ePIE / mPIE / qNewton (CPM and FPM) with
// the Fraunhofer, Fresnel and ASP propagators.
//
// One thread-block cluster of C CTAs reconstructs one scan; a grid of G
// clusters reconstructs G independent scans.  The cluster walks the positions
// of one iteration in the order the host drew (PtyLab/Engines/BaseEngine.py:637-665)
// and, for each position, runs the body of ePIE.py:84-105 / mPIE.py:280-332 /
// qNewton.py:69-90 as a sequence of passes separated by cluster barriers:
//
//   A  row pass     : gather object rows (coalesced), exit waves O_o*P_p for every
//                     (object mode, probe mode), [Fresnel chirp], [centring sign],
//                     forward row FFT -> work buffer; maxima for the update norms
//   B  column pass  : forward column FFT, I_est = sum_k |Psi_k|^2, FP64 partial of
//                     sum |I_meas - I_est|, Psi_k *= sqrt(I_meas/(I_est+1e-10)),
//                     inverse column FFT (BaseEngine.py:870-1012)
//   C  row pass     : inverse row FFT, [sign], [conj chirp] -> eswUpdate; DELTA;
//                     object patch and probe updates; scatter object rows
//
// ASP adds a transfer-function column pass on each side of a real-space
// projection row pass (Operators.py:155-230).  CTA c of the cluster owns rows
// [c*L, (c+1)*L) of every row pass and Fourier-layout columns [c*L, (c+1)*L) of
// every column pass (L = Np/C), so each CTA always updates the same probe rows:
// the probe stays in shared memory for the whole launch.
#include <cooperative_groups.h>

#include "ptyg_common.cuh"
#include "ptyg_engine.cuh"

namespace cg = cooperative_groups;

namespace ptyg {

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

// Max-reduce NV values over the CTA and fold them into the cluster slots with
// one atomicMax per value per CTA.  `scratch` holds 32*NV floats.
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

// Sum a double over the CTA; thread 0 receives the result.
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
  return __uint_as_float(__ldcg(slots + i));
}

// ------------------------------------------------------------------ passes
// Column pass over the CTA's Fourier-layout columns.  MODE 0: intensity
// projection (Fraunhofer/Fresnel); MODE 1: multiply by H (or conj(H)) / Np^2.
template <int E, int MK, int MODE>
PTYG_DEV double column_pass(const EngineArgs& a, const ScanDev& s, int frame, int crank, int L, int K,
                            float2* tile, const float2* tw, const LaneTw& lt, const float2* H, bool conjH) {
  constexpr int NP = 32 * E;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int sx0 = crank * L;
  const int ld = L + 1;
  // stage the column block of every mode (rows of L contiguous complex64)
  for (int idx = threadIdx.x; idx < K * NP * L; idx += blockDim.x) {
    const int k = idx / (NP * L);
    const int rem = idx - k * NP * L;
    const int y = rem / L;
    const int c = rem - y * L;
    tile[(k * NP + y) * ld + c] = ld_cg(s.work + (size_t)k * NP * NP + (size_t)y * NP + sx0 + c);
  }
  __syncthreads();
  const float inv2 = 1.f / (float)(NP * NP);
  double err = 0.0;
  for (int c = warp; c < L; c += nw) {
    const int sx = sx0 + c;
    float2 v[MK][E];
#pragma unroll
    for (int k = 0; k < MK; ++k) {
      if (k < K) {
#pragma unroll
        for (int jj = 0; jj < E; ++jj) v[k][jj] = tile[(k * NP + lane + 32 * jj) * ld + c];
        fft_fwd<E>(v[k], tw, lt, lane);
      }
    }
    if (MODE == 0) {
      const float* I = s.data + ((size_t)frame * NP + sx) * NP;
      float* de = (a.writeDetErr && s.detErr) ? s.detErr + ((size_t)frame * NP + sx) * NP : nullptr;
#pragma unroll
      for (int r = 0; r < E; ++r) {
        float ie = 0.f;
#pragma unroll
        for (int k = 0; k < MK; ++k)
          if (k < K) ie += cabs2(v[k][r]);
        ie *= inv2;
        const float im = __ldg(I + r * 32 + lane);
        const float d = fabsf(im - ie);
        err += (double)d;
        if (de) de[r * 32 + lane] = d;
        const float f = sqrtf(im / (ie + 1e-10f)) * inv2;
#pragma unroll
        for (int k = 0; k < MK; ++k)
          if (k < K) v[k][r] = cscale(v[k][r], f);
      }
    } else {
      const float2* h = H + (size_t)sx * NP;
#pragma unroll
      for (int r = 0; r < E; ++r) {
        float2 hv = __ldg(h + r * 32 + lane);
        if (conjH) hv.y = -hv.y;
        hv = cscale(hv, inv2);
#pragma unroll
        for (int k = 0; k < MK; ++k)
          if (k < K) v[k][r] = cmul(v[k][r], hv);
      }
    }
#pragma unroll
    for (int k = 0; k < MK; ++k) {
      if (k < K) {
        fft_inv<E>(v[k], tw, lt, lane);
#pragma unroll
        for (int jj = 0; jj < E; ++jj) tile[(k * NP + lane + 32 * jj) * ld + c] = v[k][jj];
      }
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < K * NP * L; idx += blockDim.x) {
    const int k = idx / (NP * L);
    const int rem = idx - k * NP * L;
    const int y = rem / L;
    const int c = rem - y * L;
    st_cg(s.work + (size_t)k * NP * NP + (size_t)y * NP + sx0 + c, tile[(k * NP + y) * ld + c]);
  }
  return err;
}

// ------------------------------------------------------------------ kernel
template <int E, int MO, int MP>
__global__ void __launch_bounds__(256, 1) engine_kernel(const EngineArgs a) {
  constexpr int NP = 32 * E;
  constexpr int MK = MO * MP;
  const int C = a.cluster;
  const int crank = (int)(blockIdx.x % (unsigned)C);
  const ScanDev s = a.scans[blockIdx.x / C];
  const int L = NP / C;
  const int line0 = crank * L;
  const unsigned lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int nosm = a.nosm, npsm = a.npsm, K = nosm * npsm, No = a.No;
  const bool centred = a.centred != 0;
  const bool fresnel = a.prop == PROP_FRESNEL;
  const bool asp = a.prop == PROP_ASP;
  const int eng = a.engine;

  extern __shared__ float4 smem_f4[];
  float2* tw = reinterpret_cast<float2*>(smem_f4);
  float2* probeS = tw + NP;                     // npsm * L * NP
  float2* tile = probeS + npsm * L * NP;         // K * NP * (L + 1)
  float2* U = tile + K * NP * (L + 1);           // qNewton: npsm * L * NP
  double* redD = reinterpret_cast<double*>(U + (eng == ENG_QNEWTON ? npsm * L * NP : 0));
  float* redF = reinterpret_cast<float*>(redD + 32);

  for (int i = threadIdx.x; i < NP; i += blockDim.x) tw[i] = a.twiddle[i];
  for (int i = threadIdx.x; i < npsm * L * NP; i += blockDim.x) {
    const int p = i / (L * NP);
    const int rem = i - p * L * NP;
    probeS[i] = s.probe[(size_t)p * a.nslice * NP * NP + (size_t)line0 * NP + rem];
  }
  if (crank == 0 && threadIdx.x < 2 * RED_BANK) s.red[threadIdx.x] = 0u;
  __syncthreads();
  cluster_sync(C);
  const LaneTw lt = lane_twiddles<E>(tw, lane);

  for (int it = 0; it < a.count; ++it) {
    const int frame = s.order[a.start + it];
    const int row0 = s.positions[2 * frame];
    const int col0 = s.positions[2 * frame + 1];
    if (frame < 0 || frame >= a.numFrames || row0 < 0 || col0 < 0 || row0 > No - NP || col0 > No - NP) {
      if (crank == 0 && threadIdx.x == 0) atomicCAS(s.status, 0, 2);
      continue;  // uniform across the cluster
    }
    unsigned* red = s.red + (it & 1) * RED_BANK;
    unsigned* redNext = s.red + ((it & 1) ^ 1) * RED_BANK;

    // ---------------- A: exit waves and forward row FFT
    {
      float mx[3] = {0.f, 0.f, 0.f};  // max of sum_p|P|^2, sum_o|O|^2, sum_p|P|
      for (int l = warp; l < L; l += nw) {
        const int y = line0 + l;
        const float sg = (centred && !asp && ((y + lane) & 1)) ? -1.f : 1.f;
        float2 O[MO][E];
#pragma unroll
        for (int o = 0; o < MO; ++o) {
          if (o < nosm) {
            const float2* src = s.object + (size_t)o * No * No + (size_t)(row0 + y) * No + col0 + lane;
#pragma unroll
            for (int jj = 0; jj < E; ++jj) O[o][jj] = ld_cg(src + 32 * jj);
          }
        }
#pragma unroll
        for (int jj = 0; jj < E; ++jj) {
          float so2 = 0.f;
#pragma unroll
          for (int o = 0; o < MO; ++o)
            if (o < nosm) so2 += cabs2(O[o][jj]);
          mx[1] = fmaxf(mx[1], so2);
        }
        float sp2[E], sp1[E];
#pragma unroll
        for (int jj = 0; jj < E; ++jj) sp2[jj] = sp1[jj] = 0.f;
#pragma unroll
        for (int p = 0; p < MP; ++p) {
          if (p < npsm) {
            float2 P[E];
#pragma unroll
            for (int jj = 0; jj < E; ++jj) {
              P[jj] = probeS[(p * L + l) * NP + lane + 32 * jj];
              const float q = cabs2(P[jj]);
              sp2[jj] += q;
              sp1[jj] += sqrtf(q);
            }
#pragma unroll
            for (int o = 0; o < MO; ++o) {
              if (o < nosm) {
                float2 v[E];
#pragma unroll
                for (int jj = 0; jj < E; ++jj) {
                  float2 e = cmul(O[o][jj], P[jj]);
                  if (fresnel) e = cmul(e, __ldg(a.fresnelQ + y * NP + lane + 32 * jj));
                  v[jj] = cscale(e, sg);
                }
                fft_fwd<E>(v, tw, lt, lane);
                float2* dst = s.work + (size_t)(o * npsm + p) * NP * NP + (size_t)y * NP + lane;
#pragma unroll
                for (int r = 0; r < E; ++r) st_cg(dst + 32 * r, v[r]);
              }
            }
          }
        }
#pragma unroll
        for (int jj = 0; jj < E; ++jj) {
          mx[0] = fmaxf(mx[0], sp2[jj]);
          mx[2] = fmaxf(mx[2], sp1[jj]);
        }
      }
      const int idx[3] = {RED_PMAX2, RED_OMAX2, RED_PMAX1};
      block_max_to_slots<3>(mx, redF, red, idx);
    }
    cluster_sync(C);

    double err = 0.0;
    if (!asp) {
      // ---------------- B: Fourier-plane intensity projection
      err = column_pass<E, MK, 0>(a, s, frame, crank, L, K, tile, tw, lt, nullptr, false);
    } else {
      // ---------------- ASP: B (xH), C (real-space projection), D (x conj H)
      column_pass<E, MK, 1>(a, s, frame, crank, L, K, tile, tw, lt, a.aspH, false);
      cluster_sync(C);
      for (int l = warp; l < L; l += nw) {
        const int y = line0 + l;
        float2 v[MK][E];
#pragma unroll
        for (int k = 0; k < MK; ++k) {
          if (k < K) {
            const float2* src = s.work + (size_t)k * NP * NP + (size_t)y * NP + lane;
#pragma unroll
            for (int r = 0; r < E; ++r) v[k][r] = ld_cg(src + 32 * r);
            fft_inv<E>(v[k], tw, lt, lane);
          }
        }
        const float* I = s.data + ((size_t)frame * NP + y) * NP + lane;
        float* de = (a.writeDetErr && s.detErr) ? s.detErr + ((size_t)frame * NP + y) * NP + lane : nullptr;
#pragma unroll
        for (int jj = 0; jj < E; ++jj) {
          float ie = 0.f;
#pragma unroll
          for (int k = 0; k < MK; ++k)
            if (k < K) ie += cabs2(v[k][jj]);
          const float im = __ldg(I + 32 * jj);
          const float d = fabsf(im - ie);
          err += (double)d;
          if (de) de[32 * jj] = d;
          const float f = sqrtf(im / (ie + 1e-10f));
#pragma unroll
          for (int k = 0; k < MK; ++k)
            if (k < K) v[k][jj] = cscale(v[k][jj], f);
        }
#pragma unroll
        for (int k = 0; k < MK; ++k) {
          if (k < K) {
            fft_fwd<E>(v[k], tw, lt, lane);
            float2* dst = s.work + (size_t)k * NP * NP + (size_t)y * NP + lane;
#pragma unroll
            for (int r = 0; r < E; ++r) st_cg(dst + 32 * r, v[k][r]);
          }
        }
      }
      __syncthreads();
      cluster_sync(C);
      column_pass<E, MK, 1>(a, s, frame, crank, L, K, tile, tw, lt, a.aspH, true);
    }
    {
      const double t = block_sum(err, redD);
      if (threadIdx.x == 0) s.errPart[(size_t)frame * C + crank] = t;
    }
    if (crank == 0 && threadIdx.x < RED_BANK) redNext[threadIdx.x] = 0u;
    cluster_sync(C);

    // ---------------- C: inverse row FFT, DELTA, object and probe updates
    // Streams over probe modes: for each p the lines of all object modes are
    // inverse transformed, DELTA_{o,p} formed, the object numerator accumulated
    // and probe mode p updated, so only one probe mode is live at a time.
    {
      const float pmax2 = slot_value(red, RED_PMAX2);
      const float omax2 = slot_value(red, RED_OMAX2);
      const float pmax1 = slot_value(red, RED_PMAX1);
      const float invPmax2 = 1.f / pmax2, invOmax2 = 1.f / omax2, invPmax1 = 1.f / pmax1;
      const float stepP = a.betaP * a.weightP;
      for (int l = warp; l < L; l += nw) {
        const int y = line0 + l;
        const float sg = (centred && !asp && ((y + lane) & 1)) ? -1.f : 1.f;
        float2 O[MO][E], accO[MO][E];
        float gP[MO][E];
#pragma unroll
        for (int o = 0; o < MO; ++o) {
          if (o < nosm) {
            const float2* src = s.object + (size_t)o * No * No + (size_t)(row0 + y) * No + col0 + lane;
#pragma unroll
            for (int jj = 0; jj < E; ++jj) {
              O[o][jj] = ld_cg(src + 32 * jj);
              accO[o][jj] = make_float2(0.f, 0.f);
              const float q = cabs2(O[o][jj]);
              if (eng == ENG_EPIE)
                gP[o][jj] = invOmax2;                                    // ePIE.py:154-156
              else if (eng == ENG_MPIE)
                gP[o][jj] = 1.f / (a.alphaP * omax2 + (1.f - a.alphaP) * q);  // mPIE.py:262-264
              else
                gP[o][jj] = sqrtf(q) / (q + a.regP);  // qNewton.py:131-136 (1/Omax applied later)
            }
          }
        }
#pragma unroll
        for (int p = 0; p < MP; ++p) {
          if (p < npsm) {
            float2 D[MO][E];
#pragma unroll
            for (int o = 0; o < MO; ++o) {
              if (o < nosm) {
                const float2* src = s.work + (size_t)(o * npsm + p) * NP * NP + (size_t)y * NP + lane;
#pragma unroll
                for (int r = 0; r < E; ++r) D[o][r] = ld_cg(src + 32 * r);
                fft_inv<E>(D[o], tw, lt, lane);
              }
            }
            float2* prow = (eng == ENG_QNEWTON ? U : probeS) + (p * L + l) * NP + lane;
#pragma unroll
            for (int jj = 0; jj < E; ++jj) {
              const float2 P = probeS[(p * L + l) * NP + lane + 32 * jj];
              const float q = cabs2(P);
              float gO;
              if (eng == ENG_EPIE) {
                gO = invPmax2;  // ePIE.py:138-140
              } else if (eng == ENG_MPIE) {
                gO = 1.f / (a.alphaO * pmax2 + (1.f - a.alphaO) * q);  // mPIE.py:246-248
                if (a.fpm) gO *= sqrtf(q) * invPmax2;                    // mPIE.py:237-243
              } else {
                gO = sqrtf(q) * invPmax1 / (q + a.regO);  // qNewton.py:113-119
              }
              float2 accP = make_float2(0.f, 0.f);
#pragma unroll
              for (int o = 0; o < MO; ++o) {
                if (o < nosm) {
                  float2 u = cscale(D[o][jj], sg);
                  if (fresnel) u = cmulc(__ldg(a.fresnelQ + y * NP + lane + 32 * jj), u);
                  const float2 d = csub(u, cmul(O[o][jj], P));  // DELTA = eswUpdate - esw
                  accO[o][jj] = cadd(accO[o][jj], cscale(cmulc(P, d), gO));
                  accP = cadd(accP, cscale(cmulc(O[o][jj], d), gP[o][jj]));
                }
              }
              // qNewton keeps the numerator until the whole-object maximum is known
              prow[32 * jj] = (eng == ENG_QNEWTON) ? accP : cadd(P, cscale(accP, stepP));
            }
          }
        }
#pragma unroll
        for (int o = 0; o < MO; ++o) {
          if (o < nosm) {
            float2* dst = s.object + (size_t)o * No * No + (size_t)(row0 + y) * No + col0 + lane;
#pragma unroll
            for (int jj = 0; jj < E; ++jj) st_cg(dst + 32 * jj, cadd(O[o][jj], cscale(accO[o][jj], a.betaO)));
          }
        }
      }
    }

    if (eng == ENG_QNEWTON) {
      // whole-object max of sum_o |O_o| after the object update (qNewton.py:130)
      cluster_sync(C);
      float m[1] = {0.f};
      const size_t n2 = (size_t)No * No;
      for (size_t i = (size_t)crank * blockDim.x + threadIdx.x; i < n2; i += (size_t)C * blockDim.x) {
        float sum = 0.f;
        for (int o = 0; o < nosm; ++o) sum += cabs(ld_cg(s.object + o * n2 + i));
        m[0] = fmaxf(m[0], sum);
      }
      const int idx[1] = {RED_OMAXW};
      block_max_to_slots<1>(m, redF, red, idx);
      cluster_sync(C);
      const float scale = a.betaP / slot_value(red, RED_OMAXW);
      for (int i = threadIdx.x; i < npsm * L * NP; i += blockDim.x)
        probeS[i] = cadd(probeS[i], cscale(U[i], scale));
    }

    if (eng == ENG_MPIE && s.momentum && s.momentum[a.start + it]) {
      // momentum step on the whole object and probe (mPIE.py:196-224), FP64 arithmetic
      cluster_sync(C);
      const double eta = a.frictionM, nu = a.feedbackM;
      const size_t nobj = (size_t)nosm * No * No;
      for (size_t i = (size_t)crank * blockDim.x + threadIdx.x; i < nobj; i += (size_t)C * blockDim.x) {
        const float2 X = ld_cg(s.object + i), B = ld_cg(s.objectBuffer + i), M = ld_cg(s.objectMomentum + i);
        const double mx = ((double)B.x - X.x) + eta * M.x, my = ((double)B.y - X.y) + eta * M.y;
        const float2 Mn = make_float2((float)mx, (float)my);
        const float2 Xn = make_float2((float)(X.x - nu * (double)Mn.x), (float)(X.y - nu * (double)Mn.y));
        st_cg(s.objectMomentum + i, Mn);
        st_cg(s.object + i, Xn);
        st_cg(s.objectBuffer + i, Xn);
      }
      for (int i = threadIdx.x; i < npsm * L * NP; i += blockDim.x) {
        const int p = i / (L * NP);
        const int rem = i - p * L * NP;
        const size_t gi = (size_t)p * NP * NP + (size_t)line0 * NP + rem;
        const float2 X = probeS[i], B = s.probeBuffer[gi], M = s.probeMomentum[gi];
        const double mx = ((double)B.x - X.x) + eta * M.x, my = ((double)B.y - X.y) + eta * M.y;
        const float2 Mn = make_float2((float)mx, (float)my);
        const float2 Xn = make_float2((float)(X.x - nu * (double)Mn.x), (float)(X.y - nu * (double)Mn.y));
        s.probeMomentum[gi] = Mn;
        s.probeBuffer[gi] = Xn;
        probeS[i] = Xn;
      }
    }
    __syncthreads();
    cluster_sync(C);
  }

  // write the probe rows back
  for (int i = threadIdx.x; i < npsm * L * NP; i += blockDim.x) {
    const int p = i / (L * NP);
    const int rem = i - p * L * NP;
    s.probe[(size_t)p * a.nslice * NP * NP + (size_t)line0 * NP + rem] = probeS[i];
  }
}

// ------------------------------------------------------------------ launcher
size_t engine_smem_bytes(int Np, int C, int nosm, int npsm, int engine) {
  const int L = Np / C;
  const int K = nosm * npsm;
  size_t n = (size_t)Np + (size_t)npsm * L * Np + (size_t)K * Np * (L + 1);
  if (engine == ENG_QNEWTON) n += (size_t)npsm * L * Np;
  return n * sizeof(float2) + 32 * sizeof(double) + 32 * 4 * sizeof(float) + 64;
}

template <int E, int MO, int MP>
static cudaError_t launch_t(const EngineArgs& a, int nscans, int threads, size_t smem, cudaStream_t st) {
  auto kern = engine_kernel<E, MO, MP>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (a.cluster > 8) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nscans * a.cluster);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = a.cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, a);
}

template <int E>
static cudaError_t launch_e(const EngineArgs& a, int nscans, int threads, size_t smem, cudaStream_t st) {
  if (a.nosm == 1 && a.npsm == 1) return launch_t<E, 1, 1>(a, nscans, threads, smem, st);
  if (a.nosm == 1 && a.npsm <= 2) return launch_t<E, 1, 2>(a, nscans, threads, smem, st);
  if (a.nosm == 1 && a.npsm <= 4) return launch_t<E, 1, 4>(a, nscans, threads, smem, st);
  if constexpr (E <= 4) {
    if (a.nosm <= 2 && a.npsm <= 4) return launch_t<E, 2, 4>(a, nscans, threads, smem, st);
  }
  return cudaErrorNotSupported;
}

template <int E, int MO, int MP>
static cudaError_t clusters_t(int cluster, int threads, size_t smem, int* out) {
  auto kern = engine_kernel<E, MO, MP>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (cluster > 8) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cluster);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaOccupancyMaxActiveClusters(out, (void*)kern, &cfg);
}

template <int E>
static cudaError_t clusters_e(int nosm, int npsm, int cluster, int threads, size_t smem, int* out) {
  if (nosm == 1 && npsm == 1) return clusters_t<E, 1, 1>(cluster, threads, smem, out);
  if (nosm == 1 && npsm <= 2) return clusters_t<E, 1, 2>(cluster, threads, smem, out);
  if (nosm == 1 && npsm <= 4) return clusters_t<E, 1, 4>(cluster, threads, smem, out);
  if constexpr (E <= 4) {
    if (nosm <= 2 && npsm <= 4) return clusters_t<E, 2, 4>(cluster, threads, smem, out);
  }
  return cudaErrorNotSupported;
}

// How many clusters of this shape can be resident at once (0 = cannot launch).
cudaError_t engine_max_clusters(int Np, int nosm, int npsm, int cluster, int threads, size_t smem, int* out) {
  *out = 0;
  switch (Np) {
    case 32: return clusters_e<1>(nosm, npsm, cluster, threads, smem, out);
    case 64: return clusters_e<2>(nosm, npsm, cluster, threads, smem, out);
    case 128: return clusters_e<4>(nosm, npsm, cluster, threads, smem, out);
    case 256: return clusters_e<8>(nosm, npsm, cluster, threads, smem, out);
    default: return cudaErrorNotSupported;
  }
}

// Returns cudaErrorNotSupported for mode counts without an instantiation.
cudaError_t launch_engine(const EngineArgs& a, int nscans, int threads, size_t smem, cudaStream_t st) {
  switch (a.Np) {
    case 32: return launch_e<1>(a, nscans, threads, smem, st);
    case 64: return launch_e<2>(a, nscans, threads, smem, st);
    case 128: return launch_e<4>(a, nscans, threads, smem, st);
    case 256: return launch_e<8>(a, nscans, threads, smem, st);
    default: return cudaErrorNotSupported;
  }
}

bool engine_modes_supported(int Np, int nosm, int npsm) {
  if (nosm == 1 && npsm <= 4) return true;
  return nosm <= 2 && npsm <= 4 && Np <= 128;
}

}  // namespace ptyg
