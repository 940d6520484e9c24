// Persistent position-loop kernel for e3PIE, multislice ptychography
// (PtyLab/Engines/e3PIE.py:71-225).
//
// Same cluster decomposition as ptyg_engine.cu (CTA c owns rows and
// Fourier-layout columns [c*L, (c+1)*L); DSMEM transposes; cp.async intensity
// prefetch).  Per position, with S slices and npsm probe modes (nosm = 1):
//
//   forward   esw_0 = O_0 * P_0;  for s = 1..S-1:
//             P_s = ifft2(fft2(esw_{s-1}) * H),  esw_s = P_s * O_s    (e3PIE.py:99-115)
//   detector  intensity projection of the last slice's exit waves     (e3PIE.py:118),
//             with every switch of the engines' projection but the
//             interferometric constraint (project_intensities)
//   backward  DELTA = eswUpdate - esw_{S-1}; for s = S-1..1:
//             O_s += betaObject * sum_p conj(P_s) DELTA / max sum_p |P_s|^2
//             P_s += 0.9 * conj(O_s) DELTA / max |O_s|^2
//             DELTA = ifft2(fft2(P_s) * conj(H)) - esw_{s-1}          (e3PIE.py:125-160)
//             then slice 0 with betaProbe                              (e3PIE.py:162-173)
//
// The object slices, the probe slices and the forward exit waves stay in
// global memory (L2): at Np = 256 with four slices they would not fit in a
// CTA's shared memory.  Only the last slice goes to the detector, which is all
// the reference's update uses (it propagates every slice and keeps [-1]).
#include "ptyg_engine_dev.cuh"

namespace ptyg {

constexpr int MAX_SLICES = 6;

template <int E, int L>
__global__ void __launch_bounds__(512, 1) e3pie_kernel(const EngineArgs a) {
  constexpr int NP = 32 * E;
  constexpr int C = NP / L;
  constexpr int LN = L * NP;
  const int crank = (int)(blockIdx.x % (unsigned)C);
  const ScanDev s = a.scans[blockIdx.x / C];
  const int line0 = crank * L, sx0 = crank * L;
  const unsigned lane = threadIdx.x & 31;
  const int npsm = a.npsm, K = npsm, S = a.nslice, No = a.No;
  const bool centred = a.centred != 0;
  const bool fresnel = a.prop == PROP_FRESNEL;
  const bool asp = a.prop == PROP_ASP;
  const size_t No2 = (size_t)No * No;
  const size_t NP2 = (size_t)NP * NP;
  const int blk0 = asp ? line0 : sx0;

  extern __shared__ float4 smem_f4[];
  float2* tile = reinterpret_cast<float2*>(smem_f4);  // K * NP * L (swizzled, tix)
  float2* rows = tile + K * NP * L;                   // K * LN
  float* fr = reinterpret_cast<float*>(rows + K * LN);
  float* dat = fr + LN;  // LN: this position's intensities, then (once the projection has read
                         // them) the next position's, in flight
  unsigned* slots = reinterpret_cast<unsigned*>(dat + LN);
  double* redD = reinterpret_cast<double*>(slots + 2 * RED_BANK);  // 64
  double* part = redD + 64;                                          // 64: the projection's cluster sums
  float* redF = reinterpret_cast<float*>(part + 64);
  unsigned* slots0 = dsmem(slots, 0);

  if (threadIdx.x < 2 * RED_BANK) slots[threadIdx.x] = 0u;
  prefetch_data<NP, L, false>(a, s, dat, 0, blk0);
  WarpFFT<E> F;  // the column transforms (rows: row_tasks)
  F.init(a.twiddle, lane);
  __syncthreads();
  cluster_sync(C);

  const float inv2 = 1.f / (float)NP2;

  for (int it = 0; it < a.count; ++it) {
    const int frame = s.order[a.start + it];
    const int row0 = (frame >= 0 && frame < a.numFrames) ? s.positions[2 * frame] : -1;
    const int col0 = (frame >= 0 && frame < a.numFrames) ? s.positions[2 * frame + 1] : -1;
    if (row0 < 0 || col0 < 0 || row0 > No - NP || col0 > No - NP) {
      if (crank == 0 && threadIdx.x == 0) atomicCAS(s.status, 0, 2);
      cp_async_wait_all();  // the skipped position's block, then the next one's
      __syncthreads();
      prefetch_data<NP, L, false>(a, s, dat, it + 1, blk0);
      continue;  // uniform across the cluster
    }
    unsigned* red = slots0 + (it & 1) * RED_BANK;
    const float* datc = dat;
    const size_t orow = (size_t)(row0 + line0) * No + col0;
    // this CTA's rows of object slice sl, probe mode p of slice sl, exit wave (sl, p)
    auto Ob = [&](int sl) { return s.object + sl * No2 + orow; };
    auto Pb = [&](int p, int sl) { return s.probe + ((size_t)p * S + sl) * NP2 + (size_t)line0 * NP; };
    auto Wb = [&](int sl, int p) { return s.eswStore + ((size_t)sl * npsm + p) * NP2 + (size_t)line0 * NP; };
    // the detector transform's input factor at (row y, col x): centring sign, Fresnel chirp
    auto detector_in = [&](float2 e, int y, int x) {
      if (asp) return e;
      if (fresnel) e = cmul(e, __ldg(a.fresnelQ + y * NP + x));
      return (centred && ((y + x) & 1)) ? cscale(e, -1.f) : e;
    };

    // ---------------- slice 0 exit waves into the row buffers (and the
    // exit-wave store), then the forward row FFT in place.  The maxima the
    // backward pass divides by, sum_p |P_s|^2 and |O_s|^2 of the pre-update
    // slices, are taken where the forward pass reads each slice anyway (slice
    // 0 here, slice s in its exit-wave loop).  The pixel loops of this
    // kernel keep U pixels' global loads in flight per thread before the
    // first is used: the slices live in L2 or DRAM.
    constexpr int U = 4;
    float mp0 = 0.f, mo0 = 0.f;
    for (int i0 = threadIdx.x; i0 < LN; i0 += U * (int)blockDim.x) {
      float2 Ov[U];
      float sp[U];
#pragma unroll
      for (int q = 0; q < U; ++q) {
        const int i = i0 + q * (int)blockDim.x, ic = i < LN ? i : i0;
        Ov[q] = ld_cg(Ob(0) + (size_t)(ic / NP) * No + ic % NP);
        sp[q] = 0.f;
      }
      for (int p = 0; p < npsm; ++p) {
        float2 Pv[U];
#pragma unroll
        for (int q = 0; q < U; ++q) {
          const int i = i0 + q * (int)blockDim.x;
          Pv[q] = Pb(p, 0)[i < LN ? i : i0];
        }
#pragma unroll
        for (int q = 0; q < U; ++q) {
          const int i = i0 + q * (int)blockDim.x;
          if (i < LN) {
            sp[q] += cabs2(Pv[q]);
            const float2 e = cmul(Ov[q], Pv[q]);
            Wb(0, p)[i] = e;
            rows[p * LN + i] = (S == 1) ? detector_in(e, line0 + i / NP, i % NP) : e;
          }
        }
      }
#pragma unroll
      for (int q = 0; q < U; ++q) {
        if (i0 + q * (int)blockDim.x < LN) {
          mp0 = fmaxf(mp0, sp[q]);
          mo0 = fmaxf(mo0, cabs2(Ov[q]));
        }
      }
    }
    {
      float m[2] = {mp0, mo0};
      const int idx[2] = {RED_SLICE_P, RED_SLICE_O};
      block_max_to_slots<2>(m, redF, red, idx);  // (its CTA barrier also orders the row buffers)
    }
    // every row-buffer line is a transform's own buffer (in place) or free
    auto row = [&](int t, int i) -> float2& { return rows[t * NP + i]; };
    auto pairs = [&](int t) { return reinterpret_cast<float4*>(rows + t * NP); };
    auto scatter = [&](int t, int lo, int hi, float2 v) { scatter_row<NP, L>(tile, t / L, line0 + t % L, lo, hi, v); };
    row_tasks<E, false>(
        a.twiddle, K * L, [&](int t, int lo, int hi) { return row(t, lo + hi); }, scatter, pairs);
    cp_async_wait_all();  // this position's intensities (the one group in flight)
    cluster_sync(C);

    // ---------------- forward through the slices
    for (int sl = 1; sl < S; ++sl) {
      column_filter<E, L>(tile, rows, F, a.sliceH, (size_t)NP * NP, false, false, crank, K, K);
      cluster_sync(C);
      // P_s rows (natural order) into the row buffer and the probe's slice sl
      row_tasks<E, true>(
          a.twiddle, K * L, [&](int t, int lo, int hi) { return row(t, rsw<L>(t, lo) + hi); },
          [&](int t, int lo, int hi, float2 v) {
            row(t, lo + hi) = v;
            Pb(t / L, sl)[(t % L) * NP + lo + hi] = v;
          },
          pairs);
      __syncthreads();
      {
        float m[2] = {0.f, 0.f};
        const bool last = sl == S - 1;
        for (int i0 = threadIdx.x; i0 < LN; i0 += U * (int)blockDim.x) {
          float2 Ov[U];
#pragma unroll
          for (int q = 0; q < U; ++q) {
            const int i = i0 + q * (int)blockDim.x, ic = i < LN ? i : i0;
            Ov[q] = ld_cg(Ob(sl) + (size_t)(ic / NP) * No + ic % NP);
          }
#pragma unroll
          for (int q = 0; q < U; ++q) {
            const int i = i0 + q * (int)blockDim.x;
            if (i < LN) {
              const int l = i / NP, x = i % NP;
              const float2 O = Ov[q];
              m[1] = fmaxf(m[1], cabs2(O));
              float sp = 0.f;
              for (int p = 0; p < npsm; ++p) {
                const float2 P = rows[p * LN + i];
                sp += cabs2(P);
                const float2 e = cmul(P, O);
                Wb(sl, p)[i] = e;
                rows[p * LN + i] = last ? detector_in(e, line0 + l, x) : e;
              }
              m[0] = fmaxf(m[0], sp);
            }
          }
        }
        const int idx[2] = {RED_SLICE_P + sl, RED_SLICE_O + sl};
        block_max_to_slots<2>(m, redF, red, idx);
      }
      __syncthreads();
      row_tasks<E, false>(
          a.twiddle, K * L, [&](int t, int lo, int hi) { return row(t, lo + hi); }, scatter, pairs);
      cluster_sync(C);
    }

    // ---------------- detector intensity projection (BaseEngine.py:870-1012)
    double err = 0.0;
    if (!asp) {
      auto col = [&](int t, int i) -> float2& { return tile[tix<L>((t / L) * NP + i, t % L)]; };
      fft_tasks<E, false>(
          F, K * L, [&](int t, int lo, int hi) { return col(t, lo + hi); },
          [&](int t, int lo, int hi, float2 v) { col(t, lo + hi) = v; });
      __syncthreads();
      err = project_intensities<NP, L, false, false, false>(
          a, s, frame, blk0, crank, ProjectionIO{fr, datc, part, redD},
          [&](int i) {
            const int c = i / NP, sy = i % NP;
            float ie = 0.f;
            for (int k = 0; k < K; ++k) ie += cabs2(tile[tix<L>(k * NP + sy, c)]);
            return ie * inv2;
          },
          inv2);
      __syncthreads();
      fft_tasks<E, true>(
          F, K * L, [&](int t, int lo, int hi) { return cscale(col(t, lo + hi), fr[(t % L) * NP + lo + hi]); },
          [&](int t, int lo, int hi, float2 v) { col(t, lo + hi) = v; });
      __syncthreads();
      flush_columns<NP, L>(tile, rows, K, sx0);
    } else {
      column_filter<E, L>(tile, rows, F, a.aspH, (size_t)NP * NP, false, false, crank, K, K);
      cluster_sync(C);
      row_tasks<E, true>(
          a.twiddle, K * L, [&](int t, int lo, int hi) { return row(t, rsw<L>(t, lo) + hi); },
          [&](int t, int lo, int hi, float2 v) { row(t, lo + hi) = v; }, pairs);
      __syncthreads();
      err = project_intensities<NP, L, false, false, false>(
          a, s, frame, blk0, crank, ProjectionIO{fr, datc, part, redD},
          [&](int i) {
            float ie = 0.f;
            for (int k = 0; k < K; ++k) ie += cabs2(rows[k * LN + i]);
            return ie;
          },
          1.f);
      __syncthreads();
      row_tasks<E, false>(
          a.twiddle, K * L, [&](int t, int lo, int hi) { return cscale(row(t, lo + hi), fr[(t % L) * NP + lo + hi]); },
          scatter, pairs);
      cluster_sync(C);
      column_filter<E, L>(tile, rows, F, a.aspH, (size_t)NP * NP, false, true, crank, K, K);
    }
    // every read of this position's intensities is behind a CTA barrier by
    // now: fetch the next position's while the backward pass runs
    prefetch_data<NP, L, false>(a, s, dat, it + 1, blk0);
    {
      const double t = block_sum(err, redD);
      if (threadIdx.x == 0) s.errPart[(size_t)frame * C + crank] = t;
    }
    if (crank == 0 && threadIdx.x < RED_BANK) slots[((it & 1) ^ 1) * RED_BANK + threadIdx.x] = 0u;
    cluster_sync(C);

    // ---------------- backward through the slices
    for (int sl = S - 1; sl >= 0; --sl) {
      // DELTA into the row buffer (natural order): the detector's back-propagated
      // last slice minus esw_{S-1}, or the back-propagated P_{sl+1} minus esw_sl
      const bool fromDetector = sl == S - 1;
      row_tasks<E, true>(
          a.twiddle, K * L, [&](int t, int lo, int hi) { return row(t, rsw<L>(t, lo) + hi); },
          [&](int t, int lo, int hi, float2 v) {
            const int p = t / L, l = t % L;
            const int y = line0 + l, x = lo + hi;
            float2 u = v;
            if (fromDetector && !asp) {
              if (centred && ((y + x) & 1)) u = cscale(u, -1.f);
              if (fresnel) u = cmulc(__ldg(a.fresnelQ + y * NP + x), u);
            }
            row(t, x) = csub(u, Wb(sl, p)[l * NP + x]);
          },
          pairs);
      __syncthreads();
      // O_sl and P_sl steps (e3PIE.py:192-225) with the pre-update slices
      {
        const float invP = 1.f / slot_value(red, RED_SLICE_P + sl);
        const float invO = 1.f / slot_value(red, RED_SLICE_O + sl);
        const float stepP = (sl == 0) ? a.betaP : a.bethSlice;
        for (int i0 = threadIdx.x; i0 < LN; i0 += U * (int)blockDim.x) {
          float2 Ov[U], acc[U];
#pragma unroll
          for (int q = 0; q < U; ++q) {
            const int i = i0 + q * (int)blockDim.x, ic = i < LN ? i : i0;
            Ov[q] = ld_cg(Ob(sl) + (size_t)(ic / NP) * No + ic % NP);
            acc[q] = make_float2(0.f, 0.f);
          }
          for (int p = 0; p < npsm; ++p) {
            float2 Pv[U];
#pragma unroll
            for (int q = 0; q < U; ++q) {
              const int i = i0 + q * (int)blockDim.x;
              Pv[q] = Pb(p, sl)[i < LN ? i : i0];
            }
#pragma unroll
            for (int q = 0; q < U; ++q) {
              const int i = i0 + q * (int)blockDim.x;
              if (i < LN) {
                const float2 d = rows[p * LN + i];
                acc[q] = cadd(acc[q], cmulc(Pv[q], d));
                const float2 Pn = cadd(Pv[q], cscale(cmulc(Ov[q], d), stepP * invO));
                Pb(p, sl)[i] = Pn;
                rows[p * LN + i] = Pn;
              }
            }
          }
#pragma unroll
          for (int q = 0; q < U; ++q) {
            const int i = i0 + q * (int)blockDim.x;
            if (i < LN) st_cg(Ob(sl) + (size_t)(i / NP) * No + i % NP, cadd(Ov[q], cscale(acc[q], a.betaO * invP)));
          }
        }
      }
      if (sl > 0) {
        // back-propagate the updated P_sl by conj(H)
        __syncthreads();
        row_tasks<E, false>(
            a.twiddle, K * L, [&](int t, int lo, int hi) { return row(t, lo + hi); }, scatter, pairs);
        cluster_sync(C);
        column_filter<E, L>(tile, rows, F, a.sliceH, (size_t)NP * NP, false, true, crank, K, K);
        cluster_sync(C);
      }
    }
    __syncthreads();
    cluster_sync(C);
  }
  cp_async_wait_all();
  __syncthreads();
  cluster_sync(C);
}

// ------------------------------------------------------------------ launcher
size_t e3pie_smem_bytes(int Np, int C, int npsm) {
  const int L = Np / C;
  const size_t LN = (size_t)L * Np;
  const size_t n = (size_t)npsm * Np * L + (size_t)npsm * LN;
  // redD and the projection's cluster-sum partials: 64 doubles each; redF
  // holds 32 floats per reduced value: MAX_SLICES + 1 of them
  return n * sizeof(float2) + 2 * LN * sizeof(float) + 2 * RED_BANK * sizeof(unsigned) + 128 * sizeof(double) +
         8 * 32 * sizeof(float) + 64;
}

static cudaLaunchConfig_t e3_config(int cluster, int grid, int threads, size_t smem, cudaStream_t st,
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

template <int E, int L>
static cudaError_t e3_prepare(size_t smem) {
  auto kern = e3pie_kernel<E, L>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (32 * E / L > 8) e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  return e;
}

#define PTYG_E3PIE_SHAPES(X) X(1, 8) X(1, 16) X(2, 8) X(2, 16) X(4, 8) X(4, 16) X(8, 16)

cudaError_t e3pie_max_clusters(int Np, int cluster, int threads, size_t smem, int* out) {
  *out = 0;
  const int E = Np / 32, L = Np / cluster;
#define PTYG_CALL(e, l)                                                     \
  if (E == e && L == l) {                                                   \
    cudaError_t err = e3_prepare<e, l>(smem);                               \
    if (err != cudaSuccess) return err;                                     \
    cudaLaunchAttribute attr[1];                                            \
    cudaLaunchConfig_t cfg = e3_config(32 * e / l, 32 * e / l, threads, smem, 0, attr); \
    return cudaOccupancyMaxActiveClusters(out, (void*)e3pie_kernel<e, l>, &cfg); \
  }
  PTYG_E3PIE_SHAPES(PTYG_CALL)
#undef PTYG_CALL
  return cudaErrorNotSupported;
}

cudaError_t launch_e3pie(const EngineArgs& a, int nscans, int threads, size_t smem, cudaStream_t st) {
  const int E = a.Np / 32, L = a.Np / a.cluster;
#define PTYG_CALL(e, l)                                                                   \
  if (E == e && L == l) {                                                                 \
    cudaError_t err = e3_prepare<e, l>(smem);                                             \
    if (err != cudaSuccess) return err;                                                   \
    cudaLaunchAttribute attr[1];                                                          \
    cudaLaunchConfig_t cfg = e3_config(a.cluster, nscans * a.cluster, threads, smem, st, attr); \
    return cudaLaunchKernelEx(&cfg, e3pie_kernel<e, l>, a);                              \
  }
  PTYG_E3PIE_SHAPES(PTYG_CALL)
#undef PTYG_CALL
  return cudaErrorNotSupported;
}

}  // namespace ptyg
