// Instantiations of the position-loop kernel (ptyg_engine_kernel.cuh) for
// ePIE / mPIE / qNewton at one wavelength, and the engine-independent launch
// queries.
#include "ptyg_engine_kernel.cuh"
#include "ptyg_ops.cuh"

namespace ptyg {

size_t engine_smem_bytes(int Np, int C, int nosm, int npsm, int nlambda, int engine, bool probe_in_smem,
                         bool asp_table_in_smem) {
  const int L = Np / C;
  const size_t LN = (size_t)L * Np;
  const bool qn = engine == ENG_QNEWTON || engine == ENG_MQNEWTON;
  const size_t n = smem_complex_elems(Np, L, nlambda * nosm * npsm, nlambda * nosm, nlambda * npsm, qn, probe_in_smem,
                                      asp_table_in_smem ? nlambda : 0);
  // + fr, dat (2 LN floats), slots, redD (4 x 32 doubles), redF (4 x 32
  // floats), part (4 x 16 doubles), the copy's mbarrier, alignment slack
  return n * sizeof(float2) + 2 * LN * sizeof(float) + 2 * RED_BANK * sizeof(unsigned) + 4 * 32 * sizeof(double) +
         4 * 32 * sizeof(float) + 4 * 16 * sizeof(double) + sizeof(unsigned long long) + 64;
}

bool engine_shape_supported(int Np, int cluster) {
  const int E = Np / 32, L = Np / cluster;
#define PTYG_MATCH(e, l) \
  if (E == e && L == l) return true;
  PTYG_ENGINE_SHAPES(PTYG_MATCH)
#undef PTYG_MATCH
  return false;
}

cudaError_t engine_max_clusters(int Np, int engine, int nlambda, int cluster, int threads, size_t smem, int* out) {
  // (the several-wavelength instantiation serves ePIE, mPIE and qNewton)
  if (engine == ENG_MQNEWTON)
    return nlambda > 1 ? engine_max_clusters_mq_poly(Np, cluster, threads, smem, out)
                       : engine_max_clusters_mq(Np, cluster, threads, smem, out);
  if (nlambda > 1) return engine_max_clusters_poly(Np, cluster, threads, smem, out);
  return engine_max_clusters_t<VAR_STD>(Np, cluster, threads, smem, out);
}

cudaError_t launch_engine(const EngineArgs& a, int nscans, int threads, size_t smem, cudaStream_t st) {
  if (a.engine == ENG_MQNEWTON)
    return a.nlambda > 1 ? launch_engine_mq_poly(a, nscans, threads, smem, st) : launch_engine_mq(a, nscans, threads, smem, st);
  if (a.nlambda > 1 || a.iconstraint == IC_INTERFEROMETRIC) return launch_engine_poly(a, nscans, threads, smem, st);
  // PtyLab's defaults (one object mode, Fraunhofer / Fresnel, standard
  // projection): the instantiation with those switches folded
  if (a.nosm == 1 && a.prop != PROP_ASP && a.iconstraint == IC_STANDARD && !a.denoise && !a.bgMode && !a.fmask &&
      !a.imask)
    return launch_engine_fast(a, nscans, threads, smem, st);
  return launch_engine_t<VAR_STD>(a, nscans, threads, smem, st);
}

bool engine_modes_supported(int Np, int nosm, int npsm) {
  (void)Np;
  return nosm >= 1 && nosm <= MAX_OBJECT_MODES && npsm >= 1 && npsm <= 16;
}

}  // namespace ptyg
