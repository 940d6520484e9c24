// The several-wavelength ePIE instantiations of the position-loop kernel
// (ptyg_engine_kernel.cuh): object and probe modes per wavelength, the
// updates summed over the wavelengths (ePIE.py:128-160).
#include "ptyg_engine_kernel.cuh"
#include "ptyg_ops.cuh"

namespace ptyg {

cudaError_t engine_max_clusters_poly(int Np, int cluster, int threads, size_t smem, int* out) {
  return engine_max_clusters_t<VAR_POLY>(Np, cluster, threads, smem, out);
}

cudaError_t launch_engine_poly(const EngineArgs& a, int nscans, int threads, size_t smem, cudaStream_t st) {
  return launch_engine_t<VAR_POLY>(a, nscans, threads, smem, st);
}

}  // namespace ptyg
