// The common-case instantiation of the position-loop kernel
// (ptyg_engine_kernel.cuh, VAR_FAST): ePIE / mPIE / qNewton at one wavelength
// with one object mode, Fraunhofer or Fresnel, and the standard intensity
// projection -- PtyLab's defaults -- with those switches as compile-time
// constants.
#include "ptyg_engine_kernel.cuh"
#include "ptyg_ops.cuh"

namespace ptyg {

cudaError_t launch_engine_fast(const EngineArgs& a, int nscans, int threads, size_t smem, cudaStream_t st) {
  return launch_engine_t<VAR_FAST>(a, nscans, threads, smem, st);
}

}  // namespace ptyg
