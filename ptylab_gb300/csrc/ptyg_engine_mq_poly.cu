// The mqNewton instantiations over several wavelengths (ptyg_engine_kernel.cuh).
#include "ptyg_engine_kernel.cuh"
#include "ptyg_ops.cuh"

namespace ptyg {

cudaError_t engine_max_clusters_mq_poly(int Np, int cluster, int threads, size_t smem, int* out) {
  return engine_max_clusters_t<VAR_MQ_POLY>(Np, cluster, threads, smem, out);
}

cudaError_t launch_engine_mq_poly(const EngineArgs& a, int nscans, int threads, size_t smem, cudaStream_t st) {
  return launch_engine_t<VAR_MQ_POLY>(a, nscans, threads, smem, st);
}

}  // namespace ptyg
