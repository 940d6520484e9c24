// The mqNewton instantiations of the position-loop kernel (ptyg_engine_kernel.cuh).
#include "ptyg_engine_kernel.cuh"
#include "ptyg_ops.cuh"

namespace ptyg {

cudaError_t engine_max_clusters_mq(int Np, int cluster, int threads, size_t smem, int* out) {
  return engine_max_clusters_t<VAR_MQ>(Np, cluster, threads, smem, out);
}

cudaError_t launch_engine_mq(const EngineArgs& a, int nscans, int threads, size_t smem, cudaStream_t st) {
  return launch_engine_t<VAR_MQ>(a, nscans, threads, smem, st);
}

}  // namespace ptyg
