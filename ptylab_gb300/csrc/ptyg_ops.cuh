// Host-callable launchers of ptyg_ops.cu, ptyg_engine.cu, ptyg_engine_mq.cu and ptyg_e3pie.cu.
#pragma once

#include <cuda_runtime.h>

#include "ptyg_engine.cuh"

namespace ptyg {

// Row pass of a standalone propagation: per row, x * pre (or conj) * [sign]
// -> 1D transform -> * scale * [sign] * post (or conj).  The 2D centring
// modulation is one pre-sign in the first pass and one post-sign in the last.
// Tables (pre, post, filter) are Np x Np complex64 in natural order; with
// setDiv > 0 a table holds consecutive sets of Np x Np and field f reads set
// f / setDiv (one set per wavelength), else every field reads the one table.
struct RowOp {
  int inverse;
  int preSign;   // multiply the input by (-1)^(y+x)
  int postSign;  // multiply the output by (-1)^(y+x)
  const float2* pre;
  int conjPre;
  const float2* post;
  int conjPost;
  float scale;
  int preDiv, postDiv;
};

// Column pass: transform (inverse1), optionally * filter*filterScale (or conj)
// and transform again (inverse2); then * scale * [sign] * post.
struct ColOp {
  int inverse1;
  const float2* filter;
  int conjFilter;
  float filterScale;
  int inverse2;
  int postSign;  // multiply the output by (-1)^(y+x)
  const float2* post;
  int conjPost;
  float scale;
  int filterDiv, postDiv;
};

cudaError_t prop_rows(int Np, const float2* in, float2* out, int batch, const RowOp& op, const float2* tw,
                      cudaStream_t st);
cudaError_t prop_cols(int Np, const float2* in, float2* out, int batch, const ColOp& op, const float2* tw,
                      cudaStream_t st);
cudaError_t to_fourier_layout(const float* in, float* out, int frames, int Np, cudaStream_t st);
cudaError_t from_fourier_layout(const float* in, float* out, int frames, int Np, cudaStream_t st);
// the interferometric reference field (planes of Np x Np): ones in the data
// layout and scale (N M R), and back to R in natural order
cudaError_t reference_init(float2* out, int planes, int Np, bool centred, cudaStream_t st);
cudaError_t reference_natural(const float2* in, float2* out, int planes, int Np, bool centred, cudaStream_t st);
cudaError_t sum_parts(const double* part, double* err, int frames, int C, cudaStream_t st);
cudaError_t mul_window(float2* x, const float* w, long long n, long long nw, cudaStream_t st);
cudaError_t gram(const float2* p, int modes, long long n, double2* G, cudaStream_t st);
cudaError_t mix_modes(const float2* V, const float2* p, float2* out, int modes, long long n, cudaStream_t st);

int set_last_error(int code, const char* msg);

size_t engine_smem_bytes(int Np, int C, int nosm, int npsm, int nlambda, int engine, bool probe_in_smem,
                         bool asp_table_in_smem);
cudaError_t launch_engine(const EngineArgs& a, int nscans, int threads, size_t smem, cudaStream_t st);
bool engine_modes_supported(int Np, int nosm, int npsm);
bool engine_shape_supported(int Np, int cluster);
size_t e3pie_smem_bytes(int Np, int C, int npsm);
cudaError_t e3pie_max_clusters(int Np, int cluster, int threads, size_t smem, int* out);
cudaError_t launch_e3pie(const EngineArgs& a, int nscans, int threads, size_t smem, cudaStream_t st);
cudaError_t engine_max_clusters(int Np, int engine, int nlambda, int cluster, int threads, size_t smem, int* out);
cudaError_t engine_max_clusters_mq(int Np, int cluster, int threads, size_t smem, int* out);
cudaError_t launch_engine_mq(const EngineArgs& a, int nscans, int threads, size_t smem, cudaStream_t st);
cudaError_t engine_max_clusters_poly(int Np, int cluster, int threads, size_t smem, int* out);
cudaError_t launch_engine_poly(const EngineArgs& a, int nscans, int threads, size_t smem, cudaStream_t st);
cudaError_t launch_engine_fast(const EngineArgs& a, int nscans, int threads, size_t smem, cudaStream_t st);
cudaError_t engine_max_clusters_mq_poly(int Np, int cluster, int threads, size_t smem, int* out);
cudaError_t launch_engine_mq_poly(const EngineArgs& a, int nscans, int threads, size_t smem, cudaStream_t st);

}  // namespace ptyg
