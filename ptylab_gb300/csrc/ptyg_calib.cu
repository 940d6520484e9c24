// FPM illumination calibration (PtyLab/Reconstruction/CalibrationFPM.py):
// the Fourier-domain images of the LED frames, the circle-edge search over
// radii and grid shifts, and the RMSE of every candidate shift.  The host
// keeps the reference's decision logic; these kernels do the arithmetic.
//
// Rounding follows the reference's NumPy/SciPy where it can be followed:
// products in double rounded once to float (NumPy's float32 * float64
// in-place), SciPy's symmetric correlation order for the Gaussian, its
// corner order for bilinear interpolation, NumPy's pairwise float32 sum
// for means over a row, and pupil masks decided in double.  Double
// operations use explicit __d*_rn intrinsics so no FMA contraction changes
// them.  The FFTs are this library's complex64 transforms.

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>

#include "../../include/ptyg.h"
#include "ptyg_ops.cuh"

namespace ptyg {
int set_last_error(int code, const char* msg);
}

namespace {

constexpr int kMaxGaussRadius = 63;
constexpr int kMaxAngles = 64;

int cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return PTYG_OK;
  static thread_local char buf[256];
  snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  return ptyg::set_last_error(e == cudaErrorMemoryAllocation ? PTYG_ERR_OOM : PTYG_ERR_CUDA, buf);
}

int invalid(const char* msg) { return ptyg::set_last_error(PTYG_ERR_INVALID, msg); }

// deterministic block sum of doubles (blockDim.x a multiple of 32, <= 1024)
__device__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  v = threadIdx.x < nw ? sh[threadIdx.x] : 0.0;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
  __syncthreads();
  return v;  // valid in thread 0
}

// windowed = float(double(frame) * window); complex copy for the FFT;
// per-frame FP64 sums.  One block per frame.
__global__ void window_kernel(const float* __restrict__ frames, const double* __restrict__ window,
                              float* __restrict__ windowed, float2* __restrict__ spectra, double* __restrict__ sums,
                              int NN) {
  __shared__ double sh[32];
  const size_t base = (size_t)blockIdx.x * NN;
  double acc = 0.0;
  for (int i = threadIdx.x; i < NN; i += blockDim.x) {
    const float v = __double2float_rn(__dmul_rn((double)frames[base + i], window[i]));
    windowed[base + i] = v;
    spectra[base + i] = make_float2(v, 0.f);
    acc = __dadd_rn(acc, (double)v);
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) sums[blockIdx.x] = acc;
}

// |spectrum| per frame into ft (through double, rounded once); per-pixel
// mean over the frames into norm, summed in float32 frame by frame and
// divided in float32 like NumPy's mean over the first axis.
__global__ void magnitude_mean_kernel(const float2* __restrict__ spectra, float* __restrict__ ft,
                                      float* __restrict__ norm, int n, int NN) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NN) return;
  float acc = 0.f;
  for (int f = 0; f < n; ++f) {
    const float2 z = spectra[(size_t)f * NN + p];
    const double x = z.x, y = z.y;
    const float m = __double2float_rn(sqrt(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y))));
    ft[(size_t)f * NN + p] = m;
    acc = __fadd_rn(acc, m);
  }
  norm[p] = __fdiv_rn(acc, (float)n);
}

// ft = |ft / max(norm, floor)|, floor = 2 x the mean of norm outside the
// 2-NA support (computed by the caller).
__global__ void normalise_kernel(float* __restrict__ ft, const float* __restrict__ norm, float floor_value, int NN,
                                 size_t total) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const float d = fmaxf(norm[i % NN], floor_value);
  ft[i] = fabsf(__fdiv_rn(ft[i], d));
}

struct GaussWeights {
  double w[kMaxGaussRadius + 1];  // w[k] = weight at distance k
};

// One axis of scipy.ndimage.gaussian_filter (mode "nearest"), SciPy's
// symmetric order: x0 w0, then (x[-k] + x[k]) w[k] for k = r .. 1.
__global__ void gauss_axis_kernel(const float* __restrict__ in, float* __restrict__ out, int N, int axis, int r,
                                  GaussWeights gw, size_t total) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const int NN = N * N;
  const size_t f = idx / NN;
  const int p = (int)(idx - f * NN);
  const int i = p / N, j = p - (p / N) * N;
  const float* img = in + f * NN;
  const int pos = axis == 0 ? i : j;
  auto at = [&](int q) -> double {
    q = q < 0 ? 0 : (q > N - 1 ? N - 1 : q);
    return (double)(axis == 0 ? img[q * N + j] : img[i * N + q]);
  };
  double acc = __dmul_rn(at(pos), gw.w[0]);
  for (int k = r; k >= 1; --k) acc = __dadd_rn(acc, __dmul_rn(__dadd_rn(at(pos - k), at(pos + k)), gw.w[k]));
  out[idx] = __double2float_rn(acc);
}

struct Angles {
  double s[kMaxAngles];
  double c[kMaxAngles];
};

constexpr int kMaxRadii = 64;
struct Radii {
  double r[kMaxRadii];
};

// NumPy's pairwise float32 sum of n <= 128 values (a 8-accumulator block).
__device__ float pairwise_sum_f32(const float* a, int n) {
  if (n < 8) {
    float res = 0.f;
    for (int i = 0; i < n; ++i) res = __fadd_rn(res, a[i]);
    return res;
  }
  float r[8];
  for (int k = 0; k < 8; ++k) r[k] = a[k];
  int i = 8;
  for (; i < n - (n % 8); i += 8)
    for (int k = 0; k < 8; ++k) r[k] = __fadd_rn(r[k], a[i + k]);
  float res = __fadd_rn(__fadd_rn(__fadd_rn(r[0], r[1]), __fadd_rn(r[2], r[3])),
                        __fadd_rn(__fadd_rn(r[4], r[5]), __fadd_rn(r[6], r[7])));
  for (; i < n; ++i) res = __fadd_rn(res, a[i]);
  return res;
}

// Mean over the kept angles of the bilinearly sampled image on the circle
// of radius R_r about (N/2 + p0 + g_a, N/2 + p1 + g_b).  One block per
// (task, radius): the row coordinate of every (angle, a) and the column
// coordinate of every (angle, b) are computed once into shared memory (the
// reference's float64 sums rounded to float32, floor and fraction, both
// exact), then each thread takes grid shifts (a, b) and interpolates in
// double in SciPy's corner order.  out[task][r][a][b].
__global__ void arcs_kernel(const float* __restrict__ images, int N, const int* __restrict__ task_image,
                            const double* __restrict__ task_pos, const unsigned long long* __restrict__ task_keep,
                            Radii radii, int R, Angles ang, int nang, int S, float* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char arcs_smem[];
  __shared__ int kidx[kMaxAngles];
  __shared__ int nk;
  const int t = blockIdx.x / R, r = blockIdx.x - (blockIdx.x / R) * R;
  const int G = 2 * S + 1;
  const unsigned long long keep = task_keep[t];
  if (threadIdx.x == 0) {
    int n = 0;
    for (int k = 0; k < nang; ++k)
      if ((keep >> k) & 1ull) kidx[n++] = k;
    nk = n;
  }
  __syncthreads();
  const int n = nk;
  int* xi = (int*)arcs_smem;
  float* xt = (float*)(xi + nang * G);
  int* yi = (int*)(xt + nang * G);
  float* yt = (float*)(yi + nang * G);
  const double half = (double)N / 2.0;
  const double rad = radii.r[r];
  const double p0 = task_pos[2 * t], p1 = task_pos[2 * t + 1];
  for (int e = threadIdx.x; e < n * G; e += blockDim.x) {
    const int kk = e / G, a = e - (e / G) * G;
    const int k = kidx[kk];
    const double cx = (double)__double2float_rn(
        __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(rad, ang.s[k]), half), p0), (double)(a - S)));
    const double cy = (double)__double2float_rn(
        __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(rad, ang.c[k]), half), p1), (double)(a - S)));
    const double fx = floor(cx), fy = floor(cy);
    xi[e] = (int)fx;
    xt[e] = (float)__dsub_rn(cx, fx);  // exact: a float32 coordinate's fraction
    yi[e] = (int)fy;
    yt[e] = (float)__dsub_rn(cy, fy);
  }
  __syncthreads();
  const float* img = images + (size_t)task_image[t] * N * N;
  float* o = out + (size_t)blockIdx.x * G * G;
  for (int ab = threadIdx.x; ab < G * G; ab += blockDim.x) {
    const int a = ab / G, b = ab - (ab / G) * G;
    float vals[kMaxAngles];
    for (int kk = 0; kk < n; ++kk) {
      const int x0 = xi[kk * G + a], y0 = yi[kk * G + b];
      const double tx = xt[kk * G + a], ty = yt[kk * G + b];
      const double wx[2] = {__dsub_rn(1.0, tx), tx};
      const double wy[2] = {__dsub_rn(1.0, ty), ty};
      double acc = 0.0;
      for (int u = 0; u < 2; ++u)
        for (int v = 0; v < 2; ++v) {
          const int xx = x0 + u, yy = y0 + v;
          const double px = (xx >= 0 && xx < N && yy >= 0 && yy < N) ? (double)img[xx * N + yy] : 0.0;
          acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(px, wx[u]), wy[v]));
        }
      vals[kk] = __double2float_rn(acc);
    }
    o[ab] = n ? __fdiv_rn(pairwise_sum_f32(vals, n), (float)n) : nanf("");
  }
}

// Spectrum of LED cand_led[k] inside the pupil centred where the reference
// centres it for shift (q0, q1) = position + error candidate.
__global__ void pupil_spectra_kernel(const float2* __restrict__ spectra, int N, const int* __restrict__ cand_led,
                                     const int* __restrict__ cand_q, double r2, float2* __restrict__ out,
                                     size_t total) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const int NN = N * N;
  const size_t k = idx / NN;
  const int p = (int)(idx - k * NN);
  const int i = p / N, j = p - (p / N) * N;
  const double half = (double)N / 2.0;
  const double a = __dadd_rn(__dsub_rn((double)i, half), (double)cand_q[2 * k]);
  const double b = __dadd_rn(__dsub_rn((double)j, half), (double)cand_q[2 * k + 1]);
  const bool in = __dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)) <= r2;
  out[idx] = in ? spectra[(size_t)cand_led[k] * NN + p] : make_float2(0.f, 0.f);
}

// sqrt(mean((image - |estimate|)^2)) per candidate, FP64.  One block each.
__global__ void rms_kernel(const float2* __restrict__ est, const float* __restrict__ images,
                           const int* __restrict__ cand_led, int NN, double* __restrict__ rms) {
  __shared__ double sh[32];
  const int k = blockIdx.x;
  const float2* e = est + (size_t)k * NN;
  const float* img = images + (size_t)cand_led[k] * NN;
  double acc = 0.0;
  for (int i = threadIdx.x; i < NN; i += blockDim.x) {
    const double re = e[i].x, im = e[i].y;
    const double d = __dsub_rn((double)img[i], sqrt(__dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im))));
    acc = __dadd_rn(acc, __dmul_rn(d, d));
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) rms[k] = sqrt(acc / (double)NN);
}

bool valid_size(int N) { return N == 32 || N == 64 || N == 128 || N == 256; }

int run_gauss(int n, int N, int r, const double* half_weights, const float* in, float* out, float* tmp,
              cudaStream_t st) {
  if (r < 0 || r > kMaxGaussRadius || !half_weights)
    return ptyg::set_last_error(PTYG_ERR_UNSUPPORTED, "gaussian radius must lie in 0..63");
  GaussWeights gw{};
  for (int k = 0; k <= r; ++k) gw.w[k] = half_weights[k];
  const size_t total = (size_t)n * N * N;
  const int T = 256;
  const unsigned B = (unsigned)((total + T - 1) / T);
  gauss_axis_kernel<<<B, T, 0, st>>>(in, tmp, N, 0, r, gw, total);
  gauss_axis_kernel<<<B, T, 0, st>>>(tmp, out, N, 1, r, gw, total);
  return cuda_status(cudaGetLastError(), "gaussian");
}

}  // namespace

extern "C" int ptyg_calib_spectra(int n, int N, const float* frames, const double* window, float* windowed,
                                  double* frame_sums, void* spectra, float* ft, float* norm, void* stream) {
  if (!valid_size(N)) return ptyg::set_last_error(PTYG_ERR_UNSUPPORTED, "frame size must be 32, 64, 128 or 256");
  if (n < 1 || !frames || !window || !windowed || !frame_sums || !spectra || !ft || !norm)
    return invalid("bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  const int NN = N * N;
  window_kernel<<<n, 256, 0, st>>>(frames, window, windowed, (float2*)spectra, frame_sums, NN);
  int s = cuda_status(cudaGetLastError(), "calib window");
  if (s) return s;
  s = ptyg_propagate(PTYG_FRAUNHOFER, PTYG_INVERSE, 0, N, n, spectra, spectra, nullptr, nullptr, stream);
  if (s) return s;
  magnitude_mean_kernel<<<(NN + 255) / 256, 256, 0, st>>>((const float2*)spectra, ft, norm, n, NN);
  return cuda_status(cudaGetLastError(), "calib magnitude");
}

extern "C" int ptyg_calib_normalise(int n, int N, float* ft, const float* norm, float floor_value, void* stream) {
  if (n < 0 || N < 1 || !ft || !norm) return invalid("bad arguments");
  if (n == 0) return PTYG_OK;
  const size_t total = (size_t)n * N * N;
  normalise_kernel<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(ft, norm, floor_value, N * N,
                                                                                     total);
  return cuda_status(cudaGetLastError(), "calib normalise");
}

extern "C" int ptyg_calib_gaussian(int n, int N, int radius, const double* half_weights, const float* in, float* out,
                                   void* stream) {
  if (n < 0 || N < 1 || !in || !out) return invalid("bad arguments");
  if (radius < 0 || radius > kMaxGaussRadius || !half_weights)
    return ptyg::set_last_error(PTYG_ERR_UNSUPPORTED, "gaussian radius must lie in 0..63");
  if (n == 0) return PTYG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  float* tmp = nullptr;
  int s = cuda_status(cudaMallocAsync((void**)&tmp, (size_t)n * N * N * sizeof(float), st), "gaussian scratch");
  if (s) return s;
  s = run_gauss(n, N, radius, half_weights, in, out, tmp, st);
  cudaError_t e = cudaFreeAsync(tmp, st);
  return s ? s : cuda_status(e, "gaussian scratch free");
}

extern "C" int ptyg_calib_arcs(int N, const float* images, int ntasks, const int* task_image, const double* task_pos,
                               const unsigned long long* task_keep, int nradii, const double* radii, int nangles,
                               const double* sin_angles, const double* cos_angles, int search, float* out,
                               void* stream) {
  if (N < 4 || ntasks < 0 || nradii < 1 || nradii > kMaxRadii || search < 0 || search > 255 || nangles < 1 ||
      nangles > kMaxAngles)
    return invalid("bad arguments");
  if (ntasks == 0) return PTYG_OK;
  if (!images || !task_image || !task_pos || !task_keep || !radii || !sin_angles || !cos_angles || !out)
    return invalid("null pointer");
  Angles ang{};
  for (int k = 0; k < nangles; ++k) {
    ang.s[k] = sin_angles[k];
    ang.c[k] = cos_angles[k];
  }
  Radii rad{};
  for (int k = 0; k < nradii; ++k) rad.r[k] = radii[k];
  const int G = 2 * search + 1;
  const size_t smem = (size_t)nangles * G * 16;
  if (smem > 200 * 1024) return ptyg::set_last_error(PTYG_ERR_UNSUPPORTED, "search grid too large for one block");
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(arcs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "calib arcs shared memory");
  }
  const long long blocks = (long long)ntasks * nradii;
  if (blocks > 0x7fffffffLL) return invalid("too many tasks");
  arcs_kernel<<<(unsigned)blocks, 256, smem, (cudaStream_t)stream>>>(images, N, task_image, task_pos, task_keep,
                                                                     rad, nradii, ang, nangles, search, out);
  return cuda_status(cudaGetLastError(), "calib arcs");
}

extern "C" int ptyg_calib_rms(int N, const void* spectra, const float* images, int ncand, const int* cand_led,
                              const int* cand_q, double radius, double* rms, void* stream) {
  if (!valid_size(N)) return ptyg::set_last_error(PTYG_ERR_UNSUPPORTED, "frame size must be 32, 64, 128 or 256");
  if (ncand < 0 || !(radius >= 0)) return invalid("bad arguments");
  if (ncand == 0) return PTYG_OK;
  if (!spectra || !images || !cand_led || !cand_q || !rms) return invalid("null pointer");
  cudaStream_t st = (cudaStream_t)stream;
  const int NN = N * N;
  const int chunk = ncand < 1024 ? ncand : 1024;
  float2* buf = nullptr;
  int s = cuda_status(cudaMallocAsync((void**)&buf, (size_t)chunk * NN * sizeof(float2), st), "rms scratch");
  if (s) return s;
  const double r2 = radius * radius;
  for (int k0 = 0; k0 < ncand && !s; k0 += chunk) {
    const int m = ncand - k0 < chunk ? ncand - k0 : chunk;
    const size_t total = (size_t)m * NN;
    pupil_spectra_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(
        (const float2*)spectra, N, cand_led + k0, cand_q + 2 * k0, r2, buf, total);
    s = cuda_status(cudaGetLastError(), "calib pupil spectra");
    if (!s) s = ptyg_propagate(PTYG_FRAUNHOFER, PTYG_INVERSE, 0, N, m, buf, buf, nullptr, nullptr, stream);
    if (!s) {
      rms_kernel<<<m, 256, 0, st>>>(buf, images, cand_led + k0, NN, rms + k0);
      s = cuda_status(cudaGetLastError(), "calib rms");
    }
  }
  cudaError_t e = cudaFreeAsync(buf, st);
  return s ? s : cuda_status(e, "rms scratch free");
}
