// Differentiable multislice forward model and its hand-written adjoint.
//
// Forward, for every position j and probe mode p (nosm = 1, S slices):
//   psi_0 = O_0[patch_j] * P_p
//   u_s   = ifft2(fft2(psi_{s-1}) * H),  psi_s = u_s * O_s[patch_j]     s = 1..S-1
//   Psi   = fft2c(psi_{S-1})                       (centred, unitary)
//   I_j   = sum_p |Psi_p|^2
// This is the model e3PIE inverts (PtyLab/Engines/e3PIE.py:99-118 with the
// Fraunhofer detector, BaseEngine.py:880-891).
//
// Adjoint, given g_j = dL/dI_j (real), in PyTorch's complex-gradient
// convention (grad = dL/dRe + i dL/dIm):
//   G   = 2 ifft2c(g * Psi)
//   for s = S-1..1:  dO_s[patch] += conj(u_s) * G ;  G = ifft2(fft2(conj(O_s[patch]) * G) * conj(H))
//   dO_0[patch] += conj(P) * G ;  dP += conj(O_0[patch]) * G
// summed over modes and positions.  Positions are processed in chunks; the
// adjoint recomputes each chunk's slice fields instead of keeping them for the
// whole scan.  Object gradients of overlapping patches are accumulated with
// atomic adds; the probe gradient is reduced per pixel over the chunk in a
// fixed order.
#include <cuda_runtime.h>

#include "../../include/ptyg.h"
#include "ptyg_common.cuh"
#include "ptyg_ops.cuh"

namespace ptyg {

// out[j,p] = O[patch_j] * (probe[p] if in == nullptr else in[j,p]), optionally
// also copying the multiplicand (the incident field) to `inc`.
// Frame of the j-th position of a chunk starting at `first`: order[first + j]
// when an order is given (a subset of the scan in any order), else first + j.
__device__ __forceinline__ int ms_frame(const int* order, int first, int j) {
  return order ? order[first + j] : first + j;
}

__global__ void ms_gather_mul(const float2* __restrict__ O, const float2* __restrict__ probe,
                              const float2* __restrict__ in, float2* __restrict__ out, float2* __restrict__ inc,
                              const int* __restrict__ pos, const int* __restrict__ order, int first, int count,
                              int npsm, int Np, int No) {
  const size_t n2 = (size_t)Np * Np;
  const size_t total = (size_t)count * npsm * n2;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t pix = i % n2;
    const size_t jp = i / n2;
    const int p = (int)(jp % npsm);
    const int j = (int)(jp / npsm);
    const int y = (int)(pix / Np), x = (int)(pix % Np);
    const int frame = ms_frame(order, first, j);
    const float2 o = O[(size_t)(pos[2 * frame] + y) * No + pos[2 * frame + 1] + x];
    const float2 f = in ? in[i] : probe[(size_t)p * n2 + pix];
    if (inc) inc[i] = f;
    out[i] = cmul(o, f);
  }
}

// I[j] = sum_p |Psi[j,p]|^2
__global__ void ms_intensity(const float2* __restrict__ Psi, float* __restrict__ I, int count, int npsm, int n2) {
  const size_t total = (size_t)count * n2;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t j = i / n2, pix = i % n2;
    float s = 0.f;
    for (int p = 0; p < npsm; ++p) s += cabs2(Psi[(j * npsm + p) * n2 + pix]);
    I[i] = s;
  }
}

// X[j,p] = 2 g[j] Psi[j,p]
__global__ void ms_scale_by_grad(float2* __restrict__ X, const float* __restrict__ g, int count, int npsm, int n2) {
  const size_t total = (size_t)count * npsm * n2;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t pix = i % n2, j = i / n2 / npsm;
    X[i] = cscale(X[i], 2.f * g[j * n2 + pix]);
  }
}

// dO[patch_j] += sum_p conj(u[j,p]) * G[j,p]  (atomic: patches overlap), then
// G[j,p] = conj(O[patch_j]) * G[j,p]  when `O` is given; with `illum`, also
// illum[patch_j] += sum_p |u[j,p]|^2 (the slice's illumination).
__global__ void ms_object_grad(const float2* __restrict__ u, float2* __restrict__ G, const float2* __restrict__ O,
                               float2* __restrict__ dO, float* __restrict__ illum, const int* __restrict__ pos,
                               const int* __restrict__ order, int first, int count, int npsm, int Np, int No) {
  const size_t n2 = (size_t)Np * Np;
  const size_t total = (size_t)count * n2;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t pix = i % n2, j = i / n2;
    const int y = (int)(pix / Np), x = (int)(pix % Np);
    const int frame = ms_frame(order, first, (int)j);
    const size_t oi = (size_t)(pos[2 * frame] + y) * No + pos[2 * frame + 1] + x;
    float2 acc = make_float2(0.f, 0.f);
    float w = 0.f;
    const float2 o = O ? O[oi] : make_float2(0.f, 0.f);
    for (int p = 0; p < npsm; ++p) {
      const size_t k = (j * npsm + p) * n2 + pix;
      const float2 gv = G[k];
      acc = cadd(acc, cmulc(u[k], gv));
      if (illum) w += cabs2(u[k]);
      if (O) G[k] = cmulc(o, gv);
    }
    atomicAdd(&dO[oi].x, acc.x);
    atomicAdd(&dO[oi].y, acc.y);
    if (illum) atomicAdd(&illum[oi], w);
  }
}

// dP[p, pix] += sum_j conj(O_0[patch_j]) * G[j,p]  (fixed order over j); with
// `illum`, also illum[p, pix] += sum_j |O_0[patch_j]|^2.
__global__ void ms_probe_grad(const float2* __restrict__ O, const float2* __restrict__ G, float2* __restrict__ dP,
                              float* __restrict__ illum, const int* __restrict__ pos, const int* __restrict__ order,
                              int first, int count, int npsm, int Np, int No) {
  const size_t n2 = (size_t)Np * Np;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < (size_t)npsm * n2;
       i += (size_t)gridDim.x * blockDim.x) {
    const int p = (int)(i / n2);
    const size_t pix = i % n2;
    const int y = (int)(pix / Np), x = (int)(pix % Np);
    float2 acc = dP[i];
    float w = 0.f;
    for (int j = 0; j < count; ++j) {
      const int frame = ms_frame(order, first, j);
      const float2 o = O[(size_t)(pos[2 * frame] + y) * No + pos[2 * frame + 1] + x];
      acc = cadd(acc, cmulc(o, G[((size_t)j * npsm + p) * n2 + pix]));
      w += cabs2(o);
    }
    dP[i] = acc;
    if (illum) illum[i] += w;  // the same weight for every mode plane
  }
}

// The amplitude residual at the detector: I = sum_p |Psi[j,p]|^2 against the
// measured frame, dL/dI = 1 - sqrt(I_m / (I + 1e-10)) for the amplitude loss
// L = sum (sqrt(I) - sqrt(I_m))^2, and X = 2 dL/dI Psi in place (the start of
// the adjoint, as ms_scale_by_grad).  err[frame] += sum |I_m - I| (one FP64
// atomic per warp), the reference's per-position detector error
// (BaseEngine.py:843-868).
__global__ void ms_amplitude_residual(float2* __restrict__ X, const float* __restrict__ measured,
                                      double* __restrict__ err, const int* __restrict__ order, int first, int count,
                                      int npsm, int n2) {
  const size_t total = (size_t)count * n2;
  for (size_t i0 = (size_t)blockIdx.x * blockDim.x; i0 < total; i0 += (size_t)gridDim.x * blockDim.x) {
    const size_t i = i0 + threadIdx.x;
    float e = 0.f;
    int frame = -1;
    if (i < total) {
      const size_t j = i / n2, pix = i % n2;
      frame = ms_frame(order, first, (int)j);
      float I = 0.f;
      for (int p = 0; p < npsm; ++p) I += cabs2(X[(j * npsm + p) * n2 + pix]);
      const float im = measured[(size_t)frame * n2 + pix];
      e = fabsf(im - I);
      const float g = 2.f * (1.f - sqrtf(im / (I + 1e-10f)));
      for (int p = 0; p < npsm; ++p) X[(j * npsm + p) * n2 + pix] = cscale(X[(j * npsm + p) * n2 + pix], g);
    }
    if (err) {
      // n2 is a multiple of 32: a warp's pixels belong to one frame
      for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
      if ((threadIdx.x & 31) == 0 && frame >= 0) atomicAdd(&err[frame], (double)e);
    }
  }
}

// max over a plane of non-negative floats into out[plane] (float bits order
// like the values; out zeroed by the caller)
__global__ void plane_max(const float* __restrict__ w, size_t n, float* __restrict__ out) {
  const int plane = blockIdx.y;
  float m = 0.f;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    m = fmaxf(m, w[(size_t)plane * n + i]);
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<unsigned*>(out) + plane, __float_as_uint(m));
}

// x -= (beta / 2) sqrt(w / wmax) / (w + reg) * g, then g = 0 and w = 0 (ready
// for the next accumulation): the quasi-Newton step of PtyLab's qNewton
// (qNewton.py:108-140: |P| / max|P| * conj(P) DELTA / (|P|^2 + reg)) with the
// illumination w summed over the positions of the step; g is the gradient in
// the dL/dRe + i dL/dIm convention, -2 conj(P) DELTA for one position.
__global__ void qn_apply(float2* __restrict__ x, float2* __restrict__ g, float* __restrict__ w, size_t n,
                         const float* __restrict__ wmax, float beta, float reg) {
  const int plane = blockIdx.y;
  const float inv = wmax[plane] > 0.f ? 1.f / wmax[plane] : 0.f;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t k = (size_t)plane * n + i;
    const float wk = w[k];
    const float f = 0.5f * beta * sqrtf(wk * inv) / (wk + reg);
    const float2 gk = g[k];
    const float2 xk = x[k];
    x[k] = make_float2(xk.x - f * gk.x, xk.y - f * gk.y);
    g[k] = make_float2(0.f, 0.f);
    w[k] = 0.f;
  }
}

static unsigned grid_for(size_t n) {
  const size_t b = (n + 255) / 256;
  return (unsigned)(b < 4096 ? (b ? b : 1) : 4096);
}

}  // namespace ptyg

// ---------------------------------------------------------------- C ABI
namespace {


int check_ms(const ptyg_multislice* m) {
  if (!m) return ptyg::set_last_error(PTYG_ERR_INVALID, "null multislice geometry");
  if (!(m->Np == 32 || m->Np == 64 || m->Np == 128 || m->Np == 256))
    return ptyg::set_last_error(PTYG_ERR_UNSUPPORTED, "multislice Np must be 32, 64, 128 or 256");
  if (m->No < m->Np || m->npsm < 1 || m->nslice < 1 || m->num_frames < 0 || m->chunk < 1)
    return ptyg::set_last_error(PTYG_ERR_INVALID, "bad multislice geometry");
  return PTYG_OK;
}

size_t field_bytes(const ptyg_multislice* m) { return (size_t)m->chunk * m->npsm * m->Np * m->Np * sizeof(float2); }

}  // namespace

extern "C" size_t ptyg_multislice_workspace_bytes(const ptyg_multislice* m) {
  if (check_ms(m) != PTYG_OK) return 0;
  // psi, scratch, and one incident field per slice (recomputed per chunk)
  return field_bytes(m) * (size_t)(2 + m->nslice);
}

// One pass over the positions: the forward model, and for the adjoint either
// a given dL/dI (grad_intensity) or the amplitude residual against `measured`
// (with optional per-frame errors and illuminations).  `order` (optional)
// lists the frames to visit.
struct MsExtra {
  const int32_t* order = nullptr;
  const float* measured = nullptr;
  double* err = nullptr;
  float* illum_object = nullptr;
  float* illum_probe = nullptr;
};

static int ms_run(const ptyg_multislice* m, const void* object, const void* probe, const int32_t* positions,
                  const void* slice_h, float* intensity, const float* grad_intensity, void* grad_object,
                  void* grad_probe, void* workspace, size_t workspace_bytes, void* stream, const MsExtra& x = MsExtra{}) {
  int r = check_ms(m);
  if (r) return r;
  if (!object || !probe || !positions || (m->nslice > 1 && !slice_h))
    return ptyg::set_last_error(PTYG_ERR_INVALID, "object, probe, positions (and slice_h for nslice > 1) are required");
  if (!workspace || workspace_bytes < ptyg_multislice_workspace_bytes(m))
    return ptyg::set_last_error(PTYG_ERR_INVALID, "workspace smaller than ptyg_multislice_workspace_bytes()");
  cudaStream_t st = (cudaStream_t)stream;
  const int Np = m->Np, No = m->No, npsm = m->npsm, S = m->nslice;
  const size_t n2 = (size_t)Np * Np, No2 = (size_t)No * No;
  const float2* O = (const float2*)object;
  const float2* P = (const float2*)probe;
  const float2* H = (const float2*)slice_h;
  float2* psi = (float2*)workspace;
  float2* scratch = psi + (size_t)m->chunk * npsm * n2;
  float2* inc = scratch + (size_t)m->chunk * npsm * n2;  // S fields: incident field of each slice
  const bool adjoint = grad_intensity != nullptr || x.measured != nullptr;
  const int* order = x.order;
  auto prop = [](int kind, int dir, int shift, int n, int b, const void* in, void* out, const void* tab, void* scr,
                 void* strm) { return ptyg_propagate(kind, dir, shift, n, b, in, out, tab, scr, strm); };
  for (int first = 0; first < m->num_frames; first += m->chunk) {
    const int count = (m->num_frames - first) < m->chunk ? (m->num_frames - first) : m->chunk;
    const size_t nf = (size_t)count * npsm * n2;
    const int batch = count * npsm;
    // forward: psi_0 = O_0 * P; psi_s = prop(psi_{s-1}) * O_s
    ptyg::ms_gather_mul<<<ptyg::grid_for(nf), 256, 0, st>>>(O, P, nullptr, psi, inc, positions, order, first, count,
                                                            npsm, Np, No);
    for (int s = 1; s < S; ++s) {
      r = prop(PTYG_ASP, PTYG_FORWARD, 0, Np, batch, psi, psi, H, scratch, stream);
      if (r) return r;
      ptyg::ms_gather_mul<<<ptyg::grid_for(nf), 256, 0, st>>>(O + s * No2, nullptr, psi, psi,
                                                              inc + (size_t)s * m->chunk * npsm * n2, positions,
                                                              order, first, count, npsm, Np, No);
    }
    r = prop(PTYG_FRAUNHOFER, PTYG_FORWARD, 0, Np, batch, psi, psi, nullptr, scratch, stream);
    if (r) return r;
    if (!adjoint) {
      ptyg::ms_intensity<<<ptyg::grid_for((size_t)count * n2), 256, 0, st>>>(psi, intensity + (size_t)first * n2,
                                                                             count, npsm, (int)n2);
      continue;
    }
    // adjoint: G = 2 ifft2c(g * Psi), then back through the slices
    if (x.measured)
      ptyg::ms_amplitude_residual<<<ptyg::grid_for((size_t)count * n2), 256, 0, st>>>(psi, x.measured, x.err, order,
                                                                                     first, count, npsm, (int)n2);
    else
      ptyg::ms_scale_by_grad<<<ptyg::grid_for(nf), 256, 0, st>>>(psi, grad_intensity + (size_t)first * n2, count, npsm,
                                                                 (int)n2);
    r = prop(PTYG_FRAUNHOFER, PTYG_INVERSE, 0, Np, batch, psi, psi, nullptr, scratch, stream);
    if (r) return r;
    for (int s = S - 1; s >= 1; --s) {
      ptyg::ms_object_grad<<<ptyg::grid_for((size_t)count * n2), 256, 0, st>>>(
          inc + (size_t)s * m->chunk * npsm * n2, psi, O + s * No2, (float2*)grad_object + s * No2,
          x.illum_object ? x.illum_object + s * No2 : nullptr, positions, order, first, count, npsm, Np, No);
      r = prop(PTYG_ASP, PTYG_INVERSE, 0, Np, batch, psi, psi, H, scratch, stream);
      if (r) return r;
    }
    ptyg::ms_object_grad<<<ptyg::grid_for((size_t)count * n2), 256, 0, st>>>(
        inc, psi, nullptr, (float2*)grad_object, x.illum_object, positions, order, first, count, npsm, Np, No);
    ptyg::ms_probe_grad<<<ptyg::grid_for((size_t)npsm * n2), 256, 0, st>>>(
        O, psi, (float2*)grad_probe, x.illum_probe, positions, order, first, count, npsm, Np, No);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return ptyg::set_last_error(PTYG_ERR_CUDA, cudaGetErrorString(e));
  return PTYG_OK;
}

extern "C" int ptyg_multislice_forward(const ptyg_multislice* m, const void* object, const void* probe,
                                       const int32_t* positions, const void* slice_h, float* intensity,
                                       void* workspace, size_t workspace_bytes, void* stream) {
  if (!intensity) return ptyg::set_last_error(PTYG_ERR_INVALID, "null intensity output");
  return ms_run(m, object, probe, positions, slice_h, intensity, nullptr, nullptr, nullptr, workspace,
                workspace_bytes, stream);
}

extern "C" int ptyg_multislice_adjoint(const ptyg_multislice* m, const void* object, const void* probe,
                                       const int32_t* positions, const void* slice_h, const float* grad_intensity,
                                       void* grad_object, void* grad_probe, void* workspace, size_t workspace_bytes,
                                       void* stream) {
  if (!grad_intensity || !grad_object || !grad_probe)
    return ptyg::set_last_error(PTYG_ERR_INVALID, "null gradient buffer");
  return ms_run(m, object, probe, positions, slice_h, nullptr, grad_intensity, grad_object, grad_probe, workspace,
                workspace_bytes, stream);
}

extern "C" int ptyg_multislice_amplitude_gradient(const ptyg_multislice* m, const void* object, const void* probe,
                                                  const int32_t* positions, const void* slice_h, const int32_t* order,
                                                  const float* measured, void* grad_object, void* grad_probe,
                                                  float* illum_object, float* illum_probe, double* err_at_pos,
                                                  void* workspace, size_t workspace_bytes, void* stream) {
  if (!measured || !grad_object || !grad_probe)
    return ptyg::set_last_error(PTYG_ERR_INVALID, "null measured intensities or gradient buffer");
  MsExtra x;
  x.order = order;
  x.measured = measured;
  x.err = err_at_pos;
  x.illum_object = illum_object;
  x.illum_probe = illum_probe;
  return ms_run(m, object, probe, positions, slice_h, nullptr, nullptr, grad_object, grad_probe, workspace,
                workspace_bytes, stream, x);
}

extern "C" int ptyg_qn_step(void* x, void* grad, float* weight, int planes, int64_t plane_size, float beta, float reg,
                            float* scratch, void* stream) {
  if (!x || !grad || !weight || !scratch) return ptyg::set_last_error(PTYG_ERR_INVALID, "null argument");
  if (planes < 1 || planes > 64 || plane_size < 1) return ptyg::set_last_error(PTYG_ERR_INVALID, "bad plane count or size");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(scratch, 0, (size_t)planes * sizeof(float), st);
  if (e != cudaSuccess) return ptyg::set_last_error(PTYG_ERR_CUDA, cudaGetErrorString(e));
  const size_t n = (size_t)plane_size;
  const unsigned gx = (unsigned)((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024);
  ptyg::plane_max<<<dim3(gx, (unsigned)planes), 256, 0, st>>>(weight, n, scratch);
  ptyg::qn_apply<<<dim3(gx, (unsigned)planes), 256, 0, st>>>((float2*)x, (float2*)grad, weight, n, scratch, beta, reg);
  e = cudaGetLastError();
  if (e != cudaSuccess) return ptyg::set_last_error(PTYG_ERR_CUDA, cudaGetErrorString(e));
  return PTYG_OK;
}
