// Standalone propagators (the Operators drop-in), layout permutations and
// the small per-iteration helper kernels.
#include "ptyg_common.cuh"
#include "ptyg_ops.cuh"

namespace ptyg {

// Warp-local conversions between the Fourier layout of fft_fwd/fft_inv and
// natural order, through a per-warp shared buffer of N complex64.
template <int E>
PTYG_DEV void fourier_to_natural(float2 (&v)[E], float2* buf, unsigned lane) {
#pragma unroll
  for (int r = 0; r < E; ++r) buf[fourier_index<E>(r, lane)] = v[r];
  __syncwarp();
#pragma unroll
  for (int j = 0; j < E; ++j) v[j] = buf[lane + 32 * j];
  __syncwarp();
}

template <int E>
PTYG_DEV void natural_to_fourier(float2 (&v)[E], float2* buf, unsigned lane) {
#pragma unroll
  for (int j = 0; j < E; ++j) buf[lane + 32 * j] = v[j];
  __syncwarp();
#pragma unroll
  for (int r = 0; r < E; ++r) v[r] = buf[fourier_index<E>(r, lane)];
  __syncwarp();
}

// Natural-order 1D transform of one line held by a warp.
template <int E>
PTYG_DEV void line_fft(float2 (&v)[E], bool inverse, const WarpFFT<E>& F, float2* buf, unsigned lane) {
  if (!inverse) {
    F.fwd(v);
    fourier_to_natural<E>(v, buf, lane);
  } else {
    natural_to_fourier<E>(v, buf, lane);
    F.inv(v);
  }
}

// Row pass: one warp per (field, row); natural layout in and out.
template <int E>
__global__ void prop_row_kernel(const float2* __restrict__ in, float2* __restrict__ out, int batch, RowOp op,
                                const float2* __restrict__ twiddle) {
  constexpr int NP = 32 * E;
  __shared__ float2 tw[NP];
  extern __shared__ float2 wbuf[];
  for (int i = threadIdx.x; i < NP; i += blockDim.x) tw[i] = twiddle[i];
  __syncthreads();
  const unsigned lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  WarpFFT<E> F;
  F.init(tw, lane);
  const long long line = (long long)blockIdx.x * (blockDim.x >> 5) + warp;
  if (line >= (long long)batch * NP) return;
  const int y = (int)(line % NP);
  const long long field = line / NP;
  const float2* src = in + line * NP;
  const float2* pre = op.pre ? op.pre + (op.preDiv > 0 ? (size_t)(field / op.preDiv) * NP * NP : 0) : nullptr;
  const float2* post = op.post ? op.post + (op.postDiv > 0 ? (size_t)(field / op.postDiv) * NP * NP : 0) : nullptr;
  float2 v[E];
  const float sg = (op.preSign && ((y + lane) & 1)) ? -1.f : 1.f;
#pragma unroll
  for (int j = 0; j < E; ++j) {
    float2 x = src[lane + 32 * j];
    if (pre) {
      float2 q = pre[y * NP + lane + 32 * j];
      if (op.conjPre) q.y = -q.y;
      x = cmul(x, q);
    }
    v[j] = cscale(x, sg);
  }
  line_fft<E>(v, op.inverse != 0, F, wbuf + warp * NP, lane);
  float2* dst = out + line * NP;
#pragma unroll
  for (int j = 0; j < E; ++j) {
    const int x = lane + 32 * j;
    float2 u = cscale(v[j], op.scale);
    if (op.postSign && ((y + x) & 1)) u = cscale(u, -1.f);
    if (post) {
      float2 q = post[y * NP + x];
      if (op.conjPost) q.y = -q.y;
      u = cmul(u, q);
    }
    dst[x] = u;
  }
}

// Column pass: a CTA stages a block of CB columns of one field in shared
// memory; one warp transforms one column (optionally: transform, multiply by
// a Fourier-plane filter, transform again), then the block is written back.
template <int E>
__global__ void prop_col_kernel(const float2* in, float2* out, int batch, ColOp op,
                                const float2* __restrict__ twiddle) {
  constexpr int NP = 32 * E;
  constexpr int CB = 8;
  constexpr int LD = CB + 1;
  __shared__ float2 tw[NP];
  extern __shared__ float2 smem[];
  float2* tile = smem;                  // NP * LD
  float2* wbuf = smem + NP * LD;        // nwarps * NP
  const int nblk = NP / CB;
  const int field = blockIdx.x / nblk;
  const int c0 = (blockIdx.x % nblk) * CB;
  if (field >= batch) return;
  const float2* filter =
      op.filter ? op.filter + (op.filterDiv > 0 ? (size_t)(field / op.filterDiv) * NP * NP : 0) : nullptr;
  const float2* post = op.post ? op.post + (op.postDiv > 0 ? (size_t)(field / op.postDiv) * NP * NP : 0) : nullptr;
  for (int i = threadIdx.x; i < NP; i += blockDim.x) tw[i] = twiddle[i];
  const float2* src = in + (size_t)field * NP * NP;
  for (int i = threadIdx.x; i < NP * CB; i += blockDim.x) {
    const int y = i / CB, c = i % CB;
    tile[y * LD + c] = src[(size_t)y * NP + c0 + c];
  }
  __syncthreads();
  const unsigned lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  WarpFFT<E> F;
  F.init(tw, lane);
  for (int c = warp; c < CB; c += nw) {
    const int x = c0 + c;
    float2 v[E];
#pragma unroll
    for (int j = 0; j < E; ++j) v[j] = tile[(lane + 32 * j) * LD + c];
    line_fft<E>(v, op.inverse1 != 0, F, wbuf + warp * NP, lane);
    if (filter) {
#pragma unroll
      for (int j = 0; j < E; ++j) {
        float2 h = filter[(size_t)(lane + 32 * j) * NP + x];
        if (op.conjFilter) h.y = -h.y;
        v[j] = cmul(v[j], cscale(h, op.filterScale));
      }
      line_fft<E>(v, op.inverse2 != 0, F, wbuf + warp * NP, lane);
    }
#pragma unroll
    for (int j = 0; j < E; ++j) {
      const int y = lane + 32 * j;
      float2 u = cscale(v[j], op.scale);
      if (op.postSign && ((y + x) & 1)) u = cscale(u, -1.f);
      if (post) {
        float2 q = post[(size_t)y * NP + x];
        if (op.conjPost) q.y = -q.y;
        u = cmul(u, q);
      }
      tile[y * LD + c] = u;
    }
  }
  __syncthreads();
  float2* dst = out + (size_t)field * NP * NP;
  for (int i = threadIdx.x; i < NP * CB; i += blockDim.x) {
    const int y = i / CB, c = i % CB;
    dst[(size_t)y * NP + c0 + c] = tile[y * LD + c];
  }
}

template <int E>
static cudaError_t rows_t(const float2* in, float2* out, int batch, const RowOp& op, const float2* tw,
                          cudaStream_t st) {
  constexpr int NP = 32 * E;
  const int warps = 8;
  const long long lines = (long long)batch * NP;
  const unsigned blocks = (unsigned)((lines + warps - 1) / warps);
  prop_row_kernel<E><<<blocks, warps * 32, warps * NP * sizeof(float2), st>>>(in, out, batch, op, tw);
  return cudaGetLastError();
}

template <int E>
static cudaError_t cols_t(const float2* in, float2* out, int batch, const ColOp& op, const float2* tw,
                          cudaStream_t st) {
  constexpr int NP = 32 * E;
  const int warps = 8;
  const size_t smem = (size_t)(NP * 9 + warps * NP) * sizeof(float2);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(prop_col_kernel<E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  prop_col_kernel<E><<<(unsigned)(batch * (NP / 8)), warps * 32, smem, st>>>(in, out, batch, op, tw);
  return cudaGetLastError();
}

cudaError_t prop_rows(int Np, const float2* in, float2* out, int batch, const RowOp& op, const float2* tw,
                      cudaStream_t st) {
  switch (Np) {
    case 32: return rows_t<1>(in, out, batch, op, tw, st);
    case 64: return rows_t<2>(in, out, batch, op, tw, st);
    case 128: return rows_t<4>(in, out, batch, op, tw, st);
    case 256: return rows_t<8>(in, out, batch, op, tw, st);
    default: return cudaErrorNotSupported;
  }
}

cudaError_t prop_cols(int Np, const float2* in, float2* out, int batch, const ColOp& op, const float2* tw,
                      cudaStream_t st) {
  switch (Np) {
    case 32: return cols_t<1>(in, out, batch, op, tw, st);
    case 64: return cols_t<2>(in, out, batch, op, tw, st);
    case 128: return cols_t<4>(in, out, batch, op, tw, st);
    case 256: return cols_t<8>(in, out, batch, op, tw, st);
    default: return cudaErrorNotSupported;
  }
}

// ----------------------------------------------------------------- layouts

// out[f][sx][sy] = in[f][ky(sy)][kx(sx)]  (natural -> Fourier layout, transposed)
__global__ void to_fourier_layout_kernel(const float* __restrict__ in, float* __restrict__ out, int frames, int Np) {
  const size_t n = (size_t)frames * Np * Np;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t f = i / ((size_t)Np * Np);
    const int rem = (int)(i - f * Np * Np);
    const int sx = rem / Np, sy = rem % Np;
    out[i] = in[(f * Np + slot_to_freq_y(sy, Np)) * Np + slot_to_freq_x(sx, Np)];
  }
}

// The interferometric reference field in the kernels' data layout and
// scale: the detector tile holds V = N M Psi (M = (-1)^(ky+kx) for centred
// transforms, 1 otherwise), so the field is kept as N M R.  Initial R = 1.
__global__ void reference_init_kernel(float2* __restrict__ out, int planes, int Np, int centred) {
  const size_t n = (size_t)planes * Np * Np;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int rem = (int)(i % ((size_t)Np * Np));
    const int sx = rem / Np, sy = rem % Np;
    const int ky = slot_to_freq_y(sy, Np), kx = slot_to_freq_x(sx, Np);
    const float m = (centred && ((ky + kx) & 1)) ? -1.f : 1.f;
    out[i] = make_float2(m * (float)Np, 0.f);
  }
}

// R in natural order from the data layout: out[k][ky][kx] = M in[k][sx][sy] / N
__global__ void reference_natural_kernel(const float2* __restrict__ in, float2* __restrict__ out, int planes, int Np,
                                         int centred) {
  const size_t n = (size_t)planes * Np * Np;
  const float inv = 1.f / (float)Np;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t f = i / ((size_t)Np * Np);
    const int rem = (int)(i - f * Np * Np);
    const int ky = rem / Np, kx = rem % Np;
    const int sy = freq_to_slot_y(ky, Np), sx = freq_to_slot_x(kx, Np);
    const float m = (centred && ((ky + kx) & 1)) ? -inv : inv;
    const float2 v = in[(f * Np + sx) * Np + sy];
    out[i] = make_float2(v.x * m, v.y * m);
  }
}

// out[f][ky][kx] = in[f][sx(kx)][sy(ky)]  (inverse of the above)
__global__ void from_fourier_layout_kernel(const float* __restrict__ in, float* __restrict__ out, int frames, int Np) {
  const size_t n = (size_t)frames * Np * Np;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t f = i / ((size_t)Np * Np);
    const int rem = (int)(i - f * Np * Np);
    const int ky = rem / Np, kx = rem % Np;
    const int sy = freq_to_slot_y(ky, Np), sx = freq_to_slot_x(kx, Np);
    out[i] = in[(f * Np + sx) * Np + sy];
  }
}

cudaError_t to_fourier_layout(const float* in, float* out, int frames, int Np, cudaStream_t st) {
  to_fourier_layout_kernel<<<1024, 256, 0, st>>>(in, out, frames, Np);
  return cudaGetLastError();
}

cudaError_t reference_init(float2* out, int planes, int Np, bool centred, cudaStream_t st) {
  reference_init_kernel<<<256, 256, 0, st>>>(out, planes, Np, centred ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t reference_natural(const float2* in, float2* out, int planes, int Np, bool centred, cudaStream_t st) {
  reference_natural_kernel<<<256, 256, 0, st>>>(in, out, planes, Np, centred ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t from_fourier_layout(const float* in, float* out, int frames, int Np, cudaStream_t st) {
  from_fourier_layout_kernel<<<1024, 256, 0, st>>>(in, out, frames, Np);
  return cudaGetLastError();
}

// err[f] = sum_c part[f][c] in a fixed order (deterministic)
__global__ void sum_parts_kernel(const double* __restrict__ part, double* __restrict__ err, int frames, int C) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= frames) return;
  double t = 0.0;
  for (int c = 0; c < C; ++c) t += part[(size_t)f * C + c];
  err[f] = t;
}

cudaError_t sum_parts(const double* part, double* err, int frames, int C, cudaStream_t st) {
  sum_parts_kernel<<<(frames + 255) / 256, 256, 0, st>>>(part, err, frames, C);
  return cudaGetLastError();
}

// ----------------------------------------------------------------- helpers
__global__ void mul_window_kernel(float2* x, const float* w, long long n, long long nw) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] = cscale(x[i], w[i % nw]);
}

cudaError_t mul_window(float2* x, const float* w, long long n, long long nw, cudaStream_t st) {
  mul_window_kernel<<<592, 256, 0, st>>>(x, w, n, nw);
  return cudaGetLastError();
}

// One CTA per (a, b) entry: G[a][b] = sum_i conj(p_a[i]) p_b[i] in FP64.
__global__ void gram_kernel(const float2* __restrict__ p, int modes, long long n, double2* __restrict__ G) {
  const int a = blockIdx.x / modes, b = blockIdx.x % modes;
  const float2* pa = p + (size_t)a * n;
  const float2* pb = p + (size_t)b * n;
  double re = 0.0, im = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    const float2 u = pa[i], v = pb[i];
    re += (double)u.x * v.x + (double)u.y * v.y;
    im += (double)u.x * v.y - (double)u.y * v.x;
  }
  __shared__ double sr[32], si[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_xor_sync(0xffffffffu, re, o);
    im += __shfl_xor_sync(0xffffffffu, im, o);
  }
  if (lane == 0) {
    sr[warp] = re;
    si[warp] = im;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tr = 0.0, ti = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      tr += sr[w];
      ti += si[w];
    }
    G[a * modes + b] = make_double2(tr, ti);
  }
}

cudaError_t gram(const float2* p, int modes, long long n, double2* G, cudaStream_t st) {
  gram_kernel<<<modes * modes, 512, 0, st>>>(p, modes, n, G);
  return cudaGetLastError();
}

__global__ void mix_modes_kernel(const float2* __restrict__ V, const float2* __restrict__ p, float2* __restrict__ out,
                                 int modes, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float2 x[16];
    const int m = modes < 16 ? modes : 16;
    for (int b = 0; b < m; ++b) x[b] = p[(size_t)b * n + i];
    for (int a = 0; a < m; ++a) {
      float2 acc = make_float2(0.f, 0.f);
      for (int b = 0; b < m; ++b) acc = cadd(acc, cmul(V[a * modes + b], x[b]));
      out[(size_t)a * n + i] = acc;
    }
  }
}

cudaError_t mix_modes(const float2* V, const float2* p, float2* out, int modes, long long n, cudaStream_t st) {
  if (modes > 16) return cudaErrorNotSupported;
  mix_modes_kernel<<<592, 256, 0, st>>>(V, p, out, modes, n);
  return cudaGetLastError();
}

}  // namespace ptyg
