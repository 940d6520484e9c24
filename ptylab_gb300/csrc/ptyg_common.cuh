// Common device code for the GB300 ptychography kernels: complex arithmetic,
// the register-resident warp FFT and the cluster barrier.
//
// Warp FFT layout (one warp transforms one line of N = 32*E complex64 points):
//   natural layout : lane t, register j  <->  index n = t + 32*j
//   Fourier layout : lane l, register r  <->  index k = r + E*bitrev5(l)
// The forward transform takes natural input to Fourier layout: an E-point DFT
// inside each thread, a twiddle W_N^(t*k1), then a 32-point radix-2
// decimation-in-frequency across lanes with shuffles, which leaves lane l with
// output k2 = bitrev5(l).  The inverse is the exact mirror (decimation in time
// across lanes, conjugate twiddle, inverse in-thread DFT) and takes Fourier
// layout back to natural layout.  Both are unnormalised, so inverse(forward(x))
// = N*x.  A 2D transform is a row pass and a column pass; because every
// pointwise operation in the Fourier plane is applied in Fourier layout, no
// permutation is ever materialised -- only arrays that live in the Fourier
// plane (measured intensities, ASP transfer functions) are stored pre-permuted.
//
// Centring: for N divisible by 4, fftshift(fft2(ifftshift(x))) equals
// M * fft2(M * x) with M[i,j] = (-1)^(i+j), so the centred unitary transform of
// PtyLab/utils/utils.py:12-47 costs two sign flips instead of four copies.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define PTYG_DEV __device__ __forceinline__

namespace ptyg {

// ---------------------------------------------------------------- complex64
PTYG_DEV float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
PTYG_DEV float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
PTYG_DEV float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// conj(a) * b
PTYG_DEV float2 cmulc(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.x, b.y, -a.y * b.x));
}
PTYG_DEV float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
PTYG_DEV float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
PTYG_DEV float cabs2(float2 a) { return fmaf(a.x, a.x, a.y * a.y); }
PTYG_DEV float cabs(float2 a) { return sqrtf(cabs2(a)); }

// L2-only loads/stores for data another CTA of the cluster wrote or reads
// (the cluster barrier orders them; bypassing L1 avoids stale lines).
PTYG_DEV float2 ld_cg(const float2* p) { return __ldcg(p); }
PTYG_DEV void st_cg(float2* p, float2 v) { __stcg(p, v); }
PTYG_DEV float ld_cg(const float* p) { return __ldcg(p); }

PTYG_DEV unsigned bitrev5(unsigned l) { return __brev(l) >> 27; }

// ------------------------------------------------- 16th roots of unity, W16^m
// exp(-2*pi*i*m/16) for m = 0..7 (forward sign).  Values of cos/sin(k*pi/8).
PTYG_DEV float2 w16(int m) {
  const float c1 = 0.92387953251128674f;  // cos(pi/8)
  const float s1 = 0.38268343236508978f;  // sin(pi/8)
  const float h = 0.70710678118654752f;   // sqrt(1/2)
  switch (m & 7) {
    case 0: return make_float2(1.f, 0.f);
    case 1: return make_float2(c1, -s1);
    case 2: return make_float2(h, -h);
    case 3: return make_float2(s1, -c1);
    case 4: return make_float2(0.f, -1.f);
    case 5: return make_float2(-s1, -c1);
    case 6: return make_float2(-h, -h);
    default: return make_float2(-c1, -s1);
  }
}

template <int E>
struct Log2 {
  static constexpr int v = (E <= 1) ? 0 : 1 + Log2<E / 2>::v;
};
template <>
struct Log2<1> {
  static constexpr int v = 0;
};

template <int E>
PTYG_DEV int rev_bits(int i) {
  int r = 0;
#pragma unroll
  for (int b = 0; b < Log2<E>::v; ++b) r |= ((i >> b) & 1) << (Log2<E>::v - 1 - b);
  return r;
}

// In-register E-point DFT, natural order in and out.  Radix-2 decimation in
// frequency followed by a compile-time bit-reversal (register renaming).
template <int E, bool INV>
PTYG_DEV void dft_reg(float2 (&v)[E]) {
  if constexpr (E > 1) {
#pragma unroll
    for (int span = E / 2; span >= 1; span >>= 1) {
#pragma unroll
      for (int start = 0; start < E; start += 2 * span) {
#pragma unroll
        for (int m = 0; m < span; ++m) {
          const float2 a = v[start + m];
          const float2 b = v[start + m + span];
          v[start + m] = cadd(a, b);
          float2 w = w16(m * (16 / (2 * span)));
          if (INV) w.y = -w.y;
          v[start + m + span] = cmul(csub(a, b), w);
        }
      }
    }
    float2 t[E];
#pragma unroll
    for (int i = 0; i < E; ++i) t[i] = v[i];
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = t[rev_bits<E>(i)];
  }
}

// Per-lane twiddles of the five cross-lane stages: W_{2h}^(lane mod h) for
// h = 16, 8, 4, 2, 1 (forward sign), read from the N-point table.
struct LaneTw {
  float2 w[5];
};

template <int E>
PTYG_DEV LaneTw lane_twiddles(const float2* tw /* N = 32*E entries */, unsigned lane) {
  LaneTw t;
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const int h = 16 >> s;
    t.w[s] = tw[(lane & (h - 1)) * (16 * E / h)];
  }
  return t;
}

// Forward: natural -> Fourier layout, unnormalised.
template <int E>
PTYG_DEV void fft_fwd(float2 (&v)[E], const float2* tw, const LaneTw& lt, unsigned lane) {
  dft_reg<E, false>(v);
#pragma unroll
  for (int k1 = 1; k1 < E; ++k1) v[k1] = cmul(v[k1], tw[lane * k1]);
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const int h = 16 >> s;
    const bool upper = (lane & h) != 0;
    const float sg = upper ? -1.f : 1.f;
    const float2 w = upper ? lt.w[s] : make_float2(1.f, 0.f);
#pragma unroll
    for (int r = 0; r < E; ++r) {
      float2 o;
      o.x = __shfl_xor_sync(0xffffffffu, v[r].x, h);
      o.y = __shfl_xor_sync(0xffffffffu, v[r].y, h);
      // lower lane: mine + other ; upper lane: (other - mine) * w
      const float2 s2 = make_float2(fmaf(sg, v[r].x, o.x), fmaf(sg, v[r].y, o.y));
      v[r] = cmul(s2, w);
    }
  }
}

// Inverse: Fourier layout -> natural, unnormalised (sum with exp(+i...)).
template <int E>
PTYG_DEV void fft_inv(float2 (&v)[E], const float2* tw, const LaneTw& lt, unsigned lane) {
#pragma unroll
  for (int s = 4; s >= 0; --s) {
    const int h = 16 >> s;
    const bool upper = (lane & h) != 0;
    const float2 wc = cconj(lt.w[s]);
#pragma unroll
    for (int r = 0; r < E; ++r) {
      float2 o;
      o.x = __shfl_xor_sync(0xffffffffu, v[r].x, h);
      o.y = __shfl_xor_sync(0xffffffffu, v[r].y, h);
      // lower: mine + conj(w)*other ; upper: other - conj(w)*mine
      const float2 p = upper ? o : v[r];
      const float2 q = upper ? v[r] : o;
      const float2 t = cmul(q, wc);
      v[r] = upper ? csub(p, t) : cadd(p, t);
    }
  }
#pragma unroll
  for (int k1 = 1; k1 < E; ++k1) v[k1] = cmulc(tw[lane * k1], v[k1]);
  dft_reg<E, true>(v);
}

// Index helpers for the two layouts.
template <int E>
PTYG_DEV int fourier_index(int r, unsigned lane) {
  return r + E * (int)bitrev5(lane);
}

}  // namespace ptyg
