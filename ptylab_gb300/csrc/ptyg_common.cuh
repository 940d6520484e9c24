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

#include <type_traits>

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

// ------------------------------------------------- in-register small DFTs
// Multiply by W_16^m (forward sign exp(-2*pi*i*m/16)), m a compile-time
// constant after unrolling; the trivial rotations cost no multiplies.
template <bool INV>
PTYG_DEV float2 mul_w16(float2 a, int m) {
  const float c1 = 0.92387953251128674f;  // cos(pi/8)
  const float s1 = 0.38268343236508978f;  // sin(pi/8)
  const float h = 0.70710678118654752f;   // sqrt(1/2)
  // forward W16^m = (cos, -sin); the inverse uses the conjugate
  float c, sn;
  switch (m & 15) {
    case 0: return a;
    case 4: return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);  // * (+i) / (-i)
    case 8: return make_float2(-a.x, -a.y);
    case 12: return INV ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
    case 2: c = h; sn = h; break;
    case 6: c = -h; sn = h; break;
    case 10: c = -h; sn = -h; break;
    case 14: c = h; sn = -h; break;
    case 1: c = c1; sn = s1; break;
    case 3: c = s1; sn = c1; break;
    case 5: c = -s1; sn = c1; break;
    case 7: c = -c1; sn = s1; break;
    case 9: c = -c1; sn = -s1; break;
    case 11: c = -s1; sn = -c1; break;
    case 13: c = s1; sn = -c1; break;
    default: c = c1; sn = -s1; break;  // 15
  }
  if (!INV) sn = -sn;
  return make_float2(fmaf(a.x, c, -a.y * sn), fmaf(a.x, sn, a.y * c));
}

// ------------------------------------------- packed FP32 pairs (f32x2)
// Blackwell's packed single-precision instructions (add/sub/mul/fma.rn.f32x2)
// apply one IEEE FP32 operation to both halves of a 64-bit register pair, so
// two independent lines transformed side by side cost one instruction per
// operation instead of two.  A float2 here is such a pair: .x belongs to the
// first line, .y to the second.  Every operation rounds exactly as its scalar
// counterpart, so the paired transform gives the scalar transform's bits.
PTYG_DEV float2 padd(float2 a, float2 b) {
  float2 r;
  asm("{\n.reg .b64 ra, rb, rd;\nmov.b64 ra, {%2, %3};\nmov.b64 rb, {%4, %5};\n"
      "add.rn.f32x2 rd, ra, rb;\nmov.b64 {%0, %1}, rd;\n}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
PTYG_DEV float2 psub(float2 a, float2 b) {
  float2 r;
  asm("{\n.reg .b64 ra, rb, rd;\nmov.b64 ra, {%2, %3};\nmov.b64 rb, {%4, %5};\n"
      "sub.rn.f32x2 rd, ra, rb;\nmov.b64 {%0, %1}, rd;\n}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
PTYG_DEV float2 pmul(float2 a, float2 b) {
  float2 r;
  asm("{\n.reg .b64 ra, rb, rd;\nmov.b64 ra, {%2, %3};\nmov.b64 rb, {%4, %5};\n"
      "mul.rn.f32x2 rd, ra, rb;\nmov.b64 {%0, %1}, rd;\n}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
// a * b + c, fused (one rounding), per half
PTYG_DEV float2 pfma(float2 a, float2 b, float2 c) {
  float2 r;
  asm("{\n.reg .b64 ra, rb, rc, rd;\nmov.b64 ra, {%2, %3};\nmov.b64 rb, {%4, %5};\nmov.b64 rc, {%6, %7};\n"
      "fma.rn.f32x2 rd, ra, rb, rc;\nmov.b64 {%0, %1}, rd;\n}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return r;
}
PTYG_DEV float2 pdup(float v) { return make_float2(v, v); }
// exact negation of both halves (-1 * x, signed zeros included)
PTYG_DEV float2 pneg(float2 a) { return pmul(a, pdup(-1.f)); }

// Two complex values, one per line, as a pair of real parts and a pair of
// imaginary parts.
struct CPair {
  float2 re, im;
};

// a * w (cmul's rounding) for a twiddle w shared by both lines; wx, wy, nwy
// are the pairs (w.x, w.x), (w.y, w.y), (-w.y, -w.y)
PTYG_DEV CPair pcmul(CPair a, float2 wx, float2 wy, float2 nwy) {
  return {pfma(a.re, wx, pmul(a.im, nwy)), pfma(a.re, wy, pmul(a.im, wx))};
}
// conj(w) * a (cmulc's rounding)
PTYG_DEV CPair pcmulc(CPair a, float2 wx, float2 wy, float2 nwy) {
  return {pfma(wx, a.re, pmul(wy, a.im)), pfma(wx, a.im, pmul(nwy, a.re))};
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

// In-register E-point DFT (E <= 16), natural order in and out: radix-2
// decimation in frequency, then a compile-time bit reversal (register renaming).
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
          v[start + m + span] = mul_w16<INV>(csub(a, b), m * (16 / (2 * span)));
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

// mul_w16 on a pair of lines (the same rounding and signs)
template <bool INV>
PTYG_DEV CPair pmul_w16(CPair a, int m) {
  const float c1 = 0.92387953251128674f;  // cos(pi/8)
  const float s1 = 0.38268343236508978f;  // sin(pi/8)
  const float h = 0.70710678118654752f;   // sqrt(1/2)
  float c, sn;
  switch (m & 15) {
    case 0: return a;
    case 4: return INV ? CPair{pneg(a.im), a.re} : CPair{a.im, pneg(a.re)};
    case 8: return CPair{pneg(a.re), pneg(a.im)};
    case 12: return INV ? CPair{a.im, pneg(a.re)} : CPair{pneg(a.im), a.re};
    case 2: c = h; sn = h; break;
    case 6: c = -h; sn = h; break;
    case 10: c = -h; sn = -h; break;
    case 14: c = h; sn = -h; break;
    case 1: c = c1; sn = s1; break;
    case 3: c = s1; sn = c1; break;
    case 5: c = -s1; sn = c1; break;
    case 7: c = -c1; sn = s1; break;
    case 9: c = -c1; sn = -s1; break;
    case 11: c = -s1; sn = -c1; break;
    case 13: c = s1; sn = -c1; break;
    default: c = c1; sn = -s1; break;  // 15
  }
  if (!INV) sn = -sn;
  return {pfma(a.re, pdup(c), pmul(a.im, pdup(-sn))), pfma(a.re, pdup(sn), pmul(a.im, pdup(c)))};
}

// dft_reg on a pair of lines
template <int E, bool INV>
PTYG_DEV void pdft_reg(CPair (&v)[E]) {
  if constexpr (E > 1) {
#pragma unroll
    for (int span = E / 2; span >= 1; span >>= 1) {
#pragma unroll
      for (int start = 0; start < E; start += 2 * span) {
#pragma unroll
        for (int m = 0; m < span; ++m) {
          const CPair a = v[start + m];
          const CPair b = v[start + m + span];
          v[start + m] = CPair{padd(a.re, b.re), padd(a.im, b.im)};
          v[start + m + span] = pmul_w16<INV>(CPair{psub(a.re, b.re), psub(a.im, b.im)}, m * (16 / (2 * span)));
        }
      }
    }
    CPair t[E];
#pragma unroll
    for (int i = 0; i < E; ++i) t[i] = v[i];
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = t[rev_bits<E>(i)];
  }
}

// One warp transforms one line of N = 32*E points (see the layout note at the
// top).  Per-lane twiddles live in registers for the life of the object:
// W_N^(lane*k1) for k1 = 1..E-1, and for the cross-lane stages h = 16, 8, 4
// W_(2h)^(lane mod h) on upper lanes (1 on lower lanes).  Stage h = 2 needs
// only the rotation by -i and stage h = 1 no twiddle at all.
template <int E>
struct WarpFFT {
  float2 tl[E > 1 ? E - 1 : 1];
  float2 ts[3];
  unsigned lane;

  // `tw` is the N-entry table W_N^m (global or shared memory).
  PTYG_DEV void init(const float2* tw, unsigned ln) {
    lane = ln;
#pragma unroll
    for (int k = 1; k < E; ++k) tl[k - 1] = tw[lane * k];
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      const int h = 16 >> s;
      ts[s] = (lane & h) ? tw[(lane & (h - 1)) * (16 * E / h)] : make_float2(1.f, 0.f);
    }
  }

  // natural -> Fourier layout, unnormalised, exp(-i...), on M lines at once
  // (independent lines interleave, hiding shuffle latency)
  template <int M>
  PTYG_DEV void fwdm(float2 (&v)[M][E]) const {
#pragma unroll
    for (int m = 0; m < M; ++m) {
      dft_reg<E, false>(v[m]);
#pragma unroll
      for (int k = 1; k < E; ++k) v[m][k] = cmul(v[m][k], tl[k - 1]);
    }
#pragma unroll
    for (int s = 0; s < 5; ++s) {
      const int h = 16 >> s;
      const float sg = (lane & h) ? -1.f : 1.f;
      const bool rot = (s == 3) && (lane & 2) && (lane & 1);
#pragma unroll
      for (int r = 0; r < E; ++r) {
#pragma unroll
        for (int m = 0; m < M; ++m) {
          float2 o;
          o.x = __shfl_xor_sync(0xffffffffu, v[m][r].x, h);
          o.y = __shfl_xor_sync(0xffffffffu, v[m][r].y, h);
          // lower lane: mine + other ; upper lane: (other - mine) * w
          float2 t = make_float2(fmaf(sg, v[m][r].x, o.x), fmaf(sg, v[m][r].y, o.y));
          if (s < 3) t = cmul(t, ts[s]);
          else if (s == 3) t = rot ? make_float2(t.y, -t.x) : t;
          v[m][r] = t;
        }
      }
    }
  }

  // Fourier layout -> natural, unnormalised, exp(+i...), on M lines at once
  template <int M>
  PTYG_DEV void invm(float2 (&v)[M][E]) const {
#pragma unroll
    for (int s = 4; s >= 0; --s) {
      const int h = 16 >> s;
      const bool upper = (lane & h) != 0;
      const float sg = upper ? -1.f : 1.f;
      const bool rot = (s == 3) && upper && (lane & 1);
#pragma unroll
      for (int r = 0; r < E; ++r) {
#pragma unroll
        for (int m = 0; m < M; ++m) {
          // the upper lane pre-multiplies its own value by conj(w); then
          // lower: mine + other ; upper: other - mine
          float2 c = v[m][r];
          if (s < 3) c = cmulc(ts[s], c);
          else if (s == 3) c = rot ? make_float2(-c.y, c.x) : c;
          float2 o;
          o.x = __shfl_xor_sync(0xffffffffu, c.x, h);
          o.y = __shfl_xor_sync(0xffffffffu, c.y, h);
          v[m][r] = make_float2(fmaf(sg, c.x, o.x), fmaf(sg, c.y, o.y));
        }
      }
    }
#pragma unroll
    for (int m = 0; m < M; ++m) {
#pragma unroll
      for (int k = 1; k < E; ++k) v[m][k] = cmulc(tl[k - 1], v[m][k]);
      dft_reg<E, true>(v[m]);
    }
  }

  // Two lines at once with packed FP32 pairs: the operations and roundings of
  // fwdm / invm, one paired instruction per two scalar ones.  The per-lane
  // twiddles tl multiply one register of each line, so they stay scalar.
  PTYG_DEV void fwd2(float2 (&v)[2][E]) const {
    CPair p[E];
#pragma unroll
    for (int j = 0; j < E; ++j) p[j] = CPair{make_float2(v[0][j].x, v[1][j].x), make_float2(v[0][j].y, v[1][j].y)};
    pdft_reg<E, false>(p);
#pragma unroll
    for (int k = 1; k < E; ++k) {
      const float2 a0 = cmul(make_float2(p[k].re.x, p[k].im.x), tl[k - 1]);
      const float2 a1 = cmul(make_float2(p[k].re.y, p[k].im.y), tl[k - 1]);
      p[k] = CPair{make_float2(a0.x, a1.x), make_float2(a0.y, a1.y)};
    }
#pragma unroll
    for (int s = 0; s < 5; ++s) {
      const int h = 16 >> s;
      const float2 sg = pdup((lane & h) ? -1.f : 1.f);
      const bool rot = (s == 3) && (lane & 2) && (lane & 1);
      float2 wx, wy, nwy;
      if (s < 3) {
        wx = pdup(ts[s].x);
        wy = pdup(ts[s].y);
        nwy = pdup(-ts[s].y);
      }
#pragma unroll
      for (int r = 0; r < E; ++r) {
        float2 ore, oim;
        ore.x = __shfl_xor_sync(0xffffffffu, p[r].re.x, h);
        ore.y = __shfl_xor_sync(0xffffffffu, p[r].re.y, h);
        oim.x = __shfl_xor_sync(0xffffffffu, p[r].im.x, h);
        oim.y = __shfl_xor_sync(0xffffffffu, p[r].im.y, h);
        // lower lane: mine + other ; upper lane: (other - mine) * w
        CPair t{pfma(sg, p[r].re, ore), pfma(sg, p[r].im, oim)};
        if (s < 3) t = pcmul(t, wx, wy, nwy);
        else if (s == 3 && rot) t = CPair{t.im, pneg(t.re)};
        p[r] = t;
      }
    }
#pragma unroll
    for (int j = 0; j < E; ++j) {
      v[0][j] = make_float2(p[j].re.x, p[j].im.x);
      v[1][j] = make_float2(p[j].re.y, p[j].im.y);
    }
  }

  PTYG_DEV void inv2(float2 (&v)[2][E]) const {
    CPair p[E];
#pragma unroll
    for (int j = 0; j < E; ++j) p[j] = CPair{make_float2(v[0][j].x, v[1][j].x), make_float2(v[0][j].y, v[1][j].y)};
#pragma unroll
    for (int s = 4; s >= 0; --s) {
      const int h = 16 >> s;
      const bool upper = (lane & h) != 0;
      const float2 sg = pdup(upper ? -1.f : 1.f);
      const bool rot = (s == 3) && upper && (lane & 1);
      float2 wx, wy, nwy;
      if (s < 3) {
        wx = pdup(ts[s].x);
        wy = pdup(ts[s].y);
        nwy = pdup(-ts[s].y);
      }
#pragma unroll
      for (int r = 0; r < E; ++r) {
        // the upper lane pre-multiplies its own value by conj(w); then
        // lower: mine + other ; upper: other - mine
        CPair c = p[r];
        if (s < 3) c = pcmulc(c, wx, wy, nwy);
        else if (s == 3 && rot) c = CPair{pneg(c.im), c.re};
        float2 ore, oim;
        ore.x = __shfl_xor_sync(0xffffffffu, c.re.x, h);
        ore.y = __shfl_xor_sync(0xffffffffu, c.re.y, h);
        oim.x = __shfl_xor_sync(0xffffffffu, c.im.x, h);
        oim.y = __shfl_xor_sync(0xffffffffu, c.im.y, h);
        p[r] = CPair{pfma(sg, c.re, ore), pfma(sg, c.im, oim)};
      }
    }
#pragma unroll
    for (int k = 1; k < E; ++k) {
      const float2 a0 = cmulc(tl[k - 1], make_float2(p[k].re.x, p[k].im.x));
      const float2 a1 = cmulc(tl[k - 1], make_float2(p[k].re.y, p[k].im.y));
      p[k] = CPair{make_float2(a0.x, a1.x), make_float2(a0.y, a1.y)};
    }
    pdft_reg<E, true>(p);
#pragma unroll
    for (int j = 0; j < E; ++j) {
      v[0][j] = make_float2(p[j].re.x, p[j].im.x);
      v[1][j] = make_float2(p[j].re.y, p[j].im.y);
    }
  }

  PTYG_DEV void fwd(float2 (&v)[E]) const { fwdm<1>(reinterpret_cast<float2(&)[1][E]>(v)); }
  PTYG_DEV void inv(float2 (&v)[E]) const { invm<1>(reinterpret_cast<float2(&)[1][E]>(v)); }
};

// 128-point lines, four per warp, with one shared-memory exchange.
//
// Lanes 16P .. 16P+15 (line pair P = lane / 16) hold lines 2P and 2P+1 as
// the two halves of packed FP32 pairs (CPair), 8 points per thread:
//   natural layout   : thread u = lane % 16, register a  <->  n = u + 16 a
//   frequency layout : thread v = lane % 16, register d  <->  k = v + 16 d
// so the frequency layout is plain frequency order, read and written by the
// same 16-consecutive-index pattern as the natural one.  With n = u + 16 a and
// k = b + 8 e + 16 d (b < 8, e < 2, d < 8):
//   W128^(nk) = W8^(ab) W128^(ub) W16^(ie) W2^(he) W8^(id),  u = i + 8 h.
// The forward transform is an 8-point DFT over a in registers, the twiddle
// W128^(ub), an exchange through shared memory that gives thread v = b + 8 h
// the values Y[i + 8h][b] (i < 8), a radix-2 butterfly between lanes v and
// v ^ 8 (h -> e), the twiddle W16^(ie) on e = 1, and an 8-point DFT over i.
// The inverse is its exact mirror with conjugate twiddles (unnormalised:
// inverse(forward(x)) = 128 x).
//
// The exchange uses 128 16-byte entries per line pair (a CPair: both lines'
// real parts, then both imaginary parts), e.g. the pair's own two line
// buffers when the lines are transformed in place: Y[u][b] sits in entry
// 16 b + (u ^ b), so that the writes (lanes over u) and the reads (lanes over
// (b, h): entry 16 b + (v ^ i)) each touch 8 distinct 16-byte bank groups per
// quarter-warp.
struct Fft128 {
  float2 tw[7];  // W128^(u * b), b = 1..7
  unsigned lane;

  // `table` is the 128-entry table W128^m (global or shared memory).
  PTYG_DEV void init(const float2* table, unsigned ln) {
    lane = ln;
    const int u = (int)(ln & 15);
#pragma unroll
    for (int b = 1; b < 8; ++b) tw[b - 1] = table[(u * b) & 127];
  }

  template <bool INV>
  PTYG_DEV void exchange(CPair (&p)[8], float4* xs) const {
    const int u = (int)(lane & 15), b = u & 7;
    float4* wr = INV ? xs + 16 * b : xs;  // write side: entry 16 j + (u ^ j) (fwd), 16 b + (u ^ j) (inv)
    float4* rd = INV ? xs : xs + 16 * b;
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int e = (INV ? 0 : 16 * j) + (u ^ j);
      wr[e] = make_float4(p[j].re.x, p[j].re.y, p[j].im.x, p[j].im.y);
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int e = (INV ? 16 * j : 0) + (u ^ j);
      const float4 z = rd[e];
      p[j] = CPair{make_float2(z.x, z.y), make_float2(z.z, z.w)};
    }
    __syncwarp();
  }

  // radix-2 between lanes v and v ^ 8: lower mine + other, upper other - mine
  PTYG_DEV void cross(CPair (&p)[8]) const {
    const float2 sg = pdup((lane & 8) ? -1.f : 1.f);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float2 ore, oim;
      ore.x = __shfl_xor_sync(0xffffffffu, p[j].re.x, 8);
      ore.y = __shfl_xor_sync(0xffffffffu, p[j].re.y, 8);
      oim.x = __shfl_xor_sync(0xffffffffu, p[j].im.x, 8);
      oim.y = __shfl_xor_sync(0xffffffffu, p[j].im.y, 8);
      p[j] = CPair{pfma(sg, p[j].re, ore), pfma(sg, p[j].im, oim)};
    }
  }

  PTYG_DEV void fwd(CPair (&p)[8], float4* xs) const {
    pdft_reg<8, false>(p);
#pragma unroll
    for (int b = 1; b < 8; ++b) p[b] = pcmul(p[b], pdup(tw[b - 1].x), pdup(tw[b - 1].y), pdup(-tw[b - 1].y));
    exchange<false>(p, xs);
    cross(p);
    if (lane & 8) {
#pragma unroll
      for (int i = 1; i < 8; ++i) p[i] = pmul_w16<false>(p[i], i);
    }
    pdft_reg<8, false>(p);
  }

  PTYG_DEV void inv(CPair (&p)[8], float4* xs) const {
    pdft_reg<8, true>(p);
    if (lane & 8) {
#pragma unroll
      for (int i = 1; i < 8; ++i) p[i] = pmul_w16<true>(p[i], i);
    }
    cross(p);
    exchange<true>(p, xs);
#pragma unroll
    for (int b = 1; b < 8; ++b) p[b] = pcmulc(p[b], pdup(tw[b - 1].x), pdup(tw[b - 1].y), pdup(-tw[b - 1].y));
    pdft_reg<8, true>(p);
  }
};

// Fourier-plane slot order of the line transforms, per axis, for lines of Np
// points.  Rows (x) at Np = 128 use Fft128: slot = frequency.  Columns (y),
// and rows at other sizes, use WarpFFT: slot 32 r + l holds k = r + E bitrev5(l).
__host__ __device__ inline int slot_bitrev5(int l) {
  int r = 0;
  for (int b = 0; b < 5; ++b) r |= ((l >> b) & 1) << (4 - b);
  return r;
}
__host__ __device__ inline int slot_to_freq_y(int s, int Np) {
  return (s >> 5) + (Np / 32) * slot_bitrev5(s & 31);
}
__host__ __device__ inline int freq_to_slot_y(int k, int Np) {
  const int E = Np / 32;
  return 32 * (k % E) + slot_bitrev5(k / E);
}
__host__ __device__ inline int slot_to_freq_x(int s, int Np) { return Np == 128 ? s : slot_to_freq_y(s, Np); }
__host__ __device__ inline int freq_to_slot_x(int k, int Np) { return Np == 128 ? k : freq_to_slot_y(k, Np); }

// Run `ntasks` independent line transforms over the warps of the CTA with
// WarpFFT, two per warp at a time.  Element-wise callbacks: load(task, lo,
// hi) returns element lo + hi of the line (natural index for the forward
// transform, Fourier slot for the inverse), store(task, lo, hi, value) takes
// element lo + hi of the result (slot, resp. natural index); lo = lane is the
// thread's part of the index and hi = 32 j a compile-time multiple of 32, so
// callers can keep addresses affine.  A __syncwarp separates the loads of a
// pair from its stores, so a task may store in place of what it loaded.
template <int E, bool INV, class LoadF, class StoreF>
PTYG_DEV void fft_tasks(const WarpFFT<E>& F, int ntasks, LoadF&& load, StoreF&& store) {
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int lane = threadIdx.x & 31;
  int t = warp;
  for (; t + nw < ntasks; t += 2 * nw) {
    float2 v[2][E];
#pragma unroll
    for (int j = 0; j < E; ++j) {
      v[0][j] = load(t, lane, 32 * j);
      v[1][j] = load(t + nw, lane, 32 * j);
    }
    if (INV)
      F.inv2(v);
    else
      F.fwd2(v);
    __syncwarp();
#pragma unroll
    for (int j = 0; j < E; ++j) {
      store(t, lane, 32 * j, v[0][j]);
      store(t + nw, lane, 32 * j, v[1][j]);
    }
  }
  if (t < ntasks) {
    float2 v[E];
#pragma unroll
    for (int j = 0; j < E; ++j) v[j] = load(t, lane, 32 * j);
    if (INV)
      F.inv(v);
    else
      F.fwd(v);
    __syncwarp();
#pragma unroll
    for (int j = 0; j < E; ++j) store(t, lane, 32 * j, v[j]);
  }
}

// Row transforms: at Np = 128 with Fft128, four lines per warp (ntasks must
// be a multiple of 4), lo = lane % 16 and hi = 16 a; `pairs(t)` (t even) is
// the 128-entry exchange buffer of lines t and t + 1 (their own two row
// buffers when transformed in place: every load of a line pair precedes its
// first exchange write).  Other sizes run fft_tasks with WarpFFT.
template <int E, bool INV, class LoadF, class StoreF, class PairF>
PTYG_DEV void row_tasks(const float2* twiddle, int ntasks, LoadF&& load, StoreF&& store, PairF&& pairs) {
  const int lane = threadIdx.x & 31;
  if constexpr (E == 4) {
    Fft128 F;
    F.init(twiddle, (unsigned)lane);
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int P = lane >> 4, u = lane & 15;
    for (int g = warp; 4 * g < ntasks; g += nw) {
      const int t0 = 4 * g + 2 * P, t1 = t0 + 1;
      CPair p[8];
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        const float2 x0 = load(t0, u, 16 * a), x1 = load(t1, u, 16 * a);
        p[a] = CPair{make_float2(x0.x, x1.x), make_float2(x0.y, x1.y)};
      }
      if (INV)
        F.inv(p, pairs(t0));
      else
        F.fwd(p, pairs(t0));
#pragma unroll
      for (int d = 0; d < 8; ++d) {
        store(t0, u, 16 * d, make_float2(p[d].re.x, p[d].im.x));
        store(t1, u, 16 * d, make_float2(p[d].re.y, p[d].im.y));
      }
    }
  } else {
    WarpFFT<E> F;
    F.init(twiddle, (unsigned)lane);
    fft_tasks<E, INV>(F, ntasks, load, store);
  }
}

// Index helpers for the two layouts.
template <int E>
PTYG_DEV int fourier_index(int r, unsigned lane) {
  return r + E * (int)bitrev5(lane);
}

}  // namespace ptyg
