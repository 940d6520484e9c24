// ptyg_propagate_noalloc: the propagators of ptyg_propagate for callers that
// cannot allocate GPU memory -- code running inside a host framework that owns
// every device allocation (a memory pool or arena it does not expose), a
// real-time acquisition callback where cudaMalloc's implicit device
// synchronisation would stall the detector pipeline, or a process that has
// pre-reserved all of HBM for its own buffers.  The caller passes input and
// output; the transposition scratch between the row and column passes is a
// fixed array compiled into this library instead of memory from cudaMalloc.
//
// Limit: batch * Np * Np <= PTYG_NOALLOC_MAX_POINTS (1,048,576 complex64 points,
// 8 MiB), e.g. 64 fields of 128 x 128 or 16 of 256 x 256.  Every GPU that
// loads the library holds these 8 MiB (plus 3.75 KiB of twiddle tables) until
// the process exits.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "../../include/ptyg.h"
#include "ptyg_ops.cuh"

#define PTYG_NOALLOC_MAX_POINTS (1 << 20)

namespace {

// Scratch shared by every call on a device; holds the last call's data.
static __device__ __align__(256) float2 g_noalloc_scratch[PTYG_NOALLOC_MAX_POINTS];
// Twiddle tables W_N^m for N = 32, 64, 128, 256 at offsets 0, 32, 96, 224.
static __device__ __align__(256) float2 g_noalloc_twiddles[32 + 64 + 128 + 256];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
float2* g_scratch_ptr[kMaxDevices] = {};
float2* g_twiddle_ptr[kMaxDevices] = {};

// Errors are reported through ptyg_last_error(), like every other entry point.
int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return ptyg::set_last_error(code, buf);
}

int twiddle_offset(int Np) { return Np == 32 ? 0 : Np == 64 ? 32 : Np == 128 ? 96 : 224; }

// Once per device, with that device current: check that it is an sm_103a GPU
// (as ptyg_device_init does for every other entry point), resolve the device
// addresses of the static arrays (host code may not use the symbols directly)
// and fill the twiddle tables.  cudaMemcpyToSymbol is synchronous, so the
// first call on a device must not be made while a stream is being captured.
// The addresses are cached for the life of the process: after a
// cudaDeviceReset they are stale, and this entry point must not be used again.
int setup(int dev) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_scratch_ptr[dev]) return PTYG_OK;
  int major = 0, minor = 0;
  cudaError_t ea = cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  if (ea == cudaSuccess) ea = cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  if (ea != cudaSuccess) return fail(PTYG_ERR_DEVICE, "no CUDA device: %s", cudaGetErrorString(ea));
  if (major != 10 || minor != 3)
    return fail(PTYG_ERR_DEVICE, "device %d is sm_%d%d; libptyg is built for sm_103a only", dev, major, minor);
  void* scratch = nullptr;
  void* tw = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&scratch, g_noalloc_scratch);
  if (e != cudaSuccess) return fail(PTYG_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
  e = cudaGetSymbolAddress(&tw, g_noalloc_twiddles);
  if (e != cudaSuccess) return fail(PTYG_ERR_CUDA, "cudaGetSymbolAddress(twiddles): %s", cudaGetErrorString(e));
  float2 host[32 + 64 + 128 + 256];
  const double pi = 3.14159265358979323846;
  for (int N = 32; N <= 256; N *= 2)
    for (int m = 0; m < N; ++m) {
      const double a = -2.0 * pi * (double)m / (double)N;
      host[twiddle_offset(N) + m] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
  e = cudaMemcpyToSymbol(g_noalloc_twiddles, host, sizeof(host));
  if (e != cudaSuccess) return fail(PTYG_ERR_CUDA, "cudaMemcpyToSymbol(twiddles): %s", cudaGetErrorString(e));
  g_twiddle_ptr[dev] = (float2*)tw;
  g_scratch_ptr[dev] = (float2*)scratch;
  return PTYG_OK;
}

}  // namespace

extern "C" int ptyg_propagate_noalloc(int propagator, int direction, int fftshift, int Np, int batch, const void* in,
                                      void* out, const void* table, void* stream) {
  if (!(Np == 32 || Np == 64 || Np == 128 || Np == 256))
    return fail(PTYG_ERR_UNSUPPORTED, "Np=%d: supported sizes are 32, 64, 128, 256", Np);
  if (batch < 0) return fail(PTYG_ERR_INVALID, "batch=%d", batch);
  if ((long long)batch * Np * Np > PTYG_NOALLOC_MAX_POINTS)
    return fail(PTYG_ERR_INVALID,
                "batch*Np*Np = %lld exceeds the %d complex64 points of the built-in scratch (8 MiB); "
                "split the batch or use ptyg_propagate",
                (long long)batch * Np * Np, PTYG_NOALLOC_MAX_POINTS);
  if (batch == 0) return PTYG_OK;
  if (!in || !out) return fail(PTYG_ERR_INVALID, "null field pointer");
  if (direction != PTYG_FORWARD && direction != PTYG_INVERSE) return fail(PTYG_ERR_INVALID, "direction=%d", direction);
  if (propagator < PTYG_FRAUNHOFER || propagator > PTYG_ASP)
    return fail(PTYG_ERR_UNSUPPORTED, "propagator %d is not on this path", propagator);
  if ((propagator == PTYG_FRESNEL || propagator == PTYG_ASP) && !table)
    return fail(PTYG_ERR_INVALID, "propagator %d needs its table", propagator);
  if (propagator == PTYG_ASP && fftshift)
    return fail(PTYG_ERR_INVALID, "ASP propagator only works with fftshiftSwitch == False");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(PTYG_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(PTYG_ERR_DEVICE, "device %d out of range", dev);
  int r = setup(dev);
  if (r) return r;
  cudaStream_t st = (cudaStream_t)stream;
  const float2* tw = g_twiddle_ptr[dev] + twiddle_offset(Np);
  float2* tmp = g_scratch_ptr[dev];
  const float2* src = (const float2*)in;
  float2* dst = (float2*)out;
  const float2* tab = (const float2*)table;
  const bool inv = direction == PTYG_INVERSE;
  const bool centred = !fftshift;
  if (propagator == PTYG_FRAUNHOFER || propagator == PTYG_FRESNEL) {
    ptyg::RowOp ro = {};
    ro.inverse = inv;
    ro.preSign = centred;
    ro.scale = 1.f;
    if (propagator == PTYG_FRESNEL && !inv) ro.pre = tab;
    ptyg::ColOp co = {};
    co.inverse1 = inv;
    co.postSign = centred;
    co.scale = 1.f / (float)Np;
    if (propagator == PTYG_FRESNEL && inv) {
      co.post = tab;
      co.conjPost = 1;
    }
    e = ptyg::prop_rows(Np, src, tmp, batch, ro, tw, st);
    if (e == cudaSuccess) e = ptyg::prop_cols(Np, tmp, dst, batch, co, tw, st);
  } else {
    ptyg::RowOp r1 = {};
    r1.scale = 1.f;
    ptyg::ColOp co = {};
    co.filter = tab;
    co.conjFilter = inv;
    co.filterScale = 1.f / (float)(Np * Np);
    co.inverse2 = 1;
    co.scale = 1.f;
    ptyg::RowOp r2 = {};
    r2.inverse = 1;
    r2.scale = 1.f;
    e = ptyg::prop_rows(Np, src, tmp, batch, r1, tw, st);
    if (e == cudaSuccess) e = ptyg::prop_cols(Np, tmp, tmp, batch, co, tw, st);
    if (e == cudaSuccess) e = ptyg::prop_rows(Np, tmp, dst, batch, r2, tw, st);
  }
  if (e != cudaSuccess) return fail(PTYG_ERR_CUDA, "ptyg_propagate_noalloc: %s", cudaGetErrorString(e));
  return PTYG_OK;
}
