// C ABI of libptyg.so (declared in include/ptyg.h).
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/ptyg.h"
#include "ptyg_common.cuh"
#include "ptyg_engine.cuh"
#include "ptyg_ops.cuh"

using ptyg::EngineArgs;
using ptyg::ScanDev;

// ------------------------------------------------------------------ errors
static thread_local std::string g_last_error;

static int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

namespace ptyg {
// Record a failure for ptyg_last_error() from other translation units.
int set_last_error(int code, const char* msg) {
  g_last_error = msg;
  return code;
}
}  // namespace ptyg

static int cuda_fail(cudaError_t e, const char* what) {
  if (e == cudaErrorMemoryAllocation) return fail(PTYG_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
  if (e == cudaErrorNotSupported) return fail(PTYG_ERR_UNSUPPORTED, "%s: configuration not supported", what);
  return fail(PTYG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define PTYG_CUDA(call, what)                    \
  do {                                           \
    cudaError_t e_ = (call);                     \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

static bool valid_np(int Np) { return Np == 32 || Np == 64 || Np == 128 || Np == 256; }

// ------------------------------------------------------- per-device tables
// W_N^m = exp(-2*pi*i*m/N), m = 0..N-1, built in double and rounded.  One set
// per device, in a fixed array (never resized, so readers need no lock); a set
// is published through its `ready` flag only once all four tables exist.
namespace {
constexpr int kMaxDevices = 64;
struct DeviceTables {
  float2* tw[4] = {nullptr, nullptr, nullptr, nullptr};  // N = 32, 64, 128, 256
  std::atomic<bool> ready{false};
};
std::mutex g_tables_mu;
DeviceTables g_tables[kMaxDevices];

int table_slot(int Np) { return Np == 32 ? 0 : Np == 64 ? 1 : Np == 128 ? 2 : 3; }

int ensure_tables(int device) {
  if (device < 0 || device >= kMaxDevices) return fail(PTYG_ERR_DEVICE, "device %d out of range", device);
  std::lock_guard<std::mutex> lk(g_tables_mu);
  DeviceTables& t = g_tables[device];
  if (t.ready.load(std::memory_order_acquire)) return PTYG_OK;
  const double pi = 3.14159265358979323846;
  float2* built[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaError_t e = cudaSuccess;
  for (int s = 0; s < 4 && e == cudaSuccess; ++s) {
    const int N = 32 << s;
    std::vector<float2> h(N);
    for (int m = 0; m < N; ++m) {
      const double ang = -2.0 * pi * (double)m / (double)N;
      h[m] = make_float2((float)std::cos(ang), (float)std::sin(ang));
    }
    e = cudaMalloc(&built[s], N * sizeof(float2));
    if (e == cudaSuccess) e = cudaMemcpy(built[s], h.data(), N * sizeof(float2), cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    for (float2* d : built)
      if (d) cudaFree(d);
    return cuda_fail(e, "twiddle table");
  }
  for (int s = 0; s < 4; ++s) t.tw[s] = built[s];
  t.ready.store(true, std::memory_order_release);
  return PTYG_OK;
}

int current_device(int* dev) {
  cudaError_t e = cudaGetDevice(dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  return PTYG_OK;
}

bool tables_ready(int device) {
  return device >= 0 && device < kMaxDevices && g_tables[device].ready.load(std::memory_order_acquire);
}

// Only called after tables_ready(device) (ready_device or ptyg_device_init succeeded).
const float2* twiddles(int device, int Np) { return g_tables[device].tw[table_slot(Np)]; }
}  // namespace

extern "C" int ptyg_version(void) { return PTYG_VERSION; }

extern "C" const char* ptyg_last_error(void) { return g_last_error.c_str(); }

extern "C" int ptyg_device_init(int device) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return fail(PTYG_ERR_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
  if (device < 0 || device >= n) return fail(PTYG_ERR_INVALID, "device %d out of range (%d devices)", device, n);
  PTYG_CUDA(cudaSetDevice(device), "cudaSetDevice");
  cudaDeviceProp prop;
  PTYG_CUDA(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
  if (prop.major != 10 || prop.minor != 3)
    return fail(PTYG_ERR_DEVICE, "device %d is sm_%d%d; libptyg is built for sm_103a only", device, prop.major,
                prop.minor);
  return ensure_tables(device);
}

static int ready_device(int* dev) {
  int r = current_device(dev);
  if (r) return r;
  if (!tables_ready(*dev)) {
    r = ptyg_device_init(*dev);
    if (r) return r;
  }
  return PTYG_OK;
}

// ------------------------------------------------------------ propagators
extern "C" int ptyg_propagate(int propagator, int direction, int fftshift, int Np, int batch, const void* in,
                              void* out, const void* table, void* scratch, void* stream) {
  if (!valid_np(Np)) return fail(PTYG_ERR_UNSUPPORTED, "Np=%d: supported sizes are 32, 64, 128, 256", Np);
  if (batch < 0) return fail(PTYG_ERR_INVALID, "batch=%d", batch);
  if (batch == 0) return PTYG_OK;
  if (!in || !out) return fail(PTYG_ERR_INVALID, "null field pointer");
  if (direction != PTYG_FORWARD && direction != PTYG_INVERSE) return fail(PTYG_ERR_INVALID, "direction=%d", direction);
  if ((propagator == PTYG_FRESNEL || propagator == PTYG_ASP) && !table)
    return fail(PTYG_ERR_INVALID, "propagator %d needs its table", propagator);
  if (propagator == PTYG_ASP && fftshift)
    return fail(PTYG_ERR_INVALID, "ASP propagator only works with fftshiftSwitch == False");
  if (propagator < PTYG_FRAUNHOFER || propagator > PTYG_ASP)
    return fail(PTYG_ERR_UNSUPPORTED, "propagator %d is not on this path", propagator);
  int dev;
  int r = ready_device(&dev);
  if (r) return r;
  cudaStream_t st = (cudaStream_t)stream;
  const float2* tw = twiddles(dev, Np);
  const float2* src = (const float2*)in;
  float2* dst = (float2*)out;
  float2* tmp = (float2*)scratch;
  bool own = false;
  if (!tmp) {
    PTYG_CUDA(cudaMallocAsync((void**)&tmp, (size_t)batch * Np * Np * sizeof(float2), st), "propagate scratch");
    own = true;
  }
  const bool inv = direction == PTYG_INVERSE;
  const bool centred = !fftshift;
  const float2* tab = (const float2*)table;
  cudaError_t e = cudaSuccess;
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
    co.inverse1 = 0;
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
  if (own) {
    cudaError_t e2 = cudaFreeAsync(tmp, st);
    if (e == cudaSuccess) e = e2;
  }
  if (e != cudaSuccess) return cuda_fail(e, "ptyg_propagate");
  return PTYG_OK;
}

// With N = Np, F / I the unnormalised forward / inverse DFT and M the
// checkerboard (-1)^(y+x): fft2c(x) = M F(M x) / N and ifft2c(X) = M I(M X) / N,
// and M T M = T for any elementwise table T, so
//   ifft2c(fft2c(x) * T) = M I(T F(M x)) / N^2:
// a row pass (sign, forward), a column pass (forward, * T / N^2, inverse)
// and a row pass (inverse, sign), the tables applied on the way in or out.
extern "C" int ptyg_propagate_sets(int propagator, int direction, int Np, int batch, int nsets, const void* in,
                                   void* out, const void* table_a, const void* table_b, void* scratch,
                                   void* stream) {
  if (!valid_np(Np)) return fail(PTYG_ERR_UNSUPPORTED, "Np=%d: supported sizes are 32, 64, 128, 256", Np);
  if (batch < 0) return fail(PTYG_ERR_INVALID, "batch=%d", batch);
  if (nsets < 1 || batch % nsets != 0)
    return fail(PTYG_ERR_INVALID, "nsets=%d must be >= 1 and divide batch=%d", nsets, batch);
  if (direction != PTYG_FORWARD && direction != PTYG_INVERSE) return fail(PTYG_ERR_INVALID, "direction=%d", direction);
  if (propagator < PTYG_POLYCHROME_ASP || propagator > PTYG_IDENTITY)
    return fail(PTYG_ERR_UNSUPPORTED, "propagator %d is not a ptyg_propagate_sets propagator", propagator);
  if (propagator == PTYG_SCALED_ASP && nsets != 1) return fail(PTYG_ERR_INVALID, "SCALED_ASP takes one table set");
  const bool needA = propagator != PTYG_IDENTITY;
  const bool needB = propagator == PTYG_SCALED_ASP || propagator == PTYG_SCALED_POLYCHROME_ASP ||
                     propagator == PTYG_TWO_STEP_POLYCHROME;
  if ((needA && !table_a) || (needB && !table_b)) return fail(PTYG_ERR_INVALID, "propagator %d needs its tables", propagator);
  if (batch == 0) return PTYG_OK;
  if (!in || !out) return fail(PTYG_ERR_INVALID, "null field pointer");
  int dev;
  int r = ready_device(&dev);
  if (r) return r;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t bytes = (size_t)batch * Np * Np * sizeof(float2);
  if (propagator == PTYG_IDENTITY) {
    if (in != out) PTYG_CUDA(cudaMemcpyAsync(out, in, bytes, cudaMemcpyDeviceToDevice, st), "identity copy");
    return PTYG_OK;
  }
  const float2* tw = twiddles(dev, Np);
  float2* tmp = (float2*)scratch;
  bool own = false;
  if (!tmp) {
    PTYG_CUDA(cudaMallocAsync((void**)&tmp, bytes, st), "propagate scratch");
    own = true;
  }
  const bool inv = direction == PTYG_INVERSE;
  const int div = batch / nsets;  // fields per table set
  const float2* A = (const float2*)table_a;
  const float2* B = (const float2*)table_b;
  const float n2 = 1.f / (float)(Np * Np);

  ptyg::RowOp r1 = {};  // sign, forward
  r1.preSign = 1;
  r1.scale = 1.f;
  ptyg::ColOp co = {};  // forward, * T / N^2, inverse
  co.filterScale = n2;
  co.inverse2 = 1;
  co.scale = 1.f;
  co.filterDiv = div;
  co.conjFilter = inv;
  ptyg::RowOp r2 = {};  // inverse, sign
  r2.inverse = 1;
  r2.postSign = 1;
  r2.scale = 1.f;
  bool secondFft = false;
  switch (propagator) {
    case PTYG_POLYCHROME_ASP:
      co.filter = A;
      break;
    case PTYG_SCALED_ASP:
    case PTYG_SCALED_POLYCHROME_ASP:
      co.filter = B;
      if (!inv) {
        r1.pre = A;
        r1.preDiv = div;
      } else {
        r2.post = A;
        r2.postDiv = div;
        r2.conjPost = 1;
      }
      break;
    case PTYG_TWO_STEP_POLYCHROME:
      co.filter = A;
      if (!inv) {
        // fft2c(ifft2c(fft2c(x) A) B) = M F(B I(A F(M x))) / N^3: no sign
        // between the halves (M M = 1), the chirp B after the inverse
        r2.postSign = 0;
        r2.post = B;
        secondFft = true;
      } else {
        r1.pre = B;
        r1.conjPre = 1;
      }
      break;
  }
  cudaError_t e = ptyg::prop_rows(Np, (const float2*)in, tmp, batch, r1, tw, st);
  if (e == cudaSuccess) e = ptyg::prop_cols(Np, tmp, tmp, batch, co, tw, st);
  if (!secondFft) {
    if (e == cudaSuccess) e = ptyg::prop_rows(Np, tmp, (float2*)out, batch, r2, tw, st);
  } else {
    ptyg::RowOp r3 = {};  // forward rows
    r3.scale = 1.f;
    ptyg::ColOp c2 = {};  // forward columns, sign, 1/N
    c2.postSign = 1;
    c2.scale = 1.f / (float)Np;
    // row passes never run in place (their pointers are __restrict__)
    if (e == cudaSuccess) e = ptyg::prop_rows(Np, tmp, (float2*)out, batch, r2, tw, st);
    if (e == cudaSuccess) e = ptyg::prop_rows(Np, (const float2*)out, tmp, batch, r3, tw, st);
    if (e == cudaSuccess) e = ptyg::prop_cols(Np, tmp, (float2*)out, batch, c2, tw, st);
  }
  if (own) {
    cudaError_t e2 = cudaFreeAsync(tmp, st);
    if (e == cudaSuccess) e = e2;
  }
  if (e != cudaSuccess) return cuda_fail(e, "ptyg_propagate_sets");
  return PTYG_OK;
}

// ------------------------------------------------------------------ plans
struct ScanOwned {
  float* data = nullptr;      // converted ptychogram
  float2* work = nullptr;
  float2* esw = nullptr;
  double* errPart = nullptr;
  double* err = nullptr;
  float* detErr = nullptr;
  float* tileMax = nullptr;
  float* background = nullptr;  // data layout
  double* iscale = nullptr;
  float2* reference = nullptr;  // interferometric: K planes, data layout
  unsigned* red = nullptr;
  int* status = nullptr;
  bool bound = false;
  int orderLen = 0;
  ptyg_scan_buffers buf = {};
};

struct ptyg_plan {
  ptyg_geometry g = {};
  int device = 0;
  int C = 1;
  int threads = 256;
  bool probeInSmem = true;
  bool hInSmem = false;  // ASP: the CTA's transfer-function columns in shared memory
  size_t smem = 0;
  float2* fresnelQ = nullptr;
  float2* aspH = nullptr;
  float2* sliceH = nullptr;
  ptyg_projection proj = {};
  float* W = nullptr;         // data layout
  float* imask = nullptr;     // data layout
  std::vector<ScanOwned> scans;
  ScanDev* dScans = nullptr;
  std::vector<ScanDev> hScans;
};

static void plan_free(ptyg_plan* p) {
  if (!p) return;
  cudaFree(p->fresnelQ);
  cudaFree(p->aspH);
  cudaFree(p->sliceH);
  cudaFree(p->W);
  cudaFree(p->imask);
  for (auto& s : p->scans) {
    cudaFree(s.background);
    cudaFree(s.reference);
    cudaFree(s.iscale);
    cudaFree(s.data);
    cudaFree(s.work);
    cudaFree(s.esw);
    cudaFree(s.errPart);
    cudaFree(s.err);
    cudaFree(s.detErr);
    cudaFree(s.tileMax);
    cudaFree(s.red);
    cudaFree(s.status);
  }
  cudaFree(p->dScans);
  delete p;
}

// Latency shape: one warp per 1D-transform task of a pass (K modes x L
// lines).  Throughput shape: one warp per two tasks (the line transforms run
// two per warp at a time), so a pass keeps every warp busy and smaller CTAs
// fit two or more to an SM, from different scans, hiding each other's
// barriers: at C3 (qNewton, one mode, Np 128) 36 scans at 256 threads ran
// 1.36 M positions*iterations/s against 15 scans at 512 threads, 0.92 M.
// 4..16 warps (mqNewton: 8, the bound its kernel is compiled for).
static int engine_threads(const ptyg_geometry& g, int C) {
  const int tasks = g.nlambda * g.nosm * g.npsm * (g.Np / C);
  const int want = g.throughput ? (tasks + 1) / 2 : tasks;
  const int wmax = g.engine == PTYG_MQNEWTON ? 8 : 16;
  const int w = want < 4 ? 4 : (want > wmax ? wmax : want);
  return 32 * w;
}

// Cluster sizes to try, best first.  Latency: 8 rows per CTA (more CTAs,
// shorter passes), then 16.  Throughput: 16 rows first (fewer CTAs per scan,
// so more scans are resident at once), and at Np = 64 the whole patch in one
// CTA before that.  A requested size goes first.
static std::vector<int> cluster_candidates(const ptyg_geometry& g) {
  std::vector<int> c;
  if (g.cluster > 0) c.push_back(g.cluster);
  if (g.throughput && g.Np == 64) c.push_back(1);
  const int order[2] = {g.throughput ? 16 : 8, g.throughput ? 8 : 16};
  for (int L : order) {
    const int cc = g.Np / L;
    if (cc >= 1 && cc <= 16) c.push_back(cc);
  }
  return c;
}

extern "C" int ptyg_plan_create(const ptyg_geometry* geometry, ptyg_plan** plan) {
  if (!geometry || !plan) return fail(PTYG_ERR_INVALID, "null argument");
  *plan = nullptr;
  ptyg_geometry g = *geometry;
  if (g.nlambda == 0) g.nlambda = 1;
  if (g.nlambda < 1) return fail(PTYG_ERR_INVALID, "nlambda=%d", g.nlambda);
  if (g.nlambda > 1 && g.engine != PTYG_EPIE && g.engine != PTYG_MPIE && g.engine != PTYG_QNEWTON &&
      g.engine != PTYG_MQNEWTON)
    return fail(PTYG_ERR_UNSUPPORTED, "nlambda=%d: several wavelengths run with ePIE, mPIE, qNewton and mqNewton",
                g.nlambda);
  if (g.threads != 0 &&
      (g.threads % 32 != 0 || g.threads < 128 || g.threads > (g.engine == PTYG_MQNEWTON ? 256 : 512)))
    return fail(PTYG_ERR_INVALID, "threads=%d: a multiple of 32 in [128, %d]", g.threads,
                g.engine == PTYG_MQNEWTON ? 256 : 512);
  if (g.probe_in_smem < 0 || g.probe_in_smem > 2) return fail(PTYG_ERR_INVALID, "probe_in_smem=%d", g.probe_in_smem);
  if (g.asp_table_in_smem < 0 || g.asp_table_in_smem > 2)
    return fail(PTYG_ERR_INVALID, "asp_table_in_smem=%d", g.asp_table_in_smem);
  if (!valid_np(g.Np)) return fail(PTYG_ERR_UNSUPPORTED, "Np=%d: supported sizes are 32, 64, 128, 256", g.Np);
  if (g.No < g.Np) return fail(PTYG_ERR_INVALID, "No=%d smaller than Np=%d", g.No, g.Np);
  if (g.nosm < 1 || g.npsm < 1 || g.nslice < 1 || g.num_frames < 1 || g.num_scans < 1)
    return fail(PTYG_ERR_INVALID, "mode/slice/frame/scan counts must be >= 1");
  if (g.engine < PTYG_EPIE || g.engine > PTYG_MQNEWTON) return fail(PTYG_ERR_INVALID, "engine=%d", g.engine);
  if (g.propagator < PTYG_FRAUNHOFER || g.propagator > PTYG_ASP)
    return fail(PTYG_ERR_UNSUPPORTED, "propagator %d is not on this path", g.propagator);
  if (g.propagator == PTYG_ASP && g.fftshift)
    return fail(PTYG_ERR_INVALID, "ASP propagatorType works only with fftshiftSwitch = False");
  if (g.engine == PTYG_E3PIE) {
    if (g.nosm != 1) return fail(PTYG_ERR_UNSUPPORTED, "e3PIE with nosm=%d (object modes) is not on this path", g.nosm);
    if (g.nslice > 6) return fail(PTYG_ERR_UNSUPPORTED, "e3PIE with nslice=%d > 6", g.nslice);
  } else if (g.nslice != 1) {
    return fail(PTYG_ERR_UNSUPPORTED, "nslice=%d needs the e3PIE engine", g.nslice);
  }
  if (!ptyg::engine_modes_supported(g.Np, g.nlambda * g.nosm, g.nlambda * g.npsm))
    return fail(PTYG_ERR_UNSUPPORTED, "nlambda=%d nosm=%d npsm=%d at Np=%d is not instantiated", g.nlambda, g.nosm,
                g.npsm, g.Np);
  int dev;
  int r = ready_device(&dev);
  if (r) return r;
  ptyg_plan* p = new (std::nothrow) ptyg_plan();
  if (!p) return fail(PTYG_ERR_OOM, "host allocation");
  p->g = g;
  p->device = dev;
  int maxSmem = 0;
  cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  // the first instantiated cluster shape that fits in shared memory and can
  // be co-scheduled; per shape the probe rows in shared memory first, then
  // (ASP) the transfer function's columns
  const bool e3 = g.engine == PTYG_E3PIE;
  const bool aspTable = g.propagator == PTYG_ASP && !e3;
  auto fits = [&](int c, bool psm, bool hsm) {
    if ((g.probe_in_smem == 1 && psm) || (g.probe_in_smem == 2 && !psm)) return false;
    if (aspTable && ((g.asp_table_in_smem == 1 && hsm) || (g.asp_table_in_smem == 2 && !hsm))) return false;
    if (hsm && !aspTable) return false;
    if (e3 && psm) return false;  // e3PIE keeps its probe slices in global memory
    p->C = c;
    p->probeInSmem = psm;
    p->hInSmem = hsm;
    p->threads = g.threads > 0 ? g.threads : engine_threads(g, c);
    p->smem = e3 ? ptyg::e3pie_smem_bytes(g.Np, c, g.npsm)
                 : ptyg::engine_smem_bytes(g.Np, c, g.nosm, g.npsm, g.nlambda, g.engine, psm, hsm);
    if ((int)p->smem > maxSmem) return false;
    int nclusters = 0;
    cudaError_t e = e3 ? ptyg::e3pie_max_clusters(g.Np, c, p->threads, p->smem, &nclusters)
                       : ptyg::engine_max_clusters(g.Np, g.engine, g.nlambda, c, p->threads, p->smem, &nclusters);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return nclusters > 0;
  };
  bool found = false;
  for (int c : cluster_candidates(g)) {
    if (!ptyg::engine_shape_supported(g.Np, c)) continue;
    for (bool psm : {true, false}) {
      for (bool hsm : {true, false}) {
        if ((found = fits(c, psm, hsm))) break;
      }
      if (found) break;
    }
    if (found) break;
  }
  if (!found) {
    plan_free(p);
    return fail(PTYG_ERR_UNSUPPORTED, "no launchable cluster shape for Np=%d nosm=%d npsm=%d (shared memory %zu B, max %d)",
                g.Np, g.nosm, g.npsm, p->smem, maxSmem);
  }
  const size_t np2 = (size_t)g.Np * g.Np;
  const int K = g.nlambda * g.nosm * g.npsm;
  p->scans.resize(g.num_scans);
  p->hScans.resize(g.num_scans);
  for (int s = 0; s < g.num_scans; ++s) {
    ScanOwned& o = p->scans[s];
    cudaError_t e = cudaMalloc(&o.data, (size_t)g.num_frames * np2 * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&o.work, (size_t)K * np2 * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&o.errPart, (size_t)g.num_frames * p->C * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(o.errPart, 0, (size_t)g.num_frames * p->C * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&o.err, (size_t)g.num_frames * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&o.red, 2 * ptyg::RED_BANK * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&o.status, sizeof(int));
    if (e == cudaSuccess && g.engine == PTYG_E3PIE)
      e = cudaMalloc(&o.esw, (size_t)g.nslice * g.npsm * np2 * sizeof(float2));
    if (e == cudaSuccess && (g.engine == PTYG_QNEWTON || g.engine == PTYG_MQNEWTON)) {
      const int tpr = (g.No + ptyg::TILE - 1) / ptyg::TILE;
      e = cudaMalloc(&o.tileMax, (size_t)tpr * tpr * sizeof(float));
    }
    if (e == cudaSuccess) e = cudaMemset(o.status, 0, sizeof(int));
    if (e != cudaSuccess) {
      plan_free(p);
      return cuda_fail(e, "plan allocation");
    }
  }
  cudaError_t e = cudaMalloc(&p->dScans, g.num_scans * sizeof(ScanDev));
  if (e != cudaSuccess) {
    plan_free(p);
    return cuda_fail(e, "plan allocation");
  }
  *plan = p;
  return PTYG_OK;
}

extern "C" int ptyg_plan_destroy(ptyg_plan* plan) {
  plan_free(plan);
  return PTYG_OK;
}

// Fourier-layout permutation of a centred table: out[sx][sy] = ifftshift(H)[ky][kx].
static std::vector<float2> to_fourier_layout_host(const float2* centred, int Np) {
  std::vector<float2> out((size_t)Np * Np);
  for (int sx = 0; sx < Np; ++sx)
    for (int sy = 0; sy < Np; ++sy) {
      const int ky = ptyg::slot_to_freq_y(sy, Np), kx = ptyg::slot_to_freq_x(sx, Np);
      // ifftshift: element k of the shifted array is element (k + Np/2) % Np of the centred one
      const int cy = (ky + Np / 2) % Np, cx = (kx + Np / 2) % Np;
      out[(size_t)sx * Np + sy] = centred[(size_t)cy * Np + cx];
    }
  return out;
}

static int upload(float2** dst, const void* host, size_t n) {
  if (!*dst) PTYG_CUDA(cudaMalloc(dst, n * sizeof(float2)), "table allocation");
  PTYG_CUDA(cudaMemcpy(*dst, host, n * sizeof(float2), cudaMemcpyHostToDevice), "table upload");
  return PTYG_OK;
}

extern "C" int ptyg_plan_set_tables(ptyg_plan* p, const void* fresnel_q, const void* asp_h, const void* slice_h) {
  if (!p) return fail(PTYG_ERR_INVALID, "null plan");
  const int Np = p->g.Np;
  const size_t n = (size_t)Np * Np;
  int r;
  if (fresnel_q && (r = upload(&p->fresnelQ, fresnel_q, n))) return r;
  if (asp_h) {
    const int sets = p->g.nlambda;  // one table per wavelength
    std::vector<float2> all;
    all.reserve(sets * n);
    for (int w = 0; w < sets; ++w) {
      auto t = to_fourier_layout_host((const float2*)asp_h + w * n, Np);
      all.insert(all.end(), t.begin(), t.end());
    }
    if ((r = upload(&p->aspH, all.data(), sets * n))) return r;
  }
  if (slice_h) {
    auto t = to_fourier_layout_host((const float2*)slice_h, Np);
    if ((r = upload(&p->sliceH, t.data(), n))) return r;
  }
  return PTYG_OK;
}

extern "C" int ptyg_plan_bind_scan(ptyg_plan* p, int scan, const ptyg_scan_buffers* b, const float* ptychogram,
                                   void* stream) {
  if (!p || !b) return fail(PTYG_ERR_INVALID, "null argument");
  if (scan < 0 || scan >= p->g.num_scans) return fail(PTYG_ERR_INVALID, "scan %d out of range", scan);
  if (!b->object || !b->probe || !b->positions || !b->order || !ptychogram)
    return fail(PTYG_ERR_INVALID, "object, probe, positions, order and ptychogram are required");
  if (p->g.engine == PTYG_MPIE &&
      (!b->object_buffer || !b->object_momentum || !b->probe_buffer || !b->probe_momentum))
    return fail(PTYG_ERR_INVALID, "mPIE needs object/probe buffers and momenta");
  if (p->g.engine == PTYG_MQNEWTON &&
      (!b->object_momentum || !b->probe_buffer || !b->probe_momentum || !b->second_moment))
    return fail(PTYG_ERR_INVALID, "mqNewton needs object/probe momenta, the probe buffer and the second-moment pair");
  cudaStream_t st = (cudaStream_t)stream;
  ScanOwned& o = p->scans[scan];
  o.buf = *b;
  const int Np = p->g.Np;
  const size_t n = (size_t)p->g.num_frames * Np * Np;
  if (p->g.propagator == PTYG_ASP) {
    PTYG_CUDA(cudaMemcpyAsync(o.data, ptychogram, n * sizeof(float), cudaMemcpyDeviceToDevice, st), "data copy");
  } else {
    PTYG_CUDA(ptyg::to_fourier_layout(ptychogram, o.data, p->g.num_frames, Np, st), "data layout");
  }
  PTYG_CUDA(cudaMemsetAsync(o.errPart, 0, (size_t)p->g.num_frames * p->C * sizeof(double), st), "reset");
  PTYG_CUDA(cudaMemsetAsync(o.status, 0, sizeof(int), st), "reset");
  ScanDev& d = p->hScans[scan];
  d = ScanDev{};
  d.object = (float2*)b->object;
  d.probe = (float2*)b->probe;
  d.data = o.data;
  d.positions = b->positions;
  d.order = b->order;
  d.momentum = b->momentum_flags;
  d.objectBuffer = (float2*)b->object_buffer;
  d.objectMomentum = (float2*)b->object_momentum;
  d.probeBuffer = (float2*)b->probe_buffer;
  d.probeMomentum = (float2*)b->probe_momentum;
  d.work = o.work;
  d.eswStore = o.esw;
  d.errPart = o.errPart;
  d.detErr = o.detErr;
  d.red = o.red;
  d.status = o.status;
  d.tileMax = o.tileMax;
  d.moment2 = b->second_moment;
  d.vec4 = p->g.No % 2 == 0 && ((uintptr_t)b->object % 16) == 0 && ((uintptr_t)b->object_momentum % 16) == 0;
  d.background = o.background;
  d.iscale = o.iscale;
  d.reference = o.reference;
  o.bound = true;
  o.orderLen = p->g.num_frames;
  PTYG_CUDA(cudaMemcpyAsync(p->dScans + scan, &d, sizeof(ScanDev), cudaMemcpyHostToDevice, st), "scan upload");
  // the host copy must outlive the async copy: hScans is owned by the plan
  return PTYG_OK;
}

extern "C" int ptyg_plan_run(ptyg_plan* p, const ptyg_update_params* u, int start, int count, int flags,
                             void* stream) {
  if (!p || !u) return fail(PTYG_ERR_INVALID, "null argument");
  if (start < 0 || count < 0) return fail(PTYG_ERR_INVALID, "start=%d count=%d", start, count);
  for (int s = 0; s < p->g.num_scans; ++s)
    if (!p->scans[s].bound) return fail(PTYG_ERR_INVALID, "scan %d is not bound", s);
  if (count == 0) return PTYG_OK;
  const ptyg_geometry& g = p->g;
  for (int s = 0; s < g.num_scans; ++s)
    if ((long long)start + count > p->scans[s].orderLen)
      return fail(PTYG_ERR_INVALID, "order slots [%d, %d) exceed the %d slots of scan %d", start, start + count,
                  p->scans[s].orderLen, s);
  cudaStream_t st = (cudaStream_t)stream;
  if (g.propagator == PTYG_FRESNEL && !p->fresnelQ) return fail(PTYG_ERR_INVALID, "Fresnel table not set");
  if (g.propagator == PTYG_ASP && !p->aspH) return fail(PTYG_ERR_INVALID, "ASP transfer function not set");
  const bool det = (flags & 1) != 0;
  if (det) {
    for (int s = 0; s < g.num_scans; ++s) {
      ScanOwned& o = p->scans[s];
      if (!o.detErr) {
        PTYG_CUDA(cudaMalloc(&o.detErr, (size_t)g.num_frames * g.Np * g.Np * sizeof(float)), "detector error");
        PTYG_CUDA(cudaMemsetAsync(o.detErr, 0, (size_t)g.num_frames * g.Np * g.Np * sizeof(float), st), "reset");
        p->hScans[s].detErr = o.detErr;
        PTYG_CUDA(cudaMemcpyAsync(p->dScans + s, &p->hScans[s], sizeof(ScanDev), cudaMemcpyHostToDevice, st),
                  "scan upload");
      }
    }
  }
  EngineArgs a = {};
  a.scans = p->dScans;
  a.twiddle = twiddles(p->device, g.Np);
  a.fresnelQ = p->fresnelQ;
  a.aspH = p->aspH;
  a.sliceH = p->sliceH;
  a.Np = g.Np;
  a.No = g.No;
  a.nosm = g.nosm;
  a.npsm = g.npsm;
  a.nlambda = g.nlambda;
  a.nslice = g.nslice;
  a.numFrames = g.num_frames;
  a.engine = g.engine;
  a.prop = g.propagator;
  a.centred = !g.fftshift;
  a.fpm = g.fpm;
  a.start = start;
  a.count = count;
  a.writeDetErr = det;
  a.cluster = p->C;
  a.tilesPerRow = (g.No + ptyg::TILE - 1) / ptyg::TILE;
  a.probeInSmem = p->probeInSmem ? 1 : 0;
  a.hInSmem = p->hInSmem ? 1 : 0;
  a.betaO = u->beta_object;
  a.betaP = u->beta_probe;
  a.alphaO = u->alpha_object;
  a.alphaP = u->alpha_probe;
  a.regO = u->reg_object;
  a.regP = u->reg_probe;
  a.frictionM = u->friction;
  a.feedbackM = u->feedback;
  a.weightP = u->probe_weight;
  a.bethSlice = u->slice_beta;
  if (g.engine == PTYG_MQNEWTON) {
    if (u->momentum_method < PTYG_MOMENTUM || u->momentum_method > PTYG_NADAM)
      return fail(PTYG_ERR_INVALID, "momentum_method=%d", u->momentum_method);
    if (!(u->beta1_scale != 0.f) || !(u->beta2_scale != 0.f))
      return fail(PTYG_ERR_INVALID, "beta1_scale and beta2_scale (1 - beta**itr) must be nonzero");
    a.momentum = u->momentum_method;
    // NumPy rounds each Python float operand to float32 at the operation
    a.b1 = (float)u->beta1;
    a.omb1 = (float)(1.0 - u->beta1);
    a.b2 = (float)u->beta2;
    a.omb2 = (float)(1.0 - u->beta2);
    a.b1s = u->beta1_scale;
    a.b2s = u->beta2_scale;
    a.betaOm = u->beta_object_m;
    a.betaPm = u->beta_probe_m;
  }
  a.iconstraint = p->proj.intensity_constraint;
  a.denoise = p->proj.adaptive_denoising;
  a.bgMode = p->proj.background_mode;
  a.fmask = p->proj.fourier_mask;
  a.imask = p->proj.intensity_mask;
  a.invFrames = 1.f / (float)g.num_frames;
  a.W = p->W;
  a.imaskTab = p->imask;
  if (g.engine == PTYG_E3PIE && !p->sliceH) return fail(PTYG_ERR_INVALID, "e3PIE slice transfer function not set");
  cudaError_t e = g.engine == PTYG_E3PIE ? ptyg::launch_e3pie(a, g.num_scans, p->threads, p->smem, st)
                                         : ptyg::launch_engine(a, g.num_scans, p->threads, p->smem, st);
  if (e != cudaSuccess) return cuda_fail(e, "engine launch");
  return PTYG_OK;
}

extern "C" int ptyg_plan_set_order(ptyg_plan* p, int scan, const int32_t* order, const uint8_t* momentum_flags,
                                   int length, void* stream) {
  if (!p || !order) return fail(PTYG_ERR_INVALID, "null argument");
  if (scan < 0 || scan >= p->g.num_scans) return fail(PTYG_ERR_INVALID, "scan %d out of range", scan);
  if (!p->scans[scan].bound) return fail(PTYG_ERR_INVALID, "scan %d is not bound", scan);
  if (length < 1) return fail(PTYG_ERR_INVALID, "length=%d", length);
  if (p->g.engine == PTYG_MPIE && !momentum_flags) return fail(PTYG_ERR_INVALID, "mPIE needs momentum flags");
  p->hScans[scan].order = order;
  p->hScans[scan].momentum = momentum_flags;
  p->scans[scan].orderLen = length;
  PTYG_CUDA(cudaMemcpyAsync(p->dScans + scan, &p->hScans[scan], sizeof(ScanDev), cudaMemcpyHostToDevice,
                            (cudaStream_t)stream),
            "scan upload");
  return PTYG_OK;
}

extern "C" int ptyg_plan_info(ptyg_plan* p, int* cluster, int* threads, int* smem_bytes, int* max_active_clusters) {
  if (!p) return fail(PTYG_ERR_INVALID, "null plan");
  if (cluster) *cluster = p->C;
  if (threads) *threads = p->threads;
  if (smem_bytes) *smem_bytes = (int)p->smem;
  if (max_active_clusters) {
    int n = 0;
    cudaError_t e = ptyg::engine_max_clusters(p->g.Np, p->g.engine, p->g.nlambda, p->C, p->threads, p->smem, &n);
    if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveClusters");
    *max_active_clusters = n;
  }
  return PTYG_OK;
}

extern "C" int ptyg_plan_frame_errors(ptyg_plan* p, int scan, double* host_out, void* stream) {
  if (!p || !host_out) return fail(PTYG_ERR_INVALID, "null argument");
  if (scan < 0 || scan >= p->g.num_scans) return fail(PTYG_ERR_INVALID, "scan %d out of range", scan);
  cudaStream_t st = (cudaStream_t)stream;
  ScanOwned& o = p->scans[scan];
  PTYG_CUDA(ptyg::sum_parts(o.errPart, o.err, p->g.num_frames, p->C, st), "error sum");
  PTYG_CUDA(cudaMemcpyAsync(host_out, o.err, p->g.num_frames * sizeof(double), cudaMemcpyDeviceToHost, st),
            "error readback");
  PTYG_CUDA(cudaStreamSynchronize(st), "error readback");
  return PTYG_OK;
}

extern "C" int ptyg_plan_frame_errors_device(ptyg_plan* p, int scan, double* device_out, void* stream) {
  if (!p || !device_out) return fail(PTYG_ERR_INVALID, "null argument");
  if (scan < 0 || scan >= p->g.num_scans) return fail(PTYG_ERR_INVALID, "scan %d out of range", scan);
  ScanOwned& o = p->scans[scan];
  PTYG_CUDA(ptyg::sum_parts(o.errPart, device_out, p->g.num_frames, p->C, (cudaStream_t)stream), "error sum");
  return PTYG_OK;
}

// out[scan][frame] = sum_c errPart_scan[frame][c] for every bound scan, in
// the fixed order of sum_parts: one launch for a whole batch.
__global__ void sum_parts_scans_kernel(const ScanDev* __restrict__ scans, double* __restrict__ out, int nscans,
                                       int frames, int C) {
  const size_t n = (size_t)nscans * frames;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int s = (int)(i / frames), f = (int)(i - (size_t)s * frames);
    const double* part = scans[s].errPart + (size_t)f * C;
    double t = 0.0;
    for (int c = 0; c < C; ++c) t += part[c];
    out[i] = t;
  }
}

extern "C" int ptyg_plan_frame_errors_all_device(ptyg_plan* p, double* device_out, void* stream) {
  if (!p || !device_out) return fail(PTYG_ERR_INVALID, "null argument");
  const size_t n = (size_t)p->g.num_scans * p->g.num_frames;
  const unsigned grid = (unsigned)((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024);
  sum_parts_scans_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(p->dScans, device_out, p->g.num_scans,
                                                                  p->g.num_frames, p->C);
  PTYG_CUDA(cudaGetLastError(), "error sums");
  return PTYG_OK;
}

extern "C" int ptyg_plan_detector_error(ptyg_plan* p, int scan, float* out, void* stream) {
  if (!p || !out) return fail(PTYG_ERR_INVALID, "null argument");
  if (scan < 0 || scan >= p->g.num_scans) return fail(PTYG_ERR_INVALID, "scan %d out of range", scan);
  ScanOwned& o = p->scans[scan];
  if (!o.detErr) return fail(PTYG_ERR_INVALID, "no detector error recorded (run with flags bit 0)");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t n = (size_t)p->g.num_frames * p->g.Np * p->g.Np;
  if (p->g.propagator == PTYG_ASP) {
    PTYG_CUDA(cudaMemcpyAsync(out, o.detErr, n * sizeof(float), cudaMemcpyDeviceToDevice, st), "copy");
  } else {
    PTYG_CUDA(ptyg::from_fourier_layout(o.detErr, out, p->g.num_frames, p->g.Np, st), "layout");
  }
  return PTYG_OK;
}

// a device Np x Np float table in the ptychogram's layout -> the data layout
static int to_data_layout(const ptyg_plan* p, const float* in, float* out, cudaStream_t st) {
  const int Np = p->g.Np;
  if (p->g.propagator == PTYG_ASP) {
    PTYG_CUDA(cudaMemcpyAsync(out, in, (size_t)Np * Np * sizeof(float), cudaMemcpyDeviceToDevice, st), "copy");
  } else {
    PTYG_CUDA(ptyg::to_fourier_layout(in, out, 1, Np, st), "layout");
  }
  return PTYG_OK;
}

static int from_data_layout(const ptyg_plan* p, const float* in, float* out, cudaStream_t st) {
  const int Np = p->g.Np;
  if (p->g.propagator == PTYG_ASP) {
    PTYG_CUDA(cudaMemcpyAsync(out, in, (size_t)Np * Np * sizeof(float), cudaMemcpyDeviceToDevice, st), "copy");
  } else {
    PTYG_CUDA(ptyg::from_fourier_layout(in, out, 1, Np, st), "layout");
  }
  return PTYG_OK;
}

// planes of the interferometric reference field: one per exit-wave mode
static int ref_planes(const ptyg_plan* p) {
  return (p->g.nlambda > 0 ? p->g.nlambda : 1) * p->g.nosm * p->g.npsm;
}

static __global__ void fill_kernel(float* x, size_t n, float v) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = v;
}
static __global__ void fill_kernel_d(double* x, size_t n, double v) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = v;
}

extern "C" int ptyg_plan_set_projection(ptyg_plan* p, const ptyg_projection* pr, const float* W,
                                        const float* intensity_mask, void* stream) {
  if (!p || !pr) return fail(PTYG_ERR_INVALID, "null argument");
  const ptyg_projection& q = *pr;
  if (q.intensity_constraint < PTYG_STANDARD || q.intensity_constraint > PTYG_INTERFEROMETRIC)
    return fail(PTYG_ERR_INVALID, "intensity_constraint=%d", q.intensity_constraint);
  if (q.intensity_constraint == PTYG_INTERFEROMETRIC && p->g.propagator == PTYG_ASP)
    return fail(PTYG_ERR_UNSUPPORTED, "the interferometric constraint runs with Fraunhofer and Fresnel plans");
  if (q.intensity_constraint == PTYG_INTERFEROMETRIC && p->g.engine == PTYG_MQNEWTON)
    return fail(PTYG_ERR_UNSUPPORTED, "the interferometric constraint runs with ePIE, mPIE and qNewton plans");
  if (p->g.engine == PTYG_E3PIE && q.intensity_constraint == PTYG_INTERFEROMETRIC)
    return fail(PTYG_ERR_UNSUPPORTED, "e3PIE runs every projection switch but the interferometric constraint");
  if (q.fourier_mask && !W) return fail(PTYG_ERR_INVALID, "FourierMaskSwitch needs W");
  if (q.intensity_mask && !intensity_mask) return fail(PTYG_ERR_INVALID, "intensityMask needs intensity_mask");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t n2 = (size_t)p->g.Np * p->g.Np;
  int r;
  if (q.fourier_mask) {
    if (!p->W) PTYG_CUDA(cudaMalloc(&p->W, n2 * sizeof(float)), "allocation");
    if ((r = to_data_layout(p, W, p->W, st))) return r;
  }
  if (q.intensity_mask) {
    if (!p->imask) PTYG_CUDA(cudaMalloc(&p->imask, n2 * sizeof(float)), "allocation");
    if ((r = to_data_layout(p, intensity_mask, p->imask, st))) return r;
  }
  for (int s = 0; s < p->g.num_scans; ++s) {
    ScanOwned& o = p->scans[s];
    if (q.background_mode && !o.background) {
      PTYG_CUDA(cudaMalloc(&o.background, n2 * sizeof(float)), "allocation");
      fill_kernel<<<(unsigned)((n2 + 255) / 256), 256, 0, st>>>(o.background, n2, 0.1f);
      PTYG_CUDA(cudaGetLastError(), "fill");
    }
    if (q.intensity_constraint == PTYG_FLUCTUATION && !o.iscale) {
      const size_t nf = (size_t)p->g.num_frames;
      PTYG_CUDA(cudaMalloc(&o.iscale, nf * sizeof(double)), "allocation");
      fill_kernel_d<<<(unsigned)((nf + 255) / 256), 256, 0, st>>>(o.iscale, nf, 1.0);
      PTYG_CUDA(cudaGetLastError(), "fill");
    }
    if (q.intensity_constraint == PTYG_INTERFEROMETRIC) {
      const int planes = ref_planes(p);
      if (!o.reference) PTYG_CUDA(cudaMalloc(&o.reference, (size_t)planes * n2 * sizeof(float2)), "allocation");
      PTYG_CUDA(ptyg::reference_init(o.reference, planes, p->g.Np, !p->g.fftshift, st), "reference init");
    }
    p->hScans[s].background = o.background;
    p->hScans[s].iscale = o.iscale;
    p->hScans[s].reference = o.reference;
    PTYG_CUDA(cudaMemcpyAsync(p->dScans + s, &p->hScans[s], sizeof(ScanDev), cudaMemcpyHostToDevice, st),
              "scan upload");
  }
  p->proj = q;
  return PTYG_OK;
}

extern "C" int ptyg_plan_get_reference(ptyg_plan* p, int scan, void* reference, void* stream) {
  if (!p || !reference) return fail(PTYG_ERR_INVALID, "null argument");
  if (scan < 0 || scan >= p->g.num_scans) return fail(PTYG_ERR_INVALID, "scan %d out of range", scan);
  if (!p->scans[scan].reference) return fail(PTYG_ERR_INVALID, "the interferometric constraint is off");
  PTYG_CUDA(ptyg::reference_natural(p->scans[scan].reference, (float2*)reference, ref_planes(p), p->g.Np,
                                    !p->g.fftshift, (cudaStream_t)stream),
            "reference readout");
  return PTYG_OK;
}

extern "C" int ptyg_plan_set_background(ptyg_plan* p, int scan, const float* background, void* stream) {
  if (!p || !background) return fail(PTYG_ERR_INVALID, "null argument");
  if (scan < 0 || scan >= p->g.num_scans) return fail(PTYG_ERR_INVALID, "scan %d out of range", scan);
  if (!p->scans[scan].background) return fail(PTYG_ERR_INVALID, "background mode is off (ptyg_plan_set_projection)");
  return to_data_layout(p, background, p->scans[scan].background, (cudaStream_t)stream);
}

extern "C" int ptyg_plan_get_background(ptyg_plan* p, int scan, float* background, void* stream) {
  if (!p || !background) return fail(PTYG_ERR_INVALID, "null argument");
  if (scan < 0 || scan >= p->g.num_scans) return fail(PTYG_ERR_INVALID, "scan %d out of range", scan);
  if (!p->scans[scan].background) return fail(PTYG_ERR_INVALID, "background mode is off (ptyg_plan_set_projection)");
  return from_data_layout(p, p->scans[scan].background, background, (cudaStream_t)stream);
}

extern "C" int ptyg_plan_intensity_scaling(ptyg_plan* p, int scan, double* host_out, void* stream) {
  if (!p || !host_out) return fail(PTYG_ERR_INVALID, "null argument");
  if (scan < 0 || scan >= p->g.num_scans) return fail(PTYG_ERR_INVALID, "scan %d out of range", scan);
  if (!p->scans[scan].iscale) return fail(PTYG_ERR_INVALID, "the fluctuation constraint is off");
  cudaStream_t st = (cudaStream_t)stream;
  PTYG_CUDA(cudaMemcpyAsync(host_out, p->scans[scan].iscale, (size_t)p->g.num_frames * sizeof(double),
                            cudaMemcpyDeviceToHost, st),
            "copy");
  PTYG_CUDA(cudaStreamSynchronize(st), "copy");
  return PTYG_OK;
}

extern "C" int ptyg_plan_status(ptyg_plan* p, int scan, int* host_status, void* stream) {
  if (!p || !host_status) return fail(PTYG_ERR_INVALID, "null argument");
  if (scan < 0 || scan >= p->g.num_scans) return fail(PTYG_ERR_INVALID, "scan %d out of range", scan);
  cudaStream_t st = (cudaStream_t)stream;
  PTYG_CUDA(cudaMemcpyAsync(host_status, p->scans[scan].status, sizeof(int), cudaMemcpyDeviceToHost, st), "status");
  PTYG_CUDA(cudaStreamSynchronize(st), "status");
  return PTYG_OK;
}

// ---------------------------------------------------------------- helpers
extern "C" int ptyg_mul_window(void* x, const float* window, int64_t n, int64_t n_window, void* stream) {
  if (!x || !window || n < 0 || n_window <= 0) return fail(PTYG_ERR_INVALID, "bad arguments");
  if (n == 0) return PTYG_OK;
  PTYG_CUDA(ptyg::mul_window((float2*)x, window, n, n_window, (cudaStream_t)stream), "mul_window");
  return PTYG_OK;
}

extern "C" int ptyg_gram(const void* p, int modes, int64_t n, void* gram, void* stream) {
  if (!p || !gram || modes < 1 || n < 1) return fail(PTYG_ERR_INVALID, "bad arguments");
  PTYG_CUDA(ptyg::gram((const float2*)p, modes, n, (double2*)gram, (cudaStream_t)stream), "gram");
  return PTYG_OK;
}

extern "C" int ptyg_mix_modes(const void* V, const void* p, void* out, int modes, int64_t n, void* stream) {
  if (!V || !p || !out || modes < 1 || n < 1) return fail(PTYG_ERR_INVALID, "bad arguments");
  if (modes > 16) return fail(PTYG_ERR_UNSUPPORTED, "modes=%d > 16", modes);
  if (p == out) return fail(PTYG_ERR_INVALID, "ptyg_mix_modes cannot work in place");
  PTYG_CUDA(ptyg::mix_modes((const float2*)V, (const float2*)p, (float2*)out, modes, n, (cudaStream_t)stream),
            "mix_modes");
  return PTYG_OK;
}
