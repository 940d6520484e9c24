/*
 * ptyg.h -- C ABI of libptyg.so, the GB300 (sm_103a) kernels behind the
 * ptylab_gb300 drop-in for PtyLab's per-position reconstruction loop.
 *
 * Plain C types only: every array argument is a device pointer (CUDA global
 * memory on the current device) unless its comment says "host".  complex64
 * data is interleaved (re, im) float pairs, C-contiguous, in PtyLab's 6-D
 * layout with nlambda = 1:
 *   object      (nosm, nslice, No, No)      PtyLab/Reconstruction/Reconstruction.py:362-374
 *   probe       (npsm, nslice, Np, Np)      PtyLab/Reconstruction/Reconstruction.py:395-413
 *   ptychogram  float32 (numFrames, Np, Np) PtyLab/ExperimentalData/ExperimentalData.py:234-250
 *   positions   int32 (numFrames, 2) = (row, col) of the patch corner
 *               PtyLab/Reconstruction/Reconstruction.py:676-710
 * Streams are passed as `void*` (a cudaStream_t; NULL = legacy default stream).
 *
 * Every function returns PTYG_OK (0) or a negative status; the message of the
 * last failure on the calling thread is available from ptyg_last_error().
 * No C++ exception crosses this boundary.
 */
#ifndef PTYG_H
#define PTYG_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define PTYG_API __attribute__((visibility("default")))
#else
#define PTYG_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define PTYG_VERSION 1000 /* 0.1.0 */

enum ptyg_status {
  PTYG_OK = 0,
  PTYG_ERR_INVALID = -1,     /* bad argument (maps to ValueError)            */
  PTYG_ERR_UNSUPPORTED = -2, /* valid in PtyLab, not on this path (NotImplementedError) */
  PTYG_ERR_OOM = -3,         /* device allocation failed (MemoryError)       */
  PTYG_ERR_CUDA = -4,        /* CUDA runtime error (RuntimeError)            */
  PTYG_ERR_TIMEOUT = -5,     /* a bounded device wait gave up (TimeoutError) */
  PTYG_ERR_DEVICE = -6       /* no usable sm_103a device (ImportError)       */
};

enum ptyg_engine { PTYG_EPIE = 0, PTYG_MPIE = 1, PTYG_QNEWTON = 2, PTYG_E3PIE = 3, PTYG_MQNEWTON = 4 };
/* mqNewton.momentum_method (PtyLab/Engines/mqNewton.py:68-79, 142-182) */
enum ptyg_momentum { PTYG_MOMENTUM = 0, PTYG_ADAM = 1, PTYG_NADAM = 2 };
/* params.intensityConstraint (PtyLab/Engines/BaseEngine.py:913-961) */
enum ptyg_intensity_constraint {
  PTYG_STANDARD = 0,
  PTYG_POISSION = 1,
  PTYG_EXPONENTIAL = 2,
  PTYG_FLUCTUATION = 3,
  PTYG_INTERFEROMETRIC = 4 /* a detector-plane reference field R per mode: I_est = sum |Psi + R|^2 */
};
enum ptyg_propagator {
  PTYG_FRAUNHOFER = 0,
  PTYG_FRESNEL = 1,
  PTYG_ASP = 2,
  /* ptyg_propagate_sets only: */
  PTYG_POLYCHROME_ASP = 3,
  PTYG_SCALED_ASP = 4,
  PTYG_SCALED_POLYCHROME_ASP = 5,
  PTYG_TWO_STEP_POLYCHROME = 6,
  PTYG_IDENTITY = 7
};
enum ptyg_direction { PTYG_FORWARD = 0, PTYG_INVERSE = 1 };

/* Library version (PTYG_VERSION of the build). */
PTYG_API int ptyg_version(void);

/* Message of the last failed call on this thread ("" if none). */
PTYG_API const char* ptyg_last_error(void);

/* Select `device`, check it is a compute-capability 10.3 GPU and build the
 * per-device twiddle tables.  Replaces the cupy probe of
 * PtyLab/Params/Params.py:10-28 (gpuSwitch availability). */
PTYG_API int ptyg_device_init(int device);

/* ------------------------------------------------------------------------
 * Propagators: the drop-in for Operators.object2detector / detector2object
 * (PtyLab/Operators/Operators.py:561-584) on `batch` fields of Np x Np.
 *   FRAUNHOFER  fft2c / ifft2c                    Operators.py:27-74
 *   FRESNEL     fft2c(x*Q) / ifft2c(X)*conj(Q)     Operators.py:77-152
 *   ASP         ifft2(fft2(x)*H) (conj H inverse)  Operators.py:155-230
 * `table`: FRESNEL -> Q (Np*Np complex64, natural order); ASP -> the
 * ifftshifted transfer function (Np*Np complex64); FRAUNHOFER -> NULL.
 * `fftshift` != 0 selects uncentred transforms (params.fftshiftSwitch).
 * `scratch`: batch*Np*Np complex64 of device memory, or NULL to let the call
 * allocate (stream-ordered) and free it.  in == out is allowed.
 * Np must be 32, 64, 128 or 256. */
PTYG_API int ptyg_propagate(int propagator, int direction, int fftshift, int Np, int batch, const void* in, void* out,
                   const void* table, void* scratch, void* stream);

/* The propagators of ptyg_propagate for callers that cannot allocate GPU
 * memory: code inside a host framework that owns every device allocation, a
 * real-time acquisition callback where cudaMalloc's implicit synchronisation
 * would stall the pipeline, or a process that has reserved all of HBM for its
 * own buffers.  No counterpart in the reference (PtyLab has no C interface);
 * it exists for these callers only.  The call allocates nothing: its scratch
 * is an 8 MiB array built into the library, held by every GPU that loads it
 * until the process exits, so batch*Np*Np must not exceed 1,048,576 points
 * (larger batches fail with PTYG_ERR_INVALID).  The first call on a device
 * resolves and fills that device's built-in arrays (a synchronous copy), so
 * make it before any stream capture.  All calls share the one scratch array:
 * calls that overlap on the GPU (different streams, or threads) race and must
 * be serialised by the caller.  The built-in arrays' device addresses are
 * cached per device for the life of the process; after a cudaDeviceReset
 * they are stale and this entry point must not be called again.  A device
 * other than sm_103a fails with PTYG_ERR_DEVICE, as ptyg_device_init does.
 * Same arguments as ptyg_propagate, without `scratch`. */
PTYG_API int ptyg_propagate_noalloc(int propagator, int direction, int fftshift, int Np, int batch, const void* in,
                                    void* out, const void* table, void* stream);

/* The scaled and multi-wavelength propagators (centred transforms only; the
 * reference rejects fftshiftSwitch for all of them) on `batch` fields of
 * Np x Np.  `nsets` table sets (one per wavelength); the fields are
 * wavelength-major, so field f uses set f / (batch / nsets) and batch must be
 * a multiple of nsets.  Each table is nsets consecutive Np x Np complex64
 * arrays in natural (centred-grid) order, except where noted.
 *   POLYCHROME_ASP         ifft2c(fft2c(x)*A) (conj A inverse)      Operators.py:458-505, 536-558
 *                          A: the angular-spectrum transfer function per wavelength
 *   SCALED_ASP,            ifft2c(fft2c(x*A)*B);                    Operators.py:313-375
 *   SCALED_POLYCHROME_ASP  inverse ifft2c(fft2c(x)*conj B)*conj A   Operators.py:378-455
 *                          A = Q1, B = Q2 (SCALED_ASP: nsets = 1)
 *   TWO_STEP_POLYCHROME    fft2c(ifft2c(fft2c(x)*A)*B);             Operators.py:233-282
 *                          inverse ifft2c(fft2c(x*conj B)*conj A)
 *                          A: transfer function over zo*(1 - l0/l) per wavelength l,
 *                          B: ONE Np x Np Fresnel chirp of the first wavelength
 *   IDENTITY               out = in                                 Operators.py:508-533
 * `scratch`: batch*Np*Np complex64, or NULL to let the call allocate it.
 * in == out is allowed.  Np must be 32, 64, 128 or 256. */
PTYG_API int ptyg_propagate_sets(int propagator, int direction, int Np, int batch, int nsets, const void* in,
                                 void* out, const void* table_a, const void* table_b, void* scratch, void* stream);

/* ------------------------------------------------------------------------
 * Engine plans: the drop-in for the position loop of ePIE.reconstruct_stepwise
 * (PtyLab/Engines/ePIE.py:78-112), mPIE.reconstruct (mPIE.py:110-195),
 * qNewton.reconstruct (qNewton.py:67-90), mqNewton.reconstruct
 * (mqNewton.py:81-140) and e3PIE.reconstruct (e3PIE.py:71-190), with
 * BaseEngine.intensityProjection
 * (BaseEngine.py:870-1012) and getRMSD (BaseEngine.py:843-868).
 */
typedef struct ptyg_geometry {
  int32_t Np;          /* probe/detector size: 32, 64, 128, 256 */
  int32_t No;          /* object size, >= Np */
  int32_t nosm;        /* object modes */
  int32_t npsm;        /* probe modes */
  int32_t nslice;      /* slices (e3PIE), else 1 */
  int32_t num_frames;  /* diffraction patterns per scan */
  int32_t num_scans;   /* independent scans reconstructed side by side (>= 1) */
  int32_t engine;      /* enum ptyg_engine */
  int32_t propagator;  /* enum ptyg_propagator */
  int32_t fftshift;    /* params.fftshiftSwitch: uncentred transforms, pre-shifted data */
  int32_t fpm;         /* operationMode == "FPM" (mPIE object step, mPIE.py:237-243) */
  int32_t cluster;     /* CTAs per scan (0 = choose) */
  int32_t throughput;  /* 0: shortest time per position (8 rows per CTA);
                          1: most positions per second over many scans (16
                          rows per CTA: fewer CTAs per scan, more scans at once) */
  int32_t nlambda;     /* wavelengths (reconstruction.nlambda; 0 reads as 1).  Above
                          1 (ePIE, mPIE, qNewton, mqNewton): object (nlambda, nosm, ...)
                          and probe (nlambda, npsm, ...) wavelength-major, exit
                          waves O_(l,o) P_(l,p) of each wavelength l, the ASP
                          table one per wavelength (polychromeASP,
                          Operators.py:458-505); ePIE and qNewton sum their
                          steps over the wavelengths (ePIE.py:128-160,
                          qNewton.py:108-140), mPIE keeps them per wavelength
                          (mPIE.py:226-270) */
  int32_t threads;     /* threads per CTA, a multiple of 32 in [128, 512]
                          (mqNewton: at most 256); 0 = one warp per transform
                          task of a pass, at most 16 warps.  With 256 threads
                          and a shared-memory layout under half an SM's,
                          two CTAs share an SM and hide each other's stalls */
  int32_t probe_in_smem; /* 0 = choose (shared memory when it fits), 1 = keep
                            the CTA's probe rows in global memory (L2),
                            2 = require them in shared memory */
  int32_t asp_table_in_smem; /* ASP only: 0 = choose (the CTA's columns of the
                                transfer function, one block per wavelength,
                                copied into shared memory once per launch by
                                the bulk-copy engine when they fit beside the
                                probe rows), 1 = read them from global memory
                                (L2) at every position, 2 = require them in
                                shared memory */
} ptyg_geometry;

/* Engine scalars (ePIE.py:35-42, mPIE.py:233-245, qNewton.py:43-52,
 * e3PIE.py:186-195, mqNewton.py:50-66); probe_weight is mPIE's per-update
 * weight (1).  The mqNewton fields are read by that engine only:
 * beta1/beta2 are the Python floats themselves (the kernel rounds beta and
 * 1 - beta to float32 as NumPy does), beta1_scale/beta2_scale the float32
 * values of 1 - beta**itr for the iteration itr = loop + 1 that the launch
 * belongs to (mqNewton.py:144-145), so one launch must not span iterations. */
typedef struct ptyg_update_params {
  float beta_object, beta_probe;
  float alpha_object, alpha_probe;
  float reg_object, reg_probe;
  float friction, feedback;
  float probe_weight;
  float slice_beta; /* e3PIE probe step for slices >= 1 (0.9 in e3PIE.py:140) */
  int32_t momentum_method; /* enum ptyg_momentum */
  double beta1, beta2;
  float beta1_scale, beta2_scale;
  float beta_object_m, beta_probe_m;
} ptyg_update_params;

/* Caller-owned device buffers of one scan.
 *   mPIE: object/probe buffers and momenta, and momentum_flags (one byte per
 *         order slot, nonzero -> momentum step after that position,
 *         mPIE.py:169-172).
 *   mqNewton: object_momentum and probe_momentum (the first moments),
 *         probe_buffer, and second_moment = {v_object, v_probe}: a float32
 *         device pair holding the value every element of objectMomentum_v /
 *         probeMomentum_v carries (they start as zero arrays and every ADAM /
 *         NADAM step adds a scalar, mqNewton.py:68-79, 142-153).  The object
 *         buffer must equal the object when the run starts; it then stays
 *         equal after every position, so the kernel does not read it. */
typedef struct ptyg_scan_buffers {
  void* object;
  void* probe;
  const int32_t* positions;
  const int32_t* order;
  const uint8_t* momentum_flags;
  void* object_buffer;
  void* object_momentum;
  void* probe_buffer;
  void* probe_momentum;
  float* second_moment;
} ptyg_scan_buffers;

typedef struct ptyg_plan ptyg_plan;

/* Validate the geometry and allocate the plan's scratch (transposition
 * buffers, reduction slots, error partials, the layout-converted ptychogram). */
PTYG_API int ptyg_plan_create(const ptyg_geometry* geometry, ptyg_plan** plan);
PTYG_API int ptyg_plan_destroy(ptyg_plan* plan);

/* Host complex64 tables, Np*Np each, centred (DC at Np/2), built in double
 * and rounded as PtyLab builds them; NULL where the configuration needs none:
 *   fresnel_q  __make_quad_phase      (Operators/_propagation_kernels.py:16-36)
 *   asp_h      __aspw_transfer_function at zo (Operators.py:631-684, 861-893);
 *              nlambda consecutive tables, one per wavelength (Operators.py:909-951)
 *   slice_h    aspw at dz, wavelength/refrIndex (e3PIE.py:62-69) */
PTYG_API int ptyg_plan_set_tables(ptyg_plan* plan, const void* fresnel_q, const void* asp_h, const void* slice_h);

/* Bind scan `scan`'s buffers and load its measured intensities (device
 * float32, natural layout, already fftshifted by the caller when fftshift). */
PTYG_API int ptyg_plan_bind_scan(ptyg_plan* plan, int scan, const ptyg_scan_buffers* buffers, const float* ptychogram,
                        void* stream);

/* Point scan `scan` at a new order array (and mPIE momentum flags) of
 * `length` slots without reloading its data; ptyg_plan_run's slots index it.
 * The bind call sets length = num_frames. */
PTYG_API int ptyg_plan_set_order(ptyg_plan* plan, int scan, const int32_t* order, const uint8_t* momentum_flags,
                                 int length, void* stream);

/* Launch shape the plan chose: CTAs per scan (cluster size), threads per CTA,
 * dynamic shared memory per CTA, and how many such clusters can be resident
 * on the device at once (independent scans that run concurrently). */
PTYG_API int ptyg_plan_info(ptyg_plan* plan, int* cluster, int* threads, int* smem_bytes, int* max_active_clusters);

/* Intensity-projection switches (BaseEngine.intensityProjection,
 * PtyLab/Engines/BaseEngine.py:870-1012; adaptiveDenoising :1805-1822);
 * all zero = the standard projection.  e3PIE plans take every switch but
 * the interferometric constraint (its detector projection is BaseEngine's,
 * PtyLab/Engines/e3PIE.py:118). */
typedef struct ptyg_projection {
  int32_t intensity_constraint; /* enum ptyg_intensity_constraint */
  int32_t adaptive_denoising;   /* params.adaptiveDenoisingSwitch */
  int32_t background_mode;      /* params.backgroundModeSwitch: I_est += background, updated per position */
  int32_t fourier_mask;         /* params.FourierMaskSwitch: errors (and the background update) weighted by W */
  int32_t intensity_mask;       /* params.intensityMask: ESW *= frac * mask + mask - 1 */
} ptyg_projection;

/* Set the projection switches and their detector tables: W
 * (experimentalData.W) and intensity_mask (reconstruction.intensity_mask),
 * device float32 (Np, Np) in the ptychogram's layout (already fftshifted
 * with it when fftshift), NULL where the switch is off.  Allocates each
 * scan's background (set to 0.1, BaseEngine.py:361-364) and, for the
 * fluctuation constraint, its per-frame intensity scaling (set to 1). */
PTYG_API int ptyg_plan_set_projection(ptyg_plan* plan, const ptyg_projection* projection, const float* W,
                                      const float* intensity_mask, void* stream);

/* The interferometric constraint's reference field of scan `scan`
 * (reconstruction.reference, BaseEngine.py:371-374, 883-891, 975-982):
 * ptyg_plan_set_projection sets it to ones for every mode (as the reference
 * does at every reconstruct()); each position then sets
 * Psi' = (Psi + R) frac - R and R' = (Psi + R) frac - Psi per mode.  Read
 * out as device complex64 (nlambda * nosm * npsm, Np, Np), natural layout
 * (fftshifted when fftshift).  Fraunhofer and Fresnel plans only. */
PTYG_API int ptyg_plan_get_reference(ptyg_plan* plan, int scan, void* reference, void* stream);

/* Background of scan `scan` (reconstruction.background), device float32
 * (Np, Np) in the ptychogram's layout: load it into the plan, or read it out. */
PTYG_API int ptyg_plan_set_background(ptyg_plan* plan, int scan, const float* background, void* stream);
PTYG_API int ptyg_plan_get_background(ptyg_plan* plan, int scan, float* background, void* stream);

/* The fluctuation constraint's scaling aleph of each frame as last computed
 * (params.intensityScaling, BaseEngine.py:913-938), into `host_out`
 * (num_frames doubles); synchronises. */
PTYG_API int ptyg_plan_intensity_scaling(ptyg_plan* plan, int scan, double* host_out, void* stream);

/* Process order slots [start, start+count) of every bound scan: for each
 * slot, position order[slot] goes through gather -> propagate -> intensity
 * projection -> back-propagate -> object/probe update (-> momentum step;
 * mqNewton: an adaptive-momentum step on the whole object and probe).
 * flags bit 0: also record |I_meas - I_est| per pixel (detectorError). */
PTYG_API int ptyg_plan_run(ptyg_plan* plan, const ptyg_update_params* params, int start, int count, int flags, void* stream);

/* Per-frame sum_xy |I_meas - I_est| of the frames processed since the plan
 * was bound (FP64), into `host_out` (num_frames doubles); synchronises. */
PTYG_API int ptyg_plan_frame_errors(ptyg_plan* plan, int scan, double* host_out, void* stream);

/* The same sums into `device_out` (num_frames doubles of device memory),
 * stream-ordered and without synchronising, so a host loop can queue the
 * next iteration while this one runs and read every iteration's sums once at
 * the end. */
PTYG_API int ptyg_plan_frame_errors_device(ptyg_plan* plan, int scan, double* device_out, void* stream);
/* The same for every bound scan in one launch: device_out[scan * num_frames +
 * frame] (device float64, num_scans x num_frames), for batches of many scans
 * whose per-scan calls would cost more host time than the iteration's launch.
 * An addition for batched reconstruction; PtyLab reads its errors per engine
 * (PtyLab/Engines/BaseEngine.py:819-841). */
PTYG_API int ptyg_plan_frame_errors_all_device(ptyg_plan* plan, double* device_out, void* stream);

/* The recorded |I_meas - I_est| maps (flags bit 0) in natural layout:
 * `out` is device float32 (num_frames, Np, Np). */
PTYG_API int ptyg_plan_detector_error(ptyg_plan* plan, int scan, float* out, void* stream);

/* Device status word of scan `scan` (0 = ok; 2 = a position fell outside
 * the object and was skipped; 3 = the copy of the ASP transfer function into
 * shared memory did not complete within its bounded wait, so the launch's
 * results are not to be used). */
PTYG_API int ptyg_plan_status(ptyg_plan* plan, int scan, int* host_status, void* stream);

/* ------------------------------------------------------------------------
 * Differentiable multislice forward model and its adjoint (the model e3PIE
 * inverts, PtyLab/Engines/e3PIE.py:99-118, with the Fraunhofer detector):
 *   psi_0 = O_0[patch] P,  psi_s = ifft2(fft2(psi_{s-1}) H) O_s[patch],
 *   I = sum_modes |fft2c(psi_{S-1})|^2.
 * object (nslice, No, No), probe (npsm, Np, Np) complex64; slice_h the
 * ifftshifted slice transfer function (Np*Np complex64, natural order).
 * The adjoint accumulates dL/dRe + i dL/dIm of a real loss L into
 * grad_object / grad_probe (caller zeroes them) given grad_intensity = dL/dI.
 * Positions go in chunks of `chunk`; the adjoint recomputes each chunk's slice
 * fields.  Workspace: ptyg_multislice_workspace_bytes() of device memory. */
typedef struct ptyg_multislice {
  int32_t Np, No, npsm, nslice, num_frames, chunk;
} ptyg_multislice;

PTYG_API size_t ptyg_multislice_workspace_bytes(const ptyg_multislice* geometry);
PTYG_API int ptyg_multislice_forward(const ptyg_multislice* geometry, const void* object, const void* probe,
                                     const int32_t* positions, const void* slice_h, float* intensity, void* workspace,
                                     size_t workspace_bytes, void* stream);
PTYG_API int ptyg_multislice_adjoint(const ptyg_multislice* geometry, const void* object, const void* probe,
                                     const int32_t* positions, const void* slice_h, const float* grad_intensity,
                                     void* grad_object, void* grad_probe, void* workspace, size_t workspace_bytes,
                                     void* stream);

/* One gradient pass of the multislice model against measured intensities,
 * for the quasi-Newton multislice engine (the reference has no gradient
 * engine for multislice; its comparators are e3PIE's update,
 * PtyLab/Engines/e3PIE.py:125-173, and qNewton's step, qNewton.py:108-140).
 * For the frames order[0..num_frames) (all frames when order is NULL):
 * forward model, amplitude loss L = sum (sqrt(I) - sqrt(measured))^2,
 * dL/dI = 1 - sqrt(measured / (I + 1e-10)), and the adjoint, accumulating
 * grad_object (nslice, No, No) and grad_probe (npsm, Np, Np) in the
 * dL/dRe + i dL/dIm convention.  Optional outputs, accumulated too:
 * illum_object (nslice, No, No) += sum over positions and modes of |incident
 * field of slice s|^2; illum_probe (npsm, Np, Np) += sum over positions of
 * |O_0[patch]|^2 (the same in every mode plane); err_at_pos[frame] += sum |measured - I| (FP64).
 * measured is (frames, Np, Np) float32 in natural order, indexed by frame. */
PTYG_API int ptyg_multislice_amplitude_gradient(const ptyg_multislice* geometry, const void* object, const void* probe,
                                                const int32_t* positions, const void* slice_h, const int32_t* order,
                                                const float* measured, void* grad_object, void* grad_probe,
                                                float* illum_object, float* illum_probe, double* err_at_pos,
                                                void* workspace, size_t workspace_bytes, void* stream);

/* The quasi-Newton step of qNewton.py:108-140 on accumulated gradients, per
 * plane of plane_size complex64 values (planes <= 64):
 *   x -= beta / 2 * sqrt(w / max_plane(w)) / (w + reg) * grad,
 * then grad and w are zeroed for the next accumulation.  scratch: `planes`
 * device floats. */
PTYG_API int ptyg_qn_step(void* x, void* grad, float* weight, int planes, int64_t plane_size, float beta, float reg,
                          float* scratch, void* stream);

/* ------------------------------------------------------------------------
 * Small per-iteration helpers of BaseEngine.applyConstraints
 * (BaseEngine.py:1440-1612) and orthogonalizeModes (utils.py:130-211).
 */
/* x[i] *= w[i % n_window] for complex64 x (n elements), float32 window. */
PTYG_API int ptyg_mul_window(void* x, const float* window, int64_t n, int64_t n_window, void* stream);

/* Gram matrix G[a][b] = sum_i conj(p[a][i]) * p[b][i] of `modes` complex64
 * vectors of length n, accumulated in FP64 into `gram` (device complex128). */
PTYG_API int ptyg_gram(const void* p, int modes, int64_t n, void* gram, void* stream);

/* out[a][i] = sum_b V[a][b] * p[b][i]; V is device complex64 modes x modes. */
PTYG_API int ptyg_mix_modes(const void* V, const void* p, void* out, int modes, int64_t n, void* stream);

/* ------------------------------------------------------------------------
 * Learned warm start: kernels of a small convolutional encoder-decoder
 * (BF16 operands on the tcgen05 tensor cores, FP32 accumulation).  No
 * counterpart in PtyLab.  Activations are NHWC bf16; weights [Co][3][3][Ci]
 * bf16; every pointer is device memory.  `status` (may be NULL) is set to 1
 * if a tensor-core wait gave up (the results are then invalid).
 */

/* C = A . B^T: A [M][K], B [N][K] bf16, K a multiple of 8.  Either out != NULL:
 * bf16 [M][N] = relu?(C + bias); or C: float [splits][M][N] partial sums over
 * `splits` slices of K (reduce them with ptyg_nn_reduce_splits; bias only
 * with splits = 1). */
PTYG_API int ptyg_nn_gemm(const void* A, const void* B, int M, int N, int K, int splits, float* C, void* out,
                          const float* bias, int relu, int* status, void* stream);

/* 3x3 'same' convolution of X [Bn][H][W][C0] (channel-concatenated with
 * X1 [Bn][H][W][C1] when C1 > 0; C0, C1 multiples of 8) with weights
 * Wt [Co][9 (C0 + C1)]: into out (bf16, + bias, optional ReLU) or C (float).
 * Where the shapes allow (C0, C1 multiples of min(64, C0, C1) in {16, 32, 64},
 * 128-pixel tiles of whole image rows or row blocks, Co <= 256) the operands
 * arrive by TMA (cp.async.bulk.tensor) with the padding as out-of-bounds
 * zero fill; otherwise every thread gathers them with cp.async. */
PTYG_API int ptyg_nn_conv3(const void* X, const void* X1, int C0, int C1, int Bn, int H, int W, const void* Wt, int Co,
                           float* C, void* out, const float* bias, int relu, int* status, void* stream);

/* Select the ptyg_nn_conv3 operand path for the process: 1 (default) TMA
 * where the shapes allow, 0 the cp.async gather always (for comparisons). */
PTYG_API int ptyg_nn_conv3_path(int tma);

/* Weight gradients of a 3x3 convolution: C[z][Co][9 (C0 + C1)] = partial sums
 * over `splits` pixel ranges of dY[p][co] times the patches of X (+ X1) at
 * pixel p; H and W powers of two.  No transposes: both operands are read
 * in NHWC order. */
PTYG_API int ptyg_nn_conv3_wgrad(const void* dY, int Co, const void* X, const void* X1, int C0, int C1, int Bn, int H,
                                 int W, int splits, float* C, void* status, void* stream);
/* ... and of a dense layer: C[z][Co][K] = sum over pixel ranges of dY[p][co] X[p][k] */
PTYG_API int ptyg_nn_dense_wgrad(const void* dY, int Co, const void* X, int K, int P, int splits, float* C,
                                 void* status, void* stream);
PTYG_API int ptyg_nn_reduce_splits(const float* part, float* out, int64_t n, int splits, void* stream);
/* colT [Kpad][Bn H W]: the transposed 3x3 patch matrix (rows >= 9 (C0 + C1) zero) */
PTYG_API int ptyg_nn_im2col_t(const void* X, const void* X1, int C0, int C1, int Bn, int H, int W, int Kpad,
                              void* colT, void* stream);
/* col [Bn H W][Kpad]: the patch matrix of a one-channel image (the first layer) */
PTYG_API int ptyg_nn_im2col1(const void* X, int Bn, int H, int W, int Kpad, void* col, void* stream);
PTYG_API int ptyg_nn_transpose(const void* in, void* out, int R, int C, void* stream);
/* W [Co][9][Ci] -> Wf [Ci][9][Co] with the taps flipped (backward-data weights) */
PTYG_API int ptyg_nn_flip_weights(const void* w, void* wf, int Co, int Ci, void* stream);
PTYG_API int ptyg_nn_relu_bwd(const float* dy, const void* y, void* dpre, float* dpre_f32, int64_t n, void* stream);
/* out[n] = sum_m d[m][n] (N divides 256); part: scratch of ceil(M / 256) * N floats */
PTYG_API int ptyg_nn_col_sum(const float* d, float* part, float* out, int M, int N, void* stream);
PTYG_API int ptyg_nn_pool2(const void* x, void* y, int Bn, int H, int W, int C, void* stream);
PTYG_API int ptyg_nn_pool2_bwd(const float* dy, float* dx, int Bn, int H, int W, int C, void* stream);
PTYG_API int ptyg_nn_up2(const void* x, void* y, int Bn, int H, int W, int C, void* stream);
PTYG_API int ptyg_nn_up2_bwd(const float* dy, float* dx, int Bn, int H, int W, int C, int ldy, int coff, void* stream);
PTYG_API int ptyg_nn_slice_add(const float* src, int ldsrc, int coff, float* dst, int C, int64_t M, int accumulate,
                               void* stream);
PTYG_API int ptyg_nn_cast_bf16(const float* x, void* y, int64_t n, void* stream);
/* The warm start's initial object: complex64 patches [n][Np][Np] added in
 * order into acc [No][No] (complex64) with the window [Np][Np] at the corners
 * positions [n][2] (row, column), each patch first rotated by the unit phase
 * of sum conj(patch) acc window over its footprint (1 where that is zero);
 * wsum [No][No] accumulates the window.  Corners outside [0, No - Np] are
 * skipped.  acc and wsum start as the caller leaves them (normally zero). */
PTYG_API int ptyg_stitch(const void* patches, const int32_t* positions, int n, int Np, int No, const float* window,
                         void* acc, float* wsum, void* stream);
PTYG_API int ptyg_nn_adam(float* p, const float* g, float* m, float* v, void* p16, int64_t n, float lr, float b1,
                          float b2, float eps, int step, float weight_decay, void* stream);

/* Bounded-wait policy of the network kernels (ptyg_nn_gemm, _conv3,
 * _conv3_wgrad, _dense_wgrad): every mbarrier wait polls at most `polls`
 * times (default 2^26) before it gives up; the launch then sets its status
 * word to 1, stops issuing work, waits (bounded) for what it issued, frees
 * its tensor memory and returns, and the context stays usable.  With
 * stall_launches > 0 the next that many launches first wait on a barrier
 * nothing arrives at, before issuing any copy or MMA: fault injection for
 * failure-detection tests, so a timeout can be produced without a fault.
 * No counterpart in the reference (its failure handling is Python
 * exceptions, BaseEngine.py:376-403). */
PTYG_API int ptyg_nn_set_wait_policy(long long polls, int stall_launches);

/* ---------------------------------------------------------------------
 * FPM illumination calibration (PtyLab/Reconstruction/CalibrationFPM.py).
 * PtyLab runs it in NumPy/SciPy (IlluminationCalibration, :33-919); these
 * calls do its arithmetic, the host keeps its decisions.  Frames are
 * N x N float32 (N = 32, 64, 128 or 256), C order; all pointers are device
 * pointers unless marked host.
 *
 * ptyg_calib_spectra (convertToFourierSpace, :113-136 up to the mean):
 *   windowed[f] = float(frames[f] * window)  (window: N*N float64),
 *   frame_sums[f] = sum of windowed[f] (FP64),
 *   spectra[f] = ifft2c(windowed[f])  (complex64, n*N*N),
 *   ft[f] = |spectra[f]|, norm = mean over f of ft (float32, N*N).
 * ptyg_calib_normalise (:137-145): ft = |ft / max(norm, floor_value)|.
 * ptyg_calib_gaussian (skimage.filters.gaussian = scipy.ndimage.
 *   gaussian_filter, mode "nearest"): host half_weights[0..radius], the
 *   centre weight first; in == out allowed.
 * ptyg_calib_arcs (generateCircularArcsVectorized + map_coordinates +
 *   mean, :149-288, :482-495, :586-610): for task t, radius r and grid
 *   shift (a, b), the mean over the angles k kept in task_keep[t] (bit k)
 *   of images[task_image[t]] sampled bilinearly at
 *   (float(R_r sin_k + N/2 + p0 + a - search), float(R_r cos_k + N/2 + p1 + b - search)),
 *   p = task_pos[2t..2t+1]; out[t][r][a][b], float32; NaN when no angle is kept.
 *   Host arrays: radii (nradii <= 64), sin_angles, cos_angles (nangles <= 64).
 *   task_image[t] must index a frame of `images` (not checked on the device).
 * ptyg_calib_rms (calculateRMSE, :290-358): for candidate k,
 *   sqrt(mean((images[l] - |ifft2c(pupil_k * spectra[l])|)^2)), l = cand_led[k],
 *   pupil_k = ((i - N/2 + q0)^2 + (j - N/2 + q1)^2 <= radius^2),
 *   (q0, q1) = cand_q[2k..2k+1] (position + error, integers); rms[k] FP64;
 *   cand_led[k] must index a frame of `spectra` and `images`. */
PTYG_API int ptyg_calib_spectra(int n, int N, const float* frames, const double* window, float* windowed,
                                double* frame_sums, void* spectra, float* ft, float* norm, void* stream);
PTYG_API int ptyg_calib_normalise(int n, int N, float* ft, const float* norm, float floor_value, void* stream);
PTYG_API int ptyg_calib_gaussian(int n, int N, int radius, const double* half_weights, const float* in, float* out,
                                 void* stream);
PTYG_API int ptyg_calib_arcs(int N, const float* images, int ntasks, const int* task_image, const double* task_pos,
                             const unsigned long long* task_keep, int nradii, const double* radii, int nangles,
                             const double* sin_angles, const double* cos_angles, int search, float* out,
                             void* stream);
PTYG_API int ptyg_calib_rms(int N, const void* spectra, const float* images, int ncand, const int* cand_led,
                            const int* cand_q, double radius, double* rms, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PTYG_H */
