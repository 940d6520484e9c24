// Device-side argument blocks of the persistent position-loop kernel.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ptyg {

enum Engine { ENG_EPIE = 0, ENG_MPIE = 1, ENG_QNEWTON = 2, ENG_E3PIE = 3, ENG_MQNEWTON = 4 };
enum Momentum { MOM_PLAIN = 0, MOM_ADAM = 1, MOM_NADAM = 2 };
// params.intensityConstraint (BaseEngine.py:913-961)
enum IntensityConstraint { IC_STANDARD = 0, IC_POISSON = 1, IC_EXPONENTIAL = 2, IC_FLUCTUATION = 3, IC_INTERFEROMETRIC = 4 };

// Object modes the pixel-update loop carries in registers.
constexpr int MAX_OBJECT_MODES = 4;
enum Propagator { PROP_FRAUNHOFER = 0, PROP_FRESNEL = 1, PROP_ASP = 2 };

// Reduction slots (unsigned bit patterns of non-negative floats, max-reduced
// with atomicMax), two banks alternating by position parity.
enum RedSlot {
  RED_PMAX2 = 0,   // max_xy sum_p |P_p|^2
  RED_OMAX2 = 1,   // max_xy sum_o |O_o|^2 over the patch
  RED_PMAX1 = 2,   // max_xy sum_p |P_p|        (qNewton)
  RED_OMAXW = 3,   // max over the whole object of sum_o |O_o| (qNewton)
  RED_SLICE_P = 4, // e3PIE: max_xy sum_p |P_s|^2, slices 0..5
  RED_SLICE_O = 10,// e3PIE: max_xy sum_o |O_s|^2, slices 0..5
  RED_BANK = 16
};

// Per-scan device state.  Object/probe/buffers/positions/order belong to the
// caller; work/esw/err/detErr/red/status belong to the plan.
struct ScanDev {
  float2* object;          // (nosm, nslice, No, No)
  float2* probe;           // (npsm, nslice, Np, Np)
  const float* data;       // Fraunhofer/Fresnel: [frame][sx][sy] Fourier layout; ASP: [frame][y][x]
  const int* positions;    // [frame][2] = (row, col) of the patch corner
  const int* order;        // scan order; a launch reads order[start .. start+count)
  const uint8_t* momentum; // mPIE: momentum flag per order slot
  float2* objectBuffer;
  float2* objectMomentum;
  float2* probeBuffer;
  float2* probeMomentum;
  float2* work;            // transposition buffer, K * Np * Np
  float2* eswStore;        // e3PIE: forward exit waves, nslice * npsm * Np * Np
  double* errPart;         // [frame][cluster] partial sums of |I_meas - I_est|
  float* detErr;           // optional [frame][Np*Np] |I_meas - I_est| (data layout)
  unsigned* red;           // 2 * RED_BANK reduction slots
  int* status;             // 0 = ok, else first error code seen
  float* tileMax;          // qNewton/mqNewton: max of sum_o |O_o| per TILE x TILE object tile
  float* moment2;          // mqNewton ADAM/NADAM: {v_object, v_probe}
  int vec4;                // No even and object / objectMomentum 16-byte aligned: 16-byte accesses
  float* background;       // backgroundModeSwitch: Np x Np, data layout (plan-owned)
  double* iscale;          // 'fluctuation': per-frame intensity scaling aleph (plan-owned)
  float2* reference;       // 'interferometric': K planes of Np x Np, data layout, scaled N * M * R (plan-owned)
};

// Side of the object tiles whose maxima qNewton keeps up to date.
constexpr int TILE = 16;

struct EngineArgs {
  const ScanDev* scans;
  const float2* twiddle;   // W_Np^m, m = 0..Np-1
  const float2* fresnelQ;  // Fresnel chirp, natural [y][x]
  const float2* aspH;      // ASP detector TF (ifftshifted), Fourier layout [sx][sy]; one per wavelength
  const float2* sliceH;    // e3PIE slice TF (ifftshifted), Fourier layout [sx][sy]
  int Np, No, nosm, npsm, nslice, numFrames;
  // wavelengths (ePIE only when > 1): object modes (l, o) and probe modes
  // (l, p) lie wavelength-major in memory, the exit waves are the nlambda x
  // nosm x npsm products O_(l,o) P_(l,p)
  int nlambda;
  int engine, prop, centred, fpm;
  int start, count;
  int writeDetErr;
  int cluster;
  int tilesPerRow;         // ceil(No / TILE)
  int probeInSmem;         // keep the CTA's probe rows in shared memory
  int hInSmem;             // ASP: copy the CTA's columns of aspH (each wavelength's) into shared memory
  float betaO, betaP, alphaO, alphaP, regO, regP, frictionM, feedbackM, weightP, bethSlice;
  // mqNewton: method, float32 beta1, 1-beta1, beta2, 1-beta2, 1-beta^itr, step sizes
  int momentum;
  float b1, omb1, b2, omb2, b1s, b2s, betaOm, betaPm;
  // intensity projection switches (BaseEngine.py:870-1012): constraint,
  // adaptive denoising, background mode, Fourier-mask error weights,
  // intensity mask; tables in the data layout (Np x Np)
  int iconstraint, denoise, bgMode, fmask, imask;
  float invFrames;         // 1 / numFrames (background update)
  const float* W;          // experimentalData.W
  const float* imaskTab;   // reconstruction.intensity_mask
};

}  // namespace ptyg
