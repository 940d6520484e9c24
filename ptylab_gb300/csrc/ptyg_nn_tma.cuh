// The TMA-fed 3x3 convolution of the warm-start network (ptyg_nn_tma.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace ptyg {
namespace nn {

struct ConvTmaArgs {
  int C0, C1;          // channels of the two concatenated inputs (C1 = 0: one input)
  int BK;              // channels per K block: 16, 32 or 64 (divides C0 and C1)
  int H, W;            // image size
  int BW, BH;          // pixel tile: BW x BH = 128 pixels of one image
  int tilesX, tilesY;  // W / BW, H / BH
  int N;               // output channels
  int kbPerTap, nkb;   // K blocks per tap, 9 * kbPerTap
  float* C;            // f32 output [pixels][N] (when out is null)
  __nv_bfloat16* out;  // bf16 output [pixels][N]
  const float* bias;   // + bias[n] (or null)
  int relu;            // bf16 output: max(0, .)
  int* status;         // set to 1 when a bounded wait gives up
  long long waitLimit; // try_wait polls before a wait is declared lost
  int stall;           // fault injection: the producer first waits on a barrier nothing arrives at
};

// The bounded-wait policy of the next launch (poll limit, injected stall).
void wait_policy(long long* limit, int* stall);

// Y = conv3x3(concat(X, X1), Wt) (+ bias, ReLU) with TMA operand loads;
// cudaErrorNotSupported when the shapes do not fit the tiling (the caller
// then uses the cp.async kernel).
cudaError_t conv3_tma(const void* X, const void* X1, int C0, int C1, int Bn, int H, int W, const void* Wt, int Co,
                      float* C, void* out, const float* bias, int relu, int* status, cudaStream_t st);

}  // namespace nn
}  // namespace ptyg
