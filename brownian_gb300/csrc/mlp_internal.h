// Internal interface between the closure network (mlp.cu) and the colloid-only
// step (surrogate.cu): the step reads the network's weights, biases and
// normalisation directly and evaluates the network inside its own kernel.
#pragma once
#include <cuda_runtime.h>

#include "../../include/brownian_gb300.h"

struct MlpIO {
  const float *xmean, *xistd;  // input normalisation
  const float *ymean, *yistd;  // output normalisation
  const void *w[4];            // BF16 weights [k][n] of the four layers (96 x 256, 256 x 256 twice, 256 x 16)
  const float *bias;           // FP32 biases, 256 + 256 + 256 + 16
};
constexpr int MLP_IN_PADDED = 96, MLP_OUT_PADDED = 16;
constexpr float MLP_INPUT_CLIP = 6.f, MLP_LOGVAR_CLAMP = 6.f;

MlpIO mlp_io(mpcd_mlp *n);
