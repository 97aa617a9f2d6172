// Internal interface between the closure network (mlp.cu) and the colloid-only
// step (surrogate.cu): the step writes the network's normalised BF16 inputs and
// reads its normalised outputs directly, so that one MPCD step is the network's
// four GEMMs and one dynamics kernel.
#pragma once
#include <cuda_runtime.h>

#include "../../include/brownian_gb300.h"

struct MlpIO {
  void *X;                     // normalised BF16 inputs [max_batch][MLP_IN_PADDED]
  const float *xmean, *xistd;  // input normalisation
  const float *O;              // normalised outputs [max_batch][MLP_OUT_PADDED]
  const float *ymean, *yistd;  // output normalisation
  int max_batch;
};
constexpr int MLP_IN_PADDED = 96, MLP_OUT_PADDED = 16;
constexpr float MLP_INPUT_CLIP = 6.f, MLP_LOGVAR_CLAMP = 6.f;

MlpIO mlp_io(mpcd_mlp *n);
// normalise raw inputs [rows][81] into X
int mlp_stage(mpcd_mlp *n, const float *x, int rows, cudaStream_t s);
// the four layers on rows of X into O
void mlp_layers(mpcd_mlp *n, int rows, cudaStream_t s);
