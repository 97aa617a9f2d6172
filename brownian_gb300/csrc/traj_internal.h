// Recording into a trajectory (traj.cu) from the state of a context or of the
// colloid-only step, on their stream.
#pragma once
#include <cuda_runtime.h>

struct mpcd_traj;

int traj_record_f64(mpcd_traj *t, const double *X, const double *V, const double *R, cudaStream_t s);
int traj_record_f4(mpcd_traj *t, const float4 *X, const float4 *V, const float4 *R, cudaStream_t s);
int traj_colloids(const mpcd_traj *t);
