// Colloid trajectories on the device and their statistics: the analysis the
// reference's commented-out prints stood for (cpp/active_brownian.cpp:44-46), done
// without a host round trip per frame.
//
// A trajectory holds, per recorded frame, the colloids' unwrapped positions (the
// periodic image of each displacement since the previous frame added up), their
// velocities and their orientations, FP64, frame-major ([frame][colloid][xyz]).
// mpcd_traj_analyse reduces, per lag, over every time origin and colloid:
//   MSD(lag)  = < |U(t + lag) - U(t)|^2 >,  VACF(lag) = < V(t + lag) . V(t) >,
//   OACF(lag) = < ra(t + lag) . ra(t) >,
// one block per lag with a fixed reduction order, so the results are
// deterministic.  File layout (mpcd_traj_write), little-endian:
//   char magic[8] = "BGBTRAJ1"; int32 version (1), n_colloid, n_frames, fields (7:
//   position, velocity, orientation); double box[3], dt_frame; then per frame the
//   positions, the velocities and the orientations, n_colloid x 3 doubles each.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/brownian_gb300.h"
#include "traj_internal.h"

struct mpcd_traj {
  int Nc = 0, cap = 0, nframes = 0;
  double L[3] = {0, 0, 0};
  double *U = nullptr, *V = nullptr, *R = nullptr;  // [cap][Nc][3]
  double *last = nullptr;                           // [Nc][3] wrapped positions of the latest frame
  double *out = nullptr;                            // [3][nlags] analysis results
  int *lags = nullptr;
  int lag_cap = 0;
  std::string err;
};

namespace {

int tfail(mpcd_traj *t, int code, const std::string &m) {
  if (t) t->err = m;
  return code;
}

__device__ __forceinline__ double unwrap_step(double x, double prev, double L) {
  const double d = x - prev;
  return d - L * rint(d / L);
}

// frame f from FP64 triplet arrays (a context's colloid state)
__global__ void k_traj_rec64(int Nc, int f, double Lx, double Ly, double Lz, const double *X, const double *V,
                             const double *R, double *U, double *Vo, double *Ro, double *last) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // colloid * 3 + component
  if (i >= 3 * Nc) return;
  const int k = i % 3;
  const double L = k == 0 ? Lx : (k == 1 ? Ly : Lz);
  const double x = X[i];
  const size_t o = (size_t)f * 3 * Nc + i;
  U[o] = f == 0 ? x : U[o - 3 * (size_t)Nc] + unwrap_step(x, last[i], L);
  Vo[o] = V[i];
  Ro[o] = R[i];
  last[i] = x;
}

// frame f from float4 arrays (the colloid-only step's state)
__global__ void k_traj_rec4(int Nc, int f, double Lx, double Ly, double Lz, const float4 *X, const float4 *V,
                            const float4 *R, double *U, double *Vo, double *Ro, double *last) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * Nc) return;
  const int j = i / 3, k = i % 3;
  const double L = k == 0 ? Lx : (k == 1 ? Ly : Lz);
  const float4 x4 = X[j], v4 = V[j], r4 = R[j];
  const double x = (double)(k == 0 ? x4.x : (k == 1 ? x4.y : x4.z));
  const size_t o = (size_t)f * 3 * Nc + i;
  U[o] = f == 0 ? x : U[o - 3 * (size_t)Nc] + unwrap_step(x, last[i], L);
  Vo[o] = (double)(k == 0 ? v4.x : (k == 1 ? v4.y : v4.z));
  Ro[o] = (double)(k == 0 ? r4.x : (k == 1 ? r4.y : r4.z));
  last[i] = x;
}

// block l: the three averages at lag lags[l] (NaN where no pair of frames is that far apart)
__global__ void __launch_bounds__(256) k_traj_stats(int Nc, int F, const int *lags, int nlags, const double *U,
                                                    const double *V, const double *R, double *out) {
  __shared__ double red[3][256];
  const int l = blockIdx.x;
  const int lag = lags[l];
  const long long n = lag >= 0 && lag < F ? (long long)(F - lag) * Nc * 3 : 0;
  double a = 0, b = 0, c = 0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    const size_t o = (size_t)i, o2 = o + (size_t)lag * 3 * Nc;
    const double d = U[o2] - U[o];
    a += d * d;
    b += V[o2] * V[o];
    c += R[o2] * R[o];
  }
  red[0][threadIdx.x] = a;
  red[1][threadIdx.x] = b;
  red[2][threadIdx.x] = c;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int q = 0; q < 3; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double pairs = n > 0 ? (double)(F - lag) * Nc : 0.0;
    for (int q = 0; q < 3; ++q) out[q * nlags + l] = pairs > 0 ? red[q][0] / pairs : __longlong_as_double(0x7ff8000000000000ll);
  }
}

}  // namespace

int traj_record_f64(mpcd_traj *t, const double *X, const double *V, const double *R, cudaStream_t s) {
  if (!t || !X || !V || !R) return MPCD_ERR_PARAM;
  if (t->nframes >= t->cap) return tfail(t, MPCD_ERR_CAPACITY, "trajectory full");
  const int n3 = 3 * t->Nc;
  k_traj_rec64<<<(n3 + 127) / 128, 128, 0, s>>>(t->Nc, t->nframes, t->L[0], t->L[1], t->L[2], X, V, R, t->U, t->V,
                                                t->R, t->last);
  if (cudaGetLastError() != cudaSuccess) return tfail(t, MPCD_ERR_CUDA, "record launch");
  t->nframes += 1;
  return MPCD_OK;
}

int traj_record_f4(mpcd_traj *t, const float4 *X, const float4 *V, const float4 *R, cudaStream_t s) {
  if (!t || !X || !V || !R) return MPCD_ERR_PARAM;
  if (t->nframes >= t->cap) return tfail(t, MPCD_ERR_CAPACITY, "trajectory full");
  const int n3 = 3 * t->Nc;
  k_traj_rec4<<<(n3 + 127) / 128, 128, 0, s>>>(t->Nc, t->nframes, t->L[0], t->L[1], t->L[2], X, V, R, t->U, t->V,
                                               t->R, t->last);
  if (cudaGetLastError() != cudaSuccess) return tfail(t, MPCD_ERR_CUDA, "record launch");
  t->nframes += 1;
  return MPCD_OK;
}

int traj_colloids(const mpcd_traj *t) { return t ? t->Nc : -1; }

extern "C" int mpcd_traj_create(int n_colloid, int max_frames, const double *box, mpcd_traj **out) {
  if (!out || n_colloid < 1 || max_frames < 1 || !box || !(box[0] > 0) || !(box[1] > 0) || !(box[2] > 0))
    return MPCD_ERR_PARAM;
  *out = nullptr;
  mpcd_traj *t = new mpcd_traj();
  t->Nc = n_colloid;
  t->cap = max_frames;
  for (int k = 0; k < 3; ++k) t->L[k] = box[k];
  const size_t n = (size_t)max_frames * 3 * n_colloid;
  if (cudaMalloc(&t->U, n * sizeof(double)) != cudaSuccess || cudaMalloc(&t->V, n * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&t->R, n * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&t->last, 3 * (size_t)n_colloid * sizeof(double)) != cudaSuccess) {
    mpcd_traj_destroy(t);
    return MPCD_ERR_NOMEM;
  }
  *out = t;
  return MPCD_OK;
}

extern "C" int mpcd_traj_destroy(mpcd_traj *t) {
  if (!t) return MPCD_OK;
  for (void *p : {(void *)t->U, (void *)t->V, (void *)t->R, (void *)t->last, (void *)t->out, (void *)t->lags})
    if (p) cudaFree(p);
  delete t;
  return MPCD_OK;
}

extern "C" const char *mpcd_traj_last_error(const mpcd_traj *t) { return t ? t->err.c_str() : "null trajectory"; }

extern "C" int mpcd_traj_frames(const mpcd_traj *t) { return t ? t->nframes : -1; }

extern "C" int mpcd_traj_reset(mpcd_traj *t) {
  if (!t) return MPCD_ERR_PARAM;
  t->nframes = 0;
  return MPCD_OK;
}

extern "C" int mpcd_traj_analyse(mpcd_traj *t, const int *lags, int nlags, double *msd, double *vacf, double *oacf) {
  if (!t || !lags || nlags < 1) return MPCD_ERR_PARAM;
  cudaDeviceSynchronize();  // frames come from other streams
  if (nlags > t->lag_cap) {
    if (t->out) cudaFree(t->out);
    if (t->lags) cudaFree(t->lags);
    t->out = nullptr;
    t->lags = nullptr;
    if (cudaMalloc(&t->out, 3 * (size_t)nlags * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&t->lags, (size_t)nlags * sizeof(int)) != cudaSuccess)
      return tfail(t, MPCD_ERR_NOMEM, "analysis buffers");
    t->lag_cap = nlags;
  }
  if (cudaMemcpy(t->lags, lags, nlags * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
    return tfail(t, MPCD_ERR_CUDA, "lags upload");
  k_traj_stats<<<nlags, 256>>>(t->Nc, t->nframes, t->lags, nlags, t->U, t->V, t->R, t->out);
  std::vector<double> h(3 * (size_t)nlags);
  if (cudaMemcpy(h.data(), t->out, h.size() * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    return tfail(t, MPCD_ERR_CUDA, "analysis");
  for (int l = 0; l < nlags; ++l) {
    if (msd) msd[l] = h[l];
    if (vacf) vacf[l] = h[nlags + l];
    if (oacf) oacf[l] = h[2 * nlags + l];
  }
  return MPCD_OK;
}

extern "C" int mpcd_traj_read(mpcd_traj *t, int first, int count, double *pos, double *vel, double *ra) {
  if (!t || first < 0 || count < 0 || first + count > t->nframes) return MPCD_ERR_PARAM;
  cudaDeviceSynchronize();
  const size_t off = (size_t)first * 3 * t->Nc, n = (size_t)count * 3 * t->Nc * sizeof(double);
  if ((pos && cudaMemcpy(pos, t->U + off, n, cudaMemcpyDeviceToHost) != cudaSuccess) ||
      (vel && cudaMemcpy(vel, t->V + off, n, cudaMemcpyDeviceToHost) != cudaSuccess) ||
      (ra && cudaMemcpy(ra, t->R + off, n, cudaMemcpyDeviceToHost) != cudaSuccess))
    return tfail(t, MPCD_ERR_CUDA, "frame download");
  return MPCD_OK;
}

extern "C" int mpcd_traj_write(mpcd_traj *t, const char *path, double dt_frame) {
  if (!t || !path) return MPCD_ERR_PARAM;
  const size_t per = 3 * (size_t)t->Nc;
  std::vector<double> U(per * t->nframes), V(U.size()), R(U.size());
  int r = mpcd_traj_read(t, 0, t->nframes, U.data(), V.data(), R.data());
  if (r) return r;
  FILE *f = fopen(path, "wb");
  if (!f) return tfail(t, MPCD_ERR_PARAM, std::string("cannot open ") + path);
  const char magic[8] = {'B', 'G', 'B', 'T', 'R', 'A', 'J', '1'};
  const int32_t head[4] = {1, t->Nc, t->nframes, 7};
  const double geo[4] = {t->L[0], t->L[1], t->L[2], dt_frame};
  bool ok = fwrite(magic, 1, 8, f) == 8 && fwrite(head, sizeof head, 1, f) == 1 && fwrite(geo, sizeof geo, 1, f) == 1;
  for (int fr = 0; ok && fr < t->nframes; ++fr)
    ok = fwrite(U.data() + fr * per, sizeof(double), per, f) == per &&
         fwrite(V.data() + fr * per, sizeof(double), per, f) == per &&
         fwrite(R.data() + fr * per, sizeof(double), per, f) == per;
  ok = (fclose(f) == 0) && ok;
  return ok ? MPCD_OK : tfail(t, MPCD_ERR_PARAM, std::string("write failed: ") + path);
}
