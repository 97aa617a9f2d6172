// Fluid momentum and kinetic energy of a caller's velocity array with no device
// allocation: the reduction of the diagnostics (k_diag_fluid, whose per-block
// partial sums live in memory a context allocates) with its partials in a
// fixed array of this file instead.
//
// Who needs it: a caller whose device memory is all handed out by its own pool
// (a framework's caching allocator that has already reserved the GPU, a fixed
// budget on an embedded or shared host), or one that must not take the device
// synchronisation that cudaMalloc / cudaFree can cause in the middle of its
// pipeline.  It passes its own input (velocities) and output (four doubles)
// and this call allocates nothing.
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "../../include/brownian_gb300.h"

namespace {

constexpr int kThreads = 256;
constexpr int kPerThread = 8;
constexpr int kPerBlock = kThreads * kPerThread;  // particles per block
constexpr int kMaxBlocks = 16384;                 // 512 KiB of partials

// Per-block partial sums (momentum x, y, z, sum |v|^2) of the last call.  Every
// GPU that loads the library holds this array until the process exits.  Each
// call writes every slot it reads, so nothing needs clearing between calls.
static __device__ __align__(256) double g_partials[kMaxBlocks * 4];

// block b: particles [b * kPerBlock, (b + 1) * kPerBlock), summed in a fixed order
__global__ void __launch_bounds__(kThreads) k_fluid_partials(const double *__restrict__ vel, long long n,
                                                             double *__restrict__ part) {
  __shared__ double sh[4][kThreads];
  double a[4] = {0, 0, 0, 0};
  const long long base = (long long)blockIdx.x * kPerBlock;
  for (int k = 0; k < kPerThread; ++k) {
    const long long i = base + (long long)k * kThreads + threadIdx.x;
    if (i < n) {
      const double x = vel[3 * i], y = vel[3 * i + 1], z = vel[3 * i + 2];
      a[0] += x; a[1] += y; a[2] += z;
      a[3] += x * x + y * y + z * z;
    }
  }
  for (int k = 0; k < 4; ++k) sh[k][threadIdx.x] = a[k];
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int k = 0; k < 4; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 4; ++k) part[4 * blockIdx.x + k] = sh[k][0];
}

// one block: the partials of `nblk` blocks in a fixed order -> out
__global__ void __launch_bounds__(kThreads) k_fluid_total(const double *__restrict__ part, int nblk, double mass,
                                                          double *__restrict__ out) {
  __shared__ double sh[4][kThreads];
  double a[4] = {0, 0, 0, 0};
  for (int b = threadIdx.x; b < nblk; b += kThreads)
    for (int k = 0; k < 4; ++k) a[k] += part[4 * b + k];
  for (int k = 0; k < 4; ++k) sh[k][threadIdx.x] = a[k];
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int k = 0; k < 4; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int k = 0; k < 3; ++k) out[k] = mass * sh[k][0];
    out[3] = 0.5 * mass * sh[3][0];
  }
}

// device address of g_partials, looked up once per device with that device current
// (the host-side name of the array is not a device address); it stays valid while the
// device's primary context lives, i.e. until a cudaDeviceReset of that device
constexpr int kMaxDevices = 64;
std::mutex g_setup_lock;
double *g_partials_dev[kMaxDevices] = {};

cudaError_t partials_for_current_device(double **ptr) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> hold(g_setup_lock);
  if (!g_partials_dev[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_partials);
    if (e != cudaSuccess) return e;
    g_partials_dev[dev] = static_cast<double *>(p);
  }
  *ptr = g_partials_dev[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" int mpcd_fluid_sums_noalloc(const double *vel, int64_t n, double mass, double *out, void *stream) {
  if (n < 0 || !out || (n > 0 && !vel)) return MPCD_ERR_PARAM;
  if (n > MPCD_NOALLOC_MAX_PARTICLES) {
    fprintf(stderr, "mpcd_fluid_sums_noalloc: %lld particles exceed the maximum of %lld\n", (long long)n,
            (long long)MPCD_NOALLOC_MAX_PARTICLES);
    return MPCD_ERR_CAPACITY;
  }
  // An error an earlier, unrelated launch left on this thread belongs to its owner: report it
  // without clearing it (cudaPeekAtLastError), and launch nothing.  With none pending, an
  // error after a launch below is that launch's own, and is read (and cleared) here.
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "mpcd_fluid_sums_noalloc: an earlier CUDA error is pending (%s); nothing launched\n",
            cudaGetErrorString(e));
    return MPCD_ERR_CUDA;
  }
  double *part = nullptr;
  if (partials_for_current_device(&part) != cudaSuccess) return MPCD_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nblk = n > 0 ? (int)((n + kPerBlock - 1) / kPerBlock) : 1;
  k_fluid_partials<<<nblk, kThreads, 0, s>>>(vel, n, part);
  if ((e = cudaGetLastError()) != cudaSuccess) {
    fprintf(stderr, "mpcd_fluid_sums_noalloc: partial-sum launch: %s\n", cudaGetErrorString(e));
    return MPCD_ERR_CUDA;
  }
  k_fluid_total<<<1, kThreads, 0, s>>>(part, nblk, mass, out);
  if ((e = cudaGetLastError()) != cudaSuccess) {
    fprintf(stderr, "mpcd_fluid_sums_noalloc: total launch: %s\n", cudaGetErrorString(e));
    return MPCD_ERR_CUDA;
  }
  return MPCD_OK;
}

static_assert((long long)kMaxBlocks * kPerBlock == MPCD_NOALLOC_MAX_PARTICLES, "limit and scratch size agree");
