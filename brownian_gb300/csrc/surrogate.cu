// Colloid-only dynamics with the learned closure: the fluid is not simulated;
// each MPCD step the closure network predicts, from every colloid's features,
// the mean and log-variance of the momentum and angular momentum the fluid would
// give it, a Gaussian draw of that exchange is applied as an impulse, and the
// colloids then take the step's n_sub velocity-Verlet substeps with the WCA
// forces, the active kick (run(), cpp/run.cpp:13) and the orientation update
// (cpp/update.cpp:34-46, plus rotational diffusion Dr), in FP32.
//
// Per step: the network's forward pass (mlp.cu) on the features the previous step
// left, then k_sur_md (one block: the impulse and the active kick, the substeps,
// and the next step's features; the substeps need every colloid's new position,
// and a block barrier is the cheapest wait at these sizes).  The step is one CUDA
// graph.  k_sur_features computes the inputs of a state set from the host.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/brownian_gb300.h"
#include "traj_internal.h"
#include "common.cuh"
#include "mlp_internal.h"

namespace {

using namespace bgb;

constexpr int NF = MPCD_MLP_IN, NO = MPCD_MLP_OUT, KNEAR = 12, MAXC = MPCD_SURROGATE_MAX_COLLOIDS, MAXNB = 64;
constexpr uint32_t DOM_SUR_KICK = 20, DOM_SUR_ROT = 21;

struct Sur {
  int Nc, n_sub;
  float L[3], iL[3];
  float M, I, dt, v0, rotdiff_s, ct_feat2;
  float sig6, sig12, eps, rc2, fc, rlist2, half_skin2, rforce2;
  uint2 key;
  long long *step;  // device step counter
  float4 *X, *V, *W, *ra, *f;
  float *feat, *out;
  int *nbr, *nnb;
  float4 *xref;     // positions at the last neighbour-list build
  int *built;       // a list exists
  int *err;
  const float *On, *ymean, *yistd;  // the network's normalised outputs and their normalisation
};

__device__ __forceinline__ float wrapd(float d, float L, float iL) { return d - L * rintf(d * iL); }

__device__ __forceinline__ float u01f(uint32_t w) { return ((float)(w >> 9) + 0.5f) * 1.1920928955078125e-7f; }

// Box-Muller pair from two draws
__device__ __forceinline__ float2 normal2(uint32_t a, uint32_t b) {
  const float r = sqrtf(-2.f * __logf(u01f(a)));
  float s, c;
  __sincosf(6.283185307179586f * u01f(b), &s, &c);
  return make_float2(r * c, r * s);
}

// features of colloid j (one warp): V, Omega, ra, then the 12 nearest colloids
// within three radii (relative position, relative velocity), nearest first,
// ties by index, zero padded - the layout of brownian_gb300.closure.features
__global__ void __launch_bounds__(128) k_sur_features(const Sur S) {
  __shared__ float sd[4][64];
  __shared__ int sk[4][64];
  __shared__ int scnt[4];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * 4 + w;
  if (j >= S.Nc) return;
  if (lane == 0) scnt[w] = 0;
  __syncwarp();
  const float4 xj = S.X[j], vj = S.V[j];
  for (int k0 = 0; k0 < S.Nc; k0 += 32) {
    const int k = k0 + lane;
    float d2 = 1e30f;
    if (k < S.Nc && k != j) {
      const float4 xk = S.X[k];
      const float dx = wrapd(xk.x - xj.x, S.L[0], S.iL[0]), dy = wrapd(xk.y - xj.y, S.L[1], S.iL[1]),
                  dz = wrapd(xk.z - xj.z, S.L[2], S.iL[2]);
      d2 = dx * dx + dy * dy + dz * dz;
    }
    const bool in = d2 < S.ct_feat2;
    const unsigned m = __ballot_sync(0xFFFFFFFFu, in);
    int base = 0;
    if (m) {
      const int leader = __ffs(m) - 1;
      if (lane == leader) base = atomicAdd(&scnt[w], __popc(m));
      base = __shfl_sync(0xFFFFFFFFu, base, leader);
    }
    if (in) {
      const int slot = base + __popc(m & ((1u << lane) - 1u));
      if (slot < 64) {
        sd[w][slot] = d2;
        sk[w][slot] = k;
      }
    }
  }
  __syncwarp();
  const int cnt = min(scnt[w], 64);
  float *o = S.feat + (size_t)j * NF;
  const float4 wj = S.W[j], aj = S.ra[j];
  for (int c = lane; c < NF; c += 32) o[c] = 0.f;
  __syncwarp();
  if (lane == 0) {
    o[0] = vj.x; o[1] = vj.y; o[2] = vj.z; o[3] = wj.x; o[4] = wj.y; o[5] = wj.z; o[6] = aj.x; o[7] = aj.y; o[8] = aj.z;
  }
  for (int c = lane; c < cnt; c += 32) {
    const float d2 = sd[w][c];
    const int k = sk[w][c];
    int rank = 0;
    for (int e = 0; e < cnt; ++e) rank += (sd[w][e] < d2) || (sd[w][e] == d2 && sk[w][e] < k);
    if (rank < KNEAR) {
      const float4 xk = S.X[k], vk = S.V[k];
      float *q = o + 9 + 6 * rank;
      q[0] = wrapd(xk.x - xj.x, S.L[0], S.iL[0]);
      q[1] = wrapd(xk.y - xj.y, S.L[1], S.iL[1]);
      q[2] = wrapd(xk.z - xj.z, S.L[2], S.iL[2]);
      q[3] = vk.x - vj.x; q[4] = vk.y - vj.y; q[5] = vk.z - vj.z;
    }
  }
}

__device__ __forceinline__ float3 wca_pair(const Sur &S, float dx, float dy, float dz) {
  const float r2 = dx * dx + dy * dy + dz * dz;
  if (!(r2 < S.rc2)) return make_float3(0.f, 0.f, 0.f);
  const float r = sqrtf(r2), ir = 1.f / r, ir6 = 1.f / (r2 * r2 * r2);
  const float mag = 4.f * S.eps * (12.f * S.sig12 * ir6 * ir6 * ir - 6.f * S.sig6 * ir6 * ir) - S.fc;
  return make_float3(mag * dx * ir, mag * dy * ir, mag * dz * ir);
}

// One MPCD step of every colloid in one block (one or two colloids per thread,
// their velocity, angular velocity, orientation and force in registers, all
// positions and velocities in shared memory):
//   the fluid's exchange drawn from the network's Gaussian (its outputs S.On), applied in equal
//   parts after each substep's position update, and run()'s kick at the start;
//   the neighbour list (pairs within three radii plus a skin), rebuilt only when a
//   colloid has moved more than half the skin since the last build;
//   n_sub substeps of update_pos_md, update_activity_direction, compute_force_md,
//   update_velocity_colloid;
//   the network inputs of the next step (S.feat).
constexpr int MAXF = 24;  // force partners per colloid (within the WCA cutoff plus the skin)

template <int PER>  // colloids per thread: 1 up to 1024 colloids, 2 up to MAXC
__global__ void __launch_bounds__(1024) k_sur_md(const Sur S) {
  extern __shared__ float4 smem[];
  float4 *sX = smem, *sV = smem + MAXC;
  uint16_t *sF = reinterpret_cast<uint16_t *>(smem + 2 * MAXC);  // [MAXC][MAXF] force partners
  uint8_t *sFn = reinterpret_cast<uint8_t *>(sF + MAXC * MAXF);  // [MAXC] their count
  __shared__ int s_rebuild;
  const int T = blockDim.x, tid = threadIdx.x;
  float4 v[PER], w[PER], a[PER], fo[PER], pl[PER], pa[PER];
  const uint32_t step = (uint32_t)*S.step;
  if (tid == 0) s_rebuild = 0;
  __syncthreads();
#pragma unroll
  for (int u = 0; u < PER; ++u) {
    const int j = tid + T * u;
    if (j >= S.Nc) continue;
    const float4 x = S.X[j];
    sX[j] = x;
    v[u] = S.V[j]; w[u] = S.W[j]; a[u] = S.ra[j]; fo[u] = S.f[j];
    // the exchange and the active kick
    // the network's normalised outputs -> mean and standard deviation in physical units
    const float *o = S.On + (size_t)j * MLP_OUT_PADDED;
    const uint4 r0 = draw4(S.key, DOM_SUR_KICK, 0, (uint32_t)(j + 1), 0, step);
    const uint4 r1 = draw4(S.key, DOM_SUR_KICK, 1, (uint32_t)(j + 1), 0, step);
    const float2 g0 = normal2(r0.x, r0.y), g1 = normal2(r0.z, r0.w), g2 = normal2(r1.x, r1.y);
    const float xi[6] = {g0.x, g0.y, g1.x, g1.y, g2.x, g2.y};
    float dp[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const float is = S.yistd[k];
      const float lv = fminf(fmaxf(o[6 + k], -MLP_LOGVAR_CLAMP), MLP_LOGVAR_CLAMP);
      dp[k] = (o[k] + __expf(0.5f * lv) * xi[k]) / is + S.ymean[k];
    }
    // the exchange arrives over the step's substeps (the fluid collides every substep),
    // the active kick at its start (run())
    const float fm = 1.f / (S.M * S.n_sub), fi = 1.f / (S.I * S.n_sub);
    pl[u] = make_float4(dp[0] * fm, dp[1] * fm, dp[2] * fm, 0.f);
    pa[u] = make_float4(dp[3] * fi, dp[4] * fi, dp[5] * fi, 0.f);
    v[u].x += S.v0 * a[u].x; v[u].y += S.v0 * a[u].y; v[u].z += S.v0 * a[u].z;
    const float4 x0 = S.xref[j];
    const float dx = wrapd(x.x - x0.x, S.L[0], S.iL[0]), dy = wrapd(x.y - x0.y, S.L[1], S.iL[1]),
                dz = wrapd(x.z - x0.z, S.L[2], S.iL[2]);
    if (dx * dx + dy * dy + dz * dz > S.half_skin2 || *S.built == 0) s_rebuild = 1;
  }
  __syncthreads();
  if (s_rebuild) {
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int j = tid + T * u;
      if (j >= S.Nc) continue;
      int n = 0;
      const float4 xj = sX[j];
      for (int k = 0; k < S.Nc; ++k) {
        if (k == j) continue;
        const float4 xk = sX[k];
        const float dx = wrapd(xj.x - xk.x, S.L[0], S.iL[0]), dy = wrapd(xj.y - xk.y, S.L[1], S.iL[1]),
                    dz = wrapd(xj.z - xk.z, S.L[2], S.iL[2]);
        if (dx * dx + dy * dy + dz * dz < S.rlist2) {
          if (n < MAXNB) S.nbr[j * MAXNB + n] = k;
          else atomicOr(S.err, 1);
          ++n;
        }
      }
      S.nnb[j] = min(n, MAXNB);
      S.xref[j] = xj;
    }
    if (tid == 0) *S.built = 1;
  }
  // the force partners of this step (pairs within the cutoff plus the skin), in shared memory
#pragma unroll
  for (int u = 0; u < PER; ++u) {
    const int j = tid + T * u;
    if (j >= S.Nc) continue;
    const float4 xj = sX[j];
    const int n = S.nnb[j];
    int m = 0;
    for (int e = 0; e < n; ++e) {
      const int k = S.nbr[j * MAXNB + e];
      const float4 xk = sX[k];
      const float dx = wrapd(xj.x - xk.x, S.L[0], S.iL[0]), dy = wrapd(xj.y - xk.y, S.L[1], S.iL[1]),
                  dz = wrapd(xj.z - xk.z, S.L[2], S.iL[2]);
      if (dx * dx + dy * dy + dz * dz < S.rforce2) {
        if (m < MAXF) sF[j * MAXF + m] = (uint16_t)k;
        else atomicOr(S.err, 2);
        ++m;
      }
    }
    sFn[j] = (uint8_t)min(m, MAXF);
  }
  const float hdt2m = 0.5f * S.dt * S.dt / S.M, hdtm = 0.5f * S.dt / S.M;
  for (int l = 0; l < S.n_sub; ++l) {
    __syncthreads();
#pragma unroll
    for (int u = 0; u < PER; ++u) {  // update_pos_md
      const int j = tid + T * u;
      if (j >= S.Nc) continue;
      float4 x = sX[j];
      x.x += v[u].x * S.dt + fo[u].x * hdt2m; x.y += v[u].y * S.dt + fo[u].y * hdt2m;
      x.z += v[u].z * S.dt + fo[u].z * hdt2m;
      x.x -= S.L[0] * floorf(x.x * S.iL[0]); x.y -= S.L[1] * floorf(x.y * S.iL[1]); x.z -= S.L[2] * floorf(x.z * S.iL[2]);
      sX[j] = x;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int j = tid + T * u;
      if (j >= S.Nc) continue;
      // this substep's share of the fluid exchange (fluid_colloid_collision)
      v[u].x += pl[u].x; v[u].y += pl[u].y; v[u].z += pl[u].z;
      w[u].x += pa[u].x; w[u].y += pa[u].y; w[u].z += pa[u].z;
      // update_activity_direction: the Euler matrix of Omega dt, then rotational diffusion
      float sx, cx, sy, cy, sz, cz;
      __sincosf(w[u].x * S.dt, &sx, &cx); __sincosf(w[u].y * S.dt, &sy, &cy); __sincosf(w[u].z * S.dt, &sz, &cz);
      const float4 aa = a[u];
      float ax = cy * cz * aa.x - cy * sz * aa.y + sy * aa.z;
      float ay = (sx * sy * cz + cx * sz) * aa.x + (-sx * sy * sz + cx * cz) * aa.y - sx * cy * aa.z;
      float az = (-cx * sy * cz + sx * sz) * aa.x + (cx * sy * sz + sx * cz) * aa.y + cx * cy * aa.z;
      if (S.rotdiff_s > 0.f) {
        const uint4 r = draw4(S.key, DOM_SUR_ROT, 0, (uint32_t)(j + 1), 0, step * S.n_sub + l);
        const float2 g0 = normal2(r.x, r.y), g1 = normal2(r.z, r.w);
        const float d = g0.x * ax + g0.y * ay + g1.x * az;
        ax += S.rotdiff_s * (g0.x - d * ax); ay += S.rotdiff_s * (g0.y - d * ay); az += S.rotdiff_s * (g1.x - d * az);
      }
      const float in = rsqrtf(ax * ax + ay * ay + az * az);
      a[u] = make_float4(ax * in, ay * in, az * in, 0.f);
      // compute_force_md at the new positions, update_velocity_colloid
      float3 fn = make_float3(0.f, 0.f, 0.f);
      const float4 xj = sX[j];
      const int n = sFn[j];
      for (int e = 0; e < n; ++e) {
        const float4 xk = sX[sF[j * MAXF + e]];
        const float3 fp = wca_pair(S, wrapd(xj.x - xk.x, S.L[0], S.iL[0]), wrapd(xj.y - xk.y, S.L[1], S.iL[1]),
                                   wrapd(xj.z - xk.z, S.L[2], S.iL[2]));
        fn.x += fp.x; fn.y += fp.y; fn.z += fp.z;
      }
      v[u].x += (fo[u].x + fn.x) * hdtm; v[u].y += (fo[u].y + fn.y) * hdtm; v[u].z += (fo[u].z + fn.z) * hdtm;
      fo[u] = make_float4(fn.x, fn.y, fn.z, 0.f);
    }
  }
#pragma unroll
  for (int u = 0; u < PER; ++u) {
    const int j = tid + T * u;
    if (j >= S.Nc) continue;
    sV[j] = v[u];
    S.X[j] = sX[j]; S.V[j] = v[u]; S.W[j] = w[u]; S.ra[j] = a[u]; S.f[j] = fo[u];
  }
  __syncthreads();
  // the next step's network inputs: the 12 nearest colloids within three radii from the list
#pragma unroll
  for (int u = 0; u < PER; ++u) {
    const int j = tid + T * u;
    if (j >= S.Nc) continue;
    // the nearest KNEAR as (d2, k) in registers: every candidate is passed down a
    // fully unrolled chain of compare-and-swap, nearest (then lowest index) first
    float bd[KNEAR];
    int bk[KNEAR];
#pragma unroll
    for (int m = 0; m < KNEAR; ++m) { bd[m] = 3.0e38f; bk[m] = 0x7FFFFFFF; }
    const float4 xj = sX[j];
    const int n = S.nnb[j];
    for (int e = 0; e < n; ++e) {
      int k = S.nbr[j * MAXNB + e];
      const float4 xk = sX[k];
      const float dx = wrapd(xk.x - xj.x, S.L[0], S.iL[0]), dy = wrapd(xk.y - xj.y, S.L[1], S.iL[1]),
                  dz = wrapd(xk.z - xj.z, S.L[2], S.iL[2]);
      float d2 = dx * dx + dy * dy + dz * dz;
      if (!(d2 < S.ct_feat2)) continue;
#pragma unroll
      for (int m = 0; m < KNEAR; ++m) {
        const bool less = d2 < bd[m] || (d2 == bd[m] && k < bk[m]);
        const float td = less ? bd[m] : d2;
        const int tk = less ? bk[m] : k;
        bd[m] = less ? d2 : bd[m];
        bk[m] = less ? k : bk[m];
        d2 = td;
        k = tk;
      }
    }
    float *o = S.feat + (size_t)j * NF;
    o[0] = v[u].x; o[1] = v[u].y; o[2] = v[u].z; o[3] = w[u].x; o[4] = w[u].y; o[5] = w[u].z;
    o[6] = a[u].x; o[7] = a[u].y; o[8] = a[u].z;
#pragma unroll
    for (int m = 0; m < KNEAR; ++m) {
      float *q = o + 9 + 6 * m;
      if (bk[m] != 0x7FFFFFFF) {
        const float4 xk = sX[bk[m]], vk = sV[bk[m]];
        q[0] = wrapd(xk.x - xj.x, S.L[0], S.iL[0]); q[1] = wrapd(xk.y - xj.y, S.L[1], S.iL[1]);
        q[2] = wrapd(xk.z - xj.z, S.L[2], S.iL[2]);
        q[3] = vk.x - v[u].x; q[4] = vk.y - v[u].y; q[5] = vk.z - v[u].z;
      } else {
        q[0] = q[1] = q[2] = q[3] = q[4] = q[5] = 0.f;
      }
    }
  }
  if (tid == 0) *S.step += 1;
}

__global__ void k_sur_forces(const Sur S) {
  // forces at the current positions (the set-up's compute_force_md), all pairs
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= S.Nc) return;
  float3 fj = make_float3(0.f, 0.f, 0.f);
  const float4 xj = S.X[j];
  for (int k = 0; k < S.Nc; ++k) {
    if (k == j) continue;
    const float4 xk = S.X[k];
    const float dx = wrapd(xj.x - xk.x, S.L[0], S.iL[0]), dy = wrapd(xj.y - xk.y, S.L[1], S.iL[1]),
                dz = wrapd(xj.z - xk.z, S.L[2], S.iL[2]);
    const float r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < S.rc2) {
      const float r = sqrtf(r2), ir = 1.f / r, ir6 = 1.f / (r2 * r2 * r2);
      const float mag = 4.f * S.eps * (12.f * S.sig12 * ir6 * ir6 * ir - 6.f * S.sig6 * ir6 * ir) - S.fc;
      fj.x += mag * dx * ir; fj.y += mag * dy * ir; fj.z += mag * dz * ir;
    }
  }
  S.f[j] = make_float4(fj.x, fj.y, fj.z, 0.f);
}

}  // namespace

struct mpcd_surrogate {
  Sur S;
  mpcd_mlp *net = nullptr;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<void *> allocs;
  std::string err;
};

namespace {

int sfail(mpcd_surrogate *s, int code, const std::string &e) {
  if (s) s->err = e;
  return code;
}

template <typename T>
T *salloc(mpcd_surrogate *s, size_t n) {
  void *p = nullptr;
  if (cudaMalloc(&p, n * sizeof(T) + 64) != cudaSuccess) {
    s->err = "out of device memory";
    return nullptr;
  }
  cudaMemset(p, 0, n * sizeof(T) + 64);
  s->allocs.push_back(p);
  return static_cast<T *>(p);
}

constexpr size_t kSmem = 2 * MAXC * sizeof(float4) + MAXC * MAXF * sizeof(uint16_t) + MAXC;

int enqueue_step(mpcd_surrogate *s) {
  const Sur &S = s->S;
  // S.feat holds the current state's network inputs (set_state, or the previous step)
  int r = mlp_stage(s->net, S.feat, S.Nc, s->stream);
  if (r) return sfail(s, r, std::string("closure network: ") + mpcd_mlp_last_error(s->net));
  mlp_layers(s->net, S.Nc, s->stream);
  if (S.Nc <= 1024) k_sur_md<1><<<1, 1024, kSmem, s->stream>>>(S);
  else k_sur_md<2><<<1, 1024, kSmem, s->stream>>>(S);
  return MPCD_OK;
}

}  // namespace

extern "C" int mpcd_surrogate_create(const mpcd_params *p, mpcd_mlp *net, mpcd_surrogate **out) {
  if (!p || !net || !out) return MPCD_ERR_PARAM;
  *out = nullptr;
  if (p->n_colloid < 1 || p->n_colloid > MAXC || p->n_sub < 1 || !(p->ndt > 0) || !(p->mass_colloid > 0) ||
      !(p->I_colloid > 0) || p->Lx < 1 || p->Ly < 1 || p->Lz < 1)
    return MPCD_ERR_PARAM;
  if (mlp_io(net).max_batch < p->n_colloid) return MPCD_ERR_CAPACITY;
  mpcd_surrogate *s = new mpcd_surrogate();
  s->net = net;
  Sur &S = s->S;
  memset(&S, 0, sizeof S);
  const MlpIO io = mlp_io(net);
  S.On = io.O;
  S.ymean = io.ymean;
  S.yistd = io.yistd;
  S.Nc = p->n_colloid;
  S.n_sub = p->n_sub;
  const int Ls[3] = {p->Lx, p->Ly, p->Lz};
  for (int k = 0; k < 3; ++k) {
    S.L[k] = (float)Ls[k];
    S.iL[k] = 1.f / (float)Ls[k];
  }
  S.M = (float)p->mass_colloid;
  S.I = (float)p->I_colloid;
  const double dt = p->ndt / p->n_sub;
  S.dt = (float)dt;
  S.v0 = (float)p->v0;
  S.rotdiff_s = (float)std::sqrt(2.0 * p->Dr * dt);
  const double radius = 0.5 * p->sigma;
  S.ct_feat2 = (float)(9.0 * radius * radius);
  const double rc = std::pow(2.0, 1.0 / 6.0) * p->sig_colloid;  // cpp/update.cpp:3
  S.rc2 = (float)(rc * rc);
  S.sig6 = (float)std::pow(p->sig_colloid, 6);
  S.sig12 = (float)std::pow(p->sig_colloid, 12);
  S.eps = (float)p->eps;
  S.fc = (float)(4.0 * p->eps * (12.0 * (std::pow(p->sig_colloid, 12) / std::pow(rc, 13)) -
                                 6.0 * (std::pow(p->sig_colloid, 6) / std::pow(rc, 7))));  // cpp/update.cpp:4
  // the list serves the forces (rc) and the features (three radii); skin 1
  const double rl = (rc > 3.0 * radius ? rc : 3.0 * radius) + 1.0;
  S.rlist2 = (float)(rl * rl);
  S.half_skin2 = 0.25f;
  S.rforce2 = (float)((rc + 1.0) * (rc + 1.0));
  S.key = make_uint2((uint32_t)p->seed, (uint32_t)(p->seed >> 32));
  const size_t Nc = S.Nc;
  S.step = salloc<long long>(s, 1);
  S.X = salloc<float4>(s, Nc); S.V = salloc<float4>(s, Nc); S.W = salloc<float4>(s, Nc);
  S.ra = salloc<float4>(s, Nc); S.f = salloc<float4>(s, Nc);
  S.feat = salloc<float>(s, Nc * NF); S.out = salloc<float>(s, Nc * NO);
  S.nbr = salloc<int>(s, Nc * MAXNB); S.nnb = salloc<int>(s, Nc);
  S.xref = salloc<float4>(s, Nc); S.built = salloc<int>(s, 1);
  S.err = salloc<int>(s, 1);
  if (!s->err.empty() || cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaFuncSetAttribute(k_sur_md<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem) != cudaSuccess ||
      cudaFuncSetAttribute(k_sur_md<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem) != cudaSuccess) {
    mpcd_surrogate_destroy(s);
    return MPCD_ERR_NOMEM;
  }
  *out = s;
  return MPCD_OK;
}

extern "C" int mpcd_surrogate_destroy(mpcd_surrogate *s) {
  if (!s) return MPCD_ERR_PARAM;
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->exec) cudaGraphExecDestroy(s->exec);
  for (void *a : s->allocs) cudaFree(a);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return MPCD_OK;
}

extern "C" const char *mpcd_surrogate_last_error(const mpcd_surrogate *s) { return s ? s->err.c_str() : "null"; }

extern "C" int mpcd_surrogate_set_state(mpcd_surrogate *s, const double *pos, const double *vel, const double *ang_vel,
                                        const double *ra) {
  if (!s || !pos || !vel || !ang_vel || !ra) return MPCD_ERR_PARAM;
  const Sur &S = s->S;
  const double *src[4] = {pos, vel, ang_vel, ra};
  float4 *dst[4] = {S.X, S.V, S.W, S.ra};
  std::vector<float4> h(S.Nc);
  for (int a = 0; a < 4; ++a) {
    for (int j = 0; j < S.Nc; ++j) {
      double v[3] = {src[a][3 * j], src[a][3 * j + 1], src[a][3 * j + 2]};
      if (a == 0)
        for (int k = 0; k < 3; ++k) v[k] -= S.L[k] * std::floor(v[k] / S.L[k]);
      h[j] = make_float4((float)v[0], (float)v[1], (float)v[2], 0.f);
    }
    if (cudaMemcpyAsync(dst[a], h.data(), sizeof(float4) * S.Nc, cudaMemcpyHostToDevice, s->stream) != cudaSuccess ||
        cudaStreamSynchronize(s->stream) != cudaSuccess)
      return sfail(s, MPCD_ERR_CUDA, "state upload");
  }
  k_sur_forces<<<(S.Nc + 127) / 128, 128, 0, s->stream>>>(S);
  k_sur_features<<<(S.Nc + 3) / 4, 128, 0, s->stream>>>(S);
  if (cudaMemsetAsync(S.built, 0, sizeof(int), s->stream) != cudaSuccess) return sfail(s, MPCD_ERR_CUDA, "set-up");
  return cudaStreamSynchronize(s->stream) == cudaSuccess ? MPCD_OK : sfail(s, MPCD_ERR_CUDA, "set-up forces");
}

extern "C" int mpcd_surrogate_get_state(mpcd_surrogate *s, double *pos, double *vel, double *ang_vel, double *ra) {
  if (!s) return MPCD_ERR_PARAM;
  const Sur &S = s->S;
  double *dst[4] = {pos, vel, ang_vel, ra};
  const float4 *src[4] = {S.X, S.V, S.W, S.ra};
  std::vector<float4> h(S.Nc);
  for (int a = 0; a < 4; ++a) {
    if (!dst[a]) continue;
    if (cudaMemcpyAsync(h.data(), src[a], sizeof(float4) * S.Nc, cudaMemcpyDeviceToHost, s->stream) != cudaSuccess ||
        cudaStreamSynchronize(s->stream) != cudaSuccess)
      return sfail(s, MPCD_ERR_CUDA, "state download");
    for (int j = 0; j < S.Nc; ++j) {
      dst[a][3 * j] = h[j].x; dst[a][3 * j + 1] = h[j].y; dst[a][3 * j + 2] = h[j].z;
    }
  }
  return MPCD_OK;
}

// a trajectory frame of the colloid-only step's state
extern "C" int mpcd_traj_record_surrogate(mpcd_traj *t, mpcd_surrogate *s) {
  if (!s || !t || traj_colloids(t) != s->S.Nc) return MPCD_ERR_PARAM;
  const int r = traj_record_f4(t, s->S.X, s->S.V, s->S.ra, s->stream);
  return r ? sfail(s, r, mpcd_traj_last_error(t)) : MPCD_OK;
}

extern "C" int mpcd_surrogate_features(mpcd_surrogate *s, float *out, int recompute) {
  if (!s || !out) return MPCD_ERR_PARAM;
  const Sur &S = s->S;
  if (recompute) k_sur_features<<<(S.Nc + 3) / 4, 128, 0, s->stream>>>(S);
  if (cudaMemcpyAsync(out, S.feat, sizeof(float) * NF * S.Nc, cudaMemcpyDeviceToHost, s->stream) != cudaSuccess ||
      cudaStreamSynchronize(s->stream) != cudaSuccess)
    return sfail(s, MPCD_ERR_CUDA, "features");
  return MPCD_OK;
}

extern "C" int mpcd_surrogate_step(mpcd_surrogate *s, int nsteps) {
  if (!s || nsteps < 0) return MPCD_ERR_PARAM;
  if (!s->exec) {
    cudaGraph_t g;
    if (cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return sfail(s, MPCD_ERR_CUDA, "capture");
    int r = enqueue_step(s);
    cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    if (r) return r;
    if (e != cudaSuccess) return sfail(s, MPCD_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&s->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return sfail(s, MPCD_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
  }
  for (int i = 0; i < nsteps; ++i)
    if (cudaGraphLaunch(s->exec, s->stream) != cudaSuccess) return sfail(s, MPCD_ERR_CUDA, "graph launch");
  int bits = 0;
  if (cudaMemcpyAsync(&bits, s->S.err, sizeof(int), cudaMemcpyDeviceToHost, s->stream) != cudaSuccess ||
      cudaStreamSynchronize(s->stream) != cudaSuccess)
    return sfail(s, MPCD_ERR_CUDA, std::string("step: ") + cudaGetErrorString(cudaGetLastError()));
  if (bits) return sfail(s, MPCD_ERR_CAPACITY, "a colloid has more neighbours than its lists hold (64 within three "
                                             "radii plus the skin, 24 within the force cutoff plus the skin)");
  return MPCD_OK;
}
