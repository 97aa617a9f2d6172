// Colloid-only dynamics with the learned closure: the fluid is not simulated;
// each MPCD step the closure network predicts, from every colloid's features,
// the mean and log-variance of the momentum and angular momentum the fluid would
// give it, a Gaussian draw of that exchange is applied as an impulse, and the
// colloids then take the step's n_sub velocity-Verlet substeps with the WCA
// forces, the active kick (run(), cpp/run.cpp:13) and the orientation update
// (cpp/update.cpp:34-46, plus rotational diffusion Dr), in FP32.
//
// Per step, two kernels (one CUDA graph):
//   k_sur_net, one block per 16 colloids over the whole GPU (16 compute warps, one
//     producer warp): each colloid's neighbours (from candidate lists kept with a
//     skin, all pairs when they expire), its 81 network inputs and its force partners
//     for the step, the whole network (four layers, BF16 mma.sync with FP32
//     accumulation, activations in shared memory, the weights streamed through a
//     ring of shared-memory stages by bulk copies while the block computes), the
//     Gaussian draw of the exchange, the step's rotational-diffusion draws and the
//     orientation through the substeps;
//   the substeps, k_sur_md1 (one block, up to 1024 colloids) or k_sur_md (one cluster
//     of 8 blocks): the active kick and the n_sub velocity-Verlet substeps (each needs
//     every colloid's new position: a block barrier, or distributed shared memory and
//     one cluster barrier, per substep).
// The packed weights (the layout k_sur_net reads) are rebuilt from the network at
// every mpcd_surrogate_step call.  k_sur_features computes the inputs of the
// current state on request.
#include <cooperative_groups.h>
#include <cuda_bf16.h>

#include <algorithm>
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
typedef __nv_bfloat16 bf16;

constexpr int NF = MPCD_MLP_IN, NO = MPCD_MLP_OUT, KNEAR = 12, MAXC = MPCD_SURROGATE_MAX_COLLOIDS, CAND = 64;
constexpr int H = MPCD_MLP_HIDDEN, INP = MLP_IN_PADDED, OUTP = MLP_OUT_PADDED;
constexpr uint32_t DOM_SUR_KICK = 20, DOM_SUR_ROT = 21;
constexpr int MAXF = 32;  // force partners per colloid (within the WCA cutoff plus the skin)

struct Sur {
  int Nc, n_sub;
  float L[3], iL[3];
  float M, I, dt, v0, rotdiff_s, ct_feat2;
  float sig6, sig12, eps, rc2, fc, rscan2, rlist2, half_skin2;
  float rc;          // WCA cutoff
  float *vmax;       // the largest colloid speed at the end of the last step
  long long *fast;   // steps in which a colloid moved more than half the step's partner skin
  uint2 key;
  long long *step;  // device step counter
  float4 *X, *V, *W, *ra, *f;
  float *feat;      // the last step's network inputs [Nc][81]
  float *out;       // the last step's normalised network outputs [Nc][16]
  float4 *imp;      // per-substep linear impulse of the drawn exchange [Nc], orientation at the step's start [Nc],
                    // Omega and orientation at the step's end [Nc] [Nc] (stored by the substep kernel)
  uint16_t *fpart;  // force partners [Nc][MAXF], ascending index
  uint8_t *fpn;     // their count
  uint16_t *nbl;    // candidate neighbours [Nc][CAND] (within rlist at the last rebuild), ascending index
  int *nbn;         // their count
  float4 *xref;     // positions at the last rebuild
  int *rebuild;     // a colloid moved more than half the skin since (or no lists yet)
  int *err;
  int drop_chunk;   // fault injection for tests: the producer does not issue this weight chunk (-1: none)
  float noise;      // scale of the drawn exchange's fluctuation (1: the network's variance, 0: its mean only)
  const uint4 *wpk;                   // the packed BF16 weights (k_sur_pack)
  const float *bias;                  // the network's biases [256][256][256][16]
  const float *xmean, *xistd;         // input normalisation
  const float *ymean, *yistd;         // output normalisation
};

__device__ __forceinline__ float wrapd(float d, float L, float iL) { return d - L * rintf(d * iL); }

// the skin of a step's force partners (pairs within the cutoff plus it): 2.5 times the
// largest displacement the last step's speeds give, within [0.5, 2]; the candidate lists
// cover the largest
__device__ __forceinline__ float partner_skin(const Sur &S) {
  return fminf(fmaxf(2.5f * *S.vmax * S.dt * S.n_sub, 0.5f), 2.0f);
}


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

// ---- the network block ---------------------------------------------------------
// Weights in fragment order: chunk g holds, for every 8-column tile t of a layer and
// lane l, one 16-byte word with the lane's mma.sync B fragments of two consecutive
// 16-deep K steps (k0 = 32 c + 2 (l & 3), rows k0 + {0, 1}, + 8, + 16, + 24 of column
// 8 t + (l >> 2)), so that a warp's fragments are one conflict-free 16-byte shared
// load each.  Chunks 0-2: layer 1 (K 96), 3-10: layer 2, 11-18: layer 3 (32 K rows
// x 256 columns, 16 KB each), 19: layer 4 (K 256 x 16 columns, 8 KB).
constexpr int ROWS = 16, NCW = 16, TPW = 32 / NCW, NET_THREADS = 32 * (NCW + 1), CHUNK_U4 = 1024, NCHUNK = 20, NSTAGE = 6,
              LDA = H + 8;
constexpr int PACK_U4 = 19 * CHUNK_U4 + 512;
static_assert(ROWS == NCW, "one row per compute warp");

constexpr int MAXSUB = 32;  // substeps per MPCD step the colloid-only step supports

struct __align__(128) NetSmem {
  uint4 ring[NSTAGE][CHUNK_U4];
  union {
    float4 xall[MAXC];  // every colloid's position (candidate-list rebuilds)
    struct {
      float4 cx[ROWS][CAND], cv[ROWS][CAND];  // the candidates' positions and velocities
    } c;
  } u;
  float4 nz[ROWS][MAXSUB];     // rotational-diffusion Gaussians of the step's substeps
  float4 rm[ROWS][MAXSUB][3];  // the Euler matrix of Omega dt per substep (rows)
  float4 row[4][ROWS];       // the rows' X, V, Omega, ra at the step's start
  float dp[ROWS][NO / 2];    // the drawn exchange (momentum, angular momentum)
  bf16 act[2][ROWS][LDA];
  float cd[ROWS][CAND];      // candidates within the scan distance: squared distance,
  int ck[ROWS][CAND];        // colloid,
  int ce[ROWS][CAND];        // slot in the candidate list
  alignas(16) uint16_t lst[ROWS][CAND];  // candidate lists
  int lstn[ROWS];
  int cn[ROWS];              // candidates within the scan distance per row
  float feat[ROWS][NF];
  float out[ROWS][OUTP];
  alignas(16) float bias[3 * H + OUTP];
  float xi[ROWS][NO / 2];  // the exchange's Gaussians
  float xm[NF], xs[NF], ym[NO / 2], ys[NO / 2];
  unsigned long long full[NSTAGE], empty[NSTAGE];  // a chunk landed / every compute warp is done with it
  int abort;
};

__device__ __forceinline__ uint32_t bf16_bits(const bf16 *w, long long i) {
  return (uint32_t)__bfloat16_as_ushort(w[i]);
}

// the fragment-order copy of the BF16 weights ([k][n] matrices of 256 / 16 columns)
__global__ void k_sur_pack(const bf16 *w0, const bf16 *w1, const bf16 *w2, const bf16 *w3, uint4 *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= PACK_U4) return;
  const bf16 *W;
  int npad, k0, n;
  if (i < 19 * CHUNK_U4) {
    const int g = i / CHUNK_U4, within = i % CHUNK_U4, t = within >> 5, lane = within & 31;
    const int c = g < 3 ? g : (g < 11 ? g - 3 : g - 11);
    W = g < 3 ? w0 : (g < 11 ? w1 : w2);
    npad = H;
    k0 = 32 * c + 2 * (lane & 3);
    n = 8 * t + (lane >> 2);
  } else {
    const int within = i - 19 * CHUNK_U4, kp = within >> 6, t = (within >> 5) & 1, lane = within & 31;
    W = w3;
    npad = OUTP;
    k0 = 32 * kp + 2 * (lane & 3);
    n = 8 * t + (lane >> 2);
  }
  uint32_t word[4];
#pragma unroll
  for (int h = 0; h < 4; ++h) {
    const long long kb = k0 + 8 * h;
    word[h] = bf16_bits(W, kb * npad + n) | (bf16_bits(W, (kb + 1) * npad + n) << 16);
  }
  out[i] = make_uint4(word[0], word[1], word[2], word[3]);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait for phase `parity` of a stage's barrier: gives up after 100 ms (a
// chunk arrives in microseconds) or 2^24 tries
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, uint32_t parity) {
  unsigned long long t0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (int it = 0; it < (1 << 24); ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (t - t0 > 100000000ull) break;
  }
  return false;
}

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// weight chunk g into its stage, one bulk copy counted on the stage's full barrier
__device__ __forceinline__ void issue_chunk(const Sur &S, NetSmem &sm, int g) {
  const uint32_t bytes = g < 19 ? CHUNK_U4 * 16 : 512 * 16;
  unsigned long long *bar = &sm.full[g % NSTAGE];
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(sm.ring[g % NSTAGE])),
               "l"(S.wpk + (size_t)g * CHUNK_U4), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// a compute warp's wait for chunk g (lane 0, bounded).  After a wait that gave up
// (or once any wait has) the warp goes on without the chunk and without releasing
// its stage, so the producer stops too; the results are then flagged, not used.
__device__ __forceinline__ bool chunk_ready(const Sur &S, NetSmem &sm, int g) {
  int ok = 0;
  if ((threadIdx.x & 31) == 0) {
    unsigned long long *bar = &sm.full[g % NSTAGE];
    const uint32_t parity = (uint32_t)((g / NSTAGE) & 1);
    ok = mbar_try_wait(bar, parity);
    if (!ok) {
      volatile int *ab = &sm.abort;
      ok = !*ab && mbar_wait_bounded(bar, parity);
      if (!ok && !*ab) {
        atomicOr(S.err, 4);
        *ab = 1;
      }
    }
  }
  return __shfl_sync(0xFFFFFFFFu, ok, 0) != 0;
}

__device__ __forceinline__ void chunk_release(NetSmem &sm, int g, bool ok) {
  __syncwarp();
  if (ok && (threadIdx.x & 31) == 0) mbar_arrive(&sm.empty[g % NSTAGE]);
}

__device__ __forceinline__ void compute_barrier() {  // the compute warps only
  asm volatile("bar.sync 1, %0;" ::"n"(NCW * 32) : "memory");
}

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// the A fragment of K step kk (16 rows of the activations), one ldmatrix.x4: lane l
// gives the address of row l % 16 at column kk + 8 (l / 16)
__device__ __forceinline__ void a_frag(const bf16 (*A)[LDA], int kk, uint32_t a[4]) {
  const int lane = threadIdx.x & 31;
  const uint32_t addr = (uint32_t)__cvta_generic_to_shared(&A[lane & 15][kk + 8 * (lane >> 4)]);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(a[0]), "=r"(a[1]), "=r"(a[2]), "=r"(a[3])
               : "r"(addr)
               : "memory");
}

__device__ __forceinline__ float sigm(float z) { return __fdividef(1.f, 1.f + __expf(-z)); }  // as mlp.cu

// One block per 16 colloids: eight compute warps (two colloids each in the
// neighbour and feature phases, 32 columns each in the network) and one producer
// warp that streams the weights.
//   neighbours within max(three radii, the force cutoff plus the skin): from each
//   colloid's candidate list (colloids within that distance plus a skin of 2 at the
//   last rebuild, ascending index), or, when k_sur_md has flagged that a colloid
//   moved more than half the skin since then, from all pairs (and the lists rebuilt);
//   the features (V, Omega, ra, then the 12 nearest within three radii, nearest first,
//   ties by index, zero padded: the layout of brownian_gb300.closure.features), raw
//   to S.feat and normalised (clipped to six standard deviations) as the BF16 input
//   rows; the force partners (within the cutoff plus the skin, ascending index);
//   the step's draws (rotational diffusion, the exchange's Gaussians);
//   the four layers (the mlp.cu forward pass: K steps in ascending order into one
//   FP32 accumulator, bias, SiLU, BF16 between layers), the weights streamed by bulk
//   copies NSTAGE chunks ahead (full / empty barriers per stage); from the outputs
//   the Gaussian draw of the exchange (per-substep impulses for k_sur_md);
//   the orientation over the step's substeps: Omega takes its share of the angular
//   exchange each substep and ra the Euler rotation and the rotational diffusion
//   (update_activity_direction); neither depends on positions or forces.
__global__ void __launch_bounds__(NET_THREADS) k_sur_net(const Sur S) {
  extern __shared__ __align__(128) unsigned char net_smem[];
  NetSmem &sm = *reinterpret_cast<NetSmem *>(net_smem);
  if (*S.err & 4) return;  // a weight copy of an earlier step of this call did not arrive: no more steps
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int gq = lane >> 2, q = lane & 3;
  const unsigned lt = (1u << lane) - 1u;
  const int j0 = blockIdx.x * ROWS;
  const uint32_t step = (uint32_t)*S.step;
  const bool producer = warp == NCW;
  const float rfp = S.rc + partner_skin(S), rforce2 = rfp * rfp;
  if (tid == NCW * 32) {
    for (int s = 0; s < NSTAGE; ++s) {
      mbar_init(&sm.full[s], 1);
      mbar_init(&sm.empty[s], NCW);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    sm.abort = 0;
    // the first weight chunks stream in while the neighbours are found
    for (int g = 0; g < NSTAGE; ++g) issue_chunk(S, sm, g);
  }
  // the rows' state, the biases, the normalisation and the candidate lists (or every
  // position, for a rebuild): independent loads, all in flight together
  const bool rebuild = *S.rebuild != 0;
  if (tid < 4 * ROWS) {
    const int r = tid % ROWS, f = tid / ROWS, j = j0 + r;
    const float4 *src = f == 0 ? S.X : (f == 1 ? S.V : (f == 2 ? S.W : S.ra));
    if (j < S.Nc) sm.row[f][r] = src[j];
  }
  static_assert((3 * H + OUTP) / 4 <= NET_THREADS && NF <= NET_THREADS, "one load per thread");
  if (tid < (3 * H + OUTP) / 4) reinterpret_cast<uint4 *>(sm.bias)[tid] = reinterpret_cast<const uint4 *>(S.bias)[tid];
  if (tid < NF) {
    sm.xm[tid] = S.xmean[tid];
    sm.xs[tid] = S.xistd[tid];
  }
  if (tid < NO / 2) {
    sm.ym[tid] = S.ymean[tid];
    sm.ys[tid] = S.yistd[tid];
  }
  // the lists (read on every step, so that no load waits for the flag; a rebuild replaces them)
  static_assert(ROWS * CAND / 8 <= NET_THREADS, "one 16-byte piece of the lists per thread");
  if (tid < ROWS * CAND / 8) {
    const int r = tid / (CAND / 8), qv = tid % (CAND / 8), j = j0 + r;
    if (j < S.Nc)
      reinterpret_cast<uint4 *>(sm.lst[r])[qv] = reinterpret_cast<const uint4 *>(S.nbl + (size_t)j * CAND)[qv];
  }
  if (tid < ROWS) sm.lstn[tid] = j0 + tid < S.Nc ? S.nbn[j0 + tid] : 0;
  if (rebuild) {
    for (int i0 = tid; i0 < S.Nc; i0 += 8 * NET_THREADS) {  // eight loads in flight per thread
      float4 v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (i0 + u * NET_THREADS < S.Nc) v[u] = S.X[i0 + u * NET_THREADS];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (i0 + u * NET_THREADS < S.Nc) sm.u.xall[i0 + u * NET_THREADS] = v[u];
    }
  }
  __syncthreads();
  if (rebuild) {
    // all pairs: colloids within the list distance, ascending index (compute warp w: row w)
    const int r = warp, j = j0 + r;
    if (!producer && j < S.Nc) {
      const float4 xj = sm.row[0][r];
      int nl = 0;
      for (int k0 = 0; k0 < S.Nc; k0 += 32) {
        const int k = k0 + lane;
        float d2 = 1e30f;
        if (k < S.Nc && k != j) {
          const float4 xk = sm.u.xall[k];
          const float dx = wrapd(xk.x - xj.x, S.L[0], S.iL[0]), dy = wrapd(xk.y - xj.y, S.L[1], S.iL[1]),
                      dz = wrapd(xk.z - xj.z, S.L[2], S.iL[2]);
          d2 = dx * dx + dy * dy + dz * dz;
        }
        const bool inl = d2 < S.rlist2;
        const unsigned ml = __ballot_sync(0xFFFFFFFFu, inl);
        if (inl) {
          const int slot = nl + __popc(ml & lt);
          if (slot < CAND) {
            S.nbl[(size_t)j * CAND + slot] = (uint16_t)k;
            sm.lst[r][slot] = (uint16_t)k;
          }
        }
        nl += __popc(ml);
      }
      if (lane == 0) {
        sm.lstn[r] = min(nl, CAND);
        S.nbn[j] = min(nl, CAND);
        S.xref[j] = xj;
        if (nl > CAND) atomicOr(S.err, 1);
      }
    } else if (!producer && lane == 0) {
      sm.lstn[r] = 0;
    }
    __syncthreads();  // (the candidates' positions below overwrite xall)
  }
  // the candidates' positions and velocities, all loads in flight together
  {
    constexpr int PT = (ROWS * CAND + NET_THREADS - 1) / NET_THREADS;
    float4 px[PT], pv[PT];
#pragma unroll
    for (int u = 0; u < PT; ++u) {
      const int i = tid + NET_THREADS * u, r = i / CAND, e = i % CAND;
      if (i < ROWS * CAND && e < sm.lstn[r]) {
        const int k = sm.lst[r][e];
        px[u] = S.X[k];
        pv[u] = S.V[k];
      }
    }
#pragma unroll
    for (int u = 0; u < PT; ++u) {
      const int i = tid + NET_THREADS * u, r = i / CAND, e = i % CAND;
      if (i < ROWS * CAND && e < sm.lstn[r]) {
        sm.u.c.cx[r][e] = px[u];
        sm.u.c.cv[r][e] = pv[u];
      }
    }
  }
  __syncthreads();
  if (!producer) {  // compute warp w: row w
    const int r = warp, j = j0 + r;
    float *o = sm.feat[r];
    for (int col = lane; col < NF; col += 32) o[col] = 0.f;
    __syncwarp();
    if (j < S.Nc) {
    const float4 xj = sm.row[0][r], vj = sm.row[1][r];
    // neighbours within the scan distance, ascending index
    const int nlst = sm.lstn[r];
    int n = 0;
    for (int e0 = 0; e0 < nlst; e0 += 32) {
      const int e = e0 + lane;
      float d2 = 1e30f;
      if (e < nlst) {
        const float4 xk = sm.u.c.cx[r][e];
        const float dx = wrapd(xk.x - xj.x, S.L[0], S.iL[0]), dy = wrapd(xk.y - xj.y, S.L[1], S.iL[1]),
                    dz = wrapd(xk.z - xj.z, S.L[2], S.iL[2]);
        d2 = dx * dx + dy * dy + dz * dz;
      }
      const bool in = d2 < S.rscan2;
      const unsigned m = __ballot_sync(0xFFFFFFFFu, in);
      if (in) {
        const int slot = n + __popc(m & lt);  // slot <= e < CAND
        sm.cd[r][slot] = d2;
        sm.ck[r][slot] = sm.lst[r][e];
        sm.ce[r][slot] = e;
      }
      n += __popc(m);
    }
    __syncwarp();
    if (lane == 0) {
      o[0] = vj.x; o[1] = vj.y; o[2] = vj.z;
      const float4 wj = sm.row[2][r], aj = sm.row[3][r];
      o[3] = wj.x; o[4] = wj.y; o[5] = wj.z; o[6] = aj.x; o[7] = aj.y; o[8] = aj.z;
    }
    // the 12 nearest within three radii: each candidate's rank by (distance, index)
    for (int e0 = 0; e0 < n; e0 += 32) {
      const int e = e0 + lane;
      const bool have = e < n;
      const float d2 = have ? sm.cd[r][e] : 3.0e38f;
      const int k = have ? sm.ck[r][e] : 0x7FFFFFFF;
      int rank = 0;
      if (n <= 32) {
        for (int f = 0; f < n; ++f) {
          const float df = __shfl_sync(0xFFFFFFFFu, d2, f);
          const int kf = __shfl_sync(0xFFFFFFFFu, k, f);
          rank += (df < S.ct_feat2) && (df < d2 || (df == d2 && kf < k));
        }
      } else {
        for (int f = 0; f < n; ++f) {
          const float df = sm.cd[r][f];
          rank += (df < S.ct_feat2) && (df < d2 || (df == d2 && sm.ck[r][f] < k));
        }
      }
      if (have && d2 < S.ct_feat2 && rank < KNEAR) {
        const int ce = sm.ce[r][e];
        const float4 xk = sm.u.c.cx[r][ce], vk = sm.u.c.cv[r][ce];
        float *qf = o + 9 + 6 * rank;
        qf[0] = wrapd(xk.x - xj.x, S.L[0], S.iL[0]);
        qf[1] = wrapd(xk.y - xj.y, S.L[1], S.iL[1]);
        qf[2] = wrapd(xk.z - xj.z, S.L[2], S.iL[2]);
        qf[3] = vk.x - vj.x; qf[4] = vk.y - vj.y; qf[5] = vk.z - vj.z;
      }
    }
    // the force partners, ascending index
    int m = 0;
    for (int e0 = 0; e0 < n; e0 += 32) {
      const int e = e0 + lane;
      const bool in = e < n && sm.cd[r][e] < rforce2;
      const unsigned b = __ballot_sync(0xFFFFFFFFu, in);
      if (in) {
        const int slot = m + __popc(b & lt);
        if (slot < MAXF) S.fpart[(size_t)j * MAXF + slot] = (uint16_t)sm.ck[r][e];
      }
      m += __popc(b);
    }
    if (lane == 0) {
      S.fpn[j] = (uint8_t)min(m, MAXF);
      if (m > MAXF) atomicOr(S.err, 2);
    }
    }
  }
  // the step's draws: rotational diffusion per substep, the exchange's six Gaussians
  for (int i = tid; i < ROWS * (S.n_sub + 1); i += NET_THREADS) {
    const int r = i % ROWS, l = i / ROWS, j = j0 + r;
    if (j >= S.Nc) continue;
    if (l < S.n_sub) {
      if (S.rotdiff_s > 0.f) {
        const uint4 d = draw4(S.key, DOM_SUR_ROT, 0, (uint32_t)(j + 1), 0, step * S.n_sub + l);
        const float2 g0 = normal2(d.x, d.y), g1 = normal2(d.z, d.w);
        sm.nz[r][l] = make_float4(g0.x, g0.y, g1.x, 0.f);
      }
    } else {
      const uint4 r0 = draw4(S.key, DOM_SUR_KICK, 0, (uint32_t)(j + 1), 0, step);
      const uint4 r1 = draw4(S.key, DOM_SUR_KICK, 1, (uint32_t)(j + 1), 0, step);
      const float2 g0 = normal2(r0.x, r0.y), g1 = normal2(r0.z, r0.w), g2 = normal2(r1.x, r1.y);
      sm.xi[r][0] = g0.x; sm.xi[r][1] = g0.y; sm.xi[r][2] = g1.x;
      sm.xi[r][3] = g1.y; sm.xi[r][4] = g2.x; sm.xi[r][5] = g2.y;
    }
  }
  __syncthreads();
  // raw inputs to S.feat, normalised BF16 rows to act[0]
  for (int i = tid; i < ROWS * INP; i += NET_THREADS) {
    const int r = i / INP, c = i % INP, j = j0 + r;
    float z = 0.f;
    if (c < NF) {
      const float x = sm.feat[r][c];
      if (j < S.Nc) S.feat[(size_t)j * NF + c] = x;
      z = (x - sm.xm[c]) * sm.xs[c];
    }
    sm.act[0][r][c] = __float2bfloat16(fminf(fmaxf(z, -MLP_INPUT_CLIP), MLP_INPUT_CLIP));
  }
  __syncthreads();
  if (producer) {
    if (lane == 0) {
      // chunk g into its stage once every compute warp is done with chunk g - NSTAGE
      volatile int *ab = &sm.abort;
      int issued = NSTAGE;
      for (int g = NSTAGE; g < NCHUNK && !*ab; ++g) {
        if (!mbar_wait_bounded(&sm.empty[g % NSTAGE], (uint32_t)((g / NSTAGE - 1) & 1))) {
          atomicOr(S.err, 4);
          *ab = 1;
          break;
        }
        if (g == S.drop_chunk) continue;  // injected fault: the consumers' bounded waits give up
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue_chunk(S, sm, g);
        issued = g + 1;
      }
      // every copy issued (the last one into each stage) lands before the block exits
      for (int c = issued > NSTAGE ? issued - NSTAGE : 0; c < issued; ++c)
        if (c != S.drop_chunk) mbar_wait_bounded(&sm.full[c % NSTAGE], (uint32_t)((c / NSTAGE) & 1));
    }
  } else {
    // three hidden layers: compute warp w takes columns 8 TPW w .. 8 TPW (w + 1) - 1, two
    // weight chunks per wait
    int g = 0;
#pragma unroll 1
    for (int layer = 0; layer < 3; ++layer) {
      const bf16(*A)[LDA] = sm.act[layer & 1];
      bf16(*Z)[LDA] = sm.act[(layer + 1) & 1];
      const int nch = layer == 0 ? INP / 32 : H / 32;
      float acc[TPW][4];
#pragma unroll
      for (int t = 0; t < TPW; ++t)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[t][e] = 0.f;
#pragma unroll 1
      for (int c = 0; c < nch; c += 2) {
        const bool two = c + 1 < nch;
        const bool ok0 = chunk_ready(S, sm, g), ok1 = two ? chunk_ready(S, sm, g + 1) : true;
        const uint4 *B0 = sm.ring[g % NSTAGE], *B1 = sm.ring[(g + 1) % NSTAGE];
        uint4 b0[TPW], b1[TPW];
#pragma unroll
        for (int t = 0; t < TPW; ++t) b0[t] = B0[(TPW * warp + t) * 32 + lane];
        if (two) {
#pragma unroll
          for (int t = 0; t < TPW; ++t) b1[t] = B1[(TPW * warp + t) * 32 + lane];
        }
        uint32_t a[4];
        a_frag(A, 32 * c, a);
#pragma unroll
        for (int t = 0; t < TPW; ++t) mma_bf16(acc[t], a, b0[t].x, b0[t].y);
        a_frag(A, 32 * c + 16, a);
#pragma unroll
        for (int t = 0; t < TPW; ++t) mma_bf16(acc[t], a, b0[t].z, b0[t].w);
        if (two) {
          a_frag(A, 32 * c + 32, a);
#pragma unroll
          for (int t = 0; t < TPW; ++t) mma_bf16(acc[t], a, b1[t].x, b1[t].y);
          a_frag(A, 32 * c + 48, a);
#pragma unroll
          for (int t = 0; t < TPW; ++t) mma_bf16(acc[t], a, b1[t].z, b1[t].w);
        }
        chunk_release(sm, g, ok0);
        if (two) chunk_release(sm, g + 1, ok1);
        g += two ? 2 : 1;
      }
      const float *bias = sm.bias + H * layer;
#pragma unroll
      for (int t = 0; t < TPW; ++t) {
        const int n0 = 8 * (TPW * warp + t) + 2 * q;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          float v0 = acc[t][2 * h] + bias[n0], v1 = acc[t][2 * h + 1] + bias[n0 + 1];
          v0 = v0 * sigm(v0);
          v1 = v1 * sigm(v1);
          __nv_bfloat162 pr;
          pr.x = __float2bfloat16(v0);
          pr.y = __float2bfloat16(v1);
          *reinterpret_cast<__nv_bfloat162 *>(&Z[gq + 8 * h][n0]) = pr;
        }
      }
      compute_barrier();
    }
    // the output layer (16 columns, 12 used): compute warps 0 and 1, one 8-column tile each
    if (warp < 2) {
      const bool ok = chunk_ready(S, sm, g);
      (void)ok;
      const uint4 *B = sm.ring[g % NSTAGE];
      const bf16(*A)[LDA] = sm.act[1];
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
      for (int kp = 0; kp < H / 32; ++kp) {
        const uint4 b = B[(2 * kp + warp) * 32 + lane];
        uint32_t a[4];
        a_frag(A, 32 * kp, a);
        mma_bf16(acc, a, b.x, b.y);
        a_frag(A, 32 * kp + 16, a);
        mma_bf16(acc, a, b.z, b.w);
      }
      const float *bias = sm.bias + 3 * H;
      const int n0 = 8 * warp + 2 * q;
      sm.out[gq][n0] = acc[0] + bias[n0];
      sm.out[gq][n0 + 1] = acc[1] + bias[n0 + 1];
      sm.out[gq + 8][n0] = acc[2] + bias[n0];
      sm.out[gq + 8][n0 + 1] = acc[3] + bias[n0 + 1];
    }
  }
  __syncthreads();
  for (int i = tid; i < ROWS * OUTP; i += NET_THREADS) {
    const int r = i / OUTP, j = j0 + r;
    if (j < S.Nc) S.out[(size_t)j * OUTP + i % OUTP] = sm.out[r][i % OUTP];
  }
  // the exchange, one (row, component) per thread: the network's normalised outputs ->
  // mean and standard deviation in physical units, and the Gaussian draw
  if (tid < ROWS * (NO / 2)) {
    const int r = tid / (NO / 2), k = tid % (NO / 2);
    const float *o = sm.out[r];
    const float lv = fminf(fmaxf(o[6 + k], -MLP_LOGVAR_CLAMP), MLP_LOGVAR_CLAMP);
    sm.dp[r][k] = (o[k] + S.noise * __expf(0.5f * lv) * sm.xi[r][k]) / sm.ys[k] + sm.ym[k];
  }
  __syncthreads();
  // per (row, substep): Omega after the substep's share of the angular exchange (spread
  // in equal parts over the substeps: the fluid collides every substep; the same
  // sequence of additions as the substeps make) and the Euler matrix of Omega dt
  const float fm = 1.f / (S.M * S.n_sub), fi = 1.f / (S.I * S.n_sub);
  for (int i = tid; i < ROWS * S.n_sub; i += NET_THREADS) {
    const int r = i % ROWS, l = i / ROWS, j = j0 + r;
    if (j >= S.Nc) continue;
    if (l == 0) {
      S.imp[j] = make_float4(sm.dp[r][0] * fm, sm.dp[r][1] * fm, sm.dp[r][2] * fm, 0.f);
      S.imp[S.Nc + j] = sm.row[3][r];  // the orientation run()'s kick uses
    }
    const float pax = sm.dp[r][3] * fi, pay = sm.dp[r][4] * fi, paz = sm.dp[r][5] * fi;
    float4 w = sm.row[2][r];
    for (int s = 0; s <= l; ++s) {
      w.x += pax; w.y += pay; w.z += paz;
    }
    float sx, cx, sy, cy, sz, cz;
    __sincosf(w.x * S.dt, &sx, &cx); __sincosf(w.y * S.dt, &sy, &cy); __sincosf(w.z * S.dt, &sz, &cz);
    sm.rm[r][l][0] = make_float4(cy * cz, -(cy * sz), sy, 0.f);
    sm.rm[r][l][1] = make_float4(sx * sy * cz + cx * sz, -sx * sy * sz + cx * cz, -(sx * cy), 0.f);
    sm.rm[r][l][2] = make_float4(-cx * sy * cz + sx * sz, cx * sy * sz + sx * cz, cx * cy, 0.f);
  }
  __syncthreads();
  // the orientation through the substeps: the Euler rotation, then the rotational
  // diffusion (update_activity_direction plus Dr)
  if (tid < ROWS && j0 + tid < S.Nc) {
    const int r = tid, j = j0 + r;
    const float pax = sm.dp[r][3] * fi, pay = sm.dp[r][4] * fi, paz = sm.dp[r][5] * fi;
    float4 w = sm.row[2][r], a = sm.row[3][r];
    float4 n0 = sm.rm[r][0][0], n1 = sm.rm[r][0][1], n2 = sm.rm[r][0][2];
    for (int l = 0; l < S.n_sub; ++l) {
      w.x += pax; w.y += pay; w.z += paz;
      const float4 m0 = n0, m1 = n1, m2 = n2;
      if (l + 1 < S.n_sub) {  // the next substep's matrix, in flight meanwhile
        n0 = sm.rm[r][l + 1][0]; n1 = sm.rm[r][l + 1][1]; n2 = sm.rm[r][l + 1][2];
      }
      float ax = m0.x * a.x + m0.y * a.y + m0.z * a.z;
      float ay = m1.x * a.x + m1.y * a.y + m1.z * a.z;
      float az = m2.x * a.x + m2.y * a.y + m2.z * a.z;
      if (S.rotdiff_s > 0.f) {
        const float4 gz = sm.nz[r][l];
        const float d = gz.x * ax + gz.y * ay + gz.z * az;
        ax += S.rotdiff_s * (gz.x - d * ax); ay += S.rotdiff_s * (gz.y - d * ay); az += S.rotdiff_s * (gz.z - d * az);
      }
      const float in = rsqrtf(ax * ax + ay * ay + az * az);
      a = make_float4(ax * in, ay * in, az * in, 0.f);
    }
    // the step's end state of Omega and ra, which the substep kernel stores (so a step
    // whose network failed leaves them as they were)
    S.imp[2 * S.Nc + j] = w;
    S.imp[3 * S.Nc + j] = a;
  }
}

// ---- the substeps ---------------------------------------------------------------
// squared displacement from xs to x (minimum image)
__device__ __forceinline__ float step_moved2(const Sur &S, float4 x, float4 xs) {
  const float dx = wrapd(x.x - xs.x, S.L[0], S.iL[0]), dy = wrapd(x.y - xs.y, S.L[1], S.iL[1]),
              dz = wrapd(x.z - xs.z, S.L[2], S.iL[2]);
  return dx * dx + dy * dy + dz * dz;
}

// the WCA forces on a colloid at x from its n partners (ids in row, ascending; positions
// in P): the force-shifted WCA pair force (cpp/update.cpp:14-32) in FP32 for the pairs
// within the cutoff (1/r by the fast reciprocal square root, 1/r^6 from 1/r^2), four
// positions fetched together, summed in partner order
__device__ __forceinline__ float3 partner_forces(const Sur &S, float4 x, const float4 *P, const uint16_t *row, int n,
                                                 int self) {
  float3 fn = make_float3(0.f, 0.f, 0.f);
  for (int e = 0; e < n; e += 4) {
    const uint2 kk = *reinterpret_cast<const uint2 *>(row + e);
    const int k4[4] = {(int)(kk.x & 0xFFFFu), (int)(kk.x >> 16), (int)(kk.y & 0xFFFFu), (int)(kk.y >> 16)};
    float4 xk[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) xk[i] = P[e + i < n ? k4[i] : self];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float dx = wrapd(x.x - xk[i].x, S.L[0], S.iL[0]), dy = wrapd(x.y - xk[i].y, S.L[1], S.iL[1]),
                  dz = wrapd(x.z - xk[i].z, S.L[2], S.iL[2]);
      const float r2 = dx * dx + dy * dy + dz * dz;
      if (e + i < n && r2 < S.rc2) {
        const float ir = rsqrtf(r2), ir2 = ir * ir, ir6 = ir2 * ir2 * ir2;
        const float f = (4.f * S.eps * (12.f * S.sig12 * ir6 * ir6 * ir - 6.f * S.sig6 * ir6 * ir) - S.fc) * ir;
        fn.x += f * dx; fn.y += f * dy; fn.z += f * dz;
      }
    }
  }
  return fn;
}

// One block, PER colloids per thread (position, velocity, force and the step's impulse
// in registers; positions, two copies by substep parity, and force partners in shared
// memory): run()'s kick along the orientation at the step's start, then n_sub substeps
// of update_pos_md, the substep's share of the exchange, compute_force_md at the new
// positions and update_velocity_colloid, one block barrier per substep (the copy a
// substep writes was last read two substeps before).  At the end: whether a colloid has
// moved more than half the skin since the candidate lists were built.
template <int PER>
__global__ void __launch_bounds__(1024) k_sur_md1(const Sur S) {
  extern __shared__ float4 smem[];
  if (*S.err & 4) return;  // the network's outputs of this step are incomplete: the state stays as it was
  __shared__ unsigned s_vmax;  // the largest speed at the end (float bits, non-negative)
  const float hs = 0.5f * partner_skin(S), hs2 = hs * hs;
  uint16_t *sF = reinterpret_cast<uint16_t *>(smem + 2 * MAXC);  // [MAXC][MAXF] force partners
  uint8_t *sFn = reinterpret_cast<uint8_t *>(sF + MAXC * MAXF);   // [MAXC] their count
  const int T = blockDim.x, tid = threadIdx.x;
  if (tid == 0) s_vmax = 0u;
  {
    const uint4 *src = reinterpret_cast<const uint4 *>(S.fpart);
    uint4 *dst = reinterpret_cast<uint4 *>(sF);
    const int nq = S.Nc * (MAXF * 2 / 16);
    for (int i0 = tid; i0 < nq; i0 += 4 * T) {  // four loads in flight per thread
      uint4 qv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (i0 + u * T < nq) qv[u] = src[i0 + u * T];
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (i0 + u * T < nq) dst[i0 + u * T] = qv[u];
    }
    for (int i = tid; i < S.Nc; i += T) sFn[i] = S.fpn[i];
  }
  float4 x[PER], v[PER], fo[PER], pl[PER];
#pragma unroll
  for (int u = 0; u < PER; ++u) {
    const int j = tid + T * u;
    if (j >= S.Nc) continue;
    x[u] = S.X[j]; v[u] = S.V[j]; fo[u] = S.f[j]; pl[u] = S.imp[j];
    const float4 a = S.imp[S.Nc + j];
    v[u].x += S.v0 * a.x; v[u].y += S.v0 * a.y; v[u].z += S.v0 * a.z;
  }
  const float hdt2m = 0.5f * S.dt * S.dt / S.M, hdtm = 0.5f * S.dt / S.M;
  for (int l = 0; l < S.n_sub; ++l) {
    float4 *P = (l & 1) ? smem : smem + MAXC;  // this substep's copy
#pragma unroll
    for (int u = 0; u < PER; ++u) {  // update_pos_md
      const int j = tid + T * u;
      if (j >= S.Nc) continue;
      float4 &xx = x[u];
      xx.x += v[u].x * S.dt + fo[u].x * hdt2m; xx.y += v[u].y * S.dt + fo[u].y * hdt2m;
      xx.z += v[u].z * S.dt + fo[u].z * hdt2m;
      xx.x -= S.L[0] * floorf(xx.x * S.iL[0]); xx.y -= S.L[1] * floorf(xx.y * S.iL[1]);
      xx.z -= S.L[2] * floorf(xx.z * S.iL[2]);
      P[j] = xx;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int j = tid + T * u;
      if (j >= S.Nc) continue;
      // this substep's share of the fluid exchange (fluid_colloid_collision)
      v[u].x += pl[u].x; v[u].y += pl[u].y; v[u].z += pl[u].z;
      // compute_force_md at the new positions, update_velocity_colloid
      const float3 fn = partner_forces(S, x[u], P, sF + j * MAXF, sFn[j], j);
      v[u].x += (fo[u].x + fn.x) * hdtm; v[u].y += (fo[u].y + fn.y) * hdtm; v[u].z += (fo[u].z + fn.z) * hdtm;
      fo[u] = make_float4(fn.x, fn.y, fn.z, 0.f);
    }
  }
  int moved = 0, fast = 0;
#pragma unroll
  for (int u = 0; u < PER; ++u) {
    const int j = tid + T * u;
    if (j >= S.Nc) continue;
    const float4 x0 = S.xref[j], xs = S.X[j];
    S.X[j] = x[u]; S.V[j] = v[u]; S.f[j] = fo[u];
    S.W[j] = S.imp[2 * S.Nc + j]; S.ra[j] = S.imp[3 * S.Nc + j];
    const float dx = wrapd(x[u].x - x0.x, S.L[0], S.iL[0]), dy = wrapd(x[u].y - x0.y, S.L[1], S.iL[1]),
                dz = wrapd(x[u].z - x0.z, S.L[2], S.iL[2]);
    moved |= dx * dx + dy * dy + dz * dz > S.half_skin2;
    fast |= step_moved2(S, x[u], xs) > hs2;
    atomicMax(&s_vmax, __float_as_uint(sqrtf(v[u].x * v[u].x + v[u].y * v[u].y + v[u].z * v[u].z)));
  }
  moved = __syncthreads_or(moved);
  fast = __syncthreads_or(fast);
  if (tid == 0) {
    *S.rebuild = moved;
    if (fast) *S.fast += 1;
    *S.vmax = __uint_as_float(s_vmax);
    *S.step += 1;
  }
}

// One cluster of MDC blocks, one colloid per thread (block b takes colloids
// [b per, (b + 1) per)): position, velocity, force and the step's impulse in
// registers, force partners in shared memory.  run()'s kick along the orientation at
// the step's start, then n_sub substeps of update_pos_md, the substep's share of the
// exchange, compute_force_md at the new positions and update_velocity_colloid.  Each
// substep's new positions go to every block's copy (distributed shared memory, two
// copies by substep parity), then one cluster barrier: the copy a substep writes was
// last read two substeps before, behind the barrier in between.  At the end: whether
// a colloid has moved more than half the skin since the candidate lists were built.
constexpr int MDC = 8, MD_MAXT = MAXC / MDC;

__global__ void __cluster_dims__(MDC, 1, 1) __launch_bounds__(MD_MAXT) k_sur_md(const Sur S) {
  if (*S.err & 4) return;  // the network's outputs of this step are incomplete: the state stays as it was
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ float4 smem[];
  uint16_t *sF = reinterpret_cast<uint16_t *>(smem + 2 * MAXC);          // [MD_MAXT][MAXF] force partners
  uint8_t *sFn = reinterpret_cast<uint8_t *>(sF + MD_MAXT * MAXF);       // [MD_MAXT] their count
  int *sMoved = reinterpret_cast<int *>(sFn + MD_MAXT);                  // [MDC] (block 0)
  unsigned *sVmax = reinterpret_cast<unsigned *>(sMoved + MDC);         // [MDC] (block 0)
  __shared__ unsigned s_vmax;
  const float hs = 0.5f * partner_skin(S), hs2 = hs * hs;
  const int tid = threadIdx.x, rank = (int)cl.block_rank();
  const int per = (S.Nc + MDC - 1) / MDC, j = rank * per + tid;
  const bool own = tid < per && j < S.Nc;
  if (tid == 0) s_vmax = 0u;
  float4 x = make_float4(0.f, 0.f, 0.f, 0.f), v = x, fo = x, pl = x;
  int n = 0;
  if (own) {
    const uint4 *src = reinterpret_cast<const uint4 *>(S.fpart + (size_t)j * MAXF);
    uint4 *dst = reinterpret_cast<uint4 *>(sF + tid * MAXF);
    uint4 pp[MAXF * 2 / 16];
#pragma unroll
    for (int i = 0; i < MAXF * 2 / 16; ++i) pp[i] = src[i];
    n = S.fpn[j];
    x = S.X[j]; v = S.V[j]; fo = S.f[j]; pl = S.imp[j];
    const float4 a = S.imp[S.Nc + j];
#pragma unroll
    for (int i = 0; i < MAXF * 2 / 16; ++i) dst[i] = pp[i];
    v.x += S.v0 * a.x; v.y += S.v0 * a.y; v.z += S.v0 * a.z;
  }
  cl.sync();  // every block has started before any writes to its copies
  const float hdt2m = 0.5f * S.dt * S.dt / S.M, hdtm = 0.5f * S.dt / S.M;
  for (int l = 0; l < S.n_sub; ++l) {
    const int nb = (l + 1) & 1;
    if (own) {  // update_pos_md
      x.x += v.x * S.dt + fo.x * hdt2m; x.y += v.y * S.dt + fo.y * hdt2m; x.z += v.z * S.dt + fo.z * hdt2m;
      x.x -= S.L[0] * floorf(x.x * S.iL[0]); x.y -= S.L[1] * floorf(x.y * S.iL[1]); x.z -= S.L[2] * floorf(x.z * S.iL[2]);
      float4 *mine = (nb ? smem + MAXC : smem) + j;
#pragma unroll
      for (int b = 0; b < MDC; ++b) *cl.map_shared_rank(mine, b) = x;
    }
    cl.sync();
    if (own) {
      const float4 *P = nb ? smem + MAXC : smem;  // positions, by substep parity
      // this substep's share of the fluid exchange (fluid_colloid_collision)
      v.x += pl.x; v.y += pl.y; v.z += pl.z;
      // compute_force_md at the new positions, update_velocity_colloid
      const float3 fn = partner_forces(S, x, P, sF + tid * MAXF, n, j);
      v.x += (fo.x + fn.x) * hdtm; v.y += (fo.y + fn.y) * hdtm; v.z += (fo.z + fn.z) * hdtm;
      fo = make_float4(fn.x, fn.y, fn.z, 0.f);
    }
  }
  int moved = 0;
  if (own) {
    const float4 x0 = S.xref[j], xs = S.X[j];
    S.X[j] = x; S.V[j] = v; S.f[j] = fo;
    S.W[j] = S.imp[2 * S.Nc + j]; S.ra[j] = S.imp[3 * S.Nc + j];
    const float dx = wrapd(x.x - x0.x, S.L[0], S.iL[0]), dy = wrapd(x.y - x0.y, S.L[1], S.iL[1]),
                dz = wrapd(x.z - x0.z, S.L[2], S.iL[2]);
    moved = (dx * dx + dy * dy + dz * dz > S.half_skin2 ? 1 : 0) | (step_moved2(S, x, xs) > hs2 ? 2 : 0);
    atomicMax(&s_vmax, __float_as_uint(sqrtf(v.x * v.x + v.y * v.y + v.z * v.z)));
  }
  moved = __syncthreads_or(moved & 1) | (__syncthreads_or(moved & 2) ? 2 : 0);
  if (tid == 0) {
    *cl.map_shared_rank(sMoved + rank, 0) = moved;
    *cl.map_shared_rank(sVmax + rank, 0) = s_vmax;
  }
  cl.sync();  // (also: no block leaves while another may still write its copies)
  if (rank == 0 && tid == 0) {
    int any = 0;
    unsigned vm = 0u;
    for (int b = 0; b < MDC; ++b) {
      any |= sMoved[b];
      vm = max(vm, sVmax[b]);
    }
    *S.rebuild = any & 1;
    if (any & 2) *S.fast += 1;
    *S.vmax = __uint_as_float(vm);
    *S.step += 1;
  }
}

// normalised outputs -> physical units (the arithmetic of mpcd_mlp_forward)
__global__ void k_sur_denorm(const Sur S, float *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S.Nc * NO) return;
  const int r = i / NO, k = i % NO, ny = NO / 2;
  const float v = S.out[(size_t)r * OUTP + k];
  out[i] = k < ny ? v / S.yistd[k] + S.ymean[k]
                  : fminf(fmaxf(v, -MLP_LOGVAR_CLAMP), MLP_LOGVAR_CLAMP) - 2.f * __logf(S.yistd[k - ny]);
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
  uint4 *wpk = nullptr;
  float *outd = nullptr;  // the outputs in physical units (mpcd_surrogate_outputs)
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

constexpr size_t kMd1Smem = 2 * MAXC * sizeof(float4) + MAXC * MAXF * sizeof(uint16_t) + MAXC;
constexpr int kMdBlockMax = 1024;  // colloids up to which the substeps run in one block, else in a cluster
constexpr size_t kMdSmem = 2 * MAXC * sizeof(float4) + MD_MAXT * MAXF * sizeof(uint16_t) + MD_MAXT + 2 * MDC * sizeof(int);
constexpr size_t kNetSmem = sizeof(NetSmem);

int enqueue_step(mpcd_surrogate *s) {
  const Sur &S = s->S;
  k_sur_net<<<(S.Nc + ROWS - 1) / ROWS, NET_THREADS, kNetSmem, s->stream>>>(S);
  if (S.Nc <= kMdBlockMax) {
    if (S.Nc <= 1024) k_sur_md1<1><<<1, (S.Nc + 31) / 32 * 32, kMd1Smem, s->stream>>>(S);
    else k_sur_md1<2><<<1, 1024, kMd1Smem, s->stream>>>(S);
  } else {
    const int per = (S.Nc + MDC - 1) / MDC;
    k_sur_md<<<MDC, (per + 31) / 32 * 32, kMdSmem, s->stream>>>(S);
  }
  return cudaGetLastError() == cudaSuccess ? MPCD_OK : sfail(s, MPCD_ERR_CUDA, "step launch");
}

// the network's current weights in the order k_sur_net reads them
int pack_weights(mpcd_surrogate *s) {
  const MlpIO io = mlp_io(s->net);
  s->S.bias = io.bias;
  s->S.xmean = io.xmean; s->S.xistd = io.xistd;
  s->S.ymean = io.ymean; s->S.yistd = io.yistd;
  k_sur_pack<<<(PACK_U4 + 255) / 256, 256, 0, s->stream>>>(
      static_cast<const bf16 *>(io.w[0]), static_cast<const bf16 *>(io.w[1]), static_cast<const bf16 *>(io.w[2]),
      static_cast<const bf16 *>(io.w[3]), s->wpk);
  return cudaGetLastError() == cudaSuccess ? MPCD_OK : sfail(s, MPCD_ERR_CUDA, "weight packing");
}

}  // namespace

extern "C" int mpcd_surrogate_create(const mpcd_params *p, mpcd_mlp *net, mpcd_surrogate **out) {
  if (!p || !net || !out) return MPCD_ERR_PARAM;
  *out = nullptr;
  if (p->n_colloid < 1 || p->n_colloid > MAXC || p->n_sub < 1 || p->n_sub > MAXSUB || !(p->ndt > 0) || !(p->mass_colloid > 0) ||
      !(p->I_colloid > 0) || p->Lx < 1 || p->Ly < 1 || p->Lz < 1)
    return MPCD_ERR_PARAM;
  mpcd_surrogate *s = new mpcd_surrogate();
  s->net = net;
  Sur &S = s->S;
  memset(&S, 0, sizeof S);
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
  // force partners within the cutoff plus a skin of 0.5 to 2 (partner_skin; k_sur_md counts
  // the steps in which a colloid moves more than half of it), features within three radii
  S.rc = (float)rc;
  const float rfmax2 = (float)((rc + 2.0) * (rc + 2.0));
  S.rscan2 = rfmax2 > S.ct_feat2 ? rfmax2 : S.ct_feat2;
  // candidate lists: within that distance plus a skin of 2, rebuilt once a colloid has
  // moved half the skin
  const double rl = std::sqrt((double)S.rscan2) + 2.0;
  S.rlist2 = (float)(rl * rl);
  S.half_skin2 = 1.0f;
  S.key = make_uint2((uint32_t)p->seed, (uint32_t)(p->seed >> 32));
  const size_t Nc = S.Nc;
  S.step = salloc<long long>(s, 1);
  S.X = salloc<float4>(s, Nc); S.V = salloc<float4>(s, Nc); S.W = salloc<float4>(s, Nc);
  S.ra = salloc<float4>(s, Nc); S.f = salloc<float4>(s, Nc);
  S.feat = salloc<float>(s, Nc * NF); S.out = salloc<float>(s, Nc * OUTP);
  S.imp = salloc<float4>(s, 4 * Nc);
  S.nbl = salloc<uint16_t>(s, Nc * CAND); S.nbn = salloc<int>(s, Nc);
  S.xref = salloc<float4>(s, Nc); S.rebuild = salloc<int>(s, 1);
  if (S.rebuild) cudaMemset(S.rebuild, 1, sizeof(int));  // no candidate lists yet
  S.fpart = salloc<uint16_t>(s, Nc * MAXF); S.fpn = salloc<uint8_t>(s, Nc);
  S.err = salloc<int>(s, 1);
  S.drop_chunk = -1;
  S.noise = 1.f;
  S.fast = salloc<long long>(s, 1);
  S.vmax = salloc<float>(s, 1);
  s->wpk = salloc<uint4>(s, PACK_U4);
  S.wpk = s->wpk;
  s->outd = salloc<float>(s, Nc * NO);
  if (!s->err.empty() || cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaFuncSetAttribute(k_sur_net, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kNetSmem) != cudaSuccess ||
      cudaFuncSetAttribute(k_sur_md, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMdSmem) != cudaSuccess ||
      cudaFuncSetAttribute(k_sur_md1<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMd1Smem) != cudaSuccess ||
      cudaFuncSetAttribute(k_sur_md1<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMd1Smem) != cudaSuccess ||
      pack_weights(s) != MPCD_OK) {
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
  float vm = 0.f;  // the largest speed: the first step's partner skin
  for (int j = 0; j < S.Nc; ++j)
    vm = std::max(vm, (float)std::sqrt(vel[3 * j] * vel[3 * j] + vel[3 * j + 1] * vel[3 * j + 1] +
                                       vel[3 * j + 2] * vel[3 * j + 2]));
  if (cudaMemcpyAsync(S.vmax, &vm, sizeof vm, cudaMemcpyHostToDevice, s->stream) != cudaSuccess)
    return sfail(s, MPCD_ERR_CUDA, "set-up");
  k_sur_forces<<<(S.Nc + 127) / 128, 128, 0, s->stream>>>(S);
  k_sur_features<<<(S.Nc + 3) / 4, 128, 0, s->stream>>>(S);
  if (cudaMemsetAsync(S.rebuild, 1, sizeof(int), s->stream) != cudaSuccess) return sfail(s, MPCD_ERR_CUDA, "set-up");
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

extern "C" int mpcd_surrogate_fast_steps(mpcd_surrogate *s, int64_t *count) {
  if (!s || !count) return MPCD_ERR_PARAM;
  long long c = 0;
  if (cudaMemcpyAsync(&c, s->S.fast, sizeof c, cudaMemcpyDeviceToHost, s->stream) != cudaSuccess ||
      cudaStreamSynchronize(s->stream) != cudaSuccess)
    return sfail(s, MPCD_ERR_CUDA, "fast-step count");
  *count = c;
  return MPCD_OK;
}

// the network's outputs of the last step in physical units (n_colloid x 12, host)
extern "C" int mpcd_surrogate_outputs(mpcd_surrogate *s, float *out) {
  if (!s || !out) return MPCD_ERR_PARAM;
  const Sur &S = s->S;
  k_sur_denorm<<<(S.Nc * NO + 255) / 256, 256, 0, s->stream>>>(S, s->outd);
  if (cudaMemcpyAsync(out, s->outd, sizeof(float) * NO * S.Nc, cudaMemcpyDeviceToHost, s->stream) != cudaSuccess ||
      cudaStreamSynchronize(s->stream) != cudaSuccess)
    return sfail(s, MPCD_ERR_CUDA, "outputs");
  return MPCD_OK;
}

extern "C" int mpcd_surrogate_set_fault(mpcd_surrogate *s, int drop_chunk) {
  if (!s || drop_chunk < -1 || drop_chunk >= NCHUNK || (drop_chunk >= 0 && drop_chunk < NSTAGE))
    return sfail(s, MPCD_ERR_PARAM, "drop_chunk: -1, or a weight chunk the producer loop issues");
  s->S.drop_chunk = drop_chunk;
  if (s->exec) {  // the kernels take the parameters by value: capture again
    cudaGraphExecDestroy(s->exec);
    s->exec = nullptr;
  }
  return MPCD_OK;
}

extern "C" int mpcd_surrogate_set_noise(mpcd_surrogate *s, double scale) {
  if (!s || !(scale >= 0.0) || !(scale <= 1e3)) return sfail(s, MPCD_ERR_PARAM, "noise scale: 0 .. 1000");
  s->S.noise = (float)scale;
  if (s->exec) {  // the kernels take the parameters by value: capture again
    cudaGraphExecDestroy(s->exec);
    s->exec = nullptr;
  }
  return MPCD_OK;
}

extern "C" int mpcd_surrogate_step(mpcd_surrogate *s, int nsteps) {
  if (!s || nsteps < 0) return MPCD_ERR_PARAM;
  // each call starts with the error bits clear: a failed call leaves the state as it was
  // before its failing step, and the next call may go on from there
  if (cudaMemsetAsync(s->S.err, 0, sizeof(int), s->stream) != cudaSuccess) return sfail(s, MPCD_ERR_CUDA, "step");
  if (nsteps > 0 && pack_weights(s) != MPCD_OK) return MPCD_ERR_CUDA;
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
  if (bits & 3)
    return sfail(s, MPCD_ERR_CAPACITY, "a colloid has more neighbours than its lists hold (64 within three radii "
                                       "or the force cutoff plus 4, 32 within the force cutoff plus 2)");
  if (bits) return sfail(s, MPCD_ERR_CUDA, "a weight copy of the network kernel did not arrive");
  return MPCD_OK;
}
