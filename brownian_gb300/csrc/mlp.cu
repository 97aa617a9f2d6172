// The learned closure's network: an MLP 81 -> 256 -> 256 -> 256 -> 12 with SiLU,
// trained and evaluated on the GPU by this file's own kernels.
//
// Weights are BF16 for the tensor cores (warp-level mma.sync m16n8k16, FP32
// accumulation) with FP32 master copies for Adam.  Activations and gradients
// between layers are BF16, every product accumulates in FP32.  The inputs are
// the closure's 81 colloid features, normalised by stored means and standard
// deviations; the outputs are the normalised means (6) and log-variances (6) of
// a colloid's per-step momentum and angular-momentum exchange with the fluid,
// trained by the Gaussian negative log-likelihood.
//
// One GEMM kernel serves every product: C[M x N] = A[M x K] B[K x N] with A and B
// addressed through arbitrary strides (forward x W, backward dZ W^T and A^T dZ),
// 32 x 64 block tiles, 32-wide K steps staged in shared memory through 16-byte
// loads (the next tile prefetched into registers), four warps of 32 x 16 each,
// and a fused epilogue (bias, SiLU, the SiLU derivative of the
// backward pass, BF16 / FP32 stores, FP32 atomic accumulation for split-K
// weight gradients).  Training runs every product on the 5th-generation tensor cores
// instead (tcgen05.mma with the accumulator in tensor memory, TMEM): the layer products
// (forward x W and backward dZ W^T, K and N <= 256) on k_gemm_tc, the weight gradients (a
// reduction over the batch) on k_gemm_tc_wgrad; inference (mpcd_mlp_forward) keeps the
// warp-level kernel, whose arithmetic the colloid-only step's network reproduces bit for bit.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/brownian_gb300.h"
#include "mlp_internal.h"

namespace {

typedef __nv_bfloat16 bf16;

constexpr int IN = MPCD_MLP_IN, INP = MLP_IN_PADDED, H = MPCD_MLP_HIDDEN, OUT = MPCD_MLP_OUT, OUTP = MLP_OUT_PADDED,
              NY = OUT / 2;
constexpr int BM = 32, BN = 64, BK = 32;
// normalised log-variances are used within [-6, 6] (variances between 0.0025 and 400 times
// the target's): beyond that the likelihood's gradient is zero and inference clamps
constexpr float kLogVarClamp = MLP_LOGVAR_CLAMP;
constexpr float kInputClip = MLP_INPUT_CLIP;

struct Gemm {
  const bf16 *A;
  long long sam, sak;
  const bf16 *B;
  long long sbk, sbn;
  int M, N, K;
  const float *bias;   // [N] or null
  int silu;            // apply SiLU after the bias
  const bf16 *dz;      // backward: multiply by silu'(dz[m, n]) (the layer's pre-activation)
  long long lddz;
  float *Cf;           // FP32 store
  long long ldcf;
  bf16 *Cb;            // BF16 store (after the activation)
  long long ldcb;
  bf16 *Zb;            // BF16 store of the pre-activation
  long long ldzb;
  float *Cacc;         // FP32 atomic accumulation
  long long ldca;
  int kchunk;          // K range of one blockIdx.z
};

// the logistic function, branch free (fast reciprocal: within 2 ulp, and 0 once e^-z overflows);
// the colloid-only step evaluates the network with the same arithmetic
__device__ __forceinline__ float sigm(float z) { return __fdividef(1.f, 1.f + __expf(-z)); }

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], const uint32_t b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Staging of one operand tile into shared memory as T[row][k] (rows: m for A, n for
// B), 8 elements per 16-byte load along whichever dimension is contiguous in
// memory (scalar loads where a vector would leave the matrix, is misaligned or
// neither stride is 1).  ROWS x KT elements, 128 threads.
template <int ROWS, int KT>
struct Stage {
  static constexpr int NV = ROWS * KT / 8 / 128;  // vectors per thread
  uint4 v[NV];
  __device__ __forceinline__ static void slot(int t, bool kfast, int &r, int &k) {
    if (kfast) { r = t / (KT / 8); k = (t % (KT / 8)) * 8; }
    else { k = t / (ROWS / 8); r = (t % (ROWS / 8)) * 8; }
  }
  __device__ __forceinline__ void load(const bf16 *base, long long rs, long long ks, int r0, int k0, int rmax, int kmax,
                                       bool kfast) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      int r, k;
      slot(threadIdx.x + 128 * i, kfast, r, k);
      r += r0; k += k0;
      const bf16 *p = base + r * rs + k * ks;
      const bool full = kfast ? (r < rmax && k + 8 <= kmax) : (k < kmax && r + 8 <= rmax);
      if (full && (kfast ? ks == 1 : rs == 1) && ((reinterpret_cast<uintptr_t>(p) & 15) == 0)) {
        v[i] = *reinterpret_cast<const uint4 *>(p);
      } else {
        bf16 e[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int rr = kfast ? r : r + q, kk = kfast ? k + q : k;
          e[q] = (rr < rmax && kk < kmax) ? base[rr * rs + kk * ks] : __float2bfloat16(0.f);
        }
        v[i] = *reinterpret_cast<const uint4 *>(e);
      }
    }
  }
  template <int LD>
  __device__ __forceinline__ void store(bf16 (*T)[LD], bool kfast) const {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      int r, k;
      slot(threadIdx.x + 128 * i, kfast, r, k);
      const bf16 *e = reinterpret_cast<const bf16 *>(&v[i]);
      if (kfast) {
        *reinterpret_cast<uint4 *>(&T[r][k]) = v[i];
      } else {
#pragma unroll
        for (int q = 0; q < 8; ++q) T[r + q][k] = e[q];
      }
    }
  }
};

// one element of C after the product: bias, pre-activation store, SiLU derivative
// (backward), SiLU, stores; or FP32 accumulation (split-K weight gradients)
__device__ __forceinline__ void epilogue(const Gemm &g, int m, int n, float v) {
  if (g.Cacc) {
    atomicAdd(&g.Cacc[m * g.ldca + n], v);
    return;
  }
  if (g.bias) v += g.bias[n];
  if (g.Zb) g.Zb[m * g.ldzb + n] = __float2bfloat16(v);
  if (g.dz) {
    const float z = __bfloat162float(g.dz[m * g.lddz + n]), s = sigm(z);
    v *= s * (1.f + z * (1.f - s));
  }
  if (g.silu) v = v * sigm(v);
  if (g.Cf) g.Cf[m * g.ldcf + n] = v;
  if (g.Cb) g.Cb[m * g.ldcb + n] = __float2bfloat16(v);
}

// C tile TM x TN per block of 4 warps side by side along N (each TM x TN/4: TM/16
// m16 by TN/32 n8 mma tiles), K in steps of TK; the next K tile is loaded into
// registers while the current one is multiplied.  Two shapes: TK = 256 takes a
// whole layer's K in one staging (inference-sized GEMMs: every load in flight at
// once), TK = 32 streams long reductions (weight gradients over the batch).
template <int TM, int TN, int TK>
__global__ void __launch_bounds__(128) k_gemm(const Gemm g) {
  constexpr int LD = TK + 8, MT = TM / 16, NT = TN / 32;
  __shared__ __align__(16) bf16 As[TM][LD];
  __shared__ __align__(16) bf16 Bs[TN][LD];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
  const int kbeg = blockIdx.z * g.kchunk, kend = min(g.K, kbeg + g.kchunk);
  float acc[MT][NT][4];
#pragma unroll
  for (int i = 0; i < MT; ++i)
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
  const bool a_kfast = g.sak == 1, b_kfast = g.sbk == 1;
  Stage<TM, TK> sa;
  Stage<TN, TK> sb;
  if (kbeg < kend) {
    sa.load(g.A, g.sam, g.sak, m0, kbeg, g.M, kend, a_kfast);
    sb.load(g.B, g.sbn, g.sbk, n0, kbeg, g.N, kend, b_kfast);
  }
  const int gq = lane >> 2, q = lane & 3;
  for (int k0 = kbeg; k0 < kend; k0 += TK) {
    sa.store(As, a_kfast);
    sb.store(Bs, b_kfast);
    __syncthreads();
    if (k0 + TK < kend) {
      sa.load(g.A, g.sam, g.sak, m0, k0 + TK, g.M, kend, a_kfast);
      sb.load(g.B, g.sbn, g.sbk, n0, k0 + TK, g.N, kend, b_kfast);
    }
    const int kspan = min(TK, kend - k0);
#pragma unroll 4
    for (int kk = 0; kk < kspan; kk += 16) {
      uint32_t af[MT][4], bfr[NT][2];
#pragma unroll
      for (int i = 0; i < MT; ++i) {
        const int r0 = i * 16 + gq;
        af[i][0] = *reinterpret_cast<const uint32_t *>(&As[r0][kk + q * 2]);
        af[i][1] = *reinterpret_cast<const uint32_t *>(&As[r0 + 8][kk + q * 2]);
        af[i][2] = *reinterpret_cast<const uint32_t *>(&As[r0][kk + q * 2 + 8]);
        af[i][3] = *reinterpret_cast<const uint32_t *>(&As[r0 + 8][kk + q * 2 + 8]);
      }
#pragma unroll
      for (int j = 0; j < NT; ++j) {
        const int cc = warp * (TN / 4) + j * 8 + gq;
        bfr[j][0] = *reinterpret_cast<const uint32_t *>(&Bs[cc][kk + q * 2]);
        bfr[j][1] = *reinterpret_cast<const uint32_t *>(&Bs[cc][kk + q * 2 + 8]);
      }
#pragma unroll
      for (int i = 0; i < MT; ++i)
#pragma unroll
        for (int j = 0; j < NT; ++j) mma_bf16(acc[i][j], af[i], bfr[j]);
    }
    __syncthreads();
  }
  // epilogue
#pragma unroll
  for (int i = 0; i < MT; ++i)
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int m = m0 + i * 16 + gq + (r >= 2 ? 8 : 0);
        const int n = n0 + warp * (TN / 4) + j * 8 + q * 2 + (r & 1);
        if (m >= g.M || n >= g.N) continue;
        epilogue(g, m, n, acc[i][j][r]);
      }
}

// ------------------------------------------------------------- tcgen05 products
//
// C[M x N] = A[M x K] B[K x N] for A with K contiguous (sak = 1) and B with K contiguous
// (sbk = 1: B(k, n) at B[n sbn + k]), N and K multiples of 16 up to 256.  One CTA of four
// warps per 128 rows and column tile (all N, or halves of it when the rows alone would leave
// SMs idle): the A tile (128 x K) and the B tile (N x K) staged in shared memory in
// the canonical K-major layout without swizzle (core matrices of 8 rows x 16 bytes, the K
// direction LBO = 128 bytes apart, 8-row groups SBO = K/8 x 128 bytes apart), K/16
// tcgen05.mma (kind::f16, BF16 x BF16 -> FP32, M = 128) issued by one thread into a TMEM
// accumulator of 128 lanes x N columns, their completion signalled on an mbarrier
// (tcgen05.commit) and waited for with a time limit (a wait that runs out sets *err and
// skips the epilogue); then each warp reads its 32 TMEM lanes (rows) 16 columns at a time
// (tcgen05.ld) into the same epilogue as k_gemm.
constexpr int TC_M = 128;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor (tcgen05): start address, leading and stride byte
// offsets (16-byte units), descriptor version 1 at bit 46, no base offset, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ bool tc_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// gives up after 100 ms (the products take microseconds) or 2^24 tries
__device__ __forceinline__ bool tc_wait_bounded(uint32_t bar, uint32_t parity) {
  unsigned long long t0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (int it = 0; it < (1 << 24); ++it) {
    if (tc_try_wait(bar, parity)) return true;
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (t - t0 > 100000000ull) break;
  }
  return false;
}

// shared memory of k_gemm_tc: the mbarrier and the TMEM address, then from byte 1024 the
// operand tiles (A: 128 x K, B: ntile x K, canonical layout) and, once the products are done,
// in the same place the output tiles of the epilogue (BF16 pre-activations, BF16 outputs,
// FP32 outputs, as the product asks for them; rows of ntile + 8 (BF16) or + 4 (FP32) elements)
struct TcSmem {
  size_t z, c, f, total;
};

__host__ __device__ inline TcSmem tc_smem_layout(const Gemm &g, int ntile) {
  const size_t ops = (size_t)TC_M * g.K * 2 + (size_t)ntile * g.K * 2;
  const size_t tz = g.Zb ? (size_t)TC_M * (ntile + 8) * 2 : 0, tc = g.Cb ? (size_t)TC_M * (ntile + 8) * 2 : 0,
               tf = g.Cf ? (size_t)TC_M * (ntile + 4) * 4 : 0;
  TcSmem L;
  L.z = 1024;
  L.c = L.z + tz;
  L.f = L.c + tc;
  const size_t epi = tz + tc + tf;
  L.total = 1024 + (ops > epi ? ops : epi);
  return L;
}

__global__ void __launch_bounds__(128) k_gemm_tc(const Gemm g, int ntile, int *err, int fault) {
  extern __shared__ __align__(1024) uint8_t tc_smem[];
  // this CTA: rows m0.. (128), columns n0.. (ntile of them, a multiple of 16)
  const int n0 = blockIdx.y * ntile;
  const int K = g.K, N = ntile, kv = K / 8;
  const uint32_t sbo = (uint32_t)kv * 128u;
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(tc_smem);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(tc_smem + 8);
  uint8_t *As = tc_smem + 1024;
  uint8_t *Bs = As + (size_t)TC_M * K * 2;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * TC_M;
  const int rows = min(TC_M, g.M - m0);
  const uint32_t ncols = N <= 32 ? 32u : (N <= 64 ? 64u : (N <= 128 ? 128u : 256u));
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // staging by asynchronous 16-byte copies, all in flight at once (rows past M zero-filled):
  // vector (row r, K chunk j) -> (r / 8) SBO + j LBO + (r % 8) 16
  for (int v = tid; v < TC_M * kv; v += 128) {
    const int r = v / kv, j = v - r * kv;
    const bool in = r < rows;
    const bf16 *src = in ? g.A + (long long)(m0 + r) * g.sam + j * 8 : g.A;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(As + (r >> 3) * sbo + j * 128 + (r & 7) * 16)),
                 "l"(src), "r"(in ? 16 : 0)
                 : "memory");
  }
  for (int v = tid; v < N * kv; v += 128) {
    const int r = v / kv, j = v - r * kv;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(Bs + (r >> 3) * sbo + j * 128 + (r & 7) * 16)),
                 "l"(g.B + (long long)(n0 + r) * g.sbn + j * 8)
                 : "memory");
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  // the staged tiles to the tensor cores' (async) proxy; the TMEM address to every thread
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  if (tid == 0 && !fault) {  // (fault: the test hook, nothing issued, every wait runs out)
    // instruction descriptor: FP32 accumulator (bit 4), A and B BF16 (bits 7, 10), both
    // K-major, N / 8 at bit 17, M / 16 at bit 24
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
    const uint32_t a0 = smem_addr(As), b0 = smem_addr(Bs);
    for (int k = 0; k < K / 16; ++k) {
      const uint64_t ad = tc_desc(a0 + k * 256, 128, sbo), bd = tc_desc(b0 + k * 256, 128, sbo);
      const uint32_t accumulate = k > 0 ? 1u : 0u;
      asm volatile(
          "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
          "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
          ::"r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate)
          : "memory");
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
  }
  const bool ok = tc_wait_bounded(smem_addr(bar), 0);
  if (!ok && lane == 0) atomicExch(err, 1);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // every thread past the wait before the operand tiles are overwritten
  const bool all_ok = __syncthreads_and(ok) != 0;
  const TcSmem SL = tc_smem_layout(g, ntile);
  bf16 *Zt = reinterpret_cast<bf16 *>(tc_smem + SL.z);
  bf16 *Ct = reinterpret_cast<bf16 *>(tc_smem + SL.c);
  float *Ft = reinterpret_cast<float *>(tc_smem + SL.f);
  const int ldt = N + 8, ldf = N + 4;
  if (all_ok) {
    // TMEM -> registers (one row per thread, 16 columns at a time) -> epilogue -> output tiles
    const int rr = warp * 32 + lane, m = m0 + rr;
    for (int c0 = 0; c0 < N; c0 += 16) {
      uint32_t r[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (m < g.M) {
        bf16 dzv[16];
        if (g.dz) {
          const uint4 *dp = reinterpret_cast<const uint4 *>(g.dz + (long long)m * g.lddz + n0 + c0);
          *reinterpret_cast<uint4 *>(&dzv[0]) = dp[0];
          *reinterpret_cast<uint4 *>(&dzv[8]) = dp[1];
        }
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int n = n0 + c0 + q, c = c0 + q;
          float v = __uint_as_float(r[q]);
          if (g.bias) v += g.bias[n];
          if (g.Zb) Zt[rr * ldt + c] = __float2bfloat16(v);
          if (g.dz) {
            const float z = __bfloat162float(dzv[q]), sg = sigm(z);
            v *= sg * (1.f + z * (1.f - sg));
          }
          if (g.silu) v = v * sigm(v);
          if (g.Cf) Ft[rr * ldf + c] = v;
          if (g.Cb) Ct[rr * ldt + c] = __float2bfloat16(v);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
  }
  if (!all_ok) return;
  // the output tiles to global memory, 16 bytes per store along the rows
  const int nv = N / 8;
  for (int v = tid; v < rows * nv; v += 128) {
    const int r = v / nv, c = (v - r * nv) * 8;
    if (g.Zb) *reinterpret_cast<uint4 *>(g.Zb + (long long)(m0 + r) * g.ldzb + n0 + c) =
        *reinterpret_cast<const uint4 *>(Zt + r * ldt + c);
    if (g.Cb) *reinterpret_cast<uint4 *>(g.Cb + (long long)(m0 + r) * g.ldcb + n0 + c) =
        *reinterpret_cast<const uint4 *>(Ct + r * ldt + c);
  }
  if (g.Cf) {
    const int nf = N / 4;
    for (int v = tid; v < rows * nf; v += 128) {
      const int r = v / nf, c = (v - r * nf) * 4;
      *reinterpret_cast<float4 *>(g.Cf + (long long)(m0 + r) * g.ldcf + n0 + c) =
          *reinterpret_cast<const float4 *>(Ft + r * ldf + c);
    }
  }
}

// The weight-gradient products on the tcgen05 path: C[M x N] += A[M x K] B[K x N] with A and B
// contiguous along M and N (sam = 1, sbn = 1: the reduction runs over the batch rows, K; N
// padded to a multiple of 16, the columns past it zero), the
// K range split over blockIdx.z (kchunk each) and the results added to C with FP32 atomics.
// The operands are staged row-major by 16-byte asynchronous copies, then transposed in shared
// memory into the canonical K-major layout (a thread gathers 8 consecutive k of one row into
// one 16-byte slot).  K runs in stages of 64 through two buffers; a buffer is staged
// again only after the MMAs that read it have completed (one mbarrier per buffer, every wait
// bounded).  fault: the test hook, nothing issued.
constexpr int TCW_K = 64;

__host__ __device__ inline size_t tcw_smem(int ntile) {
  // two canonical buffers (A, B), then the row-major tiles the copies land in
  return 1024 + 3 * ((size_t)TC_M * TCW_K * 2 + (size_t)ntile * TCW_K * 2);
}

__global__ void __launch_bounds__(128) k_gemm_tc_wgrad(const Gemm g, int ntile, int *err, int fault) {
  extern __shared__ __align__(1024) uint8_t tc_smem[];
  const int N = ntile, n0 = blockIdx.y * ntile, m0 = blockIdx.x * TC_M;
  const int kbeg = blockIdx.z * g.kchunk, kend = min(g.K, kbeg + g.kchunk);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(tc_smem);  // one per buffer
  uint32_t *tslot = reinterpret_cast<uint32_t *>(tc_smem + 16);
  const size_t a_bytes = (size_t)TC_M * TCW_K * 2, b_bytes = (size_t)N * TCW_K * 2;
  const uint32_t sbo = (TCW_K / 8) * 128u;
  const uint32_t ncols = N <= 32 ? 32u : (N <= 64 ? 64u : (N <= 128 ? 128u : 256u));
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar + 1)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
  const int nst = kbeg < kend ? (kend - kbeg + TCW_K - 1) / TCW_K : 0;
  uint32_t phase[2] = {0u, 0u};
  bool ok = true;
  for (int st = 0; st < nst; ++st) {
    const int q = st & 1;
    uint8_t *As = tc_smem + 1024 + q * (a_bytes + b_bytes), *Bs = As + a_bytes;
    if (st >= 2) {  // the MMAs of stage st - 2 read this buffer
      if (ok) ok = tc_wait_bounded(smem_addr(bar + q), phase[q]);
      phase[q] ^= 1u;
    }
    const int k0 = kbeg + st * TCW_K;
    // the row-major tiles (64 k rows of 128 m, of N n) by 16-byte asynchronous copies, the
    // bytes past M, N or the K range zero-filled
    {
      bf16 *Ra = reinterpret_cast<bf16 *>(tc_smem + 1024 + 2 * (a_bytes + b_bytes));
      bf16 *Rb = Ra + TC_M * TCW_K;
      for (int v = tid; v < TCW_K * (TC_M / 8); v += 128) {
        const int k = v / (TC_M / 8), mv = (v - k * (TC_M / 8)) * 8, m = m0 + mv;
        const int valid = (k0 + k < kend) ? max(0, min(8, g.M - m)) : 0;
        const bf16 *src = valid ? g.A + (long long)(k0 + k) * g.sak + m : g.A;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(Ra + k * TC_M + mv)), "l"(src),
                     "r"(valid * 2)
                     : "memory");
      }
      for (int v = tid; v < TCW_K * (N / 8); v += 128) {
        const int k = v / (N / 8), nv = (v - k * (N / 8)) * 8, n = n0 + nv;
        const int valid = (k0 + k < kend) ? max(0, min(8, g.N - n)) : 0;
        const bf16 *src = valid ? g.B + (long long)(k0 + k) * g.sbk + n : g.B;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(Rb + k * N + nv)), "l"(src),
                     "r"(valid * 2)
                     : "memory");
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
      asm volatile("cp.async.wait_group 0;" ::: "memory");
      __syncthreads();
      // transposed into the canonical K-major layout: 8 consecutive k of one row per 16 bytes
      // (consecutive threads on consecutive rows: the shared-memory reads share words)
      for (int v = tid; v < TC_M * (TCW_K / 8); v += 128) {
        const int j = v / TC_M, r = v - j * TC_M;
        bf16 e[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) e[t] = Ra[(j * 8 + t) * TC_M + r];
        *reinterpret_cast<uint4 *>(As + (r >> 3) * sbo + j * 128 + (r & 7) * 16) = *reinterpret_cast<const uint4 *>(e);
      }
      for (int v = tid; v < N * (TCW_K / 8); v += 128) {
        const int j = v / N, r = v - j * N;
        bf16 e[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) e[t] = Rb[(j * 8 + t) * N + r];
        *reinterpret_cast<uint4 *>(Bs + (r >> 3) * sbo + j * 128 + (r & 7) * 16) = *reinterpret_cast<const uint4 *>(e);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (tid == 0 && !fault) {
      const uint32_t a0 = smem_addr(As), b0 = smem_addr(Bs);
      for (int kk = 0; kk < TCW_K / 16; ++kk) {
        const uint64_t ad = tc_desc(a0 + kk * 256, 128, sbo), bd = tc_desc(b0 + kk * 256, 128, sbo);
        const uint32_t accumulate = (st > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
            ::"r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar + q))
                   : "memory");
    }
  }
  // the last commit arrives when every MMA issued before it has completed
  if (nst > 0) {
    const int q = (nst - 1) & 1;
    if (ok) ok = tc_wait_bounded(smem_addr(bar + q), phase[q]);
  }
  if (!ok && lane == 0) atomicExch(err, 1);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const bool all_ok = __syncthreads_and(ok) != 0;
  if (all_ok && nst > 0) {
    const int m = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < N; c0 += 16) {
      uint32_t r[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (m < g.M) {
#pragma unroll
        for (int q = 0; q < 16; ++q)
          if (n0 + c0 + q < g.N) atomicAdd(&g.Cacc[(long long)m * g.ldca + n0 + c0 + q], __uint_as_float(r[q]));
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
  }
}

// raw features [n][IN] -> normalised BF16 [n][INP] (zero padded), clipped to six
// standard deviations so that inputs far outside the training data (a colloid the
// dynamics has thrown) meet the network's behaviour at the edge of that data
__global__ void k_features_in(const float *x, int n, const float *mean, const float *istd, bf16 *out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)n * INP) return;
  const int r = (int)(i / INP), c = (int)(i % INP);
  const float z = c < IN ? (x[(long long)r * IN + c] - mean[c]) * istd[c] : 0.f;
  out[i] = __float2bfloat16(fminf(fmaxf(z, -kInputClip), kInputClip));
}

// Gaussian negative log-likelihood of normalised targets under (mean, log-variance)
// outputs; writes d loss / d output (BF16, mean over the batch) and adds the loss sum
__global__ void k_nll(const float *o, const float *y, int n, const float *ymean, const float *yistd, bf16 *dout,
                      double *loss) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (r < n) {
    const float inv = 1.f / (float)n;
    for (int k = 0; k < NY; ++k) {
      const float t = (y[r * NY + k] - ymean[k]) * yistd[k];
      const float mu = o[r * OUTP + k];
      const float sraw = o[r * OUTP + NY + k];
      const float s = fminf(fmaxf(sraw, -kLogVarClamp), kLogVarClamp);
      const float e = __expf(-s), d = t - mu;
      l += 0.5f * (d * d * e + s);
      dout[r * OUTP + k] = __float2bfloat16(-d * e * inv);
      dout[r * OUTP + NY + k] = __float2bfloat16((sraw == s) ? 0.5f * (1.f - d * d * e) * inv : 0.f);
    }
    for (int k = OUT; k < OUTP; ++k) dout[r * OUTP + k] = __float2bfloat16(0.f);
  }
  // block sum, one atomic per block
  __shared__ float sh[256];
  sh[threadIdx.x] = l;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, (double)sh[0]);
}

// normalised outputs -> physical units: mean * std + mean, log-variance + 2 log std
__global__ void k_denorm(const float *o, int n, const float *ymean, const float *yistd, float *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * OUT) return;
  const int r = i / OUT, k = i % OUT;
  const float v = o[r * OUTP + k];
  out[i] = k < NY ? v / yistd[k] + ymean[k]
                  : fminf(fmaxf(v, -kLogVarClamp), kLogVarClamp) - 2.f * __logf(yistd[k - NY]);
}

// column sums of a BF16 matrix into FP32 (bias gradients), one atomic per (block, column)
__global__ void k_colsum(const bf16 *a, int n, int cols, long long lda, float *out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  const int per = (n + gridDim.y - 1) / gridDim.y, r0 = blockIdx.y * per, r1 = min(n, r0 + per);
  float s = 0.f;
  for (int r = r0; r < r1; ++r) s += __bfloat162float(a[r * lda + c]);
  atomicAdd(&out[c], s);
}

// the parameter layout: flat FP32 vector (W1 [IN][H], b1, W2 [H][H], b2, W3, b3, W4 [H][OUT], b4)
// and the padded BF16 weights the GEMMs read
struct Layout {
  long long w[4], b[4], total;
  int kin[4], nout[4];
};

Layout layout() {
  Layout L;
  const int kin[4] = {IN, H, H, H}, nout[4] = {H, H, H, OUT};
  long long o = 0;
  for (int l = 0; l < 4; ++l) {
    L.kin[l] = kin[l];
    L.nout[l] = nout[l];
    L.w[l] = o;
    o += (long long)kin[l] * nout[l];
    L.b[l] = o;
    o += nout[l];
  }
  L.total = o;
  return L;
}

// Adam on the FP32 masters, then the BF16 copies (weights at [k][n] of a padded
// [kpad][npad] matrix; biases stay FP32)
struct WeightCopies {
  bf16 *w[4];   // [kpad][npad] (k major rows of n): the warp-level products, inference
  bf16 *wt[4];  // [npad][kpad] (n major rows of k): the tcgen05 products of the forward pass
};

__global__ void k_adam(float *p, const float *gr, float *m, float *v, long long n, float lr, float b1, float b2,
                       float eps, float c1, float c2, Layout L, WeightCopies W, float *bias) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = gr[i];
  const float mi = b1 * m[i] + (1.f - b1) * g, vi = b2 * v[i] + (1.f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  const float x = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  p[i] = x;
  const int npad[4] = {H, H, H, OUTP}, kpad[4] = {INP, H, H, H};
  long long boff = 0;
  for (int l = 0; l < 4; ++l) {
    if (i >= L.w[l] && i < L.b[l]) {
      const long long j = i - L.w[l];
      const int k = (int)(j / L.nout[l]), c = (int)(j % L.nout[l]);
      W.w[l][(long long)k * npad[l] + c] = __float2bfloat16(x);
      W.wt[l][(long long)c * kpad[l] + k] = __float2bfloat16(x);
      return;
    }
    if (i >= L.b[l] && i < L.b[l] + L.nout[l]) {
      bias[boff + (i - L.b[l])] = x;
      return;
    }
    boff += npad[l];
  }
}

}  // namespace

struct mpcd_mlp {
  int max_batch = 0;
  Layout L;
  float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;  // flat FP32 params, grads, Adam moments
  bf16 *w[4] = {nullptr, nullptr, nullptr, nullptr};               // padded BF16 weights [k][n]
  bf16 *wt[4] = {nullptr, nullptr, nullptr, nullptr};              // the same transposed, [n][k]
  int *tc_err = nullptr;                                           // a tcgen05 wait ran out
  int tc_fault = 0;                                                // test hook (mpcd_mlp_set_fault)
  float *bias = nullptr;                                           // padded biases [H][H][H][OUTP]
  float *xmean = nullptr, *xistd = nullptr, *ymean = nullptr, *yistd = nullptr;
  bf16 *X = nullptr, *Z[3] = {nullptr, nullptr, nullptr}, *A[3] = {nullptr, nullptr, nullptr};
  float *O = nullptr;
  bf16 *dO = nullptr, *dA = nullptr, *dZ = nullptr;
  double *loss = nullptr;
  float *host_p = nullptr;
  int adam_t = 0;
  std::vector<void *> allocs;
  std::string err;
};

namespace {

int mfail(mpcd_mlp *n, int code, const std::string &e) {
  if (n) n->err = e;
  return code;
}

template <typename T>
T *dalloc(mpcd_mlp *n, size_t count) {
  void *p = nullptr;
  if (cudaMalloc(&p, count * sizeof(T) + 256) != cudaSuccess) {
    n->err = "out of device memory";
    return nullptr;
  }
  cudaMemset(p, 0, count * sizeof(T) + 256);
  n->allocs.push_back(p);
  return static_cast<T *>(p);
}

WeightCopies copies(const mpcd_mlp *nn) {
  WeightCopies W;
  for (int l = 0; l < 4; ++l) {
    W.w[l] = nn->w[l];
    W.wt[l] = nn->wt[l];
  }
  return W;
}

// a product on the tcgen05 path (A and B with K contiguous, N and K multiples of 16 up to 256)
void gemm_tc(mpcd_mlp *nn, cudaStream_t s, const Gemm &g) {
  // at least 80 KB of shared memory per CTA, so that at most two CTAs share an SM and their
  // TMEM columns (256 each at most) always fit in its 512: an allocation never waits
  const int mt = (g.M + TC_M - 1) / TC_M;
  const int ntile = (mt < 120 && g.N % 32 == 0 && g.N >= 64) ? g.N / 2 : g.N;
  const size_t need = tc_smem_layout(g, ntile).total;
  const size_t smem = need > 80 * 1024 ? need : 80 * 1024;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 1024 + TC_M * 256 * 2 + 256 * 256 * 2);
    attr = true;
  }
  k_gemm_tc<<<dim3((unsigned)mt, (unsigned)(g.N / ntile)), 128, smem, s>>>(g, ntile, nn->tc_err, nn->tc_fault);
}

// a weight-gradient product on the tcgen05 path (A and B contiguous along M and N, K the batch)
void gemm_tc_wgrad(mpcd_mlp *nn, cudaStream_t s, Gemm g) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_gemm_tc_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tcw_smem(256));
    attr = true;
  }
  const int mt = (g.M + TC_M - 1) / TC_M;
  // (N padded to the MMA's multiple of 16; the columns past N read as zero and are not stored)
  const int np = (g.N + 15) & ~15;
  const int ntile = (np % 32 == 0 && np >= 64) ? np / 2 : np;
  // about 32 K slices of at least one stage each
  const int per = (g.K + 31) / 32;
  g.kchunk = ((per + TCW_K - 1) / TCW_K) * TCW_K;
  const int kz = (g.K + g.kchunk - 1) / g.kchunk;
  const size_t need = tcw_smem(ntile);
  const size_t smem = need > 80 * 1024 ? need : 80 * 1024;  // (two CTAs per SM at most: TMEM fits)
  k_gemm_tc_wgrad<<<dim3((unsigned)mt, (unsigned)(np / ntile), (unsigned)kz), 128, smem, s>>>(g, ntile, nn->tc_err,
                                                                                           nn->tc_fault);
}

void gemm(cudaStream_t s, Gemm g, int ksplit = 1) {
  if (g.K <= 256 && ksplit == 1) {
    // whole K in one staging, 32 x 32 tiles: many blocks for inference-sized M
    g.kchunk = g.K;
    dim3 grid((g.N + 31) / 32, (g.M + 31) / 32, 1);
    k_gemm<32, 32, 256><<<grid, 128, 0, s>>>(g);
    return;
  }
  g.kchunk = ksplit > 1 ? ((g.K + ksplit - 1) / ksplit + BK - 1) / BK * BK : g.K;
  const int kz = ksplit > 1 ? (g.K + g.kchunk - 1) / g.kchunk : 1;
  dim3 grid((g.N + BN - 1) / BN, (g.M + BM - 1) / BM, kz);
  k_gemm<BM, BN, BK><<<grid, 128, 0, s>>>(g);
}

Gemm base() {
  Gemm g;
  memset(&g, 0, sizeof g);
  return g;
}

const int kNpad[4] = {H, H, H, OUTP};
const int kKpad[4] = {INP, H, H, H};

long long bias_off(int l) {
  long long o = 0;
  for (int i = 0; i < l; ++i) o += kNpad[i];
  return o;
}

// forward of rows [0, n) of n->X; stores Z (pre-activations) and A (activations) for the backward
// pass.  tc: the products on the tcgen05 path (training), else the warp-level kernel (inference)
void forward(mpcd_mlp *nn, int n, cudaStream_t s, bool tc) {
  const bf16 *in = nn->X;
  long long ldin = INP;
  for (int l = 0; l < 4; ++l) {
    Gemm g = base();
    g.A = in; g.sam = ldin; g.sak = 1;
    if (tc) {
      g.B = nn->wt[l]; g.sbk = 1; g.sbn = kKpad[l];
    } else {
      g.B = nn->w[l]; g.sbk = kNpad[l]; g.sbn = 1;
    }
    g.M = n; g.N = kNpad[l]; g.K = kKpad[l];
    g.bias = nn->bias + bias_off(l);
    if (l < 3) {
      g.silu = 1;
      g.Zb = nn->Z[l]; g.ldzb = H;
      g.Cb = nn->A[l]; g.ldcb = H;
      in = nn->A[l];
      ldin = H;
    } else {
      g.Cf = nn->O; g.ldcf = OUTP;
    }
    if (tc) gemm_tc(nn, s, g);
    else gemm(s, g);
  }
}

// gradients of the mean loss over rows [0, n) into n->g (zeroed first)
void backward(mpcd_mlp *nn, int n, cudaStream_t s) {
  cudaMemsetAsync(nn->g, 0, sizeof(float) * nn->L.total, s);
  const bf16 *dcur = nn->dO;  // gradient w.r.t. the output of layer l (after its activation)
  long long ldd = OUTP;
  for (int l = 3; l >= 0; --l) {
    const int kin = nn->L.kin[l], nout = nn->L.nout[l];
    const bf16 *act = l > 0 ? nn->A[l - 1] : nn->X;
    const long long ldact = l > 0 ? H : INP;
    // dW[k][c] = sum_b act[b][k] dcur[b][c]  (dcur is already d/d(pre-activation) of layer l)
    Gemm gw = base();
    gw.A = act; gw.sam = 1; gw.sak = ldact;
    gw.B = dcur; gw.sbk = ldd; gw.sbn = 1;
    gw.M = kin; gw.N = nout; gw.K = n;
    gw.Cacc = nn->g + nn->L.w[l]; gw.ldca = nout;
    gemm_tc_wgrad(nn, s, gw);
    dim3 cg((nout + 127) / 128, n >= 4096 ? 32 : 1);
    k_colsum<<<cg, 128, 0, s>>>(dcur, n, nout, ldd, nn->g + nn->L.b[l]);
    if (l == 0) break;
    // d/d(pre-activation of layer l-1) = (dcur W_l^T) * silu'(Z_{l-1})
    Gemm gd = base();
    gd.A = dcur; gd.sam = ldd; gd.sak = 1;
    gd.B = nn->w[l]; gd.sbk = 1; gd.sbn = kNpad[l];  // B(k = c, n = i) = W_l[i][c]
    gd.M = n; gd.N = H; gd.K = kNpad[l];
    gd.dz = nn->Z[l - 1]; gd.lddz = H;
    bf16 *dst = (l % 2) ? nn->dA : nn->dZ;
    gd.Cb = dst; gd.ldcb = H;
    gemm_tc(nn, s, gd);
    dcur = dst;
    ldd = H;
  }
}

void init_params(mpcd_mlp *nn, uint64_t seed, std::vector<float> &h) {
  std::mt19937_64 rng(seed);
  h.assign(nn->L.total, 0.f);
  for (int l = 0; l < 4; ++l) {
    const float a = std::sqrt(6.f / (float)(nn->L.kin[l] + nn->L.nout[l]));  // Glorot uniform
    std::uniform_real_distribution<float> u(-a, a);
    for (long long i = nn->L.w[l]; i < nn->L.b[l]; ++i) h[i] = u(rng);
  }
}

int upload_params(mpcd_mlp *nn, const float *h) {
  if (cudaMemcpy(nn->p, h, sizeof(float) * nn->L.total, cudaMemcpyHostToDevice) != cudaSuccess)
    return mfail(nn, MPCD_ERR_CUDA, "parameter upload");
  // zero gradient, zero learning rate: writes the BF16 copies and biases from the masters
  cudaMemset(nn->g, 0, sizeof(float) * nn->L.total);
  const long long n = nn->L.total;
  k_adam<<<(unsigned)((n + 255) / 256), 256>>>(nn->p, nn->g, nn->m, nn->v, n, 0.f, 0.9f, 0.999f, 1e-8f, 1.f, 1.f,
                                              nn->L, copies(nn), nn->bias);
  cudaMemset(nn->m, 0, sizeof(float) * n);
  cudaMemset(nn->v, 0, sizeof(float) * n);
  return cudaDeviceSynchronize() == cudaSuccess ? MPCD_OK : mfail(nn, MPCD_ERR_CUDA, "parameter upload");
}

int stage_inputs(mpcd_mlp *nn, const float *x, int n, cudaStream_t s) {
  if (n < 1 || n > nn->max_batch) return mfail(nn, MPCD_ERR_CAPACITY, "batch larger than max_batch");
  const long long tot = (long long)n * INP;
  k_features_in<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(x, n, nn->xmean, nn->xistd, nn->X);
  return MPCD_OK;
}

}  // namespace

extern "C" int mpcd_mlp_create(int max_batch, uint64_t seed, mpcd_mlp **out) {
  if (!out || max_batch < 1) return MPCD_ERR_PARAM;
  *out = nullptr;
  mpcd_mlp *nn = new mpcd_mlp();
  nn->max_batch = max_batch;
  nn->L = layout();
  const long long P = nn->L.total;
  nn->p = dalloc<float>(nn, P); nn->g = dalloc<float>(nn, P); nn->m = dalloc<float>(nn, P); nn->v = dalloc<float>(nn, P);
  for (int l = 0; l < 4; ++l) {
    nn->w[l] = dalloc<bf16>(nn, (size_t)kKpad[l] * kNpad[l]);
    nn->wt[l] = dalloc<bf16>(nn, (size_t)kKpad[l] * kNpad[l]);
  }
  nn->tc_err = dalloc<int>(nn, 1);
  nn->bias = dalloc<float>(nn, 3 * H + OUTP);
  nn->xmean = dalloc<float>(nn, IN); nn->xistd = dalloc<float>(nn, IN);
  nn->ymean = dalloc<float>(nn, NY); nn->yistd = dalloc<float>(nn, NY);
  const size_t B = (size_t)max_batch;
  nn->X = dalloc<bf16>(nn, B * INP);
  for (int l = 0; l < 3; ++l) {
    nn->Z[l] = dalloc<bf16>(nn, B * H);
    nn->A[l] = dalloc<bf16>(nn, B * H);
  }
  nn->O = dalloc<float>(nn, B * OUTP);
  nn->dO = dalloc<bf16>(nn, B * OUTP);
  nn->dA = dalloc<bf16>(nn, B * H);
  nn->dZ = dalloc<bf16>(nn, B * H);
  nn->loss = dalloc<double>(nn, 1);
  if (!nn->err.empty()) {
    mpcd_mlp_destroy(nn);
    return MPCD_ERR_NOMEM;
  }
  std::vector<float> one(IN, 1.f), zero(IN, 0.f);
  cudaMemcpy(nn->xistd, one.data(), sizeof(float) * IN, cudaMemcpyHostToDevice);
  cudaMemcpy(nn->yistd, one.data(), sizeof(float) * NY, cudaMemcpyHostToDevice);
  std::vector<float> h;
  init_params(nn, seed, h);
  int r = upload_params(nn, h.data());
  if (r) {
    mpcd_mlp_destroy(nn);
    return r;
  }
  *out = nn;
  return MPCD_OK;
}

extern "C" int mpcd_mlp_destroy(mpcd_mlp *nn) {
  if (!nn) return MPCD_ERR_PARAM;
  cudaDeviceSynchronize();
  for (void *a : nn->allocs) cudaFree(a);
  delete nn;
  return MPCD_OK;
}

extern "C" const char *mpcd_mlp_last_error(const mpcd_mlp *nn) { return nn ? nn->err.c_str() : "null network"; }

extern "C" int64_t mpcd_mlp_param_count(const mpcd_mlp *nn) { return nn ? nn->L.total : -1; }

extern "C" int mpcd_mlp_set_normalisation(mpcd_mlp *nn, const float *x_mean, const float *x_std, const float *y_mean,
                                          const float *y_std) {
  if (!nn || !x_mean || !x_std || !y_mean || !y_std) return MPCD_ERR_PARAM;
  std::vector<float> xi(IN), yi(NY);
  for (int i = 0; i < IN; ++i) xi[i] = x_std[i] > 0 ? 1.f / x_std[i] : 0.f;
  for (int i = 0; i < NY; ++i) yi[i] = y_std[i] > 0 ? 1.f / y_std[i] : 0.f;
  if (cudaMemcpy(nn->xmean, x_mean, sizeof(float) * IN, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(nn->xistd, xi.data(), sizeof(float) * IN, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(nn->ymean, y_mean, sizeof(float) * NY, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(nn->yistd, yi.data(), sizeof(float) * NY, cudaMemcpyHostToDevice) != cudaSuccess)
    return mfail(nn, MPCD_ERR_CUDA, "normalisation upload");
  return MPCD_OK;
}

extern "C" int mpcd_mlp_get_params(mpcd_mlp *nn, float *out) {
  if (!nn || !out) return MPCD_ERR_PARAM;
  if (cudaMemcpy(out, nn->p, sizeof(float) * nn->L.total, cudaMemcpyDeviceToHost) != cudaSuccess)
    return mfail(nn, MPCD_ERR_CUDA, "parameter download");
  return MPCD_OK;
}

extern "C" int mpcd_mlp_set_params(mpcd_mlp *nn, const float *in) {
  if (!nn || !in) return MPCD_ERR_PARAM;
  return upload_params(nn, in);
}

extern "C" int mpcd_mlp_forward(mpcd_mlp *nn, const float *x, int n, float *out, void *stream) {
  if (!nn || !x || !out) return MPCD_ERR_PARAM;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int r = stage_inputs(nn, x, n, s);
  if (r) return r;
  forward(nn, n, s, false);
  k_denorm<<<(n * OUT + 255) / 256, 256, 0, s>>>(nn->O, n, nn->ymean, nn->yistd, out);
  return cudaGetLastError() == cudaSuccess ? MPCD_OK : mfail(nn, MPCD_ERR_CUDA, "forward launch");
}

extern "C" int mpcd_mlp_grad(mpcd_mlp *nn, const float *x, const float *y, int n, float *grad, double *loss) {
  if (!nn || !x || !y) return MPCD_ERR_PARAM;
  int r = stage_inputs(nn, x, n, nullptr);
  if (r) return r;
  forward(nn, n, nullptr, true);
  cudaMemset(nn->loss, 0, sizeof(double));
  k_nll<<<(n + 255) / 256, 256>>>(nn->O, y, n, nn->ymean, nn->yistd, nn->dO, nn->loss);
  backward(nn, n, nullptr);
  if (grad && cudaMemcpy(grad, nn->g, sizeof(float) * nn->L.total, cudaMemcpyDeviceToHost) != cudaSuccess)
    return mfail(nn, MPCD_ERR_CUDA, "gradient download");
  double l = 0;
  if (cudaMemcpy(&l, nn->loss, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    return mfail(nn, MPCD_ERR_CUDA, "loss download");
  int te = 0;
  if (cudaMemcpy(&te, nn->tc_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return mfail(nn, MPCD_ERR_CUDA, "status download");
  if (te) {
    // reported once; the next call starts afresh
    cudaMemset(nn->tc_err, 0, sizeof(int));
    return mfail(nn, MPCD_ERR_CUDA, "a tensor-core product did not complete within its time limit");
  }
  if (loss) *loss = l / n;
  return MPCD_OK;
}

extern "C" int mpcd_mlp_set_fault(mpcd_mlp *nn, int on) {
  if (!nn) return MPCD_ERR_PARAM;
  nn->tc_fault = on ? 1 : 0;
  return MPCD_OK;
}

extern "C" int mpcd_mlp_train_step(mpcd_mlp *nn, const float *x, const float *y, int n, float lr, double *loss) {
  int r = mpcd_mlp_grad(nn, x, y, n, nullptr, loss);
  if (r) return r;
  nn->adam_t += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f / (1.f - std::pow(b1, (float)nn->adam_t)), c2 = 1.f / (1.f - std::pow(b2, (float)nn->adam_t));
  const long long P = nn->L.total;
  k_adam<<<(unsigned)((P + 255) / 256), 256>>>(nn->p, nn->g, nn->m, nn->v, P, lr, b1, b2, 1e-8f, c1, c2, nn->L,
                                              copies(nn), nn->bias);
  return cudaGetLastError() == cudaSuccess ? MPCD_OK : mfail(nn, MPCD_ERR_CUDA, "adam launch");
}

MlpIO mlp_io(mpcd_mlp *nn) {
  MlpIO io;
  io.xmean = nn->xmean; io.xistd = nn->xistd;
  io.ymean = nn->ymean; io.yistd = nn->yistd;
  for (int l = 0; l < 4; ++l) io.w[l] = nn->w[l];
  io.bias = nn->bias;
  return io;
}
