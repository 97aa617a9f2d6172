// Device code shared by the FP64 and FP32-compensated forms: the reference's
// cell and block rules, the epoch-tagged fluid-to-colloid tables, the exact
// exchange sums, the stochastic reflection, and the per-colloid work (WCA forces,
// orientation update, table build) that both forms run in FP64.
#pragma once
#include "kernels.cuh"

namespace bgb {

constexpr unsigned FULL = 0xFFFFFFFFu;

// ----------------------------------------------------------------- cell helpers

static __device__ __forceinline__ int lin_cell(const SysF64 &S, int ix, int iy, int iz) { return ix + S.Lx * (iy + S.Ly * iz); }

static __device__ __forceinline__ bool off_ok(int d, int L) {
  int m = d % L;
  if (m < 0) m += L;
  return m <= 3 || m >= L - 3;
}

// Is cell `lin` one of the 342 neighbour boxes of cell `cb` (create_box,
// cpp/neighbour_list.cpp:12-25: periodic offsets -3..3 per axis, own box
// excluded)?  Cell numbers >= C (a coordinate exactly at L past the last row)
// have no neighbour entries in the reference.
static __device__ __forceinline__ bool in_block(const SysF64 &S, int cb, int lin) {
  if (cb >= S.C || lin >= S.C) return false;
  if (cb == lin) return S.physics != 0;  // the reference skips the own box; the fixed rules keep it
  int cx = cb % S.Lx, ct = cb / S.Lx, cy = ct % S.Ly, cz = ct / S.Ly;
  int bx = lin % S.Lx, bt = lin / S.Lx, by = bt % S.Ly, bz = bt / S.Ly;
  return off_ok(bx - cx, S.Lx) && off_ok(by - cy, S.Ly) && off_ok(bz - cz, S.Lz);
}

// 1 + cell(pos) - 1: the reference's truncating linear cell of a wrapped position.
// A wrapped coordinate lies in [0, L], so each integer part is at most L and the
// cell number stays below Cpad; anything else (NaN, a negative or runaway
// position) is clamped, flagged, and never used to index past the tables.
static __device__ __forceinline__ int cell_of_pos(const SysF64 &S, double x, double y, double z, bool &alias) {
  int ix = trunc_nonneg(x), iy = trunc_nonneg(y), iz = trunc_nonneg(z);
  bool bad = (ix > S.Lx) | (iy > S.Ly) | (iz > S.Lz) | (dbits(x) < 0) | (dbits(y) < 0) | (dbits(z) < 0);
  if (bad) {
    atomicOr(&S.ss->err, ERRB_VRANGE);
    ix = min(ix, S.Lx); iy = min(iy, S.Ly); iz = min(iz, S.Lz);
  }
  alias = (ix >= S.Lx) | (iy >= S.Ly) | (iz >= S.Lz);
  return lin_cell(S, ix, iy, iz);
}

// Base index in a shared list for the lanes in mask m of this warp, from one
// global atomic per block (the whole block must call it): for the run() records
// of a last substep, about one particle in sixteen, too many for one atomic per
// warp on a single counter.
static __device__ __forceinline__ int block_base_n(int *counter, int warp_count, int lane) {
  __shared__ int s_tot, s_base;
  if (threadIdx.x == 0) s_tot = 0;
  __syncthreads();
  int off = 0;
  if (lane == 0 && warp_count) off = atomicAdd(&s_tot, warp_count);
  __syncthreads();
  if (threadIdx.x == 0) s_base = s_tot ? atomicAdd(counter, s_tot) : 0;
  __syncthreads();
  return s_base + __shfl_sync(FULL, off, 0);
}

static __device__ __forceinline__ int block_base(int *counter, unsigned m, int lane) {
  return block_base_n(counter, __popc(m), lane);
}

// Batched launches, persistent: the systems' virtual blocks (system r has boff[r+1] -
// boff[r] of them; boff ascending, boff[nrep] in all) are shared out in contiguous runs
// over the grid's blocks, a few resident per SM: block b runs the virtual blocks
// [b T / G, (b+1) T / G) one after another, each as virtual block v - boff[r] of the
// boff[r+1] - boff[r] of its system r, with that system's SysF64 copied into shared
// memory when the run reaches it (a run crosses a system boundary at most a few times).
// body(VB, NVB) must be called by the whole block, as a kernel body would be.
template <typename Body>
static __device__ __forceinline__ void batch_for(const SysF64 *Ss, const int *boff, int nrep, SysF64 &sS, Body body) {
  __shared__ int s_r;
  const int total = boff[nrep];
  const int v0 = (int)((long long)blockIdx.x * total / gridDim.x);
  const int v1 = (int)((long long)(blockIdx.x + 1) * total / gridDim.x);
  if (v0 >= v1) return;
  if (threadIdx.x == 0) {
    int lo = 0, hi = nrep;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (boff[mid] <= v0) lo = mid;
      else hi = mid;
    }
    s_r = lo;
  }
  __syncthreads();
  int r = s_r;
  int first = boff[r], next = boff[r + 1];
  auto load = [&](int q) {
    const int *src = reinterpret_cast<const int *>(Ss + q);
    int *dst = reinterpret_cast<int *>(&sS);
    for (int k = threadIdx.x; k < (int)(sizeof(SysF64) / sizeof(int)); k += blockDim.x) dst[k] = src[k];
  };
  load(r);
  __syncthreads();
  for (int v = v0; v < v1; ++v) {
    if (v >= next) {  // the run reaches the next system (systems without blocks skipped)
      do {
        ++r;
        first = next;
        next = boff[r + 1];
      } while (v >= next);
      load(r);
      __syncthreads();
    }
    body(v - first, next - first);
    __syncthreads();  // the body's shared memory and the descriptor are reused
  }
}

// A cell-table entry is (tag << 32) | count with tag = substep + 1: substeps
// start at -1 (the set-up table), tags at 0, and tags only grow between two
// invalidations (which zero the tables), so an older entry always has a smaller
// tag.  Count of the entry if it belongs to substep g:
static __device__ __forceinline__ int tcount(unsigned long long v, long long g) {
  return (unsigned)(v >> 32) == (unsigned)(g + 1) ? (int)(unsigned)v : 0;
}

// append colloid j to cell `cell` of the table of substep e: the maximum turns
// an entry of an earlier substep into (e, 0) and leaves one of substep e as it
// is; the add then takes a slot (two atomics on one address from one thread
// take effect in program order)
static __device__ __forceinline__ void tappend(unsigned long long *Tc, uint16_t *Tl, int cell, long long e, int j, int *err) {
  const unsigned long long tag = (unsigned long long)(unsigned)(e + 1) << 32;
  atomicMax(&Tc[cell], tag);
  const int slot = (int)(unsigned)atomicAdd(&Tc[cell], 1ull);
  if (slot < TCAP) Tl[(size_t)cell * TCAP + slot] = (uint16_t)j;
  else atomicOr(err, ERRB_TTABLE);
}

// --------------------------------------------------------------- exact cell sums

// one particle's terms of the exact cell sums (count, fixed-point w or v, |w|^2)
static __device__ __forceinline__ void bin_add(CellAcc *a, int n, long long fx, long long fy, long long fz,
                                               long long f2) {
  atomicAdd(&a->n, n);
  atomicAdd((unsigned long long *)&a->sx, (unsigned long long)fx);
  atomicAdd((unsigned long long *)&a->sy, (unsigned long long)fy);
  atomicAdd((unsigned long long *)&a->sz, (unsigned long long)fz);
  atomicAdd((unsigned long long *)&a->s2, (unsigned long long)f2);
}

// The same for one particle per lane (cell c < 0: none), the whole warp calling: lanes of
// equal cell (__match_any_sync) gather their terms onto the group's first lane, which
// adds them with one set of atomics.  The gathering jumps pointers along the group
// (each lane's next higher lane of its cell): after round r a lane holds the sum of
// itself and its next 2^r - 1 group members, so ceil(log2(size)) rounds leave the total
// on the first lane.  The sums are integers, so the result does not depend on the order.
static __device__ __forceinline__ void bin_add_warp(CellAcc *acc, int c, long long fx, long long fy, long long fz,
                                                    long long f2) {
  const int lane = threadIdx.x & 31;
  const unsigned peers = __match_any_sync(0xFFFFFFFFu, c);
  const unsigned above = peers & ~((2u << lane) - 1u);
  int nxt = above ? __ffs(above) - 1 : -1;
  unsigned long long sx = (unsigned long long)fx, sy = (unsigned long long)fy, sz = (unsigned long long)fz,
                     s2 = (unsigned long long)f2;
  int n = c >= 0 ? 1 : 0;
  while (__any_sync(0xFFFFFFFFu, nxt >= 0)) {
    const int src = nxt >= 0 ? nxt : lane;
    const unsigned long long ax = __shfl_sync(0xFFFFFFFFu, sx, src), ay = __shfl_sync(0xFFFFFFFFu, sy, src),
                             az = __shfl_sync(0xFFFFFFFFu, sz, src), a2 = __shfl_sync(0xFFFFFFFFu, s2, src);
    const int an = __shfl_sync(0xFFFFFFFFu, n, src), anx = __shfl_sync(0xFFFFFFFFu, nxt, src);
    if (nxt >= 0) {
      sx += ax; sy += ay; sz += az; s2 += a2;
      n += an;
      nxt = anx;
    }
  }
  if (c >= 0 && lane == __ffs(peers) - 1) bin_add(acc + c, n, (long long)sx, (long long)sy, (long long)sz, (long long)s2);
}

// FP32 copy of a double by truncating the mantissa (integer pipe); relative
// error below 2^-23
static __device__ __forceinline__ float d2f_trunc(double x) {
  long long b = dbits(x);
  int e = (int)((b >> 52) & 0x7FF);
  if (e == 0) return 0.f;
  int fe = e - 1023 + 127;
  if (fe <= 0) return 0.f;
  if (fe >= 255) return __int_as_float(0x7f800000);
  unsigned m = (unsigned)((b >> 29) & 0x7FFFFF);
  return __uint_as_float(((unsigned)((unsigned long long)b >> 32) & 0x80000000u) | ((unsigned)fe << 23) | m);
}

static __device__ __forceinline__ float wrap_half(float d, float L) {
  if (d > 0.5f * L) d -= L;
  else if (d < -0.5f * L) d += L;
  return d;
}

// ----------------------------------------------------------- exact exchange sums

// One exchange component split as hi = to_fix(v, 20), lo = to_fix(res, 72) with
// res = v - hi 2^-20 (exact in FP64), computed on the integer pipe only.  With
// v = +-M 2^E (M the 53-bit significand) and T = E + 72: for T >= 0, v 2^72 is an
// integer and lo = v 2^72 - hi 2^52 exactly, a difference that fits 64 bits, so
// wrap-around arithmetic gives it; for T < 0, |v| < 2^-19, hi is 0 (or +-1 when
// T = -1) and lo = round_half_even((+-M - hi 2^(52-T)) 2^T).  Denormals give 0, as
// to_fix does.  |v| < 2^20 (checked by the caller) keeps T <= 40.
static __device__ __forceinline__ void exch_split(double v, long long &hi, long long &lo) {
  const long long b = dbits(v);
  const int ex = (int)((b >> 52) & 0x7FF);
  hi = to_fix(v, 20);
  const unsigned long long M = ((unsigned long long)b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const int T = ex - 1075 + 72;
  const bool neg = b < 0;
  if (ex == 0) {
    lo = 0;
  } else if (T >= 0) {
    const unsigned long long X = T < 64 ? M << T : 0ull;
    lo = (long long)((neg ? 0ull - X : X) - ((unsigned long long)hi << 52));
  } else {
    const long long N = (neg ? -(long long)M : (long long)M) - (hi != 0 ? hi * (1ll << 53) : 0ll);
    const unsigned long long A = (unsigned long long)(N < 0 ? -N : N);
    const int s = -T;
    unsigned long long r = 0;
    if (s < 63) {
      r = A >> s;
      const unsigned long long rem = A & ((1ull << s) - 1ull), half = 1ull << (s - 1);
      if (rem > half || (rem == half && (r & 1ull))) r += 1ull;
    }
    lo = N < 0 ? -(long long)r : (long long)r;
  }
}

// The six components of one collision's exchange (dv, dl) at once: range test,
// split, then the twelve atomics.
static __device__ __forceinline__ void exch_add6(ExchAcc *e, d3 dv, d3 dl, int *err) {
  const double v[6] = {dv.x, dv.y, dv.z, dl.x, dl.y, dl.z};
  long long hi[6], lo[6];
  bool bad = false;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    bad |= (dbits(v[k]) & 0x7FFFFFFFFFFFFFFFll) >= 0x4130000000000000ll;  // |v| >= 2^20 (or NaN)
    exch_split(v[k], hi[k], lo[k]);
  }
  if (bad) atomicOr(err, ERRB_DELTA);
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    atomicAdd((unsigned long long *)&e->hi[k], (unsigned long long)hi[k]);
    atomicAdd((unsigned long long *)&e->lo[k], (unsigned long long)lo[k]);
  }
}

static __device__ __forceinline__ double exch_val(const ExchAcc &e, int comp) {
  return __dadd_rn((double)e.hi[comp] * 0x1p-20, (double)e.lo[comp] * 0x1p-72);
}

// ------------------------------------------------------- stochastic reflection

struct CollDraw {
  uint2 key;
  uint32_t a, b, t;
  int idx;
  uint4 buf;
};

static __device__ __forceinline__ double cd_next(CollDraw &d) {
  int s = d.idx & 3;
  if (s == 0) d.buf = draw4(d.key, DOM_COLL, (uint32_t)(d.idx >> 2), d.a, d.b, d.t);
  d.idx++;
  uint32_t w = s == 0 ? d.buf.x : s == 1 ? d.buf.y : s == 2 ? d.buf.z : d.buf.w;
  return u01(w);
}

// stochastic_reflection (cpp/fluid_colloid_collision.cpp:7-24): Rayleigh normal
// speed along rs plus one Gaussian tangential component along unit(un x t).
// Draws in the reference's order: u, the three components of t, then pairs of
// Box-Muller tries.  The first eight come from two Philox blocks (refl_blocks); a
// third block onwards serves the rare case of two rejected tries.  The four
// independent chains below (Rayleigh speed, Gaussian, unit normal, t) are separate
// functions so that the event pass can run them on different warps; refl_combine
// joins them.  Each is the same sequence of rounded operations wherever it runs.
static __device__ __forceinline__ void refl_blocks(const SysF64 &S, uint32_t a, uint32_t b, uint32_t t, uint4 &r0,
                                                   uint4 &r1) {
  r0 = draw4(S.key, DOM_COLL, 0, a, b, t);
  r1 = draw4(S.key, DOM_COLL, 1, a, b, t);
}

// the Rayleigh speed: sqrt(-log((1 - u)^2) kT/m)  (/m_beta as * kT/m)
static __device__ __forceinline__ double refl_speed(const SysF64 &S, uint4 r0) {
  const double om = __dsub_rn(1.0, u01(r0.x));
  const double random_e = __dmul_rn(om, om);
  return __dsqrt_rn(__dmul_rn(-log(random_e), S.inv_m_beta));
}

// the tangential Gaussians x1 sqrt(-2 log z / z) sqrt(kT/m) (and, into *v2, the
// same with x2, which only the fixed rules use), polar Box-Muller: each try is a
// fixed function of the key, a try is rejected with probability 1 - pi/4, so 256
// tries never run out.  The second try is computed by every lane and selected
// (2 ran - 1 is exact: pm1 builds it from the draw's bits); only two rejections
// in a row (1 in 22) branch.
static __device__ __forceinline__ double refl_gauss(const SysF64 &S, uint4 r1, uint32_t a, uint32_t b, uint32_t t,
                                                    double *v2) {
  double x1 = pm1(r1.x), x2 = pm1(r1.y);
  double z = __dadd_rn(__dmul_rn(x1, x1), __dmul_rn(x2, x2));
  const double x1b = pm1(r1.z), x2b = pm1(r1.w);
  const double zb = __dadd_rn(__dmul_rn(x1b, x1b), __dmul_rn(x2b, x2b));
  const bool second = z > 1.0;
  x1 = second ? x1b : x1;
  x2 = second ? x2b : x2;
  z = second ? zb : z;
  if (z > 1.0) {
    CollDraw d;
    d.key = S.key; d.a = a; d.b = b; d.t = t; d.idx = 8;
    for (int it = 2; z > 1.0 && it < 256; ++it) {
      x1 = __dsub_rn(__dmul_rn(2.0, cd_next(d)), 1.0);
      x2 = __dsub_rn(__dmul_rn(2.0, cd_next(d)), 1.0);
      z = __dadd_rn(__dmul_rn(x1, x1), __dmul_rn(x2, x2));
    }
  }
  // -2 log(z) / z as -2 log(z) times 1/z (the reciprocal overlaps the logarithm; within an ulp)
  const double g = __dsqrt_rn(__dmul_rn(__dmul_rn(-2.0, log(z)), __drcp_rn(z)));
  *v2 = __dmul_rn(__dmul_rn(x2, g), S.sqrt_kt_m);
  return __dmul_rn(__dmul_rn(x1, g), S.sqrt_kt_m);
}

// vector / |vector| as one reciprocal square root and three products (within a few ulp of
// the reference's three divisions)
static __device__ __forceinline__ d3 refl_unit(d3 v) { return mul3s(v, rsqrt(norm2_ref(v.x, v.y, v.z))); }

// t = img(ran L - rf), the random point relative to the particle
static __device__ __forceinline__ d3 refl_point(const SysF64 &S, uint4 r0, d3 rf) {
  return mk(ref_img(__dsub_rn(__dmul_rn(u01(r0.y), S.dx.L), rf.x), S.dx),
            ref_img(__dsub_rn(__dmul_rn(u01(r0.z), S.dy.L), rf.y), S.dy),
            ref_img(__dsub_rn(__dmul_rn(u01(r0.w), S.dz.L), rf.z), S.dz));
}

// u = unit(un x t) v1 + un, un = n val; with the fixed rules also the second
// tangential component, (n x unit(un x t)) v2
static __device__ __forceinline__ d3 refl_combine(const SysF64 &S, d3 n, double val, d3 t, double v1, double v2) {
  const d3 un = mul3s(n, val);
  const d3 ut = refl_unit(cross_ref(un, t));
  if (!S.physics) return add3(mul3s(ut, v1), un);
  return add3(add3(mul3s(ut, v1), mul3s(cross_ref(n, ut), v2)), un);
}

static __device__ d3 stochastic_reflection(const SysF64 &S, uint32_t a, uint32_t b, uint32_t t, d3 rf, d3 rs) {
  uint4 r0, r1;
  refl_blocks(S, a, b, t, r0, r1);
  const double val = refl_speed(S, r0);
  double v2;
  const double v1 = refl_gauss(S, r1, a, b, t, &v2);
  return refl_combine(S, refl_unit(rs), val, refl_point(S, r0, rf), v1, v2);
}

// ------------------------------------------------------------ particle stream

// Colloids the cell table lists for cell `lin`, visited in ascending index
// (the reference visits colloids in order, fluid_colloid_collision.cpp:30).
struct CandIter {
  const uint16_t *lst;
  int cnt, last;
  bool brute;  // aliased cell: scan all colloids with the exact block rule
  int lin;
};

static __device__ __forceinline__ int cand_next(const SysF64 &S, CandIter &it, const int *cbox) {
  if (it.brute) {
    for (int j = it.last + 1; j < S.Nc; ++j)
      if (in_block(S, cbox[j], it.lin)) { it.last = j; return j; }
    return -1;
  }
  int best = 0x7FFFFFFF;
  for (int k = 0; k < it.cnt; ++k) {
    int j = it.lst[k];
    if (j > it.last && j < best) best = j;
  }
  if (best == 0x7FFFFFFF) return -1;
  it.last = best;
  return best;
}

// Is the particle within radius r (r2 = the reference's squared threshold) of
// colloid j?  FP32 on copies first; the exact FP64 test of the reference only
// within 1e-3 of the sphere, where FP32 could decide differently (the FP32
// copies are within 2^-22 L of the doubles).
static __device__ __forceinline__ bool within(const SysF64 &S, const double *Xc, float4 c, int j, double x, double y, double z,
                                       float r, double r2) {
  const float px = d2f_trunc(x), py = d2f_trunc(y), pz = d2f_trunc(z);
  float dx = wrap_half(c.x - px, S.Lxf), dy = wrap_half(c.y - py, S.Lyf), dz = wrap_half(c.z - pz, S.Lzf);
  float d2 = dx * dx + dy * dy + dz * dz;
  float hi = r + 1e-3f, lo = r - 1e-3f;
  if (d2 > hi * hi) return false;
  if (d2 < lo * lo) return true;
  double rx = ref_img(__dsub_rn(Xc[3 * j], x), S.dx), ry = ref_img(__dsub_rn(Xc[3 * j + 1], y), S.dy),
         rz = ref_img(__dsub_rn(Xc[3 * j + 2], z), S.dz);
  return norm2_ref(rx, ry, rz) <= r2;
}

// The state of one listed particle while the event pass works on it.  It lives in
// shared memory so that any thread of the block can carry the particle's
// collisions: the collisions of a block are gathered onto its first threads (one
// warp, as a rule) because a GB300 SM takes ~64 cycles per FP64 warp instruction
// however few lanes are active; spread over every warp the FP64 bodies would queue
// on the SM's FP64 pipe.
struct EvState {
  double x, y, z, wx, wy, wz;
  double x0, y0, z0;     // position before the first collision (displacement check)
  double vdx, vdy, vdz;  // velocity when the collision routine began (dump_vel_fl)
  int p, id, lin, last;  // fluid slot, particle id, cell, last colloid the search visited
  int cnt, j;            // cell-table candidates; colloid of the next collision (-1: none)
  bool alias, dumped, changed;
};

static __device__ __forceinline__ CandIter ev_iter(const SysF64 &S, const EvState &st, int buf) {
  CandIter it;
  it.brute = st.alias;
  it.lin = st.lin;
  it.last = st.last;
  it.cnt = st.cnt;
  it.lst = S.Tlist[buf] + (size_t)st.lin * TCAP;
  return it;
}

// the next colloid, in ascending order after the last one visited, whose sphere
// holds the particle (fluid_colloid_collision.cpp:30-33), or -1
static __device__ __forceinline__ int ev_next_hit(const SysF64 &S, EvState &st, int buf) {
  const double *Xc = S.X[buf];
  const float4 *Xf = S.Xf[buf];
  CandIter it = ev_iter(S, st, buf);
  int j;
  do {
    j = cand_next(S, it, S.cbox[buf]);
  } while (j >= 0 && !within(S, Xc, Xf[j], j, st.x, st.y, st.z, S.r_coll, S.sig2q));
  st.last = it.last;
  return j;
}

// One wall collision of the particle with colloid j (fluid_colloid_collision.cpp:34-45):
// half a substep back, stochastic reflection in the colloid's frame, the exchange
// into the colloid's exact sums, half a substep forward.
static __device__ __noinline__ void ev_collide(const SysF64 &S, EvState &st, int j, long long gs, int buf) {
  const double *Xc = S.X[buf];
  const d3 Xj = mk(Xc[3 * j], Xc[3 * j + 1], Xc[3 * j + 2]);
  // issued with Xj, used after the reflection
  const d3 Vj = mk(S.V[3 * j], S.V[3 * j + 1], S.V[3 * j + 2]), Wj = mk(S.W[3 * j], S.W[3 * j + 1], S.W[3 * j + 2]);
  double x = st.x, y = st.y, z = st.z, wx = st.wx, wy = st.wy, wz = st.wz;
  if (!st.dumped) {  // dump_vel_fl: the velocity when the collision routine began
    st.vdx = __dmul_rn(wx, S.inv_dt); st.vdy = __dmul_rn(wy, S.inv_dt); st.vdz = __dmul_rn(wz, S.inv_dt);
    st.dumped = true;
  }
  // step back half a substep with the current velocity
  x = ref_mod(__dsub_rn(x, __dmul_rn(wx, 0.5)), S.dx);
  y = ref_mod(__dsub_rn(y, __dmul_rn(wy, 0.5)), S.dy);
  z = ref_mod(__dsub_rn(z, __dmul_rn(wz, 0.5)), S.dz);
  d3 rs = mk(ref_img(__dsub_rn(x, Xj.x), S.dx), ref_img(__dsub_rn(y, Xj.y), S.dy), ref_img(__dsub_rn(z, Xj.z), S.dz));
  d3 u = stochastic_reflection(S, (uint32_t)(st.id + 1), (uint32_t)(j + 1), (uint32_t)gs, mk(x, y, z), rs);
  d3 vn = add3(add3(u, Vj), cross_ref(Wj, rs));
  d3 dv = sub3(mk(st.vdx, st.vdy, st.vdz), vn);
  d3 dl = cross_ref(rs, dv);
  exch_add6(S.exch + j, dv, dl, &S.ss->err);
  wx = __dmul_rn(vn.x, S.dt); wy = __dmul_rn(vn.y, S.dt); wz = __dmul_rn(vn.z, S.dt);
  // step forward half a substep with the new velocity
  x = ref_mod(__dadd_rn(x, __dmul_rn(wx, 0.5)), S.dx);
  y = ref_mod(__dadd_rn(y, __dmul_rn(wy, 0.5)), S.dy);
  z = ref_mod(__dadd_rn(z, __dmul_rn(wz, 0.5)), S.dz);
  // the cell table is built with a margin; a move beyond it could hide a colloid
  double ex = ref_img(__dsub_rn(x, st.x0), S.dx), ey = ref_img(__dsub_rn(y, st.y0), S.dy),
         ez = ref_img(__dsub_rn(z, st.z0), S.dz);
  if (norm2_ref(ex, ey, ez) > S.disp_margin2) atomicOr(&S.ss->err, ERRB_DISPLACE);
  st.x = x; st.y = y; st.z = z; st.wx = wx; st.wy = wy; st.wz = wz;
  st.changed = true;
}

// Per-task scratch of a cooperative collision (ev_collide_coop)
struct CollScratch {
  double xb[3], rs[3], n[3], tp[3], wr[3], vd[3];
  double val, v1, v2;
};

// The same collision as ev_collide for up to 32 gathered particles at once
// (tasks k0.. of stask), by all four warps of a 128-thread block: lane t of each
// warp takes task k0 + t, and the warps, one per SM scheduler, run the
// collision's independent FP64 chains side by side (warp 0: the step back and
// the unit normal; 1: the Rayleigh speed; 2: the Gaussian; 3: t, W x rs and the
// velocity at the start of the collision routine); warp 0 then joins them.  Every
// value is the same sequence of rounded operations as in ev_collide, so the
// results are identical.  Called by every thread of the block.
static __device__ void ev_collide_coop(const SysF64 &S, EvState *sst, const int *stask, int k0, int nt, long long gs,
                                       int buf, CollScratch *cs) {
  const int w = threadIdx.x >> 5, t = threadIdx.x & 31, k = k0 + t;
  const bool act = k < nt;
  const double *Xc = S.X[buf];
  d3 Vj = mk(0, 0, 0);
  if (act) {
    const EvState &st = sst[stask[k]];
    const int j = st.j;
    const uint32_t a = (uint32_t)(st.id + 1), b = (uint32_t)(j + 1), tt = (uint32_t)gs;
    CollScratch &c = cs[t];
    if (w == 0 || w == 3) {
      // half a substep back with the current velocity, and the particle relative to the colloid
      const d3 Xj = mk(Xc[3 * j], Xc[3 * j + 1], Xc[3 * j + 2]);
      if (w == 0) Vj = mk(S.V[3 * j], S.V[3 * j + 1], S.V[3 * j + 2]);  // used after the join
      const double x = ref_mod(__dsub_rn(st.x, __dmul_rn(st.wx, 0.5)), S.dx);
      const double y = ref_mod(__dsub_rn(st.y, __dmul_rn(st.wy, 0.5)), S.dy);
      const double z = ref_mod(__dsub_rn(st.z, __dmul_rn(st.wz, 0.5)), S.dz);
      const d3 rs = mk(ref_img(__dsub_rn(x, Xj.x), S.dx), ref_img(__dsub_rn(y, Xj.y), S.dy),
                       ref_img(__dsub_rn(z, Xj.z), S.dz));
      if (w == 0) {
        c.xb[0] = x; c.xb[1] = y; c.xb[2] = z;
        c.rs[0] = rs.x; c.rs[1] = rs.y; c.rs[2] = rs.z;
        const d3 n = refl_unit(rs);
        c.n[0] = n.x; c.n[1] = n.y; c.n[2] = n.z;
      } else {
        const d3 Wj = mk(S.W[3 * j], S.W[3 * j + 1], S.W[3 * j + 2]);
        const d3 tp = refl_point(S, draw4(S.key, DOM_COLL, 0, a, b, tt), mk(x, y, z));
        const d3 wr = cross_ref(Wj, rs);
        c.tp[0] = tp.x; c.tp[1] = tp.y; c.tp[2] = tp.z;
        c.wr[0] = wr.x; c.wr[1] = wr.y; c.wr[2] = wr.z;
        // dump_vel_fl: the velocity when the collision routine began
        if (st.dumped) {
          c.vd[0] = st.vdx; c.vd[1] = st.vdy; c.vd[2] = st.vdz;
        } else {
          c.vd[0] = __dmul_rn(st.wx, S.inv_dt); c.vd[1] = __dmul_rn(st.wy, S.inv_dt); c.vd[2] = __dmul_rn(st.wz, S.inv_dt);
        }
      }
    } else if (w == 1) {
      c.val = refl_speed(S, draw4(S.key, DOM_COLL, 0, a, b, tt));
    } else {
      c.v1 = refl_gauss(S, draw4(S.key, DOM_COLL, 1, a, b, tt), a, b, tt, &c.v2);
    }
  }
  __syncthreads();
  if (w == 0 && act) {
    EvState &st = sst[stask[k]];
    const int j = st.j;
    const CollScratch &c = cs[t];
    const d3 u = refl_combine(S, mk(c.n[0], c.n[1], c.n[2]), c.val, mk(c.tp[0], c.tp[1], c.tp[2]), c.v1, c.v2);
    const d3 vn = add3(add3(u, Vj), mk(c.wr[0], c.wr[1], c.wr[2]));
    const d3 vd = mk(c.vd[0], c.vd[1], c.vd[2]);
    const d3 dv = sub3(vd, vn);
    const d3 dl = cross_ref(mk(c.rs[0], c.rs[1], c.rs[2]), dv);
    exch_add6(S.exch + j, dv, dl, &S.ss->err);
    const double wx = __dmul_rn(vn.x, S.dt), wy = __dmul_rn(vn.y, S.dt), wz = __dmul_rn(vn.z, S.dt);
    // step forward half a substep with the new velocity
    const double x = ref_mod(__dadd_rn(c.xb[0], __dmul_rn(wx, 0.5)), S.dx);
    const double y = ref_mod(__dadd_rn(c.xb[1], __dmul_rn(wy, 0.5)), S.dy);
    const double z = ref_mod(__dadd_rn(c.xb[2], __dmul_rn(wz, 0.5)), S.dz);
    // the cell table is built with a margin; a move beyond it could hide a colloid
    const double ex = ref_img(__dsub_rn(x, st.x0), S.dx), ey = ref_img(__dsub_rn(y, st.y0), S.dy),
                 ez = ref_img(__dsub_rn(z, st.z0), S.dz);
    if (norm2_ref(ex, ey, ez) > S.disp_margin2) atomicOr(&S.ss->err, ERRB_DISPLACE);
    st.x = x; st.y = y; st.z = z; st.wx = wx; st.wy = wy; st.wz = wz;
    st.vdx = vd.x; st.vdy = vd.y; st.vdz = vd.z;
    st.dumped = true;
    st.changed = true;
  }
  __syncthreads();
}

// run() candidate record of the particle at its final position: the colloids, in
// ascending order, whose rear-shell sphere holds it
static __device__ __forceinline__ void ev_shell(const SysF64 &S, const EvState &st, int buf, ShellRec &rec) {
  const double *Xc = S.X[buf];
  const float4 *Xf = S.Xf[buf];
  CandIter it = ev_iter(S, st, buf);
  it.last = -1;
  rec.p = st.id;
  rec.n = 0;
  rec.pass = 0;
  for (int j = cand_next(S, it, S.cbox[buf]); j >= 0; j = cand_next(S, it, S.cbox[buf])) {
    if (!within(S, Xc, Xf[j], j, st.x, st.y, st.z, S.r_shell, S.rsh2)) continue;
    if (rec.n < SHELL_J) rec.j[rec.n++] = (uint16_t)j;
    else atomicOr(&S.ss->err, ERRB_SHELLSLOTS);
  }
}

// |w|^2 * 2^kw from the fixed-point w = wf 2^-kw: wf^2 2^-kw, rounded half up,
// as a 128-bit square on the integer pipe
static __device__ __forceinline__ long long sq_fix(long long wf, int kw) {
  unsigned long long a = (unsigned long long)(wf < 0 ? -wf : wf);
  unsigned long long lo = a * a, hi = __umul64hi(a, a);
  unsigned long long lo2 = lo + (1ull << (kw - 1));
  hi += lo2 < lo;
  return (long long)((hi << (64 - kw)) | (lo2 >> kw));
}

// ------------------------------------------------------------- colloid helpers

static __device__ __forceinline__ d3 ldv(const double *a, int j) { return mk(a[3 * j], a[3 * j + 1], a[3 * j + 2]); }
static __device__ __forceinline__ void stv(double *a, int j, d3 v) { a[3 * j] = v.x; a[3 * j + 1] = v.y; a[3 * j + 2] = v.z; }

// update_activity_direction (cpp/update.cpp:34-46): ra rotated by the Euler matrix
// of Omega dt; then, with Dr > 0, rotational diffusion ra += sqrt(2 Dr dt)
// (xi - (xi.ra) ra), renormalised (xi: three normals drawn for that substep)
// (sb, cb: the sines and cosines of the components of Omega dt)
static __device__ d3 activity_rot(const SysF64 &S, d3 ra, d3 sb, d3 cb, d3 xi) {
  d3 m1 = mk(__dmul_rn(cb.y, cb.z), __dmul_rn(-cb.y, sb.z), sb.y);
  d3 m2 = mk(__dadd_rn(__dmul_rn(__dmul_rn(sb.x, sb.y), cb.z), __dmul_rn(cb.x, sb.z)),
             __dadd_rn(__dmul_rn(__dmul_rn(-sb.x, sb.y), sb.z), __dmul_rn(cb.x, cb.z)), __dmul_rn(-sb.x, cb.y));
  d3 m3 = mk(__dadd_rn(__dmul_rn(__dmul_rn(-cb.x, sb.y), cb.z), __dmul_rn(sb.x, sb.z)),
             __dadd_rn(__dmul_rn(__dmul_rn(cb.x, sb.y), sb.z), __dmul_rn(sb.x, cb.z)), __dmul_rn(cb.x, cb.y));
  ra = mk(dot_ref(m1, ra), dot_ref(m2, ra), dot_ref(m3, ra));
  if (S.Dr > 0) {
    double xa = dot_ref(xi, ra);
    d3 dn = sub3(xi, mul3s(ra, xa));
    d3 a = add3(ra, mul3s(dn, S.rotdiff_s));
    ra = div3s(a, __dsqrt_rn(norm2_ref(a.x, a.y, a.z)));
  }
  return ra;
}

// sin x and cos x: for |x| < 2^-6 (the Euler angles Omega dt of a substep) by their
// Maclaurin series in Horner form, whose first omitted terms x^9/9! and x^10/10! are below
// 1e-21, so the results are within a few ulp; else sincos
static __device__ __forceinline__ void sincos_small(double x, double *s, double *c) {
  if (fabs(x) < 0.015625) {
    const double x2 = x * x;
    *s = x * (1.0 - x2 * (1.0 / 6.0) * (1.0 - x2 * (1.0 / 20.0) * (1.0 - x2 * (1.0 / 42.0))));
    *c = 1.0 - x2 * 0.5 * (1.0 - x2 * (1.0 / 12.0) * (1.0 - x2 * (1.0 / 30.0) * (1.0 - x2 * (1.0 / 56.0))));
  } else {
    sincos(x, s, c);
  }
}

static __device__ d3 activity(const SysF64 &S, d3 ra, d3 W, d3 xi) {
  d3 b = mul3s(W, S.dt), sb, cb;
  sincos_small(b.x, &sb.x, &cb.x);
  sincos_small(b.y, &sb.y, &cb.y);
  sincos_small(b.z, &sb.z, &cb.z);
  return activity_rot(S, ra, sb, cb, xi);
}

static __device__ __forceinline__ float wrapf(float d, float L) { return d - L * rintf(d / L); }
// the same with a reciprocal of L (for prefilters that carry a margin)
static __device__ __forceinline__ float wrapf_r(float d, float L, float iL) { return d - L * rintf(d * iL); }

// One pair term of compute_force_md (cpp/update.cpp:21-28) in the reference's FP64
// expression order: with temp = img(X_j - X_k) and r = |temp| < r_cutoff, the force
// on j from k (ff) and, with want_pot, the pair's potential (pt).  Returns whether
// the pair is inside the cutoff.
static __device__ __forceinline__ bool wca_pair(const SysF64 &S, d3 Xj, const double *Xc, int k, bool want_pot,
                                                d3 &ff, double &pt) {
  d3 temp = mk(ref_img(__dsub_rn(Xj.x, Xc[3 * k]), S.dx), ref_img(__dsub_rn(Xj.y, Xc[3 * k + 1]), S.dy),
               ref_img(__dsub_rn(Xj.z, Xc[3 * k + 2]), S.dz));
  double r = __dsqrt_rn(norm2_ref(temp.x, temp.y, temp.z));
  if (!(r < S.r_cutoff)) return false;
  double p13 = r, p7 = r;
  for (int i = 1; i < 13; ++i) { p13 = __dmul_rn(p13, r); if (i == 6) p7 = p13; }
  double t1 = __ddiv_rn(S.sig12, p13), t2 = __ddiv_rn(S.sig6, p7);
  double mag = __dsub_rn(__dmul_rn(__dmul_rn(4.0, S.eps), __dsub_rn(__dmul_rn(12.0, t1), __dmul_rn(6.0, t2))), S.fc);
  ff = div3s(mul3s(temp, mag), r);
  if (want_pot) {
    double q = __ddiv_rn(S.sig_colloid, r);
    pt = __dadd_rn(__dsub_rn(__dmul_rn(__dmul_rn(4.0, S.eps), __dsub_rn(pow(q, 12.0), pow(q, 6.0))), S.ufc),
                   __dmul_rn(S.fc, r));
  }
  return true;
}

// Adds the pair terms of the lanes that hit, in lane order, to f and pot (every
// lane ends with the same sums).
static __device__ __forceinline__ void wca_gather(bool hit, d3 ff, double pt, d3 &f, double &pot) {
  unsigned hm = __ballot_sync(FULL, hit);
  while (hm) {
    int src = __ffs(hm) - 1;
    hm &= hm - 1;
    double fx = __shfl_sync(FULL, ff.x, src), fy = __shfl_sync(FULL, ff.y, src), fz = __shfl_sync(FULL, ff.z, src);
    double pp = __shfl_sync(FULL, pt, src);
    f = add3(f, mk(fx, fy, fz));
    pot = __dadd_rn(pot, pp);
  }
}

// WCA force on colloid j at positions Xc (compute_force_md, cpp/update.cpp:14-32):
// partners with r < r_cutoff summed in ascending partner order, which is the
// order the reference's pair loop adds them to f[j].  FP32 prefilter over all
// colloids by the warp; exact FP64 pair terms.  Returns the force in every lane;
// pot receives this colloid's share of the potential (pairs with k > j).
static __device__ d3 wca_force(const SysF64 &S, const double *Xc, const float4 *Xf, int j, int lane, bool want_pot,
                        double &pot) {
  d3 f = mk(0, 0, 0);
  pot = 0;
  const float4 xj = Xf[j];
  const float Lx = S.Lxf, Ly = S.Lyf, Lz = S.Lzf;
  const float iLx = __frcp_rn(Lx), iLy = __frcp_rn(Ly), iLz = __frcp_rn(Lz);
  const float rcf = S.rcf;
  const d3 Xj = ldv(Xc, j);
  const int nit = (S.Nc + 31) / 32;
  for (int c0 = 0; c0 < nit; c0 += 32) {
    const int cend = min(nit, c0 + 32);
    // FP32 prefilter of up to 1024 partners: independent loads, one bit per pass
    unsigned mine = 0;
#pragma unroll 4
    for (int it = c0; it < cend; ++it) {
      const int k = it * 32 + lane;
      if (k < S.Nc && k != j) {
        const float4 xk = Xf[k];
        const float dx = wrapf_r(xj.x - xk.x, Lx, iLx), dy = wrapf_r(xj.y - xk.y, Ly, iLy),
                    dz = wrapf_r(xj.z - xk.z, Lz, iLz);
        if (dx * dx + dy * dy + dz * dz < rcf * rcf) mine |= 1u << (it - c0);
      }
    }
    for (int it = c0; it < cend; ++it) {
      const int k = it * 32 + lane;
      const bool cand = (mine >> (it - c0)) & 1u;
      unsigned m = __ballot_sync(FULL, cand);
      if (!m) continue;
      d3 ff = mk(0, 0, 0);
      double pt = 0;
      const bool hit = cand && wca_pair(S, Xj, Xc, k, want_pot && k > j, ff, pt);
      wca_gather(hit, ff, pt, f, pot);
    }
  }
  return f;
}

// The same sum with the FP32 prefilter over colloid j's pair list instead of over every
// colloid: the list holds (ascending) every colloid within r_cutoff plus twice the
// colloids' largest move in the step of j at the start of the step, so it holds every
// partner the scan of all colloids finds, and the same partners are summed in the same
// order.
static __device__ d3 wca_force_vlist(const SysF64 &S, const double *Xc, const float4 *Xf, int j, int lane) {
  d3 f = mk(0, 0, 0);
  double pot = 0;
  const float4 xj = Xf[j];
  const float Lx = S.Lxf, Ly = S.Lyf, Lz = S.Lzf;
  const float iLx = __frcp_rn(Lx), iLy = __frcp_rn(Ly), iLz = __frcp_rn(Lz);
  const float rcf = S.rcf;
  const d3 Xj = ldv(Xc, j);
  const int n = min(S.nbr_n[j], NBR_CAP);
  const uint16_t *lst = S.nbr + (size_t)j * NBR_CAP;
  for (int base = 0; base < n; base += 32) {
    const int i = base + lane;
    int k = 0;
    bool cand = false;
    if (i < n) {
      k = lst[i];
      const float4 xk = Xf[k];
      const float dx = wrapf_r(xj.x - xk.x, Lx, iLx), dy = wrapf_r(xj.y - xk.y, Ly, iLy),
                  dz = wrapf_r(xj.z - xk.z, Lz, iLz);
      cand = dx * dx + dy * dy + dz * dz < rcf * rcf;
    }
    if (!__ballot_sync(FULL, cand)) continue;
    d3 ff = mk(0, 0, 0);
    double pt = 0;
    const bool hit = cand && wca_pair(S, Xj, Xc, k, false, ff, pt);
    wca_gather(hit, ff, pt, f, pot);
  }
  return f;
}

// The same sum over colloid j's pair list (neighbour_list_md: its partners within the
// list radius, both below and above j, in ascending order), one partner per lane.
static __device__ d3 wca_force_list(const SysF64 &S, const double *Xc, int j, int lane, bool want_pot, double &pot) {
  d3 f = mk(0, 0, 0);
  pot = 0;
  const d3 Xj = ldv(Xc, j);
  const int n = min(S.nbr_n[j], NBR_CAP);
  const uint16_t *lst = S.nbr + (size_t)j * NBR_CAP;
  for (int base = 0; base < n; base += 32) {
    const int i = base + lane;
    d3 ff = mk(0, 0, 0);
    double pt = 0;
    bool hit = false;
    if (i < n) {
      const int k = lst[i];
      hit = wca_pair(S, Xj, Xc, k, want_pot && k > j, ff, pt);
    }
    wca_gather(hit, ff, pt, f, pot);
  }
  return f;
}

// Cells of the 342-box block of colloid cell cb (own box excluded) whose box
// comes within `reach` of the colloid position (minimum image, FP32 with margin):
// the cells whose particles can be inside the sphere or the run() shell.
template <typename F>
static __device__ void for_reach_cells(const SysF64 &S, int cb, float4 xc, float reach, int first, int stride, F fn) {
  if (cb >= S.C) return;
  int cx = cb % S.Lx, ct = cb / S.Lx, cy = ct % S.Ly, cz = ct / S.Ly;
  const float Lx = S.Lxf, Ly = S.Lyf, Lz = S.Lzf;
  const float iLx = __frcp_rn(Lx), iLy = __frcp_rn(Ly), iLz = __frcp_rn(Lz);
  for (int q = first; q < 343; q += stride) {
    int ox = q % 7 - 3, oy = (q / 7) % 7 - 3, oz = q / 49 - 3;
    if (!ox && !oy && !oz && !S.physics) continue;  // the own box (kept by the fixed rules)
    int bx = cx + ox, by = cy + oy, bz = cz + oz;
    bx += bx < 0 ? S.Lx : 0; bx -= bx >= S.Lx ? S.Lx : 0;
    by += by < 0 ? S.Ly : 0; by -= by >= S.Ly ? S.Ly : 0;
    bz += bz < 0 ? S.Lz : 0; bz -= bz >= S.Lz ? S.Lz : 0;
    float ex = fmaxf(fabsf(wrapf_r(xc.x - ((float)bx + 0.5f), Lx, iLx)) - 0.5f, 0.f);
    float ey = fmaxf(fabsf(wrapf_r(xc.y - ((float)by + 0.5f), Ly, iLy)) - 0.5f, 0.f);
    float ez = fmaxf(fabsf(wrapf_r(xc.z - ((float)bz + 0.5f), Lz, iLz)) - 0.5f, 0.f);
    if (ex * ex + ey * ey + ez * ez <= reach * reach) fn(bx + S.Lx * (by + S.Ly * bz));
  }
}

// grid shift of the SRD binning of step nn (rotation_mpcd draws it first,
// cpp/rotation_mpcd.cpp:9), keyed by that step: each component a uniform minus 1/2
static __device__ __forceinline__ void shift_of(const SysF64 &S, long long nn, double rr[3]) {
  const uint4 r = draw4(S.key, DOM_SHIFT, 0, 0, 0, (uint32_t)nn);
  rr[0] = u01(r.x) - 0.5; rr[1] = u01(r.y) - 0.5; rr[2] = u01(r.z) - 0.5;
}

// reach of the cell table of substep e: the run() shell on the last substep of a
// step (its candidates are recorded there), the sphere otherwise
static __device__ __forceinline__ float table_reach(const SysF64 &S, long long e) {
  return (e % S.n_sub) == S.n_sub - 1 ? S.rT_shell : S.rT_coll;
}

// update_activity_direction (cpp/update.cpp:34-46) of colloid j on lanes k = 0-2 of
// group grp: lane k takes sin and cos of (Omega dt)_k, all three gather them, lane 0
// stores the turned orientation (with the rotational-diffusion normals S.xi[j])
static __device__ __forceinline__ void activity_apply(const SysF64 &S, int j, int k, unsigned grp) {
  double s, co;
  sincos_small(__dmul_rn(S.W[3 * j + k], S.dt), &s, &co);
  const d3 sb = mk(__shfl_sync(grp, s, 0), __shfl_sync(grp, s, 1), __shfl_sync(grp, s, 2));
  const d3 cb = mk(__shfl_sync(grp, co, 0), __shfl_sync(grp, co, 1), __shfl_sync(grp, co, 2));
  const d3 rn = activity_rot(S, ldv(S.ra, j), sb, cb, ldv(S.xi, j));
  if (k == 0) stv(S.ra, j, rn);
}

// the three standard normals of substep g's rotational diffusion of colloid j
// (Box-Muller) into S.xi[j], on lanes k = 0-2 of group grp: lane 0 the pair (r0, t0)
// giving xi_x and xi_y, lane 1 the pair (r1, t1) giving xi_z
static __device__ __forceinline__ void rotdiff_draw(const SysF64 &S, long long g, int j, int k, unsigned grp) {
  uint4 r = draw4(S.key, DOM_ROTDIFF, 0, (uint32_t)(j + 1), 0, (uint32_t)g);
  const uint32_t ur = k == 0 ? r.x : r.z, ut = k == 0 ? r.y : r.w;
  double rr = 0, sn = 0, cs = 0;
  if (k < 2) {
    rr = sqrt(-2.0 * log(u01(ur)));
    sincos(__dmul_rn(S.two_pi, u01(ut)), &sn, &cs);
  }
  const double r0 = __shfl_sync(grp, rr, 0), s0 = __shfl_sync(grp, sn, 0), c0 = __shfl_sync(grp, cs, 0);
  const double r1 = __shfl_sync(grp, rr, 1), c1 = __shfl_sync(grp, cs, 1);
  if (k == 0) stv(S.xi, j, mk(__dmul_rn(r0, c0), __dmul_rn(r0, s0), __dmul_rn(r1, c1)));
}

// Colloid work that the next substep needs and nothing in this substep changes
// (k_aux, on a second stream beside the streaming and event passes of this
// substep): the WCA forces at the positions X_g (compute_force_md) and the cell
// table of substep g+1, built from X_g with a margin for the colloid's own move.
// (vlist: the forces from the pair list the free-flight schedule builds at the start of
// each step.)  The colloid has `nw` (2 to 8) warps and `w` is this thread's warp among them:
// the forces on warp 0, the table on warps 2.. (on warp 0 after the forces when
// nw = 2); the pending orientation update and this substep's
// rotational-diffusion draws on warp 1, whose lanes 0-2 take one component each.
static __device__ __noinline__ void colloid_aux(const SysF64 &S, long long g, int j, bool act, int w, int nw,
                                                bool vlist = false) {
  const int b = (int)(g & 1);
  const int lane = threadIdx.x & 31;
  if (w == 0) {
    double pot;
    d3 fn = vlist ? wca_force_vlist(S, S.X[b], S.Xf[b], j, lane) : wca_force(S, S.X[b], S.Xf[b], j, lane, false, pot);
    if (lane == 0) stv(S.fnew, j, fn);
  }
  if (!S.fin_table && (w >= 2 || (w == 0 && nw == 2))) {
    const long long e = g + 1;
    unsigned long long *Tc = S.Tcnt[e & 1];
    uint16_t *Tl = S.Tlist[e & 1];
    int *err = &S.ss->err;
    const int first = nw == 2 ? lane : (w - 2) * 32 + lane, stride = nw == 2 ? 32 : (nw - 2) * 32;
    for_reach_cells(S, S.cbox[b][j], S.Xf[b][j], table_reach(S, e), first, stride,
                    [&](int cell) { tappend(Tc, Tl, cell, e, j, err); });
  }
  if (w != 1 || lane >= 3) return;
  const unsigned grp = 0x7u;
  // update_activity_direction of the previous substep (nothing before the end of
  // this step reads the orientation), with the normals that substep drew
  if (act) activity_apply(S, j, lane, grp);
  if (S.Dr > 0) {
    __syncwarp(grp);
    rotdiff_draw(S, g, j, lane, grp);
  }
}

}  // namespace bgb
