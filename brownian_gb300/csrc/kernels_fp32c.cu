// FP32-compensated form of the MPCD + active-colloid step (sm_103a).
//
// The fluid is stored per particle as one 16-byte record {packed cell, offset x,
// offset y, offset z} (a single 128-bit load) plus FP32 velocities: 28 bytes where
// the FP64 form keeps 48, and all fluid arithmetic runs on the FP32 pipe.  A
// position is its integer cell plus an FP32 offset in [0, 1), so it is resolved to
// 2^-24 of a cell everywhere in the box, and a particle-colloid distance is an
// exact integer cell difference plus an FP32 offset difference.  What stays in
// FP64 / exact: the colloids (shared with the FP64 form), the per-cell sums
// (exact fixed-point integers, so the cell momentum is summed without rounding),
// the thermostat factor of each cell, the colloid momentum exchange (exact
// fixed-point) and every diagnostic.
//
// Kernels mirror the FP64 form: k_stream32 (stream, FP32 scan of nearby colloids,
// event list, last-substep binning), k_events32 (wall collisions in FP32, one per
// lane), k_cell_prep32, k_rotate32 / k_rotate_sort32, k_run_shell32 / k_run_kick32.
#include "device.cuh"

namespace bgb {

__device__ __forceinline__ void unpack(uint4 r, int &cx, int &cy, int &cz, float &ox, float &oy, float &oz) {
  cx = (int)(r.x & 1023u); cy = (int)((r.x >> 10) & 1023u); cz = (int)((r.x >> 20) & 1023u);
  ox = __uint_as_float(r.y); oy = __uint_as_float(r.z); oz = __uint_as_float(r.w);
}

__device__ __forceinline__ uint4 pack(int cx, int cy, int cz, float ox, float oy, float oz) {
  return make_uint4((unsigned)cx | ((unsigned)cy << 10) | ((unsigned)cz << 20), __float_as_uint(ox),
                    __float_as_uint(oy), __float_as_uint(oz));
}

// the SRD collision of one particle: v' = A v + b, the cell's FP32 affine map (A row-major, b)
__device__ __forceinline__ void apply_map32(const float *ab, float &vx, float &vy, float &vz) {
  const float4 *m = reinterpret_cast<const float4 *>(ab);
  float4 a = m[0], b = m[1], c = m[2];
  float nx = fmaf(a.x, vx, fmaf(a.y, vy, fmaf(a.z, vz, c.y)));
  float ny = fmaf(a.w, vx, fmaf(b.x, vy, fmaf(b.y, vz, c.z)));
  float nz = fmaf(b.z, vx, fmaf(b.w, vy, fmaf(c.x, vz, c.w)));
  vx = nx; vy = ny; vz = nz;
}

// keep the offset in [0, 1), carrying whole cells into the periodic cell index
__device__ __forceinline__ void carry(int &c, float &o, int L) {
  if (o >= 0.f && o < 1.f) return;
  float f = floorf(o);
  o -= f;
  if (o >= 1.f) { o = 0.f; f += 1.f; }
  if (!(f == f) || fabsf(f) > 1e6f) { o = 0.f; f = 0.f; }  // NaN / runaway: stays put (flagged by the range test)
  c += (int)f;
  c %= L;
  if (c < 0) c += L;
}

// particle minus colloid along one axis, minimum image: integer cell difference
// (exact) plus offset difference
__device__ __forceinline__ float rel(int c, float o, float cq, float co, int L) {
  int d = c - (int)cq;
  if (d > (L >> 1)) d -= L;
  else if (d < -(L >> 1)) d += L;
  return (float)d + (o - co);
}

// uniform in (0,1) from the top 23 bits: (k + 1/2) 2^-23 is exact in FP32, so the
// value is never 0 or 1 (with 24 bits the top value would round to 1 and a
// reflection would take log(0))
__device__ __forceinline__ float u01f(uint32_t w) { return ((float)(w >> 9) + 0.5f) * 1.1920928955078125e-7f; }

// round(v * 2^k) of an FP32 value from its bits (exact when the scale covers the
// value's last bit)
__device__ __forceinline__ long long to_fix_f(float v, int k) {
  unsigned b = __float_as_uint(v);
  int e = (int)((b >> 23) & 0xFF);
  if (e == 0) return 0;
  long long m = (long long)((b & 0x7FFFFFu) | 0x800000u);
  int sh = e - 150 + k;
  long long r;
  if (sh >= 0) r = m << (sh < 62 ? sh : 62);
  else if (sh > -40) {
    int s = -sh;
    r = m >> s;
    long long rem = m & ((1ll << s) - 1), half = 1ll << (s - 1);
    if (rem > half || (rem == half && (r & 1))) r += 1;
  } else r = 0;
  return (b >> 31) ? -r : r;
}

// one particle's part of the SRD binning for the next step (rotation_mpcd bins by the
// shifted position: cell + floor(offset + rr) per axis): its cell (recorded in rotcell)
// and the fixed-point v and |v|^2 the exact cell sums add up
struct BinTerm32 {
  int c;
  long long fx, fy, fz, f2;
};

// round(v^2 2^k) from the significand m of v (24 bits, so m^2 is exact in 64 bits):
// v^2 2^k = m^2 2^(2 (e - 150) + k); the same value as sq_fix of to_fix_f(v, k) whenever
// v 2^k is an integer (every |v| >= 2^(23 - k)), and within one unit below that
__device__ __forceinline__ long long sq_fix_f(float v, int k) {
  const unsigned b = __float_as_uint(v);
  const int e = (int)((b >> 23) & 0xFF);
  if (e == 0) return 0;
  const unsigned m = (b & 0x7FFFFFu) | 0x800000u;
  const unsigned long long q = (unsigned long long)m * m;
  const int sh = 2 * (e - 150) + k;
  if (sh >= 0) return (long long)(q << (sh < 16 ? sh : 16));
  if (sh <= -63) return 0;
  const int s = -sh;
  unsigned long long r = q >> s;
  const unsigned long long rem = q & ((1ull << s) - 1ull), half = 1ull << (s - 1);
  if (rem > half || (rem == half && (r & 1ull))) r += 1ull;
  return (long long)r;
}

__device__ __forceinline__ BinTerm32 bin32_term(const SysF64 &S, const float *rr, int p, int cx, int cy, int cz,
                                                float ox, float oy, float oz, float vx, float vy, float vz) {
  float tx = ox + rr[0], ty = oy + rr[1], tz = oz + rr[2];
  int bx = cx + (tx < 0.f ? -1 : (tx >= 1.f ? 1 : 0));
  int by = cy + (ty < 0.f ? -1 : (ty >= 1.f ? 1 : 0));
  int bz = cz + (tz < 0.f ? -1 : (tz >= 1.f ? 1 : 0));
  bx += bx < 0 ? S.Lx : 0; bx -= bx >= S.Lx ? S.Lx : 0;
  by += by < 0 ? S.Ly : 0; by -= by >= S.Ly ? S.Ly : 0;
  bz += bz < 0 ? S.Lz : 0; bz -= bz >= S.Lz ? S.Lz : 0;
  const int c = bx + S.Lx * (by + S.Ly * bz);
  S.rotcell[p] = c;
  if (!(fabsf(vx) <= S.vmaxf && fabsf(vy) <= S.vmaxf && fabsf(vz) <= S.vmaxf)) atomicOr(&S.ss->err, ERRB_VRANGE);
  BinTerm32 t;
  t.c = c;
  t.fx = to_fix_f(vx, S.kw); t.fy = to_fix_f(vy, S.kw); t.fz = to_fix_f(vz, S.kw);
  t.f2 = sq_fix_f(vx, S.kw) + sq_fix_f(vy, S.kw) + sq_fix_f(vz, S.kw);
  return t;
}

__device__ __forceinline__ void bin32(const SysF64 &S, int p, int cx, int cy, int cz, float ox, float oy, float oz,
                                      float vx, float vy, float vz) {
  const BinTerm32 t = bin32_term(S, S.ss->rrf, p, cx, cy, cz, ox, oy, oz, vx, vy, vz);
  bin_add(S.acc + t.c, 1, t.fx, t.fy, t.fz, t.f2);
}

struct f3 { float x, y, z; };
__device__ __forceinline__ f3 fm(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ f3 fcross(f3 a, f3 b) { return fm(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }

// stochastic_reflection (cpp/fluid_colloid_collision.cpp:7-24) in FP32 with the
// same keyed draws as the FP64 form: Rayleigh normal speed along rs plus one
// Gaussian tangential component along unit(un x t)
__device__ f3 reflect32(const SysF64 &S, uint32_t a, uint32_t b, uint32_t t, f3 rf, f3 rs) {
  int idx = 0;
  uint4 buf = make_uint4(0, 0, 0, 0);
  auto next = [&]() {
    int s = idx & 3;
    if (s == 0) buf = draw4(S.key, DOM_COLL, (uint32_t)(idx >> 2), a, b, t);
    idx++;
    uint32_t w = s == 0 ? buf.x : s == 1 ? buf.y : s == 2 ? buf.z : buf.w;
    return u01f(w);
  };
  float u = next();
  float om = 1.f - u;
  float val = sqrtf(-logf(om * om) * (float)S.inv_m_beta);
  float ir = rsqrtf(rs.x * rs.x + rs.y * rs.y + rs.z * rs.z);
  f3 un = fm(rs.x * ir * val, rs.y * ir * val, rs.z * ir * val);
  float t0 = next(), t1 = next(), t2 = next();
  f3 tt = fm(t0 * S.Lxf - rf.x, t1 * S.Lyf - rf.y, t2 * S.Lzf - rf.z);
  tt.x -= S.Lxf * rintf(tt.x / S.Lxf); tt.y -= S.Lyf * rintf(tt.y / S.Lyf); tt.z -= S.Lzf * rintf(tt.z / S.Lzf);
  f3 ut = fcross(un, tt);
  float iu = rsqrtf(ut.x * ut.x + ut.y * ut.y + ut.z * ut.z);
  float x1 = 0.f, x2 = 0.f, z = 2.f;
  for (int it = 0; z > 1.f && it < 256; ++it) {
    x1 = 2.f * next() - 1.f;
    x2 = 2.f * next() - 1.f;
    z = x1 * x1 + x2 * x2;
  }
  z = sqrtf(-2.f * logf(z) / z);
  float v1 = x1 * z * (float)S.sqrt_kt_m;
  f3 res = fm(ut.x * iu * v1 + un.x, ut.y * iu * v1 + un.y, ut.z * iu * v1 + un.z);
  if (S.physics) {  // the fixed rules: the second tangential component along n x unit(ut)
    const float v2 = x2 * z * (float)S.sqrt_kt_m;
    const f3 t2 = fcross(fm(rs.x * ir, rs.y * ir, rs.z * ir), fm(ut.x * iu, ut.y * iu, ut.z * iu));
    res = fm(res.x + t2.x * v2, res.y + t2.y * v2, res.z + t2.z * v2);
  }
  return res;
}

// One warp's wall collisions (cpp/fluid_colloid_collision.cpp:26-49) of the particles its
// lanes hold (act: the lane has one): each lane takes its colloids in ascending order, the
// ones whose sphere holds the particle, and the body of a collision (back half a substep,
// the FP32 stochastic reflection, the exact exchange sums, forward half a substep) runs
// once for all lanes that hit a colloid at that rank.  The whole warp calls it.
template <int FLAGS>
__device__ __forceinline__ void collide32_warp(const SysF64 &S, long long gs, int buf, bool act, int id, int cnt,
                                               const uint16_t *lst, int &cx, int &cy, int &cz, float &ox, float &oy,
                                               float &oz, float &vx, float &vy, float &vz) {
  const float4 *Xq = S.Xcq[buf], *Xo = S.Xco[buf];
  const float rc2 = S.r_coll * S.r_coll;
  const f3 vdump = fm(vx, vy, vz);
  bool more = act;
  int last = -1;
  while (__any_sync(FULL, more)) {
    int j = 0x7FFFFFFF;
    float4 cq = make_float4(0.f, 0.f, 0.f, 0.f), co = cq;
    if (more) {
      for (;;) {
        j = 0x7FFFFFFF;
        for (int k = 0; k < cnt; ++k) {
          int c = lst[k];
          if (c > last && c < j) j = c;
        }
        if (j == 0x7FFFFFFF) break;
        last = j;
        cq = Xq[j]; co = Xo[j];
        f3 r = fm(rel(cx, ox, cq.x, co.x, S.Lx), rel(cy, oy, cq.y, co.y, S.Ly), rel(cz, oz, cq.z, co.z, S.Lz));
        if (r.x * r.x + r.y * r.y + r.z * r.z <= rc2) break;
      }
      more = j != 0x7FFFFFFF;
    }
    __syncwarp();
    if (j == 0x7FFFFFFF) continue;
    // back half a substep, reflect, forward half a substep
    ox -= 0.5f * vx * S.dtf; oy -= 0.5f * vy * S.dtf; oz -= 0.5f * vz * S.dtf;
    carry(cx, ox, S.Lx); carry(cy, oy, S.Ly); carry(cz, oz, S.Lz);
    f3 rs = fm(rel(cx, ox, cq.x, co.x, S.Lx), rel(cy, oy, cq.y, co.y, S.Ly), rel(cz, oz, cq.z, co.z, S.Lz));
    f3 rf = fm((float)cx + ox, (float)cy + oy, (float)cz + oz);
    f3 u = reflect32(S, (uint32_t)(id + 1), (uint32_t)(j + 1), (uint32_t)gs, rf, rs);
    f3 V = fm((float)S.V[3 * j], (float)S.V[3 * j + 1], (float)S.V[3 * j + 2]);
    f3 W = fm((float)S.W[3 * j], (float)S.W[3 * j + 1], (float)S.W[3 * j + 2]);
    f3 wr = fcross(W, rs);
    vx = u.x + V.x + wr.x; vy = u.y + V.y + wr.y; vz = u.z + V.z + wr.z;
    f3 dv = fm(vdump.x - vx, vdump.y - vy, vdump.z - vz);
    f3 dl = fcross(rs, dv);
    exch_add6(S.exch + j, mk(dv.x, dv.y, dv.z), mk(dl.x, dl.y, dl.z), &S.ss->err);
    ox += 0.5f * vx * S.dtf; oy += 0.5f * vy * S.dtf; oz += 0.5f * vz * S.dtf;
    carry(cx, ox, S.Lx); carry(cy, oy, S.Ly); carry(cz, oz, S.Lz);
  }
}

// A particle after its wall collisions: the displacement check against the cell-table
// margin, on the last substep its run() record and its binning (from its state after
// the collisions), and its state written back.
template <int FLAGS>
__device__ __forceinline__ void finish32(const SysF64 &S, const Fluid32 &F, int p, int id, int buf, int cnt,
                                         const uint16_t *lst, int cx0, int cy0, int cz0, float ox0, float oy0,
                                         float oz0, int cx, int cy, int cz, float ox, float oy, float oz, float vx,
                                         float vy, float vz) {
  constexpr int flags = FLAGS;
  {
    // the cell table is built with a margin; a move beyond it could hide a colloid
    const float ex = rel(cx, ox, (float)cx0, ox0, S.Lx), ey = rel(cy, oy, (float)cy0, oy0, S.Ly),
                ez = rel(cz, oz, (float)cz0, oz0, S.Lz);
    if (ex * ex + ey * ey + ez * ez > (float)S.disp_margin2) atomicOr(&S.ss->err, ERRB_DISPLACE);
  }
  if (flags & F_SHELL) {
    const float4 *Xq = S.Xcq[buf], *Xo = S.Xco[buf];
    const float rs2 = S.r_shell * S.r_shell;
    ShellRec rec;
    rec.p = id;
    rec.n = 0;
    rec.pass = 0;
    for (int last = -1; rec.n < SHELL_J;) {
      int j = 0x7FFFFFFF;
      for (int k = 0; k < cnt; ++k) {
        int c = lst[k];
        if (c > last && c < j) j = c;
      }
      if (j == 0x7FFFFFFF) break;
      last = j;
      float4 cq = Xq[j], co = Xo[j];
      float dx = rel(cx, ox, cq.x, co.x, S.Lx), dy = rel(cy, oy, cq.y, co.y, S.Ly), dz = rel(cz, oz, cq.z, co.z, S.Lz);
      if (dx * dx + dy * dy + dz * dz <= rs2) rec.j[rec.n++] = (uint16_t)j;
    }
    if (rec.n) {
      int idx = atomicAdd(&S.ss->nshell, 1);
      if (idx < S.shell_cap) S.shell[idx] = rec;
      else atomicOr(&S.ss->err, ERRB_SHELL);
    }
  }
  if (flags & F_BINROT) bin32(S, p, cx, cy, cz, ox, oy, oz, vx, vy, vz);
  F.q[p] = pack(cx, cy, cz, ox, oy, oz);
  F.vx[p] = vx; F.vy[p] = vy; F.vz[p] = vz;
}

// STREAM32_U particles per thread (thread t of block b: particles b * 256 U + t +
// 256 u), their loads issued together so more memory requests are in flight
#ifndef STREAM32_U
#define STREAM32_U 2
#endif
// the pass that also records run() candidates and bins keeps one particle per thread
// (its register count, and so its occupancy)
#ifndef STREAM32_U_SHELL
#define STREAM32_U_SHELL 1
#endif
static constexpr __host__ __device__ int stream32_u(int flags) { return (flags & F_SHELL) ? STREAM32_U_SHELL : STREAM32_U; }
// One chunk of 256 U particles: the particles i = chunk * 256 U + threadIdx.x + 256 u
// below `count` of the fluid (NEAR false: slot i) or of the near list (NEAR true: slot
// near[i], the free-flight schedule's per-substep passes).  The whole block calls it.
template <int FLAGS, bool NEAR>
static __device__ __forceinline__ void stream32_chunk(const SysF64 &S, const int chunk, const int count, int l,
                                                      int fb) {
  constexpr int flags = FLAGS;
  constexpr int U = stream32_u(FLAGS);
  const long long step = S.ss->step;
  const long long gs = step * S.n_sub + (l - 1);
  const Fluid32 F = fluid32_at(S, fb);
  const int i0 = chunk * (256 * U) + threadIdx.x;
  const int buf = (int)(gs & 1);
  int cx[U], cy[U], cz[U], pp[U];
  float ox[U], oy[U], oz[U], vx[U], vy[U], vz[U];
  bool valid[U], ev[U];
  unsigned members[U];
  int cnt[U], lin[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int i = i0 + 256 * u;
    valid[u] = i < count;
    ev[u] = false;
    members[u] = 0;
    cnt[u] = 0;
    lin[u] = 0;
    pp[u] = i;
    if (valid[u]) {
      const int p = NEAR ? S.near[i] : i;
      pp[u] = p;
      unpack(F.q[p], cx[u], cy[u], cz[u], ox[u], oy[u], oz[u]);
      vx[u] = F.vx[p]; vy[u] = F.vy[p]; vz[u] = F.vz[p];
    }
  }
#pragma unroll
  for (int u = 0; u < U; ++u) {
    if (!valid[u]) continue;
    if (flags & F_STREAM) {
      ox[u] = fmaf(vx[u], S.dtf, ox[u]); oy[u] = fmaf(vy[u], S.dtf, oy[u]); oz[u] = fmaf(vz[u], S.dtf, oz[u]);
      carry(cx[u], ox[u], S.Lx); carry(cy[u], oy[u], S.Ly); carry(cz[u], oz[u], S.Lz);
    }
    lin[u] = cx[u] + S.Lx * (cy[u] + S.Ly * cz[u]);
    if (flags & (F_COLLIDE | F_SHELL)) cnt[u] = tcount(S.Tcnt[buf][lin[u]], gs);
  }
  float rr[3] = {0.f, 0.f, 0.f};
  if (flags & F_BINROT)
    for (int k = 0; k < 3; ++k) rr[k] = S.ss->rrf[k];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    BinTerm32 bt{-1, 0, 0, 0, 0};
    if (valid[u] && (flags & (F_COLLIDE | F_SHELL)) && cnt[u] > 0) {
      cnt[u] = cnt[u] < TCAP ? cnt[u] : TCAP;
      const uint16_t *lst = S.Tlist[buf] + (size_t)lin[u] * TCAP;
      const float4 *Xq = S.Xcq[buf], *Xo = S.Xco[buf];
      const float rc2 = S.r_coll * S.r_coll, rs2 = S.r_shell * S.r_shell;
      for (int k = 0; k < cnt[u]; ++k) {
        const int j = lst[k];
        const float4 cq = Xq[j], co = Xo[j];
        const float dx = rel(cx[u], ox[u], cq.x, co.x, S.Lx), dy = rel(cy[u], oy[u], cq.y, co.y, S.Ly),
                    dz = rel(cz[u], oz[u], cq.z, co.z, S.Lz);
        const float d2 = dx * dx + dy * dy + dz * dz;
        if (flags & F_COLLIDE) ev[u] |= d2 <= rc2;
        if ((flags & F_SHELL) && d2 <= rs2) members[u] |= 1u << k;
      }
    }
    const int p = pp[u];
    if (valid[u] && !ev[u] && (flags & F_BINROT))
      bt = bin32_term(S, rr, p, cx[u], cy[u], cz[u], ox[u], oy[u], oz[u], vx[u], vy[u], vz[u]);
    if (flags & F_BINROT) bin_add_warp(S.acc, bt.c, bt.fx, bt.fy, bt.fz, bt.f2);  // the whole warp
    if (valid[u] && (flags & F_STREAM)) F.q[p] = pack(cx[u], cy[u], cz[u], ox[u], oy[u], oz[u]);
  }
  // appends: events one atomic per warp (no block barrier), run() candidate
  // records (last substep) one atomic per block for all U rounds
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  unsigned mrecs[U];
  int nrec = 0;
#pragma unroll
  for (int u = 0; u < U; ++u) {
    mrecs[u] = __ballot_sync(FULL, (flags & F_SHELL) && valid[u] && !ev[u] && members[u] != 0);
    nrec += __popc(mrecs[u]);
  }
  int brec = 0;
  if (flags & F_SHELL) brec = block_base_n(&S.ss->nshell, nrec, lane);
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int p = pp[u];
    const unsigned mrec = mrecs[u];
    const bool has_rec = (mrec >> lane) & 1u;
    const unsigned mev = __ballot_sync(FULL, ev[u]);
    int bev = 0;
    if (lane == 0 && mev) bev = atomicAdd(&S.ss->nevents, __popc(mev));
    bev = __shfl_sync(FULL, bev, 0);
    if (ev[u]) {
      const int i = bev + __popc(mev & lt);
      if (i < S.events_cap) S.events[i] = p;
      else atomicOr(&S.ss->err, ERRB_EVENTS);
    }
    if (has_rec) {
      const int i = brec + __popc(mrec & lt);
      if (i < S.shell_cap) {
        // colloids in ascending index, the order run() visits them
        const uint16_t *lst = S.Tlist[buf] + (size_t)lin[u] * TCAP;
        ShellRec *r = S.shell + i;
        r->p = F.id[p];
        r->pass = 0;
        int n = 0, last = -1;
        for (int it = 0; it < cnt[u] && n < SHELL_J; ++it) {
          int best = 0x7FFFFFFF;
          for (int k = 0; k < cnt[u]; ++k) {
            const int j = lst[k];
            if (((members[u] >> k) & 1u) && j > last && j < best) best = j;
          }
          if (best == 0x7FFFFFFF) break;
          r->j[n++] = (uint16_t)best;
          last = best;
        }
        if (__popc(members[u]) > SHELL_J) atomicOr(&S.ss->err, ERRB_SHELLSLOTS);
        r->n = (uint8_t)n;
      } else {
        atomicOr(&S.ss->err, ERRB_SHELL);
      }
    }
    brec += __popc(mrec);
  }
}

template <int FLAGS>
static __device__ __forceinline__ void k_stream32_body(const SysF64 &S, const int VB, const int NVB, int l, int fb) {
  stream32_chunk<FLAGS, false>(S, VB, S.N, l, fb);
}

template <int FLAGS>
__global__ void __launch_bounds__(256) k_stream32(__grid_constant__ const SysF64 S, int l, int fb) {
  k_stream32_body<FLAGS>(S, blockIdx.x, gridDim.x, l, fb);
}

// the same over a batch of systems (persistent: batch_for)
template <int FLAGS>
__global__ void __launch_bounds__(256) k_stream32_b(const SysF64 *Ss, const int *boff, int nrep, int l, int fb) {
  __shared__ SysF64 sS;
  batch_for(Ss, boff, nrep, sS, [&](int VB, int NVB) { k_stream32_body<FLAGS>(sS, VB, NVB, l, fb); });
}

int stream32_per_thread(int flags) { return stream32_u(flags); }

// ------------------------------------------------------------ free-flight schedule
//
// Between two SRD collisions a fluid particle moves in a straight line unless a colloid
// wall reflects it or run() kicks it, and both need a colloid within the run() shell
// radius r_shell.  A particle farther than r_shell + (its travel in the step) + (the
// colloids' largest move in the step) + slack from every colloid at the start of the
// step can meet neither in any substep: the per-substep passes would only stream it and,
// on the last substep, bin it.  The free-flight pass does that for such a particle
// (k_free_flight32: the same FP32 operations substep by substep, so the same bits), beside
// the substeps of the other particles, which the rotation pass lists (k_rotate_classify32)
// and the per-substep passes walk (k_stream32_near).  The colloids' move is bounded by
// n_sub cm (the colloid finish fails a step in which one moves further in a substep); a
// particle's travel by n_sub dt |v| (particles faster than the table allows are near);
// the slack of 0.01 covers the FP32 rounding of the distances and offsets.

// reach of the flight table: colloids within it of a cell's box can come within a
// particle's near radius of a particle in the cell
static __device__ __forceinline__ float flight_reach(const SysF64 &S) {
  return S.r_shell + S.flight_rv + (float)S.n_sub * S.ss->cm + 0.02f;
}

// the flight table of this step (both forms: the colloids' cell + offset copies are kept by
// both): colloid j (its position at the start of the step) in every cell whose box comes
// within the flight reach of it, the own box included.  A cell
// with more than FLIGHT_CAP colloids keeps counting; its particles are all near.  Block 0
// also empties the near list and draws the next step's grid shift for the free pass.
static __device__ __forceinline__ void k_flight_table32_body(const SysF64 &S, const int j) {
  const long long step = S.ss->step;
  if (j == 0 && threadIdx.x == 0) {
    S.ss->nnear = 0;
    shift_of(S, step + 2, S.ss->rrn);
  }
  if (j >= S.Nc) return;
  const int b0 = (int)((step * S.n_sub - 1) & 1);
  const float reach = flight_reach(S);
  const float4 cq = S.Xcq[b0][j], co = S.Xco[b0][j];
  const int K = (int)ceilf(reach) + 1, side = 2 * K + 1;
  const int tot = side * side * side;
  const unsigned long long tag = (unsigned long long)(unsigned)(step + 1) << 32;
  for (int q = threadIdx.x; q < tot; q += blockDim.x) {
    const int ox = q % side - K, oy = (q / side) % side - K, oz = q / (side * side) - K;
    // gap from the colloid (its cell + offset co) to the box of cell (its cell + o)
    const float ex = ox > 0 ? (float)ox - co.x : (ox < 0 ? co.x - (float)ox - 1.f : 0.f);
    const float ey = oy > 0 ? (float)oy - co.y : (oy < 0 ? co.y - (float)oy - 1.f : 0.f);
    const float ez = oz > 0 ? (float)oz - co.z : (oz < 0 ? co.z - (float)oz - 1.f : 0.f);
    if (ex * ex + ey * ey + ez * ez > reach * reach) continue;
    int bx = ((int)cq.x + ox) % S.Lx, by = ((int)cq.y + oy) % S.Ly, bz = ((int)cq.z + oz) % S.Lz;
    bx += bx < 0 ? S.Lx : 0; by += by < 0 ? S.Ly : 0; bz += bz < 0 ? S.Lz : 0;
    FlightCell *fc = S.ftab + (bx + S.Lx * (by + S.Ly * bz));
    atomicMax(&fc->tc, tag);
    const int slot = (int)(unsigned)atomicAdd(&fc->tc, 1ull);
    if (slot < FLIGHT_CAP) fc->id[slot] = (uint16_t)j;
  }
}

__global__ void __launch_bounds__(128) k_flight_table32(__grid_constant__ const SysF64 S) {
  k_flight_table32_body(S, blockIdx.x);
}

// the same over a batch of systems (persistent: batch_for; max(Nc, 1) virtual blocks each)
__global__ void __launch_bounds__(128) k_flight_table32_b(const SysF64 *Ss, const int *boff, int nrep) {
  __shared__ SysF64 sS;
  batch_for(Ss, boff, nrep, sS, [&](int VB, int) { k_flight_table32_body(sS, VB); });
}

// rotation_mpcd of one particle (the SRD map of its cell; ROT false: a counting-sort step,
// whose scatter rotated it) and its classification: a near particle is flagged and appended to
// the near list (one atomic per block).
// U particles per thread (thread t of virtual block b: particles b 256 U + t + 256 u), their
// loads issued together so that more gathers are in flight
template <bool ROT, int U>
static __device__ __forceinline__ void k_rotate_classify32_body(const SysF64 &S, const int VB, int fb) {
  const Fluid32 F = fluid32_at(S, fb);
  const long long step = S.ss->step;
  const int b0 = (int)((step * S.n_sub - 1) & 1);
  int pp[U], cc[U];
  bool valid[U], near[U];
  float vx[U], vy[U], vz[U];
  uint4 qq[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    pp[u] = VB * (256 * U) + (int)threadIdx.x + 256 * u;
    valid[u] = pp[u] < S.N;
    near[u] = false;
    if (valid[u]) {
      const int p = pp[u];
      cc[u] = ROT ? S.rotcell[p] : S.C;
      vx[u] = F.vx[p]; vy[u] = F.vy[p]; vz[u] = F.vz[p];
      qq[u] = F.q[p];
    }
  }
#pragma unroll
  for (int u = 0; u < U; ++u) {
    if (!valid[u]) continue;
    const int p = pp[u];
    int cx, cy, cz;
    float ox, oy, oz;
    unpack(qq[u], cx, cy, cz, ox, oy, oz);
    const bool inb = cx < S.Lx && cy < S.Ly && cz < S.Lz;  // (a record within the box)
    const FlightCell *fc = S.ftab + (inb ? cx + S.Lx * (cy + S.Ly * cz) : 0);
    const uint4 w0 = reinterpret_cast<const uint4 *>(fc)[0], w1 = reinterpret_cast<const uint4 *>(fc)[1];
    if (ROT) {
      if (cc[u] < S.C) apply_map32(S.cell_ab32 + (size_t)cc[u] * 12, vx[u], vy[u], vz[u]);
      F.vx[p] = vx[u]; F.vy[p] = vy[u]; F.vz[p] = vz[u];
    }
    const float travel = (float)S.n_sub * S.dtf * sqrtf(vx[u] * vx[u] + vy[u] * vy[u] + vz[u] * vz[u]);
    const int cnt = tcount(((unsigned long long)w0.y << 32) | w0.x, step);
    bool nr = false;
    if (!inb || !(travel <= S.flight_rv) || cnt > FLIGHT_CAP) {
      nr = true;  // faster than the table allows (or not finite), or a crowded cell
    } else if (cnt > 0) {
      const float r = S.r_shell + travel + (float)S.n_sub * S.ss->cm + 0.01f, r2 = r * r;
      const unsigned ids[6] = {w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
      const float4 *Xq = S.Xcq[b0], *Xo = S.Xco[b0];
      for (int k = 0; k < cnt; ++k) {
        const int j = (int)((ids[k >> 1] >> (16 * (k & 1))) & 0xFFFFu);
        const float4 cq = Xq[j], co = Xo[j];
        const float dx = rel(cx, ox, cq.x, co.x, S.Lx), dy = rel(cy, oy, cq.y, co.y, S.Ly),
                    dz = rel(cz, oz, cq.z, co.z, S.Lz);
        nr = nr || !(dx * dx + dy * dy + dz * dz > r2);
      }
    }
    near[u] = nr;
    S.fnear[p] = nr ? 1 : 0;
  }
  // the near list: one atomic per block for all U rounds
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  unsigned m[U];
  int tot = 0;
#pragma unroll
  for (int u = 0; u < U; ++u) {
    m[u] = __ballot_sync(FULL, near[u]);
    tot += __popc(m[u]);
  }
  int base = block_base_n(&S.ss->nnear, tot, lane);
#pragma unroll
  for (int u = 0; u < U; ++u) {
    if (near[u]) S.near[base + __popc(m[u] & lt)] = pp[u];
    base += __popc(m[u]);
  }
}

template <bool ROT>
__global__ void __launch_bounds__(256) k_rotate_classify32(__grid_constant__ const SysF64 S, int fb) {
  k_rotate_classify32_body<ROT, CLASSIFY32_U>(S, blockIdx.x, fb);
}

// the same over a batch of systems (persistent: batch_for)
template <bool ROT>
__global__ void __launch_bounds__(256) k_rotate_classify32_b(const SysF64 *Ss, const int *boff, int nrep, int fb) {
  __shared__ SysF64 sS;
  batch_for(Ss, boff, nrep, sS, [&](int VB, int) { k_rotate_classify32_body<ROT, CLASSIFY32_U>(sS, VB, fb); });
}

// the free particles' whole step: n_sub streaming substeps (update_pos_mpcd, the
// streaming passes' operations in order) and the binning of the last substep with the
// next step's grid shift.  Runs beside the near particles' substeps, which touch none of
// its particles; a grid of a few blocks per SM walks the fluid (it shares the SMs with the
// substeps' latency-bound chain).
static __device__ __forceinline__ void k_free_flight32_body(const SysF64 &S, const int VB, const int NVB, int fb) {
  const Fluid32 F = fluid32_at(S, fb);
  const float rr[3] = {(float)S.ss->rrn[0], (float)S.ss->rrn[1], (float)S.ss->rrn[2]};
  for (int p0 = VB * blockDim.x; p0 < S.N; p0 += NVB * blockDim.x) {
    const int p = p0 + threadIdx.x;
    BinTerm32 bt{-1, 0, 0, 0, 0};
    if (p < S.N && !S.fnear[p]) {
      int cx, cy, cz;
      float ox, oy, oz;
      unpack(F.q[p], cx, cy, cz, ox, oy, oz);
      const float vx = F.vx[p], vy = F.vy[p], vz = F.vz[p];
      for (int l = 0; l < S.n_sub; ++l) {
        ox = fmaf(vx, S.dtf, ox); oy = fmaf(vy, S.dtf, oy); oz = fmaf(vz, S.dtf, oz);
        carry(cx, ox, S.Lx); carry(cy, oy, S.Ly); carry(cz, oz, S.Lz);
      }
      bt = bin32_term(S, rr, p, cx, cy, cz, ox, oy, oz, vx, vy, vz);
      F.q[p] = pack(cx, cy, cz, ox, oy, oz);
    }
    bin_add_warp(S.acc, bt.c, bt.fx, bt.fy, bt.fz, bt.f2);  // the whole warp
  }
}

__global__ void __launch_bounds__(256) k_free_flight32(__grid_constant__ const SysF64 S, int fb) {
  k_free_flight32_body(S, blockIdx.x, gridDim.x, fb);
}

// the same over a batch of systems (persistent: batch_for; each virtual block walks its
// system's fluid with the system's virtual blocks as stride)
__global__ void __launch_bounds__(256) k_free_flight32_b(const SysF64 *Ss, const int *boff, int nrep, int fb) {
  __shared__ SysF64 sS;
  batch_for(Ss, boff, nrep, sS, [&](int VB, int NVB) { k_free_flight32_body(sS, VB, NVB, fb); });
}

// the per-substep pass over the near list (stride over chunks of 256 U)
template <int FLAGS>
static __device__ __forceinline__ void k_stream32_near_body(const SysF64 &S, const int VB, const int NVB, int l,
                                                            int fb) {
  const int count = S.ss->nnear;
  constexpr int per = 256 * stream32_u(FLAGS);
  for (int chunk = VB; chunk * per < count; chunk += NVB) stream32_chunk<FLAGS, true>(S, chunk, count, l, fb);
}

template <int FLAGS>
__global__ void __launch_bounds__(256) k_stream32_near(__grid_constant__ const SysF64 S, int l, int fb) {
  k_stream32_near_body<FLAGS>(S, blockIdx.x, gridDim.x, l, fb);
}

// the same over a batch of systems (persistent: batch_for)
template <int FLAGS>
__global__ void __launch_bounds__(256) k_stream32_near_b(const SysF64 *Ss, const int *boff, int nrep, int l, int fb) {
  __shared__ SysF64 sS;
  batch_for(Ss, boff, nrep, sS, [&](int VB, int NVB) { k_stream32_near_body<FLAGS>(sS, VB, NVB, l, fb); });
}

ClassifyKernel classify_kernel32(bool rotate) {
  return rotate ? k_rotate_classify32<true> : k_rotate_classify32<false>;
}

ClassifyKernelB classify_kernel32_b(bool rotate) {
  return rotate ? k_rotate_classify32_b<true> : k_rotate_classify32_b<false>;
}

StreamKernelB stream_kernel32_near_b(int flags) {
  switch (flags) {
    case F_STREAM | F_COLLIDE: return k_stream32_near_b<F_STREAM | F_COLLIDE>;
    case F_STREAM | F_COLLIDE | F_SHELL | F_BINROT: return k_stream32_near_b<F_STREAM | F_COLLIDE | F_SHELL | F_BINROT>;
  }
  return nullptr;
}

StreamKernel stream_kernel32_near(int flags) {
  switch (flags) {
    case F_STREAM | F_COLLIDE: return k_stream32_near<F_STREAM | F_COLLIDE>;
    case F_STREAM | F_COLLIDE | F_SHELL | F_BINROT: return k_stream32_near<F_STREAM | F_COLLIDE | F_SHELL | F_BINROT>;
  }
  return nullptr;
}

// wall collisions of the listed particles in colloid order, then (last substep)
// their run() record and binning; one particle per lane
template <int FLAGS>
static __device__ __forceinline__ void k_events32_body(const SysF64 &S, const int VB, const int NVB, int l, int fb) {
  constexpr int flags = FLAGS;
  const long long step = S.ss->step;
  const long long gs = step * S.n_sub + (l - 1);
  const int buf = (int)(gs & 1);
  const Fluid32 F = fluid32_at(S, fb);
  const int n = min(S.ss->nevents, S.events_cap);
  const int k0 = (threadIdx.x & 31) * (blockDim.x >> 5) + (threadIdx.x >> 5);
  for (int base = 0;; base += blockDim.x) {
    const int i = VB + NVB * (k0 + base);
    const bool valid = i < n;
    if (!__any_sync(FULL, valid)) break;
    const int p = valid ? S.events[i] : 0;
    int cx = 0, cy = 0, cz = 0;
    float ox = 0.f, oy = 0.f, oz = 0.f, vx = 0.f, vy = 0.f, vz = 0.f;
    int cnt = 0, id = 0;
    if (valid) {
      unpack(F.q[p], cx, cy, cz, ox, oy, oz);
      vx = F.vx[p]; vy = F.vy[p]; vz = F.vz[p];
      id = F.id[p];
    }
    const int lin = cx + S.Lx * (cy + S.Ly * cz);
    if (valid) {
      cnt = tcount(S.Tcnt[buf][lin], gs);
      cnt = cnt < TCAP ? cnt : TCAP;
    }
    const uint16_t *lst = S.Tlist[buf] + (size_t)lin * TCAP;
    const int cx0 = cx, cy0 = cy, cz0 = cz;
    const float ox0 = ox, oy0 = oy, oz0 = oz;
    if (flags & F_COLLIDE) collide32_warp<FLAGS>(S, gs, buf, valid, id, cnt, lst, cx, cy, cz, ox, oy, oz, vx, vy, vz);
    if (!valid) continue;
    finish32<FLAGS>(S, F, p, id, buf, cnt, lst, cx0, cy0, cz0, ox0, oy0, oz0, cx, cy, cz, ox, oy, oz, vx, vy, vz);
  }
}

template <int FLAGS>
__global__ void __launch_bounds__(128) k_events32(__grid_constant__ const SysF64 S, int l, int fb) {
  k_events32_body<FLAGS>(S, blockIdx.x, gridDim.x, l, fb);
}

// the same over a batch of systems (persistent: batch_for)
template <int FLAGS>
__global__ void __launch_bounds__(128) k_events32_b(const SysF64 *Ss, const int *boff, int nrep, int l, int fb) {
  __shared__ SysF64 sS;
  batch_for(Ss, boff, nrep, sS, [&](int VB, int NVB) { k_events32_body<FLAGS>(sS, VB, NVB, l, fb); });
}

StreamKernel stream_kernel32(int flags) {
  switch (flags) {
    case F_STREAM | F_COLLIDE: return k_stream32<F_STREAM | F_COLLIDE>;
    case F_STREAM | F_COLLIDE | F_SHELL | F_BINROT: return k_stream32<F_STREAM | F_COLLIDE | F_SHELL | F_BINROT>;
    case F_SHELL | F_BINROT: return k_stream32<F_SHELL | F_BINROT>;
  }
  return nullptr;
}

EventKernel event_kernel32(int flags) {
  switch (flags) {
    case F_STREAM | F_COLLIDE: return k_events32<F_COLLIDE>;
    case F_STREAM | F_COLLIDE | F_SHELL | F_BINROT: return k_events32<F_COLLIDE | F_SHELL | F_BINROT>;
    case F_SHELL | F_BINROT: return k_events32<F_SHELL | F_BINROT>;
  }
  return nullptr;
}

StreamKernelB stream_kernel32_b(int flags) {
  switch (flags) {
    case F_STREAM | F_COLLIDE: return k_stream32_b<F_STREAM | F_COLLIDE>;
    case F_STREAM | F_COLLIDE | F_SHELL | F_BINROT: return k_stream32_b<F_STREAM | F_COLLIDE | F_SHELL | F_BINROT>;
    case F_SHELL | F_BINROT: return k_stream32_b<F_SHELL | F_BINROT>;
  }
  return nullptr;
}

EventKernelB event_kernel32_b(int flags) {
  switch (flags) {
    case F_STREAM | F_COLLIDE: return k_events32_b<F_COLLIDE>;
    case F_STREAM | F_COLLIDE | F_SHELL | F_BINROT: return k_events32_b<F_COLLIDE | F_SHELL | F_BINROT>;
    case F_SHELL | F_BINROT: return k_events32_b<F_SHELL | F_BINROT>;
  }
  return nullptr;
}

// SRD collision per cell (cpp/rotation_mpcd.cpp:14-49): cell mean from the exact
// sums, thermostat factor in FP64, rotation about the random axis in FP32, stored
// as the FP32 affine map v' = A v + b; plus the occupancy prefix of the counting sort.
static __device__ __forceinline__ void k_cell_prep32_body(const SysF64 &S, const int VB, const int NVB) {
  const int c = VB * blockDim.x + threadIdx.x;
  CellAcc a = CellAcc{0, 0, 0, 0, 0, 0};
  if (c < S.Cpad) {
    a = S.acc[c];
    S.acc[c] = CellAcc{0, 0, 0, 0, 0, 0};
    S.cursor[c] = 0;
  }
  {
    __shared__ int wsum[8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int v = a.n, incl = v;
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    int before = 0, total = 0;
    for (int q = 0; q < 8; ++q) {
      before += q < w ? wsum[q] : 0;
      total += wsum[q];
    }
    if (c < S.Cpad) S.cell_off[c] = before + incl - v;
    if (threadIdx.x == 0) S.blk_off[VB] = total;
  }
  if (c >= S.C) return;
  float4 *ab4 = reinterpret_cast<float4 *>(S.cell_ab32 + (size_t)c * 12);
  const int n = a.n;
  if (n > S.max_per_cell) atomicOr(&S.ss->err, ERRB_OCCUPANCY);
  if (n <= 1 || n > S.max_per_cell) {
    ab4[0] = make_float4(1.f, 0.f, 0.f, 0.f);
    ab4[1] = make_float4(1.f, 0.f, 0.f, 0.f);
    ab4[2] = make_float4(1.f, 0.f, 0.f, 0.f);
    return;
  }
  // mean and thermostat factor in FP64 from the exact sums
  // (2^-kw / n in one factor: the power-of-two scaling is exact)
  const double insw = S.insw_n[n];
  const double ux = (double)a.sx * insw, uy = (double)a.sy * insw, uz = (double)a.sz * insw;
  const double var = (double)a.s2 * S.inv_sw - (double)n * (ux * ux + uy * uy + uz * uz);
  // The factor sqrt(3 kT (n - 1) / (m var)) scales FP32 velocities, so it is needed to FP32
  // precision only: the variance in FP64 (from the exact sums, where the cancellation
  // happens), its reciprocal root in FP32 times sqrt(3 kT (n - 1) / m) (per n, from the host)
  const float s = var > 0 ? S.sq3kt_n32[n] * rsqrtf((float)var) : 1.f;
  // rotation axis rho = 2 ran - 1, phi = 2 pi ran (cpp/rotation_mpcd.cpp:19-20)
  uint4 r = draw4(S.key, DOM_AXIS, 0, (uint32_t)(c + 1), 0, (uint32_t)(S.ss->step + 1));
  const float rho = 2.f * u01f(r.x) - 1.f;
  float sp, cp;
  sincospif(2.f * u01f(r.y), &sp, &cp);
  const float sq = sqrtf(fmaxf(1.f - rho * rho, 0.f));
  const float r1 = cp * sq, r2 = sp * sq, r3 = rho;
  const float ct = (float)S.ct, st = (float)S.st, ict = (float)S.ict;
  const float i1 = ict * r1, i2 = ict * r2, i3 = ict * r3;
  const float R[9] = {i1 * r1 + ct, i1 * r2 - st * r3, i1 * r3 + st * r2,
                      i2 * r1 + st * r3, i2 * r2 + ct, i2 * r3 - st * r1,
                      i3 * r1 - st * r2, i3 * r2 + st * r1, i3 * r3 + ct};
  const float fx = (float)ux, fy = (float)uy, fz = (float)uz;
  float A[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) A[k] = s * R[k];
  const float b0 = fx - (A[0] * fx + A[1] * fy + A[2] * fz);
  const float b1 = fy - (A[3] * fx + A[4] * fy + A[5] * fz);
  const float b2 = fz - (A[6] * fx + A[7] * fy + A[8] * fz);
  ab4[0] = make_float4(A[0], A[1], A[2], A[3]);
  ab4[1] = make_float4(A[4], A[5], A[6], A[7]);
  ab4[2] = make_float4(A[8], b0, b1, b2);
}

__global__ void __launch_bounds__(256) k_cell_prep32(__grid_constant__ const SysF64 S) {
  k_cell_prep32_body(S, blockIdx.x, gridDim.x);
}

// the same over a batch of systems (persistent: batch_for)
__global__ void __launch_bounds__(256) k_cell_prep32_b(const SysF64 *Ss, const int *boff, int nrep) {
  __shared__ SysF64 sS;
  batch_for(Ss, boff, nrep, sS, [&](int VB, int NVB) { k_cell_prep32_body(sS, VB, NVB); });
}

static __device__ __forceinline__ void k_rotate32_body(const SysF64 &S, const int VB, const int NVB, int fb) {
  const int p = VB * blockDim.x + threadIdx.x;
  if (p >= S.N) return;
  const int c = S.rotcell[p];
  if (c >= S.C) return;
  const Fluid32 F = fluid32_at(S, fb);
  float vx = F.vx[p], vy = F.vy[p], vz = F.vz[p];
  apply_map32(S.cell_ab32 + (size_t)c * 12, vx, vy, vz);
  F.vx[p] = vx; F.vy[p] = vy; F.vz[p] = vz;
}

__global__ void __launch_bounds__(256) k_rotate32(__grid_constant__ const SysF64 S, int fb) {
  k_rotate32_body(S, blockIdx.x, gridDim.x, fb);
}

// the same over a batch of systems (persistent: batch_for)
__global__ void __launch_bounds__(256) k_rotate32_b(const SysF64 *Ss, const int *boff, int nrep, int fb) {
  __shared__ SysF64 sS;
  batch_for(Ss, boff, nrep, sS, [&](int VB, int NVB) { k_rotate32_body(sS, VB, NVB, fb); });
}

static __device__ __forceinline__ void k_rotate_sort32_body(const SysF64 &S, const int VB, const int NVB, int src, int dst) {
  const int p = VB * blockDim.x + threadIdx.x;
  if (p >= S.N) return;
  const Fluid32 F = fluid32_at(S, src), G = fluid32_at(S, dst);
  const int c = S.rotcell[p];
  float vx = F.vx[p], vy = F.vy[p], vz = F.vz[p];
  if (c < S.C) apply_map32(S.cell_ab32 + (size_t)c * 12, vx, vy, vz);
  const unsigned act = __activemask();
  const unsigned grp = __match_any_sync(act, c);
  const int lane = threadIdx.x & 31, leader = __ffs(grp) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(&S.cursor[c], __popc(grp));
  base = __shfl_sync(grp, base, leader);
  const int slot = S.blk_off[c >> 8] + S.cell_off[c] + base + __popc(grp & ((1u << lane) - 1u));
  const int id = F.id[p];
  if (slot < 0 || slot >= S.N || id < 0 || id >= S.N) {
    atomicOr(&S.ss->err, ERRB_OCCUPANCY);
    return;
  }
  G.q[slot] = F.q[p];
  G.vx[slot] = vx; G.vy[slot] = vy; G.vz[slot] = vz;
  G.id[slot] = id;
  S.newpos[id] = slot;
}

__global__ void __launch_bounds__(256) k_rotate_sort32(__grid_constant__ const SysF64 S, int src, int dst) {
  k_rotate_sort32_body(S, blockIdx.x, gridDim.x, src, dst);
}

// the same over a batch of systems (persistent: batch_for)
__global__ void __launch_bounds__(256) k_rotate_sort32_b(const SysF64 *Ss, const int *boff, int nrep, int src, int dst) {
  __shared__ SysF64 sS;
  batch_for(Ss, boff, nrep, sS, [&](int VB, int NVB) { k_rotate_sort32_body(sS, VB, NVB, src, dst); });
}

// run() (cpp/run.cpp:17-24) on the FP32 fluid: rear-shell test against V + v0 ra
static __device__ __forceinline__ void k_run_shell32_body(const SysF64 &S, const int VB, const int NVB, int fb) {
  const int n = min(S.ss->nshell, S.shell_cap);
  const int b = (int)((S.ss->step * S.n_sub - 1) & 1);
  const float4 *Xq = S.Xcq[b], *Xo = S.Xco[b];
  const Fluid32 F = fluid32_at(S, fb);
  for (int i = VB * blockDim.x + threadIdx.x; i < n; i += NVB * blockDim.x) {
    ShellRec rec = S.shell[i];
    int p = S.newpos[rec.p];
    int cx, cy, cz;
    float ox, oy, oz;
    unpack(F.q[p], cx, cy, cz, ox, oy, oz);
    uint8_t pass = 0;
    for (int k = 0; k < rec.n; ++k) {
      int j = rec.j[k];
      float4 cq = Xq[j], co = Xo[j];
      float rx = rel(cx, ox, cq.x, co.x, S.Lx), ry = rel(cy, oy, cq.y, co.y, S.Ly), rz = rel(cz, oz, cq.z, co.z, S.Lz);
      double Vx = S.V[3 * j] + S.ra[3 * j] * S.v0, Vy = S.V[3 * j + 1] + S.ra[3 * j + 1] * S.v0,
             Vz = S.V[3 * j + 2] + S.ra[3 * j + 2] * S.v0;
      if (rx * (float)Vx + ry * (float)Vy + rz * (float)Vz <= 0.f) {
        pass |= (uint8_t)(1u << k);
        atomicAdd(&S.shell_cnt[j], 1);
      }
    }
    S.shell[i].pass = pass;
  }
}

__global__ void k_run_shell32(__grid_constant__ const SysF64 S, int fb) {
  k_run_shell32_body(S, blockIdx.x, gridDim.x, fb);
}

// the same over a batch of systems (persistent: batch_for)
__global__ void k_run_shell32_b(const SysF64 *Ss, const int *boff, int nrep, int fb) {
  __shared__ SysF64 sS;
  batch_for(Ss, boff, nrep, sS, [&](int VB, int NVB) { k_run_shell32_body(sS, VB, NVB, fb); });
}

static __device__ __forceinline__ void k_run_kick32_body(const SysF64 &S, const int VB, const int NVB, int fb) {
  const int n = min(S.ss->nshell, S.shell_cap);
  const Fluid32 F = fluid32_at(S, fb);
  for (int i = VB * blockDim.x + threadIdx.x; i < n; i += NVB * blockDim.x) {
    ShellRec rec = S.shell[i];
    if (!rec.pass) continue;
    int p = S.newpos[rec.p];
    float vx = F.vx[p], vy = F.vy[p], vz = F.vz[p];
    for (int k = 0; k < rec.n; ++k) {
      if (!((rec.pass >> k) & 1)) continue;
      int j = rec.j[k];
      // M v0 / (m cnt) in FP32 (the velocity it changes is FP32): no double division
      const float f = S.kick32 / (float)S.shell_cnt[j];
      vx -= (float)S.ra[3 * j] * f; vy -= (float)S.ra[3 * j + 1] * f; vz -= (float)S.ra[3 * j + 2] * f;
    }
    F.vx[p] = vx; F.vy[p] = vy; F.vz[p] = vz;
  }
}

__global__ void k_run_kick32(__grid_constant__ const SysF64 S, int fb) {
  k_run_kick32_body(S, blockIdx.x, gridDim.x, fb);
}

// the same over a batch of systems (persistent: batch_for)
__global__ void k_run_kick32_b(const SysF64 *Ss, const int *boff, int nrep, int fb) {
  __shared__ SysF64 sS;
  batch_for(Ss, boff, nrep, sS, [&](int VB, int NVB) { k_run_kick32_body(sS, VB, NVB, fb); });
}

// AoS doubles (particle order) -> FP32 records; download scatters back by id
__global__ void __launch_bounds__(256) k_aos_to_q(const SysF64 S, const double *pos, const double *vel, int fb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S.N) return;
  const Fluid32 F = fluid32_at(S, fb);
  int c[3];
  float o[3];
  const int L[3] = {S.Lx, S.Ly, S.Lz};
  for (int k = 0; k < 3; ++k) {
    double x = pos[3 * (size_t)i + k];
    double fl = floor(x);
    double off = x - fl;
    long long ci = (long long)fl;
    float of = (float)off;
    if (of >= 1.f) { of = 0.f; ci += 1; }
    ci %= L[k];
    if (ci < 0) ci += L[k];
    c[k] = (int)ci;
    o[k] = of;
  }
  F.q[i] = pack(c[0], c[1], c[2], o[0], o[1], o[2]);
  F.vx[i] = (float)vel[3 * (size_t)i]; F.vy[i] = (float)vel[3 * (size_t)i + 1]; F.vz[i] = (float)vel[3 * (size_t)i + 2];
  F.id[i] = i;
  S.newpos[i] = i;
}

__global__ void __launch_bounds__(256) k_q_to_aos(const SysF64 S, double *pos, double *vel, int fb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S.N) return;
  const Fluid32 F = fluid32_at(S, fb);
  int cx, cy, cz;
  float ox, oy, oz;
  unpack(F.q[i], cx, cy, cz, ox, oy, oz);
  const size_t o = 3 * (size_t)F.id[i];
  if (pos) { pos[o] = (double)cx + (double)ox; pos[o + 1] = (double)cy + (double)oy; pos[o + 2] = (double)cz + (double)oz; }
  if (vel) { vel[o] = F.vx[i]; vel[o + 1] = F.vy[i]; vel[o + 2] = F.vz[i]; }
}

}  // namespace bgb
