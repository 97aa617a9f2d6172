// FP64 form of the MPCD + active-colloid step (sm_103a).
//
// Data layout (HBM, structure of arrays): fluid positions px/py/pz and per-substep
// displacements w = v*dt (wx/wy/wz) in double; one int per particle for the cell
// of the next SRD binning; per-cell exact sums (CellAcc); the 3x3 map and offset
// of each cell's SRD collision (cell_ab); colloid arrays of a few KB.
//
// Kernels of one MPCD step (one CUDA graph):
//   k_cell_prep   per cell: mean, thermostat factor, random axis -> w' = A w + b
//   k_rotate      per particle: w' = A w + b                      rotation_mpcd
//   k_run_shell   per run() candidate: rear-shell test and count   run
//   k_run_kick    per run() candidate: compensating fluid kick     run
//   k_fin         per colloid (one thread): run()'s colloid kick, update_pos_md
//   then per substep g:
//   k_stream      per particle: streaming, wall collisions with the colloids its cell
//                 table lists, and (last substep) run() candidates and the next SRD
//                 binning (update_pos_mpcd, neighbour_list_mpcd, fluid_colloid_collision);
//                 its first blocks meanwhile compute the WCA forces at the substep's
//                 colloid positions and the cell table of the next substep
//   k_fin         per colloid: end of fluid_colloid_collision, update_activity_direction,
//                 update_velocity_colloid, then update_pos_md of the next substep
#include "kernels.cuh"

namespace bgb {

constexpr unsigned FULL = 0xFFFFFFFFu;

// ----------------------------------------------------------------- cell helpers

__device__ __forceinline__ int lin_cell(const SysF64 &S, int ix, int iy, int iz) { return ix + S.Lx * (iy + S.Ly * iz); }

__device__ __forceinline__ bool off_ok(int d, int L) {
  int m = d % L;
  if (m < 0) m += L;
  return m <= 3 || m >= L - 3;
}

// Is cell `lin` one of the 342 neighbour boxes of cell `cb` (create_box,
// cpp/neighbour_list.cpp:12-25: periodic offsets -3..3 per axis, own box
// excluded)?  Cell numbers >= C (a coordinate exactly at L past the last row)
// have no neighbour entries in the reference.
__device__ __forceinline__ bool in_block(const SysF64 &S, int cb, int lin) {
  if (cb >= S.C || lin >= S.C || cb == lin) return false;
  int cx = cb % S.Lx, ct = cb / S.Lx, cy = ct % S.Ly, cz = ct / S.Ly;
  int bx = lin % S.Lx, bt = lin / S.Lx, by = bt % S.Ly, bz = bt / S.Ly;
  return off_ok(bx - cx, S.Lx) && off_ok(by - cy, S.Ly) && off_ok(bz - cz, S.Lz);
}

// 1 + cell(pos) - 1: the reference's truncating linear cell of a wrapped position.
// A wrapped coordinate lies in [0, L], so each integer part is at most L and the
// cell number stays below Cpad; anything else (NaN, a negative or runaway
// position) is clamped, flagged, and never used to index past the tables.
__device__ __forceinline__ int cell_of_pos(const SysF64 &S, double x, double y, double z, bool &alias) {
  int ix = trunc_nonneg(x), iy = trunc_nonneg(y), iz = trunc_nonneg(z);
  bool bad = (ix > S.Lx) | (iy > S.Ly) | (iz > S.Lz) | (dbits(x) < 0) | (dbits(y) < 0) | (dbits(z) < 0);
  if (bad) {
    atomicOr(&S.ss->err, ERRB_VRANGE);
    ix = min(ix, S.Lx); iy = min(iy, S.Ly); iz = min(iz, S.Lz);
  }
  alias = (ix >= S.Lx) | (iy >= S.Ly) | (iz >= S.Lz);
  return lin_cell(S, ix, iy, iz);
}

// count of the cell-table entry if it belongs to substep g
__device__ __forceinline__ int tcount(unsigned long long v, long long g) {
  return (unsigned)(v >> 32) == (unsigned)g ? (int)(unsigned)v : 0;
}

// append colloid j to cell `cell` of the table of substep e
__device__ __forceinline__ void tappend(unsigned long long *Tc, uint16_t *Tl, int cell, long long e, int j, int *err) {
  const unsigned long long tag = (unsigned long long)(unsigned)e << 32;
  unsigned long long old = Tc[cell];
  for (int it = 0; it < 256; ++it) {
    unsigned long long nv = ((unsigned)(old >> 32) == (unsigned)e) ? old + 1 : (tag | 1ull);
    unsigned long long prev = atomicCAS(&Tc[cell], old, nv);
    if (prev == old) {
      int slot = (int)(unsigned)nv - 1;
      if (slot < TCAP) Tl[(size_t)cell * TCAP + slot] = (uint16_t)j;
      else atomicOr(err, ERRB_TTABLE);
      return;
    }
    old = prev;
  }
  atomicOr(err, ERRB_TTABLE);
}

// FP32 copy of a double by truncating the mantissa (integer pipe); relative
// error below 2^-23
__device__ __forceinline__ float d2f_trunc(double x) {
  long long b = dbits(x);
  int e = (int)((b >> 52) & 0x7FF);
  if (e == 0) return 0.f;
  int fe = e - 1023 + 127;
  if (fe <= 0) return 0.f;
  if (fe >= 255) return __int_as_float(0x7f800000);
  unsigned m = (unsigned)((b >> 29) & 0x7FFFFF);
  return __uint_as_float(((unsigned)((unsigned long long)b >> 32) & 0x80000000u) | ((unsigned)fe << 23) | m);
}

__device__ __forceinline__ float wrap_half(float d, float L) {
  if (d > 0.5f * L) d -= L;
  else if (d < -0.5f * L) d += L;
  return d;
}

// ----------------------------------------------------------- exact exchange sums

__device__ __forceinline__ void exch_add(ExchAcc *e, int comp, double v, int *err) {
  if ((dbits(v) & 0x7FFFFFFFFFFFFFFFll) >= 0x4130000000000000ll) atomicOr(err, ERRB_DELTA);  // |v| >= 2^20
  long long hi = to_fix(v, 20);
  double res = __dsub_rn(v, (double)hi * 0x1p-20);
  long long lo = to_fix(res, 72);
  atomicAdd((unsigned long long *)&e->hi[comp], (unsigned long long)hi);
  atomicAdd((unsigned long long *)&e->lo[comp], (unsigned long long)lo);
}

__device__ __forceinline__ double exch_val(const ExchAcc &e, int comp) {
  return __dadd_rn((double)e.hi[comp] * 0x1p-20, (double)e.lo[comp] * 0x1p-72);
}

// ------------------------------------------------------- stochastic reflection

struct CollDraw {
  uint2 key;
  uint32_t a, b, t;
  int idx;
  uint4 buf;
};

__device__ __forceinline__ double cd_next(CollDraw &d) {
  int s = d.idx & 3;
  if (s == 0) d.buf = draw4(d.key, DOM_COLL, (uint32_t)(d.idx >> 2), d.a, d.b, d.t);
  d.idx++;
  uint32_t w = s == 0 ? d.buf.x : s == 1 ? d.buf.y : s == 2 ? d.buf.z : d.buf.w;
  return u01(w);
}

// stochastic_reflection (cpp/fluid_colloid_collision.cpp:7-24): Rayleigh normal
// speed along rs plus one Gaussian tangential component along unit(un x t)
__device__ d3 stochastic_reflection(const SysF64 &S, CollDraw &d, d3 rf, d3 rs) {
  double u = cd_next(d);
  double om = __dsub_rn(1.0, u);
  double random_e = __dmul_rn(om, om);
  // vector / |vector| as one reciprocal and three products (within an ulp of the
  // reference's three divisions); likewise /m_beta as * kT/m
  d3 n = mul3s(rs, __drcp_rn(__dsqrt_rn(norm2_ref(rs.x, rs.y, rs.z))));
  double val = __dsqrt_rn(__dmul_rn(-log(random_e), S.inv_m_beta));
  d3 un = mul3s(n, val);
  double t0 = cd_next(d), t1 = cd_next(d), t2 = cd_next(d);
  d3 t = mk(ref_img(__dsub_rn(__dmul_rn(t0, S.dx.L), rf.x), S.dx), ref_img(__dsub_rn(__dmul_rn(t1, S.dy.L), rf.y), S.dy),
            ref_img(__dsub_rn(__dmul_rn(t2, S.dz.L), rf.z), S.dz));
  d3 ut = cross_ref(un, t);
  ut = mul3s(ut, __drcp_rn(__dsqrt_rn(norm2_ref(ut.x, ut.y, ut.z))));
  double x1 = 0, x2 = 0, z = 2.0;
  // polar Box-Muller rejection; each try is a fixed function of the key, and a
  // try is rejected with probability 1 - pi/4, so 256 tries never run out
  for (int it = 0; z > 1.0 && it < 256; ++it) {
    x1 = __dsub_rn(__dmul_rn(2.0, cd_next(d)), 1.0);
    x2 = __dsub_rn(__dmul_rn(2.0, cd_next(d)), 1.0);
    z = __dadd_rn(__dmul_rn(x1, x1), __dmul_rn(x2, x2));
  }
  z = __dsqrt_rn(__ddiv_rn(__dmul_rn(-2.0, log(z)), z));
  double v1 = __dmul_rn(__dmul_rn(x1, z), S.sqrt_kt_m);
  return add3(mul3s(ut, v1), un);
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

__device__ __forceinline__ int cand_next(const SysF64 &S, CandIter &it, const int *cbox) {
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
__device__ __forceinline__ bool within(const SysF64 &S, const double *Xc, float4 c, int j, double x, double y, double z,
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

// Everything a particle does near colloids: wall collisions in colloid order
// (fluid_colloid_collision.cpp:30-45) and, on the last substep, the run()
// candidate record.  Kept out of line so the common streaming path stays lean.
__device__ __noinline__ void near_colloids(const SysF64 &S, int flags, int pid, int lin, bool alias, long long gs,
                                           int buf, double &x, double &y, double &z, double &wx, double &wy,
                                           double &wz, bool &wchanged, ShellRec &rec) {
  const double *Xc = S.X[buf];
  const float4 *Xf = S.Xf[buf];
  const int *cbox = S.cbox[buf];
  CandIter it;
  it.brute = alias;
  it.lin = lin;
  it.last = -1;
  if (!alias) {
    int c = tcount(S.Tcnt[buf][lin], gs);
    it.cnt = c < TCAP ? c : TCAP;
    it.lst = S.Tlist[buf] + (size_t)lin * TCAP;
  } else {
    it.cnt = 0;
    it.lst = nullptr;
  }
  const double x0 = x, y0 = y, z0 = z;
  d3 vdump = mk(0, 0, 0);
  bool have_dump = false;
  if (flags & F_COLLIDE) {
    for (int j = cand_next(S, it, cbox); j >= 0; j = cand_next(S, it, cbox)) {
      if (!within(S, Xc, Xf[j], j, x, y, z, S.r_coll, S.sig2q)) continue;
      d3 Xj = mk(Xc[3 * j], Xc[3 * j + 1], Xc[3 * j + 2]);
      if (!have_dump) {  // dump_vel_fl: the velocity when the collision routine began
        vdump = mk(__dmul_rn(wx, S.inv_dt), __dmul_rn(wy, S.inv_dt), __dmul_rn(wz, S.inv_dt));
        have_dump = true;
      }
      // step back half a substep with the current velocity
      x = ref_mod(__dsub_rn(x, __dmul_rn(wx, 0.5)), S.dx);
      y = ref_mod(__dsub_rn(y, __dmul_rn(wy, 0.5)), S.dy);
      z = ref_mod(__dsub_rn(z, __dmul_rn(wz, 0.5)), S.dz);
      d3 rs = mk(ref_img(__dsub_rn(x, Xj.x), S.dx), ref_img(__dsub_rn(y, Xj.y), S.dy), ref_img(__dsub_rn(z, Xj.z), S.dz));
      CollDraw d;
      d.key = S.key; d.a = (uint32_t)(pid + 1); d.b = (uint32_t)(j + 1); d.t = (uint32_t)gs; d.idx = 0;
      d3 u = stochastic_reflection(S, d, mk(x, y, z), rs);
      d3 Vj = mk(S.V[3 * j], S.V[3 * j + 1], S.V[3 * j + 2]);
      d3 Wj = mk(S.W[3 * j], S.W[3 * j + 1], S.W[3 * j + 2]);
      d3 vn = add3(add3(u, Vj), cross_ref(Wj, rs));
      d3 dv = sub3(vdump, vn);
      d3 dl = cross_ref(rs, dv);
      ExchAcc *e = S.exch + j;
      exch_add(e, 0, dv.x, &S.ss->err); exch_add(e, 1, dv.y, &S.ss->err); exch_add(e, 2, dv.z, &S.ss->err);
      exch_add(e, 3, dl.x, &S.ss->err); exch_add(e, 4, dl.y, &S.ss->err); exch_add(e, 5, dl.z, &S.ss->err);
      wx = __dmul_rn(vn.x, S.dt); wy = __dmul_rn(vn.y, S.dt); wz = __dmul_rn(vn.z, S.dt);
      wchanged = true;
      // step forward half a substep with the new velocity
      x = ref_mod(__dadd_rn(x, __dmul_rn(wx, 0.5)), S.dx);
      y = ref_mod(__dadd_rn(y, __dmul_rn(wy, 0.5)), S.dy);
      z = ref_mod(__dadd_rn(z, __dmul_rn(wz, 0.5)), S.dz);
      // the cell table is built with a margin; a move beyond it could hide a colloid
      double ex = ref_img(__dsub_rn(x, x0), S.dx), ey = ref_img(__dsub_rn(y, y0), S.dy),
             ez = ref_img(__dsub_rn(z, z0), S.dz);
      if (norm2_ref(ex, ey, ez) > S.disp_margin2) atomicOr(&S.ss->err, ERRB_DISPLACE);
    }
  }
  if (flags & F_SHELL) {
    rec.p = pid;
    rec.n = 0;
    rec.pass = 0;
    it.last = -1;
    for (int j = cand_next(S, it, cbox); j >= 0; j = cand_next(S, it, cbox)) {
      if (!within(S, Xc, Xf[j], j, x, y, z, S.r_shell, S.rsh2)) continue;
      if (rec.n < SHELL_J) rec.j[rec.n++] = (uint16_t)j;
      else atomicOr(&S.ss->err, ERRB_SHELLSLOTS);
    }
  }
}

// |w|^2 * 2^kw from the fixed-point w = wf 2^-kw: wf^2 2^-kw, rounded half up,
// as a 128-bit square on the integer pipe
__device__ __forceinline__ long long sq_fix(long long wf, int kw) {
  unsigned long long a = (unsigned long long)(wf < 0 ? -wf : wf);
  unsigned long long lo = a * a, hi = __umul64hi(a, a);
  unsigned long long lo2 = lo + (1ull << (kw - 1));
  hi += lo2 < lo;
  return (long long)((hi << (64 - kw)) | (lo2 >> kw));
}

// ------------------------------------------------------------- colloid helpers

__device__ __forceinline__ d3 ldv(const double *a, int j) { return mk(a[3 * j], a[3 * j + 1], a[3 * j + 2]); }
__device__ __forceinline__ void stv(double *a, int j, d3 v) { a[3 * j] = v.x; a[3 * j + 1] = v.y; a[3 * j + 2] = v.z; }

// update_activity_direction (cpp/update.cpp:34-46): ra rotated by the Euler matrix
// of Omega dt; then, with Dr > 0, rotational diffusion ra += sqrt(2 Dr dt)
// (xi - (xi.ra) ra), renormalised (xi: three normals drawn for that substep)
__device__ d3 activity(const SysF64 &S, d3 ra, d3 W, d3 xi) {
  d3 b = mul3s(W, S.dt), sb, cb;
  sincos(b.x, &sb.x, &cb.x);
  sincos(b.y, &sb.y, &cb.y);
  sincos(b.z, &sb.z, &cb.z);
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

__device__ __forceinline__ float wrapf(float d, float L) { return d - L * rintf(d / L); }

// WCA force on colloid j at positions Xc (compute_force_md, cpp/update.cpp:14-32):
// partners with r < r_cutoff summed in ascending partner order, which is the
// order the reference's pair loop adds them to f[j].  FP32 prefilter over all
// colloids by the warp; exact FP64 pair terms.  Returns the force in every lane;
// pot receives this colloid's share of the potential (pairs with k > j).
__device__ d3 wca_force(const SysF64 &S, const double *Xc, const float4 *Xf, int j, int lane, bool want_pot,
                        double &pot) {
  d3 f = mk(0, 0, 0);
  pot = 0;
  const float4 xj = Xf[j];
  const float Lx = S.Lxf, Ly = S.Lyf, Lz = S.Lzf;
  const float rcf = S.rcf;
  const d3 Xj = ldv(Xc, j);
  for (int base = 0; base < S.Nc; base += 32) {
    int k = base + lane;
    bool cand = false;
    if (k < S.Nc && k != j) {
      float4 xk = Xf[k];
      float dx = wrapf(xj.x - xk.x, Lx), dy = wrapf(xj.y - xk.y, Ly), dz = wrapf(xj.z - xk.z, Lz);
      cand = dx * dx + dy * dy + dz * dz < rcf * rcf;
    }
    unsigned m = __ballot_sync(FULL, cand);
    if (!m) continue;
    d3 ff = mk(0, 0, 0);
    double pt = 0;
    bool hit = false;
    if (cand) {
      d3 temp = mk(ref_img(__dsub_rn(Xj.x, Xc[3 * k]), S.dx), ref_img(__dsub_rn(Xj.y, Xc[3 * k + 1]), S.dy),
                   ref_img(__dsub_rn(Xj.z, Xc[3 * k + 2]), S.dz));
      double r = __dsqrt_rn(norm2_ref(temp.x, temp.y, temp.z));
      if (r < S.r_cutoff) {
        hit = true;
        double p13 = r, p7 = r;
        for (int i = 1; i < 13; ++i) { p13 = __dmul_rn(p13, r); if (i == 6) p7 = p13; }
        double t1 = __ddiv_rn(S.sig12, p13), t2 = __ddiv_rn(S.sig6, p7);
        double mag = __dsub_rn(__dmul_rn(__dmul_rn(4.0, S.eps), __dsub_rn(__dmul_rn(12.0, t1), __dmul_rn(6.0, t2))), S.fc);
        ff = div3s(mul3s(temp, mag), r);
        if (want_pot && k > j) {
          double q = __ddiv_rn(S.sig_colloid, r);
          pt = __dadd_rn(__dsub_rn(__dmul_rn(__dmul_rn(4.0, S.eps), __dsub_rn(pow(q, 12.0), pow(q, 6.0))), S.ufc),
                         __dmul_rn(S.fc, r));
        }
      }
    }
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
  return f;
}

// Cells of the 342-box block of colloid cell cb (own box excluded) whose box
// comes within `reach` of the colloid position (minimum image, FP32 with margin):
// the cells whose particles can be inside the sphere or the run() shell.
template <typename F>
__device__ void for_reach_cells(const SysF64 &S, int cb, float4 xc, float reach, int lane, F fn) {
  if (cb >= S.C) return;
  int cx = cb % S.Lx, ct = cb / S.Lx, cy = ct % S.Ly, cz = ct / S.Ly;
  const float Lx = S.Lxf, Ly = S.Lyf, Lz = S.Lzf;
  for (int q = lane; q < 343; q += 32) {
    int ox = q % 7 - 3, oy = (q / 7) % 7 - 3, oz = q / 49 - 3;
    if (!ox && !oy && !oz) continue;
    int bx = cx + ox, by = cy + oy, bz = cz + oz;
    bx += bx < 0 ? S.Lx : 0; bx -= bx >= S.Lx ? S.Lx : 0;
    by += by < 0 ? S.Ly : 0; by -= by >= S.Ly ? S.Ly : 0;
    bz += bz < 0 ? S.Lz : 0; bz -= bz >= S.Lz ? S.Lz : 0;
    float ex = fmaxf(fabsf(wrapf(xc.x - ((float)bx + 0.5f), Lx)) - 0.5f, 0.f);
    float ey = fmaxf(fabsf(wrapf(xc.y - ((float)by + 0.5f), Ly)) - 0.5f, 0.f);
    float ez = fmaxf(fabsf(wrapf(xc.z - ((float)bz + 0.5f), Lz)) - 0.5f, 0.f);
    if (ex * ex + ey * ey + ez * ez <= reach * reach) fn(bx + S.Lx * (by + S.Ly * bz));
  }
}

// reach of the cell table of substep e: the run() shell on the last substep of a
// step (its candidates are recorded there), the sphere otherwise
__device__ __forceinline__ float table_reach(const SysF64 &S, long long e) {
  return (e % S.n_sub) == S.n_sub - 1 ? S.rT_shell : S.rT_coll;
}

// Colloid work that the next substep needs and nothing in this substep changes,
// done by the first blocks of a streaming pass while the rest streams the fluid:
// the WCA forces at the positions X_g (compute_force_md) and the cell table of
// substep g+1, built from X_g with a margin for the colloid's own move.
__device__ __noinline__ void colloid_aux(const SysF64 &S, long long g, int j, int lane, bool act) {
  const int b = (int)(g & 1);
  double pot;
  d3 fn = wca_force(S, S.X[b], S.Xf[b], j, lane, false, pot);
  if (lane == 0) stv(S.fnew, j, fn);
  // update_activity_direction of the previous substep: nothing before the end of
  // this step reads the orientation, so it runs here, off the critical path
  if (act && lane == 0) stv(S.ra, j, activity(S, ldv(S.ra, j), ldv(S.W, j), ldv(S.xi, j)));
  if (S.Dr > 0 && lane == 0) {
    // the three standard normals of this substep's rotational diffusion (Box-Muller)
    uint4 r = draw4(S.key, DOM_ROTDIFF, 0, (uint32_t)(j + 1), 0, (uint32_t)g);
    double r0 = sqrt(-2.0 * log(u01(r.x))), r1 = sqrt(-2.0 * log(u01(r.z)));
    double s0, c0, s1, c1;
    sincos(__dmul_rn(S.two_pi, u01(r.y)), &s0, &c0);
    sincos(__dmul_rn(S.two_pi, u01(r.w)), &s1, &c1);
    stv(S.xi, j, mk(__dmul_rn(r0, c0), __dmul_rn(r0, s0), __dmul_rn(r1, c1)));
  }
  const long long e = g + 1;
  unsigned long long *Tc = S.Tcnt[e & 1];
  uint16_t *Tl = S.Tlist[e & 1];
  int *err = &S.ss->err;
  for_reach_cells(S, S.cbox[b][j], S.Xf[b][j], table_reach(S, e), lane,
                  [&](int cell) { tappend(Tc, Tl, cell, e, j, err); });
}

// the exact sums of the SRD binning for the next step: cell number, count, w, |w|^2
__device__ __forceinline__ void bin_for_rotation(const SysF64 &S, int p, double x, double y, double z, double wx,
                                                 double wy, double wz) {
  // (1 + mod(pos + rr, len).cell(len), cpp/rotation_mpcd.cpp:11)
  const double *rr = S.ss->rr;
  double ax = ref_mod(__dadd_rn(x, rr[0]), S.dx), ay = ref_mod(__dadd_rn(y, rr[1]), S.dy),
         az = ref_mod(__dadd_rn(z, rr[2]), S.dz);
  bool alias;
  int c = cell_of_pos(S, ax, ay, az, alias);
  S.rotcell[p] = c;
  long long ax_ = dbits(wx) & 0x7FFFFFFFFFFFFFFFll, ay_ = dbits(wy) & 0x7FFFFFFFFFFFFFFFll,
            az_ = dbits(wz) & 0x7FFFFFFFFFFFFFFFll;
  if (ax_ > S.wlim_bits || ay_ > S.wlim_bits || az_ > S.wlim_bits) atomicOr(&S.ss->err, ERRB_VRANGE);
  long long fx = to_fix(wx, S.kw), fy = to_fix(wy, S.kw), fz = to_fix(wz, S.kw);
  long long f2 = sq_fix(fx, S.kw) + sq_fix(fy, S.kw) + sq_fix(fz, S.kw);
  CellAcc *a = S.acc + c;
  atomicAdd(&a->n, 1);
  atomicAdd((unsigned long long *)&a->sx, (unsigned long long)fx);
  atomicAdd((unsigned long long *)&a->sy, (unsigned long long)fy);
  atomicAdd((unsigned long long *)&a->sz, (unsigned long long)fz);
  atomicAdd((unsigned long long *)&a->s2, (unsigned long long)f2);
}

// FLAGS: F_* bits.  l: substep (1..n_sub) whose streaming this is; 0 for the
// set-up pass (no streaming; bins for the first step).  fb: the fluid buffer.
// The first `naux` blocks do colloid_aux for this substep instead (`act`: with
// the pending orientation update of the previous substep).
//
// Per particle: streaming, then an FP32 scan of the colloids its cell table
// lists.  A particle that may be inside a sphere (or is on the edge of a run()
// shell, or sits in an aliased cell) goes to the event list, which k_events then
// processes with the reference's exact FP64 arithmetic, one event per lane; all
// other particles finish here (shell record, SRD binning on the last substep).
template <int FLAGS>
__global__ void __launch_bounds__(256) k_stream(const SysF64 S, int l, int naux, int act, int fb) {
  constexpr int flags = FLAGS;
  const long long step = S.ss->step;
  const long long gs = step * S.n_sub + (l - 1);
  if ((int)blockIdx.x < naux) {
    const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (j < S.Nc) colloid_aux(S, gs, j, threadIdx.x & 31, act != 0);
    return;
  }
  const Fluid F = fluid_at(S, fb);
  const int p = (blockIdx.x - naux) * blockDim.x + threadIdx.x;
  const bool valid = p < S.N;
  const int buf = (int)(gs & 1);
  bool ev = false;
  unsigned members = 0;  // run() shell members among the cell-table slots
  const uint16_t *lst = nullptr;
  int cnt = 0;
  if (valid) {
    double x = F.x[p], y = F.y[p], z = F.z[p];
    double wx = 0, wy = 0, wz = 0;
    if (flags & (F_STREAM | F_BINROT)) { wx = F.wx[p]; wy = F.wy[p]; wz = F.wz[p]; }
    if (flags & F_STREAM) {
      // update_pos_mpcd: pos = mod(pos + vel*dt, len)   cpp/update.cpp:56-60
      x = ref_mod(__dadd_rn(x, wx), S.dx);
      y = ref_mod(__dadd_rn(y, wy), S.dy);
      z = ref_mod(__dadd_rn(z, wz), S.dz);
    }
    if (flags & (F_COLLIDE | F_SHELL)) {
      bool alias;
      int lin = cell_of_pos(S, x, y, z, alias);
      ev = alias;
      if (!alias) {
        cnt = tcount(S.Tcnt[buf][lin], gs);
        if (cnt > 0) {
          cnt = cnt < TCAP ? cnt : TCAP;
          lst = S.Tlist[buf] + (size_t)lin * TCAP;
          const float4 *Xf = S.Xf[buf];
          const float px = d2f_trunc(x), py = d2f_trunc(y), pz = d2f_trunc(z);
          const float ch = S.r_coll + 1e-3f, sl = S.r_shell - 1e-3f, sh = S.r_shell + 1e-3f;
          for (int k = 0; k < cnt; ++k) {
            float4 c = Xf[lst[k]];
            float dx = wrap_half(c.x - px, S.Lxf), dy = wrap_half(c.y - py, S.Lyf), dz = wrap_half(c.z - pz, S.Lzf);
            float d2 = dx * dx + dy * dy + dz * dz;
            if (flags & F_COLLIDE) ev |= d2 <= ch * ch;
            if (flags & F_SHELL) {
              if (d2 < sl * sl) members |= 1u << k;
              else ev |= d2 <= sh * sh;
            }
          }
        }
      }
    }
    if (!ev && (flags & F_BINROT)) bin_for_rotation(S, p, x, y, z, wx, wy, wz);
    if (flags & F_STREAM) { F.x[p] = x; F.y[p] = y; F.z[p] = z; }
  }
  // block-aggregated appends: events and (last substep) run() candidate records
  __shared__ int s_ev, s_rec, s_evb, s_recb;
  if (threadIdx.x == 0) { s_ev = 0; s_rec = 0; }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const bool has_rec = (flags & F_SHELL) && !ev && members != 0;
  const unsigned mev = __ballot_sync(FULL, ev), mrec = __ballot_sync(FULL, has_rec);
  int oev = 0, orec = 0;
  if (lane == 0) {
    if (mev) oev = atomicAdd(&s_ev, __popc(mev));
    if (mrec) orec = atomicAdd(&s_rec, __popc(mrec));
  }
  oev = __shfl_sync(FULL, oev, 0);
  orec = __shfl_sync(FULL, orec, 0);
  __syncthreads();
  if (threadIdx.x == 0) {
    s_evb = s_ev ? atomicAdd(&S.ss->nevents, s_ev) : 0;
    s_recb = s_rec ? atomicAdd(&S.ss->nshell, s_rec) : 0;
  }
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  if (ev) {
    int i = s_evb + oev + __popc(mev & lt);
    if (i < S.events_cap) S.events[i] = p;
    else atomicOr(&S.ss->err, ERRB_SHELL);
  }
  if (has_rec) {
    int i = s_recb + orec + __popc(mrec & lt);
    if (i < S.shell_cap) {
      // colloids in ascending index, the order run() visits them
      ShellRec *r = S.shell + i;
      r->p = F.id[p];
      r->pass = 0;
      int n = 0, last = -1;
      for (int it = 0; it < cnt && n < SHELL_J; ++it) {
        int best = 0x7FFFFFFF;
        for (int k = 0; k < cnt; ++k) {
          int j = lst[k];
          if (((members >> k) & 1u) && j > last && j < best) best = j;
        }
        if (best == 0x7FFFFFFF) break;
        r->j[n++] = (uint16_t)best;
        last = best;
      }
      if (__popc(members) > SHELL_J) atomicOr(&S.ss->err, ERRB_SHELLSLOTS);
      r->n = (uint8_t)n;
    } else {
      atomicOr(&S.ss->err, ERRB_SHELL);
    }
  }
}

// The particles the streaming pass listed: wall collisions in colloid order with
// the reference's exact arithmetic (and, on the last substep, their run() record
// and SRD binning), one particle per lane so the FP64 work fills whole warps.
template <int FLAGS>
__global__ void __launch_bounds__(128, 4) k_events(const SysF64 S, int l, int fb) {
  constexpr int flags = FLAGS;
  const long long step = S.ss->step;
  const long long gs = step * S.n_sub + (l - 1);
  const int buf = (int)(gs & 1);
  const Fluid F = fluid_at(S, fb);
  const int n = min(S.ss->nevents, S.events_cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int p = S.events[i];
    double x = F.x[p], y = F.y[p], z = F.z[p], wx = F.wx[p], wy = F.wy[p], wz = F.wz[p];
    bool alias, wchanged = false;
    int lin = cell_of_pos(S, x, y, z, alias);
    ShellRec rec;
    rec.n = 0;
    near_colloids(S, flags, F.id[p], lin, alias, gs, buf, x, y, z, wx, wy, wz, wchanged, rec);
    if ((flags & F_SHELL) && rec.n) {
      int idx = atomicAdd(&S.ss->nshell, 1);
      if (idx < S.shell_cap) S.shell[idx] = rec;
      else atomicOr(&S.ss->err, ERRB_SHELL);
    }
    if (flags & F_BINROT) bin_for_rotation(S, p, x, y, z, wx, wy, wz);
    if (flags & F_COLLIDE) { F.x[p] = x; F.y[p] = y; F.z[p] = z; }
    if (wchanged) { F.wx[p] = wx; F.wy[p] = wy; F.wz[p] = wz; }
  }
}

StreamKernel stream_kernel(int flags) {
  switch (flags) {
    case F_STREAM | F_COLLIDE: return k_stream<F_STREAM | F_COLLIDE>;
    case F_STREAM | F_COLLIDE | F_SHELL | F_BINROT: return k_stream<F_STREAM | F_COLLIDE | F_SHELL | F_BINROT>;
    case F_SHELL | F_BINROT: return k_stream<F_SHELL | F_BINROT>;
  }
  return nullptr;
}

EventKernel event_kernel(int flags) {
  switch (flags) {
    case F_STREAM | F_COLLIDE: return k_events<F_COLLIDE>;
    case F_STREAM | F_COLLIDE | F_SHELL | F_BINROT: return k_events<F_COLLIDE | F_SHELL | F_BINROT>;
    case F_SHELL | F_BINROT: return k_events<F_SHELL | F_BINROT>;
  }
  return nullptr;
}

// ------------------------------------------------------------- SRD collision

// Per cell: the SRD collision of rotation_mpcd (cpp/rotation_mpcd.cpp:14-49) as
// one affine map of the cell's displacements, w' = u + s R (w - u) = A w + b,
// A = s R, b = u - A u.  u is the cell mean, R the rotation by theta about the
// cell's random axis (rho, phi), s the thermostat factor; the variance the
// reference computes after rotating equals sum|w - u|^2 = S2 - n|u|^2 before.
// Consumes (and clears) the exact sums k_stream accumulated.
__global__ void __launch_bounds__(256) k_cell_prep(const SysF64 S) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < S.Nc) S.shell_cnt[c] = 0;
  CellAcc a = CellAcc{0, 0, 0, 0, 0, 0};
  if (c < S.Cpad) {
    a = S.acc[c];
    S.acc[c] = CellAcc{0, 0, 0, 0, 0, 0};
    S.cursor[c] = 0;
  }
  // counting sort, first half: exclusive prefix of the occupancy within this block
  // of 256 cells, and the block's total
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
    if (threadIdx.x == 0) S.blk_off[blockIdx.x] = total;
  }
  if (c >= S.C) return;
  double *ab = S.cell_ab + (size_t)c * 12;
  int n = a.n;
  if (n > S.max_per_cell) atomicOr(&S.ss->err, ERRB_OCCUPANCY);
  if (n <= 1 || n > S.max_per_cell) {
    ab[0] = 1; ab[1] = 0; ab[2] = 0; ab[3] = 0; ab[4] = 1; ab[5] = 0; ab[6] = 0; ab[7] = 0; ab[8] = 1;
    ab[9] = 0; ab[10] = 0; ab[11] = 0;
    return;
  }
  const double inv = S.inv_n[n];
  double ux = (double)a.sx * S.inv_sw * inv, uy = (double)a.sy * S.inv_sw * inv, uz = (double)a.sz * S.inv_sw * inv;
  double s2 = (double)a.s2 * S.inv_sw;
  double var = s2 - (double)n * (ux * ux + uy * uy + uz * uz);
  double s = var > 0 ? sqrt(S.cs * (double)(n - 1) / var) : 1.0;
  // rotation axis: rho = 2 ran - 1, phi = 4 asin(1) ran (cpp/rotation_mpcd.cpp:19-20)
  uint4 r = draw4(S.key, DOM_AXIS, 0, (uint32_t)(c + 1), 0, (uint32_t)(S.ss->step + 1));
  double rho = 2.0 * u01(r.x) - 1.0, phi = S.two_pi * u01(r.y);
  double sp, cp;
  sincos(phi, &sp, &cp);
  double sq = sqrt(1.0 - rho * rho);
  double r1 = cp * sq, r2 = sp * sq, r3 = rho;
  double ct = S.ct, st = S.st, ict = S.ict;
  double i1 = ict * r1, i2 = ict * r2, i3 = ict * r3;
  double R[9] = {i1 * r1 + ct, i1 * r2 - st * r3, i1 * r3 + st * r2,
                 i2 * r1 + st * r3, i2 * r2 + ct, i2 * r3 - st * r1,
                 i3 * r1 - st * r2, i3 * r2 + st * r1, i3 * r3 + ct};
#pragma unroll
  for (int k = 0; k < 9; ++k) ab[k] = s * R[k];
  ab[9] = ux - (ab[0] * ux + ab[1] * uy + ab[2] * uz);
  ab[10] = uy - (ab[3] * ux + ab[4] * uy + ab[5] * uz);
  ab[11] = uz - (ab[6] * ux + ab[7] * uy + ab[8] * uz);
}

// counting sort, second half: exclusive prefix of the block totals (one block)
__global__ void __launch_bounds__(1024) k_scan_blocks(const SysF64 S, int nblk) {
  __shared__ int wsum[32];
  __shared__ int carry;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nblk; base += 1024) {
    int i = base + threadIdx.x;
    int v = i < nblk ? S.blk_off[i] : 0, incl = v;
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    int before = carry, total = 0;
    for (int q = 0; q < 32; ++q) {
      before += q < w ? wsum[q] : 0;
      total += wsum[q];
    }
    __syncthreads();
    if (i < nblk) S.blk_off[i] = before + incl - v;
    if (threadIdx.x == 0) carry += total;
    __syncthreads();
  }
}

// The SRD collision applied to each particle, w' = A w + b of its cell, and the
// particle written, rotated, to its slot of the other buffer in cell order (the
// slot within a cell is taken with one atomic per group of equal cells in a warp).
__global__ void __launch_bounds__(256) k_rotate_sort(const SysF64 S, int src, int dst) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= S.N) return;
  const Fluid F = fluid_at(S, src), G = fluid_at(S, dst);
  const int c = S.rotcell[p];
  double wx = F.wx[p], wy = F.wy[p], wz = F.wz[p];
  if (c < S.C) {
    const double2 *ab = reinterpret_cast<const double2 *>(S.cell_ab + (size_t)c * 12);
    double2 a01 = ab[0], a23 = ab[1], a45 = ab[2], a67 = ab[3], a8b0 = ab[4], b12 = ab[5];
    double nx = fma(a01.x, wx, fma(a01.y, wy, fma(a23.x, wz, a8b0.y)));
    double ny = fma(a23.y, wx, fma(a45.x, wy, fma(a45.y, wz, b12.x)));
    double nz = fma(a67.x, wx, fma(a67.y, wy, fma(a8b0.x, wz, b12.y)));
    wx = nx; wy = ny; wz = nz;
  }
  const unsigned act = __activemask();
  const unsigned grp = __match_any_sync(act, c);
  const int lane = threadIdx.x & 31, leader = __ffs(grp) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(&S.cursor[c], __popc(grp));
  base = __shfl_sync(grp, base, leader);
  const int slot = S.blk_off[c >> 8] + S.cell_off[c] + base + __popc(grp & ((1u << lane) - 1u));
  const int id = F.id[p];
  // occupancy and rotcell come from the same binning pass, so slots form a
  // permutation of 0..N-1; anything else is reported, never written
  if (slot < 0 || slot >= S.N || id < 0 || id >= S.N) {
    atomicOr(&S.ss->err, ERRB_OCCUPANCY);
    return;
  }
  G.x[slot] = F.x[p]; G.y[slot] = F.y[p]; G.z[slot] = F.z[p];
  G.wx[slot] = wx; G.wy[slot] = wy; G.wz[slot] = wz;
  G.id[slot] = id;
  S.newpos[id] = slot;
}

// The SRD collision applied in place, w' = A w + b of the particle's cell (the
// steps between two sorts).
__global__ void __launch_bounds__(256) k_rotate(const SysF64 S, int fb) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= S.N) return;
  const int c = S.rotcell[p];
  if (c >= S.C) return;
  const Fluid F = fluid_at(S, fb);
  const double2 *ab = reinterpret_cast<const double2 *>(S.cell_ab + (size_t)c * 12);
  double2 a01 = ab[0], a23 = ab[1], a45 = ab[2], a67 = ab[3], a8b0 = ab[4], b12 = ab[5];
  double wx = F.wx[p], wy = F.wy[p], wz = F.wz[p];
  F.wx[p] = fma(a01.x, wx, fma(a01.y, wy, fma(a23.x, wz, a8b0.y)));
  F.wy[p] = fma(a23.y, wx, fma(a45.x, wy, fma(a45.y, wz, b12.x)));
  F.wz[p] = fma(a67.x, wx, fma(a67.y, wy, fma(a8b0.x, wz, b12.y)));
}

// --------------------------------------------------------------------- run()

// rear-shell test of run() (cpp/run.cpp:17-19) against the kicked colloid
// velocity V + v0 ra, and the shell count per colloid
__global__ void k_run_shell(const SysF64 S, int fb) {
  const int n = min(S.ss->nshell, S.shell_cap);
  const double *Xc = S.X[(int)((S.ss->step * S.n_sub - 1) & 1)];
  const Fluid F = fluid_at(S, fb);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    ShellRec rec = S.shell[i];
    int p = S.newpos[rec.p];
    d3 pos = mk(F.x[p], F.y[p], F.z[p]);
    uint8_t pass = 0;
    for (int k = 0; k < rec.n; ++k) {
      int j = rec.j[k];
      d3 r = mk(ref_img(__dsub_rn(pos.x, Xc[3 * j]), S.dx), ref_img(__dsub_rn(pos.y, Xc[3 * j + 1]), S.dy),
                ref_img(__dsub_rn(pos.z, Xc[3 * j + 2]), S.dz));
      d3 V = add3(mk(S.V[3 * j], S.V[3 * j + 1], S.V[3 * j + 2]),
                  mul3s(mk(S.ra[3 * j], S.ra[3 * j + 1], S.ra[3 * j + 2]), S.v0));
      if (dot_ref(r, V) <= 0) {
        pass |= (uint8_t)(1u << k);
        atomicAdd(&S.shell_cnt[j], 1);
      }
    }
    S.shell[i].pass = pass;
  }
}

// vel_fl -= v0 ra M / (m cnt) for each rear shell the particle is in, in colloid
// order (cpp/run.cpp:20-24)
__global__ void k_run_kick(const SysF64 S, int fb) {
  const int n = min(S.ss->nshell, S.shell_cap);
  const Fluid F = fluid_at(S, fb);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    ShellRec rec = S.shell[i];
    if (!rec.pass) continue;
    int p = S.newpos[rec.p];
    d3 v = mk(__ddiv_rn(F.wx[p], S.dt), __ddiv_rn(F.wy[p], S.dt), __ddiv_rn(F.wz[p], S.dt));
    for (int k = 0; k < rec.n; ++k) {
      if (!((rec.pass >> k) & 1)) continue;
      int j = rec.j[k];
      d3 del = mul3s(mk(S.ra[3 * j], S.ra[3 * j + 1], S.ra[3 * j + 2]), S.v0);
      double f = __ddiv_rn(S.mass_colloid, __dmul_rn(S.mass_fl, (double)S.shell_cnt[j]));
      v = sub3(v, mul3s(del, f));
    }
    F.wx[p] = __dmul_rn(v.x, S.dt); F.wy[p] = __dmul_rn(v.y, S.dt); F.wz[p] = __dmul_rn(v.z, S.dt);
  }
}

// ------------------------------------------------------------------ colloids

__device__ __forceinline__ int colloid_cell(const SysF64 &S, d3 X) {
  bool alias;
  return cell_of_pos(S, X.x, X.y, X.z, alias);
}

// grid shift of the SRD binning the coming streaming pass performs (rotation_mpcd
// of that step draws it first, cpp/rotation_mpcd.cpp:9), keyed by that step
__device__ __forceinline__ void set_shift(const SysF64 &S, long long nn) {
  S.ss->nshell = 0;
  uint4 r = draw4(S.key, DOM_SHIFT, 0, 0, 0, (uint32_t)nn);
  S.ss->rr[0] = u01(r.x) - 0.5; S.ss->rr[1] = u01(r.y) - 0.5; S.ss->rr[2] = u01(r.z) - 0.5;
}

// One thread per colloid.  `l` is the substep (1..n_sub) that M_FINISH / M_ACT
// end, or 0 before the first substep of a step.  With M_ADVANCE the colloid then
// moves to the following substep (update_pos_md, cpp/update.cpp:48-54).  In the
// fused step the orientation update of substeps 1..n-1 runs in the next streaming
// pass instead (colloid_aux), off the critical path.
__global__ void __launch_bounds__(32) k_fin(const SysF64 S, int mode, int l) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const long long step = S.ss->step;
  const long long g = step * S.n_sub + (l - 1);  // substep finished (l >= 1)
  const long long gn = g + 1;                    // substep advanced to
  if (j == 0) {
    S.ss->ev_total += S.ss->nevents;
    S.ss->nevents = 0;  // the event list of the coming streaming pass
    if ((mode & M_ADVANCE) && (gn % S.n_sub) == S.n_sub - 1) set_shift(S, step + 2);  // it bins for the next step
  }
  if (j >= S.Nc) return;
  d3 V = ldv(S.V, j), W = ldv(S.W, j), ra = ldv(S.ra, j), f = ldv(S.f, j);

  if (mode & M_FINISH) {
    // end of fluid_colloid_collision: V += vc m/M, Omega += omega m/I (cpp/fluid_colloid_collision.cpp:46-47)
    ExchAcc e = S.exch[j];
    d3 vc = mk(exch_val(e, 0), exch_val(e, 1), exch_val(e, 2)), om = mk(exch_val(e, 3), exch_val(e, 4), exch_val(e, 5));
    V = add3(V, div3s(mul3s(vc, S.mass_fl), S.mass_colloid));
    W = add3(W, div3s(mul3s(om, S.mass_fl), S.I_colloid));
    // compute_force_md at X_g (done by the streaming pass) and update_velocity_colloid
    d3 fn = ldv(S.fnew, j);
    V = add3(V, mul3s(add3(f, fn), S.dtb2));
    f = fn;
    S.exch[j] = ExchAcc{};
  }
  // update_activity_direction (its noise xi was drawn by the streaming pass)
  if (mode & M_ACT) ra = activity(S, ra, W, ldv(S.xi, j));
  if (mode & M_KICK) V = add3(V, mul3s(ra, S.v0));  // run(): vel_colloid += ra v0 (cpp/run.cpp:13)

  if (mode & M_ADVANCE) {
    // update_pos_md (cpp/update.cpp:48-54)
    const int cur = (int)(g & 1), nxt = (int)(gn & 1);
    d3 Xo = ldv(S.X[cur], j);
    d3 Xn = add3(Xo, add3(mul3s(V, S.dt), mul3s(f, S.ddt)));
    Xn = mk(ref_mod(Xn.x, S.dx), ref_mod(Xn.y, S.dy), ref_mod(Xn.z, S.dz));
    // the cell table of gn was built from Xo with a margin for this move
    double ex = ref_img(Xn.x - Xo.x, S.dx), ey = ref_img(Xn.y - Xo.y, S.dy), ez = ref_img(Xn.z - Xo.z, S.dz);
    if (ex * ex + ey * ey + ez * ez > S.cmargin2) atomicOr(&S.ss->err, ERRB_DISPLACE);
    stv(S.X[nxt], j, Xn);
    S.Xf[nxt][j] = make_float4((float)Xn.x, (float)Xn.y, (float)Xn.z, 0.f);
    S.cbox[nxt][j] = colloid_cell(S, Xn);
  }
  stv(S.V, j, V); stv(S.W, j, W); stv(S.ra, j, ra); stv(S.f, j, f);
}

// Set-up (the prologue of main, cpp/active_brownian.cpp:93-96): forces at the
// current positions (compute_force_md), the cell table for the run() candidates
// of the first step (substep g0-1) and the table of the first substep g0.
__global__ void __launch_bounds__(128) k_colloid_setup(const SysF64 S) {
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long step = S.ss->step;
  const long long g0 = step * S.n_sub;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    set_shift(S, step + 1);
    S.ss->nevents = 0;
  }
  if (j >= S.Nc) return;
  const int b = (int)((g0 - 1) & 1);
  double pot;
  d3 fn = wca_force(S, S.X[b], S.Xf[b], j, lane, false, pot);
  if (lane == 0) stv(S.f, j, fn);
  int *err = &S.ss->err;
  const int cb = S.cbox[b][j];
  const float4 xc = S.Xf[b][j];
  for_reach_cells(S, cb, xc, S.rT_shell, lane,
                  [&](int cell) { tappend(S.Tcnt[b], S.Tlist[b], cell, g0 - 1, j, err); });
  for_reach_cells(S, cb, xc, table_reach(S, g0), lane,
                  [&](int cell) { tappend(S.Tcnt[b ^ 1], S.Tlist[b ^ 1], cell, g0, j, err); });
}

// WCA potential of the current configuration, per colloid (pairs k > j), for the
// diagnostics (cpp/update.cpp:23)
__global__ void __launch_bounds__(128) k_colloid_pot(const SysF64 S) {
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (j >= S.Nc) return;
  const int b = (int)((S.ss->step * S.n_sub - 1) & 1);
  double pot;
  wca_force(S, S.X[b], S.Xf[b], j, lane, true, pot);
  if (lane == 0) S.pot_part[j] = pot;
}

// completes a step: bumps the step counter
__global__ void k_end_step(const SysF64 S) {
  if (threadIdx.x == 0 && blockIdx.x == 0) S.ss->step += 1;
}

// fluid diagnostics from the exact cell sums of the last binning: per block the
// sums of S(w) (3), S(|w|^2) and the count, as doubles, in a fixed order
__global__ void __launch_bounds__(256) k_diag_fluid(const SysF64 S, double *part) {
  __shared__ double sh[5][256];
  double a[5] = {0, 0, 0, 0, 0};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < S.Cpad; c += gridDim.x * blockDim.x) {
    CellAcc q = S.acc[c];
    a[0] += (double)q.sx * S.inv_sw; a[1] += (double)q.sy * S.inv_sw; a[2] += (double)q.sz * S.inv_sw;
    a[3] += (double)q.s2 * S.inv_sw; a[4] += (double)q.n;
  }
  for (int k = 0; k < 5; ++k) sh[k][threadIdx.x] = a[k];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int k = 0; k < 5; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 5; ++k) part[blockIdx.x * 5 + k] = sh[k][0];
}

}  // namespace bgb
