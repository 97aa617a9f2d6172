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
#include "../../include/brownian_gb300.h"
#include "device.cuh"

namespace bgb {
// One particle's part of the SRD binning for the next step: its cell (recorded
// in rotcell) and the fixed-point w and |w|^2 the exact cell sums add up
struct BinTerm {
  int c;
  long long fx, fy, fz, f2;
};

// (rr: the grid shift of that binning)
__device__ __forceinline__ BinTerm bin_term(const SysF64 &S, const double *rr, int p, double x, double y, double z,
                                            double wx, double wy, double wz) {
  // (1 + mod(pos + rr, len).cell(len), cpp/rotation_mpcd.cpp:11)
  double ax = ref_mod(__dadd_rn(x, rr[0]), S.dx), ay = ref_mod(__dadd_rn(y, rr[1]), S.dy),
         az = ref_mod(__dadd_rn(z, rr[2]), S.dz);
  bool alias;
  BinTerm t;
  t.c = cell_of_pos(S, ax, ay, az, alias);
  S.rotcell[p] = t.c;
  long long ax_ = dbits(wx) & 0x7FFFFFFFFFFFFFFFll, ay_ = dbits(wy) & 0x7FFFFFFFFFFFFFFFll,
            az_ = dbits(wz) & 0x7FFFFFFFFFFFFFFFll;
  if (ax_ > S.wlim_bits || ay_ > S.wlim_bits || az_ > S.wlim_bits) atomicOr(&S.ss->err, ERRB_VRANGE);
  t.fx = to_fix(wx, S.kw); t.fy = to_fix(wy, S.kw); t.fz = to_fix(wz, S.kw);
  t.f2 = sq_fix(t.fx, S.kw) + sq_fix(t.fy, S.kw) + sq_fix(t.fz, S.kw);
  return t;
}

// the exact sums of the SRD binning for the next step: cell number, count, w, |w|^2
__device__ __forceinline__ void bin_for_rotation(const SysF64 &S, int p, double x, double y, double z, double wx,
                                                 double wy, double wz) {
  const BinTerm t = bin_term(S, S.ss->rr, p, x, y, z, wx, wy, wz);
  bin_add(S.acc + t.c, 1, t.fx, t.fy, t.fz, t.f2);
}

// FLAGS: F_* bits.  l: substep (1..n_sub) whose streaming this is; 0 for the
// set-up pass (no streaming; bins for the first step).  fb: the fluid buffer.
//
// Per particle: streaming, then an FP32 scan of the colloids its cell table
// lists.  A particle that may be inside a sphere (or is on the edge of a run()
// shell, or sits in an aliased cell) goes to the event list, which k_events then
// processes with the reference's exact FP64 arithmetic, one event per lane; all
// other particles finish here (shell record, SRD binning on the last substep).
// U particles per thread (thread t of block b: particles b * 256 U + t + 256 u),
// their loads issued together so more memory requests are in flight.  The pass
// that also lists run() shell members keeps more state per particle and one
// particle per thread, for its register count.
#ifndef STREAM64_U
#define STREAM64_U 2
#endif
#ifndef STREAM64_U_SHELL
#define STREAM64_U_SHELL 1
#endif
static constexpr __host__ __device__ int stream64_u(int flags) { return (flags & F_SHELL) ? STREAM64_U_SHELL : STREAM64_U; }
// One chunk of 256 U particles: i = chunk * 256 U + threadIdx.x + 256 u below `count`,
// slot i of the fluid (NEAR false) or slot near[i] (NEAR true: the free-flight schedule's
// passes over the near list).  The whole block calls it.
template <int FLAGS, bool NEAR>
static __device__ __forceinline__ void stream64_chunk(const SysF64 &S, const int chunk, const int count, int l,
                                                      int fb) {
  constexpr int flags = FLAGS;
  constexpr int U = stream64_u(FLAGS);
  const long long step = S.ss->step;
  const long long gs = step * S.n_sub + (l - 1);
  const Fluid F = fluid_at(S, fb);
  const int i0 = chunk * (256 * U) + threadIdx.x;
  const int buf = (int)(gs & 1);
  // F_PIPE: the colloid positions of the previous substep (this substep's are being
  // computed meanwhile) and the displacement bound as margin; pending particles
  // belong to the event passes and are skipped
  const int xb = (flags & F_PIPE) ? (int)((gs - 1) & 1) : buf;
  const float mg = (flags & F_PIPE) ? S.ss->cm : 0.f;

  double x[U], y[U], z[U], wx[U], wy[U], wz[U];
  bool valid[U], ev[U];
  unsigned members[U];  // run() shell members among the cell-table slots
  int cnt[U], lin[U], pp[U];
  uint8_t pd[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int i = i0 + 256 * u;
    valid[u] = i < count;
    ev[u] = false;
    members[u] = 0;
    cnt[u] = 0;
    lin[u] = 0;
    pd[u] = 0;
    pp[u] = i;
    wx[u] = wy[u] = wz[u] = 0;
    if (valid[u]) {
      const int p = NEAR ? S.near[i] : i;
      pp[u] = p;
      x[u] = F.x[p]; y[u] = F.y[p]; z[u] = F.z[p];
      if (flags & (F_STREAM | F_BINROT | F_COLLIDE)) { wx[u] = F.wx[p]; wy[u] = F.wy[p]; wz[u] = F.wz[p]; }
      if (flags & F_PIPE) pd[u] = S.pend[p];
    }
  }
#pragma unroll
  for (int u = 0; u < U; ++u) valid[u] = valid[u] && pd[u] == 0;
#pragma unroll
  for (int u = 0; u < U; ++u) {
    if (!valid[u]) continue;
    if (flags & F_STREAM) {
      // update_pos_mpcd: pos = mod(pos + vel*dt, len)   cpp/update.cpp:56-60
      x[u] = ref_mod(__dadd_rn(x[u], wx[u]), S.dx);
      y[u] = ref_mod(__dadd_rn(y[u], wy[u]), S.dy);
      z[u] = ref_mod(__dadd_rn(z[u], wz[u]), S.dz);
    }
    if (flags & (F_COLLIDE | F_SHELL)) {
      bool alias;
      lin[u] = cell_of_pos(S, x[u], y[u], z[u], alias);
      ev[u] = alias;
      if (!alias) cnt[u] = tcount(S.Tcnt[buf][lin[u]], gs);
    }
  }
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int u = 0; u < U; ++u) {
    if (valid[u] && (flags & (F_COLLIDE | F_SHELL)) && cnt[u] > 0) {
      cnt[u] = cnt[u] < TCAP ? cnt[u] : TCAP;
      const uint16_t *lst = S.Tlist[buf] + (size_t)lin[u] * TCAP;
      const float4 *Xf = S.Xf[xb];
      const float px = d2f_trunc(x[u]), py = d2f_trunc(y[u]), pz = d2f_trunc(z[u]);
      const float ch = S.r_coll + 1e-3f + mg, sl = S.r_shell - 1e-3f - mg, sh = S.r_shell + 1e-3f + mg;
      for (int k = 0; k < cnt[u]; ++k) {
        const float4 c = Xf[lst[k]];
        const float dx = wrap_half(c.x - px, S.Lxf), dy = wrap_half(c.y - py, S.Lyf), dz = wrap_half(c.z - pz, S.Lzf);
        const float d2 = dx * dx + dy * dy + dz * dz;
        if (flags & F_COLLIDE) ev[u] |= d2 <= ch * ch;
        if (flags & F_SHELL) {
          if (d2 < sl * sl) members[u] |= 1u << k;
          else ev[u] |= d2 <= sh * sh;
        }
      }
    }
    const int p = pp[u];
    if (valid[u]) {
      if (!ev[u] && (flags & F_BINROT)) bin_for_rotation(S, p, x[u], y[u], z[u], wx[u], wy[u], wz[u]);
      if (flags & F_STREAM) { F.x[p] = x[u]; F.y[p] = y[u]; F.z[p] = z[u]; }
    }
    // the event record, one atomic per warp (no block barrier), written while the
    // particle's state is still in registers
    const unsigned mev = __ballot_sync(FULL, ev[u]);
    int bev = 0;
    if (lane == 0 && mev) bev = atomicAdd(&S.ss->nnew[buf], __popc(mev));
    bev = __shfl_sync(FULL, bev, 0);
    if (ev[u]) {
      const int i = bev + __popc(mev & lt);
      if (i < S.events_cap) {
        EventRec r;
        r.xy = make_double2(x[u], y[u]); r.zwx = make_double2(z[u], wx[u]); r.wywz = make_double2(wy[u], wz[u]);
        r.p = p; r.id = F.id[p];
        S.newrec[buf][i] = r;
        if (flags & F_PIPE) S.pend[p] = 1;
      } else {
        atomicOr(&S.ss->err, ERRB_EVENTS);
      }
    }
  }
  // run() candidate records (last substep), one atomic per block
#pragma unroll
  for (int u = 0; u < U; ++u) {
    if (!(flags & F_SHELL)) break;
    const int p = pp[u];
    const bool has_rec = valid[u] && !ev[u] && members[u] != 0;
    const unsigned mrec = __ballot_sync(FULL, has_rec);
    const int brec = block_base(&S.ss->nshell, mrec, lane);
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
  }
}

// Five blocks per SM (48 registers, a few spilled to L1) measured faster than four
// without spills.
template <int FLAGS>
__global__ void __launch_bounds__(256, 5) k_stream(const SysF64 S, int l, int fb) {
  stream64_chunk<FLAGS, false>(S, blockIdx.x, S.N, l, fb);
}

// the same over the near list of the free-flight schedule (grid-stride over chunks)
template <int FLAGS>
__global__ void __launch_bounds__(256, 5) k_stream_near(const SysF64 S, int l, int fb) {
  const int count = S.ss->nnear;
  constexpr int per = 256 * stream64_u(FLAGS);
  for (int chunk = blockIdx.x; chunk * per < count; chunk += gridDim.x)
    stream64_chunk<FLAGS, true>(S, chunk, count, l, fb);
}

int stream64_per_thread(int flags) { return stream64_u(flags); }

// The particles the streaming pass listed: wall collisions in colloid order with
// the reference's exact arithmetic (and, on the last substep, their run() record
// and SRD binning).  Per round of up to blockDim.x particles (one per thread):
// each thread loads its particle and finds its first collision; then the block's
// collisions are gathered onto its first threads, rank by rank (a particle's
// second collision follows its first), and each particle is finished by its own
// thread.  blockDim.x <= 128.
template <int FLAGS>
static __device__ __forceinline__ void k_events_body(const SysF64 &S, const int VB, const int NVB, int l, int fb) {
  constexpr int flags = FLAGS;
  __shared__ EvState sst[128];
  __shared__ int stask[128];
  __shared__ int sntask;
  __shared__ CollScratch scs[32];
  const long long step = S.ss->step;
  const long long gs = step * S.n_sub + (l - 1);
  const int buf = (int)(gs & 1);
  const Fluid F = fluid_at(S, fb);
  // F_PIPE: items 0..np-1 are the particles pending from earlier substeps of this
  // step (their streaming of this substep is done here), items np.. the ones this
  // substep's streaming pass listed; every item's state goes back to prec[i]
  const int nn = min(S.ss->nnew[buf], S.events_cap);
  const int np = (flags & F_PIPE) ? S.ss->npend : 0;
  int n = np + nn;
  if ((flags & F_PIPE) && n > S.pend_cap) {
    if (VB == 0 && threadIdx.x == 0) atomicOr(&S.ss->err, ERRB_EVENTS);
    n = S.pend_cap;
  }
  // item i goes to block i % NVB: the items of a substep spread over all SMs
  EvState &st = sst[threadIdx.x];
  for (int base = 0;; base += blockDim.x) {
    const int i = VB + NVB * (threadIdx.x + base);
    const bool valid = i < n;
    if (!__syncthreads_or(valid)) break;  // block-uniform trip count
    const bool old = i < np;
    st.j = -1;
    if (valid) {
      const EventRec r = old ? S.prec[i] : S.newrec[buf][i - np];
      double x = r.xy.x, y = r.xy.y, z = r.zwx.x;
      const double wx = r.zwx.y, wy = r.wywz.x, wz = r.wywz.y;
      if ((flags & F_PIPE) && old) {
        // update_pos_mpcd of a pending particle (as the streaming pass does it)
        x = ref_mod(__dadd_rn(x, wx), S.dx);
        y = ref_mod(__dadd_rn(y, wy), S.dy);
        z = ref_mod(__dadd_rn(z, wz), S.dz);
      }
      bool alias;
      const int lin = cell_of_pos(S, x, y, z, alias);
      int cnt = 0;
      if (!alias) {
        cnt = tcount(S.Tcnt[buf][lin], gs);
        cnt = cnt < TCAP ? cnt : TCAP;
      }
      st.x = x; st.y = y; st.z = z; st.wx = wx; st.wy = wy; st.wz = wz;
      st.x0 = x; st.y0 = y; st.z0 = z;
      st.vdx = st.vdy = st.vdz = 0.0;
      st.p = r.p; st.id = r.id; st.lin = lin; st.last = -1; st.cnt = cnt;
      st.alias = alias; st.dumped = false; st.changed = false;
      if (flags & F_COLLIDE) st.j = ev_next_hit(S, st, buf);
    }
    if (flags & F_COLLIDE) {
      for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) sntask = 0;
        __syncthreads();
        if (st.j >= 0) stask[atomicAdd(&sntask, 1)] = threadIdx.x;
        __syncthreads();
        const int nt = sntask;
        if (nt == 0) break;
        if (blockDim.x == 128) {
          for (int k0 = 0; k0 < nt; k0 += 32) ev_collide_coop(S, sst, stask, k0, nt, gs, buf, scs);
          if ((int)threadIdx.x < nt) {
            EvState &t = sst[stask[threadIdx.x]];
            t.j = ev_next_hit(S, t, buf);
          }
        } else if ((int)threadIdx.x < nt) {
          EvState &t = sst[stask[threadIdx.x]];
          ev_collide(S, t, t.j, gs, buf);
          t.j = ev_next_hit(S, t, buf);
        }
      }
    }
    __syncthreads();
    if (valid) {
      const int p = st.p;
      if (flags & F_SHELL) {
        ShellRec rec;
        ev_shell(S, st, buf, rec);
        if (rec.n) {
          int idx = atomicAdd(&S.ss->nshell, 1);
          if (idx < S.shell_cap) S.shell[idx] = rec;
          else atomicOr(&S.ss->err, ERRB_SHELL);
        }
      }
      if (flags & F_BINROT) bin_for_rotation(S, p, st.x, st.y, st.z, st.wx, st.wy, st.wz);
      if ((flags & F_PIPE) || st.changed) {
        F.x[p] = st.x; F.y[p] = st.y; F.z[p] = st.z;
        F.wx[p] = st.wx; F.wy[p] = st.wy; F.wz[p] = st.wz;
      }
      if (flags & F_PIPE) {
        EventRec o;
        o.xy = make_double2(st.x, st.y); o.zwx = make_double2(st.z, st.wx); o.wywz = make_double2(st.wy, st.wz);
        o.p = p; o.id = st.id;
        S.prec[i] = o;
      }
    }
    __syncthreads();  // the next round reuses the shared state
  }
}

template <int FLAGS>
__global__ void __launch_bounds__(128) k_events(const SysF64 S, int l, int fb) {
  k_events_body<FLAGS>(S, blockIdx.x, gridDim.x, l, fb);
}

// the event pass (blocks 0..nevb-1) and, after them, the colloid side work of the same
// substep (colloid_aux: forces and orientation, two colloids per block of four warps),
// which needs only the positions the colloid finish of the substep before computed: one
// launch where the side work would take a second stream per substep
template <int FLAGS>
__global__ void __launch_bounds__(128) k_events_aux(const SysF64 S, int l, int fb, int nevb, int act) {
  if ((int)blockIdx.x < nevb) {
    k_events_body<FLAGS>(S, blockIdx.x, nevb, l, fb);
    return;
  }
  const int j = 2 * ((int)blockIdx.x - nevb) + (threadIdx.x >> 6);
  const long long gs = S.ss->step * S.n_sub + (l - 1);
  if (j < S.Nc) colloid_aux(S, gs, j, act != 0, (threadIdx.x >> 5) & 1, 2, S.vlist != 0);
}

// The SRD binning of the particles the last streaming pass of a step finished
// (the pending ones are binned by the event pass): a pass of its own, so that
// its atomics run beside that substep's event pass and colloid finish.  Pending
// marks stay set until the next step's rotation clears them.
// Particles sit in cell order (sorted every sort_every steps), so a warp's particles
// fall into a few cells of the shifted grid: their terms are summed per cell across the
// warp first (bin_add_warp), one set of atomics per cell and warp.
__global__ void __launch_bounds__(256) k_bin(const SysF64 S, int fb) {
  const Fluid F = fluid_at(S, fb);
  for (int base = blockIdx.x * blockDim.x; base < S.N; base += gridDim.x * blockDim.x) {
    const int p = base + threadIdx.x;
    BinTerm t{-1, 0, 0, 0, 0};
    if (p < S.N && !S.pend[p]) t = bin_term(S, S.ss->rr, p, F.x[p], F.y[p], F.z[p], F.wx[p], F.wy[p], F.wz[p]);
    bin_add_warp(S.acc, t.c, t.fx, t.fy, t.fz, t.f2);
  }
}

// ------------------------------------------------------------ free-flight schedule
// (the FP64 form's kernels; the schedule and the flight table are described with the FP32
// form's, kernels_fp32c.cu)

// the last substep's binning of the near particles the streaming pass finished (pending
// ones are binned by the event pass)
__global__ void __launch_bounds__(256) k_bin_near(const SysF64 S, int fb) {
  const Fluid F = fluid_at(S, fb);
  const int count = S.ss->nnear;
  for (int base = blockIdx.x * blockDim.x; base < count; base += gridDim.x * blockDim.x) {
    const int i = base + threadIdx.x;
    BinTerm t{-1, 0, 0, 0, 0};
    if (i < count) {
      const int p = S.near[i];
      if (!S.pend[p]) t = bin_term(S, S.ss->rr, p, F.x[p], F.y[p], F.z[p], F.wx[p], F.wy[p], F.wz[p]);
    }
    bin_add_warp(S.acc, t.c, t.fx, t.fy, t.fz, t.f2);
  }
}

// rotation_mpcd of one particle (w' = A w + b of its cell, as k_rotate; ROT false: a
// counting-sort step, whose scatter rotated it) and its classification against the flight
// table: a near particle is flagged and listed (one atomic per block).
template <bool ROT>
__global__ void __launch_bounds__(256) k_rotate_classify(const SysF64 S, int fb) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = p < S.N;
  const Fluid F = fluid_at(S, fb);
  const long long step = S.ss->step;
  const int b0 = (int)((step * S.n_sub - 1) & 1);
  bool near = false;
  if (valid) {
    S.pend[p] = 0;  // no particle is pending at the start of a step
    const int c = ROT ? S.rotcell[p] : S.C;
    double wx = F.wx[p], wy = F.wy[p], wz = F.wz[p];
    const float px = d2f_trunc(F.x[p]), py = d2f_trunc(F.y[p]), pz = d2f_trunc(F.z[p]);
    int cx = (int)px, cy = (int)py, cz = (int)pz;  // positions in (0, L]: L is cell 0
    cx -= cx == S.Lx ? S.Lx : 0; cy -= cy == S.Ly ? S.Ly : 0; cz -= cz == S.Lz ? S.Lz : 0;
    // a position outside the box (a state that is not finite) reads no table: near
    const bool inb = cx >= 0 && cx < S.Lx && cy >= 0 && cy < S.Ly && cz >= 0 && cz < S.Lz;
    const FlightCell *fc = S.ftab + (inb ? cx + S.Lx * (cy + S.Ly * cz) : 0);
    const uint4 w0 = reinterpret_cast<const uint4 *>(fc)[0], w1 = reinterpret_cast<const uint4 *>(fc)[1];
    if (c < S.C) {
      const double2 *ab = reinterpret_cast<const double2 *>(S.cell_ab + (size_t)c * 12);
      double2 a01 = ab[0], a23 = ab[1], a45 = ab[2], a67 = ab[3], a8b0 = ab[4], b12 = ab[5];
      const double nx = fma(a01.x, wx, fma(a01.y, wy, fma(a23.x, wz, a8b0.y)));
      const double ny = fma(a23.y, wx, fma(a45.x, wy, fma(a45.y, wz, b12.x)));
      const double nz = fma(a67.x, wx, fma(a67.y, wy, fma(a8b0.x, wz, b12.y)));
      wx = nx; wy = ny; wz = nz;
      F.wx[p] = wx; F.wy[p] = wy; F.wz[p] = wz;
    }
    // n_sub |w| = ndt |v| (FP32 copies by truncation, on the integer pipe: below 2^-23 of
    // the travel under it, which the slack covers)
    const float fx = d2f_trunc(wx), fy = d2f_trunc(wy), fz = d2f_trunc(wz);
    const float travel = (float)S.n_sub * sqrtf(fx * fx + fy * fy + fz * fz);
    const int cnt = tcount(((unsigned long long)w0.y << 32) | w0.x, step);
    if (!inb || !(travel <= S.flight_rv) || cnt > FLIGHT_CAP) {
      near = true;  // faster than the table allows (or not finite), or a crowded cell
    } else if (cnt > 0) {
      const float r = S.r_shell + travel + (float)S.n_sub * S.ss->cm + 0.01f, r2 = r * r;
      const unsigned ids[6] = {w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
      const float4 *Xf = S.Xf[b0];
      for (int k = 0; k < cnt; ++k) {
        const int j = (int)((ids[k >> 1] >> (16 * (k & 1))) & 0xFFFFu);
        const float4 q = Xf[j];
        const float dx = wrap_half(q.x - px, S.Lxf), dy = wrap_half(q.y - py, S.Lyf), dz = wrap_half(q.z - pz, S.Lzf);
        near = near || !(dx * dx + dy * dy + dz * dz > r2);
      }
    }
    S.fnear[p] = near ? 1 : 0;
  }
  const int lane = threadIdx.x & 31;
  const unsigned m = __ballot_sync(FULL, near);
  const int base = block_base_n(&S.ss->nnear, __popc(m), lane);
  if (near) S.near[base + __popc(m & ((1u << lane) - 1u))] = p;
}

// n substeps of update_pos_mpcd along one axis for a free particle: x = mod(x + w, L) n
// times (cpp/update.cpp:56-60), with the result of the additions one by one.  x > 0 has
// the unit u = ulp(x) of its binade [2^e, 2^(e+1)); w/u = Mw 2^-s (Mw the significand of w).
// While an exact sum x + w lies inside that binade, the nearest double to it is x plus the
// multiple of u nearest to w, k u with k = round(Mw 2^-s), the same k at every addition
// unless w/u is exactly halfway between two integers (then ties-to-even would depend on x).
// So while the results x + j k u stay at least u inside the binade (the exact sums then lie
// inside it) and inside [2^-30 L, L), where mod is the identity, j additions give x + j k u,
// built here on the integer pipe from the bits (the FP64 units stay free for the substeps'
// chains).  free_stream takes such a run of steps, then the one addition that crosses a
// binade or the box edge as the reference does it (mod(x + w, L) in FP64), then the next run
// from the new x (a few crossings at most; a coordinate crosses one in a few per cent of the
// steps of a step); on a tie, or past the crossings it allows, the additions one by one.

// the largest j in [0, left] with j step <= room (step > 0; room < 2^53 and left <= 2^10, so
// no product below overflows once step <= room)
static __device__ __forceinline__ int seg_steps(long long room, long long step, int left) {
  if (room < step) return 0;
  if ((long long)left * step <= room) return left;
  int j = (int)((float)room / (float)step);  // within one of the quotient (j < left < 2^23)
  j = j < 0 ? 0 : (j > left ? left : j);
  while (j < left && (long long)(j + 1) * step <= room) ++j;
  while (j > 0 && (long long)j * step > room) --j;
  return j;
}

// a run of up to `left` integer steps from x: false where the step does not apply (then x
// is left as it is); else *j steps taken (0 when x sits at the edge it moves towards)
static __device__ __forceinline__ bool free_run(double &x, double w, int left, const Dim &D, int *j) {
  const long long bx = dbits(x), bw = dbits(w);
  const long long aw = bw & 0x7FFFFFFFFFFFFFFFll;
  const int ex = (int)((bx >> 52) & 0x7FF), ew = (int)((aw >> 52) & 0x7FF);
  if (!(bx >= D.lo_bits && bx < D.L_bits && ex > 0 && (aw == 0 || ew > 0))) return false;
  long long k = 0;
  if (aw != 0) {
    const long long mw = (aw & 0xFFFFFFFFFFFFFll) | 0x10000000000000ll;
    const int sh = ex - ew;
    if (sh <= 0) {
      if (sh <= -8) return false;  // (a w that large leaves the binade at once)
      k = mw << -sh;
    } else if (sh <= 53) {
      k = mw >> sh;
      const long long rem = mw & ((1ll << sh) - 1), half = 1ll << (sh - 1);
      if (rem == half) return false;  // a tie
      k += rem > half ? 1 : 0;
    }  // sh > 53: |w| < u/2, every sum rounds back to x (k = 0)
    if (bw < 0) k = -k;
  }
  if (left < 1 || left > 1024) return false;
  const long long mx = (bx & 0xFFFFFFFFFFFFFll) | 0x10000000000000ll;
  const long long lo = 0x10000000000000ll + 1, hi = 0x20000000000000ll - 1;
  int n;
  if (k == 0) {
    n = left;
  } else if (k > 0) {
    long long room = hi - mx;  // inside the binade, and below L where L lies in it
    if ((int)((D.L_bits >> 52) & 0x7FF) == ex) {
      const long long rl = ((D.L_bits & 0xFFFFFFFFFFFFFll) | 0x10000000000000ll) - 1 - mx;
      room = rl < room ? rl : room;
    }
    n = seg_steps(room, k, left);
  } else {
    long long room = mx - lo;  // inside the binade, and at or above 2^-30 L where it lies in it
    if ((int)((D.lo_bits >> 52) & 0x7FF) == ex) {
      const long long rl = mx - ((D.lo_bits & 0xFFFFFFFFFFFFFll) | 0x10000000000000ll);
      room = rl < room ? rl : room;
    }
    n = seg_steps(room, -k, left);
  }
  if (n > 0) x = __longlong_as_double(((long long)ex << 52) | ((mx + (long long)n * k) & 0xFFFFFFFFFFFFFll));
  *j = n;
  return true;
}

static __device__ __forceinline__ double free_stream(double x, double w, int n, const Dim &D) {
  for (int seg = 0; seg < 3 && n > 0; ++seg) {
    int j;
    if (!free_run(x, w, n, D, &j)) break;
    n -= j;
    if (n == 0) return x;
    x = ref_mod(__dadd_rn(x, w), D);  // the crossing step, as the reference does it
    n -= 1;
  }
  for (; n > 0; --n) x = ref_mod(__dadd_rn(x, w), D);
  return x;
}

// the free particles' whole step: update_pos_mpcd of every substep (free_stream: the
// streaming passes' operations in order, or their exact result) and the binning of the
// last substep with the next step's grid shift, beside the near particles' substeps,
// which touch none of its particles.  A grid of a few blocks per SM walks the fluid (it
// shares the SMs with the substeps' latency-bound chain).
__global__ void __launch_bounds__(256) k_free_flight(const SysF64 S, int fb) {
  const Fluid F = fluid_at(S, fb);
  for (int p0 = blockIdx.x * blockDim.x; p0 < S.N; p0 += gridDim.x * blockDim.x) {
    const int p = p0 + threadIdx.x;
    BinTerm t{-1, 0, 0, 0, 0};
    if (p < S.N && !S.fnear[p]) {
      const double wx = F.wx[p], wy = F.wy[p], wz = F.wz[p];
      const double x = free_stream(F.x[p], wx, S.n_sub, S.dx), y = free_stream(F.y[p], wy, S.n_sub, S.dy),
                   z = free_stream(F.z[p], wz, S.n_sub, S.dz);
      t = bin_term(S, S.ss->rrn, p, x, y, z, wx, wy, wz);
      F.x[p] = x; F.y[p] = y; F.z[p] = z;
    }
    bin_add_warp(S.acc, t.c, t.fx, t.fy, t.fz, t.f2);  // the whole warp
  }
}

EventAuxKernel event_aux_kernel(int flags) {
  switch (flags) {
    case F_STREAM | F_COLLIDE | F_PIPE: return k_events_aux<F_COLLIDE | F_PIPE>;
    case F_STREAM | F_COLLIDE | F_SHELL | F_BINROT | F_PIPE: return k_events_aux<F_COLLIDE | F_SHELL | F_BINROT | F_PIPE>;
  }
  return nullptr;
}

ClassifyKernel classify_kernel(bool rotate) { return rotate ? k_rotate_classify<true> : k_rotate_classify<false>; }

StreamKernel stream_kernel_near(int flags) {
  switch (flags) {
    case F_STREAM | F_COLLIDE | F_PIPE: return k_stream_near<F_STREAM | F_COLLIDE | F_PIPE>;
    case F_STREAM | F_COLLIDE | F_SHELL | F_BINROT | F_PIPE:
      return k_stream_near<F_STREAM | F_COLLIDE | F_SHELL | F_PIPE>;
  }
  return nullptr;
}

StreamKernel stream_kernel(int flags) {
  // substeps run overlapped (F_PIPE; the last one's binning is k_bin); the set-up
  // pass stands alone; the routine-by-routine substep streams (F_STREAM) and tests
  // for wall collisions (F_COLLIDE) in passes of their own
  switch (flags) {
    case F_STREAM | F_COLLIDE | F_PIPE: return k_stream<F_STREAM | F_COLLIDE | F_PIPE>;
    case F_STREAM | F_COLLIDE | F_SHELL | F_BINROT | F_PIPE:
      return k_stream<F_STREAM | F_COLLIDE | F_SHELL | F_PIPE>;
    case F_SHELL | F_BINROT: return k_stream<F_SHELL | F_BINROT>;
    case F_STREAM: return k_stream<F_STREAM>;
    case F_COLLIDE: return k_stream<F_COLLIDE>;
  }
  return nullptr;
}

// colloid_aux of substep l (1..n_sub) as a kernel of its own (blocks of
// S.aux_nw warps, one colloid each); `act`: with the pending orientation update
// of substep l-1
static __device__ __forceinline__ void k_aux_body(const SysF64 &S, const int VB, const int NVB, int l, int act,
                                                  bool vlist = false) {
  const long long gs = S.ss->step * S.n_sub + (l - 1);
  if ((int)VB < S.Nc) colloid_aux(S, gs, VB, act != 0, threadIdx.x >> 5, S.aux_nw, vlist);
}

// (vl: the forces from the step's pair list, the free-flight schedule)
__global__ void __launch_bounds__(256) k_aux(__grid_constant__ const SysF64 S, int l, int act, int vl) {
  k_aux_body(S, blockIdx.x, gridDim.x, l, act, vl != 0);
}

// the same over a batch of systems (persistent: batch_for)
__global__ void __launch_bounds__(256) k_aux_b(const SysF64 *Ss, const int *boff, int nrep, int l, int act) {
  __shared__ SysF64 sS;
  batch_for(Ss, boff, nrep, sS, [&](int VB, int NVB) { k_aux_body(sS, VB, NVB, l, act); });
}

EventKernel event_kernel(int flags) {
  switch (flags) {
    case F_STREAM | F_COLLIDE | F_PIPE: return k_events<F_COLLIDE | F_PIPE>;
    case F_STREAM | F_COLLIDE | F_SHELL | F_BINROT | F_PIPE: return k_events<F_COLLIDE | F_SHELL | F_BINROT | F_PIPE>;
    case F_SHELL | F_BINROT: return k_events<F_SHELL | F_BINROT>;
    case F_COLLIDE: return k_events<F_COLLIDE>;
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
  // (sx 2^-kw) / n in one product: the power-of-two scaling is exact, so this is the same
  // rounding of the same exact product
  const double insw = S.insw_n[n];
  double ux = (double)a.sx * insw, uy = (double)a.sy * insw, uz = (double)a.sz * insw;
  double s2 = (double)a.s2 * S.inv_sw;
  double var = s2 - (double)n * (ux * ux + uy * uy + uz * uz);
  // sqrt(cs (n - 1) / var) as sqrt(cs (n - 1)) (per n, from the host) times 1/sqrt(var): within
  // a few ulp of the quotient's root, and no double division on the FP64 pipe
  double s = var > 0 ? S.sqcs_n[n] * rsqrt(var) : 1.0;
  // rotation axis: rho = 2 ran - 1, phi = 4 asin(1) ran (cpp/rotation_mpcd.cpp:19-20); the sine
  // and cosine of phi = pi (2 ran) from sincospi (2 ran is exact), within an ulp of sincos(phi)
  uint4 r = draw4(S.key, DOM_AXIS, 0, (uint32_t)(c + 1), 0, (uint32_t)(S.ss->step + 1));
  double rho = pm1(r.x);
  double sp, cp;
  sincospi(2.0 * u01(r.y), &sp, &cp);
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
static __device__ __forceinline__ void k_scan_blocks_body(const SysF64 &S, const int VB, const int NVB, int nblk) {
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

__global__ void __launch_bounds__(1024) k_scan_blocks(__grid_constant__ const SysF64 S, int nblk) {
  k_scan_blocks_body(S, blockIdx.x, gridDim.x, nblk);
}

// the same over a batch of systems (persistent: batch_for)
__global__ void __launch_bounds__(1024) k_scan_blocks_b(const SysF64 *Ss, const int *boff, int nrep, int nblk) {
  __shared__ SysF64 sS;
  // each system's own block count
  batch_for(Ss, boff, nrep, sS, [&](int VB, int NVB) { k_scan_blocks_body(sS, VB, NVB, (sS.Cpad + 255) / 256); });
}

// The SRD collision applied to each particle, w' = A w + b of its cell, and the
// particle written, rotated, to its slot of the other buffer in cell order (the
// slot within a cell is taken with one atomic per group of equal cells in a warp).
__global__ void __launch_bounds__(256) k_rotate_sort(const SysF64 S, int src, int dst) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= S.N) return;
  S.pend[p] = 0;  // no particle is pending at the start of a step
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
  S.pend[p] = 0;  // no particle is pending at the start of a step
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
    // v = w (1/dt): within an ulp of w / dt, without a double division per component
    d3 v = mk(__dmul_rn(F.wx[p], S.inv_dt), __dmul_rn(F.wy[p], S.inv_dt), __dmul_rn(F.wz[p], S.inv_dt));
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

// colloid position as integer cell + FP32 offset (the FP32 form's coordinates)
__device__ __forceinline__ void colloid_q(const SysF64 &S, int b, int j, d3 X) {
  double v[3] = {X.x, X.y, X.z};
  const int L[3] = {S.Lx, S.Ly, S.Lz};
  float c[3], o[3];
  for (int k = 0; k < 3; ++k) {
    double f = floor(v[k]);
    float of = (float)(v[k] - f);
    int ci = (int)f;
    if (of >= 1.f) { of = 0.f; ci += 1; }
    ci %= L[k];
    if (ci < 0) ci += L[k];
    c[k] = (float)ci;
    o[k] = of;
  }
  S.Xcq[b][j] = make_float4(c[0], c[1], c[2], 0.f);
  S.Xco[b][j] = make_float4(o[0], o[1], o[2], 0.f);
}

// grid shift of the SRD binning the coming streaming pass performs (rotation_mpcd
// of that step draws it first, cpp/rotation_mpcd.cpp:9), keyed by that step
__device__ __forceinline__ void set_shift(const SysF64 &S, long long nn) {
  S.ss->nshell = 0;
  double rr[3];
  shift_of(S, nn, rr);
  for (int k = 0; k < 3; ++k) {
    S.ss->rr[k] = rr[k];
    S.ss->rrf[k] = (float)rr[k];
  }
}

// One warp per colloid (warp w of block b holds colloid b + gridDim.x * w), its
// vector components on separate lanes so the FP64 latency chains run side by
// side: lane k < 3 the linear component k (V, f, X), lane 3 + k the angular
// component k (Omega); the orientation update draws the three sines and cosines
// on lanes 0-2.  `l` is the substep (1..n_sub) that M_FINISH / M_ACT end, or 0
// before the first substep of a step.  With M_ADVANCE the colloid then moves to
// the following substep (update_pos_md, cpp/update.cpp:48-54).  In the fused step
// the orientation update of substeps 1..n-1 runs in the next streaming pass
// instead (colloid_aux), off the critical path.
static __device__ __forceinline__ void k_fin_colloid(const SysF64 &S, int j, int lane, int mode, long long g,
                                                     long long gn);

static __device__ __forceinline__ void k_fin_body(const SysF64 &S, const int VB, const int NVB, int mode, int l) {
  const int lane = threadIdx.x & 31;
  // with fin_table a block per colloid (warp 0 the colloid, all warps its cell
  // table), else a warp per colloid
  const int j = S.fin_table ? VB : VB + NVB * (threadIdx.x >> 5);
  const long long step = S.ss->step;
  const long long g = step * S.n_sub + (l - 1);  // substep finished (l >= 1)
  const long long gn = g + 1;                    // substep advanced to
  if (VB == 0 && threadIdx.x == 0) {
    if (S.precision == MPCD_FP64) {
      // the list substep g's streaming pass filled has been taken over by the event
      // pass (into the pending list, empty again after the last substep); its
      // buffer serves substep g+2.  The grid shift of the next step's binning is
      // drawn two substeps ahead: the last streaming pass bins with it and runs
      // beside the finish of the substep before it.
      const int b = (int)(g & 1);
      const int nn = S.ss->nnew[b];
      S.ss->ev_total += nn;
      S.ss->nnew[b] = 0;
      if (mode & M_FINISH) {
        const int np = S.ss->npend + (nn < S.events_cap ? nn : S.events_cap);
        S.ss->npend = l >= S.n_sub ? 0 : (np < S.pend_cap ? np : S.pend_cap);
      }
      const int ahead = S.n_sub >= 2 ? S.n_sub - 2 : 0;
      if ((mode & M_ADVANCE) && (gn % S.n_sub) == ahead) set_shift(S, step + 2);
    } else {
      S.ss->ev_total += S.ss->nevents;
      S.ss->nevents = 0;  // the event list of the coming streaming pass
      if ((mode & M_ADVANCE) && (gn % S.n_sub) == S.n_sub - 1) set_shift(S, step + 2);  // it bins for the next step
    }
  }
  if (j >= S.Nc) return;  // (j is the block's or the warp's)
  if (!S.fin_table) {
    if (lane < 6) k_fin_colloid(S, j, lane, mode, g, gn);
    return;
  }
  if (threadIdx.x < 6) k_fin_colloid(S, j, lane, mode, g, gn);
  if (mode & M_ADVANCE) {
    // the cell table of substep gn+1 from the new position, by the whole block: the
    // streaming pass of gn+1 then needs this kernel only, not the side kernel of gn
    __syncthreads();
    const int nxt = (int)(gn & 1);
    const long long e = gn + 1;
    unsigned long long *Tc = S.Tcnt[e & 1];
    uint16_t *Tl = S.Tlist[e & 1];
    int *err = &S.ss->err;
    for_reach_cells(S, S.cbox[nxt][j], S.Xf[nxt][j], table_reach(S, e), threadIdx.x, blockDim.x,
                    [&](int cell) { tappend(Tc, Tl, cell, e, j, err); });
  }
}

// the per-colloid part of k_fin on lanes 0-5
static __device__ __forceinline__ void k_fin_colloid(const SysF64 &S, int j, int lane, int mode, long long g,
                                                     long long gn) {
  const unsigned grp = 0x3Fu;  // lanes 0-5
  const int k = lane < 3 ? lane : lane - 3;
  const bool lin = lane < 3;
  double v = lin ? S.V[3 * j + k] : S.W[3 * j + k];
  double f = lin ? S.f[3 * j + k] : 0.0;

  if (mode & (M_FINISH | M_COLL)) {
    // end of fluid_colloid_collision: V += vc m/M, Omega += omega m/I (cpp/fluid_colloid_collision.cpp:46-47)
    ExchAcc *e = S.exch + j;
    const double x = __dadd_rn((double)e->hi[lane] * 0x1p-20, (double)e->lo[lane] * 0x1p-72);
    e->hi[lane] = 0;
    e->lo[lane] = 0;
    const double dp = __dmul_rn(x, S.mass_fl);
    S.xacc[6 * j + lane] += dp;  // the exchange record (mpcd_exchange_read)
    v = __dadd_rn(v, __dmul_rn(dp, lin ? S.inv_mc : S.inv_ic));  // (within an ulp of dp / M)
    if (lin && (mode & M_FINISH)) {
      // compute_force_md at X_g (done by the streaming pass) and update_velocity_colloid
      const double fn = S.fnew[3 * j + k];
      v = __dadd_rn(v, __dmul_rn(__dadd_rn(f, fn), S.dtb2));
      f = fn;
    }
  }
  double ra = lin ? S.ra[3 * j + k] : 0.0;
  if (mode & M_ACT) {
    // update_activity_direction (its noise xi was drawn by the streaming pass):
    // Omega moves to lanes 0-2, each takes one sine and cosine, all gather them
    const double w = __shfl_sync(grp, v, lin ? lane + 3 : lane);
    double s = 0, co = 0;
    if (lin) sincos_small(__dmul_rn(w, S.dt), &s, &co);
    const d3 sb = mk(__shfl_sync(grp, s, 0), __shfl_sync(grp, s, 1), __shfl_sync(grp, s, 2));
    const d3 cb = mk(__shfl_sync(grp, co, 0), __shfl_sync(grp, co, 1), __shfl_sync(grp, co, 2));
    const d3 r3 = mk(__shfl_sync(grp, ra, 0), __shfl_sync(grp, ra, 1), __shfl_sync(grp, ra, 2));
    if (lin) {
      const d3 rn = activity_rot(S, r3, sb, cb, ldv(S.xi, j));
      ra = k == 0 ? rn.x : (k == 1 ? rn.y : rn.z);
    }
  }
  if (!lin) {
    S.W[3 * j + k] = v;
    return;
  }
  if (mode & M_KICK) v = __dadd_rn(v, __dmul_rn(ra, S.v0));  // run(): vel_colloid += ra v0 (cpp/run.cpp:13)

  if (mode & M_ADVANCE) {
    // update_pos_md (cpp/update.cpp:48-54)
    const int cur = (int)(g & 1), nxt = (int)(gn & 1);
    const Dim &D = k == 0 ? S.dx : (k == 1 ? S.dy : S.dz);
    const double xo = S.X[cur][3 * j + k];
    const double xn = ref_mod(__dadd_rn(xo, __dadd_rn(__dmul_rn(v, S.dt), __dmul_rn(f, S.ddt))), D);
    // the cell table of gn was built from Xo with a margin for this move
    const double ex = ref_img(__dsub_rn(xn, xo), D);
    const unsigned g3 = 0x7u;
    const double e2 = __dmul_rn(ex, ex);
    const double d2 = __shfl_sync(g3, e2, 0) + __shfl_sync(g3, e2, 1) + __shfl_sync(g3, e2, 2);
    const d3 Xn = mk(__shfl_sync(g3, xn, 0), __shfl_sync(g3, xn, 1), __shfl_sync(g3, xn, 2));
    S.X[nxt][3 * j + k] = xn;
    if (k == 0) {
      if (d2 > S.ss->cm2) atomicOr(&S.ss->err, ERRB_DISPLACE);
      S.Xf[nxt][j] = make_float4((float)Xn.x, (float)Xn.y, (float)Xn.z, 0.f);
      S.cbox[nxt][j] = colloid_cell(S, Xn);
      colloid_q(S, nxt, j, Xn);
    }
  }
  S.V[3 * j + k] = v;
  S.f[3 * j + k] = f;
  S.ra[3 * j + k] = ra;
}

__global__ void __launch_bounds__(256) k_fin(__grid_constant__ const SysF64 S, int mode, int l) {
  k_fin_body(S, blockIdx.x, gridDim.x, mode, l);
}

// the same over a batch of systems (persistent: batch_for)
__global__ void __launch_bounds__(128) k_fin_b(const SysF64 *Ss, const int *boff, int nrep, int mode, int l) {
  __shared__ SysF64 sS;
  batch_for(Ss, boff, nrep, sS, [&](int VB, int NVB) { k_fin_body(sS, VB, NVB, mode, l); });
}

// Set-up (the prologue of main, cpp/active_brownian.cpp:17-20): forces at the
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
    S.ss->nnew[0] = S.ss->nnew[1] = 0;
    S.ss->npend = 0;
    S.ss->cm = S.cmarginf;  // the static bound until a step has measured the colloids
    S.ss->cm2 = S.cmargin2;
  }
  if (j >= S.Nc) return;
  const int b = (int)((g0 - 1) & 1);
  double pot;
  d3 fn = wca_force(S, S.X[b], S.Xf[b], j, lane, false, pot);
  if (lane == 0) {
    stv(S.f, j, fn);
    colloid_q(S, b, j, ldv(S.X[b], j));
  }
  int *err = &S.ss->err;
  const int cb = S.cbox[b][j];
  const float4 xc = S.Xf[b][j];
  for_reach_cells(S, cb, xc, S.rT_shell, lane, 32,
                  [&](int cell) { tappend(S.Tcnt[b], S.Tlist[b], cell, g0 - 1, j, err); });
  for_reach_cells(S, cb, xc, table_reach(S, g0), lane, 32,
                  [&](int cell) { tappend(S.Tcnt[b ^ 1], S.Tlist[b ^ 1], cell, g0, j, err); });
}

// WCA potential of the configuration in position buffer b, per colloid (pairs k > j),
// for the diagnostics (cpp/update.cpp:24)
__global__ void __launch_bounds__(128) k_colloid_pot(const SysF64 S, int b) {
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (j >= S.Nc) return;
  double pot;
  wca_force(S, S.X[b], S.Xf[b], j, lane, true, pot);
  if (lane == 0) S.pot_part[j] = pot;
}

// completes a step: bumps the step counter
static __device__ __forceinline__ void k_end_step_body(const SysF64 &S, const int VB, const int NVB) {
  if (VB != 0) return;
  // run()'s shell counts start from zero for the next step (its rear-shell test runs beside
  // the next step's cell pass, so the cell pass cannot clear them)
  for (int j = threadIdx.x; j < S.Nc; j += blockDim.x) S.shell_cnt[j] = 0;
  if (S.Nc > 0) {
    // the next step's colloid margin: twice the largest displacement a substep gives at
    // the colloids' present speeds, within [0.005, the static bound], and never below the
    // move the FP64 form's next first streaming pass assumes (from the last substep's
    // positions to the present ones, already checked against this step's margin; from the
    // FP32 copies of the positions, plus 2e-5 for their rounding).  A colloid that moves
    // further in a substep fails the step (the finish checks every move), so the FP32
    // form's free-flight classification may take n_sub times it as the colloids' move.
    __shared__ float s_vm[32], s_dm[32];
    const long long g = (S.ss->step + 1) * S.n_sub;  // the substep the colloids are at
    const float4 *Fc = S.Xf[g & 1], *Fp = S.Xf[(g - 1) & 1];
    float vm = 0.f, dm = 0.f;
    for (int j = threadIdx.x; j < S.Nc; j += blockDim.x) {
      const float vx = (float)S.V[3 * j], vy = (float)S.V[3 * j + 1], vz = (float)S.V[3 * j + 2];
      vm = fmaxf(vm, vx * vx + vy * vy + vz * vz);
      const float4 a = Fc[j], b = Fp[j];
      const float ex = wrapf(a.x - b.x, S.Lxf), ey = wrapf(a.y - b.y, S.Lyf), ez = wrapf(a.z - b.z, S.Lzf);
      dm = fmaxf(dm, ex * ex + ey * ey + ez * ez);
    }
    for (int o = 16; o > 0; o >>= 1) {
      vm = fmaxf(vm, __shfl_xor_sync(0xFFFFFFFFu, vm, o));
      dm = fmaxf(dm, __shfl_xor_sync(0xFFFFFFFFu, dm, o));
    }
    const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0) {
      s_vm[w] = vm;
      s_dm[w] = dm;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int k = 1; k < nw; ++k) {
        vm = fmaxf(vm, s_vm[k]);
        dm = fmaxf(dm, s_dm[k]);
      }
      float cm = fminf(fmaxf(2.f * (float)S.dt * sqrtf(vm), 0.005f), S.cmarginf);
      cm = fmaxf(cm, sqrtf(dm) + 2e-5f);
      S.ss->cm = cm;
      S.ss->cm2 = (double)cm * (double)cm;
    }
  }
  if (threadIdx.x == 0) S.ss->step += 1;
}

__global__ void k_end_step(__grid_constant__ const SysF64 S) {
  k_end_step_body(S, blockIdx.x, gridDim.x);
}

// the same over a batch of systems (persistent: batch_for)
__global__ void k_end_step_b(const SysF64 *Ss, const int *boff, int nrep) {
  __shared__ SysF64 sS;
  batch_for(Ss, boff, nrep, sS, [&](int VB, int NVB) { k_end_step_body(sS, VB, NVB); });
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

// error bits of every system of a batch, for one read-back
__global__ void k_gather_err(const SysF64 *Ss, int nrep, int *out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nrep) out[r] = Ss[r].ss->err;
}

}  // namespace bgb
