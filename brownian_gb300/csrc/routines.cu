// Kernels of the routine-by-routine substep: each reference routine of the substep
// body (cpp/active_brownian.cpp:28-37) as a launch sequence of its own, for callers
// that drive the routines one at a time (include/brownian_gb300.h, mpcd_update_pos_md
// ... mpcd_update_velocity_colloid).  The fused step (mpcd_step) does the same work in
// fewer, overlapped passes; both give the same bits.
//
//   neighbour_list_md   k_cbucket + k_nlist: the colloid pair list (cpp/neighbour_list.cpp:27-39)
//                       rebuilt from a bucket grid of cells at least the list radius wide
//   compute_force_md    k_force_list: WCA forces over the list (cpp/update.cpp:14-32)
//   neighbour_list_mpcd k_table (the fluid-to-colloid cell table at the present colloid
//                       positions) + k_box_bin / k_no_neigh (the reference's box binning
//                       and candidate counts, cpp/neighbour_list.cpp:41-58, as observables)
//   update_activity_direction  k_act_now (cpp/update.cpp:34-46)
//   update_velocity_colloid    k_vel_colloid (cpp/update.cpp:62-67)
// update_pos_md, update_pos_mpcd and fluid_colloid_collision reuse the kernels of the
// fused step (k_fin, k_stream, k_events) with other flags.
#include "device.cuh"

namespace bgb {

static __device__ __forceinline__ int bucket_axis(double x, double bs, int nb) {
  int i = (int)(x / bs);
  return i < 0 ? 0 : (i >= nb ? nb - 1 : i);
}

static __device__ __forceinline__ int bucket_of(const double *Xc, int j, const NListGeo &g) {
  const int bx = bucket_axis(Xc[3 * j], g.bs[0], g.nb[0]), by = bucket_axis(Xc[3 * j + 1], g.bs[1], g.nb[1]),
            bz = bucket_axis(Xc[3 * j + 2], g.bs[2], g.nb[2]);
  return bx + g.nb[0] * (by + g.nb[1] * bz);
}

// The colloids by bucket (a counting sort, one block of 1024 threads): bkt_start[b]
// the first slot of bucket b in bkt_list, bkt_start[nbk] = Nc.
// (Xc null: the positions at the start of the present step, the free-flight schedule's list)
__global__ void __launch_bounds__(1024) k_cbucket(const SysF64 S, const double *Xc, NListGeo geo) {
  __shared__ int wsum[32];
  __shared__ int carry;
  if (!Xc) Xc = S.X[(int)((S.ss->step * S.n_sub - 1) & 1)];
  const int nbk = geo.nb[0] * geo.nb[1] * geo.nb[2];
  for (int b = threadIdx.x; b <= nbk; b += blockDim.x) S.bkt_start[b] = 0;
  __syncthreads();
  for (int j = threadIdx.x; j < S.Nc; j += blockDim.x) atomicAdd(&S.bkt_start[bucket_of(Xc, j, geo)], 1);
  __syncthreads();
  // exclusive prefix over nbk + 1 counts, 1024 at a time
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base <= nbk; base += 1024) {
    const int i = base + threadIdx.x;
    const int v = i <= nbk ? S.bkt_start[i] : 0;
    int incl = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(FULL, incl, o);
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
    if (i <= nbk) {
      S.bkt_start[i] = before + incl - v;
      if (i < nbk) S.bkt_cur[i] = before + incl - v;
    }
    if (threadIdx.x == 0) carry += total;
    __syncthreads();
  }
  for (int j = threadIdx.x; j < S.Nc; j += blockDim.x) {
    const int slot = atomicAdd(&S.bkt_cur[bucket_of(Xc, j, geo)], 1);
    if (slot >= 0 && slot < S.Nc) S.bkt_list[slot] = j;
  }
}

// The pair list of colloid j (one warp per colloid, four per block): every colloid k
// != j with |img(X_j - X_k)|^2 < r2 (the reference's test, cpp/neighbour_list.cpp:33-34,
// evaluated in its order of operations), from the buckets next to j's (all buckets of
// an axis with fewer than three), sorted ascending by a rank sort in shared memory.
__global__ void __launch_bounds__(128) k_nlist(const SysF64 S, const double *Xc, NListGeo geo) {
  __shared__ uint16_t sbuf[4][NBR_CAP];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int j = blockIdx.x * 4 + w;
  if (j >= S.Nc) return;
  const d3 Xj = ldv(Xc, j);
  const int b0[3] = {bucket_axis(Xj.x, geo.bs[0], geo.nb[0]), bucket_axis(Xj.y, geo.bs[1], geo.nb[1]),
                     bucket_axis(Xj.z, geo.bs[2], geo.nb[2])};
  int lo[3], cnt3[3];
  for (int a = 0; a < 3; ++a) {
    if (geo.nb[a] >= 3) {
      lo[a] = b0[a] - 1;
      cnt3[a] = 3;
    } else {
      lo[a] = 0;
      cnt3[a] = geo.nb[a];
    }
  }
  uint16_t *buf = sbuf[w];
  int n = 0;
  bool over = false;
  for (int oz = 0; oz < cnt3[2]; ++oz)
    for (int oy = 0; oy < cnt3[1]; ++oy)
      for (int ox = 0; ox < cnt3[0]; ++ox) {
        int bx = lo[0] + ox, by = lo[1] + oy, bz = lo[2] + oz;
        bx += bx < 0 ? geo.nb[0] : 0; bx -= bx >= geo.nb[0] ? geo.nb[0] : 0;
        by += by < 0 ? geo.nb[1] : 0; by -= by >= geo.nb[1] ? geo.nb[1] : 0;
        bz += bz < 0 ? geo.nb[2] : 0; bz -= bz >= geo.nb[2] ? geo.nb[2] : 0;
        const int b = bx + geo.nb[0] * (by + geo.nb[1] * bz);
        const int e0 = S.bkt_start[b], e1 = S.bkt_start[b + 1];
        for (int e = e0; e < e1; e += 32) {
          const int i = e + lane;
          bool in = false;
          int k = 0;
          if (i < e1) {
            k = S.bkt_list[i];
            if (k != j) {
              const double tx = ref_img(__dsub_rn(Xj.x, Xc[3 * k]), S.dx),
                           ty = ref_img(__dsub_rn(Xj.y, Xc[3 * k + 1]), S.dy),
                           tz = ref_img(__dsub_rn(Xj.z, Xc[3 * k + 2]), S.dz);
              in = norm2_ref(tx, ty, tz) < geo.r2;
            }
          }
          const unsigned m = __ballot_sync(FULL, in);
          const int slot = n + __popc(m & ((1u << lane) - 1u));
          if (in) {
            if (slot < NBR_CAP) buf[slot] = (uint16_t)k;
            else over = true;
          }
          n += __popc(m);
        }
      }
  if (__any_sync(FULL, over) && lane == 0) atomicOr(&S.ss->err, ERRB_NBR);
  n = n < NBR_CAP ? n : NBR_CAP;
  __syncwarp();
  uint16_t *out = S.nbr + (size_t)j * NBR_CAP;
  for (int e = lane; e < n; e += 32) {
    const uint16_t v = buf[e];
    int rank = 0;
    for (int q = 0; q < n; ++q) rank += buf[q] < v;
    out[rank] = v;
  }
  if (lane == 0) S.nbr_n[j] = n;
}

// The free-flight schedule's pair list of colloid j (one warp per colloid, four per
// block): every colloid k != j with |img(X_j - X_k)|^2 < r2 at the positions at the start
// of the step, ascending, for the forces of the step's substeps.  The candidates of the
// buckets next to j's are flattened across the warp (a prefix over the buckets' counts), so
// a colloid takes a round per 32 candidates instead of a round per bucket.
__global__ void __launch_bounds__(128) k_nlist_step(const SysF64 S, NListGeo geo) {
  __shared__ uint16_t sbuf[4][NBR_CAP];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int j = blockIdx.x * 4 + w;
  if (j >= S.Nc) return;
  const double *Xc = S.X[(int)((S.ss->step * S.n_sub - 1) & 1)];
  const d3 Xj = ldv(Xc, j);
  const int b0[3] = {bucket_axis(Xj.x, geo.bs[0], geo.nb[0]), bucket_axis(Xj.y, geo.bs[1], geo.nb[1]),
                     bucket_axis(Xj.z, geo.bs[2], geo.nb[2])};
  int lo[3], cnt3[3];
  for (int a = 0; a < 3; ++a) {
    if (geo.nb[a] >= 3) {
      lo[a] = b0[a] - 1;
      cnt3[a] = 3;
    } else {
      lo[a] = 0;
      cnt3[a] = geo.nb[a];
    }
  }
  const int nbb = cnt3[0] * cnt3[1] * cnt3[2];  // buckets to visit (<= 27), one per lane
  int start = 0, cnt = 0;
  if (lane < nbb) {
    int bx = lo[0] + lane % cnt3[0], by = lo[1] + (lane / cnt3[0]) % cnt3[1], bz = lo[2] + lane / (cnt3[0] * cnt3[1]);
    bx += bx < 0 ? geo.nb[0] : 0; bx -= bx >= geo.nb[0] ? geo.nb[0] : 0;
    by += by < 0 ? geo.nb[1] : 0; by -= by >= geo.nb[1] ? geo.nb[1] : 0;
    bz += bz < 0 ? geo.nb[2] : 0; bz -= bz >= geo.nb[2] ? geo.nb[2] : 0;
    const int b = bx + geo.nb[0] * (by + geo.nb[1] * bz);
    start = S.bkt_start[b];
    cnt = S.bkt_start[b + 1] - start;
  }
  int incl = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += t;
  }
  const int total = __shfl_sync(FULL, incl, 31);
  const int excl = incl - cnt;
  uint16_t *buf = sbuf[w];
  int n = 0;
  bool over = false;
  for (int t0 = 0; t0 < total; t0 += 32) {
    const int t = t0 + lane;
    // the bucket q holding candidate t: the last lane whose exclusive prefix is <= t
    int q = 0;
    for (int r = 1; r < nbb; ++r) q = __shfl_sync(FULL, excl, r) <= t ? r : q;
    const int sq = __shfl_sync(FULL, start, q), eq = __shfl_sync(FULL, excl, q);
    bool in = false;
    int k = 0;
    if (t < total) {
      k = S.bkt_list[sq + (t - eq)];
      if (k != j) {
        const double tx = ref_img(__dsub_rn(Xj.x, Xc[3 * k]), S.dx), ty = ref_img(__dsub_rn(Xj.y, Xc[3 * k + 1]), S.dy),
                     tz = ref_img(__dsub_rn(Xj.z, Xc[3 * k + 2]), S.dz);
        in = norm2_ref(tx, ty, tz) < geo.r2;
      }
    }
    const unsigned m = __ballot_sync(FULL, in);
    const int slot = n + __popc(m & ((1u << lane) - 1u));
    if (in) {
      if (slot < NBR_CAP) buf[slot] = (uint16_t)k;
      else over = true;
    }
    n += __popc(m);
  }
  if (__any_sync(FULL, over) && lane == 0) atomicOr(&S.ss->err, ERRB_NBR);
  n = n < NBR_CAP ? n : NBR_CAP;
  __syncwarp();
  uint16_t *out = S.nbr + (size_t)j * NBR_CAP;
  for (int e = lane; e < n; e += 32) {
    const uint16_t v = buf[e];
    int rank = 0;
    for (int q = 0; q < n; ++q) rank += buf[q] < v;
    out[rank] = v;
  }
  if (lane == 0) S.nbr_n[j] = n;
}

// compute_force_md over the pair list: f of every colloid (its old value was saved as
// old_force by update_pos_md) and each colloid's share of the potential (pairs k > j)
__global__ void __launch_bounds__(128) k_force_list(const SysF64 S, const double *Xc) {
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.x * 4 + (threadIdx.x >> 5);
  if (j >= S.Nc) return;
  double pot;
  const d3 f = wca_force_list(S, Xc, j, lane, true, pot);
  if (lane == 0) {
    stv(S.f, j, f);
    S.pot_part[j] = pot;
  }
}

// update_activity_direction of substep l: the substep's rotational-diffusion normals,
// then the orientation turned by Omega dt (one colloid per block of 32, lanes 0-2)
__global__ void __launch_bounds__(32) k_act_now(const SysF64 S, int l) {
  const int j = blockIdx.x, k = threadIdx.x;
  if (j >= S.Nc || k >= 3) return;
  const unsigned grp = 0x7u;
  const long long g = S.ss->step * S.n_sub + (l - 1);
  if (S.Dr > 0) rotdiff_draw(S, g, j, k, grp);
  __syncwarp(grp);
  activity_apply(S, j, k, grp);
}

// The fused FP64 substeps leave the particles they could not clear "pending" (their
// streaming done by later event passes, their state in F and in prec).  A substep run
// routine by routine streams and tests every particle itself, so it first returns the
// pending ones to the ordinary particles (F holds their present state).  One block.
__global__ void __launch_bounds__(256) k_unpend(const SysF64 S) {
  const int np = min(S.ss->npend, S.pend_cap);
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    const int p = S.prec[i].p;
    if (p >= 0 && p < S.N) S.pend[p] = 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) S.ss->npend = 0;
}

// update_velocity_colloid: V += (old_force + f) dt / (2 M), one thread per component
__global__ void __launch_bounds__(128) k_vel_colloid(const SysF64 S) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * S.Nc) return;
  S.V[i] = __dadd_rn(S.V[i], __dmul_rn(__dadd_rn(S.fold[i], S.f[i]), S.dtb2));
}

// The fluid-to-colloid cell table of substep l at the colloid positions of that
// substep (its entries cleared by the caller), one block per colloid
__global__ void __launch_bounds__(256) k_table(const SysF64 S, int l) {
  const int j = blockIdx.x;
  if (j >= S.Nc) return;
  const long long g = S.ss->step * S.n_sub + (l - 1);
  const int b = (int)(g & 1);
  int *err = &S.ss->err;
  for_reach_cells(S, S.cbox[b][j], S.Xf[b][j], table_reach(S, g), threadIdx.x, blockDim.x,
                  [&](int cell) { tappend(S.Tcnt[b], S.Tlist[b], cell, g, j, err); });
}

// The reference's box binning of neighbour_list_mpcd (cpp/neighbour_list.cpp:44-47):
// per particle id its 1-based box number 1 + cell(pos) (cpp/parameters.hpp:59), per box
// its occupancy (occ[box], box 1 .. Cpad)
__global__ void __launch_bounds__(256) k_box_bin(const SysF64 S, int fb, int *cell_of, int *occ) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= S.N) return;
  const Fluid F = fluid_at(S, fb);
  bool alias;
  const int c = cell_of_pos(S, F.x[p], F.y[p], F.z[p], alias) + 1;
  cell_of[F.id[p]] = c;
  atomicAdd(&occ[c], 1);
}

// per colloid, its candidate count no_neigh (cpp/neighbour_list.cpp:48-57): the
// occupancy of the 342 boxes around its own (create_box, cpp/neighbour_list.cpp:12-25;
// none for a colloid whose box number lies past the C boxes)
__global__ void __launch_bounds__(128) k_no_neigh(const SysF64 S, int b, const int *occ, int *no_neigh) {
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.x * 4 + (threadIdx.x >> 5);
  if (j >= S.Nc) return;
  const int cb = S.cbox[b][j];
  int s = 0;
  if (cb < S.C) {
    const int cx = cb % S.Lx, ct = cb / S.Lx, cy = ct % S.Ly, cz = ct / S.Ly;
    for (int q = lane; q < 343; q += 32) {
      const int ox = q % 7 - 3, oy = (q / 7) % 7 - 3, oz = q / 49 - 3;
      if (!ox && !oy && !oz) continue;
      int bx = cx + ox, by = cy + oy, bz = cz + oz;
      bx += bx < 0 ? S.Lx : 0; bx -= bx >= S.Lx ? S.Lx : 0;
      by += by < 0 ? S.Ly : 0; by -= by >= S.Ly ? S.Ly : 0;
      bz += bz < 0 ? S.Lz : 0; bz -= bz >= S.Lz ? S.Lz : 0;
      s += occ[1 + bx + S.Lx * (by + S.Ly * bz)];
    }
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
  if (lane == 0) no_neigh[j] = s;
}

}  // namespace bgb
