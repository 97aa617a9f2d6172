// updown_velocity (cpp/run.cpp:28-50): the fluid in each colloid's rear shells.
//
// The reference walks, per colloid, the fluid particles of the 342 boxes around
// the colloid's box (own box excluded, cpp/neighbour_list.cpp:20) and keeps those
// with |r|^2 <= (sigma/2 + 0.5)^2 (the run() shell) or <= (sigma/2 + 0.1)^2 (the
// inner shell) and r.V <= 0, r = img(pos_fl - pos_colloid).  Here one pass over
// the fluid finds them through a scratch cell table (colloids whose shell reaches
// a cell), tests them with the reference's arithmetic and adds, per colloid and
// shell, the count and the exact fixed-point sum of the fluid velocities (the
// same hi/lo split as the collision exchange), so the result is independent of
// the order the particles are visited in.
#include "../../include/brownian_gb300.h"
#include "device.cuh"

namespace bgb {

// colloid positions of the last completed substep
static __device__ __forceinline__ int cur_buf(const SysF64 &S) { return (int)((S.ss->step * S.n_sub - 1) & 1); }

// the cells each colloid's shell reaches, one warp per colloid
__global__ void __launch_bounds__(128) k_updown_table(const SysF64 S, unsigned long long *Tc, uint16_t *Tl,
                                                      long long epoch, float reach) {
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (j >= S.Nc) return;
  const int b = cur_buf(S);
  int *err = &S.ss->err;
  for_reach_cells(S, S.cbox[b][j], S.Xf[b][j], reach, lane, 32,
                  [&](int cell) { tappend(Tc, Tl, cell, epoch, j, err); });
}

// components c0..c0+2 of the per-colloid sums (|v| < 2^20, else the range bit)
static __device__ __forceinline__ void sum_add3(ExchAcc *e, int c0, d3 v, int *err) {
  const double a[3] = {v.x, v.y, v.z};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if ((dbits(a[k]) & 0x7FFFFFFFFFFFFFFFll) >= 0x4130000000000000ll) atomicOr(err, ERRB_DELTA);
    long long hi, lo;
    exch_split(a[k], hi, lo);
    atomicAdd((unsigned long long *)&e->hi[c0 + k], (unsigned long long)hi);
    atomicAdd((unsigned long long *)&e->lo[c0 + k], (unsigned long long)lo);
  }
}

// per particle: the colloids whose 342-box neighbourhood holds its box, the two
// shell tests, the counts (cnt[2j], cnt[2j+1]) and the sums (components 0-2 the
// run() shell, 3-5 the inner shell)
__global__ void __launch_bounds__(256) k_updown(const SysF64 S, int fb, const unsigned long long *Tc,
                                                const uint16_t *Tl, long long epoch, double rup2, int *cnt,
                                                ExchAcc *acc) {
  const int b = cur_buf(S);
  const double *Xc = S.X[b];
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < S.N; p += gridDim.x * blockDim.x) {
    double x, y, z;
    d3 v;
    if (S.precision == MPCD_FP32C) {  // FP32 form: cell + offset, FP32 velocity (exact in double)
      const Fluid32 F = fluid32_at(S, fb);
      const uint4 q = F.q[p];
      x = (double)(int)(q.x & 1023u) + (double)__uint_as_float(q.y);
      y = (double)(int)((q.x >> 10) & 1023u) + (double)__uint_as_float(q.z);
      z = (double)(int)((q.x >> 20) & 1023u) + (double)__uint_as_float(q.w);
      v = mk((double)F.vx[p], (double)F.vy[p], (double)F.vz[p]);
    } else {  // FP64 form stores w = v dt
      const Fluid F = fluid_at(S, fb);
      x = F.x[p]; y = F.y[p]; z = F.z[p];
      v = mk(__dmul_rn(F.wx[p], S.inv_dt), __dmul_rn(F.wy[p], S.inv_dt), __dmul_rn(F.wz[p], S.inv_dt));
    }
    bool alias;
    const int lin = cell_of_pos(S, x, y, z, alias);
    if (alias || lin >= S.C) continue;  // a box past the last row has no neighbours in the reference
    int n = tcount(Tc[lin], epoch);
    n = n < TCAP ? n : TCAP;
    for (int k = 0; k < n; ++k) {
      const int j = Tl[(size_t)lin * TCAP + k];
      if (!in_block(S, S.cbox[b][j], lin)) continue;
      const d3 r = mk(ref_img(__dsub_rn(x, Xc[3 * j]), S.dx), ref_img(__dsub_rn(y, Xc[3 * j + 1]), S.dy),
                      ref_img(__dsub_rn(z, Xc[3 * j + 2]), S.dz));
      if (!(dot_ref(r, mk(S.V[3 * j], S.V[3 * j + 1], S.V[3 * j + 2])) <= 0.0)) continue;
      const double r2 = norm2_ref(r.x, r.y, r.z);
      if (r2 <= S.rsh2) {
        atomicAdd(&cnt[2 * j], 1);
        sum_add3(acc + j, 0, v, &S.ss->err);
      }
      if (r2 <= rup2) {
        atomicAdd(&cnt[2 * j + 1], 1);
        sum_add3(acc + j, 3, v, &S.ss->err);
      }
    }
  }
}

}  // namespace bgb
