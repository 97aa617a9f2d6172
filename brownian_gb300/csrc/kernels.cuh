// Kernel entry points (defined in kernels_fp64.cu and init_fp64.cu).
#pragma once
#include "sys.cuh"

namespace bgb {

enum : int { F_STREAM = 1, F_COLLIDE = 2, F_SHELL = 4, F_BINROT = 8, F_PIPE = 16 };
enum : int { M_FINISH = 1, M_KICK = 2, M_ADVANCE = 4, M_ACT = 8, M_COLL = 16 };

// k_stream<FLAGS> instantiations, by flag set (nullptr for a set not built)
using StreamKernel = void (*)(const SysF64, int, int);
StreamKernel stream_kernel(int flags);
using EventKernel = void (*)(const SysF64, int, int);
EventKernel event_kernel(int flags);
// batched forms over an array of systems (block offsets per system in boff)
using StreamKernelB = void (*)(const SysF64 *, const int *, int, int, int);
using EventKernelB = void (*)(const SysF64 *, const int *, int, int, int);
StreamKernelB stream_kernel32_b(int flags);
EventKernelB event_kernel32_b(int flags);
__global__ void k_cell_prep32_b(const SysF64 *Ss, const int *boff, int nrep);
__global__ void k_rotate32_b(const SysF64 *Ss, const int *boff, int nrep, int fb);
__global__ void k_rotate_sort32_b(const SysF64 *Ss, const int *boff, int nrep, int src, int dst);
__global__ void k_run_shell32_b(const SysF64 *Ss, const int *boff, int nrep, int fb);
__global__ void k_run_kick32_b(const SysF64 *Ss, const int *boff, int nrep, int fb);
__global__ void k_aux_b(const SysF64 *Ss, const int *boff, int nrep, int l, int act);
__global__ void k_fin_b(const SysF64 *Ss, const int *boff, int nrep, int mode, int l);
__global__ void k_end_step_b(const SysF64 *Ss, const int *boff, int nrep);
__global__ void k_scan_blocks_b(const SysF64 *Ss, const int *boff, int nrep, int nblk);
__global__ void k_gather_err(const SysF64 *Ss, int nrep, int *out);
// FP32-compensated form (kernels_fp32c.cu)
StreamKernel stream_kernel32(int flags);
int stream32_per_thread(int flags);  // particles per thread of the FP32 streaming pass
int stream64_per_thread(int flags);  // particles per thread of the FP64 streaming pass
__global__ void k_bin(const SysF64 S, int fb);
__global__ void k_updown_table(const SysF64 S, unsigned long long *Tc, uint16_t *Tl, long long epoch, float reach);
__global__ void k_updown(const SysF64 S, int fb, const unsigned long long *Tc, const uint16_t *Tl, long long epoch,
                         double rup2, int *cnt, ExchAcc *acc);
EventKernel event_kernel32(int flags);
__global__ void k_cell_prep32(__grid_constant__ const SysF64 S);
__global__ void k_rotate32(__grid_constant__ const SysF64 S, int fb);
__global__ void k_rotate_sort32(__grid_constant__ const SysF64 S, int src, int dst);
// the FP32 free-flight schedule: flight table, rotation with the classification, the free
// particles' whole step, per-substep passes over the near list
__global__ void k_flight_table32(__grid_constant__ const SysF64 S);
// the rotation with the classification (rotate false: after a counting-sort scatter); the
// FP32 form's takes CLASSIFY32_U particles per thread (grid: N / (256 CLASSIFY32_U) blocks)
constexpr int CLASSIFY32_U = 2;
using ClassifyKernel = void (*)(const SysF64, int);
ClassifyKernel classify_kernel32(bool rotate);
__global__ void k_free_flight32(__grid_constant__ const SysF64 S, int fb);
StreamKernel stream_kernel32_near(int flags);
// the same over a batch of systems (persistent, batch_for)
__global__ void k_flight_table32_b(const SysF64 *Ss, const int *boff, int nrep);
using ClassifyKernelB = void (*)(const SysF64 *, const int *, int, int);
ClassifyKernelB classify_kernel32_b(bool rotate);
__global__ void k_free_flight32_b(const SysF64 *Ss, const int *boff, int nrep, int fb);
StreamKernelB stream_kernel32_near_b(int flags);
ClassifyKernel classify_kernel(bool rotate);
__global__ void k_free_flight(const SysF64 S, int fb);
__global__ void k_bin_near(const SysF64 S, int fb);
StreamKernel stream_kernel_near(int flags);
// the FP64 event pass fused with the substep's colloid side work (grid: nevb event blocks,
// then one block per two colloids)
using EventAuxKernel = void (*)(const SysF64, int, int, int, int);
EventAuxKernel event_aux_kernel(int flags);
__global__ void k_run_shell32(__grid_constant__ const SysF64 S, int fb);
__global__ void k_run_kick32(__grid_constant__ const SysF64 S, int fb);
__global__ void k_aos_to_q(const SysF64 S, const double *pos, const double *vel, int fb);
__global__ void k_q_to_aos(const SysF64 S, double *pos, double *vel, int fb);
__global__ void k_cell_prep(const SysF64 S);
__global__ void k_scan_blocks(__grid_constant__ const SysF64 S, int nblk);
__global__ void k_rotate_sort(const SysF64 S, int src, int dst);
__global__ void k_rotate(const SysF64 S, int fb);
__global__ void k_run_shell(const SysF64 S, int fb);
__global__ void k_run_kick(const SysF64 S, int fb);
__global__ void k_fin(__grid_constant__ const SysF64 S, int mode, int l);
__global__ void k_aux(__grid_constant__ const SysF64 S, int l, int act, int vl);
__global__ void k_colloid_setup(const SysF64 S);
__global__ void k_colloid_pot(const SysF64 S, int b);
// routine-by-routine substeps (routines.cu)
__global__ void k_cbucket(const SysF64 S, const double *Xc, NListGeo geo);
__global__ void k_nlist(const SysF64 S, const double *Xc, NListGeo geo);
__global__ void k_nlist_step(const SysF64 S, NListGeo geo);
__global__ void k_force_list(const SysF64 S, const double *Xc);
__global__ void k_act_now(const SysF64 S, int l);
__global__ void k_vel_colloid(const SysF64 S);
__global__ void k_unpend(const SysF64 S);
__global__ void k_table(const SysF64 S, int l);
__global__ void k_box_bin(const SysF64 S, int fb, int *cell_of, int *occ);
__global__ void k_no_neigh(const SysF64 S, int b, const int *occ, int *no_neigh);
__global__ void k_end_step(__grid_constant__ const SysF64 S);
__global__ void k_diag_fluid(const SysF64 S, double *part);

// initialisation
// where the initial fluid state goes: positions and velocities with an element
// stride (1: the FP64 SoA buffers; 3: AoS staging converted afterwards)
struct InitOut {
  double *x, *y, *z, *vx, *vy, *vz;
  int stride;
  int *id, *newpos;
};
__global__ void k_init_fluid(const SysF64 S, int style, double vscale, double rmin, int max_attempts, InitOut o);
__global__ void k_vsum(const SysF64 S, double *part, InitOut o);
__global__ void k_vfinish(const SysF64 S, double ax, double ay, double az, InitOut o, double scale);
__global__ void k_aos_to_soa(const double *aos, double *x, double *y, double *z, int *id, int *newpos, int n,
                             double scale);
__global__ void k_soa_to_aos(double *aos, const double *x, const double *y, const double *z, const int *id, int n,
                             double scale);

}  // namespace bgb
