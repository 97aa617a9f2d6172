// Kernel entry points (defined in kernels_fp64.cu and init_fp64.cu).
#pragma once
#include "sys.cuh"

namespace bgb {

enum : int { F_STREAM = 1, F_COLLIDE = 2, F_SHELL = 4, F_BINROT = 8 };
enum : int { M_FINISH = 1, M_KICK = 2, M_ADVANCE = 4, M_SETUP = 8, M_POT = 16 };

// k_stream<FLAGS> instantiations, by flag set (nullptr for a set not built)
using StreamKernel = void (*)(const SysF64, int);
StreamKernel stream_kernel(int flags);
__global__ void k_cell_prep(const SysF64 S);
__global__ void k_rotate(const SysF64 S);
__global__ void k_run_shell(const SysF64 S);
__global__ void k_run_kick(const SysF64 S);
__global__ void k_colloid(const SysF64 S, int mode, int l);
__global__ void k_end_step(const SysF64 S);
__global__ void k_diag_fluid(const SysF64 S, double *part);

// initialisation
__global__ void k_init_fluid(const SysF64 S, int style, double vscale, double rmin, int max_attempts);
__global__ void k_vsum(const SysF64 S, double *part);
__global__ void k_vfinish(const SysF64 S, double ax, double ay, double az);
__global__ void k_aos_to_soa(const double *aos, double *x, double *y, double *z, int n, double scale);
__global__ void k_soa_to_aos(double *aos, const double *x, const double *y, const double *z, int n, double scale);

}  // namespace bgb
