// Device-resident layout of one MPCD system and the constants every kernel needs.
#pragma once
#include <cstdint>

#include "common.cuh"

namespace bgb {

// error bits set by kernels (atomicOr), read back by the host after each call
enum : int {
  ERRB_TTABLE = 1,      // more colloids reach one cell than the cell table holds
  ERRB_SHELL = 2,       // run() candidate records overflowed
  ERRB_VRANGE = 4,      // a fluid displacement left the range of the exact cell sums
  ERRB_OCCUPANCY = 8,   // a cell holds more particles than the exact cell sums allow
  ERRB_DISPLACE = 16,   // a wall collision moved a particle further than the cell-table margin
  ERRB_SHELLSLOTS = 32, // a particle sits in the rear shells of more colloids than a record holds
  ERRB_DELTA = 64       // a colloid momentum exchange left the range of the exact sums
};

constexpr int TCAP = 16;     // colloids per cell in the fluid-to-colloid table
constexpr int SHELL_J = 8;   // colloids per run() candidate record

// one run() candidate: a particle whose binned cell is in the 342-cell block of
// each listed colloid and which lies within sigma/2 + 1/2 of it
struct ShellRec {
  int p;
  uint8_t n, pass;
  uint16_t j[SHELL_J];
};

// exact per-cell sums for the SRD collision: particle count, fixed-point sum of
// the displacements w = v dt, fixed-point sum of |w|^2
struct CellAcc {
  long long sx, sy, sz, s2;
  int n, pad;
};

// exact per-colloid momentum / angular-momentum exchange of one substep,
// each component as two fixed-point words: value = hi 2^-20 + lo 2^-72
struct ExchAcc {
  long long hi[6], lo[6];
};

// quantities that change every step, kept on the device so one captured CUDA
// graph serves every step
struct StepState {
  long long step;   // completed MPCD steps
  int err;          // error bits
  int nshell;       // run() candidate records written
  double rr[3];     // grid shift of the SRD binning the next streaming pass performs
};

struct SysF64 {
  // sizes
  int N, Nc, C, Cpad;
  int Lx, Ly, Lz, n_sub;
  Dim dx, dy, dz;
  uint2 key;
  // constants (host-computed with the host libm, as the reference computes them)
  double dt, half_dt_unused;
  double mass_fl, mass_colloid, I_colloid, kbt;
  double sig2q;        // pow(sigma, 2)*0.25            cpp/fluid_colloid_collision.cpp:35
  double rsh2;         // pow(sigma*0.5 + 0.5, 2)        cpp/run.cpp:18
  double r_cutoff, fc, ufc, sig12, sig6, eps, sig_colloid;
  double ddt;          // 0.5*dt*dt/mass_colloid         cpp/update.cpp:48
  double dtb2;         // dt/(mass_colloid*2)            cpp/update.cpp:63
  double v0, Dr, rotdiff_s;
  double ct, st, ict;  // cos, sin, 1-cos of the SRD angle
  double two_pi;       // 4.0*asin(1.0)
  double sqrt_kt_m;    // sqrt(kbt/mass_fl)
  double m_beta;       // mass_fl/kbt
  double cs;           // 3 kbt dt^2 / mass_fl (thermostat in displacement units)
  double inv_dt;
  float rT_coll, rT_shell;   // cell-table reach (with margin), FP32
  double disp_margin2;       // squared bound on collision displacement
  int kw, kw2;               // fixed-point scales of the cell sums
  double inv_sw, inv_sw2;    // 2^-kw, 2^-kw2
  long long wlim_bits;       // |w| component bound (bits of vmax*dt)
  long long w2lim_bits;      // |w|^2 bound
  int max_per_cell;
  // fluid (SoA)
  double *px, *py, *pz, *wx, *wy, *wz;
  int *rotcell;
  // cells
  CellAcc *acc;        // [Cpad]
  double *cell_ab;     // [C][12]: A (row-major 3x3), b
  const double *inv_n; // [max_per_cell+1]: 1/n
  // colloids
  double *X[2];        // [Nc][3] double-buffered by global substep parity
  float4 *Xf[2];       // FP32 copies for prefilters
  int *cbox[2];        // 0-based linear cell of each colloid (may alias or exceed C)
  double *V, *W, *ra, *f;   // [Nc][3]
  ExchAcc *exch;       // [Nc]
  int *shell_cnt;      // [Nc]
  // fluid-to-colloid table, double-buffered like X
  int *Tcnt[2];        // [C]
  uint16_t *Tlist[2];  // [C][TCAP]
  // run() candidates
  ShellRec *shell;
  int shell_cap;
  // step state
  StepState *ss;
  double *pot_part;    // [Nc] per-colloid share of the WCA potential
};

}  // namespace bgb
