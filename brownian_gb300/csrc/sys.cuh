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
  ERRB_DELTA = 64,      // a colloid momentum exchange left the range of the exact sums
  ERRB_EVENTS = 128,    // the wall-collision event (or pending-particle) lists overflowed
  ERRB_NBR = 256        // a colloid has more pair-list partners than the list holds
};

constexpr int TCAP = 16;     // colloids per cell in the fluid-to-colloid table
constexpr int SHELL_J = 8;   // colloids per run() candidate record
constexpr int NBR_CAP = 256; // partners per colloid in the colloid pair list (the reference holds 200)
constexpr int NBK_MAX = 32;  // buckets per axis of the colloid pair-list grid

// one run() candidate: a particle whose binned cell is in the 342-cell block of
// each listed colloid and which lies within sigma/2 + 1/2 of it
struct ShellRec {
  int p;  // particle id
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

// an FP64 event: the particle and its streamed position and displacement, so the
// event pass starts from one record instead of an index and a gather
struct __align__(16) EventRec {
  double2 xy, zwx, wywz;
  int p, id;  // slot in the fluid arrays and particle id
};

// quantities that change every step, kept on the device so one captured CUDA
// graph serves every step
struct StepState {
  long long step;   // completed MPCD steps
  int err;          // error bits
  int nshell;       // run() candidate records written
  int nevents;      // particles the streaming pass left to k_events (FP32 form)
  int nnew[2];      // FP64 form: particles the streaming pass of substep g listed, [g & 1]
  int npend;        // FP64 form: pending particles carried from earlier substeps of this step
  long long ev_total;  // events summed over substeps (diagnostics)
  double rr[3];     // grid shift of the SRD binning the next streaming pass performs
  float rrf[3];     // the same, FP32
  // the bound on a colloid's displacement in one substep the colloid finish checks this
  // step (cm2 = cm^2): the FP64 form's streaming pass uses it as margin, the FP32 form's
  // free-flight classification as the colloids' move over the step (n_sub cm)
  float cm;
  double cm2;
  int nnear;        // free-flight schedule: particles listed for the near passes this step
  double rrn[3];    // free-flight schedule: the next step's grid shift (the free pass bins with it)
};

// one cell of the FP32 form's flight table: (step + 1) << 32 | count, and the first
// FLIGHT_CAP colloids (a cell with more is treated as near for all its particles)
constexpr int FLIGHT_CAP = 12;
struct __align__(32) FlightCell {
  unsigned long long tc;
  uint16_t id[FLIGHT_CAP];
};

struct SysF64 {
  // sizes
  int N, Nc, C, Cpad;
  int Lx, Ly, Lz, n_sub;
  float Lxf, Lyf, Lzf;
  Dim dx, dy, dz;
  uint2 key;
  // constants (host-computed with the host libm, as the reference computes them)
  double dt, half_dt_unused;
  double mass_fl, mass_colloid, I_colloid, kbt;
  double sig2q;        // pow(sigma, 2)*0.25            cpp/fluid_colloid_collision.cpp:35
  double rsh2;         // pow(sigma*0.5 + 0.5, 2)        cpp/run.cpp:18
  double r_cutoff, fc, ufc, sig12, sig6, eps, sig_colloid;
  float rcf;           // FP32 prefilter radius of the WCA pair search
  double ddt;          // 0.5*dt*dt/mass_colloid         cpp/update.cpp:48
  double dtb2;         // dt/(mass_colloid*2)            cpp/update.cpp:63
  double inv_mc, inv_ic;  // 1/mass_colloid, 1/I_colloid (the exchange's velocity changes)
  double v0, Dr, rotdiff_s;
  double ct, st, ict;  // cos, sin, 1-cos of the SRD angle
  double two_pi;       // 4.0*asin(1.0)
  double sqrt_kt_m;    // sqrt(kbt/mass_fl)
  double m_beta;       // mass_fl/kbt
  double inv_m_beta;   // kbt/mass_fl
  double cs;           // 3 kbt dt^2 / mass_fl (thermostat in displacement units)
  double inv_dt;
  float rT_coll, rT_shell;   // cell-table reach (sphere or shell + margins), FP32
  float r_coll, r_shell;     // sphere radius sigma/2 and shell radius sigma/2 + 1/2, FP32
  double disp_margin2;       // squared bound on the displacement of one wall collision
  double cmargin2;           // squared bound on a colloid's displacement in one substep
  int kw;                    // fixed-point scale of the cell sums (w and |w|^2)
  double inv_sw;             // 2^-kw
  long long wlim_bits;       // |w| component bound (bits of vmax*dt)
  int max_per_cell;
  // fluid (SoA), two buffers: the SRD pass of each step writes the particles into the
  // other buffer sorted by their SRD cell (a counting sort), so a warp's particles sit
  // in one or two cells; id[] carries each particle's identity through the sorts
  double *fl[2][6];    // [buffer][x, y, z, wx, wy, wz]
  int *pid[2];         // [buffer][position] -> particle id
  int *newpos;         // particle id -> position in the buffer the last sort wrote
  int *rotcell;        // position in the current buffer -> cell of the next SRD binning
  int *cell_off;       // [Cpad] first slot of each cell within its block of 256 cells
  int *cursor;         // [Cpad] slots taken per cell during the sort
  int *blk_off;        // [ceil(Cpad/256)] block sums, then their exclusive prefix
  // cells
  CellAcc *acc;        // [Cpad]
  double *cell_ab;     // [C][12]: A (row-major 3x3), b
  const double *insw_n;  // [max_per_cell+1]: 2^-kw / n (exact scaling of 1/n), the cell mean of both forms
  const double *sqcs_n;  // [max_per_cell+1]: sqrt(cs (n - 1)), the FP64 thermostat's numerator
  const float *sq3kt_n32;  // [max_per_cell+1]: sqrt(3 kT (n - 1) / m), the FP32 thermostat's numerator
  // colloids
  double *X[2];        // [Nc][3] double-buffered by global substep parity
  float4 *Xf[2];       // FP32 copies for prefilters
  int *cbox[2];        // 0-based linear cell of each colloid (may alias or exceed C)
  double *V, *W, *ra, *f;   // [Nc][3]
  double *fnew;             // [Nc][3] force at the positions of the substep in flight
  double *xi;               // [Nc][3] rotational-diffusion normals of the substep in flight
  ExchAcc *exch;       // [Nc]
  double *xacc;        // [Nc][6] fluid-to-colloid momentum and angular momentum received since the last read
  int *shell_cnt;      // [Nc]
  // fluid-to-colloid table, double-buffered like X: per cell (substep << 32) | count,
  // entries of another substep read as empty, so the table is never cleared
  unsigned long long *Tcnt[2];  // [C]
  uint16_t *Tlist[2];           // [C][TCAP]
  // run() candidates
  ShellRec *shell;
  int shell_cap;
  // particles near a sphere surface in the substep in flight
  int *events;
  int events_cap;
  // FP64 form, substeps overlapped: the streaming pass of substep g tests against
  // the colloid positions of g-1 with the displacement bound as margin and lists
  // the particles it cannot clear in newrec[g & 1]; each becomes pending (pend[p])
  // for the rest of the step, its state kept in prec and advanced by the event
  // passes, so a streaming pass never touches a particle an event pass may be
  // changing at the same time
  EventRec *newrec[2];
  EventRec *prec;
  int pend_cap;
  uint8_t *pend;    // [N]
  int physics;      // MPCD_PHYSICS_FIXED: own box among the candidates, 2-D tangential reflection
  float cmarginf;   // the margin (the bound cmargin2 checks), FP32
  int fin_table;    // FP64 form: the colloid finish of substep g builds the cell table of
                    // g+2 (else the side kernel of g+1 does)
  // FP32-compensated fluid (precision MPCD_FP32C): per particle one 16-byte record
  // {cell x | y << 10 | z << 20, offset x, offset y, offset z} with offsets in
  // [0, 1) (positions exact to 2^-24 of a cell anywhere in the box) and FP32
  // velocities; both buffers as for the FP64 fluid
  int precision;
  int aux_nw;  // warps per colloid of the colloid side work (2, 4 or 8)
  uint4 *q[2];
  float *v32[2][3];
  float *cell_ab32;    // [C][12] SRD map in FP32
  float dtf;           // dt in FP32
  float kick32;        // M v0 / m in FP32: run()'s fluid kick times the shell count
  float vmaxf;         // speed bound of the exact cell sums
  float4 *Xcq[2];      // colloid cell (integer-valued floats), double-buffered like X
  float4 *Xco[2];      // colloid offset within the cell
  // free-flight schedule: a particle that no colloid can reach during a step is streamed
  // through all its substeps by one pass beside the substeps of the others, which the
  // rotation pass lists in near[] for the per-substep passes.  The flight table lists per
  // cell the colloids that come within the flight reach of it at the start of the step
  // (tag step + 1, like Tcnt).
  int *near;                    // [N] slots of the near particles
  uint8_t *fnear;               // [N] 1: the slot's particle is near this step
  FlightCell *ftab;             // [C]
  float flight_rv;              // travel allowance: particles moving further in a step are near
  int vlist;                    // the free-flight steps compute the forces from a pair list built
                                // at the start of the step
  // step state
  StepState *ss;
  double *pot_part;    // [Nc] per-colloid share of the WCA potential
  // routine-by-routine substeps (mpcd_update_pos_md ... mpcd_update_velocity_colloid)
  double *fold;        // [Nc][3] old_force: the force before this substep's compute_force_md
  int *nbr_n;          // [Nc] partners in the colloid pair list
  uint16_t *nbr;       // [Nc][NBR_CAP] partners of each colloid, ascending (both sides of j)
  int *bkt_start;      // [NBK_MAX^3 + 1] first slot of each bucket of the pair-list grid
  int *bkt_cur;        // [NBK_MAX^3] fill cursor of each bucket
  int *bkt_list;       // [Nc] colloids by bucket
};

// the bucket grid of a colloid pair list: per axis nb buckets of width bs >= the list
// radius (every partner within it is in a neighbouring bucket), r2 = radius^2
struct NListGeo {
  int nb[3];
  double bs[3];
  double r2;
};

// view of one fluid buffer
struct Fluid {
  double *x, *y, *z, *wx, *wy, *wz;
  int *id;
};

__device__ __host__ __forceinline__ Fluid fluid_at(const SysF64 &S, int b) {
  Fluid f;
  f.x = S.fl[b][0]; f.y = S.fl[b][1]; f.z = S.fl[b][2];
  f.wx = S.fl[b][3]; f.wy = S.fl[b][4]; f.wz = S.fl[b][5];
  f.id = S.pid[b];
  return f;
}

// view of one FP32-compensated fluid buffer
struct Fluid32 {
  uint4 *q;
  float *vx, *vy, *vz;
  int *id;
};

__device__ __host__ __forceinline__ Fluid32 fluid32_at(const SysF64 &S, int b) {
  Fluid32 f;
  f.q = S.q[b];
  f.vx = S.v32[b][0]; f.vy = S.v32[b][1]; f.vz = S.v32[b][2];
  f.id = S.pid[b];
  return f;
}

}  // namespace bgb
