// libbrownian_shim: the reference's routine symbols (cpp/parameters.hpp:12-14,
// `void name()` over global arrays) implemented over the C ABI, so that the
// reference's own driver (cpp/active_brownian.cpp) links against this library
// unchanged and runs its step loop on the GPU.
//
// Contract (the call order of cpp/active_brownian.cpp:14-38):
//   initialize, initialize_colloid, initialize_fluid, create_box,
//   neighbour_list_mpcd, neighbour_list_md, compute_force_md, tumble, then per
//   step rotation_mpcd, run and n substeps of update_pos_md, neighbour_list_md,
//   update_pos_mpcd, neighbour_list_mpcd, [updown_velocity], fluid_colloid_collision,
//   update_activity_direction, compute_force_md, update_velocity_colloid.
// The GPU runs a substep as one fused pass: update_pos_md starts substep l and
// the next routines of the substep only advance the position in the sequence;
// update_velocity_colloid ends it and copies the colloid arrays (and, after the
// last substep of a step, the fluid arrays) into the reference's globals.  The
// state lives on the GPU; edits the caller makes to the global arrays between
// initialize_fluid and the set-up's compute_force_md are uploaded.  Random
// numbers are the library's keyed Philox draws (key = the global `seed`), not the
// reference's ran() stream, so a run is statistically, not bitwise, the reference's.
// updown_velocity is a no-op: the reference discards its results, and the counts it leaves in
// the globals are overwritten by run() before anything reads them (the diagnostic itself is
// mpcd_updown_velocity).
// A routine called out of this order sets an error; the first error is printed
// to stderr and the process exits with status 3 (the reference's routines cannot
// return one).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "brownian_gb300.h"

// the reference's point: three doubles (cpp/parameters.hpp:44-45); only its layout matters here
struct shim_point {
  double x, y, z;
};

// globals defined by the reference's driver (cpp/active_brownian.cpp:3-7)
extern shim_point *pos_colloid, *pos_fl, *vel_colloid, *vel_fl, *ang_vel_colloid, *f, *ra, *old_force, *dump_vel_fl,
    len;
extern int n, no_of_fluid, no_of_colloid, seed, nn;
extern double kbt, kbt1, ndt, mass_fl, mass_colloid, sig_colloid, eps, v0, sigma, I_colloid, potential_colloid;

namespace {

mpcd_ctx *g_ctx = nullptr;
enum Phase { NONE, ALLOCATED, INITIALISED, READY, IN_STEP };
Phase g_phase = NONE;
int g_sub = 0;          // substep in progress (0: none)
int g_seq = 0;          // position within the substep's routine sequence
std::vector<double> g_seen_fl;  // fluid state as last copied to the globals (pos then vel)
std::vector<double> g_seen_c;   // colloid state as last copied (pos, vel, ang_vel, ra)

[[noreturn]] void die(const char *what) {
  fprintf(stderr, "brownian_shim: %s%s%s\n", what, g_ctx ? ": " : "", g_ctx ? mpcd_last_error(g_ctx) : "");
  exit(3);
}

void check(int r, const char *what) {
  if (r != MPCD_OK) die(what);
}

double *flat(shim_point *a) { return &a[1].x; }  // the reference's arrays are 1-based

void download(bool fluid) {
  double *pf = nullptr, *vf = nullptr;
  if (fluid) {
    pf = flat(pos_fl);
    vf = flat(vel_fl);
  }
  check(mpcd_get_state(g_ctx, pf, vf, flat(pos_colloid), flat(vel_colloid), flat(ang_vel_colloid), flat(ra), flat(f)),
        "copying the state to the reference's arrays");
  const size_t N3 = 3 * (size_t)no_of_fluid, C3 = 3 * (size_t)no_of_colloid;
  if (fluid) {
    g_seen_fl.resize(2 * N3);
    memcpy(g_seen_fl.data(), pf, 8 * N3);
    memcpy(g_seen_fl.data() + N3, vf, 8 * N3);
  }
  g_seen_c.resize(4 * C3);
  memcpy(g_seen_c.data(), flat(pos_colloid), 8 * C3);
  memcpy(g_seen_c.data() + C3, flat(vel_colloid), 8 * C3);
  memcpy(g_seen_c.data() + 2 * C3, flat(ang_vel_colloid), 8 * C3);
  memcpy(g_seen_c.data() + 3 * C3, flat(ra), 8 * C3);
  mpcd_diag_t d;
  if (mpcd_diag(g_ctx, &d) == MPCD_OK) potential_colloid = d.potential_colloid;
}

// upload the globals if the caller changed them since they were last copied
void upload_if_changed() {
  const size_t N3 = 3 * (size_t)no_of_fluid, C3 = 3 * (size_t)no_of_colloid;
  const bool fl_changed = g_seen_fl.size() != 2 * N3 || memcmp(g_seen_fl.data(), flat(pos_fl), 8 * N3) ||
                          memcmp(g_seen_fl.data() + N3, flat(vel_fl), 8 * N3);
  const bool c_changed = g_seen_c.size() != 4 * C3 || memcmp(g_seen_c.data(), flat(pos_colloid), 8 * C3) ||
                         memcmp(g_seen_c.data() + C3, flat(vel_colloid), 8 * C3) ||
                         memcmp(g_seen_c.data() + 2 * C3, flat(ang_vel_colloid), 8 * C3) ||
                         memcmp(g_seen_c.data() + 3 * C3, flat(ra), 8 * C3);
  if (fl_changed || c_changed)
    check(mpcd_set_state(g_ctx, fl_changed ? flat(pos_fl) : nullptr, fl_changed ? flat(vel_fl) : nullptr,
                         flat(pos_colloid), flat(vel_colloid), flat(ang_vel_colloid), flat(ra)),
          "copying the reference's arrays to the GPU");
}

shim_point *alloc_points(int count) {
  shim_point *p = (shim_point *)calloc((size_t)count + 2, sizeof(shim_point));
  if (!p) die("out of host memory");
  return p;
}

// the eight routines of a substep, in the reference's order; update_pos_md opens it
void substep_routine(int seq) {
  if (g_phase != IN_STEP || g_sub < 1 || g_seq != seq) die("substep routines called out of the reference's order");
  g_seq = seq + 1;
}

}  // namespace

// initialize (cpp/initialize.cpp:3-29): the arrays the driver reads, and the GPU context
void initialize() {
  if (g_phase != NONE) die("initialize called twice");
  mpcd_params p;
  memset(&p, 0, sizeof p);
  p.Lx = (int)len.x; p.Ly = (int)len.y; p.Lz = (int)len.z;
  p.n_fluid = no_of_fluid; p.n_colloid = no_of_colloid; p.n_sub = n;
  p.kbt = kbt; p.kbt1 = kbt1; p.ndt = ndt; p.mass_fl = mass_fl; p.mass_colloid = mass_colloid;
  p.sig_colloid = sig_colloid; p.eps = eps; p.sigma = sigma; p.I_colloid = I_colloid; p.v0 = v0;
  p.theta_deg = 130.0;  // the reference's fixed SRD angle (cpp/rotation_mpcd.cpp:19)
  p.Dr = 0.0;
  p.seed = (uint64_t)(uint32_t)seed;
  p.precision = MPCD_FP64;
  if (mpcd_create(&p, &g_ctx) != MPCD_OK) die("mpcd_create rejected the reference's parameters");
  pos_fl = alloc_points(no_of_fluid); vel_fl = alloc_points(no_of_fluid); dump_vel_fl = alloc_points(no_of_fluid);
  f = alloc_points(no_of_colloid); pos_colloid = alloc_points(no_of_colloid); vel_colloid = alloc_points(no_of_colloid);
  ang_vel_colloid = alloc_points(no_of_colloid); old_force = alloc_points(no_of_colloid); ra = alloc_points(no_of_colloid);
  g_phase = ALLOCATED;
}

void initialize_colloid() {
  if (g_phase != ALLOCATED) die("initialize_colloid before initialize");
}

// initialize_fluid: colloids, fluid and orientations (tumble) on the GPU, then copied out
void initialize_fluid() {
  if (g_phase != ALLOCATED) die("initialize_fluid before initialize");
  check(mpcd_initialize(g_ctx, MPCD_INIT_REFERENCE), "initialisation");
  check(mpcd_set_step(g_ctx, 0), "initialisation");
  download(true);
  g_phase = INITIALISED;
}

// tumble (cpp/run.cpp:3-8) already ran inside initialize_fluid
void tumble() {
  if (g_phase != READY) die("tumble outside the prologue");
}

void create_box() {}
void updown_velocity() {}

void neighbour_list_mpcd() {
  if (g_phase == IN_STEP) substep_routine(3);
}

void neighbour_list_md() {
  if (g_phase == IN_STEP) substep_routine(1);
}

// in the prologue: the set-up (create_box, neighbour lists and forces, cpp/active_brownian.cpp:17-20)
void compute_force_md() {
  if (g_phase == INITIALISED) {
    upload_if_changed();
    check(mpcd_setup(g_ctx), "set-up");
    download(false);
    g_phase = READY;
    return;
  }
  substep_routine(6);
}

void rotation_mpcd() {
  if (g_phase == INITIALISED) die("rotation_mpcd before the set-up");
  if (g_phase != READY) die("rotation_mpcd inside a step");
  upload_if_changed();
  check(mpcd_rotation_mpcd(g_ctx), "rotation_mpcd");
  g_phase = IN_STEP;
  g_sub = 0;
}

void run() {
  if (g_phase != IN_STEP || g_sub != 0) die("run out of order");
  check(mpcd_run(g_ctx), "run");
}

void update_pos_md() {
  if (g_phase != IN_STEP || g_sub >= n || (g_sub > 0 && g_seq != 8)) die("update_pos_md out of order");
  g_sub += 1;
  check(mpcd_substep(g_ctx, g_sub), "substep");
  g_seq = 1;
}

void update_pos_mpcd() { substep_routine(2); }
void fluid_colloid_collision() { substep_routine(4); }
void update_activity_direction() { substep_routine(5); }

void update_velocity_colloid() {
  substep_routine(7);
  const bool last = g_sub == n;
  download(last);
  if (last) {
    g_phase = READY;
    g_sub = 0;
  }
}
