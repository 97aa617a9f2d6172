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
// Each routine of a substep runs its own entry point (mpcd_update_pos_md ...
// mpcd_update_velocity_colloid) and then copies the arrays it writes into the
// reference's globals (pos_colloid; pos_fl; pos_fl, vel_fl, vel_colloid and
// ang_vel_colloid; ra; f and potential_colloid; vel_colloid), so the globals hold the
// GPU's state after every routine; rotation_mpcd and run copy the fluid and colloid
// velocities.  The state lives on the GPU; edits the caller makes to the global arrays
// between steps (or between initialize_fluid and the set-up's compute_force_md) are
// uploaded at the next rotation_mpcd (or the set-up), and the set-up then runs again:
// forces and cell tables at the edited positions.  Random numbers are the library's
// keyed Philox draws (key = the global `seed`), not the reference's ran() stream, so a
// run is statistically, not bitwise, the reference's.
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
// the arrays as last copied to or from the GPU, so that edits by the caller show
enum { A_POS_FL, A_VEL_FL, A_POS_C, A_VEL_C, A_ANG_C, A_RA, A_COUNT };
std::vector<double> g_seen[A_COUNT];
int g_sub = 0;  // substeps opened in the present step

[[noreturn]] void die(const char *what) {
  fprintf(stderr, "brownian_shim: %s%s%s\n", what, g_ctx ? ": " : "", g_ctx ? mpcd_last_error(g_ctx) : "");
  exit(3);
}

void check(int r, const char *what) {
  if (r != MPCD_OK) die(what);
}

double *flat(shim_point *a) { return &a[1].x; }  // the reference's arrays are 1-based

shim_point *global_of(int a) {
  shim_point *const g[A_COUNT] = {pos_fl, vel_fl, pos_colloid, vel_colloid, ang_vel_colloid, ra};
  return g[a];
}

size_t count_of(int a) { return 3 * (size_t)(a <= A_VEL_FL ? no_of_fluid : no_of_colloid); }

void remember(int a) {
  g_seen[a].resize(count_of(a));
  memcpy(g_seen[a].data(), flat(global_of(a)), 8 * count_of(a));
}

// copy the named arrays (bits of 1 << A_*), and f and the potential when `forces`, from
// the GPU into the reference's globals
void pull(unsigned which, bool forces = false) {
  double *p[A_COUNT];
  for (int a = 0; a < A_COUNT; ++a) p[a] = (which >> a) & 1u ? flat(global_of(a)) : nullptr;
  check(mpcd_get_state(g_ctx, p[A_POS_FL], p[A_VEL_FL], p[A_POS_C], p[A_VEL_C], p[A_ANG_C], p[A_RA],
                       forces ? flat(f) : nullptr),
        "copying the state to the reference's arrays");
  for (int a = 0; a < A_COUNT; ++a)
    if ((which >> a) & 1u) remember(a);
  if (forces) {
    mpcd_diag_t d;
    check(mpcd_diag(g_ctx, &d), "diagnostics");
    potential_colloid = d.potential_colloid;
  }
}

const unsigned ALL = (1u << A_COUNT) - 1u;

// upload the globals if the caller changed them since they were last copied; the set-up
// then runs again (forces and tables at the edited state).  Returns whether it uploaded.
bool upload_if_changed() {
  bool changed[A_COUNT], fl = false, any = false;
  for (int a = 0; a < A_COUNT; ++a) {
    changed[a] = g_seen[a].size() != count_of(a) || memcmp(g_seen[a].data(), flat(global_of(a)), 8 * count_of(a));
    any = any || changed[a];
  }
  fl = changed[A_POS_FL] || changed[A_VEL_FL];
  if (!any) return false;
  check(mpcd_set_state(g_ctx, fl ? flat(pos_fl) : nullptr, fl ? flat(vel_fl) : nullptr, flat(pos_colloid),
                       flat(vel_colloid), flat(ang_vel_colloid), flat(ra)),
        "copying the reference's arrays to the GPU");
  for (int a = 0; a < A_COUNT; ++a) remember(a);
  return true;
}

shim_point *alloc_points(int count) {
  shim_point *p = (shim_point *)calloc((size_t)count + 2, sizeof(shim_point));
  if (!p) die("out of host memory");
  return p;
}

// a routine of the substep body: its entry point, then its arrays to the globals
void substep_routine(int (*fn)(mpcd_ctx *), const char *name, unsigned writes, bool forces = false) {
  if (g_phase != IN_STEP) die("substep routines run inside a step (after rotation_mpcd and run)");
  check(fn(g_ctx), name);
  if (writes || forces) pull(writes, forces);
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
  pull(ALL);
  g_phase = INITIALISED;
}

// tumble (cpp/run.cpp:3-8) already ran inside initialize_fluid
void tumble() {
  if (g_phase != READY) die("tumble outside the prologue");
}

void create_box() {}
void updown_velocity() {}

// the set-up (create_box, neighbour lists and forces, cpp/active_brownian.cpp:17-20)
static void setup() {
  check(mpcd_setup(g_ctx), "set-up");
  pull(0, true);
  g_phase = READY;
}

void neighbour_list_mpcd() {
  if (g_phase == INITIALISED || g_phase == READY) return;  // the prologue: part of the set-up
  substep_routine(mpcd_neighbour_list_mpcd, "neighbour_list_mpcd", 0);
}

void neighbour_list_md() {
  if (g_phase == INITIALISED || g_phase == READY) return;  // the prologue: part of the set-up
  substep_routine(mpcd_neighbour_list_md, "neighbour_list_md", 0);
}

// in the prologue the set-up; inside a step the routine
void compute_force_md() {
  if (g_phase == INITIALISED) {
    upload_if_changed();
    setup();
    return;
  }
  substep_routine(mpcd_compute_force_md, "compute_force_md", 0, true);
}

void rotation_mpcd() {
  if (g_phase == INITIALISED) die("rotation_mpcd before the set-up");
  if (g_phase != READY) die("rotation_mpcd inside a step");
  if (upload_if_changed()) setup();
  check(mpcd_rotation_mpcd(g_ctx), "rotation_mpcd");
  g_phase = IN_STEP;
  g_sub = 0;
  pull(1u << A_VEL_FL);
}

void run() {
  if (g_phase != IN_STEP) die("run out of order");
  check(mpcd_run(g_ctx), "run");
  pull((1u << A_VEL_FL) | (1u << A_VEL_C));
}

void update_pos_md() {
  substep_routine(mpcd_update_pos_md, "update_pos_md", 1u << A_POS_C);
  g_sub += 1;
}
void update_pos_mpcd() { substep_routine(mpcd_update_pos_mpcd, "update_pos_mpcd", 1u << A_POS_FL); }
void fluid_colloid_collision() {
  substep_routine(mpcd_fluid_colloid_collision, "fluid_colloid_collision",
                  (1u << A_POS_FL) | (1u << A_VEL_FL) | (1u << A_VEL_C) | (1u << A_ANG_C));
}
void update_activity_direction() {
  substep_routine(mpcd_update_activity_direction, "update_activity_direction", 1u << A_RA);
}

void update_velocity_colloid() {
  substep_routine(mpcd_update_velocity_colloid, "update_velocity_colloid", 1u << A_VEL_C);
  if (g_sub == n) {  // the last substep closed the step
    g_phase = READY;
    g_sub = 0;
  }
}
