/*
 * brownian_gb300 — C ABI of the GB300 (sm_103a) MPCD + active-colloid step.
 *
 * The reference (shashankgandham/brownian, cpp/) exposes its step as global-state
 * C++ procedures `void f()` declared at cpp/parameters.hpp:12-14 and driven by
 * main() in cpp/active_brownian.cpp:9-60.  This library replaces them with an
 * explicit context: the context owns the device-resident state (structure of
 * arrays in HBM), every call returns a status, and each reference routine has one
 * entry point of the same name.  Calls on one context are not thread-safe;
 * distinct contexts are independent.  All arrays crossing the boundary are plain
 * host pointers to 0-based xyz triplets of doubles (the reference's 1-based
 * `point` arrays without their unused slot 0).
 *
 * Random numbers are counter-based (Philox4x32-10 keyed by `seed`): the grid
 * shift of step n, the rotation axis of cell c at step n, the reflection of
 * particle l off colloid j at substep s, ... are each a fixed function of those
 * indices, so results do not depend on thread scheduling and a run restarted
 * from a saved state and step counter continues bit for bit.
 */
#ifndef BROWNIAN_GB300_H
#define BROWNIAN_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
enum {
  MPCD_OK = 0,
  MPCD_ERR_PARAM = 1,     /* invalid parameter or argument                        */
  MPCD_ERR_CUDA = 2,      /* a CUDA call failed (message in mpcd_last_error)      */
  MPCD_ERR_CAPACITY = 3,  /* a fixed-capacity table overflowed (no data corrupted) */
  MPCD_ERR_RANGE = 4,     /* a value left the range the fixed-point sums allow   */
  MPCD_ERR_STATE = 5,     /* call out of order (e.g. step before setup)           */
  MPCD_ERR_NOMEM = 6      /* device or host allocation failed                     */
};

/* precision forms */
enum { MPCD_FP64 = 0, MPCD_FP32C = 1 };

/* initial-state styles for mpcd_initialize */
enum {
  MPCD_INIT_REFERENCE = 0, /* cpp/initialize.cpp: uniform-box velocities, colloid spacing 1.3*sig_colloid,
                              tumble() orientation of cpp/run.cpp:3-8                                    */
  MPCD_INIT_PHYSICAL = 1   /* Maxwell-Boltzmann velocities, colloid gap >= init_gap, isotropic orientation */
};

typedef struct {
  int Lx, Ly, Lz;          /* periodic box in unit cells (reference: len), each >= 7      */
  int n_fluid;             /* reference: no_of_fluid                                      */
  int n_colloid;           /* reference: no_of_colloid                                    */
  int n_sub;               /* MD substeps per MPCD step (reference: n)                    */
  double kbt, kbt1;        /* fluid temperature; colloid initial temperature              */
  double ndt;              /* MPCD time step; the MD substep is dt = ndt / n_sub          */
  double mass_fl, mass_colloid;
  double sig_colloid;      /* WCA sigma                                                   */
  double eps;              /* WCA epsilon                                                 */
  double sigma;            /* colloid diameter                                            */
  double I_colloid;        /* colloid moment of inertia                                   */
  double v0;               /* self-propulsion speed                                       */
  double theta_deg;        /* SRD rotation angle (reference: 130, cpp/rotation_mpcd.cpp:19) */
  double Dr;               /* rotational diffusion of the orientation (0: none, as the reference) */
  uint64_t seed;           /* Philox key                                                  */
  int precision;           /* MPCD_FP64 or MPCD_FP32C                                     */
  int max_per_cell;        /* occupancy bound of one cell for the exact cell sums (0: 128) */
  double vmax;             /* speed bound of one fluid particle for the exact sums (0: 24*sqrt(kbt/mass_fl)) */
  double init_gap;         /* MPCD_INIT_PHYSICAL: minimum surface gap between colloids    */
  int sort_every;          /* reorder the fluid by cell every this many steps (0: 10; <0: never) */
  int physics;             /* MPCD_PHYSICS_REFERENCE (0) or MPCD_PHYSICS_FIXED (1)           */
} mpcd_params;

/* collision rules: the reference's (bit parity), or corrected ones: a colloid's own box among
 * its candidate boxes (the reference skips it, cpp/neighbour_list.cpp:20) and both tangential
 * Gaussian components of the wall reflection (the reference draws two and uses one,
 * cpp/fluid_colloid_collision.cpp:22-23).  The initial state is chosen apart (mpcd_initialize:
 * MPCD_INIT_PHYSICAL gives Maxwell-Boltzmann velocities and isotropic orientations). */
enum { MPCD_PHYSICS_REFERENCE = 0, MPCD_PHYSICS_FIXED = 1 };

typedef struct {
  int64_t step;            /* completed MPCD steps                                        */
  double ke_fluid;         /* cpp/active_brownian.cpp:55                                  */
  double ke_colloid;       /* :52                                                         */
  double ang_ke_colloid;   /* :53                                                         */
  double potential_colloid;/* cpp/update.cpp:16-24                                        */
  double energy_colloid;   /* cpp/active_brownian.cpp:54                                  */
  double momentum[3];      /* fluid + colloid, this step (the reference never resets its sum) */
  double momentum_fluid[3];
  double temperature_fluid;/* 2 KE / (3 N kB) in units of kbt                             */
  int64_t events;          /* particles found at a colloid wall since the last mpcd_diag   */
  int64_t shell_records;   /* run() candidate particles recorded for the next step        */
} mpcd_diag_t;

typedef struct mpcd_ctx mpcd_ctx;

/* ---- lifetime and state (replaces cpp/initialize.cpp:3-29 allocation and the globals of
 *      cpp/active_brownian.cpp:3-7) ------------------------------------------------------ */
int mpcd_create(const mpcd_params *p, mpcd_ctx **out);
int mpcd_destroy(mpcd_ctx *c);
const char *mpcd_last_error(const mpcd_ctx *c);
/* launch all work of this context on `stream` (a cudaStream_t; NULL = the context's own) */
int mpcd_set_stream(mpcd_ctx *c, void *stream);

/* host arrays, 0-based xyz triplets.  Any pointer may be NULL to leave that array as is. */
int mpcd_set_state(mpcd_ctx *c, const double *pos_fl, const double *vel_fl, const double *pos_colloid,
                   const double *vel_colloid, const double *ang_vel_colloid, const double *ra);
int mpcd_get_state(mpcd_ctx *c, double *pos_fl, double *vel_fl, double *pos_colloid, double *vel_colloid,
                   double *ang_vel_colloid, double *ra, double *f);
int mpcd_set_step(mpcd_ctx *c, int64_t step);
int64_t mpcd_get_step(const mpcd_ctx *c);

/* ---- reference routines ------------------------------------------------------------- */
/* initialize_colloid + initialize_fluid (cpp/initialize.cpp:31-83) and tumble (cpp/run.cpp:3-8) */
int mpcd_initialize(mpcd_ctx *c, int style);
/* create_box + neighbour_list_mpcd + neighbour_list_md + compute_force_md, the prologue of
 * main (cpp/active_brownian.cpp:17-20); required once after set_state/initialize */
int mpcd_setup(mpcd_ctx *c);
/* rotation_mpcd (cpp/rotation_mpcd.cpp:3-50) for step counter+1 */
int mpcd_rotation_mpcd(mpcd_ctx *c);
/* run (cpp/run.cpp:10-26) */
int mpcd_run(mpcd_ctx *c);
/* one pass of the substep body l (1..n_sub) of cpp/active_brownian.cpp:28-37:
 * update_pos_md, neighbour_list_md, update_pos_mpcd, neighbour_list_mpcd,
 * fluid_colloid_collision, update_activity_direction, compute_force_md,
 * update_velocity_colloid */
int mpcd_substep(mpcd_ctx *c, int l);

/* The same substep routine by routine: one entry point per reference routine of the body of
 * cpp/active_brownian.cpp:28-37, each its own launches and its own effect on the state, for a
 * caller that drives them one at a time as main() does.  Called in the reference's order
 * after rotation_mpcd and run (MPCD_ERR_STATE otherwise), the n_sub passes give mpcd_substep's
 * bits.  update_pos_md opens substep l (the next one) and update_velocity_colloid closes it;
 * after the last substep it also bins the fluid for the next rotation_mpcd and records the
 * next run()'s rear-shell candidates (what the fused step's last streaming pass does).  The
 * FP64 form only (MPCD_ERR_STATE for MPCD_FP32C). */
/* update_pos_md (cpp/update.cpp:48-54), after old_force = f (cpp/active_brownian.cpp:28) */
int mpcd_update_pos_md(mpcd_ctx *c);
/* neighbour_list_md (cpp/neighbour_list.cpp:27-39): the colloid pair list within 3 sig_colloid,
 * built from a grid of buckets at least that wide (mpcd_get_neighbour_md reads it) */
int mpcd_neighbour_list_md(mpcd_ctx *c);
/* update_pos_mpcd (cpp/update.cpp:56-60) */
int mpcd_update_pos_mpcd(mpcd_ctx *c);
/* neighbour_list_mpcd (cpp/neighbour_list.cpp:41-58): the per-cell colloid table the collision
 * scans, rebuilt at the present colloid positions, and the reference's box binning and
 * per-colloid candidate counts (mpcd_get_box_binning reads them) */
int mpcd_neighbour_list_mpcd(mpcd_ctx *c);
/* fluid_colloid_collision (cpp/fluid_colloid_collision.cpp:26-49): the reflections and the
 * colloids' velocity and angular-velocity changes */
int mpcd_fluid_colloid_collision(mpcd_ctx *c);
/* update_activity_direction (cpp/update.cpp:34-46), with the rotational diffusion Dr */
int mpcd_update_activity_direction(mpcd_ctx *c);
/* compute_force_md (cpp/update.cpp:14-32) over the pair list of the last neighbour_list_md */
int mpcd_compute_force_md(mpcd_ctx *c);
/* update_velocity_colloid (cpp/update.cpp:62-67) */
int mpcd_update_velocity_colloid(mpcd_ctx *c);
/* the pair list of the last mpcd_neighbour_list_md as the reference keeps it
 * (neighbour[k][i], cpp/neighbour_list.cpp:35): per colloid i (0-based) count[i] partners
 * j > i, ascending, 0-based, in partners[i * cap + k] (up to cap per colloid) */
int mpcd_get_neighbour_md(mpcd_ctx *c, int32_t *count, int32_t *partners, int cap);
/* the last mpcd_neighbour_list_mpcd's binning (cpp/neighbour_list.cpp:44-47): per particle its
 * 1-based box number 1 + cell(pos) (cell_of[N]), per box 1..C its occupancy fluid_no
 * (occupancy[C]), per colloid its candidate count no_neigh (no_neigh[Nc]); NULL skips */
int mpcd_get_box_binning(mpcd_ctx *c, int32_t *cell_of, int32_t *occupancy, int32_t *no_neigh);
/* nsteps complete MPCD steps (rotation_mpcd, run, n_sub substeps) — the loop of
 * cpp/active_brownian.cpp:23-56, replayed as one CUDA graph per step */
int mpcd_step(mpcd_ctx *c, int nsteps);
/* The same steps enqueued on the context's stream without waiting for them (no host
 * synchronisation), for callers that step many contexts on one stream or overlap the steps
 * with their own work; mpcd_sync waits for them and reports what went wrong on the device
 * (as mpcd_step does before returning).  Other calls read the state only after the work
 * enqueued before them (they synchronise). */
int mpcd_step_async(mpcd_ctx *c, int nsteps);
int mpcd_sync(mpcd_ctx *c);
/* The free-flight schedule (on by default, both forms), used by mpcd_step: a fluid particle that no colloid can reach during the step (farther
 * from every colloid at its start than the run() shell radius sigma/2 + 1/2 plus its own travel
 * in the step plus n_sub times the colloids' bound on a substep's move) is streamed through all
 * substeps and binned by one pass, with the operations the substep passes would apply to it,
 * beside the substeps of the other (near) particles, which the substep passes walk alone.  The
 * results are those of the schedule without it, bit for bit.  mpcd_get_flight gives the near
 * particles of the last step that used it. */
int mpcd_set_flight(mpcd_ctx *c, int on);
int mpcd_get_flight(mpcd_ctx *c, int32_t *near);
/* diagnostics of the state now (cpp/active_brownian.cpp:39-55) */
int mpcd_diag(mpcd_ctx *c, mpcd_diag_t *out);

/* ---- observables for parity checks --------------------------------------------------- */
/* the last rotation binning: per particle its 1-based cell number as rotation_mpcd computes
 * it (1 + cell(mod(pos + rr, len)), cpp/rotation_mpcd.cpp:11) and per cell its occupancy
 * (fluid_no[1..C]); either pointer may be NULL */
int mpcd_get_rotation_binning(mpcd_ctx *c, int32_t *cell_of, int32_t *occupancy, double *shift);
/* run(): the rear-shell particle count per colloid of the last run (cnt[1..Nc]) */
int mpcd_get_shell_count(mpcd_ctx *c, int32_t *cnt);

/* ---- profiling ------------------------------------------------------------------------ */
/* when enabled, every kernel launch is bracketed by CUDA events on the launch stream */
int mpcd_profile_enable(mpcd_ctx *c, int on);
/* per kernel: name, launches, total ms; returns the number of kernels (writes up to cap) */
int mpcd_profile_read(mpcd_ctx *c, char names[][48], int64_t *launches, double *total_ms, int cap);
/* one MPCD step (a real step: the state advances) as a graph with a timing event before and
 * after every launch, replayed once and synchronised: launch i's kernel name and its start
 * and end in ms from the step's start (the graph's own timeline, streams overlapped as in
 * mpcd_step).  Returns the number of launches (entries beyond cap are not written) or a
 * negative MPCD_ERR_*. */
int mpcd_trace_step(mpcd_ctx *c, char names[][48], double *t0_ms, double *t1_ms, int cap);
/* kernels launched by this context since creation (all of them are this library's own) */
int64_t mpcd_launch_count(const mpcd_ctx *c);

/* ---- launch shapes (no counterpart in the reference: tuning of this implementation) -- */
enum { MPCD_LAUNCH_EVENTS = 0, /* wall-collision events: grid, block (<= 128, multiple of 32) */
       MPCD_LAUNCH_FIN = 1,    /* colloid finish: grid, block (<= 128, multiple of 32); the FP64
                                  form runs one block of 256 per colloid (it also builds the
                                  cell tables) and ignores this shape */
       MPCD_LAUNCH_AUX = 2,    /* colloid side work (forces, cell table, orientation; a kernel on a
                                  second stream beside the streaming and event passes): grid > 0
                                  sets, block = threads per colloid (64, 128 or 256) */
       MPCD_LAUNCH_FREE = 3 }; /* free-flight pass (a persistent grid beside the substeps): grid
                                  blocks of 256 threads; block = in the FP64 form the substep
                                  after whose colloid finish it starts (0: right after the
                                  classification; the default is 1) */
/* grid <= 0 restores the default (events: one block of 128 threads per SM; finish: one block of
 * 32 per SM; side work: 128 threads per colloid, 64 in the FP64 form, whose colloid finish builds
 * the cell tables; free flight: two blocks per SM); results do not depend on the shape (every
 * sum is exact); drops the captured step graphs */
int mpcd_set_launch(mpcd_ctx *c, int which, int grid, int block);

/* ---- exchange record (no counterpart in the reference) ------------------------------- */
/* The momentum (m sum dv, 3) and angular momentum (m sum r x dv, 3) the fluid gave each colloid
 * in the stochastic reflections (cpp/fluid_colloid_collision.cpp:46-47) since the last reset:
 * out[6 j + k], Nc x 6 doubles (NULL: reset only).  The training data of the learned closure. */
int mpcd_exchange_read(mpcd_ctx *c, double *out, int reset);

/* ---- updown_velocity (replaces cpp/run.cpp:28-50) ---------------------------------------- */
/* On the current state, per colloid j: the fluid particles of the 342 boxes around the colloid's
 * box (own box excluded) on its rear side (r.V <= 0, r = img(pos_fl - pos_colloid)) within
 * sigma/2 + 0.5 (cnt[j], the run() shell) and within sigma/2 + 0.1 (up_cnt[j]), and the sums of
 * their velocities (vel_sum[3 j + k], up_vel_sum[3 j + k]; exact sums).  The reference's slip
 * velocities follow from these (its results are discarded; the Python wrapper restates its
 * arithmetic).  Any pointer may be NULL. */
int mpcd_updown_velocity(mpcd_ctx *c, int32_t *cnt, int32_t *up_cnt, double *vel_sum, double *up_vel_sum);

/* ---- colloid trajectories and their statistics (no counterpart: the reference's analysis
 *      prints are commented out, cpp/active_brownian.cpp:44-46) ---------------------------- */
/* A device-resident recorder: per frame the colloids' unwrapped positions, velocities and
 * orientations (FP64).  Frames of one trajectory come from one source, between steps. */
typedef struct mpcd_traj mpcd_traj;
struct mpcd_surrogate; /* the colloid-only step, declared below */
int mpcd_traj_create(int n_colloid, int max_frames, const double *box /* 3 */, mpcd_traj **out);
int mpcd_traj_destroy(mpcd_traj *t);
const char *mpcd_traj_last_error(const mpcd_traj *t);
int mpcd_traj_frames(const mpcd_traj *t);
int mpcd_traj_reset(mpcd_traj *t);                              /* drops the frames */
int mpcd_traj_record(mpcd_traj *t, mpcd_ctx *c);                /* a frame of a context's colloids */
int mpcd_traj_record_surrogate(mpcd_traj *t, struct mpcd_surrogate *s); /* a frame of the colloid-only step */
/* per lag (in frames): MSD <|U(t+lag) - U(t)|^2>, VACF <V(t+lag).V(t)>, OACF <ra(t+lag).ra(t)>,
 * averaged over time origins and colloids (NaN where no two frames are lag apart); any output
 * may be NULL; deterministic */
int mpcd_traj_analyse(mpcd_traj *t, const int *lags, int nlags, double *msd, double *vacf, double *oacf);
/* frames [first, first + count) to host arrays, count x n_colloid x 3 each (NULL: skip) */
int mpcd_traj_read(mpcd_traj *t, int first, int count, double *pos, double *vel, double *ra);
/* the file "BGBTRAJ1" + int32 version, n_colloid, n_frames, fields + double box[3], dt_frame,
 * then per frame positions, velocities, orientations (n_colloid x 3 doubles each) */
int mpcd_traj_write(mpcd_traj *t, const char *path, double dt_frame);

/* ---- batched ensemble (no counterpart in the reference) ------------------------------- */
/* nrep independent systems with their own parameters p[0..nrep-1] (box, fluid, colloids,
 * activity, seed; all MPCD_FP32C with equal n_sub and sort_every) stepped together: every
 * stage of an MPCD step is one launch over all systems, the step one CUDA graph.  Each
 * system is an ordinary context (mpcd_ensemble_system): initialise or set its state, call
 * mpcd_setup and read it back through the single-system calls; step it only through
 * mpcd_ensemble_step.  The ensemble owns the contexts. */
typedef struct mpcd_ensemble mpcd_ensemble;
int mpcd_ensemble_create(const mpcd_params *p, int nrep, mpcd_ensemble **out);
int mpcd_ensemble_destroy(mpcd_ensemble *e);
const char *mpcd_ensemble_last_error(const mpcd_ensemble *e);
mpcd_ctx *mpcd_ensemble_system(mpcd_ensemble *e, int r);
/* nsteps MPCD steps of every system (all set up, at the same step); synchronises */
int mpcd_ensemble_step(mpcd_ensemble *e, int nsteps);
enum { MPCD_ENS_EVENTS = 0,  /* blocks per system of the event pass (1..64) */
       MPCD_ENS_RUN = 1,     /* blocks per system of run() (1..64) */
       MPCD_ENS_FIN = 2,     /* threads per block of the colloid finish (32, 64, 128) */
       MPCD_ENS_AUX = 3,     /* threads per colloid of the colloid side work (64, 128, 256) */
       MPCD_ENS_FREE = 4 };  /* resident blocks per SM of the free-flight pass (1..8; block ignored) */
/* launch shapes of the batched step (the autotuner's knobs); results do not depend on them */
int mpcd_ensemble_set_launch(mpcd_ensemble *e, int which, int per_system, int block);
/* kernels the ensemble launched since creation */
int64_t mpcd_ensemble_launch_count(const mpcd_ensemble *e);
/* the schedule of the batched step: the free-flight schedule (on = 1, the default: particles
 * no colloid can reach in a step streamed through all substeps by one batched pass beside the
 * other particles' substeps) or one pass over every particle per substep (on = 0).  Both
 * leave the same bits. */
int mpcd_ensemble_set_flight(mpcd_ensemble *e, int on);
int mpcd_ensemble_get_flight(const mpcd_ensemble *e);

/* ---- learned closure network (no counterpart in the reference) ----------------------- */
/* MLP 81 -> 256 -> 256 -> 256 -> 12 with SiLU, BF16 weights on the tensor cores with FP32
 * accumulation and FP32 master weights for Adam.  Inputs: a colloid's 81 closure features
 * (raw units; normalised inside by mpcd_mlp_set_normalisation's statistics).  Outputs: the
 * means (6) and log-variances (6) of its per-step momentum and angular-momentum exchange with
 * the fluid, in physical units.  x, y and out are device pointers (rows x 81, rows x 6,
 * rows x 12 floats); rows <= max_batch.  Parameters as one flat FP32 vector (W1 [81][256], b1,
 * W2 [256][256], b2, W3, b3, W4 [256][12], b4).  Weight gradients are summed with FP32 atomics,
 * so a gradient is reproducible only to rounding. */
#define MPCD_MLP_IN 81
#define MPCD_MLP_HIDDEN 256
#define MPCD_MLP_OUT 12
typedef struct mpcd_mlp mpcd_mlp;
int mpcd_mlp_create(int max_batch, uint64_t seed, mpcd_mlp **out);
int mpcd_mlp_destroy(mpcd_mlp *n);
const char *mpcd_mlp_last_error(const mpcd_mlp *n);
int64_t mpcd_mlp_param_count(const mpcd_mlp *n);
int mpcd_mlp_set_normalisation(mpcd_mlp *n, const float *x_mean, const float *x_std, const float *y_mean,
                               const float *y_std);
int mpcd_mlp_get_params(mpcd_mlp *n, float *out_host);
int mpcd_mlp_set_params(mpcd_mlp *n, const float *in_host);
/* inference, asynchronous on `stream` */
int mpcd_mlp_forward(mpcd_mlp *n, const float *x, int rows, float *out, void *stream);
/* mean Gaussian negative log-likelihood of y and its gradient (host, param_count floats; NULL: skip) */
int mpcd_mlp_grad(mpcd_mlp *n, const float *x, const float *y, int rows, float *grad_host, double *loss_host);
/* one Adam step (beta 0.9, 0.999) on the batch; loss_host receives the batch loss before the step */
int mpcd_mlp_train_step(mpcd_mlp *n, const float *x, const float *y, int rows, float lr, double *loss_host);
/* Training's layer products wait for their tensor-core results with a bound (100 ms); one that
 * runs out makes mpcd_mlp_grad / mpcd_mlp_train_step fail with MPCD_ERR_CUDA ("did not complete
 * within its time limit"), and the next call starts afresh.  For tests of that path this hook
 * (on = 1) makes the products issue nothing, so that every wait runs out; 0 clears it. */
int mpcd_mlp_set_fault(mpcd_mlp *n, int on);

/* ---- colloid-only dynamics with the learned closure (no counterpart in the reference) -- */
/* The colloids of p (box, n_colloid <= MPCD_SURROGATE_MAX_COLLOIDS, n_sub <= 32, ndt, masses, WCA
 * sig_colloid/eps, sphere diameter sigma, v0, Dr, seed; n_fluid ignored) without the fluid:
 * each MPCD step the network `net` (borrowed, not owned; its weights are read at every
 * mpcd_surrogate_step call) predicts every colloid's fluid exchange, a Gaussian draw of it is
 * applied as an impulse together with run()'s active kick, then n_sub velocity-Verlet substeps
 * with WCA forces and the orientation update, in FP32.  One CUDA graph of two kernels per
 * step: the features and the whole network in one kernel over the GPU (16 colloids per
 * block), the substeps in one cluster of 8 blocks. */
#define MPCD_SURROGATE_MAX_COLLOIDS 2048
typedef struct mpcd_surrogate mpcd_surrogate;
int mpcd_surrogate_create(const mpcd_params *p, mpcd_mlp *net, mpcd_surrogate **out);
int mpcd_surrogate_destroy(mpcd_surrogate *s);
const char *mpcd_surrogate_last_error(const mpcd_surrogate *s);
/* state as n_colloid x 3 doubles (host); set_state also computes the forces */
int mpcd_surrogate_set_state(mpcd_surrogate *s, const double *pos, const double *vel, const double *ang_vel,
                             const double *ra);
int mpcd_surrogate_get_state(mpcd_surrogate *s, double *pos, double *vel, double *ang_vel, double *ra);
/* network inputs (n_colloid x 81 floats, host): those of the current state (recompute != 0),
 * or those the last step fed the network (recompute = 0: the state before that step) */
int mpcd_surrogate_features(mpcd_surrogate *s, float *out, int recompute);
/* the network's outputs of the last step in physical units (n_colloid x 12 floats, host; the
 * arithmetic of mpcd_mlp_forward on the last step's inputs) */
int mpcd_surrogate_outputs(mpcd_surrogate *s, float *out);
/* nsteps MPCD steps; synchronises */
int mpcd_surrogate_step(mpcd_surrogate *s, int nsteps);
/* Steps so far (since create) in which some colloid moved more than 1.0: the WCA force
 * partners of a step are the pairs within the cutoff plus 2 at its start, so such a step
 * may miss a collision.  Colloids of the trained closure move about 0.01 per step; the
 * count rises for dynamics without drag (e.g. a network that predicts no exchange). */
int mpcd_surrogate_fast_steps(mpcd_surrogate *s, int64_t *count);
/* Every wait of the network kernel on its weight copies is bounded (100 ms); a copy that
 * does not arrive makes the step fail with MPCD_ERR_CUDA ("a weight copy of the network
 * kernel did not arrive"), the call's remaining steps are skipped and the colloid state stays
 * as it was before the failing step; the next mpcd_surrogate_step starts afresh.  For tests of
 * that path this hook makes the kernel's producer skip weight chunk `drop_chunk` (6..19; -1:
 * none) so that the waits run out; the copies it does issue all land before the kernel ends. */
int mpcd_surrogate_set_fault(mpcd_surrogate *s, int drop_chunk);
/* Scale of the drawn exchange's fluctuation about the network's mean: 1 (the default) draws
 * with the network's predicted variance, 0 applies the predicted mean only (a deterministic
 * drag without the fluctuations that balance it). */
int mpcd_surrogate_set_noise(mpcd_surrogate *s, double scale);

/* ---- fluid sums without allocation (no counterpart in the reference) ---------------- */
/* For callers that cannot call cudaMalloc: their device memory is all handed out by their
 * own pool (for example a framework's caching allocator that already holds the GPU), or
 * they must not take the device synchronisation an allocation can cause mid-pipeline.
 * Momentum (mass * sum v, three doubles) and kinetic energy (mass/2 * sum |v|^2) of n
 * particles whose velocities `vel` (device memory, n x 3 doubles, the layout of
 * mpcd_set_state's vel_fl) the caller owns, written to `out` (device memory, four
 * doubles), asynchronously on `stream` (NULL: the legacy default stream).  The same sums
 * as the fluid part of mpcd_diag, with no context.  Its per-block partial sums live in a
 * fixed 512 KiB array of the library that every GPU loading it holds until exit; nothing
 * is allocated.  The first call on a device looks up that array's device address (make it
 * before any stream capture); the address is kept for the life of the device's primary
 * context, so after a cudaDeviceReset of that device the process must not call this
 * function again.  All calls share the array: calls that overlap on the GPU (other
 * streams, other threads) race.  Returns MPCD_ERR_CAPACITY, with a message on stderr, for
 * n > MPCD_NOALLOC_MAX_PARTICLES; returns MPCD_ERR_CUDA without launching (and without
 * clearing that error) when an earlier CUDA error is pending on the calling thread. */
#define MPCD_NOALLOC_MAX_PARTICLES 33554432LL
int mpcd_fluid_sums_noalloc(const double *vel, int64_t n, double mass, double *out, void *stream);

#ifdef __cplusplus
}
#endif
#endif
