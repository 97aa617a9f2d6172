/*
 * CPU oracle for the MPCD + active-colloid time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * serial C++ step (cpp/ in shashankgandham/brownian), used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
 * The product (brownian_gb300) never links, loads or calls it.
 *
 * Every routine follows the reference routine of the same name operation for
 * operation (same loop order, same floating-point expression order, no FMA
 * contraction), so that with the reference's own sequential ran() stream
 * (ORC_RNG_SEQ) it reproduces the compiled reference bit for bit; that is
 * pinned by tests/test_oracle_pin.py against traces of the reference itself.
 *
 * With ORC_RNG_KEYED every random number is instead a Philox4x32-10 draw keyed
 * by what it is for (grid shift of step n, rotation axis of cell c at step n,
 * reflection of particle l off colloid j at substep s, ...), so that a parallel
 * implementation can draw the same numbers in any order.  That is the mode the
 * GPU path is compared against.
 */
#ifndef MPCD_ORACLE_H
#define MPCD_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_RNG_SEQ = 0, ORC_RNG_KEYED = 1 };

/* Philox draw domains (counter word 3, bits 24..31).  Shared numbering with the
 * GPU path; the GPU path has its own implementation of the generator. */
enum {
  ORC_DOM_SHIFT = 1,      /* ctr = (0, 0, step, dom|0)                          */
  ORC_DOM_AXIS = 2,       /* ctr = (cell(1-based), 0, step, dom|0)              */
  ORC_DOM_COLL = 3,       /* ctr = (particle, colloid, substep, dom|block)      */
  ORC_DOM_TUMBLE = 4,     /* ctr = (colloid, 0, 0, dom|0)                       */
  ORC_DOM_ROTDIFF = 5,    /* ctr = (colloid, 0, substep, dom|0)                 */
  ORC_DOM_INIT_CPOS = 6,  /* ctr = (colloid, attempt, 0, dom|0)                 */
  ORC_DOM_INIT_CVEL = 7,  /* ctr = (colloid, 0, 0, dom|0)                       */
  ORC_DOM_INIT_FPOS = 8,  /* ctr = (particle, attempt, 0, dom|0)                */
  ORC_DOM_INIT_FVEL = 9   /* ctr = (particle, 0, 0, dom|0)                      */
};

typedef struct {
  int Lx, Ly, Lz;          /* box in unit cells (reference: len)                */
  int n_fluid;             /* reference: no_of_fluid                            */
  int n_colloid;           /* reference: no_of_colloid                          */
  int n_sub;               /* MD substeps per MPCD step (reference: n)          */
  double kbt, kbt1;        /* fluid / colloid-init temperature                  */
  double ndt;              /* MPCD step (reference: ndt); dt = ndt / n_sub      */
  double mass_fl, mass_colloid;
  double sig_colloid;      /* WCA sigma (reference: sig_colloid)                */
  double eps;              /* WCA epsilon                                       */
  double sigma;            /* colloid diameter (reference: sigma)               */
  double I_colloid;        /* moment of inertia                                 */
  double v0;               /* self-propulsion speed                             */
  double theta_deg;        /* SRD rotation angle in degrees (reference: 130)    */
  double Dr;               /* rotational diffusion (no reference counterpart; 0 reproduces it) */
  int rng_mode;            /* ORC_RNG_SEQ or ORC_RNG_KEYED                      */
  int64_t seed;            /* SEQ: initial reference `seed`; KEYED: Philox key  */
  int physics;             /* 1: the corrected rules (own box a candidate, 2-D tangential
                              reflection) the library offers as MPCD_PHYSICS_FIXED; 0: the reference */
} orc_params;

typedef struct orc_ctx orc_ctx;

orc_ctx *orc_create(const orc_params *p);
void orc_destroy(orc_ctx *c);
const char *orc_error(const orc_ctx *c);

/* reference routines (cpp/): each one is the same-named reference function */
int orc_initialize_colloid(orc_ctx *c);     /* cpp/initialize.cpp:31-60     */
int orc_initialize_fluid(orc_ctx *c);       /* cpp/initialize.cpp:62-83     */
int orc_create_box(orc_ctx *c);             /* cpp/neighbour_list.cpp:12-25 */
int orc_neighbour_list_md(orc_ctx *c);      /* cpp/neighbour_list.cpp:27-39 */
int orc_neighbour_list_mpcd(orc_ctx *c);    /* cpp/neighbour_list.cpp:41-58 */
int orc_rotation_mpcd(orc_ctx *c);          /* cpp/rotation_mpcd.cpp:3-50   */
int orc_run(orc_ctx *c);                    /* cpp/run.cpp:10-26            */
int orc_tumble(orc_ctx *c);                 /* cpp/run.cpp:3-8              */
int orc_fluid_colloid_collision(orc_ctx *c);/* cpp/fluid_colloid_collision.cpp:26-49 */
int orc_compute_force_md(orc_ctx *c);       /* cpp/update.cpp:14-32         */
int orc_update_activity_direction(orc_ctx *c); /* cpp/update.cpp:34-46      */
int orc_update_pos_md(orc_ctx *c);          /* cpp/update.cpp:48-54         */
int orc_update_pos_mpcd(orc_ctx *c);        /* cpp/update.cpp:56-60         */
int orc_update_velocity_colloid(orc_ctx *c);/* cpp/update.cpp:62-67         */
int orc_updown_velocity(orc_ctx *c, double *vel_out /* 3*Nc */, double *up_vel_out /* 3 */); /* cpp/run.cpp:28-50 */
/* the same selection as orc_updown_velocity: per colloid the counts of the run() shell and of
 * the inner shell and the (sequential) sums of their velocities, 3*Nc each */
int orc_updown_sums(orc_ctx *c, int *cnt, int *up_cnt, double *vel_sum, double *up_vel_sum);

/* driver pieces (cpp/active_brownian.cpp) */
int orc_setup(orc_ctx *c);       /* create_box, neighbour_list_mpcd, neighbour_list_md, compute_force_md (:17-20) */
int orc_substep(orc_ctx *c, int l); /* one pass of the inner loop body (:28-37); sets substep counter l */
int orc_begin_substep(orc_ctx *c, int l); /* what the loop does before update_pos_md (:27-28): substep
                                             counter l, old_force = f */
int orc_step(orc_ctx *c);        /* nn += 1; rotation_mpcd, run, n_sub substeps (:23-38) */
int orc_run_steps(orc_ctx *c, int nsteps);

/* step counter nn (the reference's global, 1-based inside a step) */
int orc_get_step(const orc_ctx *c);
void orc_set_step(orc_ctx *c, int nn);

/* diagnostics of cpp/active_brownian.cpp:39-55, momentum reset per call:
 * out[0] ke_fluid, [1] ke_colloid, [2] ang_ke_colloid, [3] potential_colloid,
 * [4] energy_colloid, [5..7] total momentum (fluid + colloid), [8] sum |p_i| */
void orc_diag(const orc_ctx *c, double *out);

/* state I/O, 0-based, AoS xyz triplets.  which: 0 pos_fl, 1 vel_fl, 2 pos_colloid,
 * 3 vel_colloid, 4 ang_vel_colloid, 5 ra, 6 f, 7 old_force */
int orc_get(const orc_ctx *c, int which, double *out);
int orc_set(orc_ctx *c, int which, const double *in);
double orc_potential(const orc_ctx *c);

/* binning observables.  kind 0: the last rotation_mpcd binning (shifted cells),
 * kind 1: the last neighbour_list_mpcd binning (unshifted cells).
 * cell_of: per particle, the 1-based cell number the reference computed
 * (1 + cell(...)), may exceed Lx*Ly*Lz for coordinates exactly at L.
 * occupancy: fluid_no[1..C] (C = Lx*Ly*Lz). */
int orc_get_binning(const orc_ctx *c, int kind, int32_t *cell_of, int32_t *occupancy);
/* the last grid shift used by rotation_mpcd */
void orc_get_shift(const orc_ctx *c, double *rr3);
/* the colloid pair list of the last neighbour_list_md: partners (1-based, ascending, all > i)
 * of colloid i (1-based); returns the count, writes up to cap */
int orc_get_neighbour_md(const orc_ctx *c, int i, int32_t *out, int cap);
/* neigh_fl of colloid j (1-based): returns count, writes up to cap particle ids (1-based) */
int orc_get_neigh_fl(const orc_ctx *c, int j, int32_t *out, int cap);
/* the 342-cell neighbour table of box b (1-based) in reference order; returns count */
int orc_box_neighbours(const orc_ctx *c, int b, int32_t *out);
/* run(): number of rear-shell particles per colloid from the last call */
int orc_get_shell_count(const orc_ctx *c, int32_t *cnt);

/* raw generators (for known-answer tests) */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double orc_ran_seq(orc_ctx *c);   /* one draw of the reference ran() stream */

#ifdef __cplusplus
}
#endif
#endif
