/*
 * CPU oracle for the MPCD + active-colloid time step — TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the reference's serial C++ step (cpp/ of
 * shashankgandham/brownian).  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg use it, as the checker; the product never links it.
 *
 * Faithfulness rules followed throughout:
 *   - arrays are 1-based with the reference's loop bounds and loop order;
 *   - every floating-point expression keeps the reference's evaluation order
 *     (the `point` operators of cpp/parameters.hpp:44-71 are component-wise, and
 *     point::sum() is (x + y) + z);
 *   - the build uses -ffp-contract=off so no multiply-add is fused;
 *   - libm's pow/sqrt/log/sin/cos/asin/lround are called where the reference calls them.
 * The reference's fixed-capacity tables (maxpart = 100 per cell, 10000 candidates
 * per colloid, 200 pair neighbours, 7000 shell particles) become growable lists;
 * where the reference would overrun them this oracle keeps going correctly.
 */
#include "mpcd_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct { double x, y, z; } V3;

static inline V3 v3(double x, double y, double z) { V3 r = {x, y, z}; return r; }
static inline V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 mulv(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline V3 muls(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline V3 divs(V3 a, double s) { return v3(a.x / s, a.y / s, a.z / s); }
static inline V3 divv(V3 a, V3 b) { return v3(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline double vsum(V3 a) { return a.x + a.y + a.z; }
/* cpp/parameters.hpp:74 round(): lround per component */
static inline V3 vround(V3 a) { return v3((double)lround(a.x), (double)lround(a.y), (double)lround(a.z)); }
/* cpp/parameters.hpp:75 mod(a,b) = a - b*round((a - b/2)/b): periodic wrap to [0, L] */
static inline V3 vmod(V3 a, V3 b) { return sub(a, mulv(b, vround(divv(sub(a, divs(b, 2.0)), b)))); }
/* cpp/parameters.hpp:76 img(a,b) = a - b*round(a/b): minimum image */
static inline V3 vimg(V3 a, V3 b) { return sub(a, mulv(b, vround(divv(a, b)))); }
/* cpp/fluid_colloid_collision.cpp:3-5 */
static inline V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
/* cpp/parameters.hpp:59 point::cell(len): int(x) + len.x*int(y) + len.x*len.y*int(z) */
static inline int vcell(V3 p, V3 len) {
  return (int)((double)(int)p.x + len.x * (double)(int)p.y + len.x * len.y * (double)(int)p.z);
}

typedef struct { int32_t *v; int n, cap; } ilist;
static int ilist_push(ilist *l, int32_t x) {
  if (l->n == l->cap) {
    int nc = l->cap ? 2 * l->cap : 64;
    int32_t *nv = (int32_t *)realloc(l->v, sizeof(int32_t) * (size_t)nc);
    if (!nv) return -1;
    l->v = nv; l->cap = nc;
  }
  l->v[l->n++] = x;
  return 0;
}

struct orc_ctx {
  orc_params p;
  V3 len;
  int C;            /* Lx*Ly*Lz */
  int Cpad;         /* cell-array size: cell numbers can exceed C for coordinates exactly at L */
  double dt;
  /* constants of cpp/update.cpp:3-6, recomputed from the parameters */
  double r_cutoff, fc, ufc, sig12, sig6;
  /* state, 1-based with two spare slots as cpp/initialize.cpp:15-18 allocates */
  V3 *pos_fl, *vel_fl, *dump_vel_fl;
  V3 *pos_colloid, *vel_colloid, *ang_vel_colloid, *f, *old_force, *ra;
  double potential_colloid;
  /* binning */
  int32_t *fluid_no;       /* per cell count (Cpad)                       */
  int32_t *cell_start;     /* CSR offsets (Cpad+1)                        */
  int32_t *cell_list;      /* particles, ascending within each cell (N)   */
  int32_t *cell_of;        /* per particle cell number of the last binning */
  int last_kind;           /* 0 rotation, 1 neighbour_list_mpcd, -1 none  */
  int32_t *rot_cell_of, *rot_occ;  /* saved rotation binning            */
  int32_t *box_cell_of, *box_occ;  /* saved neighbour_list_mpcd binning */
  V3 last_rr;
  /* neighbour lists */
  ilist *neigh_fl;         /* per colloid (1-based) */
  ilist *neighbour;        /* colloid pair list, per colloid (1-based) */
  ilist *nbr, *up_nbr;     /* run() / updown_velocity() shells */
  int box_ready;
  /* reference ran() state: the global `seed`, the global `iv` table and the
   * function statics idum and iy (cpp/parameters.hpp:16-42) */
  int seed_i, idum, iy;
  int iv[34];
  /* step / substep counters */
  int nn, l;
  char err[256];
};

static void set_err(orc_ctx *c, const char *m) { snprintf(c->err, sizeof c->err, "%s", m); }
const char *orc_error(const orc_ctx *c) { return c->err; }

/* ---------------------------------------------------------------- generators */

/* The reference ran(): L'Ecuyer's two combined LCGs with a Bays-Durham shuffle
 * (Numerical Recipes ran2), including its quirks: the shuffle table is only
 * initialised for seed <= 0, and with the reference's positive seed the table
 * stays zero (cpp/parameters.hpp:16-42). */
static double ran_seq(orc_ctx *c) {
  const int im1 = 2147483563, im2 = 2147483399, ia1 = 40014, ia2 = 40692, iq1 = 53668, iq2 = 52774;
  const int imm = im1 - 1, ir1 = 12211, ir2 = 3791, ntab = 32, ndiv = 1 + imm / ntab;
  const double eps = 1.2e-7, rnmx = 1 - eps, am = 1.0 / im1;
  int k, j;
  if (c->seed_i <= 0) {
    c->seed_i = (-c->seed_i > 1) ? -c->seed_i : 1;
    c->idum = c->seed_i;
    for (j = ntab + 8; j >= 1; j--) {
      k = c->seed_i / iq1;
      c->seed_i = ia1 * (c->seed_i - k * iq1) - k * ir1;
      if (c->seed_i < 0) c->seed_i += im1;
      if (j <= ntab) c->iv[j] = c->seed_i;
    }
    c->iy = c->iv[1];
  }
  k = c->seed_i / iq1;
  c->seed_i = ia1 * (c->seed_i - k * iq1) - k * ir1;
  if (c->seed_i < 0) c->seed_i += im1;
  k = c->idum / iq2;
  c->idum = ia2 * (c->idum - k * iq2) - k * ir2;
  if (c->idum < 0) c->idum = c->idum + im2;
  j = 1 + c->iy / ndiv;
  c->iy = c->iv[j] - c->idum;
  c->iv[j] = c->seed_i;
  if (c->iy < 1) c->iy = c->iy + imm;
  double r = am * c->iy;
  return (rnmx < r) ? rnmx : r;
}
double orc_ran_seq(orc_ctx *c) { return ran_seq(c); }

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
 * as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies with a Weyl key
 * schedule. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1, n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* uniform in (0,1): (w + 1/2) * 2^-32, exact in double */
static inline double u01(uint32_t w) { return ldexp((double)w + 0.5, -32); }

static void keyed4(const orc_ctx *c, uint32_t dom, uint32_t blk, uint32_t a, uint32_t b, uint32_t t, double u[4]) {
  uint32_t ctr[4] = {a, b, t, (dom << 24) | (blk & 0xFFFFFFu)};
  uint32_t key[2] = {(uint32_t)(uint64_t)c->p.seed, (uint32_t)((uint64_t)c->p.seed >> 32)};
  uint32_t o[4];
  orc_philox4x32_10(ctr, key, o);
  for (int i = 0; i < 4; ++i) u[i] = u01(o[i]);
}

/* a sequence of draws for one purpose: the reference stream in SEQ mode, or the
 * blocks 0, 1, 2, ... of one Philox key in KEYED mode */
typedef struct { orc_ctx *c; uint32_t dom, a, b, t; int idx; double buf[4]; } drawseq;
static drawseq ds_make(orc_ctx *c, uint32_t dom, uint32_t a, uint32_t b, uint32_t t) {
  drawseq d; d.c = c; d.dom = dom; d.a = a; d.b = b; d.t = t; d.idx = 0; return d;
}
static double ds_next(drawseq *d) {
  if (d->c->p.rng_mode == ORC_RNG_SEQ) return ran_seq(d->c);
  if ((d->idx & 3) == 0) keyed4(d->c, d->dom, (uint32_t)(d->idx >> 2), d->a, d->b, d->t, d->buf);
  return d->buf[d->idx++ & 3];
}
/* point::random(dec, mul) (cpp/parameters.hpp:61-65): x, y, z drawn in order,
 * then (*this)*mul - dec */
static V3 ds_point(drawseq *d, V3 dec, V3 mul) {
  V3 t;
  t.x = ds_next(d); t.y = ds_next(d); t.z = ds_next(d);
  return sub(mulv(t, mul), dec);
}

/* ------------------------------------------------------------------ lifetime */

orc_ctx *orc_create(const orc_params *p) {
  orc_ctx *c = (orc_ctx *)calloc(1, sizeof(orc_ctx));
  if (!c) return NULL;
  c->p = *p;
  c->len = v3(p->Lx, p->Ly, p->Lz);
  c->C = p->Lx * p->Ly * p->Lz;
  /* a coordinate exactly at L gives int(x) = L; the largest cell number is then
   * 1 + L + Lx*L + Lx*Ly*L */
  c->Cpad = c->C + p->Lx * p->Ly + p->Lx + p->Lx + 4;
  c->dt = p->ndt / (double)p->n_sub;
  /* cpp/update.cpp:3-6 */
  c->r_cutoff = pow(2, 1.0 / 6.0) * p->sig_colloid;
  c->fc = 4.0 * p->eps * (12.0 * (pow(p->sig_colloid, 12) / pow(c->r_cutoff, 13)) -
                          6.0 * (pow(p->sig_colloid, 6) / pow(c->r_cutoff, 7)));
  c->ufc = 4.0 * p->eps * (pow(p->sig_colloid / c->r_cutoff, 12) - pow(p->sig_colloid / c->r_cutoff, 6)) +
           c->fc * c->r_cutoff;
  c->sig12 = pow(p->sig_colloid, 12);
  c->sig6 = pow(p->sig_colloid, 6);
  int N = p->n_fluid, Nc = p->n_colloid;
  c->pos_fl = (V3 *)calloc((size_t)N + 2, sizeof(V3));
  c->vel_fl = (V3 *)calloc((size_t)N + 2, sizeof(V3));
  c->dump_vel_fl = (V3 *)calloc((size_t)N + 2, sizeof(V3));
  V3 **cp[] = {&c->pos_colloid, &c->vel_colloid, &c->ang_vel_colloid, &c->f, &c->old_force, &c->ra};
  for (int i = 0; i < 6; ++i) *cp[i] = (V3 *)calloc((size_t)Nc + 2, sizeof(V3));
  c->fluid_no = (int32_t *)calloc((size_t)c->Cpad, sizeof(int32_t));
  c->cell_start = (int32_t *)calloc((size_t)c->Cpad + 1, sizeof(int32_t));
  c->cell_list = (int32_t *)calloc((size_t)N + 2, sizeof(int32_t));
  c->cell_of = (int32_t *)calloc((size_t)N + 2, sizeof(int32_t));
  c->rot_cell_of = (int32_t *)calloc((size_t)N + 2, sizeof(int32_t));
  c->box_cell_of = (int32_t *)calloc((size_t)N + 2, sizeof(int32_t));
  c->rot_occ = (int32_t *)calloc((size_t)c->Cpad, sizeof(int32_t));
  c->box_occ = (int32_t *)calloc((size_t)c->Cpad, sizeof(int32_t));
  c->neigh_fl = (ilist *)calloc((size_t)Nc + 2, sizeof(ilist));
  c->neighbour = (ilist *)calloc((size_t)Nc + 2, sizeof(ilist));
  c->nbr = (ilist *)calloc((size_t)Nc + 2, sizeof(ilist));
  c->up_nbr = (ilist *)calloc((size_t)Nc + 2, sizeof(ilist));
  c->last_kind = -1;
  /* reference ran() state: global seed, static idum = 123456789, static iy = 0,
   * calloc'd iv table (cpp/parameters.hpp:17-18, cpp/initialize.cpp:13) */
  c->seed_i = (int)p->seed;
  c->idum = 123456789;
  c->iy = 0;
  c->nn = 0;
  c->l = 0;
  if (!c->pos_fl || !c->vel_fl || !c->dump_vel_fl || !c->fluid_no || !c->cell_start || !c->cell_list ||
      !c->neigh_fl || !c->neighbour || !c->nbr || !c->up_nbr || !c->ra) {
    orc_destroy(c);
    return NULL;
  }
  return c;
}

void orc_destroy(orc_ctx *c) {
  if (!c) return;
  free(c->pos_fl); free(c->vel_fl); free(c->dump_vel_fl);
  free(c->pos_colloid); free(c->vel_colloid); free(c->ang_vel_colloid); free(c->f); free(c->old_force); free(c->ra);
  free(c->fluid_no); free(c->cell_start); free(c->cell_list); free(c->cell_of);
  free(c->rot_cell_of); free(c->box_cell_of); free(c->rot_occ); free(c->box_occ);
  for (int j = 0; j < c->p.n_colloid + 2; ++j) {
    if (c->neigh_fl) free(c->neigh_fl[j].v);
    if (c->neighbour) free(c->neighbour[j].v);
    if (c->nbr) free(c->nbr[j].v);
    if (c->up_nbr) free(c->up_nbr[j].v);
  }
  free(c->neigh_fl); free(c->neighbour); free(c->nbr); free(c->up_nbr);
  free(c);
}

int orc_get_step(const orc_ctx *c) { return c->nn; }
void orc_set_step(orc_ctx *c, int nn) { c->nn = nn; }

/* ---------------------------------------------------------------- binning */

/* Bin every particle into cell number cell_of[i] (1-based, possibly > C) and
 * build per-cell lists in ascending particle order — the order the reference's
 * `box_part[++fluid_no[b]][b] = i` loops produce. */
static int bin_all(orc_ctx *c) {
  int N = c->p.n_fluid;
  memset(c->fluid_no, 0, sizeof(int32_t) * (size_t)c->Cpad);
  for (int i = 1; i <= N; ++i) {
    int b = c->cell_of[i];
    if (b < 0 || b >= c->Cpad) { set_err(c, "cell number outside the padded table"); return -1; }
    c->fluid_no[b]++;
  }
  c->cell_start[0] = 0;
  for (int b = 0; b < c->Cpad; ++b) c->cell_start[b + 1] = c->cell_start[b] + c->fluid_no[b];
  int32_t *fill = (int32_t *)malloc(sizeof(int32_t) * (size_t)c->Cpad);
  if (!fill) { set_err(c, "out of memory"); return -1; }
  memcpy(fill, c->cell_start, sizeof(int32_t) * (size_t)c->Cpad);
  for (int i = 1; i <= N; ++i) c->cell_list[fill[c->cell_of[i]]++] = i;
  free(fill);
  return 0;
}

/* --------------------------------------------------------------- initialize */

/* cpp/initialize.cpp:31-60 */
int orc_initialize_colloid(orc_ctx *c) {
  int counter = 0, check, Nc = c->p.n_colloid;
  double space_limit = 1.3 * c->p.sig_colloid;
  double ang_vscale_colloid = sqrt(12.0 * c->p.kbt1 / c->p.I_colloid);
  double vscale_colloid = sqrt(12.0 * c->p.kbt1 / c->p.mass_colloid);
  V3 avr_vel = v3(0, 0, 0), t = v3(0, 0, 0), temp;
  int attempt = 0;
  /* the lattice pre-fill of :36-39 only writes slots that the loop below
   * overwrites (and slot 0, which nothing reads) */
  while (counter < Nc) {
    drawseq d = ds_make(c, ORC_DOM_INIT_CPOS, (uint32_t)(counter + 1), (uint32_t)attempt, 0);
    t = ds_point(&d, v3(0, 0, 0), c->len);
    ++attempt;
    check = 1;
    for (int j = 1; j <= counter; j++) {
      temp = vimg(sub(t, c->pos_colloid[j]), c->len);
      check = (sqrt(vsum(mulv(temp, temp))) < space_limit) ? 0 : check;
    }
    if (check) { c->pos_colloid[++counter] = t; attempt = 0; }
  }
  for (int j = 1; j <= Nc; j++) {
    drawseq d = ds_make(c, ORC_DOM_INIT_CVEL, (uint32_t)j, 0, 0);
    c->vel_colloid[j] = muls(ds_point(&d, v3(0.5, 0.5, 0.5), v3(1, 1, 1)), vscale_colloid);
    avr_vel = add(avr_vel, c->vel_colloid[j]);
  }
  avr_vel = divs(avr_vel, (double)Nc);
  for (int j = 1; j <= Nc; j++) {
    c->vel_colloid[j] = sub(c->vel_colloid[j], avr_vel);
    drawseq d = ds_make(c, ORC_DOM_INIT_CVEL, (uint32_t)j, 0, 0);
    d.idx = 4; /* keyed: block 1 */
    c->ang_vel_colloid[j] = muls(ds_point(&d, v3(0.5, 0.5, 0.5), v3(1, 1, 1)), ang_vscale_colloid);
  }
  return 0;
}

/* cpp/initialize.cpp:62-83 */
int orc_initialize_fluid(orc_ctx *c) {
  int counter = 0, check, N = c->p.n_fluid, Nc = c->p.n_colloid;
  double vscale_fluid = sqrt(12.0 * c->p.kbt / c->p.mass_fl);
  V3 avr_vel = v3(0, 0, 0), t, temp;
  int attempt = 0;
  while (counter < N) {
    drawseq d = ds_make(c, ORC_DOM_INIT_FPOS, (uint32_t)(counter + 1), (uint32_t)attempt, 0);
    t = ds_point(&d, v3(0, 0, 0), c->len);
    ++attempt;
    check = 1;
    for (int j = 1; j <= Nc; j++) {
      temp = vimg(sub(t, c->pos_colloid[j]), c->len);
      check = (sqrt(vsum(mulv(temp, temp))) < c->p.sigma * 0.5) ? 0 : check;
    }
    if (check) { c->pos_fl[++counter] = t; attempt = 0; }
  }
  for (int j = 1; j <= N; j++) {
    drawseq d = ds_make(c, ORC_DOM_INIT_FVEL, (uint32_t)j, 0, 0);
    c->vel_fl[j] = muls(ds_point(&d, v3(0.5, 0.5, 0.5), v3(1, 1, 1)), vscale_fluid);
    avr_vel = add(avr_vel, c->vel_fl[j]);
  }
  avr_vel = divs(avr_vel, (double)N);
  for (int j = 1; j <= N; j++) c->vel_fl[j] = sub(c->vel_fl[j], avr_vel);
  return 0;
}

/* ----------------------------------------------------------- neighbour_list */

/* cpp/neighbour_list.cpp:3-11 */
static inline V3 cmod(V3 a, V3 b) {
  if (a.x <= 0) a.x += b.x;
  if (a.y <= 0) a.y += b.y;
  if (a.z <= 0) a.z += b.z;
  if (a.x > b.x) a.x -= b.x;
  if (a.y > b.y) a.y -= b.y;
  if (a.z > b.z) a.z -= b.z;
  return a;
}

/* The 7x7x7 - 1 neighbour boxes of box b, in the order create_box() stores them
 * (cpp/neighbour_list.cpp:12-25): z outer, y middle, x inner, offsets -3..3,
 * periodic via cmod, own box skipped.  Returns the count (342 for L >= 7). */
int orc_box_neighbours(const orc_ctx *c, int b, int32_t *out) {
  int Lx = c->p.Lx, Ly = c->p.Ly;
  if (b < 1 || b > c->C) return 0;
  int z0 = (b - 1) / (Lx * Ly), rem = (b - 1) % (Lx * Ly), y0 = rem / Lx, x0 = rem % Lx;
  V3 iter = v3(x0 + 1, y0 + 1, z0 + 1);  /* 1-based coordinates, as create_box walks them */
  int box = vcell(sub(iter, v3(0, 1, 1)), c->len);
  int nb = 0;
  V3 start = sub(iter, v3(3, 3, 3)), stop = add(iter, v3(3, 3, 3)), jiter = start;
  for (int j = 1; j <= 343; j++) {
    int tbox = vcell(sub(cmod(jiter, c->len), v3(0, 1, 1)), c->len);
    if (tbox != box || c->p.physics) out[nb++] = tbox;  /* the corrected rules keep the own box */
    /* point::next(len, inc, start) (cpp/parameters.hpp:66-70) */
    jiter.x += 1;
    if (jiter.x > stop.x) jiter.y += 1, jiter.x = start.x;
    if (jiter.y > stop.y) jiter.z += 1, jiter.y = start.y;
  }
  return nb;
}

/* cpp/neighbour_list.cpp:12-25.  The table is regenerated on demand by
 * orc_box_neighbours() (same values, same order); this only checks the box. */
int orc_create_box(orc_ctx *c) {
  if (c->p.Lx < 1 || c->p.Ly < 1 || c->p.Lz < 1) { set_err(c, "empty box"); return -1; }
  c->box_ready = 1;
  return 0;
}

/* cpp/neighbour_list.cpp:27-39 */
int orc_neighbour_list_md(orc_ctx *c) {
  double neigh_cutoff = 3.0 * c->p.sig_colloid;
  int Nc = c->p.n_colloid;
  for (int i = 0; i < Nc + 2; ++i) c->neighbour[i].n = 0;
  for (int i = 1; i < Nc; i++) {
    for (int j = i + 1; j <= Nc; j++) {
      V3 temp = vimg(sub(c->pos_colloid[i], c->pos_colloid[j]), c->len);
      if (vsum(mulv(temp, temp)) < pow(neigh_cutoff, 2)) {
        if (ilist_push(&c->neighbour[i], j)) { set_err(c, "out of memory"); return -1; }
      }
    }
  }
  return 0;
}

/* cpp/neighbour_list.cpp:41-58 */
int orc_neighbour_list_mpcd(orc_ctx *c) {
  int N = c->p.n_fluid, Nc = c->p.n_colloid;
  int32_t nb[343];
  for (int i = 1; i <= N; i++) c->cell_of[i] = 1 + vcell(c->pos_fl[i], c->len);
  if (bin_all(c)) return -1;
  c->last_kind = 1;
  memcpy(c->box_cell_of, c->cell_of, sizeof(int32_t) * ((size_t)N + 2));
  memcpy(c->box_occ, c->fluid_no, sizeof(int32_t) * (size_t)c->Cpad);
  for (int j = 1; j <= Nc; j++) {
    c->neigh_fl[j].n = 0;
    int cbox = 1 + vcell(c->pos_colloid[j], c->len);
    /* box_neigh[k][cbox] of a cell number outside 1..C holds zeros (calloc),
     * and fluid_no[0] is 0, so such a colloid gets no candidates */
    int nbox = orc_box_neighbours(c, cbox, nb);
    for (int k = 0; k < nbox; k++) {
      int mm = nb[k];
      for (int i = c->cell_start[mm]; i < c->cell_start[mm + 1]; i++)
        if (ilist_push(&c->neigh_fl[j], c->cell_list[i])) { set_err(c, "out of memory"); return -1; }
    }
  }
  return 0;
}

/* ----------------------------------------------------------- rotation_mpcd */

/* cpp/rotation_mpcd.cpp:3-50 */
int orc_rotation_mpcd(orc_ctx *c) {
  int N = c->p.n_fluid, C = c->C;
  double r[4], ir[4], theta, phi, rho, var, scale_fac_mpcd, ct, st, ict;
  V3 del_v, rr, rot[4];
  V3 *cell_vel = (V3 *)calloc((size_t)C + 1, sizeof(V3));   /* a stack VLA of C+1 points in the reference */
  if (!cell_vel) { set_err(c, "out of memory"); return -1; }

  {
    drawseq d = ds_make(c, ORC_DOM_SHIFT, 0, 0, (uint32_t)c->nn);
    rr = ds_point(&d, v3(0.5, 0.5, 0.5), v3(1, 1, 1));
  }
  c->last_rr = rr;
  for (int i = 1; i <= N; i++) c->cell_of[i] = 1 + vcell(vmod(add(c->pos_fl[i], rr), c->len), c->len);
  if (bin_all(c)) { free(cell_vel); return -1; }
  c->last_kind = 0;
  memcpy(c->rot_cell_of, c->cell_of, sizeof(int32_t) * ((size_t)N + 2));
  memcpy(c->rot_occ, c->fluid_no, sizeof(int32_t) * (size_t)c->Cpad);

  for (int i = 1; i <= C; i++) {
    int n = c->fluid_no[i];
    if (n > 1) {
      const int32_t *lst = c->cell_list + c->cell_start[i];
      for (int j = 0; j < n; j++) cell_vel[i] = add(cell_vel[i], divs(c->vel_fl[lst[j]], (double)n));
      drawseq d = ds_make(c, ORC_DOM_AXIS, (uint32_t)i, 0, (uint32_t)c->nn);
      rho = 2 * ds_next(&d) - 1;
      phi = 4.0 * asin(1.0) * ds_next(&d);
      theta = 2 * asin(1) * (c->p.theta_deg / 180.0);
      r[1] = cos(phi) * sqrt(1 - rho * rho), r[2] = sin(phi) * sqrt(1 - rho * rho), r[3] = rho;
      ct = cos(theta), st = sin(theta), ict = 1 - cos(theta);
      ir[1] = ict * r[1], ir[2] = ict * r[2], ir[3] = ict * r[3];
      rot[1] = v3(ir[1] * r[1] + ct, ir[1] * r[2] - st * r[3], ir[1] * r[3] + st * r[2]);
      rot[2] = v3(ir[2] * r[1] + st * r[3], ir[2] * r[2] + ct, ir[2] * r[3] - st * r[1]);
      rot[3] = v3(ir[3] * r[1] - st * r[2], ir[3] * r[2] + st * r[1], ir[3] * r[3] + ct);
      for (int j = 0; j < n; j++) {
        int k = lst[j];
        del_v = sub(c->vel_fl[k], cell_vel[i]);
        c->vel_fl[k] = add(cell_vel[i], v3(vsum(mulv(rot[1], del_v)), vsum(mulv(rot[2], del_v)), vsum(mulv(rot[3], del_v))));
      }
    }
  }
  for (int i = 1; i <= C; i++) {
    int n = c->fluid_no[i];
    var = 0.0;
    if (n > 1) {
      const int32_t *lst = c->cell_list + c->cell_start[i];
      for (int j = 0; j < n; j++) {
        del_v = sub(c->vel_fl[lst[j]], cell_vel[i]);
        var += vsum(mulv(del_v, del_v));
      }
      scale_fac_mpcd = sqrt(3.0 * (n - 1) * c->p.kbt / (c->p.mass_fl * var));
      for (int j = 0; j < n; j++) {
        int k = lst[j];
        del_v = sub(c->vel_fl[k], cell_vel[i]);
        c->vel_fl[k] = add(cell_vel[i], muls(del_v, scale_fac_mpcd));
      }
    }
  }
  free(cell_vel);
  return 0;
}

/* --------------------------------------------------------------------- run */

/* cpp/run.cpp:3-8 */
int orc_tumble(orc_ctx *c) {
  for (int i = 1; i <= c->p.n_colloid; i++) {
    drawseq d = ds_make(c, ORC_DOM_TUMBLE, (uint32_t)i, 0, 0);
    c->ra[i] = vimg(sub(c->pos_colloid[i], ds_point(&d, v3(0, 0, 0), c->len)), c->len);
    c->ra[i] = divs(c->ra[i], sqrt(vsum(mulv(c->ra[i], c->ra[i]))));
  }
  return 0;
}

/* cpp/run.cpp:10-26 */
int orc_run(orc_ctx *c) {
  V3 vector, del;
  for (int i = 1; i <= c->p.n_colloid; i++) {
    c->vel_colloid[i] = add(c->vel_colloid[i], muls(c->ra[i], c->p.v0)), del = muls(c->ra[i], c->p.v0);
    c->nbr[i].n = 0;
    const ilist *nf = &c->neigh_fl[i];
    for (int j = 0; j < nf->n; j++) {
      vector = vimg(sub(c->pos_fl[nf->v[j]], c->pos_colloid[i]), c->len);
      if (vsum(mulv(vector, vector)) <= pow(c->p.sigma * 0.5 + 0.5, 2) && vsum(mulv(vector, c->vel_colloid[i])) <= 0)
        if (ilist_push(&c->nbr[i], nf->v[j])) { set_err(c, "out of memory"); return -1; }
    }
    int cnt = c->nbr[i].n;
    for (int j = 0; j < cnt; j++) {
      int k = c->nbr[i].v[j];
      c->vel_fl[k] = sub(c->vel_fl[k], muls(del, (c->p.mass_colloid / (c->p.mass_fl * cnt))));
    }
  }
  return 0;
}

int orc_get_shell_count(const orc_ctx *c, int32_t *cnt) {
  for (int i = 1; i <= c->p.n_colloid; ++i) cnt[i - 1] = c->nbr[i].n;
  return 0;
}

/* cpp/run.cpp:28-50.  The reference computes and discards these values; here
 * they are returned.  up_vel accumulates over colloids as in the reference. */
int orc_updown_velocity(orc_ctx *c, double *vel_out, double *up_vel_out) {
  V3 up_vel = v3(0, 0, 0), vector, vel;
  for (int i = 1; i <= c->p.n_colloid; i++) {
    int cnt = 0, up_cnt = 0;
    vel = v3(0, 0, 0);
    c->nbr[i].n = 0; c->up_nbr[i].n = 0;
    const ilist *nf = &c->neigh_fl[i];
    for (int j = 0; j < nf->n; j++) {
      vector = vimg(sub(c->pos_fl[nf->v[j]], c->pos_colloid[i]), c->len);
      if (vsum(mulv(vector, vector)) <= pow((c->p.sigma * 0.5 + 0.5), 2) && vsum(mulv(vector, c->vel_colloid[i])) <= 0.0) {
        ilist_push(&c->nbr[i], nf->v[j]); cnt++;
      }
      if (vsum(mulv(vector, vector)) <= pow((c->p.sigma * 0.5 + 0.1), 2) && vsum(mulv(vector, c->vel_colloid[i])) <= 0.0) {
        ilist_push(&c->up_nbr[i], nf->v[j]); up_cnt++;
      }
    }
    for (int j = 0; j < cnt; j++) vel = add(vel, c->vel_fl[c->nbr[i].v[j]]);
    for (int j = 0; j < up_cnt; j++) up_vel = add(up_vel, c->vel_fl[c->up_nbr[i].v[j]]);
    up_vel = (up_cnt > 0) ? sub(divs(up_vel, (double)up_cnt), c->vel_colloid[i]) : up_vel;
    vel = (up_cnt > 0) ? sub(divs(vel, (double)cnt), c->vel_colloid[i]) : vel;
    if (vel_out) { vel_out[3 * (i - 1)] = vel.x; vel_out[3 * (i - 1) + 1] = vel.y; vel_out[3 * (i - 1) + 2] = vel.z; }
  }
  if (up_vel_out) { up_vel_out[0] = up_vel.x; up_vel_out[1] = up_vel.y; up_vel_out[2] = up_vel.z; }
  return 0;
}

int orc_updown_sums(orc_ctx *c, int *cnt, int *up_cnt, double *vel_sum, double *up_vel_sum) {
  for (int i = 1; i <= c->p.n_colloid; i++) {
    int n = 0, un = 0;
    V3 vs = v3(0, 0, 0), us = v3(0, 0, 0), vector;
    const ilist *nf = &c->neigh_fl[i];
    for (int j = 0; j < nf->n; j++) {
      vector = vimg(sub(c->pos_fl[nf->v[j]], c->pos_colloid[i]), c->len);
      const double r2 = vsum(mulv(vector, vector)), d = vsum(mulv(vector, c->vel_colloid[i]));
      if (r2 <= pow((c->p.sigma * 0.5 + 0.5), 2) && d <= 0.0) { n++; vs = add(vs, c->vel_fl[nf->v[j]]); }
      if (r2 <= pow((c->p.sigma * 0.5 + 0.1), 2) && d <= 0.0) { un++; us = add(us, c->vel_fl[nf->v[j]]); }
    }
    cnt[i - 1] = n; up_cnt[i - 1] = un;
    vel_sum[3 * (i - 1)] = vs.x; vel_sum[3 * (i - 1) + 1] = vs.y; vel_sum[3 * (i - 1) + 2] = vs.z;
    up_vel_sum[3 * (i - 1)] = us.x; up_vel_sum[3 * (i - 1) + 1] = us.y; up_vel_sum[3 * (i - 1) + 2] = us.z;
  }
  return 0;
}

/* ------------------------------------------------- fluid_colloid_collision */

/* cpp/fluid_colloid_collision.cpp:7-24 */
static V3 stochastic_reflection(orc_ctx *c, drawseq *d, V3 rf, V3 rs) {
  double kbt = c->p.kbt, mass_fl = c->p.mass_fl;
  double m_beta = mass_fl / kbt, random_e = pow(1 - ds_next(d), 2), val, v[4], x[4], z = 2;
  V3 un, ut, t, n;
  n = divs(rs, sqrt(vsum(mulv(rs, rs))));
  val = sqrt(-log(random_e) / m_beta);
  un = muls(n, val);
  t = vimg(ds_point(d, rf, c->len), c->len);
  ut = cross(un, t);
  ut = divs(ut, sqrt(vsum(mulv(ut, ut))));
  while (z > 1) {
    x[1] = 2.0 * ds_next(d) - 1, x[2] = 2.0 * ds_next(d) - 1;
    z = x[1] * x[1] + x[2] * x[2];
  }
  z = sqrt((-2.0 * log(z)) / z);
  v[1] = x[1] * z * sqrt(kbt / mass_fl);
  v[2] = x[2] * z * sqrt(kbt / mass_fl);
  if (c->p.physics) /* the corrected rules: the second tangential component along n x ut */
    return add(add(muls(ut, v[1]), muls(cross(n, ut), v[2])), un);
  return add(muls(ut, v[1]), un);
}

/* cpp/fluid_colloid_collision.cpp:26-49 */
int orc_fluid_colloid_collision(orc_ctx *c) {
  V3 rr, rs, u, omega, vc;
  int N = c->p.n_fluid;
  double dt = c->dt;
  uint32_t gs = (uint32_t)((c->nn - 1) * c->p.n_sub + (c->l - 1));
  memcpy(c->dump_vel_fl, c->vel_fl, sizeof(V3) * ((size_t)N + 1));
  for (int j = 1; j <= c->p.n_colloid; j++) {
    vc = omega = v3(0, 0, 0);
    const ilist *nf = &c->neigh_fl[j];
    for (int i = 0; i < nf->n; i++) {
      int l = nf->v[i];
      rr = vimg(sub(c->pos_colloid[j], c->pos_fl[l]), c->len);
      if (vsum(mulv(rr, rr)) <= pow(c->p.sigma, 2) * 0.25) {
        c->pos_fl[l] = vmod(sub(c->pos_fl[l], muls(muls(c->vel_fl[l], dt), 0.5)), c->len);
        rs = vimg(sub(c->pos_fl[l], c->pos_colloid[j]), c->len);
        drawseq d = ds_make(c, ORC_DOM_COLL, (uint32_t)l, (uint32_t)j, gs);
        u = stochastic_reflection(c, &d, c->pos_fl[l], rs);
        c->vel_fl[l] = add(add(u, c->vel_colloid[j]), cross(c->ang_vel_colloid[j], rs));
        vc = add(vc, sub(c->dump_vel_fl[l], c->vel_fl[l]));
        u = sub(c->dump_vel_fl[l], c->vel_fl[l]);
        omega = add(omega, cross(rs, sub(c->dump_vel_fl[l], c->vel_fl[l])));
        c->pos_fl[l] = vmod(add(c->pos_fl[l], muls(muls(c->vel_fl[l], dt), 0.5)), c->len);
      }
    }
    c->vel_colloid[j] = add(c->vel_colloid[j], divs(muls(vc, c->p.mass_fl), c->p.mass_colloid));
    c->ang_vel_colloid[j] = add(c->ang_vel_colloid[j], divs(muls(omega, c->p.mass_fl), c->p.I_colloid));
  }
  return 0;
}

/* ------------------------------------------------------------------ update */

/* cpp/update.cpp:8-13 */
static double power(double x, int r) {
  double ans = 1;
  for (int i = 1; i <= r; i++) ans *= x;
  return ans;
}

/* cpp/update.cpp:14-32 */
int orc_compute_force_md(orc_ctx *c) {
  V3 temp, ff;
  double eps = c->p.eps, sig = c->p.sig_colloid, r, mag_f, t1, t2;
  c->potential_colloid = 0;
  for (int i = 0; i <= c->p.n_colloid; i++) c->f[i] = v3(0, 0, 0);
  for (int i = 1; i <= c->p.n_colloid; i++) {
    const ilist *nb = &c->neighbour[i];
    for (int j = 0; j < nb->n; j++) {
      int k = nb->v[j];
      temp = vimg(sub(c->pos_colloid[i], c->pos_colloid[k]), c->len);
      r = sqrt(vsum(mulv(temp, temp)));
      if (r < c->r_cutoff) {
        c->potential_colloid += 4 * eps * (pow(sig / r, 12) - pow(sig / r, 6)) - c->ufc + c->fc * r;
        t1 = c->sig12 / power(r, 13), t2 = c->sig6 / power(r, 7);
        mag_f = 4.0 * eps * (12.0 * t1 - 6.0 * t2) - c->fc;
        ff = divs(muls(temp, mag_f), r);
        c->f[i] = add(c->f[i], ff), c->f[k] = sub(c->f[k], ff);
      }
    }
  }
  return 0;
}

/* Rotational diffusion of the orientation: no reference counterpart (Dr = 0
 * reproduces the reference).  ra += sqrt(2 Dr dt) (xi - (xi.ra) ra), then
 * renormalised; xi is three standard normals by Box-Muller. */
static void rotdiff(orc_ctx *c, int i, uint32_t gs) {
  double s = sqrt(2.0 * c->p.Dr * c->dt);
  drawseq d = ds_make(c, ORC_DOM_ROTDIFF, (uint32_t)i, 0, gs);
  double u0 = ds_next(&d), u1 = ds_next(&d), u2 = ds_next(&d), u3 = ds_next(&d);
  double tpi = 4.0 * asin(1.0);
  double r0 = sqrt(-2.0 * log(u0)), r1 = sqrt(-2.0 * log(u2));
  V3 xi = v3(r0 * cos(tpi * u1), r0 * sin(tpi * u1), r1 * cos(tpi * u3));
  V3 a = c->ra[i];
  double xa = vsum(mulv(xi, a));
  V3 dn = sub(xi, muls(a, xa));
  a = add(a, muls(dn, s));
  c->ra[i] = divs(a, sqrt(vsum(mulv(a, a))));
}

/* cpp/update.cpp:34-46 (+ rotational diffusion when Dr > 0) */
int orc_update_activity_direction(orc_ctx *c) {
  V3 m[4], b, sb, cb;
  uint32_t gs = (uint32_t)((c->nn - 1) * c->p.n_sub + (c->l - 1));
  for (int i = 1; i <= c->p.n_colloid; i++) {
    b = muls(c->ang_vel_colloid[i], c->dt);
    sb = v3(sin(b.x), sin(b.y), sin(b.z)), cb = v3(cos(b.x), cos(b.y), cos(b.z));
    m[1] = v3(cb.y * cb.z, -cb.y * sb.z, sb.y);
    m[2] = v3(sb.x * sb.y * cb.z + cb.x * sb.z, -sb.x * sb.y * sb.z + cb.x * cb.z, -sb.x * cb.y);
    m[3] = v3(-cb.x * sb.y * cb.z + sb.x * sb.z, cb.x * sb.y * sb.z + sb.x * cb.z, cb.x * cb.y);
    c->ra[i] = v3(vsum(mulv(m[1], c->ra[i])), vsum(mulv(m[2], c->ra[i])), vsum(mulv(m[3], c->ra[i])));
    if (c->p.Dr > 0) rotdiff(c, i, gs);
  }
  return 0;
}

/* cpp/update.cpp:48-54 */
int orc_update_pos_md(orc_ctx *c) {
  double dt = c->dt, dt2 = dt * dt, ddt = 0.5 * dt2 / c->p.mass_colloid;
  for (int i = 1; i <= c->p.n_colloid; i++) {
    c->pos_colloid[i] = add(c->pos_colloid[i], add(muls(c->vel_colloid[i], dt), muls(c->f[i], ddt)));
    c->pos_colloid[i] = vmod(c->pos_colloid[i], c->len);
  }
  return 0;
}

/* cpp/update.cpp:56-60 */
int orc_update_pos_mpcd(orc_ctx *c) {
  double dt = c->dt;
  for (int i = 1; i <= c->p.n_fluid; i++) c->pos_fl[i] = vmod(add(c->pos_fl[i], muls(c->vel_fl[i], dt)), c->len);
  return 0;
}

/* cpp/update.cpp:62-67 */
int orc_update_velocity_colloid(orc_ctx *c) {
  double dtb2 = c->dt / (c->p.mass_colloid * 2);
  for (int i = 1; i <= c->p.n_colloid; i++)
    c->vel_colloid[i] = add(c->vel_colloid[i], muls(add(c->old_force[i], c->f[i]), dtb2));
  return 0;
}

/* ------------------------------------------------------------------ driver */

/* cpp/active_brownian.cpp:17-20 */
int orc_setup(orc_ctx *c) {
  if (orc_create_box(c)) return -1;
  if (orc_neighbour_list_mpcd(c)) return -1;
  if (orc_neighbour_list_md(c)) return -1;
  return orc_compute_force_md(c);
}

/* the start of substep l of the main loop (cpp/active_brownian.cpp:27-28): the substep
 * counter the keyed draws use, and old_force = f */
int orc_begin_substep(orc_ctx *c, int l) {
  c->l = l;
  memcpy(c->old_force, c->f, sizeof(V3) * ((size_t)c->p.n_colloid + 2));
  return 0;
}

/* cpp/active_brownian.cpp:28-37 */
int orc_substep(orc_ctx *c, int l) {
  orc_begin_substep(c, l);
  if (orc_update_pos_md(c)) return -1;
  if (orc_neighbour_list_md(c)) return -1;
  if (orc_update_pos_mpcd(c)) return -1;
  if (orc_neighbour_list_mpcd(c)) return -1;
  if (!(l % 10) && c->nn > 10000) orc_updown_velocity(c, NULL, NULL);
  if (orc_fluid_colloid_collision(c)) return -1;
  if (orc_update_activity_direction(c)) return -1;
  if (orc_compute_force_md(c)) return -1;
  return orc_update_velocity_colloid(c);
}

/* cpp/active_brownian.cpp:23-38 */
int orc_step(orc_ctx *c) {
  c->nn += 1;
  if (orc_rotation_mpcd(c)) return -1;
  if (orc_run(c)) return -1;
  for (int l = 1; l <= c->p.n_sub; l++)
    if (orc_substep(c, l)) return -1;
  return 0;
}

int orc_run_steps(orc_ctx *c, int nsteps) {
  for (int s = 0; s < nsteps; ++s)
    if (orc_step(c)) return -1;
  return 0;
}

/* cpp/active_brownian.cpp:39-55 with the momentum reset each call */
void orc_diag(const orc_ctx *c, double *out) {
  double ke_colloid = 0, ke_fluid = 0, ang_ke_colloid = 0, abs_p = 0;
  V3 mom = v3(0, 0, 0);
  for (int i = 1; i <= c->p.n_colloid; i++) {
    ke_colloid += vsum(mulv(c->vel_colloid[i], c->vel_colloid[i]));
    ang_ke_colloid += vsum(mulv(c->ang_vel_colloid[i], c->ang_vel_colloid[i]));
    mom = add(mom, muls(c->vel_colloid[i], c->p.mass_colloid));
    abs_p += c->p.mass_colloid * (fabs(c->vel_colloid[i].x) + fabs(c->vel_colloid[i].y) + fabs(c->vel_colloid[i].z));
  }
  for (int i = 1; i <= c->p.n_fluid; i++) {
    ke_fluid += vsum(mulv(c->vel_fl[i], c->vel_fl[i]));
    mom = add(mom, muls(c->vel_fl[i], c->p.mass_fl));
    abs_p += c->p.mass_fl * (fabs(c->vel_fl[i].x) + fabs(c->vel_fl[i].y) + fabs(c->vel_fl[i].z));
  }
  ke_colloid = 0.5 * c->p.mass_colloid * ke_colloid;
  ang_ke_colloid = 0.5 * c->p.I_colloid * ang_ke_colloid;
  out[0] = 0.5 * ke_fluid * c->p.mass_fl;
  out[1] = ke_colloid;
  out[2] = ang_ke_colloid;
  out[3] = c->potential_colloid;
  out[4] = c->potential_colloid + ke_colloid + ang_ke_colloid;
  out[5] = mom.x; out[6] = mom.y; out[7] = mom.z;
  out[8] = abs_p;
}

/* ------------------------------------------------------------------- state */

static V3 *arr_of(const orc_ctx *c, int which, int *n) {
  switch (which) {
    case 0: *n = c->p.n_fluid; return c->pos_fl;
    case 1: *n = c->p.n_fluid; return c->vel_fl;
    case 2: *n = c->p.n_colloid; return c->pos_colloid;
    case 3: *n = c->p.n_colloid; return c->vel_colloid;
    case 4: *n = c->p.n_colloid; return c->ang_vel_colloid;
    case 5: *n = c->p.n_colloid; return c->ra;
    case 6: *n = c->p.n_colloid; return c->f;
    case 7: *n = c->p.n_colloid; return c->old_force;
  }
  return NULL;
}

int orc_get(const orc_ctx *c, int which, double *out) {
  int n; V3 *a = arr_of(c, which, &n);
  if (!a) return -1;
  for (int i = 0; i < n; ++i) { out[3 * i] = a[i + 1].x; out[3 * i + 1] = a[i + 1].y; out[3 * i + 2] = a[i + 1].z; }
  return 0;
}

int orc_set(orc_ctx *c, int which, const double *in) {
  int n; V3 *a = arr_of(c, which, &n);
  if (!a) return -1;
  for (int i = 0; i < n; ++i) a[i + 1] = v3(in[3 * i], in[3 * i + 1], in[3 * i + 2]);
  return 0;
}

double orc_potential(const orc_ctx *c) { return c->potential_colloid; }

int orc_get_binning(const orc_ctx *c, int kind, int32_t *cell_of, int32_t *occupancy) {
  const int32_t *co = kind == 0 ? c->rot_cell_of : c->box_cell_of;
  const int32_t *oc = kind == 0 ? c->rot_occ : c->box_occ;
  if (cell_of) for (int i = 0; i < c->p.n_fluid; ++i) cell_of[i] = co[i + 1];
  if (occupancy) for (int b = 0; b < c->C; ++b) occupancy[b] = oc[b + 1];
  return 0;
}

void orc_get_shift(const orc_ctx *c, double *rr3) { rr3[0] = c->last_rr.x; rr3[1] = c->last_rr.y; rr3[2] = c->last_rr.z; }

int orc_get_neighbour_md(const orc_ctx *c, int i, int32_t *out, int cap) {
  if (i < 1 || i > c->p.n_colloid) return -1;
  const ilist *l = &c->neighbour[i];
  for (int k = 0; k < l->n && k < cap; ++k) out[k] = l->v[k];
  return l->n;
}

int orc_get_neigh_fl(const orc_ctx *c, int j, int32_t *out, int cap) {
  if (j < 1 || j > c->p.n_colloid) return -1;
  const ilist *l = &c->neigh_fl[j];
  for (int i = 0; i < l->n && i < cap; ++i) out[i] = l->v[i];
  return l->n;
}
