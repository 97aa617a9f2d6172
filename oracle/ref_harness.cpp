// Trace harness for the reference's serial C++ step — TEST INFRASTRUCTURE ONLY.
//
// Linked against the reference's own routine sources (cpp/initialize.cpp,
// cpp/neighbour_list.cpp, cpp/rotation_mpcd.cpp, cpp/fluid_colloid_collision.cpp,
// cpp/update.cpp, cpp/run.cpp), compiled where they lie by the `ref` target of oracle/Makefile.
// It replaces only cpp/active_brownian.cpp: it defines the globals that file
// defines (cpp/active_brownian.cpp:3-7, names and types fixed by the
// declarations in cpp/parameters.hpp:8-10,72), takes the parameters from the
// command line instead of compile-time constants, and calls the routines in the
// order of cpp/active_brownian.cpp:14-38, writing a record after each routine.
//
// Output: a stream of records  [char tag[48]][uint64 nbytes][bytes].
// Modes:
//   ref_harness time   L N Nc n_sub ndt kbt kbt1 mass_fl M sig_colloid eps sigma I v0 seed nsteps state
//     the reference's own step loop (cpp/active_brownian.cpp:23-38) timed over nsteps MPCD steps
//     from the given state (file as below; initialize_fluid is skipped), after the prologue and
//     one untimed step; prints {"steps": n, "seconds": s, "particle_steps_per_s": r}
//   ref_harness trace  L N Nc n_sub ndt kbt kbt1 mass_fl M sig_colloid eps sigma I v0 seed nsteps detail_steps out [state]
//     state (optional): raw doubles pos_fl[N][3] vel_fl[N][3] pos_colloid[Nc][3]
//     vel_colloid[Nc][3] ang_vel_colloid[Nc][3] that replace the state the reference
//     initialisation produced (the ran() stream has still advanced through it)
//   ref_harness ran    seed count out
#include "parameters.hpp"

#include <chrono>
#include <cstdint>
#include <string>
#include <vector>

point *pos_colloid, *pos_fl, *vel_colloid, *vel_fl, *ang_vel_colloid, *f, *ra, *old_force, *dump_vel_fl,
    len = point(30, 30, 30);
int n = 10, niter = 21000, file = 0, nbin = 300, maxpart = 100, no_of_colloid = 10, nbox, **nbr, **up_nbr, *cnt,
    *up_cnt, *fluid_no, *iv, seed = 77777;
int no_of_fluid = 27000, *no_neigh, **neigh_fl, *neighbour[256], *n_neighbour, *box_neigh[512], **box_part,
    **cell_part, ntab = 32, nn;
double kbt = 1, kbt1 = 1, ndt = 0.1, dv = 0.1, mass_fl = 1.0, mass_colloid = 654.1, sig_colloid = 5.0, eps = 1.0,
       v0 = 0.0;
double dt = 0.01, sigma = 4.0, I_colloid = 1046.56, potential_colloid;

// defined in cpp/update.cpp:3-6 from sig_colloid at static initialisation
extern double r_cutoff, fc, ufc, sig_colloid12, sig_colloid6;

static FILE *out;

static void rec(const std::string &tag, const void *p, size_t nbytes) {
  char t[48] = {0};
  snprintf(t, sizeof t, "%s", tag.c_str());
  uint64_t nb = nbytes;
  fwrite(t, 1, 48, out);
  fwrite(&nb, 8, 1, out);
  if (nbytes) fwrite(p, 1, nbytes, out);
}

static void rec_pts(const std::string &tag, const point *a, int count) { rec(tag, &a[1], sizeof(point) * count); }

static void rec_state(const std::string &pre) {
  rec_pts(pre + "/pos_fl", pos_fl, no_of_fluid);
  rec_pts(pre + "/vel_fl", vel_fl, no_of_fluid);
  rec_pts(pre + "/pos_colloid", pos_colloid, no_of_colloid);
  rec_pts(pre + "/vel_colloid", vel_colloid, no_of_colloid);
  rec_pts(pre + "/ang_vel_colloid", ang_vel_colloid, no_of_colloid);
  rec_pts(pre + "/ra", ra, no_of_colloid);
  rec_pts(pre + "/f", f, no_of_colloid);
  rec(pre + "/potential", &potential_colloid, sizeof(double));
}

// per-particle cell number and per-cell occupancy from a slot-major table
static void rec_binning(const std::string &pre, int **table) {
  int C = (int)len.prod();
  std::vector<int32_t> cell_of(no_of_fluid, 0), occ(C);
  for (int b = 1; b <= C + 1; ++b)
    for (int s = 1; s <= fluid_no[b]; ++s) cell_of[table[s][b] - 1] = b;
  for (int b = 1; b <= C; ++b) occ[b - 1] = fluid_no[b];
  rec(pre + "/cell_of", cell_of.data(), sizeof(int32_t) * cell_of.size());
  rec(pre + "/occupancy", occ.data(), sizeof(int32_t) * occ.size());
}

static void rec_neigh(const std::string &pre) {
  std::vector<int32_t> v;
  for (int j = 1; j <= no_of_colloid; ++j) {
    v.push_back(no_neigh[j]);
    for (int i = 1; i <= no_neigh[j]; ++i) v.push_back(neigh_fl[j][i]);
  }
  rec(pre + "/neigh_fl", v.data(), sizeof(int32_t) * v.size());
}

int main(int argc, char **argv) {
  if (argc >= 2 && std::string(argv[1]) == "ran") {
    if (argc != 5) return 2;
    seed = atoi(argv[2]);
    int count = atoi(argv[3]);
    out = fopen(argv[4], "wb");
    if (!out) return 3;
    iv = (int *)calloc(ntab + 2, sizeof(int));
    std::vector<double> v(count);
    for (int i = 0; i < count; ++i) v[i] = ran();
    rec("ran", v.data(), sizeof(double) * count);
    fclose(out);
    return 0;
  }
  const bool timing = argc == 19 && std::string(argv[1]) == "time";
  if (!timing && ((argc != 20 && argc != 21) || std::string(argv[1]) != "trace")) {
    fprintf(stderr, "usage: ref_harness trace L N Nc n_sub ndt kbt kbt1 mass_fl M sig eps sigma I v0 seed nsteps detail out\n");
    return 2;
  }
  int L = atoi(argv[2]);
  len = point(L, L, L);
  no_of_fluid = atoi(argv[3]);
  no_of_colloid = atoi(argv[4]);
  n = atoi(argv[5]);
  ndt = atof(argv[6]);
  kbt = atof(argv[7]);
  kbt1 = atof(argv[8]);
  mass_fl = atof(argv[9]);
  mass_colloid = atof(argv[10]);
  sig_colloid = atof(argv[11]);
  eps = atof(argv[12]);
  sigma = atof(argv[13]);
  I_colloid = atof(argv[14]);
  v0 = atof(argv[15]);
  seed = atoi(argv[16]);
  int nsteps = atoi(argv[17]), detail = timing ? 0 : atoi(argv[18]);
  out = fopen(timing ? "/dev/null" : argv[19], "wb");
  if (!out) return 3;
  dt = ndt / (double)n;
  // the derived constants of cpp/update.cpp:3-6, recomputed for the new sig_colloid
  r_cutoff = pow(2, 1.0 / 6.0) * sig_colloid;
  fc = 4.0 * eps * (12.0 * (pow(sig_colloid, 12) / pow(r_cutoff, 13)) - 6.0 * (pow(sig_colloid, 6) / pow(r_cutoff, 7)));
  ufc = 4.0 * eps * (pow(sig_colloid / r_cutoff, 12) - pow(sig_colloid / r_cutoff, 6)) + fc * r_cutoff;
  sig_colloid12 = pow(sig_colloid, 12);
  sig_colloid6 = pow(sig_colloid, 6);

  initialize();
  initialize_colloid();
  if (!timing) initialize_fluid();
  if (timing || argc == 21) {
    FILE *in = fopen(argv[timing ? 18 : 20], "rb");
    if (!in) return 4;
    size_t ok = fread(&pos_fl[1], sizeof(point), no_of_fluid, in) + fread(&vel_fl[1], sizeof(point), no_of_fluid, in) +
                fread(&pos_colloid[1], sizeof(point), no_of_colloid, in) +
                fread(&vel_colloid[1], sizeof(point), no_of_colloid, in) +
                fread(&ang_vel_colloid[1], sizeof(point), no_of_colloid, in);
    fclose(in);
    if (ok != 2 * (size_t)no_of_fluid + 3 * (size_t)no_of_colloid) return 5;
  }
  rec_state("init");
  create_box();
  {
    int C = (int)len.prod();
    std::vector<int32_t> t;
    t.reserve((size_t)C * nbox);
    for (int b = 1; b <= C; ++b)
      for (int k = 1; k <= nbox; ++k) t.push_back(box_neigh[k][b]);
    rec("setup/box_neigh", t.data(), sizeof(int32_t) * t.size());
  }
  neighbour_list_mpcd();
  rec_binning("setup.nl_mpcd", box_part);
  rec_neigh("setup.nl_mpcd");
  neighbour_list_md();
  compute_force_md();
  rec_pts("setup.force/f", f, no_of_colloid);
  rec("setup.force/potential", &potential_colloid, sizeof(double));
  tumble();
  rec_pts("setup.tumble/ra", ra, no_of_colloid);

  if (timing) {
    // the step loop of cpp/active_brownian.cpp:23-38 as it stands (one untimed step first)
    auto one = [&]() {
      rotation_mpcd();
      run();
      for (int l = 1; l <= n; l++) {
        std::copy(f, f + no_of_colloid + 2, old_force);
        update_pos_md();
        neighbour_list_md();
        update_pos_mpcd();
        neighbour_list_mpcd();
        if (!(l % 10) && nn > 10000) updown_velocity();
        fluid_colloid_collision();
        update_activity_direction();
        compute_force_md();
        update_velocity_colloid();
      }
    };
    nn = 1;
    one();
    const auto t0 = std::chrono::steady_clock::now();
    for (nn = 2; nn <= nsteps + 1; nn++) one();
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    printf("{\"steps\": %d, \"seconds\": %.6f, \"particle_steps_per_s\": %.6e}\n", nsteps, sec,
           (double)no_of_fluid * nsteps / sec);
    fclose(out);
    return 0;
  }
  for (nn = 1; nn <= niter && nn <= nsteps; nn++) {
    std::string s = "s" + std::to_string(nn);
    bool d = nn <= detail;
    rotation_mpcd();
    if (d) {
      rec_pts(s + ".rotation/vel_fl", vel_fl, no_of_fluid);
      rec_binning(s + ".rotation", cell_part);
    }
    run();
    if (d) {
      rec_pts(s + ".run/vel_fl", vel_fl, no_of_fluid);
      rec_pts(s + ".run/vel_colloid", vel_colloid, no_of_colloid);
      std::vector<int32_t> c(cnt + 1, cnt + 1 + no_of_colloid);
      rec(s + ".run/shell_count", c.data(), sizeof(int32_t) * c.size());
    }
    for (int l = 1; l <= n; l++) {
      std::string p = s + ".l" + std::to_string(l);
      bool dl = d && l <= 2;
      std::copy(f, f + no_of_colloid + 2, old_force);
      update_pos_md();
      if (dl) rec_pts(p + ".pos_md/pos_colloid", pos_colloid, no_of_colloid);
      neighbour_list_md();
      update_pos_mpcd();
      if (dl) rec_pts(p + ".pos_mpcd/pos_fl", pos_fl, no_of_fluid);
      neighbour_list_mpcd();
      if (dl) {
        rec_binning(p + ".nl_mpcd", box_part);
        rec_neigh(p + ".nl_mpcd");
      }
      if (!(l % 10) && nn > 10000) updown_velocity();
      fluid_colloid_collision();
      if (dl) {
        rec_pts(p + ".collision/pos_fl", pos_fl, no_of_fluid);
        rec_pts(p + ".collision/vel_fl", vel_fl, no_of_fluid);
        rec_pts(p + ".collision/vel_colloid", vel_colloid, no_of_colloid);
        rec_pts(p + ".collision/ang_vel_colloid", ang_vel_colloid, no_of_colloid);
      }
      update_activity_direction();
      if (dl) rec_pts(p + ".activity/ra", ra, no_of_colloid);
      compute_force_md();
      if (dl) {
        rec_pts(p + ".force/f", f, no_of_colloid);
        rec(p + ".force/potential", &potential_colloid, sizeof(double));
      }
      update_velocity_colloid();
      if (dl) rec_pts(p + ".velocity/vel_colloid", vel_colloid, no_of_colloid);
    }
    rec_state(s + ".end");
  }
  fclose(out);
  return 0;
}
