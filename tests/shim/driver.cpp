// Test driver for libbrownian_shim: defines the globals the reference's driver
// defines (same names and types as cpp/active_brownian.cpp:3-7) and calls the
// reference's routines in the order of its main loop (cpp/active_brownian.cpp:14-38),
// then writes the final state.  Built and run by tests/test_gpu_shim.py.
//   driver L density n_colloid nsteps out.bin
#include <algorithm>
#include <cstdio>
#include <cstdlib>

struct point {
  double x, y, z;
  point(double a = 0, double b = 0, double c = 0) : x(a), y(b), z(c) {}
};

point *pos_colloid, *pos_fl, *vel_colloid, *vel_fl, *ang_vel_colloid, *f, *ra, *old_force, *dump_vel_fl, len;
int n = 10, no_of_fluid, no_of_colloid, seed = 77777, nn;
double kbt = 1, kbt1 = 1, ndt = 0.1, mass_fl = 1.0, mass_colloid = 654.1, sig_colloid = 5.0, eps = 1.0, v0 = 0.02;
double sigma = 0.8 * 5.0, I_colloid = 0.1 * 654.1 * 4.0 * 4.0, potential_colloid;

void create_box(), compute_force_md(), fluid_colloid_collision(), initialize(), initialize_fluid(), initialize_colloid();
void neighbour_list_md(), neighbour_list_mpcd(), rotation_mpcd(), run(), tumble(), updown_velocity();
void update_velocity_colloid(), update_pos_md(), update_pos_mpcd(), update_activity_direction();

static void put(FILE *fp, const point *a, int count) { fwrite(&a[1], sizeof(point), count, fp); }

int main(int argc, char **argv) {
  if (argc != 6) return 2;
  const int L = atoi(argv[1]);
  len = point(L, L, L);
  no_of_fluid = L * L * L * atoi(argv[2]);
  no_of_colloid = atoi(argv[3]);
  const int nsteps = atoi(argv[4]);
  initialize();
  initialize_colloid();
  initialize_fluid();
  create_box();
  neighbour_list_mpcd();
  neighbour_list_md();
  compute_force_md();
  tumble();
  for (nn = 1; nn <= nsteps; nn++) {
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
  }
  FILE *fp = fopen(argv[5], "wb");
  if (!fp) return 2;
  put(fp, pos_fl, no_of_fluid); put(fp, vel_fl, no_of_fluid);
  put(fp, pos_colloid, no_of_colloid); put(fp, vel_colloid, no_of_colloid);
  put(fp, ang_vel_colloid, no_of_colloid); put(fp, ra, no_of_colloid);
  fwrite(&potential_colloid, sizeof(double), 1, fp);
  fclose(fp);
  return 0;
}
