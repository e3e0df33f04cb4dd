/* The reference's README scenario (README.md:80-130) driven from C through
 * include/lbswim_c.h alone, with the single calls a C++ user of liblbswim
 * makes (Lattice::ZeroForce, SwimmerArray::AddForces, Lattice::Step,
 * Lattice::CalcHydro, SwimmerArray::Move, TracerArray::Move): a 16^3 FP64
 * lattice at rest, one swimmer at (8, 8, 8) along +z, 4096 tracers on the
 * lattice nodes.
 *
 * usage: c_driver STEPS OUT
 * OUT receives, as raw doubles: rho[N], u[3N], swimmer r[3], n[3], tracer r[3N]. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "lbswim_c.h"

#define CHECK(call)                                                      \
  do {                                                                   \
    if ((call) != 0) {                                                   \
      fprintf(stderr, "%s failed: %s\n", #call, lbswim_last_error());    \
      return 1;                                                          \
    }                                                                    \
  } while (0)

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s STEPS OUT\n", argv[0]);
    return 2;
  }
  const int steps = atoi(argv[1]);
  enum { L = 16, N = L * L * L };
  static double rho[N], u[3 * N], tr_r[3 * N];
  double sw_r[3] = {8.0, 8.0, 8.0}, sw_n[3] = {0.0, 0.0, 1.0}, sw_v[3] = {0.0, 0.0, 0.0};
  const double tau = 0.25, eta = tau / 3.0, a = 0.1, hydro_radius = 1.5;
  const double pi = 3.14159265358979323846;

  lbswim_lattice* lat = NULL;
  lbswim_swimmers* sw = NULL;
  lbswim_tracers* tr = NULL;
  CHECK(lbswim_lattice_create(L, L, L, tau, tau, LBSWIM_F64, &lat));
  for (int i = 0; i < N; ++i) rho[i] = 1.0;
  CHECK(lbswim_lattice_h2d(lat, LBSWIM_FIELD_RHO, rho));
  CHECK(lbswim_lattice_h2d(lat, LBSWIM_FIELD_U, u));
  CHECK(lbswim_lattice_zero_force(lat));

  lbswim_common_params cp;
  cp.P = 1e-3;
  cp.l = 0.1;
  cp.alpha = 0.01;
  cp.mobility = (1.0 / a - 1.0 / hydro_radius) / (6.0 * pi * eta);
  cp.translational_advection_off = 0;
  cp.rotational_advection_off = 0;
  cp.seed = 1234;
  CHECK(lbswim_swimmers_create(1, &cp, &sw));
  CHECK(lbswim_swimmers_h2d(sw, LBSWIM_SW_R, sw_r));
  CHECK(lbswim_swimmers_h2d(sw, LBSWIM_SW_N, sw_n));
  CHECK(lbswim_swimmers_h2d(sw, LBSWIM_SW_V, sw_v));

  CHECK(lbswim_tracers_create(N, &tr));
  for (int x = 0; x < L; ++x)
    for (int y = 0; y < L; ++y)
      for (int z = 0; z < L; ++z) {
        const int k = (x * L + y) * L + z;
        tr_r[k] = x;
        tr_r[N + k] = y;
        tr_r[2 * N + k] = z;
      }
  CHECK(lbswim_tracers_h2d(tr, LBSWIM_TR_R, tr_r));

  CHECK(lbswim_lattice_init_from_hydro(lat));
  for (int t = 0; t < steps; ++t) {
    CHECK(lbswim_lattice_zero_force(lat));
    CHECK(lbswim_swimmers_add_forces(sw, lat));
    CHECK(lbswim_lattice_step(lat));
    CHECK(lbswim_lattice_calc_hydro(lat));
    CHECK(lbswim_swimmers_move(sw, lat));
    CHECK(lbswim_tracers_move(tr, lat));
  }
  int ts = -1;
  CHECK(lbswim_lattice_get_time_step(lat, &ts));
  if (ts != steps) {
    fprintf(stderr, "time_step %d, expected %d\n", ts, steps);
    return 1;
  }

  CHECK(lbswim_lattice_d2h(lat, LBSWIM_FIELD_RHO, rho));
  CHECK(lbswim_lattice_d2h(lat, LBSWIM_FIELD_U, u));
  CHECK(lbswim_swimmers_d2h(sw, LBSWIM_SW_R, sw_r));
  CHECK(lbswim_swimmers_d2h(sw, LBSWIM_SW_N, sw_n));
  CHECK(lbswim_tracers_d2h(tr, LBSWIM_TR_R, tr_r));
  FILE* out = fopen(argv[2], "wb");
  if (!out) {
    perror(argv[2]);
    return 1;
  }
  fwrite(rho, sizeof(double), N, out);
  fwrite(u, sizeof(double), 3 * N, out);
  fwrite(sw_r, sizeof(double), 3, out);
  fwrite(sw_n, sizeof(double), 3, out);
  fwrite(tr_r, sizeof(double), 3 * N, out);
  fclose(out);

  CHECK(lbswim_tracers_destroy(tr));
  CHECK(lbswim_swimmers_destroy(sw));
  CHECK(lbswim_lattice_destroy(lat));
  return 0;
}
