// The reference's README scenario (README.md:80-130) written against the
// reference's C++ class API -- Lattice, LatticeData, SharedArray, SharedItem,
// CommonParams, SwimmerArray, TracerArray -- as this library's headers
// (include/liblbswim/) provide it: a 16^3 FP64 lattice at rest, one swimmer at
// (8, 8, 8) along +z, 4096 tracers on the lattice nodes, the single calls of
// the README's step list.
//
// usage: cpp_driver STEPS OUT
// OUT receives, as raw doubles: rho[N], u[3N], swimmer r[3], n[3], tracer r[3N]
// (the layout tests/c_driver.c writes).
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "SwimmerArray.h"
#include "TracerArray.h"
#include "lb.h"

static int fail(const char* what) {
  std::fprintf(stderr, "cpp_driver: %s\n", what);
  return 1;
}

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s STEPS OUT\n", argv[0]);
    return 2;
  }
  const int steps = std::atoi(argv[1]);
  try {
    const int L = 16, N = L * L * L;
    const double tau = 0.25, eta = tau / 3.0, a = 0.1, hydro_radius = 1.5;
    const double pi = 3.14159265358979323846;
    // 1. the lattice and its hydrodynamic fields
    Lattice lat(L, L, L, tau, tau);
    if (lat.addr.host->n != N || lat.addr.host->strides[DQ_X] != L * L) return fail("addr");
    if (lat.params.host->tau_s != tau || std::fabs(lat.params.host->w[0] - 2.0 / 9.0) > 1e-16)
      return fail("params");
    LatticeData* d = lat.data;
    if (d->rho.size != (size_t)N || d->u.size != (size_t)(DQ_d * N) ||
        d->fOld.size != (size_t)(DQ_q * N))
      return fail("sizes");
    for (int i = 0; i < N; ++i) d->rho.host[i] = 1.0;
    d->rho.H2D();
    for (int i = 0; i < DQ_d * N; ++i) d->u.host[i] = 0.0;
    d->u.H2D();
    lat.ZeroForce();
    // 2. swimmers
    CommonParams cp;
    cp.P = 1e-3;
    cp.l = 0.1;
    cp.alpha = 0.01;
    cp.mobility = (1.0 / a - 1.0 / hydro_radius) / (6.0 * pi * eta);
    cp.translational_advection_off = false;
    cp.rotational_advection_off = false;
    cp.seed = 1234;
    SwimmerArray sw(1, &cp);
    for (int k = 0; k < 3; ++k) {
      sw.r.host[k] = 8.0;
      sw.n.host[k] = k == 2 ? 1.0 : 0.0;
      sw.v.host[k] = 0.0;
    }
    sw.r.H2D();
    sw.n.H2D();
    sw.v.H2D();
    if (sw.num != 1 || sw.common.host->seed != 1234 || sw.prng.host->seed != 1234)
      return fail("swimmer params");
    // 3. tracers on the lattice nodes
    TracerArray tr(N);
    for (int x = 0; x < L; ++x)
      for (int y = 0; y < L; ++y)
        for (int z = 0; z < L; ++z) {
          const int k = (x * L + y) * L + z;
          tr.r.host[k] = x;
          tr.r.host[N + k] = y;
          tr.r.host[2 * N + k] = z;
        }
    tr.r.H2D();
    tr.v.H2D();
    // 4. distributions from the fields; 5. the steps
    lat.InitFromHydro();
    for (int t = 0; t < steps; ++t) {
      const LDView before = d->Device();
      lat.ZeroForce();
      sw.AddForces(&lat);
      lat.Step();
      const LDView after = d->Device();
      if (after.fOld != before.fNew || after.fNew != before.fOld) return fail("f swap");
      lat.CalcHydro();
      sw.Move(&lat);
      tr.Move(&lat);
    }
    if (lat.time_step != steps) return fail("time_step");
    // 6. copy what we want to look at to the host
    d->rho.D2H();
    d->u.D2H();
    sw.r.D2H();
    sw.n.D2H();
    tr.r.D2H();
    sw.prng.D2H();
    if (sw.prng.host->step != (unsigned long long)steps) return fail("rng step");
    std::FILE* out = std::fopen(argv[2], "wb");
    if (!out) return fail("cannot open output");
    std::fwrite(d->rho.host, sizeof(double), N, out);
    std::fwrite(d->u.host, sizeof(double), 3 * N, out);
    std::fwrite(sw.r.host, sizeof(double), 3, out);
    std::fwrite(sw.n.host, sizeof(double), 3, out);
    std::fwrite(tr.r.host, sizeof(double), 3 * N, out);
    std::fclose(out);
  } catch (const lbswim_cxx::Error& e) {
    return fail(e.what());
  }
  return 0;
}
