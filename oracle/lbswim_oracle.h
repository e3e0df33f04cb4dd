/*
 * lbswim_oracle.h -- CPU restatement of the gpu-swimmers coupled step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA library is checked
 * against.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it; the product library never links or calls it.
 *
 * Everything is FP64 and follows the reference's arithmetic order, so that a
 * build with -ffp-contract=off reproduces a host build of the reference's own
 * kernels bit for bit (checked by tests/test_oracle_pin.py).
 *
 * Reference files restated (paths within rupertnash/gpu-swimmers):
 *   lbswim/liblbswim/d3q15.c:2-186        D3Q15 constants
 *   lbswim/liblbswim/lb.cu:72-218         DoStep (collide + push-stream)
 *   lbswim/liblbswim/lb.cu:250-295        DoCalcHydro
 *   lbswim/liblbswim/lb.cu:314-371        DoInitFromHydro
 *   lbswim/liblbswim/lb.cu:390-411        DoLatticeZeroForce
 *   lbswim/liblbswim/delta.cu:6-25        peskin_delta
 *   lbswim/liblbswim/interp.cu:8-47       InterpVelocity
 *   lbswim/liblbswim/SwimmerArray.cu:42-112   AccumulateDeltaForce / AddForces
 *   lbswim/liblbswim/SwimmerArray.cu:123-210  DoSwimmerArrayMove
 *   lbswim/liblbswim/TracerArray.cu:12-43     DoTracerArrayMove
 *   lbswim/System.py:9-16                 step order
 */
#ifndef LBSWIM_ORACLE_H
#define LBSWIM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
  double cs2;
  double w[15];
  double xi[15][3];
  int ci[15][3];
  double Q[15][3][3];
  int complement[15];
  double norms[15];
  double mm[15][15];
  double mmi[15][15];
  double tau_s;
  double tau_b;
} orc_params;

typedef struct orc_common {
  double P;
  double l;
  double alpha;
  double mobility;
  int translational_advection_off;
  int rotational_advection_off;
  uint64_t seed;
} orc_common;

/* D3Q15 model tables, built from their definitions (d3q15.c:2-186). */
void orc_eigenset(orc_params* p, double tau_s, double tau_b);

/* Philox4x32-10 block (Salmon et al., SC'11). */
void orc_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* Tumble uniform in (0,1] and three standard normals for (seed, swimmer, step). */
float orc_rng_uniform(uint64_t seed, uint32_t swimmer, uint64_t step);
double orc_det_log(double x);
void orc_det_sincos2pi(double u, double* s, double* c);
void orc_rng_normal3(uint64_t seed, uint32_t swimmer, uint64_t step, double out[3]);

double orc_peskin_delta(double x);

/* Lattice ops; size = {nx, ny, nz}; arrays are element-slowest SoA. */
void orc_init_from_hydro(const orc_params* p, const int size[3], const double* rho,
                         const double* u, double* f, int compat_sxz);
void orc_zero_force(const int size[3], double* force);
void orc_step(const orc_params* p, const int size[3], const double* f_old,
              const double* force, double* f_new);
void orc_calc_hydro(const orc_params* p, const int size[3], const double* f,
                    const double* force, double* rho, double* u);
void orc_interp_velocity(const int size[3], const double* u, const double r[3], double v[3]);

/* Particle ops. */
void orc_swimmers_add_forces(const int size[3], double* force, int nsw, const orc_common* c,
                             const double* r, const double* n);
void orc_swimmers_move(const int size[3], const double* u, int nsw, const orc_common* c,
                       uint64_t step, double* r, double* v, double* n);
void orc_tracers_move(const int size[3], const double* u, int ntr, double* r, double* s,
                      double* v);

/* One coupled step in the order of System.Step (System.py:9-16):
 * ZeroForce, AddForces (swimmers), Step, CalcHydro, Move (swimmers, tracers).
 * f_old/f_new are swapped by pointer on return. */
typedef struct orc_system {
  orc_params params;
  int size[3];
  double* f_old;
  double* f_new;
  double* rho;
  double* u;
  double* force;
  int nsw;
  orc_common common;
  uint64_t sw_step;
  double* sw_r;
  double* sw_v;
  double* sw_n;
  int ntr;
  double* tr_r;
  double* tr_s;
  double* tr_v;
  int time_step;
} orc_system;

void orc_system_step(orc_system* s, int nsteps);

/* Threads used by the OpenMP loops (0 = library default). */
void orc_set_threads(int n);
int orc_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
