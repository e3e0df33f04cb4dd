/*
 * lbswim_oracle.c -- CPU restatement of the gpu-swimmers coupled step.
 *
 * TEST INFRASTRUCTURE ONLY (see lbswim_oracle.h).  The product library never
 * links or calls this file.
 *
 * Each function follows the reference's arithmetic order so that, compiled
 * with -ffp-contract=off, it reproduces a host build of the reference's own
 * kernels bit for bit.  Divergences from the reference are deliberate and
 * limited to its undefined behaviour:
 *   - SwimmerArray.cu:171: `norm` is read uninitialised; here it starts at 0.
 *   - SwimmerArray.cu:202-209: with rotational advection off and no tumble the
 *     reference normalises an uninitialised vector; here n is left unchanged.
 *   - TracerArray.cu:41: `part_s[d] += v[d]` races on particle 0; here each
 *     tracer accumulates its own unwrapped displacement s[d*n + i].
 *   - cuRAND XORWOW (SwimmerArray.cu:13,173,179) is replaced by a counter-based
 *     Philox4x32-10 stream keyed by (seed, swimmer, move step).
 */
#include "lbswim_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 0;

void orc_set_threads(int n) { g_threads = n; }

int orc_get_threads(void) {
#ifdef _OPENMP
  return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* D3Q15 tables (d3q15.c:2-186), built from their definitions.               */
/* ------------------------------------------------------------------------ */

/* Velocity ordering of d3q15.c:41-55: rest, +-x, +-y, +-z, then the eight
 * corners with x slowest and '+' before '-'. */
static const int kC[15][3] = {{0, 0, 0},  {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},   {0, -1, 0},
                              {0, 0, 1},  {0, 0, -1},  {1, 1, 1},  {1, 1, -1},  {1, -1, 1},
                              {1, -1, -1}, {-1, 1, 1}, {-1, 1, -1}, {-1, -1, 1}, {-1, -1, -1}};

/* Mode m evaluated on velocity c, as a rational num/den with den = 3 or 1. */
static void mode_value(int m, const int* c, long* num, long* den) {
  const int cx = c[0], cy = c[1], cz = c[2];
  const int c2 = cx * cx + cy * cy + cz * cz;
  /* chi1 = -2 + 9/2 |c|^2 - 3/2 |c|^4 takes the values -2, 1, -2 on |c|^2 = 0,1,3 */
  const int chi1 = (c2 == 1) ? 1 : -2;
  *den = 1;
  switch (m) {
    case 0: *num = 1; break;
    case 1: *num = cx; break;
    case 2: *num = cy; break;
    case 3: *num = cz; break;
    case 4: *num = 3 * cx * cx - 1; *den = 3; break; /* Q_xx */
    case 5: *num = cx * cy; break;
    case 6: *num = cx * cz; break;
    case 7: *num = 3 * cy * cy - 1; *den = 3; break; /* Q_yy */
    case 8: *num = cy * cz; break;
    case 9: *num = 3 * cz * cz - 1; *den = 3; break; /* Q_zz */
    case 10: *num = chi1; break;
    case 11: *num = chi1 * cx; break;
    case 12: *num = chi1 * cy; break;
    case 13: *num = chi1 * cz; break;
    default: *num = cx * cy * cz; break;
  }
}

/* Weights as rationals: 2/9, 1/9, 1/72. */
static void weight_value(const int* c, long* num, long* den) {
  const int c2 = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
  *num = (c2 == 0) ? 2 : 1;
  *den = (c2 == 0) ? 9 : (c2 == 1 ? 9 : 72);
}

static long gcdl(long a, long b) {
  if (a < 0) a = -a;
  if (b < 0) b = -b;
  while (b) {
    long t = a % b;
    a = b;
    b = t;
  }
  return a ? a : 1;
}

void orc_eigenset(orc_params* P, double tau_s, double tau_b) {
  memset(P, 0, sizeof(*P));
  P->cs2 = 1. / 3.;
  P->tau_s = tau_s;
  P->tau_b = tau_b;
  long wn[15], wd[15];
  for (int p = 0; p < 15; p++) {
    weight_value(kC[p], &wn[p], &wd[p]);
    P->w[p] = (double)wn[p] / (double)wd[p];
    for (int a = 0; a < 3; a++) {
      P->ci[p][a] = kC[p][a];
      P->xi[p][a] = (double)kC[p][a];
    }
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) {
        /* Q_ab = c_a c_b - delta_ab / 3, as one rounded quotient */
        long num = 3 * kC[p][a] * kC[p][b] - (a == b ? 1 : 0);
        P->Q[p][a][b] = (num % 3 == 0) ? (double)(num / 3) : (double)num / 3.;
      }
    /* complement: the velocity with every component negated */
    for (int q = 0; q < 15; q++)
      if (kC[q][0] == -kC[p][0] && kC[q][1] == -kC[p][1] && kC[q][2] == -kC[p][2])
        P->complement[p] = q;
  }
  for (int m = 0; m < 15; m++) {
    /* norms[m] = 1 / sum_p w_p mm[m][p]^2, accumulated as an exact rational */
    long sn = 0, sd = 1;
    for (int p = 0; p < 15; p++) {
      long mn, md;
      mode_value(m, kC[p], &mn, &md);
      long tn = wn[p] * mn * mn, td = wd[p] * md * md;
      long nn = sn * td + tn * sd, nd = sd * td;
      long g = gcdl(nn, nd);
      sn = nn / g;
      sd = nd / g;
    }
    /* norm = sd / sn */
    long nn = sd, nd = sn;
    P->norms[m] = (double)nn / (double)nd;
    for (int p = 0; p < 15; p++) {
      long mn, md;
      mode_value(m, kC[p], &mn, &md);
      P->mm[m][p] = (md == 1) ? (double)mn : (double)mn / (double)md;
      /* mmi[p][m] = w_p mm[m][p] norms[m], one rounding of the exact rational */
      long in = wn[p] * mn * nn, id = wd[p] * md * nd;
      long g = gcdl(in, id);
      in /= g;
      id /= g;
      if (id < 0) {
        id = -id;
        in = -in;
      }
      P->mmi[p][m] = (in == 0) ? 0.0 : (id == 1 ? (double)in : (double)in / (double)id);
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).                          */
/* ------------------------------------------------------------------------ */
void orc_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int round = 0; round < 10; round++) {
    if (round > 0) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

static void rng_block(uint64_t seed, uint32_t swimmer, uint64_t step, uint32_t block,
                      uint32_t out[4]) {
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  const uint32_t ctr[4] = {swimmer, (uint32_t)step, (uint32_t)(step >> 32), block};
  orc_philox4x32(ctr, key, out);
}

float orc_rng_uniform(uint64_t seed, uint32_t swimmer, uint64_t step) {
  uint32_t x[4];
  rng_block(seed, swimmer, step, 0u, x);
  return (float)((x[0] >> 8) + 1u) * 0x1.0p-24f;
}

static double u53(uint32_t a, uint32_t b) {
  const uint64_t m = ((uint64_t)a << 21) | (uint64_t)(b >> 11);
  return (double)(m + 1u) * 0x1.0p-53;
}

/* log x (0 < x, x normal) as a fixed sequence of IEEE double operations, so
 * that the oracle and the GPU form identical normals (no libm call, whose last
 * bits differ between libraries).  x = m 2^e with m in [sqrt(1/2), sqrt(2)];
 * log m = 2 atanh s with s = (m - 1)/(m + 1), |s| <= 0.1716, and
 * atanh s = s + s^3/3 + s^5/5 + ... to the s^27 term (Horner in z = s^2);
 * ln 2 is split into a 40-bit head and a tail so e ln2_hi is exact.  The same
 * operations, in the same order, are in the device code. */
static const double DET_LN2_HI = 0.69314718055920821, DET_LN2_LO = 7.3710025651677989e-13;
static const double DET_ATANH[13] = {
    0.33333333333333331, 0.20000000000000001, 0.14285714285714285, 0.1111111111111111,
    0.090909090909090912, 0.076923076923076927, 0.066666666666666666, 0.058823529411764705,
    0.052631578947368418, 0.047619047619047616, 0.043478260869565216, 0.040000000000000001,
    0.037037037037037035};
double orc_det_log(double x) {
  uint64_t b;
  memcpy(&b, &x, 8);
  int e = (int)((b >> 52) & 0x7ffu) - 1023;
  b = (b & 0x000fffffffffffffull) | 0x3ff0000000000000ull; /* m in [1, 2) */
  double m;
  memcpy(&m, &b, 8);
  if (m > 1.4142135623730951) {
    m = m * 0.5;
    e += 1;
  }
  const double s = (m - 1.0) / (m + 1.0);
  const double z = s * s;
  double p = DET_ATANH[12];
  for (int k = 11; k >= 0; --k) p = p * z + DET_ATANH[k];
  const double t = 2.0 * s;
  const double lm = t + t * (z * p);
  const double de = (double)e;
  return de * DET_LN2_HI + (de * DET_LN2_LO + lm);
}

/* sin(2 pi u), cos(2 pi u) for 0 <= u <= 1 a multiple of 2^-53: u = k/8 + f
 * with |f| <= 1/16 (exact), theta = 2 pi f, Taylor series of sin and cos to
 * the theta^17 and theta^18 terms, then the angle sum with sin, cos of
 * k pi / 4 in {0, +-1, +-sqrt(1/2)}. */
static const double DET_SIN[8] = {-0.16666666666666666, 0.0083333333333333332,
                                  -0.00019841269841269841, 2.7557319223985893e-06,
                                  -2.505210838544172e-08, 1.6059043836821613e-10,
                                  -7.6471637318198164e-13, 2.8114572543455206e-15};
static const double DET_COS[9] = {-0.5, 0.041666666666666664, -0.0013888888888888889,
                                  2.4801587301587302e-05, -2.7557319223985888e-07,
                                  2.08767569878681e-09, -1.1470745597729725e-11,
                                  4.7794773323873853e-14, -1.5619206968586225e-16};
void orc_det_sincos2pi(double u, double* sn, double* cs) {
  const double k = floor(u * 8.0 + 0.5);
  const double f = u - k * 0.125;
  const double th = f * 6.2831853071795862;
  const double z = th * th;
  double ps = DET_SIN[7];
  for (int i = 6; i >= 0; --i) ps = ps * z + DET_SIN[i];
  double pc = DET_COS[8];
  for (int i = 7; i >= 0; --i) pc = pc * z + DET_COS[i];
  const double s = th + th * (z * ps);
  const double c = 1.0 + z * pc;
  const double r = 0.70710678118654757;
  static const double SA[8] = {0., 1., 1., 1., 0., -1., -1., -1.};
  static const double CA[8] = {1., 1., 0., -1., -1., -1., 0., 1.};
  const int ki = ((int)k) & 7;
  const double sa = (ki & 1) ? SA[ki] * r : SA[ki], ca = (ki & 1) ? CA[ki] * r : CA[ki];
  *sn = sa * c + ca * s;
  *cs = ca * c - sa * s;
}

void orc_rng_normal3(uint64_t seed, uint32_t swimmer, uint64_t step, double out[3]) {
  uint32_t a[4], b[4];
  rng_block(seed, swimmer, step, 1u, a);
  rng_block(seed, swimmer, step, 2u, b);
  const double u1 = u53(a[0], a[1]), u2 = u53(a[2], a[3]);
  const double u3 = u53(b[0], b[1]), u4 = u53(b[2], b[3]);
  const double r1 = sqrt(-2.0 * orc_det_log(u1));
  const double r2 = sqrt(-2.0 * orc_det_log(u3));
  double s2, c2, s4, c4;
  orc_det_sincos2pi(u2, &s2, &c2);
  orc_det_sincos2pi(u4, &s4, &c4);
  out[0] = r1 * c2;
  out[1] = r1 * s2;
  out[2] = r2 * c4;
}

/* ------------------------------------------------------------------------ */
/* Peskin 4-point delta (delta.cu:6-25).                                       */
/* ------------------------------------------------------------------------ */
double orc_peskin_delta(double x) {
  const double ax = fabs(x);
  double root = -4. * x * x;
  double phi = -2. * ax;
  if (ax >= 2.0) return 0.;
  if (ax >= 1.0) {
    root += 12. * ax - 7.;
    phi += 5.;
    phi -= sqrt(root);
  } else {
    root += 4. * ax + 1;
    phi += 3.;
    phi += sqrt(root);
  }
  return 0.125 * phi;
}

/* ------------------------------------------------------------------------ */
/* Lattice ops (lb.cu).                                                        */
/* ------------------------------------------------------------------------ */
#define SITE(s, x, y, z) ((long)(x) * (s)[1] * (s)[2] + (long)(y) * (s)[2] + (long)(z))

/* DoInitFromHydro, lb.cu:314-371.  compat_sxz reproduces lb.cu:356, where the
 * xz stress is built from u_x*u_y instead of u_x*u_z. */
void orc_init_from_hydro(const orc_params* P, const int size[3], const double* rho,
                         const double* u, double* f, int compat_sxz) {
  const long N = (long)size[0] * size[1] * size[2];
#pragma omp parallel for num_threads(orc_get_threads())
  for (long ijk = 0; ijk < N; ijk++) {
    double mode[15];
    for (int m = 0; m < 15; m++) mode[m] = 0.0;
    const double r = rho[ijk];
    const double ux = u[ijk], uy = u[N + ijk], uz = u[2 * N + ijk];
    mode[0] = r;
    mode[1] = r * ux;
    mode[2] = r * uy;
    mode[3] = r * uz;
    mode[4] = r * ux * ux;
    mode[5] = r * ux * uy;
    mode[6] = compat_sxz ? r * ux * uy : r * ux * uz;
    mode[7] = r * uy * uy;
    mode[8] = r * uy * uz;
    mode[9] = r * uz * uz;
    for (int p = 0; p < 15; p++) {
      double acc = 0.;
      for (int m = 0; m < 15; m++) acc += mode[m] * P->mmi[p][m];
      f[p * N + ijk] = acc;
    }
  }
}

/* DoLatticeZeroForce, lb.cu:390-411. */
void orc_zero_force(const int size[3], double* force) {
  const long N = (long)size[0] * size[1] * size[2];
  for (long i = 0; i < 3 * N; i++) force[i] = 0.0;
}

/* DoStep, lb.cu:72-218: MRT collision with forcing, then push-stream with
 * periodic wrap. */
void orc_step(const orc_params* P, const int size[3], const double* fOld, const double* force,
              double* fNew) {
  const long N = (long)size[0] * size[1] * size[2];
  const double tau_s = P->tau_s, tau_b = P->tau_b;
  const double omega_s = 1.0 / (tau_s + 0.5);
  const double omega_b = 1.0 / (tau_b + 0.5);
#pragma omp parallel for collapse(2) num_threads(orc_get_threads())
  for (int x = 0; x < size[0]; x++)
    for (int y = 0; y < size[1]; y++)
      for (int z = 0; z < size[2]; z++) {
        const int site[3] = {x, y, z};
        const long ijk = SITE(size, x, y, z);
        double mode[15], S[3][3], u[3], fpost[15];
        for (int m = 0; m < 15; m++) {
          mode[m] = 0.;
          for (int p = 0; p < 15; p++) mode[m] += fOld[p * N + ijk] * P->mm[m][p];
        }
        double usq = 0., uDOTf = 0.;
        for (int a = 0; a < 3; a++) {
          const double Fa = force[a * N + ijk];
          u[a] = (mode[1 + a] + 0.5 * Fa) / mode[0];
          mode[1 + a] += Fa;
          usq += u[a] * u[a];
          uDOTf += u[a] * Fa;
        }
        S[0][0] = mode[4];
        S[0][1] = mode[5];
        S[0][2] = mode[6];
        S[1][0] = mode[5];
        S[1][1] = mode[7];
        S[1][2] = mode[8];
        S[2][0] = mode[6];
        S[2][1] = mode[8];
        S[2][2] = mode[9];
        double TrS = 0.;
        for (int a = 0; a < 3; a++) TrS += S[a][a];
        for (int a = 0; a < 3; a++) S[a][a] -= TrS / 3;
        TrS -= omega_b * (TrS - mode[0] * usq);
        TrS += 2. * omega_b * tau_b * uDOTf;
        for (int a = 0; a < 3; a++) {
          for (int b = 0; b < 3; b++) {
            const double d = (a == b) ? 1.0 : 0.0;
            S[a][b] -= omega_s * (S[a][b] - mode[0] * (u[a] * u[b] - usq * d));
            S[a][b] += 2. * omega_s * tau_s *
                       (u[a] * force[b * N + ijk] + force[a * N + ijk] * u[b] - 2. * uDOTf * d);
          }
          S[a][a] += TrS / 3;
        }
        mode[4] = S[0][0];
        mode[5] = S[0][1];
        mode[6] = S[0][2];
        mode[7] = S[1][1];
        mode[8] = S[1][2];
        mode[9] = S[2][2];
        mode[10] = 0.;
        mode[11] = 0.;
        mode[12] = 0.;
        mode[13] = 0.;
        mode[14] = 0.;
        for (int p = 0; p < 15; p++) {
          fpost[p] = 0.;
          for (int m = 0; m < 15; m++) fpost[p] += mode[m] * P->mmi[p][m];
        }
        for (int p = 0; p < 15; p++) {
          long dest = 0;
          const long stride[3] = {(long)size[1] * size[2], size[2], 1};
          for (int a = 0; a < 3; a++) {
            const int d = (site[a] + P->ci[p][a] + size[a]) % size[a];
            dest += d * stride[a];
          }
          fNew[p * N + dest] = fpost[p];
        }
      }
}

/* DoCalcHydro, lb.cu:250-295. Only the density and momentum modes are used,
 * each accumulated in the same order as the reference's dense loop. */
void orc_calc_hydro(const orc_params* P, const int size[3], const double* f,
                    const double* force, double* rho, double* u) {
  const long N = (long)size[0] * size[1] * size[2];
#pragma omp parallel for num_threads(orc_get_threads())
  for (long ijk = 0; ijk < N; ijk++) {
    double mode[4];
    for (int m = 0; m < 4; m++) {
      mode[m] = 0.;
      for (int p = 0; p < 15; p++) mode[m] += f[p * N + ijk] * P->mm[m][p];
    }
    rho[ijk] = mode[0];
    for (int a = 0; a < 3; a++) u[a * N + ijk] = (mode[1 + a] + 0.5 * force[a * N + ijk]) / mode[0];
  }
}

/* Stencil set-up shared by interpolation and spreading (interp.cu:23-30,
 * SwimmerArray.cu:50-57). */
static void stencil(const int size[3], const double r[3], int idx[3][4], double dl[3][4]) {
  for (int d = 0; d < 3; d++) {
    const double x0 = ceil(r[d] - 2.);
    for (int i = 0; i < 4; i++) {
      const double x = x0 + i;
      idx[d][i] = ((int)x + size[d]) % size[d];
      dl[d][i] = orc_peskin_delta(r[d] - x);
    }
  }
}

/* InterpVelocity, interp.cu:8-47. */
void orc_interp_velocity(const int size[3], const double* u, const double r[3], double v[3]) {
  const long N = (long)size[0] * size[1] * size[2];
  int idx[3][4];
  double dl[3][4];
  v[0] = v[1] = v[2] = 0.0;
  stencil(size, r, idx, dl);
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      for (int k = 0; k < 4; ++k) {
        const double d3 = dl[0][i] * dl[1][j] * dl[2][k];
        const long ijk = SITE(size, idx[0][i], idx[1][j], idx[2][k]);
        for (int d = 0; d < 3; ++d) v[d] += d3 * u[d * N + ijk];
      }
}

/* AccumulateDeltaForce, SwimmerArray.cu:42-79 (serial, so the summation order
 * is swimmer index order, tail before head). */
static void accumulate_delta_force(const int size[3], double* force, const double r[3],
                                   const double F[3]) {
  const long N = (long)size[0] * size[1] * size[2];
  int idx[3][4];
  double dl[3][4];
  stencil(size, r, idx, dl);
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      for (int k = 0; k < 4; ++k) {
        const long ijk = SITE(size, idx[0][i], idx[1][j], idx[2][k]);
        const double d3 = dl[0][i] * dl[1][j] * dl[2][k];
        for (int d = 0; d < 3; ++d) force[d * N + ijk] += d3 * F[d];
      }
}

/* DoSwimmerArrayAddForces, SwimmerArray.cu:82-112. */
void orc_swimmers_add_forces(const int size[3], double* force, int nsw, const orc_common* c,
                             const double* r, const double* n) {
  for (int i = 0; i < nsw; i++) {
    double rr[3], F[3];
    for (int a = 0; a < 3; a++) {
      rr[a] = r[nsw * a + i] - n[nsw * a + i] * c->l;
      F[a] = -c->P * n[nsw * a + i];
    }
    accumulate_delta_force(size, force, rr, F);
    for (int a = 0; a < 3; a++) {
      rr[a] = r[nsw * a + i];
      F[a] *= -1.0;
    }
    accumulate_delta_force(size, force, rr, F);
  }
}

/* DoSwimmerArrayMove, SwimmerArray.cu:123-210. */
void orc_swimmers_move(const int size[3], const double* u, int nsw, const orc_common* c,
                       uint64_t step, double* swr, double* swv, double* swn) {
#pragma omp parallel for num_threads(orc_get_threads())
  for (int i = 0; i < nsw; i++) {
    double v[3], r[3] = {swr[i], swr[nsw + i], swr[2 * nsw + i]};
    const double n0[3] = {swn[i], swn[nsw + i], swn[2 * nsw + i]};
    orc_interp_velocity(size, u, r, v);
    double rDot[3], rMinus[3];
    for (int d = 0; d < 3; d++) {
      rDot[d] = c->mobility * c->P * n0[d];
      if (!c->translational_advection_off) rDot[d] += v[d];
      rMinus[d] = r[d] - n0[d] * c->l;
    }
    for (int d = 0; d < 3; d++) {
      swv[nsw * d + i] = rDot[d];
      r[d] += rDot[d];
      swr[nsw * d + i] = fmod(r[d] + size[d], (double)size[d]);
    }
    double newn[3] = {n0[0], n0[1], n0[2]};
    double norm = 0.;
    const float rnd = orc_rng_uniform(c->seed, (uint32_t)i, step);
    int renorm = 1;
    if (rnd < c->alpha) {
      double g[3];
      orc_rng_normal3(c->seed, (uint32_t)i, step, g);
      for (int d = 0; d < 3; d++) {
        newn[d] = g[d];
        norm += newn[d] * newn[d];
      }
    } else if (!c->rotational_advection_off) {
      double vMinus[3], nDot[3];
      orc_interp_velocity(size, u, rMinus, vMinus);
      for (int d = 0; d < 3; d++) {
        nDot[d] = v[d] - vMinus[d];
        nDot[d] /= c->l;
      }
      for (int d = 0; d < 3; d++) {
        newn[d] = n0[d] + nDot[d];
        norm += newn[d] * newn[d];
      }
    } else {
      renorm = 0;
    }
    if (renorm) {
      norm = sqrt(norm);
      for (int d = 0; d < 3; d++) swn[nsw * d + i] = newn[d] / norm;
    }
  }
}

/* DoTracerArrayMove, TracerArray.cu:12-43, with s accumulated per tracer. */
void orc_tracers_move(const int size[3], const double* u, int ntr, double* r, double* s,
                      double* v) {
#pragma omp parallel for num_threads(orc_get_threads())
  for (int i = 0; i < ntr; i++) {
    double vv[3], rr[3] = {r[i], r[ntr + i], r[2 * ntr + i]};
    orc_interp_velocity(size, u, rr, vv);
    for (int d = 0; d < 3; d++) {
      v[ntr * d + i] = vv[d];
      rr[d] += vv[d];
      r[ntr * d + i] = fmod(rr[d] + size[d], (double)size[d]);
      s[ntr * d + i] += vv[d];
    }
  }
}

/* System.Step, System.py:9-16. */
void orc_system_step(orc_system* s, int nsteps) {
  for (int t = 0; t < nsteps; t++) {
    orc_zero_force(s->size, s->force);
    if (s->nsw > 0)
      orc_swimmers_add_forces(s->size, s->force, s->nsw, &s->common, s->sw_r, s->sw_n);
    orc_step(&s->params, s->size, s->f_old, s->force, s->f_new);
    double* tmp = s->f_old;
    s->f_old = s->f_new;
    s->f_new = tmp;
    s->time_step++;
    orc_calc_hydro(&s->params, s->size, s->f_old, s->force, s->rho, s->u);
    if (s->nsw > 0) {
      orc_swimmers_move(s->size, s->u, s->nsw, &s->common, s->sw_step, s->sw_r, s->sw_v,
                        s->sw_n);
      s->sw_step++;
    }
    if (s->ntr > 0) orc_tracers_move(s->size, s->u, s->ntr, s->tr_r, s->tr_s, s->tr_v);
  }
}
