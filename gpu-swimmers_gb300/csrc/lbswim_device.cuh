// lbswim_device.cuh -- device-side building blocks shared by the kernels.
//
// D3Q15 velocity ordering (reference d3q15.c:41-55): rest, +-x, +-y, +-z, then
// the eight corners (x, y, z) = +++, ++-, +-+, +--, -++, -+-, --+, --- .
// The distributions of a site are reduced to the ten moments the collision
// uses (rho, j, S) with a 3-stage butterfly over the corners, and rebuilt from
// them with the inverse butterfly.  This is the reference's dense 15x15
// transform (lb.cu:114-119, 198-203) with the zero entries and the zeroed
// ghost modes (lb.cu:191-195) taken out: f_p = w_p (rho + 3 c_p.j + 9/2 Q_p:S).
#pragma once
#include <cstring>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace lbswim {

__host__ __device__ constexpr int cx_of(int p) {
  return p == 1 ? 1 : p == 2 ? -1 : (p >= 7 && p <= 10) ? 1 : (p >= 11) ? -1 : 0;
}
__host__ __device__ constexpr int cy_of(int p) {
  return p == 3 ? 1 : p == 4 ? -1 : (p == 7 || p == 8 || p == 11 || p == 12) ? 1
         : (p == 9 || p == 10 || p == 13 || p == 14) ? -1 : 0;
}
__host__ __device__ constexpr int cz_of(int p) {
  return p == 5 ? 1 : p == 6 ? -1 : (p >= 7 && (p & 1)) ? 1 : (p >= 8 && !(p & 1)) ? -1 : 0;
}
__host__ __device__ constexpr double w_of(int p) {
  return p == 0 ? 2.0 / 9.0 : p <= 6 ? 1.0 / 9.0 : 1.0 / 72.0;
}

// Relaxation constants of one lattice (lb.cu:105-108, 165, 174).
template <class T>
struct Relax {
  T omega_s;  // 1 / (tau_s + 1/2)
  T omega_b;  // 1 / (tau_b + 1/2)
  T force_s;  // 2 omega_s tau_s
  T force_b;  // 2 omega_b tau_b
};

template <class T>
inline Relax<T> make_relax(double tau_s, double tau_b) {
  const double ws = 1.0 / (tau_s + 0.5), wb = 1.0 / (tau_b + 0.5);
  return Relax<T>{(T)ws, (T)wb, (T)(2. * ws * tau_s), (T)(2. * wb * tau_b)};
}

// Density-deviation, momentum and stress moments of 15 (deviation) values.
template <class T>
struct Moments {
  T R, jx, jy, jz, Sxx, Syy, Szz, Sxy, Sxz, Syz;
};

template <class T>
__device__ __forceinline__ Moments<T> moments(const T d[15]) {
  const T a = d[1] + d[2], ap = d[1] - d[2];
  const T b = d[3] + d[4], bp = d[3] - d[4];
  const T c = d[5] + d[6], cp = d[5] - d[6];
  const T P1 = d[7] + d[8], M1 = d[7] - d[8];
  const T P2 = d[9] + d[10], M2 = d[9] - d[10];
  const T P3 = d[11] + d[12], M3 = d[11] - d[12];
  const T P4 = d[13] + d[14], M4 = d[13] - d[14];
  const T PPp = P1 + P2, PMp = P1 - P2, MPp = M1 + M2, MMp = M1 - M2;
  const T PPm = P3 + P4, PMm = P3 - P4, MPm = M3 + M4, MMm = M3 - M4;
  const T sum = PPp + PPm;
  Moments<T> m;
  m.R = d[0] + a + b + c + sum;
  m.jx = ap + (PPp - PPm);
  m.jy = bp + (PMp + PMm);
  m.jz = cp + (MPp + MPm);
  const T r3 = m.R * (T(1) / T(3));
  m.Sxx = (a + sum) - r3;
  m.Syy = (b + sum) - r3;
  m.Szz = (c + sum) - r3;
  m.Sxy = PMp - PMm;
  m.Sxz = MPp - MPm;
  m.Syz = MMp + MMm;
  return m;
}

// Only rho-deviation and momentum (the CalcHydro moments, lb.cu:279-293).
template <class T>
__device__ __forceinline__ void hydro_moments(const T d[15], T& R, T& jx, T& jy, T& jz) {
  const T c1 = d[7] + d[8], c2 = d[9] + d[10], c3 = d[11] + d[12], c4 = d[13] + d[14];
  const T xp = c1 + c2, xm = c3 + c4;
  R = d[0] + (d[1] + d[2]) + (d[3] + d[4]) + (d[5] + d[6]) + (xp + xm);
  jx = (d[1] - d[2]) + (xp - xm);
  jy = (d[3] - d[4]) + ((c1 - c2) + (c3 - c4));
  const T z1 = d[7] - d[8], z2 = d[9] - d[10], z3 = d[11] - d[12], z4 = d[13] - d[14];
  jz = (d[5] - d[6]) + ((z1 + z2) + (z3 + z4));
}

// out_p = w_p (R + 3 c_p.j + 9/2 Q_p:S): the projection mmi * mode with the
// ghost modes zero (lb.cu:198-203, 363-369).
template <class T>
__device__ __forceinline__ void project(T R, T jx, T jy, T jz, T Sxx, T Syy, T Szz, T Sxy,
                                        T Sxz, T Syz, T out[15]) {
  const T w0 = T(2) / T(9), w1 = T(1) / T(9), w7 = T(1) / T(72);
  const T Tr = Sxx + Syy + Szz;
  const T Tr3 = Tr * (T(1) / T(3));
  out[0] = w0 * (R - T(1.5) * Tr);
  const T ex = R + T(4.5) * (Sxx - Tr3);
  const T ey = R + T(4.5) * (Syy - Tr3);
  const T ez = R + T(4.5) * (Szz - Tr3);
  const T jx3 = T(3) * jx, jy3 = T(3) * jy, jz3 = T(3) * jz;
  out[1] = w1 * (ex + jx3);
  out[2] = w1 * (ex - jx3);
  out[3] = w1 * (ey + jy3);
  out[4] = w1 * (ey - jy3);
  out[5] = w1 * (ez + jz3);
  out[6] = w1 * (ez - jz3);
  const T A = R + T(3) * Tr;
  const T Cxy = T(9) * Sxy, Cxz = T(9) * Sxz, Cyz = T(9) * Syz;
  {  // corners with c_x = +1
    const T G = A + jx3, Hy = jy3 + Cxy, Hz = jz3 + Cxz;
    const T K1 = G + Hy, K2 = G - Hy, L1 = Hz + Cyz, L2 = Hz - Cyz;
    out[7] = w7 * (K1 + L1);
    out[8] = w7 * (K1 - L1);
    out[9] = w7 * (K2 + L2);
    out[10] = w7 * (K2 - L2);
  }
  {  // corners with c_x = -1
    const T G = A - jx3, Hy = jy3 - Cxy, Hz = jz3 - Cxz;
    const T K1 = G + Hy, K2 = G - Hy, L1 = Hz + Cyz, L2 = Hz - Cyz;
    out[11] = w7 * (K1 + L1);
    out[12] = w7 * (K1 - L1);
    out[13] = w7 * (K2 + L2);
    out[14] = w7 * (K2 - L2);
  }
}

// MRT collision with forcing, lb.cu:121-195, on deviations d_p = f_p - w_p rho0
// (rho0 = 0 gives the reference's plain distributions).  out may alias d.
template <class T>
__device__ __forceinline__ void collide(const T d[15], T Fx, T Fy, T Fz, T rho0,
                                        const Relax<T>& k, T out[15]) {
  const Moments<T> m = moments(d);
  const T rho = rho0 + m.R;
  const T inv = T(1) / rho;
  const T ux = (m.jx + T(0.5) * Fx) * inv;
  const T uy = (m.jy + T(0.5) * Fy) * inv;
  const T uz = (m.jz + T(0.5) * Fz) * inv;
  const T usq = ux * ux + uy * uy + uz * uz;
  const T uF = ux * Fx + uy * Fy + uz * Fz;
  const T third = T(1) / T(3);
  const T TrS = m.Sxx + m.Syy + m.Szz;
  const T tx = m.Sxx - TrS * third, ty = m.Syy - TrS * third, tz = m.Szz - TrS * third;
  // trace relaxed with omega_b toward rho u.u, plus forcing (lb.cu:163-165)
  const T TrN = TrS - k.omega_b * (TrS - rho * usq) + k.force_b * uF;
  const T tr3 = TrN * third;
  const T ws = k.omega_s, fs = k.force_s;
  // traceless part relaxed with omega_s, plus forcing (lb.cu:168-178)
  const T Sxx = tx - ws * (tx - rho * (ux * ux - usq)) + fs * (T(2) * ux * Fx - T(2) * uF) + tr3;
  const T Syy = ty - ws * (ty - rho * (uy * uy - usq)) + fs * (T(2) * uy * Fy - T(2) * uF) + tr3;
  const T Szz = tz - ws * (tz - rho * (uz * uz - usq)) + fs * (T(2) * uz * Fz - T(2) * uF) + tr3;
  const T Sxy = m.Sxy - ws * (m.Sxy - rho * ux * uy) + fs * (ux * Fy + Fx * uy);
  const T Sxz = m.Sxz - ws * (m.Sxz - rho * ux * uz) + fs * (ux * Fz + Fx * uz);
  const T Syz = m.Syz - ws * (m.Syz - rho * uy * uz) + fs * (uy * Fz + Fy * uz);
  project(m.R, m.jx + Fx, m.jy + Fy, m.jz + Fz, Sxx, Syy, Szz, Sxy, Sxz, Syz, out);
}

// ---- storage formats of the distributions -----------------------------------
// FP64 and FP32 hold f_p - w_p rho0 (rho0 = 0 for FP64: the plain distribution).
// BF16 and FP16 hold (f_p - w_p rho0) / w_p so all 15 values share one scale.
template <class S>
struct Store;
template <>
struct Store<double> {
  static constexpr bool scaled = false;
  __device__ static double ld(const double* p) { return *p; }
  __device__ static void st(double* p, double v) { *p = v; }
};
template <>
struct Store<float> {
  static constexpr bool scaled = false;
  __device__ static float ld(const float* p) { return *p; }
  __device__ static void st(float* p, float v) { *p = v; }
};
template <>
struct Store<__nv_bfloat16> {
  static constexpr bool scaled = true;
  __device__ static float ld(const __nv_bfloat16* p) { return __bfloat162float(*p); }
  __device__ static void st(__nv_bfloat16* p, float v) { *p = __float2bfloat16_rn(v); }
};
template <>
struct Store<__half> {
  static constexpr bool scaled = true;
  __device__ static float ld(const __half* p) { return __half2float(*p); }
  __device__ static void st(__half* p, float v) { *p = __float2half_rn(v); }
};

// Element of population p at site s in a distribution buffer of N sites.
// FP64 buffers keep the reference's [15][N]; reduced-precision buffers hold
// blocks of 32 consecutive sites, [ceil(N/32)][15][32], so that the 15 values
// of a warp's 32 sites lie at fixed offsets p * 32 from one address (the
// offsets go into the load and store instructions).
template <class S, class I>
__host__ __device__ __forceinline__ I fidx(int p, I s, I N) {
  if constexpr (sizeof(S) == 8)
    return (I)p * N + s;
  else
    return ((s >> 5) * 15 + p) * 32 + (s & 31);
}

template <class S, class T>
__device__ __forceinline__ T dev_from_stored(T g, int p) {
  return Store<S>::scaled ? g * T(w_of(p)) : g;
}
template <class S, class T>
__device__ __forceinline__ T stored_from_dev(T d, int p) {
  return Store<S>::scaled ? d * T(1.0 / w_of(p)) : d;
}

// ---- Peskin 4-point regularised delta (delta.cu:6-25) ------------------------
template <class T>
__device__ __forceinline__ T peskin_delta(T x) {
  const T ax = fabs(x);
  T root = T(-4) * x * x;
  T phi = T(-2) * ax;
  if (ax >= T(2)) return T(0);
  if (ax >= T(1)) {
    root += T(12) * ax - T(7);
    phi += T(5);
    phi -= sqrt(root);
  } else {
    root += T(4) * ax + T(1);
    phi += T(3);
    phi += sqrt(root);
  }
  return T(0.125) * phi;
}
// The four weights phi(dr - j), j = 0..3, of a stencil whose origin is
// ceil(x - 2), so that 1 <= dr <= 2 (FP32 paths).  With a = dr - 1 the four
// distances are 1 + a, a, 1 - a and 2 - a; both branches of the delta above
// then take the same square root, s = sqrt(1 + 4a(1 - a)), and
// phi = (3 - 2a - s, 3 - 2a + s, 1 + 2a + s, 1 + 2a - s) / 8: one square root
// for the four weights, which sum to one up to rounding.  Each weight is at
// most 1/2, as the delta's.
__device__ __forceinline__ void peskin_weights4(float dr, float w[4]) {
  const float a = dr - 1.f;  // exact for 1 <= dr <= 2
  const float s = sqrtf(fmaf(4.f * a, 1.f - a, 1.f));
  const float p = 3.f - 2.f * a, q = 1.f + 2.f * a;
  w[0] = 0.125f * (p - s);
  w[1] = 0.125f * (p + s);
  w[2] = 0.125f * (q + s);
  w[3] = 0.125f * (q - s);
}

// The same four weights in FP64 (the default FP64 particle moves; exact mode
// keeps the reference's delta per node, below).
__device__ __forceinline__ void peskin_weights4(double dr, double w[4]) {
  const double a = dr - 1.0;
  const double s = sqrt(fma(4.0 * a, 1.0 - a, 1.0));
  const double p = 3.0 - 2.0 * a, q = 1.0 + 2.0 * a;
  w[0] = 0.125 * (p - s);
  w[1] = 0.125 * (p + s);
  w[2] = 0.125 * (q + s);
  w[3] = 0.125 * (q - s);
}

// FP64: the reference's operations in its order, each rounded on its own (no
// fused multiply-add), so that FP64 lattices can reproduce the oracle bit for bit.
template <>
__device__ __forceinline__ double peskin_delta<double>(double x) {
  const double ax = fabs(x);
  double root = __dmul_rn(__dmul_rn(-4.0, x), x);
  double phi = __dmul_rn(-2.0, ax);
  if (ax >= 2.0) return 0.0;
  if (ax >= 1.0) {
    root = __dadd_rn(root, __dsub_rn(__dmul_rn(12.0, ax), 7.0));
    phi = __dadd_rn(phi, 5.0);
    phi = __dsub_rn(phi, __dsqrt_rn(root));
  } else {
    root = __dadd_rn(root, __dadd_rn(__dmul_rn(4.0, ax), 1.0));
    phi = __dadd_rn(phi, 3.0);
    phi = __dadd_rn(phi, __dsqrt_rn(root));
  }
  return __dmul_rn(0.125, phi);
}

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) ------------------------
__device__ __forceinline__ void philox4x32(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint32_t lo0 = 0xD2511F53u * c[0], hi0 = __umulhi(0xD2511F53u, c[0]);
    const uint32_t lo1 = 0xCD9E8D57u * c[2], hi1 = __umulhi(0xCD9E8D57u, c[2]);
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
  }
}

// Random stream of one swimmer at one move step.  Block 0 gives the tumble
// uniform in (0, 1]; blocks 1 and 2 give three Box-Muller normals.
__device__ __forceinline__ void rng_block(uint64_t seed, uint32_t swimmer, uint64_t step,
                                          uint32_t block, uint32_t out[4]) {
  out[0] = swimmer;
  out[1] = (uint32_t)step;
  out[2] = (uint32_t)(step >> 32);
  out[3] = block;
  philox4x32(out, (uint32_t)seed, (uint32_t)(seed >> 32));
}
__device__ __forceinline__ float rng_uniform(uint64_t seed, uint32_t swimmer, uint64_t step) {
  uint32_t x[4];
  rng_block(seed, swimmer, step, 0u, x);
  return (float)((x[0] >> 8) + 1u) * 0x1.0p-24f;
}
__device__ __forceinline__ double u53(uint32_t a, uint32_t b) {
  const uint64_t m = ((uint64_t)a << 21) | (uint64_t)(b >> 11);
  return (double)(m + 1u) * 0x1.0p-53;
}
// log x for a normal x > 0, as a fixed sequence of correctly rounded FP64
// operations (the oracle performs the same ones): x = m 2^e with m in
// [sqrt(1/2), sqrt(2)], log m = 2 atanh s, s = (m - 1)/(m + 1), the atanh
// series to the s^27 term in Horner form, ln 2 split into a 40-bit head
// (e ln2_hi exact) and a tail.
__device__ __forceinline__ double det_log(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  int e = (int)((b >> 52) & 0x7ffu) - 1023;
  b = (b & 0x000fffffffffffffull) | 0x3ff0000000000000ull;  // m in [1, 2)
  double m = __longlong_as_double((long long)b);
  if (m > 1.4142135623730951) {
    m = __dmul_rn(m, 0.5);
    e += 1;
  }
  const double s = __ddiv_rn(__dsub_rn(m, 1.0), __dadd_rn(m, 1.0));
  const double z = __dmul_rn(s, s);
  double p = 0.037037037037037035;  // 1/27 ... 1/3
  p = __dadd_rn(__dmul_rn(p, z), 0.040000000000000001);
  p = __dadd_rn(__dmul_rn(p, z), 0.043478260869565216);
  p = __dadd_rn(__dmul_rn(p, z), 0.047619047619047616);
  p = __dadd_rn(__dmul_rn(p, z), 0.052631578947368418);
  p = __dadd_rn(__dmul_rn(p, z), 0.058823529411764705);
  p = __dadd_rn(__dmul_rn(p, z), 0.066666666666666666);
  p = __dadd_rn(__dmul_rn(p, z), 0.076923076923076927);
  p = __dadd_rn(__dmul_rn(p, z), 0.090909090909090912);
  p = __dadd_rn(__dmul_rn(p, z), 0.1111111111111111);
  p = __dadd_rn(__dmul_rn(p, z), 0.14285714285714285);
  p = __dadd_rn(__dmul_rn(p, z), 0.20000000000000001);
  p = __dadd_rn(__dmul_rn(p, z), 0.33333333333333331);
  const double t = __dmul_rn(2.0, s);
  const double lm = __dadd_rn(t, __dmul_rn(t, __dmul_rn(z, p)));
  const double de = (double)e;
  return __dadd_rn(__dmul_rn(de, 0.69314718055920821),
                   __dadd_rn(__dmul_rn(de, 7.3710025651677989e-13), lm));
}

// sin(2 pi u), cos(2 pi u) for 0 <= u <= 1 a multiple of 2^-53 (the oracle
// performs the same operations): u = k/8 + f, |f| <= 1/16, theta = 2 pi f,
// Taylor series to theta^17 / theta^18, then the angle sum with sin, cos of
// k pi / 4.
__device__ __forceinline__ void det_sincos2pi(double u, double& sn, double& cs) {
  const double k = floor(__dadd_rn(__dmul_rn(u, 8.0), 0.5));
  const double f = __dsub_rn(u, __dmul_rn(k, 0.125));
  const double th = __dmul_rn(f, 6.2831853071795862);
  const double z = __dmul_rn(th, th);
  double ps = 2.8114572543455206e-15;
  ps = __dadd_rn(__dmul_rn(ps, z), -7.6471637318198164e-13);
  ps = __dadd_rn(__dmul_rn(ps, z), 1.6059043836821613e-10);
  ps = __dadd_rn(__dmul_rn(ps, z), -2.505210838544172e-08);
  ps = __dadd_rn(__dmul_rn(ps, z), 2.7557319223985893e-06);
  ps = __dadd_rn(__dmul_rn(ps, z), -0.00019841269841269841);
  ps = __dadd_rn(__dmul_rn(ps, z), 0.0083333333333333332);
  ps = __dadd_rn(__dmul_rn(ps, z), -0.16666666666666666);
  double pc = -1.5619206968586225e-16;
  pc = __dadd_rn(__dmul_rn(pc, z), 4.7794773323873853e-14);
  pc = __dadd_rn(__dmul_rn(pc, z), -1.1470745597729725e-11);
  pc = __dadd_rn(__dmul_rn(pc, z), 2.08767569878681e-09);
  pc = __dadd_rn(__dmul_rn(pc, z), -2.7557319223985888e-07);
  pc = __dadd_rn(__dmul_rn(pc, z), 2.4801587301587302e-05);
  pc = __dadd_rn(__dmul_rn(pc, z), -0.0013888888888888889);
  pc = __dadd_rn(__dmul_rn(pc, z), 0.041666666666666664);
  pc = __dadd_rn(__dmul_rn(pc, z), -0.5);
  const double s = __dadd_rn(th, __dmul_rn(th, __dmul_rn(z, ps)));
  const double c = __dadd_rn(1.0, __dmul_rn(z, pc));
  const int ki = ((int)k) & 7;
  const double r = 0.70710678118654757;
  double sa = (ki == 0 || ki == 4) ? 0.0 : ((ki == 2) ? 1.0 : ((ki == 6) ? -1.0 : (ki < 4 ? 1.0 : -1.0)));
  double ca = (ki == 2 || ki == 6) ? 0.0 : ((ki == 0) ? 1.0 : ((ki == 4) ? -1.0 : ((ki == 1 || ki == 7) ? 1.0 : -1.0)));
  if (ki & 1) {
    sa = __dmul_rn(sa, r);
    ca = __dmul_rn(ca, r);
  }
  sn = __dadd_rn(__dmul_rn(sa, c), __dmul_rn(ca, s));
  cs = __dsub_rn(__dmul_rn(ca, c), __dmul_rn(sa, s));
}

// Three normal deviates of a tumble (Box-Muller on 53-bit uniforms).
__device__ __forceinline__ void rng_normal3(uint64_t seed, uint32_t swimmer, uint64_t step,
                                            double g[3]) {
  uint32_t a[4], b[4];
  rng_block(seed, swimmer, step, 1u, a);
  rng_block(seed, swimmer, step, 2u, b);
  const double r1 = __dsqrt_rn(__dmul_rn(-2.0, det_log(u53(a[0], a[1]))));
  const double r2 = __dsqrt_rn(__dmul_rn(-2.0, det_log(u53(b[0], b[1]))));
  double s2, c2, s4, c4;
  det_sincos2pi(u53(a[2], a[3]), s2, c2);
  det_sincos2pi(u53(b[2], b[3]), s4, c4);
  g[0] = __dmul_rn(r1, c2);
  g[1] = __dmul_rn(r1, s2);
  g[2] = __dmul_rn(r2, c4);
}

// ---- sticky status bits (LBSWIM_STATUS_* of lbswim_c.h) ---------------------
// x is finite (false for NaN and +-inf).
__device__ __forceinline__ bool finite_f(float x) { return fabsf(x) < __int_as_float(0x7f800000); }
__device__ __forceinline__ bool finite_d(double x) {
  return fabs(x) < __longlong_as_double(0x7ff0000000000000ll);
}
__device__ __forceinline__ void raise_status(unsigned* status, unsigned bit) {
  if (status) atomicOr(status, bit);
}
// A moved particle's new coordinate must lie in [0, n) (false for NaN).
__device__ __forceinline__ bool in_box(double x, int n) { return x >= 0.0 && x < (double)n; }

__device__ __forceinline__ int wrap_once(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

__device__ __forceinline__ int wrap_any(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

// x0 = ceil(x - 2) and dr = (float)(x - x0) for one coordinate, with the
// rounding of those FP64 operations.  For 0 <= x < 2^30 both come from the
// bits of x by integer operations: x - x0 is exact in FP64 unless x < 1, where
// 1 + x is first rounded to FP64's 52 fraction bits, then to FP32's 23.  Other
// values take FP64.
__device__ __forceinline__ void stencil_axis(double x, int& x0, float& dr) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)(b >> 52);  // biased exponent; negative x gives ex >= 2048
  if (ex >= 1023 + 30) {
    const double c = ceil(x - 2.);
    x0 = (int)c;
    dr = (float)(x - c);
    return;
  }
  if (ex < 1023 - 40) {  // 0 <= x < 2^-40: x - 2 rounds to -2 when x <= 2^-53
    const bool low = b <= (970ull << 52);
    x0 = low ? -2 : -1;
    dr = low ? 2.f : 1.f;
    return;
  }
  const unsigned long long mant = (b & 0xfffffffffffffull) | (1ull << 52);
  const int shift = 1075 - ex;  // x = mant * 2^-shift, 23 <= shift <= 92
  unsigned long long f52;       // fraction of x - x0 in 2^-52 units
  if (shift <= 52) {
    const unsigned long long fr = mant & ((1ull << shift) - 1);
    const int cell = (int)(mant >> shift);
    if (fr == 0) {  // x is an integer
      x0 = cell - 2;
      dr = 2.f;
      return;
    }
    x0 = cell - 1;
    f52 = fr << (52 - shift);
  } else {  // 2^-40 <= x < 1
    x0 = -1;
    const int s = shift - 52;  // 1 .. 40
    const unsigned long long rem = mant & ((1ull << s) - 1), half = 1ull << (s - 1);
    f52 = mant >> s;
    f52 += (rem > half || (rem == half && (f52 & 1ull))) ? 1ull : 0ull;
  }
  // to 23 fraction bits; a carry out gives 2.0f
  unsigned m = (unsigned)(f52 >> 29);
  const unsigned rem = (unsigned)(f52 & 0x1fffffffull);
  m += (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ? 1u : 0u;
  dr = __int_as_float(0x3f800000 + (int)m);
}

// Exponent S of the fixed-point force contributions (scale 2^S).  One
// end-node contribution is at most w |F|: w = 1/8, the largest product of three
// Peskin weights (each at most 1/2), when every axis has 4 or more sites, and
// w = 1 when stencil nodes fold onto one site.  With the largest force
// component the float with bits `max_bits`, S keeps w max|F| 2^S below 2^30, so
// every quantised contribution fits a 32-bit integer; a site's 64-bit sum of at
// most 16 contributions from each of fewer than 2^28 ends cannot overflow.
// Integer and FP32 operations only, so every kernel that spreads derives the
// same S.
__host__ __device__ inline int fixed_scale_exp(unsigned max_bits, bool fold) {
  float m;
  memcpy(&m, &max_bits, sizeof(float));
  if (!(m > 0.f)) return 30;
  // 1 + 2^-20 covers the rounding of the weights and of this product
  const float b = m * (fold ? 1.0f : 0.125f) * 1.00000095367431640625f;
  unsigned bb;
  memcpy(&bb, &b, sizeof(float));
  const int e = (int)((bb >> 23) & 0xffu) - 127;  // floor(log2 b) for a normal b
  const int S = 29 - e;                           // b 2^S < 2^(e+1) 2^S = 2^30
  return S < -100 ? -100 : (S > 100 ? 100 : S);
}
__host__ __device__ inline float exp2_int(int S) {  // 2^S for -126 <= S <= 127
  const unsigned u = (unsigned)(S + 127) << 23;
  float f;
  memcpy(&f, &u, sizeof(float));
  return f;
}

// ---- dipole ends of the force spreading (SwimmerArray.cu:42-112) ---------------
template <class T>
struct EndRecord {
  int o[3];  // wrapped stencil origin ceil(r - 2)
  int pad;
  T phi[3][4];  // Peskin weights of the 4 stencil nodes per axis
  T F[3];       // force carried by the end
};

// Weight of one axis: sum of phi[i] over stencil nodes (o + i) mod n equal to x.
template <class T>
__device__ __forceinline__ T axis_weight(int x, int o, int n, const T phi[4]) {
  if (n >= 4) {
    int d = x - o;
    if (d < 0) d += n;
    return d <= 3 ? phi[d] : T(0);
  }
  T w = T(0);
#pragma unroll
  for (int i = 0; i < 4; ++i)
    if ((o + i) % n == x) w += phi[i];
  return w;
}

// Does the stencil of an end with origin o cover coordinate x on an axis of n
// sites?  (With n < 4 its four nodes cover every coordinate.)
__device__ __forceinline__ bool covers_axis(int x, int o, int n) {
  if (n < 4) return true;
  int d = x - o;
  if (d < 0) d += n;
  return d <= 3;
}

// Does the stencil of an end with origin o cover coordinate x on an axis of n
// sites, and with which summed weight (n < 4 folds several nodes onto x)?
template <class T>
__device__ __forceinline__ bool cover_weight(int x, int o, int n, const T phi[4], T& w) {
  if (n >= 4) {
    int d = x - o;
    if (d < 0) d += n;
    if (d > 3) return false;
    w = phi[d];
    return true;
  }
  w = axis_weight(x, o, n, phi);
  return true;
}

// One end's contribution to one force component at a site.  FP64 keeps the
// reference's order ((phi_x phi_y) phi_z) F (SwimmerArray.cu:64-73); FP32
// evaluates (phi_y phi_z)(phi_x F) so that phi_x F can be formed once per x
// plane.  Every FP32 kernel that spreads uses this one expression, so the
// step kernel's own spreading and the materialised force agree bit for bit.
__device__ __forceinline__ double end_contrib(double wx, double wy, double wz, double F) {
  return __dmul_rn(__dmul_rn(__dmul_rn(wx, wy), wz), F);
}
__device__ __forceinline__ float end_contrib_f(float wy, float wz, float wxF) {
  return (wy * wz) * wxF;
}

// ---- fixed-point force accumulation (FP32 lattices) ---------------------------
// Each end-node contribution c = (phi_y phi_z)(phi_x F) is quantised to the
// 32-bit integer round(c 2^S) (S from fixed_scale_exp) and summed in 64-bit
// integers.  Integer sums are exact, so the force is the same whatever order
// the contributions arrive in: the step kernel's shared-memory atomics and the
// force kernel give identical bits.
__device__ __forceinline__ int fx_quant32(float c, float scale) { return __float2int_rn(c * scale); }
// float of the 64-bit sum q * inv_scale, from its two 32-bit halves.  A sum
// that fits 32 bits converts in one step (a small negative sum would otherwise
// cancel between -2^32 and the rounded low half); a larger one is within two
// float roundings.
__device__ __forceinline__ float fx_value(long long q, float inv_scale) {
  const int hi = (int)(q >> 32);
  const unsigned lo = (unsigned)(q & 0xffffffffll);
  if (hi == ((int)lo >> 31)) return __int2float_rn((int)lo) * inv_scale;
  return (__int2float_rn(hi) * 4294967296.f + __uint2float_rn(lo)) * inv_scale;
}
// round(c * scale) as a 64-bit integer using only 32-bit conversions (the 64-bit
// ones run on GB300's narrow FP64 pipe).  v = c * scale is exact (power of two);
// when |v| >= 2^31 it is an integer with at most 24 significant bits, split
// exactly into hi * 2^32 + lo.
__device__ __forceinline__ long long fx_quant(float c, float scale) {
  const float v = c * scale;
  if (fabsf(v) < 2147483648.f) return (long long)__float2int_rn(v);
  const float hi = floorf(v * 2.3283064365386963e-10f);  // v / 2^32
  const float lo = v - hi * 4294967296.f;                 // exact, in [0, 2^32)
  return (long long)(int)hi * 4294967296ll + (long long)__float2uint_rn(lo);
}
__device__ __forceinline__ float node_contrib(float py, float pz, float wx, float F) {
  return (py * pz) * (wx * F);
}

// Rank of key k among the cnt distinct keys: its position in increasing order.
__device__ __forceinline__ int rank_of(int k, const int* keys, int cnt) {
  int r = 0;
  for (int j = 0; j < cnt; ++j) r += keys[j] < k;
  return r;
}



}  // namespace lbswim
