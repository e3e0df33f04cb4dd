// lattice.cu -- D3Q15 MRT lattice-Boltzmann kernels and Lattice operations.
//
// Two methods share the Lattice object:
//  * FP64 (LBSWIM_F64): the reference's method, one kernel per reference op.
//    Step is collide + push-stream (lb.cu:72-218) with Z, the contiguous axis,
//    across the warp; CalcHydro is its own kernel (lb.cu:250-295).
//  * FP32 / BF16 / FP16: one fused kernel per Step that reads f(t) and F(t),
//    collides a tile plus a one-site halo, streams inside shared memory and
//    writes f(t+1) together with rho(t+1), u(t+1).  CalcHydro then only has to
//    publish those fields (pointer swap) when nothing changed since the Step.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstring>

#include "bulk_copy.cuh"
#include "lbswim_device.cuh"
#include "lbswim_internal.h"
#include "spread_slab.cuh"

namespace lbswim {

// ---------------------------------------------------------------------------
// LBParams tables (reference d3q15.c:2-186), built from their definitions.
// ---------------------------------------------------------------------------
static const int kC[15][3] = {{0, 0, 0},   {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
                              {0, 0, 1},   {0, 0, -1},  {1, 1, 1},  {1, 1, -1}, {1, -1, 1},
                              {1, -1, -1}, {-1, 1, 1},  {-1, 1, -1}, {-1, -1, 1}, {-1, -1, -1}};

// Mode m on velocity c as num/den (den 1 or 3); rows follow d3q15.h:13-28.
static void mode_rational(int m, const int* c, long& num, long& den) {
  const int x = c[0], y = c[1], z = c[2], c2 = x * x + y * y + z * z;
  const int chi1 = c2 == 1 ? 1 : -2;
  den = 1;
  switch (m) {
    case 0: num = 1; break;
    case 1: num = x; break;
    case 2: num = y; break;
    case 3: num = z; break;
    case 4: num = 3 * x * x - 1; den = 3; break;
    case 5: num = x * y; break;
    case 6: num = x * z; break;
    case 7: num = 3 * y * y - 1; den = 3; break;
    case 8: num = y * z; break;
    case 9: num = 3 * z * z - 1; den = 3; break;
    case 10: num = chi1; break;
    case 11: num = chi1 * x; break;
    case 12: num = chi1 * y; break;
    case 13: num = chi1 * z; break;
    default: num = x * y * z; break;
  }
}

static long gcd_l(long a, long b) {
  a = a < 0 ? -a : a;
  b = b < 0 ? -b : b;
  while (b) {
    const long t = a % b;
    a = b;
    b = t;
  }
  return a ? a : 1;
}

static double ratio(long num, long den) {
  if (den < 0) {
    num = -num;
    den = -den;
  }
  const long g = gcd_l(num, den);
  num /= g;
  den /= g;
  return den == 1 ? (double)num : (double)num / (double)den;
}

void fill_params(lbswim_lbparams* P, double tau_s, double tau_b) {
  std::memset(P, 0, sizeof(*P));
  P->cs2 = 1. / 3.;
  P->tau_s = tau_s;
  P->tau_b = tau_b;
  long wn[15], wd[15];
  for (int p = 0; p < 15; ++p) {
    const int c2 = kC[p][0] * kC[p][0] + kC[p][1] * kC[p][1] + kC[p][2] * kC[p][2];
    wn[p] = c2 == 0 ? 2 : 1;
    wd[p] = c2 == 0 ? 9 : (c2 == 1 ? 9 : 72);
    P->w[p] = ratio(wn[p], wd[p]);
    for (int a = 0; a < 3; ++a) {
      P->ci[p][a] = kC[p][a];
      P->xi[p][a] = kC[p][a];
      for (int b = 0; b < 3; ++b) P->Q[p][a][b] = ratio(3 * kC[p][a] * kC[p][b] - (a == b), 3);
    }
    for (int q = 0; q < 15; ++q)
      if (kC[q][0] == -kC[p][0] && kC[q][1] == -kC[p][1] && kC[q][2] == -kC[p][2])
        P->complement[p] = q;
  }
  for (int m = 0; m < 15; ++m) {
    long sn = 0, sd = 1;  // sum_p w_p mm[m][p]^2
    for (int p = 0; p < 15; ++p) {
      long mn, md;
      mode_rational(m, kC[p], mn, md);
      const long tn = wn[p] * mn * mn, td = wd[p] * md * md;
      const long nn = sn * td + tn * sd, nd = sd * td, g = gcd_l(nn, nd);
      sn = nn / g;
      sd = nd / g;
    }
    P->norms[m] = ratio(sd, sn);
    for (int p = 0; p < 15; ++p) {
      long mn, md;
      mode_rational(m, kC[p], mn, md);
      P->mm[m][p] = ratio(mn, md);
      P->mmi[p][m] = mn == 0 ? 0.0 : ratio(wn[p] * mn * sd, wd[p] * md * sn);
    }
  }
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ void load_force(const T* F, long long N, long long s, T& fx, T& fy,
                                           T& fz) {
  if (F) {
    fx = F[s];
    fy = F[N + s];
    fz = F[2 * N + s];
  } else {
    fx = fy = fz = T(0);
  }
}

// FP64 collide + push-stream, lb.cu:72-218.  blockDim = (32, 8); grid.z = x.
__global__ void __launch_bounds__(256) k_step_push_f64(const double* __restrict__ f,
                                                       const double* __restrict__ F,
                                                       double* __restrict__ fn, int nx, int ny,
                                                       int nz, long long N, Relax<double> k) {
  const int z = blockIdx.x * 32 + threadIdx.x;
  const int y = blockIdx.y * 8 + threadIdx.y;
  const int x = blockIdx.z;
  if (z >= nz || y >= ny) return;
  const long long nynz = (long long)ny * nz;
  const long long s = x * nynz + (long long)y * nz + z;
  double d[15];
#pragma unroll
  for (int p = 0; p < 15; ++p) d[p] = f[p * N + s];
  double fx, fy, fz;
  load_force(F, N, s, fx, fy, fz);
  collide(d, fx, fy, fz, 0.0, k, d);
  const int xm = wrap_once(x - 1, nx), xp = wrap_once(x + 1, nx);
  const int ym = wrap_once(y - 1, ny), yp = wrap_once(y + 1, ny);
  const int zm = wrap_once(z - 1, nz), zp = wrap_once(z + 1, nz);
#pragma unroll
  for (int p = 0; p < 15; ++p) {
    const int dx = cx_of(p), dy = cy_of(p), dz = cz_of(p);
    const long long X = dx > 0 ? xp : (dx < 0 ? xm : x);
    const long long Y = dy > 0 ? yp : (dy < 0 ? ym : y);
    const long long Z = dz > 0 ? zp : (dz < 0 ? zm : z);
    fn[p * N + X * nynz + Y * nz + Z] = d[p];
  }
}

// rho, u from the stored distributions and the force, lb.cu:250-295.
template <class S, class H>
__global__ void k_calc_hydro(const S* __restrict__ f, const H* __restrict__ F, H* __restrict__ rho,
                             H* __restrict__ u, long long N, H rho0, unsigned* status) {
  using T = H;
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < N;
       s += (long long)gridDim.x * blockDim.x) {
    T d[15];
#pragma unroll
    for (int p = 0; p < 15; ++p) d[p] = dev_from_stored<S>((T)Store<S>::ld(f + fidx<S>(p, s, N)), p);
    T R, jx, jy, jz;
    hydro_moments(d, R, jx, jy, jz);
    T fx, fy, fz;
    load_force(F, N, s, fx, fy, fz);
    const T r = rho0 + R;
    // one division per site (GB300's FP64 pipe is narrow; within an ulp of
    // the reference's three, lb.cu:286-293)
    const T inv = T(1) / r;
    rho[s] = r;
    u[s] = (jx + T(0.5) * fx) * inv;
    u[N + s] = (jy + T(0.5) * fy) * inv;
    u[2 * N + s] = (jz + T(0.5) * fz) * inv;
    if (!finite_d((double)(r + jx + jy + jz))) raise_status(status, LBSWIM_STATUS_NONFINITE);
  }
}

// Equilibrium from rho, u, lb.cu:314-371 (compat_sxz reproduces lb.cu:356),
// FP64 lattices: rho, u from the FP64 SoA fields.
__global__ void k_init_from_hydro(const double* __restrict__ rho, const double* __restrict__ u,
                                  double* __restrict__ f, long long N, int compat_sxz) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < N;
       s += (long long)gridDim.x * blockDim.x) {
    const double r = rho[s], ux = u[s], uy = u[N + s], uz = u[2 * N + s];
    double out[15];
    project<double>(r, r * ux, r * uy, r * uz, r * ux * ux, r * uy * uy, r * uz * uz,
                    r * ux * uy, compat_sxz ? r * ux * uy : r * ux * uz, r * uy * uz, out);
#pragma unroll
    for (int p = 0; p < 15; ++p) f[fidx<double>(p, s, N)] = out[p];
  }
}

// The same for FP32/BF16/FP16 lattices, in FP32 (the stored deviations carry
// FP32 precision or less, so FP64 arithmetic would buy nothing): rho, u from
// the packed float4 fields, whose w holds rho - rho_w; it is rewritten as
// R = rho - rho0 for the new reference density, R = w + (rho_w - rho0).
template <class S>
__global__ void k_init_from_hydro_packed(float4* __restrict__ packed, S* __restrict__ f,
                                         long long N, float drho, float rho0, int compat_sxz) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < N;
       s += (long long)gridDim.x * blockDim.x) {
    const float4 h = packed[s];
    const float R = h.w + drho;
    packed[s].w = R;
    const float r = rho0 + R, ux = h.x, uy = h.y, uz = h.z;
    const float jx = r * ux, jy = r * uy, jz = r * uz;
    float out[15];
    project<float>(R, jx, jy, jz, jx * ux, jy * uy, jz * uz, jx * uy,
                   compat_sxz ? jx * uy : jx * uz, jy * uz, out);
#pragma unroll
    for (int p = 0; p < 15; ++p) Store<S>::st(f + fidx<S>(p, s, N), stored_from_dev<S>(out[p], p));
  }
}

// rho, u from the stored distributions and the force into the packed fields
// (CalcHydro of a reduced-precision lattice when the step's result is stale).
template <class S>
__global__ void k_calc_hydro_packed(const S* __restrict__ f, const float* __restrict__ F,
                                    float4* __restrict__ hydro, long long N, float rho0,
                                    unsigned* status) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < N;
       s += (long long)gridDim.x * blockDim.x) {
    float d[15];
#pragma unroll
    for (int p = 0; p < 15; ++p) d[p] = dev_from_stored<S>((float)Store<S>::ld(f + fidx<S>(p, s, N)), p);
    float R, jx, jy, jz;
    hydro_moments(d, R, jx, jy, jz);
    float fx, fy, fz;
    load_force(F, N, s, fx, fy, fz);
    const float inv = 1.0f / (rho0 + R);
    hydro[s] = make_float4((jx + 0.5f * fx) * inv, (jy + 0.5f * fy) * inv, (jz + 0.5f * fz) * inv, R);
    if (!finite_f(R + jx + jy + jz)) raise_status(status, LBSWIM_STATUS_NONFINITE);
  }
}

// Host FP64 [components][N] <-> packed float4 component c (0-2: u, 3: rho,
// held as rho - rho0 so that its float keeps the density's fluctuation).
__global__ void k_packed_from_f64(const double* __restrict__ src, float* __restrict__ packed,
                                  long long off, long long cnt, long long N, int rho_field,
                                  double rho0) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cnt;
       i += (long long)gridDim.x * blockDim.x) {
    const long long e = off + i;
    const int c = rho_field ? 3 : (int)(e / N);
    packed[4 * (e % N) + c] = (float)(rho_field ? src[i] - rho0 : src[i]);
  }
}
__global__ void k_packed_to_f64(const float* __restrict__ packed, double* __restrict__ dst,
                                long long off, long long cnt, long long N, int rho_field,
                                double rho0) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cnt;
       i += (long long)gridDim.x * blockDim.x) {
    const long long e = off + i;
    const int c = rho_field ? 3 : (int)(e / N);
    const double v = (double)packed[4 * (e % N) + c];
    dst[i] = rho_field ? v + rho0 : v;
  }
}

// The same conversions one site per thread, for a page-locked host buffer that
// the kernel reads or writes itself (no staging copy): rho as rho - rho0 in
// .w, u's three components [3][N] into .xyz.
__global__ void k_rho_from_host(const double* __restrict__ src, float4* __restrict__ packed,
                                long long N, double rho0) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x)
    packed[i].w = (float)(src[i] - rho0);
}
__global__ void k_u_from_host(const double* __restrict__ src, float4* __restrict__ packed,
                              long long N) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    float4 p = packed[i];
    p.x = (float)src[i];
    p.y = (float)src[N + i];
    p.z = (float)src[2 * N + i];
    packed[i] = p;
  }
}
__global__ void k_rho_to_host(const float4* __restrict__ packed, double* __restrict__ dst,
                              long long N, double rho0) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x)
    dst[i] = (double)packed[i].w + rho0;
}
__global__ void k_u_to_host(const float4* __restrict__ packed, double* __restrict__ dst,
                            long long N) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    const float4 p = packed[i];
    dst[i] = p.x;
    dst[N + i] = p.y;
    dst[2 * N + i] = p.z;
  }
}

// Host FP64 <-> device storage conversions for H2D / D2H of fOld and fNew:
// host element e of the reference's [15][N] order is population e / N at site
// e % N, stored at fidx.
template <class S>
__global__ void k_f_from_f64(const double* __restrict__ src, S* __restrict__ dst, long long off,
                             long long cnt, long long N, double rho0) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cnt;
       i += (long long)gridDim.x * blockDim.x) {
    const long long e = off + i;
    const int p = (int)(e / N);
    const double d = src[i] - w_of(p) * rho0;
    Store<S>::st(dst + fidx<S>(p, e - p * N, N), (S)stored_from_dev<S>(d, p));
  }
}
template <class S>
__global__ void k_f_to_f64(const S* __restrict__ src, double* __restrict__ dst, long long off,
                           long long cnt, long long N, double rho0) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cnt;
       i += (long long)gridDim.x * blockDim.x) {
    const long long e = off + i;
    const int p = (int)(e / N);
    dst[i] = dev_from_stored<S>((double)Store<S>::ld(src + fidx<S>(p, e - p * N, N)), p) +
             w_of(p) * rho0;
  }
}
__global__ void k_f64_to_f32(const double* __restrict__ src, float* __restrict__ dst, long long cnt) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cnt;
       i += (long long)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}
__global__ void k_f32_to_f64(const float* __restrict__ src, double* __restrict__ dst, long long cnt) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cnt;
       i += (long long)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}

// ---------------------------------------------------------------------------
// Fused collide + stream + hydro kernel (FP32 arithmetic).
//
// A CTA owns a TY x TZ cross-section (y, z) of FUSED_LX consecutive x planes
// and marches along x.  For each plane it collides the cross-section plus a
// one-site ring (TY*TZ interior threads + up to 96 ring threads) and parks
// the post-collision values in a ring buffer of shared memory.  Once the
// planes x-1, x, x+1 are in the ring, each interior thread pulls its 15
// post-stream populations for plane x, computes rho and u with the same force
// used in the collision (lb.cu:286-293) and writes f(t+1), rho, u.  The three
// populations that move only along x (0, 1, 2) come from the thread's own
// collisions of the planes x, x-1, x+1 and stay in registers.  The next
// plane's loads are issued before the current plane is collided.
// ---------------------------------------------------------------------------
constexpr int FUSED_LX = SLAB_LX;
constexpr int FUSED_RING_THREADS = 96;

struct FusedArgs {
  const void* f_old;
  void* f_new;
  const float* force;  // dense force base; null: zero
  float4* hydro;  // {ux, uy, uz, rho} per site
  int nx, ny, nz;
  long long n;
  float rho0;
  Relax<float> k;
  SlabEnds spread;  // pending dipole ends spread by the kernel itself (SPREAD instances)
  unsigned* status;  // sticky error bits of the lattice (LBSWIM_STATUS_*)
};

// Post-collision populations 3-14 wait in shared memory until the output plane
// can pull them: those moving +x (7-10) are read two planes later, those at
// rest in x (3-6) one plane later, those moving -x (11-14) in the same plane.
// With one barrier per plane that needs 4, 3 and 2 slots of 4 populations; the
// SPREAD instances take a second barrier per plane and need 3, 2 and 1, which
// leaves room in shared memory for the spreading without shrinking the L1
// cache that holds the loads in flight (two CTAs of either kind fit a 132 KB
// carveout).
__host__ __device__ constexpr int ring_group(int p) { return cx_of(p) > 0 ? 0 : (cx_of(p) == 0 ? 1 : 2); }
__host__ __device__ constexpr int ring_index(int p) { return p <= 6 ? p - 3 : (p <= 10 ? p - 7 : p - 11); }
constexpr int RING_POPS = 4;
template <bool SPREAD>
__host__ __device__ constexpr int ring_slots(int group) {
  return SPREAD ? 3 - group : 4 - group;
}
template <bool SPREAD>
__host__ __device__ constexpr int ring_pop_planes() {
  return RING_POPS * (ring_slots<SPREAD>(0) + ring_slots<SPREAD>(1) + ring_slots<SPREAD>(2));
}

template <int TZ, int TY>
constexpr int spread_base() {
  return align16(ring_pop_planes<true>() * (TY + 2) * (TZ + 2) * (int)sizeof(float));
}

template <int TZ, int TY, bool SPREAD>
constexpr int fused_smem_bytes() {
  return SPREAD ? SpreadLayout<TZ, TY, 1, spread_base<TZ, TY>()>::total
                : ring_pop_planes<false>() * (TY + 2) * (TZ + 2) * (int)sizeof(float);
}

// Bulk-copy staging of the distributions (TMA instances, TZ = 32 and nz a
// multiple of 32): the rows y0 - 1 .. y0 + TY of a plane are TY + 2 blocks of
// 32 sites, each one contiguous run [15][32] of the blocked layout, copied by
// one cp.async.bulk into a stage buffer; two stages, so that the next plane
// lands while the current one is collided.  The sites just outside the
// cross-section in z (z0 - 1 and z0 + 32) lie in other blocks and are still
// loaded by their ring threads.
constexpr int TMA_STAGES = 2;
template <class S, int TY>
constexpr int tma_row_bytes() { return 15 * 32 * (int)sizeof(S); }
template <class S, int TY>
constexpr int tma_stage_bytes() { return (TY + 2) * tma_row_bytes<S, TY>(); }
template <class S, int TZ, int TY, bool SPREAD>
constexpr int tma_stage_offset() { return (fused_smem_bytes<TZ, TY, SPREAD>() + 127) & ~127; }
template <class S, int TZ, int TY, bool SPREAD>
constexpr int tma_bar_offset() {
  return tma_stage_offset<S, TZ, TY, SPREAD>() + TMA_STAGES * tma_stage_bytes<S, TY>();
}
template <class S, int TZ, int TY, bool SPREAD, bool TMA>
constexpr int fused_smem_total() {
  return TMA ? tma_bar_offset<S, TZ, TY, SPREAD>() + 8 * TMA_STAGES
             : fused_smem_bytes<TZ, TY, SPREAD>();
}
// two CTAs of the bulk-copy instances fit an SM's 228 KB (1 KB reserved each)
static_assert(2 * (fused_smem_total<float, 32, 8, true, true>() + 1024) <= 228 * 1024,
              "bulk-copy slab smem");
// two CTAs per SM (1 KB of each CTA's shared memory is reserved) within 132 KB
static_assert(2 * (fused_smem_bytes<32, 8, true>() + 1024) <= 132 * 1024, "SPREAD slab smem");
static_assert(2 * (fused_smem_bytes<16, 16, true>() + 1024) <= 132 * 1024, "SPREAD slab smem");

// One slab: tile (tz, ty, tx) of the lattice in units of (TZ, TY, FUSED_LX)
// sites; `slab` indexes its bucket of pending ends.  Called by one CTA.
// I is the site-index type: int when 15 N fits it (one multiply-add per
// address), long long otherwise.
// SPLIT: the form of the slab's force sums (slab_sums_split); SPREAD only.
// TMA: the distributions of the cross-section's rows arrive by bulk copies
// into shared memory (tma_* above); the lattice has nz a multiple of 32.
template <class S, int TZ, int TY, bool SPREAD, class I, bool SPLIT, bool TMA = false>
__device__ __forceinline__ void fused_slab(const FusedArgs& a, int tz, int ty, int tx, int slab) {
  static_assert(sizeof(S) < 8, "the fused step serves the reduced-precision layouts");
  static_assert(!TMA || TZ == 32, "bulk-copied rows are whole 32-site blocks");
  constexpr int NI = TY * TZ;
  constexpr int HZ = TZ + 2, HY = TY + 2, PLANE = HY * HZ;
  constexpr int NA = ring_slots<SPREAD>(0), NB = ring_slots<SPREAD>(1);
  extern __shared__ __align__(16) unsigned char smraw[];
  constexpr int RP = RING_POPS;
  float* ringA = reinterpret_cast<float*>(smraw);  // [NA][RP][PLANE]
  float* ringB = ringA + NA * RP * PLANE;          // [NB][RP][PLANE]
  float* ringC = ringB + NB * RP * PLANE;          // [NC][RP][PLANE]
  const int tid = threadIdx.x;
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const int z0 = tz * TZ, y0 = ty * TY, x0 = tx * FUSED_LX;
  const int ez = min(TZ, nz - z0), ey = min(TY, ny - y0), ex = min(FUSED_LX, nx - x0);

  int ly = 0, lz = 0;
  bool active = false, interior = false;
  if (tid < NI) {
    ly = tid / TZ + 1;
    lz = tid % TZ + 1;
    interior = active = (ly <= ey) && (lz <= ez);
  } else {
    int h = tid - NI;
    const int rowN = ez + 2;
    if (h < 2 * rowN) {
      ly = h < rowN ? 0 : ey + 1;
      lz = h < rowN ? h : h - rowN;
      active = true;
    } else {
      h -= 2 * rowN;
      if (h < 2 * ey) {
        ly = 1 + (h >> 1);
        lz = (h & 1) ? ez + 1 : 0;
        active = true;
      }
    }
  }
  const int gy = wrap_once(y0 + ly - 1, ny), gz = wrap_once(z0 + lz - 1, nz);
  const I nynz = (I)ny * nz, N = (I)a.n;
  const I yz = (I)gy * nz + gz;
  const S* __restrict__ fo = (const S*)a.f_old;
  const float* __restrict__ F = a.force;
  const int my = ly * HZ + lz;
  // TMA: this thread's site is in a bulk-copied row (all but the z halo)
  const bool staged = TMA && active && lz >= 1 && lz <= ez;
  S* stage = TMA ? reinterpret_cast<S*>(smraw + tma_stage_offset<S, TZ, TY, SPREAD>()) : nullptr;
  uint64_t* bars =
      TMA ? reinterpret_cast<uint64_t*>(smraw + tma_bar_offset<S, TZ, TY, SPREAD>()) : nullptr;
  const int nrows = ey + 2;
  // Thread 0 arms the stage's barrier and copies the rows of local plane k
  // (x = x0 - 1 + k) into it.
  auto issue = [&](int k) {
    if constexpr (TMA) {
      const int st = k & (TMA_STAGES - 1);
      const int gx = wrap_once(x0 - 1 + k, nx);
      constexpr uint32_t rb = tma_row_bytes<S, TY>();
      mbar_arrive_expect_tx(bars + st, rb * (uint32_t)nrows);
      const long long nzb = nz >> 5;
      for (int r = 0; r < nrows; ++r) {
        const int gyr = wrap_once(y0 + r - 1, ny);
        const long long blk = ((long long)gx * ny + gyr) * nzb + tz;
        bulk_g2s(stage + (size_t)(st * (TY + 2) + r) * (15 * 32), fo + blk * (15 * 32), rb,
                 bars + st);
      }
    }
  };
  if constexpr (TMA) {
    if (tid == 0) {
      for (int st = 0; st < TMA_STAGES; ++st) mbar_init(bars + st, 1);
      mbar_init_fence();
    }
    __syncthreads();
    if (tid == 0) {
      issue(0);
      if (ex + 2 > 1) issue(1);
    }
  }

  // ---- this slab's pending dipole ends and the fixed-point force plane ----
  SlabSpreader<TZ, TY, 1, spread_base<TZ, TY>(), SPLIT> sp;
  // the ring threads, which write no output plane, take the first pairs
  const int rt = tid >= NI ? tid - NI : tid + (int)blockDim.x - NI;
  if (SPREAD) {
    sp.bind(smraw, a.spread, slab, nx, ny, nz, x0, y0, z0, ex, ey, ez);
    sp.prologue(tid, blockDim.x);
    sp.scatter(0, rt, blockDim.x);
    __syncthreads();
  }

  float pre[18];
  auto load = [&](int gx) {
    const I s = (I)gx * nynz + yz;
    if (!staged) {
      const S* __restrict__ b = fo + fidx<S, I>(0, s, N);
#pragma unroll
      for (int p = 0; p < 15; ++p) pre[p] = Store<S>::ld(b + p * 32);
    }
    if (F) {
      pre[15] = F[s];
      pre[16] = F[(N + s)];
      pre[17] = F[(2 * N + s)];
    } else {
      pre[15] = pre[16] = pre[17] = 0.f;
    }
  };
  if (active) load(wrap_once(x0 - 1, nx));

  float Fp0 = 0.f, Fp1 = 0.f, Fp2 = 0.f;
  float nonfinite = 0.f;  // stays 0 while every output density is finite
  // this site's post-collision populations 0 (plane k-1) and 1 (planes k-1, k-2)
  float keep0 = 0.f, keep1a = 0.f, keep1b = 0.f;
  int k3 = 0;  // k % 3
  for (int k = 0; k < ex + 2; ++k) {
    float cur[18];
#pragma unroll
    for (int i = 0; i < 18; ++i) cur[i] = pre[i];
    if (active && k + 1 < ex + 2) load(wrap_once(x0 + k, nx));
    if constexpr (TMA) {
      // this plane's rows have landed in stage k % 2
      const int st = k & (TMA_STAGES - 1);
      mbar_wait(bars + st, (uint32_t)(k / TMA_STAGES) & 1u, a.status, LBSWIM_STATUS_COPY_TIMEOUT);
      if (staged) {
        const S* row = stage + (size_t)(st * (TY + 2) + ly) * (15 * 32) + (lz - 1);
#pragma unroll
        for (int p = 0; p < 15; ++p) cur[p] = Store<S>::ld(row + p * 32);
      }
    }
    if (SPREAD && active) {
      // force = base + spread (k_force_slab writes the same bits)
#pragma unroll
      for (int c = 0; c < 3; ++c) cur[15 + c] += sp.take(my, c);
    }
    // ring slots: plane k is written to A[k % NA], B[k % NB], C[k % NC]
    const int wa_slot = SPREAD ? k3 : (k & 3);
    const int wb_slot = SPREAD ? (k & 1) : k3;
    const int wc_slot = SPREAD ? 0 : (k & 1);
    float new0 = 0.f, new1 = 0.f, new2 = 0.f;
    if (active) {
      float d[15];
#pragma unroll
      for (int p = 0; p < 15; ++p) d[p] = dev_from_stored<S>(cur[p], p);
      collide(d, cur[15], cur[16], cur[17], a.rho0, a.k, d);
      float* wa = ringA + wa_slot * RP * PLANE + my;
      float* wb = ringB + wb_slot * RP * PLANE + my;
      float* wc = ringC + wc_slot * RP * PLANE + my;
#pragma unroll
      for (int p = 3; p < 15; ++p) {
        float* w = ring_group(p) == 0 ? wa : (ring_group(p) == 1 ? wb : wc);
        w[ring_index(p) * PLANE] = d[p];
      }
      new0 = d[0];
      new1 = d[1];
      new2 = d[2];
    }
    __syncthreads();
    if constexpr (TMA) {
      // every thread has read stage k % 2: it takes plane k + 2
      if (tid == 0 && k + TMA_STAGES < ex + 2) {
        fence_proxy_async_smem();
        issue(k + TMA_STAGES);
      }
    }
    if (SPREAD && k + 1 < ex + 2) sp.scatter(k + 1, rt, blockDim.x);
    if (k >= 2 && interior) {
      // output plane x = x0 + k - 2 pulls A of plane x-1, B of x, C of x+1
      const int ra_slot = SPREAD ? (k3 == 2 ? 0 : k3 + 1) : ((k - 2) & 3);
      const int rb_slot = SPREAD ? ((k - 1) & 1) : (k3 == 0 ? 2 : k3 - 1);
      const int rc_slot = SPREAD ? 0 : (k & 1);
      const I s = (I)(x0 + k - 2) * nynz + yz;
      const float* ra = ringA + ra_slot * RP * PLANE + my;  // plane x-1: c_x = +1
      const float* rb = ringB + rb_slot * RP * PLANE + my;  // plane x
      const float* rc = ringC + rc_slot * RP * PLANE + my;  // plane x+1: c_x = -1
      float g[15];
      g[0] = keep0;   // plane x
      g[1] = keep1b;  // plane x-1
      g[2] = new2;    // plane x+1, collided just now
#pragma unroll
      for (int p = 3; p < 15; ++p) {
        const int off = ring_index(p) * PLANE - cy_of(p) * HZ - cz_of(p);
        g[p] = ring_group(p) == 0 ? ra[off] : (ring_group(p) == 1 ? rb[off] : rc[off]);
      }
      float R, jx, jy, jz;
      hydro_moments(g, R, jx, jy, jz);
      // 0 * R is 0 for a finite R and NaN otherwise; a non-finite population
      // makes R non-finite (it is their sum)
      nonfinite = __fmaf_rn(0.f, R, nonfinite);
      S* __restrict__ fn = (S*)a.f_new;
      S* __restrict__ bo = fn + fidx<S, I>(0, s, N);
#pragma unroll
      for (int p = 0; p < 15; ++p) Store<S>::st(bo + p * 32, stored_from_dev<S>(g[p], p));
      const float inv = 1.0f / (a.rho0 + R);
      a.hydro[s] = make_float4((jx + 0.5f * Fp0) * inv, (jy + 0.5f * Fp1) * inv,
                               (jz + 0.5f * Fp2) * inv, R);
    }
    // the next plane's collision overwrites the slots just read, and the
    // scatter must be complete before the owners read it
    if (SPREAD) __syncthreads();
    Fp0 = cur[15];
    Fp1 = cur[16];
    Fp2 = cur[17];
    keep0 = new0;
    keep1b = keep1a;
    keep1a = new1;
    k3 = k3 == 2 ? 0 : k3 + 1;
  }
  if (nonfinite != 0.f) raise_status(a.status, LBSWIM_STATUS_NONFINITE);
}

template <class S, int TZ, int TY, bool SPREAD, class I, bool TMA>
__global__ void __launch_bounds__(TY * TZ + FUSED_RING_THREADS, 2) k_fused_step(FusedArgs a) {
  const int slab = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
  if (!SPREAD || slab_sums_split(a.spread, slab, a.nx, a.ny, a.nz))
    fused_slab<S, TZ, TY, SPREAD, I, true, TMA>(a, blockIdx.x, blockIdx.y, blockIdx.z, slab);
  else
    fused_slab<S, TZ, TY, SPREAD, I, false, TMA>(a, blockIdx.x, blockIdx.y, blockIdx.z, slab);
}

// ---------------------------------------------------------------------------
// Batched step of an ensemble of FP32 lattices: one persistent launch takes the
// slabs of every member from a shared counter (both slab shapes are compiled
// in; a member's shape is its autotuned choice) and runs the step kernel's
// per-slab code on each, spreading the member's pending ends.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int ens_member_of(const int* __restrict__ prefix, int nmem, int item) {
  int lo = 0, hi = nmem - 1;  // last member whose first item is <= item
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= item)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

constexpr int ENS_STEP_SMEM =
    fused_smem_bytes<32, 8, true>() > fused_smem_bytes<16, 16, true>()
        ? fused_smem_bytes<32, 8, true>()
        : fused_smem_bytes<16, 16, true>();
static_assert(8 * 32 == 16 * 16, "both slab shapes use the same block");

__global__ void __launch_bounds__(8 * 32 + FUSED_RING_THREADS, 2) k_ens_step(EnsTable t, int parity) {
  __shared__ int s_tile;
  const int nmem = *t.nmem;
  const int total = t.tile_prefix[nmem];
  for (;;) {
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(&t.counters[parity], 1u);
    __syncthreads();
    const int tile = s_tile;
    __syncthreads();
    if (tile >= total) break;
    const int m = ens_member_of(t.tile_prefix, nmem, tile);
    const EnsMember& M = t.mem[m];
    if (*t.g_step >= M.limit) {  // the member has taken its steps of this run
      __syncthreads();
      continue;
    }
    const int lt = tile - t.tile_prefix[m];
    const int tz = lt % M.nt[2], ty = (lt / M.nt[2]) % M.nt[1], tx = lt / (M.nt[2] * M.nt[1]);
    FusedArgs a{};
    a.f_old = M.f[parity];
    a.f_new = M.f[parity ^ 1];
    a.force = nullptr;
    a.hydro = (float4*)M.hyd[parity];
    a.nx = M.size[0];
    a.ny = M.size[1];
    a.nz = M.size[2];
    a.n = M.n;
    a.rho0 = M.rho0;
    a.k = Relax<float>{M.omega_s, M.omega_b, M.force_s, M.force_b};
    a.spread = SlabEnds{(const EndRecord<float>*)M.ends, M.bucket_count, M.bucket_list,
                        2 * M.nsw, M.max_abs_f};
    a.status = M.status;
    // members have few enough swimmers for split force sums on every slab
    // (checked when the members are set)
    if (M.tile == 1)
      fused_slab<float, 16, 16, true, int, true>(a, tz, ty, tx, lt);
    else
      fused_slab<float, 32, 8, true, int, true>(a, tz, ty, tx, lt);
    __syncthreads();
  }
}

int ens_step_ctas_per_sm() { return 2; }

void ens_launch_step(const EnsTable& t, int parity, int grid, cudaStream_t s) {
  static bool configured = false;
  if (!configured) {
    LB_CUDA(cudaFuncSetAttribute(k_ens_step, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 ENS_STEP_SMEM));
    configured = true;
  }
  k_ens_step<<<grid, 8 * 32 + FUSED_RING_THREADS, ENS_STEP_SMEM, s>>>(t, parity);
  LB_CHECK_LAUNCH(1);
}

// ---------------------------------------------------------------------------
// Dense force of a reduced-precision lattice: base + the spread of the pending
// ends, slab by slab and plane by plane with the step kernel's spreading, so
// the bits are those the step kernel uses.  One thread per (y, z) site of the
// slab's cross-section writes the three components of its site on each plane.
// ---------------------------------------------------------------------------
template <int TZ, int TY, bool SPLIT>
__device__ __forceinline__ void force_slab(const SlabEnds& se, float* __restrict__ force, int nx,
                                           int ny, int nz, long long N, int accumulate,
                                           int slab) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int tid = threadIdx.x;
  const int z0 = blockIdx.x * TZ, y0 = blockIdx.y * TY, x0 = blockIdx.z * SLAB_LX;
  const int ez = min(TZ, nz - z0), ey = min(TY, ny - y0), ex = min(SLAB_LX, nx - x0);
  SlabSpreader<TZ, TY, 0, 0, SPLIT> sp;
  sp.bind(smraw, se, slab, nx, ny, nz, x0, y0, z0, ex, ey, ez);
  sp.prologue(tid, blockDim.x);
  const int ly = tid / TZ, lz = tid % TZ;
  const bool valid = ly < ey && lz < ez;
  const int my = ly * TZ + lz;
  const long long yz = (long long)(y0 + ly) * nz + (z0 + lz), nynz = (long long)ny * nz;
  for (int kk = 0; kk < ex; ++kk) {
    sp.scatter(kk, tid, blockDim.x);
    __syncthreads();
    if (valid) {
      const long long s = (long long)(x0 + kk) * nynz + yz;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float v = sp.take(my, c);
        force[c * N + s] = accumulate ? force[c * N + s] + v : v;
      }
    }
    __syncthreads();
  }
}

template <int TZ, int TY>
__global__ void __launch_bounds__(TY * TZ) k_force_slab(SlabEnds se, float* __restrict__ force,
                                                         int nx, int ny, int nz, long long N,
                                                         int accumulate) {
  const int slab = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
  if (slab_sums_split(se, slab, nx, ny, nz))
    force_slab<TZ, TY, true>(se, force, nx, ny, nz, N, accumulate, slab);
  else
    force_slab<TZ, TY, false>(se, force, nx, ny, nz, N, accumulate, slab);
}

template <int TZ, int TY>
static void force_slab_launch(Lattice* L, const SlabSpread& sp) {
  constexpr int smem = SpreadLayout<TZ, TY, 0, 0>::total;
  static bool configured = false;
  if (!configured) {
    LB_CUDA(cudaFuncSetAttribute(k_force_slab<TZ, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem));
    configured = true;
  }
  dim3 grid((L->size[2] + TZ - 1) / TZ, (L->size[1] + TY - 1) / TY,
            (L->size[0] + SLAB_LX - 1) / SLAB_LX);
  k_force_slab<TZ, TY><<<grid, TY * TZ, smem, L->stream>>>(
      SlabEnds{(const EndRecord<float>*)sp.ends, sp.count, sp.list, sp.npending, sp.max_abs_force},
      (float*)L->force, L->size[0], L->size[1], L->size[2], L->n, L->force_zero_pending ? 0 : 1);
  LB_CHECK_LAUNCH(1);
}

void lattice_force_from_slabs(Lattice* L) {
  const SlabSpread sp = spread_prepare_slabs(L);
  if (L->fused_tile == 1)
    force_slab_launch<16, 16>(L, sp);
  else
    force_slab_launch<32, 8>(L, sp);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static int grid_for(long long n, int block) {
  long long g = (n + block - 1) / block;
  return (int)std::max(1LL, std::min(g, 152LL * 16));
}

static void* dmalloc(size_t bytes) {
  void* p = nullptr;
  LB_CUDA(cudaMalloc(&p, bytes ? bytes : 16));
  return p;
}

void lattice_alloc(Lattice* L) {
  const long long N = L->n;
  const size_t fe = elem_bytes(L->precision);
  const size_t he = L->precision == LBSWIM_F64 ? 8 : 4;
  const size_t fbytes = 15 * f_sites(N, L->precision) * fe;
  L->f[0] = dmalloc(fbytes);
  L->f[1] = dmalloc(fbytes);
  if (L->precision == LBSWIM_F64) {
    L->rho = dmalloc(N * he);
    L->u = dmalloc(3 * N * he);
    LB_CUDA(cudaMemsetAsync(L->rho, 0, N * he, L->stream));
    LB_CUDA(cudaMemsetAsync(L->u, 0, 3 * N * he, L->stream));
  } else {
    L->hydro = (float4*)dmalloc(N * sizeof(float4));
    L->hydro_shadow = (float4*)dmalloc(N * sizeof(float4));
    LB_CUDA(cudaMemsetAsync(L->hydro, 0, N * sizeof(float4), L->stream));
  }
  L->force = dmalloc(3 * N * he);
  L->status = (unsigned*)dmalloc(256);
  LB_CUDA(cudaMemsetAsync(L->status, 0, 256, L->stream));
  // Contents start at zero so that reading a field before setting it is defined.
  LB_CUDA(cudaMemsetAsync(L->force, 0, 3 * N * he, L->stream));
  LB_CUDA(cudaMemsetAsync(L->f[0], 0, fbytes, L->stream));
  LB_CUDA(cudaMemsetAsync(L->f[1], 0, fbytes, L->stream));
}

void lattice_free(Lattice* L) {
  void* ptrs[] = {L->f[0], L->f[1], L->rho, L->u, L->hydro, L->hydro_shadow, L->force,
                  L->staging, L->status};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  spread_free(L->spread);
  for (auto& r : L->readers) cudaEventDestroy(r.second);
  for (cudaEvent_t e : L->reader_pool) cudaEventDestroy(e);
  if (L->hydro_ready) cudaEventDestroy(L->hydro_ready);
  for (auto& p : L->timed) {
    cudaEventDestroy(p.first);
    cudaEventDestroy(p.second);
  }
  for (auto& p : L->event_pool) {
    cudaEventDestroy(p.first);
    cudaEventDestroy(p.second);
  }
}

static double* staging(Lattice* L, size_t elems) {
  if (L->staging_elems < elems) {
    if (L->staging) {
      LB_CUDA(cudaStreamSynchronize(L->stream));
      LB_CUDA(cudaFree(L->staging));
      L->staging = nullptr;
      L->staging_elems = 0;
    }
    L->staging = (double*)dmalloc(elems * sizeof(double));
    L->staging_elems = elems;
  }
  return L->staging;
}

// Page-locked host memory (cudaMallocHost, cudaHostRegister, pinned tensors)
// is mapped into the device's address space, so a conversion kernel can read
// or write the caller's buffer itself over the host link: one pass, with no
// staging copy and no serialisation of copy and conversion.  Returns the
// buffer's device address, or null for pageable memory (which goes through
// the staging buffer).
static const void* mapped_host(const void* host) {
  cudaPointerAttributes at;
  int dev = -1;
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  // page-locked by this device's context (memory pinned under another
  // device takes the staging path)
  return at.type == cudaMemoryTypeHost && at.device == dev ? at.devicePointer : nullptr;
}

void lattice_zero_force_now(Lattice* L) {
  const size_t he = L->precision == LBSWIM_F64 ? 8 : 4;
  LB_CUDA(cudaMemsetAsync(L->force, 0, 3 * L->n * he, L->stream));
  L->force_zero_pending = false;
}

void lattice_materialise_force(Lattice* L) { spread_materialise(L); }

void lattice_zero_force(Lattice* L) {
  L->force_zero_pending = true;
  L->spread.pending = 0;
  L->spread.stepped = false;
  L->force_version++;
}

template <class S>
static void init_from_hydro_t(Lattice* L, double rho_w) {
  const long long N = L->n;
  const int compat = (L->compat & LBSWIM_COMPAT_INIT_SXZ) ? 1 : 0;
  if constexpr (sizeof(S) == 8)
    k_init_from_hydro<<<grid_for(N, 256), 256, 0, L->stream>>>(
        (const double*)L->rho, (const double*)L->u, (double*)L->f[L->cur], N, compat);
  else
    k_init_from_hydro_packed<S><<<grid_for(N, 256), 256, 0, L->stream>>>(
        L->hydro, (S*)L->f[L->cur], N, (float)(rho_w - L->rho0), (float)L->rho0, compat);
  LB_CHECK_LAUNCH(1);
}

// ---- FP64 sums over the lattice (mean density, mass, momentum) -------------
// Deterministic: every thread adds a fixed set of sites in order, blocks reduce
// in a fixed tree, and one thread adds the block sums in order.
constexpr int SUM_BLOCKS = 512, SUM_THREADS = 256;

template <class S>
__global__ void __launch_bounds__(SUM_THREADS) k_sums(const S* __restrict__ f,
                                                      const float4* __restrict__ hydro, long long N,
                                                      double rho0, double* __restrict__ part) {
  __shared__ double red[4][SUM_THREADS];
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  if (hydro) {
    // several loads in flight per thread; the adds keep their order
    const float* rw = reinterpret_cast<const float*>(hydro) + 3;
#pragma unroll 8
    for (long long s = blockIdx.x * (long long)SUM_THREADS + threadIdx.x; s < N;
         s += (long long)SUM_BLOCKS * SUM_THREADS)
      acc[0] += (double)__ldg(rw + 4 * s);
  } else {
    for (long long s = blockIdx.x * (long long)SUM_THREADS + threadIdx.x; s < N;
         s += (long long)SUM_BLOCKS * SUM_THREADS) {
      double m = 0.0, jx = 0.0, jy = 0.0, jz = 0.0;
#pragma unroll
      for (int p = 0; p < 15; ++p) {
        const double v =
            dev_from_stored<S>((double)Store<S>::ld(f + fidx<S>(p, s, N)), p) + w_of(p) * rho0;
        m += v;
        jx += cx_of(p) * v;
        jy += cy_of(p) * v;
        jz += cz_of(p) * v;
      }
      acc[0] += m;
      acc[1] += jx;
      acc[2] += jy;
      acc[3] += jz;
    }
  }
  for (int q = 0; q < 4; ++q) red[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int h = SUM_THREADS / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h)
      for (int q = 0; q < 4; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 4; ++q) part[blockIdx.x * 4 + q] = red[q][0];
}

// The block sums are staged in shared memory by the whole block; then one
// thread per quantity adds them in block order (a chain of 512 dependent adds
// that no longer waits on a global load each).
constexpr int SUM_FINAL_THREADS = 512;
__global__ void __launch_bounds__(SUM_FINAL_THREADS) k_sums_final(const double* __restrict__ part,
                                                                  double* __restrict__ out) {
  __shared__ double sp[SUM_BLOCKS * 4];
  for (int i = threadIdx.x; i < SUM_BLOCKS * 4; i += SUM_FINAL_THREADS) sp[i] = part[i];
  __syncthreads();
  if (threadIdx.x < 4) {
    double t = 0.0;
    for (int b = 0; b < SUM_BLOCKS; ++b) t += sp[b * 4 + threadIdx.x];
    out[threadIdx.x] = t;
  }
}

// out = {sum (rho - rho0), 0, 0, 0} from the packed velocity buffer, or
// {mass, momentum} from f.
template <class S>
static void sums_t(Lattice* L, bool from_hydro, double out[4]) {
  double* part = staging(L, SUM_BLOCKS * 4 + 4);
  k_sums<S><<<SUM_BLOCKS, SUM_THREADS, 0, L->stream>>>(
      (const S*)L->f[L->cur], from_hydro ? L->hydro : nullptr, L->n, L->rho0, part);
  k_sums_final<<<1, SUM_FINAL_THREADS, 0, L->stream>>>(part, part + SUM_BLOCKS * 4);
  LB_CHECK_LAUNCH(2);
  LB_CUDA(cudaMemcpyAsync(out, part + SUM_BLOCKS * 4, 4 * sizeof(double), cudaMemcpyDeviceToHost,
                          L->stream));
  LB_CUDA(cudaStreamSynchronize(L->stream));
}

void lattice_conservation(Lattice* L, double out[4]) {
  switch (L->precision) {
    case LBSWIM_F64: sums_t<double>(L, false, out); break;
    case LBSWIM_F32: sums_t<float>(L, false, out); break;
    case LBSWIM_BF16: sums_t<__nv_bfloat16>(L, false, out); break;
    default: sums_t<__half>(L, false, out); break;
  }
}

void lattice_init_from_hydro(Lattice* L) {
  double rho_w = 0.0;
  if (L->precision != LBSWIM_F64) {
    // store the distributions as deviations from w_p rho0 with rho0 the mean
    // density (as a float): the density part then averages out of them and
    // the stored values carry the flow
    double t[4];
    sums_t<float>(L, true, t);
    rho_w = L->rho0;  // reference of the packed densities just uploaded
    L->rho0 = (double)(float)(rho_w + t[0] / (double)L->n);
  }
  switch (L->precision) {
    case LBSWIM_F64:
      if (L->compat & LBSWIM_COMPAT_EXACT_F64)
        exact_init_from_hydro_f64(L);
      else
        init_from_hydro_t<double>(L, 0.0);
      break;
    case LBSWIM_F32: init_from_hydro_t<float>(L, rho_w); break;
    case LBSWIM_BF16: init_from_hydro_t<__nv_bfloat16>(L, rho_w); break;
    default: init_from_hydro_t<__half>(L, rho_w); break;
  }
  L->f_version++;
}

template <class S, int TZ, int TY, bool SPREAD, class I, bool TMA>
static void launch_fused_i(Lattice* L, const FusedArgs& a) {
  constexpr int smem = fused_smem_total<S, TZ, TY, SPREAD, TMA>();
  static bool configured = false;  // per template instance, per process
  if (!configured) {
    LB_CUDA(cudaFuncSetAttribute(k_fused_step<S, TZ, TY, SPREAD, I, TMA>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    // the bulk-copied rows bypass L1: give shared memory the whole carveout so
    // that two CTAs fit an SM
    if (TMA)
      LB_CUDA(cudaFuncSetAttribute(k_fused_step<S, TZ, TY, SPREAD, I, TMA>,
                                   cudaFuncAttributePreferredSharedMemoryCarveout,
                                   cudaSharedmemCarveoutMaxShared));
    configured = true;
  }
  dim3 grid((a.nz + TZ - 1) / TZ, (a.ny + TY - 1) / TY, (a.nx + FUSED_LX - 1) / FUSED_LX);
  k_fused_step<S, TZ, TY, SPREAD, I, TMA>
      <<<grid, TY * TZ + FUSED_RING_THREADS, smem, L->stream>>>(a);
  LB_CHECK_LAUNCH(1);
}

// 32-bit site indices while every offset of the 15 populations fits (the
// reduced-precision buffers hold 15 f_sites(n) values).
inline bool fits_int_index(long long n) { return 15 * ((n + 31) & ~31ll) < (1ll << 31); }

// Rows of whole 32-site blocks are bulk-copied (LBSWIM_COMPAT_BULK_COPY) when
// the cross-section is 32 sites wide and nz a multiple of 32 (each row of the
// slab is then one block).
inline bool fused_uses_tma(const Lattice* L, int TZ) {
  return TZ == 32 && (L->size[2] & 31) == 0 && (L->compat & LBSWIM_COMPAT_BULK_COPY);
}

template <class S, int TZ, int TY, bool SPREAD>
static void launch_fused(Lattice* L, const FusedArgs& a) {
  const bool wide = !fits_int_index(a.n) || (L->compat & LBSWIM_COMPAT_WIDE_INDEX);
  if constexpr (TZ == 32) {
    if (fused_uses_tma(L, TZ)) {
      if (wide)
        launch_fused_i<S, TZ, TY, SPREAD, long long, true>(L, a);
      else
        launch_fused_i<S, TZ, TY, SPREAD, int, true>(L, a);
      return;
    }
  }
  if (wide)
    launch_fused_i<S, TZ, TY, SPREAD, long long, false>(L, a);
  else
    launch_fused_i<S, TZ, TY, SPREAD, int, false>(L, a);
}

// Pending dipole ends are spread by the step kernel itself (true), or first
// into the dense force by k_force_slab (false); both give the same force bits.
constexpr bool STEP_SPREADS_IN_KERNEL = true;

template <class S, int TZ, int TY>
static void fused_step_tile(Lattice* L, FusedArgs& a) {
  if (L->spread.pending > 0 && STEP_SPREADS_IN_KERNEL) {
    const SlabSpread sp = spread_prepare_slabs(L);
    a.spread = SlabEnds{(const EndRecord<float>*)sp.ends, sp.count, sp.list, sp.npending,
                        sp.max_abs_force};
    launch_fused<S, TZ, TY, true>(L, a);
  } else {
    launch_fused<S, TZ, TY, false>(L, a);
  }
}

void slab_shape_of(int tile, int T[3]) {
  T[0] = FUSED_LX;
  T[1] = tile == 1 ? 16 : 8;
  T[2] = tile == 1 ? 16 : 32;
}
void fused_slab_shape(const Lattice* L, int T[3]) { slab_shape_of(L->fused_tile, T); }

template <class S>
static void fused_step_t(Lattice* L) {
  if (!STEP_SPREADS_IN_KERNEL && L->spread.pending > 0) spread_materialise(L);
  FusedArgs a{};
  a.f_old = L->f[L->cur];
  a.f_new = L->f[L->cur ^ 1];
  a.force = L->force_zero_pending ? nullptr : (const float*)L->force;
  a.hydro = L->hydro_shadow;
  a.nx = L->size[0];
  a.ny = L->size[1];
  a.nz = L->size[2];
  a.n = L->n;
  a.rho0 = (float)L->rho0;
  a.k = make_relax<float>(L->tau_s, L->tau_b);
  a.status = L->status;
  if (L->fused_tile == 1)
    fused_step_tile<S, 16, 16>(L, a);
  else
    fused_step_tile<S, 32, 8>(L, a);
}

static std::pair<cudaEvent_t, cudaEvent_t> timing_pair(Lattice* L) {
  if (!L->event_pool.empty()) {
    auto p = L->event_pool.back();
    L->event_pool.pop_back();
    return p;
  }
  std::pair<cudaEvent_t, cudaEvent_t> p;
  LB_CUDA(cudaEventCreate(&p.first));
  LB_CUDA(cudaEventCreate(&p.second));
  return p;
}

void lattice_read_timing(Lattice* L, double* total_ms, int* launches) {
  LB_CUDA(cudaStreamSynchronize(L->stream));
  double sum = 0.0;
  for (auto& p : L->timed) {
    float ms = 0.f;
    LB_CUDA(cudaEventElapsedTime(&ms, p.first, p.second));
    sum += ms;
    L->event_pool.push_back(p);
  }
  *total_ms = sum;
  *launches = (int)L->timed.size();
  L->timed.clear();
}

void lattice_wait_readers(Lattice* L, const void* buf) {
  for (size_t i = 0; i < L->readers.size();) {
    if (buf == nullptr || L->readers[i].first == buf) {
      LB_CUDA(cudaStreamWaitEvent(L->stream, L->readers[i].second, 0));
      L->reader_pool.push_back(L->readers[i].second);
      L->readers.erase(L->readers.begin() + i);
    } else {
      ++i;
    }
  }
}

void lattice_step(Lattice* L) {
  const int nx = L->size[0], ny = L->size[1], nz = L->size[2];
  // the step writes rho, u into the shadow buffer of reduced-precision lattices
  if (L->precision != LBSWIM_F64) lattice_wait_readers(L, L->hydro_shadow);
  std::pair<cudaEvent_t, cudaEvent_t> ev{nullptr, nullptr};
  if (L->timing) {
    ev = timing_pair(L);
    LB_CUDA(cudaEventRecord(ev.first, L->stream));
  }
  if (L->precision == LBSWIM_F64 && (L->compat & LBSWIM_COMPAT_EXACT_F64)) {
    exact_step_f64(L);
  } else if (L->precision == LBSWIM_F64) {
    dim3 grid((nz + 31) / 32, (ny + 7) / 8, nx);
    k_step_push_f64<<<grid, dim3(32, 8), 0, L->stream>>>(
        (const double*)L->f[L->cur], L->force_zero_pending ? nullptr : (const double*)L->force,
        (double*)L->f[L->cur ^ 1], nx, ny, nz, L->n, make_relax<double>(L->tau_s, L->tau_b));
    LB_CHECK_LAUNCH(1);
  } else {
    switch (L->precision) {
      case LBSWIM_F32: fused_step_t<float>(L); break;
      case LBSWIM_BF16: fused_step_t<__nv_bfloat16>(L); break;
      default: fused_step_t<__half>(L); break;
    }
  }
  if (L->timing) {
    LB_CUDA(cudaEventRecord(ev.second, L->stream));
    L->timed.push_back(ev);
  }
  if (L->precision != LBSWIM_F64 && L->spread.pending > 0) L->spread.stepped = true;
  L->cur ^= 1;
  L->f_version++;
  if (L->precision != LBSWIM_F64) {
    L->shadow_f_version = L->f_version;
    L->shadow_force_version = L->force_version;
  }
  L->time_step++;
  if (L->compat & LBSWIM_COMPAT_SYNC_STEP) LB_CUDA(cudaStreamSynchronize(L->stream));
}

template <class S>
static void calc_hydro_t(Lattice* L) {
  const long long N = L->n;
  if (L->precision == LBSWIM_F64)
    k_calc_hydro<double, double><<<grid_for(N, 256), 256, 0, L->stream>>>(
        (const double*)L->f[L->cur], L->force_zero_pending ? nullptr : (const double*)L->force,
        (double*)L->rho, (double*)L->u, N, 0.0, L->status);
  else
    k_calc_hydro_packed<S><<<grid_for(N, 256), 256, 0, L->stream>>>(
        (const S*)L->f[L->cur], L->force_zero_pending ? nullptr : (const float*)L->force,
        L->hydro, N, (float)L->rho0, L->status);
  LB_CHECK_LAUNCH(1);
}

void lattice_calc_hydro(Lattice* L) {
  if (L->precision != LBSWIM_F64 && L->shadow_f_version == L->f_version &&
      L->shadow_force_version == L->force_version) {
    // The last Step already produced rho, u for this fOld and this force.
    std::swap(L->hydro, L->hydro_shadow);
    L->shadow_f_version = 0;
    return;
  }
  lattice_materialise_force(L);
  lattice_wait_readers(L, L->precision == LBSWIM_F64 ? nullptr : (const void*)L->hydro);
  switch (L->precision) {
    case LBSWIM_F64:
      if (L->compat & LBSWIM_COMPAT_EXACT_F64)
        exact_calc_hydro_f64(L);
      else
        calc_hydro_t<double>(L);
      break;
    case LBSWIM_F32: calc_hydro_t<float>(L); break;
    case LBSWIM_BF16: calc_hydro_t<__nv_bfloat16>(L); break;
    default: calc_hydro_t<__half>(L); break;
  }
}

static long long field_count(const Lattice* L, int field) {
  static const int mult[5] = {1, 3, 3, 15, 15};
  return mult[field] * L->n;
}

template <class S>
static void f_h2d_t(Lattice* L, void* dst, const double* host) {
  const long long total = 15 * L->n;
  if (const double* mh = (const double*)mapped_host(host)) {
    k_f_from_f64<S><<<grid_for(total, 256), 256, 0, L->stream>>>(mh, (S*)dst, 0, total, L->n,
                                                                  L->rho0);
    LB_CHECK_LAUNCH(1);
    return;
  }
  const long long chunk = std::min<long long>(total, 1LL << 24);
  double* st = staging(L, chunk);
  for (long long off = 0; off < total; off += chunk) {
    const long long cnt = std::min(chunk, total - off);
    LB_CUDA(cudaMemcpyAsync(st, host + off, cnt * sizeof(double), cudaMemcpyHostToDevice,
                            L->stream));
    k_f_from_f64<S><<<grid_for(cnt, 256), 256, 0, L->stream>>>(st, (S*)dst, off, cnt, L->n,
                                                                L->rho0);
    LB_CHECK_LAUNCH(1);
  }
}

template <class S>
static void f_d2h_t(Lattice* L, const void* src, double* host) {
  const long long total = 15 * L->n;
  if (double* mh = (double*)mapped_host(host)) {
    k_f_to_f64<S><<<grid_for(total, 256), 256, 0, L->stream>>>((const S*)src, mh, 0, total,
                                                                L->n, L->rho0);
    LB_CHECK_LAUNCH(1);
    LB_CUDA(cudaStreamSynchronize(L->stream));
    return;
  }
  const long long chunk = std::min<long long>(total, 1LL << 24);
  double* st = staging(L, chunk);
  for (long long off = 0; off < total; off += chunk) {
    const long long cnt = std::min(chunk, total - off);
    k_f_to_f64<S><<<grid_for(cnt, 256), 256, 0, L->stream>>>((const S*)src, st, off, cnt, L->n,
                                                              L->rho0);
    LB_CHECK_LAUNCH(1);
    LB_CUDA(cudaMemcpyAsync(host + off, st, cnt * sizeof(double), cudaMemcpyDeviceToHost,
                            L->stream));
    LB_CUDA(cudaStreamSynchronize(L->stream));
  }
}

static void* field_ptr(Lattice* L, int field) {
  switch (field) {
    case LBSWIM_FIELD_RHO: return L->precision == LBSWIM_F64 ? L->rho : (void*)L->hydro;
    case LBSWIM_FIELD_U: return L->precision == LBSWIM_F64 ? L->u : (void*)L->hydro;
    case LBSWIM_FIELD_FORCE: return L->force;
    case LBSWIM_FIELD_FOLD: return L->f[L->cur];
    default: return L->f[L->cur ^ 1];
  }
}

void lattice_h2d(Lattice* L, int field, const double* host) {
  const long long cnt = field_count(L, field);
  void* dst = field_ptr(L, field);
  if (field == LBSWIM_FIELD_FORCE) {
    L->force_zero_pending = false;
    L->spread.pending = 0;
    L->spread.stepped = false;
    L->force_version++;
  }
  if (field == LBSWIM_FIELD_FOLD) L->f_version++;
  if (L->precision == LBSWIM_F64) {
    LB_CUDA(cudaMemcpyAsync(dst, host, cnt * sizeof(double), cudaMemcpyHostToDevice, L->stream));
    LB_CUDA(cudaStreamSynchronize(L->stream));
    return;
  }
  if (field == LBSWIM_FIELD_FOLD || field == LBSWIM_FIELD_FNEW) {
    switch (L->precision) {
      case LBSWIM_F32: f_h2d_t<float>(L, dst, host); break;
      case LBSWIM_BF16: f_h2d_t<__nv_bfloat16>(L, dst, host); break;
      default: f_h2d_t<__half>(L, dst, host); break;
    }
  } else if (const double* mh = (const double*)mapped_host(host)) {
    const long long N = L->n;
    if (field == LBSWIM_FIELD_FORCE)
      k_f64_to_f32<<<grid_for(cnt, 256), 256, 0, L->stream>>>(mh, (float*)dst, cnt);
    else if (field == LBSWIM_FIELD_RHO)
      k_rho_from_host<<<grid_for(N, 256), 256, 0, L->stream>>>(mh, L->hydro, N, L->rho0);
    else
      k_u_from_host<<<grid_for(N, 256), 256, 0, L->stream>>>(mh, L->hydro, N);
    LB_CHECK_LAUNCH(1);
  } else {
    const long long chunk = std::min<long long>(cnt, 1LL << 24);
    double* st = staging(L, chunk);
    for (long long off = 0; off < cnt; off += chunk) {
      const long long c = std::min(chunk, cnt - off);
      LB_CUDA(cudaMemcpyAsync(st, host + off, c * sizeof(double), cudaMemcpyHostToDevice,
                              L->stream));
      if (field == LBSWIM_FIELD_FORCE)
        k_f64_to_f32<<<grid_for(c, 256), 256, 0, L->stream>>>(st, (float*)dst + off, c);
      else
        k_packed_from_f64<<<grid_for(c, 256), 256, 0, L->stream>>>(
            st, (float*)L->hydro, off, c, L->n, field == LBSWIM_FIELD_RHO, L->rho0);
      LB_CHECK_LAUNCH(1);
    }
  }
  LB_CUDA(cudaStreamSynchronize(L->stream));
}

void lattice_d2h(Lattice* L, int field, double* host) {
  if (field == LBSWIM_FIELD_FORCE) lattice_materialise_force(L);
  const long long cnt = field_count(L, field);
  const void* src = field_ptr(L, field);
  if (L->precision == LBSWIM_F64) {
    LB_CUDA(cudaMemcpyAsync(host, src, cnt * sizeof(double), cudaMemcpyDeviceToHost, L->stream));
    LB_CUDA(cudaStreamSynchronize(L->stream));
    return;
  }
  if (field == LBSWIM_FIELD_FOLD || field == LBSWIM_FIELD_FNEW) {
    switch (L->precision) {
      case LBSWIM_F32: f_d2h_t<float>(L, src, host); break;
      case LBSWIM_BF16: f_d2h_t<__nv_bfloat16>(L, src, host); break;
      default: f_d2h_t<__half>(L, src, host); break;
    }
    return;
  }
  if (double* mh = (double*)mapped_host(host)) {
    const long long N = L->n;
    if (field == LBSWIM_FIELD_FORCE)
      k_f32_to_f64<<<grid_for(cnt, 256), 256, 0, L->stream>>>((const float*)src, mh, cnt);
    else if (field == LBSWIM_FIELD_RHO)
      k_rho_to_host<<<grid_for(N, 256), 256, 0, L->stream>>>(L->hydro, mh, N, L->rho0);
    else
      k_u_to_host<<<grid_for(N, 256), 256, 0, L->stream>>>(L->hydro, mh, N);
    LB_CHECK_LAUNCH(1);
    LB_CUDA(cudaStreamSynchronize(L->stream));
    return;
  }
  const long long chunk = std::min<long long>(cnt, 1LL << 24);
  double* st = staging(L, chunk);
  for (long long off = 0; off < cnt; off += chunk) {
    const long long c = std::min(chunk, cnt - off);
    if (field == LBSWIM_FIELD_FORCE)
      k_f32_to_f64<<<grid_for(c, 256), 256, 0, L->stream>>>((const float*)src + off, st, c);
    else
      k_packed_to_f64<<<grid_for(c, 256), 256, 0, L->stream>>>(
          (const float*)L->hydro, st, off, c, L->n, field == LBSWIM_FIELD_RHO, L->rho0);
    LB_CHECK_LAUNCH(1);
    LB_CUDA(cudaMemcpyAsync(host + off, st, c * sizeof(double), cudaMemcpyDeviceToHost,
                            L->stream));
    LB_CUDA(cudaStreamSynchronize(L->stream));
  }
}

}  // namespace lbswim
