// exact_f64.cu -- FP64 Step, CalcHydro and InitFromHydro in the reference's
// operation order (LBSWIM_COMPAT_EXACT_F64).
//
// The reference transforms the 15 distributions to modes and back with dense
// 15x15 products (lb.cu:72-218) and reads rho, u from the first four modes
// (lb.cu:250-295); InitFromHydro projects the equilibrium modes (lb.cu:314-371).
// These kernels perform the same operations in the same order, each rounded on
// its own (__dadd_rn / __dmul_rn / __ddiv_rn never fuse), with the tables of
// the lattice's LBParams in constant memory, so an FP64 lattice reproduces the
// reference's host build bit for bit.
#include <cuda_runtime.h>

#include <mutex>

#include "lbswim_device.cuh"
#include "lbswim_internal.h"

namespace lbswim {

__constant__ double c_mm[15][15];
__constant__ double c_mmi[15][15];

static void upload_tables(const lbswim_lbparams& P) {
  // the tables do not depend on tau: one upload per device
  static std::mutex mu;
  static bool done[64] = {};
  int dev = 0;
  LB_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if (dev < 64 && done[dev]) return;
  LB_CUDA(cudaMemcpyToSymbol(c_mm, P.mm, sizeof(P.mm)));
  LB_CUDA(cudaMemcpyToSymbol(c_mmi, P.mmi, sizeof(P.mmi)));
  if (dev < 64) done[dev] = true;
}

struct ExactRelax {
  double tau_s, tau_b, omega_s, omega_b;
};

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// DoStep, lb.cu:72-218: modes, relaxation with forcing, back-projection,
// push-stream with periodic wrap.  blockDim = (32, 8); grid.z = x.
__global__ void __launch_bounds__(256) k_step_exact_f64(const double* __restrict__ f,
                                                        const double* __restrict__ F,
                                                        double* __restrict__ fn, int nx, int ny,
                                                        int nz, long long N, ExactRelax k) {
  const int z = blockIdx.x * 32 + threadIdx.x;
  const int y = blockIdx.y * 8 + threadIdx.y;
  const int x = blockIdx.z;
  if (z >= nz || y >= ny) return;
  const long long nynz = (long long)ny * nz;
  const long long s = x * nynz + (long long)y * nz + z;
  double fo[15], mode[15];
#pragma unroll
  for (int p = 0; p < 15; ++p) fo[p] = f[p * N + s];
#pragma unroll
  for (int m = 0; m < 15; ++m) {
    double acc = 0.0;
#pragma unroll
    for (int p = 0; p < 15; ++p) acc = dadd(acc, dmul(fo[p], c_mm[m][p]));
    mode[m] = acc;
  }
  double Fv[3], u[3], usq = 0.0, uDOTf = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double Fa = F ? F[a * N + s] : 0.0;
    Fv[a] = Fa;
    u[a] = ddiv(dadd(mode[1 + a], dmul(0.5, Fa)), mode[0]);
    mode[1 + a] = dadd(mode[1 + a], Fa);
    usq = dadd(usq, dmul(u[a], u[a]));
    uDOTf = dadd(uDOTf, dmul(u[a], Fa));
  }
  double S[3][3] = {{mode[4], mode[5], mode[6]}, {mode[5], mode[7], mode[8]},
                    {mode[6], mode[8], mode[9]}};
  double TrS = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a) TrS = dadd(TrS, S[a][a]);
#pragma unroll
  for (int a = 0; a < 3; ++a) S[a][a] = dsub(S[a][a], ddiv(TrS, 3.0));
  TrS = dsub(TrS, dmul(k.omega_b, dsub(TrS, dmul(mode[0], usq))));
  TrS = dadd(TrS, dmul(dmul(dmul(2.0, k.omega_b), k.tau_b), uDOTf));
#pragma unroll
  for (int a = 0; a < 3; ++a) {
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const double d = (a == b) ? 1.0 : 0.0;
      S[a][b] = dsub(S[a][b],
                     dmul(k.omega_s, dsub(S[a][b], dmul(mode[0], dsub(dmul(u[a], u[b]), dmul(usq, d))))));
      S[a][b] = dadd(S[a][b], dmul(dmul(dmul(2.0, k.omega_s), k.tau_s),
                                   dsub(dadd(dmul(u[a], Fv[b]), dmul(Fv[a], u[b])),
                                        dmul(dmul(2.0, uDOTf), d))));
    }
    S[a][a] = dadd(S[a][a], ddiv(TrS, 3.0));
  }
  mode[4] = S[0][0];
  mode[5] = S[0][1];
  mode[6] = S[0][2];
  mode[7] = S[1][1];
  mode[8] = S[1][2];
  mode[9] = S[2][2];
#pragma unroll
  for (int m = 10; m < 15; ++m) mode[m] = 0.0;
  const int xm = wrap_once(x - 1, nx), xp = wrap_once(x + 1, nx);
  const int ym = wrap_once(y - 1, ny), yp = wrap_once(y + 1, ny);
  const int zm = wrap_once(z - 1, nz), zp = wrap_once(z + 1, nz);
#pragma unroll
  for (int p = 0; p < 15; ++p) {
    double acc = 0.0;
#pragma unroll
    for (int m = 0; m < 15; ++m) acc = dadd(acc, dmul(mode[m], c_mmi[p][m]));
    const int dx = cx_of(p), dy = cy_of(p), dz = cz_of(p);
    const long long X = dx > 0 ? xp : (dx < 0 ? xm : x);
    const long long Y = dy > 0 ? yp : (dy < 0 ? ym : y);
    const long long Z = dz > 0 ? zp : (dz < 0 ? zm : z);
    fn[p * N + X * nynz + Y * nz + Z] = acc;
  }
}

// DoCalcHydro, lb.cu:250-295.
__global__ void k_calc_hydro_exact_f64(const double* __restrict__ f, const double* __restrict__ F,
                                       double* __restrict__ rho, double* __restrict__ u,
                                       long long N, unsigned* status) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < N;
       s += (long long)gridDim.x * blockDim.x) {
    double fo[15], mode[4];
#pragma unroll
    for (int p = 0; p < 15; ++p) fo[p] = f[p * N + s];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      double acc = 0.0;
#pragma unroll
      for (int p = 0; p < 15; ++p) acc = dadd(acc, dmul(fo[p], c_mm[m][p]));
      mode[m] = acc;
    }
    rho[s] = mode[0];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double Fa = F ? F[a * N + s] : 0.0;
      u[a * N + s] = ddiv(dadd(mode[1 + a], dmul(0.5, Fa)), mode[0]);
    }
    if (!finite_d(mode[0] + mode[1] + mode[2] + mode[3]))
      raise_status(status, LBSWIM_STATUS_NONFINITE);
  }
}

// DoInitFromHydro, lb.cu:314-371 (compat_sxz reproduces lb.cu:356).
__global__ void k_init_exact_f64(const double* __restrict__ rho, const double* __restrict__ u,
                                 double* __restrict__ f, long long N, int compat_sxz) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < N;
       s += (long long)gridDim.x * blockDim.x) {
    const double r = rho[s], ux = u[s], uy = u[N + s], uz = u[2 * N + s];
    double mode[15];
#pragma unroll
    for (int m = 0; m < 15; ++m) mode[m] = 0.0;
    mode[0] = r;
    mode[1] = dmul(r, ux);
    mode[2] = dmul(r, uy);
    mode[3] = dmul(r, uz);
    mode[4] = dmul(dmul(r, ux), ux);
    mode[5] = dmul(dmul(r, ux), uy);
    mode[6] = compat_sxz ? dmul(dmul(r, ux), uy) : dmul(dmul(r, ux), uz);
    mode[7] = dmul(dmul(r, uy), uy);
    mode[8] = dmul(dmul(r, uy), uz);
    mode[9] = dmul(dmul(r, uz), uz);
#pragma unroll
    for (int p = 0; p < 15; ++p) {
      double acc = 0.0;
#pragma unroll
      for (int m = 0; m < 15; ++m) acc = dadd(acc, dmul(mode[m], c_mmi[p][m]));
      f[p * N + s] = acc;
    }
  }
}

static int grid_1d(long long n) {
  long long g = (n + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 152LL * 16 ? 152LL * 16 : g));
}

void exact_step_f64(Lattice* L) {
  upload_tables(L->params);
  const int nx = L->size[0], ny = L->size[1], nz = L->size[2];
  ExactRelax k;
  k.tau_s = L->tau_s;
  k.tau_b = L->tau_b;
  k.omega_s = 1.0 / (L->tau_s + 0.5);
  k.omega_b = 1.0 / (L->tau_b + 0.5);
  dim3 grid((nz + 31) / 32, (ny + 7) / 8, nx);
  k_step_exact_f64<<<grid, dim3(32, 8), 0, L->stream>>>(
      (const double*)L->f[L->cur], L->force_zero_pending ? nullptr : (const double*)L->force,
      (double*)L->f[L->cur ^ 1], nx, ny, nz, L->n, k);
  LB_CHECK_LAUNCH(1);
}

void exact_calc_hydro_f64(Lattice* L) {
  upload_tables(L->params);
  k_calc_hydro_exact_f64<<<grid_1d(L->n), 256, 0, L->stream>>>(
      (const double*)L->f[L->cur], L->force_zero_pending ? nullptr : (const double*)L->force,
      (double*)L->rho, (double*)L->u, L->n, L->status);
  LB_CHECK_LAUNCH(1);
}

void exact_init_from_hydro_f64(Lattice* L) {
  upload_tables(L->params);
  const int compat = (L->compat & LBSWIM_COMPAT_INIT_SXZ) ? 1 : 0;
  k_init_exact_f64<<<grid_1d(L->n), 256, 0, L->stream>>>((const double*)L->rho,
                                                         (const double*)L->u,
                                                         (double*)L->f[L->cur], L->n, compat);
  LB_CHECK_LAUNCH(1);
}

}  // namespace lbswim
