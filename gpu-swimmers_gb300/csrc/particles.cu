// particles.cu -- swimmer force spreading and the swimmer / tracer Move kernels.
//
// Spreading (reference SwimmerArray.cu:42-121) adds, for each swimmer, -P n at
// the tail r - l n and +P n at the head r through the 4^3 Peskin stencil.  The
// reference scatters with FP64 atomics in arbitrary order.  Here the result is
// deterministic: the 2n dipole ends are binned by the 4x4x4 block holding
// their stencil origin, each bin is put in end order, and every lattice site
// gathers the ends whose stencil covers it in a fixed (bin, end) order before
// one write of its force.  No floating-point atomics are used.
#include <algorithm>
#include <mutex>
#include <string>

#include "lbswim_device.cuh"
#include "lbswim_internal.h"

namespace lbswim {

constexpr int BIN = 4;  // spread bin edge, in lattice sites

template <class T>
struct EndRecord {
  int o[3];  // wrapped stencil origin ceil(r - 2)
  int pad;
  T phi[3][4];  // Peskin weights of the 4 stencil nodes per axis
  T F[3];       // force carried by the end
};

struct Dims {
  int n[3];
  int nb[3];  // bins per axis
  long long N;
};

__device__ __forceinline__ int wrap_any(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

template <class T>
__device__ __forceinline__ void stencil_setup(const Dims& D, const double r[3], int o[3],
                                              T phi[3][4]) {
  for (int d = 0; d < 3; ++d) {
    const double x0 = ceil(r[d] - 2.);
    o[d] = wrap_any((int)x0, D.n[d]);
#pragma unroll
    for (int i = 0; i < 4; ++i) phi[d][i] = peskin_delta<T>((T)(r[d] - (x0 + i)));
  }
}

// One record per dipole end: e = 2i is the tail, 2i + 1 the head.
template <class T>
__global__ void k_spread_bin(int nsw, const double* __restrict__ r, const double* __restrict__ nv,
                             double P, double l, Dims D, EndRecord<T>* __restrict__ ends,
                             unsigned* __restrict__ bin_count) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 2 * nsw) return;
  const int i = e >> 1;
  const bool head = e & 1;
  double rr[3], F[3];
  for (int a = 0; a < 3; ++a) {
    const double na = nv[nsw * a + i];
    rr[a] = head ? r[nsw * a + i] : r[nsw * a + i] - na * l;
    F[a] = -P * na;
    if (head) F[a] *= -1.0;
  }
  EndRecord<T> rec;
  stencil_setup<T>(D, rr, rec.o, rec.phi);
  rec.pad = 0;
  for (int a = 0; a < 3; ++a) rec.F[a] = (T)F[a];
  ends[e] = rec;
  const int b = ((rec.o[0] / BIN) * D.nb[1] + rec.o[1] / BIN) * D.nb[2] + rec.o[2] / BIN;
  atomicAdd(bin_count + b, 1u);
}

template <class T>
__global__ void k_spread_scatter(int nends, const EndRecord<T>* __restrict__ ends, Dims D,
                                 unsigned* __restrict__ bin_count,
                                 const unsigned* __restrict__ bin_start, int* __restrict__ order) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nends) return;
  const int* o = ends[e].o;
  const int b = ((o[0] / BIN) * D.nb[1] + o[1] / BIN) * D.nb[2] + o[2] / BIN;
  // Counting back down leaves bin_count at zero for the next call.
  const unsigned slot = atomicSub(bin_count + b, 1u) - 1u;
  order[bin_start[b] + slot] = e;
}

// Put each bin's ends in increasing end order (bins hold a handful of ends).
__global__ void k_spread_sort(int nbins, const unsigned* __restrict__ bin_start,
                              int* __restrict__ order) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbins) return;
  const unsigned s = bin_start[b], t = bin_start[b + 1];
  for (unsigned i = s + 1; i < t; ++i) {
    const int v = order[i];
    unsigned j = i;
    while (j > s && order[j - 1] > v) {
      order[j] = order[j - 1];
      --j;
    }
    order[j] = v;
  }
}

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

__device__ __forceinline__ int candidate_bins(int x, int n, int out[4]) {
  int nb = 0;
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int b = wrap_any(x - s, n) / BIN;
    bool seen = false;
    for (int q = 0; q < nb; ++q) seen |= (out[q] == b);
    if (!seen) out[nb++] = b;
  }
  return nb;
}

// Per-site gather.  accumulate = 0: F = sum (ZeroForce folded in); 1: F += sum.
template <class T>
__global__ void __launch_bounds__(256) k_spread_gather(Dims D, const EndRecord<T>* __restrict__ ends,
                                                       const unsigned* __restrict__ bin_start,
                                                       const int* __restrict__ order,
                                                       T* __restrict__ force, int accumulate) {
  const int z = blockIdx.x * 32 + threadIdx.x;
  const int y = blockIdx.y * 8 + threadIdx.y;
  const int x = blockIdx.z;
  if (z >= D.n[2] || y >= D.n[1]) return;
  int bx[4], by[4], bz[4];
  const int nbx = candidate_bins(x, D.n[0], bx);
  const int nby = candidate_bins(y, D.n[1], by);
  const int nbz = candidate_bins(z, D.n[2], bz);
  T acc0 = T(0), acc1 = T(0), acc2 = T(0);
  bool hit = false;
  for (int i = 0; i < nbx; ++i)
    for (int j = 0; j < nby; ++j)
      for (int k = 0; k < nbz; ++k) {
        const int b = (bx[i] * D.nb[1] + by[j]) * D.nb[2] + bz[k];
        const unsigned s = bin_start[b], t = bin_start[b + 1];
        for (unsigned q = s; q < t; ++q) {
          const EndRecord<T>& e = ends[order[q]];
          const T wx = axis_weight(x, e.o[0], D.n[0], e.phi[0]);
          const T wy = axis_weight(y, e.o[1], D.n[1], e.phi[1]);
          const T wz = axis_weight(z, e.o[2], D.n[2], e.phi[2]);
          bool cover = true;
          if (D.n[0] >= 4) cover &= ((x - e.o[0] + D.n[0]) % D.n[0]) <= 3;
          if (D.n[1] >= 4) cover &= ((y - e.o[1] + D.n[1]) % D.n[1]) <= 3;
          if (D.n[2] >= 4) cover &= ((z - e.o[2] + D.n[2]) % D.n[2]) <= 3;
          if (!cover) continue;
          const T d3 = wx * wy * wz;
          acc0 += d3 * e.F[0];
          acc1 += d3 * e.F[1];
          acc2 += d3 * e.F[2];
          hit = true;
        }
      }
  const long long s = (long long)x * D.n[1] * D.n[2] + (long long)y * D.n[2] + z;
  if (!accumulate) {
    force[s] = acc0;
    force[D.N + s] = acc1;
    force[2 * D.N + s] = acc2;
  } else if (hit) {
    force[s] += acc0;
    force[D.N + s] += acc1;
    force[2 * D.N + s] += acc2;
  }
}

// ---- exclusive scan of bin counts (three passes, 4096 entries per CTA) -------
constexpr int SCAN_THREADS = 512, SCAN_PER_THREAD = 8, SCAN_TILE = SCAN_THREADS * SCAN_PER_THREAD;

__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned* warp_sums,
                                                         unsigned& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    unsigned w = lane < nw ? warp_sums[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) warp_sums[lane] = w;
  }
  __syncthreads();
  total = warp_sums[(blockDim.x >> 5) - 1];
  const unsigned before = warp ? warp_sums[warp - 1] : 0u;
  __syncthreads();
  return before + x - v;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(const unsigned* __restrict__ in, int n,
                                                             unsigned* __restrict__ tile_sums) {
  __shared__ unsigned ws[32];
  const long long base = (long long)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER_THREAD;
  unsigned s = 0;
  for (int i = 0; i < SCAN_PER_THREAD; ++i)
    if (base + i < n) s += in[base + i];
  unsigned total;
  block_exclusive_scan(s, ws, total);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_scan_top(unsigned* __restrict__ tile_sums, int ntiles) {
  __shared__ unsigned ws[32];
  __shared__ unsigned carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < ntiles; base += 1024) {
    const int i = base + threadIdx.x;
    const unsigned v = i < ntiles ? tile_sums[i] : 0u;
    unsigned total;
    const unsigned ex = block_exclusive_scan(v, ws, total);
    if (i < ntiles) tile_sums[i] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += total;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(const unsigned* __restrict__ in, int n,
                                                             const unsigned* __restrict__ tile_off,
                                                             unsigned* __restrict__ out,
                                                             unsigned grand_total) {
  __shared__ unsigned ws[32];
  const long long base = (long long)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER_THREAD;
  unsigned v[SCAN_PER_THREAD];
  unsigned s = 0;
  for (int i = 0; i < SCAN_PER_THREAD; ++i) {
    v[i] = base + i < n ? in[base + i] : 0u;
    s += v[i];
  }
  unsigned total;
  unsigned run = block_exclusive_scan(s, ws, total) + tile_off[blockIdx.x];
  for (int i = 0; i < SCAN_PER_THREAD; ++i) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = grand_total;
}

// ---- Move kernels -----------------------------------------------------------
// InterpVelocity, interp.cu:8-47: u at r through the 4^3 Peskin stencil.
template <class U, class T>
__device__ __forceinline__ void interp_velocity(const U* __restrict__ u, const Dims& D,
                                                const double r[3], T v[3]) {
  int idx[3][4];
  T phi[3][4];
  for (int d = 0; d < 3; ++d) {
    const double x0 = ceil(r[d] - 2.);
    const int o = wrap_any((int)x0, D.n[d]);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int t = o + i;
      while (t >= D.n[d]) t -= D.n[d];
      idx[d][i] = t;
      phi[d][i] = peskin_delta<T>((T)(r[d] - (x0 + i)));
    }
  }
  v[0] = v[1] = v[2] = T(0);
  const long long nynz = (long long)D.n[1] * D.n[2];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      const T pij = phi[0][i] * phi[1][j];
      const long long row = idx[0][i] * nynz + (long long)idx[1][j] * D.n[2];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const T d3 = pij * phi[2][k];
        const long long s = row + idx[2][k];
        v[0] += d3 * (T)u[s];
        v[1] += d3 * (T)u[D.N + s];
        v[2] += d3 * (T)u[2 * D.N + s];
      }
    }
}

// DoSwimmerArrayMove, SwimmerArray.cu:123-210.
template <class U, class T>
__global__ void k_swimmers_move(int nsw, double* __restrict__ swr, double* __restrict__ swv,
                                double* __restrict__ swn, lbswim_common_params c,
                                unsigned long long seed, unsigned long long step, Dims D,
                                const U* __restrict__ u) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsw) return;
  double r[3], n0[3];
  for (int d = 0; d < 3; ++d) {
    r[d] = swr[nsw * d + i];
    n0[d] = swn[nsw * d + i];
  }
  T v[3];
  interp_velocity<U, T>(u, D, r, v);
  double rMinus[3];
  for (int d = 0; d < 3; ++d) {
    double rDot = c.mobility * c.P * n0[d];
    if (!c.translational_advection_off) rDot += (double)v[d];
    rMinus[d] = r[d] - n0[d] * c.l;
    swv[nsw * d + i] = rDot;
    swr[nsw * d + i] = fmod(r[d] + rDot + D.n[d], (double)D.n[d]);
  }
  const float rnd = rng_uniform(seed, (uint32_t)i, step);
  double nn[3];
  if (rnd < c.alpha) {  // tumble: a direction uniform on the sphere
    rng_normal3(seed, (uint32_t)i, step, nn);
  } else if (!c.rotational_advection_off) {  // rotate with the local shear
    T vm[3];
    interp_velocity<U, T>(u, D, rMinus, vm);
    for (int d = 0; d < 3; ++d) nn[d] = n0[d] + ((double)v[d] - (double)vm[d]) / c.l;
  } else {
    return;  // orientation unchanged
  }
  const double norm = sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
  for (int d = 0; d < 3; ++d) swn[nsw * d + i] = nn[d] / norm;
}

// DoTracerArrayMove, TracerArray.cu:12-43 (s accumulated per tracer).
template <class U, class T>
__global__ void k_tracers_move(int ntr, double* __restrict__ r, double* __restrict__ s,
                               double* __restrict__ v, Dims D, const U* __restrict__ u) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ntr) return;
  double rr[3];
  for (int d = 0; d < 3; ++d) rr[d] = r[ntr * d + i];
  T vv[3];
  interp_velocity<U, T>(u, D, rr, vv);
  for (int d = 0; d < 3; ++d) {
    const double vd = (double)vv[d];
    v[ntr * d + i] = vd;
    r[ntr * d + i] = fmod(rr[d] + vd + D.n[d], (double)D.n[d]);
    s[ntr * d + i] += vd;
  }
}

template <class U, class T>
__global__ void k_interp_points(int np, const double* __restrict__ r, double* __restrict__ v,
                                Dims D, const U* __restrict__ u) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const double rr[3] = {r[i], r[np + i], r[2 * np + i]};
  T vv[3];
  interp_velocity<U, T>(u, D, rr, vv);
  for (int d = 0; d < 3; ++d) v[np * d + i] = (double)vv[d];
}

__global__ void k_rng_draws(unsigned long long seed, int n, unsigned long long step,
                            float* __restrict__ uni, double* __restrict__ g) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uni[i] = rng_uniform(seed, (uint32_t)i, step);
  double nn[3];
  rng_normal3(seed, (uint32_t)i, step, nn);
  for (int d = 0; d < 3; ++d) g[n * d + i] = nn[d];
}

// ---- host side -----------------------------------------------------------------
static Dims make_dims(const Lattice* L) {
  Dims D;
  for (int a = 0; a < 3; ++a) {
    D.n[a] = L->size[a];
    D.nb[a] = (L->size[a] + BIN - 1) / BIN;
  }
  D.N = L->n;
  return D;
}

static void ensure_spread(Lattice* L, int nends) {
  SpreadScratch& S = L->spread;
  const Dims D = make_dims(L);
  const int nbins = D.nb[0] * D.nb[1] * D.nb[2];
  if (S.nbins != nbins) {
    if (S.bin_count) cudaFree(S.bin_count);
    if (S.bin_start) cudaFree(S.bin_start);
    if (S.scan_tmp) cudaFree(S.scan_tmp);
    LB_CUDA(cudaMalloc(&S.bin_count, sizeof(unsigned) * nbins));
    LB_CUDA(cudaMalloc(&S.bin_start, sizeof(unsigned) * (nbins + 1)));
    const int ntiles = (nbins + SCAN_TILE - 1) / SCAN_TILE;
    LB_CUDA(cudaMalloc(&S.scan_tmp, sizeof(unsigned) * std::max(ntiles, 1)));
    LB_CUDA(cudaMemsetAsync(S.bin_count, 0, sizeof(unsigned) * nbins, L->stream));
    S.nbins = nbins;
  }
  const size_t rec = L->precision == LBSWIM_F64 ? sizeof(EndRecord<double>) : sizeof(EndRecord<float>);
  if (S.capacity_ends < nends || S.ends_bytes < rec * (size_t)nends) {
    LB_CUDA(cudaStreamSynchronize(L->stream));
    if (S.order) cudaFree(S.order);
    if (S.ends) cudaFree(S.ends);
    const int cap = std::max(nends, 64);
    LB_CUDA(cudaMalloc(&S.order, sizeof(int) * cap));
    LB_CUDA(cudaMalloc(&S.ends, rec * cap));
    S.capacity_ends = cap;
    S.ends_bytes = rec * cap;
  }
}

static void scan_bins(Lattice* L, unsigned total) {
  SpreadScratch& S = L->spread;
  const int ntiles = (S.nbins + SCAN_TILE - 1) / SCAN_TILE;
  k_scan_tiles<<<ntiles, SCAN_THREADS, 0, L->stream>>>(S.bin_count, S.nbins, S.scan_tmp);
  k_scan_top<<<1, 1024, 0, L->stream>>>(S.scan_tmp, ntiles);
  k_scan_apply<<<ntiles, SCAN_THREADS, 0, L->stream>>>(S.bin_count, S.nbins, S.scan_tmp,
                                                       S.bin_start, total);
  LB_CHECK_LAUNCH(3);
}

template <class T>
static void add_forces_t(Swimmers* W, Lattice* L) {
  const int nends = 2 * W->n;
  ensure_spread(L, nends);
  SpreadScratch& S = L->spread;
  const Dims D = make_dims(L);
  EndRecord<T>* ends = (EndRecord<T>*)S.ends;
  const int accumulate = L->force_zero_pending ? 0 : 1;
  if (nends > 0) {
    k_spread_bin<T><<<(nends + 255) / 256, 256, 0, L->stream>>>(
        W->n, W->r, W->nv, W->common.P, W->common.l, D, ends, S.bin_count);
    LB_CHECK_LAUNCH(1);
  }
  scan_bins(L, (unsigned)nends);
  if (nends > 0) {
    k_spread_scatter<T><<<(nends + 255) / 256, 256, 0, L->stream>>>(nends, ends, D, S.bin_count,
                                                                     S.bin_start, S.order);
    k_spread_sort<<<(S.nbins + 255) / 256, 256, 0, L->stream>>>(S.nbins, S.bin_start, S.order);
    LB_CHECK_LAUNCH(2);
  }
  dim3 grid((D.n[2] + 31) / 32, (D.n[1] + 7) / 8, D.n[0]);
  k_spread_gather<T><<<grid, dim3(32, 8), 0, L->stream>>>(D, ends, S.bin_start, S.order,
                                                          (T*)L->force, accumulate);
  LB_CHECK_LAUNCH(1);
  L->force_zero_pending = false;
  L->force_version++;
}

void swimmers_add_forces(Swimmers* W, Lattice* L) {
  if (L->precision == LBSWIM_F64)
    add_forces_t<double>(W, L);
  else
    add_forces_t<float>(W, L);
}

void swimmers_move(Swimmers* W, Lattice* L) {
  const Dims D = make_dims(L);
  if (W->n > 0) {
    const int grid = (W->n + 255) / 256;
    if (L->precision == LBSWIM_F64)
      k_swimmers_move<double, double><<<grid, 256, 0, L->stream>>>(
          W->n, W->r, W->v, W->nv, W->common, W->seed, W->step, D, (const double*)L->u);
    else
      k_swimmers_move<float, float><<<grid, 256, 0, L->stream>>>(
          W->n, W->r, W->v, W->nv, W->common, W->seed, W->step, D, (const float*)L->u);
    LB_CHECK_LAUNCH(1);
  }
  W->step++;
}

void tracers_move(Tracers* T, Lattice* L) {
  if (T->n <= 0) return;
  const Dims D = make_dims(L);
  const int grid = (T->n + 255) / 256;
  if (L->precision == LBSWIM_F64)
    k_tracers_move<double, double><<<grid, 256, 0, L->stream>>>(T->n, T->r, T->s, T->v, D,
                                                                 (const double*)L->u);
  else
    k_tracers_move<float, float><<<grid, 256, 0, L->stream>>>(T->n, T->r, T->s, T->v, D,
                                                               (const float*)L->u);
  LB_CHECK_LAUNCH(1);
}

void lattice_interp_velocity(Lattice* L, int np, const double* r_host, double* v_host) {
  if (np <= 0) return;
  const Dims D = make_dims(L);
  double *r = nullptr, *v = nullptr;
  LB_CUDA(cudaMalloc(&r, sizeof(double) * 3 * np));
  cudaError_t e = cudaMalloc(&v, sizeof(double) * 3 * np);
  if (e != cudaSuccess) {
    cudaFree(r);
    LB_CUDA(e);
  }
  try {
    LB_CUDA(cudaMemcpyAsync(r, r_host, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, L->stream));
    if (L->precision == LBSWIM_F64)
      k_interp_points<double, double><<<(np + 255) / 256, 256, 0, L->stream>>>(np, r, v, D,
                                                                              (const double*)L->u);
    else
      k_interp_points<float, float><<<(np + 255) / 256, 256, 0, L->stream>>>(np, r, v, D,
                                                                            (const float*)L->u);
    LB_CHECK_LAUNCH(1);
    LB_CUDA(cudaMemcpyAsync(v_host, v, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, L->stream));
    LB_CUDA(cudaStreamSynchronize(L->stream));
  } catch (...) {
    cudaFree(r);
    cudaFree(v);
    throw;
  }
  cudaFree(r);
  cudaFree(v);
}

// ---- allocation-free spreading ------------------------------------------------
// Scratch of lbswim_spread_forces_noalloc: one file-scope device array that
// every GPU loading the library holds until exit.  Layout (bytes):
//   bin counts [NOALLOC_MAX_BINS] | bin starts [NOALLOC_MAX_BINS + 1] |
//   scan tile sums | end order [NOALLOC_MAX_ENDS] | end records [NOALLOC_MAX_ENDS]
constexpr int NOALLOC_MAX_ENDS = 2 * LBSWIM_NOALLOC_MAX_SWIMMERS;
constexpr int NOALLOC_MAX_BINS = LBSWIM_NOALLOC_MAX_SPREAD_BINS;
constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t NA_COUNT = 0;
constexpr size_t NA_START = NA_COUNT + align256(sizeof(unsigned) * NOALLOC_MAX_BINS);
constexpr size_t NA_TILES = NA_START + align256(sizeof(unsigned) * (NOALLOC_MAX_BINS + 1));
constexpr size_t NA_ORDER =
    NA_TILES + align256(sizeof(unsigned) * ((NOALLOC_MAX_BINS + SCAN_TILE - 1) / SCAN_TILE));
constexpr size_t NA_ENDS = NA_ORDER + align256(sizeof(int) * NOALLOC_MAX_ENDS);
constexpr size_t NA_BYTES = NA_ENDS + align256(sizeof(EndRecord<double>) * NOALLOC_MAX_ENDS);

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

// Device address of g_noalloc_scratch, looked up once per device with that
// device current (the symbol's name in host code is only a stand-in).
static unsigned char* noalloc_scratch_for_current_device() {
  static std::mutex mu;
  static unsigned char* addr[64] = {nullptr};
  int dev = 0;
  LB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) throw LbswimError{LBSWIM_ENOTSUP, "device index out of range"};
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    LB_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    addr[dev] = (unsigned char*)p;
  }
  return addr[dev];
}

void spread_forces_noalloc(const double* r, const double* nv, int nsw, double P, double l,
                           const int size[3], double* force, int accumulate,
                           cudaStream_t stream) {
  Dims D;
  for (int a = 0; a < 3; ++a) {
    D.n[a] = size[a];
    D.nb[a] = (size[a] + BIN - 1) / BIN;
  }
  D.N = (long long)size[0] * size[1] * size[2];
  const long long nbins = (long long)D.nb[0] * D.nb[1] * D.nb[2];
  const int nends = 2 * nsw;
  if (nends > NOALLOC_MAX_ENDS)
    throw LbswimError{LBSWIM_EINVAL, "more swimmers than the allocation-free limit of " +
                                         std::to_string(LBSWIM_NOALLOC_MAX_SWIMMERS)};
  if (nbins > NOALLOC_MAX_BINS)
    throw LbswimError{LBSWIM_EINVAL,
                      "lattice larger than the allocation-free limit (" +
                          std::to_string(NOALLOC_MAX_BINS) + " spread bins of 4^3 sites)"};
  unsigned char* base = noalloc_scratch_for_current_device();
  unsigned* bin_count = (unsigned*)(base + NA_COUNT);
  unsigned* bin_start = (unsigned*)(base + NA_START);
  unsigned* tiles = (unsigned*)(base + NA_TILES);
  int* order = (int*)(base + NA_ORDER);
  EndRecord<double>* ends = (EndRecord<double>*)(base + NA_ENDS);
  // The array keeps the previous call's contents: the counts must start at zero.
  LB_CUDA(cudaMemsetAsync(bin_count, 0, sizeof(unsigned) * nbins, stream));
  const int nb = (int)nbins;
  if (nends > 0) {
    k_spread_bin<double><<<(nends + 255) / 256, 256, 0, stream>>>(nsw, r, nv, P, l, D, ends,
                                                                  bin_count);
    LB_CHECK_LAUNCH(1);
  }
  const int ntiles = (nb + SCAN_TILE - 1) / SCAN_TILE;
  k_scan_tiles<<<ntiles, SCAN_THREADS, 0, stream>>>(bin_count, nb, tiles);
  k_scan_top<<<1, 1024, 0, stream>>>(tiles, ntiles);
  k_scan_apply<<<ntiles, SCAN_THREADS, 0, stream>>>(bin_count, nb, tiles, bin_start,
                                                    (unsigned)nends);
  LB_CHECK_LAUNCH(3);
  if (nends > 0) {
    k_spread_scatter<double><<<(nends + 255) / 256, 256, 0, stream>>>(nends, ends, D, bin_count,
                                                                      bin_start, order);
    k_spread_sort<<<(nb + 255) / 256, 256, 0, stream>>>(nb, bin_start, order);
    LB_CHECK_LAUNCH(2);
  }
  dim3 grid((D.n[2] + 31) / 32, (D.n[1] + 7) / 8, D.n[0]);
  k_spread_gather<double><<<grid, dim3(32, 8), 0, stream>>>(D, ends, bin_start, order, force,
                                                            accumulate);
  LB_CHECK_LAUNCH(1);
}

void rng_draws(unsigned long long seed, int n, unsigned long long step, float* u_host,
               double* g_host) {
  if (n <= 0) return;
  float* u = nullptr;
  double* g = nullptr;
  LB_CUDA(cudaMalloc(&u, sizeof(float) * n));
  cudaError_t e = cudaMalloc(&g, sizeof(double) * 3 * n);
  if (e != cudaSuccess) {
    cudaFree(u);
    LB_CUDA(e);
  }
  k_rng_draws<<<(n + 255) / 256, 256>>>(seed, n, step, u, g);
  cudaError_t le = cudaGetLastError();
  if (le == cudaSuccess) le = cudaMemcpy(u_host, u, sizeof(float) * n, cudaMemcpyDeviceToHost);
  if (le == cudaSuccess) le = cudaMemcpy(g_host, g, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost);
  cudaFree(u);
  cudaFree(g);
  LB_CUDA(le);
  count_launches(1);
}

}  // namespace lbswim
