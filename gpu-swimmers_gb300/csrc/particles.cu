// particles.cu -- swimmer force spreading and the swimmer / tracer Move kernels.
//
// Spreading (reference SwimmerArray.cu:42-121) adds, for each swimmer, -P n at
// the tail r - l n and +P n at the head r through the 4^3 Peskin stencil.  The
// reference scatters with FP64 atomics in arbitrary order.  Here the result is
// deterministic and uses no floating-point atomics: AddForces records the 2n
// dipole ends (origin, Peskin weights, force); the ends are then listed under
// every tile their stencil touches (integer counting sort), and each tile sums,
// for every site, the covering ends in end order.  The tiles are either force
// tiles (k_force_tile, which writes the dense force field) or, for FP32/BF16/
// FP16 lattices, the slabs of the fused step kernel, which spreads the ends
// itself so the force field never goes through HBM.
//
// The original 4^3-origin-bin kernels below (k_spread_bin ... k_spread_gather)
// serve lbswim_spread_forces_noalloc.
#include <algorithm>
#include <mutex>
#include <string>

#include "lbswim_device.cuh"
#include "lbswim_internal.h"

namespace lbswim {

constexpr int BIN = 4;  // spread bin edge, in lattice sites

struct Dims {
  int n[3];
  int nb[3];  // bins per axis
  long long N;
};

// acc + a b: FP64 rounds the product and the sum on their own (the oracle's
// order, bit for bit); FP32 lets the compiler fuse them.
template <class T>
__device__ __forceinline__ T add_prod(T acc, T a, T b) {
  if constexpr (sizeof(T) == 8)
    return __dadd_rn(acc, __dmul_rn(a, b));
  else
    return acc + a * b;
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
    rr[a] = head ? r[nsw * a + i] : __dsub_rn(r[nsw * a + i], __dmul_rn(na, l));
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

// ---- tile-touch spreading ------------------------------------------------------
// Every dipole end is listed under each force tile its stencil touches; a tile's
// list is then put in end order, and one CTA per tile sums, for each of its
// sites, the covering ends of its list in that order.  The per-site order is a
// fixed function of the input, so the result is deterministic.
struct TileGrid {
  int T[3];   // tile edge per axis
  int h;      // sites beyond the tile (every side) that also need the force
  int nt[3];  // tiles per axis
};

// Tiles along one axis whose extended region holds one of the nodes o..o+3:
// the sites o-h .. o+3+h form one cyclic interval, so the tiles form the cyclic
// range first, first+1, ... (count of them, at most nt).  An interval that
// wraps past the end covers the tiles from `first` to the last one and from 0
// to the tile of its wrapped end; if those meet, it covers every tile.  o is a
// wrapped node (0 <= o < n, as records hold them) and h < n; the tile edge T
// is a power of two (slab and force-tile shapes all are), so tiles are shifts.
__device__ __forceinline__ void touched_range(int o, int n, int T, int h, int nt, int& first,
                                              int& count) {
  const int len = 4 + 2 * h;
  if (len >= n) {
    first = 0;
    count = nt;
    return;
  }
  const int sh = __ffs(T) - 1;
  const int a = o - h < 0 ? o - h + n : o - h, b = a + len - 1;
  first = a >> sh;
  if (b < n) {
    count = (b >> sh) - first + 1;
  } else {
    const int last = (b - n) >> sh;
    count = last >= first ? nt : (nt - first) + last + 1;
  }
}

constexpr int REC_THREADS = 256;

// Slab shape of a tile choice, as slab_shape_of (lattice.cu): x planes, rows, columns.
__device__ __forceinline__ void slab_shape_of_dev(int tile, int T[3]) {
  T[0] = 32;
  T[1] = tile == 1 ? 16 : 8;
  T[2] = tile == 1 ? 16 : 32;
}

// List end e under every slab of grid G whose extended region its stencil
// touches (at most SLAB_BUCKET_CAP ends are kept per slab; the count goes on).
__device__ __forceinline__ void bucket_end(int e, const int o[3], const Dims& D, const TileGrid& G,
                                           unsigned* __restrict__ count,
                                           int* __restrict__ list) {
  int f[3], c[3];
  for (int a = 0; a < 3; ++a) touched_range(o[a], D.n[a], G.T[a], G.h, G.nt[a], f[a], c[a]);
  for (int i = 0; i < c[0]; ++i) {
    const int kx = f[0] + i < G.nt[0] ? f[0] + i : f[0] + i - G.nt[0];
    for (int j = 0; j < c[1]; ++j) {
      const int ky = f[1] + j < G.nt[1] ? f[1] + j : f[1] + j - G.nt[1];
      for (int k = 0; k < c[2]; ++k) {
        const int kz = f[2] + k < G.nt[2] ? f[2] + k : f[2] + k - G.nt[2];
        const int t = (kx * G.nt[1] + ky) * G.nt[2] + kz;
        const unsigned slot = atomicAdd(count + t, 1u);
        if (slot < (unsigned)SLAB_BUCKET_CAP) list[(long long)t * SLAB_BUCKET_CAP + slot] = e;
      }
    }
  }
}

// One record per dipole end: e = 2i is the tail, 2i + 1 the head.  Records are
// assembled in shared memory and written out as one contiguous block; with
// bucket_count set, each end is also listed under the step-kernel slabs it
// touches (its index among all pending ends is e_base + e).  FP32 records take
// the stencil origin from the bits of the position (stencil_axis) and the
// four weights from one square root (peskin_weights4), like the FP32
// interpolation.
template <class T>
__device__ __forceinline__ void end_records_block(
    int blk, int nsw, const double* __restrict__ r, const double* __restrict__ nv, double P,
    double l, Dims D, EndRecord<T>* __restrict__ ends, int e_base,
    unsigned* __restrict__ max_abs_f, TileGrid G, unsigned* __restrict__ bucket_count,
    int* __restrict__ bucket_list) {
  __shared__ EndRecord<T> srec[REC_THREADS];
  __shared__ unsigned smax;
  if (threadIdx.x == 0) smax = 0u;
  __syncthreads();
  const int e0 = blk * REC_THREADS;
  const int e = e0 + threadIdx.x;
  const int nends = 2 * nsw;
  unsigned mbits = 0u;  // largest |F| component of this thread's end, as float bits
  if (e < nends) {
    const int i = e >> 1;
    const bool head = e & 1;
    double rr[3], F[3];
    for (int a = 0; a < 3; ++a) {
      const double na = nv[nsw * a + i];
      rr[a] = head ? r[nsw * a + i] : __dsub_rn(r[nsw * a + i], __dmul_rn(na, l));
      F[a] = -P * na;
      if (head) F[a] *= -1.0;
    }
    EndRecord<T>& rec = srec[threadIdx.x];
    if constexpr (sizeof(T) == 4) {
      for (int a = 0; a < 3; ++a) {
        int x0;
        float dr;
        stencil_axis(rr[a], x0, dr);
        rec.o[a] = wrap_any(x0, D.n[a]);
        float w[4];
        peskin_weights4(dr, w);
#pragma unroll
        for (int j = 0; j < 4; ++j) rec.phi[a][j] = w[j];
      }
    } else {
      stencil_setup<T>(D, rr, rec.o, rec.phi);
    }
    rec.pad = 0;
    float m = 0.f;
    for (int a = 0; a < 3; ++a) {
      rec.F[a] = (T)F[a];
      m = fmaxf(m, fabsf((float)F[a]));
    }
    mbits = __float_as_uint(m);
    if (bucket_count) bucket_end(e_base + e, rec.o, D, G, bucket_count, bucket_list);
  }
  // non-negative floats order like their bit patterns: a warp's largest, then
  // one shared-memory atomic per warp
  mbits = __reduce_max_sync(0xffffffffu, mbits);
  if ((threadIdx.x & 31) == 0 && mbits) atomicMax(&smax, mbits);
  __syncthreads();
  if (threadIdx.x == 0 && max_abs_f) atomicMax(max_abs_f, smax);
  const int nrec = min(REC_THREADS, nends - e0);
  const int words = nrec * (int)(sizeof(EndRecord<T>) / 4);
  const unsigned* src = reinterpret_cast<const unsigned*>(srec);
  unsigned* dst = reinterpret_cast<unsigned*>(ends + e0);
  for (int w = threadIdx.x; w < words; w += REC_THREADS) dst[w] = src[w];
}

template <class T>
__global__ void __launch_bounds__(REC_THREADS) k_end_records(
    int nsw, const double* __restrict__ r, const double* __restrict__ nv, double P, double l,
    Dims D, EndRecord<T>* __restrict__ ends, int e_base, unsigned* __restrict__ max_abs_f,
    TileGrid G, unsigned* __restrict__ bucket_count, int* __restrict__ bucket_list) {
  end_records_block<T>(blockIdx.x, nsw, r, nv, P, l, D, ends, e_base, max_abs_f, G, bucket_count,
                       bucket_list);
}

// Slab buckets of recorded ends (the slab shape changed since they were recorded).
__global__ void k_bucket_ends(int nends, const EndRecord<float>* __restrict__ ends, Dims D,
                              TileGrid G, unsigned* __restrict__ count, int* __restrict__ list) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nends) return;
  const int o[3] = {ends[e].o[0], ends[e].o[1], ends[e].o[2]};
  bucket_end(e, o, D, G, count, list);
}

template <class T, int PASS>
__global__ void k_touch(int nends, const EndRecord<T>* __restrict__ ends, Dims D, TileGrid G,
                        unsigned* __restrict__ count, const unsigned* __restrict__ start,
                        int* __restrict__ list) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nends) return;
  const int ox = ends[e].o[0], oy = ends[e].o[1], oz = ends[e].o[2];
  int fx, cx, fy, cy, fz, cz;
  touched_range(ox, D.n[0], G.T[0], G.h, G.nt[0], fx, cx);
  touched_range(oy, D.n[1], G.T[1], G.h, G.nt[1], fy, cy);
  touched_range(oz, D.n[2], G.T[2], G.h, G.nt[2], fz, cz);
  for (int i = 0; i < cx; ++i) {
    const int kx = fx + i < G.nt[0] ? fx + i : fx + i - G.nt[0];
    for (int j = 0; j < cy; ++j) {
      const int ky = fy + j < G.nt[1] ? fy + j : fy + j - G.nt[1];
      for (int k = 0; k < cz; ++k) {
        const int kz = fz + k < G.nt[2] ? fz + k : fz + k - G.nt[2];
        const int t = (kx * G.nt[1] + ky) * G.nt[2] + kz;
        if (PASS == 0) {
          atomicAdd(count + t, 1u);
        } else {
          // counting back down leaves the counts at zero for the next call
          const unsigned slot = atomicSub(count + t, 1u) - 1u;
          list[start[t] + slot] = e;
        }
      }
    }
  }
}

// Exclusive-scan finish that also writes the grand total to out[n].
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply_total(
    const unsigned* __restrict__ in, int n, const unsigned* __restrict__ tile_off,
    unsigned* __restrict__ out) {
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
    if (base + i == n - 1) out[n] = run;
  }
}

// Force tile (FP64 lattices): 8 (x) x 8 (y) x 32 (z) sites, 16 warps, each
// warp owns 4 of the 64 z-rows; a warp ballot picks the ends covering a row.
// The ends are put in end order by rank and every site adds their
// contributions in that order, ((phi_x phi_y) phi_z) F as the reference does
// (SwimmerArray.cu:64-73).  FP32 lattices spread in the step kernel and in
// k_force_slab instead.
constexpr int FT_X = 8, FT_Y = 8, FT_Z = 32, FT_THREADS = 512, FT_CAP = 256;
static_assert((FT_X & (FT_X - 1)) == 0 && (FT_Y & (FT_Y - 1)) == 0 && (FT_Z & (FT_Z - 1)) == 0,
              "tile edges are powers of two (touched_range shifts)");

__global__ void __launch_bounds__(FT_THREADS) k_force_tile(Dims D, TileGrid G,
                                                           const EndRecord<double>* __restrict__ ends,
                                                           const unsigned* __restrict__ start,
                                                           const int* __restrict__ list,
                                                           int* __restrict__ sorted,
                                                           double* __restrict__ force,
                                                           int accumulate) {
  using T = double;
  __shared__ EndRecord<T> srec[FT_CAP];
  __shared__ int skey[FT_CAP];
  const int tile = blockIdx.x;
  const int kz = tile % G.nt[2], ky = (tile / G.nt[2]) % G.nt[1], kx = tile / (G.nt[1] * G.nt[2]);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned s0 = start[tile], s1 = start[tile + 1];
  const int cnt = (int)(s1 - s0);
  const bool in_smem = cnt <= FT_CAP;
  if (in_smem) {
    for (int q = tid; q < cnt; q += FT_THREADS) skey[q] = list[s0 + q];
    __syncthreads();
    for (int q = tid; q < cnt; q += FT_THREADS) srec[rank_of(skey[q], skey, cnt)] = ends[skey[q]];
  } else {
    // more ends than fit: order them in global scratch and read records from there
    for (int q = tid; q < cnt; q += FT_THREADS) {
      const int k = list[s0 + q];
      int r = 0;
      for (int j = 0; j < cnt; ++j) r += list[s0 + j] < k;
      sorted[s0 + r] = k;
    }
  }
  __syncthreads();
  auto rec = [&](int q) -> const EndRecord<T>& { return in_smem ? srec[q] : ends[sorted[s0 + q]]; };
  const int z = kz * FT_Z + lane;
  const bool zval = z < D.n[2];
  // no axis shorter than a stencil: one node of an end lands on a site
  const bool single = D.n[0] >= 4 && D.n[1] >= 4 && D.n[2] >= 4;
  for (int row = warp; row < FT_X * FT_Y; row += FT_THREADS / 32) {
    const int x = kx * FT_X + (row >> 3), y = ky * FT_Y + (row & 7);
    if (x >= D.n[0] || y >= D.n[1]) continue;
    const long long s = (long long)x * D.n[1] * D.n[2] + (long long)y * D.n[2] + z;
    // the sums start from the base force and add the ends in end order, as
    // the oracle's serial spreading does
    T acc0 = T(0), acc1 = T(0), acc2 = T(0);
    if (accumulate && zval) {
      acc0 = force[s];
      acc1 = force[D.N + s];
      acc2 = force[2 * D.N + s];
    }
    bool hit = false;
    for (int base = 0; base < cnt; base += 32) {
      const int q = base + lane;
      bool covers = false;
      if (q < cnt) {
        const EndRecord<T>& e = rec(q);
        covers = covers_axis(x, e.o[0], D.n[0]) && covers_axis(y, e.o[1], D.n[1]);
      }
      // this lane's ends among those covering the row (they also cover its z),
      // in end order; each lane then adds its own, so that the FP64 work of
      // the row's ends runs on all the lanes they cover at once
      const unsigned m = __ballot_sync(0xffffffffu, covers);  // every lane takes part
      unsigned mine = 0u;
      if (zval)
        for (unsigned mm = m; mm; mm &= mm - 1) {
          const int b = __ffs(mm) - 1;
          if (covers_axis(z, rec(base + b).o[2], D.n[2])) mine |= 1u << b;
        }
      hit |= mine != 0u;
      for (; mine; mine &= mine - 1) {
        const EndRecord<T>& e = rec(base + __ffs(mine) - 1);
        if (single) {
          int i = x - e.o[0], j = y - e.o[1], k = z - e.o[2];
          i += i < 0 ? D.n[0] : 0;
          j += j < 0 ? D.n[1] : 0;
          k += k < 0 ? D.n[2] : 0;
          acc0 = __dadd_rn(acc0, end_contrib(e.phi[0][i], e.phi[1][j], e.phi[2][k], e.F[0]));
          acc1 = __dadd_rn(acc1, end_contrib(e.phi[0][i], e.phi[1][j], e.phi[2][k], e.F[1]));
          acc2 = __dadd_rn(acc2, end_contrib(e.phi[0][i], e.phi[1][j], e.phi[2][k], e.F[2]));
          continue;
        }
        // node by node in (i, j, k) order, as AccumulateDeltaForce adds them
        // (several nodes land on one site when an axis is shorter than 4)
        for (int i = 0; i < 4; ++i) {
          if (wrap_any(e.o[0] + i, D.n[0]) != x) continue;
          for (int j = 0; j < 4; ++j) {
            if (wrap_any(e.o[1] + j, D.n[1]) != y) continue;
            for (int k = 0; k < 4; ++k) {
              if (wrap_any(e.o[2] + k, D.n[2]) != z) continue;
              acc0 = __dadd_rn(acc0, end_contrib(e.phi[0][i], e.phi[1][j], e.phi[2][k], e.F[0]));
              acc1 = __dadd_rn(acc1, end_contrib(e.phi[0][i], e.phi[1][j], e.phi[2][k], e.F[1]));
              acc2 = __dadd_rn(acc2, end_contrib(e.phi[0][i], e.phi[1][j], e.phi[2][k], e.F[2]));
            }
          }
        }
      }
    }
    if (zval && (!accumulate || hit)) {
      force[s] = acc0;
      force[D.N + s] = acc1;
      force[2 * D.N + s] = acc2;
    }
  }
}

// ---- Move kernels -----------------------------------------------------------
// Stencil nodes and Peskin weights of position r (interp.cu:23-30).  FP64
// lattices in exact mode keep the reference's arithmetic (a delta per node);
// the default FP64 moves (FAST) take the four weights of an axis from one
// square root; the FP32 path takes one FP64 difference per axis and forms the
// four arguments in FP32 (GB300's FP64 pipe is narrow).
template <class T, bool FAST = false>
__device__ __forceinline__ void interp_setup(const Dims& D, const double r[3], int idx[3][4],
                                             T phi[3][4]) {
  for (int d = 0; d < 3; ++d) {
    const double x0 = ceil(r[d] - 2.);
    const int o = wrap_any((int)x0, D.n[d]);
    T w[4];
    if constexpr (sizeof(T) == 4 || FAST) peskin_weights4((T)(r[d] - x0), w);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int t = o + i;
      while (t >= D.n[d]) t -= D.n[d];
      idx[d][i] = t;
      if constexpr (sizeof(T) == 8 && !FAST)
        phi[d][i] = peskin_delta<T>(r[d] - (x0 + i));
      else
        phi[d][i] = w[i];
    }
  }
}

// New periodic coordinate: the reference's fmod(r + size, size) on the FP64
// path (SwimmerArray.cu:167, TracerArray.cu:40), a compare-and-shift on the
// FP32 path (valid while a step moves a particle less than one box length).
template <class T>
__device__ __forceinline__ double wrap_position(double r, int n) {
  if constexpr (sizeof(T) == 8) {
    return fmod(r + n, (double)n);
  } else {
    return r >= n ? r - n : (r < 0.0 ? r + n : r);
  }
}

// InterpVelocity, interp.cu:8-47: u at r through the 4^3 Peskin stencil, from
// the FP64 SoA field (FAST: fused multiply-adds and one square root per axis,
// the default FP64 moves) ...
template <class T, bool FAST = false>
__device__ __forceinline__ void interp_velocity(const double* __restrict__ u, const Dims& D,
                                                const double r[3], T v[3]) {
  int idx[3][4];
  T phi[3][4];
  interp_setup<T, FAST>(D, r, idx, phi);
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
        if constexpr (FAST) {
          v[0] = fma(d3, (T)u[s], v[0]);
          v[1] = fma(d3, (T)u[D.N + s], v[1]);
          v[2] = fma(d3, (T)u[2 * D.N + s], v[2]);
        } else {
          v[0] = add_prod(v[0], d3, (T)u[s]);
          v[1] = add_prod(v[1], d3, (T)u[D.N + s]);
          v[2] = add_prod(v[2], d3, (T)u[2 * D.N + s]);
        }
      }
    }
}

// ... or from the packed float4 field of a reduced-precision lattice (one 16-byte
// load per node).
template <class T>
__device__ __forceinline__ void interp_velocity(const float4* __restrict__ h, const Dims& D,
                                                const double r[3], T v[3]) {
  int idx[3][4];
  T phi[3][4];
  interp_setup<T>(D, r, idx, phi);
  v[0] = v[1] = v[2] = T(0);
  const long long nynz = (long long)D.n[1] * D.n[2];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      const T pij = phi[0][i] * phi[1][j];
      const long long row = idx[0][i] * nynz + (long long)idx[1][j] * D.n[2];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const T d3 = pij * phi[2][k];
        const float4 q = __ldg(h + row + idx[2][k]);
        v[0] += d3 * (T)q.x;
        v[1] += d3 * (T)q.y;
        v[2] += d3 * (T)q.z;
      }
    }
}

// DoSwimmerArrayMove, SwimmerArray.cu:123-210 (FAST: the default FP64
// interpolation of interp_velocity).
template <class U, class T, bool FAST = false>
__global__ void k_swimmers_move(int nsw, double* __restrict__ swr, double* __restrict__ swv,
                                double* __restrict__ swn, lbswim_common_params c,
                                unsigned long long seed, unsigned long long step, Dims D,
                                const U* __restrict__ u, unsigned* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsw) return;
  double r[3], n0[3];
  for (int d = 0; d < 3; ++d) {
    r[d] = swr[nsw * d + i];
    n0[d] = swn[nsw * d + i];
  }
  T v[3];
  interp_velocity<T, FAST>(u, D, r, v);
  double rMinus[3];
  for (int d = 0; d < 3; ++d) {
    double rDot = __dmul_rn(__dmul_rn(c.mobility, c.P), n0[d]);
    if (!c.translational_advection_off) rDot = __dadd_rn(rDot, (double)v[d]);
    rMinus[d] = __dsub_rn(r[d], __dmul_rn(n0[d], c.l));
    swv[nsw * d + i] = rDot;
    const double rn = wrap_position<T>(r[d] + rDot, D.n[d]);
    swr[nsw * d + i] = rn;
    if (!in_box(rn, D.n[d])) raise_status(status, LBSWIM_STATUS_PARTICLE_OUTSIDE);
  }
  const float rnd = rng_uniform(seed, (uint32_t)i, step);
  double nn[3];
  if (rnd < c.alpha) {  // tumble: a direction uniform on the sphere
    rng_normal3(seed, (uint32_t)i, step, nn);
  } else if (!c.rotational_advection_off) {  // rotate with the local shear
    T vm[3];
    interp_velocity<T, FAST>(u, D, rMinus, vm);
    for (int d = 0; d < 3; ++d) nn[d] = n0[d] + ((double)v[d] - (double)vm[d]) / c.l;
  } else {
    return;  // orientation unchanged
  }
  const double norm = __dsqrt_rn(
      __dadd_rn(__dadd_rn(__dmul_rn(nn[0], nn[0]), __dmul_rn(nn[1], nn[1])), __dmul_rn(nn[2], nn[2])));
  for (int d = 0; d < 3; ++d) swn[nsw * d + i] = nn[d] / norm;
}

// DoTracerArrayMove, TracerArray.cu:12-43 (s accumulated per tracer; FAST: the
// default FP64 interpolation of interp_velocity).
template <class U, class T, bool FAST = false>
__global__ void k_tracers_move(int ntr, double* __restrict__ r, double* __restrict__ s,
                               double* __restrict__ v, Dims D, const U* __restrict__ u,
                               unsigned* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ntr) return;
  double rr[3], ss[3];
  for (int d = 0; d < 3; ++d) {
    rr[d] = r[ntr * d + i];
    ss[d] = s[ntr * d + i];
  }
  T vv[3];
  interp_velocity<T, FAST>(u, D, rr, vv);
  for (int d = 0; d < 3; ++d) {
    const double vd = (double)vv[d];
    v[ntr * d + i] = vd;
    const double rn = wrap_position<T>(rr[d] + vd, D.n[d]);
    r[ntr * d + i] = rn;
    s[ntr * d + i] = ss[d] + vd;
    if (!in_box(rn, D.n[d])) raise_status(status, LBSWIM_STATUS_PARTICLE_OUTSIDE);
  }
}

template <class U, class T>
__global__ void k_interp_points(int np, const double* __restrict__ r, double* __restrict__ v,
                                Dims D, const U* __restrict__ u) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const double rr[3] = {r[i], r[np + i], r[2 * np + i]};
  T vv[3];
  interp_velocity<T>(u, D, rr, vv);
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

// ---- seeded initial states made on the device ------------------------------------
// Counter streams keyed (seed, index) at steps far above any move step:
// INIT_STEP_SITE for densities, INIT_STEP_PART for particle positions and
// orientations (block 0: position uniforms, blocks 1-2: orientation normals).
constexpr unsigned long long INIT_STEP_SITE = 0xffffffffffff0001ull;
constexpr unsigned long long INIT_STEP_PART = 0xffffffffffff0002ull;

__global__ void k_init_density(long long N, unsigned long long seed, double amp, double rho0,
                               double* __restrict__ rho, double* __restrict__ u,
                               float4* __restrict__ hydro) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < N;
       s += (long long)gridDim.x * blockDim.x) {
    uint32_t x[4];
    rng_block(seed, (uint32_t)s, INIT_STEP_SITE, (uint32_t)(s >> 32), x);
    const double r = 1.0 + amp * (u53(x[0], x[1]) - 0x1.0p-53);  // 1 + amp U[0, 1)
    if (hydro) {
      hydro[s] = make_float4(0.f, 0.f, 0.f, (float)(r - rho0));
    } else {
      rho[s] = r;
      u[s] = u[N + s] = u[2 * N + s] = 0.0;
    }
  }
}

// Positions uniform in the box; orientations (when nv is set) uniform on the sphere.
__global__ void k_init_particles(int n, unsigned long long seed, Dims D, double* __restrict__ r,
                                 double* __restrict__ nv, double* __restrict__ zero_a,
                                 double* __restrict__ zero_b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t x[4];
  rng_block(seed, (uint32_t)i, INIT_STEP_PART, 0u, x);
  const double ux = u53(x[0], x[1]) - 0x1.0p-53, uy = u53(x[2], x[3]) - 0x1.0p-53;
  rng_block(seed, (uint32_t)i, INIT_STEP_PART, 3u, x);
  const double uz = u53(x[0], x[1]) - 0x1.0p-53;
  const double uu[3] = {ux, uy, uz};
  for (int d = 0; d < 3; ++d) {
    r[(long long)n * d + i] = uu[d] * D.n[d];
    if (zero_a) zero_a[(long long)n * d + i] = 0.0;
    if (zero_b) zero_b[(long long)n * d + i] = 0.0;
  }
  if (nv) {
    double g[3];
    rng_normal3(seed, (uint32_t)i, INIT_STEP_PART, g);
    const double norm = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(g[0], g[0]), __dmul_rn(g[1], g[1])),
                                             __dmul_rn(g[2], g[2])));
    for (int d = 0; d < 3; ++d) nv[(long long)n * d + i] = g[d] / norm;
  }
}

// ---- FP32-path Move kernels ------------------------------------------------------
// A block moves NP particles in three phases.  (1) One thread per particle forms
// its stencil -- wrapped origin node and Peskin weights -- in shared memory.
// (2) A group of 4 (or 8, 16) threads per interpolation point gathers the 4^3
// nodes, lane k taking z node k & 3, and the partial sums are added with a
// fixed shuffle tree, so the result does not depend on scheduling.  (3) One
// thread per particle updates it.  GB300's FP64 pipe is narrow: the stencil
// origin comes from the bits of the position by integer operations, positions
// advance in Q44 fixed point, and orientations update in FP32.

// Stencils of NP interpolation points in shared memory, one array per field so
// that one thread per point writes them without bank conflicts: wrapped origin
// node, whether the point is gathered, Peskin weights per axis and node.
template <int NP>
struct StencilSet {
  int o[3][NP];
  int active[NP];
  float w[3][4][NP];
};

// Exact FP64 value of a float, from its bits (no FP64 instruction).
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  const int e = (int)((u >> 23) & 0xffu);
  unsigned m = u & 0x7fffffu;
  if (e == 255)  // inf / nan
    return __longlong_as_double((long long)(sign | (0x7ffull << 52) | ((unsigned long long)m << 29)));
  if (e == 0) {
    if (m == 0) return __longlong_as_double((long long)sign);
    const int msb = 31 - __clz((int)m);  // subnormal: m * 2^-149
    const unsigned long long mant = ((unsigned long long)m << (52 - msb)) & 0xfffffffffffffull;
    return __longlong_as_double((long long)(sign | ((unsigned long long)(msb - 149 + 1023) << 52) | mant));
  }
  return __longlong_as_double(
      (long long)(sign | ((unsigned long long)(e + 896) << 52) | ((unsigned long long)m << 29)));
}

// Periodic coordinates as Q44 fixed point (44 fraction bits), for lattices
// shorter than 2^19 sites per axis.  pos_to_q44 takes 0 <= r < 2^19 (else
// returns false), rounding to nearest; q44_to_pos returns the FP64 nearest to
// q * 2^-44, q >= 0.  Integer operations only.
constexpr int Q44 = 44;
__device__ __forceinline__ bool pos_to_q44(double r, long long& q) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(r);
  const int ex = (int)(b >> 52);  // negative r gives ex >= 2048
  if (ex >= 1023 + 19) return false;
  if (ex < 1023 - Q44 - 2) {  // r < 2^-46 rounds to 0
    q = 0;
    return true;
  }
  const unsigned long long mant = (b & 0xfffffffffffffull) | (1ull << 52);
  const int sh = 1075 - Q44 - ex;  // q = mant * 2^-sh, -10 <= sh <= 55
  if (sh <= 0) {
    q = (long long)(mant << (-sh));
  } else {
    const unsigned long long rem = mant & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    unsigned long long v = mant >> sh;
    v += (rem > half || (rem == half && (v & 1ull))) ? 1ull : 0ull;
    q = (long long)v;
  }
  return true;
}
__device__ __forceinline__ double q44_to_pos(long long q) {
  if (q <= 0) return 0.0;
  const unsigned long long u = (unsigned long long)q;
  const int msb = 63 - __clzll((long long)u);
  int e = msb - Q44;
  unsigned long long m;
  if (msb <= 52) {
    m = u << (52 - msb);
  } else {
    const int sh = msb - 52;
    const unsigned long long rem = u & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    m = u >> sh;
    m += (rem > half || (rem == half && (m & 1ull))) ? 1ull : 0ull;
    if (m >> 53) {
      m >>= 1;
      ++e;
    }
  }
  return __longlong_as_double(
      (long long)(((unsigned long long)(e + 1023) << 52) | (m & 0xfffffffffffffull)));
}

// r + v moved back into [0, n) by one shift, like wrap_position<float>: in Q44
// when r and r + v allow it (the result then lies in the box by construction),
// else in FP64, where a result outside [0, n) -- a non-finite r or v, or a
// move longer than the box -- raises LBSWIM_STATUS_PARTICLE_OUTSIDE.
__device__ __forceinline__ double advance_position(double r, float v, int n, unsigned* status) {
  long long q;
  if (n < (1 << 19) && fabsf(v) < (float)n && pos_to_q44(r, q)) {
    q += fx_quant(v, 0x1.0p44f);
    const long long nq = (long long)n << Q44;
    q = q >= nq ? q - nq : (q < 0 ? q + nq : q);
    return q44_to_pos(q);
  }
  const double out = wrap_position<float>(r + f2d_exact(v), n);
  if (!in_box(out, n)) raise_status(status, LBSWIM_STATUS_PARTICLE_OUTSIDE);
  return out;
}

// The 53-bit uniform of rng_normal3 rounded to FP32 (relative error 2^-24 at
// every magnitude, so the logarithm of a small draw stays close to FP64's).
__device__ __forceinline__ float u53f(uint32_t a, uint32_t b) {
  const unsigned long long m = ((unsigned long long)a << 21) | (unsigned long long)(b >> 11);
  return __ull2float_rn(m + 1ull) * 0x1.0p-53f;
}

// -2 log u of that uniform in FP32; for u >= 1/2 through log1p of the exact
// 1 - u, so that draws near 1 keep their small logarithm.
__device__ __forceinline__ float neg2log_u53(uint32_t a, uint32_t b) {
  const unsigned long long m1 =
      (((unsigned long long)a << 21) | (unsigned long long)(b >> 11)) + 1ull;  // 1 .. 2^53
  if (m1 >= (1ull << 52))
    return -2.f * log1pf(-__ull2float_rn((1ull << 53) - m1) * 0x1.0p-53f);
  return -2.f * logf(__ull2float_rn(m1) * 0x1.0p-53f);
}

// Three normal deviates of a tumble in FP32 from the counter blocks and the
// uniforms of rng_normal3 (Box-Muller).
__device__ __forceinline__ void rng_normal3_f(uint64_t seed, uint32_t swimmer, uint64_t step,
                                              float g[3]) {
  uint32_t a[4], b[4];
  rng_block(seed, swimmer, step, 1u, a);
  rng_block(seed, swimmer, step, 2u, b);
  const float r1 = sqrtf(neg2log_u53(a[0], a[1]));
  const float r2 = sqrtf(neg2log_u53(b[0], b[1]));
  float s1, c1, s2, c2;
  sincospif(2.f * u53f(a[2], a[3]), &s1, &c1);
  sincospif(2.f * u53f(b[2], b[3]), &s2, &c2);
  g[0] = r1 * c1;
  g[1] = r1 * s1;
  g[2] = r2 * c2;
}

template <int NP>
__device__ __forceinline__ void point_stencil(const Dims& D, const double r[3],
                                              StencilSet<NP>& st, int p) {
  float dr[3];
  for (int d = 0; d < 3; ++d) {
    int x0;
    stencil_axis(r[d], x0, dr[d]);
    st.o[d][p] = wrap_any(x0, D.n[d]);
  }
  st.active[p] = 1;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    float w[4];
    peskin_weights4(dr[d], w);
#pragma unroll
    for (int j = 0; j < 4; ++j) st.w[d][j][p] = w[j];
  }
}

__device__ __forceinline__ int node_after(int o, int j, int n) {
  int t = o + j;
  while (t >= n) t -= n;
  return t;
}

// Sum over the L lanes of a point's group (fixed shuffle tree).
template <int L>
__device__ __forceinline__ void reduce_lanes(float& vx, float& vy, float& vz) {
#pragma unroll
  for (int off = L / 2; off > 0; off >>= 1) {
    vx += __shfl_xor_sync(0xffffffffu, vx, off);
    vy += __shfl_xor_sync(0xffffffffu, vy, off);
    vz += __shfl_xor_sync(0xffffffffu, vz, off);
  }
}

// Lane `sub` of the L lanes (4, 8 or 16) of a point gathers z node sub & 3 of
// y nodes sub >> 2, sub >> 2 + L / 4, ... for the four x nodes.  I is the type
// of the site offsets: int while N < 2^31.
template <int L, int NP, class I = int>
__device__ __forceinline__ void gather_point(const float4* __restrict__ h, const Dims& D,
                                             const StencilSet<NP>& s, int p, int sub,
                                             float& vx, float& vy, float& vz) {
  vx = vy = vz = 0.f;
  if (!s.active[p]) return;
  const int nz = D.n[2];
  const I nynz = (I)D.n[1] * D.n[2];
  const int kz = sub & 3;
  const int z = node_after(s.o[2][p], kz, nz);
  const float wz = s.w[2][kz][p];
  I xo[4];
  float wx[4];
#pragma unroll
  for (int ix = 0; ix < 4; ++ix) {
    xo[ix] = (I)node_after(s.o[0][p], ix, D.n[0]) * nynz;
    wx[ix] = s.w[0][ix][p];
  }
#pragma unroll
  for (int jy = sub >> 2; jy < 4; jy += L / 4) {
    const I yz = (I)node_after(s.o[1][p], jy, D.n[1]) * nz + z;
    const float wyz = s.w[1][jy][p] * wz;
#pragma unroll
    for (int ix = 0; ix < 4; ++ix) {
      const float4 q = __ldg(h + xo[ix] + yz);
      const float w = wx[ix] * wyz;
      vx += w * q.x;
      vy += w * q.y;
      vz += w * q.z;
    }
  }
}

// Phase 2: the block's threads, L per point and two points per group at a
// time, gather the velocity of the NP stencils.  Every thread runs the same
// number of iterations (NP * L is a multiple of 2 * blockDim).
template <int L, int NP, class I = int>
__device__ __forceinline__ void gather_block(const float4* __restrict__ h, const Dims& D,
                                             const StencilSet<NP>& st, float3* vel) {
  const int sub = threadIdx.x & (L - 1);
  const int groups = blockDim.x / L;
  for (int p = threadIdx.x / L; p < NP; p += 2 * groups) {
    float ax, ay, az, bx, by, bz;
    gather_point<L, NP, I>(h, D, st, p, sub, ax, ay, az);
    gather_point<L, NP, I>(h, D, st, p + groups, sub, bx, by, bz);
    reduce_lanes<L>(ax, ay, az);
    reduce_lanes<L>(bx, by, bz);
    if (sub == 0) {
      vel[p] = make_float3(ax, ay, az);
      vel[p + groups] = make_float3(bx, by, bz);
    }
  }
}

constexpr int TRACER_MOVE_BLOCK = 256;
constexpr int TRACER_LANES = 4;  // lanes per interpolation point

template <class I = int>
__device__ __forceinline__ void tracers_move_block(int blk, int ntr, double* __restrict__ r,
                                                   double* __restrict__ s,
                                                   double* __restrict__ v, Dims D,
                                                   const float4* __restrict__ h,
                                                   unsigned* status) {
  __shared__ StencilSet<TRACER_MOVE_BLOCK> st;
  __shared__ float3 vel[TRACER_MOVE_BLOCK];
  const int i = blk * TRACER_MOVE_BLOCK + threadIdx.x;
  const bool valid = i < ntr;
  // s is read with r, so the update at the end waits on no load of its own
  double rr[3] = {0.0, 0.0, 0.0}, ss[3] = {0.0, 0.0, 0.0};
  if (valid) {
    for (int d = 0; d < 3; ++d) {
      rr[d] = r[(long long)ntr * d + i];
      ss[d] = s[(long long)ntr * d + i];
    }
    point_stencil(D, rr, st, threadIdx.x);
  } else {
    st.active[threadIdx.x] = 0;
  }
  __syncthreads();
  gather_block<TRACER_LANES, TRACER_MOVE_BLOCK, I>(h, D, st, vel);
  __syncthreads();
  if (!valid) return;
  const float3 w = vel[threadIdx.x];
  const float vv[3] = {w.x, w.y, w.z};
  for (int d = 0; d < 3; ++d) {
    const double vd = f2d_exact(vv[d]);
    v[(long long)ntr * d + i] = vd;
    r[(long long)ntr * d + i] = advance_position(rr[d], vv[d], D.n[d], status);
    s[(long long)ntr * d + i] = ss[d] + vd;
  }
}

template <class I>
__global__ void __launch_bounds__(TRACER_MOVE_BLOCK) k_tracers_move_f32(
    int ntr, double* __restrict__ r, double* __restrict__ s, double* __restrict__ v, Dims D,
    const float4* __restrict__ h, unsigned* status) {
  tracers_move_block<I>(blockIdx.x, ntr, r, s, v, D, h, status);
}

// A block takes SWIMMERS_PER_BLOCK swimmers: two stencils (front and rear
// point) per swimmer, SWIMMER_LANES threads per stencil.
constexpr int SWIMMERS_PER_BLOCK = 64;
constexpr int SWIMMER_LANES = 4;  // lanes per interpolation point
constexpr int SWIMMER_MOVE_BLOCK = SWIMMERS_PER_BLOCK * SWIMMER_LANES;

// The update of swimmer i from the fluid velocity at its front point r (v)
// and at its rear point r - l n (vm): SwimmerArray.cu:151-209, with the FP32
// path's arithmetic (Q44 positions, FP32 turn added to the FP64 orientation,
// FP32 tumble normals).
__device__ __forceinline__ void swimmer_update(int i, int nsw, double* __restrict__ swr,
                                               double* __restrict__ swv, double* __restrict__ swn,
                                               const lbswim_common_params& c,
                                               unsigned long long seed, unsigned long long step,
                                               const Dims& D, const double r[3],
                                               const double nd[3], bool tumble, bool rotate,
                                               const float v[3], const float vm[3],
                                               unsigned* status) {
  const float mP = (float)(c.mobility * c.P);
  for (int d = 0; d < 3; ++d) {
    float rDot = mP * (float)nd[d];
    if (!c.translational_advection_off) rDot += v[d];
    swv[nsw * d + i] = f2d_exact(rDot);
    swr[nsw * d + i] = advance_position(r[d], rDot, D.n[d], status);
  }
  if (tumble) {
    float nn[3];
    rng_normal3_f(seed, (uint32_t)i, step, nn);
    const float inv = 1.f / sqrtf(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
    for (int d = 0; d < 3; ++d) swn[nsw * d + i] = f2d_exact(nn[d] * inv);
  } else if (rotate) {
    // the small turn (v - v_rear) / l is formed in FP32 and added to the FP64
    // orientation, which keeps its direction; the FP32 norm only rescales it
    const float inv_l = 1.f / (float)c.l;
    double nn[3];
    float sq = 0.f;
    for (int d = 0; d < 3; ++d) {
      nn[d] = __dadd_rn(nd[d], f2d_exact((v[d] - vm[d]) * inv_l));
      const float q = (float)nn[d];
      sq += q * q;
    }
    const double inv = f2d_exact(1.f / sqrtf(sq));
    for (int d = 0; d < 3; ++d) swn[nsw * d + i] = __dmul_rn(nn[d], inv);
  }
}

// The rear point r - l n of a swimmer, as the dipole-end records compute it.
__device__ __forceinline__ void rear_point(const double r[3], const double nd[3], double l,
                                           double out[3]) {
  for (int d = 0; d < 3; ++d) out[d] = __dsub_rn(r[d], __dmul_rn(nd[d], l));
}

template <class I = int>
__device__ __forceinline__ void swimmers_move_block(
    int blk, int nsw, double* __restrict__ swr, double* __restrict__ swv,
    double* __restrict__ swn, lbswim_common_params c, unsigned long long seed,
    unsigned long long step, Dims D, const float4* __restrict__ h, unsigned* status) {
  constexpr int B = SWIMMERS_PER_BLOCK;
  // stencils [0, B) at the swimmers, [B, 2B) at their rear points r - l n
  __shared__ StencilSet<2 * B> st;
  __shared__ float3 vel[2 * B];
  const int t = threadIdx.x, i = blk * B + t;
  const bool mine = t < B, valid = mine && i < nsw;
  double r[3] = {0.0, 0.0, 0.0}, nd[3] = {0.0, 0.0, 0.0};
  bool tumble = false, rotate = false;
  if (valid) {
    double rMinus[3];
    for (int d = 0; d < 3; ++d) {
      r[d] = swr[nsw * d + i];
      nd[d] = swn[nsw * d + i];
    }
    tumble = rng_uniform(seed, (uint32_t)i, step) < c.alpha;
    rotate = !tumble && !c.rotational_advection_off;
    point_stencil(D, r, st, t);
    if (rotate) {
      rear_point(r, nd, c.l, rMinus);
      point_stencil(D, rMinus, st, B + t);
    } else {
      st.active[B + t] = 0;
    }
  } else if (mine) {
    st.active[t] = 0;
    st.active[B + t] = 0;
  }
  __syncthreads();
  gather_block<SWIMMER_LANES, 2 * SWIMMERS_PER_BLOCK, I>(h, D, st, vel);
  __syncthreads();
  if (!valid) return;
  const float3 w = vel[t], wm = vel[B + t];
  const float v[3] = {w.x, w.y, w.z}, vm[3] = {wm.x, wm.y, wm.z};
  swimmer_update(i, nsw, swr, swv, swn, c, seed, step, D, r, nd, tumble, rotate, v, vm, status);
}

template <class I>
__global__ void __launch_bounds__(SWIMMER_MOVE_BLOCK) k_swimmers_move_f32(
    int nsw, double* __restrict__ swr, double* __restrict__ swv, double* __restrict__ swn,
    lbswim_common_params c, unsigned long long seed, unsigned long long step, Dims D,
    const float4* __restrict__ h, unsigned* status) {
  swimmers_move_block<I>(blockIdx.x, nsw, swr, swv, swn, c, seed, step, D, h, status);
}

// ---- batched ensembles: per-step reset, end records, moves --------------------
__device__ __forceinline__ int ens_find(const int* __restrict__ prefix, int nmem, int item) {
  int lo = 0, hi = nmem - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= item)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ Dims ens_dims(const EnsMember& M) {
  Dims D;
  for (int a = 0; a < 3; ++a) {
    D.n[a] = M.size[a];
    D.nb[a] = (M.size[a] + BIN - 1) / BIN;
  }
  D.N = M.n;
  return D;
}

// Advance the run's step counter (its own launch, so that every block of the
// step's kernels reads the same step index).
__global__ void k_ens_tick(EnsTable t) { *t.g_step += 1; }

// Zero the slab counts and largest |F| of every member still stepping, and
// the slab counter of this parity.

__global__ void k_ens_reset(EnsTable t, int parity) {
  const int nmem = *t.nmem;
  if (blockIdx.x == 0 && threadIdx.x == 0) t.counters[parity] = 0u;
  const long long g = *t.g_step;
  for (int m = blockIdx.x; m < nmem; m += gridDim.x) {
    const EnsMember& M = t.mem[m];
    if (g >= M.limit) continue;
    const int nslabs = M.nt[0] * M.nt[1] * M.nt[2];
    for (int i = threadIdx.x; i < nslabs; i += blockDim.x) M.bucket_count[i] = 0u;
    if (threadIdx.x == 0) *M.max_abs_f = 0u;
  }
}

__global__ void __launch_bounds__(REC_THREADS) k_ens_records(EnsTable t) {
  const int nmem = *t.nmem;
  const int total = t.rec_prefix[nmem];
  for (int vb = blockIdx.x; vb < total; vb += gridDim.x) {
    const int m = ens_find(t.rec_prefix, nmem, vb);
    const EnsMember& M = t.mem[m];
    if (*t.g_step >= M.limit) continue;
    TileGrid G;
    slab_shape_of_dev(M.tile, G.T);
    G.h = 1;
    for (int a = 0; a < 3; ++a) G.nt[a] = M.nt[a];
    end_records_block<float>(vb - t.rec_prefix[m], M.nsw, M.sw_r, M.sw_n, M.common.P,
                             M.common.l, ens_dims(M), (EndRecord<float>*)M.ends, 0, M.max_abs_f,
                             G, M.bucket_count, M.bucket_list);
    __syncthreads();
  }
}

static_assert(SWIMMER_MOVE_BLOCK == TRACER_MOVE_BLOCK, "one block size for both moves");
static_assert(ENS_ENDS_PER_BLOCK == REC_THREADS && ENS_SWIMMERS_PER_BLOCK == SWIMMERS_PER_BLOCK &&
                  ENS_TRACERS_PER_BLOCK == TRACER_MOVE_BLOCK,
              "batched work items per block");

__global__ void __launch_bounds__(TRACER_MOVE_BLOCK) k_ens_move(EnsTable t, int parity) {
  const int nmem = *t.nmem;
  const int nsb = t.sw_prefix[nmem], total = nsb + t.tr_prefix[nmem];
  const unsigned long long g = (unsigned long long)*t.g_step;
  for (int vb = blockIdx.x; vb < total; vb += gridDim.x) {
    if (vb < nsb) {
      const int m = ens_find(t.sw_prefix, nmem, vb);
      const EnsMember& M = t.mem[m];
      if ((long long)g >= M.limit) continue;  // uniform in the block: no barrier skipped
      swimmers_move_block(vb - t.sw_prefix[m], M.nsw, M.sw_r, M.sw_v, M.sw_n, M.common, M.seed,
                          M.step0 + g, ens_dims(M), (const float4*)M.hyd[parity], M.status);
    } else {
      const int m = ens_find(t.tr_prefix, nmem, vb - nsb);
      const EnsMember& M = t.mem[m];
      if ((long long)g >= M.limit) continue;
      tracers_move_block(vb - nsb - t.tr_prefix[m], M.ntr, M.tr_r, M.tr_s, M.tr_v, ens_dims(M),
                         (const float4*)M.hyd[parity], M.status);
    }
    __syncthreads();
  }
}

void ens_launch_reset(const EnsTable& t, int parity, cudaStream_t s) {
  k_ens_tick<<<1, 1, 0, s>>>(t);
  k_ens_reset<<<152, 256, 0, s>>>(t, parity);
  LB_CHECK_LAUNCH(2);
}
void ens_launch_records(const EnsTable& t, int grid, cudaStream_t s) {
  k_ens_records<<<grid, REC_THREADS, 0, s>>>(t);
  LB_CHECK_LAUNCH(1);
}
void ens_launch_move(const EnsTable& t, int parity, int grid, cudaStream_t s) {
  k_ens_move<<<grid, TRACER_MOVE_BLOCK, 0, s>>>(t, parity);
  LB_CHECK_LAUNCH(1);
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

static TileGrid force_tiles(const Lattice* L) {
  TileGrid G;
  G.T[0] = FT_X;
  G.T[1] = FT_Y;
  G.T[2] = FT_Z;
  G.h = 0;
  for (int a = 0; a < 3; ++a) G.nt[a] = (L->size[a] + G.T[a] - 1) / G.T[a];
  return G;
}

// Upper bound on the tile-list entries of one end: 4 + 2h consecutive sites per
// axis meet at most ceil((4 + 2h) / T) + 1 tiles, plus one more when they wrap
// around a partial last tile.
static long long touches_per_end(const TileGrid& G) {
  long long m = 1;
  for (int a = 0; a < 3; ++a)
    m *= std::min<long long>(G.nt[a], (4 + 2 * G.h + G.T[a] - 1) / G.T[a] + 2);
  return m;
}

static void free_lists(TileLists& TL) {
  void* ptrs[] = {TL.count, TL.start, TL.scan_tmp, TL.list, TL.sorted};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  TL = TileLists();
}

void spread_free(SpreadScratch& S) {
  {
    SpreadScratch::Prepared& P = S.prep;
    void* ptrs[] = {P.ends, P.bucket_count, P.bucket_list, P.max_abs_force};
    for (void* p : ptrs)
      if (p) cudaFree(p);
    P = SpreadScratch::Prepared();
  }
  if (S.ends) cudaFree(S.ends);
  if (S.max_abs_force) cudaFree(S.max_abs_force);
  if (S.bucket_count) cudaFree(S.bucket_count);
  if (S.bucket_list) cudaFree(S.bucket_list);
  S.ends = nullptr;
  S.max_abs_force = nullptr;
  S.bucket_count = nullptr;
  S.bucket_list = nullptr;
  S.bucket_slabs = 0;
  S.bucket_tile = -1;
  free_lists(S.ftiles);
}

static size_t record_bytes(const Lattice* L) {
  return L->precision == LBSWIM_F64 ? sizeof(EndRecord<double>) : sizeof(EndRecord<float>);
}

// Room for `total` pending ends, keeping the records already pending.
static void ensure_ends(Lattice* L, int total) {
  SpreadScratch& S = L->spread;
  const size_t rec = record_bytes(L);
  if (S.capacity_ends >= total && S.ends_bytes >= rec * (size_t)total) return;
  const int cap = std::max(total + total / 2, 64);
  void* fresh = nullptr;
  LB_CUDA(cudaMalloc(&fresh, rec * cap));
  if (S.ends && S.pending > 0)
    LB_CUDA(cudaMemcpyAsync(fresh, S.ends, rec * S.pending, cudaMemcpyDeviceToDevice, L->stream));
  LB_CUDA(cudaStreamSynchronize(L->stream));
  if (S.ends) cudaFree(S.ends);
  S.ends = fresh;
  S.capacity_ends = cap;
  S.ends_bytes = rec * cap;
}

static void ensure_lists(Lattice* L, TileLists& TL, const TileGrid& G, int nends) {
  const int ntiles = G.nt[0] * G.nt[1] * G.nt[2];
  if (TL.ntiles != ntiles) {
    LB_CUDA(cudaStreamSynchronize(L->stream));
    const long long keep = TL.capacity;
    int* keep_list = TL.list;
    int* keep_sorted = TL.sorted;
    if (TL.count) cudaFree(TL.count);
    if (TL.start) cudaFree(TL.start);
    if (TL.scan_tmp) cudaFree(TL.scan_tmp);
    TL.count = TL.start = TL.scan_tmp = nullptr;
    LB_CUDA(cudaMalloc(&TL.count, sizeof(unsigned) * ntiles));
    LB_CUDA(cudaMalloc(&TL.start, sizeof(unsigned) * (ntiles + 1)));
    const int nscan = (ntiles + SCAN_TILE - 1) / SCAN_TILE;
    LB_CUDA(cudaMalloc(&TL.scan_tmp, sizeof(unsigned) * std::max(nscan, 1)));
    LB_CUDA(cudaMemsetAsync(TL.count, 0, sizeof(unsigned) * ntiles, L->stream));
    TL.ntiles = ntiles;
    TL.capacity = keep;
    TL.list = keep_list;
    TL.sorted = keep_sorted;
  }
  const long long need = std::max<long long>((long long)nends * touches_per_end(G), 64);
  if (TL.capacity < need) {
    LB_CUDA(cudaStreamSynchronize(L->stream));
    if (TL.list) cudaFree(TL.list);
    if (TL.sorted) cudaFree(TL.sorted);
    TL.list = TL.sorted = nullptr;
    LB_CUDA(cudaMalloc(&TL.list, sizeof(int) * need));
    LB_CUDA(cudaMalloc(&TL.sorted, sizeof(int) * need));
    TL.capacity = need;
  }
}

// Lists of the pending ends per tile of G (entries unordered within a tile).
template <class T>
static void bin_ends(Lattice* L, TileLists& TL, const TileGrid& G) {
  const int nends = L->spread.pending;
  ensure_lists(L, TL, G, nends);
  const Dims D = make_dims(L);
  const EndRecord<T>* ends = (const EndRecord<T>*)L->spread.ends;
  if (nends > 0) {
    k_touch<T, 0><<<(nends + 255) / 256, 256, 0, L->stream>>>(nends, ends, D, G, TL.count,
                                                              nullptr, nullptr);
    LB_CHECK_LAUNCH(1);
  }
  const int nscan = (TL.ntiles + SCAN_TILE - 1) / SCAN_TILE;
  k_scan_tiles<<<nscan, SCAN_THREADS, 0, L->stream>>>(TL.count, TL.ntiles, TL.scan_tmp);
  k_scan_top<<<1, 1024, 0, L->stream>>>(TL.scan_tmp, nscan);
  k_scan_apply_total<<<nscan, SCAN_THREADS, 0, L->stream>>>(TL.count, TL.ntiles, TL.scan_tmp,
                                                            TL.start);
  LB_CHECK_LAUNCH(3);
  if (nends > 0) {
    k_touch<T, 1><<<(nends + 255) / 256, 256, 0, L->stream>>>(nends, ends, D, G, TL.count,
                                                              TL.start, TL.list);
    LB_CHECK_LAUNCH(1);
  }
}

// Fold the pending ends of an FP64 lattice into the dense force buffer
// (force = base + spread).
static void materialise_f64(Lattice* L) {
  SpreadScratch& S = L->spread;
  const TileGrid G = force_tiles(L);
  bin_ends<double>(L, S.ftiles, G);
  const Dims D = make_dims(L);
  k_force_tile<<<S.ftiles.ntiles, FT_THREADS, 0, L->stream>>>(
      D, G, (const EndRecord<double>*)S.ends, S.ftiles.start, S.ftiles.list, S.ftiles.sorted,
      (double*)L->force, L->force_zero_pending ? 0 : 1);
  LB_CHECK_LAUNCH(1);
  S.pending = 0;
  S.stepped = false;
  L->force_zero_pending = false;
}

void spread_materialise(Lattice* L) {
  if (L->spread.pending > 0) {
    if (L->precision == LBSWIM_F64) {
      materialise_f64(L);
    } else {
      lattice_force_from_slabs(L);
      L->spread.pending = 0;
      L->spread.stepped = false;
      L->force_zero_pending = false;
    }
  } else if (L->force_zero_pending) {
    lattice_zero_force_now(L);
  }
}

static TileGrid slab_grid(const Lattice* L) {
  TileGrid G;
  fused_slab_shape(L, G.T);
  G.h = 1;  // the step kernel collides a one-site ring around its slab
  for (int a = 0; a < 3; ++a) G.nt[a] = (L->size[a] + G.T[a] - 1) / G.T[a];
  return G;
}

// Bucket storage for the current slab grid; false when it had to be replaced
// (the buckets are then stale).
static bool ensure_buckets(Lattice* L) {
  SpreadScratch& S = L->spread;
  const TileGrid G = slab_grid(L);
  const int nslabs = G.nt[0] * G.nt[1] * G.nt[2];
  if (S.bucket_slabs == nslabs && S.bucket_count) return true;
  LB_CUDA(cudaStreamSynchronize(L->stream));
  if (S.bucket_count) cudaFree(S.bucket_count);
  if (S.bucket_list) cudaFree(S.bucket_list);
  S.bucket_count = nullptr;
  S.bucket_list = nullptr;
  LB_CUDA(cudaMalloc(&S.bucket_count, sizeof(unsigned) * nslabs));
  LB_CUDA(cudaMalloc(&S.bucket_list, sizeof(int) * (size_t)nslabs * SLAB_BUCKET_CAP));
  S.bucket_slabs = nslabs;
  S.bucket_tile = -1;
  return false;
}

void spread_reserve(Lattice* L, int nends) {
  ensure_ends(L, nends);
  SpreadScratch& S = L->spread;
  if (!S.max_abs_force) LB_CUDA(cudaMalloc(&S.max_abs_force, sizeof(unsigned)));
  ensure_buckets(L);
}

SlabSpread spread_prepare_slabs(Lattice* L) {
  SpreadScratch& S = L->spread;
  if (!ensure_buckets(L) || S.bucket_tile != L->fused_tile) {
    const TileGrid G = slab_grid(L);
    LB_CUDA(cudaMemsetAsync(S.bucket_count, 0, sizeof(unsigned) * S.bucket_slabs, L->stream));
    if (S.pending > 0) {
      k_bucket_ends<<<(S.pending + 255) / 256, 256, 0, L->stream>>>(
          S.pending, (const EndRecord<float>*)S.ends, make_dims(L), G, S.bucket_count,
          S.bucket_list);
      LB_CHECK_LAUNCH(1);
    }
    S.bucket_tile = L->fused_tile;
  }
  SlabSpread out;
  out.ends = S.ends;
  out.count = S.bucket_count;
  out.list = S.bucket_list;
  out.npending = S.pending;
  out.max_abs_force = S.max_abs_force;
  return out;
}

template <class T>
static void append_ends_t(Swimmers* W, Lattice* L) {
  SpreadScratch& S = L->spread;
  const int nends = 2 * W->n;
  ensure_ends(L, S.pending + nends);
  if (!S.max_abs_force) LB_CUDA(cudaMalloc(&S.max_abs_force, sizeof(unsigned)));
  // reduced-precision lattices list the ends under the step kernel's slabs now
  constexpr bool BUCKETS = sizeof(T) == 4;
  bool fill = false;
  if (BUCKETS) {
    const bool kept = ensure_buckets(L);
    if (S.pending == 0) {
      LB_CUDA(cudaMemsetAsync(S.bucket_count, 0, sizeof(unsigned) * S.bucket_slabs, L->stream));
      S.bucket_tile = L->fused_tile;
    } else if (!kept) {
      S.bucket_tile = -1;
    }
    fill = S.bucket_tile == L->fused_tile;
  }
  if (S.pending == 0) LB_CUDA(cudaMemsetAsync(S.max_abs_force, 0, sizeof(unsigned), L->stream));
  if (nends > 0) {
    k_end_records<T><<<(nends + REC_THREADS - 1) / REC_THREADS, REC_THREADS, 0, L->stream>>>(
        W->n, W->r, W->nv, W->common.P, W->common.l, make_dims(L),
        (EndRecord<T>*)S.ends + S.pending, S.pending, S.max_abs_force, slab_grid(L),
        fill ? S.bucket_count : nullptr, fill ? S.bucket_list : nullptr);
    LB_CHECK_LAUNCH(1);
  }
  S.pending += nends;
}

// 64-bit site offsets in the FP32 move kernels: when 32-bit ones would
// overflow, or when the lattice asks for them (LBSWIM_COMPAT_WIDE_INDEX).
static bool wide_particle_index(const Lattice* L) {
  return L->n >= (1ll << 31) || (L->compat & LBSWIM_COMPAT_WIDE_INDEX);
}

static void swimmers_mark(Swimmers* W, cudaStream_t stream) {
  if (!W->done) LB_CUDA(cudaEventCreateWithFlags(&W->done, cudaEventDisableTiming));
  LB_CUDA(cudaEventRecord(W->done, stream));
}

void swimmers_wait(Swimmers* W) {
  if (W->done) LB_CUDA(cudaEventSynchronize(W->done));
}

// SwimmerArray::AddForces (SwimmerArray.cu:114-121).
void swimmers_add_forces(Swimmers* W, Lattice* L) {
  // ends already spread by a Step belong to the base from now on
  if (L->spread.stepped) spread_materialise(L);
  if (L->precision == LBSWIM_F64) {
    append_ends_t<double>(W, L);
    spread_materialise(L);
  } else {
    append_ends_t<float>(W, L);
  }
  swimmers_mark(W, L->stream);
  L->force_version++;
}

void swimmers_move(Swimmers* W, Lattice* L) {
  const Dims D = make_dims(L);
  if (W->n > 0) {
    const int grid = (W->n + 255) / 256;
    if (L->precision == LBSWIM_F64 && (L->compat & LBSWIM_COMPAT_EXACT_F64))
      k_swimmers_move<double, double><<<grid, 256, 0, L->stream>>>(
          W->n, W->r, W->v, W->nv, W->common, W->seed, W->step, D, (const double*)L->u,
          L->status);
    else if (L->precision == LBSWIM_F64)
      k_swimmers_move<double, double, true><<<grid, 256, 0, L->stream>>>(
          W->n, W->r, W->v, W->nv, W->common, W->seed, W->step, D, (const double*)L->u,
          L->status);
    else if (wide_particle_index(L))
      k_swimmers_move_f32<long long><<<(W->n + SWIMMERS_PER_BLOCK - 1) / SWIMMERS_PER_BLOCK,
                                       SWIMMER_MOVE_BLOCK, 0, L->stream>>>(
          W->n, W->r, W->v, W->nv, W->common, W->seed, W->step, D, (const float4*)L->hydro,
          L->status);
    else
      k_swimmers_move_f32<int><<<(W->n + SWIMMERS_PER_BLOCK - 1) / SWIMMERS_PER_BLOCK,
                                 SWIMMER_MOVE_BLOCK, 0, L->stream>>>(
          W->n, W->r, W->v, W->nv, W->common, W->seed, W->step, D, (const float4*)L->hydro,
          L->status);
    LB_CHECK_LAUNCH(1);
    swimmers_mark(W, L->stream);
  }
  W->step++;
}

// The move of lbswim_system_step with one swimmer array: on reduced-precision
// lattices it is followed by the records and slab buckets of the moved
// swimmers' ends, made into the lattice's prepared set, which the next step's
// AddForces takes if nothing changed in between (swimmers_add_forces_prepared).
// A read-back of the swimmers waits for the move only; an upload also waits
// for these records.
void swimmers_move_preparing(Swimmers* W, Lattice* L, unsigned long long epoch) {
  SpreadScratch::Prepared& P = L->spread.prep;
  P.valid = false;
  swimmers_move(W, L);
  if (W->n <= 0 || L->precision == LBSWIM_F64) return;
  const TileGrid G = slab_grid(L);
  const int nslabs = G.nt[0] * G.nt[1] * G.nt[2];
  const int nends = 2 * W->n;
  const size_t rec = sizeof(EndRecord<float>);
  if (P.capacity_ends < nends || P.bucket_slabs != nslabs || !P.max_abs_force) {
    // the buffers may still be read by earlier work on the stream
    LB_CUDA(cudaStreamSynchronize(L->stream));
    if (P.capacity_ends < nends) {
      if (P.ends) cudaFree(P.ends);
      P.ends = nullptr;
      P.capacity_ends = 0;
      const int cap = std::max(nends + nends / 2, 64);
      LB_CUDA(cudaMalloc(&P.ends, rec * cap));
      P.capacity_ends = cap;
      P.ends_bytes = rec * cap;
    }
    if (P.bucket_slabs != nslabs) {
      if (P.bucket_count) cudaFree(P.bucket_count);
      if (P.bucket_list) cudaFree(P.bucket_list);
      P.bucket_count = nullptr;
      P.bucket_list = nullptr;
      P.bucket_slabs = 0;
      LB_CUDA(cudaMalloc(&P.bucket_count, sizeof(unsigned) * nslabs));
      LB_CUDA(cudaMalloc(&P.bucket_list, sizeof(int) * (size_t)nslabs * SLAB_BUCKET_CAP));
      P.bucket_slabs = nslabs;
    }
    if (!P.max_abs_force) LB_CUDA(cudaMalloc(&P.max_abs_force, sizeof(unsigned)));
  }
  LB_CUDA(cudaMemsetAsync(P.bucket_count, 0, sizeof(unsigned) * nslabs, L->stream));
  LB_CUDA(cudaMemsetAsync(P.max_abs_force, 0, sizeof(unsigned), L->stream));
  k_end_records<float><<<(nends + REC_THREADS - 1) / REC_THREADS, REC_THREADS, 0, L->stream>>>(
      W->n, W->r, W->nv, W->common.P, W->common.l, make_dims(L), (EndRecord<float>*)P.ends, 0,
      P.max_abs_force, G, P.bucket_count, P.bucket_list);
  LB_CHECK_LAUNCH(1);
  if (!W->recorded) LB_CUDA(cudaEventCreateWithFlags(&W->recorded, cudaEventDisableTiming));
  LB_CUDA(cudaEventRecord(W->recorded, L->stream));
  P.valid = true;
  P.owner = W;
  P.owner_step = W->step;
  P.epoch = epoch;
  P.tile = L->fused_tile;
  P.nends = nends;
}

// AddForces of W (right after ZeroForce) from the prepared set, when the last
// thing that happened to W and to this lattice was that preparing move.
bool swimmers_add_forces_prepared(Swimmers* W, Lattice* L, unsigned long long epoch) {
  SpreadScratch& S = L->spread;
  SpreadScratch::Prepared& P = S.prep;
  if (!P.valid || P.owner != W || P.owner_step != W->step || P.epoch != epoch ||
      P.tile != L->fused_tile || L->precision == LBSWIM_F64 || S.pending != 0 || S.stepped ||
      P.nends != 2 * W->n)
    return false;
  const TileGrid G = slab_grid(L);
  if (P.bucket_slabs != G.nt[0] * G.nt[1] * G.nt[2]) return false;
  std::swap(S.ends, P.ends);
  std::swap(S.ends_bytes, P.ends_bytes);
  std::swap(S.capacity_ends, P.capacity_ends);
  std::swap(S.bucket_count, P.bucket_count);
  std::swap(S.bucket_list, P.bucket_list);
  std::swap(S.bucket_slabs, P.bucket_slabs);
  std::swap(S.max_abs_force, P.max_abs_force);
  S.bucket_tile = L->fused_tile;
  S.pending = P.nends;
  P.valid = false;
  swimmers_mark(W, L->stream);
  L->force_version++;
  return true;
}

// ---- tracer work order ------------------------------------------------------------
// Tracer cells of 4 x 4 x 8 sites, z fastest: a block's 256 tracers lie in a
// 4 x 4 x 256 run along z, whose stencil rows share more cache lines than a
// cube's (3 us per coupled step less than 8 x 8 x 8 cells at 256^3).
constexpr int TR_BINX = 4, TR_BINY = 4, TR_BINZ = 8;

__global__ void k_tr_bin(int n, const double* __restrict__ r, Dims D, int nb1, int nb2,
                         int* __restrict__ bin_of, unsigned* __restrict__ count) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  int c[3];
  for (int d = 0; d < 3; ++d)
    c[d] = wrap_any((int)floor(r[n * d + k]), D.n[d]) / (d == 0 ? TR_BINX : d == 1 ? TR_BINY : TR_BINZ);
  const int b = (c[0] * nb1 + c[1]) * nb2 + c[2];
  bin_of[k] = b;
  atomicAdd(count + b, 1u);
}

__global__ void k_tr_permute(int n, const int* __restrict__ bin_of, unsigned* __restrict__ count,
                             const unsigned* __restrict__ start, const double* __restrict__ r,
                             const double* __restrict__ s, const double* __restrict__ v,
                             const int* __restrict__ perm, double* __restrict__ r2,
                             double* __restrict__ s2, double* __restrict__ v2,
                             int* __restrict__ perm2) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int b = bin_of[k];
  const unsigned slot = start[b] + atomicSub(count + b, 1u) - 1u;
  for (int d = 0; d < 3; ++d) {
    r2[(long long)n * d + slot] = r[(long long)n * d + k];
    s2[(long long)n * d + slot] = s[(long long)n * d + k];
    v2[(long long)n * d + slot] = v[(long long)n * d + k];
  }
  perm2[slot] = perm[k];
}

__global__ void k_iota(int n, int* __restrict__ p) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) p[k] = k;
}

// dst[d][k] = src[d][perm[k]] (user order -> work order) or the inverse.
template <bool TO_WORK>
__global__ void k_tr_reorder(int n, const int* __restrict__ perm, const double* __restrict__ src,
                             double* __restrict__ dst) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int u = perm[k];
  for (int d = 0; d < 3; ++d) {
    if (TO_WORK)
      dst[(long long)n * d + k] = src[(long long)n * d + u];
    else
      dst[(long long)n * d + u] = src[(long long)n * d + k];
  }
}

// Any non-finite value among n doubles sets *flag.
__global__ void k_any_nonfinite(const double* __restrict__ a, long long n,
                                unsigned* __restrict__ flag) {
  unsigned bad = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    bad |= !(fabs(a[i]) <= 1.7976931348623157e308);
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1u);
}

// The check runs on the device, on the uploaded copy: a host scan of the
// caller's buffer by one core reads it several times slower than the link
// delivers it (1M tracer positions: ~1.2 ms against 0.12 ms for the copy).
void upload_checked_finite(double* stage, const double* host, long long n, unsigned* flag,
                           const char* what) {
  if (n <= 0) return;
  LB_CUDA(cudaMemcpy(stage, host, sizeof(double) * n, cudaMemcpyHostToDevice));
  LB_CUDA(cudaMemset(flag, 0, sizeof(unsigned)));
  const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 8);
  k_any_nonfinite<<<(int)blocks, 256>>>(stage, n, flag);
  LB_CHECK_LAUNCH(1);
  unsigned bad = 0;
  LB_CUDA(cudaMemcpy(&bad, flag, sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (bad) throw LbswimError{LBSWIM_EINVAL, std::string(what) + " holds a non-finite value"};
}

void tracers_alloc(Tracers* T) {
  const size_t n = (size_t)(T->n > 0 ? T->n : 1);
  double** bufs[] = {&T->r, &T->s, &T->v, &T->r2, &T->s2, &T->v2, &T->staging};
  for (double** b : bufs) {
    LB_CUDA(cudaMalloc(b, sizeof(double) * 3 * n));
    LB_CUDA(cudaMemset(*b, 0, sizeof(double) * 3 * n));
  }
  LB_CUDA(cudaMalloc(&T->perm, sizeof(int) * n));
  LB_CUDA(cudaMalloc(&T->perm2, sizeof(int) * n));
  LB_CUDA(cudaMalloc(&T->bin_of, sizeof(int) * n));
  LB_CUDA(cudaMalloc(&T->flag, 256));
  k_iota<<<(int)((n + 255) / 256), 256>>>((int)n, T->perm);
  LB_CHECK_LAUNCH(1);
  LB_CUDA(cudaDeviceSynchronize());
}

void tracers_free(Tracers* T) {
  if (T->side) {
    cudaStreamSynchronize(T->side);
    cudaStreamDestroy(T->side);
    cudaEventDestroy(T->done);
    T->side = nullptr;
  }
  void* ptrs[] = {T->r,    T->s,      T->v,      T->r2,        T->s2,        T->v2,
                  T->perm, T->perm2,  T->bin_of, T->staging,   T->bin_count, T->bin_start,
                  T->scan_tmp, T->flag};
  for (void* p : ptrs)
    if (p) cudaFree(p);
}

static double* tr_field_ptr(Tracers* T, int field) {
  return field == LBSWIM_TR_R ? T->r : (field == LBSWIM_TR_S ? T->s : T->v);
}

void tracers_h2d(Tracers* T, int field, const double* host) {
  LB_CUDA(cudaDeviceSynchronize());  // particle arrays are not bound to one stream
  if (T->n <= 0) return;
  double* dst = tr_field_ptr(T, field);
  const size_t bytes = sizeof(double) * 3 * T->n;
  // positions must be finite: checked on the staged copy, before the field
  // changes
  const bool check = field == LBSWIM_TR_R;
  if (check)
    upload_checked_finite(T->staging, host, 3LL * T->n, T->flag, "tracer positions");
  if (T->identity) {
    if (check) {
      LB_CUDA(cudaMemcpyAsync(dst, T->staging, bytes, cudaMemcpyDeviceToDevice, 0));
      LB_CUDA(cudaStreamSynchronize(0));
    } else {
      LB_CUDA(cudaMemcpy(dst, host, bytes, cudaMemcpyHostToDevice));
    }
  } else {
    if (!check) LB_CUDA(cudaMemcpy(T->staging, host, bytes, cudaMemcpyHostToDevice));
    k_tr_reorder<true><<<(T->n + 255) / 256, 256>>>(T->n, T->perm, T->staging, dst);
    LB_CHECK_LAUNCH(1);
    LB_CUDA(cudaDeviceSynchronize());
  }
  if (field == LBSWIM_TR_R) T->needs_sort = true;
}

void tracers_d2h(Tracers* T, int field, double* host) {
  LB_CUDA(cudaDeviceSynchronize());
  if (T->n <= 0) return;
  const double* src = tr_field_ptr(T, field);
  if (T->identity) {
    LB_CUDA(cudaMemcpy(host, src, sizeof(double) * 3 * T->n, cudaMemcpyDeviceToHost));
  } else {
    k_tr_reorder<false><<<(T->n + 255) / 256, 256>>>(T->n, T->perm, src, T->staging);
    LB_CHECK_LAUNCH(1);
    LB_CUDA(cudaMemcpy(host, T->staging, sizeof(double) * 3 * T->n, cudaMemcpyDeviceToHost));
  }
}

static void tracers_sort(Tracers* T, Lattice* L, cudaStream_t stream) {
  const Dims D = make_dims(L);
  const int nb0 = (D.n[0] + TR_BINX - 1) / TR_BINX, nb1 = (D.n[1] + TR_BINY - 1) / TR_BINY,
            nb2 = (D.n[2] + TR_BINZ - 1) / TR_BINZ;
  const int nbins = nb0 * nb1 * nb2;
  if (T->nbins != nbins) {
    LB_CUDA(cudaStreamSynchronize(stream));
    if (T->bin_count) cudaFree(T->bin_count);
    if (T->bin_start) cudaFree(T->bin_start);
    if (T->scan_tmp) cudaFree(T->scan_tmp);
    T->bin_count = T->bin_start = T->scan_tmp = nullptr;
    LB_CUDA(cudaMalloc(&T->bin_count, sizeof(unsigned) * nbins));
    LB_CUDA(cudaMalloc(&T->bin_start, sizeof(unsigned) * (nbins + 1)));
    LB_CUDA(cudaMalloc(&T->scan_tmp, sizeof(unsigned) * ((nbins + SCAN_TILE - 1) / SCAN_TILE)));
    LB_CUDA(cudaMemsetAsync(T->bin_count, 0, sizeof(unsigned) * nbins, stream));
    T->nbins = nbins;
  }
  const int g = (T->n + 255) / 256;
  k_tr_bin<<<g, 256, 0, stream>>>(T->n, T->r, D, nb1, nb2, T->bin_of, T->bin_count);
  const int nscan = (nbins + SCAN_TILE - 1) / SCAN_TILE;
  k_scan_tiles<<<nscan, SCAN_THREADS, 0, stream>>>(T->bin_count, nbins, T->scan_tmp);
  k_scan_top<<<1, 1024, 0, stream>>>(T->scan_tmp, nscan);
  k_scan_apply<<<nscan, SCAN_THREADS, 0, stream>>>(T->bin_count, nbins, T->scan_tmp,
                                                      T->bin_start, (unsigned)T->n);
  k_tr_permute<<<g, 256, 0, stream>>>(T->n, T->bin_of, T->bin_count, T->bin_start, T->r,
                                         T->s, T->v, T->perm, T->r2, T->s2, T->v2, T->perm2);
  LB_CHECK_LAUNCH(5);
  std::swap(T->r, T->r2);
  std::swap(T->s, T->s2);
  std::swap(T->v, T->v2);
  std::swap(T->perm, T->perm2);
  T->identity = false;
  T->needs_sort = false;
  T->moves_since_sort = 0;
}

static void tracers_move_on(Tracers* T, Lattice* L, cudaStream_t stream) {
  if (T->needs_sort || T->moves_since_sort >= TRACER_RESORT_MOVES) tracers_sort(T, L, stream);
  T->moves_since_sort++;
  const Dims D = make_dims(L);
  const int grid = (T->n + 255) / 256;
  if (L->precision == LBSWIM_F64 && (L->compat & LBSWIM_COMPAT_EXACT_F64))
    k_tracers_move<double, double><<<grid, 256, 0, stream>>>(T->n, T->r, T->s, T->v, D,
                                                                 (const double*)L->u, L->status);
  else if (L->precision == LBSWIM_F64)
    k_tracers_move<double, double, true><<<grid, 256, 0, stream>>>(
        T->n, T->r, T->s, T->v, D, (const double*)L->u, L->status);
  else if (wide_particle_index(L))
    k_tracers_move_f32<long long><<<(T->n + TRACER_MOVE_BLOCK - 1) / TRACER_MOVE_BLOCK,
                                    TRACER_MOVE_BLOCK, 0, stream>>>(T->n, T->r, T->s, T->v, D,
                                                                    L->hydro, L->status);
  else
    k_tracers_move_f32<int><<<(T->n + TRACER_MOVE_BLOCK - 1) / TRACER_MOVE_BLOCK,
                              TRACER_MOVE_BLOCK, 0, stream>>>(T->n, T->r, T->s, T->v, D,
                                                              L->hydro, L->status);
  LB_CHECK_LAUNCH(1);
}

void tracers_move(Tracers* T, Lattice* L) {
  if (T->n <= 0) return;
  if (T->side_pending) LB_CUDA(cudaStreamWaitEvent(L->stream, T->done, 0));
  tracers_move_on(T, L, L->stream);
}

void tracers_move_async(Tracers* T, Lattice* L) {
  if (T->n <= 0) return;
  if (!T->side) {
    // Least priority: when the lattice's stream has a higher one, the next
    // step's blocks are dispatched ahead of tracer blocks still queued, and the
    // tracer move fills the SMs the step leaves idle.
    int least = 0, greatest = 0;
    LB_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    LB_CUDA(cudaStreamCreateWithPriority(&T->side, cudaStreamNonBlocking, least));
    LB_CUDA(cudaEventCreateWithFlags(&T->done, cudaEventDisableTiming));
  }
  LB_CUDA(cudaStreamWaitEvent(T->side, L->hydro_ready, 0));
  tracers_move_on(T, L, T->side);
  LB_CUDA(cudaEventRecord(T->done, T->side));
  T->side_pending = true;
  cudaEvent_t ev;
  if (L->reader_pool.empty()) {
    LB_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  } else {
    ev = L->reader_pool.back();
    L->reader_pool.pop_back();
  }
  LB_CUDA(cudaEventRecord(ev, T->side));
  L->readers.emplace_back(L->precision == LBSWIM_F64 ? (const void*)L->u : (const void*)L->hydro, ev);
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
      k_interp_points<float4, float><<<(np + 255) / 256, 256, 0, L->stream>>>(np, r, v, D,
                                                                             L->hydro);
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
  // Every limit is checked before anything is enqueued (the swimmer count
  // before it is doubled, so that no count can wrap past the check).
  if (nsw < 0 || nsw > LBSWIM_NOALLOC_MAX_SWIMMERS)
    throw LbswimError{LBSWIM_EINVAL, "swimmer count outside the allocation-free limit of 0.." +
                                         std::to_string(LBSWIM_NOALLOC_MAX_SWIMMERS)};
  if (nbins > NOALLOC_MAX_BINS)
    throw LbswimError{LBSWIM_EINVAL,
                      "lattice larger than the allocation-free limit (" +
                          std::to_string(NOALLOC_MAX_BINS) + " spread bins of 4^3 sites)"};
  // the gather's grid is (ceil(nz / 32), ceil(ny / 8), nx) blocks
  if (D.n[0] > 65535 || (D.n[1] + 7) / 8 > 65535)
    throw LbswimError{LBSWIM_EINVAL, "lattice axes beyond the allocation-free limit "
                                     "(nx <= 65535, ny <= 524280)"};
  const int nends = 2 * nsw;
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

void lattice_init_random(Lattice* L, unsigned long long seed, double amp) {
  const bool packed = L->precision != LBSWIM_F64;
  if (packed) L->rho0 = 1.0;  // as a new lattice: the same stored bits whatever came before
  k_init_density<<<(int)std::min<long long>((L->n + 255) / 256, 152LL * 32), 256, 0, L->stream>>>(
      L->n, seed, amp, L->rho0, packed ? nullptr : (double*)L->rho,
      packed ? nullptr : (double*)L->u, packed ? L->hydro : nullptr);
  LB_CHECK_LAUNCH(1);
  L->shadow_f_version = 0;
  lattice_init_from_hydro(L);
}

void swimmers_init_random(Swimmers* W, const Lattice* L, unsigned long long seed) {
  LB_CUDA(cudaDeviceSynchronize());
  if (W->n > 0) {
    k_init_particles<<<(W->n + 255) / 256, 256>>>(W->n, seed, make_dims(L), W->r, W->nv, W->v,
                                                   nullptr);
    LB_CHECK_LAUNCH(1);
  }
  LB_CUDA(cudaDeviceSynchronize());
}

void tracers_init_random(Tracers* T, const Lattice* L, unsigned long long seed) {
  LB_CUDA(cudaDeviceSynchronize());
  if (T->n > 0) {
    // user order = work order until the next re-binning
    k_iota<<<(T->n + 255) / 256, 256>>>(T->n, T->perm);
    k_init_particles<<<(T->n + 255) / 256, 256>>>(T->n, seed, make_dims(L), T->r, nullptr, T->s,
                                                   T->v);
    LB_CHECK_LAUNCH(2);
    T->identity = true;
    T->needs_sort = true;
    T->moves_since_sort = 0;
  }
  LB_CUDA(cudaDeviceSynchronize());
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
