// spread_slab.cuh -- spreading the pending dipole ends of one slab into
// fixed-point force sums, one x plane at a time, in shared memory.
//
// A slab is SLAB_LX x planes by TY rows (y) by TZ columns (z) of the lattice,
// plus H sites on every side (H = 1 for the step kernel, which collides a ring
// around its cross-section; H = 0 for the force kernel).  Its ends come from
// the slab buckets filled when the ends were recorded.  For every local plane
// the (end, (jy, jz) node) pairs that fall on it are quantised to 32-bit
// integers and added into exact integer sums per site and component, kept as
// two 32-bit words so that the additions are native shared-memory atomics; a
// sum does not depend on the order of its additions, so the force is
// deterministic.  While a site can take at most 65535 contributions (the usual
// case) a contribution q goes in as its low 16 bits (unsigned) and q >> 16 with
// two atomics that return nothing; otherwise as a 64-bit sum whose high word
// takes the carries of the low one.
#pragma once
#include "lbswim_device.cuh"
#include "lbswim_internal.h"

namespace lbswim {

constexpr int SLAB_LX = 32;                // x planes per slab
constexpr int SPREAD_CAP = 256;            // ends of one slab held in shared memory
constexpr int SPREAD_PLANES_PER_END = 8;   // local planes one end can cover (6 at most)
constexpr unsigned PL_FOLD = 1u << 10;     // nx < 4: several x nodes fold onto the plane
constexpr unsigned PL_DUP = 1u << 11;      // a node appears twice in the cross-section

// Local rows / columns of an end's four stencil nodes in a slab's cross-section.
struct NodeLocal {
  signed char y[4];
  signed char z[4];
};

// What the scatter needs of a pending dipole end, kept in shared memory.
struct SlabEnd {
  int ox;           // wrapped x origin of the stencil
  float F[3];       // force carried by the end
  float phi[3][4];  // Peskin weights of the 4 nodes per axis
};

__host__ __device__ constexpr int align16(int b) { return (b + 15) & ~15; }

// i mod n for i within a few n of [0, n) (no division).
__device__ __forceinline__ int wrap_small(int i, int n) {
  while (i >= n) i -= n;
  while (i < 0) i += n;
  return i;
}

// Byte offsets of the spreading state from byte BASE of shared memory:
// fixed-point sums of one plane [3][PLANE][2 words], coverage masks [CAP] (u64),
// ends [CAP], local node rows [CAP], per-plane list offsets [LX + 2H + 1],
// plane lists [CAP * SPREAD_PLANES_PER_END] (u16).
template <int TZ, int TY, int H, int BASE>
struct SpreadLayout {
  static constexpr int PLANE = (TY + 2 * H) * (TZ + 2 * H);
  static constexpr int fq = align16(BASE);
  static constexpr int xmask = align16(fq + 3 * PLANE * 8);
  static constexpr int ends = align16(xmask + SPREAD_CAP * 8);
  static constexpr int nodes = align16(ends + SPREAD_CAP * (int)sizeof(SlabEnd));
  static constexpr int poff = align16(nodes + SPREAD_CAP * (int)sizeof(NodeLocal));
  static constexpr int plist = align16(poff + (SLAB_LX + 2 * H + 1) * 4);
  static constexpr int total = align16(plist + SPREAD_CAP * SPREAD_PLANES_PER_END * 2);
};

// Where the ends of slab `slab` are: its bucket, or every pending end when the
// bucket overflowed.
struct SlabEnds {
  const EndRecord<float>* ends;
  const unsigned* count;  // [slabs]
  const int* list;        // [slabs][SLAB_BUCKET_CAP]
  int npending;
  const unsigned* max_abs_f;
};

// Whether the sums of slab `slab` can take the split form: a site takes at
// most one contribution per end of the slab (16 when stencil nodes fold onto
// one site), and 65535 contributions keep the sum of their low 16 bits below
// 2^32.  Every spreader of the slab, and the code that reads its sums, makes
// the same choice.
__device__ __forceinline__ bool slab_sums_split(const SlabEnds& se, int slab, int nx, int ny,
                                                int nz) {
  const unsigned c = se.count[slab];
  const long long cnt = c > (unsigned)SLAB_BUCKET_CAP ? se.npending : (long long)c;
  return cnt * (nx < 4 || ny < 4 || nz < 4 ? 16 : 1) <= 65535ll;
}

// SPLIT: the sums are (sum of the low 16 bits, sum of q >> 16), each added
// with an atomic that returns nothing; otherwise 64-bit sums whose high word
// takes the low word's carries (slab_sums_split decides).
template <int TZ, int TY, int H, int BASE, bool SPLIT>
struct SlabSpreader {
  static constexpr int HZ = TZ + 2 * H, PLANE = (TY + 2 * H) * HZ;
  using SL = SpreadLayout<TZ, TY, H, BASE>;
  unsigned char* smem;
  int nx, ny, nz, x0, y0, z0, ex, ey, ez;
  const EndRecord<float>* ends;
  const int* list;
  long long s0;
  int cnt;
  bool in_smem, overflow;
  float fx_scale, fx_inv;
  // shared-memory arrays at fixed offsets from smem
  __device__ unsigned* fq() const { return reinterpret_cast<unsigned*>(smem + SL::fq); }
  __device__ unsigned long long* xmask() const {
    return reinterpret_cast<unsigned long long*>(smem + SL::xmask);
  }
  __device__ SlabEnd* srec() const { return reinterpret_cast<SlabEnd*>(smem + SL::ends); }
  __device__ NodeLocal* nodes() const { return reinterpret_cast<NodeLocal*>(smem + SL::nodes); }
  __device__ int* poff() const { return reinterpret_cast<int*>(smem + SL::poff); }
  __device__ unsigned short* plist() const {
    return reinterpret_cast<unsigned short*>(smem + SL::plist);
  }

  __device__ void bind(unsigned char* smem_, const SlabEnds& se, int slab, int nx_, int ny_,
                       int nz_, int x0_, int y0_, int z0_, int ex_, int ey_, int ez_) {
    smem = smem_;
    nx = nx_, ny = ny_, nz = nz_, x0 = x0_, y0 = y0_, z0 = z0_, ex = ex_, ey = ey_, ez = ez_;
    const int e = fixed_scale_exp(*se.max_abs_f, nx < 4 || ny < 4 || nz < 4);
    fx_scale = exp2_int(e);
    fx_inv = exp2_int(-e);
    ends = se.ends;
    list = se.list;
    const unsigned c = se.count[slab];
    overflow = c > (unsigned)SLAB_BUCKET_CAP;
    cnt = overflow ? se.npending : (int)c;
    s0 = (long long)slab * SLAB_BUCKET_CAP;
    in_smem = !overflow && cnt <= SPREAD_CAP;
  }

  __device__ int planes() const { return ex + 2 * H; }

  // Records, coverage masks, local node rows and per-plane lists of the slab's
  // ends; zeroes the sums.  Every thread of the block calls it.
  __device__ void prologue(int tid, int nthreads) {
    if (in_smem) {
      for (int q = tid; q < cnt; q += nthreads) {
        const EndRecord<float>& g = ends[list[s0 + q]];
        SlabEnd e;
        e.ox = g.o[0];
        for (int c = 0; c < 3; ++c) {
          e.F[c] = g.F[c];
          for (int j = 0; j < 4; ++j) e.phi[c][j] = g.phi[c][j];
        }
        // local planes kk (x = x0 - H + kk) holding one of the x nodes
        unsigned long long m = 0ull;
        if (nx >= 4) {
          for (int i = 0; i < 4; ++i)
            for (int d = wrap_small(e.ox + i - x0 + H, nx); d < planes(); d += nx) m |= 1ull << d;
        } else {
          float w;
          for (int kk = 0; kk < planes(); ++kk)
            if (cover_weight(wrap_once(x0 - H + kk, nx), e.ox, nx, e.phi[0], w)) m |= 1ull << kk;
        }
        // local row / column of each stencil node (-1: outside); bit 63 marks
        // nodes that appear twice in the cross-section
        NodeLocal nl;
        for (int j = 0; j < 4; ++j) {
          const int ly2 = wrap_small(g.o[1] + j - y0 + H, ny);
          const int lz2 = wrap_small(g.o[2] + j - z0 + H, nz);
          nl.y[j] = (signed char)(ly2 <= ey - 1 + 2 * H ? ly2 : -1);
          nl.z[j] = (signed char)(lz2 <= ez - 1 + 2 * H ? lz2 : -1);
          if (ly2 + ny <= ey - 1 + 2 * H || lz2 + nz <= ez - 1 + 2 * H) m |= 1ull << 63;
        }
        srec()[q] = e;
        nodes()[q] = nl;
        xmask()[q] = m;
      }
    }
    for (int i = tid; i < 3 * 2 * PLANE; i += nthreads) fq()[i] = 0u;
    __syncthreads();
    if (in_smem) {
      // per-plane lists in increasing end position: count, offsets, fill
      const int lane = tid & 31, warp = tid >> 5, nwarps = nthreads >> 5;
      for (int kk = warp; kk < planes(); kk += nwarps) {
        int c = 0;
        for (int base = 0; base < cnt; base += 32) {
          const int q = base + lane;
          c += __popc(__ballot_sync(0xffffffffu, q < cnt && ((xmask()[q] >> kk) & 1ull)));
        }
        if (lane == 0) poff()[kk + 1] = c;
      }
      __syncthreads();
      if (tid == 0) {
        poff()[0] = 0;
        for (int kk = 0; kk < planes(); ++kk) poff()[kk + 1] += poff()[kk];
      }
      __syncthreads();
      for (int kk = warp; kk < planes(); kk += nwarps) {
        int at = poff()[kk];
        for (int base = 0; base < cnt; base += 32) {
          const int q = base + lane;
          const bool cov = q < cnt && ((xmask()[q] >> kk) & 1ull);
          const unsigned m = __ballot_sync(0xffffffffu, cov);
          if (cov) {
            int ix = wrap_once(x0 - H + kk, nx) - srec()[q].ox;
            if (ix < 0) ix += nx;
            const unsigned ent = (unsigned)q | (nx >= 4 ? (unsigned)ix << 8 : PL_FOLD) |
                                 ((xmask()[q] >> 63) ? PL_DUP : 0u);
            plist()[at + __popc(m & ((1u << lane) - 1u))] = (unsigned short)ent;
          }
          at += __popc(m);
        }
      }
      __syncthreads();
    }
  }

  // Exact addition of q into the two words w[0], w[1] of a sum.  Split: the
  // low 16 bits (at most 65535 of them sum below 2^32) and q >> 16 (their sum
  // stays within 32 bits).  Otherwise a 64-bit sum: the high word takes the
  // sign of q and the low word's carry, when they do not cancel.
  __device__ void add1(unsigned* w, int q) const {
    if (SPLIT) {
      atomicAdd(w, (unsigned)q & 0xffffu);
      atomicAdd(reinterpret_cast<int*>(w + 1), q >> 16);
    } else {
      const unsigned l = (unsigned)q;
      const unsigned old = atomicAdd(w, l);
      const int h = (q >> 31) + (old + l < old ? 1 : 0);
      if (h != 0) atomicAdd(reinterpret_cast<int*>(w + 1), h);
    }
  }
  __device__ void add3(int at, int q0, int q1, int q2) const {
    add1(fq() + 2 * at, q0);
    add1(fq() + 2 * (PLANE + at), q1);
    add1(fq() + 2 * (2 * PLANE + at), q2);
  }

  // Add the contributions of local plane kk; this thread takes the pairs
  // t0, t0 + stride, ...
  __device__ void scatter(int kk, int t0, int stride) const {
    const int gx = wrap_once(x0 - H + kk, nx);
    if (in_smem) {
      const int p0 = poff()[kk], np = poff()[kk + 1] - p0;
      for (int t = t0; t < np * 16; t += stride) {
        const unsigned ent = plist()[p0 + (t >> 4)];
        const int q = (int)(ent & 0xffu);
        const int jy = (t >> 2) & 3, jz = t & 3;
        const int ly2 = nodes()[q].y[jy], lz2 = nodes()[q].z[jz];
        if ((ly2 | lz2) < 0) continue;  // node outside this cross-section
        const SlabEnd& e = srec()[q];
        float wx;
        if (ent & PL_FOLD)
          cover_weight(gx, e.ox, nx, e.phi[0], wx);
        else
          wx = e.phi[0][(ent >> 8) & 3u];
        const float py = e.phi[1][jy], pz = e.phi[2][jz];
        const int q0 = fx_quant32(node_contrib(py, pz, wx, e.F[0]), fx_scale);
        const int q1 = fx_quant32(node_contrib(py, pz, wx, e.F[1]), fx_scale);
        const int q2 = fx_quant32(node_contrib(py, pz, wx, e.F[2]), fx_scale);
        if (!(ent & PL_DUP)) {
          add3(ly2 * HZ + lz2, q0, q1, q2);
        } else {
          // tiny lattice: a node can appear at several places of the cross-section
          for (int a2 = ly2; a2 <= ey - 1 + 2 * H; a2 += ny)
            for (int b2 = lz2; b2 <= ez - 1 + 2 * H; b2 += nz)
              add3(a2 * HZ + b2, q0, q1, q2);
        }
      }
    } else {
      // more ends than shared memory holds: records from global memory
      for (int t = t0; t < cnt * 16; t += stride) {
        const EndRecord<float>& e = ends[overflow ? (t >> 4) : list[s0 + (t >> 4)]];
        float wx;
        if (!cover_weight(gx, e.o[0], nx, e.phi[0], wx)) continue;
        const int jy = (t >> 2) & 3, jz = t & 3;
        const float py = e.phi[1][jy], pz = e.phi[2][jz];
        const int q0 = fx_quant32(node_contrib(py, pz, wx, e.F[0]), fx_scale);
        const int q1 = fx_quant32(node_contrib(py, pz, wx, e.F[1]), fx_scale);
        const int q2 = fx_quant32(node_contrib(py, pz, wx, e.F[2]), fx_scale);
        const int yg = wrap_any(e.o[1] + jy, ny), zg = wrap_any(e.o[2] + jz, nz);
        for (int ly2 = wrap_any(yg - y0 + H, ny); ly2 <= ey - 1 + 2 * H; ly2 += ny)
          for (int lz2 = wrap_any(zg - z0 + H, nz); lz2 <= ez - 1 + 2 * H; lz2 += nz)
            add3(ly2 * HZ + lz2, q0, q1, q2);
      }
    }
  }

  // The sum of component c at local site `at` as a float, and zero it.
  __device__ float take(int at, int c) const {
    uint2* p = reinterpret_cast<uint2*>(fq()) + c * PLANE + at;
    const uint2 w = *p;
    *p = make_uint2(0u, 0u);
    const long long q = SPLIT ? (long long)(int)w.y * 65536ll + (long long)w.x
                              : (long long)(((unsigned long long)w.y << 32) | w.x);
    return fx_value(q, fx_inv);
  }
};

}  // namespace lbswim
