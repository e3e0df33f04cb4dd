// lbswim_internal.h -- host-side objects behind the C ABI of include/lbswim_c.h.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "lbswim_c.h"

namespace lbswim {

// Thread-local message for lbswim_last_error().
void set_error(const std::string& msg);
// Kernel launch counter reported by lbswim_kernel_launches().
void count_launches(unsigned long long n);

struct LbswimError {
  int code;
  std::string msg;
};

#define LB_CUDA(call)                                                                  \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      throw ::lbswim::LbswimError{e_ == cudaErrorMemoryAllocation ? LBSWIM_ENOMEM      \
                                                                   : LBSWIM_ECUDA,    \
                                  std::string(#call) + ": " + cudaGetErrorString(e_)}; \
  } while (0)

#define LB_CHECK_LAUNCH(nkernels)                 \
  do {                                            \
    LB_CUDA(cudaPeekAtLastError());               \
    ::lbswim::count_launches(nkernels);           \
  } while (0)

// Sites a distribution buffer holds: N, or N rounded up to a multiple of 32 for
// the blocked layout of reduced-precision buffers (fidx).
inline long long f_sites(long long N, int precision) {
  return precision == LBSWIM_F64 ? N : (N + 31) & ~31ll;
}

inline int elem_bytes(int precision) {
  return precision == LBSWIM_F64 ? 8 : precision == LBSWIM_F32 ? 4 : 2;
}

// Dipole ends listed under every tile their stencil touches (one set of lists
// per tiling).
struct TileLists {
  int ntiles = 0;
  unsigned* count = nullptr;     // [ntiles], zero between uses
  unsigned* start = nullptr;     // [ntiles + 1]
  unsigned* scan_tmp = nullptr;  // block sums for the scan
  int* list = nullptr;           // [capacity] end ids grouped by tile
  int* sorted = nullptr;         // [capacity] ordered copy for oversized tiles
  long long capacity = 0;
};

// Force spreading state.  The lattice force is base + the spread of the
// `pending` dipole ends recorded since the base was set (base = zero after
// ZeroForce, else the dense force buffer).  FP64 lattices fold the ends into
// the dense buffer at once; reduced-precision lattices keep them pending and
// the step kernel spreads them itself, so the force never goes through HBM
// unless someone reads it.
// Ends listed per step-kernel slab, at most SLAB_BUCKET_CAP per slab (a slab
// with more is spread from the whole list of pending ends).
constexpr int SLAB_BUCKET_CAP = 1024;

struct SpreadScratch {
  int capacity_ends = 0;
  void* ends = nullptr;  // [capacity_ends] EndRecord of the pending ends
  size_t ends_bytes = 0;
  int pending = 0;
  bool stepped = false;  // a Step already consumed the pending ends
  unsigned* max_abs_force = nullptr;  // device: largest |F| component of the pending ends
  TileLists ftiles;      // force tiles, for materialisation
  // slab buckets of the pending ends, filled as the ends are recorded
  unsigned* bucket_count = nullptr;  // [bucket_slabs]
  int* bucket_list = nullptr;        // [bucket_slabs][SLAB_BUCKET_CAP]
  int bucket_slabs = 0;
  int bucket_tile = -1;  // slab shape the buckets hold (Lattice::fused_tile), -1: stale
  // The next step's end records and slab buckets, written by the swimmer move
  // of lbswim_system_step; its AddForces takes them in place of recording
  // again while nothing has changed since (same swimmers, moved by nothing
  // else, no other API call in between, same slab shape).
  struct Prepared {
    void* ends = nullptr;
    size_t ends_bytes = 0;
    int capacity_ends = 0;
    unsigned* bucket_count = nullptr;
    int* bucket_list = nullptr;
    int bucket_slabs = 0;
    unsigned* max_abs_force = nullptr;
    bool valid = false;
    const void* owner = nullptr;          // the Swimmers moved
    unsigned long long owner_step = 0;    // its move counter after that move
    unsigned long long epoch = 0;         // API-call count then
    int tile = -1;
    int nends = 0;
  } prep;
};

// What the fused step kernel needs to spread the pending ends itself.
struct SlabSpread {
  const void* ends = nullptr;
  const unsigned* count = nullptr;
  const int* list = nullptr;
  int npending = 0;
  const unsigned* max_abs_force = nullptr;
};

struct Lattice {
  int size[3];
  long long n;
  int precision;
  double tau_s, tau_b;
  double rho0;  // reference density of the deviation storage (0 for FP64)
  lbswim_lbparams params;
  void* f[2] = {nullptr, nullptr};  // f[cur] is fOld
  int cur = 0;
  void* rho = nullptr;  // FP64 lattices: double[N]
  void* u = nullptr;    // FP64 lattices: double[3][N]
  // FP32/BF16/FP16 lattices: rho and u packed per site as float4 {ux, uy, uz, rho};
  // the shadow holds the post-Step state the fused kernel writes.
  float4* hydro = nullptr;
  float4* hydro_shadow = nullptr;
  void* force = nullptr;
  unsigned* status = nullptr;  // device: sticky LBSWIM_STATUS_* bits
  cudaStream_t stream = 0;
  int time_step = 0;
  int compat = LBSWIM_COMPAT_INIT_SXZ;
  // versions used to decide whether the fused kernel's rho/u are current
  uint64_t f_version = 1, force_version = 1;
  uint64_t shadow_f_version = 0, shadow_force_version = 0;
  bool force_zero_pending = false;  // ZeroForce issued, buffer not yet cleared
  SpreadScratch spread;
  double* staging = nullptr;  // FP64 staging for conversions
  size_t staging_elems = 0;
  int fused_tile = 0;  // 0 = 32x8 cross-section, 1 = 16x16
  // Kernels on other streams that still read a velocity buffer: (buffer, event
  // recorded after them).  Work that writes the buffer waits for the events.
  std::vector<std::pair<const void*, cudaEvent_t>> readers;
  std::vector<cudaEvent_t> reader_pool;
  cudaEvent_t hydro_ready = nullptr;  // recorded on stream after CalcHydro
  // CUDA-event timing of the LB step kernel (lbswim_lattice_set_timing)
  bool timing = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> timed;  // recorded, not yet read
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> event_pool;
};

struct Swimmers {
  int n;
  lbswim_common_params common;
  unsigned long long seed;
  unsigned long long step;
  double* r = nullptr;
  double* v = nullptr;
  double* nv = nullptr;
  // recorded on the stream of the last kernel that read or wrote the arrays,
  // so that host copies wait for that work only (not for other streams)
  cudaEvent_t done = nullptr;
  // recorded after the end records a system step makes of the moved swimmers
  // for its next step (they read r and n after the move): uploads wait for it
  cudaEvent_t recorded = nullptr;
  cudaStream_t copy = nullptr;  // host copies of several fields in one wait
  double* stage = nullptr;      // [3][n] upload checked before it replaces a field
  unsigned* flag = nullptr;     // result of the upload check
};

// Tracers live on the device in a work order binned by position (8^3-site
// bins, re-binned every TRACER_RESORT_MOVES moves and after positions are
// uploaded) so that neighbouring threads read neighbouring velocities.
// perm[k] is the user index of work slot k.
constexpr int TRACER_RESORT_MOVES = 64;
struct Tracers {
  int n;
  double* r = nullptr;  // [3][n] work order
  double* s = nullptr;
  double* v = nullptr;
  double* r2 = nullptr;  // re-binning targets
  double* s2 = nullptr;
  double* v2 = nullptr;
  int* perm = nullptr;
  int* perm2 = nullptr;
  int* bin_of = nullptr;
  double* staging = nullptr;  // [3][n] user order, for H2D / D2H
  unsigned* flag = nullptr;   // result of the upload check
  bool identity = true;       // perm is the identity
  bool needs_sort = true;
  int moves_since_sort = 0;
  int nbins = 0;
  unsigned* bin_count = nullptr;
  unsigned* bin_start = nullptr;
  unsigned* scan_tmp = nullptr;
  // System steps move tracers on their own stream, concurrently with the
  // swimmers and the next force spreading; `done` follows the last such move.
  cudaStream_t side = nullptr;
  cudaEvent_t done = nullptr;
  bool side_pending = false;
};

// ---- batched ensembles ---------------------------------------------------------
// One member of a batched ensemble as the batched kernels see it: an FP32
// lattice with its swimmers and tracers, buffers named relative to the start
// of the current run.
struct EnsMember {
  int size[3];
  long long n;
  float rho0;
  float omega_s, omega_b, force_s, force_b;  // Relax<float>
  int tile;                                  // slab shape: 0 = 8 x 32, 1 = 16 x 16
  int nt[3];                                 // slabs per axis
  void* f[2];           // f(t) at the run's start, and the other buffer
  void* hyd[2];         // float4 {u, rho} written by steps 0, 2, 4, ... / 1, 3, 5, ...
  void* ends;           // EndRecord<float>[2 nsw]
  unsigned* bucket_count;
  int* bucket_list;
  unsigned* max_abs_f;
  int nsw;
  double* sw_r;
  double* sw_v;
  double* sw_n;
  lbswim_common_params common;
  unsigned long long seed, step0;  // swimmer RNG key and move step at the run's start
  int ntr;
  double* tr_r;
  double* tr_s;
  double* tr_v;
  unsigned* status;  // the member lattice's sticky status bits
  int limit;         // steps this member takes in the current run (the run may take more)
};

// Device tables of an ensemble; the batched kernels of a captured step read
// everything from here, so membership changes need no new graph.
struct EnsTable {
  int* nmem;           // [1]
  EnsMember* mem;      // [capacity]
  int* tile_prefix;    // [capacity + 1] first slab of each member
  int* rec_prefix;     // [capacity + 1] first end-record block
  int* sw_prefix;      // [capacity + 1] first swimmer-move block
  int* tr_prefix;      // [capacity + 1] first tracer-move block
  unsigned* counters;  // [2] slab counters of the two relative parities
  long long* g_step;   // steps of the current run, -1 before its first
};

// Work items per block of the batched kernels (particles.cu checks them).
constexpr int ENS_ENDS_PER_BLOCK = 256;
constexpr int ENS_SWIMMERS_PER_BLOCK = 64;
constexpr int ENS_TRACERS_PER_BLOCK = 256;

// Launches of the batched step (lattice.cu, particles.cu).
void ens_launch_reset(const EnsTable& t, int parity, cudaStream_t s);
void ens_launch_records(const EnsTable& t, int grid, cudaStream_t s);
void ens_launch_step(const EnsTable& t, int parity, int grid, cudaStream_t s);
void ens_launch_move(const EnsTable& t, int parity, int grid, cudaStream_t s);
int ens_step_ctas_per_sm();
// Slab shape of a tile choice (x planes, rows, columns).
void slab_shape_of(int tile, int T[3]);

// ensemble.cpp
struct Ensemble;
Ensemble* ensemble_new();
void ensemble_delete(Ensemble* E);
void ensemble_set_members(Ensemble* E, Lattice* const* lat, Swimmers* const* sw,
                          Tracers* const* tr, int n);
// nsteps batched steps; member m takes only the first limits[m] of them when
// limits is given (a member that finishes early leaves the batch).
void ensemble_step(Ensemble* E, int nsteps, const int* limits = nullptr);
void ensemble_autotune(Ensemble* E);
int ensemble_size(const Ensemble* E);

// lattice.cu
void lattice_alloc(Lattice* L);
void lattice_free(Lattice* L);
void lattice_init_from_hydro(Lattice* L);
void lattice_zero_force_now(Lattice* L);
void lattice_materialise_force(Lattice* L);
void lattice_step(Lattice* L);
void lattice_calc_hydro(Lattice* L);
void lattice_h2d(Lattice* L, int field, const double* host);
void lattice_d2h(Lattice* L, int field, double* host);
void fill_params(lbswim_lbparams* p, double tau_s, double tau_b);
void lattice_read_timing(Lattice* L, double* total_ms, int* launches);
void lattice_zero_force(Lattice* L);
// FP64 totals of mass and momentum (sum of f, sum of c f), deterministic.
void lattice_conservation(Lattice* L, double out[4]);
// Make the lattice stream wait for the other-stream readers of `buf` (all
// readers when buf is null).
void lattice_wait_readers(Lattice* L, const void* buf);
inline void lattice_join(Lattice* L) { lattice_wait_readers(L, nullptr); }

// exact_f64.cu: FP64 lattice ops in the reference's operation order
// (LBSWIM_COMPAT_EXACT_F64)
void exact_step_f64(Lattice* L);
void exact_calc_hydro_f64(Lattice* L);
void exact_init_from_hydro_f64(Lattice* L);

// particles.cu: force spreading state
void spread_materialise(Lattice* L);
SlabSpread spread_prepare_slabs(Lattice* L);
// Slab shape of the fused step kernel for a lattice: x planes per slab, rows,
// columns (lattice.cu).
void fused_slab_shape(const Lattice* L, int T[3]);
// Pending-end storage and slab buckets for `nends` ends (particles.cu).
void spread_reserve(Lattice* L, int nends);
// Dense force (base + spread of the pending ends) of a reduced-precision
// lattice, bit for bit the force the step kernel spreads (lattice.cu).
void lattice_force_from_slabs(Lattice* L);
void spread_free(SpreadScratch& S);

// particles.cu
void swimmers_add_forces(Swimmers* S, Lattice* L);
void swimmers_move(Swimmers* S, Lattice* L);
// lbswim_system_step with one swimmer array: AddForces from the records the
// last move prepared (false: nothing prepared that still holds), and the move
// that prepares them for the next step.  epoch counts the API calls made.
bool swimmers_add_forces_prepared(Swimmers* S, Lattice* L, unsigned long long epoch);
void swimmers_move_preparing(Swimmers* S, Lattice* L, unsigned long long epoch);
// Wait on the host for the last kernel that used the swimmer arrays.
void swimmers_wait(Swimmers* S);
void tracers_move(Tracers* T, Lattice* L);
// Move on the tracers' own stream after the point of the lattice stream where
// L->hydro_ready was last recorded.
void tracers_move_async(Tracers* T, Lattice* L);
void tracers_alloc(Tracers* T);
void tracers_free(Tracers* T);
void tracers_h2d(Tracers* T, int field, const double* host);
// Upload of n doubles into the device buffer `stage`, then a check on the
// device that they are all finite (LbswimError LBSWIM_EINVAL naming `what`
// otherwise).  Legacy default stream; returns once the check is read.
void upload_checked_finite(double* stage, const double* host, long long n, unsigned* flag,
                           const char* what);
void tracers_d2h(Tracers* T, int field, double* host);
void lattice_interp_velocity(Lattice* L, int npoints, const double* r_host, double* v_host);
void lattice_init_random(Lattice* L, unsigned long long seed, double amp);
void swimmers_init_random(Swimmers* W, const Lattice* L, unsigned long long seed);
void tracers_init_random(Tracers* T, const Lattice* L, unsigned long long seed);
void rng_draws(unsigned long long seed, int n, unsigned long long step, float* u_host,
               double* g_host);
void spread_forces_noalloc(const double* r, const double* nv, int nsw, double P, double l,
                           const int size[3], double* force, int accumulate,
                           cudaStream_t stream);

}  // namespace lbswim
