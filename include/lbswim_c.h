/*
 * lbswim_c.h -- C ABI of liblbswim for GB300 (sm_103a).
 *
 * The coupled time step of gpu-swimmers: a D3Q15 MRT lattice-Boltzmann fluid
 * with periodic boundaries, run-and-tumble swimmers and passive tracers,
 * coupled through the Peskin 4-point delta.  Every entry point takes plain
 * pointers and sizes and returns 0 on success or a negative LBSWIM_E* code;
 * lbswim_last_error() gives the message of the calling thread's last failure.
 * (The reference prints and calls exit() on any CUDA error, cucall.h:5-14;
 * here the caller decides.)
 *
 * Each entry point names the reference interface it replaces
 * (rupertnash/gpu-swimmers, paths within that project).
 *
 * Layout: every field is element-slowest SoA, as in the reference
 * (README.md:39).  The site index is i*ny*nz + j*nz + k (lb.cu:55-57).
 *   rho   [N]        u, force  [3][N]        fOld, fNew  [15][N]
 * (host buffers; lbswim_lattice_device_ptr gives the device layouts)
 *   swimmer r, v, n  [3][n]                  tracer r, s, v  [3][n]
 * Host buffers passed to the *_h2d / *_d2h calls are FP64 whatever the
 * lattice's device precision.
 *
 * Streams: every launch of a lattice and of the particle arrays used with it
 * goes to the lattice's stream (default: the legacy default stream, as in the
 * reference).  Calls return once work is enqueued, except *_d2h, which
 * synchronise the stream, and lbswim_lattice_step, which synchronises like
 * Lattice::Step (lb.cu:239) only when LBSWIM_COMPAT_SYNC_STEP is set.
 */
#ifndef LBSWIM_C_H
#define LBSWIM_C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define LBSWIM_OK 0
#define LBSWIM_EINVAL (-1)   /* bad argument */
#define LBSWIM_ECUDA (-2)    /* CUDA runtime error */
#define LBSWIM_ENOMEM (-3)   /* device or host allocation failed */
#define LBSWIM_ESTATE (-4)   /* call not valid in the object's current state */
#define LBSWIM_ENOTSUP (-5)  /* feature not available for this precision */

/* ---- device precision of the lattice distributions ----------------------- */
#define LBSWIM_F64 0  /* FP64 storage and arithmetic: the reference's method */
#define LBSWIM_F32 1  /* FP32 deviations from w_i*rho0, FP32 collision       */
#define LBSWIM_BF16 2 /* BF16 scaled deviations, FP32 collision              */
#define LBSWIM_F16 3  /* FP16 scaled deviations, FP32 collision              */

/* ---- lattice fields (Lattice.h:38-50, LatticeData) ----------------------- */
#define LBSWIM_FIELD_RHO 0
#define LBSWIM_FIELD_U 1
#define LBSWIM_FIELD_FORCE 2
#define LBSWIM_FIELD_FOLD 3
#define LBSWIM_FIELD_FNEW 4

/* ---- particle fields ------------------------------------------------------ */
#define LBSWIM_SW_R 0 /* SwimmerArray.h:25-27 */
#define LBSWIM_SW_V 1
#define LBSWIM_SW_N 2
#define LBSWIM_TR_R 0 /* TracerArray.h:13-15 */
#define LBSWIM_TR_S 1
#define LBSWIM_TR_V 2

/* ---- compat flags (lbswim_lattice_set_compat) ----------------------------- */
/* Reproduce lb.cu:356: InitFromHydro builds the xz stress from u_x*u_y.
 * On by default so results match the reference; inert when u = 0. */
#define LBSWIM_COMPAT_INIT_SXZ 1
/* Synchronise the device at the end of every Step, as lb.cu:239 does. */
#define LBSWIM_COMPAT_SYNC_STEP 2
/* FP64 lattices only: Step, CalcHydro and InitFromHydro use the reference's
 * dense 15x15 transforms in its operation order (lb.cu:72-218, 250-295,
 * 314-371), every operation rounded on its own, so that results are bit for
 * bit those of the reference's host build (about 3x the FP64 work of the
 * default butterfly transform).  The particle kernels of FP64 lattices always
 * follow the reference's operation order. */
#define LBSWIM_COMPAT_EXACT_F64 4
/* FP32/BF16/FP16 lattices: the step and the particle moves use 64-bit site
 * offsets whatever the lattice size; the results are the same bits.  Without
 * it they switch to 64-bit offsets by themselves when 32-bit ones would
 * overflow (15 * N >= 2^31 for the step, N >= 2^31 for the moves).  Batched
 * ensembles always use 32-bit offsets: their members are smaller. */
#define LBSWIM_COMPAT_WIDE_INDEX 8
/* FP64 lattices: ZeroForce clears the device force buffer at once instead of
 * deferring it to the next consumer, so that every device buffer of the
 * lattice holds its field as the reference's do (the reference's own kernels,
 * or a user's, may then read or add to LatticeData's device arrays).  The C++
 * class API of include/liblbswim/ sets it. */
#define LBSWIM_COMPAT_EAGER_FIELDS 16
/* FP32/BF16/FP16 lattices with nz a multiple of 32 and the 8 x 32 slab shape:
 * the step kernel bulk-copies whole rows of distributions into shared memory
 * (cp.async.bulk, completed on an mbarrier) instead of loading them thread by
 * thread.  The results are the same bits.  Off by default: on GB300 the
 * two-stage copy pipeline that fits beside the spreading state (two CTAs per
 * SM) keeps too few bytes in flight, and the step kernel ran slower (0.81 ms
 * against 0.55 ms at 256^3). */
#define LBSWIM_COMPAT_BULK_COPY 32

/* ---- sticky status bits (lbswim_lattice_get_status) ----------------------- */
/* No reference counterpart (the reference checks no kernel).  Kernels of a
 * lattice, and of the particles moved with it, set these bits in a status
 * word on the device; they stay set until read with clear != 0. */
#define LBSWIM_STATUS_NONFINITE 1        /* a step or CalcHydro gave a non-finite rho or u */
#define LBSWIM_STATUS_PARTICLE_OUTSIDE 2 /* a move left a particle non-finite or outside the box */
#define LBSWIM_STATUS_COPY_TIMEOUT 4     /* a kernel gave up waiting for its own bulk copies */

typedef struct lbswim_lattice lbswim_lattice;
typedef struct lbswim_swimmers lbswim_swimmers;
typedef struct lbswim_tracers lbswim_tracers;

/* Same field order and types as the reference's LBParams (LBParams.h:4-30). */
typedef struct lbswim_lbparams {
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
} lbswim_lbparams;

/* Same fields as LatticeAddressing (Lattice.h:8-12). */
typedef struct lbswim_addressing {
  int size[3];
  int strides[3];
  int n;
} lbswim_addressing;

/* Same fields as CommonParams (SwimmerArray.h:8-16); the bools are widened to
 * int so the struct has one layout in C, C++ and ctypes. */
typedef struct lbswim_common_params {
  double P;
  double l;
  double alpha;
  double mobility;
  int translational_advection_off;
  int rotational_advection_off;
  unsigned long long seed;
} lbswim_common_params;

/* ---- library -------------------------------------------------------------- */
const char* lbswim_last_error(void);
const char* lbswim_version(void);
/* Number of this library's kernels launched so far in this process. */
int lbswim_kernel_launches(unsigned long long* count);
/* No reference counterpart: page-locked host memory (cudaMallocHost) for the
 * host copies of particle arrays, which *_h2d / *_d2h then move at the link's
 * full rate instead of through a staging copy.  host_free takes NULL. */
int lbswim_host_alloc(size_t bytes, void** out);
int lbswim_host_free(void* ptr);

/* ---- Lattice (lb.cu, Lattice.h) ------------------------------------------- */
/* Lattice::Lattice(nx, ny, nz, tau_s, tau_b), lb.cu:40-63.  precision selects
 * the device storage (LBSWIM_F64 reproduces the reference). */
int lbswim_lattice_create(int nx, int ny, int nz, double tau_s, double tau_b, int precision,
                          lbswim_lattice** out);
/* Lattice::~Lattice, lb.cu:66-67. */
int lbswim_lattice_destroy(lbswim_lattice* lat);
/* Lattice::Step, lb.cu:220-247: collide, stream, swap fOld/fNew, time_step++. */
int lbswim_lattice_step(lbswim_lattice* lat);
/* Lattice::CalcHydro, lb.cu:297-312: rho, u from fOld and force. */
int lbswim_lattice_calc_hydro(lbswim_lattice* lat);
/* Lattice::InitFromHydro, lb.cu:373-388: fOld from rho, u. */
int lbswim_lattice_init_from_hydro(lbswim_lattice* lat);
/* Lattice::ZeroForce, lb.cu:413-428. */
int lbswim_lattice_zero_force(lbswim_lattice* lat);
/* SharedArray<double>::H2D / D2H (Shared.cu:15-27) of one LatticeData member;
 * `host` holds count = (1, 3, 3, 15, 15)[field] * N doubles. */
int lbswim_lattice_h2d(lbswim_lattice* lat, int field, const double* host);
int lbswim_lattice_d2h(lbswim_lattice* lat, int field, double* host);
/* Lattice::params.host, Lattice::addr.host, Lattice::time_step (Lattice.h:54-58). */
int lbswim_lattice_get_params(const lbswim_lattice* lat, lbswim_lbparams* out);
int lbswim_lattice_get_addressing(const lbswim_lattice* lat, lbswim_addressing* out);
int lbswim_lattice_get_time_step(const lbswim_lattice* lat, int* out);
int lbswim_lattice_set_time_step(lbswim_lattice* lat, int time_step); /* lb.pyx:237-244 */
int lbswim_lattice_get_precision(const lbswim_lattice* lat, int* out);
/* No reference counterpart: total mass and momentum, sum over sites of
 * sum_p f_p and sum_p c_p f_p, accumulated in FP64 in a fixed order (the same
 * bits every call), for conservation checks. */
int lbswim_lattice_conservation(lbswim_lattice* lat, double out[4]);
/* No reference counterpart: the sticky status bits (LBSWIM_STATUS_*) that
 * this lattice's kernels and the moves of particles on it have set; waits
 * for the lattice's queued work first, and clears them when clear != 0. */
int lbswim_lattice_get_status(lbswim_lattice* lat, unsigned* status, int clear);
/* No reference counterpart: behaviour switches and stream binding. */
int lbswim_lattice_set_compat(lbswim_lattice* lat, int flags);
int lbswim_lattice_set_stream(lbswim_lattice* lat, void* cuda_stream);
/* synchronize waits on the host for all work on this lattice, including
 * tracer moves that lbswim_system_step left running on the tracers' own
 * streams.  join only orders the lattice's stream after that work (no host
 * wait), e.g. before recording a CUDA event on that stream. */
int lbswim_lattice_synchronize(lbswim_lattice* lat);
int lbswim_lattice_join(lbswim_lattice* lat);
/* Device address and element size of a field's current buffer: 8 (FP64
 * lattices); for FP32/BF16/FP16 lattices fOld/fNew are 4 or 2 bytes (f - w_p
 * rho0, divided by w_p for the 16-bit formats) in blocks of 32 sites, value p
 * of site s at ((s / 32) * 15 + p) * 32 + s % 32 (N rounded up to a multiple
 * of 32), force 4, and rho and u share one buffer of float4
 * {ux, uy, uz, rho - rho0} per site (16).  rho0 (no
 * reference counterpart) is 1 until InitFromHydro sets it to the mean
 * density, as a float; FP64 lattices have rho0 = 0. */
int lbswim_lattice_get_rho0(const lbswim_lattice* lat, double* rho0);
int lbswim_lattice_device_ptr(const lbswim_lattice* lat, int field, void** ptr, int* elem_bytes);
/* No counterpart in the reference.  When enabled, every LB step kernel of
 * this lattice is bracketed by CUDA events on the lattice's stream (each pair
 * costs the coupled step about 10 us at 256^3, so a caller may time a sample
 * of the steps).  get_timing synchronises the stream and returns the summed
 * device time (ms) and number of timed launches since the previous call.
 * Neither call disturbs the end records a system step prepares for the next. */
int lbswim_lattice_set_timing(lbswim_lattice* lat, int enable);
int lbswim_lattice_get_timing(lbswim_lattice* lat, double* total_ms, int* launches);

/* ---- SwimmerArray (SwimmerArray.cu, SwimmerArray.h) ------------------------ */
/* SwimmerArray::SwimmerArray(n, p), SwimmerArray.cu:16-25.  The random stream
 * is keyed by (p->seed, swimmer index, move step), fixed at construction like
 * the reference's curand_init. */
int lbswim_swimmers_create(int n, const lbswim_common_params* p, lbswim_swimmers** out);
int lbswim_swimmers_destroy(lbswim_swimmers* sw);
/* SharedItem<CommonParams>::H2D after a property set (swimmers.pyx:21-68). */
int lbswim_swimmers_set_common(lbswim_swimmers* sw, const lbswim_common_params* p);
int lbswim_swimmers_get_common(const lbswim_swimmers* sw, lbswim_common_params* out);
int lbswim_swimmers_get_num(const lbswim_swimmers* sw, int* out);
/* SwimmerArray::AddForces, SwimmerArray.cu:114-121 (deterministic order). */
int lbswim_swimmers_add_forces(lbswim_swimmers* sw, lbswim_lattice* lat);
/* SwimmerArray::Move, SwimmerArray.cu:212-220. */
int lbswim_swimmers_move(lbswim_swimmers* sw, lbswim_lattice* lat);
/* SharedArray<double>::H2D / D2H of r, v or n (3*n doubles).  Positions and
 * orientations must be finite (else LBSWIM_EINVAL and the field keeps its
 * values; the check runs on the device, on a staged copy). */
int lbswim_swimmers_h2d(lbswim_swimmers* sw, int field, const double* host);
int lbswim_swimmers_d2h(lbswim_swimmers* sw, int field, double* host);
/* No reference counterpart: the D2H of r, v and n (any may be NULL) with one
 * wait, for loops that read every field each step. */
int lbswim_swimmers_d2h_all(lbswim_swimmers* sw, double* r, double* v, double* n);
/* The random-stream state that SharedArray<RandState> prng holds in the
 * reference (SwimmerArray.h:28): the key seed and the next move step. */
int lbswim_swimmers_get_rng(const lbswim_swimmers* sw, unsigned long long* seed,
                            unsigned long long* step);
int lbswim_swimmers_set_rng(lbswim_swimmers* sw, unsigned long long seed,
                            unsigned long long step);

/* InterpVelocity (interp.cu:8-47) at npoints arbitrary points: r and v are
 * [3][npoints] host arrays.  Reads the lattice's current u. */
int lbswim_lattice_interp_velocity(lbswim_lattice* lat, int npoints, const double* r, double* v);

/* Draws of the swimmer random stream, computed on the device for swimmers
 * 0..n-1 at one move step: the tumble uniform in (0, 1] (uniform[n]) and the
 * three normals of a tumble (normal[3][n]).  Stands in for the cuRAND calls of
 * SwimmerArray.cu:173,179; the stream is keyed by (seed, swimmer, step). */
int lbswim_rng_draws(unsigned long long seed, int n, unsigned long long step, float* uniform,
                     double* normal);

/* ---- allocation-free force spreading --------------------------------------- */
/* Limits of lbswim_spread_forces_noalloc's built-in scratch (about 6.5 MB of
 * device memory, held by every GPU that loads the library until exit). */
#define LBSWIM_NOALLOC_MAX_SWIMMERS 16384
#define LBSWIM_NOALLOC_MAX_SPREAD_BINS 262144 /* 4x4x4-site bins: up to 256^3 */

/* No counterpart in the reference: it always allocates through SharedArray.
 * Spreads the dipole forces of nsw swimmers (the computation of
 * lbswim_swimmers_add_forces) into a caller-owned FP64 force field without
 * allocating any memory.  It is meant for callers that cannot call
 * cudaMalloc: a host application that owns all device memory through its own
 * pool allocator and lets plug-in code use only the buffers it hands out, and
 * real-time loops in which an allocation's implicit device synchronisation,
 * or its failure half way through a time step, is not acceptable.
 * All pointers are device pointers owned by the caller: r and n are the
 * swimmers' positions and orientations, [3][nsw] doubles; force is
 * [3][nx*ny*nz] doubles, overwritten (accumulate = 0) or added to
 * (accumulate != 0).  Work is enqueued on `stream` (a cudaStream_t, NULL for
 * the legacy default stream).  Scratch lives in one static device array of
 * about 6.5 MB: nsw may be at most LBSWIM_NOALLOC_MAX_SWIMMERS, the lattice at
 * most LBSWIM_NOALLOC_MAX_SPREAD_BINS spread bins
 * (ceil(nx/4)*ceil(ny/4)*ceil(nz/4)), nx at most 65535 and ny at most 524280;
 * other inputs are rejected with LBSWIM_EINVAL before any work is enqueued.
 * The first call on a device looks up the array's device address (with that
 * device current); make that first call before any stream capture begins.
 * All calls on a device share the one scratch array, which keeps the last
 * call's contents (the call clears what must start at zero): calls whose work
 * overlaps on the GPU (different streams, or concurrent host threads) race and
 * give wrong results; serialise them on one stream. */
int lbswim_spread_forces_noalloc(const double* r, const double* n, int nsw, double P, double l,
                                 int nx, int ny, int nz, double* force, int accumulate,
                                 void* stream);

/* ---- TracerArray (TracerArray.cu, TracerArray.h) --------------------------- */
/* TracerArray::TracerArray(n), TracerArray.cu:5-10. */
int lbswim_tracers_create(int n, lbswim_tracers** out);
int lbswim_tracers_destroy(lbswim_tracers* tr);
int lbswim_tracers_get_num(const lbswim_tracers* tr, int* out);
/* TracerArray::Move, TracerArray.cu:45-52. */
int lbswim_tracers_move(lbswim_tracers* tr, lbswim_lattice* lat);
/* Positions must be finite (else LBSWIM_EINVAL and the field keeps its values;
 * the check runs on the device, on a staged copy). */
int lbswim_tracers_h2d(lbswim_tracers* tr, int field, const double* host);
int lbswim_tracers_d2h(lbswim_tracers* tr, int field, double* host);

/* ---- seeded initial states made on the device --------------------------------
 * No reference counterpart: for many short solves (serving), whose inputs need
 * not come from the host.  init_random sets rho = 1 + amplitude U[0, 1) and
 * u = 0 from a counter stream keyed by (seed, site), then InitFromHydro;
 * particles get positions uniform in the lattice's box (swimmers also
 * orientations uniform on the sphere, v = 0; tracers s = v = 0).  The same
 * seed gives the same state on any lattice precision. */
int lbswim_lattice_init_random(lbswim_lattice* lat, unsigned long long seed, double amplitude);
int lbswim_swimmers_init_random(lbswim_swimmers* sw, const lbswim_lattice* lat,
                                unsigned long long seed);
int lbswim_tracers_init_random(lbswim_tracers* tr, const lbswim_lattice* lat,
                               unsigned long long seed);
/* Relaxation times of an existing lattice (reuse of a lattice for a new solve). */
int lbswim_lattice_set_tau(lbswim_lattice* lat, double tau_s, double tau_b);

/* ---- batched ensembles ------------------------------------------------------
 * No reference counterpart (the reference steps one lattice at a time).  An
 * ensemble advances many independent FP32 solves -- each an FP32 lattice with
 * an optional swimmer array and an optional tracer array, all created and
 * initialised with the calls above -- by the same coupled step as
 * lbswim_system_step, in four batched launches per step replayed from a CUDA
 * graph.  Each member ends exactly where lbswim_system_step would have taken
 * it (bit for bit, with the same slab shape).  Membership can change between
 * calls to lbswim_ensemble_step; members stay owned by the caller and must
 * outlive their membership.  A member lattice has fewer than 143M sites and its
 * swimmer array at most 32767 swimmers (2047 when an axis is shorter than 4
 * sites); set_members returns LBSWIM_EINVAL otherwise.  autotune picks, per
 * lattice shape, the slab shape that runs fastest (timed on scratch copies;
 * results cached per shape). */
typedef struct lbswim_ensemble lbswim_ensemble;
int lbswim_ensemble_create(lbswim_ensemble** out);
int lbswim_ensemble_destroy(lbswim_ensemble* ens);
int lbswim_ensemble_set_members(lbswim_ensemble* ens, lbswim_lattice* const* lattices,
                                lbswim_swimmers* const* swimmers, lbswim_tracers* const* tracers,
                                int n);
int lbswim_ensemble_step(lbswim_ensemble* ens, int nsteps);
/* nsteps batched steps in which member m takes only the first limits[m] (a
 * member whose solve ends within the run stops there while the others go on;
 * limits[m] <= 0 leaves it as it is).  limits holds one int per member, in
 * set_members order; NULL is lbswim_ensemble_step. */
int lbswim_ensemble_step_limited(lbswim_ensemble* ens, int nsteps, const int* limits);
int lbswim_ensemble_autotune(lbswim_ensemble* ens);
/* Slab shape of a lattice's step kernel: 0 = 8 x 32 cross-section, 1 = 16 x 16. */
int lbswim_lattice_get_tile(const lbswim_lattice* lat, int* tile);
int lbswim_lattice_set_tile(lbswim_lattice* lat, int tile);

/* ---- storage behind the C++ class API (include/liblbswim/) ------------------
 * SharedArray<T>::SharedArray / ~SharedArray / H2D / D2H and the SharedItem
 * equivalents (Shared.cu:4-59) for arrays that are not a library object's
 * field: device memory, and synchronous copies between it and host memory. */
int lbswim_device_alloc(size_t bytes, void** out);
int lbswim_device_free(void* ptr);
int lbswim_memcpy_h2d(void* dst, const void* src, size_t bytes);
int lbswim_memcpy_d2h(void* dst, const void* src, size_t bytes);
/* LatticeEigenSet(LBParams*), d3q15.c:2-186: every table of p from the
 * D3Q15 definitions; p->tau_s and p->tau_b are kept. */
int lbswim_lbparams_fill(lbswim_lbparams* p);
/* LatticeData::Device(), lb.cu:28-36 (LDView): the current device buffers of
 * rho, u, force, fOld and fNew, indexed by LBSWIM_FIELD_*, without waiting for
 * queued work (lbswim_lattice_device_ptr waits for it and documents the
 * layouts).  fOld and fNew swap on every Step (lb.cu:241-244); the packed
 * rho/u buffer of a reduced-precision lattice swaps on CalcHydro. */
int lbswim_lattice_device_buffers(const lbswim_lattice* lat, void* out[5]);
/* SwimmerArray::r/v/n.device (SwimmerArray.h:25-27): [3][n] doubles. */
int lbswim_swimmers_device_ptr(const lbswim_swimmers* sw, int field, void** out);
/* TracerArray::r/s/v.device (TracerArray.h:13-15): [3][n] doubles, in the
 * library's binned work order (a permutation of the user's order, which the
 * tracers' *_h2d / *_d2h translate). */
int lbswim_tracers_device_ptr(const lbswim_tracers* tr, int field, void** out);

/* ---- coupled step (System.Step, System.py:9-16) ---------------------------- */
/* nsteps repetitions of: ZeroForce; AddForces for every swimmer array; Step;
 * CalcHydro; Move for every swimmer array, then every tracer array.  Results
 * are those of the same sequence of single calls.  Tracer moves run on the
 * tracers' own streams, ordered by events, and may still be running when the
 * call returns; every other lbswim call on these objects orders itself after
 * them. */
int lbswim_system_step(lbswim_lattice* lat, lbswim_swimmers* const* swimmers, int n_swimmers,
                       lbswim_tracers* const* tracers, int n_tracers, int nsteps);

#ifdef __cplusplus
}
#endif
#endif
