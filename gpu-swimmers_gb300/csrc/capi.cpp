// capi.cpp -- extern "C" entry points of include/lbswim_c.h.
//
// Every entry point validates its arguments, converts exceptions into a status
// code plus a thread-local message, and never exits the process (the
// reference's CUDA_SAFE_CALL prints and calls exit(), cucall.h:5-14).
#include <atomic>
#include <cmath>
#include <new>
#include <string>

#include "lbswim_internal.h"

namespace lbswim {
static thread_local std::string g_err;
static std::atomic<unsigned long long> g_launches{0};
// Calls that may change a lattice, a particle array or their streams; the
// records a system step prepares for its next step hold only while it stays
// unchanged (reads and system steps leave it alone).
static std::atomic<unsigned long long> g_calls{0};
void set_error(const std::string& m) { g_err = m; }
void count_launches(unsigned long long n) { g_launches += n; }
}  // namespace lbswim

using namespace lbswim;

#define API_BEGIN \
  try {          \
    g_calls.fetch_add(1, std::memory_order_relaxed);
// entry points that change nothing a prepared step depends on
#define API_BEGIN_READ try {
#define API_END                                 \
  }                                             \
  catch (const LbswimError& e) {                \
    set_error(e.msg);                           \
    return e.code;                              \
  }                                             \
  catch (const std::bad_alloc&) {               \
    set_error("host allocation failed");        \
    return LBSWIM_ENOMEM;                       \
  }                                             \
  catch (const std::exception& e) {             \
    set_error(e.what());                        \
    return LBSWIM_ECUDA;                        \
  }                                             \
  return LBSWIM_OK;

#define REQUIRE(cond, msg)                                   \
  do {                                                       \
    if (!(cond)) throw LbswimError{LBSWIM_EINVAL, (msg)};    \
  } while (0)

static void check_lattice(const void* lat) { REQUIRE(lat, "lattice handle is NULL"); }

extern "C" {

const char* lbswim_last_error(void) { return g_err.c_str(); }
const char* lbswim_version(void) { return "lbswim-gb300 1.0 (sm_103a)"; }

int lbswim_kernel_launches(unsigned long long* count) {
  if (!count) return LBSWIM_EINVAL;
  *count = g_launches.load();
  return LBSWIM_OK;
}

int lbswim_host_alloc(size_t bytes, void** out) {
  API_BEGIN
  REQUIRE(out, "out is NULL");
  *out = nullptr;
  LB_CUDA(cudaMallocHost(out, bytes ? bytes : 16));
  API_END
}

int lbswim_host_free(void* ptr) {
  API_BEGIN
  if (ptr) LB_CUDA(cudaFreeHost(ptr));
  API_END
}

// ---- Lattice -------------------------------------------------------------------
int lbswim_lattice_create(int nx, int ny, int nz, double tau_s, double tau_b, int precision,
                          lbswim_lattice** out) {
  API_BEGIN
  REQUIRE(out, "out is NULL");
  *out = nullptr;
  REQUIRE(nx > 0 && ny > 0 && nz > 0, "lattice dimensions must be positive");
  REQUIRE(nx <= 65535, "nx must be at most 65535");
  REQUIRE(std::isfinite(tau_s) && std::isfinite(tau_b) && tau_s > -0.5 && tau_b > -0.5,
          "relaxation times must be finite and > -1/2");
  REQUIRE(precision >= LBSWIM_F64 && precision <= LBSWIM_F16, "unknown precision");
  Lattice* L = new Lattice();
  L->size[0] = nx;
  L->size[1] = ny;
  L->size[2] = nz;
  L->n = (long long)nx * ny * nz;
  L->precision = precision;
  L->tau_s = tau_s;
  L->tau_b = tau_b;
  L->rho0 = precision == LBSWIM_F64 ? 0.0 : 1.0;
  L->fused_tile = nz <= 16 ? 1 : 0;
  fill_params(&L->params, tau_s, tau_b);
  try {
    lattice_alloc(L);
    LB_CUDA(cudaStreamSynchronize(L->stream));
  } catch (...) {
    lattice_free(L);
    delete L;
    throw;
  }
  *out = reinterpret_cast<lbswim_lattice*>(L);
  API_END
}

int lbswim_lattice_destroy(lbswim_lattice* lat) {
  API_BEGIN
  if (!lat) return LBSWIM_OK;
  Lattice* L = reinterpret_cast<Lattice*>(lat);
  lattice_join(L);
  cudaStreamSynchronize(L->stream);
  lattice_free(L);
  delete L;
  API_END
}

#define LAT(h) reinterpret_cast<Lattice*>(h)
#define CLAT(h) reinterpret_cast<const Lattice*>(h)

int lbswim_lattice_step(lbswim_lattice* lat) {
  API_BEGIN
  check_lattice(lat);
  lattice_step(LAT(lat));
  API_END
}

int lbswim_lattice_calc_hydro(lbswim_lattice* lat) {
  API_BEGIN
  check_lattice(lat);
  lattice_calc_hydro(LAT(lat));
  API_END
}

int lbswim_lattice_init_from_hydro(lbswim_lattice* lat) {
  API_BEGIN
  check_lattice(lat);
  lattice_join(LAT(lat));
  lattice_init_from_hydro(LAT(lat));
  API_END
}

int lbswim_lattice_zero_force(lbswim_lattice* lat) {
  API_BEGIN
  check_lattice(lat);
  // Deferred: the next consumer of the force either overwrites it (spreading)
  // or treats it as zero; a read of the field clears the buffer first.  With
  // LBSWIM_COMPAT_EAGER_FIELDS an FP64 lattice clears its buffer at once.
  Lattice* L = LAT(lat);
  lattice_zero_force(L);
  if ((L->compat & LBSWIM_COMPAT_EAGER_FIELDS) && L->precision == LBSWIM_F64) {
    lattice_join(L);
    lattice_zero_force_now(L);
  }
  API_END
}

int lbswim_lattice_h2d(lbswim_lattice* lat, int field, const double* host) {
  API_BEGIN
  check_lattice(lat);
  REQUIRE(field >= LBSWIM_FIELD_RHO && field <= LBSWIM_FIELD_FNEW, "unknown lattice field");
  REQUIRE(host, "host buffer is NULL");
  lattice_join(LAT(lat));
  lattice_h2d(LAT(lat), field, host);
  API_END
}

int lbswim_lattice_d2h(lbswim_lattice* lat, int field, double* host) {
  API_BEGIN
  check_lattice(lat);
  REQUIRE(field >= LBSWIM_FIELD_RHO && field <= LBSWIM_FIELD_FNEW, "unknown lattice field");
  REQUIRE(host, "host buffer is NULL");
  lattice_join(LAT(lat));
  lattice_d2h(LAT(lat), field, host);
  API_END
}

int lbswim_lattice_get_params(const lbswim_lattice* lat, lbswim_lbparams* out) {
  API_BEGIN_READ
  check_lattice(lat);
  REQUIRE(out, "out is NULL");
  *out = CLAT(lat)->params;
  API_END
}

int lbswim_lattice_get_addressing(const lbswim_lattice* lat, lbswim_addressing* out) {
  API_BEGIN_READ
  check_lattice(lat);
  REQUIRE(out, "out is NULL");
  const Lattice* L = CLAT(lat);
  for (int a = 0; a < 3; ++a) out->size[a] = L->size[a];
  out->strides[0] = L->size[1] * L->size[2];
  out->strides[1] = L->size[2];
  out->strides[2] = 1;
  out->n = (int)std::min<long long>(L->n, 0x7fffffffLL);
  API_END
}

int lbswim_lattice_get_time_step(const lbswim_lattice* lat, int* out) {
  API_BEGIN_READ
  check_lattice(lat);
  REQUIRE(out, "out is NULL");
  *out = CLAT(lat)->time_step;
  API_END
}

int lbswim_lattice_set_time_step(lbswim_lattice* lat, int time_step) {
  API_BEGIN
  check_lattice(lat);
  LAT(lat)->time_step = time_step;
  API_END
}

int lbswim_lattice_get_precision(const lbswim_lattice* lat, int* out) {
  API_BEGIN_READ
  check_lattice(lat);
  REQUIRE(out, "out is NULL");
  *out = CLAT(lat)->precision;
  API_END
}

int lbswim_lattice_set_compat(lbswim_lattice* lat, int flags) {
  API_BEGIN
  check_lattice(lat);
  REQUIRE((flags & ~(LBSWIM_COMPAT_INIT_SXZ | LBSWIM_COMPAT_SYNC_STEP |
                      LBSWIM_COMPAT_EXACT_F64 | LBSWIM_COMPAT_WIDE_INDEX |
                      LBSWIM_COMPAT_EAGER_FIELDS | LBSWIM_COMPAT_BULK_COPY)) == 0,
          "unknown compat flag");
  LAT(lat)->compat = flags;
  API_END
}

int lbswim_lattice_get_status(lbswim_lattice* lat, unsigned* status, int clear) {
  API_BEGIN_READ
  check_lattice(lat);
  REQUIRE(status, "status is NULL");
  Lattice* L = LAT(lat);
  lattice_join(L);
  LB_CUDA(cudaMemcpyAsync(status, L->status, sizeof(unsigned), cudaMemcpyDeviceToHost, L->stream));
  if (clear) LB_CUDA(cudaMemsetAsync(L->status, 0, sizeof(unsigned), L->stream));
  LB_CUDA(cudaStreamSynchronize(L->stream));
  API_END
}

int lbswim_lattice_set_stream(lbswim_lattice* lat, void* stream) {
  API_BEGIN
  check_lattice(lat);
  Lattice* L = LAT(lat);
  lattice_join(L);
  LB_CUDA(cudaStreamSynchronize(L->stream));
  L->stream = (cudaStream_t)stream;
  API_END
}

int lbswim_lattice_synchronize(lbswim_lattice* lat) {
  API_BEGIN
  check_lattice(lat);
  lattice_join(LAT(lat));
  LB_CUDA(cudaStreamSynchronize(LAT(lat)->stream));
  API_END
}

int lbswim_lattice_join(lbswim_lattice* lat) {
  API_BEGIN
  check_lattice(lat);
  lattice_join(LAT(lat));
  API_END
}

int lbswim_lattice_device_ptr(const lbswim_lattice* lat, int field, void** ptr, int* elem) {
  API_BEGIN
  check_lattice(lat);
  REQUIRE(ptr, "ptr is NULL");
  REQUIRE(field >= LBSWIM_FIELD_RHO && field <= LBSWIM_FIELD_FNEW, "unknown lattice field");
  Lattice* L = const_cast<Lattice*>(CLAT(lat));
  lattice_join(L);
  if (field == LBSWIM_FIELD_FORCE) lattice_materialise_force(L);
  LB_CUDA(cudaStreamSynchronize(L->stream));
  const bool packed = L->precision != LBSWIM_F64;
  switch (field) {
    case LBSWIM_FIELD_RHO: *ptr = packed ? (void*)L->hydro : L->rho; break;
    case LBSWIM_FIELD_U: *ptr = packed ? (void*)L->hydro : L->u; break;
    case LBSWIM_FIELD_FORCE: *ptr = L->force; break;
    case LBSWIM_FIELD_FOLD: *ptr = L->f[L->cur]; break;
    default: *ptr = L->f[L->cur ^ 1]; break;
  }
  if (elem) {
    const bool is_f = field == LBSWIM_FIELD_FOLD || field == LBSWIM_FIELD_FNEW;
    const bool is_h = field == LBSWIM_FIELD_RHO || field == LBSWIM_FIELD_U;
    *elem = is_f ? elem_bytes(L->precision) : (packed ? (is_h ? 16 : 4) : 8);
  }
  API_END
}

int lbswim_lattice_set_timing(lbswim_lattice* lat, int enable) {
  // events around the step kernel change nothing a prepared step depends on
  API_BEGIN_READ
  check_lattice(lat);
  LAT(lat)->timing = enable != 0;
  API_END
}

int lbswim_lattice_get_timing(lbswim_lattice* lat, double* total_ms, int* launches) {
  API_BEGIN_READ
  check_lattice(lat);
  REQUIRE(total_ms && launches, "NULL argument");
  lattice_read_timing(LAT(lat), total_ms, launches);
  API_END
}

// ---- SwimmerArray ----------------------------------------------------------------
static void check_common(const lbswim_common_params* p) {
  REQUIRE(p, "CommonParams is NULL");
  REQUIRE(std::isfinite(p->P) && std::isfinite(p->l) && std::isfinite(p->alpha) &&
              std::isfinite(p->mobility),
          "CommonParams fields must be finite");
}

int lbswim_swimmers_create(int n, const lbswim_common_params* p, lbswim_swimmers** out) {
  API_BEGIN
  REQUIRE(out, "out is NULL");
  *out = nullptr;
  REQUIRE(n >= 0, "swimmer count must be non-negative");
  check_common(p);
  Swimmers* W = new Swimmers();
  W->n = n;
  W->common = *p;
  W->seed = p->seed;
  W->step = 0;
  try {
    const size_t bytes = sizeof(double) * 3 * (size_t)(n > 0 ? n : 1);
    LB_CUDA(cudaMalloc(&W->r, bytes));
    LB_CUDA(cudaMalloc(&W->v, bytes));
    LB_CUDA(cudaMalloc(&W->nv, bytes));
    LB_CUDA(cudaMemset(W->r, 0, bytes));
    LB_CUDA(cudaMemset(W->v, 0, bytes));
    LB_CUDA(cudaMemset(W->nv, 0, bytes));
  } catch (...) {
    cudaFree(W->r);
    cudaFree(W->v);
    cudaFree(W->nv);
    delete W;
    throw;
  }
  *out = reinterpret_cast<lbswim_swimmers*>(W);
  API_END
}

#define SW(h) reinterpret_cast<Swimmers*>(h)

int lbswim_swimmers_destroy(lbswim_swimmers* sw) {
  API_BEGIN
  if (!sw) return LBSWIM_OK;
  Swimmers* W = SW(sw);
  cudaDeviceSynchronize();
  cudaFree(W->r);
  cudaFree(W->v);
  cudaFree(W->nv);
  if (W->stage) cudaFree(W->stage);
  if (W->flag) cudaFree(W->flag);
  if (W->done) cudaEventDestroy(W->done);
  if (W->recorded) cudaEventDestroy(W->recorded);
  if (W->copy) cudaStreamDestroy(W->copy);
  delete W;
  API_END
}

int lbswim_swimmers_set_common(lbswim_swimmers* sw, const lbswim_common_params* p) {
  API_BEGIN
  REQUIRE(sw, "swimmers handle is NULL");
  check_common(p);
  SW(sw)->common = *p;
  API_END
}

int lbswim_swimmers_get_common(const lbswim_swimmers* sw, lbswim_common_params* out) {
  API_BEGIN_READ
  REQUIRE(sw && out, "NULL argument");
  *out = reinterpret_cast<const Swimmers*>(sw)->common;
  API_END
}

int lbswim_swimmers_get_num(const lbswim_swimmers* sw, int* out) {
  API_BEGIN_READ
  REQUIRE(sw && out, "NULL argument");
  *out = reinterpret_cast<const Swimmers*>(sw)->n;
  API_END
}

int lbswim_swimmers_add_forces(lbswim_swimmers* sw, lbswim_lattice* lat) {
  API_BEGIN
  REQUIRE(sw, "swimmers handle is NULL");
  check_lattice(lat);
  swimmers_add_forces(SW(sw), LAT(lat));
  API_END
}

int lbswim_swimmers_move(lbswim_swimmers* sw, lbswim_lattice* lat) {
  API_BEGIN
  REQUIRE(sw, "swimmers handle is NULL");
  check_lattice(lat);
  swimmers_move(SW(sw), LAT(lat));
  API_END
}

static double* sw_field(Swimmers* W, int field) {
  REQUIRE(field >= LBSWIM_SW_R && field <= LBSWIM_SW_N, "unknown swimmer field");
  return field == LBSWIM_SW_R ? W->r : (field == LBSWIM_SW_V ? W->v : W->nv);
}

int lbswim_swimmers_h2d(lbswim_swimmers* sw, int field, const double* host) {
  API_BEGIN
  REQUIRE(sw && host, "NULL argument");
  Swimmers* W = SW(sw);
  const size_t bytes = sizeof(double) * 3 * W->n;
  // positions and orientations must be finite: checked on a staged copy
  // before the field changes
  const bool check = (field == LBSWIM_SW_R || field == LBSWIM_SW_N) && W->n > 0;
  if (check) {
    if (!W->stage) {
      LB_CUDA(cudaMalloc(&W->stage, bytes));
      LB_CUDA(cudaMalloc(&W->flag, 256));
    }
    upload_checked_finite(W->stage, host, 3LL * W->n, W->flag,
                          field == LBSWIM_SW_R ? "swimmer positions" : "swimmer orientations");
  }
  // the arrays are not bound to one stream: wait for the last kernel that used
  // them (on whichever stream), not for the whole device, and for the end
  // records a system step made of them after its move
  swimmers_wait(W);
  if (W->recorded) LB_CUDA(cudaEventSynchronize(W->recorded));
  if (check) {
    LB_CUDA(cudaMemcpyAsync(sw_field(W, field), W->stage, bytes, cudaMemcpyDeviceToDevice, 0));
    LB_CUDA(cudaStreamSynchronize(0));
  } else {
    LB_CUDA(cudaMemcpy(sw_field(W, field), host, bytes, cudaMemcpyHostToDevice));
  }
  API_END
}

int lbswim_swimmers_d2h(lbswim_swimmers* sw, int field, double* host) {
  API_BEGIN_READ
  REQUIRE(sw && host, "NULL argument");
  Swimmers* W = SW(sw);
  swimmers_wait(W);
  LB_CUDA(cudaMemcpy(host, sw_field(W, field), sizeof(double) * 3 * W->n, cudaMemcpyDeviceToHost));
  API_END
}

int lbswim_swimmers_d2h_all(lbswim_swimmers* sw, double* r, double* v, double* n) {
  API_BEGIN_READ
  REQUIRE(sw, "swimmers handle is NULL");
  Swimmers* W = SW(sw);
  swimmers_wait(W);
  if (!W->copy) LB_CUDA(cudaStreamCreateWithFlags(&W->copy, cudaStreamNonBlocking));
  const size_t bytes = sizeof(double) * 3 * W->n;
  double* dst[3] = {r, v, n};
  const double* src[3] = {W->r, W->v, W->nv};
  for (int f = 0; f < 3; ++f)
    if (dst[f] && bytes) LB_CUDA(cudaMemcpyAsync(dst[f], src[f], bytes, cudaMemcpyDeviceToHost, W->copy));
  LB_CUDA(cudaStreamSynchronize(W->copy));
  API_END
}

int lbswim_swimmers_get_rng(const lbswim_swimmers* sw, unsigned long long* seed,
                            unsigned long long* step) {
  API_BEGIN_READ
  REQUIRE(sw && seed && step, "NULL argument");
  *seed = reinterpret_cast<const Swimmers*>(sw)->seed;
  *step = reinterpret_cast<const Swimmers*>(sw)->step;
  API_END
}

int lbswim_swimmers_set_rng(lbswim_swimmers* sw, unsigned long long seed, unsigned long long step) {
  API_BEGIN
  REQUIRE(sw, "swimmers handle is NULL");
  SW(sw)->seed = seed;
  SW(sw)->step = step;
  API_END
}

int lbswim_lattice_interp_velocity(lbswim_lattice* lat, int npoints, const double* r, double* v) {
  API_BEGIN
  check_lattice(lat);
  REQUIRE(npoints >= 0, "npoints must be non-negative");
  REQUIRE(npoints == 0 || (r && v), "NULL argument");
  lattice_interp_velocity(LAT(lat), npoints, r, v);
  API_END
}

int lbswim_rng_draws(unsigned long long seed, int n, unsigned long long step, float* uniform,
                     double* normal) {
  API_BEGIN
  REQUIRE(n >= 0, "n must be non-negative");
  REQUIRE(n == 0 || (uniform && normal), "NULL argument");
  rng_draws(seed, n, step, uniform, normal);
  API_END
}

int lbswim_spread_forces_noalloc(const double* r, const double* n, int nsw, double P, double l,
                                 int nx, int ny, int nz, double* force, int accumulate,
                                 void* stream) {
  API_BEGIN
  REQUIRE(nsw >= 0, "swimmer count must be non-negative");
  REQUIRE(nsw == 0 || (r && n), "position or orientation pointer is NULL");
  REQUIRE(force, "force pointer is NULL");
  REQUIRE(nx > 0 && ny > 0 && nz > 0 && nx <= 65535, "bad lattice dimensions");
  REQUIRE(std::isfinite(P) && std::isfinite(l), "P and l must be finite");
  const int size[3] = {nx, ny, nz};
  spread_forces_noalloc(r, n, nsw, P, l, size, force, accumulate, (cudaStream_t)stream);
  API_END
}

// ---- TracerArray -----------------------------------------------------------------
int lbswim_tracers_create(int n, lbswim_tracers** out) {
  API_BEGIN
  REQUIRE(out, "out is NULL");
  *out = nullptr;
  REQUIRE(n >= 0, "tracer count must be non-negative");
  Tracers* T = new Tracers();
  T->n = n;
  try {
    tracers_alloc(T);
  } catch (...) {
    tracers_free(T);
    delete T;
    throw;
  }
  *out = reinterpret_cast<lbswim_tracers*>(T);
  API_END
}

#define TR(h) reinterpret_cast<Tracers*>(h)

int lbswim_tracers_destroy(lbswim_tracers* tr) {
  API_BEGIN
  if (!tr) return LBSWIM_OK;
  Tracers* T = TR(tr);
  cudaDeviceSynchronize();
  tracers_free(T);
  delete T;
  API_END
}

int lbswim_tracers_get_num(const lbswim_tracers* tr, int* out) {
  API_BEGIN_READ
  REQUIRE(tr && out, "NULL argument");
  *out = reinterpret_cast<const Tracers*>(tr)->n;
  API_END
}

int lbswim_tracers_move(lbswim_tracers* tr, lbswim_lattice* lat) {
  API_BEGIN
  REQUIRE(tr, "tracers handle is NULL");
  check_lattice(lat);
  tracers_move(TR(tr), LAT(lat));
  API_END
}

int lbswim_tracers_h2d(lbswim_tracers* tr, int field, const double* host) {
  API_BEGIN
  REQUIRE(tr && host, "NULL argument");
  REQUIRE(field >= LBSWIM_TR_R && field <= LBSWIM_TR_V, "unknown tracer field");
  tracers_h2d(TR(tr), field, host);
  API_END
}

int lbswim_tracers_d2h(lbswim_tracers* tr, int field, double* host) {
  API_BEGIN_READ
  REQUIRE(tr && host, "NULL argument");
  REQUIRE(field >= LBSWIM_TR_R && field <= LBSWIM_TR_V, "unknown tracer field");
  tracers_d2h(TR(tr), field, host);
  API_END
}

// ---- System.Step -----------------------------------------------------------------
// ---- seeded initial states -------------------------------------------------------
int lbswim_lattice_init_random(lbswim_lattice* lat, unsigned long long seed, double amplitude) {
  API_BEGIN
  check_lattice(lat);
  REQUIRE(std::isfinite(amplitude), "amplitude must be finite");
  Lattice* L = LAT(lat);
  lattice_join(L);
  lattice_init_random(L, seed, amplitude);
  API_END
}

int lbswim_swimmers_init_random(lbswim_swimmers* sw, const lbswim_lattice* lat,
                                unsigned long long seed) {
  API_BEGIN
  REQUIRE(sw, "swimmers handle is NULL");
  check_lattice(lat);
  swimmers_init_random(reinterpret_cast<Swimmers*>(sw), CLAT(lat), seed);
  API_END
}

int lbswim_tracers_init_random(lbswim_tracers* tr, const lbswim_lattice* lat,
                               unsigned long long seed) {
  API_BEGIN
  REQUIRE(tr, "tracers handle is NULL");
  check_lattice(lat);
  tracers_init_random(reinterpret_cast<Tracers*>(tr), CLAT(lat), seed);
  API_END
}

int lbswim_lattice_set_tau(lbswim_lattice* lat, double tau_s, double tau_b) {
  API_BEGIN
  check_lattice(lat);
  REQUIRE(std::isfinite(tau_s) && std::isfinite(tau_b) && tau_s > -0.5 && tau_b > -0.5,
          "relaxation times must be finite and > -1/2");
  Lattice* L = LAT(lat);
  lattice_join(L);
  LB_CUDA(cudaStreamSynchronize(L->stream));
  L->tau_s = tau_s;
  L->tau_b = tau_b;
  fill_params(&L->params, tau_s, tau_b);
  API_END
}

// ---- batched ensembles -------------------------------------------------------------
int lbswim_ensemble_create(lbswim_ensemble** out) {
  API_BEGIN
  REQUIRE(out, "out is NULL");
  *out = reinterpret_cast<lbswim_ensemble*>(ensemble_new());
  API_END
}

int lbswim_ensemble_destroy(lbswim_ensemble* ens) {
  API_BEGIN
  ensemble_delete(reinterpret_cast<Ensemble*>(ens));
  API_END
}

int lbswim_ensemble_set_members(lbswim_ensemble* ens, lbswim_lattice* const* lattices,
                                lbswim_swimmers* const* swimmers, lbswim_tracers* const* tracers,
                                int n) {
  API_BEGIN
  REQUIRE(ens, "ensemble handle is NULL");
  REQUIRE(n >= 0 && (n == 0 || lattices), "lattice list is NULL");
  ensemble_set_members(reinterpret_cast<Ensemble*>(ens),
                       reinterpret_cast<Lattice* const*>(lattices),
                       reinterpret_cast<Swimmers* const*>(swimmers),
                       reinterpret_cast<Tracers* const*>(tracers), n);
  API_END
}

int lbswim_ensemble_step(lbswim_ensemble* ens, int nsteps) {
  API_BEGIN
  REQUIRE(ens, "ensemble handle is NULL");
  REQUIRE(nsteps >= 0, "nsteps must be non-negative");
  ensemble_step(reinterpret_cast<Ensemble*>(ens), nsteps);
  API_END
}

int lbswim_ensemble_step_limited(lbswim_ensemble* ens, int nsteps, const int* limits) {
  API_BEGIN
  REQUIRE(ens, "ensemble handle is NULL");
  REQUIRE(nsteps >= 0, "nsteps must be non-negative");
  ensemble_step(reinterpret_cast<Ensemble*>(ens), nsteps, limits);
  API_END
}

int lbswim_ensemble_autotune(lbswim_ensemble* ens) {
  API_BEGIN
  REQUIRE(ens, "ensemble handle is NULL");
  ensemble_autotune(reinterpret_cast<Ensemble*>(ens));
  API_END
}

int lbswim_lattice_get_rho0(const lbswim_lattice* lat, double* rho0) {
  API_BEGIN_READ
  check_lattice(lat);
  REQUIRE(rho0, "rho0 is NULL");
  *rho0 = CLAT(lat)->rho0;
  API_END
}

int lbswim_lattice_conservation(lbswim_lattice* lat, double out[4]) {
  API_BEGIN
  check_lattice(lat);
  REQUIRE(out, "out is NULL");
  Lattice* L = LAT(lat);
  lattice_join(L);
  lattice_conservation(L, out);
  API_END
}

int lbswim_lattice_get_tile(const lbswim_lattice* lat, int* tile) {
  API_BEGIN_READ
  check_lattice(lat);
  REQUIRE(tile, "tile is NULL");
  *tile = CLAT(lat)->fused_tile;
  API_END
}

int lbswim_lattice_set_tile(lbswim_lattice* lat, int tile) {
  API_BEGIN
  check_lattice(lat);
  REQUIRE(tile == 0 || tile == 1, "tile must be 0 or 1");
  Lattice* L = LAT(lat);
  lattice_join(L);
  LB_CUDA(cudaStreamSynchronize(L->stream));
  L->fused_tile = tile;
  API_END
}

int lbswim_system_step(lbswim_lattice* lat, lbswim_swimmers* const* swimmers, int n_swimmers,
                       lbswim_tracers* const* tracers, int n_tracers, int nsteps) {
  API_BEGIN_READ
  check_lattice(lat);
  REQUIRE(n_swimmers >= 0 && n_tracers >= 0 && nsteps >= 0, "counts must be non-negative");
  REQUIRE(n_swimmers == 0 || swimmers, "swimmer list is NULL");
  REQUIRE(n_tracers == 0 || tracers, "tracer list is NULL");
  for (int i = 0; i < n_swimmers; ++i) REQUIRE(swimmers[i], "swimmer handle is NULL");
  for (int i = 0; i < n_tracers; ++i) REQUIRE(tracers[i], "tracer handle is NULL");
  Lattice* L = LAT(lat);
  // With one swimmer array, each move also records the moved swimmers' ends
  // for the next step; that step's AddForces takes them unless another call
  // changed something in between.
  const unsigned long long calls = g_calls.load(std::memory_order_relaxed);
  for (int t = 0; t < nsteps; ++t) {
    lattice_zero_force(L);  // ZeroForce
    if (n_swimmers != 1 || !swimmers_add_forces_prepared(SW(swimmers[0]), L, calls))
      for (int i = 0; i < n_swimmers; ++i) swimmers_add_forces(SW(swimmers[i]), L);
    lattice_step(L);
    lattice_calc_hydro(L);
    // Tracers move on their own streams while the swimmers move and the next
    // step spreads forces; the step after that waits before overwriting the
    // velocities they read.
    if (n_tracers > 0) {
      if (!L->hydro_ready)
        LB_CUDA(cudaEventCreateWithFlags(&L->hydro_ready, cudaEventDisableTiming));
      LB_CUDA(cudaEventRecord(L->hydro_ready, L->stream));
      for (int i = 0; i < n_tracers; ++i) tracers_move_async(TR(tracers[i]), L);
    }
    if (n_swimmers == 1)
      swimmers_move_preparing(SW(swimmers[0]), L, calls);
    else
      for (int i = 0; i < n_swimmers; ++i) swimmers_move(SW(swimmers[i]), L);
  }
  API_END
}

// ---- storage and buffers of the C++ class API (include/liblbswim/) -------------
int lbswim_device_alloc(size_t bytes, void** out) {
  API_BEGIN
  REQUIRE(out, "out is NULL");
  *out = nullptr;
  LB_CUDA(cudaMalloc(out, bytes ? bytes : 16));
  API_END
}

int lbswim_device_free(void* ptr) {
  API_BEGIN
  if (ptr) LB_CUDA(cudaFree(ptr));
  API_END
}

int lbswim_memcpy_h2d(void* dst, const void* src, size_t bytes) {
  API_BEGIN
  REQUIRE(bytes == 0 || (dst && src), "NULL argument");
  if (bytes) LB_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
  API_END
}

int lbswim_memcpy_d2h(void* dst, const void* src, size_t bytes) {
  API_BEGIN_READ
  REQUIRE(bytes == 0 || (dst && src), "NULL argument");
  if (bytes) LB_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
  API_END
}

int lbswim_lbparams_fill(lbswim_lbparams* p) {
  API_BEGIN_READ
  REQUIRE(p, "NULL argument");
  fill_params(p, p->tau_s, p->tau_b);
  API_END
}

int lbswim_lattice_device_buffers(const lbswim_lattice* lat, void* out[5]) {
  API_BEGIN_READ
  check_lattice(lat);
  REQUIRE(out, "out is NULL");
  const Lattice* L = CLAT(lat);
  const bool packed = L->precision != LBSWIM_F64;
  out[LBSWIM_FIELD_RHO] = packed ? (void*)L->hydro : L->rho;
  out[LBSWIM_FIELD_U] = packed ? (void*)L->hydro : L->u;
  out[LBSWIM_FIELD_FORCE] = L->force;
  out[LBSWIM_FIELD_FOLD] = L->f[L->cur];
  out[LBSWIM_FIELD_FNEW] = L->f[L->cur ^ 1];
  API_END
}

int lbswim_swimmers_device_ptr(const lbswim_swimmers* sw, int field, void** out) {
  API_BEGIN_READ
  REQUIRE(sw && out, "NULL argument");
  *out = sw_field(const_cast<Swimmers*>(reinterpret_cast<const Swimmers*>(sw)), field);
  API_END
}

int lbswim_tracers_device_ptr(const lbswim_tracers* tr, int field, void** out) {
  API_BEGIN_READ
  REQUIRE(tr && out, "NULL argument");
  REQUIRE(field >= LBSWIM_TR_R && field <= LBSWIM_TR_V, "unknown tracer field");
  const Tracers* T = reinterpret_cast<const Tracers*>(tr);
  *out = field == LBSWIM_TR_R ? T->r : (field == LBSWIM_TR_S ? T->s : T->v);
  API_END
}

}  // extern "C"
