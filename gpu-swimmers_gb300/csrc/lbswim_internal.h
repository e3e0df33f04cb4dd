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

inline int elem_bytes(int precision) {
  return precision == LBSWIM_F64 ? 8 : precision == LBSWIM_F32 ? 4 : 2;
}

// Device scratch for deterministic force spreading: dipole ends binned by the
// 4x4x4 block of their stencil origin.
struct SpreadScratch {
  int capacity_ends = 0;
  int nbins = 0;
  unsigned* bin_count = nullptr;  // [nbins], zero between calls
  unsigned* bin_start = nullptr;  // [nbins + 1]
  unsigned* scan_tmp = nullptr;   // block sums for the scan
  int* order = nullptr;           // [capacity_ends] end ids grouped by bin
  void* ends = nullptr;           // [capacity_ends] EndRecord
  size_t ends_bytes = 0;
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
  void* rho = nullptr;  // double (F64) or float
  void* u = nullptr;
  void* rho_shadow = nullptr;  // rho/u of the post-Step state, written by the fused kernel
  void* u_shadow = nullptr;
  void* force = nullptr;
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
};

struct Tracers {
  int n;
  double* r = nullptr;
  double* s = nullptr;
  double* v = nullptr;
};

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

// particles.cu
void swimmers_add_forces(Swimmers* S, Lattice* L);
void swimmers_move(Swimmers* S, Lattice* L);
void tracers_move(Tracers* T, Lattice* L);
void lattice_interp_velocity(Lattice* L, int npoints, const double* r_host, double* v_host);
void rng_draws(unsigned long long seed, int n, unsigned long long step, float* u_host,
               double* g_host);
void spread_forces_noalloc(const double* r, const double* nv, int nsw, double P, double l,
                           const int size[3], double* force, int accumulate,
                           cudaStream_t stream);

}  // namespace lbswim
