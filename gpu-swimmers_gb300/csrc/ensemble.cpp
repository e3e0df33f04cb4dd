// ensemble.cpp -- batched ensembles: many independent FP32 solves (each a
// lattice with its swimmers and tracers) advanced together.
//
// One batched step is five launches over all members: the step counter, a
// reset of the slab counts, the dipole-end records of every swimmer array (listed under the
// slabs they touch), one persistent step kernel that takes the slabs of every
// member from a shared counter, and one move kernel over every swimmer and
// tracer array.  Everything the kernels need comes from device tables, so the
// launches of two consecutive steps are captured once into a CUDA graph and
// replayed; a change of membership rewrites the tables only.  Members keep
// their buffers: the run starts from, and leaves, each member's state exactly
// as the single-lattice calls would.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "lbswim_internal.h"

namespace lbswim {

struct Ensemble {
  std::vector<Lattice*> lat;
  std::vector<Swimmers*> sw;
  std::vector<Tracers*> tr;
  int capacity = 0;
  void* tables = nullptr;  // one device allocation for all tables
  EnsTable t{};
  std::vector<EnsMember> hmem;
  std::vector<int> pre[4];
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  cudaGraphExec_t g2 = nullptr, g1 = nullptr;
  int grid_step = 0, grid_rec = 0, grid_move = 0;
};

static void drop_graphs(Ensemble* E) {
  if (E->g2) cudaGraphExecDestroy(E->g2);
  if (E->g1) cudaGraphExecDestroy(E->g1);
  E->g2 = E->g1 = nullptr;
}

Ensemble* ensemble_new() {
  Ensemble* E = new Ensemble();
  LB_CUDA(cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking));
  LB_CUDA(cudaEventCreateWithFlags(&E->done, cudaEventDisableTiming));
  int dev = 0, sms = 0;
  LB_CUDA(cudaGetDevice(&dev));
  LB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  E->grid_step = sms * ens_step_ctas_per_sm();
  E->grid_rec = sms * 4;
  E->grid_move = sms * 8;
  return E;
}

void ensemble_delete(Ensemble* E) {
  if (!E) return;
  cudaStreamSynchronize(E->stream);
  drop_graphs(E);
  if (E->tables) cudaFree(E->tables);
  cudaEventDestroy(E->done);
  cudaStreamDestroy(E->stream);
  delete E;
}

int ensemble_size(const Ensemble* E) { return (int)E->lat.size(); }

// Device tables for `cap` members (the graphs hold their addresses).
static void ensure_tables(Ensemble* E, int cap) {
  if (cap <= E->capacity && E->tables) return;
  cap = std::max(cap, std::max(16, E->capacity * 2));
  LB_CUDA(cudaStreamSynchronize(E->stream));
  drop_graphs(E);
  if (E->tables) cudaFree(E->tables);
  E->tables = nullptr;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off += (bytes + 255) & ~(size_t)255;
    return at;
  };
  const size_t o_n = take(sizeof(int)), o_mem = take(sizeof(EnsMember) * cap);
  size_t o_pre[4];
  for (int i = 0; i < 4; ++i) o_pre[i] = take(sizeof(int) * (cap + 1));
  const size_t o_cnt = take(2 * sizeof(unsigned)), o_step = take(sizeof(long long));
  LB_CUDA(cudaMalloc(&E->tables, off));
  LB_CUDA(cudaMemset(E->tables, 0, off));
  char* b = (char*)E->tables;
  E->t.nmem = (int*)(b + o_n);
  E->t.mem = (EnsMember*)(b + o_mem);
  E->t.tile_prefix = (int*)(b + o_pre[0]);
  E->t.rec_prefix = (int*)(b + o_pre[1]);
  E->t.sw_prefix = (int*)(b + o_pre[2]);
  E->t.tr_prefix = (int*)(b + o_pre[3]);
  E->t.counters = (unsigned*)(b + o_cnt);
  E->t.g_step = (long long*)(b + o_step);
  E->capacity = cap;
}

void ensemble_set_members(Ensemble* E, Lattice* const* lat, Swimmers* const* sw,
                          Tracers* const* tr, int n) {
  for (int i = 0; i < n; ++i) {
    if (!lat[i]) throw LbswimError{LBSWIM_EINVAL, "ensemble member lattice is NULL"};
    if (lat[i]->precision != LBSWIM_F32)
      throw LbswimError{LBSWIM_EINVAL, "ensemble members must be FP32 lattices"};
    if (15 * f_sites(lat[i]->n, LBSWIM_F32) >= (1ll << 31))
      throw LbswimError{LBSWIM_EINVAL, "ensemble members must have fewer than 143M sites"};
    for (int j = 0; j < i; ++j)
      if (lat[j] == lat[i]) throw LbswimError{LBSWIM_EINVAL, "a lattice appears twice"};
    // the batched step keeps every slab's force sums in the split form, which
    // holds up to 65535 contributions per site (16 per end on an axis below 4)
    if (sw && sw[i]) {
      const bool fold = lat[i]->size[0] < 4 || lat[i]->size[1] < 4 || lat[i]->size[2] < 4;
      if (2ll * sw[i]->n * (fold ? 16 : 1) > 65535ll)
        throw LbswimError{LBSWIM_EINVAL,
                          "ensemble members take at most 32767 swimmers (2047 when an axis is "
                          "shorter than 4 sites)"};
    }
  }
  E->lat.assign(lat, lat + n);
  E->sw.assign(n, nullptr);
  E->tr.assign(n, nullptr);
  if (sw) std::copy(sw, sw + n, E->sw.begin());
  if (tr) std::copy(tr, tr + n, E->tr.begin());
  ensure_tables(E, n);
}

static void capture(Ensemble* E, int nsteps_in_graph, cudaGraphExec_t* out) {
  cudaGraph_t g = nullptr;
  LB_CUDA(cudaStreamBeginCapture(E->stream, cudaStreamCaptureModeThreadLocal));
  for (int p = 0; p < nsteps_in_graph; ++p) {
    ens_launch_reset(E->t, p, E->stream);
    ens_launch_records(E->t, E->grid_rec, E->stream);
    ens_launch_step(E->t, p, E->grid_step, E->stream);
    ens_launch_move(E->t, p, E->grid_move, E->stream);
  }
  LB_CUDA(cudaStreamEndCapture(E->stream, &g));
  const cudaError_t e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  LB_CUDA(e);
}

// The member table of the current run: buffers named relative to the run's
// start (f[0] = f(t), hyd[p] = the velocity buffer written by steps of
// parity p, so the last one written is the lattice's current one).
static void build_tables(Ensemble* E) {
  const int n = (int)E->lat.size();
  E->hmem.assign(n, EnsMember{});
  for (auto& p : E->pre) p.assign(n + 1, 0);
  for (int m = 0; m < n; ++m) {
    Lattice* L = E->lat[m];
    Swimmers* W = E->sw[m];
    Tracers* T = E->tr[m];
    EnsMember& M = E->hmem[m];
    const int nsw = W ? W->n : 0, ntr = T ? T->n : 0;
    spread_reserve(L, 2 * nsw);
    for (int a = 0; a < 3; ++a) M.size[a] = L->size[a];
    M.n = L->n;
    M.rho0 = (float)L->rho0;
    // the constants of make_relax<float> (lbswim_device.cuh), bit for bit
    const double ws = 1.0 / (L->tau_s + 0.5), wb = 1.0 / (L->tau_b + 0.5);
    M.omega_s = (float)ws;
    M.omega_b = (float)wb;
    M.force_s = (float)(2. * ws * L->tau_s);
    M.force_b = (float)(2. * wb * L->tau_b);
    M.tile = L->fused_tile;
    int T3[3];
    slab_shape_of(M.tile, T3);
    for (int a = 0; a < 3; ++a) M.nt[a] = (L->size[a] + T3[a] - 1) / T3[a];
    M.f[0] = L->f[L->cur];
    M.f[1] = L->f[L->cur ^ 1];
    M.hyd[0] = L->hydro_shadow;
    M.hyd[1] = L->hydro;
    M.ends = L->spread.ends;
    M.bucket_count = L->spread.bucket_count;
    M.bucket_list = L->spread.bucket_list;
    M.max_abs_f = L->spread.max_abs_force;
    M.status = L->status;
    M.nsw = nsw;
    if (W) {
      M.sw_r = W->r;
      M.sw_v = W->v;
      M.sw_n = W->nv;
      M.common = W->common;
      M.seed = W->seed;
      M.step0 = W->step;
    }
    M.ntr = ntr;
    if (T) {
      M.tr_r = T->r;
      M.tr_s = T->s;
      M.tr_v = T->v;
    }
    E->pre[0][m + 1] = E->pre[0][m] + M.nt[0] * M.nt[1] * M.nt[2];
    E->pre[1][m + 1] = E->pre[1][m] + (2 * nsw + ENS_ENDS_PER_BLOCK - 1) / ENS_ENDS_PER_BLOCK;
    E->pre[2][m + 1] = E->pre[2][m] + (nsw + ENS_SWIMMERS_PER_BLOCK - 1) / ENS_SWIMMERS_PER_BLOCK;
    E->pre[3][m + 1] = E->pre[3][m] + (ntr + ENS_TRACERS_PER_BLOCK - 1) / ENS_TRACERS_PER_BLOCK;
  }
}

void ensemble_step(Ensemble* E, int nsteps, const int* limits) {
  const int n = (int)E->lat.size();
  if (n == 0 || nsteps <= 0) return;
  // every member's earlier work (its streams, tracer side streams) first
  LB_CUDA(cudaDeviceSynchronize());
  ensure_tables(E, n);
  build_tables(E);
  std::vector<int> took(n);
  for (int m = 0; m < n; ++m) {
    took[m] = limits ? std::max(0, std::min(nsteps, limits[m])) : nsteps;
    E->hmem[m].limit = took[m];
  }
  LB_CUDA(cudaMemcpyAsync(E->t.nmem, &n, sizeof(int), cudaMemcpyHostToDevice, E->stream));
  LB_CUDA(cudaMemcpyAsync(E->t.mem, E->hmem.data(), sizeof(EnsMember) * n,
                          cudaMemcpyHostToDevice, E->stream));
  int* pre_dev[4] = {E->t.tile_prefix, E->t.rec_prefix, E->t.sw_prefix, E->t.tr_prefix};
  for (int i = 0; i < 4; ++i)
    LB_CUDA(cudaMemcpyAsync(pre_dev[i], E->pre[i].data(), sizeof(int) * (n + 1),
                            cudaMemcpyHostToDevice, E->stream));
  const long long start = -1;
  LB_CUDA(cudaMemcpyAsync(E->t.g_step, &start, sizeof(start), cudaMemcpyHostToDevice,
                          E->stream));
  if (!E->g2) capture(E, 2, &E->g2);
  if (!E->g1) capture(E, 1, &E->g1);
  for (int i = 0; i < nsteps / 2; ++i) LB_CUDA(cudaGraphLaunch(E->g2, E->stream));
  if (nsteps & 1) LB_CUDA(cudaGraphLaunch(E->g1, E->stream));
  count_launches(5ull * nsteps);
  // the host copies above must outlive the copies: wait for the run
  LB_CUDA(cudaStreamSynchronize(E->stream));
  for (int m = 0; m < n; ++m) {
    Lattice* L = E->lat[m];
    const int k = took[m];
    if (k == 0) continue;
    if (k & 1) {
      L->cur ^= 1;
      std::swap(L->hydro, L->hydro_shadow);
    }
    L->time_step += k;
    L->f_version++;
    L->shadow_f_version = 0;  // rho, u of the last step are published
    L->force_version++;
    L->force_zero_pending = true;
    L->spread.pending = 2 * (E->sw[m] ? E->sw[m]->n : 0);
    L->spread.stepped = true;
    L->spread.bucket_tile = L->fused_tile;
    if (E->sw[m]) E->sw[m]->step += k;
    if (E->tr[m]) E->tr[m]->moves_since_sort += k;
  }
}

// ---- tile autotuner ---------------------------------------------------------
// For each lattice shape among the members, time a batched run of scratch
// copies with each slab shape and keep the faster one (cached per shape).
static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int>, int> g_tuned;

static float time_shape(int nx, int ny, int nz, int tile, int copies) {
  std::vector<lbswim_lattice*> lats(copies, nullptr);
  std::vector<lbswim_swimmers*> sws(copies, nullptr);
  Ensemble* E = ensemble_new();
  float ms = 0.f;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  try {
    lbswim_common_params cp{};
    cp.P = 1e-3;
    cp.l = 0.5;
    cp.alpha = 0.01;
    cp.mobility = 1.0;
    cp.seed = 1;
    for (int i = 0; i < copies; ++i) {
      if (lbswim_lattice_create(nx, ny, nz, 0.8, 0.8, LBSWIM_F32, &lats[i]) != LBSWIM_OK)
        throw LbswimError{LBSWIM_ECUDA, lbswim_last_error()};
      Lattice* L = reinterpret_cast<Lattice*>(lats[i]);
      L->fused_tile = tile;
      const int nsw = 64;
      if (lbswim_swimmers_create(nsw, &cp, &sws[i]) != LBSWIM_OK)
        throw LbswimError{LBSWIM_ECUDA, lbswim_last_error()};
      std::vector<double> r(3 * nsw), nv(3 * nsw, 0.0);
      for (int k = 0; k < nsw; ++k) {
        r[k] = (k * 7 % nx) + 0.5;
        r[nsw + k] = (k * 5 % ny) + 0.25;
        r[2 * nsw + k] = (k * 3 % nz) + 0.75;
        nv[2 * nsw + k] = 1.0;
      }
      lbswim_swimmers_h2d(sws[i], LBSWIM_SW_R, r.data());
      lbswim_swimmers_h2d(sws[i], LBSWIM_SW_N, nv.data());
      std::vector<double> rho(L->n, 1.0), u(3 * L->n, 0.0);
      lbswim_lattice_h2d(lats[i], LBSWIM_FIELD_RHO, rho.data());
      lbswim_lattice_h2d(lats[i], LBSWIM_FIELD_U, u.data());
      lbswim_lattice_init_from_hydro(lats[i]);
    }
    std::vector<Lattice*> L(copies);
    std::vector<Swimmers*> W(copies);
    for (int i = 0; i < copies; ++i) {
      L[i] = reinterpret_cast<Lattice*>(lats[i]);
      W[i] = reinterpret_cast<Swimmers*>(sws[i]);
    }
    ensemble_set_members(E, L.data(), W.data(), nullptr, copies);
    ensemble_step(E, 2);  // warm-up, graphs
    // the timed replays below run past that call's step count: no member limit
    for (auto& M : E->hmem) M.limit = 1 << 30;
    LB_CUDA(cudaMemcpyAsync(E->t.mem, E->hmem.data(), sizeof(EnsMember) * E->hmem.size(),
                            cudaMemcpyHostToDevice, E->stream));
    LB_CUDA(cudaEventCreate(&e0));
    LB_CUDA(cudaEventCreate(&e1));
    LB_CUDA(cudaEventRecord(e0, E->stream));
    for (int i = 0; i < 3; ++i) LB_CUDA(cudaGraphLaunch(E->g2, E->stream));
    LB_CUDA(cudaEventRecord(e1, E->stream));
    LB_CUDA(cudaEventSynchronize(e1));
    LB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  } catch (...) {
    ms = -1.f;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  ensemble_delete(E);
  for (auto* p : sws) lbswim_swimmers_destroy(p);
  for (auto* p : lats) lbswim_lattice_destroy(p);
  return ms;
}

void ensemble_autotune(Ensemble* E) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  for (Lattice* L : E->lat) {
    const auto key = std::make_tuple(L->size[0], L->size[1], L->size[2]);
    auto it = g_tuned.find(key);
    if (it == g_tuned.end()) {
      // enough copies to fill the GPU a few times over
      const int copies = (int)std::max<long long>(2, std::min<long long>(64, (1 << 22) / L->n));
      const float a = time_shape(L->size[0], L->size[1], L->size[2], 0, copies);
      const float b = L->size[2] >= 16 && L->size[1] >= 16
                          ? time_shape(L->size[0], L->size[1], L->size[2], 1, copies)
                          : -1.f;
      const int best = (b > 0.f && (a <= 0.f || b < a)) ? 1 : 0;
      it = g_tuned.emplace(key, best).first;
    }
    L->fused_tile = it->second;
  }
}

}  // namespace lbswim
