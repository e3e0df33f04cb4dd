/*
 * Lattice.h -- the D3Q15 MRT lattice-Boltzmann fluid, C++ class API of
 * liblbswim (header-only, over the C ABI of lbswim_c.h).
 *
 * Keeps the reference's types and public members (lbswim/liblbswim/Lattice.h:
 * LatticeAddressing 8-12, LDView 31-37, LatticeData 39-50, Lattice 53-67) so
 * that C++ code and the Cython declarations written against the reference
 * (_lb.pxd:3-49) build unchanged against this header.
 *
 * A Lattice(nx, ny, nz, tau_s, tau_b) is an FP64 lattice computing the
 * reference's method; its device buffers always hold their fields
 * (LBSWIM_COMPAT_EAGER_FIELDS), laid out as the reference's: rho [N],
 * u and force [3][N], fOld and fNew [15][N], site i*ny*nz + j*nz + k.
 * data->fOld.device / fNew.device swap on every Step, as in the reference
 * (lb.cu:241-244).  The extra constructor argument `precision` selects the
 * reduced-precision storage (LBSWIM_F32 ...), whose device buffers have the
 * layouts lbswim_lattice_device_ptr documents; H2D / D2H convert.
 */
#ifndef LBSWIM_CXX_LATTICE_H
#define LBSWIM_CXX_LATTICE_H

#include "LBParams.h"
#include "Shared.h"
#include "d3q15.h"
#include "lbswim_c.h"

struct LatticeAddressing {
  int size[DQ_d];
  int strides[DQ_d];
  int n;
};
static_assert(sizeof(LatticeAddressing) == sizeof(lbswim_addressing), "LatticeAddressing layout");

struct LDView {
  double* rho;
  double* u;
  double* force;
  double* fOld;
  double* fNew;
};

namespace lbswim_cxx {

// H2D / D2H of one LatticeData member through the library.
struct LatticeField : Binding {
  lbswim_lattice* lat;
  int field;
  LatticeField(lbswim_lattice* l, int f) : lat(l), field(f) {}
  void h2d(const void* host) override {
    check(lbswim_lattice_h2d(lat, field, static_cast<const double*>(host)), "H2D");
  }
  void d2h(void* host) override {
    check(lbswim_lattice_d2h(lat, field, static_cast<double*>(host)), "D2H");
  }
};

// Lattice::params: H2D hands the relaxation times to the library (the other
// tables are the model's constants); D2H reads the library's tables.
struct LatticeParams : Binding {
  lbswim_lattice* lat;
  explicit LatticeParams(lbswim_lattice* l) : lat(l) {}
  void h2d(const void* host) override {
    const LBParams* p = static_cast<const LBParams*>(host);
    check(lbswim_lattice_set_tau(lat, p->tau_s, p->tau_b), "params.H2D");
  }
  void d2h(void* host) override {
    check(lbswim_lattice_get_params(lat, static_cast<lbswim_lbparams*>(host)), "params.D2H");
  }
};

struct LatticeAddr : Binding {
  lbswim_lattice* lat;
  explicit LatticeAddr(lbswim_lattice* l) : lat(l) {}
  void h2d(const void*) override {}  // the addressing is fixed at construction
  void d2h(void* host) override {
    check(lbswim_lattice_get_addressing(lat, static_cast<lbswim_addressing*>(host)), "addr.D2H");
  }
};

// Owns the library lattice; a base class so that it exists before, and
// outlives, the members bound to it.
struct LatticeHandle {
  lbswim_lattice* h;
  LatticeHandle(int nx, int ny, int nz, double tau_s, double tau_b, int precision) : h(nullptr) {
    check(lbswim_lattice_create(nx, ny, nz, tau_s, tau_b, precision, &h), "Lattice");
    const int rc = lbswim_lattice_set_compat(h, LBSWIM_COMPAT_INIT_SXZ | LBSWIM_COMPAT_EAGER_FIELDS);
    if (rc != LBSWIM_OK) {
      lbswim_lattice_destroy(h);
      check(rc, "Lattice");
    }
  }
  ~LatticeHandle() { lbswim_lattice_destroy(h); }

 private:
  LatticeHandle(const LatticeHandle&);
  LatticeHandle& operator=(const LatticeHandle&);
};

inline size_t lattice_sites(lbswim_lattice* lat) {
  lbswim_addressing a;
  check(lbswim_lattice_get_addressing(lat, &a), "Lattice");
  return (size_t)a.size[0] * (size_t)a.size[1] * (size_t)a.size[2];
}

}  // namespace lbswim_cxx

struct LatticeData {
  // LatticeData::LatticeData(addr), lb.cu:11-17: five standalone arrays of the
  // lattice's sizes (not attached to any lattice).
  explicit LatticeData(const LatticeAddressing& addr_)
      : rho(addr_.n), u(addr_.n * DQ_d), force(addr_.n * DQ_d), fOld(addr_.n * DQ_q),
        fNew(addr_.n * DQ_q) {}
  // No counterpart in the reference: the five fields of a library lattice.
  explicit LatticeData(lbswim_lattice* lat)
      : rho(lbswim_cxx::lattice_sites(lat), new lbswim_cxx::LatticeField(lat, LBSWIM_FIELD_RHO),
            nullptr),
        u(DQ_d * lbswim_cxx::lattice_sites(lat),
          new lbswim_cxx::LatticeField(lat, LBSWIM_FIELD_U), nullptr),
        force(DQ_d * lbswim_cxx::lattice_sites(lat),
              new lbswim_cxx::LatticeField(lat, LBSWIM_FIELD_FORCE), nullptr),
        fOld(DQ_q * lbswim_cxx::lattice_sites(lat),
             new lbswim_cxx::LatticeField(lat, LBSWIM_FIELD_FOLD), nullptr),
        fNew(DQ_q * lbswim_cxx::lattice_sites(lat),
             new lbswim_cxx::LatticeField(lat, LBSWIM_FIELD_FNEW), nullptr) {}

  // lb.cu:19-36
  LDView Host() {
    LDView v = {rho.host, u.host, force.host, fOld.host, fNew.host};
    return v;
  }
  LDView Device() {
    LDView v = {rho.device, u.device, force.device, fOld.device, fNew.device};
    return v;
  }

  SharedArray<double> rho;
  SharedArray<double> u;
  SharedArray<double> force;
  SharedArray<double> fOld;
  SharedArray<double> fNew;
};

struct Lattice : private lbswim_cxx::LatticeHandle {
  // Lattice::Lattice, lb.cu:40-63: FP64, the reference's method.
  Lattice(int nx, int ny, int nz, double tau_s, double tau_b)
      : Lattice(nx, ny, nz, tau_s, tau_b, LBSWIM_F64) {}
  // No counterpart in the reference: the device storage of the distributions
  // (LBSWIM_F64, LBSWIM_F32, LBSWIM_BF16, LBSWIM_F16).
  Lattice(int nx, int ny, int nz, double tau_s, double tau_b, int precision)
      : lbswim_cxx::LatticeHandle(nx, ny, nz, tau_s, tau_b, precision),
        params(new lbswim_cxx::LatticeParams(h)),
        addr(new lbswim_cxx::LatticeAddr(h)),
        data(nullptr),
        time_step(0),
        known_step_(0) {
    params.D2H();
    addr.D2H();
    lbswim_cxx::check(lbswim_memcpy_h2d(params.device, params.host, sizeof(LBParams)), "Lattice");
    lbswim_cxx::check(lbswim_memcpy_h2d(addr.device, addr.host, sizeof(LatticeAddressing)),
                      "Lattice");
    data = new LatticeData(h);
    refresh();
  }
  // lb.cu:66-67
  ~Lattice() { delete data; }

  // lb.cu:220-247: collide, stream, swap fOld / fNew, time_step++.
  void Step() {
    sync_step();
    lbswim_cxx::check(lbswim_lattice_step(h), "Lattice::Step");
    known_step_ = ++time_step;
    refresh();
  }
  // lb.cu:297-312
  void CalcHydro() {
    lbswim_cxx::check(lbswim_lattice_calc_hydro(h), "Lattice::CalcHydro");
    refresh();
  }
  // lb.cu:373-388
  void InitFromHydro() {
    lbswim_cxx::check(lbswim_lattice_init_from_hydro(h), "Lattice::InitFromHydro");
    refresh();
  }
  // lb.cu:413-428
  void ZeroForce() { lbswim_cxx::check(lbswim_lattice_zero_force(h), "Lattice::ZeroForce"); }

  SharedItem<LBParams> params;
  SharedItem<LatticeAddressing> addr;
  LatticeData* data;
  /* Current timestep */
  int time_step;

  // No counterpart in the reference: the C ABI handle, for the calls of
  // lbswim_c.h (streams, batched ensembles, conservation sums, ...).
  lbswim_lattice* handle() {
    sync_step();
    return h;
  }

 private:
  // time_step is a plain member, as in the reference: a value written to it
  // (lb.pyx:237-244) reaches the library before the next Step.
  void sync_step() {
    if (time_step != known_step_) {
      lbswim_cxx::check(lbswim_lattice_set_time_step(h, time_step), "Lattice");
      known_step_ = time_step;
    }
  }
  void refresh() {
    void* b[5];
    lbswim_cxx::check(lbswim_lattice_device_buffers(h, b), "Lattice");
    data->rho.device = static_cast<double*>(b[LBSWIM_FIELD_RHO]);
    data->u.device = static_cast<double*>(b[LBSWIM_FIELD_U]);
    data->force.device = static_cast<double*>(b[LBSWIM_FIELD_FORCE]);
    data->fOld.device = static_cast<double*>(b[LBSWIM_FIELD_FOLD]);
    data->fNew.device = static_cast<double*>(b[LBSWIM_FIELD_FNEW]);
  }
  int known_step_;
};

#endif
