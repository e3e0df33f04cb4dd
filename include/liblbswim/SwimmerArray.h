/*
 * SwimmerArray.h -- run-and-tumble dipole swimmers, C++ class API of liblbswim
 * (header-only, over the C ABI of lbswim_c.h).
 *
 * Keeps the reference's types and public members (lbswim/liblbswim/
 * SwimmerArray.h:5-29) so that C++ code and the Cython declarations written
 * against the reference (SwimmerArray.pxd:4-26) build unchanged against it.
 * r, v and n are [3][num] doubles on both sides.
 *
 * The reference keeps one cuRAND XORWOW state per swimmer in prng.  The
 * library's stream is counter-based, keyed by (seed, swimmer, move step), so
 * the whole random state is one RandState {seed, step}: prng has size 1, its
 * H2D / D2H set and read that state (exact resume), and prng.device is null.
 */
#ifndef LBSWIM_CXX_SWIMMER_ARRAY_H
#define LBSWIM_CXX_SWIMMER_ARRAY_H

#include "Lattice.h"

struct RandState {
  unsigned long long seed;  // key of the swimmers' stream
  unsigned long long step;  // next move step
};

struct CommonParams {
  double P;
  double l;
  double alpha;
  double mobility;
  bool translational_advection_off;
  bool rotational_advection_off;
  unsigned long long seed;
};

namespace lbswim_cxx {

inline lbswim_common_params to_c(const CommonParams& p) {
  lbswim_common_params c;
  c.P = p.P;
  c.l = p.l;
  c.alpha = p.alpha;
  c.mobility = p.mobility;
  c.translational_advection_off = p.translational_advection_off ? 1 : 0;
  c.rotational_advection_off = p.rotational_advection_off ? 1 : 0;
  c.seed = p.seed;
  return c;
}

struct SwimmerField : Binding {
  lbswim_swimmers* sw;
  int field;
  SwimmerField(lbswim_swimmers* s, int f) : sw(s), field(f) {}
  void h2d(const void* host) override {
    check(lbswim_swimmers_h2d(sw, field, static_cast<const double*>(host)), "SwimmerArray H2D");
  }
  void d2h(void* host) override {
    check(lbswim_swimmers_d2h(sw, field, static_cast<double*>(host)), "SwimmerArray D2H");
  }
};

// SwimmerArray::common: H2D hands the parameters to the library at once (a
// property set of swimmers.pyx:21-68 does H2D).
struct SwimmerCommon : Binding {
  lbswim_swimmers* sw;
  explicit SwimmerCommon(lbswim_swimmers* s) : sw(s) {}
  void h2d(const void* host) override {
    const lbswim_common_params c = to_c(*static_cast<const CommonParams*>(host));
    check(lbswim_swimmers_set_common(sw, &c), "common.H2D");
  }
  void d2h(void* host) override {
    lbswim_common_params c;
    check(lbswim_swimmers_get_common(sw, &c), "common.D2H");
    CommonParams* p = static_cast<CommonParams*>(host);
    p->P = c.P;
    p->l = c.l;
    p->alpha = c.alpha;
    p->mobility = c.mobility;
    p->translational_advection_off = c.translational_advection_off != 0;
    p->rotational_advection_off = c.rotational_advection_off != 0;
    p->seed = c.seed;
  }
};

struct SwimmerRng : Binding {
  lbswim_swimmers* sw;
  explicit SwimmerRng(lbswim_swimmers* s) : sw(s) {}
  void h2d(const void* host) override {
    const RandState* r = static_cast<const RandState*>(host);
    check(lbswim_swimmers_set_rng(sw, r->seed, r->step), "prng.H2D");
  }
  void d2h(void* host) override {
    RandState* r = static_cast<RandState*>(host);
    check(lbswim_swimmers_get_rng(sw, &r->seed, &r->step), "prng.D2H");
  }
};

struct SwimmerHandle {
  lbswim_swimmers* h;
  SwimmerHandle(int n, const CommonParams* p) : h(nullptr) {
    if (!p) throw Error(LBSWIM_EINVAL, "SwimmerArray: CommonParams is NULL");
    const lbswim_common_params c = to_c(*p);
    check(lbswim_swimmers_create(n, &c, &h), "SwimmerArray");
  }
  ~SwimmerHandle() { lbswim_swimmers_destroy(h); }

 private:
  SwimmerHandle(const SwimmerHandle&);
  SwimmerHandle& operator=(const SwimmerHandle&);
};

inline double* swimmer_device(lbswim_swimmers* sw, int field) {
  void* p = nullptr;
  check(lbswim_swimmers_device_ptr(sw, field, &p), "SwimmerArray");
  return static_cast<double*>(p);
}

}  // namespace lbswim_cxx

struct SwimmerArray : private lbswim_cxx::SwimmerHandle {
  static const int BlockSize = 512;
  // SwimmerArray::SwimmerArray(n, p), SwimmerArray.cu:16-25: the random
  // stream is keyed by p->seed, as curand_init was.
  SwimmerArray(const int n_, const CommonParams* p)
      : lbswim_cxx::SwimmerHandle(n_, p),
        num(n_),
        common(new lbswim_cxx::SwimmerCommon(h)),
        r(3 * (size_t)n_, new lbswim_cxx::SwimmerField(h, LBSWIM_SW_R),
          lbswim_cxx::swimmer_device(h, LBSWIM_SW_R)),
        v(3 * (size_t)n_, new lbswim_cxx::SwimmerField(h, LBSWIM_SW_V),
          lbswim_cxx::swimmer_device(h, LBSWIM_SW_V)),
        n(3 * (size_t)n_, new lbswim_cxx::SwimmerField(h, LBSWIM_SW_N),
          lbswim_cxx::swimmer_device(h, LBSWIM_SW_N)),
        prng(1, new lbswim_cxx::SwimmerRng(h), nullptr) {
    *common.host = *p;
    lbswim_cxx::check(lbswim_memcpy_h2d(common.device, common.host, sizeof(CommonParams)),
                      "SwimmerArray");
    prng.D2H();
  }

  // SwimmerArray::AddForces, SwimmerArray.cu:114-121 (deterministic order).
  void AddForces(Lattice* lat) const {
    lbswim_cxx::check(lbswim_swimmers_add_forces(h, lat->handle()), "SwimmerArray::AddForces");
  }
  // SwimmerArray::Move, SwimmerArray.cu:212-220.
  void Move(Lattice* lat) {
    lbswim_cxx::check(lbswim_swimmers_move(h, lat->handle()), "SwimmerArray::Move");
  }

  int num;
  SharedItem<CommonParams> common;
  SharedArray<double> r;
  SharedArray<double> v;
  SharedArray<double> n;
  SharedArray<RandState> prng;

  // No counterpart in the reference: the C ABI handle.
  lbswim_swimmers* handle() const { return h; }
};

#endif
