/*
 * TracerArray.h -- passive tracers, C++ class API of liblbswim (header-only,
 * over the C ABI of lbswim_c.h).
 *
 * Keeps the reference's public members (lbswim/liblbswim/TracerArray.h:6-14)
 * so that C++ code and the Cython declarations written against the reference
 * (TracerArray.pxd:4-11) build unchanged against it.  The host copies r, s, v
 * are [3][num] doubles in the user's order.  On the device the library keeps
 * the tracers in a work order binned by position (re-binned from time to
 * time, which can also move the buffers): the .device pointers, refreshed
 * after every Move, address those buffers, a permutation of the user's order
 * that H2D / D2H translate.
 */
#ifndef LBSWIM_CXX_TRACER_ARRAY_H
#define LBSWIM_CXX_TRACER_ARRAY_H

#include "Lattice.h"

namespace lbswim_cxx {

struct TracerField : Binding {
  lbswim_tracers* tr;
  int field;
  TracerField(lbswim_tracers* t, int f) : tr(t), field(f) {}
  void h2d(const void* host) override {
    check(lbswim_tracers_h2d(tr, field, static_cast<const double*>(host)), "TracerArray H2D");
  }
  void d2h(void* host) override {
    check(lbswim_tracers_d2h(tr, field, static_cast<double*>(host)), "TracerArray D2H");
  }
};

struct TracerHandle {
  lbswim_tracers* h;
  explicit TracerHandle(int n) : h(nullptr) { check(lbswim_tracers_create(n, &h), "TracerArray"); }
  ~TracerHandle() { lbswim_tracers_destroy(h); }

 private:
  TracerHandle(const TracerHandle&);
  TracerHandle& operator=(const TracerHandle&);
};

}  // namespace lbswim_cxx

struct TracerArray : private lbswim_cxx::TracerHandle {
  static const int BlockSize = 512;
  // TracerArray::TracerArray(n), TracerArray.cu:5-10.
  explicit TracerArray(const int n_)
      : lbswim_cxx::TracerHandle(n_),
        num(n_),
        r(3 * (size_t)n_, new lbswim_cxx::TracerField(h, LBSWIM_TR_R), nullptr),
        s(3 * (size_t)n_, new lbswim_cxx::TracerField(h, LBSWIM_TR_S), nullptr),
        v(3 * (size_t)n_, new lbswim_cxx::TracerField(h, LBSWIM_TR_V), nullptr) {
    refresh();
  }

  // TracerArray::Move, TracerArray.cu:45-52.
  void Move(Lattice* lat) {
    lbswim_cxx::check(lbswim_tracers_move(h, lat->handle()), "TracerArray::Move");
    refresh();
  }

  int num;
  SharedArray<double> r;
  SharedArray<double> s;
  SharedArray<double> v;

  // No counterpart in the reference: the C ABI handle.
  lbswim_tracers* handle() const { return h; }

 private:
  void refresh() {
    void* p = nullptr;
    lbswim_cxx::check(lbswim_tracers_device_ptr(h, LBSWIM_TR_R, &p), "TracerArray");
    r.device = static_cast<double*>(p);
    lbswim_cxx::check(lbswim_tracers_device_ptr(h, LBSWIM_TR_S, &p), "TracerArray");
    s.device = static_cast<double*>(p);
    lbswim_cxx::check(lbswim_tracers_device_ptr(h, LBSWIM_TR_V, &p), "TracerArray");
    v.device = static_cast<double*>(p);
  }
};

#endif
