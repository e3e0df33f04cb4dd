/*
 * Shared.h -- host/device mirrored storage, C++ class API of liblbswim.
 *
 * SharedArray<T> and SharedItem<T> keep the reference's public members
 * (lbswim/liblbswim/Shared.h:4-25: host, device, size, H2D, D2H), so code and
 * Cython declarations (_shared.pxd:1-13) written against the reference use
 * them unchanged.  Two kinds exist:
 *  - standalone (the reference's constructors): host memory plus a device
 *    allocation of the same size; H2D / D2H are synchronous copies between
 *    them (Shared.cu:4-59);
 *  - bound (no counterpart in the reference): the host copy of a field that a
 *    library object owns (LatticeData's members, SwimmerArray::r, ...).  H2D /
 *    D2H go through the library, which converts to the object's device layout
 *    and orders the copy after the object's queued work; `device` is the
 *    field's current device buffer.
 * Host copies up to 1 GB are page-locked, so copies run at the link's rate.
 * A failing library call throws lbswim_cxx::Error (the reference prints the
 * CUDA error and exits, cucall.h:5-14).
 */
#ifndef LBSWIM_CXX_SHARED_H
#define LBSWIM_CXX_SHARED_H

#include <cstddef>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>

#include "lbswim_c.h"

namespace lbswim_cxx {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& what) : std::runtime_error(what), code(c) {}
};

inline void check(int rc, const char* where) {
  if (rc != LBSWIM_OK) throw Error(rc, std::string(where) + ": " + lbswim_last_error());
}

// The library-owned field behind a bound SharedArray / SharedItem.
struct Binding {
  virtual ~Binding() {}
  virtual void h2d(const void* host) = 0;
  virtual void d2h(void* host) = 0;
};

constexpr size_t kPinnedLimit = size_t(1) << 30;

// Zeroed host memory of `bytes` bytes: page-locked when at most 1 GB and
// available, else from the heap.
inline void* host_alloc(size_t bytes, bool& pinned) {
  void* p = nullptr;
  pinned = false;
  if (bytes <= kPinnedLimit && lbswim_host_alloc(bytes, &p) == LBSWIM_OK && p) {
    pinned = true;
  } else {
    p = ::operator new(bytes ? bytes : 1);
  }
  std::memset(p, 0, bytes);
  return p;
}

inline void host_free(void* p, bool pinned) {
  if (!p) return;
  if (pinned)
    lbswim_host_free(p);
  else
    ::operator delete(p);
}

}  // namespace lbswim_cxx

template <typename T>
struct SharedArray {
  T* host;
  T* device;
  size_t size;

  // SharedArray<T>::SharedArray(n), Shared.cu:4-8: n elements on the host and
  // on the device (contents start at zero here).
  explicit SharedArray(size_t n) : host(nullptr), device(nullptr), size(n), bind_(nullptr) {
    host = static_cast<T*>(lbswim_cxx::host_alloc(n * sizeof(T), pinned_));
    void* d = nullptr;
    const int rc = lbswim_device_alloc(n * sizeof(T), &d);
    if (rc != LBSWIM_OK) {
      lbswim_cxx::host_free(host, pinned_);
      lbswim_cxx::check(rc, "SharedArray");
    }
    device = static_cast<T*>(d);
    owns_device_ = true;
  }
  // No counterpart in the reference: the host copy of a field a library
  // object owns (takes ownership of the binding).
  SharedArray(size_t n, lbswim_cxx::Binding* b, T* dev)
      : host(nullptr), device(dev), size(n), bind_(b), owns_device_(false) {
    host = static_cast<T*>(lbswim_cxx::host_alloc(n * sizeof(T), pinned_));
  }
  ~SharedArray() {
    lbswim_cxx::host_free(host, pinned_);
    if (owns_device_) lbswim_device_free(device);
    delete bind_;
  }
  // Shared.cu:15-27: host -> device and device -> host, synchronous.
  void H2D() {
    if (bind_)
      bind_->h2d(host);
    else
      lbswim_cxx::check(lbswim_memcpy_h2d(device, host, size * sizeof(T)), "SharedArray::H2D");
  }
  void D2H() {
    if (bind_)
      bind_->d2h(host);
    else
      lbswim_cxx::check(lbswim_memcpy_d2h(host, device, size * sizeof(T)), "SharedArray::D2H");
  }

 private:
  SharedArray(const SharedArray&);
  SharedArray& operator=(const SharedArray&);
  lbswim_cxx::Binding* bind_;
  bool pinned_ = false;
  bool owns_device_ = false;
};

template <typename T>
struct SharedItem {
  T* host;
  T* device;

  // SharedItem<T>::SharedItem(), Shared.cu:30-34: one object on each side.
  SharedItem() : host(new T()), device(nullptr), bind_(nullptr) { alloc_device(); }
  // SharedItem<T>::SharedItem(init), Shared.cu:35-41: copies *init to both.
  explicit SharedItem(const T* init) : host(new T(*init)), device(nullptr), bind_(nullptr) {
    alloc_device();
    H2D();
  }
  // No counterpart in the reference: an item whose H2D / D2H also set / read
  // the library object it configures (takes ownership of the binding); the
  // device copy is kept as in the reference.
  explicit SharedItem(lbswim_cxx::Binding* b) : host(new T()), device(nullptr), bind_(b) {
    alloc_device();
  }
  ~SharedItem() {
    delete host;
    lbswim_device_free(device);
    delete bind_;
  }
  void H2D() {
    lbswim_cxx::check(lbswim_memcpy_h2d(device, host, sizeof(T)), "SharedItem::H2D");
    if (bind_) bind_->h2d(host);
  }
  void D2H() {
    if (bind_)
      bind_->d2h(host);
    else
      lbswim_cxx::check(lbswim_memcpy_d2h(host, device, sizeof(T)), "SharedItem::D2H");
  }

 private:
  SharedItem(const SharedItem&);
  SharedItem& operator=(const SharedItem&);
  void alloc_device() {
    void* d = nullptr;
    const int rc = lbswim_device_alloc(sizeof(T), &d);
    if (rc != LBSWIM_OK) {
      delete host;
      delete bind_;
      lbswim_cxx::check(rc, "SharedItem");
    }
    device = static_cast<T*>(d);
  }
  lbswim_cxx::Binding* bind_;
};

#endif
