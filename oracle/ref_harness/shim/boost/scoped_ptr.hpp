// Test-harness shim: boost::scoped_ptr on top of std::unique_ptr (reset/get/->).
#pragma once
#include <memory>
#include <cassert>
#include <cstring>
#include <cstdlib>
#include <algorithm>
namespace boost {
template <class T> class scoped_ptr {
 public:
  scoped_ptr() {}
  explicit scoped_ptr(T* p) : p_(p) {}
  void reset(T* p = nullptr) { p_.reset(p); }
  T* get() const { return p_.get(); }
  T* operator->() const { return p_.get(); }
  T& operator*() const { return *p_; }
  explicit operator bool() const { return (bool)p_; }
 private:
  std::unique_ptr<T> p_;
};
}
