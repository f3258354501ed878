// Test-harness shim: the subset of boost::optional the reference builder uses
// (construction from T, boost::none, operator bool / !, .get()).  Written
// without std::optional so that "using namespace std; using namespace boost;"
// in the reference sources does not make the name ambiguous.
#pragma once
#include <cassert>
#include <cstring>
#include <cstdlib>
#include <algorithm>
namespace boost {
struct none_t {};
constexpr none_t none{};
template <class T> class optional {
 public:
  optional() : has_(false) {}
  optional(none_t) : has_(false) {}
  optional(const T& v) : has_(true), v_(v) {}
  explicit operator bool() const { return has_; }
  bool operator!() const { return !has_; }
  T& get() { assert(has_); return v_; }
  const T& get() const { assert(has_); return v_; }
 private:
  bool has_;
  T v_;
};
}
