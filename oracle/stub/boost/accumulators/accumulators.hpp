// Minimal stand-in for the two Boost.Accumulators features the reference's
// density path uses (sum_kahan and lazy variance). Boost is not installed in
// this image and its version is not pinned by the reference build
// (CMakeLists.txt:38 asks only for >= 1.49), so these restate the textbook
// algorithms the feature names denote. Test infrastructure only.
#pragma once
#include <cstddef>

namespace boost {
namespace accumulators {

struct lazy {};
namespace tag {
struct sum_kahan {};
struct variance {};
}  // namespace tag

template <class... F>
struct features {};

template <class T, class Features>
struct accumulator_set;

// Kahan-compensated running sum: y = x - c; t = s + y; c = (t - s) - y; s = t.
template <class T>
struct accumulator_set<T, features<tag::sum_kahan>> {
  T s = T(0);
  T c = T(0);
  void operator()(T x) {
    volatile T y = x - c;
    volatile T t = s + y;
    volatile T tm = t - s;
    c = tm - y;
    s = t;
  }
};

template <class T>
T sum_kahan(const accumulator_set<T, features<tag::sum_kahan>>& a) {
  return a.s;
}

// Lazy variance: second raw moment minus squared mean, both from plain sums
// accumulated in the sample type, i.e. sum(x^2)/n - (sum(x)/n)^2.
template <class T>
struct accumulator_set<T, features<tag::variance(lazy)>> {
  T sum = T(0);
  T sum2 = T(0);
  std::size_t n = 0;
  void operator()(T x) {
    sum += x;
    sum2 += x * x;
    ++n;
  }
};

template <class T>
T variance(const accumulator_set<T, features<tag::variance(lazy)>>& a) {
  T m2 = a.sum2 / static_cast<T>(a.n);
  T m = a.sum / static_cast<T>(a.n);
  return m2 - m * m;
}

}  // namespace accumulators
}  // namespace boost
