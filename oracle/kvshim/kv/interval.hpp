// kv/interval.hpp -- project-written stand-in for kv::interval<T> (kv library
// absent here).  Written to kv's public API names only, so that the unmodified
// VCP headers (vcp/imats.hpp, vcp/pidblas.hpp) compile for the CPU reference
// build.  Endpoints are rounded outward with <cfenv> (each operation saves and
// restores the caller's rounding mode).  Semantics follow the published kv
// documentation: mid() rounds to nearest (halves first on overflow), rad()
// and midrad() round the radius up so [mid-rad, mid+rad] contains the
// interval; comparisons are "certainly" relations.  TEST INFRASTRUCTURE ONLY.
#ifndef INTERVAL_HPP
#define INTERVAL_HPP
#include <cfenv>
#include <cmath>
#include <algorithm>
#include <iostream>
#include <limits>
#include <stdexcept>
#include <kv/hwround.hpp>

namespace kv {

namespace shim {
struct mode_guard {
  int prev;
  explicit mode_guard(int m) : prev(std::fegetround()) { std::fesetround(m); }
  ~mode_guard() { std::fesetround(prev); }
};
// Operands are read through volatile copies after the mode switch and the
// result is stored to a volatile before it is restored, so the arithmetic
// cannot move across the fesetround calls (double; other endpoint types,
// such as kv::dd in interval<kv::dd>, only pass through the file I/O here).
#define KVSHIM_DIR(name, mode, expr)                 \
  template <class T> inline T name(T a, T b) {       \
    T x = a, y = b;                                  \
    mode_guard g(mode);                              \
    T r = expr;                                      \
    return r;                                        \
  }                                                  \
  inline double name(double a, double b) {           \
    volatile double x = a, y = b;                    \
    mode_guard g(mode);                              \
    volatile double r = expr;                        \
    return r;                                        \
  }
KVSHIM_DIR(add_dn, FE_DOWNWARD, x + y)
KVSHIM_DIR(add_up, FE_UPWARD, x + y)
KVSHIM_DIR(sub_dn, FE_DOWNWARD, x - y)
KVSHIM_DIR(sub_up, FE_UPWARD, x - y)
KVSHIM_DIR(mul_dn, FE_DOWNWARD, x * y)
KVSHIM_DIR(mul_up, FE_UPWARD, x * y)
KVSHIM_DIR(div_dn, FE_DOWNWARD, x / y)
KVSHIM_DIR(div_up, FE_UPWARD, x / y)
#undef KVSHIM_DIR
template <class T> inline T sqrt_dn(T a) { using std::sqrt; mode_guard g(FE_DOWNWARD); return sqrt(a); }
template <class T> inline T sqrt_up(T a) { using std::sqrt; mode_guard g(FE_UPWARD); return sqrt(a); }
inline double sqrt_dn(double a) { volatile double x = a; mode_guard g(FE_DOWNWARD); volatile double r = std::sqrt((double)x); return r; }
inline double sqrt_up(double a) { volatile double x = a; mode_guard g(FE_UPWARD); volatile double r = std::sqrt((double)x); return r; }
}  // namespace shim

template <class T> class interval {
  T inf, sup;

 public:
  typedef T base_type;
  interval() : inf(0), sup(0) {}
  template <class C> interval(const C& x) : inf(T(x)), sup(T(x)) {}
  interval(const interval& x) = default;
  interval(const T& l, const T& u) : inf(l), sup(u) {}
  template <class C1, class C2> interval(const C1& l, const C2& u) : inf(T(l)), sup(T(u)) {}
  interval& operator=(const interval& x) = default;
  template <class C> interval& operator=(const C& x) { inf = sup = T(x); return *this; }

  interval& assign(const T& l, const T& u) {
    inf = l;
    sup = u;
    return *this;
  }

  T& lower() { return inf; }
  const T& lower() const { return inf; }
  T& upper() { return sup; }
  const T& upper() const { return sup; }

  static interval whole() { T i = std::numeric_limits<T>::infinity(); return interval(-i, i); }

  friend interval operator+(const interval& x, const interval& y) {
    return interval(shim::add_dn(x.inf, y.inf), shim::add_up(x.sup, y.sup));
  }
  friend interval operator-(const interval& x, const interval& y) {
    return interval(shim::sub_dn(x.inf, y.sup), shim::sub_up(x.sup, y.inf));
  }
  friend interval operator-(const interval& x) { return interval(-x.sup, -x.inf); }
  friend interval operator*(const interval& x, const interval& y) {
    T a[4] = {shim::mul_dn(x.inf, y.inf), shim::mul_dn(x.inf, y.sup), shim::mul_dn(x.sup, y.inf),
              shim::mul_dn(x.sup, y.sup)};
    T b[4] = {shim::mul_up(x.inf, y.inf), shim::mul_up(x.inf, y.sup), shim::mul_up(x.sup, y.inf),
              shim::mul_up(x.sup, y.sup)};
    return interval(*std::min_element(a, a + 4), *std::max_element(b, b + 4));
  }
  friend interval operator/(const interval& x, const interval& y) {
    if (y.inf <= 0 && y.sup >= 0) throw std::domain_error("kvshim interval: division by 0");
    T a[4] = {shim::div_dn(x.inf, y.inf), shim::div_dn(x.inf, y.sup), shim::div_dn(x.sup, y.inf),
              shim::div_dn(x.sup, y.sup)};
    T b[4] = {shim::div_up(x.inf, y.inf), shim::div_up(x.inf, y.sup), shim::div_up(x.sup, y.inf),
              shim::div_up(x.sup, y.sup)};
    return interval(*std::min_element(a, a + 4), *std::max_element(b, b + 4));
  }
  template <class C> friend interval operator+(const interval& x, const C& y) { return x + interval(y); }
  template <class C> friend interval operator+(const C& x, const interval& y) { return interval(x) + y; }
  template <class C> friend interval operator-(const interval& x, const C& y) { return x - interval(y); }
  template <class C> friend interval operator-(const C& x, const interval& y) { return interval(x) - y; }
  template <class C> friend interval operator*(const interval& x, const C& y) { return x * interval(y); }
  template <class C> friend interval operator*(const C& x, const interval& y) { return interval(x) * y; }
  template <class C> friend interval operator/(const interval& x, const C& y) { return x / interval(y); }
  template <class C> friend interval operator/(const C& x, const interval& y) { return interval(x) / y; }
  template <class C> interval& operator+=(const C& y) { *this = *this + y; return *this; }
  template <class C> interval& operator-=(const C& y) { *this = *this - y; return *this; }
  template <class C> interval& operator*=(const C& y) { *this = *this * y; return *this; }
  template <class C> interval& operator/=(const C& y) { *this = *this / y; return *this; }

  // "certainly" comparisons
  friend bool operator<(const interval& x, const interval& y) { return x.sup < y.inf; }
  friend bool operator<=(const interval& x, const interval& y) { return x.sup <= y.inf; }
  friend bool operator>(const interval& x, const interval& y) { return x.inf > y.sup; }
  friend bool operator>=(const interval& x, const interval& y) { return x.inf >= y.sup; }
  friend bool operator==(const interval& x, const interval& y) { return x.inf == y.inf && x.sup == y.sup; }
  friend bool operator!=(const interval& x, const interval& y) { return !(x == y); }
  template <class C> friend bool operator<(const interval& x, const C& y) { return x < interval(y); }
  template <class C> friend bool operator<(const C& x, const interval& y) { return interval(x) < y; }
  template <class C> friend bool operator>(const interval& x, const C& y) { return x > interval(y); }
  template <class C> friend bool operator>(const C& x, const interval& y) { return interval(x) > y; }
  template <class C> friend bool operator<=(const interval& x, const C& y) { return x <= interval(y); }
  template <class C> friend bool operator<=(const C& x, const interval& y) { return interval(x) <= y; }
  template <class C> friend bool operator>=(const interval& x, const C& y) { return x >= interval(y); }
  template <class C> friend bool operator>=(const C& x, const interval& y) { return interval(x) >= y; }
  template <class C> friend bool operator==(const interval& x, const C& y) { return x == interval(y); }
  template <class C> friend bool operator!=(const interval& x, const C& y) { return x != interval(y); }

  friend T mid(const interval& x) {
    volatile T a = x.inf, b = x.sup;
    shim::mode_guard g(FE_TONEAREST);
    volatile T s = a + b;
    volatile T r = std::isfinite((T)s) ? (T)s * T(0.5) : (T)a * T(0.5) + (T)b * T(0.5);
    return r;
  }
  friend T rad(const interval& x) {
    T m = mid(x);
    return std::max(shim::sub_up(m, x.inf), shim::sub_up(x.sup, m));
  }
  friend void midrad(const interval& x, T& m, T& r) {
    m = mid(x);
    r = std::max(shim::sub_up(m, x.inf), shim::sub_up(x.sup, m));
  }
  friend T width(const interval& x) { return shim::sub_up(x.sup, x.inf); }
  friend T norm(const interval& x) { return std::max(std::fabs(x.inf), std::fabs(x.sup)); }
  friend T mag(const interval& x) { return std::max(std::fabs(x.inf), std::fabs(x.sup)); }
  friend T mig(const interval& x) {
    if (x.inf <= 0 && x.sup >= 0) return T(0);
    return std::min(std::fabs(x.inf), std::fabs(x.sup));
  }
  friend interval abs(const interval& x) {
    if (x.inf >= 0) return x;
    if (x.sup <= 0) return -x;
    return interval(T(0), std::max(-x.inf, x.sup));
  }
  friend interval sqrt(const interval& x) {
    return interval(shim::sqrt_dn(std::max(x.inf, T(0))), shim::sqrt_up(x.sup));
  }
  friend interval pow(const interval& x, int n) {
    if (n == 0) return interval(T(1));
    if (n < 0) return interval(T(1)) / pow(x, -n);
    interval r = (n % 2 == 0) ? abs(x) : x;
    interval base = r;
    for (int i = 1; i < n; ++i) r = r * base;
    return r;
  }
  friend interval pow(const interval& x, const interval& y) {
    if (y.inf == y.sup && y.inf == std::floor(y.inf)) return pow(x, (int)y.inf);
    throw std::domain_error("kvshim interval: non-integer power");
  }
  template <class C> friend interval pow(const interval& x, const C& y) { return pow(x, interval(y)); }
  friend bool in(const T& a, const interval& x) { return x.inf <= a && a <= x.sup; }
  friend bool zero_in(const interval& x) { return x.inf <= 0 && x.sup >= 0; }
  friend bool subset(const interval& x, const interval& y) { return y.inf <= x.inf && x.sup <= y.sup; }
  friend bool proper_subset(const interval& x, const interval& y) { return y.inf < x.inf && x.sup < y.sup; }
  friend bool overlap(const interval& x, const interval& y) { return x.inf <= y.sup && y.inf <= x.sup; }
  friend interval intersect(const interval& x, const interval& y) {
    return interval(std::max(x.inf, y.inf), std::min(x.sup, y.sup));
  }
  friend interval hull(const interval& x, const interval& y) {
    return interval(std::min(x.inf, y.inf), std::max(x.sup, y.sup));
  }
  friend interval max(const interval& x, const interval& y) {
    return interval(std::max(x.inf, y.inf), std::max(x.sup, y.sup));
  }
  friend interval min(const interval& x, const interval& y) {
    return interval(std::min(x.inf, y.inf), std::min(x.sup, y.sup));
  }
  friend std::ostream& operator<<(std::ostream& s, const interval& x) {
    return s << "[" << x.inf << "," << x.sup << "]";
  }
};

}  // namespace kv

namespace std {
template <class T> class numeric_limits<kv::interval<T> > : public numeric_limits<T> {};
}
#endif
