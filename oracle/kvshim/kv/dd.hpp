// kv/dd.hpp -- project-written stand-in for kv::dd (the kv library is absent
// here).  Written to kv's public API names only, so that the unmodified VCP
// headers (vcp/pddblas.hpp) compile against it.  A dd value is the unevaluated
// sum a1 + a2 of two doubles with |a2| <= ulp(a1) / 2.  The arithmetic is the
// published double-double algorithms (Knuth's TwoSum, TwoProd by fused
// multiply-add, Dekker's normalisation), in round-to-nearest.  TEST
// INFRASTRUCTURE ONLY.
#ifndef DD_HPP
#define DD_HPP
#include <cmath>
#include <iostream>

namespace kv {

class dd {
 public:
  double a1, a2;

  dd() : a1(0.0), a2(0.0) {}
  dd(double x) : a1(x), a2(0.0) {}
  dd(int x) : a1((double)x), a2(0.0) {}
  dd(double x, double y) {
    twosum(x, y, a1, a2);
  }

  static void twosum(double a, double b, double& s, double& e) {
    s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
  }
  static void fasttwosum(double a, double b, double& s, double& e) {
    s = a + b;
    e = b - (s - a);
  }
  static void twoproduct(double a, double b, double& p, double& e) {
    p = a * b;
    e = std::fma(a, b, -p);
  }

  friend dd operator+(const dd& x, const dd& y) {
    double s, e, t, f;
    twosum(x.a1, y.a1, s, e);
    twosum(x.a2, y.a2, t, f);
    e += t;
    fasttwosum(s, e, s, e);
    e += f;
    dd r;
    fasttwosum(s, e, r.a1, r.a2);
    return r;
  }
  friend dd operator-(const dd& x) {
    dd r;
    r.a1 = -x.a1;
    r.a2 = -x.a2;
    return r;
  }
  friend dd operator-(const dd& x, const dd& y) { return x + (-y); }
  friend dd operator*(const dd& x, const dd& y) {
    double p, e;
    twoproduct(x.a1, y.a1, p, e);
    // the cross terms as one explicit fused multiply-add, so that the result
    // does not depend on the compiler's contraction setting
    e += std::fma(x.a1, y.a2, x.a2 * y.a1);
    dd r;
    fasttwosum(p, e, r.a1, r.a2);
    return r;
  }
  friend dd operator/(const dd& x, const dd& y) {
    // one Newton correction of the leading quotient
    const double q1 = x.a1 / y.a1;
    const dd r = x - y * dd(q1);
    const double q2 = r.a1 / y.a1;
    dd out;
    fasttwosum(q1, q2, out.a1, out.a2);
    return out;
  }
  dd& operator+=(const dd& y) { return *this = *this + y; }
  dd& operator-=(const dd& y) { return *this = *this - y; }
  dd& operator*=(const dd& y) { return *this = *this * y; }
  dd& operator/=(const dd& y) { return *this = *this / y; }

  friend bool operator<(const dd& x, const dd& y) {
    return x.a1 < y.a1 || (x.a1 == y.a1 && x.a2 < y.a2);
  }
  friend bool operator>(const dd& x, const dd& y) { return y < x; }
  friend bool operator<=(const dd& x, const dd& y) { return !(y < x); }
  friend bool operator>=(const dd& x, const dd& y) { return !(x < y); }
  friend bool operator==(const dd& x, const dd& y) { return x.a1 == y.a1 && x.a2 == y.a2; }
  friend bool operator!=(const dd& x, const dd& y) { return !(x == y); }

  friend dd abs(const dd& x) { return x.a1 < 0.0 || (x.a1 == 0.0 && x.a2 < 0.0) ? -x : x; }
  friend dd sqrt(const dd& x) {
    if (x.a1 <= 0.0) return dd(0.0);
    const double s = std::sqrt(x.a1);
    const dd r = x - dd(s) * dd(s);
    dd out;
    fasttwosum(s, r.a1 / (2.0 * s), out.a1, out.a2);
    return out;
  }
  friend dd pow(const dd& x, int n) {  // binary powering
    dd r(1.0), b = x;
    unsigned e = n < 0 ? (unsigned)(-n) : (unsigned)n;
    while (e) {
      if (e & 1u) r *= b;
      b *= b;
      e >>= 1;
    }
    return n < 0 ? dd(1.0) / r : r;
  }
  friend std::ostream& operator<<(std::ostream& o, const dd& x) {
    return o << x.a1 << (x.a2 < 0 ? " - " : " + ") << std::fabs(x.a2);
  }
};

}  // namespace kv

#endif  // DD_HPP
