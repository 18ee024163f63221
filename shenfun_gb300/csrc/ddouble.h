// Double-double arithmetic on the host: a value is the unevaluated sum
// hi + lo of two doubles with |lo| <= ulp(hi) / 2, about 106 bits.  Used for
// the set-up of plans (twiddle factors, Rader kernel spectra, Legendre nodes
// and matrices) whose results are rounded to FP64 or to double-float pairs:
// the extra bits make every stored entry the correctly rounded (or nearly
// so) value of its exact expression.  Hardware doubles with FMA make this
// ~10-50x cheaper than a software long double (128-bit quad precision on
// aarch64 hosts).
//
// The building blocks are the classical error-free transformations: Knuth's
// TwoSum (TAOCP vol. 2, 4.2.2), the FMA form of Dekker's TwoProduct (Dekker
// 1971; Ogita, Rump & Oishi 2005), and the double-double add, multiply and
// divide built on them as in Hida, Li & Bailey, "Algorithms for quad-double
// precision floating point arithmetic" (ARITH 2001).  Sine and cosine use
// an exact rational reduction of the angle (2 pi p / q with integers p, q)
// to |theta| <= pi / 4 and the Taylor series there.
#pragma once

#include <cmath>
#include <cstdint>

namespace sgpu {
namespace ddm {

struct dd {
  double hi, lo;
  dd() : hi(0.0), lo(0.0) {}
  dd(double h) : hi(h), lo(0.0) {}  // NOLINT: implicit from double
  dd(double h, double l) : hi(h), lo(l) {}
};

// s + e = a + b exactly
inline dd two_sum(double a, double b) {
  const double s = a + b;
  const double bb = s - a;
  return dd(s, (a - (s - bb)) + (b - bb));
}

// as two_sum, for |a| >= |b|
inline dd quick_two_sum(double a, double b) {
  const double s = a + b;
  return dd(s, b - (s - a));
}

// p + e = a * b exactly
inline dd two_prod(double a, double b) {
  const double p = a * b;
  return dd(p, std::fma(a, b, -p));
}

inline dd operator+(const dd& a, const dd& b) {
  dd s = two_sum(a.hi, b.hi);
  const dd t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}

inline dd operator-(const dd& a) { return dd(-a.hi, -a.lo); }
inline dd operator-(const dd& a, const dd& b) { return a + (-b); }

inline dd operator*(const dd& a, const dd& b) {
  dd p = two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return quick_two_sum(p.hi, p.lo);
}

inline dd operator*(const dd& a, double b) {
  dd p = two_prod(a.hi, b);
  p.lo += a.lo * b;
  return quick_two_sum(p.hi, p.lo);
}
inline dd operator*(double a, const dd& b) { return b * a; }

// long division in three partial quotients
inline dd operator/(const dd& a, const dd& b) {
  const double q1 = a.hi / b.hi;
  dd r = a - b * q1;
  const double q2 = r.hi / b.hi;
  r = r - b * q2;
  const double q3 = r.hi / b.hi;
  return quick_two_sum(q1, q2) + dd(q3);
}

inline dd operator/(const dd& a, double b) { return a / dd(b); }

inline dd& operator+=(dd& a, const dd& b) { return a = a + b; }
inline dd& operator-=(dd& a, const dd& b) { return a = a - b; }
inline dd& operator*=(dd& a, const dd& b) { return a = a * b; }
inline dd& operator/=(dd& a, const dd& b) { return a = a / b; }

inline double to_double(const dd& a) { return a.hi + a.lo; }
inline dd dabs(const dd& a) { return a.hi < 0 ? -a : a; }

// pi as a double-double: the nearest double and the nearest double of the rest
inline dd dd_pi() { return dd(3.141592653589793116e+00, 1.2246467991473532072e-16); }

// cos and sin of theta, |theta| <= pi / 4, by their Taylor series (terms
// below 2^-110 of the result are dropped: at most 15 of each)
inline void sincos_reduced(const dd& theta, dd& c, dd& s) {
  const dd t2 = theta * theta;
  dd term = theta;  // theta^(2k+1) / (2k+1)!, signed
  s = theta;
  for (int k = 1; k < 20; ++k) {
    term = -(term * t2) / (double)((2 * k) * (2 * k + 1));
    s += term;
    if (std::fabs(term.hi) < 1e-34) break;
  }
  term = dd(1.0);  // theta^(2k) / (2k)!, signed
  c = dd(1.0);
  for (int k = 1; k < 20; ++k) {
    term = -(term * t2) / (double)((2 * k - 1) * (2 * k));
    c += term;
    if (std::fabs(term.hi) < 1e-34) break;
  }
}

// cos(2 pi p / q) and sin(2 pi p / q) for integers p and q > 0: the
// quadrant is taken exactly in integers, leaving theta = pi r / (2 q) with
// the integer r = 4 p' - j q, |r| <= q / 2 (p' = p mod q, j the nearest
// quarter turn), so that |theta| <= pi / 4
inline void sincos_2pi_frac(int64_t p, int64_t q, dd& c, dd& s) {
  int64_t pm = p % q;
  if (pm < 0) pm += q;
  const int64_t four_p = 4 * pm;
  int64_t j = (four_p + q / 2) / q;  // nearest quarter turn, 0..4
  const int64_t r = four_p - j * q;
  const dd theta = dd_pi() * (double)r / (double)(2 * q);
  dd ct, st;
  sincos_reduced(theta, ct, st);
  switch (j & 3) {
    case 0: c = ct; s = st; break;
    case 1: c = -st; s = ct; break;
    case 2: c = -ct; s = -st; break;
    default: c = st; s = -ct; break;
  }
}

}  // namespace ddm
}  // namespace sgpu
