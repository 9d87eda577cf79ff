// One-body transition operators of XSHLEMB (xmlshell/XSHLEMB.cpp): electric
// and magnetic multipoles, Gamow-Teller and Fermi beta operators in the
// m-scheme, with harmonic-oscillator radial integrals
// (include/sm/EMspherical2sp.cxx, include/xsm/xmlemb.cxx:121-206,
// include/sm/HO.cxx:71-112, include/sm/spherical2sp.cxx:664-700).
//
// Every operator is a list of terms v a+_f a_i (i annihilated, f created).
// The single-particle reduced matrix elements are those of Bohr and
// Mottelson vol. I (electric 3C-33, magnetic 3C-36, spin-dependent 3A-17) as
// the reference writes them, including its choices of phase: the factor
// i^(l_i - l_f + lambda) is dropped, and the full element is
// <f|| O ||i> <j_i m_i, lambda mu | j_f m_f> / sqrt(2 j_f + 1).  Radial
// integrals <n_f l_f| r^L |n_i l_i> in oscillator-length units follow
// Lawson's closed form (R. D. Lawson, Theory of the Nuclear Shell Model,
// eq. 1.11a), positive at the origin by default and positive at infinity
// (an extra (-1)^(n_f + n_i)) when `origin_positive` is false.
#include <algorithm>
#include <cmath>

#include "cosmo_gb300.h"
#include "em.h"

namespace cg {

namespace {

constexpr double kPi = 3.141592653589793238462643;

// n! with the value 1 for n <= 1 (also for negative n, where the closed form
// meets factorials of the l-forbidden cases the reference keeps)
double factorial(int n) {
  double r = 1.0;
  for (int i = 2; i <= n; ++i) r *= i;
  return r;
}
// n!! for odd n (1 for n <= 1)
double odd_factorial(int n) {
  double r = 1.0;
  for (int i = 3; i <= n; i += 2) r *= i;
  return r;
}
// (-1)^a for any integer a
inline double sgn(int a) { return (a & 1) ? -1.0 : 1.0; }

// Delta(abc) of the Racah formula, doubled arguments (0 when not a triangle)
double tri(int a, int b, int c) {
  if (c > a + b || c < std::abs(a - b) || ((a + b + c) & 1)) return 0.0;
  return std::sqrt(factorial((a + b - c) / 2) * factorial((a - b + c) / 2) * factorial((-a + b + c) / 2) /
                   factorial((a + b + c) / 2 + 1));
}

}  // namespace

double ho_radial(int L, int n1, int l1, int n2, int l2, bool origin_positive) {
  const int t1 = (l2 - l1 + L) / 2, t2 = (l1 - l2 + L) / 2;  // integers when l1 + l2 + L is even
  const int qmin = std::max(0, std::max(n1 - t1, n2 - t2)), qmax = std::min(n1, n2);
  if (qmin > qmax) return 0.0;
  double sum = 0.0;
  for (int q = qmin; q <= qmax; ++q)
    sum += odd_factorial(l1 + l2 + L + 2 * q + 1) /
           (std::pow(2.0, q) * factorial(q) * factorial(n1 - q) * factorial(n2 - q) * factorial(q + t2 - n2) *
            factorial(q + t1 - n1));
  double r = sum * std::sqrt(factorial(n1) * factorial(n2) / (odd_factorial(2 * n1 + 2 * l1 + 1) *
                                                             odd_factorial(2 * n2 + 2 * l2 + 1))) *
             std::pow(2.0, 0.5 * (n1 + n2 - L)) * factorial(t1) * factorial(t2);
  return (origin_positive && ((n1 + n2) & 1)) ? -r : r;
}

double six_j(int a, int b, int c, int d, int e, int f) {
  const double w = tri(a, b, c) * tri(a, e, f) * tri(d, b, f) * tri(d, e, c);
  if (w == 0.0) return 0.0;
  const int s1 = (a + b + c) / 2, s2 = (a + e + f) / 2, s3 = (d + b + f) / 2, s4 = (d + e + c) / 2;
  const int p1 = (a + b + d + e) / 2, p2 = (b + c + e + f) / 2, p3 = (c + a + f + d) / 2;
  double sum = 0.0;
  for (int t = std::max(std::max(s1, s2), std::max(s3, s4)); t <= std::min(p1, std::min(p2, p3)); ++t)
    sum += sgn(t) * factorial(t + 1) /
           (factorial(t - s1) * factorial(t - s2) * factorial(t - s3) * factorial(t - s4) * factorial(p1 - t) *
            factorial(p2 - t) * factorial(p3 - t));
  return w * sum;
}

double three_j(int j1, int m1, int j2, int m2, int j3, int m3) {
  if (m1 + m2 + m3 != 0) return 0.0;
  return sgn((j1 - j2 - m3) / 2) * clebsch_gordan(j1, m1, j2, m2, j3, -m3) / std::sqrt(j3 + 1.0);
}

namespace {

// <f| Q_lambda,mu |i> from the reduced element (ReducedToFull,
// include/sm/EMspherical2sp.cxx:59-68)
double reduced_to_full(const SPState& f, const SPState& i, int K, double reduced) {
  return reduced * clebsch_gordan(i.j2, i.m2, 2 * K, f.m2 - i.m2, f.j2, f.m2) / std::sqrt(double(f.j2 + 1));
}

// <f|| (Y_q sigma)_K ||i> of the spin-dependent operator (ROperator_YS,
// include/sm/EMspherical2sp.cxx:303-356), without the radial part
double y_sigma(const SPState& f, const SPState& i, int q, int K) {
  if ((i.parity - f.parity + q) & 1) return 0.0;
  const double base = std::sqrt((i.j2 + 1.0) / kPi) / 2.0;
  const double lo = clebsch_gordan(i.j2, 1, 2 * K, 0, f.j2, 1);   // <j_i 1/2, K 0 | j_f 1/2>
  const double hi = clebsch_gordan(i.j2, -1, 2 * K, 2, f.j2, 1);  // <j_i -1/2, K 1 | j_f 1/2>
  const double ph = sgn((f.j2 - 1) / 2 - f.l);                    // (-1)^(j_f - l_f - 1/2)
  switch (K - q) {
    case -1:
      return base * (sgn((i.j2 - f.j2) / 2 + K) * lo * std::sqrt(2.0 * K + 1.0) - hi * ph * std::sqrt(double(K)));
    case 0:
      return base * ph * hi * std::sqrt(2.0 * K + 1.0);
    case 1:
      return base * (sgn((i.j2 + f.j2) / 2 + K) * lo * std::sqrt(double(K)) - hi * ph * std::sqrt(K + 1.0));
    default:
      return 0.0;
  }
}

}  // namespace

std::vector<OneBodyTerm> transition_terms(const System& sys, const TransitionOp& op, int kappa) {
  std::vector<OneBodyTerm> out;
  const int ns = int(sys.sps.size());
  const int K = op.K;
  const char type = op.name.empty() ? '?' : op.name[0];
  if (type == 'F') {
    // T+ over every pair of s.p. states that differ only in tz, and its
    // conjugate (SPTPlus + Hermitian2FullOperator): a+_n a_p and a+_p a_n
    for (int a = 0; a < ns; ++a)
      for (int b = a + 1; b < ns; ++b) {
        const SPState &x = sys.sps[a], &y = sys.sps[b];
        if (x.m2 != y.m2 || x.n != y.n || x.parity != y.parity || x.l != y.l || x.t2 != y.t2 || x.j2 != y.j2) continue;
        if (std::abs(x.tz2 - y.tz2) != 2) continue;
        const SPState& p = x.tz2 < y.tz2 ? x : y;  // the proton of the pair
        const double v = std::sqrt((p.t2 - p.tz2) * (p.t2 + p.tz2 + 2.0)) / 2.0;
        const int ip = x.tz2 < y.tz2 ? a : b, in = x.tz2 < y.tz2 ? b : a;
        out.push_back({ip, in, v});
        out.push_back({in, ip, v});
      }
    return out;
  }
  for (int f = 0; f < ns; ++f)
    for (int i = 0; i < ns; ++i) {
      const SPState &sf = sys.sps[f], &si = sys.sps[i];
      if (si.m2 + 2 * kappa != sf.m2) continue;
      double v = 0.0;
      if (type == 'E') {
        if (sf.tz2 != si.tz2 || ((si.l + K - sf.l) & 1)) continue;
        v = sf.tz2 == 1 ? op.en : op.ep;
        if ((((si.j2 - sf.j2) / 2) + K) & 1) v = -v;
        v *= std::sqrt((2.0 * K + 1.0) * (si.j2 + 1.0) / (4.0 * kPi));
        v *= ho_radial(K, sf.n, sf.l, si.n, si.l, op.origin_positive);
        v *= clebsch_gordan(si.j2, 1, 2 * K, 0, sf.j2, 1);
      } else if (type == 'M') {
        if (sf.tz2 != si.tz2 || ((si.l - sf.l + K - 1) & 1)) continue;
        const bool neutron = sf.tz2 == 1;
        const double gl = neutron ? op.gl_n : op.gl_p, gs = 2.0 * (neutron ? op.mu_n : op.mu_p);
        // A term: (g_s - 2 g_l/(K+1)) K/2 <j_i 1/2, K 0|j_f 1/2> [1 + (-1)^(l_i+1/2-j_i)/K {...}]
        double a = sgn((si.j2 + sf.j2) / 2 - K) * (sf.j2 + 1.0) / 2.0 + (si.j2 + 1.0) / 2.0;
        a *= sgn(si.l - (si.j2 - 1) / 2) / double(K);
        a += 1.0;
        a *= clebsch_gordan(si.j2, 1, 2 * K, 0, sf.j2, 1);
        a *= double(K) / 2.0;
        a *= gs - 2.0 * gl / (double(K) + 1.0);
        // B term: 6j {j_i 1 j_i; K-1 j_f K} <j_i 1/2, K-1 0|j_f 1/2> ...
        double b = six_j(si.j2, 2, si.j2, 2 * K - 2, sf.j2, 2 * K);
        b *= clebsch_gordan(si.j2, 1, 2 * K - 2, 0, sf.j2, 1);
        b *= std::sqrt(K * (4.0 * K * K - 1) * si.j2 * (si.j2 + 2.0) * (si.j2 + 1)) * gl;
        b *= sgn((si.j2 + sf.j2) / 2 + K) / (double(K) + 1.0);
        v = a + b;
        if (((si.j2 - sf.j2) / 2 + K - 1) & 1) v = -v;
        v *= std::sqrt((2.0 * K + 1.0) * (si.j2 + 1.0) / (4.0 * kPi));
        v *= ho_radial(K - 1, sf.n, sf.l, si.n, si.l, op.origin_positive);
      } else if (type == 'G') {
        const bool plus = op.name.size() > 2 && op.name[2] == '+';  // GT+: p -> n, GT-: n -> p
        if (sf.tz2 != si.tz2 + (plus ? 2 : -2) || ((si.l - sf.l) & 1)) continue;
        // (the reference takes the default radial phase here whatever the flag)
        v = y_sigma(sf, si, 0, K) * ho_radial(0, sf.n, sf.l, si.n, si.l, true);
        if (v == 0.0) continue;
        v = reduced_to_full(sf, si, K, v);
        v *= plus ? std::sqrt((si.t2 - si.tz2) * (si.t2 + si.tz2 + 2.0)) / 2.0
                  : std::sqrt((si.t2 + si.tz2) * (si.t2 - si.tz2 + 2.0)) / 2.0;
        v *= std::sqrt(4.0 * kPi);  // units g_A^2 / (4 pi)
        out.push_back({i, f, v});
        continue;
      } else {
        throw Error(CG_ERR_ARG, "transition operator " + op.name + ": not E, M, GT+, GT- or F");
      }
      if (v == 0.0) continue;
      out.push_back({i, f, reduced_to_full(sf, si, K, v)});
    }
  return out;
}

double oscillator_b2(int A) {
  const double hw = 45.0 * std::pow(double(A), -1.0 / 3.0) - 25.0 * std::pow(double(A), -2.0 / 3.0);
  return kHbarC * kHbarC / (hw * 938.9186945);
}

double weisskopf_units(char type, int L, int A, double B) {
  const double b = oscillator_b2(A);
  if (type == 'E')
    return std::pow(b, L) * B /
           (std::pow(1.2, 2 * L) * (3.0 / (L + 3.0)) * (3.0 / (L + 3.0)) * std::pow(double(A), 2 * L / 3.0) / (4 * kPi));
  if (type == 'M')
    return std::pow(b, L - 1) * B /
           (10.0 * std::pow(1.2, 2 * L - 2) * (3.0 / (L + 3.0)) * (3.0 / (L + 3.0)) *
            std::pow(double(A), (2 * L - 2) / 3.0) / kPi);
  return -1.0;
}

double standard_units(char type, int L, int A, double B) {
  const double b = oscillator_b2(A);
  if (type == 'E') return std::pow(b, L) * B;
  if (type == 'M') return std::pow(b, L - 1) * B;
  return -1.0;
}

}  // namespace cg
