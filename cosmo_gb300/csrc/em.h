// One-body transition operators (electric, magnetic, Gamow-Teller, Fermi) of
// XSHLEMB (xmlshell/XSHLEMB.cpp, include/sm/EMspherical2sp.cxx) and the
// angular-momentum and oscillator helpers they need.
#pragma once
#include <string>
#include <vector>

#include "model.h"

namespace cg {

constexpr double kHbarC = 197.327053;  // MeV fm
constexpr double kMuProton = 2.792847351, kMuNeutron = -1.91304273;  // nuclear magnetons

// v a+_f a_i
struct OneBodyTerm {
  int i, f;
  double v;
};

// The <operator> node: name E<K>, M<K>, GT+, GT- or F; multipolarity K;
// effective charges (E), moments and orbital g factors (M); the oscillator
// radial phase (positive at the origin unless -p).
struct TransitionOp {
  std::string name;
  int K = 0;
  double en = 0.0, ep = 0.0;
  double mu_n = kMuNeutron, mu_p = kMuProton, gl_n = 0.0, gl_p = 1.0;
  bool origin_positive = true;
};

// <n1 l1| r^L |n2 l2> for oscillator functions (oscillator length 1).
double ho_radial(int L, int n1, int l1, int n2, int l2, bool origin_positive);
// Wigner 6j and 3j symbols, doubled arguments.
double six_j(int a, int b, int c, int d, int e, int f);
double three_j(int j1, int m1, int j2, int m2, int j3, int m3);
// The m-scheme terms of the operator component with projection kappa
// (m_f = m_i + 2 kappa in doubled units).
std::vector<OneBodyTerm> transition_terms(const System& sys, const TransitionOp& op, int kappa);
// Squared oscillator length b^2 (fm^2) for mass number A, hw = 45 A^-1/3 - 25 A^-2/3.
double oscillator_b2(int A);
// B in Weisskopf units / in e^2 fm^2L (E) or mu_N^2 fm^(2L-2) (M); -1 for other types.
double weisskopf_units(char type, int L, int A, double B);
double standard_units(char type, int L, int A, double B);

}  // namespace cg
