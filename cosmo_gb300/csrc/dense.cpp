#include "dense.h"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace cg {

// Householder reduction to tridiagonal form (accumulating the transformation)
// and implicit QL with Wilkinson shifts, written from the textbook algorithm
// (Wilkinson & Reinsch, Handbook for Automatic Computation II, tred2/tql2).
void sym_eig(int n, const std::vector<double>& a, std::vector<double>& w, std::vector<double>& zout) {
  std::vector<double> z(a), d(n), e(n);
  auto Z = [&](int i, int j) -> double& { return z[size_t(i) * n + j]; };
  // tred2
  for (int i = n - 1; i > 0; --i) {
    int l = i - 1;
    double h = 0.0, scale = 0.0;
    if (l > 0) {
      for (int k = 0; k <= l; ++k) scale += std::fabs(Z(i, k));
      if (scale == 0.0) {
        e[i] = Z(i, l);
      } else {
        for (int k = 0; k <= l; ++k) {
          Z(i, k) /= scale;
          h += Z(i, k) * Z(i, k);
        }
        double f = Z(i, l);
        double g = f >= 0.0 ? -std::sqrt(h) : std::sqrt(h);
        e[i] = scale * g;
        h -= f * g;
        Z(i, l) = f - g;
        f = 0.0;
        for (int j = 0; j <= l; ++j) {
          Z(j, i) = Z(i, j) / h;
          g = 0.0;
          for (int k = 0; k <= j; ++k) g += Z(j, k) * Z(i, k);
          for (int k = j + 1; k <= l; ++k) g += Z(k, j) * Z(i, k);
          e[j] = g / h;
          f += e[j] * Z(i, j);
        }
        double hh = f / (h + h);
        for (int j = 0; j <= l; ++j) {
          f = Z(i, j);
          e[j] = g = e[j] - hh * f;
          for (int k = 0; k <= j; ++k) Z(j, k) -= (f * e[k] + g * Z(i, k));
        }
      }
    } else {
      e[i] = Z(i, l);
    }
    d[i] = h;
  }
  d[0] = 0.0;
  e[0] = 0.0;
  for (int i = 0; i < n; ++i) {
    int l = i - 1;
    if (d[i] != 0.0) {
      for (int j = 0; j <= l; ++j) {
        double g = 0.0;
        for (int k = 0; k <= l; ++k) g += Z(i, k) * Z(k, j);
        for (int k = 0; k <= l; ++k) Z(k, j) -= g * Z(k, i);
      }
    }
    d[i] = Z(i, i);
    Z(i, i) = 1.0;
    for (int j = 0; j <= l; ++j) Z(j, i) = Z(i, j) = 0.0;
  }
  // tql2
  for (int i = 1; i < n; ++i) e[i - 1] = e[i];
  if (n > 0) e[n - 1] = 0.0;
  for (int l = 0; l < n; ++l) {
    int iter = 0, m;
    do {
      for (m = l; m < n - 1; ++m) {
        double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= 1e-16 * dd) break;
      }
      if (m != l) {
        if (++iter > 60) break;
        double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
        double r = std::hypot(g, 1.0);
        g = d[m] - d[l] + e[l] / (g + (g >= 0.0 ? std::fabs(r) : -std::fabs(r)));
        double s = 1.0, c = 1.0, p = 0.0;
        int i;
        for (i = m - 1; i >= l; --i) {
          double f = s * e[i], b = c * e[i];
          e[i + 1] = (r = std::hypot(f, g));
          if (r == 0.0) {
            d[i + 1] -= p;
            e[m] = 0.0;
            break;
          }
          s = f / r;
          c = g / r;
          g = d[i + 1] - p;
          r = (d[i] - g) * s + 2.0 * c * b;
          d[i + 1] = g + (p = s * r);
          g = c * r - b;
          for (int k = 0; k < n; ++k) {
            f = Z(k, i + 1);
            Z(k, i + 1) = s * Z(k, i) + c * f;
            Z(k, i) = c * Z(k, i) - s * f;
          }
        }
        if (r == 0.0 && i >= l) continue;
        d[l] -= p;
        e[l] = g;
        e[m] = 0.0;
      }
    } while (m != l);
  }
  // sort ascending
  std::vector<int> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return d[x] < d[y]; });
  w.resize(n);
  zout.assign(size_t(n) * n, 0.0);
  for (int k = 0; k < n; ++k) {
    w[k] = d[idx[k]];
    for (int i = 0; i < n; ++i) zout[size_t(i) * n + k] = Z(i, idx[k]);
  }
}

int cholesky(int n, std::vector<double>& a) {
  for (int j = 0; j < n; ++j) {
    double s = a[size_t(j) * n + j];
    for (int k = 0; k < j; ++k) s -= a[size_t(j) * n + k] * a[size_t(j) * n + k];
    if (!(s > 0.0)) return j;
    double l = std::sqrt(s);
    a[size_t(j) * n + j] = l;
    for (int i = j + 1; i < n; ++i) {
      double t = a[size_t(i) * n + j];
      for (int k = 0; k < j; ++k) t -= a[size_t(i) * n + k] * a[size_t(j) * n + k];
      a[size_t(i) * n + j] = t / l;
    }
  }
  return -1;
}

}  // namespace cg
