// Symmetric eigen-solvers for LMOD: the dense solver sym_eigen and the
// thick-restart Lanczos iteration LowModes that stands in for ARPACK
// (declarations and references in lowmodes.h).
#include "lowmodes.h"

#include <cmath>

namespace sffg {
namespace {

constexpr double kEps = 2.2204460492503131e-16;
// (2^-53)^(2/3): ARPACK's floor for the relative residual test
constexpr double kEps23 = 2.3099725541661633e-11;

double dot(int n, const double *a, const double *b) {
  double s = 0.0;
  for (int i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

}  // namespace

int sym_eigen(int n, double *a, double *d, double *z) {
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) z[i * n + j] = (i == j) ? 1.0 : 0.0;
  std::vector<double> v(n), p(n), e(n > 0 ? n : 1, 0.0);
  // Householder reduction: column k's entries below the subdiagonal are
  // reflected onto a[k+1][k]; the trailing block takes the two-sided update
  // A <- H A H as A - v w^T - w v^T with w = p - (beta v.p / 2) v, p = beta A v.
  for (int k = 0; k + 2 < n; k++) {
    double sigma = 0.0;
    for (int i = k + 2; i < n; i++) sigma += a[i * n + k] * a[i * n + k];
    if (sigma == 0.0) continue;
    const double x0 = a[(k + 1) * n + k];
    double alpha = std::sqrt(x0 * x0 + sigma);
    if (x0 > 0.0) alpha = -alpha;
    v[k + 1] = x0 - alpha;
    for (int i = k + 2; i < n; i++) v[i] = a[i * n + k];
    const double beta = 2.0 / (v[k + 1] * v[k + 1] + sigma);
    double vp = 0.0;
    for (int i = k + 1; i < n; i++) {
      double s = 0.0;
      for (int j = k + 1; j < n; j++) s += a[i * n + j] * v[j];
      p[i] = beta * s;
      vp += v[i] * p[i];
    }
    const double half = 0.5 * beta * vp;
    for (int i = k + 1; i < n; i++) p[i] -= half * v[i];
    for (int i = k + 1; i < n; i++)
      for (int j = k + 1; j < n; j++) a[i * n + j] -= v[i] * p[j] + p[i] * v[j];
    a[(k + 1) * n + k] = a[k * n + k + 1] = alpha;
    for (int i = k + 2; i < n; i++) a[i * n + k] = a[k * n + i] = 0.0;
    for (int r = 0; r < n; r++) {
      double s = 0.0;
      for (int i = k + 1; i < n; i++) s += z[r * n + i] * v[i];
      s *= beta;
      for (int i = k + 1; i < n; i++) z[r * n + i] -= s * v[i];
    }
  }
  for (int i = 0; i < n; i++) d[i] = a[i * n + i];
  for (int i = 0; i + 1 < n; i++) e[i] = a[(i + 1) * n + i];
  // implicit symmetric QR steps with the Wilkinson shift on the unreduced
  // trailing block lo..hi, chasing the bulge with Givens rotations
  int sweeps = 0;
  for (int hi = n - 1; hi > 0;) {
    if (std::fabs(e[hi - 1]) <= kEps * (std::fabs(d[hi - 1]) + std::fabs(d[hi]))) {
      e[hi - 1] = 0.0;
      hi--;
      continue;
    }
    int lo = hi - 1;
    while (lo > 0 && std::fabs(e[lo - 1]) > kEps * (std::fabs(d[lo - 1]) + std::fabs(d[lo]))) lo--;
    if (lo > 0) e[lo - 1] = 0.0;
    if (++sweeps > 30 * n) return -1;
    const double delta = 0.5 * (d[hi - 1] - d[hi]);
    const double b2 = e[hi - 1] * e[hi - 1];
    const double root = std::fabs(delta) + std::sqrt(delta * delta + b2);
    const double mu = d[hi] - b2 / (delta >= 0.0 ? root : -root);
    double x = d[lo] - mu, y = e[lo];
    for (int k = lo; k < hi; k++) {
      const double r = std::sqrt(x * x + y * y);
      double c = 1.0, s = 0.0;
      if (r > 0.0) {
        c = x / r;
        s = y / r;
      }
      if (k > lo) e[k - 1] = r;
      const double a0 = d[k], b = e[k], d1 = d[k + 1];
      d[k] = c * c * a0 + 2.0 * c * s * b + s * s * d1;
      d[k + 1] = s * s * a0 - 2.0 * c * s * b + c * c * d1;
      e[k] = c * s * (d1 - a0) + (c * c - s * s) * b;
      if (k + 1 < hi) {
        x = e[k];
        y = s * e[k + 1];
        e[k + 1] = c * e[k + 1];
      }
      for (int i = 0; i < n; i++) {
        const double q0 = z[i * n + k], q1 = z[i * n + k + 1];
        z[i * n + k] = c * q0 + s * q1;
        z[i * n + k + 1] = c * q1 - s * q0;
      }
    }
  }
  // descending order, columns moved with their values
  for (int i = 0; i + 1 < n; i++) {
    int k = i;
    for (int j = i + 1; j < n; j++)
      if (d[j] > d[k]) k = j;
    if (k == i) continue;
    const double t = d[i];
    d[i] = d[k];
    d[k] = t;
    for (int r = 0; r < n; r++) {
      const double q = z[r * n + i];
      z[r * n + i] = z[r * n + k];
      z[r * n + k] = q;
    }
  }
  return 0;
}

int LowModes::init(int n, int nev, int ncv, double tol, int max_restarts) {
  if (n < 1 || nev < 1 || ncv <= nev || ncv > n) return -1;
  n_ = n;
  nev_ = nev;
  ncv_ = ncv;
  tol_ = tol > 0.0 ? tol : 0.5 * kEps;
  max_restarts_ = max_restarts;
  V_.assign(static_cast<size_t>(n) * ncv, 0.0);
  H_.assign(static_cast<size_t>(ncv) * ncv, 0.0);
  x_.assign(n, 0.0);
  y_.assign(n, 0.0);
  r_.assign(n, 0.0);
  h_.assign(2 * static_cast<size_t>(ncv), 0.0);
  val_.clear();
  vec_.clear();
  j_ = restarts_ = products_ = nconv_ = 0;
  state_ = 0;
  rng_ = 0x2545F4914F6CDD1DULL;
  return 0;
}

// A unit vector of uniform(-1, 1) entries from a 64-bit linear congruential
// generator (Knuth's MMIX constants), the same on every host.
void LowModes::random_unit(double *v) {
  for (int i = 0; i < n_; i++) {
    rng_ = rng_ * 6364136223846793005ULL + 1442695040888963407ULL;
    v[i] = 2.0 * (static_cast<double>(rng_ >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
  }
  const double s = std::sqrt(dot(n_, v, v));
  for (int i = 0; i < n_; i++) v[i] /= s;
}

// w -= V h with h = V^T w over the first ncols basis vectors, twice
// (classical Gram-Schmidt with one re-orthogonalisation); h returns the sum
// of both passes' coefficients.
void LowModes::orthogonalise(double *w, int ncols, double *h) {
  double *c = h_.data() + ncv_;
  for (int i = 0; i < ncols; i++) h[i] = dot(n_, V_.data() + static_cast<size_t>(i) * n_, w);
  for (int i = 0; i < ncols; i++) {
    const double *vi = V_.data() + static_cast<size_t>(i) * n_;
    for (int t = 0; t < n_; t++) w[t] -= h[i] * vi[t];
  }
  for (int i = 0; i < ncols; i++) c[i] = dot(n_, V_.data() + static_cast<size_t>(i) * n_, w);
  for (int i = 0; i < ncols; i++) {
    const double *vi = V_.data() + static_cast<size_t>(i) * n_;
    for (int t = 0; t < n_; t++) w[t] -= c[i] * vi[t];
    h[i] += c[i];
  }
}

int LowModes::iterate() {
  if (state_ == 0) {
    random_unit(V_.data());
    j_ = 0;
    state_ = 1;
  } else if (state_ == 1) {
    // column j_'s product is in y_: extend the basis
    const double ynorm = std::sqrt(dot(n_, y_.data(), y_.data()));
    for (int t = 0; t < n_; t++) r_[t] = y_[t];
    orthogonalise(r_.data(), j_ + 1, h_.data());
    for (int i = 0; i <= j_; i++) H_[static_cast<size_t>(i) * ncv_ + j_] = H_[static_cast<size_t>(j_) * ncv_ + i] = h_[i];
    const double beta = std::sqrt(dot(n_, r_.data(), r_.data()));
    if (j_ + 1 < ncv_) {
      double *next = V_.data() + static_cast<size_t>(j_ + 1) * n_;
      if (beta > 1e-10 * ynorm && beta > 0.0) {
        for (int t = 0; t < n_; t++) next[t] = r_[t] / beta;
      } else {
        // invariant subspace: continue from a fresh direction
        random_unit(next);
        orthogonalise(next, j_ + 1, h_.data());
        const double s = std::sqrt(dot(n_, next, next));
        for (int t = 0; t < n_; t++) next[t] /= s;
      }
      j_++;
    } else {
      const int rc = finish_sweep();
      if (rc <= 0) {
        state_ = 2;
        return rc;
      }
    }
  } else {
    return 0;
  }
  const double *col = V_.data() + static_cast<size_t>(j_) * n_;
  for (int t = 0; t < n_; t++) x_[t] = col[t];
  products_++;
  return 1;
}

// Rayleigh-Ritz on the full basis: test the wanted Ritz pairs and either
// return them (0; -1 if none converged) or restart with the best half of
// the basis kept (1, j_ set to the first new column).
int LowModes::finish_sweep() {
  const int m = ncv_;
  std::vector<double> A(H_), theta(m), S(static_cast<size_t>(m) * m);
  if (sym_eigen(m, A.data(), theta.data(), S.data())) return -1;
  // Ritz values by increasing magnitude (ties keep the descending order)
  std::vector<int> idx(m);
  for (int i = 0; i < m; i++) idx[i] = i;
  for (int i = 1; i < m; i++) {
    const int t = idx[i];
    int k = i - 1;
    while (k >= 0 && std::fabs(theta[idx[k]]) > std::fabs(theta[t])) {
      idx[k + 1] = idx[k];
      k--;
    }
    idx[k + 1] = t;
  }
  const double beta = std::sqrt(dot(n_, r_.data(), r_.data()));
  std::vector<int> good;
  for (int k = 0; k < nev_; k++) {
    const int i = idx[k];
    const double res = beta * std::fabs(S[static_cast<size_t>(m - 1) * m + i]);
    const double scale = std::fabs(theta[i]) > kEps23 ? std::fabs(theta[i]) : kEps23;
    if (res <= tol_ * scale) good.push_back(i);
  }
  const bool done = static_cast<int>(good.size()) == nev_ || m == n_ || restarts_ >= max_restarts_;
  if (done) {
    // converged pairs in ascending algebraic order
    for (size_t a = 1; a < good.size(); a++) {
      const int t = good[a];
      size_t k = a;
      while (k > 0 && theta[good[k - 1]] > theta[t]) {
        good[k] = good[k - 1];
        k--;
      }
      good[k] = t;
    }
    nconv_ = static_cast<int>(good.size());
    val_.assign(nconv_, 0.0);
    vec_.assign(static_cast<size_t>(nconv_) * n_, 0.0);
    for (int k = 0; k < nconv_; k++) {
      const int i = good[k];
      val_[k] = theta[i];
      double *out = vec_.data() + static_cast<size_t>(k) * n_;
      for (int c = 0; c < m; c++) {
        const double w = S[static_cast<size_t>(c) * m + i];
        const double *vc = V_.data() + static_cast<size_t>(c) * n_;
        for (int t = 0; t < n_; t++) out[t] += w * vc[t];
      }
    }
    return nconv_ > 0 ? 0 : -1;
  }
  // thick restart: keep the nev + (ncv - nev) / 2 Ritz vectors of smallest
  // magnitude, continue from the residual direction
  int keep = nev_ + (m - nev_) / 2;
  if (keep > m - 1) keep = m - 1;
  std::vector<double> U(static_cast<size_t>(keep) * n_, 0.0);
  for (int k = 0; k < keep; k++) {
    const int i = idx[k];
    double *out = U.data() + static_cast<size_t>(k) * n_;
    for (int c = 0; c < m; c++) {
      const double w = S[static_cast<size_t>(c) * m + i];
      const double *vc = V_.data() + static_cast<size_t>(c) * n_;
      for (int t = 0; t < n_; t++) out[t] += w * vc[t];
    }
  }
  for (size_t t = 0; t < U.size(); t++) V_[t] = U[t];
  for (auto &h : H_) h = 0.0;
  for (int k = 0; k < keep; k++) H_[static_cast<size_t>(k) * ncv_ + k] = theta[idx[k]];
  double *next = V_.data() + static_cast<size_t>(keep) * n_;
  if (beta > 0.0) {
    for (int t = 0; t < n_; t++) next[t] = r_[t] / beta;
  } else {
    random_unit(next);
  }
  orthogonalise(next, keep, h_.data());
  const double s = std::sqrt(dot(n_, next, next));
  for (int t = 0; t < n_; t++) next[t] /= s;
  j_ = keep;
  restarts_++;
  return 1;
}

}  // namespace sffg

extern "C" int sffg_low_modes(int n, int nev, int ncv, double tol, int max_restarts,
                              void (*matvec)(const double *x, double *y, void *ctx), void *ctx, double *values,
                              double *vectors) {
  if (!matvec || !values || !vectors) return -1;
  sffg::LowModes lm;
  if (lm.init(n, nev, ncv, tol, max_restarts)) return -1;
  int r;
  while ((r = lm.iterate()) == 1) matvec(lm.in(), lm.out(), ctx);
  if (r < 0) return -1;
  for (int k = 0; k < lm.nconv(); k++) values[k] = lm.values()[k];
  for (size_t t = 0; t < static_cast<size_t>(lm.nconv()) * n; t++) vectors[t] = lm.vectors()[t];
  return lm.nconv();
}
