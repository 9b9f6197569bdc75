// XMIN, the reference's general-purpose minimiser (src/sff/xminC.c):
// Polak-Ribiere conjugate gradients (method 1), L-BFGS (2), L-BFGS-
// preconditioned truncated-Newton CG (3) and a finite-difference gradient
// check (4), each with the modified Armijo (ls_method 1) or the More-Thuente
// (2) line search, and forward (numdiff 1) or central (2) finite-difference
// Hessian-vector products for method 3.  Two entry points keep the
// reference's interface (include/sff.h): xmin() drives a function such as
// mme() or mme_rattle() itself; xminC() is the reverse-communication form,
// where the caller evaluates energy and gradient whenever return_flag asks
// and calls again.
//
// Each run is one C++20 coroutine.  Every place where the reference's state
// machine hands control back for an evaluation is a co_yield of the request
// code (1-9, xminC.c:57-66), and xminC() resumes the coroutine.  The
// arithmetic follows the reference term by term -- sums in index order, the
// same update formulas and tests -- so on a deterministic function the
// iterates agree with the reference's bit for bit (this file is compiled
// without floating-point contraction so that holds on every host).
//
// Behaviour kept from the reference, including its quirks:
//  * line-search failures never stop a minimisation: the reference's wrapper
//    (xminC.c:1066-1125) turns every line-search status into "done", so the
//    minimiser continues from wherever the search left the coordinates;
//  * the L-BFGS two-loop recursion walks the stored pairs in slot order
//    (m-1 .. 0, then 0 .. m-1), not in the order they were stored
//    (xminC.c:1254-1312); empty slots (rho 0) contribute nothing;
//  * a finite-difference Hessian-vector product restores the coordinates
//    and gradient but not the energy, so the line search that follows starts
//    from the energy of the last displaced point (xminC.c:189-421);
//  * in L-BFGS a zero y.s ends the run normally (its error is overwritten by
//    the final evaluation, xminC.c:2187-2196); in TNCG it is an error;
//  * mol_struct_opt=1 minimises only atoms whose incoming gradient is not
//    exactly zero (frozen atoms, xminC.c:2590-2630).
// One minimisation runs at a time per process, as in the reference.
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <exception>
#include <memory>
#include <vector>

#include "coro.h"
#include "sffg_internal.h"

namespace {

using sffg::Gen;

// Request codes a run hands back (xminC.c:57-66): evaluate energy and
// gradient, with a forced (4-6), prevented (7-9) or free (1-3) pair-list
// update.
constexpr int kDone = 0, kBothNewList = 6, kGradOldList = 8, kBothOldList = 9;
// Statuses (xminC.c:68-73).
constexpr int kParamsError = -1, kDivZero = -4, kMinimError = -5, kSearchError = -6;

constexpr double kEpsMach = 2.2204460492503131e-16;
constexpr double kBig = 1e+20, kTiny = 1e-20;
constexpr double kCgQTol = 0.5;
constexpr int kCgIterMax = 50;

// Comparisons in the reference's macro form (a NaN operand selects b).
inline double lo(double a, double b) { return a < b ? a : b; }
inline double hi(double a, double b) { return a > b ? a : b; }
inline double sq(double a) { return a * a; }

#define XMIN_RUN CORO_RUN

// Verbosity shared by all runs, as the reference's file-scope flags
// (print_level 0: none; 1: every iteration; 2: also line-search and CG
// details; n > 2: every n-th iteration).
// (per thread: batched runs start and resume on the host's worker threads,
// always quietly)
thread_local int g_print = 0;
thread_local bool g_debug = false;
thread_local int g_nfunc = 0;  // evaluations made by xmin() in the current call

struct Pair {
  double rho = 0.0, gamma = 0.0;
  std::vector<double> s, y;
};

struct Params {
  int method = 3, numdiff = 1, m = 5, ls_method = 2, ls_maxiter = 20, maxiter = 1000;
  double grms_tol = 0.05, ls_maxatmov = 0.5, beta_armijo = 0.5, c_armijo = 0.4, mu_armijo = 1.0;
  double ftol_wolfe = 1e-4, gtol_wolfe = 0.9;
  // relative precision of the gradients, which sizes the finite-difference
  // step of the Hessian products: the FP64 machine epsilon as in the
  // reference, or FP32's for this library's own GPU energy
  double grad_eps = kEpsMach;
};

class Run {
 public:
  Run(const Params &p, int ndim) : p_(p), n_(ndim), x(ndim), g(ndim) {}

  Params p_;
  int n_;
  std::vector<double> x, g;  // coordinates being minimised and their gradient
  double e = 0.0;            // energy of the last evaluation
  int last_request = 0;
  // outputs (the reference writes them through its caller's pointers)
  int iter_out = 0, ls_iter_out = 0;
  double grms_out = 0.0, total_time = 0.0;

  Gen main() {
    switch (p_.method) {
      case 1: return prcg();
      case 2: return lbfgs();
      case 3: return tncg();
      default: return debug_grad();
    }
  }

 private:
  FILE *out() const { return sffg::legacy_out(); }

  std::vector<Pair> mat_, buf_;  // the L-BFGS memory and the TNCG build buffer

  void init_pairs(std::vector<Pair> &v) {
    v.assign(p_.m, Pair());
    for (auto &q : v) {
      q.s.assign(n_, 0.0);
      q.y.assign(n_, 0.0);
    }
  }

  // Stores one (s, y) pair in a slot with rho = 1/(y.s) and the scaling
  // |y.s / y.y| (xminC.c:1224-1251).
  int load_pair(std::vector<Pair> &v, int slot, const std::vector<double> &s, const std::vector<double> &y) {
    double rho = 0.0, gamma = 0.0;
    Pair &q = v[slot];
    for (int i = 0; i < n_; i++) {
      q.s[i] = s[i];
      q.y[i] = y[i];
      rho += s[i] * y[i];
      gamma += y[i] * y[i];
    }
    if (rho == 0.0) {
      std::fprintf(stderr, "\nERROR in load_lbfgs(): YS=0.\n");
      return kDivZero;
    }
    if (gamma == 0.0) {
      std::fprintf(stderr, "\nERROR in load_lbfgs(): YY=0.\n");
      return kDivZero;
    }
    q.rho = 1.0 / rho;
    q.gamma = std::fabs(rho / gamma);
    return 0;
  }

  // L-BFGS two-loop product vout = H (sign * vin) with the scaling of slot
  // `current` (xminC.c:1254-1312).
  void two_loop(int current, double sign, const std::vector<double> &vin, std::vector<double> &vout) {
    const int m = p_.m;
    std::vector<double> alpha(m), t(n_);
    for (int i = 0; i < n_; i++) t[i] = sign * vin[i];
    for (int j = m - 1; j >= 0; j--) {
      double dot = 0.0;
      for (int i = 0; i < n_; i++) dot += mat_[j].s[i] * t[i];
      alpha[j] = mat_[j].rho * dot;
      for (int i = 0; i < n_; i++) t[i] -= alpha[j] * mat_[j].y[i];
    }
    for (int i = 0; i < n_; i++) vout[i] = t[i] * mat_[current].gamma;
    for (int j = 0; j < m; j++) {
      double dot = 0.0;
      for (int i = 0; i < n_; i++) dot += mat_[j].y[i] * vout[i];
      const double beta = mat_[j].rho * dot;
      for (int i = 0; i < n_; i++) vout[i] += mat_[j].s[i] * (alpha[j] - beta);
    }
  }

  double grms_of() const {
    double s = 0.0;
    for (int i = 0; i < n_; i++) s += sq(g[i]);
    return std::sqrt(s / n_);
  }

  Gen request(int r) {
    last_request = r;
    co_yield r;
    co_return 0;
  }

  // ---- finite-difference Hessian-vector products (xminC.c:189-421) -------
  // H v from gradients at x +- h v (central) or x + h v (forward), the step
  // of Derreumaux, Zhang, Schlick and Brooks, J. Comput. Chem. 15, 532
  // (1994), p. 541.  x and g are restored; the energy is not.
  Gen hessvec(const std::vector<double> &v, std::vector<double> &hv) {
    const double sqrt_eps = std::sqrt(p_.grad_eps);
    std::vector<double> xsave(n_), gsave(n_), gorig;
    int st = 0;
    if (p_.numdiff == 2) gorig = g;
    else gsave = g;
    xsave = x;
    double dot = 0.0;
    for (int i = 0; i < n_; i++) dot += sq(xsave[i]);
    const double xnorm = std::sqrt(dot);
    dot = 0.0;
    for (int i = 0; i < n_; i++) dot += sq(v[i]);
    if (dot == 0.0) {
      for (int i = 0; i < n_; i++) hv[i] = 0.0;
      co_return 0;
    }
    const double vnorm = std::sqrt(dot);
    if (p_.numdiff == 2) {
      double vmax = 0.0;
      for (int i = 0; i < n_; i++) {
        const double a = std::fabs(v[i]);
        if (a >= vmax) vmax = a;
      }
      const double h = lo((2. * sqrt_eps * (1.0 + xnorm) / vnorm), (sqrt_eps / vmax));
      for (int i = 0; i < n_; i++) x[i] -= h * v[i];
      XMIN_RUN(request(kGradOldList), st);
      gsave = g;
      x = xsave;
      for (int i = 0; i < n_; i++) x[i] += h * v[i];
      XMIN_RUN(request(kGradOldList), st);
      for (int i = 0; i < n_; i++) hv[i] = (g[i] - gsave[i]) / (2. * h);
      x = xsave;
      g = gorig;
    } else {
      const double h = 2. * sqrt_eps * (1.0 + xnorm) / vnorm;
      for (int i = 0; i < n_; i++) x[i] += h * v[i];
      XMIN_RUN(request(kGradOldList), st);
      for (int i = 0; i < n_; i++) hv[i] = (g[i] - gsave[i]) / h;
      x = xsave;
      g = gsave;
    }
    co_return st;
  }

  // ---- line searches ------------------------------------------------------
  // One safeguarded step of More and Thuente's line search (MINPACK
  // dcstep; J. J. More and D. J. Thuente, ACM TOMS 20, 286 (1994)), in the
  // form of xminC.c:425-640: updates the interval of uncertainty [stx, sty]
  // and returns the next trial step in stp.
  static int mt_step(double &stx, double &fx, double &dx, double &sty, double &fy, double &dy, double &stp, double fp,
                     double dp, bool &brackt, double stpmin, double stpmax) {
    if ((brackt && (stp <= lo(stx, sty) || stp >= hi(stx, sty))) || (dx * (stp - stx) >= 0) || stpmax < stpmin) {
      if (g_debug) std::fprintf(stderr, "Line minimizer aborted: inconsistent step interval\n");
      return kSearchError;
    }
    const double sgnd = dp * (dx / std::fabs(dx));
    double stpf, stpc, stpq, theta, s, gamma, p, q, r;
    bool bound;
    if (fp > fx) {
      // higher value: the minimum is bracketed; cubic step if closer to stx,
      // else the mean of cubic and quadratic
      bound = true;
      theta = 3 * (fx - fp) / (stp - stx) + dx + dp;
      s = hi(std::fabs(theta), hi(std::fabs(dx), std::fabs(dp)));
      gamma = s * std::sqrt(sq(theta / s) - (dx / s) * (dp / s));
      if (stp < stx) gamma = -gamma;
      p = (gamma - dx) + theta;
      q = ((gamma - dx) + gamma) + dp;
      r = p / q;
      stpc = stx + r * (stp - stx);
      stpq = stx + ((dx / ((fx - fp) / (stp - stx) + dx)) / 2) * (stp - stx);
      if (std::fabs(stpc - stx) < std::fabs(stpq - stx)) stpf = stpc;
      else stpf = stpc + (stpq - stpc) / 2;
      brackt = true;
    } else if (sgnd < 0) {
      // lower value, derivatives of opposite sign: bracketed; the cubic step
      // if farther from stp than the secant step
      bound = false;
      theta = 3 * (fx - fp) / (stp - stx) + dx + dp;
      s = hi(std::fabs(theta), hi(std::fabs(dx), std::fabs(dp)));
      gamma = s * std::sqrt(sq(theta / s) - (dx / s) * (dp / s));
      if (stp > stx) gamma = -gamma;
      p = (gamma - dp) + theta;
      q = ((gamma - dp) + gamma) + dx;
      r = p / q;
      stpc = stp + r * (stx - stp);
      stpq = stp + (dp / (dp - dx)) * (stx - stp);
      if (std::fabs(stpc - stp) > std::fabs(stpq - stp)) stpf = stpc;
      else stpf = stpq;
      brackt = true;
    } else if (std::fabs(dp) < std::fabs(dx)) {
      // lower value, same sign, derivative magnitude decreasing
      bound = true;
      theta = 3 * (fx - fp) / (stp - stx) + dx + dp;
      s = hi(std::fabs(theta), hi(std::fabs(dx), std::fabs(dp)));
      gamma = s * std::sqrt(hi(0.0, sq(theta / s) - (dx / s) * (dp / s)));
      if (stp > stx) gamma = -gamma;
      p = (gamma - dp) + theta;
      q = (gamma + (dx - dp)) + gamma;
      r = p / q;
      if (r < 0 && gamma != 0) stpc = stp + r * (stx - stp);
      else if (stp > stx) stpc = stpmax;
      else stpc = stpmin;
      stpq = stp + (dp / (dp - dx)) * (stx - stp);
      if (brackt) stpf = std::fabs(stp - stpc) < std::fabs(stp - stpq) ? stpc : stpq;
      else stpf = std::fabs(stp - stpc) > std::fabs(stp - stpq) ? stpc : stpq;
    } else {
      // lower value, same sign, derivative magnitude not decreasing
      bound = false;
      if (brackt) {
        theta = 3 * (fp - fy) / (sty - stp) + dy + dp;
        s = hi(std::fabs(theta), hi(std::fabs(dy), std::fabs(dp)));
        gamma = s * std::sqrt(sq(theta / s) - (dy / s) * (dp / s));
        if (stp > sty) gamma = -gamma;
        p = (gamma - dp) + theta;
        q = ((gamma - dp) + gamma) + dy;
        r = p / q;
        stpc = stp + r * (sty - stp);
        stpf = stpc;
      } else if (stp > stx) {
        stpf = stpmax;
      } else {
        stpf = stpmin;
      }
    }
    if (fp > fx) {
      sty = stp;
      fy = fp;
      dy = dp;
    } else {
      if (sgnd < 0) {
        sty = stx;
        fy = fx;
        dy = dx;
      }
      stx = stp;
      fx = fp;
      dx = dp;
    }
    stpf = lo(stpmax, stpf);
    stpf = hi(stpmin, stpf);
    stp = stpf;
    if (brackt && bound) {
      if (sty > stx) stp = lo(stx + 0.66 * (sty - stx), stp);
      else stp = hi(stx + 0.66 * (sty - stx), stp);
    }
    return 0;
  }

  // More-Thuente search for a step along d meeting the strong Wolfe
  // conditions, the full step first and no atom moving more than
  // ls_maxatmov (xminC.c:643-947).
  Gen ls_wolfe(const std::vector<double> &d) {
    const Params &o = p_;
    double dg_init = 0.0;
    for (int i = 0; i < n_; i++) dg_init += g[i] * d[i];
    double dmax = 0.0, dnorm = 0.0, gr = 0.0;
    int dmax_idx = 0;
    for (int i = 0; i < n_; i++) {
      dnorm += sq(d[i]);
      gr += sq(g[i]);
      if (std::fabs(d[i]) > dmax) {
        dmax = std::fabs(d[i]);
        dmax_idx = i;
      }
    }
    dnorm = std::sqrt(dnorm);
    double stpmax = kBig;
    if (dmax > o.ls_maxatmov) stpmax = o.ls_maxatmov / dmax;
    const double stpmin = kTiny;
    const double rhs_g = o.gtol_wolfe * std::fabs(dg_init);
    bool brackt = false, stage1 = true;
    double width = stpmax - stpmin, width1 = 2 * width;
    const double dgtest = o.ftol_wolfe * std::fabs(dg_init);
    double stx = 0.0, fx = e, dgx = dg_init, sty = 0.0, fy = e, dgy = dg_init;
    double stmin = 0.0, stmax = 0.0;
    const std::vector<double> xsave = x;
    const double fsave = e;
    double stp = 1.0;
    int status = 0, st = 0, i;
    for (i = 1; i <= o.ls_maxiter; i++) {
      if (brackt) {
        stmin = lo(stx, sty);
        stmax = hi(stx, sty);
      } else {
        stmin = stx;
        stmax = stp + 4 * (stp - stx);
      }
      stp = hi(stp, stpmin);
      stp = lo(stp, stpmax);
      if ((brackt && (stp <= stmin || stp >= stmax)) || (brackt && (stmax - stmin <= kEpsMach * stmax))) stp = stx;
      for (int j = 0; j < n_; j++) x[j] += stp * d[j];
      XMIN_RUN(request(i == 1 ? kBothNewList : kBothOldList), st);
      const double lhs_f = e - fsave;
      const double rhs_f = stp * o.ftol_wolfe * dg_init;
      double dg_try = 0.0;
      for (int j = 0; j < n_; j++) dg_try += g[j] * d[j];
      const double lhs_g = std::fabs(dg_try);
      if (g_debug) {
        std::fprintf(out(), "  LS: i=%2d  lhs_f=%16.8g  rhs_f=%16.8g\n", i, lhs_f, rhs_f);
        std::fprintf(out(), "            lhs_g=%16.8g  rhs_g=%16.8g\n", lhs_g, rhs_g);
        std::fprintf(out(), "            rel_s=%16.8g  abs_s=%16.8g\n", stp, stp * dnorm);
        std::fprintf(out(), "            max_d=%16.8g  i_xyz=%15d%c\n", stp * dmax, dmax_idx / 3 + 1,
                     static_cast<char>('x' + dmax_idx % 3));
      }
      if (lhs_f <= rhs_f && lhs_g <= rhs_g) break;  // both Wolfe conditions hold
      if ((brackt && (stp <= stmin || stp >= stmax)) ||
          (stp == stpmax && (lhs_f <= rhs_f && dg_try <= dgtest)) ||
          (stp == stpmin && (lhs_f > rhs_f || dg_try >= dgtest)) ||
          (brackt && (stmax - stmin <= kEpsMach * stmax))) {
        // rounding errors, a step at a bound, or an interval too small
        if (g_debug) std::fprintf(stderr, "Line minimizer aborted at step %16.8g\n", stp);
        status = kSearchError;
        break;
      }
      if (stage1 && lhs_f <= rhs_f && dg_try >= lo(o.ftol_wolfe, o.gtol_wolfe) * dg_init) stage1 = false;
      if (stage1 && e <= fx && lhs_f > rhs_f) {
        // the modified function f(x+stp d) - f(x) - ftol stp g.d predicts
        double fm = e - stp * dgtest;
        double fxm = fx - stx * dgtest, fym = fy - sty * dgtest;
        double dgm = dg_try - dgtest, dgxm = dgx - dgtest, dgym = dgy - dgtest;
        status = mt_step(stx, fxm, dgxm, sty, fym, dgym, stp, fm, dgm, brackt, stmin, stmax);
        if (status) break;
        fx = fxm + stx * dgtest;
        fy = fym + sty * dgtest;
        dgx = dgxm + dgtest;
        dgy = dgym + dgtest;
      } else {
        status = mt_step(stx, fx, dgx, sty, fy, dgy, stp, e, dg_try, brackt, stmin, stmax);
        if (status) break;
      }
      if (brackt) {
        if (std::fabs(sty - stx) >= .66 * width1) stp = stx + .5 * (sty - stx);
        width1 = width;
        width = std::fabs(sty - stx);
      }
      if (i < o.ls_maxiter) {
        x = xsave;
      } else {
        if (g_debug) std::fprintf(stderr, "Line minimizer aborted: max number of iterations reached\n");
        status = kSearchError;
      }
    }
    alfa_ = stp;
    ls_iter_ = i < o.ls_maxiter ? i : o.ls_maxiter;
    ls_iter_out += ls_iter_;
    co_return status;
  }

  // Backtracking search with the modified Armijo rule of Shi and Shen
  // (xminC.c:950-1063): starts at -g.d / (L |d|^2) with L estimated from the
  // last step and gradient change, shrinks by beta_armijo.
  Gen ls_armijo(int k, const std::vector<double> &d, const std::vector<double> &x_diff,
                const std::vector<double> &g_diff) {
    const Params &o = p_;
    double dir_grad = 0.0, dnorm2 = 0.0;
    for (int i = 0; i < n_; i++) {
      dir_grad += g[i] * d[i];
      dnorm2 += sq(d[i]);
    }
    double l_k = 1.0;
    if (k) {
      double sg = 0.0, sx = 0.0;
      for (int i = 0; i < n_; i++) {
        sg += sq(g_diff[i]);
        sx += sq(x_diff[i]);
      }
      l_k = std::sqrt(sg) / std::sqrt(sx);
    }
    const double s_k = -dir_grad / l_k / dnorm2;
    const double mod_test = 0.5 * o.mu_armijo * l_k * dnorm2;
    double dmax = 0.0;
    for (int i = 0; i < n_; i++)
      if (std::fabs(d[i]) > dmax) dmax = std::fabs(d[i]);
    double dlimit = kBig;
    if (dmax > o.ls_maxatmov) dlimit = o.ls_maxatmov / dmax;
    const std::vector<double> xsave = x;
    const double fsave = e;
    int i = 1, st = 0;
    // an infinite first step never shrinks below the limit; the reference
    // loops forever there, this search gives up without moving
    for (alfa_ = s_k; i <= o.ls_maxiter && alfa_ != HUGE_VAL; alfa_ *= o.beta_armijo) {
      if (alfa_ > dlimit) continue;
      for (int j = 0; j < n_; j++) x[j] += alfa_ * d[j];
      XMIN_RUN(request(i == 1 ? kBothNewList : kBothOldList), st);
      const double lhs = e - fsave;
      const double rhs = alfa_ * o.c_armijo * (dir_grad + alfa_ * mod_test);
      if (g_debug) std::fprintf(out(), "  LS: i=%2d  lhs=%16.8g  rhs=%16.8g\n", i, lhs, rhs);
      if (lhs <= rhs) break;
      if (i < o.ls_maxiter) x = xsave;
      i++;
    }
    ls_iter_ = i < o.ls_maxiter ? i : o.ls_maxiter;
    ls_iter_out += ls_iter_;
    co_return 0;
  }

  // The line search of min_iter k along d.  Its status is dropped, as the
  // reference's wrapper does.
  Gen line_search(int k, const std::vector<double> &d, const std::vector<double> &x_diff,
                  const std::vector<double> &g_diff) {
    int st = 0;
    if (p_.ls_method == 1) {
      XMIN_RUN(ls_armijo(k, d, x_diff, g_diff), st);
    } else {
      XMIN_RUN(ls_wolfe(d), st);
    }
    (void)st;
    if (g_debug) std::fprintf(out(), "  LS: step=%16.8g  it=%2d\n", alfa_, ls_iter_);
    co_return 0;
  }

  double alfa_ = 0.0;
  int ls_iter_ = 0;

  Gen finish(bool conv, std::clock_t t0) {
    int st = 0;
    XMIN_RUN(request(kBothNewList), st);
    (void)st;
    const double gr = grms_of();
    grms_out = gr;
    if (g_print) {
      std::fprintf(out(), "----------------------------------------------------------------\n");
      std::fprintf(out(), " END:          %s  E = %13.5f  RMSG = %11.7f\n\n", conv ? ":-)" : ":-(", e, gr);
    }
    total_time += static_cast<double>(std::clock() - t0);
    total_time /= CLOCKS_PER_SEC;
    co_return 0;
  }

  // ---- method 1: Polak-Ribiere CG (xminC.c:1813-2052) -----------------------
  Gen prcg() {
    std::vector<double> pdir(n_), p_old(n_), g_old(n_), x_old(n_), step(n_), g_dif(n_);
    int st = 0, min_iter = 0;
    bool conv = false;
    total_time = 0.0;
    if (g_print) std::fprintf(out(), "Starting PRCG minimisation\n");
    iter_out = 1;
    ls_iter_out = 0;
    std::clock_t t0 = std::clock();
    do {
      t0 = std::clock();
      if (min_iter == 0) XMIN_RUN(request(kBothNewList), st);
      if (min_iter) {
        for (int i = 0; i < n_; i++) {
          step[i] = x[i] - x_old[i];
          g_dif[i] = g[i] - g_old[i];
        }
      }
      double gr = 0.0, ggnew = 0.0, ggold = 0.0;
      for (int i = 0; i < n_; i++) {
        gr += sq(g[i]);
        ggold += sq(g_old[i]);
        ggnew += (g[i] - g_old[i]) * g[i];
      }
      gr = std::sqrt(gr / n_);
      if (g_print && min_iter % g_print == 0) {
        std::fprintf(out(), " return_flag: %3d\n", last_request);
        std::fprintf(out(), " MIN:  Iter = %4d  E = %13.5f  RMSG = %11.7f\n", min_iter, e, gr);
      }
      if (gr <= p_.grms_tol || min_iter == p_.maxiter) {
        conv = true;
        break;
      }
      const double gamma = min_iter ? ggnew / ggold : 0.0;
      for (int i = 0; i < n_; i++) pdir[i] = -g[i] + gamma * p_old[i];
      double dgrad = 0.0;
      for (int i = 0; i < n_; i++) dgrad += g[i] * pdir[i];
      if (dgrad > 0.0)
        for (int i = 0; i < n_; i++) pdir[i] = -g[i];
      for (int i = 0; i < n_; i++) p_old[i] = pdir[i];
      g_old = g;
      x_old = x;
      XMIN_RUN(line_search(min_iter, pdir, step, g_dif), st);
      iter_out++;
      total_time += static_cast<double>(std::clock() - t0);
    } while (++min_iter <= p_.maxiter);
    iter_out = min_iter;
    XMIN_RUN(finish(conv, t0), st);
    co_return 0;
  }

  // ---- method 2: L-BFGS (xminC.c:2055-2358) -------------------------------
  // Polak-Ribiere steps until m pairs are stored, then the L-BFGS direction.
  Gen lbfgs() {
    if (!p_.m) {
      std::fprintf(stderr, "\nERROR in lbfgs_minim(): m_lbfgs = 0\n");
      co_return kMinimError;
    }
    init_pairs(mat_);
    std::vector<double> pdir(n_), p_old(n_), g_old(n_), g_dif(n_), step(n_), x_old(n_);
    int st = 0, min_iter = 0;
    bool conv = false;
    total_time = 0.0;
    if (g_print) std::fprintf(out(), "Starting L-BFGS minimisation\n");
    iter_out = 1;
    ls_iter_out = 0;
    std::clock_t t0 = std::clock();
    do {
      t0 = std::clock();
      if (min_iter == 0) XMIN_RUN(request(kBothNewList), st);
      if (min_iter) {
        for (int i = 0; i < n_; i++) {
          step[i] = x[i] - x_old[i];
          g_dif[i] = g[i] - g_old[i];
        }
        if (load_pair(mat_, (min_iter - 1) % p_.m, step, g_dif)) break;  // ends normally
      }
      if (min_iter < p_.m) {
        double gr = 0.0, ggnew = 0.0, ggold = 0.0;
        for (int i = 0; i < n_; i++) {
          gr += sq(g[i]);
          ggold += sq(g_old[i]);
          ggnew += (g[i] - g_old[i]) * g[i];
        }
        gr = std::sqrt(gr / n_);
        if (g_print && min_iter % g_print == 0)
          std::fprintf(out(), " MIN:  Iter = %4d  E = %13.5f  RMSG = %11.7f\n", min_iter, e, gr);
        if (gr <= p_.grms_tol || min_iter == p_.maxiter) {
          conv = true;
          break;
        }
        const double gamma = min_iter ? ggnew / ggold : 0.0;
        for (int i = 0; i < n_; i++) pdir[i] = -g[i] + gamma * p_old[i];
        double dgrad = 0.0;
        for (int i = 0; i < n_; i++) dgrad += g[i] * pdir[i];
        if (dgrad > 0.0)
          for (int i = 0; i < n_; i++) pdir[i] = -g[i];
        for (int i = 0; i < n_; i++) p_old[i] = pdir[i];
      } else {
        const double gr = grms_of();
        if (g_print && min_iter % g_print == 0)
          std::fprintf(out(), " MIN:  Iter = %4d  E = %13.5f  RMSG = %11.7f\n", min_iter, e, gr);
        if (gr <= p_.grms_tol || min_iter == p_.maxiter) {
          conv = true;
          break;
        }
        two_loop((min_iter - 1) % p_.m, -1.0, g, pdir);
        double dgrad = 0.0;
        for (int i = 0; i < n_; i++) dgrad += g[i] * pdir[i];
        if (dgrad > 0.0)
          for (int i = 0; i < n_; i++) pdir[i] = -g[i];
      }
      x_old = x;
      g_old = g;
      XMIN_RUN(line_search(min_iter, pdir, step, g_dif), st);
      iter_out++;
      total_time += static_cast<double>(std::clock() - t0);
    } while (++min_iter <= p_.maxiter);
    iter_out = min_iter;
    XMIN_RUN(finish(conv, t0), st);
    co_return 0;
  }

  // ---- method 3: truncated-Newton CG (xminC.c:1315-1810) ------------------
  // Each outer step solves H p = -g by CG with finite-difference H d
  // products, stopped by the quadratic-reduction test (or at negative
  // curvature), and preconditioned by an L-BFGS matrix built from the
  // previous outer step's CG iterates (Morales and Nocedal, SIAM J. Optim.
  // 10, 1079 (2000)).
  Gen tncg() {
    if (p_.m) {
      init_pairs(mat_);
      init_pairs(buf_);
    }
    std::vector<double> pdir(n_), r(n_), s(n_), q(n_), d(n_), s_vec(n_), r_old(n_), y_vec(n_), p_old(n_), hp(n_),
        x_old(n_), g_old(n_), step(n_), g_dif(n_);
    int st = 0, min_iter = 0, last_update = 0, current_update = 0;
    bool conv = false, convex = true, reloaded = false;
    double quad_old = 0.0;
    total_time = 0.0;
    if (g_print) std::fprintf(out(), "Starting TNCG minimisation\n");
    iter_out = 1;
    ls_iter_out = 0;
    std::clock_t t0 = std::clock();
    auto precondition = [&]() {
      if (reloaded) two_loop(last_update, 1.0, r, s);
      else s = r;
    };
    do {
      t0 = std::clock();
      if (min_iter == 0) XMIN_RUN(request(kBothNewList), st);
      if (min_iter) {
        for (int i = 0; i < n_; i++) {
          step[i] = x[i] - x_old[i];
          g_dif[i] = g[i] - g_old[i];
        }
      }
      const double gr = grms_of();
      if (g_print && min_iter % g_print == 0)
        std::fprintf(out(), " MIN: Iter = %4d  NFunc = %5d  E = %13.5f  RMSG = %11.7e\n", min_iter, g_nfunc, e, gr);
      if (gr <= p_.grms_tol || min_iter == p_.maxiter) {
        conv = true;
        break;
      }
      for (int i = 0; i < n_; i++) {
        pdir[i] = 0.0;
        r[i] = -g[i];
        hp[i] = 0.0;
      }
      precondition();
      double rs_old = 0.0;
      for (int i = 0; i < n_; i++) {
        d[i] = s[i];
        rs_old += r[i] * s[i];
      }
      int cg_iter = 0, n_lbfgs = 0;
      bool cg_conv = false;
      double qtest = 999.999;
      do {
        XMIN_RUN(hessvec(d, q), st);
        if (st) co_return st;
        double dq = 0.0;
        for (int i = 0; i < n_; i++) dq += d[i] * q[i];
        if (dq < 0.0) {  // negative curvature: keep the (still downhill) p
          convex = false;
          if (!cg_iter)
            for (int i = 0; i < n_; i++) pdir[i] = -g[i];
          break;
        }
        convex = true;
        double quad_new;
        if (dq != 0.0) {
          const double alpha = rs_old / dq;
          for (int i = 0; i < n_; i++) {
            p_old[i] = pdir[i];
            r_old[i] = r[i];
            pdir[i] += alpha * d[i];
            r[i] -= alpha * q[i];
            s_vec[i] = pdir[i] - p_old[i];
            y_vec[i] = r_old[i] - r[i];
            hp[i] += alpha * q[i];
          }
          if (p_.m) {
            n_lbfgs++;
            current_update = cg_iter % p_.m;
            const int err = load_pair(buf_, current_update, s_vec, y_vec);
            if (err) co_return err;
          }
          double gp = 0.0, php = 0.0;
          for (int i = 0; i < n_; i++) {
            gp += g[i] * pdir[i];
            php += pdir[i] * hp[i];
          }
          quad_new = gp + 0.5 * php;
        } else {
          quad_new = quad_old;  // zero residual
        }
        if (cg_iter && cg_iter >= (p_.m - 1)) {  // at least m CG iterations build the preconditioner
          qtest = (cg_iter + 1) * (1.0 - quad_old / quad_new);
          if (qtest < kCgQTol) {
            cg_conv = true;
            break;
          }
        }
        quad_old = quad_new;
        precondition();
        double rs_new = 0.0;
        for (int i = 0; i < n_; i++) rs_new += r[i] * s[i];
        const double beta = rs_new / rs_old;
        rs_old = rs_new;
        for (int i = 0; i < n_; i++) d[i] = s[i] + beta * d[i];
      } while (++cg_iter < kCgIterMax);
      if (g_debug)
        std::fprintf(out(), "  CG:   It= %4d (%7.3f)q  %s%s\n",
                     (!convex || cg_iter == kCgIterMax) ? cg_iter : cg_iter + 1, qtest, cg_conv ? ":-)" : ":-(",
                     convex ? "" : "(");
      if (p_.m && n_lbfgs >= p_.m && convex) {
        reloaded = true;
        last_update = current_update;
        for (int i = 0; i < p_.m; i++) {
          mat_[i].s = buf_[i].s;
          mat_[i].y = buf_[i].y;
          mat_[i].rho = buf_[i].rho;
          mat_[i].gamma = buf_[i].gamma;
        }
      }
      g_old = g;
      x_old = x;
      XMIN_RUN(line_search(min_iter, pdir, step, g_dif), st);
      iter_out++;
      total_time += static_cast<double>(std::clock() - t0);
    } while (++min_iter <= p_.maxiter);
    iter_out = min_iter;
    XMIN_RUN(finish(conv, t0), st);
    co_return 0;
  }

  // ---- method 4: gradient check (xminC.c:2361-2442) ------------------------
  // Central-difference derivative of every coordinate against the analytic
  // gradient, printed to stderr; the coordinates end where they started.
  Gen debug_grad() {
    double xn = 0.0;
    int st = 0;
    for (int i = 0; i < n_; i++) xn += sq(x[i]);
    const double eps = std::sqrt(kEpsMach) * (1.0 + std::sqrt(xn));
    std::fprintf(stderr, "_____________________________________________________________________\n");
    std::fprintf(stderr, "GRADIENT| eps =%14.8g * (1 + %14.8g) = %14.8g\n", std::sqrt(kEpsMach), std::sqrt(xn), eps);
    std::fprintf(stderr, "_____________________________________________________________________\n");
    std::fprintf(stderr, "            atom  xyz    anal.drv     num.drv    rel.diff    abs.diff\n");
    std::fprintf(stderr, "_____________________________________________________________________\n");
    XMIN_RUN(request(kBothNewList), st);
    for (int i = 0; i < n_; i++) {
      const double hold = x[i];
      x[i] = hold - eps;
      XMIN_RUN(request(kBothOldList), st);
      const double e1 = e;
      x[i] = hold + eps;
      XMIN_RUN(request(kBothOldList), st);
      const double e2 = e;
      x[i] = hold;
      XMIN_RUN(request(kBothOldList), st);
      const double num = (e2 - e1) / (2. * eps);
      const double absdiff = std::fabs(g[i] - num);
      const double reldiff = absdiff != 0 ? absdiff / hi(std::fabs(g[i]), std::fabs(num)) : 0.0;
      std::fprintf(stderr, "       %c%8d   %c   %10.3f  %10.3f  %10.3e  %10.3f\n", reldiff >= 0.1 ? '*' : ' ',
                   i / 3 + 1, static_cast<char>('x' + i % 3), g[i], num, reldiff < 1.0 ? reldiff : absdiff, absdiff);
    }
    co_return 0;
  }
};

// One run's reverse-communication state: the moving atoms and the
// coroutine.
struct Active {
  std::unique_ptr<Run> run;
  std::unique_ptr<Gen> gen;
  bool mol = true;
  std::vector<int> atoms;  // moving atoms, in order (mol_struct_opt = 1)
};

void load_in(Active &a, double enrg, const double *grad_ext) {
  Run &r = *a.run;
  r.e = enrg;
  if (a.mol) {
    for (size_t k = 0; k < a.atoms.size(); k++)
      for (int c = 0; c < 3; c++) r.g[3 * k + c] = grad_ext[3 * a.atoms[k] + c];
  } else {
    for (int i = 0; i < static_cast<int>(r.g.size()); i++) r.g[i] = grad_ext[i];
  }
}

void store_out(const Active &a, double *xyz_ext) {
  const Run &r = *a.run;
  if (a.mol) {
    for (size_t k = 0; k < a.atoms.size(); k++)
      for (int c = 0; c < 3; c++) xyz_ext[3 * a.atoms[k] + c] = r.x[3 * k + c];
  } else {
    for (int i = 0; i < static_cast<int>(r.x.size()); i++) xyz_ext[i] = r.x[i];
  }
}

int check_params(int maxiter, double grms_tol, int m, int print_level, int natm, int ls_maxiter, double ls_maxatmov,
                 double beta, double c, double mu) {
  const char *msg = nullptr;
  if (maxiter < 0) msg = "Requested number of iterations negative.";
  else if (grms_tol < 0.0) msg = "Requested grad RMS negative.";
  else if (m < 0) msg = "LBFGS dimension negative.";
  if (msg) {
    std::fprintf(stderr, "\nERROR in xmin(): %s\n", msg);
    return kParamsError;
  }
  if (print_level == 0) {
    g_print = 0;
    g_debug = false;
  } else if (print_level == 1 || print_level == 2) {
    g_print = 1;
    g_debug = print_level == 2;
  } else {
    g_print = print_level;
    g_debug = false;
    std::printf("setting print frequency to %d\n", g_print);
  }
  if (natm < 0) msg = "Number of atoms negative.";
  else if (natm < 2) msg = "Too few atoms.";
  else if (ls_maxiter < 1) msg = "Requested number of LS steps negative.";
  else if (ls_maxatmov <= 0.0) msg = "Max LS move negative.";
  else if (beta <= 0 || beta >= 1) msg = "Armijo_beta out of range.";
  else if (c <= 0 || c >= 0.5) msg = "Armijo_c out of range.";
  else if (mu < 0 || mu >= 2) msg = "Armijo_mu out of range.";
  if (msg) {
    std::fprintf(stderr, "\nERROR in xmin(): %s\n", msg);
    return kParamsError;
  }
  return 0;
}

}  // namespace

namespace sffg {

struct XminJob::Impl {
  Active a;
};

XminJob::XminJob() : impl_(new Impl) {}
XminJob::~XminJob() = default;

int XminJob::start(const XMIN_OPT_T &xo, int natm, double *xyz, const double *grad, double energy, int *request,
                   double grad_eps) {
  Active &a = impl_->a;
  a.gen.reset();
  a.run.reset();
  int rc = check_params(xo.maxiter, xo.grms_tol, xo.m_lbfgs, xo.print_level, natm, xo.ls_maxiter, xo.ls_maxatmov,
                        xo.beta_armijo, xo.c_armijo, xo.mu_armijo);
  if (!rc && (xo.method < 1 || xo.method > 4)) {
    std::fprintf(stderr, "\nERROR in xmin(): Unknown minimization method.\n");
    rc = kParamsError;
  }
  if (!rc && xo.method != 4 && xo.ls_method != 1 && xo.ls_method != 2) {
    std::fprintf(stderr, "\nERROR in xmin(): Unknown line search method.\n");
    rc = kParamsError;
  }
  if (!rc && xo.method != 4 && xo.numdiff != 1 && xo.numdiff != 2) {
    std::fprintf(stderr, "\nERROR in xmin(): Unknown finite difference method.\n");
    rc = kParamsError;
  }
  a.mol = xo.mol_struct_opt != 0;
  a.atoms.clear();
  if (!rc && a.mol) {
    for (int i = 0; i < natm; i++)
      if (grad[3 * i] != 0 || grad[3 * i + 1] != 0 || grad[3 * i + 2] != 0) a.atoms.push_back(i);
    if (a.atoms.size() < 2) {
      std::fprintf(stderr, "\nERROR in xmin(): Too few moving atoms.\n");
      rc = kParamsError;
    }
  }
  if (rc) return rc;
  Params p;
  p.method = xo.method;
  p.numdiff = xo.numdiff;
  p.m = xo.m_lbfgs;
  p.ls_method = xo.ls_method;
  p.ls_maxiter = xo.ls_maxiter;
  p.maxiter = xo.maxiter;
  p.grms_tol = xo.grms_tol;
  p.ls_maxatmov = xo.ls_maxatmov;
  p.beta_armijo = xo.beta_armijo;
  p.c_armijo = xo.c_armijo;
  p.mu_armijo = xo.mu_armijo;
  p.ftol_wolfe = xo.ftol_wolfe;
  p.gtol_wolfe = xo.gtol_wolfe;
  p.grad_eps = grad_eps;
  const int ndim = a.mol ? 3 * static_cast<int>(a.atoms.size()) : natm;
  a.run = std::make_unique<Run>(p, ndim);
  if (a.mol) {
    for (size_t k = 0; k < a.atoms.size(); k++)
      for (int c = 0; c < 3; c++) a.run->x[3 * k + c] = xyz[3 * a.atoms[k] + c];
  } else {
    for (int i = 0; i < ndim; i++) a.run->x[i] = xyz[i];
  }
  a.gen = std::make_unique<Gen>(a.run->main());
  return resume(energy, grad, xyz, request);
}

int XminJob::resume(double energy, const double *grad, double *xyz, int *request) {
  Active &a = impl_->a;
  if (!a.gen) {
    std::fprintf(stderr, "\nERROR in xmin(): Illegal status.\n");
    return -2;
  }
  load_in(a, energy, grad);
  Run &r = *a.run;
  const bool more = a.gen->next();
  iter_ = r.iter_out;
  ls_iter_ = r.ls_iter_out;
  time_ = r.total_time;
  grms_ = r.grms_out;
  if (more) {
    store_out(a, xyz);
    *request = a.gen->request();
    return 1;
  }
  const int status = a.gen->status();
  if (status >= 0) store_out(a, xyz);
  *request = kDone;
  a.gen.reset();
  a.run.reset();
  return status < 0 ? status : 0;
}

}  // namespace sffg

namespace {
// The reverse-communication run of xminC (one at a time, as the reference's
// file-scope state).
sffg::XminJob &active_job() {
  static sffg::XminJob j;
  return j;
}
// Gradient precision for the run xmin() is about to start through xminC.
double g_next_grad_eps = kEpsMach;
}  // namespace

extern "C" {

// Reverse-communication XMIN (src/sff/xminC.c:2491-2972).  Call with
// *label = 0 to start; while it returns with *label = 1, evaluate energy
// into *enrg and gradient into grad_ext at xyz_ext (with the pair-list
// policy *return_flag names) and call again; *label = 0 with *return_flag =
// 0 means done (xyz_ext holds the result, the return value is *enrg), a
// negative *label is an error status.
double xminC(int *xyz_min, int *minim_method, int *maxiter, double *grms_tol, int *natm_ext, int *m_lbfgs,
             int *numdiff, double *xyz_ext, double *enrg, double *grad_ext, double *grms, int *iter,
             double *total_time, int *print_level, int *ls_method, int *ls_maxiter, int *ls_iter,
             double *ls_maxatmov, double *beta_armijo, double *c_armijo, double *mu_armijo, double *ftol_wolfe,
             double *gtol_wolfe, int *return_flag, int *label) {
  sffg::XminJob &job = active_job();
  int request = 0, rc;
  if (*label == 0) {
    XMIN_OPT_T xo;
    xo.mol_struct_opt = *xyz_min;
    xo.method = *minim_method;
    xo.maxiter = *maxiter;
    xo.grms_tol = *grms_tol;
    xo.m_lbfgs = *m_lbfgs;
    xo.numdiff = *numdiff;
    xo.print_level = *print_level;
    xo.ls_method = *ls_method;
    xo.ls_maxiter = *ls_maxiter;
    xo.ls_maxatmov = *ls_maxatmov;
    xo.beta_armijo = *beta_armijo;
    xo.c_armijo = *c_armijo;
    xo.mu_armijo = *mu_armijo;
    xo.ftol_wolfe = *ftol_wolfe;
    xo.gtol_wolfe = *gtol_wolfe;
    rc = job.start(xo, *natm_ext, xyz_ext, grad_ext, *enrg, &request, g_next_grad_eps);
    g_next_grad_eps = kEpsMach;
    if (rc == kParamsError) {  // before any run: outputs untouched
      *label = rc;
      return 0.0;
    }
  } else if (*label != 1) {
    std::fprintf(stderr, "\nERROR in xmin(): Illegal status.\n");
    *label = -2;
    return 0.0;
  } else {
    rc = job.resume(*enrg, grad_ext, xyz_ext, &request);
  }
  *iter = job.iter();
  *ls_iter = job.ls_iter();
  *total_time = job.time();
  *grms = job.grms();
  if (rc == 1) {
    *return_flag = request;
    *label = 1;
    return 0.0;
  }
  if (rc < 0) {
    *label = rc;
    return 0.0;
  }
  *return_flag = kDone;
  *label = 0;
  return *enrg;
}

// The options' defaults (src/sff/xminC.c:2976-2995).
INT_T xmin_opt_init(XMIN_OPT_T *xo) {
  xo->mol_struct_opt = 1;
  xo->maxiter = 1000;
  xo->grms_tol = 0.05;
  xo->method = 3;
  xo->numdiff = 1;
  xo->m_lbfgs = 5;
  xo->ls_method = 2;
  xo->ls_maxiter = 20;
  xo->ls_maxatmov = 0.5;
  xo->beta_armijo = 0.5;
  xo->c_armijo = 0.4;
  xo->mu_armijo = 1.0;
  xo->ftol_wolfe = 0.0001;
  xo->gtol_wolfe = 0.9;
  xo->print_level = 0;
  return 0;
}

// Minimises func from xyz (src/sff/xminC.c:2997-3160).  func receives the
// pair-list policy through its iteration argument as mme() reads it: -4
// forces a rebuild (requests 4-6), -2 keeps the lists (7-9), otherwise the
// current iteration count.  On entry grad must hold the gradient at xyz when
// mol_struct_opt is set (atoms with an exactly zero gradient stay fixed).
// Returns the final energy, or 0 with xo->error_flag < 0 on an error.
REAL_T xmin(REAL_T (*func)(REAL_T *, REAL_T *, INT_T *), INT_T *natm, REAL_T *xyz, REAL_T *grad, REAL_T *energy,
            REAL_T *grms, XMIN_OPT_T *xo) {
  int return_flag = 0, status = 0;
  int neg_two = -2, neg_four = -4;
  g_nfunc = 0;
  xo->error_flag = 0;
  // this library's GPU energy has FP32-accurate gradients: TNCG's
  // finite-difference Hessian products take a step sized for them (the
  // reference's formula with FP32's epsilon); any other func keeps the
  // reference's FP64 step and iterates
  if (func == &mme || func == &mme_rattle) g_next_grad_eps = FLT_EPSILON;
  for (;;) {
    xminC(&xo->mol_struct_opt, &xo->method, &xo->maxiter, &xo->grms_tol, natm, &xo->m_lbfgs, &xo->numdiff, xyz,
          energy, grad, grms, &xo->iter, &xo->xmin_time, &xo->print_level, &xo->ls_method, &xo->ls_maxiter,
          &xo->ls_iter, &xo->ls_maxatmov, &xo->beta_armijo, &xo->c_armijo, &xo->mu_armijo, &xo->ftol_wolfe,
          &xo->gtol_wolfe, &return_flag, &status);
    if (return_flag == 0) {
      xo->error_flag = status >= 0 ? 0 : status;
    } else if (return_flag >= 1 && return_flag <= 9) {
      if (status >= 0) {
        int *it = return_flag <= 3 ? &xo->iter : return_flag <= 6 ? &neg_four : &neg_two;
        *energy = func(xyz, grad, it);
        g_nfunc++;
      } else {
        xo->error_flag = status;
      }
    } else {
      std::printf("\n XMIN ERROR: return_flag corrupted.\n");
      xo->error_flag = -100;
      return 0.0;
    }
    if (xo->error_flag || !return_flag) break;
  }
  if (xo->error_flag) {
    std::printf("\n XMIN ERROR: %d\n", status);
    return 0.0;
  }
  return *energy;
}

}  // extern "C"
