// lc2_optim.cpp -- derivative-free bound-constrained optimizers with batched
// objective evaluation, and the registration driver built on them.
//
// The reference minimises -log(LC2) with NLopt: GN_ORIG_DIRECT_L on the
// entries enabled for DIRECT, then LN_BOBYQA rounds
// (src/Optimizers/optimizers.cu:734-970, 1349-1574). NLopt is not available
// here, so these are this library's own implementations, written from the
// published methods, with the same knobs (bounds, xtol_rel, maxeval). They
// differ from NLopt in that every step hands the objective a whole set of
// points at once where the method has several -- all children of DIRECT's
// potentially optimal rectangles, BOBYQA's 2n+1 initial points, the 2n+1-point
// stencil of the separable trust region, the four candidate points of a
// Nelder-Mead step -- so each step is one batched GPU launch.
//
//   DIRECT-L: Jones, Perttunen, Stuckman (1993), locally biased variant of
//     Gablonsky and Kelley (2001): one rectangle per size class, the lower
//     convex hull of (size, value) with the epsilon test, division along the
//     longest sides in order of the sampled values.
//   BOBYQA: Powell (2009), see the BOBYQA section below; one evaluation per
//     iteration after the first 2n+1, as in NLopt.
//   Separable trust region (LC2_OPT_QUAD_TR, a batched alternative): a
//     separable quadratic model from the 2n+1 points x, x +- rho e_i, its
//     minimiser inside the trust box and the bounds, accept/shrink by actual
//     decrease; stops when rho < xtol_rel (in units of the bound range).
//   Nelder-Mead: Nelder and Mead (1965) with projection onto the bounds;
//     reflection, expansion and both contractions evaluated together.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <vector>

#include "../../include/lc2.h"

void lc2_set_error_message(const char* msg);

namespace {

struct Problem {
  int n;
  std::vector<double> lo, hi;
  lc2_batch_objective f;
  void* user;
  int maxeval;
  int evals = 0, batches = 0;
  int status = LC2_OK;
  double best_f = std::numeric_limits<double>::infinity();
  std::vector<double> best_x;

  // unit-cube coordinates -> parameters
  std::vector<double> to_x(const std::vector<double>& u) const {
    std::vector<double> x(n);
    for (int i = 0; i < n; ++i) x[i] = lo[i] + u[i] * (hi[i] - lo[i]);
    return x;
  }
  bool budget_left(int k = 1) const { return maxeval <= 0 || evals + k <= maxeval; }
  // the last single-point eval() ran (it returns +inf without running once
  // the budget is spent)
  bool budget_used_once() const { return last_ran; }
  bool last_ran = false;

  // evaluate unit-cube points (truncated to the remaining budget)
  std::vector<double> eval(const std::vector<std::vector<double>>& U) {
    std::vector<double> out(U.size(), std::numeric_limits<double>::infinity());
    int count = (int)U.size();
    if (maxeval > 0) count = std::min(count, maxeval - evals);
    last_ran = false;
    if (count <= 0 || status != LC2_OK) return out;
    last_ran = true;
    std::vector<double> X((size_t)count * n);
    for (int k = 0; k < count; ++k) {
      std::vector<double> x = to_x(U[k]);
      std::copy(x.begin(), x.end(), X.begin() + (size_t)k * n);
    }
    int st = f(user, count, n, X.data(), out.data());
    if (st != 0) {
      status = st;
      return out;
    }
    evals += count;
    ++batches;
    for (int k = 0; k < count; ++k) {
      if (!std::isfinite(out[k])) out[k] = std::numeric_limits<double>::max();
      if (out[k] < best_f) {
        best_f = out[k];
        best_x.assign(X.begin() + (size_t)k * n, X.begin() + (size_t)(k + 1) * n);
      }
    }
    return out;
  }
};

// ---------------------------------------------------------------- DIRECT-L
struct Rect {
  std::vector<double> c;  // centre (unit cube)
  std::vector<int> level; // side of dimension i is 3^-level[i]
  double f;
};

double rect_size(const Rect& r) {
  // half of the longest side (locally biased measure)
  int m = *std::min_element(r.level.begin(), r.level.end());
  return 0.5 * std::pow(3.0, -m);
}

void direct_l(Problem& P, double xtol) {
  const int n = P.n;
  std::vector<Rect> rects;
  Rect r0;
  r0.c.assign(n, 0.5);
  r0.level.assign(n, 0);
  r0.f = P.eval({r0.c})[0];
  rects.push_back(r0);
  const double eps = 1e-4;
  while (P.status == LC2_OK && P.budget_left()) {
    // potentially optimal rectangles: best per size class, lower convex hull
    std::map<double, int> best;  // size -> index
    for (int i = 0; i < (int)rects.size(); ++i) {
      const double d = rect_size(rects[i]);
      auto it = best.find(d);
      if (it == best.end() || rects[i].f < rects[it->second].f) best[d] = i;
    }
    std::vector<std::pair<double, int>> cand(best.begin(), best.end());  // ascending size
    double fmin = std::numeric_limits<double>::infinity();
    for (auto& r : rects) fmin = std::min(fmin, r.f);
    std::vector<int> po;
    for (size_t a = 0; a < cand.size(); ++a) {
      const double da = cand[a].first, fa = rects[cand[a].second].f;
      double kmin = 0.0, kmax = std::numeric_limits<double>::infinity();
      bool ok = true;
      for (size_t b = 0; b < cand.size() && ok; ++b) {
        if (b == a) continue;
        const double db = cand[b].first, fb = rects[cand[b].second].f;
        if (db < da) kmin = std::max(kmin, (fa - fb) / (da - db));
        else if (db > da) kmax = std::min(kmax, (fb - fa) / (db - da));
      }
      if (kmin > kmax) ok = false;
      // epsilon condition: a meaningful improvement is possible
      if (ok && std::isfinite(kmax) && fa - kmax * da > fmin - eps * std::fabs(fmin)) ok = false;
      if (ok) po.push_back(cand[a].second);
    }
    if (po.empty()) po.push_back(cand.front().second);
    // stop when every selected rectangle is below the resolution
    bool all_small = true;
    for (int i : po)
      if (rect_size(rects[i]) * 2.0 > xtol) all_small = false;
    if (all_small && xtol > 0) break;
    // sample all children of all selected rectangles in one batch
    struct Job {
      int rect;
      std::vector<int> dims;
    };
    std::vector<Job> jobs;
    std::vector<std::vector<double>> pts;
    for (int i : po) {
      Job j;
      j.rect = i;
      const int m = *std::min_element(rects[i].level.begin(), rects[i].level.end());
      for (int d = 0; d < n; ++d)
        if (rects[i].level[d] == m) j.dims.push_back(d);
      const double delta = std::pow(3.0, -(m + 1));
      for (int d : j.dims) {
        std::vector<double> cp = rects[i].c, cm = rects[i].c;
        cp[d] += delta;
        cm[d] -= delta;
        pts.push_back(cp);
        pts.push_back(cm);
      }
      jobs.push_back(j);
    }
    if (!P.budget_left((int)pts.size())) {
      // spend the remainder on the first points; stop afterwards
      P.eval(std::vector<std::vector<double>>(pts.begin(), pts.begin() +
                                              std::max(0, P.maxeval - P.evals)));
      break;
    }
    std::vector<double> fv = P.eval(pts);
    if (P.status != LC2_OK) break;
    size_t k = 0;
    std::vector<Rect> born;
    for (auto& j : jobs) {
      const int m = *std::min_element(rects[j.rect].level.begin(), rects[j.rect].level.end());
      const double delta = std::pow(3.0, -(m + 1));
      std::vector<std::pair<double, int>> order;  // (min of the two values, dim slot)
      std::vector<double> fp(j.dims.size()), fm(j.dims.size());
      for (size_t s = 0; s < j.dims.size(); ++s) {
        fp[s] = fv[k++];
        fm[s] = fv[k++];
        order.push_back({std::min(fp[s], fm[s]), (int)s});
      }
      std::sort(order.begin(), order.end());
      Rect& parent = rects[j.rect];
      for (auto& o : order) {
        const int d = j.dims[o.second];
        parent.level[d] = m + 1;
        Rect a = parent, b = parent;
        a.c[d] += delta;
        a.f = fp[o.second];
        b.c[d] -= delta;
        b.f = fm[o.second];
        born.push_back(a);
        born.push_back(b);
      }
    }
    rects.insert(rects.end(), born.begin(), born.end());
  }
}

// ----------------------------------------------------- trust-region stage
void trust_region(Problem& P, std::vector<double> u, double rho, double xtol) {
  const int n = P.n;
  auto clamp01 = [](double v) { return std::min(1.0, std::max(0.0, v)); };
  double fx = P.eval({u})[0];
  while (P.status == LC2_OK && P.budget_left() && rho >= xtol) {
    // stencil x +- rho e_i, clipped to the unit box
    std::vector<std::vector<double>> pts;
    std::vector<double> hp(n), hm(n);
    for (int i = 0; i < n; ++i) {
      std::vector<double> a = u, b = u;
      a[i] = clamp01(u[i] + rho);
      b[i] = clamp01(u[i] - rho);
      hp[i] = a[i] - u[i];
      hm[i] = u[i] - b[i];
      pts.push_back(a);
      pts.push_back(b);
    }
    std::vector<double> fs = P.eval(pts);
    if (P.status != LC2_OK) break;
    // separable quadratic model and its minimiser in the trust box
    std::vector<double> step(n, 0.0);
    int best_k = -1;
    double best_f = fx;
    for (int k = 0; k < 2 * n; ++k)
      if (fs[k] < best_f) {
        best_f = fs[k];
        best_k = k;
      }
    for (int i = 0; i < n; ++i) {
      const double fpv = fs[2 * i], fmv = fs[2 * i + 1];
      const double a = hp[i], b = hm[i];
      double s = 0.0;
      if (a > 0 && b > 0) {
        // quadratic through (-b, fm), (0, fx), (a, fp)
        const double g = (fpv * b * b - fmv * a * a - fx * (b * b - a * a)) / (a * b * (a + b));
        const double h = 2.0 * (fpv * b + fmv * a - fx * (a + b)) / (a * b * (a + b));
        if (h > 0)
          s = -g / h;
        else
          s = (g > 0) ? -rho : rho;
      } else if (a > 0) {
        s = (fpv < fx) ? a : 0.0;
      } else if (b > 0) {
        s = (fmv < fx) ? -b : 0.0;
      }
      s = std::max(-rho, std::min(rho, s));
      step[i] = clamp01(u[i] + s) - u[i];
    }
    double sn = 0.0;
    for (double s : step) sn = std::max(sn, std::fabs(s));
    std::vector<double> cand(n);
    for (int i = 0; i < n; ++i) cand[i] = u[i] + step[i];
    double fc = std::numeric_limits<double>::infinity();
    if (sn > 0 && P.budget_left()) fc = P.eval({cand})[0];
    if (P.status != LC2_OK) break;
    if (fc < best_f) {
      u = cand;
      fx = fc;
      if (sn >= 0.999 * rho) rho = std::min(0.5, rho * 1.5);
    } else if (best_k >= 0) {
      u = pts[best_k];
      fx = best_f;
    } else {
      rho *= 0.5;
    }
  }
}

// ------------------------------------------------------------------ BOBYQA
// Powell, "The BOBYQA algorithm for bound constrained optimization without
// derivatives", DAMTP 2009/NA06 -- the method of NLopt's LN_BOBYQA, which the
// reference's local rounds call (src/Optimizers/optimizers.cu:385-390,
// 937-946, 1548-1553). Written here from the published method:
//   * m = 2n+1 interpolation points; the first model interpolates f at x0 and
//     x0 + s_i e_i, x0 + t_i e_i (s_i, t_i = +-rho_beg, or +rho_beg and
//     +2 rho_beg at a bound), all 2n+1 values requested as one batch;
//   * after each new point the model changes by the quadratic D of least
//     Frobenius norm of its Hessian that restores interpolation, i.e. the
//     solution of the (m+n+1) KKT system [[A, X'], [X, 0]] with
//     A_ij = (v_i . v_j)^2 / 2, X = [1; v_j], v_j = y_j - x_opt. Powell keeps
//     that system's inverse by updating formulas; here it is factorised
//     afresh after each change (n <= 12: a 37 x 37 LU), and the same
//     factorisation gives the Lagrange functions used below;
//   * trust-region step: the model minimised within ||d|| <= Delta and the
//     bounds by truncated conjugate gradients whose variables are fixed as
//     they reach a bound (the first phase of Powell's TRSBOX);
//   * the point replaced by a new one maximises |l_t(x_new)| weighted by
//     max(1, (|y_t - x_opt| / Delta)^2)^2 (Powell's denominator weighting);
//   * geometry steps (ALTMOV's role): a point farther than max(2 Delta,
//     10 rho) from x_opt is moved to where its Lagrange function is largest
//     in magnitude within the bounds and a ball of radius
//     max(min(dist / 10, Delta), rho), searched along the lines through the
//     other points and along the projected gradient;
//   * Delta follows the ratio of actual to predicted reduction, rho falls
//     from rho_beg to rho_end in Powell's steps (0.1, or sqrt and end
//     factors near rho_end) when steps stop succeeding.
namespace bobyqa {

// Dense LU with partial pivoting of an N x N row-major matrix.
struct LU {
  int N = 0;
  std::vector<double> a;
  std::vector<int> piv;
  bool factor() {
    piv.resize(N);
    double scale = 0.0;
    for (double v : a) scale = std::max(scale, std::fabs(v));
    for (int k = 0; k < N; ++k) {
      int p = k;
      for (int i = k + 1; i < N; ++i)
        if (std::fabs(a[(size_t)i * N + k]) > std::fabs(a[(size_t)p * N + k])) p = i;
      piv[k] = p;
      if (!(std::fabs(a[(size_t)p * N + k]) > 1e-14 * scale)) return false;
      if (p != k)
        for (int j = 0; j < N; ++j) std::swap(a[(size_t)k * N + j], a[(size_t)p * N + j]);
      const double d = a[(size_t)k * N + k];
      for (int i = k + 1; i < N; ++i) {
        const double l = a[(size_t)i * N + k] / d;
        a[(size_t)i * N + k] = l;
        if (l != 0.0)
          for (int j = k + 1; j < N; ++j) a[(size_t)i * N + j] -= l * a[(size_t)k * N + j];
      }
    }
    return true;
  }
  // rows were swapped whole during factor(), so the interchanges are applied
  // to b first, then the unit-lower and upper triangular solves
  void solve(std::vector<double>& b) const {
    for (int k = 0; k < N; ++k) std::swap(b[k], b[piv[k]]);
    for (int k = 0; k < N; ++k)
      for (int i = k + 1; i < N; ++i) b[i] -= a[(size_t)i * N + k] * b[k];
    for (int k = N - 1; k >= 0; --k) {
      for (int j = k + 1; j < N; ++j) b[k] -= a[(size_t)k * N + j] * b[j];
      b[k] /= a[(size_t)k * N + k];
    }
  }
};

class Solver {
 public:
  Solver(Problem& P, const std::vector<double>& u0, double rhobeg, double rhoend)
      : P_(P), n_(P.n), m_(2 * P.n + 1), rhobeg_(std::min(rhobeg, 0.5)),
        rhoend_(std::min(rhoend, std::min(rhobeg, 0.5))), x0_(u0) {}

  void run() {
    if (!initial_points()) return;
    double rho = rhobeg_, delta = rho;
    while (P_.status == LC2_OK && P_.budget_left()) {
      if (!update_model()) {
        // a degenerate interpolation set: restart it around x_opt, once per rho
        if (rescued_at_ == rho || !rescue(rho)) return;
        rescued_at_ = rho;
        continue;
      }
      std::vector<double> d = trsbox(delta);
      const double dnorm = norm(d);
      double ratio = -1.0;
      if (dnorm >= 0.5 * rho) {
        std::vector<double> xn(n_);
        for (int i = 0; i < n_; ++i) xn[i] = clamp01(Y_[kopt_][i] + d[i]);
        const double pred = -model_change(d);
        const double fnew = P_.eval({xn})[0];
        if (P_.status != LC2_OK || !P_.budget_used_once()) return;
        const double fopt = F_[kopt_];
        ratio = pred > 0.0 ? (fopt - fnew) / pred : -1.0;
        if (ratio <= 0.1)
          delta = std::min(0.5 * delta, dnorm);
        else if (ratio <= 0.7)
          delta = std::max(0.5 * delta, dnorm);
        else
          delta = std::max(0.5 * delta, 2.0 * dnorm);
        if (delta <= 1.5 * rho) delta = rho;
        const bool better = fnew < fopt;
        const int knew = replacement(xn, better, delta);
        Y_[knew] = xn;
        F_[knew] = fnew;
        if (better) kopt_ = knew;
        if (ratio >= 0.1) continue;
      } else {
        delta = 0.5 * delta;
        if (delta <= 1.5 * rho) delta = rho;
      }
      // poor or short step: improve the geometry where a point is far away
      const int far = far_point();
      const double dist = std::sqrt(dist2(far));
      if (dist > std::max(2.0 * delta, 10.0 * rho)) {
        if (!update_model()) continue;  // the next iteration rescues the set
        if (!geometry(far, std::max(std::min(0.1 * dist, delta), rho), rho)) return;
        continue;
      }
      // (a step on the boundary of a trust region of radius rho measures rho
      // within rounding: the comparison allows for it)
      if (ratio > 0.0 || std::max(delta, dnorm) > (1.0 + 1e-6) * rho) continue;
      // the model is as good as rho allows: refine rho
      if (rho <= rhoend_) return;
      const double r = rho / rhoend_;
      const double rho_new = r <= 16.0 ? rhoend_ : (r <= 250.0 ? std::sqrt(r) * rhoend_ : 0.1 * rho);
      delta = std::max(0.5 * rho, rho_new);
      rho = rho_new;
    }
  }

 private:
  static double clamp01(double v) { return std::min(1.0, std::max(0.0, v)); }
  static double norm(const std::vector<double>& v) {
    double s = 0.0;
    for (double x : v) s += x * x;
    return std::sqrt(s);
  }
  double dist2(int t) const {
    double s = 0.0;
    for (int i = 0; i < n_; ++i) s += (Y_[t][i] - Y_[kopt_][i]) * (Y_[t][i] - Y_[kopt_][i]);
    return s;
  }
  int far_point() const {
    int k = 0;
    double best = -1.0;
    for (int t = 0; t < m_; ++t)
      if (dist2(t) > best) {
        best = dist2(t);
        k = t;
      }
    return k;
  }

  // x0 moved to a bound where it lies within rho_beg of one (Powell's rule),
  // then the 2n+1 initial points, evaluated as one batch
  bool initial_points() {
    const double rb = rhobeg_;
    for (int i = 0; i < n_; ++i) {
      double& x = x0_[i];
      x = clamp01(x);
      if (x < rb) x = (x <= 0.5 * rb) ? 0.0 : rb;
      if (x > 1.0 - rb) x = (x >= 1.0 - 0.5 * rb) ? 1.0 : 1.0 - rb;
    }
    Y_.assign(m_, x0_);
    for (int i = 0; i < n_; ++i) {
      double s = rb, t = -rb;
      if (x0_[i] <= 0.0) t = 2.0 * rb;
      if (x0_[i] >= 1.0) {
        s = -rb;
        t = -2.0 * rb;
      }
      Y_[1 + i][i] = clamp01(x0_[i] + s);
      Y_[1 + n_ + i][i] = clamp01(x0_[i] + t);
    }
    F_ = P_.eval(Y_);
    if (P_.status != LC2_OK) return false;
    kopt_ = (int)(std::min_element(F_.begin(), F_.end()) - F_.begin());
    xb_ = Y_[kopt_];
    c_ = 0.0;
    g_.assign(n_, 0.0);
    H_.assign((size_t)n_ * n_, 0.0);
    return std::all_of(F_.begin(), F_.end(), [](double v) { return std::isfinite(v); });
  }

  // q(x) - q(x_opt) for x = x_opt + d, the model based at x_opt
  double model_change(const std::vector<double>& d) const {
    double s = 0.0;
    for (int i = 0; i < n_; ++i) {
      double hd = 0.0;
      for (int j = 0; j < n_; ++j) hd += H_[(size_t)i * n_ + j] * d[j];
      s += d[i] * (g_[i] + 0.5 * hd);
    }
    return s;
  }
  double model_at(const std::vector<double>& x) const {
    std::vector<double> d(n_);
    for (int i = 0; i < n_; ++i) d[i] = x[i] - xb_[i];
    return c_ + model_change(d);
  }

  // Rebases the model at x_opt, factorises the KKT matrix of the current
  // points (scaled by their largest distance s from x_opt) and applies the
  // least-Frobenius-norm correction that interpolates every value again.
  bool update_model() {
    const std::vector<double>& xo = Y_[kopt_];
    {
      std::vector<double> d(n_);
      for (int i = 0; i < n_; ++i) d[i] = xo[i] - xb_[i];
      c_ += model_change(d);
      for (int i = 0; i < n_; ++i) {
        double hd = 0.0;
        for (int j = 0; j < n_; ++j) hd += H_[(size_t)i * n_ + j] * d[j];
        g_[i] += hd;
      }
      xb_ = xo;
    }
    s_ = 0.0;
    for (int t = 0; t < m_; ++t) s_ = std::max(s_, std::sqrt(dist2(t)));
    if (!(s_ > 0.0)) return false;
    W_.assign((size_t)m_ * n_, 0.0);
    for (int t = 0; t < m_; ++t)
      for (int i = 0; i < n_; ++i) W_[(size_t)t * n_ + i] = (Y_[t][i] - xb_[i]) / s_;
    const int N = m_ + n_ + 1;
    lu_.N = N;
    lu_.a.assign((size_t)N * N, 0.0);
    for (int a = 0; a < m_; ++a) {
      for (int b = 0; b < m_; ++b) {
        double dot = 0.0;
        for (int i = 0; i < n_; ++i) dot += W_[(size_t)a * n_ + i] * W_[(size_t)b * n_ + i];
        lu_.a[(size_t)a * N + b] = 0.5 * dot * dot;
      }
      lu_.a[(size_t)a * N + m_] = lu_.a[(size_t)m_ * N + a] = 1.0;
      for (int i = 0; i < n_; ++i)
        lu_.a[(size_t)a * N + m_ + 1 + i] = lu_.a[(size_t)(m_ + 1 + i) * N + a] =
            W_[(size_t)a * n_ + i];
    }
    if (!lu_.factor()) return false;
    std::vector<double> rhs(N, 0.0);
    for (int t = 0; t < m_; ++t) rhs[t] = F_[t] - model_at(Y_[t]);
    lu_.solve(rhs);
    c_ += rhs[m_];
    for (int i = 0; i < n_; ++i) g_[i] += rhs[m_ + 1 + i] / s_;
    add_hessian(rhs.data(), H_);
    return true;
  }
  // H += sum_t lambda_t w_t w_t' / s^2
  void add_hessian(const double* lambda, std::vector<double>& H) const {
    for (int t = 0; t < m_; ++t) {
      const double l = lambda[t] / (s_ * s_);
      if (l == 0.0) continue;
      const double* w = &W_[(size_t)t * n_];
      for (int i = 0; i < n_; ++i)
        for (int j = 0; j < n_; ++j) H[(size_t)i * n_ + j] += l * w[i] * w[j];
    }
  }
  // The KKT column z of a point x (scaled), and u = W^-1 z: u_t = l_t(x),
  // the values of all Lagrange functions at x (W is symmetric).
  void lagrange_at(const std::vector<double>& x, std::vector<double>& z,
                   std::vector<double>& u) const {
    const int N = m_ + n_ + 1;
    std::vector<double> wx(n_);
    z.assign(N, 0.0);
    for (int i = 0; i < n_; ++i) wx[i] = (x[i] - xb_[i]) / s_;
    for (int t = 0; t < m_; ++t) {
      double dot = 0.0;
      for (int i = 0; i < n_; ++i) dot += W_[(size_t)t * n_ + i] * wx[i];
      z[t] = 0.5 * dot * dot;
    }
    z[m_] = 1.0;
    for (int i = 0; i < n_; ++i) z[m_ + 1 + i] = wx[i];
    u = z;
    lu_.solve(u);
  }

  // The point that x_new replaces: the largest |sigma_t| (the ratio of the
  // KKT determinants after and before the exchange, Powell's denominator
  // sigma_t = alpha_t beta + tau_t^2 with tau_t = l_t(x_new), alpha_t the
  // t-th diagonal element of W^-1 and beta = |v|^4 / 2 - z' W^-1 z), weighted
  // by max(1, |y_t - x_opt|^2 / Delta^2)^2 so that distant points go first.
  // A nonzero sigma keeps the interpolation system nonsingular.
  int replacement(const std::vector<double>& xn, bool better, double delta) const {
    std::vector<double> z, u;
    lagrange_at(xn, z, u);
    double vv = 0.0;
    for (int i = 0; i < n_; ++i) vv += z[m_ + 1 + i] * z[m_ + 1 + i];
    double zu = 0.0;
    for (size_t i = 0; i < z.size(); ++i) zu += z[i] * u[i];
    const double beta = 0.5 * vv * vv - zu;
    const int N = m_ + n_ + 1;
    int k = -1;
    double best = -1.0;
    for (int t = 0; t < m_; ++t) {
      if (t == kopt_ && !better) continue;
      std::vector<double> e(N, 0.0);
      e[t] = 1.0;
      lu_.solve(e);
      const double sigma = e[t] * beta + u[t] * u[t];
      const double w = std::max(1.0, dist2(t) / (delta * delta));
      const double score = w * w * std::fabs(sigma);
      if (score > best) {
        best = score;
        k = t;
      }
    }
    return k < 0 ? far_point() : k;
  }

  // A fresh interpolation set around x_opt at radius rho (the role of
  // Powell's RESCUE, here as a restart): x_opt +- rho e_i, or +rho and +2 rho
  // (-rho and -2 rho) next to a bound; the 2n new points come as one batch.
  bool rescue(double rho) {
    const std::vector<double> xo = Y_[kopt_];
    const double fo = F_[kopt_];
    std::vector<std::vector<double>> pts;
    for (int i = 0; i < n_; ++i) {
      double s = rho, t = -rho;
      if (xo[i] + rho > 1.0) {
        s = -rho;
        t = (xo[i] - 2.0 * rho >= 0.0) ? -2.0 * rho : 0.5 * rho;
      } else if (xo[i] - rho < 0.0) {
        t = (xo[i] + 2.0 * rho <= 1.0) ? 2.0 * rho : -0.5 * rho;
      }
      std::vector<double> a = xo, b = xo;
      a[i] = clamp01(xo[i] + s);
      b[i] = clamp01(xo[i] + t);
      pts.push_back(a);
      pts.push_back(b);
    }
    std::vector<double> f = P_.eval(pts);
    if (P_.status != LC2_OK || !P_.budget_used_once()) return false;
    Y_.assign(1, xo);
    F_.assign(1, fo);
    for (size_t k = 0; k < pts.size(); ++k) {
      Y_.push_back(pts[k]);
      F_.push_back(f[k]);
    }
    kopt_ = (int)(std::min_element(F_.begin(), F_.end()) - F_.begin());
    xb_ = Y_[kopt_];
    c_ = 0.0;
    g_.assign(n_, 0.0);
    H_.assign((size_t)n_ * n_, 0.0);
    return true;
  }

  // Moves point k to where |l_k| is largest within radius adelt of x_opt and
  // the bounds, evaluates it there and replaces it.
  bool geometry(int k, double adelt, double rho) {
    if (k == kopt_) return false;
    const int N = m_ + n_ + 1;
    std::vector<double> e(N, 0.0);
    e[k] = 1.0;
    lu_.solve(e);  // l_k: lambda (m), c, g (scaled)
    std::vector<double> gl(n_), Hl((size_t)n_ * n_, 0.0);
    for (int i = 0; i < n_; ++i) gl[i] = e[m_ + 1 + i] / s_;
    add_hessian(e.data(), Hl);
    const std::vector<double>& xo = Y_[kopt_];
    double best = -1.0;
    std::vector<double> xbest;
    // |l_k| along a unit direction u from x_opt within the ball and the box
    auto line = [&](const std::vector<double>& u) {
      double slope = 0.0, curv = 0.0, amax = adelt, amin = -adelt;
      for (int i = 0; i < n_; ++i) {
        slope += gl[i] * u[i];
        double hu = 0.0;
        for (int j = 0; j < n_; ++j) hu += Hl[(size_t)i * n_ + j] * u[j];
        curv += u[i] * hu;
        if (u[i] > 0) {
          amax = std::min(amax, (1.0 - xo[i]) / u[i]);
          amin = std::max(amin, -xo[i] / u[i]);
        } else if (u[i] < 0) {
          amax = std::min(amax, -xo[i] / u[i]);
          amin = std::max(amin, (1.0 - xo[i]) / u[i]);
        }
      }
      std::vector<double> cand = {amin, amax};
      if (curv != 0.0) {
        const double a = -slope / curv;
        if (a > amin && a < amax) cand.push_back(a);
      }
      for (double a : cand) {
        if (std::fabs(a) < 1e-3 * rho) continue;
        const double v = std::fabs(a * slope + 0.5 * a * a * curv);
        if (v > best) {
          best = v;
          xbest.resize(n_);
          for (int i = 0; i < n_; ++i) xbest[i] = clamp01(xo[i] + a * u[i]);
        }
      }
    };
    for (int t = 0; t < m_; ++t) {
      if (t == kopt_) continue;
      std::vector<double> u(n_);
      for (int i = 0; i < n_; ++i) u[i] = Y_[t][i] - xo[i];
      const double len = norm(u);
      if (!(len > 0)) continue;
      for (double& v : u) v /= len;
      line(u);
    }
    // projected gradient of l_k (both signs are tried by the line search)
    {
      std::vector<double> u(gl);
      for (int i = 0; i < n_; ++i)
        if ((xo[i] <= 0.0 && u[i] < 0) || (xo[i] >= 1.0 && u[i] > 0)) u[i] = 0.0;
      const double len = norm(u);
      if (len > 0) {
        for (double& v : u) v /= len;
        line(u);
      }
    }
    if (xbest.empty()) return false;
    const double f = P_.eval({xbest})[0];
    if (P_.status != LC2_OK || !P_.budget_used_once()) return false;
    Y_[k] = xbest;
    F_[k] = f;
    if (f < F_[kopt_]) kopt_ = k;
    return true;
  }

  // Truncated conjugate gradients on the model within ||d|| <= delta and the
  // unit box; a variable that reaches its bound is fixed there and the
  // iteration restarts on the others.
  std::vector<double> trsbox(double delta) const {
    const std::vector<double>& xo = Y_[kopt_];
    std::vector<double> d(n_, 0.0), gq(g_), p(n_, 0.0), hp(n_);
    std::vector<char> fixed(n_, 0);
    for (int i = 0; i < n_; ++i)
      if ((xo[i] <= 0.0 && gq[i] >= 0.0) || (xo[i] >= 1.0 && gq[i] <= 0.0)) fixed[i] = 1;
    bool restart = true;
    double gg_prev = 0.0, gg0 = -1.0;
    for (int it = 0; it < 4 * n_ + 4; ++it) {
      double gg = 0.0;
      for (int i = 0; i < n_; ++i)
        if (!fixed[i]) gg += gq[i] * gq[i];
      if (gg0 < 0) gg0 = gg;
      if (!(gg > 1e-24 * std::max(gg0, 1e-300)) || gg == 0.0) break;
      if (restart) {
        for (int i = 0; i < n_; ++i) p[i] = fixed[i] ? 0.0 : -gq[i];
      } else {
        const double beta = gg / gg_prev;
        for (int i = 0; i < n_; ++i) p[i] = fixed[i] ? 0.0 : -gq[i] + beta * p[i];
      }
      gg_prev = gg;
      restart = false;
      double pp = 0.0, dp = 0.0, dd = 0.0, gp = 0.0, php = 0.0;
      for (int i = 0; i < n_; ++i) {
        double s = 0.0;
        for (int j = 0; j < n_; ++j) s += H_[(size_t)i * n_ + j] * p[j];
        hp[i] = s;
      }
      for (int i = 0; i < n_; ++i) {
        pp += p[i] * p[i];
        dp += d[i] * p[i];
        dd += d[i] * d[i];
        gp += gq[i] * p[i];
        php += p[i] * hp[i];
      }
      if (!(pp > 0) || gp >= 0) break;
      const double a_tr = (-dp + std::sqrt(std::max(0.0, dp * dp + pp * (delta * delta - dd)))) / pp;
      const double a_cg = php > 0 ? -gp / php : std::numeric_limits<double>::infinity();
      double a_bd = std::numeric_limits<double>::infinity();
      int ib = -1;
      for (int i = 0; i < n_; ++i) {
        if (fixed[i] || p[i] == 0.0) continue;
        const double room = p[i] > 0 ? (1.0 - xo[i] - d[i]) / p[i] : (-xo[i] - d[i]) / p[i];
        if (room < a_bd) {
          a_bd = room;
          ib = i;
        }
      }
      const double a = std::max(0.0, std::min(a_tr, std::min(a_cg, a_bd)));
      for (int i = 0; i < n_; ++i) {
        d[i] += a * p[i];
        gq[i] += a * hp[i];
      }
      if (ib >= 0 && a_bd <= std::min(a_tr, a_cg)) {
        fixed[ib] = 1;
        d[ib] = (p[ib] > 0 ? 1.0 : 0.0) - xo[ib];
        restart = true;
        continue;
      }
      if (a_tr <= a_cg) break;  // on the trust-region boundary
    }
    return d;
  }

  Problem& P_;
  const int n_, m_;
  const double rhobeg_, rhoend_;
  std::vector<double> x0_;
  std::vector<std::vector<double>> Y_;
  std::vector<double> F_;
  int kopt_ = 0;
  std::vector<double> xb_, g_, H_, W_;
  double c_ = 0.0, s_ = 1.0;
  double rescued_at_ = -1.0;  // rho of the last restart of the interpolation set
  LU lu_;
};

}  // namespace bobyqa

// -------------------------------------------------------------- Nelder-Mead
void nelder_mead(Problem& P, std::vector<double> u, double step, double xtol) {
  const int n = P.n;
  auto clamp = [](std::vector<double> v) {
    for (double& x : v) x = std::min(1.0, std::max(0.0, x));
    return v;
  };
  std::vector<std::vector<double>> S{clamp(u)};
  for (int i = 0; i < n; ++i) {
    std::vector<double> v = u;
    v[i] = (u[i] + step <= 1.0) ? u[i] + step : u[i] - step;
    S.push_back(clamp(v));
  }
  std::vector<double> F = P.eval(S);
  while (P.status == LC2_OK && P.budget_left()) {
    std::vector<int> idx(n + 1);
    for (int i = 0; i <= n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int a, int b) { return F[a] < F[b]; });
    double diam = 0.0;
    for (int i = 1; i <= n; ++i)
      for (int d = 0; d < n; ++d) diam = std::max(diam, std::fabs(S[idx[i]][d] - S[idx[0]][d]));
    if (diam < xtol) break;
    std::vector<double> c(n, 0.0);
    for (int i = 0; i < n; ++i)
      for (int d = 0; d < n; ++d) c[d] += S[idx[i]][d] / n;
    const std::vector<double>& w = S[idx[n]];
    auto at = [&](double t) {
      std::vector<double> p(n);
      for (int d = 0; d < n; ++d) p[d] = c[d] + t * (w[d] - c[d]);
      return clamp(p);
    };
    // reflection, expansion, outside and inside contraction together
    std::vector<std::vector<double>> trial{at(-1.0), at(-2.0), at(-0.5), at(0.5)};
    std::vector<double> ft = P.eval(trial);
    if (P.status != LC2_OK) break;
    const double fb = F[idx[0]], fs = F[idx[n - 1]], fw = F[idx[n]];
    int pick = -1;
    if (ft[0] < fb)
      pick = (ft[1] < ft[0]) ? 1 : 0;
    else if (ft[0] < fs)
      pick = 0;
    else if (ft[0] < fw)
      pick = (ft[2] <= ft[0]) ? 2 : -1;
    else
      pick = (ft[3] < fw) ? 3 : -1;
    if (pick >= 0) {
      S[idx[n]] = trial[pick];
      F[idx[n]] = ft[pick];
    } else {
      // shrink towards the best vertex
      std::vector<std::vector<double>> sh;
      for (int i = 1; i <= n; ++i) {
        std::vector<double> p(n);
        for (int d = 0; d < n; ++d) p[d] = S[idx[0]][d] + 0.5 * (S[idx[i]][d] - S[idx[0]][d]);
        sh.push_back(p);
      }
      std::vector<double> fsh = P.eval(sh);
      for (int i = 1; i <= n; ++i) {
        S[idx[i]] = sh[i - 1];
        F[idx[i]] = fsh[i - 1];
      }
    }
  }
}

}  // namespace

extern "C" int lc2_minimize(const lc2_opt_problem* p, lc2_batch_objective f, void* user,
                            double* x, double* fmin, lc2_opt_report* rep) {
  lc2_set_error_message("");
  if (!p || !f || !x || p->dim < 1 || !p->lower || !p->upper) {
    lc2_set_error_message("lc2_minimize: bad arguments");
    return LC2_ERR_INVALID_ARGUMENT;
  }
  Problem P;
  P.n = p->dim;
  P.lo.assign(p->lower, p->lower + p->dim);
  P.hi.assign(p->upper, p->upper + p->dim);
  P.f = f;
  P.user = user;
  P.maxeval = p->maxeval;
  for (int i = 0; i < P.n; ++i) {
    if (!(P.hi[i] >= P.lo[i]) || !std::isfinite(P.lo[i]) || !std::isfinite(P.hi[i])) {
      lc2_set_error_message("lc2_minimize: bounds must be finite with lower <= upper");
      return LC2_ERR_INVALID_ARGUMENT;
    }
    if (P.hi[i] == P.lo[i]) P.hi[i] = P.lo[i] + 1e-300;  // a pinned entry
  }
  std::vector<double> u(P.n);
  for (int i = 0; i < P.n; ++i) {
    const double xi = std::min(P.hi[i], std::max(P.lo[i], x[i]));
    u[i] = (xi - P.lo[i]) / (P.hi[i] - P.lo[i]);
  }
  const double xtol = p->xtol_rel > 0 ? p->xtol_rel : 1e-6;
  const double step = p->initial_step > 0 ? p->initial_step : 0.1;
  switch (p->algorithm) {
    case LC2_OPT_DIRECT_L: direct_l(P, xtol); break;
    case LC2_OPT_BOBYQA: bobyqa::Solver(P, u, step, xtol).run(); break;
    case LC2_OPT_QUAD_TR: trust_region(P, u, step, xtol); break;
    case LC2_OPT_NELDER_MEAD: nelder_mead(P, u, step, xtol); break;
    default:
      lc2_set_error_message("lc2_minimize: unknown algorithm");
      return LC2_ERR_INVALID_ARGUMENT;
  }
  if (P.status != LC2_OK) {
    if (rep) rep->evaluations = P.evals;
    return P.status;
  }
  if (!P.best_x.empty()) std::copy(P.best_x.begin(), P.best_x.end(), x);
  if (fmin) *fmin = P.best_f;
  if (rep) {
    rep->evaluations = P.evals;
    rep->batches = P.batches;
  }
  return LC2_OK;
}

// ------------------------------------------------------- registration driver
namespace {

struct RegObjective {
  lc2_context* ctx;
  const lc2_registration* reg;
  std::vector<double> base;  // full parameter vector (reference order)
  std::vector<int> map;      // optimised entry k -> parameter index
  std::vector<float> mats;
  std::vector<double> lc2;
  long long evaluations = 0;
  int stage = 0;  // 0 = DIRECT, r + 1 = local round r
  bool maximize = false;  // NMI (PatchSize 0): maximise the value itself
};

int params_of(int mode) { return mode == LC2_MODE_2D ? 6 : 12; }

// parameter indices of an entry group (src/Optimizers/optimizers.cu:137-164, 668-700)
void entry_indices(int mode, int mask, std::vector<int>& out) {
  out.clear();
  if (mode == LC2_MODE_2D) {
    if (mask & LC2_ENTRY_TRANSLATION) { out.push_back(0); out.push_back(1); }
    if (mask & LC2_ENTRY_ROTATION) out.push_back(2);
    if (mask & LC2_ENTRY_SCALE) { out.push_back(3); out.push_back(4); }
    if (mask & LC2_ENTRY_SHEAR) out.push_back(5);
    return;
  }
  for (int g = 0; g < 4; ++g)
    if (mask & (1 << g))
      for (int i = 0; i < 3; ++i) out.push_back(3 * g + i);
}

int build_matrix(int mode, const double* p, const float* center, const float* shift, float* m) {
  if (mode == LC2_MODE_2D) {
    const float t[2] = {(float)p[0], (float)p[1]};
    const float s[2] = {(float)p[3], (float)p[4]};
    return lc2_affine_2d((float)p[2], t, s, (float)p[5], center, shift, m);
  }
  const float t[3] = {(float)p[0], (float)p[1], (float)p[2]};
  const float r[3] = {(float)p[3], (float)p[4], (float)p[5]};
  const float s[3] = {(float)p[6], (float)p[7], (float)p[8]};
  const float h[3] = {(float)p[9], (float)p[10], (float)p[11]};
  return lc2_affine_3d(r, t, s, h, center, shift, m);
}

// objective -log(LC2) of a batch (Optimizers3D::operator(), optimizers.cu:650-728)
int reg_objective(void* user, int count, int dim, const double* x, double* f) {
  RegObjective* o = static_cast<RegObjective*>(user);
  const int mode = o->reg->mode;
  const int mf = (mode == LC2_MODE_2D) ? 9 : 16;
  o->mats.resize((size_t)count * mf);
  o->lc2.resize(count);
  std::vector<double> p(o->base);
  for (int k = 0; k < count; ++k) {
    for (int j = 0; j < dim; ++j) p[o->map[j]] = x[(size_t)k * dim + j];
    int st = build_matrix(mode, p.data(), o->reg->center, o->reg->shift,
                          o->mats.data() + (size_t)k * mf);
    if (st != LC2_OK) return st;
  }
  int st;
  if (o->ctx) {
    st = lc2_evaluate_batch(o->ctx, o->mats.data(), count, o->lc2.data());
  } else {
    std::vector<double> md(o->mats.begin(), o->mats.end());
    st = o->reg->lc2_of_matrices(o->reg->user, count, mf, md.data(), o->lc2.data());
  }
  if (st != LC2_OK) return st;
  for (int k = 0; k < count; ++k) {
    const double v = o->lc2[k];
    // -log(LC2) (optimizers.cu:728), or the NMI maximised as it is (:722-724, 855-860)
    if (o->maximize)
      f[k] = -v;
    else
      f[k] = (v > 0.0) ? -std::log(v) : std::numeric_limits<double>::max();
  }
  if (o->reg->observer) {
    const int np = params_of(mode);
    std::vector<double> all((size_t)count * np);
    for (int k = 0; k < count; ++k) {
      for (int j = 0; j < np; ++j) all[(size_t)k * np + j] = o->base[j];
      for (int j = 0; j < dim; ++j) all[(size_t)k * np + o->map[j]] = x[(size_t)k * dim + j];
    }
    o->reg->observer(o->reg->observer_user, o->stage, count, np, all.data(), o->lc2.data());
  }
  o->evaluations += count;
  return 0;
}

}  // namespace

extern "C" int lc2_register(lc2_context* ctx, const lc2_registration* reg,
                            lc2_registration_result* out) {
  lc2_set_error_message("");
  if ((!ctx && (!reg || !reg->lc2_of_matrices)) || !reg || !out) {
    lc2_set_error_message("lc2_register: null argument");
    return LC2_ERR_INVALID_ARGUMENT;
  }
  if (reg->mode < LC2_MODE_2D || reg->mode > LC2_MODE_2DTO3D || reg->rounds < 0 ||
      reg->rounds > 8) {
    lc2_set_error_message("lc2_register: bad mode or number of rounds");
    return LC2_ERR_INVALID_ARGUMENT;
  }
  const int np = params_of(reg->mode);
  RegObjective o;
  o.ctx = ctx;
  o.reg = reg;
  o.maximize = reg->maximize != 0;
  if (ctx) {
    lc2_config cfg;
    if (lc2_get_config(ctx, &cfg) == LC2_OK && cfg.patch_size == 0) o.maximize = true;
  }
  o.base.assign(reg->initial, reg->initial + np);
  int launches = 0;
  auto stage = [&](int algorithm, int mask, double xtol, int maxeval) -> int {
    entry_indices(reg->mode, mask, o.map);
    if (o.map.empty()) return LC2_OK;
    const int n = (int)o.map.size();
    std::vector<double> lo(n), hi(n), x(n);
    for (int j = 0; j < n; ++j) {
      lo[j] = reg->lower[o.map[j]];
      hi[j] = reg->upper[o.map[j]];
      x[j] = o.base[o.map[j]];
    }
    lc2_opt_problem p{};
    p.algorithm = algorithm;
    p.dim = n;
    p.lower = lo.data();
    p.upper = hi.data();
    p.xtol_rel = xtol;
    p.maxeval = maxeval;
    lc2_opt_report rep{};
    double fbest = 0.0;
    int st = lc2_minimize(&p, reg_objective, &o, x.data(), &fbest, &rep);
    if (st != LC2_OK) return st;
    launches += rep.batches;
    for (int j = 0; j < n; ++j) o.base[o.map[j]] = x[j];
    return LC2_OK;
  };
  int st = LC2_OK;
  if (reg->direct_entries) {
    o.stage = 0;
    st = stage(LC2_OPT_DIRECT_L, reg->direct_entries, 1e-4, reg->direct_maxeval);
  }
  const int local = reg->local_algorithm ? reg->local_algorithm : LC2_OPT_BOBYQA;
  for (int r = 0; st == LC2_OK && r < reg->rounds; ++r)
    if (reg->round_entries[r]) {
      o.stage = r + 1;
      st = stage(local, reg->round_entries[r], reg->round_xtol[r] > 0 ? reg->round_xtol[r] : 1e-4,
                 reg->round_maxeval);
    }
  if (st != LC2_OK) return st;
  // similarity at the optimum
  const int mf = (reg->mode == LC2_MODE_2D) ? 9 : 16;
  std::vector<float> m(mf);
  st = build_matrix(reg->mode, o.base.data(), reg->center, reg->shift, m.data());
  if (st == LC2_OK) {
    if (ctx) {
      st = lc2_evaluate(ctx, m.data(), &out->lc2);
    } else {
      std::vector<double> md(m.begin(), m.end());
      st = reg->lc2_of_matrices(reg->user, 1, mf, md.data(), &out->lc2);
    }
  }
  if (st != LC2_OK) return st;
  if (reg->observer)
    reg->observer(reg->observer_user, reg->rounds + 1, 1, np, o.base.data(), &out->lc2);
  for (int i = 0; i < 12; ++i) out->params[i] = (i < np) ? o.base[i] : 0.0;
  out->evaluations = (int)o.evaluations + 1;
  out->launches = launches + 1;
  return LC2_OK;
}

extern "C" int lc2_params_to_matrix(int mode, const double* params, const float center[3],
                                    const float shift[3], float* matrix) {
  if (!params || !center || !shift || !matrix) {
    lc2_set_error_message("lc2_params_to_matrix: null argument");
    return LC2_ERR_INVALID_ARGUMENT;
  }
  return build_matrix(mode, params, center, shift, matrix);
}
