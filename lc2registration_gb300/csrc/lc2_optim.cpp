// lc2_optim.cpp -- derivative-free bound-constrained optimizers with batched
// objective evaluation, and the registration driver built on them.
//
// The reference minimises -log(LC2) with NLopt: GN_ORIG_DIRECT_L on the
// entries enabled for DIRECT, then LN_BOBYQA rounds
// (src/Optimizers/optimizers.cu:734-970, 1349-1574). NLopt is not available
// here, so these are this library's own implementations, written from the
// published methods, with the same knobs (bounds, xtol_rel, maxeval). They
// differ from NLopt in that every step hands the objective a whole set of
// points at once -- all children of DIRECT's potentially optimal rectangles,
// a 2n+1-point stencil of the trust-region model, the four candidate points
// of a Nelder-Mead step -- so each step is one batched GPU launch.
//
//   DIRECT-L: Jones, Perttunen, Stuckman (1993), locally biased variant of
//     Gablonsky and Kelley (2001): one rectangle per size class, the lower
//     convex hull of (size, value) with the epsilon test, division along the
//     longest sides in order of the sampled values.
//   Trust region (the BOBYQA stage): a separable quadratic model from the
//     2n+1 points x, x +- rho e_i (Powell's initial BOBYQA model), its
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

  // evaluate unit-cube points (truncated to the remaining budget)
  std::vector<double> eval(const std::vector<std::vector<double>>& U) {
    std::vector<double> out(U.size(), std::numeric_limits<double>::infinity());
    int count = (int)U.size();
    if (maxeval > 0) count = std::min(count, maxeval - evals);
    if (count <= 0 || status != LC2_OK) return out;
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
    case LC2_OPT_BOBYQA: trust_region(P, u, step, xtol); break;
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
