// Oracle: CPU restatement of the geometric-multigrid V-cycle (test infrastructure).
//
// Uniform periodic meshes only. On such a mesh every multigrid level is a uniform
// periodic grid, the same-level ghost exchange is the periodic image, and the
// reference's block-wise restriction (gmg_restrict_send/recv) and prolongation
// (gmg_prolongate_send/recv + ProlongateSharedLinear) act cell by cell exactly as the
// global-array operations below; every value is produced by the same operations in the
// same order as in the reference.
//
// Reference files followed (parthenon-hpc-lab/parthenon):
//   src/solvers/mg_solver.hpp:37-57        MGParams (FAS on, SRJ2, max_coarsenings)
//   src/solvers/mg_solver.hpp:119-161      iteration: V-cycle, residual, rms check
//   src/solvers/mg_solver.hpp:163-186      levels max..min
//   src/solvers/mg_solver.hpp:222-297      Jacobi (weighted, robust::ratio)
//   src/solvers/mg_solver.hpp:312-345      SRJ stages and Yang-Mittal weights
//   src/solvers/mg_solver.hpp:375-520      per-level task sequence (FAS)
//   src/solvers/solver_utils.hpp:150-306   CopyData, AddFieldsAndStore, DotProduct
//   example/poisson_gmg/poisson_equation.hpp:59-210  SetDiagonal, fluxes, Ax
//   src/prolong_restrict/pr_ops.hpp:105-285  RestrictAverage, ProlongateSharedLinear
// Deviation: poisson_equation.hpp:153-157 stores the top z-face flux of a block into the
// x2 flux array; the restatement uses the evident 7-point operator (z-face flux on the
// z array), which is what every interior face of the reference computes.
#pragma once

#include <algorithm>
#include <cmath>
#include <vector>

namespace oracle {

struct GmgLevel {
  int n;           // cells per direction (periodic)
  double xmin, dx; // cell-centre coordinate of index i: xmin + (i + 0.5) dx
  std::vector<double> u, rhs, res, temp, u0;
  int64_t size() const { return (int64_t)n * n * n; }
  int64_t id(int k, int j, int i) const {
    const int kk = (k % n + n) % n, jj = (j % n + n) % n, ii = (i % n + n) % n;
    return ((int64_t)kk * n + jj) * n + ii;
  }
};

struct GmgParams {
  int smoother_stages = 2;       // SRJ stages (1, 2, 3), or Jacobi sweeps when jacobi
  bool jacobi = false;           // weighted Jacobi with `weight` instead of SRJ weights
  double weight = 2.0 / 3.0;
  int coarse_sweeps = 0;         // extra smoother passes at the coarsest level (0 = reference)
  double D = 1.0;                // face coefficient of div(D grad u)
  double alpha = 0.0;            // diagonal shift (poisson/diagonal_alpha)
};

struct Gmg {
  std::vector<GmgLevel> lv;  // lv[0] finest
  GmgParams p;

  Gmg(int n_fine, int ncoarsen, double xmin, double xmax, const GmgParams &pp) : p(pp) {
    int n = n_fine;
    for (int l = 0; l <= ncoarsen; ++l) {
      GmgLevel g;
      g.n = n;
      g.dx = (xmax - xmin) / n;
      g.xmin = xmin;
      const size_t s = (size_t)n * n * n;
      g.u.assign(s, 0.0);
      g.rhs.assign(s, 0.0);
      g.res.assign(s, 0.0);
      g.temp.assign(s, 0.0);
      g.u0.assign(s, 0.0);
      lv.push_back(std::move(g));
      n /= 2;
    }
  }

  // poisson_equation.hpp:104-210 (fluxes then FluxMultiplyMatrix), periodic
  double Ax_cell(const GmgLevel &g, const std::vector<double> &u, int k, int j, int i) const {
    const double D = p.D, dx = g.dx;
    const double uc = u[g.id(k, j, i)];
    const double f1l = D / dx * (u[g.id(k, j, i - 1)] - uc);
    const double f1r = D / dx * (uc - u[g.id(k, j, i + 1)]);
    const double f2l = D * (u[g.id(k, j - 1, i)] - uc) / dx;
    const double f2r = D * (uc - u[g.id(k, j + 1, i)]) / dx;
    const double f3l = D * (u[g.id(k - 1, j, i)] - uc) / dx;
    const double f3r = D * (uc - u[g.id(k + 1, j, i)]) / dx;
    double out = -p.alpha * uc;
    out += (f1l - f1r) / dx;
    out += (f2l - f2r) / dx;
    out += (f3l - f3r) / dx;
    return out;
  }
  void Ax(GmgLevel &g, const std::vector<double> &u, std::vector<double> &out) const {
    for (int k = 0; k < g.n; ++k)
      for (int j = 0; j < g.n; ++j)
        for (int i = 0; i < g.n; ++i) out[g.id(k, j, i)] = Ax_cell(g, u, k, j, i);
  }
  // poisson_equation.hpp:59-102
  double diag(const GmgLevel &g) const {
    const double D = p.D, dx = g.dx;
    double d = -(D + D) / (dx * dx) - p.alpha;
    d -= (D + D) / (dx * dx);
    d -= (D + D) / (dx * dx);
    return d;
  }
  // mg_solver.hpp:222-297 with robust::ratio (robust.hpp:58-62)
  void jacobi(GmgLevel &g, double w) {
    const double dg = diag(g);
    const double small = 10 * std::numeric_limits<double>::min();
    const double den = dg + (dg >= 0 ? 1.0 : -1.0) * small;
    for (int64_t c = 0; c < g.size(); ++c) {
      const double off = g.temp[c] - dg * g.u[c];
      const double val = g.rhs[c] - off;
      g.temp[c] = w * (val / den) + (1.0 - w) * g.u[c];
    }
  }
  // mg_solver.hpp:312-345 (3D weights)
  void smooth(GmgLevel &g, int stages) {
    static const double m1[3] = {1.0, 0.0, 0.0};
    static const double m2[3] = {1.7319, 0.5695, 0.0};
    static const double m3[3] = {2.2473, 0.8571, 0.5296};
    if (stages == 0) return;
    g.temp = g.u;
    for (int s = 0; s < stages; ++s) {
      const double w = p.jacobi ? p.weight : (p.smoother_stages == 1 ? m1[s] : (p.smoother_stages == 2 ? m2[s] : m3[s]));
      Ax(g, g.u, g.temp);
      jacobi(g, w);
      g.u = g.temp;
    }
  }
  // RestrictAverage (pr_ops.hpp:105-164), uniform volumes
  void restrict_into(const GmgLevel &f, const std::vector<double> &fine, const GmgLevel &c,
                     std::vector<double> &coarse) const {
    const double vol = f.dx * f.dx * f.dx;
    for (int ck = 0; ck < c.n; ++ck)
      for (int cj = 0; cj < c.n; ++cj)
        for (int ci = 0; ci < c.n; ++ci) {
          double t[2][2][2], v[2][2][2];
          for (int ok = 0; ok < 2; ++ok)
            for (int oj = 0; oj < 2; ++oj)
              for (int oi = 0; oi < 2; ++oi) {
                v[ok][oj][oi] = vol;
                t[ok][oj][oi] = vol * fine[f.id(2 * ck + ok, 2 * cj + oj, 2 * ci + oi)];
              }
          const double tv = ((v[0][0][0] + v[0][1][0]) + (v[0][0][1] + v[0][1][1])) +
                            ((v[1][0][0] + v[1][1][0]) + (v[1][0][1] + v[1][1][1]));
          coarse[c.id(ck, cj, ci)] = (((t[0][0][0] + t[0][1][0]) + (t[0][0][1] + t[0][1][1])) +
                                      ((t[1][0][0] + t[1][1][0]) + (t[1][0][1] + t[1][1][1]))) /
                                     tv;
        }
  }
  // ProlongateSharedLinear (pr_ops.hpp:166-285, use_minmod_slope = false)
  void prolong_into(const GmgLevel &c, const std::vector<double> &coarse, const GmgLevel &f,
                    std::vector<double> &fine) const {
    for (int k = 0; k < c.n; ++k)
      for (int j = 0; j < c.n; ++j)
        for (int i = 0; i < c.n; ++i) {
          const double fc = coarse[c.id(k, j, i)];
          const int ci[3] = {i, j, k};
          double gm[3], gp[3], dfm[3], dfp[3];
          for (int d = 0; d < 3; ++d) {
            auto xcc = [&](int idx) { return c.xmin + (idx + 0.5) * c.dx; };
            auto xfc = [&](int idx) { return f.xmin + (idx + 0.5) * f.dx; };
            const double xm = xcc(ci[d] - 1), xc = xcc(ci[d]), xp = xcc(ci[d] + 1);
            const double dxm = xc - xm, dxp = xp - xc;
            dfm[d] = xc - xfc(2 * ci[d]);
            dfp[d] = xfc(2 * ci[d] + 1) - xc;
            const int dk = d == 2, dj = d == 1, di = d == 0;
            const double nm = coarse[c.id(k - dk, j - dj, i - di)];
            const double np = coarse[c.id(k + dk, j + dj, i + di)];
            gm[d] = (fc - nm) / dxm;
            gp[d] = (np - fc) / dxp;
          }
          const int fi = 2 * i, fj = 2 * j, fk = 2 * k;
          auto F = [&](int ok, int oj, int oi) -> double & { return fine[f.id(fk + ok, fj + oj, fi + oi)]; };
          F(0, 0, 0) = fc - (gm[0] * dfm[0] + gm[1] * dfm[1] + gm[2] * dfm[2]);
          F(0, 0, 1) = fc + (gp[0] * dfp[0] - gm[1] * dfm[1] - gm[2] * dfm[2]);
          F(0, 1, 0) = fc - (gm[0] * dfm[0] - gp[1] * dfp[1] + gm[2] * dfm[2]);
          F(0, 1, 1) = fc + (gp[0] * dfp[0] + gp[1] * dfp[1] - gm[2] * dfm[2]);
          F(1, 0, 0) = fc - (gm[0] * dfm[0] + gm[1] * dfm[1] - gp[2] * dfp[2]);
          F(1, 0, 1) = fc + (gp[0] * dfp[0] - gm[1] * dfm[1] + gp[2] * dfp[2]);
          F(1, 1, 0) = fc - (gm[0] * dfm[0] - gp[1] * dfp[1] - gp[2] * dfp[2]);
          F(1, 1, 1) = fc + (gp[0] * dfp[0] + gp[1] * dfp[1] + gp[2] * dfp[2]);
        }
  }

  // One V-cycle (mg_solver.hpp:375-520 with do_FAS = true)
  void vcycle() {
    const int nl = (int)lv.size();
    const int pre = p.smoother_stages, post = p.smoother_stages;
    // down: finest (index 0) to coarsest (index nl-1)
    for (int l = 0; l < nl; ++l) {
      GmgLevel &g = lv[l];
      if (l > 0) {
        GmgLevel &f = lv[l - 1];
        restrict_into(f, f.u, g, g.u);
        restrict_into(f, f.res, g, g.res);
        g.u0 = g.u;
        Ax(g, g.u, g.temp);
        for (int64_t c = 0; c < g.size(); ++c) g.rhs[c] = 1.0 * g.temp[c] + 1.0 * g.res[c];
      } else {
        g.u0 = g.u;
      }
      smooth(g, pre);
      if (l < nl - 1) {
        Ax(g, g.u, g.temp);
        for (int64_t c = 0; c < g.size(); ++c) g.res[c] = 1.0 * g.rhs[c] + -1.0 * g.temp[c];
      } else {
        for (int s = 0; s < p.coarse_sweeps; ++s) smooth(g, pre);
        g.res = g.u;
        if (l > 0)
          for (int64_t c = 0; c < g.size(); ++c) g.res[c] = 1.0 * g.u[c] + -1.0 * g.u0[c];
      }
    }
    // up
    for (int l = nl - 2; l >= 0; --l) {
      GmgLevel &g = lv[l], &c = lv[l + 1];
      prolong_into(c, c.res, g, g.res);
      for (int64_t q = 0; q < g.size(); ++q) g.u[q] = 1.0 * g.u[q] + 1.0 * g.res[q];
      smooth(g, post);
      if (l > 0)
        for (int64_t q = 0; q < g.size(); ++q) g.res[q] = 1.0 * g.u[q] + -1.0 * g.u0[q];
    }
  }

  // u <- M b: one V-cycle from u = 0 with right-hand side b on the finest level
  // (MGSolver::AddLinearOperatorTasks, mg_solver.hpp:163-186, as BiCGSTAB uses it)
  void precondition(const std::vector<double> &b, std::vector<double> &out) {
    GmgLevel &g = lv[0];
    g.rhs = b;
    std::fill(g.u.begin(), g.u.end(), 0.0);
    vcycle();
    out = g.u;
  }

  static double dot(const std::vector<double> &a, const std::vector<double> &b) {
    double s = 0.0, c = 0.0;  // compensated: the accurate value
    for (size_t q = 0; q < a.size(); ++q) {
      const double term = a[q] * b[q], t = s + term;
      c += std::fabs(s) >= std::fabs(term) ? (s - t) + term : (term - t) + s;
      s = t;
    }
    return s + c;
  }

  // Right-preconditioned BiCGSTAB (bicgstab_solver.hpp:116-315): x0 = 0, r = p =
  // rhat0 = rhs; stops when sqrt((r,r)/N) < tol, tol = rtol * sqrt((rhs,rhs)/N) if
  // relative. Returns the iterations run; x holds the solution.
  int bicgstab(const std::vector<double> &rhs, std::vector<double> &x, bool precondition_on, double rtol,
               bool relative, int max_iters, double &rms_out) {
    GmgLevel &g = lv[0];
    const size_t n = rhs.size();
    const double N = (double)n;
    std::vector<double> r = rhs, p = rhs, rhat0 = rhs, v(n), h(n), s(n), t(n), u(n);
    x.assign(n, 0.0);
    double rhat0r = dot(rhat0, r);
    const double tol = relative ? rtol * std::sqrt(dot(rhs, rhs) / N) : rtol;
    int it = 0;
    rms_out = 0.0;
    for (it = 0; it < max_iters; ++it) {
      const double rhat0r_old = rhat0r;
      if (precondition_on) precondition(p, u);
      else u = p;
      Ax(g, u, v);
      const double rhat0v = dot(rhat0, v);
      const double alpha = rhat0r_old / rhat0v;
      for (size_t q = 0; q < n; ++q) {
        h[q] = 1.0 * x[q] + alpha * u[q];
        s[q] = 1.0 * r[q] + -alpha * v[q];
      }
      if (precondition_on) precondition(s, u);
      else u = s;
      Ax(g, u, t);
      const double ts = dot(t, s), tt = dot(t, t);
      const double omega = ts / tt;
      for (size_t q = 0; q < n; ++q) {
        x[q] = 1.0 * h[q] + omega * u[q];
        r[q] = 1.0 * s[q] + -omega * t[q];
      }
      const double res = dot(r, r);
      rhat0r = dot(rhat0, r);
      const double beta = rhat0r / rhat0r_old * alpha / omega;
      for (size_t q = 0; q < n; ++q) {
        p[q] = 1.0 * p[q] + -omega * v[q];
        p[q] = 1.0 * r[q] + beta * p[q];
      }
      rms_out = std::sqrt(res / N);
      if (rms_out < tol) return it + 1;
    }
    return it;
  }

  // residual rhs - A u on the finest level; returns sum of squares (fixed order)
  double residual() {
    GmgLevel &g = lv[0];
    Ax(g, g.u, g.res);
    double s = 0.0;
    for (int64_t c = 0; c < g.size(); ++c) {
      g.res[c] = 1.0 * g.rhs[c] + -1.0 * g.res[c];
      s += g.res[c] * g.res[c];
    }
    return s;
  }
};

}  // namespace oracle
