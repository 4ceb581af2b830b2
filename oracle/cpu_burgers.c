/*
 * C/OpenMP restatement of the reference's 1-D Burgers DNS-aided LES --
 * TEST INFRASTRUCTURE ONLY: the timed CPU baseline of bench.py's Burgers
 * workload and a second oracle for the tests; never linked into or called
 * by the product library.
 *
 * Same algorithm as oracle/burgers.py (which cites src/Burgers.jl line by
 * line): `stress` (:89-94), `δ_coll` (:87), `cfl` (:97-101), `lazyfilter`
 * and `lazycoarsegrain` (:164-180) and the `dns_aided_les` loop (:350-445)
 * with its four LES (no model, classic, classic+flux, classic+flux+div),
 * forward Euler, one time step per sample.  Samples run in parallel over
 * the host cores (the reference loops over them, :307).  Arithmetic keeps
 * the reference's divisions.  Layout: [sample][cell], x fastest.
 */
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

static inline int wrap(int i, int n) { i %= n; return i < 0 ? i + n : i; }

static inline double bstress(double ua, double ub, double visc, double h) {
  return -((ua + ub) * (ua + ub)) / 8 + visc * (ub - ua) / h;
}

/* Filter of `x` (period n) with kernel w[2R+1] at fine index j. */
static inline double filt(const double* x, int n, const double* w, int R, int j) {
  double s = 0.0;
  for (int r = -R; r <= R; ++r) s += w[r + R] * x[wrap(j + r, n)];
  return s;
}

/* Advance samples [0, ns) until t >= tstop or max_steps steps; v holds
 * [ns][4][nH] LES states (nomodel, class_m, class_p, swapfil) or NULL with
 * nH == 0 for the DNS alone. */
int cref_burgers_dnsaid(int nh, int ns, int nH, double l, double visc, const double* wl, int Rl, const double* wd,
                        int Rd, double tstop, double cfl_factor, int max_steps, double* u, double* v, double* t,
                        int* steps) {
  const double h = l / nh;
  const double H = nH > 0 ? l / nH : 0.0;
  const int comp = nH > 0 ? nh / nH : 1, a = comp / 2;
#pragma omp parallel
  {
    double* su = malloc(sizeof(double) * nh);
    double* du = malloc(sizeof(double) * nh);
    double* tm = malloc(sizeof(double) * 5 * (nH > 0 ? nH : 1));
    double* sg = malloc(sizeof(double) * (nH > 0 ? nH : 1));
#pragma omp for schedule(dynamic, 1)
    for (int s = 0; s < ns; ++s) {
      double* us = u + (long)s * nh;
      double tt = t[s];
      int done = 0;
      while (tt < tstop && done < max_steps) {
        double m = 0.0;
        for (int j = 0; j < nh; ++j) m = fmax(m, fabs(us[j]));
        double dt = cfl_factor * fmin(h / m, h * h / visc);
        dt = fmin(dt, tstop - tt);
        for (int j = 0; j < nh; ++j) su[j] = bstress(us[wrap(j - 1, nh)], us[j], visc, h);
        if (nH > 0) {
          double* fsu = tm; double* vsu = tm + nH; double* vu = tm + 2 * nH; double* sVU = tm + 3 * nH;
          double* svu = tm + 4 * nH;
          for (int I = 0; I < nH; ++I) {
            const int c = (I + 1) * comp - a - 1, f = (I + 1) * comp - 1;
            fsu[I] = filt(su, nh, wl, Rl, c);
            vsu[I] = filt(su, nh, wd, Rd, c);
            vu[I] = filt(us, nh, wd, Rd, f);
            sVU[I] = bstress(filt(us, nh, wd, Rd, c - 1), filt(us, nh, wd, Rd, c), visc, h);
          }
          for (int I = 0; I < nH; ++I) svu[I] = bstress(vu[wrap(I - 1, nH)], vu[I], visc, H);
          for (int k = 0; k < 4; ++k) {
            double* x = v + (long)s * 4 * nH + (long)k * nH;
            for (int I = 0; I < nH; ++I) {
              double si = bstress(x[wrap(I - 1, nH)], x[I], visc, H);
              if (k == 1) si = si + vsu[I] - sVU[I];
              if (k == 2) si = si + vsu[I] - svu[I];
              if (k == 3) si = si + fsu[I] - svu[I];
              sg[I] = si;
            }
            for (int I = 0; I < nH; ++I) x[I] += dt * ((sg[wrap(I + 1, nH)] - sg[I]) / H);
          }
        }
        for (int j = 0; j < nh; ++j) du[j] = (su[wrap(j + 1, nh)] - su[j]) / h;
        for (int j = 0; j < nh; ++j) us[j] += dt * du[j];
        tt += dt;
        ++done;
      }
      t[s] = tt;
      steps[s] += done;
    }
    free(su); free(du); free(tm); free(sg);
  }
  return 0;
}
