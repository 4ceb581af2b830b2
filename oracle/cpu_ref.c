/*
 * C/OpenMP restatement of the DNS-aided LES hot path -- TEST INFRASTRUCTURE
 * ONLY: the timed CPU baseline of bench.py and a second oracle for the tests;
 * never linked into or called by the product library.
 *
 * It restates, in float64 on the host cores, the same algorithm as
 * oracle/ns.py (which cites the reference line by line):
 *   stress / tensordivergence!     src/N.jl:94-160
 *   divergence! / pressuregradient! src/N.jl:222-254
 *   project! (FFT Poisson)         src/N.jl:256-307 (own radix-2/3/4 FFT;
 *                                  FFTW is not installed)
 *   propose_timestep               src/N.jl:348-356
 *   randomfield / peak_profile     src/N.jl:366-476 (project's counter RNG)
 *   lazyfilter / lazycoarsegrain   src/N.jl:639-698 (+ even-ratio extension)
 *   dnsaid_project loop            src/N.jl:1239-1332 with RK4 stages
 *                                  (tableau of src/Burgers.jl:120-142)
 * Layout: x fastest, component slowest (src/N.jl:29, :45).
 */
#include <complex.h>
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef double complex cplx;

/* ------------------------------------------------------------------ FFT -- */
typedef struct {
  int L, npass, radix[16];
  cplx* tw; /* W_L^m, m < L */
} plan1d;

static void plan_init(plan1d* p, int L) {
  p->L = L;
  int m = L, a = 0, b = 0, np = 0;
  while (m % 2 == 0) { m /= 2; ++a; }
  while (m % 3 == 0) { m /= 3; ++b; }
  while (a >= 2) { p->radix[np++] = 4; a -= 2; }
  if (a == 1) p->radix[np++] = 2;
  while (b-- > 0) p->radix[np++] = 3;
  p->npass = np;
  p->tw = malloc(sizeof(cplx) * (L > 0 ? L : 1));
  for (int k = 0; k < L; ++k) {
    long double ang = -2.0L * 3.141592653589793238462643383279502884L * k / L;
    p->tw[k] = (double)cosl(ang) + I * (double)sinl(ang);
  }
}
static void plan_free(plan1d* p) { free(p->tw); }

/* Stockham autosort transform of one line; sign -1 forward, +1 inverse
 * (unnormalised).  `x` holds the input and receives the output; `y` is
 * scratch of the same length. */
static void fft1d(const plan1d* p, cplx* x, cplx* y, int inv) {
  const int L = p->L;
  int Ns = 1;
  cplx* src = x;
  cplx* dst = y;
  for (int q = 0; q < p->npass; ++q) {
    const int R = p->radix[q];
    const int nb = L / R;
    for (int j = 0; j < nb; ++j) {
      int k = j % Ns;
      cplx v[4];
      for (int r = 0; r < R; ++r) {
        cplx w = p->tw[(r * k * (L / (Ns * R))) % L];
        if (inv) w = conj(w);
        v[r] = src[j + r * nb] * (Ns > 1 ? w : 1.0);
      }
      cplx o[4];
      if (R == 2) {
        o[0] = v[0] + v[1];
        o[1] = v[0] - v[1];
      } else if (R == 4) {
        cplx t0 = v[0] + v[2], t1 = v[0] - v[2], t2 = v[1] + v[3], t3 = v[1] - v[3];
        t3 = inv ? I * t3 : -I * t3;
        o[0] = t0 + t2;
        o[2] = t0 - t2;
        o[1] = t1 + t3;
        o[3] = t1 - t3;
      } else {
        const double s3 = 0.86602540378443864676;
        cplx t1 = v[1] + v[2];
        cplx t2 = v[0] - 0.5 * t1;
        cplx t3 = (inv ? I : -I) * s3 * (v[1] - v[2]);
        o[0] = v[0] + t1;
        o[1] = t2 + t3;
        o[2] = t2 - t3;
      }
      int base = (j / Ns) * Ns * R + k;
      for (int r = 0; r < R; ++r) dst[base + r * Ns] = o[r];
    }
    cplx* t = src;
    src = dst;
    dst = t;
    Ns *= R;
  }
  if (src != x) memcpy(x, src, sizeof(cplx) * L);
}

typedef struct {
  int n, nkx;
  double h;
  plan1d pn, ph;
  double* s2; /* sin^2(pi k/n) */
  cplx* spec; /* [n][n][nkx] */
} poisson;

static void poisson_init(poisson* ps, int n, double l) {
  ps->n = n;
  ps->nkx = n / 2 + 1;
  ps->h = l / n;
  plan_init(&ps->pn, n);
  plan_init(&ps->ph, n / 2);
  ps->s2 = malloc(sizeof(double) * n);
  for (int k = 0; k < n; ++k) {
    long double s = sinl(3.141592653589793238462643383279502884L * k / n);
    ps->s2[k] = (double)(s * s);
  }
  ps->spec = malloc(sizeof(cplx) * (size_t)n * n * ps->nkx);
}
static void poisson_free(poisson* ps) {
  plan_free(&ps->pn);
  plan_free(&ps->ph);
  free(ps->s2);
  free(ps->spec);
}

/* real rows -> half spectrum along x (packing trick), then y and z */
static void fft3_forward(poisson* ps, const double* d) {
  const int n = ps->n, N2 = n / 2, nkx = ps->nkx;
  const long nn = (long)n * n;
#pragma omp parallel
  {
    cplx* z = malloc(sizeof(cplx) * n);
    cplx* s = malloc(sizeof(cplx) * n);
#pragma omp for schedule(static)
    for (long row = 0; row < nn; ++row) {
      const double* x = d + row * n;
      for (int m = 0; m < N2; ++m) z[m] = x[2 * m] + I * x[2 * m + 1];
      fft1d(&ps->ph, z, s, 0);
      cplx* out = ps->spec + row * nkx;
      for (int k = 0; k <= N2; ++k) {
        cplx zk = z[k == N2 ? 0 : k];
        cplx zc = conj(z[k == 0 ? 0 : N2 - k]);
        cplx w = ps->pn.tw[k];
        out[k] = 0.5 * (zk + zc) - 0.5 * I * w * (zk - zc);
      }
    }
    free(z);
    free(s);
  }
  /* y then z, gathering blocks of 8 kx columns */
  for (int pass = 0; pass < 2; ++pass) {
    const long es = pass == 0 ? nkx : (long)n * nkx;
    const long os = pass == 0 ? (long)n * nkx : nkx;
    const int nblk = (nkx + 7) / 8;
#pragma omp parallel
    {
      cplx* buf = malloc(sizeof(cplx) * 8 * n);
      cplx* s = malloc(sizeof(cplx) * n);
#pragma omp for schedule(static)
      for (long t = 0; t < (long)n * nblk; ++t) {
        long o = t / nblk;
        int kx0 = (int)(t % nblk) * 8;
        int w = nkx - kx0 < 8 ? nkx - kx0 : 8;
        cplx* base = ps->spec + o * os + kx0;
        for (int e = 0; e < n; ++e)
          for (int l = 0; l < w; ++l) buf[l * n + e] = base[e * es + l];
        for (int l = 0; l < w; ++l) fft1d(&ps->pn, buf + l * n, s, 0);
        for (int e = 0; e < n; ++e)
          for (int l = 0; l < w; ++l) base[e * es + l] = buf[l * n + e];
      }
      free(buf);
      free(s);
    }
  }
}

/* inverse: z, y, then half spectrum -> real rows (unnormalised) */
static void fft3_inverse(poisson* ps, double* out_real) {
  const int n = ps->n, N2 = n / 2, nkx = ps->nkx;
  const long nn = (long)n * n;
  for (int pass = 1; pass >= 0; --pass) {
    const long es = pass == 0 ? nkx : (long)n * nkx;
    const long os = pass == 0 ? (long)n * nkx : nkx;
    const int nblk = (nkx + 7) / 8;
#pragma omp parallel
    {
      cplx* buf = malloc(sizeof(cplx) * 8 * n);
      cplx* s = malloc(sizeof(cplx) * n);
#pragma omp for schedule(static)
      for (long t = 0; t < (long)n * nblk; ++t) {
        long o = t / nblk;
        int kx0 = (int)(t % nblk) * 8;
        int w = nkx - kx0 < 8 ? nkx - kx0 : 8;
        cplx* base = ps->spec + o * os + kx0;
        for (int e = 0; e < n; ++e)
          for (int l = 0; l < w; ++l) buf[l * n + e] = base[e * es + l];
        for (int l = 0; l < w; ++l) fft1d(&ps->pn, buf + l * n, s, 1);
        for (int e = 0; e < n; ++e)
          for (int l = 0; l < w; ++l) base[e * es + l] = buf[l * n + e];
      }
      free(buf);
      free(s);
    }
  }
#pragma omp parallel
  {
    cplx* z = malloc(sizeof(cplx) * n);
    cplx* s = malloc(sizeof(cplx) * n);
#pragma omp for schedule(static)
    for (long row = 0; row < nn; ++row) {
      const cplx* X = ps->spec + row * nkx;
      for (int k = 0; k < N2; ++k) {
        cplx xa = X[k], xb = conj(X[N2 - k]);
        z[k] = (xa + xb) + I * conj(ps->pn.tw[k]) * (xa - xb);
      }
      fft1d(&ps->ph, z, s, 1);
      double* x = out_real + row * n;
      for (int m = 0; m < N2; ++m) {
        x[2 * m] = creal(z[m]);
        x[2 * m + 1] = cimag(z[m]);
      }
    }
    free(z);
    free(s);
  }
}

static inline long idx3(int n, int x, int y, int z) { return ((long)z * n + y) * n + x; }
static inline int up(int i, int n) { return i + 1 == n ? 0 : i + 1; }
static inline int dn(int i, int n) { return i == 0 ? n - 1 : i - 1; }

/* d = div u; p = L^-1 d (mean 0); u -= grad p.  p is scratch (n^3). */
static void project(poisson* ps, double* u, double* p) {
  const int n = ps->n;
  const long N = (long)n * n * n;
  const double h = ps->h;
#pragma omp parallel for schedule(static)
  for (int z = 0; z < n; ++z)
    for (int y = 0; y < n; ++y)
      for (int x = 0; x < n; ++x) {
        long g = idx3(n, x, y, z);
        p[g] = (u[g] - u[idx3(n, dn(x, n), y, z)]) / h + (u[N + g] - u[N + idx3(n, x, dn(y, n), z)]) / h +
               (u[2 * N + g] - u[2 * N + idx3(n, x, y, dn(z, n))]) / h;
      }
  fft3_forward(ps, p);
  const int nkx = ps->nkx;
  const double coef = -h * h / (4.0 * (double)N);
#pragma omp parallel for schedule(static)
  for (int kz = 0; kz < n; ++kz)
    for (int ky = 0; ky < n; ++ky)
      for (int kx = 0; kx < nkx; ++kx) {
        double den = ps->s2[kx] + ps->s2[ky] + ps->s2[kz];
        double f = (kx == 0 && ky == 0 && kz == 0) ? 0.0 : coef / den;
        ps->spec[((long)kz * n + ky) * nkx + kx] *= f;
      }
  fft3_inverse(ps, p);
#pragma omp parallel for schedule(static)
  for (int z = 0; z < n; ++z)
    for (int y = 0; y < n; ++y)
      for (int x = 0; x < n; ++x) {
        long g = idx3(n, x, y, z);
        double pc = p[g];
        u[g] -= (p[idx3(n, up(x, n), y, z)] - pc) / h;
        u[N + g] -= (p[idx3(n, x, up(y, n), z)] - pc) / h;
        u[2 * N + g] -= (p[idx3(n, x, y, up(z, n))] - pc) / h;
      }
}

/* ---------------------------------------------------------------- RHS -- */
static inline double sig(const double* u, long N, int n, double h, double visc, int i, int j, int x, int y, int z) {
  int c[3] = {x, y, z};
  int off = i != j;
  int a[3] = {c[0], c[1], c[2]}, b[3] = {c[0], c[1], c[2]};
  a[j] = (a[j] + off) % n;
  b[j] = (b[j] + off - 1 + n) % n;
  double uir = u[i * N + idx3(n, a[0], a[1], a[2])], uil = u[i * N + idx3(n, b[0], b[1], b[2])];
  int e[3] = {c[0], c[1], c[2]}, f[3] = {c[0], c[1], c[2]};
  e[i] = (e[i] + off) % n;
  f[i] = (f[i] + off - 1 + n) % n;
  double ujr = u[j * N + idx3(n, e[0], e[1], e[2])], ujl = u[j * N + idx3(n, f[0], f[1], f[2])];
  return (uir + uil) / 2 * ((ujr + ujl) / 2) - visc * ((uir - uil) / h + (ujr - ujl) / h);
}

/* du = -div sigma(u) (src/N.jl:120-160) */
static void rhs(int n, double h, double visc, const double* u, double* du) {
  const long N = (long)n * n * n;
#pragma omp parallel for schedule(static)
  for (int z = 0; z < n; ++z)
    for (int y = 0; y < n; ++y)
      for (int x = 0; x < n; ++x) {
        long g = idx3(n, x, y, z);
        int xm = dn(x, n), ym = dn(y, n), zm = dn(z, n), xp = up(x, n), yp = up(y, n), zp = up(z, n);
        double s12 = sig(u, N, n, h, visc, 0, 1, x, y, z), s23 = sig(u, N, n, h, visc, 1, 2, x, y, z);
        double s31 = sig(u, N, n, h, visc, 2, 0, x, y, z);
        du[g] = -(sig(u, N, n, h, visc, 0, 0, xp, y, z) - sig(u, N, n, h, visc, 0, 0, x, y, z)) / h -
                (s12 - sig(u, N, n, h, visc, 0, 1, x, ym, z)) / h - (s31 - sig(u, N, n, h, visc, 2, 0, x, y, zm)) / h;
        du[N + g] = -(s12 - sig(u, N, n, h, visc, 0, 1, xm, y, z)) / h -
                    (sig(u, N, n, h, visc, 1, 1, x, yp, z) - sig(u, N, n, h, visc, 1, 1, x, y, z)) / h -
                    (s23 - sig(u, N, n, h, visc, 1, 2, x, y, zm)) / h;
        du[2 * N + g] = -(s31 - sig(u, N, n, h, visc, 2, 0, xm, y, z)) / h -
                        (s23 - sig(u, N, n, h, visc, 1, 2, x, ym, z)) / h -
                        (sig(u, N, n, h, visc, 2, 2, x, y, zp) - sig(u, N, n, h, visc, 2, 2, x, y, z)) / h;
      }
}

/* ------------------------------------------------------------- filters -- */
typedef struct {
  int cnt, off[64];
  double w[64];
} taps1;

static taps1 axis_taps(int c, int stag, int point) {
  taps1 t;
  int a = c / 2;
  t.cnt = 0;
  if (stag) {
    int base = c - 1;
    if (point) { t.off[0] = base; t.w[0] = 1; t.cnt = 1; }
    else {
      for (int k = -a; k <= a; ++k) { t.off[t.cnt] = base + k; t.w[t.cnt++] = 1.0 / c; }
      if (c % 2 == 0) { t.w[0] = 0.5 / c; t.w[t.cnt - 1] = 0.5 / c; }
    }
  } else {
    if (point) {
      if (c % 2) { t.off[0] = a; t.w[0] = 1; t.cnt = 1; }
      else { t.off[0] = a - 1; t.off[1] = a; t.w[0] = t.w[1] = 0.5; t.cnt = 2; }
    } else {
      for (int k = 0; k < c; ++k) { t.off[t.cnt] = k; t.w[t.cnt++] = 1.0 / c; }
    }
  }
  return t;
}

/* ubar_i = filter of u_i (volume: box/trapezoid on all axes; face: point
 * sample along i), sampled at LES faces (src/N.jl:655-698, 1228-1237) */
static void filter_vec(int n, int c, int face, const double* u, double* ub) {
  const long N = (long)n * n * n;
  const int m = n / c;
  const long M = (long)m * m * m;
  for (int i = 0; i < 3; ++i) {
    taps1 t[3];
    for (int d = 0; d < 3; ++d) t[d] = axis_taps(c, d == i, face && d == i);
    const double* f = u + i * N;
#pragma omp parallel for schedule(static)
    for (int iz = 0; iz < m; ++iz)
      for (int iy = 0; iy < m; ++iy)
        for (int ix = 0; ix < m; ++ix) {
          double acc = 0;
          for (int tz = 0; tz < t[2].cnt; ++tz) {
            int z = ((c * iz + t[2].off[tz]) % n + n) % n;
            double az = 0;
            for (int ty = 0; ty < t[1].cnt; ++ty) {
              int y = ((c * iy + t[1].off[ty]) % n + n) % n;
              double ay = 0;
              for (int tx = 0; tx < t[0].cnt; ++tx) {
                int x = ((c * ix + t[0].off[tx]) % n + n) % n;
                ay += t[0].w[tx] * f[idx3(n, x, y, z)];
              }
              az += t[1].w[ty] * ay;
            }
            acc += t[2].w[tz] * az;
          }
          ub[i * M + idx3(m, ix, iy, iz)] = acc;
        }
  }
}

/* ----------------------------------------------------------------- case -- */
typedef struct {
  int c, face, m;
  long M;
  poisson ps;
  double *ub, *mcl, *rtmp, *pscr;
  double *ve0, *ves, *vefin, *ke;
  double *vn0, *vns, *vnfin, *kn;
} les_t;

typedef struct {
  int n;
  long N;
  double l, h, visc, cfl, dt, t;
  poisson ps;
  double *u0, *us, *ufin, *rhs, *p;
  int nles;
  les_t les[4];
} cref;

int cref_threads(void) { return omp_get_max_threads(); }

static double* alloc0(long cnt) { return calloc((size_t)cnt, sizeof(double)); }

cref* cref_create(int n, double l, double visc, double cfl, int nles, const int* ratio, const int* kind) {
  cref* cs = calloc(1, sizeof(cref));
  cs->n = n;
  cs->N = (long)n * n * n;
  cs->l = l;
  cs->h = l / n;
  cs->visc = visc;
  cs->cfl = cfl;
  poisson_init(&cs->ps, n, l);
  cs->u0 = alloc0(3 * cs->N);
  cs->us = alloc0(3 * cs->N);
  cs->ufin = alloc0(3 * cs->N);
  cs->rhs = alloc0(3 * cs->N);
  cs->p = alloc0(cs->N);
  cs->nles = nles;
  for (int i = 0; i < nles; ++i) {
    les_t* L = &cs->les[i];
    L->c = ratio[i];
    L->face = kind[i];
    L->m = n / L->c;
    L->M = (long)L->m * L->m * L->m;
    poisson_init(&L->ps, L->m, l);
    L->ub = alloc0(3 * L->M); L->mcl = alloc0(3 * L->M); L->rtmp = alloc0(3 * L->M); L->pscr = alloc0(L->M);
    L->ve0 = alloc0(3 * L->M); L->ves = alloc0(3 * L->M); L->vefin = alloc0(3 * L->M); L->ke = alloc0(3 * L->M);
    L->vn0 = alloc0(3 * L->M); L->vns = alloc0(3 * L->M); L->vnfin = alloc0(3 * L->M); L->kn = alloc0(3 * L->M);
  }
  return cs;
}

void cref_destroy(cref* cs) {
  if (!cs) return;
  poisson_free(&cs->ps);
  free(cs->u0); free(cs->us); free(cs->ufin); free(cs->rhs); free(cs->p);
  for (int i = 0; i < cs->nles; ++i) {
    les_t* L = &cs->les[i];
    poisson_free(&L->ps);
    free(L->ub); free(L->mcl); free(L->rtmp); free(L->pscr);
    free(L->ve0); free(L->ves); free(L->vefin); free(L->ke);
    free(L->vn0); free(L->vns); free(L->vnfin); free(L->kn);
  }
  free(cs);
}

static void les_target(cref* cs, les_t* L, const double* src, double* out) {
  filter_vec(cs->n, L->c, L->face, src, out);
  if (!L->face) project(&L->ps, out, L->pscr);
}

static void reset_les(cref* cs) {
  for (int i = 0; i < cs->nles; ++i) {
    les_t* L = &cs->les[i];
    les_target(cs, L, cs->u0, L->ub);
    memcpy(L->ve0, L->ub, sizeof(double) * 3 * L->M);
    memcpy(L->vn0, L->ub, sizeof(double) * 3 * L->M);
  }
  cs->t = 0;
}

int cref_set_velocity(cref* cs, const double* u) {
  memcpy(cs->u0, u, sizeof(double) * 3 * cs->N);
  reset_les(cs);
  return 0;
}
int cref_get_velocity(cref* cs, double* u) {
  memcpy(u, cs->u0, sizeof(double) * 3 * cs->N);
  return 0;
}
int cref_get_les(cref* cs, int i, int which, double* out) {
  les_t* L = &cs->les[i];
  if (which == 0) { les_target(cs, L, cs->u0, L->ub); memcpy(out, L->ub, sizeof(double) * 3 * L->M); }
  else memcpy(out, which == 1 ? L->ve0 : L->vn0, sizeof(double) * 3 * L->M);
  return 0;
}
int cref_time(cref* cs, double* t, double* dt) { *t = cs->t; *dt = cs->dt; return 0; }

static uint64_t splitmix(uint64_t x) {
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

/* randomfield(peak_profile, ...) (src/N.jl:394-476) */
int cref_init_random(cref* cs, double kpeak, double energy, uint64_t seed) {
  const int n = cs->n, nkx = n / 2 + 1;
  const long N = cs->N;
  const uint64_t base = seed * 0x9E3779B97F4A7C15ull;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < 3 * N; ++i) {
    uint64_t z1 = splitmix(base + 2ull * (uint64_t)i), z2 = splitmix(base + 2ull * (uint64_t)i + 1ull);
    double u1 = ((double)(z1 >> 11) + 0.5) * 0x1.0p-53, u2 = ((double)(z2 >> 11) + 0.5) * 0x1.0p-53;
    cs->u0[i] = sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
  }
  project(&cs->ps, cs->u0, cs->p);
  const long S = (long)n * n * nkx;
  cplx* sp = malloc(sizeof(cplx) * 3 * S);
  for (int c = 0; c < 3; ++c) {
    fft3_forward(&cs->ps, cs->u0 + c * N);
    memcpy(sp + c * S, cs->ps.spec, sizeof(cplx) * S);
  }
  const int kdiag = (int)floor(sqrt(3.0) * (n / 2));
  double* esh = calloc(kdiag + 1, sizeof(double));
  double* fac = calloc(kdiag + 1, sizeof(double));
  int* shell = malloc(sizeof(int) * S);
  for (long g = 0; g < S; ++g) {
    long r = g / nkx;
    int kx = (int)(g % nkx), kz = (int)(r / n), ky = (int)(r % n);
    int a = ky <= (n - 1) / 2 ? ky : ky - n, b = kz <= (n - 1) / 2 ? kz : kz - n;
    long kk = (long)kx * kx + (long)a * a + (long)b * b;
    int s = (int)sqrt((double)kk);
    while ((long)s * s > kk) --s;
    while ((long)(s + 1) * (s + 1) <= kk) ++s;
    shell[g] = s;
    double e = 0;
    for (int c = 0; c < 3; ++c) {
      cplx v = sp[c * S + g] / (double)N;
      e += creal(v) * creal(v) + cimag(v) * cimag(v);
    }
    double w = (kx >= 1 && kx <= n / 2 - 1) ? 2.0 : 1.0;
    if (s <= kdiag) esh[s] += 0.5 * e * w;
  }
  double tot = 0;
  for (int k = 0; k <= kdiag; ++k) tot += pow(k, 4) * exp(-2 * (k / kpeak) * (k / kpeak));
  for (int k = 0; k <= kdiag; ++k) {
    double e0 = energy * pow(k, 4) * exp(-2 * (k / kpeak) * (k / kpeak)) / tot;
    fac[k] = esh[k] > 0 ? sqrt(e0 / esh[k]) : 1.0;
  }
  for (int c = 0; c < 3; ++c) {
    for (long g = 0; g < S; ++g) cs->ps.spec[g] = sp[c * S + g] * fac[shell[g]];
    fft3_inverse(&cs->ps, cs->u0 + c * N);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < N; ++i) cs->u0[c * N + i] /= (double)N;
  }
  free(sp); free(esh); free(fac); free(shell);
  project(&cs->ps, cs->u0, cs->p);
  reset_les(cs);
  return 0;
}

/* Smooth divergence-free field (u = sin 2pi y, v = sin 2pi z, w = sin 2pi x)
 * for timing samples, where the values do not matter but must stay normal
 * numbers. */
int cref_init_analytic(cref* cs) {
  const int n = cs->n;
  const long N = cs->N;
#pragma omp parallel for schedule(static)
  for (int z = 0; z < n; ++z)
    for (int y = 0; y < n; ++y)
      for (int x = 0; x < n; ++x) {
        long g = idx3(n, x, y, z);
        cs->u0[g] = sin(2 * M_PI * (y + 0.5) / n);
        cs->u0[N + g] = sin(2 * M_PI * (z + 0.5) / n);
        cs->u0[2 * N + g] = sin(2 * M_PI * (x + 0.5) / n);
      }
  reset_les(cs);
  return 0;
}

static void rk_combine(long cnt, double* k, const double* x0, double* xs, double* xfin, int s, double dt) {
  const double cf = (s == 0 || s == 3) ? dt / 6.0 : dt / 3.0, cst = s == 2 ? dt : 0.5 * dt;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < cnt; ++i) {
    if (s == 0) xfin[i] = x0[i] + cf * k[i];
    else xfin[i] += cf * k[i];
    if (s < 3) xs[i] = x0[i] + cst * k[i];
  }
}

static void propose_dt(cref* cs, double dt_fixed) {
  if (dt_fixed > 0) { cs->dt = dt_fixed; return; }
  double m = 0;
#pragma omp parallel for reduction(max : m) schedule(static)
  for (long i = 0; i < 3 * cs->N; ++i) m = fmax(m, fabs(cs->u0[i]));
  double a = cs->cfl * cs->h / m, b = cs->cfl * cs->h * cs->h / cs->visc / 6.0;
  cs->dt = a < b ? a : b;
}

static void do_stage(cref* cs, int s) {
  const double* src = s == 0 ? cs->u0 : cs->us;
  rhs(cs->n, cs->h, cs->visc, src, cs->rhs);
  for (int i = 0; i < cs->nles; ++i) les_target(cs, &cs->les[i], src, cs->les[i].ub);
  project(&cs->ps, cs->rhs, cs->p); /* rhs <- k */
  rk_combine(3 * cs->N, cs->rhs, cs->u0, cs->us, cs->ufin, s, cs->dt);
  for (int i = 0; i < cs->nles; ++i) {
    les_t* L = &cs->les[i];
    const double H = cs->l / L->m;
    filter_vec(cs->n, L->c, L->face, cs->rhs, L->mcl);
    rhs(L->m, H, cs->visc, L->ub, L->rtmp);
    for (long q = 0; q < 3 * L->M; ++q) L->mcl[q] -= L->rtmp[q];
    project(&L->ps, L->mcl, L->pscr);
    rhs(L->m, H, cs->visc, s == 0 ? L->ve0 : L->ves, L->ke);
    project(&L->ps, L->ke, L->pscr);
    for (long q = 0; q < 3 * L->M; ++q) L->ke[q] += L->mcl[q];
    rk_combine(3 * L->M, L->ke, L->ve0, L->ves, L->vefin, s, cs->dt);
    rhs(L->m, H, cs->visc, s == 0 ? L->vn0 : L->vns, L->kn);
    project(&L->ps, L->kn, L->pscr);
    rk_combine(3 * L->M, L->kn, L->vn0, L->vns, L->vnfin, s, cs->dt);
  }
}

static void swap_states(cref* cs) {
  double* t = cs->u0; cs->u0 = cs->ufin; cs->ufin = t;
  for (int i = 0; i < cs->nles; ++i) {
    les_t* L = &cs->les[i];
    t = L->ve0; L->ve0 = L->vefin; L->vefin = t;
    t = L->vn0; L->vn0 = L->vnfin; L->vnfin = t;
  }
}

int cref_step(cref* cs, int nsteps, double dt_fixed) {
  for (int it = 0; it < nsteps; ++it) {
    propose_dt(cs, dt_fixed);
    for (int s = 0; s < 4; ++s) do_stage(cs, s);
    swap_states(cs);
    cs->t += cs->dt;
  }
  return 0;
}

/* one stage in isolation (timing samples); stage 0 also proposes dt */
int cref_stage(cref* cs, int s) {
  if (s == 0) propose_dt(cs, 0.0);
  do_stage(cs, s);
  return 0;
}

/* ------------------------------------------------ standalone operators -- */
/* project!(u, poisson) (src/N.jl:256-307) on a caller-owned 3 x n^3 field,
 * in place; the pressure goes to p (n^3) when it is not NULL. */
int cref_project(int n, double l, double* u, double* p) {
  poisson ps;
  poisson_init(&ps, n, l);
  double* scr = p ? p : malloc(sizeof(double) * (size_t)n * n * n);
  if (!scr) { poisson_free(&ps); return 1; }
  project(&ps, u, scr);
  if (!p) free(scr);
  poisson_free(&ps);
  return 0;
}

/* du = tensordivergence(stresstensor(u, visc)) (src/N.jl:94-160) on caller
 * buffers (3 x n^3 each). */
int cref_rhs(int n, double l, double visc, const double* u, double* du) {
  rhs(n, l / n, visc, u, du);
  return 0;
}
