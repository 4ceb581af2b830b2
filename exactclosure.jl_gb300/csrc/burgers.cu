// Batched 1-D Burgers DNS-aided LES (the reference's `Burgers` module,
// src/Burgers.jl) on GB300.
//
// Design: one CTA owns one sample for the whole time loop.  The sample's DNS
// velocity and its stress live in shared memory with periodic ghost cells
// (2 x (nh + 2G) doubles, 219 KB at nh = 13500), so a DNS-aided step reads
// HBM not at all: every filter tap, the LES closure terms and the Euler or
// RK4 update come from shared memory, and only the small LES states and
// closure terms go through L2.  Samples advance with their own time step
// (src/Burgers.jl:307 loops over samples, each with its own `cfl`), so the
// CTAs never wait on each other; a CTA finishing one sample takes the next.
// Everything is FP64 like the reference, which makes the kernels FP64-pipe
// bound on GB300.
//
// Indexing: sample-major [ns][nh], x fastest (the reference's zeros(nh, ns)
// column-major matrices).  Fine index j (0-based) is the reference's j+1.
// Coarse cell I (0-based) reads the fine face (I+1)c - 1 and the fine centre
// (I+1)c - a - 1, a = c / 2 (`lazycoarsegrain`, src/Burgers.jl:174-180).
#include "internal.cuh"

#include <cmath>
#include <vector>

struct exc_burgers {
  int nh = 0, ns = 0;
  double l = 0, visc = 0, h = 0;
  cudaStream_t st = nullptr;
  double* u = nullptr;     // [ns][nh] current DNS velocity
  double* u0 = nullptr;    // [ns][nh] initial velocity (ustart)
  double* t = nullptr;     // [ns] time per sample
  int* steps = nullptr;    // [ns] steps taken per sample
  double* scr = nullptr;   // [2][ns][nh] RK4 uold/acc, Smagorinsky-fit filtered velocity
  // LES grid
  int nH = 0, comp = 0, a = 0, Rd = 0, Rl = 0, filter = 0;
  double H = 0, delta = 0, delta_ratio = 0;
  std::vector<double> wd_h, wl_h;
  double* wd = nullptr;    // double kernel, 2 Rd + 1
  double* wl = nullptr;    // LES kernel, 2 Rl + 1
  double* v = nullptr;     // [2][ns][4][nH] LES states, ping-pong
  double* tmp = nullptr;   // [ns][5][nH] closure terms
  double* smag = nullptr;  // [ns][nH] Smagorinsky LES
  double* tsm = nullptr;   // [ns]
  int* ssm = nullptr;      // [ns]
  bool les_on = false, smag_on = false;
  double* red = nullptr;   // [ns][8] per-sample partial sums
  double* sums = nullptr;  // [8]
  int* err = nullptr;
};

namespace exc {
namespace {

constexpr int BT = 512;        // threads per sample CTA
constexpr int NRED = 8;        // per-sample partial sums
constexpr double EPS64 = 2.220446049250313e-16;
// Steps one call may take per sample: keeps every launch finite even for a
// time step that is tiny but not collapsed.
constexpr int MAX_STEPS_PER_CALL = 1000000;

// `stress` (src/Burgers.jl:89-94) between faces ua = u[i-1], ub = u[i],
// vh = visc / h.  Divisions by the grid spacing are multiplications by its
// reciprocal throughout: an FP64 division costs about ten FP64 operations on
// GB300's FP64 pipe, and the reciprocal changes results by an ulp.
__device__ __forceinline__ double bstress(double ua, double ub, double vh) {
  const double s = ua + ub;
  return fma(-0.125 * s, s, vh * (ub - ua));
}

// Deterministic block reductions (fixed shuffle tree, warps in order).
__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (ln == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    double x = ln < nw ? sh[ln] : 0.0;
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (ln == 0) sh[32] = x;
  }
  __syncthreads();
  const double r = sh[32];
  __syncthreads();
  return r;
}

// Maximum that propagates NaN (Julia's `maximum` does; fmax would drop it).
__device__ __forceinline__ double nanmax(double m, double x) { return (x > m || x != x) ? x : m; }

__device__ __forceinline__ double block_max(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v = nanmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (ln == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    double x = ln < nw ? sh[ln] : 0.0;
    for (int o = 16; o > 0; o >>= 1) x = nanmax(x, __shfl_xor_sync(0xffffffffu, x, o));
    if (ln == 0) sh[32] = x;
  }
  __syncthreads();
  const double r = sh[32];
  __syncthreads();
  return r;
}

struct Geo {
  int nh, ns, G;       // fine size, samples, ghost width
  double h, visc;
  int nH, comp, a, Rd, Rl;
  double H;
  double ih, iH, vh, vH;  // 1/h, 1/H, visc/h, visc/H
};

// Shared-memory layout of a sample CTA: ue[np], se[np], wd[2Rd+1], wl[2Rl+1].
__host__ __device__ inline int padded(const Geo& g) { return g.nh + 2 * g.G; }
inline size_t sample_smem(const Geo& g) {
  return (size_t)(2 * padded(g) + 2 * g.Rd + 1 + 2 * g.Rl + 1) * sizeof(double);
}

__device__ void load_sample(const Geo& g, const double* __restrict__ us, double* ue) {
  const int np = padded(g);
  for (int p = threadIdx.x; p < np; p += blockDim.x) {
    int j = (p - g.G) % g.nh;
    if (j < 0) j += g.nh;
    ue[p] = us[j];
  }
}

__device__ void refresh_ghosts(const Geo& g, double* ue) {
  for (int p = threadIdx.x; p < g.G; p += blockDim.x) {
    ue[p] = ue[p + g.nh];
    ue[g.G + g.nh + p] = ue[g.G + p];
  }
}

__device__ void fill_stress(const Geo& g, const double* ue, double* se) {
  const int np = padded(g);
  for (int p = 1 + threadIdx.x; p < np; p += blockDim.x) se[p] = bstress(ue[p - 1], ue[p], g.vh);
}

// The filtered quantities of coarse cell I (src/Burgers.jl:397-412):
// fsu, vsu at the coarse centre, vu at the coarse face and sVU, the fine
// stress of the double-filtered velocity at the coarse centre.
struct Terms { double fsu, vsu, vu, sVU; };

__device__ __forceinline__ Terms coarse_terms(const Geo& g, int I, const double* ue, const double* se,
                                              const double* wd, const double* wl) {
  const int pc = g.G + (I + 1) * g.comp - g.a - 1;
  double vsu = 0.0, fsu = 0.0, vl = 0.0, vr = 0.0, vu = 0.0;
  for (int r = -g.Rd; r <= g.Rd; ++r) vsu = fma(wd[r + g.Rd], se[pc + r], vsu);
  for (int r = -g.Rl; r <= g.Rl; ++r) fsu = fma(wl[r + g.Rl], se[pc + r], fsu);
  double prev = ue[pc - 1 - g.Rd];
  for (int r = -g.Rd; r <= g.Rd; ++r) {
    const double x = ue[pc + r], w = wd[r + g.Rd];
    vl = fma(w, prev, vl);
    vr = fma(w, x, vr);
    prev = x;
  }
  const int pf = pc + g.a;
  for (int r = -g.Rd; r <= g.Rd; ++r) vu = fma(wd[r + g.Rd], ue[pf + r], vu);
  Terms t;
  t.fsu = fsu;
  t.vsu = vsu;
  t.vu = vu;
  t.sVU = bstress(vl, vr, g.vh);
  return t;
}

struct AdvanceArgs {
  Geo g;
  double cfl, tstop;
  int max_steps;
  double* u;
  double* t;
  int* steps;
  const double* wd;
  const double* wl;
  double* v0;    // [ns][4][nH] current LES states (result always lands here)
  double* v1;    // [ns][4][nH] ping-pong partner
  double* tmp;   // [ns][5][nH]
  double* uold;  // [ns][nh] (RK4)
  double* acc;   // [ns][nh] (RK4)
  int* err;
};

// Per-sample time step (src/Burgers.jl:97-101, :383-385); false = stop.
__device__ __forceinline__ bool sample_dt(const AdvanceArgs& A, double lmax, double tt, double* red, double& dt) {
  const Geo& g = A.g;
  const double m = block_max(lmax, red);
  const double dtc = A.cfl * fmin(g.h / m, g.h * g.h / g.visc);
  dt = fmin(dtc, A.tstop - tt);
  // A non-finite field, or a CFL step that collapsed, ends the sample with a
  // flag instead of a NaN time or an unbounded loop.
  if (!(m == m) || isinf(m) || !(dtc > 1e-12 * A.tstop)) {
    if (threadIdx.x == 0) atomicExch(A.err, 1);
    return false;
  }
  return true;
}

// `dns_aided_les` (src/Burgers.jl:350-445) when LES, else the DNS loop of
// `create_dns` (src/Burgers.jl:522-545) with `timestep!` or, when RK4,
// `rk4_timestep!` (src/Burgers.jl:112-142).
template <bool LES, bool RK4>
__global__ void __launch_bounds__(BT) advance_kernel(AdvanceArgs A) {
  extern __shared__ double smem[];
  __shared__ double red[40];
  const Geo g = A.g;
  const int np = padded(g);
  double* ue = smem;
  double* se = ue + np;
  double* wd = se + np;
  double* wl = wd + 2 * g.Rd + 1;
  if (LES) {
    for (int r = threadIdx.x; r < 2 * g.Rd + 1; r += blockDim.x) wd[r] = A.wd[r];
    for (int r = threadIdx.x; r < 2 * g.Rl + 1; r += blockDim.x) wl[r] = A.wl[r];
  }
  const int tid = threadIdx.x;
  const size_t vs = (size_t)4 * g.nH;
  for (int s = blockIdx.x; s < g.ns; s += gridDim.x) {
    double* us = A.u + (size_t)s * g.nh;
    load_sample(g, us, ue);
    double tt = A.t[s];
    int done = 0, par = 0;
    __syncthreads();
    // |u| maximum of this thread's cells, kept up to date by the updates.
    double lmax = 0.0;
    for (int j = tid; j < g.nh; j += blockDim.x) lmax = nanmax(lmax, fabs(ue[g.G + j]));
    while (tt < A.tstop && done < A.max_steps) {
      double dt;
      if (!sample_dt(A, lmax, tt, red, dt)) break;
      const double dth = dt * g.ih, dtH = dt * g.iH;
      lmax = 0.0;
      if (!RK4) {
        fill_stress(g, ue, se);
        __syncthreads();
        if (LES) {
          double* vc = (par ? A.v1 : A.v0) + s * vs;
          double* vn = (par ? A.v0 : A.v1) + s * vs;
          double* tm = A.tmp + (size_t)s * 5 * g.nH;
          for (int I = tid; I < g.nH; I += blockDim.x) {
            const Terms c = coarse_terms(g, I, ue, se, wd, wl);
            tm[I] = c.fsu;
            tm[g.nH + I] = c.vsu;
            tm[2 * g.nH + I] = c.vu;
            tm[3 * g.nH + I] = c.sVU;
          }
          __syncthreads();
          // LES steps: stress of each LES plus its correction
          // (src/Burgers.jl:414-430), forward Euler with the DNS time step.
          for (int i = tid; i < g.nH; i += blockDim.x) {
            const int im = i == 0 ? g.nH - 1 : i - 1, ip = i + 1 == g.nH ? 0 : i + 1;
            const double vum = tm[2 * g.nH + im], vui = tm[2 * g.nH + i], vup = tm[2 * g.nH + ip];
            const double svi = bstress(vum, vui, g.vH), svp = bstress(vui, vup, g.vH);
            const double fi = tm[i], fp = tm[ip];
            const double vsi = tm[g.nH + i], vsp = tm[g.nH + ip];
            const double Si = tm[3 * g.nH + i], Sp = tm[3 * g.nH + ip];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const double* x = vc + k * g.nH;
              const double xm = x[im], xi = x[i], xp = x[ip];
              double si = bstress(xm, xi, g.vH), sp = bstress(xi, xp, g.vH);
              if (k == 1) { si = (si + vsi) - Si; sp = (sp + vsp) - Sp; }    // classic
              if (k == 2) { si = (si + vsi) - svi; sp = (sp + vsp) - svp; }  // classic + flux
              if (k == 3) { si = (si + fi) - svi; sp = (sp + fp) - svp; }    // + div (exact)
              vn[k * g.nH + i] = fma(dtH, sp - si, xi);
            }
          }
          par ^= 1;
        }
        for (int j = tid; j < g.nh; j += blockDim.x) {
          const int p = g.G + j;
          const double x = fma(dth, se[p + 1] - se[p], ue[p]);
          ue[p] = x;
          lmax = nanmax(lmax, fabs(x));
        }
        __syncthreads();
        refresh_ghosts(g, ue);
        __syncthreads();
      } else {
        double* uo = A.uold + (size_t)s * g.nh;
        double* ac = A.acc + (size_t)s * g.nh;
        for (int q = 0; q < 4; ++q) {
          fill_stress(g, ue, se);
          __syncthreads();
          for (int j = tid; j < g.nh; j += blockDim.x) {
            const int p = g.G + j;
            const double k = (se[p + 1] - se[p]) * g.ih;
            if (q == 0) {
              const double x = ue[p];
              uo[j] = x;
              ac[j] = k;
              ue[p] = x + dt / 2 * k;
            } else if (q == 1) {
              ac[j] = ac[j] + 2 * k;
              ue[p] = uo[j] + dt / 2 * k;
            } else if (q == 2) {
              ac[j] = ac[j] + 2 * k;
              ue[p] = uo[j] + dt * k;
            } else {
              const double x = uo[j] + dt / 6 * (ac[j] + k);
              ue[p] = x;
              lmax = nanmax(lmax, fabs(x));
            }
          }
          __syncthreads();
          refresh_ghosts(g, ue);
          __syncthreads();
        }
      }
      tt += dt;
      ++done;
    }
    for (int j = tid; j < g.nh; j += blockDim.x) us[j] = ue[g.G + j];
    if (LES && par) {
      const double* src = A.v1 + s * vs;
      double* dst = A.v0 + s * vs;
      for (size_t i = tid; i < vs; i += blockDim.x) dst[i] = src[i];
    }
    if (tid == 0) {
      A.t[s] = tt;
      A.steps[s] += done;
    }
    __syncthreads();
  }
}

struct TermsArgs {
  Geo g;
  const double* u;
  const double* wd;
  const double* wl;
  double* terms;     // [ns][5][nH] fsu, vsu, vu, sVU, svu (or null)
  double* diss;      // [ns][3][nH] (or null)
  double* fine;      // [ns][nh] double-filtered DNS (or null)
  double* les_init;  // [ns][4][nH] filled with vu (or null)
  double* red;       // [ns][NRED]: fraction sums in 0..2 (or null)
};

// Closure terms and their analyses from the current DNS: `compute_fractions`
// (src/Burgers.jl:1022-1116), `compute_dissipation` (src/Burgers.jl:447-520),
// the filtered DNS `dns_ref_fil`/`dns_fil` (src/Burgers.jl:441-442) and the
// initial LES state (src/Burgers.jl:366-379).
__global__ void __launch_bounds__(BT) terms_kernel(TermsArgs A) {
  extern __shared__ double smem[];
  __shared__ double red[40];
  const Geo& g = A.g;
  const int np = padded(g);
  double* ue = smem;
  double* se = ue + np;
  double* wd = se + np;
  double* wl = wd + 2 * g.Rd + 1;
  for (int r = threadIdx.x; r < 2 * g.Rd + 1; r += blockDim.x) wd[r] = A.wd[r];
  for (int r = threadIdx.x; r < 2 * g.Rl + 1; r += blockDim.x) wl[r] = A.wl[r];
  for (int s = blockIdx.x; s < g.ns; s += gridDim.x) {
    load_sample(g, A.u + (size_t)s * g.nh, ue);
    __syncthreads();
    fill_stress(g, ue, se);
    __syncthreads();
    double* tm = A.terms ? A.terms + (size_t)s * 5 * g.nH : nullptr;
    // Terms at I and at I-1 (for svu and the dissipation's difference).
    double f0 = 0, f1 = 0, f2 = 0;
    for (int I = threadIdx.x; I < g.nH; I += blockDim.x) {
      const Terms c = coarse_terms(g, I, ue, se, wd, wl);
      const Terms cm = coarse_terms(g, I == 0 ? g.nH - 1 : I - 1, ue, se, wd, wl);
      const double svu = bstress(cm.vu, c.vu, g.vH);
      if (tm) {
        tm[I] = c.fsu;
        tm[g.nH + I] = c.vsu;
        tm[2 * g.nH + I] = c.vu;
        tm[3 * g.nH + I] = c.sVU;
        tm[4 * g.nH + I] = svu;
      }
      const double sc = c.vsu - c.sVU, sf = c.sVU - svu, sd = c.fsu - c.vsu;
      const double tot = fabs(sc) + fabs(sf) + fabs(sd) + EPS64;
      f0 += fabs(sc) / tot;
      f1 += fabs(sf) / tot;
      f2 += fabs(sd) / tot;
      if (A.diss) {
        double* d = A.diss + (size_t)s * 3 * g.nH;
        const double dv = (c.vu - cm.vu) * g.iH;
        d[I] = dv * (c.vsu - c.sVU);
        d[g.nH + I] = dv * (c.vsu - svu);
        d[2 * g.nH + I] = dv * (c.fsu - svu);
      }
      if (A.les_init) {
        double* v = A.les_init + (size_t)s * 4 * g.nH;
        for (int k = 0; k < 4; ++k) v[k * g.nH + I] = c.vu;
      }
    }
    if (A.fine) {
      double* fo = A.fine + (size_t)s * g.nh;
      for (int j = threadIdx.x; j < g.nh; j += blockDim.x) {
        double acc = 0.0;
        for (int r = -g.Rd; r <= g.Rd; ++r) acc = fma(wd[r + g.Rd], ue[g.G + j + r], acc);
        fo[j] = acc;
      }
    }
    if (A.red) {
      f0 = block_sum(f0, red);
      f1 = block_sum(f1, red);
      f2 = block_sum(f2, red);
      if (threadIdx.x == 0) {
        A.red[(size_t)s * NRED + 0] = f0 / g.nH;
        A.red[(size_t)s * NRED + 1] = f1 / g.nH;
        A.red[(size_t)s * NRED + 2] = f2 / g.nH;
      }
    }
    __syncthreads();
  }
}

// Per-sample squared norms for `compute_errors` (src/Burgers.jl:909-916):
// red[s][k] = sum (x_k - f)^2 for the four LES and the Smagorinsky LES,
// red[s][5] = sum f^2, f = dns_fil (terms slot 2).
__global__ void __launch_bounds__(BT) errors_kernel(int ns, int nH, const double* __restrict__ v,
                                                    const double* __restrict__ smag,
                                                    const double* __restrict__ terms, double* red) {
  __shared__ double sh[40];
  for (int s = blockIdx.x; s < ns; s += gridDim.x) {
    const double* f = terms + (size_t)s * 5 * nH + 2 * nH;
    double e[5] = {0, 0, 0, 0, 0}, ff = 0;
    for (int i = threadIdx.x; i < nH; i += blockDim.x) {
      const double fi = f[i];
      ff = fma(fi, fi, ff);
      for (int k = 0; k < 4; ++k) {
        const double d = v[(size_t)s * 4 * nH + k * nH + i] - fi;
        e[k] = fma(d, d, e[k]);
      }
      if (smag) {
        const double d = smag[(size_t)s * nH + i] - fi;
        e[4] = fma(d, d, e[4]);
      }
    }
    for (int k = 0; k < 5; ++k) {
      const double x = block_sum(e[k], sh);
      if (threadIdx.x == 0) red[(size_t)s * NRED + k] = x;
    }
    const double x = block_sum(ff, sh);
    if (threadIdx.x == 0) red[(size_t)s * NRED + 5] = x;
  }
}

// Sum of per-sample partials over samples, in sample order (deterministic).
__global__ void sum_samples_kernel(int ns, const double* __restrict__ red, double* out) {
  const int k = threadIdx.x;
  if (k >= NRED) return;
  double acc = 0.0;
  for (int s = 0; s < ns; ++s) acc += red[(size_t)s * NRED + k];
  out[k] = acc;
}

struct SmagFitArgs {
  Geo g;
  const double* u;
  const double* wd;
  const double* wl;
  double delta;
  double* ud;      // [ns][nh] scratch: double-filtered velocity
  double* fields;  // [ns][4][nh] Sh, Th, SH, TH (or null)
  double* red;     // [ns][NRED]: S.T, S.S classic, S.T, S.S discrete
};

// `smagorinsky_fields` (src/Burgers.jl:547-688) and the sums of the
// coefficient fit (smagorinsky.jl:32-45).
__global__ void __launch_bounds__(BT) smag_fit_kernel(SmagFitArgs A) {
  extern __shared__ double smem[];
  __shared__ double red[40];
  const Geo& g = A.g;
  const int np = padded(g);
  double* ue = smem;
  double* se = ue + np;
  double* wd = se + np;
  double* wl = wd + 2 * g.Rd + 1;
  for (int r = threadIdx.x; r < 2 * g.Rd + 1; r += blockDim.x) wd[r] = A.wd[r];
  for (int r = threadIdx.x; r < 2 * g.Rl + 1; r += blockDim.x) wl[r] = A.wl[r];
  const double cs = -(A.delta * A.delta + g.H * g.H);
  for (int s = blockIdx.x; s < g.ns; s += gridDim.x) {
    load_sample(g, A.u + (size_t)s * g.nh, ue);
    __syncthreads();
    fill_stress(g, ue, se);
    double* ud = A.ud + (size_t)s * g.nh;
    for (int j = threadIdx.x; j < g.nh; j += blockDim.x) {
      double acc = 0.0;
      for (int r = -g.Rd; r <= g.Rd; ++r) acc = fma(wd[r + g.Rd], ue[g.G + j + r], acc);
      ud[j] = acc;
    }
    __syncthreads();
    double p0 = 0, p1 = 0, p2 = 0, p3 = 0;
    for (int j = threadIdx.x; j < g.nh; j += blockDim.x) {
      const int p = g.G + j;
      double s1 = 0.0, s1H = 0.0;
      for (int r = -g.Rd; r <= g.Rd; ++r) s1 = fma(wd[r + g.Rd], se[p + r], s1);
      for (int r = -g.Rl; r <= g.Rl; ++r) s1H = fma(wl[r + g.Rl], se[p + r], s1H);
      const double um = ud[j == 0 ? g.nh - 1 : j - 1], uj = ud[j];
      const double th = s1 - bstress(um, uj, g.vh);
      const double du = (uj - um) * g.ih;
      const double sh = cs * fabs(du) * du;
      int jl = j - g.a - 1, jr = j + g.a;
      jl = ((jl % g.nh) + g.nh) % g.nh;
      jr = jr % g.nh;
      const double ul = ud[jl], ur = ud[jr];
      const double tH = s1H - bstress(ul, ur, g.vH);
      const double dH = (ur - ul) * g.iH;
      const double sH = cs * fabs(dH) * dH;
      p0 = fma(sh, th, p0);
      p1 = fma(sh, sh, p1);
      p2 = fma(sH, tH, p2);
      p3 = fma(sH, sH, p3);
      if (A.fields) {
        double* f = A.fields + (size_t)s * 4 * g.nh;
        f[j] = sh;
        f[g.nh + j] = th;
        f[2 * g.nh + j] = sH;
        f[3 * g.nh + j] = tH;
      }
    }
    p0 = block_sum(p0, red);
    p1 = block_sum(p1, red);
    p2 = block_sum(p2, red);
    p3 = block_sum(p3, red);
    if (threadIdx.x == 0) {
      double* r = A.red + (size_t)s * NRED;
      r[0] = p0; r[1] = p1; r[2] = p2; r[3] = p3;
      r[4] = r[5] = r[6] = r[7] = 0.0;
    }
    __syncthreads();
  }
}

struct SmagSolveArgs {
  Geo g;
  const double* u0;
  const double* wd;
  double C, cfl, tstop;
  int max_steps;
  double* ub;   // [ns][nH]
  double* t;    // [ns]
  int* steps;   // [ns]
  bool init;
  int* err;
};

// `solve_smagorinsky` + `smagorinsky_rhs!` (src/Burgers.jl:690-786).  The
// stages update the running state in place (`axpy!` on ubar), as written
// in the reference.  Shared memory: x[nH+2] (ghosts 0 and nH+1), x0[nH],
// acc[nH], sig[nH+2].
__global__ void __launch_bounds__(BT) smag_solve_kernel(SmagSolveArgs A) {
  extern __shared__ double smem[];
  __shared__ double red[40];
  const Geo g = A.g;
  const int nH = g.nH;
  double* x = smem;
  double* x0 = x + nH + 2;
  double* ac = x0 + nH;
  double* sg = ac + nH;
  for (int s = blockIdx.x; s < g.ns; s += gridDim.x) {
    double* ubs = A.ub + (size_t)s * nH;
    double tt = 0.0;
    if (A.init) {
      const double* us = A.u0 + (size_t)s * g.nh;
      for (int I = threadIdx.x; I < nH; I += blockDim.x) {
        const int f0 = (I + 1) * g.comp - 1;
        double acc = 0.0;
        for (int r = -g.Rd; r <= g.Rd; ++r) {
          int j = (f0 + r) % g.nh;
          if (j < 0) j += g.nh;
          acc = fma(A.wd[r + g.Rd], us[j], acc);
        }
        x[1 + I] = acc;
      }
    } else {
      for (int I = threadIdx.x; I < nH; I += blockDim.x) x[1 + I] = ubs[I];
      tt = A.t[s];
    }
    int done = 0;
    __syncthreads();
    while (tt < A.tstop && done < A.max_steps) {
      double m = 0.0;
      for (int i = threadIdx.x; i < nH; i += blockDim.x) m = nanmax(m, fabs(x[1 + i]));
      m = block_max(m, red);
      const double dtc = A.cfl * fmin(g.H / m, g.H * g.H / g.visc);
      const double dt = fmin(dtc, A.tstop - tt);
      if (!(m == m) || isinf(m) || !(dtc > 1e-12 * A.tstop)) {
        if (threadIdx.x == 0) atomicExch(A.err, 1);
        break;
      }
      tt += dt;
      for (int q = 0; q < 4; ++q) {
        if (threadIdx.x == 0) {
          x[0] = x[nH];
          x[nH + 1] = x[1];
        }
        __syncthreads();
        for (int i = 1 + threadIdx.x; i <= nH + 1; i += blockDim.x) {
          const double s0 = bstress(x[i - 1], x[i], g.vH);
          const double du = (x[i] - x[i - 1]) * g.iH;
          const double smag = -A.C * fabs(du) * du;
          sg[i] = s0 - smag;
        }
        __syncthreads();
        for (int i = 1 + threadIdx.x; i <= nH; i += blockDim.x) {
          const double k = (sg[i + 1] - sg[i]) * g.iH;
          const int o = i - 1;
          if (q == 0) {
            x0[o] = x[i];
            ac[o] = k;
            x[i] = x[i] + dt / 2 * k;
          } else if (q == 1) {
            ac[o] = ac[o] + 2 * k;
            x[i] = x[i] + dt / 2 * k;
          } else if (q == 2) {
            ac[o] = ac[o] + 2 * k;
            x[i] = x[i] + dt * k;
          } else {
            x[i] = x0[o] + dt / 6 * (ac[o] + k);
          }
        }
        __syncthreads();
      }
      ++done;
    }
    for (int I = threadIdx.x; I < nH; I += blockDim.x) ubs[I] = x[1 + I];
    if (threadIdx.x == 0) {
      A.t[s] = tt;
      A.steps[s] = (A.init ? 0 : A.steps[s]) + done;
    }
    __syncthreads();
  }
}

// `randomfield` with `bump_profile` (src/Burgers.jl:192-202): sample s has
// phases U_k from the counter hash of (seed + s, k); the inverse real DFT is
// summed directly over the modes whose amplitude is not negligible (amp[k],
// k <= kc), then scaled to the kinetic energy.
__device__ __forceinline__ uint64_t splitmix(uint64_t x) {
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__global__ void __launch_bounds__(BT) random_kernel(int nh, int ns, double l, double energy, uint64_t seed,
                                                    int kc, const double* __restrict__ amp, double* u,
                                                    double* u0) {
  extern __shared__ double smem[];
  __shared__ double red[40];
  double2* ck = reinterpret_cast<double2*>(smem);
  for (int s = blockIdx.x; s < ns; s += gridDim.x) {
    const uint64_t base = (seed + (uint64_t)s) * 0x9E3779B97F4A7C15ull;
    for (int k = threadIdx.x; k <= kc; k += blockDim.x) {
      const double U = ((double)(splitmix(base + (uint64_t)k) >> 11) + 0.5) * 0x1.0p-53;
      double sn, cs;
      sincospi(2.0 * U, &sn, &cs);
      // irfft weights: 1 for k = 0 and the Nyquist mode, 2 otherwise
      const double wk = (k == 0 || 2 * k == nh) ? 1.0 : 2.0;
      ck[k] = make_double2(wk * amp[k] * cs, wk * amp[k] * sn);
    }
    __syncthreads();
    double* us = u + (size_t)s * nh;
    double e = 0.0;
    for (int j = threadIdx.x; j < nh; j += blockDim.x) {
      double a = 0.0;
      for (int k = 0; k <= kc; ++k) {
        const long long m = ((long long)k * j) % nh;
        double sn, cs;
        sincospi(2.0 * (double)m / (double)nh, &sn, &cs);
        a = fma(ck[k].x, cs, fma(-ck[k].y, sn, a));
      }
      us[j] = a;
      e = fma(a, a, e);
    }
    e = block_sum(e, red);
    const double f = sqrt(energy / (e / 2 * (l / nh)));
    for (int j = threadIdx.x; j < nh; j += blockDim.x) {
      const double x = f * us[j];
      us[j] = x;
      u0[(size_t)s * nh + j] = x;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ host

int grid_for(const void* fn, size_t smem, int ns) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, BT, smem);
  if (per < 1) per = 1;
  const long long g = (long long)sms * per;
  return (int)(ns < g ? ns : g);
}

int smem_optin() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return v;
}

cudaError_t allow_smem(const void* fn, size_t bytes) {
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

Geo geo_of(const exc_burgers* b) {
  Geo g;
  g.nh = b->nh;
  g.ns = b->ns;
  g.h = b->h;
  g.visc = b->visc;
  g.nH = b->nH;
  g.comp = b->comp;
  g.a = b->a;
  g.Rd = b->Rd;
  g.Rl = b->Rl;
  g.H = b->H;
  g.G = (b->les_on ? b->Rd : 0) + 1;
  g.ih = 1.0 / b->h;
  g.vh = b->visc / b->h;
  g.iH = b->H > 0 ? 1.0 / b->H : 0.0;
  g.vH = b->H > 0 ? b->visc / b->H : 0.0;
  return g;
}

// Filter kernels of one LES grid (src/Burgers.jl:146-162, :218-233,
// :355-364): the LES kernel (Gaussian or odd top hat) and the double kernel
// = top hat of the compression ratio convolved with it.
int make_kernels(int nh, int nH, double l, double delta_ratio, int filter, std::vector<double>& wl, int& Rl,
                 std::vector<double>& wd, int& Rd) {
  if (nH < 1 || nH > nh || nh % nH) { set_last_error("nH must divide nh"); return EXC_ERR_RATIO; }
  const int comp = nh / nH;
  if (comp % 2 == 0) { set_last_error("compression nh/nH must be odd (top-hat kernel of the reference)"); return EXC_ERR_RATIO; }
  if (!(delta_ratio >= 0) || !std::isfinite(delta_ratio)) { set_last_error("delta_ratio must be >= 0"); return EXC_ERR_ARG; }
  const double h = l / nh, H = l / nH, delta = H * delta_ratio;
  wl.clear();
  if (filter == EXC_BURGERS_GAUSSIAN) {
    const double s2 = (delta / h) * (delta / h) / 12;
    Rl = (int)std::nearbyint(3.0 * std::sqrt(s2));
    if (delta < 1.0e-15) {
      Rl = 0;
      wl.assign(1, 1.0);
    } else {
      double sum = 0.0;
      for (int r = -Rl; r <= Rl; ++r) {
        wl.push_back(std::exp(-(double)r * r / (2 * s2)));
        sum += wl.back();
      }
      for (double& w : wl) w /= sum;
    }
  } else if (filter == EXC_BURGERS_TOPHAT) {
    const int lescomp = (int)std::nearbyint(delta / h);
    Rl = lescomp / 2;
    wl.assign(2 * Rl + 1, 1.0 / (2 * Rl + 1));
  } else {
    set_last_error("filter must be EXC_BURGERS_GAUSSIAN or EXC_BURGERS_TOPHAT");
    return EXC_ERR_ARG;
  }
  const int I = comp / 2;
  const double fv = 1.0 / comp;
  Rd = I + Rl;
  wd.assign(2 * Rd + 1, 0.0);
  for (int k = -Rd; k <= Rd; ++k) {
    double s = 0.0;
    for (int j = -Rl; j <= Rl; ++j) {
      const int i = k - j;
      if (i >= -I && i <= I) s += fv * wl[j + Rl];
    }
    wd[k + Rd] = s;
  }
  if (2 * Rd + 1 > nh) { set_last_error("filter kernel wider than the grid"); return EXC_ERR_SHAPE; }
  return EXC_OK;
}

template <typename T>
int dalloc(T** p, size_t count) {
  if (cudaMalloc(p, count * sizeof(T)) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    set_last_error("device allocation failed");
    return EXC_ERR_OOM;
  }
  return EXC_OK;
}

void free_les(exc_burgers* b) {
  cudaFree(b->wd); cudaFree(b->wl); cudaFree(b->v); cudaFree(b->tmp);
  cudaFree(b->smag); cudaFree(b->tsm); cudaFree(b->ssm);
  b->wd = b->wl = b->v = b->tmp = b->smag = b->tsm = nullptr;
  b->ssm = nullptr;
  b->les_on = b->smag_on = false;
  b->nH = b->comp = b->a = b->Rd = b->Rl = 0;
}

int check_flag(exc_burgers* b) {
  int f = 0;
  cudaError_t e = cudaMemcpyAsync(&f, b->err, sizeof(int), cudaMemcpyDeviceToHost, b->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  if (f) {
    cudaMemsetAsync(b->err, 0, sizeof(int), b->st);
    set_last_error("non-finite Burgers velocity or collapsed time step");
    return EXC_ERR_NONFINITE;
  }
  return EXC_OK;
}

int launch_err(exc_burgers* b) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  (void)b;
  return EXC_OK;
}

int max_steps_of(exc_burgers* b, int* out) {
  std::vector<int> s(b->ns);
  cudaError_t e = cudaMemcpyAsync(s.data(), b->steps, b->ns * sizeof(int), cudaMemcpyDeviceToHost, b->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  int m = 0;
  for (int x : s) m = x > m ? x : m;
  *out = m;
  return EXC_OK;
}

int run_terms(exc_burgers* b, double* terms, double* diss, double* fine, double* les_init, double* red) {
  const Geo g = geo_of(b);
  const size_t sm = sample_smem(g);
  if (allow_smem((const void*)terms_kernel, sm) != cudaSuccess) { cudaGetLastError(); set_last_error("shared memory opt-in failed"); return EXC_ERR_CUDA; }
  TermsArgs A{g, b->u, b->wd, b->wl, terms, diss, fine, les_init, red};
  terms_kernel<<<grid_for((const void*)terms_kernel, sm, b->ns), BT, sm, b->st>>>(A);
  return launch_err(b);
}

}  // namespace
}  // namespace exc

using namespace exc;

extern "C" {

int exc_burgers_kernels(int nh, int nH, double l, double delta_ratio, int filter, int* Rl, double* wl, int* Rd,
                        double* wd) {
  if (!Rl || !Rd || nh < 1) { set_last_error("null argument or bad nh"); return EXC_ERR_ARG; }
  std::vector<double> vl, vd;
  int rl = 0, rd = 0;
  int rc = make_kernels(nh, nH, l, delta_ratio, filter, vl, rl, vd, rd);
  if (rc) return rc;
  *Rl = rl;
  *Rd = rd;
  if (wl) for (size_t i = 0; i < vl.size(); ++i) wl[i] = vl[i];
  if (wd) for (size_t i = 0; i < vd.size(); ++i) wd[i] = vd[i];
  return EXC_OK;
}

int exc_burgers_create(const exc_burgers_desc* d, void* stream, exc_burgers** out) {
  if (!d || !out) { set_last_error("null argument"); return EXC_ERR_ARG; }
  *out = nullptr;
  if (d->nh < 4 || d->nsample < 1) { set_last_error("nh >= 4 and nsample >= 1 required"); return EXC_ERR_SHAPE; }
  if (!(d->l > 0) || !(d->visc > 0)) { set_last_error("l and visc must be positive"); return EXC_ERR_ARG; }
  int rc = configure_device();
  if (rc) return rc;
  // The DNS state of a sample (u and its stress with ghosts) must fit in
  // one CTA's shared memory.
  Geo g{};
  g.nh = d->nh;
  g.G = 1;
  if (sample_smem(g) + 1024 > (size_t)smem_optin()) { set_last_error("nh too large for a shared-memory resident sample"); return EXC_ERR_SHAPE; }
  exc_burgers* b = new exc_burgers();
  b->nh = d->nh;
  b->ns = d->nsample;
  b->l = d->l;
  b->visc = d->visc;
  b->h = d->l / d->nh;
  b->st = (cudaStream_t)stream;
  const size_t N = (size_t)b->nh * b->ns;
  if (dalloc(&b->u, N) || dalloc(&b->u0, N) || dalloc(&b->t, b->ns) || dalloc(&b->steps, b->ns) ||
      dalloc(&b->scr, 2 * N) || dalloc(&b->red, (size_t)b->ns * NRED) || dalloc(&b->sums, NRED) ||
      dalloc(&b->err, 1)) {
    exc_burgers_destroy(b);
    return EXC_ERR_OOM;
  }
  cudaMemsetAsync(b->u, 0, N * sizeof(double), b->st);
  cudaMemsetAsync(b->u0, 0, N * sizeof(double), b->st);
  cudaMemsetAsync(b->t, 0, b->ns * sizeof(double), b->st);
  cudaMemsetAsync(b->steps, 0, b->ns * sizeof(int), b->st);
  cudaMemsetAsync(b->err, 0, sizeof(int), b->st);
  rc = launch_err(b);
  if (rc) { exc_burgers_destroy(b); return rc; }
  *out = b;
  return EXC_OK;
}

int exc_burgers_destroy(exc_burgers* b) {
  if (!b) return EXC_OK;
  if (b->st) cudaStreamSynchronize(b->st); else cudaDeviceSynchronize();
  free_les(b);
  cudaFree(b->u); cudaFree(b->u0); cudaFree(b->t); cudaFree(b->steps); cudaFree(b->scr);
  cudaFree(b->red); cudaFree(b->sums); cudaFree(b->err);
  delete b;
  return EXC_OK;
}

static int reset_clock(exc_burgers* b) {
  cudaMemsetAsync(b->t, 0, b->ns * sizeof(double), b->st);
  cudaMemsetAsync(b->steps, 0, b->ns * sizeof(int), b->st);
  return launch_err(b);
}

int exc_burgers_init_random(exc_burgers* b, double kpeak, double energy, uint64_t seed) {
  if (!b || !(kpeak > 0) || !(energy > 0)) { set_last_error("null handle or non-positive kpeak/energy"); return EXC_ERR_ARG; }
  // Amplitudes (k/k0)^4 exp(-2 (k/k0)^2); modes below 1e-30 of the peak
  // change no double of the result and are left out of the sum.
  const int kn = b->nh / 2;
  std::vector<double> amp(kn + 1);
  double amax = 0.0;
  for (int k = 0; k <= kn; ++k) {
    const double q = k / kpeak;
    amp[k] = (q * q) * (q * q) * std::exp(-2 * q * q);
    amax = amp[k] > amax ? amp[k] : amax;
  }
  int kc = 0;
  for (int k = 0; k <= kn; ++k)
    if (amp[k] > 1e-30 * amax) kc = k;
  double* damp = nullptr;
  int rc = dalloc(&damp, kc + 1);
  if (rc) return rc;
  cudaMemcpyAsync(damp, amp.data(), (kc + 1) * sizeof(double), cudaMemcpyHostToDevice, b->st);
  const size_t sm = (size_t)(kc + 1) * sizeof(double2);
  if (allow_smem((const void*)random_kernel, sm) != cudaSuccess) { cudaGetLastError(); cudaFree(damp); set_last_error("shared memory opt-in failed"); return EXC_ERR_CUDA; }
  random_kernel<<<grid_for((const void*)random_kernel, sm, b->ns), BT, sm, b->st>>>(b->nh, b->ns, b->l, energy, seed, kc,
                                                                                    damp, b->u, b->u0);
  rc = launch_err(b);
  cudaStreamSynchronize(b->st);
  cudaFree(damp);
  if (rc) return rc;
  return reset_clock(b);
}

int exc_burgers_set_velocity(exc_burgers* b, const double* host) {
  if (!b || !host) { set_last_error("null argument"); return EXC_ERR_ARG; }
  const size_t bytes = (size_t)b->nh * b->ns * sizeof(double);
  EXC_CHECK_CUDA(cudaMemcpyAsync(b->u, host, bytes, cudaMemcpyHostToDevice, b->st));
  EXC_CHECK_CUDA(cudaMemcpyAsync(b->u0, b->u, bytes, cudaMemcpyDeviceToDevice, b->st));
  EXC_CHECK_CUDA(cudaStreamSynchronize(b->st));
  return reset_clock(b);
}

int exc_burgers_get_velocity(exc_burgers* b, int initial, double* host) {
  if (!b || !host) { set_last_error("null argument"); return EXC_ERR_ARG; }
  const size_t bytes = (size_t)b->nh * b->ns * sizeof(double);
  EXC_CHECK_CUDA(cudaMemcpyAsync(host, initial ? b->u0 : b->u, bytes, cudaMemcpyDeviceToHost, b->st));
  EXC_CHECK_CUDA(cudaStreamSynchronize(b->st));
  return EXC_OK;
}

int exc_burgers_restart(exc_burgers* b) {
  if (!b) { set_last_error("null handle"); return EXC_ERR_ARG; }
  EXC_CHECK_CUDA(cudaMemcpyAsync(b->u, b->u0, (size_t)b->nh * b->ns * sizeof(double), cudaMemcpyDeviceToDevice, b->st));
  return reset_clock(b);
}

int exc_burgers_time(exc_burgers* b, double* t, int* steps) {
  if (!b) { set_last_error("null handle"); return EXC_ERR_ARG; }
  if (t) EXC_CHECK_CUDA(cudaMemcpyAsync(t, b->t, b->ns * sizeof(double), cudaMemcpyDeviceToHost, b->st));
  if (steps) EXC_CHECK_CUDA(cudaMemcpyAsync(steps, b->steps, b->ns * sizeof(int), cudaMemcpyDeviceToHost, b->st));
  EXC_CHECK_CUDA(cudaStreamSynchronize(b->st));
  return EXC_OK;
}

int exc_burgers_les_setup(exc_burgers* b, int nH, double delta_ratio, int filter) {
  if (!b) { set_last_error("null handle"); return EXC_ERR_ARG; }
  cudaStreamSynchronize(b->st);
  free_les(b);
  if (nH == 0) return EXC_OK;
  std::vector<double> wl, wd;
  int Rl = 0, Rd = 0;
  int rc = make_kernels(b->nh, nH, b->l, delta_ratio, filter, wl, Rl, wd, Rd);
  if (rc) return rc;
  b->nH = nH;
  b->comp = b->nh / nH;
  b->a = b->comp / 2;
  b->Rl = Rl;
  b->Rd = Rd;
  b->H = b->l / nH;
  b->delta_ratio = delta_ratio;
  b->delta = b->H * delta_ratio;
  b->filter = filter;
  b->wl_h = wl;
  b->wd_h = wd;
  b->les_on = true;
  const Geo g = geo_of(b);
  if (sample_smem(g) + 1024 > (size_t)smem_optin()) {
    free_les(b);
    set_last_error("nh plus filter halo too large for a shared-memory resident sample");
    return EXC_ERR_SHAPE;
  }
  const size_t M = (size_t)b->ns * nH;
  if (dalloc(&b->wd, wd.size()) || dalloc(&b->wl, wl.size()) || dalloc(&b->v, 8 * M) || dalloc(&b->tmp, 5 * M) ||
      dalloc(&b->smag, M) || dalloc(&b->tsm, b->ns) || dalloc(&b->ssm, b->ns)) {
    free_les(b);
    return EXC_ERR_OOM;
  }
  b->les_on = true;
  b->nH = nH;
  EXC_CHECK_CUDA(cudaMemcpyAsync(b->wd, wd.data(), wd.size() * sizeof(double), cudaMemcpyHostToDevice, b->st));
  EXC_CHECK_CUDA(cudaMemcpyAsync(b->wl, wl.data(), wl.size() * sizeof(double), cudaMemcpyHostToDevice, b->st));
  // Initial double-filtered state of every LES (src/Burgers.jl:366-379).
  rc = run_terms(b, nullptr, nullptr, nullptr, b->v, nullptr);
  if (rc) return rc;
  EXC_CHECK_CUDA(cudaStreamSynchronize(b->st));
  return EXC_OK;
}

int exc_burgers_advance(exc_burgers* b, double tstop, double cfl, int scheme, int max_steps, int* steps_max) {
  if (!b || !(cfl > 0) || !(tstop >= 0)) { set_last_error("null handle or bad cfl/tstop"); return EXC_ERR_ARG; }
  if (scheme != EXC_BURGERS_EULER && scheme != EXC_BURGERS_RK4) { set_last_error("scheme must be EULER or RK4"); return EXC_ERR_ARG; }
  if (b->les_on && scheme != EXC_BURGERS_EULER) {
    set_last_error("the DNS-aided LES steps with forward Euler (dns_aided_les)");
    return EXC_ERR_STATE;
  }
  AdvanceArgs A{};
  A.g = geo_of(b);
  A.cfl = cfl;
  A.tstop = tstop;
  A.max_steps = (max_steps > 0 && max_steps < MAX_STEPS_PER_CALL) ? max_steps : MAX_STEPS_PER_CALL;
  A.u = b->u;
  A.t = b->t;
  A.steps = b->steps;
  A.wd = b->wd;
  A.wl = b->wl;
  A.v0 = b->v;
  A.v1 = b->v ? b->v + (size_t)4 * b->ns * b->nH : nullptr;
  A.tmp = b->tmp;
  A.uold = b->scr;
  A.acc = b->scr + (size_t)b->nh * b->ns;
  A.err = b->err;
  const size_t sm = sample_smem(A.g);
  const void* fn = b->les_on ? (const void*)advance_kernel<true, false>
                             : scheme == EXC_BURGERS_RK4 ? (const void*)advance_kernel<false, true>
                                                         : (const void*)advance_kernel<false, false>;
  if (allow_smem(fn, sm) != cudaSuccess) { cudaGetLastError(); set_last_error("shared memory opt-in failed"); return EXC_ERR_CUDA; }
  const int grid = grid_for(fn, sm, b->ns);
  if (b->les_on) advance_kernel<true, false><<<grid, BT, sm, b->st>>>(A);
  else if (scheme == EXC_BURGERS_RK4) advance_kernel<false, true><<<grid, BT, sm, b->st>>>(A);
  else advance_kernel<false, false><<<grid, BT, sm, b->st>>>(A);
  int rc = launch_err(b);
  if (rc) return rc;
  rc = check_flag(b);
  if (rc) return rc;
  if (steps_max) return max_steps_of(b, steps_max);
  return EXC_OK;
}

int exc_burgers_get_les(exc_burgers* b, int which, double* host) {
  if (!b || !host) { set_last_error("null argument"); return EXC_ERR_ARG; }
  if (!b->les_on) { set_last_error("no LES grid set up"); return EXC_ERR_STATE; }
  const size_t M = (size_t)b->nH;
  std::vector<double> tmp;
  if (which == EXC_BURGERS_DNS_FIL) {
    int rc = run_terms(b, b->tmp, nullptr, nullptr, nullptr, nullptr);
    if (rc) return rc;
    for (int s = 0; s < b->ns; ++s)
      EXC_CHECK_CUDA(cudaMemcpyAsync(host + s * M, b->tmp + (size_t)s * 5 * M + 2 * M, M * sizeof(double),
                                     cudaMemcpyDeviceToHost, b->st));
  } else if (which >= EXC_BURGERS_NOMODEL && which <= EXC_BURGERS_SWAPFIL) {
    const int k = which - EXC_BURGERS_NOMODEL;
    for (int s = 0; s < b->ns; ++s)
      EXC_CHECK_CUDA(cudaMemcpyAsync(host + s * M, b->v + (size_t)s * 4 * M + k * M, M * sizeof(double),
                                     cudaMemcpyDeviceToHost, b->st));
  } else if (which == EXC_BURGERS_SMAG) {
    if (!b->smag_on) { set_last_error("no Smagorinsky solve has run"); return EXC_ERR_STATE; }
    EXC_CHECK_CUDA(cudaMemcpyAsync(host, b->smag, b->ns * M * sizeof(double), cudaMemcpyDeviceToHost, b->st));
  } else {
    set_last_error("bad field selector");
    return EXC_ERR_ARG;
  }
  EXC_CHECK_CUDA(cudaStreamSynchronize(b->st));
  return EXC_OK;
}

int exc_burgers_filtered(exc_burgers* b, double* host_fine) {
  if (!b || !host_fine) { set_last_error("null argument"); return EXC_ERR_ARG; }
  if (!b->les_on) { set_last_error("no LES grid set up"); return EXC_ERR_STATE; }
  int rc = run_terms(b, nullptr, nullptr, b->scr, nullptr, nullptr);
  if (rc) return rc;
  EXC_CHECK_CUDA(cudaMemcpyAsync(host_fine, b->scr, (size_t)b->ns * b->nh * sizeof(double), cudaMemcpyDeviceToHost,
                                 b->st));
  EXC_CHECK_CUDA(cudaStreamSynchronize(b->st));
  return EXC_OK;
}

int exc_burgers_errors(exc_burgers* b, double out[5]) {
  if (!b || !out) { set_last_error("null argument"); return EXC_ERR_ARG; }
  if (!b->les_on) { set_last_error("no LES grid set up"); return EXC_ERR_STATE; }
  int rc = run_terms(b, b->tmp, nullptr, nullptr, nullptr, nullptr);
  if (rc) return rc;
  errors_kernel<<<grid_for((const void*)errors_kernel, 0, b->ns), BT, 0, b->st>>>(
      b->ns, b->nH, b->v, b->smag_on ? b->smag : nullptr, b->tmp, b->red);
  sum_samples_kernel<<<1, 32, 0, b->st>>>(b->ns, b->red, b->sums);
  rc = launch_err(b);
  if (rc) return rc;
  double s[NRED];
  EXC_CHECK_CUDA(cudaMemcpyAsync(s, b->sums, sizeof(s), cudaMemcpyDeviceToHost, b->st));
  EXC_CHECK_CUDA(cudaStreamSynchronize(b->st));
  const double nr = std::sqrt(s[5]);
  for (int k = 0; k < 5; ++k) out[k] = (k == 4 && !b->smag_on) ? NAN : std::sqrt(s[k]) / nr;
  return EXC_OK;
}

int exc_burgers_closure_terms(exc_burgers* b, double* terms, double* diss, double fractions[3]) {
  if (!b) { set_last_error("null handle"); return EXC_ERR_ARG; }
  if (!b->les_on) { set_last_error("no LES grid set up"); return EXC_ERR_STATE; }
  const size_t M = (size_t)b->ns * b->nH;
  double* dd = nullptr;
  if (diss) {
    int rc = dalloc(&dd, 3 * M);
    if (rc) return rc;
  }
  int rc = run_terms(b, b->tmp, dd, nullptr, nullptr, b->red);
  if (!rc) {
    sum_samples_kernel<<<1, 32, 0, b->st>>>(b->ns, b->red, b->sums);
    rc = launch_err(b);
  }
  double s[NRED];
  if (!rc && cudaMemcpyAsync(s, b->sums, sizeof(s), cudaMemcpyDeviceToHost, b->st) != cudaSuccess) rc = EXC_ERR_CUDA;
  if (!rc && terms && cudaMemcpyAsync(terms, b->tmp, 5 * M * sizeof(double), cudaMemcpyDeviceToHost, b->st) != cudaSuccess) rc = EXC_ERR_CUDA;
  if (!rc && diss && cudaMemcpyAsync(diss, dd, 3 * M * sizeof(double), cudaMemcpyDeviceToHost, b->st) != cudaSuccess) rc = EXC_ERR_CUDA;
  if (cudaStreamSynchronize(b->st) != cudaSuccess && !rc) rc = EXC_ERR_CUDA;
  if (dd) cudaFree(dd);
  if (rc == EXC_ERR_CUDA) set_last_error("CUDA copy failed");
  if (rc) return rc;
  if (fractions)
    for (int k = 0; k < 3; ++k) fractions[k] = s[k] / b->ns;
  return EXC_OK;
}

int exc_burgers_smagorinsky_fit(exc_burgers* b, double theta2[2], double* fields) {
  if (!b || !theta2) { set_last_error("null argument"); return EXC_ERR_ARG; }
  if (!b->les_on) { set_last_error("no LES grid set up"); return EXC_ERR_STATE; }
  const size_t N = (size_t)b->ns * b->nh;
  double* df = nullptr;
  if (fields) {
    int rc = dalloc(&df, 4 * N);
    if (rc) return rc;
  }
  SmagFitArgs A{geo_of(b), b->u, b->wd, b->wl, b->delta, b->scr, df, b->red};
  const size_t sm = sample_smem(A.g);
  int rc = EXC_OK;
  if (allow_smem((const void*)smag_fit_kernel, sm) != cudaSuccess) { cudaGetLastError(); rc = EXC_ERR_CUDA; set_last_error("shared memory opt-in failed"); }
  if (!rc) {
    smag_fit_kernel<<<grid_for((const void*)smag_fit_kernel, sm, b->ns), BT, sm, b->st>>>(A);
    sum_samples_kernel<<<1, 32, 0, b->st>>>(b->ns, b->red, b->sums);
    rc = launch_err(b);
  }
  double s[NRED];
  if (!rc && cudaMemcpyAsync(s, b->sums, sizeof(s), cudaMemcpyDeviceToHost, b->st) != cudaSuccess) rc = EXC_ERR_CUDA;
  if (!rc && fields && cudaMemcpyAsync(fields, df, 4 * N * sizeof(double), cudaMemcpyDeviceToHost, b->st) != cudaSuccess) rc = EXC_ERR_CUDA;
  if (cudaStreamSynchronize(b->st) != cudaSuccess && !rc) rc = EXC_ERR_CUDA;
  if (df) cudaFree(df);
  if (rc == EXC_ERR_CUDA) set_last_error("CUDA error in the Smagorinsky fit");
  if (rc) return rc;
  theta2[0] = -s[0] / s[1];
  theta2[1] = -s[2] / s[3];
  return EXC_OK;
}

int exc_burgers_smagorinsky_solve(exc_burgers* b, double theta, double tstop, double cfl, int max_steps,
                                  int restart, int* steps_max) {
  if (!b || !(cfl > 0) || !(tstop >= 0) || !std::isfinite(theta)) { set_last_error("null handle or bad argument"); return EXC_ERR_ARG; }
  if (!b->les_on) { set_last_error("no LES grid set up"); return EXC_ERR_STATE; }
  if (!restart && !b->smag_on) { set_last_error("no Smagorinsky solve to continue"); return EXC_ERR_STATE; }
  SmagSolveArgs A{};
  A.g = geo_of(b);
  A.u0 = b->u0;
  A.wd = b->wd;
  A.C = theta * theta * (b->delta * b->delta + b->H * b->H);
  A.cfl = cfl;
  A.tstop = tstop;
  A.max_steps = (max_steps > 0 && max_steps < MAX_STEPS_PER_CALL) ? max_steps : MAX_STEPS_PER_CALL;
  A.ub = b->smag;
  A.t = b->tsm;
  A.steps = b->ssm;
  A.init = restart != 0;
  A.err = b->err;
  const size_t sm = (size_t)(4 * b->nH + 4) * sizeof(double);
  if (sm + 1024 > (size_t)smem_optin()) { set_last_error("LES grid too large for the Smagorinsky solver"); return EXC_ERR_SHAPE; }
  if (allow_smem((const void*)smag_solve_kernel, sm) != cudaSuccess) { cudaGetLastError(); set_last_error("shared memory opt-in failed"); return EXC_ERR_CUDA; }
  smag_solve_kernel<<<grid_for((const void*)smag_solve_kernel, sm, b->ns), BT, sm, b->st>>>(A);
  int rc = launch_err(b);
  if (rc) return rc;
  b->smag_on = true;
  rc = check_flag(b);
  if (rc) return rc;
  if (steps_max) {
    std::vector<int> s(b->ns);
    EXC_CHECK_CUDA(cudaMemcpyAsync(s.data(), b->ssm, b->ns * sizeof(int), cudaMemcpyDeviceToHost, b->st));
    EXC_CHECK_CUDA(cudaStreamSynchronize(b->st));
    int m = 0;
    for (int x : s) m = x > m ? x : m;
    *steps_max = m;
  }
  return EXC_OK;
}

int exc_burgers_device_ptr(exc_burgers* b, int which, void** ptr) {
  if (!b || !ptr) { set_last_error("null argument"); return EXC_ERR_ARG; }
  switch (which) {
    case 0: *ptr = b->u; break;
    case 1: *ptr = b->u0; break;
    case 2: *ptr = b->v; break;
    default: set_last_error("bad selector"); return EXC_ERR_ARG;
  }
  return EXC_OK;
}

}  // extern "C"
