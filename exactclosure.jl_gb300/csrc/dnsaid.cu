// The reference's own DNS-aided driver `dnsaid_project` (src/N.jl:1239-1332)
// on the GPU: a forward-Euler warm-up of the DNS, then the DNS and five LES
// -- no model, classic, classic+flux, classic+flux+div (the exact closure)
// and its symmetrised form -- stepped in lockstep with the DNS time step.
// A second mode runs the paper's volume-average driver `dns_aid_volavg`
// (src/NavierStokes.jl:141-304) with four LES: no model, classic (volume-
// filtered flux), swap (face-filtered flux) and its symmetric part; a third
// its surface-average driver `dns_aid_surface` (src/NavierStokes.jl:306-468):
// the same four LES on the face-filtered DNS, classic with the surface-
// filtered flux, swap with the line-filtered flux off the diagonal.
//
// Every operator is a libexc kernel (stress/divergence, FFT projection,
// filtered fluxes); this file holds the driver, two pointwise tensor kernels
// and the error reductions.  FP64, like the reference.  The LES grids of the
// reference's setups are small next to the DNS, so the DNS right-hand side,
// its projection and the filtered fluxes of the DNS (rDHi, sigmaDH, the
// classic closure's stress of the filtered field) carry the cost.
#include <cmath>
#include <vector>

#include "fields.cuh"
#include "filter.cuh"
#include "internal.cuh"

struct exc_dnsaid {
  int n = 0, m = 0, c = 0;
  double l = 0, visc = 0, h = 0, H = 0;
  std::vector<double> fdelta;
  cudaStream_t st = nullptr;
  exc_poisson psd{}, psl{};
  double* u = nullptr;     // DNS velocity 3N
  double* du = nullptr;    // DNS right-hand side 3N
  double* p = nullptr;     // DNS pressure N
  double* les[5] = {};     // u_nomo, u_c, u_cf, u_cfd, u_cfd_symm: 3M each
  double* ub = nullptr;    // apply_DHpi(u) 3M
  double* dul = nullptr;   // LES right-hand side 3M
  double* sdh = nullptr;   // sigmaDH 6M
  double* s2 = nullptr;    // classic sigma2 6M
  double* r9 = nullptr;    // rDHi 9M
  double* sl = nullptr;    // stress of an LES field 6M
  double* sc = nullptr;    // combined stress 6M
  double* zero = nullptr;  // M zeros
  double* scal = nullptr;  // device scalars
  double* part = nullptr;  // reduction partials
  double* spec = nullptr;  // init scratch: 3 spectral arrays
  double* pl = nullptr;    // LES pressure M (paper mode)
  double* dsig = nullptr;  // closure divergence 3M (paper mode)
  double* rc9 = nullptr;   // surface-filtered flux 9M (surface mode)
  double t = 0;
  int steps = 0;
  bool started = false;
  bool paper = false;      // dns_aid_volavg instead of dnsaid_project
  bool doproject = true;   // its `doproject`
  bool surface = false;    // dns_aid_surface instead of dns_aid_volavg
};

namespace exc {
namespace {

// out6 = (a + b) - c component-wise (b may be null: a - c), the LazyField
// sums of src/N.jl:1147-1159, 1172-1184, 1193-1199.
__global__ void combine6_kernel(long long M6, const double* __restrict__ a, const double* __restrict__ b,
                                const double* __restrict__ c, double* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < M6; i += (long long)gridDim.x * blockDim.x)
    out[i] = b ? (a[i] + b[i]) - c[i] : a[i] - c[i];
}

// `symmetrize` (src/N.jl:1075-1086): 9 components (s11, s21, s31, s12, s22,
// s32, s13, s23, s33) to 6 (s11, s22, s33, (s21+s12)/2, (s32+s23)/2,
// (s31+s13)/2).
__global__ void symmetrize_kernel(long long M, const double* __restrict__ r9, double* __restrict__ s6) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x) {
    s6[i] = r9[0 * M + i];
    s6[M + i] = r9[4 * M + i];
    s6[2 * M + i] = r9[8 * M + i];
    s6[3 * M + i] = (r9[1 * M + i] + r9[3 * M + i]) / 2;
    s6[4 * M + i] = (r9[5 * M + i] + r9[7 * M + i]) / 2;
    s6[5 * M + i] = (r9[2 * M + i] + r9[6 * M + i]) / 2;
  }
}

// s6 diagonal += p: r = sigma + p I on the LES grid.
__global__ void add_diag_kernel(long long M, double* __restrict__ s6, const double* __restrict__ p) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x) {
    const double q = p[i];
    s6[i] += q;
    s6[M + i] += q;
    s6[2 * M + i] += q;
  }
}

// r9 -= s6 with the symmetric s6 (s11, s22, s33, s12, s23, s31) expanded to
// the 9-component order (s11, s21, s31, s12, s22, s32, s13, s23, s33).
__global__ void sub_sym_kernel(long long M, double* __restrict__ r9, const double* __restrict__ s6) {
  // 9-component slot -> symmetric slot
  const int map[9] = {0, 3, 5, 3, 1, 4, 5, 4, 2};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x)
#pragma unroll
    for (int k = 0; k < 9; ++k) r9[k * M + i] -= s6[map[k] * M + i];
}

int gridsz(long long cnt) {
  long long b = (cnt + 255) / 256;
  return (int)(b < 152LL * 16 ? b : 152LL * 16);
}

int cuda_rc(cudaError_t e) {
  if (e == cudaSuccess) return EXC_OK;
  set_last_error(cudaGetErrorString(e));
  return EXC_ERR_CUDA;
}

const double* fd(const exc_dnsaid* d) { return d->fdelta.size() > 1 ? d->fdelta.data() : nullptr; }
int nfd(const exc_dnsaid* d) { return d->fdelta.size() > 1 ? (int)d->fdelta.size() : 0; }

// project!(v, poisson) (src/N.jl:256-307) in place; the pressure stays in the
// solver's work array.
cudaError_t project(exc_poisson* ps, double* v, cudaStream_t st) {
  cudaError_t e = poisson_solve_inplace<double>(ps, v, true, st);
  if (e == cudaSuccess) e = launch_gradient<double>(ps->n, ps->h, v, (const double*)ps->work, 2 * ps->P, st);
  return e;
}

// dt = min(cfl h / max|u|, cfl h^2 / visc / 6) (`propose_timestep`,
// src/N.jl:348-356), read back like the reference's host loop.
int propose_dt(exc_dnsaid* d, double cfl, double* dt) {
  const long long N3 = 3LL * d->n * d->n * d->n;
  cudaError_t e = launch_max_abs<double>((size_t)N3, d->u, d->scal, d->part, RED_PARTS, d->st);
  double umax = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&umax, d->scal, sizeof(double), cudaMemcpyDeviceToHost, d->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
  if (e != cudaSuccess) return cuda_rc(e);
  if (!std::isfinite(umax)) { set_last_error("non-finite DNS velocity detected"); return EXC_ERR_NONFINITE; }
  const double dt_adv = cfl * d->h / umax, dt_visc = cfl * d->h * d->h / d->visc / 6.0;
  *dt = dt_adv < dt_visc ? dt_adv : dt_visc;
  return EXC_OK;
}

// `apply_ΔHπ` (src/N.jl:1228-1237): volume filter, coarse-grain at the
// faces, project on the LES grid.
int apply_dhpi(exc_dnsaid* d, double* out) {
  int rc = filter_vector<double>(d->n, d->c, EXC_FILTER_VOLUME, fd(d), nfd(d), d->u, out, d->st);
  if (rc) return rc;
  return cuda_rc(project(&d->psl, out, d->st));
}

// v += dt * P(-div s6) on the LES grid, optionally adding -div r9 (nonsym)
// or -div sym6 before the projection.
int les_update(exc_dnsaid* d, double* v, const double* s6, const double* r9, const double* sym6, double dt) {
  const int m = d->m;
  const long long M3 = 3LL * m * m * m;
  cudaError_t e = launch_tensordiv<double>(m, d->H, 6, s6, d->dul, false, d->st);
  if (e == cudaSuccess && r9) e = launch_tensordiv<double>(m, d->H, 9, r9, d->dul, true, d->st);
  if (e == cudaSuccess && sym6) e = launch_tensordiv<double>(m, d->H, 6, sym6, d->dul, true, d->st);
  if (e == cudaSuccess) e = project(&d->psl, d->dul, d->st);
  if (e == cudaSuccess) e = launch_axpy<double>(M3, v, d->dul, dt, d->st);
  return cuda_rc(e);
}

// step_forwardeuler! (src/N.jl:309-318): v = P(v + dt RHS(v)).
int forward_euler(exc_dnsaid* d, exc_poisson* ps, int n, double h, double* v, double* dv, double dt) {
  const long long N3 = 3LL * n * n * n;
  cudaError_t e = launch_rhs<double>(n, h, d->visc, v, dv, false, d->st);
  if (e == cudaSuccess) e = launch_axpy<double>(N3, v, dv, dt, d->st);
  if (e == cudaSuccess) e = project(ps, v, d->st);
  return cuda_rc(e);
}

// One lockstep step (src/N.jl:1295-1320).
int lockstep(exc_dnsaid* d, double dt) {
  const int n = d->n, m = d->m, c = d->c;
  const long long N3 = 3LL * n * n * n, M = (long long)m * m * m;
  cudaStream_t st = d->st;
  // DNS right-hand side, projected; its pressure enters r = sigma + p I.
  cudaError_t e = launch_rhs<double>(n, d->h, d->visc, d->u, d->du, false, st);
  if (e == cudaSuccess) e = project(&d->psd, d->du, st);
  if (e == cudaSuccess) e = copy_pressure<double>(&d->psd, d->p, st);
  if (e != cudaSuccess) return cuda_rc(e);
  int rc = closure_flux<double>(n, c, d->l, d->visc, fd(d), nfd(d), d->u, d->p, d->r9, st);
  if (!rc) rc = filtered_stress<double>(n, c, d->l, d->visc, fd(d), nfd(d), d->u, d->sdh, st);
  if (!rc) rc = classic_stress<double>(n, c, d->l, d->visc, fd(d), nfd(d), d->u, d->s2, st);
  if (!rc) rc = apply_dhpi(d, d->ub);
  if (rc) return rc;
  // no model
  rc = forward_euler(d, &d->psl, m, d->H, d->les[0], d->dul, dt);
  if (rc) return rc;
  // classic: sigma_H(v) + sigmaDH - sigma2
  e = launch_stress<double>(m, d->H, d->visc, d->les[1], d->sl, st);
  if (e == cudaSuccess) { combine6_kernel<<<gridsz(6 * M), 256, 0, st>>>(6 * M, d->sl, d->sdh, d->s2, d->sc); e = cudaGetLastError(); }
  if (e != cudaSuccess) return cuda_rc(e);
  rc = les_update(d, d->les[1], d->sc, nullptr, nullptr, dt);
  if (rc) return rc;
  // classic + flux: sigma_H(v) + sigmaDH - sigma_H(ubar)
  e = launch_stress<double>(m, d->H, d->visc, d->ub, d->s2, st);  // sigma_H(ubar) (s2 is free now)
  if (e == cudaSuccess) e = launch_stress<double>(m, d->H, d->visc, d->les[2], d->sl, st);
  if (e == cudaSuccess) { combine6_kernel<<<gridsz(6 * M), 256, 0, st>>>(6 * M, d->sl, d->sdh, d->s2, d->sc); e = cudaGetLastError(); }
  if (e != cudaSuccess) return cuda_rc(e);
  rc = les_update(d, d->les[2], d->sc, nullptr, nullptr, dt);
  if (rc) return rc;
  // classic + flux + div: sigma_H(v) - sigma_H(ubar), plus -div^ns rDHi
  e = launch_stress<double>(m, d->H, d->visc, d->les[3], d->sl, st);
  if (e == cudaSuccess) { combine6_kernel<<<gridsz(6 * M), 256, 0, st>>>(6 * M, d->sl, nullptr, d->s2, d->sc); e = cudaGetLastError(); }
  if (e != cudaSuccess) return cuda_rc(e);
  rc = les_update(d, d->les[3], d->sc, d->r9, nullptr, dt);
  if (rc) return rc;
  // symmetrised: the same with symmetrize(rDHi)
  e = launch_stress<double>(m, d->H, d->visc, d->les[4], d->sl, st);
  if (e == cudaSuccess) { combine6_kernel<<<gridsz(6 * M), 256, 0, st>>>(6 * M, d->sl, nullptr, d->s2, d->sc); e = cudaGetLastError(); }
  if (e == cudaSuccess) { symmetrize_kernel<<<gridsz(M), 256, 0, st>>>(M, d->r9, d->sdh); e = cudaGetLastError(); }
  if (e != cudaSuccess) return cuda_rc(e);
  rc = les_update(d, d->les[4], d->sc, nullptr, d->sdh, dt);
  if (rc) return rc;
  // DNS update (after the LES, which read the current DNS)
  return cuda_rc(launch_axpy<double>(N3, d->u, d->du, dt, st));
}

// `fu` of dns_aid_volavg (src/NavierStokes.jl:169-170, 290-291): the volume
// filter of the DNS, projected when `doproject`; `fiu` of dns_aid_surface
// (src/NavierStokes.jl:333, 449): the face filter, divergence free on the
// LES grid and never projected.
int paper_target(exc_dnsaid* d, double* out) {
  int rc = filter_vector<double>(d->n, d->c, d->surface ? EXC_FILTER_FACE : EXC_FILTER_VOLUME, fd(d), nfd(d), d->u,
                                 out, d->st);
  if (rc || !d->doproject || d->surface) return rc;
  return cuda_rc(project(&d->psl, out, d->st));
}

// One step of dns_aid_volavg (src/NavierStokes.jl:186-288) or of
// dns_aid_surface (src/NavierStokes.jl:350-452).
int lockstep_paper(exc_dnsaid* d, double dt) {
  const int n = d->n, m = d->m, c = d->c;
  const long long N3 = 3LL * n * n * n, M = (long long)m * m * m;
  cudaStream_t st = d->st;
  // DNS right-hand side, projected; its pressure enters r = sigma + p I
  cudaError_t e = launch_rhs<double>(n, d->h, d->visc, d->u, d->du, false, st);
  if (e == cudaSuccess) e = project(&d->psd, d->du, st);
  if (e == cudaSuccess) e = copy_pressure<double>(&d->psd, d->p, st);
  if (e != cudaSuccess) return cuda_rc(e);
  // volume: fru = volume-filtered r (sdh), firu = face-filtered r (r9);
  // surface: firu = surface-filtered r (rc9), swap flux = firu on the
  // diagonal, line-filtered r off it (r9)
  int rc;
  if (d->surface) {
    rc = surface_flux<double>(n, c, d->l, d->visc, fd(d), nfd(d), d->u, d->p, d->rc9, false, st);
    if (!rc) rc = surface_flux<double>(n, c, d->l, d->visc, fd(d), nfd(d), d->u, d->p, d->r9, true, st);
  } else {
    rc = filtered_stress<double>(n, c, d->l, d->visc, fd(d), nfd(d), d->u, d->sdh, st, d->p);
    if (!rc) rc = closure_flux<double>(n, c, d->l, d->visc, fd(d), nfd(d), d->u, d->p, d->r9, st);
  }
  // fu and rfu = sigma_H(fu) + p_H I, p_H from the LES right-hand side of fu
  if (!rc) rc = paper_target(d, d->ub);
  if (rc) return rc;
  e = launch_stress<double>(m, d->H, d->visc, d->ub, d->sl, st);
  if (e == cudaSuccess) e = launch_tensordiv<double>(m, d->H, 6, d->sl, d->dul, false, st);
  if (e == cudaSuccess) e = poisson_solve_inplace<double>(&d->psl, d->dul, true, st);
  if (e == cudaSuccess) e = copy_pressure<double>(&d->psl, d->pl, st);
  if (e == cudaSuccess) { add_diag_kernel<<<gridsz(M), 256, 0, st>>>(M, d->sl, d->pl); e = cudaGetLastError(); }
  // closures: classic fru - rfu (sc; surface: firu - rfiu in rc9), swap
  // firu - rfu (r9), its symmetric part (sdh)
  if (e == cudaSuccess && !d->surface) { combine6_kernel<<<gridsz(6 * M), 256, 0, st>>>(6 * M, d->sdh, nullptr, d->sl, d->sc); e = cudaGetLastError(); }
  if (e == cudaSuccess && d->surface) { sub_sym_kernel<<<gridsz(M), 256, 0, st>>>(M, d->rc9, d->sl); e = cudaGetLastError(); }
  if (e == cudaSuccess) { sub_sym_kernel<<<gridsz(M), 256, 0, st>>>(M, d->r9, d->sl); e = cudaGetLastError(); }
  if (e == cudaSuccess) { symmetrize_kernel<<<gridsz(M), 256, 0, st>>>(M, d->r9, d->sdh); e = cudaGetLastError(); }
  // DNS step
  if (e == cudaSuccess) e = launch_axpy<double>(N3, d->u, d->du, dt, st);
  if (e != cudaSuccess) return cuda_rc(e);
  // no model: v += dt P(RHS_H(v))
  e = launch_stress<double>(m, d->H, d->visc, d->les[0], d->sl, st);
  if (e != cudaSuccess) return cuda_rc(e);
  rc = les_update(d, d->les[0], d->sl, nullptr, nullptr, dt);
  // classic, swap, swap-symmetric: v += dt P(RHS_H(v)); v += dt dsigma; project
  const double* sig[3] = {d->surface ? d->rc9 : d->sc, d->r9, d->sdh};
  const int ncomp[3] = {d->surface ? 9 : 6, 9, 6};
  for (int k = 0; k < 3 && !rc; ++k) {
    double* v = d->les[k + 1];
    e = launch_stress<double>(m, d->H, d->visc, v, d->sl, st);
    if (e != cudaSuccess) return cuda_rc(e);
    rc = les_update(d, v, d->sl, nullptr, nullptr, dt);
    if (rc) return rc;
    e = launch_tensordiv<double>(m, d->H, ncomp[k], sig[k], d->dsig, false, st);
    if (e == cudaSuccess) e = launch_axpy<double>(3 * M, v, d->dsig, dt, st);
    if (e == cudaSuccess && d->doproject) e = project(&d->psl, v, st);
    if (e != cudaSuccess) return cuda_rc(e);
  }
  return rc;
}

template <typename P>
int dalloc(P** p, size_t count) {
  if (cudaMalloc(p, count * sizeof(P)) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    set_last_error("device allocation failed");
    return EXC_ERR_OOM;
  }
  return EXC_OK;
}

}  // namespace
}  // namespace exc

using namespace exc;

extern "C" {

int exc_dnsaid_create(const exc_dnsaid_desc* desc, void* stream, exc_dnsaid** out) {
  if (!desc || !out) { set_last_error("null argument"); return EXC_ERR_ARG; }
  *out = nullptr;
  const int n = desc->n, c = desc->ratio;
  if (!fft_size_ok(n)) { set_last_error("grid size must be 2^a 3^b 5^c 7^d 11^e 13^f 17^g, a >= 1, 4 <= n <= 1024"); return EXC_ERR_SHAPE; }
  if (c < 1 || n % c) { set_last_error("ratio must divide n"); return EXC_ERR_RATIO; }
  if (!fft_size_ok(n / c)) { set_last_error("LES grid n/ratio must be an FFT size"); return EXC_ERR_SHAPE; }
  if (!(desc->l > 0) || !(desc->visc > 0)) { set_last_error("l and visc must be positive"); return EXC_ERR_ARG; }
  if (desc->nfdelta > 1 && (!desc->fdelta || desc->nfdelta % 2 == 0)) { set_last_error("fdelta must have odd length"); return EXC_ERR_ARG; }
  int rc = configure_device();
  if (rc) return rc;
  exc_dnsaid* d = new exc_dnsaid();
  d->n = n;
  d->c = c;
  d->m = n / c;
  d->l = desc->l;
  d->visc = desc->visc;
  d->h = desc->l / n;
  d->H = desc->l / d->m;
  if (desc->nfdelta > 1) d->fdelta.assign(desc->fdelta, desc->fdelta + desc->nfdelta);
  d->st = (cudaStream_t)stream;
  const size_t N = (size_t)n * n * n, M = (size_t)d->m * d->m * d->m;
  const size_t spec = 3ull * n * n * spec_pitch(n) * 2;  // 3 complex spectral arrays, in doubles
  rc = poisson_init(&d->psd, EXC_F64, n, d->l, nullptr);
  if (!rc) rc = poisson_init(&d->psl, EXC_F64, d->m, d->l, nullptr);
  if (!rc) rc = dalloc(&d->u, 3 * N) || dalloc(&d->du, 3 * N) || dalloc(&d->p, N) || dalloc(&d->ub, 3 * M) ||
                dalloc(&d->dul, 3 * M) || dalloc(&d->sdh, 6 * M) || dalloc(&d->s2, 6 * M) || dalloc(&d->r9, 9 * M) ||
                dalloc(&d->sl, 6 * M) || dalloc(&d->sc, 6 * M) || dalloc(&d->zero, M) || dalloc(&d->scal, 16) ||
                dalloc(&d->part, (size_t)SHELL_BLOCKS * 1024 + 2048 + RED_PARTS) || dalloc(&d->spec, spec);
  for (int k = 0; k < 5 && !rc; ++k) rc = dalloc(&d->les[k], 3 * M);
  if (!rc) rc = dalloc(&d->pl, M) || dalloc(&d->dsig, 3 * M);
  if (rc) { exc_dnsaid_destroy(d); return rc; }
  cudaMemsetAsync(d->zero, 0, M * sizeof(double), d->st);
  cudaMemsetAsync(d->u, 0, 3 * N * sizeof(double), d->st);
  rc = cuda_rc(cudaGetLastError());
  if (rc) { exc_dnsaid_destroy(d); return rc; }
  *out = d;
  return EXC_OK;
}

int exc_dnsaid_destroy(exc_dnsaid* d) {
  if (!d) return EXC_OK;
  if (d->st) cudaStreamSynchronize(d->st); else cudaDeviceSynchronize();
  poisson_free(&d->psd);
  poisson_free(&d->psl);
  double* bufs[] = {d->u, d->du, d->p, d->ub, d->dul, d->sdh, d->s2, d->r9, d->sl, d->sc, d->zero, d->scal,
                    d->part, d->spec, d->pl, d->dsig, d->rc9};
  for (double* b : bufs) cudaFree(b);
  for (double* b : d->les) cudaFree(b);
  delete d;
  return EXC_OK;
}

int exc_dnsaid_init_random(exc_dnsaid* d, int profile, double param, double energy, uint64_t seed) {
  if (!d || (profile != EXC_PROFILE_PEAK && profile != EXC_PROFILE_POWER) || !(energy > 0) ||
      (profile == EXC_PROFILE_PEAK && !(param > 0))) {
    set_last_error("bad profile, parameter or energy");
    return EXC_ERR_ARG;
  }
  int rc = init_random_field<double>(&d->psd, d->u, reinterpret_cast<double2*>(d->spec), d->part, param, energy, seed,
                                     d->st, profile);
  if (rc) return rc;
  d->t = 0;
  d->steps = 0;
  d->started = false;
  return cuda_rc(cudaStreamSynchronize(d->st));
}

int exc_dnsaid_set_velocity(exc_dnsaid* d, const double* host) {
  if (!d || !host) { set_last_error("null argument"); return EXC_ERR_ARG; }
  const size_t N = (size_t)d->n * d->n * d->n;
  cudaError_t e = cudaMemcpyAsync(d->u, host, 3 * N * sizeof(double), cudaMemcpyHostToDevice, d->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
  d->t = 0;
  d->steps = 0;
  d->started = false;
  return cuda_rc(e);
}

int exc_dnsaid_get_velocity(exc_dnsaid* d, double* host) {
  if (!d || !host) { set_last_error("null argument"); return EXC_ERR_ARG; }
  const size_t N = (size_t)d->n * d->n * d->n;
  cudaError_t e = cudaMemcpyAsync(host, d->u, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, d->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
  return cuda_rc(e);
}

int exc_dnsaid_warmup(exc_dnsaid* d, double twarm, double cfl, int max_steps, int* steps) {
  if (!d || !(cfl > 0)) { set_last_error("null handle or bad cfl"); return EXC_ERR_ARG; }
  if (d->started) { set_last_error("warm-up must come before exc_dnsaid_start"); return EXC_ERR_STATE; }
  int it = 0;
  while (d->t < twarm && (max_steps <= 0 || it < max_steps)) {
    double dt;
    int rc = propose_dt(d, cfl, &dt);
    if (rc) return rc;
    dt = dt < twarm - d->t ? dt : twarm - d->t;
    d->t += dt;
    ++it;
    rc = forward_euler(d, &d->psd, d->n, d->h, d->u, d->du, dt);
    if (rc) return rc;
  }
  d->steps += it;
  if (steps) *steps = it;
  return cuda_rc(cudaStreamSynchronize(d->st));
}

int exc_dnsaid_set_paper(exc_dnsaid* d, int doproject) {
  if (!d) { set_last_error("null handle"); return EXC_ERR_ARG; }
  if (d->started) { set_last_error("the driver is chosen before exc_dnsaid_start"); return EXC_ERR_STATE; }
  d->paper = true;
  d->surface = false;
  d->doproject = doproject != 0;
  return EXC_OK;
}

int exc_dnsaid_set_surface(exc_dnsaid* d, int doproject) {
  if (!d) { set_last_error("null handle"); return EXC_ERR_ARG; }
  if (d->started) { set_last_error("the driver is chosen before exc_dnsaid_start"); return EXC_ERR_STATE; }
  if (!d->rc9) {
    int rc = dalloc(&d->rc9, 9ull * d->m * d->m * d->m);
    if (rc) return rc;
  }
  d->paper = true;
  d->surface = true;
  d->doproject = doproject != 0;
  return EXC_OK;
}

int exc_dnsaid_start(exc_dnsaid* d) {
  if (!d) { set_last_error("null handle"); return EXC_ERR_ARG; }
  if (!d->paper && d->c % 2 == 0) {
    set_last_error("dnsaid_project's classic closure needs an odd ratio (its fine-grid filter is odd-only)");
    return EXC_ERR_RATIO;
  }
  int rc = d->paper ? paper_target(d, d->ub) : apply_dhpi(d, d->ub);
  if (rc) return rc;
  const size_t M3 = 3ull * d->m * d->m * d->m;
  for (int k = 0; k < 5; ++k) {
    cudaError_t e = cudaMemcpyAsync(d->les[k], d->ub, M3 * sizeof(double), cudaMemcpyDeviceToDevice, d->st);
    if (e != cudaSuccess) return cuda_rc(e);
  }
  d->t = 0;
  d->steps = 0;
  d->started = true;
  return cuda_rc(cudaStreamSynchronize(d->st));
}

int exc_dnsaid_step(exc_dnsaid* d, double tstop, double cfl, int max_steps, int* steps) {
  if (!d || !(cfl > 0)) { set_last_error("null handle or bad cfl"); return EXC_ERR_ARG; }
  if (!d->started) { set_last_error("call exc_dnsaid_start first"); return EXC_ERR_STATE; }
  int it = 0;
  while (d->t < tstop && (max_steps <= 0 || it < max_steps)) {
    double dt;
    int rc = propose_dt(d, cfl, &dt);
    if (rc) return rc;
    dt = dt < tstop - d->t ? dt : tstop - d->t;
    d->t += dt;
    ++it;
    rc = d->paper ? lockstep_paper(d, dt) : lockstep(d, dt);
    if (rc) return rc;
  }
  d->steps += it;
  if (steps) *steps = it;
  return cuda_rc(cudaStreamSynchronize(d->st));
}

int exc_dnsaid_time(exc_dnsaid* d, double* t, int* steps) {
  if (!d) { set_last_error("null handle"); return EXC_ERR_ARG; }
  if (t) *t = d->t;
  if (steps) *steps = d->steps;
  return EXC_OK;
}

int exc_dnsaid_get(exc_dnsaid* d, int which, double* host) {
  if (!d || !host) { set_last_error("null argument"); return EXC_ERR_ARG; }
  if (which < 0 || which > 5) { set_last_error("which must be 0..5"); return EXC_ERR_ARG; }
  const size_t M3 = 3ull * d->m * d->m * d->m;
  const double* src;
  if (which == 0) {
    int rc = d->paper ? paper_target(d, d->ub) : apply_dhpi(d, d->ub);
    if (rc) return rc;
    src = d->ub;
  } else {
    if (!d->started) { set_last_error("call exc_dnsaid_start first"); return EXC_ERR_STATE; }
    src = d->les[which - 1];
  }
  cudaError_t e = cudaMemcpyAsync(host, src, M3 * sizeof(double), cudaMemcpyDeviceToHost, d->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
  return cuda_rc(e);
}

int exc_dnsaid_errors(exc_dnsaid* d, double out[5]) {
  if (!d || !out) { set_last_error("null argument"); return EXC_ERR_ARG; }
  if (!d->started) { set_last_error("call exc_dnsaid_start first"); return EXC_ERR_STATE; }
  int rc = d->paper ? paper_target(d, d->ub) : apply_dhpi(d, d->ub);
  if (rc) return rc;
  const int nles = d->paper ? 4 : 5;
  if (d->paper) out[4] = 0;
  const long long M = (long long)d->m * d->m * d->m;
  double* part = d->part + SHELL_BLOCKS * 1024 + 2048;
  // scal[0..2]: sum b_i^2; scal[3 + 3k + i]: sum (a_ki - b_i)^2
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 3 && e == cudaSuccess; ++i) e = launch_sqdiff<double>(M, d->ub + i * M, d->zero, part, d->scal + i, d->st);
  double hs[3];
  if (e == cudaSuccess) e = cudaMemcpyAsync(hs, d->scal, sizeof(hs), cudaMemcpyDeviceToHost, d->st);
  for (int k = 0; k < nles && e == cudaSuccess; ++k) {
    double ha[3];
    for (int i = 0; i < 3 && e == cudaSuccess; ++i)
      e = launch_sqdiff<double>(M, d->les[k] + i * M, d->ub + i * M, part, d->scal + 3 + i, d->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ha, d->scal + 3, sizeof(ha), cudaMemcpyDeviceToHost, d->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
    // `compute_errors` (src/N.jl:1334-1349): sqrt(mean_i |a_i - b_i|^2 / |b_i|^2)
    if (e == cudaSuccess) out[k] = std::sqrt((ha[0] / hs[0] + ha[1] / hs[1] + ha[2] / hs[2]) / 3);
  }
  return cuda_rc(e);
}

int exc_dnsaid_relerr(exc_dnsaid* d, double out[4]) {
  if (!d || !out) { set_last_error("null argument"); return EXC_ERR_ARG; }
  if (!d->started || !d->paper) { set_last_error("call exc_dnsaid_set_paper/set_surface and exc_dnsaid_start first"); return EXC_ERR_STATE; }
  int rc = paper_target(d, d->ub);
  if (rc) return rc;
  const long long M = (long long)d->m * d->m * d->m;
  double* part = d->part + SHELL_BLOCKS * 1024 + 2048;
  // scal[0]: |fu|^2; scal[1 + k]: |v_k - fu|^2, each over the 3 M words
  cudaError_t e = launch_sqdiff<double>(3 * M, d->ub, nullptr, part, d->scal, d->st);
  for (int k = 0; k < 4 && e == cudaSuccess; ++k)
    e = launch_sqdiff<double>(3 * M, d->les[k], d->ub, part, d->scal + 1 + k, d->st);
  double hs[5];
  if (e == cudaSuccess) e = cudaMemcpyAsync(hs, d->scal, sizeof(hs), cudaMemcpyDeviceToHost, d->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
  if (e == cudaSuccess)
    for (int k = 0; k < 4; ++k) out[k] = std::sqrt(hs[1 + k] / hs[0]);
  return cuda_rc(e);
}

}  // extern "C"
