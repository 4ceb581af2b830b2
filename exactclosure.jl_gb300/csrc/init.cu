// Random solenoidal initial field with a prescribed shell spectrum
// (`randomfield` + `peak_profile`, src/N.jl:366-476), shared by the case
// stepper and the serving loop.
#include <cmath>

#include "internal.cuh"
#include "fields.cuh"

namespace exc {

// u: 3 n^3 words (written); spec3: 3 spectral arrays of ps's shape (scratch);
// part: SHELL_BLOCKS * 1024 + 2048 doubles of scratch.  Enqueues on `st`
// only (no allocation, no synchronisation):
//   normals -> project -> rfft of each component -> shell energies with the
//   rfft conjugate weight -> scale shell k by sqrt(E0(k)/E(k)) -> irfft ->
//   project again (the discrete divergence is not exactly preserved by the
//   rescaling, src/N.jl:464-469).
template <typename T>
int init_random_field(exc_poisson* ps, T* u, cplx<T>* spec3, double* part, double kpeak, double energy,
                      uint64_t seed, cudaStream_t st, int profile) {
  using C = cplx<T>;
  const int n = ps->n, P = ps->P;
  const long long N = (long long)n * n * n;
  const long long cstride = (long long)n * n * P;
  auto project = [&](T* v) -> cudaError_t {
    cudaError_t e = poisson_solve_inplace<T>(ps, v, true, st);
    if (e == cudaSuccess) e = launch_gradient<T>(n, (T)ps->h, v, reinterpret_cast<const T*>(ps->work), 2 * P, st);
    return e;
  };
  cudaError_t e = launch_normals<T>(3 * N, (unsigned long long)seed, u, st);
  if (e == cudaSuccess) e = project(u);
  exc_poisson tmp = *ps;
  for (int c = 0; c < 3 && e == cudaSuccess; ++c) {
    tmp.work = spec3 + c * cstride;
    e = fft3d_forward<T>(&tmp, u + c * N, st);
  }
  const int kdiag = (int)std::floor(std::sqrt(3.0) * (n / 2));
  const int nshell = kdiag + 1;
  double* eshell = part + SHELL_BLOCKS * 1024;  // nshell <= 1024
  double* factor = eshell + 1024;
  const double Nd = (double)N;
  if (e == cudaSuccess)
    e = launch_shell_energy<T>(n, P, 3, spec3, cstride, 1.0 / (Nd * Nd), nshell, part, SHELL_BLOCKS, eshell, st);
  if (e == cudaSuccess) e = launch_shell_factor(nshell, profile, kpeak, energy, eshell, factor, st);
  if (e == cudaSuccess) e = launch_shell_scale<T>(n, P, 3, spec3, cstride, nshell, factor, st);
  for (int c = 0; c < 3 && e == cudaSuccess; ++c) {
    tmp.work = spec3 + c * cstride;
    e = fft3d_inverse<T>(&tmp, st);
    if (e == cudaSuccess)
      e = launch_unpitch<T>(n, reinterpret_cast<const T*>(tmp.work), 2 * P, u + c * N, (T)(1.0 / Nd), st);
  }
  if (e == cudaSuccess) e = project(u);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

template int init_random_field<double>(exc_poisson*, double*, double2*, double*, double, double, uint64_t,
                                       cudaStream_t, int);
template int init_random_field<float>(exc_poisson*, float*, float2*, double*, double, double, uint64_t, cudaStream_t,
                                      int);

}  // namespace exc
