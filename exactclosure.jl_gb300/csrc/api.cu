// Operator-level C ABI (device pointers owned by the caller); see include/exc.h.
#include <mutex>
#include <string>

#include "internal.cuh"
#include "fields.cuh"
#include "filter.cuh"

namespace exc {

static thread_local std::string g_last_error = "no error";
void set_last_error(const char* msg) { g_last_error = msg ? msg : "unknown error"; }

int configure_device() {
  static std::mutex mu;
  static bool done[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    set_last_error("no usable CUDA device");
    return EXC_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (done[dev]) return EXC_OK;
  cudaError_t e = configure_fft();
  if (e == cudaSuccess) e = configure_stencil();
  if (e == cudaSuccess) e = configure_fields();
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  done[dev] = true;
  return EXC_OK;
}

static int check_grid(int precision, int n, double l) {
  if (precision != EXC_F64 && precision != EXC_F32) { set_last_error("precision must be EXC_F64 or EXC_F32"); return EXC_ERR_ARG; }
  if (!fft_size_ok(n)) { set_last_error("grid size must be 2^a 3^b 5^c 7^d 11^e 13^f 17^g, a >= 1, 4 <= n <= 1024"); return EXC_ERR_SHAPE; }
  if (!(l > 0)) { set_last_error("domain size must be positive"); return EXC_ERR_ARG; }
  return configure_device();
}

static int cuda_status(cudaError_t e) {
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

}  // namespace exc

using namespace exc;

#define BY_PRECISION(prec, expr_d, expr_f) ((prec) == EXC_F64 ? (expr_d) : (expr_f))

extern "C" {

const char* exc_last_error(void) { return g_last_error.c_str(); }
int exc_version(void) { return 100; }

int exc_tensordivergence(int precision, int n, double l, double visc, const void* u, void* du, int doadd,
                         void* stream) {
  int rc = check_grid(precision, n, l);
  if (rc) return rc;
  if (!u || !du) { set_last_error("null field pointer"); return EXC_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  double h = l / n;
  return cuda_status(BY_PRECISION(precision,
      launch_rhs<double>(n, h, visc, (const double*)u, (double*)du, doadd != 0, st),
      launch_rhs<float>(n, (float)h, (float)visc, (const float*)u, (float*)du, doadd != 0, st)));
}

int exc_tensordivergence_tensor(int precision, int n, double l, int nsym, const void* s, void* du, int doadd,
                                void* stream) {
  int rc = check_grid(precision, n, l);
  if (rc) return rc;
  if (!s || !du) { set_last_error("null field pointer"); return EXC_ERR_ARG; }
  if (nsym != 6 && nsym != 9) { set_last_error("nsym must be 6 or 9"); return EXC_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  double h = l / n;
  return cuda_status(BY_PRECISION(precision,
      launch_tensordiv<double>(n, h, nsym, (const double*)s, (double*)du, doadd != 0, st),
      launch_tensordiv<float>(n, (float)h, nsym, (const float*)s, (float*)du, doadd != 0, st)));
}

int exc_stresstensor(int precision, int n, double l, double visc, const void* u, void* s6, void* stream) {
  int rc = check_grid(precision, n, l);
  if (rc) return rc;
  if (!u || !s6) { set_last_error("null field pointer"); return EXC_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  double h = l / n;
  return cuda_status(BY_PRECISION(precision,
      launch_stress<double>(n, h, visc, (const double*)u, (double*)s6, st),
      launch_stress<float>(n, (float)h, (float)visc, (const float*)u, (float*)s6, st)));
}

int exc_divergence(int precision, int n, double l, const void* u, void* d, void* stream) {
  int rc = check_grid(precision, n, l);
  if (rc) return rc;
  if (!u || !d) { set_last_error("null field pointer"); return EXC_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  double h = l / n;
  return cuda_status(BY_PRECISION(precision,
      launch_divergence<double>(n, h, (const double*)u, (double*)d, st),
      launch_divergence<float>(n, (float)h, (const float*)u, (float*)d, st)));
}

int exc_pressuregradient(int precision, int n, double l, void* u, const void* p, void* stream) {
  int rc = check_grid(precision, n, l);
  if (rc) return rc;
  if (!u || !p) { set_last_error("null field pointer"); return EXC_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  double h = l / n;
  return cuda_status(BY_PRECISION(precision,
      launch_gradient<double>(n, h, (double*)u, (const double*)p, n, st),
      launch_gradient<float>(n, (float)h, (float*)u, (const float*)p, n, st)));
}

int exc_poisson_create(int precision, int n, double l, exc_poisson** out) {
  if (!out) { set_last_error("null output pointer"); return EXC_ERR_ARG; }
  *out = nullptr;
  int rc = check_grid(precision, n, l);
  if (rc) return rc;
  exc_poisson* ps = new exc_poisson();
  rc = poisson_init(ps, precision, n, l, nullptr);
  if (rc) { delete ps; return rc; }
  *out = ps;
  return EXC_OK;
}

int exc_poisson_destroy(exc_poisson* ps) {
  if (!ps) return EXC_OK;
  cudaDeviceSynchronize();
  poisson_free(ps);
  delete ps;
  return EXC_OK;
}

int exc_poisson_set_engine(exc_poisson* ps, int engine) {
  if (!ps) { set_last_error("null solver"); return EXC_ERR_ARG; }
  if (engine < 0 || engine > 2) {
    set_last_error("engine must be 0 (default), 1 (Stockham passes) or 2 (register passes, no mixed precision)");
    return EXC_ERR_ARG;
  }
  ps->engine = engine;
  return EXC_OK;
}

int exc_poisson_solve(exc_poisson* ps, const void* d, void* p, void* stream) {
  if (!ps || !d || !p) { set_last_error("null argument"); return EXC_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  if (ps->precision == EXC_F64) {
    e = poisson_solve_inplace<double>(ps, (const double*)d, false, st);
    if (e == cudaSuccess) e = copy_pressure<double>(ps, (double*)p, st);
  } else {
    e = poisson_solve_inplace<float>(ps, (const float*)d, false, st);
    if (e == cudaSuccess) e = copy_pressure<float>(ps, (float*)p, st);
  }
  return cuda_status(e);
}

int exc_project(exc_poisson* ps, void* u, void* p_out, void* stream) {
  if (!ps || !u) { set_last_error("null argument"); return EXC_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  if (ps->precision == EXC_F64) {
    e = poisson_solve_inplace<double>(ps, (const double*)u, true, st);
    if (e == cudaSuccess) e = launch_gradient<double>(ps->n, ps->h, (double*)u, (const double*)ps->work, 2 * ps->P, st);
    if (e == cudaSuccess && p_out) e = copy_pressure<double>(ps, (double*)p_out, st);
  } else {
    e = poisson_solve_inplace<float>(ps, (const float*)u, true, st);
    if (e == cudaSuccess) e = launch_gradient<float>(ps->n, (float)ps->h, (float*)u, (const float*)ps->work, 2 * ps->P, st);
    if (e == cudaSuccess && p_out) e = copy_pressure<float>(ps, (float*)p_out, st);
  }
  return cuda_status(e);
}

int exc_max_abs(int precision, size_t count, const void* x, double* out_dev, void* stream) {
  if (!x || !out_dev || count == 0) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  if (precision != EXC_F64 && precision != EXC_F32) { set_last_error("bad precision"); return EXC_ERR_ARG; }
  int rc = configure_device();
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  // partials live just after the output slot's 8-byte word is not ours: use a
  // small scratch owned by the library
  static thread_local double* scratch = nullptr;
  static thread_local int scratch_dev = -1;
  int dev = 0;
  cudaGetDevice(&dev);
  if (!scratch || scratch_dev != dev) {
    if (cudaMalloc(&scratch, RED_PARTS * sizeof(double)) != cudaSuccess) { set_last_error("out of device memory"); return EXC_ERR_OOM; }
    scratch_dev = dev;
  }
  return cuda_status(BY_PRECISION(precision,
      launch_max_abs<double>(count, (const double*)x, out_dev, scratch, RED_PARTS, st),
      launch_max_abs<float>(count, (const float*)x, out_dev, scratch, RED_PARTS, st)));
}

int exc_propose_timestep(int precision, int n, double l, double visc, double cfl, const void* u, double* dt_host,
                         void* stream) {
  int rc = check_grid(precision, n, l);
  if (rc) return rc;
  if (!u || !dt_host || !(visc > 0) || !(cfl > 0)) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double)) != cudaSuccess) { set_last_error("out of device memory"); return EXC_ERR_OOM; }
  size_t count = 3ull * n * n * n;
  rc = exc_max_abs(precision, count, u, d, stream);
  double umax = 0;
  if (!rc) {
    cudaError_t e = cudaMemcpyAsync(&umax, d, sizeof(double), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    rc = cuda_status(e);
  }
  cudaFree(d);
  if (rc) return rc;
  double h = l / n;
  double dt_adv = cfl * h / umax;
  double dt_visc = cfl * h * h / visc / 6.0;
  *dt_host = dt_adv < dt_visc ? dt_adv : dt_visc;
  return EXC_OK;
}

static int check_filter(int precision, int n, int ratio, int kind, const double* fdelta, int nfdelta) {
  if (precision != EXC_F64 && precision != EXC_F32) { set_last_error("bad precision"); return EXC_ERR_ARG; }
  if (n < 1 || n > 4096) { set_last_error("bad grid size"); return EXC_ERR_SHAPE; }
  if (ratio < 1 || n % ratio != 0) { set_last_error("ratio must divide n"); return EXC_ERR_RATIO; }
  if (kind != EXC_FILTER_VOLUME && kind != EXC_FILTER_FACE) { set_last_error("bad filter kind"); return EXC_ERR_ARG; }
  if (nfdelta > 1 && (!fdelta || nfdelta % 2 == 0)) { set_last_error("fdelta must be an odd-length array"); return EXC_ERR_ARG; }
  return configure_device();
}

int exc_filter(int precision, int n, int ratio, int kind, const double* fdelta, int nfdelta, const void* u,
               void* ubar, void* stream) {
  int rc = check_filter(precision, n, ratio, kind, fdelta, nfdelta);
  if (rc) return rc;
  if (!u || !ubar) { set_last_error("null field pointer"); return EXC_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  return BY_PRECISION(precision,
      filter_vector<double>(n, ratio, kind, fdelta, nfdelta, (const double*)u, (double*)ubar, st),
      filter_vector<float>(n, ratio, kind, fdelta, nfdelta, (const float*)u, (float*)ubar, st));
}

int exc_closure_flux(int precision, int n, int ratio, double l, double visc, const double* fdelta, int nfdelta,
                     const void* u, const void* p, void* r9, void* stream) {
  int rc = check_filter(precision, n, ratio, EXC_FILTER_VOLUME, fdelta, nfdelta);
  if (rc) return rc;
  if (!u || !p || !r9) { set_last_error("null field pointer"); return EXC_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  return BY_PRECISION(precision,
      closure_flux<double>(n, ratio, l, visc, fdelta, nfdelta, (const double*)u, (const double*)p, (double*)r9, st),
      closure_flux<float>(n, ratio, l, visc, fdelta, nfdelta, (const float*)u, (const float*)p, (float*)r9, st));
}

int exc_filtered_stress(int precision, int n, int ratio, double l, double visc, const double* fdelta, int nfdelta,
                        const void* u, void* s6, void* stream) {
  int rc = check_filter(precision, n, ratio, EXC_FILTER_VOLUME, fdelta, nfdelta);
  if (rc) return rc;
  if (!u || !s6) { set_last_error("null field pointer"); return EXC_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  return BY_PRECISION(precision,
      filtered_stress<double>(n, ratio, l, visc, fdelta, nfdelta, (const double*)u, (double*)s6, st),
      filtered_stress<float>(n, ratio, l, visc, fdelta, nfdelta, (const float*)u, (float*)s6, st));
}

}  // extern "C"
