// Internal interfaces shared by the translation units of libexc.
#pragma once
#include "exc_common.cuh"
#include "fft.cuh"

// The FFT Poisson solver (`poissonsolver`, src/N.jl:202-220): spectral work
// array, twiddles and plans for one grid.
struct exc_poisson {
  int precision = EXC_F64;
  int n = 0;
  double l = 1.0, h = 1.0;
  int P = 0;               // padded half-axis pitch, complex words
  void* work = nullptr;    // complex [n][n][P]; real view [n][n][2P]
  void* tw = nullptr;      // W_n^m, m < n (precision's complex type)
  double* sin2 = nullptr;  // sin^2(pi k / n), k < n
  double* invlap = nullptr;  // 1/(lambda N) per mode at invlap_index (FP32 solvers: float (hi, lo) pairs), or null
  exc::FftPlan plan_n{}, plan_h{};
  bool external_work = false;
  int col_w = 0, x_rows = 0;  // tuned launch geometry of the shared-memory passes (0 = default)
  // register-resident passes (fftreg.cuh): level twiddle tables of the
  // column lines (L = n) and the x lines (L = n/2), null when the grid has
  // no register plan; engine 0 uses them when present, 1 forces the
  // shared-memory passes
  void* twl_n = nullptr;
  void* twl_h = nullptr;
  // engine 0: the mixed-precision solve where built (FP64 grids with an FP32
  // register plan, fftmix.cu), else the register passes, else Stockham;
  // 1: the FP64 shared-memory Stockham passes; 2: the FP64 register passes
  // where planned, else Stockham (no mixed precision)
  int engine = 0;
  // mixed-precision FP64 solve (fftmix.cuh): the FP32 inner solver (its own
  // work array and tables, 1/(lambda N h) divide table), the FP64 divergence
  // (n^3, unscaled by 1/h; the first residual replaces it), the first two
  // FP32 corrections (n^3 floats each) and per-CTA partial sums of p with
  // the mean last
  exc_poisson* mix = nullptr;
  double* mix_d = nullptr;
  float* mix_q = nullptr;
  float* mix_q2 = nullptr;
  double* mix_part = nullptr;
  // remove the pressure's mean (its free constant) in the mixed solve; false
  // where p is only used through its gradient
  bool mix_zero_mean = true;
};

namespace exc {

// Entry of mode (kz, ky, kx) in the 1/(lambda N) table: lambda depends on
// sin^2(pi k/n), even in k, so ky and kz fold to min(k, n - k) and the table
// holds (n/2 + 1)^3 entries [kz][ky][kx].
__host__ __device__ __forceinline__ long long invlap_index(int n, int kz, int ky, int kx) {
  const int h = n / 2;
  const int fz = kz <= h ? kz : n - kz, fy = ky <= h ? ky : n - ky;
  return ((long long)fz * (h + 1) + fy) * (h + 1) + kx;
}

// Allocate/free the device tables of a solver; `work` may be supplied by the
// caller (external_work) and is otherwise allocated here.
int poisson_init(exc_poisson* ps, int precision, int n, double l, void* work);
void poisson_free(exc_poisson* ps);

// Pressure solve into the real view of ps->work (pitch 2P):
//   src_is_vector: d = div(src) computed on the fly (scaled by 1/h),
//   otherwise src is the scalar right-hand side d.
template <typename T>
cudaError_t poisson_solve_inplace(exc_poisson* ps, const T* src, bool src_is_vector, cudaStream_t st,
                                  const SlotBatch& sb = SlotBatch(), int nslots = 1);

// The same solve on the register-resident passes (fftreg_f32.cu,
// fftreg_f64.cu); only for grids with fftreg_supported(n, precision).
bool fftreg_supported(int n, int precision);
int reg_split_host(int L);  // first factor N1 of a line length L with a register plan, else 0
cudaError_t fftreg_solve(exc_poisson* ps, const float* src, bool src_is_vector, cudaStream_t st, const SlotBatch& sb,
                         int nslots);
cudaError_t fftreg_solve(exc_poisson* ps, const double* src, bool src_is_vector, cudaStream_t st, const SlotBatch& sb,
                         int nslots);
// The mixed-precision FP64 solve (fftmix.cu): grids it is built for, the
// doubles of partial sums it needs, the solve (pressure into the FP64 real
// view of ps->work, like poisson_solve_inplace) and its shared-memory opt-ins.
bool fftmix_supported(int n);
long long fftmix_part_words(int n);
cudaError_t fftmix_solve(exc_poisson* ps, const double* src, bool src_is_vector, cudaStream_t st);
cudaError_t configure_fftmix();
// Lines per column tile and rows per x-pass CTA of a grid's register plan.
void fftreg_geometry(int n, int precision, int* col_w, int* x_rows);
// Read and clear the learned closure's tensor-core wait fault flag.
int learned_fault_take(int* flag);
// Set the tensor-core convolution's wait drill (exc_debug_wait_drill bit 1).
int learned_set_drill(int on);
cudaError_t configure_fftreg_f32();
cudaError_t configure_fftreg_f64();

// Plain forward (half spectrum into ps->work) and unnormalised inverse (reals
// at pitch 2P in ps->work) 3-D transforms.
template <typename T>
cudaError_t fft3d_forward(exc_poisson* ps, const T* src, cudaStream_t st);
template <typename T>
cudaError_t fft3d_inverse(exc_poisson* ps, cudaStream_t st);

// Random solenoidal field with a shell spectrum into u (init.cu); spec3: 3
// spectral arrays of scratch, part: SHELL_BLOCKS*1024 + 2048 doubles.
// profile 0: peak profile with k0 = kpeak; 1: power law (k > 0) k^kpeak.
template <typename T>
int init_random_field(exc_poisson* ps, T* u, cplx<T>* spec3, double* part, double kpeak, double energy,
                      uint64_t seed, cudaStream_t st, int profile = 0);

// Learned-closure network internals used by the case stepper (learned.cu).
int net_reserve(exc_net* net, long long V);
int net_workspace_gen(const exc_net* net);

// Shared-memory opt-ins of every kernel that needs them, once per device;
// called before any launch (and so before any stream capture).
int configure_device();
cudaError_t configure_fft();
cudaError_t configure_stencil();
cudaError_t configure_fields();

// Copy the pressure from the work array (pitch 2P) to a dense n^3 field.
template <typename T>
cudaError_t copy_pressure(const exc_poisson* ps, T* p, cudaStream_t st);

// ---- stencil kernels (stencil.cu) ----
// pre_shifted (FP64): u holds the sweep's shifted form (fp64_shift), as the
// RK stage kernel stores it on request
template <typename T>
cudaError_t launch_rhs(int n, T h, T visc, const T* u, T* du, bool doadd, cudaStream_t st,
                       const SlotBatch& sb = SlotBatch(), int nslots = 1, bool pre_shifted = false);
template <typename T>
cudaError_t launch_stress(int n, T h, T visc, const T* u, T* s6, cudaStream_t st);
template <typename T>
cudaError_t launch_tensordiv(int n, T h, int nsym, const T* s, T* du, bool doadd, cudaStream_t st);
template <typename T>
cudaError_t launch_divergence(int n, T h, const T* u, T* d, cudaStream_t st);
// u_i -= (p[I+e_i] - p[I]) / h with p read at row pitch `ppitch` words.
template <typename T>
cudaError_t launch_gradient(int n, T h, T* u, const T* p, int ppitch, cudaStream_t st);
template <typename T>
cudaError_t launch_max_abs(size_t count, const T* x, double* out_dev, double* partial, int npartial,
                           cudaStream_t st);

}  // namespace exc
