// Projection that allocates nothing: exc_project_noalloc.
//
// Some callers cannot call cudaMalloc: a host whose device memory is owned by
// its own pool (CUDA.jl's or PyTorch's caching allocator) and must not see
// foreign allocations, a loop under a hard memory budget, or code that cannot
// afford the device-wide synchronisation cudaFree implies.  For them this
// entry point runs the same FFT projection as exc_project, but its spectral
// work array and twiddle tables live in one file-scope static device array of
// NOALLOC_SCRATCH_BYTES (4 MiB).  Every GPU that loads the library holds that
// array until the process exits.  The caller still passes u (and optionally
// p).  The array is shared by every call: two calls whose work overlaps on the
// GPU race.  Each call writes every scratch word it reads (tables first, then
// the spectrum) before reading it, so the previous call's contents need no
// clearing.
#include "internal.cuh"

namespace exc {

constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(4) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of the scratch array in the current context, looked up on
// every call (a host-side reference to the symbol is not a device address).
// The lookup is a cheap host call; not caching it keeps the address right
// after a device reset or a new primary context, which reload the module and
// may place the array elsewhere.
static int noalloc_scratch_address(void** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    set_last_error(e != cudaSuccess ? cudaGetErrorString(e) : "cudaGetSymbolAddress returned null");
    return EXC_ERR_CUDA;
  }
  *out = p;
  return EXC_OK;
}

static inline size_t round256(size_t b) { return (b + 255) & ~size_t(255); }

// Bytes of scratch a projection of an n^3 grid needs: spectral array,
// twiddles W_n^m, sin^2 table.
static size_t noalloc_bytes(int n, size_t csz) {
  return round256((size_t)n * n * spec_pitch(n) * csz) + round256((size_t)n * csz) + (size_t)n * sizeof(double);
}

template <typename T>
__global__ void noalloc_tables_kernel(int n, cplx<T>* __restrict__ tw, double* __restrict__ sin2) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(-2.0 * m / n, &s, &c);
    tw[m] = mk<T>((T)c, (T)s);
    double q = sinpi((double)m / n);
    sin2[m] = q * q;
  }
}

template <typename T>
static int project_noalloc(int n, double l, T* u, T* p_out, cudaStream_t st) {
  using C = cplx<T>;
  void* base = nullptr;
  int rc = noalloc_scratch_address(&base);
  if (rc) return rc;
  exc_poisson ps;
  ps.precision = sizeof(T) == 8 ? EXC_F64 : EXC_F32;
  ps.n = n;
  ps.l = l;
  ps.h = l / n;
  ps.P = spec_pitch(n);
  ps.plan_n = make_plan(n);
  ps.plan_h = make_plan(n / 2);
  unsigned char* b = reinterpret_cast<unsigned char*>(base);
  ps.work = b;
  b += round256((size_t)n * n * ps.P * sizeof(C));
  ps.tw = b;
  b += round256((size_t)n * sizeof(C));
  ps.sin2 = reinterpret_cast<double*>(b);
  ps.external_work = true;
  noalloc_tables_kernel<T><<<(n + 127) / 128, 128, 0, st>>>(n, reinterpret_cast<C*>(ps.tw), ps.sin2);
  cudaError_t e = poisson_solve_inplace<T>(&ps, u, true, st);
  if (e == cudaSuccess) e = launch_gradient<T>(n, (T)ps.h, u, reinterpret_cast<const T*>(ps.work), 2 * ps.P, st);
  if (e == cudaSuccess && p_out) e = copy_pressure<T>(&ps, p_out, st);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

}  // namespace exc

using namespace exc;

extern "C" int exc_project_noalloc(int precision, int n, double l, void* u, void* p_out, void* stream) {
  if (precision != EXC_F64 && precision != EXC_F32) { set_last_error("precision must be EXC_F64 or EXC_F32"); return EXC_ERR_ARG; }
  if (!fft_size_ok(n)) { set_last_error("grid size must be 2^a 3^b 5^c 7^d 11^e 13^f 17^g, a >= 1, 4 <= n <= 1024"); return EXC_ERR_SHAPE; }
  if (!(l > 0) || !u) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  const size_t csz = precision == EXC_F64 ? sizeof(double2) : sizeof(float2);
  if (noalloc_bytes(n, csz) > NOALLOC_SCRATCH_BYTES) {
    set_last_error("grid too large for the 4 MiB static scratch of exc_project_noalloc (n <= 72 in FP64, n <= 96 in FP32)");
    return EXC_ERR_SHAPE;
  }
  int rc = configure_device();
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == EXC_F64) return project_noalloc<double>(n, l, (double*)u, (double*)p_out, st);
  return project_noalloc<float>(n, l, (float*)u, (float*)p_out, st);
}
