// Register-resident FFT Poisson solve, FP32 instantiations (grids 32..1024),
// and the mixed-precision FP64 solve built on them (fftmix.cuh).
#include "fftmix.cuh"
#include "fftreg.cuh"

namespace exc {

// Grids n with register plans for both the columns (L = n) and the x lines
// (L = n/2): FP32 up to 1024, FP64 up to 256 (longer FP64 lines exceed the
// register budget of one thread).
int reg_split_host(int L) { return reg_split(L); }

void fftreg_geometry_f64(int n, int* col_w, int* x_rows);
void fftreg_geometry_f32(int n, int* col_w, int* x_rows);
void fftreg_geometry(int n, int precision, int* col_w, int* x_rows) {
  if (precision == EXC_F32) fftreg_geometry_f32(n, col_w, x_rows);
  else fftreg_geometry_f64(n, col_w, x_rows);
}

bool fftreg_supported(int n, int precision) {
  if (n < 4 || (n & 1) || !reg_split(n) || !reg_split(n / 2)) return false;
  return precision == EXC_F32 ? n <= 1024 : n <= 256;
}

#define EXC_REG_SIZES_F32(X) X(32) X(48) X(64) X(96) X(128) X(192) X(256) X(384) X(512) X(1024)

cudaError_t fftreg_solve(exc_poisson* ps, const float* src, bool vec, cudaStream_t st, const SlotBatch& sb,
                         int ns) {
  switch (ps->n) {
#define EXC_CASE(N) \
  case N: return RegSolve<float, N>::solve(ps, src, vec, st, sb, ns);
    EXC_REG_SIZES_F32(EXC_CASE)
#undef EXC_CASE
    default: return cudaErrorInvalidValue;
  }
}

void fftreg_geometry_f32(int n, int* col_w, int* x_rows) {
  switch (n) {
#define EXC_GEOM(N) \
  case N:                                          \
    *col_w = RegSolve<float, N>::CG::W;              \
    *x_rows = RegSolve<float, N>::XG::RW;            \
    return;
    EXC_REG_SIZES_F32(EXC_GEOM)
#undef EXC_GEOM
    default:
      *col_w = *x_rows = 0;
  }
}

cudaError_t configure_fftreg_f32() {
  cudaError_t e = cudaSuccess;
#define EXC_CONF(N) \
  if (e == cudaSuccess) e = RegSolve<float, N>::configure();
  EXC_REG_SIZES_F32(EXC_CONF)
#undef EXC_CONF
  return e;
}

// ---- mixed-precision FP64 solve (fftmix.cuh) ----
#define EXC_MIX_SIZES(X) X(128) X(192) X(256) X(384) X(512) X(1024)

bool fftmix_supported(int n) {
  switch (n) {
#define EXC_CASE(N) case N:
    EXC_MIX_SIZES(EXC_CASE)
#undef EXC_CASE
    return true;
    default: return false;
  }
}

// Doubles of per-CTA partial sums (plus the mean) the solve of grid n uses.
long long fftmix_part_words(int n) {
  switch (n) {
#define EXC_CASE(N) \
  case N: return MixSolve<N>::PART_WORDS;
    EXC_MIX_SIZES(EXC_CASE)
#undef EXC_CASE
    default: return 0;
  }
}

cudaError_t fftmix_solve(exc_poisson* ps, const double* src, bool vec, cudaStream_t st) {
  switch (ps->n) {
#define EXC_CASE(N) \
  case N: return MixSolve<N>::solve(ps, src, vec, st);
    EXC_MIX_SIZES(EXC_CASE)
#undef EXC_CASE
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t configure_fftmix() {
  cudaError_t e = cudaSuccess;
#define EXC_CONF(N) \
  if (e == cudaSuccess) e = MixSolve<N>::configure();
  EXC_MIX_SIZES(EXC_CONF)
#undef EXC_CONF
  return e;
}

}  // namespace exc
