// Register-resident FFT Poisson solve, FP64 instantiations (grids 32..256).
#include "fftreg.cuh"

namespace exc {

#define EXC_REG_SIZES_F64(X) X(32) X(48) X(64) X(96) X(128) X(192) X(256)

cudaError_t fftreg_solve(exc_poisson* ps, const double* src, bool vec, cudaStream_t st, const SlotBatch& sb,
                         int ns) {
  switch (ps->n) {
#define EXC_CASE(N) \
  case N: return RegSolve<double, N>::solve(ps, src, vec, st, sb, ns);
    EXC_REG_SIZES_F64(EXC_CASE)
#undef EXC_CASE
    default: return cudaErrorInvalidValue;
  }
}

void fftreg_geometry_f64(int n, int* col_w, int* x_rows) {
  switch (n) {
#define EXC_GEOM(N) \
  case N:                                          \
    *col_w = RegSolve<double, N>::CG::W;              \
    *x_rows = RegSolve<double, N>::XG::RW;            \
    return;
    EXC_REG_SIZES_F64(EXC_GEOM)
#undef EXC_GEOM
    default:
      *col_w = *x_rows = 0;
  }
}

cudaError_t configure_fftreg_f64() {
  cudaError_t e = cudaSuccess;
#define EXC_CONF(N) \
  if (e == cudaSuccess) e = RegSolve<double, N>::configure();
  EXC_REG_SIZES_F64(EXC_CONF)
#undef EXC_CONF
  return e;
}

}  // namespace exc
