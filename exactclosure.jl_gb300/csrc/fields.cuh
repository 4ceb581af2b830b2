// Pointwise field kernels and deterministic reductions (see fields.cu).
#pragma once
#include "exc_common.cuh"

namespace exc {

constexpr int SHELL_BLOCKS = 152;

// shifted_out (FP64, rk_writes_shifted, with p): the stage state xs is stored
// in the RHS sweep's shifted form for viscosity `visc` (read with pre_shifted)
template <typename T>
cudaError_t launch_rk_stage(int n, T h, T* k, const T* p, int ppitch, const T* x0, T* xs, T* xfin, int stage,
                            const double* dtp, cudaStream_t st, const SlotBatch& sb = SlotBatch(), int nslots = 1,
                            bool store_k = true, bool shifted_out = false, double visc = 0.0);
// Whether the RK stage kernel of this grid can store the shifted form.
template <typename T>
inline bool rk_writes_shifted(int n) {
  return sizeof(T) == 8 && n % 2 == 0;
}
// RK stage (GRAD form, k not stored) that also writes the transverse box sums
// of ratio c0 of k into tbk and of the stage output xs (stages 0-2) into tbs
// (may be null), bit-identical to tb_kernel's (fields.cu); for grids with
// n % rk_sums_chunk<T>(c0) == 0.
template <typename T>
cudaError_t launch_rk_stage_sums(int n, int c0, T h, const T* k, const T* p, int ppitch, const T* x0, T* xs, T* xfin,
                                 int stage, const double* dtp, T* tbk, T* tbs, cudaStream_t st);
// Chunk width (cells per row) of rk_stage_sums_kernel for ratio c0; 0 when
// the fused stage is not used: FP64 (measured slower than the separate
// passes: 512^3 with LES ratios 8 and 4, 103.5 against 101.9 ms per RK4
// step with k's sums only and the stage-state sums by linearity), ratios
// without a kernel, or rows under 128 bytes wide (poorly coalesced).
template <typename T>
inline int rk_sums_chunk(int c0) {
  const int V = 16 / (int)sizeof(T);
  if (sizeof(T) != 4 || (c0 != 2 && c0 != 4 && c0 != 8)) return 0;
  const int xc = 256 * V / (c0 * c0);
  return xc * (int)sizeof(T) >= 128 ? xc : 0;
}


template <typename T>
cudaError_t launch_axpy(long long count, T* a, const T* b, T scale, cudaStream_t st);
cudaError_t launch_set_dt(const double* umax, double h, double visc, double cfl, double fixed, double* dt,
                          double* clock, int* flag, cudaStream_t st);
template <typename T>
cudaError_t launch_normals(long long count, unsigned long long seed, T* out, cudaStream_t st);
template <typename T>
cudaError_t launch_gradsq(int n, const T* u, double* part, double* out, cudaStream_t st);
template <typename T>
cudaError_t launch_sqdiff(long long count, const T* a, const T* b, double* part, double* out, cudaStream_t st);
template <typename T>
cudaError_t launch_shell_energy(int n, int P, int ncomp, const cplx<T>* spec, long long cstride, double scale,
                                int nshell, double* part, int nblocks, double* out, cudaStream_t st);
template <typename T>
cudaError_t launch_shell_scale(int n, int P, int ncomp, cplx<T>* spec, long long cstride, int nshell,
                               const double* factor, cudaStream_t st);
cudaError_t launch_shell_factor(int nshell, int profile, double param, double energy, const double* eshell, double* factor,
                                cudaStream_t st);
template <typename T>
cudaError_t launch_unpitch(int n, const T* src, int pitch, T* dst, T scale, cudaStream_t st);
template <typename A, typename B>
cudaError_t launch_convert(long long count, const A* a, B* b, cudaStream_t st);

constexpr int RED_PARTS = 1216;

}  // namespace exc
