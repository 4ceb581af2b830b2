// The DNS-aided LES case: one DNS with attached LES grids, advanced with
// classical RK4 and the exact closure evaluated at every stage.
//
// Mirrors the loop of `dnsaid_project` (src/N.jl:1239-1332): each stage s
// computes the projected DNS right-hand side k_s = P_h RHS_h(u_s) (pressure
// from `project!`, src/N.jl:1305-1309); each LES grid gets the filtered
// target ubar_s = P_H filter(u_s) (`apply_DHpi`, src/N.jl:1228-1237; the face
// filter needs no projection), the exact commutator
//   m_s = P_H filter(k_s) - P_H RHS_H(ubar_s)
// (equal to the projected closure of `step_DHpi_classic_flux_div!`,
// src/N.jl:1189-1206, because the box filter along a derivative axis
// telescopes the fine difference), and two LES states advance with it: the
// exact-closure LES (k = P_H RHS_H(v_s) + m_s) and the no-model LES
// (`step_forwardeuler!` on the LES grid, src/N.jl:1315).  The whole step is
// captured once into a CUDA graph (dt lives on the device, so nothing waits
// on the host) and replayed.
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.cuh"
#include "fields.cuh"
#include "filter.cuh"

namespace exc {

template <typename T>
struct LesState {
  int c = 0, kind = 0, m = 0;
  long long M = 0;
  exc_poisson ps;
  T* buf = nullptr;  // one allocation, sliced below (3M words each)
  T* tb = nullptr;   // filter scratch: 3 n (n/c)^2 words (transverse box sums)
  // source of the transverse sums: -1 = the fine field; otherwise LES tb_from,
  // whose ratio divides c (coarsened into tb) or equals it (tb_same: its
  // buffer is used as is)
  int tb_from = -1;
  bool tb_same = false;
  T* tb2 = nullptr;  // root LES of a fused stepper: sums of the stage state
  // FP64 stepper: sums of the step's initial state; the stage states u0 + cs
  // k_(s-1) take theirs by linearity from these and the sums of k_(s-1)
  T* tbu0 = nullptr;
  // overlapped FP64 stepper: the stage-state sums (targets of the next stage),
  // apart from tb, which holds k's sums while the LES streams read them
  T* tbs = nullptr;
  T *ub, *fk, *mcl, *mlast, *rtmp;
  T *ve[2], *ves, *ke;  // exact LES: state (ping-pong), stage, k
  T *vn[2], *vns, *kn;  // no-model LES
  T* ublast;            // target at stage 0 of the last step (pairs with mlast)
  T *vl[2], *vls, *kl, *nn;  // LES driven by the learned closure (when a net is attached)
  T* vgood;                  // its last state inside the energy band (fallback)
  // fallback of the learned LES (device, 8 doubles): [0] engaged (0/1), [1]
  // lower and [2] upper bound of its kinetic energy, [3] sum of squares of
  // the state ([4] the reduction's second word)
  double* fb = nullptr;
  exc_net* net = nullptr;
};

}  // namespace exc

struct exc_case {
  exc_case_desc desc{};
  int precision = EXC_F64;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  void* impl = nullptr;
  int (*step_fn)(exc_case*, int, double) = nullptr;
  void (*destroy_fn)(exc_case*) = nullptr;
};

namespace exc {

template <typename T>
struct CaseImpl {
  int fuse_root = -1;  // LES whose ratio the fused RK stage sums (-1: separate passes)
  bool tb_lin = false;  // stage-state sums by linearity (LesState::tbu0)
  // LES work on a stream of its own (FP64 with linear sums): the LES of stage
  // s runs beside the DNS of stage s + 1 (events order the shared sums)
  bool overlap = false;
  cudaStream_t lst = nullptr;  // the LES stream
  cudaEvent_t ev_s = nullptr, ev_t0 = nullptr, ev_k[4] = {}, ev_rd[4] = {};
  int n = 0;
  long long N = 0;
  double h = 0;
  exc_poisson ps;
  T* u[2] = {nullptr, nullptr};  // state ping-pong: u[cur] is the current velocity
  T* us = nullptr;               // stage state
  T* rhs = nullptr;              // RHS, then k in place
  int cur = 0;
  double* dscal = nullptr;       // [0] dt, [1] clock, [2] umax, [3..] scratch
  int* dflag = nullptr;
  double* part = nullptr;        // reduction partials
  int nles = 0;
  LesState<T> les[EXC_MAX_LES];
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  double graph_dt_fixed[2] = {NAN, NAN};
  long long net_gen = 0;  // workspace generations of attached nets at capture
  int kernels_per_step = 0;  // kernel nodes in the captured step graph
};

// No-model fallback of a learned-closure LES, checked before every step on
// the device: with E = 1/2 sum v^2 / M of the current state, a state whose E
// is not finite or leaves [fb[1], fb[2]] is replaced by the last state inside
// the band and the fallback is engaged for good (fb[0] = 1); a state inside
// the band becomes the last good one.  Every thread decides from the same
// fb[3] (written by the preceding reduction), so the grid agrees.
template <typename T>
__global__ void learned_guard_kernel(long long count, T* __restrict__ v, T* __restrict__ good,
                                     double* __restrict__ fb, double inv_m) {
  const double e = 0.5 * fb[3] * inv_m;
  const bool bad = !(e >= fb[1] && e <= fb[2]);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
    if (bad) v[i] = good[i];
    else good[i] = v[i];
  }
  if (bad && blockIdx.x == 0 && threadIdx.x == 0) fb[0] = 1.0;
}

// y += x unless the fallback is engaged (the net's closure term).
template <typename T>
__global__ void add_unless_kernel(long long count, T* __restrict__ y, const T* __restrict__ x,
                                  const double* __restrict__ fb) {
  if (fb[0] != 0.0) return;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
    y[i] += x[i];
}

static int grid_for_count(long long cnt) {
  long long b = (cnt + 255) / 256;
  return (int)(b < 152LL * 8 ? b : 152LL * 8);
}

template <typename T>
static int project_vec(exc_poisson* ps, T* u, cudaStream_t st) {
  cudaError_t e = poisson_solve_inplace<T>(ps, u, true, st);
  if (e == cudaSuccess) e = launch_gradient<T>(ps->n, (T)ps->h, u, reinterpret_cast<const T*>(ps->work), 2 * ps->P, st);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

// Transverse box sums of src for every LES: one pass over the fine field per
// LES whose ratio has no divisor among the other ratios, coarsening passes for
// the multiples (in increasing ratio), nothing for repeated ratios.
template <typename T>
static int les_tb_fill(CaseImpl<T>* ci, const T* src, cudaStream_t st) {
  int order[EXC_MAX_LES];
  for (int i = 0; i < ci->nles; ++i) order[i] = i;
  for (int i = 1; i < ci->nles; ++i)
    for (int j = i; j > 0 && ci->les[order[j]].c < ci->les[order[j - 1]].c; --j) {
      const int t = order[j];
      order[j] = order[j - 1];
      order[j - 1] = t;
    }
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < ci->nles && e == cudaSuccess; ++k) {
    LesState<T>& L = ci->les[order[k]];
    if (L.tb_same) continue;
    if (L.tb_from < 0) e = box_tb<T>(ci->n, L.c, src, L.tb, st);
    else e = box_tb_coarsen<T>(ci->n, ci->les[L.tb_from].c, L.c, ci->les[L.tb_from].tb, L.tb, st);
  }
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

template <typename T>
static const T* les_tb(const CaseImpl<T>* ci, const LesState<T>& L) {
  return L.tb_same ? ci->les[L.tb_from].tb : L.tb;
}

// y = a + cs x (y may be x) with the RK stage coefficient of stage sprev (cs =
// dt/2, dt/2, dt: the stage state u0 + cs k of the RK stage kernels), dt read
// on the device.
template <typename T>
__global__ void tb_lin_kernel(long long count, const T* __restrict__ a, const T* x, T* y,
                              const double* __restrict__ dtp, int sprev) {
  const double dt = dtp[0];
  const T cs = (T)(sprev == 2 ? dt : 0.5 * dt);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
    y[i] = fma(cs, x[i], a[i]);
}

// Keep the sums of the step's initial state (stage 0) for the linearity form.
template <typename T>
static int les_tb_keep(CaseImpl<T>* ci, cudaStream_t st) {
  for (int li = 0; li < ci->nles; ++li) {
    LesState<T>& L = ci->les[li];
    if (L.tb_same) continue;
    const cudaError_t e =
        cudaMemcpyAsync(L.tbu0, L.tb, 3 * (size_t)ci->n * L.m * L.m * sizeof(T), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  }
  return EXC_OK;
}

// Fused stepper (one root ratio for every LES): the root's sums come from
// rk_stage_sums_kernel in `root`; the other LES coarsen from them (in
// increasing ratio) into their own buffers (tb, or tbs with `stage`).
template <typename T>
static int les_tb_coarsen(CaseImpl<T>* ci, const T* root, cudaStream_t st, bool stage = false) {
  int order[EXC_MAX_LES];
  for (int i = 0; i < ci->nles; ++i) order[i] = i;
  for (int i = 1; i < ci->nles; ++i)
    for (int j = i; j > 0 && ci->les[order[j]].c < ci->les[order[j - 1]].c; --j) {
      const int t = order[j];
      order[j] = order[j - 1];
      order[j - 1] = t;
    }
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < ci->nles && e == cudaSuccess; ++k) {
    LesState<T>& L = ci->les[order[k]];
    if (L.tb_same || L.tb_from < 0) continue;
    const LesState<T>& F = ci->les[L.tb_from];
    const T* src = F.tb_from < 0 && !F.tb_same ? root : (stage ? F.tbs : F.tb);
    e = box_tb_coarsen<T>(ci->n, F.c, L.c, src, stage ? L.tbs : L.tb, st);
  }
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

// Sums used by LES L when the root's sums are in `root`.
template <typename T>
static const T* les_tb_from_root(const CaseImpl<T>* ci, const LesState<T>& L, const T* root) {
  const int r = ci->fuse_root;
  if (&L == &ci->les[r] || (L.tb_same && L.tb_from == r)) return root;
  return les_tb(ci, L);
}

// ubar from the filled transverse sums: own-axis taps, then the projection
// for the volume filter.
template <typename T>
static int les_target_tb(CaseImpl<T>* ci, LesState<T>& L, T* out, cudaStream_t st) {
  cudaError_t e = box_oa<T>(ci->n, L.c, L.kind, les_tb(ci, L), out, st);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  int rc = EXC_OK;
  if (L.kind == EXC_FILTER_VOLUME) rc = project_vec<T>(&L.ps, out, st);
  return rc;
}

// ubar = target(src) for one LES (the sums of every LES are refreshed, so the
// result has the same bits as in the stepper).
template <typename T>
static int les_target(CaseImpl<T>* ci, LesState<T>& L, const T* src, T* out, cudaStream_t st) {
  int rc = les_tb_fill<T>(ci, src, st);
  if (rc) return rc;
  return les_target_tb<T>(ci, L, out, st);
}

// One LES grid's work of RK stage s once the box sums of k_s (ksums) are
// ready, on stream sl: the closure m_s, then the exact, no-model and learned
// LES stages.
template <typename T>
static int les_stage(exc_case* cs, CaseImpl<T>* ci, LesState<T>& L, int s, int cur, const double* dt,
                     const T* ksums, cudaStream_t sl) {
  const T visc = (T)cs->desc.visc;
  cudaError_t e;
  const int m = L.m;
  const T H = (T)(cs->desc.l / m);
  // m_s = P_H(filter(k_s) - RHS_H(ubar_s)); mcl keeps the unprojected
  // difference (the projection is linear: the exact LES projects it
  // together with its own RHS, one solve instead of two)
  e = box_oa<T>(ci->n, L.c, L.kind, ksums, L.mcl, sl);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  int rc;
  e = launch_rhs<T>(m, H, visc, L.ub, L.rtmp, false, sl);
  if (e == cudaSuccess) e = launch_axpy<T>(3 * L.M, L.mcl, L.rtmp, (T)-1, sl);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  if (s == 0) {
    // the closure of stage 0 (snapshot pairs, diagnostics): m_0 itself
    e = cudaMemcpyAsync(L.mlast, L.mcl, 3 * L.M * sizeof(T), cudaMemcpyDeviceToDevice, sl);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(L.ublast, L.ub, 3 * L.M * sizeof(T), cudaMemcpyDeviceToDevice, sl);
    if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
    rc = project_vec<T>(&L.ps, L.mlast, sl);
    if (rc) return rc;
  }
  // exact-closure LES: k = P_H(RHS_H(v_s) + filter(k_s) - RHS_H(ubar_s))
  T* ve0 = L.ve[cur];
  T* vefin = L.ve[cur ^ 1];
  e = launch_rhs<T>(m, H, visc, s == 0 ? ve0 : L.ves, L.ke, false, sl);
  if (e == cudaSuccess) e = launch_axpy<T>(3 * L.M, L.ke, L.mcl, (T)1, sl);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  rc = project_vec<T>(&L.ps, L.ke, sl);
  if (rc) return rc;
  e = launch_rk_stage<T>(m, H, L.ke, nullptr, 0, ve0, L.ves, vefin, s, dt, sl);
  // no-model LES
  T* vn0 = L.vn[cur];
  T* vnfin = L.vn[cur ^ 1];
  if (e == cudaSuccess) e = launch_rhs<T>(m, H, visc, s == 0 ? vn0 : L.vns, L.kn, false, sl);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  rc = project_vec<T>(&L.ps, L.kn, sl);
  if (rc) return rc;
  e = launch_rk_stage<T>(m, H, L.kn, nullptr, 0, vn0, L.vns, vnfin, s, dt, sl);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  if (L.net) {
    // learned-closure LES: k = P_H(RHS_H(v_s) + net(v_s))
    T* vl0 = L.vl[cur];
    T* vlfin = L.vl[cur ^ 1];
    const T* vsrc = s == 0 ? vl0 : L.vls;
    e = launch_rhs<T>(m, H, visc, vsrc, L.kl, false, sl);
    if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
    rc = exc_net_forward(L.net, cs->precision, 1, m, vsrc, L.nn, sl);
    if (rc) return rc;
    add_unless_kernel<T><<<grid_for_count(3 * L.M), 256, 0, sl>>>(3 * L.M, L.kl, L.nn, L.fb);
    e = cudaGetLastError();
    if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
    rc = project_vec<T>(&L.ps, L.kl, sl);
    if (rc) return rc;
    e = launch_rk_stage<T>(m, H, L.kl, nullptr, 0, vl0, L.vls, vlfin, s, dt, sl);
    if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  }
  return EXC_OK;
}

// ubar_s of one LES from the box sums of the stage state (own-axis taps, then
// the projection for the volume filter), on stream sl.
template <typename T>
static int les_target_from(CaseImpl<T>* ci, LesState<T>& L, const T* ssums, cudaStream_t sl) {
  cudaError_t e = box_oa<T>(ci->n, L.c, L.kind, ssums, L.ub, sl);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return L.kind == EXC_FILTER_VOLUME ? project_vec<T>(&L.ps, L.ub, sl) : EXC_OK;
}

// Stage sums of LES L (shared by LES of the same ratio).
template <typename T>
static const T* les_tbs(const CaseImpl<T>* ci, const LesState<T>& L) {
  return L.tb_same ? ci->les[L.tb_from].tbs : L.tbs;
}

// The four RK stages with the LES work on the LES stream: the LES of stage s
// (closure, LES stages, the targets of stage s + 1) runs beside the DNS of
// stage s + 1.  The DNS stream writes k's box sums (tb) and the next stage
// state's sums (tbs, by linearity) only after the LES stream has finished the
// previous stage (events), and joins the LES stream at the end; the kernels
// and their inputs are those of the sequential stepper, so the results are
// the same bits.
template <typename T>
static int enqueue_stages_overlap(exc_case* cs, CaseImpl<T>* ci, int cur, T* u0, T* ufin, const double* dt,
                                  cudaStream_t st) {
  const int n = ci->n;
  const T h = (T)ci->h, visc = (T)cs->desc.visc;
  cudaStream_t sl = ci->lst;
  auto cuda_rc = [](cudaError_t err) {
    if (err == cudaSuccess) return (int)EXC_OK;
    set_last_error(cudaGetErrorString(err));
    return (int)EXC_ERR_CUDA;
  };
  // box sums of u0: kept for the linearity form and as the stage-0 targets' sums
  int rc = les_tb_fill<T>(ci, u0, st);
  if (!rc) rc = les_tb_keep<T>(ci, st);
  for (int li = 0; li < ci->nles && !rc; ++li) {
    LesState<T>& L = ci->les[li];
    if (L.tb_same) continue;
    rc = cuda_rc(cudaMemcpyAsync(L.tbs, L.tb, 3 * (size_t)n * L.m * L.m * sizeof(T), cudaMemcpyDeviceToDevice, st));
  }
  if (!rc) rc = cuda_rc(cudaEventRecord(ci->ev_s, st));
  if (!rc) rc = cuda_rc(cudaStreamWaitEvent(sl, ci->ev_s, 0));
  for (int li = 0; li < ci->nles && !rc; ++li) rc = les_target_from<T>(ci, ci->les[li], les_tbs(ci, ci->les[li]), sl);
  if (!rc) rc = cuda_rc(cudaEventRecord(ci->ev_t0, sl));
  for (int s = 0; s < 4 && !rc; ++s) {
    const T* src = s == 0 ? u0 : ci->us;
    // the stage states 1-3 are stored in the sweep's shifted form
    const bool wsh = rk_writes_shifted<T>(n);
    rc = cuda_rc(launch_rhs<T>(n, h, visc, src, ci->rhs, false, st, SlotBatch(), 1, s > 0 && wsh));
    if (!rc) rc = cuda_rc(poisson_solve_inplace<T>(&ci->ps, ci->rhs, true, st));
    if (!rc)
      rc = cuda_rc(launch_rk_stage<T>(n, h, ci->rhs, reinterpret_cast<const T*>(ci->ps.work), 2 * ci->ps.P, u0,
                                      ci->us, ufin, s, dt, st, SlotBatch(), 1, true, wsh, cs->desc.visc));
    // the LES stream is done with the sums of the previous stage (stage 0:
    // with the targets' sums)
    if (!rc) rc = cuda_rc(cudaStreamWaitEvent(st, s > 0 ? ci->ev_rd[s - 1] : ci->ev_t0, 0));
    if (!rc) rc = les_tb_fill<T>(ci, ci->rhs, st);
    if (s < 3) {
      for (int li = 0; li < ci->nles && !rc; ++li) {
        LesState<T>& L = ci->les[li];
        if (L.tb_same) continue;
        const long long cnt = 3LL * n * L.m * L.m;
        tb_lin_kernel<T><<<grid_for_count(cnt), 256, 0, st>>>(cnt, L.tbu0, L.tb, L.tbs, dt, s);
        rc = cuda_rc(cudaGetLastError());
      }
    }
    if (!rc) rc = cuda_rc(cudaEventRecord(ci->ev_k[s], st));
    if (!rc) rc = cuda_rc(cudaStreamWaitEvent(sl, ci->ev_k[s], 0));
    for (int li = 0; li < ci->nles && !rc; ++li) rc = les_stage<T>(cs, ci, ci->les[li], s, cur, dt, les_tb(ci, ci->les[li]), sl);
    if (s < 3)
      for (int li = 0; li < ci->nles && !rc; ++li)
        rc = les_target_from<T>(ci, ci->les[li], les_tbs(ci, ci->les[li]), sl);
    if (!rc) rc = cuda_rc(cudaEventRecord(ci->ev_rd[s], sl));
  }
  if (!rc) rc = cuda_rc(cudaStreamWaitEvent(st, ci->ev_rd[3], 0));
  return rc;
}

// Stage-state sums of LES L in the fused stepper: the root's (tb2, written by
// the RK stage kernel) or the coarsened ones of L's owner.
template <typename T>
static const T* les_tbs_fused(const CaseImpl<T>* ci, const LesState<T>& L) {
  const LesState<T>& O = L.tb_same ? ci->les[L.tb_from] : L;
  return O.tb_from < 0 ? ci->les[ci->fuse_root].tb2 : O.tbs;
}

// The fused stepper's four RK stages with the LES work on the LES stream, as
// in enqueue_stages_overlap: the RK stage kernel writes k's sums and the next
// stage state's sums itself, so the DNS stream waits for the LES stream's
// previous stage just before it.
template <typename T>
static int enqueue_stages_overlap_fused(exc_case* cs, CaseImpl<T>* ci, int cur, T* u0, T* ufin, const double* dt,
                                        cudaStream_t st) {
  const int n = ci->n;
  const T h = (T)ci->h, visc = (T)cs->desc.visc;
  cudaStream_t sl = ci->lst;
  LesState<T>& R = ci->les[ci->fuse_root];
  T* const root_k = R.tb;
  T* const root_s = R.tb2;
  auto cuda_rc = [](cudaError_t err) {
    if (err == cudaSuccess) return (int)EXC_OK;
    set_last_error(cudaGetErrorString(err));
    return (int)EXC_ERR_CUDA;
  };
  // box sums of u0 as the stage-0 targets' sums
  int rc = les_tb_fill<T>(ci, u0, st);
  const size_t rb = 3 * (size_t)n * R.m * R.m * sizeof(T);
  if (!rc) rc = cuda_rc(cudaMemcpyAsync(root_s, root_k, rb, cudaMemcpyDeviceToDevice, st));
  for (int li = 0; li < ci->nles && !rc; ++li) {
    LesState<T>& L = ci->les[li];
    if (L.tb_same || L.tb_from < 0) continue;
    rc = cuda_rc(cudaMemcpyAsync(L.tbs, L.tb, 3 * (size_t)n * L.m * L.m * sizeof(T), cudaMemcpyDeviceToDevice, st));
  }
  if (!rc) rc = cuda_rc(cudaEventRecord(ci->ev_s, st));
  if (!rc) rc = cuda_rc(cudaStreamWaitEvent(sl, ci->ev_s, 0));
  for (int li = 0; li < ci->nles && !rc; ++li)
    rc = les_target_from<T>(ci, ci->les[li], les_tbs_fused(ci, ci->les[li]), sl);
  if (!rc) rc = cuda_rc(cudaEventRecord(ci->ev_t0, sl));
  for (int s = 0; s < 4 && !rc; ++s) {
    const T* src = s == 0 ? u0 : ci->us;
    rc = cuda_rc(launch_rhs<T>(n, h, visc, src, ci->rhs, false, st));
    if (!rc) rc = cuda_rc(poisson_solve_inplace<T>(&ci->ps, ci->rhs, true, st));
    // the LES stream is done with the sums the RK stage kernel rewrites
    if (!rc) rc = cuda_rc(cudaStreamWaitEvent(st, s > 0 ? ci->ev_rd[s - 1] : ci->ev_t0, 0));
    if (!rc)
      rc = cuda_rc(launch_rk_stage_sums<T>(n, R.c, h, ci->rhs, reinterpret_cast<const T*>(ci->ps.work), 2 * ci->ps.P,
                                           u0, ci->us, ufin, s, dt, root_k, s < 3 ? root_s : nullptr, st));
    if (!rc) rc = les_tb_coarsen<T>(ci, root_k, st);
    if (!rc && s < 3) rc = les_tb_coarsen<T>(ci, root_s, st, true);
    if (!rc) rc = cuda_rc(cudaEventRecord(ci->ev_k[s], st));
    if (!rc) rc = cuda_rc(cudaStreamWaitEvent(sl, ci->ev_k[s], 0));
    for (int li = 0; li < ci->nles && !rc; ++li)
      rc = les_stage<T>(cs, ci, ci->les[li], s, cur, dt, les_tb_from_root(ci, ci->les[li], root_k), sl);
    if (s < 3)
      for (int li = 0; li < ci->nles && !rc; ++li)
        rc = les_target_from<T>(ci, ci->les[li], les_tbs_fused(ci, ci->les[li]), sl);
    if (!rc) rc = cuda_rc(cudaEventRecord(ci->ev_rd[s], sl));
  }
  if (!rc) rc = cuda_rc(cudaStreamWaitEvent(st, ci->ev_rd[3], 0));
  return rc;
}

// Enqueue one RK4 step (no host synchronisation).
template <typename T>
static int enqueue_step(exc_case* cs, CaseImpl<T>* ci, int cur, double dt_fixed) {
  cudaStream_t st = cs->stream;
  const int n = ci->n;
  const T h = (T)ci->h, visc = (T)cs->desc.visc;
  T* u0 = ci->u[cur];
  T* ufin = ci->u[cur ^ 1];
  double* dt = ci->dscal;
  cudaError_t e;
  // dt from the current DNS velocity (propose_timestep, src/N.jl:348-356)
  e = launch_max_abs<T>((size_t)(3 * ci->N), u0, ci->dscal + 2, ci->part, RED_PARTS, st);
  if (e == cudaSuccess)
    e = launch_set_dt(ci->dscal + 2, ci->h, cs->desc.visc, cs->desc.cfl, dt_fixed, dt, ci->dscal + 1, ci->dflag, st);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  // no-model fallback of the learned-closure LES (energy band, finiteness)
  for (int li = 0; li < ci->nles; ++li) {
    LesState<T>& L = ci->les[li];
    if (!L.net) continue;
    e = launch_sqdiff<T>(3 * L.M, L.vl[cur], nullptr, ci->part, L.fb + 3, st);
    if (e == cudaSuccess) {
      learned_guard_kernel<T><<<grid_for_count(3 * L.M), 256, 0, st>>>(3 * L.M, L.vl[cur], L.vgood, L.fb,
                                                                        1.0 / (double)L.M);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  }
  if (ci->overlap)
    return ci->fuse_root >= 0 ? enqueue_stages_overlap_fused<T>(cs, ci, cur, u0, ufin, dt, st)
                              : enqueue_stages_overlap<T>(cs, ci, cur, u0, ufin, dt, st);
  const bool fused = ci->fuse_root >= 0;
  T* const root_k = fused ? ci->les[ci->fuse_root].tb : nullptr;   // sums of k_s
  T* const root_s = fused ? ci->les[ci->fuse_root].tb2 : nullptr;  // sums of the stage state
  // without LES nothing but the next sweep reads the stage states: FP64
  // stores them in the sweep's shifted form
  const bool wsh = ci->nles == 0 && rk_writes_shifted<T>(n);
  for (int s = 0; s < 4; ++s) {
    const T* src = s == 0 ? u0 : ci->us;
    e = launch_rhs<T>(n, h, visc, src, ci->rhs, false, st, SlotBatch(), 1, s > 0 && wsh);
    if (e == cudaSuccess) e = poisson_solve_inplace<T>(&ci->ps, ci->rhs, true, st);
    if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
    // LES targets use the stage state before it is overwritten; the fused
    // stepper has the sums of stages 1-3 from the previous RK stage kernel
    const T* troot = nullptr;
    if (ci->nles > 0) {
      int rc;
      if (fused && s > 0) {
        troot = root_s;
        rc = les_tb_coarsen<T>(ci, troot, st);
      } else {
        rc = les_tb_fill<T>(ci, src, st);
        if (fused) troot = root_k;
      }
      if (rc) return rc;
    }
    for (int li = 0; li < ci->nles; ++li) {
      LesState<T>& L = ci->les[li];
      const int rc = les_target_from<T>(ci, L, fused ? les_tb_from_root(ci, L, troot) : les_tb(ci, L), st);
      if (rc) return rc;
    }
    if (fused) {
      e = launch_rk_stage_sums<T>(n, ci->les[ci->fuse_root].c, h, ci->rhs, reinterpret_cast<const T*>(ci->ps.work),
                                  2 * ci->ps.P, u0, ci->us, ufin, s, dt, root_k, s < 3 ? root_s : nullptr, st);
    } else {
      e = launch_rk_stage<T>(n, h, ci->rhs, reinterpret_cast<const T*>(ci->ps.work), 2 * ci->ps.P, u0, ci->us, ufin,
                             s, dt, st, SlotBatch(), 1, ci->nles > 0, wsh, cs->desc.visc);
    }
    if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
    if (ci->nles > 0) {
      int rc = fused ? les_tb_coarsen<T>(ci, root_k, st) : les_tb_fill<T>(ci, ci->rhs, st);
      if (rc) return rc;
    }
    for (int li = 0; li < ci->nles; ++li) {
      LesState<T>& L = ci->les[li];
      const int rc = les_stage<T>(cs, ci, L, s, cur, dt, fused ? les_tb_from_root(ci, L, root_k) : les_tb(ci, L), st);
      if (rc) return rc;
    }
  }
  return EXC_OK;
}

static int count_kernel_nodes(cudaGraph_t g) {
  size_t num = 0;
  if (cudaGraphGetNodes(g, nullptr, &num) != cudaSuccess || num == 0) return 0;
  std::vector<cudaGraphNode_t> nodes(num);
  if (cudaGraphGetNodes(g, nodes.data(), &num) != cudaSuccess) return 0;
  int k = 0;
  for (size_t i = 0; i < num; ++i) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
  }
  return k;
}

// sum of the workspace generations of the attached nets (a change means the
// captured graphs point at released buffers)
template <typename T>
static long long net_generation(CaseImpl<T>* ci) {
  long long g = 0;
  for (int li = 0; li < ci->nles; ++li)
    if (ci->les[li].net) g += net_workspace_gen(ci->les[li].net) + 1;
  return g;
}

template <typename T>
static int case_step(exc_case* cs, int nsteps, double dt_fixed) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  cudaStream_t st = cs->stream;
  for (int li = 0; li < ci->nles; ++li)
    if (ci->les[li].net) {
      int rc = net_reserve(ci->les[li].net, ci->les[li].M);
      if (rc) return rc;
    }
  const long long gen = net_generation(ci);
  if (gen != ci->net_gen) {
    for (int k = 0; k < 2; ++k)
      if (ci->graph[k]) { cudaGraphExecDestroy(ci->graph[k]); ci->graph[k] = nullptr; }
    ci->net_gen = gen;
  }
  for (int it = 0; it < nsteps; ++it) {
    int cur = ci->cur;
    double key = dt_fixed > 0 ? dt_fixed : -1.0;
    if (!ci->graph[cur] || !(ci->graph_dt_fixed[cur] == key)) {
      if (ci->graph[cur]) { cudaGraphExecDestroy(ci->graph[cur]); ci->graph[cur] = nullptr; }
      cudaGraph_t g;
      cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
      if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
      int rc = enqueue_step<T>(cs, ci, cur, key);
      e = cudaStreamEndCapture(st, &g);
      if (rc) { if (e == cudaSuccess) cudaGraphDestroy(g); return rc; }
      if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
      ci->kernels_per_step = count_kernel_nodes(g);
      e = cudaGraphInstantiate(&ci->graph[cur], g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
      ci->graph_dt_fixed[cur] = key;
    }
    cudaError_t e = cudaGraphLaunch(ci->graph[cur], st);
    if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
    ci->cur ^= 1;
  }
  return EXC_OK;
}

template <typename T>
static void case_destroy(exc_case* cs) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  if (!ci) return;
  for (int k = 0; k < 2; ++k) if (ci->graph[k]) cudaGraphExecDestroy(ci->graph[k]);
  if (ci->ev_s) cudaEventDestroy(ci->ev_s);
  if (ci->ev_t0) cudaEventDestroy(ci->ev_t0);
  for (int k = 0; k < 4; ++k) {
    if (ci->ev_k[k]) cudaEventDestroy(ci->ev_k[k]);
    if (ci->ev_rd[k]) cudaEventDestroy(ci->ev_rd[k]);
  }
  if (ci->lst) cudaStreamDestroy(ci->lst);
  poisson_free(&ci->ps);
  if (ci->u[0]) cudaFree(ci->u[0]);
  if (ci->dscal) cudaFree(ci->dscal);
  if (ci->dflag) cudaFree(ci->dflag);
  if (ci->part) cudaFree(ci->part);
  for (int li = 0; li < ci->nles; ++li) {
    poisson_free(&ci->les[li].ps);
    if (ci->les[li].buf) cudaFree(ci->les[li].buf);
    if (ci->les[li].tb) cudaFree(ci->les[li].tb);
    if (ci->les[li].tb2) cudaFree(ci->les[li].tb2);
    if (ci->les[li].tbu0) cudaFree(ci->les[li].tbu0);
    if (ci->les[li].tbs) cudaFree(ci->les[li].tbs);
    if (ci->les[li].fb) cudaFree(ci->les[li].fb);
  }
  delete ci;
  cs->impl = nullptr;
}

// The LES stream of the overlapped steppers and the events that order it.
template <typename T>
static int create_les_stream(CaseImpl<T>* ci) {
  bool ok = cudaEventCreateWithFlags(&ci->ev_s, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&ci->ev_t0, cudaEventDisableTiming) == cudaSuccess;
  for (int k = 0; k < 4 && ok; ++k)
    ok = cudaEventCreateWithFlags(&ci->ev_k[k], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&ci->ev_rd[k], cudaEventDisableTiming) == cudaSuccess;
  if (ok) ok = cudaStreamCreateWithFlags(&ci->lst, cudaStreamNonBlocking) == cudaSuccess;
  if (!ok) { set_last_error("cannot create the LES stream"); return EXC_ERR_CUDA; }
  return EXC_OK;
}

template <typename T>
static int case_create(exc_case* cs) {
  const exc_case_desc& d = cs->desc;
  CaseImpl<T>* ci = new CaseImpl<T>();
  cs->impl = ci;
  cs->step_fn = case_step<T>;
  cs->destroy_fn = case_destroy<T>;
  ci->n = d.n;
  ci->N = (long long)d.n * d.n * d.n;
  ci->h = d.l / d.n;
  int rc = poisson_init(&ci->ps, cs->precision, d.n, d.l, nullptr);
  if (rc) return rc;
  // the DNS pressure enters only through its gradient (RK stage): its
  // additive constant need not be removed
  ci->ps.mix_zero_mean = false;
  size_t vb = 3 * ci->N * sizeof(T);
  void* big = nullptr;
  if (cudaMalloc(&big, 4 * vb) != cudaSuccess) { set_last_error("out of device memory (DNS fields)"); return EXC_ERR_OOM; }
  ci->u[0] = reinterpret_cast<T*>(big);
  ci->u[1] = ci->u[0] + 3 * ci->N;
  ci->us = ci->u[1] + 3 * ci->N;
  ci->rhs = ci->us + 3 * ci->N;
  cudaMemset(big, 0, 4 * vb);
  if (cudaMalloc(&ci->dscal, 16 * sizeof(double)) != cudaSuccess || cudaMalloc(&ci->dflag, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&ci->part, (size_t)(SHELL_BLOCKS * 1024 + 2 * 1024) * sizeof(double)) != cudaSuccess) {
    set_last_error("out of device memory (scalars)");
    return EXC_ERR_OOM;
  }
  cudaMemset(ci->dscal, 0, 16 * sizeof(double));
  cudaMemset(ci->dflag, 0, sizeof(int));
  ci->nles = d.nles;
  for (int li = 0; li < d.nles; ++li) {
    LesState<T>& L = ci->les[li];
    L.c = d.les[li].ratio;
    L.kind = d.les[li].kind;
    L.m = d.n / L.c;
    L.M = (long long)L.m * L.m * L.m;
    rc = poisson_init(&L.ps, cs->precision, L.m, d.l, nullptr);
    if (rc) return rc;
    size_t nb = 21 * 3 * L.M * sizeof(T);
    if (cudaMalloc(&L.buf, nb) != cudaSuccess) { set_last_error("out of device memory (LES fields)"); return EXC_ERR_OOM; }
    cudaMemset(L.buf, 0, nb);
    size_t tbb = 3 * (size_t)d.n * L.m * L.m * sizeof(T);
    if (cudaMalloc(&L.tb, tbb) != cudaSuccess) { set_last_error("out of device memory (LES filter scratch)"); return EXC_ERR_OOM; }
    T* p = L.buf;
    auto take = [&]() { T* q = p; p += 3 * L.M; return q; };
    L.ub = take(); L.fk = take(); L.mcl = take(); L.mlast = take(); L.rtmp = take();
    L.ve[0] = take(); L.ve[1] = take(); L.ves = take(); L.ke = take();
    L.vn[0] = take(); L.vn[1] = take(); L.vns = take(); L.kn = take();
    L.ublast = take();
    L.vl[0] = take(); L.vl[1] = take(); L.vls = take(); L.kl = take(); L.nn = take();
    L.vgood = take();
    // 8 doubles: fb[3..4] receive the two-word result of the sum of squares
    if (cudaMalloc(&L.fb, 8 * sizeof(double)) != cudaSuccess) { set_last_error("out of device memory (LES fallback)"); return EXC_ERR_OOM; }
    const double fb0[8] = {0.0, 0.0, INFINITY, 0.0, 0.0, 0.0, 0.0, 0.0};
    cudaMemcpy(L.fb, fb0, sizeof(fb0), cudaMemcpyHostToDevice);
  }
  // sources of the transverse box sums: an earlier LES of the same ratio, else
  // the LES with the largest ratio that divides this one, else the fine field
  for (int li = 0; li < d.nles; ++li) {
    LesState<T>& L = ci->les[li];
    for (int lj = 0; lj < li; ++lj)
      if (ci->les[lj].c == L.c && !ci->les[lj].tb_same) {
        L.tb_from = lj;
        L.tb_same = true;
        break;
      }
    if (L.tb_same) continue;
    for (int lj = 0; lj < d.nles; ++lj) {
      const LesState<T>& S = ci->les[lj];
      if (lj == li || S.tb_same || S.c >= L.c || L.c % S.c != 0) continue;
      if (L.tb_from < 0 || S.c > ci->les[L.tb_from].c) L.tb_from = lj;
    }
  }
  // fused RK stage: one root ratio among the LES (every other LES shares or
  // coarsens from its sums) with a rk_stage_sums_kernel for the grid
  ci->fuse_root = -1;
  {
    int roots = 0, root = -1;
    for (int li = 0; li < d.nles; ++li)
      if (ci->les[li].tb_from < 0 && !ci->les[li].tb_same) {
        ++roots;
        root = li;
      }
    if (roots == 1) {
      const int xcw = rk_sums_chunk<T>(ci->les[root].c);
      if (xcw && d.n % xcw == 0) {
        LesState<T>& R = ci->les[root];
        const size_t tbb = 3 * (size_t)d.n * R.m * R.m * sizeof(T);
        if (cudaMalloc(&R.tb2, tbb) != cudaSuccess) { set_last_error("out of device memory (LES filter scratch)"); return EXC_ERR_OOM; }
        ci->fuse_root = root;
      }
    }
  }
  // fused stepper: LES work on the LES stream beside the DNS (stage sums of
  // the coarser LES in tbs)
  if (ci->fuse_root >= 0) {
    for (int li = 0; li < d.nles; ++li) {
      LesState<T>& L = ci->les[li];
      if (L.tb_same || L.tb_from < 0) continue;
      const size_t tbb = 3 * (size_t)d.n * L.m * L.m * sizeof(T);
      if (cudaMalloc(&L.tbs, tbb) != cudaSuccess) { set_last_error("out of device memory (LES filter scratch)"); return EXC_ERR_OOM; }
    }
    int rc2 = create_les_stream<T>(ci);
    if (rc2) return rc2;
    ci->overlap = true;
  }
  // FP64 with separate sum passes: stage-state sums by linearity
  ci->tb_lin = false;
  if (sizeof(T) == 8 && ci->fuse_root < 0 && d.nles > 0) {
    for (int li = 0; li < d.nles; ++li) {
      LesState<T>& L = ci->les[li];
      if (L.tb_same) continue;
      const size_t tbb = 3 * (size_t)d.n * L.m * L.m * sizeof(T);
      if (cudaMalloc(&L.tbu0, tbb) != cudaSuccess) { set_last_error("out of device memory (LES filter scratch)"); return EXC_ERR_OOM; }
    }
    ci->tb_lin = true;
    for (int li = 0; li < d.nles; ++li) {
      LesState<T>& L = ci->les[li];
      if (L.tb_same) continue;
      const size_t tbb = 3 * (size_t)d.n * L.m * L.m * sizeof(T);
      if (cudaMalloc(&L.tbs, tbb) != cudaSuccess) { set_last_error("out of device memory (LES filter scratch)"); return EXC_ERR_OOM; }
    }
    int rc2 = create_les_stream<T>(ci);
    if (rc2) return rc2;
    ci->overlap = true;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

// ---------------------------------------------------------------------------
// Host-facing helpers (templated)
// ---------------------------------------------------------------------------
template <typename T>
static int reset_les(exc_case* cs) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  cudaStream_t st = cs->stream;
  for (int li = 0; li < ci->nles; ++li) {
    LesState<T>& L = ci->les[li];
    int rc = les_target<T>(ci, L, ci->u[ci->cur], L.ub, st);
    if (rc) return rc;
    size_t b = 3 * L.M * sizeof(T);
    cudaMemcpyAsync(L.ve[ci->cur], L.ub, b, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(L.vn[ci->cur], L.ub, b, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(L.vl[ci->cur], L.ub, b, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(L.vgood, L.ub, b, cudaMemcpyDeviceToDevice, st);
    cudaMemsetAsync(L.fb, 0, sizeof(double), st);  // fallback disengaged
    cudaMemcpyAsync(L.ublast, L.ub, b, cudaMemcpyDeviceToDevice, st);
    cudaMemsetAsync(L.mlast, 0, b, st);
  }
  cudaMemsetAsync(ci->dscal, 0, 16 * sizeof(double), st);
  cudaMemsetAsync(ci->dflag, 0, sizeof(int), st);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

template <typename T>
static int set_velocity(exc_case* cs, const double* host) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  cudaStream_t st = cs->stream;
  size_t cnt = 3 * ci->N;
  if (sizeof(T) == sizeof(double)) {
    cudaError_t e = cudaMemcpyAsync(ci->u[ci->cur], host, cnt * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  } else {
    // stage through the (double-sized) rhs+us region
    double* tmp = reinterpret_cast<double*>(ci->us);
    cudaError_t e = cudaMemcpyAsync(tmp, host, cnt * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = launch_convert<double, T>((long long)cnt, tmp, ci->u[ci->cur], st);
    if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  }
  return reset_les<T>(cs);
}

template <typename T>
static int download(exc_case* cs, const T* dev, long long cnt, double* host) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  cudaStream_t st = cs->stream;
  cudaError_t e;
  if (sizeof(T) == sizeof(double)) {
    e = cudaMemcpyAsync(host, dev, cnt * sizeof(double), cudaMemcpyDeviceToHost, st);
  } else {
    // us and rhs are adjacent: 6 n^3 floats = 3 n^3 doubles of scratch
    double* tmp = reinterpret_cast<double*>(ci->us);
    e = launch_convert<T, double>(cnt, dev, tmp, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, tmp, cnt * sizeof(double), cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

// Random solenoidal field with the peak spectrum (src/N.jl:394-476).
template <typename T>
static int init_random(exc_case* cs, double kpeak, double energy, uint64_t seed) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  cudaStream_t st = cs->stream;
  const int n = ci->n, P = ci->ps.P;
  using C = cplx<T>;
  const long long cstride = (long long)n * n * P;
  C* spec = nullptr;
  if (cudaMalloc(&spec, 3 * cstride * sizeof(C)) != cudaSuccess) { set_last_error("out of device memory (init spectra)"); return EXC_ERR_OOM; }
  int rc = init_random_field<T>(&ci->ps, ci->u[ci->cur], spec, ci->part, kpeak, energy, seed, st);
  cudaError_t e = cudaStreamSynchronize(st);
  cudaFree(spec);
  if (rc) return rc;
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return reset_les<T>(cs);
}

template <typename T>
static int les_field(exc_case* cs, int li, int which, double* host) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  LesState<T>& L = ci->les[li];
  const T* src = nullptr;
  if (which == 0) {
    int rc = les_target<T>(ci, L, ci->u[ci->cur], L.ub, cs->stream);
    if (rc) return rc;
    src = L.ub;
  } else if (which == 1) src = L.ve[ci->cur];
  else if (which == 2) src = L.vn[ci->cur];
  else if (which == 3) src = L.mlast;
  else if (which == 4) src = L.vl[ci->cur];
  else src = L.ublast;
  return download<T>(cs, src, 3 * L.M, host);
}

// relative error (compute_errors, src/N.jl:1334-1349) of LES state `which`
// (1 exact, 2 no-model, 4 learned) against the filtered DNS
template <typename T>
static int les_error_one(exc_case* cs, int li, int which, double* err) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  LesState<T>& L = ci->les[li];
  cudaStream_t st = cs->stream;
  int rc = les_target<T>(ci, L, ci->u[ci->cur], L.ub, st);
  if (rc) return rc;
  const T* v = which == 1 ? L.ve[ci->cur] : which == 2 ? L.vn[ci->cur] : L.vl[ci->cur];
  double* out = ci->dscal + 4;
  double host[6];
  for (int c = 0; c < 3; ++c) {
    cudaError_t e = launch_sqdiff<T>(L.M, v + c * L.M, L.ub + c * L.M, ci->part, out + 2 * c, st);
    if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  }
  cudaError_t e = cudaMemcpyAsync(host, out, 6 * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  double s = 0;
  for (int c = 0; c < 3; ++c) s += host[2 * c] / host[2 * c + 1];
  *err = std::sqrt(s / 3.0);
  return EXC_OK;
}

// copy (target, closure) at stage 0 of the last step to caller device buffers
template <typename T>
static int snapshot(exc_case* cs, int li, void* dev_u, void* dev_m) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  LesState<T>& L = ci->les[li];
  size_t b = 3 * L.M * sizeof(T);
  cudaError_t e = cudaMemcpyAsync(dev_u, L.ublast, b, cudaMemcpyDeviceToDevice, cs->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dev_m, L.mlast, b, cudaMemcpyDeviceToDevice, cs->stream);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

template <typename T>
static int attach_net(exc_case* cs, int li, exc_net* net) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  LesState<T>& L = ci->les[li];
  cudaStreamSynchronize(cs->stream);
  if (net) {
    int rc = net_reserve(net, L.M);
    if (rc) return rc;
  }
  L.net = net;
  // the step graphs change: capture again at the next step
  for (int k = 0; k < 2; ++k)
    if (ci->graph[k]) { cudaGraphExecDestroy(ci->graph[k]); ci->graph[k] = nullptr; }
  ci->net_gen = net_generation(ci);
  size_t b = 3 * L.M * sizeof(T);
  cudaMemcpyAsync(L.vl[ci->cur], L.ve[ci->cur], b, cudaMemcpyDeviceToDevice, cs->stream);
  cudaMemcpyAsync(L.vgood, L.ve[ci->cur], b, cudaMemcpyDeviceToDevice, cs->stream);
  cudaMemsetAsync(L.fb, 0, sizeof(double), cs->stream);
  return EXC_OK;
}

template <typename T>
static int set_fallback(exc_case* cs, int li, double e_lo, double e_hi) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  const double band[2] = {e_lo, e_hi};
  cudaError_t e = cudaMemcpyAsync(ci->les[li].fb + 1, band, sizeof(band), cudaMemcpyHostToDevice, cs->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(cs->stream);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

template <typename T>
static int fallback_state(exc_case* cs, int li, int* engaged) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  double v = 0.0;
  cudaError_t e = cudaMemcpyAsync(&v, ci->les[li].fb, sizeof(double), cudaMemcpyDeviceToHost, cs->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(cs->stream);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  *engaged = v != 0.0;
  return EXC_OK;
}

template <typename T>
static int les_errors(exc_case* cs, int li, double* err2) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  LesState<T>& L = ci->les[li];
  cudaStream_t st = cs->stream;
  int rc = les_target<T>(ci, L, ci->u[ci->cur], L.ub, st);
  if (rc) return rc;
  double* out = ci->dscal + 4;  // 4..9: per-component pairs
  double host[2][6];
  for (int which = 0; which < 2; ++which) {
    const T* v = which == 0 ? L.ve[ci->cur] : L.vn[ci->cur];
    for (int c = 0; c < 3; ++c) {
      cudaError_t e = launch_sqdiff<T>(L.M, v + c * L.M, L.ub + c * L.M, ci->part, out + 2 * c, st);
      if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
    }
    cudaError_t e = cudaMemcpyAsync(host[which], out, 6 * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  }
  // compute_errors (src/N.jl:1334-1349): sqrt(mean_i sum|a_i-b_i|^2 / sum|b_i|^2)
  for (int which = 0; which < 2; ++which) {
    double s = 0;
    for (int c = 0; c < 3; ++c) s += host[which][2 * c] / host[which][2 * c + 1];
    err2[which] = std::sqrt(s / 3.0);
  }
  return EXC_OK;
}

template <typename T>
static int energy(exc_case* cs, double* out) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  cudaStream_t st = cs->stream;
  double* dv = ci->dscal + 10;
  cudaError_t e = launch_sqdiff<T>(3 * ci->N, ci->u[ci->cur], nullptr, ci->part, dv, st);
  double host[2];
  if (e == cudaSuccess) e = cudaMemcpyAsync(host, dv, 2 * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  *out = host[0] / 2.0 / (double)ci->N;
  return EXC_OK;
}

// visc * mean_ij (delta_j u_i)^2 summed over i, j (FP64).
template <typename T>
static int dissipation(exc_case* cs, double* out) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  cudaStream_t st = cs->stream;
  double* dv = ci->dscal + 12;
  cudaError_t e = launch_gradsq<T>(ci->n, ci->u[ci->cur], ci->part, dv, st);
  double host[2];
  if (e == cudaSuccess) e = cudaMemcpyAsync(host, dv, 2 * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  *out = cs->desc.visc * host[0] / (ci->h * ci->h) / (double)ci->N;
  return EXC_OK;
}

template <typename T>
static int spectrum(exc_case* cs, double* host_e, int nshell) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  cudaStream_t st = cs->stream;
  const int n = ci->n, P = ci->ps.P;
  using C = cplx<T>;
  const long long cstride = (long long)n * n * P;
  C* spec = nullptr;
  if (cudaMalloc(&spec, 3 * cstride * sizeof(C)) != cudaSuccess) { set_last_error("out of device memory (spectrum)"); return EXC_ERR_OOM; }
  exc_poisson tmp = ci->ps;
  cudaError_t e = cudaSuccess;
  for (int c = 0; c < 3 && e == cudaSuccess; ++c) {
    tmp.work = spec + c * cstride;
    e = fft3d_forward<T>(&tmp, ci->u[ci->cur] + c * ci->N, st);
  }
  const int nfull = (int)std::floor(std::sqrt(3.0) * (n / 2)) + 1;
  double* eshell = ci->part + SHELL_BLOCKS * 1024;
  const double N = (double)ci->N;
  if (e == cudaSuccess)
    e = launch_shell_energy<T>(n, P, 3, spec, cstride, 1.0 / (N * N), nfull, ci->part, SHELL_BLOCKS, eshell, st);
  std::vector<double> all(nfull);
  if (e == cudaSuccess) e = cudaMemcpyAsync(all.data(), eshell, nfull * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(spec);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  for (int k = 1; k <= nshell && k < nfull; ++k) host_e[k - 1] = all[k];
  return EXC_OK;
}

template <typename T>
static int launches(exc_case* cs) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  return ci->kernels_per_step;
}

template <typename T>
static void* device_ptr(exc_case* cs) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  return ci->u[ci->cur];
}

template <typename T>
static int read_scalars(exc_case* cs, double* host3, int* flag) {
  CaseImpl<T>* ci = reinterpret_cast<CaseImpl<T>*>(cs->impl);
  cudaError_t e = cudaMemcpyAsync(host3, ci->dscal, 3 * sizeof(double), cudaMemcpyDeviceToHost, cs->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(flag, ci->dflag, sizeof(int), cudaMemcpyDeviceToHost, cs->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(cs->stream);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

}  // namespace exc

using namespace exc;

#define DISPATCH(cs, fn, ...) ((cs)->precision == EXC_F64 ? fn<double>(__VA_ARGS__) : fn<float>(__VA_ARGS__))

extern "C" {

int exc_case_create(const exc_case_desc* desc, void* stream, exc_case** out) {
  if (!desc || !out) { set_last_error("null argument"); return EXC_ERR_ARG; }
  *out = nullptr;
  if (!fft_size_ok(desc->n)) { set_last_error("DNS grid size must be 2^a 3^b 5^c 7^d 11^e 13^f 17^g, a >= 1, 4 <= n <= 1024"); return EXC_ERR_SHAPE; }
  if (desc->precision != EXC_F64 && desc->precision != EXC_F32) { set_last_error("bad precision"); return EXC_ERR_ARG; }
  if (!(desc->l > 0) || !(desc->visc > 0) || !(desc->cfl > 0)) { set_last_error("l, visc and cfl must be positive"); return EXC_ERR_ARG; }
  if (desc->nles < 0 || desc->nles > EXC_MAX_LES) { set_last_error("nles out of range"); return EXC_ERR_ARG; }
  for (int i = 0; i < desc->nles; ++i) {
    int c = desc->les[i].ratio;
    if (c < 1 || desc->n % c != 0) { set_last_error("LES ratio must divide n"); return EXC_ERR_RATIO; }
    if (!fft_size_ok(desc->n / c)) { set_last_error("LES grid size n/ratio must be 2^a 3^b 5^c 7^d 11^e 13^f 17^g, a >= 1, >= 4"); return EXC_ERR_RATIO; }
    if (desc->les[i].kind != EXC_FILTER_VOLUME && desc->les[i].kind != EXC_FILTER_FACE) { set_last_error("bad filter kind"); return EXC_ERR_ARG; }
  }
  exc_case* cs = new exc_case();
  cs->desc = *desc;
  cs->precision = desc->precision;
  cs->stream = reinterpret_cast<cudaStream_t>(stream);
  if (!cs->stream) {
    // graph capture needs a real stream
    if (cudaStreamCreateWithFlags(&cs->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete cs;
      set_last_error("cannot create a CUDA stream");
      return EXC_ERR_CUDA;
    }
    cs->own_stream = true;
  }
  int rc = configure_device();
  if (rc == EXC_OK) rc = DISPATCH(cs, case_create, cs);
  if (rc) {
    if (cs->destroy_fn) cs->destroy_fn(cs);
    if (cs->own_stream) cudaStreamDestroy(cs->stream);
    delete cs;
    return rc;
  }
  *out = cs;
  return EXC_OK;
}

int exc_case_destroy(exc_case* cs) {
  if (!cs) return EXC_OK;
  cudaStreamSynchronize(cs->stream);
  if (cs->destroy_fn) cs->destroy_fn(cs);
  if (cs->own_stream) cudaStreamDestroy(cs->stream);
  delete cs;
  return EXC_OK;
}

int exc_case_init_random(exc_case* cs, double kpeak, double energy_, uint64_t seed) {
  if (!cs || !(kpeak > 0) || !(energy_ > 0)) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  return DISPATCH(cs, init_random, cs, kpeak, energy_, seed);
}

int exc_case_set_velocity(exc_case* cs, const double* host_u) {
  if (!cs || !host_u) { set_last_error("null argument"); return EXC_ERR_ARG; }
  return DISPATCH(cs, set_velocity, cs, host_u);
}

int exc_case_get_velocity(exc_case* cs, double* host_u) {
  if (!cs || !host_u) { set_last_error("null argument"); return EXC_ERR_ARG; }
  long long cnt = 3LL * cs->desc.n * cs->desc.n * cs->desc.n;
  if (cs->precision == EXC_F64)
    return download<double>(cs, reinterpret_cast<const double*>(device_ptr<double>(cs)), cnt, host_u);
  return download<float>(cs, reinterpret_cast<const float*>(device_ptr<float>(cs)), cnt, host_u);
}

int exc_case_get_les(exc_case* cs, int li, int which, double* host) {
  if (!cs || !host || li < 0 || li >= cs->desc.nles || which < 0 || which > 5) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  return DISPATCH(cs, les_field, cs, li, which, host);
}

int exc_case_reset_les(exc_case* cs) {
  if (!cs) { set_last_error("null argument"); return EXC_ERR_ARG; }
  return DISPATCH(cs, reset_les, cs);
}

int exc_case_les_error(exc_case* cs, int li, int which, double* err) {
  if (!cs || !err || li < 0 || li >= cs->desc.nles || !(which == 1 || which == 2 || which == 4)) {
    set_last_error("bad argument");
    return EXC_ERR_ARG;
  }
  return DISPATCH(cs, les_error_one, cs, li, which, err);
}

int exc_case_snapshot(exc_case* cs, int li, void* dev_u, void* dev_m) {
  if (!cs || !dev_u || !dev_m || li < 0 || li >= cs->desc.nles) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  return DISPATCH(cs, snapshot, cs, li, dev_u, dev_m);
}

int exc_case_attach_net(exc_case* cs, int li, exc_net* net) {
  if (!cs || li < 0 || li >= cs->desc.nles) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  return DISPATCH(cs, attach_net, cs, li, net);
}

int exc_case_set_fallback(exc_case* cs, int li, double e_lo, double e_hi) {
  if (!cs || li < 0 || li >= cs->desc.nles || !(e_lo <= e_hi)) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  return DISPATCH(cs, set_fallback, cs, li, e_lo, e_hi);
}

int exc_case_fallback(exc_case* cs, int li, int* engaged) {
  if (!cs || !engaged || li < 0 || li >= cs->desc.nles) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  return DISPATCH(cs, fallback_state, cs, li, engaged);
}

int exc_case_step(exc_case* cs, int nsteps, double dt_fixed) {
  if (!cs || nsteps < 0) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  return cs->step_fn(cs, nsteps, dt_fixed);
}

int exc_case_errors(exc_case* cs, int li, double* err2) {
  if (!cs || !err2 || li < 0 || li >= cs->desc.nles) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  return DISPATCH(cs, les_errors, cs, li, err2);
}

int exc_case_time(exc_case* cs, double* t, double* last_dt) {
  if (!cs) { set_last_error("null argument"); return EXC_ERR_ARG; }
  double h3[3];
  int flag = 0;
  int rc = DISPATCH(cs, read_scalars, cs, h3, &flag);
  if (rc) return rc;
  if (t) *t = h3[1];
  if (last_dt) *last_dt = h3[0];
  return EXC_OK;
}

int exc_case_energy(exc_case* cs, double* e) {
  if (!cs || !e) { set_last_error("null argument"); return EXC_ERR_ARG; }
  return DISPATCH(cs, energy, cs, e);
}

int exc_case_dissipation(exc_case* cs, double* eps) {
  if (!cs || !eps) { set_last_error("null argument"); return EXC_ERR_ARG; }
  return DISPATCH(cs, dissipation, cs, eps);
}

int exc_case_spectrum(exc_case* cs, double* host_e, int nshell) {
  if (!cs || !host_e || nshell < 1) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  return DISPATCH(cs, spectrum, cs, host_e, nshell);
}

int exc_case_device_ptr(exc_case* cs, int which, void** ptr) {
  if (!cs || !ptr || which != 0) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  *ptr = DISPATCH(cs, device_ptr, cs);
  return EXC_OK;
}

int exc_case_launches_per_step(exc_case* cs, int* count) {
  if (!cs || !count) { set_last_error("null argument"); return EXC_ERR_ARG; }
  *count = DISPATCH(cs, launches, cs);
  if (*count == 0) { set_last_error("no step has been captured yet"); return EXC_ERR_STATE; }
  return EXC_OK;
}

int exc_case_sync(exc_case* cs) {
  if (!cs) { set_last_error("null argument"); return EXC_ERR_ARG; }
  double h3[3];
  int flag = 0;
  int rc = DISPATCH(cs, read_scalars, cs, h3, &flag);
  if (rc) return rc;
  if (flag) { set_last_error("non-finite DNS velocity detected"); return EXC_ERR_NONFINITE; }
  return EXC_OK;
}

}  // extern "C"
