// Serving form: continuous batching of independent periodic NS solves of
// mixed grid sizes on one GPU (no counterpart in the reference, whose driver
// runs one solve at a time, src/N.jl:1239-1332).
//
// Requests queue on the host.  A chunk holds S same-size solves slot after
// slot in device memory (velocity ping-pong, stage state, RHS, spectral work
// array; nothing moves between steps).  Its stepping runs on the device: one
// captured graph whose conditional WHILE node repeats a body of two RK4 steps
// while any slot has steps left (at most kpairs times per launch).  The body's
// kernels cover all S slots at once (the slot is a grid dimension; inactive
// slots return at once, so admission never re-captures), and after each step
// a control kernel counts down every slot's steps, retires the slots that
// reached their count (GPU timestamp, final clock, buffer of the final state)
// and sets the loop condition; after the loop the energies of the retired
// slots are reduced and the control block is copied to pinned host memory.
// The host never waits on a chunk: a tick collects the chunks whose loop has
// ended (event query), reports their retired solves, admits what fits -- a
// free slot of an idle chunk of the request's grid size, or a new chunk if the
// memory budget (a share of the free HBM taken at creation) allows -- and
// relaunches every idle chunk that has work.  Each solve keeps its own
// viscosity, CFL time step and clock.  Chunks of different sizes run on their
// own streams and overlap on the device.  The FFT tile shapes of each grid
// size are chosen by timing candidates on the chunk's own batched work
// (autotuner) before capture.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <tuple>
#include <vector>

#include "internal.cuh"
#include "fields.cuh"

namespace exc {

// ---------------------------------------------------------------------------
// Batched kernels of the serving step
// ---------------------------------------------------------------------------
constexpr int SRV_RED = 256;  // partial blocks per slot for max |u|

template <typename T>
__global__ void slot_maxabs_partial(long long count, const T* __restrict__ u, long long stride,
                                    const int* __restrict__ active, double* __restrict__ part) {
  const int slot = blockIdx.y;
  if (!active[slot]) return;
  // maximum of the magnitude bits (exact, integer pipe, NaN propagates); the
  // slot strides keep 16-byte alignment and count is a multiple of 4
  using B = typename MagBits<T>::type;
  using V = typename MagBits<T>::vec;
  constexpr int E = 16 / (int)sizeof(T);
  const V* x = reinterpret_cast<const V*>(u + slot * stride);
  B m = 0;
  const long long nv = count / E;
#pragma unroll 4
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nv; i += (long long)gridDim.x * blockDim.x) {
    const V v = x[i];
    const T* e = reinterpret_cast<const T*>(&v);
#pragma unroll
    for (int k = 0; k < E; ++k) m = max(m, mag_bits(e[k]));
  }
  __shared__ B red[8];
  for (int o = 16; o > 0; o >>= 1) m = max(m, (B)__shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    B r = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = max(r, red[w]);
    part[slot * SRV_RED + blockIdx.x] = (double)from_mag_bits<T>(r);
  }
}

// per-slot dt = min(cfl h/umax, cfl h^2/visc/6) (propose_timestep,
// src/N.jl:348-356); a non-finite umax flags the slot and freezes it (dt = 0)
__global__ void slot_set_dt(int S, const int* __restrict__ active, const double* __restrict__ part, double h,
                            double cfl, const double* __restrict__ viscd, double* __restrict__ dt,
                            double* __restrict__ clock, int* __restrict__ flag) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S || !active[s]) return;
  double m = 0.0;
  for (int b = 0; b < SRV_RED; ++b) {
    double v = part[s * SRV_RED + b];
    m = (v > m || v != v) ? v : m;
  }
  double a = cfl * h / m, v = cfl * h * h / viscd[s] / 6.0;
  double d = a < v ? a : v;
  if (!(m < 1e300)) { flag[s] = 1; d = 0.0; }
  dt[s] = d;
  clock[s] += d;
}

__global__ void set_active_kernel(int S, unsigned long long mask, int* __restrict__ active) {
  const int s = threadIdx.x;
  if (s < S) active[s] = (int)((mask >> s) & 1ull);
}

// Device-side lifecycle of a chunk's slots; copied to pinned host memory at
// the end of every loop launch.
constexpr int SRV_MAXS = 64;
struct SlotCtl {
  int steps_left[SRV_MAXS];
  int fin[SRV_MAXS];         // 1 once the slot has taken its last step
  int fin_parity[SRV_MAXS];  // velocity buffer holding its final state
  int edone[SRV_MAXS];       // its energy has been reduced
  int iter;                  // body iterations (two steps each) of the current launch
  int pad[3];
  unsigned long long fin_time[SRV_MAXS];  // GPU global timer (ns) at its last step
  double fin_clock[SRV_MAXS];             // its simulated time
  double energy[SRV_MAXS];                // sum of u^2 of its final state
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__global__ void global_ns_kernel(unsigned long long* out) { *out = global_ns(); }

template <typename T>
__global__ void set_slot_kernel(int s, double visc, int nsteps, T* __restrict__ vdev, double* __restrict__ vd,
                                double* __restrict__ clock, int* __restrict__ flag, SlotCtl* __restrict__ ctl) {
  vdev[s] = (T)visc;
  vd[s] = visc;
  clock[s] = 0.0;
  flag[s] = 0;
  ctl->steps_left[s] = nsteps;
  ctl->fin[s] = 0;
  ctl->edone[s] = 0;
}

// start of a loop launch: the slots with steps left are active
__global__ void loop_begin_kernel(int S, SlotCtl* __restrict__ ctl, int* __restrict__ active) {
  const int s = threadIdx.x;
  if (s < S) active[s] = ctl->steps_left[s] > 0;
  if (s == 0) ctl->iter = 0;
}

// after one step: count down, retire the slots that took their last step,
// activity of the next step; after the body's second step, the loop
// condition (any slot active and fewer than kpairs iterations)
__global__ void slot_ctl_kernel(int S, int parity_after, int last, int kpairs, SlotCtl* __restrict__ ctl,
                                int* __restrict__ active, const double* __restrict__ clock,
                                cudaGraphConditionalHandle loop) {
  const int s = threadIdx.x;
  int act = 0;
  if (s < S) {
    if (active[s]) {
      const int left = ctl->steps_left[s] - 1;
      ctl->steps_left[s] = left;
      if (left == 0) {
        ctl->fin[s] = 1;
        ctl->fin_parity[s] = parity_after;
        ctl->fin_time[s] = global_ns();
        ctl->fin_clock[s] = clock[s];
      }
    }
    act = ctl->steps_left[s] > 0;
    active[s] = act;
  }
  const int any = __syncthreads_or(act);
  if (last && s == 0) {
    const int it = ctl->iter + 1;
    ctl->iter = it;
    cudaGraphSetConditional(loop, (any && it < kpairs) ? 1u : 0u);
  }
}

// sum of u^2 of every slot retired and not yet reduced (fixed order per slot)
template <typename T>
__global__ void slot_energy_partial(long long count, const T* __restrict__ u0, const T* __restrict__ u1,
                                    long long stride, const SlotCtl* __restrict__ ctl, double* __restrict__ part) {
  const int s = blockIdx.y;
  if (!ctl->fin[s] || ctl->edone[s]) return;
  const T* u = (ctl->fin_parity[s] ? u1 : u0) + s * stride;
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
    const double v = (double)u[i];
    acc = fma(v, v, acc);
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[s * SRV_RED + blockIdx.x] = red[0];
}

__global__ void slot_energy_fold(int S, SlotCtl* __restrict__ ctl, const double* __restrict__ part) {
  const int s = threadIdx.x;
  if (s >= S || !ctl->fin[s] || ctl->edone[s]) return;
  double e = 0.0;
  for (int b = 0; b < SRV_RED; ++b) e += part[s * SRV_RED + b];
  ctl->energy[s] = e;
  ctl->edone[s] = 1;
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct PendingReq {
  int64_t id;
  exc_solve_req req;
  double t_submit;
};

struct FinishRec {
  exc_solve_result res;
  cudaEvent_t ev = nullptr;  // completion of the final-field copy, if one was asked for
};

class ChunkBase {
 public:
  virtual ~ChunkBase() = default;
  int n = 0, S = 0;
  double l = 1.0, cfl = 0.3;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;
  std::vector<int64_t> slot_id;
  std::vector<int> nsteps;
  std::vector<double> t_submit, t_admit;
  std::vector<double*> result_host;
  cudaEvent_t done_ev = nullptr;  // end of the last loop launch
  bool in_flight = false;         // a loop launch has not been collected yet
  SlotCtl* mirror = nullptr;      // pinned copy of the control block (valid after done_ev)
  int kpairs = 1;                 // body iterations (two steps each) per launch at most
  long long ticks = 0;            // loop launches
  int free_slot() const {
    for (int s = 0; s < S; ++s)
      if (slot_id[s] < 0) return s;
    return -1;
  }
  int active_count() const {
    int c = 0;
    for (int s = 0; s < S; ++s) c += slot_id[s] >= 0;
    return c;
  }
};

template <typename T>
class Chunk : public ChunkBase {
 public:
  long long N = 0;
  exc_poisson ps;
  T* big = nullptr;  // u[0], u[1], us, rhs: S * 3N each
  T* u[2] = {nullptr, nullptr};
  T* us = nullptr;
  T* rhs = nullptr;
  void* work = nullptr;
  T* visc = nullptr;
  double *dt = nullptr, *clock = nullptr, *part = nullptr, *red = nullptr, *viscd = nullptr;
  int *active = nullptr, *flag = nullptr;
  SlotCtl* ctl = nullptr;  // device control block
  int cur = 0;             // 0: every active slot's state is in u[0] between launches
  cudaGraphExec_t loop = nullptr;
  int kernels_per_step = 0;

  ~Chunk() override {
    if (stream) cudaStreamSynchronize(stream);
    if (loop) cudaGraphExecDestroy(loop);
    if (ctl) cudaFree(ctl);
    if (mirror) cudaFreeHost(mirror);
    if (done_ev) cudaEventDestroy(done_ev);
    poisson_free(&ps);
    if (work) cudaFree(work);
    if (big) cudaFree(big);
    if (visc) cudaFree(visc);
    if (dt) cudaFree(dt);
    if (active) cudaFree(active);
    if (stream) cudaStreamDestroy(stream);
  }

  SlotBatch batch() const {
    SlotBatch sb;
    sb.ustride = 3 * N;
    sb.wstride = (long long)n * n * ps.P;
    sb.active = active;
    sb.visc = visc;
    return sb;
  }

  // one batched RK4 step (same tableau and projection as the case stepper)
  cudaError_t enqueue_step(int c) {
    const SlotBatch sb = batch();
    const T h = (T)(l / n);
    T* u0 = u[c];
    T* ufin = u[c ^ 1];
    slot_maxabs_partial<T><<<dim3(SRV_RED, S), 256, 0, stream>>>(3 * N, u0, 3 * N, active, part);
    slot_set_dt<<<(S + 63) / 64, 64, 0, stream>>>(S, active, part, l / n, cfl, viscd, dt, clock, flag);
    cudaError_t e = cudaGetLastError();
    for (int s = 0; s < 4 && e == cudaSuccess; ++s) {
      const T* src = s == 0 ? u0 : us;
      e = launch_rhs<T>(n, h, (T)0, src, rhs, false, stream, sb, S);
      if (e == cudaSuccess) e = poisson_solve_inplace<T>(&ps, rhs, true, stream, sb, S);
      if (e == cudaSuccess)
        e = launch_rk_stage<T>(n, h, rhs, reinterpret_cast<const T*>(ps.work), 2 * ps.P, u0, us, ufin, s, dt, stream,
                               sb, S, false);
    }
    return e;
  }

  // The device-side loop: WHILE (condition set by slot_ctl_kernel) { step
  // from u[0]; control; step from u[1]; control }, then the energies of the
  // retired slots and the copy of the control block to the pinned mirror.
  cudaError_t build_loop() {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    cudaGraphConditionalHandle h;
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
    cudaGraphNode_t wnode = nullptr;
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    if (e == cudaSuccess) e = cudaGraphAddNode(&wnode, g, nullptr, nullptr, 0, &cp);
    if (e == cudaSuccess) {
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      e = cudaStreamBeginCaptureToGraph(stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        cudaError_t e2 = enqueue_step(0);
        slot_ctl_kernel<<<1, SRV_MAXS, 0, stream>>>(S, 1, 0, kpairs, ctl, active, clock, h);
        if (e2 == cudaSuccess) e2 = enqueue_step(1);
        slot_ctl_kernel<<<1, SRV_MAXS, 0, stream>>>(S, 0, 1, kpairs, ctl, active, clock, h);
        if (e2 == cudaSuccess) e2 = cudaGetLastError();
        e = cudaStreamEndCapture(stream, &body);
        if (e2 != cudaSuccess) e = e2;
      }
      if (e == cudaSuccess) {
        size_t num = 0;
        cudaGraphGetNodes(body, nullptr, &num);
        kernels_per_step = (int)num / 2;
      }
    }
    if (e == cudaSuccess)
      e = cudaStreamBeginCaptureToGraph(stream, g, &wnode, nullptr, 1, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      slot_energy_partial<T><<<dim3(SRV_RED, S), 256, 0, stream>>>(3 * N, u[0], u[1], 3 * N, ctl, part);
      slot_energy_fold<<<1, SRV_MAXS, 0, stream>>>(S, ctl, part);
      cudaError_t e2 = cudaMemcpyAsync(mirror, ctl, sizeof(SlotCtl), cudaMemcpyDeviceToHost, stream);
      if (e2 == cudaSuccess) e2 = cudaGetLastError();
      cudaGraph_t g2 = g;
      e = cudaStreamEndCapture(stream, &g2);
      if (e2 != cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&loop, g, 0);
    if (g) cudaGraphDestroy(g);
    return e;
  }
};

// autotuned FFT engine and Stockham tile shape per (n, precision, S)
struct Tuned {
  int engine, col_w, x_rows;
};
static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int>, Tuned> g_tuned;

}  // namespace exc

struct exc_server {
  exc_server_desc desc{};
  size_t budget = 0, used = 0;
  std::chrono::steady_clock::time_point t0;
  cudaStream_t admit_stream = nullptr;
  cudaEvent_t ev0 = nullptr;
  std::deque<exc::PendingReq> pending;
  std::vector<std::unique_ptr<exc::ChunkBase>> chunks;
  std::vector<exc::FinishRec> finishing;
  int64_t next_id = 1;
  int max_active_per_size = 0;  // admission bound per grid size (0: none)
  unsigned long long gt0 = 0;   // GPU global timer (ns) at the server's time origin
  // init scratch (largest grid seen so far)
  void* spec3 = nullptr;
  size_t spec3_bytes = 0;
  double* init_part = nullptr;
  long long ticks = 0;
  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace exc {

template <typename T>
static int tune_chunk(exc_server* sv, Chunk<T>* ck) {
  using C = cplx<T>;
  const int prec = sizeof(T) == 8 ? EXC_F64 : EXC_F32;
  auto key = std::make_tuple(ck->n, prec, ck->S);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      ck->ps.engine = it->second.engine;
      ck->ps.col_w = it->second.col_w;
      ck->ps.x_rows = it->second.x_rows;
      return EXC_OK;
    }
  }
  const int n = ck->n;
  const int wmax = [&] { int w = 1; while (w * 2 * n <= fft_tile<C>() && w < 64) w *= 2; return w; }();
  const int rmax = fft_tile<C>() / (n / 2 + 1);
  std::vector<int> ws, rs;
  for (int w = wmax; w >= 1 && (int)ws.size() < 4; w /= 2) ws.push_back(w);
  for (int r = rmax; r >= 1 && (int)rs.size() < 3; r /= 2) rs.push_back(r);
  set_active_kernel<<<1, 64, 0, ck->stream>>>(ck->S, ~0ull, ck->active);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  // candidates: the register-resident passes (where the grid has a plan) and
  // the Stockham passes over the tile shapes above
  std::vector<Tuned> cands;
  if (ck->ps.twl_n && ck->ps.twl_h) cands.push_back({0, 0, 0});
  for (int w : ws)
    for (int r : rs) cands.push_back({1, w, r});
  float best = 1e30f;
  Tuned bc = cands.front();
  for (const Tuned& c : cands) {
    ck->ps.engine = c.engine;
    ck->ps.col_w = c.col_w;
    ck->ps.x_rows = c.x_rows;
    poisson_solve_inplace<T>(&ck->ps, ck->rhs, true, ck->stream, ck->batch(), ck->S);  // warm
    cudaEventRecord(a, ck->stream);
    for (int rep = 0; rep < 3; ++rep) poisson_solve_inplace<T>(&ck->ps, ck->rhs, true, ck->stream, ck->batch(), ck->S);
    cudaEventRecord(b, ck->stream);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    if (ms < best) { best = ms; bc = c; }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  set_active_kernel<<<1, 64, 0, ck->stream>>>(ck->S, 0ull, ck->active);
  ck->ps.engine = bc.engine;
  ck->ps.col_w = bc.col_w;
  ck->ps.x_rows = bc.x_rows;
  cudaError_t e = cudaStreamSynchronize(ck->stream);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tuned[key] = bc;
  return EXC_OK;
}

static size_t chunk_bytes(int n, int S, size_t w) {
  const size_t N = (size_t)n * n * n;
  const size_t P = (size_t)spec_pitch(n);
  return S * (12 * N * w + (size_t)n * n * P * 2 * w) + (size_t)n * n * (n / 2 + 1) * 8 + S * 128 + S * SRV_RED * 8;
}

// body iterations (two RK4 steps each) per loop launch at most: a few
// milliseconds of work per launch
static int kpairs_for(int n) {
  if (n <= 64) return 16;
  if (n <= 128) return 8;
  if (n <= 192) return 4;
  return 2;
}

static int slots_for(const exc_server* sv, int n) {
  if (sv->desc.slots_per_chunk > 0) return std::min(sv->desc.slots_per_chunk, 64);
  if (n <= 64) return 16;
  if (n <= 128) return 8;
  if (n <= 192) return 4;
  return 2;
}

template <typename T>
static int make_chunk(exc_server* sv, int n, double l, double cfl, ChunkBase** out) {
  const int S = slots_for(sv, n);
  const size_t need = chunk_bytes(n, S, sizeof(T));
  if (sv->used + need > sv->budget) return EXC_ERR_OOM;  // not an error: wait for memory
  auto ck = std::make_unique<Chunk<T>>();
  ck->n = n;
  ck->S = S;
  ck->l = l;
  ck->cfl = cfl;
  ck->N = (long long)n * n * n;
  ck->slot_id.assign(S, -1);
  ck->nsteps.assign(S, 0);
  ck->t_submit.assign(S, 0);
  ck->t_admit.assign(S, 0);
  ck->result_host.assign(S, nullptr);
  if (cudaStreamCreateWithFlags(&ck->stream, cudaStreamNonBlocking) != cudaSuccess) { set_last_error("stream"); return EXC_ERR_CUDA; }
  cudaEventCreateWithFlags(&ck->done_ev, cudaEventDisableTiming);
  ck->kpairs = kpairs_for(n);
  if (cudaMalloc(&ck->ctl, sizeof(SlotCtl)) != cudaSuccess ||
      cudaHostAlloc(&ck->mirror, sizeof(SlotCtl), cudaHostAllocDefault) != cudaSuccess) {
    set_last_error("out of memory (chunk control block)");
    return EXC_ERR_OOM;
  }
  cudaMemsetAsync(ck->ctl, 0, sizeof(SlotCtl), ck->stream);
  std::memset(ck->mirror, 0, sizeof(SlotCtl));
  using C = cplx<T>;
  const long long wst = (long long)n * n * spec_pitch(n);
  if (cudaMalloc(&ck->work, S * wst * sizeof(C)) != cudaSuccess) { set_last_error("out of device memory (chunk work)"); return EXC_ERR_OOM; }
  int rc = poisson_init(&ck->ps, sizeof(T) == 8 ? EXC_F64 : EXC_F32, n, l, ck->work);
  if (rc) return rc;
  if (cudaMalloc(&ck->big, 4 * S * 3 * ck->N * sizeof(T)) != cudaSuccess) { set_last_error("out of device memory (chunk fields)"); return EXC_ERR_OOM; }
  cudaMemsetAsync(ck->big, 0, 4 * S * 3 * ck->N * sizeof(T), ck->stream);
  ck->u[0] = ck->big;
  ck->u[1] = ck->u[0] + S * 3 * ck->N;
  ck->us = ck->u[1] + S * 3 * ck->N;
  ck->rhs = ck->us + S * 3 * ck->N;
  if (cudaMalloc(&ck->visc, S * sizeof(T)) != cudaSuccess ||
      cudaMalloc(&ck->dt, (4 * S + S * SRV_RED + 64 + 1024) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&ck->active, 2 * S * sizeof(int)) != cudaSuccess) {
    set_last_error("out of device memory (chunk scalars)");
    return EXC_ERR_OOM;
  }
  ck->clock = ck->dt + S;
  ck->viscd = ck->clock + S;
  ck->red = ck->viscd + S;  // energy reduction output (2 doubles) + spare
  ck->part = ck->red + S + 64;
  ck->flag = ck->active + S;
  cudaMemsetAsync(ck->dt, 0, (4 * S + S * SRV_RED + 64 + 1024) * sizeof(double), ck->stream);
  cudaMemsetAsync(ck->active, 0, 2 * S * sizeof(int), ck->stream);
  std::vector<T> ones(S, (T)1e-3);
  cudaMemcpyAsync(ck->visc, ones.data(), S * sizeof(T), cudaMemcpyHostToDevice, ck->stream);
  cudaStreamSynchronize(ck->stream);
  if (sv->desc.autotune) {
    rc = tune_chunk<T>(sv, ck.get());
    if (rc) return rc;
  }
  // capture the device-side step loop
  {
    cudaError_t e = ck->build_loop();
    if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  }
  ck->bytes = need;
  sv->used += need;
  *out = ck.get();
  sv->chunks.push_back(std::move(ck));
  return EXC_OK;
}

template <typename T>
static int ensure_init_scratch(exc_server* sv, int n) {
  using C = cplx<T>;
  const size_t need = 3 * (size_t)n * n * spec_pitch(n) * sizeof(C);
  if (need <= sv->spec3_bytes) return EXC_OK;
  if (sv->spec3) { cudaStreamSynchronize(sv->admit_stream); cudaFree(sv->spec3); sv->spec3 = nullptr; }
  if (cudaMalloc(&sv->spec3, need) != cudaSuccess) { sv->spec3_bytes = 0; set_last_error("out of device memory (init scratch)"); return EXC_ERR_OOM; }
  sv->spec3_bytes = need;
  return EXC_OK;
}

// Put request `pr` into a free slot (new chunk if needed and affordable).
template <typename T>
static int admit(exc_server* sv, const PendingReq& pr, bool* admitted, bool* waiting) {
  *admitted = false;
  *waiting = false;
  const exc_solve_req& q = pr.req;
  Chunk<T>* ck = nullptr;
  int slot = -1;
  bool busy_slot = false;
  for (auto& cb : sv->chunks) {
    if (cb->n != q.n || cb->l != q.l || cb->cfl != q.cfl) continue;
    int s = cb->free_slot();
    if (s < 0) continue;
    // a chunk whose loop runs takes new solves only after it is collected
    // (its launch holds a few milliseconds of work): wait for it rather than
    // open another chunk
    if (cb->in_flight) { busy_slot = true; continue; }
    ck = static_cast<Chunk<T>*>(cb.get());
    slot = s;
    break;
  }
  if (!ck && busy_slot) { *waiting = true; return EXC_OK; }
  if (!ck) {
    ChunkBase* nb = nullptr;
    int rc = make_chunk<T>(sv, q.n, q.l, q.cfl, &nb);
    if (rc == EXC_ERR_OOM && !sv->chunks.empty()) return EXC_OK;  // wait for memory to free up
    if (rc) return rc;
    ck = static_cast<Chunk<T>*>(nb);
    slot = 0;
  }
  int rc = ensure_init_scratch<T>(sv, q.n);
  if (rc) return rc;
  // the slot's previous owner may still be finishing on the chunk stream
  cudaEvent_t ready;
  cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
  cudaEventRecord(ready, ck->stream);
  cudaStreamWaitEvent(sv->admit_stream, ready, 0);
  exc_poisson view = ck->ps;
  view.work = reinterpret_cast<cplx<T>*>(ck->work) + slot * (long long)q.n * q.n * ck->ps.P;
  T* u = ck->u[ck->cur] + slot * 3 * ck->N;
  set_slot_kernel<T><<<1, 1, 0, sv->admit_stream>>>(slot, q.visc, q.nsteps, ck->visc, ck->viscd, ck->clock, ck->flag,
                                                      ck->ctl);
  rc = init_random_field<T>(&view, u, reinterpret_cast<cplx<T>*>(sv->spec3), sv->init_part, q.kpeak, q.energy, q.seed,
                            sv->admit_stream);
  cudaEventRecord(ready, sv->admit_stream);
  cudaStreamWaitEvent(ck->stream, ready, 0);
  cudaEventDestroy(ready);
  if (rc) return rc;
  ck->slot_id[slot] = pr.id;
  ck->nsteps[slot] = q.nsteps;
  ck->t_submit[slot] = pr.t_submit;
  ck->t_admit[slot] = sv->now();
  ck->result_host[slot] = q.result_host;
  *admitted = true;
  return EXC_OK;
}

// A chunk whose loop launch has ended: report its retired solves (times and
// energies from the control block's pinned mirror; the optional final-field
// copy is queued on the chunk stream) and free their slots.
template <typename T>
static int collect_chunk(exc_server* sv, Chunk<T>* ck) {
  if (!ck->in_flight) return EXC_OK;
  cudaError_t q = cudaEventQuery(ck->done_ev);
  if (q == cudaErrorNotReady) return EXC_OK;
  if (q != cudaSuccess) { set_last_error(cudaGetErrorString(q)); return EXC_ERR_CUDA; }
  ck->in_flight = false;
  const SlotCtl* m = ck->mirror;
  for (int s = 0; s < ck->S; ++s) {
    if (ck->slot_id[s] < 0 || !m->fin[s]) continue;
    FinishRec rec;
    rec.res.id = ck->slot_id[s];
    rec.res.n = ck->n;
    rec.res.nsteps = ck->nsteps[s];
    rec.res.t_submit = ck->t_submit[s];
    rec.res.t_admit = ck->t_admit[s];
    rec.res.t_finish = (double)(long long)(m->fin_time[s] - sv->gt0) * 1e-9;
    rec.res.energy = m->energy[s] / 2.0 / (double)ck->N;
    rec.res.sim_time = m->fin_clock[s];
    if (ck->result_host[s]) {
      // float64 copy of the final velocity through the slot's RHS buffer
      const T* uf = ck->u[m->fin_parity[s]] + s * 3 * ck->N;
      double* stage = reinterpret_cast<double*>(ck->rhs + s * 3 * ck->N);
      cudaError_t e = cudaSuccess;
      if (sizeof(T) == sizeof(double)) {
        e = cudaMemcpyAsync(ck->result_host[s], uf, 3 * ck->N * sizeof(double), cudaMemcpyDeviceToHost, ck->stream);
      } else {
        // rhs slot (3N floats) holds half: convert and copy component by component
        for (int c = 0; c < 3 && e == cudaSuccess; ++c) {
          e = launch_convert<T, double>(ck->N, uf + c * ck->N, stage, ck->stream);
          if (e == cudaSuccess)
            e = cudaMemcpyAsync(ck->result_host[s] + c * ck->N, stage, ck->N * sizeof(double), cudaMemcpyDeviceToHost,
                                ck->stream);
        }
      }
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&rec.ev, cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventRecord(rec.ev, ck->stream);
      if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
    }
    sv->finishing.push_back(rec);
    ck->slot_id[s] = -1;
    ck->result_host[s] = nullptr;
  }
  return EXC_OK;
}

// An idle chunk with solves that have steps left: one loop launch.
template <typename T>
static int launch_chunk(exc_server* sv, Chunk<T>* ck) {
  (void)sv;
  if (ck->in_flight || ck->active_count() == 0) return EXC_OK;
  loop_begin_kernel<<<1, SRV_MAXS, 0, ck->stream>>>(ck->S, ck->ctl, ck->active);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaGraphLaunch(ck->loop, ck->stream);
  if (e == cudaSuccess) e = cudaEventRecord(ck->done_ev, ck->stream);
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  ck->in_flight = true;
  ck->ticks++;
  return EXC_OK;
}

// Solves of grid size n in the chunks (admitted and not yet retired).
static int active_of_size(const exc_server* sv, int n) {
  int c = 0;
  for (auto& cb : sv->chunks)
    if (cb->n == n) c += cb->active_count();
  return c;
}

template <typename T>
static int server_tick(exc_server* sv, int* active, int* queued) {
  // chunks whose loop launch has ended: report and free their retired solves
  for (auto& cb : sv->chunks) {
    int rc = collect_chunk<T>(sv, static_cast<Chunk<T>*>(cb.get()));
    if (rc) return rc;
  }
  // admission (continuous batching): any queued request that fits, in
  // arrival order; with an admission bound a request also waits while its
  // grid size has max_active_per_size solves running.  When a request waits
  // for memory, idle chunks (no active slot) are released once
  for (int pass = 0; pass < 2; ++pass) {
    bool blocked = false;
    for (size_t i = 0; i < sv->pending.size();) {
      if (sv->max_active_per_size > 0 && active_of_size(sv, sv->pending[i].req.n) >= sv->max_active_per_size) {
        ++i;
        continue;
      }
      bool ok = false, waiting = false;
      int rc = admit<T>(sv, sv->pending[i], &ok, &waiting);
      if (rc) return rc;
      if (ok) sv->pending.erase(sv->pending.begin() + i);
      else if (waiting) ++i;  // a slot frees when a running chunk is collected
      else { blocked = true; ++i; }
    }
    if (!blocked || pass == 1) break;
    bool freed = false;
    for (size_t c = 0; c < sv->chunks.size();) {
      if (sv->chunks[c]->active_count() == 0) {
        sv->used -= sv->chunks[c]->bytes;
        sv->chunks.erase(sv->chunks.begin() + c);  // synchronises its stream
        freed = true;
      } else {
        ++c;
      }
    }
    if (!freed) break;
  }
  // every idle chunk with work runs its device-side loop
  int act = 0;
  for (auto& cb : sv->chunks) {
    int rc = launch_chunk<T>(sv, static_cast<Chunk<T>*>(cb.get()));
    if (rc) return rc;
    act += cb->active_count();
  }
  sv->ticks++;
  if (active) *active = act;
  if (queued) *queued = (int)sv->pending.size();
  return EXC_OK;
}

}  // namespace exc

using namespace exc;

extern "C" {

int exc_server_create(const exc_server_desc* desc, exc_server** out) {
  if (!desc || !out) { set_last_error("null argument"); return EXC_ERR_ARG; }
  *out = nullptr;
  if (desc->precision != EXC_F64 && desc->precision != EXC_F32) { set_last_error("bad precision"); return EXC_ERR_ARG; }
  if (!(desc->mem_fraction > 0) || desc->mem_fraction > 0.95) { set_last_error("mem_fraction must be in (0, 0.95]"); return EXC_ERR_ARG; }
  int rc = configure_device();
  if (rc) return rc;
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { set_last_error("cudaMemGetInfo failed"); return EXC_ERR_CUDA; }
  auto sv = new exc_server();
  sv->desc = *desc;
  sv->budget = (size_t)(desc->mem_fraction * (double)fr);
  if (desc->max_bytes > 0 && desc->max_bytes < (double)sv->budget) sv->budget = (size_t)desc->max_bytes;
  sv->t0 = std::chrono::steady_clock::now();
  if (cudaStreamCreateWithFlags(&sv->admit_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&sv->ev0) != cudaSuccess ||
      cudaMalloc(&sv->init_part, (SHELL_BLOCKS * 1024 + 2048) * sizeof(double)) != cudaSuccess) {
    delete sv;
    set_last_error("cannot create server resources");
    return EXC_ERR_CUDA;
  }
  // time origin: the GPU global timer read by a kernel, then the host clock
  // (finish times come from the global timer, submit/admit times from the host)
  unsigned long long* gt = reinterpret_cast<unsigned long long*>(sv->init_part);
  global_ns_kernel<<<1, 1, 0, sv->admit_stream>>>(gt);
  cudaError_t e = cudaMemcpyAsync(&sv->gt0, gt, sizeof(sv->gt0), cudaMemcpyDeviceToHost, sv->admit_stream);
  if (e == cudaSuccess) e = cudaEventRecord(sv->ev0, sv->admit_stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(sv->ev0);
  if (e != cudaSuccess) {
    exc_server_destroy(sv);
    set_last_error(cudaGetErrorString(e));
    return EXC_ERR_CUDA;
  }
  sv->t0 = std::chrono::steady_clock::now();
  *out = sv;
  return EXC_OK;
}

int exc_server_destroy(exc_server* sv) {
  if (!sv) return EXC_OK;
  cudaDeviceSynchronize();
  sv->chunks.clear();
  for (auto& r : sv->finishing)
    if (r.ev) cudaEventDestroy(r.ev);
  if (sv->spec3) cudaFree(sv->spec3);
  if (sv->init_part) cudaFree(sv->init_part);
  if (sv->ev0) cudaEventDestroy(sv->ev0);
  if (sv->admit_stream) cudaStreamDestroy(sv->admit_stream);
  delete sv;
  return EXC_OK;
}

int exc_server_set_admission(exc_server* sv, int max_active_per_size) {
  if (!sv || max_active_per_size < 0) { set_last_error("null server or negative bound"); return EXC_ERR_ARG; }
  sv->max_active_per_size = max_active_per_size;
  return EXC_OK;
}

int exc_server_submit(exc_server* sv, const exc_solve_req* req, int64_t* id) {
  if (!sv || !req) { set_last_error("null argument"); return EXC_ERR_ARG; }
  if (!fft_size_ok(req->n)) { set_last_error("grid size must be 2^a 3^b 5^c 7^d 11^e 13^f 17^g, a >= 1, 4 <= n <= 1024"); return EXC_ERR_SHAPE; }
  if (!(req->l > 0) || !(req->visc > 0) || !(req->cfl > 0) || !(req->kpeak > 0) || !(req->energy > 0) ||
      req->nsteps < 1) {
    set_last_error("bad request parameters");
    return EXC_ERR_ARG;
  }
  PendingReq pr;
  pr.id = sv->next_id++;
  pr.req = *req;
  pr.t_submit = sv->now();
  sv->pending.push_back(pr);
  if (id) *id = pr.id;
  return EXC_OK;
}

int exc_server_tick(exc_server* sv, int* active, int* queued) {
  if (!sv) { set_last_error("null argument"); return EXC_ERR_ARG; }
  return sv->desc.precision == EXC_F64 ? server_tick<double>(sv, active, queued) : server_tick<float>(sv, active, queued);
}

int exc_server_poll(exc_server* sv, exc_solve_result* out, int max, int* count) {
  if (!sv || !count || (max > 0 && !out)) { set_last_error("bad argument"); return EXC_ERR_ARG; }
  int c = 0;
  for (size_t i = 0; i < sv->finishing.size() && c < max;) {
    FinishRec& r = sv->finishing[i];
    if (r.ev) {
      // the final field is still on its way to the caller's buffer
      cudaError_t q = cudaEventQuery(r.ev);
      if (q == cudaErrorNotReady) { ++i; continue; }
      if (q != cudaSuccess) { set_last_error(cudaGetErrorString(q)); return EXC_ERR_CUDA; }
      cudaEventDestroy(r.ev);
    }
    out[c++] = r.res;
    sv->finishing.erase(sv->finishing.begin() + i);
  }
  *count = c;
  return EXC_OK;
}

int exc_server_drain(exc_server* sv) {
  if (!sv) { set_last_error("null argument"); return EXC_ERR_ARG; }
  int idle_ticks = 0;
  for (;;) {
    int act = 0, q = 0;
    int rc = exc_server_tick(sv, &act, &q);
    if (rc) return rc;
    if (act == 0 && q == 0) break;
    // solves retired in this tick free their slots for the next one; only a
    // second tick without any admitted solve means the queue cannot be served
    idle_ticks = act == 0 ? idle_ticks + 1 : 0;
    if (act > 0) std::this_thread::yield();  // loops run on the device meanwhile
    if (idle_ticks >= 2) { set_last_error("queued requests cannot be admitted (memory budget)"); return EXC_ERR_OOM; }
  }
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return EXC_ERR_CUDA; }
  return EXC_OK;
}

int exc_server_stats(exc_server* sv, exc_server_info* st) {
  if (!sv || !st) { set_last_error("null argument"); return EXC_ERR_ARG; }
  st->chunks = (int)sv->chunks.size();
  st->slots = 0;
  st->active = 0;
  st->kernels_per_tick = 0;
  for (auto& cb : sv->chunks) {
    st->slots += cb->S;
    st->active += cb->active_count();
  }
  st->queued = (int)sv->pending.size();
  st->bytes_used = (double)sv->used;
  st->bytes_budget = (double)sv->budget;
  st->ticks = (double)sv->ticks;
  st->clock = sv->now();
  return EXC_OK;
}

int exc_server_tuning(int precision, int n, int slots, int* engine, int* col_w, int* x_rows) {
  if (!engine || !col_w || !x_rows) { set_last_error("null argument"); return EXC_ERR_ARG; }
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tuned.find(std::make_tuple(n, precision, slots));
  if (it == g_tuned.end()) { set_last_error("no tuning recorded for this size"); return EXC_ERR_STATE; }
  *engine = it->second.engine;
  if (it->second.engine == 0) {
    fftreg_geometry(n, precision, col_w, x_rows);
  } else {
    *col_w = it->second.col_w;
    *x_rows = it->second.x_rows;
  }
  return EXC_OK;
}

}  // extern "C"
