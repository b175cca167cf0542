// Newmark (beta = 1/4, gamma = 1/2) time loop with a device-side PCG per step.
//
// Replaces the PuggleSolvers NewmarkExplicit loop driven by scatter/scatter.py:133-159.
// Per step t -> t+1 (acceleration form of the same update):
//   vp = v + dt/2 a,  up = u + dt v + dt^2/4 a
//   A x = f(t+1) - C vp - K up,          A = M + dt/2 C + dt^2/4 K
//   u = up + dt^2/4 x,  v = vp + dt/2 x,  a = x
// x is found by Jacobi-PCG stopped at ||r|| <= rtol ||rhs||, warm-started from the polynomial
// extrapolation of the previous accelerations (x0 = sum_k (-1)^k C(p+1, k+1) a_{n-k}, order p
// fixed by the caller or adapted on the device to the iteration counts: warm_start_* in
// sc_common.cuh, shared with the node-block solver).
//
// Execution: one CUDA graph per step: [force, predict, residual] -> WHILE{spmv, update,
// direction} -> [finalize, record, advance].  The WHILE node is a graph conditional whose
// value the residual and update kernels set on the device (converged / iteration cap /
// breakdown), so a step costs exactly the iterations it needs with no host round trip.  Reductions are per-block
// partials summed by the last block to finish (ticket counter, no spin-waits), in a fixed
// order, so every run is bitwise reproducible.  Matrices are CSR over the reference's
// equation numbering with a shared element-graph pattern.
#include <vector>

#include "sc_common.cuh"

namespace sc {

constexpr int kRowThreads = 256;  // 8 warps
// A row takes kRowLanes lanes (a warp takes kRowsPerWarp rows at once): on GB300 an FP64 warp
// instruction costs ~16 SM cycles, and with a whole warp per row the 5-step FP64 warp
// reduction and the partly idle last FMA pass cost more than the row's own FMAs (an 81-entry
// hexa8 row: 9 FP64 warp instructions; with 4 lanes about 3).  The 4 lanes of a row read 32
// contiguous bytes of values per pass.
constexpr int kRowLanes = 4, kRowsPerWarp = 32 / kRowLanes;

// sum over the kRowLanes lanes of a row (all 32 lanes call it); every lane of the row gets it
__device__ __forceinline__ double row_sum(double v) {
#pragma unroll
  for (int o = 1; o < kRowLanes; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

struct NmScalars {
  double rz, pw, rr, bb, alpha, beta, tol2;
  double ref_avg;  // warm start: mean iterations per step of the reference window
  long long total_iters;
  int it, max_it, max_seen, status, t;
  int hist;  // valid previous accelerations (0..kHistMax) for the warm start
  int head;  // ring slot of the most recent one (hist_slot)
  unsigned int ticket;
  // adaptive warm-start order: current order, probing direction, window and hold counters
  int pord, pdir, win_n, win_it, probing, hold;
  int pcap;          // this step's cap on the order from the force history (warm_start_order_cap)
  long long capped;  // steps whose order the cap lowered
};

struct NmArgs {
  int64_t n;
  const int64_t* rowptr;
  const int* cols;
  const double *M, *C, *K, *A;
  double *u, *v, *a;
  double *vp, *up, *x, *r, *z, *p, *w, *dinv, *f;
  double* ah[kHistMax];  // previous accelerations, a ring: a_{n-1-k} in ah[hist_slot(head, k)]
  int pred_order;        // warm-start order (1..kHistMax), 0: adaptive (NmScalars::pord)
  int order_cap;         // 1: cap the order where the force history has a kink (default)
  double* part;          // [nblocks][4]
  NmScalars* s;
  double dt;
  // force table
  int n_t;
  const int64_t* f_ptr;
  const int* f_eq;
  const double* f_val;
  // output
  int out_interval, n_rec;
  const int* rec_eq;
  double *out_u, *out_v, *out_a;
  int64_t n_out;
  float2* p2;  // p as (hi, lo) FP32 pairs for the pair SpMV, written with p (null: FP64 SpMV)
};

// returns true in every thread of the last block to arrive
__device__ inline bool last_block(unsigned int* ticket) {
  __shared__ bool am_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) am_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  return am_last;
}

// sum column k of part[nb][4] in the last block, fixed order; result in thread 0
__device__ inline double reduce_parts(const double* part, int k, double* sh) {
  double s = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s += __ldcg(part + b * 4 + k);
  return block_sum(s, sh);
}

__global__ void k_force(NmArgs g) {
  // clear the entries of step t, write those of step t+1 (dense f); then the warm start's order
  // cap from the force history (one block)
  const int t = g.s->t;
  if (g.f_ptr != nullptr) {
    if (t >= 0 && t < g.n_t)
      for (int64_t k = g.f_ptr[t] + threadIdx.x; k < g.f_ptr[t + 1]; k += blockDim.x) g.f[g.f_eq[k]] = 0.0;
    __syncthreads();
    const int t1 = t + 1;
    if (t1 >= 0 && t1 < g.n_t)
      for (int64_t k = g.f_ptr[t1] + threadIdx.x; k < g.f_ptr[t1 + 1]; k += blockDim.x)
        g.f[g.f_eq[k]] += g.f_val[k];
  }
  warm_start_order_cap(g.s, g.pred_order, g.order_cap, ForceRows{g.n_t, g.f_ptr, g.f_eq, g.f_val});
}

// vp, up ; the warm start x0 into w (w is scratch until the first k_spmv of the step)
__global__ void k_predict(NmArgs g) {
  const double dt = g.dt, h = 0.5 * dt, q = 0.25 * dt * dt;
  const int p0 = warm_start_order(g.s, g.pred_order);
  const int p = g.s->pcap < p0 ? g.s->pcap : p0;  // the force history's cap
  double cf[kHistMax + 1];
  warm_start_coeffs(p, cf);
  const double* hs[kHistMax];  // a_{n-1-k}
#pragma unroll
  for (int k = 0; k < kHistMax; ++k) hs[k] = g.ah[hist_slot(g.s->head, k)];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += (int64_t)gridDim.x * blockDim.x) {
    const double ai = g.a[i], vi = g.v[i];
    g.vp[i] = vi + h * ai;
    g.up[i] = g.u[i] + dt * vi + q * ai;
    double x0 = cf[0] * ai;  // terms summed in a fixed order
#pragma unroll
    for (int k = 1; k <= kHistMax; ++k)
      if (k <= p) x0 += cf[k] * hs[k - 1][i];
    g.w[i] = x0;
  }
}

// rhs = f - C vp - K up ; r = rhs - Op x0 ; z = dinv r ; p = z.  mode 0: x0 = w (the warm
// start, step), mode 1: x0 = 0 (initial acceleration, Op = M, vp/up point at v/u).
__global__ void __launch_bounds__(kRowThreads) k_residual(NmArgs g, const double* __restrict__ Op, int mode,
                                                          cudaGraphConditionalHandle hc) {
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31, sub = lane % kRowLanes;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const double* __restrict__ vp = mode == 0 ? g.vp : g.v;
  const double* __restrict__ up = mode == 0 ? g.up : g.u;
  double prz = 0, prr = 0, pbb = 0;
  // the loop bound depends on the warp only, so all 32 lanes reach the shuffles
  for (int64_t rb = gw * kRowsPerWarp; rb < g.n; rb += nw * kRowsPerWarp) {
    const int64_t row = rb + lane / kRowLanes;
    const bool live = row < g.n;
    double sr = 0.0, sa = 0.0;
    if (live) {
      const int64_t k0 = g.rowptr[row], k1 = g.rowptr[row + 1];
      for (int64_t k = k0 + sub; k < k1; k += kRowLanes) {
        const int c = g.cols[k];
        sr = fma(g.C[k], vp[c], sr);
        sr = fma(g.K[k], up[c], sr);
        if (mode == 0) sa = fma(Op[k], g.w[c], sa);
      }
    }
    sr = row_sum(sr);
    sa = row_sum(sa);
    if (live && sub == 0) {
      const double rhs = g.f[row] - sr;
      const double r = rhs - sa;
      const double z = g.dinv[row] * r;
      g.x[row] = mode == 0 ? g.w[row] : 0.0;
      g.r[row] = r;
      g.z[row] = z;
      g.p[row] = z;
      if (g.p2) g.p2[row] = split_pair(z);
      prz += r * z;
      prr += r * r;
      pbb += rhs * rhs;
    }
  }
  double t = block_sum(prz, sh);
  if (threadIdx.x == 0) g.part[blockIdx.x * 4 + 0] = t;
  t = block_sum(prr, sh);
  if (threadIdx.x == 0) g.part[blockIdx.x * 4 + 1] = t;
  t = block_sum(pbb, sh);
  if (threadIdx.x == 0) g.part[blockIdx.x * 4 + 2] = t;
  if (last_block(&g.s->ticket)) {
    const double rz = reduce_parts(g.part, 0, sh);
    const double rr = reduce_parts(g.part, 1, sh);
    const double bb = reduce_parts(g.part, 2, sh);
    if (threadIdx.x == 0) {
      NmScalars* s = g.s;
      s->rz = rz;
      s->rr = rr;
      s->bb = bb;
      s->it = 0;
      s->ticket = 0;
      const bool done = rr <= s->tol2 * bb;
      cudaGraphSetConditional(hc, done ? 0u : 1u);
    }
  }
}

// w = Op p ; partial p.w ; last block: alpha = rz / pw.  kInGraph = false is the same
// kernel for standalone timing (it does not touch the graph conditional).  kPair: the operator
// as FP32 (hi, lo) pairs (Op2, 8 bytes per value like FP64) and p as pairs (g.p2); the products
// and the row's 4-lane sum in pair arithmetic (about 48 bits), no FP64 instruction per entry.
template <bool kInGraph, bool kPair>
__global__ void __launch_bounds__(kRowThreads) k_spmv(NmArgs g, const double* __restrict__ Op,
                                                      const float2* __restrict__ Op2,
                                                      cudaGraphConditionalHandle hc) {
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31, sub = lane % kRowLanes;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double ppw = 0.0;
  for (int64_t rb = gw * kRowsPerWarp; rb < g.n; rb += nw * kRowsPerWarp) {
    const int64_t row = rb + lane / kRowLanes;
    const bool live = row < g.n;
    double s = 0.0;
    if (kPair) {
      float hi = 0.f, lo = 0.f;
      if (live) {
        const int64_t k0 = g.rowptr[row], k1 = g.rowptr[row + 1];
        for (int64_t k = k0 + sub; k < k1; k += kRowLanes) {
          const float2 a = __ldcs(Op2 + k);
          pair_fma(a.x, a.y, g.p2[__ldcs(g.cols + k)], hi, lo);
        }
      }
#pragma unroll
      for (int o = 1; o < kRowLanes; o <<= 1) {
        const float h2 = __shfl_xor_sync(0xffffffffu, hi, o), l2 = __shfl_xor_sync(0xffffffffu, lo, o);
        pair_add(hi, lo, h2, l2);
      }
      s = (double)hi + (double)lo;
    } else {
      if (live) {
        const int64_t k0 = g.rowptr[row], k1 = g.rowptr[row + 1];
        for (int64_t k = k0 + sub; k < k1; k += kRowLanes) s = fma(__ldcs(Op + k), g.p[__ldcs(g.cols + k)], s);
      }
      s = row_sum(s);
    }
    if (live && sub == 0) {
      g.w[row] = s;
      ppw += g.p[row] * s;
    }
  }
  const double t = block_sum(ppw, sh);
  if (threadIdx.x == 0) g.part[blockIdx.x * 4 + 3] = t;
  if (last_block(&g.s->ticket)) {
    const double pw = reduce_parts(g.part, 3, sh);
    if (threadIdx.x == 0) {
      NmScalars* s = g.s;
      s->ticket = 0;
      s->pw = pw;
      if (!kInGraph) {
        // standalone timing launch: leave the solver's scalars untouched
      } else if (!(pw > 0.0)) {  // not SPD along p (or NaN): stop this solve, keep x
        s->alpha = 0.0;
        s->status = SC_BREAKDOWN;
        cudaGraphSetConditional(hc, 0u);
      } else {
        s->alpha = s->rz / pw;
      }
    }
  }
}

// x += alpha p ; r -= alpha w ; z = dinv r ; partial r.z, r.r ; last block: beta, test
__global__ void k_update(NmArgs g, cudaGraphConditionalHandle hc) {
  __shared__ double sh[32];
  const double alpha = g.s->alpha;
  double prz = 0.0, prr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += (int64_t)gridDim.x * blockDim.x) {
    const double pi = g.p[i];
    g.x[i] = fma(alpha, pi, g.x[i]);
    const double r = fma(-alpha, g.w[i], g.r[i]);
    g.r[i] = r;
    const double z = g.dinv[i] * r;
    g.z[i] = z;
    prz += r * z;
    prr += r * r;
  }
  double t = block_sum(prz, sh);
  if (threadIdx.x == 0) g.part[blockIdx.x * 4 + 0] = t;
  t = block_sum(prr, sh);
  if (threadIdx.x == 0) g.part[blockIdx.x * 4 + 1] = t;
  if (last_block(&g.s->ticket)) {
    const double rz = reduce_parts(g.part, 0, sh);
    const double rr = reduce_parts(g.part, 1, sh);
    if (threadIdx.x == 0) {
      NmScalars* s = g.s;
      s->ticket = 0;
      s->beta = s->rz != 0.0 ? rz / s->rz : 0.0;
      s->rz = rz;
      s->rr = rr;
      s->it += 1;
      bool done = rr <= s->tol2 * s->bb;
      if (!done && s->it >= s->max_it) {
        s->status = s->status ? s->status : SC_NOT_CONVERGED;
        done = true;
      }
      if (s->status == SC_BREAKDOWN) done = true;
      if (done) cudaGraphSetConditional(hc, 0u);
    }
  }
}

__global__ void k_direction(NmArgs g) {
  const double beta = g.s->beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += (int64_t)gridDim.x * blockDim.x) {
    const double pv = fma(beta, g.p[i], g.z[i]);
    g.p[i] = pv;
    if (g.p2) g.p2[i] = split_pair(pv);
  }
}

__global__ void k_to_pairs(int64_t n, const double* __restrict__ x, float2* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = split_pair(x[i]);
}

__device__ inline void record(const NmArgs& g, int step) {
  if (g.n_rec <= 0 || g.out_interval <= 0 || step % g.out_interval) return;
  const int64_t row = step / g.out_interval;
  if (row >= g.n_out) return;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < g.n_rec; j += (int64_t)gridDim.x * blockDim.x) {
    const int e = g.rec_eq[j];
    if (g.out_u) g.out_u[row * g.n_rec + j] = g.u[e];
    if (g.out_v) g.out_v[row * g.n_rec + j] = g.v[e];
    if (g.out_a) g.out_a[row * g.n_rec + j] = g.a[e];
  }
}

// u = up + dt^2/4 x ; v = vp + dt/2 x ; a into the history ring (k_advance moves its head) ; a = x
__global__ void k_finalize(NmArgs g) {
  const double h = 0.5 * g.dt, q = 0.25 * g.dt * g.dt;
  double* __restrict__ slot = g.ah[hist_slot(g.s->head, kHistMax - 1)];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += (int64_t)gridDim.x * blockDim.x) {
    const double x = g.x[i];
    g.u[i] = fma(q, x, g.up[i]);
    g.v[i] = fma(h, x, g.vp[i]);
    slot[i] = g.a[i];
    g.a[i] = x;
  }
}

__global__ void k_record(NmArgs g, int bump) {
  // runs after k_finalize: step index t+1 is the state just computed
  const int step = g.s->t + bump;
  record(g, step);
  __syncthreads();
  if (bump && blockIdx.x == 0 && threadIdx.x == 0) {
    NmScalars* s = g.s;
    s->total_iters += s->it;
    if (s->it > s->max_seen) s->max_seen = s->it;
  }
}

// t += 1 ; the step's iterations into the warm start's order control
__global__ void k_advance(NmArgs g) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    NmScalars* s = g.s;
    s->t += 1;
    warm_start_advance(s, g.pred_order);
  }
}

__global__ void k_cap_hist(NmScalars* s, int n) {
  if (s->hist > n) s->hist = n;
}

// initial acceleration: a = x after CG on M
__global__ void k_copy_x_to_a(NmArgs g) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += (int64_t)gridDim.x * blockDim.x)
    g.a[i] = g.x[i];
}

__global__ void k_dinv(int64_t n, const int64_t* __restrict__ rowptr, const int* __restrict__ cols,
                       const double* __restrict__ Op, double* __restrict__ dinv, int* __restrict__ bad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double d = 0.0;
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
      if (cols[k] == i) d = Op[k];
    if (!(d > 0.0)) {
      atomicExch(bad, 1);
      d = 1.0;
    }
    dinv[i] = 1.0 / d;
  }
}

__global__ void k_init_scalars(NmScalars* s, double tol2, int max_it) {
  s->rz = s->pw = s->rr = s->bb = s->alpha = s->beta = 0.0;
  s->tol2 = tol2;
  s->total_iters = 0;
  s->it = 0;
  s->max_it = max_it;
  s->max_seen = 0;
  s->status = SC_OK;
  s->t = 0;
  s->ticket = 0;
  warm_start_init(s);
}

__global__ void k_set_t(NmScalars* s, int t) { s->t = t; }

}  // namespace sc

using namespace sc;

struct sc_newmark {
  NmArgs g;
  cudaStream_t user = nullptr, cap = nullptr, cap2 = nullptr;
  unsigned row_blocks = 1, vec_blocks = 1;
  cudaGraphExec_t step_exec = nullptr, init_exec = nullptr;
  cudaGraph_t step_graph = nullptr, init_graph = nullptr;
  double rtol = 1e-12;
  int pair = 1;                                 // SpMV in FP32-pair arithmetic (sc_newmark_set_options bit 0 clears)
  float2 *AP = nullptr, *MP = nullptr;          // A and M as pairs, made with the first graph
  float2* p2 = nullptr;
};

namespace {

// Build [pre] -> WHILE{spmv, update, direction} -> [post] for operator Op.
int build_pcg_graph(sc_newmark* h, const double* Op, int mode, cudaGraph_t* graph_out, cudaGraphExec_t* exec_out) {
  cudaGraph_t graph = nullptr;
  int rc = check(cudaGraphCreate(&graph, 0), "cudaGraphCreate");
  if (rc) return rc;
  cudaGraphConditionalHandle hc;
  if ((rc = check(cudaGraphConditionalHandleCreate(&hc, graph, 1, cudaGraphCondAssignDefault), "handle"))) {
    cudaGraphDestroy(graph);
    return rc;
  }
  NmArgs g = h->g;
  cudaStream_t cs = h->cap;
  do {
    if ((rc = check(cudaStreamBeginCaptureToGraph(cs, graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
                    "capture pre")))
      break;
    if (mode == 0) {
      k_force<<<1, 256, 0, cs>>>(g);
      k_predict<<<h->vec_blocks, 256, 0, cs>>>(g);
    }
    k_residual<<<h->row_blocks, kRowThreads, 0, cs>>>(g, Op, mode, hc);
    cudaStreamCaptureStatus stt;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    if ((rc = check(cudaStreamGetCaptureInfo(cs, &stt, nullptr, nullptr, &deps, nullptr, &ndeps), "capture info")))
      break;
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = hc;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cnode;
    if ((rc = check(cudaGraphAddNode(&cnode, graph, deps, nullptr, ndeps, &cp), "add conditional"))) break;
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    if ((rc = check(cudaStreamUpdateCaptureDependencies(cs, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies),
                    "update deps")))
      break;
    // body, captured on a second stream
    if ((rc = check(cudaStreamBeginCaptureToGraph(h->cap2, body, nullptr, nullptr, 0,
                                                  cudaStreamCaptureModeThreadLocal),
                    "capture body")))
      break;
    if (g.p2) {
      const float2* Op2 = Op == g.M ? h->MP : h->AP;
      k_spmv<true, true><<<h->row_blocks, kRowThreads, 0, h->cap2>>>(g, Op, Op2, hc);
    } else {
      k_spmv<true, false><<<h->row_blocks, kRowThreads, 0, h->cap2>>>(g, Op, nullptr, hc);
    }
    k_update<<<h->vec_blocks, 256, 0, h->cap2>>>(g, hc);
    k_direction<<<h->vec_blocks, 256, 0, h->cap2>>>(g);
    cudaGraph_t body_out = nullptr;
    if ((rc = check(cudaStreamEndCapture(h->cap2, &body_out), "end body"))) break;
    // post
    if (mode == 0) {
      k_finalize<<<h->vec_blocks, 256, 0, cs>>>(g);
      k_record<<<h->vec_blocks, 256, 0, cs>>>(g, 1);
      k_advance<<<1, 32, 0, cs>>>(g);
    } else {
      k_copy_x_to_a<<<h->vec_blocks, 256, 0, cs>>>(g);
      k_record<<<h->vec_blocks, 256, 0, cs>>>(g, 0);
    }
    cudaGraph_t out = nullptr;
    if ((rc = check(cudaStreamEndCapture(cs, &out), "end capture"))) break;
    if ((rc = check(cudaGraphInstantiate(exec_out, graph, 0), "instantiate"))) break;
  } while (0);
  if (rc) {
    cudaStreamCaptureStatus st;
    if (cudaStreamIsCapturing(cs, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) {
      cudaGraph_t tmp;
      cudaStreamEndCapture(cs, &tmp);
    }
    if (cudaStreamIsCapturing(h->cap2, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) {
      cudaGraph_t tmp;
      cudaStreamEndCapture(h->cap2, &tmp);
    }
    cudaGetLastError();
    cudaGraphDestroy(graph);
    return rc;
  }
  *graph_out = graph;
  return SC_OK;
}

// graphs bake in the kernel arguments: rebuilt lazily after a change
void drop_graphs(sc_newmark* h) {
  if (h->step_exec) cudaGraphExecDestroy(h->step_exec), h->step_exec = nullptr;
  if (h->step_graph) cudaGraphDestroy(h->step_graph), h->step_graph = nullptr;
  if (h->init_exec) cudaGraphExecDestroy(h->init_exec), h->init_exec = nullptr;
  if (h->init_graph) cudaGraphDestroy(h->init_graph), h->init_graph = nullptr;
}

unsigned row_blocks_for(int64_t n) {
  // kRowsPerWarp rows per warp, 8 warps per block, grid-stride; at most 16 blocks of 256 per SM
  const int64_t rows_per_block = (int64_t)kRowsPerWarp * (kRowThreads / 32);
  int64_t b = (n + rows_per_block - 1) / rows_per_block;
  const int64_t cap = 152 * 16;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

}  // namespace

extern "C" int64_t sc_newmark_workspace_doubles(int64_t n_eq, int64_t) {
  // vp up x r z p w dinv f  +  history ah[kHistMax]  +  part[blocks][4]  +  scalars
  return (9 + kHistMax) * n_eq + 4 * (int64_t)row_blocks_for(n_eq) + 4 * 152 * 16 + 64;
}

extern "C" int sc_newmark_create(sc_newmark** out, int64_t n_eq, const int64_t* rowptr, const int* cols,
                                 const double* M, const double* C, const double* K, double* A, double dt, double rtol,
                                 int max_iter, double* u, double* v, double* a, double* ws, int64_t ws_doubles,
                                 void* stream) {
  if (!out || n_eq <= 0 || !rowptr || !cols || !M || !C || !K || !A || !u || !v || !a || !ws) return SC_BAD_ARG;
  if (!(dt > 0.0) || !(rtol > 0.0) || max_iter <= 0) return SC_BAD_ARG;
  if (ws_doubles < sc_newmark_workspace_doubles(n_eq, 0)) return SC_BAD_ARG;
  if ((((uintptr_t)ws) & 15) != 0) return SC_BAD_ARG;
  sc_newmark* h = new sc_newmark();
  h->user = (cudaStream_t)stream;
  h->rtol = rtol;
  NmArgs& g = h->g;
  g = NmArgs{};
  g.n = n_eq;
  g.rowptr = rowptr;
  g.cols = cols;
  g.M = M;
  g.C = C;
  g.K = K;
  g.A = A;
  g.u = u;
  g.v = v;
  g.a = a;
  double* p = ws;
  g.vp = p; p += n_eq;
  g.up = p; p += n_eq;
  g.x = p; p += n_eq;
  g.r = p; p += n_eq;
  g.z = p; p += n_eq;
  g.p = p; p += n_eq;
  g.w = p; p += n_eq;
  g.dinv = p; p += n_eq;
  g.f = p; p += n_eq;
  for (int k = 0; k < kHistMax; ++k) {
    g.ah[k] = p;
    p += n_eq;
  }
  g.pred_order = 0;  // adaptive
  g.order_cap = 1;
  h->row_blocks = row_blocks_for(n_eq);
  h->vec_blocks = grid_for(n_eq, 256, 152 * 16);
  g.part = p; p += 4 * (int64_t)(h->row_blocks > h->vec_blocks ? h->row_blocks : h->vec_blocks);
  // scalars on a 64-byte boundary
  uintptr_t sp = ((uintptr_t)p + 63) & ~(uintptr_t)63;
  g.s = (NmScalars*)sp;
  g.dt = dt;
  cudaStream_t st = h->user;
  int rc = SC_OK;
  int* bad = nullptr;
  do {
    if ((rc = check(cudaStreamCreateWithFlags(&h->cap, cudaStreamNonBlocking), "stream"))) break;
    if ((rc = check(cudaStreamCreateWithFlags(&h->cap2, cudaStreamNonBlocking), "stream"))) break;
    // A = M + dt/2 C + dt^2/4 K on the shared pattern
    int64_t nnz = 0;
    if ((rc = check(cudaMemcpyAsync(&nnz, rowptr + n_eq, sizeof(int64_t), cudaMemcpyDeviceToHost, st), "nnz"))) break;
    if ((rc = check(cudaStreamSynchronize(st), "sync"))) break;
    if ((rc = sc_combine(nnz, 1.0, M, 0.5 * dt, C, 0.25 * dt * dt, K, A, st))) break;
    if ((rc = check(cudaMemsetAsync(g.f, 0, sizeof(double) * n_eq, st), "memset f"))) break;
    if ((rc = check(cudaMemsetAsync(g.ah[0], 0, sizeof(double) * n_eq * kHistMax, st), "memset history"))) break;
    if ((rc = check(cudaMallocAsync((void**)&bad, sizeof(int), st), "malloc"))) break;
    if ((rc = check(cudaMemsetAsync(bad, 0, sizeof(int), st), "memset"))) break;
    k_dinv<<<h->vec_blocks, 256, 0, st>>>(n_eq, rowptr, cols, A, g.dinv, bad);
    k_init_scalars<<<1, 1, 0, st>>>(g.s, rtol * rtol, max_iter);
    if ((rc = check_launch("newmark init"))) break;
    int hb = 0;
    if ((rc = check(cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, st), "memcpy"))) break;
    if ((rc = check(cudaStreamSynchronize(st), "sync"))) break;
    if (hb) {
      rc = SC_BAD_ARG;  // effective matrix has a non-positive diagonal
      break;
    }
  } while (0);
  if (bad) {
    cudaFreeAsync(bad, st);
    cudaStreamSynchronize(st);
  }
  if (rc) {
    sc_newmark_destroy(h);
    return rc;
  }
  *out = h;
  return SC_OK;
}

extern "C" int sc_newmark_set_force(sc_newmark* h, int n_t, const int64_t* f_ptr, const int* f_eq,
                                    const double* f_val) {
  if (!h || n_t < 0 || (n_t > 0 && (!f_ptr || !f_eq || !f_val))) return SC_BAD_ARG;
  h->g.n_t = n_t;
  h->g.f_ptr = n_t > 0 ? f_ptr : nullptr;
  h->g.f_eq = f_eq;
  h->g.f_val = f_val;
  drop_graphs(h);
  return SC_OK;
}

extern "C" int sc_newmark_set_output(sc_newmark* h, int out_interval, int n_rec, const int* rec_eq, double* out_u,
                                     double* out_v, double* out_a, int64_t n_out) {
  if (!h || n_rec < 0 || (n_rec > 0 && (!rec_eq || out_interval <= 0 || n_out <= 0))) return SC_BAD_ARG;
  h->g.out_interval = out_interval;
  h->g.n_rec = n_rec;
  h->g.rec_eq = rec_eq;
  h->g.out_u = out_u;
  h->g.out_v = out_v;
  h->g.out_a = out_a;
  h->g.n_out = n_out;
  drop_graphs(h);
  return SC_OK;
}

namespace {
// A and M as FP32 pairs and the pair copy of p, made before the first graph (pair SpMV only)
int pair_prepare(sc_newmark* h) {
  NmArgs& g = h->g;
  if (!h->pair) {
    g.p2 = nullptr;
    return SC_OK;
  }
  if (!h->AP) {
    cudaStream_t st = h->user;
    int64_t nnz = 0;
    int rc = check(cudaMemcpyAsync(&nnz, g.rowptr + g.n, sizeof(int64_t), cudaMemcpyDeviceToHost, st), "nnz");
    if (!rc) rc = check(cudaStreamSynchronize(st), "sync");
    if (!rc) rc = check(cudaMallocAsync((void**)&h->AP, 8 * (nnz > 0 ? nnz : 1), st), "malloc");
    if (!rc) rc = check(cudaMallocAsync((void**)&h->MP, 8 * (nnz > 0 ? nnz : 1), st), "malloc");
    if (!rc) rc = check(cudaMallocAsync((void**)&h->p2, 8 * g.n, st), "malloc");
    if (rc) return rc;
    k_to_pairs<<<grid_for(nnz, 256, 152 * 32), 256, 0, st>>>(nnz, g.A, h->AP);
    k_to_pairs<<<grid_for(nnz, 256, 152 * 32), 256, 0, st>>>(nnz, g.M, h->MP);
    if ((rc = check_launch("pair planes"))) return rc;
  }
  g.p2 = h->p2;
  return SC_OK;
}
}  // namespace

// options bit 0: the SpMV in FP64 instead of FP32-pair arithmetic; bit 1: no cap on the
// warm-start order at kinks of the force history
extern "C" int sc_newmark_set_options(sc_newmark* h, int options) {
  if (!h || options < 0 || options > 3) return SC_BAD_ARG;
  h->pair = (options & 1) ? 0 : 1;
  h->g.order_cap = (options & 2) ? 0 : 1;
  drop_graphs(h);
  return SC_OK;
}

extern "C" int sc_newmark_warm_start_status(sc_newmark* h, int* order, int64_t* capped_steps) {
  if (!h) return SC_BAD_ARG;
  int rc = check(cudaStreamSynchronize(h->user), "sync status");
  if (rc) return rc;
  NmScalars s;
  if ((rc = check(cudaMemcpy(&s, h->g.s, sizeof(s), cudaMemcpyDeviceToHost), "read scalars"))) return rc;
  if (order) *order = h->g.pred_order > 0 ? h->g.pred_order : s.pord;
  if (capped_steps) *capped_steps = s.capped;
  return SC_OK;
}

// Polynomial order (1..kHistMax; 0: adaptive, the default) of the extrapolated accelerations
// that start each step's PCG: it changes the iteration count, not the converged answer.
extern "C" int sc_newmark_set_predictor(sc_newmark* h, int order) {
  if (!h || order < 0 || order > kHistMax) return SC_BAD_ARG;
  // only the previous fixed order's entries of the history are current (adaptive keeps all)
  if (h->g.pred_order > 0 && (order == 0 || order > h->g.pred_order))
    k_cap_hist<<<1, 1, 0, h->user>>>(h->g.s, h->g.pred_order);
  h->g.pred_order = order;
  drop_graphs(h);
  return check_launch("predictor order");
}

extern "C" int sc_newmark_initial_acceleration(sc_newmark* h) {
  if (!h) return SC_BAD_ARG;
  cudaStream_t st = h->user;
  NmArgs& g = h->g;
  int rc;
  if ((rc = pair_prepare(h))) return rc;
  // f = force(0); the dinv of M for this solve
  if ((rc = check(cudaMemsetAsync(g.f, 0, sizeof(double) * g.n, st), "memset f"))) return rc;
  k_set_t<<<1, 1, 0, st>>>(g.s, -1);
  k_force<<<1, 256, 0, st>>>(g);  // writes step 0 entries (t+1 = 0)
  k_set_t<<<1, 1, 0, st>>>(g.s, 0);
  if ((rc = check_launch("initial force"))) return rc;
  // CG on M with its own Jacobi scaling: swap dinv temporarily
  int* bad = nullptr;
  if ((rc = check(cudaMallocAsync((void**)&bad, sizeof(int), st), "malloc"))) return rc;
  cudaMemsetAsync(bad, 0, sizeof(int), st);
  k_dinv<<<h->vec_blocks, 256, 0, st>>>(g.n, g.rowptr, g.cols, g.M, g.dinv, bad);
  if (!h->init_exec) {
    if ((rc = build_pcg_graph(h, g.M, 1, &h->init_graph, &h->init_exec))) {
      cudaFreeAsync(bad, st);
      return rc;
    }
  }
  rc = check(cudaGraphLaunch(h->init_exec, st), "launch init");
  // restore A's Jacobi scaling
  cudaMemsetAsync(bad, 0, sizeof(int), st);
  k_dinv<<<h->vec_blocks, 256, 0, st>>>(g.n, g.rowptr, g.cols, g.A, g.dinv, bad);
  int hb = 0;
  cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(bad, st);
  int rc2 = check(cudaStreamSynchronize(st), "sync init");
  if (rc) return rc;
  if (rc2) return rc2;
  if (hb) return SC_BAD_ARG;
  NmScalars s;
  if ((rc = check(cudaMemcpy(&s, g.s, sizeof(s), cudaMemcpyDeviceToHost), "read scalars"))) return rc;
  return s.status;
}

extern "C" int sc_newmark_run(sc_newmark* h, int t_begin, int t_end) {
  if (!h || t_begin < 0 || t_end < t_begin) return SC_BAD_ARG;
  int rc;
  if ((rc = pair_prepare(h))) return rc;
  if (!h->step_exec) {
    if ((rc = build_pcg_graph(h, h->g.A, 0, &h->step_graph, &h->step_exec))) return rc;
  }
  k_set_t<<<1, 1, 0, h->user>>>(h->g.s, t_begin);
  if ((rc = check_launch("set t"))) return rc;
  for (int t = t_begin; t < t_end; ++t)
    if ((rc = check(cudaGraphLaunch(h->step_exec, h->user), "launch step"))) return rc;
  return SC_OK;
}

__global__ void k_status3(const NmScalars* s, int64_t* out) {
  out[0] = s->status;
  out[1] = s->total_iters;
  out[2] = s->max_seen;
}

// the run's status, total iterations and largest per-step count into dev3 (device, 3 int64),
// queued on the solver's stream behind its steps: no synchronisation
extern "C" int sc_newmark_status_to(sc_newmark* h, int64_t* dev3) {
  if (!h || !dev3) return SC_BAD_ARG;
  k_status3<<<1, 1, 0, h->user>>>(h->g.s, dev3);
  return check_launch("status copy");
}

extern "C" int sc_newmark_status(sc_newmark* h, int64_t* total_iters, int* max_iters) {
  if (!h) return SC_BAD_ARG;
  int rc = check(cudaStreamSynchronize(h->user), "sync status");
  if (rc) return rc;
  NmScalars s;
  if ((rc = check(cudaMemcpy(&s, h->g.s, sizeof(s), cudaMemcpyDeviceToHost), "read scalars"))) return rc;
  if (total_iters) *total_iters = s.total_iters;
  if (max_iters) *max_iters = s.max_seen;
  return s.status;
}

extern "C" int sc_newmark_time_spmv(sc_newmark* h, int reps, float* ms_per_launch, int64_t* bytes_per_launch) {
  if (!h || reps <= 0 || !ms_per_launch) return SC_BAD_ARG;
  cudaStream_t st = h->user;
  cudaEvent_t e0, e1;
  int rc = check(cudaEventCreate(&e0), "event");
  if (rc) return rc;
  if ((rc = check(cudaEventCreate(&e1), "event"))) {
    cudaEventDestroy(e0);
    return rc;
  }
  cudaGraphConditionalHandle none = 0;
  if ((rc = pair_prepare(h))) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
  }
  auto launch = [&]() {
    if (h->g.p2) k_spmv<false, true><<<h->row_blocks, kRowThreads, 0, st>>>(h->g, h->g.A, h->AP, none);
    else k_spmv<false, false><<<h->row_blocks, kRowThreads, 0, st>>>(h->g, h->g.A, nullptr, none);
  };
  launch();  // warm
  cudaEventRecord(e0, st);
  for (int i = 0; i < reps; ++i) launch();
  cudaEventRecord(e1, st);
  rc = check_launch("k_spmv timing");
  if (!rc) rc = check(cudaEventSynchronize(e1), "event sync");
  float ms = 0.f;
  if (!rc) cudaEventElapsedTime(&ms, e0, e1);
  *ms_per_launch = ms / reps;
  if (bytes_per_launch) {
    int64_t nnz = 0;
    cudaMemcpy(&nnz, h->g.rowptr + h->g.n, sizeof(int64_t), cudaMemcpyDeviceToHost);
    // values (8 bytes: FP64 or an FP32 pair) + column indices + row pointers + p (one pass) + w
    *bytes_per_launch = nnz * 12 + (h->g.n + 1) * 8 + h->g.n * 16;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

extern "C" int sc_newmark_destroy(sc_newmark* h) {
  if (!h) return SC_OK;
  if (h->step_exec) cudaGraphExecDestroy(h->step_exec);
  if (h->step_graph) cudaGraphDestroy(h->step_graph);
  if (h->init_exec) cudaGraphExecDestroy(h->init_exec);
  if (h->init_graph) cudaGraphDestroy(h->init_graph);
  if (h->cap) cudaStreamDestroy(h->cap);
  if (h->cap2) cudaStreamDestroy(h->cap2);
  cudaStreamSynchronize(h->user);
  if (h->AP) cudaFree(h->AP);
  if (h->MP) cudaFree(h->MP);
  if (h->p2) cudaFree(h->p2);
  delete h;
  return SC_OK;
}
