// Explicit central-difference scheme with a lumped mass on the node-block handle, and the
// discrete adjoint of that scheme (gradients of a receiver-velocity misfit with respect to
// per-element E and rho).  Neither has a counterpart in the reference, whose mass is always
// consistent and which has no differentiation.
//
// Scheme (M_L: row-sum lumped mass unless the caller sets one, C = Cabs + alpha M_L + beta K):
//   a_n       = M_L^-1 (f_n - K (u_n + beta v_n) - alpha M_L v_n - Cabs v_n)
//   v_{n+1}   = v_n + dt a_n ,   u_{n+1} = u_n + dt v_{n+1}
// from rest; v_{n+1} is the velocity reported at step n + 1.
//
// Arithmetic.  GB300 runs FP64 instructions (conversions included) at 1/64 of its FP32 rate,
// so the default step keeps u, v, w = u + beta v, the force, 1/M_L, alpha M_L and the
// dashpot values as FP32 (hi, lo) pairs (about 48 significant bits) and has no FP64
// instruction: K w uses the K pair planes with pair accumulation, the update uses pair
// add/multiply.  The caller's FP64 u, v are split into pairs when a run starts and joined
// back when it ends.  The FP64 step (sc_nb_set_options bit 1) computes in FP64 throughout.
//
// One thread per node row for large meshes, 2 or 4 for small ones (tpr); the last block to
// finish a step advances the step counter and swaps the force entries (every block has read
// them by then), so a step is one kernel and one graph launch.
#include <vector>

#include "sc_nb.cuh"

using namespace sc;
using namespace sc::nb;

namespace {

// ------------------------------------------------------------------ FP32-pair arithmetic
// (hi, lo) with |lo| <= ulp(hi) / 2; _rn intrinsics keep the compiler from contracting the
// error terms.
__device__ __forceinline__ float2 p_renorm(float h, float l) {
  const float s = __fadd_rn(h, l);
  return make_float2(s, __fsub_rn(l, __fsub_rn(s, h)));
}
__device__ __forceinline__ float2 p_add(float2 a, float2 b) {
  const float s = __fadd_rn(a.x, b.x);
  const float bp = __fsub_rn(s, a.x);
  const float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bp)), __fsub_rn(b.x, bp));
  return p_renorm(s, __fadd_rn(e, __fadd_rn(a.y, b.y)));
}
__device__ __forceinline__ float2 p_sub(float2 a, float2 b) { return p_add(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 p_mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = fmaf(a.x, b.x, -p);
  e = fmaf(a.x, b.y, fmaf(a.y, b.x, e));
  return p_renorm(p, e);
}
// conversions at the FP64 boundary (run start and end, receivers, misfit)
__device__ __forceinline__ float2 p_of(double x) {
  const float h = (float)x;
  return make_float2(h, (float)(x - (double)h));
}
__device__ __forceinline__ double p_to_d(float2 a) { return (double)a.x + (double)a.y; }
__device__ __forceinline__ float2 w_of(float2 u, float2 v, float2 beta) { return p_add(u, p_mul(beta, v)); }

// pair buffers of one step
struct PairStep {
  float2* u;  // updated in place (own row)
  const float2 *v_in, *w_in;
  float2 *v_out, *w_out;
  float2* f;  // the current step's force entries (swapped by the last block)
  const float2 *aml, *iml, *cab;  // alpha M_L, 1 / M_L, dashpot values
  float2 dt, beta;
};

// Adjoint recompute: the step n -> n+1 (n = step - 1, k = n - *t0 within the segment) stores
// the element gradient's inputs of state n at k (the receiver velocities the backward needs
// are the forward's records, bitwise the same as the recomputed ones).
struct SegStore {
  float2* wp;        // w = u + beta v of state n, [k n_s + i]
  float *v32, *a32;  // v of state n and a of the step n -> n+1 (hi parts)
  const int* t0;
};

template <int D>
__device__ __forceinline__ float pick(const float (&a)[D], int c) {
  return D == 2 ? (c == 0 ? a[0] : a[1]) : (c == 0 ? a[0] : (c == 1 ? a[1] : a[2]));
}

template <int D, int TPR, int kKeep>  // kKeep: the planes' load policy at compile time, or -1 (g.keep_l2)
__device__ __forceinline__ void explicit_pair_step(const Args& g, const PairStep& p, const int* __restrict__ rec_map,
                                                   const SegStore& st) {
  const int keep = kKeep >= 0 ? kKeep : g.keep_l2;
  const int step = g.s->t + 1;
  const int64_t kn = st.wp ? (int64_t)(step - 1 - *st.t0) * g.n_s : 0;
  const bool rec_now = g.n_rec > 0 && g.out_interval > 0 && (step % g.out_interval) == 0 &&
                       step / g.out_interval < g.n_out;
  const int64_t orow = rec_now ? step / g.out_interval : 0;
  const int sub = threadIdx.x % TPR;
  SELL_ROW_LOOP_T(TPR) {
    SELL_ROW_BEGIN(g.sf_ptr)
    // the row's update inputs into L2 while its products run (one thread per row, the large
    // meshes' shape; with more threads per row the extra registers cost more than it saves)
    if (TPR == 1 && row < g.n_nodes) {
      const int64_t i0 = row * D;
      const void* pf[5] = {p.v_in + i0, p.u + i0, p.f + i0, p.aml + i0, p.iml + i0};
#pragma unroll
      for (int k = 0; k < 5; ++k) asm volatile("prefetch.global.L2 [%0];" ::"l"(__cvta_generic_to_global(pf[k])));
    }
    float hi[D], lo[D];
#pragma unroll
    for (int c = 0; c < D; ++c) hi[c] = lo[c] = 0.f;
    for (int64_t q = sub; q < nq; q += TPR) {
      const int64_t pos = p0 + 128 * q;
      int cl[4];
      cols4(g.sf_col, pos, cl, keep);
      float2 wa[4][D];
#pragma unroll
      for (int e = 0; e < 4; ++e)
#pragma unroll
        for (int d = 0; d < D; ++d) wa[e][d] = p.w_in[(int64_t)cl[e] * D + d];
#pragma unroll
      for (int c = 0; c < D; ++c)
#pragma unroll
        for (int d = 0; d < D; ++d) {
          float2 k4[4];
          ld4(g.KPS + (int64_t)(c * D + d) * g.sf_n + pos, k4, keep);
#pragma unroll
          for (int e = 0; e < 4; ++e) pair_fma(k4[e].x, k4[e].y, wa[e][d], hi[c], lo[c]);
        }
    }
#pragma unroll
    for (int c = 0; c < D; ++c) group_pair_sum<TPR>(hi[c], lo[c]);
    if (row >= g.n_nodes) continue;
    // one lane per component (all lanes in one pass when TPR >= D)
    for (int c = (TPR >= D ? sub : 0); c < D; c += (TPR >= D ? D : 1)) {
      if (TPR > 1 && TPR < D && c % TPR != sub) continue;
      const int64_t i = row * D + c;
      if (g.fixed[i]) {
        p.v_out[i] = p.w_out[i] = make_float2(0.f, 0.f);
        if (st.wp) {
          st.wp[kn + i] = make_float2(0.f, 0.f);
          st.v32[kn + i] = st.a32[kn + i] = 0.f;
        }
        continue;
      }
      float2 cab = make_float2(0.f, 0.f);
      for (int64_t k = g.cab_ptr[i]; k < g.cab_ptr[i + 1]; ++k) cab = p_add(cab, p_mul(p.cab[k], p.v_in[g.cab_col[k]]));
      const float2 vi = p.v_in[i];
      const float2 kw = p_renorm(pick<D>(hi, c), pick<D>(lo, c));
      const float2 num = p_sub(p_sub(p_sub(p.f[i], kw), p_mul(p.aml[i], vi)), cab);
      const float2 acc = p_mul(num, p.iml[i]);
      const float2 vn = p_add(vi, p_mul(p.dt, acc));
      const float2 un = p_add(p.u[i], p_mul(p.dt, vn));
      p.v_out[i] = vn;
      p.u[i] = un;
      p.w_out[i] = w_of(un, vn, p.beta);
      if (st.wp) {
        st.wp[kn + i] = p.w_in[i];
        st.v32[kn + i] = vi.x;
        st.a32[kn + i] = acc.x;
      }
      if (rec_now) {
        const int rj = rec_map[i];
        if (rj >= 0) {
          if (g.out_u) g.out_u[orow * g.n_rec + rj] = p_to_d(un);
          if (g.out_v) g.out_v[orow * g.n_rec + rj] = p_to_d(vn);
        }
      }
    }
  }
  if (last_block(&g.s->ticket)) {
    const int t = step - 1;
    if (g.f_ptr) {
      if (t >= 0 && t < g.n_t)
        for (int64_t k = g.f_ptr[t] + threadIdx.x; k < g.f_ptr[t + 1]; k += blockDim.x)
          p.f[g.f_slot[k]] = make_float2(0.f, 0.f);
      __syncthreads();
      if (t + 1 < g.n_t)
        for (int64_t k = g.f_ptr[t + 1] + threadIdx.x; k < g.f_ptr[t + 2]; k += blockDim.x)
          p.f[g.f_slot[k]] = p_of(g.f_val[k]);
    }
    if (threadIdx.x == 0) {
      g.s->ticket = 0;
      g.s->t = step;
    }
  }
}

// The explicit step at the compiler's default register budget (64 per thread at 256 threads) and
// at a wide one (minimum one block per SM: up to 174 registers, no spills), each with the
// planes' load policy read at run time or fixed at compile time; the tuner times them all with
// each threads-per-row count, as the fastest depends on the mesh size (one thread per row, wide
// budget, policy at compile time: 0.033 against 0.043 ms for the default form at 209 k DOF, but
// slower at 1.79 M DOF; at 107 k DOF with two threads per row the compile-time policy made the
// step 26 us against 21).
template <int D, int TPR, int kKeep>
__global__ void __launch_bounds__(kThreads) k_explicit_pair(Args g, PairStep p, const int* __restrict__ rec_map,
                                                            SegStore st) {
  explicit_pair_step<D, TPR, kKeep>(g, p, rec_map, st);
}
template <int D, int TPR, int kKeep>
__global__ void __launch_bounds__(kThreads, 1) k_explicit_pair_wide(Args g, PairStep p,
                                                                    const int* __restrict__ rec_map, SegStore st) {
  explicit_pair_step<D, TPR, kKeep>(g, p, rec_map, st);
}

// FP64 step: the same scheme with FP64 products and update (reference precision)
template <int D, int TPR>
__global__ void __launch_bounds__(kThreads) k_explicit_fp64(Args g, const double* __restrict__ ML,
                                                            const double* __restrict__ IML,
                                                            const double* __restrict__ v_in, double* __restrict__ v_out,
                                                            const double* __restrict__ w_in, double* __restrict__ w_out,
                                                            const int* __restrict__ rec_map) {
  const int step = g.s->t + 1;
  const bool rec_now = g.n_rec > 0 && g.out_interval > 0 && (step % g.out_interval) == 0 &&
                       step / g.out_interval < g.n_out;
  const int64_t orow = rec_now ? step / g.out_interval : 0;
  const int sub = threadIdx.x % TPR;
  SELL_ROW_LOOP_T(TPR) {
    SELL_ROW_BEGIN(g.sf_ptr)
    double s[D];
#pragma unroll
    for (int c = 0; c < D; ++c) s[c] = 0.0;
    for (int64_t q = sub; q < nq; q += TPR) {
      const int64_t pos = p0 + 128 * q;
      int cl[4];
      cols4(g.sf_col, pos, cl, g.keep_l2);
      double wa[4][D];
#pragma unroll
      for (int e = 0; e < 4; ++e)
#pragma unroll
        for (int d = 0; d < D; ++d) wa[e][d] = w_in[(int64_t)cl[e] * D + d];
#pragma unroll
      for (int c = 0; c < D; ++c)
#pragma unroll
        for (int d = 0; d < D; ++d) {
          double kv[4];
          ld4(g.KS + (int64_t)(c * D + d) * g.sf_n + pos, kv, g.keep_l2);
#pragma unroll
          for (int e = 0; e < 4; ++e) s[c] = fma(kv[e], wa[e][d], s[c]);
        }
    }
#pragma unroll
    for (int c = 0; c < D; ++c) s[c] = group_sum<TPR>(s[c]);
    if (row >= g.n_nodes) continue;
#pragma unroll
    for (int c = 0; c < D; ++c) {
      if (TPR > 1 && c % TPR != sub) continue;
      const int64_t i = row * D + c;
      if (g.fixed[i]) {
        v_out[i] = w_out[i] = 0.0;
        continue;
      }
      double cab = 0.0;
      for (int64_t k = g.cab_ptr[i]; k < g.cab_ptr[i + 1]; ++k) cab = fma(g.cab_val[k], v_in[g.cab_col[k]], cab);
      const double vi = v_in[i], ml = ML[i];
      const double acc = (g.f[i] - s[c] - g.alpha_r * ml * vi - cab) * IML[i];
      const double vn = fma(g.dt, acc, vi);
      const double un = fma(g.dt, vn, g.u[i]);
      v_out[i] = vn;
      g.u[i] = un;
      w_out[i] = fma(g.beta_r, vn, un);
      if (rec_now) {
        const int rj = rec_map[i];
        if (rj >= 0) {
          if (g.out_u) g.out_u[orow * g.n_rec + rj] = un;
          if (g.out_v) g.out_v[orow * g.n_rec + rj] = vn;
        }
      }
    }
  }
  if (last_block(&g.s->ticket)) {
    const int t = step - 1;
    if (g.f_ptr) {
      if (t >= 0 && t < g.n_t)
        for (int64_t k = g.f_ptr[t] + threadIdx.x; k < g.f_ptr[t + 1]; k += blockDim.x) g.f[g.f_slot[k]] = 0.0;
      __syncthreads();
      if (t + 1 < g.n_t)
        for (int64_t k = g.f_ptr[t + 1] + threadIdx.x; k < g.f_ptr[t + 2]; k += blockDim.x) g.f[g.f_slot[k]] += g.f_val[k];
    }
    if (threadIdx.x == 0) {
      g.s->ticket = 0;
      g.s->t = step;
    }
  }
}

// ------------------------------------------------------------------ set-up and boundary kernels
// row sums of the consistent mass over free columns (the lumped mass); fixed slots get 1
__global__ void k_lumped(Args g, double* ML) {
  for (int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; a < g.n_nodes; a += (int64_t)gridDim.x * blockDim.x) {
    for (int c = 0; c < g.D; ++c) {
      double m = 0.0;
      for (int64_t k = g.adj_ptr[a]; k < g.adj_ptr[a + 1]; ++k)
        if (!g.fixed[(int64_t)g.adj[k] * g.D + c]) m += g.MS[k];
      ML[a * g.D + c] = g.fixed[a * g.D + c] ? 1.0 : m;
    }
  }
}

__global__ void k_mass_consts(Args g, const double* __restrict__ ML, double* __restrict__ IML, float2* aml2,
                              float2* iml2) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n_s; i += (int64_t)gridDim.x * blockDim.x) {
    const double ml = g.fixed[i] ? 1.0 : ML[i];
    IML[i] = 1.0 / ml;
    if (aml2) {
      aml2[i] = p_of(g.alpha_r * ml);
      iml2[i] = p_of(1.0 / ml);
    }
  }
}

__global__ void k_copy_masked(int64_t n, const double* __restrict__ x, const int* __restrict__ fixed, double* y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = fixed[i] ? 1.0 : x[i];
}

__global__ void k_to_pairs(int64_t n, const double* __restrict__ x, float2* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = p_of(x[i]);
}

__global__ void k_from_pairs(int64_t n, const float2* __restrict__ y, double* __restrict__ x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = p_to_d(y[i]);
}

__global__ void k_w_pairs(int64_t n, const float2* __restrict__ u, const float2* __restrict__ v, float2 beta,
                          float2* __restrict__ w) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    w[i] = w_of(u[i], v[i], beta);
}

__global__ void k_w_fp64(Args g, double* w) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n_s; i += (int64_t)gridDim.x * blockDim.x)
    w[i] = fma(g.beta_r, g.v[i], g.u[i]);
}

// force entries of step t (f cleared beforehand)
__global__ void k_force_at(Args g, int t, float2* f2) {
  if (!g.f_ptr || t < 0 || t >= g.n_t) return;
  for (int64_t k = g.f_ptr[t] + threadIdx.x; k < g.f_ptr[t + 1]; k += blockDim.x) {
    if (f2) f2[g.f_slot[k]] = p_of(g.f_val[k]);
    else g.f[g.f_slot[k]] += g.f_val[k];
  }
}

__global__ void k_rec_map(Args g, int* map) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n_s; i += (int64_t)gridDim.x * blockDim.x)
    map[i] = -1;
}
__global__ void k_rec_map_fill(Args g, int* map) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < g.n_rec; j += (int64_t)gridDim.x * blockDim.x)
    map[g.rec_slot[j]] = (int)j;
}

float2 host_pair(double x) {
  const float h = (float)x;
  return make_float2(h, (float)(x - (double)h));
}

PairStep pair_step(const sc_nb_newmark* h, int k) {
  PairStep p;
  p.u = h->u2;
  p.v_in = h->v2[k];
  p.w_in = h->w2[k];
  p.v_out = h->v2[k ^ 1];
  p.w_out = h->w2[k ^ 1];
  p.f = h->f2;
  p.aml = h->aml2;
  p.iml = h->iml2;
  p.cab = h->cab2;
  p.dt = host_pair(h->g.dt);
  p.beta = host_pair(h->g.beta_r);
  return p;
}

template <int D, int TPR, int kKeep>
void launch_pair_k(const sc_nb_newmark* h, cudaStream_t st, int k, SegStore store) {
  if (h->ex_wide)
    k_explicit_pair_wide<D, TPR, kKeep><<<h->tpr_blocks, kThreads, 0, st>>>(h->g, pair_step(h, k), h->rec_map,
                                                                           store);
  else
    k_explicit_pair<D, TPR, kKeep><<<h->tpr_blocks, kThreads, 0, st>>>(h->g, pair_step(h, k), h->rec_map, store);
}
template <int D, int TPR>
void launch_pair_t(const sc_nb_newmark* h, cudaStream_t st, int k, SegStore store) {
  if (!h->ex_keep_ct) launch_pair_k<D, TPR, -1>(h, st, k, store);
  else if (h->g.keep_l2) launch_pair_k<D, TPR, 1>(h, st, k, store);
  else launch_pair_k<D, TPR, 0>(h, st, k, store);
}
template <int D>
void launch_pair(const sc_nb_newmark* h, cudaStream_t st, int k, SegStore store) {
  switch (h->tpr) {
    case 4: launch_pair_t<D, 4>(h, st, k, store); break;
    case 2: launch_pair_t<D, 2>(h, st, k, store); break;
    default: launch_pair_t<D, 1>(h, st, k, store); break;
  }
}
void launch_step(const sc_nb_newmark* h, cudaStream_t st, int k, SegStore store) {
  const Args& g = h->g;
  if (h->explicit_pair) {
    if (g.D == 3) launch_pair<3>(h, st, k, store);
    else launch_pair<2>(h, st, k, store);
    return;
  }
  const double* vin = k == 0 ? g.v : h->v1;
  double* vout = k == 0 ? h->v1 : g.v;
  const double* win = k == 0 ? h->w0 : h->w1;
  double* wout = k == 0 ? h->w1 : h->w0;
  const unsigned nb = h->tpr_blocks;
#define SC_FP64_STEP(DD, TT) \
  k_explicit_fp64<DD, TT><<<nb, kThreads, 0, st>>>(g, h->ML, h->IML, vin, vout, win, wout, h->rec_map)
  if (g.D == 3) {
    if (h->tpr == 4) SC_FP64_STEP(3, 4);
    else if (h->tpr == 2) SC_FP64_STEP(3, 2);
    else SC_FP64_STEP(3, 1);
  } else {
    if (h->tpr == 4) SC_FP64_STEP(2, 4);
    else if (h->tpr == 2) SC_FP64_STEP(2, 2);
    else SC_FP64_STEP(2, 1);
  }
#undef SC_FP64_STEP
}

int build_explicit_graphs(sc_nb_newmark* h) {
  for (int k = 0; k < 2; ++k) {
    int rc = check(cudaStreamBeginCapture(h->cap, cudaStreamCaptureModeThreadLocal), "capture explicit");
    if (rc) return rc;
    launch_step(h, h->cap, k, SegStore{});
    cudaGraph_t graph;
    if ((rc = check(cudaStreamEndCapture(h->cap, &graph), "end explicit"))) return rc;
    if ((rc = check(cudaGraphInstantiate(&h->ex_exec[k], graph, 0), "instantiate explicit"))) {
      cudaGraphDestroy(graph);
      return rc;
    }
    h->ex_graph[k] = graph;
  }
  return SC_OK;
}

// allocations, lumped mass and its derived constants, K pair planes, receiver map, graphs
int explicit_prepare(sc_nb_newmark* h) {
  Args& g = h->g;
  cudaStream_t st = h->user;
  const int64_t ns = g.n_s;
  int rc;
  auto M = [&](void** p, size_t b) { return check(cudaMallocAsync(p, b, st), "explicit malloc"); };
  if (!h->ML) {
    if ((rc = M((void**)&h->ML, 8 * ns)) || (rc = M((void**)&h->IML, 8 * ns)) || (rc = M((void**)&h->rec_map, 4 * ns)))
      return rc;
    k_lumped<<<grid_for(g.n_nodes, 256), 256, 0, st>>>(g, h->ML);
  }
  if (h->explicit_pair && !h->u2) {
    if ((rc = M((void**)&h->u2, 8 * ns)) || (rc = M((void**)&h->v2[0], 8 * ns)) || (rc = M((void**)&h->v2[1], 8 * ns)) ||
        (rc = M((void**)&h->w2[0], 8 * ns)) || (rc = M((void**)&h->w2[1], 8 * ns)) || (rc = M((void**)&h->f2, 8 * ns)) ||
        (rc = M((void**)&h->aml2, 8 * ns)) || (rc = M((void**)&h->iml2, 8 * ns)))
      return rc;
    int64_t ncab = 0;
    if ((rc = check(cudaMemcpyAsync(&ncab, g.cab_ptr + ns, 8, cudaMemcpyDeviceToHost, st), "cab size"))) return rc;
    if ((rc = check(cudaStreamSynchronize(st), "sync"))) return rc;
    if ((rc = M((void**)&h->cab2, 8 * (ncab > 0 ? ncab : 1)))) return rc;
    if (ncab > 0) k_to_pairs<<<grid_for(ncab, 256), 256, 0, st>>>(ncab, g.cab_val, h->cab2);
    const int64_t n2 = (int64_t)g.D * g.D * g.sf_n;
    if (!h->KPS) {
      if ((rc = M((void**)&h->KPS, 8 * n2))) return rc;
      k_split_pairs<<<grid_for(n2, 256, 152 * 32), 256, 0, st>>>(n2, g.KS, h->KPS);
    }
    g.KPS = h->KPS;
    cudaMemsetAsync(h->f2, 0, 8 * ns, st);
    drop_explicit_graphs(h);
  }
  if (!h->explicit_pair && !h->v1) {
    if ((rc = M((void**)&h->v1, 8 * ns)) || (rc = M((void**)&h->w0, 8 * ns)) || (rc = M((void**)&h->w1, 8 * ns)))
      return rc;
  }
  k_mass_consts<<<grid_for(ns, 256), 256, 0, st>>>(g, h->ML, h->IML, h->aml2, h->iml2);
  if (!h->ex_exec[0]) {
    k_rec_map<<<grid_for(ns, 256), 256, 0, st>>>(g, h->rec_map);
    if (g.n_rec > 0) k_rec_map_fill<<<grid_for(g.n_rec, 256), 256, 0, st>>>(g, h->rec_map);
    if ((rc = build_explicit_graphs(h))) return rc;
  }
  return check_launch("explicit prepare");
}

// force entries of step t in f (FP64 mode) or f2 (pair mode), on stream st (default: the
// handle's stream)
void force_reset(sc_nb_newmark* h, int t, cudaStream_t st = nullptr) {
  Args& g = h->g;
  if (!st) st = h->user;
  if (h->explicit_pair) {
    cudaMemsetAsync(h->f2, 0, 8 * g.n_s, st);
    k_force_at<<<1, 256, 0, st>>>(g, t, h->f2);
  } else {
    cudaMemsetAsync(g.f, 0, 8 * g.n_s, st);
    k_force_at<<<1, 256, 0, st>>>(g, t, nullptr);
  }
}

// steps t0 .. t1-1 from the state in (u2, v2[0]) or (u, v); w is rebuilt from the state first
int explicit_steps(sc_nb_newmark* h, int t0, int t1) {
  Args& g = h->g;
  cudaStream_t st = h->user;
  const int64_t ns = g.n_s;
  if (h->explicit_pair) k_w_pairs<<<h->vec_blocks, 256, 0, st>>>(ns, h->u2, h->v2[0], host_pair(g.beta_r), h->w2[0]);
  else k_w_fp64<<<h->vec_blocks, 256, 0, st>>>(g, h->w0);
  k_set_t<<<1, 1, 0, st>>>(g.s, t0);
  int rc = check_launch("explicit steps");
  if (rc) return rc;
  int k = 0;
  for (int t = t0; t < t1; ++t, k ^= 1)
    if ((rc = check(cudaGraphLaunch(h->ex_exec[k], st), "explicit launch"))) return rc;
  if (k == 1) {  // the state's v is in the second buffer: bring it back
    if (h->explicit_pair) rc = check(cudaMemcpyAsync(h->v2[0], h->v2[1], 8 * ns, cudaMemcpyDeviceToDevice, st), "copy v");
    else rc = check(cudaMemcpyAsync(g.v, h->v1, 8 * ns, cudaMemcpyDeviceToDevice, st), "copy v");
  }
  return rc;
}

}  // namespace

void drop_explicit_graphs(sc_nb_newmark* h) {
  for (int k = 0; k < 2; ++k) {
    if (h->ex_exec[k]) cudaGraphExecDestroy(h->ex_exec[k]), h->ex_exec[k] = nullptr;
    if (h->ex_graph[k]) cudaGraphDestroy(h->ex_graph[k]), h->ex_graph[k] = nullptr;
  }
}

void free_explicit(sc_nb_newmark* h) {
  void* bufs[] = {h->ML, h->IML, h->v1, h->w0, h->w1, h->KPS, h->u2, h->v2[0], h->v2[1], h->w2[0], h->w2[1],
                  h->f2, h->aml2, h->iml2, h->cab2, h->rec_map};
  for (void* q : bufs)
    if (q) cudaFree(q);
}

// Explicit steps t_begin .. t_end-1 on the handle (u, v are the handle's FP64 state vectors; a
// is not used).  At t_begin == 0 the force entries of step 0 are written; the run always ends
// with the state in the caller's u and v.
extern "C" int sc_nb_explicit_run(sc_nb_newmark* h, int t_begin, int t_end) {
  if (!h || t_begin < 0 || t_end < t_begin) return SC_BAD_ARG;
  Args& g = h->g;
  cudaStream_t st = h->user;
  int rc;
  if ((rc = explicit_prepare(h))) return rc;
  const int64_t ns = g.n_s;
  if (h->explicit_pair) {
    k_to_pairs<<<h->vec_blocks, 256, 0, st>>>(ns, g.u, h->u2);
    k_to_pairs<<<h->vec_blocks, 256, 0, st>>>(ns, g.v, h->v2[0]);
  }
  if (t_begin == 0) force_reset(h, 0);
  if ((rc = explicit_steps(h, t_begin, t_end))) return rc;
  if (h->explicit_pair) {
    k_from_pairs<<<h->vec_blocks, 256, 0, st>>>(ns, h->u2, g.u);
    k_from_pairs<<<h->vec_blocks, 256, 0, st>>>(ns, h->v2[0], g.v);
  }
  return check_launch("explicit run");
}

// A lumped mass of the caller's choosing (slot space, FP64, device; fixed slots ignored), e.g.
// a diagonal-scaled mass where row sums of the consistent mass are not positive.
extern "C" int sc_nb_set_lumped_mass(sc_nb_newmark* h, const double* ml) {
  if (!h || !ml) return SC_BAD_ARG;
  Args& g = h->g;
  cudaStream_t st = h->user;
  if (!h->ML) {
    int rc = explicit_prepare(h);
    if (rc) return rc;
  }
  k_copy_masked<<<grid_for(g.n_s, 256), 256, 0, st>>>(g.n_s, ml, g.fixed, h->ML);
  h->ml_user = 1;
  k_mass_consts<<<grid_for(g.n_s, 256), 256, 0, st>>>(g, h->ML, h->IML, h->aml2, h->iml2);
  return check_launch("lumped mass");
}

// Threads per node row of the explicit step (1, 2, 4) picked by timing `reps` launches of each
// candidate (after one untimed launch) on the handle's pair buffers; the force entries and the
// receiver setting are saved and restored, and the state is rebuilt from the caller's u, v by
// the next sc_nb_explicit_run, so the timing leaves no trace.  Pair arithmetic only.
extern "C" int sc_nb_tune_explicit(sc_nb_newmark* h, int reps, int* tpr_chosen, float* ms_per_step) {
  if (!h || reps <= 0 || !h->explicit_pair) return SC_BAD_ARG;
  int rc = explicit_prepare(h);
  if (rc) return rc;
  Args& g = h->g;
  cudaStream_t st = h->user;
  const int64_t ns = g.n_s;
  float2* f_save = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const int n_rec = g.n_rec;
  const int tpr0 = h->tpr;
  const unsigned blocks0 = h->tpr_blocks;
  float best = -1.f;
  int best_tpr = tpr0;
  const int wide0 = h->ex_wide, keep_ct0 = h->ex_keep_ct;
  int best_wide = wide0, best_keep_ct = keep_ct0;
  do {
    if ((rc = check(cudaMallocAsync((void**)&f_save, 8 * ns, st), "tune malloc"))) break;
    cudaMemcpyAsync(f_save, h->f2, 8 * ns, cudaMemcpyDeviceToDevice, st);
    if ((rc = check(cudaEventCreate(&e0), "event")) || (rc = check(cudaEventCreate(&e1), "event"))) break;
    g.n_rec = 0;  // no receiver records while timing
    // every candidate warmed up first, then timed in three rounds taken in turn (a candidate's
    // best round counts): a single pass ranked them by the order the clocks ramped in
    // candidate ci: threads per row {1, 2, 4}[ci % 3], wide register budget (ci / 3) & 1, load
    // policy at compile time ci / 6
    constexpr int kCands = 12;
    const int tprs[3] = {1, 2, 4};
    float cms[kCands];
    for (int ci = 0; ci < kCands; ++ci) cms[ci] = -1.f;
    for (int round = -1; round < 3 && !rc; ++round)
      for (int ci = 0; ci < kCands && !rc; ++ci) {
        h->tpr = tprs[ci % 3];
        h->ex_wide = (ci / 3) & 1;
        h->ex_keep_ct = ci / 6;
        const int64_t want = (((int64_t)g.n_nodes + 31) / 32 * 32 * h->tpr + kThreads - 1) / kThreads;
        h->tpr_blocks = (unsigned)(want < 152 * 16 ? (want < 1 ? 1 : want) : 152 * 16);
        if (round < 0) {
          for (int i = 0; i < 3; ++i) launch_step(h, st, i & 1, SegStore{});
          continue;
        }
        cudaEventRecord(e0, st);
        for (int i = 0; i < reps; ++i) launch_step(h, st, i & 1, SegStore{});
        cudaEventRecord(e1, st);
        if ((rc = check_launch("explicit tune"))) break;
        if ((rc = check(cudaEventSynchronize(e1), "tune sync"))) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= reps;
        if (cms[ci] < 0.f || ms < cms[ci]) cms[ci] = ms;
      }
    for (int ci = 0; ci < kCands && !rc; ++ci)
      if (best < 0.f || cms[ci] < best) {
        best = cms[ci];
        best_tpr = tprs[ci % 3];
        best_wide = (ci / 3) & 1;
        best_keep_ct = ci / 6;
      }
    cudaMemcpyAsync(h->f2, f_save, 8 * ns, cudaMemcpyDeviceToDevice, st);
  } while (0);
  g.n_rec = n_rec;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamSynchronize(st);
  if (f_save) cudaFree(f_save);
  if (rc || best < 0.f) {
    h->tpr = tpr0;
    h->ex_wide = wide0;
    h->ex_keep_ct = keep_ct0;
    h->tpr_blocks = blocks0;
    return rc ? rc : SC_BAD_ARG;
  }
  h->tpr = best_tpr;
  h->ex_wide = best_wide;
  h->ex_keep_ct = best_keep_ct;
  const int64_t want = (((int64_t)g.n_nodes + 31) / 32 * 32 * h->tpr + kThreads - 1) / kThreads;
  h->tpr_blocks = (unsigned)(want < 152 * 16 ? (want < 1 ? 1 : want) : 152 * 16);
  drop_explicit_graphs(h);
  if (tpr_chosen) *tpr_chosen = best_tpr;
  if (ms_per_step) *ms_per_step = best;
  return explicit_prepare(h);
}

extern "C" int sc_nb_time_explicit(sc_nb_newmark* h, int reps, float* ms_per_step) {
  if (!h || reps <= 0 || !ms_per_step || !h->ex_exec[0]) return SC_BAD_ARG;
  cudaStream_t st = h->user;
  cudaEvent_t e0, e1;
  int rc = check(cudaEventCreate(&e0), "event");
  if (rc) return rc;
  if ((rc = check(cudaEventCreate(&e1), "event"))) {
    cudaEventDestroy(e0);
    return rc;
  }
  cudaEventRecord(e0, st);
  for (int i = 0; i < reps; ++i) launch_step(h, st, i & 1, SegStore{});
  cudaEventRecord(e1, st);
  rc = check_launch("explicit timing");
  if (!rc) rc = check(cudaEventSynchronize(e1), "sync");
  float ms = 0.f;
  if (!rc) cudaEventElapsedTime(&ms, e0, e1);
  *ms_per_step = ms / reps;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

// ================================================================== adjoint
struct sc_adj_desc {
  int n_steps, checkpoint;
  int n_rec;
  const int* rec_slot;
  const double* target;
  int n_elem, n_en;
  const int *elem, *ke_type;
  const float* ke1;
  const double *young, *rho;
  const float* ml1;
  const int64_t* l_eptr;
  const int *l_row, *l_col;
  const float *l_c, *l_s;
};

namespace {

struct AdjState {
  // segment buffer (one of two): the element gradient's inputs for each step of the segment
  float2* wp;        // w = u + beta v of state n, [C n_s]
  float *v32, *a32;  // v of state n and a of the step n -> n+1 (hi parts), [C n_s]
  float* ys;         // y of backward step n (hi + lo rounded to FP32), [C n_s]
  int* seg_t0;       // first step of the segment the buffer holds
  // shared by both buffers
  float2 *mu_u, *mu_v;
  float2* y[2];        // (mu_v + dt mu_u) / M_L of the step being reversed ([cur]) and of the next
  double* out_v;       // the forward's receiver velocities, [(N + 1) n_rec]
  double *gE, *gR;     // gradient outputs [n_elem]
  float *iE, *iR;      // 1 / E_e, 1 / rho_e
  int* n_dev;          // step being reversed
  unsigned* ticket_r;  // blocks of the row kernel finished in its current launch
  int* rec_map;
  double* J;
};

// Backward step n (state n -> n+1 reversed), node rows, all in FP32 pairs: with y = y[cur],
//   mu_u <- mu_u - dt K y,  mu_v <- g - dt (beta K y + Cab y + alpha M_L y) + P^T (P v_n - d_n),
//   y[cur ^ 1] = (mu_v + dt mu_u) / M_L   (the y of step n - 1),  g = mu_v + dt mu_u;
// y of step n also goes to the segment buffer (one FP32 value) for the element gradients.
// The last block to finish decrements the step counter.
template <int D, int TPR>
__global__ void __launch_bounds__(kThreads) k_adj_rows(Args g, PairStep p, sc_adj_desc d, AdjState a, int cur) {
  const int n = *a.n_dev;
  float* ys = a.ys + (int64_t)(n - *a.seg_t0) * g.n_s;
  const float2* y = cur ? a.y[1] : a.y[0];  // (a select: no local copy of the parameter)
  float2* yn = cur ? a.y[0] : a.y[1];
  const int sub = threadIdx.x % TPR;
  SELL_ROW_LOOP_T(TPR) {
    SELL_ROW_BEGIN(g.sf_ptr)
    float hi[D], lo[D];
#pragma unroll
    for (int c = 0; c < D; ++c) hi[c] = lo[c] = 0.f;
    for (int64_t q = sub; q < nq; q += TPR) {
      const int64_t pos = p0 + 128 * q;
      int cl[4];
      cols4(g.sf_col, pos, cl, g.keep_l2);
      float2 ya[4][D];
#pragma unroll
      for (int e = 0; e < 4; ++e)
#pragma unroll
        for (int dd = 0; dd < D; ++dd) ya[e][dd] = y[(int64_t)cl[e] * D + dd];
#pragma unroll
      for (int c = 0; c < D; ++c)
#pragma unroll
        for (int dd = 0; dd < D; ++dd) {
          float2 k4[4];
          ld4(g.KPS + (int64_t)(c * D + dd) * g.sf_n + pos, k4, g.keep_l2);
#pragma unroll
          for (int e = 0; e < 4; ++e) pair_fma(k4[e].x, k4[e].y, ya[e][dd], hi[c], lo[c]);
        }
    }
#pragma unroll
    for (int c = 0; c < D; ++c) group_pair_sum<TPR>(hi[c], lo[c]);
    if (row >= g.n_nodes) continue;
    for (int c = (TPR >= D ? sub : 0); c < D; c += (TPR >= D ? D : 1)) {
      if (TPR > 1 && TPR < D && c % TPR != sub) continue;
      const int64_t i = row * D + c;
      const float2 yi = y[i];
      ys[i] = __fadd_rn(yi.x, yi.y);
      if (g.fixed[i]) {
        a.mu_u[i] = a.mu_v[i] = yn[i] = make_float2(0.f, 0.f);
        continue;
      }
      const float2 ky = p_renorm(pick<D>(hi, c), pick<D>(lo, c));
      float2 cy = make_float2(0.f, 0.f);
      for (int64_t q = g.cab_ptr[i]; q < g.cab_ptr[i + 1]; ++q) cy = p_add(cy, p_mul(p.cab[q], y[g.cab_col[q]]));
      const float2 mu_u = a.mu_u[i], mu_v = a.mu_v[i];
      const float2 gg = p_add(mu_v, p_mul(p.dt, mu_u));
      const float2 mu = p_sub(mu_u, p_mul(p.dt, ky));
      float2 mv = p_sub(gg, p_mul(p.dt, p_add(p_add(p_mul(p.beta, ky), cy), p_mul(p.aml[i], yi))));
      const int rj = a.rec_map[i];
      if (rj >= 0 && n >= 1)
        mv = p_add(mv, p_of(a.out_v[(int64_t)n * d.n_rec + rj] - d.target[(int64_t)n * d.n_rec + rj]));
      a.mu_u[i] = mu;
      a.mu_v[i] = mv;
      yn[i] = p_mul(p_add(mv, p_mul(p.dt, mu)), p.iml[i]);
    }
  }
  if (last_block(a.ticket_r)) {
    if (threadIdx.x == 0) {
      *a.ticket_r = 0;
      *a.n_dev = n - 1;
    }
  }
}

// A recompute step of one segment and a backward step of the next one, fused: one pass over
// the K pair planes serves K w (the explicit step n -> n+1 of the recompute, storing the
// element gradient's inputs, recording no receivers) and K y (the backward rows of step nb).
// Each half's arithmetic is that of k_explicit_pair / k_adj_rows, in the same order, so the
// results are bitwise theirs.  The last block swaps the recompute's force entries and advances
// both step counters.
template <int D, int TPR>
__global__ void __launch_bounds__(kThreads) k_adj_fused(Args g, PairStep p, SegStore st, sc_adj_desc d, AdjState a,
                                                        int cur) {
  const int step = g.s->t + 1;
  const int64_t kn = (int64_t)(step - 1 - *st.t0) * g.n_s;
  const int nb = *a.n_dev;
  float* ys = a.ys + (int64_t)(nb - *a.seg_t0) * g.n_s;
  const float2* y = cur ? a.y[1] : a.y[0];
  float2* yn = cur ? a.y[0] : a.y[1];
  const int sub = threadIdx.x % TPR;
  SELL_ROW_LOOP_T(TPR) {
    SELL_ROW_BEGIN(g.sf_ptr)
    float hf[D], lf[D], hb[D], lb[D];
#pragma unroll
    for (int c = 0; c < D; ++c) hf[c] = lf[c] = hb[c] = lb[c] = 0.f;
    for (int64_t q = sub; q < nq; q += TPR) {
      const int64_t pos = p0 + 128 * q;
      int cl[4];
      cols4(g.sf_col, pos, cl, g.keep_l2);
      float2 wa[4][D], ya[4][D];
#pragma unroll
      for (int e = 0; e < 4; ++e)
#pragma unroll
        for (int dd = 0; dd < D; ++dd) {
          wa[e][dd] = p.w_in[(int64_t)cl[e] * D + dd];
          ya[e][dd] = y[(int64_t)cl[e] * D + dd];
        }
#pragma unroll
      for (int c = 0; c < D; ++c)
#pragma unroll
        for (int dd = 0; dd < D; ++dd) {
          float2 k4[4];
          ld4(g.KPS + (int64_t)(c * D + dd) * g.sf_n + pos, k4, g.keep_l2);
#pragma unroll
          for (int e = 0; e < 4; ++e) pair_fma(k4[e].x, k4[e].y, wa[e][dd], hf[c], lf[c]);
#pragma unroll
          for (int e = 0; e < 4; ++e) pair_fma(k4[e].x, k4[e].y, ya[e][dd], hb[c], lb[c]);
        }
    }
#pragma unroll
    for (int c = 0; c < D; ++c) {
      group_pair_sum<TPR>(hf[c], lf[c]);
      group_pair_sum<TPR>(hb[c], lb[c]);
    }
    if (row >= g.n_nodes) continue;
    for (int c = (TPR >= D ? sub : 0); c < D; c += (TPR >= D ? D : 1)) {
      if (TPR > 1 && TPR < D && c % TPR != sub) continue;
      const int64_t i = row * D + c;
      // recompute: the explicit step, storing the element gradient's inputs of state n
      if (g.fixed[i]) {
        p.v_out[i] = p.w_out[i] = make_float2(0.f, 0.f);
        st.wp[kn + i] = make_float2(0.f, 0.f);
        st.v32[kn + i] = st.a32[kn + i] = 0.f;
      } else {
        float2 cab = make_float2(0.f, 0.f);
        for (int64_t k = g.cab_ptr[i]; k < g.cab_ptr[i + 1]; ++k) cab = p_add(cab, p_mul(p.cab[k], p.v_in[g.cab_col[k]]));
        const float2 vi = p.v_in[i];
        const float2 kw = p_renorm(pick<D>(hf, c), pick<D>(lf, c));
        const float2 num = p_sub(p_sub(p_sub(p.f[i], kw), p_mul(p.aml[i], vi)), cab);
        const float2 acc = p_mul(num, p.iml[i]);
        const float2 vn = p_add(vi, p_mul(p.dt, acc));
        const float2 un = p_add(p.u[i], p_mul(p.dt, vn));
        p.v_out[i] = vn;
        p.u[i] = un;
        p.w_out[i] = w_of(un, vn, p.beta);
        st.wp[kn + i] = p.w_in[i];
        st.v32[kn + i] = vi.x;
        st.a32[kn + i] = acc.x;
      }
      // backward rows of step nb
      const float2 yi = y[i];
      ys[i] = __fadd_rn(yi.x, yi.y);
      if (g.fixed[i]) {
        a.mu_u[i] = a.mu_v[i] = yn[i] = make_float2(0.f, 0.f);
        continue;
      }
      const float2 ky = p_renorm(pick<D>(hb, c), pick<D>(lb, c));
      float2 cy = make_float2(0.f, 0.f);
      for (int64_t q = g.cab_ptr[i]; q < g.cab_ptr[i + 1]; ++q) cy = p_add(cy, p_mul(p.cab[q], y[g.cab_col[q]]));
      const float2 mu_u = a.mu_u[i], mu_v = a.mu_v[i];
      const float2 gg = p_add(mu_v, p_mul(p.dt, mu_u));
      const float2 mu = p_sub(mu_u, p_mul(p.dt, ky));
      float2 mv = p_sub(gg, p_mul(p.dt, p_add(p_add(p_mul(p.beta, ky), cy), p_mul(p.aml[i], yi))));
      const int rj = a.rec_map[i];
      if (rj >= 0 && nb >= 1)
        mv = p_add(mv, p_of(a.out_v[(int64_t)nb * d.n_rec + rj] - d.target[(int64_t)nb * d.n_rec + rj]));
      a.mu_u[i] = mu;
      a.mu_v[i] = mv;
      yn[i] = p_mul(p_add(mv, p_mul(p.dt, mu)), p.iml[i]);
    }
  }
  if (last_block(&g.s->ticket)) {
    const int t = step - 1;
    if (g.f_ptr) {
      if (t >= 0 && t < g.n_t)
        for (int64_t k = g.f_ptr[t] + threadIdx.x; k < g.f_ptr[t + 1]; k += blockDim.x)
          p.f[g.f_slot[k]] = make_float2(0.f, 0.f);
      __syncthreads();
      if (t + 1 < g.n_t)
        for (int64_t k = g.f_ptr[t + 1] + threadIdx.x; k < g.f_ptr[t + 2]; k += blockDim.x)
          p.f[g.f_slot[k]] = p_of(g.f_val[k]);
    }
    if (threadIdx.x == 0) {
      g.s->ticket = 0;
      g.s->t = step;
      *a.n_dev = nb - 1;
    }
  }
}

constexpr int kAdjElemThreads = 128;

// Element gradients of one segment, steps t1 - 1 down to t0, once its backward steps are
// done: one lane per element node (32 / NEN elements per warp), lane (e, la) owning the
// element DOFs 3 la .. 3 la + 2 and holding its three rows of K1_e in registers for the whole
// segment (NEN <= 10; read per step for hexa20).  Per step, all FP32:
//   dJ/dE_e   -= dt y_e . [K1_e (u + beta v)_e + Lysmer terms]
//   dJ/drho_e -= dt sum ml1_e y_e (a + alpha v)_e + Lysmer term,
// (u + beta v) taken relative to the element's first node on the (hi, lo) pairs (K1
// annihilates rigid translations, so the FP32 products see strains); the Lysmer terms of
// boundary elements dealt to the element's lanes; per-element sums made by the element's
// first lane in lane order and accumulated in FP64 in step order, so the result does not
// depend on the checkpoint interval.
template <int NEN>
__global__ void __launch_bounds__(kAdjElemThreads) k_adj_grad_seg(Args g, sc_adj_desc d, AdjState a, int t0, int t1) {
  constexpr int ND = 3 * NEN, EPW = 32 / NEN;
  constexpr bool KREG = NEN <= 10;
  __shared__ __align__(16) float sw[kAdjElemThreads / 32][96];
  __shared__ float part[kAdjElemThreads / 32][32][2];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int grp = lane / NEN, la = lane % NEN, base = grp * NEN;
  const float alpha = (float)g.alpha_r;
  const int64_t warps = (int64_t)gridDim.x * (kAdjElemThreads / 32);
  for (int64_t wg = (int64_t)blockIdx.x * (kAdjElemThreads / 32) + wib; wg * EPW < d.n_elem; wg += warps) {
    const int64_t e = wg * EPW + grp;
    const bool on = grp < EPW && e < d.n_elem;
    int64_t sa = 0, s0 = 0, q0 = 0, q1 = 0;
    const float* K1 = d.ke1;
    float kr[KREG ? 3 * ND : 1];
    float ml[3] = {0.f, 0.f, 0.f};
    float iE = 0.f, iR = 0.f;
    double accE = 0.0, accR = 0.0;
    if (on) {
      const int* en = d.elem + e * NEN;
      sa = (int64_t)en[la] * 3;
      s0 = (int64_t)en[0] * 3;
      K1 = d.ke1 + (int64_t)d.ke_type[e] * ND * ND + (int64_t)(3 * la) * ND;
      if constexpr (KREG) {
#pragma unroll
        for (int j = 0; j < 3 * ND; ++j) kr[j] = __ldg(K1 + j);
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) ml[c] = d.ml1[e * ND + 3 * la + c];
      q0 = d.l_eptr[e];
      q1 = d.l_eptr[e + 1];
      if (q1 > q0) {
        iE = a.iE[e];
        iR = a.iR[e];
      }
      if (la == 0) {
        accE = a.gE[e];
        accR = a.gR[e];
      }
    }
    for (int n = t1 - 1; n >= t0; --n) {
      const int64_t off = (int64_t)(n - t0) * g.n_s;
      const float2* wp = a.wp + off;
      const float* v32 = a.v32 + off;
      const float* a32 = a.a32 + off;
      const float* ys = a.ys + off;
      float ya[3] = {0.f, 0.f, 0.f}, gr = 0.f;
      if (on) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float2 wb = wp[sa + c], w0 = wp[s0 + c];
          sw[wib][base * 3 + 3 * la + c] = (wb.x - w0.x) + (wb.y - w0.y);
          ya[c] = ys[sa + c];
          gr = fmaf(ml[c] * ya[c], fmaf(alpha, v32[sa + c], a32[sa + c]), gr);
        }
      }
      __syncwarp();
      float ge = 0.f;
      if (on) {
        const float* wv = &sw[wib][base * 3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float r = 0.f;
#pragma unroll
          for (int b = 0; b < ND; ++b) {
            float kv;
            if constexpr (KREG) kv = kr[c * ND + b];
            else kv = __ldg(K1 + c * ND + b);
            r = fmaf(kv, wv[b], r);
          }
          ge = fmaf(ya[c], r, ge);
        }
        // Lysmer terms of boundary elements (dashpots ~ sqrt(rho E), springs ~ E)
        for (int64_t q = q0 + la; q < q1; q += NEN) {
          const float yr = ys[d.l_row[q]];
          const float2 wq = wp[d.l_col[q]];
          const float wc = wq.x + wq.y, vc = v32[d.l_col[q]];
          const float hc = __fmul_rn(0.5f, d.l_c[q]);
          ge = fmaf(yr, fmaf(__fmul_rn(d.l_s[q], iE), wc, __fmul_rn(__fmul_rn(hc, iE), vc)), ge);
          gr = fmaf(yr, __fmul_rn(__fmul_rn(hc, iR), vc), gr);
        }
      }
      part[wib][lane][0] = ge;
      part[wib][lane][1] = gr;
      __syncwarp();
      if (on && la == 0) {
        float ge_e = 0.f, gr_e = 0.f;
        for (int q = 0; q < NEN; ++q) {
          ge_e += part[wib][base + q][0];
          gr_e += part[wib][base + q][1];
        }
        accE -= g.dt * (double)ge_e;
        accR -= g.dt * (double)gr_e;
      }
      __syncwarp();
    }
    if (on && la == 0) {
      a.gE[e] = accE;
      a.gR[e] = accR;
    }
  }
}

// start of the backward sweep: mu_u = 0, mu_v = P^T (v_N - d_N), y = mu_v / M_L
__global__ void k_adj_init(Args g, PairStep p, AdjState a, const double* target, int n_rec, int N) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n_s; i += (int64_t)gridDim.x * blockDim.x) {
    a.mu_u[i] = make_float2(0.f, 0.f);
    const int rj = a.rec_map[i];
    const float2 mv = rj >= 0 && !g.fixed[i]
                          ? p_of(a.out_v[(int64_t)N * n_rec + rj] - target[(int64_t)N * n_rec + rj])
                          : make_float2(0.f, 0.f);
    a.mu_v[i] = mv;
    a.y[0][i] = g.fixed[i] ? make_float2(0.f, 0.f) : p_mul(mv, p.iml[i]);
  }
}

__global__ void k_adj_recip(int n, const double* young, const double* rho, float* iE, float* iR) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    iE[e] = (float)(1.0 / young[e]);
    iR[e] = (float)(1.0 / rho[e]);
  }
}

__global__ void k_adj_misfit(const double* out_v, const double* target, int n_rec, int N, double* J) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int64_t q = (int64_t)n_rec + threadIdx.x; q < (int64_t)(N + 1) * n_rec; q += blockDim.x) {
    const double r = out_v[q] - target[q];
    s += r * r;
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) *J = 0.5 * s;
}

__global__ void k_adj_recmap(int n_s, int n_rec, const int* rec, int* map) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_s; i += (int64_t)gridDim.x * blockDim.x) map[i] = -1;
}
__global__ void k_adj_recmap_fill(int n_rec, const int* rec, int* map) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n_rec; j += gridDim.x * blockDim.x) map[rec[j]] = j;
}

template <int TPR>
void launch_adj_rows_t(const sc_nb_newmark* h, cudaStream_t st, const sc_adj_desc& d, const AdjState& a, int cur) {
  k_adj_rows<3, TPR><<<h->tpr_blocks, kThreads, 0, st>>>(h->g, pair_step(h, 0), d, a, cur);
}
void launch_adj_rows(const sc_nb_newmark* h, cudaStream_t st, const sc_adj_desc& d, const AdjState& a, int cur) {
  switch (h->tpr) {
    case 4: launch_adj_rows_t<4>(h, st, d, a, cur); break;
    case 2: launch_adj_rows_t<2>(h, st, d, a, cur); break;
    default: launch_adj_rows_t<1>(h, st, d, a, cur); break;
  }
}

template <int NEN>
void launch_grad_seg_t(const sc_nb_newmark* h, cudaStream_t st, const sc_adj_desc& d, const AdjState& a, int t0,
                       int t1) {
  const int64_t warps = (d.n_elem + 32 / NEN - 1) / (32 / NEN);
  k_adj_grad_seg<NEN><<<grid_for(warps, kAdjElemThreads / 32, 152 * 32), kAdjElemThreads, 0, st>>>(h->g, d, a, t0, t1);
}
void launch_grad_seg(const sc_nb_newmark* h, cudaStream_t st, const sc_adj_desc& d, const AdjState& a, int t0, int t1) {
  switch (d.n_en) {
    case 4: launch_grad_seg_t<4>(h, st, d, a, t0, t1); break;
    case 8: launch_grad_seg_t<8>(h, st, d, a, t0, t1); break;
    case 10: launch_grad_seg_t<10>(h, st, d, a, t0, t1); break;
    default: launch_grad_seg_t<20>(h, st, d, a, t0, t1); break;
  }
}

template <int TPR>
void launch_adj_fused_t(const sc_nb_newmark* h, cudaStream_t st, int kk, const SegStore& store, const sc_adj_desc& d,
                        const AdjState& a, int cur) {
  k_adj_fused<3, TPR><<<h->tpr_blocks, kThreads, 0, st>>>(h->g, pair_step(h, kk), store, d, a, cur);
}
void launch_adj_fused(const sc_nb_newmark* h, cudaStream_t st, int kk, const SegStore& store, const sc_adj_desc& d,
                      const AdjState& a, int cur) {
  switch (h->tpr) {
    case 4: launch_adj_fused_t<4>(h, st, kk, store, d, a, cur); break;
    case 2: launch_adj_fused_t<2>(h, st, kk, store, d, a, cur); break;
    default: launch_adj_fused_t<1>(h, st, kk, store, d, a, cur); break;
  }
}

}  // namespace

// Forward from rest with pair checkpoints every `checkpoint` steps, then the reverse sweep
// over the segments, last first, on the handle's stream: the last segment is recomputed from
// its checkpoint (the explicit step storing the element gradient's inputs into one of two
// segment buffers); then for each segment s the backward steps of s run fused with the
// recompute steps of s - 1 into the other buffer (one kernel per pair of steps, one pass over
// the K planes for both), the rest of either alone, then one element-gradient kernel for the
// whole of s.  The forward and the recompute run the same arithmetic from the same pair state,
// so the recomputed states are bitwise the forward's.  Requires the pair arithmetic (the
// default).
extern "C" int sc_nb_adjoint(sc_nb_newmark* h, const sc_adj_desc* dp, double* J_host, double* grad_E,
                             double* grad_rho) {
  if (!h || !dp || !grad_E || !grad_rho) return SC_BAD_ARG;
  const sc_adj_desc d = *dp;
  if (d.n_steps <= 0 || d.checkpoint <= 0 || d.n_rec <= 0 || !d.rec_slot || !d.target || d.n_elem <= 0 ||
      !(d.n_en == 4 || d.n_en == 8 || d.n_en == 10 || d.n_en == 20) || !d.elem || !d.ke_type || !d.ke1 ||
      !d.young || !d.rho || !d.ml1 || !d.l_eptr || h->g.D != 3 || !h->explicit_pair)
    return SC_BAD_ARG;
  Args& g = h->g;
  cudaStream_t st = h->user;
  const int N = d.n_steps, C = d.checkpoint < d.n_steps ? d.checkpoint : d.n_steps, nseg = (N + C - 1) / C;
  const int nbuf = nseg > 1 ? 2 : 1;
  auto buf = [&](int sgi) { return nbuf == 2 ? (sgi & 1) : 0; };
  auto seg0 = [&](int sgi) { return sgi * C; };
  auto seg1 = [&](int sgi) { return sgi * C + C < N ? sgi * C + C : N; };
  const int64_t ns = g.n_s;
  // the caller's output configuration, restored at the end
  const int o_int = g.out_interval, o_nrec = g.n_rec;
  const int* o_rec = g.rec_slot;
  double *o_u = g.out_u, *o_v = g.out_v, *o_a = g.out_a;
  const int64_t o_nout = g.n_out;
  AdjState a[2] = {};
  AdjState& s = a[0];  // the fields both buffers share are set here and copied
  float2 *ck_u = nullptr, *ck_v = nullptr;
  int* t_host = nullptr;  // [0, nseg) segment starts, [nseg, 2 nseg) backward starts; pinned
  int* t0_dev = nullptr;  // the segment start of each buffer
  int rc = SC_OK;
  auto M = [&](void** p, size_t b) { return check(cudaMallocAsync(p, b, st), "adjoint malloc"); };
  // phase timers: forward [0, 1]; the last segment's recompute [1, 2]; the rest of the sweep [2, 3]
  cudaEvent_t tev[4] = {};
  // threads per node row for the whole adjoint (forward, recompute and backward alike, so the
  // recomputed states are bitwise the forward's): the handle's tuned value, lowered until the
  // fused kernel, with its two sets of accumulators, fits in one wave of resident blocks
  const int tpr0 = h->tpr;
  const unsigned blocks0 = h->tpr_blocks;
  {
    int dev = 0, n_sm = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    int tpr = tpr0;
    while (tpr > 1) {
      int per_sm = 0;
      cudaError_t e = tpr == 4   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_adj_fused<3, 4>, kThreads, 0)
                      : tpr == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_adj_fused<3, 2>, kThreads, 0)
                                 : cudaErrorInvalidValue;
      const int64_t want = (((int64_t)g.n_nodes + 31) / 32 * 32 * tpr + kThreads - 1) / kThreads;
      if (e == cudaSuccess && want <= (int64_t)per_sm * n_sm) break;
      tpr /= 2;
    }
    cudaGetLastError();
    const int64_t want = (((int64_t)g.n_nodes + 31) / 32 * 32 * tpr + kThreads - 1) / kThreads;
    h->tpr = tpr;
    h->tpr_blocks = (unsigned)(want < 152 * 16 ? (want < 1 ? 1 : want) : 152 * 16);
  }
  do {
    if ((rc = M((void**)&ck_u, 8 * ns * nseg)) || (rc = M((void**)&ck_v, 8 * ns * nseg)) ||
        (rc = M((void**)&s.mu_u, 8 * ns)) || (rc = M((void**)&s.mu_v, 8 * ns)) || (rc = M((void**)&s.y[0], 8 * ns)) ||
        (rc = M((void**)&s.y[1], 8 * ns)) || (rc = M((void**)&s.out_v, 8 * (int64_t)(N + 1) * d.n_rec)) ||
        (rc = M((void**)&s.n_dev, 4)) || (rc = M((void**)&s.ticket_r, 4)) || (rc = M((void**)&t0_dev, 8)) ||
        (rc = M((void**)&s.rec_map, 4 * ns)) || (rc = M((void**)&s.J, 8)) ||
        (rc = M((void**)&s.iE, 4 * (size_t)d.n_elem)) || (rc = M((void**)&s.iR, 4 * (size_t)d.n_elem)))
      break;
    s.gE = grad_E;
    s.gR = grad_rho;
    a[1] = s;
    for (int b = 0; b < nbuf && !rc; ++b) {
      a[b].seg_t0 = t0_dev + b;
      if ((rc = M((void**)&a[b].wp, 8 * ns * C)) || (rc = M((void**)&a[b].v32, 4 * ns * C)) ||
          (rc = M((void**)&a[b].a32, 4 * ns * C)) || (rc = M((void**)&a[b].ys, 4 * ns * C)))
        break;
    }
    if (rc) break;
    if ((rc = check(cudaMallocHost((void**)&t_host, 8 * (size_t)nseg), "adjoint pinned"))) break;
    for (auto& ev : tev)
      if ((rc = check(cudaEventCreate(&ev), "adjoint timer"))) break;
    if (rc) break;
    cudaMemsetAsync(s.ticket_r, 0, 4, st);
    k_adj_recip<<<grid_for(d.n_elem, 256), 256, 0, st>>>(d.n_elem, d.young, d.rho, s.iE, s.iR);
    cudaMemsetAsync(grad_E, 0, 8 * (size_t)d.n_elem, st);
    cudaMemsetAsync(grad_rho, 0, 8 * (size_t)d.n_elem, st);
    cudaMemsetAsync(s.out_v, 0, 8 * (size_t)(N + 1) * d.n_rec, st);
    k_adj_recmap<<<grid_for(ns, 256), 256, 0, st>>>((int)ns, d.n_rec, d.rec_slot, s.rec_map);
    k_adj_recmap_fill<<<grid_for(d.n_rec, 128), 128, 0, st>>>(d.n_rec, d.rec_slot, s.rec_map);
    // receivers recorded into out_v; the explicit graphs are rebuilt for that output
    if ((rc = sc_nb_set_output(h, 1, d.n_rec, d.rec_slot, nullptr, s.out_v, nullptr, N + 1))) break;
    if ((rc = explicit_prepare(h))) break;
    // forward from rest with checkpoints
    cudaMemsetAsync(h->u2, 0, 8 * ns, st);
    cudaMemsetAsync(h->v2[0], 0, 8 * ns, st);
    force_reset(h, 0);
    cudaEventRecord(tev[0], st);
    for (int sgi = 0; sgi < nseg && !rc; ++sgi) {
      cudaMemcpyAsync(ck_u + sgi * ns, h->u2, 8 * ns, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(ck_v + sgi * ns, h->v2[0], 8 * ns, cudaMemcpyDeviceToDevice, st);
      rc = explicit_steps(h, seg0(sgi), seg1(sgi));
    }
    if (rc) break;
    cudaEventRecord(tev[1], st);
    k_adj_misfit<<<1, 1024, 0, st>>>(s.out_v, d.target, d.n_rec, N, s.J);
    k_adj_init<<<h->vec_blocks, 256, 0, st>>>(g, pair_step(h, 0), s, d.target, d.n_rec, N);
    // the recompute records no receivers (the forward's records stand)
    g.n_rec = 0;
    // restore segment sgi's checkpoint as the recompute's state, its start in its buffer
    auto recompute_setup = [&](int sgi) {
      const int b = buf(sgi);
      t_host[sgi] = seg0(sgi);
      cudaMemcpyAsync(h->u2, ck_u + sgi * ns, 8 * ns, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(h->v2[0], ck_v + sgi * ns, 8 * ns, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(a[b].seg_t0, t_host + sgi, 4, cudaMemcpyHostToDevice, st);
      k_w_pairs<<<h->vec_blocks, 256, 0, st>>>(ns, h->u2, h->v2[0], host_pair(g.beta_r), h->w2[0]);
      force_reset(h, seg0(sgi), st);
      k_set_t<<<1, 1, 0, st>>>(g.s, seg0(sgi));
    };
    auto store_of = [&](int sgi) {
      const AdjState& ab = a[buf(sgi)];
      return SegStore{ab.wp, ab.v32, ab.a32, ab.seg_t0};
    };
    recompute_setup(nseg - 1);
    int kk = 0;  // ping-pong parity of the recompute's state buffers
    for (int t = seg0(nseg - 1); t < seg1(nseg - 1); ++t, kk ^= 1) launch_pair<3>(h, st, kk, store_of(nseg - 1));
    cudaEventRecord(tev[2], st);
    int yk = 0;  // y[yk] holds the y of the next step to reverse
    for (int sgi = nseg - 1; sgi >= 0; --sgi) {
      const AdjState& ab = a[buf(sgi)];
      const int len_b = seg1(sgi) - seg0(sgi), len_r = sgi >= 1 ? seg1(sgi - 1) - seg0(sgi - 1) : 0;
      t_host[nseg + sgi] = seg1(sgi) - 1;
      cudaMemcpyAsync(s.n_dev, t_host + nseg + sgi, 4, cudaMemcpyHostToDevice, st);
      if (sgi >= 1) {
        recompute_setup(sgi - 1);
        kk = 0;
      }
      for (int j = 0; j < len_b; ++j, yk ^= 1) {
        if (j < len_r) {
          launch_adj_fused(h, st, kk, store_of(sgi - 1), d, ab, yk);
          kk ^= 1;
        } else {
          launch_adj_rows(h, st, d, ab, yk);
        }
      }
      for (int j = len_b; j < len_r; ++j, kk ^= 1) launch_pair<3>(h, st, kk, store_of(sgi - 1));
      launch_grad_seg(h, st, d, ab, seg0(sgi), seg1(sgi));
      if ((rc = check_launch("adjoint sweep"))) break;
    }
    if (rc) break;
    cudaEventRecord(tev[3], st);
    if (J_host && (rc = check(cudaMemcpyAsync(J_host, s.J, 8, cudaMemcpyDeviceToHost, st), "J"))) break;
    if ((rc = check(cudaStreamSynchronize(st), "sync adjoint"))) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, tev[0], tev[1]);
    h->adj_ms[0] = ms;
    cudaEventElapsedTime(&ms, tev[1], tev[2]);
    h->adj_ms[1] = ms;
    cudaEventElapsedTime(&ms, tev[2], tev[3]);
    h->adj_ms[2] = ms;
    cudaEventElapsedTime(&ms, tev[1], tev[3]);
    h->adj_ms[3] = ms;
  } while (0);
  g.n_rec = d.n_rec;
  cudaStreamSynchronize(st);
  for (auto ev : tev)
    if (ev) cudaEventDestroy(ev);
  void* frees[] = {ck_u,  ck_v,     s.mu_u, s.mu_v,  s.y[0], s.y[1], s.out_v, s.n_dev, s.ticket_r, t0_dev, s.rec_map,
                   s.J,   s.iE,     s.iR,   a[0].wp, a[0].v32, a[0].a32, a[0].ys, a[1].wp, a[1].v32, a[1].a32, a[1].ys};
  for (void* q : frees)
    if (q) cudaFree(q);
  if (t_host) cudaFreeHost(t_host);
  sc_nb_set_output(h, o_int, o_nrec, o_rec, o_u, o_v, o_a, o_nout);  // drops the explicit graphs
  h->tpr = tpr0;
  h->tpr_blocks = blocks0;
  return rc;
}

// [0] forward with checkpoints; [1] recompute of the last segment (alone); [2] the rest of the
// reverse sweep (backward steps fused with the previous segment's recompute, element
// gradients); [3] the reverse sweep's wall time, [1] + [2]
extern "C" int sc_nb_adjoint_timings(sc_nb_newmark* h, float* ms4) {
  if (!h || !ms4) return SC_BAD_ARG;
  for (int i = 0; i < 4; ++i) ms4[i] = h->adj_ms[i];
  return SC_OK;
}
