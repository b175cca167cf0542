// Shared declarations of the node-block solver (sc_nbsolver.cu: Newmark/PCG, setup) and the
// explicit scheme with its adjoint (sc_explicit.cu): kernel argument block, the handle, the
// sliced-ELL row helpers and the FP32-pair arithmetic helpers.
#pragma once
#include <math.h>
#include <stdlib.h>

#include <cuda_fp16.h>

#include "sc_common.cuh"

namespace sc {
namespace nb {

constexpr int kThreads = 256;
constexpr int kMaxFsai = 64;  // FSAI row pattern capacity (slots); larger rows fall back to Jacobi

struct Scal {
  double rz, pw, rr, bb, alpha, beta, tol2, pad0;
  long long total_iters;
  int it, max_it, max_seen, status, t, fsai_fallback;
  unsigned int ticket;
  int hist;  // valid previous accelerations (0..kHistMax) for the warm start
  int head;  // ring slot of the most recent one (hist_slot)
  int done;  // eager mode: set when the PCG loop should stop
  // adaptive warm-start order: current order, probing direction, window and hold counters
  int pord, pdir, win_n, win_it, probing, hold;
  double ref_avg;  // mean iterations per step of the reference window
  int res_fp64;       // 1: the residual runs in FP64 (for good, once the pair residual saw strong cancellation)
  int res_fp64_next;  // set by the pair residual; k_advance copies it into res_fp64 at the end of the step
  // the FP32 matrix (A's hi parts) in the PCG: with Ah = hi, A = Ah + Al, the solve runs on Ah
  // and the true residual b - A x differs from the recursive one by -Al (x - x0), at most
  // lo_norm |x - x0| (lo_norm >= ||Al||_2)
  int a32;            // 1: this step's PCG SpMV applies Ah alone
  int restart;        // 1: the bound failed; the next preconditioner pass restarts from x0, r0 in pairs
  int sw;             // 1: the solve switches to Ah now; the next preconditioner pass makes x, r the new x0, r0
  int no_switch;      // 1: this step restarted in pairs and stays there
  double lo_norm;     // sqrt(||Al||_1 ||Al||_inf)
  double rr0, dd;     // |r0|^2 of the step, |x - x0|^2 after the last update
  double dd_pre;      // |x - x0|^2 at a switch (x0 before the switch)
  double rho;         // |x - x0| / |r0| of the last step that moved (-1: none yet)
  long long a32_steps, switched, restarts;
  int pcap;           // this step's cap on the warm-start order from the force history (k_order_cap)
  long long capped;   // steps whose order the cap lowered
};

struct Args {
  int n_nodes, D;
  int64_t n_s;  // slots
  int64_t nnzb;
  const int64_t* adj_ptr;
  const int* adj;
  const int64_t* diag;  // position of the node itself in its adjacency row
  const int* fixed;     // [n_s] 1 = fixed slot
  const double *KB, *AB, *MS;
  const float *GB, *GTB;
  const int64_t* cab_ptr;
  const int* cab_col;
  const double* cab_val;
  // sliced-ELL copies used by the per-step kernels (32 node rows per slice, column-major):
  // full pattern (K, A, M), lower (G), upper (G^T)
  int64_t n_slices;
  const int64_t *sf_ptr, *sl_ptr, *su_ptr;
  const int *sf_col, *sl_col, *su_col;
  int64_t sf_n, sl_n, su_n;
  const double *KS, *AS, *MSS;
  const __half *GS, *GTS;  // FSAI factor planes, FP16, scaled by a power of two (max |entry| in [0.5, 1))
  const float2* APS;       // A as FP32 (hi, lo) pairs (hi + lo = A to 48 bits) for the pair-arithmetic SpMV
  const float* AHS;        // the pairs' hi parts alone: the FP32 matrix of the a32 SpMV
  const float2* KPS;       // K as FP32 pairs, for the explicit step and the adjoint (built on first use)
  float2* p2;              // p as (hi, lo) FP32 pairs, written with p
  // the pair residual (k_residual_kp): r = f - K (q1 + aK x0) - M (q2 + aM x0) - Cabs (y1 + aC x0)
  const float2* MSP;       // the consistent-mass plane as FP32 pairs
  float* rrec;             // per node, what the pair residual gathers (k_predict writes it): kRecFloats
                           // floats; the mass part at kRecM: [0, 2D) q2 + aM x0 as (hi, lo) pairs,
                           // [2D, 3D) q2 in FP32; the stiffness part at kRecK(D): [0, 2D) q1 + aK x0
                           // as pairs, [2D, 3D) q1 in FP32 (q1, q2 for |b| and the cancellation check)
  double* zc;              // y1 + aC x0 (dashpot rows)
  int res_pair;            // 1: k_predict writes the vectors above and the step runs k_residual_kp
  int spmv_pair;           // 1: PCG SpMV in FP32-pair arithmetic, 0: FP64
  int keep_l2;             // 1: matrix planes fit in L2, loaded with the default (keep) policy;
                           // 0: streamed with evict-first loads
  double alpha_r, beta_r;  // Rayleigh coefficients
  double aM, aK, aC;       // A = aM M + aK K + aC Cabs
  double dt;
  double *u, *v, *a;
  double* ah[kHistMax];  // previous accelerations, a ring: a_{n-1-k} in ah[hist_slot(head, k)]
  int pred_order;        // order of the warm start's extrapolation (1..kHistMax), 0: adaptive (Scal::pord)
  double *q1, *q2, *y1, *x0, *x, *r, *z, *p, *w, *f;
  float* t32;
  float* r32;  // FP32 copy of r, written with r: the lower FSAI half gathers it (no FP64 conversion per gather)
  double* r0;   // the step's initial residual, and its FP32 copy: a restart of the PCG starts from them
  float* r032;
  int a32_mode;  // FP32 matrix in the PCG: 0 never, 1 when the bound allows (default), 2 every step
  int order_cap; // 1: cap the warm-start order where the force history has a kink (default)
  double* part;
  Scal* s;
  // force (slot indices)
  int n_t;
  const int64_t* f_ptr;
  const int* f_slot;
  const double* f_val;
  // output
  int out_interval, n_rec;
  const int* rec_slot;
  double *out_u, *out_v, *out_a;
  int64_t n_out;
};

// floats per node of the pair residual's record (whole 16-byte pieces), and where its mass and
// stiffness parts start
__host__ __device__ constexpr int kRecFloats(int D) { return D == 3 ? 20 : 12; }
constexpr int kRecM = 0;
__host__ __device__ constexpr int kRecK(int D) { return 3 * D; }

// v = rec[I, E) with the widest aligned loads (a record starts on 16 bytes)
template <int I, int E>
__device__ __forceinline__ void ldrec_(const float* rec, float* v) {
  if constexpr (I < E) {
    if constexpr (I % 4 == 0 && I + 4 <= E) {
      const float4 t = *reinterpret_cast<const float4*>(rec + I);
      v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
      ldrec_<I + 4, E>(rec, v + 4);
    } else if constexpr (I % 2 == 0 && I + 2 <= E) {
      const float2 t = *reinterpret_cast<const float2*>(rec + I);
      v[0] = t.x; v[1] = t.y;
      ldrec_<I + 2, E>(rec, v + 2);
    } else {
      v[0] = rec[I];
      ldrec_<I + 1, E>(rec, v + 1);
    }
  }
}
template <int A, int N>
__device__ __forceinline__ void ldrec(const float* rec, float (&v)[N]) {
  ldrec_<A, A + N>(rec, v);
}

// node n's D values of an FP32 slot vector
template <int D>
__device__ __forceinline__ void ldvec(const float* v, int64_t n, float (&o)[D]) {
#pragma unroll
  for (int d = 0; d < D; ++d) o[d] = v[n * D + d];
}

__device__ inline bool last_block(unsigned int* ticket) {
  __shared__ bool am_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) am_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  return am_last;
}

// kMode 0: inside the step graph (drives the WHILE conditional); 1: eager launches (the host
// reads Scal::done); 2: standalone timing launch (no solver scalars touched)
template <int kMode>
__device__ inline void pcg_continue(cudaGraphConditionalHandle hc, Scal* s, bool go) {
  if (kMode == 0) cudaGraphSetConditional(hc, go ? 1u : 0u);
  else if (kMode == 1) s->done = go ? 0 : 1;
}

__device__ inline double reduce_parts(const double* part, int k, double* sh) {
  double s = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s += __ldcg(part + b * 4 + k);
  return block_sum(s, sh);
}

// reduce_parts of slots k0 and k1 in one pass (the same bits as two calls); sh: 64 doubles
__device__ inline void reduce_parts2(const double* part, int k0, int k1, double* sh, double& s0, double& s1) {
  s0 = 0.0;
  s1 = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
    s0 += __ldcg(part + b * 4 + k0);
    s1 += __ldcg(part + b * 4 + k1);
  }
  block_sum2(s0, s1, sh);
}

template <int D>
__device__ inline void warp_sum3(double* s) {
#pragma unroll
  for (int c = 0; c < D; ++c) s[c] = warp_sum(s[c]);
}


// Per-step block kernels: one thread per node row over the sliced-ELL copies.  A warp is one
// slice of 32 consecutive node rows.  The slice's width W (its longest row, rounded up to a
// multiple of 4) is stored as W/4 chunks: entry j of the row in lane l sits at
//   ptr[slice] + 128 (j / 4) + 4 l + (j % 4),
// so a lane's four entries of a chunk are adjacent (one 16-byte column load, one 16- or
// 32-byte load per plane) and a warp reads 512 contiguous bytes per 4-byte plane.  Padding
// entries point at the row's own node with zero values.
#define SELL_ROW_LOOP(ptr)                                                                      \
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < g.n_slices * 32;    \
       row += (int64_t)gridDim.x * blockDim.x)
// first entry of this lane's row and the slice's chunk count
#define SELL_ROW_BEGIN(ptr)                                 \
  const int64_t sl_ = row >> 5;                             \
  const int64_t p0 = (ptr)[sl_] + 4 * (row & 31);           \
  const int64_t nq = ((ptr)[sl_ + 1] - (ptr)[sl_]) >> 7;

__device__ __forceinline__ void cols4(const int* c, int64_t pos, int (&v)[4], int keep) {
  const int4* q = reinterpret_cast<const int4*>(c + pos);
  const int4 a = keep ? __ldg(q) : __ldcs(q);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
__device__ __forceinline__ void ld4(const double* p, double (&v)[4], int keep) {
  const double2* q = reinterpret_cast<const double2*>(p);
  const double2 a = keep ? __ldg(q) : __ldcs(q);
  const double2 b = keep ? __ldg(q + 1) : __ldcs(q + 1);
  v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
__device__ __forceinline__ void ld4(const float* p, float (&v)[4], int keep) {
  const float4* q = reinterpret_cast<const float4*>(p);
  const float4 a = keep ? __ldg(q) : __ldcs(q);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
__device__ __forceinline__ void ld4(const __half* p, float (&v)[4], int keep) {
  const uint2* q = reinterpret_cast<const uint2*>(p);
  const uint2 a = keep ? __ldg(q) : __ldcs(q);
  const float2 lo = __half22float2(*reinterpret_cast<const __half2*>(&a.x));
  const float2 hi = __half22float2(*reinterpret_cast<const __half2*>(&a.y));
  v[0] = lo.x; v[1] = lo.y; v[2] = hi.x; v[3] = hi.y;
}
__device__ __forceinline__ void ld4(const float2* p, float2 (&v)[4], int keep) {
  const float4* q = reinterpret_cast<const float4*>(p);
  const float4 a = keep ? __ldg(q) : __ldcs(q);
  const float4 b = keep ? __ldg(q + 1) : __ldcs(q + 1);
  v[0] = make_float2(a.x, a.y); v[1] = make_float2(a.z, a.w); v[2] = make_float2(b.x, b.y); v[3] = make_float2(b.z, b.w);
}
__device__ __forceinline__ void ld2(const double* p, double (&v)[2], int keep) {
  const double2* q = reinterpret_cast<const double2*>(p);
  const double2 a = keep ? __ldg(q) : __ldcs(q);
  v[0] = a.x; v[1] = a.y;
}
__device__ __forceinline__ void ld2f(const float* p, float2& v, int keep) {
  const float2* q = reinterpret_cast<const float2*>(p);
  v = keep ? __ldg(q) : __ldcs(q);
}
__device__ __forceinline__ void ld2(const float2* p, float2 (&v)[2], int keep) {
  const float4* q = reinterpret_cast<const float4*>(p);
  const float4 a = keep ? __ldg(q) : __ldcs(q);
  v[0] = make_float2(a.x, a.y); v[1] = make_float2(a.z, a.w);
}
// TPR threads per node row (TPR divides 32): the row's chunks are dealt round-robin to its
// TPR lanes and the partial sums combined by shuffles.  A warp covers 32 / TPR rows of one
// slice, so loop trips are warp-uniform (full-mask shuffles are safe).
#define SELL_ROW_LOOP_T(tpr)                                                                            \
  for (int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / (tpr); row < g.n_slices * 32; \
       row += (int64_t)gridDim.x * blockDim.x / (tpr))

// combine the TPR lanes' partial sums of a row; every lane ends with the group leader's result
template <int TPR>
__device__ __forceinline__ void group_pair_sum(float& hi, float& lo) {
  if constexpr (TPR > 1) {
#pragma unroll
    for (int o = 1; o < TPR; o <<= 1) {
      const float h2 = __shfl_xor_sync(0xffffffffu, hi, o), l2 = __shfl_xor_sync(0xffffffffu, lo, o);
      pair_add(hi, lo, h2, l2);
    }
    const int lead = (threadIdx.x & 31) & ~(TPR - 1);
    hi = __shfl_sync(0xffffffffu, hi, lead);
    lo = __shfl_sync(0xffffffffu, lo, lead);
  }
}
template <int TPR>
__device__ __forceinline__ double group_sum(double x) {
  if constexpr (TPR > 1) {
#pragma unroll
    for (int o = 1; o < TPR; o <<= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    x = __shfl_sync(0xffffffffu, x, (threadIdx.x & 31) & ~(TPR - 1));
  }
  return x;
}


static __global__ void k_set_t(Scal* s, int t) { s->t = t; }

static __global__ void k_hi_parts(int64_t n, const float2* __restrict__ hl, float* __restrict__ hi) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    hi[i] = hl[i].x;
}

static __global__ void k_split_pairs(int64_t n, const double* __restrict__ x, float2* __restrict__ hl) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float h = (float)x[i];
    hl[i] = make_float2(h, (float)(x[i] - (double)h));
  }
}

}  // namespace nb
}  // namespace sc

struct sc_nb_newmark {
  sc::nb::Args g;
  void* sell_mem[16] = {};
  int n_sell_mem = 0;
  cudaStream_t user = nullptr, cap = nullptr, cap2 = nullptr;
  unsigned node_blocks = 1, vec_blocks = 1, pred_blocks = 1;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // ---- explicit scheme (sc_explicit.cu), allocated on first use
  int explicit_pair = 1;  // 1: FP32-pair state and products (no FP64 in the step); 0: FP64
  // threads per node row of the explicit step and the adjoint rows (more on small meshes, so
  // the SMs have enough warps to cover load latency) and their grid
  int tpr = 1;
  unsigned tpr_blocks = 1;
  int ex_wide = 0;     // explicit step kernel at the wide register budget (sc_nb_tune_explicit)
  int ex_keep_ct = 0;  // explicit step kernel with the planes' load policy at compile time (the same)
  double *ML = nullptr, *IML = nullptr;  // lumped mass (row sums unless set by the caller)
  int ml_user = 0;                       // 1: ML set by sc_nb_set_lumped_mass
  double *v1 = nullptr, *w0 = nullptr, *w1 = nullptr;  // FP64 mode ping-pong buffers
  float2* KPS = nullptr;                               // K pair planes
  float2 *u2 = nullptr, *v2[2] = {nullptr, nullptr}, *w2[2] = {nullptr, nullptr};  // pair state
  float2 *f2 = nullptr, *aml2 = nullptr, *iml2 = nullptr, *cab2 = nullptr;
  int* rec_map = nullptr;
  cudaGraphExec_t ex_exec[2] = {nullptr, nullptr};
  cudaGraph_t ex_graph[2] = {nullptr, nullptr};
  float adj_ms[4] = {0.f, 0.f, 0.f, 0.f};  // last sc_nb_adjoint: forward, recompute, backward, reverse sweep (ms)
  int res_pair = 1;                        // pair residual allowed (sc_nb_set_options bit 2 clears it)
  void* res_mem[6] = {};                   // its mass pairs and vectors, made on first use
};

// sc_explicit.cu
void drop_explicit_graphs(sc_nb_newmark* h);
void free_explicit(sc_nb_newmark* h);
