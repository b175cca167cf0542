// Node-block Newmark solver: the time loop of the reference (PuggleSolvers NewmarkExplicit as
// driven by scatter/scatter.py:120-159: beta = 1/4, gamma = 1/2, consistent mass, constant
// effective matrix) on a 3x3 (2x2 in 2D) node-block layout.
//
// Layout (HBM).  Unknowns live in "slot" space: slot = node * D + d for every node and DOF,
// fixed DOFs included as decoupled slots whose values stay 0.  Matrices are blocks over the
// node adjacency of the element graph (adj_ptr/adj, neighbours sorted, self included):
//   KB, AB  [D*D][nnzb] FP64, one plane per block component (lane-coalesced loads)
//   MS      [nnzb] FP64   the consistent mass is m_ab * I per node pair (Me = rho N^T N)
//   GB, GTB [D*D][nnzb] FP32  factorised sparse approximate inverse (FSAI) of A: G on the
//           lower part of each node row (neighbours b <= a), G^T on the upper part
//   Cabs    small slot-space CSR holding the Lysmer dashpots (boundary rows only)
// with A = M + dt/2 C + dt^2/4 K and C = Cabs + alpha M + beta K (Rayleigh), so
//   b  = f - C vp - K up = f - K q1 - M q2 - Cabs y1
//   q1 = up + beta y1, q2 = alpha y1, y1 = vp (+ the usual predictor terms, see k_predict)
// Each step solves A x = b for the new acceleration by PCG with preconditioner G^T G,
// warm-started from the quadratic extrapolation 3a_n - 3a_{n-1} + a_{n-2}, stopped at
// ||r|| <= rtol ||b||; then u, v, a are updated exactly as the reference's update.
//
// Kernels: one warp per node row (lanes over the row's blocks) for every block product;
// per-block partial sums reduced by the last block (ticket, fixed order, no spin-waits);
// one CUDA graph per step with a device-side WHILE conditional around the PCG body.
#include <math.h>
#include <stdlib.h>

#include <vector>

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
  int hist;  // valid previous accelerations (0..2) for the warm start
  int done;  // eager mode: set when the PCG loop should stop
  unsigned int pad2[1];
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
  const float *GS, *GTS;
  const float2* APS;       // A as FP32 (hi, lo) pairs (hi + lo = A to 48 bits) for the pair-arithmetic SpMV
  const float2* KPS;       // K as FP32 pairs, for the explicit step and the adjoint (built on first use)
  float2* p2;              // p as (hi, lo) FP32 pairs, written with p
  int spmv_pair;           // 1: PCG SpMV in FP32-pair arithmetic, 0: FP64
  int keep_l2;             // 1: matrix planes fit in L2, loaded with the default (keep) policy;
                           // 0: streamed with evict-first loads
  double alpha_r, beta_r;  // Rayleigh coefficients
  double aM, aK, aC;       // A = aM M + aK K + aC Cabs
  double dt;
  double *u, *v, *a, *a1, *a2;
  double *q1, *q2, *y1, *x0, *x, *r, *z, *p, *w, *f;
  float* t32;
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

template <int D>
__device__ inline void warp_sum3(double* s) {
#pragma unroll
  for (int c = 0; c < D; ++c) s[c] = warp_sum(s[c]);
}

// (hi, lo) FP32 pair of a double: hi + lo reproduces x to 48 bits
__device__ inline float2 split_pair(double x) {
  const float hi = (float)x;
  return make_float2(hi, (float)(x - (double)hi));
}

// ------------------------------------------------------------------ per-step kernels
__global__ void k_force(Args g) {
  const int t = g.s->t;
  if (!g.f_ptr) return;
  if (t >= 0 && t < g.n_t)
    for (int64_t k = g.f_ptr[t] + threadIdx.x; k < g.f_ptr[t + 1]; k += blockDim.x) g.f[g.f_slot[k]] = 0.0;
  __syncthreads();
  const int t1 = t + 1;
  if (t1 >= 0 && t1 < g.n_t)
    for (int64_t k = g.f_ptr[t1] + threadIdx.x; k < g.f_ptr[t1 + 1]; k += blockDim.x)
      g.f[g.f_slot[k]] += g.f_val[k];
}

// Predictor vectors (slot space):
//   vp = v + dt/2 a, up = u + dt v + dt^2/4 a                  (Newmark predictors)
//   b = f - C vp - K up,  C = Cabs + alpha M + beta K
//     = f - K (up + beta vp) - M (alpha vp) - Cabs vp
//   x0 = warm start;  A x0 = aM M x0 + aK K x0 + aC Cabs x0
// stored: q1 = up + beta vp, q2 = alpha vp, y1 = vp, x0.
__global__ void k_predict(Args g) {
  const double dt = g.dt, h = 0.5 * dt, qq = 0.25 * dt * dt;
  const int hist = g.s->hist;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n_s; i += (int64_t)gridDim.x * blockDim.x) {
    const double ai = g.a[i], vi = g.v[i];
    const double vp = vi + h * ai;
    const double up = g.u[i] + dt * vi + qq * ai;
    g.q1[i] = up + g.beta_r * vp;
    g.q2[i] = g.alpha_r * vp;
    g.y1[i] = vp;
    double x0 = ai;
    if (hist >= 2) x0 = 3.0 * ai - 3.0 * g.a1[i] + g.a2[i];
    else if (hist == 1) x0 = 2.0 * ai - g.a1[i];
    if (g.fixed[i]) x0 = 0.0;
    g.x0[i] = x0;
    if (g.spmv_pair) g.p2[i] = split_pair(x0);  // p2 is scratch until p is first written
  }
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

// hi/lo accumulation of a * p in FP32-pair arithmetic (a = ah + al, p = p.x + p.y): the
// product's rounding error (fmaf) and the sum's (two-sum) go to lo; _rn intrinsics keep the
// compiler from contracting the error terms
__device__ __forceinline__ void pair_fma(float ah, float al, float2 pv, float& hi, float& lo) {
  const float pr = __fmul_rn(ah, pv.x);
  const float pe = fmaf(ah, pv.x, -pr);
  const float t = __fadd_rn(hi, pr);
  const float bp = __fsub_rn(t, hi);
  const float e2 = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, bp)), __fsub_rn(pr, bp));
  hi = t;
  lo += (pe + e2) + fmaf(ah, pv.y, al * pv.x);
}

// (hi, lo) += (h2, l2), the rounding error of the hi sum kept in lo
__device__ __forceinline__ void pair_add(float& hi, float& lo, float h2, float l2) {
  const float t = __fadd_rn(hi, h2);
  const float bp = __fsub_rn(t, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, bp)), __fsub_rn(h2, bp));
  hi = t;
  lo = __fadd_rn(__fadd_rn(lo, l2), e);
}

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

// r = b - A x0 with b = f - K q1 - M q2 - Cabs y1; bb = |b|^2.  x = x0.
template <int D, bool kPair>
__global__ void __launch_bounds__(kThreads) k_residual(Args g) {
  __shared__ double sh[32];
  double pbb = 0.0;
  SELL_ROW_LOOP(g.sf_ptr) {
    SELL_ROW_BEGIN(g.sf_ptr)
    double sb[D], sx[D];
    float xh[D], xl[D];
#pragma unroll
    for (int c = 0; c < D; ++c) {
      sb[c] = sx[c] = 0.0;
      xh[c] = xl[c] = 0.f;
    }
    for (int64_t q = 0; q < nq; ++q) {
      int cl[4];
      cols4(g.sf_col, p0 + 128 * q, cl, g.keep_l2);
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {  // two entries at a time (registers)
        const int64_t pos = p0 + 128 * q + 2 * hh;
        double qa[2][D], xa[2][D], q2a[2][D], m2[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int64_t bs = (int64_t)cl[2 * hh + e] * D;
#pragma unroll
          for (int d = 0; d < D; ++d) {
            qa[e][d] = g.q1[bs + d];
            q2a[e][d] = g.q2[bs + d];
            xa[e][d] = kPair ? 0.0 : g.x0[bs + d];
          }
        }
        ld2(g.MSS + pos, m2, g.keep_l2);
        if (kPair) {
          // b part in FP64 (elastic forces cancel); A x0 in FP32-pair arithmetic on the A planes
          float2 xp[2][D];
#pragma unroll
          for (int e = 0; e < 2; ++e)
#pragma unroll
            for (int d = 0; d < D; ++d) xp[e][d] = g.p2[(int64_t)cl[2 * hh + e] * D + d];
#pragma unroll
          for (int c = 0; c < D; ++c) {
            double sq = fma(m2[1], q2a[1][c], m2[0] * q2a[0][c]);
#pragma unroll
            for (int d = 0; d < D; ++d) {
              double k2[2];
              ld2(g.KS + (int64_t)(c * D + d) * g.sf_n + pos, k2, g.keep_l2);
              sq = fma(k2[1], qa[1][d], fma(k2[0], qa[0][d], sq));
            }
            sb[c] += sq;
#pragma unroll
            for (int d = 0; d < D; ++d) {
              float2 a2[2];
              ld2(g.APS + (int64_t)(c * D + d) * g.sf_n + pos, a2, g.keep_l2);
              pair_fma(a2[0].x, a2[0].y, xp[0][d], xh[c], xl[c]);
              pair_fma(a2[1].x, a2[1].y, xp[1][d], xh[c], xl[c]);
            }
          }
        } else {
#pragma unroll
          for (int c = 0; c < D; ++c) {
            double sq = fma(m2[1], q2a[1][c], m2[0] * q2a[0][c]), sxx = 0.0;
#pragma unroll
            for (int d = 0; d < D; ++d) {
              double k2[2];
              ld2(g.KS + (int64_t)(c * D + d) * g.sf_n + pos, k2, g.keep_l2);
              sq = fma(k2[1], qa[1][d], fma(k2[0], qa[0][d], sq));
              sxx = fma(k2[1], xa[1][d], fma(k2[0], xa[0][d], sxx));
            }
            sb[c] += sq;
            sx[c] = fma(g.aK, sxx, fma(g.aM * m2[1], xa[1][c], fma(g.aM * m2[0], xa[0][c], sx[c])));
          }
        }
      }
    }
    if (kPair) {
#pragma unroll
      for (int c = 0; c < D; ++c) sx[c] = (double)xh[c] + (double)xl[c];
    }
    if (row < g.n_nodes) {
#pragma unroll
      for (int c = 0; c < D; ++c) {
        const int64_t i = row * D + c;
        double bv = 0.0, rv = 0.0;
        if (!g.fixed[i]) {
          double cb = 0.0, cx = 0.0;  // Lysmer dashpots (boundary rows only)
          for (int64_t k = g.cab_ptr[i]; k < g.cab_ptr[i + 1]; ++k) {
            const int jj = g.cab_col[k];
            cb = fma(g.cab_val[k], g.y1[jj], cb);
            if (!kPair) cx = fma(g.cab_val[k], g.x0[jj], cx);
          }
          bv = g.f[i] - sb[c] - cb;
          // the A planes of the pair path already hold the dashpots (A = M + dt/2 C + dt^2/4 K)
          rv = kPair ? bv - sx[c] : bv - (sx[c] + g.aC * cx);
        }
        g.r[i] = rv;
        g.x[i] = g.x0[i];
        pbb += bv * bv;
      }
    }
  }
  const double t = block_sum(pbb, sh);
  if (threadIdx.x == 0) g.part[blockIdx.x * 4 + 2] = t;
  if (last_block(&g.s->ticket)) {
    const double bb = reduce_parts(g.part, 2, sh);
    if (threadIdx.x == 0) {
      g.s->bb = bb;
      g.s->it = 0;
      g.s->ticket = 0;
    }
  }
}

// t = G r  (lower pattern, FP32 factor, FP32 result)
template <int D>
__global__ void __launch_bounds__(kThreads) k_prec_lower(Args g) {
  SELL_ROW_LOOP(g.sl_ptr) {
    SELL_ROW_BEGIN(g.sl_ptr)
    float s[D];
#pragma unroll
    for (int c = 0; c < D; ++c) s[c] = 0.f;
    for (int64_t q = 0; q < nq; ++q) {
      const int64_t pos = p0 + 128 * q;
      int cl[4];
      cols4(g.sl_col, pos, cl, g.keep_l2);
      float ra[4][D];
#pragma unroll
      for (int e = 0; e < 4; ++e)
#pragma unroll
        for (int d = 0; d < D; ++d) ra[e][d] = (float)g.r[(int64_t)cl[e] * D + d];
#pragma unroll
      for (int c = 0; c < D; ++c)
#pragma unroll
        for (int d = 0; d < D; ++d) {
          float gv[4];
          ld4(g.GS + (int64_t)(c * D + d) * g.sl_n + pos, gv, g.keep_l2);
#pragma unroll
          for (int e = 0; e < 4; ++e) s[c] = fmaf(gv[e], ra[e][d], s[c]);
        }
    }
    if (row < g.n_nodes) {
#pragma unroll
      for (int c = 0; c < D; ++c) g.t32[row * D + c] = s[c];
    }
  }
}

// z = G^T t ; partial r.z ; mode 0 (inside PCG): last block computes beta, rz;
// mode 1 (after the residual): p = z, rz, rr and the conditional from |r| vs |b|.
template <int D, int kMode>
__global__ void __launch_bounds__(kThreads) k_prec_upper(Args g, int mode, cudaGraphConditionalHandle hc) {
  __shared__ double sh[32];
  double prz = 0.0, prr = 0.0;
  SELL_ROW_LOOP(g.su_ptr) {
    SELL_ROW_BEGIN(g.su_ptr)
    float s[D];
#pragma unroll
    for (int c = 0; c < D; ++c) s[c] = 0.f;
    for (int64_t q = 0; q < nq; ++q) {
      const int64_t pos = p0 + 128 * q;
      int cl[4];
      cols4(g.su_col, pos, cl, g.keep_l2);
      float ta[4][D];
#pragma unroll
      for (int e = 0; e < 4; ++e)
#pragma unroll
        for (int d = 0; d < D; ++d) ta[e][d] = g.t32[(int64_t)cl[e] * D + d];
#pragma unroll
      for (int c = 0; c < D; ++c)
#pragma unroll
        for (int d = 0; d < D; ++d) {
          float gv[4];
          ld4(g.GTS + (int64_t)(c * D + d) * g.su_n + pos, gv, g.keep_l2);
#pragma unroll
          for (int e = 0; e < 4; ++e) s[c] = fmaf(gv[e], ta[e][d], s[c]);
        }
    }
    if (row < g.n_nodes) {
#pragma unroll
      for (int c = 0; c < D; ++c) {
        const int64_t i = row * D + c;
        const double z = (double)s[c];
        const double r = g.r[i];
        g.z[i] = z;
        if (mode == 1) {
          g.p[i] = z;
          if (g.spmv_pair) g.p2[i] = split_pair(z);
        }
        prz += r * z;
        prr += r * r;
      }
    }
  }
  double t = block_sum(prz, sh);
  if (threadIdx.x == 0) g.part[blockIdx.x * 4 + 0] = t;
  if (mode == 1) {
    t = block_sum(prr, sh);
    if (threadIdx.x == 0) g.part[blockIdx.x * 4 + 1] = t;
  }
  if (last_block(&g.s->ticket)) {
    const double rz = reduce_parts(g.part, 0, sh);
    const double rr = mode == 1 ? reduce_parts(g.part, 1, sh) : 0.0;
    if (threadIdx.x == 0) {
      Scal* s = g.s;
      s->ticket = 0;
      if (mode == 1) {
        s->rz = rz;
        s->rr = rr;
        const bool done = rr <= s->tol2 * s->bb;
        pcg_continue<kMode>(hc, s, !done);
      } else {
        s->beta = s->rz != 0.0 ? rz / s->rz : 0.0;
        s->rz = rz;
      }
    }
  }
}

// z = G^T t only (no reductions, no graph conditional): used by sc_nb_apply
template <int D>
__global__ void __launch_bounds__(kThreads) k_prec_upper_nograph(Args g) {
  SELL_ROW_LOOP(g.su_ptr) {
    SELL_ROW_BEGIN(g.su_ptr)
    float s[D];
#pragma unroll
    for (int c = 0; c < D; ++c) s[c] = 0.f;
    for (int64_t q = 0; q < nq; ++q) {
      const int64_t pos = p0 + 128 * q;
      int cl[4];
      cols4(g.su_col, pos, cl, g.keep_l2);
#pragma unroll
      for (int c = 0; c < D; ++c)
#pragma unroll
        for (int d = 0; d < D; ++d) {
          float gv[4];
          ld4(g.GTS + (int64_t)(c * D + d) * g.su_n + pos, gv, g.keep_l2);
#pragma unroll
          for (int e = 0; e < 4; ++e) s[c] = fmaf(gv[e], g.t32[(int64_t)cl[e] * D + d], s[c]);
        }
    }
    if (row < g.n_nodes) {
#pragma unroll
      for (int c = 0; c < D; ++c) g.z[row * D + c] = (double)s[c];
    }
  }
}

// w = A p ; partial p.w ; last block: alpha
template <int D, int kMode>
__global__ void __launch_bounds__(kThreads) k_spmv(Args g, cudaGraphConditionalHandle hc) {
  __shared__ double sh[32];
  double ppw = 0.0;
  SELL_ROW_LOOP(g.sf_ptr) {
    SELL_ROW_BEGIN(g.sf_ptr)
    double s[D][D];
#pragma unroll
    for (int c = 0; c < D; ++c)
#pragma unroll
      for (int d = 0; d < D; ++d) s[c][d] = 0.0;
    for (int64_t q = 0; q < nq; ++q) {
      const int64_t pos = p0 + 128 * q;
      int cl[4];
      cols4(g.sf_col, pos, cl, g.keep_l2);
      double pa[4][D];
#pragma unroll
      for (int e = 0; e < 4; ++e)
#pragma unroll
        for (int d = 0; d < D; ++d) pa[e][d] = g.p[(int64_t)cl[e] * D + d];
#pragma unroll
      for (int c = 0; c < D; ++c)
#pragma unroll
        for (int d = 0; d < D; ++d) {
          double av[4];
          ld4(g.AS + (int64_t)(c * D + d) * g.sf_n + pos, av, g.keep_l2);
#pragma unroll
          for (int e = 0; e < 4; ++e) s[c][d] = fma(av[e], pa[e][d], s[c][d]);
        }
    }
    if (row < g.n_nodes) {
#pragma unroll
      for (int c = 0; c < D; ++c) {
        double wv = 0.0;
#pragma unroll
        for (int d = 0; d < D; ++d) wv += s[c][d];
        const int64_t i = row * D + c;
        g.w[i] = wv;
        ppw += g.p[i] * wv;
      }
    }
  }
  const double t = block_sum(ppw, sh);
  if (threadIdx.x == 0) g.part[blockIdx.x * 4 + 3] = t;
  if (last_block(&g.s->ticket)) {
    const double pw = reduce_parts(g.part, 3, sh);
    if (threadIdx.x == 0) {
      Scal* s = g.s;
      s->ticket = 0;
      s->pw = pw;
      if (kMode != 2) {
        if (!(pw > 0.0)) {
          s->alpha = 0.0;
          s->status = SC_BREAKDOWN;
          pcg_continue<kMode>(hc, s, false);
        } else {
          s->alpha = s->rz / pw;
        }
      }
    }
  }
}

// w = A p in FP32-pair arithmetic.  Each product A_cd p_d = (ah + al)(ph + pl) is formed as
// the exact FP32 product ah*ph (TwoProd through fmaf) plus the cross terms ah*pl + al*ph;
// the row sums are carried as an unevaluated (hi, lo) FP32 pair with TwoSum (Knuth) and
// converted to FP64 once per row.  Relative accuracy ~2^-46 per product, no FP64 pipe work
// in the block loop; same bytes as the FP64 kernel (A: 2 x 4 B per value, p: 8 B pairs).
template <int D, int kMode>
__global__ void __launch_bounds__(kThreads) k_spmv_pair(Args g, cudaGraphConditionalHandle hc) {
  __shared__ double sh[32];
  double ppw = 0.0;
  SELL_ROW_LOOP(g.sf_ptr) {
    SELL_ROW_BEGIN(g.sf_ptr)
    float hi[D], lo[D];
#pragma unroll
    for (int c = 0; c < D; ++c) hi[c] = lo[c] = 0.f;
    for (int64_t q = 0; q < nq; ++q) {
      const int64_t pos = p0 + 128 * q;
      int cl[4];
      cols4(g.sf_col, pos, cl, g.keep_l2);
      float2 pv[4][D];
#pragma unroll
      for (int e = 0; e < 4; ++e)
#pragma unroll
        for (int d = 0; d < D; ++d) pv[e][d] = g.p2[(int64_t)cl[e] * D + d];
#pragma unroll
      for (int c = 0; c < D; ++c)
#pragma unroll
        for (int d = 0; d < D; ++d) {
          float2 a4[4];
          ld4(g.APS + (int64_t)(c * D + d) * g.sf_n + pos, a4, g.keep_l2);
#pragma unroll
          for (int e = 0; e < 4; ++e) pair_fma(a4[e].x, a4[e].y, pv[e][d], hi[c], lo[c]);
        }
    }
    if (row < g.n_nodes) {
#pragma unroll
      for (int c = 0; c < D; ++c) {
        const double wv = (double)hi[c] + (double)lo[c];
        const int64_t i = row * D + c;
        g.w[i] = wv;
        ppw += g.p[i] * wv;
      }
    }
  }
  const double t = block_sum(ppw, sh);
  if (threadIdx.x == 0) g.part[blockIdx.x * 4 + 3] = t;
  if (last_block(&g.s->ticket)) {
    const double pw = reduce_parts(g.part, 3, sh);
    if (threadIdx.x == 0) {
      Scal* s = g.s;
      s->ticket = 0;
      s->pw = pw;
      if (kMode != 2) {
        if (!(pw > 0.0)) {
          s->alpha = 0.0;
          s->status = SC_BREAKDOWN;
          pcg_continue<kMode>(hc, s, false);
        } else {
          s->alpha = s->rz / pw;
        }
      }
    }
  }
}

// x += alpha p ; r -= alpha w ; partial r.r ; last block: convergence test
template <int kMode>
__global__ void k_update(Args g, cudaGraphConditionalHandle hc) {
  __shared__ double sh[32];
  const double alpha = g.s->alpha;
  double prr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n_s; i += (int64_t)gridDim.x * blockDim.x) {
    g.x[i] = fma(alpha, g.p[i], g.x[i]);
    const double r = fma(-alpha, g.w[i], g.r[i]);
    g.r[i] = r;
    prr += r * r;
  }
  const double t = block_sum(prr, sh);
  if (threadIdx.x == 0) g.part[blockIdx.x * 4 + 1] = t;
  if (last_block(&g.s->ticket)) {
    const double rr = reduce_parts(g.part, 1, sh);
    if (threadIdx.x == 0) {
      Scal* s = g.s;
      s->ticket = 0;
      s->rr = rr;
      s->it += 1;
      bool done = rr <= s->tol2 * s->bb;
      if (!done && s->it >= s->max_it) {
        if (!s->status) s->status = SC_NOT_CONVERGED;
        done = true;
      }
      if (s->status == SC_BREAKDOWN) done = true;
      if (done) pcg_continue<kMode>(hc, s, false);
    }
  }
}

__global__ void k_direction(Args g) {
  const double beta = g.s->beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n_s; i += (int64_t)gridDim.x * blockDim.x) {
    const double pv = fma(beta, g.p[i], g.z[i]);
    g.p[i] = pv;
    if (g.spmv_pair) g.p2[i] = split_pair(pv);
  }
}

// u = up + dt^2/4 x ; v = vp + dt/2 x ; shift the acceleration history ; record ; t += 1
__global__ void k_finalize(Args g) {
  const double dt = g.dt, h = 0.5 * dt, qq = 0.25 * dt * dt;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n_s; i += (int64_t)gridDim.x * blockDim.x) {
    const double x = g.x[i], ai = g.a[i], vi = g.v[i];
    const double up = g.u[i] + dt * vi + qq * ai;
    const double vp = vi + h * ai;
    g.u[i] = fma(qq, x, up);
    g.v[i] = fma(h, x, vp);
    g.a2[i] = g.a1[i];
    g.a1[i] = ai;
    g.a[i] = x;
  }
}

__global__ void k_record(Args g) {
  const int step = g.s->t + 1;
  if (g.n_rec > 0 && g.out_interval > 0 && step % g.out_interval == 0) {
    const int64_t row = step / g.out_interval;
    if (row < g.n_out)
      for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < g.n_rec;
           j += (int64_t)gridDim.x * blockDim.x) {
        const int e = g.rec_slot[j];
        if (g.out_u) g.out_u[row * g.n_rec + j] = g.u[e];
        if (g.out_v) g.out_v[row * g.n_rec + j] = g.v[e];
        if (g.out_a) g.out_a[row * g.n_rec + j] = g.a[e];
      }
  }
}

__global__ void k_advance(Args g) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    Scal* s = g.s;
    s->total_iters += s->it;
    if (s->it > s->max_seen) s->max_seen = s->it;
    s->t += 1;
    if (s->hist < 2) s->hist += 1;
  }
}

// ------------------------------------------------------------------ setup kernels
__device__ inline int64_t find_in(const int* adj, int64_t lo, int64_t hi, int key) {
  const int64_t end = hi;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (adj[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return (lo < end && adj[lo] == key) ? lo : -1;
}

__device__ inline double csr_value(const int64_t* rowptr, const int* cols, const double* val, int row, int col) {
  int64_t lo = rowptr[row], hi = rowptr[row + 1];
  const int64_t end = hi;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (cols[mid] < col) lo = mid + 1;
    else hi = mid;
  }
  return (lo < end && cols[lo] == col) ? val[lo] : 0.0;
}

// diag position and fixed-slot flags
__global__ void k_setup_nodes(int n_nodes, int D, const int* eqmap, const int64_t* adj_ptr, const int* adj,
                              int64_t* diag, int* fixed, int* bad) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n_nodes; a += gridDim.x * blockDim.x) {
    const int64_t k = find_in(adj, adj_ptr[a], adj_ptr[a + 1], a);
    if (k < 0) atomicExch(bad, 1);
    diag[a] = k < 0 ? adj_ptr[a] : k;
    for (int d = 0; d < D; ++d) fixed[(int64_t)a * D + d] = eqmap[(int64_t)a * D + d] < 0;
  }
}

// Gather eq-space CSR K, M, C into node blocks; A = M + (dt/2 C + dt^2/4 K) entry by entry
// (the same expression as the CSR solver); fixed slots get A = 1 on their diagonal.
template <int D>
__global__ void k_gather_blocks(Args g, const int* eqmap, const int64_t* rowptr, const int* cols, const double* K,
                                const double* M, const double* C, double* KB, double* AB, double* MS) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const double h = 0.5 * g.dt, qq = 0.25 * g.dt * g.dt;
  for (int64_t a = gw; a < g.n_nodes; a += nw) {
    for (int64_t k = g.adj_ptr[a] + lane; k < g.adj_ptr[a + 1]; k += 32) {
      const int b = g.adj[k];
      double m = 0.0;
      bool have_m = false;
      for (int c = 0; c < D; ++c)
        for (int d = 0; d < D; ++d) {
          const int ea = eqmap[a * D + c], eb = eqmap[(int64_t)b * D + d];
          double kv = 0.0, mv = 0.0, cv = 0.0;
          if (ea >= 0 && eb >= 0) {
            kv = csr_value(rowptr, cols, K, ea, eb);
            mv = csr_value(rowptr, cols, M, ea, eb);
            cv = csr_value(rowptr, cols, C, ea, eb);
            if (c == d && !have_m) {
              m = mv;
              have_m = true;
            }
          }
          double av = mv + (h * cv + qq * kv);
          if (ea < 0 && b == a && c == d) av = 1.0;
          KB[(int64_t)(c * D + d) * g.nnzb + k] = kv;
          AB[(int64_t)(c * D + d) * g.nnzb + k] = av;
        }
      MS[k] = m;
    }
  }
}

// FSAI row for slot i = (a, c): pattern S = free-or-fixed slots of the lower neighbours
// b < a (all d) then (a, d <= c); g = L^-T L^-1 e_last / sqrt(.) with A[S,S] = L L^T.
// One warp per block (the dense pattern matrix takes 32 KB of shared memory).  Rows whose
// pattern has more than kMaxFsai - 1 slots use a Jacobi row instead (counted).
template <int D>
__global__ void __launch_bounds__(32) k_fsai(Args g, float* GB, int* fallback, int jacobi_only) {
  __shared__ double Am[kMaxFsai * kMaxFsai];
  __shared__ int sl[kMaxFsai];
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = gw; i < g.n_s; i += nw) {
    const int64_t a = i / D;
    const int c = (int)(i - a * D);
    const int64_t k0 = g.adj_ptr[a], kd = g.diag[a];
    const int nlow = (int)(kd - k0);
    const int m = nlow * D + c + 1;
    const int64_t ga = a * D;
    if (g.fixed[i] || m > kMaxFsai - 1 || jacobi_only) {
      // identity row for fixed slots; Jacobi row when the pattern exceeds the capacity
      if (lane == 0) {
        const double aii = g.AB[(int64_t)(c * D + c) * g.nnzb + kd];
        GB[(int64_t)(c * D + c) * g.nnzb + kd] = (float)(g.fixed[i] ? 1.0 : 1.0 / sqrt(aii));
        if (!g.fixed[i] && !jacobi_only) atomicAdd(fallback, 1);
      }
      continue;
    }
    for (int p = lane; p < m; p += 32) {
      if (p < nlow * D) sl[p] = g.adj[k0 + p / D] * D + (p % D);
      else sl[p] = (int)(ga + (p - nlow * D));
    }
    __syncwarp();
    // lower triangle of A[S,S]
    for (int e = lane; e < m * m; e += 32) {
      const int pp = e / m, qq = e - pp * m;
      if (qq > pp) continue;
      const int sp = sl[pp], sq = sl[qq];
      const int bp = sp / D, dp = sp - bp * D, bq = sq / D, dq = sq - bq * D;
      double v = 0.0;
      const int64_t kk = (bp == bq) ? g.diag[bp] : find_in(g.adj, g.adj_ptr[bp], g.adj_ptr[bp + 1], bq);
      if (kk >= 0) v = g.AB[(int64_t)(dp * D + dq) * g.nnzb + kk];
      Am[pp * kMaxFsai + qq] = v;
    }
    __syncwarp();
    // Cholesky, right-looking, in place (lower)
    bool ok = true;
    for (int j = 0; j < m; ++j) {
      const double djj = Am[j * kMaxFsai + j];
      if (!(djj > 0.0)) {
        ok = false;
        break;
      }
      const double ljj = sqrt(djj);
      __syncwarp();
      if (lane == 0) Am[j * kMaxFsai + j] = ljj;
      for (int r = j + 1 + lane; r < m; r += 32) Am[r * kMaxFsai + j] /= ljj;
      __syncwarp();
      const int rem = m - j - 1;
      for (int e = lane; e < rem * rem; e += 32) {
        const int r = j + 1 + e / rem, q = j + 1 + (e - (e / rem) * rem);
        if (q <= r) Am[r * kMaxFsai + q] -= Am[r * kMaxFsai + j] * Am[q * kMaxFsai + j];
      }
      __syncwarp();
    }
    ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
    if (!ok) {
      if (lane == 0) {
        const double aii = g.AB[(int64_t)(c * D + c) * g.nnzb + kd];
        GB[(int64_t)(c * D + c) * g.nnzb + kd] = (float)(1.0 / sqrt(aii > 0 ? aii : 1.0));
        atomicAdd(fallback, 1);
      }
      __syncwarp();
      continue;
    }
    // y = L^-1 e_last = e_last / L_ll ; g = L^-T y, kept in the unused last row of Am
    // (m <= kMaxFsai - 1)
    double* gv = Am + (kMaxFsai - 1) * kMaxFsai;
    // backward substitution g_k = (y_k - sum_{j>k} L_jk g_j) / L_kk
    const double lll = Am[(m - 1) * kMaxFsai + (m - 1)];
    if (lane == 0) gv[m - 1] = 1.0 / (lll * lll);
    __syncwarp();
    for (int k = m - 2; k >= 0; --k) {
      double s = 0.0;
      for (int j = k + 1 + lane; j < m; j += 32) s += Am[j * kMaxFsai + k] * gv[j];
      s = warp_sum(s);
      if (lane == 0) gv[k] = -s / Am[k * kMaxFsai + k];
      __syncwarp();
    }
    const double scale = 1.0 / sqrt(gv[m - 1]);
    for (int p = lane; p < m; p += 32) {
      const float val = (float)(gv[p] * scale);
      int64_t kk;
      int d;
      if (p < nlow * D) {
        kk = k0 + p / D;
        d = p % D;
      } else {
        kk = kd;
        d = p - nlow * D;
      }
      GB[(int64_t)(c * D + d) * g.nnzb + kk] = val;
    }
    __syncwarp();
  }
}

// G^T on the upper part of each node row: GTB(a, b)[c][d] = GB(b, a)[d][c]
template <int D>
__global__ void k_transpose_g(Args g, const float* GB, float* GTB) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t a = gw; a < g.n_nodes; a += nw) {
    for (int64_t k = g.diag[a] + lane; k < g.adj_ptr[a + 1]; k += 32) {
      const int b = g.adj[k];
      const int64_t kk = (b == a) ? g.diag[a] : find_in(g.adj, g.adj_ptr[b], g.diag[b], (int)a);
      for (int c = 0; c < D; ++c)
        for (int d = 0; d < D; ++d)
          GTB[(int64_t)(c * D + d) * g.nnzb + k] = kk >= 0 ? GB[(int64_t)(d * D + c) * g.nnzb + kk] : 0.f;
    }
  }
}

// ------------------------------------------------------------------ explicit scheme
// Central difference with the row-sum lumped mass M_L (no counterpart in the reference, whose
// mass is always consistent):
//   a_n = M_L^-1 (f_n - K (u_n + beta v_{n-1/2}) - alpha M_L v_{n-1/2} - Cabs v_{n-1/2})
//   v_{n+1/2} = v_{n-1/2} + dt a_n ;  u_{n+1} = u_n + dt v_{n+1/2}
// Where a step also stores its new state (the adjoint's recompute): u, v of state k of the
// current segment go to u[k n_s ...], v[k n_s ...], k = state index - *t0.
struct StateStore {
  double *u, *v;
  const int* t0;
};

// One thread per node row over the sliced-ELL K; w = u + beta v and v are ping-ponged
// (neighbours read the previous step's values), u is updated in place (own row only).  kPair:
// K w in FP32-pair arithmetic on the K pair planes with w kept as (hi, lo) pairs (GB300's
// FP64 rate, not HBM, bounds the FP64 products); the update itself stays FP64.  The last
// block to finish advances the step counter and swaps the force entries in f from step t to
// step t + 1 (every block has read f by then).
template <int D, bool kPair, int TPR>
__global__ void __launch_bounds__(kThreads) k_explicit(Args g, const double* __restrict__ ML,
                                                       const double* __restrict__ IML,
                                                       const double* __restrict__ v_in, double* __restrict__ v_out,
                                                       const double* __restrict__ w_in, double* __restrict__ w_out,
                                                       const int* __restrict__ rec_map, StateStore store) {
  const float2* w2_in = reinterpret_cast<const float2*>(w_in);
  float2* w2_out = reinterpret_cast<float2*>(w_out);
  const int step = g.s->t + 1;
  const int64_t sk = store.u ? (int64_t)(step - *store.t0) * g.n_s : 0;
  const bool rec_now = g.n_rec > 0 && g.out_interval > 0 && (step % g.out_interval) == 0 &&
                       step / g.out_interval < g.n_out;
  const int64_t orow = rec_now ? step / g.out_interval : 0;
  const int sub = threadIdx.x % TPR;
  SELL_ROW_LOOP_T(TPR) {
    SELL_ROW_BEGIN(g.sf_ptr)
    double s[D][D];
    float hi[D], lo[D];
#pragma unroll
    for (int c = 0; c < D; ++c) {
      hi[c] = lo[c] = 0.f;
#pragma unroll
      for (int d = 0; d < D; ++d) s[c][d] = 0.0;
    }
    for (int64_t q = sub; q < nq; q += TPR) {
      const int64_t pos = p0 + 128 * q;
      int cl[4];
      cols4(g.sf_col, pos, cl, g.keep_l2);
      if constexpr (kPair) {
        float2 wa[4][D];
#pragma unroll
        for (int e = 0; e < 4; ++e)
#pragma unroll
          for (int d = 0; d < D; ++d) wa[e][d] = w2_in[(int64_t)cl[e] * D + d];
#pragma unroll
        for (int c = 0; c < D; ++c)
#pragma unroll
          for (int d = 0; d < D; ++d) {
            float2 k4[4];
            ld4(g.KPS + (int64_t)(c * D + d) * g.sf_n + pos, k4, g.keep_l2);
#pragma unroll
            for (int e = 0; e < 4; ++e) pair_fma(k4[e].x, k4[e].y, wa[e][d], hi[c], lo[c]);
          }
      } else {
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
            for (int e = 0; e < 4; ++e) s[c][d] = fma(kv[e], wa[e][d], s[c][d]);
          }
      }
    }
#pragma unroll
    for (int c = 0; c < D; ++c) {
      if (kPair) {
        group_pair_sum<TPR>(hi[c], lo[c]);
      } else {
#pragma unroll
        for (int d = 0; d < D; ++d) s[c][d] = group_sum<TPR>(s[c][d]);
      }
    }
    if (row < g.n_nodes) {
#pragma unroll
      for (int c = 0; c < D; ++c) {
        if (TPR > 1 && c % TPR != sub) continue;  // one lane per component
        const int64_t i = row * D + c;
        if (g.fixed[i]) {
          v_out[i] = 0.0;
          if (kPair) w2_out[i] = make_float2(0.f, 0.f);
          else w_out[i] = 0.0;
          if (store.u) store.u[sk + i] = store.v[sk + i] = 0.0;
          continue;
        }
        double kw = 0.0;
        if (kPair) {
          kw = (double)hi[c] + (double)lo[c];
        } else {
#pragma unroll
          for (int d = 0; d < D; ++d) kw += s[c][d];
        }
        double cab = 0.0;
        for (int64_t k = g.cab_ptr[i]; k < g.cab_ptr[i + 1]; ++k) cab = fma(g.cab_val[k], v_in[g.cab_col[k]], cab);
        const double vi = v_in[i], ml = ML[i];
        const double acc = (g.f[i] - kw - g.alpha_r * ml * vi - cab) * IML[i];
        const double vn = fma(g.dt, acc, vi);
        const double un = fma(g.dt, vn, g.u[i]);
        v_out[i] = vn;
        g.u[i] = un;
        if (kPair) w2_out[i] = split_pair(fma(g.beta_r, vn, un));
        else w_out[i] = fma(g.beta_r, vn, un);
        if (store.u) {
          store.u[sk + i] = un;
          store.v[sk + i] = vn;
        }
        if (rec_now) {
          const int rj = rec_map[i];
          if (rj >= 0) {
            if (g.out_u) g.out_u[orow * g.n_rec + rj] = un;
            if (g.out_v) g.out_v[orow * g.n_rec + rj] = vn;
          }
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
      if (t + 1 >= 0 && t + 1 < g.n_t)
        for (int64_t k = g.f_ptr[t + 1] + threadIdx.x; k < g.f_ptr[t + 2]; k += blockDim.x) g.f[g.f_slot[k]] += g.f_val[k];
    }
    if (threadIdx.x == 0) {
      g.s->ticket = 0;
      g.s->t = step;
    }
  }
}

// f = entries of step s->t (f zeroed beforehand)
__global__ void k_force_explicit0(Args g) {
  const int t = g.s->t;
  if (!g.f_ptr || t < 0 || t >= g.n_t) return;
  for (int64_t k = g.f_ptr[t] + threadIdx.x; k < g.f_ptr[t + 1]; k += blockDim.x) g.f[g.f_slot[k]] += g.f_val[k];
}

// f holds the entries of step t (= s->t); clear those of t-1
__global__ void k_force_explicit(Args g) {
  const int t = g.s->t;
  if (!g.f_ptr) return;
  const int t0 = t - 1;
  if (t0 >= 0 && t0 < g.n_t)
    for (int64_t k = g.f_ptr[t0] + threadIdx.x; k < g.f_ptr[t0 + 1]; k += blockDim.x) g.f[g.f_slot[k]] = 0.0;
  __syncthreads();
  if (t >= 0 && t < g.n_t)
    for (int64_t k = g.f_ptr[t] + threadIdx.x; k < g.f_ptr[t + 1]; k += blockDim.x) g.f[g.f_slot[k]] += g.f_val[k];
}

// row-sum lumped mass over free columns, and w = u + beta v
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

__global__ void k_w_init(Args g, double* w, int pair) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n_s; i += (int64_t)gridDim.x * blockDim.x) {
    const double x = fma(g.beta_r, g.v[i], g.u[i]);
    if (pair) reinterpret_cast<float2*>(w)[i] = split_pair(x);
    else w[i] = x;
  }
}

__global__ void k_reciprocal(int64_t n, const double* __restrict__ x, double* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = 1.0 / x[i];
}

__global__ void k_rec_map(Args g, int* map) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n_s; i += (int64_t)gridDim.x * blockDim.x)
    map[i] = -1;
}
__global__ void k_rec_map_fill(Args g, int* map) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < g.n_rec; j += (int64_t)gridDim.x * blockDim.x)
    map[g.rec_slot[j]] = (int)j;
}

// ------------------------------------------------------------------ sliced-ELL construction
// kind 0: full row [adj_ptr[a], adj_ptr[a+1]); 1: lower [adj_ptr[a], diag[a]]; 2: upper [diag[a], adj_ptr[a+1])
__device__ inline void row_range(int kind, const int64_t* adj_ptr, const int64_t* diag, int64_t a, int64_t& b,
                                 int64_t& e) {
  if (kind == 0) { b = adj_ptr[a]; e = adj_ptr[a + 1]; }
  else if (kind == 1) { b = adj_ptr[a]; e = diag[a] + 1; }
  else { b = diag[a]; e = adj_ptr[a + 1]; }
}

__global__ void k_sell_width(int kind, int n_nodes, int64_t n_slices, const int64_t* adj_ptr, const int64_t* diag,
                             int64_t* slen) {
  for (int64_t sl = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; sl < n_slices;
       sl += (int64_t)gridDim.x * blockDim.x) {
    int64_t w = 0;
    for (int l = 0; l < 32; ++l) {
      const int64_t a = sl * 32 + l;
      if (a >= n_nodes) break;
      int64_t b, e;
      row_range(kind, adj_ptr, diag, a, b, e);
      if (e - b > w) w = e - b;
    }
    slen[sl] = 32 * ((w + 3) & ~(int64_t)3);
  }
}

__global__ void k_sell_fill(int kind, int n_nodes, int64_t n_slices, const int64_t* adj_ptr, const int64_t* diag,
                            const int* adj, const int64_t* sptr, int* col, int64_t* src) {
  for (int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; a < n_slices * 32;
       a += (int64_t)gridDim.x * blockDim.x) {
    const int64_t sl = a >> 5, l = a & 31;
    const int64_t W = (sptr[sl + 1] - sptr[sl]) >> 5;
    int64_t b = 0, e = 0;
    if (a < n_nodes) row_range(kind, adj_ptr, diag, a, b, e);
    for (int64_t j = 0; j < W; ++j) {
      const int64_t pos = sptr[sl] + 128 * (j >> 2) + 4 * l + (j & 3);
      if (j < e - b) {
        col[pos] = adj[b + j];
        src[pos] = b + j;
      } else {
        col[pos] = a < n_nodes ? (int)a : 0;
        src[pos] = -1;
      }
    }
  }
}

template <typename T>
__global__ void k_sell_permute(int planes, int64_t n_out, int64_t n_in, const int64_t* src, const T* in, T* out) {
  for (int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pos < n_out;
       pos += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = src[pos];
    for (int c = 0; c < planes; ++c) out[(int64_t)c * n_out + pos] = k >= 0 ? in[(int64_t)c * n_in + k] : T(0);
  }
}

__global__ void k_init_scal(Scal* s, double tol2, int max_it) {
  s->rz = s->pw = s->rr = s->bb = s->alpha = s->beta = 0.0;
  s->tol2 = tol2;
  s->total_iters = 0;
  s->it = 0;
  s->max_it = max_it;
  s->max_seen = 0;
  s->status = SC_OK;
  s->t = 0;
  s->fsai_fallback = 0;
  s->ticket = 0;
  s->hist = 0;
}

__global__ void k_set_t(Scal* s, int t) { s->t = t; }

}  // namespace nb
}  // namespace sc

using namespace sc;
using namespace sc::nb;

struct sc_nb_newmark {
  Args g;
  void* sell_mem[16] = {};
  int n_sell_mem = 0;
  // explicit scheme state (allocated on first use)
  double *ML = nullptr, *IML = nullptr, *v1 = nullptr, *w0 = nullptr, *w1 = nullptr;
  float2* KPS = nullptr;
  int explicit_pair = 1;  // K w of the explicit step and the adjoint in FP32-pair arithmetic
  float adj_ms[3] = {0.f, 0.f, 0.f};  // last sc_nb_adjoint: forward, recompute, backward (device time)
  int* rec_map = nullptr;
  cudaGraphExec_t ex_exec[2] = {nullptr, nullptr};
  cudaGraph_t ex_graph[2] = {nullptr, nullptr};
  cudaStream_t user = nullptr, cap = nullptr, cap2 = nullptr;
  unsigned node_blocks = 1, vec_blocks = 1;
  // threads per node row of the explicit step and the adjoint rows (more on small meshes, so
  // the SMs have enough warps to cover load latency) and their grid
  int tpr = 1;
  unsigned tpr_blocks = 1;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

unsigned node_grid(int64_t n_nodes) {
  // per-step block kernels: one thread per node row, 256 threads per block
  int64_t b = (n_nodes + 255) / 256;
  const int64_t cap = 152 * 16;
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

template <int D>
int build_graph(sc_nb_newmark* h) {
  cudaGraph_t graph = nullptr;
  int rc = check(cudaGraphCreate(&graph, 0), "graph create");
  if (rc) return rc;
  cudaGraphConditionalHandle hc;
  if ((rc = check(cudaGraphConditionalHandleCreate(&hc, graph, 1, cudaGraphCondAssignDefault), "handle"))) {
    cudaGraphDestroy(graph);
    return rc;
  }
  Args g = h->g;
  cudaStream_t cs = h->cap, c2 = h->cap2;
  const unsigned nbk = h->node_blocks, vbk = h->vec_blocks;
  do {
    if ((rc = check(cudaStreamBeginCaptureToGraph(cs, graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
                    "capture")))
      break;
    k_force<<<1, 256, 0, cs>>>(g);
    k_predict<<<vbk, 256, 0, cs>>>(g);
    if (g.spmv_pair) k_residual<D, true><<<nbk, kThreads, 0, cs>>>(g);
    else k_residual<D, false><<<nbk, kThreads, 0, cs>>>(g);
    k_prec_lower<D><<<nbk, kThreads, 0, cs>>>(g);
    k_prec_upper<D, 0><<<nbk, kThreads, 0, cs>>>(g, 1, hc);
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
    if ((rc = check(cudaStreamBeginCaptureToGraph(c2, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
                    "capture body")))
      break;
    if (g.spmv_pair) k_spmv_pair<D, 0><<<nbk, kThreads, 0, c2>>>(g, hc);
    else k_spmv<D, 0><<<nbk, kThreads, 0, c2>>>(g, hc);
    k_update<0><<<vbk, 256, 0, c2>>>(g, hc);
    k_prec_lower<D><<<nbk, kThreads, 0, c2>>>(g);
    k_prec_upper<D, 0><<<nbk, kThreads, 0, c2>>>(g, 0, hc);
    k_direction<<<vbk, 256, 0, c2>>>(g);
    cudaGraph_t bo;
    if ((rc = check(cudaStreamEndCapture(c2, &bo), "end body"))) break;
    k_finalize<<<vbk, 256, 0, cs>>>(g);
    k_record<<<vbk, 256, 0, cs>>>(g);
    k_advance<<<1, 32, 0, cs>>>(g);
    cudaGraph_t out;
    if ((rc = check(cudaStreamEndCapture(cs, &out), "end capture"))) break;
    if ((rc = check(cudaGraphInstantiate(&h->exec, graph, 0), "instantiate"))) break;
  } while (0);
  if (rc) {
    cudaStreamCaptureStatus st;
    cudaGraph_t tmp;
    if (cudaStreamIsCapturing(cs, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) cudaStreamEndCapture(cs, &tmp);
    if (cudaStreamIsCapturing(c2, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) cudaStreamEndCapture(c2, &tmp);
    cudaGetLastError();
    cudaGraphDestroy(graph);
    return rc;
  }
  h->graph = graph;
  return SC_OK;
}

}  // namespace
static void drop_explicit_graphs(sc_nb_newmark* h);
namespace {

void drop_graph(sc_nb_newmark* h) {
  if (h->exec) cudaGraphExecDestroy(h->exec), h->exec = nullptr;
  if (h->graph) cudaGraphDestroy(h->graph), h->graph = nullptr;
}

}  // namespace

__global__ void k_split_pairs(int64_t n, const double* __restrict__ x, float2* __restrict__ hl) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float h = (float)x[i];
    hl[i] = make_float2(h, (float)(x[i] - (double)h));
  }
}

// Sliced-ELL copies of K, A, M (full pattern), G (lower) and G^T (upper) for the per-step
// kernels; allocated here (setup) from the stream-ordered pool and freed by sc_nb_destroy.
static int build_sell(sc_nb_newmark* h, const double* KB, const double* AB, const double* MS, const float* GB,
                      const float* GTB) {
  Args& g = h->g;
  cudaStream_t st = h->user;
  const int D2 = g.D * g.D;
  g.n_slices = ((int64_t)g.n_nodes + 31) / 32;
  int rc = SC_OK;
  auto alloc = [&](void** p, size_t bytes) {
    int r = check(cudaMallocAsync(p, bytes > 0 ? bytes : 8, st), "sell malloc");
    if (!r) h->sell_mem[h->n_sell_mem++] = *p;
    return r;
  };
  int64_t* scan_work = nullptr;
  int64_t* src = nullptr;
  const int64_t nsl = g.n_slices;
  if ((rc = check(cudaMallocAsync((void**)&scan_work, 8 * sc_scan_work_size(nsl), st), "malloc"))) return rc;
  for (int kind = 0; kind < 3 && !rc; ++kind) {
    int64_t* ptr = nullptr;
    if ((rc = alloc((void**)&ptr, 8 * (nsl + 1)))) break;
    k_sell_width<<<grid_for(nsl, 128), 128, 0, st>>>(kind, g.n_nodes, nsl, g.adj_ptr, g.diag, ptr);
    if ((rc = sc_exclusive_scan_i64(nsl, ptr, ptr, scan_work, st))) break;
    int64_t total = 0;
    if ((rc = check(cudaMemcpyAsync(&total, ptr + nsl, 8, cudaMemcpyDeviceToHost, st), "memcpy"))) break;
    if ((rc = check(cudaStreamSynchronize(st), "sync"))) break;
    int* col = nullptr;
    if ((rc = alloc((void**)&col, 4 * total))) break;
    if ((rc = check(cudaMallocAsync((void**)&src, 8 * (total > 0 ? total : 1), st), "malloc"))) break;
    k_sell_fill<<<grid_for(nsl * 32, 128), 128, 0, st>>>(kind, g.n_nodes, nsl, g.adj_ptr, g.diag, g.adj, ptr, col,
                                                        src);
    const unsigned pb = grid_for(total, 256, 152 * 32);
    if (kind == 0) {
      double *ks = nullptr, *as = nullptr, *ms = nullptr;
      if ((rc = alloc((void**)&ks, 8 * D2 * total))) break;
      if ((rc = alloc((void**)&as, 8 * D2 * total))) break;
      if ((rc = alloc((void**)&ms, 8 * total))) break;
      k_sell_permute<double><<<pb, 256, 0, st>>>(D2, total, g.nnzb, src, KB, ks);
      k_sell_permute<double><<<pb, 256, 0, st>>>(D2, total, g.nnzb, src, AB, as);
      k_sell_permute<double><<<pb, 256, 0, st>>>(1, total, g.nnzb, src, MS, ms);
      float2* ap = nullptr;
      if ((rc = alloc((void**)&ap, 8 * D2 * total))) break;
      k_split_pairs<<<pb, 256, 0, st>>>((int64_t)D2 * total, as, ap);
      g.sf_ptr = ptr; g.sf_col = col; g.sf_n = total; g.KS = ks; g.AS = as; g.MSS = ms;
      g.APS = ap;
    } else {
      float* gs = nullptr;
      if ((rc = alloc((void**)&gs, 4 * D2 * total))) break;
      k_sell_permute<float><<<pb, 256, 0, st>>>(D2, total, g.nnzb, src, kind == 1 ? GB : GTB, gs);
      if (kind == 1) { g.sl_ptr = ptr; g.sl_col = col; g.sl_n = total; g.GS = gs; }
      else { g.su_ptr = ptr; g.su_col = col; g.su_n = total; g.GTS = gs; }
    }
    rc = check_launch("sell build");
    cudaFreeAsync(src, st);
    src = nullptr;
  }
  if (src) cudaFreeAsync(src, st);
  cudaFreeAsync(scan_work, st);
  if (!rc) rc = check(cudaStreamSynchronize(st), "sync sell");
  if (!rc) {
    // one pass over a full-pattern plane set (K or A, FP64 or pairs, plus columns): keep it in
    // L2 across steps when it fits in three quarters of it, else stream it past L2
    int dev = 0, l2 = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) == cudaSuccess)
      g.keep_l2 = g.sf_n * (8 * D2 + 4 + 8) < (int64_t)l2 * 3 / 4 ? 1 : 0;
    cudaGetLastError();
  }
  return rc;
}

// Workspace layout (bytes, 256-aligned pieces), see sc_nb_workspace_bytes.
static int64_t align256(int64_t x) { return (x + 255) & ~(int64_t)255; }

extern "C" int64_t sc_nb_workspace_bytes(int n_nodes, int dim, int64_t nnzb) {
  const int64_t ns = (int64_t)n_nodes * dim, D2 = (int64_t)dim * dim;
  int64_t b = 0;
  b += align256(8 * n_nodes);                 // diag
  b += align256(4 * ns);                      // fixed
  b += 2 * align256(8 * D2 * nnzb);           // KB, AB
  b += align256(8 * nnzb);                    // MS
  b += 2 * align256(4 * D2 * nnzb);           // GB, GTB
  b += 13 * align256(8 * ns);                 // a1 a2 q1 q2 y1 x0 x r z p w f (+1 spare)
  b += align256(4 * ns);                      // t32
  b += align256(8 * 4 * 152 * 16);            // partials
  b += align256(sizeof(Scal));
  return b;
}

extern "C" int sc_nb_create(sc_nb_newmark** out, int n_nodes, int dim, const int* eqmap, const int64_t* adj_ptr,
                            const int* adj, int64_t nnzb, const int64_t* rowptr, const int* cols, const double* K,
                            const double* M, const double* C, int64_t n_cab, const int64_t* cab_ptr,
                            const int* cab_col, const double* cab_val, double alpha, double beta, double dt,
                            double rtol, int max_iter, int precond, double* u, double* v, double* a,
                            void* workspace, int64_t workspace_bytes, void* stream) {
  if (!out || n_nodes <= 0 || (dim != 2 && dim != 3) || !eqmap || !adj_ptr || !adj || nnzb <= 0 || !rowptr ||
      !cols || !K || !M || !C || !cab_ptr || !u || !v || !a || !workspace)
    return SC_BAD_ARG;
  if (n_cab > 0 && (!cab_col || !cab_val)) return SC_BAD_ARG;
  if (!(dt > 0) || !(rtol > 0) || max_iter <= 0) return SC_BAD_ARG;
  if (workspace_bytes < sc_nb_workspace_bytes(n_nodes, dim, nnzb)) return SC_BAD_ARG;
  if (((uintptr_t)workspace & 255) != 0) return SC_BAD_ARG;
  sc_nb_newmark* h = new sc_nb_newmark();
  h->user = (cudaStream_t)stream;
  Args& g = h->g;
  g = Args{};
  const int64_t ns = (int64_t)n_nodes * dim, D2 = (int64_t)dim * dim;
  g.n_nodes = n_nodes;
  g.D = dim;
  g.n_s = ns;
  g.nnzb = nnzb;
  g.adj_ptr = adj_ptr;
  g.adj = adj;
  g.cab_ptr = cab_ptr;
  g.cab_col = cab_col;
  g.cab_val = cab_val;
  g.alpha_r = alpha;
  g.beta_r = beta;
  g.aM = 1.0 + alpha * 0.5 * dt;
  g.aK = beta * 0.5 * dt + 0.25 * dt * dt;
  g.aC = 0.5 * dt;
  g.dt = dt;
  g.u = u;
  g.v = v;
  g.a = a;
  char* p = (char*)workspace;
  auto take = [&](int64_t bytes) {
    char* q = p;
    p += align256(bytes);
    return (void*)q;
  };
  int64_t* diag = (int64_t*)take(8 * n_nodes);
  int* fixed = (int*)take(4 * ns);
  double* KB = (double*)take(8 * D2 * nnzb);
  double* AB = (double*)take(8 * D2 * nnzb);
  double* MS = (double*)take(8 * nnzb);
  float* GB = (float*)take(4 * D2 * nnzb);
  float* GTB = (float*)take(4 * D2 * nnzb);
  g.diag = diag;
  g.fixed = fixed;
  g.KB = KB;
  g.AB = AB;
  g.MS = MS;
  g.GB = GB;
  g.GTB = GTB;
  g.a1 = (double*)take(8 * ns);
  g.a2 = (double*)take(8 * ns);
  g.q1 = (double*)take(8 * ns);
  g.q2 = (double*)take(8 * ns);
  g.y1 = (double*)take(8 * ns);
  g.x0 = (double*)take(8 * ns);
  g.x = (double*)take(8 * ns);
  g.r = (double*)take(8 * ns);
  g.z = (double*)take(8 * ns);
  g.p = (double*)take(8 * ns);
  g.w = (double*)take(8 * ns);
  g.f = (double*)take(8 * ns);
  g.p2 = (float2*)take(8 * ns);
  g.spmv_pair = 1;
  g.t32 = (float*)take(4 * ns);
  g.part = (double*)take(8 * 4 * 152 * 16);
  g.s = (Scal*)take(sizeof(Scal));
  h->node_blocks = node_grid(n_nodes);
  h->tpr = n_nodes >= 150000 ? 1 : (n_nodes >= 60000 ? 2 : 4);
  {
    const int64_t want = (((int64_t)n_nodes + 31) / 32 * 32 * h->tpr + kThreads - 1) / kThreads;
    h->tpr_blocks = (unsigned)(want < 152 * 16 ? (want < 1 ? 1 : want) : 152 * 16);
  }
  h->vec_blocks = grid_for(ns, 256, 152 * 16);
  cudaStream_t st = h->user;
  int rc = SC_OK;
  int* dflag = nullptr;
  do {
    if ((rc = check(cudaStreamCreateWithFlags(&h->cap, cudaStreamNonBlocking), "stream"))) break;
    if ((rc = check(cudaStreamCreateWithFlags(&h->cap2, cudaStreamNonBlocking), "stream"))) break;
    if ((rc = check(cudaMallocAsync((void**)&dflag, 2 * sizeof(int), st), "malloc"))) break;
    cudaMemsetAsync(dflag, 0, 2 * sizeof(int), st);
    cudaMemsetAsync(g.f, 0, 8 * ns, st);
    cudaMemsetAsync(g.a1, 0, 8 * ns, st);
    cudaMemsetAsync(g.a2, 0, 8 * ns, st);
    cudaMemsetAsync(GB, 0, 4 * D2 * nnzb, st);
    k_setup_nodes<<<grid_for(n_nodes, 128), 128, 0, st>>>(n_nodes, dim, eqmap, adj_ptr, adj, diag, fixed, dflag);
    if (dim == 3)
      k_gather_blocks<3><<<h->node_blocks, kThreads, 0, st>>>(g, eqmap, rowptr, cols, K, M, C, KB, AB, MS);
    else
      k_gather_blocks<2><<<h->node_blocks, kThreads, 0, st>>>(g, eqmap, rowptr, cols, K, M, C, KB, AB, MS);
    const unsigned fb = grid_for(ns, 1, 152 * 64);
    if (dim == 3) {
      k_fsai<3><<<fb, 32, 0, st>>>(g, GB, dflag + 1, precond == 1);
      k_transpose_g<3><<<h->node_blocks, kThreads, 0, st>>>(g, GB, GTB);
    } else {
      k_fsai<2><<<fb, 32, 0, st>>>(g, GB, dflag + 1, precond == 1);
      k_transpose_g<2><<<h->node_blocks, kThreads, 0, st>>>(g, GB, GTB);
    }
    k_init_scal<<<1, 1, 0, st>>>(g.s, rtol * rtol, max_iter);
    if ((rc = check_launch("nb setup"))) break;
    if ((rc = build_sell(h, KB, AB, MS, GB, GTB))) break;
    int hf[2] = {0, 0};
    if ((rc = check(cudaMemcpyAsync(hf, dflag, 2 * sizeof(int), cudaMemcpyDeviceToHost, st), "memcpy"))) break;
    if ((rc = check(cudaStreamSynchronize(st), "sync"))) break;
    if (hf[0]) rc = SC_BAD_ARG;  // a node missing from its own adjacency row
    int fallback = hf[1];
    cudaMemcpy(&g.s->fsai_fallback, &fallback, sizeof(int), cudaMemcpyHostToDevice);
  } while (0);
  if (dflag) {
    cudaFreeAsync(dflag, st);
    cudaStreamSynchronize(st);
  }
  if (rc) {
    cudaStreamSynchronize(st);
    for (int i = 0; i < h->n_sell_mem; ++i) cudaFree(h->sell_mem[i]);
    if (h->cap) cudaStreamDestroy(h->cap);
    if (h->cap2) cudaStreamDestroy(h->cap2);
    delete h;
    return rc;
  }
  *out = h;
  return SC_OK;
}

extern "C" int sc_nb_set_options(sc_nb_newmark* h, int options) {
  if (!h) return SC_BAD_ARG;
  h->g.spmv_pair = (options & 1) ? 0 : 1;
  h->explicit_pair = (options & 2) ? 0 : 1;
  drop_graph(h);
  drop_explicit_graphs(h);
  return SC_OK;
}

extern "C" int sc_nb_set_force(sc_nb_newmark* h, int n_t, const int64_t* f_ptr, const int* f_slot,
                               const double* f_val) {
  if (!h || n_t < 0 || (n_t > 0 && (!f_ptr || !f_slot || !f_val))) return SC_BAD_ARG;
  h->g.n_t = n_t;
  h->g.f_ptr = n_t > 0 ? f_ptr : nullptr;
  h->g.f_slot = f_slot;
  h->g.f_val = f_val;
  drop_graph(h);
  drop_explicit_graphs(h);
  // dense f holds the entries of the current step
  cudaMemsetAsync(h->g.f, 0, 8 * h->g.n_s, h->user);
  return SC_OK;
}

extern "C" int sc_nb_set_output(sc_nb_newmark* h, int out_interval, int n_rec, const int* rec_slot, double* out_u,
                                double* out_v, double* out_a, int64_t n_out) {
  if (!h || n_rec < 0 || (n_rec > 0 && (!rec_slot || out_interval <= 0 || n_out <= 0))) return SC_BAD_ARG;
  h->g.out_interval = out_interval;
  h->g.n_rec = n_rec;
  h->g.rec_slot = rec_slot;
  h->g.out_u = out_u;
  h->g.out_v = out_v;
  h->g.out_a = out_a;
  h->g.n_out = n_out;
  drop_graph(h);
  drop_explicit_graphs(h);
  return SC_OK;
}

// t_begin: state index of u/v/a on entry (the force entries of step t_begin are assumed in f
// when t_begin > 0; at t_begin == 0 they are written here).  The warm start uses the
// acceleration history (a1, a2) once steps of this solver have filled it.
// One step with eager launches (no graph): the same kernels, the PCG loop driven by the host
// reading Scal::done after each iteration.  Used for profiling (kernels inside graphs with
// conditional nodes cannot be captured by the profiler); selected by SCATTER_GB300_EAGER=1.
template <int D>
static int eager_step(sc_nb_newmark* h) {
  Args g = h->g;
  cudaStream_t st = h->user;
  const unsigned nbk = h->node_blocks, vbk = h->vec_blocks;
  cudaGraphConditionalHandle none = 0;
  k_force<<<1, 256, 0, st>>>(g);
  k_predict<<<vbk, 256, 0, st>>>(g);
  if (g.spmv_pair) k_residual<D, true><<<nbk, kThreads, 0, st>>>(g);
  else k_residual<D, false><<<nbk, kThreads, 0, st>>>(g);
  k_prec_lower<D><<<nbk, kThreads, 0, st>>>(g);
  k_prec_upper<D, 1><<<nbk, kThreads, 0, st>>>(g, 1, none);
  int done = 0;
  int rc;
  for (int guard = 0; guard < 100000; ++guard) {
    if ((rc = check(cudaMemcpyAsync(&done, &g.s->done, sizeof(int), cudaMemcpyDeviceToHost, st), "read done")))
      return rc;
    if ((rc = check(cudaStreamSynchronize(st), "sync eager"))) return rc;
    if (done) break;
    if (g.spmv_pair) k_spmv_pair<D, 1><<<nbk, kThreads, 0, st>>>(g, none);
    else k_spmv<D, 1><<<nbk, kThreads, 0, st>>>(g, none);
    k_update<1><<<vbk, 256, 0, st>>>(g, none);
    k_prec_lower<D><<<nbk, kThreads, 0, st>>>(g);
    k_prec_upper<D, 1><<<nbk, kThreads, 0, st>>>(g, 0, none);
    k_direction<<<vbk, 256, 0, st>>>(g);
  }
  k_finalize<<<vbk, 256, 0, st>>>(g);
  k_record<<<vbk, 256, 0, st>>>(g);
  k_advance<<<1, 32, 0, st>>>(g);
  return check_launch("eager step");
}

extern "C" int sc_nb_run(sc_nb_newmark* h, int t_begin, int t_end) {
  if (!h || t_begin < 0 || t_end < t_begin) return SC_BAD_ARG;
  int rc;
  const char* eager = getenv("SCATTER_GB300_EAGER");
  if (eager && eager[0] == '1') {
    cudaStream_t st = h->user;
    if (t_begin == 0 && h->g.f_ptr) {
      k_set_t<<<1, 1, 0, st>>>(h->g.s, -1);
      k_force<<<1, 256, 0, st>>>(h->g);
    }
    k_set_t<<<1, 1, 0, st>>>(h->g.s, t_begin);
    for (int t = t_begin; t < t_end; ++t)
      if ((rc = h->g.D == 3 ? eager_step<3>(h) : eager_step<2>(h))) return rc;
    return SC_OK;
  }
  if (!h->exec) {
    rc = h->g.D == 3 ? build_graph<3>(h) : build_graph<2>(h);
    if (rc) return rc;
  }
  cudaStream_t st = h->user;
  if (t_begin == 0 && h->g.f_ptr) {
    k_set_t<<<1, 1, 0, st>>>(h->g.s, -1);
    k_force<<<1, 256, 0, st>>>(h->g);  // step 0 entries
  }
  k_set_t<<<1, 1, 0, st>>>(h->g.s, t_begin);
  if ((rc = check_launch("nb run"))) return rc;
  for (int t = t_begin; t < t_end; ++t)
    if ((rc = check(cudaGraphLaunch(h->exec, st), "graph launch"))) return rc;
  return SC_OK;
}

static void drop_explicit_graphs(sc_nb_newmark* h) {
  for (int k = 0; k < 2; ++k) {
    if (h->ex_exec[k]) cudaGraphExecDestroy(h->ex_exec[k]), h->ex_exec[k] = nullptr;
    if (h->ex_graph[k]) cudaGraphDestroy(h->ex_graph[k]), h->ex_graph[k] = nullptr;
  }
}

template <int D, int TPR>
static void launch_explicit_t(const sc_nb_newmark* h, cudaStream_t st, const Args& g, const double* vin,
                              double* vout, const double* win, double* wout, StateStore store) {
  if (h->explicit_pair)
    k_explicit<D, true, TPR><<<h->tpr_blocks, kThreads, 0, st>>>(g, h->ML, h->IML, vin, vout, win, wout, h->rec_map,
                                                                 store);
  else
    k_explicit<D, false, TPR><<<h->tpr_blocks, kThreads, 0, st>>>(g, h->ML, h->IML, vin, vout, win, wout, h->rec_map,
                                                                  store);
}
template <int D>
static void launch_explicit(const sc_nb_newmark* h, cudaStream_t st, const Args& g, const double* vin, double* vout,
                            const double* win, double* wout, StateStore store) {
  switch (h->tpr) {
    case 4: launch_explicit_t<D, 4>(h, st, g, vin, vout, win, wout, store); break;
    case 2: launch_explicit_t<D, 2>(h, st, g, vin, vout, win, wout, store); break;
    default: launch_explicit_t<D, 1>(h, st, g, vin, vout, win, wout, store); break;
  }
}

template <int D>
static int build_explicit_graph(sc_nb_newmark* h, int k) {
  Args g = h->g;
  const double* vin = k == 0 ? g.v : h->v1;
  double* vout = k == 0 ? h->v1 : g.v;
  const double* win = k == 0 ? h->w0 : h->w1;
  double* wout = k == 0 ? h->w1 : h->w0;
  cudaStream_t cs = h->cap;
  int rc = check(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "capture explicit");
  if (rc) return rc;
  launch_explicit<D>(h, cs, g, vin, vout, win, wout, StateStore{});
  cudaGraph_t graph;
  if ((rc = check(cudaStreamEndCapture(cs, &graph), "end explicit"))) return rc;
  if ((rc = check(cudaGraphInstantiate(&h->ex_exec[k], graph, 0), "instantiate explicit"))) {
    cudaGraphDestroy(graph);
    return rc;
  }
  h->ex_graph[k] = graph;
  return SC_OK;
}

// Explicit central-difference steps t_begin .. t_end-1 on the same handle (u, v are the
// handle's state vectors; a is not used).  At t_begin == 0 the force entries of step 0 are
// written; the run always ends with the state in the caller's u and v.
extern "C" int sc_nb_explicit_run(sc_nb_newmark* h, int t_begin, int t_end) {
  if (!h || t_begin < 0 || t_end < t_begin) return SC_BAD_ARG;
  Args& g = h->g;
  cudaStream_t st = h->user;
  int rc;
  if (!h->ML) {
    const int64_t ns = g.n_s;
    if ((rc = check(cudaMallocAsync((void**)&h->ML, 8 * ns, st), "malloc"))) return rc;
    if ((rc = check(cudaMallocAsync((void**)&h->v1, 8 * ns, st), "malloc"))) return rc;
    if ((rc = check(cudaMallocAsync((void**)&h->w0, 8 * ns, st), "malloc"))) return rc;
    if ((rc = check(cudaMallocAsync((void**)&h->w1, 8 * ns, st), "malloc"))) return rc;
    if ((rc = check(cudaMallocAsync((void**)&h->rec_map, 4 * ns, st), "malloc"))) return rc;
    if ((rc = check(cudaMallocAsync((void**)&h->IML, 8 * ns, st), "malloc"))) return rc;
    k_lumped<<<grid_for(g.n_nodes, 256), 256, 0, st>>>(g, h->ML);
    k_reciprocal<<<grid_for(ns, 256), 256, 0, st>>>(ns, h->ML, h->IML);
  }
  if (h->explicit_pair && !h->KPS) {
    const int64_t n2 = (int64_t)g.D * g.D * g.sf_n;
    if ((rc = check(cudaMallocAsync((void**)&h->KPS, 8 * n2, st), "malloc"))) return rc;
    k_split_pairs<<<grid_for(n2, 256, 152 * 32), 256, 0, st>>>(n2, g.KS, h->KPS);
    g.KPS = h->KPS;
    drop_explicit_graphs(h);
  }
  if (!h->ex_exec[0]) {
    k_rec_map<<<grid_for(g.n_s, 256), 256, 0, st>>>(g, h->rec_map);
    if (g.n_rec > 0) k_rec_map_fill<<<grid_for(g.n_rec, 256), 256, 0, st>>>(g, h->rec_map);
    for (int k = 0; k < 2; ++k) {
      rc = g.D == 3 ? build_explicit_graph<3>(h, k) : build_explicit_graph<2>(h, k);
      if (rc) return rc;
    }
  }
  k_w_init<<<h->vec_blocks, 256, 0, st>>>(g, h->w0, h->explicit_pair);
  if (t_begin == 0 && g.f_ptr) {
    cudaMemsetAsync(g.f, 0, 8 * g.n_s, st);
    k_set_t<<<1, 1, 0, st>>>(g.s, 0);
    k_force_explicit<<<1, 256, 0, st>>>(g);  // step 0 entries
  }
  k_set_t<<<1, 1, 0, st>>>(g.s, t_begin);
  if ((rc = check_launch("explicit prepare"))) return rc;
  int k = 0;
  for (int t = t_begin; t < t_end; ++t, k ^= 1)
    if ((rc = check(cudaGraphLaunch(h->ex_exec[k], st), "explicit launch"))) return rc;
  if (k == 1) {  // state is in v1 / w1: bring v back to the caller's buffer
    if ((rc = check(cudaMemcpyAsync(g.v, h->v1, 8 * g.n_s, cudaMemcpyDeviceToDevice, st), "copy v"))) return rc;
  }
  return SC_OK;
}

extern "C" int sc_nb_time_explicit(sc_nb_newmark* h, int reps, float* ms_per_step) {
  if (!h || reps <= 0 || !ms_per_step || !h->ex_exec[0]) return SC_BAD_ARG;
  cudaStream_t st = h->user;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int t = 0;
  (void)t;
  cudaEventRecord(e0, st);
  for (int i = 0; i < reps; ++i) {
    const Args& g = h->g;
    if (g.D == 3) launch_explicit<3>(h, st, g, g.v, h->v1, h->w0, h->w1, StateStore{});
    else launch_explicit<2>(h, st, g, g.v, h->v1, h->w0, h->w1, StateStore{});
  }
  cudaEventRecord(e1, st);
  int rc = check_launch("explicit timing");
  if (!rc) rc = check(cudaEventSynchronize(e1), "sync");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  *ms_per_step = ms / reps;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

// ------------------------------------------------------------------ adjoint of the explicit scheme
// Discrete adjoint of sc_nb_explicit_run for the receiver-velocity misfit
//   J = 1/2 sum_{n=1..N} |P v_n - d_n|^2
// with respect to per-element E and rho (K = sum E_e K1_e + springs, M_L = sum rho_e ml1_e,
// Cab = sum sqrt(rho_e E_e) C1_f).  Forward with checkpoints every C steps, then per segment
// (last first) recompute the states and run the backward recursion (g = mu_v + dt mu_u,
// y = M_L^-1 g, mu_u -= dt K y, mu_v = g - dt (beta K y + Cab y + alpha M_L y) + P^T(P v_n - d_n))
// accumulating dJ/dE_e, dJ/drho_e element by element (deterministic, no atomics).
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
  const double *l_c, *l_s;
};
namespace {

struct AdjState {
  double *seg_u, *seg_v, *mu_u, *mu_v, *out_v, *gE, *gR;
  double* y[2];        // (mu_v + dt mu_u) / M_L of the step being reversed, and of the next one
  int *n_dev, *n_dev_e;  // step being reversed, one counter per backward kernel
  unsigned* ticket_e;  // finished blocks of the element kernel
  int *seg_t0, *rec_map;
  double* J;
  // FP32 inputs of the element kernel for the step being reversed ([cur]) and the next
  // ([cur ^ 1]): w = u + beta v as (hi, lo) pairs, v, a = (v_{n+1} - v_n) / dt, y
  float2* wp[2];
  float *v32[2], *a32[2], *y32[2];
};

__device__ __forceinline__ double y_at(const double* y, int64_t i, bool pair) {
  if (pair) {
    const float2 p = reinterpret_cast<const float2*>(y)[i];
    return (double)p.x + (double)p.y;
  }
  return y[i];
}

// FP32 element inputs of step n = *n_dev from the segment's FP64 states (k = n - t0)
__device__ __forceinline__ void adj_prep_slot(const Args& g, const AdjState& a, int buf, int64_t k, int64_t i,
                                              double y_i) {
  float2* wp = buf ? a.wp[1] : a.wp[0];
  float* v32 = buf ? a.v32[1] : a.v32[0];
  float* a32 = buf ? a.a32[1] : a.a32[0];
  float* y32 = buf ? a.y32[1] : a.y32[0];
  if (g.fixed[i]) {
    wp[i] = make_float2(0.f, 0.f);
    v32[i] = a32[i] = y32[i] = 0.f;
    return;
  }
  const double u0 = a.seg_u[k * g.n_s + i], v0 = a.seg_v[k * g.n_s + i], v1 = a.seg_v[(k + 1) * g.n_s + i];
  wp[i] = split_pair(fma(g.beta_r, v0, u0));
  v32[i] = (float)v0;
  a32[i] = (float)((v1 - v0) / g.dt);
  y32[i] = (float)y_i;
}

// Backward step n (state n -> n+1 reversed), node rows: with y = y[cur],
//   mu_u <- mu_u - dt K y,  mu_v <- g - dt (beta K y + Cab y + alpha M_L y) + P^T (P v_n - d_n),
//   y[cur ^ 1] = (mu_v + dt mu_u) / M_L   (the y of step n - 1).
// kPair: K y in FP32-pair arithmetic on the K pair planes, y kept as (hi, lo) pairs.
// The last block to finish decrements the row kernel's step counter.

template <int D, bool kPair, int TPR>
__global__ void __launch_bounds__(kThreads) k_adj_rows(Args g, const double* __restrict__ ML,
                                                       const double* __restrict__ IML, sc_adj_desc d, AdjState a,
                                                       int cur) {
  const int n = *a.n_dev;
  const int k = n - *a.seg_t0;
  const double* y = cur ? a.y[1] : a.y[0];  // (a select: no local copy of the parameter)
  double* yn = cur ? a.y[0] : a.y[1];
  const float2* y2 = reinterpret_cast<const float2*>(y);
  const int sub = threadIdx.x % TPR;
  SELL_ROW_LOOP_T(TPR) {
    SELL_ROW_BEGIN(g.sf_ptr)
    double s[D];
    float hi[D], lo[D];
#pragma unroll
    for (int c = 0; c < D; ++c) {
      s[c] = 0.0;
      hi[c] = lo[c] = 0.f;
    }
    for (int64_t q = sub; q < nq; q += TPR) {
      const int64_t pos = p0 + 128 * q;
      int cl[4];
      cols4(g.sf_col, pos, cl, g.keep_l2);
      if constexpr (kPair) {
        float2 ya[4][D];
#pragma unroll
        for (int e = 0; e < 4; ++e)
#pragma unroll
          for (int dd = 0; dd < D; ++dd) ya[e][dd] = y2[(int64_t)cl[e] * D + dd];
#pragma unroll
        for (int c = 0; c < D; ++c)
#pragma unroll
          for (int dd = 0; dd < D; ++dd) {
            float2 k4[4];
            ld4(g.KPS + (int64_t)(c * D + dd) * g.sf_n + pos, k4, g.keep_l2);
#pragma unroll
            for (int e = 0; e < 4; ++e) pair_fma(k4[e].x, k4[e].y, ya[e][dd], hi[c], lo[c]);
          }
      } else {
        double ya[4][D];
#pragma unroll
        for (int e = 0; e < 4; ++e)
#pragma unroll
          for (int dd = 0; dd < D; ++dd) ya[e][dd] = y[(int64_t)cl[e] * D + dd];
#pragma unroll
        for (int c = 0; c < D; ++c)
#pragma unroll
          for (int dd = 0; dd < D; ++dd) {
            double kv[4];
            ld4(g.KS + (int64_t)(c * D + dd) * g.sf_n + pos, kv, g.keep_l2);
#pragma unroll
            for (int e = 0; e < 4; ++e) s[c] = fma(kv[e], ya[e][dd], s[c]);
          }
      }
    }
#pragma unroll
    for (int c = 0; c < D; ++c) {
      if (kPair) group_pair_sum<TPR>(hi[c], lo[c]);
      else s[c] = group_sum<TPR>(s[c]);
    }
    if (row < g.n_nodes) {
#pragma unroll
      for (int c = 0; c < D; ++c) {
        if (TPR > 1 && c % TPR != sub) continue;  // one lane per component
        const int64_t i = row * D + c;
        if (g.fixed[i]) {
          a.mu_u[i] = a.mu_v[i] = 0.0;
          if (kPair) reinterpret_cast<float2*>(yn)[i] = make_float2(0.f, 0.f);
          else yn[i] = 0.0;
          if (k >= 1) adj_prep_slot(g, a, cur ^ 1, k - 1, i, 0.0);
          continue;
        }
        const double ky = kPair ? (double)hi[c] + (double)lo[c] : s[c];
        double cy = 0.0;
        for (int64_t q = g.cab_ptr[i]; q < g.cab_ptr[i + 1]; ++q) cy = fma(g.cab_val[q], y_at(y, g.cab_col[q], kPair), cy);
        const double yi = y_at(y, i, kPair);
        const double gg = fma(g.dt, a.mu_u[i], a.mu_v[i]);
        const double mu = fma(-g.dt, ky, a.mu_u[i]);
        double mv = gg - g.dt * (g.beta_r * ky + cy + g.alpha_r * ML[i] * yi);
        const int rj = a.rec_map[i];
        if (rj >= 0 && n >= 1) mv += a.seg_v[(int64_t)k * g.n_s + i] - d.target[(int64_t)n * d.n_rec + rj];
        a.mu_u[i] = mu;
        a.mu_v[i] = mv;
        const double ynext = fma(g.dt, mu, mv) * IML[i];
        if (kPair) reinterpret_cast<float2*>(yn)[i] = split_pair(ynext);
        else yn[i] = ynext;
        // the element kernel's FP32 inputs of step n - 1 when its state is in this segment
        // (the first step reversed in a segment gets them from k_adj_prep)
        if (k >= 1) adj_prep_slot(g, a, cur ^ 1, k - 1, i, ynext);
      }
    }
  }
  if (last_block(&g.s->ticket)) {
    if (threadIdx.x == 0) {
      g.s->ticket = 0;
      *a.n_dev = n - 1;
    }
  }
}

constexpr int kAdjElemThreads = 128;

// Backward step n, element gradients: one lane per element node (32 / n_en elements per
// warp), lane (e, la) owning the element DOFs 3 la .. 3 la + 2:
//   dJ/dE_e   -= dt y_e . [K1_e (u + beta v)_e + Lysmer terms]
//   dJ/drho_e -= dt sum ml1_e y_e (a + alpha v)_e + Lysmer term.
// Differences of FP64 states (translations removed, v_{n+1} - v_n) are taken in FP64 and the
// products in FP32 (GB300's FP64 rate is a fraction of its FP32 rate); per-element sums are
// FP64, made by the element's first lane in lane order (deterministic).  The last block to
// finish decrements the element kernel's step counter.
__global__ void __launch_bounds__(kAdjElemThreads) k_adj_elems(Args g, sc_adj_desc d, AdjState a, int cur, int ypair) {
  __shared__ float sw[kAdjElemThreads / 32][96];
  __shared__ float part[kAdjElemThreads / 32][32][2];
  const int n = *a.n_dev_e;
  const int k = n - *a.seg_t0;
  const double* y = cur ? a.y[1] : a.y[0];
  const float2* wp = cur ? a.wp[1] : a.wp[0];
  const float* v32 = cur ? a.v32[1] : a.v32[0];
  const float* a32 = cur ? a.a32[1] : a.a32[0];
  const float* y32 = cur ? a.y32[1] : a.y32[0];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int ne = d.n_en, nd = 3 * ne, epw = 32 / ne;
  const int grp = lane / ne, la = lane % ne, base = grp * ne;
  const float alpha = (float)g.alpha_r;
  const int64_t warps = (int64_t)gridDim.x * (kAdjElemThreads / 32);
  for (int64_t wg = (int64_t)blockIdx.x * (kAdjElemThreads / 32) + wib; wg * epw < d.n_elem; wg += warps) {
    const int64_t e = wg * epw + grp;
    const bool on = grp < epw && e < d.n_elem;
    float ya[3] = {0.f, 0.f, 0.f}, gr = 0.f;
    if (on) {
      const int* en = d.elem + e * ne;
      const int64_t sa = (int64_t)en[la] * 3, s0 = (int64_t)en[0] * 3;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        // K1 annihilates rigid translations: (u + beta v) relative to the element's first
        // node, differenced on the (hi, lo) pairs, so the FP32 products see strains
        const float2 wb = wp[sa + c], w0 = wp[s0 + c];
        sw[wib][base * 3 + 3 * la + c] = (wb.x - w0.x) + (wb.y - w0.y);
        ya[c] = y32[sa + c];
        gr = fmaf(d.ml1[e * nd + 3 * la + c] * ya[c], fmaf(alpha, v32[sa + c], a32[sa + c]), gr);
      }
    }
    __syncwarp();
    float ge = 0.f;
    if (on) {
      const float* K1 = d.ke1 + (int64_t)d.ke_type[e] * nd * nd + (int64_t)(3 * la) * nd;
      const float* wv = &sw[wib][base * 3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float row = 0.f;
        for (int b = 0; b < nd; ++b) row = fmaf(__ldg(K1 + c * nd + b), wv[b], row);
        ge = fmaf(ya[c], row, ge);
      }
    }
    part[wib][lane][0] = ge;
    part[wib][lane][1] = gr;
    __syncwarp();
    if (on && la == 0) {
      float ge_e = 0.f, gr_e = 0.f;
      for (int q = 0; q < ne; ++q) {
        ge_e += part[wib][base + q][0];
        gr_e += part[wib][base + q][1];
      }
      double gE = (double)ge_e, gR = (double)gr_e;
      const int64_t q0 = d.l_eptr[e], q1 = d.l_eptr[e + 1];
      if (q1 > q0) {  // Lysmer terms of boundary elements, FP64
        const double* u = a.seg_u + (int64_t)k * g.n_s;
        const double* v = a.seg_v + (int64_t)k * g.n_s;
        const double iE = 1.0 / d.young[e], iR = 1.0 / d.rho[e];
        for (int64_t q = q0; q < q1; ++q) {
          const double yr = y_at(y, d.l_row[q], ypair);
          const int cl = d.l_col[q];
          gE += yr * (d.l_s[q] * iE * fma(g.beta_r, v[cl], u[cl]) + 0.5 * d.l_c[q] * iE * v[cl]);
          gR += yr * 0.5 * d.l_c[q] * iR * v[cl];
        }
      }
      a.gE[e] -= g.dt * gE;
      a.gR[e] -= g.dt * gR;
    }
    __syncwarp();
  }
  if (last_block(a.ticket_e)) {
    if (threadIdx.x == 0) {
      *a.ticket_e = 0;
      *a.n_dev_e = n - 1;
    }
  }
}

// the element kernel's FP32 inputs of the first step reversed in a segment
__global__ void k_adj_prep(Args g, AdjState a, int buf, int pair) {
  const int64_t k = *a.n_dev - *a.seg_t0;
  const double* y = buf ? a.y[1] : a.y[0];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n_s; i += (int64_t)gridDim.x * blockDim.x)
    adj_prep_slot(g, a, buf, k, i, y_at(y, i, pair));
}

// start of the backward sweep: mu_u = 0, mu_v = P^T (v_N - d_N), y = mu_v / M_L
__global__ void k_adj_init(Args g, const double* __restrict__ IML, AdjState a, const double* target, int n_rec,
                           int N, int pair) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n_s; i += (int64_t)gridDim.x * blockDim.x) {
    a.mu_u[i] = 0.0;
    const int rj = a.rec_map[i];
    const double mv = rj >= 0 && !g.fixed[i] ? a.out_v[(int64_t)N * n_rec + rj] - target[(int64_t)N * n_rec + rj] : 0.0;
    a.mu_v[i] = mv;
    const double y0 = g.fixed[i] ? 0.0 : mv * IML[i];
    if (pair) reinterpret_cast<float2*>(a.y[0])[i] = split_pair(y0);
    else a.y[0][i] = y0;
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

__global__ void k_rec_map2(int n_s, int n_rec, const int* rec, int* map) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_s; i += (int64_t)gridDim.x * blockDim.x) map[i] = -1;
}
__global__ void k_rec_map2_fill(int n_rec, const int* rec, int* map) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n_rec; j += gridDim.x * blockDim.x) map[rec[j]] = j;
}

}  // namespace

template <int TPR>
static void launch_adj_rows_t(const sc_nb_newmark* h, cudaStream_t st, const Args& g, const sc_adj_desc& d,
                              const AdjState& a, int cur) {
  if (h->explicit_pair) k_adj_rows<3, true, TPR><<<h->tpr_blocks, kThreads, 0, st>>>(g, h->ML, h->IML, d, a, cur);
  else k_adj_rows<3, false, TPR><<<h->tpr_blocks, kThreads, 0, st>>>(g, h->ML, h->IML, d, a, cur);
}
static void launch_adj_rows(const sc_nb_newmark* h, cudaStream_t st, const Args& g, const sc_adj_desc& d,
                            const AdjState& a, int cur) {
  switch (h->tpr) {
    case 4: launch_adj_rows_t<4>(h, st, g, d, a, cur); break;
    case 2: launch_adj_rows_t<2>(h, st, g, d, a, cur); break;
    default: launch_adj_rows_t<1>(h, st, g, d, a, cur); break;
  }
}

extern "C" int sc_nb_adjoint(sc_nb_newmark* h, const sc_adj_desc* dp, double* J_host, double* grad_E,
                             double* grad_rho) {
  if (!h || !dp || !grad_E || !grad_rho) return SC_BAD_ARG;
  const sc_adj_desc d = *dp;
  if (d.n_steps <= 0 || d.checkpoint <= 0 || d.n_rec <= 0 || !d.rec_slot || !d.target || d.n_elem <= 0 ||
      d.n_en <= 0 || d.n_en > 32 || !d.elem || !d.ke_type || !d.ke1 || !d.young || !d.rho || !d.ml1 ||
      !d.l_eptr || h->g.D != 3)
    return SC_BAD_ARG;
  Args& g = h->g;
  cudaStream_t st = h->user;
  const int N = d.n_steps, C = d.checkpoint < d.n_steps ? d.checkpoint : d.n_steps, nseg = (N + C - 1) / C;
  const int64_t ns = g.n_s;
  // save the caller's output configuration
  const int o_int = g.out_interval, o_nrec = g.n_rec;
  const int* o_rec = g.rec_slot;
  double *o_u = g.out_u, *o_v = g.out_v, *o_a = g.out_a;
  const int64_t o_nout = g.n_out;
  AdjState a{};
  double *ck_u = nullptr, *ck_v = nullptr;
  int* t_host = nullptr;  // segment starts and backward starts, pinned (copied by the stream)
  int rc = SC_OK;
  auto M = [&](void** p, size_t b) { return check(cudaMallocAsync(p, b, st), "adjoint malloc"); };
  cudaGraphExec_t rec_exec[2] = {nullptr, nullptr}, bwd_exec[2] = {nullptr, nullptr};
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // phase timers: [0, 1] forward, then per segment [2 + 4 s ... 5 + 4 s] recompute and backward
  std::vector<cudaEvent_t> tev;
  cudaGraph_t rec_graph[2] = {nullptr, nullptr}, bwd_graph[2] = {nullptr, nullptr};
  do {
    if ((rc = M((void**)&ck_u, 8 * ns * nseg)) || (rc = M((void**)&ck_v, 8 * ns * nseg)) ||
        (rc = M((void**)&a.seg_u, 8 * ns * (C + 1))) || (rc = M((void**)&a.seg_v, 8 * ns * (C + 1))) ||
        (rc = M((void**)&a.mu_u, 8 * ns)) || (rc = M((void**)&a.mu_v, 8 * ns)) || (rc = M((void**)&a.y[0], 8 * ns)) ||
        (rc = M((void**)&a.y[1], 8 * ns)) || (rc = M((void**)&a.out_v, 8 * (int64_t)(N + 1) * d.n_rec)) ||
        (rc = M((void**)&a.n_dev, 4)) || (rc = M((void**)&a.n_dev_e, 4)) || (rc = M((void**)&a.ticket_e, 4)) ||
        (rc = M((void**)&a.seg_t0, 4)) || (rc = M((void**)&a.rec_map, 4 * ns)) || (rc = M((void**)&a.J, 8)) ||
        (rc = M((void**)&a.wp[0], 8 * ns)) || (rc = M((void**)&a.wp[1], 8 * ns)) || (rc = M((void**)&a.v32[0], 4 * ns)) ||
        (rc = M((void**)&a.v32[1], 4 * ns)) || (rc = M((void**)&a.a32[0], 4 * ns)) || (rc = M((void**)&a.a32[1], 4 * ns)) ||
        (rc = M((void**)&a.y32[0], 4 * ns)) || (rc = M((void**)&a.y32[1], 4 * ns)))
      break;
    if ((rc = check(cudaMallocHost((void**)&t_host, 8 * (size_t)nseg), "adjoint pinned"))) break;
    tev.assign(2 + 4 * (size_t)nseg, nullptr);
    for (auto& ev : tev)
      if ((rc = check(cudaEventCreate(&ev), "adjoint timer"))) break;
    if (rc) break;
    a.gE = grad_E;
    a.gR = grad_rho;
    cudaMemsetAsync(a.ticket_e, 0, 4, st);
    cudaMemsetAsync(grad_E, 0, 8 * (size_t)d.n_elem, st);
    cudaMemsetAsync(grad_rho, 0, 8 * (size_t)d.n_elem, st);
    cudaMemsetAsync(a.out_v, 0, 8 * (size_t)(N + 1) * d.n_rec, st);
    k_rec_map2<<<grid_for(ns, 256), 256, 0, st>>>((int)ns, d.n_rec, d.rec_slot, a.rec_map);
    k_rec_map2_fill<<<grid_for(d.n_rec, 128), 128, 0, st>>>(d.n_rec, d.rec_slot, a.rec_map);
    // forward from rest with checkpoints; receivers recorded into a.out_v
    cudaMemsetAsync(g.u, 0, 8 * ns, st);
    cudaMemsetAsync(g.v, 0, 8 * ns, st);
    if ((rc = sc_nb_set_output(h, 1, d.n_rec, d.rec_slot, nullptr, a.out_v, nullptr, N + 1))) break;
    cudaEventRecord(tev[0], st);
    for (int sgi = 0; sgi < nseg && !rc; ++sgi) {
      const int t0 = sgi * C, t1 = t0 + C < N ? t0 + C : N;
      cudaMemcpyAsync(ck_u + sgi * ns, g.u, 8 * ns, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(ck_v + sgi * ns, g.v, 8 * ns, cudaMemcpyDeviceToDevice, st);
      rc = sc_nb_explicit_run(h, t0, t1);
    }
    if (rc) break;
    cudaEventRecord(tev[1], st);
    k_adj_misfit<<<1, 1024, 0, st>>>(a.out_v, d.target, d.n_rec, N, a.J);
    // graphs: recompute step (explicit step storing its state), backward step (y ping-pong)
    const StateStore store{a.seg_u, a.seg_v, a.seg_t0};
    for (int kk = 0; kk < 2 && !rc; ++kk) {
      const double* vin = kk == 0 ? g.v : h->v1;
      double* vout = kk == 0 ? h->v1 : g.v;
      const double* win = kk == 0 ? h->w0 : h->w1;
      double* wout = kk == 0 ? h->w1 : h->w0;
      if ((rc = check(cudaStreamBeginCapture(h->cap, cudaStreamCaptureModeThreadLocal), "capture rec"))) break;
      launch_explicit<3>(h, h->cap, g, vin, vout, win, wout, store);
      if ((rc = check(cudaStreamEndCapture(h->cap, &rec_graph[kk]), "end rec"))) break;
      rc = check(cudaGraphInstantiate(&rec_exec[kk], rec_graph[kk], 0), "inst rec");
    }
    // backward step: the element kernel (forked onto the second capture stream) and the row
    // kernel run side by side; they read y[cur] and the segment's states and write disjoint data
    const int64_t elem_warps = (d.n_elem + 32 / d.n_en - 1) / (32 / d.n_en);
    const unsigned elem_blocks = grid_for(elem_warps, kAdjElemThreads / 32, 152 * 32);
    if (!ev_fork && (rc = check(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming), "event"))) break;
    if (!ev_join && (rc = check(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming), "event"))) break;
    for (int kk = 0; kk < 2 && !rc; ++kk) {
      if ((rc = check(cudaStreamBeginCapture(h->cap, cudaStreamCaptureModeThreadLocal), "capture bwd"))) break;
      cudaEventRecord(ev_fork, h->cap);
      cudaStreamWaitEvent(h->cap2, ev_fork, 0);
      k_adj_elems<<<elem_blocks, kAdjElemThreads, 0, h->cap2>>>(g, d, a, kk, h->explicit_pair);
      launch_adj_rows(h, h->cap, g, d, a, kk);
      cudaEventRecord(ev_join, h->cap2);
      cudaStreamWaitEvent(h->cap, ev_join, 0);
      if ((rc = check(cudaStreamEndCapture(h->cap, &bwd_graph[kk]), "end bwd"))) break;
      rc = check(cudaGraphInstantiate(&bwd_exec[kk], bwd_graph[kk], 0), "inst bwd");
    }
    if (rc) break;
    k_adj_init<<<h->vec_blocks, 256, 0, st>>>(g, h->IML, a, d.target, d.n_rec, N, h->explicit_pair);
    int yk = 0;  // y[yk] holds the y of the next step to reverse
    for (int sgi = nseg - 1; sgi >= 0 && !rc; --sgi) {
      const int t0 = sgi * C, t1 = t0 + C < N ? t0 + C : N;
      t_host[2 * sgi] = t0;
      t_host[2 * sgi + 1] = t1 - 1;
      cudaMemcpyAsync(g.u, ck_u + sgi * ns, 8 * ns, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(g.v, ck_v + sgi * ns, 8 * ns, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(a.seg_u, g.u, 8 * ns, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(a.seg_v, g.v, 8 * ns, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(a.seg_t0, t_host + 2 * sgi, 4, cudaMemcpyHostToDevice, st);
      // recompute states t0+1 .. t1 from the checkpoint (f = the entries of step t0)
      k_w_init<<<h->vec_blocks, 256, 0, st>>>(g, h->w0, h->explicit_pair);
      cudaMemsetAsync(g.f, 0, 8 * ns, st);
      k_set_t<<<1, 1, 0, st>>>(g.s, t0);
      k_force_explicit0<<<1, 256, 0, st>>>(g);
      int kk = 0;
      cudaEventRecord(tev[2 + 4 * sgi], st);
      for (int t = t0; t < t1 && !rc; ++t, kk ^= 1) rc = check(cudaGraphLaunch(rec_exec[kk], st), "rec launch");
      cudaEventRecord(tev[3 + 4 * sgi], st);
      // backward t1-1 .. t0
      cudaMemcpyAsync(a.n_dev, t_host + 2 * sgi + 1, 4, cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(a.n_dev_e, t_host + 2 * sgi + 1, 4, cudaMemcpyHostToDevice, st);
      cudaEventRecord(tev[4 + 4 * sgi], st);
      k_adj_prep<<<h->vec_blocks, 256, 0, st>>>(g, a, yk, h->explicit_pair);
      for (int t = t1 - 1; t >= t0 && !rc; --t, yk ^= 1) rc = check(cudaGraphLaunch(bwd_exec[yk], st), "bwd launch");
      cudaEventRecord(tev[5 + 4 * sgi], st);
    }
    if (!rc && J_host) {
      rc = check(cudaMemcpyAsync(J_host, a.J, 8, cudaMemcpyDeviceToHost, st), "J");
    }
    if (!rc) rc = check(cudaStreamSynchronize(st), "sync adjoint");
    if (!rc) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, tev[0], tev[1]);
      h->adj_ms[0] = ms;
      h->adj_ms[1] = h->adj_ms[2] = 0.f;
      for (int sgi = 0; sgi < nseg; ++sgi) {
        cudaEventElapsedTime(&ms, tev[2 + 4 * sgi], tev[3 + 4 * sgi]);
        h->adj_ms[1] += ms;
        cudaEventElapsedTime(&ms, tev[4 + 4 * sgi], tev[5 + 4 * sgi]);
        h->adj_ms[2] += ms;
      }
    }
  } while (0);
  cudaStreamSynchronize(st);
  for (int kk = 0; kk < 2; ++kk) {
    if (rec_exec[kk]) cudaGraphExecDestroy(rec_exec[kk]);
    if (rec_graph[kk]) cudaGraphDestroy(rec_graph[kk]);
    if (bwd_exec[kk]) cudaGraphExecDestroy(bwd_exec[kk]);
    if (bwd_graph[kk]) cudaGraphDestroy(bwd_graph[kk]);
  }
  for (auto ev : tev)
    if (ev) cudaEventDestroy(ev);
  if (ev_fork) cudaEventDestroy(ev_fork);
  if (ev_join) cudaEventDestroy(ev_join);
  void* frees[] = {ck_u, ck_v, a.seg_u, a.seg_v, a.mu_u, a.mu_v, a.y[0], a.y[1], a.out_v, a.n_dev, a.n_dev_e,
                   a.ticket_e, a.seg_t0, a.rec_map, a.J, a.wp[0], a.wp[1], a.v32[0], a.v32[1], a.a32[0], a.a32[1],
                   a.y32[0], a.y32[1]};
  for (void* q : frees)
    if (q) cudaFree(q);
  if (t_host) cudaFreeHost(t_host);
  sc_nb_set_output(h, o_int, o_nrec, o_rec, o_u, o_v, o_a, o_nout);
  return rc;
}

extern "C" int sc_nb_adjoint_timings(sc_nb_newmark* h, float* ms3) {
  if (!h || !ms3) return SC_BAD_ARG;
  for (int i = 0; i < 3; ++i) ms3[i] = h->adj_ms[i];
  return SC_OK;
}

extern "C" int sc_nb_status(sc_nb_newmark* h, int64_t* total_iters, int* max_iters, int* fsai_fallback_rows) {
  if (!h) return SC_BAD_ARG;
  int rc = check(cudaStreamSynchronize(h->user), "sync");
  if (rc) return rc;
  Scal s;
  if ((rc = check(cudaMemcpy(&s, h->g.s, sizeof(s), cudaMemcpyDeviceToHost), "read"))) return rc;
  if (total_iters) *total_iters = s.total_iters;
  if (max_iters) *max_iters = s.max_seen;
  if (fsai_fallback_rows) *fsai_fallback_rows = s.fsai_fallback;
  return s.status;
}

extern "C" int sc_nb_time_spmv(sc_nb_newmark* h, int reps, float* ms_per_launch, int64_t* bytes_per_launch) {
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
  const unsigned nbk = h->node_blocks;
  auto launch = [&]() {
    if (h->g.spmv_pair) {
      if (h->g.D == 3) k_spmv_pair<3, 2><<<nbk, kThreads, 0, st>>>(h->g, none);
      else k_spmv_pair<2, 2><<<nbk, kThreads, 0, st>>>(h->g, none);
    } else {
      if (h->g.D == 3) k_spmv<3, 2><<<nbk, kThreads, 0, st>>>(h->g, none);
      else k_spmv<2, 2><<<nbk, kThreads, 0, st>>>(h->g, none);
    }
  };
  launch();
  cudaEventRecord(e0, st);
  for (int i = 0; i < reps; ++i) launch();
  cudaEventRecord(e1, st);
  rc = check_launch("nb spmv timing");
  if (!rc) rc = check(cudaEventSynchronize(e1), "event sync");
  float ms = 0.f;
  if (!rc) cudaEventElapsedTime(&ms, e0, e1);
  *ms_per_launch = ms / reps;
  if (bytes_per_launch) {
    const int64_t D2 = (int64_t)h->g.D * h->g.D;
    // A blocks + block columns + row pointers + one read of p + the write of w
    *bytes_per_launch = h->g.nnzb * (8 * D2 + 4) + (int64_t)(h->g.n_slices + 1) * 8 + h->g.n_s * 16;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

// Operator application for testing and profiling: y = Op x in slot space, with
// which = 0: A (the PCG operator), 1: K, 2: consistent mass (m_ab I blocks), 3: the
// preconditioner G^T G, 4: the Lysmer dashpot matrix.  Synchronous.  Uses the solver's
// scratch vectors (call between steps).
__global__ void k_apply_blocks(Args g, const double* __restrict__ planes, int scalar, const double* __restrict__ x,
                               double* __restrict__ y) {
  const int D = g.D;
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < g.n_nodes;
       row += (int64_t)gridDim.x * blockDim.x) {
    const int64_t sl = row >> 5;
    const int64_t p0 = g.sf_ptr[sl] + 4 * (row & 31), W = (g.sf_ptr[sl + 1] - g.sf_ptr[sl]) >> 5;
    double s[3] = {0, 0, 0};
    for (int64_t j = 0; j < W; ++j) {
      const int64_t pos = p0 + 128 * (j >> 2) + (j & 3);
      const int64_t bs = (int64_t)g.sf_col[pos] * D;
      for (int c = 0; c < D; ++c) {
        if (scalar) s[c] += planes[pos] * x[bs + c];
        else
          for (int d = 0; d < D; ++d) s[c] += planes[(int64_t)(c * D + d) * g.sf_n + pos] * x[bs + d];
      }
    }
    for (int c = 0; c < D; ++c) y[row * D + c] = s[c];
  }
}

__global__ void k_apply_cab(Args g, const double* __restrict__ x, double* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n_s; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int64_t k = g.cab_ptr[i]; k < g.cab_ptr[i + 1]; ++k) s += g.cab_val[k] * x[g.cab_col[k]];
    y[i] = s;
  }
}

__global__ void k_copy(int64_t n, const double* __restrict__ x, double* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = x[i];
}

extern "C" int sc_nb_apply(sc_nb_newmark* h, int which, const double* x, double* y) {
  if (!h || !x || !y || which < 0 || which > 4) return SC_BAD_ARG;
  Args g = h->g;
  cudaStream_t st = h->user;
  const unsigned nb = grid_for(g.n_nodes, 128, 152 * 64);
  switch (which) {
    case 0: k_apply_blocks<<<nb, 128, 0, st>>>(g, g.AS, 0, x, y); break;
    case 1: k_apply_blocks<<<nb, 128, 0, st>>>(g, g.KS, 0, x, y); break;
    case 2: k_apply_blocks<<<nb, 128, 0, st>>>(g, g.MSS, 1, x, y); break;
    case 4: k_apply_cab<<<grid_for(g.n_s, 256), 256, 0, st>>>(g, x, y); break;
    case 3: {
      // r <- x, t = G r, z = G^T t (the solver's own kernels), y <- z
      k_copy<<<grid_for(g.n_s, 256), 256, 0, st>>>(g.n_s, x, g.r);
      cudaGraphConditionalHandle none = 0;
      if (g.D == 3) {
        k_prec_lower<3><<<h->node_blocks, kThreads, 0, st>>>(g);
        k_prec_upper_nograph<3><<<h->node_blocks, kThreads, 0, st>>>(g);
      } else {
        k_prec_lower<2><<<h->node_blocks, kThreads, 0, st>>>(g);
        k_prec_upper_nograph<2><<<h->node_blocks, kThreads, 0, st>>>(g);
      }
      (void)none;
      k_copy<<<grid_for(g.n_s, 256), 256, 0, st>>>(g.n_s, g.z, y);
      break;
    }
  }
  int rc = check_launch("nb apply");
  if (!rc) rc = check(cudaStreamSynchronize(st), "sync apply");
  return rc;
}

extern "C" int sc_nb_destroy(sc_nb_newmark* h) {
  if (!h) return SC_OK;
  drop_graph(h);
  drop_explicit_graphs(h);
  for (int i = 0; i < h->n_sell_mem; ++i) cudaFree(h->sell_mem[i]);
  if (h->ML) cudaFree(h->ML);
  if (h->IML) cudaFree(h->IML);
  if (h->KPS) cudaFree(h->KPS);
  if (h->v1) cudaFree(h->v1);
  if (h->w0) cudaFree(h->w0);
  if (h->w1) cudaFree(h->w1);
  if (h->rec_map) cudaFree(h->rec_map);
  if (h->cap) cudaStreamDestroy(h->cap);
  if (h->cap2) cudaStreamDestroy(h->cap2);
  delete h;
  return SC_OK;
}
