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
// warm-started from the polynomial extrapolation of the accelerations of order p
// (x0 = sum_k (-1)^k C(p+1, k+1) a_{n-k}, e.g. 3a_n - 3a_{n-1} + a_{n-2} for p = 2; p is
// fixed by the caller or, by default, adapted to the iteration counts, see k_advance), stopped at
// ||r|| <= rtol ||b||; then u, v, a are updated exactly as the reference's update.
//
// Kernels: one warp per node row (lanes over the row's blocks) for every block product;
// per-block partial sums reduced by the last block (ticket, fixed order, no spin-waits);
// one CUDA graph per step with a device-side WHILE conditional around the PCG body.
#include <string.h>
#include <math.h>
#include <stdlib.h>

#include <vector>

#include "sc_nb.cuh"

namespace sc {
namespace nb {

// ------------------------------------------------------------------ per-step kernels

// The step's force (step t's entries cleared, step t + 1's added), then the warm start's order cap
// (one block)
__global__ void k_force(Args g) {
  const int t = g.s->t;
  if (g.f_ptr) {
    if (t >= 0 && t < g.n_t)
      for (int64_t k = g.f_ptr[t] + threadIdx.x; k < g.f_ptr[t + 1]; k += blockDim.x) g.f[g.f_slot[k]] = 0.0;
    __syncthreads();
    const int t1 = t + 1;
    if (t1 >= 0 && t1 < g.n_t)
      for (int64_t k = g.f_ptr[t1] + threadIdx.x; k < g.f_ptr[t1 + 1]; k += blockDim.x)
        g.f[g.f_slot[k]] += g.f_val[k];
  }
  warm_start_order_cap(g.s, g.pred_order, g.order_cap, ForceRows{g.n_t, g.f_ptr, g.f_slot, g.f_val});
}

// Predictor vectors (slot space):
//   vp = v + dt/2 a, up = u + dt v + dt^2/4 a                  (Newmark predictors)
//   b = f - C vp - K up,  C = Cabs + alpha M + beta K
//     = f - K (up + beta vp) - M (alpha vp) - Cabs vp
//   x0 = warm start;  A x0 = aM M x0 + aK K x0 + aC Cabs x0
// stored: q1 = up + beta vp, q2 = alpha vp, y1 = vp, x0.
// One thread per slot (coalesced loads and stores), kPredNodes nodes per block of
// D * kPredNodes threads: the pair residual's records of the block's nodes are assembled in
// shared memory and leave as whole 16-byte stores.
constexpr int kPredNodes = 128;

template <int D>
__global__ void __launch_bounds__(D * kPredNodes) k_predict(Args g) {
  constexpr int R = kRecFloats(D);
  __shared__ float4 srec[kPredNodes * R / 4];
  float* sr = reinterpret_cast<float*>(srec);
  const double dt = g.dt, h = 0.5 * dt, qq = 0.25 * dt * dt;
  // warm-start order p = min(history, order, the force history's cap) and its coefficients,
  // once per thread
  const int p0 = warm_start_order(g.s, g.pred_order);
  const int p = g.s->pcap < p0 ? g.s->pcap : p0;
  double cf[kHistMax + 1];
  warm_start_coeffs(p, cf);
  const double* hs[kHistMax];  // a_{n-1-k}
#pragma unroll
  for (int k = 0; k < kHistMax; ++k) hs[k] = g.ah[hist_slot(g.s->head, k)];
  // while the pair residual runs, q1, q2 and the pair copy of x0 are read by no one
  const bool fp64_res = !g.res_pair || g.s->res_fp64;
  for (int64_t n0 = (int64_t)blockIdx.x * kPredNodes; n0 < g.n_nodes; n0 += (int64_t)gridDim.x * kPredNodes) {
    const int64_t i = n0 * D + threadIdx.x;
    const int ln = threadIdx.x / D, c = threadIdx.x - ln * D;
    if (i < g.n_s) {
      const double ai = g.a[i], vi = g.v[i], ui = g.u[i];
      const int fx = g.fixed[i];
      // x0 = sum_{k=0..p} (-1)^k C(p+1, k+1) a_{n-k}, terms summed in a fixed order
      double xs = cf[0] * ai;
#pragma unroll
      for (int k = 1; k <= kHistMax; ++k)
        if (k <= p) xs += cf[k] * hs[k - 1][i];
      const double vp = vi + h * ai;
      const double up = ui + dt * vi + qq * ai;
      const double q1 = up + g.beta_r * vp, q2 = g.alpha_r * vp;
      if (fp64_res) {
        g.q1[i] = q1;
        g.q2[i] = q2;
      }
      g.y1[i] = vp;
      const double x0 = fx ? 0.0 : xs;
      g.x0[i] = x0;
      if (g.spmv_pair && fp64_res) g.p2[i] = split_pair(x0);  // p2 is scratch until p is first written
      if (g.res_pair) {
        const float2 zk = split_pair(fma(g.aK, x0, q1)), zm = split_pair(fma(g.aM, x0, q2));
        float* rec = sr + ln * R;
        rec[kRecM + 2 * c] = zm.x;
        rec[kRecM + 2 * c + 1] = zm.y;
        rec[kRecM + 2 * D + c] = (float)q2;
        rec[kRecK(D) + 2 * c] = zk.x;
        rec[kRecK(D) + 2 * c + 1] = zk.y;
        rec[kRecK(D) + 2 * D + c] = (float)q1;
        if (c == 0)
          for (int k = 6 * D; k < R; ++k) rec[k] = 0.f;
        g.zc[i] = fma(g.aC, x0, vp);
      }
    }
    if (g.res_pair) {
      __syncthreads();
      const int64_t nodes = g.n_nodes - n0 < kPredNodes ? g.n_nodes - n0 : kPredNodes;
      float4* dst = reinterpret_cast<float4*>(g.rrec + n0 * R);
      for (int k = threadIdx.x; k < nodes * (R / 4); k += blockDim.x) dst[k] = srec[k];
      __syncthreads();
    }
  }
}

// r = b - A x0 with b = f - K q1 - M q2 - Cabs y1; bb = |b|^2.  x = x0.  gate = 1: only when the
// pair residual has handed over to this one (Scal::res_fp64), else the kernel returns at once.
template <int D, bool kPair>
__global__ void __launch_bounds__(kThreads) k_residual(Args g, int gate) {
  if (gate && !g.s->res_fp64) return;
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
        g.r32[i] = (float)rv;
        g.r0[i] = rv;
        g.r032[i] = (float)rv;
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

// The residual in FP32-pair arithmetic, one pass over the K pair planes and the mass pairs.
// With A = aM M + aK K + aC Cabs,
//   r = b - A x0 = f - K (q1 + aK x0) - M (q2 + aM x0) - Cabs (y1 + aC x0),
// so r needs no A pass and no FP64 product: the pair products keep about 48 bits, and r is
// exact to that rounding of its own terms.  b = f - K q1 - M q2 - Cabs y1 only scales the
// tolerance, so it is formed from the pairs' hi parts in FP32.  When the elastic and inertial
// terms cancel the load strongly (|K q1 + M q2| above kResRatio |b|, slow motion), 48 bits of
// the terms would no longer carry r to the tolerance: the last block then sets
// Scal::res_fp64 and every later step runs the FP64 residual instead (this step's r is still
// good to about kResRatio 2^-48 of |b|).  gate: returns at once when res_fp64 is set.
constexpr double kResRatio = 30.0;

template <int D, int kKeep>  // kKeep = g.keep_l2 at compile time
__global__ void __launch_bounds__(kThreads) k_residual_kp(Args g) {
  if (g.s->res_fp64) return;
  __shared__ double sh[64];
  double pbb = 0.0, pkq = 0.0;
  SELL_ROW_LOOP(g.sf_ptr) {
    SELL_ROW_BEGIN(g.sf_ptr)
    float rh[D], rl[D], bq[D];
#pragma unroll
    for (int c = 0; c < D; ++c) rh[c] = rl[c] = bq[c] = 0.f;
    for (int64_t q = 0; q < nq; ++q) {
      int cl[4];
      cols4(g.sf_col, p0 + 128 * q, cl, kKeep);
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {  // two entries at a time (registers)
        const int64_t pos = p0 + 128 * q + 2 * hh;
        const float* rp[2] = {g.rrec + (int64_t)cl[2 * hh] * kRecFloats(D),
                              g.rrec + (int64_t)cl[2 * hh + 1] * kRecFloats(D)};
        // the mass part first: M is diagonal in the components, so the two entries' M records
        // are used up before their K records are loaded (half the registers live at a time)
        {
          float mv[2][3 * D];
          ldrec<kRecM, 3 * D>(rp[0], mv[0]);
          ldrec<kRecM, 3 * D>(rp[1], mv[1]);
          float2 m2[2];
          ld2(g.MSP + pos, m2, kKeep);
#pragma unroll
          for (int c = 0; c < D; ++c) {
            pair_fma(m2[0].x, m2[0].y, make_float2(mv[0][2 * c], mv[0][2 * c + 1]), rh[c], rl[c]);
            pair_fma(m2[1].x, m2[1].y, make_float2(mv[1][2 * c], mv[1][2 * c + 1]), rh[c], rl[c]);
            bq[c] = fmaf(m2[1].x, mv[1][2 * D + c], fmaf(m2[0].x, mv[0][2 * D + c], bq[c]));
          }
        }
        float kv[2][3 * D];
        ldrec<kRecK(D), 3 * D>(rp[0], kv[0]);
        ldrec<kRecK(D), 3 * D>(rp[1], kv[1]);
#pragma unroll
        for (int c = 0; c < D; ++c) {
#pragma unroll
          for (int d = 0; d < D; ++d) {
            float2 k2[2];
            ld2(g.KPS + (int64_t)(c * D + d) * g.sf_n + pos, k2, kKeep);
            pair_fma(k2[0].x, k2[0].y, make_float2(kv[0][2 * d], kv[0][2 * d + 1]), rh[c], rl[c]);
            pair_fma(k2[1].x, k2[1].y, make_float2(kv[1][2 * d], kv[1][2 * d + 1]), rh[c], rl[c]);
            bq[c] = fmaf(k2[1].x, kv[1][2 * D + d], fmaf(k2[0].x, kv[0][2 * D + d], bq[c]));
          }
        }
      }
    }
    if (row < g.n_nodes) {
#pragma unroll
      for (int c = 0; c < D; ++c) {
        const int64_t i = row * D + c;
        double bv = 0.0, rv = 0.0;
        if (!g.fixed[i]) {
          double cb = 0.0, cz = 0.0;  // Lysmer dashpots (boundary rows only)
          for (int64_t k = g.cab_ptr[i]; k < g.cab_ptr[i + 1]; ++k) {
            const int jj = g.cab_col[k];
            cb = fma(g.cab_val[k], g.y1[jj], cb);
            cz = fma(g.cab_val[k], g.zc[jj], cz);
          }
          bv = g.f[i] - (double)bq[c] - cb;
          rv = g.f[i] - ((double)rh[c] + (double)rl[c]) - cz;
          pkq += (double)bq[c] * (double)bq[c];
        }
        g.r[i] = rv;
        g.r32[i] = (float)rv;
        g.r0[i] = rv;
        g.r032[i] = (float)rv;
        g.x[i] = g.x0[i];
        pbb += bv * bv;
      }
    }
  }
  block_sum2(pbb, pkq, sh);
  if (threadIdx.x == 0) {
    g.part[blockIdx.x * 4 + 2] = pbb;
    g.part[blockIdx.x * 4 + 3] = pkq;
  }
  if (last_block(&g.s->ticket)) {
    double bb, kq;
    reduce_parts2(g.part, 2, 3, sh, bb, kq);
    if (threadIdx.x == 0) {
      g.s->bb = bb;
      if (kq > kResRatio * kResRatio * bb) g.s->res_fp64_next = 1;  // k_advance makes it current
      g.s->it = 0;
      g.s->ticket = 0;
    }
  }
}

// s[c] += sum over the row's chunks of the factor planes (c, d) times the gathered FP32 vector's
// d component.  Two chunks at a time, so that two chunks' column, gather and plane loads are in
// flight together (the chunk count is the slice's, uniform across the warp); the products are
// summed in the same order as one chunk at a time.  The kernels that use it are held to 64
// registers (four blocks of 256 per SM): the latency of the column -> gather chain bounds them,
// and at their natural 72 registers (three blocks) they were slower than one chunk at a time.
template <int D>
__device__ __forceinline__ void fsai_chunk(const __half* planes, int64_t plane_n, const float* vec, int64_t pos,
                                           const int (&cl)[4], int keep, float (&s)[D]) {
  float va[4][D];
#pragma unroll
  for (int e = 0; e < 4; ++e) ldvec<D>(vec, cl[e], va[e]);
#pragma unroll
  for (int c = 0; c < D; ++c)
#pragma unroll
    for (int d = 0; d < D; ++d) {
      float gv[4];
      ld4(planes + (int64_t)(c * D + d) * plane_n + pos, gv, keep);
#pragma unroll
      for (int e = 0; e < 4; ++e) s[c] = fmaf(gv[e], va[e][d], s[c]);
    }
}

template <int D>
__device__ __forceinline__ void fsai_row(const __half* planes, int64_t plane_n, const int* col, const float* vec,
                                         int64_t p0, int64_t nq, int keep, float (&s)[D]) {
  int64_t q = 0;
  for (; q + 1 < nq; q += 2) {
    const int64_t pos = p0 + 128 * q;
    int c0[4], c1[4];
    cols4(col, pos, c0, keep);
    cols4(col, pos + 128, c1, keep);
    fsai_chunk<D>(planes, plane_n, vec, pos, c0, keep, s);
    fsai_chunk<D>(planes, plane_n, vec, pos + 128, c1, keep, s);
  }
  if (q < nq) {
    const int64_t pos = p0 + 128 * q;
    int c0[4];
    cols4(col, pos, c0, keep);
    fsai_chunk<D>(planes, plane_n, vec, pos, c0, keep, s);
  }
}

// t = G r  (lower pattern, FP16 factor planes, FP32 products and result).  With kDot (inside a
// solve) also the PCG's r.z: the preconditioner is split, z = G^T G r, so r.z = (G r).(G r) =
// |t|^2, and the last block forms beta and rz here.  The upper half then knows beta and writes
// the new direction p = z + beta p itself (no separate direction pass, z never stored).
template <int D, int kKeep, bool kDot>  // kKeep = g.keep_l2 at compile time
__global__ void __launch_bounds__(kThreads, 4) k_prec_lower(Args g) {
  const float* rv = g.s->restart ? g.r032 : g.r32;  // a restart preconditions r0
  double ptt = 0.0;
  SELL_ROW_LOOP(g.sl_ptr) {
    SELL_ROW_BEGIN(g.sl_ptr)
    float s[D];
#pragma unroll
    for (int c = 0; c < D; ++c) s[c] = 0.f;
    fsai_row<D>(g.GS, g.sl_n, g.sl_col, rv, p0, nq, kKeep, s);
    if (row < g.n_nodes) {
#pragma unroll
      for (int c = 0; c < D; ++c) {
        g.t32[row * D + c] = s[c];
        if (kDot) ptt = fma((double)s[c], (double)s[c], ptt);
      }
    }
  }
  if (kDot) {
    __shared__ double sh[32];
    const double t = block_sum(ptt, sh);
    if (threadIdx.x == 0) g.part[blockIdx.x * 4 + 0] = t;
    if (last_block(&g.s->ticket)) {
      const double rz = reduce_parts(g.part, 0, sh);
      if (threadIdx.x == 0) {
        Scal* s = g.s;
        s->ticket = 0;
        // a restart starts a fresh direction; after the residual beta is not used (p = z)
        s->beta = s->restart ? 0.0 : (s->rz != 0.0 ? rz / s->rz : 0.0);
        s->rz = rz;
      }
    }
  }
}

constexpr double kA32Margin = 16.0;

// z = G^T t and the new direction from it.  mode 0 (inside the PCG): p = z + beta p, with beta
// from the lower half; mode 1 (after the residual): p = z, rr, and the conditional from |r| vs
// |b|.  rz comes from the lower half in both modes.
template <int D, int kMode, int kKeep>  // kKeep = g.keep_l2 at compile time
__global__ void __launch_bounds__(kThreads, 4) k_prec_upper(Args g, int mode, cudaGraphConditionalHandle hc) {
  __shared__ double sh[32];
  double prr = 0.0;
  // a restart (inside the PCG): x, r back to x0, r0 and a fresh direction (beta = 0); a switch
  // to Ah: x, r become x0, r0 (the CG goes on).  k_update clears both flags before it decides
  // the next iteration's.
  const bool rs = mode == 0 && g.s->restart;
  const bool sw = mode == 0 && g.s->sw;
  const double beta = mode == 0 ? g.s->beta : 0.0;
  SELL_ROW_LOOP(g.su_ptr) {
    SELL_ROW_BEGIN(g.su_ptr)
    float s[D];
#pragma unroll
    for (int c = 0; c < D; ++c) s[c] = 0.f;
    fsai_row<D>(g.GTS, g.su_n, g.su_col, g.t32, p0, nq, kKeep, s);
    if (row < g.n_nodes) {
#pragma unroll
      for (int c = 0; c < D; ++c) {
        const int64_t i = row * D + c;
        const double z = (double)s[c];
        if (mode == 1) {
          const double r = g.r[i];
          g.p[i] = z;
          if (g.spmv_pair) g.p2[i] = make_float2(s[c], 0.f);  // z is an FP32 value: the pair is exact
          prr += r * r;
        } else {
          if (rs) {
            g.r[i] = g.r0[i];
            g.x[i] = g.x0[i];
          } else if (sw) {
            g.r0[i] = g.r[i];
            g.r032[i] = g.r32[i];
            g.x0[i] = g.x[i];
          }
          const double pv = rs ? z : fma(beta, g.p[i], z);
          g.p[i] = pv;
          if (g.spmv_pair) g.p2[i] = split_pair(pv);
        }
      }
    }
  }
  if (mode == 0) return;
  const double t = block_sum(prr, sh);
  if (threadIdx.x == 0) g.part[blockIdx.x * 4 + 1] = t;
  if (last_block(&g.s->ticket)) {
    const double rr = reduce_parts(g.part, 1, sh);
    if (threadIdx.x == 0) {
      Scal* s = g.s;
      s->ticket = 0;
      s->rr = rr;
      s->rr0 = rr;
      s->dd = s->dd_pre = 0.0;
      s->restart = s->sw = s->no_switch = 0;
      const bool done = rr <= s->tol2 * s->bb;
      // the FP32 matrix when the last step's |x - x0| / |r0|, scaled to this r0, keeps the
      // bound lo_norm |x - x0| below tol |b| / kA32Margin
      int a = 0;
      if (g.a32_mode == 2) a = 1;
      else if (g.a32_mode == 1 && s->rho >= 0.0)
        a = s->lo_norm * s->rho * sqrt(rr) * kA32Margin <= sqrt(s->tol2 * s->bb) ? 1 : 0;
      s->a32 = a;
      if (a && !done) s->a32_steps += 1;
      pcg_continue<kMode>(hc, s, !done);
    }
  }
}

// z = G^T t only (no reductions, no graph conditional): used by sc_nb_apply
template <int D>
__global__ void __launch_bounds__(kThreads, 4) k_prec_upper_nograph(Args g) {
  SELL_ROW_LOOP(g.su_ptr) {
    SELL_ROW_BEGIN(g.su_ptr)
    float s[D];
#pragma unroll
    for (int c = 0; c < D; ++c) s[c] = 0.f;
    fsai_row<D>(g.GTS, g.su_n, g.su_col, g.t32, p0, nq, g.keep_l2, s);
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
// With a32 it reads the hi parts alone (a copy, 4 B per value): w = Ah p, the FP32 matrix Ah
// applied to p in the same pair arithmetic (to ~2^-46 for Ah itself).
template <int D, int kKeep>  // kKeep: the planes' load policy (g.keep_l2) fixed at compile time, or -1
__device__ __forceinline__ void spmv_chunk(const Args& g, int64_t pos, const int (&cl)[4], bool a32, float (&hi)[D],
                                           float (&lo)[D]) {
  const int keep = kKeep >= 0 ? kKeep : g.keep_l2;
  float2 pv[4][D];
#pragma unroll
  for (int e = 0; e < 4; ++e)
#pragma unroll
    for (int d = 0; d < D; ++d) pv[e][d] = g.p2[(int64_t)cl[e] * D + d];
#pragma unroll
  for (int c = 0; c < D; ++c)
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const int64_t off = (int64_t)(c * D + d) * g.sf_n + pos;
      if (a32) {
        float ah[4];
        ld4(g.AHS + off, ah, keep);
#pragma unroll
        for (int e = 0; e < 4; ++e) pair_fma(ah[e], 0.f, pv[e][d], hi[c], lo[c]);
      } else {
        float2 a4[4];
        ld4(g.APS + off, a4, keep);
#pragma unroll
        for (int e = 0; e < 4; ++e) pair_fma(a4[e].x, a4[e].y, pv[e][d], hi[c], lo[c]);
      }
    }
}

// the SpMV's rows: pair planes one chunk at a time (kA32 = false), or the hi planes alone two
// chunks at a time (half the bytes per chunk, so twice the loads in flight); then p.w and alpha
template <int D, int kMode, bool kA32, int kKeep>
__device__ __forceinline__ void spmv_rows(const Args& g, cudaGraphConditionalHandle hc) {
  __shared__ double sh[32];
  double ppw = 0.0;
  const int keep = kKeep >= 0 ? kKeep : g.keep_l2;
  SELL_ROW_LOOP(g.sf_ptr) {
    SELL_ROW_BEGIN(g.sf_ptr)
    float hi[D], lo[D];
#pragma unroll
    for (int c = 0; c < D; ++c) hi[c] = lo[c] = 0.f;
    if (kA32) {
      int64_t q = 0;
      for (; q + 1 < nq; q += 2) {
        const int64_t pos = p0 + 128 * q;
        int c0[4], c1[4];
        cols4(g.sf_col, pos, c0, keep);
        cols4(g.sf_col, pos + 128, c1, keep);
        spmv_chunk<D, kKeep>(g, pos, c0, true, hi, lo);
        spmv_chunk<D, kKeep>(g, pos + 128, c1, true, hi, lo);
      }
      if (q < nq) {
        int c0[4];
        cols4(g.sf_col, p0 + 128 * q, c0, keep);
        spmv_chunk<D, kKeep>(g, p0 + 128 * q, c0, true, hi, lo);
      }
    } else {
      for (int64_t q = 0; q < nq; ++q) {
        int c0[4];
        cols4(g.sf_col, p0 + 128 * q, c0, keep);
        spmv_chunk<D, kKeep>(g, p0 + 128 * q, c0, false, hi, lo);
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

// Both forms are launched in the PCG loop; the one that does not match Scal::a32 returns at once
// (kMode 2, the timing launch, always runs).  Separate kernels keep the pair form at 64 registers;
// the FP32-matrix form is held to 80 (three blocks per SM: 0.140 ms at the 1.79 M-equation box
// against 0.203 ms at its natural 105 registers and 0.210 ms one chunk at a time).
template <int D, int kMode, int kKeep>
__global__ void __launch_bounds__(kThreads, 4) k_spmv_pair(Args g, cudaGraphConditionalHandle hc) {
  if (kMode != 2 && g.s->a32) return;
  spmv_rows<D, kMode, false, kKeep>(g, hc);
}

// kKeep = g.keep_l2, fixed at compile time (the launch picks the instance)
template <int D, int kMode, int kKeep>
__global__ void __launch_bounds__(kThreads, 3) k_spmv_a32(Args g, cudaGraphConditionalHandle hc) {
  if (kMode != 2 && !g.s->a32) return;
  spmv_rows<D, kMode, true, kKeep>(g, hc);
}

template <int D, int kMode>
static void launch_spmv_a32(const Args& g, unsigned blocks, cudaStream_t st, cudaGraphConditionalHandle hc) {
  if (g.keep_l2) k_spmv_a32<D, kMode, 1><<<blocks, kThreads, 0, st>>>(g, hc);
  else k_spmv_a32<D, kMode, 0><<<blocks, kThreads, 0, st>>>(g, hc);
}
template <int D, int kMode>
static void launch_spmv_pair(const Args& g, unsigned blocks, cudaStream_t st, cudaGraphConditionalHandle hc) {
  if (g.keep_l2) k_spmv_pair<D, kMode, 1><<<blocks, kThreads, 0, st>>>(g, hc);
  else k_spmv_pair<D, kMode, 0><<<blocks, kThreads, 0, st>>>(g, hc);
}
template <int D, bool kDot = true>
static void launch_prec_lower(const Args& g, unsigned blocks, cudaStream_t st) {
  if (g.keep_l2) k_prec_lower<D, 1, kDot><<<blocks, kThreads, 0, st>>>(g);
  else k_prec_lower<D, 0, kDot><<<blocks, kThreads, 0, st>>>(g);
}
template <int D, int kMode>
static void launch_prec_upper(const Args& g, unsigned blocks, cudaStream_t st, int mode,
                              cudaGraphConditionalHandle hc) {
  if (g.keep_l2) k_prec_upper<D, kMode, 1><<<blocks, kThreads, 0, st>>>(g, mode, hc);
  else k_prec_upper<D, kMode, 0><<<blocks, kThreads, 0, st>>>(g, mode, hc);
}

// x += alpha p ; r -= alpha w ; partial r.r and |x - x0|^2 ; last block: convergence test.
// With the FP32 matrix Ah (Scal::a32) the true residual is within lo_norm |x - x0| of the
// recursive one, so the test is |r| + lo_norm |x - x0| <= tol |b|; once that bound alone passes
// half the tolerance the solve restarts from x0 in pairs (Scal::restart).  A solve on the pairs
// switches to Ah (Scal::sw) when |r| has fallen as far as a step needs r0 to start on Ah; x and
// r then become the x0 and r0 that the bound and a restart refer to.
template <int kMode>
__global__ void k_update(Args g, cudaGraphConditionalHandle hc) {
  __shared__ double sh[64];
  const double alpha = g.s->alpha;
  double prr = 0.0, pdd = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n_s; i += (int64_t)gridDim.x * blockDim.x) {
    const double x = fma(alpha, g.p[i], g.x[i]);
    g.x[i] = x;
    const double dx = x - g.x0[i];
    pdd += dx * dx;
    const double r = fma(-alpha, g.w[i], g.r[i]);
    g.r[i] = r;
    g.r32[i] = (float)r;
    prr += r * r;
  }
  block_sum2(prr, pdd, sh);
  if (threadIdx.x == 0) {
    g.part[blockIdx.x * 4 + 1] = prr;
    g.part[blockIdx.x * 4 + 2] = pdd;
  }
  if (last_block(&g.s->ticket)) {
    double rr, dd;
    reduce_parts2(g.part, 1, 2, sh, rr, dd);
    if (threadIdx.x == 0) {
      Scal* s = g.s;
      s->ticket = 0;
      s->rr = rr;
      s->dd = dd;
      s->it += 1;
      s->restart = s->sw = 0;  // the last iteration's, carried out by its preconditioner halves
      bool done;
      if (s->a32) {
        const double tb = sqrt(s->tol2 * s->bb), e = s->lo_norm * sqrt(dd);
        if (e > 0.5 * tb) {
          s->a32 = 0;
          s->restart = 1;
          s->no_switch = 1;
          s->restarts += 1;
          done = false;
        } else {
          done = sqrt(rr) + e <= tb;
        }
      } else {
        done = rr <= s->tol2 * s->bb;
        // switch to Ah once |r| is as small as a step that starts on Ah needs its r0 to be
        if (!done && g.a32_mode == 1 && !s->no_switch && s->rho >= 0.0 &&
            s->lo_norm * s->rho * sqrt(rr) * kA32Margin <= sqrt(s->tol2 * s->bb)) {
          s->a32 = 1;
          s->sw = 1;
          s->dd_pre = dd;
          s->switched += 1;
        }
      }
      if (!done && s->it >= s->max_it) {
        if (!s->status) s->status = SC_NOT_CONVERGED;
        done = true;
      }
      if (s->status == SC_BREAKDOWN) done = true;
      if (done) pcg_continue<kMode>(hc, s, false);
    }
  }
}

// u = up + dt^2/4 x ; v = vp + dt/2 x ; a into the history ring (k_advance moves its head)
__global__ void k_finalize(Args g) {
  const double dt = g.dt, h = 0.5 * dt, qq = 0.25 * dt * dt;
  double* __restrict__ slot = g.ah[hist_slot(g.s->head, kHistMax - 1)];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n_s; i += (int64_t)gridDim.x * blockDim.x) {
    const double x = g.x[i], ai = g.a[i], vi = g.v[i];
    const double up = g.u[i] + dt * vi + qq * ai;
    const double vp = vi + h * ai;
    g.u[i] = fma(qq, x, up);
    g.v[i] = fma(h, x, vp);
    slot[i] = ai;
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

__global__ void k_cap_hist(Scal* s, int n) {
  if (s->hist > n) s->hist = n;
}

__global__ void k_advance(Args g) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    Scal* s = g.s;
    s->total_iters += s->it;
    if (s->it > s->max_seen) s->max_seen = s->it;
    s->t += 1;
    if (s->res_fp64_next) s->res_fp64 = 1;  // the next step's predictor and residual see it
    // |x - x0| over the whole step (across a switch: the two legs' lengths added)
    const double dx = sqrt(s->dd_pre) + sqrt(s->dd);
    if (s->rr0 > 0.0 && dx > 0.0) s->rho = dx / sqrt(s->rr0);
    s->a32 = 0;
    warm_start_advance(s, g.pred_order);
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

// FSAI planes: permuted into the sliced-ELL order and rounded to FP16 after scaling by a
// power of two (CG is invariant under scaling the preconditioner; the power of two keeps the
// iterates' bits and keeps every entry inside FP16's range whatever the units)
__global__ void k_sell_permute_half(int planes, int64_t n_out, int64_t n_in, const int64_t* src, const float* in,
                                    __half* out, float scale) {
  for (int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pos < n_out;
       pos += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = src[pos];
    for (int c = 0; c < planes; ++c)
      out[(int64_t)c * n_out + pos] = __float2half_rn(k >= 0 ? scale * in[(int64_t)c * n_in + k] : 0.f);
  }
}

// largest |x| (as the bits of a non-negative float, which order like the values)
__global__ void k_absmax_bits(int64_t n, const float* __restrict__ x, unsigned* out) {
  unsigned m = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float a = fabsf(x[i]);
    if (a <= 3.0e38f) m = max(m, __float_as_uint(a));  // finite values only
  }
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
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
  s->res_fp64 = s->res_fp64_next = 0;
  s->a32 = s->restart = s->sw = s->no_switch = 0;
  s->lo_norm = 0.0;
  s->rr0 = s->dd = s->dd_pre = 0.0;
  s->rho = -1.0;
  s->a32_steps = s->switched = s->restarts = 0;
  warm_start_init(s);
}

}  // namespace nb
}  // namespace sc

using namespace sc;
using namespace sc::nb;


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
    k_predict<D><<<h->pred_blocks, D * kPredNodes, 0, cs>>>(g);
    if (g.res_pair) {
      if (g.keep_l2) k_residual_kp<D, 1><<<nbk, kThreads, 0, cs>>>(g);
      else k_residual_kp<D, 0><<<nbk, kThreads, 0, cs>>>(g);
      k_residual<D, true><<<nbk, kThreads, 0, cs>>>(g, 1);
    } else if (g.spmv_pair) {
      k_residual<D, true><<<nbk, kThreads, 0, cs>>>(g, 0);
    } else {
      k_residual<D, false><<<nbk, kThreads, 0, cs>>>(g, 0);
    }
    launch_prec_lower<D>(g, nbk, cs);
    launch_prec_upper<D, 0>(g, nbk, cs, 1, hc);
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
    if (g.spmv_pair) {
      launch_spmv_pair<D, 0>(g, nbk, c2, hc);
      launch_spmv_a32<D, 0>(g, nbk, c2, hc);
    }
    else k_spmv<D, 0><<<nbk, kThreads, 0, c2>>>(g, hc);
    k_update<0><<<vbk, 256, 0, c2>>>(g, hc);
    launch_prec_lower<D>(g, nbk, c2);
    launch_prec_upper<D, 0>(g, nbk, c2, 0, hc);
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
namespace {

void drop_graph(sc_nb_newmark* h) {
  if (h->exec) cudaGraphExecDestroy(h->exec), h->exec = nullptr;
  if (h->graph) cudaGraphDestroy(h->graph), h->graph = nullptr;
}

}  // namespace


// Sliced-ELL copies of K, A, M (full pattern), G (lower) and G^T (upper) for the per-step
// kernels; allocated here (setup) from the stream-ordered pool and freed by sc_nb_destroy.
// lo_norm = sqrt(||Al||_1 ||Al||_inf) >= ||Al||_2 for Al = A - Ah, the lo parts of the pair
// planes: each row's sum of |lo| (largest kept by an atomic max on the bits of a non-negative
// double, which order like the values) and each column's (atomic adds into colsum)
template <int D>
__global__ void k_lo_sums(Args g, double* colsum, unsigned long long* rowmax) {
  SELL_ROW_LOOP(g.sf_ptr) {
    SELL_ROW_BEGIN(g.sf_ptr)
    double rs[D];
#pragma unroll
    for (int c = 0; c < D; ++c) rs[c] = 0.0;
    for (int64_t q = 0; q < nq; ++q) {
      const int64_t pos = p0 + 128 * q;
      int cl[4];
      cols4(g.sf_col, pos, cl, 1);
#pragma unroll
      for (int c = 0; c < D; ++c)
#pragma unroll
        for (int d = 0; d < D; ++d)
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const double lo = fabs((double)g.APS[(int64_t)(c * D + d) * g.sf_n + pos + e].y);
            if (lo > 0.0) {
              rs[c] += lo;
              atomicAdd(colsum + (int64_t)cl[e] * D + d, lo);
            }
          }
    }
    if (row < g.n_nodes) {
      double m = 0.0;
#pragma unroll
      for (int c = 0; c < D; ++c) m = fmax(m, rs[c]);
      atomicMax(rowmax, (unsigned long long)__double_as_longlong(m));
    }
  }
}

__global__ void k_col_max(int64_t n, const double* colsum, unsigned long long* colmax) {
  double m = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmax(m, colsum[i]);
  atomicMax(colmax, (unsigned long long)__double_as_longlong(m));
}

__global__ void k_lo_norm(const unsigned long long* mx, Scal* s) {
  s->lo_norm = sqrt(__longlong_as_double((long long)mx[0]) * __longlong_as_double((long long)mx[1]));
}

static int lo_norm(sc_nb_newmark* h) {
  Args& g = h->g;
  cudaStream_t st = h->user;
  double* colsum = nullptr;
  unsigned long long* mx = nullptr;
  int rc = check(cudaMallocAsync((void**)&colsum, 8 * g.n_s, st), "malloc");
  if (rc) return rc;
  if ((rc = check(cudaMallocAsync((void**)&mx, 16, st), "malloc"))) {
    cudaFreeAsync(colsum, st);
    return rc;
  }
  cudaMemsetAsync(colsum, 0, 8 * g.n_s, st);
  cudaMemsetAsync(mx, 0, 16, st);
  if (g.D == 3) k_lo_sums<3><<<h->node_blocks, kThreads, 0, st>>>(g, colsum, mx);
  else k_lo_sums<2><<<h->node_blocks, kThreads, 0, st>>>(g, colsum, mx);
  k_col_max<<<grid_for(g.n_s, 256, 152 * 8), 256, 0, st>>>(g.n_s, colsum, mx + 1);
  k_lo_norm<<<1, 1, 0, st>>>(mx, g.s);
  rc = check_launch("lo norm");
  cudaFreeAsync(colsum, st);
  cudaFreeAsync(mx, st);
  return rc;
}

static int build_sell(sc_nb_newmark* h, const double* KB, const double* AB, const double* MS, const float* GB,
                      const float* GTB, float gscale) {
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
      float* ah = nullptr;
      if ((rc = alloc((void**)&ap, 8 * D2 * total))) break;
      if ((rc = alloc((void**)&ah, 4 * D2 * total))) break;
      k_split_pairs<<<pb, 256, 0, st>>>((int64_t)D2 * total, as, ap);
      k_hi_parts<<<pb, 256, 0, st>>>((int64_t)D2 * total, ap, ah);
      g.sf_ptr = ptr; g.sf_col = col; g.sf_n = total; g.KS = ks; g.AS = as; g.MSS = ms;
      g.APS = ap;
      g.AHS = ah;
    } else {
      __half* gs = nullptr;
      if ((rc = alloc((void**)&gs, 2 * D2 * total))) break;
      k_sell_permute_half<<<pb, 256, 0, st>>>(D2, total, g.nnzb, src, kind == 1 ? GB : GTB, gs, gscale);
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
  b += (kHistMax + 12) * align256(8 * ns);    // history ah[kHistMax], q1 q2 y1 x0 x r z p w f, p2, r0
  b += 3 * align256(4 * ns);                  // t32, r32, r032
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
  for (int k = 0; k < kHistMax; ++k) g.ah[k] = (double*)take(8 * ns);
  g.pred_order = 0;  // adaptive
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
  g.r32 = (float*)take(4 * ns);
  g.r0 = (double*)take(8 * ns);
  g.r032 = (float*)take(4 * ns);
  g.a32_mode = 1;
  g.order_cap = 1;
  g.part = (double*)take(8 * 4 * 152 * 16);
  g.s = (Scal*)take(sizeof(Scal));
  h->node_blocks = node_grid(n_nodes);
  h->tpr = n_nodes >= 150000 ? 1 : (n_nodes >= 60000 ? 2 : 4);
  {
    const int64_t want = (((int64_t)n_nodes + 31) / 32 * 32 * h->tpr + kThreads - 1) / kThreads;
    h->tpr_blocks = (unsigned)(want < 152 * 16 ? (want < 1 ? 1 : want) : 152 * 16);
  }
  h->vec_blocks = grid_for(ns, 256, 152 * 16);
  h->pred_blocks = grid_for(n_nodes, kPredNodes, 152 * 16);
  cudaStream_t st = h->user;
  int rc = SC_OK;
  int* dflag = nullptr;
  do {
    if ((rc = check(cudaStreamCreateWithFlags(&h->cap, cudaStreamNonBlocking), "stream"))) break;
    if ((rc = check(cudaStreamCreateWithFlags(&h->cap2, cudaStreamNonBlocking), "stream"))) break;
    if ((rc = check(cudaMallocAsync((void**)&dflag, 3 * sizeof(int), st), "malloc"))) break;
    cudaMemsetAsync(dflag, 0, 3 * sizeof(int), st);
    cudaMemsetAsync(g.f, 0, 8 * ns, st);
    for (int k = 0; k < kHistMax; ++k) cudaMemsetAsync(g.ah[k], 0, 8 * ns, st);
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
    k_absmax_bits<<<grid_for((int64_t)D2 * nnzb, 256, 152 * 8), 256, 0, st>>>((int64_t)D2 * nnzb, GB,
                                                                               (unsigned*)(dflag + 2));
    if ((rc = check_launch("nb setup"))) break;
    unsigned gmax_bits = 0;
    if ((rc = check(cudaMemcpyAsync(&gmax_bits, dflag + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, st), "memcpy")))
      break;
    if ((rc = check(cudaStreamSynchronize(st), "sync"))) break;
    float gmax = 0.f;
    memcpy(&gmax, &gmax_bits, sizeof(float));
    // the power of two that brings the largest FSAI entry into [0.5, 1)
    const float gscale = gmax > 0.f ? ldexpf(1.f, -(ilogbf(gmax) + 1)) : 1.f;
    if ((rc = build_sell(h, KB, AB, MS, GB, GTB, gscale))) break;
    if ((rc = lo_norm(h))) break;
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

// Polynomial order (1..kHistMax; 0: adaptive, the default) of the extrapolated accelerations
// that start each step's PCG: it changes the iteration count, not the converged answer.
extern "C" int sc_nb_set_predictor(sc_nb_newmark* h, int order) {
  if (!h || order < 0 || order > kHistMax) return SC_BAD_ARG;
  // only the previous fixed order's entries of the history are current (adaptive keeps all)
  if (h->g.pred_order > 0 && (order == 0 || order > h->g.pred_order))
    k_cap_hist<<<1, 1, 0, h->user>>>(h->g.s, h->g.pred_order);
  h->g.pred_order = order;
  drop_graph(h);
  return check_launch("predictor order");
}

extern "C" int sc_nb_set_options(sc_nb_newmark* h, int options) {
  if (!h || options < 0 || options > 63 || (options & 24) == 24) return SC_BAD_ARG;
  h->g.spmv_pair = (options & 1) ? 0 : 1;
  h->explicit_pair = (options & 2) ? 0 : 1;
  h->res_pair = (options & 4) ? 0 : 1;
  h->g.a32_mode = !h->g.spmv_pair || (options & 8) ? 0 : ((options & 16) ? 2 : 1);
  h->g.order_cap = (options & 32) ? 0 : 1;
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
// acceleration history once steps of this solver have filled it.
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
  k_predict<D><<<h->pred_blocks, D * kPredNodes, 0, st>>>(g);
  if (g.res_pair) {
    if (g.keep_l2) k_residual_kp<D, 1><<<nbk, kThreads, 0, st>>>(g);
    else k_residual_kp<D, 0><<<nbk, kThreads, 0, st>>>(g);
    k_residual<D, true><<<nbk, kThreads, 0, st>>>(g, 1);
  } else if (g.spmv_pair) {
    k_residual<D, true><<<nbk, kThreads, 0, st>>>(g, 0);
  } else {
    k_residual<D, false><<<nbk, kThreads, 0, st>>>(g, 0);
  }
  launch_prec_lower<D>(g, nbk, st);
  launch_prec_upper<D, 1>(g, nbk, st, 1, none);
  int done = 0;
  int rc;
  for (int guard = 0; guard < 100000; ++guard) {
    if ((rc = check(cudaMemcpyAsync(&done, &g.s->done, sizeof(int), cudaMemcpyDeviceToHost, st), "read done")))
      return rc;
    if ((rc = check(cudaStreamSynchronize(st), "sync eager"))) return rc;
    if (done) break;
    if (g.spmv_pair) {
      launch_spmv_pair<D, 1>(g, nbk, st, none);
      launch_spmv_a32<D, 1>(g, nbk, st, none);
    }
    else k_spmv<D, 1><<<nbk, kThreads, 0, st>>>(g, none);
    k_update<1><<<vbk, 256, 0, st>>>(g, none);
    launch_prec_lower<D>(g, nbk, st);
    launch_prec_upper<D, 1>(g, nbk, st, 0, none);
  }
  k_finalize<<<vbk, 256, 0, st>>>(g);
  k_record<<<vbk, 256, 0, st>>>(g);
  k_advance<<<1, 32, 0, st>>>(g);
  return check_launch("eager step");
}

// The pair residual's planes and vectors, made on first use: K as pairs (shared with the explicit
// scheme), the mass plane as pairs, the per-node records and zc.  It runs with the pair SpMV only.
static int residual_prepare(sc_nb_newmark* h) {
  Args& g = h->g;
  const int want = h->res_pair && g.spmv_pair ? 1 : 0;
  if (want == g.res_pair && (!want || h->res_mem[0])) return SC_OK;
  g.res_pair = 0;
  if (!want) return SC_OK;
  cudaStream_t st = h->user;
  const int64_t ns = g.n_s, n2 = (int64_t)g.D * g.D * g.sf_n;
  int rc;
  auto M = [&](void** p, size_t b) { return check(cudaMallocAsync(p, b, st), "residual malloc"); };
  if (!h->KPS) {
    if ((rc = M((void**)&h->KPS, 8 * n2))) return rc;
    k_split_pairs<<<grid_for(n2, 256, 152 * 32), 256, 0, st>>>(n2, g.KS, h->KPS);
  }
  g.KPS = h->KPS;
  if (!h->res_mem[0]) {
    const size_t sizes[3] = {(size_t)(8 * g.sf_n), (size_t)(4 * (int64_t)g.n_nodes * kRecFloats(g.D)),
                             (size_t)(8 * ns)};
    for (int k = 0; k < 3; ++k)
      if ((rc = M(&h->res_mem[k], sizes[k]))) return rc;
    k_split_pairs<<<grid_for(g.sf_n, 256, 152 * 32), 256, 0, st>>>(g.sf_n, g.MSS, (float2*)h->res_mem[0]);
    cudaMemsetAsync(h->res_mem[1], 0, sizes[1], st);  // the records' pad floats
  }
  g.MSP = (const float2*)h->res_mem[0];
  g.rrec = (float*)h->res_mem[1];
  g.zc = (double*)h->res_mem[2];
  g.res_pair = 1;
  drop_graph(h);
  return check_launch("residual prepare");
}

extern "C" int sc_nb_run(sc_nb_newmark* h, int t_begin, int t_end) {
  if (!h || t_begin < 0 || t_end < t_begin) return SC_BAD_ARG;
  int rc;
  if ((rc = residual_prepare(h))) return rc;
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

__global__ void k_status3(const Scal* s, int64_t* out) {
  out[0] = s->status;
  out[1] = s->total_iters;
  out[2] = s->max_seen;
}

// the run's status, total iterations and largest per-step count into dev3 (device, 3 int64),
// queued on the solver's stream behind its steps: no synchronisation
extern "C" int sc_nb_status_to(sc_nb_newmark* h, int64_t* dev3) {
  if (!h || !dev3) return SC_BAD_ARG;
  k_status3<<<1, 1, 0, h->user>>>(h->g.s, dev3);
  return check_launch("status copy");
}

extern "C" int sc_nb_a32_status(sc_nb_newmark* h, int64_t* a32_steps, int64_t* switched, int64_t* restarts,
                                double* lo_norm) {
  if (!h) return SC_BAD_ARG;
  Scal s;
  int rc = check(cudaStreamSynchronize(h->user), "sync");
  if (rc) return rc;
  if ((rc = check(cudaMemcpy(&s, h->g.s, sizeof(s), cudaMemcpyDeviceToHost), "read"))) return rc;
  if (a32_steps) *a32_steps = s.a32_steps;
  if (switched) *switched = s.switched;
  if (restarts) *restarts = s.restarts;
  if (lo_norm) *lo_norm = s.lo_norm;
  return SC_OK;
}

extern "C" int sc_nb_warm_start_status(sc_nb_newmark* h, int* order, int64_t* capped_steps) {
  if (!h) return SC_BAD_ARG;
  Scal s;
  int rc = check(cudaStreamSynchronize(h->user), "sync");
  if (rc) return rc;
  if ((rc = check(cudaMemcpy(&s, h->g.s, sizeof(s), cudaMemcpyDeviceToHost), "read"))) return rc;
  if (order) *order = h->g.pred_order > 0 ? h->g.pred_order : s.pord;
  if (capped_steps) *capped_steps = s.capped;
  return SC_OK;
}

extern "C" int sc_nb_time_spmv(sc_nb_newmark* h, int reps, float* ms_per_launch, int64_t* bytes_per_launch) {
  return sc_nb_time_spmv_a32(h, 0, reps, ms_per_launch, bytes_per_launch);
}

extern "C" int sc_nb_time_spmv_a32(sc_nb_newmark* h, int a32, int reps, float* ms_per_launch,
                                   int64_t* bytes_per_launch) {
  if (!h || reps <= 0 || !ms_per_launch || (a32 != 0 && a32 != 1)) return SC_BAD_ARG;
  if (a32 && !h->g.spmv_pair) return SC_BAD_ARG;
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
      if (a32) {
        if (h->g.D == 3) launch_spmv_a32<3, 2>(h->g, nbk, st, none);
        else launch_spmv_a32<2, 2>(h->g, nbk, st, none);
      } else {
        if (h->g.D == 3) launch_spmv_pair<3, 2>(h->g, nbk, st, none);
        else launch_spmv_pair<2, 2>(h->g, nbk, st, none);
      }
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
    // A blocks (4 B per value for the FP32 matrix) + block columns + row pointers + one read of p
    // + the write of w
    *bytes_per_launch = h->g.nnzb * ((a32 ? 4 : 8) * D2 + 4) + (int64_t)(h->g.n_slices + 1) * 8 + h->g.n_s * 16;
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

__global__ void k_copy_r(int64_t n, int D, const double* __restrict__ x, double* __restrict__ r,
                         float* __restrict__ r32) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    r[i] = x[i];
    r32[i] = (float)x[i];
  }
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
      k_copy_r<<<grid_for(g.n_s, 256), 256, 0, st>>>(g.n_s, g.D, x, g.r, g.r32);
      if (g.D == 3) {
        launch_prec_lower<3, false>(g, h->node_blocks, st);
        k_prec_upper_nograph<3><<<h->node_blocks, kThreads, 0, st>>>(g);
      } else {
        launch_prec_lower<2, false>(g, h->node_blocks, st);
        k_prec_upper_nograph<2><<<h->node_blocks, kThreads, 0, st>>>(g);
      }
      k_copy<<<grid_for(g.n_s, 256), 256, 0, st>>>(g.n_s, g.z, y);
      break;
    }
  }
  int rc = check_launch("nb apply");
  if (!rc) rc = check(cudaStreamSynchronize(st), "sync apply");
  return rc;
}

extern "C" int sc_nb_residual_fp64(sc_nb_newmark* h, int* fp64) {
  if (!h || !fp64) return SC_BAD_ARG;
  int rc = check(cudaStreamSynchronize(h->user), "sync");
  if (rc) return rc;
  Scal s;
  if ((rc = check(cudaMemcpy(&s, h->g.s, sizeof(s), cudaMemcpyDeviceToHost), "read"))) return rc;
  *fp64 = h->g.res_pair ? s.res_fp64 : 1;
  return SC_OK;
}

extern "C" int sc_nb_destroy(sc_nb_newmark* h) {
  if (!h) return SC_OK;
  drop_graph(h);
  drop_explicit_graphs(h);
  for (int i = 0; i < h->n_sell_mem; ++i) cudaFree(h->sell_mem[i]);
  cudaStreamSynchronize(h->user);
  for (void* q : h->res_mem)
    if (q) cudaFree(q);
  free_explicit(h);
  if (h->cap) cudaStreamDestroy(h->cap);
  if (h->cap2) cudaStreamDestroy(h->cap2);
  delete h;
  return SC_OK;
}
