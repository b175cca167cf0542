// Shared helpers for the scatter_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/scatter_gb300.h"

namespace sc {

constexpr int kWarp = 32;

// Records the last CUDA error text for sc_last_error().
void set_last_error(const char* where, cudaError_t e);
// Records a message (no CUDA error) for sc_last_error().
void set_last_message(const char* text);

inline int check_launch(const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(where, e);
    return SC_CUDA_ERROR;
  }
  return SC_OK;
}

inline int check(cudaError_t e, const char* where) {
  if (e != cudaSuccess) {
    set_last_error(where, e);
    return SC_CUDA_ERROR;
  }
  return SC_OK;
}

inline unsigned grid_for(int64_t n, int threads, int64_t cap = 152 * 64) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (unsigned)b;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of one double per thread (blockDim.x multiple of 32, <= 1024).
// Result valid in thread 0.  `sh` has at least 32 doubles.
__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    s = lane < nw ? sh[lane] : 0.0;
    s = warp_sum(s);
  }
  return s;
}

// Block-wide sums of two doubles per thread in one pass (each summed in the same order as
// block_sum would, so the results are the same bits).  Results valid in thread 0.  `sh` has at
// least 64 doubles.
__device__ __forceinline__ void block_sum2(double& a, double& b, double* sh) {
  a = warp_sum(a);
  b = warp_sum(b);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) {
    sh[wid] = a;
    sh[32 + wid] = b;
  }
  __syncthreads();
  double sa = 0.0, sb = 0.0;
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    sa = lane < nw ? sh[lane] : 0.0;
    sb = lane < nw ? sh[32 + lane] : 0.0;
    sa = warp_sum(sa);
    sb = warp_sum(sb);
  }
  a = sa;
  b = sb;
}

// ------------------------------------------------ warm start of the per-step PCG (Newmark)
// Both Newmark solvers start each step's PCG from the polynomial of degree p through the last
// p+1 accelerations, evaluated one step ahead: x0 = sum_{k=0..p} (-1)^k C(p+1, k+1) a_{n-k}
// (p = 0: a_n; p = 2: 3a_n - 3a_{n-1} + a_{n-2}).  The order only changes the iteration
// count, not the converged answer.
constexpr int kHistMax = 8;  // acceleration history kept for the warm start
// order control (fixed order 0 = adaptive): start at kPredStart, then compare the mean PCG
// iterations of windows of kPredWin steps, keep climbing while a probed neighbour order is
// better, step back when it is worse and hold there kPredHold windows
constexpr int kPredStart = 6, kPredWin = 16, kPredHold = 8;

// cf[k] = (-1)^k C(p+1, k+1) for k <= p, 0 beyond: exact integers, in a fixed order
__device__ __forceinline__ void warm_start_coeffs(int p, double* cf) {
  long long c = p + 1;
  cf[0] = (double)c;
#pragma unroll
  for (int k = 1; k <= kHistMax; ++k) {
    if (k <= p) c = c * (p + 1 - k) / (k + 1);
    cf[k] = k <= p ? ((k & 1) ? -(double)c : (double)c) : 0.0;
  }
}

// The controller's state lives in each solver's scalar block S, which has the int fields
// hist, head, pord, pdir, win_n, win_it, probing, hold, it and the double ref_avg.
template <class S>
__device__ __forceinline__ int warm_start_order(const S* s, int fixed) {
  const int ord = fixed > 0 ? fixed : s->pord;
  return s->hist < ord ? s->hist : ord;
}

// The history is a ring of kHistMax vectors: a_{n-1-k} sits in slot (head + k) mod kHistMax,
// and a step writes its outgoing acceleration into slot head - 1 and moves head there (one
// write per step instead of shifting the whole history).
static_assert((kHistMax & (kHistMax - 1)) == 0, "the history ring's index wraps with a mask");
__device__ __forceinline__ int hist_slot(int head, int k) { return (head + k) & (kHistMax - 1); }

// The warm start's order cap.  The accelerations respond to the load at once, so a window of
// past accelerations that straddles a kink in the load history (the end of a ramp, a load that
// starts to move, a point load that moves onto another face) extrapolates badly, and a lower
// order whose window lies after the kink does better (at the benchmark workload, the steps
// after a 5-step ramp took 15, 14, 12, 10, 8, 6 PCG iterations at orders 1..5 against 18, 19,
// 19, 18, 17, 15 at order 6).  So each step takes the largest order q <= the controller's order
// whose extrapolation of the force itself reproduces, to kCapTol of the rows' largest entry,
// the force of the newest row from the q + 1 rows before it.  One block (the force kernel's);
// each distinct index of the rows is summed by the thread holding its first entry, rows in a
// fixed order (deterministic); windows whose rows hold more than kCapRow entries keep the order.
constexpr double kCapTol = 1e-6;
constexpr int kCapRow = 256;

// the force table: rows 0..n_t-1, row t's entries ptr[t] .. ptr[t+1]-1 at indices idx, values val
struct ForceRows {
  int n_t;
  const int64_t* ptr;
  const int* idx;
  const double* val;
};

// rows r0 .. r0 + nr - 1 of a force table staged in shared memory (the cap reads them many times)
constexpr int kCapStage = 2048;
struct CapRows {
  int r0, nr;
  const int* ptr;  // nr + 1 offsets into idx / val
  const int* idx;
  const double* val;
  __device__ int find(int row, int i) const {
    if (row < r0 || row >= r0 + nr) return -1;
    for (int e = ptr[row - r0]; e < ptr[row - r0 + 1]; ++e)
      if (idx[e] == i) return e;
    return -1;
  }
};

// max |f_{m+1} - sum_{k<=q} cf[k] f_{m-k}| / max |f| over those rows (0 when they hold no force),
// in thread 0
__device__ inline double cap_misfit(const CapRows& F, int q, int m, const double* cf) {
  __shared__ double mx[2][32];
  double rmx = 0.0, fmx = 0.0;
  for (int j = 0; j <= q + 1; ++j) {  // rows in the order m+1, m, m-1, ..., m-q
    const int row = m + 1 - j;
    if (row < F.r0 || row >= F.r0 + F.nr) continue;
    for (int e = F.ptr[row - F.r0] + threadIdx.x; e < F.ptr[row - F.r0 + 1]; e += blockDim.x) {
      const int i = F.idx[e];
      fmx = fmax(fmx, fabs(F.val[e]));
      bool first = true;
      for (int k = 0; k < j && first; ++k) first = F.find(m + 1 - k, i) < 0;
      if (!first) continue;
      double r = 0.0;
      for (int k = 0; k <= q + 1; ++k) {
        const int h = k == j ? e : F.find(m + 1 - k, i);
        if (h >= 0) r += (k == 0 ? 1.0 : -cf[k - 1]) * F.val[h];
      }
      rmx = fmax(rmx, fabs(r));
    }
  }
  // block maxima (order-independent, so the cap is deterministic)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    rmx = fmax(rmx, __shfl_xor_sync(0xffffffffu, rmx, o));
    fmx = fmax(fmx, __shfl_xor_sync(0xffffffffu, fmx, o));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) {
    mx[0][wid] = rmx;
    mx[1][wid] = fmx;
  }
  __syncthreads();
  double r = 0.0, f = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      r = fmax(r, mx[0][w]);
      f = fmax(f, mx[1][w]);
    }
  return f > 0.0 ? r / f : 0.0;
}

// sets s->pcap for step s->t (counting in s->capped the steps it lowers); all threads of the
// block call it.  The window's rows t-p .. t+1 are staged in shared memory first; a window of
// more than kCapStage entries, or a row of more than kCapRow, keeps the order.
template <class S>
__device__ void warm_start_order_cap(S* s, int fixed, int enabled, const ForceRows& F) {
  __shared__ int cap_s;
  __shared__ int s_ptr[kHistMax + 3];
  __shared__ int s_idx[kCapStage];
  __shared__ double s_val[kCapStage];
  const int t = s->t;
  const int p = warm_start_order(s, fixed);
  int cap = p;
  const int r0 = t - p < 0 ? 0 : t - p, r1 = t + 1 < F.n_t - 1 ? t + 1 : F.n_t - 1;  // rows r0..r1
  const int nr = r1 >= r0 ? r1 - r0 + 1 : 0;
  bool small = enabled && F.ptr && p > 0;
  if (small && nr > 0) {
    for (int row = r0; row <= r1; ++row)
      if (F.ptr[row + 1] - F.ptr[row] > kCapRow) small = false;
    if (small && F.ptr[r1 + 1] - F.ptr[r0] > kCapStage) small = false;
  }
  if (small) {
    const int64_t base = nr > 0 ? F.ptr[r0] : 0;
    if (threadIdx.x <= nr) s_ptr[threadIdx.x] = nr > 0 ? (int)(F.ptr[r0 + threadIdx.x] - base) : 0;
    const int n = nr > 0 ? (int)(F.ptr[r1 + 1] - base) : 0;
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
      s_idx[e] = F.idx[base + e];
      s_val[e] = F.val[base + e];
    }
    __syncthreads();
    const CapRows C{r0, nr, s_ptr, s_idx, s_val};
    double cf[kHistMax + 1];
    for (cap = p; cap > 0; --cap) {
      warm_start_coeffs(cap, cf);
      const double e1 = cap_misfit(C, cap, t, cf);
      if (threadIdx.x == 0) cap_s = e1 <= kCapTol ? 1 : 0;
      __syncthreads();
      const int ok = cap_s;
      __syncthreads();
      if (ok) break;
    }
  }
  if (threadIdx.x == 0) {
    s->pcap = cap;
    if (cap < p) s->capped += 1;
  }
}

template <class S>
__device__ inline void warm_start_init(S* s) {
  s->hist = 0;
  s->head = 0;
  s->pcap = kHistMax;
  s->capped = 0;
  s->pord = kPredStart;
  s->pdir = 1;
  s->win_n = s->win_it = s->probing = s->hold = 0;
  s->ref_avg = 0.0;
}

// After a step (one thread): one more history entry, and the step's iterations (s->it) into
// the adaptive order's window.
template <class S>
__device__ inline void warm_start_advance(S* s, int fixed) {
  if (s->hist < kHistMax) s->hist += 1;
  s->head = hist_slot(s->head, kHistMax - 1);  // the slot k_finalize just wrote
  if (fixed > 0) return;
  if (++s->win_n < kPredWin) {
    s->win_it += s->it;
    return;
  }
  // the window just ended: its mean iterations per step
  const double avg = (double)(s->win_it + s->it) / kPredWin;
  s->win_n = 0;
  s->win_it = 0;
  if (s->probing) {
    if (avg <= s->ref_avg) {  // the probed order is no worse: keep it, probe further
      s->ref_avg = avg;
      const int np = s->pord + s->pdir;
      if (np >= 1 && np <= kHistMax) {
        s->pord = np;
      } else {
        s->probing = 0;
        s->pdir = -s->pdir;
        s->hold = kPredHold;
      }
    } else {  // worse: back to the better order, hold, probe the other side next
      s->pord -= s->pdir;
      s->pdir = -s->pdir;
      s->probing = 0;
      s->hold = kPredHold;
    }
  } else if (s->hold > 0) {
    s->hold -= 1;
  } else {  // this window is the reference: probe the neighbour in the current direction
    s->ref_avg = avg;
    const int np = s->pord + s->pdir;
    if (np >= 1 && np <= kHistMax) {
      s->pord = np;
      s->probing = 1;
    } else {
      s->pdir = -s->pdir;
    }
  }
}

// (hi, lo) FP32 pair of a double: hi + lo reproduces x to 48 bits
__device__ inline float2 split_pair(double x) {
  const float hi = (float)x;
  return make_float2(hi, (float)(x - (double)hi));
}

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

}  // namespace sc
