// Batched explicit scheme: R realisations of the per-element Young's modulus advanced
// together, one kernel per step, FP32 stiffness products with FP64 state accumulators.
//
// Physics per realisation r is the explicit lumped-mass scheme of sc_nbsolver.cu
// (k_explicit) with K_r = sum_e E_{e,r} K1_e (K1_e: element stiffness at E = 1, which is
// what scatter/discretisation.py:177-201 gives for D(E=1, nu)), density and Poisson ratio
// shared, and the Lysmer terms of scatter/system_matrix.py:362-376 scaled per realisation:
// rho v_p, rho v_s grow as sqrt(E) (dashpots), E_c and G as E (springs).
//
// Layout: every per-realisation array is [slot or element][R] (realisation fastest).  A node
// is handled by ceil(R / RPT) threads, each owning RPT consecutive realisations: the node's
// incident elements are walked once, each K1 entry (the same for every realisation, a
// broadcast load) feeds RPT FMAs, and w, E, u, v are read as 8- to 32-byte vectors.  The
// accumulators u and v are FP32 (hi, lo) pairs (about 48 significant bits) updated in place
// (own node only): the step has no FP64 instruction, which on GB300 runs at 1/64 of the FP32
// rate; the caller's FP64 u, v are converted in at the start of a run and out at its end.
// w = u + beta v and v are also kept as FP32 ping-pong copies that neighbours read.  RPT and the nodes per block come from a short
// timing of the candidates on scratch copies of the state when the handle is created.
#include <utility>
#include <vector>

#include "sc_common.cuh"

struct sc_batch_desc {
  int n_nodes, n_elem, n_en, R, n_types;
  const int *elem, *inc_ptr, *inc, *ke_type;
  const float *ke1, *young;
  const double* ml;
  const int* fixed;
  double alpha, beta, dt;
  const int64_t* l_ptr;
  const int *l_col, *l_elem;
  const float *l_c, *l_s;
  const unsigned char* node_nen;  // mixed element types: nodes per element of each node's mesh (NULL: all n_en)
};

namespace sc {
namespace bt {

struct Args {
  sc_batch_desc d;
  double *u, *v;        // the caller's FP64 state (converted at run start and end)
  float2 *u2, *v2;      // the accumulators as (hi, lo) pairs, [slot][R]
  const float *ml32, *iml32;  // lumped mass and its reciprocal, FP32
  float dth, dtl, alpha32, beta32;  // dt as a pair; Rayleigh coefficients
  double* f;    // dense force, slot space (shared by the realisations)
  float* f32;   // its FP32 copy, what the update reads (kept by the force swap)
  int* t;     // device step counter
  int n_t;
  const int64_t* f_ptr;
  const int* f_slot;
  const double* f_val;
  int n_rec, out_interval;
  const int* rec_map;  // slot -> receiver index or -1
  double* out_v;       // [n_out][n_rec][R]
  int64_t n_out;
  unsigned* ticket;    // blocks finished in the current launch (last-block detection)
  const unsigned char* vneed;  // slot -> 1 when a Lysmer row reads its velocity (FP32 copy kept)
};

template <int RPT>
__device__ __forceinline__ void ldf(const float* p, float (&v)[RPT]) {
  if constexpr (RPT % 4 == 0) {
#pragma unroll
    for (int q = 0; q < RPT / 4; ++q) {
      const float4 a = __ldg(reinterpret_cast<const float4*>(p) + q);
      v[4 * q] = a.x; v[4 * q + 1] = a.y; v[4 * q + 2] = a.z; v[4 * q + 3] = a.w;
    }
  } else if constexpr (RPT == 2) {
    const float2 a = __ldg(reinterpret_cast<const float2*>(p));
    v[0] = a.x; v[1] = a.y;
  } else {
#pragma unroll
    for (int q = 0; q < RPT; ++q) v[q] = __ldg(p + q);
  }
}
// ldf with the L1 eviction priority "last": the neighbours' w, read by up to 27 nodes' threads
template <int RPT>
__device__ __forceinline__ void ldf_keep(const float* p, float (&v)[RPT]) {
  if constexpr (RPT % 4 == 0) {
#pragma unroll
    for (int q = 0; q < RPT / 4; ++q) {
      float4 a;
      asm("ld.global.nc.L1::evict_last.v4.f32 {%0, %1, %2, %3}, [%4];"
          : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w)
          : "l"(reinterpret_cast<const float4*>(p) + q));
      v[4 * q] = a.x; v[4 * q + 1] = a.y; v[4 * q + 2] = a.z; v[4 * q + 3] = a.w;
    }
  } else if constexpr (RPT == 2) {
    float2 a;
    asm("ld.global.nc.L1::evict_last.v2.f32 {%0, %1}, [%2];" : "=f"(a.x), "=f"(a.y) : "l"(p));
    v[0] = a.x; v[1] = a.y;
  } else {
    ldf<RPT>(p, v);
  }
}

template <int RPT>
__device__ __forceinline__ void stf(float* p, const float (&v)[RPT]) {
  if constexpr (RPT % 4 == 0) {
#pragma unroll
    for (int q = 0; q < RPT / 4; ++q)
      reinterpret_cast<float4*>(p)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
  } else if constexpr (RPT == 2) {
    *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
  } else {
#pragma unroll
    for (int q = 0; q < RPT; ++q) p[q] = v[q];
  }
}
template <int RPT>
__device__ __forceinline__ void ldp(const float2* p, float2 (&v)[RPT]) {
  if constexpr (RPT % 2 == 0) {
#pragma unroll
    for (int q = 0; q < RPT / 2; ++q) {
      const float4 a = reinterpret_cast<const float4*>(p)[q];
      v[2 * q] = make_float2(a.x, a.y);
      v[2 * q + 1] = make_float2(a.z, a.w);
    }
  } else {
#pragma unroll
    for (int q = 0; q < RPT; ++q) v[q] = p[q];
  }
}
template <int RPT>
__device__ __forceinline__ void stp(float2* p, const float2 (&v)[RPT]) {
  if constexpr (RPT % 2 == 0) {
#pragma unroll
    for (int q = 0; q < RPT / 2; ++q)
      reinterpret_cast<float4*>(p)[q] = make_float4(v[2 * q].x, v[2 * q].y, v[2 * q + 1].x, v[2 * q + 1].y);
  } else {
#pragma unroll
    for (int q = 0; q < RPT; ++q) p[q] = v[q];
  }
}

// x += a b + extra for a (hi, lo) pair x: the product split exactly with fmaf, the sum's
// rounding error kept by two-sum, then renormalised (extra is below a b's last bit)
__device__ __forceinline__ void pair_madd(float2& x, float a, float b, float extra) {
  const float p = __fmul_rn(a, b);
  const float pe = fmaf(a, b, -p);
  const float t = __fadd_rn(x.x, p);
  const float bp = __fsub_rn(t, x.x);
  const float e = __fadd_rn(__fsub_rn(x.x, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  const float lo = __fadd_rn(x.y, __fadd_rn(e, __fadd_rn(pe, extra)));
  const float h = __fadd_rn(t, lo);
  x = make_float2(h, __fsub_rn(lo, __fsub_rn(h, t)));
}

// t += k2 w2, then k1 w1, then k0 w0, per realisation; pairs of realisations use the paired
// FP32 FMA (two independently rounded FMAs in one instruction: the same values as fmaf, half
// the issue slots)
template <int RPT>
__device__ __forceinline__ void fma3(float (&t)[RPT], float k0, float k1, float k2, const float (&w0)[RPT],
                                     const float (&w1)[RPT], const float (&w2)[RPT]) {
  if constexpr (RPT % 2 == 0) {
    const float2 K0 = make_float2(k0, k0), K1 = make_float2(k1, k1), K2 = make_float2(k2, k2);
#pragma unroll
    for (int r = 0; r < RPT; r += 2) {
      float2 x = make_float2(t[r], t[r + 1]);
      x = __ffma2_rn(K2, make_float2(w2[r], w2[r + 1]), x);
      x = __ffma2_rn(K1, make_float2(w1[r], w1[r + 1]), x);
      x = __ffma2_rn(K0, make_float2(w0[r], w0[r + 1]), x);
      t[r] = x.x;
      t[r + 1] = x.y;
    }
  } else {
#pragma unroll
    for (int r = 0; r < RPT; ++r) t[r] = fmaf(k0, w0[r], fmaf(k1, w1[r], fmaf(k2, w2[r], t[r])));
  }
}

// acc += E t per realisation (paired as above)
template <int RPT>
__device__ __forceinline__ void fma1(float (&acc)[RPT], const float (&E)[RPT], const float (&t)[RPT]) {
  if constexpr (RPT % 2 == 0) {
#pragma unroll
    for (int r = 0; r < RPT; r += 2) {
      const float2 x = __ffma2_rn(make_float2(E[r], E[r + 1]), make_float2(t[r], t[r + 1]),
                                  make_float2(acc[r], acc[r + 1]));
      acc[r] = x.x;
      acc[r + 1] = x.y;
    }
  } else {
#pragma unroll
    for (int r = 0; r < RPT; ++r) acc[r] = fmaf(E[r], t[r], acc[r]);
  }
}

__device__ inline bool batch_last_block(unsigned* ticket) {
  __shared__ bool am_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) am_last = (atomicAdd(ticket, 1u) == gridDim.x * gridDim.y - 1);
  __syncthreads();
  return am_last;
}

// Stiffness forces on node a for RPT realisations: sum over the node's incident elements of
// E_e K1_e(a, :) w_e.  Element connectivity rows have `estride` entries and K1 tables rows of
// `kstride` (3 NEN for a single element type; the largest type's for mixed meshes).
template <int NEN, int RPT>
__device__ __forceinline__ void node_forces(const Args& g, const float* __restrict__ w_in, int a, int r0, int estride,
                                            int kstride, float (&acc)[3][RPT]) {
  const sc_batch_desc& d = g.d;
  const int R = d.R;
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < RPT; ++r) acc[c][r] = 0.f;
  for (int k = d.inc_ptr[a]; k < d.inc_ptr[a + 1]; ++k) {
    const int e = d.inc[k];
    const int* en = d.elem + (int64_t)e * estride;
    int la = 0;
#pragma unroll
    for (int q = 0; q < NEN; ++q)
      if (en[q] == a) la = q;
    const float* K1 = d.ke1 + (int64_t)d.ke_type[e] * kstride * kstride + (int64_t)(la * 3) * kstride;
    float t[3][RPT];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int r = 0; r < RPT; ++r) t[c][r] = 0.f;
#pragma unroll 2
    for (int lb = 0; lb < NEN; ++lb) {
      const int64_t bs = (int64_t)en[lb] * 3;
      float w0[RPT], w1[RPT], w2[RPT];
      ldf<RPT>(w_in + (bs + 0) * R + r0, w0);
      ldf<RPT>(w_in + (bs + 1) * R + r0, w1);
      ldf<RPT>(w_in + (bs + 2) * R + r0, w2);
      const float* kr = K1 + lb * 3;
#pragma unroll
      for (int c = 0; c < 3; ++c)
        fma3<RPT>(t[c], __ldg(kr + c * kstride + 0), __ldg(kr + c * kstride + 1), __ldg(kr + c * kstride + 2), w0,
                  w1, w2);
    }
    float Ee[RPT];
    ldf<RPT>(d.young + (int64_t)e * R + r0, Ee);
#pragma unroll
    for (int c = 0; c < 3; ++c) fma1<RPT>(acc[c], Ee, t[c]);
  }
}

// The update of node a's DOFs for RPT realisations (Lysmer terms, FP32 acceleration, pair
// accumulators, FP32 copies, receivers)
template <int RPT>
__device__ __forceinline__ void node_update(const Args& g, int a, int r0, const float (&acc)[3][RPT],
                                            const float* __restrict__ w_in, float* __restrict__ w_out,
                                            const float* __restrict__ vf_in, float* __restrict__ vf_out, int step,
                                            bool rec_now) {
  const sc_batch_desc& d = g.d;
  const int R = d.R;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int64_t i = (int64_t)a * 3 + c;
    const int64_t ir = i * R + r0;
    float wo[RPT], vo[RPT];
    if (d.fixed[i]) {
#pragma unroll
      for (int r = 0; r < RPT; ++r) wo[r] = vo[r] = 0.f;
      stf<RPT>(w_out + ir, wo);
      if (g.vneed[i]) stf<RPT>(vf_out + ir, vo);
      continue;
    }
    float spring[RPT], dash[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r) spring[r] = dash[r] = 0.f;
    for (int64_t q = d.l_ptr[i]; q < d.l_ptr[i + 1]; ++q) {
      const int64_t jr = (int64_t)d.l_col[q] * R + r0;
      float Eq[RPT], wj[RPT], vj[RPT];
      ldf<RPT>(d.young + (int64_t)d.l_elem[q] * R + r0, Eq);
      ldf<RPT>(w_in + jr, wj);
      ldf<RPT>(vf_in + jr, vj);
      const float ls = d.l_s[q], lc = d.l_c[q];
#pragma unroll
      for (int r = 0; r < RPT; ++r) {
        spring[r] = fmaf(__fmul_rn(ls, Eq[r]), wj[r], spring[r]);
        dash[r] = fmaf(__fmul_rn(lc, sqrtf(Eq[r])), vj[r], dash[r]);
      }
    }
    float2 vp[RPT], up[RPT];
    ldp<RPT>(g.v2 + ir, vp);
    ldp<RPT>(g.u2 + ir, up);
    const float fi = g.f32[i], mlf = g.ml32[i], imlf = g.iml32[i];
    const float aml = __fmul_rn(g.alpha32, mlf);
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      // FP32 acceleration (its inputs are FP32 products); _rn intrinsics keep the rounding
      // the same for every kernel shape
      const float kw = __fadd_rn(acc[c][r], spring[r]);
      // own velocity: the pair's hi part, which is what the FP32 copy holds
      const float num = __fsub_rn(__fsub_rn(__fsub_rn(fi, kw), __fmul_rn(aml, vp[r].x)), dash[r]);
      const float accel = __fmul_rn(num, imlf);
      pair_madd(vp[r], g.dth, accel, __fmul_rn(g.dtl, accel));                           // v += dt a
      pair_madd(up[r], g.dth, vp[r].x, fmaf(g.dth, vp[r].y, __fmul_rn(g.dtl, vp[r].x)));  // u += dt v
      wo[r] = fmaf(g.beta32, vp[r].x, up[r].x);
      vo[r] = vp[r].x;
    }
    stp<RPT>(g.v2 + ir, vp);
    stp<RPT>(g.u2 + ir, up);
    stf<RPT>(w_out + ir, wo);
    if (g.vneed[i]) stf<RPT>(vf_out + ir, vo);
    if (rec_now) {
      const int rj = g.rec_map[i];
      if (rj >= 0) {
        double* o = g.out_v + ((int64_t)(step / g.out_interval) * g.n_rec + rj) * R + r0;
#pragma unroll
        for (int r = 0; r < RPT; ++r) o[r] = (double)vp[r].x + (double)vp[r].y;
      }
    }
  }
}

// The last block to finish advances the step counter and swaps the force entries in f from
// step t to step t + 1 (every block has read f by then).
__device__ __forceinline__ void step_epilogue(const Args& g, int step) {
  if (batch_last_block(g.ticket)) {
    const int t = step - 1;
    if (g.f_ptr) {
      if (t >= 0 && t < g.n_t)
        for (int64_t k = g.f_ptr[t] + threadIdx.x; k < g.f_ptr[t + 1]; k += blockDim.x) {
          g.f[g.f_slot[k]] = 0.0;
          g.f32[g.f_slot[k]] = 0.f;
        }
      __syncthreads();
      if (t + 1 < g.n_t) {
        for (int64_t k = g.f_ptr[t + 1] + threadIdx.x; k < g.f_ptr[t + 2]; k += blockDim.x) g.f[g.f_slot[k]] += g.f_val[k];
        __syncthreads();
        for (int64_t k = g.f_ptr[t + 1] + threadIdx.x; k < g.f_ptr[t + 2]; k += blockDim.x)
          g.f32[g.f_slot[k]] = (float)g.f[g.f_slot[k]];
      }
    }
    if (threadIdx.x == 0) {
      *g.ticket = 0;
      *g.t = step;
    }
  }
}

__device__ __forceinline__ bool record_now(const Args& g, int step) {
  return g.n_rec > 0 && g.out_interval > 0 && step % g.out_interval == 0 && step / g.out_interval < g.n_out;
}

// One step for all realisations.  tpn threads per node (tpn * RPT >= R), blockDim / tpn
// nodes per block.
template <int NEN, int RPT>
__global__ void __launch_bounds__(256) k_batch_step(Args g, const float* __restrict__ w_in, float* __restrict__ w_out,
                                                    const float* __restrict__ vf_in, float* __restrict__ vf_out,
                                                    int tpn) {
  const int npb = blockDim.x / tpn;
  const int sub = threadIdx.x / tpn;
  const int r0 = (threadIdx.x % tpn) * RPT;
  const bool active = sub < npb && r0 < g.d.R;
  const int step = *g.t + 1;
  const bool rec_now = record_now(g, step);
  for (int a = blockIdx.x * npb + sub; active && a < g.d.n_nodes; a += gridDim.x * npb) {
    float acc[3][RPT];
    node_forces<NEN, RPT>(g, w_in, a, r0, NEN, 3 * NEN, acc);
    node_update<RPT>(g, a, r0, acc, w_in, w_out, vf_in, vf_out, step, rec_now);
  }
  step_epilogue(g, step);
}

// Mixed element types (independent meshes of different types concatenated, one realisation):
// one thread per node, the node's mesh type selecting the element loop.  Connectivity rows
// and K1 tables use the largest type's stride.
__global__ void __launch_bounds__(256) k_batch_step_mixed(Args g, const float* __restrict__ w_in,
                                                          float* __restrict__ w_out, const float* __restrict__ vf_in,
                                                          float* __restrict__ vf_out) {
  const int step = *g.t + 1;
  const bool rec_now = record_now(g, step);
  const int es = g.d.n_en, ks = 3 * g.d.n_en;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < g.d.n_nodes; a += gridDim.x * blockDim.x) {
    float acc[3][1];
    switch (g.d.node_nen[a]) {
      case 4: node_forces<4, 1>(g, w_in, a, 0, es, ks, acc); break;
      case 8: node_forces<8, 1>(g, w_in, a, 0, es, ks, acc); break;
      case 10: node_forces<10, 1>(g, w_in, a, 0, es, ks, acc); break;
      default: node_forces<20, 1>(g, w_in, a, 0, es, ks, acc); break;
    }
    node_update<1>(g, a, 0, acc, w_in, w_out, vf_in, vf_out, step, rec_now);
  }
  step_epilogue(g, step);
}

// ------------------------------------------------------------------ uniform hexa8 grids
// Meshes of one hexa8 element shape on a structured node lattice: lattice coordinates along
// the elements' natural axes (xi, eta, zeta), an element's local node l at its first node's
// lattice point plus the natural offset of l.  The lattice is cut into tiles of kTX x kTY x
// kTZ points; halo [tile][kHN] lists the nodes of the tile grown by one point on every side
// (-1 where the lattice has no node), point (hx, hy, hz) at hx + kHX (hy + kHY hz); elem8
// [node][8] the element in which the node is local node la (-1 where none).  A block takes
// one tile and 32 RPT consecutive realisations: it stages the halo's w in shared memory with
// coalesced loads (about 4.5 loads per owned node where the incidence-list kernel gathers 64
// node vectors), then a warp per owned node reads its 27 neighbours at fixed offsets into
// registers, and the unit-E stiffness is a kernel parameter, so every FMA takes its K1 entry
// from the constant bank.  Elements are visited in local-index order with the FMA sequence
// of node_forces, which visits incidence lists sorted the same way: the results are bitwise
// those of the incidence-list kernel.
constexpr int kTX = 4, kTY = 4, kTZ = 2;
constexpr int kHX = kTX + 2, kHY = kTY + 2, kHZ = kTZ + 2, kHN = kHX * kHY * kHZ;

struct K1Hex8 {
  float k[576];  // [3 la + c][3 lb + comp]
};

__host__ __device__ constexpr int hex8_nat(int l, int axis) {  // natural coordinate of local node l, 0 or 1
  return axis == 0 ? ((l == 1 || l == 2 || l == 5 || l == 6) ? 1 : 0)
                   : (axis == 1 ? ((l == 2 || l == 3 || l == 6 || l == 7) ? 1 : 0) : (l >= 4 ? 1 : 0));
}
// 27-neighbour index (dxi + 1) + 3 (deta + 1) + 9 (dzeta + 1) of lb seen from la, and the halo
// offset of neighbour q
__host__ __device__ constexpr int hex8_q(int la, int lb) {
  return (hex8_nat(lb, 0) - hex8_nat(la, 0) + 1) + 3 * (hex8_nat(lb, 1) - hex8_nat(la, 1) + 1) +
         9 * (hex8_nat(lb, 2) - hex8_nat(la, 2) + 1);
}
__host__ __device__ constexpr int q_off(int q) { return (q % 3 - 1) + kHX * ((q / 3) % 3 - 1 + kHY * (q / 9 - 1)); }

template <int RPT>
__device__ __forceinline__ void lds_f(const float* p, float (&v)[RPT]) {
  if constexpr (RPT == 2) {
    const float2 a = *reinterpret_cast<const float2*>(p);
    v[0] = a.x;
    v[1] = a.y;
  } else {
#pragma unroll
    for (int q = 0; q < RPT; ++q) v[q] = p[q];
  }
}

// One step for all realisations on a uniform hexa8 grid, node-centric like k_batch_step (tpn
// threads per node, RPT realisations each).  elem8 gives the node's incident elements with its
// local index la known at compile time, so every K1 entry is a constant-bank operand of its
// FMAs (k1 is a kernel parameter): per node the loads are the 8 elements' node lists (the same
// for the whole warp), their w as RPT-vectors and E, against 576 RPT FMAs.  k_batch_step instead
// loads each K1 entry it uses (576 per node and thread).  The elements are taken in la order and
// the products in the same order as there, so the results are bitwise the same.
template <int RPT>
__device__ __forceinline__ void hex8c_step(const Args& g, const K1Hex8& k1, const int* __restrict__ elem8,
                                           const float* __restrict__ w_in, float* __restrict__ w_out,
                                           const float* __restrict__ vf_in, float* __restrict__ vf_out, int tpn) {
  const int npb = blockDim.x / tpn;
  const int sub = threadIdx.x / tpn;
  const int r0 = (threadIdx.x % tpn) * RPT;
  const bool active = sub < npb && r0 < g.d.R;
  const int step = *g.t + 1;
  const bool rec_now = record_now(g, step);
  const int R = g.d.R;
  for (int a = blockIdx.x * npb + sub; active && a < g.d.n_nodes; a += gridDim.x * npb) {
    float acc[3][RPT];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int r = 0; r < RPT; ++r) acc[c][r] = 0.f;
#pragma unroll
    for (int la = 0; la < 8; ++la) {
      const int e = __ldg(elem8 + (int64_t)a * 8 + la);
      if (e < 0) continue;
      const int* en = g.d.elem + (int64_t)e * 8;
      float t[3][RPT];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < RPT; ++r) t[c][r] = 0.f;
#pragma unroll
      for (int lb = 0; lb < 8; ++lb) {
        const int64_t bs = (int64_t)__ldg(en + lb) * 3;
        float w0[RPT], w1[RPT], w2[RPT];
        ldf_keep<RPT>(w_in + (bs + 0) * R + r0, w0);
        ldf_keep<RPT>(w_in + (bs + 1) * R + r0, w1);
        ldf_keep<RPT>(w_in + (bs + 2) * R + r0, w2);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float* kr = k1.k + (3 * la + c) * 24 + 3 * lb;
          fma3<RPT>(t[c], kr[0], kr[1], kr[2], w0, w1, w2);
        }
      }
      float Ee[RPT];
      ldf<RPT>(g.d.young + (int64_t)e * R + r0, Ee);
#pragma unroll
      for (int c = 0; c < 3; ++c) fma1<RPT>(acc[c], Ee, t[c]);
    }
    node_update<RPT>(g, a, r0, acc, w_in, w_out, vf_in, vf_out, step, rec_now);
  }
  step_epilogue(g, step);
}

// the node-centric step at the compiler's default register budget (64 at 256 threads) and at a
// wide one (one block per SM minimum: 79 registers at 2 realisations per thread, 144 at 4);
// both are tuner candidates
template <int RPT>
__global__ void __launch_bounds__(256) k_batch_step_hex8c(Args g, const __grid_constant__ K1Hex8 k1,
                                                         const int* __restrict__ elem8, const float* __restrict__ w_in,
                                                         float* __restrict__ w_out, const float* __restrict__ vf_in,
                                                         float* __restrict__ vf_out, int tpn) {
  hex8c_step<RPT>(g, k1, elem8, w_in, w_out, vf_in, vf_out, tpn);
}
template <int RPT>
__global__ void __launch_bounds__(256, 1) k_batch_step_hex8c_wide(Args g, const __grid_constant__ K1Hex8 k1,
                                                                 const int* __restrict__ elem8,
                                                                 const float* __restrict__ w_in,
                                                                 float* __restrict__ w_out,
                                                                 const float* __restrict__ vf_in,
                                                                 float* __restrict__ vf_out, int tpn) {
  hex8c_step<RPT>(g, k1, elem8, w_in, w_out, vf_in, vf_out, tpn);
}

// One step for all realisations on a uniform hexa8 grid: grid (tiles, realisation chunks of
// 32 RPT), dynamic shared memory kHN * 3 * 32 RPT floats.
template <int RPT>
__global__ void __launch_bounds__(256) k_batch_step_hex8g(Args g, const __grid_constant__ K1Hex8 k1,
                                                         const int* __restrict__ halo, const int* __restrict__ elem8,
                                                         const float* __restrict__ w_in, float* __restrict__ w_out,
                                                         const float* __restrict__ vf_in, float* __restrict__ vf_out) {
  extern __shared__ __align__(16) float sw[];  // [kHN][3][RC]
  constexpr int RC = 32 * RPT;
  const int R = g.d.R;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int* ht = halo + (int64_t)blockIdx.x * kHN;
  const int r0 = blockIdx.y * RC + lane * RPT;
  const int step = *g.t + 1;
  const bool rec_now = record_now(g, step);
  // the halo's w for this chunk staged by asynchronous copies (zeros where there is no node
  // and beyond R): 16-byte pieces when rows are 16-byte aligned (R % 4 == 0), else 4-byte
  const int rc0 = blockIdx.y * RC;
  const unsigned sbase = (unsigned)__cvta_generic_to_shared(sw);
  if (R % 4 == 0) {
    constexpr int PR = RC / 4;  // pieces per row
    for (int pc = threadIdx.x; pc < kHN * 3 * PR; pc += blockDim.x) {
      const int row = pc / PR, k = pc - row * PR;
      const int node = __ldg(ht + row / 3), r = rc0 + 4 * k;
      const int bytes = node < 0 || r >= R ? 0 : (R - r >= 4 ? 16 : 4 * (R - r));
      const float* src = bytes ? w_in + ((int64_t)node * 3 + row % 3) * R + r : w_in;
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sbase + 4u * (row * RC + 4 * k)),
                   "l"(src), "r"(bytes));
    }
  } else {
    for (int pc = threadIdx.x; pc < kHN * 3 * RC; pc += blockDim.x) {
      const int row = pc / RC, k = pc - row * RC;
      const int node = __ldg(ht + row / 3), r = rc0 + k;
      const int bytes = node < 0 || r >= R ? 0 : 4;
      const float* src = bytes ? w_in + ((int64_t)node * 3 + row % 3) * R + r : w_in;
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sbase + 4u * (row * RC + k)), "l"(src),
                   "r"(bytes));
    }
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncthreads();
  if (r0 < R) {
    for (int n = warp; n < kTX * kTY * kTZ; n += nw) {
      const int hb = (n % kTX + 1) + kHX * ((n / kTX) % kTY + 1 + kHY * (n / (kTX * kTY) + 1));
      const int a = __ldg(ht + hb);
      if (a < 0) continue;
      // the node's pair state into L2 ahead of its update, and its elements' E
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int64_t ir = ((int64_t)a * 3 + c) * R + r0;
        asm volatile("prefetch.global.L2 [%0];" ::"l"(__cvta_generic_to_global(g.u2 + ir)));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(__cvta_generic_to_global(g.v2 + ir)));
      }
      int el[8];
      float Eall[8][RPT];
#pragma unroll
      for (int la = 0; la < 8; ++la) el[la] = __ldg(elem8 + (int64_t)a * 8 + la);
#pragma unroll
      for (int la = 0; la < 8; ++la) {
        if (el[la] >= 0) {
          ldf<RPT>(g.d.young + (int64_t)el[la] * R + r0, Eall[la]);
        } else {
#pragma unroll
          for (int r = 0; r < RPT; ++r) Eall[la][r] = 0.f;
        }
      }
      const float* sb = sw + hb * 3 * RC + lane * RPT;
      float wv[27][3][RPT];
#pragma unroll
      for (int q = 0; q < 27; ++q)
#pragma unroll
        for (int c = 0; c < 3; ++c) lds_f<RPT>(sb + (q_off(q) * 3 + c) * RC, wv[q][c]);
      float acc[3][RPT];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < RPT; ++r) acc[c][r] = 0.f;
#pragma unroll
      for (int la = 0; la < 8; ++la) {
        if (el[la] < 0) continue;
        float t[3][RPT];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int r = 0; r < RPT; ++r) t[c][r] = 0.f;
#pragma unroll
        for (int lb = 0; lb < 8; ++lb) {
          const int q = hex8_q(la, lb);
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const int kb = (la * 3 + c) * 24 + lb * 3;
            fma3<RPT>(t[c], k1.k[kb], k1.k[kb + 1], k1.k[kb + 2], wv[q][0], wv[q][1], wv[q][2]);
          }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) fma1<RPT>(acc[c], Eall[la], t[c]);
      }
      node_update<RPT>(g, a, r0, acc, w_in, w_out, vf_in, vf_out, step, rec_now);
    }
  }
  step_epilogue(g, step);
}

// ------------------------------------------------------------------ tensor-core step (uniform hexa8 grids)
// The element products on the 5th-generation tensor cores.  Per element e and 128 realisations
// (one CTA of 128 threads, thread t = realisation r0 + t = TMEM lane t):
//   D[r, j] = sum_k W[r, k] K1[j, k]           (K1: the unit-E 24 x 24 element stiffness)
//   f_node(j)[r] += E_e[r] D[r, j]             (FP32, CUDA cores)
// W (the element's 24 w values per realisation) is written into tensor memory by the threads
// (tcgen05.st), K1 sits in shared memory (K-major, no swizzle), D accumulates in tensor memory
// and is read back with tcgen05.ld.  TF32 keeps 11 significant bits, so W and K1 are split into
// hi = rna_tf32(x) and lo = x - hi and D takes the three products hi hi + hi lo + lo hi
// (tcgen05.mma kind::tf32, M = 128, N = 32 with 8 zero columns, K = 3 x 8): the dropped lo lo
// term and the lo parts' own TF32 rounding leave about 2^-21 of each product.
//
// Decomposition: the lattice (the hexa8 grid tables of hex8_grid_tables) is cut into columns
// of kCX x kCY points across the first two lattice axes, each column into segments along the
// third (the sweep axis).  A CTA owns one segment of one column for one group of 128
// realisations and sweeps it layer by layer: element layer k (between point planes k and k + 1)
// has kCEX x kCEY element positions touching the owned points; their forces on owned points are
// added to shared-memory accumulators of planes k and k + 1 (each thread its own realisation's
// column, so no two threads touch the same word); after layer k, plane k is complete and its
// owned nodes are updated (node_update, as in the other kernels).  Elements on the ring are
// computed by both neighbouring columns (25 element positions per 16 owned points).
// The ring planes of w are copied into shared memory by asynchronous bulk copies (512 bytes
// per node and DOF, completing on one barrier per plane slot), three slots deep: layer k reads
// planes k and k + 1 while plane k + 2 arrives.  The update state of the plane finished by the
// layer is prefetched into L2 when the layer starts.  The element loop is software-pipelined
// over two TMEM buffers: element i's W is staged and its MMAs issued before element i - 1's D is
// read back.  Waits on barriers are bounded: after kTcSpin tries a thread records the failure,
// the CTA leaves its sweep at the next layer, frees its tensor memory and sets *err.
constexpr int kCX = 4, kCY = 4, kCP = kCX * kCY;
constexpr int kCHX = kCX + 2, kCHY = kCY + 2, kCHN = kCHX * kCHY;  // the ring plane: 6 x 6 points
constexpr int kCEX = kCX + 1, kCEY = kCY + 1, kCEN = kCEX * kCEY;  // element positions per layer: 5 x 5
constexpr int kTcThreads = 128;
constexpr uint32_t kTcCols = 256;  // A buffers at columns 0 and 64 (hi +0, lo +32), D buffers at 128 and 160
constexpr uint32_t kTcIdesc = (1u << 4)             // D: FP32
                              | (2u << 7)            // A: TF32
                              | (2u << 10)           // B: TF32
                              | ((32u >> 3) << 17)   // N = 32
                              | ((128u >> 4) << 24);  // M = 128
constexpr int kTcSpin = 1 << 22;
constexpr int kPlaneFloats = kCHN * 3 * kTcThreads;    // one ring plane of w: [point][dof][realisation]
constexpr int kAccFloats = kCP * 3 * kTcThreads;       // one plane of force accumulators: [point][dof][realisation]
constexpr size_t kTcSmem = sizeof(float) * (3 * kPlaneFloats + 2 * kAccFloats);  // 215,040 bytes

struct TcTables {
  const int* nodes;  // [n_col][nzp][kCHN]: node at ring point (hx, hy) of plane z, -1 where none
  const int* elems;  // [n_col][nzp - 1][kCEN]: element whose local node 0 is at ring point (ex, ey) of layer z
  int nzp, seg, n_segs;
  int* err;          // set when a barrier wait gives up
};

// local node l of the element at position P: ring point, plane (0: k, 1: k + 1) and owned point
// (-1 when outside the owned 4 x 4), packed as ring | plane << 8 | (owned + 1) << 9
struct TcPos {
  short code[kCEN][8];
};
__host__ __device__ constexpr TcPos tc_positions() {
  TcPos t{};
  for (int P = 0; P < kCEN; ++P)
    for (int l = 0; l < 8; ++l) {
      const int hx = P % kCEX + hex8_nat(l, 0), hy = P / kCEX + hex8_nat(l, 1), hz = hex8_nat(l, 2);
      const bool owned = hx >= 1 && hx <= kCX && hy >= 1 && hy <= kCY;
      const int p = owned ? (hy - 1) * kCX + (hx - 1) : -1;
      t.code[P][l] = (short)((hy * kCHX + hx) | (hz << 8) | ((p + 1) << 9));
    }
  return t;
}
__constant__ TcPos c_tc_pos = tc_positions();

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start, leading (K direction) and stride (M/N direction) byte
// offsets, the fixed version bit, no swizzle
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t h;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
  return __uint_as_float(h);
}

__device__ __forceinline__ void tc_st8(uint32_t taddr, const float* v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
               "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]));
}

__device__ __forceinline__ void tc_ld24(uint32_t taddr, float* d) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3]), "=f"(d[4]), "=f"(d[5]), "=f"(d[6]), "=f"(d[7]), "=f"(d[8]),
        "=f"(d[9]), "=f"(d[10]), "=f"(d[11]), "=f"(d[12]), "=f"(d[13]), "=f"(d[14]), "=f"(d[15])
      : "r"(taddr));
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=f"(d[16]), "=f"(d[17]), "=f"(d[18]), "=f"(d[19]), "=f"(d[20]), "=f"(d[21]), "=f"(d[22]), "=f"(d[23])
               : "r"(taddr + 16));
  // the registers are valid only after the wait: tie them to it so no use moves above it
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3]), "+f"(d[4]), "+f"(d[5]), "+f"(d[6]), "+f"(d[7]),
                 "+f"(d[8]), "+f"(d[9]), "+f"(d[10]), "+f"(d[11]), "+f"(d[12]), "+f"(d[13]), "+f"(d[14]), "+f"(d[15]),
                 "+f"(d[16]), "+f"(d[17]), "+f"(d[18]), "+f"(d[19]), "+f"(d[20]), "+f"(d[21]), "+f"(d[22]), "+f"(d[23])
               :
               : "memory");
}

__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity) {
  for (int it = 0; it < kTcSpin; ++it) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tc_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// plane z of the column's ring into plane slot `dst` (one thread): one 512-byte bulk copy per
// node and DOF, completing on `mbar`
__device__ __forceinline__ void tc_load_plane(const int* __restrict__ ring_nodes, const float* __restrict__ w_in,
                                              int R, int r0, float* dst, uint32_t mbar) {
  uint32_t bytes = 0;
  for (int i = 0; i < kCHN; ++i) bytes += ring_nodes[i] >= 0 ? 3u * 512u : 0u;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
  for (int i = 0; i < kCHN; ++i) {
    const int node = ring_nodes[i];
    if (node < 0) continue;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float* src = w_in + ((int64_t)node * 3 + c) * R + r0;
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], 512, [%2];" ::"r"(
              smem_addr(dst + (i * 3 + c) * kTcThreads)),
          "l"(src), "r"(mbar)
          : "memory");
    }
  }
}

__global__ void __launch_bounds__(kTcThreads, 1) k_batch_step_tc(Args g, const __grid_constant__ K1Hex8 k1,
                                                                 TcTables tt, const float* __restrict__ w_in,
                                                                 float* __restrict__ w_out,
                                                                 const float* __restrict__ vf_in,
                                                                 float* __restrict__ vf_out) {
  extern __shared__ __align__(1024) float tc_dyn[];  // 3 ring planes of w, then 2 planes of accumulators
  __shared__ __align__(1024) float sB[2 * 3 * 256];  // K1 hi then lo: 3 K-slices of 32 (N) x 8 (K), 1 KB each
  __shared__ int s_nodes[2 * kCHN];                   // ring planes k and k + 1 (node indices)
  __shared__ int s_elems[kCEN];
  __shared__ uint32_t s_tmem;
  __shared__ int s_fail;
  __shared__ __align__(8) uint64_t s_mbar[2];   // MMA completion, per TMEM buffer
  __shared__ __align__(8) uint64_t s_pbar[3];   // plane arrival, per plane slot
  float* planes = tc_dyn;
  float* accs = tc_dyn + 3 * kPlaneFloats;
  const int t = threadIdx.x;
  const int R = g.d.R;
  const int r0 = blockIdx.y * kTcThreads, r = r0 + t;
  const int col = blockIdx.x / tt.n_segs, sg = blockIdx.x - col * tt.n_segs;
  const int step = *g.t + 1;
  const bool rec_now = record_now(g, step);
  const int* col_nodes = tt.nodes + (int64_t)col * tt.nzp * kCHN;
  const int* col_elems = tt.elems + (int64_t)col * (tt.nzp - 1) * kCEN;
  const int z0 = sg * tt.seg, z1 = min(z0 + tt.seg, tt.nzp);
  const int kbeg = max(z0 - 1, 0), kend = min(z1, tt.nzp - 1);
  // K1 into the canonical K-major layout: element (k, n) of slice k / 8 at
  // (n / 8) 256 + (k % 8 / 4) 128 + (n % 8) 16 + (k % 4) 4 bytes; B[k][n] = K1[n][k], zero for n >= 24
  for (int i = t; i < 24 * 32; i += kTcThreads) {
    const int k = i >> 5, n = i & 31, kk = k & 7;
    const int off = (k >> 3) * 256 + (n >> 3) * 64 + (kk >> 2) * 32 + (n & 7) * 4 + (kk & 3);
    const float b = n < 24 ? k1.k[n * 24 + k] : 0.f;
    const float bh = tf32_hi(b);
    sB[off] = bh;
    sB[3 * 256 + off] = b - bh;
  }
  for (int i = t; i < 2 * kAccFloats; i += kTcThreads) accs[i] = 0.f;
  if (t < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&s_tmem)),
                 "r"(kTcCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  const uint32_t mbar0 = smem_addr(&s_mbar[0]), pbar0 = smem_addr(&s_pbar[0]);
  if (t == 0) {
    s_fail = 0;
    for (int q = 0; q < 2; ++q) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar0 + 8 * q));
    for (int q = 0; q < 3; ++q) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(pbar0 + 8 * q));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_sync();
  const uint32_t tmem = s_tmem, sb = smem_addr(sB);
  const uint32_t lane_base = (uint32_t)(t & ~31) << 16;  // this warp's TMEM lane quadrant
  uint32_t mpar = 0, ppar = 0;                          // parity bits of the MMA and plane barriers
  bool ok = true;
  // what thread 0 started and what this thread has waited for (a failure exit drains the rest)
  int n_commit[2] = {0, 0}, n_mwait[2] = {0, 0}, last_loaded = kbeg + 1, last_waited = kbeg - 1;
  // planes kbeg and kbeg + 1 start arriving
  if (t == 0) {
    for (int z = kbeg; z <= kbeg + 1; ++z)
      tc_load_plane(col_nodes + (int64_t)z * kCHN, w_in, R, r0, planes + (z % 3) * kPlaneFloats, pbar0 + 8 * (z % 3));
  }
  int cur = 0;  // accumulator plane of point plane k (the other one is k + 1)
  for (int k = kbeg; k < kend; ++k) {
    __syncthreads();  // the previous layer's readers of s_nodes, s_elems and plane slot (k - 1) % 3 are done
    if (s_fail) break;
    for (int i = t; i < 2 * kCHN + kCEN; i += kTcThreads) {
      if (i < 2 * kCHN) s_nodes[i] = col_nodes[(int64_t)k * kCHN + i];
      else s_elems[i - 2 * kCHN] = col_elems[(int64_t)k * kCEN + (i - 2 * kCHN)];
    }
    if (k + 2 <= kend) {  // the next layer's upper plane, into the slot plane k - 1 used
      if (t == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_load_plane(col_nodes + (int64_t)(k + 2) * kCHN, w_in, R, r0, planes + ((k + 2) % 3) * kPlaneFloats,
                      pbar0 + 8 * ((k + 2) % 3));
      }
      last_loaded = k + 2;
    }
    __syncthreads();
    // the update state of plane k into L2 while the layer computes (two lanes per warp cover a
    // warp's 256 bytes of pairs)
    if (k >= z0 && (t & 15) == 0) {
      for (int p = 0; p < kCP; ++p) {
        const int a = s_nodes[(p / kCX + 1) * kCHX + (p % kCX) + 1];
        if (a < 0) continue;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const int64_t ir = ((int64_t)a * 3 + c) * R + r;
          asm volatile("prefetch.global.L2 [%0];" ::"l"(g.u2 + ir));
          asm volatile("prefetch.global.L2 [%0];" ::"l"(g.v2 + ir));
        }
      }
    }
    // planes k and k + 1 present (plane k was waited for in the previous layer, except the first)
    for (int z = (k == kbeg ? k : k + 1); z <= k + 1 && ok; ++z) {
      const int slot = z % 3;
      ok = tc_wait(pbar0 + 8 * slot, (ppar >> slot) & 1);
      ppar ^= 1u << slot;
      last_waited = z;
      if (!ok) s_fail = 1;
    }
    const float* pl[2] = {planes + (k % 3) * kPlaneFloats + t, planes + ((k + 1) % 3) * kPlaneFloats + t};
    float* acc[2] = {accs + cur * kAccFloats + t, accs + (cur ^ 1) * kAccFloats + t};
    float E_prev = 0.f;
    for (int P = 0; P <= kCEN; ++P) {
      const int e = P < kCEN ? s_elems[P] : -1;
      const uint32_t b = P & 1;
      float E = 0.f;
      if (e >= 0) {
        const short* code = c_tc_pos.code[P];
        float hi[8], lo[8];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int kk = 8 * q + j, l = kk / 3, c = kk % 3;
            const int cd = code[l];
            const float x = pl[(cd >> 8) & 1][((cd & 255) * 3 + c) * kTcThreads];
            hi[j] = tf32_hi(x);
            lo[j] = x - hi[j];
          }
          tc_st8(tmem + lane_base + b * 64 + 8 * q, hi);
          tc_st8(tmem + lane_base + b * 64 + 32 + 8 * q, lo);
        }
        E = __ldg(g.d.young + (int64_t)e * R + r);
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      }
      tc_sync();
      if (e >= 0 && t == 0) {
        const uint32_t d_col = 128 + b * 32;
#pragma unroll
        for (int pass = 0; pass < 3; ++pass) {
          const uint32_t a_off = pass == 2 ? 32 : 0;        // A lo in the last pass
          const uint32_t b_off = pass == 1 ? 3 * 1024 : 0;  // K1 lo in the middle pass
#pragma unroll
          for (int sl = 0; sl < 3; ++sl) {
            const uint64_t bd = tc_sdesc(sb + b_off + sl * 1024, 128, 256);
            const uint32_t accum = (pass | sl) ? 1u : 0u;
            asm volatile(
                "{\n.reg .pred pp;\nsetp.ne.u32 pp, %4, 0;\n"
                "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, pp;\n}" ::"r"(tmem + d_col),
                "r"(tmem + b * 64 + a_off + 8 * sl), "l"(bd), "r"(kTcIdesc), "r"(accum)
                : "memory");
          }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         mbar0 + 8 * b)
                     : "memory");
        ++n_commit[b];
      }
      // element P - 1: its forces into the accumulators of its owned points
      if (P > 0 && s_elems[P - 1] >= 0 && ok) {
        const uint32_t pb = (P - 1) & 1;
        ok = tc_wait(mbar0 + 8 * pb, (mpar >> pb) & 1);
        mpar ^= 1u << pb;
        ++n_mwait[pb];
        if (!ok) s_fail = 1;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        float d[24];
        tc_ld24(tmem + lane_base + 128 + pb * 32, d);
        const short* code = c_tc_pos.code[P - 1];
#pragma unroll
        for (int l = 0; l < 8; ++l) {
          const int cd = code[l], p = (cd >> 9) - 1;
          if (p < 0) continue;
          float* a = acc[(cd >> 8) & 1] + p * 3 * kTcThreads;
#pragma unroll
          for (int c = 0; c < 3; ++c) a[c * kTcThreads] = fmaf(E_prev, d[3 * l + c], a[c * kTcThreads]);
        }
      }
      E_prev = E;
    }
    if (k >= z0) {
      for (int p = 0; p < kCP; ++p) {
        const int a = s_nodes[(p / kCX + 1) * kCHX + (p % kCX) + 1];
        if (a < 0) continue;
        const float* ap = acc[0] + p * 3 * kTcThreads;
        const float f[3][1] = {{ap[0]}, {ap[kTcThreads]}, {ap[2 * kTcThreads]}};
        node_update<1>(g, a, r, f, w_in, w_out, vf_in, vf_out, step, rec_now);
      }
    }
    for (int i = 0; i < kAccFloats; i += kTcThreads) acc[0][i] = 0.f;  // this thread's column of plane k
    cur ^= 1;
  }
  // the top plane of the lattice (no layer above it) when it belongs to this segment
  __syncthreads();
  const bool failed = s_fail != 0;
  if (kend < z1 && !failed) {
    for (int p = 0; p < kCP; ++p) {
      const int a = s_nodes[kCHN + (p / kCX + 1) * kCHX + (p % kCX) + 1];
      if (a < 0) continue;
      const float* ap = accs + cur * kAccFloats + t + p * 3 * kTcThreads;
      const float f[3][1] = {{ap[0]}, {ap[kTcThreads]}, {ap[2 * kTcThreads]}};
      node_update<1>(g, a, r, f, w_in, w_out, vf_in, vf_out, step, rec_now);
    }
  }
  // after a failure: wait (bounded) for the bulk copies and MMAs thread 0 started that nobody
  // waited for, so none is in flight when the CTA frees its tensor memory and exits
  if (t == 0 && failed) {
    atomicExch(tt.err, 1);
    for (int z = last_waited + 1; z <= last_loaded; ++z) {
      const int slot = z % 3;
      tc_wait(pbar0 + 8 * slot, (ppar >> slot) & 1);
      ppar ^= 1u << slot;
    }
    for (int q = 0; q < 2; ++q)
      for (; n_mwait[q] < n_commit[q]; ++n_mwait[q]) {
        tc_wait(mbar0 + 8 * q, (mpar >> q) & 1);
        mpar ^= 1u << q;
      }
  }
  tc_sync();
  if (t < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols));
  step_epilogue(g, step);
}

__global__ void k_mark_slots(int64_t n, const int* __restrict__ idx, unsigned char* flag) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    flag[idx[q]] = 1;
}

__device__ inline float2 split2(double x) {
  const float h = (float)x;
  return make_float2(h, (float)(x - (double)h));
}

// run start: the caller's FP64 u, v into the pair accumulators and the FP32 copies
__global__ void k_batch_init(Args g, float* w, float* vf) {
  const int64_t n = (int64_t)g.d.n_nodes * 3 * g.d.R;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const float2 u2 = split2(g.u[q]), v2 = split2(g.v[q]);
    g.u2[q] = u2;
    g.v2[q] = v2;
    w[q] = fmaf(g.beta32, v2.x, u2.x);
    vf[q] = v2.x;
  }
}

// run end: the pair accumulators back into the caller's FP64 u, v
__global__ void k_batch_final(Args g) {
  const int64_t n = (int64_t)g.d.n_nodes * 3 * g.d.R;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    g.u[q] = (double)g.u2[q].x + (double)g.u2[q].y;
    g.v[q] = (double)g.v2[q].x + (double)g.v2[q].y;
  }
}

__global__ void k_batch_consts(int64_t n, const double* ml, float* ml32, float* iml32) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    ml32[q] = (float)ml[q];
    iml32[q] = (float)(1.0 / ml[q]);
  }
}

__global__ void k_batch_force0(Args g, int t) {
  if (!g.f_ptr || t < 0 || t >= g.n_t) return;
  for (int64_t k = g.f_ptr[t] + threadIdx.x; k < g.f_ptr[t + 1]; k += blockDim.x) g.f[g.f_slot[k]] += g.f_val[k];
  __syncthreads();
  for (int64_t k = g.f_ptr[t] + threadIdx.x; k < g.f_ptr[t + 1]; k += blockDim.x) g.f32[g.f_slot[k]] = (float)g.f[g.f_slot[k]];
}

__global__ void k_set_int(int* p, int v) { *p = v; }

}  // namespace bt
}  // namespace sc

using namespace sc;
using namespace sc::bt;

struct sc_batch {
  Args g;
  cudaStream_t user = nullptr, cap = nullptr;
  float *w[2] = {nullptr, nullptr}, *vf[2] = {nullptr, nullptr};
  int* rec_map = nullptr;
  double* f = nullptr;
  float* f32 = nullptr;
  int* t = nullptr;
  unsigned* ticket = nullptr;
  float2 *u2 = nullptr, *v2 = nullptr;
  float *ml32 = nullptr, *iml32 = nullptr;
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  cudaGraph_t graph[2] = {nullptr, nullptr};
  unsigned blocks = 1;
  int rpt = 1, threads = 32, tpn = 32;  // shape chosen by the tuner
  int grid = 0;                         // 1: the uniform hexa8 grid kernel
  float tuned_ms = 0.f;
  unsigned char* vneed = nullptr;
  int n_tiles = 0;
  const int *halo = nullptr, *elem8 = nullptr;  // uniform hexa8 grid tables (caller's), or null
  K1Hex8 k1{};
  TcTables tt{};   // column tables of the tensor-core kernel (caller's), nodes == null when not enabled
  int n_col = 0;
  int* tc_err = nullptr;
};

static void batch_drop_graphs(sc_batch* h) {
  for (int k = 0; k < 2; ++k) {
    if (h->exec[k]) cudaGraphExecDestroy(h->exec[k]), h->exec[k] = nullptr;
    if (h->graph[k]) cudaGraphDestroy(h->graph[k]), h->graph[k] = nullptr;
  }
}

template <int NEN>
static void launch_rpt(int rpt, unsigned blocks, int threads, int tpn, cudaStream_t st, const Args& g,
                       const float* wi, float* wo, const float* vi, float* vo) {
  switch (rpt) {
    case 8: k_batch_step<NEN, 8><<<blocks, threads, 0, st>>>(g, wi, wo, vi, vo, tpn); break;
    case 4: k_batch_step<NEN, 4><<<blocks, threads, 0, st>>>(g, wi, wo, vi, vo, tpn); break;
    case 2: k_batch_step<NEN, 2><<<blocks, threads, 0, st>>>(g, wi, wo, vi, vo, tpn); break;
    default: k_batch_step<NEN, 1><<<blocks, threads, 0, st>>>(g, wi, wo, vi, vo, tpn); break;
  }
}

template <int RPT>
static void launch_hex8g(const sc_batch* h, const Args& g, int threads, cudaStream_t st, const float* wi, float* wo,
                         const float* vi, float* vo) {
  const unsigned by = (unsigned)((g.d.R + 32 * RPT - 1) / (32 * RPT));
  const size_t smem = sizeof(float) * kHN * 3 * 32 * RPT;
  k_batch_step_hex8g<RPT><<<dim3((unsigned)h->n_tiles, by), threads, smem, st>>>(g, h->k1, h->halo, h->elem8, wi, wo,
                                                                                 vi, vo);
}

// grid = 1: the uniform hexa8 grid kernel (threads per block, realisations per thread; tpn unused);
// grid = 2: the tensor-core kernel (rpt = points per column segment along the sweep axis);
// grid = 3: the node-centric uniform hexa8 kernel (shapes as grid = 0)
static void batch_launch(const sc_batch* h, const Args& g, int grid, int rpt, int threads, int tpn, cudaStream_t st,
                         const float* wi, float* wo, const float* vi, float* vo) {
  if (grid == 2) {
    TcTables tt = h->tt;
    tt.seg = rpt;
    tt.n_segs = (tt.nzp + rpt - 1) / rpt;
    k_batch_step_tc<<<dim3((unsigned)(h->n_col * tt.n_segs), (unsigned)(g.d.R / kTcThreads)), kTcThreads, kTcSmem,
                      st>>>(g, h->k1, tt, wi, wo, vi, vo);
    return;
  }
  if (grid == 1) {
    if (rpt == 2) launch_hex8g<2>(h, g, threads, st, wi, wo, vi, vo);
    else launch_hex8g<1>(h, g, threads, st, wi, wo, vi, vo);
    return;
  }
  const int npb = threads / tpn;
  const int64_t want = ((int64_t)g.d.n_nodes + npb - 1) / npb;
  const unsigned blocks = (unsigned)(want < 152 * 32 ? want : 152 * 32);
  if (grid == 4) {  // the wide register budget
    if (rpt == 4) k_batch_step_hex8c_wide<4><<<blocks, threads, 0, st>>>(g, h->k1, h->elem8, wi, wo, vi, vo, tpn);
    else k_batch_step_hex8c_wide<2><<<blocks, threads, 0, st>>>(g, h->k1, h->elem8, wi, wo, vi, vo, tpn);
    return;
  }
  if (grid == 3) {
    switch (rpt) {
      case 8: k_batch_step_hex8c<8><<<blocks, threads, 0, st>>>(g, h->k1, h->elem8, wi, wo, vi, vo, tpn); break;
      case 4: k_batch_step_hex8c<4><<<blocks, threads, 0, st>>>(g, h->k1, h->elem8, wi, wo, vi, vo, tpn); break;
      default: k_batch_step_hex8c<2><<<blocks, threads, 0, st>>>(g, h->k1, h->elem8, wi, wo, vi, vo, tpn); break;
    }
    return;
  }
  if (g.d.node_nen) {
    k_batch_step_mixed<<<blocks, threads, 0, st>>>(g, wi, wo, vi, vo);
    return;
  }
  switch (g.d.n_en) {
    case 8: launch_rpt<8>(rpt, blocks, threads, tpn, st, g, wi, wo, vi, vo); break;
    case 4: launch_rpt<4>(rpt, blocks, threads, tpn, st, g, wi, wo, vi, vo); break;
    case 10: launch_rpt<10>(rpt, blocks, threads, tpn, st, g, wi, wo, vi, vo); break;
    default: launch_rpt<20>(rpt, blocks, threads, tpn, st, g, wi, wo, vi, vo); break;
  }
}

// Realisations per thread (1, 2, 4, 8; vector loads need R divisible by it, and by 4 for
// 4 and 8) and threads per block (128, 256): each candidate advances scratch copies of the
// state (no force, no receivers) 2 + 5 times, and the fastest of the 5 timed launches wins.
// Every candidate performs the same operations in the same order per realisation, so the
// choice changes the speed, not the results.
static int batch_tune(sc_batch* h) {
  const Args& g0 = h->g;
  const int R = g0.d.R;
  cudaStream_t st = h->user;
  const int64_t nsr = (int64_t)g0.d.n_nodes * 3 * R;
  double *u = nullptr, *v = nullptr;
  float *w = nullptr, *vf = nullptr;
  int* t = nullptr;
  unsigned* tk = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = SC_OK;
  float best = -1.f;
  do {
    if ((rc = check(cudaMallocAsync((void**)&u, 8 * nsr, st), "tune malloc")) ||
        (rc = check(cudaMallocAsync((void**)&v, 8 * nsr, st), "tune malloc")) ||
        (rc = check(cudaMallocAsync((void**)&w, 8 * nsr, st), "tune malloc")) ||
        (rc = check(cudaMallocAsync((void**)&vf, 8 * nsr, st), "tune malloc")) ||
        (rc = check(cudaMallocAsync((void**)&t, sizeof(int), st), "tune malloc")) ||
        (rc = check(cudaMallocAsync((void**)&tk, sizeof(unsigned), st), "tune malloc")))
      break;
    cudaMemsetAsync(u, 0, 8 * nsr, st);
    cudaMemsetAsync(v, 0, 8 * nsr, st);
    cudaMemsetAsync(w, 0, 8 * nsr, st);
    cudaMemsetAsync(vf, 0, 8 * nsr, st);
    cudaMemsetAsync(t, 0, sizeof(int), st);
    cudaMemsetAsync(tk, 0, sizeof(unsigned), st);
    if ((rc = check(cudaEventCreate(&e0), "event")) || (rc = check(cudaEventCreate(&e1), "event"))) break;
    Args g = g0;
    g.u = u;
    g.v = v;
    g.u2 = reinterpret_cast<float2*>(u);  // zeros: valid pairs
    g.v2 = reinterpret_cast<float2*>(v);
    g.t = t;
    g.ticket = tk;
    g.f_ptr = nullptr;
    g.n_rec = 0;
    // candidates: (grid kernel, realisations per thread, threads per block)
    struct Cand {
      int grid, rpt, threads, tpn;
    };
    std::vector<Cand> cands;
    const int rpts[4] = {1, 2, 4, 8};
    const int tpbs[3] = {128, 256, 64};
    const bool mixed = g0.d.node_nen != nullptr;  // one realisation, one thread per node
    for (int ri = 0; ri < 4; ++ri) {
      const int rpt = rpts[ri];
      if (R % rpt != 0 || (rpt >= 4 && R % 4 != 0)) continue;
      if (mixed && rpt != 1) continue;
      const int tpn = (R + rpt - 1) / rpt;
      for (int bi = 0; bi < (mixed ? 3 : 2); ++bi)
        if (tpn <= tpbs[bi]) cands.push_back({0, rpt, (tpbs[bi] / tpn) * tpn, tpn});
    }
    if (h->halo) {
      for (int rpt = 1; rpt <= 2; ++rpt)
        if (R % rpt == 0)
          for (int threads : {256, 128}) cands.push_back({1, rpt, threads, 0});
      for (int rpt : {2, 4, 8}) {
        if (R % rpt != 0 || (rpt >= 4 && R % 4 != 0)) continue;
        const int tpn = R / rpt;
        for (int threads : {128, 256})
          if (tpn <= threads) {
            cands.push_back({3, rpt, (threads / tpn) * tpn, tpn});
            if (rpt <= 4) cands.push_back({4, rpt, (threads / tpn) * tpn, tpn});
          }
      }
    }
    if (h->tt.nodes) {  // tensor-core kernel: segments of the whole column, a half, a third, a quarter
      int last = 0;
      for (int parts = 1; parts <= 4; ++parts) {
        const int seg = (h->tt.nzp + parts - 1) / parts;
        if (seg != last) cands.push_back({2, seg, kTcThreads, 0});
        last = seg;
      }
    }
    for (size_t ci = 0; ci < cands.size() && !rc; ++ci) {
      const Cand& c = cands[ci];
      float* wh = w;
      float* wl = w + nsr;
      float* vh = vf;
      float* vl = vf + nsr;
      for (int q = 0; q < 2; ++q) batch_launch(h, g, c.grid, c.rpt, c.threads, c.tpn, st, wh, wl, vh, vl);
      float ms_min = -1.f;
      for (int q = 0; q < 5 && !rc; ++q) {
        cudaEventRecord(e0, st);
        batch_launch(h, g, c.grid, c.rpt, c.threads, c.tpn, st, (q & 1) ? wl : wh, (q & 1) ? wh : wl,
                     (q & 1) ? vl : vh, (q & 1) ? vh : vl);
        cudaEventRecord(e1, st);
        if ((rc = check_launch("batch tune"))) break;
        if ((rc = check(cudaEventSynchronize(e1), "tune sync"))) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms_min < 0.f || ms < ms_min) ms_min = ms;
      }
      if (!rc && (best < 0.f || ms_min < best)) {
        best = ms_min;
        h->grid = c.grid;
        h->rpt = c.rpt;
        h->threads = c.threads;
        h->tpn = c.tpn;
      }
    }
  } while (0);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamSynchronize(st);
  void* frees[] = {u, v, w, vf, t, tk};
  for (void* q : frees)
    if (q) cudaFree(q);
  h->tuned_ms = best;
  if (!rc && best < 0.f) rc = SC_BAD_ARG;  // no candidate fits (R > 2048)
  return rc;
}

static int batch_build(sc_batch* h) {
  for (int k = 0; k < 2; ++k) {
    int rc = check(cudaStreamBeginCapture(h->cap, cudaStreamCaptureModeThreadLocal), "capture batch");
    if (rc) return rc;
    batch_launch(h, h->g, h->grid, h->rpt, h->threads, h->tpn, h->cap, h->w[k], h->w[k ^ 1], h->vf[k],
                 h->vf[k ^ 1]);
    cudaGraph_t gr;
    if ((rc = check(cudaStreamEndCapture(h->cap, &gr), "end batch"))) return rc;
    if ((rc = check(cudaGraphInstantiate(&h->exec[k], gr, 0), "instantiate batch"))) {
      cudaGraphDestroy(gr);
      return rc;
    }
    h->graph[k] = gr;
  }
  return SC_OK;
}

extern "C" int sc_batch_create(sc_batch** out, const sc_batch_desc* d, double* u, double* v, void* stream) {
  if (!out || !d || !u || !v || d->n_nodes <= 0 || d->R <= 0 || d->R > 1024 || !d->elem || !d->inc_ptr || !d->inc ||
      !d->ke_type || !d->ke1 || !d->young || !d->ml || !d->fixed || !d->l_ptr)
    return SC_BAD_ARG;
  if (d->n_en != 8 && d->n_en != 4 && d->n_en != 10 && d->n_en != 20) return SC_BAD_ARG;
  if (!(d->dt > 0)) return SC_BAD_ARG;
  if (d->node_nen && d->R != 1) return SC_BAD_ARG;  // mixed element types: one realisation
  // at most 256 threads per node: R > 256 needs 2 (R <= 512) or 4 realisations per thread
  if (d->R > 256 && !(d->R % 4 == 0 || (d->R <= 512 && d->R % 2 == 0))) return SC_BAD_ARG;
  sc_batch* h = new sc_batch();
  h->user = (cudaStream_t)stream;
  h->g = Args{};
  h->g.d = *d;
  h->g.u = u;
  h->g.v = v;
  cudaStream_t st = h->user;
  const int64_t ns = (int64_t)d->n_nodes * 3, nsr = ns * d->R;
  int rc = SC_OK;
  do {
    if ((rc = check(cudaStreamCreateWithFlags(&h->cap, cudaStreamNonBlocking), "stream"))) break;
    for (int k = 0; k < 2 && !rc; ++k) {
      rc = check(cudaMallocAsync((void**)&h->w[k], 4 * nsr, st), "malloc");
      if (!rc) rc = check(cudaMallocAsync((void**)&h->vf[k], 4 * nsr, st), "malloc");
    }
    if (rc) break;
    if ((rc = check(cudaMallocAsync((void**)&h->rec_map, 4 * ns, st), "malloc"))) break;
    if ((rc = check(cudaMallocAsync((void**)&h->f, 8 * ns, st), "malloc"))) break;
    if ((rc = check(cudaMallocAsync((void**)&h->f32, 4 * ns, st), "malloc"))) break;
    if ((rc = check(cudaMallocAsync((void**)&h->t, sizeof(int), st), "malloc"))) break;
    if ((rc = check(cudaMallocAsync((void**)&h->ticket, sizeof(unsigned), st), "malloc"))) break;
    if ((rc = check(cudaMallocAsync((void**)&h->u2, 8 * nsr, st), "malloc"))) break;
    if ((rc = check(cudaMallocAsync((void**)&h->v2, 8 * nsr, st), "malloc"))) break;
    if ((rc = check(cudaMallocAsync((void**)&h->ml32, 4 * ns, st), "malloc"))) break;
    if ((rc = check(cudaMallocAsync((void**)&h->iml32, 4 * ns, st), "malloc"))) break;
    if ((rc = check(cudaMallocAsync((void**)&h->vneed, ns, st), "malloc"))) break;
    k_batch_consts<<<grid_for(ns, 256), 256, 0, st>>>(ns, d->ml, h->ml32, h->iml32);
    // slots whose FP32 velocity copy a Lysmer row reads
    cudaMemsetAsync(h->vneed, 0, ns, st);
    int64_t n_l = 0;
    if ((rc = check(cudaMemcpyAsync(&n_l, d->l_ptr + ns, 8, cudaMemcpyDeviceToHost, st), "lysmer size"))) break;
    if ((rc = check(cudaStreamSynchronize(st), "sync"))) break;
    if (n_l > 0) k_mark_slots<<<grid_for(n_l, 256), 256, 0, st>>>(n_l, d->l_col, h->vneed);
    h->g.vneed = h->vneed;
    h->g.u2 = h->u2;
    h->g.v2 = h->v2;
    h->g.ml32 = h->ml32;
    h->g.iml32 = h->iml32;
    h->g.dth = (float)d->dt;
    h->g.dtl = (float)(d->dt - (double)h->g.dth);
    h->g.alpha32 = (float)d->alpha;
    h->g.beta32 = (float)d->beta;
    cudaMemsetAsync(h->rec_map, 0xff, 4 * ns, st);
    cudaMemsetAsync(h->f, 0, 8 * ns, st);
    cudaMemsetAsync(h->f32, 0, 4 * ns, st);
    cudaMemsetAsync(h->t, 0, sizeof(int), st);
    cudaMemsetAsync(h->ticket, 0, sizeof(unsigned), st);
    h->g.f = h->f;
    h->g.f32 = h->f32;
    h->g.t = h->t;
    h->g.ticket = h->ticket;
    h->g.rec_map = h->rec_map;
    if ((rc = batch_tune(h))) break;
    rc = check(cudaStreamSynchronize(st), "sync");
  } while (0);
  if (rc) {
    sc_batch_destroy(h);
    return rc;
  }
  *out = h;
  return SC_OK;
}

// Enables the uniform hexa8 grid kernel (tables as described at k_batch_step_hex8g; the
// incidence lists must be sorted by the node's local index in the element) and re-runs the
// tuner over both kernels.
extern "C" int sc_batch_set_hex8_grid(sc_batch* h, int n_tiles, const int* halo, const int* elem8) {
  if (!h || n_tiles <= 0 || !halo || !elem8 || h->g.d.n_en != 8 || h->g.d.n_types != 1 || h->g.d.node_nen)
    return SC_BAD_ARG;
  if ((h->g.d.R + 63) / 64 > 65535) return SC_BAD_ARG;
  cudaStream_t st = h->user;
  int rc = check(cudaMemcpyAsync(h->k1.k, h->g.d.ke1, sizeof(h->k1.k), cudaMemcpyDeviceToHost, st), "k1");
  if (!rc) rc = check(cudaStreamSynchronize(st), "sync");
  if (!rc) rc = check(cudaFuncSetAttribute(k_batch_step_hex8g<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)(sizeof(float) * kHN * 3 * 32)), "smem attribute");
  if (!rc) rc = check(cudaFuncSetAttribute(k_batch_step_hex8g<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)(sizeof(float) * kHN * 3 * 64)), "smem attribute");
  if (rc) return rc;
  h->n_tiles = n_tiles;
  h->halo = halo;
  h->elem8 = elem8;
  batch_drop_graphs(h);
  return batch_tune(h);
}

// Selects the uniform hexa8 grid kernel with 1 or 2 realisations per thread and 128 or 256
// threads per block (testing aid; needs sc_batch_set_hex8_grid).
extern "C" int sc_batch_set_grid_shape(sc_batch* h, int realisations_per_thread, int threads_per_block) {
  if (!h || !h->halo) return SC_BAD_ARG;
  const int rpt = realisations_per_thread;
  if ((rpt != 1 && rpt != 2) || h->g.d.R % rpt != 0) return SC_BAD_ARG;
  if (threads_per_block != 128 && threads_per_block != 256) return SC_BAD_ARG;
  h->grid = 1;
  h->rpt = rpt;
  h->threads = threads_per_block;
  h->tpn = 0;
  batch_drop_graphs(h);
  return SC_OK;
}

// Selects the node-centric uniform hexa8 kernel with 2, 4 or 8 realisations per thread and 128
// or 256 threads per block (testing aid; needs sc_batch_set_hex8_grid).
extern "C" int sc_batch_set_node_shape(sc_batch* h, int realisations_per_thread, int threads_per_block) {
  return sc_batch_set_node_shape_budget(h, realisations_per_thread, threads_per_block, 0);
}

// the same with wide = 1: the kernel at the wide register budget (2 or 4 realisations per thread)
extern "C" int sc_batch_set_node_shape_budget(sc_batch* h, int realisations_per_thread, int threads_per_block,
                                              int wide) {
  if (!h || !h->halo || (wide != 0 && wide != 1)) return SC_BAD_ARG;
  if (wide && realisations_per_thread == 8) return SC_BAD_ARG;
  const int rpt = realisations_per_thread, R = h->g.d.R;
  if ((rpt != 2 && rpt != 4 && rpt != 8) || R % rpt != 0 || (rpt >= 4 && R % 4 != 0)) return SC_BAD_ARG;
  if (threads_per_block != 128 && threads_per_block != 256) return SC_BAD_ARG;
  const int tpn = R / rpt;
  if (tpn > threads_per_block) return SC_BAD_ARG;
  h->grid = wide ? 4 : 3;
  h->rpt = rpt;
  h->threads = (threads_per_block / tpn) * tpn;
  h->tpn = tpn;
  batch_drop_graphs(h);
  return SC_OK;
}

// Enables the tensor-core kernel on a uniform hexa8 grid (tables as described at
// k_batch_step_tc; R a multiple of 128) and re-runs the tuner over all kernels.
extern "C" int sc_batch_set_hex8_columns(sc_batch* h, int n_col, int nzp, const int* nodes, const int* elems) {
  if (!h || n_col <= 0 || nzp < 2 || !nodes || !elems || h->g.d.n_en != 8 || h->g.d.n_types != 1 || h->g.d.node_nen)
    return SC_BAD_ARG;
  if (h->g.d.R % kTcThreads != 0 || h->g.d.R / kTcThreads > 65535 || (int64_t)n_col * nzp > (1ll << 30))
    return SC_BAD_ARG;
  cudaStream_t st = h->user;
  int rc = SC_OK;
  if (!h->tc_err) rc = check(cudaMallocAsync((void**)&h->tc_err, sizeof(int), st), "malloc");
  if (!rc) rc = check(cudaMemsetAsync(h->tc_err, 0, sizeof(int), st), "memset");
  if (!rc) rc = check(cudaMemcpyAsync(h->k1.k, h->g.d.ke1, sizeof(h->k1.k), cudaMemcpyDeviceToHost, st), "k1");
  if (!rc) rc = check(cudaStreamSynchronize(st), "sync");
  if (!rc) rc = check(cudaFuncSetAttribute(k_batch_step_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem),
                      "smem attribute");
  if (rc) return rc;
  h->tt.nodes = nodes;
  h->tt.elems = elems;
  h->tt.nzp = nzp;
  h->tt.err = h->tc_err;
  h->n_col = n_col;
  batch_drop_graphs(h);
  return batch_tune(h);
}

// Selects the tensor-core kernel with column segments of `seg` points (testing aid; needs
// sc_batch_set_hex8_columns).
extern "C" int sc_batch_set_tc_shape(sc_batch* h, int seg) {
  if (!h || !h->tt.nodes || seg < 1) return SC_BAD_ARG;
  h->grid = 2;
  h->rpt = seg;
  h->threads = kTcThreads;
  h->tpn = 0;
  batch_drop_graphs(h);
  return SC_OK;
}

// Synchronises the stream; SC_CUDA_ERROR when a tensor-core step gave up waiting for its MMAs
// (its results are then not valid), else the stream's status.
extern "C" int sc_batch_status(sc_batch* h) {
  if (!h) return SC_BAD_ARG;
  int rc = check(cudaStreamSynchronize(h->user), "batch sync");
  if (rc || !h->tc_err) return rc;
  int flag = 0;
  if ((rc = check(cudaMemcpy(&flag, h->tc_err, sizeof(int), cudaMemcpyDeviceToHost), "batch status"))) return rc;
  if (flag) {
    set_last_message("tensor-core batched step: an MMA completion wait gave up");
    return SC_CUDA_ERROR;
  }
  return SC_OK;
}

extern "C" int sc_batch_set_shape(sc_batch* h, int realisations_per_thread, int threads_per_block) {
  if (!h) return SC_BAD_ARG;
  const int R = h->g.d.R, rpt = realisations_per_thread;
  if (rpt != 1 && rpt != 2 && rpt != 4 && rpt != 8) return SC_BAD_ARG;
  if (R % rpt != 0 || (rpt >= 4 && R % 4 != 0)) return SC_BAD_ARG;
  const int tpn = (R + rpt - 1) / rpt;
  if (threads_per_block < tpn || threads_per_block > 256 || threads_per_block % tpn != 0) return SC_BAD_ARG;
  h->grid = 0;
  h->rpt = rpt;
  h->threads = threads_per_block;
  h->tpn = tpn;
  batch_drop_graphs(h);
  return SC_OK;
}

extern "C" int sc_batch_config(sc_batch* h, int* realisations_per_thread, int* threads_per_block, float* ms_per_step,
                               int* grid_kernel) {
  if (!h) return SC_BAD_ARG;
  if (realisations_per_thread) *realisations_per_thread = h->rpt;
  if (threads_per_block) *threads_per_block = h->threads;
  if (ms_per_step) *ms_per_step = h->tuned_ms;
  if (grid_kernel) *grid_kernel = h->grid;
  return SC_OK;
}

extern "C" int sc_batch_set_force(sc_batch* h, int n_t, const int64_t* f_ptr, const int* f_slot, const double* f_val) {
  if (!h || n_t < 0 || (n_t > 0 && (!f_ptr || !f_slot || !f_val))) return SC_BAD_ARG;
  h->g.n_t = n_t;
  h->g.f_ptr = n_t > 0 ? f_ptr : nullptr;
  h->g.f_slot = f_slot;
  h->g.f_val = f_val;
  batch_drop_graphs(h);
  return SC_OK;
}

__global__ void k_batch_recmap(int n_rec, const int* rec_slot, int* map) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n_rec; j += gridDim.x * blockDim.x) map[rec_slot[j]] = j;
}

extern "C" int sc_batch_set_output(sc_batch* h, int out_interval, int n_rec, const int* rec_slot, double* out_v,
                                   int64_t n_out) {
  if (!h || n_rec < 0 || (n_rec > 0 && (!rec_slot || !out_v || out_interval <= 0 || n_out <= 0))) return SC_BAD_ARG;
  cudaMemsetAsync(h->rec_map, 0xff, 4 * (int64_t)h->g.d.n_nodes * 3, h->user);
  if (n_rec > 0) k_batch_recmap<<<grid_for(n_rec, 128), 128, 0, h->user>>>(n_rec, rec_slot, h->rec_map);
  h->g.n_rec = n_rec;
  h->g.out_interval = out_interval;
  h->g.out_v = out_v;
  h->g.n_out = n_out;
  batch_drop_graphs(h);
  return check_launch("batch output");
}

// Steps t_begin .. t_end-1 for every realisation (state in u, v; t_begin == 0 starts the
// force history at step 0).
extern "C" int sc_batch_run(sc_batch* h, int t_begin, int t_end) {
  if (!h || t_begin < 0 || t_end < t_begin) return SC_BAD_ARG;
  int rc;
  if (!h->exec[0] && (rc = batch_build(h))) return rc;
  cudaStream_t st = h->user;
  k_batch_init<<<grid_for((int64_t)h->g.d.n_nodes * 3 * h->g.d.R, 256, 152 * 32), 256, 0, st>>>(h->g, h->w[0],
                                                                                                 h->vf[0]);
  cudaMemsetAsync(h->f, 0, 8 * (int64_t)h->g.d.n_nodes * 3, st);
  cudaMemsetAsync(h->f32, 0, 4 * (int64_t)h->g.d.n_nodes * 3, st);
  k_batch_force0<<<1, 256, 0, st>>>(h->g, t_begin);
  k_set_int<<<1, 1, 0, st>>>(h->t, t_begin);
  if ((rc = check_launch("batch prepare"))) return rc;
  int k = 0;
  for (int t = t_begin; t < t_end; ++t, k ^= 1)
    if ((rc = check(cudaGraphLaunch(h->exec[k], st), "batch launch"))) return rc;
  k_batch_final<<<grid_for((int64_t)h->g.d.n_nodes * 3 * h->g.d.R, 256, 152 * 32), 256, 0, st>>>(h->g);
  return check_launch("batch final");
}

extern "C" int sc_batch_destroy(sc_batch* h) {
  if (!h) return SC_OK;
  batch_drop_graphs(h);
  cudaStreamSynchronize(h->user);
  for (int k = 0; k < 2; ++k) {
    if (h->w[k]) cudaFree(h->w[k]);
    if (h->vf[k]) cudaFree(h->vf[k]);
  }
  if (h->rec_map) cudaFree(h->rec_map);
  if (h->f) cudaFree(h->f);
  if (h->f32) cudaFree(h->f32);
  if (h->t) cudaFree(h->t);
  if (h->ticket) cudaFree(h->ticket);
  void* more[] = {h->u2, h->v2, h->ml32, h->iml32, h->vneed, h->tc_err};
  for (void* q : more)
    if (q) cudaFree(q);
  if (h->cap) cudaStreamDestroy(h->cap);
  delete h;
  return SC_OK;
}
