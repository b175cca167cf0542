// Batched explicit scheme: R realisations of the per-element Young's modulus advanced
// together, one kernel per step, FP32 stiffness products with FP64 state accumulators.
//
// Physics per realisation r is the explicit lumped-mass scheme of sc_nbsolver.cu
// (k_explicit) with K_r = sum_e E_{e,r} K1_e (K1_e: element stiffness at E = 1, which is
// what scatter/discretisation.py:177-201 gives for D(E=1, nu)), density and Poisson ratio
// shared, and the Lysmer terms of scatter/system_matrix.py:362-376 scaled per realisation:
// rho v_p, rho v_s grow as sqrt(E) (dashpots), E_c and G as E (springs).
//
// Layout: every per-realisation array is [slot or element][R] (realisation fastest), so the
// R threads of a block (one per realisation) read and write 32-wide coalesced rows.  A block
// takes one node at a time (grid-stride), gathers K1 blocks of the node's elements (shared
// across threads, L1 broadcasts), scales by E_{e,r} and updates the node's DOFs.  u and v
// are FP64 and updated in place (own node only); w = u + beta v and v are also kept as FP32
// ping-pong copies that neighbours read.
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
};

namespace sc {
namespace bt {

struct Args {
  sc_batch_desc d;
  double *u, *v;
  double* f;  // dense force, slot space (shared by the realisations)
  int* t;     // device step counter
  int n_t;
  const int64_t* f_ptr;
  const int* f_slot;
  const double* f_val;
  int n_rec, out_interval;
  const int* rec_map;  // slot -> receiver index or -1
  double* out_v;       // [n_out][n_rec][R]
  int64_t n_out;
};

template <int NEN>
__global__ void __launch_bounds__(256) k_batch_step(Args g, const float* __restrict__ w_in, float* __restrict__ w_out,
                                                    const float* __restrict__ vf_in, float* __restrict__ vf_out) {
  const sc_batch_desc& d = g.d;
  const int R = d.R;
  const int r = threadIdx.x;
  const bool active = r < R;
  constexpr int ND = NEN * 3;
  const int step = *g.t + 1;
  const bool rec_now = g.n_rec > 0 && g.out_interval > 0 && step % g.out_interval == 0 &&
                       step / g.out_interval < g.n_out;
  for (int a = blockIdx.x; a < d.n_nodes; a += gridDim.x) {
    float acc[3] = {0.f, 0.f, 0.f};
    for (int k = d.inc_ptr[a]; k < d.inc_ptr[a + 1]; ++k) {
      const int e = d.inc[k];
      const int* en = d.elem + (int64_t)e * NEN;
      int la = 0;
#pragma unroll
      for (int q = 0; q < NEN; ++q)
        if (en[q] == a) la = q;
      const float* K1 = d.ke1 + (int64_t)d.ke_type[e] * ND * ND + (int64_t)(la * 3) * ND;
      float t0 = 0.f, t1 = 0.f, t2 = 0.f;
      if (active) {
#pragma unroll 4
        for (int lb = 0; lb < NEN; ++lb) {
          const int64_t bs = (int64_t)en[lb] * 3;
          const float w0 = w_in[(bs + 0) * R + r], w1 = w_in[(bs + 1) * R + r], w2 = w_in[(bs + 2) * R + r];
          const float* kr = K1 + lb * 3;
          t0 = fmaf(__ldg(kr + 0), w0, fmaf(__ldg(kr + 1), w1, fmaf(__ldg(kr + 2), w2, t0)));
          t1 = fmaf(__ldg(kr + ND + 0), w0, fmaf(__ldg(kr + ND + 1), w1, fmaf(__ldg(kr + ND + 2), w2, t1)));
          t2 = fmaf(__ldg(kr + 2 * ND + 0), w0, fmaf(__ldg(kr + 2 * ND + 1), w1, fmaf(__ldg(kr + 2 * ND + 2), w2, t2)));
        }
        const float Ee = d.young[(int64_t)e * R + r];
        acc[0] = fmaf(Ee, t0, acc[0]);
        acc[1] = fmaf(Ee, t1, acc[1]);
        acc[2] = fmaf(Ee, t2, acc[2]);
      }
    }
    if (!active) continue;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int64_t i = (int64_t)a * 3 + c;
      const int64_t ir = i * R + r;
      if (d.fixed[i]) {
        w_out[ir] = 0.f;
        vf_out[ir] = 0.f;
        continue;
      }
      float spring = 0.f, dash = 0.f;
      for (int64_t q = d.l_ptr[i]; q < d.l_ptr[i + 1]; ++q) {
        const int64_t jr = (int64_t)d.l_col[q] * R + r;
        const float Eq = d.young[(int64_t)d.l_elem[q] * R + r];
        spring = fmaf(d.l_s[q] * Eq, w_in[jr], spring);
        dash = fmaf(d.l_c[q] * sqrtf(Eq), vf_in[jr], dash);
      }
      const double vi = g.v[ir], ml = d.ml[i];
      const double kw = (double)acc[c] + (double)spring;
      const double accel = (g.f[i] - kw - d.alpha * ml * vi - (double)dash) / ml;
      const double vn = fma(d.dt, accel, vi);
      const double un = fma(d.dt, vn, g.u[ir]);
      g.v[ir] = vn;
      g.u[ir] = un;
      w_out[ir] = (float)fma(d.beta, vn, un);
      vf_out[ir] = (float)vn;
      if (rec_now) {
        const int rj = g.rec_map[i];
        if (rj >= 0) g.out_v[((int64_t)(step / g.out_interval) * g.n_rec + rj) * R + r] = vn;
      }
    }
  }
}

// advance the step counter and set the force of the new step (f holds step t's entries)
__global__ void k_batch_force(Args g) {
  __shared__ int t;
  if (threadIdx.x == 0) t = *g.t + 1;
  __syncthreads();
  if (g.f_ptr) {
    if (t - 1 >= 0 && t - 1 < g.n_t)
      for (int64_t k = g.f_ptr[t - 1] + threadIdx.x; k < g.f_ptr[t]; k += blockDim.x) g.f[g.f_slot[k]] = 0.0;
    __syncthreads();
    if (t < g.n_t)
      for (int64_t k = g.f_ptr[t] + threadIdx.x; k < g.f_ptr[t + 1]; k += blockDim.x) g.f[g.f_slot[k]] += g.f_val[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) *g.t = t;
}

__global__ void k_batch_init(Args g, float* w, float* vf) {
  const int64_t n = (int64_t)g.d.n_nodes * 3 * g.d.R;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    w[q] = (float)fma(g.d.beta, g.v[q], g.u[q]);
    vf[q] = (float)g.v[q];
  }
}

__global__ void k_batch_force0(Args g, int t) {
  if (!g.f_ptr || t < 0 || t >= g.n_t) return;
  for (int64_t k = g.f_ptr[t] + threadIdx.x; k < g.f_ptr[t + 1]; k += blockDim.x) g.f[g.f_slot[k]] += g.f_val[k];
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
  int* t = nullptr;
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  cudaGraph_t graph[2] = {nullptr, nullptr};
  unsigned blocks = 1;
  int parity = 0;
};

static void batch_drop_graphs(sc_batch* h) {
  for (int k = 0; k < 2; ++k) {
    if (h->exec[k]) cudaGraphExecDestroy(h->exec[k]), h->exec[k] = nullptr;
    if (h->graph[k]) cudaGraphDestroy(h->graph[k]), h->graph[k] = nullptr;
  }
}

static int batch_build(sc_batch* h) {
  for (int k = 0; k < 2; ++k) {
    int rc = check(cudaStreamBeginCapture(h->cap, cudaStreamCaptureModeThreadLocal), "capture batch");
    if (rc) return rc;
    const float* wi = h->w[k];
    float* wo = h->w[k ^ 1];
    const float* vi = h->vf[k];
    float* vo = h->vf[k ^ 1];
    const int threads = ((h->g.d.R + 31) / 32) * 32;
    switch (h->g.d.n_en) {
      case 8: k_batch_step<8><<<h->blocks, threads, 0, h->cap>>>(h->g, wi, wo, vi, vo); break;
      case 4: k_batch_step<4><<<h->blocks, threads, 0, h->cap>>>(h->g, wi, wo, vi, vo); break;
      case 10: k_batch_step<10><<<h->blocks, threads, 0, h->cap>>>(h->g, wi, wo, vi, vo); break;
      default: k_batch_step<20><<<h->blocks, threads, 0, h->cap>>>(h->g, wi, wo, vi, vo); break;
    }
    k_batch_force<<<1, 256, 0, h->cap>>>(h->g);
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
    if ((rc = check(cudaMallocAsync((void**)&h->t, sizeof(int), st), "malloc"))) break;
    cudaMemsetAsync(h->rec_map, 0xff, 4 * ns, st);
    cudaMemsetAsync(h->f, 0, 8 * ns, st);
    cudaMemsetAsync(h->t, 0, sizeof(int), st);
    h->g.f = h->f;
    h->g.t = h->t;
    h->g.rec_map = h->rec_map;
    h->blocks = (unsigned)(d->n_nodes < 152 * 16 ? d->n_nodes : 152 * 16);
    rc = check(cudaStreamSynchronize(st), "sync");
  } while (0);
  if (rc) {
    sc_batch_destroy(h);
    return rc;
  }
  *out = h;
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
  k_batch_force0<<<1, 256, 0, st>>>(h->g, t_begin);
  k_set_int<<<1, 1, 0, st>>>(h->t, t_begin);
  if ((rc = check_launch("batch prepare"))) return rc;
  int k = 0;
  for (int t = t_begin; t < t_end; ++t, k ^= 1)
    if ((rc = check(cudaGraphLaunch(h->exec[k], st), "batch launch"))) return rc;
  return SC_OK;
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
  if (h->t) cudaFree(h->t);
  if (h->cap) cudaStreamDestroy(h->cap);
  delete h;
  return SC_OK;
}
