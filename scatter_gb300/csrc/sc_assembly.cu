// Deterministic CSR assembly over the element graph (no atomics on values).
//
// Replaces the per-element dict accumulation of GenerateMatrix.generate_stiffness_and_mass
// (scatter/system_matrix.py:87-121).  The reference sums, for every (row, col) pair of free
// equations, the element contributions in element order and stores the element-graph
// pattern with rows/cols sorted.  Here:
//   1. node -> element incidence, element ids ascending per node (counting sort + per-node
//      insertion sort, so the result does not depend on atomic ordering);
//   2. node adjacency: sorted unique neighbour nodes per node (warp-level bitonic sort);
//   3. CSR rows over free DOFs; with node-major, DOF-minor equation numbers
//      (scatter/mesher.py:276-310) a row's columns are the free DOFs of the sorted
//      neighbour nodes, already ascending;
//   4. values: one warp per node walks the node's elements in ascending order and adds
//      each element's entries into the rows of that node, so every entry is the
//      element-order sum the reference forms.
#include <stdio.h>

#include <mutex>

#include "sc_common.cuh"

namespace sc {

// ------------------------------------------------------------------ exclusive scan (int64)
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 8;
constexpr int64_t kScanTile = (int64_t)kScanThreads * kScanItems;

__device__ inline int64_t block_exclusive_scan(int64_t v, int64_t* sh, int64_t* total) {
  // sh: 32 int64
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    int64_t s = lane < nw ? sh[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    sh[lane] = s;  // inclusive warp totals
  }
  __syncthreads();
  const int64_t warp_off = wid > 0 ? sh[wid - 1] : 0;
  if (total) *total = sh[(blockDim.x >> 5) - 1];
  return warp_off + x - v;
}

// in and out may alias (each element is read and written by the same thread only)
__global__ void k_scan_tiles(int64_t n, const int64_t* in, int64_t* out, int64_t* __restrict__ tile_sums) {
  __shared__ int64_t sh[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems];
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < n) ? in[base + k] : 0;
    s += v[k];
  }
  int64_t tot;
  int64_t off = block_exclusive_scan(s, sh, &tot);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = off;
    off += v[k];
  }
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

// single block: exclusive scan of up to kScanTile tile sums, in place; writes grand total
__global__ void k_scan_sums(int64_t n_tiles, int64_t* __restrict__ sums, int64_t* __restrict__ total) {
  __shared__ int64_t sh[32];
  const int64_t base = (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems];
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < n_tiles) ? sums[base + k] : 0;
    s += v[k];
  }
  int64_t tot;
  int64_t off = block_exclusive_scan(s, sh, &tot);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n_tiles) sums[base + k] = off;
    off += v[k];
  }
  if (threadIdx.x == 0) *total = tot;
}

__global__ void k_scan_add(int64_t n, int64_t* __restrict__ out, const int64_t* __restrict__ sums) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += sums[i / kScanTile];
}

int exclusive_scan_i64(int64_t n, const int64_t* in, int64_t* out, int64_t* work, cudaStream_t st) {
  if (n < 0) return SC_BAD_ARG;
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles > kScanTile) return SC_CAPACITY;
  if (n == 0) {
    int64_t z = 0;
    return check(cudaMemcpyAsync(out, &z, sizeof(int64_t), cudaMemcpyHostToDevice, st), "scan zero");
  }
  // in == out is allowed: each element is read before it is written by the same thread
  k_scan_tiles<<<(unsigned)tiles, kScanThreads, 0, st>>>(n, in, out, work);
  k_scan_sums<<<1, kScanThreads, 0, st>>>(tiles, work, out + n);
  k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, out, work);
  return check_launch("exclusive_scan_i64");
}

// ------------------------------------------------------------------ grouping helpers
__global__ void k_count_keys(int64_t n, const int* __restrict__ keys, int n_keys, int* __restrict__ cnt,
                             int* __restrict__ bad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int k = keys[i];
    if (k < 0 || k >= n_keys) {
      atomicExch(bad, 1);
      continue;
    }
    atomicAdd(cnt + k, 1);
  }
}

__global__ void k_i32_to_i64(int64_t n, const int* __restrict__ a, int64_t* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = a[i];
}

__global__ void k_i64_to_i32(int64_t n, const int64_t* __restrict__ a, int* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (int)a[i];
}

// scatter item i to ptr[key] + cursor, then each key's segment is insertion-sorted by the
// stored payload so the final order is independent of the atomic order.
__global__ void k_scatter_keys(int64_t n, const int* __restrict__ keys, int n_keys, const int* __restrict__ ptr,
                               int* __restrict__ cursor, int* __restrict__ out, int payload_div) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int k = keys[i];
    if (k < 0 || k >= n_keys) continue;
    const int pos = atomicAdd(cursor + k, 1);
    out[ptr[k] + pos] = (int)(i / payload_div);
  }
}

__global__ void k_sort_segments(int n_keys, const int* __restrict__ ptr, int* __restrict__ vals) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n_keys; k += gridDim.x * blockDim.x) {
    const int b = ptr[k], e = ptr[k + 1];
    for (int i = b + 1; i < e; ++i) {
      const int x = vals[i];
      int j = i - 1;
      while (j >= b && vals[j] > x) {
        vals[j + 1] = vals[j];
        --j;
      }
      vals[j + 1] = x;
    }
  }
}

// group n items by key: ptr [n_keys+1] (int32), out [n] = item index / payload_div, ascending
// per key.  scratch64 holds n_keys+1 int64 + scan work; cnt n_keys int32.
int group_by_key(int64_t n, const int* keys, int n_keys, int payload_div, int* ptr, int* out, int* cnt,
                 cudaStream_t st) {
  if (n < 0 || n_keys < 0 || n >= (1ll << 31)) return SC_BAD_ARG;
  int* bad = nullptr;
  int64_t* tmp = nullptr;
  int rc = SC_OK;
  const int64_t tiles = ((int64_t)n_keys + kScanTile - 1) / kScanTile;
  // small host-invisible temporaries: allocated once per call of this setup routine
  if ((rc = check(cudaMallocAsync((void**)&bad, sizeof(int), st), "malloc"))) return rc;
  if ((rc = check(cudaMallocAsync((void**)&tmp, sizeof(int64_t) * (n_keys + 1 + tiles + 1), st), "malloc"))) {
    cudaFreeAsync(bad, st);
    return rc;
  }
  int hbad = 0;
  do {
    if ((rc = check(cudaMemsetAsync(bad, 0, sizeof(int), st), "memset"))) break;
    if ((rc = check(cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)n_keys, st), "memset"))) break;
    if (n > 0) k_count_keys<<<grid_for(n, 256), 256, 0, st>>>(n, keys, n_keys, cnt, bad);
    if (n_keys > 0) k_i32_to_i64<<<grid_for(n_keys, 256), 256, 0, st>>>(n_keys, cnt, tmp);
    if ((rc = exclusive_scan_i64(n_keys, tmp, tmp, tmp + n_keys + 1, st))) break;
    k_i64_to_i32<<<grid_for(n_keys + 1, 256), 256, 0, st>>>(n_keys + 1, tmp, ptr);
    if ((rc = check(cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)n_keys, st), "memset"))) break;
    if (n > 0) k_scatter_keys<<<grid_for(n, 256), 256, 0, st>>>(n, keys, n_keys, ptr, cnt, out, payload_div);
    if (n_keys > 0) k_sort_segments<<<grid_for(n_keys, 128), 128, 0, st>>>(n_keys, ptr, out);
    if ((rc = check_launch("group_by_key"))) break;
    if ((rc = check(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st), "memcpy"))) break;
    if ((rc = check(cudaStreamSynchronize(st), "sync"))) break;
    if (hbad) rc = SC_BAD_ARG;
  } while (0);
  cudaFreeAsync(bad, st);
  cudaFreeAsync(tmp, st);
  return rc;
}

// ------------------------------------------------------------------ adjacency
constexpr int kAdjCap = 2048;   // candidate (element, node) pairs per node
constexpr int kAdjWarps = 4;

// bitonic sort of len (power of two) ints in shared memory by one warp, then unique;
// returns number of unique values (compacted at the front).
__device__ int warp_sort_unique(int* s, int len) {
  const int lane = threadIdx.x & 31;
  for (int k = 2; k <= len; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < len; i += 32) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const int a = s[i], b = s[ixj];
          const bool up = (i & k) == 0;
          if ((a > b) == up) {
            s[i] = b;
            s[ixj] = a;
          }
        }
      }
      __syncwarp();
    }
  }
  // unique by a sequential pass in lane 0 (lists are short)
  int m = 0;
  if (lane == 0) {
    int prev = -1;
    for (int i = 0; i < len; ++i) {
      const int x = s[i];
      if (x == 0x7fffffff) break;
      if (x != prev) {
        s[m++] = x;
        prev = x;
      }
    }
  }
  m = __shfl_sync(0xffffffffu, m, 0);
  __syncwarp();
  return m;
}

__global__ void __launch_bounds__(kAdjWarps * 32) k_adjacency(int n_nodes, int n_en, const int* __restrict__ elem,
                                                               const int* __restrict__ inc_ptr,
                                                               const int* __restrict__ inc,
                                                               const int64_t* __restrict__ adj_ptr,
                                                               int* __restrict__ deg, int* __restrict__ adj,
                                                               int* __restrict__ overflow) {
  __shared__ int buf[kAdjWarps][kAdjCap];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int* s = buf[wib];
  for (int a = blockIdx.x * kAdjWarps + wib; a < n_nodes; a += gridDim.x * kAdjWarps) {
    const int b = inc_ptr[a], e = inc_ptr[a + 1];
    const int cand = (e - b) * n_en;
    if (cand > kAdjCap) {
      if (lane == 0) {
        atomicExch(overflow, 1);
        if (!adj) deg[a] = 0;
      }
      continue;
    }
    int len = 32;
    while (len < cand) len <<= 1;
    for (int i = lane; i < len; i += 32) {
      if (i < cand) {
        const int el = inc[b + i / n_en];
        s[i] = elem[(int64_t)el * n_en + (i % n_en)];
      } else {
        s[i] = 0x7fffffff;
      }
    }
    __syncwarp();
    const int m = warp_sort_unique(s, len);
    if (!adj) {
      if (lane == 0) deg[a] = m;
    } else {
      const int64_t o = adj_ptr[a];
      for (int i = lane; i < m; i += 32) adj[o + i] = s[i];
    }
    __syncwarp();
  }
}

// ------------------------------------------------------------------ CSR pattern
__device__ inline int nfree(const int* eqmap, int dim, int node) {
  int c = 0;
  for (int d = 0; d < dim; ++d) c += eqmap[(int64_t)node * dim + d] >= 0;
  return c;
}

// rowlen[eq(a,c)] = sum over neighbours b of nfree(b); one thread per node
__global__ void k_rowlen(int n_nodes, int dim, const int* __restrict__ eqmap, const int64_t* __restrict__ adj_ptr,
                         const int* __restrict__ adj, int64_t* __restrict__ rowlen) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n_nodes; a += gridDim.x * blockDim.x) {
    int64_t len = 0;
    for (int64_t k = adj_ptr[a]; k < adj_ptr[a + 1]; ++k) len += nfree(eqmap, dim, adj[k]);
    for (int c = 0; c < dim; ++c) {
      const int eq = eqmap[(int64_t)a * dim + c];
      if (eq >= 0) rowlen[eq] = len;
    }
  }
}

// one warp per node: write the column list of the node's rows
__global__ void k_fill_cols(int n_nodes, int dim, const int* __restrict__ eqmap, const int64_t* __restrict__ adj_ptr,
                            const int* __restrict__ adj, const int64_t* __restrict__ rowptr, int* __restrict__ cols) {
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  for (int a = blockIdx.x * wpb + wib; a < n_nodes; a += gridDim.x * wpb) {
    const int64_t b0 = adj_ptr[a], b1 = adj_ptr[a + 1];
    int first = -1;
    for (int c = 0; c < dim; ++c) {
      const int eq = eqmap[(int64_t)a * dim + c];
      if (eq >= 0) {
        first = eq;
        break;
      }
    }
    if (first < 0) continue;
    // offsets of neighbour blocks inside the row, computed in chunks of 32 with a warp scan
    int64_t run = 0;
    for (int64_t k0 = b0; k0 < b1; k0 += 32) {
      const int64_t k = k0 + lane;
      const int nb = k < b1 ? adj[k] : -1;
      const int nf = nb >= 0 ? nfree(eqmap, dim, nb) : 0;
      int incl = nf;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      const int64_t off = run + incl - nf;
      if (nb >= 0) {
        int q = 0;
        for (int d = 0; d < dim; ++d) {
          const int eqb = eqmap[(int64_t)nb * dim + d];
          if (eqb < 0) continue;
          for (int c = 0; c < dim; ++c) {
            const int eqa = eqmap[(int64_t)a * dim + c];
            if (eqa >= 0) cols[rowptr[eqa] + off + q] = eqb;
          }
          ++q;
        }
      }
      run += __shfl_sync(0xffffffffu, incl, 31);
    }
  }
}

// ------------------------------------------------------------------ values
// position of node b in the sorted adjacency slice [b0, b1); -1 if absent
__device__ inline int64_t find_sorted(const int* adj, int64_t b0, int64_t b1, int key) {
  int64_t lo = b0, hi = b1;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (adj[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return (lo < b1 && adj[lo] == key) ? lo : -1;
}

// One warp per node a.  Elements of a are walked in ascending order; within an element the
// lanes own distinct (c, lb, d) entries, so each global entry receives its contributions in
// element order.  Column offset of neighbour b inside row (a, c) is recovered from the
// row's own column list (cols are the free eqs of the sorted neighbours).
__global__ void k_assemble(int n_nodes, int n_en, int dim, const int* __restrict__ elem, const int* __restrict__ eqmap,
                           const int* __restrict__ inc_ptr, const int* __restrict__ inc,
                           const int64_t* __restrict__ adj_ptr, const int* __restrict__ adj,
                           const int64_t* __restrict__ rowptr, const int* __restrict__ cols,
                           const double* __restrict__ Ke, const double* __restrict__ Me, double* __restrict__ K,
                           double* __restrict__ M, int* __restrict__ bad) {
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  const int nd = n_en * dim;
  for (int a = blockIdx.x * wpb + wib; a < n_nodes; a += gridDim.x * wpb) {
    const int64_t ab0 = adj_ptr[a], ab1 = adj_ptr[a + 1];
    for (int k = inc_ptr[a]; k < inc_ptr[a + 1]; ++k) {
      const int e = inc[k];
      const int* en = elem + (int64_t)e * n_en;
      int la = -1;
      for (int i = 0; i < n_en; ++i)
        if (en[i] == a) la = i;
      for (int idx = lane; idx < dim * nd; idx += 32) {
        const int c = idx / nd, j = idx - c * nd;
        const int lb = j / dim, d = j - lb * dim;
        const int eqa = eqmap[(int64_t)a * dim + c];
        const int b = en[lb];
        const int eqb = eqmap[(int64_t)b * dim + d];
        if (eqa < 0 || eqb < 0 || la < 0) continue;
        // the row of eqa lists, for every neighbour, its free eqs ascending; eqb is unique
        const int64_t r0 = rowptr[eqa], r1 = rowptr[eqa + 1];
        int64_t lo = r0, hi = r1;
        while (lo < hi) {
          const int64_t mid = (lo + hi) >> 1;
          if (cols[mid] < eqb) lo = mid + 1;
          else hi = mid;
        }
        if (lo >= r1 || cols[lo] != eqb) {
          atomicExch(bad, 1);
          continue;
        }
        const int64_t src = (int64_t)e * nd * nd + (int64_t)(la * dim + c) * nd + j;
        if (K) K[lo] += Ke[src];
        if (M) M[lo] += Me[src];
      }
      __syncwarp();
    }
    (void)ab0;
    (void)ab1;
  }
}

// ------------------------------------------------------------------ Lysmer scatter
__global__ void k_face_rows(int64_t n, int nf, const int* __restrict__ eqs, int* __restrict__ keys) {
  // contribution (f, a, b) -> row eqs[f][a]
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = i / (nf * nf);
    const int a = (int)((i / nf) % nf);
    keys[i] = eqs[f * nf + a];
  }
}

// one thread per row: adds that row's contributions in contribution (= face) order
__global__ void k_lysmer(int nf, const int* __restrict__ eqs, const double* __restrict__ Fm,
                         const double* __restrict__ fct, const double* __restrict__ fct2, int n_eq,
                         const int* __restrict__ row_ptr, const int* __restrict__ order,
                         const int64_t* __restrict__ rowptr, const int* __restrict__ cols, double* __restrict__ Cabs,
                         double* __restrict__ Kabs, int* __restrict__ bad) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_eq; r += gridDim.x * blockDim.x) {
    for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k) {
      const int64_t i = order[k];
      const int64_t f = i / (nf * nf);
      const int b = (int)(i % nf);
      const int eqb = eqs[f * nf + b];
      int64_t lo = rowptr[r], hi = rowptr[r + 1];
      const int64_t end = hi;
      while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (cols[mid] < eqb) lo = mid + 1;
        else hi = mid;
      }
      if (lo >= end || cols[lo] != eqb) {
        atomicExch(bad, 1);
        continue;
      }
      const double F = Fm[i];
      if (Cabs) Cabs[lo] += F * fct[f * nf + b];
      if (Kabs) Kabs[lo] += fabs(F) * fct2[f * nf + b];
    }
  }
}

__global__ void k_combine(int64_t n, double c0, const double* __restrict__ x, double c1, const double* __restrict__ y,
                          double c2, const double* __restrict__ z, double* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double xv = x ? x[i] : 0.0, yv = y ? y[i] : 0.0, zv = z ? z[i] : 0.0;
    out[i] = c0 * xv + (c1 * yv + c2 * zv);
  }
}

int read_flag(int* dflag, cudaStream_t st, int* out) {
  int rc = check(cudaMemcpyAsync(out, dflag, sizeof(int), cudaMemcpyDeviceToHost, st), "memcpy flag");
  if (rc) return rc;
  return check(cudaStreamSynchronize(st), "sync flag");
}

}  // namespace sc

using namespace sc;

extern "C" int64_t sc_scan_work_size(int64_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

extern "C" int sc_exclusive_scan_i64(int64_t n, const int64_t* in, int64_t* out, int64_t* work, void* stream) {
  if (n < 0 || !in || !out || !work) return SC_BAD_ARG;
  return exclusive_scan_i64(n, in, out, work, (cudaStream_t)stream);
}

extern "C" int sc_node_incidence(int n_elem, int n_en, int n_nodes, const int* elem, int* inc_ptr, int* inc,
                                 int* work, void* stream) {
  if (n_elem < 0 || n_en <= 0 || n_nodes <= 0 || !elem || !inc_ptr || !inc || !work) return SC_BAD_ARG;
  return group_by_key((int64_t)n_elem * n_en, elem, n_nodes, n_en, inc_ptr, inc, work, (cudaStream_t)stream);
}

extern "C" int sc_node_adjacency(int n_nodes, int n_en, const int* elem, const int* inc_ptr, const int* inc,
                                 const int64_t* adj_ptr, int* deg, int* adj, void* stream) {
  if (n_nodes <= 0 || n_en <= 0 || !elem || !inc_ptr || !inc) return SC_BAD_ARG;
  if (!adj && !deg) return SC_BAD_ARG;
  if (adj && !adj_ptr) return SC_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int* ovf = nullptr;
  int rc = check(cudaMallocAsync((void**)&ovf, sizeof(int), st), "malloc");
  if (rc) return rc;
  int h = 0;
  do {
    if ((rc = check(cudaMemsetAsync(ovf, 0, sizeof(int), st), "memset"))) break;
    k_adjacency<<<grid_for(n_nodes, kAdjWarps, 152 * 16), kAdjWarps * 32, 0, st>>>(n_nodes, n_en, elem, inc_ptr, inc,
                                                                                   adj_ptr, deg, adj, ovf);
    if ((rc = check_launch("k_adjacency"))) break;
    if ((rc = read_flag(ovf, st, &h))) break;
    if (h) rc = SC_CAPACITY;
  } while (0);
  cudaFreeAsync(ovf, st);
  return rc;
}

extern "C" int sc_csr_pattern(int n_nodes, int dim, const int* eqmap, const int64_t* adj_ptr, const int* adj,
                              const int64_t* rowptr, int64_t* rowlen, int* cols, void* stream) {
  if (n_nodes <= 0 || dim < 2 || dim > 3 || !eqmap || !adj_ptr || !adj) return SC_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (!cols) {
    if (!rowlen) return SC_BAD_ARG;
    k_rowlen<<<grid_for(n_nodes, 128), 128, 0, st>>>(n_nodes, dim, eqmap, adj_ptr, adj, rowlen);
    return check_launch("k_rowlen");
  }
  if (!rowptr) return SC_BAD_ARG;
  k_fill_cols<<<grid_for(n_nodes, 8, 152 * 64), 256, 0, st>>>(n_nodes, dim, eqmap, adj_ptr, adj, rowptr, cols);
  return check_launch("k_fill_cols");
}

extern "C" int sc_assemble_values(int n_nodes, int n_en, int dim, const int* elem, const int* eqmap,
                                  const int* inc_ptr, const int* inc, const int64_t* adj_ptr, const int* adj,
                                  const int64_t* rowptr, const int* cols, const double* Ke, const double* Me,
                                  double* K, double* M, void* stream) {
  if (n_nodes <= 0 || n_en <= 0 || dim < 2 || dim > 3 || !elem || !eqmap || !inc_ptr || !inc || !rowptr || !cols)
    return SC_BAD_ARG;
  if ((K && !Ke) || (M && !Me)) return SC_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int* bad = nullptr;
  int rc = check(cudaMallocAsync((void**)&bad, sizeof(int), st), "malloc");
  if (rc) return rc;
  int h = 0;
  do {
    if ((rc = check(cudaMemsetAsync(bad, 0, sizeof(int), st), "memset"))) break;
    k_assemble<<<grid_for(n_nodes, 8, 152 * 64), 256, 0, st>>>(n_nodes, n_en, dim, elem, eqmap, inc_ptr, inc, adj_ptr,
                                                               adj, rowptr, cols, Ke, Me, K, M, bad);
    if ((rc = check_launch("k_assemble"))) break;
    if ((rc = read_flag(bad, st, &h))) break;
    if (h) rc = SC_BAD_ARG;
  } while (0);
  cudaFreeAsync(bad, st);
  return rc;
}

extern "C" int sc_group_rows(int n_face, int nf, const int* eqs, int n_eq, int* row_ptr, int* order, int* work,
                             void* stream) {
  if (n_face < 0 || nf <= 0 || n_eq <= 0 || !row_ptr || !work || (n_face > 0 && (!eqs || !order))) return SC_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t n = (int64_t)n_face * nf * nf;
  int* keys = nullptr;
  int rc = check(cudaMallocAsync((void**)&keys, sizeof(int) * (n > 0 ? n : 1), st), "malloc");
  if (rc) return rc;
  if (n > 0) k_face_rows<<<grid_for(n, 256), 256, 0, st>>>(n, nf, eqs, keys);
  rc = check_launch("k_face_rows");
  if (!rc) rc = group_by_key(n, keys, n_eq, 1, row_ptr, order, work, st);
  cudaFreeAsync(keys, st);
  return rc;
}

extern "C" int sc_lysmer_values(int n_face, int nf, const int* eqs, const double* Fm, const double* fct,
                                const double* fct2, int n_eq, const int* row_ptr, const int* order,
                                const int64_t* rowptr, const int* cols, double* C_abs, double* K_abs, void* stream) {
  if (n_face < 0 || nf <= 0 || n_eq <= 0 || !row_ptr || !rowptr || !cols) return SC_BAD_ARG;
  if (n_face == 0) return SC_OK;
  if (!eqs || !Fm || !fct || !fct2 || !order) return SC_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int* bad = nullptr;
  int rc = check(cudaMallocAsync((void**)&bad, sizeof(int), st), "malloc");
  if (rc) return rc;
  int h = 0;
  do {
    if ((rc = check(cudaMemsetAsync(bad, 0, sizeof(int), st), "memset"))) break;
    k_lysmer<<<grid_for(n_eq, 128), 128, 0, st>>>(nf, eqs, Fm, fct, fct2, n_eq, row_ptr, order, rowptr, cols, C_abs,
                                                  K_abs, bad);
    if ((rc = check_launch("k_lysmer"))) break;
    if ((rc = read_flag(bad, st, &h))) break;
    if (h) rc = SC_BAD_ARG;
  } while (0);
  cudaFreeAsync(bad, st);
  return rc;
}

__global__ void k_row_sums(int64_t n, const int64_t* __restrict__ rowptr, const double* __restrict__ vals, int absolute,
                           double* __restrict__ out) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) s += absolute ? fabs(vals[k]) : vals[k];
    out[r] = s;
  }
}

extern "C" int sc_csr_row_sums(int64_t n, const int64_t* rowptr, const double* vals, int absolute, double* out,
                               void* stream) {
  if (n < 0 || (n > 0 && (!rowptr || !vals || !out))) return SC_BAD_ARG;
  if (n == 0) return SC_OK;
  k_row_sums<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, rowptr, vals, absolute, out);
  return check_launch("sc_csr_row_sums");
}

extern "C" int sc_combine(int64_t n, double c0, const double* x, double c1, const double* y, double c2,
                          const double* z, double* out, void* stream) {
  if (n < 0 || !out) return SC_BAD_ARG;
  if (n == 0) return SC_OK;
  k_combine<<<grid_for(n, 256, 152 * 32), 256, 0, (cudaStream_t)stream>>>(n, c0, x, c1, y, c2, z, out);
  return check_launch("k_combine");
}

// ------------------------------------------------------------------ scan without allocation
// sc_exclusive_scan_i64_noalloc is the same three-kernel scan as sc_exclusive_scan_i64, for
// callers that must not allocate device memory and cannot hand over a workspace: a host
// whose device memory is all taken by the solver's resident matrices and that accounts for
// every allocation itself, or a binding (cgo, JNI, ctypes without torch) that owns no device
// allocator.  cudaMalloc and cudaFree can also synchronise the whole device, which such a
// caller may not afford between the launches of a running time loop.  The tile sums live in
// this file-scope device array instead; it exists once per device that loads the library.
namespace {

constexpr int64_t kNoAllocTiles = 1024;  // 8 KB of tile sums: n <= 1024 * 8192 = 8,388,608
static_assert(kNoAllocTiles * kScanTile == SC_SCAN_NOALLOC_MAX_N, "header maximum out of date");
static __device__ __align__(256) int64_t g_scan_tile_sums[kNoAllocTiles];

constexpr int kNoAllocDevices = 64;
std::mutex g_tile_sums_lock;
int64_t* g_tile_sums_ptr[kNoAllocDevices] = {};

// Address of the array on the current device, looked up on the first call per device and
// kept for the process (a device reset that recreates the context leaves it stale; the header
// tells callers not to use the entry point after one).
int tile_sums_on_current_device(int64_t** out) {
  int dev = -1;
  int rc = check(cudaGetDevice(&dev), "sc_exclusive_scan_i64_noalloc: current device");
  if (rc) return rc;
  if (dev < 0 || dev >= kNoAllocDevices) {
    set_last_message("sc_exclusive_scan_i64_noalloc: device ordinal beyond the 64 this entry point tracks");
    return SC_CAPACITY;
  }
  std::lock_guard<std::mutex> guard(g_tile_sums_lock);
  if (!g_tile_sums_ptr[dev]) {
    int64_t* ptr = nullptr;
    rc = check(cudaGetSymbolAddress((void**)&ptr, g_scan_tile_sums), "sc_exclusive_scan_i64_noalloc: scratch address");
    if (rc) return rc;
    g_tile_sums_ptr[dev] = ptr;
  }
  *out = g_tile_sums_ptr[dev];
  return SC_OK;
}

}  // namespace

extern "C" int sc_exclusive_scan_i64_noalloc(int64_t n, const int64_t* in, int64_t* out, void* stream) {
  if (n < 0 || !in || !out) return SC_BAD_ARG;
  if (n > SC_SCAN_NOALLOC_MAX_N) {
    char msg[160];
    snprintf(msg, sizeof(msg), "sc_exclusive_scan_i64_noalloc: n = %lld exceeds the maximum of %lld values",
             (long long)n, (long long)SC_SCAN_NOALLOC_MAX_N);
    set_last_message(msg);
    return SC_CAPACITY;
  }
  int64_t* tile_sums = nullptr;
  int rc = tile_sums_on_current_device(&tile_sums);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  // Nothing in the array has to start at zero: every tile sum read below is written earlier
  // in the same call, and the entries past this call's tiles (left by earlier calls) are not read.
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles > 0) k_scan_tiles<<<(unsigned)tiles, kScanThreads, 0, st>>>(n, in, out, tile_sums);
  k_scan_sums<<<1, kScanThreads, 0, st>>>(tiles, tile_sums, out + n);  // also writes out[0] = 0 when n == 0
  if (tiles > 0) k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, out, tile_sums);
  return check_launch("sc_exclusive_scan_i64_noalloc");
}
