// Element integration kernels: Gauss-point Ke/Me for the eight element families and the
// 2D face mass used by the Lysmer boundaries.
//
// Maths: shape functions and gmsh node order of scatter/element_types.py, Gauss rules of
// scatter/discretisation.py:436-497, Jacobian / global derivatives of discretisation.py:107-137
// (3D) and :361-373 (2D), consistent mass discretisation.py:203-222.  The stiffness uses the
// isotropic closed form of B^T D B with the D of scatter/material_models.py:5-43:
//   K[(a,c),(b,d)] = sum_g w_g detJ_g (lam dNa_c dNb_d + mu dNa_d dNb_c + mu delta_cd dNa.dNb)
// which is B^T D B written out for D = lam 1x1 + 2 mu I (engineering shear, Voigt order
// xx,yy,zz,xy,yz,zx as discretisation.py:146-156); plane strain in 2D.
//
// Layout: one warp per element.  Lanes 0..NG-1 each own one Gauss point and write its
// global derivatives dN/dx, N and w*detJ to the warp's shared-memory slice; then the 32
// lanes stride over the (n_en*dim)^2 output entries, so each Ke row is written coalesced.
#include <math.h>

#include "sc_common.cuh"

namespace sc {

enum Family { kQuad = 0, kTri = 1, kTetra = 2 };

template <int ET> struct ElemInfo;
template <> struct ElemInfo<SC_HEXA8> { static constexpr int NN = 8, DIM = 3, FAM = kQuad; };
template <> struct ElemInfo<SC_HEXA20> { static constexpr int NN = 20, DIM = 3, FAM = kQuad; };
template <> struct ElemInfo<SC_TETRA4> { static constexpr int NN = 4, DIM = 3, FAM = kTetra; };
template <> struct ElemInfo<SC_TETRA10> { static constexpr int NN = 10, DIM = 3, FAM = kTetra; };
template <> struct ElemInfo<SC_QUAD4> { static constexpr int NN = 4, DIM = 2, FAM = kQuad; };
template <> struct ElemInfo<SC_QUAD8> { static constexpr int NN = 8, DIM = 2, FAM = kQuad; };
template <> struct ElemInfo<SC_TRI3> { static constexpr int NN = 3, DIM = 2, FAM = kTri; };
template <> struct ElemInfo<SC_TRI6> { static constexpr int NN = 6, DIM = 2, FAM = kTri; };

__host__ __device__ inline int num_gauss(int fam, int dim, int order) {
  if (fam == kQuad) return dim == 3 ? order * order * order : order * order;
  if (fam == kTri) return order == 1 ? 1 : (order == 2 ? 3 : 4);
  return order == 1 ? 1 : 4;
}

__host__ inline bool order_ok(int fam, int order) {
  if (fam == kQuad || fam == kTri) return order >= 1 && order <= 3;
  return order == 1 || order == 2;
}

// Gauss point g of the rule: natural coordinates p[dim] and weight w
// (discretisation.py:436-497; hexahedra loop i1 (u) outermost as discretisation.py:34-38).
__device__ inline void gauss_point(int fam, int dim, int order, int g, double* p, double& w) {
  if (fam == kQuad) {
    double x[3], ww[3];
    if (order == 1) {
      x[0] = 0.0; ww[0] = 2.0;
    } else if (order == 2) {
      const double s = sqrt(1.0 / 3.0);
      x[0] = -s; x[1] = s; ww[0] = 1.0; ww[1] = 1.0;
    } else {
      const double s = sqrt(3.0 / 5.0);
      x[0] = -s; x[1] = 0.0; x[2] = s;
      ww[0] = 5.0 / 9.0; ww[1] = 8.0 / 9.0; ww[2] = 5.0 / 9.0;
    }
    if (dim == 3) {
      const int i = g / (order * order), j = (g / order) % order, k = g % order;
      p[0] = x[i]; p[1] = x[j]; p[2] = x[k];
      w = ww[i] * ww[j] * ww[k];
    } else {
      const int i = g / order, j = g % order;
      p[0] = x[i]; p[1] = x[j];
      w = ww[i] * ww[j];
    }
    return;
  }
  if (fam == kTri) {
    if (order == 1) {
      p[0] = 1.0 / 3.0; p[1] = 1.0 / 3.0; w = 0.5;
    } else if (order == 2) {
      const double a = 1.0 / 6.0, b = 2.0 / 3.0;
      p[0] = (g == 1) ? b : a;
      p[1] = (g == 2) ? b : a;
      w = 1.0 / 6.0;
    } else {
      if (g == 0) { p[0] = 1.0 / 3.0; p[1] = 1.0 / 3.0; w = -27.0 / 96.0; }
      else {
        p[0] = (g == 2) ? 3.0 / 5.0 : 1.0 / 5.0;
        p[1] = (g == 3) ? 3.0 / 5.0 : 1.0 / 5.0;
        w = 25.0 / 96.0;
      }
    }
    return;
  }
  // tetra
  if (order == 1) {
    p[0] = p[1] = p[2] = 0.25; w = 1.0 / 6.0;
  } else {
    const double a = 0.25 - sqrt(5.0) / 20.0, b = 0.25 + 3.0 * sqrt(5.0) / 20.0;
    // columns of discretisation.py:479-486: point g has (x, y, z) = (row0[g], row1[g], row2[g])
    p[0] = (g == 3) ? b : a;
    p[1] = (g == 2) ? b : a;
    p[2] = (g == 1) ? b : a;
    w = 1.0 / 24.0;
  }
}

// Shape functions N[NN] and natural derivatives dN[NN][DIM] (element_types.py).
template <int ET> __device__ void shape(const double* p, double* N, double* dN);

template <> __device__ void shape<SC_HEXA8>(const double* p, double* N, double* dN) {
  const double u = p[0], v = p[1], w = p[2];
  const signed char s[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                               {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const double a = 1.0 + s[n][0] * u, b = 1.0 + s[n][1] * v, c = 1.0 + s[n][2] * w;
    N[n] = a * b * c / 8.0;
    dN[n * 3 + 0] = s[n][0] * b * c / 8.0;
    dN[n * 3 + 1] = s[n][1] * a * c / 8.0;
    dN[n * 3 + 2] = s[n][2] * a * b / 8.0;
  }
}

template <> __device__ void shape<SC_HEXA20>(const double* p, double* N, double* dN) {
  const double x[3] = {p[0], p[1], p[2]};
  const signed char s[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                               {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  for (int n = 0; n < 8; ++n) {
    const double a = 1.0 + s[n][0] * x[0], b = 1.0 + s[n][1] * x[1], c = 1.0 + s[n][2] * x[2];
    const double q = s[n][0] * x[0] + s[n][1] * x[1] + s[n][2] * x[2] - 2.0;
    N[n] = a * b * c * q / 8.0;
    dN[n * 3 + 0] = (s[n][0] * b * c * q + a * b * c * s[n][0]) / 8.0;
    dN[n * 3 + 1] = (s[n][1] * a * c * q + a * b * c * s[n][1]) / 8.0;
    dN[n * 3 + 2] = (s[n][2] * a * b * q + a * b * c * s[n][2]) / 8.0;
  }
  // mid-side nodes 8..19: axis along which the node sits mid-edge, then the signs of the
  // three coordinates (0 on that axis), gmsh order (element_types.py:196-215)
  const signed char m[12][4] = {{0, 0, -1, -1}, {1, -1, 0, -1}, {2, -1, -1, 0}, {1, 1, 0, -1},
                                {2, 1, -1, 0},  {0, 0, 1, -1},  {2, 1, 1, 0},   {2, -1, 1, 0},
                                {0, 0, -1, 1},  {1, -1, 0, 1},  {1, 1, 0, 1},   {0, 0, 1, 1}};
  for (int k = 0; k < 12; ++k) {
    double f[3], df[3];
    for (int d = 0; d < 3; ++d) {
      if (d == m[k][0]) {
        f[d] = 1.0 - x[d] * x[d];
        df[d] = -2.0 * x[d];
      } else {
        f[d] = 1.0 + m[k][1 + d] * x[d];
        df[d] = m[k][1 + d];
      }
    }
    const int n = 8 + k;
    N[n] = f[0] * f[1] * f[2] / 4.0;
    dN[n * 3 + 0] = df[0] * f[1] * f[2] / 4.0;
    dN[n * 3 + 1] = f[0] * df[1] * f[2] / 4.0;
    dN[n * 3 + 2] = f[0] * f[1] * df[2] / 4.0;
  }
}

template <> __device__ void shape<SC_TETRA4>(const double* p, double* N, double* dN) {
  N[0] = 1.0 - p[0] - p[1] - p[2];
  N[1] = p[0]; N[2] = p[1]; N[3] = p[2];
  const double t[12] = {-1, -1, -1, 1, 0, 0, 0, 1, 0, 0, 0, 1};
  for (int i = 0; i < 12; ++i) dN[i] = t[i];
}

template <> __device__ void shape<SC_TETRA10>(const double* p, double* N, double* dN) {
  const double u = p[0], v = p[1], w = p[2], L = 1.0 - u - v - w;
  N[0] = (2 * L - 1) * L; N[1] = (2 * u - 1) * u; N[2] = (2 * v - 1) * v; N[3] = (2 * w - 1) * w;
  N[4] = 4 * u * L; N[5] = 4 * u * v; N[6] = 4 * v * L; N[7] = 4 * w * L; N[8] = 4 * v * w; N[9] = 4 * u * w;
  const double d0 = 4 * u + 4 * v + 4 * w - 3;
  const double t[30] = {d0, d0, d0,
                        4 * u - 1, 0, 0,
                        0, 4 * v - 1, 0,
                        0, 0, 4 * w - 1,
                        4 * L - 4 * u, -4 * u, -4 * u,
                        4 * v, 4 * u, 0,
                        -4 * v, 4 * L - 4 * v, -4 * v,
                        -4 * w, -4 * w, 4 * L - 4 * w,
                        0, 4 * w, 4 * v,
                        4 * w, 0, 4 * u};
  for (int i = 0; i < 30; ++i) dN[i] = t[i];
}

template <> __device__ void shape<SC_QUAD4>(const double* p, double* N, double* dN) {
  const double u = p[0], v = p[1];
  const signed char s[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
  for (int n = 0; n < 4; ++n) {
    const double a = 1.0 + s[n][0] * u, b = 1.0 + s[n][1] * v;
    N[n] = a * b / 4.0;
    dN[n * 2 + 0] = s[n][0] * b / 4.0;
    dN[n * 2 + 1] = s[n][1] * a / 4.0;
  }
}

template <> __device__ void shape<SC_QUAD8>(const double* p, double* N, double* dN) {
  // corners bilinear as written in element_types.py:398-401, mid-sides :402-405
  const double u = p[0], v = p[1];
  shape<SC_QUAD4>(p, N, dN);
  N[4] = (1 - u * u) * (1 - v) / 2; dN[8] = -u * (1 - v); dN[9] = -(1 - u * u) / 2;
  N[5] = (1 + u) * (1 - v * v) / 2; dN[10] = (1 - v * v) / 2; dN[11] = -v * (1 + u);
  N[6] = (1 - u * u) * (1 + v) / 2; dN[12] = -u * (1 + v); dN[13] = (1 - u * u) / 2;
  N[7] = (1 - u) * (1 - v * v) / 2; dN[14] = -(1 - v * v) / 2; dN[15] = -v * (1 - u);
}

template <> __device__ void shape<SC_TRI3>(const double* p, double* N, double* dN) {
  N[0] = 1.0 - p[0] - p[1]; N[1] = p[0]; N[2] = p[1];
  dN[0] = -1; dN[1] = -1; dN[2] = 1; dN[3] = 0; dN[4] = 0; dN[5] = 1;
}

template <> __device__ void shape<SC_TRI6>(const double* p, double* N, double* dN) {
  const double u = p[0], v = p[1], L = 1.0 - u - v;
  N[0] = (2 * L - 1) * L; N[1] = (2 * u - 1) * u; N[2] = (2 * v - 1) * v;
  N[3] = 4 * L * u; N[4] = 4 * u * v; N[5] = 4 * L * v;
  const double t[12] = {1 - 4 * L, 1 - 4 * L, 4 * u - 1, 0, 0, 4 * v - 1,
                        4 * L - 4 * u, -4 * u, 4 * v, 4 * u, -4 * v, 4 * L - 4 * v};
  for (int i = 0; i < 12; ++i) dN[i] = t[i];
}

// Jacobian J[k][d] = sum_n x_n,k dN_n/dxi_d; returns det, writes inverse Ji (J^-1).
template <int DIM> __device__ inline double jac_inverse(const double* J, double* Ji);

template <> __device__ inline double jac_inverse<3>(const double* J, double* Ji) {
  const double c00 = J[4] * J[8] - J[5] * J[7];
  const double c01 = J[5] * J[6] - J[3] * J[8];
  const double c02 = J[3] * J[7] - J[4] * J[6];
  const double det = J[0] * c00 + J[1] * c01 + J[2] * c02;
  const double r = 1.0 / det;
  Ji[0] = c00 * r;
  Ji[1] = (J[2] * J[7] - J[1] * J[8]) * r;
  Ji[2] = (J[1] * J[5] - J[2] * J[4]) * r;
  Ji[3] = c01 * r;
  Ji[4] = (J[0] * J[8] - J[2] * J[6]) * r;
  Ji[5] = (J[2] * J[3] - J[0] * J[5]) * r;
  Ji[6] = c02 * r;
  Ji[7] = (J[1] * J[6] - J[0] * J[7]) * r;
  Ji[8] = (J[0] * J[4] - J[1] * J[3]) * r;
  return det;
}

template <> __device__ inline double jac_inverse<2>(const double* J, double* Ji) {
  const double det = J[0] * J[3] - J[1] * J[2];
  const double r = 1.0 / det;
  Ji[0] = J[3] * r; Ji[1] = -J[1] * r; Ji[2] = -J[2] * r; Ji[3] = J[0] * r;
  return det;
}

constexpr int kElemWarps = 4;  // warps per block

template <int ET>
__global__ void __launch_bounds__(kElemWarps * 32) k_element(int order, int n_elem, const double* __restrict__ coords,
                                                             const double* __restrict__ young,
                                                             const double* __restrict__ poisson,
                                                             const double* __restrict__ density, double* __restrict__ Ke,
                                                             double* __restrict__ Me) {
  constexpr int NN = ElemInfo<ET>::NN, DIM = ElemInfo<ET>::DIM, FAM = ElemInfo<ET>::FAM, ND = NN * DIM;
  const int NG = num_gauss(FAM, DIM, order);
  extern __shared__ double smem[];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // per-warp slice: X[NN*DIM] | G[NG][NN][DIM] | Nv[NG][NN] | wd[NG]
  const int slice = NN * DIM + NG * NN * DIM + NG * NN + NG;
  double* X = smem + (size_t)wib * slice;
  double* G = X + NN * DIM;
  double* Nv = G + NG * NN * DIM;
  double* wd = Nv + NG * NN;
  const int64_t warps_total = (int64_t)gridDim.x * kElemWarps;
  for (int64_t e = (int64_t)blockIdx.x * kElemWarps + wib; e < n_elem; e += warps_total) {
    for (int i = lane; i < NN * DIM; i += 32) X[i] = coords[e * NN * DIM + i];
    __syncwarp();
    if (lane < NG) {
      double p[3] = {0, 0, 0}, w;
      gauss_point(FAM, DIM, order, lane, p, w);
      double N[NN], dN[NN * DIM];
      shape<ET>(p, N, dN);
      double J[DIM * DIM], Ji[DIM * DIM];
#pragma unroll
      for (int k = 0; k < DIM; ++k)
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          double s = 0.0;
          for (int n = 0; n < NN; ++n) s += X[n * DIM + k] * dN[n * DIM + d];
          J[k * DIM + d] = s;
        }
      const double det = jac_inverse<DIM>(J, Ji);
      double* Gg = G + lane * NN * DIM;
      for (int n = 0; n < NN; ++n) {
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
          double s = 0.0;
#pragma unroll
          for (int d = 0; d < DIM; ++d) s += dN[n * DIM + d] * Ji[d * DIM + k];
          Gg[n * DIM + k] = s;
        }
        Nv[lane * NN + n] = N[n];
      }
      wd[lane] = w * det;
    }
    __syncwarp();
    const double E = young[e], nu = poisson[e];
    const double lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    const double mu = E / (2.0 * (1.0 + nu));
    const double rho = density ? density[e] : 0.0;
    for (int idx = lane; idx < ND * ND; idx += 32) {
      const int i = idx / ND, j = idx - (idx / ND) * ND;
      const int a = i / DIM, c = i - a * DIM, b = j / DIM, d = j - b * DIM;
      double sk = 0.0, sm = 0.0;
      for (int g = 0; g < NG; ++g) {
        const double* Ga = G + (g * NN + a) * DIM;
        const double* Gb = G + (g * NN + b) * DIM;
        double kv = lam * Ga[c] * Gb[d] + mu * Ga[d] * Gb[c];
        if (c == d) {
          double dot = 0.0;
#pragma unroll
          for (int k = 0; k < DIM; ++k) dot += Ga[k] * Gb[k];
          kv += mu * dot;
          sm += Nv[g * NN + a] * Nv[g * NN + b] * wd[g];
        }
        sk += kv * wd[g];
      }
      if (Ke) Ke[e * ND * ND + idx] = sk;
      if (Me) Me[e * ND * ND + idx] = (c == d) ? sm * rho : 0.0;
    }
    __syncwarp();
  }
}

template <int ET>
int launch_element(int order, int n_elem, const double* coords, const double* young, const double* poisson,
                   const double* density, double* Ke, double* Me, cudaStream_t st) {
  constexpr int NN = ElemInfo<ET>::NN, DIM = ElemInfo<ET>::DIM, FAM = ElemInfo<ET>::FAM;
  if (!order_ok(FAM, order)) return SC_BAD_ARG;
  if (n_elem <= 0) return SC_OK;
  const int NG = num_gauss(FAM, DIM, order);
  const size_t smem = sizeof(double) * kElemWarps * (size_t)(NN * DIM + NG * NN * DIM + NG * NN + NG);
  if (smem > 48 * 1024) {
    int rc = check(cudaFuncSetAttribute(k_element<ET>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                   "cudaFuncSetAttribute(k_element)");
    if (rc) return rc;
  }
  const unsigned blocks = grid_for(n_elem, kElemWarps, 152 * 128);
  k_element<ET><<<blocks, kElemWarps * 32, smem, st>>>(order, n_elem, coords, young, poisson, density, Ke, Me);
  return check_launch("k_element");
}

// Face mass: one thread per face; F[a][b] = sum_g Na Nb detJ w over the face's 2D rule.
template <int FT>
__global__ void k_face(int order, int n_face, const double* __restrict__ xy, double* __restrict__ Fm) {
  constexpr int NN = ElemInfo<FT>::NN, FAM = ElemInfo<FT>::FAM;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= n_face) return;
  const int NG = num_gauss(FAM, 2, order);
  double X[NN * 2];
  for (int i = 0; i < NN * 2; ++i) X[i] = xy[(int64_t)f * NN * 2 + i];
  double F[NN * NN];
  for (int i = 0; i < NN * NN; ++i) F[i] = 0.0;
  for (int g = 0; g < NG; ++g) {
    double p[3] = {0, 0, 0}, w;
    gauss_point(FAM, 2, order, g, p, w);
    double N[NN], dN[NN * 2];
    shape<FT>(p, N, dN);
    double J[4], Ji[4];
    for (int k = 0; k < 2; ++k)
      for (int d = 0; d < 2; ++d) {
        double s = 0.0;
        for (int n = 0; n < NN; ++n) s += X[n * 2 + k] * dN[n * 2 + d];
        J[k * 2 + d] = s;
      }
    const double wdet = w * jac_inverse<2>(J, Ji);
    for (int a = 0; a < NN; ++a)
      for (int b = 0; b < NN; ++b) F[a * NN + b] += N[a] * N[b] * wdet;
  }
  for (int i = 0; i < NN * NN; ++i) Fm[(int64_t)f * NN * NN + i] = F[i];
}

template <int FT> int launch_face(int order, int n_face, const double* xy, double* Fm, cudaStream_t st) {
  if (!order_ok(ElemInfo<FT>::FAM, order)) return SC_BAD_ARG;
  if (n_face <= 0) return SC_OK;
  k_face<FT><<<(n_face + 127) / 128, 128, 0, st>>>(order, n_face, xy, Fm);
  return check_launch("k_face");
}

}  // namespace sc

using namespace sc;

extern "C" int sc_element_matrices(int etype, int order, int n_elem, const double* coords, const double* young,
                                   const double* poisson, const double* density, double* Ke, double* Me,
                                   void* stream) {
  if (n_elem < 0 || (n_elem > 0 && (!coords || !young || !poisson))) return SC_BAD_ARG;
  if (Me && !density) return SC_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  switch (etype) {
    case SC_HEXA8: return launch_element<SC_HEXA8>(order, n_elem, coords, young, poisson, density, Ke, Me, st);
    case SC_HEXA20: return launch_element<SC_HEXA20>(order, n_elem, coords, young, poisson, density, Ke, Me, st);
    case SC_TETRA4: return launch_element<SC_TETRA4>(order, n_elem, coords, young, poisson, density, Ke, Me, st);
    case SC_TETRA10: return launch_element<SC_TETRA10>(order, n_elem, coords, young, poisson, density, Ke, Me, st);
    case SC_QUAD4: return launch_element<SC_QUAD4>(order, n_elem, coords, young, poisson, density, Ke, Me, st);
    case SC_QUAD8: return launch_element<SC_QUAD8>(order, n_elem, coords, young, poisson, density, Ke, Me, st);
    case SC_TRI3: return launch_element<SC_TRI3>(order, n_elem, coords, young, poisson, density, Ke, Me, st);
    case SC_TRI6: return launch_element<SC_TRI6>(order, n_elem, coords, young, poisson, density, Ke, Me, st);
    default: return SC_BAD_ARG;
  }
}

extern "C" int sc_face_matrices(int ftype, int order, int n_face, const double* xy, double* Fm, void* stream) {
  if (n_face < 0 || (n_face > 0 && (!xy || !Fm))) return SC_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  switch (ftype) {
    case SC_QUAD4: return launch_face<SC_QUAD4>(order, n_face, xy, Fm, st);
    case SC_QUAD8: return launch_face<SC_QUAD8>(order, n_face, xy, Fm, st);
    case SC_TRI3: return launch_face<SC_TRI3>(order, n_face, xy, Fm, st);
    case SC_TRI6: return launch_face<SC_TRI6>(order, n_face, xy, Fm, st);
    default: return SC_BAD_ARG;
  }
}
