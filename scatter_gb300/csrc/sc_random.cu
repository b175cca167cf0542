// Seeded random fields for the batched path: log-normal Young's modulus per element and
// realisation.
//
// The reference draws its fields with gstools' SRF (scatter/random_fields.py:59-120), a
// third-party package absent here; its log-normal transform is kept:
//   sigma_ln^2 = ln(1 + (sd/mean)^2), mu_ln = ln(mean^2 / sqrt(mean^2 + sd^2))  (:73-75)
//   E = exp(mu_ln + g(x)) at element centroids                                    (:100-104)
// g is a zero-mean Gaussian field with one of the covariance models the reference offers
// (:79-88), as functions of the scaled distance h = |R^T (x - y) / l| (axis lengths
// l = (lx, ly, lz) in the frame rotated by R):
//   Gaussian     rho = exp(-(pi/4) h^2)
//   Exponential  rho = exp(-h)
//   Matern(nu)   rho = 2^(1-nu) / Gamma(nu) (sqrt(nu) h)^nu K_nu(sqrt(nu) h)
// drawn by the randomisation (spectral) method of Kraichnan (1970) / Hesse et al. (2014):
//   g(x) = sqrt(sigma^2 / N) sum_j [Z1_j cos(k_j . x) + Z2_j sin(k_j . x)],  Z ~ N(0, 1),
// with the wave vectors k_j = R (kappa_j / l) and kappa_j drawn from each model's spectral
// density in scaled coordinates:
//   Gaussian     kappa = sqrt(pi/2) Z3                (normal)
//   Exponential  kappa = Z3 / |Z'|                    (multivariate Cauchy: density ~ (1 + kappa^2)^-(d+1)/2)
//   Matern(nu)   kappa = Z3 sqrt(nu / (2 G)), G ~ Gamma(nu, 1)   (multivariate t, 2 nu degrees
//                of freedom: density ~ (nu + kappa^2)^-(nu + d/2)); G by Marsaglia & Tsang (2000)
// Every uniform comes from a counter-based generator (splitmix64 finaliser of Steele, Lea &
// Flood 2014 over (seed, realisation, mode, index)), normals by Box-Muller, so a field depends
// only on (seed, realisation) and is reproducible on any device.
#include <math.h>

#include "sc_common.cuh"

namespace sc {

__host__ __device__ inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ inline double uniform01(uint64_t seed, int r, int j, int k) {
  uint64_t h = mix64(seed + 0x632BE59BD9B4E019ull * (uint64_t)(r + 1));
  h = mix64(h + (uint64_t)j * 0x9E3779B97F4A7C15ull + (uint64_t)k);
  return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

__device__ inline double normal01(uint64_t seed, int r, int j, int k) {  // Box-Muller, uniforms k, k + 1
  const double u1 = uniform01(seed, r, j, k), u2 = uniform01(seed, r, j, k + 1);
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

// Gamma(a, 1) by Marsaglia & Tsang (2000), a >= 1 directly, a < 1 as Gamma(a + 1) U^(1/a);
// uniforms from index 16 on, 3 per attempt, at most 64 attempts (the acceptance rate is
// above 95 % per attempt, so running out has probability below 1e-80)
__device__ inline double gamma_draw(uint64_t seed, int r, int j, double a) {
  const double boost = a < 1.0 ? pow(uniform01(seed, r, j, 15), 1.0 / a) : 1.0;
  const double aa = a < 1.0 ? a + 1.0 : a;
  const double d = aa - 1.0 / 3.0, c = 1.0 / sqrt(9.0 * d);
  double g = d;
  for (int t = 0; t < 64; ++t) {
    const double x = normal01(seed, r, j, 16 + 3 * t);
    const double v1 = 1.0 + c * x;
    if (v1 <= 0.0) continue;
    const double v = v1 * v1 * v1;
    const double u = uniform01(seed, r, j, 18 + 3 * t);
    if (log(u) < 0.5 * x * x + d - d * v + d * log(v)) {
      g = d * v;
      break;
    }
  }
  return g * boost;
}

struct RfModel {
  int model;        // 0 Gaussian, 1 Exponential, 2 Matern
  double nu;        // Matern smoothness
  double il[3];     // 1 / axis lengths
  double rot[9];    // R, row-major: k = R kappa_scaled
};

// modes[r][j] = (k_x, k_y, k_z, Z1, Z2)
__global__ void k_rf_modes(uint64_t seed, int R, int N, RfModel m, float* modes) {
  const double two_pi = 6.283185307179586;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < (int64_t)R * N;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(q / N), j = (int)(q - (q / N) * N);
    double n[6];
    for (int p = 0; p < 3; ++p) {
      const double u1 = uniform01(seed, r, j, 2 * p), u2 = uniform01(seed, r, j, 2 * p + 1);
      const double rad = sqrt(-2.0 * log(u1));
      n[2 * p] = rad * cos(two_pi * u2);
      n[2 * p + 1] = rad * sin(two_pi * u2);
    }
    double scale;
    if (m.model == 0) {
      scale = sqrt(M_PI / 2.0);
    } else if (m.model == 1) {
      scale = 1.0 / fabs(normal01(seed, r, j, 6));
    } else {
      scale = sqrt(m.nu / (2.0 * gamma_draw(seed, r, j, m.nu)));
    }
    double kl[3];
    for (int a = 0; a < 3; ++a) kl[a] = n[a] * scale * m.il[a];
    float* out = modes + q * 5;
    for (int a = 0; a < 3; ++a)
      out[a] = (float)(m.rot[3 * a] * kl[0] + m.rot[3 * a + 1] * kl[1] + m.rot[3 * a + 2] * kl[2]);
    out[3] = (float)n[3];
    out[4] = (float)n[4];
  }
}

constexpr int kRfChunk = 256;

// out[p][r] = exp(mu_ln + sigma sqrt(1/N) sum_j (Z1 cos + Z2 sin)); one block per
// (realisation, point tile), modes staged through shared memory.
__global__ void k_rf_eval(int n_pts, const float* __restrict__ xyz, int R, int N, const float* __restrict__ modes,
                          double mu_ln, double sigma, float* __restrict__ out, int tiles) {
  __shared__ float sm[kRfChunk * 5];
  const int r = blockIdx.x / tiles, tile = blockIdx.x - (blockIdx.x / tiles) * tiles;
  const int64_t p = (int64_t)tile * blockDim.x + threadIdx.x;
  float x = 0.f, y = 0.f, z = 0.f;
  if (p < n_pts) {
    x = xyz[p * 3];
    y = xyz[p * 3 + 1];
    z = xyz[p * 3 + 2];
  }
  double acc = 0.0;
  const float* mr = modes + (int64_t)r * N * 5;
  for (int j0 = 0; j0 < N; j0 += kRfChunk) {
    const int nc = min(kRfChunk, N - j0);
    __syncthreads();
    for (int i = threadIdx.x; i < nc * 5; i += blockDim.x) sm[i] = mr[(int64_t)j0 * 5 + i];
    __syncthreads();
    float part = 0.f;
    for (int j = 0; j < nc; ++j) {
      const float ph = sm[j * 5] * x + sm[j * 5 + 1] * y + sm[j * 5 + 2] * z;
      float s, c;
      sincosf(ph, &s, &c);
      part = fmaf(sm[j * 5 + 3], c, fmaf(sm[j * 5 + 4], s, part));
    }
    acc += part;
  }
  if (p < n_pts) out[p * R + r] = (float)exp(mu_ln + sigma * sqrt(1.0 / N) * acc);
}

}  // namespace sc

using namespace sc;

extern "C" int sc_rf_modes_model(uint64_t seed, int R, int n_modes, int model, double nu, double lx, double ly,
                                 double lz, const double* rot_host, float* modes, void* stream) {
  if (R <= 0 || n_modes <= 0 || !modes || !(lx > 0) || !(ly > 0) || !(lz > 0)) return SC_BAD_ARG;
  if (model < 0 || model > 2 || (model == 2 && !(nu > 0 && nu <= 1e3))) return SC_BAD_ARG;
  RfModel m;
  m.model = model;
  m.nu = nu;
  m.il[0] = 1.0 / lx;
  m.il[1] = 1.0 / ly;
  m.il[2] = 1.0 / lz;
  for (int i = 0; i < 9; ++i) m.rot[i] = rot_host ? rot_host[i] : (i % 4 == 0 ? 1.0 : 0.0);
  k_rf_modes<<<grid_for((int64_t)R * n_modes, 256), 256, 0, (cudaStream_t)stream>>>(seed, R, n_modes, m, modes);
  return check_launch("k_rf_modes");
}

extern "C" int sc_rf_modes(uint64_t seed, int R, int n_modes, double lx, double ly, double lz, float* modes,
                           void* stream) {
  return sc_rf_modes_model(seed, R, n_modes, 0, 0.0, lx, ly, lz, nullptr, modes, stream);
}

extern "C" int sc_rf_lognormal(int n_pts, const float* xyz, int R, int n_modes, const float* modes, double mu_ln,
                               double sigma_ln, float* out, void* stream) {
  if (n_pts <= 0 || R <= 0 || n_modes <= 0 || !xyz || !modes || !out) return SC_BAD_ARG;
  const int tiles = (n_pts + 255) / 256;
  if ((int64_t)tiles * R > (1ll << 31) - 1) return SC_BAD_ARG;
  k_rf_eval<<<tiles * R, 256, 0, (cudaStream_t)stream>>>(n_pts, xyz, R, n_modes, modes, mu_ln, sigma_ln, out, tiles);
  return check_launch("k_rf_eval");
}
