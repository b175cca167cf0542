// Seeded random fields for the batched path: log-normal Young's modulus per element and
// realisation.
//
// The reference draws its fields with gstools' SRF (scatter/random_fields.py:59-120), a
// third-party package absent here; its log-normal transform is kept:
//   sigma_ln^2 = ln(1 + (sd/mean)^2), mu_ln = ln(mean^2 / sqrt(mean^2 + sd^2))  (:73-75)
//   E = exp(mu_ln + g(x)) at element centroids                                    (:100-104)
// g is a zero-mean Gaussian field with covariance sigma_ln^2 exp(-(pi/4) |r/l|^2) (axis
// lengths l = (lx, ly, lz)), drawn by the randomisation (spectral) method of Kraichnan
// (1970) / Hesse et al. (2014):
//   g(x) = sqrt(sigma^2 / N) sum_j [Z1_j cos(k_j . x) + Z2_j sin(k_j . x)],
//   k_j,axis ~ N(0, pi / (2 l_axis^2)),  Z ~ N(0, 1),
// with every normal drawn from a counter-based generator (splitmix64 finaliser of
// Steele, Lea & Flood 2014 over (seed, realisation, mode, index), Box-Muller), so a field
// depends only on (seed, realisation) and is reproducible on any device.
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

// modes[r][j] = (k_x, k_y, k_z, Z1, Z2)
__global__ void k_rf_modes(uint64_t seed, int R, int N, double lx, double ly, double lz, float* modes) {
  const double two_pi = 6.283185307179586;
  const double sx = sqrt(M_PI / 2.0) / lx, sy = sqrt(M_PI / 2.0) / ly, sz = sqrt(M_PI / 2.0) / lz;
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
    float* m = modes + q * 5;
    m[0] = (float)(n[0] * sx);
    m[1] = (float)(n[1] * sy);
    m[2] = (float)(n[2] * sz);
    m[3] = (float)n[3];
    m[4] = (float)n[4];
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

extern "C" int sc_rf_modes(uint64_t seed, int R, int n_modes, double lx, double ly, double lz, float* modes,
                           void* stream) {
  if (R <= 0 || n_modes <= 0 || !modes || !(lx > 0) || !(ly > 0) || !(lz > 0)) return SC_BAD_ARG;
  k_rf_modes<<<grid_for((int64_t)R * n_modes, 256), 256, 0, (cudaStream_t)stream>>>(seed, R, n_modes, lx, ly, lz,
                                                                                     modes);
  return check_launch("k_rf_modes");
}

extern "C" int sc_rf_lognormal(int n_pts, const float* xyz, int R, int n_modes, const float* modes, double mu_ln,
                               double sigma_ln, float* out, void* stream) {
  if (n_pts <= 0 || R <= 0 || n_modes <= 0 || !xyz || !modes || !out) return SC_BAD_ARG;
  const int tiles = (n_pts + 255) / 256;
  if ((int64_t)tiles * R > (1ll << 31) - 1) return SC_BAD_ARG;
  k_rf_eval<<<tiles * R, 256, 0, (cudaStream_t)stream>>>(n_pts, xyz, R, n_modes, modes, mu_ln, sigma_ln, out, tiles);
  return check_launch("k_rf_eval");
}
