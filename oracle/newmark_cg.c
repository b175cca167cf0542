/* CPU restatement of the Newmark time loop (oracle / timed CPU baseline; test infrastructure).
 *
 * Same scheme as oracle/newmark.py (PuggleSolvers NewmarkExplicit as driven by
 * scatter/scatter.py:120-159: beta = 1/4, gamma = 1/2, consistent mass, constant effective
 * matrix) in acceleration form, with the per-step linear solve done by Jacobi-preconditioned
 * CG on A = M + dt/2 C + dt^2/4 K instead of a sparse LU: at the benchmark's 1.79M equations
 * the reference's SuperLU factorisation does not fit in host memory.  CSR matrices on a
 * shared pattern, OpenMP over rows.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static double dot(int64_t n, const double* x, const double* y) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int64_t i = 0; i < n; ++i) s += x[i] * y[i];
  return s;
}

int oc_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Runs steps t_begin .. t_begin+n_steps-1 (state t -> t+1).  u, v, a: state in/out.
 * Force table: CSR over time (f_ptr[n_t+1]).  Receivers: out_v[step][n_rec] (may be NULL).
 * Returns 0, or 2 when a solve hit max_iter. */
int oc_newmark_run(int64_t n, const int64_t* rowptr, const int* cols, const double* M, const double* C, const double* K,
                   double dt, double rtol, int max_iter, int t_begin, int n_steps, int n_t, const int64_t* f_ptr,
                   const int* f_eq, const double* f_val, double* u, double* v, double* a, int n_rec, const int* rec,
                   double* out_v, int64_t* iters_out) {
  const int64_t nnz = rowptr[n];
  double* A = (double*)malloc(sizeof(double) * (size_t)nnz);
  double* work = (double*)malloc(sizeof(double) * (size_t)n * 9);
  if (!A || !work) {
    free(A);
    free(work);
    return 1;
  }
  double *vp = work, *up = work + n, *x = work + 2 * n, *r = work + 3 * n, *z = work + 4 * n, *p = work + 5 * n,
         *w = work + 6 * n, *dinv = work + 7 * n, *f = work + 8 * n;
  const double h = 0.5 * dt, q = 0.25 * dt * dt;
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < nnz; ++k) A[k] = M[k] + (h * C[k] + q * K[k]);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double d = 1.0;
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
      if (cols[k] == i) d = A[k];
    dinv[i] = 1.0 / d;
    f[i] = 0.0;
  }
  int status = 0;
  int64_t iters = 0;
  const double tol2 = rtol * rtol;
  for (int s = 0; s < n_steps; ++s) {
    const int t1 = t_begin + s + 1;
    memset(f, 0, sizeof(double) * (size_t)n);
    if (t1 < n_t)
      for (int64_t k = f_ptr[t1]; k < f_ptr[t1 + 1]; ++k) f[f_eq[k]] += f_val[k];
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      vp[i] = v[i] + h * a[i];
      up[i] = u[i] + dt * v[i] + q * a[i];
    }
    double rz = 0.0, bb = 0.0, rr = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : rz, bb, rr)
    for (int64_t i = 0; i < n; ++i) {
      double sr = 0.0, sa = 0.0;
      for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
        const int c = cols[k];
        sr += C[k] * vp[c] + K[k] * up[c];
        sa += A[k] * a[c];
      }
      const double rhs = f[i] - sr;
      r[i] = rhs - sa;
      x[i] = a[i];
      z[i] = dinv[i] * r[i];
      p[i] = z[i];
      rz += r[i] * z[i];
      bb += rhs * rhs;
      rr += r[i] * r[i];
    }
    int it = 0;
    while (!(rr <= tol2 * bb)) {
      if (it >= max_iter) {
        status = 2;
        break;
      }
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) {
        double sw = 0.0;
        for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) sw += A[k] * p[cols[k]];
        w[i] = sw;
      }
      const double pw = dot(n, p, w);
      if (!(pw > 0.0)) {
        status = 3;
        break;
      }
      const double alpha = rz / pw;
      double rzn = 0.0;
      rr = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : rzn, rr)
      for (int64_t i = 0; i < n; ++i) {
        x[i] += alpha * p[i];
        r[i] -= alpha * w[i];
        z[i] = dinv[i] * r[i];
        rzn += r[i] * z[i];
        rr += r[i] * r[i];
      }
      const double beta = rzn / rz;
      rz = rzn;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
      ++it;
    }
    iters += it;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      u[i] = up[i] + q * x[i];
      v[i] = vp[i] + h * x[i];
      a[i] = x[i];
    }
    if (out_v && rec)
      for (int j = 0; j < n_rec; ++j) out_v[(int64_t)s * n_rec + j] = v[rec[j]];
  }
  if (iters_out) *iters_out = iters;
  free(A);
  free(work);
  return status;
}
