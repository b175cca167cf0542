/*
 * scatter_gb300 -- C ABI of the GB300 (sm_103a) finite-element wave-propagation path.
 *
 * The reference (PlatypusBytes/scatter) is pure Python; its hot path is the element
 * integration + assembly in scatter/system_matrix.py, the Lysmer boundaries and Rayleigh
 * damping in the same file, and the Newmark time loop that scatter/scatter.py:120-159
 * drives through PuggleSolvers.  Each entry point below replaces one of those pieces; the
 * reference calls them through a ctypes binding (scatter_gb300/_native.py loads this library
 * and raises on any non-zero status).
 *
 * Conventions
 *   - every pointer is a DEVICE pointer unless its name ends in _host;
 *   - every function works on `stream` (a cudaStream_t passed as void*) and returns a status
 *     code (SC_*).  The time-loop calls (sc_newmark_run) allocate nothing; the one-off setup
 *     calls that need small temporaries or a flag read-back (incidence, adjacency, values,
 *     Lysmer grouping) take them from the stream-ordered allocator and synchronise `stream`;
 *   - doubles are IEEE binary64; integer index arrays are int32 unless typed int64_t;
 *   - equation numbers follow the reference (scatter/mesher.py:276-310): node-major,
 *     DOF-minor over the node list, fixed DOFs excluded (encoded here as -1).
 */
#ifndef SCATTER_GB300_H
#define SCATTER_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (the Python layer raises RuntimeError(code, text)) */
#define SC_OK 0
#define SC_BAD_ARG 1
#define SC_NOT_CONVERGED 2
#define SC_BREAKDOWN 3
#define SC_CAPACITY 4
#define SC_CUDA_ERROR 5

/* element type codes: element_types.py classes HexEight, HexTwenty, TetraFour, TetraTen,
 * QuadFour, QuadEight, TriThree, TriSix (gmsh node order) */
#define SC_HEXA8 0
#define SC_HEXA20 1
#define SC_TETRA4 2
#define SC_TETRA10 3
#define SC_QUAD4 4
#define SC_QUAD8 5
#define SC_TRI3 6
#define SC_TRI6 7

int sc_version(void);
const char* sc_status_string(int status);
/* last CUDA error text recorded by a failing call on this host thread */
const char* sc_last_error(void);

/* ------------------------------------------------------------------ element integration
 * Replaces VolumeElement/SurfaceElement.generate + compute_stiffness + compute_mass
 * (scatter/discretisation.py:83-222 and :241-418) with the isotropic D of
 * scatter/material_models.py:5-43, as called per element in
 * GenerateMatrix.generate_stiffness_and_mass (scatter/system_matrix.py:55-85).
 *   coords  [n_elem][n_en][dim]   element node coordinates (3D: x,y,z; 2D: x,y)
 *   young, poisson, density [n_elem]
 *   Ke, Me  [n_elem][n_en*dim][n_en*dim]  (row-major; either may be NULL)
 *   order   Gauss order per axis (discretisation.py:436-497): quad 1..3, tri 1..3, tetra 1..2 */
int sc_element_matrices(int etype, int order, int n_elem, const double* coords, const double* young,
                        const double* poisson, const double* density, double* Ke, double* Me, void* stream);

/* Lysmer face mass F[a][b] = sum_g Na Nb detJ w on 2D faces (quad4, quad8, tri3, tri6), the
 * matrix of SurfaceElement.compute_abs_bound (scatter/discretisation.py:420-433) without its
 * 2-DOF expansion.  xy [n_face][nf][2] in-plane coordinates in the caller's node order. */
int sc_face_matrices(int ftype, int order, int n_face, const double* xy, double* Fm, void* stream);

/* ------------------------------------------------------------------ assembly
 * Replaces the dict accumulation + COO->lil of GenerateMatrix.generate_stiffness_and_mass
 * (scatter/system_matrix.py:87-121).  The sparsity pattern is the element graph over free
 * DOFs with rows and columns sorted (the reference's M pattern); values are summed per
 * entry in element order, as the reference's defaultdict does.  Deterministic, no atomics
 * on values.
 *
 * Step 1: node -> element incidence (grouped, element ids ascending per node).
 *   elem [n_elem][n_en] 0-based node indices.  inc_ptr [n_nodes+1], inc [n_elem*n_en],
 *   work [n_nodes] int32 scratch. */
int sc_node_incidence(int n_elem, int n_en, int n_nodes, const int* elem, int* inc_ptr, int* inc, int* work,
                      void* stream);

/* Step 2: node adjacency (sorted unique neighbour nodes, self included).
 *   pass 0 (adj == NULL): writes deg[n_nodes]; pass 1: fills adj using adj_ptr [n_nodes+1]
 *   (exclusive prefix of deg, e.g. from sc_exclusive_scan_i64).  Capacity: at most 2048
 *   candidate (element, node) pairs per node, else SC_CAPACITY. */
int sc_node_adjacency(int n_nodes, int n_en, const int* elem, const int* inc_ptr, const int* inc,
                      const int64_t* adj_ptr, int* deg, int* adj, void* stream);

/* exclusive prefix sum of n int64 values (out[n] = total); in == out allowed.
 * work: int64 scratch of at least sc_scan_work_size(n) elements. */
int64_t sc_scan_work_size(int64_t n);
int sc_exclusive_scan_i64(int64_t n, const int64_t* in, int64_t* out, int64_t* work, void* stream);

/* The same scan without a workspace and without allocating (no counterpart in the
 * reference, which has no device code).  For callers that must not allocate device memory:
 * a host that keeps every byte of HBM for the solver's resident matrices and accounts for
 * each allocation itself, or a binding (cgo, JNI, ctypes without torch) with no device
 * allocator of its own; cudaMalloc/cudaFree can also synchronise the device mid-loop.  The
 * tile sums go to one fixed 8 KB device array per device instead, so
 *   - n is at most SC_SCAN_NOALLOC_MAX_N; larger n returns SC_CAPACITY (message in
 *     sc_last_error) before any launch;
 *   - the first call on a device looks up that array's address (cudaGetSymbolAddress) with
 *     the device current and keeps it for the life of the process; make that first call
 *     before any stream capture on the device.  A cudaDeviceReset (or anything else that
 *     tears down and recreates the device's primary context) reloads the module and leaves
 *     the kept address stale, so do not use this entry point after one;
 *   - every call shares the array, which keeps what the last call wrote; nothing in it needs
 *     to start at zero.  Calls whose work overlaps on the GPU (different streams, or another
 *     host thread, without ordering between them) race on it: order them.
 * It calls no cudaMalloc, cudaFree or allocating library routine. */
#define SC_SCAN_NOALLOC_MAX_N 8388608LL
int sc_exclusive_scan_i64_noalloc(int64_t n, const int64_t* in, int64_t* out, void* stream);

/* Step 3: CSR rows over free DOFs.  eqmap [n_nodes][dim] (-1 = fixed).
 *   rowlen [n_eq] (pass: cols == NULL) then cols [nnz] using rowptr [n_eq+1]. */
int sc_csr_pattern(int n_nodes, int dim, const int* eqmap, const int64_t* adj_ptr, const int* adj,
                   const int64_t* rowptr, int64_t* rowlen, int* cols, void* stream);

/* Step 4: values.  Ke/Me as from sc_element_matrices; K, M [nnz] are overwritten. */
int sc_assemble_values(int n_nodes, int n_en, int dim, const int* elem, const int* eqmap, const int* inc_ptr,
                       const int* inc, const int64_t* adj_ptr, const int* adj, const int64_t* rowptr,
                       const int* cols, const double* Ke, const double* Me, double* K, double* M, void* stream);

/* ------------------------------------------------------------------ Lysmer + Rayleigh
 * Replaces the scatter of GenerateMatrix.absorbing_boundaries (scatter/system_matrix.py:355-376).
 * For face f with sorted equation numbers eqs[f][a] (a < nf), face matrix Fm[f][a][b] and
 * per-column factors fct[f][b] (dashpot rho*v) and fct2[f][b] (spring Ec or G):
 *   C_abs[eqs[a], eqs[b]] += Fm[a][b] * fct[b];  K_abs[..] += |Fm[a][b]| * fct2[b]
 * accumulated per entry in face order.  Contributions are grouped by row with
 * sc_group_rows (row_ptr [n_eq+1], order [n_face*nf*nf]); work [n_eq] int32 scratch. */
int sc_group_rows(int n_face, int nf, const int* eqs, int n_eq, int* row_ptr, int* order, int* work, void* stream);
int sc_lysmer_values(int n_face, int nf, const int* eqs, const double* Fm, const double* fct, const double* fct2,
                     int n_eq, const int* row_ptr, const int* order, const int64_t* rowptr, const int* cols,
                     double* C_abs, double* K_abs, void* stream);

/* out[i] = c0*x[i] + (c1*y[i] + c2*z[i]) for i < n (x, y or z may be NULL = 0).
 * Rayleigh: C = C_abs + (alpha M + beta K) (scatter/system_matrix.py:189-198);
 * Lysmer spring: K = K0 + K_abs / k_div (system_matrix.py:376). */
/* out[r] = sum of row r of a CSR matrix (|values| when absolute != 0), summed in column order
 * (deterministic): the row-sum lumped mass of the explicit scheme (no reference counterpart;
 * the reference keeps the consistent mass, scatter/discretisation.py:203-222). */
int sc_csr_row_sums(int64_t n, const int64_t* rowptr, const double* vals, int absolute, double* out, void* stream);
int sc_combine(int64_t n, double c0, const double* x, double c1, const double* y, double c2, const double* z,
               double* out, void* stream);

/* ------------------------------------------------------------------ Newmark time loop
 * Replaces the PuggleSolvers NewmarkExplicit loop the reference drives from
 * scatter/scatter.py:133-159 (average acceleration, beta = 1/4, gamma = 1/2, consistent
 * mass, constant effective matrix).  Each step solves, for the new acceleration x,
 *     A x = f(t) - C vp - K up,   A = M + dt/2 C + dt^2/4 K,
 *     vp = v + dt/2 a,  up = u + dt v + dt^2/4 a,
 * then u = up + dt^2/4 x, v = vp + dt/2 x, a = x -- the same update as the reference's
 * K^ u = rhs form.  The solve is Jacobi-preconditioned CG on A to ||r|| <= rtol ||rhs||
 * (FP64 dot products, deterministic reductions), warm-started from the polynomial
 * extrapolation of the previous accelerations, as sc_nb_set_predictor describes.  One step
 * is one CUDA graph launch with a device-side conditional loop.
 *
 * The caller owns every buffer.  sc_newmark_workspace_doubles() gives the scratch size.
 * Force table (CSR over time): f_ptr [n_t+1], f_eq [f_ptr[n_t]], f_val [..]: the force at
 * step t is sum over k in [f_ptr[t], f_ptr[t+1]) of f_val[k] e_{f_eq[k]}
 * (Force.update_load_at_t, scatter/force_external.py:55-74).
 * Output: every out_interval steps (step 0 included) the solver writes u, v, a at the
 * n_rec equations rec_eq into out_u/out_v/out_a [n_out][n_rec] (any may be NULL).
 */
typedef struct sc_newmark sc_newmark;

int64_t sc_newmark_workspace_doubles(int64_t n_eq, int64_t n_blocks_hint);
int sc_newmark_create(sc_newmark** h, int64_t n_eq, const int64_t* rowptr, const int* cols, const double* M,
                      const double* C, const double* K, double* A, double dt, double rtol, int max_iter,
                      double* u, double* v, double* a, double* workspace, int64_t workspace_doubles, void* stream);
int sc_newmark_set_force(sc_newmark* h, int n_t, const int64_t* f_ptr, const int* f_eq, const double* f_val);
int sc_newmark_set_output(sc_newmark* h, int out_interval, int n_rec, const int* rec_eq, double* out_u,
                          double* out_v, double* out_a, int64_t n_out);
/* a0 = M^-1 (f(0) - C v - K u) by CG on M (scatter/scatter.py:158 numerical.update(0)) and
 * writes the step-0 output row.  Synchronous. */
int sc_newmark_initial_acceleration(sc_newmark* h);
/* run steps t = t_begin .. t_end-1 -> states t+1; asynchronous (graph launches) */
int sc_newmark_run(sc_newmark* h, int t_begin, int t_end);
/* Warm start of each step (no reference counterpart), as sc_nb_set_predictor: order 1..8
 * fixed, 0 adaptive (the default); 1..8 then 0 keeps the history entries that are current. */
int sc_newmark_set_predictor(sc_newmark* h, int order);
/* options bit 0: run the PCG SpMV in FP64 (one FP64 FMA per stored value) instead of the
 * default FP32-pair arithmetic (A and M copied once as hi + lo FP32 pairs, 8 bytes per value
 * like FP64, products and the row sum by exact TwoProd/TwoSum, about 48 bits; the residual,
 * dot products and state stay FP64).  bit 1: no cap on the warm-start order at kinks of the
 * force history (the cap is on by default, as for sc_nb_set_options bit 5).  Options outside
 * 0..3 are rejected.  No reference counterpart. */
int sc_newmark_set_options(sc_newmark* h, int options);
/* the controller's current warm-start order and the steps whose order the force history
 * capped (synchronises) */
int sc_newmark_warm_start_status(sc_newmark* h, int* order, int64_t* capped_steps);
/* synchronous: CG status of the run so far (SC_OK / SC_NOT_CONVERGED / SC_BREAKDOWN),
 * total and maximum CG iterations per step */
int sc_newmark_status(sc_newmark* h, int64_t* total_iters, int* max_iters_per_step);
/* asynchronous form, as sc_nb_status_to */
int sc_newmark_status_to(sc_newmark* h, int64_t* dev3);
/* Timing aid: launches the step loop's SpMV kernel (w = A p, with its p.w partials) `reps`
 * times on the solver's stream between CUDA events, outside any graph; returns the mean
 * device time per launch and the algorithmic bytes of one launch (12 B per stored entry +
 * row pointers + one read of p + the write of w).  Touches only scratch vectors. */
int sc_newmark_time_spmv(sc_newmark* h, int reps, float* ms_per_launch, int64_t* bytes_per_launch);
int sc_newmark_destroy(sc_newmark* h);

/* ------------------------------------------------------------------ random fields
 * Input of the batched path (the reference draws per-element fields with gstools' SRF,
 * scatter/random_fields.py:59-120, and maps them log-normally, :73-77).  The randomisation
 * (spectral) method with n_modes modes per realisation, drawn from a counter-based generator
 * so a field depends only on (seed, r).
 *   sc_rf_modes_model: the covariance models of random_fields.py:79-86 as functions of the
 *                    scaled distance h = |R^T (x - y) / l|: model 0 Gaussian exp(-(pi/4) h^2),
 *                    1 Exponential exp(-h), 2 Matern(nu); rot_host: 9 doubles, row-major R
 *                    (the rotation by `angles`, :80-86), NULL for none
 *   sc_rf_modes:     the Gaussian model without rotation
 *   sc_rf_lognormal: out [n_pts][R] = exp(mu_ln + sigma_ln g_r(x_p)), xyz [n_pts][3] float32
 * modes [R][n_modes][5] (k_x, k_y, k_z, Z1, Z2), float32 */
int sc_rf_modes_model(uint64_t seed, int R, int n_modes, int model, double nu, double lx, double ly, double lz,
                      const double* rot_host, float* modes, void* stream);
int sc_rf_modes(uint64_t seed, int R, int n_modes, double lx, double ly, double lz, float* modes, void* stream);
int sc_rf_lognormal(int n_pts, const float* xyz, int R, int n_modes, const float* modes, double mu_ln,
                    double sigma_ln, float* out, void* stream);

/* ------------------------------------------------------------------ node-block Newmark
 * The same time loop as sc_newmark_* for matrices assembled by this library from a mesh
 * (node adjacency known), on a node-block layout: unknowns in slot space (slot = node*dim +
 * dof, fixed DOFs kept as decoupled zero slots), K and A = M + dt/2 C + dt^2/4 K as dim x dim
 * FP64 blocks over the node adjacency (one plane per block component), the consistent mass
 * as one scalar per node pair, and Rayleigh damping C = Cabs + alpha M + beta K with the
 * Lysmer dashpots Cabs as a small slot-space CSR (scatter/system_matrix.py:166-198,375).
 * Each step solves A x = f - C vp - K up by PCG preconditioned with a factorised sparse
 * approximate inverse G^T G of A (factor on the lower node pattern, built on the GPU in FP32 and
 * applied from FP16 planes scaled by a power of two),
 * warm-started from the quadratic extrapolation of the acceleration history, to
 * ||r|| <= rtol ||rhs||.  eqmap [n_nodes][dim] (-1 fixed); rowptr/cols/K/M/C the eq-space
 * CSR from sc_csr_pattern + sc_assemble_values (+ Lysmer / Rayleigh); cab_* the Lysmer
 * dashpot matrix in slot space (n_cab entries).  u, v, a: slot-space state [n_nodes*dim].
 * Force table and receivers use slot indices.  workspace: sc_nb_workspace_bytes(), 256-byte
 * aligned.  precond: 0 = FSAI (rows whose pattern exceeds 63 slots use a Jacobi row, counted
 * in sc_nb_status), 1 = Jacobi (the FSAI factor restricted to the diagonal). */
typedef struct sc_nb_newmark sc_nb_newmark;
int64_t sc_nb_workspace_bytes(int n_nodes, int dim, int64_t nnzb);
int sc_nb_create(sc_nb_newmark** h, int n_nodes, int dim, const int* eqmap, const int64_t* adj_ptr, const int* adj,
                 int64_t nnzb, const int64_t* rowptr, const int* cols, const double* K, const double* M,
                 const double* C, int64_t n_cab, const int64_t* cab_ptr, const int* cab_col, const double* cab_val,
                 double alpha, double beta, double dt, double rtol, int max_iter, int precond, double* u, double* v,
                 double* a, void* workspace, int64_t workspace_bytes, void* stream);
/* Warm start of each Newmark step (no reference counterpart): the PCG starts from the
 * polynomial extrapolation of order p of the previous accelerations,
 * x0 = sum_{k=0..p} (-1)^k C(p+1, k+1) a_{n-k} (p = 2: 3 a_n - 3 a_{n-1} + a_{n-2}).  order 1..8
 * fixes p; 0 (the default) adapts it on the device: starting from 6 it moves to a neighbouring
 * order while the mean PCG iterations over windows of 16 steps fall, steps back when they
 * rise, and holds 8 windows before probing again.  The order changes the iteration count,
 * not the answer, which meets the same tolerance. */
int sc_nb_set_predictor(sc_nb_newmark* h, int order);
/* options bit 0: run the PCG SpMV in FP64 instead of the default FP32-pair arithmetic
 * (A as hi + lo FP32 pairs, exact TwoProd/TwoSum accumulation, ~2^-46 relative per product;
 * the residual, dot products and state stay FP64).  bit 1: run the explicit scheme in FP64
 * instead of its default FP32-pair state and products (sc_nb_explicit_run); the adjoint needs
 * the default.  bit 2: always form the step's residual r = b - A x0 in FP64 (K q1 and the mass
 * term in FP64, A x0 in pairs).  By default, with the pair SpMV, the residual is formed in one
 * pass over K and mass pair planes as f - K (q1 + aK x0) - M (q2 + aM x0) - Cabs (y1 + aC x0),
 * with A = aM M + aK K + aC Cabs (~48 bits per term, no FP64 product); a step that finds the
 * elastic and inertial terms cancelling the load by more than 30x (slow motion) switches every
 * later step to the FP64 residual, see sc_nb_residual_fp64.
 * The FP32 matrix: with the pair SpMV, a step whose initial residual is small runs its PCG on
 * Ah = the pairs' hi parts alone (4 B per value instead of 8).  With Al = A - Ah and
 * L = sqrt(||Al||_1 ||Al||_inf) >= ||Al||_2 (computed at creation), the true residual of x
 * differs from the PCG's recursive one by -Al (x - x0), so the loop stops at
 * |r| + L |x - x0| <= rtol |b|: the answer meets the same tolerance.  A step uses Ah when the
 * previous step's |x - x0| / |r0|, applied to this step's r0, keeps L |x - x0| below
 * rtol |b| / 16; a step that starts on the pairs switches to Ah (continuing the CG, x and r
 * becoming the new x0 and r0) once |r| is that small.  If the bound passes rtol |b| / 2 during
 * the solve, the PCG restarts from x0 with the pairs and stays there for the step.
 * bit 3: never use Ah.  bit 4: start every step on Ah (exercises the restart).
 * bit 5: no cap on the warm-start order from the force history.  By default each step takes
 * the largest order, up to the controller's, whose extrapolation of the force table itself
 * reproduces the newest row to 1e-6 of the rows' largest entry: a window of
 * accelerations that straddles a kink in the load (the end of a ramp, a load that starts to
 * move) extrapolates badly, and a lower order whose window lies after the kink does better.
 * The cap changes the iteration count, not the answer.
 * Bits 3 and 4 together, and options outside 0..63, are rejected. */
int sc_nb_set_options(sc_nb_newmark* h, int options);
/* the controller's current warm-start order and the steps whose order the force history
 * capped (synchronises) */
int sc_nb_warm_start_status(sc_nb_newmark* h, int* order, int64_t* capped_steps);
/* steps whose PCG started on the FP32 matrix, steps that switched to it during the solve,
 * restarts in pairs, and L (synchronises) */
int sc_nb_a32_status(sc_nb_newmark* h, int64_t* a32_steps, int64_t* switched, int64_t* restarts,
                     double* lo_norm);
/* Whether the step's residual runs in FP64 (always with option bit 2 or the FP64 SpMV, else
 * once the pair residual has handed over); synchronises the stream (no reference
 * counterpart). */
int sc_nb_residual_fp64(sc_nb_newmark* h, int* fp64);
int sc_nb_set_force(sc_nb_newmark* h, int n_t, const int64_t* f_ptr, const int* f_slot, const double* f_val);
int sc_nb_set_output(sc_nb_newmark* h, int out_interval, int n_rec, const int* rec_slot, double* out_u,
                     double* out_v, double* out_a, int64_t n_out);
/* steps t_begin .. t_end-1 (asynchronous graph launches) */
int sc_nb_run(sc_nb_newmark* h, int t_begin, int t_end);
int sc_nb_status(sc_nb_newmark* h, int64_t* total_iters, int* max_iters_per_step, int* fsai_fallback_rows);
/* asynchronous form: status, total iterations and the largest per-step count written to dev3
 * (3 int64 in device memory) in stream order behind the queued steps; no synchronisation */
int sc_nb_status_to(sc_nb_newmark* h, int64_t* dev3);
/* timing aid: the step loop's block SpMV (w = A p) launched `reps` times between CUDA events */
int sc_nb_time_spmv(sc_nb_newmark* h, int reps, float* ms_per_launch, int64_t* bytes_per_launch);
/* the same with a32 = 1: the SpMV form that applies the FP32 matrix (A's hi planes) alone */
int sc_nb_time_spmv_a32(sc_nb_newmark* h, int a32, int reps, float* ms_per_launch, int64_t* bytes_per_launch);
/* Explicit central-difference steps on the same handle (no reference counterpart: the
 * reference's mass is always consistent):
 *   a_n = M_L^-1 (f_n - K (u_n + beta v_{n-1/2}) - alpha M_L v_{n-1/2} - Cabs v_{n-1/2}),
 *   v_{n+1/2} = v_{n-1/2} + dt a_n,  u_{n+1} = u_n + dt v_{n+1/2},
 * M_L the row-sum lumped mass (or sc_nb_set_lumped_mass); one fused kernel per step over the
 * sliced-ELL K.  By default u, v, w, the force and the mass terms are FP32 (hi, lo) pairs
 * (~48 significant bits, no FP64 instruction in the step; the FP64 u, v are split at the start
 * and joined at the end of a run).  Receivers record u_{n+1} and v_{n+1/2}.  Conditionally
 * stable (dt below the lumped-mass CFL limit).  The first call allocates the scheme's extra
 * vectors (setup); later calls allocate nothing. */
int sc_nb_explicit_run(sc_nb_newmark* h, int t_begin, int t_end);
/* The explicit scheme's lumped mass set by the caller (slot space, FP64, device; fixed slots
 * ignored), e.g. a diagonal-scaled mass for element types whose consistent-mass row sums are
 * not positive (the reference's 4-point tetra10 mass has negative corner row sums).  No
 * reference counterpart. */
int sc_nb_set_lumped_mass(sc_nb_newmark* h, const double* ml);
/* Autotuner of the explicit step (no reference counterpart): threads per node row (1, 2, 4)
 * chosen by timing `reps` launches of each candidate on the handle; leaves the force entries,
 * receivers and the caller's u, v as they were.  Pair arithmetic only.  Reports the choice and
 * its time per step. */
int sc_nb_tune_explicit(sc_nb_newmark* h, int reps, int* tpr_chosen, float* ms_per_step);
/* timing aid: the explicit step kernel alone, `reps` launches between CUDA events */
int sc_nb_time_explicit(sc_nb_newmark* h, int reps, float* ms_per_step);
/* Adjoint of the explicit scheme (no reference counterpart): misfit
 *   J = 1/2 sum_{n=1..n_steps} sum_r (v_n[rec_slot[r]] - target[n][r])^2
 * of the receiver velocities of a run from rest (sc_nb_explicit_run semantics, the handle's
 * force table), and dJ/dE_e, dJ/drho_e for per-element Young's modulus and density, with
 *   K = sum_e E_e K1_e + Lysmer springs, M_L = sum_e rho_e ml1_e, Lysmer dashpots ~ sqrt(rho_e E_e)
 * (the operators the handle was built from must be these at the given young/rho).  Forward
 * with FP32-pair checkpoints every `checkpoint` steps; the reverse sweep (last segment
 * first) runs each backward step fused with a recompute step of the segment before it (one
 * kernel per pair of steps) and one element-gradient kernel per segment, all on the handle's
 * stream; gradients accumulated per element in step order (deterministic, independent of the
 * checkpoint interval).  Descriptor fields:
 *   elem [n_elem][n_en] node indices; ke_type [n_elem] -> ke1 [types][3 n_en][3 n_en] FP32
 *   unit-E element stiffness; young, rho [n_elem]; ml1 [n_elem][n_en][3] FP32 unit lumped mass
 *   (free columns); l_eptr [n_elem+1], l_row, l_col (slots), l_c, l_s (FP32): the element's
 *   Lysmer dashpot and spring entries at the current parameters.  3D only.  grad_E, grad_rho [n_elem]
 *   device outputs; J_host may be NULL.  Allocates its checkpoint buffers (setup). */
typedef struct sc_adj_desc sc_adj_desc;
int sc_nb_adjoint(sc_nb_newmark* h, const sc_adj_desc* desc, double* J_host, double* grad_E, double* grad_rho);
/* device time of the last sc_nb_adjoint call's phases, ms: [0] forward with checkpoints,
 * [1] recompute of the last segment (alone), [2] the rest of the reverse sweep (backward
 * steps fused with the previous segment's recompute, element gradients), [3] the whole
 * reverse sweep, [1] + [2] */
int sc_nb_adjoint_timings(sc_nb_newmark* h, float* ms4);
/* testing aid: y = Op x in slot space; which = 0: A, 1: K, 2: consistent mass, 3: the
 * preconditioner G^T G, 4: Lysmer dashpots.  Synchronous; call between steps. */
int sc_nb_apply(sc_nb_newmark* h, int which, const double* x, double* y);
int sc_nb_destroy(sc_nb_newmark* h);

/* ------------------------------------------------------------------ batched realisations
 * R realisations of the per-element Young's modulus (the reference's random-field input,
 * scatter/random_fields.py:109-118, one material per element) advanced together with the
 * explicit lumped-mass scheme of sc_nb_explicit_run: K_r = sum_e E_{e,r} K1_e, with K1_e the
 * element stiffness at E = 1 (sc_element_matrices with young = 1), shared density and Poisson
 * ratio, and per-realisation Lysmer terms (dashpot coefficients scale with sqrt(E), spring
 * coefficients with E; scatter/system_matrix.py:362-376).  FP32 stiffness products, FP64
 * u and v.  All per-realisation arrays are [slot or element][R] (realisation fastest).
 *   elem [n_elem][n_en] node indices; inc_ptr/inc node -> element incidence (each node's list in
 *     any fixed order: it is the summation order)
 *   ke_type [n_elem] -> ke1 [n_types][3 n_en][3 n_en] float32; young [n_elem][R] float32
 *   ml [3 n_nodes] lumped mass; fixed [3 n_nodes]; alpha, beta Rayleigh; dt time step
 *   l_ptr [3 n_nodes + 1], l_col, l_elem, l_c, l_s: Lysmer entries per slot row: column slot,
 *     element whose E scales it, unit dashpot coefficient (x sqrt(E)), unit spring (x E)
 *   u, v [3 n_nodes][R] FP64 state, read at the start and written at the end of each run (the
 *   step kernel accumulates in FP32 (hi, lo) pairs).  Setup allocates the ping-pong copies and
 *   the pair accumulators; runs allocate nothing.
 *   node_nen [n_nodes] (optional, uint8): for independent meshes of different element types
 *     concatenated into one system (one realisation, R = 1): each node's element size; elem
 *     rows and ke1 tables then use the largest type's stride (n_en, 3 n_en), shorter types
 *     padded.  NULL: every element has n_en nodes.
 * R <= 1024 (above 256: even up to 512, else divisible by 4); n_en in {4, 8, 10, 20}. */
typedef struct sc_batch_desc sc_batch_desc;
typedef struct sc_batch sc_batch;
int sc_batch_create(sc_batch** h, const sc_batch_desc* desc, double* u, double* v, void* stream);
/* The step kernel and its shape (realisations per thread, threads per block) are picked at
 * create time, and again by sc_batch_set_hex8_grid, by timing the candidates on scratch
 * copies of the state (no reference counterpart); this reports the choice, its per-step time
 * and which kernel it is: 0 the incidence-list kernel, 1 the uniform hexa8 grid kernel (tiled),
 * 2 the tensor-core kernel (realisations_per_thread then reports its column segment length),
 * 3 the node-centric uniform hexa8 kernel, 4 the same at the wide register budget. */
int sc_batch_config(sc_batch* h, int* realisations_per_thread, int* threads_per_block, float* ms_per_step,
                    int* grid_kernel);
/* Uniform hexa8 grids (no reference counterpart; the meshes scatter/mesher.py reads from
 * structured gmsh boxes): every element the same shape (n_types = 1), nodes on an integer
 * lattice along the elements' natural axes (xi, eta, zeta), an element's local node l at its
 * first node's lattice point plus the natural offset of l (scatter/element_types.py:52-104
 * order).  The lattice is cut into tiles of 4 x 4 x 2 points; halo [n_tiles][144] int32 lists
 * the nodes of each tile grown by one point on every side, point (hx, hy, hz) of the 6 x 6 x 4
 * box at hx + 6 (hy + 6 hz) (-1 where the lattice has no node); elem8 [n_nodes][8] int32 the
 * element in which the node is local node la (-1 where none).  The incidence lists must be
 * sorted by the node's local index in the element (that order is the summation order of the
 * kernels, so they give bitwise the same results).  Two kernels use these tables: the tiled
 * one (the tiles' w staged in shared memory) and a node-centric one that takes each incident
 * element's local index at compile time, so that every K1 entry is an operand of its FMAs
 * rather than a load.  Device arrays owned by the caller; the tuner then times all kernels. */
int sc_batch_set_hex8_grid(sc_batch* h, int n_tiles, const int* halo, const int* elem8);
/* The tensor-core step on a uniform hexa8 grid (no reference counterpart): the element
 * products D = W K1 for 128 realisations at a time on tcgen05 (TF32 in three hi/lo products,
 * FP32 accumulation; about 2^-21 of each product, so its results agree with the other kernels
 * to that rounding, not bitwise).  The lattice (as above) is cut into columns of 4 x 4 points
 * across its first two axes; nzp is the number of points along the third.  nodes
 * [n_col][nzp][36] int32: the node at point (hx, hy) of the column's 6 x 6 ring (its points grown
 * by one on each side) in plane z, at hx + 6 hy, -1 where none; elems [n_col][nzp - 1][25]
 * int32: the element whose local node 0 sits at ring point (ex, ey) of plane z, at ex + 5 ey,
 * -1 where none.  Columns numbered as the caller likes.  Needs R a multiple of 128.  Device
 * arrays owned by the caller; the tuner then times every kernel.  sc_batch_status
 * synchronises the stream and returns SC_CUDA_ERROR if a tensor-core step gave up waiting for
 * its tensor-core work (its results are then not valid). */
int sc_batch_set_hex8_columns(sc_batch* h, int n_col, int nzp, const int* nodes, const int* elems);
int sc_batch_status(sc_batch* h);
/* testing aids: force a shape of the incidence-list kernel (realisations per thread in
 * {1, 2, 4, 8} dividing R, by 4 for 4 and 8; threads per block a multiple of R / rpt, at most
 * 256), or of the tiled uniform hexa8 grid kernel (1 or 2 realisations per thread, 128 or 256
 * threads per block), or of the node-centric uniform hexa8 kernel (2, 4 or 8 realisations per
 * thread dividing R, by 4 for 4 and 8; 128 or 256 threads per block, at least R / rpt), or the
 * tensor-core kernel with column segments of seg points */
int sc_batch_set_shape(sc_batch* h, int realisations_per_thread, int threads_per_block);
int sc_batch_set_grid_shape(sc_batch* h, int realisations_per_thread, int threads_per_block);
int sc_batch_set_node_shape(sc_batch* h, int realisations_per_thread, int threads_per_block);
/* wide = 1: the node-centric kernel at the wide register budget (one block per SM minimum; 2 or
 * 4 realisations per thread); sc_batch_config reports it as kernel 4 */
int sc_batch_set_node_shape_budget(sc_batch* h, int realisations_per_thread, int threads_per_block, int wide);
int sc_batch_set_tc_shape(sc_batch* h, int seg);
int sc_batch_set_force(sc_batch* h, int n_t, const int64_t* f_ptr, const int* f_slot, const double* f_val);
/* receivers record v [n_out][n_rec][R] every out_interval steps */
int sc_batch_set_output(sc_batch* h, int out_interval, int n_rec, const int* rec_slot, double* out_v, int64_t n_out);
int sc_batch_run(sc_batch* h, int t_begin, int t_end);
int sc_batch_destroy(sc_batch* h);

#ifdef __cplusplus
}
#endif
#endif
