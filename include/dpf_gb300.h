/*
 * dpf_gb300.h — C ABI of the GB300 bonded-DEM Newton path (libdpf_gb300.so).
 *
 * Every entry point takes borrowed device pointers in the reference's tensor
 * layouts, sizes, and a cudaStream_t passed as void*.  The library never
 * allocates, frees or keeps a pointer after the call returns; scratch buffers
 * are supplied by the caller and their sizes are given next to each entry.
 *
 * Layouts (row-major, float64 unless stated):
 *   per-site 6-vectors  (N, 6) = [tx, ty, tz, rx, ry, rz]
 *   positions           (N, 3); radii, masses (N); mass (N, 6)
 *   fixed               (N) uint8 (0/1, the bytes of a torch.bool tensor)
 *   edges               (M, 2) int64, the bond normal points edges[b,0] -> edges[b,1]
 *   per-bond vectors    (M, 3); per-bond scalars (M)
 *   6x6 site blocks     (N, 6, 6)
 *
 * Incidence CSR (built once by the caller from edges): for site s the entries
 * inc_bond[inc_ptr[s] .. inc_ptr[s+1]) list first the bonds b with
 * edges[b,0] == s as the value b, in increasing b, then the bonds with
 * edges[b,1] == s as the value ~b (= -b-1), in increasing b.  This order is the
 * order in which the reference's index_add_ adds the two endpoints.
 *
 * Status: every entry returns 0 on success or a bitmask of dpf_status.  Guard
 * failures detected on the device (the reference's 'Subdivide:' errors) are
 * OR-ed into a caller-supplied device int (`status`), which the caller reads
 * after the stream reaches the call; the return value only reports argument
 * and launch errors.  No kernel traps or waits without a time limit.
 */
#ifndef DPF_GB300_H
#define DPF_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum dpf_status {
    DPF_OK = 0,
    DPF_ERR_ROTATION = 1,        /* body rotation > 0.25 rad in a step        */
    DPF_ERR_COINCIDENT = 2,      /* bond length <= 1e-12                       */
    DPF_ERR_NORMAL_TURN = 4,     /* contact normal turns > 0.25 rad per half step */
    DPF_ERR_NONFINITE = 8,       /* non-finite value in a reduction            */
    DPF_ERR_NOT_CONVERGED = 16,  /* bounded iteration limit reached            */
    DPF_ERR_BARRIER_TIMEOUT = 32,/* a grid barrier gave up after its time limit */
    DPF_ERR_ARGUMENT = 1 << 16,  /* invalid argument (host check)              */
    DPF_ERR_CUDA = 1 << 17,      /* CUDA launch/runtime error                  */
    DPF_ERR_TOO_LARGE = 1 << 18  /* problem exceeds a fixed static capacity    */
};

/* Bond capacity of the static scratch of dpf_stiffness_apply_static. */
#define DPF_STATIC_MAX_BONDS 65536

/* Bond graph: reference edges plus the incidence CSR described above. */
typedef struct dpf_graph {
    int64_t n_sites;
    int64_t n_bonds;
    const int64_t *edges;      /* (M, 2)   */
    const int32_t *inc_ptr;    /* (N + 1)  */
    const int32_t *inc_bond;   /* (2 M)    */
} dpf_graph;

/* Bond stiffnesses kn = E A/L, ks = G A/L, kb = E I/L, kt = 2 G I/L (M each). */
typedef struct dpf_stiffness {
    const double *kn, *ks, *kb, *kt;
} dpf_stiffness;

/* Committed state of the finite-motion rate law (FiniteBondsGPU attributes). */
typedef struct dpf_history {
    const double *x;       /* (N, 3) centres            */
    const double *radii;   /* (N)                        */
    const double *normal;  /* (M, 3) committed normals   */
    const double *offset;  /* (M, 3) contact offsets     */
    const double *fn;      /* (M)   normal force         */
    const double *fs;      /* (M, 3) shear force on i    */
    const double *mt;      /* (M)   twist couple         */
    const double *mb;      /* (M, 3) bending couple      */
} dpf_history;

/* Frozen tangent geometry: bond normal and contact levers (M, 3) each. */
typedef struct dpf_tangent {
    const double *n, *ri, *rj;
} dpf_tangent;

/* Outputs of a constitutive trial.  Any pointer except `force` may be NULL. */
typedef struct dpf_trial_out {
    double *force;                       /* (N, 6) midpoint force and torque       */
    double *n, *ri, *rj;                 /* (M, 3) midpoint tangent geometry        */
    double *x_end;                       /* (N, 3)                                  */
    double *normal_end, *offset_end;     /* (M, 3)                                  */
    double *fs_end, *mb_end;             /* (M, 3)                                  */
    double *fn_end, *mt_end;             /* (M)                                     */
} dpf_trial_out;

/* Size in doubles of the per-bond wrench scratch used by bond sweeps: 9 M. */
int64_t dpf_wrench_scratch_doubles(int64_t n_bonds);

/* K q, the frozen-tangent stiffness product.
 * Replaces LinearBondsGPU.stiffness (experiments/bonded_dem_linear_gpu.py:42-52)
 * and WarpTangent.__call__ (experiments/bonded_dem_tangent_warp.py:33-44).
 * wrench: scratch of dpf_wrench_scratch_doubles(M) doubles. */
int dpf_stiffness_apply(const dpf_graph *g, const dpf_stiffness *k, const dpf_tangent *t,
                        const double *q, double *out, double *wrench, void *stream);

/* K q like dpf_stiffness_apply, but nobody allocates scratch: no counterpart
 * in the reference.  It exists for callers that cannot call cudaMalloc, such
 * as a host application that gives this library only its inputs and outputs
 * from a device-memory pool it manages itself under a fixed budget, where an
 * extra allocation could fail, or a cudaFree could stall the whole device, in
 * the middle of the host's own work.
 * The bond-wrench scratch is a file-scope device array of
 * 9 * DPF_STATIC_MAX_BONDS doubles (4.5 MiB) that every GPU which loads the
 * library holds until the process exits.  Graphs with more than
 * DPF_STATIC_MAX_BONDS bonds are rejected with DPF_ERR_TOO_LARGE before any
 * launch.  Every call looks up the array's device address on the current
 * device (cudaGetSymbolAddress; the first lookup on a device loads the
 * module there, so make the first call before any stream capture).  All
 * calls on a device share the one array: calls whose work overlaps on the
 * GPU (concurrent streams, several host threads) race on it, so serialise
 * them.  The array keeps the last call's contents; every value a
 * call reads from it is written earlier in the same call, so nothing needs
 * clearing.  The function allocates nothing and frees nothing. */
int dpf_stiffness_apply_static(const dpf_graph *g, const dpf_stiffness *k, const dpf_tangent *t,
                               const double *q, double *out, void *stream);

/* DPF_STATIC_MAX_BONDS, for callers binding the library without the header. */
int64_t dpf_static_max_bonds(void);

/* Per-site 6x6 diagonal blocks of K (N, 6, 6).
 * Replaces LinearBondsGPU._diagonal_blocks (experiments/bonded_dem_linear_gpu.py:54-72)
 * and WarpDiagonal.__call__ (experiments/bonded_dem_precondition_warp.py:111-118). */
int dpf_diagonal_blocks(const dpf_graph *g, const dpf_stiffness *k, const dpf_tangent *t,
                        double *diagonal, void *stream);

/* Block scaling of the Newton system: diagonal = D(K), block = diag(mass) +
 * dt^2/4 D with identity rows on fixed sites, preconditioner = block^-1,
 * units = [r, r, r, 1, 1, 1] (1 on fixed sites).  Any output may be NULL
 * except preconditioner.
 * Replaces NewtonBonds.prepare_scaling (experiments/bonded_dem_newton.py:94-102). */
int dpf_prepare_scaling(const dpf_graph *g, const dpf_stiffness *k, const dpf_tangent *t,
                        const double *mass, const uint8_t *fixed, const double *radii, double dt,
                        double *diagonal, double *block, double *preconditioner, double *units,
                        void *stream);

/* Pure constitutive trial at increment y (N, 6); no committed state changes.
 * mid_positions / end_positions (N, 3) may be NULL (then x + y/2, x + y).
 * want_end = 0 skips the end-of-step histories but keeps every guard.
 * Replaces FiniteBondsGPU.trial (experiments/bonded_dem_finite_gpu.py:87-116). */
int dpf_trial(const dpf_graph *g, const dpf_stiffness *k, const dpf_history *h,
              const double *y, const double *mid_positions, const double *end_positions,
              int want_end, const dpf_trial_out *out, double *wrench, int *status, void *stream);

/* Midpoint residual r = M (y - dt v) - dt^2/2 (f_mid(y) + external), fixed
 * rows r = y, computed with the guards of a full trial; optionally also the
 * scaled residual s = P r / units and, in `norms` (3 doubles, device),
 * [|r|_2, max|s|, |s|_2].  preconditioner/units/scaled may be NULL.
 * Replaces NewtonBonds.residual + scale_residual (experiments/bonded_dem_newton.py:83-86, 104-105). */
int dpf_residual(const dpf_graph *g, const dpf_stiffness *k, const dpf_history *h,
                 const double *y, const double *v, const double *external, const double *mass,
                 const uint8_t *fixed, double dt, const dpf_trial_out *trial,
                 const double *preconditioner, const double *units,
                 double *residual, double *scaled, double *norms,
                 double *wrench, double *partials, int *status, void *stream);

/* Scaled residual s = P r / units and norms[0..2] = [|r|_2, max|s|, |s|_2]
 * (device doubles; scaled and norms may be NULL).
 * Replaces NewtonBonds.scale_residual and the norms of NewtonBonds.step
 * (experiments/bonded_dem_newton.py:104-105, 146-147). */
int dpf_scale_residual(int64_t n_sites, const double *preconditioner, const double *units,
                       const double *residual, double *scaled, double *norms, double *partials,
                       void *stream);

/* Jacobian-vector product of the midpoint residual:
 * out = mass * d - dt^2/2 * (d f_mid(y)[d]), fixed rows out = d, where
 * d = units * direction when units != NULL.  When preconditioner != NULL the
 * result is scaled: out = P (J d) / units (the Newton operator).
 * Replaces NewtonBonds.jacobian_vector (experiments/bonded_dem_newton.py:88-92)
 * and WarpJacobian (experiments/bonded_dem_jvp_warp.py:45-116). */
int dpf_jacobian_vector(const dpf_graph *g, const dpf_stiffness *k, const dpf_history *h,
                        const double *y, const double *direction, const double *mass,
                        const uint8_t *fixed, double dt, const double *units,
                        const double *preconditioner, double *out, double *wrench, void *stream);

/* Size in doubles of the elastic PCG workspace for N sites. */
int64_t dpf_elastic_workspace_doubles(int64_t n_sites);

/* Block-Jacobi PCG on (diag M + dt^2/4 K) with the reference's stopping rule
 * (test every 5th iteration at r.z <= tol^2 r0.z0), rhs = block (units * vector),
 * result out = x / units.  One cooperative launch runs all iterations; the
 * iteration count (0 when the right-hand side vanishes) is ADDED to
 * *iterations (device int), as the reference adds to inner_iterations.  workspace: dpf_elastic_workspace_doubles(N);
 * barrier: 2 zeroed unsigned ints (device).
 * Replaces NewtonBonds.elastic_precondition (experiments/bonded_dem_newton.py:107-130)
 * and WarpElastic (experiments/bonded_dem_precondition_warp.py:127-151). */
int dpf_elastic_precondition(const dpf_graph *g, const dpf_stiffness *k, const dpf_tangent *t,
                             const double *mass, const uint8_t *fixed, const double *block,
                             const double *preconditioner, const double *units,
                             const double *vector, double dt, double tolerance, int max_iterations,
                             double *out, int *iterations, double *wrench, double *workspace,
                             unsigned *barrier, int *status, void *stream);

/* Bond setup on the device: normal n, contact levers ri = c - p_i, rj = c - p_j,
 * kn = E A/L, ks = G A/L, kb = E I/L, kt = 2 G I/L (I = A^2/(4 pi)), the contact
 * offset c - classical (may be NULL) and the (N, 6) mass [m, m, m, 0.4 m r^2 x 3]
 * (may be NULL).  contacts (M, 3) may be NULL (classical ball contacts);
 * young_b / shear_b (M) give per-bond moduli (NULL: the scalars young, shear).
 * Replaces LinearBondsGPU.__init__ / FiniteBondsGPU.__init__ arithmetic
 * (experiments/bonded_dem_linear_gpu.py:15-40, experiments/bonded_dem_finite_gpu.py:49-63). */
int dpf_bond_setup(int64_t n_sites, int64_t n_bonds, const int64_t *edges, const double *points,
                   const double *radii, const double *areas, const double *contacts,
                   const double *masses, double young, double shear, const double *young_b,
                   const double *shear_b, double *n, double *ri, double *rj, double *kn, double *ks,
                   double *kb, double *kt, double *offset, double *mass6, void *stream);

/* Net loads (force, torque) of the committed state (N, 6).
 * Replaces FiniteBondsGPU.loads (experiments/bonded_dem_finite_gpu.py:82-85). */
int dpf_loads(const dpf_graph *g, const dpf_history *h, double *out, double *wrench, void *stream);

/* Accepted-step update: v <- 2 y / dt - v and rotation <- exp(y_w) rotation.
 * Replaces the commit block of NewtonBonds.step (experiments/bonded_dem_newton.py:149-154)
 * with exp_rotation (experiments/bonded_dem_finite_gpu.py:35-43). */
int dpf_accept_step(int64_t n_sites, const double *y, double dt, double *v, double *rotation,
                    void *stream);

/* Elastic plus kinetic energy (one double, device).
 * Replaces FiniteBondsGPU.energy (experiments/bonded_dem_finite_gpu.py:122-125). */
int dpf_energy(const dpf_graph *g, const dpf_stiffness *k, const dpf_history *h,
               const double *mass, const double *v, double *energy, double *partials, void *stream);

/* ---- FGMRES building blocks (experiments/bonded_dem_newton.py:13-60) ---- */

/* Size in doubles of the reduction partials used by the vector kernels. */
int64_t dpf_partials_doubles(void);

/* Twice-iterated classical Gram-Schmidt of w against basis rows 0..j
 * (row stride ld) followed by h[0..j] = projections, h[j+1] = |w|, and, when
 * |w| >= 1e-14, basis row j+1 = w / |w|.  h is a device array of j+2 doubles.
 * Replaces the Arnoldi body of fgmres (experiments/bonded_dem_newton.py:35-43). */
int dpf_arnoldi_cgs2(int64_t length, double *basis, int64_t ld, int j, double *w, double *h,
                     double *partials, void *stream);

/* dpf_arnoldi_cgs2 on float32 vectors in one cooperative launch (three grid
 * barriers): orthogonalises v (kept unchanged) against basis rows 0..j into
 * w and writes row j+1 = w/|w|.  Dot products and the projection are summed
 * exactly as float32 pairs (TwoProd by FMA and TwoSum), block partials and h
 * in float64, w and the new row rounded to float32 once.  length and ld are
 * even, the vectors 8-byte aligned; partials: dpf_partials_doubles();
 * barrier: 2 words (reset by the call); a barrier wait that runs out sets
 * DPF_ERR_BARRIER_TIMEOUT in *status. */
int dpf_arnoldi_cgs2_f32(int64_t length, float *basis, int64_t ld, int j, const float *v, float *w, double *h,
                         double *partials, unsigned *barrier, int *status, void *stream);

/* x += sum_{k<count} coefficients[k] * rows[k]  (coefficients on the host, count <= 64).
 * Replaces `x += transformed[:j+1].T @ coefficients` (experiments/bonded_dem_newton.py:54). */
int dpf_combine_rows(int64_t length, const double *rows, int64_t ld, int count,
                     const double *coefficients, double *x, void *stream);

/* x += sum_k coefficients[k] rows[k] for float32 rows into float64 x (the
 * sum as a float32 pair). */
int dpf_combine_rows_f32(int64_t length, const float *rows, int64_t ld, int count,
                         const double *coefficients, double *x, void *stream);

/* out = (float)(alpha a) */
int dpf_scale_to_float(int64_t length, double alpha, const double *a, float *out, void *stream);

/* result[0] = sum a*b and result[1] = sqrt(sum a*a) over `length` doubles (device). */
int dpf_dot_norm(int64_t length, const double *a, const double *b, double *result,
                 double *partials, void *stream);

/* out = alpha * a + beta * b over `length` doubles. */
int dpf_axpby(int64_t length, double alpha, const double *a, double beta, const double *b,
              double *out, void *stream);

/* out[0] = |dt mass*v + dt^2/2 external|_2, out[1] = |loads on free sites|_2
 * (device doubles); the two terms of rhs_scale in NewtonBonds.step
 * (experiments/bonded_dem_newton.py:138-139). */
int dpf_rhs_scale(int64_t n_sites, const double *mass, const double *v, const double *external,
                  const double *loads, const uint8_t *fixed, double dt, double *out,
                  double *partials, void *stream);

/* out = units * a with zero rows on fixed sites, the Newton correction of
 * NewtonBonds.step (experiments/bonded_dem_newton.py:186-187). */
int dpf_masked_scale(int64_t n_sites, const double *a, const double *units, const uint8_t *fixed,
                     double *out, void *stream);

/* ---- Linear model and the previous solver (float64) ----
 * out = (diag M + alpha K) q with identity rows on fixed sites; the operator
 * of LinearBondsGPU._operator (experiments/bonded_dem_linear_gpu.py:74-77).
 * wrench: dpf_wrench_scratch_doubles(M) doubles. */
int dpf_operator_apply(const dpf_graph *g, const dpf_stiffness *k, const dpf_tangent *t, const double *mass,
                       const uint8_t *fixed, double alpha, const double *q, double *out, double *wrench,
                       void *stream);

/* Block preconditioner of the linear solves: block = diag M + alpha diagonal
 * per site (the identity on fixed sites; optional output) and
 * preconditioner = block^-1, both (N, 6, 6) doubles; diagonal (N, 6, 6) are
 * the K blocks.  Replaces the inverse in LinearBondsGPU.solve_increment
 * (experiments/bonded_dem_linear_gpu.py:82-86) and
 * FiniteBondsGPU.solve_increment (experiments/bonded_dem_finite_gpu.py:141-143). */
int dpf_block_inverse(int64_t n_sites, const double *mass, const uint8_t *fixed, const double *diagonal, double alpha,
                      double *block, double *preconditioner, void *stream);

/* Doubles of the workspace of dpf_block_pcg for N sites. */
int64_t dpf_block_pcg_workspace_doubles(int64_t n_sites);

/* Block-Jacobi PCG on (diag M + alpha K) x = rhs (identity rows on fixed
 * sites, rhs rows of fixed sites read as zero) in one cooperative launch.
 * preconditioner: (N, 6, 6) block inverse.  mode 0 replaces
 * LinearBondsGPU.solve_increment (experiments/bonded_dem_linear_gpu.py:79-112):
 * starts from x (use_guess != 0; fixed rows zeroed) or zero, stops at the
 * first 10th iteration with |r|/|rhs| < tolerance, and returns the true
 * residual |rhs - A x|/|rhs|.  mode 1 replaces FiniteBondsGPU.solve_increment
 * (experiments/bonded_dem_finite_gpu.py:133-167): starts from zero and, every
 * 10th iteration with |r|/|rhs| < tolerance and max|P r / scale| < 2e-8,
 * accepts when the true residual a satisfies |a|/|rhs| < 5 tolerance and
 * max|P a / scale| < 1e-7 (scale (N, 6) required).  x (N, 6): guess in,
 * solution out.  info (device, 4 doubles): [iterations, relative residual,
 * state (0 converged, 1 iteration cap, 2 non-finite residual at a test),
 * |rhs|]; a right-hand side below 1e-30 (mode 0) or 1e-40 (mode 1) gives
 * x = 0 and 0 iterations.  workspace: dpf_block_pcg_workspace_doubles(N);
 * barrier: 2 unsigned ints (device), zeroed by the call on its stream. */
int dpf_block_pcg(const dpf_graph *g, const dpf_stiffness *k, const dpf_tangent *t, const double *mass,
                  const uint8_t *fixed, const double *preconditioner, const double *scale, const double *rhs,
                  double alpha, double tolerance, int max_iterations, int mode, int use_guess, double *x,
                  double *info, double *wrench, double *workspace, unsigned *barrier, int *status, void *stream);

/* Linear implicit midpoint (experiments/bonded_dem_linear_gpu.py:114-121):
 * rhs = dt M v + dt^2/2 (external - kq) and guess = dt v; then, with the
 * increment dq, v <- 2 dq/dt - v and q <- q + dq.  All (N, 6) doubles. */
int dpf_linear_midpoint_rhs(int64_t n_sites, const double *mass, const double *v, const double *external,
                            const double *kq, double dt, double *rhs, double *guess, void *stream);
int dpf_linear_midpoint_advance(int64_t n_sites, const double *dq, double dt, double *v, double *q, void *stream);

/* Doubles of the partials buffer of dpf_linear_sums and dpf_anderson_gram
 * (zeroed once before first use; the kernels leave their counters at zero). */
int64_t dpf_small_partials_doubles(void);

/* out[0] = sum a.b (when a is given), out[1] = (sum m v^2 + sum q kq) / 2
 * (when mass is given): the step work and LinearBondsGPU.energy
 * (experiments/bonded_dem_linear_gpu.py:121, 123-124).  Device doubles. */
int dpf_linear_sums(int64_t n_sites, const double *a, const double *b, const double *mass, const double *v,
                    const double *q, const double *kq, double *out, double *partials, void *stream);

/* Anderson mixing of the previous solver (experiments/bonded_dem_finite_gpu.py:215-229)
 * over device history slots: iterates and corrections are (slots, N, 6)
 * doubles, order[0..count) (host ints) lists the slots oldest first
 * (2 <= count <= slots <= 8).  With dc_h = c_{h+1} - c_h and weights
 * u = [1, 1, 1, radius x 3], dpf_anderson_gram writes the upper triangle of
 * gram[h][l] = (u dc_h).(u dc_l) row by row, then proj[h] = (u dc_h).(u c_last)
 * (device doubles); dpf_anderson_mix writes out = c_last - sum_h coef_h
 * (dy_h + dc_h) and ORs 1 into *flag (device int) if an entry is not finite. */
int dpf_anderson_gram(int64_t n_sites, const double *iterates, const double *corrections, int slots,
                      const int32_t *order, int count, const double *radii, double *out, double *partials,
                      void *stream);
int dpf_anderson_mix(int64_t n_sites, const double *iterates, const double *corrections, int slots,
                     const int32_t *order, int count, const double *coefficients, double *out, int *flag,
                     void *stream);

/* Self-test of the time-limited grid barrier every cooperative kernel here
 * uses (no reference counterpart).  `blocks` blocks (1..64) each wait for
 * blocks + missing arrivals: with missing = 0 they pass and add their count
 * to *passed; with missing > 0 nobody can release the barrier, every wait
 * gives up after timeout_ns (<= 2 s) and DPF_ERR_BARRIER_TIMEOUT is ORed
 * into *status, and the kernel returns.  barrier (2 unsigned ints, zeroed
 * by the call), status and passed are device memory. */
int dpf_barrier_selftest(int blocks, int64_t timeout_ns, int missing, unsigned *barrier, int *status, int *passed,
                         void *stream);

/* ---- Mixed precision: float32 bond sweeps, float64 reductions and residual ----
 * One step of NewtonBonds.step (experiments/bonded_dem_newton.py:132-201) in
 * float32 bulk arithmetic.  The residual keeps float64 accuracy: a float64
 * setup per step computes r0 = -dt M v - dt^2/2 (loads(x) + external); for an
 * increment y the residual is r0 + M y - dt^2/2 sum of per-bond float32
 * increments f_mid(y) - f_mid(0), evaluated from small quantities only and
 * summed per site in compensated float32 (about float64 accuracy).
 * bond_data: dpf_mixed_bond_floats(M) floats (float4 records + float32
 * tangent, 16-byte aligned); wrench: dpf_mixed_wrench_floats(M) floats, 16-byte
 * aligned (one 48-byte record [F, T_i, T_j] per bond).  The *32 arguments are
 * float32 copies of the float64 arrays of the same name (y32 of the increment,
 * mass32 of the (N, 6) mass, units32 of the units written by
 * dpf_mixed_scaling); d32 is a float32 (N, 6) scratch. */
int64_t dpf_mixed_bond_floats(int64_t n_bonds);

/* Float workspace of dpf_mixed_precondition for N sites and M bonds
 * (16-byte aligned; holds the padded work vectors and the bond wrench). */
int64_t dpf_mixed_workspace_floats(int64_t n_sites, int64_t n_bonds);

/* Size in floats of the float32 bond wrench of the mixed passes (12 M). */
int64_t dpf_mixed_wrench_floats(int64_t n_bonds);

/* The residual at y = 0 of a step whose records a commit wrote (dpf_mixed_commit
 * with dloads, or dpf_mixed_commit_lazy): every bond increment vanishes there,
 * so residual = r0 on free sites and 0 on fixed ones, y32 = 0, and the commit
 * already stored the tangent at y = 0 in bond_data.  Equal to
 * dpf_mixed_residual(y = 0) without its bond pass and site gather; not valid
 * after a float64 setup (its records carry dn0 != 0). */
int dpf_mixed_initial_residual(int64_t n_sites, const double *r0, const uint8_t *fixed, float *y32, double *residual,
                               void *stream);

/* Lazy float64 history.  The bond records (bond_data) carry fn, mt, fs, mb
 * and offset in float32 and every commit advances them; `corrections`
 * (dpf_history_correction_floats(M) floats, 16-byte aligned) hold per bond
 * what float32 rounding dropped, so that record + correction is the float64
 * history to about 48 bits.
 * dpf_mixed_history_corrections: corrections = h - record, right after a
 * float64 dpf_mixed_setup wrote the records from h (the same values that
 * dpf_mixed_setup writes itself when given a corrections array).
 * dpf_mixed_commit_lazy: the accepted increment y as dpf_mixed_commit
 * applies it (x_end = x + y (N, 3), records and loads advanced; dloads: 9 M
 * floats) with the exact rounding error of each record update added to the
 * corrections, and no float64 end state written.
 * dpf_mixed_fold_history: the float64 history from the records and
 * corrections, normal = the unit vector from x_i to x_j (as dpf_mixed_commit
 * forms normal_end). */
int64_t dpf_history_correction_floats(int64_t n_bonds);
int dpf_mixed_history_corrections(const dpf_graph *g, const dpf_history *h, const float *bond_data,
                                  float *corrections, void *stream);
int dpf_mixed_commit_lazy(const dpf_graph *g, float *bond_data, const double *x, const double *y, const float *y32,
                          double *x_end, float *corrections, float *dloads, double *loads, void *stream);
int dpf_mixed_fold_history(const dpf_graph *g, const double *x, const float *bond_data, const float *corrections,
                           double *normal, double *offset, double *fn, double *fs, double *mt, double *mb,
                           void *stream);

/* Per-step float64 setup: bond records from the committed state, r0 (N, 6),
 * optionally loads(x) (N, 6), and scales[0..1] = [|dt M v + dt^2/2 ext|,
 * |loads on free sites|] (the two terms of rhs_scale).  wrench: 9 M doubles.
 * corrections (optional, dpf_history_correction_floats(M) floats, 16-byte
 * aligned): the lazy history's corrections of the records just written.
 * Replaces the loads/rhs_scale prologue of NewtonBonds.step
 * (experiments/bonded_dem_newton.py:137-139, experiments/bonded_dem_finite_gpu.py:82-85). */
int dpf_mixed_setup(const dpf_graph *g, const dpf_stiffness *k, const dpf_history *h,
                    const double *mass, const double *v, const double *external,
                    const uint8_t *fixed, double dt, float *bond_data, double *r0, double *loads,
                    double *scales, double *wrench, float *corrections, double *partials, int *status,
                    void *stream);

/* Residual at increment y with every trial guard (status bits as dpf_trial);
 * want_tangent stores the midpoint tangent for dpf_mixed_scaling and K q;
 * preconditioner (float32 (N, 6, 6)) / units / scaled / norms as in dpf_residual.
 * y, mass, r0 and residual are 16-byte aligned, preconditioner 8-byte aligned
 * (DPF_ERR_ARGUMENT otherwise).
 * Replaces NewtonBonds.residual + scale_residual (experiments/bonded_dem_newton.py:83-86, 104-105). */
int dpf_mixed_residual(const dpf_graph *g, float *bond_data, const double *y, const float *y32,
                       const double *mass, const uint8_t *fixed, double dt, const double *r0,
                       int want_tangent, const float *preconditioner, const float *units32,
                       double *residual, double *scaled, double *norms, float *wrench,
                       double *partials, int *status, void *stream);

/* Blocks and scaling from the stored float32 tangent: block (float32 (N,6,6),
 * may be NULL), preconditioner = block^-1 (float32, Jacobi-scaled Cholesky),
 * units (float64 (N, 6)).
 * Replaces NewtonBonds.prepare_scaling (experiments/bonded_dem_newton.py:94-102). */
int dpf_mixed_scaling(const dpf_graph *g, float *bond_data, const float *mass32, const uint8_t *fixed,
                      const double *radii, double dt, float *block, float *preconditioner,
                      double *units, float *units32, void *stream);

/* Scaled residual with the float32 block inverse: s = P r / units and
 * norms = [|r|, max|s|, |s|] (float64; |s|^2 is summed exactly in float32
 * pairs).  P and residual/scaled are 16-byte aligned, units32 8-byte aligned.
 * Replaces NewtonBonds.scale_residual (experiments/bonded_dem_newton.py:104-105). */
int dpf_mixed_scale_residual(int64_t n_sites, const float *preconditioner, const float *units32,
                             const double *residual, double *scaled, double *norms, double *partials,
                             void *stream);

/* J d, the forward-mode derivative of the float32 residual increment; the
 * same options as dpf_jacobian_vector (units, float32 preconditioner).
 * seg_bond/active (optional, for batches): a bond b with active[seg_bond[b]]
 * == 0 contributes nothing (the rows of its request's sites are not read).
 * The preconditioner is 8-byte aligned (DPF_ERR_ARGUMENT otherwise).
 * Replaces NewtonBonds.jacobian_vector (experiments/bonded_dem_newton.py:88-92). */
int dpf_mixed_jacobian_vector(const dpf_graph *g, float *bond_data, const float *y32,
                              const double *direction, const float *mass32, const uint8_t *fixed,
                              double dt, const float *units32, const float *preconditioner,
                              double *out, float *d32, float *wrench, const int32_t *seg_bond,
                              const uint8_t *active, void *stream);

/* dpf_mixed_jacobian_vector with a float32 direction and float32 output (the
 * float32 Krylov vectors of the mixed Newton path); no batch masks. */
int dpf_mixed_jacobian_vector_f32(const dpf_graph *g, float *bond_data, const float *y32,
                                  const float *direction, const float *mass32, const uint8_t *fixed,
                                  double dt, const float *units32, const float *preconditioner,
                                  float *out, float *d32, float *wrench, void *stream);

/* K q in float32 from the stored tangent; q float32 (N, 6), out float64 (N, 6).
 * Replaces LinearBondsGPU.stiffness (experiments/bonded_dem_linear_gpu.py:42-52). */
int dpf_mixed_stiffness_apply(const dpf_graph *g, float *bond_data, const float *q, double *out,
                              float *wrench, void *stream);

/* out[e] = (float) a[e] for e < count. */
int dpf_to_float(int64_t count, const double *a, float *out, void *stream);

/* Elastic PCG in float32 with float64 dot products (same stopping rule and
 * iteration accounting as dpf_elastic_precondition); workspace:
 * dpf_mixed_workspace_floats(N, M) floats (the wrench argument is unused);
 * block/preconditioner float32; seg_bond/active as dpf_mixed_jacobian_vector.
 * Replaces NewtonBonds.elastic_precondition (experiments/bonded_dem_newton.py:107-130). */
int dpf_mixed_precondition(const dpf_graph *g, float *bond_data, const float *mass32,
                           const uint8_t *fixed, const float *block, const float *preconditioner,
                           const float *units32, const double *vector, double dt, double tolerance,
                           int max_iterations, double *out, int *iterations, float *wrench,
                           float *workspace, unsigned *barrier, int *status, const int32_t *seg_bond,
                           const uint8_t *active, void *stream);

/* End state of the accepted increment y: float32 increments added to the
 * float64 committed history (end normal recomputed in float64 from x + y).
 * With dloads (9 M floats scratch) and loads (float64 (N, 6), the committed
 * loads(x) kept by the caller) it also rewrites the bond records for the next
 * step and adds loads(x_end) - loads(x), from float32 increments, to loads.
 * Replaces FiniteBondsGPU.trial's end-of-step outputs and commit
 * (experiments/bonded_dem_finite_gpu.py:102-120). */
int dpf_mixed_commit(const dpf_graph *g, float *bond_data, const dpf_history *h, const double *y,
                     const float *y32, double *x_end, double *normal_end, double *offset_end,
                     double *fn_end, double *fs_end, double *mt_end, double *mb_end, float *dloads,
                     double *loads, void *stream);

/* Per-step constants from loads maintained by dpf_mixed_commit: r0 (N, 6) and
 * scales[0..1] as dpf_mixed_setup, without rebuilding the bond records.
 * Replaces the loads/rhs_scale prologue of NewtonBonds.step
 * (experiments/bonded_dem_newton.py:137-139). */
int dpf_mixed_begin(int64_t n_sites, const double *loads, const double *mass, const double *v,
                    const double *external, const uint8_t *fixed, double dt, double *r0,
                    double *scales, double *partials, void *stream);

/* ---- Batches of requests: contiguous per-request site ranges ----
 * A batch concatenates the graphs of several requests (sites and bonds of
 * request r in one contiguous range each).  These entry points keep every
 * request's scalars separate, so a request follows its own Newton control
 * (experiments/bonded_dem_newton.py:132-201) inside the batch. */

/* dpf_mixed_residual with guard bits per request: status[seg_site[s]] and
 * status[seg_bond[b]] (status is an array of request ints); with active,
 * bonds of requests whose flag is 0 are skipped (no tangent, no guard bits,
 * zero wrench), so those requests' residual rows are not meaningful. */
int dpf_mixed_residual_segmented(const dpf_graph *g, float *bond_data, const double *y,
                                 const float *y32, const double *mass, const uint8_t *fixed, double dt,
                                 const double *r0, int want_tangent, const float *preconditioner,
                                 const float *units32, double *residual, double *scaled,
                                 double *norms, float *wrench, double *partials, int *status,
                                 const int32_t *seg_bond, const int32_t *seg_site, const uint8_t *active,
                                 void *stream);

/* Per-request [|a|_2, max|a|, |b|_2] (or [.., .., a.b] with b_dot) over the
 * 6-vectors of sites seg_ptr[r] .. seg_ptr[r+1]-1, skipping sites with mask
 * != 0 when mask is given; out: 3 doubles per request (device); partials:
 * dpf_segment_partials_doubles(n_segments) doubles of scratch (at most 65,535
 * requests).  Each request is split into fixed slices whose partials are added
 * in slice order (deterministic). */
int64_t dpf_segment_partials_doubles(int n_segments);
int dpf_segment_norms(int n_segments, const int64_t *seg_ptr, const double *a, const double *b,
                      int b_dot, const uint8_t *mask, double *out, double *partials, void *stream);

/* out = a + factor[seg[s]] * c for every site's 6-vector (factor: device doubles). */
int dpf_segment_axpy(int64_t n_sites, const int32_t *seg, const double *factor, const double *a,
                     const double *c, double *out, void *stream);

/* out = keep[seg[s]] ? a : b for every site's 6-vector. */
int dpf_segment_select(int64_t n_sites, const int32_t *seg, const uint8_t *keep, const double *a,
                       const double *b, double *out, void *stream);

/* ---- Adjoint of the implicit step (implicit-function theorem) ----
 * Replace the dense autograd Jacobians of _ImplicitIncrement.backward and of
 * DifferentiableBonds.step (experiments/bonded_dem_differentiable.py:26-38,
 * 139-144) with per-bond forward-mode derivatives of the float64 trial
 * (experiments/bonded_dem_finite_gpu.py:87-116).  Bond inputs, in order:
 * y_i (6), y_j (6), x_i (3), x_j (3), normal (3), offset (3), fn, fs (3), mt,
 * mb (3), kn, ks, kb, kt.  Bond outputs: the midpoint wrench F, T_i, T_j
 * (site i receives (F, T_i), site j (-F, T_j)) and the end history normal (3),
 * offset (3), fn, fs (3), mt, mb (3). */

/* Doubles of the local-Jacobian array (108 per bond) and of the per-bond
 * slot scratch (18 per bond) of the entry points below. */
int64_t dpf_adjoint_jacobian_doubles(int64_t n_bonds);
int64_t dpf_adjoint_slot_doubles(int64_t n_bonds);

/* jacobian[b] = d(F, T_i, T_j)/d(y_i, y_j) at increment y (9 x 12 row-major). */
int dpf_adjoint_local_jacobian(const dpf_graph *g, const dpf_stiffness *k, const dpf_history *h,
                               const double *y, double *jacobian, void *stream);

/* out = J^T lam of the unscaled midpoint residual M y - M dt v - dt^2/2 (F + e)
 * on free sites, out = lam on fixed sites; lam's fixed rows must be zero.
 * slots: dpf_adjoint_slot_doubles scratch. */
int dpf_adjoint_apply_jt(const dpf_graph *g, const double *jacobian, const double *mass,
                         const uint8_t *fixed, double dt, const double *lam, double *out,
                         double *slots, void *stream);

/* Vector-Jacobian product of the trial at increment y for the output adjoints
 * coef * (wrench adjoint of the site vector lam) + end_adjoint (M x 14, the
 * end-history layout); either may be null.  ADDS the input adjoints to
 * history_adjoint (M x 14, same layout), stiffness_adjoint (M x 4: kn ks kb kt),
 * y_adjoint (N x 6, only when with_increment) and x_adjoint (N x 3); a null
 * site array is skipped.  Site sums follow the incidence order: deterministic. */
int dpf_adjoint_bond_vjp(const dpf_graph *g, const dpf_stiffness *k, const dpf_history *h,
                         const double *y, const double *lam, double coef, const double *end_adjoint,
                         int with_increment, double *history_adjoint, double *stiffness_adjoint,
                         double *y_adjoint, double *x_adjoint, double *slots, void *stream);

/* ---- Site tiles and the tiled float32 HVP / elastic PCG ----
 * A tile is a contiguous site range (sites ordered along a space-filling
 * curve make it a compact patch), the bonds touching it ("entries"; a bond
 * between two tiles is an entry of both) and the outside endpoints of those
 * bonds ("halo").  One CTA per tile stages the tile's site vectors and entry
 * wrenches in shared memory; site sums follow the incidence order
 * (deterministic, no atomics).  Replaces LinearBondsGPU.stiffness /
 * _operator (experiments/bonded_dem_linear_gpu.py:42-52, 74-77) inside the
 * elastic PCG (experiments/bonded_dem_newton.py:107-130); the reference
 * fuses the same operator in Warp (bonded_dem_precondition_warp.py:36-151). */
typedef struct {
    int64_t n_tiles, n_entries, n_halo, meta_words;
    int32_t max_entries, max_sites, max_halo, max_meta_words;  /* per-tile maxima */
    const int32_t *tile_site;      /* n_tiles + 1: first site of each tile */
    const int32_t *tile_entry;     /* n_tiles + 1: first entry */
    const int32_t *tile_halo;      /* n_tiles + 1: first halo slot */
    const int32_t *tile_meta_off;  /* n_tiles + 1: first metadata word (multiples of 4) */
    const int32_t *halo_site;      /* n_halo: global site of each halo slot */
    const int32_t *entry_bond;     /* n_entries: bond of each entry */
    const uint32_t *entry_ends;    /* n_entries: local i | local j << 16 (halo slots after own sites) */
    const int32_t *tile_desc;      /* 8 per tile, 16-byte aligned: first site, sites, entries, halo
                                      sites, first entry, first halo slot, first metadata word, words */
    const uint32_t *tile_meta;     /* per tile: T + 1 spans start | mid << 16 (the site's incidences
                                      [start, mid) are i ends, [mid, next start) j ends; offsets
                                      from the tile's first incidence), then the entry (uint16) of
                                      each incidence in incidence order, padded to 16 bytes; then the
                                      tile's halo sites (int32), padded to 16 bytes */
} dpf_tiles;

/* Host function (plain host pointers): greedy tiling in site order, each tile
 * holding at most max_entries entries (<= 32767) and max_stage own + halo
 * sites (<= 65535).  Output arrays: tile_* n_sites + 1; halo_site,
 * entry_bond, entry_ends 2 n_bonds; tile_meta meta_capacity words
 * (dpf_tile_meta_capacity); tile_desc 8 n_sites.  counts (9): n_tiles, n_entries, n_halo,
 * meta_words, max entries, max own sites, max halo sites, max metadata words
 * of a tile, max own + halo sites.  DPF_ERR_TOO_LARGE when one site's bonds
 * alone exceed the limits. */
int dpf_tile_graph(int64_t n_sites, int64_t n_bonds, const int64_t *edges, const int32_t *inc_ptr,
                   const int32_t *inc_bond, int32_t max_entries, int32_t max_stage, int32_t *tile_site,
                   int32_t *tile_entry, int32_t *tile_halo, int32_t *tile_meta_off, int32_t *halo_site,
                   int32_t *entry_bond, uint32_t *entry_ends, uint32_t *tile_meta, int64_t meta_capacity,
                   int32_t *tile_desc, int64_t *counts);
int64_t dpf_tile_meta_capacity(int64_t n_sites, int64_t n_bonds);

/* Floats of the packed entry records (three float4 planes per entry). */
int64_t dpf_tile_entry_floats(int64_t n_entries);

/* Pack the float32 tangent of dpf_mixed_bond_floats bond data into entry
 * records with alpha (= dt^2/4) folded into the stiffnesses; optionally pack
 * the float32 block inverse P36 (N, 6, 6) into 24 floats per site (upper
 * triangle) and the site records site4 (N, 4) = (m, I, 1, 0) from mass32
 * (N, 6), (1, 1, 0, 0) on fixed sites. */
int dpf_tile_pack(const dpf_tiles *t, const float *bond_data, int64_t n_bonds, double alpha, const float *P36,
                  const float *mass32, const uint8_t *fixed, int64_t n_sites, float *entries, float *P24,
                  float *site4, void *stream);

/* y = (diag M + alpha K) q in float32 with identity rows on fixed sites;
 * q, y float32 (N, 6), 16-byte aligned; site4 the site records of
 * dpf_tile_pack.  Persistent
 * CTAs of `threads` consumer threads (<= 192, >= max_entries / 2) plus a
 * bulk-copy warp and a halo-gather warp walk their tiles through a ring of
 * `stages` shared-memory buffers (3 or 4; 0 = the deepest that fits): TMA
 * bulk copies (records, metadata, own-site q) and cp.async (halo q) stream
 * up to stages - 1 tiles ahead of the consumers; a wait past its time limit
 * sets DPF_ERR_BARRIER_TIMEOUT in *status. */
int dpf_tiled_hvp(const dpf_graph *g, const dpf_tiles *t, const float *entries, const float *site4, const float *q,
                  float *y, int *status, int threads, int stages, void *stream);

/* Elastic PCG of dpf_mixed_precondition on the tiled operator, two grid
 * barriers per iteration (single-reduction recurrence); same stopping rule
 * and iteration accounting.  workspace: dpf_tiled_workspace_floats(N)
 * floats; partials: dpf_tiled_partials_doubles() doubles; barrier: 2
 * unsigned ints (device), zeroed by the call on its stream.  stages: tile
 * buffers per CTA (2..4; 0 = the deepest that fits). */
int64_t dpf_tiled_workspace_floats(int64_t n_sites);
int64_t dpf_tiled_partials_doubles(void);

/* ---- Bond-end sweep: the same float32 operator over the site-sorted
 * incidence CSR ----
 * One end record per incidence (bond seen from one of its sites, in the
 * CSR's order): 3 float4 (n', r_s.x) (r_s.y, r_s.z, L, a kn)
 * (a ks, a kb, a kt, other site) with n' pointing from the site to the other
 * end; a group of lanes per site sums its ends' wrenches in registers and a
 * fixed shuffle tree adds the lanes (no shared memory, no atomics).
 * Replaces the same operator as dpf_tiled_hvp
 * (experiments/bonded_dem_linear_gpu.py:42-52, 74-77). */

/* Floats of the end records of a graph with n_bonds bonds (24 n_bonds). */
int64_t dpf_end_floats(int64_t n_bonds);

/* End records from the float32 tangent of dpf_mixed_residual (bond_data)
 * with alpha folded into the stiffnesses; optionally P24 and site4 as
 * dpf_tile_pack. */
int dpf_end_pack(const dpf_graph *g, const float *bond_data, double alpha, const float *P36, const float *mass32,
                 const uint8_t *fixed, float *ends, float *P24, float *site4, void *stream);

/* Number of bond-end sweep variants, and the launch shape of variant
 * `variant` (0 .. count - 1): lanes per site (4, 8 or 16) and resident
 * 256-thread CTAs per SM (2, 3 or 4; fewer CTAs leave more registers per
 * thread).  Variant 0 (8 lanes, 4 CTAs) is the default; an autotuner may
 * pick another per graph size.  Output pointers may be NULL. */
int dpf_end_variant_count(void);
int dpf_end_variant_shape(int variant, int *lanes, int *blocks_per_sm);

/* y = (diag M + alpha K) q in float32 from the end records; q, y (N, 6)
 * float32, 8-byte aligned; variant as dpf_end_variant_shape. */
int dpf_end_hvp(const dpf_graph *g, const float *ends, const float *site4, const float *q, float *y, int variant,
                void *stream);

/* dpf_tiled_precondition on the bond-end operator (one cooperative launch;
 * workspace dpf_tiled_workspace_floats(N), partials
 * dpf_tiled_partials_doubles(); barrier: 2 unsigned ints (device), zeroed
 * by the call on its stream).  seg_site/active (optional, for batches):
 * a site s with active[seg_site[s]] == 0 skips its ends (its request's
 * vector is zero, so its rows stay zero).  variant: the sweep's launch
 * shape (dpf_end_variant_shape); every variant gives the same iterates up
 * to float32 rounding of the lane sums. */
int dpf_end_precondition(const dpf_graph *g, const float *ends, const float *site4, const uint8_t *fixed,
                         const float *block32, const float *P24, const float *units32, const double *vector,
                         double tolerance, int max_iterations, double *out, int *iterations, float *workspace,
                         double *partials, unsigned *barrier, int *status, const int32_t *seg_site,
                         const uint8_t *active, int variant, void *stream);

/* dpf_end_precondition with a float32 input vector and float32 output (the
 * float32 Krylov vectors of the mixed Newton path); no batch masks. */
int dpf_end_precondition_f32(const dpf_graph *g, const float *ends, const float *site4, const uint8_t *fixed,
                             const float *block32, const float *P24, const float *units32, const float *vector,
                             double tolerance, int max_iterations, float *out, int *iterations, float *workspace,
                             double *partials, unsigned *barrier, int *status, int variant, void *stream);
int dpf_tiled_precondition(const dpf_graph *g, const dpf_tiles *t, const float *entries, const float *site4,
                           const uint8_t *fixed, const float *block32, const float *P24, const float *units32,
                           const double *vector, double tolerance, int max_iterations, double *out, int *iterations,
                           float *workspace, double *partials, unsigned *barrier, int *status, int threads,
                           int stages, void *stream);

/* ---- Energy law (bond part of EnergyFoam with volume=False, kinematics='small') ----
 * Replaces EnergyFoam._bond_kinematics / energy / forces
 * (experiments/foam_dem_energy.py:303-315, 405-421, 797-811).  base (M, 4):
 * rest stiffnesses kn, ks, kb, kt; theta: per-site log multipliers (the first
 * four of each row of theta_stride doubles); x (N, 3); q (N, 4) unit
 * quaternions (w, x, y, z); n0, ri, rj (M, 3) rest normal and body-frame
 * levers.  Outputs (any may be NULL, not all): force and torque (N, 3) =
 * -dE/dx and -dE/d(world rotation), energy (1 double, device).  wrench: 9 M
 * doubles when forces are requested; partials: dpf_energy_partials_doubles()
 * doubles when the energy is.  Sums are in a fixed order (deterministic). */
int64_t dpf_energy_partials_doubles(void);
int dpf_bond_energy(const dpf_graph *g, const double *base, const double *theta, int64_t theta_stride,
                    const double *x, const double *q, const double *n0, const double *ri, const double *rj,
                    double *force, double *torque, double *energy, double *wrench, double *partials,
                    void *stream);

/* Frozen tangent of the bond potential at the configuration (x, q) for the
 * Newton direction of the energy-law solver (no reference counterpart; at the
 * reference configuration it is the LinearBondsGPU stiffness, the exact
 * Hessian there, foam_dem_energy.py:14-16): bond axis n = (x_j - x_i)/L,
 * contact point c = ((x_i + R_i ri0) + (x_j + R_j rj0))/2, levers c - x_i,
 * c - x_j, stiffness base * exp((theta_i + theta_j)/2); written into the
 * float32 tangent part of bond_data (dpf_mixed_bond_floats(M) floats,
 * 16-byte aligned) that dpf_mixed_scaling and dpf_end_pack read. */
int dpf_energy_tangent(const dpf_graph *g, const double *base, const double *theta, int64_t theta_stride,
                       const double *x, const double *q, const double *ri0, const double *rj0, float *bond_data,
                       void *stream);

/* ---- Parallel-bond component with brittle failure ----
 * Replaces ParallelBonds.advance / loads (experiments/bonded_dem_core.py:132-208).
 * Per bond: stiffnesses kn = kbar_n A, ks = kbar_s A, kb = kbar_n I, kt = kbar_s J,
 * section area A, second and polar moments I, J, bond radius, tensile
 * strength and cohesion (may be +inf); tan(friction angle) and the moment
 * factor are shared. */
typedef struct dpf_parallel_params {
    const double *kn, *ks, *kb, *kt;
    const double *area, *second_moment, *polar_moment, *radius;
    const double *tensile, *cohesion;
    double tan_phi, beta;
} dpf_parallel_params;

/* Bond history: normal, fs, mb (M, 3); fn, mt, break_energy (M); failure (M)
 * int8 (0 intact, 1 tension, 2 shear).  Read through `in`, written to `out`. */
typedef struct dpf_parallel_state {
    double *normal, *fn, *fs, *mt, *mb, *break_energy;
    int8_t *failure;
} dpf_parallel_state;

/* One step from the committed centres x to end (N, 3) with midpoint samples
 * v, w (N, 3) (mid = (x + end)/2 when NULL).  Writes the new history to `out`
 * (distinct arrays from `in`) and sums[4] = [constitutive work, elastic energy
 * of the new state, removed energy of all broken bonds, newly broken bonds]
 * (device doubles); guard failures (rotation > 0.25 rad, normal turn > 0.25
 * rad per half step, coincident centres) are OR-ed into *status, and the
 * caller then keeps `in`.  partials: dpf_parallel_partials_doubles(). */
int64_t dpf_parallel_partials_doubles(void);
int dpf_parallel_advance(const dpf_graph *g, const dpf_parallel_params *p, const double *radii, const double *x,
                         const double *end, const double *mid, const double *v, const double *w, double dt,
                         const dpf_parallel_state *in, const dpf_parallel_state *out, double *sums,
                         double *partials, int *status, void *stream);

/* Forces and torques about the centres x of the bond history (N, 3 each);
 * wrench: 9 M doubles of scratch. */
int dpf_parallel_loads(const dpf_graph *g, const double *radii, const double *x, const double *fn, const double *fs,
                       const double *mt, const double *mb, double *force, double *torque, double *wrench,
                       int *status, void *stream);

/* ---- native step driver of the mixed-precision Newton solver -------------
 * One implicit step of MixedNewtonBonds.step (bond-end PCG, FGMRES, elastic
 * preconditioning) driven from host code in this library: the same entry
 * points, in the same order, with the same arguments and the same host
 * decisions (convergence tests, Givens rotations, triangular solve, line
 * search) as the Python control path, so both give bit-identical results.
 * Replaces the control flow of NewtonBonds.step and fgmres
 * (experiments/bonded_dem_newton.py:13-60, 132-201).
 *
 * Device pointers unless noted; float64 vectors are (N, 6) = 6 N doubles. */
#define DPF_NEWTON_VECTORS 10      /* scratch vectors of 6 N doubles in `vectors` */
#define DPF_NEWTON_HOST_DOUBLES 128 /* pinned host doubles in `host` */
#define DPF_NEWTON_TRACE 32         /* residual trace entries kept */
#define DPF_NEWTON_TIMERS 11        /* setup, residual, scaling, pcg, jvp, commit, pack, krylov, norms, vector, accept */

typedef struct dpf_mixed_newton {
    const dpf_graph *graph;        /* host struct */
    dpf_stiffness stiffness;       /* float64 stiffnesses (the float64 setup) */
    const double *radii;           /* (N) */
    const double *mass;            /* (N, 6) diagonal mass */
    const float *mass32;           /* (N, 6) */
    const uint8_t *fixed;          /* (N) */
    float *bond_data;              /* dpf_mixed_bond_floats(M) */
    double *r0, *loads;            /* (N, 6) */
    double *scales;                /* 2: the rhs scale terms of the step */
    double *wrench64;              /* 9 M doubles (float64 setup) */
    double *partials;              /* dpf_partials_doubles() */
    double *scalars;               /* >= 8 */
    int *status;                   /* guard bits */
    float *y32, *d32, *wrench32;   /* (N, 6), (N, 6), dpf_mixed_wrench_floats(M) */
    float *block32, *p32;          /* (N, 6, 6) */
    double *units;                 /* (N, 6) */
    float *units32;                /* (N, 6) */
    float *block32_b, *p32_b;      /* a second set of the four scaling arrays: the scaling of a */
    double *units_b;               /* line-search candidate goes there until it is accepted */
    float *units32_b;
    float *ends, *site4, *p24;     /* dpf_end_pack outputs */
    float *end_workspace;          /* dpf_tiled_workspace_floats(N) */
    double *end_partials;          /* dpf_tiled_partials_doubles() */
    unsigned *barrier;             /* 2 words */
    int *inner;                    /* CG iteration counter (added to) */
    float *basis, *transformed;    /* float32 Krylov vectors (width + 1, 6 N), (width, 6 N) */
    float *products;               /* float32 J z_k of the transformed rows, (width, 6 N) */
    float *w32;                    /* 6 N floats */
    double *h;                     /* >= width + 2 */
    int krylov_width;              /* FGMRES restart length, <= 62 */
    double *krylov_partials;       /* dpf_partials_doubles() */
    double *krylov_scalars;        /* 2 */
    double *vectors;               /* DPF_NEWTON_VECTORS x 6 N, 16-byte aligned */
    double *host;                  /* pinned host memory, DPF_NEWTON_HOST_DOUBLES */
    int end_variant;               /* launch shape of the bond-end sweep */
    float *history_corrections;    /* dpf_history_correction_floats(M), or NULL: with it the accepted
                                      step is committed lazily (dpf_mixed_commit_lazy: x_end only;
                                      a float64 refresh also writes the corrections); without it the
                                      float64 end state goes to the step's outputs */
} dpf_mixed_newton;

typedef struct dpf_newton_step {
    double dt;
    const double *external;        /* (N, 6) */
    double *v;                     /* (N, 6) velocity, advanced on convergence */
    double *rotation;              /* (N, 3, 3), advanced on convergence */
    dpf_history history;           /* committed state */
    double *x_end, *normal_end, *offset_end, *fn_end, *fs_end, *mt_end, *mb_end;  /* end state */
    double tolerance, pose_tolerance, linear_tolerance;
    int max_iterations;            /* Newton iterations */
    int refresh;                   /* 1: float64 setup of the records; 0: begin from the maintained loads */
    int timing;                    /* 1: CUDA-event times of the hot launches into the info */
    const double *v_in;            /* optional: the step's start velocity, copied into v first */
    const double *rotation_in;     /* optional: the start rotations, copied into rotation first */
    int committed_start;           /* 1: the records and the tangent at y = 0 come from the last commit
                                      (dpf_mixed_initial_residual replaces the first residual pass) */
} dpf_newton_step;

/* outcome of a step */
enum {
    DPF_NEWTON_CONVERGED = 0,
    DPF_NEWTON_GUARD = 1,          /* a trial guard fired (bits in guard) */
    DPF_NEWTON_NONFINITE = 2,      /* non-finite Newton residual */
    DPF_NEWTON_SINGULAR = 3,       /* zero Givens denominator */
    DPF_NEWTON_KRYLOV = 4,         /* FGMRES iteration budget spent (krylov_relative) */
    DPF_NEWTON_LINE_SEARCH = 5,    /* no admissible step length */
    DPF_NEWTON_DIVERGED = 6        /* Newton iteration budget spent */
};

typedef struct dpf_newton_info {
    int outcome, guard;
    int scaling_alternate;         /* 1: the last scaling is in the *_b arrays (the caller swaps its sets) */
    int nonlinear_iterations, krylov_iterations, cg_iterations;
    int launches;                  /* kernels launched by the step */
    double relative, local;        /* last relative residual and pose defect */
    double work, max_rotation;     /* on convergence: external . y, max |y_w| */
    double krylov_relative;
    int trace_len;
    double trace[2 * DPF_NEWTON_TRACE];          /* [relative, local] per Newton iteration */
    double time_ms[DPF_NEWTON_TIMERS];
    int timed_launches[DPF_NEWTON_TIMERS];
} dpf_newton_info;

/* Returns DPF_OK with the outcome in info (DPF_NEWTON_CONVERGED: the end state
 * is in the step's outputs, v and rotation advanced), or the error code of a
 * failed entry point (DPF_ERR_ARGUMENT / DPF_ERR_CUDA). */
int dpf_mixed_newton_step(const dpf_mixed_newton *solver, const dpf_newton_step *step, dpf_newton_info *info,
                          void *stream);

/* sizeof(dpf_mixed_newton), sizeof(dpf_newton_step), sizeof(dpf_newton_info)
 * into out[0..3): lets a binding check its struct layouts (host only). */
int dpf_newton_struct_sizes(int64_t *out);

#ifdef __cplusplus
}
#endif

#endif /* DPF_GB300_H */
