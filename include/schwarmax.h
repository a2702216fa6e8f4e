/*
 * schwarmax.h -- C ABI of the GB300 (sm_103a) SchwarMAX model-evaluation path.
 *
 * The reference (Hanyuan0908/SchwarMax) is pure Python + JAX; its hot path is
 * a chain of jitted functions.  Each entry point below replaces one stage of
 * that chain (the reference function it stands in for is cited on each), so
 * that a host holding device buffers (PyTorch tensors here, or any caller via
 * ctypes/cffi) can run a model evaluation without XLA.
 *
 * Conventions
 *   - Every buffer is a DEVICE pointer owned by the caller, with explicit sizes.
 *     Arrays named "SoA (k, n)" hold component c of item i at [c*n + i].
 *   - `precision` selects the element type of the floating-point buffers of a
 *     call: SMX_FP32 -> float, SMX_FP64 -> double.  Parameter structs are
 *     always double.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *     asynchronous with respect to the host unless documented otherwise.
 *   - Every call returns an smx_status; no exception crosses the ABI.  The
 *     message of the last failure on the calling thread is returned by
 *     smx_last_error().
 *   - Units: kpc, Gyr, Msun; velocities in kpc/Gyr unless stated; angles in
 *     radians; G = 4.498502151469554e-6 kpc^3 / Msun / Gyr^2.
 */
#ifndef SCHWARMAX_H
#define SCHWARMAX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    SMX_OK = 0,
    SMX_ERR_ARGUMENT = 1,      /* bad size, pointer or option */
    SMX_ERR_UNSUPPORTED = 2,   /* model or option the library does not implement */
    SMX_ERR_NONFINITE = 3,     /* non-finite input or result where it is not allowed */
    SMX_ERR_ITERATION_CAP = 4, /* an iteration limit was reached */
    SMX_ERR_CUDA = 5,          /* CUDA runtime / library error */
    SMX_ERR_WORKSPACE = 6,     /* workspace too small */
    SMX_ERR_NUMERIC = 7        /* factorisation failed (matrix not positive definite) */
} smx_status;

typedef enum { SMX_FP32 = 0, SMX_FP64 = 1 } smx_precision;

/* Dehnen & Aly (2022) needle models of the bar and bulge slots
 * (_make_explicit_fns, dehnen_bar.py:1272-1555): T1..T4 and V1..V4.  0 selects the
 * slot's canonical model (bar T3, bulge V4).  T0 and V0 are not built. */
enum { SMX_DEHNEN_DEFAULT = 0, SMX_DEHNEN_T1 = 1, SMX_DEHNEN_T2 = 2, SMX_DEHNEN_T3 = 3, SMX_DEHNEN_T4 = 4,
       SMX_DEHNEN_V1 = 11, SMX_DEHNEN_V2 = 12, SMX_DEHNEN_V3 = 13, SMX_DEHNEN_V4 = 14 };

/* Potential Phi = NFW + Miyamoto-Nagai + Dehnen-Aly bar + Dehnen-Aly bulge, all
 * centred at the origin with symmetry axis +z.  With the default model types it is
 * the canonical potential_func / density_func of likelihood.py:13-71 (built from
 * potentials.py:18-65 and dehnen_bar.py:1318-1543): a T3 bar and a V4 bulge; gamma
 * is the needle slope (dehnen_bar.py:211-241).  bar_type / bulge_type choose another
 * member of the family for either slot (SMX_DEHNEN_*), for the forces, the
 * integrator, the initial conditions and the density target alike. */
typedef struct {
    double halo_M, halo_Rs, halo_qa, halo_qb, halo_qc;      /* NFW: M = 10**logM */
    double disc_M, disc_a, disc_b;                            /* MN: M, Rs_disc, Hs_disc */
    double bar_M, bar_a, bar_b, bar_L, bar_gamma;             /* T3 by default */
    double bulge_M, bulge_a, bulge_b, bulge_L, bulge_gamma;   /* V4 by default */
    int bar_type, bulge_type;                                 /* SMX_DEHNEN_* (0: default) */
    /* Optional cylindrical-spline component (CylindricalSpline.py:354-519), added to the
     * potential and the forces (not to the stellar density); cyl_n_modes = 0 leaves it
     * out.  The table is get_phi_m's (CylindricalSpline.py:270-352) in DEVICE memory:
     * cyl_r_grid (cyl_n_r), cyl_z_grid (cyl_n_z): increasing, in asinh(R/cyl_r0) and
     * asinh(|z|/cyl_r0); cyl_coef (cyl_n_modes, 6, cyl_n_r, cyl_n_z): for m = 0 .. n-1,
     * Phi_m_real, Phi_m_img, Mx_real, My_real, Mx_img, My_img.  Outside the grid the
     * component is 0, as in the reference's fill value. */
    int cyl_n_r, cyl_n_z, cyl_n_modes;
    double cyl_r0;
    const double *cyl_r_grid, *cyl_z_grid, *cyl_coef;
} smx_potential;

/* One parameter point of a batched call: its potential and the frame's angular
 * velocity Omega = -Omega_bar (kpc/Gyr). */
typedef struct {
    smx_potential pot;
    double omega;
} smx_point;

/* Library version (major*10000 + minor*100 + patch). */
int smx_version(void);
const char *smx_status_string(int status);
/* Number of kernels this library has launched in the process so far (its own
 * kernels only; cuBLAS/cuSOLVER calls are not counted). */
unsigned long long smx_kernel_launches(void);
/* Copies the last error message of the calling thread into buf (NUL
 * terminated, truncated to len) and returns its full length. */
size_t smx_last_error(char *buf, size_t len);

/* Phi, -grad Phi and stellar rho at n points.  x, y, z: (n,); any output may
 * be NULL.  Replaces potential_func, acc_fn (model.py:152-157, jax.grad) and
 * density_func (likelihood.py:13-71). */
int smx_potential_eval(const smx_potential *pot, int precision, const void *x, const void *y,
                       const void *z, int64_t n, void *phi, void *ax, void *ay, void *az,
                       void *rho, void *stream);

/* Per-particle set-up of the orbit library, fused: axisymmetric Jeans
 * velocities (jeans.py:8-93, 1000-point trapezoids), V_c and T_orb by central
 * differences (utils.py:182-273) and the jitter into n_real realisations
 * (model.py:127-148).
 *   pos      SoA (3, n)          particle positions (dict_data['w0'])
 *   normals  SoA (3, n)          standard normals g1, g2, g3
 *   uniforms (6, n, n_real)      uniform [0,1) draws for the jitter
 * Outputs (NULL allowed for the optional ones):
 *   w_out    SoA (6, n*n_real)   start states, orbit index p*n_real + r
 *   t_total  (n*n_real)          n_periods * T_orb
 *   dt_init  (n*n_real)          T_orb / steps_per_period
 *   w0_new   SoA (6, n)  opt.    un-jittered Jeans state
 *   t_orb    (n)         opt.
 *   vc       (n)         opt. */
int smx_initial_conditions(const smx_potential *pot, int precision, const void *pos,
                           const void *normals, const void *uniforms, int64_t n, int n_real,
                           double n_periods, double steps_per_period, void *w_out,
                           void *t_total, void *dt_init, void *w0_new, void *t_orb, void *vc,
                           void *stream);

/* 3-D density target (model.py:192-213): for each cell c,
 * out[c] = dR dz dphi mean_j rho(R_j cos phi_j, R_j sin phi_j, z_j) R_j with
 * (R,z,phi)_j = (R,z,phi)_c + (sample_j - 1/2)(dR,dz,dphi).
 *   R_grid, z_grid, phi_grid (n_cells) and sample (n_sample, 3) are double;
 *   out (n_cells) has the call's precision. */
int smx_density_target(const smx_potential *pot, int precision, const double *R_grid,
                       const double *z_grid, const double *phi_grid, int64_t n_cells, double dR,
                       double dz, double dphi, const double *sample, int n_sample, void *out,
                       void *stream);

/* ---------------------------------------------------------------- orbits */
enum { SMX_MODE_REFERENCE = 0, SMX_MODE_SAMPLED = 1 };

typedef struct {
    int mode;              /* SMX_MODE_REFERENCE: n_attempts BS23 attempts per orbit,
                              each accepted attempt one sample of weight dt
                              (integrates.py:90-205).
                              SMX_MODE_SAMPLED: integrate to t_total and emit
                              n_samples uniform-time samples (cubic Hermite dense
                              output), weight t_total/n_samples each. */
    int store_all;         /* reference mode: keep every attempt (rejected ones with
                              weight 0) in slot = attempt index, as the trajectory
                              variant does (integrates.py:319-512) */
    int n_attempts;        /* reference mode: N_max */
    int n_samples;         /* sampled mode */
    int64_t max_attempts;  /* sampled mode: cap per orbit (status bit 1 when hit) */
    double atol, rtol, dt_min, dt_max;
    double omega;          /* frame angular velocity Omega = -Omega_bar (kpc/Gyr) */
    const int32_t *order;  /* optional (NULL = 0, 1, 2, ...): device array of n_orb orbit
                              indices, the order in which the work queue hands orbits out.
                              Orbits sorted by expected cost, longest first, keep the
                              lanes of a warp busy for similar times.  Results do not
                              depend on it.  Entries outside [0, n_orb) are skipped; an
                              orbit missing from it is not integrated.  No counterpart in
                              the reference. */
} smx_integrator;

/* Per-orbit record written by smx_integrate (array of n_orb, precision of the
 * call):  t_final, EJ0, EJ_final, weight_sum, n_accepted, n_attempts. */
enum { SMX_INFO_T = 0, SMX_INFO_EJ0 = 1, SMX_INFO_EJ = 2, SMX_INFO_WSUM = 3,
       SMX_INFO_NACC = 4, SMX_INFO_NATT = 5, SMX_INFO_FIELDS = 6 };

/* Adaptive Bogacki-Shampine 3(2) orbits in the bar frame with the canonical
 * forces inline (integrate_adaptive_barred_chunked, integrates.py:37-238;
 * _deriv_barred 8-27; _compute_EJ 29-35).  One GPU thread per orbit; a device
 * work queue hands out orbits.
 *   w0       SoA (6, n_orb)
 *   dt_init  (n_orb)
 *   t_total  (n_orb)           sampled mode: end time; unused otherwise
 *   samples  (7, n_orb, slots) x, y, z, vx, vy, vz, weight of each stored sample
 *   n_stored (n_orb) int32     samples written per orbit
 *   info     (SMX_INFO_FIELDS, n_orb)
 *   status   (n_orb) int32     bit 0 non-finite state, bit 1 attempt cap,
 *                              bit 2 slot overflow, bit 3 stalled: an attempt at
 *                              dt = dt_min was rejected, so (the step being
 *                              deterministic) all later attempts would be too and
 *                              the orbit stops there (0 = clean)
 *   queue    one int32 of device scratch (the call zeroes it).
 * n_orb <= 2^31 - 2^24 (the work counter is 32-bit); larger sizes return
 * SMX_ERR_UNSUPPORTED. */
int smx_integrate(const smx_potential *pot, const smx_integrator *cfg, int precision,
                  const void *w0, const void *dt_init, const void *t_total, int64_t n_orb,
                  int64_t slots, void *samples, int32_t *n_stored, void *info, int32_t *status,
                  int32_t *queue, void *stream);

/* Same as smx_integrate for callers that cannot allocate device memory (a
 * fixed-pool host runtime, code running where allocation is not allowed, a
 * binding with no access to the CUDA allocator): the int32 work counter lives
 * in a 256-byte static device array of the library instead of caller scratch,
 * so only inputs and outputs are passed.  No counterpart in the reference.
 * Limits and rules: n_orb <= 2^31 - 2^24 (32-bit counter; larger sizes return
 * SMX_ERR_UNSUPPORTED); the first call on each device looks up the array's
 * address (make it before any stream capture); calls share the counter, which
 * each call zeroes on its stream, so calls that overlap on the GPU race and
 * must be serialised by the caller.  The device address of the array is looked
 * up once per device and kept: after cudaDeviceReset it is stale, so a process
 * that resets a device must not call this entry point on it again.  Allocates
 * nothing. */
int smx_integrate_noalloc(const smx_potential *pot, const smx_integrator *cfg, int precision,
                          const void *w0, const void *dt_init, const void *t_total, int64_t n_orb,
                          int64_t slots, void *samples, int32_t *n_stored, void *info, int32_t *status,
                          void *stream);

/* The orbits of n_points parameter points in one launch with one work queue
 * (the batched evaluation of jax.vmap(model_likelihood) over parameter points,
 * example/example_schwarmax.ipynb cells 8 and 12): orbit g of
 * n_orb = n_points * per_point belongs to point g / per_point and is integrated
 * in points[g / per_point] (device array of n_points smx_point; cfg->omega is not
 * used).  Every other argument is as for smx_integrate, over all n_orb orbits:
 * w0 SoA (6, n_orb), samples (7, n_orb, slots), info (SMX_INFO_FIELDS, n_orb).
 * blocks_per_sm caps the resident blocks per SM (0 = as many as fit; a tuning
 * knob, results do not depend on it).  n_points <= 1024. */
int smx_integrate_batch(const smx_point *points, int n_points, int64_t per_point, const smx_integrator *cfg,
                        int precision, const void *w0, const void *dt_init, const void *t_total, int64_t slots,
                        void *samples, int32_t *n_stored, void *info, int32_t *status, int32_t *queue,
                        int blocks_per_sm, void *stream);

/* ------------------------------------------------------------- projection */
typedef struct {
    int n_part, n_real;
    int nR, nz, nphi;           /* Rzphi grid, cell = iR + nR*(iz + nz*iphi) */
    double R_lo, R_hi, z_lo, z_hi, phi_lo, phi_hi;
    int nX, nY;                 /* sky grid, pixel = ix + nX*iy */
    double X_lo, X_hi, Y_lo, Y_hi;
    int n_bins;                 /* Voronoi apertures */
    int symmetry;               /* 1: fourfold bar images (library), 0: none (trajectory) */
    double rot[9];              /* row-major X = rot @ x (makeRotationMatrix, utils.py:176-179) */
} smx_binning;

/* Library row layout (rows = n_cells + 6*n_bins): [Rzphi | xy | h0 | h1 | h2 | h3 | h4]. */

/* Projection, aperture assignment and Gauss-Hermite accumulation of stored
 * samples, with the T_integrated normalisation, the E_J / time validity rule
 * and the realisation mean fused (integrates.py:115-174, 207-238, 287-298).
 * One CTA per particle accumulates its n_real realisations in a
 * shared-memory histogram.  Cell indices use IEEE single (double) operations
 * in the order of assign_regular_grid (utils.py:10-42) without contraction.
 *   samples, n_stored, info: as written by smx_integrate (orbit p*n_real + r)
 *   t_total     (n_part*n_real)        validity needs t_final > t_total/10
 *   bin_mapping (nX*nY + 1) int32      last entry is the -1 sentinel
 *   num_per_bin (n_bins) double; v0, s (n_bins) double (km/s)
 *   library     (n_part, rows)         precision of the call
 *   valid       (n_part*n_real) int8   optional */
int smx_project_bin(const smx_binning *geo, int precision, const void *samples,
                    const int32_t *n_stored, int64_t slots, const void *info,
                    const void *t_total, const int32_t *bin_mapping, const double *num_per_bin,
                    const double *v0, const double *s, void *library, int8_t *valid,
                    void *stream);

/* smx_project_bin for the orbits of n_points parameter points stored one point
 * after another (as smx_integrate_batch writes them): point q has the rotation
 * rots[9 q .. 9 q + 8] (device array, row-major like geo->rot, which is not used);
 * geo->n_part is the particle count of one point.  library (n_points, n_part, rows),
 * valid (n_points * n_part * n_real). */
int smx_project_bin_batch(const smx_binning *geo, int n_points, const double *rots, int precision,
                          const void *samples, const int32_t *n_stored, int64_t slots, const void *info,
                          const void *t_total, const int32_t *bin_mapping, const double *num_per_bin,
                          const double *v0, const double *s, void *library, int8_t *valid, void *stream);

/* Cells of individual points (fourfold images when geo->symmetry), with the
 * same arithmetic as smx_project_bin; replaces the index part of bin_chunk
 * (integrates.py:115-146) and assign_regular_grid (utils.py:10-42).
 *   points SoA (6, n); cells, bins (n_img, n) int32 with n_img = 4 or 1
 *   (cell = n_cells and bin = -1 mark points outside); vlos (n_img, n) km/s,
 *   optional. */
int smx_sample_cells(const smx_binning *geo, int precision, const void *points, int64_t n,
                     const int32_t *bin_mapping, int32_t *cells, int32_t *bins, void *vlos, void *stream);

/* ------------------------------------------------- differentiable projection */
/* Sky rows [xy | h0..h4] of the library (rows n_cells .. n_cells + 6 n_bins of each
 * particle's column, same normalisation and validity as smx_project_bin) with soft
 * aperture assignment: each sample image is spread over the pixels by a Gaussian of
 * sigma_pix pixels integrated over each pixel (window +-3 pixels), and its
 * line-of-sight velocity is multiplied by vscale.  geo->rot is the rotation for the
 * viewing angles.  The Rzphi rows are not written.  In double the sums are exact
 * fixed-point sums (units of 2^-56, so the rows are deterministic); they hold for
 * finite dispersions s >= 0.01 km/s, which keep every row sum below 64.  No reference
 * counterpart (the reference has no gradient: stop_gradient at nnls.py:66,165). */
int smx_soft_project(const smx_binning *geo, int precision, double sigma_pix, double vscale, const void *samples,
                     const int32_t *n_stored, int64_t slots, const void *info, const void *t_total,
                     const int32_t *bin_mapping, const double *num_per_bin, const double *v0, const double *s,
                     void *library, void *stream);

/* Adjoint of smx_soft_project: grad[0..3] += dL/d(alpha, beta, gamma, vscale) for a
 * cotangent dL/dlibrary (n_part, rows) of the call's precision (only the sky rows are
 * read).  drot (3 x 9 doubles, host memory, like geo->rot) holds d rot / d alpha,
 * d beta, d gamma.  The rotated samples are recomputed, not stored. */
int smx_soft_project_adjoint(const smx_binning *geo, int precision, double sigma_pix, double vscale,
                             const double *drot, const void *samples, const int32_t *n_stored, int64_t slots,
                             const void *info, const void *t_total, const int32_t *bin_mapping,
                             const double *num_per_bin, const double *v0, const double *s, const void *cotangent,
                             double *grad, void *stream);

/* ------------------------------------------------------------------- NNLS */
enum { SMX_NNLS_FP64 = 0, SMX_NNLS_MIXED = 1 };

typedef struct {
    int64_t n;          /* orbits (columns) */
    int64_t m;          /* design rows */
    int64_t n_rhs;      /* bootstrap right-hand sides */
    int64_t ld_lib;     /* row stride of the library (rows per orbit) */
    int lib_precision;  /* SMX_FP32 / SMX_FP64 element type of the library */
    int mode;           /* SMX_NNLS_FP64 or SMX_NNLS_MIXED */
    int maxiter;
    double lambda_reg;
    double w_init;      /* initial w = z (sum(y_Rzphi)/n) */
} smx_nnls_problem;

/* Bytes of device workspace smx_nnls_admm needs. */
int smx_nnls_workspace_size(const smx_nnls_problem *prob, size_t *bytes);

/* ADMM NNLS shared by n_rhs right-hand sides (solve_nnls_admm_bootstrap,
 * nnls.py:68-166; with n_rhs = 1 it is solve_nnls_admm, nnls.py:6-66).
 * The design matrix is U[r, i] = library[i*ld_lib + row_map[r]] * row_scale[r];
 * Q = U^T U + (lambda/n) I, rho = tr(Q)/n and each of maxiter iterations
 * applies (Q + rho I)^-1, evaluated through the Woodbury identity with the
 * m x m matrix rho' I + U U^T (rho' = rho + lambda/n) factorised by Cholesky.
 *   row_map (m) int32, row_scale (m) double, Y (n_rhs, m) double scaled data
 *   Z_out   (n_rhs, n) double: final z of every right-hand side. */
int smx_nnls_admm(const smx_nnls_problem *prob, const void *library, const int32_t *row_map,
                  const double *row_scale, const double *Y, double *Z_out, void *workspace,
                  size_t workspace_bytes, void *stream);

/* Leave-group-out jackknife of the single right-hand-side ADMM NNLS, all
 * replicates in one batched solve (model_deltaChi2_jackknife, model.py:480-603,
 * with solve_nnls_admm, nnls.py:6-66, per replicate).  Replicate j solves the
 * problem of smx_nnls_admm with the design rows drop_rows[j*max_drop ..
 * (j+1)*max_drop) removed (-1 entries are padding; the reference raises their
 * sigma to 1e20, which differs from removing them by 1e-40 of ||U||^2): its own
 * rho_j = tr(Q_j)/n and data row, the shared w_init.  Every replicate's inverse
 * comes from the one G^-1 of the full problem (Schur complement of the dropped
 * rows, Neumann series for the shift of rho_j; the number of terms follows the
 * largest group's share of ||U||_F^2, which must stay below 1/2).  A design row
 * may be dropped by one replicate at most.  Mixed mode only (split products).
 *   prob->n_rhs = replicates G;  Y (m) double: the scaled data row;
 *   drop_rows (G, max_drop) int32, max_drop <= 40;  Z_out (G, n) double. */
int smx_nnls_jackknife_workspace_size(const smx_nnls_problem *prob, int max_drop, size_t *bytes);
int smx_nnls_jackknife(const smx_nnls_problem *prob, const void *library, const int32_t *row_map,
                       const double *row_scale, const double *Y, const int32_t *drop_rows, int max_drop,
                       double *Z_out, void *workspace, size_t workspace_bytes, void *stream);

/* FP64-accurate product C = A B (A: M x K, B: K x N, C: M x N, all column-major
 * double) on the bf16 tensor cores by Ozaki splitting: every row of A and column
 * of B is scaled by a power of two and split into a_slices / b_slices bf16
 * slices of 8 bits (4 slices: 31 bits, 5 slices: 39 bits below the largest
 * magnitude of the row or column); slice products are accumulated exactly in
 * FP32 tensor memory where the result needs it.  The error is about 2^-39 of
 * sum_k |A_ik| |B_kj|.  Supported (a_slices, b_slices): (4, 4) and (5, 4) for
 * N <= 112, (4, 4), (5, 5) and (7, 7) for any N.  lower != 0 computes only the
 * 128 x 128 output tiles on and below the diagonal (symmetric products, M == N;
 * the other entries of C are 0).  No reference counterpart: this is the
 * product the mixed-precision NNLS is built on, exposed so that it can be
 * tested on its own.  Synchronises the stream. */
int smx_split_gemm_workspace_size(int64_t M, int64_t N, int64_t K, int a_slices, int b_slices, size_t *bytes);
int smx_split_gemm(int64_t M, int64_t N, int64_t K, int a_slices, int b_slices, int lower, const double *A,
                   const double *B, double *C, void *workspace, size_t workspace_bytes, void *stream);

/* FP32 inverse of a symmetric positive definite m x m matrix G (column-major
 * double input, float output Xinv (m x m)) by blocked Gauss-Jordan elimination
 * without pivoting, 2 m^3 flops on the FP32 pipe.  It is the seed that the mixed
 * NNLS refines by Newton-Schulz steps to FP64 accuracy (in place of the reference's
 * Cholesky factorisation, nnls.py:121); exposed so that it can be tested on its own.
 * Returns SMX_ERR_NUMERIC when a pivot is not positive.  Synchronises the stream. */
int smx_spd_inverse_f32_workspace_size(int64_t m, size_t *bytes);
int smx_spd_inverse_f32(const double *G, int64_t m, float *Xinv, void *workspace, size_t workspace_bytes,
                        void *stream);

/* The seed the mixed NNLS actually refines: G^-1 (double, exactly symmetric) of FP32
 * quality by block elimination on Schur complements, G = [A B; B^T C] ->
 * [A^-1 + V W^T, -V; -V^T, S^-1] with W = A^-1 B, S = C - B^T W, V = W S^-1, recursing
 * on A and S down to blocks of 1,024 rows (inverted by the Gauss-Jordan above); the
 * products run on the split tensor-core kernel (4 slices, pairs s + t <= 5).  About
 * m^3 tensor flops per slice pair instead of 2 m^3 FP32 flops.  Returns SMX_ERR_NUMERIC
 * when a pivot is not positive.  Synchronises the stream. */
int smx_spd_inverse_seed_workspace_size(int64_t m, size_t *bytes);
int smx_spd_inverse_seed(const double *G, int64_t m, double *X, void *workspace, size_t workspace_bytes,
                         void *stream);

/* ------------------------------------------------------- model maps, chi2 */
typedef struct {
    int64_t n;           /* orbits */
    int64_t n_rhs;       /* weight vectors */
    int64_t ld_lib;      /* library row stride */
    int lib_precision;
    int n_cells, n_bins;
    double lum_factor;   /* mean_mass_per_orb / (M/L) */
    double sigma_amplify;
} smx_maps_problem;

/* Model maps per weight vector and the chi^2 of each
 * (compute_model_single, model.py:14-68; h_to_V_sigma, ghmoments.py:53-78;
 * model_likelihood, likelihood.py:192-238).
 *   W (n_rhs, n) double.  gamma_kin, v0, s (n_bins) double.
 *   data: y_rz (n_cells) normalised 3-D target, y_xy (n_bins) observed surface
 *         density, y_xy_boot (n_rhs, n_bins), y_h_boot (4, n_rhs, n_bins),
 *         sig_h_raw (4, n_bins) = h_k errors + EPSILON, all double.  The chi^2
 *         uses sigma = 0.1 y_rz, 0.1 y_xy and sig_h_raw, each times sigma_amplify.
 *   maps_out (n_rhs, n_cells + 7*n_bins) double, layout
 *         [density_3d | surface | h1 | h2 | h3 | h4 | V | sigma]  (optional)
 *   logl_out (n_rhs) double: -1/2 chi^2 of each weight vector, with the
 *         Rzphi term summed over all vectors as the reference does. */
int smx_model_maps(const smx_maps_problem *prob, const void *library, const double *W,
                   const double *gamma_kin, const double *v0, const double *s,
                   const double *y_rz, const double *y_xy, const double *y_xy_boot, const double *y_h_boot,
                   const double *sig_h_raw, double *maps_out, double *logl_out,
                   void *workspace, size_t workspace_bytes, void *stream);

int smx_model_maps_workspace_size(const smx_maps_problem *prob, size_t *bytes);

/* ------------------------------------------------------------- post-analysis */
/* Circular-orbit table of build_Lcirc_of_E (utils.py:275-341): n_grid radii
 * R_i = np.logspace(log10 R_min, log10 R_max, n_grid) on the x axis,
 * Vc^2 = max(R (Phi(R + dR) - Phi(R - dR)) / (2 dR), 0), E_i = Phi(R_i) + Vc^2 / 2,
 * L_i = R_i Vc, all in double.  E_out, L_out (n_grid) double (device). */
int smx_lcirc_table(const smx_potential *pot, double R_min, double R_max, int n_grid, double dR, double *E_out,
                    double *L_out, void *stream);

/* Cubic spline (the interp1d(kind='cubic') of build_Lcirc_of_E) at n points x:
 * knots (n_knots) increasing, coef (4, n_knots - 1) the coefficients of each piece in
 * powers of (x - knot_j), highest first; below / above: the values outside the knots
 * (interp1d's fill_value).  x, out (n) double. */
int smx_spline_eval(const double *knots, const double *coef, int n_knots, double below, double above,
                    const double *x, int64_t n, double *out, void *stream);

/* Circularity lambda_z = L_z / (L_circ(E) + 1e-10) of n phase-space points (the
 * analysis of get_model_with_orbit's trajectories, example/example_analysis.ipynb,
 * model-side circularity cell): E = v^2 / 2 + Phi(x), L_z = -(x v_y - y v_x), v in
 * kpc/Gyr, L_circ the spline of smx_spline_eval.  points SoA (6, n) of the call's
 * precision; lam, R (cylindrical radius), E (n) optional outputs. */
int smx_circularity(const smx_potential *pot, int precision, const void *points, int64_t n, const double *knots,
                    const double *coef, int n_knots, double L_below, double L_above, void *lam, void *R, void *E,
                    void *stream);

/* Weighted 2-D histogram with np.histogram2d's binning over the given edges
 * (edges_a (na + 1), edges_b (nb + 1) increasing double; a value equal to the last
 * edge falls in the last bin; values outside are dropped).  w may be NULL (weight
 * 1).  The sums are exact fixed point in units of 2^-40 weight_scale (every |w| and
 * every bin's sum must stay below 2^23 weight_scale), so the result does not depend
 * on the order of the adds.  scratch: na * nb uint64; out (na, nb) double. */
int smx_histogram2d(int precision, const void *a, const void *b, const void *w, int64_t n, const double *edges_a,
                    int na, const double *edges_b, int nb, double weight_scale, unsigned long long *scratch,
                    double *out, void *stream);

/* PSF transfer matrix of compute_transfer_matrix (utils.py:413-485): a grid_res^2
 * fine grid over the field of view (np.linspace edges and centres), each point
 * assigned to a Voronoi bin through the nX x nY pixel map bin_mapping (nX * nY
 * entries; -1 = no bin); P[i, j] = sum over fine points q of bin i of the Gaussian
 * filter of bin j's indicator image at q (separable kernel kernel_weights of
 * 2 radius + 1 normalised taps, zero outside the grid, as
 * scipy.ndimage.gaussian_filter(mode='constant')), then every column divided by its
 * sum.  P (total_bins, total_bins) double, row-major.  Sums are exact fixed point.
 * At most 16 distinct bins may fall within one row window of the kernel. */
int smx_psf_transfer_workspace_size(int grid_res, int total_bins, int radius, size_t *bytes);
int smx_psf_transfer(const double *kernel_weights, int radius, int nX, int nY, double X_lo, double X_hi, double Y_lo,
                     double Y_hi, const int32_t *bin_mapping, int total_bins, int grid_res, double *P, void *workspace,
                     size_t workspace_bytes, void *stream);

/* ---------------------------------------------------- MCMC driver (RMH step) */
/* One random-walk Metropolis-Hastings step of n_chains chains in ndim dimensions
 * on the device (the reference's BlackJAX additive random walk with a normal
 * proposal and a uniform box prior, example/example_schwarmax.ipynb cell 12), in
 * two halves around the batched likelihood of the proposals:
 *   smx_rmh_propose: x_prop = x + L eps (L (ndim, ndim) lower triangular row-major,
 *     eps (n_chains, ndim) standard normals), logprior = -log_vol inside
 *     [lo, hi], -inf outside;
 *   smx_rmh_accept: with lp' = logprior_prop + loglike_prop (a non-finite
 *     log-likelihood counts as -1e30), accept where u < min(1, exp(lp' - logdensity))
 *     (u (n_chains) uniform draws): x and logdensity are updated in place and
 *     accepted (n_chains) int32 records the decision.
 * All arrays double (int32 for accepted) on the device; draws are inputs. */
int smx_rmh_propose(const double *x, const double *L, const double *eps, int n_chains, int ndim, const double *lo,
                    const double *hi, double log_vol, double *x_prop, double *logprior, void *stream);
int smx_rmh_accept(double *x, double *logdensity, const double *x_prop, const double *logprior_prop,
                   const double *loglike_prop, const double *u, int n_chains, int ndim, int32_t *accepted,
                   void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SCHWARMAX_H */
