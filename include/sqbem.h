/* sqbem.h -- C ABI of the GB300 boundary-element library for a squirmer in a
 * closed tube (drop-in for the hot path of squirmer-bem-3dtube).
 *
 * Conventions
 *   - Plain pointers and sizes only.  Arrays are HOST memory unless an entry
 *     point says otherwise; the library copies them to and from the GPU.
 *   - A panel is given by its three vertices: V[9*p + 3*k + c] = coordinate c of
 *     vertex k of panel p.  Normals follow from the vertex order (out of the
 *     fluid), exactly as Mesh::geometry does in the reference
 *     (src/utils/mesh.hpp:61-72).
 *   - Vectors per panel or per point are packed xyz: v[3*p + c].
 *   - Every call returns an int status (SQBEM_OK = 0).  sqbem_last_error()
 *     gives the message of the last failure on the calling thread; the C++
 *     headers rethrow it as std::runtime_error with the reference's wording
 *     ("dgetrf failed", "dgesv failed", ...).
 *   - Handles own their device memory and are bound to one CUDA stream.  Calls
 *     on distinct handles may run on different host threads.
 *   - There is no CPU fallback: without a CUDA device, compute entry points
 *     return SQBEM_ERR_NO_DEVICE.
 *   - Device state the library sets up once per process (quadrature tables,
 *     kernel attributes, cached device addresses) does not survive a
 *     cudaDeviceReset by the caller: do not call the library after one.
 */
#ifndef SQBEM_H
#define SQBEM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define SQBEM_OK 0
#define SQBEM_ERR_ARG 1           /* bad argument or size                       */
#define SQBEM_ERR_SINGULAR 2      /* zero pivot (reference: "dgetrf failed")    */
#define SQBEM_ERR_CUDA 3          /* CUDA runtime error                         */
#define SQBEM_ERR_NOT_CONVERGED 4 /* mixed-precision refinement did not reach
                                     its tolerance within its iteration cap     */
#define SQBEM_ERR_NO_DEVICE 5     /* no CUDA device                             */
#define SQBEM_ERR_ALLOC 6         /* device allocation failed                   */
#define SQBEM_ERR_TIMEOUT 7       /* a bounded device wait gave up              */

/* precision modes */
#define SQBEM_FP64 0  /* FP64 assembly and FP64 LU/TRSM/GEMM (matches the FP64
                         reference to 1e-10 relative)                           */
#define SQBEM_MIXED 1 /* FP32 assembly (FP64 self panels), split-BF16 tensor-core
                         LU/TRSM/GEMM accumulated in FP32, FP64 refinement      */

/* Message of the last failure on this thread ("" if none). */
const char* sqbem_last_error(void);
/* Library version string. */
const char* sqbem_version(void);
/* Number of kernel launches issued by this process so far (all entry points). */
long long sqbem_launch_count(void);
/* Limits of the device-side safeguards (no counterpart in the reference, whose
 * LAPACK calls neither wait on the device nor iterate):
 *   gemm_wait_cycles       SM clock cycles a role of the tensor-core GEMM waits
 *                          for one pipeline stage before the call fails with
 *                          SQBEM_ERR_TIMEOUT (default 4e9, about 2 s);
 *   refine_max_iterations  mixed-precision refinement steps before the call
 *                          fails with SQBEM_ERR_NOT_CONVERGED (default 30; 0
 *                          allows none, so every mixed solve then fails).
 * A negative value restores the default.  Process-wide; affects calls that
 * start after it returns. */
int sqbem_set_limits(long long gemm_wait_cycles, int refine_max_iterations);
/* Test hook for the timeout path (no counterpart in the reference): the next
 * `calls` calls of the tensor-core GEMM each make one of their waits a wait on
 * a barrier that nothing completes, so it runs out after gemm_wait_cycles and
 * the entry point that issued the GEMM returns SQBEM_ERR_TIMEOUT, with the
 * device and the library usable afterwards.  0 cancels pending stalls. */
int sqbem_test_gemm_stall(int calls);
/* FMA throughput of this GPU's FP64 and FP32 pipes in TFLOP/s (2 flops per
 * FMA), measured on the spot with independent FMA chains on every SM (about
 * 40 ms; no counterpart in the reference).  The benchmark divides the
 * assembly kernels' flop rates by these. */
int sqbem_pipe_rates(double* fp64_tflops, double* fp32_tflops);
/* Host->device and device->host bytes copied by the library so far. */
int sqbem_transfer_bytes(long long* h2d, long long* d2h);
/* Opt-in per-kernel-class timing (no counterpart in the reference; used by the
 * benchmark): when enabled, CUDA events bracket every launch of the timed
 * kernel classes ("dgemm", "tc_gemm", "assemble_far", "assemble_near", ...)
 * on their own stream, and each launch is credited with its algorithmic flops
 * and bytes.  Enabling clears the totals. */
int sqbem_kernel_stats_enable(int on);
int sqbem_kernel_stats(const char* cls, long long* launches, double* seconds, double* flops, double* bytes);
/* comma-separated names of the classes seen so far */
int sqbem_kernel_stats_classes(char* buf, int cap);

/* Device memory: the library allocates from its own stream-ordered pool, which
 * keeps freed memory for reuse (no re-mapping between batches); the workers of
 * the batched calls also keep up to 1/32 of the device's memory each in idle
 * blocks of their own stream, reused by the next call without the driver's
 * allocator.  trim_pool empties those caches (of workers not running), waits for
 * the device and returns the cached memory to the CUDA driver.  (No counterpart in
 * the reference, which has no device memory.) */
int sqbem_trim_pool(void);

/* ---------------------------------------------------------------- geometry
 * Host-side mesh generators; the output is bit-identical to the reference.
 * Each returns the panel count in *P.  V (9 per panel) and tags (1 per panel)
 * are written only when non-NULL and cap >= *P. */

/* tube_mesh, src/utils/mesh.hpp:149-190 (z: nz1 axial nodes) */
int sqbem_tube_mesh(double R, const double* z, int nz1, int n_theta, int n_r, double* V, int* tags,
                    int cap, int* P);
/* swimmer_tube_mesh, src/utils/mesh.hpp:194-197 */
int sqbem_swimmer_tube_mesh(double R, double L, double a, int n_theta, int n_r, double* V, int* tags,
                            int cap, int* P);
/* uniform_z, src/utils/mesh.hpp:112-116 (nz + 1 nodes into z) */
int sqbem_uniform_z(double z0, double z1, int nz, double* z);
/* icosphere, src/utils/mesh.hpp:208-245 (center: 3 doubles) */
int sqbem_icosphere(double a, int level, const double* center, int tag, double* V, int* tags, int cap,
                    int* P);
/* Mesh::geometry, src/utils/mesh.hpp:61-72: per-panel normal (3), centroid (3),
 * area and h = sqrt(2 area); any output may be NULL. */
int sqbem_geometry(int P, const double* V, double* normal, double* centroid, double* area, double* h);

/* ---------------------------------------------------------------- quadrature
 * panel_integrals, src/utils/kernels.hpp:67-82, batched on the GPU: for each of
 * n (panel, target, self) triples, SL (9, row-major) = int_p G dS and
 * DL (9) = int_p T.m dS with the reference's adaptive rule (7/28/112/448 points
 * by distance / panel size, Duffy self integral).  FP64. */
int sqbem_panel_integrals(int n, const double* V9, const double* x0, const int* self, double* SL,
                          double* DL);

/* ---------------------------------------------------------------- dense
 * solve_dense, src/utils/linalg.hpp:53-58 (dgesv) with LUFactor semantics
 * (linalg.hpp:62-78): B (n x nrhs, column-major) <- A^{-1} B for A (n x n,
 * column-major), FP64 on the GPU.  *pivoted (may be NULL) reports whether row
 * exchanges were needed.  A zero pivot returns SQBEM_ERR_SINGULAR with the
 * message "dgesv failed". */
int sqbem_solve_dense(int n, int nrhs, const double* A, double* B, int* pivoted);

/* gemm, src/utils/linalg.hpp:42-48, in the form the SQBEM_MIXED path uses:
 * C = alpha A B + beta C for column-major FP32 host arrays (A: M x K, B: K x N,
 * C: M x N), with A and B split into BF16 hi and lo parts and the products
 * hi*hi + hi*lo + lo*hi accumulated in FP32 on the tensor cores (tcgen05).
 * Relative accuracy about 2^-16 per product. */
int sqbem_gemm_mixed(int M, int N, int K, float alpha, const float* A, int lda, const float* B, int ldb,
                     float beta, float* C, int ldc);
/* The same with the kernel's tile variant chosen by the caller (-1: the one
 * the tuning table gives for the shape; see sqbem_gemm_variants) and 3
 * products (hi*hi + hi*lo + lo*hi) or 2 (hi*hi + hi*lo: A rounded to BF16,
 * about 2^-8 relative per product).  No counterpart in the reference. */
int sqbem_gemm_mixed_ex(int variant, int products, int M, int N, int K, float alpha, const float* A, int lda,
                        const float* B, int ldb, float beta, float* C, int ldc);
/* Number of tile variants of the tensor-core GEMM kernel (0: 128 x 128 tiles,
 * 3-stage pipeline; 1: 128 x 256 tiles, 2 stages).  The library picks one per
 * launch from the tuning table tuning/tc_gemm.txt beside lib/ (written by the
 * package's tune_gemm.py; SQBEM_TC_TABLE names another file, SQBEM_TC_VARIANT
 * forces one variant).  No counterpart in the reference. */
int sqbem_gemm_variants(int* count);
/* Device time of one grouped launch of `count` (<= 48) problems M x N x K with
 * device-resident pseudo-random split operands, averaged over `reps` launches
 * after one warm-up (the tuner's and the profiles' measurement; no host copies
 * in the timed region).  No counterpart in the reference. */
int sqbem_gemm_timing(int variant, int products, int M, int N, int K, int count, float beta, int reps,
                      double* seconds);

/* ---------------------------------------------------------------- field
 * velocity_at, src/utils/field.hpp:18-34: lab-frame velocity at npts points
 * from the boundary solution (u, f per panel) on the P panels V. */
int sqbem_velocity_at(int P, const double* V, const double* u, const double* f, double mu, int npts,
                      const double* pts, double* out, int precision);

/* velocity_at without device allocation.  No counterpart in the reference.
 * For callers that cannot allocate device memory themselves -- e.g. a host
 * framework that owns all device memory in a pre-reserved arena and forbids
 * allocations inside its time loop.  Same result as sqbem_velocity_at, but
 * V (9 per panel), u, f (3 per panel), pts and out (3 per point) are DEVICE
 * pointers owned by the caller, and stream is a cudaStream_t (NULL: the
 * default stream).  The per-panel records and the overflow flag the kernels
 * need live in a file-scope device array for at most
 * SQBEM_NOALLOC_MAX_PANELS panels (2.3 MB, held by every GPU that loads the
 * library until the process exits); larger P is rejected with SQBEM_ERR_ARG.
 * The first call on each device does a one-time set-up: it looks up the
 * array's device address (cached per device ordinal) and uploads the library's
 * quadrature tables, which synchronizes the whole device; make that first call
 * before any stream capture begins.  Every call shares the array and
 * overwrites it: calls that overlap on the GPU race.  The call returns after
 * its work on `stream` has completed. */
#define SQBEM_NOALLOC_MAX_PANELS 16384
int sqbem_velocity_at_noalloc(int P, const double* V, const double* u, const double* f, double mu, int npts,
                              const double* pts, double* out, int precision, void* stream);

/* ---------------------------------------------------------------- tube
 * Tube, src/swimmer.hpp:33-75: swimmer_tube_mesh + assembly of the tube-tube
 * single-layer block T (3Nt x 3Nt) + Wielandt deflation + LU, all on the GPU.
 * The factor stays in device memory for the handle's lifetime. */
typedef struct sqbem_tube sqbem_tube;
int sqbem_tube_create(double R, double L, double a, int n_theta, int n_r, double mu, int precision,
                      sqbem_tube** out);
/* panel count Nt */
int sqbem_tube_panels(const sqbem_tube* t, int* Nt);
/* tube panels (9 doubles each) and tags (Nt each), host arrays */
int sqbem_tube_mesh_get(const sqbem_tube* t, double* V, int* tags);
void sqbem_tube_destroy(sqbem_tube* t);
/* The tube mesh of these parameters is n_theta-fold rotationally symmetric
 * (tube_mesh, src/utils/mesh.hpp:149-196, puts every node at an angle
 * 2 pi i / n_theta), so the mixed path assembles the tube block from the rows
 * of one sector and rotates 3 x 3 blocks for the others.  No counterpart in
 * the reference.  sqbem_tube_symmetry (host only): *nb = panels per sector, 0
 * if the mesh has no such symmetry; sector[p] and rep[p] (Nt each, may be
 * NULL): panel p is representative rep[p] of sector 0 rotated by sector[p]
 * sectors.  sqbem_tube_block_f32: the deflated FP32 tube block of the mixed
 * path (3 Nt x 3 Nt, column-major) assembled directly (symmetric = 0) or from
 * the rows of one sector (symmetric = 1); for tests. */
int sqbem_tube_symmetry(double R, double L, double a, int n_theta, int n_r, int* nb, int* sector, int* rep);
int sqbem_tube_block_f32(double R, double L, double a, int n_theta, int n_r, double mu, int symmetric, float* out);
/* Y = T^{-1} X (3 Nt x nc, column-major, host FP64) through the Fourier blocks
 * of the tube: with every panel's vectors in its sector's frame T is
 * block-circulant, and a DFT over the sectors splits it into n_theta / 2 + 1
 * complex blocks of order 3 nb, which the mixed path inverts (FP32) and applies
 * on the tensor cores instead of factoring T.  T is the block
 * sqbem_tube_block_f32 returns with symmetric = 1; for tests.  No counterpart in
 * the reference. */
int sqbem_tube_fourier_solve(double R, double L, double a, int n_theta, int n_r, double mu, int nc, const double* X,
                             double* Y);

/* ---------------------------------------------------------------- swimmer
 * SwimmerSolver, src/swimmer.hpp:83-289.  create = constructor + build()
 * (swimmer.hpp:92-97, 180-251): sphere-tube and sphere-sphere blocks, completed
 * double layer, deflation, rigid-body map and the Schur complement onto the
 * sphere tractions and (U, Omega).  tube == NULL is the unbounded fluid.
 * The tube must outlive the swimmer (non-owning, as in the reference). */
typedef struct sqbem_swimmer sqbem_swimmer;
int sqbem_swimmer_create(const sqbem_tube* tube, int Ns, const double* V, const int* tags,
                         const double* center, double mu, int precision, sqbem_swimmer** out);
/* solve_free, swimmer.hpp:107-139: force- and torque-free swimming for nrhs slip
 * fields (slips: nrhs x Ns x 3).  Outputs per right-hand side k: U[3k..],
 * Om[3k..], f_sphere[k*3Ns..], f_tube[k*3Nt..] (the last two may be NULL). */
int sqbem_swimmer_solve_free(sqbem_swimmer* s, int nrhs, const double* slips, double* U, double* Om,
                             double* f_sphere, double* f_tube);
/* solve_prescribed, swimmer.hpp:142-153: rigid sphere with given U, Omega. */
int sqbem_swimmer_solve_prescribed(sqbem_swimmer* s, const double* U, const double* Om,
                                   double* f_sphere, double* f_tube);
/* t_assembly and t_schur, swimmer.hpp:90 (seconds, device-timed) */
int sqbem_swimmer_timings(const sqbem_swimmer* s, double* t_assembly, double* t_schur);
/* refinement diagnostics of the last mixed-precision solve: iterations used and
 * the final relative FP64 residual (max over right-hand sides) */
int sqbem_swimmer_refinement(const sqbem_swimmer* s, int* iterations, double* residual);
/* Adjoint sensitivities (no counterpart in the reference, which has no
 * derivatives; it differentiates the system of swimmer.hpp:107-139, 188-249):
 * solve_free for nrhs slip fields plus, per right-hand side k, the derivatives
 * of U and Omega with respect to a rigid translation c of the sphere (panels
 * and centre together, slip field carried along), row-major 3 x 3 blocks
 * dU_dc[9k + 3a + j] = dU_a/dc_j and dOm_dc likewise.  One transpose solve with
 * the stored LU factors serves every right-hand side; the sphere-tube kernel
 * derivatives are recomputed, not stored.  FP64 swimmers only
 * (SQBEM_ERR_ARG otherwise). */
int sqbem_swimmer_adjoint(sqbem_swimmer* s, int nrhs, const double* slips, double* U, double* Om,
                          double* dU_dc, double* dOm_dc);
void sqbem_swimmer_destroy(sqbem_swimmer* s);

/* ---------------------------------------------------------------- duct flow
 * DuctFlow, src/duct_flow.hpp:22-109: mixed-BC completed BIE on a closed tube
 * (tube_mesh(R, uniform_z(0, L, n_z), n_theta, n_r)), LU once, one solve per
 * pressure drop. */
typedef struct sqbem_duct sqbem_duct;
int sqbem_duct_create(double R, double L, int n_theta, int n_z, int n_r, double mu, int precision,
                      sqbem_duct** out);
int sqbem_duct_panels(const sqbem_duct* d, int* P);
int sqbem_duct_mesh_get(const sqbem_duct* d, double* V, int* tags);
/* DuctFlow::solve, duct_flow.hpp:41-63: u, f (3 per panel, may be NULL), Q */
int sqbem_duct_solve(sqbem_duct* d, double p_in, double p_out, double* u, double* f, double* Q);
void sqbem_duct_destroy(sqbem_duct* d);

/* ---------------------------------------------------------------- batch
 * Batched kinematics: the per-(a/R, beta) body of run_kinematics
 * (src/main.cpp:69-101) for n independent instances in one call.  Instance k:
 * a = 1, tube Tube(1/a_over_R, L_over_R/a_over_R, 1, n_theta, n_r), sphere
 * icosphere(1, sphere_level, (beta (R - 1), 0, 0)), solve_free for the B1 = 1
 * and B2 = 1 slip modes with swimming direction e (main.cpp:88-89), and, if
 * towed != 0 and beta == 0, the towed drag K = -F_z/(6 pi) (main.cpp:90-91).
 * Any squirmer B2/B1 = alpha follows as U = U_B1 + alpha U_B2.
 * results[k * SQBEM_RESULT_STRIDE + ...]: U_B1 (3), Om_B1 (3), U_B2 (3),
 * Om_B2 (3), drag_K (NaN if not computed), Nt, Ns, refinement iterations.
 * *device_seconds (may be NULL) is the GPU time of the whole batch (CUDA events
 * on the batch stream), excluding host-side mesh generation. */
typedef struct {
    double a_over_R, beta, L_over_R;
    double e[3];
    int n_theta, n_r, sphere_level, towed;
} sqbem_instance;

#define SQBEM_RESULT_STRIDE 16
int sqbem_kinematics_batch(int n, const sqbem_instance* inst, int precision, double* results,
                           double* device_seconds);
/* The same batch, also returning the tractions of the solves (the f_sphere
 * and f_tube of SwimmerSolution, swimmer.hpp:78-81): for instance k,
 * f_sphere[k] receives 2 x 3 Ns values (the B1 = 1 mode, then the B2 = 1
 * mode; Ns = 20 * 4^sphere_level) and f_tube[k] 2 x 3 Nt values (Nt as in
 * results).  Either array, or any entry of it, may be NULL. */
int sqbem_kinematics_batch_tractions(int n, const sqbem_instance* inst, int precision, double* results,
                                     double* const* f_sphere, double* const* f_tube, double* device_seconds);

/* Batched adjoint sensitivities: instance k as in sqbem_kinematics_batch
 * (towed ignored), FP64 only.  results[k * SQBEM_ADJOINT_STRIDE + 24 m + ...]
 * for the slip mode m (0: B1 = 1, 1: B2 = 1): U (3), Om (3), dU/dc (9,
 * row-major [a][j]), dOm/dc (9).  For a squirmer B2/B1 = alpha, every quantity
 * is mode 0 + alpha * mode 1, and d(U, Om)/d alpha is mode 1's (U, Om). */
#define SQBEM_ADJOINT_STRIDE 48
int sqbem_adjoint_batch(int n, const sqbem_instance* inst, int precision, double* results,
                        double* device_seconds);

/* ---------------------------------------------------------------- trajectories
 * TrajectoryParams, src/trajectory.hpp:23-36 (same fields, same defaults when
 * filled by sqbem_trajectory_defaults). */
typedef struct {
    double alpha;       /* B2/B1 (pusher < 0 < puller) */
    double a_over_R;    /* confinement */
    double beta0;       /* initial offset from the axis, in units of (R - a) */
    double pitch0_deg;  /* initial tilt toward +x */
    double yaw0_deg;    /* initial tilt toward +y */
    double dt;          /* time step, units a/B1 */
    double t_max;
    double L_over_R;    /* truncated tube length */
    int n_theta;        /* tube panels around the circumference */
    int sphere_level;   /* icosphere refinement */
    double beta_stop;   /* stop when beta exceeds this (wall contact) */
    double budget_s;    /* wall-clock budget per call, 0 = unlimited */
} sqbem_traj_params;

int sqbem_trajectory_defaults(sqbem_traj_params* p);

/* Factored tubes shared across calls (the tube factor cache of the
 * trajectory calls; the reference factors its tube once per run_trajectory,
 * src/trajectory.hpp:47).  sqbem_run_trajectory, sqbem_trajectory_ensemble and
 * sqbem_ensemble_field take their tube -- keyed by R, L, a, n_theta, n_r, mu
 * and the precision mode -- from a process-wide least-recently-used cache of
 * SQBEM_TUBE_CACHE entries (environment variable, default 4, 0 = off), so
 * calls with the same tube assemble and factor it once.  stats: tubes built
 * and cache hits so far, entries held; clear drops every entry (memory is
 * returned once no running call uses it). */
int sqbem_tube_cache_stats(long long* builds, long long* hits, int* entries);
int sqbem_tube_cache_clear(void);

/* run_trajectory, src/trajectory.hpp:42-151: integrates (or resumes) one
 * trajectory -- 3 RK4 start-up steps then 4th-order Adams-Bashforth, |e|
 * renormalised -- rebuilding only the swimmer couplings each evaluation against
 * the tube factored once.  Writes <out_prefix>.csv (t, x, y, z, ex, ey, ez, Ux,
 * Uy, Uz, Omx, Omy, Omz, beta; 10 significant digits) and keeps
 * <out_prefix>.ckpt (17 digits) for restart, in the reference's formats.
 * status receives "finished", "wall contact" or "paused". */
int sqbem_run_trajectory(const sqbem_traj_params* p, const char* out_prefix, int verbose, int precision,
                         char* status, int status_cap);

/* Ensemble of n swimmers in one tube (a_over_R, L_over_R, n_theta and
 * sphere_level from *p), advanced together: every time-stepping stage
 * evaluates all active swimmers with grouped launches.  y0: n x 6 initial
 * states (x, y, z, ex, ey, ez); alpha: n values of B2/B1.  scheme 0 = the
 * reference's RK4 start-up + AB4, 1 = classical RK4 every step.  Outputs:
 * states (n x (steps + 1) x 6), U and Om (n x steps x 3, at the start of each
 * step), status (n: 0 running / finished, 1 wall contact; a swimmer past
 * p->beta_stop is frozen).  *device_seconds (may be NULL): GPU time. */
int sqbem_trajectory_ensemble(int n, const double* y0, const double* alpha, const sqbem_traj_params* p,
                              int steps, int scheme, int precision, double* states, double* U, double* Om,
                              int* status, double* device_seconds);

/* Velocity field of n swimmers (the field mode of src/main.cpp:109-150 over a
 * 3-D grid, per swimmer, for an ensemble): swimmer k at states[6k..] = (x, y,
 * z, ex, ey, ez) with B1 = 1, B2 = alpha[k], in the tube of *p (centred on the
 * swimmer, so z is not used).  Grid: x_i = -0.97 R + 1.94 R i / (nx - 1), y_j
 * likewise, z_l = -z_extent + 2 z_extent l / (nz - 1); the lab-frame velocity
 * (swimmer.hpp:163-173) goes to u[(((k nx + i) ny + j) nz + l) * 3 ..], NaN at
 * points outside r = 0.97 R or within 1.03 a of the sphere centre.  Mixed
 * precision evaluates the 7-point rule in FP32 and the near panels (d < 3) in
 * FP32 / FP64 (448-point rule); FP64 everywhere otherwise. */
int sqbem_ensemble_field(int n, const double* states, const double* alpha, const sqbem_traj_params* p,
                         int nx, int ny, int nz, double z_extent, int precision, double* u,
                         double* device_seconds);

#ifdef __cplusplus
}
#endif

#endif /* SQBEM_H */
