/*
 * phelm_gb300.h -- C ABI of the GB300 sphere-FEM library (libphelm_gb300.so).
 *
 * This is the drop-in boundary for the reference's sphere hot path
 * (resetius/mke "Phelm"): the icosahedral sphere mesh, the P1
 * SphereLaplace / SphereJacobian / SphereNorm operators with their GMRES
 * solves, and the BarVortex / Baroclin Crank-Nicolson steps.  The C++ facade
 * in phelm_gb300.hpp keeps the reference's class API on top of it.
 *
 * Conventions
 *   - Every function returns PHG_OK (0) or a PHG_ERR_* code; phg_last_error()
 *     gives a message for the calling thread's last failure.
 *   - Sizes follow the mesh: V points, rs inner points, os boundary points.
 *     Vectors over the mesh are "full" (V entries, point order) or "inner"
 *     (rs entries, inner order); boundary values have os entries.  A NULL
 *     boundary pointer means a zero boundary, as in the reference
 *     (src/proj.cpp:57-67).
 *   - Vector arguments may be host or device (cudaMalloc'd) pointers.  Device
 *     pointers are used in place and the call only enqueues work on `stream`
 *     (NULL = the handle's own stream); host pointers are staged through the
 *     handle's device buffers and the call returns after the result is back.
 *   - Scalars (norms) are written to host memory and the call synchronises.
 *   - A handle may be used from one thread / stream at a time; different
 *     handles may run concurrently on different streams.
 *   - Outputs may alias inputs where the reference allows it
 *     (BarVortex::calc with u1 == u, examples/test_barvortex.cpp:529).
 *   - Handles may be destroyed in any order: an operator set holds its mesh
 *     and a time stepper holds its operator set until it is destroyed itself
 *     (the reference's classes keep references to the mesh in the same way).
 */
#ifndef PHELM_GB300_H
#define PHELM_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define PHG_OK 0
#define PHG_ERR_ARG 1           /* bad argument / size / handle */
#define PHG_ERR_CUDA 2          /* CUDA runtime error (no device, OOM, launch failure) */
#define PHG_ERR_NOT_CONVERGED 3 /* a linear solve missed its tolerance */
#define PHG_ERR_TIMEOUT 4       /* a device-side wait ran out (kernel returned early) */
#define PHG_ERR_IO 5            /* mesh file unreadable or malformed */
#define PHG_ERR_BUDGET 6        /* serving: the request's lane does not fit in the HBM budget */
#define PHG_ERR_HOST 7          /* host-side failure: host memory exhausted, a thread not started */

#define PHG_FP64 0   /* every operator, vector and coefficient in double */
#define PHG_MIXED 1  /* FP32 Krylov vectors and operator inside FP64 iterative refinement */

typedef struct phg_mesh_s *phg_mesh;
typedef struct phg_ops_s *phg_ops;
typedef struct phg_barvortex_s *phg_barvortex;
typedef struct phg_baroclin_s *phg_baroclin;

const char *phg_last_error(void);
const char *phg_version(void);
/* Instrumentation, no reference counterpart: number of CUDA kernels this
 * library has enqueued since it was loaded. */
long long phg_kernel_launches(void);

/* ------------------------------------------------------------------ mesh --
 * Host-only (no GPU needed). */

/* Icosahedral sphere mesh, `level` subdivisions (1..9), south pole as the
 * single boundary point, Cuthill-McKee point order.  Replaces running
 * "mke_mesh_sphere --type full --coord local --iter level"
 * (utils/icosahedron.cpp:481-624, utils/mesh_builder.cpp:52-585) and then
 * Mesh::load (src/mesh.cpp:323-519); the result is identical. */
int phg_mesh_generate(int level, phg_mesh *out);
/* Host-side level cache (no reference counterpart).  Mesh handles of the same
 * generated level share one copy of the mesh, its assembled operators and its
 * multigrid hierarchy while any of them is alive.  With a cache directory
 * (this call, or the environment variable PHG_CACHE_DIR) a generated level is
 * read from <dir>/phelm_level<n>.cache when present and valid, else generated,
 * fully assembled and written there (atomically, best effort), so later
 * processes skip generation and assembly; the data are stored byte for byte.
 * NULL or "" disables the directory. */
int phg_cache_dir(const char *path);
/* Mesh::load(FILE*) (src/mesh.h:411, src/mesh.cpp:323-519) from a file in
 * the reference's text format (charts stdsphere1..4). */
int phg_mesh_load_file(const char *path, phg_mesh *out);
void phg_mesh_destroy(phg_mesh m);
/* The reference's mesh text file (the output of "mke_mesh_sphere --type full
 * --coord local", utils/icosahedron.cpp:268-457).  For a generated mesh the
 * file equals the reference generator's byte for byte; a loaded mesh is
 * written from its parsed coordinates. */
int phg_mesh_save_file(phg_mesh m, const char *path);
/* print_function / print_inner_function (src/phelm.cpp:160-321): a full
 * vector ans[V] as text; x, y, z (host, V values each, or NULL) replace the
 * zone-0 coordinates (u, v, 0), i.e. the values of the reference's x_t
 * callbacks at the points.  The inner variant lists inner points and the
 * triangles made of them.  Host memory only. */
int phg_print_function(phg_mesh m, const char *path, const double *ans, const double *x, const double *y,
                       const double *z);
int phg_print_inner_function(phg_mesh m, const char *path, const double *ans, const double *x, const double *y,
                             const double *z);
/* Binary checkpoints of a model state (nfields full vectors of the mesh, the
 * model time and step count); the file records the mesh (size and a digest of
 * its points and triangles) and loading into another mesh is refused.  No
 * reference counterpart.  Host memory only. */
int phg_state_save(phg_mesh m, const char *path, const double *const *fields, int nfields, double t, long long step);
int phg_state_load(phg_mesh m, const char *path, double *const *fields, int nfields, double *t, long long *step);
/* Mesh::size / inner_size / outer_size / tr.size() (src/mesh.h:381-383). */
int phg_mesh_info(phg_mesh m, int *V, int *T, int *rs, int *os);
/* Copies of Mesh::ps (xyz: V x 3; uv: V x 4 x 2 chart coordinates), Mesh::tr
 * (tri: T x 3, tz: T zones), boundary flags (V); any pointer may be NULL. */
int phg_mesh_arrays(phg_mesh m, double *xyz, double *uv, int *tri, int *tz, int *bnd);
/* Mesh::inner / outer / p2io (src/mesh.h:375-379); any pointer may be NULL. */
int phg_mesh_maps(phg_mesh m, int *inner, int *outer, int *p2io);
/* Host-assembled operator in CSR, as phelm::Solver::add accumulates it.
 * name: "idt" "lapl" "bnd2" "bnd3" (SphereLaplace, src/impl/slaplace_impl.h:133-145),
 * "jidt" "d1" "d2" "d1c" "d2c" "d1b" "d2b" "d1cb" "d2cb" (SphereJacobian,
 * src/sjacobian.cpp:413-454), "norm" (SphereNorm, src/norm.h:70-73).
 * Call with ptr/col/val NULL to get n (rows) and nnz first. */
int phg_mesh_csr(phg_mesh m, const char *name, int *n, int *nnz, int *ptr, int *col, double *val);

/* ------------------------------------------------------------- operators --
 * Uploads the mesh maps and every SphereLaplace / SphereJacobian /
 * SphereNorm operator to the current CUDA device.  Replaces the three
 * constructors SphereLaplace(m) (src/impl/slaplace_impl.h:133-145),
 * SphereJacobian(m) (src/sjacobian.cpp:413-454), SphereNorm(m)
 * (src/norm.h:67-74).  precision: PHG_FP64 or PHG_MIXED. */
int phg_ops_create(phg_mesh m, int precision, phg_ops *out);
void phg_ops_destroy(phg_ops o);
/* GMRES(restart) tolerance (relative residual ||b - A x|| / ||b||) and
 * iteration cap for the solves of this handle.  Defaults: restart 30,
 * tol 1e-12, max_iter 20000; mass-matrix solves inside operator applies use
 * min(tol, 1e-14). */
int phg_ops_set_solver(phg_ops o, int restart, double tol, int max_iter);
/* Persistent solver launches of this handle fill at most max_sms SMs
 * (0 = the whole GPU, the default).  Launches of different handles that run
 * at the same time on different streams then share the GPU instead of
 * queueing behind each other.  No reference counterpart. */
int phg_ops_set_sms(phg_ops o, int max_sms);
/* Bounded waits (no reference counterpart): a group-barrier wait inside the
 * persistent solver kernels of this handle gives up after `cycles` GPU clock
 * cycles (0 = the default, about one second); the launch then ends early and
 * the call (or the next phg_ops_check) returns PHG_ERR_TIMEOUT.  The handle
 * stays usable. */
int phg_ops_set_wait_limit(phg_ops o, long long cycles);
/* Statistics of the last solve on this handle (host memory). */
int phg_ops_last_solve(phg_ops o, int *iters, int *cycles, double *relres);
/* phelm::Solver::mult_vector (src/impl/slaplace_impl.h:109-113,
 * src/sjacobian.cpp:160-181): y = A x for nv member-major inner vectors
 * (nv x rs), A one of the handle's inner x inner operators: "idt" "lapl"
 * (SphereLaplace), "jidt" "d1" "d2" "d1c" "d2c" (SphereJacobian).  FP64,
 * ascending column order: the same bits as the CPU CSR product. */
int phg_ops_mult(phg_ops o, const char *name, double *y, const double *x, int nv, void *stream);
/* The FP32 operator apply of the mixed-precision path ("idt" "lapl" "jidt")
 * on an interleaved multi-vector: x, y are rs x nv with the nv members of a
 * point contiguous (nv = 4, 8, 16, ..., 256; 16-byte aligned device pointers),
 * so every gathered row of x is one contiguous read.  No reference
 * counterpart. */
int phg_ops_mult32(phg_ops o, const char *name, float *y, const float *x, int nv, void *stream);
/* Index validation (debug aid, no reference counterpart): counts the entries
 * of the handle's device index arrays outside their valid range -- the shared
 * ELL pattern, the inner / outer / p2io maps, the norm pattern, the boundary
 * column lists and the multigrid hierarchy (columns, prolongation and
 * restriction lists).  Only the indices are read.  Synchronises the stream. */
int phg_ops_validate(phg_ops o, long long *bad_entries, void *stream);

/* Autotuner (no reference counterpart).  Times the candidate launch shapes
 * of the kernels a barotropic step of nmembers states runs on this handle's
 * mesh and precision -- rows per block of the persistent solver (128, 256,
 * 512, 1024) for the mass solves at nmembers and 8 x nmembers right-hand
 * sides and the Laplace solve at nmembers, the lockstep path for mass solves
 * in mixed precision (8 or more right-hand sides), and threads per row of
 * phg_ops_mult32 at nmembers vectors -- and keeps the fastest in a
 * process-wide table consulted by every later launch of the same kernel
 * family, size, precision and right-hand-side bucket (powers of two).  A
 * shape whose solve misses the tolerance is never chosen.  Solves are timed
 * captured in a CUDA graph and replayed (as the steps of phg_barvortex_run
 * run them); on the legacy or per-thread default stream, enqueued directly.  report (may be
 * NULL) receives one text line per candidate timed and per choice. */
int phg_ops_autotune(phg_ops o, int nmembers, char *report, int report_len, void *stream);
/* The table as text: "solve <family> <rows> <precision> <bucket> <rows per
 * block> <path>" and "spmm <rows> <bucket> <threads per row>" lines
 * (family 0 GMRES, 1 Chebyshev, 2 multigrid, 3 baroclinic block system). */
int phg_tune_describe(char *buf, int len);
/* Save / load the table (a text file headed by the device model; a file
 * from another model loads 0 entries).  Loading adds to the table. */
int phg_tune_save(const char *path);
int phg_tune_load(const char *path, int *entries);
void phg_tune_clear(void);

/* Synchronise `stream` and check the solves enqueued on this handle since the
 * last check (calls with device pointers do not wait for their solves):
 * PHG_ERR_NOT_CONVERGED / PHG_ERR_TIMEOUT as a host-pointer call would
 * return.  No reference counterpart (the reference's calls are synchronous). */
int phg_ops_check(phg_ops o, void *stream);
/* Device bytes held by the library: in total, and allocated by the calling
 * thread.  Instrumentation for memory budgets, no reference counterpart. */
int phg_device_bytes(long long *total, long long *this_thread);
/* Instrumentation, no reference counterpart: while enabled, every solver
 * launch of this handle (and of models built on it) is bracketed by CUDA
 * events on its stream and its algorithmic byte count is kept (up to 4096
 * launches).  profile_read synchronises and returns the number of solver
 * launches, their summed device time in ms and their summed algorithmic
 * bytes since the last enable. */
int phg_ops_profile(phg_ops o, int enable);
int phg_ops_profile_read(phg_ops o, int *launches, double *ms, double *bytes);
/* The same restricted to the launches of one solver family (0 GMRES, 1
 * Chebyshev, 2 multigrid-preconditioned GMRES, 3 baroclinic block system;
 * -1 = all), e.g. the Laplacian solves' gmres_kernel launches alone. */
int phg_ops_profile_read_family(phg_ops o, int family, int *launches, double *ms, double *bytes);

/* SphereLaplace::calc1 (src/impl/slaplace_impl.h:176-192): ans[V] = Laplacian
 * of F[V] with boundary values bnd[os] written on the boundary. */
int phg_laplace_calc1(phg_ops o, double *ans, const double *F, const double *bnd, void *stream);
/* SphereLaplace::calc2 (src/impl/slaplace_impl.h:147-174): ans[rs] on inner points. */
int phg_laplace_calc2(phg_ops o, double *ans, const double *F, void *stream);
/* SphereLaplace::solve (src/impl/slaplace_impl.h:84-131): ans[V] with
 * Laplacian(ans) = F[V] and ans = bnd[os] on the boundary. */
int phg_laplace_solve(phg_ops o, double *ans, const double *F, const double *bnd, void *stream);
/* nv independent SphereLaplace::solve calls in one persistent launch
 * (member-major: ans, F: nv x V; bnd: nv x os or NULL).  The reference calls
 * solve once per right-hand side. */
int phg_laplace_solve_batch(phg_ops o, int nv, double *ans, const double *F, const double *bnd, void *stream);
/* SphereLaplace::solve (src/impl/slaplace_impl.h:84-131) for right-hand sides
 * on meshes of DIFFERENT levels in one persistent launch (no reference
 * counterpart: the reference solves one mesh at a time).  Handle k (count <=
 * 6 handles of one precision on one device, each with its multigrid
 * hierarchy) takes nv[k] right-hand sides F[k] (nv[k] x V_k, member-major)
 * with boundary values bnd[k] (nv[k] x os_k, or bnd / bnd[k] NULL) into
 * ans[k].  Every solve runs to the first handle's restart, tolerance and
 * iteration cap; the solve record goes to the first handle (phg_ops_check /
 * phg_ops_last_solve on ops[0]).  Groups of blocks of the one launch take
 * right-hand sides of any mesh, each with its own operator and hierarchy, so
 * small meshes share the GPU instead of each holding a launch. */
int phg_laplace_solve_levels(int count, const phg_ops *ops, const int *nv, double *const *ans, const double *const *F,
                             const double *const *bnd, void *stream);
/* No counterpart in the reference.  phg_laplace_calc2 for callers that cannot
 * let a library allocate device memory (memory owned by their own pool or
 * allocator, or loops where the device synchronisation of a cudaMalloc would
 * stall their other streams).  It calls no cudaMalloc/cudaFree: its
 * right-hand side and solver workspace live in one fixed 16 MiB device array
 * inside the library (held by every GPU that loads the library until the
 * process exits).  That holds the default Chebyshev mass solve up to level 7
 * in FP64 (163,841 inner points), or a GMRES(30) mass solve up to level 6;
 * larger needs are rejected with PHG_ERR_ARG.
 * ans[rs] and F[V] must be device pointers; the call only enqueues work on
 * `stream`, so it reports no solver failure itself: call phg_ops_check to
 * learn whether the mass solve converged (PHG_ERR_NOT_CONVERGED for a
 * non-finite F or a missed tolerance).  The first call on each device looks
 * up the array's device address (make it before any stream capture).  All
 * calls share the array: calls that overlap on the GPU (e.g. on two streams)
 * race. */
int phg_laplace_calc2_noalloc(phg_ops o, double *ans, const double *F, void *stream);
/* SphereJacobian::calc1 / calc2 / calc2t (src/sjacobian.cpp:348-408, 456-461). */
int phg_jacobian_calc1(phg_ops o, double *ans, const double *u, const double *v, const double *bnd, void *stream);
int phg_jacobian_calc2(phg_ops o, double *ans, const double *u, const double *v, void *stream);
int phg_jacobian_calc2t(phg_ops o, double *ans, const double *u, const double *v, void *stream);
/* The 8 derivative products inside SphereJacobian::calc2 before its mass
 * solves (src/sjacobian.cpp:136-362: D2cos u, D1 v, D1cos u, D2 v, D2 u,
 * D1cos v, D1 u, D2cos v, each with its boundary columns) for nv members:
 * u, v full vectors (nv x V, member-major), out nv x 8 x rs.  quad = 0: the
 * assembled FP64 operators (the same bits as the CPU CSR products); quad = 1:
 * the FP32 element-loop quadrature the mixed-precision time steps use (the
 * integrals formed from the mesh geometry on the fly).  Device pointers only;
 * the call only enqueues work. */
int phg_jacobian_derivs(phg_ops o, int quad, double *out, const double *u, const double *v, int nv, void *stream);
/* SphereJacobian::calc1t (src/sjacobian.h:116, src/sjacobian.cpp:463-468):
 * the adjoint -J(u, v) on the inner points, ans[V] with bnd[os] on the boundary. */
int phg_jacobian_calc1t(phg_ops o, double *ans, const double *u, const double *v, const double *bnd, void *stream);
/* SphereJacobian::calc2_diff_x / calc2_diff_cos_y (src/sjacobian.h:143-148,
 * src/sjacobian.cpp:364-402): ans[rs] = du/dx, resp. (1/cos y) du/dy, of the
 * full vector v[V] on the inner points (derivative operator with its boundary
 * columns, then the Jacobian mass solve). */
int phg_jacobian_calc2_diff_x(phg_ops o, double *ans, const double *v, void *stream);
int phg_jacobian_calc2_diff_cos_y(phg_ops o, double *ans, const double *v, void *stream);
/* SphereNorm::norm / dist / scalar (src/norm.h:81-94); result to *out (host). */
int phg_norm(phg_ops o, const double *u, double *out, void *stream);
int phg_dist(phg_ops o, const double *u, const double *v, double *out, void *stream);
int phg_scalar(phg_ops o, const double *u, const double *v, double *out, void *stream);

/* ------------------------------------------------------------- barvortex --
 * BarVortexConf (examples/barvortex.h:62-96); theta is explicit (the
 * reference leaves it uninitialised).  picard_iters: Picard iterations per
 * step; the reference loops up to 1000 and stops when the update is below
 * 1e-14 of the state norm (examples/barvortex_impl.h:260, 300-306) -- the
 * same stop test is applied here within picard_iters. */
typedef struct {
	double tau, sigma, mu, k1, k2, theta;
	int picard_iters;
} phg_bv_conf;

/* BarVortex(m, conf) (examples/barvortex_impl.h:109-154); coriolis[V] is
 * l + h at every point (the reference evaluates conf.coriolis with proj). */
int phg_barvortex_create(phg_ops o, const phg_bv_conf *conf, const double *coriolis, phg_barvortex *out);
void phg_barvortex_destroy(phg_barvortex b);
/* BarVortex::calc(u1, u, bnd_u, bnd_w, t) (examples/barvortex_impl.h:171-310):
 * one step of the stream function u[V] -> u1[V]; forcing[V] is f at time t
 * (NULL = no forcing).  u1 may equal u. */
int phg_barvortex_calc(phg_barvortex b, double *u1, const double *u, const double *bnd_u,
                       const double *bnd_w, const double *forcing, void *stream);
/* nmembers independent states advanced together (member-major: member k at
 * u + k * V; bnd_u / bnd_w: os values per member; forcing shared, V values).
 * Each member's result equals a phg_barvortex_calc of that member alone
 * within the solve tolerance.  No reference counterpart (ensemble mode). */
int phg_barvortex_calc_batch(phg_barvortex b, int nmembers, double *u1, const double *u,
                             const double *bnd_u, const double *bnd_w, const double *forcing, void *stream);
/* nsteps steps of nmembers states in place (member-major u, as in
 * phg_barvortex_calc_batch), the same bnd_u / bnd_w / forcing every step:
 * the loop of examples/test_barvortex.cpp:529 (calc(u, u, ...) per step).
 * One step is captured as a CUDA graph and replayed (one graph launch per
 * step); the graph stays on the handle and serves later calls with the same
 * members, pointers and stream, as long as no buffer of the library was
 * reallocated since (otherwise the first step of the call is enqueued kernel
 * by kernel and the next one re-captured).  Results equal nsteps
 * phg_barvortex_calc_batch calls bit for bit.  With host arrays the call
 * returns after the copy back and checks every solve of every step; with
 * device arrays it returns at once, and phg_barvortex_last_stats checks every
 * step run since the previous check.  stream: a created stream or NULL (the
 * handle's own), not the legacy default stream. */
int phg_barvortex_run(phg_barvortex b, int nmembers, int nsteps, double *u, const double *bnd_u,
                      const double *bnd_w, const double *forcing, void *stream);
/* BarVortex::calc_L (examples/barvortex_impl.h:326-400): the step
 * linearised around the background z, applied to u (u1 = L_z u).  Outputs
 * may alias inputs. */
int phg_barvortex_calc_L(phg_barvortex b, double *u1, const double *u, const double *z, const double *bnd_u,
                         const double *bnd_w, void *stream);
/* BarVortex::calc_L_1 (examples/barvortex_impl.h:402-467): the inverse of the
 * linearised step, with the backward matrix Ab_ (built on the first call).
 * Like the reference it ADDS into u1 (u1 is read and written). */
int phg_barvortex_calc_L_1(phg_barvortex b, double *u1, const double *u, const double *z, const double *bnd_u,
                           const double *bnd_w, void *stream);
/* BarVortex::calc_LT (examples/barvortex_impl.h:469-536): the adjoint of the
 * linearised step around z applied to v. */
int phg_barvortex_calc_LT(phg_barvortex b, double *v1, const double *v, const double *z, const double *bnd_u,
                          const double *bnd_w, void *stream);
/* Totals of the last calc on this handle: GMRES iterations of each solve
 * kind (L, A, mass J, mass L) summed over the step, and the worst relative
 * residual of any solve. */
int phg_barvortex_last_stats(phg_barvortex b, int *iters_lapl, int *iters_a, int *iters_mj,
                             int *iters_ml, double *worst_relres);

/* -------------------------------------------------------------- baroclin --
 * Baroclin(m, f, g, coriolis, tau, sigma, mu, sigma1, mu1, alpha)
 * (examples/baroclin.cpp:69-106); theta = 0.5 as in the reference.
 * picard_iters / picard_tol: at most picard_iters iterations, stop when
 * max(dist(u1), dist(u2)) < picard_tol (reference: 20 and 1e-8,
 * examples/baroclin.cpp:547, 600). */
typedef struct {
	double tau, sigma, mu, sigma1, mu1, alpha;
	int picard_iters;
	double picard_tol;
} phg_bc_conf;

int phg_baroclin_create(phg_ops o, const phg_bc_conf *conf, const double *coriolis, phg_baroclin *out);
void phg_baroclin_destroy(phg_baroclin b);
/* Baroclin::calc(u11, u21, u1, u2, bnd, t) (examples/baroclin.cpp:445-606);
 * f, g: forcing fields at time t (V each, NULL = none).  The call reads the
 * Picard stop flag after each iteration (one stream synchronisation per
 * iteration), so it returns after the last iteration's work is done. */
int phg_baroclin_calc(phg_baroclin b, double *u11, double *u21, const double *u1, const double *u2,
                      const double *bnd, const double *f, const double *g, void *stream);
/* Baroclin::calc_L (examples/baroclin.cpp:620-802): the step linearised around
 * (z1, z2) applied to (u1, u2), one iteration.  Outputs may alias inputs. */
int phg_baroclin_calc_L(phg_baroclin b, double *u11, double *u21, const double *u1, const double *u2,
                        const double *z1, const double *z2, const double *bnd, void *stream);
/* Baroclin::calc_L_1 (examples/baroclin.cpp:804-986): the inverse linearised
 * step with the backward block matrix Ab_ (built on the first call), up to 10
 * iterations with the reference's 1e-8 stop test. */
int phg_baroclin_calc_L_1(phg_baroclin b, double *u11, double *u21, const double *u1, const double *u2,
                          const double *z1, const double *z2, const double *bnd, void *stream);

/* --------------------------------------------------------------- serving --
 * Request loop with continuous batching; no reference counterpart (the
 * reference has no serving layer).  Requests are Laplace solves and short
 * barotropic integrations on icosahedral meshes of mixed levels.  Each
 * (kind, level) gets a lane: resident operators, a CUDA stream, a host
 * thread and a number of member slots whose device memory is reserved when
 * the lane opens and counted against the HBM budget.  Requests join a lane as
 * slots free up (barotropic members between two time steps, Laplace solves in
 * the next batched solve) and lanes run concurrently on their streams.  Idle
 * lanes are closed when a new lane needs their memory.  With PHG_SERVE_PACK=L
 * in the environment (default 0: off), Laplace solves of levels up to L share
 * one lane that solves each turn's requests of all those levels in one
 * phg_laplace_solve_levels launch.  Barotropic lanes use
 * l + h = sin(latitude) (2 Omega = 1, no orography) and conf.bv. */
#define PHG_REQ_LAPLACE_SOLVE 0 /* input: F[V]; output: solution[V]; bnd: os values or NULL */
#define PHG_REQ_BARVORTEX 1     /* input: stream function u[V]; `steps` BarVortex::calc steps;
                                   bnd: bnd_u (os values or NULL), bnd_w = 0 */

typedef struct {
	double hbm_budget_bytes; /* device memory the lanes may reserve */
	int precision;           /* PHG_FP64 or PHG_MIXED */
	int max_slots;           /* members per lane (0 = 64); fewer if the budget is short */
	double solve_tol;        /* relative residual of Laplace solve requests */
	double step_tol;         /* relative residual of the solves inside time steps */
	phg_bv_conf bv;          /* barotropic step configuration */
} phg_serve_conf;

typedef struct {
	int kind;              /* PHG_REQ_* */
	int level;             /* icosahedral level 1..9 */
	int steps;             /* PHG_REQ_BARVORTEX: time steps (>= 1) */
	const double *input;   /* host, V values; read when the request is admitted */
	const double *bnd;     /* host, os values or NULL */
	double *output;        /* host, V values; written before the completion is reported */
	long long tag;         /* returned in the completion */
} phg_request;

typedef struct {
	long long tag;
	int status;            /* PHG_OK or the request's PHG_ERR_* */
	int kind, level;
	double t_submit, t_admit, t_done;  /* seconds on phg_serve_clock */
	int batch;             /* members in the launch that finished it */
	char error[128];       /* message when status != PHG_OK */
} phg_completion;

typedef struct phg_serve_s *phg_serve;

int phg_serve_create(const phg_serve_conf *conf, phg_serve *out);
/* Open the lane of (kind, level) ahead of traffic and wait until it is ready. */
int phg_serve_preload(phg_serve s, int kind, int level);
/* Queue a request; input/output must stay valid until its completion is
 * polled.  Bad requests and requests whose lane cannot open complete with
 * their error status (the call itself returns PHG_OK). */
int phg_serve_submit(phg_serve s, const phg_request *req);
/* Up to `max` completions; waits up to wait_s seconds when none is ready. */
int phg_serve_poll(phg_serve s, phg_completion *out, int max, double wait_s, int *n);
int phg_serve_stats(phg_serve s, double *bytes_in_use, int *lanes_open, long long *completed);
double phg_serve_clock(phg_serve s);
/* Finishes every queued request, then frees the lanes. */
void phg_serve_destroy(phg_serve s);

#ifdef __cplusplus
}
#endif
#endif
