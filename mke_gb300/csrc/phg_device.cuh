// phg_device.cuh -- device-side layout of the sphere operators and the kernel
// entry points shared by the .cu files.
//
// HBM layout.  All rs x rs operators of one mesh share a single sparsity
// pattern (every one is assembled over the same point/triangle adjacency), so
// the pattern is stored once as a slot-major ELL table: col[k * n + i] is the
// k-th smallest column of row i (k < W, W = 7 on icosahedral meshes), padded
// with (col = i, val = 0).  Each operator adds only its value table
// val[k * n + i].  A warp reading slot k of 32 consecutive rows therefore
// issues fully coalesced 128-byte (int) / 256-byte (double) loads, and the
// Cuthill-McKee point order keeps the gathered x[col] within a few cache lines.
// Vectors of several members (ensemble members, right-hand sides) are stored
// member-major: x[v * ld + i].
#pragma once
#include <string>
#include <cstdint>
#include <cuda_runtime.h>

namespace phg {

struct DevEll {
    int n = 0, W = 0;
    const int *col = nullptr;      // W x n
    const double *val = nullptr;   // W x n, the assembled values
};

// One level of a geometric multigrid hierarchy in HBM.  Level 0 is the
// operator being solved; level k+1 is the mesh one refinement coarser.
struct MgLevelDev {
    int n = 0, W = 0;
    const int *col = nullptr;                       // W x n, slot-major
    const double *a64 = nullptr; const float *a32 = nullptr;  // A
    const double *d64 = nullptr; const float *d32 = nullptr;  // 1 / diag(A)
    // prolongation from level k+1: row i takes pc[2i], pc[2i+1] (-1 = none)
    const int *pc = nullptr; const double *pw64 = nullptr; const float *pw32 = nullptr;
    // restriction to level k+1: coarse row c sums rw[q*nc+c] * r[rf[q*nc+c]]
    int Wr = 0;
    const int *rf = nullptr; const double *rw64 = nullptr; const float *rw32 = nullptr;
};

constexpr int MG_MAXLEV = 10;

struct MgDev {
    int nlev = 0;    // 0 = Jacobi preconditioning only
    int nred = 0;    // levels [nred, nlev) run redundantly per block in shared memory
    MgLevelDev lev[MG_MAXLEV];
    int nc = 0;      // coarsest size; dense inverse row-major
    const double *cinv64 = nullptr; const float *cinv32 = nullptr;
    double omega = 0.9;
    int nu1 = 1, nu2 = 1;
    int red_off[MG_MAXLEV] = {0};  // shared-memory element offsets of levels [nred, nlev)
    size_t red_elems = 0;          // shared-memory elements of those levels (x, xt, b, r each)
    size_t group_elems = 0;        // global elements per group for levels [0, nred)
    // Cluster tail: levels [ncl, nred) of a group's V-cycle run inside the
    // group's first thread-block cluster (cl_size CTAs) from distributed shared
    // memory with hardware cluster barriers, instead of over the whole group
    // with global-memory group barriers (ncl == nred: no tail).  Level l's rows
    // are split in chunks of cl_chunk[l] over the cluster's CTAs; each CTA keeps
    // its rows' x, xt, b, r at cl_off[l] (elements) of its cluster region of
    // cl_elems elements.  cl_magic[l]: q = umulhi(i, cl_magic[l]) is the owner
    // CTA of row i (exact for every row, checked when built).
    int ncl = 0, cl_size = 0;
    int cl_chunk[MG_MAXLEV] = {0};
    int cl_off[MG_MAXLEV] = {0};
    unsigned cl_magic[MG_MAXLEV] = {0};
    size_t cl_elems = 0;
};

// Operator of the Krylov solver: the exact A (FP64 residuals), Jacobi-scaled
// copies A D^{-1} for the plain Jacobi path, and optionally a multigrid
// V-cycle used as a flexible right preconditioner instead of Jacobi.
struct DevSolveOp {
    DevEll A;                      // exact values for the FP64 residual b - A x
    const double *as64 = nullptr;  // A D^{-1} (column scaled), FP64
    const float *as32 = nullptr;   // A D^{-1}, FP32 (mixed precision)
    const double *dinv = nullptr;  // 1 / diag(A)
    const float *a32 = nullptr;    // A in FP32 (multigrid path, mixed precision)
    MgDev mg;                      // host copy (sizes)
    const MgDev *mgd = nullptr;    // the same descriptor in device memory (read by the kernel)
    // Block preconditioner of a vertex-interleaved 4-field system (unknown
    // 4i+q, q = 0,1 "w" rows, q = 2,3 "u" rows whose diagonal blocks are -L):
    // z_w = D^-1 v_w, z_u = -Vcycle_L(v_u - M z_w); mgd is then the hierarchy
    // of L and cpl the coupling mass matrix (rs x rs).
    int block4 = 0;
    DevEll cpl;
    const float *cpl32 = nullptr;
    const float *dinv32 = nullptr;
    // Spectrum interval of D^{-1} A for well-conditioned operators (mass
    // matrices, whose Jacobi-scaled eigenvalues lie in about [1/2, 2]): when
    // set, the solver runs Chebyshev iterations inside the FP64 refinement
    // loop instead of GMRES -- no inner products, one group barrier per step.
    double cheb_lmin = 0.0, cheb_lmax = 0.0;
    // FP32 row records of A (8 (column, value) pairs per row, padding (i, 0)):
    // one sequential matrix stream for the lockstep kernels; null if absent
    const uint4 *pk32 = nullptr;
};

// rs x os boundary columns in CSR over rows (few nonzero rows).
struct DevCols {
    int n = 0;
    const int *ptr = nullptr, *col = nullptr;
    const double *val = nullptr;
};

enum Precision { PREC_FP64 = 0, PREC_MIXED = 1 };

struct GmresStats {
    double relres;   // max final ||b - A x|| / ||b|| (FP64)
    double bytes;    // algorithmic HBM bytes of the launch (model in phg_gmres.cu)
    int iters;       // Arnoldi steps taken (max over right-hand sides)
    int cycles;      // restarts / refinement sweeps (max over right-hand sides)
    int status;      // 0 ok, 1 not converged, 2 barrier timeout, 3 launch error
    int steps_total; // Arnoldi steps summed over right-hand sides
};

// Solve A X = B for nv right-hand sides (member-major, leading dim ld) by
// restarted GMRES(m) right-preconditioned with Jacobi, one cooperative
// persistent launch; X holds the initial guess on entry.  FP64: every vector
// and coefficient in double.  MIXED: Arnoldi vectors and the operator in
// FP32 (FP32 accumulation), Hessenberg / Givens / least squares and the
// residual b - A x of every restart in FP64 (iterative refinement).
// `work` must hold gmres_work_bytes(...) bytes; `stats_dev` receives a
// GmresStats on the device.


// Launch shape of a solve.  rpb: rows per block of the persistent kernels
// (no block gets fewer rows; 0 = 256).  path, for Chebyshev-solvable
// operators in mixed precision: 1 = lockstep launches over an interleaved
// FP32 multi-vector (8 or more right-hand sides), 0 = per-member persistent
// kernels, -1 = the built-in rule (lockstep from 32 right-hand sides).
struct SolveShape {
    int rpb = 0;
    int path = -1;
};
// the autotuner's table (phg_tune.cu); family: 0 plain GMRES, 1 Chebyshev,
// 2 multigrid-preconditioned, 3 4-field block system
int nv_bucket(int nv);
int solve_family(const DevSolveOp &op);
bool tune_get_solve(int family, int n, Precision p, int nv, SolveShape *out);
void tune_set_solve(int family, int n, Precision p, int nv, const SolveShape &s);
bool tune_get_spmm(int n, int nv, int *tpr);
void tune_set_spmm(int n, int nv, int tpr);
void tune_clear();
std::string tune_describe();
int tune_save(const char *path);
int tune_load(const char *path);

// launch paths of a solve: per-member persistent kernels, or lockstep
// launches over all right-hand sides (Chebyshev / multigrid FGMRES)
enum class SolvePath { Persistent, ChebLockstep, MgLockstep };
SolvePath choose_path(const DevSolveOp &op, int nv, int m, Precision prec, bool no_alloc, const SolveShape *shape,
                      SolveShape *sh_out);
// query the lockstep kernels' launch grids once; call outside any stream
// capture (operator creation does) so that a captured solve only reads them
void lockstep_prepare();
// workspace bytes of the path a solve with this shape (null = tuned/default) takes
size_t gmres_work_bytes(const DevSolveOp &op, int nv, int m, Precision p, const SolveShape *shape = nullptr);
// no_alloc: never allocate (the optional debug phase timers stay off)
// max_sms: use at most this many SMs' worth of co-resident blocks (0 = all);
// callers that run several persistent launches at once partition the SMs
// shape: the launch shape to use (null = the tuned one for this operator,
// else the defaults); the environment variables PHG_ROWS_PER_BLOCK and
// PHG_CHEB_LOCKSTEP override both
// wait_limit: clock64 cycles a group-barrier wait of the persistent kernels
// may spin before the launch gives up with status 2 (0 = the default, ~1 s)
cudaError_t gmres_solve(const DevSolveOp &op, const double *B, double *X, int nv, int ld,
                        int m, int max_iter, double tol, Precision p,
                        void *work, GmresStats *stats_dev, cudaStream_t s, bool no_alloc = false,
                        int max_sms = 0, const SolveShape *shape = nullptr, long long wait_limit = 0);

// Several multigrid Laplacians (meshes of different levels) in ONE
// persistent launch: segment k has nvk[k] right-hand sides B[k] + j ldk[k]
// (solutions X[k] + j ldk[k], initial guesses on entry), all to the same
// tolerance; groups of blocks take right-hand sides of any segment, each with
// its own operator, multigrid hierarchy and vectors.  At most 6 segments;
// work must hold gmres_multi_work_bytes bytes; one GmresStats (the worst
// right-hand side) in stats_dev.
size_t gmres_multi_work_bytes(const DevSolveOp *const *ops, const int *nvk, int nseg, int m, Precision p);
cudaError_t gmres_solve_multi(const DevSolveOp *const *ops, const int *nvk, const double *const *B, double *const *X,
                              const int *ldk, int nseg, int m, int max_iter, double tol, Precision p, void *work,
                              GmresStats *stats_dev, cudaStream_t s, int max_sms = 0, long long wait_limit = 0);

// y[v] = A x_in[v] + C x_bnd[v] with every row summed in ascending column
// order from 0.0 and no fused multiply-add (same rounding as a CPU CSR
// product); the two partial sums are added last.  x_bnd may be null.
cudaError_t apply_exact(const DevEll &A, const DevCols &C, const double *x_in, int ldx,
                        const double *x_bnd, int ldb, double *y, int ldy, int nv, cudaStream_t s);

}  // namespace phg
