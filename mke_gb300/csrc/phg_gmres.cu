// phg_gmres.cu -- persistent restarted (flexible) GMRES on GB300.
//
// One cooperative launch solves nv systems A x = b that share A (ensemble
// members, the 8 derivative right-hand sides of a Jacobian, ...).  The grid is
// split into groups of G blocks; a group owns one right-hand side at a time
// and its blocks own contiguous row ranges, so every dot product, AXPY and
// normalisation touches only rows the block owns -- only operator applies
// gather neighbours.  Groups synchronise among themselves only (G = 1 is a
// plain __syncthreads), so independent right-hand sides converge independently
// and nothing waits for the whole GPU.
//
// Preconditioning (right, flexible): Jacobi, folded into the stored values
// (A D^-1), or a geometric multigrid V-cycle over the nested icosahedral
// meshes.  In the V-cycle the fine levels are smoothed by the group's blocks
// with group barriers; the coarse levels (a few hundred points) are solved by
// every block redundantly in shared memory with __syncthreads only, so the
// coarse half of the cycle costs no cross-block synchronisation.
//
// Per Arnoldi step: [V-cycle z_j = M^-1 v_j], (1) w = A z_j, then the
// classical Gram-Schmidt dots <v_l, w>, (2) w -= sum h_l v_l fused with
// ||w||^2, (3) v_{j+1} = w / |w| and the Givens update (computed redundantly,
// identically, by every block of the group).  Every restart recomputes
// r = b - A x in FP64 with the exact operator, which is also the outer loop
// of mixed-precision iterative refinement.
//
// Register discipline: the kernel copies the fields it needs out of its
// parameter block into locals and the hot loops take no references to it,
// so the parameter block never has to be materialised in local memory; the
// multigrid descriptor is read from device memory through a pointer.
//
// Every wait is bounded: a barrier that spins longer than ~1 s (clock64)
// raises a device error flag; all blocks see the flag at their next barrier
// and return, and the host reports status 2.
#include <cmath>
#include <cstdio>
#include <mutex>

#include <cooperative_groups.h>

#include "phg_kernels.cuh"

namespace phg {

namespace cg = cooperative_groups;

namespace {

constexpr int MAXM = 48;         // largest restart length
constexpr int BLOCK = 256;
constexpr int NWARP = BLOCK / 32;
constexpr double INNER_RTOL = 1e-5;  // FP32 cycle: reduce the residual 1e5x, then refine
constexpr long long SPIN_LIMIT = 2000000000LL;  // default wait limit, clock64 cycles (~1 s)
constexpr int CHEB_KMAX = 64;    // most Chebyshev steps per refinement cycle
constexpr int LS_MIN_RHS = 32;   // right-hand sides from which the lockstep path runs
constexpr int LS_MIN_TUNED = 8;  // the fewest for which the autotuner may choose it
// the multigrid Laplacian runs in lockstep by default from this many
// right-hand sides on meshes of at least LSG_DEFAULT_ROWS rows (measured,
// graph-replayed ensemble steps: L5 x 256 -15 %, L6 x 32 -14 %, L7 x 16 -5 %,
// but L4 x 64 +9 %); elsewhere only when the autotuner chose it
constexpr int LSG_DEFAULT_RHS = 16;
constexpr int LSG_DEFAULT_ROWS = 10000;

// One operator's share of a multi-operator launch (meshes of several levels
// in one persistent launch): right-hand sides [v0, next v0) use this
// operator, read B + k ld and write X + k ld (k = v - v0), and own the Krylov,
// multigrid-direction, work and residual vectors at the given element offsets
// (+ k (m+1) n, k m n, k n, k n).
constexpr int MAXSEG = 6;
struct MultiSeg {
    int v0, n, W, ld;
    int nv;                  // right-hand sides of this segment
    int blk0, G, groups;     // its blocks [blk0, blk0 + groups * G): groups of G
    int gbase;               // launch-wide index of its first group

    const int *col;
    const double *aval;
    const double *sval64;
    const float *sval32;
    const double *dinv;
    const MgDev *mgd;
    const double *B;
    double *X;
    size_t voff, zoff, woff, roff;
    double mg_row_bytes;
};

struct Params {
    DevSolveOp op;
    const double *B;
    double *X;
    int n, nv, ld, m, max_iter;
    double tol;
    void *V;          // nv x vstride (VT): m + 1 Krylov vectors, or 4 Chebyshev vectors
    size_t vstride;   // elements of V per right-hand side
    void *Z;          // nv x m x n (VT), multigrid path only
    void *Wv;         // nv x n (VT)
    double *R;        // nv x n (FP64 residual)
    void *mgbuf;      // groups x per-group V-cycle buffers (parallel levels)
    double *part;     // groups x 2 x (MAXM + 2) x G
    unsigned *bar;    // groups x 2 (one 64-bit arrival count per group)
    int *err;
    GmresStats *stats;
    int groups, G;
    long long *timers;       // optional phase cycle counters (block 0)
    double mg_row_bytes;     // algorithmic bytes of one V-cycle per fine row
    size_t group_elems;      // per-group scratch elements (V-cycle + block preconditioner)
    double inner_rtol;       // mixed path: residual reduction of one FP32 cycle
    // Chebyshev path: steps per refinement cycle and the recurrence
    // coefficients d_k = ca[k] d_{k-1} + cb[k] D^-1 r_k, d_0 = c0 D^-1 r_0
    int cheb_k;
    double cheb_c0, cheb_ca[CHEB_KMAX], cheb_cb[CHEB_KMAX];
    // steps for a residual reduction eps: ceil((cheb_lg - log eps) / cheb_ls) + 1
    double cheb_lg, cheb_ls;
    long long wait_limit;    // clock64 cycles a barrier wait may take before the launch gives up
    int cluster;             // > 0: clustered launch, V-cycle levels [ncl, nred) as a cluster tail
    unsigned long long *ccnt;  // groups: cluster-tail entry counters
    int nseg;                // > 0: multi-operator launch, right-hand sides by segment (op: sizes only)
    MultiSeg seg[MAXSEG];
};

// phase cycle counters kept by block 0 when PHG_PHASE_TIMING is set
enum { T_RESID, T_VCYCLE, T_SPMV_DOT, T_DOT_SUM, T_UPDATE, T_NORM_SUM, T_GIVENS, T_CORR, T_BARRIER,
       T_BARRIERS, T_TOTAL, T_NPHASE };

__device__ __forceinline__ int ld_volatile(const int *p) { return *(const volatile int *)p; }

// Barrier over the G blocks of one group; false if the grid is aborting.
__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// The launch's barrier wait limit, held by thread 0 of every block (the only
// thread that waits): set once at kernel entry from Params::wait_limit.
__device__ __forceinline__ long long &wait_limit_slot() {
    __shared__ long long lim;
    return lim;
}

// Barriers this block has passed in the launch, held by thread 0 (set to 0 at
// kernel entry, with the wait limit).
__device__ __forceinline__ unsigned long long &bar_epoch() {
    __shared__ unsigned long long e;
    return e;
}

// Barrier of the G blocks of one group.  The group's 64-bit word at bar
// counts arrivals and is never reset within a launch (nor wraps).  Every
// block of a group passes the same sequence of barriers, so at its k-th
// barrier (k from 1) a block adds one and waits until the count reaches
// k * G: the last arrival releases everyone (no reset, no second flag), and a
// block that runs ahead into the next barrier only raises the count further.
// The arrival is a release reduction that returns nothing: the block starts
// polling at once instead of waiting a round trip to L2 for an atomic's old
// value.  The wait gives up after the launch's wait limit (wait_limit_slot,
// SPIN_LIMIT by default) and raises the launch's error flag.
__device__ bool group_sync(unsigned *bar, int G, int *err, long long *tm) {
    __shared__ int ok;
    long long tb = (tm && threadIdx.x == 0) ? clock64() : 0;
    __syncthreads();
    if (G == 1) {
        if (tm && threadIdx.x == 0) { tm[T_BARRIER] += clock64() - tb; tm[T_BARRIERS]++; }
        return ld_volatile(err) == 0;
    }
    if (threadIdx.x == 0) {
        ok = 1;
        unsigned long long *cnt = reinterpret_cast<unsigned long long *>(bar);   // 8-byte aligned
        const unsigned long long target = ++bar_epoch() * (unsigned long long)G;
        // release: the block's writes (ordered before this thread by the
        // __syncthreads above) are visible device-wide before the arrival
        asm volatile("red.release.gpu.global.add.u64 [%0], 1;" ::"l"(cnt) : "memory");
        const long long t0 = clock64(), lim = wait_limit_slot();
        while (ld_acquire(cnt) < target) {
            if (ld_volatile(err)) { ok = 0; break; }
            if (clock64() - t0 > lim) { atomicExch(err, 1); ok = 0; break; }
        }
        // acquire: the load that saw the count completes before any later
        // access of the block (the __syncthreads below orders the others)
        asm volatile("fence.acq_rel.gpu;" ::: "memory");
        if (ld_volatile(err)) ok = 0;
        if (tm) { tm[T_BARRIER] += clock64() - tb; tm[T_BARRIERS]++; }
    }
    __syncthreads();
    return ok;
}

template <typename T> __device__ __forceinline__ T ldcg(const T *p) { return __ldcg(p); }

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// maximum that keeps a NaN (fmax drops it): a non-finite residual must reach
// the host as such, never as the other operand
__device__ __forceinline__ double max_nan(double a, double b) { return a != a ? a : (b != b ? b : fmax(a, b)); }

__device__ __forceinline__ float warp_sum(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// block-reduce K (<= KMAX) per-thread values, result in red[off + l][0].
// The warps reduce in the type of the values (FP32 in the mixed path: FP64
// runs at a small fraction of the FP32 rate on this part), the NWARP warp
// sums are added in FP64.
template <int KMAX, typename T>
__device__ __forceinline__ void block_reduce(const T (&acc)[KMAX], int K, double (*red)[NWARP], int off) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int l = 0; l < KMAX; ++l) {
        if (l < K) {
            T v = warp_sum(acc[l]);
            if (lane == 0) red[off + l][warp] = (double)v;
        }
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double s = 0.0;
        for (int w = 0; w < NWARP; ++w) s += red[off + threadIdx.x][w];
        red[off + threadIdx.x][0] = s;
    }
    __syncthreads();
}

// group-wide sums of K values held in red[l][0] by every block: publish into
// one of two alternating partial buffers ([value][block] layout), barrier,
// then warp w sums value l = w, w + NWARP, ... over the G blocks
// T: the type the partials are published and summed in (FP32 for the inner
// Krylov scalars of the mixed path, FP64 otherwise)
template <typename T = double>
__device__ __forceinline__ bool group_sum(int K, double *out, double (*red)[NWARP], double *part2, int &parity,
                                          int G, int bi, unsigned *bar, int *err, long long *tm) {
    T *part = (T *)(part2 + (size_t)parity * G * (MAXM + 2));
    parity ^= 1;
    if (threadIdx.x < K) part[(size_t)threadIdx.x * G + bi] = (T)red[threadIdx.x][0];
    if (!group_sync(bar, G, err, tm)) return false;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int l = warp; l < K; l += NWARP) {
        T s = 0;
        for (int b = lane; b < G; b += 32) s += ldcg(&part[(size_t)l * G + b]);
        s = warp_sum(s);
        if (lane == 0) out[l] = (double)s;
    }
    __syncthreads();
    return true;
}

template <typename VT> struct Prec;
template <> struct Prec<double> {
    __device__ static const double *la(const MgLevelDev &l) { return l.a64; }
    __device__ static const double *ld(const MgLevelDev &l) { return l.d64; }
    __device__ static const double *lp(const MgLevelDev &l) { return l.pw64; }
    __device__ static const double *lr(const MgLevelDev &l) { return l.rw64; }
    __device__ static const double *ci(const MgDev &m) { return m.cinv64; }
};
template <> struct Prec<float> {
    __device__ static const float *la(const MgLevelDev &l) { return l.a32; }
    __device__ static const float *ld(const MgLevelDev &l) { return l.d32; }
    __device__ static const float *lp(const MgLevelDev &l) { return l.pw32; }
    __device__ static const float *lr(const MgLevelDev &l) { return l.rw32; }
    __device__ static const float *ci(const MgDev &m) { return m.cinv32; }
};

// rows [r0, r1) of a level of size n split over G blocks
__device__ __forceinline__ void own_rows(int n, int G, int bi, int &r0, int &r1) {
    const int rpb = (n + G - 1) / G;
    r0 = min(n, bi * rpb);
    r1 = min(n, r0 + rpb);
}

// sum_k A[k][i] x[col]; CG: x read through L2 (written by other blocks).
// All column/value loads of the row are issued together, then all gathers
// (one memory round trip each instead of one per entry).
template <typename VT, bool CG>
__device__ __forceinline__ VT spmv_row(const int *__restrict__ col, const VT *__restrict__ val, int n, int W,
                                       const VT *x, int i) {
    VT s = 0;
    if (W <= 8) {
        int c[8];
        VT a[8], xv[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < W) { c[k] = __ldg(&col[(size_t)k * n + i]); a[k] = __ldg(&val[(size_t)k * n + i]); }
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < W) xv[k] = CG ? ldcg(&x[c[k]]) : x[c[k]];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < W) s += a[k] * xv[k];
        return s;
    }
    for (int k = 0; k < W; ++k) {
        const size_t e = (size_t)k * n + i;
        const VT xv = CG ? ldcg(&x[__ldg(&col[e])]) : x[__ldg(&col[e])];
        s += __ldg(&val[e]) * xv;
    }
    return s;
}

// wide rows (block systems, W > 8): eight entries' loads in flight at a time
template <typename VT>
__device__ __noinline__ VT spmv_row_wide(const int *__restrict__ col, const VT *__restrict__ val, int n, int W,
                                         const VT *x, int i) {
    VT s = 0;
    for (int k0 = 0; k0 < W; k0 += 8) {
        int c[8];
        VT a[8], xv[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k0 + k < W) { c[k] = __ldg(&col[(size_t)(k0 + k) * n + i]); a[k] = __ldg(&val[(size_t)(k0 + k) * n + i]); }
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k0 + k < W) xv[k] = ldcg(&x[c[k]]);
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k0 + k < W) s += a[k] * xv[k];
    }
    return s;
}

template <typename VT, bool CG>
__device__ __forceinline__ VT restrict_row(const int *__restrict__ rf, const VT *__restrict__ rw, int Wr, int nc,
                                           const VT *r, int c) {
    VT s = 0;
    if (Wr <= 8) {
        int f[8];
        VT w[8], rv[8];
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (q < Wr) { f[q] = __ldg(&rf[(size_t)q * nc + c]); w[q] = __ldg(&rw[(size_t)q * nc + c]); }
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (q < Wr) rv[q] = f[q] >= 0 ? (CG ? ldcg(&r[f[q]]) : r[f[q]]) : (VT)0;
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (q < Wr && f[q] >= 0) s += w[q] * rv[q];
        return s;
    }
    for (int q = 0; q < Wr; ++q) {
        const int f = __ldg(&rf[(size_t)q * nc + c]);
        if (f >= 0) s += __ldg(&rw[(size_t)q * nc + c]) * (CG ? ldcg(&r[f]) : r[f]);
    }
    return s;
}

template <typename VT, bool CG>
__device__ __forceinline__ VT prolong_row(const int *__restrict__ pc, const VT *__restrict__ pw, const VT *xc,
                                          int i) {
    const int c0 = __ldg(&pc[2 * i]), c1 = __ldg(&pc[2 * i + 1]);
    const VT w0 = __ldg(&pw[2 * i]), w1 = __ldg(&pw[2 * i + 1]);
    VT s = 0;
    if (c0 >= 0) s += w0 * (CG ? ldcg(&xc[c0]) : xc[c0]);
    if (c1 >= 0) s += w1 * (CG ? ldcg(&xc[c1]) : xc[c1]);
    return s;
}

// one damped-Jacobi sweep on rows [r0, r1): xo = x + w D^-1 (b - A x)
// (first == true: x = 0, so xo = w D^-1 b)
template <typename VT, bool CG>
__device__ __forceinline__ void jacobi_rows(const MgLevelDev &L, const VT *b, const VT *x, VT *xo, VT omega,
                                            int r0, int r1, bool first) {
    const VT *A = Prec<VT>::la(L), *D = Prec<VT>::ld(L);
    const int n = L.n, W = L.W;
    const int *cl = L.col;
    for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) {
        const VT bi_ = CG ? ldcg(&b[i]) : b[i];
        const VT d = __ldg(&D[i]);
        xo[i] = first ? omega * d * bi_ : x[i] + omega * d * (bi_ - spmv_row<VT, CG>(cl, A, n, W, x, i));
    }
}

template <typename VT, bool CG>
__device__ __forceinline__ void residual_rows(const MgLevelDev &L, const VT *b, const VT *x, VT *r, int r0, int r1) {
    const VT *A = Prec<VT>::la(L);
    for (int i = r0 + threadIdx.x; i < r1; i += BLOCK)
        r[i] = (CG ? ldcg(&b[i]) : b[i]) - spmv_row<VT, CG>(L.col, A, L.n, L.W, x, i);
}

// sum_k A[k][i] fx(col): spmv_row with the gathered values computed by fx
// (same load grouping and summation order)
template <typename VT, typename F>
__device__ __forceinline__ VT spmv_row_fx(const int *__restrict__ col, const VT *__restrict__ val, int n, int W, int i,
                                          F fx) {
    VT s = 0;
    if (W <= 8) {
        int c[8];
        VT a[8], xv[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < W) { c[k] = __ldg(&col[(size_t)k * n + i]); a[k] = __ldg(&val[(size_t)k * n + i]); }
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < W) xv[k] = fx(c[k]);
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < W) s += a[k] * xv[k];
        return s;
    }
    for (int k = 0; k < W; ++k) s += __ldg(&val[(size_t)k * n + i]) * fx(__ldg(&col[(size_t)k * n + i]));
    return s;
}

// r = b - A x1 on rows [r0, r1) where x1 = w D^-1 b is the first damped-Jacobi
// sweep from zero, formed from b alone (b complete on every block): the
// residual needs no barrier after the sweep
template <typename VT>
__device__ __forceinline__ void residual_first_rows(const MgLevelDev &L, const VT *b, VT omega, VT *r, int r0, int r1) {
    const VT *A = Prec<VT>::la(L), *D = Prec<VT>::ld(L);
    for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) {
        const VT s = spmv_row_fx<VT>(L.col, A, L.n, L.W, i,
                                     [&](int c) { return omega * __ldg(&D[c]) * ldcg(&b[c]); });
        r[i] = ldcg(&b[i]) - s;
    }
}

// The redundant levels [nred, nlev) of a V-cycle, entirely in this block's
// shared memory (x, xt, b, r per level at red_off): level nred's right-hand
// side is in place; on return level nred's x holds the coarse correction.
template <typename VT>
__device__ __forceinline__ void smem_levels(const MgDev *__restrict__ mgp, VT *sm) {
    const int nred = mgp->nred, nlev = mgp->nlev, nu1 = mgp->nu1, nu2 = mgp->nu2;
    const VT omega = (VT)mgp->omega;
    const int last = nlev - 1;
    for (int l = nred; l < last; ++l) {
        const MgLevelDev &L = mgp->lev[l];
        const int n = L.n, nc = mgp->lev[l + 1].n;
        VT *x = sm + mgp->red_off[l], *xt = x + n, *b = xt + n, *r = b + n;
        jacobi_rows<VT, false>(L, b, nullptr, x, omega, 0, n, true);
        __syncthreads();
        for (int s = 1; s < nu1; ++s) {
            jacobi_rows<VT, false>(L, b, x, xt, omega, 0, n, false);
            __syncthreads();
            for (int i = threadIdx.x; i < n; i += BLOCK) x[i] = xt[i];
            __syncthreads();
        }
        residual_rows<VT, false>(L, b, x, r, 0, n);
        __syncthreads();
        VT *cb = sm + mgp->red_off[l + 1] + 2 * nc;
        const VT *rw = Prec<VT>::lr(L);
        for (int c = threadIdx.x; c < nc; c += BLOCK) cb[c] = restrict_row<VT, false>(L.rf, rw, L.Wr, nc, r, c);
        __syncthreads();
    }
    {   // coarsest: dense inverse, four independent partial sums per row
        const int n = mgp->nc;
        VT *x = sm + mgp->red_off[last], *b = x + 2 * n;
        const VT *Ci = Prec<VT>::ci(*mgp);
        for (int i = threadIdx.x; i < n; i += BLOCK) {
            VT s0 = 0, s1 = 0, s2 = 0, s3 = 0;
            int j = 0;
            for (; j + 4 <= n; j += 4) {
                const VT c0 = __ldg(&Ci[(size_t)i * n + j]), c1 = __ldg(&Ci[(size_t)i * n + j + 1]);
                const VT c2 = __ldg(&Ci[(size_t)i * n + j + 2]), c3 = __ldg(&Ci[(size_t)i * n + j + 3]);
                s0 += c0 * b[j]; s1 += c1 * b[j + 1]; s2 += c2 * b[j + 2]; s3 += c3 * b[j + 3];
            }
            for (; j < n; ++j) s0 += __ldg(&Ci[(size_t)i * n + j]) * b[j];
            x[i] = (s0 + s1) + (s2 + s3);
        }
        __syncthreads();
    }
    for (int l = last - 1; l >= nred; --l) {
        const MgLevelDev &L = mgp->lev[l];
        const int n = L.n;
        VT *x = sm + mgp->red_off[l], *xt = x + n, *b = xt + n;
        const VT *xc = sm + mgp->red_off[l + 1];
        const VT *pw = Prec<VT>::lp(L);
        for (int i = threadIdx.x; i < n; i += BLOCK) x[i] += prolong_row<VT, false>(L.pc, pw, xc, i);
        __syncthreads();
        for (int s = 0; s < nu2; ++s) {
            jacobi_rows<VT, false>(L, b, x, xt, omega, 0, n, false);
            __syncthreads();
            for (int i = threadIdx.x; i < n; i += BLOCK) x[i] = xt[i];
            __syncthreads();
        }
    }
}

// ------------------------------------------------------------ cluster tail --
// Levels [ncl, nred) of the V-cycle in the group's first cluster of cl_size
// CTAs: each level's rows are split in chunks over the CTAs, each CTA keeps its
// rows' x, xt, b, r in its own shared memory, reads neighbours' values through
// distributed shared memory (one remote load, ~250 cycles, instead of an L2
// round trip) and the CTAs synchronise with the hardware cluster barrier
// (~400 cycles) instead of the group's global-memory barrier.  The arithmetic
// and its order are those of the group-wide levels, so the correction is the
// same bit for bit.
//
// Entry is agreed through a per-group counter in global memory before any
// distributed shared memory is touched: every CTA of the cluster adds one and
// waits (bounded) for all cl_size arrivals.  A CTA that gives up marks the
// counter poisoned -- only while it is still incomplete -- so either every CTA
// of the cluster sees the count complete and runs the whole tail (whose
// control flow depends only on the level sizes: the cluster barriers always
// match and no CTA leaves while a peer may read its memory), or every CTA sees
// the poison and none enters.  A cluster barrier at the end keeps each CTA's
// memory alive until its peers are done with it.
constexpr unsigned long long CCNT_POISON = 1ull << 62;
constexpr unsigned long long CCNT_MASK = (1ull << 40) - 1;

__device__ __forceinline__ bool tail_enter(unsigned long long *ccnt, int CS, int *err) {
    __shared__ int go;
    if (threadIdx.x == 0) {
        const unsigned long long old = atomicAdd(ccnt, 1ull);
        int g = 0;
        if (!(old & CCNT_POISON)) {
            const unsigned long long target = ((old & CCNT_MASK) / CS + 1) * CS;
            const long long t0 = clock64(), lim = wait_limit_slot();
            for (;;) {
                unsigned long long v = ld_acquire(ccnt);
                if (v & CCNT_POISON) break;
                if ((v & CCNT_MASK) >= target) { g = 1; break; }
                if (clock64() - t0 > lim) {
                    // give up only while the count is incomplete
                    while (!(v & CCNT_POISON) && (v & CCNT_MASK) < target) {
                        const unsigned long long prev = atomicCAS(ccnt, v, v | CCNT_POISON);
                        if (prev == v) { v |= CCNT_POISON; break; }
                        v = prev;
                    }
                    g = (v & CCNT_POISON) ? 0 : 1;
                    if (!g) atomicExch(err, 1);
                    break;
                }
            }
        }
        go = g;
    }
    __syncthreads();
    return go != 0;
}

template <typename VT>
__device__ __noinline__ bool cluster_tail(const MgDev *__restrict__ mgp, const VT *rprev, VT *xout, VT *sm, VT *csm,
                                          unsigned long long *ccnt, int *err) {
    cg::cluster_group cl = cg::this_cluster();
    const int CS = (int)cl.num_blocks(), rank = (int)cl.block_rank();
    if (!tail_enter(ccnt, CS, err)) return false;
    const int ncl = mgp->ncl, nred = mgp->nred, nu1 = mgp->nu1, nu2 = mgp->nu2;
    const VT omega = (VT)mgp->omega;
    int cur[MG_MAXLEV];   // which of x (0) / xt (1) holds the level's iterate
    int chunk[MG_MAXLEV];
    unsigned magic[MG_MAXLEV];
    VT *lbase[MG_MAXLEV];
    for (int l = ncl; l < nred; ++l) {
        chunk[l] = mgp->cl_chunk[l];
        magic[l] = mgp->cl_magic[l];
        lbase[l] = csm + mgp->cl_off[l];
    }
    // element c of the cluster level vector whose slice in this CTA starts at
    // v (x, xt, b or r of a level with chunk ch and owner magic mg)
    auto rdv = [&](const VT *v, int ch, unsigned mg, int c) -> VT {
        const int q = (int)__umulhi((unsigned)c, mg);
        return cl.map_shared_rank(v, q)[c - q * ch];
    };
    auto rd = [&](int l, int v, int c) -> VT { return rdv(lbase[l] + (size_t)v * chunk[l], chunk[l], magic[l], c); };
    // ---- down
    for (int l = ncl; l < nred; ++l) {
        const MgLevelDev &L = mgp->lev[l];
        const int n = L.n, ch = mgp->cl_chunk[l];
        const int i0 = min(n, rank * ch), i1 = min(n, i0 + ch);
        VT *xl = csm + mgp->cl_off[l], *bl = xl + 2 * ch, *rl = xl + 3 * ch;
        const VT *A = Prec<VT>::la(L), *D = Prec<VT>::ld(L);
        if (l == ncl) {   // right-hand side: restriction of the group's residual (global)
            const MgLevelDev &F = mgp->lev[l - 1];
            const VT *rw = Prec<VT>::lr(F);
            for (int i = i0 + threadIdx.x; i < i1; i += BLOCK)
                bl[i - i0] = restrict_row<VT, true>(F.rf, rw, F.Wr, n, rprev, i);
        }
        cl.sync();   // b complete
        if (nu1 == 1) {
            // x1 = w D^-1 b and r = b - A x1 from b alone (no barrier between)
            for (int i = i0 + threadIdx.x; i < i1; i += BLOCK) {
                const VT bi_ = bl[i - i0];
                xl[i - i0] = omega * __ldg(&D[i]) * bi_;
                const VT s = spmv_row_fx<VT>(L.col, A, n, L.W, i,
                                             [&](int c) { return omega * __ldg(&D[c]) * rd(l, 2, c); });
                rl[i - i0] = bi_ - s;
            }
            cur[l] = 0;
        } else {
            for (int i = i0 + threadIdx.x; i < i1; i += BLOCK) xl[i - i0] = omega * __ldg(&D[i]) * bl[i - i0];
            int c = 0;
            for (int s = 1; s < nu1; ++s) {
                cl.sync();
                VT *xo = xl + (size_t)(1 - c) * ch;
                for (int i = i0 + threadIdx.x; i < i1; i += BLOCK)
                    xo[i - i0] = rd(l, c, i) + omega * __ldg(&D[i]) *
                                 (bl[i - i0] - spmv_row_fx<VT>(L.col, A, n, L.W, i, [&](int q) { return rd(l, c, q); }));
                c = 1 - c;
            }
            cl.sync();
            for (int i = i0 + threadIdx.x; i < i1; i += BLOCK)
                rl[i - i0] = bl[i - i0] - spmv_row_fx<VT>(L.col, A, n, L.W, i, [&](int q) { return rd(l, c, q); });
            cur[l] = c;
        }
        cl.sync();   // r complete
        const MgLevelDev &C = mgp->lev[l + 1];
        const VT *rw = Prec<VT>::lr(L);
        auto rsum = [&](int cc) {   // restrict_row with r read wherever it lives
            VT acc = 0;
            for (int q = 0; q < L.Wr; ++q) {
                const int f = __ldg(&L.rf[(size_t)q * C.n + cc]);
                if (f >= 0) acc += __ldg(&rw[(size_t)q * C.n + cc]) * rd(l, 3, f);
            }
            return acc;
        };
        if (l + 1 < nred) {
            const int chc = mgp->cl_chunk[l + 1];
            const int c0 = min(C.n, rank * chc), c1 = min(C.n, c0 + chc);
            VT *bc = csm + mgp->cl_off[l + 1] + 2 * chc;
            for (int cc = c0 + threadIdx.x; cc < c1; cc += BLOCK) bc[cc - c0] = rsum(cc);
        } else {
            VT *sb = sm + mgp->red_off[l + 1] + 2 * C.n;
            for (int cc = threadIdx.x; cc < C.n; cc += BLOCK) sb[cc] = rsum(cc);
        }
    }
    __syncthreads();
    smem_levels<VT>(mgp, sm);
    // ---- up
    for (int l = nred - 1; l >= ncl; --l) {
        const MgLevelDev &L = mgp->lev[l];
        const int n = L.n, ch = mgp->cl_chunk[l];
        const int i0 = min(n, rank * ch), i1 = min(n, i0 + ch);
        VT *xl = csm + mgp->cl_off[l], *bl = xl + 2 * ch;
        const VT *A = Prec<VT>::la(L), *D = Prec<VT>::ld(L), *pw = Prec<VT>::lp(L);
        int c = cur[l];
        VT *x = xl + (size_t)c * ch;
        if (l + 1 == nred) {
            const VT *xc = sm + mgp->red_off[l + 1];
            for (int i = i0 + threadIdx.x; i < i1; i += BLOCK) x[i - i0] += prolong_row<VT, false>(L.pc, pw, xc, i);
        } else {
            cl.sync();   // level l + 1 smoothed on every CTA
            const int cc = cur[l + 1];
            for (int i = i0 + threadIdx.x; i < i1; i += BLOCK) {
                const int q0 = __ldg(&L.pc[2 * i]), q1 = __ldg(&L.pc[2 * i + 1]);
                const VT w0 = __ldg(&pw[2 * i]), w1 = __ldg(&pw[2 * i + 1]);
                VT s = 0;
                if (q0 >= 0) s += w0 * rd(l + 1, cc, q0);
                if (q1 >= 0) s += w1 * rd(l + 1, cc, q1);
                x[i - i0] += s;
            }
        }
        for (int s = 0; s < nu2; ++s) {
            cl.sync();
            VT *xo = xl + (size_t)(1 - c) * ch;
            for (int i = i0 + threadIdx.x; i < i1; i += BLOCK)
                xo[i - i0] = rd(l, c, i) + omega * __ldg(&D[i]) *
                             (bl[i - i0] - spmv_row_fx<VT>(L.col, A, n, L.W, i, [&](int q) { return rd(l, c, q); }));
            c = 1 - c;
        }
        cur[l] = c;
        if (l == ncl) {
            const VT *xf = xl + (size_t)c * ch;
            for (int i = i0 + threadIdx.x; i < i1; i += BLOCK) xout[i] = xf[i - i0];
        }
    }
    cl.sync();   // no CTA reuses or leaves its memory while a peer may still read it
    return true;
}

// Damped-Jacobi V-cycle: x0 = M^-1 b0 for the group's right-hand side.
// Returns false if the grid is aborting.
// b0_visible: b0 is complete on every block at entry (a barrier since it was
// written), so the finest level's residual is formed without a barrier.
// csm / ccnt: this block's cluster region and the group's tail counter when
// the launch runs levels [ncl, nred) as a cluster tail (null: no tail).
template <typename VT>
__device__ __noinline__ bool vcycle(const MgDev *__restrict__ mgp, const VT *b0, VT *x0, VT *gbuf, VT *sm,
                                    unsigned *bar, int G, int bi, int *err, long long *tm, bool b0_visible,
                                    VT *csm, unsigned long long *ccnt) {
    const int nred = mgp->nred, nu1 = mgp->nu1, nu2 = mgp->nu2;
    const bool tail = ccnt != nullptr;
    const int npar = tail ? mgp->ncl : nred;   // levels run over the whole group
    const VT omega = (VT)mgp->omega;
    VT *xcur[MG_MAXLEV];
    const VT *bl[MG_MAXLEV];
    size_t offs[MG_MAXLEV];
    // ---- parallel levels, down
    size_t off = 0;
    for (int l = 0; l < npar; ++l) {
        const MgLevelDev &L = mgp->lev[l];
        const int n = L.n;
        offs[l] = off;
        VT *xa = gbuf + off, *xb = xa + n, *r = xb + n;
        VT *bn = r + n;  // rhs of level l+1 when that level is parallel too
        off += 4 * (size_t)n;
        const VT *b = l == 0 ? b0 : bl[l];
        bl[l] = b;
        int r0, r1;
        own_rows(n, G, bi, r0, r1);
        VT *x = xa, *xo = xb;
        jacobi_rows<VT, true>(L, b, nullptr, x, omega, r0, r1, true);
        // FP32 only: in FP64 the two extra multiplies per gathered entry cost
        // more than the barrier (measured at level 6)
        if (sizeof(VT) == 4 && l == 0 && b0_visible && nu1 == 1) {
            residual_first_rows<VT>(L, b, omega, r, r0, r1);
        } else {
            for (int s = 1; s < nu1; ++s) {
                if (!group_sync(bar, G, err, tm)) return false;
                jacobi_rows<VT, true>(L, b, x, xo, omega, r0, r1, false);
                VT *t = x; x = xo; xo = t;
            }
            if (!group_sync(bar, G, err, tm)) return false;
            residual_rows<VT, true>(L, b, x, r, r0, r1);
        }
        xcur[l] = x;
        if (!group_sync(bar, G, err, tm)) return false;
        const MgLevelDev &C = mgp->lev[l + 1];
        const VT *rw = Prec<VT>::lr(L);
        if (l + 1 < npar) {
            int c0, c1;
            own_rows(C.n, G, bi, c0, c1);
            for (int c = c0 + threadIdx.x; c < c1; c += BLOCK) bn[c] = restrict_row<VT, true>(L.rf, rw, L.Wr, C.n, r, c);
            bl[l + 1] = bn;
        } else if (!tail) {
            VT *sb = sm + mgp->red_off[l + 1] + 2 * C.n;
            for (int c = threadIdx.x; c < C.n; c += BLOCK) sb[c] = restrict_row<VT, true>(L.rf, rw, L.Wr, C.n, r, c);
        } else if (bi < mgp->cl_size) {
            // the group's first cluster runs the remaining levels and leaves
            // the coarse correction of level npar in the group buffer
            xcur[npar] = gbuf + off;
            if (!cluster_tail<VT>(mgp, r, gbuf + off, sm, csm, ccnt, err)) return false;
        } else {
            xcur[npar] = gbuf + off;
        }
    }
    if (!tail) {
        __syncthreads();
        smem_levels<VT>(mgp, sm);
    }
    // ---- parallel levels, up
    for (int l = npar - 1; l >= 0; --l) {
        const MgLevelDev &L = mgp->lev[l];
        const int n = L.n;
        VT *xa = gbuf + offs[l], *xb = xa + n;
        VT *x = xcur[l], *xo = (x == xa) ? xb : xa;
        const VT *b = bl[l];
        const VT *pw = Prec<VT>::lp(L);
        const bool coarse_in_smem = !tail && (l + 1 == nred);
        const VT *xc = coarse_in_smem ? sm + mgp->red_off[l + 1] : xcur[l + 1];
        if (!coarse_in_smem && !group_sync(bar, G, err, tm)) return false;
        int r0, r1;
        own_rows(n, G, bi, r0, r1);
        if (coarse_in_smem)
            for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) x[i] += prolong_row<VT, false>(L.pc, pw, xc, i);
        else
            for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) x[i] += prolong_row<VT, true>(L.pc, pw, xc, i);
        for (int s = 0; s < nu2; ++s) {
            if (!group_sync(bar, G, err, tm)) return false;
            VT *dst = (l == 0 && s == nu2 - 1) ? x0 : xo;
            jacobi_rows<VT, true>(L, b, x, dst, omega, r0, r1, false);
            if (dst == x0) x = x0;
            else { VT *t = x; x = xo; xo = t; }
        }
        if (l == 0 && x != x0)
            for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) x0[i] = x[i];
        xcur[l] = x;
    }
    return true;
}

// MULTI: the multi-operator variant (segments of right-hand sides with their
// own operators); the single-operator launches use the plain instantiation
template <typename VT, bool MULTI>
__global__ void __launch_bounds__(BLOCK, 2) gmres_kernel(const __grid_constant__ Params p) {
    extern __shared__ double smem[];
    double *H = smem;                       // (m+1) x m
    double *cs = H + (MAXM + 1) * MAXM;     // m
    double *sn = cs + MAXM;                 // m
    double *g = sn + MAXM;                  // m+1
    double *y = g + MAXM + 1;               // m
    double *hcol = y + MAXM;                // m+2 (current column / scalars)
    VT *msm = (VT *)(hcol + MAXM + 2);      // redundant multigrid levels
    __shared__ double red[MAXM + 2][NWARP];
    __shared__ int flag[4];
    // scalars computed by thread 0 and read by all (FP64 division and square
    // roots are slow on this part; one thread does them, not every thread)
    __shared__ double scal[4];
    __shared__ VT vscal[1];

    // everything the loops need, copied out of the parameter block
    const int m = p.m, max_iter = p.max_iter;
    int n = p.n;              // per right-hand side in a multi-operator launch
    size_t ld = (size_t)p.ld;
    const double tol = p.tol;
    // this block's group: groups of p.G blocks over the launch, or, in a
    // multi-operator launch, groups sized for this block's segment (its mesh)
    // that take that segment's right-hand sides only
    int G = p.G, grp = blockIdx.x / G, bi = blockIdx.x % G;
    int vbeg = grp, vend = p.nv, vstep = p.groups;
    if (MULTI) {
        int k = 0;
        while (k + 1 < p.nseg && (int)blockIdx.x >= p.seg[k + 1].blk0) ++k;
        const int lb = (int)blockIdx.x - p.seg[k].blk0;
        G = p.seg[k].G;
        const int lg = lb / G;
        bi = lb % G;
        if (lg >= p.seg[k].groups) return;
        grp = p.seg[k].gbase + lg;
        vbeg = p.seg[k].v0 + lg;
        vend = p.seg[k].v0 + p.seg[k].nv;
        vstep = p.seg[k].groups;
    } else if (grp >= p.groups) {
        return;
    }
    if (threadIdx.x == 0) {   // read by this thread only
        wait_limit_slot() = p.wait_limit;
        bar_epoch() = 0;
    }
    unsigned *bar = p.bar + 2 * grp;
    int *err = p.err;
    // the group's partial sums: 2 (MAXM + 2) doubles per block from its first block
    double *part2 = p.part + (size_t)(blockIdx.x - bi) * 2 * (MAXM + 2);
    int parity = 0;
    int r0, r1;
    own_rows(n, G, bi, r0, r1);
    int W = p.op.A.W;
    const int *__restrict__ col = p.op.A.col;
    const double *__restrict__ aval = p.op.A.val;
    const MgDev *mgp = MULTI ? p.seg[0].mgd : p.op.mgd;
    const bool use_mg = mgp != nullptr;   // every segment of a multi-operator launch is multigrid
    const VT *__restrict__ sval;
    if (sizeof(VT) == 8) sval = (const VT *)(use_mg ? (const void *)p.op.A.val : (const void *)p.op.as64);
    else sval = (const VT *)(use_mg ? (const void *)p.op.a32 : (const void *)p.op.as32);
    const double *__restrict__ dinv = p.op.dinv;
    VT *gbuf = use_mg ? (VT *)p.mgbuf + (size_t)grp * p.group_elems : nullptr;
    const int block4 = p.op.block4;
    const int rsb = block4 ? n / 4 : 0;          // vertices of a block system
    // block preconditioner: the second V-cycle gets its own level scratch so
    // that it can start while other blocks still read the first one's
    VT *gbuf2 = (gbuf && block4) ? gbuf + p.op.mg.group_elems : nullptr;
    // cluster tail: this block's region after the redundant levels, and the group's entry counter
    VT *csm = p.cluster ? msm + p.op.mg.red_elems : nullptr;
    unsigned long long *tcnt = p.cluster ? p.ccnt + grp : nullptr;
    VT *bt3 = gbuf2 ? gbuf2 + p.op.mg.group_elems : nullptr;
    VT *bt4 = bt3 ? bt3 + rsb : nullptr, *bu3 = bt4 ? bt4 + rsb : nullptr, *bu4 = bu3 ? bu3 + rsb : nullptr;
    const int *cpl_col = p.op.cpl.col;
    const VT *cpl_val = (const VT *)(sizeof(VT) == 8 ? (const void *)p.op.cpl.val : (const void *)p.op.cpl32);
    const int cpl_W = p.op.cpl.W;
    long long *tm = (p.timers && blockIdx.x == 0) ? p.timers : nullptr;
    const double *Bp = p.B;
    double *Xp = p.X;
    VT *Vp = (VT *)p.V, *Zp = (VT *)p.Z, *Wp = (VT *)p.Wv;
    double *Rp = p.R;
    const double inner_rtol = sizeof(VT) == 4 ? p.inner_rtol : 0.0;
    const double es = (double)sizeof(VT);
    double nrows = (double)(r1 - r0);
    double mg_row_bytes = p.mg_row_bytes;
    long long t_start = clock64(), tph = 0;
#define PHG_TICK(ph)                                                         \
    do {                                                                     \
        if (tm && threadIdx.x == 0) { long long t_ = clock64(); tm[ph] += t_ - tph; tph = t_; } \
    } while (0)

    int my_iters = 0, my_cycles = 0, my_status = 0, my_steps = 0;
    double my_rel = 0.0;
    // algorithmic bytes per owned row (minimal traffic, no re-reads):
    //   residual   W (col 4 B + val 8 B) + gathered x 8 + b 8 + r 8
    //   Arnoldi j  W (col 4 + val es) + gathered z_j es + w es (write)
    //              + (j+1) es (V reads, dots) + (j+1) es (V reads, update)
    //              + 2 es (w read/write) + 2 es (w read, v_{j+1} write)
    //   V-cycle    per level and sweep: W (4 + es) + 4 es, plus transfers
    //   correction jlast es (V or Z reads) + 16 (x read/write) + 8
    double my_bytes = 0.0;

    for (int v = vbeg; v < vend; v += vstep) {
        const double *__restrict__ b = Bp + (size_t)v * ld;
        double *x = Xp + (size_t)v * ld;
        VT *V = Vp + (size_t)v * (m + 1) * n;
        VT *Z = use_mg ? Zp + (size_t)v * m * n : nullptr;
        VT *w = Wp + (size_t)v * n;
        double *R = Rp + (size_t)v * n;
        if (MULTI) {   // the operator, rows and vectors of this right-hand side's segment
            int k = 0;
            while (k + 1 < p.nseg && v >= p.seg[k + 1].v0) ++k;
            const MultiSeg &S = p.seg[k];
            const int lv = v - S.v0;
            n = S.n; W = S.W; ld = (size_t)S.ld;
            col = S.col; aval = S.aval; dinv = S.dinv; mgp = S.mgd;
            sval = (const VT *)(sizeof(VT) == 8 ? (const void *)S.sval64 : (const void *)S.sval32);
            mg_row_bytes = S.mg_row_bytes;
            own_rows(n, G, bi, r0, r1);
            nrows = (double)(r1 - r0);
            b = S.B + (size_t)lv * ld;
            x = S.X + (size_t)lv * ld;
            V = Vp + S.voff + (size_t)lv * (m + 1) * n;
            Z = Zp + S.zoff + (size_t)lv * m * n;
            w = Wp + S.woff + (size_t)lv * n;
            R = Rp + S.roff + (size_t)lv * n;
        }

        double acc[1];
        {
            double s = 0.0;
            for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) { const double t = b[i]; s += t * t; }
            acc[0] = s;
        }
        block_reduce<1>(acc, 1, red, 0);
        if (!group_sum(1, hcol, red, part2, parity, G, bi, bar, err, tm)) return;
        if (threadIdx.x == 0) scal[0] = sqrt(hcol[0]);
        __syncthreads();
        const double bnorm = scal[0];
        int iters = 0, cycles = 0, status = 1;
        double beta_prev = 0.0, rel = 0.0;
        if (bnorm == 0.0) {
            for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) x[i] = 0.0;
            status = 0; rel = 0.0;
            if (!group_sync(bar, G, err, tm)) return;
        }
        while (bnorm != 0.0) {
            // r = b - A x (FP64, exact operator); needs all of x
            if (!group_sync(bar, G, err, tm)) return;
            if (tm && threadIdx.x == 0) tph = clock64();
            {
                double s = 0.0;
                for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) {
                    const double q = b[i] - (W <= 8 ? spmv_row<double, true>(col, aval, n, W, x, i)
                                                    : spmv_row_wide<double>(col, aval, n, W, x, i));
                    R[i] = q;
                    s += q * q;
                }
                acc[0] = s;
            }
            block_reduce<1>(acc, 1, red, 0);
            if (!group_sum(1, hcol, red, part2, parity, G, bi, bar, err, tm)) return;
            if (threadIdx.x == 0) {
                const double bt = sqrt(hcol[0]);
                scal[1] = bt;
                scal[2] = bt / bnorm;
                scal[3] = bt > 0.0 ? 1.0 / bt : 0.0;
            }
            __syncthreads();
            const double beta = scal[1];
            PHG_TICK(T_RESID);
            my_bytes += nrows * (W * 12.0 + 24.0);
            rel = scal[2];
            if (rel <= tol) { status = 0; break; }
            if (iters >= max_iter) { status = 1; break; }
            if (cycles > 0 && !(beta < 0.9999 * beta_prev)) { status = 1; break; }
            beta_prev = beta;
            ++cycles;
            const double target = threadIdx.x == 0 ? fmax(tol * bnorm, inner_rtol * beta) : 0.0;
            {
                const double ib = scal[3];
                for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) V[i] = (VT)(R[i] * ib);
            }
            if (threadIdx.x == 0) {
                g[0] = beta;
                for (int l = 1; l <= m; ++l) g[l] = 0.0;
            }
            int jlast = 0;
            for (int j = 0; j < m; ++j) {
                if (!group_sync(bar, G, err, tm)) return;   // v_j complete
                if (tm && threadIdx.x == 0) tph = clock64();
                const VT *vj = V + (size_t)j * n;
                const VT *zj = vj;
                if (use_mg && block4) {
                    // z_w = D^-1 v_w ; t = v_u - M z_w ; z_u = -Vcycle(t)
                    VT *zz = Z + (size_t)j * n;
                    for (int i = r0 + threadIdx.x; i < r1; i += BLOCK)
                        if ((i & 3) < 2) zz[i] = (VT)(dinv[i] * (double)vj[i]);
                    if (!group_sync(bar, G, err, tm)) return;
                    int k0, k1;
                    own_rows(rsb, G, bi, k0, k1);
                    for (int k = k0 + threadIdx.x; k < k1; k += BLOCK) {
                        VT s3 = 0, s4 = 0;
                        for (int e = 0; e < cpl_W; ++e) {
                            const int c = __ldg(&cpl_col[(size_t)e * rsb + k]);
                            const VT a = __ldg(&cpl_val[(size_t)e * rsb + k]);
                            s3 += a * ldcg(&zz[4 * c]);
                            s4 += a * ldcg(&zz[4 * c + 1]);
                        }
                        bt3[k] = ldcg(&vj[4 * k + 2]) - s3;
                        bt4[k] = ldcg(&vj[4 * k + 3]) - s4;
                    }
                    if (!vcycle<VT>(mgp, bt3, bu3, gbuf, msm, bar, G, bi, err, tm, false, csm, tcnt)) return;
                    if (!vcycle<VT>(mgp, bt4, bu4, gbuf2, msm, bar, G, bi, err, tm, false, csm, tcnt)) return;
                    if (!group_sync(bar, G, err, tm)) return;
                    for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) {
                        const int q = i & 3;
                        if (q >= 2) zz[i] = -ldcg(q == 2 ? &bu3[i >> 2] : &bu4[i >> 2]);
                    }
                    if (!group_sync(bar, G, err, tm)) return;   // z_j complete
                    PHG_TICK(T_VCYCLE);
                    zj = zz;
                    my_bytes += nrows * mg_row_bytes;
                } else if (use_mg) {
                    VT *zz = Z + (size_t)j * n;
                    if (!vcycle<VT>(mgp, vj, zz, gbuf, msm, bar, G, bi, err, tm, true, csm, tcnt)) return;
                    if (!group_sync(bar, G, err, tm)) return;   // z_j complete
                    PHG_TICK(T_VCYCLE);
                    zj = zz;
                    my_bytes += nrows * mg_row_bytes;
                }
                // (1) w = A z_j (Jacobi: (A D^-1) v_j); each row issues all
                // its loads at once
                for (int i = r0 + threadIdx.x; i < r1; i += BLOCK)
                    w[i] = W <= 8 ? spmv_row<VT, true>(col, sval, n, W, zj, i) : spmv_row_wide<VT>(col, sval, n, W, zj, i);
                // dots with v_0..v_j, eight basis vectors per pass; per-thread
                // sums in the Krylov precision (FP32 in the mixed path: GB300's
                // FP64 rate is a small fraction of FP32), FP64 across threads
                for (int l0 = 0; l0 <= j; l0 += 8) {
                    VT t0 = 0, t1 = 0, t2 = 0, t3 = 0, t4 = 0, t5 = 0, t6 = 0, t7 = 0;
                    const int kk = min(8, j + 1 - l0);
                    const VT *Vl = V + (size_t)l0 * n;
                    for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) {
                        const VT s = w[i];
                        const VT q0 = Vl[i];
                        const VT q1 = kk > 1 ? Vl[(size_t)n + i] : (VT)0;
                        const VT q2 = kk > 2 ? Vl[(size_t)2 * n + i] : (VT)0;
                        const VT q3 = kk > 3 ? Vl[(size_t)3 * n + i] : (VT)0;
                        const VT q4 = kk > 4 ? Vl[(size_t)4 * n + i] : (VT)0;
                        const VT q5 = kk > 5 ? Vl[(size_t)5 * n + i] : (VT)0;
                        const VT q6 = kk > 6 ? Vl[(size_t)6 * n + i] : (VT)0;
                        const VT q7 = kk > 7 ? Vl[(size_t)7 * n + i] : (VT)0;
                        t0 += q0 * s; t1 += q1 * s; t2 += q2 * s; t3 += q3 * s;
                        t4 += q4 * s; t5 += q5 * s; t6 += q6 * s; t7 += q7 * s;
                    }
                    const VT a8[8] = {t0, t1, t2, t3, t4, t5, t6, t7};
                    block_reduce<8>(a8, kk, red, l0);
                }
                PHG_TICK(T_SPMV_DOT);
                if (!group_sum<VT>(j + 1, hcol, red, part2, parity, G, bi, bar, err, tm)) return;
                PHG_TICK(T_DOT_SUM);
                // (2) w -= sum h_l v_l, ||w||^2; the coefficients converted to
                // the Krylov precision once (y is free until the cycle ends)
                VT *hv = (VT *)y;
                if (threadIdx.x <= j) hv[threadIdx.x] = (VT)hcol[threadIdx.x];
                __syncthreads();
                {
                    VT a2 = 0;
                    for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) {
                        VT s = w[i];
                        for (int l0 = 0; l0 <= j; l0 += 8) {
                            const int kk = min(8, j + 1 - l0);
                            const VT *Vl = V + (size_t)l0 * n;
                            const VT q0 = Vl[i];
                            const VT q1 = kk > 1 ? Vl[(size_t)n + i] : (VT)0;
                            const VT q2 = kk > 2 ? Vl[(size_t)2 * n + i] : (VT)0;
                            const VT q3 = kk > 3 ? Vl[(size_t)3 * n + i] : (VT)0;
                            const VT q4 = kk > 4 ? Vl[(size_t)4 * n + i] : (VT)0;
                            const VT q5 = kk > 5 ? Vl[(size_t)5 * n + i] : (VT)0;
                            const VT q6 = kk > 6 ? Vl[(size_t)6 * n + i] : (VT)0;
                            const VT q7 = kk > 7 ? Vl[(size_t)7 * n + i] : (VT)0;
                            s -= hv[l0] * q0;
                            if (kk > 1) s -= hv[l0 + 1] * q1;
                            if (kk > 2) s -= hv[l0 + 2] * q2;
                            if (kk > 3) s -= hv[l0 + 3] * q3;
                            if (kk > 4) s -= hv[l0 + 4] * q4;
                            if (kk > 5) s -= hv[l0 + 5] * q5;
                            if (kk > 6) s -= hv[l0 + 6] * q6;
                            if (kk > 7) s -= hv[l0 + 7] * q7;
                        }
                        w[i] = s;
                        a2 += s * s;
                    }
                    const VT a1[1] = {a2};
                    block_reduce<1>(a1, 1, red, 0);
                }
                PHG_TICK(T_UPDATE);
                if (!group_sum<VT>(1, hcol + j + 1, red, part2, parity, G, bi, bar, err, tm)) return;
                PHG_TICK(T_NORM_SUM);
                // (3) thread 0: ||w||, the rotations and the stopping test;
                // then every thread scales w into v_{j+1}
                if (threadIdx.x == 0) {
                    const double hn = sqrt(hcol[j + 1]);
                    vscal[0] = hn > 0.0 ? (VT)(1.0 / hn) : (VT)0;
                    hcol[j + 1] = hn;
                    for (int l = 0; l < j; ++l) {
                        double a = hcol[l], c = hcol[l + 1];
                        hcol[l] = cs[l] * a + sn[l] * c;
                        hcol[l + 1] = -sn[l] * a + cs[l] * c;
                    }
                    double a = hcol[j], c = hcol[j + 1];
                    double r = hypot(a, c);
                    cs[j] = r > 0.0 ? a / r : 1.0;
                    sn[j] = r > 0.0 ? c / r : 0.0;
                    for (int l = 0; l < j; ++l) H[l * MAXM + j] = hcol[l];
                    H[j * MAXM + j] = r;
                    g[j + 1] = -sn[j] * g[j];
                    g[j] = cs[j] * g[j];
                    flag[0] = (fabs(g[j + 1]) <= target) || hn == 0.0;
                }
                __syncthreads();
                {
                    const VT inv = vscal[0];
                    VT *vn = V + (size_t)(j + 1) * n;
                    if (inv != (VT)0)
                        for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) vn[i] = w[i] * inv;
                }
                PHG_TICK(T_GIVENS);
                ++iters;
                ++my_steps;
                my_bytes += nrows * (W * (4.0 + es) + es * (2.0 * (j + 1) + 6.0));
                jlast = j + 1;
                if (flag[0] || iters >= max_iter) break;
            }
            // y = H^-1 g; x += D^-1 V y (Jacobi) or Z y (multigrid)
            // The correction sum_l y_l z_l is formed in the Krylov precision
            // (in the mixed path it only has to be as accurate as the FP32
            // inner solve) and added to the FP64 iterate once.
            VT *yv = (VT *)cs;   // the rotations are not needed any more
            if (threadIdx.x == 0) {
                for (int l = jlast - 1; l >= 0; --l) {
                    double s = g[l];
                    for (int k = l + 1; k < jlast; ++k) s -= H[l * MAXM + k] * y[k];
                    y[l] = s / H[l * MAXM + l];
                }
                for (int l = 0; l < jlast; ++l) yv[l] = (VT)y[l];
            }
            __syncthreads();
            {
                const VT *Bb = use_mg ? Z : V;
                for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) {
                    VT s = 0;
                    for (int l = 0; l < jlast; ++l) s += yv[l] * Bb[(size_t)l * n + i];
                    x[i] += use_mg ? (double)s : dinv[i] * (double)s;
                }
            }
            my_bytes += nrows * (jlast * es + 24.0);
            PHG_TICK(T_CORR);
        }
        my_iters = max(my_iters, iters);
        my_cycles = max(my_cycles, cycles);
        my_rel = max_nan(my_rel, rel);
        my_status = max(my_status, status);
    }
#undef PHG_TICK
    if (tm && threadIdx.x == 0) tm[T_TOTAL] += clock64() - t_start;
    if (threadIdx.x == 0) atomicAdd(&p.stats->bytes, my_bytes);
    if (threadIdx.x == 0 && bi == 0) {
        atomicAdd(&p.stats->steps_total, my_steps);
        atomicMax(&p.stats->iters, my_iters);
        atomicMax(&p.stats->cycles, my_cycles);
        atomicMax(&p.stats->status, my_status);
        // relres >= 0: max via the integer order of non-negative doubles
        atomicMax((unsigned long long *)&p.stats->relres, (unsigned long long)__double_as_longlong(my_rel));
    }
}

// Chebyshev iteration (Saad, Iterative Methods for Sparse Linear Systems,
// 2nd ed., Alg. 12.1, Jacobi-preconditioned) inside the same FP64 iterative
// refinement as the GMRES kernel: per cycle r = b - A x in FP64, then
// cheb_k steps on A e = r / ||r|| in the Krylov precision, x += ||r|| e.
// For operators whose Jacobi-scaled spectrum is known to lie in a small real
// interval (mass matrices) this needs no inner products: one SpMV and one
// group barrier per step.  Work vectors (in the V region): rv, d, e0, e1.
template <typename VT>
__global__ void __launch_bounds__(BLOCK, 2) cheb_kernel(const Params p) {
    extern __shared__ double smem[];
    double *hcol = smem;
    VT *cf = (VT *)(smem + 4);              // ca[k], cb[k] in the Krylov precision
    __shared__ double red[MAXM + 2][NWARP];
    __shared__ double scal[4];
    __shared__ int kcyc;
    const int n = p.n, G = p.G, nv = p.nv, groups = p.groups, max_iter = p.max_iter, K = p.cheb_k;
    const size_t ld = (size_t)p.ld;
    const double tol = p.tol;
    const int grp = blockIdx.x / G, bi = blockIdx.x % G;
    if (grp >= groups) return;
    if (threadIdx.x == 0) {   // constant indices: the parameter block stays in param space
        wait_limit_slot() = p.wait_limit;
        bar_epoch() = 0;
#pragma unroll
        for (int k = 0; k < CHEB_KMAX; ++k) {
            cf[k] = (VT)p.cheb_ca[k];
            cf[CHEB_KMAX + k] = (VT)p.cheb_cb[k];
        }
    }
    __syncthreads();
    const VT c0 = (VT)p.cheb_c0;
    unsigned *bar = p.bar + 2 * grp;
    int *err = p.err;
    double *part2 = p.part + (size_t)grp * 2 * G * (MAXM + 2);
    int parity = 0;
    int r0, r1;
    own_rows(n, G, bi, r0, r1);
    const int W = p.op.A.W;
    const int *__restrict__ col = p.op.A.col;
    const double *__restrict__ aval = p.op.A.val;
    const VT *__restrict__ sval = sizeof(VT) == 8 ? (const VT *)(const void *)p.op.A.val
                                                   : (const VT *)(const void *)p.op.a32;
    const VT *__restrict__ dv = sizeof(VT) == 8 ? (const VT *)(const void *)p.op.dinv
                                                 : (const VT *)(const void *)p.op.dinv32;
    const double *Bp = p.B;
    double *Xp = p.X;
    VT *Vp = (VT *)p.V;
    double *Rp = p.R;
    const double inner_rtol = sizeof(VT) == 4 ? p.inner_rtol : 0.0;
    const double es = (double)sizeof(VT), nrows = (double)(r1 - r0);
    int my_iters = 0, my_cycles = 0, my_status = 0, my_steps = 0;
    double my_rel = 0.0, my_bytes = 0.0;
    (void)inner_rtol;

    for (int v = grp; v < nv; v += groups) {
        const double *__restrict__ b = Bp + (size_t)v * ld;
        double *x = Xp + (size_t)v * ld;
        VT *rv = Vp + (size_t)v * p.vstride;
        VT *d = rv + n, *e0 = d + n, *e1 = e0 + n;
        double *R = Rp + (size_t)v * n;
        {
            double s = 0.0;
            for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) { const double t = b[i]; s += t * t; }
            const double a1[1] = {s};
            block_reduce<1>(a1, 1, red, 0);
        }
        if (!group_sum(1, hcol, red, part2, parity, G, bi, bar, err, nullptr)) return;
        if (threadIdx.x == 0) scal[0] = sqrt(hcol[0]);
        __syncthreads();
        const double bnorm = scal[0];
        int iters = 0, cycles = 0, status = 1;
        double beta_prev = 0.0, rel = 0.0;
        if (bnorm == 0.0) {
            for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) x[i] = 0.0;
            status = 0;
        }
        while (bnorm != 0.0) {
            if (!group_sync(bar, G, err, nullptr)) return;   // x complete
            {
                double s = 0.0;
                for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) {
                    const double q = b[i] - spmv_row<double, true>(col, aval, n, W, x, i);
                    R[i] = q;
                    s += q * q;
                }
                const double a1[1] = {s};
                block_reduce<1>(a1, 1, red, 0);
            }
            if (!group_sum(1, hcol, red, part2, parity, G, bi, bar, err, nullptr)) return;
            if (threadIdx.x == 0) {
                const double bt = sqrt(hcol[0]);
                scal[1] = bt;
                scal[2] = bt / bnorm;
                scal[3] = bt > 0.0 ? 1.0 / bt : 0.0;
                // this cycle's steps: K, or fewer when the reduction still
                // needed (tol / rel, with a factor 2 margin) is smaller than
                // the one K steps guarantee
                int kc = K;
                const double rl = bt / bnorm;
                if (rl > tol && p.cheb_ls > 0.0) {
                    const double need = (p.cheb_lg + log(2.0 * rl / tol)) / p.cheb_ls;
                    if (need + 1.0 < (double)K) kc = max(2, (int)ceil(need) + 1);
                }
                kcyc = kc;
            }
            __syncthreads();
            const double beta = scal[1];
            const int Kc = kcyc;
            my_bytes += nrows * (W * 12.0 + 24.0);
            rel = scal[2];
            if (rel <= tol) { status = 0; break; }
            if (iters >= max_iter) { status = 1; break; }
            if (cycles > 0 && !(beta < 0.9999 * beta_prev)) { status = 1; break; }
            beta_prev = beta;
            ++cycles;
            // e_1 = d_0 = c0 D^-1 r / beta
            {
                const double ib = scal[3];
                for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) {
                    const VT r = (VT)(R[i] * ib);
                    const VT dd = c0 * dv[i] * r;
                    rv[i] = r;
                    d[i] = dd;
                    e0[i] = dd;
                }
            }
            VT *ec = e0, *en = e1;
            for (int k = 1; k < Kc; ++k) {
                if (!group_sync(bar, G, err, nullptr)) return;   // e_k complete
                const VT ca = cf[k], cb = cf[CHEB_KMAX + k];
                for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) {
                    const VT s = spmv_row<VT, true>(col, sval, n, W, ec, i);
                    const VT dd = ca * d[i] + cb * dv[i] * (rv[i] - s);
                    d[i] = dd;
                    en[i] = ec[i] + dd;
                }
                VT *t = ec; ec = en; en = t;
                ++iters;
                ++my_steps;
                my_bytes += nrows * (W * (4.0 + es) + 7.0 * es);
            }
            ++iters;
            for (int i = r0 + threadIdx.x; i < r1; i += BLOCK) x[i] += beta * (double)ec[i];
            my_bytes += nrows * (es + 16.0);
        }
        my_iters = max(my_iters, iters);
        my_cycles = max(my_cycles, cycles);
        my_rel = max_nan(my_rel, rel);
        my_status = max(my_status, status);
    }
    if (threadIdx.x == 0) atomicAdd(&p.stats->bytes, my_bytes);
    if (threadIdx.x == 0 && bi == 0) {
        atomicAdd(&p.stats->steps_total, my_steps);
        atomicMax(&p.stats->iters, my_iters);
        atomicMax(&p.stats->cycles, my_cycles);
        atomicMax(&p.stats->status, my_status);
        atomicMax((unsigned long long *)&p.stats->relres, (unsigned long long)__double_as_longlong(my_rel));
    }
}

__global__ void fold_err(const int *err, GmresStats *st) {
    if (*err) st->status = 2;
}

size_t smem_gmres_bytes() { return sizeof(double) * ((MAXM + 1) * MAXM + 2 * MAXM + (MAXM + 1) + MAXM + (MAXM + 2)); }

constexpr int GROUPS_CAP = 4096;

struct Layout { size_t v, z, w, r, mg, part, bar, err, ccnt, total; };

// per-group multigrid scratch: one V-cycle's levels, or two V-cycles' levels
// and the 4 vertex vectors of the block preconditioner
size_t block_group_elems(const DevSolveOp &op) {
    if (!op.block4) return op.mg.group_elems;
    return 2 * op.mg.group_elems + 4 * (size_t)(op.A.n / 4);
}

// whether gmres_solve runs op's solves as Chebyshev iterations (the same test)
bool uses_cheb(const DevSolveOp &op, int m) {
    return op.cheb_lmax > 0.0 && op.cheb_lmin > 0.0 && op.cheb_lmin < op.cheb_lmax && m >= 3 && !op.mgd &&
           !op.block4 && op.A.W <= 8;
}

Layout layout(const DevSolveOp &op, int nv, int m, Precision prec) {
    Layout L;
    const int n = op.A.n;
    size_t es = prec == PREC_MIXED ? 4 : 8;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    const bool mg = op.mgd != nullptr;
    // per right-hand side: the m + 1 Krylov vectors of GMRES, or the four
    // vectors of a Chebyshev solve (rv, d, e_k, e_k+1); the lockstep Chebyshev
    // path needs three interleaved FP32 vectors and the norm partials instead
    size_t vregion = es * (size_t)nv * (m + 1) * n;
    if (uses_cheb(op, m)) {
        vregion = es * (size_t)nv * 4 * n;
        if (prec == PREC_MIXED) {
            const size_t nvp = (size_t)(nv + 31) / 32 * 32, nbx = ((size_t)n + 255) / 256;
            vregion = std::max(vregion, 3 * al(4 * (size_t)n * nvp) + 16 * (size_t)nv * nbx);
        }
    }
    L.v = 0;
    L.z = L.v + al(vregion);
    L.w = L.z + (mg ? al(es * (size_t)nv * m * n) : 0);
    L.r = L.w + al(es * (size_t)nv * n);
    L.mg = L.r + al(8 * (size_t)nv * n);
    const int groups = nv < GROUPS_CAP ? nv : GROUPS_CAP;
    const size_t ge = block_group_elems(op);
    L.part = L.mg + (mg ? al(es * ge * (size_t)groups) : 0);
    // groups * G <= co-resident blocks (< 4096)
    L.bar = L.part + al(8 * (size_t)4096 * 2 * (MAXM + 2));
    L.err = L.bar + al(8 * (size_t)GROUPS_CAP);
    L.ccnt = L.err + 256;
    L.total = L.ccnt + al(8 * (size_t)GROUPS_CAP);
    return L;
}

// ------------------------------------------------- lockstep Chebyshev ---
// Many right-hand sides of one mass-like operator (the Jacobian's 8 x members
// solves of an ensemble step) in lockstep: the FP32 Chebyshev vectors are
// kept interleaved (row i holds the nvp members contiguously), so every step
// is one pass of an SpMM that reads each matrix row once for all members and
// gathers whole 16-byte member chunks, fused with the recurrence update.
// The FP64 residual, the norms and the stopping test run between cycles in
// separate launches; a device flag ends the remaining launches once every
// member has converged (no host synchronisation).
constexpr int LS_MAXC = 6;     // refinement cycles at most
constexpr int LS_MG = 16;      // members per thread in the FP64 residual

// R = B - A X for LS_MG members per 256-row block (FP64, ascending slot
// order), and each member's sum of R^2 over the block's rows into
// part[v][row block] (fixed order: the norms are reproducible).  Grid-stride
// over (row block, member group) tiles, at most one resident wave of blocks:
// a launch after convergence then costs one short wave.
template <int W>
__global__ void __launch_bounds__(256) k_ls_resid(const int *__restrict__ col, const double *__restrict__ val, int n,
                                                  const double *__restrict__ B, const double *__restrict__ X, int ld,
                                                  double *__restrict__ R, int nv, double *__restrict__ part, int nbx,
                                                  const int *done) {
    if (*(volatile const int *)done) return;
    __shared__ double sq[LS_MG][256];
    const int ntile = nbx * ((nv + LS_MG - 1) / LS_MG);
    for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
        const int rb = tile % nbx, i = rb * 256 + threadIdx.x;
        const bool row = i < n;
        const int v0 = (tile / nbx) * LS_MG, v1 = min(nv, v0 + LS_MG);
        int c[W];
        double a[W];
#pragma unroll
        for (int k = 0; k < W; ++k) {
            c[k] = row ? __ldg(&col[(size_t)k * n + i]) : 0;
            a[k] = row ? __ldg(&val[(size_t)k * n + i]) : 0.0;
        }
        for (int v = v0; v < v1; ++v) {
            double r = 0.0;
            if (row) {
                const double *x = X + (size_t)v * ld;
                double sum = 0.0;
#pragma unroll
                for (int k = 0; k < W; ++k) sum += a[k] * x[c[k]];
                r = B[(size_t)v * ld + i] - sum;
                R[(size_t)v * n + i] = r;
            }
            sq[v - v0][threadIdx.x] = r * r;
        }
        __syncthreads();
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        for (int j = warp; j < v1 - v0; j += NWARP) {
            double t = 0.0;
            for (int q = lane; q < 256; q += 32) t += sq[j][q];
            t = warp_sum(t);
            if (lane == 0) part[(size_t)(v0 + j) * nbx + rb] = t;
        }
        __syncthreads();   // sq is refilled by the next tile
    }
}

// each member's sum of A^2 over block rows into part[v][block] (as k_ls_resid)
__global__ void __launch_bounds__(256) k_ls_sq(const double *__restrict__ A, int n, int ld, int nv,
                                               double *__restrict__ part) {
    __shared__ double sq[LS_MG][256];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int v0 = blockIdx.y * LS_MG, v1 = min(nv, v0 + LS_MG);
    for (int v = v0; v < v1; ++v) {
        const double x = i < n ? A[(size_t)v * ld + i] : 0.0;
        sq[v - v0][threadIdx.x] = x * x;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int j = warp; j < v1 - v0; j += NWARP) {
        double t = 0.0;
        for (int q = lane; q < 256; q += 32) t += sq[j][q];
        t = warp_sum(t);
        if (lane == 0) part[(size_t)(v0 + j) * gridDim.x + blockIdx.x] = t;
    }
}

// ||r||^2 and ||b||^2 of every member: the sums of its nbx block partials
// (one warp per member, fixed order)
__global__ void __launch_bounds__(256) k_ls_nrm(const double *rpart, const double *bpart, int nbx, double *nrm,
                                                int nv, const int *done) {
    if (*(volatile const int *)done) return;
    const int v = blockIdx.x * NWARP + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (v >= nv) return;
    double tr = 0.0, tb = 0.0;
    for (int q = lane; q < nbx; q += 32) {
        tr += rpart[(size_t)v * nbx + q];
        tb += bpart[(size_t)v * nbx + q];
    }
    tr = warp_sum(tr);
    tb = warp_sum(tb);
    if (lane == 0) { nrm[2 * v] = tr; nrm[2 * v + 1] = tb; }
}

// per-member scales 1/||r|| (0 once converged), the stopping test and the stats
// The cycle's steps (*kc): K, or fewer when every open member needs a smaller
// reduction (tol / rel, factor 2 margin; steps for a reduction eps:
// ceil((lg - log eps) / ls) + 1), rounded up to K's parity so that the
// iterate ends in the buffer the K-step sequence ends in.
__global__ void __launch_bounds__(256) k_ls_scale(const double *nrm, int nv, int nvp, double tol, double *beta,
                                                  double *sc, int *done, GmresStats *st, int cycle, int K,
                                                  double bytes, double lg, double ls, int *kc) {
    if (*(volatile int *)done) return;
    __shared__ double rmax[NWARP];
    __shared__ int open[NWARP], kneed[NWARP];
    double mx = 0.0;
    int op = 0, kn = 2;
    for (int v = threadIdx.x; v < nvp; v += blockDim.x) {
        if (v >= nv) { sc[v] = 0.0; beta[v] = 0.0; continue; }
        const double bt = sqrt(nrm[2 * v]), bn = sqrt(nrm[2 * v + 1]);
        const double rel = bn > 0.0 ? bt / bn : 0.0;
        const bool conv = rel <= tol || bt == 0.0;
        beta[v] = bt;
        sc[v] = conv ? 0.0 : 1.0 / bt;
        mx = max_nan(mx, rel);
        if (!(rel == rel)) mx = rel;   // NaN propagates into the stats
        op += conv ? 0 : 1;
        if (!conv) {
            const double need = ls > 0.0 ? (lg + log(2.0 * rel / tol)) / ls : (double)K;
            kn = need + 1.0 < (double)K ? max(kn, (int)ceil(need) + 1) : K;   // NaN: K
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        mx = max_nan(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        op += __shfl_xor_sync(0xffffffffu, op, o);
        kn = max(kn, __shfl_xor_sync(0xffffffffu, kn, o));
    }
    if ((threadIdx.x & 31) == 0) { rmax[threadIdx.x >> 5] = mx; open[threadIdx.x >> 5] = op; kneed[threadIdx.x >> 5] = kn; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0.0;
        int o = 0, k = 2;
        for (int w = 0; w < NWARP; ++w) { m = max_nan(m, rmax[w]); o += open[w]; k = max(k, kneed[w]); }
        k = min(K, k + ((K - k) & 1));
        if (cycle == 0) st->steps_total = 0;
        else st->steps_total += *kc;   // the previous cycle's steps
        st->relres = m;
        st->cycles = cycle;
        st->iters = st->steps_total;
        st->status = o ? 1 : 0;
        st->bytes += bytes;
        *kc = k;
        *done = o ? 0 : 1;
    }
}

// rv = (float)(r * scale), e_1 = c0 D^-1 rv, e_0 = 0: member-major FP64 -> interleaved FP32 (tiled transpose,
// grid-stride over the 32 x 32 tiles, row tiles fastest)
__global__ void __launch_bounds__(256) k_ls_init(const double *__restrict__ R, int n, int nv, int nvp,
                                                 const double *__restrict__ sc, const float *__restrict__ dinv, float c0,
                                                 float *rv, float *e0, float *e1, const int *done) {
    if (*(volatile const int *)done) return;
    __shared__ float t[32][33];
    const int ntx = (n + 31) / 32, ntile = ntx * (nvp / 32), tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
        const int i0 = (tile % ntx) * 32, v0 = (tile / ntx) * 32;
        for (int j = ty; j < 32; j += 8) {
            const int v = v0 + j, i = i0 + tx;
            t[j][tx] = (v < nv && i < n) ? (float)(R[(size_t)v * n + i] * sc[v]) : 0.f;
        }
        __syncthreads();
        for (int j = ty; j < 32; j += 8) {
            const int i = i0 + j, v = v0 + tx;
            if (i >= n) continue;
            const float r = t[tx][j];
            const size_t q = (size_t)i * nvp + v;
            rv[q] = r;
            e0[q] = 0.f;
            e1[q] = c0 * dinv[i] * r;
        }
        __syncthreads();   // t is refilled by the next tile
    }
}

// one step for every member, three-term form of the Chebyshev recurrence
// (d_{k-1} = e_k - e_{k-1}): s = A e_k,
// e_{k+1} = e_k + ca (e_k - e_{k-1}) + cb D^-1 (rv - s), written over e_{k-1}
// (each element is read and then written by the same thread; other threads
// gather only e_k) -- four vectors touched per step instead of five
// the stop flag and the cycle's step count sit side by side (8-byte aligned):
// one load decides whether step k of the cycle runs
__device__ __forceinline__ bool ls_stop(const int *done, int k) {
    int f, kc;
    asm volatile("ld.volatile.global.v2.s32 {%0, %1}, [%2];" : "=r"(f), "=r"(kc) : "l"(done));
    return f != 0 || k >= kc;
}

template <int W>
__global__ void __launch_bounds__(256) k_ls_step(const int *__restrict__ col, const float *__restrict__ a32,
                                                 const float *__restrict__ dinv, int n, int q4,
                                                 const float4 *__restrict__ ec, const float4 *__restrict__ rv,
                                                 float4 *ep, float ca, float cb, const int *done, int k,
                                                 const int *kc) {
    if (ls_stop(done, k)) return;
    const unsigned total = (unsigned)n * (unsigned)q4;   // < 2^31 (checked by the caller)
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const int i = (int)(t / (unsigned)q4), q = (int)(t - (unsigned)i * (unsigned)q4);
        int c[W];
        float a[W];
#pragma unroll
        for (int k = 0; k < W; ++k) { c[k] = __ldg(&col[(size_t)k * n + i]); a[k] = __ldg(&a32[(size_t)k * n + i]); }
        float4 g[W];
#pragma unroll
        for (int k = 0; k < W; ++k) g[k] = ec[(size_t)c[k] * q4 + q];
        float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int k = 0; k < W; ++k) {
            sum.x = fmaf(a[k], g[k].x, sum.x); sum.y = fmaf(a[k], g[k].y, sum.y);
            sum.z = fmaf(a[k], g[k].z, sum.z); sum.w = fmaf(a[k], g[k].w, sum.w);
        }
        const size_t idx = (size_t)i * q4 + q;
        const float di = cb * __ldg(&dinv[i]);
        const float4 r = rv[idx], e = ec[idx], eo = ep[idx];
        float4 dn;
        dn.x = ca * (e.x - eo.x) + di * (r.x - sum.x); dn.y = ca * (e.y - eo.y) + di * (r.y - sum.y);
        dn.z = ca * (e.z - eo.z) + di * (r.z - sum.z); dn.w = ca * (e.w - eo.w) + di * (r.w - sum.w);
        ep[idx] = make_float4(e.x + dn.x, e.y + dn.y, e.z + dn.z, e.w + dn.w);
    }
}

// k_ls_step reading A from the 64-byte row records (one matrix stream)
__global__ void __launch_bounds__(256) k_ls_step_pk(const uint4 *__restrict__ pk, const float *__restrict__ dinv,
                                                    int n, int q4, const float4 *__restrict__ ec,
                                                    const float4 *__restrict__ rv, float4 *ep, float ca, float cb,
                                                    const int *done, int k, const int *kc) {
    if (ls_stop(done, k)) return;   // converged, or past the cycle's steps
    const unsigned total = (unsigned)n * (unsigned)q4;   // < 2^31 (checked by the caller)
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const int i = (int)(t / (unsigned)q4), q = (int)(t - (unsigned)i * (unsigned)q4);
        int c[8];
        float a[8];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint4 e = __ldg(&pk[(size_t)i * 4 + k]);
            c[2 * k] = (int)e.x; a[2 * k] = __uint_as_float(e.y);
            c[2 * k + 1] = (int)e.z; a[2 * k + 1] = __uint_as_float(e.w);
        }
        float4 g[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) g[k] = ec[(size_t)c[k] * q4 + q];
        float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            sum.x = fmaf(a[k], g[k].x, sum.x); sum.y = fmaf(a[k], g[k].y, sum.y);
            sum.z = fmaf(a[k], g[k].z, sum.z); sum.w = fmaf(a[k], g[k].w, sum.w);
        }
        const size_t idx = (size_t)i * q4 + q;
        const float di = cb * __ldg(&dinv[i]);
        const float4 r = rv[idx], e = ec[idx], eo = ep[idx];
        float4 dn;
        dn.x = ca * (e.x - eo.x) + di * (r.x - sum.x); dn.y = ca * (e.y - eo.y) + di * (r.y - sum.y);
        dn.z = ca * (e.z - eo.z) + di * (r.z - sum.z); dn.w = ca * (e.w - eo.w) + di * (r.w - sum.w);
        ep[idx] = make_float4(e.x + dn.x, e.y + dn.y, e.z + dn.z, e.w + dn.w);
    }
}

// x += beta * e: interleaved FP32 -> member-major FP64 (tiled transpose, grid-stride as k_ls_init)
__global__ void __launch_bounds__(256) k_ls_update(double *X, int ld, int n, int nv, int nvp,
                                                   const double *__restrict__ beta, const float *__restrict__ e,
                                                   const int *done) {
    if (*(volatile const int *)done) return;
    __shared__ float t[32][33];
    const int ntx = (n + 31) / 32, ntile = ntx * (nvp / 32), tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
        const int i0 = (tile % ntx) * 32, v0 = (tile / ntx) * 32;
        for (int j = ty; j < 32; j += 8) {
            const int i = i0 + j, v = v0 + tx;
            t[j][tx] = i < n ? e[(size_t)i * nvp + v] : 0.f;
        }
        __syncthreads();
        for (int j = ty; j < 32; j += 8) {
            const int v = v0 + j, i = i0 + tx;
            if (v < nv && i < n) X[(size_t)v * ld + i] += beta[v] * (double)t[tx][j];
        }
        __syncthreads();   // t is refilled by the next tile
    }
}

int sm_count();

// Blocks of 256 threads resident at once for `kernel`: the grid of a
// grid-stride lockstep launch.  The launches of cycles after convergence only
// read the stop flag, and a full-size grid (one block per 256 work items)
// took about as long to retire as a short real step.
template <typename Kern>
unsigned resident_grid(Kern kernel, size_t smem) {
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, 256, smem) != cudaSuccess || per < 1) {
        cudaGetLastError();
        per = 1;
    }
    return (unsigned)(per * sm_count());
}

unsigned capped(long long want, unsigned cap) { return (unsigned)std::max(1LL, std::min<long long>(want, cap)); }

// the resident grids, queried once (lockstep_prepare runs this at operator
// creation, outside any stream capture); index W - 6 for the templates
struct LsGrids {
    unsigned step_pk, step[3], resid[3], init, update;
};
const LsGrids &ls_grids() {
    static std::once_flag once;
    static LsGrids g;
    std::call_once(once, [] {
        g.step_pk = resident_grid(k_ls_step_pk, 0);
        g.step[0] = resident_grid(k_ls_step<6>, 0);
        g.step[1] = resident_grid(k_ls_step<7>, 0);
        g.step[2] = resident_grid(k_ls_step<8>, 0);
        g.resid[0] = resident_grid(k_ls_resid<6>, 0);
        g.resid[1] = resident_grid(k_ls_resid<7>, 0);
        g.resid[2] = resident_grid(k_ls_resid<8>, 0);
        g.init = resident_grid(k_ls_init, 0);
        g.update = resident_grid(k_ls_update, 0);
    });
    return g;
}

// grid of a k_ls_resid<W> launch over `tiles` (row block, member group) tiles
unsigned resid_grid(int W, long long tiles) { return capped(tiles, ls_grids().resid[W - 6]); }

template <int W>
cudaError_t ls_steps(const DevSolveOp &op, int n, int q4, float *&ec, float *&ep, const float *rv,
                     const double *ca, const double *cb, int K, const int *done, const int *kc, cudaStream_t s) {
    const long long work = (long long)n * q4;
    const bool pk = op.pk32 != nullptr;   // row records: one matrix stream (ensemble steps -0.6 %)
    const unsigned blocks = capped((work + 255) / 256, pk ? ls_grids().step_pk : ls_grids().step[W - 6]);
    for (int k = 1; k < K; ++k) {
        if (pk)
            k_ls_step_pk<<<blocks, 256, 0, s>>>(op.pk32, op.dinv32, n, q4, (const float4 *)ec, (const float4 *)rv,
                                                (float4 *)ep, (float)ca[k], (float)cb[k], done, k, kc);
        else
            k_ls_step<W><<<blocks, 256, 0, s>>>(op.A.col, op.a32, op.dinv32, n, q4, (const float4 *)ec,
                                                (const float4 *)rv, (float4 *)ep, (float)ca[k], (float)cb[k], done,
                                                k, kc);
        float *t = ec; ec = ep; ep = t;   // e_{k+1} is in the old e_{k-1} buffer
    }
    return cudaGetLastError();
}

// returns cudaErrorNotSupported when this path does not apply (the caller
// then runs the per-member kernels)
cudaError_t cheb_lockstep(const DevSolveOp &op, const double *B, double *X, int nv, int ld, double tol,
                          double inner_rtol, char *w, const Layout &L, GmresStats *st, cudaStream_t s) {
    const int n = op.A.n, W = op.A.W;
    if (W < 6 || W > 8 || !op.a32 || !op.dinv32) return cudaErrorNotSupported;
    const int nvp = (nv + 31) / 32 * 32, q4 = nvp / 4;
    if ((long long)n * q4 >= (1LL << 31)) return cudaErrorNotSupported;
    const size_t vec = ((size_t)n * nvp * 4 + 255) & ~size_t(255);
    const int nbx = (n + 255) / 256;   // row blocks of the residual: one norm partial each
    if (3 * vec + (size_t)16 * nv * nbx > L.r - L.v) return cudaErrorNotSupported;
    if ((size_t)(4 * nvp + 64) * 8 > L.bar - L.part) return cudaErrorNotSupported;
    float *rv = (float *)(w + L.v), *e0 = (float *)(w + L.v + vec), *e1 = (float *)(w + L.v + 2 * vec);
    double *rpart = (double *)(w + L.v + 3 * vec), *bpart = rpart + (size_t)nv * nbx;
    double *R = (double *)(w + L.r);
    double *nrm = (double *)(w + L.part), *beta = nrm + 2 * nvp, *sc = beta + nvp;
    int *done = (int *)(sc + nvp), *kcp = done + 1;   // stop flag; the cycle's steps
    // coefficients (as the per-member Chebyshev kernel)
    const double lo = op.cheb_lmin, hi = op.cheb_lmax;
    const double kappa = hi / lo, sq = sqrt(kappa), sigma = (sq - 1.0) / (sq + 1.0);
    int K = (int)ceil(log(2.0 * kappa / inner_rtol) / log(1.0 / sigma)) + 1;
    K = K < 2 ? 2 : (K > CHEB_KMAX ? CHEB_KMAX : K);
    const double lg = log(2.0 * kappa), ls = log(1.0 / sigma);
    const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), s1 = theta / delta;
    double ca[CHEB_KMAX], cb[CHEB_KMAX], rho_prev = 1.0 / s1;
    ca[0] = cb[0] = 0.0;
    for (int k = 1; k < K; ++k) {
        const double rho = 1.0 / (2.0 * s1 - rho_prev);
        ca[k] = rho * rho_prev;
        cb[k] = 2.0 * rho / delta;
        rho_prev = rho;
    }
    // algorithmic bytes of one cycle: FP64 residual, init, K - 1 steps, update
    const double rowsb = (double)n;
    const double cyc = rowsb * nv * (8.0 * 3) + rowsb * W * 12.0 +
                       rowsb * nvp * (8.0 + 12.0) + (K - 1) * (rowsb * W * 8.0 + rowsb * nvp * 4.0 * 4.0) +
                       rowsb * nvp * 4.0 + rowsb * nv * 16.0;
    cudaError_t e;
    if ((e = cudaMemsetAsync(done, 0, sizeof(int), s)) != cudaSuccess) return e;
    const dim3 rgrid((unsigned)nbx, (unsigned)((nv + LS_MG - 1) / LS_MG));
    k_ls_sq<<<rgrid, 256, 0, s>>>(B, n, ld, nv, bpart);
    const unsigned cap_init = ls_grids().init, cap_upd = ls_grids().update;
    const long long ntile = (long long)((n + 31) / 32) * (nvp / 32);
    const unsigned rblocks = resid_grid(W, (long long)rgrid.x * rgrid.y);
    for (int c = 0; c <= LS_MAXC; ++c) {
        switch (W) {
        case 6: k_ls_resid<6><<<rblocks, 256, 0, s>>>(op.A.col, op.A.val, n, B, X, ld, R, nv, rpart, nbx, done); break;
        case 7: k_ls_resid<7><<<rblocks, 256, 0, s>>>(op.A.col, op.A.val, n, B, X, ld, R, nv, rpart, nbx, done); break;
        default: k_ls_resid<8><<<rblocks, 256, 0, s>>>(op.A.col, op.A.val, n, B, X, ld, R, nv, rpart, nbx, done); break;
        }
        k_ls_nrm<<<(nv + NWARP - 1) / NWARP, 256, 0, s>>>(rpart, bpart, nbx, nrm, nv, done);
        k_ls_scale<<<1, 256, 0, s>>>(nrm, nv, nvp, tol, beta, sc, done, st, c, K, c ? cyc : 0.0, lg, ls, kcp);
        if (c == LS_MAXC) break;
        k_ls_init<<<capped(ntile, cap_init), 256, 0, s>>>(R, n, nv, nvp, sc, op.dinv32, (float)(1.0 / theta), rv, e0,
                                                          e1, done);
        float *ec = e1, *ep = e0;
        switch (W) {
        case 6: e = ls_steps<6>(op, n, q4, ec, ep, rv, ca, cb, K, done, kcp, s); break;
        case 7: e = ls_steps<7>(op, n, q4, ec, ep, rv, ca, cb, K, done, kcp, s); break;
        default: e = ls_steps<8>(op, n, q4, ec, ep, rv, ca, cb, K, done, kcp, s); break;
        }
        if (e != cudaSuccess) return e;
        k_ls_update<<<capped(ntile, cap_upd), 256, 0, s>>>(X, ld, n, nv, nvp, beta, ec, done);
    }
    g_kernel_launches += 1 + (LS_MAXC + 1) * 3 + LS_MAXC * (K + 1);
    return cudaGetLastError();
}

// the device's SM count, read once (serving lanes call this from several threads)
std::atomic<int> g_sms{0};

int sm_count() {
    int n = g_sms.load(std::memory_order_relaxed);
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        g_sms.store(n, std::memory_order_relaxed);
    }
    return n;
}

int env_int(const char *name, int dflt) {
    const char *e = getenv(name);
    return e ? atoi(e) : dflt;
}

// ------------------------------------------------ lockstep multigrid FGMRES ---
// Many right-hand sides of the multigrid-preconditioned Laplacian solve in
// lockstep (the Laplace solves of an ensemble step).  The algorithm is the one
// gmres_kernel runs for each member -- restarted FGMRES, right-preconditioned
// by a V-cycle with one damped-Jacobi sweep down and one up and a dense
// coarsest solve, FP32 inner cycles inside an FP64 refinement loop with the
// same stopping tests -- but the Krylov and multigrid vectors of all members
// are interleaved FP32 multi-vectors (row i holds the nvp members
// contiguously) and every phase is one short kernel over all members: a
// gathered row is read once as whole 16-byte member chunks, and no block
// waits on another.  Per-member state (Hessenberg factor, rotations,
// stopping tests) lives in device arrays.  Device flags end the remaining
// launches of a cycle once every member has met its inner target and of the
// solve once every member has stopped, without a host synchronisation, so
// the whole solve can sit in a captured step graph; every kernel walks its
// index range with a grid-stride loop over a grid capped at a few blocks per
// SM, so a launch that finds its flag set costs little.
constexpr int LSG_M = 8;        // Arnoldi steps per refinement cycle
// refinement cycles at most: three cycles of an 1e-5 inner reduction reach
// 1e-12 from a zero start; a fourth only added skipped launches (L6 x 32
// ensemble step 22.5 -> 21.9 ms without it)
constexpr int LSG_MAXC = 3;
constexpr int LSG_MINRHS = 8;   // fewest right-hand sides the path accepts
constexpr int LSG_SMALL = 700;  // levels of at most this many rows run in one shared-memory kernel
constexpr size_t LSG_SMALL_SMEM = 160 * 1024;

struct LsgLevel {               // one multigrid level; buffers n x nvp FP32
    int n, W, Wr;
    const int *col; const float *a; const float *d;
    const int *pc; const float *pw;      // prolongation from level + 1
    const int *rf; const float *rw;      // restriction to level + 1
    float *x, *xo, *r, *b;
};

struct LsgParams {
    int n, nv, nvp, q4, m, nlev, W, RB, nbx, ld, max_iter, maxc;
    double tol, inner_rtol, step_row_bytes, resid_row_bytes;
    float omega;
    const int *col; const float *a32;    // fine operator, FP32 (w = A z)
    LsgLevel lev[MG_MAXLEV];
    int nc; const float *cinv;           // coarsest level, dense inverse
    int lc;                              // levels [lc, nlev) run in one kernel, in shared memory
    LsgLevel *levs;                      // device copy of lev[] (indexed at run time by that kernel)
    const double *B; double *X;          // member-major FP64, leading dimension ld
    float *V, *Z, *w;                    // (m + 1), m and 1 interleaved vectors
    double *R, *rpart, *bpart, *nrm;     // FP64 residual, norm partials, norms (2 per member)
    double *dpart, *npart;               // RB x (m + 1) x nvp dot partials; RB x nvp norm partials
    double *hcol, *H, *cs, *sn, *g;      // per member: column (m + 1), R factor (m + 1) x m, rotations, rhs
    float *hv, *yv;                      // per member: FP32 column, FP32 solution
    double *bnorm, *beta_prev, *target, *relv;
    float *scale, *vscale;
    int *stt, *arn, *jl, *iters, *cycles, *zerox, *cnt, *done;
    GmresStats *st;
};

__device__ __forceinline__ unsigned lsg_grid_stride() { return gridDim.x * blockDim.x; }

// per member: the refinement test on ||b - A x|| (norms from k_ls_nrm) and the
// start of the next cycle; 0 members left sets the solve's done flag
__global__ void __launch_bounds__(256) k_lsg_begin(LsgParams P, int c) {
    if (*(volatile int *)P.done) return;
    __shared__ double rmax[NWARP];
    __shared__ int open[NWARP], bad[NWARP], itm[NWARP], cym[NWARP], its[NWARP];
    double mx = 0.0;
    int nopen = 0, nbad = 0, imax = 0, cmax = 0, isum = 0;
    const int m = P.m;
    for (int v = threadIdx.x; v < P.nvp; v += blockDim.x) {
        P.jl[v] = 0;
        P.vscale[v] = 0.f;
        if (v >= P.nv) { P.scale[v] = 0.f; P.arn[v] = 0; continue; }
        if (c == 0) {
            P.bnorm[v] = sqrt(P.nrm[2 * v + 1]);
            P.stt[v] = 0; P.iters[v] = 0; P.cycles[v] = 0; P.beta_prev[v] = 0.0; P.relv[v] = 0.0;
            P.zerox[v] = P.bnorm[v] == 0.0;
        }
        int s = P.stt[v];
        if (s == 0) {
            const double bn = P.bnorm[v];
            if (bn == 0.0) { s = 1; P.relv[v] = 0.0; }
            else {
                const double beta = sqrt(P.nrm[2 * v]), rel = beta / bn;
                P.relv[v] = rel;
                if (rel <= P.tol) s = 1;
                else if (P.iters[v] >= P.max_iter) s = 2;
                else if (P.cycles[v] > 0 && !(beta < 0.9999 * P.beta_prev[v])) s = 2;
                else if (c == P.maxc) s = 2;   // out of cycles
                if (s == 0) {
                    P.beta_prev[v] = beta;
                    P.cycles[v] += 1;
                    P.target[v] = fmax(P.tol * bn, P.inner_rtol * beta);
                    double *g = P.g + (size_t)v * (m + 1);
                    g[0] = beta;
                    for (int l = 1; l <= m; ++l) g[l] = 0.0;
                    P.scale[v] = (float)(1.0 / beta);
                    P.arn[v] = 1;
                    ++nopen;
                }
            }
            P.stt[v] = s;
        }
        if (s != 0) { P.scale[v] = 0.f; P.arn[v] = 0; }
        const double rel = P.relv[v];
        mx = max_nan(mx, rel);
        if (!(rel == rel)) mx = rel;
        nbad += s == 2 ? 1 : 0;
        imax = max(imax, P.iters[v]);
        cmax = max(cmax, P.cycles[v]);
        isum += P.iters[v];
    }
    for (int o = 16; o > 0; o >>= 1) {
        mx = max_nan(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        nopen += __shfl_xor_sync(0xffffffffu, nopen, o);
        nbad += __shfl_xor_sync(0xffffffffu, nbad, o);
        imax = max(imax, __shfl_xor_sync(0xffffffffu, imax, o));
        cmax = max(cmax, __shfl_xor_sync(0xffffffffu, cmax, o));
        isum += __shfl_xor_sync(0xffffffffu, isum, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { rmax[w] = mx; open[w] = nopen; bad[w] = nbad; itm[w] = imax; cym[w] = cmax; its[w] = isum; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        int o = 0, b = 0, im = 0, cm = 0, is = 0;
        for (int k = 0; k < NWARP; ++k) {
            r = max_nan(r, rmax[k]); o += open[k]; b += bad[k]; im = max(im, itm[k]); cm = max(cm, cym[k]); is += its[k];
        }
        P.st->relres = r;
        P.st->status = (o || b) ? 1 : 0;
        P.st->iters = im;
        P.st->cycles = cm;
        P.st->steps_total = is;
        P.st->bytes += P.resid_row_bytes * P.n * (double)P.nv;
        P.cnt[0] = o;
        for (int l = 1; l <= m; ++l) P.cnt[l] = 0;
        if (!o) *P.done = 1;
    }
}

// x = 0 for members whose right-hand side is zero (as the per-member solver)
__global__ void __launch_bounds__(256) k_lsg_zero(LsgParams P) {
    const long long total = (long long)P.nv * P.n;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += lsg_grid_stride()) {
        const int v = (int)(t / P.n), i = (int)(t - (long long)v * P.n);
        if (P.zerox[v]) P.X[(size_t)v * P.ld + i] = 0.0;
    }
}

// V_0 = (float)(R * scale): member-major FP64 -> interleaved FP32 (tiled transpose)
__global__ void __launch_bounds__(256) k_lsg_v0(LsgParams P) {
    if (*(volatile int *)P.done) return;
    __shared__ float t[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int ntile = (P.n + 31) / 32, mtile = P.nvp / 32;
    for (int tile = blockIdx.x; tile < ntile * mtile; tile += gridDim.x) {
        const int i0 = (tile % ntile) * 32, v0 = (tile / ntile) * 32;
        for (int j = ty; j < 32; j += 8) {
            const int v = v0 + j, i = i0 + tx;
            t[j][tx] = (v < P.nv && i < P.n) ? (float)(P.R[(size_t)v * P.n + i] * (double)P.scale[v]) : 0.f;
        }
        __syncthreads();
        for (int j = ty; j < 32; j += 8) {
            const int i = i0 + j;
            if (i < P.n) P.V[(size_t)i * P.nvp + v0 + tx] = t[tx][j];
        }
        __syncthreads();
    }
}

__device__ __forceinline__ float4 f4fma(float a, float4 x, float4 s) {
    return make_float4(fmaf(a, x.x, s.x), fmaf(a, x.y, s.y), fmaf(a, x.z, s.z), fmaf(a, x.w, s.w));
}

__device__ __forceinline__ bool lsg_skip(const LsgParams &P, int j) {
    return *(volatile const int *)P.done || (j >= 0 && *(volatile const int *)&P.cnt[j] == 0);
}

__device__ __forceinline__ float4 f4mul(float4 a, float4 b) { return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }

// down sweep at level l: x = w D^-1 b, r = b - A x (from b alone).  With
// vout set, b = src * vscale (the Krylov vector v_j = w / ||w|| formed on the
// fly from the previous step's w) and the block's own rows of v_j are stored.
__global__ void __launch_bounds__(256) k_mg_down(LsgParams P, LsgLevel L, const float *src, float *vout, int j) {
    if (lsg_skip(P, j)) return;
    const int q4 = P.q4;
    const float4 *b = (const float4 *)src;
    float4 *x = (float4 *)L.x, *r = (float4 *)L.r;
    const float om = P.omega;
    const long long total = (long long)L.n * q4;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += lsg_grid_stride()) {
        const int i = (int)(t / q4), q = (int)(t - (long long)i * q4);
        const float4 sc = vout ? ((const float4 *)P.vscale)[q] : make_float4(1.f, 1.f, 1.f, 1.f);
        int c[8];
        float a[8];
        float4 g[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < L.W) { c[k] = __ldg(&L.col[(size_t)k * L.n + i]); a[k] = __ldg(&L.a[(size_t)k * L.n + i]); }
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < L.W) g[k] = f4mul(b[(size_t)c[k] * q4 + q], sc);
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < L.W) s = f4fma(a[k] * (om * __ldg(&L.d[c[k]])), g[k], s);
        const float4 bi = f4mul(b[(size_t)i * q4 + q], sc);
        if (vout) ((float4 *)vout)[(size_t)i * q4 + q] = bi;
        const float di = om * __ldg(&L.d[i]);
        x[(size_t)i * q4 + q] = make_float4(di * bi.x, di * bi.y, di * bi.z, di * bi.w);
        r[(size_t)i * q4 + q] = make_float4(bi.x - s.x, bi.y - s.y, bi.z - s.z, bi.w - s.w);
    }
}

// b_{l+1} = R r_l
__global__ void __launch_bounds__(256) k_mg_restrict(LsgParams P, LsgLevel L, LsgLevel C, int j) {
    if (lsg_skip(P, j)) return;
    const int q4 = P.q4, nc = C.n;
    const float4 *r = (const float4 *)L.r;
    float4 *bc = (float4 *)C.b;
    const long long total = (long long)nc * q4;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += lsg_grid_stride()) {
        const int cc = (int)(t / q4), q = (int)(t - (long long)cc * q4);
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int k = 0; k < L.Wr; ++k) {
            const int f = __ldg(&L.rf[(size_t)k * nc + cc]);
            if (f >= 0) s = f4fma(__ldg(&L.rw[(size_t)k * nc + cc]), r[(size_t)f * q4 + q], s);
        }
        bc[(size_t)cc * q4 + q] = s;
    }
}

// threads of a k_mg_small block: one per row of the 641-row level (a block runs
// one 4-member chunk alone, so the small levels' sweeps are its latency)
constexpr int MG_SMALL_TB = 1024;

// Levels [lc, nlev) for one 4-member chunk per block, in shared memory (four
// float4 vectors per level: x, t, b, r): b_lc = R r_{lc-1} (or the input when
// lc = 0), down sweeps and restrictions, the dense coarsest solve, the
// prolongations and up sweeps; x_lc is written to out (the coarse correction
// of level lc - 1, or the V-cycle's output when lc = 0).  Replaces one launch
// per small level and phase by a single launch.
__global__ void __launch_bounds__(MG_SMALL_TB) k_mg_small(LsgParams P, const float *src, float *vout, float *out, int j) {
    if (lsg_skip(P, j)) return;
    extern __shared__ float4 sm4[];
    const int q4 = P.q4, lc = P.lc, last = P.nlev - 1;
    const float om = P.omega;
    const LsgLevel *LV = P.levs;
    for (int q = blockIdx.x; q < q4; q += gridDim.x) {
        // shared-memory offsets of the levels
        int off[MG_MAXLEV];
        int o = 0;
        for (int l = lc; l <= last; ++l) { off[l] = o; o += 4 * LV[l].n; }
        // b at level lc
        {
            const LsgLevel L = LV[lc];
            float4 *b = sm4 + off[lc] + 2 * L.n;
            if (lc == 0) {
                const float4 sc = vout ? ((const float4 *)P.vscale)[q] : make_float4(1.f, 1.f, 1.f, 1.f);
                for (int i = threadIdx.x; i < L.n; i += blockDim.x) {
                    const float4 v = f4mul(((const float4 *)src)[(size_t)i * q4 + q], sc);
                    b[i] = v;
                    if (vout) ((float4 *)vout)[(size_t)i * q4 + q] = v;
                }
            } else {
                const LsgLevel F = LV[lc - 1];
                const float4 *r = (const float4 *)F.r;
                for (int c = threadIdx.x; c < L.n; c += blockDim.x) {
                    float4 sacc = make_float4(0.f, 0.f, 0.f, 0.f);
                    for (int k = 0; k < F.Wr; ++k) {
                        const int f = __ldg(&F.rf[(size_t)k * L.n + c]);
                        if (f >= 0) sacc = f4fma(__ldg(&F.rw[(size_t)k * L.n + c]), r[(size_t)f * q4 + q], sacc);
                    }
                    b[c] = sacc;
                }
            }
        }
        __syncthreads();
        // down: x = w D^-1 b, r = b - A x, b_{l+1} = R r
        for (int l = lc; l < last; ++l) {
            const LsgLevel L = LV[l];
            float4 *x = sm4 + off[l], *b = x + 2 * L.n, *r = x + 3 * L.n;
            for (int i = threadIdx.x; i < L.n; i += blockDim.x) {
                const float di = om * __ldg(&L.d[i]);
                x[i] = make_float4(di * b[i].x, di * b[i].y, di * b[i].z, di * b[i].w);
            }
            __syncthreads();
            for (int i = threadIdx.x; i < L.n; i += blockDim.x) {
                float4 sacc = make_float4(0.f, 0.f, 0.f, 0.f);
                for (int k = 0; k < L.W; ++k)
                    sacc = f4fma(__ldg(&L.a[(size_t)k * L.n + i]), x[__ldg(&L.col[(size_t)k * L.n + i])], sacc);
                r[i] = make_float4(b[i].x - sacc.x, b[i].y - sacc.y, b[i].z - sacc.z, b[i].w - sacc.w);
            }
            __syncthreads();
            const LsgLevel C = LV[l + 1];
            float4 *bc = sm4 + off[l + 1] + 2 * C.n;
            for (int c = threadIdx.x; c < C.n; c += blockDim.x) {
                float4 sacc = make_float4(0.f, 0.f, 0.f, 0.f);
                for (int k = 0; k < L.Wr; ++k) {
                    const int f = __ldg(&L.rf[(size_t)k * C.n + c]);
                    if (f >= 0) sacc = f4fma(__ldg(&L.rw[(size_t)k * C.n + c]), r[f], sacc);
                }
                bc[c] = sacc;
            }
            __syncthreads();
        }
        // coarsest: x = C^-1 b
        {
            const int n = P.nc;
            float4 *x = sm4 + off[last], *b = x + 2 * n;
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                float4 sacc = make_float4(0.f, 0.f, 0.f, 0.f);
                for (int k = 0; k < n; ++k) sacc = f4fma(__ldg(&P.cinv[(size_t)i * n + k]), b[k], sacc);
                x[i] = sacc;
            }
            __syncthreads();
        }
        // up: x += P x_{l+1}; x = x + w D^-1 (b - A x)
        for (int l = last - 1; l >= lc; --l) {
            const LsgLevel L = LV[l];
            float4 *x = sm4 + off[l], *t = x + L.n, *b = x + 2 * L.n;
            const float4 *xc = sm4 + off[l + 1];
            for (int i = threadIdx.x; i < L.n; i += blockDim.x) {
                const int c0 = __ldg(&L.pc[2 * i]), c1 = __ldg(&L.pc[2 * i + 1]);
                float4 sacc = make_float4(0.f, 0.f, 0.f, 0.f);
                if (c0 >= 0) sacc = f4fma(__ldg(&L.pw[2 * i]), xc[c0], sacc);
                if (c1 >= 0) sacc = f4fma(__ldg(&L.pw[2 * i + 1]), xc[c1], sacc);
                x[i] = make_float4(x[i].x + sacc.x, x[i].y + sacc.y, x[i].z + sacc.z, x[i].w + sacc.w);
            }
            __syncthreads();
            for (int i = threadIdx.x; i < L.n; i += blockDim.x) {
                float4 sacc = make_float4(0.f, 0.f, 0.f, 0.f);
                for (int k = 0; k < L.W; ++k)
                    sacc = f4fma(__ldg(&L.a[(size_t)k * L.n + i]), x[__ldg(&L.col[(size_t)k * L.n + i])], sacc);
                const float di = om * __ldg(&L.d[i]);
                t[i] = make_float4(x[i].x + di * (b[i].x - sacc.x), x[i].y + di * (b[i].y - sacc.y),
                                   x[i].z + di * (b[i].z - sacc.z), x[i].w + di * (b[i].w - sacc.w));
            }
            __syncthreads();
            float4 *dst = l == lc ? (float4 *)out : x;
            if (l == lc)
                for (int i = threadIdx.x; i < L.n; i += blockDim.x) dst[(size_t)i * q4 + q] = t[i];
            else
                for (int i = threadIdx.x; i < L.n; i += blockDim.x) x[i] = t[i];
            __syncthreads();
        }
        if (lc == last)   // the whole cycle is the dense solve
            for (int i = threadIdx.x; i < P.nc; i += blockDim.x) ((float4 *)out)[(size_t)i * q4 + q] = sm4[off[last] + i];
        __syncthreads();
    }
}

// copy of the level descriptors into device memory (static indices only)
__global__ void k_lsg_levels(LsgParams P) {
    if (threadIdx.x || blockIdx.x) return;
#pragma unroll
    for (int k = 0; k < MG_MAXLEV; ++k) P.levs[k] = P.lev[k];
}

// x_l += P x_{l+1}
__global__ void __launch_bounds__(256) k_mg_prolong(LsgParams P, LsgLevel L, const float *xcoarse, int j) {
    if (lsg_skip(P, j)) return;
    const int q4 = P.q4;
    const float4 *xc = (const float4 *)xcoarse;
    float4 *x = (float4 *)L.x;
    const long long total = (long long)L.n * q4;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += lsg_grid_stride()) {
        const int i = (int)(t / q4), q = (int)(t - (long long)i * q4);
        const int c0 = __ldg(&L.pc[2 * i]), c1 = __ldg(&L.pc[2 * i + 1]);
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
        if (c0 >= 0) s = f4fma(__ldg(&L.pw[2 * i]), xc[(size_t)c0 * q4 + q], s);
        if (c1 >= 0) s = f4fma(__ldg(&L.pw[2 * i + 1]), xc[(size_t)c1 * q4 + q], s);
        float4 xi = x[(size_t)i * q4 + q];
        x[(size_t)i * q4 + q] = make_float4(xi.x + s.x, xi.y + s.y, xi.z + s.z, xi.w + s.w);
    }
}

// post-smoothing at level l: out = x + w D^-1 (b - A x)
__global__ void __launch_bounds__(256) k_mg_smooth(LsgParams P, LsgLevel L, const float *bsrc, float *out, int j) {
    if (lsg_skip(P, j)) return;
    const int q4 = P.q4;
    const float4 *b = (const float4 *)bsrc, *x = (const float4 *)L.x;
    float4 *o = (float4 *)out;
    const float om = P.omega;
    const long long total = (long long)L.n * q4;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += lsg_grid_stride()) {
        const int i = (int)(t / q4), q = (int)(t - (long long)i * q4);
        int c[8];
        float a[8];
        float4 g[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < L.W) { c[k] = __ldg(&L.col[(size_t)k * L.n + i]); a[k] = __ldg(&L.a[(size_t)k * L.n + i]); }
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < L.W) g[k] = x[(size_t)c[k] * q4 + q];
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < L.W) s = f4fma(a[k], g[k], s);
        const float4 bi = b[(size_t)i * q4 + q], xi = x[(size_t)i * q4 + q];
        const float di = om * __ldg(&L.d[i]);
        o[(size_t)i * q4 + q] = make_float4(xi.x + di * (bi.x - s.x), xi.y + di * (bi.y - s.y),
                                            xi.z + di * (bi.z - s.z), xi.w + di * (bi.w - s.w));
    }
}

// w = A z_j (fine operator, FP32)
__global__ void __launch_bounds__(256) k_lsg_spmm(LsgParams P, int j) {
    if (lsg_skip(P, j)) return;
    const int q4 = P.q4, n = P.n, W = P.W;
    const float4 *z = (const float4 *)(P.Z + (size_t)j * n * P.nvp);
    float4 *w = (float4 *)P.w;
    const long long total = (long long)n * q4;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += lsg_grid_stride()) {
        const int i = (int)(t / q4), q = (int)(t - (long long)i * q4);
        int c[8];
        float a[8];
        float4 g[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < W) { c[k] = __ldg(&P.col[(size_t)k * n + i]); a[k] = __ldg(&P.a32[(size_t)k * n + i]); }
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < W) g[k] = z[(size_t)c[k] * q4 + q];
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < W) s = f4fma(a[k], g[k], s);
        w[(size_t)i * q4 + q] = s;
    }
}

// dot partials: dpart[rb][l][v] = sum over the block's rows of V_l[r][v] w[r][v], l <= j
// (grid RB x nvp/32; lane = member, warps stride the rows; eight vectors per pass)
__global__ void __launch_bounds__(256) k_lsg_dot(LsgParams P, int j) {
    if (lsg_skip(P, j)) return;
    __shared__ double red[NWARP][8][32];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const int v = blockIdx.y * 32 + lane, nvp = P.nvp, n = P.n;
    const int rpr = (n + P.RB - 1) / P.RB;
    const int r0 = min(n, (int)blockIdx.x * rpr), r1 = min(n, r0 + rpr);
    const size_t vs = (size_t)n * nvp;
    for (int l0 = 0; l0 <= j; l0 += 8) {
        const int kk = min(8, j + 1 - l0);
        float t[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int r = r0 + wp; r < r1; r += NWARP) {
            const float s = P.w[(size_t)r * nvp + v];
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (k < kk) t[k] += P.V[(size_t)(l0 + k) * vs + (size_t)r * nvp + v] * s;
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) red[wp][k][lane] = (double)t[k];
        __syncthreads();
        for (int e = threadIdx.x; e < kk * 32; e += blockDim.x) {
            const int k = e >> 5, ln = e & 31;
            double s = 0.0;
            for (int q = 0; q < NWARP; ++q) s += red[q][k][ln];
            P.dpart[((size_t)blockIdx.x * (P.m + 1) + l0 + k) * nvp + blockIdx.y * 32 + ln] = s;
        }
        __syncthreads();
    }
}

// h[v][l] = sum over row blocks of the partials (one warp per (member, l), fixed order)
__global__ void __launch_bounds__(256) k_lsg_hsum(LsgParams P, int j) {
    if (lsg_skip(P, j)) return;
    const int pair = blockIdx.x * NWARP + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (pair >= P.nv * (j + 1)) return;
    const int v = pair / (j + 1), l = pair - v * (j + 1);
    double s = 0.0;
    for (int rb = lane; rb < P.RB; rb += 32) s += P.dpart[((size_t)rb * (P.m + 1) + l) * P.nvp + v];
    s = warp_sum(s);
    if (lane == 0) {
        P.hcol[(size_t)v * (P.m + 1) + l] = s;
        P.hv[(size_t)v * (P.m + 1) + l] = (float)s;
    }
}

// w -= sum_l h_l V_l; ||w||^2 partials per row block
__global__ void __launch_bounds__(256) k_lsg_update(LsgParams P, int j) {
    if (lsg_skip(P, j)) return;
    __shared__ double red[NWARP][32];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const int v = blockIdx.y * 32 + lane, nvp = P.nvp, n = P.n;
    const int rpr = (n + P.RB - 1) / P.RB;
    const int r0 = min(n, (int)blockIdx.x * rpr), r1 = min(n, r0 + rpr);
    const size_t vs = (size_t)n * nvp;
    float h[LSG_M];
#pragma unroll
    for (int l = 0; l < LSG_M; ++l) h[l] = (l <= j && v < P.nv) ? P.hv[(size_t)v * (P.m + 1) + l] : 0.f;
    float a2 = 0.f;
    for (int r = r0 + wp; r < r1; r += NWARP) {
        float s = P.w[(size_t)r * nvp + v];
#pragma unroll
        for (int l = 0; l < LSG_M; ++l)
            if (l <= j) s -= h[l] * P.V[(size_t)l * vs + (size_t)r * nvp + v];
        P.w[(size_t)r * nvp + v] = s;
        a2 += s * s;
    }
    red[wp][lane] = (double)a2;
    __syncthreads();
    if (threadIdx.x < 32) {
        double s = 0.0;
        for (int q = 0; q < NWARP; ++q) s += red[q][threadIdx.x];
        P.npart[(size_t)blockIdx.x * nvp + blockIdx.y * 32 + threadIdx.x] = s;
    }
}

// ||w||, the rotations, the stopping test (one warp per member)
__global__ void __launch_bounds__(256) k_lsg_givens(LsgParams P, int j) {
    if (lsg_skip(P, j)) return;
    const int v = blockIdx.x * NWARP + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (v >= P.nv) return;
    double s = 0.0;
    for (int rb = lane; rb < P.RB; rb += 32) s += P.npart[(size_t)rb * P.nvp + v];
    s = warp_sum(s);
    if (lane != 0) return;
    if (!P.arn[v]) { P.vscale[v] = 0.f; return; }
    const int m = P.m;
    double *hc = P.hcol + (size_t)v * (m + 1), *H = P.H + (size_t)v * (m + 1) * m;
    double *cs = P.cs + (size_t)v * m, *sn = P.sn + (size_t)v * m, *g = P.g + (size_t)v * (m + 1);
    const double hn = sqrt(s);
    hc[j + 1] = hn;
    for (int l = 0; l < j; ++l) {
        const double a = hc[l], c = hc[l + 1];
        hc[l] = cs[l] * a + sn[l] * c;
        hc[l + 1] = -sn[l] * a + cs[l] * c;
    }
    const double a = hc[j], c = hc[j + 1];
    const double r = hypot(a, c);
    cs[j] = r > 0.0 ? a / r : 1.0;
    sn[j] = r > 0.0 ? c / r : 0.0;
    for (int l = 0; l < j; ++l) H[(size_t)l * m + j] = hc[l];
    H[(size_t)j * m + j] = r;
    g[j + 1] = -sn[j] * g[j];
    g[j] = cs[j] * g[j];
    P.iters[v] += 1;
    P.jl[v] = j + 1;
    atomicAdd(&P.st->bytes, P.step_row_bytes * P.n + 8.0 * (j + 1) * P.n);
    const bool stop = fabs(g[j + 1]) <= P.target[v] || hn == 0.0 || P.iters[v] >= P.max_iter || j + 1 == m;
    if (stop) { P.arn[v] = 0; P.vscale[v] = 0.f; }
    else { P.vscale[v] = (float)(1.0 / hn); atomicAdd(&P.cnt[j + 1], 1); }
}

// y = H^-1 g over each member's jl columns (FP64), FP32 copy for the correction
__global__ void __launch_bounds__(256) k_lsg_solve(LsgParams P) {
    if (*(volatile int *)P.done) return;
    const int m = P.m;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < P.nvp; v += lsg_grid_stride()) {
        float *yv = P.yv + (size_t)v * m;
        const int jl = v < P.nv ? P.jl[v] : 0;
        double y[LSG_M];
        const double *H = P.H + (size_t)v * (m + 1) * m, *g = P.g + (size_t)v * (m + 1);
        for (int l = jl - 1; l >= 0; --l) {
            double s = g[l];
            for (int k = l + 1; k < jl; ++k) s -= H[(size_t)l * m + k] * y[k];
            y[l] = s / H[(size_t)l * m + l];
        }
        for (int l = 0; l < m; ++l) yv[l] = l < jl ? (float)y[l] : 0.f;
    }
}

// x += sum_l y_l z_l: interleaved FP32 -> member-major FP64 (tiled transpose)
__global__ void __launch_bounds__(256) k_lsg_correct(LsgParams P) {
    if (*(volatile int *)P.done) return;
    __shared__ float t[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5, m = P.m, n = P.n, nvp = P.nvp;
    const int ntile = (n + 31) / 32, mtile = nvp / 32;
    const size_t vs = (size_t)n * nvp;
    for (int tile = blockIdx.x; tile < ntile * mtile; tile += gridDim.x) {
        const int i0 = (tile % ntile) * 32, v0 = (tile / ntile) * 32;
        const int v = v0 + tx;
        // only the member's own Arnoldi columns: later ones were not written this cycle
        const int jv = v < P.nv ? P.jl[v] : 0;
        float y[LSG_M];
#pragma unroll
        for (int l = 0; l < LSG_M; ++l) y[l] = l < jv ? P.yv[(size_t)v * m + l] : 0.f;
        for (int jj = ty; jj < 32; jj += 8) {
            const int i = i0 + jj;
            float s = 0.f;
            if (i < n)
#pragma unroll
                for (int l = 0; l < LSG_M; ++l)
                    if (l < jv) s += y[l] * P.Z[(size_t)l * vs + (size_t)i * nvp + v];
            t[jj][tx] = s;
        }
        __syncthreads();
        for (int jj = ty; jj < 32; jj += 8) {
            const int vv = v0 + jj, i = i0 + tx;
            if (vv < P.nv && i < n && P.jl[vv] > 0) P.X[(size_t)vv * P.ld + i] += (double)t[tx][jj];
        }
        __syncthreads();
    }
}

struct LsgLayout {
    size_t V, Z, w, R, lev[MG_MAXLEV], rpart, bpart, nrm, dpart, npart, hcol, H, cs, sn, g, hv, yv;
    size_t bnorm, beta_prev, target, relv, scale, vscale, ints, levs, total;
    int nvp, m, RB, nbx;
};

LsgLayout lsg_layout(const DevSolveOp &op, int nv, int restart) {
    LsgLayout L;
    const size_t n = (size_t)op.A.n;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    L.nvp = (nv + 31) / 32 * 32;
    L.m = restart < LSG_M ? restart : LSG_M;
    L.nbx = (int)((n + 255) / 256);
    int rb = 4 * sm_count() / (L.nvp / 32);
    const int rbmax = (int)((n + 63) / 64);
    L.RB = rb < 1 ? 1 : (rb > rbmax ? rbmax : rb);
    const size_t nvp = (size_t)L.nvp, m = (size_t)L.m, vec = al(4 * n * nvp);
    size_t o = 0;
    L.V = o; o += (m + 1) * vec;
    L.Z = o; o += m * vec;
    L.w = o; o += vec;
    L.R = o; o += al(8 * n * (size_t)nv);
    for (int l = 0; l < op.mg.nlev && l < MG_MAXLEV; ++l) { L.lev[l] = o; o += 4 * al(4 * (size_t)op.mg.lev[l].n * nvp); }
    L.rpart = o; o += al(8 * (size_t)nv * L.nbx);
    L.bpart = o; o += al(8 * (size_t)nv * L.nbx);
    L.nrm = o; o += al(16 * nvp);
    L.dpart = o; o += al(8 * (size_t)L.RB * (m + 1) * nvp);
    L.npart = o; o += al(8 * (size_t)L.RB * nvp);
    L.hcol = o; o += al(8 * nvp * (m + 1));
    L.H = o; o += al(8 * nvp * (m + 1) * m);
    L.cs = o; o += al(8 * nvp * m);
    L.sn = o; o += al(8 * nvp * m);
    L.g = o; o += al(8 * nvp * (m + 1));
    L.hv = o; o += al(4 * nvp * (m + 1));
    L.yv = o; o += al(4 * nvp * m);
    L.bnorm = o; o += al(8 * nvp);
    L.beta_prev = o; o += al(8 * nvp);
    L.target = o; o += al(8 * nvp);
    L.relv = o; o += al(8 * nvp);
    L.scale = o; o += al(4 * nvp);
    L.vscale = o; o += al(4 * nvp);
    L.ints = o; o += al(4 * (6 * nvp + m + 2 + 1));
    L.levs = o; o += al(sizeof(LsgLevel) * MG_MAXLEV);
    L.total = o;
    return L;
}

bool lsg_applicable(const DevSolveOp &op, int nv, Precision p, int restart) {
    if (p != PREC_MIXED || !op.mgd || op.block4 || op.A.W > 8 || !op.a32 || nv < LSG_MINRHS || restart < 2) return false;
    if (op.mg.nu1 != 1 || op.mg.nu2 != 1 || op.mg.nlev < 2 || op.mg.nlev > MG_MAXLEV || !op.mg.cinv32) return false;
    for (int l = 0; l < op.mg.nlev; ++l) {
        const MgLevelDev &D = op.mg.lev[l];
        if (D.W > 8 || !D.a32 || !D.d32) return false;
        if (l + 1 < op.mg.nlev && (!D.pc || !D.pw32 || !D.rf || !D.rw32)) return false;
    }
    return (long long)op.A.n * ((nv + 31) / 32 * 8) < (1LL << 31);
}

unsigned lsg_blocks(long long work, unsigned resident = 0) {
    long long b = (work + 255) / 256;
    long long cap = 4LL * sm_count();
    if (resident > 0 && resident < cap) cap = resident;   // no partial second wave
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (unsigned)b;
}

// resident grids of the register-heavy lockstep multigrid kernels (80 registers:
// 3 blocks of 256 threads per SM, fewer than the 4 per SM the other kernels
// launch with), queried once at operator creation like ls_grids.  Capping
// their grid at one resident wave instead of 4 blocks per SM avoids a second,
// partial wave.
struct LsgGrids {
    unsigned down, smooth, spmm;
};
const LsgGrids &lsg_grids() {
    static std::once_flag once;
    static LsgGrids g;
    std::call_once(once, [] {
        g.down = resident_grid(k_mg_down, 0);
        g.smooth = resident_grid(k_mg_smooth, 0);
        g.spmm = resident_grid(k_lsg_spmm, 0);
    });
    return g;
}

cudaError_t lsg_solve(const DevSolveOp &op, const double *B, double *X, int nv, int ld, int restart, int max_iter,
                      double tol, double inner_rtol, char *w, GmresStats *st, double mg_row_bytes, cudaStream_t s) {
    const int lsg_maxc = LSG_MAXC;
    const LsgLayout Lo = lsg_layout(op, nv, restart);
    const int n = op.A.n, W = op.A.W, nvp = Lo.nvp, m = Lo.m, nlev = op.mg.nlev, last = nlev - 1;
    LsgParams P;
    memset(&P, 0, sizeof P);
    P.n = n; P.nv = nv; P.nvp = nvp; P.q4 = nvp / 4; P.m = m; P.nlev = nlev; P.W = W; P.RB = Lo.RB; P.nbx = Lo.nbx;
    P.ld = ld; P.max_iter = max_iter; P.tol = tol; P.inner_rtol = inner_rtol;
    // algorithmic bytes per member and row (the per-member solver's model, FP32 vectors)
    P.step_row_bytes = W * 8.0 + 4.0 * 6.0 + mg_row_bytes;
    P.resid_row_bytes = W * 12.0 + 24.0;
    P.omega = (float)op.mg.omega;
    P.col = op.A.col; P.a32 = op.a32;
    for (int l = 0; l < nlev; ++l) {
        const MgLevelDev &D = op.mg.lev[l];
        LsgLevel &E = P.lev[l];
        E.n = D.n; E.W = D.W; E.Wr = D.Wr; E.col = D.col; E.a = D.a32; E.d = D.d32;
        E.pc = D.pc; E.pw = D.pw32; E.rf = D.rf; E.rw = D.rw32;
        const size_t lv = (((size_t)D.n * nvp * 4) + 255) & ~size_t(255);
        E.x = (float *)(w + Lo.lev[l]); E.xo = (float *)(w + Lo.lev[l] + lv);
        E.r = (float *)(w + Lo.lev[l] + 2 * lv); E.b = (float *)(w + Lo.lev[l] + 3 * lv);
    }
    P.nc = op.mg.nc; P.cinv = op.mg.cinv32;
    // the small levels: from the first with <= LSG_SMALL rows whose levels fit in shared memory
    int lc = last;
    for (int l = last; l >= 0; --l) {
        size_t rows = 0;
        for (int k = l; k <= last; ++k) rows += (size_t)op.mg.lev[k].n;
        if (op.mg.lev[l].n > LSG_SMALL || 64 * rows > LSG_SMALL_SMEM) break;
        lc = l;
    }
    size_t small_rows = 0;
    for (int k = lc; k <= last; ++k) small_rows += (size_t)op.mg.lev[k].n;
    const size_t small_smem = 64 * small_rows;
    P.lc = lc;
    P.levs = (LsgLevel *)(w + Lo.levs);
    P.B = B; P.X = X;
    P.V = (float *)(w + Lo.V); P.Z = (float *)(w + Lo.Z); P.w = (float *)(w + Lo.w);
    P.R = (double *)(w + Lo.R); P.rpart = (double *)(w + Lo.rpart); P.bpart = (double *)(w + Lo.bpart);
    P.nrm = (double *)(w + Lo.nrm); P.dpart = (double *)(w + Lo.dpart); P.npart = (double *)(w + Lo.npart);
    P.hcol = (double *)(w + Lo.hcol); P.H = (double *)(w + Lo.H); P.cs = (double *)(w + Lo.cs);
    P.sn = (double *)(w + Lo.sn); P.g = (double *)(w + Lo.g); P.hv = (float *)(w + Lo.hv); P.yv = (float *)(w + Lo.yv);
    P.bnorm = (double *)(w + Lo.bnorm); P.beta_prev = (double *)(w + Lo.beta_prev);
    P.target = (double *)(w + Lo.target); P.relv = (double *)(w + Lo.relv);
    P.scale = (float *)(w + Lo.scale); P.vscale = (float *)(w + Lo.vscale);
    int *ip = (int *)(w + Lo.ints);
    P.stt = ip; P.arn = ip + nvp; P.jl = ip + 2 * nvp; P.iters = ip + 3 * nvp; P.cycles = ip + 4 * nvp;
    P.zerox = ip + 5 * nvp; P.cnt = ip + 6 * nvp; P.done = P.cnt + m + 1;
    P.st = st;
    cudaError_t e;
    if ((e = cudaMemsetAsync(st, 0, sizeof(GmresStats), s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(P.done, 0, sizeof(int), s)) != cudaSuccess) return e;
    static std::once_flag smem_once;
    static cudaError_t smem_err = cudaSuccess;
    std::call_once(smem_once, [] {
        smem_err = cudaFuncSetAttribute((const void *)k_mg_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)LSG_SMALL_SMEM);
    });
    if (smem_err != cudaSuccess) return smem_err;
    if (small_smem > LSG_SMALL_SMEM) return cudaErrorInvalidValue;
    long long launches = 0;
    const dim3 rgrid((unsigned)Lo.nbx, (unsigned)((nv + LS_MG - 1) / LS_MG));
    const unsigned rblocks = resid_grid(W, (long long)rgrid.x * rgrid.y);
    k_lsg_levels<<<1, 32, 0, s>>>(P);
    k_ls_sq<<<rgrid, 256, 0, s>>>(B, n, ld, nv, P.bpart);
    launches += 2;
    const unsigned gsmall = (unsigned)std::min(P.q4, 4 * sm_count());
    const unsigned gn = lsg_blocks((long long)n * P.q4, lsg_grids().spmm);
    const dim3 red_grid((unsigned)Lo.RB, (unsigned)(nvp / 32));
    const unsigned tiles = lsg_blocks((long long)((n + 31) / 32) * (nvp / 32) * 256);
    P.maxc = lsg_maxc;
    for (int c = 0; c <= lsg_maxc; ++c) {
        switch (W) {
        case 6: k_ls_resid<6><<<rblocks, 256, 0, s>>>(op.A.col, op.A.val, n, B, X, ld, P.R, nv, P.rpart, Lo.nbx, P.done); break;
        case 7: k_ls_resid<7><<<rblocks, 256, 0, s>>>(op.A.col, op.A.val, n, B, X, ld, P.R, nv, P.rpart, Lo.nbx, P.done); break;
        default: k_ls_resid<8><<<rblocks, 256, 0, s>>>(op.A.col, op.A.val, n, B, X, ld, P.R, nv, P.rpart, Lo.nbx, P.done); break;
        }
        k_ls_nrm<<<(nv + NWARP - 1) / NWARP, 256, 0, s>>>(P.rpart, P.bpart, Lo.nbx, P.nrm, nv, P.done);
        k_lsg_begin<<<1, 256, 0, s>>>(P, c);
        launches += 3;
        if (c == 0) { k_lsg_zero<<<lsg_blocks((long long)nv * n), 256, 0, s>>>(P); ++launches; }
        if (c == lsg_maxc) break;
        k_lsg_v0<<<tiles, 256, 0, s>>>(P);
        ++launches;
        for (int j = 0; j < m; ++j) {
            // v_0 comes from k_lsg_v0; v_j (j > 0) = w / ||w|| is formed by the
            // first kernel of the V-cycle, which stores it
            float *vj = P.V + (size_t)j * n * nvp;
            const float *src0 = j == 0 ? vj : P.w;
            float *vout0 = j == 0 ? nullptr : vj;
            float *zj = P.Z + (size_t)j * n * nvp;
            for (int l = 0; l < lc; ++l) {
                k_mg_down<<<lsg_blocks((long long)P.lev[l].n * P.q4, lsg_grids().down), 256, 0, s>>>(
                    P, P.lev[l], l == 0 ? src0 : P.lev[l].b, l == 0 ? vout0 : nullptr, j);
                if (l + 1 < lc)
                    k_mg_restrict<<<lsg_blocks((long long)P.lev[l + 1].n * P.q4), 256, 0, s>>>(P, P.lev[l], P.lev[l + 1], j);
                launches += l + 1 < lc ? 2 : 1;
            }
            k_mg_small<<<gsmall, MG_SMALL_TB, small_smem, s>>>(P, src0, lc == 0 ? vout0 : nullptr, lc == 0 ? zj : P.lev[lc].x, j);
            ++launches;
            for (int l = lc - 1; l >= 0; --l) {
                const float *xc = (l + 1 == lc) ? P.lev[lc].x : P.lev[l + 1].xo;
                k_mg_prolong<<<lsg_blocks((long long)P.lev[l].n * P.q4), 256, 0, s>>>(P, P.lev[l], xc, j);
                float *out = l == 0 ? zj : P.lev[l].xo;
                k_mg_smooth<<<lsg_blocks((long long)P.lev[l].n * P.q4, lsg_grids().smooth), 256, 0, s>>>(
                    P, P.lev[l], l == 0 ? vj : P.lev[l].b, out, j);
                launches += 2;
            }
            k_lsg_spmm<<<gn, 256, 0, s>>>(P, j);
            k_lsg_dot<<<red_grid, 256, 0, s>>>(P, j);
            k_lsg_hsum<<<(unsigned)((nv * (j + 1) + NWARP - 1) / NWARP), 256, 0, s>>>(P, j);
            k_lsg_update<<<red_grid, 256, 0, s>>>(P, j);
            k_lsg_givens<<<(unsigned)((nv + NWARP - 1) / NWARP), 256, 0, s>>>(P, j);
            launches += 5;
        }
        k_lsg_solve<<<lsg_blocks(nvp), 256, 0, s>>>(P);
        k_lsg_correct<<<tiles, 256, 0, s>>>(P);
        launches += 2;
    }
    g_kernel_launches += launches;
    return cudaGetLastError();
}

}  // namespace

// The kernels may use all the opt-in shared memory; set once per kernel, so
// that threads launching with different sizes never race on the attribute.
static cudaError_t allow_smem(Precision prec, bool multi = false) {
    static std::once_flag once[4];
    static cudaError_t err[4] = {cudaSuccess, cudaSuccess, cudaSuccess, cudaSuccess};
    const int k = (prec == PREC_MIXED ? 1 : 0) + (multi ? 2 : 0);
    std::call_once(once[k], [k] {
        void *fn = k == 0 ? (void *)gmres_kernel<double, false> : k == 1 ? (void *)gmres_kernel<float, false>
                 : k == 2 ? (void *)gmres_kernel<double, true> : (void *)gmres_kernel<float, true>;
        int dev = 0, optin = 0;
        cudaFuncAttributes fa;
        if ((err[k] = cudaGetDevice(&dev)) != cudaSuccess) return;
        if ((err[k] = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess)
            return;
        if ((err[k] = cudaFuncGetAttributes(&fa, fn)) != cudaSuccess) return;
        err[k] = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      optin - (int)fa.sharedSizeBytes);
    });
    return err[k];
}

// The launch path gmres_solve takes for these right-hand sides: the shape
// (given, else the tuned one; environment overrides) decides between the
// persistent kernels and the lockstep launches.  sh_out: the shape used.
SolvePath choose_path(const DevSolveOp &op, int nv, int m, Precision prec, bool no_alloc, const SolveShape *shape,
                      SolveShape *sh_out) {
    SolveShape sh;
    if (shape) sh = *shape;
    else tune_get_solve(solve_family(op), op.A.n, prec, nv, &sh);
    if (getenv("PHG_ROWS_PER_BLOCK")) sh.rpb = env_int("PHG_ROWS_PER_BLOCK", 256);
    if (getenv("PHG_CHEB_LOCKSTEP") && !env_int("PHG_CHEB_LOCKSTEP", 1)) sh.path = 0;
    if (sh_out) *sh_out = sh;
    if (no_alloc) return SolvePath::Persistent;
    if (uses_cheb(op, m)) {
        const bool ls = sh.path == 1 ? nv >= LS_MIN_TUNED : (sh.path == 0 ? false : nv >= LS_MIN_RHS);
        return prec == PREC_MIXED && ls ? SolvePath::ChebLockstep : SolvePath::Persistent;
    }
    if (lsg_applicable(op, nv, prec, m) &&
        (sh.path == 1 || (sh.path == -1 && nv >= LSG_DEFAULT_RHS && op.A.n >= LSG_DEFAULT_ROWS)))
        return SolvePath::MgLockstep;
    return SolvePath::Persistent;
}

// workspace of the path the solve will take (the lockstep multigrid path
// needs only its own 2m + 1 interleaved vectors; the others the layout above)
size_t gmres_work_bytes(const DevSolveOp &op, int nv, int m, Precision p, const SolveShape *shape) {
    if (choose_path(op, nv, m, p, false, shape, nullptr) == SolvePath::MgLockstep) return lsg_layout(op, nv, m).total;
    return layout(op, nv, m, p).total;
}

cudaError_t gmres_solve(const DevSolveOp &op, const double *B, double *X, int nv, int ld,
                        int m, int max_iter, double tol, Precision prec,
                        void *work, GmresStats *stats_dev, cudaStream_t s, bool no_alloc, int max_sms,
                        const SolveShape *shape, long long wait_limit) {
    if (m < 1 || m > MAXM || nv < 1) return cudaErrorInvalidValue;
    const int n = op.A.n;
    Params p;
    const size_t es = prec == PREC_MIXED ? 4 : 8;
    const bool cheb = uses_cheb(op, m);
    SolveShape sh;
    const SolvePath path = choose_path(op, nv, m, prec, no_alloc, shape, &sh);
    const bool lockstep = path == SolvePath::ChebLockstep;
    // ensembles of the multigrid Laplacian in the mixed path: lockstep launches
    if (path == SolvePath::MgLockstep) {
        const char *ev = getenv("PHG_INNER_RTOL");
        double rowb = 0.0;
        for (int l = 0; l < op.mg.nlev; ++l) {
            const MgLevelDev &Lv = op.mg.lev[l];
            rowb += (double)Lv.n / (double)n * ((op.mg.nu1 + op.mg.nu2 + 1) * (Lv.W * 8.0 + 16.0) + 16.0);
        }
        return lsg_solve(op, B, X, nv, ld, m, max_iter, tol, ev ? atof(ev) : INNER_RTOL, (char *)work, stats_dev,
                         rowb, s);
    }
    // ensembles in the mixed path: all right-hand sides in lockstep
    if (cheb && prec == PREC_MIXED && lockstep && !no_alloc) {
        const char *ev = getenv("PHG_INNER_RTOL");
        cudaError_t e0 = cudaMemsetAsync(stats_dev, 0, sizeof(GmresStats), s);
        if (e0 != cudaSuccess) return e0;
        e0 = cheb_lockstep(op, B, X, nv, ld, tol, ev ? atof(ev) : INNER_RTOL, (char *)work,
                           layout(op, nv, m, prec), stats_dev, s);
        if (e0 != cudaErrorNotSupported) return e0;
    }
    // cluster tail of the V-cycle: the levels [ncl, nred) in the group's first
    // cluster (needs a group of at least one whole cluster, see below)
    const bool want_tail = !cheb && op.mgd && op.mg.cl_size > 1 && op.mg.ncl < op.mg.nred;
    const size_t smem = cheb ? sizeof(double) * (4 + 2 * CHEB_KMAX)
                             : smem_gmres_bytes() +
                                   (op.mgd ? es * (op.mg.red_elems + (want_tail ? op.mg.cl_elems : 0)) : 0) + 16;
    if (smem > 227 * 1024) return cudaErrorInvalidValue;
    void *fn = cheb ? (prec == PREC_MIXED ? (void *)cheb_kernel<float> : (void *)cheb_kernel<double>)
                    : (prec == PREC_MIXED ? (void *)gmres_kernel<float, false> : (void *)gmres_kernel<double, false>);
    cudaError_t e = cheb ? cudaSuccess : allow_smem(prec);
    if (e != cudaSuccess) return e;
    int per = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, BLOCK, smem);
    if (e != cudaSuccess) return e;
    if (per < 1) return cudaErrorInvalidConfiguration;
    const int sms = (max_sms > 0 && max_sms < sm_count()) ? max_sms : sm_count();
    const int cap = sms * per;
    // as many right-hand sides in flight as there are blocks; the blocks are
    // shared out evenly, but no block gets fewer than `rpb` rows
    const int rpb = sh.rpb > 0 ? sh.rpb : 256;
    int groups = nv < cap ? nv : cap;
    if (groups > GROUPS_CAP) groups = GROUPS_CAP;
    int G = cap / groups;
    const int Gmax = (n + rpb - 1) / (rpb > 32 ? rpb : 32);
    if (G > Gmax) G = Gmax;
    if (G < 1) G = 1;
    // groups of whole clusters (the first one runs the tail) when the grid
    // of clusters is co-resident; otherwise the plain launch
    int CS = 0;
    if (want_tail && G >= op.mg.cl_size) {
        CS = op.mg.cl_size;
        G = G / CS * CS;
        cudaLaunchConfig_t qc = {};
        cudaLaunchAttribute qa[1];
        qa[0].id = cudaLaunchAttributeClusterDimension;
        qa[0].val.clusterDim.x = CS; qa[0].val.clusterDim.y = 1; qa[0].val.clusterDim.z = 1;
        qc.gridDim = dim3(groups * G);
        qc.blockDim = dim3(BLOCK);
        qc.dynamicSmemBytes = smem;
        qc.attrs = qa;
        qc.numAttrs = 1;
        int nclu = 0;
        if (cudaOccupancyMaxActiveClusters(&nclu, fn, &qc) != cudaSuccess || (long long)nclu * CS < (long long)groups * G) {
            cudaGetLastError();
            CS = 0;
        }
    }
    Layout L = layout(op, nv, m, prec);
    char *w = (char *)work;
    p.op = op; p.B = B; p.X = X; p.n = n; p.nv = nv; p.ld = ld; p.m = m; p.max_iter = max_iter; p.tol = tol;
    p.V = w + L.v; p.Z = w + L.z; p.Wv = w + L.w; p.R = (double *)(w + L.r);
    p.vstride = (size_t)(cheb ? 4 : m + 1) * n;
    p.mgbuf = w + L.mg;
    p.group_elems = block_group_elems(op);
    {
        const char *e = getenv("PHG_INNER_RTOL");
        p.inner_rtol = e ? atof(e) : INNER_RTOL;
    }
    p.cheb_k = 0;
    p.cheb_lg = p.cheb_ls = 0.0;
    if (cheb) {
        // steps for an error reduction eps (residual: one more factor kappa)
        const double lo = op.cheb_lmin, hi = op.cheb_lmax;
        const double kappa = hi / lo, sq = sqrt(kappa), sigma = (sq - 1.0) / (sq + 1.0);
        const double eps = prec == PREC_MIXED ? p.inner_rtol : fmax(0.25 * tol, 1e-15);
        int K = (int)ceil(log(2.0 * kappa / eps) / log(1.0 / sigma)) + 1;
        K = K < 2 ? 2 : (K > CHEB_KMAX ? CHEB_KMAX : K);
        const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), s1 = theta / delta;
        p.cheb_k = K;
        p.cheb_lg = log(2.0 * kappa);
        p.cheb_ls = log(1.0 / sigma);
        p.cheb_c0 = 1.0 / theta;
        double rho_prev = 1.0 / s1;
        p.cheb_ca[0] = p.cheb_cb[0] = 0.0;
        for (int k = 1; k < K; ++k) {
            const double rho = 1.0 / (2.0 * s1 - rho_prev);
            p.cheb_ca[k] = rho * rho_prev;
            p.cheb_cb[k] = 2.0 * rho / delta;
            rho_prev = rho;
        }
    }
    p.part = (double *)(w + L.part);
    p.bar = (unsigned *)(w + L.bar); p.err = (int *)(w + L.err); p.stats = stats_dev;
    p.groups = groups; p.G = G;
    p.wait_limit = wait_limit > 0 ? wait_limit : SPIN_LIMIT;
    p.cluster = CS;
    p.ccnt = (unsigned long long *)(w + L.ccnt);
    p.nseg = 0;
    p.mg_row_bytes = 0.0;
    if (op.mgd)
        for (int l = 0; l < op.mg.nlev; ++l) {
            const MgLevelDev &Lv = op.mg.lev[l];
            const double frac = (double)Lv.n / (double)n * (op.block4 ? 2.0 : 1.0);
            p.mg_row_bytes += frac * ((op.mg.nu1 + op.mg.nu2 + 1) * (Lv.W * (4.0 + es) + 4.0 * es) + 4.0 * es);
        }
    static std::once_flag timers_once;
    static long long *timers = nullptr;
    const bool timing = !no_alloc && getenv("PHG_PHASE_TIMING") != nullptr;
    if (timing) std::call_once(timers_once, [] { cudaMalloc(&timers, sizeof(long long) * T_NPHASE); });
    p.timers = timing ? timers : nullptr;
    if (p.timers) cudaMemsetAsync(timers, 0, sizeof(long long) * T_NPHASE, s);
    if ((e = cudaMemsetAsync(w + L.bar, 0, L.total - L.bar, s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(stats_dev, 0, sizeof(GmresStats), s)) != cudaSuccess) return e;
    void *args[] = {&p};
    // cooperative (all blocks co-resident) through the attribute form, which
    // stream capture records as a cooperative kernel node
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute coop[2];
    coop[0].id = cudaLaunchAttributeCooperative;
    coop[0].val.cooperative = 1;
    coop[1].id = cudaLaunchAttributeClusterDimension;
    coop[1].val.clusterDim.x = CS; coop[1].val.clusterDim.y = 1; coop[1].val.clusterDim.z = 1;
    cfg.gridDim = dim3(groups * G);
    cfg.blockDim = dim3(BLOCK);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = coop;
    cfg.numAttrs = CS > 0 ? 2 : 1;
    e = cudaLaunchKernelExC(&cfg, fn, args);
    if (e != cudaSuccess) return e;
    g_kernel_launches += 2;
    // a barrier timeout lands in stats->status (2)
    fold_err<<<1, 1, 0, s>>>(p.err, stats_dev);
    if (p.timers) {   // debug: print block 0's phase cycles for this launch
        long long h[T_NPHASE];
        GmresStats st;
        cudaMemcpyAsync(h, timers, sizeof(h), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(&st, stats_dev, sizeof(st), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        static const char *nm[T_NPHASE] = {"resid", "vcycle", "spmv_dot", "dot_sum", "update", "norm_sum",
                                           "givens", "corr", "barrier_wait", "barriers", "total"};
        fprintf(stderr, "[phases] n=%d nv=%d groups=%d G=%d mg=%d iters=%d cycles=%d |", n, nv, groups, G,
                op.mgd ? op.mg.nlev : 0, st.iters, st.cycles);
        for (int k = 0; k < T_NPHASE; ++k) fprintf(stderr, " %s=%lld", nm[k], k == T_BARRIERS ? h[k] : h[k] / 1000);
        fprintf(stderr, " (kcycles)\n");
    }
    return cudaGetLastError();
}

// ------------------------------------------------ several mesh levels ---
// Workspace of a multi-operator launch: the per-RHS vectors of every segment
// back to back, one group scratch sized for the largest hierarchy.
struct MultiLayout {
    size_t v, z, w, r, mg, part, bar, err, ccnt, total;
    size_t voff[MAXSEG], zoff[MAXSEG], woff[MAXSEG], roff[MAXSEG];
};

static MultiLayout multi_layout(const DevSolveOp *const *ops, const int *nvk, int nseg, int m, Precision prec) {
    MultiLayout L{};
    const size_t es = prec == PREC_MIXED ? 4 : 8;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    size_t ev = 0, ez = 0, ew = 0, er = 0, ge = 0;
    int nv = 0;
    for (int k = 0; k < nseg; ++k) {
        const size_t n = (size_t)ops[k]->A.n;
        L.voff[k] = ev; L.zoff[k] = ez; L.woff[k] = ew; L.roff[k] = er;
        ev += (size_t)nvk[k] * (m + 1) * n;
        ez += (size_t)nvk[k] * m * n;
        ew += (size_t)nvk[k] * n;
        er += (size_t)nvk[k] * n;
        ge = std::max(ge, ops[k]->mg.group_elems);
        nv += nvk[k];
    }
    const int groups = nv < GROUPS_CAP ? nv : GROUPS_CAP;
    L.v = 0;
    L.z = L.v + al(es * ev);
    L.w = L.z + al(es * ez);
    L.r = L.w + al(es * ew);
    L.mg = L.r + al(8 * er);
    L.part = L.mg + al(es * ge * (size_t)groups);
    L.bar = L.part + al(8 * (size_t)4096 * 2 * (MAXM + 2));
    L.err = L.bar + al(8 * (size_t)GROUPS_CAP);
    L.ccnt = L.err + 256;
    L.total = L.ccnt + al(8 * (size_t)GROUPS_CAP);
    return L;
}

size_t gmres_multi_work_bytes(const DevSolveOp *const *ops, const int *nvk, int nseg, int m, Precision prec) {
    if (nseg < 1 || nseg > MAXSEG) return 0;
    return multi_layout(ops, nvk, nseg, m, prec).total;
}

cudaError_t gmres_solve_multi(const DevSolveOp *const *ops, const int *nvk, const double *const *B, double *const *X,
                              const int *ldk, int nseg, int m, int max_iter, double tol, Precision prec, void *work,
                              GmresStats *stats_dev, cudaStream_t s, int max_sms, long long wait_limit) {
    if (nseg < 1 || nseg > MAXSEG || m < 1 || m > MAXM) return cudaErrorInvalidValue;
    int nv = 0, nmax = 0;
    size_t red = 0, ge = 0;
    for (int k = 0; k < nseg; ++k) {
        const DevSolveOp &op = *ops[k];
        if (!op.mgd || op.block4 || nvk[k] < 1) return cudaErrorInvalidValue;   // multigrid Laplacians only
        nv += nvk[k];
        nmax = std::max(nmax, op.A.n);
        red = std::max(red, op.mg.red_elems);
        ge = std::max(ge, op.mg.group_elems);
    }
    const size_t es = prec == PREC_MIXED ? 4 : 8;
    const size_t smem = smem_gmres_bytes() + es * red + 16;
    if (smem > 227 * 1024) return cudaErrorInvalidValue;
    void *fn = prec == PREC_MIXED ? (void *)gmres_kernel<float, true> : (void *)gmres_kernel<double, true>;
    cudaError_t e = allow_smem(prec, true);
    if (e != cudaSuccess) return e;
    int per = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, BLOCK, smem)) != cudaSuccess) return e;
    if (per < 1) return cudaErrorInvalidConfiguration;
    const int sms = (max_sms > 0 && max_sms < sm_count()) ? max_sms : sm_count();
    int cap = sms * per;
    if (cap < nseg) cap = nseg;   // one block per mesh at least (an SM cap below that is exceeded)
    // the resident blocks split between the segments in proportion to their
    // work (right-hand sides x rows), at least one block each; within a
    // segment as the single-operator launch does it: as many groups as
    // right-hand sides fit, then groups of up to one block per 256 rows
    int bk[MAXSEG], gk[MAXSEG], Gk[MAXSEG];
    {
        double tw = 0.0;
        for (int k = 0; k < nseg; ++k) tw += (double)nvk[k] * ops[k]->A.n;
        int used = 0;
        for (int k = 0; k < nseg; ++k) {
            bk[k] = std::max(1, (int)((double)cap * nvk[k] * ops[k]->A.n / tw));
            used += bk[k];
        }
        while (used > cap) {   // rounding up the smallest shares: take back from the largest
            int kmax = 0;
            for (int k = 1; k < nseg; ++k) if (bk[k] > bk[kmax]) kmax = k;
            --bk[kmax];
            --used;
        }
        for (int k = 0; k < nseg; ++k) {
            gk[k] = std::min(nvk[k], bk[k]);
            Gk[k] = std::max(1, std::min(bk[k] / gk[k], (ops[k]->A.n + 255) / 256));
        }
    }
    int groups = 0, blocks = 0;
    for (int k = 0; k < nseg; ++k) { groups += gk[k]; blocks += gk[k] * Gk[k]; }
    if (groups > GROUPS_CAP || blocks > cap) return cudaErrorInvalidConfiguration;
    int G = 1;
    for (int k = 0; k < nseg; ++k) G = std::max(G, Gk[k]);
    (void)nmax;
    const MultiLayout L = multi_layout(ops, nvk, nseg, m, prec);
    char *w = (char *)work;
    Params p;
    p.op = *ops[0];   // launch bookkeeping only: every right-hand side reads its segment
    p.B = B[0]; p.X = X[0]; p.n = ops[0]->A.n; p.nv = nv; p.ld = ldk[0]; p.m = m; p.max_iter = max_iter;
    p.tol = tol;
    p.V = w + L.v; p.Z = w + L.z; p.Wv = w + L.w; p.R = (double *)(w + L.r);
    p.vstride = 0;
    p.mgbuf = w + L.mg;
    p.group_elems = ge;
    {
        const char *ev = getenv("PHG_INNER_RTOL");
        p.inner_rtol = ev ? atof(ev) : INNER_RTOL;
    }
    p.cheb_k = 0;
    p.cheb_lg = p.cheb_ls = 0.0;
    p.part = (double *)(w + L.part);
    p.bar = (unsigned *)(w + L.bar); p.err = (int *)(w + L.err); p.stats = stats_dev;
    p.groups = groups; p.G = G;
    p.wait_limit = wait_limit > 0 ? wait_limit : SPIN_LIMIT;
    p.cluster = 0;
    p.ccnt = (unsigned long long *)(w + L.ccnt);
    p.mg_row_bytes = 0.0;
    p.timers = nullptr;
    p.nseg = nseg;
    int v0 = 0, blk0 = 0, gbase = 0;
    for (int k = 0; k < MAXSEG; ++k) p.seg[k] = MultiSeg{};
    for (int k = 0; k < nseg; ++k) {
        const DevSolveOp &op = *ops[k];
        MultiSeg &S = p.seg[k];
        S.v0 = v0; S.n = op.A.n; S.W = op.A.W; S.ld = ldk[k];
        S.nv = nvk[k];
        S.blk0 = blk0; S.G = Gk[k]; S.groups = gk[k]; S.gbase = gbase;
        blk0 += gk[k] * Gk[k];
        gbase += gk[k];
        S.col = op.A.col; S.aval = op.A.val; S.sval64 = op.A.val; S.sval32 = op.a32; S.dinv = op.dinv;
        S.mgd = op.mgd;
        S.B = B[k]; S.X = X[k];
        S.voff = L.voff[k]; S.zoff = L.zoff[k]; S.woff = L.woff[k]; S.roff = L.roff[k];
        S.mg_row_bytes = 0.0;
        for (int l = 0; l < op.mg.nlev; ++l) {
            const MgLevelDev &Lv = op.mg.lev[l];
            S.mg_row_bytes += (double)Lv.n / (double)op.A.n *
                              ((op.mg.nu1 + op.mg.nu2 + 1) * (Lv.W * (4.0 + es) + 4.0 * es) + 4.0 * es);
        }
        v0 += nvk[k];
    }
    if ((e = cudaMemsetAsync(w + L.bar, 0, L.total - L.bar, s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(stats_dev, 0, sizeof(GmresStats), s)) != cudaSuccess) return e;
    void *args[] = {&p};
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute coop[1];
    coop[0].id = cudaLaunchAttributeCooperative;
    coop[0].val.cooperative = 1;
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(BLOCK);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = coop;
    cfg.numAttrs = 1;
    if ((e = cudaLaunchKernelExC(&cfg, fn, args)) != cudaSuccess) return e;
    g_kernel_launches += 2;
    fold_err<<<1, 1, 0, s>>>(p.err, stats_dev);
    return cudaGetLastError();
}

void lockstep_prepare() {
    (void)ls_grids();
    (void)lsg_grids();
}

}  // namespace phg
