#include <cstdint>
// phg_kernels.cu -- operator applies and fused elementwise kernels.
//
// This file is compiled with -fmad=false: every product and sum below is
// rounded separately, in the order written, so an FP64 apply on the GPU
// returns the same bits as the reference's CPU CSR product
// (ascending columns, starting from 0.0) and the elementwise formulas of the
// time steps round exactly like the reference's vec_sum1 / vec_sum2 calls.
//
// All kernels take nv members stored member-major (x[v * ld + i]).
#include <atomic>

#include "phg_kernels.cuh"

namespace phg {

std::atomic<long long> g_kernel_launches{0};

namespace {
constexpr int TB = 256;

inline unsigned grid_for(long long work) {
    long long b = (work + TB - 1) / TB;
    if (b < 1) b = 1;
    if (b > 152LL * 64) b = 152LL * 64;
    return (unsigned)b;
}

// ascending-column row sum; loads are issued together, the sum keeps the order
__device__ __forceinline__ double row_sum(const DevEll &A, const double *x, const int *imap, int i) {
    double s = 0.0;
    const int n = A.n;
    if (A.W <= 8) {
        int c[8];
        double a[8], xv[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < A.W) { c[k] = __ldg(&A.col[(size_t)k * n + i]); a[k] = __ldg(&A.val[(size_t)k * n + i]); }
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < A.W) xv[k] = imap ? x[imap[c[k]]] : x[c[k]];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < A.W) s += a[k] * xv[k];
        return s;
    }
    for (int k = 0; k < A.W; ++k) {
        int c = __ldg(&A.col[(size_t)k * n + i]);
        double xv = imap ? x[imap[c]] : x[c];
        s += __ldg(&A.val[(size_t)k * n + i]) * xv;
    }
    return s;
}

__device__ __forceinline__ double cols_sum(const DevCols &C, const double *xb, const int *bmap, int i) {
    double s = 0.0;
    if (!C.ptr || !xb) return s;
    for (int k = C.ptr[i]; k < C.ptr[i + 1]; ++k) {
        int c = C.col[k];
        s += C.val[k] * (bmap ? xb[bmap[c]] : xb[c]);
    }
    return s;
}

__global__ void k_apply(DevEll A, DevCols C, const double *xin, int ldx, const int *imap,
                        const double *xb, int ldb, const int *bmap, double *y, int ldy, int nv) {
    const long long total = (long long)nv * A.n;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        int v = (int)(t / A.n), i = (int)(t % A.n);
        double s = row_sum(A, xin + (size_t)v * ldx, imap, i);
        if (C.ptr && xb) s = s + cols_sum(C, xb + (size_t)v * ldb, bmap, i);
        y[(size_t)v * ldy + i] = s;
    }
}

// the 8 derivative right-hand sides of SphereJacobian::calc2
// (src/sjacobian.cpp:136-362), out[(v * 8 + k) * ldo + i]:
//   k: 0 D2c u, 1 D1 v, 2 D1c u, 3 D2 v, 4 D2 u, 5 D1c v, 6 D1 u, 7 D2c v
__global__ void k_jac_rhs(JacOps J, const double *u, const double *w, int ld, const int *imap,
                          const int *bmap, double *out, int ldo, int nv) {
    const int n = J.d1.n;
    const long long total = (long long)nv * n;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        int v = (int)(t / n), i = (int)(t % n);
        const double *fu = u + (size_t)v * ld, *fv = w + (size_t)v * ld;
        double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int k = 0; k < J.d1.W; ++k) {
            size_t e = (size_t)k * n + i;
            int c = __ldg(&J.d1.col[e]);
            int cc = imap ? imap[c] : c;
            double xu = fu[cc], xv = fv[cc];
            double a1 = __ldg(&J.d1.val[e]), a2 = __ldg(&J.d2.val[e]);
            double c1 = __ldg(&J.d1c.val[e]), c2 = __ldg(&J.d2c.val[e]);
            s[0] += c2 * xu; s[1] += a1 * xv; s[2] += c1 * xu; s[3] += a2 * xv;
            s[4] += a2 * xu; s[5] += c1 * xv; s[6] += a1 * xu; s[7] += c2 * xv;
        }
        const double *bu = fu, *bv = fv;
        double b[8];
        b[0] = cols_sum(J.d2cb, bu, bmap, i); b[1] = cols_sum(J.d1b, bv, bmap, i);
        b[2] = cols_sum(J.d1cb, bu, bmap, i); b[3] = cols_sum(J.d2b, bv, bmap, i);
        b[4] = cols_sum(J.d2b, bu, bmap, i); b[5] = cols_sum(J.d1cb, bv, bmap, i);
        b[6] = cols_sum(J.d1b, bu, bmap, i); b[7] = cols_sum(J.d2cb, bv, bmap, i);
        for (int k = 0; k < 8; ++k) out[((size_t)v * 8 + k) * ldo + i] = b[k] + s[k];
    }
}

// jac = 1/4 sum of the four splittings; optional F = FC[inner] - jac
__global__ void k_jac_combine(const double *d, int ldd, int n, double *jac, int ldj,
                              const double *FC, int ldf, const int *inner, int nv) {
    const long long total = (long long)nv * n;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        int v = (int)(t / n), i = (int)(t % n);
        const double *q = d + (size_t)v * 8 * ldd;
        double c2u = q[0 * ldd + i], a1v = q[1 * ldd + i], c1u = q[2 * ldd + i], a2v = q[3 * ldd + i];
        double a2u = q[4 * ldd + i], c1v = q[5 * ldd + i], a1u = q[6 * ldd + i], c2v = q[7 * ldd + i];
        double j1 = c2u * a1v - c1u * a2v;
        double j2 = a2u * c1v - a1u * c2v;
        double j3 = c2u * a1v - a1u * c2v;
        double j4 = a2u * c1v - c1u * a2v;
        double s = j1;
        s = s + j2;
        s = s + j3;
        s = s + j4;
        double r = 0.25 * s;
        if (FC) r = FC[(size_t)v * ldf + (inner ? inner[i] : i)] - r;
        jac[(size_t)v * ldj + i] = r;
    }
}

// u[p] = boundary ? (bnd ? bnd[p2io[p]] : 0) : p[p2io[p]]   (src/proj.cpp:49-75)
__global__ void k_p2u(double *u, int ldu, const double *p, int ldp, const double *bnd, int ldb,
                      const int *p2io, const int *isb, int V, int nv) {
    const long long total = (long long)nv * V;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        int v = (int)(t / V), i = (int)(t % V);
        double r;
        if (isb[i]) r = bnd ? bnd[(size_t)v * ldb + p2io[i]] : 0.0;
        else r = p[(size_t)v * ldp + p2io[i]];
        u[(size_t)v * ldu + i] = r;
    }
}

// y = a * x + b * z (both products rounded, then the sum) -- vec_sum1
__global__ void k_axpbz(double *y, const double *x, double a, const double *z, double b, long long n) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        y[t] = a * x[t] + b * z[t];
}

// FC = (1/tau) w + mu(1-theta) dw ; FC = 1.0 FC + (-sigma(1-theta)) w ; FC += rp
// (examples/barvortex_impl.h:238-256)
// rp: one forcing field of V values shared by every member (null = none)
__global__ void k_bv_fc(double *FC, const double *w, const double *dw, const double *rp,
                        double c_w, double c_dw, double c_w2, int V, long long n) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        double f = c_w * w[t] + c_dw * dw[t];
        f = 1.0 * f + c_w2 * w[t];
        if (rp) f += rp[t % V];
        FC[t] = f;
    }
}

// tmp1 = k1 theta w_n + k1 (1-theta) w ; tmp1 = tmp1 + k2 lh ; tmp2 = theta u_n + (1-theta) u
// (examples/barvortex_impl.h:267-272); lh is one field shared by all members
__global__ void k_bv_mix(double *tmp1, double *tmp2, const double *w_n, const double *w,
                         const double *u_n, const double *u, const double *lh, int V,
                         double a1, double a2, double k2, double t1, double t2, long long n) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        double s = a1 * w_n[t] + a2 * w[t];
        s = s + k2 * lh[t % V];
        tmp1[t] = s;
        tmp2[t] = t1 * u_n[t] + t2 * u[t];
    }
}

// elementwise a - b
__global__ void k_sub(double *y, const double *a, const double *b, long long n) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        y[t] = a[t] - b[t];
}

// per-member partial sums of a[i] * b[i] over chunks of `chunk` rows
__global__ void k_dot_partial(const double *a, const double *b, int ld, int n, int chunk, int nchunk,
                              double *part, int nv) {
    __shared__ double red[TB];
    int v = blockIdx.x / nchunk, c = blockIdx.x % nchunk;
    if (v >= nv) return;
    const double *x = a + (size_t)v * ld, *y = b + (size_t)v * ld;
    int i0 = c * chunk, i1 = min(n, i0 + chunk);
    double s = 0.0;
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) s += x[i] * y[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// out[v] = sum of the member's partials (sqrt if take_sqrt)
__global__ void k_dot_final(const double *part, int nchunk, double *out, int nv, int take_sqrt) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    double s = 0.0;
    for (int c = 0; c < nchunk; ++c) s += part[(size_t)v * nchunk + c];
    out[v] = take_sqrt ? sqrt(s) : s;
}

// Picard bookkeeping: u_n <- u_n1 for members still iterating, then stop a
// member once dist/norm0 < 1e-14 or the distance is NaN
// (examples/barvortex_impl.h:300-306)
__global__ void k_bv_commit(double *u_n, const double *u_n1, const double *nr, const double *nr0,
                            int *done, int V, int nv) {
    const long long total = (long long)nv * V;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        int v = (int)(t / V);
        if (!done[v]) u_n[t] = u_n1[t];
    }
}

__global__ void k_bv_done(const double *nr, const double *nr0, int *done, int nv) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv || done[v]) return;
    double r = nr[v];
    if (r / nr0[v] < 1e-14 || isnan(r)) done[v] = 1;
}

__global__ void k_gather(double *y, int ldy, const double *x, int ldx, const int *map, int n, int nv) {
    const long long total = (long long)nv * n;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        int v = (int)(t / n), i = (int)(t % n);
        y[(size_t)v * ldy + i] = x[(size_t)v * ldx + (map ? map[i] : i)];
    }
}

}  // namespace

__device__ __forceinline__ double hash_unit(unsigned long long i, unsigned seed) {
    // splitmix64 finaliser of (i, seed), top 53 bits -> [-1, 1)
    unsigned long long z = i + 0x9E3779B97F4A7C15ull * (seed + 1ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

__global__ void k_fill_hash(double *x, long long n, unsigned seed) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] = hash_unit((unsigned long long)i, seed);
}

__global__ void k_fill_hash32(float *x, long long n, unsigned seed) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] = (float)hash_unit((unsigned long long)i, seed);
}

cudaError_t fill_hash(double *x, long long n, unsigned seed, cudaStream_t s) {
    k_fill_hash<<<grid_for(n), TB, 0, s>>>(x, n, seed);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t fill_hash32(float *x, long long n, unsigned seed, cudaStream_t s) {
    k_fill_hash32<<<grid_for(n), TB, 0, s>>>(x, n, seed);
    g_kernel_launches++;
    return cudaGetLastError();
}

// Index validation (debug aid): count the entries of an index array outside
// [lo, hi); only the indices themselves are read, never what they point to.
__global__ void k_check_range(const int *a, long long n, int lo, int hi, unsigned long long *bad) {
    unsigned long long cnt = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int v = a[i];
        cnt += (v < lo || v >= hi) ? 1ull : 0ull;
    }
    if (cnt) atomicAdd(bad, cnt);
}

// p2io: inner points map into [0, rs), boundary points (isb) into [0, os)
__global__ void k_check_p2io(const int *p2io, const int *isb, int V, int rs, int os, unsigned long long *bad) {
    unsigned long long cnt = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < V; i += gridDim.x * blockDim.x) {
        const int v = p2io[i], b = isb[i];
        cnt += (b != 0 && b != 1) || v < 0 || v >= (b ? os : rs) ? 1ull : 0ull;
    }
    if (cnt) atomicAdd(bad, cnt);
}

// CSR row pointers: ptr[0] = 0, non-decreasing, ptr[n] = nnz
__global__ void k_check_ptr(const int *ptr, int n, int nnz, unsigned long long *bad) {
    unsigned long long cnt = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        cnt += ptr[i + 1] < ptr[i] ? 1ull : 0ull;
    if (blockIdx.x == 0 && threadIdx.x == 0) cnt += (ptr[0] != 0) + (ptr[n] != nnz);
    if (cnt) atomicAdd(bad, cnt);
}

cudaError_t check_range(const int *a, long long n, int lo, int hi, unsigned long long *bad, cudaStream_t s) {
    if (!a || n <= 0) return cudaSuccess;
    k_check_range<<<grid_for(n), TB, 0, s>>>(a, n, lo, hi, bad);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t check_p2io(const int *p2io, const int *isb, int V, int rs, int os, unsigned long long *bad,
                       cudaStream_t s) {
    k_check_p2io<<<grid_for(V), TB, 0, s>>>(p2io, isb, V, rs, os, bad);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t check_ptr(const int *ptr, int n, int nnz, unsigned long long *bad, cudaStream_t s) {
    if (!ptr || n <= 0) return cudaSuccess;
    k_check_ptr<<<grid_for(n), TB, 0, s>>>(ptr, n, nnz, bad);
    g_kernel_launches++;
    return cudaGetLastError();
}

__global__ void k_stats_fold(const GmresStats *slots, int n, GmresStats *agg) {
    if (threadIdx.x || blockIdx.x) return;
    GmresStats a = *agg;
    for (int k = 0; k < n; ++k) {
        const GmresStats g = slots[k];
        a.relres = fmax(a.relres, g.relres);
        a.bytes += g.bytes;
        a.iters += g.iters;
        a.cycles += g.cycles;
        a.status = max(a.status, g.status);
        a.steps_total += g.steps_total;
    }
    *agg = a;
}

cudaError_t stats_fold(const GmresStats *slots, int n, GmresStats *agg, cudaStream_t s) {
    k_stats_fold<<<1, 32, 0, s>>>(slots, n, agg);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t apply_exact(const DevEll &A, const DevCols &C, const double *x_in, int ldx,
                        const double *x_bnd, int ldb, double *y, int ldy, int nv, cudaStream_t s) {
    k_apply<<<grid_for((long long)nv * A.n), TB, 0, s>>>(A, C, x_in, ldx, nullptr, x_bnd, ldb, nullptr, y, ldy, nv);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t apply_op(const DevEll &A, const DevCols &C, const double *xin, int ldx, const int *imap,
                     const double *xb, int ldb, const int *bmap, double *y, int ldy, int nv, cudaStream_t s) {
    k_apply<<<grid_for((long long)nv * A.n), TB, 0, s>>>(A, C, xin, ldx, imap, xb, ldb, bmap, y, ldy, nv);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t jac_rhs(const JacOps &J, const double *u, const double *v, int ld, const int *imap,
                    const int *bmap, double *out, int ldo, int nv, cudaStream_t s) {
    k_jac_rhs<<<grid_for((long long)nv * J.d1.n), TB, 0, s>>>(J, u, v, ld, imap, bmap, out, ldo, nv);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t jac_combine(const double *d, int ldd, int n, double *jac, int ldj, const double *FC, int ldf,
                        const int *inner, int nv, cudaStream_t s) {
    k_jac_combine<<<grid_for((long long)nv * n), TB, 0, s>>>(d, ldd, n, jac, ldj, FC, ldf, inner, nv);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t p2u(double *u, int ldu, const double *p, int ldp, const double *bnd, int ldb,
                const int *p2io, const int *isb, int V, int nv, cudaStream_t s) {
    k_p2u<<<grid_for((long long)nv * V), TB, 0, s>>>(u, ldu, p, ldp, bnd, ldb, p2io, isb, V, nv);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t axpbz(double *y, const double *x, double a, const double *z, double b, long long n, cudaStream_t s) {
    k_axpbz<<<grid_for(n), TB, 0, s>>>(y, x, a, z, b, n);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t bv_fc(double *FC, const double *w, const double *dw, const double *rp, double c_w, double c_dw,
                  double c_w2, int V, long long n, cudaStream_t s) {
    k_bv_fc<<<grid_for(n), TB, 0, s>>>(FC, w, dw, rp, c_w, c_dw, c_w2, V, n);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t bv_mix(double *tmp1, double *tmp2, const double *w_n, const double *w, const double *u_n,
                   const double *u, const double *lh, int V, double a1, double a2, double k2, double t1,
                   double t2, long long n, cudaStream_t s) {
    k_bv_mix<<<grid_for(n), TB, 0, s>>>(tmp1, tmp2, w_n, w, u_n, u, lh, V, a1, a2, k2, t1, t2, n);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t vsub(double *y, const double *a, const double *b, long long n, cudaStream_t s) {
    k_sub<<<grid_for(n), TB, 0, s>>>(y, a, b, n);
    g_kernel_launches++;
    return cudaGetLastError();
}

int dot_chunks(int n) { return (n + 8191) / 8192; }

cudaError_t dot(const double *a, const double *b, int ld, int n, int nv, double *part, double *out,
                bool take_sqrt, cudaStream_t s) {
    int nch = dot_chunks(n);
    k_dot_partial<<<nv * nch, TB, 0, s>>>(a, b, ld, n, 8192, nch, part, nv);
    g_kernel_launches++;
    k_dot_final<<<(nv + 127) / 128, 128, 0, s>>>(part, nch, out, nv, take_sqrt ? 1 : 0);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t bv_commit(double *u_n, const double *u_n1, const double *nr, const double *nr0, int *done,
                      int V, int nv, cudaStream_t s) {
    k_bv_commit<<<grid_for((long long)nv * V), TB, 0, s>>>(u_n, u_n1, nr, nr0, done, V, nv);
    g_kernel_launches++;
    k_bv_done<<<(nv + 127) / 128, 128, 0, s>>>(nr, nr0, done, nv);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t gather(double *y, int ldy, const double *x, int ldx, const int *map, int n, int nv, cudaStream_t s) {
    k_gather<<<grid_for((long long)nv * n), TB, 0, s>>>(y, ldy, x, ldx, map, n, nv);
    g_kernel_launches++;
    return cudaGetLastError();
}

}  // namespace phg

// ------------------------------------------------------------ baroclin ----
namespace phg {
namespace {

// FC / GC of Baroclin::calc (examples/baroclin.cpp:501-536), vectors of V
__global__ void k_bc_fcgc(double *FC, double *GC, const double *w1, const double *w2, const double *dw1,
                          const double *dw2, const double *u2, const double *f, const double *g, BcCoef c, int V) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < V; t += gridDim.x * blockDim.x) {
        double fc = c.a * w1[t] + c.b * w2[t];
        fc = 1.0 * fc + c.mu1t * dw1[t];
        fc = 1.0 * fc + c.itau * w1[t];
        double gc = c.ga * w1[t] + c.gb * w2[t];
        gc = 1.0 * gc + c.mu1t * dw2[t];
        gc = 1.0 * gc + c.itau * w2[t];
        gc = 1.0 * gc + c.g_u2 * u2[t];
        gc = 1.0 * gc + c.g_w2 * w2[t];
        gc = 1.0 * gc + c.g_u2b * u2[t];
        if (f) fc += f[t];
        if (g) gc += c.alpha2 * g[t];
        FC[t] = fc;
        GC[t] = gc;
    }
}

// Jacobian argument pairs of the linearised steps, in the reference's order
// (examples/baroclin.cpp:717-776): U = wa u + wb u_n, W = wa w + wb w_n
//   0 (U1, dz1 + l)  1 (z1, W1)  2 (z2, W2)  3 (U2, dz2)  4 (dz1, W2)
//   5 (dz2, U1)      6 (U2, dz1 + l)  7 (z2, W1)  8 (z1, U2)  9 (U1, z2)
__global__ void k_bc_lin_jin(double *ju, double *jv, const double *U, const double *Wv, const double *Un,
                             const double *Wn, const double *Z, const double *dZ, const double *lh, double wa,
                             double wb, int V) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < V; t += gridDim.x * blockDim.x) {
        const double U1 = wa * U[t] + wb * Un[t], U2 = wa * U[V + t] + wb * Un[V + t];
        const double W1 = wa * Wv[t] + wb * Wn[t], W2 = wa * Wv[V + t] + wb * Wn[V + t];
        const double z1 = Z[t], z2 = Z[V + t], dz1 = dZ[t], dz2 = dZ[V + t];
        const double dzl = dz1 + lh[t];
        const double a[10] = {U1, z1, z2, U2, dz1, dz2, U2, z2, z1, U1};
        const double b[10] = {dzl, W1, W2, dz2, W2, U1, dzl, W1, U2, z2};
#pragma unroll
        for (int k = 0; k < 10; ++k) {
            ju[(size_t)k * V + t] = a[k];
            jv[(size_t)k * V + t] = b[k];
        }
    }
}

__global__ void k_bc_lin_fg(double *F, double *G, const double *jac, const double *FC, const double *GC,
                            const int *inner, int kind, double ka2, int rs) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rs; i += gridDim.x * blockDim.x) {
        double j[10];
#pragma unroll
        for (int k = 0; k < 10; ++k) j[k] = jac[(size_t)k * rs + i];
        double f, g;
        if (kind == 0) {
            f = -1.0 * j[0] + -1.0 * j[1];
            f = 1.0 * f + -1.0 * j[2];
            f = 1.0 * f + -1.0 * j[3];
            g = -1.0 * j[4] + -1.0 * j[5];
            g = 1.0 * g + -1.0 * j[6];
            g = 1.0 * g + -1.0 * j[7];
        } else {
            f = j[0] + j[1];
            f = f + j[2];
            f = f + j[3];
            g = j[4] + j[5];
            g = g + j[6];
            g = g + j[7];
        }
        g = 1.0 * g + ka2 * j[8];
        g = 1.0 * g + ka2 * j[9];
        const int p = inner[i];
        F[i] = f + FC[p];
        G[i] = g + GC[p];
    }
}

// the five Jacobian argument pairs of one Picard iteration
// (examples/baroclin.cpp:551-575): out ju[k], jv[k] for k = 0..4
__global__ void k_bc_jin(double *ju, double *jv, const double *u1, const double *u2, const double *w1,
                         const double *w2, const double *u1n, const double *u2n, const double *w1n,
                         const double *w2n, const double *lh, double th, int V) {
    const double a = 1.0 - th;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < V; t += gridDim.x * blockDim.x) {
        const double U1 = a * u1[t] + th * u1n[t];
        const double U2 = a * u2[t] + th * u2n[t];
        double W1 = a * w1[t] + th * w1n[t];
        const double W1l = W1 + lh[t];
        const double W2 = a * w2[t] + th * w2n[t];
        ju[t] = U1;              jv[t] = W1l;
        ju[V + t] = U2;          jv[V + t] = W2;
        ju[2 * (size_t)V + t] = U1; jv[2 * (size_t)V + t] = W2;
        ju[3 * (size_t)V + t] = U2; jv[3 * (size_t)V + t] = W1l;
        ju[4 * (size_t)V + t] = U1; jv[4 * (size_t)V + t] = U2;
    }
}

// F = -jac0 - jac1 + FC[inner]; G = -jac2 - jac3 + alpha^2 jac4 + GC[inner]
__global__ void k_bc_fg(double *F, double *G, const double *jac, const double *FC, const double *GC,
                        const int *inner, double alpha2, int rs) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rs; i += gridDim.x * blockDim.x) {
        double f = -1.0 * jac[i] + -1.0 * jac[rs + i];
        double g = -1.0 * jac[2 * (size_t)rs + i] + -1.0 * jac[3 * (size_t)rs + i];
        g = 1.0 * g + alpha2 * jac[4 * (size_t)rs + i];
        const int p = inner ? inner[i] : i;
        F[i] = f + FC[p];
        G[i] = g + GC[p];
    }
}

// interleaved right-hand side: [M F, M G, 0, 0] minus the boundary columns,
// the u rows scaled by su
__global__ void k_bc_rhs(double *rp, const double *MF, const double *MG, BcCols bc, const double *bnd, double su,
                         int rs) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rs; i += gridDim.x * blockDim.x) {
        double t[4] = {0, 0, 0, 0};
        if (bnd)
            for (int q = 0; q < 4; ++q)
                if (bc.c[q].ptr)
                    for (int k = bc.c[q].ptr[i]; k < bc.c[q].ptr[i + 1]; ++k) t[q] += -bnd[bc.c[q].col[k]] * bc.c[q].val[k];
        rp[4 * (size_t)i] = MF[i] + t[0];
        rp[4 * (size_t)i + 1] = MG[i] + t[1];
        rp[4 * (size_t)i + 2] = su * t[2];
        rp[4 * (size_t)i + 3] = su * t[3];
    }
}

// interleave the inner parts of four full vectors (initial guess), the u
// unknowns scaled by su
__global__ void k_bc_pack(double *x, const double *a, const double *b, const double *c, const double *d,
                          const int *inner, double su, int rs) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rs; i += gridDim.x * blockDim.x) {
        const int p = inner[i];
        x[4 * (size_t)i] = a[p];
        x[4 * (size_t)i + 1] = b[p];
        x[4 * (size_t)i + 2] = su * c[p];
        x[4 * (size_t)i + 3] = su * d[p];
    }
}

// de-interleave into four full vectors with the boundary values (p2u)
__global__ void k_bc_unpack(double *a, double *b, double *c, double *d, const double *x, const double *bnd,
                            const int *p2io, const int *isb, double isu, int V) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < V; p += gridDim.x * blockDim.x) {
        const int j = p2io[p];
        if (isb[p]) {
            const double v = bnd ? bnd[j] : 0.0;
            a[p] = v; b[p] = v; c[p] = v; d[p] = v;
        } else {
            a[p] = x[4 * (size_t)j]; b[p] = x[4 * (size_t)j + 1];
            c[p] = isu * x[4 * (size_t)j + 2]; d[p] = isu * x[4 * (size_t)j + 3];
        }
    }
}

// u_n <- u_n1 (both layers) unless stopped; stop once max(nr) < tol
__global__ void k_bc_commit(double *un, const double *un1, const int *done, int n) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
        if (!*done) un[t] = un1[t];
}

__global__ void k_bc_done(const double *nr, int *done, double tol) {
    if (threadIdx.x == 0 && blockIdx.x == 0 && !*done) {
        const double m = nr[0] > nr[1] ? nr[0] : nr[1];
        if (m < tol) *done = 1;
    }
}

}  // namespace

cudaError_t bc_fcgc(double *FC, double *GC, const double *w1, const double *w2, const double *dw1, const double *dw2,
                    const double *u2, const double *f, const double *g, const BcCoef &c, int V, cudaStream_t s) {
    k_bc_fcgc<<<grid_for(V), TB, 0, s>>>(FC, GC, w1, w2, dw1, dw2, u2, f, g, c, V);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t bc_jin(double *ju, double *jv, const double *u1, const double *u2, const double *w1, const double *w2,
                   const double *u1n, const double *u2n, const double *w1n, const double *w2n, const double *lh,
                   double th, int V, cudaStream_t s) {
    k_bc_jin<<<grid_for(V), TB, 0, s>>>(ju, jv, u1, u2, w1, w2, u1n, u2n, w1n, w2n, lh, th, V);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t bc_fg(double *F, double *G, const double *jac, const double *FC, const double *GC, const int *inner,
                  double alpha2, int rs, cudaStream_t s) {
    k_bc_fg<<<grid_for(rs), TB, 0, s>>>(F, G, jac, FC, GC, inner, alpha2, rs);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t bc_rhs(double *rp, const double *MF, const double *MG, const BcCols &bc, const double *bnd, double su,
                   int rs, cudaStream_t s) {
    k_bc_rhs<<<grid_for(rs), TB, 0, s>>>(rp, MF, MG, bc, bnd, su, rs);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t bc_pack(double *x, const double *a, const double *b, const double *c, const double *d, const int *inner,
                    double su, int rs, cudaStream_t s) {
    k_bc_pack<<<grid_for(rs), TB, 0, s>>>(x, a, b, c, d, inner, su, rs);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t bc_unpack(double *a, double *b, double *c, double *d, const double *x, const double *bnd,
                      const int *p2io, const int *isb, double isu, int V, cudaStream_t s) {
    k_bc_unpack<<<grid_for(V), TB, 0, s>>>(a, b, c, d, x, bnd, p2io, isb, isu, V);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t bc_lin_jin(double *ju, double *jv, const double *U, const double *Wv, const double *Un, const double *Wn,
                       const double *Z, const double *dZ, const double *lh, double wa, double wb, int V,
                       cudaStream_t s) {
    k_bc_lin_jin<<<grid_for(V), TB, 0, s>>>(ju, jv, U, Wv, Un, Wn, Z, dZ, lh, wa, wb, V);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t bc_lin_fg(double *F, double *G, const double *jac, const double *FC, const double *GC, const int *inner,
                      int kind, double ka2, int rs, cudaStream_t s) {
    k_bc_lin_fg<<<grid_for(rs), TB, 0, s>>>(F, G, jac, FC, GC, inner, kind, ka2, rs);
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t bc_commit(double *un, const double *un1, const double *nr, int *done, double tol, int n, cudaStream_t s) {
    k_bc_commit<<<grid_for(n), TB, 0, s>>>(un, un1, done, n);
    k_bc_done<<<1, 32, 0, s>>>(nr, done, tol);
    g_kernel_launches += 2;
    return cudaGetLastError();
}

}  // namespace phg

// ------------------------------------------------------- operator apply ---
namespace phg {
namespace {

// y_v = A x_v for nv member-major vectors on the shared inner x inner
// pattern.  A thread owns one row: it loads the row's columns and values once
// (the matrix streams from memory once per launch) and applies them to every
// member.  Ascending column order; FP64 sums round like the CPU CSR product.
template <typename T>
__global__ void __launch_bounds__(TB) k_spmm(const int *__restrict__ col, const T *__restrict__ val, int n, int W,
                                             const T *__restrict__ x, int ldx, T *__restrict__ y, int ldy, int nv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c[8];
    T a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (k < W) { c[k] = __ldg(&col[(size_t)k * n + i]); a[k] = __ldg(&val[(size_t)k * n + i]); }
    for (int v = 0; v < nv; ++v) {
        const T *xv = x + (size_t)v * ldx;
        T g[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < W) g[k] = __ldg(&xv[c[k]]);
        T s = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < W) s += a[k] * g[k];
        y[(size_t)v * ldy + i] = s;
    }
}

// Y = A X for an interleaved FP32 multi-vector (row r of X holds the nv
// members of point r contiguously, nv = 4 q4).  TPR = q4 / CH threads share
// a row; thread q forms the 4-member chunks q, q + TPR, ... (CH of them), so
// consecutive threads read consecutive 16-byte chunks of each gathered row
// of X and every sector fetched is used in full; the row's columns and values
// are loaded once per thread and reused for its CH chunks.  W is a
// compile-time slot count (7 for the P1 sphere pattern).
template <int W, int CH>
__global__ void __launch_bounds__(TB) k_spmm_il(const int *__restrict__ col, const float *__restrict__ val, int n,
                                                const float4 *__restrict__ x, float4 *__restrict__ y, int q4,
                                                int tpr_log2) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;   // n * q4 / CH < 2^31 (host check)
    const int i = (int)(t >> tpr_log2), q = (int)(t & ((1u << tpr_log2) - 1u));
    if (i >= n) return;
    const int tpr = 1 << tpr_log2;
    int c[W];
    float a[W];
#pragma unroll
    for (int k = 0; k < W; ++k) { c[k] = __ldg(&col[(size_t)k * n + i]); a[k] = __ldg(&val[(size_t)k * n + i]); }
    // all CH x W gathers are issued before any arithmetic (more bytes in flight)
    float4 g[CH][W];
#pragma unroll
    for (int j = 0; j < CH; ++j)
#pragma unroll
        for (int k = 0; k < W; ++k) g[j][k] = __ldg(&x[(size_t)c[k] * q4 + q + j * tpr]);
#pragma unroll
    for (int j = 0; j < CH; ++j) {
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int k = 0; k < W; ++k) {
            s.x = __fmaf_rn(a[k], g[j][k].x, s.x); s.y = __fmaf_rn(a[k], g[j][k].y, s.y);
            s.z = __fmaf_rn(a[k], g[j][k].z, s.z); s.w = __fmaf_rn(a[k], g[j][k].w, s.w);
        }
        y[(size_t)i * q4 + q + j * tpr] = s;
    }
}

template <int W>
cudaError_t launch_il(const int *col, const float *val, int n, const float4 *x, float4 *y, int q4, int tpr,
                      cudaStream_t s) {
    // Default: eight threads per row (fewer when the row has fewer chunks),
    // each with q4 / 8 chunks -- the best of a sweep over 1..16 chunks per
    // thread and 256/1024-thread blocks on a level-8 Laplacian with 32 and 64
    // members.  The autotuner may choose another power of two.
    if (tpr <= 0 || tpr > q4 || q4 % tpr || q4 / tpr > 8) tpr = q4 < 8 ? q4 : 8;
    const int ch = q4 / tpr;
    if (tpr * ch != q4) return cudaErrorInvalidValue;
    int lg = 0;
    while ((1 << lg) < tpr) ++lg;
    if ((1 << lg) != tpr) return cudaErrorInvalidValue;
    const long long work = (long long)n * tpr;
    if (work >= (1LL << 31)) return cudaErrorInvalidValue;
    const unsigned blocks = (unsigned)((work + TB - 1) / TB);
    switch (ch) {
    case 1: k_spmm_il<W, 1><<<blocks, TB, 0, s>>>(col, val, n, x, y, q4, lg); break;
    case 2: k_spmm_il<W, 2><<<blocks, TB, 0, s>>>(col, val, n, x, y, q4, lg); break;
    case 4: k_spmm_il<W, 4><<<blocks, TB, 0, s>>>(col, val, n, x, y, q4, lg); break;
    case 8: k_spmm_il<W, 8><<<blocks, TB, 0, s>>>(col, val, n, x, y, q4, lg); break;
    default: return cudaErrorInvalidValue;   // more than 256 members: split the call
    }
    return cudaGetLastError();
}

// Y = A X as k_spmm_il, with each row's eight (column, value) pairs in one
// 64-byte record (pk[8 i + k]; padding slots (i, 0) add an exact zero): the
// matrix is one sequential stream instead of one per slot for the columns and
// one per slot for the values
template <int CH>
__global__ void __launch_bounds__(TB) k_spmm_pk(const uint4 *__restrict__ pk, int n, const float4 *__restrict__ x,
                                                float4 *__restrict__ y, int q4, int tpr_log2) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;   // n * q4 / CH < 2^31 (host check)
    const int i = (int)(t >> tpr_log2), q = (int)(t & ((1u << tpr_log2) - 1u));
    if (i >= n) return;
    const int tpr = 1 << tpr_log2;
    int c[8];
    float a[8];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint4 e = __ldg(&pk[(size_t)i * 4 + k]);
        c[2 * k] = (int)e.x; a[2 * k] = __uint_as_float(e.y);
        c[2 * k + 1] = (int)e.z; a[2 * k + 1] = __uint_as_float(e.w);
    }
    float4 g[CH][8];
#pragma unroll
    for (int j = 0; j < CH; ++j)
#pragma unroll
        for (int k = 0; k < 8; ++k) g[j][k] = __ldg(&x[(size_t)c[k] * q4 + q + j * tpr]);
#pragma unroll
    for (int j = 0; j < CH; ++j) {
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            s.x = __fmaf_rn(a[k], g[j][k].x, s.x); s.y = __fmaf_rn(a[k], g[j][k].y, s.y);
            s.z = __fmaf_rn(a[k], g[j][k].z, s.z); s.w = __fmaf_rn(a[k], g[j][k].w, s.w);
        }
        y[(size_t)i * q4 + q + j * tpr] = s;
    }
}

}  // namespace

template <typename T>
cudaError_t spmm(const int *col, const T *val, int n, int W, const T *x, int ldx, T *y, int ldy, int nv,
                 cudaStream_t s) {
    if (W > 8 || n < 1 || nv < 1) return cudaErrorInvalidValue;
    k_spmm<T><<<(unsigned)((n + TB - 1) / TB), TB, 0, s>>>(col, val, n, W, x, ldx, y, ldy, nv);
    g_kernel_launches++;
    return cudaGetLastError();
}

template cudaError_t spmm<double>(const int *, const double *, int, int, const double *, int, double *, int, int,
                                  cudaStream_t);
template cudaError_t spmm<float>(const int *, const float *, int, int, const float *, int, float *, int, int,
                                 cudaStream_t);

cudaError_t spmm_pk32(const unsigned *pk, int n, const float *x, float *y, int nv, cudaStream_t s, int tpr) {
    if (n < 1 || nv < 4 || nv % 4 || ((uintptr_t)x & 15) || ((uintptr_t)y & 15) || ((uintptr_t)pk & 15))
        return cudaErrorInvalidValue;
    const int q4 = nv / 4;
    if (tpr <= 0) tune_get_spmm(n, nv, &tpr);
    if (tpr <= 0 || tpr > q4 || q4 % tpr || q4 / tpr > 8) tpr = q4 < 8 ? q4 : 8;
    int lg = 0;
    while ((1 << lg) < tpr) ++lg;
    if ((1 << lg) != tpr) return cudaErrorInvalidValue;
    const long long work = (long long)n * tpr;
    if (work >= (1LL << 31)) return cudaErrorInvalidValue;
    const unsigned blocks = (unsigned)((work + TB - 1) / TB);
    const uint4 *p4 = (const uint4 *)pk;
    switch (q4 / tpr) {
    case 1: k_spmm_pk<1><<<blocks, TB, 0, s>>>(p4, n, (const float4 *)x, (float4 *)y, q4, lg); break;
    case 2: k_spmm_pk<2><<<blocks, TB, 0, s>>>(p4, n, (const float4 *)x, (float4 *)y, q4, lg); break;
    case 4: k_spmm_pk<4><<<blocks, TB, 0, s>>>(p4, n, (const float4 *)x, (float4 *)y, q4, lg); break;
    case 8: k_spmm_pk<8><<<blocks, TB, 0, s>>>(p4, n, (const float4 *)x, (float4 *)y, q4, lg); break;
    default: return cudaErrorInvalidValue;
    }
    g_kernel_launches++;
    return cudaGetLastError();
}

cudaError_t spmm_il32(const int *col, const float *val, int n, int W, const float *x, float *y, int nv,
                      cudaStream_t s, int tpr) {
    if (n < 1 || nv < 4 || nv % 4 || ((uintptr_t)x & 15) || ((uintptr_t)y & 15)) return cudaErrorInvalidValue;
    const int q4 = nv / 4;
    if (tpr <= 0) tune_get_spmm(n, nv, &tpr);
    cudaError_t e;
    switch (W) {   // the ELL arrays hold exactly W slots (padding: diagonal column, zero value)
    case 8: e = launch_il<8>(col, val, n, (const float4 *)x, (float4 *)y, q4, tpr, s); break;
    case 7: e = launch_il<7>(col, val, n, (const float4 *)x, (float4 *)y, q4, tpr, s); break;
    case 6: e = launch_il<6>(col, val, n, (const float4 *)x, (float4 *)y, q4, tpr, s); break;
    default: return cudaErrorInvalidValue;
    }
    g_kernel_launches++;
    return e;
}

}  // namespace phg
