// phg_kernels.cuh -- launchers of the operator-apply and elementwise kernels.
#pragma once
#include "phg_device.cuh"

#include <atomic>

namespace phg {

// kernels enqueued by this library since load (instrumentation)
extern std::atomic<long long> g_kernel_launches;

// the four derivative operators of SphereJacobian on the shared pattern
// (d1.col == d2.col == ...) and their boundary columns
struct JacOps {
    DevEll d1, d2, d1c, d2c;
    DevCols d1b, d2b, d1cb, d2cb;
};

// y = A xin[imap] + C xb[bmap] (null map = identity; null xb or empty C =
// no boundary term); member v reads xin + v*ldx, xb + v*ldb
cudaError_t apply_op(const DevEll &A, const DevCols &C, const double *xin, int ldx, const int *imap,
                     const double *xb, int ldb, const int *bmap, double *y, int ldy, int nv, cudaStream_t s);
cudaError_t jac_rhs(const JacOps &J, const double *u, const double *v, int ld, const int *imap,
                    const int *bmap, double *out, int ldo, int nv, cudaStream_t s);
cudaError_t jac_combine(const double *d, int ldd, int n, double *jac, int ldj, const double *FC, int ldf,
                        const int *inner, int nv, cudaStream_t s);
cudaError_t p2u(double *u, int ldu, const double *p, int ldp, const double *bnd, int ldb,
                const int *p2io, const int *isb, int V, int nv, cudaStream_t s);
cudaError_t axpbz(double *y, const double *x, double a, const double *z, double b, long long n, cudaStream_t s);
// FC = c_w w + c_dw dw, then FC + c_w2 w, then + rp (one field of V values
// shared by the members, or null), over n = members x V entries
cudaError_t bv_fc(double *FC, const double *w, const double *dw, const double *rp, double c_w, double c_dw,
                  double c_w2, int V, long long n, cudaStream_t s);
cudaError_t bv_mix(double *tmp1, double *tmp2, const double *w_n, const double *w, const double *u_n,
                   const double *u, const double *lh, int V, double a1, double a2, double k2, double t1,
                   double t2, long long n, cudaStream_t s);
cudaError_t vsub(double *y, const double *a, const double *b, long long n, cudaStream_t s);
int dot_chunks(int n);
// out[v] = sum_i a[v][i] b[v][i] (sqrt if take_sqrt); part holds nv * dot_chunks(n) doubles
cudaError_t dot(const double *a, const double *b, int ld, int n, int nv, double *part, double *out,
                bool take_sqrt, cudaStream_t s);
cudaError_t bv_commit(double *u_n, const double *u_n1, const double *nr, const double *nr0, int *done,
                      int V, int nv, cudaStream_t s);
cudaError_t gather(double *y, int ldy, const double *x, int ldx, const int *map, int n, int nv, cudaStream_t s);
// index validation: add to *bad the entries outside their valid range
cudaError_t check_range(const int *a, long long n, int lo, int hi, unsigned long long *bad, cudaStream_t s);
cudaError_t check_p2io(const int *p2io, const int *isb, int V, int rs, int os, unsigned long long *bad,
                       cudaStream_t s);
cudaError_t check_ptr(const int *ptr, int n, int nnz, unsigned long long *bad, cudaStream_t s);
// agg += the n solve records in slots (iterations summed; residual and status: the worst)
cudaError_t stats_fold(const GmresStats *slots, int n, GmresStats *agg, cudaStream_t s);

// y_v = A x_v, v < nv, member-major, on a slot-major ELL pattern of at most 8 slots
template <typename T>
cudaError_t spmm(const int *col, const T *val, int n, int W, const T *x, int ldx, T *y, int ldy, int nv,
                 cudaStream_t s);
// Y = A X, X and Y interleaved (n x nv, member-minor), FP32, nv = 4 * 2^k <= 256,
// 16-byte aligned; tpr: threads per row (a power of two with nv / 4 / tpr
// in 1..8; 0 = the tuned value, else 8)
cudaError_t spmm_il32(const int *col, const float *val, int n, int W, const float *x, float *y, int nv,
                      cudaStream_t s, int tpr = 0);
// the same product from 64-byte row records (8 (column, value) pairs per row)
cudaError_t spmm_pk32(const unsigned *pk, int n, const float *x, float *y, int nv, cudaStream_t s, int tpr = 0);
// deterministic test data: x[i] = a hash of (i, seed) in [-1, 1)
cudaError_t fill_hash(double *x, long long n, unsigned seed, cudaStream_t s);
cudaError_t fill_hash32(float *x, long long n, unsigned seed, cudaStream_t s);

// Baroclin step helpers (examples/baroclin.cpp:445-606)
struct BcCoef {
    double a;       // -0.5 (1-theta) sigma
    double b;       //  0.5 (1-theta) sigma
    double mu1t;    // mu (1-theta)
    double itau;    // 1/tau
    double g_u2;    // -alpha^2 / tau
    double g_w2;    // -alpha^2 mu1 (1-theta)
    double g_u2b;   //  alpha^2 sigma1 (1-theta)
    double alpha2;  //  alpha^2
    double ga, gb;  //  GC's w1, w2 coefficients (the step: a, a)
};
struct BcCols { DevCols c[4]; };
cudaError_t bc_fcgc(double *FC, double *GC, const double *w1, const double *w2, const double *dw1, const double *dw2,
                    const double *u2, const double *f, const double *g, const BcCoef &c, int V, cudaStream_t s);
cudaError_t bc_jin(double *ju, double *jv, const double *u1, const double *u2, const double *w1, const double *w2,
                   const double *u1n, const double *u2n, const double *w1n, const double *w2n, const double *lh,
                   double th, int V, cudaStream_t s);
cudaError_t bc_fg(double *F, double *G, const double *jac, const double *FC, const double *GC, const int *inner,
                  double alpha2, int rs, cudaStream_t s);
cudaError_t bc_rhs(double *rp, const double *MF, const double *MG, const BcCols &bc, const double *bnd, double su,
                   int rs, cudaStream_t s);
cudaError_t bc_pack(double *x, const double *a, const double *b, const double *c, const double *d, const int *inner,
                    double su, int rs, cudaStream_t s);
cudaError_t bc_unpack(double *a, double *b, double *c, double *d, const double *x, const double *bnd,
                      const int *p2io, const int *isb, double isu, int V, cudaStream_t s);
cudaError_t bc_commit(double *un, const double *un1, const double *nr, int *done, double tol, int n, cudaStream_t s);
// linearised steps (examples/baroclin.cpp:620-986): the 10 Jacobian argument
// pairs (weights wa on the input, wb on the iterate) and the F, G combination
// (kind 0: calc_L signs, 1: calc_L_1 signs; ka2 the alpha^2 coefficient)
cudaError_t bc_lin_jin(double *ju, double *jv, const double *U, const double *Wv, const double *Un, const double *Wn,
                       const double *Z, const double *dZ, const double *lh, double wa, double wb, int V,
                       cudaStream_t s);
cudaError_t bc_lin_fg(double *F, double *G, const double *jac, const double *FC, const double *GC, const int *inner,
                      int kind, double ka2, int rs, cudaStream_t s);

}  // namespace phg
