/*
 * orc_linalg.c -- oracle sparse matrices and linear solves.
 *
 * TEST INFRASTRUCTURE ONLY (see phelm_oracle.h).
 *
 * Restates the role of the reference's missing linear-algebra dependency
 * ("linal", github resetius/linal, un-vendored, no pinned version) as the
 * reference calls it:
 *   - Solver<T>::add(i, j, a) accumulates repeated (i, j) in call order
 *     (call sites src/generators.cpp:49-55, src/impl/generators_impl.h:36-72);
 *   - Solver<T>::mult_vector(y, x) is a CSR product
 *     (src/impl/slaplace_impl.h:109-113, src/sjacobian.cpp:160-181);
 *   - Solver<T>::solve(x, b) is "GMRES" (src/phelm.h:123; call sites
 *     src/impl/slaplace_impl.h:171, src/mesh.h:745, examples/baroclin.cpp:586).
 * The solve is restarted GMRES with an ILU(0) right preconditioner driven to a
 * 1e-13 relative residual, so the oracle reports the discrete solution itself;
 * the reference's own GMRES tolerance/restart are unknown (unpinned).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "phelm_oracle.h"

static double g_tol = 1e-13;
static int g_restart = 60;
static int g_maxit = 40000;
static double g_last_res = 0.0;

void orc_set_solver(double rel_tol, int restart, int max_iter)
{
	g_tol = rel_tol;
	g_restart = restart;
	g_maxit = max_iter;
}

double orc_last_residual(void) { return g_last_res; }

int orc_csr_nnz(const orc_csr *A) { return A->ptr ? A->ptr[A->n] : 0; }

void orc_csr_free(orc_csr *A)
{
	free(A->ptr); free(A->col); free(A->val); free(A->ilu); free(A->diag);
	memset(A, 0, sizeof(*A));
}

void orc_csr_mult(const orc_csr *A, double *y, const double *x)
{
	for (int i = 0; i < A->n; ++i) {
		double s = 0.0;
		for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k)
			s += A->val[k] * x[A->col[k]];
		y[i] = s;
	}
}

/* ------------------------------------------------------------ builder --- */
typedef struct { int n, cap; int *c; double *v; } orc_row;
struct orc_builder { int n, m; orc_row *rows; };

orc_builder *orc_builder_new(int n, int m)
{
	orc_builder *b = (orc_builder *)calloc(1, sizeof(*b));
	b->n = n; b->m = m;
	b->rows = (orc_row *)calloc((size_t)n, sizeof(orc_row));
	return b;
}

void orc_builder_add(orc_builder *b, int i, int j, double a)
{
	orc_row *r = &b->rows[i];
	for (int k = 0; k < r->n; ++k)
		if (r->c[k] == j) { r->v[k] += a; return; }
	if (r->n == r->cap) {
		r->cap = r->cap ? 2 * r->cap : 8;
		r->c = (int *)realloc(r->c, sizeof(int) * (size_t)r->cap);
		r->v = (double *)realloc(r->v, sizeof(double) * (size_t)r->cap);
	}
	/* the first contribution is stored as 0.0 + a, like a value-initialised
	 * map entry followed by += */
	r->c[r->n] = j; r->v[r->n] = 0.0 + a; r->n++;
}

void orc_builder_finish(orc_builder *b, orc_csr *A)
{
	memset(A, 0, sizeof(*A));
	A->n = b->n; A->m = b->m;
	A->ptr = (int *)malloc(sizeof(int) * (size_t)(b->n + 1));
	int nnz = 0;
	for (int i = 0; i < b->n; ++i) nnz += b->rows[i].n;
	A->col = (int *)malloc(sizeof(int) * (size_t)(nnz ? nnz : 1));
	A->val = (double *)malloc(sizeof(double) * (size_t)(nnz ? nnz : 1));
	int p = 0;
	for (int i = 0; i < b->n; ++i) {
		orc_row *r = &b->rows[i];
		/* insertion sort by column */
		for (int k = 1; k < r->n; ++k) {
			int c = r->c[k]; double v = r->v[k]; int q = k - 1;
			while (q >= 0 && r->c[q] > c) { r->c[q + 1] = r->c[q]; r->v[q + 1] = r->v[q]; --q; }
			r->c[q + 1] = c; r->v[q + 1] = v;
		}
		A->ptr[i] = p;
		for (int k = 0; k < r->n; ++k) { A->col[p] = r->c[k]; A->val[p] = r->v[k]; ++p; }
		free(r->c); free(r->v);
	}
	A->ptr[b->n] = p;
	free(b->rows); free(b);
}

/* -------------------------------------------------------------- ILU(0) --- */
static int ilu0_build(orc_csr *A)
{
	int n = A->n, nnz = orc_csr_nnz(A);
	A->ilu = (double *)malloc(sizeof(double) * (size_t)(nnz ? nnz : 1));
	A->diag = (int *)malloc(sizeof(int) * (size_t)n);
	memcpy(A->ilu, A->val, sizeof(double) * (size_t)nnz);
	int *pos = (int *)malloc(sizeof(int) * (size_t)A->m);
	for (int j = 0; j < A->m; ++j) pos[j] = -1;
	for (int i = 0; i < n; ++i) {
		A->diag[i] = -1;
		for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) {
			pos[A->col[k]] = k;
			if (A->col[k] == i) A->diag[i] = k;
		}
		if (A->diag[i] < 0) { free(pos); return -1; }
		for (int k = A->ptr[i]; k < A->ptr[i + 1] && A->col[k] < i; ++k) {
			int r = A->col[k];
			double lik = A->ilu[k] / A->ilu[A->diag[r]];
			A->ilu[k] = lik;
			for (int q = A->diag[r] + 1; q < A->ptr[r + 1]; ++q) {
				int p = pos[A->col[q]];
				if (p >= 0) A->ilu[p] -= lik * A->ilu[q];
			}
		}
		for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) pos[A->col[k]] = -1;
		if (A->ilu[A->diag[i]] == 0.0) { free(pos); return -1; }
	}
	free(pos);
	return 0;
}

static void ilu0_apply(const orc_csr *A, double *z, const double *v)
{
	int n = A->n;
	for (int i = 0; i < n; ++i) {
		double s = v[i];
		for (int k = A->ptr[i]; k < A->diag[i]; ++k) s -= A->ilu[k] * z[A->col[k]];
		z[i] = s;
	}
	for (int i = n - 1; i >= 0; --i) {
		double s = z[i];
		for (int k = A->diag[i] + 1; k < A->ptr[i + 1]; ++k) s -= A->ilu[k] * z[A->col[k]];
		z[i] = s / A->ilu[A->diag[i]];
	}
}

static double dot(const double *a, const double *b, int n)
{
	double s = 0.0;
	for (int i = 0; i < n; ++i) s += a[i] * b[i];
	return s;
}

/* Restarted GMRES(m), right-preconditioned with ILU(0), modified
 * Gram-Schmidt, Givens rotations; zero initial guess. */
int orc_csr_solve(orc_csr *A, double *x, const double *b)
{
	int n = A->n, m = g_restart;
	if (!A->ilu && ilu0_build(A) != 0) return -1;
	double *V = (double *)malloc(sizeof(double) * (size_t)n * (size_t)(m + 1));
	double *Z = (double *)malloc(sizeof(double) * (size_t)n * (size_t)m);
	double *w = (double *)malloc(sizeof(double) * (size_t)n);
	double *H = (double *)calloc((size_t)(m + 1) * (size_t)m, sizeof(double));
	double *cs = (double *)malloc(sizeof(double) * (size_t)m);
	double *sn = (double *)malloc(sizeof(double) * (size_t)m);
	double *g = (double *)malloc(sizeof(double) * (size_t)(m + 1));
	double *y = (double *)malloc(sizeof(double) * (size_t)m);
	for (int i = 0; i < n; ++i) x[i] = 0.0;
	double bn = sqrt(dot(b, b, n));
	int it = 0;
	double prev = INFINITY;
	g_last_res = 0.0;
	if (bn == 0.0) goto done;
	for (;;) {
		orc_csr_mult(A, w, x);
		for (int i = 0; i < n; ++i) w[i] = b[i] - w[i];
		double beta = sqrt(dot(w, w, n));
		g_last_res = beta / bn;
		if (g_last_res <= g_tol || it >= g_maxit || !(beta < 0.999 * prev)) break;
		prev = beta;
		for (int i = 0; i < n; ++i) V[i] = w[i] / beta;
		memset(g, 0, sizeof(double) * (size_t)(m + 1));
		g[0] = beta;
		int j;
		for (j = 0; j < m && it < g_maxit; ++j, ++it) {
			double *vj = V + (size_t)j * n, *zj = Z + (size_t)j * n;
			ilu0_apply(A, zj, vj);
			orc_csr_mult(A, w, zj);
			for (int i = 0; i <= j; ++i) {
				double *vi = V + (size_t)i * n;
				double h = dot(w, vi, n);
				H[i * m + j] = h;
				for (int q = 0; q < n; ++q) w[q] -= h * vi[q];
			}
			double hn = sqrt(dot(w, w, n));
			H[(j + 1) * m + j] = hn;
			if (hn > 0.0) {
				double *vn = V + (size_t)(j + 1) * n;
				for (int q = 0; q < n; ++q) vn[q] = w[q] / hn;
			}
			for (int i = 0; i < j; ++i) {
				double a = H[i * m + j], c = H[(i + 1) * m + j];
				H[i * m + j] = cs[i] * a + sn[i] * c;
				H[(i + 1) * m + j] = -sn[i] * a + cs[i] * c;
			}
			double a = H[j * m + j], c = H[(j + 1) * m + j];
			double r = hypot(a, c);
			cs[j] = r > 0 ? a / r : 1.0; sn[j] = r > 0 ? c / r : 0.0;
			H[j * m + j] = r; H[(j + 1) * m + j] = 0.0;
			g[j + 1] = -sn[j] * g[j]; g[j] = cs[j] * g[j];
			if (fabs(g[j + 1]) <= 0.1 * g_tol * bn || hn == 0.0) { ++j; ++it; break; }
		}
		for (int i = j - 1; i >= 0; --i) {
			double s = g[i];
			for (int k = i + 1; k < j; ++k) s -= H[i * m + k] * y[k];
			y[i] = s / H[i * m + i];
		}
		for (int i = 0; i < j; ++i) {
			double *zi = Z + (size_t)i * n;
			for (int q = 0; q < n; ++q) x[q] += y[i] * zi[q];
		}
	}
done:
	free(V); free(Z); free(w); free(H); free(cs); free(sn); free(g); free(y);
	return it;
}
