/*
 * phelm_oracle.h -- CPU oracle for the sphere-FEM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * (resetius/mke, "Phelm") algorithm for the icosahedral sphere mesh, the P1
 * SphereLaplace / SphereJacobian / SphereNorm operators, their solves and the
 * barvortex / baroclin Crank-Nicolson steps.  Only the test suite, the smoke
 * check and the CPU-baseline leg of the benchmark may load it; the product
 * library never links or calls it.
 *
 * Parity pin: the restatement is checked against outputs of the reference's
 * own C++ sources compiled here (see oracle/Makefile, target "ref") through
 * golden fixtures under tests/golden/, and against the reference's unit-test
 * known-answer values (tests/test_integrate.cpp, tests/test_quadrature.c).
 *
 * The third-party linear-algebra library the reference calls ("linal",
 * github resetius/linal, not vendored, no pinned version) is restated here by
 * its published role only: an accumulate-then-CSR sparse matrix and a GMRES
 * solve.  Its iteration-level behaviour is unpinned; the oracle solves every
 * system to a relative residual of 1e-13 (restarted GMRES, ILU(0) right
 * preconditioner), i.e. to the exact discrete answer within rounding.
 */
#ifndef PHELM_ORACLE_H
#define PHELM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- CSR --- */
typedef struct {
	int n;        /* rows */
	int m;        /* columns */
	int *ptr;     /* n + 1 */
	int *col;     /* nnz, sorted within each row */
	double *val;  /* nnz */
	/* solver cache (ILU(0) factors), built lazily by orc_csr_solve */
	double *ilu;
	int *diag;
} orc_csr;

int  orc_csr_nnz(const orc_csr *A);
void orc_csr_free(orc_csr *A);
/* y = A x, each row summed in ascending column order starting from 0.0 */
void orc_csr_mult(const orc_csr *A, double *y, const double *x);
/* Solve A x = b (x is overwritten; the initial guess is zero).
 * Returns the number of GMRES iterations, negative on failure. */
int  orc_csr_solve(orc_csr *A, double *x, const double *b);
/* Tolerance / restart used by orc_csr_solve (process-wide). */
void orc_set_solver(double rel_tol, int restart, int max_iter);
double orc_last_residual(void);

/* Accumulating builder: add(i, j, a) sums repeated (i, j) in call order. */
typedef struct orc_builder orc_builder;
orc_builder *orc_builder_new(int n, int m);
void orc_builder_add(orc_builder *b, int i, int j, double a);
/* Moves the accumulated entries into A (sorted columns) and frees b. */
void orc_builder_finish(orc_builder *b, orc_csr *A);

/* --------------------------------------------------------------- mesh --- */
typedef struct {
	int V, T;            /* points, triangles */
	double *xyz;         /* V x 3, global coordinates as loaded */
	double *uv;          /* V x 4 x 2, per-zone local coordinates as loaded */
	int nz;              /* zones per point (4 for the full sphere) */
	int *tri;            /* T x 3, 0-based */
	int *tz;             /* T, 0-based zone */
	int *bnd;            /* V, 1 = boundary */
	int rs, os;          /* inner / outer counts */
	int *inner, *outer, *p2io;
	int *adj_ptr, *adj;  /* point -> triangles (ascending triangle id) */
} orc_mesh;

/* Icosahedron subdivided `level` times, projected to the unit sphere,
 * reordered and written/parsed with 16 decimals exactly as the reference's
 * mesh generator + Mesh::load produce it ("--type full --coord local"). */
int  orc_mesh_sphere(orc_mesh *m, int level);
void orc_mesh_free(orc_mesh *m);

/* --------------------------------------------------------- quadrature --- */
typedef double (*orc_fx)(double x, void *d);
typedef double (*orc_fxy)(double x, double y, void *d);
double orc_gauss_kronrod15(double a, double b, orc_fx f, void *d);
double orc_cubature7(double x1, double y1, double x2, double y2,
                     double x3, double y3, orc_fxy f, void *d);
double orc_trapezoid_integral(int k, int n, double k1, double b1,
                              double k2, double b2, double x1, double x3);
double orc_ipow(double x, int n);
/* integral over a triangle of a polynomial (coefficients k[i*(yd+1)+j]);
 * kind 0 plain, 1 times cos x, 2 times sin x, 3 divided by cos x */
double orc_integrate_poly(int kind, const double xs[3], const double ys[3],
                          int xd, int yd, const double *koef);

/* ----------------------------------------------------------- operators --- */
typedef struct {
	const orc_mesh *m;
	/* SphereLaplace: mass (integrate_cos), Laplacian, boundary columns */
	orc_csr idt, lapl, bnd1, bnd2, bnd3;
	/* SphereJacobian: cubature7 mass, derivative matrices and boundary parts */
	orc_csr jidt, d1, d2, d1c, d2c, d1b, d2b, d1cb, d2cb;
	/* SphereNorm: full sz x sz cos-weighted mass */
	orc_csr norm;
} orc_ops;

int  orc_ops_build(orc_ops *o, const orc_mesh *m);
void orc_ops_free(orc_ops *o);

void orc_u2p(const orc_mesh *m, double *p, const double *u);
void orc_p2u(const orc_mesh *m, double *u, const double *p, const double *bnd);
void orc_proj_bnd(const orc_mesh *m, double *F, const double *u);

void orc_laplace_calc2(orc_ops *o, double *ans, const double *F);
void orc_laplace_calc1(orc_ops *o, double *ans, const double *F, const double *bnd);
void orc_laplace_solve(orc_ops *o, double *ans, const double *F, const double *bnd);
void orc_jacobian_calc2(orc_ops *o, double *ans, const double *u, const double *v);
void orc_jacobian_calc1(orc_ops *o, double *ans, const double *u, const double *v,
                        const double *bnd);
void orc_jacobian_calc1t(orc_ops *o, double *ans, const double *u, const double *v,
                         const double *bnd);
void orc_jacobian_diff_x(orc_ops *o, double *ans, const double *v);
void orc_jacobian_diff_cos_y(orc_ops *o, double *ans, const double *v);
double orc_norm(orc_ops *o, const double *u);
double orc_dist(orc_ops *o, const double *u, const double *v);
double orc_scalar(orc_ops *o, const double *u, const double *v);

/* --------------------------------------------------------------- models --- */
typedef struct {
	double tau, sigma, mu, k1, k2, theta;
	int max_iter;        /* Picard iterations (reference: 1000 with 1e-14 break) */
} orc_bv_conf;

typedef struct {
	orc_ops *o;
	orc_bv_conf c;
	orc_csr A, bndA;     /* forward CN matrix and its boundary columns */
	orc_csr Ab, bndAb;   /* backward matrix Ab_ and bndb_ (linearised inverse step) */
	double *lh;          /* l + h at every point */
	int last_iters;
} orc_barvortex;

/* coriolis[V]: l + h evaluated at each point (caller computes it). */
int  orc_bv_init(orc_barvortex *bv, orc_ops *o, const orc_bv_conf *c,
                 const double *coriolis);
void orc_bv_free(orc_barvortex *bv);
/* One step: u1 <- step(u); bnd_u / bnd_w may be NULL (zero boundary);
 * rp[V] is the forcing f already evaluated at time t (NULL = none). */
void orc_bv_step(orc_barvortex *bv, double *u1, const double *u,
                 const double *bnd_u, const double *bnd_w, const double *rp);
/* Linearised step around the background z, its inverse and its adjoint
 * (BarVortex::calc_L / calc_L_1 / calc_LT).  calc_L1 adds into u1. */
void orc_bv_calc_L(orc_barvortex *bv, double *u1, const double *u, const double *z,
                   const double *bnd_u, const double *bnd_w);
void orc_bv_calc_L1(orc_barvortex *bv, double *u1, const double *u, const double *z,
                    const double *bnd_u, const double *bnd_w);
void orc_bv_calc_LT(orc_barvortex *bv, double *v1, const double *v, const double *z,
                    const double *bnd_u, const double *bnd_w);

typedef struct {
	double tau, sigma, mu, sigma1, mu1, alpha, theta;
	int max_iter;        /* reference: 20 with 1e-8 break */
	double tol;          /* break when max(dist) < tol (reference 1e-8) */
} orc_bc_conf;

typedef struct {
	orc_ops *o;
	orc_bc_conf c;
	orc_csr A;           /* 4 rs x 4 rs block matrix [w1 | w2 | u1 | u2] */
	orc_csr Ab;          /* the backward matrix Ab_ (inverse linearised step) */
	double *lh;
	int last_iters;
} orc_baroclin;

int  orc_bc_init(orc_baroclin *bc, orc_ops *o, const orc_bc_conf *c,
                 const double *coriolis);
void orc_bc_free(orc_baroclin *bc);
/* f, g: forcing fields at the points (NULL = none). */
void orc_bc_step(orc_baroclin *bc, double *u11, double *u21,
                 const double *u1, const double *u2, const double *bnd,
                 const double *f, const double *g);
/* Baroclin::calc_L / calc_L_1 linearised around (z1, z2). */
void orc_bc_calc_L(orc_baroclin *bc, double *u11, double *u21, const double *u1, const double *u2,
                   const double *z1, const double *z2, const double *bnd);
void orc_bc_calc_L1(orc_baroclin *bc, double *u11, double *u21, const double *u1, const double *u2,
                    const double *z1, const double *z2, const double *bnd);

#ifdef __cplusplus
}
#endif
#endif
