/*
 * orc_assemble.c -- oracle restatement of the reference's P1 assembly on the
 * sphere.  TEST INFRASTRUCTURE ONLY (see phelm_oracle.h).
 *
 * Restated reference pieces (arithmetic order kept so results match the
 * reference bit for bit on the same platform):
 *   Polynom apply / diff / product / difference  src/polynom.cpp:63-87, 147-184, 667-714
 *   P1 basis in a zone chart                     src/mesh.cpp:563-607
 *   integrate1 (two-trapezoid split)             src/polynom.cpp:188-315
 *   trapezoid integrals (exact / cos / 1/cos)    src/util.cpp:99-227
 *   Gauss-Kronrod 15 on an interval              src/quadrature.c:48-128
 *   7-point degree-5 triangle cubature           src/quadrature.c:130-171
 *   slaplace form                                src/slaplace.cpp:75-105
 *   SphereLaplace matrices                       src/slaplace.cpp:120-200, src/impl/slaplace_impl.h:133-145
 *   SphereJacobian matrices                      src/sjacobian.cpp:53-134, 413-454
 *   SphereNorm full matrix                       src/norm.h:70-73, src/phelm.cpp:330-335
 *   generate_matrix / _boundary / _full          src/generators.cpp:57-212, src/generators.h:200-234
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "phelm_oracle.h"
#include "orc_internal.h"

double orc_ipow(double x, int n)
{
	double r = 1.0;
	for (int i = 0; i < n; ++i) r *= x;
	return r;
}

/* ---------------------------------------------------------- polynomial --- */
#define KOEF(p, i, j) ((p)->k[(i) * ((p)->yd + 1) + (j)])

static double poly_k(const orc_poly *p, int i, int j)
{
	if (i > p->xd || j > p->yd) return 0;
	return KOEF(p, i, j);
}

static void poly_init(orc_poly *p, int xd, int yd)
{
	memset(p, 0, sizeof(*p));
	p->xd = (short)xd; p->yd = (short)yd;
}

double orc_poly_apply(const orc_poly *p, double x, double y)
{
	double xi[ORC_PMAX], yj[ORC_PMAX], r = 0.0;
	for (int i = 0; i <= p->xd; i++) xi[i] = orc_ipow(x, i);
	for (int i = 0; i <= p->yd; i++) yj[i] = orc_ipow(y, i);
	for (int i = 0; i <= p->xd; i++)
		for (int j = 0; j <= p->yd; j++) {
			double k = KOEF(p, i, j);
			r += k * xi[i] * yj[j];
		}
	return r;
}

void orc_poly_mul(orc_poly *r, const orc_poly *a, const orc_poly *b)
{
	poly_init(r, a->xd + b->xd, a->yd + b->yd);
	int deg = r->yd;
	for (int i = 0; i <= a->xd; ++i)
		for (int j = 0; j <= a->yd; ++j)
			for (int k = 0; k <= b->xd; ++k)
				for (int m = 0; m <= b->yd; ++m)
					r->k[(i + k) * (deg + 1) + (j + m)] +=
						a->k[i * (a->yd + 1) + j] * b->k[k * (b->yd + 1) + m];
}

static void poly_sub(orc_poly *r, const orc_poly *a, const orc_poly *b)
{
	poly_init(r, a->xd > b->xd ? a->xd : b->xd, a->yd > b->yd ? a->yd : b->yd);
	for (int i = 0; i <= r->xd; ++i)
		for (int j = 0; j <= r->yd; ++j)
			KOEF(r, i, j) = poly_k(a, i, j) - poly_k(b, i, j);
}

void orc_poly_diff(orc_poly *r, const orc_poly *p, int d)
{
	int deg = p->yd;
	if (d == 0) {
		poly_init(r, p->xd - 1, p->yd);
		for (int j = 0; j <= r->yd; ++j)
			for (int i = 0; i <= r->xd; ++i)
				r->k[i * (r->yd + 1) + j] = (double)(i + 1) * p->k[(i + 1) * (deg + 1) + j];
	} else {
		poly_init(r, p->xd, p->yd - 1);
		for (int i = 0; i <= r->xd; ++i)
			for (int j = 0; j <= r->yd; ++j)
				r->k[i * (r->yd + 1) + j] = (double)(j + 1) * p->k[i * (deg + 1) + j + 1];
	}
}

/* (x - p1.x)(p2.y - p1.y) - (y - p1.y)(p2.x - p1.x) */
static void poly_line(orc_poly *r, double p1x, double p1y, double p2x, double p2y)
{
	orc_poly a, b;
	poly_init(&a, 1, 0); a.k[0] = 0.0; a.k[1] = 1.0;
	a.k[0] -= p1x;
	double d = p2y - p1y;
	for (int i = 0; i < 2; ++i) a.k[i] *= d;
	poly_init(&b, 0, 1); b.k[0] = 0.0; b.k[1] = 1.0;
	b.k[0] -= p1y;
	double e = p2x - p1x;
	for (int i = 0; i < 2; ++i) b.k[i] *= e;
	poly_sub(r, &a, &b);
}

void orc_basis1(const orc_mesh *m, int t, int z, orc_poly phi[3])
{
	const int *v = m->tri + 3 * t;
	double x[3], y[3];
	for (int q = 0; q < 3; ++q) {
		x[q] = m->uv[8 * (size_t)v[q] + 2 * z];
		y[q] = m->uv[8 * (size_t)v[q] + 2 * z + 1];
	}
	poly_line(&phi[0], x[1], y[1], x[2], y[2]);
	poly_line(&phi[1], x[0], y[0], x[2], y[2]);
	poly_line(&phi[2], x[0], y[0], x[1], y[1]);
	for (int q = 0; q < 3; ++q) {
		double k1 = 1.0 / orc_poly_apply(&phi[q], x[q], y[q]);
		int n = (phi[q].xd + 1) * (phi[q].yd + 1);
		for (int i = 0; i < n; ++i) phi[q].k[i] *= k1;
	}
}

/* ---------------------------------------------------------- quadrature --- */
/* Kronrod 15-point nodes/weights as the reference tabulates them (15 digits). */
static const double k15n[15][2] = {
	{ +0.949107912342759, 0.063092092629979 }, { -0.949107912342759, 0.063092092629979 },
	{ +0.741531185599394, 0.140653259715525 }, { -0.741531185599394, 0.140653259715525 },
	{ +0.405845151377397, 0.190350578064785 }, { -0.405845151377397, 0.190350578064785 },
	{ 0.000000000000000, 0.209482141084728 },
	{ +0.991455371120813, 0.022935322010529 }, { -0.991455371120813, 0.022935322010529 },
	{ +0.864864423359769, 0.104790010322250 }, { -0.864864423359769, 0.104790010322250 },
	{ +0.586087235467691, 0.169004726639267 }, { -0.586087235467691, 0.169004726639267 },
	{ +0.207784955007898, 0.204432940075298 }, { -0.207784955007898, 0.204432940075298 },
};

double orc_gauss_kronrod15(double a, double b, orc_fx f, void *d)
{
	double k15 = 0.0, p1 = 0.5 * (b - a), p2 = 0.5 * (b + a);
	for (int i = 0; i < 7; ++i) {
		double f1 = f(p1 * k15n[i][0] + p2, d);
		k15 += k15n[i][1] * f1;
	}
	for (int i = 7; i < 15; ++i) k15 += k15n[i][1] * f(p1 * k15n[i][0] + p2, d);
	k15 *= p1;
	return k15;
}

/* Radon's 7-point degree-5 rule (Stroud T2:5-1) with the reference's
 * 16-digit barycentric nodes and weights. */
static const double w7[7] = {
	0.225, 0.1259391805448265, 0.1259391805448265, 0.1259391805448265,
	0.1323941527885112, 0.1323941527885112, 0.1323941527885112,
};
#define A1 0.7974269853530880
#define B1 0.1012865073234560
#define A2 0.0597158717897742
#define B2 0.4701420641051129
static const double c7[7][3] = {
	{ 1. / 3., 1. / 3., 1. / 3. }, { A1, B1, B1 }, { B1, A1, B1 }, { B1, B1, A1 },
	{ A2, B2, B2 }, { B2, A2, B2 }, { B2, B2, A2 },
};

double orc_cubature7(double x1, double y1, double x2, double y2, double x3, double y3,
                     orc_fxy f, void *d)
{
	double s = 0.0;
	for (int i = 0; i < 7; ++i) {
		double a = c7[i][0], b = c7[i][1], c = c7[i][2];
		double u = a * x1 + b * x2 + c * x3;
		double v = a * y1 + b * y2 + c * y3;
		s += w7[i] * f(u, v, d);
	}
	s *= 0.5 * fabs(((x1 - x3) * (y2 - y3) - (y1 - y3) * (x2 - x3)));
	return s;
}

/* binomial coefficients (the reference reads them from a table) */
static double cnk(int n, int k)
{
	double r = 1.0;
	for (int i = 1; i <= k; ++i) r = r * (double)(n - k + i) / (double)i;
	return r;
}

static double ssum(double x, int k, int n, double k1, double b1, double k2, double b2)
{
	double sum1 = 0, sum2 = 0;
	if (k2 && b2) {
		for (int i = 0; i <= n + 1; i++)
			sum1 += cnk(n + 1, i) * orc_ipow(k2, n + 1 - i) * orc_ipow(x, n + k + 2 - i)
			        * orc_ipow(b2, i) / (double)(n + k + 2 - i);
	} else if (k2 && !b2) {
		sum1 = orc_ipow(k2, n + 1) * orc_ipow(x, k + n + 2) / (double)(k + n + 2);
	} else if (!k2 && b2) {
		sum1 = orc_ipow(b2, n + 1) * orc_ipow(x, k + 1) / (double)(k + 1);
	}
	if (k1 && b1) {
		for (int i = 0; i <= n + 1; i++)
			sum2 += cnk(n + 1, i) * orc_ipow(k1, n + 1 - i) * orc_ipow(x, n + k + 2 - i)
			        * orc_ipow(b1, i) / (double)(n + k + 2 - i);
	} else if (k1 && !b1) {
		sum2 = orc_ipow(k1, n + 1) * orc_ipow(x, k + n + 2) / (double)(k + n + 2);
	} else if (!k1 && b1) {
		sum2 = orc_ipow(b1, n + 1) * orc_ipow(x, k + 1) / (double)(k + 1);
	}
	return sum1 - sum2;
}

double orc_trapezoid_integral(int k, int n, double k1, double b1, double k2, double b2,
                              double x1, double x3)
{
	return (ssum(x3, k, n, k1, b1, k2, b2) - ssum(x1, k, n, k1, b1, k2, b2)) / (double)(n + 1);
}

typedef struct { int k, n; double k1, b1, k2, b2; } trap_data;

static double f_cos(double x, void *vd)
{
	trap_data *d = (trap_data *)vd;
	double pt1 = (orc_ipow((d->k2 * x + d->b2), d->n + 1) - orc_ipow((d->k1 * x + d->b1), d->n + 1)) / (double)(d->n + 1);
	return orc_ipow(x, d->k) * pt1 * cos(x);
}

static double f_sin(double x, void *vd)
{
	trap_data *d = (trap_data *)vd;
	double pt1 = (orc_ipow((d->k2 * x + d->b2), d->n + 1) - orc_ipow((d->k1 * x + d->b1), d->n + 1)) / (double)(d->n + 1);
	return orc_ipow(x, d->k) * pt1 * sin(x);
}

static double f_1_cos(double x, void *vd)
{
	trap_data *d = (trap_data *)vd;
	double pt1 = (orc_ipow((d->k2 * x + d->b2), d->n + 1) - orc_ipow((d->k1 * x + d->b1), d->n + 1)) / (double)(d->n + 1);
	return orc_ipow(x, d->k) * pt1 / cos(x);
}

double orc_trapezoid_cos(int k, int n, double k1, double b1, double k2, double b2, double x1, double x3)
{
	trap_data d = { k, n, k1, b1, k2, b2 };
	return orc_gauss_kronrod15(x1, x3, f_cos, &d);
}

double orc_trapezoid_sin(int k, int n, double k1, double b1, double k2, double b2, double x1, double x3)
{
	trap_data d = { k, n, k1, b1, k2, b2 };
	return orc_gauss_kronrod15(x1, x3, f_sin, &d);
}

double orc_trapezoid_1_cos(int k, int n, double k1, double b1, double k2, double b2, double x1, double x3)
{
	trap_data d = { k, n, k1, b1, k2, b2 };
	return orc_gauss_kronrod15(x1, x3, f_1_cos, &d);
}

/* Integral of p over the planar triangle (x[q], y[q]) split into two
 * trapezoids by the vertical line through the middle vertex. */
double orc_integrate1(const orc_poly *p, const double xs[3], const double ys[3], orc_trap_fn trapezoid)
{
	double k1, b1, k2, b2, k3, b3, t;
	double x1 = xs[0], x2 = xs[1], x3 = xs[2], y1 = ys[0], y2 = ys[1], y3 = ys[2];
	double int1 = 0.0, int2 = 0.0;
	if (x1 <= x2 && x2 <= x3) {
		t = x2; x2 = x3; x3 = t; t = y2; y2 = y3; y3 = t;
	} else if (x2 <= x1 && x1 <= x3) {
		t = x1; x1 = x2; x2 = t; t = x2; x2 = x3; x3 = t;
		t = y1; y1 = y2; y2 = t; t = y2; y2 = y3; y3 = t;
	} else if (x2 <= x3 && x3 <= x1) {
		t = x1; x1 = x2; x2 = t; t = y1; y1 = y2; y2 = t;
	} else if (x3 <= x1 && x1 <= x2) {
		t = x1; x1 = x3; x3 = t; t = y1; y1 = y3; y3 = t;
	} else if (x3 <= x2 && x2 <= x1) {
		t = x1; x1 = x3; x3 = t; t = x2; x2 = x3; x3 = t;
		t = y1; y1 = y3; y3 = t; t = y2; y2 = y3; y3 = t;
	}
	k1 = (y2 - y1) / (x2 - x1);
	b1 = (y1 * x2 - x1 * y2) / (x2 - x1);
	int xd = p->xd, yd = p->yd;
	if (fabs(x1 - x3) > 1e-15) {
		k3 = (y3 - y1) / (x3 - x1);
		b3 = (y1 * x3 - x1 * y3) / (x3 - x1);
		for (int k = 0; k <= xd; ++k)
			for (int n = 0; n <= yd; ++n)
				int1 += p->k[k * (yd + 1) + n] * trapezoid(k, n, k1, b1, k3, b3, x1, x3);
	} else {
		int1 = 0;
	}
	if (fabs(x3 - x2) > 1e-15) {
		k2 = (y2 - y3) / (x2 - x3);
		b2 = (y3 * x2 - x3 * y2) / (x2 - x3);
		for (int k = 0; k <= xd; ++k)
			for (int n = 0; n <= yd; ++n)
				int2 += p->k[k * (yd + 1) + n] * trapezoid(k, n, k1, b1, k2, b2, x3, x2);
	} else {
		int2 = 0;
	}
	if (y3 >= y1 && y3 >= y2) return int1 + int2;
	else if (y3 <= y1 && y3 <= y2) return -int1 - int2;
	else if (y3 >= k1 * x3 + b1) return int1 + int2;
	else return -int1 - int2;
}

void orc_tri_coords(const orc_mesh *m, int t, int z, double xs[3], double ys[3])
{
	const int *v = m->tri + 3 * t;
	for (int q = 0; q < 3; ++q) {
		xs[q] = m->uv[8 * (size_t)v[q] + 2 * z];
		ys[q] = m->uv[8 * (size_t)v[q] + 2 * z + 1];
	}
}

double orc_integrate_cos(const orc_poly *p, const orc_mesh *m, int t, int z)
{
	double xs[3], ys[3];
	orc_tri_coords(m, t, z, xs, ys);
	return orc_integrate1(p, xs, ys, orc_trapezoid_cos);
}

double orc_integrate_1_cos(const orc_poly *p, const orc_mesh *m, int t, int z)
{
	double xs[3], ys[3];
	orc_tri_coords(m, t, z, xs, ys);
	return orc_integrate1(p, xs, ys, orc_trapezoid_1_cos);
}

static double apply_cos(double x, double y, void *d)
{
	return cos(x) * orc_poly_apply((const orc_poly *)d, x, y);
}

static double apply_plain(double x, double y, void *d)
{
	return orc_poly_apply((const orc_poly *)d, x, y);
}

static double integrate_generic(const orc_poly *p, const orc_mesh *m, int t, int z, int with_cos)
{
	double xs[3], ys[3];
	orc_tri_coords(m, t, z, xs, ys);
	return orc_cubature7(xs[0], ys[0], xs[1], ys[1], xs[2], ys[2],
	                     with_cos ? apply_cos : apply_plain, (void *)p);
}

/* slaplace(phi_i, phi_j) = -int cos dx phi_i dx phi_j - int 1/cos dy phi_i dy phi_j */
double orc_slaplace(const orc_poly *pi, const orc_poly *pj, const orc_mesh *m, int t, int z)
{
	orc_poly a, b, prod;
	orc_poly_diff(&a, pi, 0); orc_poly_diff(&b, pj, 0);
	orc_poly_mul(&prod, &a, &b);
	double l1 = -orc_integrate_cos(&prod, m, t, z);
	orc_poly_diff(&a, pi, 1); orc_poly_diff(&b, pj, 1);
	orc_poly_mul(&prod, &a, &b);
	double l2 = -orc_integrate_1_cos(&prod, m, t, z);
	return (l1 + l2);
}

double orc_mass_cos(const orc_poly *pi, const orc_poly *pj, const orc_mesh *m, int t, int z)
{
	orc_poly prod;
	orc_poly_mul(&prod, pi, pj);
	return orc_integrate_cos(&prod, m, t, z);
}

/* ---------------------------------------------------------- callbacks --- */
enum {
	CB_MASS_COS, CB_SLAPL_JI, CB_NEG_SLAPL_JI, CB_JMASS, CB_D1, CB_D2, CB_D1C, CB_D2C, CB_BV
};

typedef struct { int kind; double c1, c2; } cb_t;

static double eval_cb(const cb_t *cb, const orc_poly *pi, const orc_poly *pj,
                      const orc_mesh *m, int t, int z)
{
	orc_poly prod, dj;
	switch (cb->kind) {
	case CB_MASS_COS: return orc_mass_cos(pi, pj, m, t, z);
	case CB_SLAPL_JI: return orc_slaplace(pj, pi, m, t, z);
	case CB_NEG_SLAPL_JI: return -orc_slaplace(pj, pi, m, t, z);
	case CB_JMASS: orc_poly_mul(&prod, pi, pj); return integrate_generic(&prod, m, t, z, 1);
	case CB_D1: orc_poly_diff(&dj, pj, 0); orc_poly_mul(&prod, &dj, pi); return 1 * integrate_generic(&prod, m, t, z, 0);
	case CB_D2: orc_poly_diff(&dj, pj, 1); orc_poly_mul(&prod, &dj, pi); return 1 * integrate_generic(&prod, m, t, z, 0);
	case CB_D1C: orc_poly_diff(&dj, pj, 0); orc_poly_mul(&prod, &dj, pi); return 1 * integrate_generic(&prod, m, t, z, 1);
	case CB_D2C: orc_poly_diff(&dj, pj, 1); orc_poly_mul(&prod, &dj, pi); return 1 * integrate_generic(&prod, m, t, z, 1);
	case CB_BV: {
		/* examples/barvortex_impl.h:57-78 (c1 = 1/tau + sigma theta,
		 * c2 = -theta mu) and :80-101 for the backward form */
		double pt1 = orc_mass_cos(pi, pj, m, t, z);
		pt1 *= cb->c1;
		double pt2 = orc_slaplace(pj, pi, m, t, z);
		pt2 *= cb->c2;
		return pt1 + pt2;
	}
	}
	return 0.0;
}

int orc_row_zone(const orc_mesh *m, int p) { return m->tz[m->adj[m->adj_ptr[p]]]; }

int orc_tri_pos(const orc_mesh *m, int t, int p)
{
	for (int q = 0; q < 3; ++q) if (m->tri[3 * t + q] == p) return q;
	abort();
	return -1;
}

static void gen_matrix(orc_csr *A, const orc_mesh *m, const cb_t *cb)
{
	orc_builder *b = orc_builder_new(m->rs, m->rs);
	#pragma omp parallel for schedule(dynamic, 64)
	for (int i = 0; i < m->rs; ++i) {
		int p = m->inner[i], zone = orc_row_zone(m, p);
		for (int k = m->adj_ptr[p]; k < m->adj_ptr[p + 1]; ++k) {
			int t = m->adj[k];
			orc_poly phi[3];
			orc_basis1(m, t, zone, phi);
			const orc_poly *pi = &phi[orc_tri_pos(m, t, p)];
			for (int i0 = 0; i0 < 3; ++i0) {
				int p2 = m->tri[3 * t + i0];
				if (m->bnd[p2]) continue;
				orc_builder_add(b, i, m->p2io[p2], eval_cb(cb, pi, &phi[i0], m, t, zone));
			}
		}
	}
	orc_builder_finish(b, A);
}

static void gen_boundary_matrix(orc_csr *A, const orc_mesh *m, const cb_t *cb)
{
	orc_builder *b = orc_builder_new(m->rs, m->os);
	for (int j = 0; j < m->os; ++j) {
		int p2 = m->outer[j], zone = orc_row_zone(m, p2);
		for (int k = m->adj_ptr[p2]; k < m->adj_ptr[p2 + 1]; ++k) {
			int t = m->adj[k];
			orc_poly phi[3];
			orc_basis1(m, t, zone, phi);
			const orc_poly *pj = &phi[orc_tri_pos(m, t, p2)];
			for (int i0 = 0; i0 < 3; ++i0) {
				int p = m->tri[3 * t + i0];
				if (m->bnd[p]) continue;
				orc_builder_add(b, m->p2io[p], j, eval_cb(cb, &phi[i0], pj, m, t, zone));
			}
		}
	}
	orc_builder_finish(b, A);
}

static void gen_full_matrix(orc_csr *A, const orc_mesh *m, const cb_t *cb)
{
	orc_builder *b = orc_builder_new(m->V, m->V);
	#pragma omp parallel for schedule(dynamic, 64)
	for (int p = 0; p < m->V; ++p) {
		int zone = orc_row_zone(m, p);
		for (int k = m->adj_ptr[p]; k < m->adj_ptr[p + 1]; ++k) {
			int t = m->adj[k];
			orc_poly phi[3];
			orc_basis1(m, t, zone, phi);
			const orc_poly *pi = &phi[orc_tri_pos(m, t, p)];
			for (int i0 = 0; i0 < 3; ++i0)
				orc_builder_add(b, p, m->tri[3 * t + i0], eval_cb(cb, pi, &phi[i0], m, t, zone));
		}
	}
	orc_builder_finish(b, A);
}

void orc_gen_bv(orc_csr *A, orc_csr *bndA, const orc_mesh *m, double c1, double c2)
{
	cb_t cb = { CB_BV, c1, c2 };
	gen_matrix(A, m, &cb);
	gen_boundary_matrix(bndA, m, &cb);
}

int orc_ops_build(orc_ops *o, const orc_mesh *m)
{
	memset(o, 0, sizeof(*o));
	o->m = m;
	cb_t mass = { CB_MASS_COS, 0, 0 }, sl = { CB_SLAPL_JI, 0, 0 }, nsl = { CB_NEG_SLAPL_JI, 0, 0 };
	cb_t jm = { CB_JMASS, 0, 0 }, d1 = { CB_D1, 0, 0 }, d2 = { CB_D2, 0, 0 };
	cb_t d1c = { CB_D1C, 0, 0 }, d2c = { CB_D2C, 0, 0 };
	gen_matrix(&o->idt, m, &mass);
	gen_matrix(&o->lapl, m, &sl);
	gen_boundary_matrix(&o->bnd1, m, &mass);
	gen_boundary_matrix(&o->bnd2, m, &nsl);
	gen_boundary_matrix(&o->bnd3, m, &sl);
	gen_matrix(&o->jidt, m, &jm);
	gen_matrix(&o->d1, m, &d1);
	gen_matrix(&o->d2, m, &d2);
	gen_matrix(&o->d1c, m, &d1c);
	gen_matrix(&o->d2c, m, &d2c);
	gen_boundary_matrix(&o->d1b, m, &d1);
	gen_boundary_matrix(&o->d2b, m, &d2);
	gen_boundary_matrix(&o->d1cb, m, &d1c);
	gen_boundary_matrix(&o->d2cb, m, &d2c);
	gen_full_matrix(&o->norm, m, &mass);
	return 0;
}

void orc_ops_free(orc_ops *o)
{
	orc_csr *all[] = { &o->idt, &o->lapl, &o->bnd1, &o->bnd2, &o->bnd3, &o->jidt, &o->d1, &o->d2,
	                   &o->d1c, &o->d2c, &o->d1b, &o->d2b, &o->d1cb, &o->d2cb, &o->norm };
	for (size_t i = 0; i < sizeof(all) / sizeof(all[0]); ++i) orc_csr_free(all[i]);
}
