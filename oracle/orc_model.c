/*
 * orc_model.c -- oracle restatement of the sphere operators' applies/solves
 * and of the barvortex / baroclin time steps.  TEST INFRASTRUCTURE ONLY.
 *
 *   u2p / p2u / proj_bnd            src/proj.cpp:49-160
 *   SphereLaplace::calc2/calc1/solve src/impl/slaplace_impl.h:84-192
 *   SphereJacobian::calc2 (4 splittings, 16 mass solves in the reference;
 *     the 8 distinct ones are solved once -- identical results since every
 *     solve is deterministic)       src/sjacobian.cpp:136-362, 456-461
 *   SphereNorm norm/dist/scalar      src/norm.h:81-94, src/mesh.h:550-591
 *   BarVortex ctor + calc            examples/barvortex_impl.h:57-154, 171-310
 *   Baroclin ctor + calc             examples/baroclin.cpp:69-606
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "phelm_oracle.h"
#include "orc_internal.h"

#define VEC(n) ((double *)calloc((size_t)((n) > 0 ? (n) : 1), sizeof(double)))

void orc_u2p(const orc_mesh *m, double *p, const double *u)
{
	for (int i = 0; i < m->rs; ++i) p[i] = u[m->inner[i]];
}

void orc_p2u(const orc_mesh *m, double *u, const double *p, const double *bnd)
{
	for (int i = 0; i < m->V; ++i) {
		if (m->bnd[i]) u[i] = bnd ? bnd[m->p2io[i]] : 0;
		else u[i] = p[m->p2io[i]];
	}
}

void orc_proj_bnd(const orc_mesh *m, double *F, const double *u)
{
	for (int i = 0; i < m->os; ++i) F[i] = u[m->outer[i]];
}

void orc_laplace_calc2(orc_ops *o, double *ans, const double *F)
{
	const orc_mesh *m = o->m;
	double *in = VEC(m->rs), *out = VEC(m->rs), *tmp = VEC(m->os);
	orc_u2p(m, in, F);
	orc_proj_bnd(m, tmp, F);
	orc_csr_mult(&o->lapl, out, in);
	orc_csr_mult(&o->bnd3, in, tmp);
	for (int i = 0; i < m->rs; ++i) out[i] = out[i] + in[i];
	orc_csr_solve(&o->idt, ans, out);
	free(in); free(out); free(tmp);
}

void orc_laplace_calc1(orc_ops *o, double *ans, const double *F, const double *bnd)
{
	double *p1 = VEC(o->m->rs);
	orc_laplace_calc2(o, p1, F);
	orc_p2u(o->m, ans, p1, bnd);
	free(p1);
}

void orc_laplace_solve(orc_ops *o, double *ans, const double *F, const double *bnd)
{
	const orc_mesh *m = o->m;
	double *b = VEC(m->rs), *x = VEC(m->rs);
	orc_u2p(m, x, F);
	orc_csr_mult(&o->idt, b, x);
	if (bnd) {
		orc_csr_mult(&o->bnd2, x, bnd);
		for (int i = 0; i < m->rs; ++i) b[i] = b[i] + x[i];
	}
	orc_csr_solve(&o->lapl, x, b);
	orc_p2u(m, ans, x, bnd);
	free(b); free(x);
}

/* M_J^{-1} (D f_in + D_bnd f_bnd) */
static void jderiv(orc_ops *o, orc_csr *D, orc_csr *Db, double *out,
                   const double *f_in, const double *f_bnd)
{
	int rs = o->m->rs;
	double *tmp = VEC(rs), *rp = VEC(rs);
	orc_csr_mult(D, tmp, f_in);
	orc_csr_mult(Db, rp, f_bnd);
	for (int i = 0; i < rs; ++i) rp[i] = rp[i] + tmp[i];
	orc_csr_solve(&o->jidt, out, rp);
	free(tmp); free(rp);
}

void orc_jacobian_calc2(orc_ops *o, double *ans, const double *u, const double *v)
{
	const orc_mesh *m = o->m;
	int rs = m->rs;
	double *ui = VEC(rs), *vi = VEC(rs), *ub = VEC(m->os), *vb = VEC(m->os);
	orc_u2p(m, vi, v); orc_u2p(m, ui, u);
	orc_proj_bnd(m, vb, v); orc_proj_bnd(m, ub, u);
	double *c2u = VEC(rs), *a1v = VEC(rs), *c1u = VEC(rs), *a2v = VEC(rs);
	double *a2u = VEC(rs), *c1v = VEC(rs), *a1u = VEC(rs), *c2v = VEC(rs);
	jderiv(o, &o->d2c, &o->d2cb, c2u, ui, ub);
	jderiv(o, &o->d1, &o->d1b, a1v, vi, vb);
	jderiv(o, &o->d1c, &o->d1cb, c1u, ui, ub);
	jderiv(o, &o->d2, &o->d2b, a2v, vi, vb);
	jderiv(o, &o->d2, &o->d2b, a2u, ui, ub);
	jderiv(o, &o->d1c, &o->d1cb, c1v, vi, vb);
	jderiv(o, &o->d1, &o->d1b, a1u, ui, ub);
	jderiv(o, &o->d2c, &o->d2cb, c2v, vi, vb);
	for (int i = 0; i < rs; ++i) {
		double j1 = c2u[i] * a1v[i] - c1u[i] * a2v[i];
		double j2 = a2u[i] * c1v[i] - a1u[i] * c2v[i];
		double j3 = c2u[i] * a1v[i] - a1u[i] * c2v[i];
		double j4 = a2u[i] * c1v[i] - c1u[i] * a2v[i];
		double s = j1;
		s = s + j2;
		s = s + j3;
		s = s + j4;
		ans[i] = 0.25 * s;
	}
	free(ui); free(vi); free(ub); free(vb);
	free(c2u); free(a1v); free(c1u); free(a2v); free(a2u); free(c1v); free(a1u); free(c2v);
}

void orc_jacobian_calc1(orc_ops *o, double *ans, const double *u, const double *v, const double *bnd)
{
	double *p1 = VEC(o->m->rs);
	orc_jacobian_calc2(o, p1, u, v);
	orc_p2u(o->m, ans, p1, bnd);
	free(p1);
}

/* SphereJacobian::calc1t (src/sjacobian.cpp:463-468 with calc2t :404-408):
 * -J(u, v) on the inner points, boundary values bnd */
void orc_jacobian_calc1t(orc_ops *o, double *ans, const double *u, const double *v, const double *bnd)
{
	int rs = o->m->rs;
	double *p1 = VEC(rs);
	orc_jacobian_calc2(o, p1, u, v);
	for (int i = 0; i < rs; ++i) p1[i] = p1[i] * -1.0;
	orc_p2u(o->m, ans, p1, bnd);
	free(p1);
}

/* SphereJacobian::calc2_diff_x / calc2_diff_cos_y (src/sjacobian.cpp:364-402):
 * M_J^{-1} (D1 v_in + D1_bnd v_bnd) and M_J^{-1} (D2cos v_in + D2cos_bnd v_bnd) */
static void jac_diff(orc_ops *o, orc_csr *D, orc_csr *Db, double *ans, const double *v)
{
	const orc_mesh *m = o->m;
	double *vi = VEC(m->rs), *vb = VEC(m->os);
	orc_u2p(m, vi, v);
	orc_proj_bnd(m, vb, v);
	jderiv(o, D, Db, ans, vi, vb);
	free(vi); free(vb);
}

void orc_jacobian_diff_x(orc_ops *o, double *ans, const double *v) { jac_diff(o, &o->d1, &o->d1b, ans, v); }

void orc_jacobian_diff_cos_y(orc_ops *o, double *ans, const double *v) { jac_diff(o, &o->d2c, &o->d2cb, ans, v); }

double orc_scalar(orc_ops *o, const double *u, const double *v)
{
	int sz = o->m->V;
	double *tmp = VEC(sz), s = 0;
	orc_csr_mult(&o->norm, tmp, v);
	for (int i = 0; i < sz; ++i) s += u[i] * tmp[i];
	free(tmp);
	return s;
}

double orc_norm(orc_ops *o, const double *u) { return sqrt(orc_scalar(o, u, u)); }

double orc_dist(orc_ops *o, const double *u, const double *v)
{
	int sz = o->m->V;
	double *d = VEC(sz);
	for (int i = 0; i < sz; ++i) d[i] = u[i] - v[i];
	double r = orc_norm(o, d);
	free(d);
	return r;
}

/* ------------------------------------------------------------ barvortex --- */
int orc_bv_init(orc_barvortex *bv, orc_ops *o, const orc_bv_conf *c, const double *coriolis)
{
	memset(bv, 0, sizeof(*bv));
	bv->o = o; bv->c = *c;
	int V = o->m->V;
	bv->lh = VEC(V);
	if (coriolis) memcpy(bv->lh, coriolis, sizeof(double) * (size_t)V);
	orc_gen_bv(&bv->A, &bv->bndA, o->m, 1.0 / c->tau + c->sigma * c->theta, -c->theta * c->mu);
	/* backward matrix Ab_ / bndb_ (examples/barvortex_impl.h:84-105, 150-151) */
	orc_gen_bv(&bv->Ab, &bv->bndAb, o->m, 1.0 / c->tau - c->sigma * (1.0 - c->theta), (1.0 - c->theta) * c->mu);
	return 0;
}

void orc_bv_free(orc_barvortex *bv)
{
	orc_csr_free(&bv->A); orc_csr_free(&bv->bndA);
	orc_csr_free(&bv->Ab); orc_csr_free(&bv->bndAb); free(bv->lh);
	memset(bv, 0, sizeof(*bv));
}

void orc_bv_step(orc_barvortex *bv, double *u1, const double *u,
                 const double *bnd_u, const double *bnd_w, const double *rp_f)
{
	orc_ops *o = bv->o;
	const orc_mesh *m = o->m;
	int rs = m->rs, sz = m->V;
	double k1 = bv->c.k1, k2 = bv->c.k2, theta = bv->c.theta;
	double mu = bv->c.mu, sigma = bv->c.sigma, tau = bv->c.tau;
	double nr0 = orc_norm(o, u);
	double *w = VEC(sz), *dw = VEC(sz), *FC = VEC(sz);
	double *u_n = VEC(sz), *w_n = VEC(sz), *u_n1 = VEC(sz);
	double *tmp1 = VEC(sz), *tmp2 = VEC(sz), *jac = VEC(rs), *F = VEC(rs);
	double *rp = VEC(rs), *x = VEC(rs);

	orc_laplace_calc1(o, w, u, bnd_w);
	orc_laplace_calc1(o, dw, w, NULL);
	for (int i = 0; i < sz; ++i) FC[i] = 1.0 / tau * w[i] + mu * (1.0 - theta) * dw[i];
	for (int i = 0; i < sz; ++i) FC[i] = 1.0 * FC[i] + -sigma * (1.0 - theta) * w[i];
	if (rp_f) for (int i = 0; i < sz; ++i) FC[i] += rp_f[i];

	bv->last_iters = 0;
	for (int it = 0; it < bv->c.max_iter; ++it) {
		for (int i = 0; i < sz; ++i) tmp1[i] = k1 * theta * w_n[i] + k1 * (1.0 - theta) * w[i];
		for (int i = 0; i < sz; ++i) tmp1[i] = tmp1[i] + k2 * bv->lh[i];
		for (int i = 0; i < sz; ++i) tmp2[i] = theta * u_n[i] + (1.0 - theta) * u[i];
		orc_jacobian_calc2(o, jac, tmp2, tmp1);
		for (int i = 0; i < rs; ++i) F[i] = FC[m->inner[i]] - jac[i];
		orc_csr_mult(&o->idt, rp, F);
		if (bnd_w) {
			orc_csr_mult(&bv->bndA, tmp1, bnd_w);
			for (int i = 0; i < rs; ++i) rp[i] = rp[i] + tmp1[i];
		}
		orc_csr_solve(&bv->A, x, rp);
		orc_p2u(m, w_n, x, bnd_w);
		orc_laplace_solve(o, u_n1, w_n, bnd_u);
		double nr = orc_dist(o, u_n1, u_n);
		double *s = u_n1; u_n1 = u_n; u_n = s;
		bv->last_iters = it + 1;
		if (nr / nr0 < 1e-14 || isnan(nr)) break;
	}
	memcpy(u1, u_n, sizeof(double) * (size_t)sz);
	free(w); free(dw); free(FC); free(u_n); free(w_n); free(u_n1);
	free(tmp1); free(tmp2); free(jac); free(F); free(rp); free(x);
}

/* ------------------------------------------- linearised / adjoint steps --- */
/* J^T(u, v) on the full vector: -J(u, v) with boundary values bnd
 * (src/sjacobian.cpp:404-408, 463-468) */
static void jac_calc1t(orc_ops *o, double *ans, const double *u, const double *v, const double *bnd)
{
	orc_jacobian_calc1(o, ans, u, v, NULL);
	double *p = VEC(o->m->rs);
	orc_u2p(o->m, p, ans);
	for (int i = 0; i < o->m->rs; ++i) p[i] = -1.0 * p[i];
	orc_p2u(o->m, ans, p, bnd);
	free(p);
}

/* rp = idt u2p(u) (+ B bnd_w); x = M^-1 rp; ans = p2u(x, bnd_w)
 * (phelm::solve, src/mesh.h:720-746, with the right-hand side of
 * examples/barvortex_impl.h:379-390) */
static void bv_solve(orc_barvortex *bv, double *ans, const double *u, const orc_csr *M, const orc_csr *B,
                     const double *bnd_w)
{
	orc_ops *o = bv->o;
	const orc_mesh *m = o->m;
	int rs = m->rs;
	double *tmp = VEC(rs), *rp = VEC(rs), *x = VEC(rs);
	orc_u2p(m, tmp, u);
	orc_csr_mult(&o->idt, rp, tmp);
	if (bnd_w) {
		orc_csr_mult(B, tmp, bnd_w);
		for (int i = 0; i < rs; ++i) rp[i] = rp[i] + tmp[i];
	}
	orc_csr_solve((orc_csr *)M, x, rp);
	orc_p2u(m, ans, x, bnd_w);
	free(tmp); free(rp); free(x);
}

/* the shared first part of calc_L / calc_L_1 (examples/barvortex_impl.h:343-362) */
static void bv_lin_parts(orc_barvortex *bv, const double *u, const double *z, const double *bnd_w,
                         double *pt1, double *pt3)
{
	orc_ops *o = bv->o;
	int sz = o->m->V;
	double k1 = bv->c.k1, k2 = bv->c.k2;
	double *z_lapl = VEC(sz), *jac1 = VEC(sz), *jac2 = VEC(sz), *jac3 = VEC(sz);
	orc_laplace_calc1(o, z_lapl, z, bnd_w);
	orc_laplace_calc1(o, pt1, u, bnd_w);
	orc_jacobian_calc1(o, jac1, u, bv->lh, NULL);
	orc_jacobian_calc1(o, jac2, z, pt1, NULL);
	orc_jacobian_calc1(o, jac3, u, z_lapl, NULL);
	for (int i = 0; i < sz; ++i) pt3[i] = 0.0;
	for (int i = 0; i < sz; ++i) pt3[i] = pt3[i] + k2 * jac1[i];
	for (int i = 0; i < sz; ++i) pt3[i] = pt3[i] + k1 * jac2[i];
	for (int i = 0; i < sz; ++i) pt3[i] = pt3[i] + k1 * jac3[i];
	free(z_lapl); free(jac1); free(jac2); free(jac3);
}

/* BarVortex::calc_L (examples/barvortex_impl.h:326-400) */
void orc_bv_calc_L(orc_barvortex *bv, double *u1, const double *u, const double *z,
                   const double *bnd_u, const double *bnd_w)
{
	orc_ops *o = bv->o;
	int sz = o->m->V;
	double theta = bv->c.theta, mu = bv->c.mu, sigma = bv->c.sigma, tau = bv->c.tau;
	double *pt1 = VEC(sz), *pt2 = VEC(sz), *pt3 = VEC(sz);
	bv_lin_parts(bv, u, z, bnd_w, pt1, pt3);
	for (int i = 0; i < sz; ++i) pt3[i] = -1.0 * pt3[i];
	orc_laplace_calc1(o, pt2, pt1, NULL);
	for (int i = 0; i < sz; ++i) pt2[i] = (1. - theta) * mu * pt2[i];
	for (int i = 0; i < sz; ++i) pt1[i] = (1.0 / tau - (1. - theta) * sigma) * pt1[i];
	for (int i = 0; i < sz; ++i) u1[i] = 0.0;
	for (int i = 0; i < sz; ++i) u1[i] = u1[i] + pt1[i];
	for (int i = 0; i < sz; ++i) u1[i] = u1[i] + pt2[i];
	for (int i = 0; i < sz; ++i) u1[i] = u1[i] + pt3[i];
	bv_solve(bv, u1, u1, &bv->A, &bv->bndA, bnd_w);
	orc_laplace_solve(o, u1, u1, bnd_u);
	free(pt1); free(pt2); free(pt3);
}

/* BarVortex::calc_L_1 (examples/barvortex_impl.h:402-467); adds into u1 as
 * the reference does (it does not clear u1 first) */
void orc_bv_calc_L1(orc_barvortex *bv, double *u1, const double *u, const double *z,
                    const double *bnd_u, const double *bnd_w)
{
	orc_ops *o = bv->o;
	int sz = o->m->V;
	double theta = bv->c.theta, mu = bv->c.mu, sigma = bv->c.sigma, tau = bv->c.tau;
	double *pt1 = VEC(sz), *pt2 = VEC(sz), *pt3 = VEC(sz);
	bv_lin_parts(bv, u, z, bnd_w, pt1, pt3);
	orc_laplace_calc1(o, pt2, pt1, NULL);
	for (int i = 0; i < sz; ++i) pt2[i] = -theta * mu * pt2[i];
	for (int i = 0; i < sz; ++i) pt1[i] = (1.0 / tau + theta * sigma) * pt1[i];
	for (int i = 0; i < sz; ++i) u1[i] = u1[i] + pt1[i];
	for (int i = 0; i < sz; ++i) u1[i] = u1[i] + pt2[i];
	for (int i = 0; i < sz; ++i) u1[i] = u1[i] + pt3[i];
	bv_solve(bv, u1, u1, &bv->Ab, &bv->bndAb, bnd_w);
	orc_laplace_solve(o, u1, u1, bnd_u);
	free(pt1); free(pt2); free(pt3);
}

/* BarVortex::calc_LT (examples/barvortex_impl.h:469-536) */
void orc_bv_calc_LT(orc_barvortex *bv, double *v1, const double *v, const double *z,
                    const double *bnd_u, const double *bnd_w)
{
	orc_ops *o = bv->o;
	const orc_mesh *m = o->m;
	int sz = m->V;
	double k1 = bv->c.k1, k2 = bv->c.k2;
	double theta = bv->c.theta, mu = bv->c.mu, sigma = bv->c.sigma, tau = bv->c.tau;
	double *lz = VEC(sz), *pt1 = VEC(sz), *pt2 = VEC(sz), *h1 = VEC(sz), *p_lapl = VEC(sz), *tmp = VEC(sz);
	orc_laplace_calc1(o, lz, z, bnd_w);
	orc_laplace_solve(o, v1, v, bnd_u);
	bv_solve(bv, v1, v1, &bv->A, &bv->bndA, bnd_w);
	orc_laplace_calc1(o, pt1, v1, bnd_w);
	for (int i = 0; i < sz; ++i) pt1[i] = (1.0 / tau - (1.0 - theta) * sigma) * pt1[i];
	orc_laplace_calc1(o, pt2, v1, bnd_w);
	orc_laplace_calc1(o, pt2, pt2, NULL);
	for (int i = 0; i < sz; ++i) pt2[i] = (1.0 - theta) * mu * pt2[i];
	jac_calc1t(o, tmp, v1, bv->lh, NULL);
	jac_calc1t(o, p_lapl, z, v1, NULL);
	orc_laplace_calc1(o, p_lapl, p_lapl, NULL);
	jac_calc1t(o, h1, v1, lz, NULL);
	for (int i = 0; i < sz; ++i) h1[i] = k1 * h1[i] + k1 * p_lapl[i];
	for (int i = 0; i < sz; ++i) h1[i] = h1[i] + k2 * tmp[i];
	for (int i = 0; i < sz; ++i) h1[i] = -1.0 * h1[i];
	for (int i = 0; i < sz; ++i) v1[i] = 0.0;
	for (int i = 0; i < sz; ++i) v1[i] = v1[i] + pt1[i];
	for (int i = 0; i < sz; ++i) v1[i] = v1[i] + pt2[i];
	for (int i = 0; i < sz; ++i) v1[i] = v1[i] + h1[i];
	for (int p = 0; p < sz; ++p)   /* set_bnd (src/proj.cpp:110-133) */
		if (m->bnd[p]) v1[p] = bnd_u ? bnd_u[m->p2io[p]] : 0.0;
	free(lz); free(pt1); free(pt2); free(h1); free(p_lapl); free(tmp);
}

/* ------------------------------------------------------------- baroclin --- */
typedef struct { double a, e[9]; int bnd_j; } bc_pair; /* one (row, triangle, vertex) term */

static void bc_elements(const orc_bc_conf *c, double a, double b, double e[9])
{
	double tau = c->tau, mu = c->mu, mu1 = c->mu1, sigma = c->sigma, sigma1 = c->sigma1;
	double alpha = c->alpha, theta = c->theta;
	e[0] = a * (1.0 / tau + 0.5 * theta * sigma) - theta * mu * b;
	e[1] = -0.5 * a * sigma * theta;
	e[2] = 0.5 * theta * sigma * a;
	e[3] = a * (1.0 / tau + 0.5 * theta * sigma + alpha * alpha * theta * mu1) - theta * mu * b;
	e[4] = a * (-alpha * alpha / tau - alpha * alpha * theta * sigma1);
	e[5] = a;
	e[6] = -b;
	e[7] = a;
	e[8] = -b;
}
/* the backward (inverse linearised step) entries, examples/baroclin.cpp:182-243 */
static void bc_elements_back(const orc_bc_conf *c, double a, double b, double e[9])
{
	double tau = c->tau, mu = c->mu, mu1 = c->mu1, sigma = c->sigma, sigma1 = c->sigma1;
	double alpha = c->alpha, theta = c->theta;
	e[0] = a * (1.0 / tau - 0.5 * (1.0 - theta) * sigma) + (1.0 - theta) * mu * b;
	e[1] = 0.5 * a * sigma * (1.0 - theta);
	e[2] = -0.5 * (1.0 - theta) * sigma * a;
	e[3] = a * (1.0 / tau - 0.5 * (1.0 - theta) * sigma - alpha * alpha * (1.0 - theta) * mu1)
	       + (1.0 - theta) * mu * b;
	e[4] = a * (-alpha * alpha / tau + alpha * alpha * (1.0 - theta) * sigma1);
	e[5] = a;
	e[6] = -b;
	e[7] = a;
	e[8] = -b;
}
static void bc_entries(const orc_bc_conf *c, int backward, double a, double b, double e[9])
{
	if (backward) bc_elements_back(c, a, b, e);
	else bc_elements(c, a, b, e);
}
/* element (row block, column block) for e[0..8] (examples/baroclin.cpp:157-177) */
static const int bc_ri[9] = { 0, 0, 1, 1, 1, 2, 2, 3, 3 };
static const int bc_cj[9] = { 0, 1, 0, 1, 3, 0, 2, 1, 3 };

static void bc_assemble(orc_baroclin *bc, int backward, orc_csr *M)
{
	const orc_mesh *m = bc->o->m;
	int rs = m->rs;
	orc_builder *b = orc_builder_new(4 * rs, 4 * rs);
	#pragma omp parallel for schedule(dynamic, 64)
	for (int i = 0; i < rs; ++i) {
		int p = m->inner[i], zone = orc_row_zone(m, p);
		for (int k = m->adj_ptr[p]; k < m->adj_ptr[p + 1]; ++k) {
			int t = m->adj[k];
			orc_poly phi[3];
			orc_basis1(m, t, zone, phi);
			const orc_poly *pi = &phi[orc_tri_pos(m, t, p)];
			for (int i0 = 0; i0 < 3; ++i0) {
				int p2 = m->tri[3 * t + i0];
				if (m->bnd[p2]) continue;
				int j = m->p2io[p2];
				double a = orc_mass_cos(pi, &phi[i0], m, t, zone);
				double bb = orc_slaplace(&phi[i0], pi, m, t, zone);
				double e[9];
				bc_entries(&bc->c, backward, a, bb, e);
				for (int q = 0; q < 9; ++q)
					orc_builder_add(b, i + bc_ri[q] * rs, j + bc_cj[q] * rs, e[q]);
			}
		}
	}
	orc_builder_finish(b, M);
}

int orc_bc_init(orc_baroclin *bc, orc_ops *o, const orc_bc_conf *c, const double *coriolis)
{
	memset(bc, 0, sizeof(*bc));
	bc->o = o; bc->c = *c;
	bc->lh = VEC(o->m->V);
	if (coriolis) memcpy(bc->lh, coriolis, sizeof(double) * (size_t)o->m->V);
	bc_assemble(bc, 0, &bc->A);
	bc_assemble(bc, 1, &bc->Ab);   /* Ab_ (examples/baroclin.cpp:69-106, 182-243) */
	return 0;
}

void orc_bc_free(orc_baroclin *bc)
{
	orc_csr_free(&bc->A); orc_csr_free(&bc->Ab); free(bc->lh);
	memset(bc, 0, sizeof(*bc));
}

/* generate_right_part with right_part_cb (examples/baroclin.cpp:245-339,
 * src/generators.h:236-276): rp = mass * [F; G] - boundary columns * bnd */
static void bc_rhs(orc_baroclin *bc, double *rp, const double *F, const double *G, const double *bnd,
                   int backward)
{
	const orc_mesh *m = bc->o->m;
	int rs = m->rs;
	memset(rp, 0, sizeof(double) * 4 * (size_t)rs);
	#pragma omp parallel for schedule(dynamic, 64)
	for (int i = 0; i < rs; ++i) {
		int p = m->inner[i], zone = orc_row_zone(m, p);
		rp[i] = 0.0;
		for (int k = m->adj_ptr[p]; k < m->adj_ptr[p + 1]; ++k) {
			int t = m->adj[k];
			orc_poly phi[3];
			orc_basis1(m, t, zone, phi);
			const orc_poly *pi = &phi[orc_tri_pos(m, t, p)];
			for (int i0 = 0; i0 < 3; ++i0) {
				int p2 = m->tri[3 * t + i0];
				if (m->bnd[p2]) {
					int j0 = m->p2io[p2];
					double a = orc_mass_cos(pi, &phi[i0], m, t, zone);
					double bb = orc_slaplace(&phi[i0], pi, m, t, zone);
					double e[9], acc[4] = { 0, 0, 0, 0 };
					bc_entries(&bc->c, backward, a, bb, e);
					for (int q = 0; q < 9; ++q)
						if (bnd) acc[bc_ri[q]] += -bnd[j0] * e[q];
					for (int q = 0; q < 4; ++q) rp[i + q * rs] += acc[q];
				} else {
					double a = orc_mass_cos(pi, &phi[i0], m, t, zone);
					int j = m->p2io[p2];
					rp[i] += F[j] * a;
					rp[i + rs] += G[j] * a;
				}
			}
		}
	}
}

void orc_bc_step(orc_baroclin *bc, double *u11, double *u21,
                 const double *u1, const double *u2, const double *bnd,
                 const double *f, const double *g)
{
	orc_ops *o = bc->o;
	const orc_mesh *m = o->m;
	int rs = m->rs, sz = m->V;
	double th = bc->c.theta, sigma = bc->c.sigma, mu = bc->c.mu, tau = bc->c.tau;
	double alpha = bc->c.alpha, mu1 = bc->c.mu1, sigma1 = bc->c.sigma1;
	double *w1 = VEC(sz), *w2 = VEC(sz), *dw1 = VEC(sz), *dw2 = VEC(sz), *FC = VEC(sz), *GC = VEC(sz);
	double *u1_n = VEC(sz), *u2_n = VEC(sz), *w1_n = VEC(sz), *w2_n = VEC(sz);
	double *u1_n1 = VEC(sz), *u2_n1 = VEC(sz), *tmp1 = VEC(sz), *tmp2 = VEC(sz);
	double *jac1 = VEC(rs), *jac2 = VEC(rs), *jac3 = VEC(rs), *F = VEC(rs), *G = VEC(rs);
	double *rp = VEC(4 * rs), *ans = VEC(4 * rs);

	orc_laplace_calc1(o, w1, u1, bnd);
	orc_laplace_calc1(o, w2, u2, bnd);
	orc_laplace_calc1(o, dw1, w1, bnd);
	orc_laplace_calc1(o, dw2, w2, bnd);
	for (int i = 0; i < sz; ++i) FC[i] = -0.5 * (1.0 - th) * sigma * w1[i] + 0.5 * (1.0 - th) * sigma * w2[i];
	for (int i = 0; i < sz; ++i) FC[i] = 1.0 * FC[i] + mu * (1.0 - th) * dw1[i];
	for (int i = 0; i < sz; ++i) FC[i] = 1.0 * FC[i] + 1.0 / tau * w1[i];
	for (int i = 0; i < sz; ++i) GC[i] = -0.5 * (1.0 - th) * sigma * w1[i] + -0.5 * (1.0 - th) * sigma * w2[i];
	for (int i = 0; i < sz; ++i) GC[i] = 1.0 * GC[i] + mu * (1.0 - th) * dw2[i];
	for (int i = 0; i < sz; ++i) GC[i] = 1.0 * GC[i] + 1.0 / tau * w2[i];
	for (int i = 0; i < sz; ++i) GC[i] = 1.0 * GC[i] + -alpha * alpha / tau * u2[i];
	for (int i = 0; i < sz; ++i) GC[i] = 1.0 * GC[i] + -alpha * alpha * mu1 * (1 - th) * w2[i];
	for (int i = 0; i < sz; ++i) GC[i] = 1.0 * GC[i] + alpha * alpha * sigma1 * (1 - th) * u2[i];
	memcpy(u1_n, u1, sizeof(double) * (size_t)sz);
	memcpy(u2_n, u2, sizeof(double) * (size_t)sz);
	memcpy(w1_n, w1, sizeof(double) * (size_t)sz);
	memcpy(w2_n, w2, sizeof(double) * (size_t)sz);
	for (int i = 0; i < sz; ++i) {
		if (f) FC[i] += f[i];
		if (g) GC[i] += alpha * alpha * g[i];
	}
	bc->last_iters = 0;
	for (int it = 0; it < bc->c.max_iter; ++it) {
		for (int i = 0; i < sz; ++i) tmp1[i] = (1.0 - th) * u1[i] + th * u1_n[i];
		for (int i = 0; i < sz; ++i) tmp2[i] = (1.0 - th) * w1[i] + th * w1_n[i];
		for (int i = 0; i < sz; ++i) tmp2[i] = tmp2[i] + bc->lh[i];
		orc_jacobian_calc2(o, jac1, tmp1, tmp2);
		for (int i = 0; i < sz; ++i) tmp1[i] = (1.0 - th) * u2[i] + th * u2_n[i];
		for (int i = 0; i < sz; ++i) tmp2[i] = (1.0 - th) * w2[i] + th * w2_n[i];
		orc_jacobian_calc2(o, jac2, tmp1, tmp2);
		for (int i = 0; i < rs; ++i) F[i] = -1.0 * jac1[i] + -1.0 * jac2[i];

		for (int i = 0; i < sz; ++i) tmp1[i] = (1.0 - th) * u1[i] + th * u1_n[i];
		for (int i = 0; i < sz; ++i) tmp2[i] = (1.0 - th) * w2[i] + th * w2_n[i];
		orc_jacobian_calc2(o, jac1, tmp1, tmp2);
		for (int i = 0; i < sz; ++i) tmp1[i] = (1.0 - th) * u2[i] + th * u2_n[i];
		for (int i = 0; i < sz; ++i) tmp2[i] = (1.0 - th) * w1[i] + th * w1_n[i];
		for (int i = 0; i < sz; ++i) tmp2[i] = tmp2[i] + bc->lh[i];
		orc_jacobian_calc2(o, jac2, tmp1, tmp2);
		for (int i = 0; i < sz; ++i) tmp1[i] = (1.0 - th) * u1[i] + th * u1_n[i];
		for (int i = 0; i < sz; ++i) tmp2[i] = (1.0 - th) * u2[i] + th * u2_n[i];
		orc_jacobian_calc2(o, jac3, tmp1, tmp2);
		for (int i = 0; i < rs; ++i) G[i] = -1.0 * jac1[i] + -1.0 * jac2[i];
		for (int i = 0; i < rs; ++i) G[i] = 1.0 * G[i] + alpha * alpha * jac3[i];
		for (int i = 0; i < rs; ++i) {
			int point = m->inner[i];
			F[i] += FC[point];
			G[i] += GC[point];
		}
		bc_rhs(bc, rp, F, G, bnd, 0);
		orc_csr_solve(&bc->A, ans, rp);
		orc_p2u(m, w1_n, ans, bnd);
		orc_p2u(m, w2_n, ans + rs, bnd);
		orc_p2u(m, u1_n1, ans + 2 * rs, bnd);
		orc_p2u(m, u2_n1, ans + 3 * rs, bnd);
		double nr1 = orc_dist(o, u1_n1, u1_n), nr2 = orc_dist(o, u2_n1, u2_n);
		double nr = nr1 > nr2 ? nr1 : nr2;
		double *s = u1_n1; u1_n1 = u1_n; u1_n = s;
		s = u2_n1; u2_n1 = u2_n; u2_n = s;
		bc->last_iters = it + 1;
		if (nr < bc->c.tol) break;
	}
	memcpy(u11, u1_n, sizeof(double) * (size_t)sz);
	memcpy(u21, u2_n, sizeof(double) * (size_t)sz);
	free(w1); free(w2); free(dw1); free(dw2); free(FC); free(GC);
	free(u1_n); free(u2_n); free(w1_n); free(w2_n); free(u1_n1); free(u2_n1);
	free(tmp1); free(tmp2); free(jac1); free(jac2); free(jac3); free(F); free(G); free(rp); free(ans);
}

/* Baroclin::calc_L (kind 0, examples/baroclin.cpp:620-802: one iteration,
 * forward matrix) and calc_L_1 (kind 1, :804-986: up to 10 iterations,
 * backward matrix Ab_), linearised around (z1, z2). */
static void bc_linear(orc_baroclin *bc, int kind, double *u11, double *u21,
                      const double *u1, const double *u2, const double *z1, const double *z2,
                      const double *bnd)
{
	orc_ops *o = bc->o;
	const orc_mesh *m = o->m;
	int rs = m->rs, sz = m->V;
	double th = bc->c.theta, sigma = bc->c.sigma, mu = bc->c.mu, tau = bc->c.tau;
	double alpha = bc->c.alpha, mu1 = bc->c.mu1, sigma1 = bc->c.sigma1;
	double *w1 = VEC(sz), *w2 = VEC(sz), *dw1 = VEC(sz), *dw2 = VEC(sz), *dz1 = VEC(sz), *dz2 = VEC(sz);
	double *FC = VEC(sz), *GC = VEC(sz);
	double *u1_n = VEC(sz), *u2_n = VEC(sz), *w1_n = VEC(sz), *w2_n = VEC(sz);
	double *u1_n1 = VEC(sz), *u2_n1 = VEC(sz), *tmp1 = VEC(sz), *tmp2 = VEC(sz);
	double *jac1 = VEC(rs), *jac2 = VEC(rs), *F = VEC(rs), *G = VEC(rs);
	double *rp = VEC(4 * rs), *ans = VEC(4 * rs);
	/* weights of the input and of the iterate in the Jacobian arguments */
	double wa = kind == 0 ? 1.0 - th : th, wb = kind == 0 ? th : 1.0 - th;
	double sgn = kind == 0 ? -1.0 : 1.0;

	orc_laplace_calc1(o, w1, u1, bnd);
	orc_laplace_calc1(o, w2, u2, bnd);
	orc_laplace_calc1(o, dw1, w1, bnd);
	orc_laplace_calc1(o, dw2, w2, bnd);
	orc_laplace_calc1(o, dz1, z1, bnd);
	orc_laplace_calc1(o, dz2, z2, bnd);
	if (kind == 0) {
		for (int i = 0; i < sz; ++i) FC[i] = -0.5 * (1.0 - th) * sigma * w1[i] + 0.5 * (1.0 - th) * sigma * w2[i];
		for (int i = 0; i < sz; ++i) FC[i] = 1.0 * FC[i] + mu * (1.0 - th) * dw1[i];
		for (int i = 0; i < sz; ++i) FC[i] = 1.0 * FC[i] + 1.0 / tau * w1[i];
		for (int i = 0; i < sz; ++i) GC[i] = -0.5 * (1.0 - th) * sigma * w1[i] + -0.5 * (1.0 - th) * sigma * w2[i];
		for (int i = 0; i < sz; ++i) GC[i] = 1.0 * GC[i] + mu * (1.0 - th) * dw2[i];
		for (int i = 0; i < sz; ++i) GC[i] = 1.0 * GC[i] + 1.0 / tau * w2[i];
		for (int i = 0; i < sz; ++i) GC[i] = 1.0 * GC[i] + -alpha * alpha / tau * u2[i];
		for (int i = 0; i < sz; ++i) GC[i] = 1.0 * GC[i] + -alpha * alpha * mu1 * (1 - th) * w2[i];
		for (int i = 0; i < sz; ++i) GC[i] = 1.0 * GC[i] + alpha * alpha * sigma1 * (1 - th) * u2[i];
	} else {
		for (int i = 0; i < sz; ++i) FC[i] = 0.5 * th * sigma * w1[i] + -0.5 * th * sigma * w2[i];
		for (int i = 0; i < sz; ++i) FC[i] = 1.0 * FC[i] + -mu * th * dw1[i];
		for (int i = 0; i < sz; ++i) FC[i] = 1.0 * FC[i] + 1.0 / tau * w1[i];
		for (int i = 0; i < sz; ++i) GC[i] = 0.5 * th * sigma * w1[i] + 0.5 * th * sigma * w2[i];
		for (int i = 0; i < sz; ++i) GC[i] = 1.0 * GC[i] + -mu * th * dw2[i];
		for (int i = 0; i < sz; ++i) GC[i] = 1.0 * GC[i] + 1.0 / tau * w2[i];
		for (int i = 0; i < sz; ++i) GC[i] = 1.0 * GC[i] + -alpha * alpha / tau * u2[i];
		for (int i = 0; i < sz; ++i) GC[i] = 1.0 * GC[i] + alpha * alpha * mu1 * th * w2[i];
		for (int i = 0; i < sz; ++i) GC[i] = 1.0 * GC[i] + -alpha * alpha * sigma1 * th * u2[i];
	}
	memcpy(u1_n, u1, sizeof(double) * (size_t)sz);
	memcpy(u2_n, u2, sizeof(double) * (size_t)sz);
	memcpy(w1_n, w1, sizeof(double) * (size_t)sz);
	memcpy(w2_n, w2, sizeof(double) * (size_t)sz);
	int iters = kind == 0 ? 1 : 10;
	for (int it = 0; it < iters; ++it) {
#define MIX(d, a, b) for (int i = 0; i < sz; ++i) d[i] = wa * a[i] + wb * b[i]
		/* F */
		MIX(tmp1, u1, u1_n);
		for (int i = 0; i < sz; ++i) tmp2[i] = dz1[i] + bc->lh[i];
		orc_jacobian_calc2(o, jac1, tmp1, tmp2);
		MIX(tmp1, w1, w1_n);
		orc_jacobian_calc2(o, jac2, z1, tmp1);
		if (kind == 0) for (int i = 0; i < rs; ++i) F[i] = -1.0 * jac1[i] + -1.0 * jac2[i];
		else for (int i = 0; i < rs; ++i) F[i] = jac1[i] + jac2[i];
		MIX(tmp1, w2, w2_n);
		orc_jacobian_calc2(o, jac1, z2, tmp1);
		if (kind == 0) for (int i = 0; i < rs; ++i) F[i] = 1.0 * F[i] + -1.0 * jac1[i];
		else for (int i = 0; i < rs; ++i) F[i] = F[i] + jac1[i];
		MIX(tmp1, u2, u2_n);
		orc_jacobian_calc2(o, jac1, tmp1, dz2);
		if (kind == 0) for (int i = 0; i < rs; ++i) F[i] = 1.0 * F[i] + -1.0 * jac1[i];
		else for (int i = 0; i < rs; ++i) F[i] = F[i] + jac1[i];
		/* G (the reference's J(z1, .) uses L(z1) here) */
		MIX(tmp1, w2, w2_n);
		orc_jacobian_calc2(o, jac1, dz1, tmp1);
		MIX(tmp1, u1, u1_n);
		orc_jacobian_calc2(o, jac2, dz2, tmp1);
		if (kind == 0) for (int i = 0; i < rs; ++i) G[i] = -1.0 * jac1[i] + -1.0 * jac2[i];
		else for (int i = 0; i < rs; ++i) G[i] = jac1[i] + jac2[i];
		MIX(tmp1, u2, u2_n);
		for (int i = 0; i < sz; ++i) tmp2[i] = dz1[i] + bc->lh[i];
		orc_jacobian_calc2(o, jac1, tmp1, tmp2);
		if (kind == 0) for (int i = 0; i < rs; ++i) G[i] = 1.0 * G[i] + -1.0 * jac1[i];
		else for (int i = 0; i < rs; ++i) G[i] = G[i] + jac1[i];
		MIX(tmp1, w1, w1_n);
		orc_jacobian_calc2(o, jac1, z2, tmp1);
		if (kind == 0) for (int i = 0; i < rs; ++i) G[i] = 1.0 * G[i] + -1.0 * jac1[i];
		else for (int i = 0; i < rs; ++i) G[i] = G[i] + jac1[i];
		MIX(tmp1, u2, u2_n);
		orc_jacobian_calc2(o, jac1, z1, tmp1);
		for (int i = 0; i < rs; ++i) G[i] = 1.0 * G[i] + -sgn * alpha * alpha * jac1[i];
		MIX(tmp1, u1, u1_n);
		orc_jacobian_calc2(o, jac1, tmp1, z2);
		for (int i = 0; i < rs; ++i) G[i] = 1.0 * G[i] + -sgn * alpha * alpha * jac1[i];
#undef MIX
		for (int i = 0; i < rs; ++i) {
			int point = m->inner[i];
			F[i] += FC[point];
			G[i] += GC[point];
		}
		bc_rhs(bc, rp, F, G, bnd, kind);
		orc_csr_solve(kind == 0 ? &bc->A : &bc->Ab, ans, rp);
		orc_p2u(m, w1_n, ans, bnd);
		orc_p2u(m, w2_n, ans + rs, bnd);
		orc_p2u(m, u1_n1, ans + 2 * rs, bnd);
		orc_p2u(m, u2_n1, ans + 3 * rs, bnd);
		double nr1 = orc_dist(o, u1_n1, u1_n), nr2 = orc_dist(o, u2_n1, u2_n);
		double nr = nr1 > nr2 ? nr1 : nr2;
		double *s = u1_n1; u1_n1 = u1_n; u1_n = s;
		s = u2_n1; u2_n1 = u2_n; u2_n = s;
		bc->last_iters = it + 1;
		if (nr < 1e-8) break;
	}
	memcpy(u11, u1_n, sizeof(double) * (size_t)sz);
	memcpy(u21, u2_n, sizeof(double) * (size_t)sz);
	free(w1); free(w2); free(dw1); free(dw2); free(dz1); free(dz2); free(FC); free(GC);
	free(u1_n); free(u2_n); free(w1_n); free(w2_n); free(u1_n1); free(u2_n1); free(tmp1); free(tmp2);
	free(jac1); free(jac2); free(F); free(G); free(rp); free(ans);
}

void orc_bc_calc_L(orc_baroclin *bc, double *u11, double *u21, const double *u1, const double *u2,
                   const double *z1, const double *z2, const double *bnd)
{
	bc_linear(bc, 0, u11, u21, u1, u2, z1, z2, bnd);
}

void orc_bc_calc_L1(orc_baroclin *bc, double *u11, double *u21, const double *u1, const double *u2,
                    const double *z1, const double *z2, const double *bnd)
{
	bc_linear(bc, 1, u11, u21, u1, u2, z1, z2, bnd);
}

/* ------------------------------------------------- known-answer helpers --- */
/* Integral over the triangle (xs, ys) of the polynomial with coefficients
 * koef (x degree xd, y degree yd); kind 0 plain, 1 cos x, 2 sin x, 3 1/cos x. */
double orc_integrate_poly(int kind, const double xs[3], const double ys[3],
                          int xd, int yd, const double *koef)
{
	orc_poly p;
	memset(&p, 0, sizeof(p));
	p.xd = (short)xd; p.yd = (short)yd;
	memcpy(p.k, koef, sizeof(double) * (size_t)((xd + 1) * (yd + 1)));
	orc_trap_fn fn = kind == 0 ? orc_trapezoid_integral : kind == 1 ? orc_trapezoid_cos
	               : kind == 2 ? orc_trapezoid_sin : orc_trapezoid_1_cos;
	return orc_integrate1(&p, xs, ys, fn);
}
