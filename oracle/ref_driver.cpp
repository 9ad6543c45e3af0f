/*
 * ref_driver.cpp -- runs the reference's own C++ sources (compiled into
 * oracle/_ref by oracle/Makefile) and writes their results as .npy files, so
 * that tests/golden/make_golden.py can pin the oracle restatement and the
 * product's host-side mesh/assembly against the reference itself.
 *
 * TEST INFRASTRUCTURE ONLY.  Never shipped, never run on the product path.
 *
 * Usage: ref_driver MESH.txt OUTDIR [key=value ...]
 *   reads optional inputs OUTDIR/in_u.npy, in_v.npy, in_bnd.npy (f8)
 *   keys: bv_steps, bv_iters, bv_lin, bc_steps, bc_iters, coriolis (0 zero, 1 sin(phi))
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>
#include <map>
#include <set>
#include <list>
#include <functional>
#include <algorithm>
#include <memory>
#include <stdexcept>
#include <initializer_list>

int orc_ref_bv_max_iter = 1000;
int orc_ref_bc_max_iter = 20;

/* BarVortex / Baroclin keep their matrices private; the driver reads them. */
#define private public
#include "barvortex.h"
/* examples/baroclin.h reuses the BARVORTEX_H include guard */
#undef BARVORTEX_H
#include "baroclin.h"
#undef private

using namespace phelm;

/* ------------------------------------------------------------ npy I/O --- */
static void npy_write(const std::string &path, const char *descr,
                      const std::vector<size_t> &shape, const void *data, size_t elsize)
{
	std::string sh = "(";
	size_t count = 1;
	for (size_t i = 0; i < shape.size(); ++i) {
		sh += std::to_string(shape[i]);
		sh += (shape.size() == 1) ? "," : (i + 1 < shape.size() ? ", " : "");
		count *= shape[i];
	}
	sh += ")";
	std::string hdr = std::string("{'descr': '") + descr + "', 'fortran_order': False, 'shape': " + sh + ", }";
	size_t total = 10 + hdr.size() + 1;
	size_t pad = (64 - total % 64) % 64;
	hdr.append(pad, ' ');
	hdr += '\n';
	FILE *f = fopen(path.c_str(), "wb");
	if (!f) { perror(path.c_str()); exit(2); }
	unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
	fwrite(magic, 1, 8, f);
	unsigned short hl = (unsigned short)hdr.size();
	fwrite(&hl, 2, 1, f);
	fwrite(hdr.data(), 1, hdr.size(), f);
	if (count) fwrite(data, elsize, count, f);
	fclose(f);
}

static bool npy_read_f8(const std::string &path, std::vector<double> &out)
{
	FILE *f = fopen(path.c_str(), "rb");
	if (!f) return false;
	unsigned char magic[8];
	if (fread(magic, 1, 8, f) != 8) { fclose(f); return false; }
	unsigned short hl = 0;
	if (fread(&hl, 2, 1, f) != 1) { fclose(f); return false; }
	std::string hdr(hl, ' ');
	if (fread(&hdr[0], 1, hl, f) != hl) { fclose(f); return false; }
	if (hdr.find("<f8") == std::string::npos) { fclose(f); return false; }
	long pos = ftell(f);
	fseek(f, 0, SEEK_END);
	long end = ftell(f);
	fseek(f, pos, SEEK_SET);
	out.resize((size_t)(end - pos) / 8);
	size_t got = out.empty() ? 0 : fread(&out[0], 8, out.size(), f);
	fclose(f);
	return got == out.size();
}

static void wf8(const std::string &dir, const char *name, const std::vector<double> &v)
{
	npy_write(dir + "/" + name + ".npy", "<f8", {v.size()}, v.data(), 8);
}

static void wi4(const std::string &dir, const char *name, const std::vector<int> &v)
{
	npy_write(dir + "/" + name + ".npy", "<i4", {v.size()}, v.data(), 4);
}

template <typename M>
static void dump_csr(const std::string &dir, const std::string &name, const M &A)
{
	std::vector<int> ptr(1, 0), col;
	std::vector<double> val;
	const auto &rows = A.rows();
	for (size_t i = 0; i < rows.size(); ++i) {
		for (auto it = rows[i].begin(); it != rows[i].end(); ++it) {
			col.push_back(it->first);
			val.push_back(it->second);
		}
		ptr.push_back((int)col.size());
	}
	wi4(dir, (name + "_ptr").c_str(), ptr);
	wi4(dir, (name + "_col").c_str(), col);
	wf8(dir, (name + "_val").c_str(), val);
}

static double cor_zero(double, double) { return 0.0; }
static double cor_sin(double phi, double) { return sin(phi); }
/* a smooth, time-dependent forcing for the boundary + forcing run (any
 * function of the reference's rp_t shape would do) */
static double rp_test(double phi, double lambda, double t, double mu, double sigma)
{
	(void)mu; (void)sigma;
	return 0.05 * cos(phi) * sin(2.0 * lambda + 40.0 * t) + 0.02 * sin(phi);
}

/* The analytic fields of tests/manufactured.py (same formulas, see there for
 * their derivation), for the reference's own accuracy checks run on the
 * same inputs as the GPU tests. */
static double mf_lap_u(double phi, double lam)
{
	double x = cos(phi) * cos(lam), z = sin(phi);
	return 0.5 * (x - 1.0) * (x - 1.0) + (x - z) * (x - z) + 2.0 * (z - 3.0) * (z - 3.0);
}
static double mf_lap_f(double phi, double lam)
{
	double x = cos(phi) * cos(lam), z = sin(phi);
	return 9.0 - 9.0 * x * x + 12.0 * x * z - 18.0 * z * z + 2.0 * x + 24.0 * z;
}
static double mf_jac_f1(double phi, double lam) { return sin(phi) * sin(lam); }
static double mf_jac_f2(double phi, double lam) { return cos(phi) * cos(lam); }
static double mf_jac_an(double phi, double lam)
{
	double c = cos(phi), s = sin(phi);
	return (-s * s * cos(lam) * cos(lam) + c * c * sin(lam) * sin(lam)) / c;
}
static double mf_bv_psi(double phi, double lam, double t)
{
	double c = cos(phi);
	return phi * c * c * c * c * sin(lam + t);
}
static double mf_bv_forcing(double phi, double lam, double t, double mu, double sigma)
{
	double c = cos(phi), s = sin(phi), S = sin(lam + t), C = cos(lam + t);
	double g = phi * c * c * c * c, g1 = c * c * c * c - 4.0 * phi * c * c * c * s;
	double w = -9.0 * c * c * c * s + 15.0 * phi * c * c - 20.0 * phi * c * c * c * c;
	double w1 = 27.0 * c * c * s * s - 29.0 * c * c * c * c + 15.0 * c * c - 30.0 * phi * c * s
	            + 80.0 * phi * c * c * c * s;
	double w2 = -54.0 * c * s * s * s + 250.0 * c * c * c * s - 60.0 * c * s - 30.0 * phi * c * c
	            + 30.0 * phi * s * s - 240.0 * phi * c * c * s * s + 80.0 * phi * c * c * c * c;
	double jac = C * S * (g * w1 - g1 * w) / c;
	double lap_w = w2 - tan(phi) * w1 - w / (c * c);
	return w * C + jac + sigma * w * S - mu * lap_w * S;
}

/* examples/test_slaplace.cpp:100-199, examples/test_barvortex.cpp:57-105 and
 * 488-559 on the fields above; writes out_pin_* */
static void run_pins(const Mesh &m, const std::string &dir, bool with_bv)
{
	int sz = (int)m.ps.size(), os = (int)m.outer.size();
	std::vector<double> U(sz), LU(sz), LU1(sz), Ans(sz), B1(std::max(os, 1)), B2(std::max(os, 1));
	proj(&U[0], m, mf_lap_u);
	proj(&LU[0], m, mf_lap_f);
	proj_bnd(&B1[0], m, mf_lap_f);
	proj_bnd(&B2[0], m, mf_lap_u);
	SphereLaplace<double> l(m);
	SphereNorm<double> nr(m);
	std::vector<double> e;
	l.solve(&Ans[0], &LU[0], &B2[0]);
	e.push_back(nr.dist(&Ans[0], &U[0]));            // L1: invert
	l.calc1(&LU1[0], &U[0], &B1[0]);
	e.push_back(nr.dist(&LU[0], &LU1[0]));           // L2: laplace
	l.solve(&LU[0], &LU1[0], &B2[0]);
	e.push_back(nr.dist(&U[0], &LU[0]));             // L3: round trip
	wf8(dir, "out_pin_slaplace", e);

	SphereJacobian j(m);
	std::vector<double> F1(sz), F2(sz), a1(sz), r1(sz), bj(std::max(os, 1));
	proj(&F1[0], m, mf_jac_f1);
	proj(&F2[0], m, mf_jac_f2);
	proj(&r1[0], m, mf_jac_an);
	proj_bnd(&bj[0], m, mf_jac_an);
	j.calc1(&a1[0], &F1[0], &F2[0], &bj[0]);
	std::vector<double> ej(1, phelm::dist(&a1[0], &r1[0], m, sphere_scalar_cb, (void *)0));
	wf8(dir, "out_pin_jacobian", ej);

	if (!with_bv) return;
	BarVortexConf conf;
	memset(&conf, 0, sizeof(conf));
	conf.tau = 0.001; conf.sigma = 1.6e-2; conf.mu = 8e-5; conf.k1 = 1.0; conf.k2 = 1.0; conf.theta = 0.5;
	conf.rp = mf_bv_forcing;
	conf.coriolis = cor_zero;
	orc_ref_bv_max_iter = 1000;
	SBarVortex bv(m, conf);
	std::vector<double> u(sz), bu(std::max(os, 1), 0.0), bw(std::max(os, 1), 0.0), an(sz);
	for (int i = 0; i < sz; ++i) u[i] = mf_bv_psi(m.ps[i].x(), m.ps[i].y(), 0.0);
	double t = 0.0, T = 0.01;
	while (t < T) {
		bv.calc(&u[0], &u[0], &bu[0], &bw[0], t);
		t += conf.tau;
	}
	for (int i = 0; i < sz; ++i) an[i] = mf_bv_psi(m.ps[i].x(), m.ps[i].y(), t);
	std::vector<double> eb(1, bv.dist(&u[0], &an[0]));
	wf8(dir, "out_pin_barvortex", eb);
}

int main(int argc, char **argv)
{
	if (argc < 3) { fprintf(stderr, "usage: %s MESH OUTDIR [k=v ...]\n", argv[0]); return 1; }
	std::string dir = argv[2];
	std::map<std::string, double> kv;
	for (int i = 3; i < argc; ++i) {
		const char *eq = strchr(argv[i], '=');
		if (eq) kv[std::string(argv[i], (size_t)(eq - argv[i]))] = atof(eq + 1);
	}
	auto get = [&](const char *k, double d) { return kv.count(k) ? kv[k] : d; };

	FILE *f = fopen(argv[1], "rb");
	if (!f) { perror(argv[1]); return 1; }
	Mesh m;
	if (!m.load(f)) { fprintf(stderr, "bad mesh\n"); return 1; }
	fclose(f);
	int sz = m.size, rs = m.inner_size, os = m.outer_size;
	(void)sz;
	sz = (int)m.ps.size(); rs = (int)m.inner.size(); os = (int)m.outer.size();

	/* mesh arrays */
	{
		std::vector<double> xyz, uv;
		for (int i = 0; i < sz; ++i) {
			xyz.push_back(m.ps[i].pr.x); xyz.push_back(m.ps[i].pr.y); xyz.push_back(m.ps[i].pr.z);
			for (int z = 0; z < 4; ++z) {
				uv.push_back(z < (int)m.ps[i].p.size() ? m.ps[i].p[z].x : NAN);
				uv.push_back(z < (int)m.ps[i].p.size() ? m.ps[i].p[z].y : NAN);
			}
		}
		wf8(dir, "mesh_xyz", xyz);
		wf8(dir, "mesh_uv", uv);
		std::vector<int> tri, tz, bnd, aptr(1, 0), adj;
		for (size_t t = 0; t < m.tr.size(); ++t) {
			for (int k = 0; k < 3; ++k) tri.push_back(m.tr[t].p[k]);
			tz.push_back(m.tr[t].z);
		}
		for (int i = 0; i < sz; ++i) {
			bnd.push_back(m.is_boundary(i) ? 1 : 0);
			for (size_t k = 0; k < m.adj[i].size(); ++k) adj.push_back(m.adj[i][k]);
			aptr.push_back((int)adj.size());
		}
		wi4(dir, "mesh_tri", tri); wi4(dir, "mesh_tz", tz); wi4(dir, "mesh_bnd", bnd);
		wi4(dir, "mesh_inner", m.inner); wi4(dir, "mesh_outer", m.outer); wi4(dir, "mesh_p2io", m.p2io);
		wi4(dir, "mesh_adj_ptr", aptr); wi4(dir, "mesh_adj", adj);
	}

	SphereLaplace<double> l(m);
	SphereJacobian j(m);
	SphereNorm<double> nrm(m);
	dump_csr(dir, "idt", l.idt_); dump_csr(dir, "lapl", l.laplace_);
	dump_csr(dir, "bnd1", l.bnd1_); dump_csr(dir, "bnd2", l.bnd2_); dump_csr(dir, "bnd3", l.bnd3_);
	dump_csr(dir, "jidt", j.idt_);
	dump_csr(dir, "d1", j.diff1_); dump_csr(dir, "d2", j.diff2_);
	dump_csr(dir, "d1c", j.diff1_cos_); dump_csr(dir, "d2c", j.diff2_cos_);
	dump_csr(dir, "d1b", j.diff1_rp_); dump_csr(dir, "d2b", j.diff2_rp_);
	dump_csr(dir, "d1cb", j.diff1_cos_rp_); dump_csr(dir, "d2cb", j.diff2_cos_rp_);
	dump_csr(dir, "norm", nrm.NORM_);

	std::vector<double> u, v, bnd;
	bool have_u = npy_read_f8(dir + "/in_u.npy", u) && (int)u.size() == sz;
	bool have_v = npy_read_f8(dir + "/in_v.npy", v) && (int)v.size() == sz;
	if (!npy_read_f8(dir + "/in_bnd.npy", bnd) || (int)bnd.size() != os) bnd.assign(std::max(os, 1), 0.0);

	if (have_u) {
		std::vector<double> a(sz), b(rs);
		l.calc1(&a[0], &u[0], &bnd[0]); wf8(dir, "out_lap_calc1", a);
		l.calc2(&b[0], &u[0]); wf8(dir, "out_lap_calc2", b);
		l.solve(&a[0], &u[0], &bnd[0]); wf8(dir, "out_lap_solve", a);
		std::vector<double> ns;
		ns.push_back(nrm.norm(&u[0]));
		if (have_v) {
			ns.push_back(nrm.dist(&u[0], &v[0]));
			ns.push_back(nrm.scalar(&u[0], &v[0]));
			j.calc2(&b[0], &u[0], &v[0]); wf8(dir, "out_jac_calc2", b);
			j.calc1(&a[0], &u[0], &v[0], &bnd[0]); wf8(dir, "out_jac_calc1", a);
			j.calc1t(&a[0], &u[0], &v[0], &bnd[0]); wf8(dir, "out_jac_calc1t", a);
			j.calc2_diff_x(&b[0], &u[0]); wf8(dir, "out_jac_diff_x", b);
			j.calc2_diff_cos_y(&b[0], &u[0]); wf8(dir, "out_jac_diff_cos_y", b);
		}
		wf8(dir, "out_norms", ns);
		// the text output routines (src/phelm.cpp:160-321), default coordinates
		print_function((dir + "/print_function.txt").c_str(), &u[0], m);
		print_inner_function((dir + "/print_inner_function.txt").c_str(), &u[0], m);
	}

	BarVortexConf conf;
	memset(&conf, 0, sizeof(conf));
	conf.tau = get("tau", 1e-3);
	conf.sigma = get("sigma", 1.6e-2);
	conf.mu = get("mu", 8e-5);
	conf.k1 = get("k1", 1.0);
	conf.k2 = get("k2", 1.0);
	conf.theta = get("theta", 0.5);
	conf.rp = 0;
	conf.coriolis = get("coriolis", 1) ? cor_sin : cor_zero;
	int bv_steps = (int)get("bv_steps", 0);
	if (bv_steps > 0 && have_u) {
		orc_ref_bv_max_iter = (int)get("bv_iters", 3);
		SBarVortex bv(m, conf);
		dump_csr(dir, "bvA", bv.A_);
		dump_csr(dir, "bvAbnd", bv.bnd_);
		std::vector<double> st(u), bu(std::max(os, 1), 0.0), bw(std::max(os, 1), 0.0);
		double t = 0.0;
		for (int s = 0; s < bv_steps; ++s) {
			bv.calc(&st[0], &st[0], &bu[0], &bw[0], t);
			t += conf.tau;
			if (s == 0) wf8(dir, "out_bv_step1", st);
		}
		wf8(dir, "out_bv_final", st);
		if (get("bv_bf", 0)) {
			// two steps with non-zero pole values (bnd_u = in_bnd, bnd_w = -2 in_bnd)
			// and the time-dependent forcing rp_test at t = 0 and t = tau; the
			// forcing values at the points are written for the callers
			BarVortexConf cf = conf;
			cf.rp = rp_test;
			SBarVortex bvf(m, cf);
			std::vector<double> sf(u), fu(std::max(os, 1)), fw(std::max(os, 1)), f0(sz), f1(sz);
			for (int k = 0; k < os; ++k) { fu[k] = bnd[k]; fw[k] = -2.0 * bnd[k]; }
			for (int i = 0; i < sz; ++i) {
				f0[i] = rp_test(m.ps[i].x(), m.ps[i].y(), 0.0, cf.mu, cf.sigma);
				f1[i] = rp_test(m.ps[i].x(), m.ps[i].y(), cf.tau, cf.mu, cf.sigma);
			}
			wf8(dir, "out_bv_bf_forcing0", f0);
			wf8(dir, "out_bv_bf_forcing1", f1);
			wf8(dir, "out_bv_bf_bnd_u", fu);
			wf8(dir, "out_bv_bf_bnd_w", fw);
			bvf.calc(&sf[0], &sf[0], &fu[0], &fw[0], 0.0);
			wf8(dir, "out_bv_bf_step1", sf);
			bvf.calc(&sf[0], &sf[0], &fu[0], &fw[0], cf.tau);
			wf8(dir, "out_bv_bf_step2", sf);
		}
		if (have_v && get("bv_lin", 0)) {
			// linearised step around z = u, its inverse and its adjoint, applied to v
			std::vector<double> r(sz, 0.0);
			bv.calc_L(&r[0], &v[0], &u[0], &bu[0], &bw[0], 0.0); wf8(dir, "out_bv_L", r);
			std::fill(r.begin(), r.end(), 0.0);
			bv.calc_L_1(&r[0], &v[0], &u[0], &bu[0], &bw[0], 0.0); wf8(dir, "out_bv_L1", r);
			std::fill(r.begin(), r.end(), 0.0);
			bv.calc_LT(&r[0], &v[0], &u[0], &bu[0], &bw[0], 0.0); wf8(dir, "out_bv_LT", r);
		}
	}

	if (get("pins", 0)) run_pins(m, dir, get("pins", 0) > 1);

	int bc_steps = (int)get("bc_steps", 0);
	if (bc_steps > 0 && have_u && have_v) {
		orc_ref_bc_max_iter = (int)get("bc_iters", 3);
		Baroclin bc(m, 0, 0, conf.coriolis, get("bc_tau", 1e-3), get("bc_sigma", 0.05),
		            get("bc_mu", 6.77e-5), get("bc_sigma1", 0.05), get("bc_mu1", 6.77e-5),
		            get("bc_alpha", sqrt(0.1)));
		dump_csr(dir, "bcA", bc.A_);
		std::vector<double> u1(u), u2(v), z(std::max(os, 1), 0.0);
		for (int s = 0; s < bc_steps; ++s) {
			bc.calc(&u1[0], &u2[0], &u1[0], &u2[0], &z[0], 0.0);
			if (s == 0) { wf8(dir, "out_bc_step1_u1", u1); wf8(dir, "out_bc_step1_u2", u2); }
		}
		wf8(dir, "out_bc_final_u1", u1);
		wf8(dir, "out_bc_final_u2", u2);
		if (get("bc_lin", 0)) {
			// linearised step around (z1, z2) = (u, v) and its inverse, applied to (v, u)
			std::vector<double> a1(sz), a2(sz);
			bc.calc_L(&a1[0], &a2[0], &v[0], &u[0], &u[0], &v[0], &z[0], 0.0);
			wf8(dir, "out_bc_L_u1", a1); wf8(dir, "out_bc_L_u2", a2);
			bc.calc_L_1(&a1[0], &a2[0], &v[0], &u[0], &u[0], &v[0], &z[0], 0.0);
			wf8(dir, "out_bc_L1_u1", a1); wf8(dir, "out_bc_L1_u2", a2);
		}
	}
	return 0;
}
