/*
 * phelm_gb300.hpp -- C++ facade over the C ABI (phelm_gb300.h) that keeps the
 * class shapes of the reference's sphere path (resetius/mke "Phelm"), so that
 * code written against
 *
 *   phelm::Mesh                     (src/mesh.h:354-427)
 *   phelm::SphereLaplace<double>    (src/slaplace.h:60-108)
 *   phelm::SphereJacobian           (src/sjacobian.h:65-149)
 *   phelm::SphereNorm<double>       (src/norm.h:58-120)
 *   SBarVortex = BarVortex<...>     (examples/barvortex.h:109-238)
 *   Baroclin                        (examples/baroclin.h:147-175)
 *
 * compiles against phelm_gb300:: with the same member functions and argument
 * meanings.  Header-only; link libphelm_gb300.so.
 *
 * What differs from the reference, and why:
 *   - The operator constructors take an Operators object (one device upload
 *     of every operator of the mesh, shared by the classes) instead of the
 *     Mesh itself; Operators(mesh) replaces the three constructors.
 *   - Function-pointer callbacks (BarVortexConf::rp / coriolis, Baroclin's
 *     f / g / coriolis) become vectors of their values at the mesh points,
 *     evaluated by the caller in the zone-0 chart as the reference's proj
 *     does (src/phelm.cpp:338-350): set_forcing() for the barotropic forcing.
 *   - Errors: every C ABI status other than PHG_OK throws phelm_gb300::Error
 *     (the reference aborts or lets NaN propagate).
 *   - Pointers may be host memory (the call copies and blocks) or device
 *     memory (the call is ordered on the handle's stream and does not block).
 */
#ifndef PHELM_GB300_HPP
#define PHELM_GB300_HPP

#include <algorithm>
#include <stdexcept>
#include <string>
#include <vector>

#include "phelm_gb300.h"

namespace phelm_gb300 {

struct Error : std::runtime_error {
    int code;
    Error(int c, const char *msg) : std::runtime_error(msg ? msg : "phelm_gb300 error"), code(c) {}
};

inline void ck(int rc) {
    if (rc != PHG_OK) throw Error(rc, phg_last_error());
}

/* phelm::Mesh: an icosahedral sphere of `level` subdivisions (the file
 * mke_mesh_sphere --type full --coord local --iter level would write), or a
 * mesh file in the reference's text format (Mesh::load, src/mesh.cpp:323-519). */
class Mesh {
public:
    explicit Mesh(int level) { ck(phg_mesh_generate(level, &h_)); info(); }
    explicit Mesh(const char *path) { ck(phg_mesh_load_file(path, &h_)); info(); }
    ~Mesh() { phg_mesh_destroy(h_); }
    Mesh(const Mesh &) = delete;
    Mesh &operator=(const Mesh &) = delete;

    int size = 0;        // Mesh::size (points)
    int inner_size = 0;  // Mesh::inner_size
    int outer_size = 0;  // Mesh::outer_size
    int ntri = 0;        // Mesh::tr.size()

    /* Mesh::inner / outer / p2io (src/mesh.h:375-379) */
    std::vector<int> inner() const { std::vector<int> v(inner_size); ck(phg_mesh_maps(h_, v.data(), nullptr, nullptr)); return v; }
    std::vector<int> outer() const { std::vector<int> v(outer_size); ck(phg_mesh_maps(h_, nullptr, v.data(), nullptr)); return v; }
    std::vector<int> p2io() const { std::vector<int> v(size); ck(phg_mesh_maps(h_, nullptr, nullptr, v.data())); return v; }

    phg_mesh handle() const { return h_; }

private:
    phg_mesh h_ = nullptr;
    void info() { ck(phg_mesh_info(h_, &size, &ntri, &inner_size, &outer_size)); }
};

/* The device-resident operators of one mesh: replaces the constructors
 * SphereLaplace(m), SphereJacobian(m), SphereNorm(m).  precision: PHG_FP64
 * (the reference's double path) or PHG_MIXED (FP32 inner solves inside FP64
 * iterative refinement). */
class Operators {
public:
    explicit Operators(const Mesh &m, int precision = PHG_FP64) : mesh_(m) { ck(phg_ops_create(m.handle(), precision, &h_)); }
    ~Operators() { phg_ops_destroy(h_); }
    Operators(const Operators &) = delete;
    Operators &operator=(const Operators &) = delete;

    /* GMRES(restart) relative-residual tolerance and iteration cap */
    void set_solver(int restart, double tol, int max_iter) { ck(phg_ops_set_solver(h_, restart, tol, max_iter)); }
    /* phelm::Solver<double>::mult_vector of one of the handle's inner x inner
     * operators ("idt" "lapl" "jidt" "d1" "d2" "d1c" "d2c") */
    void mult_vector(const char *name, double *y, const double *x) { ck(phg_ops_mult(h_, name, y, x, 1, nullptr)); }
    /* wait for (and check) the solves of calls made with device pointers */
    void check() { ck(phg_ops_check(h_, nullptr)); }

    const Mesh &mesh() const { return mesh_; }
    phg_ops handle() const { return h_; }

private:
    const Mesh &mesh_;
    phg_ops h_ = nullptr;
};

/* SphereLaplace<T> (src/slaplace.h:60-108); T = double (the precision of the
 * device path is the Operators' precision). */
template <typename T> class SphereLaplace;
template <> class SphereLaplace<double> {
public:
    explicit SphereLaplace(Operators &o) : o_(o) {}
    /* Ans[size] = Laplacian of F[size], bnd[outer_size] on the boundary (NULL = 0) */
    void calc1(double *Ans, const double *F, const double *bnd) { ck(phg_laplace_calc1(o_.handle(), Ans, F, bnd, nullptr)); }
    /* Ans[inner_size] = Laplacian of F[size] on the inner points */
    void calc2(double *Ans, const double *F) { ck(phg_laplace_calc2(o_.handle(), Ans, F, nullptr)); }
    /* Ans[size]: Laplacian(Ans) = F on the inner points, Ans = bnd on the boundary */
    void solve(double *Ans, const double *F, const double *bnd) { ck(phg_laplace_solve(o_.handle(), Ans, F, bnd, nullptr)); }

private:
    Operators &o_;
};

/* SphereJacobian (src/sjacobian.h:65-149) */
class SphereJacobian {
public:
    explicit SphereJacobian(Operators &o) : o_(o) {}
    void calc1(double *Ans, const double *u, const double *v, const double *bnd) {
        ck(phg_jacobian_calc1(o_.handle(), Ans, u, v, bnd, nullptr));
    }
    void calc1t(double *Ans, const double *u, const double *v, const double *bnd) {
        ck(phg_jacobian_calc1t(o_.handle(), Ans, u, v, bnd, nullptr));
    }
    void calc2(double *Ans, const double *u, const double *v) { ck(phg_jacobian_calc2(o_.handle(), Ans, u, v, nullptr)); }
    void calc2t(double *Ans, const double *u, const double *v) { ck(phg_jacobian_calc2t(o_.handle(), Ans, u, v, nullptr)); }
    void calc2_diff_x(double *Ans, const double *v) { ck(phg_jacobian_calc2_diff_x(o_.handle(), Ans, v, nullptr)); }
    void calc2_diff_cos_y(double *Ans, const double *v) { ck(phg_jacobian_calc2_diff_cos_y(o_.handle(), Ans, v, nullptr)); }

private:
    Operators &o_;
};

/* SphereNorm<T> (src/norm.h:58-120); T = double */
template <typename T> class SphereNorm;
template <> class SphereNorm<double> {
public:
    explicit SphereNorm(Operators &o) : o_(o) {}
    double norm(const double *u) { double r; ck(phg_norm(o_.handle(), u, &r, nullptr)); return r; }
    double dist(const double *u, const double *v) { double r; ck(phg_dist(o_.handle(), u, v, &r, nullptr)); return r; }
    double scalar(const double *u, const double *v) { double r; ck(phg_scalar(o_.handle(), u, v, &r, nullptr)); return r; }

private:
    Operators &o_;
};

/* BarVortexConf (examples/barvortex.h:62-96) without the callbacks: theta
 * is set explicitly (the reference leaves it uninitialised); picard_iters is
 * the most Picard iterations per step, with the reference's 1e-14 stop test. */
inline phg_bv_conf barvortex_conf(double tau, double sigma, double mu, double k1 = 1.0, double k2 = 1.0,
                                  double theta = 0.5, int picard_iters = 1000) {
    phg_bv_conf c;
    c.tau = tau; c.sigma = sigma; c.mu = mu; c.k1 = k1; c.k2 = k2; c.theta = theta;
    c.picard_iters = picard_iters;
    return c;
}

/* SBarVortex (examples/barvortex.h:109-238).  coriolis: l + h at the points
 * (the reference evaluates conf.coriolis). */
class BarVortex {
public:
    BarVortex(Operators &o, const phg_bv_conf &conf, const double *coriolis) : size_(o.mesh().size) {
        ck(phg_barvortex_create(o.handle(), &conf, coriolis, &h_));
    }
    ~BarVortex() { phg_barvortex_destroy(h_); }
    BarVortex(const BarVortex &) = delete;
    BarVortex &operator=(const BarVortex &) = delete;

    /* the forcing f at the points, used by every later calc / S_step until
     * changed (NULL = none); the reference evaluates conf.rp at time t */
    void set_forcing(const double *f) {
        if (f) forcing_.assign(f, f + size_);
        else forcing_.clear();
    }

    /* BarVortex::calc (examples/barvortex_impl.h:171-310); Ans may equal F */
    void calc(double *Ans, const double *F, const double *bnd_u, const double *bnd_w, double t = 0.0) {
        (void)t;   // time enters only through the forcing values
        ck(phg_barvortex_calc(h_, Ans, F, bnd_u, bnd_w, forcing_.empty() ? nullptr : forcing_.data(), nullptr));
    }
    /* BarVortex::calc_L / calc_L_1 / calc_LT (examples/barvortex_impl.h:326-536);
     * calc_L_1 adds into Ans as the reference does */
    void calc_L(double *Ans, const double *F, const double *z, const double *bnd_u, const double *bnd_w, double = 0.0) {
        ck(phg_barvortex_calc_L(h_, Ans, F, z, bnd_u, bnd_w, nullptr));
    }
    void calc_L_1(double *Ans, const double *F, const double *z, const double *bnd_u, const double *bnd_w,
                  double = 0.0) {
        ck(phg_barvortex_calc_L_1(h_, Ans, F, z, bnd_u, bnd_w, nullptr));
    }
    void calc_LT(double *Ans, const double *F, const double *z, const double *bnd_u, const double *bnd_w,
                 double = 0.0) {
        ck(phg_barvortex_calc_LT(h_, Ans, F, z, bnd_u, bnd_w, nullptr));
    }

    /* the helpers of examples/barvortex_impl.h:539-570: zero boundary, t = 0
     * (host arrays) */
    void S_step(double *Ans, const double *F) { calc(Ans, F, nullptr, nullptr, 0.0); }
    void L_step(double *Ans, const double *F, const double *z) {
        std::vector<double> tmp(size_);
        calc_L(tmp.data(), F, z, nullptr, nullptr);
        std::copy(tmp.begin(), tmp.end(), Ans);
    }
    void L_1_step(double *Ans, const double *F, const double *z) {
        std::vector<double> tmp(size_, 0.0);   // calc_L_1 adds into its output
        calc_L_1(tmp.data(), F, z, nullptr, nullptr);
        std::copy(tmp.begin(), tmp.end(), Ans);
    }
    void LT_step(double *Ans, const double *F, const double *z) {
        std::vector<double> tmp(size_);
        calc_LT(tmp.data(), F, z, nullptr, nullptr);
        std::copy(tmp.begin(), tmp.end(), Ans);
    }

    /* solver work of the last calc: iterations per solve kind, worst residual */
    void last_stats(int *iters_lapl, int *iters_a, int *iters_mj, int *iters_ml, double *worst_relres) {
        ck(phg_barvortex_last_stats(h_, iters_lapl, iters_a, iters_mj, iters_ml, worst_relres));
    }
    phg_barvortex handle() const { return h_; }

private:
    int size_;
    std::vector<double> forcing_;
    phg_barvortex h_ = nullptr;
};

/* Baroclin(m, f, g, coriolis, tau, sigma, mu, sigma1, mu1, alpha)
 * (examples/baroclin.h:147-175, examples/baroclin.cpp:69-106); f, g become
 * forcing values per call, coriolis its values at the points. */
class Baroclin {
public:
    Baroclin(Operators &o, const double *coriolis, double tau, double sigma, double mu, double sigma1, double mu1,
             double alpha, int picard_iters = 20, double picard_tol = 1e-8) {
        phg_bc_conf c;
        c.tau = tau; c.sigma = sigma; c.mu = mu; c.sigma1 = sigma1; c.mu1 = mu1; c.alpha = alpha;
        c.picard_iters = picard_iters; c.picard_tol = picard_tol;
        ck(phg_baroclin_create(o.handle(), &c, coriolis, &h_));
    }
    ~Baroclin() { phg_baroclin_destroy(h_); }
    Baroclin(const Baroclin &) = delete;
    Baroclin &operator=(const Baroclin &) = delete;

    /* Baroclin::calc (examples/baroclin.cpp:445-606); f, g: forcing at time t */
    void calc(double *u11, double *u21, const double *u1, const double *u2, const double *bnd, double t = 0.0,
              const double *f = nullptr, const double *g = nullptr) {
        (void)t;
        ck(phg_baroclin_calc(h_, u11, u21, u1, u2, bnd, f, g, nullptr));
    }
    /* Baroclin::calc_L / calc_L_1 (examples/baroclin.cpp:620-986) */
    void calc_L(double *u11, double *u21, const double *u1, const double *u2, const double *z1, const double *z2,
                const double *bnd, double = 0.0) {
        ck(phg_baroclin_calc_L(h_, u11, u21, u1, u2, z1, z2, bnd, nullptr));
    }
    void calc_L_1(double *u11, double *u21, const double *u1, const double *u2, const double *z1, const double *z2,
                  const double *bnd, double = 0.0) {
        ck(phg_baroclin_calc_L_1(h_, u11, u21, u1, u2, z1, z2, bnd, nullptr));
    }
    phg_baroclin handle() const { return h_; }

private:
    phg_baroclin h_ = nullptr;
};

typedef BarVortex SBarVortex;

}  // namespace phelm_gb300

#endif
