// phg_assemble.cpp -- host assembly of the P1 sphere operators.
//
// Matrix entries must equal the reference's bit for bit: at level 6 a
// Laplacian apply cancels about four decimal digits, so two assemblies that
// differ only in rounding disagree at ~1e-9 after one apply.  The entry
// formulas therefore keep the reference's arithmetic order:
//   P1 basis in the row point's chart          src/mesh.cpp:563-607
//   polynomial product / derivative / value    src/polynom.cpp:63-87, 147-184, 667-696
//   triangle = two trapezoids, exact in v,
//   Gauss-Kronrod 15 in u (15-digit table)     src/polynom.cpp:188-315, src/util.cpp:165-227,
//                                              src/quadrature.c:48-128
//   7-point degree-5 cubature (16-digit table) src/quadrature.c:130-171
//   slaplace form                              src/slaplace.cpp:75-105
//   Jacobian derivative forms                  src/sjacobian.cpp:53-134
//   row loop / boundary-column loop            src/generators.cpp:57-212
// What differs is the organisation: every (row, triangle, vertex) triple is
// visited once and yields the contributions of all operators at the same
// time (the reference runs one full assembly per matrix), and rows run in
// parallel with no shared caches.
#include <cmath>
#include <cstring>
#include <algorithm>

#include "phg_host.hpp"

namespace phg {

CsrBuilder::CsrBuilder(int n, int m) : n_(n), m_(m), rows_(n) {}

void CsrBuilder::add(int i, int j, double a) {
    auto &r = rows_[i];
    for (auto &e : r)
        if (e.first == j) { e.second += a; return; }
    r.emplace_back(j, 0.0 + a);
}

void CsrBuilder::finish(Csr &out) {
    out.n = n_; out.m = m_;
    out.ptr.assign(n_ + 1, 0);
    for (int i = 0; i < n_; ++i) out.ptr[i + 1] = out.ptr[i] + (int)rows_[i].size();
    out.col.resize(out.ptr[n_]);
    out.val.resize(out.ptr[n_]);
    for (int i = 0; i < n_; ++i) {
        auto &r = rows_[i];
        std::stable_sort(r.begin(), r.end(), [](const std::pair<int, double> &a, const std::pair<int, double> &b) {
            return a.first < b.first;
        });
        for (size_t k = 0; k < r.size(); ++k) {
            out.col[out.ptr[i] + k] = r[k].first;
            out.val[out.ptr[i] + k] = r[k].second;
        }
        std::vector<std::pair<int, double>>().swap(r);
    }
}

namespace {

inline double ipow(double x, int n) {
    double r = 1.0;
    for (int i = 0; i < n; ++i) r *= x;
    return r;
}

// sum_{i<=xd, j<=yd} k[i*(yd+1)+j] x^i y^j, degrees <= 2
struct Poly {
    int xd = 0, yd = 0;
    double k[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double at(int i, int j) const { return (i > xd || j > yd) ? 0.0 : k[i * (yd + 1) + j]; }
    double eval(double x, double y) const {
        double xi[3], yj[3], r = 0.0;
        for (int i = 0; i <= xd; ++i) xi[i] = ipow(x, i);
        for (int j = 0; j <= yd; ++j) yj[j] = ipow(y, j);
        for (int i = 0; i <= xd; ++i)
            for (int j = 0; j <= yd; ++j) r += k[i * (yd + 1) + j] * xi[i] * yj[j];
        return r;
    }
};

Poly mul(const Poly &a, const Poly &b) {
    Poly r;
    r.xd = a.xd + b.xd; r.yd = a.yd + b.yd;
    for (int i = 0; i <= a.xd; ++i)
        for (int j = 0; j <= a.yd; ++j)
            for (int p = 0; p <= b.xd; ++p)
                for (int q = 0; q <= b.yd; ++q)
                    r.k[(i + p) * (r.yd + 1) + (j + q)] += a.k[i * (a.yd + 1) + j] * b.k[p * (b.yd + 1) + q];
    return r;
}

Poly ddx(const Poly &p) {  // d/du
    Poly r;
    r.xd = p.xd - 1; r.yd = p.yd;
    for (int j = 0; j <= r.yd; ++j)
        for (int i = 0; i <= r.xd; ++i) r.k[i * (r.yd + 1) + j] = (double)(i + 1) * p.k[(i + 1) * (p.yd + 1) + j];
    return r;
}

Poly ddy(const Poly &p) {  // d/dv
    Poly r;
    r.xd = p.xd; r.yd = p.yd - 1;
    for (int i = 0; i <= r.xd; ++i)
        for (int j = 0; j <= r.yd; ++j) r.k[i * (r.yd + 1) + j] = (double)(j + 1) * p.k[i * (p.yd + 1) + j + 1];
    return r;
}

// linear form vanishing on the edge (a, b): (u - a.u)(b.v - a.v) - (v - a.v)(b.u - a.u)
Poly edge_form(double au, double av, double bu, double bv) {
    double du = bv - av, dv = bu - au;
    double x0 = (0.0 - au) * du, x1 = 1.0 * du;   // (u - au) * du
    double y0 = (0.0 - av) * dv, y1 = 1.0 * dv;   // (v - av) * dv
    Poly r;
    r.xd = 1; r.yd = 1;
    r.k[0] = x0 - y0;    // (0,0)
    r.k[1] = 0.0 - y1;   // (0,1)
    r.k[2] = x1 - 0.0;   // (1,0)
    r.k[3] = 0.0 - 0.0;  // (1,1)
    return r;
}

// The 15-point Kronrod rule on [-1, 1] with the reference's 15-digit table
// (nodes +-x with equal weights; Gauss points first).
const double KR[15][2] = {
    {+0.949107912342759, 0.063092092629979}, {-0.949107912342759, 0.063092092629979},
    {+0.741531185599394, 0.140653259715525}, {-0.741531185599394, 0.140653259715525},
    {+0.405845151377397, 0.190350578064785}, {-0.405845151377397, 0.190350578064785},
    {0.000000000000000, 0.209482141084728},
    {+0.991455371120813, 0.022935322010529}, {-0.991455371120813, 0.022935322010529},
    {+0.864864423359769, 0.104790010322250}, {-0.864864423359769, 0.104790010322250},
    {+0.586087235467691, 0.169004726639267}, {-0.586087235467691, 0.169004726639267},
    {+0.207784955007898, 0.204432940075298}, {-0.207784955007898, 0.204432940075298}};

enum Weight { W_COS, W_INV_COS };

// int_{x1}^{x3} x^k [(k2 x + b2)^{n+1} - (k1 x + b1)^{n+1}]/(n+1) w(x) dx
double strip(Weight w, int k, int n, double k1, double b1, double k2, double b2, double x1, double x3) {
    double acc = 0.0, h = 0.5 * (x3 - x1), c = 0.5 * (x3 + x1);
    for (int q = 0; q < 15; ++q) {
        double x = h * KR[q][0] + c;
        double s = (ipow(k2 * x + b2, n + 1) - ipow(k1 * x + b1, n + 1)) / (double)(n + 1);
        double f = w == W_COS ? ipow(x, k) * s * std::cos(x) : ipow(x, k) * s / std::cos(x);
        acc += KR[q][1] * f;
    }
    return acc * h;
}

// integral of p * w(u) over the planar triangle (xs[q], ys[q])
double tri_integral(const Poly &p, Weight w, const double xs[3], const double ys[3]) {
    double x1 = xs[0], x2 = xs[1], x3 = xs[2], y1 = ys[0], y2 = ys[1], y3 = ys[2], t;
    // order so that x3 (the split line) is the middle abscissa
    if (x1 <= x2 && x2 <= x3) { t = x2; x2 = x3; x3 = t; t = y2; y2 = y3; y3 = t; }
    else if (x2 <= x1 && x1 <= x3) {
        t = x1; x1 = x2; x2 = t; t = x2; x2 = x3; x3 = t;
        t = y1; y1 = y2; y2 = t; t = y2; y2 = y3; y3 = t;
    } else if (x2 <= x3 && x3 <= x1) { t = x1; x1 = x2; x2 = t; t = y1; y1 = y2; y2 = t; }
    else if (x3 <= x1 && x1 <= x2) { t = x1; x1 = x3; x3 = t; t = y1; y1 = y3; y3 = t; }
    else if (x3 <= x2 && x2 <= x1) {
        t = x1; x1 = x3; x3 = t; t = x2; x2 = x3; x3 = t;
        t = y1; y1 = y3; y3 = t; t = y2; y2 = y3; y3 = t;
    }
    const double k1 = (y2 - y1) / (x2 - x1), b1 = (y1 * x2 - x1 * y2) / (x2 - x1);
    double left = 0.0, right = 0.0;
    if (std::fabs(x1 - x3) > 1e-15) {
        const double k3 = (y3 - y1) / (x3 - x1), b3 = (y1 * x3 - x1 * y3) / (x3 - x1);
        for (int a = 0; a <= p.xd; ++a)
            for (int b = 0; b <= p.yd; ++b) left += p.k[a * (p.yd + 1) + b] * strip(w, a, b, k1, b1, k3, b3, x1, x3);
    }
    if (std::fabs(x3 - x2) > 1e-15) {
        const double k2 = (y2 - y3) / (x2 - x3), b2 = (y3 * x2 - x3 * y2) / (x2 - x3);
        for (int a = 0; a <= p.xd; ++a)
            for (int b = 0; b <= p.yd; ++b) right += p.k[a * (p.yd + 1) + b] * strip(w, a, b, k1, b1, k2, b2, x3, x2);
    }
    if (y3 >= y1 && y3 >= y2) return left + right;
    if (y3 <= y1 && y3 <= y2) return -left - right;
    if (y3 >= k1 * x3 + b1) return left + right;
    return -left - right;
}

// Radon's 7-point degree-5 rule (barycentric nodes/weights, 16 digits as the
// reference tabulates them).
const double C7W[7] = {0.225, 0.1259391805448265, 0.1259391805448265, 0.1259391805448265,
                       0.1323941527885112, 0.1323941527885112, 0.1323941527885112};
const double C7A = 0.7974269853530880, C7B = 0.1012865073234560;
const double C7C = 0.0597158717897742, C7D = 0.4701420641051129;
const double C7N[7][3] = {{1. / 3., 1. / 3., 1. / 3.}, {C7A, C7B, C7B}, {C7B, C7A, C7B}, {C7B, C7B, C7A},
                          {C7C, C7D, C7D}, {C7D, C7C, C7D}, {C7D, C7D, C7C}};

double cub7(const Poly &p, bool with_cos, const double xs[3], const double ys[3]) {
    double s = 0.0;
    for (int q = 0; q < 7; ++q) {
        double a = C7N[q][0], b = C7N[q][1], c = C7N[q][2];
        double u = a * xs[0] + b * xs[1] + c * xs[2];
        double v = a * ys[0] + b * ys[1] + c * ys[2];
        double f = with_cos ? std::cos(u) * p.eval(u, v) : p.eval(u, v);
        s += C7W[q] * f;
    }
    s *= 0.5 * std::fabs(((xs[0] - xs[2]) * (ys[1] - ys[2]) - (ys[0] - ys[2]) * (xs[1] - xs[2])));
    return s;
}

// One triangle seen from one chart: vertex coordinates and the P1 basis.
struct Element {
    double xs[3], ys[3];
    Poly phi[3];
    Element(const Mesh &m, int t, int z) {
        const int *v = &m.tri[3 * (size_t)t];
        for (int q = 0; q < 3; ++q) { xs[q] = m.u(v[q], z); ys[q] = m.v(v[q], z); }
        phi[0] = edge_form(xs[1], ys[1], xs[2], ys[2]);
        phi[1] = edge_form(xs[0], ys[0], xs[2], ys[2]);
        phi[2] = edge_form(xs[0], ys[0], xs[1], ys[1]);
        for (int q = 0; q < 3; ++q) {
            double s = 1.0 / phi[q].eval(xs[q], ys[q]);
            for (double &c : phi[q].k) c *= s;
        }
    }
    double mass(int i, int j) const { return tri_integral(mul(phi[i], phi[j]), W_COS, xs, ys); }
    // slaplace(phi_a, phi_b)
    double slap(int a, int b) const {
        double l1 = -tri_integral(mul(ddx(phi[a]), ddx(phi[b])), W_COS, xs, ys);
        double l2 = -tri_integral(mul(ddy(phi[a]), ddy(phi[b])), W_INV_COS, xs, ys);
        return (l1 + l2);
    }
    double jmass(int i, int j) const { return cub7(mul(phi[i], phi[j]), true, xs, ys); }
    // int phi_i d(phi_j)/du [cos u] and int phi_i d(phi_j)/dv [cos u]
    double d1(int i, int j, bool c) const { return cub7(mul(ddx(phi[j]), phi[i]), c, xs, ys); }
    double d2(int i, int j, bool c) const { return cub7(mul(ddy(phi[j]), phi[i]), c, xs, ys); }
};

int vertex_slot(const Mesh &m, int t, int p) {
    for (int q = 0; q < 3; ++q)
        if (m.tri[3 * (size_t)t + q] == p) return q;
    return -1;
}

// Visit every (row point, triangle through it, vertex of that triangle) in
// the reference's order; f(element, slot of row point, slot of vertex).
template <typename F>
void for_row(const Mesh &m, int p, F &&f) {
    const int zone = m.row_zone(p);
    for (int k = m.adj_ptr[p]; k < m.adj_ptr[p + 1]; ++k) {
        const int t = m.adj[k];
        Element e(m, t, zone);
        const int ip = vertex_slot(m, t, p);
        for (int q = 0; q < 3; ++q) f(e, t, ip, q);
    }
}

}  // namespace

void assemble_sphere(const Mesh &m, SphereOps &o) {
    const int rs = m.rs, os = m.os, V = m.V;
    CsrBuilder idt(rs, rs), lapl(rs, rs), jidt(rs, rs), d1(rs, rs), d2(rs, rs), d1c(rs, rs), d2c(rs, rs);
    CsrBuilder norm(V, V);
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < rs; ++i) {
        for_row(m, m.inner[i], [&](const Element &e, int t, int ip, int q) {
            const int p2 = m.tri[3 * (size_t)t + q];
            if (m.bnd[p2]) return;
            const int j = m.p2io[p2];
            idt.add(i, j, e.mass(ip, q));
            lapl.add(i, j, e.slap(q, ip));
            jidt.add(i, j, e.jmass(ip, q));
            d1.add(i, j, e.d1(ip, q, false));
            d2.add(i, j, e.d2(ip, q, false));
            d1c.add(i, j, e.d1(ip, q, true));
            d2c.add(i, j, e.d2(ip, q, true));
        });
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (int p = 0; p < V; ++p)
        for_row(m, p, [&](const Element &e, int t, int ip, int q) { norm.add(p, m.tri[3 * (size_t)t + q], e.mass(ip, q)); });
    // boundary columns: integrated in the boundary point's chart
    CsrBuilder b2(rs, os), b3(rs, os), db1(rs, os), db2(rs, os), db1c(rs, os), db2c(rs, os);
    for (int j = 0; j < os; ++j) {
        for_row(m, m.outer[j], [&](const Element &e, int t, int jp, int q) {
            const int p = m.tri[3 * (size_t)t + q];
            if (m.bnd[p]) return;
            const int i = m.p2io[p];
            const double s = e.slap(jp, q);
            b2.add(i, j, -s);
            b3.add(i, j, s);
            db1.add(i, j, e.d1(q, jp, false));
            db2.add(i, j, e.d2(q, jp, false));
            db1c.add(i, j, e.d1(q, jp, true));
            db2c.add(i, j, e.d2(q, jp, true));
        });
    }
    idt.finish(o.idt); lapl.finish(o.lapl); jidt.finish(o.jidt);
    d1.finish(o.d1); d2.finish(o.d2); d1c.finish(o.d1c); d2c.finish(o.d2c);
    norm.finish(o.norm);
    b2.finish(o.bnd2); b3.finish(o.bnd3);
    db1.finish(o.d1b); db2.finish(o.d2b); db1c.finish(o.d1cb); db2c.finish(o.d2cb);
}

void assemble_barvortex(const Mesh &m, double c1, double c2, Csr &A, Csr &Abnd) {
    const int rs = m.rs, os = m.os;
    CsrBuilder a(rs, rs), ab(rs, os);
    auto entry = [&](const Element &e, int i0, int j0) {
        double pt1 = e.mass(i0, j0);
        pt1 *= c1;
        double pt2 = e.slap(j0, i0);
        pt2 *= c2;
        return pt1 + pt2;
    };
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < rs; ++i) {
        for_row(m, m.inner[i], [&](const Element &e, int t, int ip, int q) {
            const int p2 = m.tri[3 * (size_t)t + q];
            if (!m.bnd[p2]) a.add(i, m.p2io[p2], entry(e, ip, q));
        });
    }
    for (int j = 0; j < os; ++j) {
        for_row(m, m.outer[j], [&](const Element &e, int t, int jp, int q) {
            const int p = m.tri[3 * (size_t)t + q];
            if (!m.bnd[p]) ab.add(m.p2io[p], j, entry(e, q, jp));
        });
    }
    a.finish(A);
    ab.finish(Abnd);
}

namespace {
// the nine block entries of one (row, column) contribution
// (examples/baroclin.cpp:138-177), rows/cols in blocks [w1 | w2 | u1 | u2]
void baroclin_blocks(const BaroclinParams &c, double a, double b, double e[9]) {
    const double tau = c.tau, mu = c.mu, mu1 = c.mu1, sigma = c.sigma, sigma1 = c.sigma1;
    const double alpha = c.alpha, theta = c.theta;
    if (c.backward) {   // examples/baroclin.cpp:214-241
        e[0] = a * (1.0 / tau - 0.5 * (1.0 - theta) * sigma) + (1.0 - theta) * mu * b;
        e[1] = 0.5 * a * sigma * (1.0 - theta);
        e[2] = -0.5 * (1.0 - theta) * sigma * a;
        e[3] = a * (1.0 / tau - 0.5 * (1.0 - theta) * sigma - alpha * alpha * (1.0 - theta) * mu1) +
               (1.0 - theta) * mu * b;
        e[4] = a * (-alpha * alpha / tau + alpha * alpha * (1.0 - theta) * sigma1);
        e[5] = a;
        e[6] = -b;
        e[7] = a;
        e[8] = -b;
        return;
    }
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
const int BR[9] = {0, 0, 1, 1, 1, 2, 2, 3, 3};
const int BC[9] = {0, 1, 0, 1, 3, 0, 2, 1, 3};
}  // namespace

void assemble_baroclin(const Mesh &m, const BaroclinParams &c, Csr &A, Csr bcol[4]) {
    const int rs = m.rs, os = m.os;
    CsrBuilder a(4 * rs, 4 * rs);
    CsrBuilder bc0(rs, os), bc1(rs, os), bc2(rs, os), bc3(rs, os);
    CsrBuilder *bcb[4] = {&bc0, &bc1, &bc2, &bc3};
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < rs; ++i) {
        for_row(m, m.inner[i], [&](const Element &e, int t, int ip, int q) {
            const int p2 = m.tri[3 * (size_t)t + q];
            double blk[9];
            baroclin_blocks(c, e.mass(ip, q), e.slap(q, ip), blk);
            if (!m.bnd[p2]) {
                const int j = m.p2io[p2];
                for (int k = 0; k < 9; ++k) a.add(i + BR[k] * rs, j + BC[k] * rs, blk[k]);
            } else {
                double acc[4] = {0, 0, 0, 0};
                for (int k = 0; k < 9; ++k) acc[BR[k]] += blk[k];
                for (int r = 0; r < 4; ++r) bcb[r]->add(i, m.p2io[p2], acc[r]);
            }
        });
    }
    a.finish(A);
    for (int r = 0; r < 4; ++r) bcb[r]->finish(bcol[r]);
}

}  // namespace phg

namespace phg {

void assemble_laplacian(const Mesh &m, Csr &lapl) {
    const int rs = m.rs;
    CsrBuilder b(rs, rs);
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < rs; ++i) {
        for_row(m, m.inner[i], [&](const Element &e, int t, int ip, int q) {
            const int p2 = m.tri[3 * (size_t)t + q];
            if (!m.bnd[p2]) b.add(i, m.p2io[p2], e.slap(q, ip));
        });
    }
    b.finish(lapl);
}

namespace {

Csr transpose(const Csr &a) {
    Csr t;
    t.n = a.m; t.m = a.n;
    t.ptr.assign(t.n + 1, 0);
    for (int k = 0; k < a.nnz(); ++k) t.ptr[a.col[k] + 1]++;
    for (int i = 0; i < t.n; ++i) t.ptr[i + 1] += t.ptr[i];
    t.col.resize(a.nnz()); t.val.resize(a.nnz());
    std::vector<int> fill(t.ptr.begin(), t.ptr.end() - 1);
    for (int i = 0; i < a.n; ++i)
        for (int k = a.ptr[i]; k < a.ptr[i + 1]; ++k) {
            int q = fill[a.col[k]]++;
            t.col[q] = i; t.val[q] = a.val[k];
        }
    return t;
}

// prolongation from the coarse mesh (one refinement less) to the fine mesh
Csr prolongation(const Mesh &f, const Mesh &c) {
    std::vector<int> rcm_of(c.V);
    for (int i = 0; i < c.V; ++i) rcm_of[c.orig[i]] = i;
    CsrBuilder b(f.rs, c.rs);
    for (int r = 0; r < f.rs; ++r) {
        const int p = f.orig[f.inner[r]];
        auto put = [&](int pre, double w) {
            const int ci = rcm_of[pre];
            if (!c.bnd[ci]) b.add(r, c.p2io[ci], w);
        };
        if (p < c.V) put(p, 1.0);
        else { put(f.par_a[p], 0.5); put(f.par_b[p], 0.5); }
    }
    Csr P;
    b.finish(P);
    return P;
}

bool dense_inverse(const Csr &a, std::vector<double> &inv) {
    const int n = a.n;
    std::vector<double> M((size_t)n * 2 * n, 0.0);
    for (int i = 0; i < n; ++i) {
        for (int k = a.ptr[i]; k < a.ptr[i + 1]; ++k) M[(size_t)i * 2 * n + a.col[k]] = a.val[k];
        M[(size_t)i * 2 * n + n + i] = 1.0;
    }
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(M[(size_t)r * 2 * n + c]) > std::fabs(M[(size_t)piv * 2 * n + c])) piv = r;
        if (M[(size_t)piv * 2 * n + c] == 0.0) return false;
        if (piv != c)
            for (int k = 0; k < 2 * n; ++k) std::swap(M[(size_t)c * 2 * n + k], M[(size_t)piv * 2 * n + k]);
        const double d = M[(size_t)c * 2 * n + c];
        for (int k = 0; k < 2 * n; ++k) M[(size_t)c * 2 * n + k] /= d;
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            const double f = M[(size_t)r * 2 * n + c];
            if (f == 0.0) continue;
            for (int k = 0; k < 2 * n; ++k) M[(size_t)r * 2 * n + k] -= f * M[(size_t)c * 2 * n + k];
        }
    }
    inv.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) inv[(size_t)i * n + j] = M[(size_t)i * 2 * n + n + j];
    return true;
}

}  // namespace

bool build_mg(const Mesh &fine, int coarsest_level, MgHierarchy &h, std::string &err) {
    h = MgHierarchy();
    if (fine.level < 0 || fine.orig.empty()) { err = "multigrid needs a generated icosahedral mesh"; return false; }
    if (coarsest_level < 1) coarsest_level = 1;
    const int nlev = fine.level - coarsest_level + 1;
    if (nlev < 2) { err = "mesh too coarse for multigrid"; return false; }
    h.mesh.resize(nlev);
    h.A.resize(nlev);
    h.P.resize(nlev - 1);
    h.R.resize(nlev - 1);
    for (int k = 1; k < nlev; ++k) {
        if (!generate_sphere(fine.level - k, h.mesh[k], err)) return false;
        assemble_laplacian(h.mesh[k], h.A[k]);
    }
    for (int k = 0; k + 1 < nlev; ++k) {
        const Mesh &f = k == 0 ? fine : h.mesh[k];
        h.P[k] = prolongation(f, h.mesh[k + 1]);
        h.R[k] = transpose(h.P[k]);
    }
    if (!dense_inverse(h.A[nlev - 1], h.coarse_inv)) { err = "coarsest Laplacian is singular"; return false; }
    return true;
}

}  // namespace phg
