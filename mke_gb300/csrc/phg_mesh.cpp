// phg_mesh.cpp -- icosahedral sphere meshes for the GB300 sphere-FEM library.
//
// The point order must be the reference's own, because every matrix row,
// chart choice and boundary index follows it, so this generator reproduces
// the reference mesh generator step by step:
//   icosahedron table and orthogonal projection  utils/mesh_builder.cpp:52-125
//   midpoint refinement, one new point per edge   utils/mesh_builder.cpp:143-201
//   south pole = boundary                         utils/icosahedron.cpp:416-421
//   Cuthill-McKee over inner points, neighbours
//   by (degree incl. self, id), outer points last utils/mesh_builder.cpp:316-402, 504-585
//   4 charts + triangle zone rule                 utils/icosahedron.cpp:251-266, 327-393
//   16-decimal text round trip of coordinates     utils/icosahedron.cpp:320, src/mesh.cpp:365-402
// The text loader follows src/mesh.cpp:323-519.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <unordered_map>

#include "phg_host.hpp"

namespace phg {
namespace {

struct P3 { double x, y, z; };

void to_sphere(P3 &p) {
    double l = std::sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
    p.x /= l; p.y /= l; p.z /= l;
}

double lat_of(double, double, double z) { return std::asin(z); }

double lon_of(double x, double y, double) {
    double r = std::sqrt(x * x + y * y);
    if (r < 1e-15) return 0.0;
    double a = std::acos(x / r);
    return y < 0 ? 2.0 * M_PI - a : a;
}

// value after printf("%.16lf") and strtod
double text16(double v) {
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.16lf", v);
    return std::strtod(buf, nullptr);
}

}  // namespace

void finish_mesh(Mesh &m) {
    m.rs = m.os = 0;
    m.inner.clear(); m.outer.clear();
    m.p2io.assign(m.V, 0);
    for (int i = 0; i < m.V; ++i) {
        if (m.bnd[i]) { m.p2io[i] = m.os++; m.outer.push_back(i); }
        else { m.p2io[i] = m.rs++; m.inner.push_back(i); }
    }
    m.adj_ptr.assign(m.V + 1, 0);
    for (int k = 0; k < 3 * m.T; ++k) m.adj_ptr[m.tri[k] + 1]++;
    for (int i = 0; i < m.V; ++i) m.adj_ptr[i + 1] += m.adj_ptr[i];
    m.adj.assign(3 * (size_t)m.T, 0);
    std::vector<int> fill(m.adj_ptr.begin(), m.adj_ptr.end() - 1);
    for (int t = 0; t < m.T; ++t)
        for (int q = 0; q < 3; ++q) m.adj[fill[m.tri[3 * t + q]]++] = t;
}

bool generate_sphere(int level, Mesh &m, std::string &err) {
    if (level < 1 || level > 9) { err = "level must be in 1..9 (level 0 has no boundary point)"; return false; }
    const double g = (1.0 + std::sqrt(5.0)) / 2.0;
    std::vector<P3> pts = {
        {g, 1, 0}, {-g, 1, 0}, {g, -1, 0}, {-g, -1, 0}, {1, 0, g}, {1, 0, -g},
        {-1, 0, g}, {-1, 0, -g}, {0, g, 1}, {0, -g, 1}, {0, g, -1}, {0, -g, -1}};
    std::vector<int> tr = {0, 8, 4, 1, 10, 7, 2, 9, 11, 7, 3, 1, 0, 5, 10, 3, 9, 6, 3, 11, 9,
                           8, 6, 4, 2, 4, 9, 3, 7, 11, 4, 2, 0, 9, 4, 6, 2, 11, 5, 0, 10, 8,
                           5, 0, 2, 10, 5, 7, 1, 6, 8, 1, 8, 10, 6, 1, 3, 11, 7, 5};
    for (auto &p : pts) to_sphere(p);

    std::vector<int> par_a(12, -1), par_b(12, -1);
    for (int it = 0; it < level; ++it) {
        const int V_old = (int)pts.size();
        par_a.assign(V_old, -1);
        par_b.assign(V_old, -1);
        std::unordered_map<long long, int> mid;
        mid.reserve(tr.size());
        std::vector<int> out;
        out.reserve(tr.size() * 4);
        const long long base = (long long)pts.size() + 1;
        auto midpoint = [&](int a, int b) {
            long long key = a < b ? a * base + b : b * base + a;
            auto f = mid.find(key);
            if (f != mid.end()) return f->second;
            P3 p{(pts[a].x + pts[b].x) / 2, (pts[a].y + pts[b].y) / 2, (pts[a].z + pts[b].z) / 2};
            to_sphere(p);
            int id = (int)pts.size();
            pts.push_back(p);
            par_a.push_back(a);
            par_b.push_back(b);
            mid.emplace(key, id);
            return id;
        };
        for (size_t t = 0; t < tr.size(); t += 3) {
            int a = tr[t], b = tr[t + 1], c = tr[t + 2];
            int ab = midpoint(a, b), ac = midpoint(a, c), bc = midpoint(b, c);
            int quad[12] = {a, ab, ac, c, ac, bc, b, bc, ab, ab, ac, bc};
            out.insert(out.end(), quad, quad + 12);
        }
        tr.swap(out);
    }
    const int V = (int)pts.size(), T = (int)tr.size() / 3;

    // boundary = south pole, inner numbering in point order
    std::vector<char> is_b(V, 0);
    std::vector<int> pos(V);
    int rs = 0, ob = 0;
    for (int i = 0; i < V; ++i) is_b[i] = std::fabs(pts[i].z + 1.0) < 1e-14;
    for (int i = 0; i < V; ++i) pos[i] = is_b[i] ? ob++ : rs++;

    // inner graph incl. self, as sorted sets
    std::vector<std::vector<int>> nb(rs);
    for (int t = 0; t < T; ++t)
        for (int q = 0; q < 3; ++q) {
            int a = tr[3 * t + q];
            if (is_b[a]) continue;
            for (int r = 0; r < 3; ++r)
                if (!is_b[tr[3 * t + r]]) nb[pos[a]].push_back(pos[tr[3 * t + r]]);
        }
    for (auto &s : nb) { std::sort(s.begin(), s.end()); s.erase(std::unique(s.begin(), s.end()), s.end()); }
    for (auto &s : nb)
        std::stable_sort(s.begin(), s.end(), [&](int x, int y) { return nb[x].size() < nb[y].size(); });
    // degrees were read while sorting; the sets' sizes do not change
    std::vector<int> cm(rs, -1);
    int next = 0;
    for (int start = 0; start < rs; ++start) {
        if (cm[start] >= 0) continue;
        std::deque<int> q{start};
        while (!q.empty()) {
            int v = q.front(); q.pop_front();
            if (cm[v] >= 0) continue;
            cm[v] = next++;
            for (int w : nb[v]) if (cm[w] < 0) q.push_back(w);
        }
    }
    std::vector<int> perm(V);  // old point -> new point
    for (int i = 0, o = rs; i < V; ++i) perm[i] = is_b[i] ? o++ : cm[pos[i]];

    m = Mesh();
    m.level = level; m.V = V; m.T = T; m.nz = 4;
    m.xyz.resize(3 * (size_t)V); m.uv.resize(8 * (size_t)V); m.bnd.assign(V, 0);
    std::vector<P3> np(V);
    for (int i = 0; i < V; ++i) np[perm[i]] = pts[i];
    m.raw_xyz.resize(3 * (size_t)V);
    for (int i = 0; i < V; ++i) { m.raw_xyz[3 * i] = np[i].x; m.raw_xyz[3 * i + 1] = np[i].y; m.raw_xyz[3 * i + 2] = np[i].z; }
    for (int i = 0; i < V; ++i) {
        const double x = np[i].x, y = np[i].y, z = np[i].z;
        m.xyz[3 * i] = text16(x); m.xyz[3 * i + 1] = text16(y); m.xyz[3 * i + 2] = text16(z);
        const double c[4][3] = {{x, y, z}, {-x, -y, z}, {x, -z, y}, {x, z, -y}};
        for (int k = 0; k < 4; ++k) {
            m.uv[8 * i + 2 * k] = text16(lat_of(c[k][0], c[k][1], c[k][2]));
            m.uv[8 * i + 2 * k + 1] = text16(lon_of(c[k][0], c[k][1], c[k][2]));
        }
        m.bnd[i] = std::fabs(z + 1.0) < 1e-14;
    }
    m.tri.resize(3 * (size_t)T); m.tz.resize(T);
    for (int t = 0; t < T; ++t) {
        int a = perm[tr[3 * t]], b = perm[tr[3 * t + 1]], c = perm[tr[3 * t + 2]];
        m.tri[3 * t] = a; m.tri[3 * t + 1] = b; m.tri[3 * t + 2] = c;
        const double za = np[a].z, zb = np[b].z, zc = np[c].z;
        const double la = lon_of(np[a].x, np[a].y, za), lb = lon_of(np[b].x, np[b].y, zb);
        int zone = 1;
        if (za > 0.9 || zb > 0.9 || zc > 0.9) zone = 4;
        else if (za < -0.9 || zb < -0.9 || zc < -0.9) zone = 3;
        // the reference tests the second vertex twice and never the third
        else if (la < M_PI_2 || lb < M_PI_2 || la > 1.5 * M_PI || lb > 1.5 * M_PI) zone = 2;
        m.tz[t] = zone - 1;
    }
    finish_mesh(m);
    m.orig.assign(V, 0);
    for (int i = 0; i < V; ++i) m.orig[perm[i]] = i;
    m.par_a = par_a;
    m.par_b = par_b;
    return true;
}

bool load_mesh_text(FILE *f, Mesh &m, std::string &err) {
    m = Mesh();
    static const char *conv_names[4] = {"stdsphere1", "stdsphere2", "stdsphere3", "stdsphere4"};
    std::vector<char> buf(1 << 16);
    char *s = buf.data();
    int lineno = 0;
    auto next = [&]() { ++lineno; return std::fgets(s, (int)buf.size() - 1, f) != nullptr; };
    if (!next()) { err = "empty mesh file"; return false; }
    // header comments; zone conversions must be the 4 sphere charts in order
    while (*s == '#') {
        const char *pre = "#predef: zone";
        if (std::strncmp(s, pre, std::strlen(pre)) == 0) {
            int zone = 0; char name[256] = {0};
            if (std::sscanf(s + std::strlen(pre), "%d %255s", &zone, name) == 2) {
                if (zone < 1 || zone > 4 || std::strcmp(name, conv_names[zone - 1]) != 0) {
                    err = "unsupported chart '" + std::string(name) + "' (only stdsphere1..4 in order)";
                    return false;
                }
            }
        }
        if (!next()) { err = "no points"; return false; }
    }
    // points
    do {
        if (*s == '#') break;
        double xyz[3] = {0, 0, 0};
        double uv[8];
        for (double &d : uv) d = NAN;
        int nuv = 0; bool have_xyz = false;
        // the ';'-separated fields, empty ones skipped (strtok's splitting,
        // without its hidden state: several threads may load meshes at once)
        for (char *tok = s, *semi; tok; tok = semi ? semi + 1 : nullptr) {
            semi = std::strchr(tok, ';');
            if (semi) *semi = '\0';
            if (!*tok) continue;
            double a = 0, b = 0, c = 0;
            int k = std::sscanf(tok, "%lf%lf%lf", &a, &b, &c);
            if (k == 3) { xyz[0] = a; xyz[1] = b; xyz[2] = c; have_xyz = true; }
            else if (k == 2) { if (nuv < 4) { uv[2 * nuv] = a; uv[2 * nuv + 1] = b; } ++nuv; }
            else { err = "bad point line " + std::to_string(lineno); return false; }
        }
        if (!have_xyz) { xyz[0] = uv[0]; xyz[1] = uv[1]; xyz[2] = 0; }
        m.xyz.insert(m.xyz.end(), xyz, xyz + 3);
        m.uv.insert(m.uv.end(), uv, uv + 8);
        m.V++;
    } while (next());
    if (!next()) { err = "no triangles"; return false; }
    do {
        if (*s == '#') break;
        int a, b, c, z = 1;
        if (std::sscanf(s, "%d%d%d ; %d", &a, &b, &c, &z) < 3) { err = "bad triangle line " + std::to_string(lineno); return false; }
        --a; --b; --c; --z;
        if (a < 0 || b < 0 || c < 0 || a >= m.V || b >= m.V || c >= m.V || z < 0 || z > 3) {
            err = "triangle out of range at line " + std::to_string(lineno); return false;
        }
        m.tri.push_back(a); m.tri.push_back(b); m.tri.push_back(c); m.tz.push_back(z);
        m.T++;
    } while (next());
    m.bnd.assign(m.V, 0);
    if (next()) {
        do {
            if (*s == '#') break;
            int n;
            if (std::sscanf(s, "%d", &n) != 1 || n < 1 || n > m.V) { err = "bad boundary line " + std::to_string(lineno); return false; }
            m.bnd[n - 1] = 1;
        } while (next());
    }
    for (int t = 0; t < m.T; ++t)
        for (int q = 0; q < 3; ++q)
            if (std::isnan(m.u(m.tri[3 * t + q], m.tz[t]))) { err = "triangle uses a missing chart"; return false; }
    finish_mesh(m);
    for (int i = 0; i < m.V; ++i)
        if (m.adj_ptr[i + 1] == m.adj_ptr[i]) { err = "point without triangles"; return false; }
    return true;
}

}  // namespace phg

namespace phg {

bool save_mesh_text(FILE *f, const Mesh &m) {
    if (m.nz != 4) return false;
    const bool raw = m.raw_xyz.size() == 3 * (size_t)m.V;
    if (m.level >= 0)   // the generator's command line and build tag (utils/icosahedron.cpp:565-570)
        std::fprintf(f, "#cmd:mke_mesh_sphere --type full --coord local --iter %d \n#build:$Id$\n", m.level);
    std::fprintf(f, "#points:%lu\n", (unsigned long)m.V);
    std::fprintf(f, "#triangles:%lu\n", (unsigned long)m.T);
    std::fprintf(f, "# zone1 ; zone2 ; zone 3; ... \n");
    std::fprintf(f, "# u = theta  [-pi/2, pi/2]\n# v = lambda [0, 2pi]\n");
    std::fprintf(f, "#predef: zone 1 stdsphere1\n");
    std::fprintf(f, "#predef: zone 2 stdsphere2\n");
    std::fprintf(f, "# zone 1\n# x = cos(u)*cos(v) \n# y = cos(u)*sin(v) \n# z = sin(u) \n"
                    "# zone 2\n# x = -cos(u)*cos(v) \n# y = -cos(u)*sin(v) \n# z = sin(u) \n");
    std::fprintf(f, "#predef: zone 3 stdsphere3\n");
    std::fprintf(f, "#predef: zone 4 stdsphere4\n");
    std::fprintf(f, "# zone 3\n# x = cos(u)*cos(v) \n# y = cos(u)*sin(v) \n# z = -sin(u) \n"
                    "# zone 4\n# x = cos(u)*cos(v) \n# y = -cos(u)*sin(v) \n# z = sin(u) \n");
    for (int i = 0; i < m.V; ++i) {
        const double *p = raw ? &m.raw_xyz[3 * (size_t)i] : &m.xyz[3 * (size_t)i];
        const double x = p[0], y = p[1], z = p[2];
        std::fprintf(f, "%.16lf %.16lf %.16lf", x, y, z);
        if (raw) {
            const double c[4][3] = {{x, y, z}, {-x, -y, z}, {x, -z, y}, {x, z, -y}};
            for (int k = 0; k < 4; ++k)
                std::fprintf(f, " ; %.16lf %.16lf ", lat_of(c[k][0], c[k][1], c[k][2]), lon_of(c[k][0], c[k][1], c[k][2]));
        } else {
            for (int k = 0; k < 4; ++k) std::fprintf(f, " ; %.16lf %.16lf ", m.u(i, k), m.v(i, k));
        }
        std::fprintf(f, "\n");
    }
    std::fprintf(f, "# triangles %lu \n", (unsigned long)m.T);
    for (int t = 0; t < m.T; ++t) {
        std::fprintf(f, "%d %d %d ", m.tri[3 * t] + 1, m.tri[3 * t + 1] + 1, m.tri[3 * t + 2] + 1);
        if (m.tz[t] > 0) std::fprintf(f, " ; %d ", m.tz[t] + 1);
        std::fprintf(f, "\n");
    }
    std::fprintf(f, "# boundary \n");
    for (int i = 0; i < m.V; ++i)
        if (m.bnd[i]) std::fprintf(f, "%lu \n", (unsigned long)(i + 1));
    return true;
}

void print_function_text(FILE *f, const Mesh &m, const double *ans, const double *x, const double *y,
                         const double *z, bool inner_only) {
    const int n = inner_only ? m.rs : m.V;
    std::fprintf(f, "# points %lu\n", (unsigned long)n);
    for (int k = 0; k < n; ++k) {
        const int p = inner_only ? m.inner[k] : k;
        const double u = m.u(p, 0), v = m.v(p, 0);
        std::fprintf(f, "%.16lf ", x ? x[p] : u);
        std::fprintf(f, "%.16lf ", y ? y[p] : v);
        std::fprintf(f, "%.16lf ", z ? z[p] : 0.0);
        std::fprintf(f, "%.16lf %.16lf %.16lf \n", ans[p], u, v);
    }
    std::fprintf(f, "# triangles %lu\n", (unsigned long)m.T);
    for (int t = 0; t < m.T; ++t) {
        const int a = m.tri[3 * t], b = m.tri[3 * t + 1], c = m.tri[3 * t + 2];
        if (!inner_only) std::fprintf(f, "%d %d %d\n", a + 1, b + 1, c + 1);
        // the reference prints the triangles whose three points are all NOT
        // regular (src/phelm.cpp:208-218), i.e. boundary triangles; kept as is
        else if (m.bnd[a] && m.bnd[b] && m.bnd[c])
            std::fprintf(f, "%d %d %d\n", m.p2io[a] + 1, m.p2io[b] + 1, m.p2io[c] + 1);
    }
    std::fprintf(f, "# end \n");
}

}  // namespace phg
