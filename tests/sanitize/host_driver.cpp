// Runs the library's host code (mesh generation, text round trip, operator
// assembly, multigrid hierarchy, barotropic and baroclinic matrices, text
// output) at levels 1-4 under AddressSanitizer and UndefinedBehaviorSanitizer.
// Built and run by tests/test_sanitizers.py; exits non-zero on the first
// inconsistency (the sanitizers abort on their own findings).
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "phg_host.hpp"

using namespace phg;

static int check(bool ok, const char *what, int level) {
    if (!ok) fprintf(stderr, "level %d: %s\n", level, what);
    return ok ? 0 : 1;
}

static bool csr_ok(const Csr &a) {
    if ((int)a.ptr.size() != a.n + 1 || a.ptr[0] != 0) return false;
    for (int i = 0; i < a.n; ++i)
        if (a.ptr[i + 1] < a.ptr[i]) return false;
    for (int q = 0; q < a.nnz(); ++q)
        if (a.col[q] < 0 || a.col[q] >= a.m || !std::isfinite(a.val[q])) return false;
    return true;
}

int main() {
    int bad = 0;
    for (int level = 1; level <= 4; ++level) {
        Mesh m;
        std::string err;
        bad += check(generate_sphere(level, m, err), "generate_sphere", level);
        // text round trip
        FILE *f = tmpfile();
        bad += check(f && save_mesh_text(f, m), "save_mesh_text", level);
        rewind(f);
        Mesh back;
        bad += check(load_mesh_text(f, back, err), "load_mesh_text", level);
        fclose(f);
        bad += check(back.V == m.V && back.T == m.T && back.rs == m.rs && back.tri == m.tri, "round trip", level);
        // operators
        SphereOps ops;
        assemble_sphere(m, ops);
        const Csr *all[] = {&ops.idt, &ops.lapl, &ops.jidt, &ops.d1, &ops.d2, &ops.d1c, &ops.d2c,
                            &ops.bnd2, &ops.bnd3, &ops.d1b, &ops.d2b, &ops.d1cb, &ops.d2cb, &ops.norm};
        for (const Csr *a : all) bad += check(csr_ok(*a), "operator pattern", level);
        if (level >= 2) {
            MgHierarchy h;
            bad += check(build_mg(m, 1, h, err), "build_mg", level);
            for (size_t k = 1; k < h.A.size(); ++k) bad += check(csr_ok(h.A[k]), "coarse Laplacian", level);
            for (size_t k = 0; k < h.P.size(); ++k) bad += check(csr_ok(h.P[k]) && csr_ok(h.R[k]), "transfer", level);
        }
        Csr A, Ab;
        assemble_barvortex(m, 1e3 + 0.008, -4e-5, A, Ab);
        bad += check(csr_ok(A) && csr_ok(Ab), "barvortex matrices", level);
        for (int back_dir = 0; back_dir < 2; ++back_dir) {
            BaroclinParams p{1e-3, 0.05, 6.77e-5, 0.05, 6.77e-5, std::sqrt(0.1), 0.5, back_dir == 1};
            Csr B, bcol[4];
            assemble_baroclin(m, p, B, bcol);
            bad += check(csr_ok(B), "baroclin matrix", level);
            for (auto &c : bcol) bad += check(csr_ok(c), "baroclin boundary columns", level);
        }
        // text output of a field
        std::vector<double> u(m.V);
        for (int i = 0; i < m.V; ++i) u[i] = std::sin(3.0 * m.xyz[3 * i]) * std::cos(2.0 * m.xyz[3 * i + 2]);
        FILE *g = tmpfile();
        print_function_text(g, m, u.data(), nullptr, nullptr, nullptr, false);
        print_function_text(g, m, u.data(), nullptr, nullptr, nullptr, true);
        fclose(g);
    }
    if (!bad) printf("host code clean at levels 1-4\n");
    return bad ? 1 : 0;
}
