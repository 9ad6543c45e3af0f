/* Runs the CPU oracle (oracle/orc_*.c) under AddressSanitizer and
 * UndefinedBehaviorSanitizer: mesh, operators, a Laplace solve, a Jacobian,
 * one barotropic step with its linearised / inverse / adjoint steps and one
 * baroclinic step with its linearised steps, at levels 2 and 3.  Built and
 * run by tests/test_sanitizers.py. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "phelm_oracle.h"

static int finite_all(const double *a, int n) {
    for (int i = 0; i < n; ++i)
        if (!isfinite(a[i])) return 0;
    return 1;
}

int main(void) {
    int bad = 0;
    orc_set_solver(1e-12, 30, 20000);
    for (int level = 2; level <= 3; ++level) {
        orc_mesh m;
        if (orc_mesh_sphere(&m, level)) { fprintf(stderr, "mesh %d\n", level); return 1; }
        orc_ops o;
        if (orc_ops_build(&o, &m)) { fprintf(stderr, "ops %d\n", level); return 1; }
        const int V = m.V;
        double *u = calloc(V, sizeof(double)), *v = calloc(V, sizeof(double)), *w = calloc(V, sizeof(double));
        double *z = calloc(V, sizeof(double)), *lh = calloc(V, sizeof(double)), *ans = calloc(V, sizeof(double));
        double *u2 = calloc(V, sizeof(double)), *a1 = calloc(V, sizeof(double)), *a2 = calloc(V, sizeof(double));
        double bnd[4] = {0.0, 0.0, 0.0, 0.0};
        for (int i = 0; i < V; ++i) {
            const double x = m.xyz[3 * i], y = m.xyz[3 * i + 1], zz = m.xyz[3 * i + 2];
            u[i] = 0.1 * x * y + 0.05 * zz * zz;
            v[i] = 0.2 * y - 0.1 * x * zz;
            z[i] = 0.05 * x;
            u2[i] = 0.03 * y * zz;
            lh[i] = zz;
        }
        orc_laplace_solve(&o, ans, u, bnd);
        bad += !finite_all(ans, V);
        orc_jacobian_calc2(&o, w, u, v);
        bad += !finite_all(w, m.rs);
        bad += !isfinite(orc_norm(&o, u)) || !isfinite(orc_dist(&o, u, v));
        orc_bv_conf bc = {1e-3, 1.6e-2, 8e-5, 1.0, 1.0, 0.5, 3};
        orc_barvortex bv;
        if (orc_bv_init(&bv, &o, &bc, lh)) { fprintf(stderr, "bv %d\n", level); return 1; }
        orc_bv_step(&bv, ans, u, bnd, bnd, NULL);
        bad += !finite_all(ans, V);
        orc_bv_calc_L(&bv, a1, v, z, bnd, bnd);
        orc_bv_calc_L1(&bv, a2, v, z, bnd, bnd);
        orc_bv_calc_LT(&bv, ans, v, z, bnd, bnd);
        bad += !finite_all(a1, V) || !finite_all(a2, V) || !finite_all(ans, V);
        orc_bv_free(&bv);
        orc_bc_conf cc = {1e-3, 0.05, 6.77e-5, 0.05, 6.77e-5, sqrt(0.1), 0.5, 3, 1e-8};
        orc_baroclin b;
        if (orc_bc_init(&b, &o, &cc, lh)) { fprintf(stderr, "bc %d\n", level); return 1; }
        orc_bc_step(&b, a1, a2, u, u2, bnd, NULL, NULL);
        bad += !finite_all(a1, V) || !finite_all(a2, V);
        orc_bc_calc_L(&b, a1, a2, u, u2, z, v, bnd);
        bad += !finite_all(a1, V) || !finite_all(a2, V);
        for (int i = 0; i < V; ++i) a1[i] = a2[i] = 0.0;
        orc_bc_calc_L1(&b, a1, a2, u, u2, z, v, bnd);
        bad += !finite_all(a1, V) || !finite_all(a2, V);
        orc_bc_free(&b);
        free(u); free(v); free(w); free(z); free(lh); free(ans); free(u2); free(a1); free(a2);
        orc_ops_free(&o);
        orc_mesh_free(&m);
    }
    if (!bad) printf("oracle clean at levels 2-3\n");
    return bad ? 1 : 0;
}
