/* orc_internal.h -- helpers shared by the oracle's C files (test infrastructure). */
#ifndef ORC_INTERNAL_H
#define ORC_INTERNAL_H
#include "phelm_oracle.h"

#define ORC_PMAX 8
/* 2-D polynomial sum_{i<=xd, j<=yd} k[i*(yd+1)+j] x^i y^j (src/polynom.h:81-148) */
typedef struct { short xd, yd; double k[16]; } orc_poly;

typedef double (*orc_trap_fn)(int, int, double, double, double, double, double, double);

double orc_poly_apply(const orc_poly *p, double x, double y);
void orc_poly_mul(orc_poly *r, const orc_poly *a, const orc_poly *b);
void orc_poly_diff(orc_poly *r, const orc_poly *p, int d);
void orc_basis1(const orc_mesh *m, int t, int z, orc_poly phi[3]);
void orc_tri_coords(const orc_mesh *m, int t, int z, double xs[3], double ys[3]);
double orc_integrate1(const orc_poly *p, const double xs[3], const double ys[3], orc_trap_fn trapezoid);
double orc_trapezoid_cos(int k, int n, double k1, double b1, double k2, double b2, double x1, double x3);
double orc_trapezoid_sin(int k, int n, double k1, double b1, double k2, double b2, double x1, double x3);
double orc_trapezoid_1_cos(int k, int n, double k1, double b1, double k2, double b2, double x1, double x3);
double orc_integrate_cos(const orc_poly *p, const orc_mesh *m, int t, int z);
double orc_integrate_1_cos(const orc_poly *p, const orc_mesh *m, int t, int z);
double orc_slaplace(const orc_poly *pi, const orc_poly *pj, const orc_mesh *m, int t, int z);
double orc_mass_cos(const orc_poly *pi, const orc_poly *pj, const orc_mesh *m, int t, int z);
int orc_row_zone(const orc_mesh *m, int p);
int orc_tri_pos(const orc_mesh *m, int t, int p);
void orc_gen_bv(orc_csr *A, orc_csr *bndA, const orc_mesh *m, double c1, double c2);

#endif
