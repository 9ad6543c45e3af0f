/*
 * orc_mesh.c -- oracle restatement of the reference's icosahedral sphere mesh
 * ("mke_mesh_sphere --type full --coord local --iter N" followed by
 * phelm::Mesh::load).  TEST INFRASTRUCTURE ONLY (see phelm_oracle.h).
 *
 * Steps and the reference lines they restate:
 *   icosahedron (12 points, 20 faces)       utils/mesh_builder.cpp:52-113
 *   orthogonal projection to the sphere     utils/mesh_builder.cpp:115-125
 *   midpoint subdivision, edge dedupe       utils/mesh_builder.cpp:143-201
 *   south-pole boundary (|z+1| < 1e-14)     utils/icosahedron.cpp:416-421
 *   Cuthill-McKee order of inner points,
 *   ties by (degree, point id), outer last  utils/mesh_builder.cpp:316-402, 504-585
 *   per-zone (u, v) charts                  utils/icosahedron.cpp:251-266, 327-347
 *   triangle zone rule (incl. the repeated
 *   v2 test in place of v3)                 utils/icosahedron.cpp:380-393
 *   %.16lf text round trip                  utils/icosahedron.cpp:320, src/mesh.cpp:365-402
 *   inner/outer/p2io, adjacency             src/mesh.cpp:301-319, 487-507
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "phelm_oracle.h"

typedef struct { double x, y, z; } pt3;
typedef struct { int a, b, c; } tri3;

static void project(pt3 *p)
{
	double l = sqrt(p->x * p->x + p->y * p->y + p->z * p->z);
	p->x /= l; p->y /= l; p->z /= l;
}

/* midpoint cache: per old point, up to 8 (neighbour, midpoint) pairs */
typedef struct { int n; int nb[8]; int mid[8]; } edge_cache;

static int cache_find(const edge_cache *c, int nb)
{
	for (int k = 0; k < c->n; ++k) if (c->nb[k] == nb) return c->mid[k];
	return -1;
}

static void cache_put(edge_cache *c, int nb, int mid)
{
	c->nb[c->n] = nb; c->mid[c->n] = mid; c->n++;
}

static int midpoint(pt3 *pts, int *np, edge_cache *ec, int v1, int v2)
{
	int m = cache_find(&ec[v1], v2);
	if (m >= 0) return m;
	pt3 a = pts[v1], b = pts[v2];
	pt3 p = { (a.x + b.x) / 2, (a.y + b.y) / 2, (a.z + b.z) / 2 };
	project(&p);
	m = (*np)++;
	pts[m] = p;
	cache_put(&ec[v1], v2, m);
	cache_put(&ec[v2], v1, m);
	return m;
}

static double chart_u(double x, double y, double z) { (void)x; (void)y; return asin(z); }

static double chart_v(double x, double y, double z)
{
	(void)z;
	double r = sqrt(x * x + y * y);
	if (r < 1e-15) return 0.0;
	double v1 = acos(x / r);
	if (y < 0) v1 = 2.0 * M_PI - v1;
	return v1;
}

/* the value a reader gets back after "%.16lf" */
static double round16(double v)
{
	char buf[64];
	snprintf(buf, sizeof(buf), "%.16lf", v);
	return strtod(buf, NULL);
}

static int cmp_int(const void *a, const void *b)
{
	int x = *(const int *)a, y = *(const int *)b;
	return (x > y) - (x < y);
}

int orc_mesh_sphere(orc_mesh *m, int level)
{
	double t = (1.0 + sqrt(5.0)) / 2.0;
	const double ico[12][3] = {
		{ t, 1.0, 0.0 }, { -t, 1.0, 0.0 }, { t, -1.0, 0.0 },
		{ -t, -1.0, 0.0 }, { 1.0, 0.0, t }, { 1.0, 0.0, -t },
		{ -1.0, 0.0, t }, { -1.0, 0.0, -t }, { 0.0, t, 1.0 },
		{ 0.0, -t, 1.0 }, { 0.0, t, -1.0 }, { 0.0, -t, -1.0 },
	};
	const int faces[20][3] = {
		{ 0, 8, 4 }, { 1, 10, 7 }, { 2, 9, 11 }, { 7, 3, 1 },
		{ 0, 5, 10 }, { 3, 9, 6 }, { 3, 11, 9 }, { 8, 6, 4 },
		{ 2, 4, 9 }, { 3, 7, 11 }, { 4, 2, 0 }, { 9, 4, 6 },
		{ 2, 11, 5 }, { 0, 10, 8 }, { 5, 0, 2 }, { 10, 5, 7 },
		{ 1, 6, 8 }, { 1, 8, 10 }, { 6, 1, 3 }, { 11, 7, 5 },
	};
	if (level < 0 || level > 10) return -1;
	memset(m, 0, sizeof(*m));
	int V = 10 * (1 << (2 * level)) + 2, T = 20 * (1 << (2 * level));
	pt3 *pts = (pt3 *)malloc(sizeof(pt3) * (size_t)V);
	tri3 *tr = (tri3 *)malloc(sizeof(tri3) * (size_t)T);
	tri3 *tr2 = (tri3 *)malloc(sizeof(tri3) * (size_t)T);
	int np = 12, nt = 20;
	for (int i = 0; i < 12; ++i) { pts[i].x = ico[i][0]; pts[i].y = ico[i][1]; pts[i].z = ico[i][2]; project(&pts[i]); }
	for (int i = 0; i < 20; ++i) { tr[i].a = faces[i][0]; tr[i].b = faces[i][1]; tr[i].c = faces[i][2]; }

	for (int it = 0; it < level; ++it) {
		edge_cache *ec = (edge_cache *)calloc((size_t)np, sizeof(edge_cache));
		int nt2 = 0;
		for (int k = 0; k < nt; ++k) {
			int v1 = tr[k].a, v2 = tr[k].b, v3 = tr[k].c;
			int p1 = midpoint(pts, &np, ec, v1, v2);
			int p2 = midpoint(pts, &np, ec, v1, v3);
			int p3 = midpoint(pts, &np, ec, v2, v3);
			tr2[nt2].a = v1; tr2[nt2].b = p1; tr2[nt2].c = p2; nt2++;
			tr2[nt2].a = v3; tr2[nt2].b = p2; tr2[nt2].c = p3; nt2++;
			tr2[nt2].a = v2; tr2[nt2].b = p3; tr2[nt2].c = p1; nt2++;
			tr2[nt2].a = p1; tr2[nt2].b = p2; tr2[nt2].c = p3; nt2++;
		}
		free(ec);
		tri3 *s = tr; tr = tr2; tr2 = s; nt = nt2;
	}

	/* boundary before reordering: the south pole */
	int *flag = (int *)calloc((size_t)np, sizeof(int));
	for (int i = 0; i < np; ++i) if (fabs(pts[i].z + 1.0) < 1e-14) flag[i] = 1;

	/* inner numbering in point order, graph of inner points (with self) */
	int *p2io = (int *)malloc(sizeof(int) * (size_t)np);
	int rs = 0, os = 0;
	for (int i = 0; i < np; ++i) p2io[i] = flag[i] ? os++ : rs++;
	int *inner = (int *)malloc(sizeof(int) * (size_t)(rs ? rs : 1));
	for (int i = 0, k = 0; i < np; ++i) if (!flag[i]) inner[k++] = i;

	/* neighbour sets: every inner vertex of every triangle through the point */
	int cap = 16;
	int *nbn = (int *)calloc((size_t)rs, sizeof(int));
	int *nb = (int *)malloc(sizeof(int) * (size_t)rs * (size_t)cap);
	for (int k = 0; k < nt; ++k) {
		int vv[3] = { tr[k].a, tr[k].b, tr[k].c };
		for (int q = 0; q < 3; ++q) {
			if (flag[vv[q]]) continue;
			int i = p2io[vv[q]];
			for (int r = 0; r < 3; ++r) {
				if (flag[vv[r]]) continue;
				int j = p2io[vv[r]], seen = 0;
				for (int s = 0; s < nbn[i]; ++s) if (nb[i * cap + s] == j) { seen = 1; break; }
				if (!seen) nb[i * cap + nbn[i]++] = j;
			}
		}
	}
	for (int i = 0; i < rs; ++i) qsort(nb + i * cap, (size_t)nbn[i], sizeof(int), cmp_int);
	/* neighbours ordered by (degree, id): stable sort of the ascending set */
	int *srt = (int *)malloc(sizeof(int) * (size_t)rs * (size_t)cap);
	for (int i = 0; i < rs; ++i) {
		int n = nbn[i], *o = srt + i * cap;
		memcpy(o, nb + i * cap, sizeof(int) * (size_t)n);
		for (int a = 1; a < n; ++a) {
			int x = o[a], q = a - 1;
			while (q >= 0 && nbn[o[q]] > nbn[x]) { o[q + 1] = o[q]; --q; }
			o[q + 1] = x;
		}
	}
	/* breadth-first numbering with a queue that may hold repeats */
	int *order = (int *)malloc(sizeof(int) * (size_t)(rs ? rs : 1));
	for (int i = 0; i < rs; ++i) order[i] = -1;
	int qcap = rs * cap + 16;
	int *queue = (int *)malloc(sizeof(int) * (size_t)qcap);
	int knum = 0;
	for (int start = 0; start < rs; ++start) {
		if (order[start] != -1) continue;
		int qh = 0, qt = 0;
		queue[qt++] = start;
		while (qh < qt) {
			int v = queue[qh++];
			if (order[v] != -1) continue;
			order[v] = knum++;
			int n = nbn[v], *o = srt + v * cap;
			for (int a = 0; a < n; ++a)
				if (order[o[a]] < 0) queue[qt++] = o[a];
		}
	}
	/* full order: inner points by CM order, outer points after them */
	int *full = (int *)malloc(sizeof(int) * (size_t)np);
	for (int i = 0, ob = rs; i < np; ++i) full[i] = flag[i] ? ob++ : order[p2io[i]];
	pt3 *pn = (pt3 *)malloc(sizeof(pt3) * (size_t)np);
	for (int i = 0; i < np; ++i) pn[full[i]] = pts[i];
	for (int k = 0; k < nt; ++k) { tr[k].a = full[tr[k].a]; tr[k].b = full[tr[k].b]; tr[k].c = full[tr[k].c]; }

	/* output as loaded */
	m->V = np; m->T = nt; m->nz = 4;
	m->xyz = (double *)malloc(sizeof(double) * 3 * (size_t)np);
	m->uv = (double *)malloc(sizeof(double) * 8 * (size_t)np);
	m->tri = (int *)malloc(sizeof(int) * 3 * (size_t)nt);
	m->tz = (int *)malloc(sizeof(int) * (size_t)nt);
	m->bnd = (int *)calloc((size_t)np, sizeof(int));
	for (int i = 0; i < np; ++i) {
		double x = pn[i].x, y = pn[i].y, z = pn[i].z;
		double *c = m->uv + 8 * (size_t)i;
		m->xyz[3 * i] = round16(x); m->xyz[3 * i + 1] = round16(y); m->xyz[3 * i + 2] = round16(z);
		c[0] = round16(chart_u(x, y, z));   c[1] = round16(chart_v(x, y, z));
		c[2] = round16(chart_u(-x, -y, z)); c[3] = round16(chart_v(-x, -y, z));
		c[4] = round16(chart_u(x, -z, y)); c[5] = round16(chart_v(x, -z, y));
		c[6] = round16(chart_u(x, z, -y)); c[7] = round16(chart_v(x, z, -y));
		if (fabs(z + 1.0) < 1e-14) m->bnd[i] = 1;
	}
	for (int k = 0; k < nt; ++k) {
		int a = tr[k].a, b = tr[k].b, c = tr[k].c;
		m->tri[3 * k] = a; m->tri[3 * k + 1] = b; m->tri[3 * k + 2] = c;
		double z1 = pn[a].z, z2 = pn[b].z, z3 = pn[c].z;
		double v1 = chart_v(pn[a].x, pn[a].y, z1);
		double v2 = chart_v(pn[b].x, pn[b].y, z2);
		int zone = 1;
		if (z1 > 0.9 || z2 > 0.9 || z3 > 0.9) zone = 4;
		else if (z1 < -0.9 || z2 < -0.9 || z3 < -0.9) zone = 3;
		else if (v1 < M_PI_2 || v2 < M_PI_2 || v2 < M_PI_2 ||
		         v1 > 1.5 * M_PI || v2 > 1.5 * M_PI || v2 > 1.5 * M_PI) zone = 2;
		m->tz[k] = zone - 1;
	}
	/* Mesh::load: inner/outer/p2io in file order, adjacency by triangle id */
	m->p2io = (int *)malloc(sizeof(int) * (size_t)np);
	m->rs = 0; m->os = 0;
	for (int i = 0; i < np; ++i) { if (m->bnd[i]) m->os++; else m->rs++; }
	m->inner = (int *)malloc(sizeof(int) * (size_t)(m->rs ? m->rs : 1));
	m->outer = (int *)malloc(sizeof(int) * (size_t)(m->os ? m->os : 1));
	for (int i = 0, a = 0, b = 0; i < np; ++i) {
		if (m->bnd[i]) { m->p2io[i] = b; m->outer[b++] = i; }
		else { m->p2io[i] = a; m->inner[a++] = i; }
	}
	m->adj_ptr = (int *)calloc((size_t)np + 1, sizeof(int));
	m->adj = (int *)malloc(sizeof(int) * 3 * (size_t)nt);
	for (int k = 0; k < 3 * nt; ++k) m->adj_ptr[m->tri[k] + 1]++;
	for (int i = 0; i < np; ++i) m->adj_ptr[i + 1] += m->adj_ptr[i];
	int *fill = (int *)malloc(sizeof(int) * (size_t)np);
	memcpy(fill, m->adj_ptr, sizeof(int) * (size_t)np);
	for (int k = 0; k < nt; ++k)
		for (int q = 0; q < 3; ++q) { int p = m->tri[3 * k + q]; m->adj[fill[p]++] = k; }

	free(fill); free(pn); free(full); free(queue); free(order); free(srt); free(nb); free(nbn);
	free(inner); free(p2io); free(flag); free(tr); free(tr2); free(pts);
	return 0;
}

void orc_mesh_free(orc_mesh *m)
{
	free(m->xyz); free(m->uv); free(m->tri); free(m->tz); free(m->bnd);
	free(m->inner); free(m->outer); free(m->p2io); free(m->adj_ptr); free(m->adj);
	memset(m, 0, sizeof(*m));
}
