// phg_host.hpp -- host-side data of the GB300 sphere-FEM library: the mesh
// and the assembled sparse operators (built once per mesh on the CPU, then
// uploaded to HBM).
#pragma once
#include <cstdio>
#include <string>
#include <vector>

namespace phg {

// An icosahedral sphere mesh exactly as the reference's Mesh::load sees it
// (src/mesh.h:354-427): points with up to 4 per-zone (u, v) charts,
// triangles with a 0-based zone, boundary flags and the inner/outer maps.
struct Mesh {
    int level = -1;            // subdivision level when generated, -1 if loaded
    int V = 0, T = 0;          // points, triangles
    int rs = 0, os = 0;        // inner / outer (boundary) counts
    int nz = 4;                // charts per point
    std::vector<double> xyz;   // V x 3
    std::vector<double> uv;    // V x 4 x 2 (missing charts are NaN)
    std::vector<int> tri;      // T x 3
    std::vector<int> tz;       // T
    std::vector<int> bnd;      // V (1 = boundary)
    std::vector<int> inner, outer, p2io;
    std::vector<int> adj_ptr, adj;  // point -> triangles, ascending triangle id
    // generated meshes only: refinement history for multigrid
    std::vector<int> orig;          // point -> index before the Cuthill-McKee reorder
    std::vector<int> par_a, par_b;  // pre-reorder index -> endpoints (pre-reorder, level-1
                                    // numbering) of the coarse edge it bisects; -1 for coarse points
    std::vector<double> raw_xyz;    // point coordinates before the text round trip

    double u(int p, int z) const { return uv[8 * (size_t)p + 2 * z]; }
    double v(int p, int z) const { return uv[8 * (size_t)p + 2 * z + 1]; }
    int row_zone(int p) const { return tz[adj[adj_ptr[p]]]; }
};

// Icosahedron refined `level` times on the unit sphere, south pole as the
// single boundary point, Cuthill-McKee order, charts rounded through the
// 16-decimal text format -- identical to "mke_mesh_sphere --type full
// --coord local --iter level" followed by Mesh::load.
bool generate_sphere(int level, Mesh &m, std::string &err);
// Parse the reference's mesh text format (src/mesh.cpp:323-519).
bool load_mesh_text(FILE *f, Mesh &m, std::string &err);
// The reference's mesh text (utils/icosahedron.cpp:268-457, full sphere with
// local charts).  Generated meshes print their coordinates before the text
// round trip, so the file equals mke_mesh_sphere's byte for byte; loaded
// meshes print the parsed values.
bool save_mesh_text(FILE *f, const Mesh &m);
// print_function / print_inner_function (src/phelm.cpp:160-321); x, y, z:
// values at every point replacing the zone-0 (u, v, 0), or null
void print_function_text(FILE *f, const Mesh &m, const double *ans, const double *x, const double *y,
                         const double *z, bool inner_only);
// Finish a mesh whose points/triangles/boundary flags are filled in:
// inner/outer/p2io in point order and the point->triangle adjacency.
void finish_mesh(Mesh &m);

struct Csr {
    int n = 0, m = 0;
    std::vector<int> ptr, col;
    std::vector<double> val;
    int nnz() const { return ptr.empty() ? 0 : ptr[n]; }
};

// Accumulates add(i, j, a) in call order per entry, then sorts each row.
class CsrBuilder {
public:
    CsrBuilder(int n, int m);
    void add(int i, int j, double a);
    void finish(Csr &out);
private:
    int n_, m_;
    std::vector<std::vector<std::pair<int, double>>> rows_;
};

// Every operator the sphere path needs, assembled on the host.
struct SphereOps {
    // rs x rs, one shared sparsity pattern
    Csr idt;    // SphereLaplace mass, int cos(u) phi_i phi_j
    Csr lapl;   // SphereLaplace Laplacian (slaplace form)
    Csr jidt;   // SphereJacobian mass (7-point cubature)
    Csr d1, d2, d1c, d2c;  // derivative matrices (plain / cos-weighted)
    // rs x os boundary columns
    Csr bnd2, bnd3, d1b, d2b, d1cb, d2cb;
    // V x V norm matrix
    Csr norm;
};

void assemble_sphere(const Mesh &m, SphereOps &ops);
// only the Laplacian (slaplace form), rs x rs
void assemble_laplacian(const Mesh &m, Csr &lapl);

// Geometric multigrid hierarchy over the nested icosahedral meshes: level 0
// is the mesh itself, level k+1 the mesh one refinement coarser.  P[k] maps
// level k+1 inner values to level k inner points (1 at coincident points,
// 1/2 at both ends of the bisected edge; boundary columns dropped) and R[k]
// = P[k]^T; A[k] is the Laplacian re-assembled on level k (A[0] unused).
struct MgHierarchy {
    std::vector<Mesh> mesh;        // mesh[0] unused (the caller's mesh)
    std::vector<Csr> A, P, R;
    std::vector<double> coarse_inv;  // dense inverse of the coarsest A (row-major)
};
bool build_mg(const Mesh &fine, int coarsest_level, MgHierarchy &h, std::string &err);
// BarVortex forward matrix c1 * mass + c2 * slaplace (examples/barvortex_impl.h:57-78)
void assemble_barvortex(const Mesh &m, double c1, double c2, Csr &A, Csr &Abnd);
// Baroclin 4rs x 4rs block matrix (examples/baroclin.cpp:119-180) and the
// per-boundary-point columns its right-hand side uses, integrated in the row
// point's chart (examples/baroclin.cpp:245-339): bcol[q] is rs x os for the
// row block q = 0..3 and carries the summed coefficient of bnd[j].
// backward: the entries of Ab_, the matrix of the inverse linearised step
// (examples/baroclin.cpp:182-243) instead of A_ (:119-180)
struct BaroclinParams { double tau, sigma, mu, sigma1, mu1, alpha, theta; bool backward = false; };
void assemble_baroclin(const Mesh &m, const BaroclinParams &p, Csr &A, Csr bcol[4]);

// On-disk cache of a generated level (phg_cache.cpp): the mesh, the operators
// and, when built, the multigrid hierarchy, stored byte for byte.  load
// rejects files of another format or level, truncated files and checksum
// mismatches (err says why).
bool save_level_cache(const char *path, const Mesh &m, const SphereOps &ops, const MgHierarchy *mg);
bool load_level_cache(const char *path, int level, Mesh &m, SphereOps &ops, MgHierarchy &mg, bool &has_mg,
                      std::string &err);

}  // namespace phg
