// phg_jacquad.cuh -- element-loop quadrature of the Jacobian right-hand sides
// (phg_jacquad.cu): geometry layout and launcher.
#pragma once
#include <vector>

#include "phg_kernels.cuh"

namespace phg {

struct Mesh;

// Per inner row i and triangle slot k < 8 (at most 6 used), row-major
// [i * 8 + k] so that the 8 lanes of a row read consecutive words:
//   idx: point indices (full vectors) of the triangle's two other vertices,
//        -1 for the boundary point (its value does not enter: the inner
//        matrices have no boundary column), INT_MIN in x for an empty slot;
//   geo: their chart coordinates minus the row point's, (xa, ya, xb, yb), in
//        the chart of the row point's first triangle, rounded from FP64;
//   cs0: cos and sin of the row point's chart x.
struct JacQuadDev {
    int n = 0;
    const int2 *idx = nullptr;
    const float4 *geo = nullptr;
    const float2 *cs0 = nullptr;
};

struct JacQuadHost {
    std::vector<int> idx;     // rs x 8 x 2
    std::vector<float> geo;   // rs x 8 x 4
    std::vector<float> cs0;   // rs x 2
    int max_tri = 0;          // most triangles at one inner point (the kernel takes <= 6)
};

void build_jac_quad(const Mesh &m, JacQuadHost &h);
// algorithmic bytes of one launch for nv members
size_t jac_quad_bytes(int rs, int V, int nv);
// the 8 right-hand sides of SphereJacobian::calc2 for nv members (member-major
// u, v with leading dimension ld; out[(v * 8 + k) * ldo + i]), FP32 element
// loop; J supplies the boundary columns (FP64)
cudaError_t jac_quad(const JacQuadDev &G, const JacOps &J, const double *u, const double *v, int ld, const int *imap,
                     const int *bmap, double *out, int ldo, int nv, cudaStream_t s);

}  // namespace phg
