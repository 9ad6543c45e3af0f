// phg_jacquad.cuh -- element-loop quadrature of the Jacobian right-hand sides
// (phg_jacquad.cu): geometry layout and launcher.
#pragma once
#include <vector>

#include "phg_kernels.cuh"

namespace phg {

struct Mesh;

// Per inner row i, the ring of points around it in order (k < 8, at most 6
// used), row-major [i * 8 + k] so that the 8 lanes of a row read consecutive
// words; triangle k of the row is (row point, ring[k], ring[k + 1 mod deg]):
//   ring: point index (full vectors) of ring vertex k, -1 for the boundary
//         point (its value does not enter: the inner matrices have no
//         boundary column), INT_MIN for an unused slot;
//   rxy:  its chart coordinates minus the row point's, in the chart of the
//         row point's first triangle, rounded from FP64;
//   cs0:  cos and sin of the row point's chart x.
struct JacQuadDev {
    int n = 0;
    const int *ring = nullptr;
    const float2 *rxy = nullptr;
    const float2 *cs0 = nullptr;
};

struct JacQuadHost {
    std::vector<int> ring;    // rs x 8
    std::vector<float> rxy;   // rs x 8 x 2
    std::vector<float> cs0;   // rs x 2
    int max_tri = 0;          // most triangles at one inner point (> 6: the kernel does not apply)
};

void build_jac_quad(const Mesh &m, JacQuadHost &h);
// algorithmic bytes of one call (split pass and quadrature) for nv members
size_t jac_quad_bytes(int rs, int V, int nv);
// the 8 right-hand sides of SphereJacobian::calc2 for nv members (member-major
// u, v with leading dimension ld; out[(v * 8 + k) * ldo + i]), FP32 element
// loop; J supplies the boundary columns (FP64); split: scratch for both
// fields as float pairs, 2 x nv x V float2
cudaError_t jac_quad(const JacQuadDev &G, const JacOps &J, const double *u, const double *v, int ld, const int *imap,
                     const int *bmap, double *out, int ldo, int nv, int V, float2 *split, cudaStream_t s);

}  // namespace phg
