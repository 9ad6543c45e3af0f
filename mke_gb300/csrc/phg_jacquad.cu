// phg_jacquad.cu -- element-loop Gauss quadrature for the right-hand sides of
// the spherical Jacobian (FP32, the mixed-precision time steps).
//
// SphereJacobian::calc2 (src/sjacobian.cpp:136-362) needs, for two fields f =
// u, v, the products D1 f, D2 f, D1cos f, D2cos f of four derivative matrices
// with entries (src/sjacobian.cpp:76-134, src/generators.cpp:57-104)
//     D1_ij    = sum_T int_T dphi_j/dx phi_i,     D1cos_ij = ... cos(x) ...,
//     D2_ij    = sum_T int_T dphi_j/dy phi_i,     D2cos_ij = ... cos(x) ...,
// over the triangles T at row point i, in the chart (x, y) of the row point's
// first triangle, each integral by the 7-point degree-5 rule.  For P1
// elements dphi_j/dx is constant on T, so a row's products are
//     (D1 f)_i = sum_{T at i} (df_T/dx) int_T phi_i,  (D1cos f)_i = ... int_T phi_i cos x,
// with df_T/dx the x-derivative of the linear interpolant of f on T.  This
// kernel evaluates exactly that from the mesh geometry, with no assembled
// matrix: per (row, triangle) the chart coordinates of the triangle's other
// two vertices relative to the row point, from which it forms the interpolant
// gradient weights, the area and the 7-point rule of int phi_i cos(x).
//
// Mapping: 8 lanes per row (lane = triangle slot; at most 6 triangles meet at a
// point of an icosahedral mesh, lanes 6-7 carry zeros), 4 rows per warp.  The
// quadrature is done once per row and kept in registers; the member loop then
// gathers the two fields at the triangle's vertices (FP64 differences, then
// FP32), forms the 8 per-triangle contributions and sums them over the row's
// lanes with a 3-stage butterfly of warp shuffles that leaves lane k holding
// right-hand side k (7 shuffles per lane instead of 24 for 8 separate
// reductions).  Lane k adds the row's boundary-column product of RHS k (the
// reference integrates those in the boundary point's chart,
// src/generators.cpp:142-178, so they stay assembled, FP64) and writes RHS k.
// A boundary vertex of T contributes 0 to the interpolant (the inner matrix
// has no boundary column).  Members are split over grid.y in chunks of
// MCHUNK, so one launch reads the geometry once per MCHUNK members.
//
// RHS order k: 0 D2c u, 1 D1 v, 2 D1c u, 3 D2 v, 4 D2 u, 5 D1c v, 6 D1 u,
// 7 D2c v (the order of k_jac_rhs), out[(v * 8 + k) * ldo + i].
#include <climits>
#include <cmath>
#include <vector>

#include "phg_host.hpp"
#include "phg_kernels.cuh"
#include "phg_jacquad.cuh"

namespace phg {

namespace {

constexpr int MCHUNK = 16;      // members per block (grid.y splits the rest)
constexpr int ROWS_PER_BLOCK = 32;

// The 7-point degree-5 rule on a triangle (Radon's formula): barycentric
// nodes (1/3, 1/3, 1/3) with weight 9/40, and the three permutations of
// (a, a, 1 - 2a) for a = (6 -+ sqrt 15) / 21 with weights (155 -+ sqrt 15) / 1200;
// the weights sum to 1 (the rule returns area x weighted sum).
constexpr double S15 = 3.8729833462074168852;
constexpr double A1 = (6.0 - S15) / 21.0, A2 = (6.0 + S15) / 21.0;
constexpr double W0 = 9.0 / 40.0, W1 = (155.0 - S15) / 1200.0, W2 = (155.0 + S15) / 1200.0;

__device__ __forceinline__ void rule_node(int q, float &l0, float &la, float &lb, float &w) {
    // node q: barycentric coordinates of (row vertex, vertex a, vertex b)
    const float a1 = (float)A1, b1 = (float)(1.0 - 2.0 * A1), a2 = (float)A2, b2 = (float)(1.0 - 2.0 * A2);
    switch (q) {
    case 0: l0 = la = lb = (float)(1.0 / 3.0); w = (float)W0; break;
    case 1: l0 = b1; la = a1; lb = a1; w = (float)W1; break;
    case 2: l0 = a1; la = b1; lb = a1; w = (float)W1; break;
    case 3: l0 = a1; la = a1; lb = b1; w = (float)W1; break;
    case 4: l0 = b2; la = a2; lb = a2; w = (float)W2; break;
    case 5: l0 = a2; la = b2; lb = a2; w = (float)W2; break;
    default: l0 = a2; la = a2; lb = b2; w = (float)W2; break;
    }
}

// keep the half of 2H values whose index bit is `hi`, add the partner's copy
template <int H>
__device__ __forceinline__ void fold(float (&s)[8], int hi, int off) {
#pragma unroll
    for (int j = 0; j < H; ++j) {
        const float keep = hi ? s[H + j] : s[j];
        const float give = hi ? s[j] : s[H + j];
        s[j] = keep + __shfl_xor_sync(0xffffffffu, give, off);
    }
}

__global__ void __launch_bounds__(256) k_jac_quad(JacQuadDev G, JacOps J, const double *__restrict__ u,
                                                  const double *__restrict__ w, int ld, const int *__restrict__ imap,
                                                  const int *__restrict__ bmap, double *__restrict__ out, int ldo,
                                                  int nv) {
    const int slot = threadIdx.x & 7;
    const int n = G.n;
    const int v0 = blockIdx.y * MCHUNK, v1 = min(nv, v0 + MCHUNK);
    // this lane's boundary-column operator and field (RHS k = slot)
    const int opk = (slot == 0 || slot == 7) ? 3 : (slot == 1 || slot == 6) ? 0 : (slot == 2 || slot == 5) ? 2 : 1;
    const int *cptr = opk == 0 ? J.d1b.ptr : opk == 1 ? J.d2b.ptr : opk == 2 ? J.d1cb.ptr : J.d2cb.ptr;
    const int *ccol = opk == 0 ? J.d1b.col : opk == 1 ? J.d2b.col : opk == 2 ? J.d1cb.col : J.d2cb.col;
    const double *cval = opk == 0 ? J.d1b.val : opk == 1 ? J.d2b.val : opk == 2 ? J.d1cb.val : J.d2cb.val;
    const bool on_u = (slot & 1) == 0;
    for (int i0 = blockIdx.x * ROWS_PER_BLOCK; i0 < n; i0 += gridDim.x * ROWS_PER_BLOCK) {
        const int i = i0 + (threadIdx.x >> 3);
        const bool row = i < n;
        // quadrature of this lane's triangle (once per row)
        float ca = 0.f, cb = 0.f, ea = 0.f, eb = 0.f, m = 0.f, mc = 0.f;
        int pa = INT_MIN, pb = INT_MIN;
        if (row && slot < 6) {
            const int2 id = G.idx[(size_t)i * 8 + slot];
            if (id.x != INT_MIN) {
                const float4 g = G.geo[(size_t)i * 8 + slot];   // (xa, ya, xb, yb) - (x0, y0)
                const float D = g.x * g.w - g.z * g.y;           // twice the signed area
                const float iD = 1.0f / D;
                // grad f = (ca (fa - f0) + cb (fb - f0), ea (fa - f0) + eb (fb - f0))
                ca = g.w * iD; cb = -g.y * iD; ea = -g.z * iD; eb = g.x * iD;
                const float area = 0.5f * fabsf(D);
                m = area * (1.0f / 3.0f);                        // int_T phi_i (the rule is exact)
                const float2 cs = G.cs0[i];                      // cos x0, sin x0
                float acc = 0.f;
#pragma unroll
                for (int q = 0; q < 7; ++q) {
                    float l0, la, lb, wq;
                    rule_node(q, l0, la, lb, wq);
                    float sd, cd;
                    sincosf(la * g.x + lb * g.z, &sd, &cd);     // x - x0 at the node (small)
                    acc += wq * l0 * (cs.x * cd - cs.y * sd);   // phi_i cos(x) at the node
                }
                mc = area * acc;                                 // int_T phi_i cos(x)
                pa = id.x; pb = id.y;
            }
        }
        const int p = row ? imap[i] : 0;
        const int kb0 = (row && cptr) ? cptr[i] : 0, kb1 = (row && cptr) ? cptr[i + 1] : 0;
        for (int v = v0; v < v1; ++v) {
            const double *fu = u + (size_t)v * ld, *fw = w + (size_t)v * ld;
            float s[8];
            if (pa != INT_MIN) {
                const double u0 = fu[p], w0 = fw[p];
                const double ua = pa >= 0 ? fu[pa] : 0.0, ub = pb >= 0 ? fu[pb] : 0.0;
                const double wa = pa >= 0 ? fw[pa] : 0.0, wb = pb >= 0 ? fw[pb] : 0.0;
                const float dua = (float)(ua - u0), dub = (float)(ub - u0);
                const float dwa = (float)(wa - w0), dwb = (float)(wb - w0);
                const float ux = ca * dua + cb * dub, uy = ea * dua + eb * dub;
                const float wx = ca * dwa + cb * dwb, wy = ea * dwa + eb * dwb;
                s[0] = uy * mc; s[1] = wx * m; s[2] = ux * mc; s[3] = wy * m;
                s[4] = uy * m; s[5] = wx * mc; s[6] = ux * m; s[7] = wy * mc;
            } else {
#pragma unroll
                for (int k = 0; k < 8; ++k) s[k] = 0.f;
            }
            // butterfly over the row's 8 lanes: lane `slot` ends with RHS `slot`
            fold<4>(s, (slot >> 2) & 1, 4);
            fold<2>(s, (slot >> 1) & 1, 2);
            fold<1>(s, slot & 1, 1);
            if (row) {
                double b = 0.0;
                const double *fb = on_u ? fu : fw;
                for (int k = kb0; k < kb1; ++k) {
                    const int c = ccol[k];
                    b += cval[k] * fb[bmap ? bmap[c] : c];
                }
                out[((size_t)v * 8 + slot) * ldo + i] = b + (double)s[0];
            }
        }
    }
}

}  // namespace

void build_jac_quad(const Mesh &m, JacQuadHost &h) {
    const int rs = m.rs;
    h.max_tri = 0;
    h.idx.assign((size_t)rs * 8 * 2, INT_MIN);
    h.geo.assign((size_t)rs * 8 * 4, 0.f);
    h.cs0.assign((size_t)rs * 2, 0.f);
    for (int i = 0; i < rs; ++i) {
        const int p = m.inner[i];
        const int z = m.row_zone(p);
        const double x0 = m.u(p, z), y0 = m.v(p, z);
        h.cs0[2 * i] = (float)std::cos(x0);
        h.cs0[2 * i + 1] = (float)std::sin(x0);
        int k = 0;
        h.max_tri = std::max(h.max_tri, m.adj_ptr[p + 1] - m.adj_ptr[p]);
        for (int q = m.adj_ptr[p]; q < m.adj_ptr[p + 1] && k < 6; ++q, ++k) {
            const int t = m.adj[q];
            int other[2], no = 0;
            for (int c = 0; c < 3; ++c)
                if (m.tri[3 * t + c] != p && no < 2) other[no++] = m.tri[3 * t + c];
            const size_t e = (size_t)i * 8 + k;
            for (int c = 0; c < 2; ++c)
                h.idx[2 * e + c] = m.bnd[other[c]] ? -1 : other[c];
            h.geo[4 * e + 0] = (float)(m.u(other[0], z) - x0);
            h.geo[4 * e + 1] = (float)(m.v(other[0], z) - y0);
            h.geo[4 * e + 2] = (float)(m.u(other[1], z) - x0);
            h.geo[4 * e + 3] = (float)(m.v(other[1], z) - y0);
        }
    }
}

size_t jac_quad_bytes(int rs, int V, int nv) {
    // per row: 6 triangles x (2 indices + 4 coordinates) + cos/sin of the row
    // point; both fields read once per member; 8 FP64 right-hand sides written
    return (size_t)rs * (6 * 24 + 8) + (size_t)nv * (2 * (size_t)V * 8 + 8 * (size_t)rs * 8);
}

cudaError_t jac_quad(const JacQuadDev &G, const JacOps &J, const double *u, const double *v, int ld, const int *imap,
                     const int *bmap, double *out, int ldo, int nv, cudaStream_t s) {
    if (G.n <= 0 || nv <= 0) return cudaSuccess;
    const int rowblocks = (G.n + ROWS_PER_BLOCK - 1) / ROWS_PER_BLOCK;
    const int chunks = (nv + MCHUNK - 1) / MCHUNK;
    if (chunks > 65535) return cudaErrorInvalidValue;
    dim3 grid(rowblocks, chunks);
    k_jac_quad<<<grid, 256, 0, s>>>(G, J, u, v, ld, imap, bmap, out, ldo, nv);
    g_kernel_launches++;
    return cudaGetLastError();
}

}  // namespace phg
