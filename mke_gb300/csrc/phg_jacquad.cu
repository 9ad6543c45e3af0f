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
// gathers the two fields at the triangle's vertices, splits each FP64 value
// into two floats with integer instructions (split_f64: no FP64 pipe work in
// the loop) and forms the field differences from them, forms the 8
// per-triangle contributions in FP32 and sums them over the row's
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

// x = hi + lo as two floats (|x - hi - lo| < 2^-46 |x|) by 32-bit integer
// instructions on the two words of x.  GB300 runs FP64 arithmetic, FP64 <->
// FP32 conversions and (by the counters) 64-bit integer work on its narrow
// FP64 pipe: with a DSUB and a conversion per field difference that pipe was
// 85 % busy and bounded this kernel (ncu, level 6 x 32 members).  hi takes the
// top 24 significand bits, lo the next 24; zero gives zeros, magnitudes
// outside [2^-96, 2^128) the hardware conversion.
__device__ __forceinline__ void split_f64(double x, float &hi, float &lo) {
    const unsigned w1 = (unsigned)__double2hiint(x), w0 = (unsigned)__double2loint(x);
    if (((w1 << 1) | w0) == 0u) { hi = lo = 0.f; return; }
    const unsigned sgn = w1 & 0x80000000u;
    const int e = (int)((w1 >> 20) & 0x7ffu) - 1023;
    if (e < -96 || e > 127) { hi = (float)x; lo = 0.f; return; }
    // significand bits 51..29 (hi) and 28..0 (r)
    hi = __uint_as_float(sgn | ((unsigned)(e + 127) << 23) | ((w1 & 0xFFFFFu) << 3) | (w0 >> 29));
    const unsigned r = w0 & 0x1FFFFFFFu;
    if (r == 0u) { lo = 0.f; return; }
    const int msb = 31 - __clz(r);
    const int ex = e - 52 + msb + 127;
    if (ex < 1) { lo = 0.f; return; }
    const unsigned mant = msb <= 23 ? (r << (23 - msb)) & 0x7fffffu : (r >> (msb - 23)) & 0x7fffffu;
    lo = __uint_as_float(sgn | ((unsigned)ex << 23) | mant);
}

// the double of a float by 32-bit integer instructions (exact; subnormal
// floats become zero, infinities and NaN stay so)
__device__ __forceinline__ double widen(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned sgn = u & 0x80000000u;
    if (e == 0u) return __hiloint2double((int)sgn, 0);
    const unsigned E = e == 255u ? 0x7ffu : e + 1023u - 127u;
    const unsigned m = u & 0x7fffffu;
    return __hiloint2double((int)(sgn | (E << 20) | (m >> 3)), (int)(m << 29));
}

// x_a - x_0 from the (hi, lo) splits: the hi difference is exact when the two
// are within a factor 2 (Sterbenz), so the cancellation of nearby values
// loses nothing; otherwise it is one rounding of a difference that did not cancel
__device__ __forceinline__ float diff2(float ah, float al, float zh, float zl) { return (ah - zh) + (al - zl); }

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

// both fields of nv members as (hi, lo) float pairs, member-major with
// leading dimension V (one pass; the quadrature then gathers 8 bytes a value
// and does no conversion work)
__global__ void __launch_bounds__(256) k_split2(const double *__restrict__ u, const double *__restrict__ w, int ld,
                                                int V, long long total, float2 *__restrict__ su,
                                                float2 *__restrict__ sw) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long v = t / V, i = t - v * V;
        float h, l;
        split_f64(u[v * ld + i], h, l);
        su[t] = make_float2(h, l);
        split_f64(w[v * ld + i], h, l);
        sw[t] = make_float2(h, l);
    }
}

__global__ void __launch_bounds__(256) k_jac_quad(JacQuadDev G, JacOps J, const float2 *__restrict__ su,
                                                  const float2 *__restrict__ sw, int V, const double *__restrict__ u,
                                                  const double *__restrict__ w, int ld, const int *__restrict__ imap,
                                                  const int *__restrict__ bmap, double *__restrict__ out, int ldo,
                                                  int nv) {
    const int lane = threadIdx.x & 31, slot = lane & 7, base = lane & ~7;
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
        // ring vertex `slot` of the row (triangle slot = (row point, ring[slot], ring[slot + 1]))
        int rk = INT_MIN;
        float2 g = make_float2(0.f, 0.f);
        if (row && slot < 6) {
            rk = G.ring[(size_t)i * 8 + slot];
            if (rk != INT_MIN) g = G.rxy[(size_t)i * 8 + slot];
        }
        const unsigned valid = __ballot_sync(0xffffffffu, rk != INT_MIN);
        const int deg = __popc((valid >> base) & 0xffu);
        const int nxt = base + (deg > 0 ? (slot + 1) % deg : 0);   // the lane holding ring[slot + 1]
        const float gbx = __shfl_sync(0xffffffffu, g.x, nxt), gby = __shfl_sync(0xffffffffu, g.y, nxt);
        const bool tri = slot < deg;
        // quadrature of this lane's triangle (once per row): vertices 0 (the
        // row point, at the origin), a = ring[slot], b = ring[slot + 1]
        float ca = 0.f, cb = 0.f, ea = 0.f, eb = 0.f, m = 0.f, mc = 0.f;
        if (tri) {
            const float D = g.x * gby - gbx * g.y;   // twice the signed area
            const float iD = 1.0f / D;
            // grad f = (ca (fa - f0) + cb (fb - f0), ea (fa - f0) + eb (fb - f0))
            ca = gby * iD; cb = -g.y * iD; ea = -gbx * iD; eb = g.x * iD;
            const float area = 0.5f * fabsf(D);
            m = area * (1.0f / 3.0f);                // int_T phi_i (the rule is exact)
            const float2 cs = G.cs0[i];              // cos x0, sin x0
            float acc = 0.f;
#pragma unroll
            for (int q = 0; q < 7; ++q) {
                float l0, la, lb, wq;
                rule_node(q, l0, la, lb, wq);
                float sd, cd;
                sincosf(la * g.x + lb * gbx, &sd, &cd);     // x - x0 at the node (small)
                acc += wq * l0 * (cs.x * cd - cs.y * sd);   // phi_i cos(x) at the node
            }
            mc = area * acc;                         // int_T phi_i cos(x)
        }
        const int p = row ? imap[i] : 0;
        const int kb0 = (row && cptr) ? cptr[i] : 0, kb1 = (row && cptr) ? cptr[i + 1] : 0;
        for (int v = v0; v < v1; ++v) {
            const float2 *fu = su + (size_t)v * V, *fw = sw + (size_t)v * V;
            // lane `slot` < deg: the fields at ring[slot]; lane 6: at the row point
            float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
            if (row && slot < 6 && rk >= 0) { a = fu[rk]; b = fw[rk]; }
            if (row && slot == 6) { a = fu[p]; b = fw[p]; }
            const int l6 = base + 6;
            const float u0h = __shfl_sync(0xffffffffu, a.x, l6), u0l = __shfl_sync(0xffffffffu, a.y, l6);
            const float w0h = __shfl_sync(0xffffffffu, b.x, l6), w0l = __shfl_sync(0xffffffffu, b.y, l6);
            // differences from the row point: the hi parts cancel exactly for nearby values
            const float du = (a.x - u0h) + (a.y - u0l), dw = (b.x - w0h) + (b.y - w0l);
            const float dub = __shfl_sync(0xffffffffu, du, nxt), dwb = __shfl_sync(0xffffffffu, dw, nxt);
            float s[8];
            if (tri) {
                const float ux = ca * du + cb * dub, uy = ea * du + eb * dub;
                const float wx = ca * dw + cb * dwb, wy = ea * dw + eb * dwb;
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
                double r;
                if (kb0 < kb1) {   // rows at the boundary point (FP64, a handful of rows)
                    double bs = 0.0;
                    const double *fb = (on_u ? u : w) + (size_t)v * ld;
                    for (int k = kb0; k < kb1; ++k) {
                        const int c = ccol[k];
                        bs += cval[k] * fb[bmap ? bmap[c] : c];
                    }
                    r = bs + (double)s[0];
                } else {
                    r = widen(s[0]);
                }
                out[((size_t)v * 8 + slot) * ldo + i] = r;
            }
        }
    }
}

}  // namespace

void build_jac_quad(const Mesh &m, JacQuadHost &h) {
    const int rs = m.rs;
    h.max_tri = 0;
    h.ring.assign((size_t)rs * 8, INT_MIN);
    h.rxy.assign((size_t)rs * 8 * 2, 0.f);
    h.cs0.assign((size_t)rs * 2, 0.f);
    for (int i = 0; i < rs; ++i) {
        const int p = m.inner[i];
        const int z = m.row_zone(p);
        const double x0 = m.u(p, z), y0 = m.v(p, z);
        h.cs0[2 * i] = (float)std::cos(x0);
        h.cs0[2 * i + 1] = (float)std::sin(x0);
        const int nt = m.adj_ptr[p + 1] - m.adj_ptr[p];
        h.max_tri = std::max(h.max_tri, nt);
        if (nt > 6 || nt < 3) { h.max_tri = std::max(h.max_tri, 7); continue; }
        // the triangles' other two vertices, then the closed ring around p
        std::vector<int> ea(nt), eb(nt);
        for (int q = 0; q < nt; ++q) {
            const int t = m.adj[m.adj_ptr[p] + q];
            int o[2], no = 0;
            for (int c = 0; c < 3; ++c)
                if (m.tri[3 * t + c] != p && no < 2) o[no++] = m.tri[3 * t + c];
            ea[q] = o[0]; eb[q] = o[1];
        }
        std::vector<int> ring(1, ea[0]);
        std::vector<char> used(nt, 0);
        used[0] = 1;
        int cur = eb[0];
        bool closed = false;
        for (int step = 1; step < nt; ++step) {
            ring.push_back(cur);
            int nextv = -1;
            for (int q = 0; q < nt; ++q) {
                if (used[q]) continue;
                if (ea[q] == cur) nextv = eb[q];
                else if (eb[q] == cur) nextv = ea[q];
                if (nextv >= 0) { used[q] = 1; break; }
            }
            if (nextv < 0) break;
            cur = nextv;
            if (step == nt - 1) closed = cur == ring[0];
        }
        if (!closed || (int)ring.size() != nt) { h.max_tri = std::max(h.max_tri, 7); continue; }
        for (int k = 0; k < nt; ++k) {
            const int v = ring[k];
            const size_t e = (size_t)i * 8 + k;
            h.ring[e] = m.bnd[v] ? -1 : v;
            h.rxy[2 * e] = (float)(m.u(v, z) - x0);
            h.rxy[2 * e + 1] = (float)(m.v(v, z) - y0);
        }
    }
}

size_t jac_quad_bytes(int rs, int V, int nv) {
    // split pass: both fields read (FP64) and written (float pairs) once;
    // quadrature: per row 6 ring vertices x (index + 2 coordinates) + cos/sin
    // of the row point, both fields read once per member as float pairs, 8
    // FP64 right-hand sides written
    return (size_t)nv * 2 * (size_t)V * 16 + (size_t)rs * (6 * 12 + 8) +
           (size_t)nv * (2 * (size_t)V * 8 + 8 * (size_t)rs * 8);
}

cudaError_t jac_quad(const JacQuadDev &G, const JacOps &J, const double *u, const double *v, int ld, const int *imap,
                     const int *bmap, double *out, int ldo, int nv, int V, float2 *split, cudaStream_t s) {
    if (G.n <= 0 || nv <= 0) return cudaSuccess;
    const long long total = (long long)nv * V;
    float2 *su = split, *sw = split + total;
    long long blocks = (total + 255) / 256;
    if (blocks > 152LL * 16) blocks = 152LL * 16;
    k_split2<<<(unsigned)blocks, 256, 0, s>>>(u, v, ld, V, total, su, sw);
    const int rowblocks = (G.n + ROWS_PER_BLOCK - 1) / ROWS_PER_BLOCK;
    const int chunks = (nv + MCHUNK - 1) / MCHUNK;
    if (chunks > 65535) return cudaErrorInvalidValue;
    dim3 grid(rowblocks, chunks);
    k_jac_quad<<<grid, 256, 0, s>>>(G, J, su, sw, V, u, v, ld, imap, bmap, out, ldo, nv);
    g_kernel_launches += 2;
    return cudaGetLastError();
}

}  // namespace phg
