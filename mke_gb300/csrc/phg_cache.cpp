// phg_cache.cpp -- the on-disk cache of a generated mesh level: the mesh, every
// assembled operator and the multigrid hierarchy, written once and read back
// by later processes instead of regenerating and reassembling them.  The
// data are stored byte for byte, so a cached level is bit-identical to a
// freshly built one.
//
// File: "PHGLVL01", int32 level, then the payload (every array as a uint64
// count followed by its raw elements), then a uint64 FNV-1a hash of the
// payload.  A file with another magic, level, a short payload or a hash
// mismatch is rejected (the caller rebuilds the level and rewrites it), and
// so is a well-formed file whose contents are inconsistent (an index out of
// range, operator or multigrid dimensions that do not fit the mesh): the
// checksum only catches damage, and every index read here is later
// dereferenced by the host assembly or the device kernels.
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <unistd.h>

#include "phg_host.hpp"

namespace phg {

namespace {

const char kMagic[8] = {'P', 'H', 'G', 'L', 'V', 'L', '0', '1'};

struct Writer {
    std::vector<unsigned char> buf;
    void raw(const void *p, size_t n) {
        const unsigned char *c = static_cast<const unsigned char *>(p);
        buf.insert(buf.end(), c, c + n);
    }
    template <typename T> void scalar(T v) { raw(&v, sizeof v); }
    template <typename T> void vec(const std::vector<T> &v) {
        scalar<uint64_t>(v.size());
        if (!v.empty()) raw(v.data(), sizeof(T) * v.size());
    }
};

struct Reader {
    const unsigned char *p, *end;
    bool ok = true;
    bool raw(void *dst, size_t n) {
        if (!ok || (size_t)(end - p) < n) return ok = false;
        std::memcpy(dst, p, n);
        p += n;
        return true;
    }
    template <typename T> bool scalar(T &v) { return raw(&v, sizeof v); }
    template <typename T> bool vec(std::vector<T> &v) {
        uint64_t n = 0;
        if (!scalar(n) || n > (uint64_t)(end - p) / sizeof(T)) return ok = false;
        v.resize((size_t)n);
        return n == 0 || raw(v.data(), sizeof(T) * (size_t)n);
    }
};

uint64_t fnv1a(const unsigned char *p, size_t n) {
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < n; ++i) { h ^= p[i]; h *= 1099511628211ull; }
    return h;
}

void put_mesh(Writer &w, const Mesh &m) {
    w.scalar<int32_t>(m.level); w.scalar<int32_t>(m.V); w.scalar<int32_t>(m.T);
    w.scalar<int32_t>(m.rs); w.scalar<int32_t>(m.os); w.scalar<int32_t>(m.nz);
    w.vec(m.xyz); w.vec(m.uv); w.vec(m.tri); w.vec(m.tz); w.vec(m.bnd);
    w.vec(m.inner); w.vec(m.outer); w.vec(m.p2io); w.vec(m.adj_ptr); w.vec(m.adj);
    w.vec(m.orig); w.vec(m.par_a); w.vec(m.par_b); w.vec(m.raw_xyz);
}

// every index a consumer of a generated level dereferences lies in range
bool mesh_indices_ok(const Mesh &m) {
    const int V = m.V, T = m.T;
    if (m.level < 1 || m.level > 9 || V != 10 * (1 << (2 * m.level)) + 2 || m.nz < 1 || m.nz > 4) return false;
    for (int x : m.tri)
        if (x < 0 || x >= V) return false;
    for (int z : m.tz)
        if (z < 0 || z >= m.nz) return false;
    int nb = 0;
    for (int b : m.bnd) {
        if (b != 0 && b != 1) return false;
        nb += b;
    }
    if (nb != m.os) return false;
    // the inner/outer maps and the point -> triangle adjacency are exactly
    // what finish_mesh derives from the triangles and the boundary flags
    Mesh d;
    d.V = V;
    d.T = T;
    d.tri = m.tri;
    d.bnd = m.bnd;
    finish_mesh(d);
    if (d.rs != m.rs || d.inner != m.inner || d.outer != m.outer || d.p2io != m.p2io || d.adj_ptr != m.adj_ptr ||
        d.adj != m.adj)
        return false;
    for (int p = 0; p < V; ++p)
        if (m.adj_ptr[p + 1] == m.adj_ptr[p]) return false;   // every point lies on a triangle
    // refinement history: orig is a permutation, the parents of a midpoint are
    // points of the level below (which has (V - 2) / 4 + 2 points)
    if (m.orig.size() != (size_t)V || m.par_a.size() != (size_t)V || m.par_b.size() != (size_t)V ||
        m.raw_xyz.size() != 3 * (size_t)V)
        return false;
    std::vector<char> seen((size_t)V, 0);
    for (int o : m.orig) {
        if (o < 0 || o >= V || seen[o]) return false;
        seen[o] = 1;
    }
    const int Vc = (V - 2) / 4 + 2;
    for (int p = Vc; p < V; ++p)
        if (m.par_a[p] < 0 || m.par_a[p] >= Vc || m.par_b[p] < 0 || m.par_b[p] >= Vc) return false;
    return true;
}

bool get_mesh(Reader &r, Mesh &m, bool allow_empty = false) {
    int32_t lv, V, T, rs, os, nz;
    r.scalar(lv); r.scalar(V); r.scalar(T); r.scalar(rs); r.scalar(os); r.scalar(nz);
    m.level = lv; m.V = V; m.T = T; m.rs = rs; m.os = os; m.nz = nz;
    r.vec(m.xyz); r.vec(m.uv); r.vec(m.tri); r.vec(m.tz); r.vec(m.bnd);
    r.vec(m.inner); r.vec(m.outer); r.vec(m.p2io); r.vec(m.adj_ptr); r.vec(m.adj);
    r.vec(m.orig); r.vec(m.par_a); r.vec(m.par_b); r.vec(m.raw_xyz);
    if (!r.ok) return false;
    if (allow_empty && V == 0 && T == 0 && m.xyz.empty() && m.tri.empty()) return true;   // an unused slot
    // the sizes the rest of the library relies on
    return V > 0 && T > 0 && rs >= 0 && os >= 0 && rs + os == V && m.xyz.size() == 3 * (size_t)V &&
           m.uv.size() == 8 * (size_t)V && m.tri.size() == 3 * (size_t)T && m.tz.size() == (size_t)T &&
           m.bnd.size() == (size_t)V && m.inner.size() == (size_t)rs && m.outer.size() == (size_t)os &&
           m.p2io.size() == (size_t)V && m.adj_ptr.size() == (size_t)V + 1 &&
           m.adj.size() == (size_t)m.adj_ptr[V] && mesh_indices_ok(m);
}

void put_csr(Writer &w, const Csr &a) {
    w.scalar<int32_t>(a.n); w.scalar<int32_t>(a.m);
    w.vec(a.ptr); w.vec(a.col); w.vec(a.val);
}

bool get_csr(Reader &r, Csr &a) {
    int32_t n, m;
    r.scalar(n); r.scalar(m);
    a.n = n; a.m = m;
    r.vec(a.ptr); r.vec(a.col); r.vec(a.val);
    if (r.ok && n == 0 && a.ptr.empty() && a.col.empty() && a.val.empty()) return true;   // an unused slot
    if (!r.ok || n < 0 || a.ptr.size() != (size_t)n + 1 || a.ptr[0] != 0) return false;
    for (int i = 0; i < n; ++i)
        if (a.ptr[i + 1] < a.ptr[i]) return false;
    const size_t nnz = (size_t)a.ptr[n];
    if (a.col.size() != nnz || a.val.size() != nnz) return false;
    for (int c : a.col)
        if (c < 0 || c >= m) return false;
    return true;
}

// the operators' shapes (inner x inner, inner x boundary, all x all)
bool ops_dims_ok(const SphereOps &o, const Mesh &m) {
    const Csr *sq[] = {&o.idt, &o.lapl, &o.jidt, &o.d1, &o.d2, &o.d1c, &o.d2c};
    const Csr *bc[] = {&o.bnd2, &o.bnd3, &o.d1b, &o.d2b, &o.d1cb, &o.d2cb};
    for (const Csr *a : sq)
        if (a->n != m.rs || a->m != m.rs) return false;
    for (const Csr *a : bc)
        if (a->n != m.rs || a->m != m.os) return false;
    return o.norm.n == m.V && o.norm.m == m.V;
}

// the hierarchy's levels one refinement apart, transfers and coarse
// operators sized by the inner points of the levels they connect
bool hierarchy_ok(const MgHierarchy &h, const Mesh &fine) {
    const size_t nlev = h.mesh.size();
    if (nlev < 2 || nlev > (size_t)fine.level || h.A.size() != nlev || h.P.size() != nlev - 1 ||
        h.R.size() != nlev - 1 || h.mesh[0].V != 0 || h.A[0].n != 0)
        return false;
    auto rows = [&](size_t k) { return k == 0 ? fine.rs : h.mesh[k].rs; };
    for (size_t k = 1; k < nlev; ++k)
        if (h.mesh[k].level != fine.level - (int)k || h.A[k].n != rows(k) || h.A[k].m != rows(k)) return false;
    for (size_t k = 0; k + 1 < nlev; ++k)
        if (h.P[k].n != rows(k) || h.P[k].m != rows(k + 1) || h.R[k].n != rows(k + 1) || h.R[k].m != rows(k))
            return false;
    const size_t nc = (size_t)rows(nlev - 1);
    return h.coarse_inv.size() == nc * nc;
}

}  // namespace

bool save_level_cache(const char *path, const Mesh &m, const SphereOps &ops, const MgHierarchy *mg) {
    Writer w;
    put_mesh(w, m);
    const Csr *all[] = {&ops.idt, &ops.lapl, &ops.jidt, &ops.d1, &ops.d2, &ops.d1c, &ops.d2c,
                        &ops.bnd2, &ops.bnd3, &ops.d1b, &ops.d2b, &ops.d1cb, &ops.d2cb, &ops.norm};
    for (const Csr *a : all) put_csr(w, *a);
    w.scalar<int32_t>(mg ? 1 : 0);
    if (mg) {
        w.scalar<uint64_t>(mg->mesh.size());
        for (const Mesh &x : mg->mesh) put_mesh(w, x);
        const std::vector<Csr> *lists[] = {&mg->A, &mg->P, &mg->R};
        for (const auto *l : lists) {
            w.scalar<uint64_t>(l->size());
            for (const Csr &a : *l) put_csr(w, a);
        }
        w.vec(mg->coarse_inv);
    }
    // write to a temporary name of this writer (process and call) and rename:
    // readers never see a partial file, and processes that build the same
    // level at once each write their own copy (the last rename wins; the
    // copies are identical)
    static std::atomic<unsigned> seq{0};
    const std::string tmp = std::string(path) + "." + std::to_string((long)getpid()) + "." +
                            std::to_string(seq.fetch_add(1)) + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) return false;
    const int32_t level = m.level;
    const uint64_t h = fnv1a(w.buf.data(), w.buf.size());
    bool ok = std::fwrite(kMagic, 1, 8, f) == 8 && std::fwrite(&level, sizeof level, 1, f) == 1 &&
              std::fwrite(w.buf.data(), 1, w.buf.size(), f) == w.buf.size() && std::fwrite(&h, sizeof h, 1, f) == 1;
    ok = (std::fclose(f) == 0) && ok;
    if (!ok || std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        return false;
    }
    return true;
}

bool load_level_cache(const char *path, int level, Mesh &m, SphereOps &ops, MgHierarchy &mg, bool &has_mg,
                      std::string &err) {
    FILE *f = std::fopen(path, "rb");
    if (!f) { err = "no cache file"; return false; }
    std::vector<unsigned char> all;
    unsigned char chunk[1 << 16];
    size_t k;
    while ((k = std::fread(chunk, 1, sizeof chunk, f)) > 0) all.insert(all.end(), chunk, chunk + k);
    std::fclose(f);
    if (all.size() < 8 + 4 + 8 || std::memcmp(all.data(), kMagic, 8) != 0) { err = "not a level cache"; return false; }
    int32_t lv;
    std::memcpy(&lv, all.data() + 8, sizeof lv);
    if (lv != level) { err = "cached level differs"; return false; }
    const unsigned char *pay = all.data() + 12;
    const size_t npay = all.size() - 12 - 8;
    uint64_t h;
    std::memcpy(&h, pay + npay, sizeof h);
    if (fnv1a(pay, npay) != h) { err = "cache checksum mismatch"; return false; }
    Reader r{pay, pay + npay};
    Mesh mm;
    SphereOps oo;
    if (!get_mesh(r, mm) || mm.level != level) { err = "bad mesh record"; return false; }
    Csr *all_ops[] = {&oo.idt, &oo.lapl, &oo.jidt, &oo.d1, &oo.d2, &oo.d1c, &oo.d2c,
                      &oo.bnd2, &oo.bnd3, &oo.d1b, &oo.d2b, &oo.d1cb, &oo.d2cb, &oo.norm};
    for (Csr *a : all_ops)
        if (!get_csr(r, *a)) { err = "bad operator record"; return false; }
    if (!ops_dims_ok(oo, mm)) { err = "operator shapes do not fit the mesh"; return false; }
    int32_t flag = 0;
    MgHierarchy hh;
    if (!r.scalar(flag)) { err = "truncated"; return false; }
    if (flag) {
        uint64_t nm = 0;
        if (!r.scalar(nm) || nm > 64) { err = "bad hierarchy record"; return false; }
        hh.mesh.resize((size_t)nm);
        for (Mesh &x : hh.mesh)
            if (!get_mesh(r, x, true)) { err = "bad hierarchy mesh"; return false; }
        std::vector<Csr> *lists[] = {&hh.A, &hh.P, &hh.R};
        for (auto *l : lists) {
            uint64_t nl = 0;
            if (!r.scalar(nl) || nl > 64) { err = "bad hierarchy record"; return false; }
            l->resize((size_t)nl);
            for (Csr &a : *l)
                if (!get_csr(r, a)) { err = "bad hierarchy operator"; return false; }
        }
        if (!r.vec(hh.coarse_inv)) { err = "bad coarse inverse"; return false; }
        if (!hierarchy_ok(hh, mm)) { err = "hierarchy does not fit the mesh"; return false; }
    }
    if (r.p != r.end) { err = "trailing bytes"; return false; }
    m = std::move(mm);
    ops = std::move(oo);
    has_mg = flag != 0;
    if (has_mg) mg = std::move(hh);
    return true;
}

}  // namespace phg
