// Runs the library's host code (mesh generation, text round trip, operator
// assembly, multigrid hierarchy, barotropic and baroclinic matrices, text
// output) at levels 1-4 under AddressSanitizer and UndefinedBehaviorSanitizer,
// then the level cache: a round trip, and the reader on damaged files --
// truncated payloads and flipped bytes, each with its checksum recomputed so
// that the parser itself sees them; what it accepts goes through the
// assembly and the multigrid build -- and the mesh text parser on truncated
// and edited files, an accepted mesh going through the assembly.  Built and run by
// tests/test_sanitizers.py (argument: a scratch directory); exits non-zero on
// the first inconsistency (the sanitizers abort on their own findings).
#include <cmath>
#include <cstdint>
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

static uint64_t fnv1a(const unsigned char *p, size_t n) {
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < n; ++i) { h ^= p[i]; h *= 1099511628211ull; }
    return h;
}

static std::vector<unsigned char> read_all(const std::string &path) {
    std::vector<unsigned char> b;
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return b;
    unsigned char chunk[1 << 16];
    size_t k;
    while ((k = fread(chunk, 1, sizeof chunk, f)) > 0) b.insert(b.end(), chunk, chunk + k);
    fclose(f);
    return b;
}

// magic + level, then `payload` and its recomputed checksum
static void write_with_hash(const std::string &path, const std::vector<unsigned char> &head,
                            const std::vector<unsigned char> &payload) {
    FILE *f = fopen(path.c_str(), "wb");
    const uint64_t h = fnv1a(payload.data(), payload.size());
    fwrite(head.data(), 1, head.size(), f);
    if (!payload.empty()) fwrite(payload.data(), 1, payload.size(), f);
    fwrite(&h, sizeof h, 1, f);
    fclose(f);
}

// load a (possibly damaged) cache file; when accepted, run the consumers of
// its indices.  Returns whether the reader accepted it.
static bool load_and_use(const std::string &path, int level) {
    Mesh m;
    SphereOps ops;
    MgHierarchy h;
    bool has_mg = false;
    std::string err;
    if (!load_level_cache(path.c_str(), level, m, ops, h, has_mg, err)) return false;
    SphereOps again;
    assemble_sphere(m, again);
    MgHierarchy h2;
    build_mg(m, 1, h2, err);
    return true;
}

static int cache_checks(const std::string &dir) {
    int bad = 0;
    std::string err;
    // round trip at level 3
    {
        Mesh m;
        generate_sphere(3, m, err);
        SphereOps ops;
        assemble_sphere(m, ops);
        MgHierarchy h;
        build_mg(m, 1, h, err);
        const std::string path = dir + "/level3.cache";
        bad += check(save_level_cache(path.c_str(), m, ops, &h), "save_level_cache", 3);
        Mesh m2;
        SphereOps o2;
        MgHierarchy h2;
        bool has_mg = false;
        bad += check(load_level_cache(path.c_str(), 3, m2, o2, h2, has_mg, err) && has_mg, "load_level_cache", 3);
        bad += check(m2.tri == m.tri && m2.xyz == m.xyz && o2.lapl.val == ops.lapl.val && o2.norm.col == ops.norm.col &&
                     h2.P.size() == h.P.size() && h2.coarse_inv == h.coarse_inv, "cache round trip", 3);
        bad += check(!load_level_cache(path.c_str(), 4, m2, o2, h2, has_mg, err), "wrong level accepted", 3);
    }
    // damaged files at level 2
    Mesh m;
    generate_sphere(2, m, err);
    SphereOps ops;
    assemble_sphere(m, ops);
    MgHierarchy h;
    build_mg(m, 1, h, err);
    const std::string good = dir + "/level2.cache", path = dir + "/damaged.cache";
    bad += check(save_level_cache(good.c_str(), m, ops, &h), "save_level_cache", 2);
    const std::vector<unsigned char> file = read_all(good);
    bad += check(file.size() > 20, "cache size", 2);
    if (bad) return bad;
    const std::vector<unsigned char> head(file.begin(), file.begin() + 12);
    const std::vector<unsigned char> payload(file.begin() + 12, file.end() - 8);
    const size_t n = payload.size();
    bad += check(load_and_use(good, 2), "intact file rejected", 2);
    // truncations: never accepted
    int accepted = 0;
    for (size_t k = 0; k < 200; ++k) {
        const size_t cut = k < 32 ? k : k < 64 ? n - (64 - k) : (n * (k - 64)) / 136;
        write_with_hash(path, head, std::vector<unsigned char>(payload.begin(), payload.begin() + cut));
        accepted += load_and_use(path, 2);
    }
    bad += check(accepted == 0, "truncated payload accepted", 2);
    // flipped bytes: every byte of the mesh scalars and the first counts, then
    // positions spread over the payload; accepted files must be usable
    uint64_t x = 88172645463325252ull;
    int tried = 0;
    const unsigned char flips[3] = {0xFF, 0x80, 0x01};
    for (size_t k = 0; k < 64 + 300; ++k) {
        size_t pos;
        if (k < 64) {
            pos = k;
        } else {
            x ^= x << 13; x ^= x >> 7; x ^= x << 17;
            pos = (size_t)(x % n);
        }
        for (int f = 0; f < 3; ++f) {
            if (k >= 64 && f != (int)(k % 3)) continue;   // one flip per spread position
            std::vector<unsigned char> p = payload;
            p[pos] ^= flips[f];
            write_with_hash(path, head, p);
            load_and_use(path, 2);
            ++tried;
        }
    }
    // garbage and empty files
    {
        FILE *f = fopen(path.c_str(), "wb");
        fclose(f);
        bad += check(!load_and_use(path, 2), "empty file accepted", 2);
        f = fopen(path.c_str(), "wb");
        for (int i = 0; i < 4096; ++i) fputc((i * 131 + 7) & 255, f);
        fclose(f);
        bad += check(!load_and_use(path, 2), "garbage accepted", 2);
    }
    printf("cache: %d damaged files read\n", tried + 200);
    return bad;
}

// the mesh text parser on damaged files: truncations and single-character
// edits of a level-2 mesh; an accepted mesh goes through the assembly
static int text_checks(const std::string &dir) {
    int bad = 0;
    std::string err;
    Mesh m;
    generate_sphere(2, m, err);
    const std::string good = dir + "/level2.txt", path = dir + "/damaged.txt";
    FILE *f = fopen(good.c_str(), "wb");
    bad += check(f && save_mesh_text(f, m), "save_mesh_text", 2);
    if (f) fclose(f);
    const std::vector<unsigned char> text = read_all(good);
    bad += check(text.size() > 1000, "mesh text size", 2);
    if (bad) return bad;
    auto try_load = [&](const std::vector<unsigned char> &t) {
        FILE *g = fopen(path.c_str(), "wb");
        if (!t.empty()) fwrite(t.data(), 1, t.size(), g);
        fclose(g);
        g = fopen(path.c_str(), "rb");
        Mesh back;
        const bool ok = load_mesh_text(g, back, err);
        fclose(g);
        if (ok) {
            SphereOps ops;
            assemble_sphere(back, ops);
        }
        return ok;
    };
    bad += check(try_load(text), "intact mesh text rejected", 2);
    const size_t n = text.size();
    int tried = 0;
    for (size_t k = 0; k < 100; ++k) {   // truncations
        try_load(std::vector<unsigned char>(text.begin(), text.begin() + (n * k) / 100));
        ++tried;
    }
    const char edits[] = "0123456789;; -\nex";
    uint64_t x = 2463534242ull;
    for (int k = 0; k < 400; ++k) {      // one character replaced
        x ^= x << 13; x ^= x >> 7; x ^= x << 17;
        std::vector<unsigned char> t = text;
        t[(size_t)(x % n)] = (unsigned char)edits[(x >> 32) % (sizeof edits - 1)];
        try_load(t);
        ++tried;
    }
    printf("text: %d damaged mesh files read\n", tried);
    return bad;
}

int main(int argc, char **argv) {
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
    bad += cache_checks(argc > 1 ? argv[1] : ".");
    bad += text_checks(argc > 1 ? argv[1] : ".");
    if (!bad) printf("host code clean at levels 1-4\n");
    return bad ? 1 : 0;
}
