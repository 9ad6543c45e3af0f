// phg_tune.cu -- the launch-shape table filled by the autotuner.
//
// Two kinds of shape are tuned on the device they run on:
//  * solves: rows per block of the persistent solver kernels (how many
//    blocks share one right-hand side) and, for Chebyshev-solvable
//    operators in mixed precision, whether a batch runs as per-member
//    persistent kernels or as lockstep launches over an interleaved FP32
//    multi-vector;
//  * operator applies on interleaved FP32 multi-vectors: threads per row
//    (the vector width one thread carries is then nv / 4 / threads-per-row
//    float4 chunks).
// The key is (kernel family, rows, precision, right-hand-side bucket), so
// every operator of the same size and family shares a tuned shape (the mass
// matrices of one mesh level, say).  Buckets are powers of two: nv in
// (2^(b-1), 2^b] maps to b.  The table is process-wide and can be saved to /
// loaded from a text file; entries loaded from a file written on another
// device model are ignored.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "phg_device.cuh"

namespace phg {

namespace {

using Key = std::tuple<int, int, int, int>;   // family, rows, precision, bucket
std::mutex g_mu;
std::map<Key, SolveShape> g_solve;
std::map<std::pair<int, int>, int> g_spmm;   // (rows, bucket) -> threads per row

std::string device_name() {
    int dev = 0;
    cudaDeviceProp p;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess) return "unknown";
    std::string s = p.name;
    for (char &c : s)
        if (c == ' ' || c == '\t') c = '_';
    char cc[32];
    snprintf(cc, sizeof cc, "_sm%d%d", p.major, p.minor);
    return s + cc;
}

}  // namespace

int nv_bucket(int nv) {
    int b = 0;
    while ((1 << b) < nv && b < 30) ++b;
    return b;
}

int solve_family(const DevSolveOp &op) {
    if (op.block4) return 3;
    if (op.mgd) return 2;
    if (op.cheb_lmax > 0.0 && op.cheb_lmin > 0.0) return 1;
    return 0;
}

bool tune_get_solve(int family, int n, Precision p, int nv, SolveShape *out) {
    std::lock_guard<std::mutex> g(g_mu);
    auto it = g_solve.find(Key(family, n, (int)p, nv_bucket(nv)));
    if (it == g_solve.end()) return false;
    *out = it->second;
    return true;
}

void tune_set_solve(int family, int n, Precision p, int nv, const SolveShape &s) {
    std::lock_guard<std::mutex> g(g_mu);
    g_solve[Key(family, n, (int)p, nv_bucket(nv))] = s;
}

bool tune_get_spmm(int n, int nv, int *tpr) {
    std::lock_guard<std::mutex> g(g_mu);
    auto it = g_spmm.find({n, nv_bucket(nv)});
    if (it == g_spmm.end()) return false;
    *tpr = it->second;
    return true;
}

void tune_set_spmm(int n, int nv, int tpr) {
    std::lock_guard<std::mutex> g(g_mu);
    g_spmm[{n, nv_bucket(nv)}] = tpr;
}

void tune_clear() {
    std::lock_guard<std::mutex> g(g_mu);
    g_solve.clear();
    g_spmm.clear();
}

// one line per entry:
//   solve <family> <rows> <precision> <bucket> <rows_per_block> <path>
//   spmm <rows> <bucket> <threads_per_row>
std::string tune_describe() {
    std::lock_guard<std::mutex> g(g_mu);
    std::string s;
    char line[160];
    for (auto &kv : g_solve) {
        snprintf(line, sizeof line, "solve %d %d %d %d %d %d\n", std::get<0>(kv.first), std::get<1>(kv.first),
                 std::get<2>(kv.first), std::get<3>(kv.first), kv.second.rpb, kv.second.path);
        s += line;
    }
    for (auto &kv : g_spmm) {
        snprintf(line, sizeof line, "spmm %d %d %d\n", kv.first.first, kv.first.second, kv.second);
        s += line;
    }
    return s;
}

int tune_save(const char *path) {
    FILE *f = fopen(path, "w");
    if (!f) return -1;
    const std::string body = tune_describe();
    fprintf(f, "phelm-gb300-tune 1 %s\n", device_name().c_str());
    fputs(body.c_str(), f);
    return fclose(f) == 0 ? 0 : -1;
}

// returns the entries read (0 when the file was written on another device
// model), -1 when the file cannot be read or is malformed
int tune_load(const char *path) {
    FILE *f = fopen(path, "r");
    if (!f) return -1;
    char dev[256] = {0};
    int ver = 0;
    if (fscanf(f, "phelm-gb300-tune %d %255s", &ver, dev) != 2 || ver != 1) { fclose(f); return -1; }
    if (device_name() != dev) { fclose(f); return 0; }
    int count = 0;
    char kind[16];
    while (fscanf(f, "%15s", kind) == 1) {
        if (!strcmp(kind, "solve")) {
            int fam, n, p, b, rpb, path;
            if (fscanf(f, "%d %d %d %d %d %d", &fam, &n, &p, &b, &rpb, &path) != 6 || rpb < 0 || rpb > 65536 ||
                path < -1 || path > 1 || b < 0 || b > 30) { fclose(f); return -1; }
            SolveShape s;
            s.rpb = rpb;
            s.path = path;
            std::lock_guard<std::mutex> g(g_mu);
            g_solve[Key(fam, n, p, b)] = s;
        } else if (!strcmp(kind, "spmm")) {
            int n, b, tpr;
            if (fscanf(f, "%d %d %d", &n, &b, &tpr) != 3 || tpr < 1 || tpr > 64 || (tpr & (tpr - 1)) || b < 0 ||
                b > 30) { fclose(f); return -1; }
            std::lock_guard<std::mutex> g(g_mu);
            g_spmm[{n, b}] = tpr;
        } else {
            fclose(f);
            return -1;
        }
        ++count;
    }
    fclose(f);
    return count;
}

}  // namespace phg
