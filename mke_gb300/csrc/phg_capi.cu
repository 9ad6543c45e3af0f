// phg_capi.cu -- the C ABI (include/phelm_gb300.h): handles, HBM residency of
// the operators, host/device argument staging and the time-step drivers.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/phelm_gb300.h"
#include "phg_api.hpp"
#include "phg_host.hpp"
#include <nvtx3/nvToolsExt.h>
#include "phg_kernels.cuh"
#include "phg_jacquad.cuh"

using namespace phg;

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    try {
        g_err = buf;
    } catch (...) {   // no memory for the message: keep the code
    }
    return code;
}

// a FILE closed on every exit, an exception included; close() reports fclose's result
struct OpenFile {
    FILE *f;
    OpenFile(const char *path, const char *mode) : f(fopen(path, mode)) {}
    ~OpenFile() {
        if (f) fclose(f);
    }
    bool close() {
        FILE *g = f;
        f = nullptr;
        return g && fclose(g) == 0;
    }
    OpenFile(const OpenFile &) = delete;
    OpenFile &operator=(const OpenFile &) = delete;
};

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) return fail(PHG_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

// NVTX range for profiler timelines (a no-op without a tool attached)
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// owning device allocation
// device bytes held by the library: in total, and allocated by this thread
// (a serving lane creates, uses and frees its handles on its own thread)
std::atomic<long long> g_dev_bytes{0};
thread_local long long t_dev_bytes = 0;
// bumped by every device (re)allocation: a captured step graph holds raw
// buffer addresses and is re-captured when this moved since its capture
std::atomic<long long> g_alloc_epoch{0};
// bumped when the tuned launch shapes change: captured steps re-capture
std::atomic<long long> g_shape_epoch{0};

struct DBuf {
    void *p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    ~DBuf() { release(); }
    void release() {
        if (!p) return;
        cudaFree(p);
        g_dev_bytes -= (long long)n;
        t_dev_bytes -= (long long)n;
        p = nullptr; n = 0;
    }
    cudaError_t ensure(size_t bytes) {
        if (bytes <= n) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(&p, bytes ? bytes : 1);
        g_alloc_epoch++;
        if (e == cudaSuccess) {
            n = bytes;
            g_dev_bytes += (long long)n;
            t_dev_bytes += (long long)n;
        } else {
            p = nullptr;
        }
        return e;
    }
    template <typename T> T *as() const { return (T *)p; }
};

template <typename T>
cudaError_t upload(DBuf &b, const std::vector<T> &v) {
    cudaError_t e = b.ensure(sizeof(T) * v.size());
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpy(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice);
}

bool is_device_ptr(const void *p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

int phg::api_exception() noexcept {
    try {
        throw;
    } catch (const std::bad_alloc &) {
        return fail(PHG_ERR_HOST, "host memory exhausted");
    } catch (const std::exception &e) {
        return fail(PHG_ERR_HOST, "host failure: %s", e.what());
    } catch (...) {
        return fail(PHG_ERR_HOST, "host failure");
    }
}

// ----------------------------------------------------------------- mesh ---
// A level's host data -- the mesh, its assembled operators and the multigrid
// hierarchy -- shared by every mesh handle of that level in the process (and,
// with a cache directory, read from / written to disk once per level).
struct LevelData {
    Mesh m;
    std::once_flag assembled;
    SphereOps ops;
    bool ops_ready = false;          // filled from the disk cache
    void assemble() { std::call_once(assembled, [this] { if (!ops_ready) assemble_sphere(m, ops); }); }
    std::once_flag mg_once;
    MgHierarchy mg;
    bool mg_ready = false;           // filled from the disk cache
    bool mg_ok = false;
    std::string mg_err;
    const MgHierarchy *hierarchy(std::string &err) {
        std::call_once(mg_once, [this] { mg_ok = mg_ready || build_mg(m, 1, mg, mg_err); });
        if (!mg_ok) err = mg_err;
        return mg_ok ? &mg : nullptr;
    }
};

struct phg_mesh_s {
    std::atomic<int> refs{1};   // the caller's, plus one per operator set
    std::shared_ptr<LevelData> d;
    Mesh &m;
    SphereOps &ops;
    explicit phg_mesh_s(std::shared_ptr<LevelData> dd) : d(std::move(dd)), m(d->m), ops(d->ops) {}
    void assemble() { d->assemble(); }
    const MgHierarchy *hierarchy(std::string &err) { return d->hierarchy(err); }
};

namespace {

// generated levels alive in the process (one slot per level: different levels
// are built concurrently, one level once), and the optional cache directory
struct LevelSlot {
    std::mutex mu;
    std::weak_ptr<LevelData> live;
};
std::mutex g_level_mu;   // guards g_levels and g_cache_dir
std::map<int, std::shared_ptr<LevelSlot>> g_levels;
std::string g_cache_dir = [] {
    const char *e = getenv("PHG_CACHE_DIR");
    return std::string(e ? e : "");
}();

std::string cache_path(const std::string &dir, int level) {
    return dir + "/phelm_level" + std::to_string(level) + ".cache";
}

// write a level's data to the cache directory (best effort: a missing or
// read-only directory is not an error)
void save_level(const std::string &dir, int level, LevelData &d) {
    d.assemble();
    std::string mg_err;
    const MgHierarchy *h = level >= 2 ? d.hierarchy(mg_err) : nullptr;
    save_level_cache(cache_path(dir, level).c_str(), d.m, d.ops, h);
}

// the shared data of a generated level: a live one, else the disk cache, else
// generate (and, with a cache directory, assemble everything and save it)
int level_data(int level, std::shared_ptr<LevelData> &out) {
    std::shared_ptr<LevelSlot> slot;
    std::string dir;
    {
        std::lock_guard<std::mutex> g(g_level_mu);
        std::shared_ptr<LevelSlot> &e = g_levels[level];
        if (!e) e = std::make_shared<LevelSlot>();
        slot = e;
        dir = g_cache_dir;
    }
    std::lock_guard<std::mutex> g(slot->mu);   // one level is built once; other levels proceed
    if ((out = slot->live.lock())) {
        // a live level and a cache directory without its file (the directory
        // was set after the level was built): write it now
        if (!dir.empty()) {
            if (FILE *f = fopen(cache_path(dir, level).c_str(), "rb")) fclose(f);
            else save_level(dir, level, *out);
        }
        return PHG_OK;
    }
    auto d = std::make_shared<LevelData>();
    std::string err;
    bool loaded = false;
    if (!dir.empty()) {
        bool has_mg = false;
        if (load_level_cache(cache_path(dir, level).c_str(), level, d->m, d->ops, d->mg, has_mg, err)) {
            loaded = true;
            d->ops_ready = true;
            d->mg_ready = has_mg;
        }
    }
    if (!loaded) {
        if (!generate_sphere(level, d->m, err)) return fail(PHG_ERR_ARG, "%s", err.c_str());
        if (!dir.empty()) save_level(dir, level, *d);
    }
    slot->live = d;
    out = std::move(d);
    return PHG_OK;
}

}  // namespace

extern "C" int phg_cache_dir(const char *path) {
    PHG_API_BEGIN
    std::lock_guard<std::mutex> g(g_level_mu);
    g_cache_dir = path ? path : "";
    return PHG_OK;
    PHG_API_END
}

extern "C" const char *phg_last_error(void) { return g_err.c_str(); }
extern "C" const char *phg_version(void) { return "phelm-gb300 0.1 (sm_103a)"; }
extern "C" long long phg_kernel_launches(void) { return g_kernel_launches.load(); }

extern "C" int phg_mesh_generate(int level, phg_mesh *out) {
    PHG_API_BEGIN
    if (!out) return fail(PHG_ERR_ARG, "out is NULL");
    std::shared_ptr<LevelData> d;
    int r = level_data(level, d);
    if (r) return r;
    *out = new phg_mesh_s(std::move(d));
    return PHG_OK;
    PHG_API_END
}

extern "C" int phg_mesh_load_file(const char *path, phg_mesh *out) {
    PHG_API_BEGIN
    if (!path || !out) return fail(PHG_ERR_ARG, "NULL argument");
    OpenFile f(path, "rb");
    if (!f.f) return fail(PHG_ERR_IO, "cannot open %s", path);
    auto d = std::make_shared<LevelData>();   // a loaded mesh keeps its own data
    std::string err;
    bool ok = load_mesh_text(f.f, d->m, err);
    f.close();
    if (!ok) return fail(PHG_ERR_IO, "%s: %s", path, err.c_str());
    *out = new phg_mesh_s(std::move(d));
    return PHG_OK;
    PHG_API_END
}

static void mesh_release(phg_mesh m) {
    if (m && m->refs.fetch_sub(1) == 1) delete m;
}

extern "C" void phg_mesh_destroy(phg_mesh m) { PHG_API_BEGIN mesh_release(m); PHG_API_END_VOID }

extern "C" int phg_mesh_save_file(phg_mesh h, const char *path) {
    PHG_API_BEGIN
    if (!h || !path) return fail(PHG_ERR_ARG, "NULL argument");
    OpenFile f(path, "wb");
    if (!f.f) return fail(PHG_ERR_IO, "cannot open %s", path);
    const bool ok = save_mesh_text(f.f, h->m);
    const bool closed = f.close();
    if (!ok) return fail(PHG_ERR_ARG, "only 4-chart sphere meshes can be written");
    if (!closed) return fail(PHG_ERR_IO, "cannot write %s", path);
    return PHG_OK;
    PHG_API_END
}

static int print_common(phg_mesh h, const char *path, const double *ans, const double *x, const double *y,
                        const double *z, bool inner) {
    if (!h || !path || !ans) return fail(PHG_ERR_ARG, "NULL argument");
    if (is_device_ptr(ans) || (x && is_device_ptr(x)) || (y && is_device_ptr(y)) || (z && is_device_ptr(z)))
        return fail(PHG_ERR_ARG, "host arrays only");
    OpenFile f(path, "wb");
    if (!f.f) return fail(PHG_ERR_IO, "cannot open %s", path);
    print_function_text(f.f, h->m, ans, x, y, z, inner);
    if (!f.close()) return fail(PHG_ERR_IO, "cannot write %s", path);
    return PHG_OK;
}

// Binary state checkpoints: "PHGSTAT1", int32 V, int32 nfields, float64 t,
// int64 step, uint64 mesh digest (FNV-1a over the point coordinates and
// triangles), then nfields x V float64, all little-endian as in memory.
static unsigned long long mesh_digest(const Mesh &m) {
    unsigned long long h = 1469598103934665603ULL;
    auto add = [&](const void *p, size_t n) {
        const unsigned char *c = (const unsigned char *)p;
        for (size_t i = 0; i < n; ++i) { h ^= c[i]; h *= 1099511628211ULL; }
    };
    add(m.xyz.data(), 8 * m.xyz.size());
    add(m.tri.data(), 4 * m.tri.size());
    return h;
}

extern "C" int phg_state_save(phg_mesh h, const char *path, const double *const *fields, int nfields, double t,
                              long long step) {
    PHG_API_BEGIN
    if (!h || !path || !fields || nfields < 1) return fail(PHG_ERR_ARG, "bad argument");
    for (int k = 0; k < nfields; ++k)
        if (!fields[k] || is_device_ptr(fields[k])) return fail(PHG_ERR_ARG, "field %d: host array required", k);
    OpenFile of(path, "wb");
    FILE *f = of.f;
    if (!f) return fail(PHG_ERR_IO, "cannot open %s", path);
    const int V = h->m.V;
    const unsigned long long dg = mesh_digest(h->m);
    bool ok = fwrite("PHGSTAT1", 1, 8, f) == 8 && fwrite(&V, 4, 1, f) == 1 && fwrite(&nfields, 4, 1, f) == 1 &&
              fwrite(&t, 8, 1, f) == 1 && fwrite(&step, 8, 1, f) == 1 && fwrite(&dg, 8, 1, f) == 1;
    for (int k = 0; ok && k < nfields; ++k) ok = fwrite(fields[k], 8, (size_t)V, f) == (size_t)V;
    ok = of.close() && ok;
    return ok ? PHG_OK : fail(PHG_ERR_IO, "cannot write %s", path);
    PHG_API_END
}

extern "C" int phg_state_load(phg_mesh h, const char *path, double *const *fields, int nfields, double *t,
                              long long *step) {
    PHG_API_BEGIN
    if (!h || !path || !fields || nfields < 1) return fail(PHG_ERR_ARG, "bad argument");
    OpenFile of(path, "rb");
    FILE *f = of.f;
    if (!f) return fail(PHG_ERR_IO, "cannot open %s", path);
    char magic[8];
    int V = 0, nf = 0;
    double tt = 0;
    long long st = 0;
    unsigned long long dg = 0;
    bool ok = fread(magic, 1, 8, f) == 8 && !memcmp(magic, "PHGSTAT1", 8) && fread(&V, 4, 1, f) == 1 &&
              fread(&nf, 4, 1, f) == 1 && fread(&tt, 8, 1, f) == 1 && fread(&st, 8, 1, f) == 1 &&
              fread(&dg, 8, 1, f) == 1;
    if (!ok) return fail(PHG_ERR_IO, "%s: not a state checkpoint", path);
    if (V != h->m.V || dg != mesh_digest(h->m)) return fail(PHG_ERR_ARG, "%s: written for another mesh", path);
    if (nf != nfields) return fail(PHG_ERR_ARG, "%s: holds %d fields, %d requested", path, nf, nfields);
    for (int k = 0; ok && k < nfields; ++k) {
        if (!fields[k] || is_device_ptr(fields[k])) return fail(PHG_ERR_ARG, "field %d: host array required", k);
        ok = fread(fields[k], 8, (size_t)V, f) == (size_t)V;
    }
    if (!ok) return fail(PHG_ERR_IO, "%s: truncated", path);
    if (t) *t = tt;
    if (step) *step = st;
    return PHG_OK;
    PHG_API_END
}

extern "C" int phg_print_function(phg_mesh h, const char *path, const double *ans, const double *x, const double *y,
                                  const double *z) {
    PHG_API_BEGIN
    return print_common(h, path, ans, x, y, z, false);
    PHG_API_END
}

extern "C" int phg_print_inner_function(phg_mesh h, const char *path, const double *ans, const double *x,
                                        const double *y, const double *z) {
    PHG_API_BEGIN
    return print_common(h, path, ans, x, y, z, true);
    PHG_API_END
}

extern "C" int phg_mesh_info(phg_mesh h, int *V, int *T, int *rs, int *os) {
    PHG_API_BEGIN
    if (!h) return fail(PHG_ERR_ARG, "NULL mesh");
    if (V) *V = h->m.V;
    if (T) *T = h->m.T;
    if (rs) *rs = h->m.rs;
    if (os) *os = h->m.os;
    return PHG_OK;
    PHG_API_END
}

extern "C" int phg_mesh_arrays(phg_mesh h, double *xyz, double *uv, int *tri, int *tz, int *bnd) {
    PHG_API_BEGIN
    if (!h) return fail(PHG_ERR_ARG, "NULL mesh");
    const Mesh &m = h->m;
    if (xyz) memcpy(xyz, m.xyz.data(), 8 * m.xyz.size());
    if (uv) memcpy(uv, m.uv.data(), 8 * m.uv.size());
    if (tri) memcpy(tri, m.tri.data(), 4 * m.tri.size());
    if (tz) memcpy(tz, m.tz.data(), 4 * m.tz.size());
    if (bnd) memcpy(bnd, m.bnd.data(), 4 * m.bnd.size());
    return PHG_OK;
    PHG_API_END
}

extern "C" int phg_mesh_maps(phg_mesh h, int *inner, int *outer, int *p2io) {
    PHG_API_BEGIN
    if (!h) return fail(PHG_ERR_ARG, "NULL mesh");
    const Mesh &m = h->m;
    if (inner) memcpy(inner, m.inner.data(), 4 * m.inner.size());
    if (outer) memcpy(outer, m.outer.data(), 4 * m.outer.size());
    if (p2io) memcpy(p2io, m.p2io.data(), 4 * m.p2io.size());
    return PHG_OK;
    PHG_API_END
}

static const Csr *find_csr(phg_mesh_s *h, const char *name) {
    SphereOps &o = h->ops;
    struct { const char *n; const Csr *c; } t[] = {
        {"idt", &o.idt}, {"lapl", &o.lapl}, {"bnd2", &o.bnd2}, {"bnd3", &o.bnd3}, {"jidt", &o.jidt},
        {"d1", &o.d1}, {"d2", &o.d2}, {"d1c", &o.d1c}, {"d2c", &o.d2c}, {"d1b", &o.d1b}, {"d2b", &o.d2b},
        {"d1cb", &o.d1cb}, {"d2cb", &o.d2cb}, {"norm", &o.norm}};
    for (auto &e : t)
        if (!strcmp(e.n, name)) return e.c;
    return nullptr;
}

extern "C" int phg_mesh_csr(phg_mesh h, const char *name, int *n, int *nnz, int *ptr, int *col, double *val) {
    PHG_API_BEGIN
    if (!h || !name) return fail(PHG_ERR_ARG, "NULL argument");
    h->assemble();
    const Csr *c = find_csr(h, name);
    if (!c) return fail(PHG_ERR_ARG, "unknown operator '%s'", name);
    if (n) *n = c->n;
    if (nnz) *nnz = c->nnz();
    if (ptr) memcpy(ptr, c->ptr.data(), 4 * c->ptr.size());
    if (col) memcpy(col, c->col.data(), 4 * c->col.size());
    if (val) memcpy(val, c->val.data(), 8 * c->val.size());
    return PHG_OK;
    PHG_API_END
}

// ------------------------------------------------------- device operators ---
namespace {

// slot-major ELL of an rs x rs CSR on a given pattern
void to_ell(const Csr &c, int W, std::vector<int> *col, std::vector<double> &val) {
    const int n = c.n;
    if (col) col->assign((size_t)W * n, 0);
    val.assign((size_t)W * n, 0.0);
    for (int i = 0; i < n; ++i) {
        int k = 0;
        for (int q = c.ptr[i]; q < c.ptr[i + 1]; ++q, ++k) {
            if (col) (*col)[(size_t)k * n + i] = c.col[q];
            val[(size_t)k * n + i] = c.val[q];
        }
        for (; k < W; ++k)
            if (col) (*col)[(size_t)k * n + i] = i;
    }
}

struct SolveOpBufs {
    DBuf val, as64, as32, a32, dinv, dinv32;
    DBuf pk;   // FP32 row records for the interleaved apply: 8 (column, value) pairs per row
    DevSolveOp op;
};

// one uploaded multigrid level (level 0 reuses the solve operator's arrays)
struct MgLevelBufs {
    DBuf col, a64, a32, d64, d32, pc, pw64, pw32, rf, rw64, rw32;
};

struct MgBufs {
    std::vector<std::unique_ptr<MgLevelBufs>> lev;
    DBuf cinv64, cinv32;
    DBuf desc;   // the MgDev descriptor in device memory
};

struct ColsBufs {
    DBuf ptr, col, val;
    DevCols c;
};

}  // namespace

struct phg_ops_s {
    std::atomic<int> refs{1};   // the caller's, plus one per time stepper
    phg_mesh_s *mesh = nullptr;
    int prec = PHG_FP64;
    int dev = 0;
    cudaStream_t stream = nullptr;
    int V = 0, rs = 0, os = 0, W = 0;
    DBuf inner, outer, p2io, isb;
    DBuf pcol;                       // shared rs x rs pattern (W x rs)
    SolveOpBufs ML, L, MJ;           // mass (Laplace), Laplacian, mass (Jacobian)
    MgBufs mgL;                      // multigrid hierarchy preconditioning L
    DBuf vd1, vd2, vd1c, vd2c;
    ColsBufs bnd2, bnd3, d1b, d2b, d1cb, d2cb;
    JacOps J;
    // element-loop geometry of the FP32 Jacobian right-hand sides (mixed time steps)
    DBuf jq_ring, jq_rxy, jq_cs, jq_split;
    JacQuadDev jq;
    // which Picard iterations of a mixed-precision step use it: 2 (the default)
    // every iteration of a barotropic step but the last, whose Jacobian is the
    // assembled FP64 product, so the step's result carries no FP32 Jacobian
    // error beyond what the Picard contraction leaves of the earlier ones
    // (measured: <= 2e-9 relative on strongly nonlinear level-2..4 states, 1e-7
    // with the quadrature in every iteration); 1 every iteration, barotropic and
    // baroclinic; 0 never (PHG_JAC_QUAD at creation)
    int jq_mode = 0;
    DBuf ncol, nval;                 // V x V norm matrix (its own pattern)
    DevEll norm;
    int restart = 30, max_iter = 20000;
    double tol = 1e-12;
    int max_sms = 0;                 // SMs the persistent solver may fill (0 = all)
    long long wait_limit = 0;        // barrier wait limit of the persistent solvers (0 = default ~1 s)
    // scratch
    DBuf work, stats, s_a, s_b, s_c, s_d, s_e, s_part, s_out;
    GmresStats last{};
    bool stats_pending = false;
    int pending_slots = 0;           // stats slots written since the last check
    // staging for host pointers
    DBuf st[8];
    // solver-launch profiling
    bool prof = false;
    std::vector<cudaEvent_t> ev;
    std::vector<int> ev_family;      // solver family of each recorded launch
    int nev = 0;
    DBuf hist;
    ~phg_ops_s() { for (auto e : ev) cudaEventDestroy(e); }

    DevEll ell(const DBuf &vals) const { DevEll e; e.n = rs; e.W = W; e.col = pcol.as<int>(); e.val = vals.as<double>(); return e; }
    const int *imap() const { return inner.as<int>(); }
    const int *bmap() const { return outer.as<int>(); }
    cudaStream_t str(void *s) const { return s ? (cudaStream_t)s : stream; }
};

namespace {

int env_int(const char *name, int dflt);

// Real interval holding the spectrum of D^-1 A, or false when it is not a
// small one (then the solver keeps GMRES).  Upper end: Gershgorin (the rows
// of D^-1 A have unit diagonal, so Re(lambda) <= 1 + max off-diagonal row
// sum).  Lower end: power iteration on lmax I - D^-1 A, which approaches
// lmax - lmin from below, so the estimate of lmin is high; 0.9 of it is used.
bool cheb_interval(const Csr &c, const std::vector<double> &dinv, double &lmin, double &lmax) {
    const int n = c.n;
    if (n < 2) return false;
    double g = 0.0;
    for (int i = 0; i < n; ++i) {
        double r = 0.0;
        for (int q = c.ptr[i]; q < c.ptr[i + 1]; ++q)
            if (c.col[q] != i) r += std::fabs(c.val[q]);
        g = std::max(g, 1.0 + r * std::fabs(dinv[i]));
    }
    std::vector<double> v(n), w(n);
    uint64_t st = 0x9e3779b97f4a7c15ULL;
    for (int i = 0; i < n; ++i) {
        st = st * 6364136223846793005ULL + 1442695040888963407ULL;
        v[i] = (double)(st >> 11) / 9007199254740992.0 - 0.5;
    }
    double mu = 0.0;
    for (int it = 0; it < 100; ++it) {
        double nv = 0.0, num = 0.0;
        for (int i = 0; i < n; ++i) {
            double s = 0.0;
            for (int q = c.ptr[i]; q < c.ptr[i + 1]; ++q) s += c.val[q] * v[c.col[q]];
            w[i] = g * v[i] - dinv[i] * s;
        }
        for (int i = 0; i < n; ++i) { num += v[i] * w[i]; nv += v[i] * v[i]; }
        mu = num / nv;
        double nw = 0.0;
        for (int i = 0; i < n; ++i) nw += w[i] * w[i];
        nw = std::sqrt(nw);
        if (!(nw > 0.0)) return false;
        for (int i = 0; i < n; ++i) v[i] = w[i] / nw;
    }
    const double est = g - mu;
    if (!(est > 0.05 * g)) return false;
    lmin = 0.9 * est;
    lmax = g;
    return true;
}

int build_solve_op(phg_ops_s *o, const Csr &c, SolveOpBufs &b, bool try_cheb = false) {
    std::vector<double> v;
    to_ell(c, o->W, nullptr, v);
    std::vector<double> dinv(o->rs, 0.0), as64(v.size());
    std::vector<float> as32(v.size()), a32(v.size());
    for (int i = 0; i < c.n; ++i)
        for (int q = c.ptr[i]; q < c.ptr[i + 1]; ++q)
            if (c.col[q] == i) dinv[i] = 1.0 / c.val[q];
    for (int i = 0; i < o->rs; ++i)
        if (!(dinv[i] != 0.0) || !std::isfinite(dinv[i])) return fail(PHG_ERR_ARG, "zero diagonal in row %d", i);
    const int n = o->rs;
    std::vector<int> col;
    to_ell(c, o->W, &col, v);
    for (size_t e = 0; e < v.size(); ++e) {
        as64[e] = v[e] * dinv[col[e]];
        as32[e] = (float)as64[e];
        a32[e] = (float)v[e];
    }
    if (o->W <= 8) {   // row records: slot k of row i at pk[8 i + k], padding = (i, 0)
        std::vector<unsigned> pk(16 * (size_t)n);
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 8; ++k) {
                const bool real = k < o->W;
                const float a = real ? a32[(size_t)k * n + i] : 0.0f;
                unsigned bits;
                memcpy(&bits, &a, sizeof bits);
                pk[16 * (size_t)i + 2 * k] = (unsigned)(real ? col[(size_t)k * n + i] : i);
                pk[16 * (size_t)i + 2 * k + 1] = bits;
            }
        CK(upload(b.pk, pk));
    }
    CK(upload(b.val, v)); CK(upload(b.as64, as64)); CK(upload(b.as32, as32)); CK(upload(b.a32, a32));
    CK(upload(b.dinv, dinv)); CK(upload(b.dinv32, std::vector<float>(dinv.begin(), dinv.end())));
    b.op.A = o->ell(b.val);
    b.op.as64 = b.as64.as<double>(); b.op.as32 = b.as32.as<float>(); b.op.dinv = b.dinv.as<double>();
    b.op.a32 = b.a32.as<float>();
    b.op.dinv32 = b.dinv32.as<float>();
    b.op.pk32 = b.pk.p ? b.pk.as<uint4>() : nullptr;
    b.op.cheb_lmin = b.op.cheb_lmax = 0.0;
    if (try_cheb && o->W <= 8 && env_int("PHG_CHEB", 1)) {
        double lo = 0.0, hi = 0.0;
        if (cheb_interval(c, dinv, lo, hi)) { b.op.cheb_lmin = lo; b.op.cheb_lmax = hi; }
    }
    return PHG_OK;
}

int build_cols(const Csr &c, ColsBufs &b) {
    b.c = DevCols();
    b.c.n = c.n;
    if (c.nnz() == 0) return PHG_OK;
    CK(upload(b.ptr, c.ptr)); CK(upload(b.col, c.col)); CK(upload(b.val, c.val));
    b.c.ptr = b.ptr.as<int>(); b.c.col = b.col.as<int>(); b.c.val = b.val.as<double>();
    return PHG_OK;
}

int build_vals(phg_ops_s *o, const Csr &c, DBuf &b) {
    std::vector<double> v;
    to_ell(c, o->W, nullptr, v);
    CK(upload(b, v));
    return PHG_OK;
}

bool same_pattern(const Csr &a, const Csr &b) { return a.n == b.n && a.ptr == b.ptr && a.col == b.col; }

template <typename T>
std::vector<float> to_f32(const std::vector<T> &v) { return std::vector<float>(v.begin(), v.end()); }

int env_int(const char *name, int dflt) { const char *e = getenv(name); return e ? atoi(e) : dflt; }
double env_dbl(const char *name, double dflt) { const char *e = getenv(name); return e ? atof(e) : dflt; }

// Geometric multigrid for the Laplacian of a generated icosahedral mesh:
// levels down to the 42-point icosahedron refinement, Jacobi smoothing,
// coarse levels of at most `red_max` points solved per block in shared memory.
int build_mg_dev(phg_ops_s *o, phg_mesh_s *mh, SolveOpBufs &Lb, MgBufs &mb, int prec) {
    const Mesh &m = mh->m;
    Lb.op.mg = MgDev();
    if (env_int("PHG_MG", 1) == 0 || m.level < 3) return PHG_OK;
    std::string err;
    const MgHierarchy *hp = mh->hierarchy(err);
    if (!hp) return fail(PHG_ERR_ARG, "multigrid: %s", err.c_str());
    const MgHierarchy &h = *hp;
    const int nlev = (int)h.A.size();
    if (nlev > MG_MAXLEV) return PHG_OK;
    MgDev &mg = Lb.op.mg;
    mg.nlev = nlev;
    // one damped-Jacobi sweep before and after the coarse correction: at
    // these sizes a V-cycle is latency-bound (group barriers), so cheap
    // cycles win over strong ones (measured: nu 1 / omega 0.9 beats 2 / 0.7)
    mg.omega = env_dbl("PHG_MG_OMEGA", 0.9);
    mg.nu1 = env_int("PHG_MG_NU", 1);
    mg.nu2 = mg.nu1;
    const size_t es = prec == PHG_MIXED ? 4 : 8;
    // levels of at most red_max points run redundantly per block in shared
    // memory, the larger ones with group barriers; with the arrival-count
    // barrier the 641-point level is cheaper in parallel (L6 step mixed
    // 5.30 -> 5.20 ms, FP64 6.35 -> 6.06 ms, baroclin +5 %), so only the
    // 161-point level and the dense coarsest one stay redundant
    const int red_max = env_int("PHG_MG_REDUNDANT", 200);
    // shared memory: the solver's own ~21 KB plus 4 vectors per redundant level
    const size_t smem_cap = 200 * 1024;
    int nred = nlev - 1;
    size_t used = 0;
    for (int l = nlev - 1; l >= 1; --l) {
        const int n = l == 0 ? m.rs : h.mesh[l].rs;
        if (n > red_max || 21 * 1024 + es * (used + 4 * (size_t)n) > smem_cap) break;
        used += 4 * (size_t)n;
        nred = l;
    }
    mg.nred = nred;
    mb.lev.clear();
    for (int l = 0; l < nlev; ++l) {
        mb.lev.emplace_back(new MgLevelBufs());
        MgLevelBufs &B = *mb.lev.back();
        MgLevelDev &D = mg.lev[l];
        if (l == 0) {
            D.n = o->rs; D.W = o->W; D.col = o->pcol.as<int>();
            D.a64 = Lb.op.A.val; D.a32 = Lb.op.a32; D.d64 = Lb.op.dinv;
            std::vector<double> dd(o->rs);
            CK(cudaMemcpy(dd.data(), Lb.op.dinv, 8 * dd.size(), cudaMemcpyDeviceToHost));
            CK(upload(B.d32, to_f32(dd)));
            D.d32 = B.d32.as<float>();
        } else {
            const Csr &A = h.A[l];
            int W = 0;
            for (int i = 0; i < A.n; ++i) W = std::max(W, A.ptr[i + 1] - A.ptr[i]);
            std::vector<int> col;
            std::vector<double> val, dinv(A.n, 0.0);
            to_ell(A, W, &col, val);
            for (int i = 0; i < A.n; ++i)
                for (int q = A.ptr[i]; q < A.ptr[i + 1]; ++q)
                    if (A.col[q] == i) dinv[i] = 1.0 / A.val[q];
            CK(upload(B.col, col)); CK(upload(B.a64, val)); CK(upload(B.a32, to_f32(val)));
            CK(upload(B.d64, dinv)); CK(upload(B.d32, to_f32(dinv)));
            D.n = A.n; D.W = W; D.col = B.col.as<int>();
            D.a64 = B.a64.as<double>(); D.a32 = B.a32.as<float>();
            D.d64 = B.d64.as<double>(); D.d32 = B.d32.as<float>();
        }
        if (l + 1 < nlev) {
            const Csr &P = h.P[l], &R = h.R[l];
            std::vector<int> pc(2 * (size_t)P.n, -1);
            std::vector<double> pw(2 * (size_t)P.n, 0.0);
            for (int i = 0; i < P.n; ++i)
                for (int q = P.ptr[i], k = 0; q < P.ptr[i + 1] && k < 2; ++q, ++k) {
                    pc[2 * i + k] = P.col[q];
                    pw[2 * i + k] = P.val[q];
                }
            int Wr = 0;
            for (int c = 0; c < R.n; ++c) Wr = std::max(Wr, R.ptr[c + 1] - R.ptr[c]);
            std::vector<int> rf((size_t)Wr * R.n, -1);
            std::vector<double> rw((size_t)Wr * R.n, 0.0);
            for (int c = 0; c < R.n; ++c)
                for (int q = R.ptr[c], k = 0; q < R.ptr[c + 1]; ++q, ++k) {
                    rf[(size_t)k * R.n + c] = R.col[q];
                    rw[(size_t)k * R.n + c] = R.val[q];
                }
            CK(upload(B.pc, pc)); CK(upload(B.pw64, pw)); CK(upload(B.pw32, to_f32(pw)));
            CK(upload(B.rf, rf)); CK(upload(B.rw64, rw)); CK(upload(B.rw32, to_f32(rw)));
            D.pc = B.pc.as<int>(); D.pw64 = B.pw64.as<double>(); D.pw32 = B.pw32.as<float>();
            D.Wr = Wr; D.rf = B.rf.as<int>(); D.rw64 = B.rw64.as<double>(); D.rw32 = B.rw32.as<float>();
        }
    }
    CK(upload(mb.cinv64, h.coarse_inv));
    CK(upload(mb.cinv32, to_f32(h.coarse_inv)));
    mg.nc = h.A[nlev - 1].n;
    mg.cinv64 = mb.cinv64.as<double>();
    mg.cinv32 = mb.cinv32.as<float>();
    size_t e = 0;
    for (int l = nred; l < nlev; ++l) { mg.red_off[l] = (int)e; e += 4 * (size_t)mg.lev[l].n; }
    mg.red_elems = e;
    mg.group_elems = 0;
    for (int l = 0; l < nred; ++l) mg.group_elems += 4 * (size_t)mg.lev[l].n;
    // cluster tail: the parallel levels of at most cl_rows rows (never the
    // finest) run in one cluster of cl CTAs, as long as a CTA's share of their
    // four vectors keeps two blocks per SM within the shared memory.  Off by
    // default (PHG_MG_CLUSTER=8 turns it on): measured on the level-6 step, the
    // tail is bit-identical but slower -- 5.23 -> 5.34 ms mixed with levels
    // <= 2561 rows in the cluster, 6.01 ms with levels <= 10241 rows (8 CTAs
    // then stream a level's matrix and restriction through L2 alone), 5.38 ms
    // with the 641-row level only: the cluster barrier (~400 cycles) and
    // distributed shared memory loads (~250 cycles) save less than the entry
    // handshake and the serialised restriction into the tail cost.
    mg.ncl = nred;
    mg.cl_size = 0;
    mg.cl_elems = 0;
    {
        const int cl = env_int("PHG_MG_CLUSTER", 0);
        const int cl_rows = env_int("PHG_MG_CLUSTER_ROWS", 12000);
        if (cl >= 2 && cl <= 16) {
            int ncl = nred;
            size_t elems = 0;
            for (int l = nred - 1; l >= 1; --l) {
                const int n = mg.lev[l].n;
                const size_t ch = ((size_t)n + cl - 1) / cl;
                if (n > cl_rows || 21 * 1024 + es * (e + elems + 4 * ch) > 100 * 1024) break;
                elems += 4 * ch;
                ncl = l;
            }
            bool exact = true;
            for (int l = ncl; l < nred && exact; ++l) {
                const int n = mg.lev[l].n, ch = (n + cl - 1) / cl;
                const unsigned magic = (unsigned)((0x100000000ULL + ch - 1) / ch);
                for (int i = 0; i < n && exact; ++i)
                    exact = (int)(((unsigned long long)(unsigned)i * magic) >> 32) == i / ch;
                mg.cl_chunk[l] = ch;
                mg.cl_magic[l] = magic;
            }
            if (exact && ncl < nred) {
                size_t off = 0;
                for (int l = ncl; l < nred; ++l) { mg.cl_off[l] = (int)off; off += 4 * (size_t)mg.cl_chunk[l]; }
                mg.ncl = ncl;
                mg.cl_size = cl;
                mg.cl_elems = off;
            }
        }
    }
    CK(mb.desc.ensure(sizeof(MgDev)));
    CK(cudaMemcpy(mb.desc.p, &mg, sizeof(MgDev), cudaMemcpyHostToDevice));
    Lb.op.mgd = mb.desc.as<MgDev>();
    return PHG_OK;
}

}  // namespace

extern "C" int phg_ops_create(phg_mesh h, int precision, phg_ops *out) {
    PHG_API_BEGIN
    if (!h || !out) return fail(PHG_ERR_ARG, "NULL argument");
    if (precision != PHG_FP64 && precision != PHG_MIXED) return fail(PHG_ERR_ARG, "bad precision %d", precision);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(PHG_ERR_CUDA, "no CUDA device");
    }
    h->assemble();
    const Mesh &m = h->m;
    const SphereOps &so = h->ops;
    if (m.rs < 1) return fail(PHG_ERR_ARG, "mesh has no inner points");
    const Csr *shared[] = {&so.lapl, &so.jidt, &so.d1, &so.d2, &so.d1c, &so.d2c};
    for (const Csr *c : shared)
        if (!same_pattern(so.idt, *c)) return fail(PHG_ERR_ARG, "operators do not share one pattern");
    auto o = std::make_unique<phg_ops_s>();
    o->mesh = h;
    o->prec = precision;
    CK(cudaGetDevice(&o->dev));
    CK(cudaStreamCreateWithFlags(&o->stream, cudaStreamNonBlocking));
    lockstep_prepare();
    o->V = m.V; o->rs = m.rs; o->os = m.os;
    int W = 0;
    for (int i = 0; i < m.rs; ++i) W = std::max(W, so.idt.ptr[i + 1] - so.idt.ptr[i]);
    o->W = W;
    std::vector<int> col;
    std::vector<double> tmp;
    to_ell(so.idt, W, &col, tmp);
    CK(upload(o->pcol, col));
    CK(upload(o->inner, m.inner)); CK(upload(o->outer, m.outer.empty() ? std::vector<int>{0} : m.outer));
    CK(upload(o->p2io, m.p2io)); CK(upload(o->isb, m.bnd));
    int r;
    if ((r = build_solve_op(o.get(), so.idt, o->ML, true))) return r;
    if ((r = build_solve_op(o.get(), so.lapl, o->L))) return r;
    if ((r = build_mg_dev(o.get(), h, o->L, o->mgL, precision))) return r;
    if ((r = build_solve_op(o.get(), so.jidt, o->MJ, true))) return r;
    if ((r = build_vals(o.get(), so.d1, o->vd1)) || (r = build_vals(o.get(), so.d2, o->vd2)) ||
        (r = build_vals(o.get(), so.d1c, o->vd1c)) || (r = build_vals(o.get(), so.d2c, o->vd2c)))
        return r;
    if ((r = build_cols(so.bnd2, o->bnd2)) || (r = build_cols(so.bnd3, o->bnd3)) ||
        (r = build_cols(so.d1b, o->d1b)) || (r = build_cols(so.d2b, o->d2b)) ||
        (r = build_cols(so.d1cb, o->d1cb)) || (r = build_cols(so.d2cb, o->d2cb)))
        return r;
    o->J.d1 = o->ell(o->vd1); o->J.d2 = o->ell(o->vd2); o->J.d1c = o->ell(o->vd1c); o->J.d2c = o->ell(o->vd2c);
    o->J.d1b = o->d1b.c; o->J.d2b = o->d2b.c; o->J.d1cb = o->d1cb.c; o->J.d2cb = o->d2cb.c;
    {
        JacQuadHost jh;
        build_jac_quad(m, jh);
        if (jh.max_tri <= 6) {   // the kernel's 8-lane rows take closed rings of at most 6 triangles
            CK(upload(o->jq_ring, jh.ring)); CK(upload(o->jq_rxy, jh.rxy)); CK(upload(o->jq_cs, jh.cs0));
            o->jq.n = m.rs;
            o->jq.ring = o->jq_ring.as<int>();
            o->jq.rxy = (const float2 *)o->jq_rxy.p;
            o->jq.cs0 = (const float2 *)o->jq_cs.p;
            o->jq_mode = precision == PHG_MIXED ? env_int("PHG_JAC_QUAD", 2) : 0;
        }
    }
    // norm matrix: V x V on its own pattern
    int Wn = 0;
    for (int i = 0; i < m.V; ++i) Wn = std::max(Wn, so.norm.ptr[i + 1] - so.norm.ptr[i]);
    std::vector<int> ncol;
    std::vector<double> nval;
    {
        Csr c = so.norm;
        ncol.assign((size_t)Wn * m.V, 0);
        nval.assign((size_t)Wn * m.V, 0.0);
        for (int i = 0; i < m.V; ++i) {
            int k = 0;
            for (int q = c.ptr[i]; q < c.ptr[i + 1]; ++q, ++k) {
                ncol[(size_t)k * m.V + i] = c.col[q];
                nval[(size_t)k * m.V + i] = c.val[q];
            }
            for (; k < Wn; ++k) ncol[(size_t)k * m.V + i] = i;
        }
    }
    CK(upload(o->ncol, ncol)); CK(upload(o->nval, nval));
    o->norm.n = m.V; o->norm.W = Wn; o->norm.col = o->ncol.as<int>(); o->norm.val = o->nval.as<double>();
    CK(o->stats.ensure(sizeof(GmresStats) * 64));
    CK(cudaMemset(o->stats.p, 0, sizeof(GmresStats) * 64));
    h->refs++;
    *out = o.release();
    return PHG_OK;
    PHG_API_END
}

static void ops_release(phg_ops o) {
    if (!o || o->refs.fetch_sub(1) != 1) return;
    if (o->stream) { cudaStreamSynchronize(o->stream); cudaStreamDestroy(o->stream); }
    phg_mesh_s *m = o->mesh;
    delete o;
    mesh_release(m);
}

extern "C" void phg_ops_destroy(phg_ops o) { PHG_API_BEGIN ops_release(o); PHG_API_END_VOID }

extern "C" int phg_ops_set_solver(phg_ops o, int restart, double tol, int max_iter) {
    PHG_API_BEGIN
    if (!o) return fail(PHG_ERR_ARG, "NULL handle");
    if (restart < 1 || restart > 48) return fail(PHG_ERR_ARG, "restart must be in 1..48");
    if (!(tol > 0) || max_iter < 1) return fail(PHG_ERR_ARG, "bad tolerance / iteration cap");
    o->restart = restart; o->tol = tol; o->max_iter = max_iter;
    return PHG_OK;
    PHG_API_END
}

namespace {

Precision prec_of(const phg_ops_s *o) { return o->prec == PHG_MIXED ? PREC_MIXED : PREC_FP64; }

// enqueue one solve; stats go to slot `slot` of the handle's device stats array
int solve(phg_ops_s *o, const DevSolveOp &op, const double *B, double *X, int nv, int ld, double tol,
          int slot, cudaStream_t s) {
    NvtxRange nvtx("phg:solve");
    if (slot < 0 || (size_t)(slot + 1) * sizeof(GmresStats) > o->stats.n)
        return fail(PHG_ERR_ARG, "solve record slot %d beyond the handle's %zu", slot, o->stats.n / sizeof(GmresStats));
    size_t need = gmres_work_bytes(op, nv, o->restart, prec_of(o));
    if (need > o->work.n) {
        CK(cudaStreamSynchronize(s));
        CK(o->work.ensure(need));
    }
    const bool rec = o->prof && o->nev + 2 <= (int)o->ev.size();
    if (rec) CK(cudaEventRecord(o->ev[o->nev], s));
    CK(gmres_solve(op, B, X, nv, ld, o->restart, o->max_iter, tol, prec_of(o), o->work.p,
                   o->stats.as<GmresStats>() + slot, s, false, o->max_sms, nullptr, o->wait_limit));
    if (rec) {
        o->ev_family[o->nev / 2] = solve_family(op);
        CK(cudaEventRecord(o->ev[o->nev + 1], s));
        CK(cudaMemcpyAsync(o->hist.as<GmresStats>() + o->nev / 2, o->stats.as<GmresStats>() + slot,
                           sizeof(GmresStats), cudaMemcpyDeviceToDevice, s));
        o->nev += 2;
    }
    o->stats_pending = true;
    o->pending_slots = std::max(o->pending_slots, slot + 1);
    return PHG_OK;
}

// maximum that keeps a NaN (std::max drops one on the right)
double max_keep_nan(double a, double b) { return a != a ? a : (b != b ? b : std::max(a, b)); }

// read back and check the stats of slots [0, nslots)
int check_stats(phg_ops_s *o, int nslots, cudaStream_t s, GmresStats *agg = nullptr, GmresStats *each = nullptr) {
    nslots = std::min<int>(nslots, (int)(o->stats.n / sizeof(GmresStats)));
    std::vector<GmresStats> st(nslots);
    CK(cudaMemcpyAsync(st.data(), o->stats.p, sizeof(GmresStats) * nslots, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    GmresStats a{0.0, 0.0, 0, 0, 0, 0};
    for (auto &x : st) {
        a.iters += x.iters; a.cycles += x.cycles;
        a.relres = max_keep_nan(a.relres, x.relres);
        a.status = std::max(a.status, x.status);
    }
    if (each) memcpy(each, st.data(), sizeof(GmresStats) * nslots);
    o->last = a;
    o->stats_pending = false;
    o->pending_slots = 0;
    if (agg) *agg = a;
    if (a.status == 2) return fail(PHG_ERR_TIMEOUT, "device barrier wait timed out");
    if (!std::isfinite(a.relres) || (a.status == 1 && !(a.relres <= std::max(1e3 * o->tol, 1e-8))))
        return fail(PHG_ERR_NOT_CONVERGED, "GMRES stopped at relative residual %.3e", a.relres);
    return PHG_OK;
}

// host/device argument staging
struct Stage {
    phg_ops_s *o;
    cudaStream_t s;
    bool host = false;
    int next = 0;
    struct Out { double *host; double *dev; size_t n; };
    std::vector<Out> outs;
    Stage(phg_ops_s *o_, cudaStream_t s_) : o(o_), s(s_) {}
    cudaError_t in(const double *p, size_t n, const double **dp) {
        if (!p || is_device_ptr(p)) { *dp = p; return cudaSuccess; }
        host = true;
        DBuf &b = o->st[next++];
        cudaError_t e = b.ensure(8 * n);
        if (e != cudaSuccess) return e;
        *dp = b.as<double>();
        return cudaMemcpyAsync(b.p, p, 8 * n, cudaMemcpyHostToDevice, s);
    }
    cudaError_t out(double *p, size_t n, double **dp) {
        if (is_device_ptr(p)) { *dp = p; return cudaSuccess; }
        host = true;
        DBuf &b = o->st[next++];
        cudaError_t e = b.ensure(8 * n);
        if (e != cudaSuccess) return e;
        *dp = b.as<double>();
        outs.push_back({p, b.as<double>(), n});
        return cudaSuccess;
    }
    cudaError_t finish() {
        for (auto &x : outs) {
            cudaError_t e = cudaMemcpyAsync(x.host, x.dev, 8 * x.n, cudaMemcpyDeviceToHost, s);
            if (e != cudaSuccess) return e;
        }
        return host ? cudaStreamSynchronize(s) : cudaSuccess;
    }
};

double mass_tol(const phg_ops_s *o) { return std::min(o->tol, 1e-14); }

// ans (rs) = M_L^{-1} (L F_in + B3 F_bnd) for nv members of full vectors F;
// the mass solve runs to `tol` (standalone applies: 1e-14, time steps: the
// handle's tolerance)
int laplace_calc2_dev(phg_ops_s *o, double *ans, int lda, const double *F, int ldf, int nv, int slot, cudaStream_t s,
                      double tol) {
    CK(o->s_a.ensure(8 * (size_t)o->rs * nv));
    double *rhs = o->s_a.as<double>();
    CK(apply_op(o->L.op.A, o->bnd3.c, F, ldf, o->imap(), F, ldf, o->bmap(), rhs, o->rs, nv, s));
    for (int v = 0; v < nv; ++v) CK(cudaMemsetAsync(ans + (size_t)v * lda, 0, 8 * (size_t)o->rs, s));
    return solve(o, o->ML.op, rhs, ans, nv, lda, tol, slot, s);
}

// the 8 derivative solves of a Jacobian for nv members; sol: nv x 8 x rs.
// quad: right-hand sides by the FP32 element-loop quadrature (the mixed
// precision time steps) instead of the assembled FP64 operators.  warm: the
// solves start from sol's contents (the previous Picard iteration's
// derivatives of the same step) instead of zero
int jacobian_derivs_dev(phg_ops_s *o, const double *u, const double *v, int ld, double *sol, int nv, int slot,
                        cudaStream_t s, double tol, bool quad = false, bool warm = false) {
    CK(o->s_b.ensure(8 * (size_t)o->rs * 8 * nv));
    double *rhs = o->s_b.as<double>();
    if (quad && o->jq.n) {
        CK(o->jq_split.ensure(16 * (size_t)o->V * nv));
        CK(jac_quad(o->jq, o->J, u, v, ld, o->imap(), o->bmap(), rhs, o->rs, nv, o->V, (float2 *)o->jq_split.p, s));
    }
    else CK(jac_rhs(o->J, u, v, ld, o->imap(), o->bmap(), rhs, o->rs, nv, s));
    if (!warm) CK(cudaMemsetAsync(sol, 0, 8 * (size_t)o->rs * 8 * nv, s));
    return solve(o, o->MJ.op, rhs, sol, 8 * nv, o->rs, tol, slot, s);
}

int norm_dev(phg_ops_s *o, const double *u, const double *v, int nv, double *out_dev, bool dist, bool take_sqrt,
             cudaStream_t s) {
    const int V = o->V;
    CK(o->s_d.ensure(8 * (size_t)V * nv * 2));
    double *diff = o->s_d.as<double>(), *y = diff + (size_t)V * nv;
    const double *x = u;
    if (dist) { CK(vsub(diff, u, v, (long long)V * nv, s)); x = diff; }
    CK(apply_op(o->norm, DevCols(), x, V, nullptr, nullptr, 0, nullptr, y, V, nv, s));
    CK(o->s_part.ensure(8 * (size_t)nv * dot_chunks(V)));
    const double *a = dist ? x : u;
    const double *bb = dist ? y : y;
    if (!dist && v) {  // scalar(u, v) = u . (NORM v)
        CK(apply_op(o->norm, DevCols(), v, V, nullptr, nullptr, 0, nullptr, y, V, nv, s));
        a = u;
    }
    CK(dot(a, bb, V, V, nv, o->s_part.as<double>(), out_dev, take_sqrt, s));
    return PHG_OK;
}

}  // namespace

extern "C" int phg_ops_set_sms(phg_ops o, int max_sms) {
    PHG_API_BEGIN
    if (!o || max_sms < 0) return fail(PHG_ERR_ARG, "bad argument");
    o->max_sms = max_sms;
    return PHG_OK;
    PHG_API_END
}

extern "C" int phg_ops_set_wait_limit(phg_ops o, long long cycles) {
    PHG_API_BEGIN
    if (!o || cycles < 0) return fail(PHG_ERR_ARG, "bad argument");
    o->wait_limit = cycles;
    return PHG_OK;
    PHG_API_END
}

extern "C" int phg_ops_last_solve(phg_ops o, int *iters, int *cycles, double *relres) {
    PHG_API_BEGIN
    if (!o) return fail(PHG_ERR_ARG, "NULL handle");
    if (iters) *iters = o->last.iters;
    if (cycles) *cycles = o->last.cycles;
    if (relres) *relres = o->last.relres;
    return PHG_OK;
    PHG_API_END
}

extern "C" int phg_ops_profile(phg_ops o, int enable) {
    PHG_API_BEGIN
    if (!o) return fail(PHG_ERR_ARG, "NULL handle");
    if (enable && o->ev.empty()) {
        o->ev.resize(8192);
        o->ev_family.assign(4096, -1);
        for (auto &e : o->ev) CK(cudaEventCreate(&e));
        CK(o->hist.ensure(sizeof(GmresStats) * 4096));
    }
    CK(cudaStreamSynchronize(o->stream));
    o->prof = enable != 0;
    if (enable) o->nev = 0;
    return PHG_OK;
    PHG_API_END
}

extern "C" int phg_ops_profile_read_family(phg_ops o, int family, int *launches, double *ms, double *bytes) {
    PHG_API_BEGIN
    if (!o) return fail(PHG_ERR_ARG, "NULL handle");
    const int n = o->nev / 2;
    double t = 0.0, b = 0.0;
    int cnt = 0;
    if (n > 0) {
        CK(cudaEventSynchronize(o->ev[o->nev - 1]));
        std::vector<GmresStats> h(n);
        CK(cudaMemcpy(h.data(), o->hist.p, sizeof(GmresStats) * n, cudaMemcpyDeviceToHost));
        for (int k = 0; k < n; ++k) {
            if (family >= 0 && o->ev_family[k] != family) continue;
            float dt = 0.f;
            CK(cudaEventElapsedTime(&dt, o->ev[2 * k], o->ev[2 * k + 1]));
            t += dt;
            b += h[k].bytes;
            ++cnt;
        }
    }
    if (launches) *launches = cnt;
    if (ms) *ms = t;
    if (bytes) *bytes = b;
    return PHG_OK;
    PHG_API_END
}

extern "C" int phg_ops_profile_read(phg_ops o, int *launches, double *ms, double *bytes) {
    PHG_API_BEGIN
    return phg_ops_profile_read_family(o, -1, launches, ms, bytes);
    PHG_API_END
}

extern "C" int phg_laplace_calc2(phg_ops o, double *ans, const double *F, void *stream) {
    PHG_API_BEGIN
    if (!o || !ans || !F) return fail(PHG_ERR_ARG, "NULL argument");
    cudaStream_t s = o->str(stream);
    Stage st(o, s);
    const double *dF; double *dA;
    CK(st.in(F, o->V, &dF)); CK(st.out(ans, o->rs, &dA));
    int r = laplace_calc2_dev(o, dA, o->rs, dF, o->V, 1, 0, s, mass_tol(o));
    if (r) return r;
    CK(st.finish());
    return st.host ? check_stats(o, 1, s) : PHG_OK;
    PHG_API_END
}

extern "C" int phg_laplace_calc1(phg_ops o, double *ans, const double *F, const double *bnd, void *stream) {
    PHG_API_BEGIN
    if (!o || !ans || !F) return fail(PHG_ERR_ARG, "NULL argument");
    cudaStream_t s = o->str(stream);
    Stage st(o, s);
    const double *dF, *dB; double *dA;
    CK(st.in(F, o->V, &dF)); CK(st.in(bnd, o->os, &dB)); CK(st.out(ans, o->V, &dA));
    CK(o->s_c.ensure(8 * (size_t)o->rs));
    int r = laplace_calc2_dev(o, o->s_c.as<double>(), o->rs, dF, o->V, 1, 0, s, mass_tol(o));
    if (r) return r;
    CK(p2u(dA, o->V, o->s_c.as<double>(), o->rs, dB, o->os, o->p2io.as<int>(), o->isb.as<int>(), o->V, 1, s));
    CK(st.finish());
    return st.host ? check_stats(o, 1, s) : PHG_OK;
    PHG_API_END
}

extern "C" int phg_laplace_solve(phg_ops o, double *ans, const double *F, const double *bnd, void *stream) {
    PHG_API_BEGIN
    if (!o || !ans || !F) return fail(PHG_ERR_ARG, "NULL argument");
    cudaStream_t s = o->str(stream);
    Stage st(o, s);
    const double *dF, *dB; double *dA;
    CK(st.in(F, o->V, &dF)); CK(st.in(bnd, o->os, &dB)); CK(st.out(ans, o->V, &dA));
    CK(o->s_a.ensure(8 * (size_t)o->rs)); CK(o->s_c.ensure(8 * (size_t)o->rs));
    double *b = o->s_a.as<double>(), *x = o->s_c.as<double>();
    // b = M_L F_in + B2 bnd
    CK(apply_op(o->ML.op.A, o->bnd2.c, dF, o->V, o->imap(), dB, o->os, nullptr, b, o->rs, 1, s));
    CK(cudaMemsetAsync(x, 0, 8 * (size_t)o->rs, s));
    int r = solve(o, o->L.op, b, x, 1, o->rs, o->tol, 0, s);
    if (r) return r;
    CK(p2u(dA, o->V, x, o->rs, dB, o->os, o->p2io.as<int>(), o->isb.as<int>(), o->V, 1, s));
    CK(st.finish());
    return st.host ? check_stats(o, 1, s) : PHG_OK;
    PHG_API_END
}

extern "C" int phg_laplace_solve_batch(phg_ops o, int nv, double *ans, const double *F, const double *bnd,
                                       void *stream) {
    PHG_API_BEGIN
    if (!o || !ans || !F || nv < 1) return fail(PHG_ERR_ARG, "NULL argument");
    cudaStream_t s = o->str(stream);
    Stage st(o, s);
    const int V = o->V, rs = o->rs, os = o->os;
    const double *dF, *dB; double *dA;
    CK(st.in(F, (size_t)V * nv, &dF)); CK(st.in(bnd, (size_t)os * nv, &dB)); CK(st.out(ans, (size_t)V * nv, &dA));
    if (os == 0) dB = nullptr;
    CK(o->s_a.ensure(8 * (size_t)rs * nv)); CK(o->s_c.ensure(8 * (size_t)rs * nv));
    double *b = o->s_a.as<double>(), *x = o->s_c.as<double>();
    CK(apply_op(o->ML.op.A, o->bnd2.c, dF, V, o->imap(), dB, os, nullptr, b, rs, nv, s));
    CK(cudaMemsetAsync(x, 0, 8 * (size_t)rs * nv, s));
    int r = solve(o, o->L.op, b, x, nv, rs, o->tol, 0, s);
    if (r) return r;
    CK(p2u(dA, V, x, rs, dB, os, o->p2io.as<int>(), o->isb.as<int>(), V, nv, s));
    CK(st.finish());
    return st.host ? check_stats(o, 1, s) : PHG_OK;
    PHG_API_END
}

extern "C" int phg_laplace_solve_levels(int count, const phg_ops *ops, const int *nv, double *const *ans,
                                        const double *const *F, const double *const *bnd, void *stream) {
    PHG_API_BEGIN
    if (count < 1 || count > 6 || !ops || !nv || !ans || !F) return fail(PHG_ERR_ARG, "bad argument (1 <= count <= 6)");
    phg_ops o0 = ops[0];
    for (int k = 0; k < count; ++k) {
        phg_ops o = ops[k];
        if (!o || nv[k] < 1 || !ans[k] || !F[k]) return fail(PHG_ERR_ARG, "bad argument for mesh %d", k);
        if (o->prec != o0->prec || o->dev != o0->dev) return fail(PHG_ERR_ARG, "handles of one precision and device only");
        if (!o->L.op.mgd) return fail(PHG_ERR_ARG, "mesh %d has no multigrid hierarchy", k);
    }
    cudaStream_t s = o0->str(stream);
    std::vector<Stage> st;
    st.reserve(count);
    std::vector<const DevSolveOp *> opk(count);
    std::vector<const double *> Bk(count), dB(count);
    std::vector<double *> Xk(count), dA(count);
    std::vector<int> ldk(count);
    for (int k = 0; k < count; ++k) {
        phg_ops o = ops[k];
        st.emplace_back(o, s);
        const int V = o->V, rs = o->rs, os = o->os, n = nv[k];
        const double *dF;
        CK(st[k].in(F[k], (size_t)V * n, &dF));
        CK(st[k].in(bnd ? bnd[k] : nullptr, (size_t)os * n, &dB[k]));
        CK(st[k].out(ans[k], (size_t)V * n, &dA[k]));
        if (os == 0) dB[k] = nullptr;
        CK(o->s_a.ensure(8 * (size_t)rs * n)); CK(o->s_c.ensure(8 * (size_t)rs * n));
        double *b = o->s_a.as<double>(), *x = o->s_c.as<double>();
        // b = M_L F_in + B2 bnd, x = 0 (src/impl/slaplace_impl.h:84-131)
        CK(apply_op(o->ML.op.A, o->bnd2.c, dF, V, o->imap(), dB[k], os, nullptr, b, rs, n, s));
        CK(cudaMemsetAsync(x, 0, 8 * (size_t)rs * n, s));
        opk[k] = &o->L.op; Bk[k] = b; Xk[k] = x; ldk[k] = rs;
    }
    const size_t need = gmres_multi_work_bytes(opk.data(), nv, count, o0->restart, prec_of(o0));
    if (need > o0->work.n) {
        CK(cudaStreamSynchronize(s));
        CK(o0->work.ensure(need));
    }
    CK(gmres_solve_multi(opk.data(), nv, Bk.data(), Xk.data(), ldk.data(), count, o0->restart, o0->max_iter,
                         o0->tol, prec_of(o0), o0->work.p, o0->stats.as<GmresStats>(), s, o0->max_sms,
                         o0->wait_limit));
    o0->stats_pending = true;
    o0->pending_slots = std::max(o0->pending_slots, 1);
    for (int k = 0; k < count; ++k) {
        phg_ops o = ops[k];
        CK(p2u(dA[k], o->V, Xk[k], o->rs, dB[k], o->os, o->p2io.as<int>(), o->isb.as<int>(), o->V, nv[k], s));
    }
    bool host = false;
    for (int k = 0; k < count; ++k) {
        CK(st[k].finish());
        host = host || st[k].host;
    }
    return host ? check_stats(o0, 1, s) : PHG_OK;
    PHG_API_END
}

// the handle's copy of a named inner x inner operator (FP64 values, and the
// FP32 copy where the mixed path keeps one)
static int named_op(phg_ops o, const char *name, const double **v64, const float **v32,
                    const unsigned **pk = nullptr) {
    struct { const char *n; const double *d; const float *f; const unsigned *p; } t[] = {
        {"idt", o->ML.op.A.val, o->ML.op.a32, o->ML.pk.as<unsigned>()},
        {"lapl", o->L.op.A.val, o->L.op.a32, o->L.pk.as<unsigned>()},
        {"jidt", o->MJ.op.A.val, o->MJ.op.a32, o->MJ.pk.as<unsigned>()}, {"d1", o->vd1.as<double>(), nullptr, nullptr},
        {"d2", o->vd2.as<double>(), nullptr, nullptr}, {"d1c", o->vd1c.as<double>(), nullptr, nullptr},
        {"d2c", o->vd2c.as<double>(), nullptr, nullptr}};
    for (auto &e : t)
        if (name && !strcmp(name, e.n)) {
            *v64 = e.d; *v32 = e.f;
            if (pk) *pk = e.p;
            return PHG_OK;
        }
    return fail(PHG_ERR_ARG, "unknown operator '%s'", name ? name : "(null)");
}

extern "C" int phg_ops_mult(phg_ops o, const char *name, double *y, const double *x, int nv, void *stream) {
    PHG_API_BEGIN
    if (!o || !y || !x || nv < 1) return fail(PHG_ERR_ARG, "NULL argument");
    const double *v64; const float *v32;
    int r = named_op(o, name, &v64, &v32);
    if (r) return r;
    cudaStream_t s = o->str(stream);
    Stage st(o, s);
    const double *dx; double *dy;
    CK(st.in(x, (size_t)o->rs * nv, &dx)); CK(st.out(y, (size_t)o->rs * nv, &dy));
    CK(spmm<double>(o->pcol.as<int>(), v64, o->rs, o->W, dx, o->rs, dy, o->rs, nv, s));
    CK(st.finish());
    return PHG_OK;
    PHG_API_END
}

extern "C" int phg_ops_mult32(phg_ops o, const char *name, float *y, const float *x, int nv, void *stream) {
    PHG_API_BEGIN
    if (!o || !y || !x || nv < 1) return fail(PHG_ERR_ARG, "NULL argument");
    if (!is_device_ptr(x) || !is_device_ptr(y)) return fail(PHG_ERR_ARG, "device pointers only");
    if (nv < 4 || nv > 256 || nv % 4 || ((nv / 4) & (nv / 4 - 1)) || ((uintptr_t)x & 15) || ((uintptr_t)y & 15))
        return fail(PHG_ERR_ARG, "nv must be 4 times a power of two, at most 256, and x, y 16-byte aligned");
    const double *v64; const float *v32; const unsigned *pk = nullptr;
    int r = named_op(o, name, &v64, &v32, &pk);
    if (r) return r;
    if (!v32) return fail(PHG_ERR_ARG, "no FP32 copy of '%s'", name);
    // row records where the operator has them (one matrix stream: 72 % of the HBM copy peak at level 8 x 64
    // vs 62 % for the slot-major arrays' 14 streams); the same bits either way
    if (pk) CK(spmm_pk32(pk, o->rs, x, y, nv, o->str(stream)));
    else CK(spmm_il32(o->pcol.as<int>(), v32, o->rs, o->W, x, y, nv, o->str(stream)));
    return PHG_OK;
    PHG_API_END
}

// --------------------------------------------------------- validation ---
extern "C" int phg_ops_validate(phg_ops o, long long *bad_entries, void *stream) {
    PHG_API_BEGIN
    if (!o || !bad_entries) return fail(PHG_ERR_ARG, "NULL argument");
    cudaStream_t s = o->str(stream);
    DBuf cnt;
    CK(cnt.ensure(sizeof(unsigned long long)));
    unsigned long long *bad = cnt.as<unsigned long long>();
    CK(cudaMemsetAsync(bad, 0, sizeof(unsigned long long), s));
    const int V = o->V, rs = o->rs, os = o->os;
    // the shared inner pattern and the index maps
    CK(check_range(o->pcol.as<int>(), (long long)o->W * rs, 0, rs, bad, s));
    CK(check_range(o->inner.as<int>(), rs, 0, V, bad, s));
    if (os > 0) CK(check_range(o->outer.as<int>(), os, 0, V, bad, s));
    CK(check_p2io(o->p2io.as<int>(), o->isb.as<int>(), V, rs, os, bad, s));
    // the norm matrix's own pattern
    CK(check_range(o->norm.col, (long long)o->norm.W * o->norm.n, 0, V, bad, s));
    // boundary columns (CSR over the inner rows, columns in [0, os))
    const ColsBufs *cols[] = {&o->bnd2, &o->bnd3, &o->d1b, &o->d2b, &o->d1cb, &o->d2cb};
    for (const ColsBufs *c : cols) {
        if (c->c.n <= 0 || !c->c.ptr) continue;
        int nnz = 0;
        CK(cudaMemcpyAsync(&nnz, c->c.ptr + c->c.n, sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        CK(check_ptr(c->c.ptr, c->c.n, nnz, bad, s));
        if (nnz > 0) CK(check_range(c->c.col, nnz, 0, std::max(os, 1), bad, s));
    }
    // the multigrid hierarchy of the Laplacian
    const MgDev &mg = o->L.op.mg;
    for (int l = 0; l < mg.nlev; ++l) {
        const MgLevelDev &D = mg.lev[l];
        CK(check_range(D.col, (long long)D.W * D.n, 0, D.n, bad, s));
        if (l + 1 < mg.nlev) {
            const int nc = mg.lev[l + 1].n;
            CK(check_range(D.pc, 2LL * D.n, -1, nc, bad, s));
            CK(check_range(D.rf, (long long)D.Wr * nc, -1, D.n, bad, s));
        }
    }
    unsigned long long h = 0;
    CK(cudaMemcpyAsync(&h, bad, sizeof h, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    *bad_entries = (long long)h;
    return PHG_OK;
    PHG_API_END
}

// ------------------------------------------------------------- autotuner ---
namespace {

struct EvPair {
    cudaEvent_t a = nullptr, b = nullptr;
    ~EvPair() { if (a) cudaEventDestroy(a); if (b) cudaEventDestroy(b); }
};

struct Report {
    std::string text;
    void add(const char *fmt, ...) {
        char line[256];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(line, sizeof line, fmt, ap);
        va_end(ap);
        text += line;
    }
};

// device milliseconds of fn() on s: the best of `reps` runs after one warm-up
template <typename F>
int time_best(cudaStream_t s, int reps, F fn, float *best) {
    EvPair e;
    CK(cudaEventCreate(&e.a));
    CK(cudaEventCreate(&e.b));
    int r = fn();
    if (r) return r;
    *best = 1e30f;
    for (int k = 0; k < reps; ++k) {
        CK(cudaEventRecord(e.a, s));
        if ((r = fn())) return r;
        CK(cudaEventRecord(e.b, s));
        CK(cudaEventSynchronize(e.b));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e.a, e.b));
        *best = std::min(*best, ms);
    }
    return PHG_OK;
}

// the fastest launch shape of op's solves at nv right-hand sides b = A x*
// (x* hashed), among rows per block 128..1024 and, for Chebyshev-solvable
// operators in mixed precision with 8 or more right-hand sides, the lockstep
// path; candidates that do not reach the tolerance are not chosen
int tune_solve(phg_ops_s *o, const char *label, const DevSolveOp &op, int nv, cudaStream_t s, Report &rep) {
    const int n = op.A.n;
    const Precision pr = prec_of(o);
    const int fam = solve_family(op);
    const size_t len = (size_t)n * nv;
    DBuf xs, b, x, st;
    CK(xs.ensure(8 * len)); CK(b.ensure(8 * len)); CK(x.ensure(8 * len)); CK(st.ensure(sizeof(GmresStats)));
    CK(fill_hash(xs.as<double>(), (long long)len, 12345u + (unsigned)nv, s));
    CK(apply_op(op.A, DevCols(), xs.as<double>(), n, nullptr, nullptr, 0, nullptr, b.as<double>(), n, nv, s));
    std::vector<SolveShape> cand;
    for (int rpb : {128, 256, 512, 1024}) { SolveShape c; c.rpb = rpb; c.path = 0; cand.push_back(c); }
    if ((fam == 1 || fam == 2) && pr == PREC_MIXED && nv >= 8) { SolveShape c; c.rpb = 0; c.path = 1; cand.push_back(c); }
    size_t need = 0;   // the largest workspace among the candidates' paths
    for (const SolveShape &c : cand) need = std::max(need, gmres_work_bytes(op, nv, o->restart, pr, &c));
    if (need > o->work.n) { CK(cudaStreamSynchronize(s)); CK(o->work.ensure(need)); }
    float best = 1e30f;
    SolveShape pick;
    bool any = false;
    // Candidates are timed as a captured and replayed solve: ensemble and
    // single-trajectory steps run from step graphs (phg_barvortex_run), where
    // a shape's many short launches cost far less than when enqueued one by one.
    const bool graphs = s != cudaStreamLegacy && s != cudaStreamPerThread;
    for (const SolveShape &c : cand) {
        auto enqueue = [&]() -> int {
            CK(cudaMemsetAsync(x.p, 0, 8 * len, s));
            CK(gmres_solve(op, b.as<double>(), x.as<double>(), nv, n, o->restart, o->max_iter, o->tol, pr, o->work.p,
                           st.as<GmresStats>(), s, false, o->max_sms, &c));
            return PHG_OK;
        };
        float ms = 0.f;
        int r;
        if (graphs) {
            // one direct run first (function attributes, first-use set-up), then the capture
            if ((r = enqueue())) return r;
            CK(cudaStreamSynchronize(s));
            const long long l0 = g_kernel_launches.load();
            CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            r = enqueue();
            cudaGraph_t g = nullptr;
            cudaError_t ec = cudaStreamEndCapture(s, &g);
            const long long per = g_kernel_launches.load() - l0;
            g_kernel_launches -= per;   // captured, not run
            if (r || ec != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                if (r) return r;
                return fail(PHG_ERR_CUDA, "autotune capture: %s", cudaGetErrorString(ec));
            }
            cudaGraphExec_t ge = nullptr;
            cudaError_t ei = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
            if (ei != cudaSuccess) return fail(PHG_ERR_CUDA, "autotune instantiate: %s", cudaGetErrorString(ei));
            r = time_best(s, 2, [&]() -> int {
                CK(cudaGraphLaunch(ge, s));
                g_kernel_launches += per;
                return PHG_OK;
            }, &ms);
            cudaGraphExecDestroy(ge);
        } else {
            r = time_best(s, 2, enqueue, &ms);
        }
        if (r) return r;
        GmresStats g{};
        CK(cudaMemcpy(&g, st.p, sizeof g, cudaMemcpyDeviceToHost));
        const bool ok = std::isfinite(g.relres) &&
                        (g.status == 0 || (g.status == 1 && g.relres <= std::max(1e3 * o->tol, 1e-8)));
        rep.add("solve %s family=%d rows=%d nv=%d rpb=%d path=%d ms=%.4f iters=%d relres=%.2e%s\n", label, fam, n,
                nv, c.rpb, c.path, ms, g.iters, g.relres, ok ? "" : " (not converged)");
        if (ok && ms < best) { best = ms; pick = c; any = true; }
    }
    if (!any) return fail(PHG_ERR_NOT_CONVERGED, "autotune: no launch shape reached the tolerance (%s)", label);
    tune_set_solve(fam, n, pr, nv, pick);
    rep.add("chose %s nv=%d rpb=%d path=%d\n", label, nv, pick.rpb, pick.path);
    return PHG_OK;
}

// threads per row of the interleaved FP32 operator apply at nv vectors
int tune_spmm(phg_ops_s *o, int nv, cudaStream_t s, Report &rep) {
    const float *v32 = o->L.op.a32 ? o->L.op.a32 : o->ML.op.a32;
    const unsigned *pk = o->L.op.a32 ? o->L.pk.as<unsigned>() : o->ML.pk.as<unsigned>();
    if (!v32 || nv < 4 || nv > 256 || nv % 4 || ((nv / 4) & (nv / 4 - 1))) return PHG_OK;
    const int q4 = nv / 4;
    const size_t len = (size_t)o->rs * nv;
    DBuf x, y;
    CK(x.ensure(4 * len)); CK(y.ensure(4 * len));
    CK(fill_hash32(x.as<float>(), (long long)len, 777u, s));
    float best = 1e30f;
    int pick = 0;
    for (int tpr = 1; tpr <= q4; tpr *= 2) {
        if (q4 / tpr > 8) continue;
        float ms = 0.f;
        int r = time_best(s, 5, [&]() -> int {
            if (pk) CK(spmm_pk32(pk, o->rs, x.as<float>(), y.as<float>(), nv, s, tpr));
            else CK(spmm_il32(o->pcol.as<int>(), v32, o->rs, o->W, x.as<float>(), y.as<float>(), nv, s, tpr));
            return PHG_OK;
        }, &ms);
        if (r) return r;
        rep.add("spmm rows=%d nv=%d threads_per_row=%d ms=%.4f\n", o->rs, nv, tpr, ms);
        if (ms < best) { best = ms; pick = tpr; }
    }
    if (pick) {
        tune_set_spmm(o->rs, nv, pick);
        rep.add("chose spmm nv=%d threads_per_row=%d\n", nv, pick);
    }
    return PHG_OK;
}

void copy_out(const std::string &t, char *buf, int len) {
    if (!buf || len <= 0) return;
    const size_t k = std::min(t.size(), (size_t)len - 1);
    memcpy(buf, t.data(), k);
    buf[k] = 0;
}

}  // namespace

extern "C" int phg_ops_autotune(phg_ops o, int nmembers, char *report, int report_len, void *stream) {
    PHG_API_BEGIN
    if (!o || nmembers < 1) return fail(PHG_ERR_ARG, "bad argument");
    cudaStream_t s = o->str(stream);
    Report rep;
    int r;
    // the solves of a barotropic step of nmembers states: mass (and the step
    // matrix, same family and size) at nmembers, the Jacobian's mass solves
    // at 8 x nmembers, the Laplace inverse at nmembers
    if ((r = tune_solve(o, "mass", o->ML.op, nmembers, s, rep))) return r;
    if ((r = tune_solve(o, "mass_jacobian", o->MJ.op, 8 * nmembers, s, rep))) return r;
    if ((r = tune_solve(o, "laplace", o->L.op, nmembers, s, rep))) return r;
    if ((r = tune_spmm(o, nmembers, s, rep))) return r;
    CK(cudaStreamSynchronize(s));
    g_shape_epoch++;   // captured steps pick up the new shapes
    copy_out(rep.text, report, report_len);
    return PHG_OK;
    PHG_API_END
}

extern "C" int phg_tune_describe(char *buf, int len) {
    PHG_API_BEGIN
    if (!buf || len <= 0) return fail(PHG_ERR_ARG, "bad argument");
    copy_out(tune_describe(), buf, len);
    return PHG_OK;
    PHG_API_END
}

extern "C" int phg_tune_save(const char *path) {
    PHG_API_BEGIN
    if (!path) return fail(PHG_ERR_ARG, "NULL path");
    return tune_save(path) ? fail(PHG_ERR_IO, "cannot write %s", path) : PHG_OK;
    PHG_API_END
}

extern "C" int phg_tune_load(const char *path, int *entries) {
    PHG_API_BEGIN
    if (!path) return fail(PHG_ERR_ARG, "NULL path");
    const int k = tune_load(path);
    g_shape_epoch++;   // captured steps pick up the new shapes
    if (k < 0) return fail(PHG_ERR_IO, "cannot read %s (missing or malformed)", path);
    if (entries) *entries = k;
    return PHG_OK;
    PHG_API_END
}

extern "C" void phg_tune_clear(void) {
    PHG_API_BEGIN
    tune_clear();
    g_shape_epoch++;
    PHG_API_END_VOID
}

extern "C" int phg_ops_check(phg_ops o, void *stream) {
    PHG_API_BEGIN
    if (!o) return fail(PHG_ERR_ARG, "NULL handle");
    cudaStream_t s = o->str(stream);
    if (o->pending_slots == 0) {
        CK(cudaStreamSynchronize(s));
        return PHG_OK;
    }
    return check_stats(o, o->pending_slots, s);
    PHG_API_END
}

extern "C" int phg_device_bytes(long long *total, long long *this_thread) {
    PHG_API_BEGIN
    if (total) *total = g_dev_bytes.load();
    if (this_thread) *this_thread = t_dev_bytes;
    return PHG_OK;
    PHG_API_END
}

static int jacobian_common(phg_ops o, double *ans, const double *u, const double *v, const double *bnd,
                           bool full, bool transpose, void *stream) {
    if (!o || !ans || !u || !v) return fail(PHG_ERR_ARG, "NULL argument");
    cudaStream_t s = o->str(stream);
    Stage st(o, s);
    const double *du, *dv, *dB; double *dA;
    CK(st.in(u, o->V, &du)); CK(st.in(v, o->V, &dv)); CK(st.in(bnd, o->os, &dB));
    CK(st.out(ans, full ? o->V : o->rs, &dA));
    CK(o->s_e.ensure(8 * (size_t)o->rs * 8));
    CK(o->s_c.ensure(8 * (size_t)o->rs));
    int r = jacobian_derivs_dev(o, du, dv, o->V, o->s_e.as<double>(), 1, 0, s, mass_tol(o));
    if (r) return r;
    double *jac = full ? o->s_c.as<double>() : dA;
    CK(jac_combine(o->s_e.as<double>(), o->rs, o->rs, jac, o->rs, nullptr, 0, nullptr, 1, s));
    if (transpose) CK(axpbz(jac, jac, -1.0, jac, 0.0, o->rs, s));
    if (full) CK(p2u(dA, o->V, jac, o->rs, dB, o->os, o->p2io.as<int>(), o->isb.as<int>(), o->V, 1, s));
    CK(st.finish());
    return st.host ? check_stats(o, 1, s) : PHG_OK;
}

extern "C" int phg_jacobian_calc1(phg_ops o, double *ans, const double *u, const double *v, const double *bnd, void *s) {
    PHG_API_BEGIN
    return jacobian_common(o, ans, u, v, bnd, true, false, s);
    PHG_API_END
}
extern "C" int phg_jacobian_calc2(phg_ops o, double *ans, const double *u, const double *v, void *s) {
    PHG_API_BEGIN
    return jacobian_common(o, ans, u, v, nullptr, false, false, s);
    PHG_API_END
}
extern "C" int phg_jacobian_calc2t(phg_ops o, double *ans, const double *u, const double *v, void *s) {
    PHG_API_BEGIN
    return jacobian_common(o, ans, u, v, nullptr, false, true, s);
    PHG_API_END
}

extern "C" int phg_jacobian_derivs(phg_ops o, int quad, double *out, const double *u, const double *v, int nv,
                                   void *stream) {
    PHG_API_BEGIN
    if (!o || !out || !u || !v || nv < 1) return fail(PHG_ERR_ARG, "bad argument");
    if (!is_device_ptr(out) || !is_device_ptr(u) || !is_device_ptr(v))
        return fail(PHG_ERR_ARG, "phg_jacobian_derivs takes device pointers");
    if (quad && !o->jq.n) return fail(PHG_ERR_ARG, "this mesh has points with more than 6 triangles");
    cudaStream_t s = o->str(stream);
    if (quad) {
        CK(o->jq_split.ensure(16 * (size_t)o->V * nv));
        CK(jac_quad(o->jq, o->J, u, v, o->V, o->imap(), o->bmap(), out, o->rs, nv, o->V, (float2 *)o->jq_split.p, s));
    }
    else CK(jac_rhs(o->J, u, v, o->V, o->imap(), o->bmap(), out, o->rs, nv, s));
    return PHG_OK;
    PHG_API_END
}

extern "C" int phg_jacobian_calc1t(phg_ops o, double *ans, const double *u, const double *v, const double *bnd,
                                   void *s) {
    PHG_API_BEGIN
    return jacobian_common(o, ans, u, v, bnd, true, true, s);
    PHG_API_END
}

// M_J^-1 (D v_in + D_bnd v_bnd): one derivative of SphereJacobian
static int jacobian_diff(phg_ops o, double *ans, const double *v, bool cos_y, void *stream) {
    if (!o || !ans || !v) return fail(PHG_ERR_ARG, "NULL argument");
    cudaStream_t s = o->str(stream);
    Stage st(o, s);
    const double *dv; double *dA;
    CK(st.in(v, o->V, &dv));
    CK(st.out(ans, o->rs, &dA));
    CK(o->s_c.ensure(8 * (size_t)o->rs));
    double *rhs = o->s_c.as<double>();
    const DevEll &D = cos_y ? o->J.d2c : o->J.d1;
    const DevCols &Db = cos_y ? o->J.d2cb : o->J.d1b;
    CK(apply_op(D, Db, dv, o->V, o->imap(), dv, o->V, o->bmap(), rhs, o->rs, 1, s));
    CK(cudaMemsetAsync(dA, 0, 8 * (size_t)o->rs, s));
    int r = solve(o, o->MJ.op, rhs, dA, 1, o->rs, mass_tol(o), 0, s);
    if (r) return r;
    CK(st.finish());
    return st.host ? check_stats(o, 1, s) : PHG_OK;
}

extern "C" int phg_jacobian_calc2_diff_x(phg_ops o, double *ans, const double *v, void *s) {
    PHG_API_BEGIN
    return jacobian_diff(o, ans, v, false, s);
    PHG_API_END
}
extern "C" int phg_jacobian_calc2_diff_cos_y(phg_ops o, double *ans, const double *v, void *s) {
    PHG_API_BEGIN
    return jacobian_diff(o, ans, v, true, s);
    PHG_API_END
}

static int norm_common(phg_ops o, const double *u, const double *v, double *out, bool dist, bool sq, void *stream) {
    if (!o || !u || !out) return fail(PHG_ERR_ARG, "NULL argument");
    cudaStream_t s = o->str(stream);
    Stage st(o, s);
    const double *du, *dv;
    CK(st.in(u, o->V, &du)); CK(st.in(v, o->V, &dv));
    CK(o->s_out.ensure(64));
    int r = norm_dev(o, du, dv, 1, o->s_out.as<double>(), dist, sq, s);
    if (r) return r;
    CK(cudaMemcpyAsync(out, o->s_out.p, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return PHG_OK;
}

extern "C" int phg_norm(phg_ops o, const double *u, double *out, void *s) { PHG_API_BEGIN return norm_common(o, u, nullptr, out, false, true, s); PHG_API_END }
extern "C" int phg_dist(phg_ops o, const double *u, const double *v, double *out, void *s) {
    PHG_API_BEGIN
    if (!v) return fail(PHG_ERR_ARG, "NULL argument");
    return norm_common(o, u, v, out, true, true, s);
    PHG_API_END
}
extern "C" int phg_scalar(phg_ops o, const double *u, const double *v, double *out, void *s) {
    PHG_API_BEGIN
    if (!v) return fail(PHG_ERR_ARG, "NULL argument");
    return norm_common(o, u, v, out, false, false, s);
    PHG_API_END
}

// ------------------------------------------------------------ barvortex ---
struct phg_barvortex_s {
    phg_ops_s *o = nullptr;
    phg_bv_conf c{};
    SolveOpBufs A;
    ColsBufs Ab;
    DBuf lh;
    int cap = 0;   // members the buffers hold
    DBuf w, dw, FC, u_n, w_n, u_n1, tmp1, tmp2, uin, F, rp, x, jsol, nr0, nr, done, ubnd, wbnd, frc;
    std::vector<GmresStats> each;   // the last step's solve records, one per slot
    int nslots = 0;
    cudaStream_t last_stream = nullptr;   // stream of the last step (its stats live there)
    // linearised / adjoint steps: the backward matrix Ab_ and its boundary
    // columns bndb_ (built on first use), and their scratch vectors
    bool have_back = false;
    SolveOpBufs Aback;
    ColsBufs Abackb;
    DBuf lz, lp1, lp2, lp3, lju, ljv, ljac, ljf, lx, lrp, lin;
    // phg_barvortex_run: one step captured as a CUDA graph, replayed per step;
    // valid for the key it was captured with
    struct GraphKey {
        int nv = 0;
        const double *u = nullptr, *bnd_u = nullptr, *bnd_w = nullptr, *forcing = nullptr;
        cudaStream_t s = nullptr;
        long long epoch = -1;           // tuned-shape epoch
        unsigned long long sig = 0;     // addresses and sizes of the step's scratch buffers
        bool operator==(const GraphKey &k) const {
            return nv == k.nv && u == k.u && bnd_u == k.bnd_u && bnd_w == k.bnd_w && forcing == k.forcing &&
                   s == k.s && epoch == k.epoch && sig == k.sig;
        }
    };
    // captured steps by key (member count, arrays, stream, tuned shapes and the
    // scratch buffers' addresses),
    // the least recently used dropped beyond GRAPHS: a caller whose member
    // count changes between runs (a serving lane) replays the graph of each
    // count it meets again instead of capturing anew
    static constexpr int GRAPHS = 8;
    struct Graph {
        GraphKey key;
        cudaGraphExec_t exec = nullptr;
        long long launches = 0;   // kernels in one replay
        long long used = 0;
    };
    std::vector<Graph> graphs;
    long long graph_clock = 0;
    DBuf agg;                   // solve records folded over the steps of runs since the last check
    bool agg_pending = false;
    ~phg_barvortex_s() {
        for (auto &g : graphs)
            if (g.exec) cudaGraphExecDestroy(g.exec);
    }
};

extern "C" int phg_barvortex_create(phg_ops o, const phg_bv_conf *c, const double *coriolis, phg_barvortex *out) {
    PHG_API_BEGIN
    if (!o || !c || !out) return fail(PHG_ERR_ARG, "NULL argument");
    if (!(c->tau > 0) || c->picard_iters < 1 || c->picard_iters > 1000)
        return fail(PHG_ERR_ARG, "bad configuration (tau > 0, 1 <= picard_iters <= 1000)");
    auto b = std::make_unique<phg_barvortex_s>();
    b->o = o;
    b->c = *c;
    // solve records of one step: two Laplace applies, then a Jacobian, an A
    // and a Laplace solve per Picard iteration (the linearised steps use fewer)
    const int slots = std::max(64, 2 + 3 * c->picard_iters);
    if (o->stats.n < sizeof(GmresStats) * (size_t)slots) {
        CK(cudaStreamSynchronize(o->stream));
        CK(o->stats.ensure(sizeof(GmresStats) * (size_t)slots));
        CK(cudaMemset(o->stats.p, 0, sizeof(GmresStats) * (size_t)slots));
    }
    b->each.assign(slots, GmresStats{});
    Csr A, Ab;
    const double c1 = 1.0 / c->tau + c->sigma * c->theta;
    const double c2 = -c->theta * c->mu;
    assemble_barvortex(o->mesh->m, c1, c2, A, Ab);
    if (!same_pattern(A, o->mesh->ops.idt)) return fail(PHG_ERR_ARG, "barvortex matrix pattern mismatch");
    int r;
    if ((r = build_solve_op(o, A, b->A, true))) return r;
    if ((r = build_cols(Ab, b->Ab))) return r;
    std::vector<double> lh(o->V, 0.0);
    if (coriolis) {
        if (is_device_ptr(coriolis)) CK(cudaMemcpy(lh.data(), coriolis, 8 * lh.size(), cudaMemcpyDeviceToHost));
        else memcpy(lh.data(), coriolis, 8 * lh.size());
    }
    CK(upload(b->lh, lh));
    o->refs++;
    *out = b.release();
    return PHG_OK;
    PHG_API_END
}

extern "C" void phg_barvortex_destroy(phg_barvortex b) {
    PHG_API_BEGIN
    if (!b) return;
    phg_ops_s *o = b->o;
    cudaStreamSynchronize(o->stream);
    delete b;
    ops_release(o);
    PHG_API_END_VOID
}

namespace {

int bv_reserve(phg_barvortex_s *b, int nv) {
    if (nv <= b->cap) return PHG_OK;
    const size_t V = b->o->V, rs = b->o->rs, os = std::max(1, b->o->os);
    DBuf *full[] = {&b->w, &b->dw, &b->FC, &b->u_n, &b->w_n, &b->u_n1, &b->tmp1, &b->tmp2, &b->uin};
    for (DBuf *d : full) CK(d->ensure(8 * V * nv));
    DBuf *inner[] = {&b->F, &b->rp, &b->x};
    for (DBuf *d : inner) CK(d->ensure(8 * rs * nv));
    CK(b->jsol.ensure(8 * rs * 8 * nv));
    CK(b->nr0.ensure(8 * nv)); CK(b->nr.ensure(8 * nv)); CK(b->done.ensure(4 * nv));
    CK(b->ubnd.ensure(8 * os * nv)); CK(b->wbnd.ensure(8 * os * nv)); CK(b->frc.ensure(8 * V));
    b->cap = nv;
    return PHG_OK;
}

// One Crank-Nicolson / Picard step for nv members, all arguments on the
// device (examples/barvortex_impl.h:171-310).
int bv_step_dev(phg_barvortex_s *b, int nv, double *u1, const double *u, const double *bnd_u,
                const double *bnd_w, const double *forcing, cudaStream_t s) {
    NvtxRange nvtx("phg:barvortex_step");
    phg_ops_s *o = b->o;
    const int V = o->V, rs = o->rs, os = o->os;
    const long long NV = (long long)V * nv;
    const phg_bv_conf &c = b->c;
    int r, slot = 0;
    double *w = b->w.as<double>(), *dw = b->dw.as<double>(), *FC = b->FC.as<double>();
    double *u_n = b->u_n.as<double>(), *w_n = b->w_n.as<double>(), *u_n1 = b->u_n1.as<double>();
    double *tmp1 = b->tmp1.as<double>(), *tmp2 = b->tmp2.as<double>(), *uu = b->uin.as<double>();
    double *F = b->F.as<double>(), *rp = b->rp.as<double>(), *x = b->x.as<double>();
    double *jsol = b->jsol.as<double>();
    const int *p2io = o->p2io.as<int>(), *isb = o->isb.as<int>();
    // keep the input: u1 may alias u
    CK(cudaMemcpyAsync(uu, u, 8 * NV, cudaMemcpyDeviceToDevice, s));
    // nr0 = norm(u)
    if ((r = norm_dev(o, uu, nullptr, nv, b->nr0.as<double>(), false, true, s))) return r;
    // w = L(u) with bnd_w, dw = L(w) with zero boundary
    if ((r = laplace_calc2_dev(o, x, rs, uu, V, nv, slot++, s, o->tol))) return r;
    CK(p2u(w, V, x, rs, bnd_w, os, p2io, isb, V, nv, s));
    if ((r = laplace_calc2_dev(o, x, rs, w, V, nv, slot++, s, o->tol))) return r;
    CK(p2u(dw, V, x, rs, nullptr, os, p2io, isb, V, nv, s));
    // FC = w/tau + mu(1-theta) dw - sigma(1-theta) w (+ f)
    CK(bv_fc(FC, w, dw, forcing, 1.0 / c.tau, c.mu * (1.0 - c.theta), -c.sigma * (1.0 - c.theta), V, NV, s));
    CK(cudaMemsetAsync(u_n, 0, 8 * NV, s));
    CK(cudaMemsetAsync(w_n, 0, 8 * NV, s));
    CK(cudaMemsetAsync(b->done.p, 0, 4 * (size_t)nv, s));
    for (int it = 0; it < c.picard_iters; ++it) {
        CK(bv_mix(tmp1, tmp2, w_n, w, u_n, uu, b->lh.as<double>(), V, c.k1 * c.theta, c.k1 * (1.0 - c.theta), c.k2,
                  c.theta, 1.0 - c.theta, NV, s));
        // F = FC[inner] - J(tmp2, tmp1)
        const bool quad = o->jq_mode == 1 || (o->jq_mode == 2 && it + 1 < c.picard_iters);
        if ((r = jacobian_derivs_dev(o, tmp2, tmp1, V, jsol, nv, slot++, s, o->tol, quad, it > 0))) return r;
        CK(jac_combine(jsol, rs, rs, F, rs, FC, V, o->imap(), nv, s));
        // rp = M_L F + bnd_ bnd_w ; w_n = p2u(A^-1 rp, bnd_w)
        CK(apply_op(o->ML.op.A, b->Ab.c, F, rs, nullptr, bnd_w, os, nullptr, rp, rs, nv, s));
        // warm start: previous w_n (first iteration: w), inner part
        CK(gather(x, rs, it == 0 ? w : w_n, V, o->imap(), rs, nv, s));
        if ((r = solve(o, b->A.op, rp, x, nv, rs, o->tol, slot++, s))) return r;
        CK(p2u(w_n, V, x, rs, bnd_w, os, p2io, isb, V, nv, s));
        // u_n1 = Laplace^-1(w_n) with bnd_u: b = M_L w_n_in + B2 bnd_u
        CK(apply_op(o->ML.op.A, o->bnd2.c, w_n, V, o->imap(), bnd_u, os, nullptr, rp, rs, nv, s));
        CK(gather(x, rs, it == 0 ? uu : u_n, V, o->imap(), rs, nv, s));
        if ((r = solve(o, o->L.op, rp, x, nv, rs, o->tol, slot++, s))) return r;
        CK(p2u(u_n1, V, x, rs, bnd_u, os, p2io, isb, V, nv, s));
        // nr = dist(u_n1, u_n); u_n <- u_n1; stop test
        if ((r = norm_dev(o, u_n1, u_n, nv, b->nr.as<double>(), true, true, s))) return r;
        CK(bv_commit(u_n, u_n1, b->nr.as<double>(), b->nr0.as<double>(), b->done.as<int>(), V, nv, s));
    }
    CK(cudaMemcpyAsync(u1, u_n, 8 * NV, cudaMemcpyDeviceToDevice, s));
    b->nslots = slot;
    return PHG_OK;
}

}  // namespace

static int bv_calc(phg_barvortex b, int nv, double *u1, const double *u, const double *bnd_u,
                   const double *bnd_w, const double *forcing, void *stream) {
    if (!b || !u1 || !u || nv < 1) return fail(PHG_ERR_ARG, "NULL argument");
    phg_ops_s *o = b->o;
    cudaStream_t s = o->str(stream);
    int r = bv_reserve(b, nv);
    if (r) return r;
    Stage st(o, s);
    const double *du, *dbu, *dbw, *df; double *du1;
    CK(st.in(u, (size_t)o->V * nv, &du));
    CK(st.in(bnd_u, (size_t)o->os * nv, &dbu));
    CK(st.in(bnd_w, (size_t)o->os * nv, &dbw));
    CK(st.in(forcing, (size_t)o->V, &df));
    CK(st.out(u1, (size_t)o->V * nv, &du1));
    if (o->os == 0) { dbu = nullptr; dbw = nullptr; }
    if ((r = bv_step_dev(b, nv, du1, du, dbu, dbw, df, s))) return r;
    b->last_stream = s;
    CK(st.finish());
    if (!st.host) return PHG_OK;
    return check_stats(o, b->nslots, s, nullptr, b->each.data());
}

extern "C" int phg_barvortex_calc(phg_barvortex b, double *u1, const double *u, const double *bnd_u,
                                  const double *bnd_w, const double *forcing, void *stream) {
    PHG_API_BEGIN
    return bv_calc(b, 1, u1, u, bnd_u, bnd_w, forcing, stream);
    PHG_API_END
}

extern "C" int phg_barvortex_calc_batch(phg_barvortex b, int nmembers, double *u1, const double *u,
                                        const double *bnd_u, const double *bnd_w, const double *forcing,
                                        void *stream) {
    PHG_API_BEGIN
    return bv_calc(b, nmembers, u1, u, bnd_u, bnd_w, forcing, stream);
    PHG_API_END
}

// check the solves folded into b->agg since the last check
static int bv_check_agg(phg_barvortex_s *b, cudaStream_t s) {
    GmresStats a{};
    CK(cudaMemcpyAsync(&a, b->agg.p, sizeof a, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    b->agg_pending = false;
    const double tol = b->o->tol;
    if (a.status == 2) return fail(PHG_ERR_TIMEOUT, "device barrier wait timed out");
    if (!std::isfinite(a.relres) || (a.status == 1 && !(a.relres <= std::max(1e3 * tol, 1e-8))))
        return fail(PHG_ERR_NOT_CONVERGED, "GMRES stopped at relative residual %.3e", a.relres);
    return PHG_OK;
}

// nsteps steps in place.  With a graph captured for this key every step is
// one replay; otherwise the first step is enqueued kernel by kernel (it
// sizes every buffer) and the next one is captured.
// A signature of what a captured barotropic step bakes in beyond its
// arguments: every scratch buffer it writes or reads (the handle's and the
// stepper's) and the handle's solver settings and SM cap, which become
// kernel parameters and grid sizes.  A captured step is valid only while the
// signature is unchanged.  Per stepper, so that allocations by other handles
// (other threads) do not invalidate its graphs.
static unsigned long long bv_sig(const phg_barvortex_s *b) {
    const phg_ops_s *o = b->o;
    unsigned long long h = 1469598103934665603ull;
    auto word = [&](unsigned long long v) { h = (h ^ v) * 1099511628211ull; };
    auto mix = [&](const DBuf &d) {
        word((unsigned long long)(uintptr_t)d.p);
        word((unsigned long long)d.n);
    };
    word((unsigned long long)o->max_sms);
    word((unsigned long long)o->restart);
    word((unsigned long long)o->max_iter);
    double tol = o->tol;
    unsigned long long tb = 0;
    memcpy(&tb, &tol, sizeof tb);
    word(tb);
    word((unsigned long long)o->wait_limit);
    word((unsigned long long)o->jq_mode);
    for (const DBuf *d : {&o->work, &o->stats, &o->s_a, &o->s_b, &o->s_c, &o->s_d, &o->s_e, &o->s_part, &o->s_out,
                          &o->jq_split, &o->hist})
        mix(*d);
    for (const DBuf &d : o->st) mix(d);
    for (const DBuf *d : {&b->w, &b->dw, &b->FC, &b->u_n, &b->w_n, &b->u_n1, &b->tmp1, &b->tmp2, &b->uin, &b->F,
                          &b->rp, &b->x, &b->jsol, &b->nr0, &b->nr, &b->done, &b->ubnd, &b->wbnd, &b->frc, &b->agg})
        mix(*d);
    return h;
}

static int bv_run(phg_barvortex b, int nv, int nsteps, double *u, const double *bnd_u, const double *bnd_w,
                  const double *forcing, void *stream) {
    if (!b || !u || nv < 1 || nsteps < 0) return fail(PHG_ERR_ARG, "bad argument");
    if (nsteps == 0) return PHG_OK;
    NvtxRange nvtx("phg:barvortex_run");
    phg_ops_s *o = b->o;
    cudaStream_t s = o->str(stream);
    if (s == cudaStreamLegacy || s == cudaStreamPerThread)
        return fail(PHG_ERR_ARG, "a captured step needs a created stream (pass NULL for the handle's own)");
    int r = bv_reserve(b, nv);
    if (r) return r;
    CK(b->agg.ensure(sizeof(GmresStats)));
    Stage st(o, s);
    const double *dbu, *dbw, *df, *du;
    CK(st.in(u, (size_t)o->V * nv, &du));
    double *dio = const_cast<double *>(du);
    if (st.host) st.outs.push_back({u, dio, (size_t)o->V * nv});
    CK(st.in(bnd_u, (size_t)o->os * nv, &dbu));
    CK(st.in(bnd_w, (size_t)o->os * nv, &dbw));
    CK(st.in(forcing, (size_t)o->V, &df));
    if (o->os == 0) { dbu = nullptr; dbw = nullptr; }
    GmresStats *agg = b->agg.as<GmresStats>(), *slots = o->stats.as<GmresStats>();
    if (!b->agg_pending) CK(cudaMemsetAsync(agg, 0, sizeof(GmresStats), s));
    b->agg_pending = true;
    phg_barvortex_s::GraphKey k;
    k.nv = nv; k.u = dio; k.bnd_u = dbu; k.bnd_w = dbw; k.forcing = df; k.s = s;
    k.epoch = g_shape_epoch.load();
    k.sig = bv_sig(b);
    int left = nsteps;
    // drop graphs of other tuned shapes or moved buffers; find this key's
    for (size_t q = 0; q < b->graphs.size();) {
        if (b->graphs[q].key.epoch != k.epoch || b->graphs[q].key.sig != k.sig) {
            cudaGraphExecDestroy(b->graphs[q].exec);
            b->graphs.erase(b->graphs.begin() + q);
        } else {
            ++q;
        }
    }
    phg_barvortex_s::Graph *gr = nullptr;
    for (auto &g : b->graphs)
        if (g.key == k) gr = &g;
    if (!gr) {
        if ((r = bv_step_dev(b, nv, dio, dio, dbu, dbw, df, s))) return r;
        CK(stats_fold(slots, b->nslots, agg, s));
        --left;
        k.sig = bv_sig(b);   // the eager step may have grown a buffer
        if (left > 0) {
            const bool prof = o->prof;
            o->prof = false;
            const long long l0 = g_kernel_launches.load();
            CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            r = bv_step_dev(b, nv, dio, dio, dbu, dbw, df, s);
            cudaError_t ef = r ? cudaSuccess : stats_fold(slots, b->nslots, agg, s);
            cudaGraph_t g = nullptr;
            cudaError_t ec = cudaStreamEndCapture(s, &g);
            o->prof = prof;
            const long long nl = g_kernel_launches.load() - l0;
            g_kernel_launches -= nl;   // captured, not run
            if (r || ef != cudaSuccess || ec != cudaSuccess || !g) {
                if (g) cudaGraphDestroy(g);
                if (r) return r;
                return fail(PHG_ERR_CUDA, "step capture: %s", cudaGetErrorString(ef != cudaSuccess ? ef : ec));
            }
            cudaGraphExec_t ex = nullptr;
            cudaError_t ei = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            if (ei != cudaSuccess) return fail(PHG_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ei));
            if (bv_sig(b) != k.sig) {   // the capture itself moved a buffer: run the rest uncaptured
                cudaGraphExecDestroy(ex);
                ex = nullptr;
                for (; left > 0; --left) {
                    if ((r = bv_step_dev(b, nv, dio, dio, dbu, dbw, df, s))) return r;
                    CK(stats_fold(slots, b->nslots, agg, s));
                }
            }
            if (ex && (int)b->graphs.size() >= phg_barvortex_s::GRAPHS) {   // drop the least recently used
                size_t lru = 0;
                for (size_t q = 1; q < b->graphs.size(); ++q)
                    if (b->graphs[q].used < b->graphs[lru].used) lru = q;
                cudaGraphExecDestroy(b->graphs[lru].exec);
                b->graphs.erase(b->graphs.begin() + lru);
            }
            if (ex) {
                phg_barvortex_s::Graph ng;
                ng.key = k;
                ng.exec = ex;
                ng.launches = nl;
                b->graphs.push_back(ng);
                gr = &b->graphs.back();
            }
        }
    }
    if (gr) {
        gr->used = ++b->graph_clock;
        for (int i = 0; i < left; ++i) CK(cudaGraphLaunch(gr->exec, s));
        g_kernel_launches += gr->launches * left;
    }
    b->last_stream = s;
    CK(st.finish());
    if (!st.host) return PHG_OK;   // device arguments: checked by phg_barvortex_last_stats
    r = check_stats(o, b->nslots, s, nullptr, b->each.data());   // the last step, for phg_barvortex_last_stats
    int r2 = bv_check_agg(b, s);
    return r2 ? r2 : r;
}

extern "C" int phg_barvortex_run(phg_barvortex b, int nmembers, int nsteps, double *u, const double *bnd_u,
                                 const double *bnd_w, const double *forcing, void *stream) {
    PHG_API_BEGIN
    return bv_run(b, nmembers, nsteps, u, bnd_u, bnd_w, forcing, stream);
    PHG_API_END
}

// ------------------------------------------- linearised / adjoint steps ---
namespace {

// full vector out = p2u(M_L^-1 (L F + B3 bnd), bnd): SphereLaplace::calc1
int lin_calc1(phg_barvortex_s *b, double *out, const double *F, const double *bnd, int &slot, cudaStream_t s) {
    phg_ops_s *o = b->o;
    int r = laplace_calc2_dev(o, b->lx.as<double>(), o->rs, F, o->V, 1, slot++, s, mass_tol(o));
    if (r) return r;
    CK(p2u(out, o->V, b->lx.as<double>(), o->rs, bnd, o->os, o->p2io.as<int>(), o->isb.as<int>(), o->V, 1, s));
    return PHG_OK;
}

// full vector out = SphereLaplace::solve(F, bnd)
int lin_lsolve(phg_barvortex_s *b, double *out, const double *F, const double *bnd, int &slot, cudaStream_t s) {
    phg_ops_s *o = b->o;
    double *rp = b->lrp.as<double>(), *x = b->lx.as<double>();
    CK(apply_op(o->ML.op.A, o->bnd2.c, F, o->V, o->imap(), bnd, o->os, nullptr, rp, o->rs, 1, s));
    CK(cudaMemsetAsync(x, 0, 8 * (size_t)o->rs, s));
    int r = solve(o, o->L.op, rp, x, 1, o->rs, o->tol, slot++, s);
    if (r) return r;
    CK(p2u(out, o->V, x, o->rs, bnd, o->os, o->p2io.as<int>(), o->isb.as<int>(), o->V, 1, s));
    return PHG_OK;
}

// out = p2u(M^-1 (idt u2p(F) + Bc bnd_w), bnd_w): phelm::solve with the step's
// right-hand side (src/mesh.h:720-746, examples/barvortex_impl.h:379-390)
int lin_msolve(phg_barvortex_s *b, double *out, const double *F, const DevSolveOp &M, const DevCols &Bc,
               const double *bnd_w, int &slot, cudaStream_t s) {
    phg_ops_s *o = b->o;
    double *rp = b->lrp.as<double>(), *x = b->lx.as<double>();
    CK(apply_op(o->ML.op.A, Bc, F, o->V, o->imap(), bnd_w, o->os, nullptr, rp, o->rs, 1, s));
    CK(cudaMemsetAsync(x, 0, 8 * (size_t)o->rs, s));
    int r = solve(o, M, rp, x, 1, o->rs, o->tol, slot++, s);
    if (r) return r;
    CK(p2u(out, o->V, x, o->rs, bnd_w, o->os, o->p2io.as<int>(), o->isb.as<int>(), o->V, 1, s));
    return PHG_OK;
}

// three Jacobians in one batched solve, as full vectors with zero boundary:
// jf[k] = sign * J(u_k, v_k) (SphereJacobian::calc1 / calc1t with bnd = 0)
int lin_jac3(phg_barvortex_s *b, const double *const u[3], const double *const v[3], double sign, int &slot,
             cudaStream_t s) {
    phg_ops_s *o = b->o;
    const int V = o->V, rs = o->rs;
    double *ju = b->lju.as<double>(), *jv = b->ljv.as<double>(), *jac = b->ljac.as<double>();
    for (int k = 0; k < 3; ++k) {
        CK(cudaMemcpyAsync(ju + (size_t)k * V, u[k], 8 * (size_t)V, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(jv + (size_t)k * V, v[k], 8 * (size_t)V, cudaMemcpyDeviceToDevice, s));
    }
    int r = jacobian_derivs_dev(o, ju, jv, V, o->s_e.as<double>(), 3, slot++, s, mass_tol(o));
    if (r) return r;
    CK(jac_combine(o->s_e.as<double>(), rs, rs, jac, rs, nullptr, 0, nullptr, 3, s));
    if (sign != 1.0) CK(axpbz(jac, jac, sign, jac, 0.0, 3LL * rs, s));
    CK(p2u(b->ljf.as<double>(), V, jac, rs, nullptr, o->os, o->p2io.as<int>(), o->isb.as<int>(), V, 3, s));
    return PHG_OK;
}

int lin_reserve(phg_barvortex_s *b) {
    phg_ops_s *o = b->o;
    const size_t V = o->V, rs = o->rs;
    DBuf *full[] = {&b->lz, &b->lp1, &b->lp2, &b->lp3, &b->lin};
    for (DBuf *d : full) CK(d->ensure(8 * V));
    CK(b->lju.ensure(8 * 3 * V)); CK(b->ljv.ensure(8 * 3 * V)); CK(b->ljf.ensure(8 * 3 * V));
    CK(b->ljac.ensure(8 * 3 * rs)); CK(b->lx.ensure(8 * rs)); CK(b->lrp.ensure(8 * rs));
    CK(o->s_e.ensure(8 * rs * 8 * 3));
    return PHG_OK;
}

int lin_backward(phg_barvortex_s *b) {
    if (b->have_back) return PHG_OK;
    phg_ops_s *o = b->o;
    const phg_bv_conf &c = b->c;
    Csr A, Ab;
    // Ab_ = (1/tau - sigma (1 - theta)) M + (1 - theta) mu L (examples/barvortex_impl.h:84-105)
    assemble_barvortex(o->mesh->m, 1.0 / c.tau - c.sigma * (1.0 - c.theta), (1.0 - c.theta) * c.mu, A, Ab);
    if (!same_pattern(A, o->mesh->ops.idt)) return fail(PHG_ERR_ARG, "backward matrix pattern mismatch");
    int r;
    if ((r = build_solve_op(o, A, b->Aback, true))) return r;
    if ((r = build_cols(Ab, b->Abackb))) return r;
    b->have_back = true;
    return PHG_OK;
}

// kind 0: calc_L, 1: calc_L_1 (adds into u1), 2: calc_LT; device pointers
int lin_dev(phg_barvortex_s *b, int kind, double *u1, const double *u, const double *z, const double *bnd_u,
            const double *bnd_w, cudaStream_t s) {
    phg_ops_s *o = b->o;
    const int V = o->V;
    const long long NV = V;
    const phg_bv_conf &c = b->c;
    const double k1 = c.k1, k2 = c.k2, th = c.theta, mu = c.mu, sg = c.sigma, tau = c.tau;
    int r, slot = 0;
    if ((r = lin_reserve(b))) return r;
    if (kind == 1 && (r = lin_backward(b))) return r;
    double *zl = b->lz.as<double>(), *pt1 = b->lp1.as<double>(), *pt2 = b->lp2.as<double>(),
           *pt3 = b->lp3.as<double>(), *jf = b->ljf.as<double>(), *in = b->lin.as<double>();
    const double *lh = b->lh.as<double>();
    if (kind < 2) {
        // examples/barvortex_impl.h:343-362 (calc_L) and 421-440 (calc_L_1)
        CK(cudaMemcpyAsync(in, u, 8 * NV, cudaMemcpyDeviceToDevice, s));   // u1 may alias u
        if ((r = lin_calc1(b, zl, z, bnd_w, slot, s))) return r;
        if ((r = lin_calc1(b, pt1, in, bnd_w, slot, s))) return r;
        const double *ju[3] = {in, z, in}, *jv[3] = {lh, pt1, zl};
        if ((r = lin_jac3(b, ju, jv, 1.0, slot, s))) return r;
        CK(axpbz(pt3, jf, k2, jf, 0.0, NV, s));
        CK(axpbz(pt3, pt3, 1.0, jf + V, k1, NV, s));
        CK(axpbz(pt3, pt3, 1.0, jf + 2 * (size_t)V, k1, NV, s));
        if (kind == 0) CK(axpbz(pt3, pt3, -1.0, pt3, 0.0, NV, s));
        if ((r = lin_calc1(b, pt2, pt1, nullptr, slot, s))) return r;
        if (kind == 0) {
            CK(axpbz(pt2, pt2, (1. - th) * mu, pt2, 0.0, NV, s));
            CK(axpbz(pt1, pt1, 1.0 / tau - (1. - th) * sg, pt1, 0.0, NV, s));
            CK(axpbz(u1, pt1, 1.0, pt1, 0.0, NV, s));
        } else {
            CK(axpbz(pt2, pt2, -th * mu, pt2, 0.0, NV, s));
            CK(axpbz(pt1, pt1, 1.0 / tau + th * sg, pt1, 0.0, NV, s));
            CK(axpbz(u1, u1, 1.0, pt1, 1.0, NV, s));
        }
        CK(axpbz(u1, u1, 1.0, pt2, 1.0, NV, s));
        CK(axpbz(u1, u1, 1.0, pt3, 1.0, NV, s));
        const DevSolveOp &M = kind == 0 ? b->A.op : b->Aback.op;
        const DevCols &Bc = kind == 0 ? b->Ab.c : b->Abackb.c;
        if ((r = lin_msolve(b, u1, u1, M, Bc, bnd_w, slot, s))) return r;
        if ((r = lin_lsolve(b, u1, u1, bnd_u, slot, s))) return r;
    } else {
        // examples/barvortex_impl.h:485-535
        CK(cudaMemcpyAsync(in, z, 8 * NV, cudaMemcpyDeviceToDevice, s));   // v1 may alias z
        if ((r = lin_calc1(b, zl, in, bnd_w, slot, s))) return r;
        if ((r = lin_lsolve(b, u1, u, bnd_u, slot, s))) return r;
        if ((r = lin_msolve(b, u1, u1, b->A.op, b->Ab.c, bnd_w, slot, s))) return r;
        if ((r = lin_calc1(b, pt1, u1, bnd_w, slot, s))) return r;
        CK(axpbz(pt1, pt1, 1.0 / tau - (1.0 - th) * sg, pt1, 0.0, NV, s));
        if ((r = lin_calc1(b, pt2, u1, bnd_w, slot, s))) return r;
        if ((r = lin_calc1(b, pt2, pt2, nullptr, slot, s))) return r;
        CK(axpbz(pt2, pt2, (1.0 - th) * mu, pt2, 0.0, NV, s));
        // tmp = J^T(v1, l), p = J^T(z, v1), h1 = J^T(v1, lz)
        const double *ju[3] = {u1, in, u1}, *jv[3] = {lh, u1, zl};
        if ((r = lin_jac3(b, ju, jv, -1.0, slot, s))) return r;
        double *tmp = jf, *pl = jf + V, *h1 = jf + 2 * (size_t)V;
        if ((r = lin_calc1(b, pl, pl, nullptr, slot, s))) return r;
        CK(axpbz(h1, h1, k1, pl, k1, NV, s));
        CK(axpbz(h1, h1, 1.0, tmp, k2, NV, s));
        CK(axpbz(h1, h1, -1.0, h1, 0.0, NV, s));
        CK(axpbz(u1, pt1, 1.0, pt1, 0.0, NV, s));
        CK(axpbz(u1, u1, 1.0, pt2, 1.0, NV, s));
        CK(axpbz(u1, u1, 1.0, h1, 1.0, NV, s));
        // set_bnd (src/proj.cpp:110-133): inner values kept, boundary = bnd_u
        CK(gather(b->lx.as<double>(), o->rs, u1, V, o->imap(), o->rs, 1, s));
        CK(p2u(u1, V, b->lx.as<double>(), o->rs, bnd_u, o->os, o->p2io.as<int>(), o->isb.as<int>(), V, 1, s));
    }
    b->nslots = slot;
    b->last_stream = s;
    return PHG_OK;
}

}  // namespace

static int bv_linear(phg_barvortex b, int kind, double *u1, const double *u, const double *z, const double *bnd_u,
                     const double *bnd_w, void *stream) {
    if (!b || !u1 || !u || !z) return fail(PHG_ERR_ARG, "NULL argument");
    phg_ops_s *o = b->o;
    cudaStream_t s = o->str(stream);
    Stage st(o, s);
    const double *du, *dz, *dbu, *dbw, *dacc = nullptr; double *d1;
    CK(st.in(u, o->V, &du)); CK(st.in(z, o->V, &dz));
    CK(st.in(bnd_u, o->os, &dbu)); CK(st.in(bnd_w, o->os, &dbw));
    if (kind == 1) CK(st.in(u1, o->V, &dacc));   // calc_L_1 adds into u1
    CK(st.out(u1, o->V, &d1));
    if (kind == 1 && dacc != d1) CK(cudaMemcpyAsync(d1, dacc, 8 * (size_t)o->V, cudaMemcpyDeviceToDevice, s));
    if (o->os == 0) { dbu = nullptr; dbw = nullptr; }
    int r = lin_dev(b, kind, d1, du, dz, dbu, dbw, s);
    if (r) return r;
    CK(st.finish());
    if (!st.host) return PHG_OK;
    return check_stats(o, b->nslots, s, nullptr, b->each.data());
}

extern "C" int phg_barvortex_calc_L(phg_barvortex b, double *u1, const double *u, const double *z,
                                    const double *bnd_u, const double *bnd_w, void *stream) {
    PHG_API_BEGIN
    return bv_linear(b, 0, u1, u, z, bnd_u, bnd_w, stream);
    PHG_API_END
}

extern "C" int phg_barvortex_calc_L_1(phg_barvortex b, double *u1, const double *u, const double *z,
                                      const double *bnd_u, const double *bnd_w, void *stream) {
    PHG_API_BEGIN
    return bv_linear(b, 1, u1, u, z, bnd_u, bnd_w, stream);
    PHG_API_END
}

extern "C" int phg_barvortex_calc_LT(phg_barvortex b, double *v1, const double *v, const double *z,
                                     const double *bnd_u, const double *bnd_w, void *stream) {
    PHG_API_BEGIN
    return bv_linear(b, 2, v1, v, z, bnd_u, bnd_w, stream);
    PHG_API_END
}

extern "C" int phg_barvortex_last_stats(phg_barvortex b, int *il, int *ia, int *imj, int *iml, double *worst) {
    PHG_API_BEGIN
    if (!b) return fail(PHG_ERR_ARG, "NULL handle");
    phg_ops_s *o = b->o;
    cudaStream_t ls = b->last_stream ? b->last_stream : o->stream;
    int r = check_stats(o, b->nslots, ls, nullptr, b->each.data());
    if (b->agg_pending) {   // every step of the runs since the last check
        int r2 = bv_check_agg(b, ls);
        if (r2) r = r2;
    }
    // slot layout: 0,1 mass L (calc1 x2); then per Picard iteration: J, A, L
    int l = 0, a = 0, mj = 0, ml = 0;
    double wr = 0.0;
    for (int k = 0; k < b->nslots; ++k) {
        const GmresStats &g = b->each[k];
        wr = max_keep_nan(wr, g.relres);
        if (k < 2) ml += g.iters;
        else if ((k - 2) % 3 == 0) mj += g.iters;
        else if ((k - 2) % 3 == 1) a += g.iters;
        else l += g.iters;
    }
    if (il) *il = l;
    if (ia) *ia = a;
    if (imj) *imj = mj;
    if (iml) *iml = ml;
    if (worst) *worst = wr;
    return r;
    PHG_API_END
}

// ------------------------------------------------------------- baroclin ---
// The 4rs x 4rs system of Baroclin (examples/baroclin.cpp:107-243) is stored
// vertex-interleaved: the reference's unknown q*rs + i (blocks w1 | w2 | u1 |
// u2) is 4i + q, so one ELL row slice covers the four fields of a vertex.
// The w rows carry the mass matrix times 1/tau, the u rows (M w - L u) only
// the mass matrix, so a relative residual over all rows would leave the u
// rows 1/tau times less accurate: the u rows and the u unknowns are scaled
// by su, the power of two nearest 1/tau (exact scaling; the solution is the
// same).
namespace {
// one interleaved 4rs block system (A_ of the step or Ab_ of the inverse
// linearised step) with its block preconditioner and boundary columns
struct BcSystem {
    DBuf col, val, a32, dinv, as64, as32, cpl64, cpl32;
    DevSolveOp op;
    ColsBufs bc[4];
    BcCols bcols;
};
}  // namespace

struct phg_baroclin_s {
    phg_ops_s *o = nullptr;
    phg_bc_conf c{};
    double theta = 0.5;
    double su = 1.0;
    BcSystem fwd, back;
    bool have_back = false;
    DBuf lh;
    // linearised steps: background fields, their Laplacians, 10 Jacobian pairs
    DBuf Z, dZ, lju, ljv, ljsol, ljac;
    DBuf U, w, dw, FC, un, wn, un1, ju, jv, jsol, jac, FG, MFG, rp, x, xi, nr, done;
    std::vector<GmresStats> each;   // the last step's solve records, one per slot
    int nslots = 0;
    int *hdone = nullptr;   // pinned copy of the Picard stop flag
    ~phg_baroclin_s() { if (hdone) cudaFreeHost(hdone); }
};

namespace {

BaroclinParams bc_params(const phg_bc_conf &c, double theta, bool backward) {
    BaroclinParams bp;
    bp.tau = c.tau; bp.sigma = c.sigma; bp.mu = c.mu; bp.sigma1 = c.sigma1; bp.mu1 = c.mu1;
    bp.alpha = c.alpha; bp.theta = theta; bp.backward = backward;
    return bp;
}

// assemble one 4rs block system, interleave it (unknown q*rs + i -> 4i + q),
// scale the u rows and u unknowns by su and set up its preconditioner
int build_bc_system(phg_ops_s *o, const BaroclinParams &bp, double su, BcSystem &S) {
    const int rs = o->rs, n = 4 * rs;
    Csr A, bcol[4];
    assemble_baroclin(o->mesh->m, bp, A, bcol);
    // interleave: block-order row/column q*rs + i -> 4i + q, columns ascending
    std::vector<std::vector<std::pair<int, double>>> rows(n);
    for (int r = 0; r < A.n; ++r) {
        const int nr_ = 4 * (r % rs) + r / rs;
        for (int k = A.ptr[r]; k < A.ptr[r + 1]; ++k) rows[nr_].push_back({4 * (A.col[k] % rs) + A.col[k] / rs, A.val[k]});
    }
    int W = 0;
    for (int i = 0; i < n; ++i) {
        auto &row = rows[i];
        std::sort(row.begin(), row.end());
        W = std::max(W, (int)row.size());
        for (auto &e : row) {
            const bool urow = (i & 3) >= 2, ucol = (e.first & 3) >= 2;
            if (urow && !ucol) e.second *= su;
            if (!urow && ucol) e.second /= su;
        }
    }
    std::vector<int> col((size_t)W * n);
    std::vector<double> val((size_t)W * n, 0.0), dinv(n, 0.0);
    for (int i = 0; i < n; ++i) {
        int k = 0;
        for (auto &e : rows[i]) {
            col[(size_t)k * n + i] = e.first;
            val[(size_t)k * n + i] = e.second;
            if (e.first == i) dinv[i] = 1.0 / e.second;
            ++k;
        }
        for (; k < W; ++k) col[(size_t)k * n + i] = i;
        if (!(dinv[i] != 0.0) || !std::isfinite(dinv[i])) return fail(PHG_ERR_ARG, "zero diagonal in row %d", i);
    }
    CK(upload(S.col, col)); CK(upload(S.val, val)); CK(upload(S.a32, to_f32(val))); CK(upload(S.dinv, dinv));
    DevSolveOp &op = S.op;
    op.A.n = n; op.A.W = W; op.A.col = S.col.as<int>(); op.A.val = S.val.as<double>();
    op.a32 = S.a32.as<float>(); op.dinv = S.dinv.as<double>();
    if (o->L.op.mgd) {
        // w rows: Jacobi; u rows: -L u = r_u - M w with the Laplacian's multigrid
        op.mg = o->L.op.mg; op.mgd = o->L.op.mgd;
        op.block4 = 1;
        std::vector<double> mv;
        to_ell(o->mesh->ops.idt, o->W, nullptr, mv);
        for (auto &x : mv) x *= su;
        CK(upload(S.cpl64, mv)); CK(upload(S.cpl32, to_f32(mv)));
        op.cpl = o->ell(S.cpl64); op.cpl32 = S.cpl32.as<float>();
    } else {
        // small meshes (no multigrid hierarchy): Jacobi-scaled GMRES
        std::vector<double> as64(val.size());
        for (size_t e = 0; e < val.size(); ++e) as64[e] = val[e] * dinv[col[e]];
        CK(upload(S.as64, as64)); CK(upload(S.as32, to_f32(as64)));
        op.as64 = S.as64.as<double>(); op.as32 = S.as32.as<float>();
    }
    int r;
    for (int q = 0; q < 4; ++q) {
        if ((r = build_cols(bcol[q], S.bc[q]))) return r;
        S.bcols.c[q] = S.bc[q].c;
    }
    return PHG_OK;
}

}  // namespace

extern "C" int phg_baroclin_create(phg_ops o, const phg_bc_conf *c, const double *coriolis, phg_baroclin *out) {
    PHG_API_BEGIN
    if (!o || !c || !out) return fail(PHG_ERR_ARG, "NULL argument");
    if (!(c->tau > 0) || c->picard_iters < 1 || c->picard_iters > 30) return fail(PHG_ERR_ARG, "bad configuration");
    auto b = std::make_unique<phg_baroclin_s>();
    b->o = o;
    b->c = *c;
    b->each.assign(64, GmresStats{});   // 2 + 2 x picard_iters <= 62 solve records a step
    const int rs = o->rs, n = 4 * rs;
    b->su = std::ldexp(1.0, (int)std::lround(std::log2(1.0 / c->tau)));
    int r;
    if ((r = build_bc_system(o, bc_params(*c, b->theta, false), b->su, b->fwd))) return r;
    std::vector<double> lh(o->V, 0.0);
    if (coriolis) {
        if (is_device_ptr(coriolis)) CK(cudaMemcpy(lh.data(), coriolis, 8 * lh.size(), cudaMemcpyDeviceToHost));
        else memcpy(lh.data(), coriolis, 8 * lh.size());
    }
    CK(upload(b->lh, lh));
    const size_t V = o->V;
    DBuf *two[] = {&b->U, &b->w, &b->dw, &b->FC, &b->un, &b->wn, &b->un1};
    for (DBuf *d : two) CK(d->ensure(8 * 2 * V));
    CK(b->ju.ensure(8 * 5 * V)); CK(b->jv.ensure(8 * 5 * V));
    CK(b->jsol.ensure(8 * 5 * 8 * (size_t)rs)); CK(b->jac.ensure(8 * 5 * (size_t)rs));
    CK(b->FG.ensure(8 * 2 * (size_t)rs)); CK(b->MFG.ensure(8 * 2 * (size_t)rs)); CK(b->xi.ensure(8 * 2 * (size_t)rs));
    CK(b->rp.ensure(8 * (size_t)n)); CK(b->x.ensure(8 * (size_t)n));
    CK(b->nr.ensure(16)); CK(b->done.ensure(4));
    CK(cudaHostAlloc(&b->hdone, sizeof(int), cudaHostAllocDefault));
    o->refs++;
    *out = b.release();
    return PHG_OK;
    PHG_API_END
}

extern "C" void phg_baroclin_destroy(phg_baroclin b) {
    PHG_API_BEGIN
    if (!b) return;
    phg_ops_s *o = b->o;
    cudaStreamSynchronize(o->stream);
    delete b;
    ops_release(o);
    PHG_API_END_VOID
}

namespace {

// One Crank-Nicolson / Picard step (examples/baroclin.cpp:445-606), all
// arguments on the device.
int bc_step_dev(phg_baroclin_s *b, double *u11, double *u21, const double *u1, const double *u2,
                const double *bnd, const double *f, const double *g, cudaStream_t s) {
    NvtxRange nvtx("phg:baroclin_step");
    phg_ops_s *o = b->o;
    const int V = o->V, rs = o->rs, os = o->os;
    const phg_bc_conf &c = b->c;
    const double th = b->theta;
    int r, slot = 0;
    double *U = b->U.as<double>(), *w = b->w.as<double>(), *dw = b->dw.as<double>();
    double *FC = b->FC.as<double>(), *GC = FC + V;
    double *un = b->un.as<double>(), *wn = b->wn.as<double>(), *un1 = b->un1.as<double>();
    double *xi = b->xi.as<double>(), *x = b->x.as<double>(), *rp = b->rp.as<double>();
    const int *p2io = o->p2io.as<int>(), *isb = o->isb.as<int>();
    // inputs first: the outputs may alias them
    CK(cudaMemcpyAsync(U, u1, 8 * (size_t)V, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(U + V, u2, 8 * (size_t)V, cudaMemcpyDeviceToDevice, s));
    // w = L(u), dw = L(w), both layers at once, with the boundary values bnd
    if ((r = laplace_calc2_dev(o, xi, rs, U, V, 2, slot++, s, o->tol))) return r;
    CK(p2u(w, V, xi, rs, bnd, 0, p2io, isb, V, 2, s));
    if ((r = laplace_calc2_dev(o, xi, rs, w, V, 2, slot++, s, o->tol))) return r;
    CK(p2u(dw, V, xi, rs, bnd, 0, p2io, isb, V, 2, s));
    BcCoef k;
    k.a = -0.5 * (1.0 - th) * c.sigma;
    k.b = 0.5 * (1.0 - th) * c.sigma;
    k.mu1t = c.mu * (1.0 - th);
    k.itau = 1.0 / c.tau;
    k.g_u2 = -c.alpha * c.alpha / c.tau;
    k.g_w2 = -c.alpha * c.alpha * c.mu1 * (1 - th);
    k.g_u2b = c.alpha * c.alpha * c.sigma1 * (1 - th);
    k.alpha2 = c.alpha * c.alpha;
    k.ga = k.gb = k.a;
    CK(bc_fcgc(FC, GC, w, w + V, dw, dw + V, U + V, f, g, k, V, s));
    CK(cudaMemcpyAsync(un, U, 16 * (size_t)V, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(wn, w, 16 * (size_t)V, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemsetAsync(b->done.p, 0, 4, s));
    double *F = b->FG.as<double>(), *G = F + rs, *MF = b->MFG.as<double>(), *MG = MF + rs;
    for (int it = 0; it < c.picard_iters; ++it) {
        // the five Jacobians J(U1, W1 + l), J(U2, W2), J(U1, W2), J(U2, W1 + l), J(U1, U2)
        CK(bc_jin(b->ju.as<double>(), b->jv.as<double>(), U, U + V, w, w + V, un, un + V, wn, wn + V,
                  b->lh.as<double>(), th, V, s));
        if ((r = jacobian_derivs_dev(o, b->ju.as<double>(), b->jv.as<double>(), V, b->jsol.as<double>(), 5, slot++, s,
                                     o->tol, o->jq_mode == 1, it > 0)))
            return r;
        CK(jac_combine(b->jsol.as<double>(), rs, rs, b->jac.as<double>(), rs, nullptr, 0, nullptr, 5, s));
        CK(bc_fg(F, G, b->jac.as<double>(), FC, GC, o->imap(), k.alpha2, rs, s));
        // rp = [M F, M G, 0, 0] - boundary columns * bnd, interleaved
        CK(apply_op(o->ML.op.A, DevCols(), F, rs, nullptr, nullptr, 0, nullptr, MF, rs, 2, s));
        CK(bc_rhs(rp, MF, MG, b->fwd.bcols, os ? bnd : nullptr, b->su, rs, s));
        // warm start from the current iterate
        CK(bc_pack(x, wn, wn + V, un, un + V, o->imap(), b->su, rs, s));
        if ((r = solve(o, b->fwd.op, rp, x, 1, 4 * rs, o->tol, slot++, s))) return r;
        CK(bc_unpack(wn, wn + V, un1, un1 + V, x, os ? bnd : nullptr, p2io, isb, 1.0 / b->su, V, s));
        // nr = max(dist(u1_n1, u1_n), dist(u2_n1, u2_n)); commit unless stopped
        if ((r = norm_dev(o, un1, un, 2, b->nr.as<double>(), true, true, s))) return r;
        CK(bc_commit(un, un1, b->nr.as<double>(), b->done.as<int>(), c.picard_tol, 2 * V, s));
        // the reference leaves the loop once max(nr) < tol (examples/baroclin.cpp:600): read the
        // flag so that converged steps do not run the remaining iterations
        if (it + 1 < c.picard_iters) {
            CK(cudaMemcpyAsync(b->hdone, b->done.p, sizeof(int), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            if (*b->hdone) break;
        }
    }
    CK(cudaMemcpyAsync(u11, un, 8 * (size_t)V, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(u21, un + V, 8 * (size_t)V, cudaMemcpyDeviceToDevice, s));
    b->nslots = slot;
    return PHG_OK;
}

}  // namespace

namespace {

// Baroclin::calc_L (kind 0: one iteration, forward matrix A_,
// examples/baroclin.cpp:620-802) and calc_L_1 (kind 1: up to 10 iterations,
// backward matrix Ab_, :804-986), linearised around (z1, z2); device pointers
int bc_lin_dev(phg_baroclin_s *b, int kind, double *u11, double *u21, const double *u1, const double *u2,
               const double *z1, const double *z2, const double *bnd, cudaStream_t s) {
    phg_ops_s *o = b->o;
    const int V = o->V, rs = o->rs, os = o->os;
    const phg_bc_conf &c = b->c;
    const double th = b->theta, sg = c.sigma, mu = c.mu, tau = c.tau, al = c.alpha;
    int r, slot = 0;
    if (kind == 1 && !b->have_back) {
        if ((r = build_bc_system(o, bc_params(c, th, true), b->su, b->back))) return r;
        b->have_back = true;
    }
    const BcSystem &S = kind == 0 ? b->fwd : b->back;
    CK(b->Z.ensure(16 * (size_t)V)); CK(b->dZ.ensure(16 * (size_t)V));
    CK(b->lju.ensure(80 * (size_t)V)); CK(b->ljv.ensure(80 * (size_t)V));
    CK(b->ljsol.ensure(8 * 80 * (size_t)rs)); CK(b->ljac.ensure(80 * (size_t)rs));
    double *U = b->U.as<double>(), *w = b->w.as<double>(), *dw = b->dw.as<double>();
    double *FC = b->FC.as<double>(), *GC = FC + V, *Z = b->Z.as<double>(), *dZ = b->dZ.as<double>();
    double *un = b->un.as<double>(), *wn = b->wn.as<double>(), *un1 = b->un1.as<double>();
    double *xi = b->xi.as<double>(), *x = b->x.as<double>(), *rp = b->rp.as<double>();
    const int *p2io = o->p2io.as<int>(), *isb = o->isb.as<int>();
    // inputs first: the outputs may alias them
    CK(cudaMemcpyAsync(U, u1, 8 * (size_t)V, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(U + V, u2, 8 * (size_t)V, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(Z, z1, 8 * (size_t)V, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(Z + V, z2, 8 * (size_t)V, cudaMemcpyDeviceToDevice, s));
    // w = L(u), dw = L(w), dz = L(z), all with the boundary values bnd
    const double *src[3] = {U, w, Z};
    double *dst[3] = {w, dw, dZ};
    for (int k = 0; k < 3; ++k) {
        if ((r = laplace_calc2_dev(o, xi, rs, src[k], V, 2, slot++, s, o->tol))) return r;
        CK(p2u(dst[k], V, xi, rs, bnd, 0, p2io, isb, V, 2, s));
    }
    BcCoef k;
    if (kind == 0) {
        k.a = -0.5 * (1.0 - th) * sg; k.b = 0.5 * (1.0 - th) * sg; k.ga = k.gb = k.a;
        k.mu1t = mu * (1.0 - th);
        k.g_w2 = -al * al * c.mu1 * (1 - th); k.g_u2b = al * al * c.sigma1 * (1 - th);
    } else {
        k.a = 0.5 * th * sg; k.b = -0.5 * th * sg; k.ga = k.gb = 0.5 * th * sg;
        k.mu1t = -mu * th;
        k.g_w2 = al * al * c.mu1 * th; k.g_u2b = -al * al * c.sigma1 * th;
    }
    k.itau = 1.0 / tau;
    k.g_u2 = -al * al / tau;
    k.alpha2 = 0.0;
    CK(bc_fcgc(FC, GC, w, w + V, dw, dw + V, U + V, nullptr, nullptr, k, V, s));
    CK(cudaMemcpyAsync(un, U, 16 * (size_t)V, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(wn, w, 16 * (size_t)V, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemsetAsync(b->done.p, 0, 4, s));
    double *F = b->FG.as<double>(), *G = F + rs, *MF = b->MFG.as<double>(), *MG = MF + rs;
    const double wa = kind == 0 ? 1.0 - th : th, wb = kind == 0 ? th : 1.0 - th;
    const double ka2 = kind == 0 ? al * al : -al * al;
    const int iters = kind == 0 ? 1 : 10;
    for (int it = 0; it < iters; ++it) {
        CK(bc_lin_jin(b->lju.as<double>(), b->ljv.as<double>(), U, w, un, wn, Z, dZ, b->lh.as<double>(), wa, wb, V, s));
        if ((r = jacobian_derivs_dev(o, b->lju.as<double>(), b->ljv.as<double>(), V, b->ljsol.as<double>(), 10, slot++,
                                     s, o->tol)))
            return r;
        CK(jac_combine(b->ljsol.as<double>(), rs, rs, b->ljac.as<double>(), rs, nullptr, 0, nullptr, 10, s));
        CK(bc_lin_fg(F, G, b->ljac.as<double>(), FC, GC, o->imap(), kind, ka2, rs, s));
        CK(apply_op(o->ML.op.A, DevCols(), F, rs, nullptr, nullptr, 0, nullptr, MF, rs, 2, s));
        CK(bc_rhs(rp, MF, MG, S.bcols, os ? bnd : nullptr, b->su, rs, s));
        CK(bc_pack(x, wn, wn + V, un, un + V, o->imap(), b->su, rs, s));
        if ((r = solve(o, S.op, rp, x, 1, 4 * rs, o->tol, slot++, s))) return r;
        CK(bc_unpack(wn, wn + V, un1, un1 + V, x, os ? bnd : nullptr, p2io, isb, 1.0 / b->su, V, s));
        if ((r = norm_dev(o, un1, un, 2, b->nr.as<double>(), true, true, s))) return r;
        CK(bc_commit(un, un1, b->nr.as<double>(), b->done.as<int>(), 1e-8, 2 * V, s));   // :797, :981
        if (it + 1 < iters) {
            CK(cudaMemcpyAsync(b->hdone, b->done.p, sizeof(int), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            if (*b->hdone) break;
        }
    }
    CK(cudaMemcpyAsync(u11, un, 8 * (size_t)V, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(u21, un + V, 8 * (size_t)V, cudaMemcpyDeviceToDevice, s));
    b->nslots = slot;
    return PHG_OK;
}

}  // namespace

static int bc_linear(phg_baroclin b, int kind, double *u11, double *u21, const double *u1, const double *u2,
                     const double *z1, const double *z2, const double *bnd, void *stream) {
    if (!b || !u11 || !u21 || !u1 || !u2 || !z1 || !z2) return fail(PHG_ERR_ARG, "NULL argument");
    phg_ops_s *o = b->o;
    cudaStream_t s = o->str(stream);
    Stage st(o, s);
    const double *d1, *d2, *dz1, *dz2, *db; double *o1, *o2;
    CK(st.in(u1, o->V, &d1)); CK(st.in(u2, o->V, &d2)); CK(st.in(z1, o->V, &dz1)); CK(st.in(z2, o->V, &dz2));
    CK(st.in(bnd, o->os, &db));
    CK(st.out(u11, o->V, &o1)); CK(st.out(u21, o->V, &o2));
    if (o->os == 0) db = nullptr;
    int r = bc_lin_dev(b, kind, o1, o2, d1, d2, dz1, dz2, db, s);
    if (r) return r;
    CK(st.finish());
    if (!st.host) return PHG_OK;
    return check_stats(o, b->nslots, s, nullptr, b->each.data());
}

extern "C" int phg_baroclin_calc_L(phg_baroclin b, double *u11, double *u21, const double *u1, const double *u2,
                                   const double *z1, const double *z2, const double *bnd, void *stream) {
    PHG_API_BEGIN
    return bc_linear(b, 0, u11, u21, u1, u2, z1, z2, bnd, stream);
    PHG_API_END
}

extern "C" int phg_baroclin_calc_L_1(phg_baroclin b, double *u11, double *u21, const double *u1, const double *u2,
                                     const double *z1, const double *z2, const double *bnd, void *stream) {
    PHG_API_BEGIN
    return bc_linear(b, 1, u11, u21, u1, u2, z1, z2, bnd, stream);
    PHG_API_END
}

extern "C" int phg_baroclin_calc(phg_baroclin b, double *u11, double *u21, const double *u1, const double *u2,
                                 const double *bnd, const double *f, const double *g, void *stream) {
    PHG_API_BEGIN
    if (!b || !u11 || !u21 || !u1 || !u2) return fail(PHG_ERR_ARG, "NULL argument");
    phg_ops_s *o = b->o;
    cudaStream_t s = o->str(stream);
    Stage st(o, s);
    const double *d1, *d2, *db, *df, *dg; double *o1, *o2;
    CK(st.in(u1, o->V, &d1)); CK(st.in(u2, o->V, &d2)); CK(st.in(bnd, o->os, &db));
    CK(st.in(f, o->V, &df)); CK(st.in(g, o->V, &dg));
    CK(st.out(u11, o->V, &o1)); CK(st.out(u21, o->V, &o2));
    if (o->os == 0) db = nullptr;
    int r = bc_step_dev(b, o1, o2, d1, d2, db, df, dg, s);
    if (r) return r;
    CK(st.finish());
    if (!st.host) return PHG_OK;
    return check_stats(o, b->nslots, s, nullptr, b->each.data());
    PHG_API_END
}

// ------------------------------------------------------- no allocation ---
// phg_laplace_calc2_noalloc: SphereLaplace::calc2 for callers that cannot
// let the library allocate device memory -- e.g. applications whose device
// memory is owned by their own pool or allocator, or loops where the device
// synchronisation a cudaMalloc brings would stall their other streams.  The
// right-hand side and the GMRES workspace live in the fixed array below,
// which every GPU that loads this library holds until the process exits.
namespace {

constexpr size_t NOALLOC_BYTES = 16u << 20;   // 16 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

std::mutex g_noalloc_mu;
void *g_noalloc_ptr[64] = {nullptr};

// Device address of the scratch array on `dev`, looked up once per device
// with that device current (a host-side use of the symbol's name is not a
// device address).
int noalloc_scratch(int dev, unsigned char **out) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (dev < 0 || dev >= 64) return fail(PHG_ERR_ARG, "device ordinal %d out of range", dev);
    if (!g_noalloc_ptr[dev]) {
        int cur = 0;
        CK(cudaGetDevice(&cur));
        if (cur != dev) CK(cudaSetDevice(dev));
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (cur != dev) cudaSetDevice(cur);
        if (e != cudaSuccess) return fail(PHG_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        g_noalloc_ptr[dev] = p;
    }
    *out = (unsigned char *)g_noalloc_ptr[dev];
    return PHG_OK;
}

}  // namespace

extern "C" int phg_laplace_calc2_noalloc(phg_ops o, double *ans, const double *F, void *stream) {
    PHG_API_BEGIN
    if (!o || !ans || !F) return fail(PHG_ERR_ARG, "NULL argument");
    if (!is_device_ptr(ans) || !is_device_ptr(F))
        return fail(PHG_ERR_ARG, "phg_laplace_calc2_noalloc takes device pointers only");
    const size_t al = 256;
    const size_t rhs_bytes = (8 * (size_t)o->rs + al - 1) / al * al;
    const size_t work_bytes = gmres_work_bytes(o->ML.op, 1, o->restart, prec_of(o));
    const size_t need = rhs_bytes + work_bytes;
    if (need > NOALLOC_BYTES)
        return fail(PHG_ERR_ARG,
                    "phg_laplace_calc2_noalloc needs %zu bytes of scratch for %d inner points at restart %d; "
                    "it holds %zu (16 MiB: the Chebyshev mass solve up to level 7 in FP64, a GMRES(30) one up "
                    "to level 6)",
                    need, o->rs, o->restart, NOALLOC_BYTES);
    unsigned char *base = nullptr;
    int r = noalloc_scratch(o->dev, &base);
    if (r) return r;
    cudaStream_t s = o->str(stream);
    double *rhs = (double *)base;
    void *work = base + rhs_bytes;
    // rhs = L F_in + B3 F_bnd ; ans = M_L^-1 rhs from a zero start.  The solve
    // record goes to the handle's slot 0 (allocated with the handle), where
    // phg_ops_check and phg_ops_last_solve read it, as for phg_laplace_calc2.
    CK(apply_op(o->L.op.A, o->bnd3.c, F, o->V, o->imap(), F, o->V, o->bmap(), rhs, o->rs, 1, s));
    CK(cudaMemsetAsync(ans, 0, 8 * (size_t)o->rs, s));
    CK(gmres_solve(o->ML.op, rhs, ans, 1, o->rs, o->restart, o->max_iter, mass_tol(o), prec_of(o), work,
                   o->stats.as<GmresStats>(), s, /*no_alloc=*/true, o->max_sms, nullptr, o->wait_limit));
    o->stats_pending = true;
    o->pending_slots = std::max(o->pending_slots, 1);
    return PHG_OK;
    PHG_API_END
}
