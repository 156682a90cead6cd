// api.cu -- the C ABI of libraftgb (declared in include/raftgb.h).
//
// Each entry point validates its rg_image arguments, looks up (or builds and
// caches) the plan of per-view constants for the geometry, takes its scratch
// from the caller's workspace or from stream-ordered memory, and queues the
// kernels on the caller's stream.  No entry point synchronises, except the
// *_host wrappers and rg_dda_trace.
#include <cuda_runtime.h>
#include <ctype.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <algorithm>
#include <complex>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "rg_internal.cuh"

namespace rg {

// ----------------------------------------------------------------------------
// Errors

static thread_local std::string g_err;

int set_error(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

bool pdl_enabled()
{
    static const bool on = [] {
        const char *e = getenv("RG_PDL");
        return !(e && !strcmp(e, "0"));
    }();
    return on;
}

int cuda_error(cudaError_t e, const char *what)
{
    return set_error(RG_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

// ----------------------------------------------------------------------------
// Scratch

int scratch_begin(Scratch &s, void *ws, size_t ws_bytes, size_t need, cudaStream_t st)
{
    s.stream = st;
    s.off = 0;
    s.owned = false;
    s.base = nullptr;
    s.size = 0;
    if (need == 0) return RG_OK;
    if (ws) {
        if (((uintptr_t)ws & 255) != 0)
            return set_error(RG_EINVAL, "workspace must be 256-byte aligned");
        if (ws_bytes < need)
            return set_error(RG_EWORKSPACE, "workspace of %zu bytes, %zu needed", ws_bytes, need);
        s.base = (char *)ws;
        s.size = ws_bytes;
        return RG_OK;
    }
    // RG_TEST_FAIL_ALLOC=1 (a test switch) makes this allocation fail as an
    // exhausted pool would, so tests can see the call report RG_ENOMEM and
    // leave its output and the library's state untouched
    cudaError_t e = test_switch("RG_TEST_FAIL_ALLOC") ? cudaErrorMemoryAllocation
                                                      : cudaMallocAsync((void **)&s.base, need, st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(RG_ENOMEM, "stream-ordered allocation of %zu bytes failed: %s", need,
                         cudaGetErrorString(e));
    }
    s.size = need;
    s.owned = true;
    return RG_OK;
}

void scratch_end(Scratch &s)
{
    if (s.owned && s.base) cudaFreeAsync(s.base, s.stream);
    s.base = nullptr;
    s.owned = false;
}

// Sum of pieces as Scratch::take lays them out.
static size_t ws_total(std::initializer_list<size_t> pieces)
{
    size_t t = 0;
    for (size_t p : pieces) t = Scratch::align(t) + p;
    return t ? Scratch::align(t) : 0;
}

// Quad scratch of the paired gathers for nz sinograms of this shape (an
// even view count; whether the geometry pairs is known only to its plan).
static size_t quads_ws(const rg_image &sino, int nz = 1)
{
    return sino.columns % 2 == 0 ? gather_quads_bytes(sino.columns, sino.lines, nz) : 0;
}

// ----------------------------------------------------------------------------
// Caches (per device, keyed by the raw bytes of the geometry).

template <class T>
struct Cache {
    std::mutex mu;
    std::list<std::pair<std::string, std::shared_ptr<T>>> items;   // MRU first
    size_t cap = 64;
    std::shared_ptr<T> find(const std::string &k)
    {
        for (auto it = items.begin(); it != items.end(); ++it)
            if (it->first == k) {
                items.splice(items.begin(), items, it);
                return items.front().second;
            }
        return nullptr;
    }
    void put(const std::string &k, std::shared_ptr<T> v)
    {
        items.emplace_front(k, std::move(v));
        while (items.size() > cap) items.pop_back();
    }
};

struct KeyBuilder {
    std::string s;
    template <class T> KeyBuilder &add(const T &v)
    {
        s.append(reinterpret_cast<const char *>(&v), sizeof v);
        return *this;
    }
};

static int current_device()
{
    int d = 0;
    cudaGetDevice(&d);
    return d;
}

// One device int per GPU that kernels with bounded waits or in-kernel
// checks OR their error bits into (1: a window check failed and a strip was
// skipped; 2: an mbarrier wait ran out).  Allocated with the first plan on
// the device, so no allocation happens inside a stream capture.
static std::mutex g_errw_mu;
static std::map<int, int *> g_errw;

int *device_error_word()
{
    const int d = current_device();
    std::lock_guard<std::mutex> lock(g_errw_mu);
    auto it = g_errw.find(d);
    return it == g_errw.end() ? nullptr : it->second;
}

int ensure_device_error_word()
{
    const int d = current_device();
    std::lock_guard<std::mutex> lock(g_errw_mu);
    if (g_errw.count(d)) return RG_OK;
    int *w = nullptr;
    RG_CK(cudaMalloc(&w, sizeof(int)));
    RG_CK(cudaMemset(w, 0, sizeof(int)));
    g_errw[d] = w;
    return RG_OK;
}

struct PlanHolder {
    SSPlan p;
    ~PlanHolder() { ss_plan_free(p); }
};

static Cache<PlanHolder> g_plans;

// Plan over views {first, first + stride, ...} of the geometry.
static int get_plan(const SSGeom &g, int stride, int first, std::shared_ptr<PlanHolder> &out)
{
    KeyBuilder kb;
    kb.add(current_device()).add(g.N).add(g.R).add(g.A).add(g.itl_x).add(g.itl_y).add(g.ibr_x)
        .add(g.ibr_y).add(g.stl_x).add(g.stl_y).add(g.sbr_x).add(g.sbr_y).add(stride).add(first);
    std::lock_guard<std::mutex> lock(g_plans.mu);
    out = g_plans.find(kb.s);
    if (out) return RG_OK;
    std::vector<int> views;
    for (int j = first; j < g.A; j += stride) views.push_back(j);
    auto h = std::make_shared<PlanHolder>();
    int rc = ss_plan_build(h->p, g, views.data(), (int)views.size());
    if (rc != RG_OK) return rc;
    g_plans.put(kb.s, h);
    out = h;
    return RG_OK;
}

struct DevTable {
    void *p = nullptr;
    float h0 = 0.f;   // Ram-Lak centre tap, or the FFT filter's DC gain / 2^fft_p
    int fft_p = 0;    // filter by FFT of size 2^fft_p (0: direct-sum taps)
    bool fft_circ = false;   // ... as a circular convolution of length 2^fft_p
    ~DevTable() { if (p) cudaFree(p); }
};
static Cache<DevTable> g_tables;

// Device copy of a host table, cached by key.
static int get_table(const std::string &key, const void *host, size_t bytes,
                     std::shared_ptr<DevTable> &out)
{
    KeyBuilder kb;
    kb.add(current_device());
    kb.s += key;
    std::lock_guard<std::mutex> lock(g_tables.mu);
    out = g_tables.find(kb.s);
    if (out) return RG_OK;
    auto t = std::make_shared<DevTable>();
    RG_CK(cudaMalloc(&t->p, bytes));
    RG_CK(cudaMemcpy(t->p, host, bytes, cudaMemcpyHostToDevice));
    g_tables.put(kb.s, t);
    out = t;
    return RG_OK;
}

// Device copy of a host table that `fill` builds only when the key is not
// cached yet (for tables that are costly to compute).
template <class F>
static int get_table_lazy(const std::string &key, F fill, std::shared_ptr<DevTable> &out)
{
    // fill(bytes, table): the host bytes, and the table's scalar fields
    KeyBuilder kb;
    kb.add(current_device());
    kb.s += key;
    std::lock_guard<std::mutex> lock(g_tables.mu);
    out = g_tables.find(kb.s);
    if (out) return RG_OK;
    auto t = std::make_shared<DevTable>();
    std::vector<unsigned char> host;
    fill(host, *t);
    RG_CK(cudaMalloc(&t->p, host.size()));
    RG_CK(cudaMemcpy(t->p, host.data(), host.size(), cudaMemcpyHostToDevice));
    g_tables.put(kb.s, t);
    out = t;
    return RG_OK;
}

// ----------------------------------------------------------------------------
// Validation helpers

static int check_image(const rg_image &im, const char *what)
{
    if (!im.data) return set_error(RG_EINVAL, "%s: null data pointer", what);
    if (im.lines < 1 || im.columns < 1)
        return set_error(RG_EINVAL, "%s: empty (%d x %d)", what, im.lines, im.columns);
    if (im.line_stride == 0 || im.column_stride == 0)
        return set_error(RG_EINVAL, "%s: zero stride", what);
    if (!(std::isfinite(im.tl_x) && std::isfinite(im.tl_y) && std::isfinite(im.br_x) &&
          std::isfinite(im.br_y)))
        return set_error(RG_EINVAL, "%s: non-finite corner", what);
    return RG_OK;
}

static SSGeom ss_geom(const rg_image &img, const rg_image &sino)
{
    SSGeom g;
    g.N = img.lines;
    g.itl_x = img.tl_x; g.itl_y = img.tl_y; g.ibr_x = img.br_x; g.ibr_y = img.br_y;
    g.R = sino.lines;
    g.A = sino.columns;
    g.stl_x = sino.tl_x; g.stl_y = sino.tl_y; g.sbr_x = sino.br_x; g.sbr_y = sino.br_y;
    return g;
}

static int check_ss(const rg_image &img, const rg_image &sino)
{
    int rc;
    if ((rc = check_image(img, "image")) != RG_OK) return rc;
    if ((rc = check_image(sino, "sinogram")) != RG_OK) return rc;
    if (img.lines != img.columns)
        return set_error(RG_EINVAL, "slant-stack images are square (got %d x %d)", img.lines,
                         img.columns);
    if (img.lines < 2 || sino.lines < 2)
        return set_error(RG_EINVAL, "slant-stack needs size >= 2 and nrays >= 2");
    return RG_OK;
}

int validate_ss(const rg_image &img, const rg_image &sino) { return check_ss(img, sino); }
SSGeom make_ss_geom(const rg_image &img, const rg_image &sino) { return ss_geom(img, sino); }

int check_ws(const void *ws)
{
    if (ws && ((uintptr_t)ws & 255) != 0)
        return set_error(RG_EINVAL, "workspace must be 256-byte aligned");
    return RG_OK;
}

static bool is_view_major(const rg_image &s)
{
    return s.column_stride == 1 && s.line_stride == s.lines;
}

// ----------------------------------------------------------------------------
// Autotuner for the gathers' launch shape: rows per thread (4 -> 32x32
// tiles, 8 -> 32x64, 16 -> 32x128) and the cluster view split (1, 2 or 4
// CTAs per tile).  The first out-of-place backprojection or adjoint of a
// geometry (and the first EM/OSEM run, for its gathers) times the variants
// on the caller's own buffers, CUDA events on the caller's stream, the
// median of three timed runs after one warm-up (this first call
// synchronises), and keeps the fastest for the process.  For each tile
// height the occupancy rule's split (gather_pick_split) is timed first and
// another split replaces it only when it is at least 2 % faster, so that
// timing noise does not move a launch away from the rule; the tile height
// with the fastest time wins.  One choice holds per geometry, whether the
// call is one slice or a stack (a stack call times the candidates on the
// whole stack, whose larger grid may favour another split), so that a
// stack's members equal separate calls bit for bit; the call that first
// meets a geometry sets it.
// Calls that never tune (inside a stream capture) use the cached choice, or
// a default by image size: 16 rows from N = 512 up (the measured best on
// GB300 at 512^2, 1024^2 and 2048^2), 8 from 128, else 4, with the rule's
// split.  RG_GATHER_ROWS=4|8|16 and RG_GATHER_SPLIT=1|2|4 force a choice.
//
// RG_TUNE_CACHE=<file> keeps the choices across processes: the file is a
// JSON object, read when a process first needs a choice and rewritten
// (through a temporary file and a rename) after each new tuning, with one
// entry per line,
//     "<GPU name>|sm<cc>|<bp|adj>|N<size>|R<rays>|V<views>|W<windows>":
//         {"rows": 8, "split": 1}
// (split 0 stands for the occupancy rule).  Summation order depends on the
// split, so runs that must agree bit for bit across processes (a resumed EM)
// pin it with the cache or the two variables.  Processes that tune the same
// file at the same time may drop each other's new entries.

static std::mutex g_tune_mu;
static std::map<std::string, TuneChoice> g_tune;
static bool g_tune_loaded = false;

static std::string device_tag()
{
    static std::mutex mu;
    static std::map<int, std::string> tags;
    const int d = current_device();
    std::lock_guard<std::mutex> lock(mu);
    auto it = tags.find(d);
    if (it != tags.end()) return it->second;
    cudaDeviceProp pr;
    std::string t = "gpu";
    if (cudaGetDeviceProperties(&pr, d) == cudaSuccess) {
        t = pr.name;
        for (char &c : t)
            if (c == '"' || c == '\\' || c == '|' || (unsigned char)c < 32) c = '_';
        t += "|sm" + std::to_string(pr.major * 10 + pr.minor);
    } else {
        cudaGetLastError();
    }
    tags[d] = t;
    return t;
}

static std::string tune_key(const SSPlan &p, int mode)
{
    char b[160];
    snprintf(b, sizeof b, "|%s|N%d|R%d|V%d|W%d,%d", mode == 0 ? "bp" : "adj", p.g.N, p.g.R, p.nv,
             p.wmax_bp[0], p.wmax_adj[0]);
    return device_tag() + b;
}

static const char *tune_cache_path()
{
    const char *e = getenv("RG_TUNE_CACHE");
    return (e && *e) ? e : nullptr;
}

// Integer value of "name" inside the JSON object text [b, e), or -1.
static int json_int_field(const std::string &t, size_t b, size_t e, const char *name)
{
    const std::string key = std::string("\"") + name + "\"";
    const size_t k = t.find(key, b);
    if (k == std::string::npos || k >= e) return -1;
    size_t i = k + key.size();
    while (i < e && (t[i] == ' ' || t[i] == '\t' || t[i] == '\n' || t[i] == '\r')) ++i;
    if (i >= e || t[i] != ':') return -1;
    ++i;
    while (i < e && (t[i] == ' ' || t[i] == '\t' || t[i] == '\n' || t[i] == '\r')) ++i;
    if (i >= e || t[i] < '0' || t[i] > '9') return -1;
    return atoi(t.c_str() + i);
}

// Caller holds g_tune_mu.  Reads every "key": {"rows": r, "split": s} pair
// of the file, whatever its layout; anything else (a truncated or foreign
// file) is skipped.
static void tune_cache_load()
{
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char *path = tune_cache_path();
    FILE *f = path ? fopen(path, "r") : nullptr;
    if (!f) return;
    std::string t;
    char buf[4096];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, f)) > 0 && t.size() < (1u << 24)) t.append(buf, n);
    fclose(f);
    size_t pos = 0;
    while (true) {
        const size_t q1 = t.find('"', pos);
        if (q1 == std::string::npos) break;
        const size_t q2 = t.find('"', q1 + 1);
        if (q2 == std::string::npos) break;
        pos = q2 + 1;
        size_t i = q2 + 1;
        while (i < t.size() && isspace((unsigned char)t[i])) ++i;
        if (i >= t.size() || t[i] != ':') continue;
        ++i;
        while (i < t.size() && isspace((unsigned char)t[i])) ++i;
        if (i >= t.size() || t[i] != '{') continue;
        const size_t e = t.find('}', i);
        if (e == std::string::npos) break;
        const int rows = json_int_field(t, i, e, "rows");
        const int split = json_int_field(t, i, e, "split");
        if ((rows == 4 || rows == 8 || rows == 16) &&
            (split == 0 || split == 1 || split == 2 || split == 4))
            g_tune.emplace(t.substr(q1 + 1, q2 - q1 - 1), TuneChoice{rows, split});
        pos = e + 1;
    }
}

// Caller holds g_tune_mu.  A file that cannot be written is left alone: the
// choices still hold for this process.
static void tune_cache_save()
{
    const char *path = tune_cache_path();
    if (!path) return;
    const std::string tmp = std::string(path) + ".tmp" + std::to_string((long long)getpid());
    FILE *f = fopen(tmp.c_str(), "w");
    if (!f) return;
    fprintf(f, "{\n");
    size_t i = 0;
    for (const auto &kv : g_tune)
        fprintf(f, "  \"%s\": {\"rows\": %d, \"split\": %d}%s\n", kv.first.c_str(),
                kv.second.rows, kv.second.split, ++i < g_tune.size() ? "," : "");
    fprintf(f, "}\n");
    if (fclose(f) != 0 || rename(tmp.c_str(), path) != 0) remove(tmp.c_str());
}

static int env_rows()
{
    const char *e = getenv("RG_GATHER_ROWS");
    if (!e) return 0;
    const int v = atoi(e);
    return (v == 4 || v == 8 || v == 16) ? v : 0;
}

TuneChoice tuned_choice(const SSPlan &p, int mode)
{
    if (int v = env_rows()) return {v, 0};
    const std::string key = tune_key(p, mode);
    std::lock_guard<std::mutex> lock(g_tune_mu);
    tune_cache_load();
    auto it = g_tune.find(key);
    if (it != g_tune.end()) return it->second;
    return {p.g.N >= 512 ? 16 : p.g.N >= 128 ? 8 : 4, 0};
}

int autotune_gather(const SSPlan &p, int mode, const float *s_am, int s_ld, float *out,
                    long long cs, long long ls, cudaStream_t st, void *quads, const Stack &z)
{
    if (env_rows()) return RG_OK;
    const std::string key = tune_key(p, mode);
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        tune_cache_load();
        if (g_tune.count(key)) return RG_OK;
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    RG_CK(cudaStreamIsCapturing(st, &cap));
    if (cap != cudaStreamCaptureStatusNone) return RG_OK;
    cudaEvent_t a, b;
    RG_CK(cudaEventCreate(&a));
    RG_CK(cudaEventCreate(&b));
    // median of three timed runs after a warm-up
    auto time_one = [&](int rows, int split, float &med) {
        SplitPref pref(split);
        float t[3];
        for (int rep = 0; rep < 4; ++rep) {
            cudaEventRecord(a, st);
            int rc = launch_gather(p, mode, s_am, s_ld, out, cs, ls, nullptr, nullptr, nullptr, st,
                                   rows, z, quads);
            cudaEventRecord(b, st);
            cudaError_t e = cudaEventSynchronize(b);
            if (!rc && e != cudaSuccess) rc = cuda_error(e, "autotune");
            if (rc) return rc;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, a, b);
            if (rep > 0) t[rep - 1] = ms;
        }
        std::sort(t, t + 3);
        med = t[1];
        return (int)RG_OK;
    };
    // A shape that the geometry does not support (a window too wide for the
    // tile height) is skipped; any other failure ends the call.
    float best = 1e30f;
    TuneChoice pick{4, 0};
    int rc = RG_OK, unsupported = RG_OK;
    for (int rows : {4, 8, 16}) {
        float t_rule = 0.f;
        if ((rc = time_one(rows, 0, t_rule)) == RG_EUNSUPPORTED) {
            unsupported = rc;
            rc = RG_OK;
            continue;
        }
        if (rc) break;
        TuneChoice c{rows, 0};
        float t_c = t_rule;
        for (int split : {1, 2, 4}) {
            float t = 0.f;
            if (rows % split) continue;
            if ((rc = time_one(rows, split, t)) == RG_EUNSUPPORTED) {
                rc = RG_OK;
                continue;
            }
            if (rc) break;
            if (t < 0.98f * t_rule && t < t_c) { t_c = t; c.split = split; }
        }
        if (rc) break;
        if (t_c < best) { best = t_c; pick = c; }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc) return rc;
    if (best == 1e30f) return unsupported;   // no tile height fits this geometry
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune[key] = pick;
    tune_cache_save();
    return RG_OK;
}

// Helpers for em.cu: hand out plans with an opaque owner handle
// (a heap-allocated std::shared_ptr<void>, released by release_holder).
int get_ss_plan(const SSGeom &g, int stride, int first, const SSPlan **out, void **holder)
{
    std::shared_ptr<PlanHolder> ph;
    int rc = get_plan(g, stride, first, ph);
    if (rc) return rc;
    *out = &ph->p;
    *holder = new std::shared_ptr<void>(ph);
    return RG_OK;
}

void release_holder(void *holder)
{
    delete static_cast<std::shared_ptr<void> *>(holder);
}

size_t ws_sum(std::initializer_list<size_t> pieces) { return ws_total(pieces); }

}  // namespace rg

using namespace rg;

// ============================================================================
// C ABI

extern "C" {

const char *rg_last_error(void) { return g_err.c_str(); }
int rg_version(void) { return 100; }

int rg_device_status(void)
{
    int *w = device_error_word();
    if (!w) return 0;
    int v = 0;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(&v, w, sizeof v, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemset(w, 0, sizeof(int));
    if (e != cudaSuccess) return cuda_error(e, "rg_device_status");
    return v;
}

// ---------------------------------------------------------------- Radon
size_t rg_radon_slantstack_workspace(rg_image phantom, rg_image radon)
{
    const int N = phantom.lines;
    return ws_total({radon_pairs_bytes(N), radon_pairs_bytes(N),
                     (size_t)radon.lines * radon.columns * sizeof(float)});
}

int rg_radon_slantstack(rg_image phantom, rg_image radon, void *ws, size_t wsb, void *stream)
{
    RG_TRACE();
    int rc = check_ss(phantom, radon);
    if (!rc) rc = check_ws(ws);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    std::shared_ptr<PlanHolder> ph;
    if ((rc = get_plan(ss_geom(phantom, radon), 1, 0, ph))) return rc;
    const int N = phantom.lines, R = radon.lines, A = radon.columns;
    Scratch s;
    if ((rc = scratch_begin(s, ws, wsb, rg_radon_slantstack_workspace(phantom, radon), st))) return rc;
    float2 *prow = (float2 *)s.take(radon_pairs_bytes(N));
    float2 *pcol = (float2 *)s.take(radon_pairs_bytes(N));
    float *out_am = (float *)s.take((size_t)R * A * sizeof(float));
    const bool direct = is_view_major(radon);
    if (!(rc = launch_line_pairs(phantom.data, phantom.column_stride, phantom.line_stride, N,
                                 prow, pcol, st)))
        rc = launch_radon(ph->p, prow, pcol, direct ? radon.data : out_am, R, nullptr, 0, st);
    if (!rc && !direct)
        rc = launch_from_am(out_am, R, A, radon.data, radon.column_stride, radon.line_stride, st);
    scratch_end(s);
    return rc;
}

// ---------------------------------------------------------------- stacks
size_t rg_radon_slantstack_stack_workspace(rg_image phantom, rg_image radon, int nstack)
{
    const int N = phantom.lines;
    const size_t am = is_view_major(radon) ? 0 : (size_t)radon.lines * radon.columns * sizeof(float);
    return ws_total({radon_pairs_bytes(N) * (size_t)nstack, radon_pairs_bytes(N) * (size_t)nstack,
                     am * (size_t)nstack});
}

int rg_radon_slantstack_stack(rg_image phantom, long long phantom_stride, rg_image radon,
                              long long radon_stride, int nstack, void *ws, size_t wsb,
                              void *stream)
{
    RG_TRACE();
    int rc = check_ss(phantom, radon);
    if (!rc) rc = check_ws(ws);
    if (rc) return rc;
    if (nstack < 1 || nstack > 65535) return set_error(RG_EINVAL, "stack size must be in [1, 65535]");
    cudaStream_t st = (cudaStream_t)stream;
    std::shared_ptr<PlanHolder> ph;
    if ((rc = get_plan(ss_geom(phantom, radon), 1, 0, ph))) return rc;
    const int N = phantom.lines, R = radon.lines, A = radon.columns;
    Scratch s;
    if ((rc = scratch_begin(s, ws, wsb, rg_radon_slantstack_stack_workspace(phantom, radon, nstack), st)))
        return rc;
    const long long zp = (long long)N * pairs_pitch(N);
    float2 *prow = (float2 *)s.take(radon_pairs_bytes(N) * (size_t)nstack);
    float2 *pcol = (float2 *)s.take(radon_pairs_bytes(N) * (size_t)nstack);
    const bool direct = is_view_major(radon);
    float *out_am = direct ? radon.data : (float *)s.take((size_t)R * A * sizeof(float) * nstack);
    const long long zo = direct ? radon_stride : (long long)R * A;
    if (!(rc = launch_line_pairs(phantom.data, phantom.column_stride, phantom.line_stride, N, prow,
                                 pcol, st, nstack, phantom_stride, zp)))
        rc = launch_radon(ph->p, prow, pcol, out_am, R, nullptr, 0, st, nstack, zp, zo);
    if (!rc && !direct)
        rc = launch_from_am(out_am, R, A, radon.data, radon.column_stride, radon.line_stride, st,
                            nstack, (long long)R * A, radon_stride);
    scratch_end(s);
    return rc;
}

size_t rg_radon_transpose_slantstack_stack_workspace(rg_image sino, rg_image image, int nstack)
{
    (void)image;
    return ws_total({is_view_major(sino) ? 0 : (size_t)sino.lines * sino.columns * sizeof(float) * nstack,
                     quads_ws(sino, nstack)});
}

int rg_radon_transpose_slantstack_stack(rg_image sino, long long sino_stride, rg_image image,
                                        long long image_stride, int nstack, void *ws, size_t wsb,
                                        void *stream)
{
    RG_TRACE();
    int rc = check_ss(image, sino);
    if (!rc) rc = check_ws(ws);
    if (rc) return rc;
    if (nstack < 1 || nstack > 65535) return set_error(RG_EINVAL, "stack size must be in [1, 65535]");
    cudaStream_t st = (cudaStream_t)stream;
    std::shared_ptr<PlanHolder> ph;
    if ((rc = get_plan(ss_geom(image, sino), 1, 0, ph))) return rc;
    const int R = sino.lines, A = sino.columns;
    Scratch s;
    if ((rc = scratch_begin(s, ws, wsb, rg_radon_transpose_slantstack_stack_workspace(sino, image, nstack), st)))
        return rc;
    const float *s_am = sino.data;
    long long zs = sino_stride;
    if (!is_view_major(sino)) {
        float *t = (float *)s.take((size_t)R * A * sizeof(float) * nstack);
        rc = launch_to_am(sino.data, sino.column_stride, sino.line_stride, R, A, t, st, nstack,
                          sino_stride, (long long)R * A);
        s_am = t;
        zs = (long long)R * A;
    }
    const size_t qb = quads_ws(sino, nstack);
    void *quads = qb ? s.take(qb) : nullptr;
    Stack zz;
    zz.n = nstack;
    zz.in = zs;
    zz.out = image_stride;
    // launch shape tuned on the whole stack (its output is rewritten below)
    if (!rc)
        rc = autotune_gather(ph->p, 1, s_am, R, image.data, image.column_stride, image.line_stride,
                             st, quads, zz);
    if (!rc)
        rc = launch_gather(ph->p, 1, s_am, R, image.data, image.column_stride, image.line_stride,
                           nullptr, nullptr, nullptr, st, 0, zz, quads);
    scratch_end(s);
    return rc;
}

// ---------------------------------------------------------------- FP64 pair
static rg_image as_f32_view(const rg_image_f64 &d)
{
    rg_image im;
    im.data = (float *)d.data;
    im.lines = d.lines; im.line_stride = d.line_stride;
    im.columns = d.columns; im.column_stride = d.column_stride;
    im.tl_x = d.tl_x; im.tl_y = d.tl_y; im.br_x = d.br_x; im.br_y = d.br_y;
    return im;
}

int rg_radon_slantstack_f64(rg_image_f64 phantom, rg_image_f64 radon, void *stream)
{
    RG_TRACE();
    const rg_image a = as_f32_view(phantom), b = as_f32_view(radon);
    int rc = check_ss(a, b);
    if (rc) return rc;
    std::shared_ptr<PlanHolder> ph;
    if ((rc = get_plan(ss_geom(a, b), 1, 0, ph))) return rc;
    return launch_radon_f64(ph->p, phantom.data, phantom.column_stride, phantom.line_stride,
                            radon.data, radon.column_stride, radon.line_stride,
                            (cudaStream_t)stream);
}

int rg_radon_transpose_slantstack_f64(rg_image_f64 sino, rg_image_f64 image, void *stream)
{
    RG_TRACE();
    const rg_image a = as_f32_view(image), b = as_f32_view(sino);
    int rc = check_ss(a, b);
    if (rc) return rc;
    if (image.column_stride != image.columns || image.line_stride != 1)
        return set_error(RG_EINVAL, "FP64 transpose writes a contiguous image");
    std::shared_ptr<PlanHolder> ph;
    if ((rc = get_plan(ss_geom(a, b), 1, 0, ph))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    RG_CK(cudaMemsetAsync(image.data, 0, sizeof(double) * image.lines * image.columns, st));
    return launch_radon_transpose_f64(ph->p, sino.data, sino.column_stride, sino.line_stride,
                                      image.data, st);
}

// ---------------------------------------------------------------- gathers
static size_t gather_ws(const rg_image &sino)
{
    return ws_total({is_view_major(sino) ? 0 : (size_t)sino.lines * sino.columns * sizeof(float),
                     quads_ws(sino)});
}

static int run_gather(int mode, rg_image sino, rg_image img, void *ws, size_t wsb, void *stream)
{
    int rc = check_ss(img, sino);
    if (!rc) rc = check_ws(ws);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    std::shared_ptr<PlanHolder> ph;
    if ((rc = get_plan(ss_geom(img, sino), 1, 0, ph))) return rc;
    const int R = sino.lines, A = sino.columns;
    Scratch s;
    if ((rc = scratch_begin(s, ws, wsb, gather_ws(sino), st))) return rc;
    const float *s_am = sino.data;
    if (!is_view_major(sino)) {
        float *t = (float *)s.take((size_t)R * A * sizeof(float));
        rc = launch_to_am(sino.data, sino.column_stride, sino.line_stride, R, A, t, st);
        s_am = t;
    }
    const size_t qb = quads_ws(sino);
    void *quads = qb ? s.take(qb) : nullptr;
    if (!rc)
        rc = autotune_gather(ph->p, mode, s_am, R, img.data, img.column_stride, img.line_stride, st,
                             quads);
    if (!rc)
        rc = launch_gather(ph->p, mode, s_am, R, img.data, img.column_stride, img.line_stride,
                           nullptr, nullptr, nullptr, st, 0, Stack(), quads);
    scratch_end(s);
    return rc;
}

size_t rg_backprojection_slantstack_workspace(rg_image sino, rg_image bp)
{
    (void)bp;
    return gather_ws(sino);
}

int rg_backprojection_slantstack(rg_image sino, rg_image bp, void *ws, size_t wsb, void *stream)
{
    RG_TRACE();
    return run_gather(0, sino, bp, ws, wsb, stream);
}

size_t rg_radon_transpose_slantstack_workspace(rg_image sino, rg_image img)
{
    (void)img;
    return gather_ws(sino);
}

int rg_radon_transpose_slantstack(rg_image sino, rg_image img, void *ws, size_t wsb, void *stream)
{
    RG_TRACE();
    return run_gather(1, sino, img, ws, wsb, stream);
}

// ---------------------------------------------------------------- filters
// Filters by FFT for transforms of up to 2^kFilterFftMaxLog points: Ram-Lak
// (zero-padded linear convolution) for any R, the lowpass filter (circular
// convolution of length R) when R is a power of two >= 4.
// RG_FILTER_KERNEL=direct selects the direct-sum kernels.
static bool filter_use_fft(int kind, int R)
{
    const char *e = getenv("RG_FILTER_KERNEL");
    if (e && !strcmp(e, "direct")) return false;
    if (kind == RG_FILTER_LOWPASS)
        return R >= 4 && (R & (R - 1)) == 0 && R <= (1 << kFilterFftMaxLog);
    return 2 * (long long)R - 1 <= (1LL << kFilterFftMaxLog);
}

// In-place radix-2 FFT (forward, e^{-2 pi i k n / M}) of length M = 2^p in
// FP64, for the filter tables.
static void host_fft(std::vector<std::complex<double>> &a, int p)
{
    const double pi = 3.14159265358979323846;
    const int M = 1 << p;
    for (int i = 0; i < M; ++i) {
        int r = 0;
        for (int b = 0; b < p; ++b) r |= ((i >> b) & 1) << (p - 1 - b);
        if (i < r) std::swap(a[i], a[r]);
    }
    std::vector<std::complex<double>> w(M / 2);
    for (int t = 0; t < M / 2; ++t) w[t] = std::complex<double>(cos(2.0 * pi * t / M), -sin(2.0 * pi * t / M));
    for (int len = 2; len <= M; len <<= 1) {
        const int half = len / 2, step = M / len;
        for (int i = 0; i < M; i += len)
            for (int j = 0; j < half; ++j) {
                const std::complex<double> u = a[i + j], v = a[i + j + half] * w[(size_t)j * step];
                a[i + j] = u + v;
                a[i + j + half] = u - v;
            }
    }
}

// Tables of launch_filter_fft for the 2R-1 taps t[m] (taps[m + R - 1], |m| <
// R): twiddles, then the difference-domain filter G'[k] = T[k] / (M (1 -
// e^{-2 pi i k / M})) in bit-reversed order (G'[0] = 0), T the DFT of the
// taps wrapped to length M = 2^p >= 2R - 1 (circ: of one period of
// R-periodic taps, M = R); g0 = T[0] / M.  All in FP64.
static void filter_fft_tables(const std::vector<double> &taps, int R, bool circ,
                              std::vector<unsigned char> &bytes, float &g0, int &p)
{
    const double pi = 3.14159265358979323846;
    p = 2;
    while ((1LL << p) < (circ ? (long long)R : 2 * (long long)R - 1)) ++p;
    const int M = 1 << p, H = M / 2;
    std::vector<std::complex<double>> T(M);
    if (circ)             // one period of the R-periodic taps
        for (int m = 0; m < R; ++m) T[m] = taps[(size_t)(m + R - 1)];
    else
        for (int m = -(R - 1); m <= R - 1; ++m) T[(m + M) & (M - 1)] = taps[(size_t)(m + R - 1)];
    host_fft(T, p);
    bytes.assign(sizeof(float2) * ((size_t)H + M), 0);
    float2 *tw = reinterpret_cast<float2 *>(bytes.data());
    float2 *gb = tw + H;
    for (int i = 0; i < H; ++i) tw[i] = make_float2((float)cos(2.0 * pi * i / M), (float)-sin(2.0 * pi * i / M));
    for (int k = 0; k < M; ++k) {
        int r = 0;
        for (int b = 0; b < p; ++b) r |= ((k >> b) & 1) << (p - 1 - b);
        if (r == 0) { gb[k] = make_float2(0.f, 0.f); continue; }
        // 1 / (1 - e^{-i th}) = (1 - i cot(th / 2)) / 2, th = 2 pi r / M
        const double a = pi * r / M;
        const std::complex<double> g = T[r] * std::complex<double>(1.0, -cos(a) / sin(a)) / (2.0 * M);
        gb[k] = make_float2((float)g.real(), (float)g.imag());
    }
    g0 = (float)(T[0].real() / M);
}

// The 2R-1 taps in FP64 (index m + R - 1, |m| < R): dt h[m] for the
// discrete Ram-Lak kernel h (linear convolution), or g[m mod R] for pyraft's
// lowpassino_fbp (circular convolution): g = Re(ifft(fftshift(|w| cos(pi w
// dt)))), w = linspace(-wc, wc, R), wc = 1/(2 dt), so that applying g equals
// the FFT filter of pyraft/filters/filters.py:13-68 (real part of the
// filtered data).
static std::vector<double> filter_taps64(int kind, int R, double dt)
{
    const double pi = 3.14159265358979323846;
    std::vector<double> taps(2 * (size_t)R - 1, 0.0);
    if (kind == RG_FILTER_RAMLAK) {
        taps[R - 1] = dt / (4.0 * dt * dt);
        for (int m = 1; m < R; m += 2) {
            const double v = -dt / (pi * pi * (double)m * (double)m * dt * dt);
            taps[(size_t)(R - 1 + m)] = v;
            taps[(size_t)(R - 1 - m)] = v;
        }
        return taps;
    }
    const double wc = 1.0 / (2.0 * dt);
    std::vector<double> h(R), G(R), g(R), ctab(R);
    const double step = (R > 1) ? (2.0 * wc) / (R - 1) : 0.0;
    for (int i = 0; i < R; ++i) {
        double w = (i == R - 1) ? wc : -wc + i * step;
        h[i] = fabs(w) * cos(pi * w * dt);
    }
    const int sh = R / 2;              // fftshift: G[k] = h[(k + R/2) mod R]... numpy
    for (int k = 0; k < R; ++k) G[k] = h[(k + (R - sh)) % R];
    for (int k = 0; k < R; ++k) ctab[k] = cos(2.0 * pi * (double)k / (double)R);
    for (int m = 0; m < R; ++m) {
        double acc = 0.0;
        for (int k = 0; k < R; ++k) acc += G[k] * ctab[(size_t)k * m % R];
        g[m] = acc / R;
    }
    for (int m = -(R - 1); m <= R - 1; ++m) taps[(size_t)(m + R - 1)] = g[((m % R) + R) % R];
    return taps;
}

static int filter_taps(const rg_image &sino, int kind, std::shared_ptr<DevTable> &out)
{
    const int R = sino.lines;
    const double tmin = sino.br_y, tmax = sino.tl_y;
    const double dt = (tmax - tmin) / (R - 1);
    if (!(std::isfinite(dt)) || dt == 0.0) return set_error(RG_EINVAL, "degenerate t extent");
    if (kind != RG_FILTER_RAMLAK && kind != RG_FILTER_LOWPASS)
        return set_error(RG_EINVAL, "unknown filter kind %d", kind);
    KeyBuilder kb;
    kb.add(kind).add(R).add(tmin).add(tmax);
    if (filter_use_fft(kind, R)) {
        return get_table_lazy("fft" + kb.s, [&](std::vector<unsigned char> &b, DevTable &t) {
            t.fft_circ = kind == RG_FILTER_LOWPASS;
            filter_fft_tables(filter_taps64(kind, R, dt), R, t.fft_circ, b, t.h0, t.fft_p);
        }, out);
    }
    return get_table_lazy("taps" + kb.s, [&](std::vector<unsigned char> &b, DevTable &tab) {
        const std::vector<double> t = filter_taps64(kind, R, dt);
        if (kind == RG_FILTER_RAMLAK) {
            // odd taps godd[q] = dt h[2q - 2R + 1], q in [0, 2R), then dt h[0]
            // (the layout k_ramlak_rows reads)
            b.assign(sizeof(float) * (2 * (size_t)R + 1), 0);
            float *g = reinterpret_cast<float *>(b.data());
            for (int q = 0; q < 2 * R; ++q) {
                const int m = 2 * q - 2 * R + 1;
                if (m >= -(R - 1) && m <= R - 1) g[q] = (float)t[(size_t)(m + R - 1)];
            }
            g[2 * (size_t)R] = (float)t[R - 1];
            tab.h0 = g[2 * (size_t)R];
        } else {
            b.assign(sizeof(float) * t.size(), 0);
            float *g = reinterpret_cast<float *>(b.data());
            for (size_t i = 0; i < t.size(); ++i) g[i] = (float)t[i];
        }
    }, out);
}

static int filter_rows(int kind, const float *in_am, float *out_am, int R, int A,
                       const std::shared_ptr<DevTable> &taps, cudaStream_t st)
{
    if (taps->fft_p)
        return launch_filter_fft(in_am, out_am, R, A, taps->fft_p, (const float2 *)taps->p,
                                 taps->h0, taps->fft_circ, st);
    if (kind == RG_FILTER_RAMLAK)     // odd taps + centre tap (parity-split kernel)
        return launch_ramlak_rows(in_am, out_am, R, A, (const float *)taps->p, taps->h0, st);
    return launch_conv_rows(in_am, out_am, R, A, (const float *)taps->p, st);
}

size_t rg_filter_workspace(rg_image sino, int kind)
{
    (void)kind;
    const size_t b = (size_t)sino.lines * sino.columns * sizeof(float);
    return ws_total({b, b});
}

int rg_filter(rg_image in, rg_image out, int kind, void *ws, size_t wsb, void *stream)
{
    RG_TRACE();
    int rc;
    if ((rc = check_image(in, "input sinogram")) || (rc = check_image(out, "output sinogram")))
        return rc;
    if (in.lines != out.lines || in.columns != out.columns)
        return set_error(RG_EINVAL, "filter input and output shapes differ");
    if (in.lines < 2) return set_error(RG_EINVAL, "filter needs nrays >= 2");
    if ((rc = check_ws(ws))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    std::shared_ptr<DevTable> taps;
    if ((rc = filter_taps(in, kind, taps))) return rc;
    const int R = in.lines, A = in.columns;
    Scratch s;
    if ((rc = scratch_begin(s, ws, wsb, rg_filter_workspace(in, kind), st))) return rc;
    float *a = (float *)s.take((size_t)R * A * sizeof(float));
    float *b = (float *)s.take((size_t)R * A * sizeof(float));
    if (!(rc = launch_to_am(in.data, in.column_stride, in.line_stride, R, A, a, st)) &&
        !(rc = filter_rows(kind, a, b, R, A, taps, st)))
        rc = launch_from_am(b, R, A, out.data, out.column_stride, out.line_stride, st);
    scratch_end(s);
    return rc;
}

size_t rg_fbp_workspace(rg_image sino, rg_image image, int kind)
{
    (void)image;
    (void)kind;
    const size_t b = (size_t)sino.lines * sino.columns * sizeof(float);
    return ws_total({b, b, quads_ws(sino)});
}

}  // extern "C"
namespace rg {
// RG_FBP_QUADS=0 (read per call) keeps the FBP's filter and the gather's quad
// prepass as separate launches: the reference arrangement for tests, which
// must give the same bits.
static bool fbp_quads_enabled()
{
    const char *e = getenv("RG_FBP_QUADS");
    return !(e && e[0] == '0' && e[1] == 0);
}
}  // namespace rg
extern "C" {

int rg_fbp(rg_image sino, rg_image image, int kind, void *ws, size_t wsb, void *stream)
{
    RG_TRACE();
    int rc = check_ss(image, sino);
    if (!rc) rc = check_ws(ws);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    std::shared_ptr<DevTable> taps;
    if ((rc = filter_taps(sino, kind, taps))) return rc;
    std::shared_ptr<PlanHolder> ph;
    if ((rc = get_plan(ss_geom(image, sino), 1, 0, ph))) return rc;
    const int R = sino.lines, A = sino.columns;
    Scratch s;
    if ((rc = scratch_begin(s, ws, wsb, rg_fbp_workspace(sino, image, kind), st))) return rc;
    float *a = (float *)s.take((size_t)R * A * sizeof(float));
    float *b = (float *)s.take((size_t)R * A * sizeof(float));
    const size_t qb = quads_ws(sino);
    void *quads = qb ? s.take(qb) : nullptr;
    const float *src = sino.data;
    if (!is_view_major(sino)) {
        rc = launch_to_am(sino.data, sino.column_stride, sino.line_stride, R, A, a, st);
        src = a;
    }
    // The gather's launch shape is tuned (the first call for a geometry)
    // before the filter runs, on the unfiltered rows: its timings do not
    // depend on the data.
    if (!rc)
        rc = autotune_gather(ph->p, 0, src, R, image.data, image.column_stride,
                             image.line_stride, st, quads);
    if (!rc) {
        if (taps->fft_p && !taps->fft_circ && fbp_quads_enabled() &&
            gather_quads_form(ph->p, quads)) {
            // the FFT filter writes the paired gather's quads and zeroes the
            // image itself: the filtered rows are never stored, and the
            // gather's prepass launch is not needed
            rc = launch_filter_fft_quads(src, R, A, taps->fft_p, (const float2 *)taps->p,
                                         taps->h0, (const View *)ph->p.d_views, ph->p.nv / 2,
                                         ph->p.g.A / 2, (float4 *)quads, image.data, ph->p.g.N,
                                         image.column_stride, image.line_stride, st);
            if (!rc) {
                QuadsPrefilled given;
                rc = launch_gather(ph->p, 0, b, R, image.data, image.column_stride,
                                   image.line_stride, nullptr, nullptr, nullptr, st, 0, Stack(),
                                   quads);
            }
        } else if (!(rc = filter_rows(kind, src, b, R, A, taps, st))) {
            rc = launch_gather(ph->p, 0, b, R, image.data, image.column_stride,
                               image.line_stride, nullptr, nullptr, nullptr, st, 0, Stack(),
                               quads);
        }
    }
    scratch_end(s);
    return rc;
}

// ---------------------------------------------------------------- DDA
}  // extern "C"
namespace rg {
static int check_dda(const rg_image &img, const rg_image &sino)
{
    int rc;
    if ((rc = check_image(img, "image")) || (rc = check_image(sino, "sinogram"))) return rc;
    if (img.lines < 2 || img.columns < 2 || sino.lines < 2 || sino.columns < 2)
        return set_error(RG_EINVAL, "DDA projector needs >= 2 lines and columns in image and "
                                    "sinogram (the sampling distances divide by n - 1)");
    if (sino.columns > 65535) return set_error(RG_EINVAL, "DDA projector: at most 65535 views");
    return RG_OK;
}

static DDAGeom dda_geom(const rg_image &img, const rg_image &sino)
{
    DDAGeom g;
    g.lines = img.lines; g.columns = img.columns;
    g.itl_x = img.tl_x; g.itl_y = img.tl_y; g.ibr_x = img.br_x; g.ibr_y = img.br_y;
    g.R = sino.lines; g.A = sino.columns;
    g.stl_x = sino.tl_x; g.stl_y = sino.tl_y; g.sbr_x = sino.br_x; g.sbr_y = sino.br_y;
    return g;
}

// cos/sin of the views tl_x + j*(br_x - tl_x)/(columns - 1) (host libm).
static int dda_views(const DDAGeom &g, std::shared_ptr<DevTable> &out)
{
    KeyBuilder kb;
    kb.add(g.A).add(g.stl_x).add(g.sbr_x);
    std::vector<double> cs(2 * (size_t)g.A);
    const double dth = (g.sbr_x - g.stl_x) / (g.A - 1);
    for (int j = 0; j < g.A; ++j) {
        const double th = g.stl_x + (j * dth);
        cs[2 * j] = cos(th);
        cs[2 * j + 1] = sin(th);
    }
    return get_table(std::string("ddaviews") + kb.s, cs.data(), cs.size() * sizeof(double), out);
}

int get_dda_views(const DDAGeom &g, const double **d_cs, void **holder)
{
    std::shared_ptr<DevTable> t;
    int rc = dda_views(g, t);
    if (rc) return rc;
    *d_cs = (const double *)t->p;
    *holder = new std::shared_ptr<void>(t);
    return RG_OK;
}
}  // namespace rg
extern "C" {

size_t rg_radon_bresenham_workspace(rg_image image, rg_image sino)
{
    (void)image;
    return is_view_major(sino) ? 0 : ws_total({(size_t)sino.lines * sino.columns * sizeof(float)});
}

int rg_radon_bresenham(rg_image image, rg_image sino, void *ws, size_t wsb, void *stream)
{
    RG_TRACE();
    int rc = check_dda(image, sino);
    if (!rc) rc = check_ws(ws);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const DDAGeom g = dda_geom(image, sino);
    std::shared_ptr<DevTable> cs;
    if ((rc = dda_views(g, cs))) return rc;
    Scratch s;
    if ((rc = scratch_begin(s, ws, wsb, rg_radon_bresenham_workspace(image, sino), st))) return rc;
    if (is_view_major(sino)) {
        rc = launch_bres_radon(g, (const double *)cs->p, image.data, image.column_stride,
                               image.line_stride, sino.data, 1, g.R, nullptr, 0, 1, st);
    } else {
        float *am = (float *)s.take((size_t)g.R * g.A * sizeof(float));
        if (!(rc = launch_bres_radon(g, (const double *)cs->p, image.data, image.column_stride,
                                     image.line_stride, am, 1, g.R, nullptr, 0, 1, st)))
            rc = launch_from_am(am, g.R, g.A, sino.data, sino.column_stride, sino.line_stride, st);
    }
    scratch_end(s);
    return rc;
}

size_t rg_radon_transpose_bresenham_workspace(rg_image sino, rg_image image)
{
    return ws_total({(size_t)sino.lines * sino.columns * sizeof(float),
                     (size_t)image.lines * image.columns * sizeof(float)});
}

int rg_radon_transpose_bresenham(rg_image sino, rg_image image, void *ws, size_t wsb, void *stream)
{
    RG_TRACE();
    int rc = check_dda(image, sino);
    if (!rc) rc = check_ws(ws);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const DDAGeom g = dda_geom(image, sino);
    std::shared_ptr<DevTable> cs;
    if ((rc = dda_views(g, cs))) return rc;
    Scratch s;
    if ((rc = scratch_begin(s, ws, wsb, rg_radon_transpose_bresenham_workspace(sino, image), st)))
        return rc;
    float *am = (float *)s.take((size_t)g.R * g.A * sizeof(float));
    float *img = (float *)s.take((size_t)g.lines * g.columns * sizeof(float));
    if (!(rc = launch_to_am(sino.data, sino.column_stride, sino.line_stride, g.R, g.A, am, st)) &&
        !(rc = launch_fill(img, (size_t)g.lines * g.columns, 0.f, st)) &&
        !(rc = launch_bres_transpose(g, (const double *)cs->p, am, img, 0, 1, st)))
        rc = launch_copy2d(img, g.columns, 1, image.data, image.column_stride, image.line_stride,
                           g.lines, g.columns, st);
    scratch_end(s);
    return rc;
}

size_t rg_backprojection_bresenham_workspace(rg_image sino, rg_image image)
{
    return ws_total({(size_t)sino.lines * sino.columns * sizeof(float),
                     (size_t)image.lines * image.columns * sizeof(double),
                     (size_t)image.lines * image.columns * sizeof(double)});
}

int rg_backprojection_bresenham(rg_image sino, rg_image image, void *ws, size_t wsb, void *stream)
{
    RG_TRACE();
    int rc = check_dda(image, sino);
    if (!rc) rc = check_ws(ws);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const DDAGeom g = dda_geom(image, sino);
    std::shared_ptr<DevTable> cs;
    if ((rc = dda_views(g, cs))) return rc;
    Scratch s;
    if ((rc = scratch_begin(s, ws, wsb, rg_backprojection_bresenham_workspace(sino, image), st)))
        return rc;
    const size_t npix = (size_t)g.lines * g.columns;
    float *am = (float *)s.take((size_t)g.R * g.A * sizeof(float));
    double *num = (double *)s.take(npix * sizeof(double));
    double *den = (double *)s.take(npix * sizeof(double));
    if (!(rc = launch_to_am(sino.data, sino.column_stride, sino.line_stride, g.R, g.A, am, st))) {
        cudaError_t e = cudaMemsetAsync(num, 0, npix * sizeof(double), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(den, 0, npix * sizeof(double), st);
        if (e != cudaSuccess) rc = cuda_error(e, "normalised backprojection zeroing");
    }
    if (!rc)
        rc = launch_bres_normalised(g, (const double *)cs->p, am, num, den, image.data,
                                    image.column_stride, image.line_stride, st);
    scratch_end(s);
    return rc;
}

int rg_dda_trace(int lines, int columns, const double img_corners[4], const double *thetas,
                 const double *ts, int n, int cap, int *oi, int *oj, double *os, int *ocount,
                 void *stream)
{
    RG_TRACE();
    if (lines < 2 || columns < 2 || n < 0 || cap < 0 || !img_corners || (n > 0 && (!thetas || !ts)))
        return set_error(RG_EINVAL, "rg_dda_trace: bad arguments");
    if (n == 0) return RG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<double> cst(3 * (size_t)n);
    for (int r = 0; r < n; ++r) {
        cst[3 * r] = cos(thetas[r]);
        cst[3 * r + 1] = sin(thetas[r]);
        cst[3 * r + 2] = ts[r];
    }
    double *d = nullptr;
    RG_CK(cudaMalloc(&d, cst.size() * sizeof(double)));
    int rc = RG_OK;
    cudaError_t e = cudaMemcpyAsync(d, cst.data(), cst.size() * sizeof(double),
                                    cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) rc = cuda_error(e, "rg_dda_trace upload");
    if (!rc) rc = launch_dda_trace(lines, columns, img_corners, d, n, cap, oi, oj, os, ocount, st);
    e = cudaStreamSynchronize(st);
    if (!rc && e != cudaSuccess) rc = cuda_error(e, "rg_dda_trace");
    cudaFree(d);
    return rc;
}

// ---------------------------------------------------------------- TV
int rg_tv(const float *x, int nslices, int size, float eps, double *value, float *grad,
          void *stream)
{
    RG_TRACE();
    if (!x || !value) return set_error(RG_EINVAL, "rg_tv: null pointer");
    if (nslices < 1 || nslices > 65535 || size < 1)
        return set_error(RG_EINVAL, "rg_tv: need 1 <= nslices <= 65535 and size >= 1");
    if (!(eps >= 0.f)) return set_error(RG_EINVAL, "rg_tv: eps must be >= 0");
    return launch_tv(x, nslices, size, eps, value, grad, (cudaStream_t)stream);
}

// ---------------------------------------------------------------- phantoms
int rg_phantom_fromdesc(rg_image image, const double *desc, int n, void *stream)
{
    RG_TRACE();
    int rc = check_image(image, "image");
    if (rc) return rc;
    if (n < 0 || (n > 0 && !desc)) return set_error(RG_EINVAL, "bad ellipse table");
    if (image.lines < 2 || image.columns < 2)
        return set_error(RG_EINVAL, "phantom needs >= 2 lines and columns");
    if (n == 0) return RG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<double> h(7 * (size_t)n);
    for (int e = 0; e < n; ++e) {
        const double *q = desc + 6 * e;
        double *o = h.data() + 7 * e;
        o[0] = q[0]; o[1] = q[1]; o[2] = q[2]; o[3] = q[3]; o[4] = q[4];
        o[5] = cos(q[5]);
        o[6] = sin(q[5]);
    }
    Scratch s;
    if ((rc = scratch_begin(s, nullptr, 0, h.size() * sizeof(double), st))) return rc;
    double *d = (double *)s.take(h.size() * sizeof(double));
    cudaError_t e = cudaMemcpyAsync(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) rc = cuda_error(e, "phantom upload");
    if (!rc)
        rc = launch_phantom(image.data, image.column_stride, image.line_stride, image.lines,
                            image.columns, image.tl_x, image.tl_y, image.br_x, image.br_y, d, n, st);
    scratch_end(s);
    return rc;
}

int rg_radon_fromdesc(rg_image sino, const double *desc, int n, void *stream)
{
    RG_TRACE();
    int rc = check_image(sino, "sinogram");
    if (rc) return rc;
    if (n < 0 || (n > 0 && !desc)) return set_error(RG_EINVAL, "bad ellipse table");
    if (sino.lines < 2 || sino.columns < 2)
        return set_error(RG_EINVAL, "analytic sinogram needs >= 2 rays and views");
    if (n == 0) return RG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int V = sino.columns;
    const double ths = (sino.br_x - sino.tl_x) / (V - 1);
    std::vector<double> h(6 * (size_t)n + 2 * (size_t)V + 2 * (size_t)n * V);
    memcpy(h.data(), desc, 6 * (size_t)n * sizeof(double));
    double *cv = h.data() + 6 * n, *cp = cv + 2 * V;
    for (int j = 0; j < V; ++j) {
        const double th = sino.tl_x + j * ths;
        cv[2 * j] = cos(th);
        cv[2 * j + 1] = sin(th);
        for (int e = 0; e < n; ++e) {
            const double d = th - desc[6 * e + 5];
            cp[((size_t)e * V + j) * 2] = cos(d);
            cp[((size_t)e * V + j) * 2 + 1] = sin(d);
        }
    }
    Scratch s;
    if ((rc = scratch_begin(s, nullptr, 0, h.size() * sizeof(double), st))) return rc;
    double *d = (double *)s.take(h.size() * sizeof(double));
    cudaError_t e = cudaMemcpyAsync(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) rc = cuda_error(e, "fromdesc upload");
    if (!rc)
        rc = launch_radon_fromdesc(sino.data, sino.column_stride, sino.line_stride, sino.lines,
                                   V, sino.tl_x, sino.tl_y, sino.br_x, sino.br_y, d, n, st);
    scratch_end(s);
    return rc;
}

// ---------------------------------------------------------------- host wrappers
static rg_image host_img(float *d, int lines, int cols, double tlx, double tly, double brx,
                         double bry)
{
    rg_image im;
    im.data = d; im.lines = lines; im.line_stride = 1; im.columns = cols; im.column_stride = cols;
    im.tl_x = tlx; im.tl_y = tly; im.br_x = brx; im.br_y = bry;
    return im;
}

static int host_call(int op, float *h_out, const float *h_in, int size, int nrays, int nangles,
                     int niter)
{
    if (!h_out || !h_in || size < 2 || nrays < 2 || nangles < 1)
        return set_error(RG_EINVAL, "bad host-wrapper arguments");
    const size_t ni = (size_t)size * size * sizeof(float), ns = (size_t)nrays * nangles * sizeof(float);
    float *di = nullptr, *ds = nullptr;
    RG_CK(cudaMalloc(&di, ni));
    cudaError_t e = cudaMalloc(&ds, ns);
    if (e != cudaSuccess) { cudaFree(di); return cuda_error(e, "cudaMalloc"); }
    const double pi = 3.14159265358979323846;
    rg_image img = host_img(di, size, size, -1.0, 1.0, 1.0, -1.0);
    rg_image sino = host_img(ds, nrays, nangles, 0.0, 1.0, pi, -1.0);
    int rc = RG_OK;
    if (op == 0) {
        e = cudaMemcpy(di, h_in, ni, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) rc = cuda_error(e, "upload");
        if (!rc) rc = rg_radon_slantstack(img, sino, nullptr, 0, nullptr);
        if (!rc && (e = cudaMemcpy(h_out, ds, ns, cudaMemcpyDeviceToHost)) != cudaSuccess)
            rc = cuda_error(e, "download");
    } else {
        e = cudaMemcpy(ds, h_in, ns, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) rc = cuda_error(e, "upload");
        if (!rc && op == 1) rc = rg_backprojection_slantstack(sino, img, nullptr, 0, nullptr);
        if (!rc && op == 2) {
            rc = launch_fill(di, (size_t)size * size, 1.f, nullptr);
            if (!rc) rc = rg_em(sino, img, RG_SLANTSTACK_BP, niter, 1, nullptr, 0, nullptr);
        }
        if (!rc && (e = cudaMemcpy(h_out, di, ni, cudaMemcpyDeviceToHost)) != cudaSuccess)
            rc = cuda_error(e, "download");
    }
    cudaFree(di);
    cudaFree(ds);
    return rc;
}

int rg_radon_slantstack_host(float *h_output, const float *h_input, int size, int nrays, int nangles)
{
    RG_TRACE();
    return host_call(0, h_output, h_input, size, nrays, nangles, 0);
}

int rg_backprojection_slantstack_host(float *h_image, const float *h_sino, int size, int nrays,
                                      int nangles)
{
    RG_TRACE();
    return host_call(1, h_image, h_sino, size, nrays, nangles, 0);
}

int rg_em_host(float *h_output, const float *h_sino, int size, int nrays, int nangles, int niter)
{
    RG_TRACE();
    return host_call(2, h_output, h_sino, size, nrays, nangles, niter);
}

}  // extern "C"
