// em.cu -- emission EM / OSEM drivers.
//
// MLEM, x <- x * A^T(y / A x) / A^T 1 (pyraft/iterative/em.py:109-144,
// raft/raft_em_gpu.cu:20-87), and OSEM over interleaved view subsets
// (subset s = views s, s+S, ...; the reference's osem, pyraft/iterative/
// em.py:265-320, uses contiguous blocks of Fourier-slice operators, which
// are not available here; interleaved subsets are the standard choice).
//
// Slant-stack path, per sub-iteration (3 launches, no host round trip):
//   1. pack the iterate into line pairs (k_line_pairs);
//   2. Radon over the subset's views with the EM ratio fused into the
//      epilogue: r = y / (A x), 0 where A x == 0;
//   3. matched-adjoint gather of r over the subset's views with the update
//      fused into the epilogue: x <- x * (A^T r) * (1 / A^T 1).  Where the
//      subset's views pair up a quarter turn apart (gather_rot.cu), each
//      pixel gets two partial sums from two CTAs: they are added into a
//      zeroed scratch image, and the last CTA to add to a 32 x 32 block
//      applies the update to it (EmFuse; the edge pixels first, by their own
//      kernel).  For N not a multiple of 32 the update is its own pass.
// The sensitivities A_s^T 1 of each subset are accumulated in FP64 once per
// call and stored as reciprocals (0 where the sensitivity is 0, which also
// zeroes pixels that no ray of the subset reaches).
//
// DDA path (pyraft's em() default): the same loop over the DDA Radon with
// the fused ratio, the DDA transpose, and an elementwise update.  The walks
// are FP64-bound, so with two or more iterations each subset's walks are
// recorded once (DDAPlan, bresenham.cu) and replayed as streamed reads.
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "rg_internal.cuh"

namespace rg {

namespace {

struct Holders {
    std::vector<void *> h;
    ~Holders()
    {
        for (void *p : h) release_holder(p);
    }
};

// Quad scratch of the paired gathers for the largest of S subsets of A views.
static size_t em_quads_bytes(int R, int A, int S)
{
    return gather_quads_bytes((A + S - 1) / S, R, 1);
}

// Block counters of the EM update fused into the paired gathers (EmFuse).
static size_t em_cnt_bytes(int N)
{
    return em_fusable(N) ? (size_t)(N / 32) * (N / 32) * sizeof(int) : 0;
}

size_t em_ss_ws(int N, int R, int A, int S)
{
    const size_t sino = (size_t)R * A * sizeof(float), img = (size_t)N * N * sizeof(float);
    return ws_sum({sino, sino, radon_pairs_bytes(N), radon_pairs_bytes(N), img, img * S, img,
                   em_quads_bytes(R, A, S), em_cnt_bytes(N)});
}

// The DDA EM's recorded walks (freed with the call).  RG_DDA_PLAN=0 walks
// every time; RG_DDA_PLAN_MAX_GB caps a plan's step array (default 48).
struct DDAPlans {
    std::vector<DDAPlan> p;
    explicit DDAPlans(int n) : p(n) {}
    ~DDAPlans()
    {
        for (auto &q : p) dda_plan_free(q);
    }
};

// RG_EM_UNFUSED=1: the paired gathers write their sums to scratch and the EM
// update runs as its own pass even where it could be fused (A/B timing).
bool em_unfused()
{
    const char *e = getenv("RG_EM_UNFUSED");
    return e && !strcmp(e, "1");
}

bool dda_plans_enabled()
{
    const char *e = getenv("RG_DDA_PLAN");
    return !(e && !strcmp(e, "0"));
}

size_t dda_plan_max_bytes()
{
    const char *e = getenv("RG_DDA_PLAN_MAX_GB");
    const double gb = e ? atof(e) : 48.0;
    return (size_t)(std::max(gb, 0.0) * (double)(1ull << 30));
}

size_t em_dda_ws(int L, int C, int R, int A, int S)
{
    const size_t sino = (size_t)R * A * sizeof(float), img = (size_t)L * C * sizeof(float);
    // y, ratio, x, bp, sensitivities, and the column-major copies of x and
    // bp that the replayed walks use
    return ws_sum({sino, sino, img, img, img * S, img, img});
}

}  // namespace

// Runs EM on one slice whose buffers are already laid out internally:
// y_am (A x R view-major), x (N x N contiguous).  Scratch `s` must have room
// for ratio, pairs and sensitivities (em_ss_ws minus y and x).
// bp: the slant-stack backprojection is the backprojector (RG_SLANTSTACK_BP,
// raft_em_gpu's pairing) instead of the matched adjoint; its sensitivity
// B 1 is the FP32-compensated backprojection of ones (the dth scale of B
// cancels between B r and B 1).
// Runs sub-iterations first .. first + count - 1; sub-iteration j uses
// subset j mod S (rg_em: first 0, count niter * S).
static int em_ss_core(const SSGeom &g, long long first, long long count, int S,
                      const float *y_am, float *x, Scratch &s, cudaStream_t st, bool bp = false)
{
    const int N = g.N, R = g.R, A = g.A;
    Holders hold;
    std::vector<const SSPlan *> plans(S);
    for (int k = 0; k < S; ++k) {
        void *h = nullptr;
        int rc = get_ss_plan(g, S, k, &plans[k], &h);
        if (rc) return rc;
        hold.h.push_back(h);
        if (!bp && !plans[k]->adj_ok)
            return set_error(RG_EUNSUPPORTED, "EM needs ray spacing >= pixel spacing (nrays <= size)");
    }
    float *ratio = (float *)s.take((size_t)R * A * sizeof(float));
    float2 *prow = (float2 *)s.take(radon_pairs_bytes(N));
    float2 *pcol = (float2 *)s.take(radon_pairs_bytes(N));
    float *inv = (float *)s.take((size_t)N * N * sizeof(float) * S);
    // Partial sums of the paired gathers (two per pixel).  For N a multiple
    // of 32 the gathers apply the update themselves (EmFuse: zeroed here
    // once, left zero by every gather); otherwise x <- x * g * inv follows
    // as its own pass.
    float *gsum = (float *)s.take((size_t)N * N * sizeof(float));
    const size_t qb = em_quads_bytes(R, A, S);
    void *quads = qb ? s.take(qb) : nullptr;
    const size_t cb = em_cnt_bytes(N);
    EmFuse fuse;
    fuse.gsum = gsum;
    fuse.cnt = cb ? (int *)s.take(cb) : nullptr;
    bool any_rot = false;
    for (int k = 0; k < S; ++k) any_rot = any_rot || plans[k]->rot_ok;
    const bool fused = any_rot && gather_rot_enabled() && em_fusable(N) && !em_unfused();
    // launch shape of each plan's gathers: timed on the first run of a
    // geometry outside a stream capture, on gsum (zeroed below)
    int rc = RG_OK;
    for (int k = 0; k < S && !rc; ++k)
        rc = autotune_gather(*plans[k], bp ? 0 : 1, y_am, R, gsum, N, 1, st, quads);
    if (!rc) rc = launch_fill(ratio, (size_t)R * A, 1.f, st);
    if (!rc && fused) rc = launch_fill(gsum, (size_t)N * N, 0.f, st);
    if (!rc && fused) RG_CK(cudaMemsetAsync(fuse.cnt, 0, cb, st));
    for (int k = 0; k < S && !rc; ++k) {
        float *ik = inv + (size_t)k * N * N;
        if (bp) {
            rc = launch_gather(*plans[k], 0, ratio, R, ik, N, 1, nullptr, nullptr, nullptr, st);
            if (!rc) rc = launch_invert(ik, ik, (size_t)N * N, st);
        } else {
            rc = launch_gather(*plans[k], 2, ratio, R, ik, N, 1, nullptr, nullptr, nullptr, st);
        }
    }
    for (long long j = first; j < first + count && !rc; ++j) {
            const int k = (int)(j % S);
            if ((rc = launch_line_pairs(x, N, 1, N, prow, pcol, st))) break;
            if ((rc = launch_radon(*plans[k], prow, pcol, ratio, R, y_am, R, st))) break;
            if (plans[k]->rot_ok && fused) {
                rc = launch_gather(*plans[k], bp ? 0 : 1, ratio, R, nullptr, 0, 0, x,
                                   inv + (size_t)k * N * N, nullptr, st, 0, Stack(), quads,
                                   &fuse);
            } else if (plans[k]->rot_ok && gather_rot_enabled()) {
                rc = launch_gather(*plans[k], bp ? 0 : 1, ratio, R, gsum, N, 1, nullptr, nullptr,
                                   nullptr, st, 0, Stack(), quads);
                if (!rc) rc = launch_em_update(x, gsum, inv + (size_t)k * N * N, (size_t)N * N, st);
            } else {
                rc = launch_gather(*plans[k], bp ? 0 : 1, ratio, R, nullptr, 0, 0, x,
                                   inv + (size_t)k * N * N, nullptr, st);
            }
        }
    return rc;
}

static int em_dda(const rg_image &sino, const rg_image &image, long long first, long long count,
                  int S, void *ws, size_t wsb, cudaStream_t st)
{
    DDAGeom g;
    g.lines = image.lines; g.columns = image.columns;
    g.itl_x = image.tl_x; g.itl_y = image.tl_y; g.ibr_x = image.br_x; g.ibr_y = image.br_y;
    g.R = sino.lines; g.A = sino.columns;
    g.stl_x = sino.tl_x; g.stl_y = sino.tl_y; g.sbr_x = sino.br_x; g.sbr_y = sino.br_y;
    if (g.lines < 2 || g.columns < 2 || g.R < 2 || g.A < 2)
        return set_error(RG_EINVAL, "DDA EM needs >= 2 lines and columns in image and sinogram");
    const double *cs = nullptr;
    void *holder = nullptr;
    int rc = get_dda_views(g, &cs, &holder);
    if (rc) return rc;
    Holders hold;
    hold.h.push_back(holder);
    const int L = g.lines, C = g.columns, R = g.R, A = g.A;
    const size_t npix = (size_t)L * C;
    Scratch s;
    if ((rc = scratch_begin(s, ws, wsb, em_dda_ws(L, C, R, A, S), st))) return rc;
    float *y = (float *)s.take((size_t)R * A * sizeof(float));
    float *ratio = (float *)s.take((size_t)R * A * sizeof(float));
    float *x = (float *)s.take(npix * sizeof(float));
    float *bp = (float *)s.take(npix * sizeof(float));
    float *inv = (float *)s.take(npix * sizeof(float) * S);
    float *xT = (float *)s.take(npix * sizeof(float));
    float *bpT = (float *)s.take(npix * sizeof(float));
    rc = launch_to_am(sino.data, sino.column_stride, sino.line_stride, R, A, y, st);
    if (!rc) rc = launch_copy2d(image.data, image.column_stride, image.line_stride, x, C, 1, L, C, st);
    if (!rc) rc = launch_fill(ratio, (size_t)R * A, 1.f, st);
    // Record each subset's walks once when they will be replayed (two walks
    // per sub-iteration), memory permitting (dda_plan_build).
    // (not while the stream is captured into a graph: building a plan
    // allocates and synchronises)
    DDAPlans plans(S);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (!rc) {
        const cudaError_t ce = cudaStreamIsCapturing(st, &cap);
        if (ce != cudaSuccess) rc = cuda_error(ce, "rg_em");
    }
    // (a subset's walks are recorded when the range runs it at least twice)
    auto uses = [&](int k) {
        const long long r = ((k - first) % S + S) % S;    // first j >= first with j % S == k
        return r < count ? (count - r - 1) / S + 1 : 0;
    };
    if (!rc && dda_plans_enabled() && cap == cudaStreamCaptureStatusNone)
        for (int k = 0; k < S && !rc; ++k)
            if (uses(k) >= 2)
                rc = dda_plan_build(g, cs, k, S, dda_plan_max_bytes(), plans.p[k], st);
    // bp must be zero on entry to transpose_k
    auto radon_k = [&](int k) {
        if (!plans.p[k].steps) return launch_bres_radon(g, cs, x, C, 1, ratio, 1, R, y, k, S, st);
        int rc2 = launch_to_am(x, C, 1, L, C, xT, st);          // xT[c * L + r] = x[r][c]
        return rc2 ? rc2 : launch_dda_plan_radon(g, plans.p[k], x, xT, ratio, y, st);
    };
    auto transpose_k = [&](int k) {
        if (!plans.p[k].steps) return launch_bres_transpose(g, cs, ratio, bp, k, S, st);
        int rc2 = launch_fill(bpT, npix, 0.f, st);
        if (!rc2) rc2 = launch_dda_plan_transpose(g, plans.p[k], ratio, bp, bpT, st);
        return rc2 ? rc2 : launch_add_from_am(bpT, L, C, bp, C, 1, st);
    };
    for (int k = 0; k < S && !rc; ++k) {
        if ((rc = launch_fill(bp, npix, 0.f, st))) break;
        if ((rc = transpose_k(k))) break;
        rc = launch_invert(bp, inv + (size_t)k * npix, npix, st);
    }
    for (long long j = first; j < first + count && !rc; ++j) {
            const int k = (int)(j % S);
            if ((rc = radon_k(k))) break;
            if ((rc = launch_fill(bp, npix, 0.f, st))) break;
            if ((rc = transpose_k(k))) break;
            rc = launch_em_update(x, bp, inv + (size_t)k * npix, npix, st);
        }
    if (!rc) rc = launch_copy2d(x, C, 1, image.data, image.column_stride, image.line_stride, L, C, st);
    scratch_end(s);
    return rc;
}

// Transmission EM (the update of raft/raft_transmission_em.cu:53-60 applied
// once per iteration; the reference multiplies twice, :57,59):
//   x <- x * A^T(b exp(-A x)) / A^T y,  y = max(raw - dark, 0),
//   b = max(flat - dark, 0),
// whose fixed point A^T(b exp(-A x)) = A^T y is the stationarity condition
// of the Poisson transmission likelihood.  exp is fused into the Radon
// epilogue and the update into the adjoint epilogue; 1 / A^T y is formed
// once in FP64 (0 where A^T y == 0).
static int tr_em_ss(const rg_image &raw, const rg_image &flat, const rg_image &dark,
                    const rg_image &image, int niter, void *ws, size_t wsb, cudaStream_t st)
{
    SSGeom g = make_ss_geom(image, raw);
    const int N = g.N, R = g.R, A = g.A;
    const SSPlan *p = nullptr;
    void *h = nullptr;
    int rc = get_ss_plan(g, 1, 0, &p, &h);
    if (rc) return rc;
    Holders hold;
    hold.h.push_back(h);
    if (!p->adj_ok)
        return set_error(RG_EUNSUPPORTED, "EM needs ray spacing >= pixel spacing (nrays <= size)");
    const size_t sb = (size_t)R * A * sizeof(float), ib = (size_t)N * N * sizeof(float);
    Scratch s;
    if ((rc = scratch_begin(s, ws, wsb, ws_sum({sb, sb, sb, sb, radon_pairs_bytes(N),
                                                radon_pairs_bytes(N), ib, ib}), st)))
        return rc;
    float *y = (float *)s.take(sb), *b = (float *)s.take(sb), *q = (float *)s.take(sb);
    float *d = (float *)s.take(sb);
    float2 *prow = (float2 *)s.take(radon_pairs_bytes(N));
    float2 *pcol = (float2 *)s.take(radon_pairs_bytes(N));
    float *x = (float *)s.take(ib), *inv = (float *)s.take(ib);
    rc = launch_to_am(raw.data, raw.column_stride, raw.line_stride, R, A, y, st);
    if (!rc) rc = launch_to_am(flat.data, flat.column_stride, flat.line_stride, R, A, b, st);
    if (!rc && dark.data) rc = launch_to_am(dark.data, dark.column_stride, dark.line_stride, R, A, d, st);
    if (!rc) rc = launch_sub_clamp(y, dark.data ? d : nullptr, y, (size_t)R * A, st);
    if (!rc) rc = launch_sub_clamp(b, dark.data ? d : nullptr, b, (size_t)R * A, st);
    if (!rc) rc = launch_copy2d(image.data, image.column_stride, image.line_stride, x, N, 1, N, N, st);
    if (!rc) rc = launch_gather(*p, 2, y, R, inv, N, 1, nullptr, nullptr, nullptr, st);
    for (int it = 0; it < niter && !rc; ++it) {
        if ((rc = launch_line_pairs(x, N, 1, N, prow, pcol, st))) break;
        if ((rc = launch_radon(*p, prow, pcol, q, R, b, R, st, 1, 0, 0, kEpiTransmissionId))) break;
        rc = launch_gather(*p, 1, q, R, nullptr, 0, 0, x, inv, nullptr, st);
    }
    if (!rc) rc = launch_copy2d(x, N, 1, image.data, image.column_stride, image.line_stride, N, N, st);
    scratch_end(s);
    return rc;
}

}  // namespace rg

using namespace rg;

extern "C" {

size_t rg_em_transmission_workspace(rg_image rawsino, rg_image image)
{
    const size_t sb = (size_t)rawsino.lines * rawsino.columns * sizeof(float);
    const size_t ib = (size_t)image.lines * image.columns * sizeof(float);
    return ws_sum({sb, sb, sb, sb, radon_pairs_bytes(image.lines), radon_pairs_bytes(image.lines),
                   ib, ib});
}

int rg_em_transmission(rg_image rawsino, rg_image flat, rg_image dark, rg_image image, int niter,
                       void *ws, size_t wsb, void *stream)
{
    RG_TRACE();
    if (!rawsino.data || !flat.data || !image.data)
        return set_error(RG_EINVAL, "rg_em_transmission: null data pointer");
    if (niter < 0) return set_error(RG_EINVAL, "rg_em_transmission: niter < 0");
    if (int rc0 = check_ws(ws)) return rc0;
    if (int rc0 = validate_ss(image, rawsino)) return rc0;
    if (flat.lines != rawsino.lines || flat.columns != rawsino.columns ||
        (dark.data && (dark.lines != rawsino.lines || dark.columns != rawsino.columns)))
        return set_error(RG_EINVAL, "rg_em_transmission: flat/dark shapes differ from the sinogram");
    return tr_em_ss(rawsino, flat, dark, image, niter, ws, wsb, (cudaStream_t)stream);
}

size_t rg_em_workspace(rg_image sino, rg_image image, int method, int nsubsets)
{
    const int S = nsubsets < 1 ? 1 : nsubsets;
    if (method == RG_BRESENHAM)
        return em_dda_ws(image.lines, image.columns, sino.lines, sino.columns, S);
    return em_ss_ws(image.lines, sino.lines, sino.columns, S);
}

static int em_range(rg_image sino, rg_image image, int method, int nsubsets, long long first,
                    long long count, void *ws, size_t wsb, void *stream)
{
    if (!sino.data || !image.data) return set_error(RG_EINVAL, "rg_em: null data pointer");
    if (int rc0 = check_ws(ws)) return rc0;
    if (nsubsets < 1 || nsubsets > sino.columns)
        return set_error(RG_EINVAL, "rg_em: nsubsets must be in [1, nviews]");
    cudaStream_t st = (cudaStream_t)stream;
    if (method == RG_BRESENHAM) return em_dda(sino, image, first, count, nsubsets, ws, wsb, st);
    if (method != RG_SLANTSTACK && method != RG_SLANTSTACK_BP)
        return set_error(RG_EINVAL, "rg_em: unknown method %d", method);
    if (image.lines != image.columns || image.lines < 2 || sino.lines < 2)
        return set_error(RG_EINVAL, "slant-stack EM needs a square image, size >= 2, nrays >= 2");
    SSGeom g;
    g.N = image.lines;
    g.itl_x = image.tl_x; g.itl_y = image.tl_y; g.ibr_x = image.br_x; g.ibr_y = image.br_y;
    g.R = sino.lines; g.A = sino.columns;
    g.stl_x = sino.tl_x; g.stl_y = sino.tl_y; g.sbr_x = sino.br_x; g.sbr_y = sino.br_y;
    const int N = g.N, R = g.R, A = g.A;
    Scratch s;
    int rc = scratch_begin(s, ws, wsb, rg_em_workspace(sino, image, method, nsubsets), st);
    if (rc) return rc;
    float *y = (float *)s.take((size_t)R * A * sizeof(float));
    float *x = (float *)s.take((size_t)N * N * sizeof(float));
    rc = launch_to_am(sino.data, sino.column_stride, sino.line_stride, R, A, y, st);
    if (!rc) rc = launch_copy2d(image.data, image.column_stride, image.line_stride, x, N, 1, N, N, st);
    if (!rc) rc = em_ss_core(g, first, count, nsubsets, y, x, s, st, method == RG_SLANTSTACK_BP);
    if (!rc) rc = launch_copy2d(x, N, 1, image.data, image.column_stride, image.line_stride, N, N, st);
    scratch_end(s);
    return rc;
}

int rg_em(rg_image sino, rg_image image, int method, int niter, int nsubsets, void *ws,
          size_t wsb, void *stream)
{
    RG_TRACE();
    if (niter < 0) return set_error(RG_EINVAL, "rg_em: niter < 0");
    const long long S = nsubsets < 1 ? 1 : nsubsets;
    return em_range(sino, image, method, nsubsets, 0, (long long)niter * S, ws, wsb, stream);
}

int rg_em_subiterations(rg_image sino, rg_image image, int method, int nsubsets, long long first,
                        long long count, void *ws, size_t wsb, void *stream)
{
    RG_TRACE();
    if (first < 0 || count < 0)
        return set_error(RG_EINVAL, "rg_em_subiterations: first and count must be >= 0");
    return em_range(sino, image, method, nsubsets, first, count, ws, wsb, stream);
}

}  // extern "C"
