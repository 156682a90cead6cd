// slantstack.cu -- slant-stack Radon, backprojection and matched adjoint.
//
// Reference semantics (restated, not translated):
//  * Radon  raft/raft_radon_slantstack.c:122-214 -- one line integral per
//    (view j, ray k): views th0 + j*(thf-th0)/nviews, rays tmin + k*dt; if
//    |cos| < 1/sqrt 2 the integral walks image columns i and interpolates
//    linearly between rows m, m+1 at y = t/sin - x_i/tan, else it walks rows
//    i (y_i = xmin + i*dy, as the reference) and interpolates between
//    columns at x = t/cos - y_i*tan; a sample counts iff its floor index m
//    lies in [0, N-2]; the sum is scaled by Delta = dy/|sin| or dx/|cos|.
//  * Backprojection raft/raft_backprojection_slantstack.c:121-180 -- pixel
//    (row j, col k) at (xmin + k dx, ymin + j dy) sums, over views, the
//    linear interpolation of the view's column at t = x cos + y sin (valid
//    iff the floor index is in [0, nrays-2]), times dth.
//  * Matched adjoint -- the exact transpose of the Radon above (no reference
//    counterpart): pixel (line i, position m) receives S[k]*Delta*hat(u_i(k)
//    - m) from every ray k whose sample on line i lies within one pixel, with
//    hat(x) = max(0, 1-|x|) and the same [0, N-2] floor validity.
//
// GB300 design:
//  * Radon is ray-driven over "line pairs": the image is pre-packed once per
//    call into (s - d, d) with d = s[n+1] - s[n], (0, 0) at n = N-1 and in
//    the pad entries, for both orientations (rows and columns).  One 8-byte
//    load then yields a sample, value = (s - d) + (1 + w) d, and invalid
//    samples read zeros, so the walks have no validity branch.  Ray sums
//    accumulate in FP32 in blocks of samples, compensated (Kahan) across
//    blocks.  Plans whose views come in runs of adjacent views use the
//    TMA-staged kernel of radon_tma.cu; the direct kernels here walk the
//    line pairs from L1/L2: a warp owns 32 consecutive rays of one view (a
//    CTA four views, or eight with two views per thread), and launches too
//    small for the GPU split their lines over a thread-block cluster.
//  * Backprojection and adjoint are pixel-driven gathers over tiles of 32
//    columns x 8 ROWS rows per CTA (256 threads, ROWS rows per thread, ROWS
//    autotuned over 4, 8 and 16).  Views are processed in chunks of 32: for
//    each view the tile needs a window of < W consecutive sinogram samples,
//    which is staged into shared memory as 8-byte pairs; the inner loop is
//    then one LDS.64 + two FP32 ops per (pixel, view) for the
//    backprojection, plus the two hat weights for the adjoint.  Grids of
//    few tiles split each tile's views over a thread-block cluster and add
//    the partials in distributed shared memory.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "ss_tiles.cuh"

namespace rg {

// ============================================================================
// Plans

static bool to_q32(double v, long long &out)
{
    double s = v * 4294967296.0;
    if (!(fabs(s) < 8.0e18)) return false;
    out = llrint(s);
    return true;
}

// Fills hv[0..nv) with the per-view constants and p's metadata (no device
// work).  Shared by the cached plans and the no-allocation Radon entry point.
int ss_views_compute(SSPlan &p, const SSGeom &g, const int *views, int nv, View *hv)
{
    if (g.N < 2 || g.R < 2 || g.A < 1)
        return set_error(RG_EINVAL, "slant-stack geometry needs size >= 2, nrays >= 2, "
                                    "nviews >= 1 (got %d, %d, %d)", g.N, g.R, g.A);
    const double xmin = g.itl_x, xmax = g.ibr_x, ymin = g.ibr_y, ymax = g.itl_y;
    const double dx = (xmax - xmin) / (g.N - 1), dy = (ymax - ymin) / (g.N - 1);
    const double th0 = g.stl_x, thf = g.sbr_x, dth = (thf - th0) / (g.A);
    const double tmin = g.sbr_y, tmax = g.stl_y, dt = (tmax - tmin) / (g.R - 1);
    if (!(std::isfinite(dx) && std::isfinite(dy) && std::isfinite(dth) && std::isfinite(dt)) ||
        dx == 0.0 || dy == 0.0 || dt == 0.0)
        return set_error(RG_EINVAL, "degenerate or non-finite corners");
    const double tol = 1.0 / sqrt(2);

    double wbp[3] = {0.0, 0.0, 0.0}, wadj[3] = {0.0, 0.0, 0.0};
    bool adj_ok = true;
    for (int e = 0; e < nv; ++e) {
        int j = views ? views[e] : e;
        if (j < 0 || j >= g.A) return set_error(RG_EINVAL, "view index %d out of range", j);
        const double theta = th0 + j * dth;
        const double c = cos(theta), s = sin(theta), tn = tan(theta);
        double rk, ri, r0, delta;
        View v = {};
        if (fabs(c) < tol) {            // lines are image columns
            rk = dt / (s * dy);
            ri = -dx / (tn * dy);
            r0 = (tmin / s - xmin / tn - ymin) / dy;
            delta = dy / fabs(s);
        } else {                         // lines are image rows
            rk = dt / (c * dx);
            ri = -dy * tn / dx;
            r0 = (tmin / c - xmin * tn - xmin) / dx;
            delta = dx / fabs(c);
            v.flags |= kLinesAreRows;
        }
        if (rk < 0) v.flags |= kRkNegative;
        double krow, kcol, k0 = -r0 / rk;
        if (v.flags & kLinesAreRows) { krow = -ri / rk; kcol = 1.0 / rk; }
        else                         { krow = 1.0 / rk;  kcol = -ri / rk; }
        const double brow = dy * s / dt, bcol = dx * c / dt;
        const double b0 = (xmin * c + ymin * s - tmin) / dt;
        bool ok = to_q32(rk, v.rk) && to_q32(ri, v.ri) && to_q32(r0, v.r0) &&
                  to_q32(brow, v.brow) && to_q32(bcol, v.bcol) && to_q32(b0, v.b0) &&
                  to_q32(krow, v.krow) && to_q32(kcol, v.kcol) && to_q32(k0, v.k0);
        // Every position the kernels form (origin + index * step, in Q32.32)
        // must stay far inside int64: bound them by 2^30 samples.
        const double lim = 1073741824.0;
        ok = ok && fabs(r0) + (g.R - 1) * fabs(rk) + (g.N - 1) * fabs(ri) < lim &&
             fabs(b0) + (g.N - 1) * (fabs(brow) + fabs(bcol)) < lim &&
             fabs(k0) + (g.N - 1) * (fabs(krow) + fabs(kcol)) < lim;
        if (!ok) return set_error(RG_EUNSUPPORTED, "view %d: positions exceed 2^30 samples "
                                                   "(image and sinogram extents too different)", j);
        v.delta = (float)delta;
        v.delta64 = delta;
        v.P = (float)fabs(rk);
        v.view = j;
        if (fabs(rk) < 1.0 - 1e-9) adj_ok = false;
        for (int t = 0; t < 3; ++t) {
            const double th = t == 2 ? 127.0 : t ? 63.0 : 31.0;   // tile height - 1
            wbp[t] = std::max(wbp[t], th * fabs(brow) + 31.0 * fabs(bcol));
            wadj[t] = std::max(wadj[t], th * fabs(krow) + 31.0 * fabs(kcol));
        }
        hv[e] = v;
    }
    p.g = g;
    p.nv = nv;
    p.contiguous = true;
    for (int e = 1; e < nv; ++e)
        if ((views ? views[e] : e) != (views ? views[e - 1] : e - 1) + 1) p.contiguous = false;
    p.dth = (float)dth;
    p.adj_ok = adj_ok;
    // The plan's second half of views is its first half a quarter turn on
    // (view j + A/2 for view j: all views, or an OSEM subset when the
    // subset count divides A/2), over a span of pi, on a grid that the turn
    // maps onto itself (x and y on the same points, centred on 0).
    const double pi = 3.14159265358979323846;
    p.rot_ok = nv >= 2 && nv % 2 == 0 && g.A % 2 == 0 && fabs((thf - th0) - pi) <= 1e-12 * pi &&
               g.itl_x == g.ibr_y && g.ibr_x == g.itl_y && g.itl_x == -g.ibr_x;
    // A half turn maps the grid onto itself and t onto -t: x and y each
    // centred on 0, and the detector's t range centred on 0.
    p.mirror_ok = g.itl_x == -g.ibr_x && g.itl_y == -g.ibr_y && g.stl_y == -g.sbr_y;
    for (int e = 0; e < nv / 2 && p.rot_ok; ++e) {
        const int j = views ? views[e] : e, j2 = views ? views[e + nv / 2] : e + nv / 2;
        p.rot_ok = j2 == j + g.A / 2;
    }
    for (int t = 0; t < 3; ++t) {
        p.wmax_bp[t] = (int)ceil(wbp[t] + 1e-6) + 4;
        p.wmax_adj[t] = (int)ceil(wadj[t] + 1e-6) + 4;
    }
    return RG_OK;
}

int ss_plan_build(SSPlan &p, const SSGeom &g, const int *views, int nv)
{
    std::vector<View> hv(nv > 0 ? nv : 1);
    int rc = ss_views_compute(p, g, views, nv, hv.data());
    if (rc) return rc;
    RG_CK(cudaGetDevice(&p.device));
    if (nv > 0) {
        RG_CK(cudaMalloc(&p.d_views, sizeof(View) * nv));
        RG_CK(cudaMemcpy(p.d_views, hv.data(), sizeof(View) * nv, cudaMemcpyHostToDevice));
        if ((rc = ensure_device_error_word())) return rc;
        if ((rc = st_blocks_build(p, hv.data()))) return rc;
        if ((rc = tt_build(p, hv.data()))) return rc;
    }
    return RG_OK;
}

void ss_plan_free(SSPlan &p)
{
    if (p.d_views) cudaFree(p.d_views);
    p.d_views = nullptr;
    if (p.d_blocks) cudaFree(p.d_blocks);
    p.d_blocks = nullptr;
    p.d_border = nullptr;
    p.nblocks = 0;
    if (p.d_ovid) cudaFree(p.d_ovid);
    p.d_ovid = nullptr;
    p.tt_ok = false;
}

// ============================================================================
// Line pairs for the Radon.  pitch = pairs_pitch(N) (N + 2 rounded up to
// even): entry 1 + n holds the pair of sample n, entry 0 and every entry
// from N + 1 on are zero pads.

size_t radon_pairs_bytes(int N) { return (size_t)N * pairs_pitch(N) * sizeof(float2); }

// blockIdx.z selects one image of a stack (strides zi in floats, zp in pairs).
__global__ __launch_bounds__(256) void k_line_pairs(const float *__restrict__ img, long long cs,
                                                    long long ls, int N,
                                                    float2 *__restrict__ prow,
                                                    float2 *__restrict__ pcol, long long zi,
                                                    long long zp)
{
    pdl_gate();
    line_pairs_tile(img + blockIdx.z * zi, cs, ls, N, prow + blockIdx.z * zp,
                    pcol + blockIdx.z * zp, blockIdx.x, blockIdx.y);
}

int launch_line_pairs(const float *img, long long cs, long long ls, int N, float2 *prow,
                      float2 *pcol, cudaStream_t st, int nz, long long zi, long long zp)
{
    dim3 grid((N + 31) / 32, (N + 31) / 32, nz);
    RG_CK(launch_pdl(k_line_pairs, grid, 256, 0, st, 1, img, cs, ls, N, prow, pcol, zi, zp));
    RG_CK_LAUNCH("k_line_pairs");
    return RG_OK;
}

template <int EPI>
__global__ __launch_bounds__(128) void k_radon(const float2 *__restrict__ prow,
                                               const float2 *__restrict__ pcol, int N,
                                               const View *__restrict__ views, int nv, int R,
                                               float *__restrict__ out_am, int out_ld,
                                               const float *__restrict__ y_am, int y_ld,
                                               long long zp, long long zo, int split)
{
    pdl_gate();
    radon_tile<EPI>(prow + blockIdx.z * zp, pcol + blockIdx.z * zp, N, views, nv, R,
                    out_am + blockIdx.z * zo, out_ld, y_am, y_ld, blockIdx.x / split, blockIdx.y,
                    split, blockIdx.x % split);
}

// Line split of the direct Radon (clusters of `split` CTAs, see radon_tile):
// the largest of 1, 2, 4 that keeps the grid within two waves of resident
// CTAs, so launches smaller than the GPU get more CTAs in flight.  The
// per-SM occupancy is cached per kernel and device (queried outside stream
// captures; an uncached query during a capture gives 1).
// RG_RADON_SPLIT=1|2|4 forces a choice.
static std::mutex g_rocc_mu;
static std::map<std::pair<const void *, int>, int> g_rocc;

template <typename K>
static int radon_split(K k, long long ctas, cudaStream_t st)
{
    if (const char *e = getenv("RG_RADON_SPLIT")) {
        const int v = atoi(e);
        if (v == 1 || v == 2 || v == 4) return v;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    const auto key = std::make_pair((const void *)k, dev);
    int cap = 0;
    {
        std::lock_guard<std::mutex> lock(g_rocc_mu);
        auto it = g_rocc.find(key);
        if (it != g_rocc.end()) cap = it->second;
    }
    if (!cap) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)
            return 1;
        int per_sm = 0, sms = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 128, 0) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return 1;
        cap = per_sm * sms;
        std::lock_guard<std::mutex> lock(g_rocc_mu);
        g_rocc[key] = cap;
    }
    int s = 1;
    while (s < 4 && ctas * 2 * s <= 2 * cap) s *= 2;   // up to two waves
    return s;
}

template <int EPI>
static int launch_radon_direct1(const SSPlan &p, const float2 *prow, const float2 *pcol,
                                float *out_am, int out_ld, const float *y_am, int y_ld,
                                cudaStream_t st, int nz, long long zp, long long zo)
{
    const int N = p.g.N, R = p.g.R;
    dim3 grid((R + 31) / 32, (p.nv + 3) / 4, nz);
    auto k = k_radon<EPI>;
    const int split = radon_split(k, (long long)grid.x * grid.y * grid.z, st);
    RG_CK(launch_pdl(k, dim3(grid.x * split, grid.y, grid.z), 128, 0, st, split,
                     prow, pcol, N, (const View *)p.d_views, p.nv, R, out_am,
                     out_ld, y_am, y_ld, zp, zo, split));
    RG_CK_LAUNCH("k_radon");
    return RG_OK;
}

template <int EPI>
__global__ __launch_bounds__(128) void k_radon2(const float2 *__restrict__ prow,
                                                const float2 *__restrict__ pcol, int N,
                                                const View *__restrict__ views, int nv, int R,
                                                float *__restrict__ out_am, int out_ld,
                                                const float *__restrict__ y_am, int y_ld,
                                                long long zp, long long zo)
{
    pdl_gate();
    radon_tile2<EPI>(prow + blockIdx.z * zp, pcol + blockIdx.z * zp, N, views, nv, R,
                       out_am + blockIdx.z * zo, out_ld, y_am, y_ld, blockIdx.x, blockIdx.y);
}

int radon_views_per_thread(const SSPlan &p)
{
    const char *e = getenv("RG_RADON_VIEWS");
    if (e && (atoi(e) == 1 || atoi(e) == 2)) return atoi(e);
    return p.contiguous ? 2 : 1;
}

int launch_radon(const SSPlan &p, const float2 *prow, const float2 *pcol, float *out_am,
                 int out_ld, const float *y_am, int y_ld, cudaStream_t st, int nz, long long zp,
                 long long zo, int epi)
{
    if (p.nv == 0) return RG_OK;
    if (epi < 0) epi = y_am ? kEpiRatio : kEpiSum;
    if (radon_tma_usable(p))
        return launch_radon_tma(p, prow, pcol, out_am, out_ld, y_am, y_ld, st, nz, zp, zo, epi);
    if (radon_tiles_usable(p))
        return launch_radon_tiles(p, prow, pcol, out_am, out_ld, y_am, y_ld, st, nz, zp, zo, epi);
    const int N = p.g.N, R = p.g.R;
    if (radon_views_per_thread(p) == 2) {
        dim3 grid((R + 31) / 32, (p.nv + 7) / 8, nz);
        if (epi == kEpiRatio)
            RG_CK(launch_pdl(k_radon2<kEpiRatio>, grid, 128, 0, st, 1, prow, pcol, N, p.d_views,
                             p.nv, R, out_am, out_ld, y_am, y_ld, zp, zo));
        else if (epi == kEpiTransmission)
            RG_CK(launch_pdl(k_radon2<kEpiTransmission>, grid, 128, 0, st, 1, prow, pcol, N,
                             p.d_views, p.nv, R, out_am, out_ld, y_am, y_ld, zp, zo));
        else
            RG_CK(launch_pdl(k_radon2<kEpiSum>, grid, 128, 0, st, 1, prow, pcol, N, p.d_views,
                             p.nv, R, out_am, out_ld, nullptr, 0, zp, zo));
        RG_CK_LAUNCH("k_radon2");
        return RG_OK;
    }
    if (epi == kEpiRatio)
        return launch_radon_direct1<kEpiRatio>(p, prow, pcol, out_am, out_ld, y_am, y_ld, st, nz,
                                               zp, zo);
    if (epi == kEpiTransmission)
        return launch_radon_direct1<kEpiTransmission>(p, prow, pcol, out_am, out_ld, y_am, y_ld,
                                                      st, nz, zp, zo);
    return launch_radon_direct1<kEpiSum>(p, prow, pcol, out_am, out_ld, nullptr, 0, st, nz, zp,
                                         zo);
}

template <int MODE, int WMAX, int ROWS, bool EM>
__global__ __launch_bounds__(256) void k_gather(const float *__restrict__ s_am, int s_ld, int R,
                                                const View *__restrict__ views, int nv, int N,
                                                float scale, float *__restrict__ out,
                                                long long cs, long long ls,
                                                float *__restrict__ em_x,
                                                const float *__restrict__ inv_sens,
                                                int *__restrict__ err, long long zs,
                                                long long zo, unsigned pair_bytes, int split)
{
    pdl_gate();
    extern __shared__ float2 pairs[];          // [kSlots][WMAX]
    gather_tile<MODE, WMAX, ROWS, EM>(s_am + blockIdx.z * zs, s_ld, R, views, nv, N, scale,
                                      out + blockIdx.z * zo, cs, ls, em_x, inv_sens, err,
                                      blockIdx.x / split, blockIdx.y, pairs, pair_bytes, split,
                                      blockIdx.x % split, MODE != 0);
}

// The matched adjoint (optionally with the EM update) on tile pairs related
// by a half turn (gather_tile_mirror, ss_tiles.cuh): blockIdx.y covers the
// upper half of the tile rows, and the views of a pair may be split over a
// cluster along x as in k_gather.  Registers are held to 64 (four CTAs per
// SM), without spills at any tile height: the batched form measured that
// much faster than the compiler's choice (73 registers at 16 rows).
template <int WMAX, int ROWS, bool EM>
__global__ __launch_bounds__(256, 4) void k_gather_mirror(
    const float *__restrict__ s_am, int s_ld, int R, const View *__restrict__ views, int nv, int N,
    float *__restrict__ out, long long cs, long long ls, float *__restrict__ em_x,
    const float *__restrict__ inv_sens, int *__restrict__ err, long long zs, long long zo,
    unsigned quad_bytes, int split)
{
    pdl_gate();
    extern __shared__ __align__(16) float4 mq[];   // [kSlots / 2][WMAX], or 2 ROWS x 256 floats
    gather_tile_mirror<WMAX, ROWS, EM>(s_am + blockIdx.z * zs, s_ld, R, views, nv, N,
                                       out + blockIdx.z * zo, cs, ls, em_x, inv_sens, err,
                                       blockIdx.x / split, blockIdx.y, mq, quad_bytes, split,
                                       blockIdx.x % split);
}

// RG_GATHER_MIRROR=0: the one-view adjoint runs tile by tile even where its
// tiles pair with their half-turn mirrors.
static bool gather_mirror_enabled()
{
    const char *e = getenv("RG_GATHER_MIRROR");
    return !(e && !strcmp(e, "0"));
}

// Edge pixels of the matched adjoint and of its FP64 sensitivity
// (adjoint_edge_group, ss_tiles.cuh): one CTA per 32 consecutive pixels of
// the image's first and last rows and columns, its WARPS warps splitting
// the views: 32 for the gathers whose edge pixels have no other home; 8 for
// the stacks of the paired gathers, whose one-slice form computes its edges
// with 8 warps inside the gather's own launch (rot_edges), so that the
// same split sums in the same order and a stack's members equal separate
// calls bit for bit.
template <int MODE, bool EM, int WARPS>
__global__ __launch_bounds__(WARPS * 32) void k_adjoint_edges(const float *__restrict__ s_am,
                                                              int s_ld, int R,
                                                              const View *__restrict__ views,
                                                              int nv, int N,
                                                              float *__restrict__ out,
                                                              long long cs, long long ls,
                                                              float *__restrict__ em_x,
                                                              const float *__restrict__ inv_sens,
                                                              long long zs, long long zo)
{
    pdl_gate();
    adjoint_edge_group<MODE, EM, WARPS>(s_am + blockIdx.z * zs, s_ld, R, views, nv, N,
                                        blockIdx.x * 32, out + blockIdx.z * zo, cs, ls, em_x,
                                        inv_sens);
}

template <int MODE, bool EM, int WARPS = 32>
static int adjoint_edges(const SSPlan &p, const float *s_am, int s_ld, float *out, long long cs,
                         long long ls, float *em_x, const float *inv_sens, cudaStream_t st,
                         const Stack &z)
{
    const int N = p.g.N;
    dim3 grid((4 * N - 4 + 31) / 32, 1, z.n);   // 32 edge pixels per CTA
    RG_CK(launch_pdl(k_adjoint_edges<MODE, EM, WARPS>, grid, WARPS * 32, 0, st, 1, s_am, s_ld,
                     p.g.R, p.d_views, p.nv, N, out, cs, ls, em_x, inv_sens, z.in, z.out));
    RG_CK_LAUNCH("k_adjoint_edges");
    return RG_OK;
}

// Cluster size for the view split of a gather launch of `tiles` CTAs.  The
// calling thread's preference (the autotuner's choice for the geometry, or
// the candidate it is timing) is taken where ROWS is divisible by it, every
// rank keeps 16 views and the kernel's clusters fit; otherwise the occupancy
// rule: the split in {1, 2, 4} (ROWS divisible by it, >= 64 views per rank)
// whose last wave is fullest, from the occupancy of the kernel (clusters
// counted by cudaOccupancyMaxActiveClusters), on the tiles of one slice:
// the split changes the summation order, so it follows the geometry alone
// and a stack's members equal separate calls bit for bit.  Occupancies are
// cached per kernel, so launches inside a stream capture make no queries
// once the plain call has run; an uncached query during a capture gives
// split 1.  RG_GATHER_SPLIT=1|2|4 forces a choice.
struct SplitOcc {
    int slots[3] = {0, 0, 0};      // concurrent CTAs at split 1, 2, 4
};
static std::mutex g_occ_mu;
static std::map<std::pair<const void *, int>, SplitOcc> g_occ;

static int env_split()
{
    const char *e = getenv("RG_GATHER_SPLIT");
    if (!e) return 0;
    const int v = atoi(e);
    return (v == 1 || v == 2 || v == 4) ? v : 0;
}

template <typename K>
static int pick_split(K k, size_t smem, int rows, int nv, dim3 grid, cudaStream_t st)
{
    return gather_pick_split((const void *)k, smem, rows, nv, grid, st);
}

static thread_local int t_split_pref = 0;

int split_preference() { return t_split_pref; }
SplitPref::SplitPref(int split) : saved(t_split_pref) { t_split_pref = split; }
SplitPref::~SplitPref() { t_split_pref = saved; }

int gather_pick_split(const void *k, size_t smem, int rows, int nv, dim3 grid, cudaStream_t st)
{
    const int forced = env_split();
    if (forced) return (rows % forced == 0 && nv >= forced) ? forced : 1;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    const auto key = std::make_pair(k, dev * 4096 + (int)(smem >> 10));
    SplitOcc occ;
    bool have = false;
    {
        std::lock_guard<std::mutex> lock(g_occ_mu);
        auto it = g_occ.find(key);
        if (it != g_occ.end()) { occ = it->second; have = true; }
    }
    if (!have) {
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
            return 1;
        int per_sm = 0, sms = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, smem) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return 1;
        occ.slots[0] = per_sm * sms;
        for (int t = 1; t < 3; ++t) {
            const int S = 1 << t;
            cudaLaunchConfig_t cfg = {};
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = S;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.gridDim = dim3(grid.x * S, grid.y, grid.z);
            cfg.blockDim = dim3(256);
            cfg.dynamicSmemBytes = smem;
            cfg.stream = st;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int ncl = 0;
            if (cudaOccupancyMaxActiveClusters(&ncl, k, &cfg) != cudaSuccess) {
                cudaGetLastError();
                ncl = 0;
            }
            occ.slots[t] = ncl * S;
        }
        std::lock_guard<std::mutex> lock(g_occ_mu);
        g_occ[key] = occ;
    }
    // a preferred split (the autotuner's) where every rank keeps 16 views
    // and the clusters fit on the device
    const int pref = t_split_pref;
    if (pref == 1) return 1;
    if (pref == 2 || pref == 4) {
        const int t = pref == 2 ? 1 : 2;
        if (rows % pref == 0 && nv >= 16 * pref && occ.slots[t] > 0) return pref;
    }
    // one slice's tiles: the split follows the geometry alone, so a stack
    // (grid z) sums in the same order as separate calls
    const double tiles = (double)grid.x * grid.y;
    int best = 1;
    double best_e = 0.0;
    for (int t = 0; t < 3; ++t) {
        const int S = 1 << t;
        if (rows % S || nv < 64 * S || occ.slots[t] <= 0) continue;
        const double w = tiles * S / occ.slots[t];
        // fullness of the last wave, less a small cost per extra CTA
        const double e = w / ceil(w) - 0.01 * (S - 1);
        if (e > best_e + 1e-9) { best_e = e; best = S; }
    }
    return best;
}

// Whether the matched adjoint of plan p with ROWS rows per thread runs on
// half-turn mirrored tile pairs: a centred geometry whose tiles pair up.
static bool mirror_applies(const SSPlan &p, int rows)
{
    const int N = p.g.N;
    return p.mirror_ok && N % 64 == 0 && N % (2 * kWarps * rows) == 0 && gather_mirror_enabled();
}

template <int WMAX, int ROWS, bool EM>
static int gather_w_mirror(const SSPlan &p, const float *s_am, int s_ld, float *out, long long cs,
                           long long ls, float *em_x, const float *inv_sens, int *d_err,
                           cudaStream_t st, const Stack &z)
{
    const int N = p.g.N;
    // quads of kSlots / 2 views, or the cluster reduction's 2 ROWS x 256 floats
    const size_t smem = std::max((size_t)(kSlots / 2) * WMAX * sizeof(float4),
                                 (size_t)2 * ROWS * 256 * sizeof(float));
    dim3 grid(N / kTile, N / (2 * kWarps * ROWS), z.n);
    auto k = k_gather_mirror<WMAX, ROWS, EM>;
    RG_CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int split = pick_split(k, smem, ROWS, p.nv, grid, st);
    const unsigned qb = (unsigned)sizeof(float4);
    if (int rc = adjoint_edges<1, EM>(p, s_am, s_ld, out, cs, ls, em_x, inv_sens, st, z)) return rc;
    RG_CK(launch_pdl(k, dim3(grid.x * split, grid.y, grid.z), 256, smem, st, split,
                     s_am, s_ld, p.g.R, (const View *)p.d_views, p.nv, N, out, cs,
                     ls, em_x, inv_sens, d_err, z.in, z.out, qb, split));
    RG_CK_LAUNCH("k_gather_mirror");
    return RG_OK;
}

template <int MODE, int WMAX, int ROWS, bool EM>
static int gather_w(const SSPlan &p, const float *s_am, int s_ld, float *out, long long cs,
                    long long ls, float *em_x, const float *inv_sens, int *d_err,
                    cudaStream_t st, const Stack &z)
{
    const size_t smem = (size_t)kSlots * WMAX * sizeof(float2);
    dim3 grid((p.g.N + kTile - 1) / kTile, (p.g.N + kWarps * ROWS - 1) / (kWarps * ROWS), z.n);
    const float scale = (MODE == 0) ? p.dth : 1.f;
    if constexpr (MODE == 1) {
        // Half-turn mirrored tile pairs (gather_tile_mirror) on a centred
        // geometry whose tiles pair up.
        if (mirror_applies(p, ROWS))
            return gather_w_mirror<WMAX, ROWS, EM>(p, s_am, s_ld, out, cs, ls, em_x, inv_sens,
                                                   d_err, st, z);
    }
    auto k = k_gather<MODE, WMAX, ROWS, EM>;
    RG_CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int split = (MODE == 2) ? 1 : pick_split(k, smem, ROWS, p.nv, grid, st);
    const unsigned pb = (unsigned)sizeof(float2);
    if constexpr (MODE != 0) {
        // the gather leaves the edge pixels to k_adjoint_edges
        if (int rc = adjoint_edges<MODE, EM>(p, s_am, s_ld, out, cs, ls, em_x, inv_sens, st, z))
            return rc;
    }
    RG_CK(launch_pdl(k, dim3(grid.x * split, grid.y, grid.z), 256, smem, st, split,
                     s_am, s_ld, p.g.R, (const View *)p.d_views, p.nv, p.g.N,
                     scale, out, cs, ls, em_x, inv_sens, d_err, z.in, z.out, pb, split));
    RG_CK_LAUNCH("k_gather");
    return RG_OK;
}

template <int MODE, int ROWS, bool EM>
static int gather_mode(const SSPlan &p, int wneed, const float *s_am, int s_ld, float *out,
                       long long cs, long long ls, float *em_x, const float *inv_sens,
                       int *d_err, cudaStream_t st, const Stack &z)
{
    if (wneed <= 64) return gather_w<MODE, 64, ROWS, EM>(p, s_am, s_ld, out, cs, ls, em_x, inv_sens, d_err, st, z);
    if (wneed <= 128) return gather_w<MODE, 128, ROWS, EM>(p, s_am, s_ld, out, cs, ls, em_x, inv_sens, d_err, st, z);
    if (wneed <= 256) return gather_w<MODE, 256, ROWS, EM>(p, s_am, s_ld, out, cs, ls, em_x, inv_sens, d_err, st, z);
    if (wneed <= 512) return gather_w<MODE, 512, ROWS, EM>(p, s_am, s_ld, out, cs, ls, em_x, inv_sens, d_err, st, z);
    return set_error(RG_EUNSUPPORTED,
                     "gather window of %d samples per tile exceeds 512 "
                     "(image much coarser than the ray spacing)", wneed);
}

template <int MODE, bool EM>
static int gather_rows(const SSPlan &p, int rows, const float *s_am, int s_ld, float *out,
                       long long cs, long long ls, float *em_x, const float *inv_sens, int *d_err,
                       cudaStream_t st, const Stack &z)
{
    const int t = rows == 16 ? 2 : rows == 8 ? 1 : 0;
    const int w = (MODE == 0) ? p.wmax_bp[t] : p.wmax_adj[t];
    if (rows == 16)
        return gather_mode<MODE, 16, EM>(p, w, s_am, s_ld, out, cs, ls, em_x, inv_sens, d_err, st, z);
    if (rows == 8)
        return gather_mode<MODE, 8, EM>(p, w, s_am, s_ld, out, cs, ls, em_x, inv_sens, d_err, st, z);
    return gather_mode<MODE, 4, EM>(p, w, s_am, s_ld, out, cs, ls, em_x, inv_sens, d_err, st, z);
}

// RG_GATHER_ROT=0 keeps the one-view backprojection and adjoint where the
// paired ones apply.
bool gather_rot_enabled()
{
    const char *e = getenv("RG_GATHER_ROT");
    return !(e && !strcmp(e, "0"));
}

int launch_gather(const SSPlan &p, int mode, const float *s_am, int s_ld, float *out,
                  long long cs, long long ls, float *em_x, const float *inv_sens, int *d_err,
                  cudaStream_t st, int rows, Stack z, void *quads, const EmFuse *fuse)
{
    // launch shape: the caller's rows and split preference, else the tuned
    // choice for this geometry (a stack takes the one-slice choice, so its
    // members come out as separate calls would give them)
    int pref = split_preference();
    if (rows == 0) {
        const TuneChoice c = tuned_choice(p, mode);
        rows = c.rows;
        pref = c.split;
    }
    SplitPref use_split(pref);
    // the kernels OR their error bits (window checks, bounded waits) into the
    // device's status word, which rg_device_status() reads and clears
    if (!d_err) d_err = device_error_word();
    // EM update fused into the paired gathers (EmFuse): the adjoint's edge
    // pixels are updated first by their own kernel, the rest by the gather
    EmFuse ef;
    const bool fused = em_x && fuse && mode != 2 && p.rot_ok && gather_rot_enabled() &&
                       em_fusable(p.g.N) && z.n == 1;
    if (fused) {
        ef = *fuse;
        ef.x = em_x;
        ef.inv = inv_sens;
    }
    if (mode == 0) {
        if (!em_x && p.rot_ok && gather_rot_enabled())
            return launch_gather_rot(p, 0, s_am, s_ld, out, cs, ls, d_err, st, rows, z, quads,
                                     true);
        if (fused)
            return launch_gather_rot(p, 0, s_am, s_ld, ef.gsum, p.g.N, 1, d_err, st, rows, z,
                                     quads, false, &ef);
        if (em_x)
            return gather_rows<0, true>(p, rows, s_am, s_ld, out, cs, ls, em_x, inv_sens, d_err, st, z);
        return gather_rows<0, false>(p, rows, s_am, s_ld, out, cs, ls, nullptr, nullptr, d_err, st, z);
    }
    if (!p.adj_ok)
        return set_error(RG_EUNSUPPORTED,
                         "matched adjoint needs ray spacing >= pixel spacing along each line "
                         "(nrays <= size for the default extents)");
    if (mode == 1) {
        // For one slice, the paired gathers compute the edge pixels in extra
        // CTAs of their own launch (rot_edges), which fill the grid's last
        // wave; a stack's many-wave grid gains nothing from them, and its
        // edges keep a kernel of their own, with the same 8-warp view split.
        if (!em_x && p.rot_ok && gather_rot_enabled()) {
            if (int rc = launch_zero_image(out, p.g.N, cs, ls, st, z)) return rc;
            if (z.n > 1)
                if (int rc = adjoint_edges<1, false, kWarps>(p, s_am, s_ld, out, cs, ls, nullptr,
                                                             nullptr, st, z))
                    return rc;
            return launch_gather_rot(p, 1, s_am, s_ld, out, cs, ls, d_err, st, rows, z, quads,
                                     false, nullptr, z.n == 1);
        }
        if (fused)
            return launch_gather_rot(p, 1, s_am, s_ld, ef.gsum, p.g.N, 1, d_err, st, rows, z,
                                     quads, false, &ef, true);
        if (em_x)
            return gather_rows<1, true>(p, rows, s_am, s_ld, out, cs, ls, em_x, inv_sens, d_err, st, z);
        return gather_rows<1, false>(p, rows, s_am, s_ld, out, cs, ls, nullptr, nullptr, d_err, st, z);
    }
    return gather_rows<2, false>(p, rows, s_am, s_ld, out, cs, ls, nullptr, nullptr, d_err, st, z);
}

}  // namespace rg
