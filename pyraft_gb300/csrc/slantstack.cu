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
//  * Radon is ray-driven: a warp owns 32 consecutive rays of one view and a
//    CTA four adjacent views, so at every line the four warps read
//    overlapping windows of the same image line (L1 reuse).  The image is
//    pre-packed once per call into "line pairs" (s - d, d) with
//    d = s[n+1] - s[n] and (0, 0) at n = N-1 and in one pad entry at each
//    end, for both orientations (rows and columns).  One 8-byte load then
//    yields a sample: value = (s - d) + (1 + w) d, and invalid samples read
//    zeros, so the loop has no validity branch.  Ray sums accumulate in FP32
//    in blocks of 32 samples, compensated (Kahan) across blocks.
//  * Backprojection and adjoint are pixel-driven gathers over a 32 x 32
//    pixel tile per CTA (256 threads, 4 rows each).  Views are processed in
//    chunks of 32: for each view the tile needs a window of < W consecutive
//    sinogram samples, which is staged into shared memory as 8-byte pairs;
//    the inner loop is then one LDS.64 + two FP32 ops per (pixel, view) for
//    the backprojection, plus the two hat weights for the adjoint.
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <vector>

#include "rg_internal.cuh"

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

    double wbp = 0.0, wadj = 0.0;
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
        v.P = (float)fabs(rk);
        v.view = j;
        if (fabs(rk) < 1.0 - 1e-9) adj_ok = false;
        wbp = std::max(wbp, 31.0 * (fabs(brow) + fabs(bcol)));
        wadj = std::max(wadj, 31.0 * (fabs(krow) + fabs(kcol)));
        hv[e] = v;
    }
    p.g = g;
    p.nv = nv;
    p.dth = (float)dth;
    p.adj_ok = adj_ok;
    p.wmax_bp = (int)ceil(wbp + 1e-6) + 4;
    p.wmax_adj = (int)ceil(wadj + 1e-6) + 4;
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
    }
    return RG_OK;
}

void ss_plan_free(SSPlan &p)
{
    if (p.d_views) cudaFree(p.d_views);
    p.d_views = nullptr;
}

// ============================================================================
// Line pairs for the Radon.  pitch = N + 2: entry 0 and N+1 are zero pads,
// entry 1 + n holds the pair of sample n.

size_t radon_pairs_bytes(int N) { return (size_t)N * (N + 2) * sizeof(float2); }

__device__ __forceinline__ float2 make_pair(float s0, float s1, bool valid)
{
    float d = s1 - s0;
    return valid ? make_float2(s0 - d, d) : make_float2(0.f, 0.f);
}

// One CTA packs a 32 x 32 image tile into both orientations.
__global__ __launch_bounds__(256) void k_line_pairs(const float *__restrict__ img, long long cs,
                                                    long long ls, int N,
                                                    float2 *__restrict__ prow,
                                                    float2 *__restrict__ pcol)
{
    __shared__ float t[33][33];
    const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
    const int pitch = N + 2;
    for (int e = threadIdx.x; e < 33 * 33; e += 256) {
        int y = e / 33, x = e % 33;
        int r = r0 + y, c = c0 + x;
        t[y][x] = (r < N && c < N) ? img[(long long)r * cs + (long long)c * ls] : 0.f;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int y = w; y < 32; y += 8) {        // rows: consecutive lanes = columns
        int r = r0 + y, c = c0 + lane;
        if (r < N && c < N)
            prow[(size_t)r * pitch + 1 + c] = make_pair(t[y][lane], t[y][lane + 1], c <= N - 2);
    }
    for (int x = w; x < 32; x += 8) {        // columns: consecutive lanes = rows
        int c = c0 + x, r = r0 + lane;
        if (r < N && c < N)
            pcol[(size_t)c * pitch + 1 + r] = make_pair(t[lane][x], t[lane + 1][x], r <= N - 2);
    }
    // zero pads of the lines this tile starts / ends
    if (c0 == 0 && threadIdx.x < 32 && r0 + lane < N) {
        prow[(size_t)(r0 + lane) * pitch] = make_float2(0.f, 0.f);
        prow[(size_t)(r0 + lane) * pitch + N + 1] = make_float2(0.f, 0.f);
    }
    if (r0 == 0 && threadIdx.x < 32 && c0 + lane < N) {
        pcol[(size_t)(c0 + lane) * pitch] = make_float2(0.f, 0.f);
        pcol[(size_t)(c0 + lane) * pitch + N + 1] = make_float2(0.f, 0.f);
    }
}

int launch_line_pairs(const float *img, long long cs, long long ls, int N, float2 *prow,
                      float2 *pcol, cudaStream_t st)
{
    dim3 grid((N + 31) / 32, (N + 31) / 32);
    k_line_pairs<<<grid, 256, 0, st>>>(img, cs, ls, N, prow, pcol);
    RG_CK_LAUNCH("k_line_pairs");
    return RG_OK;
}

// ============================================================================
// Radon: CTA = 32 rays x 4 views (one warp per view).

__device__ __forceinline__ void kahan_add(float &sum, float &c, float x)
{
    float y = x - c;
    float t = sum + y;
    c = (t - sum) - y;
    sum = t;
}

template <bool RATIO>
__global__ __launch_bounds__(128) void k_radon(const float2 *__restrict__ prow,
                                               const float2 *__restrict__ pcol, int N,
                                               const View *__restrict__ views, int nv, int R,
                                               float *__restrict__ out_am, int out_ld,
                                               const float *__restrict__ y_am, int y_ld)
{
    const int k = blockIdx.x * 32 + (threadIdx.x & 31);
    const int e = blockIdx.y * 4 + (threadIdx.x >> 5);
    if (e >= nv || k >= R) return;
    const View v = views[e];
    const int pitch = N + 2;
    const float2 *__restrict__ base = (v.flags & kLinesAreRows) ? prow : pcol;

    // Position on line 0 and per-line step, Q32.32.
    const long long u0 = v.r0 + (long long)k * v.rk;
    const long long q = v.ri;
    // Lines whose sample lies in [-0.5, N - 0.5]: a superset of the valid
    // samples [0, N-1) with half a sample of margin, and every index stays in
    // [-1, N-1] (the pads).  Float error here is < 1e-3 samples.
    const float uf0 = (float)u0 * 2.3283064365386963e-10f;
    const float qf = (float)q * 2.3283064365386963e-10f;
    int lo, hi;
    if (fabsf(qf) < 1e-20f) {
        bool in = uf0 >= -0.5f && uf0 <= (float)N - 0.5f;
        lo = in ? 0 : 1;
        hi = in ? N - 1 : 0;
    } else {
        float t1 = (-0.5f - uf0) / qf, t2 = ((float)N - 0.5f - uf0) / qf;
        float tlo = fmaxf(fminf(t1, t2), 0.f), thi = fminf(fmaxf(t1, t2), (float)(N - 1));
        lo = (int)ceilf(tlo);
        hi = (int)floorf(thi);
    }
    // Exact check of the ends (positions are monotone in i): every sample
    // index used stays in [-1, N-1], i.e. inside the padded line.
    const long long ulo = -(1LL << 32), uhi = (long long)N << 32;
    while (lo <= hi && (u0 + (long long)lo * q < ulo || u0 + (long long)lo * q >= uhi)) ++lo;
    while (hi >= lo && (u0 + (long long)hi * q < ulo || u0 + (long long)hi * q >= uhi)) --hi;

    float acc = 0.f, comp = 0.f;
    if (lo <= hi) {
        long long u = u0 + (long long)lo * q;
        const float2 *__restrict__ line = base + (size_t)lo * pitch + 1;
        int i = lo;
        while (i <= hi) {
            const int iend = min(hi, i + 31);
            float part = 0.f;
#pragma unroll 4
            for (; i <= iend; ++i) {
                const int n = (int)(u >> 32);
                const float w1 = __uint_as_float(((unsigned)u >> 9) | 0x3F800000u);
                const float2 pr = __ldg(line + n);
                part += fmaf(w1, pr.y, pr.x);
                u += q;
                line += pitch;
            }
            kahan_add(acc, comp, part);
        }
    }
    float val = (acc - comp) * v.delta;
    if (RATIO) {
        const float y = y_am[(size_t)v.view * y_ld + k];
        val = (val != 0.f) ? y / val : 0.f;
    }
    out_am[(size_t)v.view * out_ld + k] = val;
}

int launch_radon(const SSPlan &p, const float2 *prow, const float2 *pcol, float *out_am,
                 int out_ld, const float *y_am, int y_ld, cudaStream_t st)
{
    if (p.nv == 0) return RG_OK;
    dim3 grid((p.g.R + 31) / 32, (p.nv + 3) / 4);
    if (y_am)
        k_radon<true><<<grid, 128, 0, st>>>(prow, pcol, p.g.N, p.d_views, p.nv, p.g.R, out_am,
                                            out_ld, y_am, y_ld);
    else
        k_radon<false><<<grid, 128, 0, st>>>(prow, pcol, p.g.N, p.d_views, p.nv, p.g.R, out_am,
                                             out_ld, nullptr, 0);
    RG_CK_LAUNCH("k_radon");
    return RG_OK;
}

// ============================================================================
// Gathers (backprojection / matched adjoint).

constexpr int kTile = 32;    // pixels per tile side
constexpr int kSlots = 32;   // views per staged chunk
constexpr int kRows = 4;     // rows per thread (8 warps x 4 = 32)

struct SlotInfo {
    unsigned base;   // Q9.23 position of the tile origin within the window
    int a;           // Q9.23 step per column
    int b;           // Q9.23 step per row
    int nlo;         // first staged sample index (INT_MIN: empty slot)
};

// Inner loop over the staged views of one chunk for one thread's 4 pixels.
//
// Adjoint weights: with kappa the ray-index position of the pixel's ray,
// k0 = floor(kappa), f = kappa - k0, the rays k0 and k0+1 sample the pixel's
// line at u - m = -p f and p (1 - f); their hat weights are 1 - P f and
// 1 - P (1 - f), clipped at 0 (P = |p| >= 1, so no other ray reaches the
// pixel).  At line positions m = 0 and m = N-1 the Radon drops samples with
// u < 0 and u >= N-1; BORDER applies exactly that rule.
template <int MODE, int WMAX, bool BORDER, typename Acc>
__device__ __forceinline__ void accumulate(Acc (&part)[kRows], const float2 *__restrict__ pairs,
                                           const SlotInfo *slot, const float *slotP,
                                           const int *slotFlags, int nslot, int lane, int warp,
                                           int col, int myrow, int N)
{
    for (int s = 0; s < nslot; ++s) {
        const SlotInfo si = slot[s];
        if (si.nlo == INT_MIN) continue;
        const float2 *__restrict__ pw = pairs + s * WMAX;
        unsigned vpos = si.base + (unsigned)(lane * si.a) + (unsigned)(warp * kRows * si.b);
        if (MODE == 0) {
#pragma unroll
            for (int r = 0; r < kRows; ++r) {
                const float w1 = __uint_as_float((vpos & 0x7FFFFFu) | 0x3F800000u);
                const float2 pr = pw[vpos >> 23];
                part[r] += fmaf(w1, pr.y, pr.x);
                vpos += (unsigned)si.b;
            }
        } else {
            const float P = slotP[s];
            const float c0 = 1.f + P, c1 = 1.f - 2.f * P;
            int fl = 0;
            if (BORDER) fl = slotFlags[s];
            const bool pneg = (fl & kRkNegative) != 0;
#pragma unroll
            for (int r = 0; r < kRows; ++r) {
                const float w1 = __uint_as_float((vpos & 0x7FFFFFu) | 0x3F800000u);
                const float2 pr = pw[vpos >> 23];
                float wa = fmaxf(0.f, fmaf(-P, w1, c0));
                float wb = fmaxf(0.f, fmaf(P, w1, c1));
                if (BORDER) {
                    const int m = (fl & kLinesAreRows) ? col : (myrow + r);
                    const bool f0 = (w1 == 1.0f);
                    if (m == 0) {                       // drop u < 0
                        if (!pneg && !f0) wa = 0.f;
                        if (pneg) wb = 0.f;
                    } else if (m == N - 1) {            // drop u >= N-1
                        if (pneg || f0) wa = 0.f;
                        if (!pneg) wb = 0.f;
                    }
                }
                part[r] += (Acc)fmaf(pr.x, wa, pr.y * wb);
                vpos += (unsigned)si.b;
            }
        }
    }
}

// MODE 0: backprojection; 1: adjoint (FP32 accumulate); 2: adjoint, FP64.
template <int MODE, int WMAX, bool EM>
__global__ __launch_bounds__(256) void k_gather(const float *__restrict__ s_am, int s_ld, int R,
                                                const View *__restrict__ views, int nv, int N,
                                                float scale, float *__restrict__ out,
                                                long long cs, long long ls,
                                                float *__restrict__ em_x,
                                                const float *__restrict__ inv_sens,
                                                int *__restrict__ err)
{
    extern __shared__ float2 pairs[];          // [kSlots][WMAX]
    __shared__ SlotInfo slot[kSlots];
    __shared__ float slotP[kSlots];
    __shared__ int slotFlags[kSlots];
    using Acc = typename std::conditional<MODE == 2, double, float>::type;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int row0 = blockIdx.y * kTile, col0 = blockIdx.x * kTile;
    const int col = col0 + lane;
    const int myrow = row0 + warp * kRows;
    const bool border = row0 == 0 || col0 == 0 || row0 + kTile >= N || col0 + kTile >= N;

    Acc acc[kRows], comp[kRows];
#pragma unroll
    for (int r = 0; r < kRows; ++r) { acc[r] = 0; comp[r] = 0; }

    for (int chunk = 0; chunk < nv; chunk += kSlots) {
        const int nslot = min(kSlots, nv - chunk);
        if (warp == 0) {
            SlotInfo si = {0u, 0, 0, INT_MIN};
            float P = 0.f;
            int flags = 0;
            if (lane < nslot) {
                const View v = views[chunk + lane];
                long long cr, cc, c0;
                if (MODE == 0) { cr = v.brow; cc = v.bcol; c0 = v.b0; }
                else           { cr = v.krow; cc = v.kcol; c0 = v.k0; }
                const long long origin = c0 + (long long)row0 * cr + (long long)col0 * cc;
                const long long dr = 31LL * cr, dc = 31LL * cc;
                const long long mn = origin + min(0LL, dr) + min(0LL, dc);
                const long long mx = origin + max(0LL, dr) + max(0LL, dc);
                const int nlo = (int)(mn >> 32) - 1;
                const int nhi = (int)(mx >> 32) + 1;
                if (nhi - nlo + 1 <= WMAX) {
                    si.nlo = nlo;
                    si.base = (unsigned)((origin - ((long long)nlo << 32)) >> 9);
                    si.a = (int)((cc + 256) >> 9);
                    si.b = (int)((cr + 256) >> 9);
                } else if (err) {
                    atomicOr(err, 1);
                }
                P = v.P;
                flags = v.flags;
            }
            slot[lane] = si;
            slotP[lane] = P;
            slotFlags[lane] = flags;
        }
        __syncthreads();

        // Stage the windows.
        for (int e = threadIdx.x; e < nslot * WMAX; e += 256) {
            const int s = e / WMAX, w = e - s * WMAX;
            const int nlo = slot[s].nlo;
            float2 pr = make_float2(0.f, 0.f);
            if (nlo != INT_MIN) {
                const View &v = views[chunk + s];
                const float *__restrict__ row = s_am + (size_t)v.view * s_ld;
                const int n = nlo + w;
                if (MODE == 0) {
                    if (n >= 0 && n <= R - 2) {
                        const float s0 = __ldg(row + n), s1 = __ldg(row + n + 1);
                        pr = make_pair(s0, s1, true);
                    }
                } else {
                    const float d = v.delta;
                    const float s0 = (n >= 0 && n < R) ? __ldg(row + n) : 0.f;
                    const float s1 = (n + 1 >= 0 && n + 1 < R) ? __ldg(row + n + 1) : 0.f;
                    pr = make_float2(s0 * d, s1 * d);
                }
            }
            pairs[e] = pr;
        }
        __syncthreads();

        // Accumulate.  Border tiles of the adjoint apply the reference's
        // sample validity at positions 0 and N-1 of a line (CTA-uniform branch).
        Acc part[kRows];
#pragma unroll
        for (int r = 0; r < kRows; ++r) part[r] = 0;
        if (MODE != 0 && border)
            accumulate<MODE, WMAX, true, Acc>(part, pairs, slot, slotP, slotFlags, nslot, lane,
                                              warp, col, myrow, N);
        else
            accumulate<MODE, WMAX, false, Acc>(part, pairs, slot, slotP, slotFlags, nslot, lane,
                                               warp, col, myrow, N);
#pragma unroll
        for (int r = 0; r < kRows; ++r) {
            if (MODE == 2) {
                acc[r] += part[r];
            } else {
                float a = acc[r], c = comp[r];
                kahan_add(a, c, (float)part[r]);
                acc[r] = a; comp[r] = c;
            }
        }
        __syncthreads();
    }

    if (col >= N) return;
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
        const int row = myrow + r;
        if (row >= N) break;
        if (MODE == 2) {
            const double sv = (double)acc[r];
            out[(long long)row * cs + (long long)col * ls] = (sv > 0.0) ? (float)(1.0 / sv) : 0.f;
        } else {
            const float val = ((float)acc[r] - (float)comp[r]) * scale;
            if (EM) {
                const size_t idx = (size_t)row * N + col;
                em_x[idx] = em_x[idx] * val * inv_sens[idx];
            } else {
                out[(long long)row * cs + (long long)col * ls] = val;
            }
        }
    }
}

template <int MODE, int WMAX, bool EM>
static int gather_w(const SSPlan &p, const float *s_am, int s_ld, float *out, long long cs,
                    long long ls, float *em_x, const float *inv_sens, int *d_err,
                    cudaStream_t st)
{
    const size_t smem = (size_t)kSlots * WMAX * sizeof(float2);
    const int tiles = (p.g.N + kTile - 1) / kTile;
    dim3 grid(tiles, tiles);
    const float scale = (MODE == 0) ? p.dth : 1.f;
    auto k = k_gather<MODE, WMAX, EM>;
    RG_CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k<<<grid, 256, smem, st>>>(s_am, s_ld, p.g.R, p.d_views, p.nv, p.g.N, scale, out, cs, ls,
                               em_x, inv_sens, d_err);
    RG_CK_LAUNCH("k_gather");
    return RG_OK;
}

template <int MODE, bool EM>
static int gather_mode(const SSPlan &p, int wneed, const float *s_am, int s_ld, float *out,
                       long long cs, long long ls, float *em_x, const float *inv_sens,
                       int *d_err, cudaStream_t st)
{
    if (wneed <= 64) return gather_w<MODE, 64, EM>(p, s_am, s_ld, out, cs, ls, em_x, inv_sens, d_err, st);
    if (wneed <= 128) return gather_w<MODE, 128, EM>(p, s_am, s_ld, out, cs, ls, em_x, inv_sens, d_err, st);
    if (wneed <= 256) return gather_w<MODE, 256, EM>(p, s_am, s_ld, out, cs, ls, em_x, inv_sens, d_err, st);
    if (wneed <= 512) return gather_w<MODE, 512, EM>(p, s_am, s_ld, out, cs, ls, em_x, inv_sens, d_err, st);
    return set_error(RG_EUNSUPPORTED,
                     "gather window of %d samples per 32-pixel tile exceeds 512 "
                     "(image much coarser than the ray spacing)", wneed);
}

int launch_gather(const SSPlan &p, int mode, const float *s_am, int s_ld, float *out,
                  long long cs, long long ls, float *em_x, const float *inv_sens, int *d_err,
                  cudaStream_t st)
{
    if (mode == 0)
        return gather_mode<0, false>(p, p.wmax_bp, s_am, s_ld, out, cs, ls, nullptr, nullptr,
                                     d_err, st);
    if (!p.adj_ok)
        return set_error(RG_EUNSUPPORTED,
                         "matched adjoint needs ray spacing >= pixel spacing along each line "
                         "(nrays <= size for the default extents)");
    if (mode == 1) {
        if (em_x)
            return gather_mode<1, true>(p, p.wmax_adj, s_am, s_ld, out, cs, ls, em_x, inv_sens,
                                        d_err, st);
        return gather_mode<1, false>(p, p.wmax_adj, s_am, s_ld, out, cs, ls, nullptr, nullptr,
                                     d_err, st);
    }
    return gather_mode<2, false>(p, p.wmax_adj, s_am, s_ld, out, cs, ls, nullptr, nullptr, d_err,
                                 st);
}

}  // namespace rg
