// ss_tiles.cuh -- per-tile device bodies of the slant-stack kernels, shared
// by the one-slice launches (slantstack.cu) and the batched persistent
// launches (batch.cu).  The algorithms and their reference semantics are
// described at the top of slantstack.cu.
#pragma once

#include <cooperative_groups.h>

#include <climits>
#include <type_traits>

#include "rg_internal.cuh"

namespace rg {

__device__ __forceinline__ float2 make_pair(float s0, float s1, bool valid)
{
    float d = s1 - s0;
    return valid ? make_float2(s0 - d, d) : make_float2(0.f, 0.f);
}

// One CTA (256 threads) packs the 32 x 32 image tile (bx, by) into both
// orientations.
__device__ __forceinline__ void line_pairs_tile(const float *__restrict__ img, long long cs,
                                                long long ls, int N, float2 *__restrict__ prow,
                                                float2 *__restrict__ pcol, int bx, int by)
{
    __shared__ float t[33][33];
    const int r0 = by * 32, c0 = bx * 32;
    const int pitch = pairs_pitch(N);
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
    // zero pads of the lines this tile starts / ends (entry 0 and entries
    // N + 1 .. pitch - 1)
    if (c0 == 0 && threadIdx.x < 32 && r0 + lane < N) {
        prow[(size_t)(r0 + lane) * pitch] = make_float2(0.f, 0.f);
        for (int e = N + 1; e < pitch; ++e)
            prow[(size_t)(r0 + lane) * pitch + e] = make_float2(0.f, 0.f);
    }
    if (r0 == 0 && threadIdx.x < 32 && c0 + lane < N) {
        pcol[(size_t)(c0 + lane) * pitch] = make_float2(0.f, 0.f);
        for (int e = N + 1; e < pitch; ++e)
            pcol[(size_t)(c0 + lane) * pitch + e] = make_float2(0.f, 0.f);
    }
    __syncthreads();   // t is reused by the next tile of a persistent CTA
}

__device__ __forceinline__ void kahan_add(float &sum, float &c, float x)
{
    float y = x - c;
    float t = sum + y;
    c = (t - sum) - y;
    sum = t;
}

// Lines i (in [0, N-1]) whose sample u0 + i*q lies in [-0.5, N - 0.5]: a
// superset of the valid samples [0, N-1) with half a sample of margin,
// checked exactly at both ends so every index used stays in [-1, N-1].
// (Also called on the host, to estimate the TMA Radon's work per CTA.)
__host__ __device__ __forceinline__ void radon_line_range(long long u0, long long q, int N, int &lo,
                                                 int &hi)
{
    // float error of the estimate is < 1e-3 samples; the ends are then exact
    const float uf0 = (float)u0 * 2.3283064365386963e-10f;
    const float qf = (float)q * 2.3283064365386963e-10f;
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

}

// Radon epilogues: kEpiSum writes the ray sum; kEpiRatio the EM ratio
// y / (A x) (0 where A x == 0); kEpiTransmission b exp(-(A x)), with b read
// from the y argument.
enum { kEpiSum = 0, kEpiRatio = 1, kEpiTransmission = 2 };

__device__ __forceinline__ float radon_epilogue(int epi, float val, const float *y, size_t idx)
{
    if (epi == kEpiRatio) {
        const float yv = y[idx];
        return (val != 0.f) ? yv / val : 0.f;
    }
    if (epi == kEpiTransmission) return y[idx] * expf(-val);
    return val;
}

// UNROLL of the direct Radon walks: the walks are bound by load latency
// (line pairs from L1, L2 or, for batches larger than L2, DRAM), and a
// deeper unroll keeps more independent loads in flight per thread at the
// cost of registers.  Measured on GB300: 8 for one-view walks over few
// CTAs (OSEM subsets of one slice), 16 for two-view walks of the batched
// OSEM.
// One CTA (128 threads) = rays [32 bx, 32 bx + 32) of views [4 by, 4 by + 4).
//
// split > 1: the CTA is rank `rank` of a thread-block cluster of `split`
// CTAs along x that share the rays and views; it walks lines
// [rank N / split, (rank + 1) N / split) only, and rank 0 adds the partial
// sums (in rank order, from distributed shared memory) and writes the
// epilogue.  Splitting the lines multiplies the CTA count of launches too
// small to fill the GPU (one slice's OSEM subset).
template <int EPI, int UNROLL = 8>
__device__ __forceinline__ void radon_tile(const float2 *__restrict__ prow,
                                           const float2 *__restrict__ pcol, int N,
                                           const View *__restrict__ views, int nv, int R,
                                           float *__restrict__ out_am, int out_ld,
                                           const float *__restrict__ y_am, int y_ld, int bx,
                                           int by, int split = 1, int rank = 0)
{
    const int k = bx * 32 + (threadIdx.x & 31);
    const int e = by * 4 + (threadIdx.x >> 5);
    const bool active = e < nv && k < R;
    if (!active && split == 1) return;   // no barrier below: early exit is safe
    const View v = views[active ? e : 0];
    const int pitch = pairs_pitch(N);
    const float2 *__restrict__ base = (v.flags & kLinesAreRows) ? prow : pcol;

    // Position on line 0 and per-line step, Q32.32.
    const long long u0 = v.r0 + (long long)k * v.rk;
    const long long q = v.ri;
    int lo, hi;
    radon_line_range(u0, q, N, lo, hi);
    if (split > 1) {
        lo = max(lo, (int)((long long)N * rank / split));
        hi = min(hi, (int)((long long)N * (rank + 1) / split) - 1);
        if (!active) { lo = 1; hi = 0; }
    }
    float acc = 0.f, comp = 0.f;
    if (lo <= hi) {
        long long u = u0 + (long long)lo * q;
        const float2 *__restrict__ line = base + (size_t)lo * pitch + 1;
        int i = lo;
        while (i <= hi) {
            const int iend = min(hi, i + 31);
            float part = 0.f;
#pragma unroll UNROLL
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
    if (split > 1) {
        namespace cg = cooperative_groups;
        cg::cluster_group cl = cg::this_cluster();
        __shared__ float red[128];
        red[threadIdx.x] = acc - comp;
        cl.sync();
        if (rank == 0 && active) {
            float sum = 0.f;
            for (int src = 0; src < split; ++src)
                sum += cl.map_shared_rank(red, src)[threadIdx.x];
            out_am[(size_t)v.view * out_ld + k] =
                radon_epilogue(EPI, sum * v.delta, y_am, (size_t)v.view * y_ld + k);
        }
        cl.sync();    // no CTA leaves while rank 0 still reads its partials
        return;
    }
    const float val = (acc - comp) * v.delta;
    out_am[(size_t)v.view * out_ld + k] = radon_epilogue(EPI, val, y_am, (size_t)v.view * y_ld + k);
}

// Two views per thread: a CTA (128 threads) covers rays [32 bx, 32 bx + 32) of
// views [8 by, 8 by + 8); warp w carries views 8 by + 2w and 8 by + 2w + 1.
// The two views of a thread are adjacent, so their samples on each line lie
// a few positions apart: the two independent load streams share L1 lines
// and double the loads in flight per thread.  The loop runs over the union
// of both views' line ranges; a sample index outside a view's own range is
// clamped (one unsigned min) onto the line's zero pad at N+1, so it adds 0
// and never leaves the padded line.
template <int EPI, int UNROLL = 4>
__device__ __forceinline__ void radon_tile2(const float2 *__restrict__ prow,
                                            const float2 *__restrict__ pcol, int N,
                                            const View *__restrict__ views, int nv, int R,
                                            float *__restrict__ out_am, int out_ld,
                                            const float *__restrict__ y_am, int y_ld, int bx,
                                            int by)
{
    const int k = bx * 32 + (threadIdx.x & 31);
    const int e0 = by * 8 + 2 * (threadIdx.x >> 5);
    if (e0 >= nv || k >= R) return;   // no barrier below: early exit is safe
    const bool two = e0 + 1 < nv;
    const View va = views[e0];
    const View vb = two ? views[e0 + 1] : va;
    const unsigned pitch = (unsigned)pairs_pitch(N);
    const float2 *__restrict__ ba = (va.flags & kLinesAreRows) ? prow : pcol;
    const float2 *__restrict__ bb = (vb.flags & kLinesAreRows) ? prow : pcol;
    const long long ua0 = va.r0 + (long long)k * va.rk, ub0 = vb.r0 + (long long)k * vb.rk;
    int loa, hia, lob, hib;
    radon_line_range(ua0, va.ri, N, loa, hia);
    radon_line_range(ub0, vb.ri, N, lob, hib);
    const int lo = min(loa, lob), hi = max(hia, hib);
    float acca = 0.f, compa = 0.f, accb = 0.f, compb = 0.f;
    if (lo <= hi) {
        long long ua = ua0 + (long long)lo * va.ri, ub = ub0 + (long long)lo * vb.ri;
        unsigned off = (unsigned)lo * pitch;
        const unsigned pad = (unsigned)(N + 1);
        int i = lo;
        while (i <= hi) {
            const int iend = min(hi, i + 31);
            float pa = 0.f, pb = 0.f;
#pragma unroll UNROLL
            for (; i <= iend; ++i) {
                const unsigned ia = min((unsigned)((int)(ua >> 32) + 1), pad);
                const unsigned ib = min((unsigned)((int)(ub >> 32) + 1), pad);
                const float2 qa = __ldg(ba + off + ia);
                const float2 qb = __ldg(bb + off + ib);
                pa += fmaf(__uint_as_float(((unsigned)ua >> 9) | 0x3F800000u), qa.y, qa.x);
                pb += fmaf(__uint_as_float(((unsigned)ub >> 9) | 0x3F800000u), qb.y, qb.x);
                ua += va.ri;
                ub += vb.ri;
                off += pitch;
            }
            kahan_add(acca, compa, pa);
            kahan_add(accb, compb, pb);
        }
    }
    const float vala = (acca - compa) * va.delta, valb = (accb - compb) * vb.delta;
    out_am[(size_t)va.view * out_ld + k] =
        radon_epilogue(EPI, vala, y_am, (size_t)va.view * y_ld + k);
    if (two)
        out_am[(size_t)vb.view * out_ld + k] =
            radon_epilogue(EPI, valb, y_am, (size_t)vb.view * y_ld + k);
}

// ============================================================================
// Gathers (backprojection / matched adjoint).

constexpr int kTile = 32;    // pixel columns per tile (one warp lane each)
constexpr int kSlots = 32;   // views per staged chunk
constexpr int kWarps = 8;    // 256 threads; warp w owns rows [w*ROWS, (w+1)*ROWS) of the tile

struct SlotInfo {
    unsigned base;   // Q9.23 position of the tile origin within the window
    int a;           // Q9.23 step per column
    int b;           // Q9.23 step per row
    int nlo;         // first staged sample index (INT_MIN: empty slot)
};

// Position weight 1 + w from the low 23 bits of a Q9.23 position.
__device__ __forceinline__ float frac_plus_one(unsigned v)
{
    return __uint_as_float((v & 0x7FFFFFu) | 0x3F800000u);
}

// a * b + c, clamped to [0, 1] by the FMA itself (fma.rn.sat).
__device__ __forceinline__ float fma_sat(float a, float b, float c)
{
    float d;
    asm("fma.rn.sat.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Inner loop over the staged views of one chunk for one thread's ROWS pixels.
//
// Backprojection: the staged pair (s - d, d) at the floor index gives the
// linear interpolation (s - d) + (1 + w) d.
//
// Adjoint weights: with kappa the ray-index position of the pixel's ray,
// k0 = floor(kappa), f = kappa - k0, the rays k0 and k0+1 sample the pixel's
// line at u - m = -p f and p (1 - f); their hat weights are 1 - P f and
// 1 - P (1 - f) clipped to [0, 1] (P = |p| >= 1, so no other ray reaches
// the pixel); with w1 = 1 + f they are sat(-P w1 + 1 + P) and
// sat(P w1 + 1 - 2P).  At line positions m = 0 and m = N-1 the Radon drops
// samples with u < 0 and u >= N-1; BORDER applies exactly that rule.
// One staged pair from the 32-bit shared address base + idx * pair_bytes.
// pair_bytes (== 8) arrives as a kernel argument, so the address is an
// integer multiply-add on the FMA pipe rather than a shift + LEA on the
// integer ALU pipe, which the inner loops keep busy with the weight bits.
// RG_LDS_ADDR_IMAD=0 at compile time selects plain indexing instead.
#ifndef RG_LDS_ADDR_IMAD
#define RG_LDS_ADDR_IMAD 1
#endif
__device__ __forceinline__ float2 lds_pair(unsigned base, unsigned idx, unsigned pair_bytes)
{
    float2 v;
#if RG_LDS_ADDR_IMAD
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];"
                 : "=f"(v.x), "=f"(v.y) : "r"(idx * pair_bytes + base));
#else
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];"
                 : "=f"(v.x), "=f"(v.y) : "r"((idx << 3) + base));
#endif
    return v;
}

template <int MODE, int WMAX, int ROWS, bool BORDER>
__device__ __forceinline__ void accumulate(float (&part)[ROWS], const float2 *__restrict__ pairs,
                                           const SlotInfo *slot, const float *slotP,
                                           const int *slotFlags, int nslot, int lane, int warp,
                                           int col, int myrow, int N, unsigned pair_bytes)
{
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(pairs);
    for (int s = 0; s < nslot; ++s) {
        const SlotInfo si = slot[s];
        if (si.nlo == INT_MIN) continue;
        const unsigned pw = sbase + (unsigned)(s * WMAX) * pair_bytes;
        unsigned vpos = si.base + (unsigned)(lane * si.a) + (unsigned)(warp * ROWS * si.b);
        if (MODE == 0) {
#pragma unroll
            for (int r = 0; r < ROWS; ++r) {
                const float2 pr = lds_pair(pw, vpos >> 23, pair_bytes);
                part[r] += fmaf(frac_plus_one(vpos), pr.y, pr.x);
                vpos += (unsigned)si.b;
            }
        } else {
            const float P = slotP[s];
            const float c0 = 1.f + P, c1 = 1.f - 2.f * P;
            int fl = 0;
            if (BORDER) fl = slotFlags[s];
            const bool pneg = (fl & kRkNegative) != 0;
#pragma unroll
            for (int r = 0; r < ROWS; ++r) {
                const float w1 = frac_plus_one(vpos);
                const float2 pr = lds_pair(pw, vpos >> 23, pair_bytes);
                float wa = fma_sat(-P, w1, c0);
                float wb = fma_sat(P, w1, c1);
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
                part[r] = fmaf(pr.x, wa, part[r]);
                part[r] = fmaf(pr.y, wb, part[r]);
                vpos += (unsigned)si.b;
            }
        }
    }
}

template <int OFF>
__device__ __forceinline__ float2 lds_pair_at(unsigned addr)
{
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2+%3];"
                 : "=f"(v.x), "=f"(v.y)
                 : "r"(addr), "n"(OFF));
    return v;
}

constexpr int kTtLines = 32;                  // lines per tile
constexpr int kTtWin = 160;                   // owned entries per tile row
constexpr int kTtPad = 48;                    // zero entries on each side
constexpr int kTtRow = kTtWin + 2 * kTtPad;   // smem row stride (entries): 2 KB

// ROW: smem row stride of the staged tile in entries (>= WIN + 2 PAD);
// LINES: lines of the tile.
template <int ROW, int LINES, int R0>
__device__ __forceinline__ void tt_walk(unsigned sb, unsigned &L, unsigned dq, unsigned pb,
                                        float &part)
{
    // pb (== 8) is a runtime value: the address is one multiply-add on the
    // FMA pipe (the integer pipe carries the position and weight bits)
    if constexpr (R0 < LINES) {
        const float2 pr = lds_pair_at<R0 * ROW * 8>((L >> 23) * pb + sb);
        part += fmaf(frac_plus_one(L), pr.y, pr.x);
        L += dq;
        tt_walk<ROW, LINES, R0 + 1>(sb, L, dq, pb, part);
    }
}

// The views loop of the tile-driven Radon (radon_tma.cu, k_radon_tiles, and
// the batched OSEM): the tile of kTtLines lines x kTtRow entries is staged
// at shared address sbase (entry p0 - kTtPad at index 0, zero pads around
// the window [p0, p0 + kTtWin)).  Views are taken in batches of up to 256:
// thread t finds view t's rays that cross the window on lines
// [i0, i0 + kTtLines) (FP32, two rays of margin; the exact int64 check below
// drops rays that do not cross), the batch's 32-ray chunks are numbered by
// a prefix sum, and each warp takes a contiguous range of them, so the work
// spreads evenly whatever the number of views and rays.  A lane walks its ray
// across the tile's lines and adds partial * Delta to out_am[view][ray].
// Must be reached by every thread of the CTA (it has barriers).
constexpr int kTtBatch = 256;

template <int ROW, int LINES = kTtLines, int PAD = kTtPad>
__device__ __forceinline__ void tt_views(unsigned sbase, int p0, int i0,
                                         const TtView *__restrict__ tv, int nvo, int R,
                                         float *__restrict__ out_am, int out_ld,
                                         int *__restrict__ err, unsigned pb)
{
    __shared__ int s_klo[kTtBatch], s_off[kTtBatch + 1], s_wsum[kTtBatch / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int i1 = i0 + LINES - 1;
    const float a = p0 - 1.0f, b = p0 - 1.0f + kTtWin;     // window samples [a, b)
    const long long base_q = (long long)(p0 - PAD - 1) << 32;      // smem index 0
    const long long lo_q = 1LL << 32, hi_q = (long long)(kTtWin + 2 * PAD - 1) << 32;
    for (int v0 = 0; v0 < nvo; v0 += kTtBatch) {
        const int nb = min(kTtBatch, nvo - v0);
        int nch = 0;
        if ((int)threadIdx.x < nb) {
            const TtView v = tv[v0 + threadIdx.x];
            const float rk = (float)v.rk * 2.3283064365386963e-10f;
            const float c0 = ((float)v.r0 + (float)i0 * (float)v.ri) * 2.3283064365386963e-10f;
            const float c1 = ((float)v.r0 + (float)i1 * (float)v.ri) * 2.3283064365386963e-10f;
            float ka = (a - fmaxf(c0, c1)) / rk, kb = (b - fminf(c0, c1)) / rk;
            if (ka > kb) { const float t = ka; ka = kb; kb = t; }
            const int klo = max(0, (int)floorf(fminf(fmaxf(ka, -2.f), R + 2.f)) - 2);
            const int khi = min(R - 1, (int)ceilf(fmaxf(fminf(kb, R + 2.f), -2.f)) + 2);
            s_klo[threadIdx.x] = klo;
            nch = khi >= klo ? (khi - klo + 32) >> 5 : 0;
        }
        // prefix sum of the chunk counts over the CTA (blockDim.x == kTtBatch):
        // within each warp by shuffles, then over the warps' totals;
        // s_off[t] = chunks of views < t
        int acc = nch;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, acc, o);
            if (lane >= o) acc += y;
        }
        if (lane == 31) s_wsum[warp] = acc;
        __syncthreads();
        for (int w = 0; w < warp; ++w) acc += s_wsum[w];
        s_off[threadIdx.x + 1] = acc;
        if (threadIdx.x == 0) s_off[0] = 0;
        __syncthreads();
        const int nchunks = s_off[nb];
        // Warp w takes the contiguous chunks [g0, g1): consecutive chunks
        // mostly belong to one view, whose constants it keeps in registers
        // and reloads only when the view changes.
        const int per = (nchunks + nw - 1) / nw;
        const int g0 = min(nchunks, warp * per), g1 = min(nchunks, g0 + per);
        int t = -1;                                     // view of the loaded constants
        long long ub = 0, vrk = 0, vspan = 0;
        float vdelta = 0.f;
        unsigned dq = 0;
        int vview = 0, kl = 0, off = 0;
        for (int g = g0; g < g1; ++g) {
            int tn = t < 0 ? 0 : t;
            if (t < 0) {                                // first view: binary search
                int lo = 0, hi = nb - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (s_off[mid] <= g) lo = mid; else hi = mid - 1;
                }
                tn = lo;
            }
            while (s_off[tn + 1] <= g) ++tn;            // chunks grow, so t only advances
            if (tn != t) {
                t = tn;
                const TtView v = tv[v0 + t];
                kl = s_klo[t];
                off = s_off[t];
                vrk = v.rk;
                vspan = (long long)(LINES - 1) * v.ri;
                dq = (unsigned)((v.ri + 256) >> 9);
                ub = v.r0 + (long long)i0 * v.ri - base_q;
                vdelta = v.delta;
                vview = v.view;
            }
            const int k = kl + ((g - off) << 5) + lane;
            if (k >= R) continue;
            const long long u = ub + (long long)k * vrk;
            const long long ue = u + vspan;
            // a crossing ray stays inside the pads (one entry of slack for the
            // Q9.23 stepping); others are margin rays, or (flagged) the plan's
            // pad check failed: they add nothing here
            if (u < lo_q || u >= hi_q || ue < lo_q || ue >= hi_q) {
                if (err && u >= (long long)PAD << 32 && u < (long long)(PAD + kTtWin) << 32)
                    atomicOr(err, 1);
                continue;
            }
            unsigned L = (unsigned)(u >> 9);
            float part = 0.f;
            tt_walk<ROW, LINES, 0>(sbase, L, dq, pb, part);
            if (part != 0.f) atomicAdd(out_am + (size_t)vview * out_ld + k, part * vdelta);
        }
        __syncthreads();                                // s_klo / s_off reused
    }
}

// Edge pixels e0 .. e0 + 31 (of 4N - 4: rows 0 and N-1, then columns 0 and
// N-1) of the matched adjoint (MODE 1, optionally with the EM update) or of
// its FP64-accumulated sensitivity (MODE 2), computed by one CTA of WARPS
// warps.  The image's first and last rows and columns are the only pixels
// where the Radon's validity rules at line positions 0 and N-1 apply; the
// gathers leave them out (edge_fixup) and run the rule-free interior path
// on every tile.  Lane l takes pixel e0 + l, and warp w the views
// [w nv / WARPS, (w + 1) nv / WARPS): a warp reads each view's constants once for
// its 32 pixels (the same address in every lane), and neighbouring edge
// pixels read neighbouring sinogram samples.  Each lane sums its views with
// the hat weights and rules of the border path of `accumulate` (Kahan-
// compensated FP32, or FP64 for MODE 2), and the warps' sums meet in
// shared memory in warp order.  One slice's edges make few groups (128 at
// 1024^2), so its kernel splits the views over 32 warps; the batch, with
// many slices, over 8.
template <int MODE, bool EM, int WARPS>
__device__ __forceinline__ void adjoint_edge_group(const float *__restrict__ s_am, int s_ld, int R,
                                                   const View *__restrict__ views, int nv, int N,
                                                   int e0, float *__restrict__ out, long long cs,
                                                   long long ls, float *__restrict__ em_x,
                                                   const float *__restrict__ inv_sens)
{
    __shared__ float red[WARPS][32];
    __shared__ double red64[MODE == 2 ? WARPS : 1][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int e = e0 + lane;
    const bool live = e < 4 * N - 4;
    int row = 0, col = 0;
    if (!live) { row = 0; col = 0; }
    else if (e < N) { row = 0; col = e; }
    else if (e < 2 * N) { row = N - 1; col = e - N; }
    else if (e < 3 * N - 2) { row = e - 2 * N + 1; col = 0; }
    else { row = e - (3 * N - 2) + 1; col = N - 1; }
    float acc = 0.f, comp = 0.f;
    double acc64 = 0.0;
    const int vb = (int)((long long)nv * warp / WARPS);
    const int ve = (int)((long long)nv * (warp + 1) / WARPS);
    // unrolled so that several views' loads are in flight per lane
#pragma unroll 4
    for (int j = vb; j < ve; ++j) {
        const View &v = views[j];
        const long long kap = v.k0 + (long long)row * v.krow + (long long)col * v.kcol;
        const int k = (int)(kap >> 32);
        const float w1 = frac_plus_one((unsigned)kap >> 9);
        const float P = v.P;
        float wa = fma_sat(-P, w1, 1.f + P);
        float wb = fma_sat(P, w1, 1.f - 2.f * P);
        const bool pneg = (v.flags & kRkNegative) != 0;
        const int m = (v.flags & kLinesAreRows) ? col : row;
        const bool f0 = (w1 == 1.0f);
        if (m == 0) {                       // drop u < 0
            if (!pneg && !f0) wa = 0.f;
            if (pneg) wb = 0.f;
        } else if (m == N - 1) {            // drop u >= N-1
            if (pneg || f0) wa = 0.f;
            if (!pneg) wb = 0.f;
        }
        const float *__restrict__ srow = s_am + (size_t)v.view * s_ld;
        const float s0 = (k >= 0 && k < R) ? __ldg(srow + k) * v.delta : 0.f;
        const float s1 = (k + 1 >= 0 && k + 1 < R) ? __ldg(srow + k + 1) * v.delta : 0.f;
        const float term = fmaf(s1, wb, s0 * wa);
        if (MODE == 2) acc64 += (double)term;
        else kahan_add(acc, comp, term);
    }
    if (MODE == 2) red64[warp][lane] = acc64;
    else red[warp][lane] = acc - comp;
    __syncthreads();
    if (warp != 0 || !live) return;
    if (MODE == 2) {
        double sum = 0.0;
        for (int w = 0; w < WARPS; ++w) sum += red64[w][lane];
        out[(long long)row * cs + (long long)col * ls] = (sum > 0.0) ? (float)(1.0 / sum) : 0.f;
        return;
    }
    float sum = 0.f;
    for (int w = 0; w < WARPS; ++w) sum += red[w][lane];
    if (EM) {
        const size_t idx = (size_t)row * N + col;
        em_x[idx] = em_x[idx] * sum * inv_sens[idx];
    } else {
        out[(long long)row * cs + (long long)col * ls] = sum;
    }
}

// Final value of pixel (row, col) of a gather: stored, or (EM) folded into
// the multiplicative update x <- x * val * inv_sens.
template <int MODE, bool EM>
__device__ __forceinline__ void gather_store(float val, int row, int col, int N,
                                             float *__restrict__ out, long long cs, long long ls,
                                             float *__restrict__ em_x,
                                             const float *__restrict__ inv_sens)
{
    if (EM) {
        const size_t idx = (size_t)row * N + col;
        em_x[idx] = em_x[idx] * val * inv_sens[idx];
    } else {
        out[(long long)row * cs + (long long)col * ls] = val;
    }
}

// MODE 0: backprojection; 1: adjoint (FP32 accumulate); 2: adjoint, FP64.
// One CTA (256 threads) = the tile of 32 columns x 8*ROWS rows at tile
// coordinates (tx, ty); `pairs` is kSlots * WMAX float2 of shared memory.
//
// split > 1 (MODE 0 and 1; the CTA is rank `rank` of a thread-block cluster
// of `split` CTAs along x that share the tile): this CTA sums views
// [rank nv / split, (rank + 1) nv / split) only.  The partial sums meet in
// distributed shared memory and each rank finishes ROWS / split of the rows,
// adding the partials in rank order (deterministic).  Splitting the views
// of every tile over a cluster multiplies the CTA count, so the last wave of
// a grid of few large tiles no longer leaves most SMs idle.
//
// KAHAN (MODE 0 and 1): FP32 partial sums per chunk of kSlots views, added
// across chunks with Kahan compensation (3 ROWS accumulator registers);
// without it the views' terms are summed straight into ROWS FP32
// accumulators, for callers whose view count is small (OSEM subsets of the
// batch: at most a few chunks), where the registers buy occupancy.
template <int MODE, int WMAX, int ROWS, bool EM, bool KAHAN = true>
__device__ __forceinline__ void gather_tile(const float *__restrict__ s_am, int s_ld, int R,
                                            const View *__restrict__ views, int nv, int N,
                                            float scale, float *__restrict__ out, long long cs,
                                            long long ls, float *__restrict__ em_x,
                                            const float *__restrict__ inv_sens,
                                            int *__restrict__ err, int tx, int ty,
                                            float2 *__restrict__ pairs, unsigned pair_bytes,
                                            int split = 1, int rank = 0, bool edge_fixup = false)
{
    constexpr int TH = kWarps * ROWS;          // tile height
    __shared__ SlotInfo slot[kSlots];
    __shared__ int slotW[kSlots];
    __shared__ int slotView[kSlots];
    __shared__ float slotDelta[kSlots];
    __shared__ float slotP[kSlots];
    __shared__ int slotFlags[kSlots];
    using Acc = typename std::conditional<MODE == 2, double, float>::type;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int row0 = ty * TH, col0 = tx * kTile;
    const int col = col0 + lane;
    const int myrow = row0 + warp * ROWS;
    // edge_fixup (adjoint modes): every tile takes the interior path and the
    // image's edge pixels (row or column 0 or N-1, the only pixels where the
    // position-0 / N-1 validity rules apply) are left to the edge kernels,
    // which compute them with the rules; otherwise border tiles apply the
    // rules inline.
    const bool border = !edge_fixup &&
                        (row0 == 0 || col0 == 0 || row0 + TH >= N || col0 + kTile >= N);

    Acc acc[ROWS], comp[ROWS];
#pragma unroll
    for (int r = 0; r < ROWS; ++r) { acc[r] = 0; comp[r] = 0; }

    const int vbeg = (int)((long long)nv * rank / split);
    const int vend = (int)((long long)nv * (rank + 1) / split);
    for (int chunk = vbeg; chunk < vend; chunk += kSlots) {
        const int nslot = min(kSlots, vend - chunk);
        if (warp == 0) {
            SlotInfo si = {0u, 0, 0, INT_MIN};
            int W = 0, view = 0, flags = 0;
            float P = 0.f, delta = 0.f;
            if (lane < nslot) {
                const View &v = views[chunk + lane];
                long long cr, cc, c0;
                if (MODE == 0) { cr = v.brow; cc = v.bcol; c0 = v.b0; }
                else           { cr = v.krow; cc = v.kcol; c0 = v.k0; }
                const long long origin = c0 + (long long)row0 * cr + (long long)col0 * cc;
                const long long dr = (long long)(TH - 1) * cr, dc = (long long)(kTile - 1) * cc;
                const long long mn = origin + min(0LL, dr) + min(0LL, dc);
                const long long mx = origin + max(0LL, dr) + max(0LL, dc);
                const int nlo = (int)(mn >> 32) - 1;
                const int nhi = (int)(mx >> 32) + 1;
                if (nhi - nlo + 1 <= WMAX) {
                    si.nlo = nlo;
                    si.base = (unsigned)((origin - ((long long)nlo << 32)) >> 9);
                    si.a = (int)((cc + 256) >> 9);
                    si.b = (int)((cr + 256) >> 9);
                    W = nhi - nlo + 1;
                } else if (err) {
                    atomicOr(err, 1);
                }
                view = v.view;
                delta = v.delta;
                P = v.P;
                flags = v.flags;
            }
            slot[lane] = si;
            slotW[lane] = W;
            slotView[lane] = view;
            slotDelta[lane] = delta;
            slotP[lane] = P;
            slotFlags[lane] = flags;
        }
        __syncthreads();

        // Stage each view's window (warp w stages slots w, w + 8, ...).
        for (int s = warp; s < nslot; s += kWarps) {
            const int nlo = slot[s].nlo, W = slotW[s];
            const float *__restrict__ row = s_am + (size_t)slotView[s] * s_ld;
            const float d = slotDelta[s];
            for (int e = lane; e < W; e += 32) {
                const int n = nlo + e;
                float2 pr = make_float2(0.f, 0.f);
                if (MODE == 0) {
                    if (n >= 0 && n <= R - 2) pr = make_pair(__ldg(row + n), __ldg(row + n + 1), true);
                } else {
                    const float s0 = (n >= 0 && n < R) ? __ldg(row + n) : 0.f;
                    const float s1 = (n + 1 >= 0 && n + 1 < R) ? __ldg(row + n + 1) : 0.f;
                    pr = make_float2(s0 * d, s1 * d);
                }
                pairs[s * WMAX + e] = pr;
            }
        }
        __syncthreads();

        // Accumulate.  Border tiles of the adjoint apply the reference's
        // sample validity at positions 0 and N-1 of a line (CTA-uniform branch).
        // FP32 partial sums over the chunk (<= 32 views); across chunks they
        // are added with Kahan compensation (FP32) or in FP64 (MODE 2).
        if constexpr (MODE != 2 && !KAHAN) {
            if (MODE != 0 && border)
                accumulate<MODE, WMAX, ROWS, true>(acc, pairs, slot, slotP, slotFlags, nslot,
                                                   lane, warp, col, myrow, N, pair_bytes);
            else
                accumulate<MODE, WMAX, ROWS, false>(acc, pairs, slot, slotP, slotFlags, nslot,
                                                    lane, warp, col, myrow, N, pair_bytes);
        } else {
            float part[ROWS];
#pragma unroll
            for (int r = 0; r < ROWS; ++r) part[r] = 0.f;
            if (MODE != 0 && border)
                accumulate<MODE, WMAX, ROWS, true>(part, pairs, slot, slotP, slotFlags, nslot,
                                                   lane, warp, col, myrow, N, pair_bytes);
            else
                accumulate<MODE, WMAX, ROWS, false>(part, pairs, slot, slotP, slotFlags, nslot,
                                                    lane, warp, col, myrow, N, pair_bytes);
#pragma unroll
            for (int r = 0; r < ROWS; ++r) {
                if (MODE == 2) {
                    acc[r] += (double)part[r];
                } else {
                    float a = acc[r], c = comp[r];
                    kahan_add(a, c, part[r]);
                    acc[r] = a; comp[r] = c;
                }
            }
        }
        __syncthreads();
    }

    if (MODE != 2 && split > 1) {
        // The last chunk ended with a barrier: the staging area is free.
        namespace cg = cooperative_groups;
        cg::cluster_group cl = cg::this_cluster();
        float *red = reinterpret_cast<float *>(pairs);    // [ROWS][256]
#pragma unroll
        for (int r = 0; r < ROWS; ++r)
            red[r * 256 + threadIdx.x] = (float)acc[r] - (float)comp[r];
        cl.sync();
        const int per = ROWS / split;
        for (int q = 0; q < per; ++q) {
            const int r = rank * per + q;
            float sum = 0.f;
            for (int src = 0; src < split; ++src)
                sum += cl.map_shared_rank(red, src)[r * 256 + threadIdx.x];
            const int row = myrow + r;
            const bool edge = edge_fixup && (row == 0 || col == 0 || row == N - 1 || col == N - 1);
            if (row < N && col < N && !edge)
                gather_store<MODE, EM>(sum * scale, row, col, N, out, cs, ls, em_x, inv_sens);
        }
        cl.sync();    // no CTA leaves while a peer still reads its partials
        return;
    }
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
        const int row = myrow + r;
        if (row >= N || col >= N) break;
        if (edge_fixup && (row == 0 || col == 0 || row == N - 1 || col == N - 1)) continue;
        if (MODE == 2) {
            const double sv = (double)acc[r];
            out[(long long)row * cs + (long long)col * ls] = (sv > 0.0) ? (float)(1.0 / sv) : 0.f;
        } else {
            gather_store<MODE, EM>(((float)acc[r] - (float)comp[r]) * scale, row, col, N, out, cs,
                                   ls, em_x, inv_sens);
        }
    }
}

// The matched adjoint with the EM update for the tile (tx, ty) and its
// half-turn mirror, for plans with mirror_ok (image and detector centred on
// 0).  Pixel (r, c) at ray position kappa = k + f of a view and pixel
// (N-1-r, N-1-c) at (R-1) - kappa = (R-2-k) + (1-f) of the same view: the
// mirror's hat weights are the primary's swapped,
//     primary: s[k] w_a + s[k+1] w_b,   mirror: s[R-2-k] w_b + s[R-1-k] w_a,
// so one position, one pair of weights and one 128-bit load of the quad
// {s[k], s[k+1], s[R-2-k], s[R-1-k]} (times the view's Delta) serve both.
// (The hat weights are continuous where a ray leaves the detector, so this
// holds at exact ties too; the backprojection's half-open validity range
// is not symmetric there, so it keeps gather_tile.)  Unlike the
// quarter-turn pairing it needs no partner view: every view of an OSEM
// subset pairs with itself.  One CTA sums all views for both tiles, so
// every pixel's sum is complete here and the update x <- x * sum * inv is
// applied in this epilogue.  The mirror tile must be another tile of the
// grid (N a multiple of 2 * 8 * ROWS and of 64); edge pixels are left to
// adjoint_edge_group.  Windows are staged in chunks of kSlots / 2 views of
// WMAX quads, the same shared memory as gather_tile's pairs.
//
// EM: x <- x * sum * inv for both pixels (the sums are whole); else the sums
// are stored to out.  split > 1: the CTA is rank `rank` of a cluster of
// `split` CTAs sharing the tile pair; it sums views [rank nv / split,
// (rank + 1) nv / split), the partials meet in distributed shared memory
// (`quads` must then hold 2 ROWS x 256 floats) and each rank finishes
// ROWS / split of the rows of both tiles, adding the ranks in order.
template <int WMAX, int ROWS, bool EM>
__device__ __forceinline__ void gather_tile_mirror(const float *__restrict__ s_am, int s_ld, int R,
                                                   const View *__restrict__ views, int nv, int N,
                                                   float *__restrict__ out, long long cs,
                                                   long long ls, float *__restrict__ em_x,
                                                   const float *__restrict__ inv_sens,
                                                   int *__restrict__ err, int tx, int ty,
                                                   float4 *__restrict__ quads, unsigned quad_bytes,
                                                   int split = 1, int rank = 0)
{
    constexpr int TH = kWarps * ROWS;
    constexpr int kMSlots = kSlots / 2;
    __shared__ SlotInfo slot[kMSlots];
    __shared__ int slotW[kMSlots];
    __shared__ int slotView[kMSlots];
    __shared__ float slotDelta[kMSlots];
    __shared__ float slotP[kMSlots];

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int row0 = ty * TH, col0 = tx * kTile;
    const int col = col0 + lane;
    const int myrow = row0 + warp * ROWS;
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(quads);

    float accP[ROWS], accM[ROWS];
#pragma unroll
    for (int r = 0; r < ROWS; ++r) { accP[r] = 0.f; accM[r] = 0.f; }

    const int vbeg = (int)((long long)nv * rank / split);
    const int vend = (int)((long long)nv * (rank + 1) / split);
    for (int chunk = vbeg; chunk < vend; chunk += kMSlots) {
        const int nslot = min(kMSlots, vend - chunk);
        if (warp == 0 && lane < kMSlots) {
            SlotInfo si = {0u, 0, 0, INT_MIN};
            int W = 0, view = 0;
            float P = 0.f, delta = 0.f;
            if (lane < nslot) {
                const View &v = views[chunk + lane];
                const long long cr = v.krow, cc = v.kcol;
                const long long origin = v.k0 + (long long)row0 * cr + (long long)col0 * cc;
                const long long dr = (long long)(TH - 1) * cr, dc = (long long)(kTile - 1) * cc;
                const long long mn = origin + min(0LL, dr) + min(0LL, dc);
                const long long mx = origin + max(0LL, dr) + max(0LL, dc);
                const int nlo = (int)(mn >> 32) - 1;
                const int nhi = (int)(mx >> 32) + 1;
                if (nhi - nlo + 1 <= WMAX) {
                    si.nlo = nlo;
                    si.base = (unsigned)((origin - ((long long)nlo << 32)) >> 9);
                    si.a = (int)((cc + 256) >> 9);
                    si.b = (int)((cr + 256) >> 9);
                    W = nhi - nlo + 1;
                } else if (err) {
                    atomicOr(err, 1);
                }
                view = v.view;
                delta = v.delta;
                P = v.P;
            }
            slot[lane] = si;
            slotW[lane] = W;
            slotView[lane] = view;
            slotDelta[lane] = delta;
            slotP[lane] = P;
        }
        __syncthreads();

        // Stage each view's quads: entry e holds samples n, n + 1 and their
        // mirrors R-2-n, R-1-n (n = nlo + e), zero outside the row.
        for (int s = warp; s < nslot; s += kWarps) {
            const int nlo = slot[s].nlo, W = slotW[s];
            const float *__restrict__ row = s_am + (size_t)slotView[s] * s_ld;
            const float d = slotDelta[s];
            for (int e = lane; e < W; e += 32) {
                const int n = nlo + e, m = R - 2 - n;
                const float v0 = (n >= 0 && n < R) ? __ldg(row + n) * d : 0.f;
                const float v1 = (n + 1 >= 0 && n + 1 < R) ? __ldg(row + n + 1) * d : 0.f;
                const float u0 = (m >= 0 && m < R) ? __ldg(row + m) * d : 0.f;
                const float u1 = (m + 1 >= 0 && m + 1 < R) ? __ldg(row + m + 1) * d : 0.f;
                quads[s * WMAX + e] = make_float4(v0, v1, u0, u1);
            }
        }
        __syncthreads();

        for (int s = 0; s < nslot; ++s) {
            const SlotInfo si = slot[s];
            if (si.nlo == INT_MIN) continue;
            const unsigned pw = sbase + (unsigned)(s * WMAX) * quad_bytes;
            unsigned vpos = si.base + (unsigned)(lane * si.a) + (unsigned)(warp * ROWS * si.b);
            const float P = slotP[s];
            const float c0 = 1.f + P, c1 = 1.f - 2.f * P;
#pragma unroll
            for (int r = 0; r < ROWS; ++r) {
                const unsigned addr = (vpos >> 23) * quad_bytes + pw;
                float a, b, c, d;
                asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                             : "=f"(a), "=f"(b), "=f"(c), "=f"(d) : "r"(addr));
                const float w1 = frac_plus_one(vpos);
                const float wa = fma_sat(-P, w1, c0), wb = fma_sat(P, w1, c1);
                accP[r] = fmaf(b, wb, fmaf(a, wa, accP[r]));
                accM[r] = fmaf(c, wb, fmaf(d, wa, accM[r]));
                vpos += (unsigned)si.b;
            }
        }
        __syncthreads();
    }

    if (split > 1) {
        // The last chunk ended with a barrier: the staging area is free.
        namespace cg = cooperative_groups;
        cg::cluster_group cl = cg::this_cluster();
        float *red = reinterpret_cast<float *>(quads);    // [2 ROWS][256]
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            red[r * 256 + threadIdx.x] = accP[r];
            red[(ROWS + r) * 256 + threadIdx.x] = accM[r];
        }
        cl.sync();
        const int per = ROWS / split;
        for (int q = 0; q < per; ++q) {
            const int r = rank * per + q;
            float sp = 0.f, sm = 0.f;
            for (int src = 0; src < split; ++src) {
                const float *peer = cl.map_shared_rank(red, src);
                sp += peer[r * 256 + threadIdx.x];
                sm += peer[(ROWS + r) * 256 + threadIdx.x];
            }
            const int row = myrow + r;
            if (row == 0 || col == 0 || row == N - 1 || col == N - 1) continue;   // edge pixels
            gather_store<1, EM>(sp, row, col, N, out, cs, ls, em_x, inv_sens);
            gather_store<1, EM>(sm, N - 1 - row, N - 1 - col, N, out, cs, ls, em_x, inv_sens);
        }
        cl.sync();    // no CTA leaves while a peer still reads its partials
        return;
    }
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
        const int row = myrow + r;
        if (row == 0 || col == 0 || row == N - 1 || col == N - 1) continue;   // edge pixels
        gather_store<1, EM>(accP[r], row, col, N, out, cs, ls, em_x, inv_sens);
        gather_store<1, EM>(accM[r], N - 1 - row, N - 1 - col, N, out, cs, ls, em_x, inv_sens);
    }
}

}  // namespace rg
