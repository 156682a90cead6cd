// gather_rot.cu -- the slant-stack backprojection with views paired a
// quarter turn apart.
//
// The backprojection (raft/raft_backprojection_slantstack.c:43-180) samples
// view theta of the sinogram at t = x cos(theta) + y sin(theta) for every
// pixel.  When the views come in pairs theta, theta' = theta + pi/2 (an
// even number of views over [theta0, theta0 + pi)) and the pixel grid is
// symmetric (x and y on the same points, centred on 0), the quarter turn
// maps the grid onto itself, and
//     x cos(theta') + y sin(theta') = y cos(theta) + (-x) sin(theta):
// pixel (x, y) at theta' meets the detector where pixel (y, -x) meets it at
// theta.  In the indices of the N x N grid (x = xmin + col dx, y = ymin +
// row dy): pixel (col N-1-r, row c) at theta' sits at the detector position
// of pixel (col c, row r) at theta.
//
// So one position -- its sample index, interpolation weight and step to
// the next pixel -- serves two views: a thread that walks the pixels (col
// c, row r), (c, r + 4), ... of its tile for view theta reads the partner
// view's staged window at the same entries and accumulates the pixels (col
// N-1-r, row c), (N-5-r, c), ... of the quarter-turned tile for view
// theta + pi/2.  The partner's window covers the same sample indices, so
// the staging area interleaves the two: entry e holds the view's sample
// pair and the partner's, 16 bytes, and one 128-bit shared load serves both
// updates.  Per update this leaves a shared load, the position arithmetic
// and two FP32 adds of the seven instructions of the one-view inner loop
// (gather_tile<0>), and the per-view set-up is shared too.  The 128-bit load
// takes as many shared-memory wavefronts per update as the 64-bit one (8
// lanes of 16 bytes, against 16 of 8), but half the load instructions.
//
// Each pixel then gets two partial sums: views [theta0, theta0 + pi/2) from
// the CTA whose tile holds it, views [theta0 + pi/2, theta0 + pi) from the
// CTA whose quarter-turned tile holds it.  The output is zeroed first and
// both partials are added atomically: two adds onto zero give the same
// float in either order, so the result does not depend on timing.
//
// Staging.  When the caller supplies scratch for it, a prepass
// (k_pair_quads) writes every quad of the plan to global memory once, [view
// pair][sample entry], and the gather (k_gather_rot_tma) loads each view
// pair's window as one TMA box into shared memory, double-buffered on two
// mbarriers, so the next chunk of 16 pairs streams in while the current one
// is summed and no thread spends issue slots on staging.  (In the FBP the
// FFT filter writes the quads and zeroes the output in its epilogue, and
// the gather runs without its prepass: QuadsPrefilled.)  Without that
// scratch, below kTmaMinPairs view pairs (where the prepass launch and the
// pipeline fill cost more) or for windows wider than a TMA box,
// k_gather_rot stages the quads itself with loads from the sinogram.
//
// Tail.  T uniform tiles over S SMs put floor(T / S) or one more tile on
// each SM, so with whole tiles the SMs that drew fewer idle through the last
// tile-time.  The TMA backprojection of one slice without a cluster split
// runs its last T mod S tiles as half tiles, two CTAs each (the rows of
// warps 0-3, or of warps 4-7, summed; the other warps only stage and wait),
// which the SMs that finish first pick up.  Every pixel still receives
// exactly two partial sums, so the bits are those of whole tiles.
//
// Precision: both kernels sum straight into FP32 accumulators (in
// k_gather_rot_tma, per-chunk partial sums would cost 2 ROWS registers: 48
// instead of 40 at 4 rows, 5 resident CTAs per SM instead of 6).  An FP32
// emulation of that order on a Ram-Lak-filtered phantom sinogram with 1800
// views (450-term sums per pixel, cluster ranks and halves added after) is
// within 2.9e-7 (rel-L2) of the FP64 sum, against 9.0e-8 with partial sums
// over chunks of 16 pairs; the error grows as the square root of the view
// count.
#include <string.h>

#include <algorithm>

#include "ss_tiles.cuh"
#include "tma.cuh"

namespace rg {

namespace {

constexpr int kPairSlots = kSlots / 2;    // view pairs per staged chunk
constexpr int kQuadBox = 256;             // widest TMA box (entries)
constexpr int kStages = 2;                // TMA window buffers (double buffering)
// Fewest view pairs for the TMA-staged form: with fewer, its prepass launch
// and pipeline fill cost more than staging by loads (measured on OSEM
// subsets of 36 pairs and 64-slice stacks of 180 pairs).
constexpr int kTmaMinPairs = 256;

// Set by QuadsPrefilled: the backprojection's quads and zeroed output were
// written by the FBP filter, so the TMA-staged gather skips its prepass.
thread_local bool t_quads_prefilled = false;

__global__ void k_zero_image(float *__restrict__ out, int N, long long cs, long long ls,
                             long long zo)
{
    pdl_gate();
    out += (long long)blockIdx.z * zo;
    const long long n = (long long)N * N;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e / N), c = (int)(e - (long long)r * N);
        out[(long long)r * cs + (long long)c * ls] = 0.f;
    }
}

// Window of view v over the tile whose first pixel is (row0, col0), TH rows
// x kTile columns: si gets the Q9.23 origin and steps and the first sample
// index nlo; the return value is the window's width in entries.
template <int MODE, int TH>
__device__ __forceinline__ int rot_window(const View &v, int row0, int col0, SlotInfo &si)
{
    long long cr, cc, c0;
    if (MODE == 0) { cr = v.brow; cc = v.bcol; c0 = v.b0; }
    else           { cr = v.krow; cc = v.kcol; c0 = v.k0; }
    const long long origin = c0 + (long long)row0 * cr + (long long)col0 * cc;
    const long long dr = (long long)(TH - 1) * cr, dc = (long long)(kTile - 1) * cc;
    const long long mn = origin + min(0LL, dr) + min(0LL, dc);
    const long long mx = origin + max(0LL, dr) + max(0LL, dc);
    const int nlo = (int)(mn >> 32) - 1;
    const int nhi = (int)(mx >> 32) + 1;
    si.nlo = nlo;
    si.base = (unsigned)((origin - ((long long)nlo << 32)) >> 9);
    si.a = (int)((cc + 256) >> 9);
    si.b = (int)((cr + 256) >> 9);
    return nhi - nlo + 1;
}

// One slot: the thread's ROWS positions for a view, each read as one
// 16-byte quad {view pair, partner pair} at shared address pw + entry *
// quad_bytes (quad_bytes == 16 arrives as an argument, so the address is an
// integer multiply-add on the FMA pipe).
template <int MODE, int ROWS>
__device__ __forceinline__ void rot_slot(const SlotInfo &si, float P, unsigned pw,
                                         unsigned quad_bytes, int cofs, int rofs,
                                         float (&partB)[ROWS], float (&partA)[ROWS])
{
    unsigned vpos = si.base + (unsigned)(cofs * si.a) + (unsigned)(rofs * si.b);
    const unsigned step = 4u * (unsigned)si.b;
    // adjoint hat weights (gather_tile): sat(-P w1 + 1 + P), sat(P w1 + 1 - 2P);
    // P is the same for a view and its partner
    const float c0 = 1.f + P, c1 = 1.f - 2.f * P;
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
        const unsigned addr = (vpos >> 23) * quad_bytes + pw;
        float2 pb, pa;
        asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                     : "=f"(pb.x), "=f"(pb.y), "=f"(pa.x), "=f"(pa.y) : "r"(addr));
        const float w1 = frac_plus_one(vpos);
        if (MODE == 0) {
            partB[r] += fmaf(w1, pb.y, pb.x);
            partA[r] += fmaf(w1, pa.y, pa.x);
        } else {
            const float wa = fma_sat(-P, w1, c0), wb = fma_sat(P, w1, c1);
            partB[r] = fmaf(pb.y, wb, fmaf(pb.x, wa, partB[r]));
            partA[r] = fmaf(pa.y, wb, fmaf(pa.x, wa, partA[r]));
        }
        vpos += step;
    }
}

// Add the tile's two partial sums to the output (through the cluster's
// distributed shared memory first when the views are split over `split`
// CTAs).  `red` is at least 2 ROWS x 256 floats of shared memory that no
// copy writes any more; every thread of the CTA calls this.
template <int MODE, int ROWS>
__device__ __forceinline__ void rot_finish(const float (&accB)[ROWS], const float (&accA)[ROWS],
                                           float *red, int split, int rank, int myrow, int col,
                                           int N, float *__restrict__ out, long long cs,
                                           long long ls, float scale, bool active = true)
{
    if (split > 1) {
        namespace cg = cooperative_groups;
        cg::cluster_group cl = cg::this_cluster();
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            red[r * 256 + threadIdx.x] = accB[r];
            red[(ROWS + r) * 256 + threadIdx.x] = accA[r];
        }
        cl.sync();
        const int per = ROWS / split;
        for (int q = 0; q < per; ++q) {
            const int r = rank * per + q;
            float sb = 0.f, sa = 0.f;
            for (int src = 0; src < split; ++src) {
                const float *peer = cl.map_shared_rank(red, src);
                sb += peer[r * 256 + threadIdx.x];
                sa += peer[(ROWS + r) * 256 + threadIdx.x];
            }
            const int row = myrow + 4 * r;
            const bool edge = MODE != 0 && (row == 0 || col == 0 || row == N - 1 || col == N - 1);
            if (row < N && col < N && !edge) {
                atomicAdd(out + (long long)row * cs + (long long)col * ls, sb * scale);
                atomicAdd(out + (long long)col * cs + (long long)(N - 1 - row) * ls, sa * scale);
            }
        }
        cl.sync();    // no CTA leaves while a peer still reads its partials
        return;
    }
    if (!active) return;   // the other half of a half-tile CTA's rows
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
        const int row = myrow + 4 * r;
        if (row >= N || col >= N) break;
        // a quarter turn maps edge pixels onto edge pixels
        if (MODE != 0 && (row == 0 || col == 0 || row == N - 1 || col == N - 1)) continue;
        atomicAdd(out + (long long)row * cs + (long long)col * ls, accB[r] * scale);
        atomicAdd(out + (long long)col * cs + (long long)(N - 1 - row) * ls, accA[r] * scale);
    }
}

// The fused EM update (EmFuse), after rot_finish.  The CTA whose tile
// starts at (row0, col0) added partial sums to the 32 x 32 pixel blocks of
// its tile (TH / 32 blocks in a column) and of the quarter-turned tile
// (TH / 32 blocks in a row).  Every block receives partials from `arrivals`
// CTAs (its tile's and its turned tile's, times the cluster split).  Each
// CTA counts itself in on each block it added to, after all of its adds
// (barrier, then a device-scope fence by the counting thread); the CTA that
// arrives last fences again, resets the counter and applies
// x <- x * gsum * inv to the block, zeroing gsum there for the next call.
// The adjoint's edge pixels are updated by the launch's edge CTAs
// (rot_edges) or by the caller's edge kernel, never here.  No thread waits
// on another CTA.  Every thread of the CTA calls this.
template <int MODE, int ROWS>
__device__ __forceinline__ void rot_em_finish(int row0, int col0, int N, float *__restrict__ gsum,
                                              float *__restrict__ x,
                                              const float *__restrict__ inv, int *cnt,
                                              int arrivals)
{
    constexpr int NB = kWarps * ROWS / 32;            // blocks per tile column
    __shared__ int s_fin[2 * NB];
    __syncthreads();                                  // this CTA's adds are issued
    const int nb = N / 32;
    if ((int)threadIdx.x < 2 * NB) {
        int br, bc;
        if ((int)threadIdx.x < NB) {                  // the tile's own blocks
            br = row0 / 32 + (int)threadIdx.x;
            bc = col0 / 32;
        } else {                                      // the quarter-turned tile's
            br = col0 / 32;
            bc = (N - row0) / 32 - NB + ((int)threadIdx.x - NB);
        }
        int fin = -1;
        if (br >= 0 && br < nb && bc >= 0 && bc < nb) {
            __threadfence();
            const int b = br * nb + bc;
            if (atomicAdd(cnt + b, 1) == arrivals - 1) {
                __threadfence();
                cnt[b] = 0;
                fin = b;
            }
        }
        s_fin[threadIdx.x] = fin;
    }
    __syncthreads();
    // 256 threads = one float4 each of a 32 x 32 block: row t / 8, columns
    // 4 (t % 8) .. + 3 (rows of a block start on 128 bytes: N % 32 == 0 and
    // 256-byte aligned buffers).  The loads of the next finished block are
    // issued before the current one is used.
    const int er = (int)threadIdx.x >> 3, ec = ((int)threadIdx.x & 7) * 4;
    auto next = [&](int k) {
        while (k < 2 * NB && s_fin[k] < 0) ++k;
        return k;
    };
    auto at = [&](int b) { return (size_t)((b / nb) * 32 + er) * N + (b % nb) * 32 + ec; };
    int k = next(0);
    float4 g = make_float4(0.f, 0.f, 0.f, 0.f), xv = g, iv = g;
    if (k < 2 * NB) {
        const size_t i = at(s_fin[k]);
        g = __ldcg(reinterpret_cast<const float4 *>(gsum + i));   // the partials' sum, from L2
        xv = *reinterpret_cast<const float4 *>(x + i);
        iv = *reinterpret_cast<const float4 *>(inv + i);
    }
    while (k < 2 * NB) {
        const int b = s_fin[k];
        const float4 cg = g, cx = xv, ci = iv;
        k = next(k + 1);
        if (k < 2 * NB) {
            const size_t i = at(s_fin[k]);
            g = __ldcg(reinterpret_cast<const float4 *>(gsum + i));
            xv = *reinterpret_cast<const float4 *>(x + i);
            iv = *reinterpret_cast<const float4 *>(inv + i);
        }
        const int r = (b / nb) * 32 + er, c = (b % nb) * 32 + ec;
        const size_t i = (size_t)r * N + c;
        const float4 o = make_float4(cx.x * cg.x * ci.x, cx.y * cg.y * ci.y,
                                     cx.z * cg.z * ci.z, cx.w * cg.w * ci.w);
        // The adjoint's edge pixels belong to the edge CTAs of the same
        // launch (rot_edges), which may update them at the same time: only
        // the interior ones are stored here.
        if (MODE == 0 || (r != 0 && r != N - 1 && c != 0 && c + 3 != N - 1)) {
            *reinterpret_cast<float4 *>(x + i) = o;
        } else if (r != 0 && r != N - 1) {
            if (c != 0) x[i] = o.x;
            x[i + 1] = o.y;
            x[i + 2] = o.z;
            if (c + 3 != N - 1) x[i + 3] = o.w;
        }
        __stcg(reinterpret_cast<float4 *>(gsum + i), make_float4(0.f, 0.f, 0.f, 0.f));
    }
}

// The matched adjoint's edge pixels (the first and last rows and columns,
// where the Radon's validity rules at line positions 0 and N - 1 apply, and
// which the paired gathers leave out), computed by the last `edge_rows` rows
// of CTAs of a paired gather's grid: 32 pixels per CTA, the views split over
// its warps (adjoint_edge_group), with the EM update where the gather fuses
// it.  They run beside the tiles, in the grid's last wave, instead of as a
// launch of their own.  Every thread of the CTA calls this.
template <bool EMF>
__device__ __forceinline__ void rot_edges(const float *__restrict__ s_am, int s_ld, int R,
                                          const View *__restrict__ views, int nv, int N,
                                          float *__restrict__ out, long long cs, long long ls,
                                          float *__restrict__ em_x,
                                          const float *__restrict__ em_inv, int edge_rows)
{
    const int g = ((int)blockIdx.y - ((int)gridDim.y - edge_rows)) * (int)gridDim.x +
                  (int)blockIdx.x;
    if (g * 32 < 4 * N - 4)
        adjoint_edge_group<1, EMF, kWarps>(s_am, s_ld, R, views, nv, N, g * 32, out, cs, ls, em_x,
                                           em_inv);
}

// Warp w covers columns 8 (w & 3) .. + 8 and rows 4 ROWS (w >> 2) .. + 4
// ROWS of the tile; lane l takes column l & 7 and rows l >> 3, + 4, + 8, ...
// So the 32 lanes of one load read 8 columns x 4 adjacent rows.  A
// quarter-warp (the 8 columns of one row) spans about 8 entries of the
// window: one shared-memory wavefront for its 128-bit loads.
__device__ __forceinline__ int rot_cofs() { return 8 * ((threadIdx.x >> 5) & 3) + (threadIdx.x & 7); }
template <int ROWS>
__device__ __forceinline__ int rot_rofs()
{
    return 4 * ROWS * (threadIdx.x >> 7) + ((threadIdx.x & 31) >> 3);
}

// MODE 0: backprojection; MODE 1: matched adjoint (edge pixels left to the
// edge CTAs, rot_edges, or to k_adjoint_edges, as in gather_tile with
// edge_fixup).  Stages each chunk's
// quads with loads from the sinogram.
template <int MODE, int WMAX, int ROWS, bool EMF>
__device__ __forceinline__ void gather_tile_rot(const float *__restrict__ s_am, int s_ld, int R,
                                                const View *__restrict__ views, int half,
                                                int roff, int N, float scale,
                                                float *__restrict__ out, long long cs,
                                                long long ls, int *__restrict__ err, int tx,
                                                int ty, float2 *__restrict__ pairs,
                                                unsigned quad_bytes, int split, int rank,
                                                float *__restrict__ em_x,
                                                const float *__restrict__ em_inv, int *em_cnt)
{
    constexpr int TH = kWarps * ROWS;                     // tile height
    __shared__ SlotInfo slot[kPairSlots];
    __shared__ int slotW[kPairSlots];
    __shared__ int slotView[kPairSlots];
    __shared__ float slotP[kPairSlots];
    __shared__ float slotDelta[2 * kPairSlots];           // views, then partners

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int row0 = ty * TH, col0 = tx * kTile;
    const int cofs = rot_cofs(), rofs = rot_rofs<ROWS>();
    const int col = col0 + cofs;
    const int myrow = row0 + rofs;             // rows myrow + 4 r

    float accB[ROWS], accA[ROWS];
#pragma unroll
    for (int r = 0; r < ROWS; ++r) { accB[r] = 0.f; accA[r] = 0.f; }

    const int vbeg = (int)((long long)half * rank / split);
    const int vend = (int)((long long)half * (rank + 1) / split);
    const unsigned sbase = smem_addr(pairs);
    for (int chunk = vbeg; chunk < vend; chunk += kPairSlots) {
        const int nslot = min(kPairSlots, vend - chunk);
        if (warp == 0 && lane < kPairSlots) {
            SlotInfo si = {0u, 0, 0, INT_MIN};
            int W = 0, view = 0;
            float P = 0.f, d0 = 0.f, d1 = 0.f;
            if (lane < nslot) {
                const View &v = views[chunk + lane];
                SlotInfo w;
                const int width = rot_window<MODE, TH>(v, row0, col0, w);
                if (width <= WMAX) {
                    si = w;
                    W = width;
                } else if (err) {
                    atomicOr(err, 1);
                }
                view = v.view;
                P = v.P;
                d0 = v.delta;
                d1 = views[chunk + lane + half].delta;
            }
            slot[lane] = si;
            slotW[lane] = W;
            slotView[lane] = view;
            slotP[lane] = P;
            slotDelta[lane] = d0;
            slotDelta[kPairSlots + lane] = d1;
        }
        __syncthreads();

        // Stage the windows: entry e of slot s holds the view's pair and its
        // partner's, side by side (one 16-byte load serves both).
        float4 *quads = reinterpret_cast<float4 *>(pairs);
        for (int s = warp; s < nslot; s += kWarps) {
            const int nlo = slot[s].nlo, W = slotW[s];
            const float *__restrict__ rv = s_am + (size_t)slotView[s] * s_ld;
            const float *__restrict__ rp = s_am + (size_t)(slotView[s] + roff) * s_ld;
            const float dv = slotDelta[s], dp = slotDelta[kPairSlots + s];
            for (int e = lane; e < W; e += 32) {
                const int n = nlo + e;
                float4 qd = make_float4(0.f, 0.f, 0.f, 0.f);
                if (MODE == 0) {
                    if (n >= 0 && n <= R - 2) {
                        const float2 a = make_pair(__ldg(rv + n), __ldg(rv + n + 1), true);
                        const float2 b = make_pair(__ldg(rp + n), __ldg(rp + n + 1), true);
                        qd = make_float4(a.x, a.y, b.x, b.y);
                    }
                } else {
                    const bool in0 = n >= 0 && n < R, in1 = n + 1 >= 0 && n + 1 < R;
                    const float v0 = in0 ? __ldg(rv + n) : 0.f, v1 = in1 ? __ldg(rv + n + 1) : 0.f;
                    const float p0 = in0 ? __ldg(rp + n) : 0.f, p1 = in1 ? __ldg(rp + n + 1) : 0.f;
                    qd = make_float4(v0 * dv, v1 * dv, p0 * dp, p1 * dp);
                }
                quads[s * WMAX + e] = qd;
            }
        }
        __syncthreads();

        for (int s = 0; s < nslot; ++s) {
            const SlotInfo si = slot[s];
            if (si.nlo == INT_MIN) continue;
            const unsigned pw = sbase + (unsigned)(s * WMAX) * quad_bytes;
            rot_slot<MODE, ROWS>(si, MODE == 0 ? 0.f : slotP[s], pw, quad_bytes, cofs, rofs,
                                 accB, accA);
        }
        __syncthreads();
    }
    // the last chunk ended with a barrier: the staging area is free
    rot_finish<MODE, ROWS>(accB, accA, reinterpret_cast<float *>(pairs), split, rank, myrow, col,
                           N, out, cs, ls, scale);
    if (EMF) rot_em_finish<MODE, ROWS>(row0, col0, N, out, em_x, em_inv, em_cnt, 2 * split);
}

// EMF: the EM update fused into the epilogue (EmFuse); a separate
// instantiation, so that the plain gathers keep their registers.
template <int MODE, int WMAX, int ROWS, bool EMF>
__global__ __launch_bounds__(256) void k_gather_rot(const float *__restrict__ s_am, int s_ld, int R,
                                                    const View *__restrict__ views, int half,
                                                    int roff, int N, float scale,
                                                    float *__restrict__ out,
                                                    long long cs, long long ls,
                                                    int *__restrict__ err, long long zs,
                                                    long long zo, unsigned quad_bytes, int split,
                                                    float *__restrict__ em_x,
                                                    const float *__restrict__ em_inv, int *em_cnt,
                                                    int edge_rows)
{
    pdl_gate();
    if (MODE == 1 && (int)blockIdx.y >= (int)gridDim.y - edge_rows) {
        rot_edges<EMF>(s_am + blockIdx.z * zs, s_ld, R, views, 2 * half, N, out + blockIdx.z * zo,
                       cs, ls, em_x, em_inv, edge_rows);
        return;
    }
    extern __shared__ __align__(16) float2 pairs[];  // [kPairSlots][WMAX] x {view, partner}
    gather_tile_rot<MODE, WMAX, ROWS, EMF>(s_am + blockIdx.z * zs, s_ld, R, views, half, roff, N, scale,
                                out + blockIdx.z * zo, cs, ls, err, blockIdx.x / split,
                                blockIdx.y, pairs, quad_bytes, split, blockIdx.x % split,
                                em_x, em_inv, em_cnt);
}

// ---------------------------------------------------------------------------
// TMA-staged form.

// Entries per view pair in the quad array: the backprojection's quads are
// samples n, n + 1 for n = 0 .. R - 2 (entry n); the adjoint's are n = -1 ..
// R - 1 (entry n + 1), zero outside the row.
__host__ __device__ constexpr int quad_entries(int mode, int R) { return mode == 0 ? R - 1 : R + 1; }

// quads[z][j][e] for view pair j (view views[j], partner views[j + half],
// sinogram rows views[j].view and views[j].view + roff): the quad that
// k_gather_rot stages for entry e.  zout != nullptr: also zero the N x N
// output of slice z (strides cs, ls; slices zo apart), which the gather then
// adds its partial sums to, in place of a launch of its own.
template <int MODE>
__global__ void k_pair_quads(const float *__restrict__ s_am, int s_ld, long long zs, int R,
                             const View *__restrict__ views, int half, int roff,
                             float4 *__restrict__ quads, float *__restrict__ zout, int N,
                             long long cs, long long ls, long long zo)
{
    pdl_gate();
    if (zout) {
        const long long n = (long long)N * N;
        const long long nt = (long long)gridDim.x * gridDim.y * blockDim.x;
        float *o = zout + blockIdx.z * zo;
        for (long long i = ((long long)blockIdx.y * gridDim.x + blockIdx.x) * blockDim.x +
                           threadIdx.x;
             i < n; i += nt) {
            const int r = (int)(i / N), c = (int)(i - (long long)r * N);
            o[(long long)r * cs + (long long)c * ls] = 0.f;
        }
    }
    const int Rq = quad_entries(MODE, R);
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (e >= Rq) return;
    const View &v = views[j];
    const float *__restrict__ rv = s_am + blockIdx.z * zs + (size_t)v.view * s_ld;
    const float *__restrict__ rp = rv + (size_t)roff * s_ld;
    float4 qd;
    if (MODE == 0) {
        const float2 a = make_pair(__ldg(rv + e), __ldg(rv + e + 1), true);
        const float2 b = make_pair(__ldg(rp + e), __ldg(rp + e + 1), true);
        qd = make_float4(a.x, a.y, b.x, b.y);
    } else {
        const int n = e - 1;
        const float dv = v.delta, dp = views[j + half].delta;
        const bool in0 = n >= 0, in1 = n + 1 < R;
        const float v0 = in0 ? __ldg(rv + n) : 0.f, v1 = in1 ? __ldg(rv + n + 1) : 0.f;
        const float p0 = in0 ? __ldg(rp + n) : 0.f, p1 = in1 ? __ldg(rp + n + 1) : 0.f;
        qd = make_float4(v0 * dv, v1 * dv, p0 * dp, p1 * dp);
    }
    quads[((size_t)blockIdx.z * half + j) * Rq + e] = qd;
}

// The paired gather on TMA-staged windows.  tm is a 3-D map over the quad
// array, (float of the quad, entry, z * half + pair), with a box of 4 x wb
// x 1 (wb a multiple of 8, so every slot's buffer starts on 128 bytes).
// There are two buffers of 16 windows.  Warp 0 sets up chunk c + 1 (its
// windows and one TMA load per view pair onto the buffer's mbarrier) while
// all warps sum chunk c; the buffer it fills was last read in chunk c - 1,
// which every thread finished before the barrier that closed it.  That
// barrier, one per chunk, also orders the slot tables.  (Three buffers cost
// a resident CTA per SM at 8 rows and measured slower.)  A
// window wider than wb is skipped with error bit 1; a wait that runs out
// sets bit 2, waits (bounded) for the CTA's copies still in flight and ends
// the view loop, and the CTA still takes part in its cluster's reduction.
// expire_first (a test switch, 0 in normal use) makes the first wait give up
// at once, so that tests can see that path run and report.
template <int MODE, int ROWS, bool EMF>
__global__ __launch_bounds__(256) void k_gather_rot_tma(const __grid_constant__ CUtensorMap tm,
                                                        const View *__restrict__ views, int half,
                                                        int N, float scale,
                                                        float *__restrict__ out, long long cs,
                                                        long long ls, int *__restrict__ err,
                                                        long long zo, int wb,
                                                        unsigned quad_bytes, int split,
                                                        int expire_first,
                                                        float *__restrict__ em_x,
                                                        const float *__restrict__ em_inv,
                                                        int *em_cnt,
                                                        const float *__restrict__ s_am, int s_ld,
                                                        int R, long long zs, int edge_rows,
                                                        int nfull, int nhalf)
{
    pdl_gate();
    if (MODE == 1 && (int)blockIdx.y >= (int)gridDim.y - edge_rows) {
        rot_edges<EMF>(s_am + blockIdx.z * zs, s_ld, R, views, 2 * half, N, out + blockIdx.z * zo,
                       cs, ls, em_x, em_inv, edge_rows);
        return;
    }
    // Tiles in launch order.  nhalf > 0 (the backprojection of one slice,
    // no cluster split, no fused update): the first nfull CTAs take whole
    // tiles, the next 2 nhalf the last nhalf tiles by halves (`part` 0: the
    // rows of warps 0-3, 1: those of warps 4-7), so that the launch's last
    // wave spreads evenly over the SMs; the grid's spare CTAs return here.
    // (The adjoint's launches, split over clusters where the tuner finds it
    // faster, compile without it.)
    int tx = blockIdx.x / split, ty = blockIdx.y, part = -1;
    if (MODE == 0 && nhalf > 0) {
        int t = blockIdx.y * gridDim.x + blockIdx.x;
        if (t >= nfull) {
            const int h = t - nfull;
            if (h >= 2 * nhalf) return;                 // CTA-uniform, before any barrier
            t = nfull + (h >> 1);
            part = h & 1;
        }
        tx = t % gridDim.x;
        ty = t / gridDim.x;
    }
    const bool active = MODE != 0 || part < 0 || (int)(threadIdx.x >> 7) == part;
    extern __shared__ __align__(128) float4 qbuf[];   // [kStages][kPairSlots][wb]
    __shared__ __align__(8) unsigned long long full[kStages];
    __shared__ SlotInfo slot[kStages][kPairSlots];
    __shared__ float slotP[kStages][kPairSlots];
    constexpr int TH = kWarps * ROWS;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int rank = blockIdx.x % split;
    const int z = blockIdx.z;
    out += (long long)z * zo;
    const int row0 = ty * TH, col0 = tx * kTile;
    const int cofs = rot_cofs(), rofs = rot_rofs<ROWS>();
    const int col = col0 + cofs;
    const int myrow = row0 + rofs;

    float accB[ROWS], accA[ROWS];
#pragma unroll
    for (int r = 0; r < ROWS; ++r) { accB[r] = 0.f; accA[r] = 0.f; }

    const int vbeg = (int)((long long)half * rank / split);
    const int vend = (int)((long long)half * (rank + 1) / split);
    const int nchunks = (vend - vbeg + kPairSlots - 1) / kPairSlots;
    const unsigned qbase = smem_addr(qbuf);
    const unsigned slot_bytes = (unsigned)wb * 16u;
    if (threadIdx.x == 0) {
        for (int b = 0; b < kStages; ++b) mbar_init(smem_addr(&full[b]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    // Warp 0: windows of chunk c into slot[c % kStages], then the loads.
    auto issue = [&](int c) {
        const int chunk = vbeg + c * kPairSlots;
        const int nslot = min(kPairSlots, vend - chunk);
        const int b = c % kStages;
        SlotInfo si = {0u, 0, 0, INT_MIN};
        float P = 0.f;
        bool ok = false;
        if (lane < nslot) {
            const View &v = views[chunk + lane];
            SlotInfo w;
            if (rot_window<MODE, TH>(v, row0, col0, w) <= wb) {
                si = w;
                ok = true;
            } else if (err) {
                atomicOr(err, 1);
            }
            P = v.P;
        }
        if (lane < kPairSlots) {
            slot[b][lane] = si;
            slotP[b][lane] = P;
        }
        const unsigned valid = __ballot_sync(0xffffffffu, ok);
        const unsigned bar = smem_addr(&full[b]);
        if (lane == 0) mbar_expect_tx(bar, (unsigned)__popc(valid) * slot_bytes);
        __syncwarp();
        if (ok)
            tma_load_3d(qbase + (unsigned)(b * kPairSlots + lane) * slot_bytes, &tm, 0,
                        si.nlo + (MODE == 0 ? 0 : 1), z * half + chunk + lane, bar);
    };

    if (warp == 0 && nchunks > 0) issue(0);
    // chunk 0's slot tables; those of chunk c + 1, written during chunk c,
    // are ordered by chunk c's closing barrier
    __syncthreads();
    int c = 0;
    bool failed = false;
    for (; c < nchunks; ++c) {
        const int b = c % kStages;
        if (warp == 0 && c + 1 < nchunks) issue(c + 1);
        // A wait that runs out is acted on at the chunk's closing barrier:
        // until then the thread sums whatever the buffer holds (its reads
        // stay inside it), and the call reports the error.
        const bool ok = (expire_first && c == 0) ? false
                                                 : mbar_wait(smem_addr(&full[b]), (c / kStages) & 1);
        const int nslot = active ? min(kPairSlots, vend - (vbeg + c * kPairSlots)) : 0;
        for (int s = 0; s < nslot; ++s) {
            const SlotInfo si = slot[b][s];
            if (si.nlo == INT_MIN) continue;
            const unsigned pw = qbase + (unsigned)(b * kPairSlots + s) * slot_bytes;
            rot_slot<MODE, ROWS>(si, MODE == 0 ? 0.f : slotP[b][s], pw, quad_bytes, cofs, rofs,
                                 accB, accA);
        }
        // closes chunk c: every thread is done with its buffer and slots
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
    }
    if (failed) {
        if (threadIdx.x == 0) {
            if (err) atomicOr(err, 2);
            // copies still in flight: chunk c and, if issued, chunk c + 1
            for (int q = c; q < min(c + kStages, nchunks); ++q)
                mbar_wait(smem_addr(&full[q % kStages]), (q / kStages) & 1);
        }
        __syncthreads();
    }
    rot_finish<MODE, ROWS>(accB, accA, reinterpret_cast<float *>(qbuf), split, rank, myrow, col,
                           N, out, cs, ls, scale, active);
    if (EMF) rot_em_finish<MODE, ROWS>(row0, col0, N, out, em_x, em_inv, em_cnt, 2 * split);
}

// CTA rows to append to a paired gather's grid of gx CTAs per row for the
// adjoint's edge pixels (32 per CTA), or 0.
static int edge_rows_for(int N, int gx, bool edges)
{
    if (!edges) return 0;
    const int groups = (4 * N - 4 + 31) / 32;
    return (groups + gx - 1) / gx;
}

template <int MODE, int WMAX, int ROWS>
int gather_rot_w(const SSPlan &p, const float *s_am, int s_ld, float *out, long long cs,
                 long long ls, int *d_err, cudaStream_t st, const Stack &z, const EmFuse *em,
                 bool edges)
{
    float *ex = em ? em->x : nullptr;
    const float *ei = em ? em->inv : nullptr;
    int *ec = em ? em->cnt : nullptr;
    // half: view pairs; roff: sinogram rows between a view and its partner
    const int N = p.g.N, half = p.nv / 2, roff = p.g.A / 2;
    // the staging area, which also holds the cluster reduction's partials
    const size_t smem = std::max((size_t)kPairSlots * WMAX * sizeof(float4),
                                 (size_t)2 * ROWS * 256 * sizeof(float));
    dim3 grid((N + kTile - 1) / kTile, (N + kWarps * ROWS - 1) / (kWarps * ROWS), z.n);
    auto k = em ? k_gather_rot<MODE, WMAX, ROWS, true> : k_gather_rot<MODE, WMAX, ROWS, false>;
    RG_CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int split = gather_pick_split((const void *)k, smem, ROWS, half, grid, st);
    const unsigned pb = (unsigned)sizeof(float4);
    const float scale = MODE == 0 ? p.dth : 1.f;
    const int er = edge_rows_for(N, (int)grid.x * split, MODE == 1 && edges);
    RG_CK(launch_pdl(k, dim3(grid.x * split, grid.y + er, grid.z), 256, smem, st, split,
                     s_am, s_ld, p.g.R, (const View *)p.d_views, half, roff, N,
                     scale, out, cs, ls, d_err, z.in, z.out, pb, split, ex, ei, ec, er));
    RG_CK_LAUNCH("k_gather_rot");
    return RG_OK;
}

// RG_GATHER_HALF_TILES=0 (read per call) launches whole tiles only.
bool half_tiles_enabled()
{
    const char *e = getenv("RG_GATHER_HALF_TILES");
    return !(e && e[0] == '0' && e[1] == 0);
}

// SMs of the current device (cached per device).
int sm_count()
{
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    if (!cache[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return 0;
        cache[dev] = n;
    }
    return cache[dev];
}

// TMA box width for a window bound w: a multiple of 8 entries (128 bytes).
int quad_box(int w) { return (w + 7) & ~7; }

template <int MODE, int ROWS>
int gather_rot_tma(const SSPlan &p, const float *s_am, int s_ld, float *out, long long cs,
                   long long ls, int *d_err, cudaStream_t st, const Stack &z, float4 *quads,
                   int w, bool zero_out, const EmFuse *em, bool edges)
{
    float *ex = em ? em->x : nullptr;
    const float *ei = em ? em->inv : nullptr;
    int *ec = em ? em->cnt : nullptr;
    const int N = p.g.N, R = p.g.R, half = p.nv / 2, roff = p.g.A / 2;
    const int Rq = quad_entries(MODE, R);
    if (!(MODE == 0 && t_quads_prefilled)) {
        dim3 g((Rq + 255) / 256, half, z.n);
        RG_CK(launch_pdl(k_pair_quads<MODE>, g, 256, 0, st, 1, s_am, s_ld, z.in, R, p.d_views,
                         half, roff, quads, zero_out ? out : nullptr, N, cs, ls, z.out));
        RG_CK_LAUNCH("k_pair_quads");
    }
    // RG_TEST_WINDOW_CUT=1 (a test switch) under-reports the window bound by
    // one step of 8: the box and the buffers shrink with it, and the slots
    // whose windows no longer fit are skipped with error bit 1.
    const int wb = quad_box(w) - (test_switch("RG_TEST_WINDOW_CUT") && quad_box(w) > 8 ? 8 : 0);
    const int expire = test_switch("RG_TEST_EXPIRE_WAIT") ? 1 : 0;
    CUtensorMap tm;
    {
        EncodeTiledFn fn = tensor_map_encoder();
        if (!fn) return set_error(RG_ECUDA, "cuTensorMapEncodeTiled is not available");
        cuuint64_t dims[3] = {4, (cuuint64_t)Rq, (cuuint64_t)half * z.n};
        cuuint64_t strides[2] = {16, (cuuint64_t)Rq * 16};
        cuuint32_t box[3] = {4, (cuuint32_t)wb, 1};
        cuuint32_t estr[3] = {1, 1, 1};
        CUresult r = fn(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void *)quads, dims, strides,
                        box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS)
            return set_error(RG_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    }
    auto k = em ? k_gather_rot_tma<MODE, ROWS, true> : k_gather_rot_tma<MODE, ROWS, false>;
    // two buffers of 16 windows, which also hold the cluster reduction's partials
    const size_t smem = std::max((size_t)kStages * kPairSlots * wb * sizeof(float4),
                                 (size_t)2 * ROWS * 256 * sizeof(float));
    dim3 grid((N + kTile - 1) / kTile, (N + kWarps * ROWS - 1) / (kWarps * ROWS), z.n);
    RG_CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int split = gather_pick_split((const void *)k, smem, ROWS, half, grid, st);
    const unsigned qb = (unsigned)sizeof(float4);
    const float scale = MODE == 0 ? p.dth : 1.f;
    const int er = edge_rows_for(N, (int)grid.x * split, MODE == 1 && edges);
    // Uniform tiles leave the last wave uneven: T tiles over S SMs put
    // floor(T / S) or one more on each SM.  The backprojection of one slice
    // without a cluster split or fused update runs its last T mod S tiles
    // as half tiles (two CTAs each), which the SMs that finish first pick
    // up: 2048^2 x 1800 (2048 tiles, 72 in halves) 1.797 -> 1.748 ms.
    int nfull = 0, nhalf = 0;
    dim3 g = grid;
    if (MODE == 0 && split == 1 && !em && z.n == 1 && half_tiles_enabled()) {
        const int T = (int)(grid.x * grid.y), S = sm_count();
        if (S > 0 && T > S && T % S) {
            nhalf = T % S;
            nfull = T - nhalf;
            g.y = (unsigned)((nfull + 2 * nhalf + (int)grid.x - 1) / (int)grid.x);
        }
    }
    RG_CK(launch_pdl(k, dim3(g.x * split, g.y + er, g.z), 256, smem, st, split,
                     tm, (const View *)p.d_views, half, N, scale, out, cs, ls,
                     d_err, z.out, wb, qb, split, expire, ex, ei, ec, s_am, s_ld, R, z.in, er,
                     nfull, nhalf));
    RG_CK_LAUNCH("k_gather_rot_tma");
    return RG_OK;
}

// RG_GATHER_ROT_TMA: 0 stages by loads, 1 by TMA whenever the call brings
// the quad scratch; unset: by TMA from kTmaMinPairs view pairs.
bool gather_rot_use_tma(int pairs)
{
    const char *e = getenv("RG_GATHER_ROT_TMA");
    if (e && !strcmp(e, "0")) return false;
    if (e && !strcmp(e, "1")) return true;
    return pairs >= kTmaMinPairs;
}

// The TMA-staged form serves (plan, mode, tile height) with quad scratch.
bool tma_form(const SSPlan &p, int mode, int rows, bool quads)
{
    const int t = rows == 16 ? 2 : rows == 8 ? 1 : 0;
    const int w = mode == 0 ? p.wmax_bp[t] : p.wmax_adj[t];
    return quads && quad_box(w) <= kQuadBox && p.nv / 2 <= 65535 && gather_rot_use_tma(p.nv / 2);
}

template <int MODE, int ROWS>
int gather_rot_rows(const SSPlan &p, const float *s_am, int s_ld, float *out, long long cs,
                    long long ls, int *d_err, cudaStream_t st, const Stack &z, void *quads,
                    bool zero_out, const EmFuse *em, bool edges)
{
    const int t = ROWS == 16 ? 2 : ROWS == 8 ? 1 : 0;
    const int w = MODE == 0 ? p.wmax_bp[t] : p.wmax_adj[t];
    if (tma_form(p, MODE, ROWS, quads != nullptr))
        return gather_rot_tma<MODE, ROWS>(p, s_am, s_ld, out, cs, ls, d_err, st, z,
                                          (float4 *)quads, w, zero_out, em, edges);
    if (MODE == 0 && t_quads_prefilled)
        return set_error(RG_EINVAL, "prefilled quads for a backprojection that stages by loads");
    if (zero_out)
        if (int rc = launch_zero_image(out, p.g.N, cs, ls, st, z)) return rc;
    if (w <= 64)
        return gather_rot_w<MODE, 64, ROWS>(p, s_am, s_ld, out, cs, ls, d_err, st, z, em, edges);
    if (w <= 128)
        return gather_rot_w<MODE, 128, ROWS>(p, s_am, s_ld, out, cs, ls, d_err, st, z, em, edges);
    if (w <= 256)
        return gather_rot_w<MODE, 256, ROWS>(p, s_am, s_ld, out, cs, ls, d_err, st, z, em, edges);
    if (w <= 512)
        return gather_rot_w<MODE, 512, ROWS>(p, s_am, s_ld, out, cs, ls, d_err, st, z, em, edges);
    return set_error(RG_EUNSUPPORTED,
                     "gather window of %d samples per tile exceeds 512 "
                     "(image much coarser than the ray spacing)", w);
}

}  // namespace

QuadsPrefilled::QuadsPrefilled() { t_quads_prefilled = true; }
QuadsPrefilled::~QuadsPrefilled() { t_quads_prefilled = false; }

bool gather_quads_form(const SSPlan &p, void *quads)
{
    return quads && p.rot_ok && gather_rot_enabled() && tma_form(p, 0, tuned_rows(p, 0), true);
}

int launch_zero_image(float *out, int N, long long cs, long long ls, cudaStream_t st,
                      const Stack &z)
{
    const long long n = (long long)N * N;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 4096);
    RG_CK(launch_pdl(k_zero_image, dim3(blocks, 1, z.n), 256, 0, st, 1, out, N, cs, ls, z.out));
    RG_CK_LAUNCH("k_zero_image");
    return RG_OK;
}

size_t gather_quads_bytes(int nv, int R, int nz)
{
    if (nv < 2 || R < 2 || nz < 1) return 0;
    return (size_t)nz * (size_t)(nv / 2) * (size_t)quad_entries(1, R) * sizeof(float4);
}

int launch_gather_rot(const SSPlan &p, int mode, const float *s_am, int s_ld, float *out,
                      long long cs, long long ls, int *d_err, cudaStream_t st, int rows,
                      const Stack &z, void *quads, bool zero_out, const EmFuse *em, bool edges)
{
    const bool zo = zero_out;
    if (em && (!em_fusable(p.g.N) || z.n != 1 || out != em->gsum || cs != p.g.N || ls != 1 ||
               zero_out))
        return set_error(RG_EINVAL, "fused EM gather: one N x N slice, N a multiple of 32, "
                                    "into its own zeroed partial-sum buffer");
    if (mode == 0) {
        auto f = rows == 16 ? gather_rot_rows<0, 16> : rows == 8 ? gather_rot_rows<0, 8>
                                                                  : gather_rot_rows<0, 4>;
        return f(p, s_am, s_ld, out, cs, ls, d_err, st, z, quads, zo, em, false);
    }
    auto f = rows == 16 ? gather_rot_rows<1, 16> : rows == 8 ? gather_rot_rows<1, 8>
                                                              : gather_rot_rows<1, 4>;
    return f(p, s_am, s_ld, out, cs, ls, d_err, st, z, quads, zo, em, edges);
}

}  // namespace rg
