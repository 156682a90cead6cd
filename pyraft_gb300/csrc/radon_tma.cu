// radon_tma.cu -- slant-stack Radon with TMA-staged line windows.
//
// Same operator as radon_tile (raft/raft_radon_slantstack.c:122-214; see
// slantstack.cu): ray k of view j sums, over the lines i of the image, the
// linear interpolation at u = r0 + k rk + i ri (Q32.32), read as one pair
// (s - d, d) of the padded line-pair arrays.
//
// GB300 design.  A CTA owns 64 consecutive rays of a block of up to 16
// adjacent views of one orientation (lines = image rows, or columns).  On
// every image line those 64 x 16 sample positions fall inside one window of
// at most BW consecutive entries: the rays of a view are ~1 entry apart and
// adjacent views move the positions by a few entries.  The CTA walks the
// lines in strips of 16; for each strip one elected thread issues a single
// 3-D TMA load (cp.async.bulk.tensor) of the BW x 16 window box into shared
// memory, double-buffered on two mbarriers, so the next strip streams in
// while the current one is summed.  Entries outside the line-pair array
// (left of entry 0, right of the pitch, past line N-1) are zero-filled by the
// TMA unit, so the box needs no clamping.  Every (ray, view) then reads its
// samples with LDS.64 at a Q9.23 local position (index = bits 23..31, weight
// 1 + w from the low 23 bits); a thread carries one ray of four views.
//
// The host partitions the plan's views into blocks whose window provably
// fits: positions are affine in (ray, line), so the window width over all
// ray tiles and strips is largest at the corner tiles and strips, which are
// checked exactly in integer arithmetic.  The kernel re-derives each strip's
// window start from the same corner positions and checks the width again;
// a strip that would not fit is skipped with an error flag, never read out
// of bounds.  The plan also fixes the order in which the (ray tile, view
// block) CTAs are dispatched, most strips first (st_cta_order), so that the
// launch's last wave holds its lightest CTAs.  Every mbarrier wait is
// bounded; a CTA whose wait runs out sets
// the error flag, waits (bounded) for its own copies and leaves.
// expire_first (a test switch, 0 in normal use) makes each CTA's first strip
// wait give up at once, so that tests can see that path run and report.
#include <cuda.h>
#include <string.h>

#include <algorithm>
#include <climits>
#include <mutex>
#include <vector>

#include "ss_tiles.cuh"
#include "tma.cuh"

namespace rg {

constexpr int kTmRays = 64;     // rays per CTA (two warps of 32)
constexpr int kTmViews = 16;    // views per block (max)
constexpr int kTmVpt = 4;       // views per thread
constexpr int kTmLines = 16;    // lines per strip
// One full strip of a (ray, view): 16 lines, line r of the strip buffer at
// byte offset r * BW * 8 (an immediate of the load).  pb (== 8, the bytes
// of a pair) arrives as a kernel argument, so the sample's address is one
// integer multiply-add on the FMA pipe instead of a shift and an add on the
// integer pipe, which the position and weight bits keep busy.
template <int BW, int R0>
__device__ __forceinline__ void strip16(unsigned sb, unsigned &L, unsigned dq, unsigned pb,
                                        float &part)
{
    if constexpr (R0 < kTmLines) {
        const float2 pr = lds_pair_at<R0 * BW * 8>((L >> 23) * pb + sb);
        part += fmaf(frac_plus_one(L), pr.y, pr.x);
        L += dq;
        strip16<BW, R0 + 1>(sb, L, dq, pb, part);
    }
}

// Lane layout: each shared load of a warp covers RPL consecutive rays of
// 32 / RPL adjacent views.  Rays are >= 1 entry apart on a line while
// adjacent views sit a few entries apart, so fewer rays per load (more
// views) packs the 32 lanes' 8-byte reads into fewer shared-memory
// wavefronts.  A thread carries 4 (ray, view) pairs m: the warp's 32 rays x
// 4 views are covered as ray group m % (32 / RPL) and view group
// m / (32 / RPL).
template <int EPI, int BW, int RPL>
__global__ __launch_bounds__(256, 3) void k_radon_tma(const __grid_constant__ CUtensorMap tm_rows,
                                                   const __grid_constant__ CUtensorMap tm_cols,
                                                   int N, const View *__restrict__ views,
                                                   const StBlock *__restrict__ blocks,
                                                   const unsigned *__restrict__ order, int R,
                                                   float *__restrict__ out_am, int out_ld,
                                                   const float *__restrict__ y_am, int y_ld,
                                                   long long zo, int *__restrict__ err,
                                                   unsigned pb, int expire_first, int split)
{
    pdl_gate();
    extern __shared__ __align__(128) float2 sbuf[];   // [2][kTmLines][BW]
    __shared__ __align__(8) unsigned long long full[2];
    __shared__ int xs[2];                             // window start entry per buffer
    __shared__ int bad[2];                            // window did not fit
    __shared__ long long cr0[kTmViews], crk[kTmViews], cri[kTmViews];
    __shared__ int s_lo, s_hi;
    __shared__ float red[kTmVpt][256];                 // cluster partials (split > 1)

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // split > 1: this CTA is rank `rank` of a cluster of `split` CTAs along x
    // that share the ray tile and view block; it walks its share of the
    // strips, and rank 0 sums the partials (distributed shared memory, rank
    // order) and writes the epilogue.  The cluster's (ray tile, view block)
    // comes from the plan's dispatch order (most lines first).
    const int rank = blockIdx.x % split;
    const unsigned ord = order[blockIdx.x / split + (gridDim.x / split) * blockIdx.y];
    const StBlock blk = blocks[ord & 0xffffu];
    const int k0 = (int)(ord >> 16) * kTmRays;
    constexpr int kRG = 32 / RPL;
    static_assert(RPL == 32 || RPL == 16 || RPL == 8, "rays per load");
    // pair m: ray k0 + 32 (warp & 1) + RPL (m % kRG) + lane % RPL,
    //         view (warp >> 1) * 4 + lane / RPL + (32 / RPL) (m / kRG)
    int kk_[kTmVpt], vv_[kTmVpt];
#pragma unroll
    for (int m = 0; m < kTmVpt; ++m) {
        kk_[m] = k0 + (warp & 1) * 32 + RPL * (m % kRG) + lane % RPL;
        vv_[m] = (warp >> 1) * kTmVpt + lane / RPL + (32 / RPL) * (m / kRG);
    }
    const int z = blockIdx.z;
    const CUtensorMap *tm = (blk.flags & kLinesAreRows) ? &tm_rows : &tm_cols;
    out_am += (long long)z * zo;

    long long u0[kTmVpt], q[kTmVpt];
    int lo[kTmVpt], hi[kTmVpt];
    int mylo = INT_MAX, myhi = INT_MIN;
#pragma unroll
    for (int v = 0; v < kTmVpt; ++v) {
        lo[v] = 1;
        hi[v] = 0;
        u0[v] = 0;
        q[v] = 0;
        if (vv_[v] < blk.count && kk_[v] < R) {
            const View &V = views[blk.first + vv_[v]];
            u0[v] = V.r0 + (long long)kk_[v] * V.rk;
            q[v] = V.ri;
            radon_line_range(u0[v], q[v], N, lo[v], hi[v]);
            if (lo[v] <= hi[v]) {
                mylo = min(mylo, lo[v]);
                myhi = max(myhi, hi[v]);
            }
        }
    }
    if (threadIdx.x < kTmViews && threadIdx.x < blk.count) {
        const View &V = views[blk.first + threadIdx.x];
        cr0[threadIdx.x] = V.r0;
        crk[threadIdx.x] = V.rk;
        cri[threadIdx.x] = V.ri;
    }
    if (threadIdx.x == 0) {
        s_lo = INT_MAX;
        s_hi = INT_MIN;
        mbar_init(smem_addr(&full[0]), 1);
        mbar_init(smem_addr(&full[1]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    mylo = __reduce_min_sync(0xffffffffu, mylo);
    myhi = __reduce_max_sync(0xffffffffu, myhi);
    if (lane == 0) {
        atomicMin(&s_lo, mylo);
        atomicMax(&s_hi, myhi);
    }
    __syncthreads();
    const int Lo = s_lo, Hi = s_hi;

    float acc[kTmVpt], comp[kTmVpt];
#pragma unroll
    for (int v = 0; v < kTmVpt; ++v) acc[v] = comp[v] = 0.f;

    if (Lo <= Hi) {
        const int nall = Hi / kTmLines - Lo / kTmLines + 1;
        const int s0 = (int)((long long)nall * rank / split);
        const int sfirst = Lo / kTmLines + s0;
        const int nstrips = (int)((long long)nall * (rank + 1) / split) - s0;
        const unsigned sbase = smem_addr(sbuf);
        constexpr unsigned kBufBytes = kTmLines * BW * 8;

        // Warp 0: window of strip n from the block's corner positions, then
        // lane 0 arms the buffer's barrier and issues the TMA load.
        auto issue = [&](int n) {
            const int i0 = (sfirst + n) * kTmLines;
            const int i1 = min(i0 + kTmLines - 1, N - 1);
            const int c = lane >> 1;
            int emin = INT_MAX, emax = INT_MIN;
            if (c < blk.count) {
                const int kk = (lane & 1) ? min(k0 + kTmRays - 1, R - 1) : k0;
                const long long ua = cr0[c] + (long long)kk * crk[c] + (long long)i0 * cri[c];
                const long long ub = ua + (long long)(i1 - i0) * cri[c];
                const int ea = (int)(ua >> 32) + 1, eb = (int)(ub >> 32) + 1;
                emin = min(ea, eb);
                emax = max(ea, eb);
            }
            emin = __reduce_min_sync(0xffffffffu, emin);
            emax = __reduce_max_sync(0xffffffffu, emax);
            // one entry of slack on both sides for the Q9.23 stepping
            const int x0 = (emin - 1) & ~1;
            if (lane == 0) {
                const int b = n & 1;
                xs[b] = x0;
                bad[b] = (emax + 1 - x0 >= BW) ? 1 : 0;
                fence_proxy_async_smem();
                mbar_expect_tx(smem_addr(&full[b]), kBufBytes);
                tma_load_3d(sbase + b * kBufBytes, tm, x0, i0, z, smem_addr(&full[b]));
            }
        };

        if (warp == 0 && nstrips > 0) issue(0);
        int n = 0;
        bool failed = false;
        for (; n < nstrips; ++n) {
            const int b = n & 1;
            // buffer b ^ 1 was last read in strip n - 1, which every thread
            // finished before the barrier that closed it
            if (warp == 0 && n + 1 < nstrips) issue(n + 1);
            const bool ok = (expire_first && n == 0) ? false
                                                     : mbar_wait(smem_addr(&full[b]), (n >> 1) & 1);
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            const int i0 = (sfirst + n) * kTmLines;
            if (!bad[b]) {
                const int x0 = xs[b];
                const unsigned sb = sbase + b * kBufBytes;
#pragma unroll
                for (int v = 0; v < kTmVpt; ++v) {
                    const int a = max(lo[v], i0), e = min(hi[v], i0 + kTmLines - 1);
                    if (a > e) continue;
                    const long long ua = u0[v] + (long long)a * q[v];
                    unsigned L = (unsigned)((ua - ((long long)(x0 - 1) << 32)) >> 9);
                    const unsigned dq = (unsigned)((q[v] + 256) >> 9);
                    float part = 0.f;
                    if (a == i0 && e == i0 + kTmLines - 1) {
                        strip16<BW, 0>(sb, L, dq, pb, part);
                    } else {
                        unsigned lb = sb + (unsigned)(a - i0) * (BW * 8);
                        for (int i = a; i <= e; ++i) {
                            const float2 pr = lds_pair_at<0>((L >> 23) * pb + lb);
                            part += fmaf(frac_plus_one(L), pr.y, pr.x);
                            L += dq;
                            lb += BW * 8;
                        }
                    }
                    kahan_add(acc[v], comp[v], part);
                }
            } else if (threadIdx.x == 0 && err) {
                atomicOr(err, 1);
            }
            __syncthreads();
        }
        if (failed && threadIdx.x == 0) {
            if (err) atomicOr(err, 2);
            // copies still in flight: strip n (buffer n & 1) and, if issued,
            // strip n + 1; wait for them (bounded) before leaving
            mbar_wait(smem_addr(&full[n & 1]), (n >> 1) & 1);
            if (n + 1 < nstrips) mbar_wait(smem_addr(&full[(n + 1) & 1]), ((n + 1) >> 1) & 1);
        }
    }

    float tot[kTmVpt];
#pragma unroll
    for (int v = 0; v < kTmVpt; ++v) tot[v] = acc[v] - comp[v];
    if (split > 1) {
        namespace cg = cooperative_groups;
        cg::cluster_group cl = cg::this_cluster();
#pragma unroll
        for (int v = 0; v < kTmVpt; ++v) red[v][threadIdx.x] = tot[v];
        cl.sync();
        if (rank == 0) {
#pragma unroll
            for (int v = 0; v < kTmVpt; ++v) tot[v] = 0.f;
            for (int src = 0; src < split; ++src) {
                const float *peer = cl.map_shared_rank(&red[0][0], src);
#pragma unroll
                for (int v = 0; v < kTmVpt; ++v) tot[v] += peer[v * 256 + threadIdx.x];
            }
        }
        cl.sync();    // no CTA leaves while rank 0 still reads its partials
        if (rank != 0) return;
    }
#pragma unroll
    for (int v = 0; v < kTmVpt; ++v) {
        if (vv_[v] >= blk.count || kk_[v] >= R) continue;
        const View &V = views[blk.first + vv_[v]];
        const float val = tot[v] * V.delta;
        out_am[(size_t)V.view * out_ld + kk_[v]] =
            radon_epilogue(EPI, val, y_am, (size_t)V.view * y_ld + kk_[v]);
    }
}

// ----------------------------------------------------------------------------
// Host side.

// Window width (entries, with the kernel's slack) of a growing block of
// views, over the corner ray tiles and strips (positions are affine in
// (ray, line), so the width over every tile and strip is largest there).
struct BlockSpan {
    long long emin[4], emax[4];
    int k0[2], i0[2];
    BlockSpan(int N, int R)
    {
        k0[0] = 0;
        k0[1] = ((R - 1) / kTmRays) * kTmRays;
        i0[0] = 0;
        i0[1] = ((N - 1) / kTmLines) * kTmLines;
        for (int c = 0; c < 4; ++c) { emin[c] = LLONG_MAX; emax[c] = LLONG_MIN; }
    }
    void add(const View &v, long long *mn, long long *mx) const
    {
        for (int c = 0; c < 4; ++c) {
            mn[c] = emin[c];
            mx[c] = emax[c];
            const int ka = k0[c & 1], ia = i0[c >> 1];
            for (int kk : {ka, ka + kTmRays - 1})
                for (int ii : {ia, ia + kTmLines - 1}) {
                    const long long u = v.r0 + (long long)kk * v.rk + (long long)ii * v.ri;
                    const long long en = (u >> 32) + 1;
                    mn[c] = std::min(mn[c], en);
                    mx[c] = std::max(mx[c], en);
                }
        }
    }
    static long long width(const long long *mn, const long long *mx)
    {
        long long w = 0;
        for (int c = 0; c < 4; ++c) w = std::max(w, mx[c] + 2 - ((mn[c] - 1) & ~1LL));
        return w;
    }
};

static bool radon_kernel_direct()
{
    const char *e = getenv("RG_RADON_KERNEL");
    return e && !strcmp(e, "direct");
}

// Dispatch order of the TMA Radon's CTAs, as (ray tile << 16 | block): the
// CTA of ray tile t and view block b walks the strips of lines that any of
// its rays meets, so the central ray tiles of oblique views carry several
// times the lines of the edge tiles.  Launched in grid order, the last wave
// mixes heavy and light CTAs and the SMs that drew heavy ones finish late;
// issued longest first (CTAs are dispatched in linear order), the last wave
// holds the lightest CTAs.  A CTA's lines are estimated from its corner
// rays (a ray's first and last line are monotone in its position on the
// detector, so the corner rays bound the tile's).
static std::vector<unsigned> st_cta_order(const std::vector<StBlock> &bl, const View *hv, int N,
                                          int R)
{
    const int T = (R + kTmRays - 1) / kTmRays, nb = (int)bl.size();
    std::vector<int> strips((size_t)T * nb, 0);
    for (int b = 0; b < nb; ++b)
        for (int t = 0; t < T; ++t) {
            int Lo = INT_MAX, Hi = INT_MIN;
            for (int c = 0; c < bl[b].count; ++c) {
                const View &v = hv[bl[b].first + c];
                for (int kk : {t * kTmRays, std::min(t * kTmRays + kTmRays - 1, R - 1)}) {
                    int lo, hi;
                    radon_line_range(v.r0 + (long long)kk * v.rk, v.ri, N, lo, hi);
                    if (lo <= hi) {
                        Lo = std::min(Lo, lo);
                        Hi = std::max(Hi, hi);
                    }
                }
            }
            strips[(size_t)b * T + t] = Lo <= Hi ? Hi / kTmLines - Lo / kTmLines + 1 : 0;
        }
    std::vector<unsigned> order((size_t)T * nb);
    for (size_t i = 0; i < order.size(); ++i) order[i] = (unsigned)i;
    std::stable_sort(order.begin(), order.end(),
                     [&](unsigned a, unsigned b) { return strips[a] > strips[b]; });
    for (unsigned &o : order) o = ((o % (unsigned)T) << 16) | (o / (unsigned)T);
    return order;
}

int st_blocks_build(SSPlan &p, const View *hv)
{
    p.nblocks = 0;
    p.st_bw = 0;
    const int N = p.g.N, R = p.g.R, nv = p.nv;
    // the dispatch order packs the ray tile into 16 bits
    if (nv < 1 || (R + kTmRays - 1) / kTmRays > 65535) return RG_OK;
    for (int bw : {128, 256}) {
        std::vector<StBlock> bl;
        bool fits = true;
        for (int e = 0; e < nv && fits;) {
            BlockSpan sp(N, R);
            long long mn[4], mx[4];
            sp.add(hv[e], mn, mx);
            if (BlockSpan::width(mn, mx) > bw) { fits = false; break; }
            memcpy(sp.emin, mn, sizeof mn);
            memcpy(sp.emax, mx, sizeof mx);
            int c = 1;
            while (c < kTmViews && e + c < nv &&
                   (hv[e + c].flags & kLinesAreRows) == (hv[e].flags & kLinesAreRows)) {
                sp.add(hv[e + c], mn, mx);
                if (BlockSpan::width(mn, mx) > bw) break;
                memcpy(sp.emin, mn, sizeof mn);
                memcpy(sp.emax, mx, sizeof mx);
                ++c;
            }
            bl.push_back(StBlock{e, c, hv[e].flags & kLinesAreRows, 0});
            e += c;
        }
        // worth it only when blocks share their windows among several views
        if (!fits || (int)bl.size() > 65535 || nv < 6 * (int)bl.size()) continue;
        if (bw == 128 && nv < 12 * (int)bl.size()) continue;   // 256 packs more views
        const std::vector<unsigned> order = st_cta_order(bl, hv, N, R);
        const size_t bb = sizeof(StBlock) * bl.size();
        RG_CK(cudaMalloc(&p.d_blocks, bb + sizeof(unsigned) * order.size()));
        RG_CK(cudaMemcpy(p.d_blocks, bl.data(), bb, cudaMemcpyHostToDevice));
        p.d_border = (const unsigned *)((char *)p.d_blocks + bb);
        RG_CK(cudaMemcpy((void *)p.d_border, order.data(), sizeof(unsigned) * order.size(),
                         cudaMemcpyHostToDevice));
        p.nblocks = (int)bl.size();
        p.st_bw = bw;
        return RG_OK;
    }
    return RG_OK;
}

EncodeTiledFn tensor_map_encoder()
{
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)f;
        else
            cudaGetLastError();
    });
    return fn;
}

// 3-D map over nz stacked line-pair arrays: (entry, line, image), 8-byte
// elements, box bw x box_lines x 1, zero fill outside.
static int encode_pairs_map(CUtensorMap *tm, const float2 *pairs, int N, int nz, long long zp,
                            int bw, int box_lines = kTmLines)
{
    EncodeTiledFn fn = tensor_map_encoder();
    if (!fn) return set_error(RG_ECUDA, "cuTensorMapEncodeTiled is not available");
    const int pitch = pairs_pitch(N);
    cuuint64_t dims[3] = {(cuuint64_t)pitch, (cuuint64_t)N, (cuuint64_t)nz};
    cuuint64_t strides[2] = {(cuuint64_t)pitch * 8,
                             (cuuint64_t)(nz > 1 ? zp : (long long)N * pitch) * 8};
    cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)box_lines, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, (void *)pairs, dims, strides, box,
                    estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return set_error(RG_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return RG_OK;
}

bool radon_tma_usable(const SSPlan &p)
{
    return p.nblocks > 0 && p.d_blocks && !radon_kernel_direct();
}

// Rays per shared load (lane layout); RG_RADON_RPL=32|16|8 overrides.
static int radon_rpl()
{
    const char *e = getenv("RG_RADON_RPL");
    const int v = e ? atoi(e) : 0;
    return (v == 32 || v == 16 || v == 8) ? v : 8;
}

// Cluster size of the strip split for a grid of `ctas` CTAs at `slots`
// resident CTAs.  Measured on GB300 with the CTAs dispatched longest first
// (GUPS, split 1 / 2 / 4; waves of the unsplit grid): 2048^2 x 1800 (8.1)
// 3462 / 3419 / 3195; 1536^2 x 1080 (3.6) 3297 / 3267 / 3036; 1024^2 x 1440
// (3.2) 2993 / 2945 / 2668; 1024^2 x 720 (1.6) 2862 / 2873-2895 / 2665;
// 512^2 x 360 (0.4) 916 / 1519 / 1628.  Each rank repeats the CTA's set-up
// and the ranks' partials meet in distributed shared memory, so a split pays
// only where the unsplit grid leaves SMs idle: 1 from 2.5 waves up, 2 from
// one wave, else 4, with at least 4 strips of kTmLines lines per rank.
// RG_RADON_SPLIT_TMA=1|2|4 forces it.
static int tma_pick_split(long long ctas, int slots, int N)
{
    const char *e = getenv("RG_RADON_SPLIT_TMA");
    const int forced = e ? atoi(e) : 0;
    if (forced == 1 || forced == 2 || forced == 4) return forced;
    int s = ctas >= 5LL * slots / 2 ? 1 : ctas >= slots ? 2 : 4;
    while (s > 1 && (N / kTmLines) / s < 4) s /= 2;
    return s;
}

template <int EPI, int BW, int RPL>
static int launch_tma_rpl(const SSPlan &p, const CUtensorMap &tr, const CUtensorMap &tc,
                          float *out_am, int out_ld, const float *y_am, int y_ld, int nz,
                          long long zo, int *d_err, cudaStream_t st)
{
    const size_t smem = (size_t)2 * kTmLines * BW * 8;
    auto k = k_radon_tma<EPI, BW, RPL>;
    RG_CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((p.g.R + kTmRays - 1) / kTmRays, p.nblocks, nz);
    // resident CTAs of this instantiation (cached: no queries in a capture)
    static int slots = 0;
    if (!slots) {
        int dev = 0, sms = 0, per = 0;
        RG_CK(cudaGetDevice(&dev));
        RG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        RG_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, 256, smem));
        slots = std::max(1, per) * sms;
    }
    const int split = tma_pick_split((long long)grid.x * grid.y * grid.z, slots, p.g.N);
    const int expire = test_switch("RG_TEST_EXPIRE_WAIT") ? 1 : 0;
    RG_CK(launch_pdl(k, dim3(grid.x * split, grid.y, grid.z), 256, smem, st, split,
                     tr, tc, p.g.N, (const View *)p.d_views,
                     (const StBlock *)p.d_blocks, p.d_border, p.g.R, out_am, out_ld, y_am,
                     y_ld, zo,
                     d_err, (unsigned)sizeof(float2), expire, split));
    RG_CK_LAUNCH("k_radon_tma");
    return RG_OK;
}

template <int EPI, int BW>
static int launch_tma_bw(const SSPlan &p, const CUtensorMap &tr, const CUtensorMap &tc,
                         float *out_am, int out_ld, const float *y_am, int y_ld, int nz,
                         long long zo, int *d_err, cudaStream_t st)
{
    switch (radon_rpl()) {
    case 32: return launch_tma_rpl<EPI, BW, 32>(p, tr, tc, out_am, out_ld, y_am, y_ld, nz, zo, d_err, st);
    case 16: return launch_tma_rpl<EPI, BW, 16>(p, tr, tc, out_am, out_ld, y_am, y_ld, nz, zo, d_err, st);
    default: return launch_tma_rpl<EPI, BW, 8>(p, tr, tc, out_am, out_ld, y_am, y_ld, nz, zo, d_err, st);
    }
}

template <int EPI>
static int launch_tma_epi(const SSPlan &p, const CUtensorMap &tr, const CUtensorMap &tc,
                          float *out_am, int out_ld, const float *y_am, int y_ld, int nz,
                          long long zo, int *d_err, cudaStream_t st)
{
    if (p.st_bw == 128)
        return launch_tma_bw<EPI, 128>(p, tr, tc, out_am, out_ld, y_am, y_ld, nz, zo, d_err, st);
    return launch_tma_bw<EPI, 256>(p, tr, tc, out_am, out_ld, y_am, y_ld, nz, zo, d_err, st);
}

int launch_radon_tma(const SSPlan &p, const float2 *prow, const float2 *pcol, float *out_am,
                     int out_ld, const float *y_am, int y_ld, cudaStream_t st, int nz,
                     long long zp, long long zo, int epi)
{
    CUtensorMap tr, tc;
    int rc = encode_pairs_map(&tr, prow, p.g.N, nz, zp, p.st_bw);
    if (!rc) rc = encode_pairs_map(&tc, pcol, p.g.N, nz, zp, p.st_bw);
    if (rc) return rc;
    int *d_err = device_error_word();
    if (epi == kEpiRatio)
        return launch_tma_epi<kEpiRatio>(p, tr, tc, out_am, out_ld, y_am, y_ld, nz, zo, d_err, st);
    if (epi == kEpiTransmission)
        return launch_tma_epi<kEpiTransmission>(p, tr, tc, out_am, out_ld, y_am, y_ld, nz, zo,
                                                d_err, st);
    return launch_tma_epi<kEpiSum>(p, tr, tc, out_am, out_ld, nullptr, 0, nz, zo, d_err, st);
}


// ============================================================================
// Tile-driven Radon for plans of scattered views (OSEM subsets).
//
// The view-block windows above need adjacent views; a subset's views are S
// apart, so their positions on a line spread too far for one window.  Here
// the loop order is turned around: a CTA owns an image tile -- kTtLines lines
// x kTtWin line-pair entries [p0, p0 + kTtWin) of one orientation -- staged
// once by TMA (one row copy per line, zero-filled outside the array), and
// every view of the plan with that orientation sends through it the rays
// that cross it.  Each staged entry then serves every view (tens to
// hundreds), not the few views of a block.
//
// Ownership: a sample (ray, line) belongs to the tile whose line block holds
// the line and whose window holds the sample's entry.  Each smem row carries
// kTtPad zero entries on both sides of the window, wide enough for any
// crossing ray's positions on the tile's lines (checked per plan on the host
// and per ray in the kernel), so a ray adds exactly its owned samples with
// the plain 7-instruction walk of the other kernels, and samples outside
// the window read zeros.  Each (ray, view, tile) partial, times Delta, is
// added to the sinogram with one atomic add (the zeroing pass before and
// the epilogue pass after are separate launches); the order of those adds
// varies between runs, at the level of FP32 rounding.

__global__ __launch_bounds__(256) void k_radon_tiles(const __grid_constant__ CUtensorMap tm_rows,
                                                     const __grid_constant__ CUtensorMap tm_cols,
                                                     int N, const TtView *__restrict__ ttv,
                                                     int n_rows,
                                                     int n_cols, int R,
                                                     float *__restrict__ out_am, int out_ld,
                                                     long long zo, int *__restrict__ err,
                                                     unsigned pb)
{
    pdl_gate();
    extern __shared__ __align__(128) float2 tile[];   // [kTtLines][kTtRow]
    __shared__ __align__(8) unsigned long long full;
    const int o = blockIdx.z & 1, z = blockIdx.z >> 1;
    const int nvo = o ? n_cols : n_rows;
    if (nvo == 0) return;                              // CTA-uniform, before any barrier
    const TtView *__restrict__ tv = ttv + (o ? n_rows : 0);
    const CUtensorMap *tm = o ? &tm_cols : &tm_rows;
    const int p0 = blockIdx.x * kTtWin, i0 = blockIdx.y * kTtLines;
    const unsigned sbase = smem_addr(tile);
    out_am += (long long)z * zo;

    if (threadIdx.x == 0) {
        mbar_init(smem_addr(&full), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // zero pads (the TMA rows fill the middle of each row)
    for (int e = threadIdx.x; e < kTtLines * 2 * kTtPad; e += blockDim.x) {
        const int r = e / (2 * kTtPad), c = e - r * (2 * kTtPad);
        tile[r * kTtRow + (c < kTtPad ? c : kTtWin + c)] = make_float2(0.f, 0.f);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        fence_proxy_async_smem();
        mbar_expect_tx(smem_addr(&full), kTtLines * kTtWin * 8);
        for (int r = 0; r < kTtLines; ++r)
            tma_load_3d(sbase + (r * kTtRow + kTtPad) * 8, tm, p0, i0 + r, z, smem_addr(&full));
    }
    const bool ok = mbar_wait(smem_addr(&full), 0);
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) {
            if (err) atomicOr(err, 2);
            mbar_wait(smem_addr(&full), 0);            // bounded: copies still in flight
        }
        return;
    }

    tt_views<kTtRow>(sbase, p0, i0, tv, nvo, R, out_am, out_ld, err, pb);
}

// out[view][k] = 0 (zeroing pass) or the epilogue of the summed rays, for
// the plan's views only.
template <int EPI, bool ZERO>
__global__ __launch_bounds__(256) void k_views_rows(const View *__restrict__ views, int nv, int R,
                                                    float *__restrict__ out_am, int out_ld,
                                                    const float *__restrict__ y_am, int y_ld,
                                                    long long zo)
{
    pdl_gate();
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (k >= R || j >= nv) return;
    const int view = views[j].view;
    float *o = out_am + (long long)blockIdx.z * zo + (size_t)view * out_ld + k;
    if (ZERO) *o = 0.f;
    else *o = radon_epilogue(EPI, *o, y_am, (size_t)view * y_ld + k);
}

bool tt_pads_fit(const SSPlan &p, int lines, int pad)
{
    return (lines - 1) * p.tt_ri_max + 3.0 * p.tt_rk_max + 3.0 <= pad;
}

int tt_build(SSPlan &p, const View *hv)
{
    p.tt_ok = false;
    p.n_ovid[0] = p.n_ovid[1] = 0;
    const int nv = p.nv;
    if (nv < 1) return RG_OK;
    std::vector<int> ids;
    for (int o = 0; o < 2; ++o)
        for (int e = 0; e < nv; ++e)
            if (((hv[e].flags & kLinesAreRows) ? 0 : 1) == o) {
                ids.push_back(e);
                ++p.n_ovid[o];
            }
    // pads must hold any crossing ray's positions on the tile's lines: the
    // walk across the tile's lines plus the margin rays (two each side)
    for (int e = 0; e < nv; ++e) {
        p.tt_ri_max = std::max(p.tt_ri_max, fabs((double)hv[e].ri) * 2.3283064365386963e-10);
        p.tt_rk_max = std::max(p.tt_rk_max, fabs((double)hv[e].rk) * 2.3283064365386963e-10);
    }
    if (!tt_pads_fit(p, kTtLines, kTtPad)) return RG_OK;
    std::vector<TtView> tv(ids.size());
    for (size_t q = 0; q < ids.size(); ++q) {
        const View &v = hv[ids[q]];
        tv[q].r0 = v.r0;
        tv[q].rk = v.rk;
        tv[q].ri = v.ri;
        tv[q].delta = v.delta;
        tv[q].view = v.view;
    }
    RG_CK(cudaMalloc(&p.d_ovid, sizeof(TtView) * tv.size()));
    RG_CK(cudaMemcpy(p.d_ovid, tv.data(), sizeof(TtView) * tv.size(), cudaMemcpyHostToDevice));
    p.tt_ok = true;
    return RG_OK;
}

bool radon_tiles_usable(const SSPlan &p)
{
    const char *e = getenv("RG_RADON_KERNEL");
    if (e && !strcmp(e, "direct")) return false;
    if (!p.tt_ok || !p.d_ovid) return false;
    if (e && !strcmp(e, "tiles")) return true;
    return !radon_tma_usable(p) && p.nv >= 16;
}

int launch_radon_tiles(const SSPlan &p, const float2 *prow, const float2 *pcol, float *out_am,
                       int out_ld, const float *y_am, int y_ld, cudaStream_t st, int nz,
                       long long zp, long long zo, int epi)
{
    const int N = p.g.N, R = p.g.R;
    CUtensorMap tr, tc;
    int rc = encode_pairs_map(&tr, prow, N, nz, zp, kTtWin, 1);
    if (!rc) rc = encode_pairs_map(&tc, pcol, N, nz, zp, kTtWin, 1);
    if (rc) return rc;
    const dim3 gv((R + 255) / 256, p.nv, nz);
    RG_CK(launch_pdl(k_views_rows<kEpiSum, true>, gv, 256, 0, st, 1, p.d_views, p.nv, R, out_am,
                     out_ld, nullptr, 0, zo));
    RG_CK_LAUNCH("k_views_rows (zero)");
    const size_t smem = (size_t)kTtLines * kTtRow * 8;
    RG_CK(cudaFuncSetAttribute(k_radon_tiles, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
    const dim3 grid((pairs_pitch(N) + kTtWin - 1) / kTtWin, (N + kTtLines - 1) / kTtLines,
                    2 * nz);
    RG_CK(launch_pdl(k_radon_tiles, grid, 256, smem, st, 1, tr, tc, N, (const TtView *)p.d_ovid,
                     p.n_ovid[0], p.n_ovid[1], R, out_am, out_ld, zo, device_error_word(),
                     (unsigned)sizeof(float2)));
    RG_CK_LAUNCH("k_radon_tiles");
    if (epi == kEpiRatio)
        RG_CK(launch_pdl(k_views_rows<kEpiRatio, false>, gv, 256, 0, st, 1, p.d_views, p.nv, R,
                         out_am, out_ld, y_am, y_ld, zo));
    else if (epi == kEpiTransmission)
        RG_CK(launch_pdl(k_views_rows<kEpiTransmission, false>, gv, 256, 0, st, 1, p.d_views,
                         p.nv, R, out_am, out_ld, y_am, y_ld, zo));
    RG_CK_LAUNCH("k_views_rows (epilogue)");
    return RG_OK;
}

}  // namespace rg
