// batch.cu -- batched uneven OSEM, and the plain one-slice-per-call form.
//
// Batched form (rg_osem_batch).  Many independent slices, each with its own
// image size N, view count A and rays R, run OSEM with interleaved subsets.
// One OSEM sub-iteration of ALL slices is, with the tile-driven Radon (the
// default):
//   1. zero the subset's rows of every slice's ratio buffer  (one CTA per row)
//   2. tile-driven Radon, line pairs formed while staging    (items: slice x
//      orientation x image tile of 16 lines x 160 entries)
//   3. ratio y / (A x) of those rows                          (one CTA per row)
//   4. matched adjoint + EM update                            (items: slice x
//      tile of 32 x 128 pixels)
//   5. the adjoint's edge pixels                              (one warp each)
// and, with the direct walks (RG_RADON_KERNEL=direct, or a geometry whose
// pads do not fit), line pairs of every iterate, then a Radon with the ratio
// fused (items: slice x 8 views x 32 rays), then steps 4 and 5.
// Persistent launches size their grid to the resident-CTA capacity of the GPU; every
// CTA pulls work items from one atomic counter until the list is exhausted,
// so slices of very different cost share the SMs without tail effects.
// Slices are ordered by decreasing cost, so the largest items are taken
// first.  Item -> (slice, tile) uses a binary search over per-slice prefix
// offsets.  The counters are reset by memset nodes before each launch, so
// one sub-iteration sequence is captured once into a CUDA graph and the
// graph is replayed for every iteration (no per-iteration host work).
//
// Plain form (rg_em_plain_host).  What one slice costs when handled the way
// the reference's GPU EM does it (raft/raft_em_gpu.cu:20-87): allocate and
// upload per call, then per sub-iteration a Radon launch, a ratio launch, a
// backprojection launch, a divide launch and a multiply launch, each
// followed by a device synchronisation (raft/raft_radon_gpu_function.cu:152,
// raft/raft_backprojection_gpu_function.cu:106), then download and free.
// Its kernels are one thread per output with float positions and global
// loads, no staging and no fusion; they compute the same operators as the
// batched path (slant-stack Radon, matched adjoint) so both reconstruct the
// same iterate.
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "ss_tiles.cuh"

namespace rg {

namespace {

struct BatchSlice {
    const View *views;     // this subset's per-view constants
    int nv, N, R;
    const float *y_am;     // measured sinogram, view-major (A x R)
    float *ratio_am;       // ratio / ones buffer (A x R)
    float2 *prow, *pcol;   // line pairs of the iterate
    float *x;              // iterate, N x N contiguous
    float *inv_sens;       // 1 / A_s^T 1 of this subset, N x N
    const TtView *ttv;     // tile-driven Radon: per-view records by orientation
    int n_rows, n_cols;
    int begin[8];          // first item of this slice in each work list
};

// Work lists: kGather holds every slice's gather tiles (the sensitivities),
// kAdj those of the slices whose adjoint runs tile by tile, kMirror the
// tile pairs of the slices whose adjoint pairs each tile with its half-turn
// mirror (gather_tile_mirror).
enum { kLP = 0, kRadon = 1, kGather = 2, kEdges = 3, kTiles = 4, kRows = 5, kAdj = 6,
       kMirror = 7 };

__device__ __forceinline__ int find_slice(const BatchSlice *__restrict__ d, int n, int item, int w)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (d[mid].begin[w] <= item) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Pull the next item (CTA-uniform).
__device__ __forceinline__ int next_item(int *counter)
{
    __shared__ int s_item;
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    return it;
}

__global__ __launch_bounds__(256) void k_batch_pairs(const BatchSlice *__restrict__ d, int n,
                                                     int total, int *counter)
{
    for (;;) {
        const int item = next_item(counter);
        if (item >= total) break;
        const BatchSlice &b = d[find_slice(d, n, item, kLP)];
        const int local = item - b.begin[kLP], tiles = (b.N + 31) / 32;
        line_pairs_tile(b.x, b.N, 1, b.N, b.prow, b.pcol, local % tiles, local / tiles);
    }
}

// VPT: views per thread (radon_tile with 4 views per CTA, or radon_tile2 with 8).
template <int VPT>
__global__ __launch_bounds__(128) void k_batch_radon(const BatchSlice *__restrict__ d, int n,
                                                     int total, int *counter)
{
    for (;;) {
        const int item = next_item(counter);
        if (item >= total) break;
        const BatchSlice &b = d[find_slice(d, n, item, kRadon)];
        const int local = item - b.begin[kRadon], rb = (b.R + 31) / 32;
        if (VPT == 2)
            radon_tile2<kEpiRatio, 16>(b.prow, b.pcol, b.N, b.views, b.nv, b.R, b.ratio_am, b.R, b.y_am,
                              b.R, local % rb, local / rb);
        else
            radon_tile<kEpiRatio>(b.prow, b.pcol, b.N, b.views, b.nv, b.R, b.ratio_am, b.R, b.y_am,
                             b.R, local % rb, local / rb);
    }
}

// Tile-driven Radon of one subset for every slice (tt_views, ss_tiles.cuh):
// items are slice x orientation x tile; a CTA stages the tile (kBtLines
// lines x kTtWin line-pair entries, with zero pads) -- one staging serves
// every view of the subset with that orientation -- and adds each crossing
// ray's partial to the slice's ratio buffer atomically.  The line pairs are
// formed while staging, straight from the iterate x (N x N, row-major): an
// image-row line reads consecutive floats of one row, an image-column line
// reads a 32-column strip row by row, both coalesced.  Rows of the staged
// tile are kTtRowB = kTtRow + 1 entries apart, so the column-strip staging
// (consecutive threads on consecutive lines) hits distinct banks.
// 16-line batch tiles (28.8 KB) let five CTAs share an SM where 32-line
// tiles allowed three, to hide the staging latency: 1.3 % faster measured.
constexpr int kBtLines = 16;                             // lines per batch tile
constexpr int kBtPad = 32;                               // checked per plan (tt_pads_fit)
constexpr int kTtRowB = kTtWin + 2 * kBtPad + 1;

__global__ __launch_bounds__(256) void k_batch_tiles(const BatchSlice *__restrict__ d, int n,
                                                     int total, int *counter, int *err,
                                                     unsigned pb)
{
    extern __shared__ __align__(128) float2 tile[];   // [kBtLines][kTtRowB]
    static_assert(kBtLines == 16 && kTtWin % 32 == 0 && kTtWin % 16 == 0, "staging layout");
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(tile);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // The pads stay zero for the kernel's life: items rewrite the window only.
    for (int e = threadIdx.x; e < kBtLines * kTtRowB; e += blockDim.x)
        tile[e] = make_float2(0.f, 0.f);
    for (;;) {
        const int item = next_item(counter);          // its barriers also end the last item
        if (item >= total) break;
        const BatchSlice &b = d[find_slice(d, n, item, kTiles)];
        const int local = item - b.begin[kTiles];
        const int N = b.N, pitch = pairs_pitch(N);
        const int tx = (pitch + kTtWin - 1) / kTtWin, ty = (N + kBtLines - 1) / kBtLines;
        const int o = local / (tx * ty), rem = local - o * (tx * ty);
        const int p0 = (rem % tx) * kTtWin, i0 = (rem / tx) * kBtLines;
        const int nvo = o ? b.n_cols : b.n_rows;
        if (nvo == 0) continue;                        // CTA-uniform
        const float *__restrict__ x = b.x;
        // Window entry c of tile line r holds the pair of sample p0 + c - 1 of
        // line i0 + r, read once per sample.
        if (o == 0) {
            // along image rows: warp w stages lines w, w + 8, lanes along the
            // row (coalesced); the next sample comes from the next lane, and
            // lane 31 reads its own
            for (int r = warp; r < kBtLines; r += kWarps) {
                const int line = i0 + r;
                const bool lv = line < N;
                const float *__restrict__ xr = x + (size_t)(lv ? line : 0) * N;
#pragma unroll 1
                for (int c0 = 0; c0 < kTtWin; c0 += 32) {
                    const int smp = p0 + c0 + lane - 1;
                    const float s0 = (lv && smp >= 0 && smp < N) ? __ldg(xr + smp) : 0.f;
                    float s1 = __shfl_down_sync(0xffffffffu, s0, 1);
                    if (lane == 31) s1 = (lv && smp + 1 < N) ? __ldg(xr + smp + 1) : 0.f;
                    tile[r * kTtRowB + kBtPad + c0 + lane] =
                        make_pair(s0, s1, lv && smp >= 0 && smp <= N - 2);
                }
            }
        } else {
            // across a column strip: thread (line t % 16, group t / 16) stages
            // the group's entries in order, keeping the previous sample;
            // 16 consecutive lines are 16 consecutive floats of x
            constexpr int per = kTtWin / 16;
            const int r = threadIdx.x & 15, cb = (threadIdx.x >> 4) * per;
            const int line = i0 + r;
            const bool lv = line < N;
            int smp = p0 + cb - 1;
            float s0 = (lv && smp >= 0 && smp < N) ? __ldg(x + (size_t)smp * N + line) : 0.f;
#pragma unroll 2
            for (int j = 0; j < per; ++j) {
                const int sn = smp + 1;
                const float s1 = (lv && sn >= 0 && sn < N) ? __ldg(x + (size_t)sn * N + line) : 0.f;
                tile[r * kTtRowB + kBtPad + cb + j] = make_pair(s0, s1, lv && smp >= 0 && smp <= N - 2);
                s0 = s1;
                smp = sn;
            }
        }
        __syncthreads();
        tt_views<kTtRowB, kBtLines, kBtPad>(sbase, p0, i0, b.ttv + (o ? b.n_rows : 0), nvo, b.R,
                                            b.ratio_am, b.R, err, pb);
    }
}

// The subset's rows of every slice's ratio buffer (one CTA per row): zeroed
// before the tile-driven Radon, or turned into the EM ratio y / (A x)
// (0 where A x == 0) after it.
template <bool ZERO>
__global__ __launch_bounds__(256) void k_batch_rows(const BatchSlice *__restrict__ d, int n)
{
    const int item = blockIdx.x;
    const BatchSlice &b = d[find_slice(d, n, item, kRows)];
    const int view = b.views[item - b.begin[kRows]].view;
    float *__restrict__ o = b.ratio_am + (size_t)view * b.R;
    const float *__restrict__ y = b.y_am + (size_t)view * b.R;
    for (int k = threadIdx.x; k < b.R; k += blockDim.x)
        o[k] = ZERO ? 0.f : radon_epilogue(kEpiRatio, o[k], y, k);
}

// MODE 1: adjoint with the EM update; MODE 2: FP64 sensitivity -> inv_sens.
// Tiles are 32 columns x 8*kBatchRows rows.
// 16 rows per thread measured 2 % faster than 8 on the config-5 batch with
// Kahan-compensated sums, and 6 % faster (37.8 against 35.5 slices/s)
// once the sums went straight into the accumulators.
constexpr int kBatchRows = 16;

template <int MODE, int WMAX>
__global__ __launch_bounds__(256) void k_batch_gather(const BatchSlice *__restrict__ d, int n,
                                                      int total, int *counter,
                                                      unsigned pair_bytes)
{
    extern __shared__ float2 pairs[];
    for (;;) {
        const int item = next_item(counter);
        if (item >= total) break;
        constexpr int kList = MODE == 1 ? kAdj : kGather;
        const BatchSlice &b = d[find_slice(d, n, item, kList)];
        const int local = item - b.begin[kList], tiles = (b.N + 31) / 32;
        if (MODE == 1)
            gather_tile<1, WMAX, kBatchRows, true, false>(b.ratio_am, b.R, b.R, b.views, b.nv,
                                                          b.N, 1.f, nullptr, 0, 0, b.x,
                                                          b.inv_sens, nullptr, local % tiles,
                                                          local / tiles, pairs, pair_bytes, 1,
                                                          0, true);
        else
            gather_tile<2, WMAX, kBatchRows, false>(b.ratio_am, b.R, b.R, b.views, b.nv, b.N, 1.f,
                                                    b.inv_sens, b.N, 1, nullptr, nullptr, nullptr,
                                                    local % tiles, local / tiles, pairs,
                                                    pair_bytes, 1, 0, true);
    }
}

// Adjoint + EM update of the slices with mirrored tile pairs
// (gather_tile_mirror): items are slice x tile pairs, tile (tx, ty) of the
// upper half of the tile rows with its half-turn mirror.
// 16 rows per thread, registers held to 64 for four CTAs per SM: 44.7
// slices/s on the config-5 batch, against 32.3 with the compiler's 73
// registers (three CTAs per SM) and 37.3 with 8-row tiles (58 registers).
constexpr int kMirrorRows = 16;
template <int WMAX>
__global__ __launch_bounds__(256, 4) void k_batch_mirror(const BatchSlice *__restrict__ d, int n,
                                                      int total, int *counter,
                                                      unsigned quad_bytes)
{
    extern __shared__ __align__(16) float4 mquads[];
    for (;;) {
        const int item = next_item(counter);
        if (item >= total) break;
        const BatchSlice &b = d[find_slice(d, n, item, kMirror)];
        const int local = item - b.begin[kMirror], tiles = b.N / 32;
        gather_tile_mirror<WMAX, kMirrorRows, true>(b.ratio_am, b.R, b.R, b.views, b.nv, b.N,
                                                   nullptr, 0, 0, b.x, b.inv_sens, nullptr,
                                                   local % tiles, local / tiles, mquads,
                                                   quad_bytes);
    }
}

// Edge pixels left out by k_batch_gather (adjoint_edge_group): one CTA per
// 32 consecutive edge pixels of a slice (items: slice x groups of 32 of its
// 4N - 4 edge pixels).
template <int MODE>
__global__ __launch_bounds__(256) void k_batch_edges(const BatchSlice *__restrict__ d, int n,
                                                     int total)
{
    const int item = blockIdx.x;
    if (item >= total) return;        // CTA-uniform
    const BatchSlice &b = d[find_slice(d, n, item, kEdges)];
    const int e0 = (item - b.begin[kEdges]) * 32;
    if (MODE == 1)
        adjoint_edge_group<1, true, 8>(b.ratio_am, b.R, b.R, b.views, b.nv, b.N, e0, nullptr, 0, 0,
                                    b.x, b.inv_sens);
    else
        adjoint_edge_group<2, false, 8>(b.ratio_am, b.R, b.R, b.views, b.nv, b.N, e0, b.inv_sens, b.N,
                                     1, nullptr, nullptr);
}

// RG_BATCH_MIRROR=0: every slice's adjoint runs tile by tile (gather_tile),
// also where its tiles pair with their half-turn mirrors (A/B timing).
bool batch_mirror_enabled()
{
    const char *e = getenv("RG_BATCH_MIRROR");
    return !(e && !strcmp(e, "0"));
}

// Grid of a persistent launch: resident capacity, capped by the item count.
template <class K>
int persistent_grid(K kernel, int threads, size_t smem, int items, int *out)
{
    int dev = 0, sms = 0, per = 0;
    RG_CK(cudaGetDevice(&dev));
    RG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    RG_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem));
    *out = std::max(1, std::min(items, sms * std::max(per, 1)));
    return RG_OK;
}

struct BatchRun {
    int n = 0, S = 0, wmax = 64, vpt = 2;
    bool tiles = false;               // tile-driven Radon (else the direct walks)
    int total[8][64] = {};            // [kind][subset] item counts (subset 0 for pairs)
    int grid[6][64] = {};             // persistent grids: pairs, radon[s], gather1, gather2, tiles,
                                      // mirror
    BatchSlice *d_desc = nullptr;     // S x n descriptors (device, in scratch)
    int *counter = nullptr;
};

// Grid sizes of every launch, computed before any stream capture.
template <int WMAX>
int prepare_grids(BatchRun &br)
{
    const size_t smem = (size_t)kSlots * WMAX * sizeof(float2);
    if (int rc = persistent_grid(k_batch_pairs, 256, 0, br.total[kLP][0], &br.grid[0][0])) return rc;
    if (br.tiles)
        if (int rc = persistent_grid(k_batch_tiles, 256, (size_t)kBtLines * kTtRowB * 8,
                                     br.total[kTiles][0], &br.grid[4][0]))
            return rc;
    for (int s = 0; s < br.S; ++s)
        if (int rc = persistent_grid(br.vpt == 2 ? k_batch_radon<2> : k_batch_radon<1>, 128, 0,
                                     br.total[kRadon][s], &br.grid[1][s]))
            return rc;
    if (br.total[kMirror][0])
        if (int rc = persistent_grid(k_batch_mirror<WMAX>, 256, smem, br.total[kMirror][0],
                                     &br.grid[5][0]))
            return rc;
    if (int rc = persistent_grid(k_batch_gather<1, WMAX>, 256, smem, br.total[kAdj][0],
                                 &br.grid[2][0]))
        return rc;
    return persistent_grid(k_batch_gather<2, WMAX>, 256, smem, br.total[kGather][0],
                           &br.grid[3][0]);
}

template <int WMAX>
int enqueue_iteration(const BatchRun &br, cudaStream_t st)
{
    const size_t smem = (size_t)kSlots * WMAX * sizeof(float2);
    for (int s = 0; s < br.S; ++s) {
        const BatchSlice *d = br.d_desc + (size_t)s * br.n;
        if (!br.tiles) {   // the tile-driven Radon forms its line pairs while staging
            RG_CK(cudaMemsetAsync(br.counter, 0, sizeof(int), st));
            k_batch_pairs<<<br.grid[0][0], 256, 0, st>>>(d, br.n, br.total[kLP][0], br.counter);
            RG_CK_LAUNCH("k_batch_pairs");
        }
        if (br.tiles) {
            k_batch_rows<true><<<br.total[kRows][s], 256, 0, st>>>(d, br.n);
            RG_CK_LAUNCH("k_batch_rows (zero)");
            RG_CK(cudaMemsetAsync(br.counter, 0, sizeof(int), st));
            k_batch_tiles<<<br.grid[4][0], 256, (size_t)kBtLines * kTtRowB * 8, st>>>(
                d, br.n, br.total[kTiles][0], br.counter, device_error_word(),
                (unsigned)sizeof(float2));
            RG_CK_LAUNCH("k_batch_tiles");
            k_batch_rows<false><<<br.total[kRows][s], 256, 0, st>>>(d, br.n);
            RG_CK_LAUNCH("k_batch_rows (ratio)");
        } else {
            RG_CK(cudaMemsetAsync(br.counter, 0, sizeof(int), st));
            if (br.vpt == 2)
                k_batch_radon<2><<<br.grid[1][s], 128, 0, st>>>(d, br.n, br.total[kRadon][s],
                                                                br.counter);
            else
                k_batch_radon<1><<<br.grid[1][s], 128, 0, st>>>(d, br.n, br.total[kRadon][s],
                                                                br.counter);
            RG_CK_LAUNCH("k_batch_radon");
        }
        RG_CK(cudaMemsetAsync(br.counter, 0, sizeof(int), st));
        if (br.total[kMirror][0]) {
            k_batch_mirror<WMAX><<<br.grid[5][0], 256, smem, st>>>(d, br.n, br.total[kMirror][0],
                                                                   br.counter,
                                                                   (unsigned)sizeof(float4));
            RG_CK_LAUNCH("k_batch_mirror");
            RG_CK(cudaMemsetAsync(br.counter, 0, sizeof(int), st));
        }
        if (br.total[kAdj][0]) {
            k_batch_gather<1, WMAX><<<br.grid[2][0], 256, smem, st>>>(d, br.n, br.total[kAdj][0],
                                                                      br.counter,
                                                                      (unsigned)sizeof(float2));
            RG_CK_LAUNCH("k_batch_gather<1>");
        }
        k_batch_edges<1><<<br.total[kEdges][0], 256, 0, st>>>(d, br.n, br.total[kEdges][0]);
        RG_CK_LAUNCH("k_batch_edges<1>");
    }
    return RG_OK;
}

template <int WMAX>
int enqueue_sensitivity(const BatchRun &br, cudaStream_t st)
{
    const size_t smem = (size_t)kSlots * WMAX * sizeof(float2);
    for (int s = 0; s < br.S; ++s) {
        const BatchSlice *d = br.d_desc + (size_t)s * br.n;
        RG_CK(cudaMemsetAsync(br.counter, 0, sizeof(int), st));
        k_batch_gather<2, WMAX><<<br.grid[3][0], 256, smem, st>>>(d, br.n, br.total[kGather][0],
                                                                  br.counter,
                                                                  (unsigned)sizeof(float2));
        RG_CK_LAUNCH("k_batch_gather<2>");
        k_batch_edges<2><<<br.total[kEdges][0], 256, 0, st>>>(d, br.n, br.total[kEdges][0]);
        RG_CK_LAUNCH("k_batch_edges<2>");
    }
    return RG_OK;
}

template <int WMAX>
int set_smem_attrs()
{
    const int smem = kSlots * WMAX * (int)sizeof(float2);
    RG_CK(cudaFuncSetAttribute(k_batch_gather<1, WMAX>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    RG_CK(cudaFuncSetAttribute(k_batch_gather<2, WMAX>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    RG_CK(cudaFuncSetAttribute(k_batch_mirror<WMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               smem));
    RG_CK(cudaFuncSetAttribute(k_batch_tiles, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               kBtLines * kTtRowB * 8));
    return RG_OK;
}

int dispatch_iteration(const BatchRun &br, cudaStream_t st)
{
    switch (br.wmax) {
    case 64: return enqueue_iteration<64>(br, st);
    case 128: return enqueue_iteration<128>(br, st);
    case 160: return enqueue_iteration<160>(br, st);
    case 256: return enqueue_iteration<256>(br, st);
    default: return enqueue_iteration<512>(br, st);
    }
}

int dispatch_sensitivity(const BatchRun &br, cudaStream_t st)
{
    switch (br.wmax) {
    case 64: return enqueue_sensitivity<64>(br, st);
    case 128: return enqueue_sensitivity<128>(br, st);
    case 160: return enqueue_sensitivity<160>(br, st);
    case 256: return enqueue_sensitivity<256>(br, st);
    default: return enqueue_sensitivity<512>(br, st);
    }
}

int dispatch_attrs(BatchRun &br)
{
    switch (br.wmax) {
    case 64: { int rc = set_smem_attrs<64>(); return rc ? rc : prepare_grids<64>(br); }
    case 128: { int rc = set_smem_attrs<128>(); return rc ? rc : prepare_grids<128>(br); }
    case 160: { int rc = set_smem_attrs<160>(); return rc ? rc : prepare_grids<160>(br); }
    case 256: { int rc = set_smem_attrs<256>(); return rc ? rc : prepare_grids<256>(br); }
    default: { int rc = set_smem_attrs<512>(); return rc ? rc : prepare_grids<512>(br); }
    }
}

struct SliceBuf {
    size_t y, ratio, pairs, x, inv;   // byte sizes of this slice's pieces
};

SliceBuf slice_bytes(const rg_image &s, const rg_image &i, int S)
{
    SliceBuf b;
    b.y = b.ratio = (size_t)s.lines * s.columns * sizeof(float);
    b.pairs = radon_pairs_bytes(i.lines);
    b.x = (size_t)i.lines * i.lines * sizeof(float);
    b.inv = b.x * S;
    return b;
}

}  // namespace

// ============================================================================
// Plain per-call form

namespace {

struct PlainView {
    float rk, ri, r0, delta;       // Radon position along line i of ray k
    float krow, kcol, k0, P;       // adjoint ray-index position of pixel
    int flags, view, pad0, pad1;
};

// One thread per (ray, subset view); float positions; global loads.
__global__ void k_plain_radon(const float *__restrict__ x, int N, const PlainView *__restrict__ v,
                              int nv, int R, int A, float *__restrict__ ax)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x, e = blockIdx.y;
    if (k >= R || e >= nv) return;
    const PlainView pv = v[e];
    const bool rows = pv.flags & kLinesAreRows;
    float acc = 0.f;
    for (int i = 0; i < N; ++i) {
        const float u = pv.r0 + k * pv.rk + i * pv.ri;
        const float fm = floorf(u);
        const int m = (int)fm;
        if (m >= 0 && m <= N - 2) {
            const float w = u - fm;
            const float f0 = rows ? x[(size_t)i * N + m] : x[(size_t)m * N + i];
            const float f1 = rows ? x[(size_t)i * N + m + 1] : x[(size_t)(m + 1) * N + i];
            acc += f0 + w * (f1 - f0);
        }
    }
    ax[(size_t)k * A + pv.view] = acc * pv.delta;
}

__global__ void k_plain_ratio(const float *__restrict__ y, float *__restrict__ r, size_t n)
{
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e < n) r[e] = (r[e] != 0.f) ? y[e] / r[e] : 0.f;
}

// One thread per pixel; loops over the subset views; matched-adjoint weights.
__global__ void k_plain_adjoint(const float *__restrict__ s, int R, int A,
                                const PlainView *__restrict__ v, int nv, int N,
                                float *__restrict__ out)
{
    const int col = blockIdx.x * blockDim.x + threadIdx.x, row = blockIdx.y;
    if (col >= N) return;
    float acc = 0.f;
    for (int e = 0; e < nv; ++e) {
        const PlainView pv = v[e];
        const float kap = pv.k0 + row * pv.krow + col * pv.kcol;
        const float fk = floorf(kap);
        const int k0 = (int)fk;
        const float f = kap - fk;
        float wa = fmaxf(0.f, 1.f - pv.P * f), wb = fmaxf(0.f, 1.f - pv.P * (1.f - f));
        const bool pneg = pv.flags & kRkNegative;
        const int m = (pv.flags & kLinesAreRows) ? col : row;
        if (m == 0) { if (!pneg && f > 0.f) wa = 0.f; if (pneg) wb = 0.f; }
        else if (m == N - 1) { if (pneg || f == 0.f) wa = 0.f; if (!pneg) wb = 0.f; }
        const float s0 = (k0 >= 0 && k0 < R) ? s[(size_t)k0 * A + pv.view] : 0.f;
        const float s1 = (k0 + 1 >= 0 && k0 + 1 < R) ? s[(size_t)(k0 + 1) * A + pv.view] : 0.f;
        acc += pv.delta * (s0 * wa + s1 * wb);
    }
    out[(size_t)row * N + col] = acc;
}

__global__ void k_plain_div(const float *__restrict__ a, const float *__restrict__ b,
                            float *__restrict__ o, size_t n)
{
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e < n) o[e] = (b[e] != 0.f) ? a[e] / b[e] : 0.f;
}

__global__ void k_plain_mul(float *__restrict__ x, const float *__restrict__ a, size_t n)
{
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e < n) x[e] *= a[e];
}

}  // namespace

}  // namespace rg

using namespace rg;

extern "C" {

size_t rg_osem_batch_workspace(const rg_image *sinos, const rg_image *images, int nslices,
                               int nsubsets)
{
    const int S = std::max(1, nsubsets);
    size_t t = Scratch::align(sizeof(int)) + Scratch::align(sizeof(BatchSlice) * S * nslices);
    for (int k = 0; k < nslices; ++k) {
        const SliceBuf b = slice_bytes(sinos[k], images[k], S);
        t += Scratch::align(b.y) + Scratch::align(b.ratio) + 2 * Scratch::align(b.pairs) +
             Scratch::align(b.x) + Scratch::align(b.inv);
    }
    return t;
}

int rg_osem_batch(const rg_image *sinos, rg_image *images, int nslices, int niter, int nsubsets,
                  int graph, void *ws, size_t wsb, void *stream)
{
    RG_TRACE();
    if (nslices < 0 || (nslices > 0 && (!sinos || !images)))
        return set_error(RG_EINVAL, "rg_osem_batch: bad slice arrays");
    if (niter < 0) return set_error(RG_EINVAL, "rg_osem_batch: niter < 0");
    if (nsubsets < 1 || nsubsets > 64)
        return set_error(RG_EINVAL, "rg_osem_batch: nsubsets must be in [1, 64]");
    if (int rc = check_ws(ws)) return rc;
    if (nslices == 0) return RG_OK;
    const int S = nsubsets;
    for (int k = 0; k < nslices; ++k) {
        if (int rc = validate_ss(images[k], sinos[k])) return rc;
        if (sinos[k].columns < S)
            return set_error(RG_EINVAL, "slice %d: fewer views (%d) than subsets (%d)", k,
                             sinos[k].columns, S);
    }
    cudaStream_t st = (cudaStream_t)stream;

    // Plans per (slice, subset); order slices by decreasing cost.
    std::vector<int> order(nslices);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const double ca = (double)images[a].lines * images[a].lines * sinos[a].columns;
        const double cb = (double)images[b].lines * images[b].lines * sinos[b].columns;
        return ca > cb;
    });
    std::vector<void *> holders;
    struct HolderGuard {
        std::vector<void *> &h;
        ~HolderGuard() { for (void *p : h) release_holder(p); }
    } guard{holders};
    std::vector<const SSPlan *> plans((size_t)nslices * S);
    int wneed = 0;
    for (int q = 0; q < nslices; ++q) {
        const int k = order[q];
        const SSGeom g = make_ss_geom(images[k], sinos[k]);
        for (int s = 0; s < S; ++s) {
            void *h = nullptr;
            if (int rc = get_ss_plan(g, S, s, &plans[(size_t)q * S + s], &h)) return rc;
            holders.push_back(h);
            const SSPlan *p = plans[(size_t)q * S + s];
            if (!p->adj_ok)
                return set_error(RG_EUNSUPPORTED, "slice %d: nrays must not exceed the image size", k);
            wneed = std::max(wneed, p->wmax_adj[kBatchRows == 16 ? 2 : kBatchRows == 8 ? 1 : 0]);
        }
    }
    BatchRun br;
    br.n = nslices;
    br.S = S;
    // two views per thread with a 16-deep unroll: the batch has parallelism
    // to spare, so more loads in flight per thread beat occupancy
    // (RG_RADON_VIEWS=1|2 overrides)
    br.vpt = getenv("RG_RADON_VIEWS") ? radon_views_per_thread(*plans[0]) : 2;
    const int vpb = br.vpt == 2 ? 8 : 4;   // views per Radon item
    // tile-driven Radon when every subset plan supports it (its pads cover
    // the geometry); RG_RADON_KERNEL=direct keeps the direct walks
    {
        const char *e = getenv("RG_RADON_KERNEL");
        br.tiles = !(e && !strcmp(e, "direct"));
        for (const SSPlan *p : plans)
            br.tiles = br.tiles && p->tt_ok && p->d_ovid && tt_pads_fit(*p, kBtLines, kBtPad);
    }
    // 160 entries (40 KB of windows) covers 16-row tiles whenever rays are no
    // denser than pixels (window <= 31 + 127 sample units + 3), and leaves
    // room for five CTAs per SM where 256 (64 KB) allows three.
    br.wmax = wneed <= 64 ? 64 : wneed <= 128 ? 128 : wneed <= 160 ? 160 : wneed <= 256 ? 256 : 512;
    if (wneed > 512) return set_error(RG_EUNSUPPORTED, "gather window of %d exceeds 512", wneed);

    Scratch sc;
    if (int rc = scratch_begin(sc, ws, wsb, rg_osem_batch_workspace(sinos, images, nslices, S), st))
        return rc;
    int rc = RG_OK;
    br.counter = (int *)sc.take(sizeof(int));
    br.d_desc = (BatchSlice *)sc.take(sizeof(BatchSlice) * S * nslices);
    std::vector<BatchSlice> hd((size_t)S * nslices);
    int items_lp = 0, items_g = 0, items_e = 0, items_t = 0, items_a = 0, items_m = 0;
    std::vector<int> items_r(S, 0), items_rows(S, 0);
    std::vector<float *> xs(nslices);
    for (int q = 0; q < nslices && !rc; ++q) {
        const int k = order[q];
        const rg_image &si = sinos[k];
        const rg_image &im = images[k];
        const SliceBuf b = slice_bytes(si, im, S);
        const int N = im.lines, R = si.lines, A = si.columns;
        float *y = (float *)sc.take(b.y);
        float *ratio = (float *)sc.take(b.ratio);
        float2 *prow = (float2 *)sc.take(b.pairs);
        float2 *pcol = (float2 *)sc.take(b.pairs);
        float *x = (float *)sc.take(b.x);
        float *inv = (float *)sc.take(b.inv);
        xs[q] = x;
        rc = launch_to_am(si.data, si.column_stride, si.line_stride, R, A, y, st);
        if (!rc) rc = launch_copy2d(im.data, im.column_stride, im.line_stride, x, N, 1, N, N, st);
        if (!rc) rc = launch_fill(ratio, (size_t)R * A, 1.f, st);
        const int tiles = (N + 31) / 32, tiles_y = (N + 8 * kBatchRows - 1) / (8 * kBatchRows);
        // mirrored tile pairs: a symmetric geometry whose tiles pair up
        // (every subset plan of the slice shares its geometry)
        const bool mirror = batch_mirror_enabled() && plans[(size_t)q * S]->mirror_ok &&
                            N % 64 == 0 && N % (16 * kMirrorRows) == 0;
        const int tiles_m = N / (8 * kMirrorRows);
        for (int s = 0; s < S; ++s) {
            BatchSlice &d = hd[(size_t)s * nslices + q];
            const SSPlan *p = plans[(size_t)q * S + s];
            d.views = p->d_views;
            d.nv = p->nv;
            d.N = N;
            d.R = R;
            d.y_am = y;
            d.ratio_am = ratio;
            d.prow = prow;
            d.pcol = pcol;
            d.x = x;
            d.inv_sens = inv + (size_t)s * N * N;
            d.begin[kLP] = items_lp;
            d.begin[kRadon] = items_r[s];
            d.begin[kGather] = items_g;
            d.begin[kAdj] = items_a;
            d.begin[kMirror] = items_m;
            d.begin[kEdges] = items_e;
            d.begin[kTiles] = items_t;
            d.begin[kRows] = items_rows[s];
            d.ttv = (const TtView *)p->d_ovid;
            d.n_rows = p->n_ovid[0];
            d.n_cols = p->n_ovid[1];
            items_rows[s] += p->nv;
            items_r[s] += ((R + 31) / 32) * ((p->nv + vpb - 1) / vpb);
        }
        items_lp += tiles * tiles;
        items_g += tiles * tiles_y;
        if (mirror) items_m += tiles * tiles_m / 2;
        else items_a += tiles * tiles_y;
        items_e += (4 * N - 4 + 31) / 32;
        items_t += 2 * ((pairs_pitch(N) + kTtWin - 1) / kTtWin) * ((N + kBtLines - 1) / kBtLines);
    }
    br.total[kLP][0] = items_lp;
    br.total[kGather][0] = items_g;
    br.total[kAdj][0] = items_a;
    br.total[kMirror][0] = items_m;
    br.total[kEdges][0] = items_e;
    br.total[kTiles][0] = items_t;
    for (int s = 0; s < S; ++s) br.total[kRows][s] = items_rows[s];
    for (int s = 0; s < S; ++s) br.total[kRadon][s] = items_r[s];
    if (!rc) {
        cudaError_t e = cudaMemcpyAsync(br.d_desc, hd.data(), sizeof(BatchSlice) * hd.size(),
                                        cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) rc = cuda_error(e, "batch descriptors upload");
    }
    if (!rc) rc = dispatch_attrs(br);
    if (!rc) rc = dispatch_sensitivity(br, st);

    if (!rc && niter > 0) {
        if (graph) {
            // Capture one iteration on a private stream, replay it niter times.
            cudaStream_t cs = nullptr;
            cudaGraph_t gr = nullptr;
            cudaGraphExec_t ge = nullptr;
            cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
            if (e != cudaSuccess) rc = cuda_error(e, "cudaStreamCreate");
            if (!rc && (e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
                rc = cuda_error(e, "cudaStreamBeginCapture");
            if (!rc) {
                int rc2 = dispatch_iteration(br, cs);
                e = cudaStreamEndCapture(cs, &gr);
                rc = rc2 ? rc2 : (e != cudaSuccess ? cuda_error(e, "cudaStreamEndCapture") : RG_OK);
            }
            if (!rc && (e = cudaGraphInstantiate(&ge, gr, 0)) != cudaSuccess)
                rc = cuda_error(e, "cudaGraphInstantiate");
            for (int it = 0; it < niter && !rc; ++it)
                if ((e = cudaGraphLaunch(ge, st)) != cudaSuccess) rc = cuda_error(e, "cudaGraphLaunch");
            if (ge) cudaGraphExecDestroy(ge);
            if (gr) cudaGraphDestroy(gr);
            if (cs) cudaStreamDestroy(cs);
        } else {
            for (int it = 0; it < niter && !rc; ++it) rc = dispatch_iteration(br, st);
        }
    }
    for (int q = 0; q < nslices && !rc; ++q) {
        const rg_image &im = images[order[q]];
        rc = launch_copy2d(xs[q], im.lines, 1, im.data, im.column_stride, im.line_stride,
                           im.lines, im.lines, st);
    }
    scratch_end(sc);
    return rc;
}

int rg_em_plain_host(float *h_out, const float *h_sino, int size, int nrays, int nangles,
                     int niter, int nsubsets)
{
    RG_TRACE();
    if (!h_out || !h_sino || size < 2 || nrays < 2 || nangles < 1 || niter < 0 || nsubsets < 1 ||
        nsubsets > nangles)
        return set_error(RG_EINVAL, "rg_em_plain_host: bad arguments");
    const int N = size, R = nrays, A = nangles, S = nsubsets;
    const double pi = 3.14159265358979323846;
    SSGeom g;
    g.N = N; g.itl_x = -1.0; g.itl_y = 1.0; g.ibr_x = 1.0; g.ibr_y = -1.0;
    g.R = R; g.A = A; g.stl_x = 0.0; g.stl_y = 1.0; g.sbr_x = pi; g.sbr_y = -1.0;
    // per-subset float view tables, built on the host as the reference's
    // kernels would take their float constants
    std::vector<std::vector<PlainView>> pv(S);
    for (int s = 0; s < S; ++s) {
        std::vector<int> idx;
        for (int j = s; j < A; j += S) idx.push_back(j);
        std::vector<View> hv(idx.size());
        SSPlan meta;
        if (int rc = ss_views_compute(meta, g, idx.data(), (int)idx.size(), hv.data())) return rc;
        if (!meta.adj_ok) return set_error(RG_EUNSUPPORTED, "nrays must not exceed size");
        const double q = 1.0 / 4294967296.0;
        for (const View &v : hv)
            pv[s].push_back(PlainView{(float)(v.rk * q), (float)(v.ri * q), (float)(v.r0 * q),
                                      v.delta, (float)(v.krow * q), (float)(v.kcol * q),
                                      (float)(v.k0 * q), v.P, v.flags, v.view, 0, 0});
    }
    const size_t ns = (size_t)R * A, ni = (size_t)N * N;
    float *d_y = nullptr, *d_r = nullptr, *d_x = nullptr, *d_b = nullptr, *d_sens = nullptr,
          *d_t = nullptr;
    PlainView *d_v = nullptr;
    int rc = RG_OK;
    auto ck = [&](cudaError_t e, const char *w) {
        if (e != cudaSuccess && rc == RG_OK) rc = cuda_error(e, w);
        return rc == RG_OK;
    };
    size_t maxv = 0;
    for (auto &t : pv) maxv = std::max(maxv, t.size());
    ck(cudaMalloc(&d_y, ns * 4), "cudaMalloc") && ck(cudaMalloc(&d_r, ns * 4), "cudaMalloc") &&
        ck(cudaMalloc(&d_x, ni * 4), "cudaMalloc") && ck(cudaMalloc(&d_b, ni * 4), "cudaMalloc") &&
        ck(cudaMalloc(&d_sens, ni * 4 * S), "cudaMalloc") && ck(cudaMalloc(&d_t, ni * 4), "cudaMalloc") &&
        ck(cudaMalloc(&d_v, sizeof(PlainView) * maxv * S), "cudaMalloc");
    if (rc == RG_OK) ck(cudaMemcpy(d_y, h_sino, ns * 4, cudaMemcpyHostToDevice), "upload");
    for (int s = 0; s < S && rc == RG_OK; ++s)
        ck(cudaMemcpy(d_v + maxv * s, pv[s].data(), sizeof(PlainView) * pv[s].size(),
                      cudaMemcpyHostToDevice), "upload views");
    const dim3 gi((N + 127) / 128, N);
    const int eb = (int)((ni + 255) / 256), sb = (int)((ns + 255) / 256);
    if (rc == RG_OK) {
        launch_fill(d_x, ni, 1.f, nullptr);
        launch_fill(d_r, ns, 1.f, nullptr);
        for (int s = 0; s < S && rc == RG_OK; ++s) {
            k_plain_adjoint<<<gi, 128>>>(d_r, R, A, d_v + maxv * s, (int)pv[s].size(), N,
                                         d_sens + ni * s);
            ck(cudaDeviceSynchronize(), "plain sensitivity");
        }
    }
    for (int it = 0; it < niter && rc == RG_OK; ++it)
        for (int s = 0; s < S && rc == RG_OK; ++s) {
            const int nv = (int)pv[s].size();
            k_plain_radon<<<dim3((R + 127) / 128, nv), 128>>>(d_x, N, d_v + maxv * s, nv, R, A, d_r);
            if (!ck(cudaDeviceSynchronize(), "plain radon")) break;
            k_plain_ratio<<<sb, 256>>>(d_y, d_r, ns);
            if (!ck(cudaDeviceSynchronize(), "plain ratio")) break;
            k_plain_adjoint<<<gi, 128>>>(d_r, R, A, d_v + maxv * s, nv, N, d_b);
            if (!ck(cudaDeviceSynchronize(), "plain adjoint")) break;
            k_plain_div<<<eb, 256>>>(d_b, d_sens + ni * s, d_t, ni);
            if (!ck(cudaDeviceSynchronize(), "plain divide")) break;
            k_plain_mul<<<eb, 256>>>(d_x, d_t, ni);
            ck(cudaDeviceSynchronize(), "plain multiply");
        }
    if (rc == RG_OK) ck(cudaMemcpy(h_out, d_x, ni * 4, cudaMemcpyDeviceToHost), "download");
    cudaFree(d_y); cudaFree(d_r); cudaFree(d_x); cudaFree(d_b); cudaFree(d_sens); cudaFree(d_t);
    cudaFree(d_v);
    return rc;
}

}  // extern "C"
