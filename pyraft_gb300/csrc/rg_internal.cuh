// rg_internal.cuh -- shared declarations of libraftgb (GB300, sm_103a).
//
// Fixed-point positions.  Every projector evaluates a sample position that
// is affine in two integer indices (ray/line for the Radon, row/column for
// the gathers).  The per-view coefficients are computed once on the host in
// FP64 (the same libm cos/sin/tan values the reference evaluates) and stored
// as signed Q32.32 integers (int64).  The kernels then form positions with
// exact integer arithmetic: an origin in Q32.32 plus small local offsets in
// Q9.23 (uint32), whose low 23 bits become the float interpolation weight by
// a single bit operation (0x3F800000 | frac gives 1 + w).  This keeps the
// floor decision and the weight at ~1e-7 sample precision without FP64 in
// the hot loops and without float<->int conversion instructions, which issue
// at a quarter of the FFMA rate.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>

#include <initializer_list>
#include <utility>
#include <string>

#include <nvtx3/nvToolsExt.h>

#include "../../include/raftgb.h"

namespace rg {

// ----------------------------------------------------------------------------
// Tracing.  Every compute entry point of the C ABI opens an NVTX range named
// after itself for the duration of the call (host side: argument checks,
// plan look-up and the launches it enqueues), so a profiler's timeline shows
// which library call issued which kernels.  NVTX is header-only; without a
// profiler attached a range costs a few nanoseconds.
struct TraceRange {
    explicit TraceRange(const char *name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange &) = delete;
    TraceRange &operator=(const TraceRange &) = delete;
};
#define RG_TRACE() ::rg::TraceRange rg_trace_range_(__func__)

// ----------------------------------------------------------------------------
// Per-view constants (one per view of a plan, device resident).
struct alignas(16) View {
    // Slant-stack Radon: position along line i of ray k (in samples of the
    // line) u = r0 + k*rk + i*ri, Q32.32.  Lines are image columns when
    // (flags & kLinesAreRows) == 0 (|cos| < 1/sqrt 2), image rows otherwise.
    long long rk, ri, r0;
    // Slant-stack backprojection: t-sample position of pixel (row, col),
    // u = b0 + row*brow + col*bcol, Q32.32.
    long long brow, bcol, b0;
    // Matched adjoint: ray-index position of the ray through pixel (row, col)
    // on the pixel's line, kappa = k0 + row*krow + col*kcol, Q32.32.
    long long krow, kcol, k0;
    float delta;      // Radon step length Delta (dy/|sin| or dx/|cos|)
    float P;          // |rk|: ray spacing in line samples
    int flags;        // kLinesAreRows | kRkNegative
    int view;         // sinogram column this entry refers to
    double delta64;   // Delta in FP64 (FP64 operator pair)
    int pad[2];
};
static_assert(sizeof(View) == 112, "View layout");

enum { kLinesAreRows = 1, kRkNegative = 2 };

// ----------------------------------------------------------------------------
// Host-side helpers (api.cu).
int set_error(int code, const char *fmt, ...);
int cuda_error(cudaError_t e, const char *what);
// True when environment variable `name` is "1" (read per call).  Used for the
// failure-path test switches RG_TEST_EXPIRE_WAIT (the first mbarrier wait of
// every CTA of the TMA kernels gives up at once), RG_TEST_WINDOW_CUT (the
// TMA gather under-reports its window bound) and RG_TEST_FAIL_ALLOC (the
// stream-ordered scratch allocation fails); none is set in normal use.
inline bool test_switch(const char *name)
{
    const char *e = getenv(name);
    return e && e[0] == '1' && e[1] == 0;
}

#define RG_CK(call)                                                     \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) return ::rg::cuda_error(e_, #call);      \
    } while (0)

#define RG_CK_LAUNCH(what)                                              \
    do {                                                                \
        cudaError_t e_ = cudaGetLastError();                            \
        if (e_ != cudaSuccess) return ::rg::cuda_error(e_, what);       \
    } while (0)

// ----------------------------------------------------------------------------
// Programmatic dependent launch.  The operators run as chains of short
// kernels on one stream (an EM/OSEM sub-iteration is four or five).  A kernel
// launched by launch_pdl may be scheduled while the kernel before it on the
// stream is still finishing its last wave: its CTAs are dispatched and reach
// pdl_gate(), which first lets the next kernel be scheduled the same way and
// then waits (griddepcontrol.wait) until the preceding grid has completed and
// its memory operations are visible.  Every kernel launched by launch_pdl
// calls pdl_gate() before it touches global memory, so the stream's order is
// kept exactly; what overlaps is launch latency and the dispatch of CTAs
// into the previous kernel's tail.  A dependent grid is scheduled only once
// every CTA of its predecessor has started, so waiting CTAs never keep a
// predecessor's CTAs off the GPU.  For a kernel launched without the
// attribute (or after a copy or another library's kernel) the gate returns
// at once.  RG_PDL=0 (read once per process) launches without the
// attribute.
bool pdl_enabled();
__device__ __forceinline__ void pdl_gate()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Launch kernel k (which begins with pdl_gate()) on `grid` x `block` with
// `smem` bytes of dynamic shared memory on stream st, in clusters of
// `cluster` CTAs along x when cluster > 1, with programmatic dependent
// launch unless RG_PDL=0.
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       int cluster, Args &&...args)
{
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[2];
    unsigned na = 0;
    if (pdl_enabled()) {
        at[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[na].val.programmaticStreamSerializationAllowed = 1;
        ++na;
    }
    if (cluster > 1) {
        at[na].id = cudaLaunchAttributeClusterDimension;
        at[na].val.clusterDim.x = (unsigned)cluster;
        at[na].val.clusterDim.y = 1;
        at[na].val.clusterDim.z = 1;
        ++na;
    }
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = na ? at : nullptr;
    cfg.numAttrs = na;
    return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

// Bump allocator over one scratch block (caller's workspace or a
// stream-ordered allocation that is released on the same stream).
struct Scratch {
    char *base = nullptr;
    size_t size = 0, off = 0;
    bool owned = false;
    cudaStream_t stream = nullptr;
    static size_t align(size_t b) { return (b + 255) & ~size_t(255); }
    void *take(size_t bytes) {
        off = align(off);
        void *p = base + off;
        off += bytes;
        return p;
    }
};
// Sizes are summed with Scratch::align per piece; begin() checks or allocates.
int check_ws(const void *ws);
int scratch_begin(Scratch &s, void *ws, size_t ws_bytes, size_t need, cudaStream_t st);
void scratch_end(Scratch &s);

// ----------------------------------------------------------------------------
// Geometry of a slant-stack plan.
struct SSGeom {
    int N;                         // image size (N x N)
    double itl_x, itl_y, ibr_x, ibr_y;
    int R, A;                      // rays, views of the full sinogram
    double stl_x, stl_y, sbr_x, sbr_y;
};

// A plan: geometry plus device-resident per-view constants for a list of
// views (all views, or one OSEM subset).
struct SSPlan {
    SSGeom g;
    int nv = 0;                    // number of views in this plan
    View *d_views = nullptr;       // device
    // gather window widths (entries) needed for 32-column tiles of 32, 64 and
    // 128 rows (index 0, 1, 2: 4, 8, 16 rows per thread)
    int wmax_bp[3] = {0, 0, 0}, wmax_adj[3] = {0, 0, 0};
    float dth = 0.f;               // view spacing (backprojection scale)
    bool adj_ok = true;            // every |rk| >= 1 (two-tap adjoint)
    bool contiguous = true;        // views are consecutive (not an OSEM subset)
    bool rot_ok = false;           // second half of the views = first half + pi/2, on a grid
                                   // symmetric under a quarter turn (gather_rot.cu)
    bool mirror_ok = false;        // image and detector centred on 0: pixel (r, c) and
                                   // (N-1-r, N-1-c) meet a view at mirrored ray positions
                                   // (gather_tile_mirror)
    int device = -1;
    // TMA-staged Radon (radon_tma.cu): blocks of adjacent views whose line
    // windows fit st_bw entries (nblocks == 0: the direct kernels are used)
    void *d_blocks = nullptr;      // StBlock[nblocks], device
    // the same allocation, after the blocks: the TMA Radon's CTA order,
    // (ray tile << 16 | block) for ceil(R / 64) x nblocks CTAs, most lines first
    const unsigned *d_border = nullptr;
    int nblocks = 0, st_bw = 0;
    // tile-driven Radon (radon_tma.cu): TtView records grouped by
    // orientation (rows first), device
    void *d_ovid = nullptr;
    int n_ovid[2] = {0, 0};
    bool tt_ok = false;
    double tt_ri_max = 0.0, tt_rk_max = 0.0;   // max |ri|, |rk| over the views (samples)
};

// Per-view constants of the tile-driven Radon, grouped by line orientation
// (rows first): one 32-byte record per view, so that the threads of a CTA
// read consecutive records (the 112-byte View records, reached through an
// index, scattered each warp's loads over 32 records).
struct __align__(16) TtView {
    long long r0, rk, ri;   // Q32.32 Radon position u = r0 + k rk + i ri
    float delta;            // ray-sum scale
    int view;               // sinogram column
};
static_assert(sizeof(TtView) == 32, "TtView layout");

// A block of the TMA-staged Radon: views [first, first + count) of a plan,
// all with the same line orientation.
struct StBlock {
    int first, count, flags, pad;
};

int ss_plan_build(SSPlan &p, const SSGeom &g, const int *views, int nv);
int ss_views_compute(SSPlan &p, const SSGeom &g, const int *views, int nv, View *hv);
// Argument checks of the slant-stack entry points (api.cu).
int validate_ss(const rg_image &img, const rg_image &sino);
SSGeom make_ss_geom(const rg_image &img, const rg_image &sino);
void ss_plan_free(SSPlan &p);

// Kernel launchers (slantstack.cu).  Images handed to the kernels are
// strided views: element (row, col) at ptr[row*cs + col*ls].
// Line pairs: N lines of pairs_pitch(N) float2 entries; entry 1 + n holds
// the pair of sample n, entries 0, N and above N are zeros.  The pitch is
// even, so every line starts on a 16-byte boundary (TMA rows).
__host__ __device__ __forceinline__ int pairs_pitch(int N) { return (N + 3) & ~1; }
size_t radon_pairs_bytes(int N);
// nz > 1: a stack of nz images, consecutive ones zi floats apart, their
// line pairs zp pairs apart.
int launch_line_pairs(const float *img, long long cs, long long ls, int N,
                      float2 *pairs_rows, float2 *pairs_cols, cudaStream_t st,
                      int nz = 1, long long zi = 0, long long zp = 0);
// Radon over the plan's views; out row v.view (angle-major, ld = out_ld)
// gets the ray sums, or the EM ratio y/Ax when y_am != nullptr.
// epi: -1 = ray sums (y_am == nullptr) or EM ratio (y_am != nullptr);
// kEpiTransmissionId = transmission, out = y_am * exp(-sum).
constexpr int kEpiTransmissionId = 2;
int launch_radon(const SSPlan &p, const float2 *pairs_rows, const float2 *pairs_cols,
                 float *out_am, int out_ld, const float *y_am, int y_ld, cudaStream_t st,
                 int nz = 1, long long zp = 0, long long zo = 0, int epi = -1);
// radon_tma.cu: view blocks of a plan (after its views are computed), and
// the staged Radon over them (same arguments as launch_radon).
int st_blocks_build(SSPlan &p, const View *hv);
// Tile-driven Radon over plans of scattered views (same arguments).
int tt_build(SSPlan &p, const View *hv);
// Zero pads of `pad` entries hold every crossing ray's walk over `lines`
// lines for this plan's views (with two margin rays each side).
bool tt_pads_fit(const SSPlan &p, int lines, int pad);
bool radon_tiles_usable(const SSPlan &p);
int launch_radon_tiles(const SSPlan &p, const float2 *pairs_rows, const float2 *pairs_cols,
                       float *out_am, int out_ld, const float *y_am, int y_ld, cudaStream_t st,
                       int nz, long long zp, long long zo, int epi);
bool radon_tma_usable(const SSPlan &p);
int launch_radon_tma(const SSPlan &p, const float2 *pairs_rows, const float2 *pairs_cols,
                     float *out_am, int out_ld, const float *y_am, int y_ld, cudaStream_t st,
                     int nz, long long zp, long long zo, int epi);
// Per-device error word of kernels with bounded waits (api.cu): nullptr
// until ensure_device_error_word ran on the current device.
int *device_error_word();
int ensure_device_error_word();
// Views per thread of the Radon for this plan: 2 when its views are
// consecutive (the two share L1 lines), else 1.  RG_RADON_VIEWS=1|2 overrides.
int radon_views_per_thread(const SSPlan &p);
// Gathers.  mode 0: backprojection (scaled by dth); 1: matched adjoint;
// 2: matched adjoint accumulated in FP64, epilogue writes 1/x (0 where 0).
// em_x != nullptr (modes 0, 1): x <- x * gather * inv_sens, with x, inv_sens
// contiguous N x N.
// A stack of n equal-geometry problems in one launch (grid z): consecutive
// inputs `in` floats apart, outputs `out` floats apart.
struct Stack {
    int n = 1;
    long long in = 0, out = 0;
};
// The EM update fused into the paired gathers (launch_gather_rot with `em`):
// each pixel's two partial sums are added into gsum (N x N contiguous, zero
// on entry and left zero on exit), and the last of the CTAs that add to a
// 32 x 32 block of pixels (cnt: one counter per block, zero on entry and
// left zero) applies x <- x * gsum * inv to the block's pixels -- the
// adjoint's interior pixels, whose edge pixels the caller updates -- and
// zeroes the block's gsum.  Needs N % 32 == 0 (blocks map onto blocks under
// the quarter turn).
struct EmFuse {
    float *x = nullptr;
    const float *inv = nullptr;
    float *gsum = nullptr;
    int *cnt = nullptr;
};
inline bool em_fusable(int N) { return N >= 32 && N % 32 == 0; }
// rows: rows per thread (4, 8 or 16; 0 = the tuned choice for this geometry).
// quads: device scratch of gather_quads_bytes(p.nv, p.g.R, z.n) bytes
// (16-byte aligned) through which the paired path (p.rot_ok, modes 0 and 1)
// stages its windows by TMA; null makes it stage them with loads.
int launch_gather(const SSPlan &p, int mode, const float *s_am, int s_ld,
                  float *out, long long cs, long long ls,
                  float *em_x, const float *inv_sens, int *d_err, cudaStream_t st,
                  int rows = 0, Stack z = Stack(), void *quads = nullptr,
                  const EmFuse *fuse = nullptr);
// Bytes of the paired gathers' quad scratch for nz problems of nv views over
// R rays: a 16-byte quad per (view pair, sample entry), R + 1 entries.
size_t gather_quads_bytes(int nv, int R, int nz);
// The gather launch shape picked for (geometry, mode) by the autotuner
// (api.cu): rows per thread and the cluster view split (0: the occupancy
// rule of gather_pick_split).
struct TuneChoice {
    int rows;
    int split;
};
TuneChoice tuned_choice(const SSPlan &p, int mode);
inline int tuned_rows(const SSPlan &p, int mode) { return tuned_choice(p, mode).rows; }
// Times the gather variants of (plan, mode) on the caller's buffers (a
// stack of z.n problems when z says so) the first time a geometry is seen
// outside a stream capture (out is overwritten) and caches the fastest
// (api.cu).  quads as for launch_gather.
int autotune_gather(const SSPlan &p, int mode, const float *s_am, int s_ld, float *out,
                    long long cs, long long ls, cudaStream_t st, void *quads = nullptr,
                    const Stack &z = Stack());
// Cluster size (1, 2 or 4) for the view split of a gather kernel k launched
// on `grid` with `smem` bytes of shared memory (slantstack.cu): the calling
// thread's preference (SplitPref) where the kernel can run it, else the
// occupancy rule.
int gather_pick_split(const void *k, size_t smem, int rows, int nv, dim3 grid, cudaStream_t st);
// Scoped split preference of the calling thread for the gather launches it
// makes (0: none); launch_gather sets the tuned one, the autotuner each
// candidate.
int split_preference();
struct SplitPref {
    explicit SplitPref(int split);
    ~SplitPref();
    SplitPref(const SplitPref &) = delete;
    SplitPref &operator=(const SplitPref &) = delete;
    int saved;
};
// Backprojection (mode 0) or matched adjoint (mode 1) with views paired a
// quarter turn apart (p.rot_ok).  Two partial sums are added to each
// interior pixel of an output that is zeroed first: by this call when
// zero_out (in the quad prepass where it runs), else by the caller.  The
// adjoint's edge pixels are computed by extra CTAs of the same launch when
// `edges` (stored, or EM-updated), else left to the caller.  With `em` (one
// slice, out = em->gsum, N x N contiguous) the EM update is fused as
// described at EmFuse.
int launch_gather_rot(const SSPlan &p, int mode, const float *s_am, int s_ld, float *out,
                      long long cs, long long ls, int *d_err, cudaStream_t st, int rows,
                      const Stack &z, void *quads, bool zero_out, const EmFuse *em = nullptr,
                      bool edges = false);
// Whether launch_gather takes the paired path where a plan allows it
// (RG_GATHER_ROT=0 turns it off).
bool gather_rot_enabled();
// Whether a one-slice backprojection (mode 0) with quad scratch runs the
// TMA-staged paired gather (at the tuned launch shape), whose prepass
// (quads from the filtered rows, output zeroed) the FBP filter can do in
// its epilogue (launch_filter_fft_quads).
bool gather_quads_form(const SSPlan &p, void *quads);
// While alive, the calling thread's backprojection gathers of that form
// take the quads and the zeroed output as given and skip their prepass; a
// backprojection that would stage otherwise fails with RG_EINVAL.
struct QuadsPrefilled {
    QuadsPrefilled();
    ~QuadsPrefilled();
    QuadsPrefilled(const QuadsPrefilled &) = delete;
    QuadsPrefilled &operator=(const QuadsPrefilled &) = delete;
};
// Zero an N x N strided image (a stack of z.n, z.out apart).
int launch_zero_image(float *out, int N, long long cs, long long ls, cudaStream_t st,
                      const Stack &z);

// f64.cu: FP64 operator pair (exact transposes), one thread per (ray, view).
int launch_radon_f64(const SSPlan &p, const double *img, long long ics, long long ils,
                     double *out, long long ocs, long long ols, cudaStream_t st);
int launch_radon_transpose_f64(const SSPlan &p, const double *sino, long long scs, long long sls,
                               double *img_c, cudaStream_t st);

// aux.cu
// nz > 1: a stack, consecutive inputs zi and outputs zo floats apart.
int launch_to_am(const float *in, long long cs, long long ls, int R, int A, float *out_am,
                 cudaStream_t st, int nz = 1, long long zi = 0, long long zo = 0);
int launch_from_am(const float *am, int R, int A, float *out, long long cs, long long ls,
                   cudaStream_t st, int nz = 1, long long zi = 0, long long zo = 0);
// out(k, j) += am[j * R + k] (k < R, j < A)
int launch_add_from_am(const float *am, int R, int A, float *out, long long cs, long long ls,
                       cudaStream_t st);
int launch_copy2d(const float *in, long long ics, long long ils, float *out, long long ocs,
                  long long ols, int rows, int cols, cudaStream_t st);
int launch_fill(float *p, size_t n, float v, cudaStream_t st);
// Smoothed isotropic TV of nz contiguous N x N images into *value (device
// FP64, zeroed first) and, if grad != nullptr, its gradient.
int launch_tv(const float *x, int nz, int N, float eps, double *value, float *grad,
              cudaStream_t st);
int launch_phantom(float *img, long long cs, long long ls, int lines, int cols,
                   double tl_x, double tl_y, double br_x, double br_y,
                   const double *d_desc, int n, cudaStream_t st);
int launch_radon_fromdesc(float *sino, long long cs, long long ls, int lines, int cols,
                          double tl_x, double tl_y, double br_x, double br_y,
                          const double *d_desc, int n, cudaStream_t st);

// filter.cu: out_am[a][n] = sum_k taps[n - k + R - 1] * in_am[a][k].
int launch_conv_rows(const float *in_am, float *out_am, int R, int A, const float *d_taps,
                     cudaStream_t st);

// Ram-Lak only: odd taps godd[q] = h[2q - 2R + 1] (q in [0, 2R)), h0 = h[0].
int launch_ramlak_rows(const float *in_am, float *out_am, int R, int A, const float *d_godd,
                       float h0, cudaStream_t st);

// A filter by FFT of size 2^p (2^p >= 2R - 1; circ: 2^p = R, a circular
// convolution of length R; p <= kFilterFftMaxLog): d_tab = twiddles
// e^{-2 pi i t / 2^p} (t < 2^(p-1)), then the difference-domain filter in
// bit-reversed order (2^p entries); g0 = the DC gain / 2^p.
constexpr int kFilterFftMaxLog = 14;
int launch_filter_fft(const float *in_am, float *out_am, int R, int A, int p, const float2 *d_tab,
                      float g0, bool circ, cudaStream_t st);
// The same filter (linear form) for the FBP: CTA j filters rows
// d_views[j].view and d_views[j].view + roff of in_am (j < pairs) and writes
// the paired backprojection's quads[j][e] (e < R - 1) instead of the rows,
// and the CTAs zero the N x N output (strides cs, ls).
int launch_filter_fft_quads(const float *in_am, int R, int A, int p, const float2 *d_tab, float g0,
                            const View *d_views, int pairs, int roff, float4 *quads, float *out,
                            int N, long long cs, long long ls, cudaStream_t st);

// bresenham.cu
struct DDAGeom {
    int lines, columns;
    double itl_x, itl_y, ibr_x, ibr_y;
    int R, A;
    double stl_x, stl_y, sbr_x, sbr_y;
};
int launch_bres_radon(const DDAGeom &g, const double *d_cs, const float *img, long long ics,
                      long long ils, float *out, long long cs, long long ls,
                      const float *y_am, int first, int stride, cudaStream_t st);
int launch_bres_transpose(const DDAGeom &g, const double *d_cs, const float *s_am,
                          float *img_c, int first, int stride, cudaStream_t st);
// elementwise on view-major sinograms: out = max(a - b, 0) (b may be null)
int launch_sub_clamp(const float *a, const float *b, float *out, size_t n, cudaStream_t st);
int launch_em_update(float *x, const float *bp, const float *inv_sens, size_t n, cudaStream_t st);
int launch_invert(const float *sens, float *inv, size_t n, cudaStream_t st);

// api.cu helpers shared with em.cu
int get_ss_plan(const SSGeom &g, int stride, int first, const SSPlan **out, void **holder);
void release_holder(void *holder);
int get_dda_views(const DDAGeom &g, const double **d_cs, void **holder);
size_t ws_sum(std::initializer_list<size_t> pieces);
// num, den: contiguous lines x columns FP64, pre-zeroed; out strided.
int launch_bres_normalised(const DDAGeom &g, const double *d_cs, const float *s_am, double *num,
                           double *den, float *out, long long cs, long long ls, cudaStream_t st);
// Recorded DDA walks of views first, first + stride, ... (bresenham.cu):
// built once, replayed by the Radon and transpose of iterative methods.
struct DDAPlan {
    void *rays = nullptr;      // DDARayRec[nrays] (device)
    void *steps = nullptr;     // FP32 per step (device); null: no plan
    long long nrays = 0, total = 0;
    int first = 0, stride = 1;
};
int dda_plan_build(const DDAGeom &g, const double *d_cs, int first, int stride,
                   size_t max_bytes, DDAPlan &p, cudaStream_t st);
void dda_plan_free(DDAPlan &p);
// img_c contiguous lines x columns and imgT_c its column-major copy (the
// Radon reads both; the transpose adds to both, to be summed by the
// caller); out_am / s_am view-major (view row x R).
int launch_dda_plan_radon(const DDAGeom &g, const DDAPlan &p, const float *img_c,
                          const float *imgT_c, float *out_am, const float *y_am, cudaStream_t st);
int launch_dda_plan_transpose(const DDAGeom &g, const DDAPlan &p, const float *s_am, float *img_c,
                              float *imgT_c, cudaStream_t st);
int launch_dda_trace(int lines, int columns, const double *corners, const double *d_cst, int n,
                     int cap, int *oi, int *oj, double *os, int *ocount, cudaStream_t st);

}  // namespace rg
