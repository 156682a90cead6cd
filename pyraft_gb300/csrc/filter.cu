// filter.cu -- the FBP filter step as a row-wise convolution.
//
// out_am[a][n] = sum_{k=0}^{R-1} taps[n - k + R - 1] * in_am[a][k] for every
// view a of a view-major sinogram (rows of length R).  The 2R-1 taps are
// computed on the host in FP64: the discrete Ram-Lak kernel for linear
// convolution, or the periodised spatial form of pyraft's lowpassino_fbp
// filter (pyraft/filters/filters.py:13-68) for circular convolution.
//
// Kernels: k_filter_fft (either filter by FFT, the default up to 8192 rays:
// O(R log R) per view and more accurate), and above that the direct sums of
// k_ramlak_rows (Ram-Lak, its odd taps only) and k_conv_rows (any taps).
//
// k_conv_rows:
// CTA = 256 outputs x 16 views.  The input is walked in tiles of 256
// samples: the tile (16 views, stored [k][view] so one LDS.128 feeds four
// FFMAs) and the 511 taps it meets are staged in shared memory; each thread
// keeps 16 accumulators, i.e. 16 FFMA per 1 + 4 shared loads.  Per-tile
// partial sums are added with Kahan compensation.
#include "ss_tiles.cuh"

namespace rg {

constexpr int kTN = 256, kTK = 256, kNA = 16;

__global__ __launch_bounds__(256) void k_conv_rows(const float *__restrict__ in, float *__restrict__ out,
                                                   int R, int A, const float *__restrict__ taps)
{
    pdl_gate();
    __shared__ float4 sx[kTK][kNA / 4];
    __shared__ float sh[kTN + kTK];
    const int t = threadIdx.x;
    const int n0 = blockIdx.x * kTN, a0 = blockIdx.y * kNA;
    const int n = n0 + t;
    float acc[kNA], comp[kNA];
#pragma unroll
    for (int a = 0; a < kNA; ++a) { acc[a] = 0.f; comp[a] = 0.f; }

    for (int k0 = 0; k0 < R; k0 += kTK) {
        // input tile, transposed to [k][view]
        float *sxf = reinterpret_cast<float *>(sx);
        for (int e = t; e < kTK * kNA; e += 256) {
            const int a = e / kTK, kk = e - a * kTK;
            const int k = k0 + kk, av = a0 + a;
            sxf[kk * kNA + a] = (k < R && av < A) ? __ldg(in + (size_t)av * R + k) : 0.f;
        }
        // taps m = n - k for n in [n0, n0+256), k in [k0, k0+256)
        const int mbase = n0 - k0 - (kTK - 1);
        for (int e = t; e < kTN + kTK - 1; e += 256) {
            const int m = mbase + e;
            sh[e] = (m > -R && m < R) ? __ldg(taps + m + R - 1) : 0.f;
        }
        __syncthreads();
        float part[kNA];
#pragma unroll
        for (int a = 0; a < kNA; ++a) part[a] = 0.f;
        const int kend = min(kTK, R - k0);
#pragma unroll 4
        for (int kk = 0; kk < kend; ++kk) {
            const float h = sh[t - kk + kTK - 1];
#pragma unroll
            for (int q = 0; q < kNA / 4; ++q) {
                const float4 x = sx[kk][q];
                part[4 * q + 0] = fmaf(h, x.x, part[4 * q + 0]);
                part[4 * q + 1] = fmaf(h, x.y, part[4 * q + 1]);
                part[4 * q + 2] = fmaf(h, x.z, part[4 * q + 2]);
                part[4 * q + 3] = fmaf(h, x.w, part[4 * q + 3]);
            }
        }
#pragma unroll
        for (int a = 0; a < kNA; ++a) {
            const float y = part[a] - comp[a];
            const float s = acc[a] + y;
            comp[a] = (s - acc[a]) - y;
            acc[a] = s;
        }
        __syncthreads();
    }
    if (n >= R) return;
#pragma unroll
    for (int a = 0; a < kNA; ++a)
        if (a0 + a < A) out[(size_t)(a0 + a) * R + n] = acc[a] - comp[a];
}

int launch_conv_rows(const float *in_am, float *out_am, int R, int A, const float *d_taps,
                     cudaStream_t st)
{
    dim3 grid((R + kTN - 1) / kTN, (A + kNA - 1) / kNA);
    RG_CK(launch_pdl(k_conv_rows, grid, 256, 0, st, 1, in_am, out_am, R, A, d_taps));
    RG_CK_LAUNCH("k_conv_rows");
    return RG_OK;
}

}  // namespace rg

namespace rg {

// ----------------------------------------------------------------------------
// Ram-Lak specialisation.  Its taps vanish at even offsets except 0, so
// out[n] = h0 in[n] + sum_{n-k odd} h[n-k] in[k]: an even output meets only
// odd inputs and an odd output only even inputs, both through odd taps
// g[q] = h[2q - 2R + 1] (q in [0, 2R); dt included; zero beyond |m| = R-1).
//
// Output pair t' (outputs n0 + 2t', n0 + 2t' + 1) and input pair j (inputs
// k0 + 2j, k0 + 2j + 1) meet through the taps Q = (n0 - k0)/2 + R - 1 + t' - j
// (even output x odd input) and Q + 1 (odd output x even input).
//
// CTA = 1024 outputs x 4 views; thread t owns output pairs 2t and 2t + 1, so
// at input pair j it needs the three taps G0 = g[Q(2t, j)], G1 = G0's
// successor and G2 the next one; stepping j by one shifts the three by one
// place, so each step loads one new tap from shared memory and reuses two.
// Per step: one LDS.32 (the new tap) + two broadcast LDS.128 (the even and
// odd inputs of four views) feed 16 FFMAs.  The taps are staged split by
// index parity so the lanes (which read every other tap) hit distinct banks.
// Inputs are walked in tiles of 512; per-tile partial sums are added with
// Kahan compensation.
constexpr int kRN = 1024, kRK = 512, kRA = 4;
constexpr int kRT = kRN / 2 + kRK / 2 + 2;      // staged taps per tile (even count)

__global__ __launch_bounds__(256) void k_ramlak_rows(const float *__restrict__ in,
                                                     float *__restrict__ out, int R, int A,
                                                     const float *__restrict__ godd, float h0)
{
    pdl_gate();
    __shared__ float4 sxe[kRK / 2];             // even inputs of the tile, 4 views
    __shared__ float4 sxo[kRK / 2];             // odd inputs
    __shared__ float sg0[kRT / 2], sg1[kRT / 2];  // staged taps: index 2i -> sg0[i], 2i+1 -> sg1[i]
    const int t = threadIdx.x;
    const int n0 = blockIdx.x * kRN, a0 = blockIdx.y * kRA;
    // accumulator index: 8 * pair + 4 * (odd output) + view
    float acc[16], comp[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) { acc[i] = 0.f; comp[i] = 0.f; }

    for (int k0 = 0; k0 < R; k0 += kRK) {
        float *xe = reinterpret_cast<float *>(sxe), *xo = reinterpret_cast<float *>(sxo);
        for (int e = t; e < kRK * kRA; e += 256) {
            const int a = e / kRK, kk = e - a * kRK;
            const int k = k0 + kk, av = a0 + a;
            const float v = (k < R && av < A) ? __ldg(in + (size_t)av * R + k) : 0.f;
            if (kk & 1) xo[(kk >> 1) * kRA + a] = v; else xe[(kk >> 1) * kRA + a] = v;
        }
        // sg[e] = g[qbase + e]; Q(t', j) - qbase = t' - j + kRK/2 - 1
        const int qbase = (n0 - k0) / 2 + R - kRK / 2;
        for (int e = t; e < kRT; e += 256) {
            const int q = qbase + e;
            const float g = (q >= 0 && q < 2 * R) ? __ldg(godd + q) : 0.f;
            if (e & 1) sg1[e >> 1] = g; else sg0[e >> 1] = g;
        }
        __syncthreads();
        float part[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) part[i] = 0.f;
        // input pairs of this tile that hold data, rounded up to even (the
        // staged inputs past R are zeros)
        const int jend = min(kRK / 2, ((R - k0 + 1) / 2 + 1) & ~1);
        // at step j: G0 = sg[2t + kRK/2 - 1 - j], G1 = sg[.. + 1], G2 = sg[.. + 2]
        float G1 = sg0[t + kRK / 4], G2 = sg1[t + kRK / 4];
        for (int j = 0; j < jend; j += 2) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                // 2t + kRK/2 - 1 - (j + h): odd for h = 0, even for h = 1
                const float G0 = h == 0 ? sg1[t + kRK / 4 - 1 - j / 2]
                                        : sg0[t + kRK / 4 - 1 - j / 2];
                const float4 xo4 = sxo[j + h];
                const float4 xe4 = sxe[j + h];
                const float o[4] = {xo4.x, xo4.y, xo4.z, xo4.w};
                const float ev[4] = {xe4.x, xe4.y, xe4.z, xe4.w};
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    part[v] = fmaf(G0, o[v], part[v]);              // pair 2t, even output
                    part[4 + v] = fmaf(G1, ev[v], part[4 + v]);     // pair 2t, odd output
                    part[8 + v] = fmaf(G1, o[v], part[8 + v]);      // pair 2t+1, even output
                    part[12 + v] = fmaf(G2, ev[v], part[12 + v]);   // pair 2t+1, odd output
                }
                G2 = G1;
                G1 = G0;
            }
        }
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const float y = part[i] - comp[i], s = acc[i] + y;
            comp[i] = (s - acc[i]) - y;
            acc[i] = s;
        }
        __syncthreads();
    }
    const int nb = n0 + 4 * t;
#pragma unroll
    for (int v = 0; v < kRA; ++v) {
        const int av = a0 + v;
        if (av >= A) break;
        const float *row = in + (size_t)av * R;
        float *orow = out + (size_t)av * R;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int n = nb + u;
            const int i = 8 * (u >> 1) + 4 * (u & 1) + v;
            if (n < R) orow[n] = fmaf(h0, __ldg(row + n), acc[i] - comp[i]);
        }
    }
}

int launch_ramlak_rows(const float *in_am, float *out_am, int R, int A, const float *d_godd,
                       float h0, cudaStream_t st)
{
    dim3 grid((R + kRN - 1) / kRN, (A + kRA - 1) / kRA);
    RG_CK(launch_pdl(k_ramlak_rows, grid, 256, 0, st, 1, in_am, out_am, R, A, d_godd, h0));
    RG_CK_LAUNCH("k_ramlak_rows");
    return RG_OK;
}

// ----------------------------------------------------------------------------
// Filter by FFT: the same sum over the 2R-1 taps, through a circular
// convolution of length M = 2^p >= 2R - 1 (outputs [0, R) see no
// wrap-around).  The circular form (circ; R = M a power of two) computes
// pyraft's lowpass filter as what it is, a circular convolution of length
// R: its taps are R-periodic, and their zero-padded transform would
// oscillate and amplify rounding at low frequencies.
//
// Two views per CTA, packed as one complex signal v = x + i y: the taps are
// real, so the real and imaginary parts of the result are the two filtered
// views.
//
// Accuracy: the FFT's rounding error scales with the norm of what it
// transforms, while a ramp filter all but removes the low frequencies that
// carry most of a sinogram's norm.  So the kernel transforms the first difference
// D[n] = v[n] - v[n-1] (v zero outside [0, R); circular: v[-1] = v[R-1])
// and applies G'[k] =
// G[k] / (M (1 - e^{-2 pi i k / M})) for k != 0, with G the filter's DFT;
// the DC term G[0] sum(v) / M is added at the end.  On FP32 inputs this
// keeps the result within a few 1e-7 (relative L2) of the FP64 convolution
// even for smooth profiles, where transforming v itself loses 1e-5.
//
// Ordering: a decimation-in-frequency forward pass (natural order in,
// bit-reversed out), the filter applied in bit-reversed order (G' is stored
// that way), and a decimation-in-time inverse pass (bit-reversed in,
// natural out), so no permutation pass is needed.
//
// Passes over shared memory: the first forward stage (span M/2) is fused
// with the load and the last inverse stage with the store.  The other
// radix-2 stages run in registers, up to four consecutive stages per pass:
// a thread takes the 2^nst entries base + k q (q = the pass's smallest
// span) that those stages combine, and writes them back in place.  The
// forward stages of spans 4, 2, 1, the filter and the inverse stages of
// spans 1, 2, 4 touch the same eight contiguous entries and form one pass.
// So M = 4096 takes 6 passes, not 22.  Entry i lives at i + i/16 (one pad
// per 16) so that strided groups and contiguous blocks spread over banks.
//
// Tables (host-computed in FP64): tw[t] = e^{-2 pi i t / M}, t < M/2, then
// gb[k] = G'[bitrev_p(k)], k < M; g0 = G[0] / M.
constexpr int kFftThreads = 256;

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 w)
{
    return make_float2(fmaf(a.x, w.x, -a.y * w.y), fmaf(a.x, w.y, a.y * w.x));
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 w)   // a * conj(w)
{
    return make_float2(fmaf(a.x, w.x, a.y * w.y), fmaf(a.y, w.x, -a.x * w.y));
}
__device__ __forceinline__ int fpad(int i) { return i + (i >> 4); }

// e^{-i pi e / 8}, e in [0, 16): the roots of unity of order <= 16.
__device__ __forceinline__ float2 root16(int e)
{
    constexpr float c[5] = {1.0f, 0.92387953251128674f, 0.70710678118654752f,
                            0.38268343236508979f, 0.0f};
    const int q = e & 7;
    const float cs = q <= 4 ? c[q] : -c[8 - q];     // cos(pi q / 8)
    const float sn = q <= 4 ? c[4 - q] : c[q - 4];  // sin(pi q / 8)
    return e < 8 ? make_float2(cs, -sn) : make_float2(-cs, sn);
}

// w * e^{-i pi kl / d} (kl < d <= 8, both compile-time after unrolling).
__device__ __forceinline__ float2 rot(float2 w, int kl, int d)
{
    if (kl == 0) return w;
    const int e = kl * (8 / d);
    if (e == 4) return make_float2(w.y, -w.x);      // times -i
    return cmul(w, root16(e));
}

// Forward stages of spans 2^lt, 2^(lt-1), ..., 2^(lt-NST+1).  In the stage
// of span h = d q (d = 2^(NST-1-s) in entries of the group), butterfly
// (k, k + d) has twiddle index (r + kl q) (M / 2h), r = g mod q, kl = k mod
// d: one table value W^{r M / 2h} times the constant e^{-i pi kl / d}.
template <int NST>
__device__ __forceinline__ void fft_fwd_pass(float2 *z, int p, int lt,
                                             const float2 *__restrict__ tw)
{
    constexpr int K = 1 << NST;
    const int lq = lt - NST + 1, q = 1 << lq;
    for (int g = threadIdx.x; g < (1 << (p - NST)); g += kFftThreads) {
        const int r = g & (q - 1);
        const int base = ((g >> lq) << (lt + 1)) + r;
        float2 v[K];
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] = z[fpad(base + k * q)];
#pragma unroll
        for (int s = 0; s < NST; ++s) {
            const int d = 1 << (NST - 1 - s);
            const float2 w0 = __ldg(tw + (r << (p - 1 - (lt - s))));
#pragma unroll
            for (int kl = 0; kl < d; ++kl) {
                const float2 w = rot(w0, kl, d);
#pragma unroll
                for (int k = kl; k < K; k += 2 * d) {
                    const float2 a = v[k], c = v[k + d];
                    v[k] = cadd(a, c);
                    v[k + d] = cmul(csub(a, c), w);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < K; ++k) z[fpad(base + k * q)] = v[k];
    }
}

// Inverse stages of spans 2^lb, ..., 2^(lb+NST-1) (conjugate twiddles).
template <int NST>
__device__ __forceinline__ void fft_inv_pass(float2 *z, int p, int lb,
                                             const float2 *__restrict__ tw)
{
    constexpr int K = 1 << NST;
    const int q = 1 << lb;
    for (int g = threadIdx.x; g < (1 << (p - NST)); g += kFftThreads) {
        const int r = g & (q - 1);
        const int base = ((g >> lb) << (lb + NST)) + r;
        float2 v[K];
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] = z[fpad(base + k * q)];
#pragma unroll
        for (int s = 0; s < NST; ++s) {
            const int d = 1 << s;
            const float2 w0 = __ldg(tw + (r << (p - 1 - (lb + s))));
#pragma unroll
            for (int kl = 0; kl < d; ++kl) {
                const float2 w = rot(w0, kl, d);
#pragma unroll
                for (int k = kl; k < K; k += 2 * d) {
                    const float2 a = v[k], c = cmulc(v[k + d], w);
                    v[k] = cadd(a, c);
                    v[k + d] = csub(a, c);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < K; ++k) z[fpad(base + k * q)] = v[k];
    }
}

// Forward stages of spans 2^(NM-1) .. 1, the filter, inverse stages of
// spans 1 .. 2^(NM-1), on blocks of 2^NM contiguous entries (r = 0: the
// twiddles are the constants e^{-i pi kl / d}).
template <int NM>
__device__ __forceinline__ void fft_mid_pass(float2 *z, int p, const float2 *__restrict__ gb)
{
    constexpr int K = 1 << NM;
    const float2 one = make_float2(1.f, 0.f);
    for (int g = threadIdx.x; g < (1 << (p - NM)); g += kFftThreads) {
        const int base = g * K;
        float2 v[K];
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] = z[fpad(base + k)];
#pragma unroll
        for (int s = 0; s < NM; ++s) {
            const int d = 1 << (NM - 1 - s);
#pragma unroll
            for (int kl = 0; kl < d; ++kl) {
                const float2 w = rot(one, kl, d);
#pragma unroll
                for (int k = kl; k < K; k += 2 * d) {
                    const float2 a = v[k], c = v[k + d];
                    v[k] = cadd(a, c);
                    v[k + d] = kl ? cmul(csub(a, c), w) : csub(a, c);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] = cmul(v[k], __ldg(gb + base + k));
#pragma unroll
        for (int s = 0; s < NM; ++s) {
            const int d = 1 << s;
#pragma unroll
            for (int kl = 0; kl < d; ++kl) {
                const float2 w = rot(one, kl, d);
#pragma unroll
                for (int k = kl; k < K; k += 2 * d) {
                    const float2 a = v[k], c = kl ? cmulc(v[k + d], w) : v[k + d];
                    v[k] = cadd(a, c);
                    v[k + d] = csub(a, c);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < K; ++k) z[fpad(base + k)] = v[k];
    }
}

// QUADS (the FBP form, launch_filter_fft_quads): the CTA of view pair j
// transforms sinogram rows views[j].view and views[j].view + roff, the rows
// of a view and its partner a quarter turn on, and writes the pair's quads
// for the paired backprojection instead of the filtered rows: entry e < R - 1
// holds both rows' sample pairs at e, the float4 that the gather's prepass
// (k_pair_quads<0>) builds from the filtered rows, bit for bit.  The CTAs
// also zero the N x N output that the gather adds its partial sums to, as
// that prepass does.  Linear convolution only (circ false).
struct FilterQuads {
    const View *views;
    int roff;
    float4 *quads;
    float *zout;
    int N;
    long long cs, ls;
};

template <bool QUADS>
__global__ __launch_bounds__(kFftThreads) void k_filter_fft(const float *__restrict__ in,
                                                            float *__restrict__ out, int R, int A,
                                                            int p, const float2 *__restrict__ tab,
                                                            float g0, bool circ, FilterQuads fq)
{
    pdl_gate();
    extern __shared__ __align__(16) float2 z[];          // [M + M/16]
    __shared__ float2 wsum[kFftThreads / 32];
    const int M = 1 << p, H = M >> 1, t = threadIdx.x;
    const float2 *__restrict__ tw = tab;
    const float2 *__restrict__ gb = tab + H;
    const int a0 = QUADS ? fq.views[blockIdx.x].view : 2 * blockIdx.x;
    const bool two = QUADS || a0 + 1 < A;
    const float *__restrict__ x = in + (size_t)a0 * R;
    const float *__restrict__ y = x + (size_t)(QUADS ? fq.roff : 1) * R;   // read only when `two`

    // v[n] for n in [0, R), else 0
    auto v = [&](int n) {
        float2 r = make_float2(0.f, 0.f);
        if (n >= 0 && n < R) {
            r.x = __ldg(x + n);
            if (two) r.y = __ldg(y + n);
        }
        return r;
    };
    // load D, forward stage of span H.  v[i - 1] comes from the lane below
    // (lane 0 loads it); the loop runs warp-uniformly so that every lane
    // takes part in the shuffles.
    float2 s = make_float2(0.f, 0.f);
    const int lane = t & 31;
    for (int ib = t - lane; ib < H; ib += kFftThreads) {
        const int i = ib + lane;
        const float2 vi = v(i);                    // zero for i >= R (and so for i >= H)
        float2 vp;
        vp.x = __shfl_up_sync(0xffffffffu, vi.x, 1);
        vp.y = __shfl_up_sync(0xffffffffu, vi.y, 1);
        if (i >= H) continue;
        if (lane == 0) vp = v(i == 0 && circ ? R - 1 : i - 1);
        s = cadd(s, vi);
        const float2 a = csub(vi, vp);
        float2 c = make_float2(0.f, 0.f);
        if (i + H <= R) {                          // circular: always; else i = 0, R = H
            const float2 vh = v(i + H);
            if (circ) s = cadd(s, vh);
            c = csub(vh, v(i + H - 1));
        }
        z[fpad(i)] = cadd(a, c);
        z[fpad(i + H)] = cmul(csub(a, c), __ldg(tw + i));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
        s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
    }
    if ((t & 31) == 0) wsum[t >> 5] = s;
    __syncthreads();

    // forward stages of spans H/2 .. 2^nm, in passes of up to four
    const int nm = min(3, p - 1);
    for (int lt = p - 2; lt >= nm;) {
        const int nst = min(4, lt - nm + 1);
        if (nst == 4) fft_fwd_pass<4>(z, p, lt, tw);
        else if (nst == 3) fft_fwd_pass<3>(z, p, lt, tw);
        else if (nst == 2) fft_fwd_pass<2>(z, p, lt, tw);
        else fft_fwd_pass<1>(z, p, lt, tw);
        lt -= nst;
        __syncthreads();
    }
    if (nm == 3) fft_mid_pass<3>(z, p, gb);
    else if (nm == 2) fft_mid_pass<2>(z, p, gb);
    else fft_mid_pass<1>(z, p, gb);
    __syncthreads();
    for (int lb = nm; lb <= p - 2;) {
        const int nst = min(4, p - 1 - lb);
        if (nst == 4) fft_inv_pass<4>(z, p, lb, tw);
        else if (nst == 3) fft_inv_pass<3>(z, p, lb, tw);
        else if (nst == 2) fft_inv_pass<2>(z, p, lb, tw);
        else fft_inv_pass<1>(z, p, lb, tw);
        lb += nst;
        __syncthreads();
    }
    // inverse span H (outputs [0, R) only) and the DC term
    float2 tot = make_float2(0.f, 0.f);
#pragma unroll
    for (int w = 0; w < kFftThreads / 32; ++w) tot = cadd(tot, wsum[w]);
    const float dcx = tot.x * g0, dcy = tot.y * g0;
    if constexpr (QUADS) {
        // output n < R <= H reads z[n] and z[n + H] only: store it in z[n]
        for (int n = t; n < R; n += kFftThreads) {
            const float2 u = cmulc(z[fpad(n + H)], __ldg(tw + n));
            const float2 r = cadd(z[fpad(n)], u);
            z[fpad(n)] = make_float2(r.x + dcx, r.y + dcy);
        }
        __syncthreads();
        float4 *__restrict__ qd = fq.quads + (size_t)blockIdx.x * (R - 1);
        for (int e = t; e < R - 1; e += kFftThreads) {
            const float2 s0 = z[fpad(e)], s1 = z[fpad(e + 1)];
            const float2 a = make_pair(s0.x, s1.x, true), b = make_pair(s0.y, s1.y, true);
            qd[e] = make_float4(a.x, a.y, b.x, b.y);
        }
        const long long n = (long long)fq.N * fq.N;
        for (long long i = (long long)blockIdx.x * kFftThreads + t; i < n;
             i += (long long)gridDim.x * kFftThreads) {
            const int r = (int)(i / fq.N), c = (int)(i - (long long)r * fq.N);
            fq.zout[(long long)r * fq.cs + (long long)c * fq.ls] = 0.f;
        }
    } else {
        float *__restrict__ ox = out + (size_t)a0 * R;
        for (int n = t; n < R; n += kFftThreads) {
            // n >= H only in the circular form (R = M)
            const int n0 = n < H ? n : n - H;
            const float2 u = cmulc(z[fpad(n0 + H)], __ldg(tw + n0));
            const float2 r = n < H ? cadd(z[fpad(n0)], u) : csub(z[fpad(n0)], u);
            ox[n] = r.x + dcx;
            if (two) ox[R + n] = r.y + dcy;
        }
    }
}

int launch_filter_fft(const float *in_am, float *out_am, int R, int A, int p, const float2 *d_tab,
                      float g0, bool circ, cudaStream_t st)
{
    if (p < 2 || p > kFilterFftMaxLog || (circ ? (1 << p) != R : (1 << p) < 2 * R - 1))
        return set_error(RG_EUNSUPPORTED, "filter FFT: bad transform size 2^%d for %d rays", p, R);
    const size_t smem = sizeof(float2) * (((size_t)1 << p) + ((size_t)1 << p) / 16);
    RG_CK(cudaFuncSetAttribute(k_filter_fft<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
    RG_CK(launch_pdl(k_filter_fft<false>, (A + 1) / 2, kFftThreads, smem, st, 1, in_am, out_am, R,
                     A, p, d_tab, g0, circ, FilterQuads{}));
    RG_CK_LAUNCH("k_filter_fft");
    return RG_OK;
}

int launch_filter_fft_quads(const float *in_am, int R, int A, int p, const float2 *d_tab, float g0,
                            const View *d_views, int pairs, int roff, float4 *quads, float *out,
                            int N, long long cs, long long ls, cudaStream_t st)
{
    if (p < 2 || p > kFilterFftMaxLog || (1 << p) < 2 * R - 1)
        return set_error(RG_EUNSUPPORTED, "filter FFT: bad transform size 2^%d for %d rays", p, R);
    if (pairs < 1 || roff < 1 || roff >= A)
        return set_error(RG_EINVAL, "filter quads: %d view pairs %d rows apart in %d views",
                         pairs, roff, A);
    const size_t smem = sizeof(float2) * (((size_t)1 << p) + ((size_t)1 << p) / 16);
    RG_CK(cudaFuncSetAttribute(k_filter_fft<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
    RG_CK(launch_pdl(k_filter_fft<true>, pairs, kFftThreads, smem, st, 1, in_am, nullptr, R, A, p,
                     d_tab, g0, false, FilterQuads{d_views, roff, quads, out, N, cs, ls}));
    RG_CK_LAUNCH("k_filter_fft");
    return RG_OK;
}

}  // namespace rg
