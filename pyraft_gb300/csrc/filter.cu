// filter.cu -- the FBP filter step as a row-wise spatial convolution.
//
// out_am[a][n] = sum_{k=0}^{R-1} taps[n - k + R - 1] * in_am[a][k] for every
// view a of a view-major sinogram (rows of length R).  The 2R-1 taps are
// computed on the host in FP64: the discrete Ram-Lak kernel for linear
// convolution, or the periodised spatial form of pyraft's lowpassino_fbp
// filter (pyraft/filters/filters.py:13-68) for circular convolution.
//
// CTA = 256 outputs x 16 views.  The input is walked in tiles of 256
// samples: the tile (16 views, stored [k][view] so one LDS.128 feeds four
// FFMAs) and the 511 taps it meets are staged in shared memory; each thread
// keeps 16 accumulators, i.e. 16 FFMA per 1 + 4 shared loads.  Per-tile
// partial sums are added with Kahan compensation.
#include "rg_internal.cuh"

namespace rg {

constexpr int kTN = 256, kTK = 256, kNA = 16;

__global__ __launch_bounds__(256) void k_conv_rows(const float *__restrict__ in, float *__restrict__ out,
                                                   int R, int A, const float *__restrict__ taps)
{
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
    k_conv_rows<<<grid, 256, 0, st>>>(in_am, out_am, R, A, d_taps);
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
    k_ramlak_rows<<<grid, 256, 0, st>>>(in_am, out_am, R, A, d_godd, h0);
    RG_CK_LAUNCH("k_ramlak_rows");
    return RG_OK;
}

}  // namespace rg
