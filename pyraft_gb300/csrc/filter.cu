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
// out[n] = h0 in[n] + sum_{n-k odd} h[n-k] in[k].  A thread owns the output
// pair (n_e, n_o) = (n0 + 2t, n0 + 2t + 1): the even output meets only odd
// inputs and the odd output only even inputs, both through odd taps.  With
// g[q] = h[2q + 1 - ...] stored compactly (odd taps only), input pair j
// (k_e = k0 + 2j, k_o = k_e + 1) contributes
//     out_e += g[c + t - j] * x[k_o],   out_o += g[c + t - j + 1] * x[k_e],
// so one new tap is loaded per step and the other is the previous step's.
// CTA = 512 outputs x 8 views; inputs walked in tiles of 256 (128 pairs).
constexpr int kRN = 512, kRK = 256, kRA = 8;

// godd[q] = h[2q - 2R + 1] (dt included) for q in [0, 2R): every odd offset
// of [-(2R-1), 2R-1], zero where |m| > R-1.  For the tile (n0, k0) the even
// output's tap has q1 = (n0 - k0)/2 + R - 1 + t - j and the odd output's
// q1 + 1; t - j spans [-(kRK/2 - 1), kRN/2 - 1], so the staged taps start at
// qbase = (n0 - k0)/2 + R - kRK/2 and sg[t - j + kRK/2 - 1] is g1.
__global__ __launch_bounds__(256) void k_ramlak_rows(const float *__restrict__ in,
                                                     float *__restrict__ out, int R, int A,
                                                     const float *__restrict__ godd, float h0)
{
    __shared__ float4 sxe[kRK / 2][kRA / 4];   // even inputs  [pair][view]
    __shared__ float4 sxo[kRK / 2][kRA / 4];   // odd inputs
    __shared__ float sg[kRN / 2 + kRK / 2 + 1];
    const int t = threadIdx.x;
    const int n0 = blockIdx.x * kRN, a0 = blockIdx.y * kRA;
    const int ne = n0 + 2 * t;
    float acc_e[kRA], acc_o[kRA], ce[kRA], co[kRA];
#pragma unroll
    for (int a = 0; a < kRA; ++a) { acc_e[a] = acc_o[a] = ce[a] = co[a] = 0.f; }

    for (int k0 = 0; k0 < R; k0 += kRK) {
        float *xe = reinterpret_cast<float *>(sxe), *xo = reinterpret_cast<float *>(sxo);
        for (int e = t; e < kRK * kRA; e += 256) {
            const int a = e / kRK, kk = e - a * kRK;
            const int k = k0 + kk, av = a0 + a;
            const float v = (k < R && av < A) ? __ldg(in + (size_t)av * R + k) : 0.f;
            if (kk & 1) xo[(kk >> 1) * kRA + a] = v; else xe[(kk >> 1) * kRA + a] = v;
        }
        const int qbase = (n0 - k0) / 2 + R - kRK / 2;
        for (int e = t; e < kRN / 2 + kRK / 2 + 1; e += 256) {
            const int q = qbase + e;
            sg[e] = (q >= 0 && q < 2 * R) ? __ldg(godd + q) : 0.f;
        }
        __syncthreads();
        float pe[kRA], po[kRA];
#pragma unroll
        for (int a = 0; a < kRA; ++a) { pe[a] = po[a] = 0.f; }
        const int jend = min(kRK / 2, (R - k0 + 1) / 2);
        // tap for (n_e, k_o = k0 + 2j + 1): m = ne - k0 - 2j - 1 (odd);
        // its q - qbase = t - j + (kRK / 2 - 1); for (n_o, k_e) it is one more
        float gnext = sg[t + (kRK / 2 - 1) + 1];
#pragma unroll 2
        for (int j = 0; j < jend; ++j) {
            const float g1 = sg[t - j + (kRK / 2 - 1)];
            const float g2 = gnext;
            gnext = g1;
#pragma unroll
            for (int q = 0; q < kRA / 4; ++q) {
                const float4 xo4 = sxo[j][q];
                const float4 xe4 = sxe[j][q];
                pe[4 * q + 0] = fmaf(g1, xo4.x, pe[4 * q + 0]);
                pe[4 * q + 1] = fmaf(g1, xo4.y, pe[4 * q + 1]);
                pe[4 * q + 2] = fmaf(g1, xo4.z, pe[4 * q + 2]);
                pe[4 * q + 3] = fmaf(g1, xo4.w, pe[4 * q + 3]);
                po[4 * q + 0] = fmaf(g2, xe4.x, po[4 * q + 0]);
                po[4 * q + 1] = fmaf(g2, xe4.y, po[4 * q + 1]);
                po[4 * q + 2] = fmaf(g2, xe4.z, po[4 * q + 2]);
                po[4 * q + 3] = fmaf(g2, xe4.w, po[4 * q + 3]);
            }
        }
#pragma unroll
        for (int a = 0; a < kRA; ++a) {
            float y = pe[a] - ce[a], s = acc_e[a] + y;
            ce[a] = (s - acc_e[a]) - y;
            acc_e[a] = s;
            y = po[a] - co[a];
            s = acc_o[a] + y;
            co[a] = (s - acc_o[a]) - y;
            acc_o[a] = s;
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < kRA; ++a) {
        const int av = a0 + a;
        if (av >= A) break;
        const float *row = in + (size_t)av * R;
        if (ne < R) out[(size_t)av * R + ne] = fmaf(h0, __ldg(row + ne), acc_e[a] - ce[a]);
        if (ne + 1 < R) out[(size_t)av * R + ne + 1] = fmaf(h0, __ldg(row + ne + 1), acc_o[a] - co[a]);
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
