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
