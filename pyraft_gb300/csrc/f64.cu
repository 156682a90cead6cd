// f64.cu -- FP64 slant-stack Radon and its exact transpose.
//
// For gradient checks of the autograd operator in float64 (finite
// differences need a forward and backward that are transposes to ~1e-15).
// Both kernels walk the same Q32.32 sample positions as the FP32 Radon
// (u = r0 + k rk + i ri, floor index valid in [0, N-2],
// raft/raft_radon_slantstack.c:174-211) with FP64 weights and sums: the
// forward gathers, the transpose scatters with FP64 atomics into a zeroed
// image.  One thread per (ray, view); meant for small problems (the FP32
// kernels are the fast path).
#include "rg_internal.cuh"

namespace rg {

__global__ void k_radon_f64(const double *__restrict__ img, long long ics, long long ils,
                            int N, const View *__restrict__ views, int nv, int R,
                            double *__restrict__ out, long long ocs, long long ols)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x, e = blockIdx.y;
    if (k >= R || e >= nv) return;
    const View v = views[e];
    const bool rows = v.flags & kLinesAreRows;
    long long u = v.r0 + (long long)k * v.rk;
    double sum = 0.0;
    for (int i = 0; i < N; ++i, u += v.ri) {
        const long long n = u >> 32;
        if (n < 0 || n > N - 2) continue;
        const double w = (double)(unsigned)u * 2.3283064365386962890625e-10;
        const double a = rows ? img[i * ics + n * ils] : img[n * ics + i * ils];
        const double b = rows ? img[i * ics + (n + 1) * ils] : img[(n + 1) * ics + i * ils];
        sum += (1.0 - w) * a + w * b;
    }
    out[(long long)k * ocs + (long long)v.view * ols] = sum * v.delta64;
}

__global__ void k_radon_transpose_f64(const double *__restrict__ sino, long long scs,
                                      long long sls, int N, const View *__restrict__ views,
                                      int nv, int R, double *__restrict__ img)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x, e = blockIdx.y;
    if (k >= R || e >= nv) return;
    const View v = views[e];
    const double sv = sino[(long long)k * scs + (long long)v.view * sls] * v.delta64;
    if (sv == 0.0) return;
    const bool rows = v.flags & kLinesAreRows;
    long long u = v.r0 + (long long)k * v.rk;
    for (int i = 0; i < N; ++i, u += v.ri) {
        const long long n = u >> 32;
        if (n < 0 || n > N - 2) continue;
        const double w = (double)(unsigned)u * 2.3283064365386962890625e-10;
        const long long ia = rows ? (long long)i * N + n : n * N + i;
        const long long ib = rows ? ia + 1 : ia + N;
        atomicAdd(img + ia, sv * (1.0 - w));
        atomicAdd(img + ib, sv * w);
    }
}

int launch_radon_f64(const SSPlan &p, const double *img, long long ics, long long ils,
                     double *out, long long ocs, long long ols, cudaStream_t st)
{
    if (p.nv == 0) return RG_OK;
    dim3 grid((p.g.R + 127) / 128, p.nv);
    k_radon_f64<<<grid, 128, 0, st>>>(img, ics, ils, p.g.N, p.d_views, p.nv, p.g.R, out, ocs, ols);
    RG_CK_LAUNCH("k_radon_f64");
    return RG_OK;
}

// img_c: contiguous N x N, zeroed by the caller.
int launch_radon_transpose_f64(const SSPlan &p, const double *sino, long long scs, long long sls,
                               double *img_c, cudaStream_t st)
{
    if (p.nv == 0) return RG_OK;
    dim3 grid((p.g.R + 127) / 128, p.nv);
    k_radon_transpose_f64<<<grid, 128, 0, st>>>(sino, scs, sls, p.g.N, p.d_views, p.nv, p.g.R,
                                                img_c);
    RG_CK_LAUNCH("k_radon_transpose_f64");
    return RG_OK;
}

}  // namespace rg
