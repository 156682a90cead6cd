// aux.cu -- layout changes and ellipse phantoms.
//
// Sinograms cross the API as (nrays x nviews) strided views (line = ray,
// column = view, raft/raft_radon_slantstack.c:114).  Inside the library the
// projectors work on the view-major transpose S_am[view][ray] so that a
// view's samples are contiguous; these kernels convert with 32 x 32
// shared-memory tiles so that both the read and the write are coalesced.
#include <math.h>

#include <algorithm>

#include "rg_internal.cuh"

namespace rg {

// out_am[j * R + k] = in[k * cs + j * ls]
// blockIdx.z: one sinogram of a stack (zi, zo: strides in floats).
__global__ __launch_bounds__(256) void k_to_am(const float *__restrict__ in, long long cs,
                                               long long ls, int R, int A,
                                               float *__restrict__ out, long long zi,
                                               long long zo)
{
    pdl_gate();
    in += blockIdx.z * zi;
    out += blockIdx.z * zo;
    __shared__ float t[32][33];
    const int k0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int y = w; y < 32; y += 8) {
        int k = k0 + y, j = j0 + lane;
        t[y][lane] = (k < R && j < A) ? in[(long long)k * cs + (long long)j * ls] : 0.f;
    }
    __syncthreads();
    for (int x = w; x < 32; x += 8) {
        int j = j0 + x, k = k0 + lane;
        if (k < R && j < A) out[(size_t)j * R + k] = t[lane][x];
    }
}

// out[k * cs + j * ls] = am[j * R + k]
// ADD: out += the transposed view-major array, instead of out =.
template <bool ADD>
__global__ __launch_bounds__(256) void k_from_am(const float *__restrict__ am, int R, int A,
                                                 float *__restrict__ out, long long cs,
                                                 long long ls, long long zi, long long zo)
{
    pdl_gate();
    am += blockIdx.z * zi;
    out += blockIdx.z * zo;
    __shared__ float t[32][33];
    const int k0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int x = w; x < 32; x += 8) {
        int j = j0 + x, k = k0 + lane;
        t[lane][x] = (k < R && j < A) ? am[(size_t)j * R + k] : 0.f;
    }
    __syncthreads();
    for (int y = w; y < 32; y += 8) {
        int k = k0 + y, j = j0 + lane;
        if (k < R && j < A) {
            float *o = out + (long long)k * cs + (long long)j * ls;
            *o = ADD ? *o + t[y][lane] : t[y][lane];
        }
    }
}

int launch_to_am(const float *in, long long cs, long long ls, int R, int A, float *out_am,
                 cudaStream_t st, int nz, long long zi, long long zo)
{
    dim3 grid((A + 31) / 32, (R + 31) / 32, nz);
    RG_CK(launch_pdl(k_to_am, grid, 256, 0, st, 1, in, cs, ls, R, A, out_am, zi, zo));
    RG_CK_LAUNCH("k_to_am");
    return RG_OK;
}

int launch_from_am(const float *am, int R, int A, float *out, long long cs, long long ls,
                   cudaStream_t st, int nz, long long zi, long long zo)
{
    dim3 grid((A + 31) / 32, (R + 31) / 32, nz);
    RG_CK(launch_pdl(k_from_am<false>, grid, 256, 0, st, 1, am, R, A, out, cs, ls, zi, zo));
    RG_CK_LAUNCH("k_from_am");
    return RG_OK;
}

int launch_add_from_am(const float *am, int R, int A, float *out, long long cs, long long ls,
                       cudaStream_t st)
{
    dim3 grid((A + 31) / 32, (R + 31) / 32, 1);
    RG_CK(launch_pdl(k_from_am<true>, grid, 256, 0, st, 1, am, R, A, out, cs, ls, 0, 0));
    RG_CK_LAUNCH("k_from_am (add)");
    return RG_OK;
}

__global__ void k_copy2d(const float *__restrict__ in, long long ics, long long ils,
                         float *__restrict__ out, long long ocs, long long ols, int rows, int cols)
{
    pdl_gate();
    const int c = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y;
    if (c < cols) out[(long long)r * ocs + (long long)c * ols] = in[(long long)r * ics + (long long)c * ils];
}

int launch_copy2d(const float *in, long long ics, long long ils, float *out, long long ocs,
                  long long ols, int rows, int cols, cudaStream_t st)
{
    if (rows <= 0 || cols <= 0) return RG_OK;
    dim3 grid((cols + 255) / 256, rows);
    RG_CK(launch_pdl(k_copy2d, grid, 256, 0, st, 1, in, ics, ils, out, ocs, ols, rows, cols));
    RG_CK_LAUNCH("k_copy2d");
    return RG_OK;
}

__global__ void k_fill(float *p, size_t n, float v)
{
    pdl_gate();
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
         e += (size_t)gridDim.x * blockDim.x)
        p[e] = v;
}

int launch_fill(float *p, size_t n, float v, cudaStream_t st)
{
    if (n == 0) return RG_OK;
    int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
    RG_CK(launch_pdl(k_fill, blocks, 256, 0, st, 1, p, n, v));
    RG_CK_LAUNCH("k_fill");
    return RG_OK;
}

// ----------------------------------------------------------------------------
// Ellipse phantoms, FP64 so the inside test matches the reference bit for bit
// (raft/raft_image_phantom_fromdesc.c:4-59).  Each desc row is pre-expanded
// on the host to [alpha, a, b, x0, y0, cos(theta), sin(theta)] so the trig
// values are the host libm's, as in the reference.

__global__ void k_phantom(float *__restrict__ img, long long cs, long long ls, int lines,
                          int cols, double tl_x, double tl_y, double xs, double ys,
                          const double *__restrict__ d, int n)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (j >= cols) return;
    // FP64 accumulation as the reference's double image, rounded once.
    double acc = img[(long long)i * cs + (long long)j * ls];
    for (int e = 0; e < n; ++e) {
        const double *q = d + 7 * e;
        const double alpha = q[0], a = q[1], b = q[2], x0 = q[3], y0 = q[4], c = q[5], s = q[6];
        const double x = __dsub_rn(__dadd_rn(tl_x, __dmul_rn(j, xs)), x0);
        const double y = __dsub_rn(__dadd_rn(tl_y, __dmul_rn(i, ys)), y0);
        double val = __dadd_rn(__dmul_rn(y, s), __dmul_rn(x, c));
        val = __ddiv_rn(val, a);
        val = __dmul_rn(val, val);
        double tmp = __dsub_rn(__dmul_rn(y, c), __dmul_rn(x, s));
        tmp = __ddiv_rn(tmp, b);
        tmp = __dmul_rn(tmp, tmp);
        val = __dadd_rn(val, tmp);
        val = __dsqrt_rn(val);
        if (val <= 1.0) acc = __dadd_rn(acc, alpha);
    }
    img[(long long)i * cs + (long long)j * ls] = (float)acc;
}

int launch_phantom(float *img, long long cs, long long ls, int lines, int cols, double tl_x,
                   double tl_y, double br_x, double br_y, const double *d_desc, int n,
                   cudaStream_t st)
{
    const double xs = (br_x - tl_x) / (cols - 1), ys = (br_y - tl_y) / (lines - 1);
    dim3 grid((cols + 127) / 128, lines);
    k_phantom<<<grid, 128, 0, st>>>(img, cs, ls, lines, cols, tl_x, tl_y, xs, ys, d_desc, n);
    RG_CK_LAUNCH("k_phantom");
    return RG_OK;
}

// Analytic line integrals of the ellipses (raft/raft_radon_fromdesc.c:4-67);
// views endpoint-inclusive.  Per ellipse, the host pre-computes per view
// nothing: d holds [alpha, a, b, x0, y0, theta_e] and the view trig comes
// from `cs_view` (2 * cols doubles: cos, sin of each view, host libm) and
// `csp_view` (cos, sin of theta_view - theta_e per ellipse and view).
__global__ void k_radon_fromdesc(float *__restrict__ sino, long long cs, long long ls, int lines,
                                 int cols, double tl_y, double tss, const double *__restrict__ d,
                                 int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= lines) return;
    const double *cv = d + 6 * n;                  // [cols][2] view cos/sin
    const double *cp = cv + 2 * cols;              // [n][cols][2] cos/sin(theta - theta_e)
    double acc = sino[(long long)i * cs + (long long)j * ls];
    const double c = cv[2 * j], s = cv[2 * j + 1];
    for (int e = 0; e < n; ++e) {
        const double *q = d + 6 * e;
        const double ea = q[0], ax = q[1], bx = q[2], ex = q[3], ey = q[4];
        const double cpp = cp[(size_t)(e * cols + j) * 2], spp = cp[(size_t)(e * cols + j) * 2 + 1];
        double m = __ddiv_rn(1.0, __dsqrt_rn(__dadd_rn(__ddiv_rn(__dmul_rn(cpp, cpp), __dmul_rn(bx, bx)),
                                                         __ddiv_rn(__dmul_rn(spp, spp), __dmul_rn(ax, ax)))));
        double mab = __ddiv_rn(m, __dmul_rn(ax, bx));
        m = __dmul_rn(m, 2.0);
        m = __dmul_rn(m, ea);
        const double delt = __dmul_rn(mab, __dsub_rn(__dadd_rn(__dmul_rn(ex, c), __dmul_rn(ey, s)), tl_y));
        mab = __dmul_rn(mab, tss);
        double tp = __dsub_rn(__dmul_rn(mab, (double)i), delt);
        tp = __dmul_rn(tp, tp);
        if (tp <= 1.0) acc = __dadd_rn(acc, __dmul_rn(m, __dsqrt_rn(__dsub_rn(1.0, tp))));
    }
    sino[(long long)i * cs + (long long)j * ls] = (float)acc;
}

int launch_radon_fromdesc(float *sino, long long cs, long long ls, int lines, int cols,
                          double tl_x, double tl_y, double br_x, double br_y,
                          const double *d_desc, int n, cudaStream_t st)
{
    (void)tl_x; (void)br_x;
    const double tss = (br_y - tl_y) / (lines - 1);
    dim3 grid((lines + 127) / 128, cols);
    k_radon_fromdesc<<<grid, 128, 0, st>>>(sino, cs, ls, lines, cols, tl_y, tss, d_desc, n);
    RG_CK_LAUNCH("k_radon_fromdesc");
    return RG_OK;
}

}  // namespace rg

namespace rg {

// x <- x * bp * inv_sens (EM update; inv_sens is 0 where the sensitivity is 0)
__global__ void k_em_update(float *__restrict__ x, const float *__restrict__ bp,
                            const float *__restrict__ inv, size_t n)
{
    pdl_gate();
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
         e += (size_t)gridDim.x * blockDim.x)
        x[e] = x[e] * bp[e] * inv[e];
}

__global__ void k_invert(const float *__restrict__ s, float *__restrict__ inv, size_t n)
{
    pdl_gate();
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
         e += (size_t)gridDim.x * blockDim.x)
        inv[e] = (s[e] > 0.f) ? 1.f / s[e] : 0.f;
}

__global__ void k_sub_clamp(const float *__restrict__ a, const float *__restrict__ b,
                            float *__restrict__ o, size_t n)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
         e += (size_t)gridDim.x * blockDim.x)
        o[e] = fmaxf(a[e] - (b ? b[e] : 0.f), 0.f);
}

int launch_sub_clamp(const float *a, const float *b, float *out, size_t n, cudaStream_t st)
{
    if (n == 0) return RG_OK;
    int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
    k_sub_clamp<<<blocks, 256, 0, st>>>(a, b, out, n);
    RG_CK_LAUNCH("k_sub_clamp");
    return RG_OK;
}

int launch_em_update(float *x, const float *bp, const float *inv, size_t n, cudaStream_t st)
{
    if (n == 0) return RG_OK;
    int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
    RG_CK(launch_pdl(k_em_update, blocks, 256, 0, st, 1, x, bp, inv, n));
    RG_CK_LAUNCH("k_em_update");
    return RG_OK;
}

int launch_invert(const float *sens, float *inv, size_t n, cudaStream_t st)
{
    if (n == 0) return RG_OK;
    int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
    RG_CK(launch_pdl(k_invert, blocks, 256, 0, st, 1, sens, inv, n));
    RG_CK_LAUNCH("k_invert");
    return RG_OK;
}


// ----------------------------------------------------------------------------
// Smoothed isotropic total variation of a stack of N x N images,
// sum sqrt(dx^2 + dy^2 + eps^2) with forward differences and the last row /
// column replicated (so its difference is identically 0), and its gradient.
// One thread per pixel (32 x 8 per CTA, grid z = image): the pixel's own term
// and those of its left and upper neighbours, whose differences it enters.
// The value is summed per CTA in FP32 and across CTAs in FP64.
__global__ __launch_bounds__(256) void k_tv(const float *__restrict__ x, int N, float eps,
                                            double *__restrict__ value,
                                            float *__restrict__ grad)
{
    const int j = blockIdx.x * 32 + (threadIdx.x & 31), i = blockIdx.y * 8 + (threadIdx.x >> 5);
    const size_t off = (size_t)blockIdx.z * N * N;
    x += off;
    const float e2 = eps * eps;
    float g = 0.f;
    if (i < N && j < N) {
        const float c = x[(size_t)i * N + j];
        const float r = j + 1 < N ? x[(size_t)i * N + j + 1] : c;
        const float d = i + 1 < N ? x[(size_t)(i + 1) * N + j] : c;
        const float dx = r - c, dy = d - c;
        g = sqrtf(dx * dx + dy * dy + e2);
        if (grad) {
            float gr = -(dx + dy) / g;
            if (j >= 1) {                                 // left neighbour's dx = c - l
                const float l = x[(size_t)i * N + j - 1];
                const float ld = i + 1 < N ? x[(size_t)(i + 1) * N + j - 1] : l;
                const float ax = c - l, ay = ld - l;
                gr += ax / sqrtf(ax * ax + ay * ay + e2);
            }
            if (i >= 1) {                                 // upper neighbour's dy = c - u
                const float u = x[(size_t)(i - 1) * N + j];
                const float ur = j + 1 < N ? x[(size_t)(i - 1) * N + j + 1] : u;
                const float bx = ur - u, by = c - u;
                gr += by / sqrtf(bx * bx + by * by + e2);
            }
            grad[off + (size_t)i * N + j] = gr;
        }
    }
    // CTA sum of the values
    __shared__ float red[8];
    float v = g;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < 8; ++w) t += red[w];
        atomicAdd(value, (double)t);
    }
}

int launch_tv(const float *x, int nz, int N, float eps, double *value, float *grad,
              cudaStream_t st)
{
    RG_CK(cudaMemsetAsync(value, 0, sizeof(double), st));
    dim3 grid((N + 31) / 32, (N + 7) / 8, nz);
    k_tv<<<grid, 256, 0, st>>>(x, N, eps, value, grad);
    RG_CK_LAUNCH("k_tv");
    return RG_OK;
}

}  // namespace rg
