// mesh.cu -- slant-stack Radon on an explicit (t, theta) mesh, for single
// slices and for stacks of slices (3-D volumes).
//
// Restates eval_rayintegral_mesh (raft/raft_radon_slantstack_withmesh.c:
// 122-211): the ray integral of the slant-stack Radon with theta_j = theta[j]
// and t_k = t[k] given as vectors instead of uniform grids.  Per view the
// host computes, in FP64 with the host libm, the position of ray t on line i
// as u = t * c1 + r0 + i * ri (samples along the line; lines are image
// columns when |cos| < 1/sqrt 2, rows otherwise, as the reference).  Each
// thread forms its ray's start u0 = t_k * c1 + r0 in FP64 once and converts
// it to Q32.32; the line walk is then the fixed-point walk over the padded
// line pairs of the plain Radon (one 8-byte load per sample, invalid samples
// read zeros).  Every output is computed (the reference's thread split
// drops the remainder, raft/raft_radon_slantstack_withmesh.c:65-67).
// The stack dimension (blockIdx.z) serves pyraft's radon_3d_stack and
// snapshot, which loop over slices in Python (pyraft/sinogram/sino.py:
// 284-342).
#include <math.h>

#include <vector>

#include "ss_tiles.cuh"

namespace rg {

struct MeshView {
    double c1, r0;     // u0 = t * c1 + r0 (samples)
    long long ri;      // Q32.32 step per line
    float delta;       // Delta = dy/|sin| or dx/|cos|
    int flags;         // kLinesAreRows
};

__global__ __launch_bounds__(128) void k_radon_mesh(const float2 *__restrict__ prow,
                                                    const float2 *__restrict__ pcol, int N,
                                                    const MeshView *__restrict__ mv,
                                                    const double *__restrict__ t, int R, int A,
                                                    float *__restrict__ out, long long cs,
                                                    long long ls, long long zp, long long zo)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (k >= R) return;
    const MeshView v = mv[j];
    const int pitch = pairs_pitch(N);
    const float2 *__restrict__ base =
        ((v.flags & kLinesAreRows) ? prow : pcol) + blockIdx.z * zp;
    const double u0d = __dadd_rn(__dmul_rn(t[k], v.c1), v.r0);
    const long long u0 = __double2ll_rn(__dmul_rn(u0d, 4294967296.0));
    int lo, hi;
    radon_line_range(u0, v.ri, N, lo, hi);
    float acc = 0.f, comp = 0.f;
    if (lo <= hi) {
        long long u = u0 + (long long)lo * v.ri;
        const float2 *__restrict__ line = base + (size_t)lo * pitch + 1;
        int i = lo;
        while (i <= hi) {
            const int iend = min(hi, i + 31);
            float part = 0.f;
#pragma unroll 4
            for (; i <= iend; ++i) {
                const float2 pr = __ldg(line + (int)(u >> 32));
                part += fmaf(__uint_as_float(((unsigned)u >> 9) | 0x3F800000u), pr.y, pr.x);
                u += v.ri;
                line += pitch;
            }
            kahan_add(acc, comp, part);
        }
    }
    out[blockIdx.z * zo + (long long)k * cs + (long long)j * ls] = (acc - comp) * v.delta;
}

}  // namespace rg

using namespace rg;

extern "C" {

size_t rg_radon_slantstack_withmesh_workspace(rg_image phantom, rg_image radon, int nstack)
{
    const size_t pb = radon_pairs_bytes(phantom.lines) * (size_t)(nstack < 1 ? 1 : nstack);
    return ws_sum({pb, pb, sizeof(MeshView) * (size_t)radon.columns,
                   sizeof(double) * (size_t)radon.lines});
}

int rg_radon_slantstack_withmesh(rg_image phantom, long long phantom_stride, rg_image radon,
                                 long long radon_stride, int nstack, const double *t,
                                 const double *theta, void *ws, size_t wsb, void *stream)
{
    RG_TRACE();
    int rc = validate_ss(phantom, radon);
    if (!rc) rc = check_ws(ws);
    if (rc) return rc;
    if (!t || !theta) return set_error(RG_EINVAL, "mesh Radon: null t or theta");
    if (nstack < 1 || nstack > 65535) return set_error(RG_EINVAL, "stack size must be in [1, 65535]");
    const int N = phantom.lines, R = radon.lines, A = radon.columns;
    if (A > 65535) return set_error(RG_EINVAL, "mesh Radon: at most 65535 views");
    const double xmin = phantom.tl_x, xmax = phantom.br_x, ymin = phantom.br_y, ymax = phantom.tl_y;
    const double dx = (xmax - xmin) / (N - 1), dy = (ymax - ymin) / (N - 1);
    if (!(std::isfinite(dx) && std::isfinite(dy)) || dx == 0.0 || dy == 0.0)
        return set_error(RG_EINVAL, "degenerate image corners");
    double tmax = 0.0;
    for (int k = 0; k < R; ++k) {
        if (!std::isfinite(t[k])) return set_error(RG_EINVAL, "mesh Radon: non-finite t[%d]", k);
        tmax = std::max(tmax, fabs(t[k]));
    }
    const double tol = 1.0 / sqrt(2);
    std::vector<MeshView> hv(A);
    for (int j = 0; j < A; ++j) {
        const double th = theta[j];
        if (!std::isfinite(th)) return set_error(RG_EINVAL, "mesh Radon: non-finite theta[%d]", j);
        const double c = cos(th), s = sin(th), tn = tan(th);
        MeshView v = {};
        double ri;
        if (fabs(c) < tol) {
            v.c1 = 1.0 / (s * dy);
            ri = -dx / (tn * dy);
            v.r0 = (-xmin / tn - ymin) / dy;
            v.delta = (float)(dy / fabs(s));
        } else {
            v.c1 = 1.0 / (c * dx);
            ri = -dy * tn / dx;
            v.r0 = (-xmin * tn - xmin) / dx;
            v.delta = (float)(dx / fabs(c));
            v.flags = kLinesAreRows;
        }
        if (!(tmax * fabs(v.c1) + fabs(v.r0) + (N - 1) * fabs(ri) < 1073741824.0))
            return set_error(RG_EUNSUPPORTED, "mesh Radon: positions exceed 2^30 samples");
        v.ri = llrint(ri * 4294967296.0);
        hv[j] = v;
    }
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if ((rc = scratch_begin(sc, ws, wsb, rg_radon_slantstack_withmesh_workspace(phantom, radon, nstack),
                            st)))
        return rc;
    const long long zp = (long long)N * pairs_pitch(N);
    float2 *prow = (float2 *)sc.take(radon_pairs_bytes(N) * (size_t)nstack);
    float2 *pcol = (float2 *)sc.take(radon_pairs_bytes(N) * (size_t)nstack);
    MeshView *dv = (MeshView *)sc.take(sizeof(MeshView) * A);
    double *dt = (double *)sc.take(sizeof(double) * R);
    cudaError_t e = cudaMemcpyAsync(dv, hv.data(), sizeof(MeshView) * A, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dt, t, sizeof(double) * R, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) rc = cuda_error(e, "mesh upload");
    if (!rc)
        rc = launch_line_pairs(phantom.data, phantom.column_stride, phantom.line_stride, N, prow,
                               pcol, st, nstack, phantom_stride, zp);
    if (!rc) {
        dim3 grid((R + 127) / 128, A, nstack);
        k_radon_mesh<<<grid, 128, 0, st>>>(prow, pcol, N, dv, dt, R, A, radon.data,
                                           radon.column_stride, radon.line_stride, zp,
                                           radon_stride);
        cudaError_t le = cudaGetLastError();
        if (le != cudaSuccess) rc = cuda_error(le, "k_radon_mesh");
    }
    scratch_end(sc);
    return rc;
}

}  // extern "C"
