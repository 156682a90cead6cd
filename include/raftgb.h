/*
 * raftgb.h -- C ABI of libraftgb.so, the GB300 (sm_103a) implementation of
 * pyraft's reconstruction hot path: slant-stack Radon, its backprojection and
 * matched adjoint, the DDA (Bresenham) projector pair, the ramp filter step,
 * and the EM/OSEM multiplicative update.
 *
 * Conventions shared by every entry point
 *  - Images and sinograms are passed as rg_image, which mirrors the
 *    reference's raft_image (raft/raft_image.h:11-19, raft/raft_matrix.h:
 *    11-19, marshalled by pyraft/raftypes.py:85-100,413-449): element (i, j)
 *    lives at data[i * column_stride + j * line_stride]; tl_/br_ give the
 *    top-left / bottom-right corners.  Sinograms are (nrays x nviews): line =
 *    ray, column = view, as in raft/raft_radon_slantstack.c:114.  Unlike the
 *    reference (host double*), data is a DEVICE float* owned by the caller.
 *  - The reference passes `int nthreads` and blocks; here every operator
 *    takes a CUDA stream (cudaStream_t passed as void*, NULL = legacy default
 *    stream) and returns as soon as the work is queued.
 *  - Scratch: operators need device scratch memory.  Pass `workspace` /
 *    `workspace_bytes` (size from the matching *_workspace query), or
 *    workspace == NULL to let the call take stream-ordered memory from the
 *    device's default pool (cudaMallocAsync/cudaFreeAsync on `stream`).
 *  - Every entry point returns RG_OK (0) or a negative RG_E* code; the text
 *    of the last error on the calling thread is available from
 *    rg_last_error().  The reference reports no errors at all (its
 *    allocation failures silently return, raft/raft_filter.cpp:131-133).
 *  - Nothing here calls cudaDeviceReset (the reference's GPU wrappers do,
 *    raft/raft_radon_gpu.cu:34) and no call synchronises the device, except
 *    the *_host convenience wrappers, which return when their result is in
 *    host memory.
 *  - Plans: per-view constants are computed on the host in FP64 (with the
 *    host libm, the same cos/sin/tan the reference evaluates) and uploaded
 *    once per geometry.  The rg_image entry points keep a small per-device
 *    cache of plans keyed by geometry; the rg_plan_* entry points expose
 *    them for CUDA-graph capture and batching.
 */
#ifndef RAFTGB_H
#define RAFTGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RG_OK            0
#define RG_EINVAL       -1   /* bad size, stride, corner or pointer         */
#define RG_ECUDA        -2   /* a CUDA runtime call or kernel launch failed */
#define RG_ENOMEM       -3   /* device or host allocation failed            */
#define RG_EUNSUPPORTED -4   /* geometry outside what the kernels handle    */
#define RG_EWORKSPACE   -5   /* workspace smaller than the query returned   */

typedef struct {
    float *data;          /* device pointer                                  */
    int lines;            /* rows                                            */
    int line_stride;      /* distance between elements of one row (floats)   */
    int columns;          /* columns                                         */
    int column_stride;    /* distance between rows (floats)                  */
    double tl_x, tl_y;    /* top-left corner                                 */
    double br_x, br_y;    /* bottom-right corner                             */
} rg_image;

/* Method ids, as raft/raft_enums.h:4-9 and pyraft/sinogram/sino.py:159-167. */
#define RG_BRESENHAM  1
#define RG_SLANTSTACK 2
/* EM only: slant-stack Radon with the slant-stack BACKPROJECTION as the EM
 * backprojector (x <- x * B(y / Ax) / B1), the operator pair of
 * raft_em_gpu (raft/raft_em_gpu.cu:20-87); not a transpose pair. */
#define RG_SLANTSTACK_BP 3

/* Text of the last error on this thread ("" if none). */
const char *rg_last_error(void);
/* ABI version (major * 100 + minor). */
int rg_version(void);
/* Error bits that kernels with in-kernel checks recorded on the current
 * device since the last call, then cleared (synchronises the device):
 * 1 = a Radon window check failed (a TMA-staged strip, or a ray of the
 *     tile-driven Radon, was skipped rather than read out of bounds),
 * 2 = a bounded wait for an asynchronous copy ran out.  0 = none; a
 * negative RG_E* code if the query itself failed.  No counterpart in the
 * reference, whose kernels have no such checks. */
int rg_device_status(void);

/* ----------------------------------------------------------------------
 * Slant-stack projector family (square images).
 * -------------------------------------------------------------------- */

/* Radon transform, ray-driven line integral with linear interpolation.
 * Replaces raft_radon_slantstack (raft/raft_radon_slantstack.c:44,
 * declared raft/raft_radon_slantstack.h:10; bound at pyraft/raftypes.py:159).
 * phantom: size x size; radon: nrays x nviews.                              */
size_t rg_radon_slantstack_workspace(rg_image phantom, rg_image radon);
int rg_radon_slantstack(rg_image phantom, rg_image radon,
                        void *workspace, size_t workspace_bytes, void *stream);

/* Same Radon transform for callers that cannot allocate device memory (no
 * counterpart in the reference): a process whose device memory is already
 * committed to another framework's pool, or an acquisition loop that must
 * not allocate once it runs (cudaMalloc/cudaFree may synchronise the whole
 * device).  All scratch (per-view table, line pairs, result staging) lives
 * in one static 32 MiB device array that every GPU loading the library
 * holds until exit; the call makes no cudaMalloc, cudaFree or other
 * allocation.  Geometries needing more scratch (about size 1200 with 1800
 * views and as many rays) or more than 4096 views are rejected with
 * RG_EINVAL.  The first call on a device (and the first after its context
 * was replaced) resolves the array's device address with
 * cudaGetSymbolAddress; make that first call before any stream capture
 * begins on the device.  Calls share the array, so calls that overlap on
 * the GPU race; each call rewrites all the scratch it reads, so nothing
 * needs clearing between calls.                                             */
int rg_radon_slantstack_noalloc(rg_image phantom, rg_image radon, void *stream);

/* Pixel-driven backprojection with linear interpolation in t, scaled by
 * the view spacing.  Replaces raft_backprojection_slantstack
 * (raft/raft_backprojection_slantstack.c:43; bound at pyraft/raftypes.py:161).
 * Not the transpose of rg_radon_slantstack, exactly like the reference.    */
size_t rg_backprojection_slantstack_workspace(rg_image sinogram, rg_image backprojection);
int rg_backprojection_slantstack(rg_image sinogram, rg_image backprojection,
                                 void *workspace, size_t workspace_bytes, void *stream);

/* Matched adjoint: the exact transpose of rg_radon_slantstack (the
 * reference has none; pyraft's radon_transpose offers only the DDA pair,
 * pyraft/backprojection/backprojection.py:220-233).  Backward pass of the
 * autograd Radon and backprojector of the EM/OSEM update.                   */
size_t rg_radon_transpose_slantstack_workspace(rg_image sinogram, rg_image image);
int rg_radon_transpose_slantstack(rg_image sinogram, rg_image image,
                                  void *workspace, size_t workspace_bytes, void *stream);

/* Stacks of equal-geometry problems in one launch per kernel (grid z).
 * phantom/image/radon/sino describe the first member; consecutive members
 * are *_stride floats apart.  Same results as nstack separate calls.  Used
 * by the batched autograd operator (no reference counterpart: the
 * reference loops over slices in Python, pyraft/sinogram/sino.py:307-310). */
size_t rg_radon_slantstack_stack_workspace(rg_image phantom, rg_image radon, int nstack);
int rg_radon_slantstack_stack(rg_image phantom, long long phantom_stride, rg_image radon,
                              long long radon_stride, int nstack,
                              void *workspace, size_t workspace_bytes, void *stream);
size_t rg_radon_transpose_slantstack_stack_workspace(rg_image sino, rg_image image, int nstack);
int rg_radon_transpose_slantstack_stack(rg_image sino, long long sino_stride, rg_image image,
                                        long long image_stride, int nstack,
                                        void *workspace, size_t workspace_bytes, void *stream);

/* FP64 slant-stack Radon and its exact transpose (same sample positions,
 * FP64 weights and sums; the transpose scatters with FP64 atomics into a
 * contiguous image it zeroes first).  For float64 gradient checks of the
 * autograd operator; the FP32 entry points above are the fast path.  The
 * layout is rg_image's with double data.  (The reference's C path is FP64,
 * raft/raft_radon_slantstack.c:122-214; no transpose exists there.)        */
typedef struct {
    double *data;
    int lines, line_stride, columns, column_stride;
    double tl_x, tl_y, br_x, br_y;
} rg_image_f64;
int rg_radon_slantstack_f64(rg_image_f64 phantom, rg_image_f64 radon, void *stream);
int rg_radon_transpose_slantstack_f64(rg_image_f64 sino, rg_image_f64 image, void *stream);

/* ----------------------------------------------------------------------
 * DDA (Bresenham) projector pair (rectangular images, top-down rows).
 * -------------------------------------------------------------------- */

/* Replaces raft_radon_bresenham (raft/raft_radon_bresenham.cpp:63;
 * bound at pyraft/raftypes.py:152).                                         */
size_t rg_radon_bresenham_workspace(rg_image image, rg_image sino);
int rg_radon_bresenham(rg_image image, rg_image sino,
                       void *workspace, size_t workspace_bytes, void *stream);

/* Replaces raft_radon_transpose_bresenham
 * (raft/raft_radon_transpose_bresenham.cpp:97; bound at pyraft/raftypes.py:156). */
size_t rg_radon_transpose_bresenham_workspace(rg_image sino, rg_image image);
int rg_radon_transpose_bresenham(rg_image sino, rg_image image,
                                 void *workspace, size_t workspace_bytes, void *stream);

/* Normalised backprojection: per pixel sum(s * sigma) / sum(sigma) over
 * every ray step through it; 0 where no ray passes (the reference divides
 * 0 by 0).  Replaces raft_backprojection_bresenham
 * (raft/raft_backprojection_bresenham.cpp:17-251; bound at
 * pyraft/raftypes.py:154, called by backprojection(), pyraft/backprojection/
 * backprojection.py:188-189).                                               */
size_t rg_backprojection_bresenham_workspace(rg_image sino, rg_image image);
int rg_backprojection_bresenham(rg_image sino, rg_image image,
                                void *workspace, size_t workspace_bytes, void *stream);

/* Pixel index sequences of a list of rays, for checking the traversal:
 * replaces stepping raft_ddaiterator_set_theta/_set_t/_update/_end
 * (raft/raft_ddaiterator.h:26-33) by hand.  thetas, ts: nrays_in HOST
 * doubles (cos/sin are taken on the host, as the reference does);
 * out_i/out_j/out_sigma: nrays_in * cap DEVICE entries (ray r at offset
 * r*cap); out_count: nrays_in device ints (full step counts).  Synchronous. */
int rg_dda_trace(int lines, int columns, const double img_corners[4],
                 const double *thetas, const double *ts, int nrays_in, int cap,
                 int *out_i, int *out_j, double *out_sigma, int *out_count,
                 void *stream);

/* Slant-stack Radon on an explicit mesh: t (radon.lines host doubles) and
 * theta (radon.columns host doubles) replace the uniform grids; the corners
 * of `radon` are not used.  nstack slices in one launch (consecutive ones
 * *_stride floats apart).  Replaces raft_radon_slantstack_withmesh
 * (raft/raft_radon_slantstack_withmesh.c:45; bound at pyraft/raftypes.py:176,
 * called by radon_withmesh / radon_3d_stack, pyraft/sinogram/sino.py:251-311). */
size_t rg_radon_slantstack_withmesh_workspace(rg_image phantom, rg_image radon, int nstack);
int rg_radon_slantstack_withmesh(rg_image phantom, long long phantom_stride, rg_image radon,
                                 long long radon_stride, int nstack, const double *t,
                                 const double *theta, void *workspace, size_t workspace_bytes,
                                 void *stream);

/* ----------------------------------------------------------------------
 * Ramp filter step of FBP: row-wise spatial convolution along t.
 * kind RG_FILTER_RAMLAK: discrete Ram-Lak kernel, linear convolution,
 *   q[n] = dt * sum_k h[n-k] p[k], h[0] = 1/(4dt^2), h[odd m] =
 *   -1/(pi^2 m^2 dt^2) (replaces the FFT ramp of raft_filter1d_ramp,
 *   raft/raft_filter.cpp:184, bound at pyraft/raftypes.py:185).
 * kind RG_FILTER_LOWPASS: the cosine-windowed ramp of pyraft's
 *   lowpassino_fbp (pyraft/filters/filters.py:13-68), applied as the
 *   equivalent circular convolution.
 * in and out: nrays x nviews; may be the same image.                        */
#define RG_FILTER_RAMLAK  1
#define RG_FILTER_LOWPASS 2
size_t rg_filter_workspace(rg_image sino, int kind);
int rg_filter(rg_image sino_in, rg_image sino_out, int kind,
              void *workspace, size_t workspace_bytes, void *stream);

/* FBP: filter + slant-stack backprojection (replaces raft_fbp,
 * raft/raft_fbp.c:5-24, and pyraft's fbp_gpu, pyraft/inversion/inversion.py:32). */
size_t rg_fbp_workspace(rg_image sino, rg_image image, int kind);
int rg_fbp(rg_image sino, rg_image image, int kind,
           void *workspace, size_t workspace_bytes, void *stream);

/* ----------------------------------------------------------------------
 * EM / OSEM (emission MLEM, x <- x * A^T(y / Ax) / A^T 1).
 * Replaces raft_em_gpu (raft/raft_em_gpu.cu:20, bound at
 * pyraft/raftypes.py:211) and pyraft's make_em/em
 * (pyraft/iterative/em.py:109-169).  image holds x0 on entry and the
 * iterate on return.  method RG_SLANTSTACK uses the slant-stack Radon with
 * its matched adjoint (true MLEM); RG_SLANTSTACK_BP the slant-stack Radon
 * with the slant-stack backprojection, as raft_em_gpu pairs them;
 * RG_BRESENHAM the DDA pair, as pyraft's em().
 * nsubsets == 1 is plain EM; > 1 is OSEM over interleaved view subsets
 * (subset s = views s, s+S, s+2S, ...).  Guards: y/0 -> 0, and pixels with
 * zero sensitivity are set to 0 (the reference divides by zero).
 * The sensitivity A^T 1 is accumulated in FP64.
 * RG_BRESENHAM with niter >= 2 also allocates, outside the workspace, device
 * memory for the rays' walks recorded once and replayed each sub-iteration
 * (4 bytes per traversal step: 3.2 GB at 1024^2 x 720), within a third of
 * the free device memory and RG_DDA_PLAN_MAX_GB (48 by default), freed
 * before return; RG_DDA_PLAN=0 walks every time instead.                   */
size_t rg_em_workspace(rg_image sino, rg_image image, int method, int nsubsets);
int rg_em(rg_image sino, rg_image image, int method, int niter, int nsubsets,
          void *workspace, size_t workspace_bytes, void *stream);

/* The same EM/OSEM loop over a range of sub-iterations, for checkpointing
 * and resuming a long reconstruction (the reference keeps no loop state;
 * its iterates are only pickled, pyraft/raftypes.py:369-390): runs
 * sub-iterations first .. first + count - 1 from the iterate in image,
 * where sub-iteration j uses subset j mod nsubsets (rg_em runs 0 ..
 * niter * nsubsets - 1).  Splitting a run into ranges gives the same
 * iterate as one call, up to the rounding order of the tile-driven Radon's
 * atomic ray sums (OSEM subsets).  Workspace: rg_em_workspace.             */
int rg_em_subiterations(rg_image sino, rg_image image, int method, int nsubsets,
                        long long first, long long count, void *workspace,
                        size_t workspace_bytes, void *stream);

/* Transmission EM: x <- x * A^T(b exp(-A x)) / A^T y with
 * y = max(rawsino - dark, 0), b = max(flat - dark, 0) (dark.data may be
 * NULL: no dark field); slant-stack Radon with the exp fused into its
 * epilogue, matched adjoint with the update fused.  Replaces raft_tr_em_gpu
 * (raft/raft_transmission_em.cu:16-77), whose update multiplies twice per
 * iteration (:57,59) and whose Python caller passes one argument too many
 * (pyraft/iterative/em.py:246); image holds x0 on entry.                    */
size_t rg_em_transmission_workspace(rg_image rawsino, rg_image image);
int rg_em_transmission(rg_image rawsino, rg_image flat, rg_image dark, rg_image image,
                       int niter, void *workspace, size_t workspace_bytes, void *stream);

/* ----------------------------------------------------------------------
 * Batched uneven OSEM: nslices independent reconstructions of different
 * sizes and view counts.  Each sub-iteration is three persistent launches
 * (line pairs, Radon + ratio, adjoint + update) over (slice, tile) work
 * queues.  Each slice k reads sinos[k] and updates images[k] in place
 * (images hold x0 on entry).  Work runs on `stream`; with graph != 0 one
 * iteration is captured into a CUDA graph on a private stream and replayed
 * niter times on `stream` (do not call it while `stream` is itself being
 * captured).  1 <= nsubsets <= 64, nsubsets <= every slice's view count.
 * Replaces the reference's Python loop radon_3d_stack / per-slice em calls
 * (pyraft/sinogram/sino.py:284-311, pyraft/iterative/em.py:151-169).       */
size_t rg_osem_batch_workspace(const rg_image *sinos, const rg_image *images,
                               int nslices, int nsubsets);
int rg_osem_batch(const rg_image *sinos, rg_image *images, int nslices,
                  int niter, int nsubsets, int graph,
                  void *workspace, size_t workspace_bytes, void *stream);

/* The plain one-slice-per-call form the batched path is measured against:
 * one slice (host float buffers, default geometry as the *_host wrappers),
 * OSEM with nsubsets interleaved subsets (1 = plain EM), handled the way
 * the reference's GPU EM handles a slice (raft/raft_em_gpu.cu:20-87): per
 * call allocation and upload, then per sub-iteration separate Radon, ratio,
 * backprojection, divide and multiply launches, each followed by a device
 * synchronisation, with one-thread-per-output kernels (float positions,
 * global loads); download and free.  Same operators (slant-stack Radon and
 * matched adjoint) as rg_osem_batch.  h_out receives the iterate from x0 = 1. */
int rg_em_plain_host(float *h_out, const float *h_sino, int size_image, int nrays,
                     int nangles, int niter, int nsubsets);

/* ----------------------------------------------------------------------
 * Ellipse phantoms (test inputs; replace raft_image_phantom_fromdesc,
 * raft/raft_image_phantom_fromdesc.c:4, and raft_radon_fromdesc,
 * raft/raft_radon_fromdesc.c:4).  desc: host (n x 6) row-major doubles
 * [alpha, a, b, x0, y0, theta]; results are ADDED into image / sino.         */
int rg_phantom_fromdesc(rg_image image, const double *desc, int n, void *stream);

/* Smoothed isotropic total variation of nslices contiguous size x size device
 * images x: *value (device double) = sum sqrt(dx^2 + dy^2 + eps^2) with
 * forward differences and the last row / column replicated; grad (device,
 * same shape as x, or NULL) receives its gradient.  For TV-regularised
 * reconstructions built on the operator pair; no counterpart in the
 * reference.                                                                */
int rg_tv(const float *x, int nslices, int size, float eps, double *value, float *grad,
          void *stream);
int rg_radon_fromdesc(rg_image sino, const double *desc, int n, void *stream);

/* ----------------------------------------------------------------------
 * Host-pointer convenience wrappers, the shape of the reference's GPU entry
 * points (raft/raft_radon_gpu.h:8, raft/raft_backprojection_gpu.h:8,
 * raft/raft_em_gpu.cu:20): float host buffers, default [-1,1]^2 image, views
 * on [0, pi) and rays on [-1, 1]; allocate, copy, run, copy back, free.
 * Unlike the reference they return a status and do not reset the device.
 * The backprojection wrapper computes the C slant-stack backprojection
 * (not the reference GPU kernel's nearest-sample, x-flipped variant); the
 * EM wrapper pairs the slant-stack Radon with it (RG_SLANTSTACK_BP), as
 * raft_em_gpu pairs its Radon with its backprojection.                     */
int rg_radon_slantstack_host(float *h_output, const float *h_input,
                             int size_image, int nrays, int nangles);
int rg_backprojection_slantstack_host(float *h_image, const float *h_sino,
                                      int size_image, int nrays, int nangles);
int rg_em_host(float *h_output, const float *h_sino, int size_image,
               int nrays, int nangles, int niter);

#ifdef __cplusplus
}
#endif

#endif /* RAFTGB_H */
