/*
 * oracle/blas_shim.c -- the two Fortran-BLAS level-1 routines that the
 * reference's Bresenham sources link against (dcopy_ and daxpy_, called from
 * raft/raft_radon_bresenham.cpp:28, raft/raft_radon_transpose_bresenham.cpp:
 * 38-43,61-66 and raft/raft_backprojection_bresenham.cpp).  The image ships no
 * system BLAS, so the reference build in oracle/Makefile links this file
 * instead.  Plain strided loops with the Fortran calling convention (every
 * argument by pointer); a zero increment on x broadcasts x[0], which is how
 * the reference zero-fills its buffers.
 *
 * TEST INFRASTRUCTURE: linked only into oracle/_ref/libraft_ref.so, which the
 * tests and the golden-fixture script load as a checker.
 */

void dcopy_(const int *n, const double *x, const int *incx, double *y,
            const int *incy)
{
    int count = *n, sx = *incx, sy = *incy;
    int ix = (sx < 0) ? (1 - count) * sx : 0;
    int iy = (sy < 0) ? (1 - count) * sy : 0;
    for (int e = 0; e < count; ++e, ix += sx, iy += sy)
        y[iy] = x[ix];
}

void daxpy_(const int *n, const double *alpha, const double *x,
            const int *incx, double *y, const int *incy)
{
    int count = *n, sx = *incx, sy = *incy;
    double a = *alpha;
    int ix = (sx < 0) ? (1 - count) * sx : 0;
    int iy = (sy < 0) ? (1 - count) * sy : 0;
    for (int e = 0; e < count; ++e, ix += sx, iy += sy)
        y[iy] += a * x[ix];
}
