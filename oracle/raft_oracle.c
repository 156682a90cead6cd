/*
 * oracle/raft_oracle.c -- FP64 CPU restatement of pyraft's reconstruction hot
 * path.  TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load this library, as the checker of the CUDA
 * path or as the timed CPU baseline.  The product (pyraft_gb300/) never calls
 * it.
 *
 * Each routine restates one reference routine (file:line cited beside it) in
 * the same floating-point operation order, so that with -ffp-contract=off it
 * reproduces the compiled reference bit for bit (pinned by
 * tests/test_oracle_golden.py against fixtures made from the reference).
 *
 * Data layout: every image or sinogram is a C-contiguous row-major double
 * array with `lines` rows and `columns` columns; element (i, j) is
 * p[i * columns + j].  Corners follow raft_image (raft/raft_image.h:11-19):
 * tl = top-left (x, y), br = bottom-right (x, y).
 *
 * Departures, each deliberate and documented:
 *  - The DDA's axis-aligned branches (sin == 0 or cos == 0) never set sigma in
 *    the reference (raft/raft_ddaiterator.c:118-129); the first pixel of such
 *    a ray then reads a stale or uninitialised value.  Here it is set to the
 *    typical intersection length sigma_tilde, which is what every later step
 *    of the same ray uses.
 *  - Thread splitting: the reference's slant-stack workers compute nothing
 *    when there are fewer outputs than threads (raft/raft_radon_slantstack.c:
 *    62, e = floor(N / nthreads) == 0).  Work here is split so every output is
 *    computed.
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    double *p;
    int lines, columns;
    double tl_x, tl_y, br_x, br_y;
} orc_img;

#define AT(im, i, j) ((im)->p[(size_t)(i) * (size_t)(im)->columns + (size_t)(j)])

/* ------------------------------------------------------------------------ */
/* A tiny static-partition parallel-for over [0, n).                        */

typedef void (*orc_body)(void *ctx, int lo, int hi, int worker);

typedef struct {
    orc_body fn;
    void *ctx;
    int lo, hi, worker;
} orc_task;

static void *orc_run(void *arg)
{
    orc_task *t = (orc_task *)arg;
    t->fn(t->ctx, t->lo, t->hi, t->worker);
    return NULL;
}

static int orc_workers(int n, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if (nthreads > n) nthreads = n;
    return nthreads < 1 ? 1 : nthreads;
}

static void orc_parallel(int n, int nthreads, orc_body fn, void *ctx)
{
    int w = orc_workers(n, nthreads);
    if (n <= 0) return;
    if (w == 1) { fn(ctx, 0, n, 0); return; }
    pthread_t th[256];
    orc_task task[256];
    int base = n / w, extra = n % w, start = 0;
    for (int k = 0; k < w; ++k) {
        int cnt = base + (k < extra);
        task[k].fn = fn; task[k].ctx = ctx;
        task[k].lo = start; task[k].hi = start + cnt; task[k].worker = k;
        start += cnt;
        pthread_create(&th[k], NULL, orc_run, &task[k]);
    }
    for (int k = 0; k < w; ++k) pthread_join(th[k], NULL);
}

/* ------------------------------------------------------------------------ */
/* Slant-stack Radon, a ray-driven line integral with linear interpolation.
 * Restates eval_rayintegral (raft/raft_radon_slantstack.c:122-214): angles
 * endpoint-exclusive th0 + j*(thf-th0)/nviews (:154-158), rays
 * tmin + k*(tmax-tmin)/(nrays-1) (:168-172), image row m at y = ymin + m*dy
 * (bottom-up).  Branch on |cos| < 1/sqrt(2) (:174).                          */

typedef struct {
    const orc_img *img;
    orc_img *sino;
    orc_img *adj;        /* non-NULL: scatter the transpose instead          */
    const orc_img *in;   /* sinogram read by the transpose                   */
    double *partials;    /* per-worker images for the transpose              */
} ss_ctx;

/* Geometry of one (view j, ray k); `mode` 0 = forward sum, 1 = transpose
 * scatter of weight `sv` into `out` (an image laid out like `img`).        */
static double ss_ray(const orc_img *img, int nviews, int nrays,
                     double s_tl_x, double s_tl_y, double s_br_x, double s_br_y,
                     int j, int k, int mode, double sv, double *out)
{
    const int size = img->lines;
    const double tol = 1.0 / sqrt(2);
    double xmin = img->tl_x, xmax = img->br_x;
    double ymin = img->br_y, ymax = img->tl_y;
    double dx = (xmax - xmin) / (size - 1);
    double dy = (ymax - ymin) / (size - 1);
    double th0 = s_tl_x, thf = s_br_x;
    double dth = (thf - th0) / (nviews);
    double theta = th0 + j * dth;
    double cost = cos(theta), sint = sin(theta), tant = tan(theta);
    double tmin = s_br_y, tmax = s_tl_y;
    double dt = (tmax - tmin) / (nrays - 1);
    double t = tmin + k * dt;
    double sum = 0.0;
    const int cols = img->columns;

    if (fabs(cost) < tol) {
        double Delta = dy / fabs(sint);
        for (int i = 0; i < size; ++i) {
            double x = (double)(xmin + i * dx);
            double y = (double)(t / sint - x / tant);
            int m = (int)floor((y - ymin) / dy);
            if (m > -1 && m < size - 1) {
                if (mode == 0) {
                    double f0 = AT(img, m, i), f1 = AT(img, m + 1, i);
                    sum += (f1 - f0) * (y - (ymin + m * dy)) / dy + f0;
                } else {
                    double w = (y - (ymin + m * dy)) / dy;
                    out[(size_t)m * cols + i] += sv * Delta * (1.0 - w);
                    out[(size_t)(m + 1) * cols + i] += sv * Delta * w;
                }
            }
        }
        return sum * Delta;
    } else {
        double Delta = dx / fabs(cost);
        for (int i = 0; i < size; ++i) {
            double y = (double)(xmin + i * dy);   /* xmin: as the reference */
            double x = (double)(t / cost - y * tant);
            int m = (int)floor((x - xmin) / dx);
            if (m > -1 && m < size - 1) {
                if (mode == 0) {
                    double f0 = AT(img, i, m), f1 = AT(img, i, m + 1);
                    sum += (f1 - f0) * (x - (xmin + m * dx)) / dx + f0;
                } else {
                    double w = (x - (xmin + m * dx)) / dx;
                    out[(size_t)i * cols + m] += sv * Delta * (1.0 - w);
                    out[(size_t)i * cols + m + 1] += sv * Delta * w;
                }
            }
        }
        return sum * Delta;
    }
}

static void ss_radon_body(void *vctx, int lo, int hi, int worker)
{
    ss_ctx *c = (ss_ctx *)vctx;
    orc_img *s = c->sino;
    (void)worker;
    for (int w = lo; w < hi; ++w) {
        int j = w / s->lines, k = w % s->lines;
        AT(s, k, j) = ss_ray(c->img, s->columns, s->lines, s->tl_x, s->tl_y,
                             s->br_x, s->br_y, j, k, 0, 0.0, NULL);
    }
}

void orc_radon_slantstack(const orc_img *img, orc_img *sino, int nthreads)
{
    ss_ctx c = {img, sino, NULL, NULL, NULL};
    orc_parallel(sino->lines * sino->columns, nthreads, ss_radon_body, &c);
}

/* Matched adjoint: the exact transpose of orc_radon_slantstack (no
 * counterpart in the reference).  Each worker scatters a contiguous range of
 * views into a private image; the private images are then summed in worker
 * order, so the result does not depend on scheduling.                      */
static void ss_adj_body(void *vctx, int lo, int hi, int worker)
{
    ss_ctx *c = (ss_ctx *)vctx;
    const orc_img *s = c->in;
    const orc_img *img = c->adj;
    size_t npix = (size_t)img->lines * img->columns;
    double *out = c->partials + (size_t)worker * npix;
    memset(out, 0, npix * sizeof(double));
    for (int j = lo; j < hi; ++j)
        for (int k = 0; k < s->lines; ++k) {
            double sv = AT(s, k, j);
            if (sv != 0.0)
                ss_ray(img, s->columns, s->lines, s->tl_x, s->tl_y, s->br_x,
                       s->br_y, j, k, 1, sv, out);
        }
}

int orc_radon_slantstack_transpose(const orc_img *sino, orc_img *img, int nthreads)
{
    int w = orc_workers(sino->columns, nthreads);
    size_t npix = (size_t)img->lines * img->columns;
    double *part = (double *)malloc((size_t)w * npix * sizeof(double));
    if (!part) return -1;
    ss_ctx c = {img, NULL, img, sino, part};
    orc_parallel(sino->columns, w, ss_adj_body, &c);
    for (size_t e = 0; e < npix; ++e) {
        double acc = 0.0;
        for (int k = 0; k < w; ++k) acc += part[(size_t)k * npix + e];
        img->p[e] = acc;
    }
    free(part);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Slant-stack backprojection, pixel-driven angle sum.  Restates
 * eval_anglesum_slantstack (raft/raft_backprojection_slantstack.c:121-180):
 * pixel (j, k) at x = xmin + k*dx, y = ymin + j*dy; t = x cos + y sin;
 * linear interpolation in t, valid iff 0 <= n <= nrays-2; result * dth.     */

typedef struct { const orc_img *sino; orc_img *img; } bp_ctx;

static void ss_bp_body(void *vctx, int lo, int hi, int worker)
{
    bp_ctx *c = (bp_ctx *)vctx;
    const orc_img *s = c->sino;
    orc_img *b = c->img;
    int size = b->lines;
    int nrays = s->lines, nviews = s->columns;
    double tmin = s->br_y, tmax = s->tl_y;
    double dt = (tmax - tmin) / (nrays - 1);
    double th0 = s->tl_x, thf = s->br_x;
    double dth = (thf - th0) / (nviews);
    double xmin = b->tl_x, xmax = b->br_x;
    double dx = (xmax - xmin) / (size - 1);
    double ymin = b->br_y, ymax = b->tl_y;
    double dy = (ymax - ymin) / (size - 1);
    (void)worker;
    for (int w = lo; w < hi; ++w) {
        int j = w / size, k = w % size;
        double x = xmin + k * dx;
        double y = ymin + j * dy;
        double sum = 0.0;
        for (int i = 0; i < nviews; ++i) {
            double th = th0 + i * dth;
            double cost = cos(th), sint = sin(th);
            double t = x * cost + y * sint;
            int n = (int)floor((t - tmin) / dt);
            if (n > -1 && n < nrays - 1) {
                double f0 = AT(s, n, i), f1 = AT(s, n + 1, i);
                sum += (f1 - f0) * (t - (tmin + n * dt)) / dt + f0;
            }
        }
        AT(b, j, k) = sum * dth;
    }
}

void orc_backprojection_slantstack(const orc_img *sino, orc_img *img, int nthreads)
{
    bp_ctx c = {sino, img};
    orc_parallel(img->lines * img->lines, nthreads, ss_bp_body, &c);
}

/* Rows [row0, row1) only (a bounded sample for CPU timing). */
typedef struct { bp_ctx c; int off; } bp_rows_ctx;

static void ss_bp_rows_body(void *vctx, int lo, int hi, int worker)
{
    bp_rows_ctx *r = (bp_rows_ctx *)vctx;
    ss_bp_body(&r->c, lo + r->off, hi + r->off, worker);
}

void orc_backprojection_slantstack_rows(const orc_img *sino, orc_img *img, int row0, int row1,
                                        int nthreads)
{
    bp_rows_ctx r = {{sino, img}, row0 * img->lines};
    orc_parallel((row1 - row0) * img->lines, nthreads, ss_bp_rows_body, &r);
}

/* Rows row0, row0 + step, ... (count rows): a sample spread over the whole
 * image, for CPU timing and for parity checks of full-size GPU results. */
typedef struct { bp_ctx c; int row0, step; } bp_rowstep_ctx;

static void ss_bp_rowstep_body(void *vctx, int lo, int hi, int worker)
{
    bp_rowstep_ctx *r = (bp_rowstep_ctx *)vctx;
    int size = r->c.img->lines;
    for (int w = lo; w < hi; ++w) {
        int idx = (r->row0 + (w / size) * r->step) * size + w % size;
        ss_bp_body(&r->c, idx, idx + 1, worker);
    }
}

void orc_backprojection_slantstack_rowstep(const orc_img *sino, orc_img *img, int row0,
                                           int step, int count, int nthreads)
{
    bp_rowstep_ctx r = {{sino, img}, row0, step};
    orc_parallel(count * img->lines, nthreads, ss_bp_rowstep_body, &r);
}

/* ------------------------------------------------------------------------ */
/* DDA (Bresenham-like) pixel walk.  Restates raft_ddaiterator
 * (raft/raft_ddaiterator.c:16-257, struct raft/raft_ddaiterator.h:10-47):
 * same FP64 decisions in the same order, so the pixel index sequences agree
 * bit for bit.  The fast/slow index pointers become a flag.                 */

typedef struct {
    int i, j;
    double sigma;
    int slow_move;
    int fast_is_i;               /* 1: fast index is i (vertical fast)       */
    double epsilon, epsilon_update;
    double delta_x, delta_y, delta_slow;
    int Delta_i, Delta_j, Delta_slow, Delta_fast;
    double sigma_tilde;
    int lines, columns;
    double bbox_tl_x, bbox_tl_y, bbox_br_x, bbox_br_y;
    double tl_x, tl_y, br_x, br_y;
    double x0, y0;
    int i_init, j_init;
    double sin_theta, cos_theta;
} orc_dda;

static double sgn(double v) { return v > 0.0 ? 1.0 : (v < 0.0 ? -1.0 : 0.0); }

static double dda_index(double x, double x_i, double delta, int D)
{
    return (D >= 0) ? floor(((x - x_i) / delta) - 0.5) + 1
                    : ceil(((x - x_i) / delta) - 0.5);
}

void orc_dda_set_image(orc_dda *it, int lines, int columns,
                       double tl_x, double tl_y, double br_x, double br_y)
{
    it->delta_x = (br_x - tl_x) / (columns - 1);
    it->delta_y = (br_y - tl_y) / (lines - 1);
    it->bbox_tl_x = tl_x - (it->delta_x / 2.0);
    it->bbox_br_x = br_x + (it->delta_x / 2.0);
    it->bbox_tl_y = tl_y - (it->delta_y / 2.0);
    it->bbox_br_y = br_y + (it->delta_y / 2.0);
    it->tl_x = tl_x; it->br_x = br_x; it->tl_y = tl_y; it->br_y = br_y;
    it->lines = lines; it->columns = columns;
}

static void dda_slowfast(orc_dda *it, int fast_is_i, double d_fast,
                         double d_slow, double small_trig, double large_trig,
                         int D_fast, int D_slow)
{
    it->fast_is_i = fast_is_i;
    it->epsilon_update = fabs(d_fast * small_trig / large_trig);
    it->delta_slow = fabs(d_slow);
    it->Delta_slow = D_slow;
    it->Delta_fast = D_fast;
    it->sigma_tilde = fabs(d_fast / large_trig);
}

static double dmax(double a, double b) { return (a > b) ? a : b; }
static double dmin(double a, double b) { return (a < b) ? a : b; }

void orc_dda_update(orc_dda *it);

/* cos/sin are passed in so that callers can share one trig table; the
 * reference evaluates cos(theta), sin(theta) (raft/raft_ddaiterator.c:68). */
void orc_dda_set_theta_cs(orc_dda *it, double c, double s)
{
    it->cos_theta = c; it->sin_theta = s;
    int sign;
    sign = (int)sgn(it->sin_theta);
    it->x0 = sign * dmax(sign * it->bbox_br_x, sign * it->bbox_tl_x);
    it->Delta_j = (int)(-sgn(it->delta_x) * sign);
    sign = (int)sgn(it->cos_theta);
    it->y0 = sign * dmin(sign * it->bbox_br_y, sign * it->bbox_tl_y);
    it->Delta_i = (int)(sgn(it->delta_y) * sign);
    it->i_init = (it->Delta_i < 0) ? (it->lines - 1) : 0;
    it->j_init = (it->Delta_j < 0) ? (it->columns - 1) : 0;
    if (fabs(it->delta_x * it->sin_theta) <= fabs(it->delta_y * it->cos_theta))
        dda_slowfast(it, 1, it->delta_y, it->delta_x, it->sin_theta,
                     it->cos_theta, it->Delta_i, it->Delta_j);
    else
        dda_slowfast(it, 0, it->delta_x, it->delta_y, it->cos_theta,
                     it->sin_theta, it->Delta_j, it->Delta_i);
}

void orc_dda_set_theta(orc_dda *it, double theta)
{
    orc_dda_set_theta_cs(it, cos(theta), sin(theta));
}

/* raft/raft_ddaiterator.c:108-194 */
void orc_dda_set_t(orc_dda *it, double t)
{
    double sx, sy, xy;
    it->slow_move = 0;
    if (it->sin_theta == 0.0) {
        it->j = (int)dda_index(t, it->tl_x, it->delta_x, it->Delta_j);
        it->i = it->i_init;
        it->epsilon = 0.0;
        it->epsilon_update = 0.0;
        it->sigma = it->sigma_tilde;          /* unset in the reference */
    } else if (it->cos_theta == 0.0) {
        it->i = (int)dda_index(t, it->tl_y, it->delta_y, it->Delta_i);
        it->j = it->j_init;
        it->epsilon = 0.0;
        it->epsilon_update = 0.0;
        it->sigma = it->sigma_tilde;          /* unset in the reference */
    } else if ((sx = ((t * it->cos_theta - it->x0) / it->sin_theta)) >
               (sy = ((it->y0 - t * it->sin_theta) / it->cos_theta))) {
        xy = (sx * it->cos_theta) + (t * it->sin_theta);
        it->i = (int)dda_index(xy, it->tl_y, it->delta_y, it->Delta_i);
        it->j = it->j_init;
        it->epsilon = fabs(xy - (it->tl_y + (it->i - (0.5 * it->Delta_i)) * it->delta_y));
        if (!it->fast_is_i) {           /* slow index is i */
            it->j -= it->Delta_j;
            orc_dda_update(it);
        } else {
            it->epsilon -= fabs(it->delta_y);
            it->sigma = fabs(it->epsilon /= it->cos_theta);
            it->epsilon = fabs(it->sigma * it->sin_theta);
        }
    } else {
        xy = (-sy * it->sin_theta) + (t * it->cos_theta);
        it->j = (int)dda_index(xy, it->tl_x, it->delta_x, it->Delta_j);
        it->i = it->i_init;
        it->epsilon = fabs(xy - (it->tl_x + (it->j - (0.5 * it->Delta_j)) * it->delta_x));
        if (it->fast_is_i) {            /* slow index is j */
            it->i -= it->Delta_i;
            orc_dda_update(it);
        } else {
            it->epsilon -= fabs(it->delta_x);
            it->sigma = fabs(it->epsilon /= it->sin_theta);
            it->epsilon = fabs(it->sigma * it->cos_theta);
        }
    }
}

/* raft/raft_ddaiterator.c:196-248 */
void orc_dda_update(orc_dda *it)
{
    double eps_prev, alpha;
    if (it->slow_move) {
        if (it->fast_is_i) it->j += it->Delta_slow; else it->i += it->Delta_slow;
        it->sigma = it->sigma_tilde - it->sigma;
        it->slow_move = 0;
    } else {
        if (it->fast_is_i) it->i += it->Delta_fast; else it->j += it->Delta_fast;
        eps_prev = it->epsilon;
        it->epsilon += it->epsilon_update;
        it->slow_move = (it->epsilon > it->delta_slow);
        if (it->slow_move) {
            it->epsilon -= it->delta_slow;
            if (it->epsilon) {
                alpha = (it->delta_slow - eps_prev) / it->epsilon;
                alpha /= (1.0 + alpha);
            } else {
                alpha = 1.0;
            }
            it->sigma = alpha * it->sigma_tilde;
        } else {
            it->sigma = it->sigma_tilde;
        }
    }
}

int orc_dda_end(const orc_dda *it)
{
    return (it->i < 0) || (it->i >= it->lines) || (it->j < 0) || (it->j >= it->columns);
}

/* Walk one ray and record its pixels: writes at most `cap` (i, j, sigma)
 * triples and returns the full step count.                                 */
int orc_dda_trace(int lines, int columns, double tl_x, double tl_y, double br_x,
                  double br_y, double theta, double t, int *ii, int *jj,
                  double *sig, int cap)
{
    orc_dda it;
    int n = 0;
    orc_dda_set_image(&it, lines, columns, tl_x, tl_y, br_x, br_y);
    orc_dda_set_theta(&it, theta);
    orc_dda_set_t(&it, t);
    while (!orc_dda_end(&it)) {
        if (n < cap) { ii[n] = it.i; jj[n] = it.j; sig[n] = it.sigma; }
        ++n;
        orc_dda_update(&it);
    }
    return n;
}

/* ------------------------------------------------------------------------ */
/* Bresenham/DDA Radon and its exact transpose.  Restate
 * raft_radon_bresenham_worker (raft/raft_radon_bresenham.cpp:16-61) and
 * raft_radon_transpose_bresenham_worker (raft/raft_radon_transpose_bresenham
 * .cpp:48-95): views tl_x + j*(br_x-tl_x)/(columns-1) (endpoint-inclusive),
 * rays tl_y + i*(br_y-tl_y)/(lines-1).  The transpose sums per-worker images
 * in worker order, like the reference's summer (:17-46).                    */

typedef struct { const orc_img *img; orc_img *sino; const orc_img *in;
                 orc_img *out; double *partials; } br_ctx;

static void bres_radon_body(void *vctx, int lo, int hi, int worker)
{
    br_ctx *c = (br_ctx *)vctx;
    const orc_img *im = c->img;
    orc_img *s = c->sino;
    orc_dda it;
    double dth = (s->br_x - s->tl_x) / (s->columns - 1);
    double dts = (s->br_y - s->tl_y) / (s->lines - 1);
    (void)worker;
    orc_dda_set_image(&it, im->lines, im->columns, im->tl_x, im->tl_y, im->br_x, im->br_y);
    for (int j = lo; j < hi; ++j) {
        orc_dda_set_theta(&it, s->tl_x + (j * dth));
        for (int i = 0; i < s->lines; ++i) {
            double acc = 0.0;
            orc_dda_set_t(&it, s->tl_y + (i * dts));
            while (!orc_dda_end(&it)) {
                acc += AT(im, it.i, it.j) * it.sigma;
                orc_dda_update(&it);
            }
            AT(s, i, j) = acc;
        }
    }
}

void orc_radon_bresenham(const orc_img *img, orc_img *sino, int nthreads)
{
    br_ctx c = {img, sino, NULL, NULL, NULL};
    orc_parallel(sino->columns, nthreads, bres_radon_body, &c);
}

static void bres_T_body(void *vctx, int lo, int hi, int worker)
{
    br_ctx *c = (br_ctx *)vctx;
    const orc_img *s = c->in;
    orc_img *img = c->out;
    size_t npix = (size_t)img->lines * img->columns;
    double *out = c->partials + (size_t)worker * npix;
    orc_dda it;
    double dth = (s->br_x - s->tl_x) / (s->columns - 1);
    double dts = (s->br_y - s->tl_y) / (s->lines - 1);
    memset(out, 0, npix * sizeof(double));
    orc_dda_set_image(&it, img->lines, img->columns, img->tl_x, img->tl_y, img->br_x, img->br_y);
    for (int j = lo; j < hi; ++j) {
        orc_dda_set_theta(&it, s->tl_x + (j * dth));
        for (int i = 0; i < s->lines; ++i) {
            double sv = AT(s, i, j);
            orc_dda_set_t(&it, s->tl_y + (i * dts));
            while (!orc_dda_end(&it)) {
                out[(size_t)it.i * img->columns + it.j] += sv * it.sigma;
                orc_dda_update(&it);
            }
        }
    }
}

int orc_radon_transpose_bresenham(const orc_img *sino, orc_img *img, int nthreads)
{
    int w = orc_workers(sino->columns, nthreads);
    size_t npix = (size_t)img->lines * img->columns;
    double *part = (double *)malloc((size_t)w * npix * sizeof(double));
    if (!part) return -1;
    br_ctx c = {NULL, NULL, sino, img, part};
    orc_parallel(sino->columns, w, bres_T_body, &c);
    for (size_t e = 0; e < npix; ++e) {
        double acc = 0.0;
        for (int k = 0; k < w; ++k) acc += part[(size_t)k * npix + e];
        img->p[e] = acc;
    }
    free(part);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Ellipse phantoms.  desc is an (n x 6) row-major table of
 * [alpha, a, b, x0, y0, theta] per ellipse.                                 */

/* raft/raft_image_phantom_fromdesc.c:4-59 (adds into img) */
void orc_phantom_fromdesc(orc_img *img, const double *desc, int n)
{
    double xs = (img->br_x - img->tl_x) / (img->columns - 1);
    double ys = (img->br_y - img->tl_y) / (img->lines - 1);
    for (int e = 0; e < n; ++e) {
        const double *d = desc + 6 * e;
        double alpha = d[0], a = d[1], b = d[2], x0 = d[3], y0 = d[4], th = d[5];
        double c = cos(th), s = sin(th);
        for (int i = 0; i < img->lines; ++i)
            for (int j = 0; j < img->columns; ++j) {
                double x = img->tl_x + j * xs - x0;
                double y = img->tl_y + i * ys - y0;
                double val = (y * s) + (x * c);
                val /= a;
                val *= val;
                double tmp = (y * c) - (x * s);
                tmp /= b;
                tmp *= tmp;
                val += tmp;
                val = sqrt(val);
                if (val <= 1) AT(img, i, j) += alpha;
            }
    }
}

/* raft/raft_radon_fromdesc.c:4-67 (adds into sino); views endpoint-inclusive */
void orc_radon_fromdesc(orc_img *sino, const double *desc, int n)
{
    double ths = (sino->br_x - sino->tl_x) / (sino->columns - 1);
    double tss = (sino->br_y - sino->tl_y) / (sino->lines - 1);
    for (int e = 0; e < n; ++e) {
        const double *d = desc + 6 * e;
        double ea = d[0], ax = d[1], bx = d[2], eth = d[5], ex = d[3], ey = d[4];
        for (int j = 0; j < sino->columns; ++j) {
            double th = sino->tl_x + j * ths;
            double c = cos(th), s = sin(th);
            th -= eth;
            double cp = cos(th), sp = sin(th);
            double m = 1.0 / sqrt(((cp * cp) / (bx * bx)) + ((sp * sp) / (ax * ax)));
            double mab = m / (ax * bx);
            m *= 2.0; m *= ea;
            double delt = mab * ((ex * c) + (ey * s) - sino->tl_y);
            mab *= tss;
            for (int i = 0; i < sino->lines; ++i) {
                double tp = mab * i - delt;
                tp *= tp;
                if (tp <= 1.0) AT(sino, i, j) += m * sqrt(1.0 - tp);
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Ram-Lak ramp filter as a linear spatial convolution along t (no
 * counterpart in the reference, whose filters are FFT based:
 * raft/raft_filter.cpp:184-213, pyraft/filters/filters.py:13-68).
 * Discrete Ram-Lak kernel (Kak & Slaney, ch. 3): h[0] = 1/(4 dt^2),
 * h[odd m] = -1/(pi^2 m^2 dt^2), h[even m != 0] = 0, and
 * q[n] = dt * sum_k h[n-k] p[k].  Operates on each column of an
 * (nrays x nviews) sinogram; out may not alias in.                         */

typedef struct { const double *in; double *out; int R, V; double dt;
                 const double *taps; int circular; } rl_ctx;

static void conv_body(void *vctx, int lo, int hi, int worker)
{
    rl_ctx *c = (rl_ctx *)vctx;
    int R = c->R, V = c->V;
    (void)worker;
    for (int v = lo; v < hi; ++v)
        for (int n = 0; n < R; ++n) {
            double acc = 0.0;
            for (int k = 0; k < R; ++k) {
                int m = n - k;
                double h = c->circular ? c->taps[(m % R + R) % R] : c->taps[m + R - 1];
                acc += h * c->in[(size_t)k * V + v];
            }
            c->out[(size_t)n * V + v] = acc;
        }
}

void orc_ramlak_taps(double *taps, int R, double dt)
{
    const double pi = 3.14159265358979323846;
    for (int m = -(R - 1); m <= R - 1; ++m) {
        double h;
        if (m == 0) h = 1.0 / (4.0 * dt * dt);
        else if (m % 2 == 0) h = 0.0;
        else h = -1.0 / (pi * pi * (double)m * (double)m * dt * dt);
        taps[m + R - 1] = h * dt;
    }
}

/* Ram-Lak on the first `nv` views only (a bounded sample for CPU timing). */
int orc_ramlak_views(const double *in, double *out, int R, int V, int nv, double dt,
                     int nthreads)
{
    double *taps = (double *)malloc((size_t)(2 * R - 1) * sizeof(double));
    if (!taps) return -1;
    orc_ramlak_taps(taps, R, dt);
    rl_ctx c = {in, out, R, V, dt, taps, 0};
    orc_parallel(nv, nthreads, conv_body, &c);
    free(taps);
    return 0;
}

int orc_ramlak(const double *in, double *out, int R, int V, double dt, int nthreads)
{
    double *taps = (double *)malloc((size_t)(2 * R - 1) * sizeof(double));
    if (!taps) return -1;
    orc_ramlak_taps(taps, R, dt);
    rl_ctx c = {in, out, R, V, dt, taps, 0};
    orc_parallel(V, nthreads, conv_body, &c);
    free(taps);
    return 0;
}

/* Circular convolution along t with an R-tap kernel g (g[m] multiplies
 * p[n-m mod R]); the spatial form of an FFT filter.                        */
void orc_circular_filter(const double *in, double *out, int R, int V,
                         const double *g, int nthreads)
{
    rl_ctx c = {in, out, R, V, 0.0, g, 1};
    orc_parallel(V, nthreads, conv_body, &c);
}

/* ------------------------------------------------------------------------ */
/* Normalised DDA backprojection, restating raft_backprojection_bresenham
 * (raft/raft_backprojection_bresenham.cpp:17-251): per pixel
 * sum(s * sigma) / sum(sigma) over every ray step that visits it.  Pixels no
 * ray visits give 0 here (the reference divides 0 by 0).                    */
typedef struct { const orc_img *in; orc_img *out; double *num, *den; } bn_ctx;

static void bres_norm_body(void *vctx, int lo, int hi, int worker)
{
    bn_ctx *c = (bn_ctx *)vctx;
    const orc_img *s = c->in;
    orc_img *img = c->out;
    size_t npix = (size_t)img->lines * img->columns;
    double *num = c->num + (size_t)worker * npix, *den = c->den + (size_t)worker * npix;
    orc_dda it;
    double dth = (s->br_x - s->tl_x) / (s->columns - 1);
    double dts = (s->br_y - s->tl_y) / (s->lines - 1);
    memset(num, 0, npix * sizeof(double));
    memset(den, 0, npix * sizeof(double));
    orc_dda_set_image(&it, img->lines, img->columns, img->tl_x, img->tl_y, img->br_x, img->br_y);
    for (int j = lo; j < hi; ++j) {
        orc_dda_set_theta(&it, s->tl_x + (j * dth));
        for (int i = 0; i < s->lines; ++i) {
            double sv = AT(s, i, j);
            orc_dda_set_t(&it, s->tl_y + (i * dts));
            while (!orc_dda_end(&it)) {
                size_t e = (size_t)it.i * img->columns + it.j;
                num[e] += sv * it.sigma;
                den[e] += it.sigma;
                orc_dda_update(&it);
            }
        }
    }
}

int orc_backprojection_bresenham(const orc_img *sino, orc_img *img, int nthreads)
{
    int w = orc_workers(sino->columns, nthreads);
    size_t npix = (size_t)img->lines * img->columns;
    double *num = (double *)malloc((size_t)w * npix * sizeof(double));
    double *den = (double *)malloc((size_t)w * npix * sizeof(double));
    if (!num || !den) { free(num); free(den); return -1; }
    bn_ctx c = {sino, img, num, den};
    orc_parallel(sino->columns, w, bres_norm_body, &c);
    for (size_t e = 0; e < npix; ++e) {
        double a = 0.0, b = 0.0;
        for (int k = 0; k < w; ++k) { a += num[(size_t)k * npix + e]; b += den[(size_t)k * npix + e]; }
        img->p[e] = (b != 0.0) ? a / b : 0.0;
    }
    free(num);
    free(den);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Slant-stack Radon on an explicit (t, theta) mesh, restating
 * eval_rayintegral_mesh (raft/raft_radon_slantstack_withmesh.c:122-211):
 * the ray integral of orc_radon_slantstack with theta_j = theta[j] and
 * t_k = t[k] instead of the uniform grids.  Every output is computed (the
 * reference's thread split drops the remainder, :65-67).                   */
typedef struct { const orc_img *img; orc_img *sino; const double *t, *th; } mesh_ctx;

static double mesh_ray(const orc_img *img, double tt, double th)
{
    const int size = img->lines;
    const double tol = 1.0 / sqrt(2);
    double xmin = img->tl_x, xmax = img->br_x, ymin = img->br_y, ymax = img->tl_y;
    double dx = (xmax - xmin) / (size - 1), dy = (ymax - ymin) / (size - 1);
    double cost = cos(th), sint = sin(th), tant = tan(th);
    double sum = 0.0;
    if (fabs(cost) < tol) {
        double Delta = (dy / fabs(sint));
        for (int i = 0; i < size; ++i) {
            double x = (double)(xmin + i * dx);
            double y = (double)(tt / sint - x / tant);
            int m = (int)floor((y - ymin) / dy);
            if (m > -1 && m < size - 1)
                sum += (AT(img, m + 1, i) - AT(img, m, i)) * (y - (ymin + m * dy)) / dy + AT(img, m, i);
        }
        return sum * Delta;
    }
    double Delta = (dx / fabs(cost));
    for (int i = 0; i < size; ++i) {
        double y = (double)(xmin + i * dy);
        double x = (double)(tt / cost - y * tant);
        int m = (int)floor((x - xmin) / dx);
        if (m > -1 && m < size - 1)
            sum += (AT(img, i, m + 1) - AT(img, i, m)) * (x - (xmin + m * dx)) / dx + AT(img, i, m);
    }
    return sum * Delta;
}

static void mesh_body(void *vctx, int lo, int hi, int worker)
{
    mesh_ctx *c = (mesh_ctx *)vctx;
    orc_img *s = c->sino;
    (void)worker;
    for (int w = lo; w < hi; ++w) {
        int j = w / s->lines, k = w % s->lines;
        AT(s, k, j) = mesh_ray(c->img, c->t[k], c->th[j]);
    }
}

void orc_radon_slantstack_withmesh(const orc_img *img, orc_img *sino, const double *t,
                                   const double *theta, int nthreads)
{
    mesh_ctx c = {img, sino, t, theta};
    orc_parallel(sino->lines * sino->columns, nthreads, mesh_body, &c);
}
