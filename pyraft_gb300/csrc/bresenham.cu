// bresenham.cu -- DDA (Bresenham-like) ray traversal, its Radon transform and
// the exact transpose.
//
// The traversal restates raft_ddaiterator (raft/raft_ddaiterator.c:16-257):
// entry pixel from the ray's first crossing of the pixel-centre bounding box,
// then fast-axis steps with an epsilon accumulator deciding slow-axis steps
// and splitting the intersection length sigma.  Its pixel decisions are made
// in FP64 with every operation written as an explicit round-to-nearest
// intrinsic (__dadd_rn, __dmul_rn, __ddiv_rn), which the compiler never
// contracts into FMA; with the view cos/sin taken from the host libm (as the
// reference does) the visited pixel sequence is bit-identical to the
// reference's.  The axis-aligned branches set sigma to sigma_tilde on entry
// (the reference leaves it unset, raft/raft_ddaiterator.c:118-129).  The
// Radon, transpose, walk recording and normalised backprojection continue
// each walk after its first epsilon add in exact 64-bit integer arithmetic
// that reproduces those FP64 operations (DDAInt, dda_walk): the same pixels
// and the same FP32 or FP64 sigma, without most of the FP64 work.
//
// Radon: one thread per (ray, view); lanes run over rays, so the
// view-major output is written coalesced.  Sums are FP32 products of the
// FP32 image and an FP32 sigma (dda_update: the reference's sigma to within
// FP32 rounding, without its FP64 divisions), accumulated in FP32 with
// Kahan compensation.  Transpose: same walk, FP32 atomicAdd scatter into
// the image (order of additions varies between runs, at FP32 rounding level).
//
// Every walk is capped at 2 * (lines + columns) + 8 steps; the walk is
// monotone in both indices, so the cap is never reached by a valid ray.
#include <math.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "rg_internal.cuh"

namespace rg {

struct DDA {
    int i, j;
    double sigma;
    int slow_move, fast_is_i;
    double epsilon, epsilon_update, delta_x, delta_y, delta_slow;
    int Delta_i, Delta_j, Delta_slow, Delta_fast;
    double sigma_tilde;
    double sigma_per_eps;        // sigma_tilde / epsilon_update (0 when the update is 0)
    float sigma32, sigma_tilde32, sigma_per_eps32;   // FP32 sigma (kDdaSigma32)
    int lines, columns;
    double bbox_tl_x, bbox_tl_y, bbox_br_x, bbox_br_y;
    double tl_x, tl_y;
    double x0, y0;
    int i_init, j_init;
    double sin_theta, cos_theta;
};

__device__ __forceinline__ double sgnd(double v) { return v > 0.0 ? 1.0 : (v < 0.0 ? -1.0 : 0.0); }

__device__ __forceinline__ double dda_index(double x, double xi, double delta, int D)
{
    const double q = __dsub_rn(__ddiv_rn(__dsub_rn(x, xi), delta), 0.5);
    return (D >= 0) ? __dadd_rn(floor(q), 1.0) : ceil(q);
}

__device__ __forceinline__ void dda_set_image(DDA &it, int lines, int columns, double tl_x,
                                              double tl_y, double br_x, double br_y)
{
    it.delta_x = __ddiv_rn(__dsub_rn(br_x, tl_x), (double)(columns - 1));
    it.delta_y = __ddiv_rn(__dsub_rn(br_y, tl_y), (double)(lines - 1));
    it.bbox_tl_x = __dsub_rn(tl_x, __ddiv_rn(it.delta_x, 2.0));
    it.bbox_br_x = __dadd_rn(br_x, __ddiv_rn(it.delta_x, 2.0));
    it.bbox_tl_y = __dsub_rn(tl_y, __ddiv_rn(it.delta_y, 2.0));
    it.bbox_br_y = __dadd_rn(br_y, __ddiv_rn(it.delta_y, 2.0));
    it.tl_x = tl_x;
    it.tl_y = tl_y;
    it.lines = lines;
    it.columns = columns;
}

__device__ __forceinline__ void dda_set_theta(DDA &it, double c, double s)
{
    it.cos_theta = c;
    it.sin_theta = s;
    int sign = (int)sgnd(s);
    double a = __dmul_rn((double)sign, it.bbox_br_x), b = __dmul_rn((double)sign, it.bbox_tl_x);
    it.x0 = __dmul_rn((double)sign, (a > b) ? a : b);
    it.Delta_j = (int)(-sgnd(it.delta_x) * sign);
    sign = (int)sgnd(c);
    a = __dmul_rn((double)sign, it.bbox_br_y);
    b = __dmul_rn((double)sign, it.bbox_tl_y);
    it.y0 = __dmul_rn((double)sign, (a < b) ? a : b);
    it.Delta_i = (int)(sgnd(it.delta_y) * sign);
    it.i_init = (it.Delta_i < 0) ? (it.lines - 1) : 0;
    it.j_init = (it.Delta_j < 0) ? (it.columns - 1) : 0;
    double df, ds, sm, lg;
    if (fabs(__dmul_rn(it.delta_x, s)) <= fabs(__dmul_rn(it.delta_y, c))) {
        it.fast_is_i = 1;
        df = it.delta_y; ds = it.delta_x; sm = s; lg = c;
        it.Delta_fast = it.Delta_i; it.Delta_slow = it.Delta_j;
    } else {
        it.fast_is_i = 0;
        df = it.delta_x; ds = it.delta_y; sm = c; lg = s;
        it.Delta_fast = it.Delta_j; it.Delta_slow = it.Delta_i;
    }
    it.epsilon_update = fabs(__ddiv_rn(__dmul_rn(df, sm), lg));
    it.delta_slow = fabs(ds);
    it.sigma_tilde = fabs(__ddiv_rn(df, lg));
    it.sigma_per_eps = it.epsilon_update > 0.0 ? __ddiv_rn(it.sigma_tilde, it.epsilon_update) : 0.0;
    it.sigma_tilde32 = (float)it.sigma_tilde;
    it.sigma_per_eps32 = (float)it.sigma_per_eps;
}

// Forms of the walk's sigma (the pixel decisions are the same in all).
constexpr int kDdaExact = 0;     // the reference's FP64 sigma (traced sequences)
constexpr int kDdaSigma64 = 1;   // FP64 sigma without divisions (FP64 sums)
constexpr int kDdaSigma32 = 2;   // FP32 sigma without divisions (FP32 sums)

// One step of the walk.  The pixel decisions (epsilon's adds, subtracts and
// comparison) are the reference's FP64 operations in every form; epsilon
// and delta_slow are never negative, so the comparison is made on their bit
// patterns, whose integer order is theirs.  kDdaExact also splits sigma at
// a slow move as the reference does, with two divisions: alpha =
// (delta_slow - eps_prev) / eps, sigma = sigma_tilde alpha / (1 + alpha).
// Since eps + delta_slow - eps_prev = epsilon_update, that is sigma =
// (delta_slow - eps_prev) * sigma_tilde / epsilon_update, which the other
// forms compute with one subtract and one multiply by a per-ray constant
// (equal to within rounding: FP64 for kDdaSigma64, FP32 for kDdaSigma32,
// whose kernels sum in FP32).  FP64 division is a long sequence on a slow
// pipe, and a slow move can come every other step.
template <int FORM>
__device__ __forceinline__ void dda_update(DDA &it)
{
    if (it.slow_move) {
        if (it.fast_is_i) it.j += it.Delta_slow; else it.i += it.Delta_slow;
        if (FORM == kDdaSigma32) it.sigma32 = it.sigma_tilde32 - it.sigma32;
        else it.sigma = __dsub_rn(it.sigma_tilde, it.sigma);
        it.slow_move = 0;
    } else {
        if (it.fast_is_i) it.i += it.Delta_fast; else it.j += it.Delta_fast;
        const double eps_prev = it.epsilon;
        it.epsilon = __dadd_rn(it.epsilon, it.epsilon_update);
        if (FORM == kDdaExact)
            it.slow_move = (it.epsilon > it.delta_slow);
        else
            it.slow_move = __double_as_longlong(it.epsilon) > __double_as_longlong(it.delta_slow);
        if (it.slow_move) {
            it.epsilon = __dsub_rn(it.epsilon, it.delta_slow);
            if (FORM == kDdaExact) {
                double alpha;
                if (it.epsilon != 0.0) {
                    alpha = __ddiv_rn(__dsub_rn(it.delta_slow, eps_prev), it.epsilon);
                    alpha = __ddiv_rn(alpha, __dadd_rn(1.0, alpha));
                } else {
                    alpha = 1.0;
                }
                it.sigma = __dmul_rn(alpha, it.sigma_tilde);
            } else if (FORM == kDdaSigma64) {
                it.sigma = __dmul_rn(__dsub_rn(it.delta_slow, eps_prev), it.sigma_per_eps);
            } else {
                it.sigma32 = (float)__dsub_rn(it.delta_slow, eps_prev) * it.sigma_per_eps32;
            }
        } else {
            if (FORM == kDdaSigma32) it.sigma32 = it.sigma_tilde32;
            else it.sigma = it.sigma_tilde;
        }
    }
}

template <int FORM>
__device__ __forceinline__ void dda_set_t(DDA &it, double t)
{
    it.slow_move = 0;
    if (it.sin_theta == 0.0) {
        it.j = (int)dda_index(t, it.tl_x, it.delta_x, it.Delta_j);
        it.i = it.i_init;
        it.epsilon = 0.0;
        it.epsilon_update = 0.0;
        it.sigma = it.sigma_tilde;
        it.sigma32 = it.sigma_tilde32;
        return;
    }
    if (it.cos_theta == 0.0) {
        it.i = (int)dda_index(t, it.tl_y, it.delta_y, it.Delta_i);
        it.j = it.j_init;
        it.epsilon = 0.0;
        it.epsilon_update = 0.0;
        it.sigma = it.sigma_tilde;
        it.sigma32 = it.sigma_tilde32;
        return;
    }
    const double sx = __ddiv_rn(__dsub_rn(__dmul_rn(t, it.cos_theta), it.x0), it.sin_theta);
    const double sy = __ddiv_rn(__dsub_rn(it.y0, __dmul_rn(t, it.sin_theta)), it.cos_theta);
    if (sx > sy) {
        const double xy = __dadd_rn(__dmul_rn(sx, it.cos_theta), __dmul_rn(t, it.sin_theta));
        it.i = (int)dda_index(xy, it.tl_y, it.delta_y, it.Delta_i);
        it.j = it.j_init;
        it.epsilon = fabs(__dsub_rn(xy, __dadd_rn(it.tl_y, __dmul_rn(__dsub_rn((double)it.i,
                                         __dmul_rn(0.5, (double)it.Delta_i)), it.delta_y))));
        if (!it.fast_is_i) {
            it.j -= it.Delta_j;
            dda_update<FORM>(it);
        } else {
            it.epsilon = __dsub_rn(it.epsilon, fabs(it.delta_y));
            it.epsilon = __ddiv_rn(it.epsilon, it.cos_theta);
            it.sigma = fabs(it.epsilon);
            it.sigma32 = (float)it.sigma;
            it.epsilon = fabs(__dmul_rn(it.sigma, it.sin_theta));
        }
    } else {
        const double xy = __dadd_rn(__dmul_rn(-sy, it.sin_theta), __dmul_rn(t, it.cos_theta));
        it.j = (int)dda_index(xy, it.tl_x, it.delta_x, it.Delta_j);
        it.i = it.i_init;
        it.epsilon = fabs(__dsub_rn(xy, __dadd_rn(it.tl_x, __dmul_rn(__dsub_rn((double)it.j,
                                         __dmul_rn(0.5, (double)it.Delta_j)), it.delta_x))));
        if (it.fast_is_i) {
            it.i -= it.Delta_i;
            dda_update<FORM>(it);
        } else {
            it.epsilon = __dsub_rn(it.epsilon, fabs(it.delta_x));
            it.epsilon = __ddiv_rn(it.epsilon, it.sin_theta);
            it.sigma = fabs(it.epsilon);
            it.sigma32 = (float)it.sigma;
            it.epsilon = fabs(__dmul_rn(it.sigma, it.cos_theta));
        }
    }
}

__device__ __forceinline__ bool dda_end(const DDA &it)
{
    // i outside [0, lines) or j outside [0, columns): negative indices wrap
    // to large unsigned values
    return ((unsigned)it.i >= (unsigned)it.lines) | ((unsigned)it.j >= (unsigned)it.columns);
}

// ----------------------------------------------------------------------------
// The walk's decisions in integer arithmetic.  After the walk's first FP64
// add, epsilon is a multiple of ulp(epsilon) >= ulp(epsilon_update), so
// epsilon, epsilon_update u and delta_slow d are all integer multiples of
// q = min(ulp(u), ulp(d)), a power of two.  In units of q:
// - fl(eps + u) is the integer sum rounded to 53 significant bits, to
//   nearest, ties to even (round53): the FP64 add of two multiples of q;
// - with u <= d and eps <= d before every add (it holds by induction once
//   it holds at the start), an eps above d is at most 2d, so fl(eps - d) is
//   exact (Sterbenz) and is the integer difference;
// - the comparison eps > d is the integer comparison;
// - the sigma split at a slow move, (float)fl(d - eps_prev), is
//   __ll2float_rn(round53(D - E_prev)) times q as a float (exact scaling).
// So the integer walk visits the pixels the FP64 walk visits and gives the
// same FP32 sigma bit for bit, without the FP64 pipe (a small fraction of
// the FP32 rate on GB300).  A ray takes it when the conditions hold (u in
// (0, d], eps in [0, d] and a multiple of q, d / q and u / q below 2^60, q
// representable as a normal float); otherwise it stays on the FP64 walk.
struct DDAInt {
    unsigned long long E, U, D;
    int kq;        // q = 2^kq
};

// s rounded to 53 significant bits, to nearest, ties to even: the bits of
// s above bit 52 (m = s >> 53; at most 8 of them in the walk, whose sums
// stay below 2^61) say how many low bits go (sh = their count); adding
// half - 1 plus the kept part's lowest bit and clearing the dropped bits
// rounds to nearest with ties to even.  No branch, and besides the add's
// carry only the low word changes: sh is 0 below 2^53.
__device__ __forceinline__ unsigned long long round53(unsigned long long s)
{
    const unsigned m = (unsigned)(s >> 53);
    const int sh = 32 - __clz((int)m);                  // 0 .. 11
    const unsigned low = (1u << sh) - 1u;               // the dropped bits
    const unsigned bias = (low >> 1) + ((((unsigned)s >> sh) & 1u) & (m != 0u ? 1u : 0u));
    return (s + bias) & ~(unsigned long long)low;
}

// round53 for s < 2^54, where at most one bit is dropped: m = 1 when s has
// 54 bits, and then s + (bit 1 of s) with bit 0 cleared is the nearest even
// multiple of 2 (ties to even); below 2^53 s is returned unchanged.  Four
// 64-bit integer operations in place of round53's bit length and variable
// shifts.
__device__ __forceinline__ unsigned long long round53_small(unsigned long long s)
{
    const unsigned long long m = s >> 53;
    return (s + ((s >> 1) & m)) & ~m;
}

// RN_f32(r) * 2^kq for an integer r < 2^62, built from the integer (r is
// rounded to 24 bits, to nearest, ties to even) so that no 64-bit
// conversion runs on the FP64 pipe.  The result is a normal float for the
// kq that dda_int_init admits.
__device__ __forceinline__ float f32_scaled(unsigned long long r, int kq)
{
    if (r == 0) return 0.f;
    int n = 64 - __clzll((long long)r);
    unsigned long long m;
    if (n > 24) {
        const int sh = n - 24;
        m = (r + ((1ull << (sh - 1)) - 1) + ((r >> sh) & 1ull)) >> sh;
        if (m >> 24) {
            m >>= 1;
            ++n;
        }
    } else {
        m = r << (24 - n);
    }
    return __uint_as_float(((unsigned)(n - 1 + kq + 127) << 23) | ((unsigned)m & 0x7FFFFFu));
}

__device__ __forceinline__ bool dda_int_init(const DDA &it, DDAInt &w)
{
    const double u = it.epsilon_update, d = it.delta_slow, e = it.epsilon;
    if (!(u > 0.0) || !(u <= d) || !(e >= 0.0) || !(e <= d)) return false;
    const int eu = (int)((__double_as_longlong(u) >> 52) & 0x7FF);
    const int ed = (int)((__double_as_longlong(d) >> 52) & 0x7FF);
    if (eu == 0 || ed == 0 || eu == 0x7FF || ed == 0x7FF) return false;
    const int kq = min(eu, ed) - 1023 - 52;               // q = 2^kq
    if (kq < -100 || kq > 60) return false;
    const double inv_q = __longlong_as_double((long long)(1023 - kq) << 52);
    const double Ud = u * inv_q, Dd = d * inv_q, Ed = e * inv_q;   // exact scalings
    if (!(Dd < 0x1p60) || !(Ud < 0x1p60)) return false;
    const long long E = __double2ll_rn(Ed);
    if ((double)E != Ed) return false;                    // epsilon not a multiple of q
    w.U = (unsigned long long)__double2ll_rn(Ud);
    w.D = (unsigned long long)__double2ll_rn(Dd);
    w.E = (unsigned long long)E;
    w.kq = kq;
    return true;
}

// The walk of `it` (set up by dda_set_t<FORM>, FORM kDdaSigma32 or
// kDdaSigma64), at most cap steps: visit(i, j, sigma, slow_move) before each
// update, sigma being it.sigma32 (FP32 form) or it.sigma (FP64 form) and
// slow_move the move that update makes.  FP64 updates run until the walk's
// first epsilon add (at most two), then the integer walk where it applies
// (fp64_walk == 0), else FP64 to the end.  The integer walk makes one fast
// move per iteration in every lane, so that the lanes of a warp, whose rays
// are at different phases of their slow moves, stay together; only the
// visit and the slow move that a fast move triggers are predicated.  The
// sigma split at a slow move is the FP64 walk's: (float)fl(d - eps_prev) * s
// in FP32 (built from the rounded integer, f32_scaled), fl(fl(d - eps_prev)
// * s) in FP64 (the difference is an exact double, and scaling s by 2^kq
// first leaves the product's rounding unchanged).
template <int FORM, class Visit>
__device__ __forceinline__ int dda_walk(DDA &it, int cap, int fp64_walk, Visit &&visit)
{
    static_assert(FORM == kDdaSigma32 || FORM == kDdaSigma64, "sigma form");
    auto sig = [&]() {
        if constexpr (FORM == kDdaSigma32) return it.sigma32;
        else return it.sigma;
    };
    int step = 0;
    bool added = false;
    for (; step < cap && !dda_end(it) && !added; ++step) {
        visit(it.i, it.j, sig(), it.slow_move);
        added = !it.slow_move;
        dda_update<FORM>(it);
    }
    DDAInt w;
    if (added && !fp64_walk && dda_int_init(it, w)) {
        // sigma_per_eps times q, exact (a power-of-two scaling)
        const double sp_q = it.sigma_per_eps * __longlong_as_double((long long)(1023 + w.kq) << 52);
        if (it.slow_move && step < cap && !dda_end(it)) {   // pending from the FP64 steps
            visit(it.i, it.j, sig(), 1);
            ++step;
            if (it.fast_is_i) it.j += it.Delta_slow; else it.i += it.Delta_slow;
            if constexpr (FORM == kDdaSigma32) it.sigma32 = it.sigma_tilde32 - it.sigma32;
            else it.sigma = __dsub_rn(it.sigma_tilde, it.sigma);
            it.slow_move = 0;
        }
        // Every sum the loop rounds (E + U, D - E_prev) is below D + U.  When
        // that is below 2^54, which holds for all the rays of a view more
        // than about 18 degrees from its fast axis, at most one bit is
        // dropped and round53_small does it; the rays of a warp share their
        // view, so the choice is the same across the warp.
        auto walk = [&](auto small) {
            constexpr bool kSmall = decltype(small)::value;
            auto rnd = [](unsigned long long v) {
                if constexpr (kSmall) return round53_small(v);
                else return round53(v);
            };
            while (step < cap && !dda_end(it)) {
                visit(it.i, it.j, sig(), 0);
                ++step;
                if (it.fast_is_i) it.i += it.Delta_fast; else it.j += it.Delta_fast;
                const unsigned long long prev = w.E;
                w.E = rnd(w.E + w.U);
                if (w.E <= w.D) {
                    if constexpr (FORM == kDdaSigma32) it.sigma32 = it.sigma_tilde32;
                    else it.sigma = it.sigma_tilde;
                    continue;
                }
                w.E -= w.D;                          // fl(eps - d), exact
                const unsigned long long diff = rnd(w.D - prev);
                if constexpr (FORM == kDdaSigma32)
                    it.sigma32 = f32_scaled(diff, w.kq) * it.sigma_per_eps32;
                else
                    it.sigma = __dmul_rn(__ll2double_rn((long long)diff), sp_q);
                if (step >= cap || dda_end(it)) break;
                visit(it.i, it.j, sig(), 1);
                ++step;
                if (it.fast_is_i) it.j += it.Delta_slow; else it.i += it.Delta_slow;
                if constexpr (FORM == kDdaSigma32) it.sigma32 = it.sigma_tilde32 - it.sigma32;
                else it.sigma = __dsub_rn(it.sigma_tilde, it.sigma);
            }
        };
        if (w.D + w.U < (1ull << 54)) walk(std::true_type{});
        else walk(std::false_type{});
    } else {
        for (; step < cap && !dda_end(it); ++step) {
            visit(it.i, it.j, sig(), it.slow_move);
            dda_update<FORM>(it);
        }
    }
    return step;
}

// ----------------------------------------------------------------------------

// I32: every pixel offset (row ics + column ils) fits in an int, so the
// walk's per-pixel address is 32-bit arithmetic.
template <bool RATIO, bool I32>
__global__ __launch_bounds__(128) void k_bres_radon(DDAGeom g, const double *__restrict__ cs_tab,
                                                    const float *__restrict__ img, long long ics,
                                                    long long ils, float *__restrict__ out,
                                                    long long ocs, long long ols,
                                                    const float *__restrict__ y_am, int first,
                                                    int stride, int fp64_walk)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;   // ray
    const int j = first + blockIdx.y * stride;             // view
    if (i >= g.R) return;
    DDA it;
    dda_set_image(it, g.lines, g.columns, g.itl_x, g.itl_y, g.ibr_x, g.ibr_y);
    dda_set_theta(it, cs_tab[2 * j], cs_tab[2 * j + 1]);
    const double dts = __ddiv_rn(__dsub_rn(g.sbr_y, g.stl_y), (double)(g.R - 1));
    dda_set_t<kDdaSigma32>(it, __dadd_rn(g.stl_y, __dmul_rn((double)i, dts)));
    float acc = 0.f, comp = 0.f;
    const int cap = 2 * (g.lines + g.columns) + 8;
    const int ics32 = (int)ics, ils32 = (int)ils;
    dda_walk<kDdaSigma32>(it, cap, fp64_walk, [&](int pi, int pj, float sg, int) {
        const float *px = I32 ? img + (pi * ics32 + pj * ils32)
                              : img + (long long)pi * ics + (long long)pj * ils;
        const float x = __ldg(px) * sg;
        const float y = x - comp, t = acc + y;
        comp = (t - acc) - y;
        acc = t;
    });
    float val = acc - comp;
    if (RATIO) {
        const float yv = y_am[(size_t)j * g.R + i];
        val = (val != 0.f) ? yv / val : 0.f;
    }
    out[(long long)i * ocs + (long long)j * ols] = val;
}

// RG_DDA_FP64=1 (read per call) keeps the DDA Radon, transpose, walk
// recording and normalised backprojection on the FP64 walk: the integer
// walk's reference for tests and A/B timing; both visit the same pixels
// with the same sigma.
static int dda_fp64_walk()
{
    const char *e = getenv("RG_DDA_FP64");
    return (e && e[0] == '1' && e[1] == 0) ? 1 : 0;
}

int launch_bres_radon(const DDAGeom &g, const double *d_cs, const float *img, long long ics,
                      long long ils, float *out, long long ocs, long long ols,
                      const float *y_am, int first, int stride, cudaStream_t st)
{
    const int nv = (g.A - first + stride - 1) / stride;
    if (nv <= 0) return RG_OK;
    dim3 grid((g.R + 127) / 128, nv);
    // offsets of the image's pixels in 32 bits when they fit
    const long long span = (long long)(g.lines - 1) * (ics < 0 ? -ics : ics) +
                           (long long)(g.columns - 1) * (ils < 0 ? -ils : ils);
    const bool i32 = span < (1LL << 31) - 1;
    auto k = y_am ? (i32 ? k_bres_radon<true, true> : k_bres_radon<true, false>)
                  : (i32 ? k_bres_radon<false, true> : k_bres_radon<false, false>);
    k<<<grid, 128, 0, st>>>(g, d_cs, img, ics, ils, out, ocs, ols, y_am, first, stride,
                            dda_fp64_walk());
    RG_CK_LAUNCH("k_bres_radon");
    return RG_OK;
}

// s(i, j) = s_am[j * R + i]; img_c: contiguous lines x columns, pre-zeroed.
// den != nullptr: also accumulate the intersection lengths.  I32: lines x
// columns fits in an int, so pixel indices are 32-bit arithmetic.
template <bool I32>
__global__ __launch_bounds__(128) void k_bres_transpose(DDAGeom g, const double *__restrict__ cs_tab,
                                                        const float *__restrict__ s_am,
                                                        float *__restrict__ img_c, int first,
                                                        int stride, float *__restrict__ den,
                                                        int fp64_walk)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = first + blockIdx.y * stride;
    if (i >= g.R) return;
    const float sv = s_am[(size_t)j * g.R + i];
    if (sv == 0.f && !den) return;
    DDA it;
    dda_set_image(it, g.lines, g.columns, g.itl_x, g.itl_y, g.ibr_x, g.ibr_y);
    dda_set_theta(it, cs_tab[2 * j], cs_tab[2 * j + 1]);
    const double dts = __ddiv_rn(__dsub_rn(g.sbr_y, g.stl_y), (double)(g.R - 1));
    dda_set_t<kDdaSigma32>(it, __dadd_rn(g.stl_y, __dmul_rn((double)i, dts)));
    const int cap = 2 * (g.lines + g.columns) + 8;
    dda_walk<kDdaSigma32>(it, cap, fp64_walk, [&](int pi, int pj, float sg, int) {
        const long long e = I32 ? (long long)(pi * g.columns + pj)
                                : (long long)pi * g.columns + pj;
        if (sv != 0.f) atomicAdd(img_c + e, sv * sg);
        if (den) atomicAdd(den + e, sg);
    });
}

// Normalised backprojection in FP64: sum(s sigma) and sum(sigma) per pixel.
// A pixel grazed by a single short intersection has a tiny weight sum, and
// the quotient inherits the relative error of that sum, so both sums stay in
// FP64 (sigma is FP64 already).
__global__ __launch_bounds__(128) void k_bres_norm_sums(DDAGeom g, const double *__restrict__ cs_tab,
                                                        const float *__restrict__ s_am,
                                                        double *__restrict__ num,
                                                        double *__restrict__ den, int fp64_walk)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= g.R) return;
    const double sv = s_am[(size_t)j * g.R + i];
    DDA it;
    dda_set_image(it, g.lines, g.columns, g.itl_x, g.itl_y, g.ibr_x, g.ibr_y);
    dda_set_theta(it, cs_tab[2 * j], cs_tab[2 * j + 1]);
    const double dts = __ddiv_rn(__dsub_rn(g.sbr_y, g.stl_y), (double)(g.R - 1));
    dda_set_t<kDdaSigma64>(it, __dadd_rn(g.stl_y, __dmul_rn((double)i, dts)));
    const int cap = 2 * (g.lines + g.columns) + 8;
    dda_walk<kDdaSigma64>(it, cap, fp64_walk, [&](int pi, int pj, double sg, int) {
        const size_t e = (size_t)pi * g.columns + pj;
        if (sv != 0.0) atomicAdd(num + e, sv * sg);
        atomicAdd(den + e, sg);
    });
}

// out(strided) = num / den, 0 where den == 0.
__global__ void k_bres_normalise(const double *__restrict__ num, const double *__restrict__ den,
                                 int lines, int cols, float *__restrict__ out, long long cs,
                                 long long ls)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y;
    if (c >= cols) return;
    const size_t e = (size_t)r * cols + c;
    out[(long long)r * cs + (long long)c * ls] = den[e] != 0.0 ? (float)(num[e] / den[e]) : 0.f;
}

int launch_bres_normalised(const DDAGeom &g, const double *d_cs, const float *s_am, double *num,
                           double *den, float *out, long long cs, long long ls, cudaStream_t st)
{
    dim3 grid((g.R + 127) / 128, g.A);
    k_bres_norm_sums<<<grid, 128, 0, st>>>(g, d_cs, s_am, num, den, dda_fp64_walk());
    RG_CK_LAUNCH("k_bres_norm_sums");
    dim3 g2((g.columns + 127) / 128, g.lines);
    k_bres_normalise<<<g2, 128, 0, st>>>(num, den, g.lines, g.columns, out, cs, ls);
    RG_CK_LAUNCH("k_bres_normalise");
    return RG_OK;
}

int launch_bres_transpose(const DDAGeom &g, const double *d_cs, const float *s_am, float *img_c,
                          int first, int stride, cudaStream_t st)
{
    const int nv = (g.A - first + stride - 1) / stride;
    if (nv <= 0) return RG_OK;
    dim3 grid((g.R + 127) / 128, nv);
    auto k = (long long)g.lines * g.columns < (1LL << 31) ? k_bres_transpose<true>
                                                          : k_bres_transpose<false>;
    k<<<grid, 128, 0, st>>>(g, d_cs, s_am, img_c, first, stride, nullptr, dda_fp64_walk());
    RG_CK_LAUNCH("k_bres_transpose");
    return RG_OK;
}

// Pixel sequences of arbitrary rays (cos, sin, t per ray).
__global__ void k_dda_trace(int lines, int columns, double tl_x, double tl_y, double br_x,
                            double br_y, const double *__restrict__ cst, int n, int cap,
                            int *__restrict__ oi, int *__restrict__ oj, double *__restrict__ os,
                            int *__restrict__ ocount)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    DDA it;
    dda_set_image(it, lines, columns, tl_x, tl_y, br_x, br_y);
    dda_set_theta(it, cst[3 * r], cst[3 * r + 1]);
    dda_set_t<kDdaExact>(it, cst[3 * r + 2]);
    int cnt = 0;
    const int limit = 2 * (lines + columns) + 8;
    while (!dda_end(it) && cnt < limit) {
        if (cnt < cap) {
            oi[(size_t)r * cap + cnt] = it.i;
            oj[(size_t)r * cap + cnt] = it.j;
            os[(size_t)r * cap + cnt] = it.sigma;
        }
        ++cnt;
        dda_update<kDdaExact>(it);
    }
    ocount[r] = cnt;
}

int launch_dda_trace(int lines, int columns, const double *corners, const double *d_cst, int n,
                     int cap, int *oi, int *oj, double *os, int *ocount, cudaStream_t st)
{
    k_dda_trace<<<(n + 127) / 128, 128, 0, st>>>(lines, columns, corners[0], corners[1],
                                                  corners[2], corners[3], d_cst, n, cap, oi, oj,
                                                  os, ocount);
    RG_CK_LAUNCH("k_dda_trace");
    return RG_OK;
}

// ============================================================================
// Recorded walks (DDAPlan).  Iterative reconstruction walks the same rays
// in every sub-iteration, and the walk is bound by the FP64 pipe.  A plan
// records each ray's walk once: per step one FP32 word, the step's sigma
// (kDdaSigma32, what the walking kernels use) whose lowest mantissa bit is
// replaced by the move flag (1: the step moved along the slow axis; the
// weight changes by at most one unit in the last place, and unlike the
// sign bit the flag survives a sigma of zero or a rounding just below
// zero, which a slow move's remainder can be); per ray its entry pixel, the
// pixel-index increments of a fast and a slow move, and its steps' offset
// and count.  Replaying a ray is then a streamed read: a warp takes a ray,
// its lanes consecutive steps, and a ballot over the slow bits gives each
// lane its pixel (entry + s fast moves + (slow moves so far) x (slow - fast
// increment)).  The pixel sequences are those of the walk, and the sigmas
// within one unit in the last place, so results match the walking kernels
// to FP32 rounding.

struct DDARayRec {
    long long off;     // first step in the step array
    int count;         // steps (pixels) of the ray; 0 if it misses the image
    int start;         // entry pixel index, in the ray's layout
    int dfast, dslow;  // pixel-index increment of a fast / slow move
    int colmajor;      // layout: 1 column-major (rays whose fast axis runs
                       // down the columns), 0 row-major; a warp's 32
                       // consecutive steps then lie on one or two lines
};

// Walk (ray i of view first + y * stride) and count (W = false) or record
// (W = true) its steps.
template <bool W>
__global__ __launch_bounds__(128) void k_dda_plan(DDAGeom g, const double *__restrict__ cs_tab,
                                                  int first, int stride,
                                                  DDARayRec *__restrict__ rays,
                                                  float *__restrict__ steps, int fp64_walk)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = first + blockIdx.y * stride;
    if (i >= g.R) return;
    const size_t r = (size_t)blockIdx.y * g.R + i;
    DDA it;
    dda_set_image(it, g.lines, g.columns, g.itl_x, g.itl_y, g.ibr_x, g.ibr_y);
    dda_set_theta(it, cs_tab[2 * j], cs_tab[2 * j + 1]);
    const double dts = __ddiv_rn(__dsub_rn(g.sbr_y, g.stl_y), (double)(g.R - 1));
    dda_set_t<kDdaSigma32>(it, __dadd_rn(g.stl_y, __dmul_rn((double)i, dts)));
    const int cap = 2 * (g.lines + g.columns) + 8;
    const long long off = W ? rays[r].off : 0;
    int n = 0;
    if (!W) {
        // fast axis i (down the columns): column-major, index j * lines + i
        const int cm = it.fast_is_i;
        rays[r].colmajor = cm;
        rays[r].start = cm ? it.j * g.lines + it.i : it.i * g.columns + it.j;
        rays[r].dfast = it.Delta_fast;
        rays[r].dslow = cm ? it.Delta_slow * g.lines : it.Delta_slow * g.columns;
    }
    int moved_slow = 0;
    dda_walk<kDdaSigma32>(it, cap, fp64_walk, [&](int, int, float sg, int slow) {
        if (W) steps[off + n] = __uint_as_float((__float_as_uint(sg) & ~1u) | moved_slow);
        moved_slow = slow;
        ++n;
    });
    if (!W) rays[r].count = n;
}

// Replay: warp per ray.  Radon: out_am[view row][i] = sum img * sigma (the
// EM ratio y / Ax if y_am); transpose: img += s * sigma (atomics).  Each
// reads or adds to the image in its ray's layout: img_c / img_o row-major,
// imgT_c / imgT_o the column-major copy.
// Four 32-step chunks per round: their step words are loaded first, then
// their pixels, so that a warp keeps several loads in flight (a ray has ~30
// to ~140 chunks, and one chunk at a time leaves the replay latency-bound).
template <int OP>
__device__ __forceinline__ void dda_replay(const DDARayRec &rec, const float *__restrict__ steps,
                                           const float *__restrict__ img_c, float *__restrict__ img_o,
                                           float sv, float &sum)
{
    constexpr int kU = 4;
    const int lane = threadIdx.x & 31;
    const int dd = rec.dslow - rec.dfast;
    const unsigned le = 0xffffffffu >> (31 - lane);
    int slows = 0;                     // slow moves before this round
    for (int c = 0; c < rec.count; c += 32 * kU) {
        float w[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const int s = c + 32 * u + lane;
            w[u] = s < rec.count ? __ldg(steps + rec.off + s) : 0.f;
        }
        int pix[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const unsigned sb = __ballot_sync(0xffffffffu, __float_as_uint(w[u]) & 1u);
            const int s = c + 32 * u + lane;
            pix[u] = rec.start + s * rec.dfast + (slows + __popc(sb & le)) * dd;
            slows += __popc(sb);
        }
        if (OP == 0) {
            float v[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int s = c + 32 * u + lane;
                v[u] = s < rec.count ? __ldg(img_c + pix[u]) : 0.f;
            }
#pragma unroll
            for (int u = 0; u < kU; ++u) sum = fmaf(v[u], w[u], sum);
        } else {
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int s = c + 32 * u + lane;
                if (s < rec.count) atomicAdd(img_o + pix[u], sv * w[u]);
            }
        }
    }
}

__global__ __launch_bounds__(256) void k_dda_plan_radon(const DDARayRec *__restrict__ rays,
                                                        const float *__restrict__ steps,
                                                        long long nrays, int R, int first,
                                                        int stride, const float *__restrict__ img,
                                                        const float *__restrict__ imgT,
                                                        float *__restrict__ out_am,
                                                        const float *__restrict__ y_am)
{
    const long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (r >= nrays) return;                        // warp-uniform
    const DDARayRec rec = rays[r];
    float sum = 0.f;
    dda_replay<0>(rec, steps, rec.colmajor ? imgT : img, nullptr, 0.f, sum);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31) == 0) {
        const int i = (int)(r % R), j = first + (int)(r / R) * stride;
        const size_t e = (size_t)j * R + i;
        float val = sum;
        if (y_am) val = (val != 0.f) ? y_am[e] / val : 0.f;
        out_am[e] = val;
    }
}

__global__ __launch_bounds__(256) void k_dda_plan_transpose(const DDARayRec *__restrict__ rays,
                                                            const float *__restrict__ steps,
                                                            long long nrays, int R, int first,
                                                            int stride,
                                                            const float *__restrict__ s_am,
                                                            float *__restrict__ img_c,
                                                            float *__restrict__ imgT_c)
{
    const long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (r >= nrays) return;                        // warp-uniform
    const int i = (int)(r % R), j = first + (int)(r / R) * stride;
    const float sv = s_am[(size_t)j * R + i];
    if (sv == 0.f) return;                         // warp-uniform
    float unused = 0.f;
    const DDARayRec rec = rays[r];
    dda_replay<1>(rec, steps, nullptr, rec.colmajor ? imgT_c : img_c, sv, unused);
}

void dda_plan_free(DDAPlan &p)
{
    if (p.rays) cudaFree(p.rays);
    if (p.steps) cudaFree(p.steps);
    p.rays = nullptr;
    p.steps = nullptr;
    p.nrays = 0;
    p.total = 0;
}

// Builds the plan of views first, first + stride, ... (two walks: count,
// then record).  Leaves p empty (and returns RG_OK) when its steps would
// take more than `max_bytes` or more than a third of the free device memory.
int dda_plan_build(const DDAGeom &g, const double *d_cs, int first, int stride,
                   size_t max_bytes, DDAPlan &p, cudaStream_t st)
{
    dda_plan_free(p);
    const int nv = (g.A - first + stride - 1) / stride;
    if (nv <= 0) return RG_OK;
    p.first = first;
    p.stride = stride;
    p.nrays = (long long)g.R * nv;
    RG_CK(cudaMalloc(&p.rays, sizeof(DDARayRec) * (size_t)p.nrays));
    DDARayRec *rays = (DDARayRec *)p.rays;
    dim3 grid((g.R + 127) / 128, nv);
    k_dda_plan<false><<<grid, 128, 0, st>>>(g, d_cs, first, stride, rays, nullptr,
                                            dda_fp64_walk());
    RG_CK_LAUNCH("k_dda_plan (count)");
    std::vector<DDARayRec> h((size_t)p.nrays);
    RG_CK(cudaMemcpyAsync(h.data(), rays, sizeof(DDARayRec) * h.size(), cudaMemcpyDeviceToHost, st));
    RG_CK(cudaStreamSynchronize(st));
    long long total = 0;
    for (auto &rec : h) {
        rec.off = total;
        total += rec.count;
    }
    size_t freeb = 0, totb = 0;
    RG_CK(cudaMemGetInfo(&freeb, &totb));
    const size_t bytes = sizeof(float) * (size_t)std::max(total, 1LL);
    if (bytes > max_bytes || bytes > freeb / 3) {
        dda_plan_free(p);
        return RG_OK;
    }
    RG_CK(cudaMemcpyAsync(rays, h.data(), sizeof(DDARayRec) * h.size(), cudaMemcpyHostToDevice, st));
    RG_CK(cudaMalloc(&p.steps, bytes));
    k_dda_plan<true><<<grid, 128, 0, st>>>(g, d_cs, first, stride, rays, (float *)p.steps,
                                           dda_fp64_walk());
    RG_CK_LAUNCH("k_dda_plan (record)");
    RG_CK(cudaStreamSynchronize(st));   // h is released on return
    p.total = total;
    return RG_OK;
}

int launch_dda_plan_radon(const DDAGeom &g, const DDAPlan &p, const float *img_c,
                          const float *imgT_c, float *out_am, const float *y_am, cudaStream_t st)
{
    const long long threads = p.nrays * 32;
    k_dda_plan_radon<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
        (const DDARayRec *)p.rays, (const float *)p.steps, p.nrays, g.R, p.first, p.stride, img_c,
        imgT_c, out_am, y_am);
    RG_CK_LAUNCH("k_dda_plan_radon");
    return RG_OK;
}

int launch_dda_plan_transpose(const DDAGeom &g, const DDAPlan &p, const float *s_am, float *img_c,
                              float *imgT_c, cudaStream_t st)
{
    const long long threads = p.nrays * 32;
    k_dda_plan_transpose<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
        (const DDARayRec *)p.rays, (const float *)p.steps, p.nrays, g.R, p.first, p.stride, s_am,
        img_c, imgT_c);
    RG_CK_LAUNCH("k_dda_plan_transpose");
    return RG_OK;
}

}  // namespace rg
