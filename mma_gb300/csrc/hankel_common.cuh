// hankel_common.cuh -- helpers shared by the far-field kernels (hankel.cu, hankel_tc.cu).
#pragma once

#include <cmath>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/mma_hankel.h"

namespace mma {
namespace hk {

constexpr double kC = 299792458.0;  // shared_python/units.py:3

__device__ __forceinline__ double trap_w(const double* x, int64_t i, int64_t n)
{
    double w = 0.0;
    if (i + 1 < n) w += 0.5 * (x[i + 1] - x[i]);
    if (i > 0) w += 0.5 * (x[i] - x[i - 1]);
    return w;
}

__device__ __forceinline__ double2 load_src_d(const void* src, int64_t idx, int64_t c128)
{
    if (c128) return reinterpret_cast<const double2*>(src)[idx];
    const float2 v = reinterpret_cast<const float2*>(src)[idx];
    return make_double2(v.x, v.y);
}

__device__ __forceinline__ float2 load_src_f(const void* src, int64_t idx, int64_t c128)
{
    if (c128) {
        const double2 v = reinterpret_cast<const double2*>(src)[idx];
        return make_float2((float)v.x, (float)v.y);
    }
    return reinterpret_cast<const float2*>(src)[idx];
}

// ------------------------------------------------------------------------ fast form helpers
__device__ __forceinline__ void split_d(double v, float& hi, float& lo)
{
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

// The largest x = sigma y / 2 at which m series terms still meet the plan's truncation bound,
// x^m / m! e^x <= trunc_bound (bisection; the bound grows with x); -1 if m < 2 (never taken).
// Stage 2 takes fewer terms where the chunk's largest y is small enough, so every term of the
// sum keeps the plan's bound.
inline float series_cut(const mma_hankel_fast_plan_t* plan, int m)
{
    if (m < 2) return -1.f;
    auto bound = [m](double x) {
        double t = 1.0;
        for (int q = 1; q <= m; q++) t *= x / q;
        return t * std::exp(x);
    };
    double lo = 0.0, hi = 0.5 * plan->sigma * plan->y_max;
    if (bound(hi) <= plan->trunc_bound) return (float)hi;
    for (int it = 0; it < 80; it++) {
        const double mid = 0.5 * (lo + hi);
        (bound(mid) <= plan->trunc_bound ? lo : hi) = mid;
    }
    return (float)(lo * (1.0 - 1e-6));
}

// (yh + yl) reduced mod 2 pi with 2 pi = C1 + C2 + C3 (C1, C2 short enough that k*C is exact)
__device__ __forceinline__ float reduce_2pi(float yh, float yl)
{
    const float kk = rintf(yh * 0.159154943f);
    float r = fmaf(-kk, 6.28125f, yh);
    r = fmaf(-kk, 1.93500518798828125e-3f, r);
    r = fmaf(-kk, 3.0199159819370158e-07f, r);
    return r + yl;
}

// sin and cos of x for |x| <= 5 (phases already reduced mod 2 pi by reduce_2pi, and the Bessel
// phases below): x = k pi/2 + r by Cody and Waite's
// two-part additive reduction (pi/2 = 1.5703125 + 4.83826794896619e-4, the first part exact
// times k), |r| <= pi/4, then the Taylor polynomials of sin (to r^9) and cos (to r^8), whose
// remainders stay below 3e-8 there; the quadrant is k mod 4.  Max |error| 9e-8 on [-4.2, 3.6]
// (float32 emulation against FP64).
__device__ __forceinline__ void sincos_reduced(float x, float& s, float& c)
{
    const float k = rintf(x * 0.636619772f);
    float r = fmaf(-k, 1.5703125f, x);
    r = fmaf(-k, 4.83826794896619e-4f, r);
    const float r2 = r * r;
    const float ps =
        r * fmaf(r2, fmaf(r2, fmaf(r2, fmaf(r2, 2.75573192e-6f, -1.98412698e-4f), 8.33333333e-3f), -1.66666667e-1f), 1.0f);
    const float pc = fmaf(r2, fmaf(r2, fmaf(r2, fmaf(r2, 2.48015873e-5f, -1.38888889e-3f), 4.16666667e-2f), -0.5f), 1.0f);
    const int q = (int)k & 3;
    const float ss = (q & 1) ? pc : ps, cc = (q & 1) ? ps : pc;
    s = (q & 2) ? -ss : ss;
    c = ((q + 1) & 2) ? -cc : cc;
}

// sin and cos of a small angle |p| <= 0.13 (Taylor to p^5 and p^4; remainders below 6e-9)
__device__ __forceinline__ void sincos_small(float p, float& s, float& c)
{
    const float p2 = p * p;
    s = p * fmaf(p2, fmaf(p2, 8.33333333e-3f, -1.66666667e-1f), 1.0f);
    c = fmaf(p2, fmaf(p2, 4.16666667e-2f, -0.5f), 1.0f);
}

// sincos_small with the two polynomials as one packed pair, (cos p, sin p / p): each lane the
// operations of sincos_small in the same order (the same bits)
__device__ __forceinline__ void sincos_small_p(float p, float& s, float& c)
{
    const float p2 = p * p;
    const float2 q2 = make_float2(p2, p2);
    float2 cs = __ffma2_rn(q2, make_float2(4.16666667e-2f, 8.33333333e-3f), make_float2(-0.5f, -1.66666667e-1f));
    cs = __ffma2_rn(q2, cs, make_float2(1.0f, 1.0f));
    c = cs.x;
    s = p * cs.y;
}

// J0 and J1 in FP32 from the rational/asymptotic approximations of Abramowitz & Stegun
// 9.4.1, 9.4.4 (x < 3) and 9.4.3, 9.4.6 (x >= 3; modulus and phase, |error| < 1e-7 absolute),
// with the phase argument x reduced mod 2 pi in float-float (x = yh + yl).  For x >= 3 the two
// cosines cos(x - pi/4 + p0) and cos(x - 3 pi/4 + p1) come from one sin/cos of the reduced x,
// rotated by the small phase corrections p0, p1 through the angle-addition identities
// (cos(-pi/4) = sin(pi/4) = 1/sqrt 2): max |J - J_exact| 1.0e-7 (J0) and 1.25e-7 (J1) on
// [3, 3000] in a float32 emulation, the approximations' own error.
template <bool WANT_J1>
__device__ __forceinline__ void bessel01(float yh, float yl, float& J0, float& J1)
{
    if (yh < 3.0f) {
        const float y = yh + yl;
        const float u = (y * 0.333333343f) * (y * 0.333333343f);
        J0 = fmaf(u, fmaf(u, fmaf(u, fmaf(u, fmaf(u, fmaf(u, 0.0002100f, -0.0039444f), 0.0444479f), -0.3163866f),
                                      1.2656208f), -2.2499997f), 1.0f);
        if (WANT_J1)
            J1 = y * fmaf(u, fmaf(u, fmaf(u, fmaf(u, fmaf(u, fmaf(u, 0.00001109f, -0.00031761f), 0.00443319f),
                                               -0.03954289f), 0.21093573f), -0.56249985f), 0.5f);
    } else {
        const float t = __fdividef(3.0f, yh);
        const float red = reduce_2pi(yh, yl);
        const float sq = rsqrtf(yh);
        float sr, cr;
        sincos_reduced(red, sr, cr);
        const float a = cr + sr, b = cr - sr;
        const float f0 = fmaf(t, fmaf(t, fmaf(t, fmaf(t, fmaf(t, fmaf(t, 0.00014476f, -0.00072805f), 0.00137237f),
                                                   -0.00009512f), -0.00552740f), -0.00000077f), 0.79788456f);
        const float p0 = t * fmaf(t, fmaf(t, fmaf(t, fmaf(t, fmaf(t, 0.00013558f, -0.00029333f), -0.00054125f),
                                               0.00262573f), -0.00003954f), -0.04166397f);
        float s0, c0;
        sincos_small(p0, s0, c0);
        J0 = f0 * sq * (0.707106781f * fmaf(c0, a, s0 * b));  // cos(x - pi/4 + p0)
        if (WANT_J1) {
            const float f1 = fmaf(t, fmaf(t, fmaf(t, fmaf(t, fmaf(t, fmaf(t, -0.00020033f, 0.00113653f), -0.00249511f),
                                                       0.00017105f), 0.01659667f), 0.00000156f), 0.79788456f);
            const float p1 = t * fmaf(t, fmaf(t, fmaf(t, fmaf(t, fmaf(t, -0.00029166f, 0.00079824f), 0.00074348f),
                                                   -0.00637879f), 0.00005650f), 0.12499612f);
            float s1, c1;
            sincos_small(p1, s1, c1);
            J1 = f1 * sq * (0.707106781f * fmaf(s1, a, -c1 * b));  // cos(x - 3 pi/4 + p1)
        }
    }
}

// The same J0 and J1 for two arguments at once (x = (yh + yl).x and .y).  When both are >= 3 the
// modulus/phase branch runs as packed FP32x2 instructions, each lane the operations of bessel01 in
// the same order (the same bits); otherwise each lane takes bessel01.
__device__ __forceinline__ float2 b2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 poly6(float2 t, float c6, float c5, float c4, float c3, float c2, float c1, float c0)
{
    return __ffma2_rn(t, __ffma2_rn(t, __ffma2_rn(t, __ffma2_rn(t, __ffma2_rn(t, __ffma2_rn(t, b2(c6), b2(c5)), b2(c4)),
                                                              b2(c3)), b2(c2)), b2(c1)), b2(c0));
}
__device__ __forceinline__ float2 poly5(float2 t, float c5, float c4, float c3, float c2, float c1, float c0)
{
    return __ffma2_rn(t, __ffma2_rn(t, __ffma2_rn(t, __ffma2_rn(t, __ffma2_rn(t, b2(c5), b2(c4)), b2(c3)), b2(c2)),
                                    b2(c1)), b2(c0));
}
__device__ __forceinline__ void sincos_small2(float2 p, float2& s, float2& c)
{
    const float2 p2 = __fmul2_rn(p, p);
    s = __fmul2_rn(p, __ffma2_rn(p2, __ffma2_rn(p2, b2(8.33333333e-3f), b2(-1.66666667e-1f)), b2(1.0f)));
    c = __ffma2_rn(p2, __ffma2_rn(p2, b2(4.16666667e-2f), b2(-0.5f)), b2(1.0f));
}
template <bool WANT_J1>
__device__ __forceinline__ void bessel01x2(float2 yh, float2 yl, float2& J0, float2& J1)
{
    if (!(yh.x >= 3.0f && yh.y >= 3.0f)) {
        bessel01<WANT_J1>(yh.x, yl.x, J0.x, J1.x);
        bessel01<WANT_J1>(yh.y, yl.y, J0.y, J1.y);
        return;
    }
    const float2 t = make_float2(__fdividef(3.0f, yh.x), __fdividef(3.0f, yh.y));
    // reduce_2pi, lane by lane
    const float2 kk = make_float2(rintf(yh.x * 0.159154943f), rintf(yh.y * 0.159154943f));
    const float2 nk = make_float2(-kk.x, -kk.y);
    float2 red = __ffma2_rn(nk, b2(6.28125f), yh);
    red = __ffma2_rn(nk, b2(1.93500518798828125e-3f), red);
    red = __ffma2_rn(nk, b2(3.0199159819370158e-07f), red);
    red = __fadd2_rn(red, yl);
    const float2 sq = make_float2(rsqrtf(yh.x), rsqrtf(yh.y));
    // sincos_reduced, lane by lane
    const float2 k = make_float2(rintf(red.x * 0.636619772f), rintf(red.y * 0.636619772f));
    const float2 mk = make_float2(-k.x, -k.y);
    float2 r = __ffma2_rn(mk, b2(1.5703125f), red);
    r = __ffma2_rn(mk, b2(4.83826794896619e-4f), r);
    const float2 r2 = __fmul2_rn(r, r);
    const float2 ps = __fmul2_rn(
        r, __ffma2_rn(r2, __ffma2_rn(r2, __ffma2_rn(r2, __ffma2_rn(r2, b2(2.75573192e-6f), b2(-1.98412698e-4f)),
                                                    b2(8.33333333e-3f)), b2(-1.66666667e-1f)), b2(1.0f)));
    const float2 pc = __ffma2_rn(r2, __ffma2_rn(r2, __ffma2_rn(r2, __ffma2_rn(r2, b2(2.48015873e-5f), b2(-1.38888889e-3f)),
                                                              b2(4.16666667e-2f)), b2(-0.5f)), b2(1.0f));
    float2 sr, cr;
    {
        const int qx = (int)k.x & 3, qy = (int)k.y & 3;
        const float ssx = (qx & 1) ? pc.x : ps.x, ccx = (qx & 1) ? ps.x : pc.x;
        const float ssy = (qy & 1) ? pc.y : ps.y, ccy = (qy & 1) ? ps.y : pc.y;
        sr = make_float2((qx & 2) ? -ssx : ssx, (qy & 2) ? -ssy : ssy);
        cr = make_float2(((qx + 1) & 2) ? -ccx : ccx, ((qy + 1) & 2) ? -ccy : ccy);
    }
    const float2 a = __fadd2_rn(cr, sr), b = __fadd2_rn(cr, make_float2(-sr.x, -sr.y));
    const float2 f0 = poly6(t, 0.00014476f, -0.00072805f, 0.00137237f, -0.00009512f, -0.00552740f, -0.00000077f,
                            0.79788456f);
    const float2 p0 = __fmul2_rn(t, poly5(t, 0.00013558f, -0.00029333f, -0.00054125f, 0.00262573f, -0.00003954f,
                                          -0.04166397f));
    float2 s0, c0;
    sincos_small2(p0, s0, c0);
    J0 = __fmul2_rn(__fmul2_rn(f0, sq), __fmul2_rn(b2(0.707106781f), __ffma2_rn(c0, a, __fmul2_rn(s0, b))));
    if (WANT_J1) {
        const float2 f1 = poly6(t, -0.00020033f, 0.00113653f, -0.00249511f, 0.00017105f, 0.01659667f, 0.00000156f,
                                0.79788456f);
        const float2 p1 = __fmul2_rn(t, poly5(t, -0.00029166f, 0.00079824f, 0.00074348f, -0.00637879f, 0.00005650f,
                                              0.12499612f));
        float2 s1, c1;
        sincos_small2(p1, s1, c1);
        const float2 cb = __fmul2_rn(c1, b);
        J1 = __fmul2_rn(__fmul2_rn(f1, sq), __fmul2_rn(b2(0.707106781f), __ffma2_rn(s1, a, make_float2(-cb.x, -cb.y))));
    }
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// add a partial sum into a float-float accumulator (hi, lo)
__device__ __forceinline__ void ff_acc(float& hi, float& lo, float part)
{
    float s, e;
    two_sum(hi, part, s, e);
    hi = s;
    lo += e;
}

// pre-factor of plane kz, frequency o, radius r: per (plane, frequency) or, for a radially
// modulated medium, per (plane, frequency, radius); NULL means 1
__device__ __forceinline__ double2 pre_at(const mma_hankel_problem& P, const double2* pre, int64_t kz, int64_t o,
                                          int64_t r)
{
    if (!pre) return make_double2(1.0, 0.0);
    return P.pre_radial ? pre[(kz * P.n_omega + o) * P.n_r + r] : pre[kz * P.n_omega + o];
}

inline bool valid(const mma_hankel_problem* p)
{
    return p && p->n_omega > 0 && p->n_r > 1 && p->n_z > 0 && p->n_rho > 0 && p->distance == p->distance &&
           p->plane_stride >= 0 && p->omega_stride >= p->n_r;
}

}  // namespace hk
}  // namespace mma
