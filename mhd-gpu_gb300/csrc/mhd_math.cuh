// mhd_math.cuh - per-cell arithmetic of the relaxing TVD MHD step in FP32.
//
// Every operation is written with an explicit rounding so that nvcc does not
// contract a multiply and an add into one FMA where the reference C path
// (Heterogeneous_MHD/C/*.c) rounds them separately.  Where the reference
// evaluates a sub-expression in double because of a `2.0`-style literal and
// then rounds it to float once, the code below reproduces that single rounding
// in FP32 with error-free transformations (TwoSum / TwoProduct, Knuth and
// Dekker) instead of paying for FP64, whose rate on GB300 is a small fraction
// of FP32.  The functions are __host__ __device__ so that the same formulas can
// be exercised on the CPU.
#pragma once

#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define MHD_HD __host__ __device__ __forceinline__
#else
#define MHD_HD inline
#endif

namespace mhd {

constexpr float kGamma = 1.66666662693023681640625f;     // (float)(5.0/3.0)
constexpr float kGammaM1 = 0.66666662693023681640625f;   // gamma - 1, exact in float
constexpr float kTwoMGammaHalf = 0.166666686534881591796875f;  // (2 - gamma)/2, exact

#if defined(__CUDA_ARCH__)
MHD_HD float fmul(float a, float b) { return __fmul_rn(a, b); }
MHD_HD float fadd(float a, float b) { return __fadd_rn(a, b); }
MHD_HD float fsub(float a, float b) { return __fsub_rn(a, b); }
MHD_HD float fdiv(float a, float b) { return __fdiv_rn(a, b); }
MHD_HD float fsqrt(float a) { return __fsqrt_rn(a); }
MHD_HD float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
MHD_HD float fdiv_approx(float a, float b) { return __fdividef(a, b); }
#else
MHD_HD float fmul(float a, float b) { volatile float r = a * b; return r; }
MHD_HD float fadd(float a, float b) { volatile float r = a + b; return r; }
MHD_HD float fsub(float a, float b) { volatile float r = a - b; return r; }
MHD_HD float fdiv(float a, float b) { volatile float r = a / b; return r; }
MHD_HD float fsqrt(float a) { return sqrtf(a); }
MHD_HD float ffma(float a, float b, float c) { return fmaf(a, b, c); }
MHD_HD float fdiv_approx(float a, float b) { return a / b; }
#endif

// s + e == a + b exactly (TwoSum, Knuth).
MHD_HD void two_sum(float a, float b, float &s, float &e)
{
    s = fadd(a, b);
    float bb = fsub(s, a);
    float aa = fsub(s, bb);
    e = fadd(fsub(a, aa), fsub(b, bb));
}

// p + e == a * b exactly (TwoProduct via FMA).
MHD_HD void two_prod(float a, float b, float &p, float &e)
{
    p = fmul(a, b);
    e = ffma(a, b, -p);
}

MHD_HD unsigned f2u(float x)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    unsigned u;
    memcpy(&u, &x, sizeof u);
    return u;
#endif
}
MHD_HD float u2f(unsigned u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float x;
    memcpy(&x, &u, sizeof x);
    return x;
#endif
}

// Whether a float-float value v = r + d (r = RN(v), d the small remainder)
// lies within 2^-K |d| of a float rounding boundary: v nudged by +-2^-K of
// its remainder rounds to two different floats.  Where it does not, every
// value within that distance of v -- the exact value included, when the
// float-float error is below it -- rounds to r.  Pure FP32: two FMAs and a
// compare, and a power-of-two r (whose lower rounding interval is half as
// wide) needs no special case.
template <int K>
MHD_HD bool near_boundary(float r, float d)
{
    const float up = 1.0f + 1.0f / (float)(1 << K), dn = 1.0f - 1.0f / (float)(1 << K);
    return ffma(d, up, r) != ffma(d, dn, r);
}

// Windows of the near-boundary tests, as powers of two of the remainder d
// (near a boundary |d| is half an ulp of the result), each about 4-6 times
// the helper's error bound: total pressure within 2^-46 of ps (2^-21
// half-ulps), the van Leer quotient's d within 2^-21.2 of itself, the fast
// speed within 2^-44.2 of the root (2^-19.2 half-ulps), the CFL speed within
// 2^-19.5 half-ulps.  The largest errors measured on GB300 over 2 x 10^9
// random operands per helper (realistic ranges, and random mantissas over
// wide exponent ranges) stay below these: 2^-21.8, 2^-20.0 (with the
// quotient's earlier remainder, q0 + e y - q), 2^-19.8 and 2^-20.7.
// Outside the window the float-float value and the C path's double round to
// the same float.
constexpr int kKPressure = 19;
constexpr int kKSlope = 19;
constexpr int kKSpeed = 17;
constexpr int kKCfl = 17;

// Double arithmetic with one rounding per operation: the fallbacks below
// must not be contracted into FMAs (a*b + c fused rounds once where the C
// path rounds the product and the sum separately; on a double tie the float
// result then differs).
#if defined(__CUDA_ARCH__)
MHD_HD double dmul(double a, double b) { return __dmul_rn(a, b); }
MHD_HD double dadd(double a, double b) { return __dadd_rn(a, b); }
MHD_HD double dsub(double a, double b) { return __dsub_rn(a, b); }
MHD_HD double ddiv(double a, double b) { return __ddiv_rn(a, b); }
MHD_HD double dsqrt(double a) { return __dsqrt_rn(a); }
#else
MHD_HD double dmul(double a, double b) { volatile double r = a * b; return r; }
MHD_HD double dadd(double a, double b) { volatile double r = a + b; return r; }
MHD_HD double dsub(double a, double b) { volatile double r = a - b; return r; }
MHD_HD double ddiv(double a, double b) { volatile double r = a / b; return r; }
MHD_HD double dsqrt(double a) { return sqrt(a); }
#endif

// The reference's double expressions, evaluated in FP64 for the rare
// operands whose float-float value lies too close to a rounding boundary to
// decide the float result: exactly what the C path computes, operation by
// operation.
MHD_HD
#if defined(__CUDA_ARCH__)
__noinline__
#endif
float exact_pressure(float e, float q, float b2)
{
    // ((E - q/2.0)*(gamma - 1.0) + (2.0 - gamma)*B2/2.0), mhdflux.c:28
    const double a = dsub((double)e, ddiv((double)q, 2.0));
    const double m = ddiv(dmul(dsub(2.0, (double)kGamma), (double)b2), 2.0);
    return (float)dadd(dmul(a, dsub((double)kGamma, 1.0)), m);
}
MHD_HD
#if defined(__CUDA_ARCH__)
__noinline__
#endif
float exact_quotient(float ph, float pl, float s)
{
    return (float)ddiv(dadd((double)ph, (double)pl), (double)s);
}
MHD_HD
#if defined(__CUDA_ARCH__)
__noinline__
#endif
float exact_speed(float x, float a)
{
    return (float)dadd((double)x, dsqrt((double)a));
}
MHD_HD
#if defined(__CUDA_ARCH__)
__noinline__
#endif
float exact_cfl_speed(float v, float b2, float gp, float r)
{
    // v + sqrt(fabs(B2*2.0 + gamma p) / rho), calcfl.c:54 (fabs of the numerator only)
    return (float)dadd((double)v, dsqrt(ddiv(fabs(dadd(dmul((double)b2, 2.0), (double)gp)), (double)r)));
}

// Total pressure of one cell,
//   ps = (E - |m|^2/rho/2)(gamma-1) + (2-gamma)|B|^2/2,
// with q = |m|^2/rho and B2 = |B|^2 already rounded to float.  The reference
// forms the whole expression in double (Heterogeneous_MHD/C/mhdflux.c:28,
// calcfl.c:50) and rounds once to float.  Here it is formed in float-float
// (error below 2^-46 of ps when E >= q/2, as in any physical cell); where
// that value lies within 2^-19 of its remainder of a float rounding boundary
// (near_boundary), or E < q/2, the double expression itself decides
// (exact_pressure), so the result is the reference's float in every case.
// The float-float value, and nb set where it lies near a rounding boundary
// (or E < q/2): the caller then takes exact_pressure.
// the float-float value r + d (r rounded, d its remainder); neg when E < q/2
MHD_HD float total_pressure_rd(float e, float q, float b2, float &d, bool &neg)
{
    float ah, al;
    two_sum(e, -0.5f * q, ah, al);          // E - q/2 exactly
    float ph, pl;
    two_prod(ah, kGammaM1, ph, pl);
    pl = ffma(al, kGammaM1, pl);
    float mh, ml;
    two_prod(b2, kTwoMGammaHalf, mh, ml);
    float sh, sl;
    two_sum(ph, mh, sh, sl);
    const float t = fadd(sl, fadd(pl, ml));
    const float r = fadd(sh, t);
    d = fadd(fsub(sh, r), t);   // the value's distance from r
    neg = ah < 0.0f;
    return r;
}
MHD_HD float total_pressure_ff(float e, float q, float b2, bool &nb)
{
    float d;
    bool neg;
    const float r = total_pressure_rd(e, q, b2, d, neg);
    nb |= near_boundary<kKPressure>(r, d) || neg;
    return r;
}
MHD_HD float total_pressure(float e, float q, float b2)
{
    bool nb = false;
    const float r = total_pressure_ff(e, q, b2, nb);
    return nb ? exact_pressure(e, q, b2) : r;
}

// ---------------------------------------------------------------------------
// Approximate hardware reciprocal and reciprocal square root (MUFU).  They
// only ever seed a correction step below, never produce a result on their own
// in the faithful policy.
// ---------------------------------------------------------------------------
#if defined(__CUDA_ARCH__)
MHD_HD float rcp_approx(float d)
{
    float y;
    asm("rcp.approx.f32 %0, %1;" : "=f"(y) : "f"(d));
    return y;
}
MHD_HD float rsqrt_approx(float a)
{
    float y;
    asm("rsqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(a));
    return y;
}
MHD_HD float rcp_rn(float d) { return __frcp_rn(d); }
#else
MHD_HD float rcp_approx(float d) { return 1.0f / d; }
MHD_HD float rsqrt_approx(float a) { return 1.0f / sqrtf(a); }
MHD_HD float rcp_rn(float d) { volatile float r = 1.0f / d; return r; }
#endif

// Faithful policy: the rounding of the reference C path.
//  - mul/add/sub round separately (no contraction);
//  - a quotient a/d whose divisor is shared (1/rho of a cell, 1/c of a pencil)
//    uses y = RN(1/d) once and Markstein's correction q = RN(q0 + (a - d q0) y),
//    q0 = RN(a y) (P. Markstein, IBM J. Res. Dev. 34(1), 1990), which equals
//    the IEEE quotient RN(a/d) for normal operands;
//  - slope(X, Y) is the van Leer limiter 2ab/(a+b) of a = X/2, b = Y/2, i.e.
//    XY/(X+Y), with the exact product XY as the reference's double numerator
//    (Heterogeneous_MHD/C/tvd1.c:78, tvdb.c:75) and one correction step from
//    the approximate reciprocal (error below 2^-19 half-ulps of the result);
//    its remainder comes from its own residual, within 2^-21.2 of itself.
//    The reference's RN_f(RN_d(XY/S)) equals RN_f(XY/S) (XY/S is a multiple of
//    2^-49 of itself away from every float midpoint or on one), so where the
//    corrected quotient lies near a boundary (near_boundary, a window of 2^-19
//    of its remainder, i.e. of 2^-19 half-ulps where it matters) the double
//    quotient decides (exact_quotient) and the result is the reference's.
struct Faithful {
    MHD_HD static float mul(float a, float b) { return fmul(a, b); }
    MHD_HD static float add(float a, float b) { return fadd(a, b); }
    MHD_HD static float sub(float a, float b) { return fsub(a, b); }
    MHD_HD static float recip(float d) { return rcp_rn(d); }
    MHD_HD static float divy(float a, float d, float y)
    {
        const float q = fmul(a, y);
        const float e = ffma(-q, d, a);
        return ffma(e, y, q);
    }
    MHD_HD static float div(float a, float d) { return fdiv(a, d); }
    // RN(2 v + s) formed once (the reference's double (s + 2.0*v)/4.0)
    MHD_HD static float twice_plus(float v, float s) { return ffma(2.0f, v, s); }
    // RN(b - p/2) formed once (the reference's double b - p/2.0)
    MHD_HD static float minus_half(float b, float p) { return ffma(-0.5f, p, b); }
    // (branch-free: where XY <= 0 the quotient is formed and discarded);
    // slope_ff is the float-float value with nb set near a boundary
    // the corrected quotient q and its remainder d; ph = RN(XY)
    MHD_HD static float slope_rd(float X, float Y, float &d, float &ph)
    {
        ph = fmul(X, Y);
        const float pl = ffma(X, Y, -ph);
        const float s = fadd(X, Y);
        const float y = rcp_approx(s);
        const float q0 = fmul(ph, y);
        const float e = fadd(ffma(-q0, s, ph), pl);
        const float q = ffma(e, y, q0);
        // the remainder (XY - q s)/s of q from its own residual: ph - q s is
        // exact, or rounded once (q lies within 1.5 ulps of ph/s), and near a
        // boundary it is at most 3 times the residual, so the roundings of
        // the FMA, the sum, y and the product leave d within 7 * 2^-24 of
        // itself (2^-21.2)
        d = fmul(fadd(ffma(-q, s, ph), pl), y);
        return q;
    }
    MHD_HD static float slope_ff(float X, float Y, bool &nb)
    {
        float d, ph;
        const float q = slope_rd(X, Y, d, ph);
        nb |= near_boundary<kKSlope>(q, d) && ph > 0.0f;
        return (ph > 0.0f) ? q : 0.0f;
    }
    MHD_HD static float slope(float X, float Y)
    {
        bool nb = false;
        const float q = slope_ff(X, Y, nb);
        if (!nb) return q;
        const float ph = fmul(X, Y);
        return exact_quotient(ph, ffma(X, Y, -ph), fadd(X, Y));
    }
    MHD_HD static float pressure(float e, float q, float b2) { return total_pressure(e, q, b2); }
    // total pressure ps (mhdflux.c:26-29) and gas pressure p = ps - B^2/2
    // (mhdflux.c:39-42) of a cell; s2 = |m|^2, b2 = |B|^2, yr = RN(1/rho)
    MHD_HD static void recover(const float u[5], const float bc[3], float yr, float s2, float b2,
                               float &ps, float &p)
    {
        (void)bc;
        ps = pressure(u[4], divy(s2, u[0], yr), b2);
        p = fsub(ps, 0.5f * b2);
    }
    // RN(x + sqrt(a)) as the reference forms it (the root and the sum in
    // double, Heterogeneous_MHD/C/mhdflux.c:45): the root in float-float, zh
    // ~ sqrt(a) from the hardware rsqrt, zl = (a - zh^2)/(2 zh) with the FMA
    // residual, summed with x by Fast2Sum (error below 2^-19 half-ulps of the
    // result); near a rounding boundary (a window of 2^-17 of the remainder)
    // the double expression decides (exact_speed).
    // e0 = a - zh^2 (exact): 0 when zh is the root itself, and then r + d is
    // x + sqrt(a) exactly, so r is its correctly rounded value even on a tie
    MHD_HD static float speed_rd(float x, float a, float &d, float &e0)
    {
        d = 0.0f;
        e0 = 0.0f;
        if (!(a > 0.0f)) return x;
        const float r = rsqrt_approx(a);
        const float zh = fmul(a, r);
        e0 = ffma(-zh, zh, a);
        const float zl = fmul(e0, 0.5f * r);
        const float hi = fmaxf(x, zh), lo = fminf(x, zh);
        const float sh = fadd(hi, lo);
        const float sl = fsub(lo, fsub(sh, hi));          // Fast2Sum, |hi| >= |lo|
        const float t = fadd(sl, zl);
        const float res = fadd(sh, t);
        d = fadd(fsub(sh, res), t);
        return res;
    }
    MHD_HD static float speed_ff(float x, float a, bool &nb)
    {
        float d, e0;
        const float res = speed_rd(x, a, d, e0);
        nb |= near_boundary<kKSpeed>(res, d) && e0 != 0.0f;
        return res;
    }
    MHD_HD static float speed(float x, float a)
    {
        bool nb = false;
        const float res = speed_ff(x, a, nb);
        return nb ? exact_speed(x, a) : res;
    }
    static constexpr bool kFlagged = false;
};

// The faithful policy's float-float values without their FP64 fallbacks: an
// instance ORs into nb whether any value it formed lies near a float rounding
// boundary.  A tile computed with it is kept only where no lane of its CTA
// saw one; otherwise it is computed again with Faithful (identical wherever
// nb stays false, so the bits are Faithful's in every case).  The fallbacks'
// calls out of the hot code cost registers (the call convention) that the
// tiles otherwise spend on their state.
struct FaithfulNB : Faithful {
    bool nb = false;
    MHD_HD float slope(float X, float Y) { return slope_ff(X, Y, nb); }
    MHD_HD float pressure(float e, float q, float b2) { return total_pressure_ff(e, q, b2, nb); }
    MHD_HD void recover(const float u[5], const float bc[3], float yr, float s2, float b2, float &ps, float &p)
    {
        (void)bc;
        ps = pressure(u[4], divy(s2, u[0], yr), b2);
        p = fsub(ps, 0.5f * b2);
    }
    MHD_HD float speed(float x, float a) { return speed_ff(x, a, nb); }
    static constexpr bool kFlagged = true;
};

// Fast policy: plain FP32 with FMA contraction allowed, hardware reciprocal
// and root.  Measured against the oracle like the faithful policy.
struct Fast {
    MHD_HD static float mul(float a, float b) { return a * b; }
    MHD_HD static float add(float a, float b) { return a + b; }
    MHD_HD static float sub(float a, float b) { return a - b; }
    MHD_HD static float recip(float d) { return rcp_approx(d); }
    MHD_HD static float divy(float a, float d, float y) { (void)d; return a * y; }
    MHD_HD static float div(float a, float d) { return a * rcp_approx(d); }
    MHD_HD static float twice_plus(float v, float s) { return 2.0f * v + s; }
    MHD_HD static float minus_half(float b, float p) { return b - 0.5f * p; }
    MHD_HD static float slope(float X, float Y)
    {
        const float p = X * Y;
        return (p > 0.0f) ? p * rcp_approx(X + Y) : 0.0f;
    }
    MHD_HD static float pressure(float e, float q, float b2)
    {
        return (e - 0.5f * q) * kGammaM1 + b2 * kTwoMGammaHalf;
    }
    MHD_HD static void recover(const float u[5], const float bc[3], float yr, float s2, float b2,
                               float &ps, float &p)
    {
        (void)bc;
        ps = pressure(u[4], divy(s2, u[0], yr), b2);
        p = ps - 0.5f * b2;
    }
    MHD_HD static float speed(float x, float a) { return (a > 0.0f) ? x + a * rsqrt_approx(a) : x; }
    static constexpr bool kFlagged = false;
};

// Faithful arithmetic except for the pressure of low-beta cells, which is
// recovered in FP64: where the FP32 gas pressure gives beta = 2p/B^2 below
// kLowBeta (or p <= 0), p = (gamma-1)(E - |m|^2/(2 rho) - |B|^2/2) is formed
// in double from the cell's float state and ps = p + |B|^2/2, both rounded
// once to float.  At low beta the FP32 chain ps -> p = ps - B^2/2 cancels
// (ps ~ B^2/2 >> p); the double chain does not.  gamma is the solver's float
// constant.  Costs ~15 FP64 operations (one divide) per low-beta cell-flux.
constexpr float kLowBeta = 0.1f;
struct Recover64 : Faithful {
    MHD_HD static void recover(const float u[5], const float bc[3], float yr, float s2, float b2,
                               float &ps, float &p)
    {
        Faithful::recover(u, bc, yr, s2, b2, ps, p);
        if (p >= kLowBeta * 0.5f * b2) return;
        const double bx = bc[0], by = bc[1], bz = bc[2];
        const double m1 = u[1], m2 = u[2], m3 = u[3];
        const double b2d = bx * bx + by * by + bz * bz;
        const double qd = (m1 * m1 + m2 * m2 + m3 * m3) / (double)u[0];
        const double pd = ((double)kGamma - 1.0) * ((double)u[4] - 0.5 * qd - 0.5 * b2d);
        p = (float)pd;
        ps = (float)(pd + 0.5 * b2d);
    }
};

// Fluxes v (not yet divided by the pencil's c) and fast speed of one cell
// (Heterogeneous_MHD/C/mhdflux.c:9-59).  u = (rho, m1, m2, m3, E) of the
// frame, bc = cell-centred B of the frame.  Returns the gas pressure in p.
// (m: the policy, an instance so that FaithfulNB can carry its flag)
template <class M>
MHD_HD void cell_flux(M &m, const float u[5], const float bc[3], float v[5], float &cs, float &p)
{
    const float r = u[0], m1 = u[1], m2 = u[2], m3 = u[3], e = u[4];
    const float bx = bc[0], by = bc[1], bz = bc[2];
    const float yr = m.recip(r);
    const float vx = m.divy(m1, r, yr);
    const float b2 = m.add(m.add(m.mul(bx, bx), m.mul(by, by)), m.mul(bz, bz));
    const float s2 = m.add(m.add(m.mul(m1, m1), m.mul(m2, m2)), m.mul(m3, m3));
    float ps, pg;
    m.recover(u, bc, yr, s2, b2, ps, pg);
    v[0] = m1;
    v[1] = m.sub(m.add(m.mul(m1, vx), ps), m.mul(bx, bx));
    v[2] = m.sub(m.mul(m2, vx), m.mul(by, bx));
    v[3] = m.sub(m.mul(m3, vx), m.mul(bz, bx));
    const float dot = m.add(m.add(m.mul(bx, m1), m.mul(by, m2)), m.mul(bz, m3));
    v[4] = m.sub(m.mul(m.add(e, ps), vx), m.divy(m.mul(bx, dot), r, yr));
    p = pg;
    const float a = m.divy(m.add(b2, m.mul(kGamma, p)), r, yr);
    cs = m.speed(fabsf(vx), fabsf(a));
}
template <class M>
MHD_HD void cell_flux(const float u[5], const float bc[3], float v[5], float &cs, float &p)
{
    M m;
    cell_flux(m, u, bc, v, cs, p);
}

// Fast speed of one cell for the CFL condition, C-path formula with the
// cell's own (unaveraged) face B (Heterogeneous_MHD/C/calcfl.c:39-54):
//   c = max|m/rho| + sqrt(|2 B2 + gamma p| / rho), the root argument and the
// final sum formed in double there; here in float-float.
// v + sqrt(|2 B2 + gp| / rho) in float-float: the rounded value and its
// remainder d (mk: rho is a positive finite number, yr = RN(1/rho))
MHD_HD float cfl_tail_rd(float v, float b2, float gp, float r, bool mk, float yr, float &d)
{
    auto qdiv = [&](float x) { return mk ? Faithful::divy(x, r, yr) : fdiv(x, r); };
    // X = 2*B2 + gp exactly as a float pair, then |X| / r in float-float
    float xh, xl;
    two_sum(2.0f * b2, gp, xh, xl);
    if (xh < 0.0f) { xh = -xh; xl = -xl; }
    const float yh = qdiv(xh);
    const float rem = ffma(-yh, r, xh);                 // exact remainder
    const float yl = fdiv_approx(fadd(rem, xl), r);
    // sqrt(yh + yl) + v
    const float zh = fsqrt(yh);
    float zl = 0.0f;
    if (zh > 0.0f) zl = fdiv_approx(fadd(ffma(-zh, zh, yh), yl), 2.0f * zh);
    float sh, sl;
    two_sum(v, zh, sh, sl);
    const float t = fadd(sl, zl);
    const float res = fadd(sh, t);
    d = fadd(fsub(sh, res), t);
    return res;
}

// EXACT: the C path's value (FP64 fallbacks); else the float-float value with
// nb set where it, or the pressure under it, lies near a rounding boundary.
template <bool EXACT>
MHD_HD float cfl_speed_c_impl(const float u[5], const float b[3], bool &nb)
{
    const float r = u[0], m1 = u[1], m2 = u[2], m3 = u[3], e = u[4];
    // The five quotients by rho share one correctly rounded reciprocal with
    // Markstein's correction (Faithful::divy: the IEEE quotient for normal
    // operands, as in the fluxes); a density that is not a positive finite
    // number takes the IEEE divisions, so inf and NaN propagate as before.
    const bool mk = r > 0.0f && r <= 3.40282347e38f;
    const float yr = mk ? Faithful::recip(r) : 0.0f;
    auto qdiv = [&](float x) { return mk ? Faithful::divy(x, r, yr) : fdiv(x, r); };
    const float t1 = fabsf(qdiv(m1)), t2 = fabsf(qdiv(m2)), t3 = fabsf(qdiv(m3));
    float v;
    if (t1 > t2) v = (t1 > t3) ? t1 : t3; else v = (t2 > t3) ? t2 : t3;
    const float b2 = fadd(fadd(fmul(b[0], b[0]), fmul(b[1], b[1])), fmul(b[2], b[2]));
    const float s2 = fadd(fadd(fmul(m1, m1), fmul(m2, m2)), fmul(m3, m3));
    const float ps = EXACT ? total_pressure(e, qdiv(s2), b2) : total_pressure_ff(e, qdiv(s2), b2, nb);
    const float p = fsub(ps, 0.5f * b2);
    const float gp = fmul(kGamma, p);
    float d;
    const float res = cfl_tail_rd(v, b2, gp, r, mk, yr, d);
    // near a rounding boundary the double expression decides
    if (EXACT) {
        if (near_boundary<kKCfl>(res, d)) return exact_cfl_speed(v, b2, gp, r);
    } else {
        nb |= near_boundary<kKCfl>(res, d);
    }
    return res;
}
MHD_HD float cfl_speed_c(const float u[5], const float b[3])
{
    bool nb = false;
    return cfl_speed_c_impl<true>(u, b, nb);
}
MHD_HD float cfl_speed_c_ff(const float u[5], const float b[3], bool &nb)
{
    return cfl_speed_c_impl<false>(u, b, nb);
}

// Release 0.2 CFL fast speed with cell-centred B (OpenMP/mhd.f90:108-120),
// all in single precision as the Fortran source is.  bc = averaged B.
MHD_HD float cfl_speed_averaged(const float u[5], const float bc[3])
{
    const float r = u[0], m1 = u[1], m2 = u[2], m3 = u[3], e = u[4];
    const float a1 = fabsf(fdiv(m1, r)), a2 = fabsf(fdiv(m2, r)), a3 = fabsf(fdiv(m3, r));
    float v;
    if (a1 > a2) v = (a1 > a3) ? a1 : a3; else v = (a2 > a3) ? a2 : a3;
    const float b2 = fadd(fadd(fmul(bc[0], bc[0]), fmul(bc[1], bc[1])), fmul(bc[2], bc[2]));
    const float s2 = fadd(fadd(fmul(m1, m1), fmul(m2, m2)), fmul(m3, m3));
    const float ps = fadd(fmul(fsub(e, fdiv(fdiv(s2, r), 2.0f)), fsub(kGamma, 1.0f)),
                          fdiv(fmul(fsub(2.0f, kGamma), b2), 2.0f));
    const float p = fsub(ps, fdiv(b2, 2.0f));
    const float q = fdiv(fadd(fmul(b2, 2.0f), fmul(kGamma, p)), r);
    return fadd(v, fsqrt(fabsf(q)));
}

}  // namespace mhd
