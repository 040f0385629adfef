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
// that value lies within 2^-14 of its remainder of a float rounding boundary
// (near_boundary), or E < q/2, the double expression itself decides
// (exact_pressure), so the result is the reference's float in every case.
MHD_HD float total_pressure(float e, float q, float b2)
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
    const float d = fadd(fsub(sh, r), t);   // the value's distance from r
    if (near_boundary<14>(r, d) || ah < 0.0f) return exact_pressure(e, q, b2);
    return r;
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
//    the approximate reciprocal: error below 2^-18 half-ulps of the result.
//    The reference's RN_f(RN_d(XY/S)) equals RN_f(XY/S) (XY/S is a multiple of
//    2^-49 of itself away from every float midpoint or on one), so where the
//    corrected quotient lies near a boundary (near_boundary, a window of 2^-14
//    of its remainder, i.e. of 2^-14 half-ulps where it matters) the double
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
    // (branch-free: where XY <= 0 the quotient is formed and discarded)
    MHD_HD static float slope(float X, float Y)
    {
        const float ph = fmul(X, Y);
        const float pl = ffma(X, Y, -ph);
        const float s = fadd(X, Y);
        const float y = rcp_approx(s);
        const float q0 = fmul(ph, y);
        const float e = fadd(ffma(-q0, s, ph), pl);
        float q = ffma(e, y, q0);
        const float d = ffma(e, y, fsub(q0, q));   // q0 + e y - q (q0 - q is exact)
        if (near_boundary<14>(q, d) && ph > 0.0f) q = exact_quotient(ph, pl, s);
        return (ph > 0.0f) ? q : 0.0f;
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
    // residual, summed with x by Fast2Sum (error below 2^-16 half-ulps of the
    // result); near a rounding boundary (a window of 2^-12 of the remainder)
    // the double expression decides (exact_speed).
    MHD_HD static float speed(float x, float a)
    {
        if (!(a > 0.0f)) return x;
        const float r = rsqrt_approx(a);
        const float zh = fmul(a, r);
        const float zl = fmul(ffma(-zh, zh, a), 0.5f * r);
        const float hi = fmaxf(x, zh), lo = fminf(x, zh);
        const float sh = fadd(hi, lo);
        const float sl = fsub(lo, fsub(sh, hi));          // Fast2Sum, |hi| >= |lo|
        const float t = fadd(sl, zl);
        const float res = fadd(sh, t);
        const float d = fadd(fsub(sh, res), t);
        if (near_boundary<12>(res, d)) return exact_speed(x, a);
        return res;
    }
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
template <class M>
MHD_HD void cell_flux(const float u[5], const float bc[3], float v[5], float &cs, float &p)
{
    const float r = u[0], m1 = u[1], m2 = u[2], m3 = u[3], e = u[4];
    const float bx = bc[0], by = bc[1], bz = bc[2];
    const float yr = M::recip(r);
    const float vx = M::divy(m1, r, yr);
    const float b2 = M::add(M::add(M::mul(bx, bx), M::mul(by, by)), M::mul(bz, bz));
    const float s2 = M::add(M::add(M::mul(m1, m1), M::mul(m2, m2)), M::mul(m3, m3));
    float ps, pg;
    M::recover(u, bc, yr, s2, b2, ps, pg);
    v[0] = m1;
    v[1] = M::sub(M::add(M::mul(m1, vx), ps), M::mul(bx, bx));
    v[2] = M::sub(M::mul(m2, vx), M::mul(by, bx));
    v[3] = M::sub(M::mul(m3, vx), M::mul(bz, bx));
    const float dot = M::add(M::add(M::mul(bx, m1), M::mul(by, m2)), M::mul(bz, m3));
    v[4] = M::sub(M::mul(M::add(e, ps), vx), M::divy(M::mul(bx, dot), r, yr));
    p = pg;
    const float a = M::divy(M::add(b2, M::mul(kGamma, p)), r, yr);
    cs = M::speed(fabsf(vx), fabsf(a));
}

// Fast speed of one cell for the CFL condition, C-path formula with the
// cell's own (unaveraged) face B (Heterogeneous_MHD/C/calcfl.c:39-54):
//   c = max|m/rho| + sqrt(|2 B2 + gamma p| / rho), the root argument and the
// final sum formed in double there; here in float-float.
MHD_HD float cfl_speed_c(const float u[5], const float b[3])
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
    const float ps = total_pressure(e, qdiv(s2), b2);
    const float p = fsub(ps, 0.5f * b2);
    const float gp = fmul(kGamma, p);
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
    const float d = fadd(fsub(sh, res), t);
    // near a rounding boundary (2^-10 of the remainder) the double expression decides
    if (near_boundary<10>(res, d)) return exact_cfl_speed(v, b2, gp, r);
    return res;
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
