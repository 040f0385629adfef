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

// Total pressure of one cell,
//   ps = (E - |m|^2/rho/2)(gamma-1) + (2-gamma)|B|^2/2,
// with q = |m|^2/rho and B2 = |B|^2 already rounded to float.  The reference
// forms the whole expression in double (Heterogeneous_MHD/C/mhdflux.c:18,
// calcfl.c:50) and rounds once; this forms it in float-float.
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
    return fadd(sh, fadd(sl, fadd(pl, ml)));
}

// round_to_float(x + sqrt(a)) with the sum and the root formed in double
// (the reference calls the double libm sqrt and adds in double,
// Heterogeneous_MHD/C/mhdflux.c:45, calcfl.c:54).  a >= 0, x >= 0.
MHD_HD float add_sqrt(float x, float a)
{
    float zh = fsqrt(a);
    float zl = 0.0f;
    if (zh > 0.0f) zl = fdiv_approx(ffma(-zh, zh, a), 2.0f * zh);
    float sh, sl;
    two_sum(x, zh, sh, sl);
    return fadd(sh, fadd(sl, zl));
}

// Fluxes v (already divided by nothing) and fast speed of one cell
// (Heterogeneous_MHD/C/mhdflux.c:9-59).  u = (rho, m1, m2, m3, E) of the
// frame, bc = cell-centred B of the frame.  Returns the gas pressure in p.
MHD_HD void cell_flux(const float u[5], const float bc[3], float v[5], float &cs, float &p)
{
    const float r = u[0], m1 = u[1], m2 = u[2], m3 = u[3], e = u[4];
    const float bx = bc[0], by = bc[1], bz = bc[2];
    const float vx = fdiv(m1, r);
    const float b2 = fadd(fadd(fmul(bx, bx), fmul(by, by)), fmul(bz, bz));
    const float s2 = fadd(fadd(fmul(m1, m1), fmul(m2, m2)), fmul(m3, m3));
    const float ps = total_pressure(e, fdiv(s2, r), b2);
    v[0] = m1;
    v[1] = fsub(fadd(fmul(m1, vx), ps), fmul(bx, bx));
    v[2] = fsub(fmul(m2, vx), fmul(by, bx));
    v[3] = fsub(fmul(m3, vx), fmul(bz, bx));
    const float dot = fadd(fadd(fmul(bx, m1), fmul(by, m2)), fmul(bz, m3));
    v[4] = fsub(fmul(fadd(e, ps), vx), fdiv(fmul(bx, dot), r));
    p = fsub(ps, 0.5f * b2);                               // mhdflux.c:39-42, one rounding
    const float a = fdiv(fadd(b2, fmul(kGamma, p)), r);
    cs = add_sqrt(fabsf(vx), fabsf(a));
}

// van Leer slope of two one-sided differences: 2ab/(a+b) if ab > 0 else 0
// (Heterogeneous_MHD/C/tvd1.c:71-81).
MHD_HD float van_leer(float a, float b)
{
    const float ab = fmul(a, b);
    return (ab > 0.0f) ? fdiv(2.0f * ab, fadd(a, b)) : 0.0f;
}

// Fast speed of one cell for the CFL condition, C-path formula with the
// cell's own (unaveraged) face B (Heterogeneous_MHD/C/calcfl.c:39-54):
//   c = max|m/rho| + sqrt(|2 B2 + gamma p| / rho), the root argument and the
// final sum formed in double there; here in float-float.
MHD_HD float cfl_speed_c(const float u[5], const float b[3])
{
    const float r = u[0], m1 = u[1], m2 = u[2], m3 = u[3], e = u[4];
    const float t1 = fabsf(fdiv(m1, r)), t2 = fabsf(fdiv(m2, r)), t3 = fabsf(fdiv(m3, r));
    float v;
    if (t1 > t2) v = (t1 > t3) ? t1 : t3; else v = (t2 > t3) ? t2 : t3;
    const float b2 = fadd(fadd(fmul(b[0], b[0]), fmul(b[1], b[1])), fmul(b[2], b[2]));
    const float s2 = fadd(fadd(fmul(m1, m1), fmul(m2, m2)), fmul(m3, m3));
    const float ps = total_pressure(e, fdiv(s2, r), b2);
    const float p = fsub(ps, 0.5f * b2);
    const float gp = fmul(kGamma, p);
    // X = 2*B2 + gp exactly as a float pair, then |X| / r in float-float
    float xh, xl;
    two_sum(2.0f * b2, gp, xh, xl);
    if (xh < 0.0f) { xh = -xh; xl = -xl; }
    const float yh = fdiv(xh, r);
    const float rem = ffma(-yh, r, xh);                 // exact remainder
    const float yl = fdiv_approx(fadd(rem, xl), r);
    // sqrt(yh + yl) + v
    const float zh = fsqrt(yh);
    float zl = 0.0f;
    if (zh > 0.0f) zl = fdiv_approx(fadd(ffma(-zh, zh, yh), yl), 2.0f * zh);
    float sh, sl;
    two_sum(v, zh, sh, sl);
    return fadd(sh, fadd(sl, zl));
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
