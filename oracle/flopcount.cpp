/*
 * flopcount.cpp - TEST INFRASTRUCTURE ONLY: counts the floating-point
 * operations of one full step of the oracle (the CPU restatement of the
 * reference C path), per cell-update, by compiling mhd_oracle.c with its real
 * type replaced by a counting type.  Every +, -, *, / and sqrt of the
 * restatement counts one, as the reference writes them (constant
 * sub-expressions such as gamma - 1.0 included); fabs, comparisons, copies and
 * transposes count nothing.  The values computed are doubles (the count does
 * not depend on the precision).
 *
 *   make -C oracle flopcount && oracle/lib/flopcount 16 16 16
 *
 * prints the operations per cell-update of the fluid update, the field update,
 * the CFL reduction (C-path formula) and the total.
 */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

struct Counted {
    double v = 0.0;
    static uint64_t n;
    Counted() = default;
    Counted(double x) : v(x) {}
    explicit operator double() const { return v; }
    explicit operator float() const { return (float)v; }
    explicit operator int() const { return (int)v; }
};
uint64_t Counted::n = 0;

#define MHD_CNT_BIN(op)                                                                    \
    inline Counted operator op(Counted a, Counted b) { ++Counted::n; return Counted(a.v op b.v); } \
    inline Counted operator op(Counted a, double b) { ++Counted::n; return Counted(a.v op b); }    \
    inline Counted operator op(double a, Counted b) { ++Counted::n; return Counted(a op b.v); }
MHD_CNT_BIN(+)
MHD_CNT_BIN(-)
MHD_CNT_BIN(*)
MHD_CNT_BIN(/)
#undef MHD_CNT_BIN
inline Counted operator-(Counted a) { return Counted(-a.v); }
#define MHD_CNT_CMP(op)                                                    \
    inline bool operator op(Counted a, Counted b) { return a.v op b.v; }  \
    inline bool operator op(Counted a, double b) { return a.v op b; }     \
    inline bool operator op(double a, Counted b) { return a op b.v; }
MHD_CNT_CMP(<)
MHD_CNT_CMP(>)
MHD_CNT_CMP(<=)
MHD_CNT_CMP(>=)
MHD_CNT_CMP(==)
MHD_CNT_CMP(!=)
#undef MHD_CNT_CMP
inline Counted fabs(Counted a) { return Counted(std::fabs(a.v)); }
inline Counted sqrt(Counted a) { ++Counted::n; return Counted(std::sqrt(a.v)); }

#define ORACLE_REAL Counted
#define ORACLE_F32
#undef _OPENMP
#include "mhd_oracle.c"

int main(int argc, char **argv)
{
    const int nx = argc > 1 ? atoi(argv[1]) : 16, ny = argc > 2 ? atoi(argv[2]) : nx,
              nz = argc > 3 ? atoi(argv[3]) : nx;
    const size_t nc = (size_t)nx * ny * nz;
    Counted *u = new Counted[5 * nc], *b = new Counted[3 * nc], *wu = new Counted[5 * nc], *wb = new Counted[3 * nc];
    for (size_t c = 0; c < nc; ++c) {   // a smooth physical state with flow and field
        const double s = 1e-3 * std::sin(0.1 * (double)c);
        u[5 * c + 0] = 1.0 + s;
        u[5 * c + 1] = 0.1 + s;
        u[5 * c + 2] = -0.05 + s;
        u[5 * c + 3] = 0.02;
        u[5 * c + 4] = 2.0;
        b[3 * c + 0] = 1.0 + s;
        b[3 * c + 1] = 0.2;
        b[3 * c + 2] = -0.1 + s;
    }
    const double per = 1.0 / (double)nc;
    Counted dt = 0.01;
    Counted::n = 0;
    PFX(fluidx)(u, b, (int *)&nx, (int *)&ny, (int *)&nz, &dt, u, b, 0);
    const double fl = (double)Counted::n * per;
    Counted::n = 0;
    PFX(advectbyzx)(u, b, (int *)&nx, (int *)&ny, (int *)&nz, &dt, wu, wb);
    const double ad = (double)Counted::n * per;
    Counted::n = 0;
    (void)PFX(calcfl)(u, b, (int *)&nx, (int *)&ny, (int *)&nz);
    const double cf = (double)Counted::n * per;
    // a full step: 6 fluid sweeps, 6 field sweeps, one CFL reduction
    printf("per cell-sweep: fluidx %.1f advectbyzx %.1f; per step: cfl %.1f\n", fl, ad, cf);
    printf("flops per cell-update: %.1f\n", 6.0 * (fl + ad) + cf);
    delete[] u; delete[] b; delete[] wu; delete[] wb;
    return 0;
}
