/*
 * mhd_oracle.c - CPU restatement of the reference C path of Pen's relaxing
 * TVD MHD step.  TEST INFRASTRUCTURE ONLY: it is the checker of the CUDA
 * kernels, never the thing measured or shipped.
 *
 * Compiled twice by oracle/Makefile:
 *   -DORACLE_REAL=float  -DORACLE_F32   -> oracle_*   (bit-exact vs reference)
 *   -DORACLE_REAL=double                -> oracle64_* (FP64 solver)
 * Always with -ffp-contract=off so that x86-64 and aarch64 builds give the
 * same bits: the reference's own makefile passes no flags, and without FMA
 * contraction every '*' and '+' below rounds separately, as in the reference.
 *
 * Every literal keeps the type it has in the reference (2.0 and /2.0 are
 * double, so with real=float those sub-expressions are evaluated in double
 * and rounded once on assignment, exactly as C promotion does there).
 *
 * Citations are paths inside pandaPQY/MHD-GPU.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef ORACLE_REAL
#define ORACLE_REAL float
#endif
typedef ORACLE_REAL real;

#ifdef ORACLE_F32
#define PFX(name) oracle_##name
#else
#define PFX(name) oracle64_##name
#endif

/* pencil-local AoS accessors: matrix2D(nub,n,ii,i) = i*nub+ii */
#define PU(p, ii, i) ((p)[(size_t)(i) * 5 + (ii)])
#define PB(p, ii, i) ((p)[(size_t)(i) * 3 + (ii)])

/* grid accessors: matrix4D(nub,nx,ny,nz,ii,i,j,k) = ((k*ny+j)*nx+i)*nub+ii */
static inline size_t cidx(int nx, int ny, int i, int j, int k)
{
    return ((size_t)k * (size_t)ny + (size_t)j) * (size_t)nx + (size_t)i;
}
#define GU(a, ii, c) ((a)[(c) * 5 + (ii)])
#define GB(a, ii, c) ((a)[(c) * 3 + (ii)])

/* a*x + b*y + c with the rounding of abXYc_matrix2D/1D
 * (Heterogeneous_MHD/C/includefunc_spu.h:91-113). */
static inline real abxyc(real a, real x, real b, real y, real c)
{
    return a * x + b * y + c;
}

static inline int wrap_up(int i, int n) { return (i + 1) % n; }
static inline int wrap_dn(int i, int n) { return (i + n - 1) % n; }

/* ------------------------------------------------------------------------ */
/* per-thread pencil workspace                                               */
/* ------------------------------------------------------------------------ */
typedef struct {
    int cap;
    real *su, *bc, *bjp, *bkp, *t1;           /* fluidx gather */
    real *v, *u1, *wr, *wl, *fr, *fl, *flux;  /* tvd1, 5n each */
    real *dfr, *dfl, *tmp1, *tmp2;
    real *vx, *ps, *pp, *tc;                  /* mhdflux, n each */
    real *avx, *at1, *at2, *ab, *aflux;       /* advect, n each */
    real *vh, *f1, *b1, *tb1, *tb2;           /* tvdb, n each */
} pencil_ws;

static void ws_init(pencil_ws *w, int n)
{
    size_t n5 = (size_t)5 * n, n3 = (size_t)3 * n, n1 = (size_t)n;
    size_t total = n5 * 13 + n3 * 3 + n1 * 15;
    real *m = (real *)calloc(total, sizeof(real));
    w->cap = n;
    w->su = m;     m += n5;
    w->bc = m;     m += n3;
    w->bjp = m;    m += n3;
    w->bkp = m;    m += n3;
    w->t1 = m;     m += n1;
    w->v = m;      m += n5;
    w->u1 = m;     m += n5;
    w->wr = m;     m += n5;
    w->wl = m;     m += n5;
    w->fr = m;     m += n5;
    w->fl = m;     m += n5;
    w->flux = m;   m += n5;
    w->dfr = m;    m += n5;
    w->dfl = m;    m += n5;
    w->tmp1 = m;   m += n5;
    w->tmp2 = m;   m += n5;
    m += n5; /* spare */
    w->vx = m;     m += n1;
    w->ps = m;     m += n1;
    w->pp = m;     m += n1;
    w->tc = m;     m += n1;
    w->avx = m;    m += n1;
    w->at1 = m;    m += n1;
    w->at2 = m;    m += n1;
    w->ab = m;     m += n1;
    w->aflux = m;  m += n1;
    w->vh = m;     m += n1;
    w->f1 = m;     m += n1;
    w->b1 = m;     m += n1;
    w->tb1 = m;    m += n1;
    w->tb2 = m;    m += n1;
}

static void ws_free(pencil_ws *w) { free(w->su); }

/* ------------------------------------------------------------------------ */
/* mhdflux: flux vector v and pencil-wide max fast speed c                   */
/* Heterogeneous_MHD/C/mhdflux.c:9-59 (find_max :61-72)                      */
/* ------------------------------------------------------------------------ */
static void pencil_flux(real *v, real *c_out, const real *u, const real *b, int n,
                        pencil_ws *w)
{
    real gamma = 5.0 / 3.0;
    real *vx = w->vx, *ps = w->ps, *pp = w->pp, *tc = w->tc;
    int i, ii;

    for (i = 0; i < n; i++)
        vx[i] = PU(u, 1, i) / PU(u, 0, i);

    for (i = 0; i < n; i++) {
        real r = PU(u, 0, i), m1 = PU(u, 1, i), m2 = PU(u, 2, i), m3 = PU(u, 3, i);
        real e = PU(u, 4, i);
        real bx = PB(b, 0, i), by = PB(b, 1, i), bz = PB(b, 2, i);
        /* total pressure; '/2.0' and '1.0','2.0' promote to double */
        ps[i] = (e - (m1 * m1 + m2 * m2 + m3 * m3) / r / 2.0) * (gamma - 1.0)
              + (2.0 - gamma) * (bx * bx + by * by + bz * bz) / 2.0;
    }

    for (i = 0; i < n; i++) {
        real r = PU(u, 0, i), m1 = PU(u, 1, i), m2 = PU(u, 2, i), m3 = PU(u, 3, i);
        real e = PU(u, 4, i);
        real bx = PB(b, 0, i), by = PB(b, 1, i), bz = PB(b, 2, i);
        PU(v, 0, i) = m1;
        PU(v, 1, i) = m1 * vx[i] + ps[i] - bx * bx;
        PU(v, 2, i) = m2 * vx[i] - by * bx;
        PU(v, 3, i) = m3 * vx[i] - bz * bx;
        PU(v, 4, i) = (e + ps[i]) * vx[i] - bx * (bx * m1 + by * m2 + bz * m3) / r;
    }

    for (i = 0; i < n; i++) {
        real bx = PB(b, 0, i), by = PB(b, 1, i), bz = PB(b, 2, i);
        pp[i] = ps[i] - (bx * bx + by * by + bz * bz) / 2.0;
    }

    for (i = 0; i < n; i++) {
        real bx = PB(b, 0, i), by = PB(b, 1, i), bz = PB(b, 2, i);
        /* fabs/sqrt are the double libm functions in the reference */
        tc[i] = fabs(vx[i]) + sqrt(fabs((bx * bx + by * by + bz * bz + gamma * pp[i]) / PU(u, 0, i)));
    }

    {
        real cmax = 0.0;
        for (i = 0; i < n; i++)
            if (tc[i] > cmax) cmax = tc[i];
        *c_out = cmax;
    }

    if (*c_out > 0) {
        for (i = 0; i < n; i++)
            for (ii = 0; ii < 5; ii++)
                PU(v, ii, i) = PU(v, ii, i) / (*c_out);
    }
}

/* ------------------------------------------------------------------------ */
/* tvd1: relaxing TVD, RK2 half step then full step with van Leer limiter    */
/* Heterogeneous_MHD/C/tvd1.c:8-118                                          */
/* ------------------------------------------------------------------------ */
static void pencil_tvd(real *u, const real *b, int n, real dt, pencil_ws *w)
{
    real *v = w->v, *u1 = w->u1, *wr = w->wr, *wl = w->wl, *fr = w->fr, *fl = w->fl;
    real *flux = w->flux, *dfr = w->dfr, *dfl = w->dfl;
    real c;
    int i, ii;
    real half_dt = -1.0 * dt / 2.0; /* converted to float like the abXYc argument */
    real full_dt = -1.0 * dt;

    /* half step */
    pencil_flux(v, &c, u, b, n, w);
    for (i = 0; i < n; i++)
        for (ii = 0; ii < 5; ii++) {
            PU(wr, ii, i) = abxyc(1.0, PU(u, ii, i), 1.0, PU(v, ii, i), 0.0);
            PU(wl, ii, i) = abxyc(1.0, PU(u, ii, i), -1.0, PU(v, ii, i), 0.0);
        }
    for (i = 0; i < n; i++)
        for (ii = 0; ii < 5; ii++) {
            PU(fr, ii, i) = abxyc(c, PU(wr, ii, i), 0.0, PU(wr, ii, i), 0.0);
            real wlp = PU(wl, ii, wrap_up(i, n));
            PU(fl, ii, i) = abxyc(c, wlp, 0.0, wlp, 0.0);
        }
    for (i = 0; i < n; i++)
        for (ii = 0; ii < 5; ii++)
            PU(flux, ii, i) = abxyc(0.5, PU(fr, ii, i), -0.5, PU(fl, ii, i), 0.0);
    for (i = 0; i < n; i++)
        for (ii = 0; ii < 5; ii++) {
            real d = abxyc(1.0, PU(flux, ii, i), -1.0, PU(flux, ii, wrap_dn(i, n)), 0.0);
            PU(u1, ii, i) = abxyc(1.0, PU(u, ii, i), half_dt, d, 0.0);
        }

    /* full step */
    pencil_flux(v, &c, u1, b, n, w);
    for (i = 0; i < n; i++)
        for (ii = 0; ii < 5; ii++) {
            PU(wr, ii, i) = abxyc(1.0, PU(u1, ii, i), 1.0, PU(v, ii, i), 0.0);
            PU(wl, ii, i) = abxyc(1.0, PU(u1, ii, i), -1.0, PU(v, ii, i), 0.0);
        }
    for (i = 0; i < n; i++)
        for (ii = 0; ii < 5; ii++)
            PU(fr, ii, i) = abxyc(c, PU(wr, ii, i), 0.0, PU(wr, ii, i), 0.0);
    for (i = 0; i < n; i++)
        for (ii = 0; ii < 5; ii++) {
            real frp = PU(fr, ii, wrap_up(i, n)), frm = PU(fr, ii, wrap_dn(i, n));
            real dp = abxyc(0.5, frp, -0.5, PU(fr, ii, i), 0.0);
            real dm = abxyc(0.5, PU(fr, ii, i), -0.5, frm, 0.0);
            PU(dfr, ii, i) = 0.0;
            if (dp * dm > 0)
                PU(dfr, ii, i) = 2.0 * dp * dm / (dp + dm); /* van Leer */
        }
    for (i = 0; i < n; i++)
        for (ii = 0; ii < 5; ii++) {
            real wlp = PU(wl, ii, wrap_up(i, n));
            PU(fl, ii, i) = abxyc(c, wlp, 0.0, wlp, 0.0);
        }
    for (i = 0; i < n; i++)
        for (ii = 0; ii < 5; ii++) {
            real flp = PU(fl, ii, wrap_up(i, n)), flm = PU(fl, ii, wrap_dn(i, n));
            real dp = abxyc(0.5, PU(fl, ii, i), -0.5, flp, 0.0);
            real dm = abxyc(0.5, flm, -0.5, PU(fl, ii, i), 0.0);
            PU(dfl, ii, i) = 0.0;
            if (dp * dm > 0)
                PU(dfl, ii, i) = 2.0 * dp * dm / (dp + dm);
        }
    for (i = 0; i < n; i++)
        for (ii = 0; ii < 5; ii++) {
            real a = abxyc(1.0, PU(fr, ii, i), -1.0, PU(fl, ii, i), 0.0);
            real d = abxyc(1.0, PU(dfr, ii, i), -1.0, PU(dfl, ii, i), 0.0);
            PU(flux, ii, i) = abxyc(0.5, a, 0.5, d, 0.0);
        }
    for (i = 0; i < n; i++)
        for (ii = 0; ii < 5; ii++) {
            real d = abxyc(1.0, PU(flux, ii, i), -1.0, PU(flux, ii, wrap_dn(i, n)), 0.0);
            PU(u, ii, i) = abxyc(1.0, PU(u, ii, i), full_dt, d, 0.0);
        }
}

/* ------------------------------------------------------------------------ */
/* tvdb: upwind + van Leer advection of a face field along the pencil        */
/* Heterogeneous_MHD/C/tvdb.c:10-91                                          */
/* ------------------------------------------------------------------------ */
static void pencil_tvdb(real *flux, real *bf, const real *vg, int n, real dt, pencil_ws *w)
{
    real *vh = w->vh, *f1 = w->f1, *b1 = w->b1, *bv = w->tb2;
    int i;

    for (i = 0; i < n; i++)
        vh[i] = abxyc(0.5, vg[i], 0.5, vg[wrap_up(i, n)], 0.0);
    for (i = 0; i < n; i++)
        bv[i] = bf[i] * vg[i];
    for (i = 0; i < n; i++)
        f1[i] = (vh[i] > 0) ? bv[i] : bv[wrap_up(i, n)];
    for (i = 0; i < n; i++)
        b1[i] = bf[i] - (f1[i] - f1[wrap_dn(i, n)]) * dt / 2.0;
    for (i = 0; i < n; i++) {
        int ip = wrap_up(i, n), ipp = wrap_up(ip, n), im = wrap_dn(i, n);
        real wv, wp, wm, dw;
        if (vh[i] > 0) {
            wv = vg[i] * b1[i];
            wp = (vg[ip] * b1[ip] - wv) / 2.0;
            wm = (wv - vg[im] * b1[im]) / 2.0;
        } else {
            wv = vg[ip] * b1[ip];
            wp = (wv - vg[ipp] * b1[ipp]) / 2.0;
            wm = (vg[i] * b1[i] - wv) / 2.0;
        }
        dw = 0;
        if (wm * wp > 0)
            dw = 2.0 * wm * wp / (wm + wp);
        flux[i] = (wv + dw) * dt;
    }
    {
        /* b = b - (flux - cshift(flux,-1)); flux lives on the right face */
        real *prev = w->tb1;
        for (i = 0; i < n; i++)
            prev[i] = flux[wrap_dn(i, n)];
        for (i = 0; i < n; i++)
            bf[i] = bf[i] - (flux[i] - prev[i]);
    }
}

/* ------------------------------------------------------------------------ */
/* OpenMP plumbing                                                           */
/* ------------------------------------------------------------------------ */
static int g_threads = 1;

#ifdef ORACLE_F32
void oracle_set_threads(int nthreads) { g_threads = nthreads > 0 ? nthreads : 1; }
int oracle_get_threads(void) { return g_threads; }
#else
extern void oracle_set_threads(int nthreads);
extern int oracle_get_threads(void);
#endif

static int nthreads_now(void)
{
#ifdef ORACLE_F32
    return g_threads;
#else
    (void)g_threads;
    return oracle_get_threads();
#endif
}

/* ------------------------------------------------------------------------ */
/* fluidx: gather pencil + cell-centred B, tvd1, scatter                     */
/* Heterogeneous_MHD/C/fluidx.c:19-102                                       */
/* ------------------------------------------------------------------------ */
void PFX(fluidx)(real *u, real *b, int *pnx, int *pny, int *pnz, real *pdt,
                 real *update_u, real *update_b, int iter)
{
    int nx = *pnx, ny = *pny, nz = *pnz;
    long npen = (long)ny * nz;
    real dt = *pdt;
    (void)b;
    (void)iter;
#pragma omp parallel num_threads(nthreads_now())
    {
        pencil_ws w;
        long p;
        ws_init(&w, nx);
#pragma omp for schedule(static)
        for (p = 0; p < npen; p++) {
            int j = (int)(p % ny), k = (int)(p / ny);
            int jp = (j + 1) % ny, kp = (k + 1) % nz;
            int i, ii;
            for (i = 0; i < nx; i++) {
                size_t c0 = cidx(nx, ny, i, j, k);
                for (ii = 0; ii < 5; ii++) PU(w.su, ii, i) = GU(update_u, ii, c0);
                /* multiple_itself_matrix2D(b3x,3,nx,0.5) */
                for (ii = 0; ii < 3; ii++) PB(w.bc, ii, i) = (real)0.5 * GB(update_b, ii, c0);
            }
            for (i = 0; i < nx; i++)
                w.t1[i] = PB(w.bc, 0, wrap_up(i, nx));
            for (i = 0; i < nx; i++) {
                PB(w.bc, 0, i) = PB(w.bc, 0, i) + w.t1[i];
                PB(w.bc, 1, i) = PB(w.bc, 1, i) + GB(update_b, 1, cidx(nx, ny, i, jp, k)) / 2;
                PB(w.bc, 2, i) = PB(w.bc, 2, i) + GB(update_b, 2, cidx(nx, ny, i, j, kp)) / 2;
            }
            pencil_tvd(w.su, w.bc, nx, dt, &w);
            for (i = 0; i < nx; i++) {
                size_t c0 = cidx(nx, ny, i, j, k);
                for (ii = 0; ii < 5; ii++) GU(u, ii, c0) = PU(w.su, ii, i);
            }
        }
        ws_free(&w);
    }
}

/* ------------------------------------------------------------------------ */
/* advectbyzx: constrained-transport advection of the two transverse face    */
/* fields along the pencil.                                                  */
/*   stage A: Heterogeneous_MHD/C/advectbyzxA1.c:18-63 then A2.c:9-28        */
/*   stage B: Heterogeneous_MHD/C/advectbyzxB1.c:19-62 then B2.c:9-29        */
/* The per-cell rounding order of b(1) is (((bx-fA)+fA(j+1))-fB)+fB(k+1).    */
/* ------------------------------------------------------------------------ */
static void advect_stage(real *b, int nx, int ny, int nz, real dt,
                         const real *update_u, const real *update_b,
                         int comp /* 1: A (b_y, jm); 2: B (b_z, km) */, real *tmpgrid)
{
    long npen = (long)ny * nz;
    long p;
#pragma omp parallel num_threads(nthreads_now())
    {
        pencil_ws w;
        ws_init(&w, nx);
#pragma omp for schedule(static)
        for (p = 0; p < npen; p++) {
            int j = (int)(p % ny), k = (int)(p / ny);
            int jn = (comp == 1) ? (j + ny - 1) % ny : j;
            int kn = (comp == 1) ? k : (k + nz - 1) % nz;
            int i;
            for (i = 0; i < nx; i++) {
                size_t cs = cidx(nx, ny, i, j, k), cn = cidx(nx, ny, i, jn, kn);
                w.avx[i] = (GU(update_u, 1, cn) + GU(update_u, 1, cs))
                         / (GU(update_u, 0, cn) + GU(update_u, 0, cs));
            }
            for (i = 0; i < nx; i++) {
                w.at1[i] = w.avx[wrap_dn(i, nx)];
                w.at2[i] = w.avx[wrap_up(i, nx)];
            }
            for (i = 0; i < nx; i++) {
                w.avx[i] = (w.at1[i] + w.at2[i] + 2.0 * w.avx[i]) / 4.0;
                w.ab[i] = GB(update_b, comp, cidx(nx, ny, i, j, k));
            }
            pencil_tvdb(w.aflux, w.ab, w.avx, nx, dt, &w);
            for (i = 0; i < nx; i++)
                w.at1[i] = w.aflux[wrap_dn(i, nx)];
            for (i = 0; i < nx; i++) {
                size_t cs = cidx(nx, ny, i, j, k);
                GB(b, comp, cs) = w.ab[i];
                GB(b, 0, cs) = GB(b, 0, cs) - w.at1[i];
                tmpgrid[cs] = w.at1[i];
            }
        }
        ws_free(&w);
    }
    /* second pass: b(1) of the jm (or km) pencil += the flux of this pencil */
#pragma omp parallel for schedule(static) num_threads(nthreads_now())
    for (p = 0; p < npen; p++) {
        int j = (int)(p % ny), k = (int)(p / ny);
        int jn = (comp == 1) ? (j + ny - 1) % ny : j;
        int kn = (comp == 1) ? k : (k + nz - 1) % nz;
        int i;
        for (i = 0; i < nx; i++) {
            size_t cn = cidx(nx, ny, i, jn, kn);
            GB(b, 0, cn) = GB(b, 0, cn) + tmpgrid[cidx(nx, ny, i, j, k)];
        }
    }
}

void PFX(advectbyzx)(real *u, real *b, int *pnx, int *pny, int *pnz, real *pdt,
                     real *update_u, real *update_b)
{
    int nx = *pnx, ny = *pny, nz = *pnz;
    size_t ncell = (size_t)nx * ny * nz;
    real *tmpgrid = (real *)malloc(ncell * sizeof(real));
    (void)u;
    advect_stage(b, nx, ny, nz, *pdt, update_u, update_b, 1, tmpgrid);
    advect_stage(b, nx, ny, nz, *pdt, update_u, update_b, 2, tmpgrid);
    free(tmpgrid);
}

/* ------------------------------------------------------------------------ */
/* transposes: pure component-permuting axis swaps (bit-exact copies)        */
/* transpose12: Heterogeneous_MHD/C/transpose12.c:7-47, OpenMP/mhd.f90:410   */
/* transpose13: Heterogeneous_MHD/C/transpose13.c:9-62, OpenMP/mhd.f90:433   */
/* The reference refuses transpose13 when nx != nz; the Fortran original's   */
/* nz==1 and nx==1 branches reduce to the same formula as the cubic case,    */
/* which is applied here for every shape.                                    */
/* ------------------------------------------------------------------------ */
void PFX(transpose12)(real *u, real *b, real *update_u, real *update_b,
                      int *pnx, int *pny, int *pnz, int iter)
{
    static const int pu[5] = {0, 2, 1, 3, 4};
    static const int pb[3] = {1, 0, 2};
    int nx = *pnx, ny = *pny, nz = *pnz;
    long k;
    (void)iter;
#pragma omp parallel for schedule(static) num_threads(nthreads_now())
    for (k = 0; k < nz; k++) {
        int i, j, ii;
        for (j = 0; j < ny; j++)
            for (i = 0; i < nx; i++) {
                size_t src = cidx(nx, ny, i, j, (int)k);
                size_t dst = cidx(ny, nx, j, i, (int)k);
                for (ii = 0; ii < 5; ii++) GU(u, ii, dst) = GU(update_u, pu[ii], src);
                for (ii = 0; ii < 3; ii++) GB(b, ii, dst) = GB(update_b, pb[ii], src);
            }
    }
}

void PFX(transpose13)(real *u, real *b, real *update_u, real *update_b,
                      int *pnx, int *pny, int *pnz)
{
    static const int pu[5] = {0, 3, 2, 1, 4};
    static const int pb[3] = {2, 1, 0};
    int nx = *pnx, ny = *pny, nz = *pnz;
    long j;
#pragma omp parallel for schedule(static) num_threads(nthreads_now())
    for (j = 0; j < ny; j++) {
        int i, k, ii;
        for (k = 0; k < nz; k++)
            for (i = 0; i < nx; i++) {
                size_t src = cidx(nx, ny, i, (int)j, k);
                size_t dst = cidx(nz, ny, k, (int)j, i); /* out dims (nz,ny,nx) */
                for (ii = 0; ii < 5; ii++) GU(u, ii, dst) = GU(update_u, pu[ii], src);
                for (ii = 0; ii < 3; ii++) GB(b, ii, dst) = GB(update_b, pb[ii], src);
            }
    }
}

void PFX(copy_matrix)(real *u, real *b, int *pnx, int *pny, int *pnz,
                      real *update_u, real *update_b)
{
    size_t ncell = (size_t)(*pnx) * (*pny) * (*pnz);
    memcpy(update_u, u, ncell * 5 * sizeof(real));
    memcpy(update_b, b, ncell * 3 * sizeof(real));
}

/* ------------------------------------------------------------------------ */
/* CFL: max over cells of the fast speed; returns 1/c                        */
/* Heterogeneous_MHD/C/calcfl.c:13-65 (max_3num :67, max_2num :93).           */
/* The C path uses the cell's own face B, unaveraged.                        */
/* ------------------------------------------------------------------------ */
static inline real max3(real a, real b, real c)
{
    if (a > b) return (a > c) ? a : c;
    return (b > c) ? b : c;
}

static inline real max2(real a, real b) { return (a > b) ? a : b; }

real PFX(calcfl)(real *u, real *b, int *pnx, int *pny, int *pnz)
{
    int nx = *pnx, ny = *pny, nz = *pnz;
    real gamma = 5.0 / 3.0;
    real c = 0.0;
    real tmp;
    long k;
#pragma omp parallel num_threads(nthreads_now())
    {
        real cl = 0.0;
#pragma omp for schedule(static)
        for (k = 0; k < nz; k++) {
            int i, j;
            for (j = 0; j < ny; j++)
                for (i = 0; i < nx; i++) {
                    size_t c0 = cidx(nx, ny, i, j, (int)k);
                    real r = GU(u, 0, c0), m1 = GU(u, 1, c0), m2 = GU(u, 2, c0);
                    real m3 = GU(u, 3, c0), e = GU(u, 4, c0);
                    real bx = GB(b, 0, c0), by = GB(b, 1, c0), bz = GB(b, 2, c0);
                    real t1 = fabs(m1 / r), t2 = fabs(m2 / r), t3 = fabs(m3 / r);
                    real v = max3(t1, t2, t3);
                    real ps = (e - (m1 * m1 + m2 * m2 + m3 * m3) / r / 2.0) * (gamma - 1.0)
                            + (2.0 - gamma) * (bx * bx + by * by + bz * bz) / 2.0;
                    real p = ps - (bx * bx + by * by + bz * bz) / 2.0;
                    /* fabs wraps the numerator only here (calcfl.c:54), unlike mhdflux.c:45 */
                    real cc = v + sqrt(fabs((bx * bx + by * by + bz * bz) * 2.0 + gamma * p) / r);
                    cl = max2(cl, cc);
                }
        }
#pragma omp critical
        c = max2(c, cl);
    }
    tmp = 1.0 / c;
    return tmp;
}

/* Release 0.2 CFL with cell-centred B (OpenMP/mhd.f90:96-125), evaluated in
 * the solver's own precision as the Fortran source does. */
real PFX(calcfl_averaged)(real *u, real *b, int *pnx, int *pny, int *pnz)
{
    int nx = *pnx, ny = *pny, nz = *pnz;
    real gamma = (real)5 / (real)3;
    real c = 0;
    long k;
#pragma omp parallel num_threads(nthreads_now())
    {
        real cl = 0;
#pragma omp for schedule(static)
        for (k = 0; k < nz; k++) {
            int i, j, kp = (int)((k + 1) % nz);
            for (j = 0; j < ny; j++) {
                int jp = (j + 1) % ny;
                for (i = 0; i < nx; i++) {
                    int ip = (i + 1) % nx;
                    size_t c0 = cidx(nx, ny, i, j, (int)k);
                    real r = GU(u, 0, c0), m1 = GU(u, 1, c0), m2 = GU(u, 2, c0);
                    real m3 = GU(u, 3, c0), e = GU(u, 4, c0);
                    real bx = (GB(b, 0, c0) + GB(b, 0, cidx(nx, ny, ip, j, (int)k))) / (real)2;
                    real by = (GB(b, 1, c0) + GB(b, 1, cidx(nx, ny, i, jp, (int)k))) / (real)2;
                    real bz = (GB(b, 2, c0) + GB(b, 2, cidx(nx, ny, i, j, kp))) / (real)2;
                    real a1 = m1 / r, a2 = m2 / r, a3 = m3 / r;
                    real v = max3(a1 < 0 ? -a1 : a1, a2 < 0 ? -a2 : a2, a3 < 0 ? -a3 : a3);
                    real b2 = bx * bx + by * by + bz * bz;
                    real ps = (e - (m1 * m1 + m2 * m2 + m3 * m3) / r / (real)2) * (gamma - (real)1)
                            + ((real)2 - gamma) * b2 / (real)2;
                    real p = ps - b2 / (real)2;
                    real q = (b2 * (real)2 + gamma * p) / r;
                    real s = (real)sqrt((double)(q < 0 ? -q : q));
                    real cc = v + s;
                    cl = (cl > cc) ? cl : cc;
                }
            }
        }
#pragma omp critical
        c = (c > cl) ? c : cl;
    }
    return (real)1 / c;
}

/* dt = cfl_number * (1/c), clamped so that t never passes tf
 * (Heterogeneous_MHD/C/mhd.c:63-64; the product is formed in double as the
 * reference's 0.9*calcfl(...) is). tf <= 0 disables the clamp. */
real PFX(dt_from_cfl)(real inv_c, double cfl_number, real t, real tf)
{
    real dt = cfl_number * inv_c;
    if (tf > 0 && dt > (tf - t) / 2) dt = (tf - t) / 2;
    return dt;
}

/* ------------------------------------------------------------------------ */
/* one full Strang-symmetric step x,y,z,z,y,x at a given dt                  */
/* Heterogeneous_MHD/C/mhd.c:72-119; (u,b) is ctx, (wu,wb) is ctx_update.    */
/* ------------------------------------------------------------------------ */
void PFX(step)(real *u, real *b, int nx, int ny, int nz, real dt, real *wu, real *wb)
{
    real d = dt;
    PFX(copy_matrix)(u, b, &nx, &ny, &nz, wu, wb);
    /* x */
    PFX(fluidx)(u, b, &nx, &ny, &nz, &d, wu, wb, 0);
    PFX(copy_matrix)(u, b, &nx, &ny, &nz, wu, wb);
    PFX(advectbyzx)(u, b, &nx, &ny, &nz, &d, wu, wb);
    PFX(copy_matrix)(u, b, &nx, &ny, &nz, wu, wb);
    /* y */
    PFX(transpose12)(u, b, wu, wb, &nx, &ny, &nz, 0);
    PFX(copy_matrix)(u, b, &ny, &nx, &nz, wu, wb);
    PFX(fluidx)(u, b, &ny, &nx, &nz, &d, wu, wb, 0);
    PFX(copy_matrix)(u, b, &ny, &nx, &nz, wu, wb);
    PFX(advectbyzx)(u, b, &ny, &nx, &nz, &d, wu, wb);
    PFX(copy_matrix)(u, b, &ny, &nx, &nz, wu, wb);
    /* z (twice) */
    PFX(transpose13)(u, b, wu, wb, &ny, &nx, &nz);
    PFX(copy_matrix)(u, b, &nz, &nx, &ny, wu, wb);
    PFX(fluidx)(u, b, &nz, &nx, &ny, &d, wu, wb, 0);
    PFX(copy_matrix)(u, b, &nz, &nx, &ny, wu, wb);
    PFX(advectbyzx)(u, b, &nz, &nx, &ny, &d, wu, wb);
    PFX(copy_matrix)(u, b, &nz, &nx, &ny, wu, wb);
    PFX(advectbyzx)(u, b, &nz, &nx, &ny, &d, wu, wb);
    PFX(copy_matrix)(u, b, &nz, &nx, &ny, wu, wb);
    PFX(fluidx)(u, b, &nz, &nx, &ny, &d, wu, wb, 0);
    PFX(copy_matrix)(u, b, &nz, &nx, &ny, wu, wb);
    /* y back */
    PFX(transpose13)(u, b, wu, wb, &nz, &nx, &ny);
    PFX(copy_matrix)(u, b, &ny, &nx, &nz, wu, wb);
    PFX(advectbyzx)(u, b, &ny, &nx, &nz, &d, wu, wb);
    PFX(copy_matrix)(u, b, &ny, &nx, &nz, wu, wb);
    PFX(fluidx)(u, b, &ny, &nx, &nz, &d, wu, wb, 0);
    PFX(copy_matrix)(u, b, &ny, &nx, &nz, wu, wb);
    /* x back */
    PFX(transpose12)(u, b, wu, wb, &ny, &nx, &nz, 0);
    PFX(copy_matrix)(u, b, &nx, &ny, &nz, wu, wb);
    PFX(advectbyzx)(u, b, &nx, &ny, &nz, &d, wu, wb);
    PFX(copy_matrix)(u, b, &nx, &ny, &nz, wu, wb);
    PFX(fluidx)(u, b, &nx, &ny, &nz, &d, wu, wb, 0);
    PFX(copy_matrix)(u, b, &nx, &ny, &nz, wu, wb);
}

/* time loop of Heterogeneous_MHD/C/mhd.c:60-125 with a step cap.
 * cfl_mode 0: C path formula (calcfl); 1: release 0.2 averaged formula.
 * With tf > 0 the loop is the reference's do { } while (t < tf); with
 * tf <= 0 it runs exactly max_steps steps.  Returns the number of steps;
 * dt_log (optional) receives each step's dt. */
int PFX(run)(real *u, real *b, int nx, int ny, int nz, double cfl_number, int cfl_mode,
             real *t, real tf, int max_steps, real *dt_log)
{
    size_t ncell = (size_t)nx * ny * nz;
    real *wu = (real *)malloc(ncell * 5 * sizeof(real));
    real *wb = (real *)malloc(ncell * 3 * sizeof(real));
    int s;
    for (s = 0; s < max_steps; s++) {
        real inv_c, dt;
        if (tf > 0 && s > 0 && !(*t < tf)) break;
        inv_c = cfl_mode ? PFX(calcfl_averaged)(u, b, &nx, &ny, &nz)
                         : PFX(calcfl)(u, b, &nx, &ny, &nz);
        dt = PFX(dt_from_cfl)(inv_c, cfl_number, *t, tf);
        *t = *t + 2 * dt;
        if (dt_log) dt_log[s] = dt;
        PFX(step)(u, b, nx, ny, nz, dt, wu, wb);
    }
    free(wu);
    free(wb);
    return s;
}
