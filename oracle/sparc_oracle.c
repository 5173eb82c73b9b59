/*
 * sparc_oracle.c -- CPU FP64 restatement of SPARC's 2-D displacement-formulation
 * wave-solver hot path.  TEST INFRASTRUCTURE ONLY: this file is the checker that the
 * CUDA path is compared against (tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / reference arm).  Nothing in the product links or calls it.
 *
 * PARITY UNPINNED against a run of the reference: the reference is Fortran 90/77 +
 * MPI + FFTW + CFITSIO and none of those toolchains exist here, and the reference
 * ships no tests or golden vectors.  What pins this restatement instead:
 *   - FFT and spectral derivative vs numpy.fft and analytic trigonometric derivatives;
 *   - compact finite differences: exactness on low-degree polynomials, 6th-order
 *     convergence, and the float32-rounded coefficients of dbyd2.f (implicit REAL);
 *   - the RK coefficients from step.f90:28-40 (float32-rounded literals);
 *   - an independent NumPy restatement (oracle/oracle.py) of single operators.
 *
 * Layout follows the Fortran arrays: every field is x-fastest, f[k*nx + i], i = 0..nx-1
 * (Fortran i = 1..nx), k = 0..nz-1 (Fortran k = 1..nz, k = 1 the deepest level).
 * The state a(:,:,:,1:6) keeps the six displacement-formulation variables
 * (xi_x, xi_y, xi_z, v_x, v_y, v_z) as in initialize.f90:484-496.
 * Option 17 (MP_QUIET_PML_2D_DISPL) by default; orc_set_magnetic switches a run without flow to
 * option 18 (MP_MHD_PML_2D_DISPL, physics2d.f90:719-938), which has no GPU counterpart yet.
 *
 * Build: oracle/Makefile (gcc -O2 -ffp-contract=off, no fast-math) -> oracle/_build/.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.141592653589793 /* initialize.f90:42 */
#define ORC_RSUN 6.95989467700e10 /* initialize.f90:42, cm */

/* ------------------------------------------------------------------------- */
/* FFT (FFTW 3 is an un-vendored dependency of the reference, makefile:25;    */
/* this is an independent mixed-radix Stockham FFT, checked against numpy).   */
/* ------------------------------------------------------------------------- */
typedef struct {
    int n, nf, fac[40];
    double *wr, *wi; /* exp(-2 pi i t / n), t = 0..n-1 */
} orc_fft;

static int fft_plan(orc_fft *f, int n)
{
    int m = n, nf = 0;
    f->n = n;
    while (m % 4 == 0) { f->fac[nf++] = 4; m /= 4; }
    while (m % 2 == 0) { f->fac[nf++] = 2; m /= 2; }
    while (m % 3 == 0) { f->fac[nf++] = 3; m /= 3; }
    while (m % 5 == 0) { f->fac[nf++] = 5; m /= 5; }
    if (m != 1) return -1;
    f->nf = nf;
    f->wr = (double *)malloc(sizeof(double) * n);
    f->wi = (double *)malloc(sizeof(double) * n);
    for (int t = 0; t < n; t++) {
        double ang = -2.0 * ORC_PI * (double)t / (double)n;
        f->wr[t] = cos(ang);
        f->wi[t] = sin(ang);
    }
    return 0;
}

static void fft_free(orc_fft *f)
{
    free(f->wr);
    free(f->wi);
}

/* Stockham autosort; sign = -1 forward (numpy convention), +1 unnormalised inverse.
 * Result returned in (re, im); (tr, ti) are scratch of length n. */
static void fft_exec(const orc_fft *f, double *re, double *im, double *tr, double *ti, int sign)
{
    int n = f->n, ns = 1;
    double *xr = re, *xi = im, *yr = tr, *yi = ti;
    for (int s = 0; s < f->nf; s++) {
        int R = f->fac[s], nr = n / R;
        int tstep = n / (ns * R);
        for (int j = 0; j < nr; j++) {
            int k = j % ns;
            double vr[5], vi[5];
            for (int r = 0; r < R; r++) {
                int t = (r * k * tstep) % n;
                double wr = f->wr[t], wi = sign < 0 ? f->wi[t] : -f->wi[t];
                double ar = xr[j + r * nr], ai = xi[j + r * nr];
                vr[r] = ar * wr - ai * wi;
                vi[r] = ar * wi + ai * wr;
            }
            double or_[5], oi[5];
            if (R == 2) {
                or_[0] = vr[0] + vr[1]; oi[0] = vi[0] + vi[1];
                or_[1] = vr[0] - vr[1]; oi[1] = vi[0] - vi[1];
            } else if (R == 4) {
                double s0r = vr[0] + vr[2], s0i = vi[0] + vi[2];
                double d0r = vr[0] - vr[2], d0i = vi[0] - vi[2];
                double s1r = vr[1] + vr[3], s1i = vi[1] + vi[3];
                double d1r = vr[1] - vr[3], d1i = vi[1] - vi[3];
                /* multiply d1 by -i (forward) or +i (inverse) */
                double jr = sign < 0 ? d1i : -d1i, ji = sign < 0 ? -d1r : d1r;
                or_[0] = s0r + s1r; oi[0] = s0i + s1i;
                or_[1] = d0r + jr;  oi[1] = d0i + ji;
                or_[2] = s0r - s1r; oi[2] = s0i - s1i;
                or_[3] = d0r - jr;  oi[3] = d0i - ji;
            } else {
                for (int q = 0; q < R; q++) {
                    double sr = 0.0, si = 0.0;
                    for (int r = 0; r < R; r++) {
                        int t = ((r * q) % R) * (n / R);
                        double wr = f->wr[t], wi = sign < 0 ? f->wi[t] : -f->wi[t];
                        sr += vr[r] * wr - vi[r] * wi;
                        si += vr[r] * wi + vi[r] * wr;
                    }
                    or_[q] = sr; oi[q] = si;
                }
            }
            int base = (j / ns) * ns * R + k;
            for (int r = 0; r < R; r++) {
                yr[base + r * ns] = or_[r];
                yi[base + r * ns] = oi[r];
            }
        }
        double *t1 = xr, *t2 = xi;
        xr = yr; xi = yi; yr = t1; yi = t2;
        ns *= R;
    }
    if (xr != re) {
        memcpy(re, xr, sizeof(double) * n);
        memcpy(im, xi, sizeof(double) * n);
    }
}

/* Reusable plans for the 3-D restatement (sparc_oracle3d.c). */
void *orc_fft_new(int n)
{
    orc_fft *f = (orc_fft *)calloc(1, sizeof(orc_fft));
    if (!f || fft_plan(f, n)) { free(f); return NULL; }
    return f;
}
void orc_fft_delete(void *f)
{
    if (!f) return;
    fft_free((orc_fft *)f);
    free(f);
}
void orc_fft_exec(const void *f, double *re, double *im, double *tr, double *ti, int sign)
{
    fft_exec((const orc_fft *)f, re, im, tr, ti, sign);
}

/* Public complex FFT for the tests (sign -1 forward / +1 inverse, unnormalised). */
int orc_fft_c2c(int n, double *re, double *im, int sign)
{
    orc_fft f;
    if (fft_plan(&f, n)) return -1;
    double *tr = (double *)malloc(sizeof(double) * n), *ti = (double *)malloc(sizeof(double) * n);
    fft_exec(&f, re, im, tr, ti, sign);
    free(tr); free(ti); fft_free(&f);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Compact finite differences: dbyd2.f:8-235 with mtridag.f:96-112.          */
/* The coefficients d2i, C1..C5, alpha, alpha2, gamma2, alpha1, beta1, const, */
/* up1 are implicitly REAL(4) in dbyd2.f (no declaration, dbyd2.f:28-31), so   */
/* they are computed here in float and promoted to double where they meet the  */
/* REAL(8) data.                                                               */
/* ------------------------------------------------------------------------- */
int orc_dbyd2(double *A, const double *B, int n1, int n2, int ibc)
{
    if (ibc < 0 || ibc > 4) return -1; /* ibc 5 (periodic) is not on this path */
    float d2i = (float)(n2 - 1);       /* dbyd2.f:44-48 */
    if (n2 < 5) {                      /* dbyd2.f:51-80 */
        for (int j = 0; j < n2; j++)
            for (int i = 0; i < n1; i++) {
                if (ibc == 0) A[j * n1 + i] = 0.0;
                else if (ibc == 1) A[j * n1 + i] = B[(n2 - 1) * n1 + i] - B[i];
                else if (ibc == 2) A[j * n1 + i] = A[i];
                else if (ibc == 3) A[j * n1 + i] = A[(n2 - 1) * n1 + i];
                else A[j * n1 + i] = ((float)j * A[i] + (float)(n2 - 1 - j) * A[(n2 - 1) * n1 + i]) / d2i;
            }
        return 0;
    }
    float C1 = d2i * 7.0f / 9.0f; /* dbyd2.f:82-83 */
    float C2 = d2i / 36.0f;
    for (int k = 2; k <= n2 - 3; k++) /* dbyd2.f:88-93 interior, I=3..N2-2 */
        for (int i = 0; i < n1; i++)
            A[k * n1 + i] = (double)C1 * (B[(k + 1) * n1 + i] - B[(k - 1) * n1 + i]) +
                            (double)C2 * (B[(k + 2) * n1 + i] - B[(k - 2) * n1 + i]);
    float C3, C4, C5;
    C1 = -(43.0f / 96.0f * d2i); /* dbyd2.f:101-105 */
    C2 = -(5.0f / 6.0f * d2i);
    C3 = 9.0f / 8.0f * d2i;
    C4 = 1.0f / 6.0f * d2i;
    C5 = -(1.0f / 96.0f * d2i);
    for (int i = 0; i < n1; i++) /* dbyd2.f:107-111 */
        A[1 * n1 + i] = (double)C1 * B[i] + (double)C2 * B[n1 + i] + (double)C3 * B[2 * n1 + i] +
                        (double)C4 * B[3 * n1 + i] + (double)C5 * B[4 * n1 + i];
    for (int i = 0; i < n1; i++) /* dbyd2.f:112-115 */
        A[(n2 - 2) * n1 + i] = -((double)C1 * B[(n2 - 1) * n1 + i] + (double)C2 * B[(n2 - 2) * n1 + i] +
                                 (double)C3 * B[(n2 - 3) * n1 + i] + (double)C4 * B[(n2 - 4) * n1 + i] +
                                 (double)C5 * B[(n2 - 5) * n1 + i]);
    C1 = -(10.0f / 3.0f * d2i); /* dbyd2.f:119-122 fifth order closures */
    C2 = -(3.0f * d2i);
    C3 = 6.0f * d2i;
    C4 = 1.0f / 3.0f * d2i;
    if (ibc == 0) { /* dbyd2.f:123-132 */
        for (int i = 0; i < n1; i++) A[i] = 0.0;
    } else if (ibc == 1 || ibc == 3) {
        for (int i = 0; i < n1; i++)
            A[i] = (double)C1 * B[i] + (double)C2 * B[n1 + i] + (double)C3 * B[2 * n1 + i] +
                   (double)C4 * B[3 * n1 + i];
    }
    if (ibc == 0) { /* dbyd2.f:133-145 */
        for (int i = 0; i < n1; i++) A[(n2 - 1) * n1 + i] = 0.0;
    } else if (ibc == 1 || ibc == 2) {
        for (int i = 0; i < n1; i++)
            A[(n2 - 1) * n1 + i] = -((double)C1 * B[(n2 - 1) * n1 + i] + (double)C2 * B[(n2 - 2) * n1 + i] +
                                     (double)C3 * B[(n2 - 3) * n1 + i] + (double)C4 * B[(n2 - 4) * n1 + i]);
    }
    /* matrix, dbyd2.f:151-196 */
    double *uppr = (double *)malloc(sizeof(double) * n2);
    double *lowr = (double *)malloc(sizeof(double) * n2);
    double *gam = (double *)malloc(sizeof(double) * n2);
    double *betad = (double *)malloc(sizeof(double) * n2);
    double *ud = (double *)malloc(sizeof(double) * n2);
    float alpha = 1.0f / 3.0f;
    for (int j = 0; j < n2; j++) uppr[j] = 0.0; /* uppr(N2) is never set in dbyd2.f; unused */
    for (int j = 2; j <= n2 - 3; j++) uppr[j] = (double)alpha;
    float alpha2 = 3.0f / 4.0f, gamma2 = 1.0f / 8.0f, alpha1 = 6.0f, beta1 = 3.0f;
    float cnst = 1.0f / (alpha2 - beta1 * gamma2);
    float up1 = (alpha1 * alpha2 - beta1) * cnst;
    if (ibc % 2 != 0)
        for (int i = 0; i < n1; i++)
            A[i] = ((double)alpha2 * A[i] - (double)beta1 * A[n1 + i]) * (double)cnst;
    if (ibc == 1 || ibc == 2)
        for (int i = 0; i < n1; i++)
            A[(n2 - 1) * n1 + i] =
                ((double)alpha2 * A[(n2 - 1) * n1 + i] - (double)beta1 * A[(n2 - 2) * n1 + i]) * (double)cnst;
    uppr[0] = (ibc % 2 == 0) ? 0.0 : (double)up1;
    uppr[1] = (double)alpha2;
    uppr[n2 - 2] = (double)gamma2;
    for (int j = 0; j < n2; j++) lowr[j] = uppr[n2 - 1 - j];
    lowr[n2 - 1] = (ibc != 1 && ibc != 2) ? 0.0 : (double)up1;
    /* MTRIDAG(LOWR, DIAG=1, UPPR, A, A, N1, N2, 0): mtridag.f:96-112 */
    betad[0] = 1.0;
    for (int j = 1; j < n2; j++) {
        gam[j] = uppr[j - 1] / betad[j - 1];
        betad[j] = 1.0 - lowr[j] * gam[j];
    }
    for (int i = 0; i < n1; i++) {
        ud[0] = A[i] / betad[0];
        for (int j = 1; j < n2; j++) ud[j] = (A[j * n1 + i] - lowr[j] * ud[j - 1]) / betad[j];
        for (int j = n2 - 2; j >= 0; j--) ud[j] = ud[j] - gam[j + 1] * ud[j + 1];
        for (int j = 0; j < n2; j++) A[j * n1 + i] = ud[j];
    }
    free(uppr); free(lowr); free(gam); free(betad); free(ud);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Simulation state                                                          */
/* ------------------------------------------------------------------------- */
typedef struct {
    int nx, nz;
    int npmlbot, npmltop, npmlhor;
    double xlength;   /* cm, params.i:28 */
    double timestep;  /* s, params.i:28 */
    double excitdep;  /* cm, params.i:148 */
    double obsheight; /* cm, params.i:137 */
    int flows;        /* BACKGROUND_FLOWS_EXIST, params.i:70 */
    int adjoint;      /* COMPUTE_ADJOINT (0 = forward) */
    int steps_out;    /* steps = floor(outputcad/timestep), driver.f90:209 */
    int src_until;    /* forcing_length*cadforcing_step, physics2d.f90:1049 */
    double cadforcing;/* params.i:46 */
    int filter_kst;   /* first row (1-based) FILTER_VARS_2D writes: 6 as physics2d.f90:544 */
    int filter_all_x; /* 1: filter every column instead of [npmlhor, nx-npmlhor+1] */
} orc_params;

typedef struct orc_sim {
    orc_params p;
    int nx, nz, nzpml, nhx;
    double dimc, dimrho, diml, deltat, stretchx;
    double betas[5];
    double *z, *x, *stretch, *unstretch, *g;
    double *c_speed, *c2, *rho0, *p0, *rhoinv, *c2rho0, *gradrho0_z, *gradp0_z;
    double *az, *bzpml, *axpml, *bxpml;
    double *v0x, *v0z;
    int e_rad, o_rad; /* 0-based */
    double delta_width;
    double *a, *temp, *scr;                /* 6 * nx * nz */
    double *pmlvars, *psipml, *scrpml;     /* 2 * nx * nzpml */
    double *pmlvarsx, *psipmlx, *scrpmlx;  /* 2 * (2 npmlhor) * nz */
    double *dxixdx, *dxizdz, *div, *pp, *rho, *gradp_x, *gradp_z, *tmp1, *tmp2;
    double *kappa; /* imaginary part of eyekx, initialize.f90:206-208 */
    orc_fft fft;
    double *fre, *fim, *ftr, *fti;
    /* sources */
    double *vr;        /* nx * nvr */
    int nvr;
    double *fwdsource; /* forward time series, driver.f90:1120-1145 */
    int nfwd;
    double *forcing;   /* nx, adjoint Lagrange result, physics.f90:678-737 */
    int num_steps;     /* driver.f90:223-224 */
    int time;
    /* option 18 (MP_MHD_PML_2D_DISPL, physics2d.f90:719-938), set by orc_set_magnetic */
    int magnetic;
    double *box, *boz, *curlboy;           /* nx * nz, B / dimb */
    double *pmlm, *psipmlm, *scrpmlm;      /* 2 * nx * nzpml: psi of d flux2/dz (induction b_x), of d b_x/dz */
    double *flux, *bxp, *bzp, *dzbx, *curlby;
} orc_sim;

static double *zalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }

#define F(s, l) ((s)->a + (size_t)(l) * (s)->nx * (s)->nz)

/* spectral x-derivative, derivatives.f90:28-58: r2c, times eyekx, c2r, times stretchx.
 * Two real rows are transformed at once as the real and imaginary parts of one complex
 * row (the derivative operator maps real rows to real rows). */
static void orc_ddx_rows(orc_sim *s, const double *var, double *dvar, int nrows)
{
    int nx = s->nx;
    for (int r = 0; r < nrows; r += 2) {
        int two = (r + 1 < nrows);
        for (int i = 0; i < nx; i++) {
            s->fre[i] = var[(size_t)r * nx + i];
            s->fim[i] = two ? var[(size_t)(r + 1) * nx + i] : 0.0;
        }
        fft_exec(&s->fft, s->fre, s->fim, s->ftr, s->fti, -1);
        for (int k = 0; k < nx; k++) {
            double kap;
            if (2 * k < nx) kap = s->kappa[k];
            else if (2 * k == nx) kap = 0.0; /* Nyquist: eyekx(nx/2+1)=i*pi makes the bin imaginary, c2r drops it */
            else kap = -s->kappa[nx - k];
            double re = s->fre[k], im = s->fim[k];
            s->fre[k] = -kap * im;
            s->fim[k] = kap * re;
        }
        fft_exec(&s->fft, s->fre, s->fim, s->ftr, s->fti, +1);
        for (int i = 0; i < nx; i++) {
            dvar[(size_t)r * nx + i] = s->fre[i] * s->stretchx;
            if (two) dvar[(size_t)(r + 1) * nx + i] = s->fim[i] * s->stretchx;
        }
    }
}

/* ddz, derivatives.f90:10-24 */
static void orc_ddz(orc_sim *s, const double *var, double *dvar, int bc)
{
    orc_dbyd2(dvar, var, s->nx, s->nz, bc);
    for (int k = 0; k < s->nz; k++)
        for (int i = 0; i < s->nx; i++) dvar[(size_t)k * s->nx + i] *= s->stretch[k];
}

/* public wrappers for the tests */
int orc_sim_ddx(orc_sim *s, const double *var, double *dvar) { orc_ddx_rows(s, var, dvar, s->nz); return 0; }
int orc_sim_ddz(orc_sim *s, const double *var, double *dvar, int bc) { orc_ddz(s, var, dvar, bc); return 0; }

/* ------------------------------------------------------------------------- */
/* Setup: initialize.f90:185-225, 466-474 (grid, eyekx, stretch), solar_data  */
/* initialize.f90:731-794, step.f90:24-41, physics2d.f90:23-405 (2-D RHS).    */
/* model: nz rows x 6 columns (r/Rsun, c, rho, p, g, Gamma1) in cgs,           */
/* deepest row first.  cmul: optional nx*nz multiplier on c (like c_bump,       */
/* initialize.f90:781-791), NULL for none.                                      */
/* ------------------------------------------------------------------------- */
orc_sim *orc_create(const orc_params *prm, const double *model, const double *cmul)
{
    orc_sim *s = (orc_sim *)calloc(1, sizeof(orc_sim));
    s->p = *prm;
    int nx = prm->nx, nz = prm->nz;
    s->nx = nx; s->nz = nz;
    s->nzpml = prm->npmlbot + prm->npmltop;
    s->nhx = 2 * prm->npmlhor;
    size_t N = (size_t)nx * nz;
    if (fft_plan(&s->fft, nx)) { free(s); return NULL; }
    s->fre = zalloc(nx); s->fim = zalloc(nx); s->ftr = zalloc(nx); s->fti = zalloc(nx);
    s->z = zalloc(nz); s->x = zalloc(nx); s->stretch = zalloc(nz); s->unstretch = zalloc(nz); s->g = zalloc(nz);
    s->c_speed = zalloc(N); s->c2 = zalloc(N); s->rho0 = zalloc(N); s->p0 = zalloc(N);
    s->rhoinv = zalloc(N); s->c2rho0 = zalloc(N); s->gradrho0_z = zalloc(N); s->gradp0_z = zalloc(N);
    s->az = zalloc(N); s->bzpml = zalloc(N);
    s->axpml = zalloc((size_t)s->nhx * nz); s->bxpml = zalloc((size_t)s->nhx * nz);
    s->v0x = zalloc(N); s->v0z = zalloc(N);
    s->a = zalloc(6 * N); s->temp = zalloc(6 * N); s->scr = zalloc(6 * N);
    s->pmlvars = zalloc(2 * (size_t)nx * s->nzpml); s->psipml = zalloc(2 * (size_t)nx * s->nzpml);
    s->scrpml = zalloc(2 * (size_t)nx * s->nzpml);
    s->pmlvarsx = zalloc(2 * (size_t)s->nhx * nz); s->psipmlx = zalloc(2 * (size_t)s->nhx * nz);
    s->scrpmlx = zalloc(2 * (size_t)s->nhx * nz);
    s->dxixdx = zalloc(N); s->dxizdz = zalloc(N); s->div = zalloc(N); s->pp = zalloc(N);
    s->rho = zalloc(N); s->gradp_x = zalloc(N); s->gradp_z = zalloc(N); s->tmp1 = zalloc(N); s->tmp2 = zalloc(N);
    s->kappa = zalloc(nx / 2 + 1);
    s->forcing = zalloc(nx);

    /* grid, initialize.f90:195-209 (PERIODIC) */
    double normx = 1.0 / (double)nx;
    for (int i = 0; i < nx; i++) s->x[i] = (double)i / (double)nx;
    for (int i = 0; i <= nx / 2; i++) s->kappa[i] = (double)i * normx * 2.0 * ORC_PI;
    s->stretchx = ORC_RSUN / prm->xlength; /* initialize.f90:225 */

    /* solar_data, initialize.f90:731-794 */
    s->dimc = 1e6; s->dimrho = 1e-3; s->diml = ORC_RSUN;
    for (int k = 0; k < nz; k++) {
        const double *d = model + 6 * k;
        s->z[k] = d[0];
        for (int i = 0; i < nx; i++) {
            size_t q = (size_t)k * nx + i;
            s->c_speed[q] = d[1] / s->dimc;
            s->rho0[q] = d[2] / s->dimrho;
            s->p0[q] = d[3] / (s->dimrho * s->dimc * s->dimc);
        }
        s->g[k] = d[4] * s->diml / (s->dimc * s->dimc);
    }
    if (cmul)
        for (size_t q = 0; q < N; q++) s->c_speed[q] *= cmul[q];
    for (size_t q = 0; q < N; q++) s->c2[q] = s->c_speed[q] * s->c_speed[q];

    /* unstretch = dbyd2(z, ibc=1), stretch = 1/unstretch, initialize.f90:466-470 */
    orc_dbyd2(s->unstretch, s->z, 1, nz, 1);
    for (int k = 0; k < nz; k++) s->stretch[k] = 1.0 / s->unstretch[k];
    s->deltat = prm->timestep * s->dimc / s->diml; /* initialize.f90:474 */

    /* INITIALIZE_STEP, step.f90:24-41; optimals(3:5) are single-precision literals */
    double opt[5];
    opt[0] = 1.0; opt[1] = 0.5;
    opt[2] = (double)0.1665579725791151184f;
    opt[3] = (double)0.03950410250586729987f;
    opt[4] = (double)0.007810706393337838236f;
    s->betas[4] = opt[1];
    s->betas[3] = opt[2] / s->betas[4];
    s->betas[2] = opt[3] / (s->betas[4] * s->betas[3]);
    s->betas[1] = opt[4] / (s->betas[4] * s->betas[3] * s->betas[2]);
    s->betas[0] = 0.0;
    for (int r = 0; r < 5; r++) s->betas[r] *= s->deltat;

    /* mp_Initialize_RHS_2d, physics2d.f90:23-405 */
    double temp2 = 1.0 + prm->excitdep / ORC_RSUN, tmin = 1.0;
    for (int k = 0; k < nz; k++)
        if (fabs(s->z[k] - temp2) <= tmin) { tmin = fabs(s->z[k] - temp2); s->e_rad = k; }
    double temp_r = 1.0 + prm->obsheight / ORC_RSUN;
    tmin = 1.0;
    for (int k = 0; k < nz; k++)
        if (fabs(s->z[k] - temp_r) <= tmin) { tmin = fabs(s->z[k] - temp_r); s->o_rad = k; }
    if (prm->adjoint) s->delta_width = 2.0 / (s->z[s->o_rad + 1] - s->z[s->o_rad - 1]);
    else s->delta_width = 2.0 / (s->z[s->e_rad + 1] - s->z[s->e_rad - 1]);

    for (size_t q = 0; q < N; q++) {
        s->rhoinv[q] = 1.0 / s->rho0[q];
        s->c2rho0[q] = s->c2[q] * s->rho0[q];
    }
    orc_ddz(s, s->rho0, s->gradrho0_z, 1);
    orc_ddz(s, s->p0, s->gradp0_z, 1);

    /* PML, physics2d.f90:288-332 (0.005 is a single-precision literal) */
    {
        int nb = prm->npmlbot, nt = prm->npmltop;
        double l005 = (double)0.005f;
        double *tempin = s->tmp1;
        for (size_t q = 0; q < N; q++) tempin[q] = sqrt(s->c2[q]);
        for (int k = 0; k < nz; k++) {
            double alphaz = ORC_PI * l005 * s->diml / s->dimc;
            for (int i = 0; i < nx; i++) {
                size_t q = (size_t)k * nx + i;
                double dampz = 0.0, fd;
                double alk = alphaz;
                if (k < nb) {
                    alk = ORC_PI * l005 * s->diml / s->dimc * (s->z[k] - s->z[0]) / (s->z[nb - 1] - s->z[0]);
                    double rr = (s->z[nb - 1] - s->z[k]) / (s->z[nb - 1] - s->z[0]);
                    dampz = 3. * 3. * tempin[i] / (s->z[nb - 1] - s->z[0]) * (rr * rr);
                    fd = alk / (dampz + alk);
                    s->gradp0_z[q] *= fd;
                    s->gradrho0_z[q] *= fd;
                    if (i == 0) s->g[k] *= fd;
                }
                if (k > nz - nt - 1) {
                    alk = ORC_PI * l005 * s->diml / s->dimc * (s->z[nz - 1] - s->z[k]) /
                          (s->z[nz - 1] - s->z[nz - nt]);
                    double rr = (s->z[nz - nt] - s->z[k]) / (s->z[nz - 1] - s->z[nz - nt]);
                    dampz = 3. * 3. * tempin[(size_t)(nz - 6) * nx + i] / (s->z[nz - 1] - s->z[nz - nt]) * (rr * rr);
                    fd = alk / (dampz + alk);
                    s->gradp0_z[q] *= fd;
                    s->gradrho0_z[q] *= fd;
                    if (i == 0) s->g[k] *= fd;
                }
                s->bzpml[q] = -alk - dampz;
                s->az[q] = -dampz;
            }
        }
    }
    /* horizontal PML, physics2d.f90:335-357 */
    {
        int nh = prm->npmlhor;
        double l005 = (double)0.005f;
        const double *x = s->x;
        for (int k = 0; k < nz; k++) {
            double c1 = sqrt(s->c2[(size_t)k * nx + 0]);
            for (int i = 0; i < nh; i++) {
                double rr = (x[i] - x[nh - 1]) / (x[nh - 1] - x[0]);
                double ax = -0.25 * 3. * 3. * c1 / (x[nh - 1] - x[0]) * (rr * rr);
                s->axpml[(size_t)k * s->nhx + i] = ax;
                s->bxpml[(size_t)k * s->nhx + i] = ax - l005 * s->diml / s->dimc * ORC_PI * (x[i] - x[0]) / (x[nh - 1] - x[0]);
            }
            int counter = nh;
            for (int i = nx - nh; i < nx; i++) {
                double rr = (x[nx - nh] - x[i]) / (x[nx - nh] - x[nx - 1]);
                double ax = -0.25 * 3. * 3. * c1 / (x[nx - 1] - x[nx - nh]) * (rr * rr);
                s->axpml[(size_t)k * s->nhx + counter] = ax;
                s->bxpml[(size_t)k * s->nhx + counter] =
                    ax - l005 * s->diml / s->dimc * ORC_PI * (x[nx - 1] - x[i]) / (x[nx - 1] - x[nx - nh]);
                counter++;
            }
        }
    }
    s->time = 0;
    return s;
}

void orc_destroy(orc_sim *s)
{
    if (!s) return;
    double *ptrs[] = {s->fre, s->fim, s->ftr, s->fti, s->z, s->x, s->stretch, s->unstretch, s->g,
                      s->c_speed, s->c2, s->rho0, s->p0, s->rhoinv, s->c2rho0, s->gradrho0_z, s->gradp0_z,
                      s->az, s->bzpml, s->axpml, s->bxpml, s->v0x, s->v0z, s->a, s->temp, s->scr,
                      s->pmlvars, s->psipml, s->scrpml, s->pmlvarsx, s->psipmlx, s->scrpmlx,
                      s->dxixdx, s->dxizdz, s->div, s->pp, s->rho, s->gradp_x, s->gradp_z, s->tmp1, s->tmp2,
                      s->kappa, s->forcing, s->vr, s->fwdsource, s->box, s->boz, s->curlboy, s->pmlm,
                      s->psipmlm, s->scrpmlm, s->flux, s->bxp, s->bzp, s->dzbx, s->curlby};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++) free(ptrs[i]);
    fft_free(&s->fft);
    free(s);
}

/* Flow from the stream function, driver.f90:94-147: psi in Mm (nx*nz, x fastest).
 * psivar = rho0 c psi / (diml/1e8); v0x = -ddz(psivar,1)/rho0; v0z = ddx(psivar)/rho0;
 * the adjoint run negates the flow (driver.f90:144-147). */
int orc_set_psi(orc_sim *s, const double *psi)
{
    size_t N = (size_t)s->nx * s->nz;
    double *pv = s->tmp1;
    for (size_t q = 0; q < N; q++) pv[q] = s->rho0[q] * sqrt(s->c2[q]) * (psi[q] / (s->diml / 1.0e8));
    orc_ddz(s, pv, s->v0x, 1);
    for (size_t q = 0; q < N; q++) s->v0x[q] = -s->v0x[q] / s->rho0[q];
    orc_ddx_rows(s, pv, s->v0z, s->nz);
    for (size_t q = 0; q < N; q++) s->v0z[q] = s->v0z[q] / s->rho0[q];
    if (s->p.adjoint)
        for (size_t q = 0; q < N; q++) { s->v0x[q] = -s->v0x[q]; s->v0z[q] = -s->v0z[q]; }
    return 0;
}

/* Direct flow (nondimensional units, same sign convention as v0 after orc_set_psi). */
int orc_set_flow(orc_sim *s, const double *v0x, const double *v0z)
{
    size_t N = (size_t)s->nx * s->nz;
    memcpy(s->v0x, v0x, N * sizeof(double));
    memcpy(s->v0z, v0z, N * sizeof(double));
    return 0;
}

/* Forward source.  Spatial profile (driver.f90:536-553): kind 0 = reference
 * exp(-d^2/(400 dx^2)) sinc(0.43 pi d), kind 1 = Gaussian exp(-d^2/(2 sigma^2)).
 * Temporal (driver.f90:1120-1145): kind 0 = reference cos * Gaussian, kind 1 = Ricker
 * wavelet with peak frequency nu0 (Hz), centred at 1.5/nu0 (no thresholding).  xloc, sigma
 * in Mm. */
int orc_set_forward_source(orc_sim *s, double xloc, int spatial_kind, double sigma_mm,
                           int temporal_kind, double nu0, int nt)
{
    int nx = s->nx;
    free(s->vr); free(s->fwdsource);
    s->vr = zalloc(nx); s->nvr = 1;
    s->fwdsource = zalloc(nt); s->nfwd = nt;
    double l1e8 = (double)1e-8f; /* 10.**(-8) is a single-precision constant, driver.f90:545-546 */
    double dx = (s->x[1] - s->x[0]) * s->p.xlength * l1e8;
    double *xdist = s->tmp1;
    int imin = 0;
    for (int i = 0; i < nx; i++) {
        xdist[i] = (s->x[i] - 0.5) * s->p.xlength * l1e8 - xloc;
        if (fabs(xdist[i]) < fabs(xdist[imin])) imin = i;
    }
    double l043 = (double)0.43f;
    for (int i = 0; i < nx; i++) {
        if (spatial_kind == 0) {
            double sx = sin(l043 * ORC_PI * xdist[i]) / (l043 * ORC_PI * xdist[i]);
            if (i == imin) sx = 1.0;
            s->vr[i] = exp(-(xdist[i] * xdist[i]) / (400. * (dx * dx))) * sx;
        } else {
            s->vr[i] = exp(-(xdist[i] * xdist[i]) / (2.0 * sigma_mm * sigma_mm));
        }
    }
    double nupeak = (double)0.0017f, nuwidth = (double)0.0055f; /* params.i:66 */
    for (int k = 0; k < nt; k++) {
        double ttime = (double)k * s->p.timestep;
        double v;
        if (temporal_kind == 0) {
            double dd = ttime - 0.5 / nupeak;
            v = cos(2. * ORC_PI * nupeak * ttime) * exp(-2. * (dd * dd) * (nuwidth * nuwidth));
            if (fabs(v) < (double)0.00001f) v = 0.0;
            v *= (double)1e-5f;
        } else {
            double arg = ORC_PI * nu0 * (ttime - 1.5 / nu0);
            v = (1.0 - 2.0 * arg * arg) * exp(-arg * arg) * 1e-5;
        }
        s->fwdsource[k] = v;
    }
    return 0;
}

/* Adjoint source: src is forcing_length rows of nx values at cadforcing cadence
 * (driver.f90:584-594: vr(nx,1,forcing_length+8), zero padded). */
int orc_set_adjoint_source(orc_sim *s, const double *src, int forcing_length, int num_steps)
{
    free(s->vr);
    s->nvr = forcing_length + 8;
    s->vr = zalloc((size_t)s->nx * s->nvr);
    memcpy(s->vr, src, sizeof(double) * (size_t)s->nx * forcing_length);
    s->num_steps = num_steps;
    return 0;
}

/* LAGRANGE_INTERP, physics.f90:678-737 (7-point Lagrange in time) */
static void orc_lagrange(orc_sim *s)
{
    double cad = s->p.cadforcing, ts = s->p.timestep;
    double xt = (double)s->time * ts / cad;
    int time1 = (int)floor(xt) + 1;
    xt = s->time * ts;
    double xs[7];
    for (int j = 0; j < 7; j++) xs[j] = (double)(time1 - 4 + j) * cad;
    int use[7];
    for (int j = 0; j < 4; j++) use[j] = xs[j] >= 0;
    use[4] = 1;
    use[5] = time1 < s->num_steps;
    use[6] = time1 < s->num_steps - 1;
    for (int i = 0; i < s->nx; i++) s->forcing[i] = 0.0;
    for (int j = 0; j < 7; j++) {
        if (!use[j]) continue;
        double den = 1.0, num = 1.0;
        for (int m = 0; m < 7; m++) if (m != j) { den *= (xs[j] - xs[m]); num *= (xt - xs[m]); }
        int idx = time1 - 4 + j; /* Fortran vr(:,:,time1-3+j) -> 0-based time1-4+j */
        if (idx < 0 || idx >= s->nvr) continue;
        for (int i = 0; i < s->nx; i++) s->forcing[i] += s->vr[(size_t)idx * s->nx + i] / den * num;
    }
}

/* ------------------------------------------------------------------------- */
/* MP_QUIET_PML_2D_DISPL, physics2d.f90:943-1094                              */
/* ------------------------------------------------------------------------- */
static inline int pml_index(const orc_sim *s, int k)
{
    if (k < s->p.npmlbot) return k;
    if (k >= s->nz - s->p.npmltop) return s->p.npmlbot + (k - (s->nz - s->p.npmltop));
    return -1;
}

static void orc_rhs(orc_sim *s)
{
    int nx = s->nx, nz = s->nz, nh = s->p.npmlhor, nhx = s->nhx;
    size_t N = (size_t)nx * nz;
    const double *T = s->temp;
    const double *xi_x = T, *xi_z = T + 2 * N, *v_x = T + 3 * N, *v_z = T + 5 * N;
    double *S = s->scr;
    double *RHSxi_x = S, *RHSxi_z = S + 2 * N, *RHSv_x = S + 3 * N, *RHSv_z = S + 5 * N;
    double *psivz = s->psipml, *psip = s->psipml + (size_t)nx * s->nzpml;
    double *RHSpsivz = s->scrpml, *RHSpsip = s->scrpml + (size_t)nx * s->nzpml;
    double *psivx = s->psipmlx, *psi_gradp_x = s->psipmlx + (size_t)nhx * nz;
    double *RHSpsivx = s->scrpmlx, *RHS_psi_gradp_x = s->scrpmlx + (size_t)nhx * nz;
    double *dxixdx = s->dxixdx, *dxizdz = s->dxizdz;

    orc_ddx_rows(s, xi_x, dxixdx, nz);
    for (int i = 0; i < nx; i++) dxizdz[(size_t)(nz - 1) * nx + i] = -dxixdx[(size_t)(nz - 1) * nx + i] * s->unstretch[nz - 1];
    orc_ddz(s, xi_z, dxizdz, 3);
    for (int k = 0; k < nz; k++) {
        int pi = pml_index(s, k);
        if (pi < 0) continue;
        for (int i = 0; i < nx; i++) {
            size_t q = (size_t)k * nx + i, qp = (size_t)pi * nx + i;
            RHSpsivz[qp] = s->az[q] * dxizdz[q] + s->bzpml[q] * psivz[qp];
            dxizdz[q] = dxizdz[q] + psivz[qp];
        }
    }
    for (int k = 0; k < nz; k++)
        for (int i = 0; i < nh; i++) {
            size_t ql = (size_t)k * nx + i, qr = (size_t)k * nx + (nx - nh + i);
            size_t al = (size_t)k * nhx + i, ar = (size_t)k * nhx + i + nh;
            dxixdx[ql] = dxixdx[ql] + psivx[al];
            RHSpsivx[al] = s->axpml[al] * dxixdx[ql] + s->bxpml[al] * psivx[al];
            dxixdx[qr] = dxixdx[qr] + psivx[ar];
            RHSpsivx[ar] = s->axpml[ar] * dxixdx[qr] + s->bxpml[ar] * psivx[ar];
        }
    for (size_t q = 0; q < N; q++) {
        s->div[q] = dxixdx[q] + dxizdz[q];
        s->pp[q] = -s->c2rho0[q] * s->div[q] - s->gradp0_z[q] * xi_z[q];
    }
    orc_ddx_rows(s, s->pp, s->gradp_x, nz);
    for (int k = 0; k < nz; k++)
        for (int i = 0; i < nh; i++) {
            size_t ql = (size_t)k * nx + i, qr = (size_t)k * nx + (nx - nh + i);
            size_t al = (size_t)k * nhx + i, ar = (size_t)k * nhx + i + nh;
            s->gradp_x[ql] = s->gradp_x[ql] + psi_gradp_x[al];
            RHS_psi_gradp_x[al] = s->axpml[al] * s->gradp_x[ql] + s->bxpml[al] * psi_gradp_x[al];
            s->gradp_x[qr] = s->gradp_x[qr] + psi_gradp_x[ar];
            RHS_psi_gradp_x[ar] = s->axpml[ar] * s->gradp_x[qr] + s->bxpml[ar] * psi_gradp_x[ar];
        }
    /* ddz(p, gradp_z, 2): gradp_z(:,:,1) keeps its previous value (physics2d.f90:1023) */
    orc_ddz(s, s->pp, s->gradp_z, 2);
    for (int k = 0; k < nz; k++) {
        int pi = pml_index(s, k);
        if (pi < 0) continue;
        for (int i = 0; i < nx; i++) {
            size_t q = (size_t)k * nx + i, qp = (size_t)pi * nx + i;
            RHSpsip[qp] = s->az[q] * s->gradp_z[q] + s->bzpml[q] * psip[qp];
            s->gradp_z[q] = s->gradp_z[q] + psip[qp];
        }
    }
    for (size_t q = 0; q < N; q++) RHSv_x[q] = -s->rhoinv[q] * s->gradp_x[q];
    for (size_t q = 0; q < N; q++) s->rho[q] = -s->rho0[q] * s->div[q] - s->gradrho0_z[q] * xi_z[q];
    for (int k = 0; k < nz; k++)
        for (int i = 0; i < nx; i++) {
            size_t q = (size_t)k * nx + i;
            RHSv_z[q] = -s->rhoinv[q] * (s->gradp_z[q] + s->rho[q] * s->g[k]);
        }
    memcpy(RHSxi_x, v_x, N * sizeof(double));
    memcpy(RHSxi_z, v_z, N * sizeof(double));
    if (s->time <= s->p.src_until) {
        if (s->p.adjoint) {
            int k = s->o_rad;
            for (int i = 0; i < nx; i++)
                RHSv_z[(size_t)k * nx + i] += s->forcing[i] * s->delta_width / s->rho0[(size_t)k * nx + i];
        } else {
            int k = s->e_rad;
            double fs = (s->time < s->nfwd) ? s->fwdsource[s->time] : 0.0; /* fwdsource(time+1) */
            for (int i = 0; i < nx; i++)
                RHSv_z[(size_t)k * nx + i] += s->vr[i] * fs * s->delta_width / s->rho0[(size_t)k * nx + i];
        }
    }
    if (s->p.flows) {
        double *d = s->tmp2;
        orc_ddx_rows(s, v_x, d, nz);
        for (size_t q = 0; q < N; q++) RHSv_x[q] = RHSv_x[q] - 2. * s->v0x[q] * d[q];
        orc_ddz(s, v_x, d, 1);
        for (size_t q = 0; q < N; q++) RHSv_x[q] = RHSv_x[q] - 2. * s->v0z[q] * d[q];
        orc_ddx_rows(s, v_z, d, nz);
        for (size_t q = 0; q < N; q++) RHSv_z[q] = RHSv_z[q] - 2. * s->v0x[q] * d[q];
        orc_ddz(s, v_z, d, 1);
        for (size_t q = 0; q < N; q++) RHSv_z[q] = RHSv_z[q] - 2. * s->v0z[q] * d[q];
    }
    for (int i = 0; i < nx; i++) { RHSv_x[i] = 0.; RHSv_z[i] = 0.; RHSxi_x[i] = 0.; RHSxi_z[i] = 0.; }
    for (int l = 0; l < 6; l++)
        for (int k = 0; k < nz; k++) {
            S[l * N + (size_t)k * nx + 0] = 0.0;
            S[l * N + (size_t)k * nx + nx - 1] = 0.0;
        }
}

/* Option 18: the background field (nx * nz, B / dimb, initialize.f90:759) and
 * curlboy = d box/dz - d boz/dx (physics2d.f90:166-168); switches the step to MP_MHD_PML_2D_DISPL.
 * The flow must be off (magnetic and flows exclude each other, PARSE_OPTIONS). */
int orc_set_magnetic(orc_sim *s, const double *box, const double *boz)
{
    const size_t N = (size_t)s->nx * s->nz, Np = 2 * (size_t)s->nx * s->nzpml;
    if (s->p.flows) return -1;
    if (!s->magnetic) {
        s->box = zalloc(N); s->boz = zalloc(N); s->curlboy = zalloc(N);
        s->pmlm = zalloc(Np); s->psipmlm = zalloc(Np); s->scrpmlm = zalloc(Np);
        s->flux = zalloc(N); s->bxp = zalloc(N); s->bzp = zalloc(N); s->dzbx = zalloc(N); s->curlby = zalloc(N);
        s->magnetic = 1;
    }
    memcpy(s->box, box, N * sizeof(double));
    memcpy(s->boz, boz, N * sizeof(double));
    orc_ddz(s, s->box, s->curlboy, 1);
    orc_ddx_rows(s, s->boz, s->tmp1, s->nz);
    for (size_t q = 0; q < N; q++) s->curlboy[q] -= s->tmp1[q];
    return 0;
}

/* MP_MHD_PML_2D_DISPL (physics2d.f90:719-938): the displacement formulation with the background
 * field.  As orc_rhs for div xi (ibc 3 with the top preset), the PMLs of psi_vz, psi_vx, p with
 * d p/dz at ibc 0 (both boundary rows zero, where option 17 uses ibc 2); the field perturbation
 * b_x = -(d flux2/dz + psi), b_z = d flux2/dx of flux2 = -(xi_x boz - xi_z box); curl b =
 * d b_x/dz (+ psi) - d b_z/dx; the Lorentz force (curl b boz + curlboy b_z, -curl b box -
 * curlboy b_x) / rho0; the source as option 17; the bottom row and the first and last columns of
 * the RHS zero (the top row is not, physics2d.f90:928-935).  The background is laterally
 * uniform: gradp0_x = gradrho0_x = 0. */
static void orc18_rhs(orc_sim *s)
{
    int nx = s->nx, nz = s->nz, nh = s->p.npmlhor, nhx = s->nhx;
    size_t N = (size_t)nx * nz, P = (size_t)nx * s->nzpml;
    const double *T = s->temp;
    const double *xi_x = T, *xi_z = T + 2 * N, *v_x = T + 3 * N, *v_z = T + 5 * N;
    double *S = s->scr;
    double *RHSv_x = S + 3 * N, *RHSv_z = S + 5 * N;
    double *psivz = s->psipml, *psip = s->psipml + P;
    double *RHSpsivz = s->scrpml, *RHSpsip = s->scrpml + P;
    double *psivx = s->psipmlx, *psi_gradp_x = s->psipmlx + (size_t)nhx * nz;
    double *RHSpsivx = s->scrpmlx, *RHS_psi_gradp_x = s->scrpmlx + (size_t)nhx * nz;
    double *psiind = s->psipmlm, *psidzbx = s->psipmlm + P;
    double *RHSpsiind = s->scrpmlm, *RHSpsidzbx = s->scrpmlm + P;
    double *dxixdx = s->dxixdx, *dxizdz = s->dxizdz;

    orc_ddx_rows(s, xi_x, dxixdx, nz);
    for (int i = 0; i < nx; i++) dxizdz[(size_t)(nz - 1) * nx + i] = -dxixdx[(size_t)(nz - 1) * nx + i] * s->unstretch[nz - 1];
    orc_ddz(s, xi_z, dxizdz, 3);
    for (int k = 0; k < nz; k++) {
        int pi = pml_index(s, k);
        if (pi < 0) continue;
        for (int i = 0; i < nx; i++) {
            size_t q = (size_t)k * nx + i, qp = (size_t)pi * nx + i;
            RHSpsivz[qp] = s->az[q] * dxizdz[q] + s->bzpml[q] * psivz[qp];
            dxizdz[q] = dxizdz[q] + psivz[qp];
        }
    }
    for (int k = 0; k < nz; k++)
        for (int i = 0; i < nh; i++) {
            size_t ql = (size_t)k * nx + i, qr = (size_t)k * nx + (nx - nh + i);
            size_t al = (size_t)k * nhx + i, ar = (size_t)k * nhx + i + nh;
            dxixdx[ql] = dxixdx[ql] + psivx[al];
            RHSpsivx[al] = s->axpml[al] * dxixdx[ql] + s->bxpml[al] * psivx[al];
            dxixdx[qr] = dxixdx[qr] + psivx[ar];
            RHSpsivx[ar] = s->axpml[ar] * dxixdx[qr] + s->bxpml[ar] * psivx[ar];
        }
    for (size_t q = 0; q < N; q++) {
        s->div[q] = dxixdx[q] + dxizdz[q];
        s->pp[q] = -s->c2rho0[q] * s->div[q] - s->gradp0_z[q] * xi_z[q];
        s->rho[q] = -s->rho0[q] * s->div[q] - s->gradrho0_z[q] * xi_z[q];
    }
    orc_ddx_rows(s, s->pp, s->gradp_x, nz);
    memset(s->gradp_z, 0, N * sizeof(double));
    orc_ddz(s, s->pp, s->gradp_z, 0);
    for (int k = 0; k < nz; k++) {
        int pi = pml_index(s, k);
        if (pi < 0) continue;
        for (int i = 0; i < nx; i++) {
            size_t q = (size_t)k * nx + i, qp = (size_t)pi * nx + i;
            RHSpsip[qp] = s->az[q] * s->gradp_z[q] + s->bzpml[q] * psip[qp];
            s->gradp_z[q] = s->gradp_z[q] + psip[qp];
        }
    }
    for (int k = 0; k < nz; k++)
        for (int i = 0; i < nh; i++) {
            size_t ql = (size_t)k * nx + i, qr = (size_t)k * nx + (nx - nh + i);
            size_t al = (size_t)k * nhx + i, ar = (size_t)k * nhx + i + nh;
            s->gradp_x[ql] = s->gradp_x[ql] + psi_gradp_x[al];
            RHS_psi_gradp_x[al] = s->axpml[al] * s->gradp_x[ql] + s->bxpml[al] * psi_gradp_x[al];
            s->gradp_x[qr] = s->gradp_x[qr] + psi_gradp_x[ar];
            RHS_psi_gradp_x[ar] = s->axpml[ar] * s->gradp_x[qr] + s->bxpml[ar] * psi_gradp_x[ar];
        }
    for (size_t q = 0; q < N; q++) s->flux[q] = -(xi_x[q] * s->boz[q] - xi_z[q] * s->box[q]);
    orc_ddz(s, s->flux, s->bxp, 0);
    orc_ddx_rows(s, s->flux, s->bzp, nz);
    for (int k = 0; k < nz; k++) {
        int pi = pml_index(s, k);
        if (pi < 0) continue;
        for (int i = 0; i < nx; i++) {
            size_t q = (size_t)k * nx + i, qp = (size_t)pi * nx + i;
            RHSpsiind[qp] = s->az[q] * s->bxp[q] + s->bzpml[q] * psiind[qp];
            s->bxp[q] = s->bxp[q] + psiind[qp];
        }
    }
    for (size_t q = 0; q < N; q++) s->bxp[q] = -s->bxp[q];
    orc_ddz(s, s->bxp, s->dzbx, 0);
    orc_ddx_rows(s, s->bzp, s->curlby, nz);
    for (int k = 0; k < nz; k++) {
        int pi = pml_index(s, k);
        if (pi < 0) continue;
        for (int i = 0; i < nx; i++) {
            size_t q = (size_t)k * nx + i, qp = (size_t)pi * nx + i;
            RHSpsidzbx[qp] = s->az[q] * s->dzbx[q] + s->bzpml[q] * psidzbx[qp];
            s->dzbx[q] = s->dzbx[q] + psidzbx[qp];
        }
    }
    for (int k = 0; k < nz; k++)
        for (int i = 0; i < nx; i++) {
            size_t q = (size_t)k * nx + i;
            const double cb = -s->curlby[q] + s->dzbx[q];
            RHSv_x[q] = s->rhoinv[q] * (-s->gradp_x[q] + cb * s->boz[q]);
            RHSv_z[q] = s->rhoinv[q] * (-s->gradp_z[q] - cb * s->box[q]);
            RHSv_x[q] = RHSv_x[q] + s->rhoinv[q] * (s->curlboy[q] * s->bzp[q]);
            RHSv_z[q] = RHSv_z[q] + s->rhoinv[q] * (-s->curlboy[q] * s->bxp[q]);
            RHSv_z[q] = RHSv_z[q] - s->rhoinv[q] * s->rho[q] * s->g[k];
        }
    memcpy(S, v_x, N * sizeof(double));
    memcpy(S + 2 * N, v_z, N * sizeof(double));
    if (s->time <= s->p.src_until) {
        if (s->p.adjoint) {
            int k = s->o_rad;
            for (int i = 0; i < nx; i++)
                RHSv_z[(size_t)k * nx + i] += s->forcing[i] * s->delta_width / s->rho0[(size_t)k * nx + i];
        } else {
            int k = s->e_rad;
            double fs = (s->time < s->nfwd) ? s->fwdsource[s->time] : 0.0;
            for (int i = 0; i < nx; i++)
                RHSv_z[(size_t)k * nx + i] += s->vr[i] * fs * s->delta_width / s->rho0[(size_t)k * nx + i];
        }
    }
    for (int l = 0; l < 6; l++) {
        memset(S + (size_t)l * N, 0, nx * sizeof(double));
        for (int k = 0; k < nz; k++) {
            S[l * N + (size_t)k * nx + 0] = 0.0;
            S[l * N + (size_t)k * nx + nx - 1] = 0.0;
        }
    }
}

/* FILTER_VARS_2D, physics2d.f90:509-583 (HORIZONTAL_PMLS: x-FFT filter skipped) */
static void orc_filter_vars_2d(orc_sim *s)
{
    int nx = s->nx, nz = s->nz, nh = s->p.npmlhor;
    size_t N = (size_t)nx * nz;
    static const double c[6] = {0.75390625000000, 0.41015625000000, -0.23437500000000,
                                0.08789062500000, -0.01953125000000, 0.00195312500000};
    double *temp = s->tmp1;
    for (int l = 0; l < 6; l++) {
        double *a = s->a + l * N;
#define A_(k, i) a[(size_t)(k) * nx + (i)]
#define T_(k, i) temp[(size_t)(k) * nx + (i)]
        for (int k = 5; k <= nz - 6; k++)
            for (int i = 0; i < nx; i++)
                T_(k, i) = c[0] * A_(k, i) + 0.5 * c[1] * (A_(k - 1, i) + A_(k + 1, i)) +
                           0.5 * c[2] * (A_(k - 2, i) + A_(k + 2, i)) + 0.5 * c[3] * (A_(k - 3, i) + A_(k + 3, i)) +
                           0.5 * c[4] * (A_(k - 4, i) + A_(k + 4, i)) + 0.5 * c[5] * (A_(k - 5, i) + A_(k + 5, i));
        for (int i = 0; i < nx; i++) {
            T_(nz - 5, i) = 0.5 * (A_(nz - 4, i) + A_(nz - 6, i));
            T_(nz - 4, i) = 0.5 * (A_(nz - 3, i) + A_(nz - 5, i));
            T_(nz - 3, i) = 0.5 * (A_(nz - 2, i) + A_(nz - 4, i));
            T_(nz - 2, i) = 0.5 * (A_(nz - 1, i) + A_(nz - 3, i));
        }
        for (int i = 0; i < nx; i++) { /* temp(2..5) under USE_PML, physics2d.f90:539-544 */
            T_(1, i) = 0.5 * (A_(2, i) + A_(0, i));
            T_(2, i) = 0.5 * (A_(3, i) + A_(1, i));
            T_(3, i) = 0.5 * (A_(4, i) + A_(2, i));
            T_(4, i) = 0.5 * (A_(5, i) + A_(3, i));
        }
        int kst = s->p.filter_kst > 0 ? s->p.filter_kst : 6;
        int i0 = s->p.filter_all_x ? 0 : nh - 1, i1 = s->p.filter_all_x ? nx - 1 : nx - nh;
        for (int k = kst - 1; k <= nz - 2; k++) /* kst .. nz-1 (1-based) */
            for (int i = i0; i <= i1; i++) A_(k, i) = T_(k, i);
#undef A_
#undef T_
    }
}

/* FILTER_VARS_2D alone on the current state (for the tests). */
void orc_apply_filter(orc_sim *s) { orc_filter_vars_2d(s); }

/* STEP, step.f90:43-119 */
void orc_step(orc_sim *s)
{
    size_t N6 = 6 * (size_t)s->nx * s->nz;
    size_t Np = 2 * (size_t)s->nx * s->nzpml, Nx = 2 * (size_t)s->nhx * s->nz;
    size_t Nm = s->magnetic ? Np : 0;
    if (s->p.adjoint && s->time <= s->p.src_until) orc_lagrange(s); /* driver.f90:359-360 */
    for (int rk = 0; rk < 5; rk++) {
        if (rk == 0) {
            memcpy(s->temp, s->a, N6 * sizeof(double));
            memcpy(s->psipml, s->pmlvars, Np * sizeof(double));
            memcpy(s->psipmlx, s->pmlvarsx, Nx * sizeof(double));
            if (Nm) memcpy(s->psipmlm, s->pmlm, Nm * sizeof(double));
        } else {
            double b = s->betas[rk];
            for (size_t q = 0; q < N6; q++) s->temp[q] = s->a[q] + b * s->scr[q];
            for (size_t q = 0; q < Np; q++) s->psipml[q] = s->pmlvars[q] + b * s->scrpml[q];
            for (size_t q = 0; q < Nx; q++) s->psipmlx[q] = s->pmlvarsx[q] + b * s->scrpmlx[q];
            for (size_t q = 0; q < Nm; q++) s->psipmlm[q] = s->pmlm[q] + b * s->scrpmlm[q];
        }
        if (s->magnetic) orc18_rhs(s);
        else orc_rhs(s);
    }
    for (size_t q = 0; q < N6; q++) s->a[q] = s->a[q] + s->deltat * s->scr[q];
    for (size_t q = 0; q < Np; q++) s->pmlvars[q] = s->pmlvars[q] + s->deltat * s->scrpml[q];
    for (size_t q = 0; q < Nm; q++) s->pmlm[q] = s->pmlm[q] + s->deltat * s->scrpmlm[q];
    orc_filter_vars_2d(s);
    for (size_t q = 0; q < Nx; q++) s->pmlvarsx[q] = s->pmlvarsx[q] + s->deltat * s->scrpmlx[q];
}

/* TIMESTEPPING, driver.f90:337-475: run nsteps steps from the current time; after each
 * step whose index is a multiple of steps_out, append a(:,o_rad,v_z) to seis (nx values per
 * record) and, if snaps != NULL, the partial state of all_modules.f90:750-784 as six nx*nz
 * fields (xi_x, xi_z, v_x, v_z, acc_x = scr v_x, acc_z = scr v_z).  Returns the record count. */
int orc_run(orc_sim *s, int nsteps, double *seis, double *snaps)
{
    int nrec = 0, nx = s->nx;
    size_t N = (size_t)nx * s->nz;
    for (int it = 0; it < nsteps; it++) {
        orc_step(s);
        if (s->time % s->p.steps_out == 0) {
            if (seis)
                for (int i = 0; i < nx; i++) seis[(size_t)nrec * nx + i] = s->a[5 * N + (size_t)s->o_rad * nx + i];
            if (snaps) {
                double *o = snaps + (size_t)nrec * 6 * N;
                memcpy(o + 0 * N, s->a + 0 * N, N * sizeof(double));
                memcpy(o + 1 * N, s->a + 2 * N, N * sizeof(double));
                memcpy(o + 2 * N, s->a + 3 * N, N * sizeof(double));
                memcpy(o + 3 * N, s->a + 5 * N, N * sizeof(double));
                memcpy(o + 4 * N, s->scr + 3 * N, N * sizeof(double));
                memcpy(o + 5 * N, s->scr + 5 * N, N * sizeof(double));
            }
            nrec++;
        }
        s->time++;
    }
    return nrec;
}

/* ------------------------------------------------------------------------- */
/* Accessors                                                                  */
/* ------------------------------------------------------------------------- */
int orc_get_int(const orc_sim *s, const char *name)
{
    if (!strcmp(name, "e_rad")) return s->e_rad;
    if (!strcmp(name, "o_rad")) return s->o_rad;
    if (!strcmp(name, "time")) return s->time;
    if (!strcmp(name, "nx")) return s->nx;
    if (!strcmp(name, "nz")) return s->nz;
    return -1;
}

double orc_get_double(const orc_sim *s, const char *name)
{
    if (!strcmp(name, "deltat")) return s->deltat;
    if (!strcmp(name, "stretchx")) return s->stretchx;
    if (!strcmp(name, "delta_width")) return s->delta_width;
    if (!strncmp(name, "betas", 5)) return s->betas[name[5] - '0'];
    return NAN;
}

/* Copy a named array out (returns element count, or -1). */
long orc_get_array(const orc_sim *s, const char *name, double *out)
{
    size_t N = (size_t)s->nx * s->nz;
    const double *src = NULL;
    size_t n = 0;
#define GA(nm, ptr, cnt) if (!strcmp(name, nm)) { src = (ptr); n = (cnt); }
    GA("z", s->z, s->nz) GA("x", s->x, s->nx) GA("stretch", s->stretch, s->nz) GA("unstretch", s->unstretch, s->nz)
    GA("g", s->g, s->nz) GA("c2", s->c2, N) GA("rho0", s->rho0, N) GA("p0", s->p0, N) GA("rhoinv", s->rhoinv, N)
    GA("c2rho0", s->c2rho0, N) GA("gradrho0_z", s->gradrho0_z, N) GA("gradp0_z", s->gradp0_z, N)
    GA("az", s->az, N) GA("bzpml", s->bzpml, N) GA("axpml", s->axpml, (size_t)s->nhx * s->nz)
    GA("bxpml", s->bxpml, (size_t)s->nhx * s->nz) GA("v0x", s->v0x, N) GA("v0z", s->v0z, N)
    GA("a", s->a, 6 * N) GA("scr", s->scr, 6 * N) GA("pmlvars", s->pmlvars, 2 * (size_t)s->nx * s->nzpml)
    GA("pmlvarsx", s->pmlvarsx, 2 * (size_t)s->nhx * s->nz) GA("vr", s->vr, (size_t)s->nx * s->nvr)
    GA("fwdsource", s->fwdsource, (size_t)s->nfwd) GA("forcing", s->forcing, (size_t)s->nx)
    GA("kappa", s->kappa, (size_t)s->nx / 2 + 1)
#undef GA
    if (!src) return -1;
    if (out) memcpy(out, src, n * sizeof(double));
    return (long)n;
}

int orc_set_array(orc_sim *s, const char *name, const double *in)
{
    size_t N = (size_t)s->nx * s->nz;
    if (!strcmp(name, "a")) { memcpy(s->a, in, 6 * N * sizeof(double)); return 0; }
    if (!strcmp(name, "time")) { s->time = (int)in[0]; return 0; }
    return -1;
}

/* ------------------------------------------------------------------------- */
/* Kernel construction, kernels.f90:13-612 with helpers 648-928 (2-D, flows,   */
/* sound speed).  fsn: forward partial states, asn: adjoint partial states,     */
/* both as written by orc_run (6 fields per record).  Record j of the forward   */
/* (time fwd_start + 15 j) pairs with adjoint record adj_end/15 - j            */
/* (kernels.f90:215, 258).  Outputs (nx*nz each): kernel_c, kernel_vx,          */
/* kernel_vz, kernel_psi, hessian, already scaled as in kernels.f90:495-581.    */
/* The kernel stage reads its own background with kernel_back                  */
/* (initialize.f90:936-978: dimrho = 10.0**(-3.0), a single-precision value).   */
/* ------------------------------------------------------------------------- */
static void filter_var_z(orc_sim *s, double *var) /* kernels.f90:891-928 */
{
    int nx = s->nx, nz = s->nz;
    static const double c[6] = {0.75390625000000, 0.41015625000000, -0.23437500000000,
                                0.08789062500000, -0.01953125000000, 0.00195312500000};
    double *temp = s->tmp1;
#define V_(k, i) var[(size_t)(k) * nx + (i)]
#define T_(k, i) temp[(size_t)(k) * nx + (i)]
    for (int i = 0; i < nx; i++) {
        T_(1, i) = 0.5 * (V_(2, i) + V_(0, i));
        T_(2, i) = 0.5 * (V_(3, i) + V_(1, i));
        T_(3, i) = 0.5 * (V_(4, i) + V_(2, i));
        T_(4, i) = 0.5 * (V_(5, i) + V_(3, i));
    }
    for (int k = 5; k <= nz - 6; k++)
        for (int i = 0; i < nx; i++)
            T_(k, i) = c[0] * V_(k, i) + 0.5 * c[1] * (V_(k - 1, i) + V_(k + 1, i)) +
                       0.5 * c[2] * (V_(k - 2, i) + V_(k + 2, i)) + 0.5 * c[3] * (V_(k - 3, i) + V_(k + 3, i)) +
                       0.5 * c[4] * (V_(k - 4, i) + V_(k + 4, i)) + 0.5 * c[5] * (V_(k - 5, i) + V_(k + 5, i));
    for (int i = 0; i < nx; i++) {
        T_(nz - 5, i) = 0.5 * (V_(nz - 4, i) + V_(nz - 6, i));
        T_(nz - 4, i) = 0.5 * (V_(nz - 3, i) + V_(nz - 5, i));
        T_(nz - 3, i) = 0.5 * (V_(nz - 2, i) + V_(nz - 4, i));
        T_(nz - 2, i) = 0.5 * (V_(nz - 1, i) + V_(nz - 3, i));
    }
    for (int k = 1; k <= nz - 2; k++)
        for (int i = 0; i < nx; i++) V_(k, i) = T_(k, i);
#undef V_
#undef T_
}

static void ddzkern(orc_sim *s, const double *var, double *dvar, int bc) /* kernels.f90:648-661 */
{
    orc_ddz(s, var, dvar, bc);
    filter_var_z(s, dvar);
}

int orc_kernels(orc_sim *s, const double *fsn, int nf, const double *asn, int na, int nt_kern,
                double *kc, double *kvx, double *kvz, double *kpsi, double *hess)
{
    int nx = s->nx, nz = s->nz;
    size_t N = (size_t)nx * nz;
    double *kc2 = (double *)calloc(N, sizeof(double));
    double *kv1 = (double *)calloc(N, sizeof(double));
    double *kv3 = (double *)calloc(N, sizeof(double));
    double *hes = (double *)calloc(N, sizeof(double));
    double *t2 = (double *)malloc(N * sizeof(double));
    double *t3 = (double *)malloc(N * sizeof(double));
    double *tt = (double *)malloc(N * sizeof(double));
    double *d11 = (double *)malloc(N * sizeof(double)), *d13 = (double *)malloc(N * sizeof(double));
    double *d31 = (double *)malloc(N * sizeof(double)), *d33 = (double *)malloc(N * sizeof(double));
    /* kernel-stage background (kernel_back, initialize.f90:958-976) */
    double dimc = 1e6, dimrho = (double)1e-3f, diml = ORC_RSUN;
    double *rho0k = (double *)malloc(N * sizeof(double)), *c2k = (double *)malloc(N * sizeof(double));
    for (int k = 0; k < nz; k++)
        for (int i = 0; i < nx; i++) {
            size_t q = (size_t)k * nx + i;
            c2k[q] = s->c_speed[q] * s->dimc / dimc; /* model c (with the optional multiplier) */
            c2k[q] = c2k[q] * c2k[q];
            rho0k[q] = s->rho0[q] * s->dimrho / dimrho;
        }
    int adj_end_rec = na - 1;
    for (int k = 0; k < nt_kern; k++) {
        int jf = k, ja = adj_end_rec - k;
        if (jf >= nf || ja < 0) break;
        const double *F6 = fsn + (size_t)jf * 6 * N, *A6 = asn + (size_t)ja * 6 * N;
        const double *f_xi_x = F6, *f_xi_z = F6 + N, *f_vx = F6 + 2 * N, *f_vz = F6 + 3 * N;
        const double *f_acc_x = F6 + 4 * N, *f_acc_z = F6 + 5 * N;
        const double *a_vx = A6 + 2 * N, *a_vz = A6 + 3 * N;
        for (size_t q = 0; q < N; q++) hes[q] = hes[q] + f_acc_z[q] * f_acc_z[q] + f_acc_x[q] * f_acc_x[q];
        /* compute_div (kernels.f90:843-861) of forward xi and adjoint v */
        orc_ddx_rows(s, f_xi_x, t2, nz);
        ddzkern(s, f_xi_z, tt, 1);
        for (size_t q = 0; q < N; q++) t2[q] = t2[q] + tt[q];
        orc_ddx_rows(s, a_vx, t3, nz);
        ddzkern(s, a_vz, tt, 1);
        for (size_t q = 0; q < N; q++) t3[q] = t3[q] + tt[q];
        for (size_t q = 0; q < N; q++) kc2[q] = kc2[q] + t2[q] * t3[q];
        /* compute_del of forward v (kernels.f90:866-887) */
        orc_ddx_rows(s, f_vx, d11, nz);
        orc_ddx_rows(s, f_vz, d13, nz);
        ddzkern(s, f_vx, d31, 1);
        ddzkern(s, f_vz, d33, 1);
        for (size_t q = 0; q < N; q++) {
            kv1[q] = d11[q] * a_vx[q] + d13[q] * a_vz[q] + kv1[q];
            kv3[q] = d31[q] * a_vx[q] + d33[q] * a_vz[q] + kv3[q];
        }
    }
    double stepskern = (double)s->p.steps_out; /* floor(outputcad/timestep), kernels.f90:193 */
    double l1e8 = (double)1e-8f, l1e5 = (double)1e-5f;
    double dimen = 1.0 / (diml * l1e8 * s->p.xlength * l1e8 * dimc * l1e5); /* kernels.f90:502 */
    /* kernelpsi = curl_y(kernelv) with bcz = 0 (module default), kernels.f90:510-513 */
    orc_ddz(s, kv1, t2, 0);
    filter_var_z(s, t2);
    orc_ddx_rows(s, kv3, t3, nz);
    for (size_t q = 0; q < N; q++) {
        double cur = t2[q] - t3[q];
        kpsi[q] = 2.0 * cur * dimen * 1.0 * (rho0k[q] * sqrt(c2k[q])) * stepskern * s->p.timestep * dimen;
        kvx[q] = -2.0 * kv1[q] * rho0k[q] * stepskern * s->p.timestep * dimen;
        kvz[q] = -2.0 * kv3[q] * rho0k[q] * stepskern * s->p.timestep * dimen;
    }
    double dimc2 = 1.0 / (diml * l1e8 * s->p.xlength * l1e8); /* kernels.f90:555 */
    for (size_t q = 0; q < N; q++) {
        kc[q] = -kc2[q] * rho0k[q] * c2k[q] * stepskern * s->p.timestep * dimc2 * 2.0;
        hess[q] = hes[q];
    }
    free(kc2); free(kv1); free(kv3); free(hes); free(t2); free(t3); free(tt);
    free(d11); free(d13); free(d31); free(d33); free(rho0k); free(c2k);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Batch runner for the CPU baseline: nb independent forward solves, one per   */
/* thread (the reference runs one single-rank process per source).            */
/* ------------------------------------------------------------------------- */
int orc_run_batch(const orc_params *prm, const double *model, int nb, const double *xlocs,
                  const double *psi, int nsteps, int nthreads, double *seis_out)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int b = 0; b < nb; b++) {
        orc_sim *s = orc_create(prm, model, NULL);
        if (psi) orc_set_psi(s, psi);
        orc_set_forward_source(s, xlocs[b], 0, 0.5, 0, 0.003, nsteps + 8);
        int nrec = (nsteps - 1) / prm->steps_out + 1;
        orc_run(s, nsteps, seis_out ? seis_out + (size_t)b * nrec * prm->nx : NULL, NULL);
        orc_destroy(s);
    }
    (void)nthreads;
    return 0;
}
