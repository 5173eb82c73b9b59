/* sparc_oracle3d.c -- CPU FP64 oracle of the 3-D displacement step (test infrastructure).
 *
 * A plain-C restatement of the reference's 3-D option 16 (MP_FLOWS_PML_3D_DISPL), used only
 * by the tests as the checker of the GPU 3-D path (csrc/sparc_3d.cu).  Nothing in the product
 * links it.  Fields are [nz][ny][nx], x fastest (the Fortran a(nx,ny,nz) order); the state is
 * six such fields: xi_x, xi_y, xi_z, v_x, v_y, v_z.
 *
 * Followed lines:
 *   grid, eyekx/eyeky, stretchx/y     initialize.f90:195-226
 *   stretch = 1/dbyd2(z, 1)           initialize.f90:466-470
 *   solar_data (laterally uniform)    initialize.f90:731-794
 *   RK betas                          step.f90:24-41
 *   mp_Initialize_RHS                 physics.f90:34-404: e_rad / o_rad (44-62), source_dep
 *                                     (109), rhoinv, c2rho0, d rho0/dz, d p0/dz (204-208),
 *                                     vertical PML (255-295; 0.005 single precision)
 *   ddxyz                             derivatives.f90:175-305 (x, y by FFT, z by dbyd2)
 *   RHS                               displacement.f90:377-477
 *   STEP                              step.f90:43-119 with FILTER_VARS_3D_HORIZ_PML after
 *                                     every step whose index is odd (physics.f90:836-882,
 *                                     step.f90:114: HORIZONTAL_PMLS on, as params.i sets it)
 *   records                           driver.f90:388-409 (a(:,:,o_rad,6) every steps_out)
 *
 * Forcing.  In the reference's 3-D forward run the array `forcing` that the RHS injects
 * (forcing * source_dep(k) for |k - e_rad| <= 4, displacement.f90:456-462) is assigned only by
 * LAGRANGE_INTERP (physics.f90:678-737), i.e. in adjoint runs.  This restatement (and the GPU
 * path) takes forcing(x, y, t) = pattern(x, y) * amp(t) from the caller: pattern * fwdsource
 * for a forward run as the 2-D routine does (physics2d.f90:1056-1058), the interpolated
 * adjoint source for an adjoint run.
 *
 * Supported: laterally uniform background (sound speed, density, pressure as profiles in z),
 * 3-D flows v0 = (v0x, v0y, v0z) given as fields.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC3_PI 3.141592653589793 /* initialize.f90:42 */
#define ORC3_RSUN 6.95989467700e10

int orc_dbyd2(double *A, const double *B, int n1, int n2, int ibc);
void *orc_fft_new(int n);
void orc_fft_delete(void *f);
void orc_fft_exec(const void *f, double *re, double *im, double *tr, double *ti, int sign);

typedef struct {
    int nx, ny, nz;
    int npmlbot, npmltop;
    double xlength, ylength; /* cm */
    double timestep;         /* s */
    double excitdep, obsheight; /* cm */
    int steps_out;
    int filter_every; /* 2: FILTER_VARS_3D_HORIZ_PML after odd steps; 0: never */
} orc3_params;

typedef struct {
    orc3_params p;
    int nx, ny, nz, nzpml;
    size_t N;
    double dimc, dimrho, diml, deltat, stretchx, stretchy, betas[5];
    double *z, *stretch, *unstretch, *g, *source_dep;
    double *rho0, *p0, *c2, *rhoinv, *c2rho0, *gradrho0_z, *gradp0_z, *az, *bzpml; /* [nz] */
    double *v0x, *v0y, *v0z; /* [N] */
    int e_rad, o_rad;
    double *a, *temp, *scr;            /* 6 N */
    double *pmlvars, *psipml, *scrpml; /* 2 nx ny nzpml */
    double *d1, *d2, *d3, *div, *pp, *rho, *gpx, *gpy, *gpz;
    void *fx, *fy;
    double *fre, *fim, *ftr, *fti;
    double *pattern, *amp;
    int namp;
    /* kernel-mode adjoint source (displacement.f90:615-627): slices [nrows][ny][nx] and the
     * per-step LAGRANGE_INTERP table (physics.f90:678-737) */
    int adj, adj_nrows, adj_ntab;
    double *adj_rows, *adj_w, adj_scale;
    int *adj_idx;
    int time;
} orc3_sim;

static double *z3(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }

/* x-derivative of every row (derivatives.f90:218-235): r2c, times eyekx, c2r, times stretchx;
 * two rows per complex transform. */
static void d_x(orc3_sim *s, const double *var, double *dvar)
{
    const int nx = s->nx;
    const size_t nrows = (size_t)s->ny * s->nz;
    for (size_t r = 0; r < nrows; r += 2) {
        const int two = r + 1 < nrows;
        for (int i = 0; i < nx; i++) {
            s->fre[i] = var[r * nx + i];
            s->fim[i] = two ? var[(r + 1) * nx + i] : 0.0;
        }
        orc_fft_exec(s->fx, s->fre, s->fim, s->ftr, s->fti, -1);
        for (int k = 0; k < nx; k++) {
            double kap = 2 * k < nx ? (double)k / nx * 2.0 * ORC3_PI : (2 * k == nx ? 0.0 : -(double)(nx - k) / nx * 2.0 * ORC3_PI);
            const double re = s->fre[k], im = s->fim[k];
            s->fre[k] = -kap * im;
            s->fim[k] = kap * re;
        }
        orc_fft_exec(s->fx, s->fre, s->fim, s->ftr, s->fti, +1);
        for (int i = 0; i < nx; i++) {
            dvar[r * nx + i] = s->fre[i] * s->stretchx;
            if (two) dvar[(r + 1) * nx + i] = s->fim[i] * s->stretchx;
        }
    }
}

/* y-derivative (derivatives.f90:240-270, the transposed r2c / eyeky / c2r), times stretchy;
 * two x-columns per complex transform. */
static void d_y(orc3_sim *s, const double *var, double *dvar)
{
    const int nx = s->nx, ny = s->ny;
    for (int k = 0; k < s->nz; k++) {
        const double *v = var + (size_t)k * nx * ny;
        double *dv = dvar + (size_t)k * nx * ny;
        for (int i = 0; i < nx; i += 2) {
            const int two = i + 1 < nx;
            for (int j = 0; j < ny; j++) {
                s->fre[j] = v[(size_t)j * nx + i];
                s->fim[j] = two ? v[(size_t)j * nx + i + 1] : 0.0;
            }
            orc_fft_exec(s->fy, s->fre, s->fim, s->ftr, s->fti, -1);
            for (int q = 0; q < ny; q++) {
                double kap = 2 * q < ny ? (double)q / ny * 2.0 * ORC3_PI : (2 * q == ny ? 0.0 : -(double)(ny - q) / ny * 2.0 * ORC3_PI);
                const double re = s->fre[q], im = s->fim[q];
                s->fre[q] = -kap * im;
                s->fim[q] = kap * re;
            }
            orc_fft_exec(s->fy, s->fre, s->fim, s->ftr, s->fti, +1);
            for (int j = 0; j < ny; j++) {
                dv[(size_t)j * nx + i] = s->fre[j] * s->stretchy;
                if (two) dv[(size_t)j * nx + i + 1] = s->fim[j] * s->stretchy;
            }
        }
    }
}

/* z-derivative (derivatives.f90:292-298): dbyd2 over nx*ny columns, times stretch(k). */
static void d_z(orc3_sim *s, const double *var, double *dvar, int bc)
{
    const size_t n1 = (size_t)s->nx * s->ny;
    orc_dbyd2(dvar, var, (int)n1, s->nz, bc);
    for (int k = 0; k < s->nz; k++)
        for (size_t q = 0; q < n1; q++) dvar[(size_t)k * n1 + q] *= s->stretch[k];
}

/* model: nz rows x 6 columns (r/Rsun, c, rho, p, g, Gamma1), cgs, deepest row first. */
orc3_sim *orc3_create(const orc3_params *prm, const double *model)
{
    orc3_sim *s = (orc3_sim *)calloc(1, sizeof(orc3_sim));
    s->p = *prm;
    const int nx = prm->nx, ny = prm->ny, nz = prm->nz;
    s->nx = nx; s->ny = ny; s->nz = nz;
    s->nzpml = prm->npmlbot + prm->npmltop;
    s->N = (size_t)nx * ny * nz;
    const size_t N = s->N, P = (size_t)nx * ny * s->nzpml;
    s->fx = orc_fft_new(nx);
    s->fy = orc_fft_new(ny);
    if (!s->fx || !s->fy) { free(s); return NULL; }
    const int nm = nx > ny ? nx : ny;
    s->fre = z3(nm); s->fim = z3(nm); s->ftr = z3(nm); s->fti = z3(nm);
    s->z = z3(nz); s->stretch = z3(nz); s->unstretch = z3(nz); s->g = z3(nz); s->source_dep = z3(nz);
    s->rho0 = z3(nz); s->p0 = z3(nz); s->c2 = z3(nz); s->rhoinv = z3(nz); s->c2rho0 = z3(nz);
    s->gradrho0_z = z3(nz); s->gradp0_z = z3(nz); s->az = z3(nz); s->bzpml = z3(nz);
    s->v0x = z3(N); s->v0y = z3(N); s->v0z = z3(N);
    s->a = z3(6 * N); s->temp = z3(6 * N); s->scr = z3(6 * N);
    s->pmlvars = z3(2 * P); s->psipml = z3(2 * P); s->scrpml = z3(2 * P);
    s->d1 = z3(N); s->d2 = z3(N); s->d3 = z3(N); s->div = z3(N); s->pp = z3(N); s->rho = z3(N);
    s->gpx = z3(N); s->gpy = z3(N); s->gpz = z3(N);
    s->pattern = z3((size_t)nx * ny);

    s->stretchx = ORC3_RSUN / prm->xlength; /* initialize.f90:225-226 */
    s->stretchy = ORC3_RSUN / prm->ylength;
    s->dimc = 1e6; s->dimrho = 1e-3; s->diml = ORC3_RSUN;
    for (int k = 0; k < nz; k++) {
        const double *d = model + 6 * k;
        s->z[k] = d[0];
        const double c = d[1] / s->dimc;
        s->c2[k] = c * c;
        s->rho0[k] = d[2] / s->dimrho;
        s->p0[k] = d[3] / (s->dimrho * s->dimc * s->dimc);
        s->g[k] = d[4] * s->diml / (s->dimc * s->dimc);
    }
    orc_dbyd2(s->unstretch, s->z, 1, nz, 1);
    for (int k = 0; k < nz; k++) s->stretch[k] = 1.0 / s->unstretch[k];
    s->deltat = prm->timestep * s->dimc / s->diml;
    double opt[5] = {1.0, 0.5, (double)0.1665579725791151184f, (double)0.03950410250586729987f,
                     (double)0.007810706393337838236f};
    s->betas[4] = opt[1];
    s->betas[3] = opt[2] / s->betas[4];
    s->betas[2] = opt[3] / (s->betas[4] * s->betas[3]);
    s->betas[1] = opt[4] / (s->betas[4] * s->betas[3] * s->betas[2]);
    s->betas[0] = 0.0;
    for (int r = 0; r < 5; r++) s->betas[r] *= s->deltat;

    /* physics.f90:44-62 */
    double t2 = 1.0 + prm->excitdep / ORC3_RSUN, tmin = 1.0;
    for (int k = 0; k < nz; k++)
        if (fabs(s->z[k] - t2) <= tmin) { tmin = fabs(s->z[k] - t2); s->e_rad = k; }
    double tr = 1.0 + prm->obsheight / ORC3_RSUN;
    tmin = 1.0;
    for (int k = 0; k < nz; k++)
        if (fabs(s->z[k] - tr) <= tmin) { tmin = fabs(s->z[k] - tr); s->o_rad = k; }
    for (int k = 0; k < nz; k++) { /* physics.f90:109 (10.0**(7.0) and 4.0 are exact in float) */
        const double dz = s->z[k] - s->z[s->e_rad];
        s->source_dep[k] = exp(-1e7 * 4.0 * (dz * dz));
    }
    /* physics.f90:204-208 */
    for (int k = 0; k < nz; k++) {
        s->rhoinv[k] = 1.0 / s->rho0[k];
        s->c2rho0[k] = s->c2[k] * s->rho0[k];
    }
    orc_dbyd2(s->gradrho0_z, s->rho0, 1, nz, 1);
    orc_dbyd2(s->gradp0_z, s->p0, 1, nz, 1);
    for (int k = 0; k < nz; k++) {
        s->gradrho0_z[k] *= s->stretch[k];
        s->gradp0_z[k] *= s->stretch[k];
    }
    /* vertical PML, physics.f90:255-295 */
    {
        const int nb = prm->npmlbot, nt = prm->npmltop;
        const double l005 = (double)0.005f;
        const double *z = s->z;
        const double cb = sqrt(s->c2[0]), ct = sqrt(s->c2[nz - 1]);
        for (int k = 0; k < nz; k++) {
            double alk = ORC3_PI * l005 * s->diml / s->dimc, dampz = 0.0;
            if (k < nb) {
                alk = ORC3_PI * l005 * s->diml / s->dimc * (z[k] - z[0]) / (z[nb - 1] - z[0]);
                const double rr = (z[nb - 1] - z[k]) / (z[nb - 1] - z[0]);
                dampz = 2. * 3. * 3. * cb / (z[nb - 1] - z[0]) * (rr * rr);
                const double fd = alk / (dampz + alk);
                s->gradp0_z[k] *= fd;
                s->gradrho0_z[k] *= fd;
                s->g[k] *= fd;
            }
            if (k > nz - nt - 1) {
                alk = ORC3_PI * l005 * s->diml / s->dimc * (z[nz - 1] - z[k]) / (z[nz - 1] - z[nz - nt]);
                const double rr = (z[nz - nt] - z[k]) / (z[nz - 1] - z[nz - nt]);
                dampz = 3. * 3. * ct / (z[nz - 1] - z[nz - nt]) * (rr * rr);
                const double fd = alk / (dampz + alk);
                s->gradp0_z[k] *= fd;
                s->gradrho0_z[k] *= fd;
                s->g[k] *= fd;
            }
            s->bzpml[k] = -alk - dampz;
            s->az[k] = -dampz;
        }
    }
    return s;
}

void orc3_destroy(orc3_sim *s)
{
    if (!s) return;
    double *ptrs[] = {s->fre, s->fim, s->ftr, s->fti, s->z, s->stretch, s->unstretch, s->g, s->source_dep,
                      s->rho0, s->p0, s->c2, s->rhoinv, s->c2rho0, s->gradrho0_z, s->gradp0_z, s->az, s->bzpml,
                      s->v0x, s->v0y, s->v0z, s->a, s->temp, s->scr, s->pmlvars, s->psipml, s->scrpml,
                      s->d1, s->d2, s->d3, s->div, s->pp, s->rho, s->gpx, s->gpy, s->gpz, s->pattern, s->amp,
                      s->adj_rows, s->adj_w};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++) free(ptrs[i]);
    free(s->adj_idx);
    orc_fft_delete(s->fx);
    orc_fft_delete(s->fy);
    free(s);
}

int orc3_set_flow(orc3_sim *s, const double *v0x, const double *v0y, const double *v0z)
{
    memcpy(s->v0x, v0x, s->N * sizeof(double));
    memcpy(s->v0y, v0y, s->N * sizeof(double));
    memcpy(s->v0z, v0z, s->N * sizeof(double));
    return 0;
}

/* forcing(x, y, step) = pattern(x, y) * amp[step] (0 past the table). */
int orc3_set_source(orc3_sim *s, const double *pattern, const double *amp, int namp)
{
    memcpy(s->pattern, pattern, (size_t)s->nx * s->ny * sizeof(double));
    free(s->amp);
    s->amp = z3(namp);
    memcpy(s->amp, amp, (size_t)namp * sizeof(double));
    s->namp = namp;
    return 0;
}

/* Kernel-mode adjoint source: forcing(x, y, step t) = scale * sum_j w[t][j] rows[idx[t] + j](x, y),
 * injected into RHS v_z at o_rad in place of the pattern source. */
int orc3_set_adjoint_source(orc3_sim *s, const double *rows, int nrows, const double *w, const int *idx, int ntab,
                            double scale)
{
    const size_t nxy = (size_t)s->nx * s->ny;
    free(s->adj_rows);
    free(s->adj_w);
    free(s->adj_idx);
    s->adj_rows = z3((size_t)nrows * nxy);
    memcpy(s->adj_rows, rows, (size_t)nrows * nxy * sizeof(double));
    s->adj_w = z3((size_t)ntab * 7);
    memcpy(s->adj_w, w, (size_t)ntab * 7 * sizeof(double));
    s->adj_idx = (int *)calloc((size_t)ntab, sizeof(int));
    memcpy(s->adj_idx, idx, (size_t)ntab * sizeof(int));
    s->adj_nrows = nrows;
    s->adj_ntab = ntab;
    s->adj_scale = scale;
    s->adj = 1;
    return 0;
}

static int pml_index(const orc3_sim *s, int k)
{
    if (k < s->p.npmlbot) return k;
    if (k >= s->nz - s->p.npmltop) return s->p.npmlbot + (k - (s->nz - s->p.npmltop));
    return -1;
}

/* displacement.f90:377-477 on s->temp (psi from s->psipml), result in s->scr, s->scrpml. */
static void orc3_rhs(orc3_sim *s)
{
    const int nx = s->nx, ny = s->ny, nz = s->nz;
    const size_t N = s->N, nxy = (size_t)nx * ny, P = nxy * s->nzpml;
    const double *xix = s->temp, *xiy = s->temp + N, *xiz = s->temp + 2 * N;
    const double *vx = s->temp + 3 * N, *vy = s->temp + 4 * N, *vz = s->temp + 5 * N;
    const double *psivz = s->psipml, *psip = s->psipml + P;
    double *rpsivz = s->scrpml, *rpsip = s->scrpml + P;
    d_x(s, xix, s->d1);
    d_y(s, xiy, s->d2);
    d_z(s, xiz, s->d3, 1);
    for (int k = 0; k < nz; k++) {
        const int pi = pml_index(s, k);
        for (size_t q = 0; q < nxy; q++) {
            const size_t i = (size_t)k * nxy + q;
            if (pi >= 0) {
                const size_t m = (size_t)pi * nxy + q;
                rpsivz[m] = s->az[k] * s->d3[i] + s->bzpml[k] * psivz[m];
                s->d3[i] = s->d3[i] + psivz[m];
            }
            s->div[i] = s->d1[i] + s->d2[i] + s->d3[i];
            s->pp[i] = -s->c2rho0[k] * s->div[i] - xiz[i] * s->gradp0_z[k];
            s->rho[i] = -s->rho0[k] * s->div[i] - xiz[i] * s->gradrho0_z[k];
        }
    }
    d_x(s, s->pp, s->gpx);
    d_y(s, s->pp, s->gpy);
    d_z(s, s->pp, s->gpz, 0);
    for (int k = 0; k < nz; k++) {
        const int pi = pml_index(s, k);
        if (pi < 0) continue;
        for (size_t q = 0; q < nxy; q++) {
            const size_t i = (size_t)k * nxy + q, m = (size_t)pi * nxy + q;
            rpsip[m] = s->az[k] * s->gpz[i] + s->bzpml[k] * psip[m];
            s->gpz[i] = s->gpz[i] + psip[m];
        }
    }
    const double *vv[3] = {vx, vy, vz};
    const double *gp[3] = {s->gpx, s->gpy, s->gpz};
    for (int c = 0; c < 3; c++) {
        d_x(s, vv[c], s->d1);
        d_y(s, vv[c], s->d2);
        d_z(s, vv[c], s->d3, 1);
        double *r = s->scr + (size_t)(3 + c) * N;
        for (int k = 0; k < nz; k++)
            for (size_t q = 0; q < nxy; q++) {
                const size_t i = (size_t)k * nxy + q;
                r[i] = -2.0 * (s->v0x[i] * s->d1[i] + s->v0y[i] * s->d2[i] + s->v0z[i] * s->d3[i]) -
                       s->rhoinv[k] * gp[c][i];
            }
    }
    const double amp = s->time < s->namp ? s->amp[s->time] : 0.0;
    double *rvz = s->scr + 5 * N;
    for (int k = 0; k < nz; k++)
        for (size_t q = 0; q < nxy; q++) {
            const size_t i = (size_t)k * nxy + q;
            rvz[i] = rvz[i] - s->rhoinv[k] * s->rho[i] * s->g[k];
            if (s->adj) {
                if (k == s->o_rad && s->time >= 0 && s->time < s->adj_ntab) {
                    const double *w = s->adj_w + (size_t)s->time * 7;
                    double f = 0.0;
                    for (int j = 0; j < 7; j++) {
                        const int r = s->adj_idx[s->time] + j;
                        if (r >= 0 && r < s->adj_nrows && w[j] != 0.0) f += w[j] * s->adj_rows[(size_t)r * nxy + q];
                    }
                    rvz[i] = rvz[i] + f * s->adj_scale;
                }
            } else if (abs(k - s->e_rad) <= 4) {
                rvz[i] = rvz[i] + (s->pattern[q] * amp) * s->source_dep[k];
            }
        }
    memcpy(s->scr, vx, N * sizeof(double));
    memcpy(s->scr + N, vy, N * sizeof(double));
    memcpy(s->scr + 2 * N, vz, N * sizeof(double));
    for (int l = 0; l < 6; l++) {
        memset(s->scr + (size_t)l * N, 0, nxy * sizeof(double));
        memset(s->scr + (size_t)l * N + (size_t)(nz - 1) * nxy, 0, nxy * sizeof(double));
    }
}

/* FILTER_VARS_3D_HORIZ_PML, physics.f90:836-882: rows k = npmlbot+1 .. nz-npmltop (1-based). */
static void orc3_filter(orc3_sim *s)
{
    static const double c[6] = {0.75390625, 0.41015625, -0.234375, 0.087890625, -0.01953125, 0.001953125};
    const int nz = s->nz;
    const size_t nxy = (size_t)s->nx * s->ny;
    const int k0 = s->p.npmlbot, k1 = nz - s->p.npmltop; /* 0-based [k0, k1) */
    double *tmp = s->d1;
    for (int l = 0; l < 6; l++) {
        double *a = s->a + (size_t)l * s->N;
        for (int k = k0; k < k1; k++)
            for (size_t q = 0; q < nxy; q++) {
#define A3(kk) a[(size_t)(kk) * nxy + q]
                tmp[(size_t)k * nxy + q] = c[0] * A3(k) + 0.5 * c[1] * (A3(k - 1) + A3(k + 1)) +
                                           0.5 * c[2] * (A3(k - 2) + A3(k + 2)) + 0.5 * c[3] * (A3(k - 3) + A3(k + 3)) +
                                           0.5 * c[4] * (A3(k - 4) + A3(k + 4)) + 0.5 * c[5] * (A3(k - 5) + A3(k + 5));
#undef A3
            }
        for (int k = k0; k < k1; k++) memcpy(a + (size_t)k * nxy, tmp + (size_t)k * nxy, nxy * sizeof(double));
    }
}

/* step.f90:43-119 for option 16 with HORIZONTAL_PMLS. */
void orc3_step(orc3_sim *s)
{
    const size_t N6 = 6 * s->N, P2 = 2 * (size_t)s->nx * s->ny * s->nzpml;
    for (int rk = 0; rk < 5; rk++) {
        if (rk == 0) {
            memcpy(s->temp, s->a, N6 * sizeof(double));
            memcpy(s->psipml, s->pmlvars, P2 * sizeof(double));
        } else {
            const double b = s->betas[rk];
            for (size_t q = 0; q < N6; q++) s->temp[q] = s->a[q] + b * s->scr[q];
            for (size_t q = 0; q < P2; q++) s->psipml[q] = s->pmlvars[q] + b * s->scrpml[q];
        }
        orc3_rhs(s);
    }
    for (size_t q = 0; q < N6; q++) s->a[q] = s->a[q] + s->deltat * s->scr[q];
    for (size_t q = 0; q < P2; q++) s->pmlvars[q] = s->pmlvars[q] + s->deltat * s->scrpml[q];
    if (s->p.filter_every == 2 && (s->time + 1) % 2 == 0) orc3_filter(s);
}

/* TIMESTEPPING (driver.f90:337-409): nsteps steps; after each step whose index is a multiple
 * of steps_out, append a(:,:,o_rad,6) (nx*ny values) to seis.  Returns the record count. */
int orc3_run(orc3_sim *s, int nsteps, double *seis)
{
    int nrec = 0;
    const size_t nxy = (size_t)s->nx * s->ny;
    for (int it = 0; it < nsteps; it++) {
        orc3_step(s);
        if (s->time % s->p.steps_out == 0) {
            if (seis) memcpy(seis + (size_t)nrec * nxy, s->a + 5 * s->N + (size_t)s->o_rad * nxy, nxy * sizeof(double));
            nrec++;
        }
        s->time++;
    }
    return nrec;
}

/* One step of TIMESTEPPING; returns the index of the step made (the record test of orc3_run). */
int orc3_advance(orc3_sim *s)
{
    orc3_step(s);
    return s->time++;
}

/* RHS of the last stage of the last step, [6][nz][ny][nx] (the acceleration is entries 3..5). */
int orc3_get_scr(const orc3_sim *s, double *scr)
{
    memcpy(scr, s->scr, 6 * s->N * sizeof(double));
    return 0;
}

/* the whole state [6][nz][ny][nx] and the PML auxiliaries [2][nzpml][ny][nx] */
int orc3_get_state(const orc3_sim *s, double *a, double *pml)
{
    if (a) memcpy(a, s->a, 6 * s->N * sizeof(double));
    if (pml) memcpy(pml, s->pmlvars, 2 * (size_t)s->nx * s->ny * s->nzpml * sizeof(double));
    return 0;
}

int orc3_get_int(const orc3_sim *s, const char *name)
{
    if (!strcmp(name, "e_rad")) return s->e_rad;
    if (!strcmp(name, "o_rad")) return s->o_rad;
    if (!strcmp(name, "time")) return s->time;
    return -1;
}

/* profiles [nz]: stretch, rhoinv, rho0, gradp0_z, gradrho0_z, g, c2rho0, source_dep, az, bz */
long orc3_get_profile(const orc3_sim *s, const char *name, double *out)
{
    const double *src = NULL;
    if (!strcmp(name, "stretch")) src = s->stretch;
    else if (!strcmp(name, "rhoinv")) src = s->rhoinv;
    else if (!strcmp(name, "rho0")) src = s->rho0;
    else if (!strcmp(name, "gradp0_z")) src = s->gradp0_z;
    else if (!strcmp(name, "gradrho0_z")) src = s->gradrho0_z;
    else if (!strcmp(name, "g")) src = s->g;
    else if (!strcmp(name, "c2rho0")) src = s->c2rho0;
    else if (!strcmp(name, "source_dep")) src = s->source_dep;
    else if (!strcmp(name, "az")) src = s->az;
    else if (!strcmp(name, "bz")) src = s->bzpml;
    if (!src) return -1;
    memcpy(out, src, s->nz * sizeof(double));
    return s->nz;
}

double orc3_get_double(const orc3_sim *s, const char *name)
{
    if (!strcmp(name, "deltat")) return s->deltat;
    if (!strcmp(name, "stretchx")) return s->stretchx;
    if (!strcmp(name, "stretchy")) return s->stretchy;
    for (int r = 0; r < 5; r++) {
        char nm[8] = "beta0";
        nm[4] = (char)('0' + r);
        if (!strcmp(name, nm)) return s->betas[r];
    }
    return NAN;
}

/* public derivative wrappers for the tests */
int orc3_ddx(orc3_sim *s, const double *var, double *dvar) { d_x(s, var, dvar); return 0; }
int orc3_ddy(orc3_sim *s, const double *var, double *dvar) { d_y(s, var, dvar); return 0; }
int orc3_ddz(orc3_sim *s, const double *var, double *dvar, int bc) { d_z(s, var, dvar, bc); return 0; }
