/* sparc_oracle_sponge.c -- CPU FP64 oracle of the 2-D sponge step (test infrastructure).
 *
 * A plain-C restatement of the reference's option 5, MP_QUIET_SPONGE_2D: the velocity-pressure-
 * density formulation with a sponge layer instead of a PML, of option 6, MP_QUIET_PML_2D
 * (the same formulation with the vertical PML, physics2d.f90:662-713, 1142-1160, 288-332), and
 * of option 12, MP_MHD_PML_2d (physics2d.f90:411-474 with the magnetic part of
 * PML_BOUNDARY_ACCOUNTING_2D, 1162-1200), and of option 11, MP_MHD_SPONGE_2D (physics2d.f90:
 * 588-658), used only by the tests as the checker of the GPU path (csrc/sparc_sponge.cu; option
 * 11 has no GPU plan yet).  Fields are [nz][nx], x fastest; the state is five of them: rho, v_x,
 * v_y (zero in 2-D), v_z, p (initialize.f90:500-512), and for option 12 eight: b_x, b_y (zero in
 * 2-D), b_z follow.  Option 12's background field (box, boz) is given; curlboy = d box/dz -
 * d boz/dx as physics2d.f90:166-168 (the reduction factor there ends as 1).  The background
 * stratification stays laterally uniform (gradrho0_x = gradp0_x = 0: a current-free field needs
 * no change of it).
 *
 * Followed lines:
 *   grid, stretch, solar_data, betas  as sparc_oracle.c (initialize.f90:195-226, 466-474,
 *                                     731-794; step.f90:24-41)
 *   e_rad, o_rad, source_dep, sponge  physics2d.f90:35-69 (spongez; spongexyz = spongez for a
 *                                     periodic box, physics2d.f90:210-216); single-precision
 *                                     literals 1.002, 0.0001, 0.005, 0.0005 rounded as Fortran does
 *   rhoinv, c2rho0, d rho0/dz, d p0/dz physics2d.f90:226-230 (no PML decay: USE_PML off)
 *   RHS                               physics2d.f90:1099-1137
 *   STEP                              step.f90:43-119 (no PML auxiliaries) with FILTER_VARS_2D
 *                                     (physics2d.f90:509-583) on the five fields: rows kst = 6 ..
 *                                     nz-1, x in [npmlhor, nx-npmlhor+1] with HORIZONTAL_PMLS
 *   records                           v_z at o_rad every steps_out (the reference's record
 *                                     a(:,:,o_rad,6) of driver.f90:391 lies past the five fields
 *                                     of this formulation; v_z is the field it stands for)
 * Forcing: forcing(x, step) = pattern(x) * amp[step] times source_dep(k) on |k - e_rad| <= 4
 * (physics2d.f90:1124-1128; the reference assigns forcing only in LAGRANGE_INTERP).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC5_PI 3.141592653589793
#define ORC5_RSUN 6.95989467700e10

int orc_dbyd2(double *A, const double *B, int n1, int n2, int ibc);
void *orc_fft_new(int n);
void orc_fft_delete(void *f);
void orc_fft_exec(const void *f, double *re, double *im, double *tr, double *ti, int sign);

typedef struct {
    int nx, nz, npmlhor;
    double xlength, timestep, excitdep, obsheight;
    int steps_out;
    int filter_all_x; /* 1: every column (HORIZONTAL_PMLS off) */
    int option;       /* 5: MP_QUIET_SPONGE_2D; 6: MP_QUIET_PML_2D (USE_PML, no sponge); 11: MP_MHD_SPONGE_2D;
                         12: MP_MHD_PML_2d */
    int npmlbot, npmltop;
} orc5_params;

typedef struct {
    orc5_params p;
    int nx, nz;
    size_t N;
    double deltat, stretchx, betas[5];
    double *z, *stretch, *g, *rho0, *p0, *c2, *rhoinv, *c2rho0, *gradrho0_z, *gradp0_z, *sponge, *source_dep;
    int e_rad, o_rad;
    double *a, *temp, *scr, *dvxdx, *dvzdz, *gpx, *gpz, *tmp;
    void *fx;
    double *fre, *fim, *ftr, *fti;
    double *pattern, *amp;
    int namp, time;
    int nzpml;
    double *az, *bz;                    /* [nz], options 6 and 12 */
    double *pmlvars, *psipml, *scrpml;  /* [npa][nzpml][nx]: psi_p, psi_vz (+ psi of dz flux2, dz b_x) */
    int nf, npa;                        /* fields of the state, PML auxiliaries */
    double *box, *boz, *curlboy;        /* [nz][nx], option 12 */
    double *flux, *dzbx, *dzf, *dxf, *dxbz;
} orc5_sim;

static double *z5(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }

static void d5_x(orc5_sim *s, const double *var, double *dvar)
{
    const int nx = s->nx;
    for (int r = 0; r < s->nz; r += 2) {
        const int two = r + 1 < s->nz;
        for (int i = 0; i < nx; i++) {
            s->fre[i] = var[(size_t)r * nx + i];
            s->fim[i] = two ? var[(size_t)(r + 1) * nx + i] : 0.0;
        }
        orc_fft_exec(s->fx, s->fre, s->fim, s->ftr, s->fti, -1);
        for (int k = 0; k < nx; k++) {
            const double kap = 2 * k < nx ? (double)k / nx * 2.0 * ORC5_PI
                                          : (2 * k == nx ? 0.0 : -(double)(nx - k) / nx * 2.0 * ORC5_PI);
            const double re = s->fre[k], im = s->fim[k];
            s->fre[k] = -kap * im;
            s->fim[k] = kap * re;
        }
        orc_fft_exec(s->fx, s->fre, s->fim, s->ftr, s->fti, +1);
        for (int i = 0; i < nx; i++) {
            dvar[(size_t)r * nx + i] = s->fre[i] * s->stretchx;
            if (two) dvar[(size_t)(r + 1) * nx + i] = s->fim[i] * s->stretchx;
        }
    }
}

static void d5_z(orc5_sim *s, const double *var, double *dvar, int bc)
{
    orc_dbyd2(dvar, var, s->nx, s->nz, bc);
    for (int k = 0; k < s->nz; k++)
        for (int i = 0; i < s->nx; i++) dvar[(size_t)k * s->nx + i] *= s->stretch[k];
}

orc5_sim *orc5_create(const orc5_params *prm, const double *model)
{
    orc5_sim *s = (orc5_sim *)calloc(1, sizeof(orc5_sim));
    s->p = *prm;
    const int nx = prm->nx, nz = prm->nz;
    s->nx = nx; s->nz = nz;
    s->N = (size_t)nx * nz;
    const size_t N = s->N;
    s->fx = orc_fft_new(nx);
    if (!s->fx) { free(s); return NULL; }
    s->fre = z5(nx); s->fim = z5(nx); s->ftr = z5(nx); s->fti = z5(nx);
    s->z = z5(nz); s->stretch = z5(nz); s->g = z5(nz); s->rho0 = z5(nz); s->p0 = z5(nz); s->c2 = z5(nz);
    s->rhoinv = z5(nz); s->c2rho0 = z5(nz); s->gradrho0_z = z5(nz); s->gradp0_z = z5(nz); s->sponge = z5(nz);
    s->source_dep = z5(nz);
    s->nf = (prm->option == 11 || prm->option == 12) ? 8 : 5;
    s->npa = prm->option == 12 ? 4 : (prm->option == 6 ? 2 : 0);
    s->a = z5(s->nf * N); s->temp = z5(s->nf * N); s->scr = z5(s->nf * N);
    s->box = z5(N); s->boz = z5(N); s->curlboy = z5(N);
    s->flux = z5(N); s->dzbx = z5(N); s->dzf = z5(N); s->dxf = z5(N); s->dxbz = z5(N);
    s->dvxdx = z5(N); s->dvzdz = z5(N); s->gpx = z5(N); s->gpz = z5(N); s->tmp = z5(N);
    s->pattern = z5(nx);
    const double dimc = 1e6, dimrho = 1e-3, diml = ORC5_RSUN;
    s->stretchx = ORC5_RSUN / prm->xlength;
    for (int k = 0; k < nz; k++) {
        const double *d = model + 6 * k;
        s->z[k] = d[0];
        const double c = d[1] / dimc;
        s->c2[k] = c * c;
        s->rho0[k] = d[2] / dimrho;
        s->p0[k] = d[3] / (dimrho * dimc * dimc);
        s->g[k] = d[4] * diml / (dimc * dimc);
    }
    double *un = s->tmp;
    orc_dbyd2(un, s->z, 1, nz, 1);
    for (int k = 0; k < nz; k++) s->stretch[k] = 1.0 / un[k];
    s->deltat = prm->timestep * dimc / diml;
    const double opt[5] = {1.0, 0.5, (double)0.1665579725791151184f, (double)0.03950410250586729987f,
                           (double)0.007810706393337838236f};
    s->betas[4] = opt[1];
    s->betas[3] = opt[2] / s->betas[4];
    s->betas[2] = opt[3] / (s->betas[4] * s->betas[3]);
    s->betas[1] = opt[4] / (s->betas[4] * s->betas[3] * s->betas[2]);
    s->betas[0] = 0.0;
    for (int r = 0; r < 5; r++) s->betas[r] *= s->deltat;
    double t2 = 1.0 + prm->excitdep / ORC5_RSUN, tmin = 1.0;
    for (int k = 0; k < nz; k++)
        if (fabs(s->z[k] - t2) <= tmin) { tmin = fabs(s->z[k] - t2); s->e_rad = k; }
    double tr = 1.0 + prm->obsheight / ORC5_RSUN;
    tmin = 1.0;
    for (int k = 0; k < nz; k++)
        if (fabs(s->z[k] - tr) <= tmin) { tmin = fabs(s->z[k] - tr); s->o_rad = k; }
    for (int k = 0; k < nz; k++) { /* physics2d.f90:62-69 */
        s->sponge[k] = 200.0 / (1.0 + exp(((double)1.002f - s->z[k]) / (double)0.0001f)) +
                       300.0 / (1.0 + exp((s->z[k] - (s->z[0] + (double)0.005f)) / (double)0.0005f));
        const double dz = s->z[k] - s->z[s->e_rad];
        s->source_dep[k] = exp(-1e7 * 4.0 * (dz * dz));
        s->rhoinv[k] = 1.0 / s->rho0[k];
        s->c2rho0[k] = s->c2[k] * s->rho0[k];
    }
    orc_dbyd2(s->gradrho0_z, s->rho0, 1, nz, 1);
    orc_dbyd2(s->gradp0_z, s->p0, 1, nz, 1);
    for (int k = 0; k < nz; k++) {
        s->gradrho0_z[k] *= s->stretch[k];
        s->gradp0_z[k] *= s->stretch[k];
    }
    s->nzpml = (prm->option == 6 || prm->option == 12) ? prm->npmlbot + prm->npmltop : 0;
    s->az = z5(nz); s->bz = z5(nz);
    s->pmlvars = z5((size_t)s->npa * s->nzpml * nx); s->psipml = z5((size_t)s->npa * s->nzpml * nx);
    s->scrpml = z5((size_t)s->npa * s->nzpml * nx);
    if (prm->option == 6 || prm->option == 12) {
        /* USE_PML: no sponge (physics2d.f90:289-290) and the vertical PML of physics2d.f90:288-332
         * (laterally uniform background; the top layer's damping takes c at level nz-5) */
        const int nb = prm->npmlbot, nt = prm->npmltop;
        const double l005 = (double)0.005f;
        const double *z = s->z;
        for (int k = 0; k < nz; k++) {
            s->sponge[k] = 0.0;
            double alk = ORC5_PI * l005 * diml / dimc, dampz = 0.0;
            if (k < nb) {
                alk = ORC5_PI * l005 * diml / dimc * (z[k] - z[0]) / (z[nb - 1] - z[0]);
                const double rr = (z[nb - 1] - z[k]) / (z[nb - 1] - z[0]);
                dampz = 3. * 3. * sqrt(s->c2[0]) / (z[nb - 1] - z[0]) * (rr * rr);
                const double fd = alk / (dampz + alk);
                s->gradp0_z[k] *= fd;
                s->gradrho0_z[k] *= fd;
                s->g[k] *= fd;
            }
            if (k > nz - nt - 1) {
                alk = ORC5_PI * l005 * diml / dimc * (z[nz - 1] - z[k]) / (z[nz - 1] - z[nz - nt]);
                const double rr = (z[nz - nt] - z[k]) / (z[nz - 1] - z[nz - nt]);
                dampz = 3. * 3. * sqrt(s->c2[nz - 6]) / (z[nz - 1] - z[nz - nt]) * (rr * rr);
                const double fd = alk / (dampz + alk);
                s->gradp0_z[k] *= fd;
                s->gradrho0_z[k] *= fd;
                s->g[k] *= fd;
            }
            s->bz[k] = -alk - dampz;
            s->az[k] = -dampz;
        }
    }
    return s;
}

static int pml5(const orc5_sim *s, int k)
{
    if (k < s->p.npmlbot) return k;
    if (k >= s->nz - s->p.npmltop) return s->p.npmlbot + (k - (s->nz - s->p.npmltop));
    return -1;
}

/* MP_QUIET_PML_2D (physics2d.f90:662-713) with PML_BOUNDARY_ACCOUNTING_2D (1142-1160). */
static void orc6_rhs(orc5_sim *s)
{
    const int nx = s->nx, nz = s->nz;
    const size_t N = s->N, P = (size_t)s->nzpml * nx;
    const double *rho = s->temp, *vx = s->temp + N, *vz = s->temp + 3 * N, *p = s->temp + 4 * N;
    double *rc = s->scr, *rvx = s->scr + N, *rvy = s->scr + 2 * N, *rvz = s->scr + 3 * N, *rp = s->scr + 4 * N;
    d5_z(s, vz, s->dvzdz, 1);
    d5_z(s, p, s->gpz, 1);
    for (int k = 0; k < nz; k++) {
        const int pi = pml5(s, k);
        if (pi < 0) continue;
        for (int i = 0; i < nx; i++) {
            const size_t q = (size_t)k * nx + i, m = (size_t)pi * nx + i;
            s->scrpml[m] = s->az[k] * s->gpz[q] + s->bz[k] * s->psipml[m];
            s->gpz[q] = s->gpz[q] + s->psipml[m];
            s->scrpml[P + m] = s->az[k] * s->dvzdz[q] + s->bz[k] * s->psipml[P + m];
            s->dvzdz[q] = s->dvzdz[q] + s->psipml[P + m];
        }
    }
    d5_x(s, vx, s->dvxdx);
    d5_x(s, p, s->gpx);
    const double amp = s->time < s->namp ? s->amp[s->time] : 0.0;
    for (int k = 0; k < nz; k++)
        for (int i = 0; i < nx; i++) {
            const size_t q = (size_t)k * nx + i;
            const double div = s->dvxdx[q] + s->dvzdz[q];
            rc[q] = -s->rho0[k] * div - s->gradrho0_z[k] * vz[q];
            rp[q] = -s->c2rho0[k] * div - vz[q] * s->gradp0_z[k];
            rvx[q] = -s->rhoinv[k] * s->gpx[q];
            double r = -s->rhoinv[k] * (s->gpz[q] + rho[q] * s->g[k]);
            if (abs(k - s->e_rad) <= 4) r = r + (s->pattern[i] * amp) * s->source_dep[k];
            rvz[q] = r;
            rvy[q] = 0.0;
        }
    for (int i = 0; i < nx; i++) {
        const size_t t0 = i, t1 = (size_t)(nz - 1) * nx + i;
        rvx[t0] = rvx[t1] = rvz[t0] = rvz[t1] = rp[t0] = rp[t1] = rc[t0] = rc[t1] = 0.0;
    }
}

/* The background field of option 12 (nondimensional, B / dimb, initialize.f90:759): box, boz
 * [nz][nx] and curlboy = d box/dz - d boz/dx (physics2d.f90:166-168). */
int orc5_set_magnetic(orc5_sim *s, const double *box, const double *boz)
{
    if (s->p.option != 11 && s->p.option != 12) return -1;
    memcpy(s->box, box, s->N * sizeof(double));
    memcpy(s->boz, boz, s->N * sizeof(double));
    d5_z(s, s->box, s->curlboy, 1);
    d5_x(s, s->boz, s->tmp);
    for (size_t q = 0; q < s->N; q++) s->curlboy[q] -= s->tmp[q];
    return 0;
}

/* MP_MHD_PML_2d (physics2d.f90:411-474) with PML_BOUNDARY_ACCOUNTING_2D (1142-1200): the
 * non-magnetic accounting of psi_p, psi_vz, then the two-point smoothing of dv_z/dz on the PML
 * rows 2..npmlbot and nz-npmltop+1..nz-1 (1-based) and the PML of d flux2/dz and d b_x/dz. */
static void orc12_rhs(orc5_sim *s)
{
    const int nx = s->nx, nz = s->nz, nb = s->p.npmlbot, nt = s->p.npmltop;
    const size_t N = s->N, P = (size_t)s->nzpml * nx;
    const double *rho = s->temp, *vx = s->temp + N, *vz = s->temp + 3 * N, *p = s->temp + 4 * N;
    const double *bx = s->temp + 5 * N, *bz = s->temp + 7 * N;
    double *sc = s->scr;
    for (size_t q = 0; q < N; q++) s->flux[q] = -(vx[q] * s->boz[q] - vz[q] * s->box[q]);
    d5_z(s, vz, s->dvzdz, 1);
    d5_z(s, p, s->gpz, 1);
    d5_z(s, bx, s->dzbx, 1);
    d5_z(s, s->flux, s->dzf, 1);
    for (int k = 0; k < nz; k++) {
        const int pi = pml5(s, k);
        if (pi < 0) continue;
        for (int i = 0; i < nx; i++) {
            const size_t q = (size_t)k * nx + i, m = (size_t)pi * nx + i;
            s->scrpml[m] = s->az[k] * s->gpz[q] + s->bz[k] * s->psipml[m];
            s->gpz[q] = s->gpz[q] + s->psipml[m];
            s->scrpml[P + m] = s->az[k] * s->dvzdz[q] + s->bz[k] * s->psipml[P + m];
            s->dvzdz[q] = s->dvzdz[q] + s->psipml[P + m];
        }
    }
    double *t = s->tmp;
    for (int k = 1; k <= nb - 1; k++)
        for (int i = 0; i < nx; i++)
            t[(size_t)k * nx + i] = 0.5 * (s->dvzdz[(size_t)(k - 1) * nx + i] + s->dvzdz[(size_t)(k + 1) * nx + i]);
    for (int k = nz - nt; k <= nz - 2; k++)
        for (int i = 0; i < nx; i++)
            t[(size_t)k * nx + i] = 0.5 * (s->dvzdz[(size_t)(k - 1) * nx + i] + s->dvzdz[(size_t)(k + 1) * nx + i]);
    for (int k = 1; k <= nb - 1; k++) memcpy(s->dvzdz + (size_t)k * nx, t + (size_t)k * nx, nx * sizeof(double));
    for (int k = nz - nt; k <= nz - 2; k++) memcpy(s->dvzdz + (size_t)k * nx, t + (size_t)k * nx, nx * sizeof(double));
    for (int k = 0; k < nz; k++) {
        const int pi = pml5(s, k);
        if (pi < 0) continue;
        for (int i = 0; i < nx; i++) {
            const size_t q = (size_t)k * nx + i, m = (size_t)pi * nx + i;
            s->scrpml[2 * P + m] = s->az[k] * s->dzf[q] + s->bz[k] * s->psipml[2 * P + m];
            s->dzf[q] = s->dzf[q] + s->psipml[2 * P + m];
            s->scrpml[3 * P + m] = s->az[k] * s->dzbx[q] + s->bz[k] * s->psipml[3 * P + m];
            s->dzbx[q] = s->dzbx[q] + s->psipml[3 * P + m];
        }
    }
    d5_x(s, vx, s->dvxdx);
    d5_x(s, p, s->gpx);
    d5_x(s, s->flux, s->dxf);
    d5_x(s, bz, s->dxbz);
    const double amp = s->time < s->namp ? s->amp[s->time] : 0.0;
    for (int k = 0; k < nz; k++)
        for (int i = 0; i < nx; i++) {
            const size_t q = (size_t)k * nx + i;
            const double div = s->dvxdx[q] + s->dvzdz[q];
            const double cur = s->dzbx[q] - s->dxbz[q];
            const double t1 = s->boz[q] * cur + bz[q] * s->curlboy[q];
            const double t3 = -s->box[q] * cur - bx[q] * s->curlboy[q];
            sc[q] = -s->gradrho0_z[k] * vz[q] - s->rho0[k] * div;
            sc[N + q] = s->rhoinv[k] * (t1 - s->gpx[q]);
            sc[2 * N + q] = 0.0;
            double r = s->rhoinv[k] * (t3 - s->gpz[q]);
            r = r - s->rhoinv[k] * rho[q] * s->g[k];
            if (abs(k - s->e_rad) <= 4) r = r + (s->pattern[i] * amp) * s->source_dep[k];
            sc[3 * N + q] = r;
            sc[4 * N + q] = -s->c2rho0[k] * div - vz[q] * s->gradp0_z[k];
            sc[5 * N + q] = -s->dzf[q];
            sc[6 * N + q] = 0.0;
            sc[7 * N + q] = s->dxf[q];
        }
    for (int l = 0; l < 8; l++)
        for (int i = 0; i < nx; i++) {
            sc[(size_t)l * N + i] = 0.0;
            sc[(size_t)l * N + (size_t)(nz - 1) * nx + i] = 0.0;
        }
}

/* MP_MHD_SPONGE_2D (physics2d.f90:588-658): the sponge formulation with the background field;
 * d p/dz with both boundary rows set by the caller (ibc 4, dbyd2.f:129-140): row 1
 * (-c rho0 dv_z/dz - rho g) unstretch, row nz (c rho0 dv_z/dz - rho g) unstretch
 * (physics2d.f90:605-611, c the sound speed, not its square; unstretch = 1 / stretch); d b_x/dz
 * with ibc 0. */
static void orc11_rhs(orc5_sim *s)
{
    const int nx = s->nx, nz = s->nz;
    const size_t N = s->N;
    const double *rho = s->temp, *vx = s->temp + N, *vz = s->temp + 3 * N, *p = s->temp + 4 * N;
    const double *bx = s->temp + 5 * N, *bz = s->temp + 7 * N;
    double *sc = s->scr;
    d5_x(s, vx, s->dvxdx);
    d5_z(s, vz, s->dvzdz, 1);
    d5_x(s, p, s->gpx);
    for (int i = 0; i < nx; i++) {
        const size_t t0 = i, t1 = (size_t)(nz - 1) * nx + i;
        s->gpz[t0] = (-sqrt(s->c2[0]) * s->rho0[0] * s->dvzdz[t0] - rho[t0] * s->g[0]) / s->stretch[0];
        s->gpz[t1] = (sqrt(s->c2[nz - 1]) * s->rho0[nz - 1] * s->dvzdz[t1] - rho[t1] * s->g[nz - 1]) /
                     s->stretch[nz - 1];
    }
    d5_z(s, p, s->gpz, 4);
    d5_x(s, bz, s->dxbz);
    d5_z(s, bx, s->dzbx, 0);
    for (size_t q = 0; q < N; q++) s->flux[q] = -(vx[q] * s->boz[q] - vz[q] * s->box[q]);
    d5_z(s, s->flux, s->dzf, 1);
    d5_x(s, s->flux, s->dxf);
    const double amp = s->time < s->namp ? s->amp[s->time] : 0.0;
    for (int k = 0; k < nz; k++)
        for (int i = 0; i < nx; i++) {
            const size_t q = (size_t)k * nx + i;
            const double sp = s->sponge[k];
            const double div = s->dvxdx[q] + s->dvzdz[q];
            const double cur = s->dzbx[q] - s->dxbz[q];
            const double t1 = s->boz[q] * cur + bz[q] * s->curlboy[q];
            const double t3 = -s->box[q] * cur - bx[q] * s->curlboy[q];
            sc[q] = -s->gradrho0_z[k] * vz[q] - s->rho0[k] * div - sp * rho[q];
            sc[N + q] = s->rhoinv[k] * (t1 - s->gpx[q]) - sp * vx[q];
            sc[2 * N + q] = 0.0;
            double r = s->rhoinv[k] * (t3 - s->gpz[q]) - sp * vz[q];
            r = r - s->rhoinv[k] * rho[q] * s->g[k];
            if (abs(k - s->e_rad) <= 4) r = r + (s->pattern[i] * amp) * s->source_dep[k];
            sc[3 * N + q] = r;
            sc[4 * N + q] = -s->c2rho0[k] * div - vz[q] * s->gradp0_z[k] - sp * p[q];
            sc[5 * N + q] = -s->dzf[q];
            sc[6 * N + q] = 0.0;
            sc[7 * N + q] = s->dxf[q];
        }
    for (int l = 0; l < 8; l++)
        for (int i = 0; i < nx; i++) {
            sc[(size_t)l * N + i] = 0.0;
            sc[(size_t)l * N + (size_t)(nz - 1) * nx + i] = 0.0;
        }
}

void orc5_destroy(orc5_sim *s)
{
    if (!s) return;
    double *ptrs[] = {s->fre, s->fim, s->ftr, s->fti, s->z, s->stretch, s->g, s->rho0, s->p0, s->c2, s->rhoinv,
                      s->c2rho0, s->gradrho0_z, s->gradp0_z, s->sponge, s->source_dep, s->a, s->temp, s->scr,
                      s->dvxdx, s->dvzdz, s->gpx, s->gpz, s->tmp, s->pattern, s->amp, s->az, s->bz,
                      s->pmlvars, s->psipml, s->scrpml, s->box, s->boz, s->curlboy, s->flux, s->dzbx,
                      s->dzf, s->dxf, s->dxbz};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++) free(ptrs[i]);
    orc_fft_delete(s->fx);
    free(s);
}

int orc5_set_source(orc5_sim *s, const double *pattern, const double *amp, int namp)
{
    memcpy(s->pattern, pattern, (size_t)s->nx * sizeof(double));
    free(s->amp);
    s->amp = z5(namp);
    memcpy(s->amp, amp, (size_t)namp * sizeof(double));
    s->namp = namp;
    return 0;
}

/* physics2d.f90:1099-1137 on s->temp, into s->scr. */
static void orc5_rhs(orc5_sim *s)
{
    const int nx = s->nx, nz = s->nz;
    const size_t N = s->N;
    const double *rho = s->temp, *vx = s->temp + N, *vz = s->temp + 3 * N, *p = s->temp + 4 * N;
    double *rc = s->scr, *rvx = s->scr + N, *rvy = s->scr + 2 * N, *rvz = s->scr + 3 * N, *rp = s->scr + 4 * N;
    d5_x(s, vx, s->dvxdx);
    d5_z(s, vz, s->dvzdz, 1);
    d5_x(s, p, s->gpx);
    d5_z(s, p, s->gpz, 1);
    const double amp = s->time < s->namp ? s->amp[s->time] : 0.0;
    for (int k = 0; k < nz; k++)
        for (int i = 0; i < nx; i++) {
            const size_t q = (size_t)k * nx + i;
            const double sp = s->sponge[k];
            const double div = s->dvxdx[q] + s->dvzdz[q];
            rc[q] = -s->gradrho0_z[k] * vz[q] - s->rho0[k] * div - sp * rho[q];
            rvx[q] = -s->rhoinv[k] * s->gpx[q] - sp * vx[q];
            double r = -s->rhoinv[k] * s->gpz[q] - sp * vz[q];
            r = r - rho[q] * s->g[k] * s->rhoinv[k];
            if (abs(k - s->e_rad) <= 4) r = r + (s->pattern[i] * amp) * s->source_dep[k];
            rvz[q] = r;
            rp[q] = -s->c2rho0[k] * div - vz[q] * s->gradp0_z[k] - sp * p[q];
            rvy[q] = 0.0;
        }
    for (int i = 0; i < nx; i++) {
        const size_t t0 = i, t1 = (size_t)(nz - 1) * nx + i;
        rvx[t0] = rvx[t1] = 0.0;
        rvz[t0] = rvz[t1] = 0.0;
        rp[t0] = rp[t1] = 0.0;
    }
}

/* FILTER_VARS_2D (physics2d.f90:509-560) on the five fields, USE_PML off. */
static void orc5_filter(orc5_sim *s)
{
    static const double c[6] = {0.75390625, 0.41015625, -0.234375, 0.087890625, -0.01953125, 0.001953125};
    const int nx = s->nx, nz = s->nz, nh = s->p.npmlhor;
    double *temp = s->tmp;
    const int i0 = s->p.filter_all_x ? 0 : nh - 1, i1 = s->p.filter_all_x ? nx - 1 : nx - nh;
    for (int l = 0; l < s->nf; l++) {
        double *a = s->a + (size_t)l * s->N;
#define A5(k, i) a[(size_t)(k) * nx + (i)]
#define T5(k, i) temp[(size_t)(k) * nx + (i)]
        for (int k = 5; k <= nz - 6; k++)
            for (int i = 0; i < nx; i++)
                T5(k, i) = c[0] * A5(k, i) + 0.5 * c[1] * (A5(k - 1, i) + A5(k + 1, i)) +
                           0.5 * c[2] * (A5(k - 2, i) + A5(k + 2, i)) + 0.5 * c[3] * (A5(k - 3, i) + A5(k + 3, i)) +
                           0.5 * c[4] * (A5(k - 4, i) + A5(k + 4, i)) + 0.5 * c[5] * (A5(k - 5, i) + A5(k + 5, i));
        for (int k = nz - 5; k <= nz - 2; k++)
            for (int i = 0; i < nx; i++) T5(k, i) = 0.5 * (A5(k + 1, i) + A5(k - 1, i));
        for (int k = 5; k <= nz - 2; k++)
            for (int i = i0; i <= i1; i++) A5(k, i) = T5(k, i);
#undef A5
#undef T5
    }
}

void orc5_step(orc5_sim *s)
{
    const size_t N5 = (size_t)s->nf * s->N, P2 = (size_t)s->npa * s->nzpml * s->nx;
    for (int rk = 0; rk < 5; rk++) {
        if (rk == 0) {
            memcpy(s->temp, s->a, N5 * sizeof(double));
            memcpy(s->psipml, s->pmlvars, P2 * sizeof(double));
        } else {
            for (size_t q = 0; q < N5; q++) s->temp[q] = s->a[q] + s->betas[rk] * s->scr[q];
            for (size_t q = 0; q < P2; q++) s->psipml[q] = s->pmlvars[q] + s->betas[rk] * s->scrpml[q];
        }
        if (s->p.option == 12) orc12_rhs(s);
        else if (s->p.option == 11) orc11_rhs(s);
        else if (s->p.option == 6) orc6_rhs(s);
        else orc5_rhs(s);
    }
    for (size_t q = 0; q < N5; q++) s->a[q] = s->a[q] + s->deltat * s->scr[q];
    for (size_t q = 0; q < P2; q++) s->pmlvars[q] = s->pmlvars[q] + s->deltat * s->scrpml[q];
    orc5_filter(s);
}

int orc5_run(orc5_sim *s, int nsteps, double *seis)
{
    int nrec = 0;
    for (int it = 0; it < nsteps; it++) {
        orc5_step(s);
        if (s->time % s->p.steps_out == 0) {
            if (seis) memcpy(seis + (size_t)nrec * s->nx, s->a + 3 * s->N + (size_t)s->o_rad * s->nx, s->nx * sizeof(double));
            nrec++;
        }
        s->time++;
    }
    return nrec;
}

int orc5_get_state(const orc5_sim *s, double *a)
{
    memcpy(a, s->a, (size_t)s->nf * s->N * sizeof(double));
    return 0;
}

int orc5_get_int(const orc5_sim *s, const char *name)
{
    if (!strcmp(name, "e_rad")) return s->e_rad;
    if (!strcmp(name, "o_rad")) return s->o_rad;
    if (!strcmp(name, "nf")) return s->nf;
    return -1;
}

long orc5_get_profile(const orc5_sim *s, const char *name, double *out)
{
    const double *src = NULL;
    if (!strcmp(name, "sponge")) src = s->sponge;
    else if (!strcmp(name, "az")) src = s->az;
    else if (!strcmp(name, "bz")) src = s->bz;
    else if (!strcmp(name, "g")) src = s->g;
    else if (!strcmp(name, "stretch")) src = s->stretch;
    else if (!strcmp(name, "gradp0_z")) src = s->gradp0_z;
    else if (!strcmp(name, "gradrho0_z")) src = s->gradrho0_z;
    if (!src) return -1;
    memcpy(out, src, s->nz * sizeof(double));
    return s->nz;
}
