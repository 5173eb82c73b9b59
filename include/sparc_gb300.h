/*
 * sparc_gb300.h -- C ABI of the GB300 wave-solver hot path (2-D displacement formulation
 * with flows and PML, 5-stage low-storage Runge-Kutta, seismograms and kernel snapshots).
 *
 * Conventions
 *   - Bulk arrays are DEVICE pointers owned by the caller (PyTorch tensors on the Python
 *     side); the library never frees caller memory.  Small tables are host pointers.
 *   - Every field is x-fastest: f[k*nx + i], k = 0 the deepest level (the Fortran layout
 *     a(nx,ny,nz) of the reference with ny = 1); batch (solve) index outermost.
 *   - Every function returns SPARC_OK (0) or a negative code and never throws; the message
 *     of the last failure on the calling thread is sparc_last_error().
 *   - One plan per host thread.  All work is queued on the stream given (cudaStream_t
 *     passed as void*), nothing synchronises the device except where stated.
 */
#ifndef SPARC_GB300_H
#define SPARC_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define SPARC_OK 0
#define SPARC_ERR_ARG (-1)         /* bad argument (null pointer, inconsistent sizes) */
#define SPARC_ERR_SIZE (-2)        /* unsupported size (nx not in the FFT table, nz too small) */
#define SPARC_ERR_NONFINITE (-3)   /* non-finite values found in the state */
#define SPARC_ERR_TIMEOUT (-4)     /* a bounded device wait gave up */
#define SPARC_ERR_CUDA (-5)        /* CUDA runtime error */
#define SPARC_ERR_STATE (-6)       /* call out of order (e.g. run before background) */

typedef struct sparc_plan sparc_plan_t;

/* Grid, batch and run parameters.  Replaces the compile-time params.i (params.i:26-165) and
 * the module globals set by Initialize_all / mp_Initialize_RHS_2d / INITIALIZE_STEP
 * (initialize.f90:167-474, physics2d.f90:23-405, step.f90:24-41). */
typedef struct {
    int nx, nz, nbatch;        /* grid and number of independent solves in the batch */
    int precision;             /* 32 (FP32 state and arithmetic) or 64 (FP64) */
    int npmlbot, npmltop;      /* vertical PML layers (params.i:121) */
    int npmlhor;               /* horizontal PML columns per side (params.i:91) */
    double deltat;             /* nondimensional step timestep*dimc/diml (initialize.f90:474) */
    double stretchx;           /* rsun/xlength (initialize.f90:225) */
    double betas[5];           /* RK stage coefficients times deltat (step.f90:34-40) */
    int flows;                 /* BACKGROUND_FLOWS_EXIST: advection terms on (params.i:70) */
    int c2d;                   /* 1: c2rho0 is a 2-D (nz x nx) field, 0: a profile in z */
    int bg_per_solve;          /* 1: 2-D background arrays are given per solve */
    int steps_out;             /* record cadence in steps (driver.f90:209) */
    int k_inj;                 /* 0-based injection row (e_rad forward, o_rad adjoint) */
    int k_obs;                 /* 0-based observation row o_rad (physics2d.f90:43-50) */
    int src_until;             /* inject while time <= src_until (physics2d.f90:1049) */
    int filter_k0;             /* first 0-based row FILTER_VARS_2D writes: 5 as the reference
                                  (kst = 6), 1 to also apply its 2-point rows 2..5 (the
                                  commented-out kst = 2, physics2d.f90:545) */
    int filter_all_x;          /* 0: filter only x in [npmlhor, nx-npmlhor+1] (HORIZONTAL_PMLS,
                                  physics2d.f90:548-556); 1: every column */
    int compensated;           /* FP32 plans: 1 keeps a low-order part of the state so the RK
                                  update and filter round like FP64 arithmetic (no reference
                                  counterpart; the reference state is FP64) */
    int column_block;          /* column-pass block width in x-columns (tuning): 32, 8 or 4 for
                                  the partitioned solve (other values: 32 if nbatch * nx / 32
                                  blocks fill the GPU, else 8), 32, 16 or 8 for the banded pass
                                  (other values: 32) */
    int column_impl;           /* column pass: 0 partitioned solve with direct loads, 1 partitioned
                                  solve with TMA-staged tiles, 2 (FP32 plans) geometric-band
                                  inverse of the compact operator with direct loads (32-column
                                  blocks on nz = 300, nx = 128, 256, 384, 512, 1024: the inputs of its
                                  first and third phases TMA-staged), 3 (FP32 plans) geometric
                                  band in 8-column blocks with TMA-staged tiles; FP64 plans use 0
                                  for 2, 3 */
} sparc_config_t;

/* Background, all DEVICE pointers to FP64 arrays; copied (and rounded for FP32 plans) into
 * the plan.  nbg = nbatch if bg_per_solve else 1; nzpml = npmlbot + npmltop;
 * nhx = 2*npmlhor.  Mirrors the arrays of mp_Initialize_RHS_2d (physics2d.f90:226-357). */
typedef struct {
    const double *stretch, *unstretch;            /* [nz] (initialize.f90:466-470) */
    const double *rhoinv, *rho0;                  /* [nz] */
    const double *gradp0_z, *gradrho0_z;          /* [nz], before the PML decay factor */
    const double *g;                              /* [nz], with the PML decay factor applied */
    const double *fdz;                            /* [nbg][nzpml][nx] PML decay (functiondecay) */
    const double *az, *bz;                        /* [nbg][nzpml][nx] vertical PML coefficients */
    const double *ax, *bx;                        /* [nbg][nz][nhx] horizontal PML coefficients */
    const double *c2rho0;                         /* [nbg][nz][nx] if c2d else [nz] */
    const double *v0x, *v0z;                      /* [nbg][nz][nx] or NULL when flows == 0 */
} sparc_background_t;

/* Create / destroy.  Replaces the allocation and FFT planning of Initialize_all
 * (initialize.f90:317-346) and the compact-FD matrix set-up of dbyd2.f:151-196. */
int sparc_plan_create(const sparc_config_t *cfg, sparc_plan_t **plan);
int sparc_plan_destroy(sparc_plan_t *plan);
const char *sparc_last_error(void);

/* Sixth-order compact z-derivative of n1 columns of nz values (FP64, device pointers):
 * dvar = stretch .* dbyd2(var, ibc).  ibc 0..3 as dbyd2.f:19-24; for ibc 2 (3) the row-0
 * (row nz-1) value is taken from preset[n1] (NULL means zero).  stretch NULL means 1.
 * Replaces ddz (derivatives.f90:10-24) and DBYD2 (dbyd2.f:8-235). */
int sparc_ddz(sparc_plan_t *plan, const double *var, double *dvar, int n1, int ibc,
              const double *preset, const double *stretch, void *stream);

/* The kernel-stage z-derivative ddzkern (kernels.f90:648-661): sparc_ddz followed by the
 * FILTER_VAR_Z smoothing of rows 2..nz-1 (kernels.f90:891-928).  FP64 device pointers. */
int sparc_ddzkern(sparc_plan_t *plan, const double *var, double *dvar, int n1, int ibc,
                  const double *stretch, void *stream);

/* Spectral x-derivative of nrows rows of nx values (FP64, device pointers), times stretchx.
 * Replaces ddx (derivatives.f90:28-58). */
int sparc_ddx(sparc_plan_t *plan, const double *var, double *dvar, int nrows, double stretchx,
              void *stream);

/* Upload the background (see sparc_background_t). */
int sparc_set_background(sparc_plan_t *plan, const sparc_background_t *bg, void *stream);

/* Sources (DEVICE pointers, FP64).  The forcing added to RHS v_z at row k_inj at step t is
 *   inj_scale[b][x] * sum_j wts[t][j] * rows[b][idx[t]+j][x],  j = 0..6,
 * rows beyond nrows count as zero.  This covers the forward source vr(x)*fwdsource(t+1)
 * (physics2d.f90:1056-1058, nrows = 1, wts[t][0] = fwdsource(t+1)) and the 7-point
 * Lagrange-interpolated adjoint source (physics.f90:678-737, physics2d.f90:1052-1054).
 * inj_scale = delta_width / rho0(x, k_inj).  wts: [ntab][7], idx: [ntab] (host pointers). */
int sparc_set_source(sparc_plan_t *plan, const double *inj_scale, const double *rows, int nrows,
                     const double *wts, const int *idx, int ntab, void *stream);

/* Zero the state, PML auxiliaries and RHS registers and set the step counter to time0. */
int sparc_reset_state(sparc_plan_t *plan, int time0, void *stream);

/* Advance every solve of the batch by nsteps steps of STEP (step.f90:43-119) inside
 * TIMESTEPPING (driver.f90:351-456).  flow_sign multiplies v0 (+1 forward, -1 for the
 * reference adjoint, driver.f90:144-147).  After each step whose counter is a multiple of
 * steps_out the record a(:,k_obs,v_z) is written to seis (DEVICE, plan precision,
 * [nbatch][nrec_cap][nx]) at index time/steps_out; if snaps is not NULL the partial state of
 * all_modules.f90:750-784 (xi_x, xi_z, v_x, v_z, acc_x, acc_z) goes to snaps
 * ([nbatch][nrec_cap][6][nz][nx]).  Records past nrec_cap are dropped.  use_graph != 0
 * captures one step in a CUDA graph and replays it. */
int sparc_forward(sparc_plan_t *plan, int nsteps, double flow_sign, void *seis, void *snaps,
                  int nrec_cap, int use_graph, void *stream);

/* sparc_forward with a record window: records rec0 .. rec0 + nrec_cap - 1 (the record index is
 * time/steps_out) go to slots 0 .. nrec_cap - 1 of seis / snaps; others are dropped.  With a
 * checkpoint (below) this recomputes one segment of a forward run's partial states
 * (all_modules.f90:750-784) into a buffer of nrec_cap records instead of keeping them all. */
int sparc_forward_window(sparc_plan_t *plan, int nsteps, double flow_sign, void *seis, void *snaps, int rec0,
                         int nrec_cap, int use_graph, void *stream);

/* Checkpoint of everything a step carries to the next: the step counter, the state, the
 * compensated low parts (if any) and the PML auxiliaries of every solve.  The reference has none
 * (it restarts from its partial-state dumps); here the forward field is checkpointed in DEVICE
 * memory every few records and recomputed per segment during the adjoint run.  save / load copy
 * sparc_checkpoint_bytes(plan) bytes to / from a 16-byte aligned DEVICE buffer (stream-ordered). */
size_t sparc_checkpoint_bytes(const sparc_plan_t *plan);
int sparc_checkpoint_save(sparc_plan_t *plan, void *dst, void *stream);
int sparc_checkpoint_load(sparc_plan_t *plan, const void *src, void *stream);

/* The state of solve b: copy the four live fields (xi_x, xi_z, v_x, v_z), each nz*nx of the
 * plan precision, to or from DEVICE memory (for checkpoints and tests). */
int sparc_get_state(sparc_plan_t *plan, void *dst, void *stream);
int sparc_set_state(sparc_plan_t *plan, const void *src, void *stream);

/* Timing of the passes of nsteps steps run without a graph, each launch bracketed by CUDA events
 * on the given stream: ms[0] row passes, ms[1] column passes, ms[2] end-of-step passes,
 * ms[3] wall time of the whole sequence (synchronises the stream; advances the state). */
int sparc_profile_passes(sparc_plan_t *plan, int nsteps, double *ms, void *stream);

/* L2 norm of v_z of every solve, sqrt(sum a(:,:,:,6)^2) (the per-step rms_hist monitor of
 * TIMESTEPPING, driver.f90:364-383), into norms[nbatch] (host).  Returns SPARC_ERR_NONFINITE if
 * any norm is not finite (a diverged solve).  Synchronises the stream. */
int sparc_check_state(sparc_plan_t *plan, double *norms, void *stream);

/* Current step counter (synchronises the stream). */
int sparc_get_time(sparc_plan_t *plan, int *time, void *stream);

/* Diagnostics (no counterpart in the reference): the kernels this plan launches for its column
 * and end-of-step passes and whether each row pass starts on the SMs the column pass's last wave
 * leaves idle, as "column=<kernel> end=<kernel> stage_overlap=<0|1>" (NUL-terminated, at most len
 * bytes).  The overlap is on for FP32 plans of 512 columns with the banded column pass unless
 * SPARC_STAGE_OVERLAP=0 is set when the plan is created. */
int sparc_plan_describe(const sparc_plan_t *plan, char *buf, int len);

/* Kernel construction from paired snapshots (kernels.f90:209-358): for record pair
 * (j, jadj = nadj-1-j), j = 0..npair-1, accumulate in FP64
 *   kc  += div(f_xi) * div(a_v),  kvx += d_x(f_v) . a_v,  kvz += d_z(f_v) . a_v,
 *   hes += |f_acc|^2
 * with d_z filtered by FILTER_VAR_Z (kernels.f90:891-928).  fsn / asn are DEVICE snapshot
 * arrays of the plan precision as written by sparc_forward ([nbatch][nrec][6][nz][nx]);
 * out is DEVICE FP64 [nbatch][4][nz][nx] (kc, kvx, kvz, hes), accumulated into. */
int sparc_kernels(sparc_plan_t *plan, const void *fsn, int nfwd, const void *asn, int nadj,
                  int npair, double *out, void *stream);

/* One record pair of the kernel integral with the plan's CURRENT state as the adjoint fields:
 * forward record jf of fsn ([nbatch][nfwd][6][nz][nx], DEVICE, plan precision) pairs with the
 * adjoint v_x, v_z of every solve as they stand now, accumulating into out as sparc_kernels does.
 * Called after the adjoint step that produces a record, it replaces the adjoint partial-state
 * dumps and their re-reading (all_modules.f90:750-784, kernels.f90:258-280). */
int sparc_kernels_accumulate(sparc_plan_t *plan, const void *fsn, int nfwd, int jf, double *out, void *stream);

/* The adjoint stage of one iteration: the reference's sparc run with the Adjoint instruction
 * (TIMESTEPPING with the flow negated and the Lagrange-interpolated adjoint source, driver.f90:
 * 144-147, 337-475, 584-594; physics.f90:678-737) followed by its kernel stage (PRODUCE_KERNELS,
 * kernels.f90:209-358), without the partial-state dumps between the two.  The plan must be set up
 * for the adjoint (k_inj = o_rad) with its adjoint source already uploaded by sparc_set_source
 * (the residual as source rows, the LAGRANGE_INTERP weights as the table).  Resets the plan,
 * zeroes out (DEVICE FP64 [nbatch][4][nz][nx]), then advances nsteps steps; after the step that
 * writes adjoint record ja (ja = 0 .. nfwd-1, at time ja*steps_out, the first after one step) the
 * integrands of adjoint v_x, v_z against forward record nfwd-1-ja of fsn ([nbatch][nfwd][6][nz][nx],
 * DEVICE, plan precision, as written by sparc_forward) are accumulated into out as
 * sparc_kernels_accumulate does.  Needs 1 + (nfwd-1)*steps_out <= nsteps.  Stream-ordered. */
int sparc_adjoint(sparc_plan_t *plan, const void *fsn, int nfwd, int nsteps, double *out, void *stream);

/* sparc_kernels_accumulate without any device allocation.  No counterpart in the reference:
 * it serves callers that cannot let the library call cudaMalloc during a run: an embedding host
 * whose own allocator owns all device memory, or a run whose device-memory budget is fixed
 * before it starts.  Its scratch (the x-derivatives of one record pair, nbatch*4*nz*nx values of the
 * plan precision) is a file-scope device array of 8 MiB held by every GPU that loads the
 * library until exit; larger batches return SPARC_ERR_SIZE.  The first call on a device looks
 * up the array's address (cudaGetSymbolAddress) and should come before any stream capture; the
 * address is kept per device index for the life of the process, so a reset of the device's
 * context (cudaDeviceReset) after that first call is not supported.
 * Every call reuses the same array: calls that overlap on the GPU (other streams, other
 * plans) race and must be serialised by the caller.  Nothing in the array needs clearing: each
 * call writes every element it reads.  Same arguments and results as sparc_kernels_accumulate. */
int sparc_kernels_accumulate_static(sparc_plan_t *plan, const void *fsn, int nfwd, int jf, double *out,
                                    void *stream);

/* Host-only FP64 evaluation of the banded form of dbyd2 that FP32 plans use on the device:
 * the right-hand side as dbyd2 forms it, then T^{-1} as a Toeplitz band of half-width 20 plus
 * rank-2 corrections on the 24 x 24 corners (ibc 1..3; preset as in sparc_zsolve_host).
 * *band_err (may be NULL) receives max |T^{-1} - band form| / max |T^{-1}|.  (dbyd2.f:8-235) */
int sparc_zband_host(int nz, int ibc, const double *b, double *x, const double *preset, int n1,
                     double *band_err);

/* Dense column operator for the discrete adjoint of the step (FP64, DEVICE pointers): for each
 * of nb planes [nz][nx], out[k][j] = sum_m W[k][m] in[m][j] for columns i0 <= j <= i1 and
 * out[k][j] = in[k][j] for the others; accumulate != 0 adds to out instead.  W is [nz][nz]
 * row-major; in and out must not alias.  With W the transpose of a tabulated ddz (dbyd2.f:8-235
 * times stretch, derivatives.f90:10-24) or of FILTER_VARS_2D's z filter (physics2d.f90:509-583),
 * this applies the adjoint of that operator. */
int sparc_colmat_apply(const double *W, int nz, const double *in, double *out, int nb, int nx, int i0, int i1,
                       int accumulate, void *stream);

/* Host-only FP64 evaluation of the partitioned compact-derivative algebra that the device
 * code applies (no GPU needed): x[nz][n1] = dbyd2(b, ibc) without the stretch factor, with
 * the same chunking as a plan whose chunks hold at most lmax rows.  For validating the
 * precomputed tables against dbyd2.f (dbyd2.f:8-235). */
int sparc_zsolve_host(int nz, int ibc, int lmax, const double *b, double *x, const double *preset, int n1);

/* ---------------------------------------------------------------------------------------------
 * 3-D solver: option 16, MP_FLOWS_PML_3D_DISPL (displacement.f90:377-477) with ddxyz
 * (derivatives.f90:175-305), the 5-stage RK of STEP (step.f90:43-119) and
 * FILTER_VARS_3D_HORIZ_PML after every step of odd index (physics.f90:836-882, step.f90:114).
 * A batch of nbatch independent solves shares the background and the flow.  Device fields are
 * [nz][nbatch][ny][nx] (level-major, x fastest); the state is six of them (xi_x, xi_y, xi_z,
 * v_x, v_y, v_z), in the plan precision.  Laterally uniform background (profiles in z).
 * ------------------------------------------------------------------------------------------- */
typedef struct sparc3d_plan sparc3d_plan_t;

typedef struct {
    int nx, ny, nz, nbatch;    /* nx in the FFT table and a multiple of 16; ny in 64..512 (2, 3) */
    int precision;             /* 32 or 64 */
    int npmlbot, npmltop;      /* vertical PML levels, each >= 5 (params.i:121) */
    double deltat;             /* timestep*dimc/diml (initialize.f90:474) */
    double stretchx, stretchy; /* rsun/xlength, rsun/ylength (initialize.f90:225-226) */
    double betas[5];           /* RK coefficients times deltat (step.f90:34-40) */
    int flows;                 /* 1: advection by v0 (v0 arrays required) */
    int steps_out;             /* record cadence (driver.f90:388) */
    int k_src;                 /* 0-based e_rad: source rows |k - e_rad| <= 4 (displacement.f90:456-462) */
    int k_obs;                 /* 0-based o_rad: recorded level of v_z (driver.f90:391) */
    int filter_every;          /* 2: FILTER_VARS_3D_HORIZ_PML after odd steps (HORIZONTAL_PMLS); 0: none */
} sparc3d_config_t;

/* FP64 device pointers, copied (and rounded for FP32 plans) into the plan.  Profiles are [nz]:
 * stretch (initialize.f90:466-470), rhoinv, rho0, c2rho0 (physics.f90:204-205), gradp0_z,
 * gradrho0_z and g with the PML decay factor applied (physics.f90:206-208, 263-286),
 * source_dep (physics.f90:109); az, bz: [npmlbot + npmltop] (physics.f90:287-288);
 * v0x, v0y, v0z: [nz][ny][nx] (NULL when flows == 0). */
typedef struct {
    const double *stretch, *rhoinv, *rho0, *c2rho0, *gradp0_z, *gradrho0_z, *g, *source_dep;
    const double *az, *bz;
    const double *v0x, *v0y, *v0z;
} sparc3d_background_t;

int sparc3d_plan_create(const sparc3d_config_t *cfg, sparc3d_plan_t **plan);
int sparc3d_plan_destroy(sparc3d_plan_t *plan);
int sparc3d_set_background(sparc3d_plan_t *plan, const sparc3d_background_t *bg, void *stream);

/* Forcing of the RHS of v_z (displacement.f90:456-462): forcing(x, y) * source_dep(k) on rows
 * |k - k_src| <= 4 with forcing = pattern[b][y][x] * amp[step] (0 past the table).  pattern:
 * device FP64 [nbatch][ny][nx]; amp: host [namp].  (The reference assigns forcing only in
 * LAGRANGE_INTERP, physics.f90:678-737: the caller supplies pattern * fwdsource for a forward
 * run, as the 2-D routine injects vr * fwdsource, physics2d.f90:1056-1058.) */
int sparc3d_set_source(sparc3d_plan_t *plan, const double *pattern, const double *amp, int namp, void *stream);

/* Zero the state and PML auxiliaries; the next step has index time0. */
int sparc3d_reset_state(sparc3d_plan_t *plan, int time0, void *stream);

/* nsteps time steps (TIMESTEPPING, driver.f90:337-409).  After each step whose index is a
 * multiple of steps_out, v_z at level k_obs ([nbatch][ny][nx]) is appended to seis (device,
 * plan precision, room for nrec_cap records, may be NULL); *nrec (host, may be NULL) receives
 * the number of records this call made. */
int sparc3d_forward(sparc3d_plan_t *plan, int nsteps, void *seis, int nrec_cap, int *nrec, void *stream);

/* State copy out / in: [6][nz][nbatch][ny][nx] of the plan precision (device). */
int sparc3d_get_state(sparc3d_plan_t *plan, void *dst, void *stream);
int sparc3d_set_state(sparc3d_plan_t *plan, const void *src, void *stream);

/* Kernel-mode adjoint source (displacement.f90:615-627, LAGRANGE_INTERP physics.f90:678-737): at
 * step t the forcing added to RHS v_z at level k_obs is
 *   scale * sum_j wts[t][j] * rows[b][idx[t] + j][y][x],  j = 0..6
 * (rows beyond nrows count as zero; no forcing for t >= ntab), scale = delta_width / rho0(o_rad);
 * it replaces the pattern source.  rows: DEVICE FP64 [nbatch][nrows][ny][nx], kept by pointer
 * (it must stay valid while the plan steps); wts [ntab][7], idx [ntab]: host, copied. */
int sparc3d_set_adjoint_source(sparc3d_plan_t *plan, const double *rows, int nrows, const double *wts, const int *idx,
                               int ntab, double scale, void *stream);

/* sparc3d_forward that also writes kernel-stage records: after a step whose index t is a
 * multiple of steps_out, record j = t / steps_out, if rec0 <= j < rec0 + snap_cap, goes to slot
 * j - rec0 of snaps (DEVICE, plan precision, [snap_cap][5][nz][nbatch][ny][nx]): div xi (x, y
 * and filtered z derivatives, FILTER_VAR_Z kernels.f90:891-928), v_x, v_y, v_z and |acc|^2 of the
 * last stage's RHS of v -- what the kernel integral reads of the forward partial states
 * (kernels.f90:221-280) in a 3-D restatement of the 2-D kernel stage. */
int sparc3d_forward_records(sparc3d_plan_t *plan, int nsteps, void *seis, int nrec_cap, int *nrec, void *snaps,
                            int rec0, int snap_cap, void *stream);

/* One record pair of the 3-D kernel integral (kernels.f90:293-358 with a y term; the reference's
 * kernel stage is 2-D only, kernels.f90:32): with the plan's CURRENT state as the adjoint fields
 * and slot `slot` of snaps (as written by sparc3d_forward_records) as the forward record, add in
 * FP64 to out ([5][nz][nbatch][ny][nx], DEVICE): div xi_f div v_a, sum_j d_x(v_f,j) v_a,j,
 * sum_j d_y(v_f,j) v_a,j, sum_j d_z(v_f,j) v_a,j (z derivatives filtered) and |acc_f|^2. */
int sparc3d_kernels_accumulate(sparc3d_plan_t *plan, const void *snaps, int slot, double *out, void *stream);

/* Checkpoint of what a step carries to the next (state and PML auxiliaries): the reference has
 * none (it restarts from its full dumps).  save copies sparc3d_checkpoint_bytes(plan) bytes to a
 * 16-byte aligned DEVICE buffer and returns the step counter in *time; load restores both. */
size_t sparc3d_checkpoint_bytes(const sparc3d_plan_t *plan);
int sparc3d_checkpoint_save(sparc3d_plan_t *plan, void *dst, int *time, void *stream);
int sparc3d_checkpoint_load(sparc3d_plan_t *plan, const void *src, int time, void *stream);

/* ---------------------------------------------------------------------------------------------
 * 2-D velocity-pressure-density solver: option 5, MP_QUIET_SPONGE_2D (physics2d.f90:1099-1137,
 * a sponge layer, USE_PML off), option 6, MP_QUIET_PML_2D (physics2d.f90:662-713, the
 * vertical PML) or option 12, MP_MHD_PML_2d (physics2d.f90:411-474 with the magnetic part of
 * PML_BOUNDARY_ACCOUNTING_2D, 1162-1200), the RK of STEP and FILTER_VARS_2D on every field.
 * Fields [nz][nbatch][nx]; the state is five of them: rho, v_x, v_y (zero), v_z, p
 * (initialize.f90:500-504), and for option 12 eight: b_x, b_y (zero), b_z follow.
 * ------------------------------------------------------------------------------------------- */
typedef struct sparc5_plan sparc5_plan_t;

typedef struct {
    int nx, nz, nbatch, precision;  /* nx in the FFT table; nz >= 11; precision 32 or 64 */
    int npmlhor;                    /* FILTER_VARS_2D columns [npmlhor, nx-npmlhor+1] (HORIZONTAL_PMLS) */
    int filter_all_x;               /* 1: filter every column */
    double deltat, stretchx;        /* as sparc_config_t */
    double betas[5];
    int steps_out, k_src, k_obs;    /* record cadence, 0-based e_rad, o_rad */
    int option;                     /* 5: MP_QUIET_SPONGE_2D (physics2d.f90:1099-1137);
                                       6: MP_QUIET_PML_2D (physics2d.f90:662-713);
                                       12: MP_MHD_PML_2d (physics2d.f90:411-474) */
    int npmlbot, npmltop;           /* vertical PML levels (options 6 and 12) */
} sparc5_config_t;

/* FP64 device profiles [nz]: stretch, rhoinv, rho0, c2rho0, gradp0_z, gradrho0_z, g (no PML
 * decay), source_dep, sponge (spongez, physics2d.f90:62-69). */
typedef struct {
    const double *stretch, *rhoinv, *rho0, *c2rho0, *gradp0_z, *gradrho0_z, *g, *source_dep, *sponge;
    const double *az, *bz;  /* [npmlbot + npmltop] (physics2d.f90:288-332), options 6 and 12 */
    const double *box, *boz; /* option 12: background field [nz][nx], B / dimb (initialize.f90:759);
                                curlboy = d box/dz - d boz/dx is formed on the device
                                (physics2d.f90:166-168) */
} sparc5_background_t;

int sparc5_plan_create(const sparc5_config_t *cfg, sparc5_plan_t **plan);
int sparc5_plan_destroy(sparc5_plan_t *plan);
int sparc5_set_background(sparc5_plan_t *plan, const sparc5_background_t *bg, void *stream);
/* forcing(x, step) = pattern[b][x] * amp[step] times source_dep(k) on rows |k - k_src| <= 4
 * (physics2d.f90:1124-1128); pattern device FP64 [nbatch][nx], amp host [namp]. */
int sparc5_set_source(sparc5_plan_t *plan, const double *pattern, const double *amp, int namp, void *stream);
int sparc5_reset_state(sparc5_plan_t *plan, int time0, void *stream);
/* nsteps steps; v_z at k_obs ([nbatch][nx]) appended to seis after each step whose index is a
 * multiple of steps_out. */
int sparc5_forward(sparc5_plan_t *plan, int nsteps, void *seis, int nrec_cap, int *nrec, void *stream);
/* [nf][nz][nbatch][nx] of the plan precision (device): nf = 5, or 8 for option 12. */
int sparc5_get_state(sparc5_plan_t *plan, void *dst, void *stream);

/* ---------------------------------------------------------------------------------------------
 * Travel-time adjoint source (ADJOINT_SOURCE_FILT, driver.f90:1758-2238), FP64, for a batch of
 * sources.  Records are [nbatch][nt][nx] (x fastest; nt records of vz at o_rad), device.
 * ------------------------------------------------------------------------------------------- */
typedef struct sparc_tt_plan sparc_tt_plan_t;

/* nx in the FFT table; nt (records) in 2..860; max_rows: most receivers measured by one mode
 * call over the batch. */
int sparc_tt_plan_create(int nx, int nt, int nbatch, int max_rows, sparc_tt_plan_t **plan);
int sparc_tt_plan_destroy(sparc_tt_plan_t *plan);

/* Forward (x, t) transforms of the synthetic and observed records (driver.f90:1838-1844) and a
 * zero adjoint source. */
int sparc_tt_set_records(sparc_tt_plan_t *plan, const double *synth, const double *data, void *stream);

/* One ridge filter ("mode", driver.f90:1948-2113): filter [nt][nx] device, real (the ridge times
 * its frequency filter).  rows: host [nrows][7] = source b, receiver x (0-based), search range
 * timest, timefin (1-based, clipped to the record), lef, rig (1-based window: in when given,
 * out otherwise), loc (out: the picked maximum); halftime = nint(window / (2 dt)); dt_min = the
 * record cadence in minutes.  tau: host [nrows] out, travel-time shifts in minutes (COMPUTE_TT_
 * GIZONBIRCH, driver.f90:894-940).  The mode's contribution is added, time-reversed, to the
 * adjoint source.  Waits for the stream. */
int sparc_tt_mode(sparc_tt_plan_t *plan, const double *filter, int nrows, int *rows, int halftime, int given,
                  double dt_min, double *tau, void *stream);

/* MISFIT_ALL (driver.f90:2294-2651) for one ridge filter of one frequency band: filter as in
 * sparc_tt_mode; rows as in sparc_tt_mode with the window loc -+ halftime not clipped; tau: host
 * [nrows] out, COMPUTE_TT (driver.f90:855-890) cross-correlation travel times in minutes, NaN
 * where the window leaves the record or the correlation peak sits at the end of its lag range
 * (the reference reads past its arrays there).  Does not touch the adjoint source. */
int sparc_tt_misfit_mode(sparc_tt_plan_t *plan, const double *filter, int nrows, int *rows, int halftime,
                         int given, double dt_min, double *tau, void *stream);

/* The adjoint source of every source, [nbatch][nt][nx] device, times nt / 60 (driver.f90:2201),
 * in the reference's time-reversed order (ready for source.fits). */
int sparc_tt_adjoint(sparc_tt_plan_t *plan, double *adj, void *stream);

/* ---------------------------------------------------------------------------------------------
 * FITS payloads on the device: n values of a device array (FP32 or FP64) to / from the
 * big-endian IEEE payload of a FITS primary array (BITPIX -64 or -32), device to device.  The
 * partial-state files of the reference's forward / adjoint runs and kernel stage
 * (WRITE_OUT_PARTIAL_STATE all_modules.f90:750-784, readfits kernels.f90:221-280, writefits /
 * readfits all_modules.f90:99-378) are these payloads behind a 2880-byte header.
 * ------------------------------------------------------------------------------------------- */
int sparc_fits_encode(const void *src, int precision, long long n, int bitpix, void *dst, void *stream);
int sparc_fits_decode(const void *src, int bitpix, long long n, void *dst, int precision, void *stream);

/* ---------------------------------------------------------------------------------------------
 * Gradient post-processing (replaces grad.py's array work, grad.py:42-117, 188-364).  Every
 * array is FP64 on the device, x-fastest [nz][nx] as the kernels above; no call allocates: the
 * caller passes a workspace of sparc_grad_workspace_bytes(nx, nz) bytes (the vector calls need
 * sparc_grad_workspace_bytes(0, 0)).  Reductions are deterministic: fixed block count, fixed
 * summation order, independent of the stream and of earlier calls.
 * ------------------------------------------------------------------------------------------- */
#define SPARC_SYM_NONE 0
#define SPARC_SYM_SYM 1        /* symmetrize: 0.5 (a + a reversed in x) (grad.py:101) */
#define SPARC_SYM_ASYM (-1)    /* antisymmetrize: 0.5 (a - a reversed in x) (grad.py:100) */
#define SPARC_ZFILT_NONE 0
#define SPARC_ZFILT_GAUSSIAN 1 /* scipy gaussian_filter1d along z, mode reflect, truncate 4 */
#define SPARC_ZFILT_SMOOTH 2   /* grad.py's 11-point filter 'smooth' (grad.py:66-87), nz >= 11 */

typedef struct {
    int nx, nz;          /* grid; nx in the FFT table (64..1024, factors 2 and 3) */
    int nsrc;            /* number of per-source kernels and hessians to sum */
    double nk;           /* filterx width in wavenumbers (grad.py:111: 30) */
    int sym;             /* SPARC_SYM_* (grad.py:112-115; main uses ASYM, grad.py:200) */
    int zfilt;           /* SPARC_ZFILT_* (main: GAUSSIAN, grad.py:200) */
    double zsigma;       /* Gaussian width in rows (grad.py:200: 2.0); radius int(4 sigma + 0.5) <= 32 */
    double hess_floor;   /* floor of the normalised preconditioner (grad.py:196: 5e-3) */
    int precondition;    /* 1: H as grad.py main forms it (below); 0: H = sum_s hessians[s] used
                            as given, rho ignored (filter_and_symmetrize(totkern, hess),
                            grad.py:109-117) */
} sparc_grad_config_t;

/* Workspace bytes for sparc_gradient on an nx x nz grid (and for the vector calls). */
unsigned long long sparc_grad_workspace_bytes(int nx, int nz);

/* The gradient of grad.py's main (grad.py:188-202, 109-117), precondition = 1:
 *   K = sum_s kernels[s],  H = sum_s |hessians[s]| * rho[k],  H <- max(H / max H, hess_floor),
 *   grad = zfilter(sym(filterx(K / H, nk))).
 * kernels, hessians: [nsrc][nz][nx]; rho: [nz] device (column 3 of the model file);
 * grad: [nz][nx]. */
int sparc_gradient(const sparc_grad_config_t *cfg, const double *kernels, const double *hessians,
                   const double *rho, double *grad, void *work, void *stream);

/* *result (host) = sum_i a[i] * (b[i] - c[i]), or sum_i a[i] * b[i] when c is NULL.  Waits for
 * the stream.  (np.sum(grad * (grad - lastgrad)), grad.py:227-233) */
int sparc_vec_dot(long long n, const double *a, const double *b, const double *c, double *result,
                  void *work, void *stream);

/* y[i] = alpha * x[i] + beta * z[i] (z may be NULL: y = alpha x); y may alias x or z. */
int sparc_vec_axpby(long long n, double alpha, const double *x, double beta, const double *z, double *y,
                    void *stream);

/* Update direction (grad.py:204-250).  algo 0: steepest descent, p = -g; 1: conjugate gradient,
 * Polak-Ribiere (the reference's choice, grad.py:222-228), p = -g + beta p_prev with
 * beta = g.(g - g_prev) / g_prev.g_prev; 2: Hestenes-Stiefel (grad.py:230-233),
 * beta = g.(g - g_prev) / (g - g_prev).p_prev.  *beta (host, may be NULL) receives beta (0 for
 * algo 0).  Waits for the stream for algo 1 and 2. */
int sparc_update_direction(int algo, long long n, const double *g, const double *g_prev, const double *p_prev,
                           double *p, double *beta, void *work, void *stream);

/* L-BFGS direction p = -H g by the two-loop recursion over npairs (<= 64) pairs s[i] =
 * m_{i+1} - m_i, y[i] = g_{i+1} - g_i, oldest first, H0 = (s.y / y.y) of the newest pair.
 * s, y: HOST arrays of device pointers.  p must not alias g, s or y.  (grad.py:257-325 sets out
 * to compute this with m = 4; its own code cannot run: np.dot with one argument.)  Waits for
 * the stream. */
int sparc_lbfgs_direction(long long n, int npairs, const double *const *s, const double *const *y,
                          const double *g, double *p, void *work, void *stream);

/* Line-search models (grad.py:351-364, kind 'linear'):
 *   out[e][i] = model[i] + eps[e] * (update[i] / max(update)) * rms(model),
 * max(update) signed and skipped when 0, rms(model) = sqrt(sum model^2 / n) replaced by 1 when
 * 0.  eps: host [neps]; out: device [neps][n].  Waits for the stream. */
int sparc_linesearch_models(long long n, const double *model, const double *update, int neps, const double *eps,
                            double *out, void *work, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SPARC_GB300_H */
