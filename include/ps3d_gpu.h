/*
 * ps3d_gpu.h - C ABI of the GB300 (sm_103a) implementation of the ps3d
 * per-step vorticity right-hand side and time steppers.
 *
 * The reference (matt-frey/ps3d) keeps this path in Fortran module procedures
 * that act on module-global arrays.  This header is the drop-in boundary a
 * Fortran `iso_c_binding` interface (or ctypes/cffi) binds: plain pointers,
 * sizes and int status codes, no C++ or torch types.  Every routine below
 * names the reference procedure it replaces.
 *
 * Host arrays use the reference layout (src/fields/fields.f90:59-79): a
 * scalar field is (0:nz, 0:ny-1, 0:nx-1), column-major, z fastest, i.e. the
 * element (iz, iy, ix) sits at iz + (nz+1)*(iy + ny*ix); a vector field is
 * three scalar fields back to back.  Host arrays are only read or written
 * during a call; no host pointer is retained.
 *
 * Threading: one context per host thread; calls on one context are not
 * thread-safe.  Each context owns its device buffers and its CUDA stream.
 * Errors: every entry point returns PS3D_OK (0) or a PS3D_ERR_* code; the
 * library never aborts the process and never traps on the device.
 */
#ifndef PS3D_GPU_H
#define PS3D_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define PS3D_OK 0
#define PS3D_ERR_INVALID_ARG 1      /* bad pointer, enum or size            */
#define PS3D_ERR_UNSUPPORTED_SIZE 2 /* grid the kernels do not implement    */
#define PS3D_ERR_CUDA 3             /* CUDA runtime error (see last_error)  */
#define PS3D_ERR_OUT_OF_MEMORY 4    /* device allocation failed             */
#define PS3D_ERR_NOT_READY 5        /* e.g. step before init_diffusion      */
#define PS3D_ERR_NONFINITE 6        /* NaN/Inf detected in a diagnostic     */
#define PS3D_ERR_DEVICE_LIMIT 7     /* a bounded device loop hit its limit  */
#define PS3D_ERR_NO_DEVICE 8        /* no CUDA device / wrong architecture  */

/* ---- enums (string options of the &PS3D namelist, options.f90) --------- */
#define PS3D_PRE_CONSTANT 0              /* pretype 'constant'             */
#define PS3D_PRE_VORCH 1                 /* 'vorch'                        */
#define PS3D_PRE_BFMAX 2                 /* 'bfmax' (0: no buoyancy)       */
#define PS3D_PRE_ROLL_MEAN_MAX_STRAIN 3  /* 'roll-mean-max-strain'         */
#define PS3D_PRE_MAX_STRAIN 4            /* 'max-strain'                   */
#define PS3D_PRE_US_MAX_STRAIN 5         /* 'us-max-strain'                */
#define PS3D_PRE_ROLL_MEAN_BFMAX 6       /* 'roll-mean-bfmax' (buoyancy)   */
#define PS3D_KOLMOGOROV 0                /* length_scale                   */
#define PS3D_GEOPHYSICAL 1
#define PS3D_HOU_LI 0                    /* filtering 'Hou & Li'           */
#define PS3D_TWO_THIRDS 1                /* filtering '2/3-rule'           */
#define PS3D_IMPL_DIFF_RK4 0             /* stepper 'impl-diff-rk4'        */
#define PS3D_CN2 1                       /* stepper 'cn2'                  */
#define PS3D_PRECISION_FP64 0            /* every field and transform FP64 */
#define PS3D_PRECISION_MIXED 1           /* FP32 transforms/products/stage
                                            arithmetic; FP64 prognostic
                                            vorticity, RK accumulators,
                                            low-mode inversion, reductions */

/* Run configuration: the hot-path subset of the &PS3D namelist
 * (src/utils/options.f90:11-96) and the box (src/utils/parameters.f90).
 * The first 17 members match the oracle's ps3o_config field for field. */
typedef struct {
    int nx, ny, nz;             /* cells; even, factors 2, 3, 5; 8..2048     */
    int nnu;                    /* vor_visc%nnu                              */
    double lower[3];            /* box lower corner                          */
    double extent[3];           /* box extent                                */
    double prediss;             /* vor_visc%prediss                          */
    int pretype;                /* PS3D_PRE_*                                */
    int length_scale;           /* PS3D_KOLMOGOROV | PS3D_GEOPHYSICAL        */
    int filtering;              /* PS3D_HOU_LI | PS3D_TWO_THIRDS             */
    int stepper;                /* PS3D_IMPL_DIFF_RK4 | PS3D_CN2             */
    double cflmax;              /* reference constant 0.8 (constants.f90:47) */
    double alpha;               /* time%alpha                                */
    double time_limit;          /* time%limit                                */
    int roll_mean_win_size;     /* vor_visc%roll_mean_win_size               */
    int nthreads;               /* unused on the GPU (oracle compatibility)  */
    int hold_source;            /* test hook: keep svorts fixed in step()    */
    double f_cor[3];            /* planetary vorticity (physics.f90:61)      */
    int precision;              /* PS3D_PRECISION_*                          */
    int device;                 /* CUDA device ordinal                       */
    /* Buoyancy (the reference configured with --enable-buoyancy,
     * configure.ac:213-223): a Boussinesq buoyancy perturbation b' about the
     * basic state N^2 z is stepped with the vorticity. */
    int buoyancy;               /* 0: vorticity only                         */
    double bfsq;                /* N^2 (physics.f90:90-94)                   */
    int bfsq_given;             /* 0: N^2 from the initial buoyancy
                                   (calculate_basic_reference_state)         */
    int buoy_nnu;               /* buoy_visc%nnu (options.f90:78-80)         */
    double buoy_prediss;        /* buoy_visc%prediss                         */
    int buoy_pretype;           /* buoy_visc%pretype, PS3D_PRE_*             */
    int buoy_length_scale;      /* buoy_visc%length_scale                    */
    int buoy_roll_mean_win_size;/* buoy_visc%roll_mean_win_size              */
} ps3d_gpu_config;

/* Diagnostics of one adapt() call (src/stepper/advance.f90:109-377) plus the
 * kinetic energy, enstrophy (field_diagnostics.f90:85-206) and helicity
 * <u.omega> (no reference counterpart; same z-trapezoid weights). */
typedef struct {
    double t, dt;
    double ke, en, hel;
    double vortmax, vortrms, vorch;
    double vormean[3];
    double ggmax, usggmax, lsggmax;
    double umax, vmax, wmax;
    double bfmax, rmv, pref;
    double rmb, bpref;          /* buoyancy: rolling mean of bfmax (advance.f90:358-361)
                                   and the buoyancy prefactor (:370-373)     */
} ps3d_gpu_diag;

typedef struct ps3d_gpu_ctx ps3d_gpu_ctx;

/* ---- lifetime ----------------------------------------------------------
 * create: init_inversion (inversion_utils.f90:222-372) + initialise_fft
 * (sta3dfft.f90:53-110) + field_alloc (fields.f90:45-84).  nx, ny, nz:
 * even, 8..2048 (nz up to 1024 in the FP64 form), prime factors 2, 3 and 5
 * only (factorisen, stafft.f90:128-187); otherwise PS3D_ERR_UNSUPPORTED_SIZE. */
int ps3d_gpu_create(const ps3d_gpu_config *cfg, ps3d_gpu_ctx **ctx);
int ps3d_gpu_destroy(ps3d_gpu_ctx *ctx);
const char *ps3d_gpu_strerror(int status);
const char *ps3d_gpu_last_error(const ps3d_gpu_ctx *ctx);
/* device bytes held by the context */
long long ps3d_gpu_device_bytes(const ps3d_gpu_ctx *ctx);

/* ---- state transfer ----------------------------------------------------
 * which: 0 svor (mixed-spectral vorticity), 1 vor, 2 vel (physical),
 * 3 svel (semi-spectral velocity), 4 svorts (vorticity source); 3 fields each
 * (fields.f90:17-23).  Mixed precision converts at the boundary. */
#define PS3D_FIELD_SVOR 0
#define PS3D_FIELD_VOR 1
#define PS3D_FIELD_VEL 2
#define PS3D_FIELD_SVEL 3
#define PS3D_FIELD_SVORTS 4
/* buoyancy contexts (one scalar field each, fields.f90:25-31): sbuoy
 * (mixed-spectral b'), buoy (physical b'), sbuoys (its source) */
#define PS3D_FIELD_SBUOY 5
#define PS3D_FIELD_BUOY 6
#define PS3D_FIELD_SBUOYS 7
int ps3d_gpu_set_field(ps3d_gpu_ctx *ctx, int which, const double *host);
int ps3d_gpu_get_field(ps3d_gpu_ctx *ctx, int which, double *host);
int ps3d_gpu_set_ini_vor_mean(ps3d_gpu_ctx *ctx, const double v[2]);
int ps3d_gpu_get_ini_vor_mean(ps3d_gpu_ctx *ctx, double v[2]);
/* tables, numbering as the oracle: 0 k2l2, 1 k2l2i, 2 filt, 3 green, 4 phim,
 * 5 phip, 6 thetam, 7 thetap, 8 dthetam, 9 dthetap, 10 gamtop, 11 gambot,
 * 12 vhdis, 13 rkx, 14 rky, 15 rkz (inversion_utils.f90:222-372); buoyancy
 * contexts: 16 dphim, 17 dphip, 18 bhdis, 19 bbarz (N^2 z). */
int ps3d_gpu_get_table(ps3d_gpu_ctx *ctx, int which, double *host);

/* ---- reference procedures ---------------------------------------------- */
/* setup_fields (utils.f90:136-184): decompose the physical vorticity
 * vor_phys (3 fields), add the optional mixed-spectral perturbation pert
 * (3 fields, may be NULL), record ini_vor_mean, vor2vel, then te = kinetic
 * energy, en = enstrophy and init_diffusion(te, en). */
int ps3d_gpu_setup_fields(ps3d_gpu_ctx *ctx, const double *vor_phys,
                          const double *pert, double *te, double *en);
/* setup_fields of a buoyancy context (utils.f90:136-184): buoy_phys is the
 * total physical buoyancy (1 field); N^2 from it unless bfsq_given
 * (physics.f90:310-340), the basic state N^2 z removed and decomposed into
 * sbuoy, then as above with te = kinetic + available potential energy
 * (linear stratification, ape_density.f90:31-32) and en = enstrophy + the
 * buoyancy-gradient integral (field_diagnostics.f90:351-397).  On a context
 * without buoyancy this is ps3d_gpu_setup_fields (buoy_phys ignored). */
int ps3d_gpu_setup_fields_buoyancy(ps3d_gpu_ctx *ctx, const double *vor_phys, const double *pert,
                                   const double *buoy_phys, double *te, double *en);
/* N^2 and the buoyancy viscosity bvisc of a buoyancy context */
int ps3d_gpu_buoyancy_params(ps3d_gpu_ctx *ctx, double *bfsq, double *bvisc);
/* init_diffusion (inversion_utils.f90:124-153), vorticity and buoyancy */
int ps3d_gpu_init_diffusion(ps3d_gpu_ctx *ctx, double te, double en);
/* vor2vel (inversion.f90:23-226) */
int ps3d_gpu_vor2vel(ps3d_gpu_ctx *ctx);
/* source (inversion.f90:376-388): buoyancy_tendency (:232-292) on buoyancy
 * contexts, then vorticity_tendency (:298-371).  svorts is left
 * unprojected, as the reference leaves it; the mixed form also keeps the z
 * part of the tendency's solenoidal projection, which its stage updates
 * use to project each source term as they apply it. */
int ps3d_gpu_source(ps3d_gpu_ctx *ctx);
/* adapt (advance.f90:109-377) incl. set_diffusion of the stepper */
int ps3d_gpu_adapt(ps3d_gpu_ctx *ctx, double t, double *dt, ps3d_gpu_diag *diag);
/* base_stepper%set_diffusion (impl_rk4.f90:37-53, cn2.f90:40-77) with the
 * vorticity prefactor (the buoyancy prefactor 0) */
int ps3d_gpu_set_diffusion(ps3d_gpu_ctx *ctx, double dt, double pref);
/* set_diffusion(dt, vorch, bf) with both prefactors */
int ps3d_gpu_set_diffusion_vb(ps3d_gpu_ctx *ctx, double dt, double vpref, double bpref);
/* base_stepper%step (impl_rk4.f90:76-207, cn2.f90:92-181) */
int ps3d_gpu_step(ps3d_gpu_ctx *ctx, double *t, double dt);
/* advance (advance.f90:77-104) repeated nsteps times; diag (nullable) gets
 * nsteps records, one per step, taken by adapt at the start of the step. */
int ps3d_gpu_advance(ps3d_gpu_ctx *ctx, double *t, int nsteps, ps3d_gpu_diag *diag);
/* One advance for a caller that owns the state on the host (the Fortran
 * driver's arrays): upload svor (3 fields), advance once, download svor.
 * A state bitwise equal to the device's (the previous call's result) is
 * taken as it is; any other state is projected first, as set_field does.
 * Page-locked svor (ps3d_gpu_host_alloc, 16-byte aligned) is read and
 * written over the host link by the library's kernels; in the mixed form
 * the upload and its comparison run on a second stream beside the step's
 * first right-hand side, which is evaluated again from the new state when
 * the comparison finds a difference.  PS3D_ERR_INVALID_ARG on a buoyancy
 * context (its state includes sbuoy). */
int ps3d_gpu_advance_host(ps3d_gpu_ctx *ctx, double *svor, double *t, ps3d_gpu_diag *diag);
/* calc_vorticity_mean / adjust_vorticity_mean (field_diagnostics.f90:584-619) */
int ps3d_gpu_calc_vorticity_mean(ps3d_gpu_ctx *ctx, double out[2]);
int ps3d_gpu_adjust_vorticity_mean(ps3d_gpu_ctx *ctx);
/* get_kinetic_energy, get_enstrophy and helicity of the current vel/vor */
int ps3d_gpu_energy_series(ps3d_gpu_ctx *ctx, double *ke, double *en, double *hel);

/* ---- single-field operators (host in/out, one scalar field) ------------ */
#define PS3D_OP_FFTXYP2S 0        /* sta3dfft.f90:136-194                   */
#define PS3D_OP_FFTXYS2P 1        /* sta3dfft.f90:202-260                   */
#define PS3D_OP_DIFFX 2           /* sta3dfft.f90:304-339 + reverse_x       */
#define PS3D_OP_DIFFY 3           /* sta3dfft.f90:345-377 + reverse_y       */
#define PS3D_OP_FFTSINE 4         /* sta3dfft.f90:264-277                   */
#define PS3D_OP_FFTCOSINE 5       /* sta3dfft.f90:282-298                   */
#define PS3D_OP_CENTRAL_DIFFZ 6   /* inversion_utils.f90:653-673            */
#define PS3D_OP_DECOMPOSE_SEMI 7  /* inversion_utils.f90:563-595            */
#define PS3D_OP_COMBINE_SEMI 8    /* inversion_utils.f90:617-647            */
#define PS3D_OP_DECOMPOSE_PHYS 9  /* inversion_utils.f90:549-557            */
#define PS3D_OP_COMBINE_PHYS 10   /* inversion_utils.f90:599-611            */
#define PS3D_OP_DIFFZ 11          /* inversion_utils.f90:683-719 (buoyancy
                                     contexts only)                         */
int ps3d_gpu_field_op(ps3d_gpu_ctx *ctx, int op, const double *in, double *out);

/* ---- benchmark helpers ------------------------------------------------- */
/* Time nsteps advance() calls on the context stream with CUDA events (the
 * state stays resident); *ms is the elapsed device time. */
int ps3d_gpu_time_advance(ps3d_gpu_ctx *ctx, double *t, int nsteps, double *ms);
/* Kernel launches issued by this context since creation. */
long long ps3d_gpu_launch_count(const ps3d_gpu_ctx *ctx);
int ps3d_gpu_synchronize(ps3d_gpu_ctx *ctx);
/* Derived fields (src/fields/fields_derived.f90:67-182) from the current
 * vel, vor and svel (call after ps3d_gpu_vor2vel, as the reference's adapt
 * does): pres solves Lap(p) = 2[J_xy(u,v) + J_yz(v,w) + J_zx(w,u)] with
 * dp/dz = 0 on the walls (buoyancy contexts add b'_z + f_z zeta to the
 * right-hand side and the harmonic boundary terms of b', :108-151);
 * delta = du/dx + dv/dy.  Physical host arrays (nz+1, ny, nx) column-major;
 * NULL skips one. */
int ps3d_gpu_derived_fields(ps3d_gpu_ctx *ctx, double *pres, double *delta);

/* Buoyancy diagnostics of the current state (field_diagnostics.f90, buoyancy
 * contexts): out[0] available potential energy (:29-60, linear
 * stratification b'^2 / (2 N^2)), out[1] buoyancy-gradient integral
 * (:351-397; the reference's |grad b| is sqrt(b_x^2 + 2 b_y^2), its z term
 * being overwritten at :369-370), out[2] minimum static stability
 * 1 + min(b'_z) / N^2 (:327-344), out[3] minimum Richardson number
 * min((N^2 + b'_z) / (xi^2 + eta^2)) (:268-287, from the current vor). */
int ps3d_gpu_buoyancy_diagnostics(ps3d_gpu_ctx *ctx, double out[4]);

/* Kinetic-energy shell spectrum (src/genspec.f90:42-123) of the current
 * vel: squared spectral amplitudes (dct of u, v and dst of w along z) summed
 * into shells of |K| = nint(sqrt(kx^2 + ky^2 + kz^2)), scaled by shell volume
 * over count and normalised so that sum(spec) * dk is the domain-average
 * kinetic energy.  nbins = kmax + 1 shells (at most nmax written). */
int ps3d_gpu_ke_spectrum(ps3d_gpu_ctx *ctx, int nmax, double *spec, int *nbins, double *dk);

/* Page-locked host memory from the library's CUDA runtime (no reference
 * counterpart): host arrays passed to ps3d_gpu_advance_host (or any
 * transfer) move at the full host-device bandwidth when allocated here; a
 * Fortran driver can map its svor onto it with c_f_pointer. */
int ps3d_gpu_host_alloc(size_t bytes, void **ptr);
int ps3d_gpu_host_free(void *ptr);

/* Captured steps (no reference counterpart): nsteps advances of the mixed
 * form with impl-diff-rk4, each one CUDA graph launch with adapt's scalar
 * logic on the device (no host synchronisation inside a step).  Same
 * arithmetic as ps3d_gpu_advance.  t in/out; diag (optional) receives the
 * last step's diagnostics, ms (optional) the device time.  A non-finite
 * diagnostic or a Jacobi limit is reported after the launches
 * (PS3D_ERR_NONFINITE / PS3D_ERR_DEVICE_LIMIT; the state is then invalid).
 * PS3D_ERR_INVALID_ARG for the FP64 form, cn2, a held source or buoyancy. */
int ps3d_gpu_advance_graph(ps3d_gpu_ctx *ctx, double *t, int nsteps, ps3d_gpu_diag *diag, double *ms);
/* Batching (no reference counterpart): nsteps steps of n independent
 * contexts (any grid sizes, one device; the conditions of
 * ps3d_gpu_advance_graph), each step one CUDA graph for the whole batch:
 * every run's right-hand sides on the run's own stream, and each of the
 * four stage updates one persistent launch over the (run, partner orbit)
 * work items of all runs.  The graph is captured on the first call and
 * kept (by ctx[0]) while the same contexts come in the same order.  The
 * states equal those of the runs stepped alone, bitwise.  t[n] in/out; ms =
 * device time of the whole batch.  A context listed twice is
 * PS3D_ERR_INVALID_ARG. */
int ps3d_gpu_batch_advance(ps3d_gpu_ctx *const *ctx, int n, double *t, int nsteps, double *ms);

/* Line-FFT autotuner (no reference counterpart): at creation the mixed form
 * times each kernel shape of the FP32 line FFTs where a line length has more
 * than one, for the passes forward y, forward x, inverse y, inverse x, and
 * keeps the fastest.  Shapes: 0 the default blocks (at 512 points 512
 * threads, two per SM), 1 256-thread blocks, three per SM (512 points), 2
 * the TMA-fed persistent kernel (128, 256 and 512 points: one block per SM
 * with two tile buffers, tensor copies of the next tile overlapping the
 * current one's butterflies).  shape[4]: the choice per pass (-1 = the
 * only shape); ms[12]: ms per launch of shapes 0, 1, 2 per pass (0 = not
 * timed). */
int ps3d_gpu_tuning(ps3d_gpu_ctx *ctx, int shape[4], double ms[12]);
/* Pin the line-FFT block shapes (e.g. for reproducible timings); -1 = the
 * default shape.  PS3D_ERR_INVALID_ARG for a shape the line length lacks. */
int ps3d_gpu_set_tuning(ps3d_gpu_ctx *ctx, const int shape[4]);

/* Kernel probe: bracket every launch of one kernel class with CUDA events on
 * the context stream.  kind: 0 off, 1 y-line transforms, 2 x-line
 * transforms, 3 column (z) transforms, 4 line transforms of both
 * directions, 5 the mixed source's products formed in its forward y-line
 * kernel.  probe resets the counters;
 * probe_result returns the summed device time, the number of bracketed
 * launches and their algorithmic bytes (the fields each launch must read
 * and write, nx*ny*(nz+1) elements per field: two for a transform pass). */
int ps3d_gpu_probe(ps3d_gpu_ctx *ctx, int kind);
int ps3d_gpu_probe_result(ps3d_gpu_ctx *ctx, double *total_ms, long long *launches, double *bytes);

/* ---- energy series without device allocation ---------------------------
 * No counterpart in the reference.  For callers that keep vel and vor in
 * device arrays they manage themselves and cannot let the library allocate
 * (a device-resident CUDA Fortran/OpenACC time loop, a fixed device-memory
 * budget, or code that must not call cudaMalloc/cudaFree because they
 * synchronise the device).  Computes the kinetic energy, enstrophy and
 * helicity of ps3d_gpu_energy_series from caller-owned FP64 device fields:
 * component c, level iz, column (iy, ix) at c*comp_stride + iz +
 * pitch*(iy + ny*ix), pitch >= nz+1 (nz+1 is the reference layout).  Writes
 * out[0..2] (device memory) on `stream` (a cudaStream_t, NULL for the legacy
 * default stream) and returns without synchronising.
 * Scratch: a fixed array in the library's device image (about 6 MB per GPU
 * that loads the library), so nx*ny may not exceed 524288 (returns
 * PS3D_ERR_UNSUPPORTED_SIZE beyond that).  Every call looks up that array's
 * address in the current device's context (cudaGetSymbolAddress); the first
 * call on a device may load the library's device code into the context and
 * should therefore come before any stream capture.  pitch above INT_MAX or
 * comp_stride below pitch*nx*ny is PS3D_ERR_INVALID_ARG.  All calls share
 * the array: calls that overlap on the GPU race.  No context is needed and
 * nothing is allocated. */
int ps3d_gpu_energy_series_noalloc(const double *vel, const double *vor, int nx, int ny, int nz,
                                   long long pitch, long long comp_stride, void *stream, double *out);

/* ---- checkpoint ----------------------------------------------------------
 * Raw-binary checkpoint of a context's run state: svor (FP64, and the FP32
 * copy of the mixed form), sbuoy, the rolling means of adapt, ini_vor_mean,
 * the viscosities and hyperdiffusion tables, N^2 and the model time t.  A
 * context of the same grid, box, form and configuration that loads it
 * continues the run bitwise.  Replaces, for the GPU state, the reference's
 * restart from a NetCDF field file (utils.f90:102-116, field_netcdf.f90:
 * 276-300), which starts its rolling means afresh.  Errors: PS3D_ERR_INVALID_ARG
 * for an unreadable, truncated or mismatched file (see last_error). */
int ps3d_gpu_save_state(ps3d_gpu_ctx *ctx, const char *path, double t);
int ps3d_gpu_load_state(ps3d_gpu_ctx *ctx, const char *path, double *t);

/* ---- learned sub-grid closure --------------------------------------------
 * No counterpart in the reference, whose only sub-grid model is the
 * horizontal hyperdiffusion of init_diffusion (inversion_utils.f90:124-218);
 * that hyperdiffusion stays in force and is the fallback whenever no
 * closure is attached.
 *
 * The network maps the physical vorticity and velocity of a run, each
 * divided by its rms over the grid points (6 input channels), to a
 * vorticity-tendency correction in physical space (3 channels): four
 * 3x3x3 convolutions (periodic in x and y, zero-padded in z), widths
 * 6 -> 32 -> 32 -> 32 -> 3, GELU after the first three.  Weights and
 * activations are BF16 on tensor cores with FP32 accumulation; the FP32
 * master parameters and the Adam moments stay on the device.  The output
 * is scaled by ct * <|omega|^2> (ct fixed from the training targets), then
 * taken to the mixed-spectral form and added to svorts.
 *
 * Parameter vector (FP32, PS3D_CLOSURE_NPARAM values): for each layer its
 * weights W[tap][ci][co] (tap = (dx+1)*9 + (dy+1)*3 + (dz+1), the input
 * point being (ix+dx, iy+dy, iz+dz)) followed by its bias[co].
 * Host fields: component-major, each component in the reference layout
 * (0:nz, 0:ny-1, 0:nx-1) column-major. */
#define PS3D_CLOSURE_NPARAM 63171
typedef struct ps3d_closure ps3d_closure;
/* max_samples: training samples held on the device (9 fields each). */
int ps3d_closure_create(int nx, int ny, int nz, int max_samples, int device, unsigned long long seed,
                        ps3d_closure **cl);
/* PS3D_ERR_INVALID_ARG while attached to a context (detach first). */
int ps3d_closure_destroy(ps3d_closure *cl);
const char *ps3d_closure_last_error(const ps3d_closure *cl);
int ps3d_closure_get_params(ps3d_closure *cl, float *params);
int ps3d_closure_set_params(ps3d_closure *cl, const float *params);
/* ct: the output scale (0 until fixed by the first ps3d_closure_train or
 * set here). */
int ps3d_closure_get_scale(ps3d_closure *cl, double *ct);
int ps3d_closure_set_scale(ps3d_closure *cl, double ct);
/* One training sample: the coarse run's vor and vel (3 components each)
 * and the target tendency correction (3 components), all physical. */
int ps3d_closure_add_sample(ps3d_closure *cl, const double *vor, const double *vel, const double *target);
int ps3d_closure_num_samples(ps3d_closure *cl, int *n);
/* iters Adam steps (beta 0.9 / 0.999, eps 1e-8), one stored sample each,
 * visiting the samples in a fresh seeded order every pass; the learning rate
 * decays from lr0 to lr1 on a cosine.  Fixes ct on the first call when it
 * is still 0.  loss[iters] (optional) receives each step's normalised mean
 * squared error before the update. */
int ps3d_closure_train(ps3d_closure *cl, int iters, double lr0, double lr1, unsigned long long seed,
                       double *loss);
/* Forward pass on host fields: the physical tendency correction (3
 * components) that an attached closure would add for this state. */
int ps3d_closure_predict(ps3d_closure *cl, const double *vor, const double *vel, double *corr);
/* Test hook: forward, loss and backward on stored sample `sample` without
 * an update.  out (optional): the normalised prediction, 3 x npts FP32;
 * grad (optional): the PS3D_CLOSURE_NPARAM parameter gradients; loss
 * (optional): the normalised mean squared error. */
int ps3d_closure_gradients(ps3d_closure *cl, int sample, float *out, float *grad, double *loss);
/* Inference engine of the forward pass (predict, time_forward and an
 * attached closure; training always uses the warp-level engine):
 * PS3D_CLOSURE_ENGINE_MMA warp-level mma.sync on the plain channels-last
 * activations; PS3D_CLOSURE_ENGINE_TCGEN05 tcgen05.mma with TMEM accumulators
 * on padded activations fed by TMA bulk copies (PS3D_ERR_UNSUPPORTED_SIZE when
 * a tile of the grid's columns does not fit shared memory: nz above 160).
 * The default is TCGEN05 where the grid allows it, else MMA. */
#define PS3D_CLOSURE_ENGINE_MMA 0
#define PS3D_CLOSURE_ENGINE_TCGEN05 1
int ps3d_closure_set_engine(ps3d_closure *cl, int engine);
int ps3d_closure_get_engine(ps3d_closure *cl, int *engine);
/* Synchronise and report a bounded device wait of the tcgen05 engine that ran
 * out since the last check (PS3D_ERR_DEVICE_LIMIT; the word is cleared). */
int ps3d_closure_check(ps3d_closure *cl);
/* Device time (CUDA events on the closure's stream) of one forward pass
 * (the four convolutions) over the input of the last predict, averaged over
 * reps passes after one untimed pass. */
int ps3d_closure_time_forward(ps3d_closure *cl, int reps, double *ms);
/* Attach a closure to a context of the same grid and device (NULL
 * detaches: plain hyperdiffusion).  flags, an OR of:
 *   PS3D_CLOSURE_EVERY_STAGE  evaluate the correction at every right-hand
 *                             side (default: at the first right-hand side of
 *                             each advance, and at every ps3d_gpu_source
 *                             call, then held over the stepper's stages);
 *   PS3D_CLOSURE_CLIP         zero the correction where it would raise the
 *                             local enstrophy (omega . correction > 0);
 *   PS3D_CLOSURE_WALLS        zero its horizontal components on the walls
 *                             (free slip: xi = eta = 0 there).
 * A closure serves one context at a time. */
#define PS3D_CLOSURE_EVERY_STAGE 1
#define PS3D_CLOSURE_CLIP 2
#define PS3D_CLOSURE_WALLS 4
int ps3d_gpu_set_closure(ps3d_gpu_ctx *ctx, ps3d_closure *cl, int flags);

#ifdef __cplusplus
}
#endif
#endif
