/*
 * CPU oracle for the ps3d vorticity right-hand side and time steppers.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C FP64 restatement of the
 * reference Fortran (matt-frey/ps3d, BSD-3-Clause) used as the parity checker
 * for the GPU library and as the timed CPU baseline.  Only tests/, the smoke
 * entry point and the benchmark's CPU-baseline leg may load it; the product
 * path never does.
 *
 * Parity pinning: the restatement is checked against every known-answer unit
 * test the reference ships for this path (unit-tests/test_vor2vel_1..5,
 * test_diffz_1..4, test_diffx, test_diffy, test_omp_collapse,
 * test_implicit_rk), ported to tests/test_oracle_kat.py.  The reference
 * itself cannot be compiled in this environment (no Fortran compiler, MPI or
 * NetCDF), so no run of the reference is available as a further check.
 *
 * Array layout (the reference's, src/fields/fields.f90:17-79): a scalar field
 * is (0:nz, 0:ny-1, 0:nx-1) with z fastest, offset iz + (nz+1)*(iy + ny*ix);
 * a vector field appends a component index (3 consecutive scalar fields).
 */
#ifndef PS3D_ORACLE_H
#define PS3D_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* 1-D transforms (oracle/stafft.c, restating src/fft/stafft.f90) */
int ps3o_factorise(int n, int factors[5]);
int ps3o_initfft(int n, int factors[5], double *trig);
void ps3o_forfft(int m, int n, double *x, double *wk, const double *trig,
                 const int factors[5]);
void ps3o_revfft(int m, int n, double *x, double *wk, const double *trig,
                 const int factors[5]);
void ps3o_dct(int m, int n, double *x, double *wk, double *wk2,
              const double *trig, const int factors[5]);
void ps3o_dst(int m, int n, double *x1, double *wk, double *wk2,
              const double *trig, const int factors[5]);

/* Run configuration: the subset of the &PS3D namelist (src/utils/options.f90)
 * and box (src/utils/parameters.f90) that the hot path consumes. */
enum { PS3O_PRE_CONSTANT = 0, PS3O_PRE_VORCH = 1, PS3O_PRE_BFMAX = 2,
       PS3O_PRE_ROLL_MEAN_MAX_STRAIN = 3, PS3O_PRE_MAX_STRAIN = 4,
       PS3O_PRE_US_MAX_STRAIN = 5, PS3O_PRE_ROLL_MEAN_BFMAX = 6 };
enum { PS3O_KOLMOGOROV = 0, PS3O_GEOPHYSICAL = 1 };
enum { PS3O_HOU_LI = 0, PS3O_TWO_THIRDS = 1 };
enum { PS3O_IMPL_DIFF_RK4 = 0, PS3O_CN2 = 1 };

typedef struct {
    int nx, ny, nz;
    int nnu;
    double lower[3];
    double extent[3];
    double prediss;
    int pretype;
    int length_scale;
    int filtering;
    int stepper;
    double cflmax;
    double alpha;
    double time_limit;
    int roll_mean_win_size;
    int nthreads;            /* OpenMP threads (0: runtime default) */
    int hold_source;         /* test hook: keep svorts fixed inside step()
                                (unit-tests/test_implicit_rk.f90) */
    double f_cor[3];
    /* buoyancy (the reference built with ENABLE_BUOYANCY): N^2 of the basic
     * state (physics.f90:90-94; computed from the initial buoyancy by
     * calculate_basic_reference_state when bfsq_given is 0) and buoy_visc
     * (options.f90:78-80) */
    int buoyancy;
    double bfsq;
    int bfsq_given;
    int buoy_nnu;
    double buoy_prediss;
    int buoy_pretype;
    int buoy_length_scale;
    int buoy_roll_mean_win_size;
} ps3o_config;

/* Per-step diagnostics (adapt, src/stepper/advance.f90:109-377, plus the
 * energy/enstrophy/helicity series). */
typedef struct {
    double t, dt;
    double ke, en, hel;
    double vortmax, vortrms, vorch;
    double vormean[3];
    double ggmax, usggmax, lsggmax;
    double umax, vmax, wmax;
    double bfmax, rmv, pref;
    double rmb, bpref;       /* buoyancy: rolling mean of bfmax, prefactor */
} ps3o_diag;

typedef struct ps3o_model ps3o_model;

int ps3o_create(const ps3o_config *cfg, ps3o_model **out);
void ps3o_destroy(ps3o_model *m);

/* transforms on whole fields (single-rank semantics of src/fft/sta3dfft.f90) */
void ps3o_fftxyp2s(ps3o_model *m, const double *fp, double *fs);
void ps3o_fftxys2p(ps3o_model *m, const double *fs, double *fp);
void ps3o_diffx(ps3o_model *m, const double *fs, double *ds);
void ps3o_diffy(ps3o_model *m, const double *fs, double *ds);
void ps3o_fftsine(ps3o_model *m, double *fs);
void ps3o_fftcosine(ps3o_model *m, double *fs);
void ps3o_central_diffz(ps3o_model *m, const double *fs, double *ds);
void ps3o_decompose_semi_spectral(ps3o_model *m, double *sf);
void ps3o_combine_semi_spectral(ps3o_model *m, double *sf);
void ps3o_decompose_physical(ps3o_model *m, const double *fc, double *sf);
void ps3o_combine_physical(ps3o_model *m, const double *sf, double *fc);

/* tables: which = 0 k2l2, 1 k2l2i (ny*nx); 2 filt, 3 green, 4 phim, 5 phip,
 * 6 thetam, 7 thetap, 8 dthetam, 9 dthetap (N); 10 gamtop, 11 gambot (nz+1);
 * 12 vhdis (ny*nx); 13 rkx (nx), 14 rky (ny), 15 rkz (nz+1); buoyancy:
 * 16 dphim, 17 dphip (N), 18 bhdis (ny*nx), 19 bbarz (nz+1) */
int ps3o_get_table(ps3o_model *m, int which, double *out);

/* state access: which = 0 svor, 1 vor, 2 vel, 3 svel, 4 svorts (3N each);
 * buoyancy: 5 sbuoy, 6 buoy (physical), 7 sbuoys (N each) */
int ps3o_get_field(ps3o_model *m, int which, double *out);
int ps3o_set_field(ps3o_model *m, int which, const double *in);
void ps3o_get_ini_vor_mean(ps3o_model *m, double out[2]);
void ps3o_set_ini_vor_mean(ps3o_model *m, const double in[2]);
double ps3o_get_vvisc(ps3o_model *m);

/* setup_fields (src/utils/utils.f90:136-184) from physical vorticity (3N);
 * pert (3N mixed-spectral, may be NULL) is added after the decomposition */
void ps3o_setup_fields(ps3o_model *m, const double *vor_phys, const double *pert, double *te,
                       double *en);
void ps3o_init_diffusion(ps3o_model *m, double te, double en);
/* setup_fields with buoyancy (utils.f90:136-184): buoy_phys is the total
 * physical buoyancy (N); N^2 from calculate_basic_reference_state unless
 * given, the basic state N^2 z removed, te = kinetic + available potential
 * energy, en = enstrophy + the buoyancy-gradient integral */
void ps3o_setup_fields_buoyancy(ps3o_model *m, const double *vor_phys, const double *pert,
                                const double *buoy_phys, double *te, double *en);
double ps3o_get_bfsq(ps3o_model *m);
double ps3o_get_bvisc(ps3o_model *m);
/* diffz (inversion_utils.f90:683-719): d/dz of a mixed-spectral field,
 * returned mixed-spectral (1: model built without buoyancy) */
int ps3o_diffz(ps3o_model *m, const double *fs, double *ds);
/* buoyancy_tendency (inversion.f90:232-292): sbuoys from sbuoy and vel */
void ps3o_buoyancy_tendency(ps3o_model *m);
/* buoyancy diagnostics of the current fields (field_diagnostics.f90):
 * out[0] available potential energy (:29-60, linear stratification),
 * out[1] buoyancy-gradient integral (:351-397), out[2] minimum static
 * stability (:327-344), out[3] minimum Richardson number (:268-287) */
void ps3o_buoyancy_diagnostics(ps3o_model *m, double out[4]);

void ps3o_vor2vel(ps3o_model *m);
void ps3o_source(ps3o_model *m);
void ps3o_adapt(ps3o_model *m, double t, double *dt, ps3o_diag *d);
void ps3o_step(ps3o_model *m, double *t, double dt);
/* set_diffusion of the configured stepper with prefactor pref */
void ps3o_set_diffusion(ps3o_model *m, double dt, double pref);
/* set_diffusion(dt, vorch, bf) with both prefactors (impl_rk4.f90:37-53,
 * cn2.f90:40-77) */
void ps3o_set_diffusion_vb(ps3o_model *m, double dt, double vpref, double bpref);
/* one advance() (src/stepper/advance.f90:77-104): vor2vel, adapt, source, step */
void ps3o_advance(ps3o_model *m, double *t, ps3o_diag *d);

/* diagnostics of the current physical fields */
void ps3o_energy_series(ps3o_model *m, double *ke, double *en, double *hel);
void ps3o_calc_vorticity_mean(ps3o_model *m, double out[2]);
void ps3o_adjust_vorticity_mean(ps3o_model *m);
/* rolling mean of gamma_max (src/utils/rolling_mean.f90) exposed for tests */
double ps3o_rolling_mean_next(ps3o_model *m, double v);

/* Rutishauser Jacobi eigenvalues of a symmetric 3x3 (src/utils/jacobi.f90);
 * a is column-major 3x3 (only the upper triangle is read), eigs descending. */
int ps3o_jacobi_eigenvalues(double a[9], double eigs[3]);

/* derived fields (fields_derived.f90:67-182, with the buoyancy terms on
 * buoyancy models) from the
 * current vel/vor/svel; outputs physical (nz+1, ny, nx) */
void ps3o_pressure(ps3o_model *m, double *pres);
void ps3o_horizontal_divergence(ps3o_model *m, double *delta);
/* kinetic-energy shell spectrum (genspec.f90:42-123) of the current vel */
int ps3o_ke_spectrum(ps3o_model *m, int nmax, double *spec, double *dk);

#ifdef __cplusplus
}
#endif
#endif
