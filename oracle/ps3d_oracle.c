/*
 * CPU oracle (TEST INFRASTRUCTURE, not the product): FP64 restatement of the
 * reference's single-rank hot path, matt-frey/ps3d (BSD-3-Clause):
 *   src/fft/sta3dfft.f90, src/fft/sta2dfft.f90:44-90, src/fft/deriv1d.f90:10-33
 *   src/mpi/mpi_reverse.f90 (single-rank index reversal + periodic halo)
 *   src/inversion/inversion_utils.f90, src/inversion/inversion.f90
 *   src/stepper/advance.f90, impl_rk4.f90, cn2.f90
 *   src/fields/field_diagnostics.f90, src/utils/jacobi.f90,
 *   src/utils/rolling_mean.f90, src/utils/utils.f90:136-184
 * Operation order follows the reference routine by routine (including the
 * combine/scale/decompose sandwiches of the steppers).  OpenMP parallelises
 * the outer column loops; every per-point result is independent of the
 * thread count except the order of the global sums.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "ps3d_oracle.h"

/* rolling_mean_t (rolling_mean.f90:6-69) */
typedef struct {
    double *hist;
    int inew, iold, filled, len;
    double sma;
} ps3o_roll;

struct ps3o_model {
    ps3o_config cfg;
    int nx, ny, nz, nz1;
    size_t nplane, ncol, nfield; /* ny*nx, ny*nx, (nz+1)*ny*nx */
    double lower[3], extent[3], upper[3], dx[3], dxi[3];
    double ncelli, fnzi, dzi, hdzi;
    long ncell;
    /* transforms */
    int xfac[5], yfac[5], zfac[5];
    double *xtrig, *ytrig, *ztrig;
    double *rkx, *hrkx, *rky, *hrky, *rkz, *rkzi;
    /* inversion tables */
    double *k2l2, *k2l2i, *filt, *green, *phim, *phip, *thetam, *thetap,
        *dthetam, *dthetap, *gamtop, *gambot, *vhdis;
    double vvisc;
    int diffusion_ready;
    /* fields */
    double *svor, *vor, *vel, *svel, *svorts, *vortsm, *vdiss;
    double ini_vor_mean[2];
    /* impl-diff-rk4 stepper state */
    double *svori, *svorf, *epq, *emq;
    /* rolling means of gamma_max (vorticity) and bfmax (buoyancy) */
    ps3o_roll rv, rb;
    /* diagnostics kept between adapt and set_diffusion */
    double vorch, ggmax, usggmax, lsggmax, bfmax, rmv, rmb;
    /* buoyancy (ENABLE_BUOYANCY): tables, fields, stepper state */
    double *dphim, *dphip, *bhdis, *bdiss, *bbarz;
    double *sbuoy, *buoy, *sbuoys, *bsm, *sbuoyi, *sbuoyf, *bpq, *bmq;
    double bfsq, bvisc;
};

#define IDX(m, iz, iy, ix) ((size_t)(iz) + (size_t)(m)->nz1 * ((size_t)(iy) + (size_t)(m)->ny * (size_t)(ix)))
#define PIDX(m, iy, ix) ((size_t)(iy) + (size_t)(m)->ny * (size_t)(ix))

static double *dalloc(size_t n)
{
    double *p = (double *)calloc(n ? n : 1, sizeof(double));
    return p;
}

static double ipow(double x, int p)
{
    /* integer power as gfortran evaluates x**p for integer p */
    double r = 1.0, b = x;
    int e = p < 0 ? -p : p;
    while (e) {
        if (e & 1) r *= b;
        b *= b;
        e >>= 1;
    }
    return p < 0 ? 1.0 / r : r;
}

/* rolling_mean_t%alloc (rolling_mean.f90:21-31); default window 1000
 * (options.f90:66) */
static void roll_init(ps3o_roll *r, int len)
{
    r->len = len > 0 ? len : 1000;
    r->hist = dalloc((size_t)r->len);
    r->inew = 1; r->iold = 1; r->filled = 0; r->sma = 0.0;
}

/* ====================================================================== */
/* set-up: initialise_fft (sta3dfft.f90:53-110), init_inversion            */
/* (inversion_utils.f90:222-372), filters (:377-455), hyperbolic functions  */
/* (:484-542)                                                             */
/* ====================================================================== */
static void set_hyperbolic_functions(ps3o_model *m, int kx, int ky,
                                     const double *zm, const double *zp)
{
    const int nz = m->nz;
    const size_t p = PIDX(m, ky, kx);
    const double kl = sqrt(m->k2l2[p]);
    const double fac = kl * m->extent[2];
    const double ef = exp(-fac);
    const double div = 1.0 / (1.0 - ef * ef);
    const double k2ifac = 0.5 * m->k2l2i[p];
    const double Q = div * (1.0 + ef * ef);
    const double R = div * 2.0 * ef;
    for (int iz = 0; iz <= nz; ++iz) {
        const double Lm = kl * zm[iz], Lp = kl * zp[iz];
        const double ep = exp(-Lp), em = exp(-Lm);
        const double phm = div * (ep - ef * em);
        const double php = div * (em - ef * ep);
        const double dphm = -kl * div * (ep + ef * em);
        const double dphp = kl * div * (em + ef * ep);
        const size_t q = IDX(m, iz, ky, kx);
        m->phim[q] = phm;
        m->phip[q] = php;
        m->thetam[q] = k2ifac * (R * Lm * php - Q * Lp * phm);
        m->thetap[q] = k2ifac * (R * Lp * phm - Q * Lm * php);
        m->dthetam[q] = -k2ifac * ((Q * Lp - 1.0) * dphm - R * Lm * dphp);
        m->dthetap[q] = -k2ifac * ((Q * Lm - 1.0) * dphp - R * Lp * dphm);
        if (m->dphim) {
            m->dphim[q] = dphm;
            m->dphip[q] = dphp;
        }
    }
}

int ps3o_create(const ps3o_config *cfg, ps3o_model **out)
{
    *out = NULL;
    if (cfg->nx < 2 || cfg->ny < 2 || cfg->nz < 2) return 1;
    ps3o_model *m = (ps3o_model *)calloc(1, sizeof(ps3o_model));
    if (!m) return 2;
    m->cfg = *cfg;
#ifdef _OPENMP
    if (cfg->nthreads > 0) omp_set_num_threads(cfg->nthreads);
#endif
    const int nx = cfg->nx, ny = cfg->ny, nz = cfg->nz;
    m->nx = nx; m->ny = ny; m->nz = nz; m->nz1 = nz + 1;
    m->nplane = (size_t)ny * nx;
    m->ncol = m->nplane;
    m->nfield = (size_t)(nz + 1) * m->nplane;
    const double pi = acos(-1.0);
    /* update_parameters (parameters.f90:61-87) */
    const int ncells[3] = {nx, ny, nz};
    for (int d = 0; d < 3; ++d) {
        m->lower[d] = cfg->lower[d];
        m->extent[d] = cfg->extent[d];
        m->upper[d] = cfg->lower[d] + cfg->extent[d];
        m->dx[d] = cfg->extent[d] / (double)ncells[d];
        m->dxi[d] = 1.0 / m->dx[d];
    }
    m->ncell = (long)nx * ny * nz;
    m->ncelli = 1.0 / (double)m->ncell;
    m->fnzi = 1.0 / (double)nz;
    m->dzi = m->dxi[2];
    m->hdzi = 0.5 * m->dxi[2];

    m->xtrig = dalloc(2 * (size_t)nx);
    m->ytrig = dalloc(2 * (size_t)ny);
    m->ztrig = dalloc(2 * (size_t)nz);
    if (ps3o_initfft(nx, m->xfac, m->xtrig) || ps3o_initfft(ny, m->yfac, m->ytrig) ||
        ps3o_initfft(nz, m->zfac, m->ztrig)) {
        ps3o_destroy(m);
        return 3;
    }
    m->rkx = dalloc(nx); m->hrkx = dalloc(nx + 1);
    m->rky = dalloc(ny); m->hrky = dalloc(ny + 1);
    m->rkz = dalloc(nz + 1); m->rkzi = dalloc(nz + 1);
    /* init2dfft: hrkx(k) = pi k / Lx, k = 1..nx (1-based kept) */
    for (int k = 1; k <= nx; ++k) m->hrkx[k] = (pi / m->extent[0]) * (double)k;
    for (int k = 1; k <= ny; ++k) m->hrky[k] = (pi / m->extent[1]) * (double)k;
    const int nwx = nx / 2, nwy = ny / 2;
    m->rkx[0] = 0.0;
    for (int kx = 1; kx < nwx; ++kx) { m->rkx[kx] = m->hrkx[2 * kx]; m->rkx[nx - kx] = m->hrkx[2 * kx]; }
    m->rkx[nwx] = m->hrkx[nx];
    m->rky[0] = 0.0;
    for (int ky = 1; ky < nwy; ++ky) { m->rky[ky] = m->hrky[2 * ky]; m->rky[ny - ky] = m->hrky[2 * ky]; }
    m->rky[nwy] = m->hrky[ny];
    /* init_deriv (deriv1d.f90:10-33) */
    m->rkz[0] = 0.0;
    for (int i = 1; i <= nz; ++i) m->rkz[i] = (pi / m->extent[2]) * (double)i;
    for (int i = 1; i < nz; ++i) m->rkzi[i] = 1.0 / m->rkz[i];

    /* tables */
    const size_t N = m->nfield, P = m->nplane;
    m->k2l2 = dalloc(P); m->k2l2i = dalloc(P); m->vhdis = dalloc(P);
    m->filt = dalloc(N); m->green = dalloc(N);
    m->phim = dalloc(N); m->phip = dalloc(N);
    m->thetam = dalloc(N); m->thetap = dalloc(N);
    m->dthetam = dalloc(N); m->dthetap = dalloc(N);
    m->gamtop = dalloc(nz + 1); m->gambot = dalloc(nz + 1);
    if (cfg->buoyancy) {
        m->dphim = dalloc(N); m->dphip = dalloc(N);
    }
    for (int kx = 0; kx < nx; ++kx)
        for (int ky = 0; ky < ny; ++ky)
            m->k2l2[PIDX(m, ky, kx)] = m->rkx[kx] * m->rkx[kx] + m->rky[ky] * m->rky[ky];
    m->k2l2[0] = 1.0;
    for (size_t p = 0; p < P; ++p) m->k2l2i[p] = 1.0 / m->k2l2[p];
    m->k2l2[0] = 0.0;
    m->k2l2i[0] = 0.0;

    /* de-aliasing filter */
    {
        double *skx = dalloc(nx), *sky = dalloc(ny), *skz = dalloc(nz + 1);
        double rkxmax = 0, rkymax = 0, rkzmax = 0;
        for (int i = 0; i < nx; ++i) rkxmax = fmax(rkxmax, m->rkx[i]);
        for (int i = 0; i < ny; ++i) rkymax = fmax(rkymax, m->rky[i]);
        for (int i = 0; i <= nz; ++i) rkzmax = fmax(rkzmax, m->rkz[i]);
        if (cfg->filtering == PS3O_TWO_THIRDS) {
            const double f23 = 2.0 / 3.0;
            for (int i = 0; i < nx; ++i) skx[i] = (m->rkx[i] <= f23 * rkxmax) ? 1.0 : 0.0;
            for (int i = 0; i < ny; ++i) sky[i] = (m->rky[i] <= f23 * rkymax) ? 1.0 : 0.0;
            for (int i = 0; i <= nz; ++i) skz[i] = (m->rkz[i] <= f23 * rkzmax) ? 1.0 : 0.0;
            for (int kx = 0; kx < nx; ++kx)
                for (int ky = 0; ky < ny; ++ky) {
                    const double f0 = skx[kx] * sky[ky];
                    m->filt[IDX(m, 0, ky, kx)] = f0;
                    m->filt[IDX(m, nz, ky, kx)] = f0;
                    for (int kz = 1; kz < nz; ++kz) m->filt[IDX(m, kz, ky, kx)] = f0 * skz[kz];
                }
        } else {
            const double kxmaxi = 1.0 / rkxmax, kymaxi = 1.0 / rkymax, kzmaxi = 1.0 / rkzmax;
            for (int i = 0; i < nx; ++i) skx[i] = -36.0 * ipow(kxmaxi * m->rkx[i], 36);
            for (int i = 0; i < ny; ++i) sky[i] = -36.0 * ipow(kymaxi * m->rky[i], 36);
            for (int i = 0; i <= nz; ++i) skz[i] = -36.0 * ipow(kzmaxi * m->rkz[i], 36);
            for (int kx = 0; kx < nx; ++kx)
                for (int ky = 0; ky < ny; ++ky) {
                    const double f0 = exp(skx[kx] + sky[ky]);
                    m->filt[IDX(m, 0, ky, kx)] = f0;
                    m->filt[IDX(m, nz, ky, kx)] = f0;
                    for (int kz = 1; kz < nz; ++kz) m->filt[IDX(m, kz, ky, kx)] = f0 * exp(skz[kz]);
                }
        }
        for (int iz = 0; iz <= nz; ++iz) m->filt[IDX(m, iz, 0, 0)] = 1.0;
        free(skx); free(sky); free(skz);
    }

    /* Green function */
    for (int kx = 0; kx < nx; ++kx)
        for (int ky = 0; ky < ny; ++ky) {
            const size_t p = PIDX(m, ky, kx);
            for (int kz = 1; kz <= nz; ++kz)
                m->green[IDX(m, kz, ky, kx)] = -1.0 / (m->k2l2[p] + m->rkz[kz] * m->rkz[kz]);
            m->green[IDX(m, 0, ky, kx)] = -m->k2l2i[p];
        }

    /* hyperbolic functions */
    {
        double *zm = dalloc(nz + 1), *zp = dalloc(nz + 1);
        for (int iz = 0; iz <= nz; ++iz) {
            const double z = m->lower[2] + m->dx[2] * (double)iz;
            zm[iz] = m->upper[2] - z;
            zp[iz] = z - m->lower[2];
        }
#pragma omp parallel for schedule(static)
        for (int kx = 0; kx < nx; ++kx)
            for (int ky = 0; ky < ny; ++ky)
                if (kx != 0 || ky != 0) set_hyperbolic_functions(m, kx, ky, zm, zp);
        for (int iz = 0; iz <= nz; ++iz) {
            const size_t q = IDX(m, iz, 0, 0);
            m->phim[q] = zm[iz] / m->extent[2];
            m->phip[q] = zp[iz] / m->extent[2];
            m->thetam[q] = m->thetap[q] = m->dthetam[q] = m->dthetap[q] = 0.0;
            if (m->dphim) {
                m->dphim[q] = -1.0 / m->extent[2];
                m->dphip[q] = 1.0 / m->extent[2];
            }
        }
        for (int iz = 0; iz <= nz; ++iz) {
            const double php = m->phip[IDX(m, iz, 0, 0)];
            m->gamtop[iz] = 0.5 * m->extent[2] * (php * php - 1.0 / 3.0);
        }
        for (int iz = 0; iz <= nz; ++iz) m->gambot[iz] = m->gamtop[nz - iz];
        free(zm); free(zp);
    }

    /* fields (fields.f90:45-106) and stepper state */
    m->svor = dalloc(3 * N); m->vor = dalloc(3 * N); m->vel = dalloc(3 * N);
    m->svel = dalloc(3 * N); m->svorts = dalloc(3 * N); m->vortsm = dalloc(3 * N);
    m->vdiss = dalloc(P);
    m->svori = dalloc(3 * N); m->svorf = dalloc(3 * N);
    m->epq = dalloc(P); m->emq = dalloc(P);
    roll_init(&m->rv, cfg->roll_mean_win_size);
    roll_init(&m->rb, cfg->buoy_roll_mean_win_size);
    m->bfsq = cfg->bfsq;
    m->bbarz = dalloc(nz + 1);
    if (cfg->buoyancy) {
        m->bhdis = dalloc(P); m->bdiss = dalloc(P);
        m->sbuoy = dalloc(N); m->buoy = dalloc(N); m->sbuoys = dalloc(N); m->bsm = dalloc(N);
        m->sbuoyi = dalloc(N); m->sbuoyf = dalloc(N);
        m->bpq = dalloc(P); m->bmq = dalloc(P);
        if (!m->dphim || !m->dphip || !m->sbuoy || !m->buoy || !m->sbuoys || !m->bsm || !m->sbuoyi ||
            !m->sbuoyf) {
            ps3o_destroy(m);
            return 2;
        }
        for (int iz = 0; iz <= nz; ++iz) m->bbarz[iz] = m->bfsq * (m->lower[2] + m->dx[2] * (double)iz);
    }
    if (!m->svor || !m->vor || !m->vel || !m->svel || !m->svorts || !m->vortsm ||
        !m->svori || !m->svorf || !m->phim || !m->dthetap) {
        ps3o_destroy(m);
        return 2;
    }
    *out = m;
    return 0;
}

void ps3o_destroy(ps3o_model *m)
{
    if (!m) return;
    double *ps[] = {m->xtrig, m->ytrig, m->ztrig, m->rkx, m->hrkx, m->rky, m->hrky,
                    m->rkz, m->rkzi, m->k2l2, m->k2l2i, m->filt, m->green, m->phim,
                    m->phip, m->thetam, m->thetap, m->dthetam, m->dthetap, m->gamtop,
                    m->gambot, m->vhdis, m->svor, m->vor, m->vel, m->svel, m->svorts,
                    m->vortsm, m->vdiss, m->svori, m->svorf, m->epq, m->emq, m->rv.hist,
                    m->rb.hist, m->dphim, m->dphip, m->bhdis, m->bdiss, m->bbarz, m->sbuoy,
                    m->buoy, m->sbuoys, m->bsm, m->sbuoyi, m->sbuoyf, m->bpq, m->bmq};
    for (size_t i = 0; i < sizeof(ps) / sizeof(ps[0]); ++i) free(ps[i]);
    free(m);
}

/* ====================================================================== */
/* horizontal transforms: fftxyp2s / fftxys2p (sta3dfft.f90:136-260).      */
/* On one rank the pencil transposes (fft_pencil.f90:283-401) reduce to    */
/* gathering each y (then x) line into a contiguous buffer.               */
/* ====================================================================== */
static void lines_y(ps3o_model *m, const double *in, double *out, int inverse)
{
    const int nx = m->nx, ny = m->ny, nz1 = m->nz1;
#pragma omp parallel
    {
        double *line = dalloc(ny), *wk = dalloc(ny);
#pragma omp for schedule(static)
        for (int ix = 0; ix < nx; ++ix)
            for (int iz = 0; iz < nz1; ++iz) {
                for (int iy = 0; iy < ny; ++iy) line[iy] = in[IDX(m, iz, iy, ix)];
                if (inverse) ps3o_revfft(1, ny, line, wk, m->ytrig, m->yfac);
                else ps3o_forfft(1, ny, line, wk, m->ytrig, m->yfac);
                for (int iy = 0; iy < ny; ++iy) out[IDX(m, iz, iy, ix)] = line[iy];
            }
        free(line); free(wk);
    }
}

static void lines_x(ps3o_model *m, const double *in, double *out, int inverse)
{
    const int nx = m->nx, ny = m->ny, nz1 = m->nz1;
#pragma omp parallel
    {
        double *line = dalloc(nx), *wk = dalloc(nx);
#pragma omp for schedule(static)
        for (int iy = 0; iy < ny; ++iy)
            for (int iz = 0; iz < nz1; ++iz) {
                for (int ix = 0; ix < nx; ++ix) line[ix] = in[IDX(m, iz, iy, ix)];
                if (inverse) ps3o_revfft(1, nx, line, wk, m->xtrig, m->xfac);
                else ps3o_forfft(1, nx, line, wk, m->xtrig, m->xfac);
                for (int ix = 0; ix < nx; ++ix) out[IDX(m, iz, iy, ix)] = line[ix];
            }
        free(line); free(wk);
    }
}

void ps3o_fftxyp2s(ps3o_model *m, const double *fp, double *fs)
{
    lines_y(m, fp, fs, 0);
    lines_x(m, fs, fs, 0);
}

void ps3o_fftxys2p(ps3o_model *m, const double *fs, double *fp)
{
    lines_x(m, fs, fp, 1);
    lines_y(m, fp, fp, 1);
}

/* diffx/diffy (sta3dfft.f90:304-377) with reverse_x/y (mpi_reverse.f90:
 * 332-398) on one rank: g(k) = f(n-1-k), so ds(k) = s * hrk(min(2k,2(n-k))) *
 * f(n-k), s = +1 for k >= n/2+1 else -1, ds(0) = 0, Nyquist zeroed. */
void ps3o_diffx(ps3o_model *m, const double *fs, double *ds)
{
    const int nx = m->nx, ny = m->ny, nz1 = m->nz1, nwx = nx / 2;
#pragma omp parallel for schedule(static)
    for (int kx = 0; kx < nx; ++kx) {
        double c = 0.0;
        if (kx >= 1) {
            const int dkx = (2 * kx < 2 * (nx - kx)) ? 2 * kx : 2 * (nx - kx);
            const double si = (kx >= nwx + 1) ? 1.0 : -1.0;
            c = si * m->hrkx[dkx];
        }
        if (nx % 2 == 0 && kx == nwx) c = 0.0;
        const int src = (kx == 0) ? 0 : nx - kx;
        for (int ky = 0; ky < ny; ++ky)
            for (int iz = 0; iz < nz1; ++iz)
                ds[IDX(m, iz, ky, kx)] = (kx == 0) ? 0.0 : c * fs[IDX(m, iz, ky, src)];
    }
}

void ps3o_diffy(ps3o_model *m, const double *fs, double *ds)
{
    const int nx = m->nx, ny = m->ny, nz1 = m->nz1, nwy = ny / 2;
#pragma omp parallel for schedule(static)
    for (int kx = 0; kx < nx; ++kx)
        for (int ky = 0; ky < ny; ++ky) {
            double c = 0.0;
            if (ky >= 1) {
                const int dky = (2 * ky < 2 * (ny - ky)) ? 2 * ky : 2 * (ny - ky);
                const double si = (ky >= nwy + 1) ? 1.0 : -1.0;
                c = si * m->hrky[dky];
            }
            if (ny % 2 == 0 && ky == nwy) c = 0.0;
            const int src = (ky == 0) ? 0 : ny - ky;
            for (int iz = 0; iz < nz1; ++iz)
                ds[IDX(m, iz, ky, kx)] = (ky == 0) ? 0.0 : c * fs[IDX(m, iz, src, kx)];
        }
}

/* fftsine / fftcosine (sta3dfft.f90:264-300): column DST on 1..nz / DCT on
 * 0..nz for every (ky, kx). */
void ps3o_fftsine(ps3o_model *m, double *fs)
{
    const int nz = m->nz;
    const long nc = (long)m->ncol;
#pragma omp parallel
    {
        double *wk = dalloc(nz), *wk2 = dalloc(nz);
#pragma omp for schedule(static)
        for (long c = 0; c < nc; ++c) ps3o_dst(1, nz, fs + (size_t)c * m->nz1 + 1, wk, wk2, m->ztrig, m->zfac);
        free(wk); free(wk2);
    }
}

void ps3o_fftcosine(ps3o_model *m, double *fs)
{
    const int nz = m->nz;
    const long nc = (long)m->ncol;
#pragma omp parallel
    {
        double *wk = dalloc(nz), *wk2 = dalloc(nz);
#pragma omp for schedule(static)
        for (long c = 0; c < nc; ++c) ps3o_dct(1, nz, fs + (size_t)c * m->nz1, wk, wk2, m->ztrig, m->zfac);
        free(wk); free(wk2);
    }
}

/* central_diffz (inversion_utils.f90:653-673) */
void ps3o_central_diffz(ps3o_model *m, const double *fs, double *ds)
{
    const int nz = m->nz;
    const long nc = (long)m->ncol;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < nc; ++c) {
        const double *f = fs + (size_t)c * m->nz1;
        double *d = ds + (size_t)c * m->nz1;
        d[0] = m->dzi * (f[1] - f[0]);
        d[nz] = m->dzi * (f[nz] - f[nz - 1]);
        for (int iz = 1; iz < nz; ++iz) d[iz] = (f[iz + 1] - f[iz - 1]) * m->hdzi;
    }
}

/* field_decompose_semi_spectral (inversion_utils.f90:563-595) */
void ps3o_decompose_semi_spectral(ps3o_model *m, double *sf)
{
    const int nz = m->nz;
    const long nc = (long)m->ncol;
#pragma omp parallel
    {
        double *wk = dalloc(nz), *wk2 = dalloc(nz);
#pragma omp for schedule(static)
        for (long c = 0; c < nc; ++c) {
            double *f = sf + (size_t)c * m->nz1;
            const double *pm = m->phim + (size_t)c * m->nz1, *pp = m->phip + (size_t)c * m->nz1;
            for (int iz = 1; iz < nz; ++iz) f[iz] = f[iz] - (f[0] * pm[iz] + f[nz] * pp[iz]);
            const double top = f[nz];
            ps3o_dst(1, nz, f + 1, wk, wk2, m->ztrig, m->zfac);
            f[nz] = top;
        }
        free(wk); free(wk2);
    }
}

/* field_combine_semi_spectral (inversion_utils.f90:617-647) */
void ps3o_combine_semi_spectral(ps3o_model *m, double *sf)
{
    const int nz = m->nz;
    const long nc = (long)m->ncol;
#pragma omp parallel
    {
        double *wk = dalloc(nz), *wk2 = dalloc(nz);
#pragma omp for schedule(static)
        for (long c = 0; c < nc; ++c) {
            double *f = sf + (size_t)c * m->nz1;
            const double *pm = m->phim + (size_t)c * m->nz1, *pp = m->phip + (size_t)c * m->nz1;
            const double top = f[nz];
            f[nz] = 0.0;
            ps3o_dst(1, nz, f + 1, wk, wk2, m->ztrig, m->zfac);
            f[nz] = top;
            for (int iz = 1; iz < nz; ++iz) f[iz] = f[iz] + f[0] * pm[iz] + f[nz] * pp[iz];
        }
        free(wk); free(wk2);
    }
}

/* field_decompose_physical (:549-557) and field_combine_physical (:599-611) */
void ps3o_decompose_physical(ps3o_model *m, const double *fc, double *sf)
{
    ps3o_fftxyp2s(m, fc, sf);
    ps3o_decompose_semi_spectral(m, sf);
}

void ps3o_combine_physical(ps3o_model *m, const double *sf, double *fc)
{
    double *sfc = dalloc(m->nfield);
    memcpy(sfc, sf, sizeof(double) * m->nfield);
    ps3o_combine_semi_spectral(m, sfc);
    ps3o_fftxys2p(m, sfc, fc);
    free(sfc);
}

/* ====================================================================== */
/* vor2vel (inversion.f90:23-226)                                          */
/* ====================================================================== */
static void axpby_k2l2i(ps3o_model *m, double *out, const double *a, const double *b, double sb)
{
    /* out(iz,:,:) = k2l2i * (a + sb*b) */
    const long nc = (long)m->ncol;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < nc; ++c) {
        const double k = m->k2l2i[c];
        for (int iz = 0; iz < m->nz1; ++iz) {
            const size_t q = (size_t)c * m->nz1 + iz;
            out[q] = k * (a[q] + sb * b[q]);
        }
    }
}

void ps3o_vor2vel(ps3o_model *m)
{
    const size_t N = m->nfield;
    const int nz = m->nz;
    double *as = dalloc(N), *bs = dalloc(N), *ds = dalloc(N), *es = dalloc(N), *cs = dalloc(N);
    double *ubar = dalloc(nz + 1), *vbar = dalloc(nz + 1);
    double *A = m->svor, *B = m->svor + N, *C = m->svor + 2 * N;

    /* enforce solenoidality */
    ps3o_diffx(m, B, as);
    ps3o_diffy(m, A, bs);
    for (size_t i = 0; i < N; ++i) { ds[i] = as[i] - bs[i]; cs[i] = C[i]; }
    ps3o_combine_semi_spectral(m, cs);
    ps3o_central_diffz(m, cs, es);
    ps3o_decompose_semi_spectral(m, es);
    for (int iz = 0; iz <= nz; ++iz) { ubar[iz] = A[iz]; vbar[iz] = B[iz]; }
    ps3o_diffx(m, es, A);
    ps3o_diffy(m, ds, cs);
    axpby_k2l2i(m, A, A, cs, 1.0);
    ps3o_diffy(m, es, B);
    ps3o_diffx(m, ds, cs);
    axpby_k2l2i(m, B, B, cs, -1.0);
    for (int iz = 0; iz <= nz; ++iz) { A[iz] = ubar[iz]; B[iz] = vbar[iz]; }

    /* vorticity in physical space */
    for (int nc = 0; nc < 3; ++nc) ps3o_combine_physical(m, m->svor + nc * N, m->vor + nc * N);

    /* source term for vertical velocity */
    ps3o_diffy(m, A, ds);
    ps3o_diffx(m, B, es);
    for (size_t i = 0; i < N; ++i) ds[i] = ds[i] - es[i];
    {
        const long ncol = (long)m->ncol;
#pragma omp parallel for schedule(static)
        for (long c = 0; c < ncol; ++c) {
            const size_t o = (size_t)c * m->nz1;
            const double d0 = ds[o], dn = ds[o + nz];
            for (int iz = 1; iz < nz; ++iz) bs[o + iz] = d0 * m->thetam[o + iz] + dn * m->thetap[o + iz];
            for (int iz = 0; iz <= nz; ++iz) es[o + iz] = d0 * m->dthetam[o + iz] + dn * m->dthetap[o + iz];
            for (int iz = 1; iz < nz; ++iz) ds[o + iz] = m->green[o + iz] * ds[o + iz];
            as[o] = 0.0;
            for (int kz = 1; kz < nz; ++kz) as[o + kz] = m->rkz[kz] * ds[o + kz];
            as[o + nz] = 0.0;
        }
    }
    ps3o_fftcosine(m, as);
    ps3o_fftsine(m, ds);
    {
        const long ncol = (long)m->ncol;
#pragma omp parallel for schedule(static)
        for (long c = 0; c < ncol; ++c) {
            const size_t o = (size_t)c * m->nz1;
            ds[o] = 0.0;
            for (int iz = 1; iz < nz; ++iz) ds[o + iz] = ds[o + iz] + bs[o + iz];
            ds[o + nz] = 0.0;
            for (int iz = 0; iz <= nz; ++iz) es[o + iz] = es[o + iz] + as[o + iz];
        }
    }
    memcpy(cs, C, sizeof(double) * N);
    ps3o_combine_semi_spectral(m, cs);

    /* horizontally averaged flow */
    {
        ubar[0] = 0.0; vbar[0] = 0.0;
        for (int iz = 1; iz < nz; ++iz) { ubar[iz] = -m->rkzi[iz] * B[iz]; vbar[iz] = m->rkzi[iz] * A[iz]; }
        ubar[nz] = 0.0; vbar[nz] = 0.0;
        double *wk = dalloc(nz), *wk2 = dalloc(nz);
        ps3o_dct(1, nz, ubar, wk, wk2, m->ztrig, m->zfac);
        ps3o_dct(1, nz, vbar, wk, wk2, m->ztrig, m->zfac);
        free(wk); free(wk2);
        for (int iz = 0; iz <= nz; ++iz) {
            ubar[iz] = ubar[iz] + B[nz] * m->gamtop[iz] - B[0] * m->gambot[iz];
            vbar[iz] = vbar[iz] - A[nz] * m->gamtop[iz] + A[0] * m->gambot[iz];
        }
    }

    /* u */
    ps3o_diffx(m, es, as);
    ps3o_diffy(m, cs, bs);
    axpby_k2l2i(m, as, as, bs, 1.0);
    for (int iz = 0; iz <= nz; ++iz) as[iz] = ubar[iz];
    memcpy(m->svel, as, sizeof(double) * N);
    ps3o_fftxys2p(m, as, m->vel);
    /* v */
    ps3o_diffy(m, es, as);
    ps3o_diffx(m, cs, bs);
    axpby_k2l2i(m, as, as, bs, -1.0);
    for (int iz = 0; iz <= nz; ++iz) as[iz] = vbar[iz];
    memcpy(m->svel + N, as, sizeof(double) * N);
    ps3o_fftxys2p(m, as, m->vel + N);
    /* w */
    memcpy(m->svel + 2 * N, ds, sizeof(double) * N);
    ps3o_fftxys2p(m, ds, m->vel + 2 * N);

    free(as); free(bs); free(ds); free(es); free(cs); free(ubar); free(vbar);
}

/* ====================================================================== */
/* vorticity_tendency / source (inversion.f90:298-388)                     */
/* ====================================================================== */
/* diffz (inversion_utils.f90:683-719): the linear part from the boundary
 * rows and dphim/dphip, the sine series differentiated into a cosine series
 * and transformed to semi-spectral space, then decomposed */
int ps3o_diffz(ps3o_model *m, const double *fs, double *ds)
{
    if (!m->dphim) return 1;
    const int nz = m->nz;
    const long nc = (long)m->ncol;
    double *as = dalloc(m->nfield);
#pragma omp parallel for schedule(static)
    for (long c = 0; c < nc; ++c) {
        const size_t o = (size_t)c * m->nz1;
        const double f0 = fs[o], fn = fs[o + nz];
        for (int iz = 0; iz <= nz; ++iz) ds[o + iz] = f0 * m->dphim[o + iz] + fn * m->dphip[o + iz];
        as[o] = 0.0;
        for (int kz = 1; kz < nz; ++kz) as[o + kz] = m->rkz[kz] * fs[o + kz];
        as[o + nz] = 0.0;
    }
    ps3o_fftcosine(m, as);
    for (size_t i = 0; i < m->nfield; ++i) ds[i] = ds[i] + as[i];
    ps3o_decompose_semi_spectral(m, ds);
    free(as);
    return 0;
}

/* buoyancy_tendency (inversion.f90:232-292): b_t = -div(u b) - N^2 w in flux
 * form, each flux decomposed, differentiated and combined back */
void ps3o_buoyancy_tendency(ps3o_model *m)
{
    const size_t N = m->nfield;
    double *fp = dalloc(N), *fs = dalloc(N), *ds = dalloc(N), *btend = dalloc(N);
    const double *u = m->vel, *v = m->vel + N, *w = m->vel + 2 * N;
    ps3o_combine_physical(m, m->sbuoy, m->buoy);
    for (size_t i = 0; i < N; ++i) fp[i] = u[i] * m->buoy[i];
    ps3o_decompose_physical(m, fp, fs);
    ps3o_diffx(m, fs, ds);
    ps3o_combine_physical(m, ds, btend);
    for (size_t i = 0; i < N; ++i) fp[i] = v[i] * m->buoy[i];
    ps3o_decompose_physical(m, fp, fs);
    ps3o_diffy(m, fs, ds);
    ps3o_combine_physical(m, ds, fp);
    for (size_t i = 0; i < N; ++i) btend[i] = -btend[i] - fp[i];
    for (size_t i = 0; i < N; ++i) fp[i] = w[i] * m->buoy[i];
    ps3o_decompose_physical(m, fp, fs);
    ps3o_diffz(m, fs, ds);
    ps3o_combine_physical(m, ds, fp);
    for (size_t i = 0; i < N; ++i) btend[i] = btend[i] - m->bfsq * w[i] - fp[i];
    ps3o_decompose_physical(m, btend, m->sbuoys);
    free(fp); free(fs); free(ds); free(btend);
}

/* source (inversion.f90:376-388): buoyancy_tendency, then
 * vorticity_tendency (:298-371) */
void ps3o_source(ps3o_model *m)
{
    const size_t N = m->nfield;
    if (m->cfg.buoyancy) ps3o_buoyancy_tendency(m);
    double *fp = dalloc(N), *gp = dalloc(N), *p = dalloc(N), *q = dalloc(N), *r = dalloc(N);
    double *u = m->vel, *v = m->vel + N, *w = m->vel + 2 * N;
    double *xi = m->vor, *eta = m->vor + N, *zeta = m->vor + 2 * N;
    double *s1 = m->svorts, *s2 = m->svorts + N, *s3 = m->svorts + 2 * N;

    for (int nc = 0; nc < 3; ++nc) {
        const double f = m->cfg.f_cor[nc];
        double *vv = m->vor + nc * N;
        for (size_t i = 0; i < N; ++i) vv[i] = vv[i] + f;
    }
    /* r = u*eta - v*xi (+ b) */
    if (m->cfg.buoyancy) ps3o_combine_physical(m, m->sbuoy, m->buoy);
    for (size_t i = 0; i < N; ++i) fp[i] = u[i] * eta[i] - v[i] * xi[i];
    if (m->cfg.buoyancy)
        for (size_t i = 0; i < N; ++i) fp[i] = fp[i] + m->buoy[i];
    ps3o_decompose_physical(m, fp, r);
    /* q = w*xi - u*zeta */
    for (size_t i = 0; i < N; ++i) fp[i] = w[i] * xi[i] - u[i] * zeta[i];
    ps3o_decompose_physical(m, fp, q);
    /* dxi/dt = dr/dy - dq/dz */
    ps3o_diffy(m, r, s1);
    ps3o_central_diffz(m, fp, gp);
    ps3o_decompose_physical(m, gp, p);
    for (size_t i = 0; i < N; ++i) s1[i] = s1[i] - p[i];
    /* p = v*zeta - w*eta */
    for (size_t i = 0; i < N; ++i) fp[i] = v[i] * zeta[i] - w[i] * eta[i];
    ps3o_decompose_physical(m, fp, p);
    /* deta/dt = dp/dz - dr/dx */
    ps3o_diffx(m, r, s2);
    ps3o_central_diffz(m, fp, gp);
    ps3o_decompose_physical(m, gp, r);
    for (size_t i = 0; i < N; ++i) s2[i] = r[i] - s2[i];
    /* dzeta/dt = dq/dx - dp/dy */
    ps3o_diffx(m, q, s3);
    ps3o_diffy(m, p, r);
    for (size_t i = 0; i < N; ++i) s3[i] = s3[i] - r[i];
    free(fp); free(gp); free(p); free(q); free(r);
}

/* ====================================================================== */
/* diagnostics (field_diagnostics.f90)                                     */
/* ====================================================================== */
/* sum over the grid with the z-trapezoid weights: interior 1, walls 1/2 */
static double wsum_fn(ps3o_model *m, double (*f)(ps3o_model *, size_t, void *), void *ctx)
{
    const int nz = m->nz;
    const long nc = (long)m->ncol;
    double s_in = 0.0, s_w = 0.0;
#pragma omp parallel for reduction(+ : s_in, s_w) schedule(static)
    for (long c = 0; c < nc; ++c) {
        const size_t o = (size_t)c * m->nz1;
        for (int iz = 1; iz < nz; ++iz) s_in += f(m, o + iz, ctx);
        s_w += f(m, o, ctx) + f(m, o + nz, ctx);
    }
    return s_in + 0.5 * s_w;
}

static double f_vel2(ps3o_model *m, size_t q, void *c)
{
    (void)c;
    const size_t N = m->nfield;
    return m->vel[q] * m->vel[q] + m->vel[N + q] * m->vel[N + q] + m->vel[2 * N + q] * m->vel[2 * N + q];
}
static double f_vor2(ps3o_model *m, size_t q, void *c)
{
    (void)c;
    const size_t N = m->nfield;
    return m->vor[q] * m->vor[q] + m->vor[N + q] * m->vor[N + q] + m->vor[2 * N + q] * m->vor[2 * N + q];
}
static double f_hel(ps3o_model *m, size_t q, void *c)
{
    (void)c;
    const size_t N = m->nfield;
    return m->vel[q] * m->vor[q] + m->vel[N + q] * m->vor[N + q] + m->vel[2 * N + q] * m->vor[2 * N + q];
}
static double f_comp(ps3o_model *m, size_t q, void *c)
{
    (void)m;
    return ((const double *)c)[q];
}

/* get_kinetic_energy (:85-122), get_enstrophy (:172-206); helicity <u.w> uses
 * the same z-trapezoid weights (it has no counterpart in the reference). */
void ps3o_energy_series(ps3o_model *m, double *ke, double *en, double *hel)
{
    *ke = 0.5 * wsum_fn(m, f_vel2, NULL) * m->ncelli;
    *en = 0.5 * wsum_fn(m, f_vor2, NULL) * m->ncelli;
    *hel = wsum_fn(m, f_hel, NULL) * m->ncelli;
}

/* calc_vorticity_mean (:584-600) */
void ps3o_calc_vorticity_mean(ps3o_model *m, double out[2])
{
    const int nz = m->nz;
    double *wk = dalloc(nz + 1), *w1 = dalloc(nz), *w2 = dalloc(nz);
    for (int nc = 0; nc < 2; ++nc) {
        const double *s = m->svor + nc * m->nfield;
        for (int iz = 1; iz < nz; ++iz) wk[iz] = s[iz];
        wk[nz] = 0.0;
        ps3o_dst(1, nz, wk + 1, w1, w2, m->ztrig, m->zfac);
        double sum = 0.0;
        for (int iz = 1; iz < nz; ++iz) sum += wk[iz];
        out[nc] = 0.5 * (s[0] + s[nz]) + m->fnzi * sum;
    }
    free(wk); free(w1); free(w2);
}

/* adjust_vorticity_mean (:604-619) */
void ps3o_adjust_vorticity_mean(ps3o_model *m)
{
    double savg[2];
    ps3o_calc_vorticity_mean(m, savg);
    for (int nc = 0; nc < 2; ++nc) {
        double *s = m->svor + nc * m->nfield;
        s[0] = s[0] + m->ini_vor_mean[nc] - savg[nc];
        s[m->nz] = s[m->nz] + m->ini_vor_mean[nc] - savg[nc];
    }
}

/* ====================================================================== */
/* Jacobi eigenvalues (jacobi.f90): A column-major, upper triangle used    */
/* ====================================================================== */
#define AM(i, j) a[((i) - 1) + 3 * ((j) - 1)]
static void givens(const double *a, const double *D, int i, int j, double *c, double *s,
                   double *t, double *tau)
{
    const double aij = AM(i, j);
    const double g = 100.0 * fabs(aij);
    const double h = D[j - 1] - D[i - 1];
    if (fabs(h) + g == fabs(h)) {
        *t = aij / (h + copysign(DBL_EPSILON, h));
    } else {
        const double theta = 0.5 * h / (aij + copysign(DBL_EPSILON, aij));
        double tt = 1.0 / (fabs(theta) + sqrt(1.0 + theta * theta));
        if (theta < 0.0) tt = -tt;
        *t = tt;
    }
    *c = 1.0 / sqrt(1.0 + (*t) * (*t));
    *s = (*t) * (*c);
    *tau = (*s) / (1.0 + *c);
}

static void apply_rotation(double *a, double *D, double *Z, int i, int j)
{
    double c, s, t, tau, g, h;
    givens(a, D, i, j, &c, &s, &t, &tau);
    h = t * AM(i, j);
    Z[i - 1] -= h; Z[j - 1] += h;
    D[i - 1] -= h; D[j - 1] += h;
    AM(i, j) = 0.0;
    for (int k = 1; k <= i - 1; ++k) {
        g = AM(k, i); h = AM(k, j);
        AM(k, i) = g - s * (h + g * tau);
        AM(k, j) = h + s * (g - h * tau);
    }
    for (int k = i + 1; k <= j - 1; ++k) {
        g = AM(i, k); h = AM(k, j);
        AM(i, k) = g - s * (h + g * tau);
        AM(k, j) = h + s * (g - h * tau);
    }
    for (int k = j + 1; k <= 3; ++k) {
        g = AM(i, k); h = AM(j, k);
        AM(i, k) = g - s * (h + g * tau);
        AM(j, k) = h + s * (g - h * tau);
    }
}

int ps3o_jacobi_eigenvalues(double a[9], double D[3])
{
    double B[3], Z[3];
    for (int j = 1; j <= 3; ++j) { D[j - 1] = AM(j, j); B[j - 1] = D[j - 1]; Z[j - 1] = 0.0; }
    double sm = fabs(AM(1, 2)) + fabs(AM(1, 3)) + fabs(AM(2, 3));
    int sweeps = 0;
    while (sm > 1.0e-15) {
        for (int i = 1; i <= 2; ++i)
            for (int j = i + 1; j <= 3; ++j) apply_rotation(a, D, Z, i, j);
        for (int k = 0; k < 3; ++k) { B[k] += Z[k]; D[k] = B[k]; Z[k] = 0.0; }
        sm = fabs(AM(1, 2)) + fabs(AM(1, 3)) + fabs(AM(2, 3));
        ++sweeps;
    }
    double te;
    if (D[1] > D[0]) { te = D[0]; D[0] = D[1]; D[1] = te; }
    if (D[2] > D[1]) { te = D[1]; D[1] = D[2]; D[2] = te; }
    if (D[1] > D[0]) { te = D[0]; D[0] = D[1]; D[1] = te; }
    return sweeps;
}
#undef AM

/* rolling_mean_t%get_next (rolling_mean.f90:36-69), 1-based indices kept */
static double roll_next(ps3o_roll *r, double vnew)
{
    const int L = r->len;
    if (r->filled) {
        const double vold = r->hist[r->iold - 1];
        r->iold = r->iold % L + 1;
        r->sma = r->sma + (vnew - vold) / (double)L;
        r->hist[r->inew - 1] = vnew;
        r->inew = r->inew % L + 1;
    } else {
        r->hist[r->inew - 1] = vnew;
        double s = 0.0;
        for (int i = 0; i < r->inew; ++i) s += r->hist[i];
        r->sma = s / (double)r->inew;
        r->filled = (L == r->inew);
        r->inew = r->inew % L + 1;
    }
    return r->sma;
}

double ps3o_rolling_mean_next(ps3o_model *m, double vnew) { return roll_next(&m->rv, vnew); }

/* ====================================================================== */
/* init_diffusion (inversion_utils.f90:124-218)                           */
/* ====================================================================== */
/* get_viscosity (:157-185) */
static double get_viscosity(ps3o_model *m, int length_scale, double prediss, int p, double te, double en)
{
    double rkxmax = 0.0, rkymax = 0.0;
    for (int i = 0; i < m->nx; ++i) rkxmax = fmax(rkxmax, m->rkx[i]);
    for (int i = 0; i < m->ny; ++i) rkymax = fmax(rkymax, m->rky[i]);
    const double k2max = ipow(fmax(rkxmax, rkymax), 2);
    const double rkmsi = 1.0 / k2max;
    if (length_scale == PS3O_GEOPHYSICAL) return prediss * ipow(rkmsi, p);
    return prediss * pow(k2max * te / en, 1.0 / 3.0) * ipow(rkmsi, p);
}

/* init_dissipation (:189-218) */
static void init_dissipation(ps3o_model *m, double vis, int p, double *hdis)
{
    for (size_t i = 0; i < m->nplane; ++i) hdis[i] = (p == 1) ? vis * m->k2l2[i] : vis * ipow(m->k2l2[i], p);
}

void ps3o_init_diffusion(ps3o_model *m, double te, double en)
{
    m->vvisc = get_viscosity(m, m->cfg.length_scale, m->cfg.prediss, m->cfg.nnu, te, en);
    init_dissipation(m, m->vvisc, m->cfg.nnu, m->vhdis);
    if (m->cfg.buoyancy) {
        m->bvisc = get_viscosity(m, m->cfg.buoy_length_scale, m->cfg.buoy_prediss, m->cfg.buoy_nnu, te, en);
        init_dissipation(m, m->bvisc, m->cfg.buoy_nnu, m->bhdis);
    }
    m->diffusion_ready = 1;
}

/* setup_fields (utils.f90:136-184), without the NetCDF read */
void ps3o_setup_fields(ps3o_model *m, const double *vor_phys, const double *pert, double *te_out,
                       double *en_out)
{
    const size_t N = m->nfield;
    memset(m->svor, 0, sizeof(double) * 3 * N);
    memset(m->vel, 0, sizeof(double) * 3 * N);
    memset(m->svel, 0, sizeof(double) * 3 * N);
    memset(m->svorts, 0, sizeof(double) * 3 * N);
    memset(m->vortsm, 0, sizeof(double) * 3 * N);
    memcpy(m->vor, vor_phys, sizeof(double) * 3 * N);
    for (int nc = 0; nc < 3; ++nc) ps3o_decompose_physical(m, m->vor + nc * N, m->svor + nc * N);
    if (pert)
        for (size_t i = 0; i < 3 * N; ++i) m->svor[i] += pert[i];
    ps3o_calc_vorticity_mean(m, m->ini_vor_mean);
    ps3o_vor2vel(m);
    double ke, en, hel;
    ps3o_energy_series(m, &ke, &en, &hel);
    ps3o_init_diffusion(m, ke, en);
    if (te_out) *te_out = ke;
    if (en_out) *en_out = en;
}

/* ---- buoyancy diagnostics (field_diagnostics.f90) -------------------- */
/* z-trapezoid sum of one field: interior levels 1, walls 1/2 */
static double wsum_field(ps3o_model *m, const double *f)
{
    return wsum_fn(m, f_comp, (void *)f);
}

/* get_available_potential_energy (:29-60) with the linear-stratification
 * density ape_den(b, z) = b^2 / (2 N^2) (ape_density.f90:10-34) */
static double available_potential_energy(ps3o_model *m, const double *b)
{
    double *a = dalloc(m->nfield);
    for (size_t i = 0; i < m->nfield; ++i) a[i] = b[i] * b[i] / (2.0 * m->bfsq);
    const double ape = wsum_field(m, a) * m->ncelli;
    free(a);
    return ape;
}

/* get_gradb_integral (:351-397).  The reference's z term is overwritten
 * before use (central_diffz writes mag, then fftxys2p(ds, mag) replaces it
 * with the y derivative, :369-370), so |grad b| there is
 * sqrt(b_x^2 + 2 b_y^2); restated as is.  sbuoy makes the combine /
 * decompose round trip in place. */
static double gradb_integral(ps3o_model *m)
{
    const size_t N = m->nfield;
    double *ds = dalloc(N), *mag = dalloc(N), *bx = dalloc(N), *by = dalloc(N);
    ps3o_combine_semi_spectral(m, m->sbuoy);
    ps3o_diffx(m, m->sbuoy, ds);
    ps3o_fftxys2p(m, ds, bx);
    ps3o_diffy(m, m->sbuoy, ds);
    ps3o_fftxys2p(m, ds, by);
    ps3o_central_diffz(m, m->sbuoy, mag);
    ps3o_fftxys2p(m, ds, mag);
    ps3o_decompose_semi_spectral(m, m->sbuoy);
    for (size_t i = 0; i < N; ++i) mag[i] = sqrt(bx[i] * bx[i] + by[i] * by[i] + mag[i] * mag[i]);
    const double enb = wsum_field(m, mag) * m->ncelli;
    free(ds); free(mag); free(bx); free(by);
    return enb;
}

void ps3o_buoyancy_diagnostics(ps3o_model *m, double out[4])
{
    const size_t N = m->nfield;
    out[0] = out[1] = out[2] = out[3] = 0.0;
    if (!m->cfg.buoyancy) return;
    ps3o_combine_physical(m, m->sbuoy, m->buoy);
    out[0] = available_potential_energy(m, m->buoy);
    out[1] = gradb_integral(m);
    double *dbdz = dalloc(N);
    ps3o_central_diffz(m, m->buoy, dbdz);
    /* get_minimum_static_stability (:327-344) */
    double mn = DBL_MAX;
    for (size_t i = 0; i < N; ++i) mn = fmin(mn, dbdz[i]);
    out[2] = 1.0 + mn / m->bfsq;
    /* get_min_richardson_number (:268-287) */
    double ri = DBL_MAX;
    for (size_t i = 0; i < N; ++i)
        ri = fmin(ri, (m->bfsq + dbdz[i]) / (m->vor[i] * m->vor[i] + m->vor[N + i] * m->vor[N + i]));
    out[3] = ri;
    free(dbdz);
}

void ps3o_setup_fields_buoyancy(ps3o_model *m, const double *vor_phys, const double *pert,
                                const double *buoy_phys, double *te_out, double *en_out)
{
    const size_t N = m->nfield;
    const int nz = m->nz;
    if (!m->cfg.buoyancy) {
        ps3o_setup_fields(m, vor_phys, pert, te_out, en_out);
        return;
    }
    memset(m->svor, 0, sizeof(double) * 3 * N);
    memset(m->vel, 0, sizeof(double) * 3 * N);
    memset(m->svel, 0, sizeof(double) * 3 * N);
    memset(m->svorts, 0, sizeof(double) * 3 * N);
    memset(m->vortsm, 0, sizeof(double) * 3 * N);
    memset(m->sbuoys, 0, sizeof(double) * N);
    memset(m->bsm, 0, sizeof(double) * N);
    memcpy(m->vor, vor_phys, sizeof(double) * 3 * N);
    memcpy(m->buoy, buoy_phys, sizeof(double) * N);
    /* calculate_basic_reference_state (physics.f90:310-340) */
    if (!m->cfg.bfsq_given) {
        double sum = 0.0;
        for (size_t c = 0; c < m->ncol; ++c) sum += m->buoy[c * m->nz1 + nz] - m->buoy[c * m->nz1];
        m->bfsq = sum / ((double)m->nx * (double)m->ny * m->extent[2]);
    }
    /* remove the basic state (utils.f90:152-158) */
    for (int iz = 0; iz <= nz; ++iz) m->bbarz[iz] = m->bfsq * (m->lower[2] + (double)iz * m->dx[2]);
    for (size_t c = 0; c < m->ncol; ++c)
        for (int iz = 0; iz <= nz; ++iz) m->buoy[c * m->nz1 + iz] -= m->bbarz[iz];
    ps3o_decompose_physical(m, m->buoy, m->sbuoy);
    for (int nc = 0; nc < 3; ++nc) ps3o_decompose_physical(m, m->vor + nc * N, m->svor + nc * N);
    if (pert)
        for (size_t i = 0; i < 3 * N; ++i) m->svor[i] += pert[i];
    ps3o_calc_vorticity_mean(m, m->ini_vor_mean);
    ps3o_vor2vel(m);
    double ke, en, hel;
    ps3o_energy_series(m, &ke, &en, &hel);
    const double ape = available_potential_energy(m, m->buoy);
    const double te = ke + ape;
    en = en + gradb_integral(m);
    ps3o_init_diffusion(m, te, en);
    if (te_out) *te_out = te;
    if (en_out) *en_out = en;
}

/* ====================================================================== */
/* adapt (advance.f90:109-377) and get_diffusion_pre_factor (:381-410)     */
/* ====================================================================== */
void ps3o_set_diffusion_vb(ps3o_model *m, double dt, double vorch, double bf)
{
    const int buoy = m->cfg.buoyancy;
    if (m->cfg.stepper == PS3O_CN2) {
        /* cn2_set_diffusion (cn2.f90:40-77) */
        const double dfac = (m->cfg.nnu == 1) ? dt : vorch * dt;
        for (size_t i = 0; i < m->nplane; ++i) m->vdiss[i] = 1.0 / (1.0 + dfac * m->vhdis[i]);
        if (buoy) {
            const double dbac = (m->cfg.buoy_nnu == 1) ? dt : bf * dt;
            for (size_t i = 0; i < m->nplane; ++i) m->bdiss[i] = 1.0 / (1.0 + dbac * m->bhdis[i]);
        }
    } else {
        /* impl_rk4_set_diffusion (impl_rk4.f90:37-53) */
        const double dfac = 0.5 * vorch * dt, dbac = 0.5 * bf * dt;
        for (size_t i = 0; i < m->nplane; ++i) m->vdiss[i] = dfac * m->vhdis[i];
        if (buoy)
            for (size_t i = 0; i < m->nplane; ++i) m->bdiss[i] = dbac * m->bhdis[i];
    }
}

void ps3o_set_diffusion(ps3o_model *m, double dt, double vorch) { ps3o_set_diffusion_vb(m, dt, vorch, 0.0); }

/* get_diffusion_pre_factor (advance.f90:381-410) */
static double pre_factor(int pretype, double vorch, double bfmax, double rmv, double rmb, double ggmax,
                         double usggmax)
{
    switch (pretype) {
    case PS3O_PRE_CONSTANT: return 1.0;
    case PS3O_PRE_VORCH: return vorch;
    case PS3O_PRE_BFMAX: return bfmax;
    case PS3O_PRE_ROLL_MEAN_BFMAX: return rmb;
    case PS3O_PRE_MAX_STRAIN: return ggmax;
    case PS3O_PRE_US_MAX_STRAIN: return usggmax;
    default: return rmv;
    }
}

/* maximum buoyancy frequency (advance.f90:147-168): gradient of the
 * buoyancy perturbation plus N^2 in z; sbuoy makes the reference's
 * combine / decompose round trip in place */
static double buoyancy_frequency_max(ps3o_model *m)
{
    const size_t N = m->nfield;
    double *xs = dalloc(N), *xp = dalloc(N), *yp = dalloc(N), *zp = dalloc(N);
    ps3o_combine_semi_spectral(m, m->sbuoy);
    ps3o_diffx(m, m->sbuoy, xs);
    ps3o_fftxys2p(m, xs, xp);
    ps3o_diffy(m, m->sbuoy, xs);
    ps3o_fftxys2p(m, xs, yp);
    ps3o_central_diffz(m, m->sbuoy, xs);
    ps3o_fftxys2p(m, xs, zp);
    ps3o_decompose_semi_spectral(m, m->sbuoy);
    double mx = -DBL_MAX;
    for (size_t i = 0; i < N; ++i) {
        const double zz = zp[i] + m->bfsq;
        mx = fmax(mx, xp[i] * xp[i] + yp[i] * yp[i] + zz * zz);
    }
    free(xs); free(xp); free(yp); free(zp);
    return sqrt(sqrt(mx));
}

void ps3o_adapt(ps3o_model *m, double t, double *dt_out, ps3o_diag *d)
{
    const size_t N = m->nfield;
    const int nz = m->nz;
    const long ncol = (long)m->ncol;
    double *xp = dalloc(N);
    for (size_t i = 0; i < N; ++i)
        xp[i] = m->vor[i] * m->vor[i] + m->vor[N + i] * m->vor[N + i] + m->vor[2 * N + i] * m->vor[2 * N + i];
    double amax = 0.0;
    for (size_t i = 0; i < N; ++i) amax = fmax(amax, fabs(xp[i]));
    const double vortmax = sqrt(amax);
    /* get_mean (:405-432) */
    const double vortrms = sqrt(wsum_fn(m, f_comp, xp) / (double)m->ncell);
    /* get_char_vorticity (:501-545) */
    double vorl1 = 1.0e-12, vorl2 = 0.0;
#pragma omp parallel for reduction(+ : vorl1, vorl2) schedule(static)
    for (long c = 0; c < ncol; ++c) {
        const size_t o = (size_t)c * m->nz1;
        for (int iz = 1; iz <= nz; ++iz) {
            const double v1 = 0.5 * fabs(m->vor[o + iz - 1] + m->vor[o + iz]);
            const double v2 = 0.5 * fabs(m->vor[N + o + iz - 1] + m->vor[N + o + iz]);
            const double v3 = 0.5 * fabs(m->vor[2 * N + o + iz - 1] + m->vor[2 * N + o + iz]);
            if (v1 + v2 + v3 > vortrms) {
                vorl1 += v1 + v2 + v3;
                vorl2 += v1 * v1 + v2 * v2 + v3 * v3;
            }
        }
    }
    const double vorch = vorl2 / vorl1;
    /* get_mean_vorticity (:549-579) */
    double vormean[3];
    for (int nc = 0; nc < 3; ++nc) vormean[nc] = wsum_fn(m, f_comp, m->vor + nc * N) * m->ncelli;

    /* velocity strain */
    double *xs = dalloc(N);
    double *dudx = dalloc(N), *dudy = dalloc(N), *dvdy = dalloc(N), *dwdx = dalloc(N), *dwdy = dalloc(N);
    ps3o_diffx(m, m->svel, xs);          ps3o_fftxys2p(m, xs, dudx);
    ps3o_diffy(m, m->svel, xs);          ps3o_fftxys2p(m, xs, dudy);
    ps3o_diffx(m, m->svel + 2 * N, xs);  ps3o_fftxys2p(m, xs, dwdx);
    ps3o_diffy(m, m->svel + N, xs);      ps3o_fftxys2p(m, xs, dvdy);
    ps3o_diffy(m, m->svel + 2 * N, xs);  ps3o_fftxys2p(m, xs, dwdy);
    double ggmax = DBL_EPSILON, usggmax = 0.0, lsggmax = 0.0;
#pragma omp parallel for reduction(max : ggmax, usggmax, lsggmax) schedule(static)
    for (long c = 0; c < ncol; ++c) {
        const size_t o = (size_t)c * m->nz1;
        for (int iz = 0; iz <= nz; ++iz) {
            const size_t q = o + iz;
            double a[9] = {0};
            a[0] = dudx[q];                               /* S11 */
            a[3] = dudy[q] + 0.5 * m->vor[2 * N + q];     /* S12 */
            a[6] = dwdx[q] + 0.5 * m->vor[N + q];         /* S13 */
            a[4] = dvdy[q];                               /* S22 */
            a[7] = dwdy[q] - 0.5 * m->vor[q];             /* S23 */
            a[8] = -(dudx[q] + dvdy[q]);                  /* S33 */
            double e[3];
            ps3o_jacobi_eigenvalues(a, e);
            const double lmax = fmax(fmax(fabs(e[0]), fabs(e[1])), fabs(e[2]));
            ggmax = fmax(ggmax, lmax);
            if (iz == nz) usggmax = fmax(usggmax, lmax);
            if (iz == 0) lsggmax = fmax(lsggmax, lmax);
        }
    }
    /* maximum (signed) speeds */
    double umax = -DBL_MAX, vmax = -DBL_MAX, wmax = -DBL_MAX;
    for (size_t i = 0; i < N; ++i) {
        umax = fmax(umax, m->vel[i]);
        vmax = fmax(vmax, m->vel[N + i]);
        wmax = fmax(wmax, m->vel[2 * N + i]);
    }
    const double small = 1.0e-12;
    const double bfmax = m->cfg.buoyancy ? buoyancy_frequency_max(m) : 0.0;
    const double dtcfl = m->cfg.cflmax * fmin(fmin(m->dx[0] / (umax + small), m->dx[1] / (vmax + small)),
                                              m->dx[2] / (wmax + small));
    double dt = fmin(fmin(m->cfg.alpha / (ggmax + small), m->cfg.alpha / (bfmax + small)),
                     fmin(dtcfl, m->cfg.time_limit - t));
    /* the buoyancy rolling mean is updated before the vorticity one
     * (advance.f90:358-366) */
    const double rmb = m->cfg.buoyancy ? roll_next(&m->rb, bfmax) : 0.0;
    const double rmv = roll_next(&m->rv, ggmax);
    const double val = pre_factor(m->cfg.pretype, vorch, bfmax, rmv, rmb, ggmax, usggmax);
    const double bval =
        m->cfg.buoyancy ? pre_factor(m->cfg.buoy_pretype, vorch, bfmax, rmv, rmb, ggmax, usggmax) : 0.0;
    ps3o_set_diffusion_vb(m, dt, val, bval);
    m->vorch = vorch; m->ggmax = ggmax; m->usggmax = usggmax; m->lsggmax = lsggmax;
    m->bfmax = bfmax; m->rmv = rmv; m->rmb = rmb;
    if (d) {
        d->t = t; d->dt = dt;
        ps3o_energy_series(m, &d->ke, &d->en, &d->hel);
        d->vortmax = vortmax; d->vortrms = vortrms; d->vorch = vorch;
        d->vormean[0] = vormean[0]; d->vormean[1] = vormean[1]; d->vormean[2] = vormean[2];
        d->ggmax = ggmax; d->usggmax = usggmax; d->lsggmax = lsggmax;
        d->umax = umax; d->vmax = vmax; d->wmax = wmax;
        d->bfmax = bfmax; d->rmv = rmv; d->pref = val;
        d->rmb = rmb; d->bpref = bval;
    }
    *dt_out = dt;
    free(xp); free(xs); free(dudx); free(dudy); free(dvdy); free(dwdx); free(dwdy);
}

/* ====================================================================== */
/* impl-diff-rk4 (impl_rk4.f90:76-364) and cn2 (cn2.f90:92-181)            */
/* ====================================================================== */
static void scale_columns(ps3o_model *m, double *q, const double *s)
{
    const long nc = (long)m->ncol;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < nc; ++c)
        for (int iz = 0; iz < m->nz1; ++iz) q[(size_t)c * m->nz1 + iz] *= s[c];
}

static void sandwich(ps3o_model *m, double *q, const double *s)
{
    ps3o_combine_semi_spectral(m, q);
    scale_columns(m, q, s);
    ps3o_decompose_semi_spectral(m, q);
}

/* vor2vel + source inside a step; with the hold_source test hook the source
 * is instead reset to its value at the start of the step */
static void stage_rhs(ps3o_model *m, const double *held)
{
    if (held) {
        memcpy(m->svorts, held, sizeof(double) * 3 * m->nfield);
        if (m->cfg.buoyancy) memcpy(m->sbuoys, held + 3 * m->nfield, sizeof(double) * m->nfield);
        return;
    }
    ps3o_vor2vel(m);
    ps3o_source(m);
}

/* impl_rk4_substep_one (impl_rk4.f90:211-240) */
static void rk4_sub1(ps3o_model *m, double *q, double *sqs, double *qdi, double *qdf, const double *mq,
                     double dt2, double dt6)
{
    const size_t N = m->nfield, P = m->nplane;
    for (size_t c = 0; c < P; ++c) {
        const double f0 = m->filt[c * m->nz1];
        for (int iz = 0; iz < m->nz1; ++iz) sqs[c * m->nz1 + iz] *= f0;
    }
    memcpy(qdi, q, sizeof(double) * N);
    for (size_t i = 0; i < N; ++i) q[i] = qdi[i] + dt2 * sqs[i];
    sandwich(m, q, mq);
    for (size_t i = 0; i < N; ++i) qdf[i] = qdi[i] + dt6 * sqs[i];
}

/* impl_rk4_substep_two / _three (impl_rk4.f90:245-324): dtq = dt/2, dt */
static void rk4_sub23(ps3o_model *m, double *q, double *sqs, const double *qdi, double *qdf, const double *mq,
                      const double *pq, double dtq, double dt3)
{
    const size_t N = m->nfield;
    sandwich(m, sqs, pq);
    for (size_t i = 0; i < N; ++i) q[i] = qdi[i] + dtq * sqs[i];
    sandwich(m, q, mq);
    for (size_t i = 0; i < N; ++i) qdf[i] = qdf[i] + dt3 * sqs[i];
}

/* impl_rk4_substep_four (impl_rk4.f90:329-362) */
static void rk4_sub4(ps3o_model *m, double *q, double *sqs, const double *qdf, const double *mq, const double *pq,
                     double dt6)
{
    const size_t N = m->nfield;
    sandwich(m, sqs, pq);
    for (size_t i = 0; i < N; ++i) q[i] = qdf[i] + dt6 * sqs[i];
    sandwich(m, q, mq);
}

/* copy of the sources for the hold_source test hook */
static double *hold_sources(ps3o_model *m)
{
    if (!m->cfg.hold_source) return NULL;
    const size_t N = m->nfield;
    double *held = dalloc(4 * N);
    memcpy(held, m->svorts, sizeof(double) * 3 * N);
    if (m->cfg.buoyancy) memcpy(held + 3 * N, m->sbuoys, sizeof(double) * N);
    return held;
}

static void impl_rk4_step(ps3o_model *m, double *t, double dt)
{
    const size_t N = m->nfield, P = m->nplane;
    const int buoy = m->cfg.buoyancy;
    double *held = hold_sources(m);
    const double dt2 = 0.5 * dt, dt3 = dt / 3.0, dt6 = dt / 6.0;
    for (size_t i = 0; i < P; ++i) {
        m->epq[i] = exp(m->vdiss[i]);
        m->emq[i] = 1.0 / m->epq[i];
        m->epq[i] = m->epq[i] * m->filt[i * m->nz1]; /* filt(0, ky, kx) */
    }
    if (buoy)
        for (size_t i = 0; i < P; ++i) {
            m->bpq[i] = exp(m->bdiss[i]);
            m->bmq[i] = 1.0 / m->bpq[i];
            m->bpq[i] = m->bpq[i] * m->filt[i * m->nz1];
        }
    /* substep 1 (buoyancy first, impl_rk4.f90:99-115) */
    if (buoy) rk4_sub1(m, m->sbuoy, m->sbuoys, m->sbuoyi, m->sbuoyf, m->bmq, dt2, dt6);
    for (int nc = 0; nc < 3; ++nc)
        rk4_sub1(m, m->svor + nc * N, m->svorts + nc * N, m->svori + nc * N, m->svorf + nc * N, m->emq, dt2,
                 dt6);
    stage_rhs(m, held);
    *t += dt2;
    /* substep 2 */
    if (buoy) rk4_sub23(m, m->sbuoy, m->sbuoys, m->sbuoyi, m->sbuoyf, m->bmq, m->bpq, dt2, dt3);
    for (int nc = 0; nc < 3; ++nc)
        rk4_sub23(m, m->svor + nc * N, m->svorts + nc * N, m->svori + nc * N, m->svorf + nc * N, m->emq,
                  m->epq, dt2, dt3);
    stage_rhs(m, held);
    *t += dt2;
    for (size_t i = 0; i < P; ++i) m->emq[i] = m->emq[i] * m->emq[i];
    if (buoy)
        for (size_t i = 0; i < P; ++i) m->bmq[i] = m->bmq[i] * m->bmq[i];
    /* substep 3 */
    if (buoy) rk4_sub23(m, m->sbuoy, m->sbuoys, m->sbuoyi, m->sbuoyf, m->bmq, m->bpq, dt, dt3);
    for (int nc = 0; nc < 3; ++nc)
        rk4_sub23(m, m->svor + nc * N, m->svorts + nc * N, m->svori + nc * N, m->svorf + nc * N, m->emq,
                  m->epq, dt, dt3);
    stage_rhs(m, held);
    for (size_t i = 0; i < P; ++i) m->epq[i] = m->epq[i] * m->epq[i];
    if (buoy)
        for (size_t i = 0; i < P; ++i) m->bpq[i] = m->bpq[i] * m->bpq[i];
    /* substep 4 */
    if (buoy) rk4_sub4(m, m->sbuoy, m->sbuoys, m->sbuoyf, m->bmq, m->bpq, dt6);
    for (int nc = 0; nc < 3; ++nc)
        rk4_sub4(m, m->svor + nc * N, m->svorts + nc * N, m->svorf + nc * N, m->emq, m->epq, dt6);
    ps3o_adjust_vorticity_mean(m);
    free(held);
}

static void cn2_update(ps3o_model *m, double dt2)
{
    const size_t N = m->nfield;
    if (m->cfg.buoyancy) {
        /* cn2.f90:107-117, 151-160 */
        for (size_t i = 0; i < N; ++i) m->sbuoy[i] = m->filt[i] * (m->bsm[i] + dt2 * m->sbuoys[i]);
        sandwich(m, m->sbuoy, m->bdiss);
    }
    for (int nc = 0; nc < 3; ++nc) {
        double *q = m->svor + nc * N;
        const double *vs = m->vortsm + nc * N, *sqs = m->svorts + nc * N;
        for (size_t i = 0; i < N; ++i) q[i] = m->filt[i] * (vs[i] + dt2 * sqs[i]);
        sandwich(m, q, m->vdiss);
    }
    ps3o_adjust_vorticity_mean(m);
}

static void cn2_step(ps3o_model *m, double *t, double dt)
{
    const size_t N = m->nfield;
    const double dt2 = 0.5 * dt;
    if (m->cfg.buoyancy)
        for (size_t i = 0; i < N; ++i) m->bsm[i] = m->sbuoy[i] + dt2 * m->sbuoys[i];
    for (size_t i = 0; i < 3 * N; ++i) m->vortsm[i] = m->svor[i] + dt2 * m->svorts[i];
    cn2_update(m, dt2);
    double *held = hold_sources(m);
    for (int iter = 0; iter < 2; ++iter) {
        stage_rhs(m, held);
        cn2_update(m, dt2);
    }
    free(held);
    *t += dt;
}

void ps3o_step(ps3o_model *m, double *t, double dt)
{
    if (m->cfg.stepper == PS3O_CN2) cn2_step(m, t, dt);
    else impl_rk4_step(m, t, dt);
}

void ps3o_advance(ps3o_model *m, double *t, ps3o_diag *d)
{
    double dt;
    ps3o_vor2vel(m);
    ps3o_adapt(m, *t, &dt, d);
    ps3o_source(m);
    ps3o_step(m, t, dt);
}

/* ====================================================================== */
/* accessors                                                              */
/* ====================================================================== */
int ps3o_get_table(ps3o_model *m, int which, double *out)
{
    const size_t N = m->nfield, P = m->nplane;
    const double *src = NULL;
    size_t n = 0;
    switch (which) {
    case 0: src = m->k2l2; n = P; break;
    case 1: src = m->k2l2i; n = P; break;
    case 2: src = m->filt; n = N; break;
    case 3: src = m->green; n = N; break;
    case 4: src = m->phim; n = N; break;
    case 5: src = m->phip; n = N; break;
    case 6: src = m->thetam; n = N; break;
    case 7: src = m->thetap; n = N; break;
    case 8: src = m->dthetam; n = N; break;
    case 9: src = m->dthetap; n = N; break;
    case 10: src = m->gamtop; n = m->nz1; break;
    case 11: src = m->gambot; n = m->nz1; break;
    case 12: src = m->vhdis; n = P; break;
    case 13: src = m->rkx; n = m->nx; break;
    case 14: src = m->rky; n = m->ny; break;
    case 15: src = m->rkz; n = m->nz1; break;
    case 16: src = m->dphim; n = N; break;
    case 17: src = m->dphip; n = N; break;
    case 18: src = m->bhdis; n = P; break;
    case 19: src = m->bbarz; n = m->nz1; break;
    default: return 1;
    }
    if (!src) return 1;
    memcpy(out, src, sizeof(double) * n);
    return 0;
}

static double *field_ptr(ps3o_model *m, int which, size_t *n)
{
    *n = 3 * m->nfield;
    switch (which) {
    case 0: return m->svor;
    case 1: return m->vor;
    case 2: return m->vel;
    case 3: return m->svel;
    case 4: return m->svorts;
    }
    *n = m->nfield;
    switch (which) {
    case 5: return m->sbuoy;
    case 6: return m->buoy;
    case 7: return m->sbuoys;
    default: return NULL;
    }
}

int ps3o_get_field(ps3o_model *m, int which, double *out)
{
    size_t n;
    double *p = field_ptr(m, which, &n);
    if (!p) return 1;
    memcpy(out, p, sizeof(double) * n);
    return 0;
}

int ps3o_set_field(ps3o_model *m, int which, const double *in)
{
    size_t n;
    double *p = field_ptr(m, which, &n);
    if (!p) return 1;
    memcpy(p, in, sizeof(double) * n);
    return 0;
}

double ps3o_get_bfsq(ps3o_model *m) { return m->bfsq; }
double ps3o_get_bvisc(ps3o_model *m) { return m->bvisc; }

void ps3o_get_ini_vor_mean(ps3o_model *m, double out[2])
{
    out[0] = m->ini_vor_mean[0];
    out[1] = m->ini_vor_mean[1];
}

void ps3o_set_ini_vor_mean(ps3o_model *m, const double in[2])
{
    m->ini_vor_mean[0] = in[0];
    m->ini_vor_mean[1] = in[1];
}

double ps3o_get_vvisc(ps3o_model *m) { return m->vvisc; }

/* ====================================================================== */
/* derived fields (fields_derived.f90:67-182): pressure                    */
/* from Lap(p) = 2[J_xy(u,v) + J_yz(v,w) + J_zx(w,u)] with dp/dz = 0 on the */
/* walls (DCT - Green function - DCT), and the horizontal divergence       */
/* ====================================================================== */
void ps3o_pressure(ps3o_model *m, double *pres)
{
    const size_t N = m->nfield;
    double *xs = dalloc(N), *rs = dalloc(N);
    double *dudx = dalloc(N), *dudy = dalloc(N), *dvdy = dalloc(N), *dwdx = dalloc(N), *dwdy = dalloc(N);
    /* velocity gradients as in adapt (advance.f90:193-217) */
    ps3o_diffx(m, m->svel, xs);          ps3o_fftxys2p(m, xs, dudx);
    ps3o_diffy(m, m->svel, xs);          ps3o_fftxys2p(m, xs, dudy);
    ps3o_diffx(m, m->svel + 2 * N, xs);  ps3o_fftxys2p(m, xs, dwdx);
    ps3o_diffy(m, m->svel + N, xs);      ps3o_fftxys2p(m, xs, dvdy);
    ps3o_diffy(m, m->svel + 2 * N, xs);  ps3o_fftxys2p(m, xs, dwdy);
    const double *xi = m->vor, *eta = m->vor + N, *zeta = m->vor + 2 * N;
    for (size_t i = 0; i < N; ++i) {
        const double dwdz = -(dudx[i] + dvdy[i]);
        pres[i] = 2.0 * (dudx[i] * dvdy[i] - dudy[i] * (zeta[i] + dudy[i]) +
                         dvdy[i] * dwdz - dwdy[i] * (dwdy[i] - xi[i]) +
                         dwdz * dudx[i] - dwdx[i] * (dwdx[i] + eta[i]));
    }
    if (m->cfg.buoyancy) {
        /* fields_derived.f90:108-112 */
        double *dbdz = dalloc(N);
        ps3o_combine_physical(m, m->sbuoy, m->buoy);
        ps3o_central_diffz(m, m->buoy, dbdz);
        for (size_t i = 0; i < N; ++i) pres[i] = pres[i] + dbdz[i] + m->cfg.f_cor[2] * zeta[i];
        free(dbdz);
    }
    ps3o_fftxyp2s(m, pres, rs);
    ps3o_fftcosine(m, rs);
    for (size_t i = 0; i < N; ++i) rs[i] = m->green[i] * rs[i];
    ps3o_fftcosine(m, rs);
    if (m->cfg.buoyancy) {
        /* fields_derived.f90:142-151 */
        for (size_t c = 0; c < m->ncol; ++c) {
            const size_t o = c * m->nz1;
            for (int iz = 0; iz <= m->nz; ++iz)
                rs[o + iz] = rs[o + iz] + m->sbuoy[o + m->nz] * m->k2l2i[c] * m->dphip[o + iz] +
                             m->sbuoy[o] * m->k2l2i[c] * m->dphim[o + iz];
        }
    }
    ps3o_fftxys2p(m, rs, pres);
    free(xs); free(rs); free(dudx); free(dudy); free(dvdy); free(dwdx); free(dwdy);
}

void ps3o_horizontal_divergence(ps3o_model *m, double *delta)
{
    const size_t N = m->nfield;
    double *uxs = dalloc(N), *vys = dalloc(N);
    ps3o_diffx(m, m->svel, uxs);
    ps3o_diffy(m, m->svel + N, vys);
    for (size_t i = 0; i < N; ++i) uxs[i] = uxs[i] + vys[i];
    ps3o_fftxys2p(m, uxs, delta);
    free(uxs); free(vys);
}

/* kinetic-energy shell spectrum (genspec.f90:42-123): svel = fftxyp2s(vel),  */
/* dct of u and v, dst of w's interior per column, squared amplitudes summed */
/* into shells m = int(nint(|K|) / dk), scaled by the shell volume over the   */
/* count and normalised to the domain-average kinetic energy.  Returns the  */
/* number of shells (kmax + 1, at most nmax written) and dk.                */
int ps3o_ke_spectrum(ps3o_model *m, int nmax, double *spec, double *dk_out)
{
    const int nx = m->nx, ny = m->ny, nz = m->nz;
    const size_t N = m->nfield;
    double *sv = dalloc(3 * N);
    for (int nc = 0; nc < 3; ++nc) ps3o_fftxyp2s(m, m->vel + nc * N, sv + nc * N);
    double *w1 = dalloc(nz + 1), *w2 = dalloc(nz + 1);
    for (size_t c = 0; c < m->ncol; ++c) {
        const size_t o = c * m->nz1;
        ps3o_dct(1, nz, sv + o, w1, w2, m->ztrig, m->zfac);
        ps3o_dct(1, nz, sv + N + o, w1, w2, m->ztrig, m->zfac);
        ps3o_dst(1, nz, sv + 2 * N + o + 1, w1, w2, m->ztrig, m->zfac);
    }
    int kmax = 0;
    for (int kx = 0; kx < nx; ++kx)
        for (int ky = 0; ky < ny; ++ky)
            for (int kz = 0; kz <= nz; ++kz) {
                const int km = (int)lround(sqrt(m->rkx[kx] * m->rkx[kx] + m->rky[ky] * m->rky[ky] +
                                                m->rkz[kz] * m->rkz[kz]));
                if (km > kmax) kmax = km;
            }
    const double dk = (double)kmax / sqrt((0.5 * nx) * (0.5 * nx) + (0.5 * ny) * (0.5 * ny) + (double)nz * nz);
    const double dki = 1.0 / dk;
    double *sp = dalloc(kmax + 1);
    long *num = (long *)calloc((size_t)kmax + 1, sizeof(long));
    for (int kx = 0; kx < nx; ++kx)
        for (int ky = 0; ky < ny; ++ky)
            for (int kz = 0; kz <= nz; ++kz) {
                const int km = (int)lround(sqrt(m->rkx[kx] * m->rkx[kx] + m->rky[ky] * m->rky[ky] +
                                                m->rkz[kz] * m->rkz[kz]));
                int b = (int)((double)km * dki);
                if (b > kmax) b = kmax;
                const size_t q = IDX(m, kz, ky, kx);
                sp[b] += sv[q] * sv[q] + sv[N + q] * sv[N + q] + sv[2 * N + q] * sv[2 * N + q];
                num[b] += 1;
            }
    const double pi = 3.14159265358979323846;
    const double pref = 4.0 / 3.0 * pi * dk * dk * dk;
    for (int b = 0; b <= kmax; ++b)
        if (num[b] > 0) sp[b] = sp[b] * pref * (double)((long)(b + 1) * (b + 1) * (b + 1) - (long)b * b * b) / (double)num[b];
    double ke, en, hel;
    ps3o_energy_series(m, &ke, &en, &hel);
    double tot = 0.0;
    for (int b = 0; b <= kmax; ++b) tot += sp[b] * dk;
    const double snorm = ke / tot;
    for (int b = 0; b <= kmax && b < nmax; ++b) spec[b] = sp[b] * snorm;
    *dk_out = dk;
    free(sv); free(w1); free(w2); free(sp); free(num);
    return kmax + 1;
}
