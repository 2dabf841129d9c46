// Elementwise, stencil, stepper and reduction kernels of the ps3d hot path.
//
// All kernels walk columns: a block is 32 x 8 threads, threadIdx.x runs along
// z (coalesced: 32 consecutive z of one column per warp), threadIdx.y picks
// one of 8 columns.  Spectral x/y derivatives read the partner column
// src(k) = (n - k) mod n, which is itself a contiguous z run.  Arithmetic is
// done in FP64 registers whatever the storage type, so the mixed-precision
// form only rounds at loads and stores.
#include <float.h>
#include <limits.h>

#include "kernels.h"

namespace ps3d {

#define COLS_PER_BLOCK 8

__device__ __forceinline__ int xsrc(int kx, int nx) { return kx == 0 ? 0 : nx - kx; }

#define COLUMN_HEADER                                                          \
    const long long col = (long long)blockIdx.x * COLS_PER_BLOCK + threadIdx.y; \
    if (col >= d.ncol) return;                                                 \
    const int kx = (int)(col / d.ny);                                          \
    const int ky = (int)(col - (long long)kx * d.ny);                          \
    const long long o = col * d.P;                                             \
    (void)kx; (void)ky;

#define PARTNERS                                                               \
    const long long ox = ((long long)ky + (long long)d.ny * xsrc(kx, d.nx)) * d.P; \
    const long long oy = ((long long)xsrc(ky, d.ny) + (long long)d.ny * kx) * d.P; \
    const double cxk = D.cx[kx], cyk = D.cy[ky];

static inline dim3 col_grid(const Dims &d)
{
    return dim3((unsigned)((d.ncol + COLS_PER_BLOCK - 1) / COLS_PER_BLOCK));
}
static const dim3 COL_BLOCK(32, COLS_PER_BLOCK);

// ---------------------------------------------------------------- diff x/y
template <typename T>
__global__ void k_diff(Dims d, Deriv D, int axis, const T *__restrict__ in, T *__restrict__ out)
{
    COLUMN_HEADER
    PARTNERS
    const long long os = axis == 0 ? ox : oy;
    const T c = (T)(axis == 0 ? cxk : cyk);
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) out[o + iz] = c * in[os + iz];
}
template <typename T> void op_diff(const Dims &d, cudaStream_t st, const Deriv &D, int axis, const T *in, T *out)
{
    k_diff<T><<<col_grid(d), COL_BLOCK, 0, st>>>(d, D, axis, in, out);
}

// ------------------------------------------------------------ central diffz
template <typename T>
__global__ void k_diffz(Dims d, double dzi, const T *__restrict__ in, T *__restrict__ out)
{
    COLUMN_HEADER
    const int nz = d.nz;
    const T dz = (T)dzi, hdz = (T)(0.5 * dzi);
    for (int iz = threadIdx.x; iz <= nz; iz += 32) {
        T v;
        if (iz == 0) v = dz * (in[o + 1] - in[o]);
        else if (iz == nz) v = dz * (in[o + nz] - in[o + nz - 1]);
        else v = (in[o + iz + 1] - in[o + iz - 1]) * hdz;
        out[o + iz] = v;
    }
}
template <typename T> void op_diffz(const Dims &d, cudaStream_t st, double dzi, const T *in, T *out)
{
    k_diffz<T><<<col_grid(d), COL_BLOCK, 0, st>>>(d, dzi, in, out);
}

// ------------------------------------------------------------------ vor2vel
// ds = D_x B - D_y A   (inversion.f90:39-42 and :86-90 with A, B swapped roles)
template <typename T, typename S>
__global__ void k_v2v_ds(Dims d, Deriv D, const S *__restrict__ A, const S *__restrict__ B, T *__restrict__ ds)
{
    COLUMN_HEADER
    PARTNERS
    const T cx = (T)cxk, cy = (T)cyk;
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) ds[o + iz] = cx * (T)B[ox + iz] - cy * (T)A[oy + iz];
}
template <typename T, typename S>
void op_v2v_ds(const Dims &d, cudaStream_t st, const Deriv &D, const S *A, const S *B, T *ds)
{
    k_v2v_ds<T, S><<<col_grid(d), COL_BLOCK, 0, st>>>(d, D, A, B, ds);
}

// ds = D_y A - D_x B   (inversion.f90:86-90)
template <typename T, typename S>
__global__ void k_v2v_wsrc(Dims d, Deriv D, const S *__restrict__ A, const S *__restrict__ B, T *__restrict__ ds)
{
    COLUMN_HEADER
    PARTNERS
    const T cx = (T)cxk, cy = (T)cyk;
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) ds[o + iz] = cy * (T)A[oy + iz] - cx * (T)B[ox + iz];
}
template <typename T, typename S>
void op_v2v_wsrc(const Dims &d, cudaStream_t st, const Deriv &D, const S *A, const S *B, T *ds)
{
    k_v2v_wsrc<T, S><<<col_grid(d), COL_BLOCK, 0, st>>>(d, D, A, B, ds);
}

// Orbit form of the two horizontal inversions below (the projection of
// inversion.f90:50-76 and u, v of :169-213):
//   a = k2l2i (D_x e + D_y f),  b = k2l2i (D_y e - D_x f),
// D_x f at (kx, ky) reading f at (nx - kx, ky) and D_y at (kx, ny - ky).  The
// columns (kx, ky), (nx-kx, ky), (kx, ny-ky), (nx-kx, ny-ky) read only one
// another, so one block takes the whole orbit: e and f are read once instead
// of twice.  Same expression per output as the per-column form.  MEAN: the
// (0,0) column gets ubar, vbar; otherwise it is left as it is.
template <typename T, typename S, bool MEAN>
__global__ void __launch_bounds__(128) k_v2v_orbit(Dims d, Deriv D, const double *__restrict__ k2l2i,
                                                   const T *__restrict__ e, const T *__restrict__ f,
                                                   const double *__restrict__ ubar, const double *__restrict__ vbar,
                                                   S *__restrict__ a, S *__restrict__ b)
{
    // one 128-thread block per orbit, warp w on member (x partner if w & 1,
    // y partner if w & 2); the members' e and f meet in shared memory (two
    // buffers, alternating), next levels' loads issued before the barrier
    __shared__ S sh_e[2][4][32], sh_f[2][4][32];
    const int hy = d.ny / 2 + 1;
    const long long orb = blockIdx.x;
    const int kx = (int)(orb / hy), ky = (int)(orb - (long long)kx * hy);
    const int x2 = xsrc(kx, d.nx), y2 = xsrc(ky, d.ny);
    const bool dx = x2 != kx, dy = y2 != ky;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool active = (!(w & 1) || dx) && (!(w & 2) || dy);
    const int mx = (w & 1) ? x2 : kx, my = (w & 2) ? y2 : ky;
    const int xw = dx ? (w ^ 1) : w, yw = dy ? (w ^ 2) : w;
    const long long col = (long long)my + (long long)d.ny * mx, o = col * d.P;
    if (col == 0) {  // the (0,0) column: the mean flow, or left as it is
        if (MEAN && active)
            for (int iz = lane; iz <= d.nz; iz += 32) {
                a[iz] = (S)ubar[iz];
                b[iz] = (S)vbar[iz];
            }
        return;  // the (0,0) orbit has no other member
    }
    const S cx = (S)D.cx[mx], cy = (S)D.cy[my], kk = (S)k2l2i[col];
    auto ld = [&](const T *g, int iz) { return (active && iz <= d.nz) ? (S)g[o + iz] : (S)0; };
    S ev = ld(e, lane), fv = ld(f, lane);
    int buf = 0;
    for (int z0 = 0; z0 <= d.nz; z0 += 32, buf ^= 1) {
        const int iz = z0 + lane;
        sh_e[buf][w][lane] = ev;
        sh_f[buf][w][lane] = fv;
        if (z0 + 32 <= d.nz) {
            ev = ld(e, iz + 32);
            fv = ld(f, iz + 32);
        }
        __syncthreads();
        if (active && iz <= d.nz) {
            a[o + iz] = kk * (cx * sh_e[buf][xw][lane] + cy * sh_f[buf][yw][lane]);
            b[o + iz] = kk * (cy * sh_e[buf][yw][lane] - cx * sh_f[buf][xw][lane]);
        }
    }
}
// one block per partner orbit
static inline unsigned orbit_blocks(const Dims &d) { return (unsigned)((long long)(d.nx / 2 + 1) * (d.ny / 2 + 1)); }

// A = k2l2i (D_x es + D_y ds), B = k2l2i (D_y es - D_x ds); the (0,0) column
// keeps its mean vorticity (inversion.f90:50-76)
template <typename T, typename S>
void op_v2v_project(const Dims &d, cudaStream_t st, const Deriv &D, const double *k2l2i, const T *es,
                    const T *ds, S *A, S *B)
{
    k_v2v_orbit<T, S, false><<<orbit_blocks(d), 128, 0, st>>>(d, D, k2l2i, es, ds, nullptr, nullptr, A, B);
}

// boundary contributions and Green-function inversion for w
// (inversion.f90:94-122)
template <typename T>
__global__ void k_v2v_wprep(Dims d, const T *__restrict__ ds, const T *__restrict__ thetam,
                            const T *__restrict__ thetap, const T *__restrict__ dthetam,
                            const T *__restrict__ dthetap, const T *__restrict__ green,
                            const double *__restrict__ rkz, T *__restrict__ bs, T *__restrict__ es,
                            T *__restrict__ dsg, T *__restrict__ as)
{
    COLUMN_HEADER
    const int nz = d.nz;
    const T d0 = ds[o], dn = ds[o + nz];
    for (int iz = threadIdx.x; iz <= nz; iz += 32) {
        const long long q = o + iz;
        es[q] = d0 * dthetam[q] + dn * dthetap[q];
        if (iz > 0 && iz < nz) {
            bs[q] = d0 * thetam[q] + dn * thetap[q];
            const T g = green[q] * ds[q];
            dsg[q] = g;
            as[q] = (T)rkz[iz] * g;
        } else {
            bs[q] = (T)0;
            dsg[q] = (T)0;
            as[q] = (T)0;
        }
    }
}
template <typename T>
void op_v2v_wprep(const Dims &d, cudaStream_t st, const T *ds, const T *thetam, const T *thetap,
                  const T *dthetam, const T *dthetap, const T *green, const double *rkz, T *bs, T *es,
                  T *dsg, T *as)
{
    k_v2v_wprep<T><<<col_grid(d), COL_BLOCK, 0, st>>>(d, ds, thetam, thetap, dthetam, dthetap, green, rkz, bs,
                                                      es, dsg, as);
}

// w = [0, dst(green ds) + bs, 0], dw/dz = es + dct(rkz green ds)
// (inversion.f90:136-139)
template <typename T>
__global__ void k_v2v_wfinish(Dims d, const T *__restrict__ dsg, const T *__restrict__ bs,
                              const T *__restrict__ as, T *__restrict__ w, T *__restrict__ es)
{
    COLUMN_HEADER
    const int nz = d.nz;
    for (int iz = threadIdx.x; iz <= nz; iz += 32) {
        const long long q = o + iz;
        w[q] = (iz > 0 && iz < nz) ? dsg[q] + bs[q] : (T)0;
        es[q] = es[q] + as[q];
    }
}
template <typename T>
void op_v2v_wfinish(const Dims &d, cudaStream_t st, const T *dsg, const T *bs, const T *as, T *w, T *es)
{
    k_v2v_wfinish<T><<<col_grid(d), COL_BLOCK, 0, st>>>(d, dsg, bs, as, w, es);
}

// horizontally averaged flow from the (0,0) column (inversion.f90:150-165):
// ubar = dct(-rkzi B) + B(nz) gamtop - B(0) gambot, vbar likewise.  The
// cosine transform of the single column is a direct O(nz^2) sum, one warp
// per output level.
template <typename S>
__global__ void k_v2v_meanflow(int nz, const S *__restrict__ A, const S *__restrict__ B,
                               const double *__restrict__ rkzi, const double *__restrict__ dctcos,
                               const double *__restrict__ gamtop, const double *__restrict__ gambot,
                               double *__restrict__ ubar, double *__restrict__ vbar)
{
    const int lane = threadIdx.x & 31;
    const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (k > nz) return;
    double su = 0.0, sv = 0.0;
    for (int j = 1 + lane; j < nz; j += 32) {
        const double c = dctcos[(int)(((long long)j * k) % (2 * nz))];
        su -= rkzi[j] * (double)B[j] * c;
        sv += rkzi[j] * (double)A[j] * c;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        su += __shfl_xor_sync(0xffffffffu, su, o);
        sv += __shfl_xor_sync(0xffffffffu, sv, o);
    }
    if (lane == 0) {
        const double s = sqrt(2.0 / (double)nz);
        const double a0 = (double)A[0], an = (double)A[nz], b0 = (double)B[0], bn = (double)B[nz];
        ubar[k] = s * su + bn * gamtop[k] - b0 * gambot[k];
        vbar[k] = s * sv - an * gamtop[k] + a0 * gambot[k];
    }
}
template <typename S>
void op_v2v_meanflow(const Dims &d, cudaStream_t st, const S *A, const S *B, const Tables &tb, double *ubar,
                     double *vbar)
{
    k_v2v_meanflow<S><<<(d.nz + 1 + 7) / 8, 256, 0, st>>>(d.nz, A, B, tb.rkzi, tb.dctcos, tb.gamtop, tb.gambot,
                                                          ubar, vbar);
}

// u = k2l2i (D_x es + D_y cs), v = k2l2i (D_y es - D_x cs), (0,0) = ubar, vbar
// (inversion.f90:169-213)
template <typename T>
void op_v2v_uv(const Dims &d, cudaStream_t st, const Deriv &D, const double *k2l2i, const T *es, const T *cs,
               const double *ubar, const double *vbar, T *u, T *v)
{
    k_v2v_orbit<T, T, true><<<orbit_blocks(d), 128, 0, st>>>(d, D, k2l2i, es, cs, ubar, vbar, u, v);
}

// ------------------------------------------------------------------- source
template <typename T>
__global__ void k_add_const(Dims d, T *__restrict__ f, double c)
{
    COLUMN_HEADER
    const T cc = (T)c;
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) f[o + iz] = f[o + iz] + cc;
}
template <typename T> void op_add_const(const Dims &d, cudaStream_t st, T *f, double c)
{
    k_add_const<T><<<col_grid(d), COL_BLOCK, 0, st>>>(d, f, c);
}

// r = u eta - v xi, q = w xi - u zeta, p = v zeta - w eta (inversion.f90:327-352)
template <typename T>
__global__ void k_products(Dims d, const T *__restrict__ vel, const T *__restrict__ vor, T *__restrict__ r,
                           T *__restrict__ q, T *__restrict__ p)
{
    COLUMN_HEADER
    const long long N = d.nfield;
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) {
        const long long i = o + iz;
        const T u = vel[i], v = vel[N + i], w = vel[2 * N + i];
        const T xi = vor[i], eta = vor[N + i], zeta = vor[2 * N + i];
        r[i] = u * eta - v * xi;
        q[i] = w * xi - u * zeta;
        p[i] = v * zeta - w * eta;
    }
}
template <typename T>
void op_products(const Dims &d, cudaStream_t st, const T *vel, const T *vor, T *r, T *q, T *p)
{
    k_products<T><<<col_grid(d), COL_BLOCK, 0, st>>>(d, vel, vor, r, q, p);
}

// The products together with the z derivatives of q and p (central_diffz,
// inversion_utils.f90:653-673) in one pass over each column: the
// neighbours iz -+ 1 come from the adjacent lanes, and across 32-level
// chunks from the previous chunk (carried) or the next one (the last lane's
// derivative is written one chunk later).  Same arithmetic as k_products
// followed by k_diffz.
template <typename T>
__global__ void k_products_dz(Dims d, T dzi, T hdzi, const T *__restrict__ vel, const T *__restrict__ vor,
                              T *__restrict__ r, T *__restrict__ q, T *__restrict__ p, T *__restrict__ gq,
                              T *__restrict__ gp)
{
    COLUMN_HEADER
    const long long N = d.nfield;
    const int nz = d.nz, lane = threadIdx.x;
    T q1 = 0, p1 = 0, q2 = 0, p2 = 0;  // levels 32c - 1 and 32c - 2 of the previous chunk
    for (int c0 = 0; c0 <= nz; c0 += 32) {
        const int iz = c0 + lane;
        T qv = 0, pv = 0;
        if (iz <= nz) {
            const long long i = o + iz;
            const T u = vel[i], v = vel[N + i], w = vel[2 * N + i];
            const T xi = vor[i], eta = vor[N + i], zeta = vor[2 * N + i];
            r[i] = u * eta - v * xi;
            qv = w * xi - u * zeta;
            pv = v * zeta - w * eta;
            q[i] = qv;
            p[i] = pv;
        }
        T qm = __shfl_up_sync(0xffffffffu, qv, 1), pm = __shfl_up_sync(0xffffffffu, pv, 1);
        const T qn = __shfl_down_sync(0xffffffffu, qv, 1), pn = __shfl_down_sync(0xffffffffu, pv, 1);
        const T q0 = __shfl_sync(0xffffffffu, qv, 0), p0 = __shfl_sync(0xffffffffu, pv, 0);
        if (lane == 0) {
            qm = q1;
            pm = p1;
        }
        // the previous chunk's last level, now that its upper neighbour is known
        if (c0 > 0 && lane == 31) {
            gq[o + c0 - 1] = (q0 - q2) * hdzi;
            gp[o + c0 - 1] = (p0 - p2) * hdzi;
        }
        if (iz <= nz) {
            T a = 0, b = 0;
            bool put = true;
            if (iz == 0) {
                a = (qn - qv) * dzi;
                b = (pn - pv) * dzi;
            } else if (iz == nz) {
                a = (qv - qm) * dzi;
                b = (pv - pm) * dzi;
            } else if (lane < 31) {
                a = (qn - qm) * hdzi;
                b = (pn - pm) * hdzi;
            } else {
                put = false;
            }
            if (put) {
                gq[o + iz] = a;
                gp[o + iz] = b;
            }
        }
        q1 = __shfl_sync(0xffffffffu, qv, 31);
        p1 = __shfl_sync(0xffffffffu, pv, 31);
        q2 = __shfl_sync(0xffffffffu, qv, 30);
        p2 = __shfl_sync(0xffffffffu, pv, 30);
    }
}
template <typename T>
void op_products_dz(const Dims &d, cudaStream_t st, double dzi, const T *vel, const T *vor, T *r, T *q, T *p,
                    T *gq, T *gp)
{
    k_products_dz<T><<<col_grid(d), COL_BLOCK, 0, st>>>(d, (T)dzi, (T)(0.5 * dzi), vel, vor, r, q, p, gq, gp);
}
template void op_products_dz<float>(const Dims &, cudaStream_t, double, const float *, const float *, float *,
                                    float *, float *, float *, float *);

// svorts = (D_y r - dq/dz, dp/dz - D_x r, D_x q - D_y p) (inversion.f90:341-367)
// in orbit form: one 128-thread block per partner orbit {(kx,ky), (nx-kx,ky),
// (kx,ny-ky), (nx-kx,ny-ky)}, warp w on member (x partner if w & 1, y
// partner if w & 2), 32 levels at a time.  The members' r, q, p meet in
// shared memory (two buffers, alternating), so every product column is read
// once from HBM; the next 32 levels' loads are issued before the current
// levels' barrier.  The same expression per output as the per-column form.
template <typename T>
__global__ void __launch_bounds__(128) k_svorts_orbit(Dims d, Deriv D, const T *__restrict__ r,
                                                      const T *__restrict__ q, const T *__restrict__ p,
                                                      const T *__restrict__ gq, const T *__restrict__ gp,
                                                      T *__restrict__ s1, T *__restrict__ s2, T *__restrict__ s3)
{
    __shared__ T sh_r[2][4][32], sh_q[2][4][32], sh_p[2][4][32];
    const int hy = d.ny / 2 + 1;
    const long long orb = blockIdx.x;
    const int kx = (int)(orb / hy), ky = (int)(orb - (long long)kx * hy);
    const int x2 = xsrc(kx, d.nx), y2 = xsrc(ky, d.ny);
    const bool dx = x2 != kx, dy = y2 != ky;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool active = (!(w & 1) || dx) && (!(w & 2) || dy);
    const int mx = (w & 1) ? x2 : kx, my = (w & 2) ? y2 : ky;
    const int xw = dx ? (w ^ 1) : w, yw = dy ? (w ^ 2) : w;  // partner members
    const long long o = ((long long)my + (long long)d.ny * mx) * d.P;
    const T cx = (T)D.cx[mx], cy = (T)D.cy[my];
    auto ld = [&](const T *f, int iz) { return (active && iz <= d.nz) ? f[o + iz] : (T)0; };
    T rv = ld(r, lane), qv = ld(q, lane), pv = ld(p, lane), gqv = ld(gq, lane), gpv = ld(gp, lane);
    int buf = 0;
    for (int z0 = 0; z0 <= d.nz; z0 += 32, buf ^= 1) {
        const int iz = z0 + lane;
        sh_r[buf][w][lane] = rv;
        sh_q[buf][w][lane] = qv;
        sh_p[buf][w][lane] = pv;
        const T gqc = gqv, gpc = gpv;
        if (z0 + 32 <= d.nz) {
            rv = ld(r, iz + 32);
            qv = ld(q, iz + 32);
            pv = ld(p, iz + 32);
            gqv = ld(gq, iz + 32);
            gpv = ld(gp, iz + 32);
        }
        __syncthreads();
        if (active && iz <= d.nz) {
            const long long i = o + iz;
            s1[i] = cy * sh_r[buf][yw][lane] - gqc;
            s2[i] = gpc - cx * sh_r[buf][xw][lane];
            s3[i] = cx * sh_q[buf][xw][lane] - cy * sh_p[buf][yw][lane];
        }
    }
}
template <typename T>
void op_svorts(const Dims &d, cudaStream_t st, const Deriv &D, const T *r, const T *q, const T *p,
               const T *gq, const T *gp, T *s1, T *s2, T *s3)
{
    const unsigned norb = (unsigned)((long long)(d.nx / 2 + 1) * (d.ny / 2 + 1));
    k_svorts_orbit<T><<<norb, 128, 0, st>>>(d, D, r, q, p, gq, gp, s1, s2, s3);
}

// spectral velocity gradients for the strain (advance.f90:193-217):
// du/dx, du/dy, dw/dx, dv/dy, dw/dy
// Orbit form (as k_v2v_orbit): each velocity column read once.
template <typename T>
__global__ void __launch_bounds__(128) k_strain_orbit(Dims d, Deriv D, const T *__restrict__ svel,
                                                      T *__restrict__ g5)
{
    // one 128-thread block per orbit as k_v2v_orbit: the members' u, v, w
    // meet in shared memory
    __shared__ T sh_u[2][4][32], sh_v[2][4][32], sh_w[2][4][32];
    const long long N = d.nfield;
    const int hy = d.ny / 2 + 1;
    const long long orb = blockIdx.x;
    const int kx = (int)(orb / hy), ky = (int)(orb - (long long)kx * hy);
    const int x2 = xsrc(kx, d.nx), y2 = xsrc(ky, d.ny);
    const bool dx = x2 != kx, dy = y2 != ky;
    const int wp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool active = (!(wp & 1) || dx) && (!(wp & 2) || dy);
    const int mx = (wp & 1) ? x2 : kx, my = (wp & 2) ? y2 : ky;
    const int xw = dx ? (wp ^ 1) : wp, yw = dy ? (wp ^ 2) : wp;
    const long long o = ((long long)my + (long long)d.ny * mx) * d.P;
    const T cx = (T)D.cx[mx], cy = (T)D.cy[my];
    const T *u = svel, *v = svel + N, *w = svel + 2 * N;
    auto ld = [&](const T *g, int iz) { return (active && iz <= d.nz) ? g[o + iz] : (T)0; };
    T uv = ld(u, lane), vv = ld(v, lane), wv = ld(w, lane);
    int buf = 0;
    for (int z0 = 0; z0 <= d.nz; z0 += 32, buf ^= 1) {
        const int iz = z0 + lane;
        sh_u[buf][wp][lane] = uv;
        sh_v[buf][wp][lane] = vv;
        sh_w[buf][wp][lane] = wv;
        if (z0 + 32 <= d.nz) {
            uv = ld(u, iz + 32);
            vv = ld(v, iz + 32);
            wv = ld(w, iz + 32);
        }
        __syncthreads();
        if (active && iz <= d.nz) {
            const long long i = o + iz;
            // du/dx, du/dy, dw/dx, dv/dy, dw/dy (advance.f90:193-217)
            g5[i] = cx * sh_u[buf][xw][lane];
            g5[N + i] = cy * sh_u[buf][yw][lane];
            g5[2 * N + i] = cx * sh_w[buf][xw][lane];
            g5[3 * N + i] = cy * sh_v[buf][yw][lane];
            g5[4 * N + i] = cy * sh_w[buf][yw][lane];
        }
    }
}
template <typename T>
void op_strain_fields(const Dims &d, cudaStream_t st, const Deriv &D, const T *svel, T *g5)
{
    k_strain_orbit<T><<<orbit_blocks(d), 128, 0, st>>>(d, D, svel, g5);
}

// Derived fields (fields_derived.f90:67-182, buoyancy disabled).
// Right-hand side of the pressure Poisson equation from the physical
// velocity gradients g5 = (du/dx, du/dy, dw/dx, dv/dy, dw/dy) and the
// vorticity: 2 [J_xy(u,v) + J_yz(v,w) + J_zx(w,u)] with dv/dx = zeta + du/dy,
// du/dz = eta + dw/dx, dv/dz = dw/dy - xi, dw/dz = -(du/dx + dv/dy).
template <typename T>
__global__ void k_pressure_rhs(Dims d, const T *__restrict__ g5, const T *__restrict__ vor, T *__restrict__ out)
{
    COLUMN_HEADER
    const long long N = d.nfield;
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) {
        const long long i = o + iz;
        const T dudx = g5[i], dudy = g5[N + i], dwdx = g5[2 * N + i], dvdy = g5[3 * N + i], dwdy = g5[4 * N + i];
        const T xi = vor[i], eta = vor[N + i], zeta = vor[2 * N + i];
        const T dwdz = -(dudx + dvdy);
        out[i] = (T)2 * (dudx * dvdy - dudy * (zeta + dudy) + dvdy * dwdz - dwdy * (dwdy - xi) + dwdz * dudx -
                         dwdx * (dwdx + eta));
    }
}
template <typename T> void op_pressure_rhs(const Dims &d, cudaStream_t st, const T *g5, const T *vor, T *out)
{
    k_pressure_rhs<T><<<col_grid(d), COL_BLOCK, 0, st>>>(d, g5, vor, out);
}
// f *= tab (a field-shaped table, e.g. the Green function)
template <typename T>
__global__ void k_mul_field(Dims d, const T *__restrict__ tab, T *__restrict__ f)
{
    COLUMN_HEADER
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) f[o + iz] = tab[o + iz] * f[o + iz];
}
template <typename T> void op_mul_field(const Dims &d, cudaStream_t st, const T *tab, T *f)
{
    k_mul_field<T><<<col_grid(d), COL_BLOCK, 0, st>>>(d, tab, f);
}
// du/dx + dv/dy in spectral space (diffx, diffy of sta3dfft.f90:304-377)
template <typename T>
__global__ void k_hdiv(Dims d, Deriv D, const T *__restrict__ svel, T *__restrict__ out)
{
    COLUMN_HEADER
    PARTNERS
    const long long N = d.nfield;
    const T cx = (T)cxk, cy = (T)cyk;
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) out[o + iz] = cx * svel[ox + iz] + cy * svel[N + oy + iz];
}
template <typename T> void op_hdiv(const Dims &d, cudaStream_t st, const Deriv &D, const T *svel, T *out)
{
    k_hdiv<T><<<col_grid(d), COL_BLOCK, 0, st>>>(d, D, svel, out);
}
template void op_pressure_rhs<float>(const Dims &, cudaStream_t, const float *, const float *, float *);
template void op_pressure_rhs<double>(const Dims &, cudaStream_t, const double *, const double *, double *);
template void op_mul_field<float>(const Dims &, cudaStream_t, const float *, float *);
template void op_mul_field<double>(const Dims &, cudaStream_t, const double *, double *);
template void op_hdiv<float>(const Dims &, cudaStream_t, const Deriv &, const float *, float *);
template void op_hdiv<double>(const Dims &, cudaStream_t, const Deriv &, const double *, double *);

// Kinetic-energy shell binning (genspec.f90:67-99): for every spectral
// element, |K| = nint(sqrt(rkx^2 + rky^2 + rkz^2)), shell int(|K| / dk)
// (clamped to kmax), sum of u^2 + v^2 + w^2 and a count per shell; block
// histograms in shared memory, then global atomics.
template <typename T>
__global__ void k_spec_bins(Dims d, const double *__restrict__ rkx, const double *__restrict__ rky,
                            const double *__restrict__ rkz, const T *__restrict__ f, double dki, int kmax,
                            double *__restrict__ bins, unsigned long long *__restrict__ cnt)
{
    extern __shared__ double shb[];
    unsigned long long *shc = reinterpret_cast<unsigned long long *>(shb + kmax + 1);
    const int tid = threadIdx.y * 32 + threadIdx.x;
    for (int b = tid; b <= kmax; b += 32 * COLS_PER_BLOCK) {
        shb[b] = 0.0;
        shc[b] = 0ull;
    }
    __syncthreads();
    const long long N = d.nfield;
    const long long col = (long long)blockIdx.x * COLS_PER_BLOCK + threadIdx.y;
    if (col < d.ncol) {
        const int kx = (int)(col / d.ny), ky = (int)(col - (long long)kx * d.ny);
        const long long o = col * d.P;
        const double h2 = rkx[kx] * rkx[kx] + rky[ky] * rky[ky];
        for (int iz = threadIdx.x; iz <= d.nz; iz += 32) {
            const int km = (int)llround(sqrt(h2 + rkz[iz] * rkz[iz]));
            int b = (int)((double)km * dki);
            b = b > kmax ? kmax : b;
            const double u = (double)f[o + iz], v = (double)f[N + o + iz], w = (double)f[2 * N + o + iz];
            atomicAdd(&shb[b], u * u + v * v + w * w);
            atomicAdd(&shc[b], 1ull);
        }
    }
    __syncthreads();
    for (int b = tid; b <= kmax; b += 32 * COLS_PER_BLOCK) {
        if (shc[b]) {
            atomicAdd(&bins[b], shb[b]);
            atomicAdd(&cnt[b], shc[b]);
        }
    }
}
template <typename T>
void op_spec_bins(const Dims &d, cudaStream_t st, const double *rkx, const double *rky, const double *rkz,
                  const T *f, double dki, int kmax, double *bins, unsigned long long *cnt)
{
    const size_t sm = (size_t)(kmax + 1) * (sizeof(double) + sizeof(unsigned long long));
    k_spec_bins<T><<<col_grid(d), COL_BLOCK, sm, st>>>(d, rkx, rky, rkz, f, dki, kmax, bins, cnt);
}
template void op_spec_bins<float>(const Dims &, cudaStream_t, const double *, const double *, const double *,
                                  const float *, double, int, double *, unsigned long long *);
template void op_spec_bins<double>(const Dims &, cudaStream_t, const double *, const double *, const double *,
                                   const double *, double, int, double *, unsigned long long *);

// flat conversions / accumulation over n elements
template <typename T, typename S>
__global__ void k_convert(const S *__restrict__ in, T *__restrict__ out, long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (T)in[i];
}
template <typename T, typename S>
void op_convert(const Dims &, cudaStream_t st, const S *in, T *out, long long n)
{
    k_convert<T, S><<<1216, 256, 0, st>>>(in, out, n);
}
template <typename T, typename S>
__global__ void k_add(S *__restrict__ acc, const T *__restrict__ add, long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        acc[i] = (S)((double)acc[i] + (double)add[i]);
}
template <typename T, typename S>
void op_add(const Dims &, cudaStream_t st, S *acc, const T *add, long long n)
{
    k_add<T, S><<<1216, 256, 0, st>>>(acc, add, n);
}

// ----------------------------------------------------------------- steppers
// The reference wraps every column scaling of the steppers in
// field_combine_semi_spectral ... field_decompose_semi_spectral
// (impl_rk4.f90:232-238, 264-280, 307-323, 346-362; cn2.f90:110-116,
// 128-134, 166-172).  Both are linear per column and the factors depend on
// (ky, kx) only, so the sandwich equals the bare column scaling; it is
// applied directly here (identical up to rounding).

// integrating factors (impl_rk4.f90:87-89, 151, 185)
__global__ void k_rk4_factors(long long ncol, const double *__restrict__ vdiss, const double *__restrict__ filt0,
                              double *epq, double *emq, double *epq2, double *emq2)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncol) return;
    const double e = exp(vdiss[c]);
    const double m = 1.0 / e;
    const double p = e * filt0[c];
    epq[c] = p;
    emq[c] = m;
    epq2[c] = p * p;
    emq2[c] = m * m;
}
void op_rk4_factors(const Dims &d, cudaStream_t st, const double *vdiss, const double *filt0, double *epq,
                    double *emq, double *epq2, double *emq2)
{
    k_rk4_factors<<<(unsigned)((d.ncol + 255) / 256), 256, 0, st>>>(d.ncol, vdiss, filt0, epq, emq, epq2, emq2);
}

// substep 1 (impl_rk4.f90:212-242)
template <typename T>
__global__ void k_rk4_sub1(Dims d, double *__restrict__ q, double *__restrict__ qdi, double *__restrict__ qdf,
                           T *__restrict__ sqs, const double *__restrict__ filt0, const double *__restrict__ emq,
                           double dt2, double dt6)
{
    COLUMN_HEADER
    const double f0 = filt0[col], m = emq[col];
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) {
        const long long i = o + iz;
        const double s = f0 * (double)sqs[i];
        const double q0 = q[i];
        sqs[i] = (T)s;
        qdi[i] = q0;
        q[i] = (q0 + dt2 * s) * m;
        qdf[i] = q0 + dt6 * s;
    }
}
template <typename T>
void op_rk4_sub1(const Dims &d, cudaStream_t st, double *q, double *qdi, double *qdf, T *sqs,
                 const double *filt0, const double *emq, double dt2, double dt6)
{
    k_rk4_sub1<T><<<col_grid(d), COL_BLOCK, 0, st>>>(d, q, qdi, qdf, sqs, filt0, emq, dt2, dt6);
}

// substeps 2 and 3 (impl_rk4.f90:247-326): c1 = dt/2 or dt
template <typename T>
__global__ void k_rk4_sub23(Dims d, double *__restrict__ q, const double *__restrict__ qdi,
                            double *__restrict__ qdf, const T *__restrict__ sqs, const double *__restrict__ epq,
                            const double *__restrict__ emq, double c1, double dt3)
{
    COLUMN_HEADER
    const double pp = epq[col], m = emq[col];
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) {
        const long long i = o + iz;
        const double s = pp * (double)sqs[i];
        q[i] = (qdi[i] + c1 * s) * m;
        qdf[i] = qdf[i] + dt3 * s;
    }
}
template <typename T>
void op_rk4_sub23(const Dims &d, cudaStream_t st, double *q, const double *qdi, double *qdf, const T *sqs,
                  const double *epq, const double *emq, double c1, double dt3)
{
    k_rk4_sub23<T><<<col_grid(d), COL_BLOCK, 0, st>>>(d, q, qdi, qdf, sqs, epq, emq, c1, dt3);
}

// substep 4 (impl_rk4.f90:331-364)
template <typename T>
__global__ void k_rk4_sub4(Dims d, double *__restrict__ q, const double *__restrict__ qdf,
                           const T *__restrict__ sqs, const double *__restrict__ epq,
                           const double *__restrict__ emq, double dt6)
{
    COLUMN_HEADER
    const double pp = epq[col], m = emq[col];
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) {
        const long long i = o + iz;
        q[i] = (qdf[i] + dt6 * (pp * (double)sqs[i])) * m;
    }
}
template <typename T>
void op_rk4_sub4(const Dims &d, cudaStream_t st, double *q, const double *qdf, const T *sqs,
                 const double *epq, const double *emq, double dt6)
{
    k_rk4_sub4<T><<<col_grid(d), COL_BLOCK, 0, st>>>(d, q, qdf, sqs, epq, emq, dt6);
}

// Mixed form: the increment (c1 * epq * sqs, an FP32 source term scaled by
// per-column factors) is formed in FP32 and widened exactly; the state keeps
// its FP64 accumulation with one fused multiply-add (q = qdi*m + inc) per
// element, and the FP32 copy of the new state that the next vor2vel reads is
// written alongside.  The reference's FP64 accumulator qdf = qdi + d is kept
// as its FP32 part d = dt/6 s1 + dt/3 s2 + dt/3 s3 alone (a source-sized
// term, of order dt |s| against the state), and the last substep forms
// qdf m + c s4 = qdi m + (d m + c s4).  The filtered stage-1 source is not
// written back: the next source evaluation overwrites it.
__global__ void k_rk4m_sub1(Dims d, double *__restrict__ q, double *__restrict__ qdi, float *__restrict__ acc,
                            const float *__restrict__ sqs, float *__restrict__ q32, const double *__restrict__ filt0,
                            const double *__restrict__ emq, const double *__restrict__ dtp)
{
    COLUMN_HEADER
    const double dt = *dtp, dt2 = 0.5 * dt, dt6 = dt / 6.0;
    const double m = emq[col];
    const float f0 = (float)filt0[col];
    const float c2 = (float)(dt2 * m), c6 = (float)dt6;
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) {
        const long long i = o + iz;
        const float s = f0 * sqs[i];
        const double q0 = q[i];
        qdi[i] = q0;
        const double qn = fma(q0, m, widen64(c2 * s));
        q[i] = qn;
        q32[i] = narrow32(qn);
        acc[i] = c6 * s;
    }
}
__global__ void k_rk4m_sub23(Dims d, double *__restrict__ q, const double *__restrict__ qdi,
                             float *__restrict__ acc, const float *__restrict__ sqs, float *__restrict__ q32,
                             const double *__restrict__ epq, const double *__restrict__ emq,
                             const double *__restrict__ dtp, int full)
{
    COLUMN_HEADER
    const double dt = *dtp, c1 = full ? dt : 0.5 * dt, dt3 = dt / 3.0;
    const double m = emq[col];
    const float pp = (float)epq[col];
    const float cq = (float)(c1 * m), c3 = (float)dt3;
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) {
        const long long i = o + iz;
        const float s = pp * sqs[i];
        const double qn = fma(qdi[i], m, widen64(cq * s));
        q[i] = qn;
        q32[i] = narrow32(qn);
        acc[i] = fmaf(c3, s, acc[i]);
    }
}
__global__ void k_rk4m_sub4(Dims d, double *__restrict__ q, const double *__restrict__ qdi,
                            const float *__restrict__ acc, const float *__restrict__ sqs, float *__restrict__ q32,
                            const double *__restrict__ epq, const double *__restrict__ emq,
                            const double *__restrict__ dtp)
{
    COLUMN_HEADER
    const double dt6 = *dtp / 6.0;
    const double m = emq[col];
    const float mf = (float)m, c = (float)(dt6 * epq[col] * m);
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) {
        const long long i = o + iz;
        const double qn = fma(qdi[i], m, widen64(fmaf(acc[i], mf, c * sqs[i])));
        q[i] = qn;
        q32[i] = narrow32(qn);
    }
}
void op_rk4m_sub1(const Dims &d, cudaStream_t st, double *q, double *qdi, float *acc, const float *sqs, float *q32,
                  const double *filt0, const double *emq, const double *dtp)
{
    k_rk4m_sub1<<<col_grid(d), COL_BLOCK, 0, st>>>(d, q, qdi, acc, sqs, q32, filt0, emq, dtp);
}
void op_rk4m_sub23(const Dims &d, cudaStream_t st, double *q, const double *qdi, float *acc, const float *sqs,
                   float *q32, const double *epq, const double *emq, const double *dtp, bool full)
{
    k_rk4m_sub23<<<col_grid(d), COL_BLOCK, 0, st>>>(d, q, qdi, acc, sqs, q32, epq, emq, dtp, full ? 1 : 0);
}
void op_rk4m_sub4(const Dims &d, cudaStream_t st, double *q, const double *qdi, const float *acc, const float *sqs,
                  float *q32, const double *epq, const double *emq, const double *dtp)
{
    k_rk4m_sub4<<<col_grid(d), COL_BLOCK, 0, st>>>(d, q, qdi, acc, sqs, q32, epq, emq, dtp);
}

// ------------------------------------------------ fused stage update (mixed)
// The solenoidal projection of the tendency, the horizontal filter and one
// integrating-factor substep of impl_rk4.f90:212-364 in one pass over the
// tendency.  The projection is vor2vel's (inversion.f90:34-76) applied to
// svorts:
//   ds = D_x S2 - D_y S1,  S1 <- k2l2i (D_x es + D_y ds),
//   S2 <- k2l2i (D_y es - D_x ds),  S3 unchanged,  (0,0) column kept,
// es = decompose(diffz(S3)) from the source.  The projection is linear and
// commutes with the per-column factors, so projecting each source term keeps
// the state on the reference's projected trajectory.  One warp per partner
// orbit (as k_v2v_orbit): the four columns (kx, ky), (nx-kx, ky), (kx, ny-ky),
// (nx-kx, ny-ky) read only one another, so ds never leaves registers.
//
// State traffic: the FP64 state q is the step's initial state (qdi of the
// reference) throughout substeps 1-3 and is not rewritten until substep 4.
// Each substep writes the FP32 copy q32 of its stage state (what the next
// vor2vel reads) and the FP32 source accumulator acc (the reference's qdf
// minus qdi, see k_rk4m_sub1); the stage state of the (0,0) column also goes
// to mf in FP64 (components 1 and 2, pitch P) for the mean-flow inversion of
// the next vor2vel.  Substep 4 writes q.  Per element and substep, the same
// FP32 increments and FP64 fused multiply-adds as k_rk4m_sub1/23/4.
//   SUB 1: factors filt0, emq;           s = f s,  q' = q m + (dt/2 m) s,  acc  = dt/6 s
//   SUB 2: factors epq, emq,  c1 = dt/2: s = p s,  q' = q m + (c1 m) s,    acc += dt/3 s
//   SUB 3: factors epq, emq2, c1 = dt:   (as SUB 2)
//   SUB 4: factors epq2, emq2:           q' = q m + (acc m + (dt/6 p m) s)
template <int SUB> struct StageCol {
    double m;
    float a, b, c;
    __device__ __forceinline__ void make(double dt, const double *fp, const double *fm, long long col)
    {
        m = fm[col];
        if (SUB == 1) {
            a = (float)fp[col];
            b = (float)(0.5 * dt * m);
            c = (float)(dt / 6.0);
        } else if (SUB == 4) {
            a = (float)m;
            b = (float)(dt / 6.0 * fp[col] * m);
        } else {
            a = (float)fp[col];
            b = (float)((SUB == 3 ? dt : 0.5 * dt) * m);
            c = (float)(dt / 3.0);
        }
    }
    // one element: s the projected source, q0 the step's initial state
    __device__ __forceinline__ double apply(float s, double q0, float &acc) const
    {
        if (SUB == 4) return fma(q0, m, widen64(fmaf(acc, a, b * s)));
        const float fs = a * s;
        const double qn = fma(q0, m, widen64(b * fs));
        acc = (SUB == 1) ? c * fs : fmaf(c, fs, acc);
        return qn;
    }
};

// One block of four warps per partner orbit, warp w on member (x partner if
// w & 1, y partner if w & 2) over 32 levels at a time: the members' S1, S2,
// es and then ds meet in shared memory (two buffers, alternating), so each
// value is read from HBM once and every warp keeps only its own column in
// registers.  All global loads of the next 32 levels are issued before the
// current levels' barriers.
template <int SUB> struct StageLoads {
    float a, b, e, s3, acc[3];
    double q[3];
};

template <int SUB>
__device__ __forceinline__ void stage_load(StageLoads<SUB> &v, bool on, long long N, long long i,
                                           const float *__restrict__ S, const float *__restrict__ es,
                                           const double *__restrict__ q, const float *__restrict__ acc)
{
    v.a = on ? S[i] : 0.f;
    v.b = on ? S[N + i] : 0.f;
    v.e = on ? es[i] : 0.f;
    v.s3 = on ? S[2 * N + i] : 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        v.q[k] = on ? q[(long long)k * N + i] : 0.0;
        v.acc[k] = (on && SUB != 1) ? acc[(long long)k * N + i] : 0.f;
    }
}

struct StageShared {
    float a[2][4][32], b[2][4][32], e[2][4][32], d[2][4][32];
};

// the stage update of partner orbit orb by the block's 128 threads
template <int SUB>
__device__ __forceinline__ void stage_orbit(const Dims &d, const Deriv &D, const double *__restrict__ k2l2i,
                                            const float *__restrict__ S, const float *__restrict__ es,
                                            double *__restrict__ q, float *__restrict__ acc,
                                            float *__restrict__ q32, double *__restrict__ mf,
                                            const double *__restrict__ fp, const double *__restrict__ fm,
                                            double dt, long long orb, StageShared &sh)
{
    auto &sh_a = sh.a;
    auto &sh_b = sh.b;
    auto &sh_e = sh.e;
    auto &sh_d = sh.d;
    const int hy = d.ny / 2 + 1;
    const long long N = d.nfield;
    const int kx = (int)(orb / hy), ky = (int)(orb - (long long)kx * hy);
    const int x2 = xsrc(kx, d.nx), y2 = xsrc(ky, d.ny);
    const bool dx = x2 != kx, dy = y2 != ky;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool active = (!(w & 1) || dx) && (!(w & 2) || dy);
    const int mx = (w & 1) ? x2 : kx, my = (w & 2) ? y2 : ky;
    const int xw = dx ? (w ^ 1) : w, yw = dy ? (w ^ 2) : w;  // partner members
    const long long col = (long long)my + (long long)d.ny * mx, o = col * d.P;
    const bool mean = col == 0;  // the (0,0) column keeps its mean vorticity
    const float cx = (float)D.cx[mx], cy = (float)D.cy[my], kk = (float)k2l2i[col];
    StageCol<SUB> f;
    f.make(dt, fp, fm, col);
    StageLoads<SUB> cur, nxt;
    stage_load<SUB>(cur, active && lane <= d.nz, N, o + lane, S, es, q, acc);
    int buf = 0;
    for (int z0 = 0; z0 <= d.nz; z0 += 32, buf ^= 1) {
        const int iz = z0 + lane;
        const bool on = active && iz <= d.nz;
        sh_a[buf][w][lane] = cur.a;
        sh_b[buf][w][lane] = cur.b;
        sh_e[buf][w][lane] = cur.e;
        if (z0 + 32 <= d.nz) stage_load<SUB>(nxt, active && iz + 32 <= d.nz, N, o + iz + 32, S, es, q, acc);
        __syncthreads();
        // ds = D_x S2 - D_y S1 (k_v2v_ds)
        sh_d[buf][w][lane] = cx * sh_b[buf][xw][lane] - cy * sh_a[buf][yw][lane];
        __syncthreads();
        // projected S1, S2 (k_v2v_orbit with e = es, f = ds)
        const float p1 = mean ? cur.a : kk * (cx * sh_e[buf][xw][lane] + cy * sh_d[buf][yw][lane]);
        const float p2 = mean ? cur.b : kk * (cy * sh_e[buf][yw][lane] - cx * sh_d[buf][xw][lane]);
        if (on) {
            const float sv[3] = {p1, p2, cur.s3};
            const long long i = o + iz;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const long long ik = (long long)k * N + i;
                float a = cur.acc[k];
                const double qn = f.apply(sv[k], cur.q[k], a);
                if (SUB == 4) q[ik] = qn;
                else acc[ik] = a;
                q32[ik] = narrow32(qn);
                if (mean && k < 2) mf[(long long)k * d.P + iz] = qn;
            }
        }
        cur = nxt;
    }
}


template <int SUB>
__global__ void __launch_bounds__(128) k_stage_orbit(Dims d, Deriv D, const double *__restrict__ k2l2i,
                                                     const float *__restrict__ S, const float *__restrict__ es,
                                                     double *__restrict__ q, float *__restrict__ acc,
                                                     float *__restrict__ q32, double *__restrict__ mf,
                                                     const double *__restrict__ fp, const double *__restrict__ fm,
                                                     const double *__restrict__ dtp)
{
    __shared__ StageShared sh;
    stage_orbit<SUB>(d, D, k2l2i, S, es, q, acc, q32, mf, fp, fm, *dtp, blockIdx.x, sh);
}

// The stage update of every run of a batch in one persistent launch: the
// work items are (run, partner orbit), numbered run by run (item0), and the
// blocks take items item b, b + gridDim.x, ...; each item is the same
// computation as the single-run kernel above, so a batch and the runs
// stepped alone agree bitwise.
template <int SUB>
__global__ void __launch_bounds__(128) k_batch_stage(const StageRun *__restrict__ runs, int nruns, long long nitems)
{
    __shared__ StageShared sh;
    for (long long it = blockIdx.x; it < nitems; it += gridDim.x) {
        int lo = 0, hi = nruns - 1;  // the run whose items contain it
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (runs[mid].item0 <= it) lo = mid;
            else hi = mid - 1;
        }
        const StageRun &r = runs[lo];
        stage_orbit<SUB>(r.d, r.D, r.k2l2i, r.S, r.es, r.q, r.acc, r.q32, r.mf, r.fp[SUB - 1], r.fm[SUB - 1],
                         *r.dtp, it - r.item0, sh);
        __syncthreads();
    }
}

int batch_stage_blocks()
{
    int dev = 0, sms = 1, per = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_stage<2>, 128, 0);
    return sms * (per > 0 ? per : 1);
}

void op_batch_stage(cudaStream_t st, int sub, const StageRun *runs, int nruns, long long nitems, int blocks)
{
    switch (sub) {
    case 1: k_batch_stage<1><<<blocks, 128, 0, st>>>(runs, nruns, nitems); break;
    case 2: k_batch_stage<2><<<blocks, 128, 0, st>>>(runs, nruns, nitems); break;
    case 3: k_batch_stage<3><<<blocks, 128, 0, st>>>(runs, nruns, nitems); break;
    default: k_batch_stage<4><<<blocks, 128, 0, st>>>(runs, nruns, nitems); break;
    }
}

void op_stage_orbit(const Dims &d, cudaStream_t st, int sub, const Deriv &D, const double *k2l2i, const float *S,
                    const float *es, double *q, float *acc, float *q32, double *mf, const double *fp,
                    const double *fm, const double *dtp)
{
    const dim3 g((unsigned)((long long)(d.nx / 2 + 1) * (d.ny / 2 + 1)));
    switch (sub) {
    case 1: k_stage_orbit<1><<<g, 128, 0, st>>>(d, D, k2l2i, S, es, q, acc, q32, mf, fp, fm, dtp); break;
    case 2: k_stage_orbit<2><<<g, 128, 0, st>>>(d, D, k2l2i, S, es, q, acc, q32, mf, fp, fm, dtp); break;
    case 3: k_stage_orbit<3><<<g, 128, 0, st>>>(d, D, k2l2i, S, es, q, acc, q32, mf, fp, fm, dtp); break;
    default: k_stage_orbit<4><<<g, 128, 0, st>>>(d, D, k2l2i, S, es, q, acc, q32, mf, fp, fm, dtp); break;
    }
}

// Host-layout state (nz+1 values per column, the three components one after
// another) <-> the device's P-pitched columns, FP64.  The unpack raises
// *changed when any element differs bitwise from the device state it
// overwrites.
//
// The host side of these copies is page-locked memory read or written over
// the host link (zero copy), where the link, not HBM, sets the pace.  A
// block takes FLAT_COLS consecutive columns, one contiguous run of
// FLAT_COLS * (nz+1) doubles on the host (16-byte aligned when the host
// array is, FLAT_COLS being even), and moves it as 16-byte pairs, each
// thread holding FLAT_U pairs in flight; the device side scatters each pair
// to its one or two columns.  The per-column kernels (8-byte accesses) serve
// host arrays that are not 16-byte aligned.
constexpr int FLAT_COLS = 8, FLAT_U = 4, FLAT_T = 256;

// (column, level) of element e of a chunk of columns of n1 levels; e <
// FLAT_COLS * n1 < 2^24, where e + 0.5 is never within 1/(2 n1) of a
// multiple of n1, so the single-precision quotient truncates correctly
__device__ __forceinline__ void chunk_pos(int e, int n1, float inv_n1, int &col, int &iz)
{
    col = (int)(((float)e + 0.5f) * inv_n1);
    iz = e - col * n1;
}

__global__ void __launch_bounds__(FLAT_T) k_unpack_flat(Dims d, const double2 *__restrict__ src,
                                                        double *__restrict__ dst, long long ncols, float inv_n1,
                                                        int *__restrict__ changed)
{
    const int n1 = d.nz + 1;
    const long long c0 = (long long)blockIdx.x * FLAT_COLS;
    const int ne = (int)min((long long)FLAT_COLS, ncols - c0) * n1;  // elements of this chunk
    const double2 *s = src + ((c0 * n1) >> 1);                         // c0 even: whole pairs
    double *t = dst + c0 * d.P;
    bool diff = false;
    for (int q0 = threadIdx.x; 2 * q0 < ne; q0 += FLAT_T * FLAT_U) {
        double2 v[FLAT_U];
#pragma unroll
        for (int u = 0; u < FLAT_U; ++u) {
            const int q = q0 + FLAT_T * u;
            if (2 * q + 1 < ne) v[u] = s[q];
            else if (2 * q < ne) v[u].x = reinterpret_cast<const double *>(s)[2 * q];  // odd tail
        }
#pragma unroll
        for (int u = 0; u < FLAT_U; ++u) {
            const int e = 2 * (q0 + FLAT_T * u);
            if (e < ne) {
                int col, iz;
                chunk_pos(e, n1, inv_n1, col, iz);
                double *p0 = t + (long long)col * d.P + iz;
                diff |= __double_as_longlong(v[u].x) != __double_as_longlong(*p0);
                *p0 = v[u].x;
                if (e + 1 < ne) {
                    if (++iz == n1) {
                        iz = 0;
                        ++col;
                    }
                    double *p1 = t + (long long)col * d.P + iz;
                    diff |= __double_as_longlong(v[u].y) != __double_as_longlong(*p1);
                    *p1 = v[u].y;
                }
            }
        }
    }
    if (__any_sync(0xffffffffu, diff) && (threadIdx.x & 31) == 0) atomicOr(changed, 1);
}

__global__ void __launch_bounds__(FLAT_T) k_pack_flat(Dims d, const double *__restrict__ src,
                                                      double2 *__restrict__ dst, long long ncols, float inv_n1)
{
    const int n1 = d.nz + 1;
    const long long c0 = (long long)blockIdx.x * FLAT_COLS;
    const int ne = (int)min((long long)FLAT_COLS, ncols - c0) * n1;
    double2 *t = dst + ((c0 * n1) >> 1);
    const double *s = src + c0 * d.P;
    for (int q0 = threadIdx.x; 2 * q0 < ne; q0 += FLAT_T * FLAT_U) {
        double2 v[FLAT_U];
#pragma unroll
        for (int u = 0; u < FLAT_U; ++u) {
            const int e = 2 * (q0 + FLAT_T * u);
            if (e < ne) {
                int col, iz;
                chunk_pos(e, n1, inv_n1, col, iz);
                v[u].x = s[(long long)col * d.P + iz];
                if (e + 1 < ne) {
                    if (++iz == n1) {
                        iz = 0;
                        ++col;
                    }
                    v[u].y = s[(long long)col * d.P + iz];
                }
            }
        }
#pragma unroll
        for (int u = 0; u < FLAT_U; ++u) {
            const int e = 2 * (q0 + FLAT_T * u);
            if (e + 1 < ne) t[e >> 1] = v[u];
            else if (e < ne) reinterpret_cast<double *>(t)[e] = v[u].x;  // odd tail
        }
    }
}

// The same copy for a state check that runs beside the step on a second
// stream: the host state goes into a staging array (device layout) and is
// compared bitwise with the state it would replace (cmp), which the step
// reads meanwhile and nobody writes.  A small persistent grid, CHECK_U pairs
// in flight per thread, keeps the host link busy while leaving the SMs to
// the step's kernels.
constexpr int CHECK_BLOCKS = 48, CHECK_U = 8;
__global__ void __launch_bounds__(FLAT_T) k_unpack_check(Dims d, const double2 *__restrict__ src,
                                                         const double *__restrict__ cmp, double *__restrict__ dst,
                                                         long long ncols, float inv_n1, int *__restrict__ changed)
{
    const int n1 = d.nz + 1;
    const long long nchunks = (ncols + FLAT_COLS - 1) / FLAT_COLS;
    bool diff = false;
    for (long long ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const long long c0 = ch * FLAT_COLS;
        const int ne = (int)min((long long)FLAT_COLS, ncols - c0) * n1;
        const double2 *s = src + ((c0 * n1) >> 1);
        const long long tb = c0 * d.P;
        for (int q0 = threadIdx.x; 2 * q0 < ne; q0 += FLAT_T * CHECK_U) {
            double2 v[CHECK_U];
#pragma unroll
            for (int u = 0; u < CHECK_U; ++u) {
                const int q = q0 + FLAT_T * u;
                if (2 * q + 1 < ne) v[u] = s[q];
                else if (2 * q < ne) v[u].x = reinterpret_cast<const double *>(s)[2 * q];  // odd tail
            }
#pragma unroll
            for (int u = 0; u < CHECK_U; ++u) {
                const int e = 2 * (q0 + FLAT_T * u);
                if (e < ne) {
                    int col, iz;
                    chunk_pos(e, n1, inv_n1, col, iz);
                    long long o = tb + (long long)col * d.P + iz;
                    diff |= __double_as_longlong(v[u].x) != __double_as_longlong(cmp[o]);
                    dst[o] = v[u].x;
                    if (e + 1 < ne) {
                        if (++iz == n1) {
                            iz = 0;
                            ++col;
                        }
                        o = tb + (long long)col * d.P + iz;
                        diff |= __double_as_longlong(v[u].y) != __double_as_longlong(cmp[o]);
                        dst[o] = v[u].y;
                    }
                }
            }
        }
    }
    if (__any_sync(0xffffffffu, diff) && (threadIdx.x & 31) == 0) atomicOr(changed, 1);
}

__global__ void k_unpack_cols(Dims d, const double *__restrict__ src, double *__restrict__ dst, long long ncols,
                              int *__restrict__ changed)
{
    const long long c = (long long)blockIdx.x * COLS_PER_BLOCK + threadIdx.y;
    if (c >= ncols) return;
    const int n1 = d.nz + 1;
    const double *s = src + c * n1;
    double *t = dst + c * d.P;
    bool diff = false;
    for (int iz = threadIdx.x; iz < n1; iz += 32) {
        const double v = s[iz];
        diff |= __double_as_longlong(v) != __double_as_longlong(t[iz]);
        t[iz] = v;
    }
    if (__any_sync(0xffffffffu, diff) && threadIdx.x == 0) atomicOr(changed, 1);
}
__global__ void k_pack_cols(Dims d, const double *__restrict__ src, double *__restrict__ dst, long long ncols)
{
    const long long c = (long long)blockIdx.x * COLS_PER_BLOCK + threadIdx.y;
    if (c >= ncols) return;
    const int n1 = d.nz + 1;
    const double *s = src + c * d.P;
    double *t = dst + c * n1;
    for (int iz = threadIdx.x; iz < n1; iz += 32) t[iz] = s[iz];
}

static bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

void op_unpack_cols(const Dims &d, cudaStream_t st, const double *src, double *dst, int ncomp, int *changed)
{
    const long long ncols = (long long)ncomp * d.ncol;
    if (aligned16(src)) {
        k_unpack_flat<<<(unsigned)((ncols + FLAT_COLS - 1) / FLAT_COLS), FLAT_T, 0, st>>>(
            d, reinterpret_cast<const double2 *>(src), dst, ncols, 1.0f / (float)(d.nz + 1), changed);
        return;
    }
    k_unpack_cols<<<(unsigned)((ncols + COLS_PER_BLOCK - 1) / COLS_PER_BLOCK), COL_BLOCK, 0, st>>>(d, src, dst,
                                                                                                   ncols, changed);
}
bool op_unpack_check(const Dims &d, cudaStream_t st, const double *src, const double *cmp, double *dst, int ncomp,
                     int *changed)
{
    if (!aligned16(src)) return false;
    const long long ncols = (long long)ncomp * d.ncol;
    const long long nchunks = (ncols + FLAT_COLS - 1) / FLAT_COLS;
    k_unpack_check<<<(unsigned)(nchunks < CHECK_BLOCKS ? nchunks : CHECK_BLOCKS), FLAT_T, 0, st>>>(
        d, reinterpret_cast<const double2 *>(src), cmp, dst, ncols, 1.0f / (float)(d.nz + 1), changed);
    return true;
}
void op_pack_cols(const Dims &d, cudaStream_t st, const double *src, double *dst, int ncomp)
{
    const long long ncols = (long long)ncomp * d.ncol;
    if (aligned16(dst)) {
        k_pack_flat<<<(unsigned)((ncols + FLAT_COLS - 1) / FLAT_COLS), FLAT_T, 0, st>>>(
            d, src, reinterpret_cast<double2 *>(dst), ncols, 1.0f / (float)(d.nz + 1));
        return;
    }
    k_pack_cols<<<(unsigned)((ncols + COLS_PER_BLOCK - 1) / COLS_PER_BLOCK), COL_BLOCK, 0, st>>>(d, src, dst,
                                                                                                 ncols);
}

// FP32 copy of an FP64 field (integer narrowing)
__global__ void k_narrow(const double *__restrict__ in, float *__restrict__ out, long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = narrow32(in[i]);
}
void op_narrow(cudaStream_t st, const double *in, float *out, long long n)
{
    k_narrow<<<2432, 256, 0, st>>>(in, out, n);
}

// cn2 (cn2.f90:119-175)
template <typename T>
__global__ void k_cn2_init(Dims d, double *__restrict__ vortsm, const double *__restrict__ svor,
                           const T *__restrict__ svorts, double dt2)
{
    COLUMN_HEADER
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) vortsm[o + iz] = svor[o + iz] + dt2 * (double)svorts[o + iz];
}
template <typename T>
void op_cn2_init(const Dims &d, cudaStream_t st, double *vortsm, const double *svor, const T *svorts, double dt2,
                 int ncomp)
{
    for (int c = 0; c < ncomp; ++c)
        k_cn2_init<T><<<col_grid(d), COL_BLOCK, 0, st>>>(d, vortsm + c * d.nfield, svor + c * d.nfield,
                                                         svorts + c * d.nfield, dt2);
}
template <typename T>
__global__ void k_cn2_update(Dims d, double *__restrict__ svor, const double *__restrict__ vortsm,
                             const T *__restrict__ svorts, const double *__restrict__ filt0,
                             const double *__restrict__ fz, const double *__restrict__ vdiss, double dt2)
{
    COLUMN_HEADER
    const double f0 = filt0[col], vd = vdiss[col];
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) {
        const long long i = o + iz;
        double f = f0;
        if (col == 0) f = 1.0;
        else if (iz > 0 && iz < d.nz) f = f0 * fz[iz];
        svor[i] = f * (vortsm[i] + dt2 * (double)svorts[i]) * vd;
    }
}
template <typename T>
void op_cn2_update(const Dims &d, cudaStream_t st, double *svor, const double *vortsm, const T *svorts,
                   const double *filt0, const double *fz, const double *vdiss, double dt2, int ncomp)
{
    for (int c = 0; c < ncomp; ++c)
        k_cn2_update<T><<<col_grid(d), COL_BLOCK, 0, st>>>(d, svor + c * d.nfield, vortsm + c * d.nfield,
                                                           svorts + c * d.nfield, filt0, fz, vdiss, dt2);
}

// calc_vorticity_mean / adjust_vorticity_mean (field_diagnostics.f90:584-619).
// The sum of the sine transform of the (0,0) column is the dot product with
// dstsum[j] = sqrt(2/nz) sum_k sin(pi j k / nz).
__global__ void k_mean_fix(int nz, long long nfield, double *svor, const double *__restrict__ dstsum, double fnzi,
                           const double *__restrict__ ini, double *savg_out, int apply, float *svor32)
{
    __shared__ double red[2][256];
    for (int nc = 0; nc < 2; ++nc) {
        const double *s = svor + nc * nfield;
        double acc = 0.0;
        for (int j = 1 + threadIdx.x; j < nz; j += blockDim.x) acc += dstsum[j] * s[j];
        red[nc][threadIdx.x] = acc;
    }
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            red[0][threadIdx.x] += red[0][threadIdx.x + w];
            red[1][threadIdx.x] += red[1][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int nc = 0; nc < 2; ++nc) {
            double *s = svor + nc * nfield;
            const double savg = 0.5 * (s[0] + s[nz]) + fnzi * red[nc][0];
            if (savg_out) savg_out[nc] = savg;
            if (apply) {
                s[0] = s[0] + ini[nc] - savg;
                s[nz] = s[nz] + ini[nc] - savg;
                if (svor32) {
                    svor32[nc * nfield] = narrow32(s[0]);
                    svor32[nc * nfield + nz] = narrow32(s[nz]);
                }
            }
        }
    }
}
void op_mean_fix(const Dims &d, cudaStream_t st, double *svor, const double *dstsum, double fnzi,
                 const double *ini, double *savg_out, int apply, float *svor32)
{
    k_mean_fix<<<1, 256, 0, st>>>(d.nz, d.nfield, svor, dstsum, fnzi, ini, savg_out, apply, svor32);
}

// --------------------------------------------------------------- reductions
// Compensated accumulation per thread (Neumaier in FP64 for the FP64 form;
// Knuth two-sum in FP32 registers for the mixed form, so its error is that
// of an FP64 sum without FP64 arithmetic per element), then an FP64 tree
// across threads and a fixed-order FP64 compensated sum across blocks.
struct KSum {
    double s, c;
    __device__ void add(double v)
    {
        const double t = s + v;
        if (fabs(s) >= fabs(v)) c += (s - t) + v;
        else c += (v - t) + s;
        s = t;
    }
    __device__ double value() const { return s + c; }
};

template <typename T> struct Acc;
template <> struct Acc<double> {
    KSum k{0.0, 0.0};
    __device__ void add(double v) { k.add(v); }
    __device__ double value() const { return k.value(); }
};
template <> struct Acc<float> {
    float s = 0.0f, c = 0.0f;
    __device__ void add(float v)
    {
        const float t = s + v;
        const float bp = t - s;
        const float err = (s - (t - bp)) + (v - bp);
        s = t;
        c += err;
    }
    __device__ double value() const { return (double)s + (double)c; }
};

int red_nblocks(const Dims &d)
{
    long long nb = (d.ncol + COLS_PER_BLOCK - 1) / COLS_PER_BLOCK;
    if (nb > 1216) nb = 1216;
    return (int)nb;
}

// Reduction grid: at most red_nblocks, and no more blocks than fit on the
// device at once (a partial second wave would leave most SMs idle while it
// runs; the kernels stride over the columns)
template <typename K> int red_grid(const Dims &d, K kern)
{
    int dev = 0, sms = 1, per = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, COLS_PER_BLOCK * 32, 0);
    const int cap = sms * (per > 0 ? per : 1);
    const int nb = red_nblocks(d);
    return nb < cap ? nb : cap;
}

// block-level reduce of NV values: kinds[v] = 0 sum, 1 max
template <int NV>
__device__ void block_reduce_store(double (&vals)[NV], const int (&kinds)[NV], double *part)
{
    __shared__ double sh[NV][8];
    const int lane = threadIdx.x, wy = threadIdx.y;  // 32 x 8 block: one warp per row
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        double x = vals[v];
        for (int off = 16; off > 0; off >>= 1) {
            const double y = __shfl_down_sync(0xffffffffu, x, off);
            x = kinds[v] ? fmax(x, y) : x + y;
        }
        if (lane == 0) sh[v][wy] = x;
    }
    __syncthreads();
    if (wy == 0 && lane < NV) {
        double x = sh[lane][0];
        for (int w = 1; w < COLS_PER_BLOCK; ++w) x = kinds[lane] ? fmax(x, sh[lane][w]) : x + sh[lane][w];
        part[(long long)blockIdx.x * NV + lane] = x;
    }
}

template <int NV>
__global__ void k_finish(const double *__restrict__ part, int nblk, const int *kinds_in, double *result)
{
    // single block, one warp per value, fixed order
    const int v = threadIdx.y;
    if (v >= NV) return;
    const int kind = kinds_in[v];
    double x = kind ? -DBL_MAX : 0.0;
    KSum ks{0.0, 0.0};
    for (int b = threadIdx.x; b < nblk; b += 32) {
        const double y = part[(long long)b * NV + v];
        if (kind) x = fmax(x, y);
        else ks.add(y);
    }
    if (!kind) x = ks.value();
    for (int off = 16; off > 0; off >>= 1) {
        const double y = __shfl_down_sync(0xffffffffu, x, off);
        x = kind ? fmax(x, y) : x + y;
    }
    if (threadIdx.x == 0) result[v] = x;
}

__constant__ int c_kinds1[RED1_N] = {1, 0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0};
__constant__ int c_kinds2[RED2_N] = {0, 0, 1, 1, 1};

// pass 1: 0 max|w|^2, 1 sum_w |w|^2, 2 sum_w |u|^2, 3 sum_w u.w, 4..6 sum_w w_c,
// 7..9 max u, v, w (signed)   (advance.f90:171-185, 285-288;
// field_diagnostics.f90:85-206, 405-432, 549-579)
template <typename T>
__global__ void k_red1(Dims d, const T *__restrict__ vel, const T *__restrict__ vor, double *part)
{
    const long long N = d.nfield;
    const T lowest = sizeof(T) == 8 ? (T)-DBL_MAX : (T)-FLT_MAX;
    T vmx[3] = {lowest, lowest, lowest};
    T wmax2 = 0;
    Acc<T> s_w2, s_u2, s_h, s_m0, s_m1, s_m2;
    for (long long col = (long long)blockIdx.x * COLS_PER_BLOCK + threadIdx.y; col < d.ncol;
         col += (long long)gridDim.x * COLS_PER_BLOCK) {
        const long long o = col * d.P;
#pragma unroll 4
        for (int iz = threadIdx.x; iz <= d.nz; iz += 32) {
            const long long i = o + iz;
            const T wt = (iz == 0 || iz == d.nz) ? (T)0.5 : (T)1;
            const T x = vor[i], y = vor[N + i], z = vor[2 * N + i];
            const T u = vel[i], v = vel[N + i], w = vel[2 * N + i];
            const T w2 = x * x + y * y + z * z;
            wmax2 = w2 > wmax2 ? w2 : wmax2;
            s_w2.add(wt * w2);
            s_u2.add(wt * (u * u + v * v + w * w));
            s_h.add(wt * (u * x + v * y + w * z));
            s_m0.add(wt * x);
            s_m1.add(wt * y);
            s_m2.add(wt * z);
            vmx[0] = u > vmx[0] ? u : vmx[0];
            vmx[1] = v > vmx[1] ? v : vmx[1];
            vmx[2] = w > vmx[2] ? w : vmx[2];
        }
    }
    double vals[RED1_N] = {(double)wmax2, s_w2.value(), s_u2.value(), s_h.value(), s_m0.value(), s_m1.value(),
                           s_m2.value(), (double)vmx[0], (double)vmx[1], (double)vmx[2], 0.0, 0.0};
    const int kinds[RED1_N] = {1, 0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0};
    block_reduce_store<RED1_N>(vals, kinds, part);
}

template <typename T>
void red_pass1(const Dims &d, cudaStream_t st, const T *vel, const T *vor, double *part, double *result)
{
    const int nb = red_grid(d, k_red1<T>);
    k_red1<T><<<nb, COL_BLOCK, 0, st>>>(d, vel, vor, part);
    int *kinds;
    cudaGetSymbolAddress((void **)&kinds, c_kinds1);
    k_finish<RED1_N><<<1, dim3(32, RED1_N), 0, st>>>(part, nb, kinds, result);
}

// Rutishauser cyclic Jacobi eigenvalues of a symmetric 3x3 (jacobi.f90),
// upper triangle a01 a02 a12, diagonal d0 d1 d2; returns max |lambda|.
// FP64: the reference's absolute tolerance 1e-15 with a bounded sweep count
// (*hit set if the bound is reached).  FP32 (unused by the mixed form,
// which takes the closed form below): the same rotations stopped at FP32
// resolution after at most 12 sweeps.
template <typename A>
__device__ __forceinline__ void givens_rot(A aij, A di, A dj, A &c, A &s, A &t, A &tau)
{
    const A eps = sizeof(A) == 8 ? (A)DBL_EPSILON : (A)FLT_EPSILON;
    const A g = (A)100 * fabs(aij);
    const A h = dj - di;
    if (fabs(h) + g == fabs(h)) {
        t = aij / (h + copysign(eps, h));
    } else {
        const A theta = (A)0.5 * h / (aij + copysign(eps, aij));
        t = (A)1 / (fabs(theta) + sqrt((A)1 + theta * theta));
        if (theta < (A)0) t = -t;
    }
    c = (A)1 / sqrt((A)1 + t * t);
    s = t * c;
    tau = s / ((A)1 + c);
}

template <typename A>
__device__ A jacobi_maxabs(A a00, A a01, A a02, A a11, A a12, A a22, int *hit)
{
    A Am[3][3] = {{a00, a01, a02}, {0, a11, a12}, {0, 0, a22}};
    A D[3] = {a00, a11, a22}, Bv[3] = {a00, a11, a22}, Z[3] = {0, 0, 0};
    A sm = fabs(Am[0][1]) + fabs(Am[0][2]) + fabs(Am[1][2]);
    const bool f64 = sizeof(A) == 8;
    const int maxsweeps = f64 ? 100 : 12;
    int sweeps = 0;
    while (f64 ? (sm > (A)1.0e-15)
               : (sm > (A)1.0e-7 * (fabs(D[0]) + fabs(D[1]) + fabs(D[2])) && sm > (A)1.0e-30)) {
        if (++sweeps > maxsweeps) {
            if (f64) *hit = 1;
            break;
        }
#pragma unroll
        for (int i = 0; i < 2; ++i) {
#pragma unroll
            for (int j = i + 1; j < 3; ++j) {
                A c, s, t, tau;
                givens_rot<A>(Am[i][j], D[i], D[j], c, s, t, tau);
                A h = t * Am[i][j];
                Z[i] -= h;
                Z[j] += h;
                D[i] -= h;
                D[j] += h;
                Am[i][j] = 0;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    if (k < i) {
                        const A g = Am[k][i], hh = Am[k][j];
                        Am[k][i] = g - s * (hh + g * tau);
                        Am[k][j] = hh + s * (g - hh * tau);
                    } else if (k > i && k < j) {
                        const A g = Am[i][k], hh = Am[k][j];
                        Am[i][k] = g - s * (hh + g * tau);
                        Am[k][j] = hh + s * (g - hh * tau);
                    } else if (k > j) {
                        const A g = Am[i][k], hh = Am[j][k];
                        Am[i][k] = g - s * (hh + g * tau);
                        Am[j][k] = hh + s * (g - hh * tau);
                    }
                }
            }
        }
        for (int k = 0; k < 3; ++k) {
            Bv[k] += Z[k];
            D[k] = Bv[k];
            Z[k] = 0;
        }
        sm = fabs(Am[0][1]) + fabs(Am[0][2]) + fabs(Am[1][2]);
    }
    return fmax(fmax(fabs(D[0]), fabs(D[1])), fabs(D[2]));
}

// Largest |eigenvalue| of a symmetric 3x3 in closed form (FP32 path):
// with m = tr/3 and B = A - m I, the eigenvalues are m + 2 s cos(psi/3 -
// 2 pi k/3), s = sqrt(tr(B^2)/6), cos(psi) = det(B) / (2 s^3) (Smith 1961,
// Commun. ACM 4:168).  The extreme eigenvalues (k = 0, 2) are well
// conditioned in this form, which gives them to a few FP32 rounding units,
// the resolution of the FP32 gradients they come from.
__device__ __forceinline__ float sym3_maxabs(float a00, float a01, float a02, float a11, float a12, float a22)
{
    const float m = (a00 + a11 + a22) * (1.0f / 3.0f);
    const float b00 = a00 - m, b11 = a11 - m, b22 = a22 - m;
    const float p2 = b00 * b00 + b11 * b11 + b22 * b22 + 2.0f * (a01 * a01 + a02 * a02 + a12 * a12);
    if (!(p2 > 0.0f)) return fabsf(m);
    const float s = sqrtf(p2 * (1.0f / 6.0f));
    const float det = b00 * (b11 * b22 - a12 * a12) - a01 * (a01 * b22 - a12 * a02) + a02 * (a01 * a12 - b11 * a02);
    const float r = fminf(fmaxf(det / (2.0f * s * s * s), -1.0f), 1.0f);
    const float th = acosf(r) * (1.0f / 3.0f);
    float sn, cs;
    sincosf(th, &sn, &cs);
    const float lmax = m + 2.0f * s * cs;                                          // k = 0
    const float lmin = m + 2.0f * s * (-0.5f * cs - 0.86602540378443865f * sn);   // k = 2
    return fmaxf(fabsf(lmax), fabsf(lmin));
}

template <typename T> struct StrainMax;
template <> struct StrainMax<double> {
    __device__ static double get(double a00, double a01, double a02, double a11, double a12, double a22, int *hit)
    {
        return jacobi_maxabs<double>(a00, a01, a02, a11, a12, a22, hit);
    }
};
template <> struct StrainMax<float> {
    __device__ static float get(float a00, float a01, float a02, float a11, float a12, float a22, int *)
    {
        return sym3_maxabs(a00, a01, a02, a11, a12, a22);
    }
};

// pass 2: 0 vorl1, 1 vorl2 (characteristic vorticity, field_diagnostics.f90:
// 501-545), 2 ggmax, 3 usggmax, 4 lsggmax (advance.f90:222-276)
template <typename T>
__global__ void k_red2(Dims d, const T *__restrict__ vor, const T *__restrict__ g5, double vortrms,
                       const double *__restrict__ res1, double ncell, double *part, int *flag)
{
    const long long N = d.nfield;
    // the characteristic-vorticity threshold from the pass-1 results when
    // they stay on the device (sqrt(sum w^2 / ncell), as the host computes)
    const T vr = (T)(res1 ? sqrt(res1[1] / ncell) : vortrms);
    Acc<T> l1, l2;
    T gg = sizeof(T) == 8 ? (T)DBL_EPSILON : (T)FLT_EPSILON, us = 0, ls = 0;
    int hit = 0;
    for (long long col = (long long)blockIdx.x * COLS_PER_BLOCK + threadIdx.y; col < d.ncol;
         col += (long long)gridDim.x * COLS_PER_BLOCK) {
        const long long o = col * d.P;
        for (int iz = threadIdx.x; iz <= d.nz; iz += 32) {
            const long long i = o + iz;
            const T x = vor[i], y = vor[N + i], z = vor[2 * N + i];
            if (iz >= 1) {
                const T v1 = (T)0.5 * fabs(vor[i - 1] + x);
                const T v2 = (T)0.5 * fabs(vor[N + i - 1] + y);
                const T v3 = (T)0.5 * fabs(vor[2 * N + i - 1] + z);
                if (v1 + v2 + v3 > vr) {
                    l1.add(v1 + v2 + v3);
                    l2.add(v1 * v1 + v2 * v2 + v3 * v3);
                }
            }
            const T dudx = g5[i], dudy = g5[N + i], dwdx = g5[2 * N + i], dvdy = g5[3 * N + i],
                    dwdy = g5[4 * N + i];
            const T lmax = StrainMax<T>::get(dudx, dudy + (T)0.5 * z, dwdx + (T)0.5 * y, dvdy,
                                             dwdy - (T)0.5 * x, -(dudx + dvdy), &hit);
            gg = fmax(gg, lmax);
            if (iz == d.nz) us = fmax(us, lmax);
            if (iz == 0) ls = fmax(ls, lmax);
        }
    }
    if (hit) atomicExch(flag, 1);
    double vals[RED2_N] = {l1.value(), l2.value(), (double)gg, (double)us, (double)ls};
    const int kinds[RED2_N] = {0, 0, 1, 1, 1};
    block_reduce_store<RED2_N>(vals, kinds, part);
}

template <typename T>
void red_pass2(const Dims &d, cudaStream_t st, const T *vor, const T *g5, double vortrms, double *part,
               double *result, int *flag, const double *res1, double ncell)
{
    const int nb = red_grid(d, k_red2<T>);
    k_red2<T><<<nb, COL_BLOCK, 0, st>>>(d, vor, g5, vortrms, res1, ncell, part, flag);
    int *kinds;
    cudaGetSymbolAddress((void **)&kinds, c_kinds2);
    k_finish<RED2_N><<<1, dim3(32, RED2_N), 0, st>>>(part, nb, kinds, result);
}

// ------------------------------------------------------------------- tables
// phim, phip, thetam, thetap, dthetam, dthetap (inversion_utils.f90:484-542)
// and the Green function (:281-288) per column
template <typename T>
__global__ void k_hyperbolic(Dims d, const double *__restrict__ k2l2, const double *__restrict__ k2l2i,
                             const double *__restrict__ rkz, const double *__restrict__ zm,
                             const double *__restrict__ zp, double Lz, T *phim, T *phip, T *thetam, T *thetap,
                             T *dthetam, T *dthetap, T *green)
{
    COLUMN_HEADER
    const int nz = d.nz;
    const double kk = k2l2[col], ki = k2l2i[col];
    if (col == 0) {
        for (int iz = threadIdx.x; iz <= nz; iz += 32) {
            const long long q = o + iz;
            phim[q] = (T)(zm[iz] / Lz);
            phip[q] = (T)(zp[iz] / Lz);
            thetam[q] = thetap[q] = dthetam[q] = dthetap[q] = (T)0;
            green[q] = (T)(iz == 0 ? -ki : -1.0 / (kk + rkz[iz] * rkz[iz]));
        }
        return;
    }
    const double kl = sqrt(kk);
    const double ef = exp(-kl * Lz);
    const double div = 1.0 / (1.0 - ef * ef);
    const double k2ifac = 0.5 * ki;
    const double Q = div * (1.0 + ef * ef);
    const double R = div * 2.0 * ef;
    for (int iz = threadIdx.x; iz <= nz; iz += 32) {
        const long long q = o + iz;
        const double Lm = kl * zm[iz], Lp = kl * zp[iz];
        const double ep = exp(-Lp), em = exp(-Lm);
        const double phm = div * (ep - ef * em);
        const double php = div * (em - ef * ep);
        const double dphm = -kl * div * (ep + ef * em);
        const double dphp = kl * div * (em + ef * ep);
        phim[q] = (T)phm;
        phip[q] = (T)php;
        thetam[q] = (T)(k2ifac * (R * Lm * php - Q * Lp * phm));
        thetap[q] = (T)(k2ifac * (R * Lp * phm - Q * Lm * php));
        dthetam[q] = (T)(-k2ifac * ((Q * Lp - 1.0) * dphm - R * Lm * dphp));
        dthetap[q] = (T)(-k2ifac * ((Q * Lm - 1.0) * dphp - R * Lp * dphm));
        green[q] = (T)(iz == 0 ? -ki : -1.0 / (kk + rkz[iz] * rkz[iz]));
    }
}
template <typename T>
void op_hyperbolic_tables(const Dims &d, cudaStream_t st, const double *k2l2, const double *k2l2i,
                          const double *rkz, const double *zm, const double *zp, double Lz, T *phim, T *phip,
                          T *thetam, T *thetap, T *dthetam, T *dthetap, T *green)
{
    k_hyperbolic<T><<<col_grid(d), COL_BLOCK, 0, st>>>(d, k2l2, k2l2i, rkz, zm, zp, Lz, phim, phip, thetam,
                                                       thetap, dthetam, dthetap, green);
}

// ------------------------------------------------------------ instantiation
#define INST_T(T)                                                                                              \
    template void op_diff<T>(const Dims &, cudaStream_t, const Deriv &, int, const T *, T *);                   \
    template void op_diffz<T>(const Dims &, cudaStream_t, double, const T *, T *);                              \
    template void op_v2v_ds<T, double>(const Dims &, cudaStream_t, const Deriv &, const double *,              \
                                       const double *, T *);                                                   \
    template void op_v2v_project<T, double>(const Dims &, cudaStream_t, const Deriv &, const double *,         \
                                            const T *, const T *, double *, double *);                         \
    template void op_v2v_wsrc<T, double>(const Dims &, cudaStream_t, const Deriv &, const double *,            \
                                         const double *, T *);                                                 \
    template void op_v2v_wprep<T>(const Dims &, cudaStream_t, const T *, const T *, const T *, const T *,      \
                                  const T *, const T *, const double *, T *, T *, T *, T *);                   \
    template void op_v2v_wfinish<T>(const Dims &, cudaStream_t, const T *, const T *, const T *, T *, T *);    \
    template void op_v2v_uv<T>(const Dims &, cudaStream_t, const Deriv &, const double *, const T *,           \
                               const T *, const double *, const double *, T *, T *);                           \
    template void op_add_const<T>(const Dims &, cudaStream_t, T *, double);                                    \
    template void op_products<T>(const Dims &, cudaStream_t, const T *, const T *, T *, T *, T *);             \
    template void op_svorts<T>(const Dims &, cudaStream_t, const Deriv &, const T *, const T *, const T *,     \
                               const T *, const T *, T *, T *, T *);                                           \
    template void op_strain_fields<T>(const Dims &, cudaStream_t, const Deriv &, const T *, T *);              \
    template void op_add<T, double>(const Dims &, cudaStream_t, double *, const T *, long long);              \
    template void op_rk4_sub1<T>(const Dims &, cudaStream_t, double *, double *, double *, T *,               \
                                 const double *, const double *, double, double);                              \
    template void op_rk4_sub23<T>(const Dims &, cudaStream_t, double *, const double *, double *, const T *,  \
                                  const double *, const double *, double, double);                             \
    template void op_rk4_sub4<T>(const Dims &, cudaStream_t, double *, const double *, const T *,             \
                                 const double *, const double *, double);                                      \
    template void op_cn2_init<T>(const Dims &, cudaStream_t, double *, const double *, const T *, double, int); \
    template void op_cn2_update<T>(const Dims &, cudaStream_t, double *, const double *, const T *,           \
                                   const double *, const double *, const double *, double, int);               \
    template void red_pass1<T>(const Dims &, cudaStream_t, const T *, const T *, double *, double *);         \
    template void red_pass2<T>(const Dims &, cudaStream_t, const T *, const T *, double, double *, double *,  \
                               int *, const double *, double);                                                 \
    template void op_hyperbolic_tables<T>(const Dims &, cudaStream_t, const double *, const double *,         \
                                          const double *, const double *, const double *, double, T *, T *,   \
                                          T *, T *, T *, T *, T *);

INST_T(double)
INST_T(float)
template void op_convert<float, double>(const Dims &, cudaStream_t, const double *, float *, long long);
template void op_v2v_ds<float, float>(const Dims &, cudaStream_t, const Deriv &, const float *, const float *,
                                      float *);
template void op_v2v_wsrc<float, float>(const Dims &, cudaStream_t, const Deriv &, const float *, const float *,
                                        float *);
template void op_v2v_project<float, float>(const Dims &, cudaStream_t, const Deriv &, const double *,
                                           const float *, const float *, float *, float *);
template void op_convert<double, float>(const Dims &, cudaStream_t, const float *, double *, long long);
template void op_v2v_meanflow<double>(const Dims &, cudaStream_t, const double *, const double *, const Tables &,
                                      double *, double *);

}  // namespace ps3d

// ======================================================================
// Energy series without any device allocation.
//
// Some callers cannot let this library allocate device memory: a driver
// that already keeps vel and vor resident in device arrays it manages itself
// (a CUDA Fortran or OpenACC port of the reference's time loop), code running
// under a fixed device-memory budget, or a loop that must not call
// cudaMalloc/cudaFree because those synchronise the whole device.  For them
// ps3d_gpu_energy_series_noalloc runs the same reduction kernels as
// ps3d_gpu_energy_series, with the per-block partial sums kept in the
// file-scope array below instead of in a context buffer.
//
// The array lives in every GPU that loads the library, for the life of the
// process.  It holds the partials of at most NOALLOC_MAX_BLOCKS blocks (one
// block per 8 columns), so nx*ny is limited to 8*NOALLOC_MAX_BLOCKS.  All
// calls share it: every call overwrites the entries it uses before reading
// them (nothing has to start at zero), and two calls that overlap on the GPU
// (for example on two streams at once) race on it.
// ======================================================================
namespace ps3d {
constexpr int NOALLOC_MAX_BLOCKS = 65536;
static __device__ __align__(256) double g_noalloc_scratch[(size_t)NOALLOC_MAX_BLOCKS * RED1_N + 2 * RED1_N];

__global__ void k_noalloc_energy_out(const double *res, double ncelli, double *out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        out[0] = 0.5 * res[2] * ncelli;  // kinetic energy
        out[1] = 0.5 * res[1] * ncelli;  // enstrophy
        out[2] = res[3] * ncelli;        // helicity
    }
}
}  // namespace ps3d

extern "C" int ps3d_gpu_energy_series_noalloc(const double *vel, const double *vor, int nx, int ny, int nz,
                                              long long pitch, long long comp_stride, void *stream, double *out)
{
    using namespace ps3d;
    if (!vel || !vor || !out || nx < 1 || ny < 1 || nz < 2 || pitch < nz + 1 || pitch > INT_MAX)
        return 1;  // PS3D_ERR_INVALID_ARG
    const long long ncol = (long long)nx * ny;
    // comp_stride >= pitch * ncol, checked by division (no overflow)
    if (comp_stride < 1 || comp_stride / ncol < pitch) return 1;
    const long long nblocks = (ncol + COLS_PER_BLOCK - 1) / COLS_PER_BLOCK;
    if (nblocks > NOALLOC_MAX_BLOCKS) return 2;  // PS3D_ERR_UNSUPPORTED_SIZE: nx*ny above the scratch capacity
    // Set-up: the device address of the scratch array in the current
    // device's context.  It is looked up on every call (a table lookup in
    // the runtime, no allocation), so it is right after cudaDeviceReset or
    // when the caller switches contexts.  The very first call on a device
    // may load this library's device code into the context, which is not
    // allowed during stream capture: make that first call outside a capture.
    double *part = nullptr;
    int *kinds = nullptr;
    if (cudaGetSymbolAddress((void **)&part, g_noalloc_scratch) != cudaSuccess || !part ||
        cudaGetSymbolAddress((void **)&kinds, c_kinds1) != cudaSuccess || !kinds) {
        const cudaError_t e = cudaGetLastError();
        return (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? 8 : 3;  // NO_DEVICE or CUDA
    }
    double *result = part + (size_t)NOALLOC_MAX_BLOCKS * RED1_N;
    Dims d;
    d.nx = nx;
    d.ny = ny;
    d.nz = nz;
    d.P = (int)pitch;
    d.ncol = ncol;
    d.nfield = comp_stride;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    k_red1<double><<<(unsigned)nblocks, COL_BLOCK, 0, st>>>(d, vel, vor, part);
    k_finish<RED1_N><<<1, dim3(32, RED1_N), 0, st>>>(part, (int)nblocks, kinds, result);
    k_noalloc_energy_out<<<1, 32, 0, st>>>(result, 1.0 / ((double)nx * (double)ny * (double)nz), out);
    return cudaGetLastError() == cudaSuccess ? 0 : 3;
}
