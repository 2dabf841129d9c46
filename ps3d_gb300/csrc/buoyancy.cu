// Buoyancy kernels (the reference built with ENABLE_BUOYANCY): the tables
// and column pieces of diffz (inversion_utils.f90:683-719), the flux products
// and the assembly of the buoyancy tendency (inversion.f90:232-292), the
// maximum buoyancy frequency of adapt (advance.f90:147-168) and the buoyancy
// diagnostics (field_diagnostics.f90:29-60, 268-397).
//
// Same walking scheme as ops.cu: a block is 32 x 8 threads, threadIdx.x runs
// along z (32 consecutive levels of one column per warp, coalesced),
// threadIdx.y picks one of 8 columns; x / y derivatives read the partner
// column (n - k) mod n.
#include <float.h>

#include "kernels.h"

namespace ps3d {

namespace {

constexpr int BCOLS = 8;
const dim3 BBLOCK(32, BCOLS);

inline dim3 bgrid(const Dims &d) { return dim3((unsigned)((d.ncol + BCOLS - 1) / BCOLS)); }

__device__ __forceinline__ int bsrc(int k, int n) { return k == 0 ? 0 : n - k; }

#define BCOLUMN                                                                \
    const long long col = (long long)blockIdx.x * BCOLS + threadIdx.y;         \
    if (col >= d.ncol) return;                                                 \
    const int kx = (int)(col / d.ny);                                          \
    const int ky = (int)(col - (long long)kx * d.ny);                          \
    const long long o = col * d.P;                                             \
    (void)kx; (void)ky;

// dphim / dphip, the z derivatives of the harmonic functions
// (set_hyperbolic_functions, inversion_utils.f90:484-542, with the linear
// (0,0) column of :333-336)
template <typename T>
__global__ void k_dphi(Dims d, const double *__restrict__ k2l2, const double *__restrict__ zm,
                       const double *__restrict__ zp, double Lz, T *dphim, T *dphip)
{
    BCOLUMN
    const int nz = d.nz;
    if (col == 0) {
        for (int iz = threadIdx.x; iz <= nz; iz += 32) {
            dphim[o + iz] = (T)(-1.0 / Lz);
            dphip[o + iz] = (T)(1.0 / Lz);
        }
        return;
    }
    const double kl = sqrt(k2l2[col]);
    const double ef = exp(-kl * Lz);
    const double div = 1.0 / (1.0 - ef * ef);
    for (int iz = threadIdx.x; iz <= nz; iz += 32) {
        const double ep = exp(-kl * zp[iz]), em = exp(-kl * zm[iz]);
        dphim[o + iz] = (T)(-kl * div * (ep + ef * em));
        dphip[o + iz] = (T)(kl * div * (em + ef * ep));
    }
}

// as(kz) = rkz(kz) fs(kz) on the interior, 0 on the walls (diffz, :696-707)
template <typename T>
__global__ void k_dz_sine(Dims d, const double *__restrict__ rkz, const T *__restrict__ fs, T *__restrict__ as)
{
    BCOLUMN
    const int nz = d.nz;
    for (int iz = threadIdx.x; iz <= nz; iz += 32)
        as[o + iz] = (iz == 0 || iz == nz) ? (T)0 : (T)(rkz[iz] * (double)fs[o + iz]);
}

// ds = (fs(0) dphim + fs(nz) dphip) + as: the semi-spectral derivative before
// its decomposition (diffz, :690-714)
template <typename T>
__global__ void k_dz_join(Dims d, const T *__restrict__ fs, const T *__restrict__ dphim,
                          const T *__restrict__ dphip, const T *__restrict__ as, T *__restrict__ ds)
{
    BCOLUMN
    const double f0 = (double)fs[o], fn = (double)fs[o + d.nz];
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) {
        const long long i = o + iz;
        ds[i] = (T)((f0 * (double)dphim[i] + fn * (double)dphip[i]) + (double)as[i]);
    }
}

// the three flux components u b, v b, w b (inversion.f90:245, 253, 261)
template <typename T>
__global__ void k_bflux(Dims d, const T *__restrict__ vel, const T *__restrict__ b, T *__restrict__ f)
{
    BCOLUMN
    const long long N = d.nfield;
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) {
        const long long i = o + iz;
        const double bb = (double)b[i];
        f[i] = (T)((double)vel[i] * bb);
        f[N + i] = (T)((double)vel[N + i] * bb);
        f[2 * N + i] = (T)((double)vel[2 * N + i] * bb);
    }
}

// Semi-spectral buoyancy tendency before its decomposition:
//   X = -D_x F_u - D_y F_v - N^2 W - Z,
// F the horizontal transforms of the fluxes, W the semi-spectral vertical
// velocity and Z the semi-spectral z derivative of F_w.
template <typename T>
__global__ void k_btend(Dims d, Deriv D, const T *__restrict__ fu, const T *__restrict__ fv,
                        const T *__restrict__ wsemi, const T *__restrict__ zs, double bfsq, T *__restrict__ out)
{
    BCOLUMN
    const long long ox = ((long long)ky + (long long)d.ny * bsrc(kx, d.nx)) * d.P;
    const long long oy = ((long long)bsrc(ky, d.ny) + (long long)d.ny * kx) * d.P;
    const double cx = D.cx[kx], cy = D.cy[ky];
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) {
        const long long i = o + iz;
        const double bx = cx * (double)fu[ox + iz], by = cy * (double)fv[oy + iz];
        out[i] = (T)(((-bx - by) - bfsq * (double)wsemi[i]) - (double)zs[i]);
    }
}

// f(iz) -= prof(iz): removal of the basic state N^2 z (utils.f90:152-157)
__global__ void k_sub_zprof(Dims d, double *__restrict__ f, const double *__restrict__ prof)
{
    BCOLUMN
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) f[o + iz] = f[o + iz] - prof[iz];
}

// f += g
template <typename T>
__global__ void k_addf(Dims d, T *__restrict__ f, const T *__restrict__ g)
{
    BCOLUMN
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) f[o + iz] = (T)((double)f[o + iz] + (double)g[o + iz]);
}

// pressure with buoyancy (fields_derived.f90:108-112): rhs += b_z + f_z zeta,
// b_z the central difference of the physical b'
template <typename T>
__global__ void k_pres_buoy_rhs(Dims d, const T *__restrict__ b, const T *__restrict__ zeta, double dzi, double fz,
                                T *__restrict__ out)
{
    BCOLUMN
    const int nz = d.nz;
    for (int iz = threadIdx.x; iz <= nz; iz += 32) {
        const long long i = o + iz;
        double bz;
        if (iz == 0) bz = dzi * ((double)b[o + 1] - (double)b[o]);
        else if (iz == nz) bz = dzi * ((double)b[o + nz] - (double)b[o + nz - 1]);
        else bz = ((double)b[i + 1] - (double)b[i - 1]) * (0.5 * dzi);
        out[i] = (T)(((double)out[i] + bz) + fz * (double)zeta[i]);
    }
}

// pressure with buoyancy, semi-spectral (fields_derived.f90:142-151):
// rs += sb(nz) k2l2i dphip + sb(0) k2l2i dphim
template <typename T>
__global__ void k_pres_buoy_bc(Dims d, const T *__restrict__ sb, const double *__restrict__ k2l2i,
                               const T *__restrict__ dphim, const T *__restrict__ dphip, T *__restrict__ rs)
{
    BCOLUMN
    const double ki = k2l2i[col];
    const double cn = (double)sb[o + d.nz] * ki, c0 = (double)sb[o] * ki;
    for (int iz = threadIdx.x; iz <= d.nz; iz += 32) {
        const long long i = o + iz;
        rs[i] = (T)(((double)rs[i] + cn * (double)dphip[i]) + c0 * (double)dphim[i]);
    }
}

// Order-preserving bits of a non-negative double (atomicMax on the bits)
__device__ __forceinline__ unsigned long long dbits(double v) { return (unsigned long long)__double_as_longlong(v); }

// max over the grid of b_x^2 + b_y^2 + (b_z + N^2)^2, b_z the central
// difference of the physical buoyancy (central_diffz commutes with the
// horizontal transform, advance.f90:157-163)
template <typename T>
__global__ void k_bgrad_max(Dims d, const T *__restrict__ bx, const T *__restrict__ by, const T *__restrict__ b,
                            double dzi, double bfsq, unsigned long long *out)
{
    __shared__ double red[BCOLS * 32];
    const long long col = (long long)blockIdx.x * BCOLS + threadIdx.y;
    double mx = 0.0;
    if (col < d.ncol) {
        const long long o = col * d.P;
        const int nz = d.nz;
        for (int iz = threadIdx.x; iz <= nz; iz += 32) {
            const long long i = o + iz;
            double bz;
            if (iz == 0) bz = dzi * ((double)b[o + 1] - (double)b[o]);
            else if (iz == nz) bz = dzi * ((double)b[o + nz] - (double)b[o + nz - 1]);
            else bz = ((double)b[i + 1] - (double)b[i - 1]) * (0.5 * dzi);
            const double gx = (double)bx[i], gy = (double)by[i], gz = bz + bfsq;
            mx = fmax(mx, gx * gx + gy * gy + gz * gz);
        }
    }
    const int t = threadIdx.y * 32 + threadIdx.x;
    red[t] = mx;
    __syncthreads();
    for (int w = BCOLS * 16; w > 0; w >>= 1) {
        if (t < w) red[t] = fmax(red[t], red[t + w]);
        __syncthreads();
    }
    if (t == 0) atomicMax(out, dbits(red[0]));
}

// Buoyancy diagnostics, per-block partials:
//   [0] z-trapezoid sum of b^2, [1] of sqrt(b_x^2 + 2 b_y^2) (the reference's
//   |grad b|, field_diagnostics.f90:369-374), [2] min b_z, [3] min of
//   (N^2 + b_z) / (xi^2 + eta^2)
constexpr int BDIAG_N = 4;
template <typename T>
__global__ void k_bdiag(Dims d, const T *__restrict__ b, const T *__restrict__ bx, const T *__restrict__ by,
                        const T *__restrict__ vor, double dzi, double bfsq, double *part)
{
    __shared__ double red[BDIAG_N][BCOLS * 32];
    const long long col = (long long)blockIdx.x * BCOLS + threadIdx.y;
    double s0 = 0.0, s1 = 0.0, m2 = DBL_MAX, m3 = DBL_MAX;
    if (col < d.ncol) {
        const long long o = col * d.P, N = d.nfield;
        const int nz = d.nz;
        for (int iz = threadIdx.x; iz <= nz; iz += 32) {
            const long long i = o + iz;
            const double w = (iz == 0 || iz == nz) ? 0.5 : 1.0;
            const double bb = (double)b[i], gx = (double)bx[i], gy = (double)by[i];
            double bz;
            if (iz == 0) bz = dzi * ((double)b[o + 1] - (double)b[o]);
            else if (iz == nz) bz = dzi * ((double)b[o + nz] - (double)b[o + nz - 1]);
            else bz = ((double)b[i + 1] - (double)b[i - 1]) * (0.5 * dzi);
            s0 += w * bb * bb;
            s1 += w * sqrt(gx * gx + gy * gy + gy * gy);
            m2 = fmin(m2, bz);
            const double xi = (double)vor[i], eta = (double)vor[N + i];
            m3 = fmin(m3, (bfsq + bz) / (xi * xi + eta * eta));
        }
    }
    const int t = threadIdx.y * 32 + threadIdx.x;
    red[0][t] = s0;
    red[1][t] = s1;
    red[2][t] = m2;
    red[3][t] = m3;
    __syncthreads();
    for (int w = BCOLS * 16; w > 0; w >>= 1) {
        if (t < w) {
            red[0][t] += red[0][t + w];
            red[1][t] += red[1][t + w];
            red[2][t] = fmin(red[2][t], red[2][t + w]);
            red[3][t] = fmin(red[3][t], red[3][t + w]);
        }
        __syncthreads();
    }
    if (t < BDIAG_N) part[(long long)blockIdx.x * BDIAG_N + t] = red[t][0];
}

__global__ void k_bdiag_finish(long long nblk, const double *__restrict__ part, double *out)
{
    __shared__ double red[BDIAG_N][256];
    double s0 = 0.0, s1 = 0.0, m2 = DBL_MAX, m3 = DBL_MAX;
    for (long long b = threadIdx.x; b < nblk; b += blockDim.x) {
        s0 += part[b * BDIAG_N];
        s1 += part[b * BDIAG_N + 1];
        m2 = fmin(m2, part[b * BDIAG_N + 2]);
        m3 = fmin(m3, part[b * BDIAG_N + 3]);
    }
    const int t = threadIdx.x;
    red[0][t] = s0;
    red[1][t] = s1;
    red[2][t] = m2;
    red[3][t] = m3;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (t < w) {
            red[0][t] += red[0][t + w];
            red[1][t] += red[1][t + w];
            red[2][t] = fmin(red[2][t], red[2][t + w]);
            red[3][t] = fmin(red[3][t], red[3][t + w]);
        }
        __syncthreads();
    }
    if (t < BDIAG_N) out[t] = red[t][0];
}

}  // namespace

long long bdiag_blocks(const Dims &d) { return (d.ncol + BCOLS - 1) / BCOLS; }

template <typename T>
void op_dphi_tables(const Dims &d, cudaStream_t st, const double *k2l2, const double *zm, const double *zp, double Lz,
                    T *dphim, T *dphip)
{
    k_dphi<T><<<bgrid(d), BBLOCK, 0, st>>>(d, k2l2, zm, zp, Lz, dphim, dphip);
}
template <typename T> void op_dz_sine(const Dims &d, cudaStream_t st, const double *rkz, const T *fs, T *as)
{
    k_dz_sine<T><<<bgrid(d), BBLOCK, 0, st>>>(d, rkz, fs, as);
}
template <typename T>
void op_dz_join(const Dims &d, cudaStream_t st, const T *fs, const T *dphim, const T *dphip, const T *as, T *ds)
{
    k_dz_join<T><<<bgrid(d), BBLOCK, 0, st>>>(d, fs, dphim, dphip, as, ds);
}
template <typename T> void op_bflux(const Dims &d, cudaStream_t st, const T *vel, const T *b, T *f)
{
    k_bflux<T><<<bgrid(d), BBLOCK, 0, st>>>(d, vel, b, f);
}
template <typename T>
void op_btend(const Dims &d, cudaStream_t st, const Deriv &D, const T *fu, const T *fv, const T *wsemi, const T *zs,
              double bfsq, T *out)
{
    k_btend<T><<<bgrid(d), BBLOCK, 0, st>>>(d, D, fu, fv, wsemi, zs, bfsq, out);
}
template <typename T>
void op_pres_buoy_rhs(const Dims &d, cudaStream_t st, const T *b, const T *zeta, double dzi, double fz, T *out)
{
    k_pres_buoy_rhs<T><<<bgrid(d), BBLOCK, 0, st>>>(d, b, zeta, dzi, fz, out);
}
template <typename T>
void op_pres_buoy_bc(const Dims &d, cudaStream_t st, const T *sb, const double *k2l2i, const T *dphim, const T *dphip,
                     T *rs)
{
    k_pres_buoy_bc<T><<<bgrid(d), BBLOCK, 0, st>>>(d, sb, k2l2i, dphim, dphip, rs);
}
void op_sub_zprof(const Dims &d, cudaStream_t st, double *f, const double *prof)
{
    k_sub_zprof<<<bgrid(d), BBLOCK, 0, st>>>(d, f, prof);
}
template <typename T> void op_addf(const Dims &d, cudaStream_t st, T *f, const T *g)
{
    k_addf<T><<<bgrid(d), BBLOCK, 0, st>>>(d, f, g);
}
template <typename T>
void op_bgrad_max(const Dims &d, cudaStream_t st, const T *bx, const T *by, const T *b, double dzi, double bfsq,
                  unsigned long long *out)
{
    cudaMemsetAsync(out, 0, sizeof(unsigned long long), st);
    k_bgrad_max<T><<<bgrid(d), BBLOCK, 0, st>>>(d, bx, by, b, dzi, bfsq, out);
}
template <typename T>
void op_bdiag(const Dims &d, cudaStream_t st, const T *b, const T *bx, const T *by, const T *vor, double dzi,
              double bfsq, double *part, double *out)
{
    k_bdiag<T><<<bgrid(d), BBLOCK, 0, st>>>(d, b, bx, by, vor, dzi, bfsq, part);
    k_bdiag_finish<<<1, 256, 0, st>>>(bdiag_blocks(d), part, out);
}

#define INST_B(T)                                                                                             \
    template void op_dphi_tables<T>(const Dims &, cudaStream_t, const double *, const double *, const double *, \
                                    double, T *, T *);                                                         \
    template void op_dz_sine<T>(const Dims &, cudaStream_t, const double *, const T *, T *);                   \
    template void op_dz_join<T>(const Dims &, cudaStream_t, const T *, const T *, const T *, const T *, T *);   \
    template void op_bflux<T>(const Dims &, cudaStream_t, const T *, const T *, T *);                           \
    template void op_btend<T>(const Dims &, cudaStream_t, const Deriv &, const T *, const T *, const T *,      \
                              const T *, double, T *);                                                         \
    template void op_addf<T>(const Dims &, cudaStream_t, T *, const T *);                                       \
    template void op_pres_buoy_rhs<T>(const Dims &, cudaStream_t, const T *, const T *, double, double, T *);  \
    template void op_pres_buoy_bc<T>(const Dims &, cudaStream_t, const T *, const double *, const T *,        \
                                     const T *, T *);                                                          \
    template void op_bgrad_max<T>(const Dims &, cudaStream_t, const T *, const T *, const T *, double, double, \
                                  unsigned long long *);                                                       \
    template void op_bdiag<T>(const Dims &, cudaStream_t, const T *, const T *, const T *, const T *, double,   \
                              double, double *, double *);
INST_B(float)
INST_B(double)

}  // namespace ps3d
