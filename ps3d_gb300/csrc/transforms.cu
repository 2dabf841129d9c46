// Spectral transform kernels for the ps3d hot path on sm_103a.
//
// Device layout of a scalar field: z fastest with a padded column pitch P
// (P >= nz+1, a multiple of 8), element (iz, iy, ix) at iz + P*(iy + ny*ix).
// Rows nz+1..P-1 are padding: every column operation ignores them, and the
// line transforms read them as zero (two z rows share one complex line, so
// leftover content would otherwise reach the top row's last bit).
//
//  * lines kernels (fftxyp2s / fftxys2p of src/fft/sta3dfft.f90:136-260):
//    real FFTs along y (or x) in the reference's Hermitian storage
//    (src/fft/stafft.f90:55-58, scale 1/sqrt(n)).  A block owns a tile of
//    2*B consecutive z values of one x (or y) line set; consecutive z pairs
//    are packed as one complex sequence (two real transforms for the price
//    of one complex FFT) and transformed with the shared-memory Stockham
//    FFT; the pencil transposes of the reference (fft_pencil.f90) disappear
//    because the tile loads are coalesced along z.
//  * column kernels (dst/dct of stafft.f90:410-550 on every column, fused
//    with the harmonic subtract/add of field_decompose_semi_spectral /
//    field_combine_semi_spectral, inversion_utils.f90:563-647): two columns
//    are packed as one complex sequence of their odd (DST) or even (DCT)
//    extension of length 2*nz, so the transform is a single complex FFT.
#include "kernels.h"

namespace ps3d {

// ------------------------------------------------------------------------
// y / x line transforms
// ------------------------------------------------------------------------
template <typename T, bool INV>
__global__ void __launch_bounds__(256) k_lines(const T *__restrict__ in, T *__restrict__ out, int n,
                                               int logB, int P, int zv, long long line_stride,
                                               long long batch_stride,
                                               const typename cplx<T>::type *__restrict__ tw)
{
    using C = typename cplx<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *buf0 = reinterpret_cast<C *>(smem_raw);
    const int B = 1 << logB;
    C *buf1 = buf0 + (size_t)n * B;
    const int z0 = blockIdx.x * 2 * B;
    const long long base = (long long)blockIdx.y * batch_stride + z0;
    const T s = (T)(1.0 / sqrt((double)n));
    const C *inC = reinterpret_cast<const C *>(in);
    C *outC = reinterpret_cast<C *>(out);

    if (!INV) {
        for (int e = threadIdx.x; e < n * B; e += blockDim.x) {
            const int i = e >> logB, p = e & (B - 1);
            C v = mk<C>(0, 0);
            if (z0 + 2 * p < P) v = inC[(base + i * line_stride + 2 * p) >> 1];
            // padding rows (z >= zv) enter as zero: the paired real line
            // must not pick up leftover content
            if (z0 + 2 * p + 1 >= zv) v.y = 0;
            if (z0 + 2 * p >= zv) v.x = 0;
            buf0[e] = v;
        }
    } else {
        // rebuild the complex spectrum C_k = A_k + i B_k of the two packed
        // real sequences from their Hermitian storage
        const int h = n / 2;
        for (int e = threadIdx.x; e < (h + 1) * B; e += blockDim.x) {
            const int k = e >> logB, p = e & (B - 1);
            C lo = mk<C>(0, 0), hi = mk<C>(0, 0);
            if (z0 + 2 * p < P) {
                lo = inC[(base + k * line_stride + 2 * p) >> 1];
                if (k > 0 && k < h) hi = inC[(base + (n - k) * line_stride + 2 * p) >> 1];
            }
            if (z0 + 2 * p + 1 >= zv) lo.y = hi.y = 0;
            if (z0 + 2 * p >= zv) lo.x = hi.x = 0;
            // A_k = (lo.x, hi.x), B_k = (lo.y, hi.y)
            buf0[(k << logB) + p] = mk<C>(lo.x - hi.y, hi.x + lo.y);
            if (k > 0 && k < h) buf0[((n - k) << logB) + p] = mk<C>(lo.x + hi.y, lo.y - hi.x);
        }
    }
    __syncthreads();
    C *res = smem_fft<INV>(buf0, buf1, n, logB, tw);
    if (!INV) {
        const int h = n / 2;
        const T half = (T)0.5;
        for (int e = threadIdx.x; e < (h + 1) * B; e += blockDim.x) {
            const int k = e >> logB, p = e & (B - 1);
            if (z0 + 2 * p >= P) continue;
            const C ck = res[(k << logB) + p];
            const C cn = res[((k == 0 ? 0 : n - k) << logB) + p];
            const T are = half * (ck.x + cn.x), aim = half * (ck.y - cn.y);
            const T bre = half * (ck.y + cn.y), bim = -half * (ck.x - cn.x);
            outC[(base + k * line_stride + 2 * p) >> 1] = mk<C>(are * s, bre * s);
            if (k > 0 && k < h) outC[(base + (n - k) * line_stride + 2 * p) >> 1] = mk<C>(aim * s, bim * s);
        }
    } else {
        for (int e = threadIdx.x; e < n * B; e += blockDim.x) {
            const int i = e >> logB, p = e & (B - 1);
            if (z0 + 2 * p >= P) continue;
            const C v = res[e];
            outC[(base + i * line_stride + 2 * p) >> 1] = mk<C>(v.x * s, v.y * s);
        }
    }
}

template <typename T>
int lines_lanes(int n)
{
    // complex lanes per block: keep the two shared buffers within 64 KiB
    const int bytes_per_lane = 2 * n * (int)sizeof(typename cplx<T>::type);
    int B = 1;
    while (B < 16 && (2 * B) * bytes_per_lane <= 65536) B *= 2;
    return B;
}

// nf fields (field f at in + f fs_in, out + f fs_out): one launch for the
// FP32 line kernels, one per field otherwise
template <typename T>
void launch_lines(cudaStream_t st, const T *in, T *out, int n, int P, int zv, long long line_stride,
                  long long nbatch, long long batch_stride, bool inverse,
                  const typename cplx<T>::type *tw, int shape = -1, int nf = 1, long long fs_in = 0,
                  long long fs_out = 0)
{
    if constexpr (sizeof(T) == sizeof(float)) {
        if (lines32_supported(n)) {
            launch_lines32(st, reinterpret_cast<const float *>(in), reinterpret_cast<float *>(out), n, P, zv,
                           line_stride, nbatch, batch_stride, inverse, reinterpret_cast<const float2 *>(tw), shape,
                           nf, fs_in, fs_out);
            return;
        }
    }
    const int B = lines_lanes<T>(n);
    const int logB = ilog2(B);
    dim3 grid((P + 2 * B - 1) / (2 * B), (unsigned)nbatch);
    const size_t sm = 2 * (size_t)n * B * sizeof(typename cplx<T>::type);
    for (int f = 0; f < nf; ++f) {
        const T *fi = in + f * fs_in;
        T *fo = out + f * fs_out;
        if (inverse)
            k_lines<T, true><<<grid, 256, sm, st>>>(fi, fo, n, logB, P, zv, line_stride, batch_stride, tw);
        else
            k_lines<T, false><<<grid, 256, sm, st>>>(fi, fo, n, logB, P, zv, line_stride, batch_stride, tw);
    }
}

// algorithmic bytes of one pass over a field: read + write nx*ny*(nz+1)
template <typename T> static double pass_bytes(const Dims &d)
{
    return 2.0 * (double)d.ncol * (double)(d.nz + 1) * sizeof(T);
}

// The horizontal transforms of nf consecutive fields (nfield apart) in one
// launch per pass.  y lines: line stride P (one column), batches over x
// (stride ny P); x lines: line stride ny P, batches over y (stride P).
template <typename T>
void y_forward(const Dims &d, cudaStream_t st, const T *in, T *out, const typename cplx<T>::type *twy, Probe *pr,
               int nf)
{
    if (pr) pr->begin(PROBE_YLINES, st);
    launch_lines<T>(st, in, out, d.ny, d.P, d.nz + 1, d.P, d.nx, (long long)d.ny * d.P, false, twy, d.line_shape[0],
                    nf, d.nfield, d.nfield);
    if (pr) pr->end(PROBE_YLINES, st, nf * pass_bytes<T>(d));
}

template <typename T>
void x_forward(const Dims &d, cudaStream_t st, const T *in, T *out, const typename cplx<T>::type *twx, Probe *pr,
               int nf)
{
    if (pr) pr->begin(PROBE_XLINES, st);
    launch_lines<T>(st, in, out, d.nx, d.P, d.nz + 1, (long long)d.ny * d.P, d.ny, d.P, false, twx, d.line_shape[1],
                    nf, d.nfield, d.nfield);
    if (pr) pr->end(PROBE_XLINES, st, nf * pass_bytes<T>(d));
}

template <typename T>
void x_inverse(const Dims &d, cudaStream_t st, const T *in, T *out, const typename cplx<T>::type *twx, Probe *pr,
               int nf)
{
    if (pr) pr->begin(PROBE_XLINES, st);
    launch_lines<T>(st, in, out, d.nx, d.P, d.nz + 1, (long long)d.ny * d.P, d.ny, d.P, true, twx, d.line_shape[3],
                    nf, d.nfield, d.nfield);
    if (pr) pr->end(PROBE_XLINES, st, nf * pass_bytes<T>(d));
}

template <typename T>
void y_inverse(const Dims &d, cudaStream_t st, const T *in, T *out, const typename cplx<T>::type *twy, Probe *pr,
               int nf)
{
    if (pr) pr->begin(PROBE_YLINES, st);
    launch_lines<T>(st, in, out, d.ny, d.P, d.nz + 1, d.P, d.nx, (long long)d.ny * d.P, true, twy, d.line_shape[2],
                    nf, d.nfield, d.nfield);
    if (pr) pr->end(PROBE_YLINES, st, nf * pass_bytes<T>(d));
}

template <typename T>
void xy_forward(const Dims &d, cudaStream_t st, const T *in, T *out, const typename cplx<T>::type *twx,
                const typename cplx<T>::type *twy, Probe *pr, int nf)
{
    y_forward<T>(d, st, in, out, twy, pr, nf);
    x_forward<T>(d, st, out, out, twx, pr, nf);
}

template <typename T>
void xy_inverse(const Dims &d, cudaStream_t st, const T *in, T *out, const typename cplx<T>::type *twx,
                const typename cplx<T>::type *twy, Probe *pr, int nf)
{
    x_inverse<T>(d, st, in, out, twx, pr, nf);
    y_inverse<T>(d, st, out, out, twy, pr, nf);
}

// ------------------------------------------------------------------------
// column transforms (DST / DCT along z) with fused harmonic parts
// ------------------------------------------------------------------------
// mode: COL_DST      plain dst of rows 1..nz-1, row nz := 0 (stafft dst)
//       COL_DCT      plain dct of rows 0..nz
//       COL_DECOMP   rows 1..nz-1 -= f0*phim + fnz*phip, then dst; rows 0, nz kept
//       COL_COMBINE  dst of rows 1..nz-1, then += f0*phim + fnz*phip; rows 0, nz kept
template <typename T, int MODE, typename TIN>
__global__ void __launch_bounds__(256) k_columns(const TIN *__restrict__ in, T *__restrict__ out, int nz,
                                                 int P, int logB, const T *__restrict__ phim,
                                                 const T *__restrict__ phip,
                                                 const typename cplx<T>::type *__restrict__ tw)
{
    using C = typename cplx<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int B = 1 << logB;
    const int L = 2 * nz;
    C *buf0 = reinterpret_cast<C *>(smem_raw);
    C *buf1 = buf0 + (size_t)L * B;
    T *bnd = reinterpret_cast<T *>(buf1 + (size_t)L * B);  // f0, fnz per column (2*2*B)
    const long long col0 = (long long)blockIdx.x * 2 * B;

    // boundary values of the 2B columns
    for (int e = threadIdx.x; e < 2 * B; e += blockDim.x) {
        const long long c = col0 + e;
        bnd[2 * e] = (T)in[c * P];
        bnd[2 * e + 1] = (T)in[c * P + nz];
    }
    __syncthreads();
    // load the 2B columns into the extension buffer (column 2p -> .x, 2p+1 -> .y)
    const int nrow = nz + 1;
    for (int e = threadIdx.x; e < 2 * B * nrow; e += blockDim.x) {
        const int cl = e / nrow, iz = e - cl * nrow;
        const int p = cl >> 1, comp = cl & 1;
        T v = (T)in[(col0 + cl) * P + iz];
        if (MODE == COL_DECOMP && iz > 0 && iz < nz) {
            const long long q = (col0 + cl) * P + iz;
            v = v - (bnd[2 * cl] * phim[q] + bnd[2 * cl + 1] * phip[q]);
        }
        T *b0 = reinterpret_cast<T *>(buf0);
        if (MODE == COL_DCT) {
            b0[2 * ((iz << logB) + p) + comp] = v;
            if (iz > 0 && iz < nz) b0[2 * (((L - iz)) << logB) + 2 * p + comp] = v;
        } else {
            if (iz > 0 && iz < nz) {
                b0[2 * ((iz << logB) + p) + comp] = v;
                b0[2 * (((L - iz)) << logB) + 2 * p + comp] = -v;
            } else if (iz == 0) {
                b0[2 * ((0 << logB) + p) + comp] = (T)0;
            } else {
                b0[2 * ((nz << logB) + p) + comp] = (T)0;
            }
        }
    }
    __syncthreads();
    C *res = smem_fft<false>(buf0, buf1, L, logB, tw);
    const T s = (T)(1.0 / sqrt(2.0 * (double)nz));
    for (int e = threadIdx.x; e < 2 * B * nrow; e += blockDim.x) {
        const int cl = e / nrow, iz = e - cl * nrow;
        const int p = cl >> 1, comp = cl & 1;
        const long long q = (col0 + cl) * P + iz;
        const C c = res[(iz << logB) + p];
        T v;
        if (MODE == COL_DCT) {
            v = (comp == 0 ? c.x : c.y) * s;
        } else {
            if (iz == 0) {
                v = bnd[2 * cl];
                if (MODE == COL_DST) v = (T)in[q];
            } else if (iz == nz) {
                v = (MODE == COL_DST) ? (T)0 : bnd[2 * cl + 1];
            } else {
                v = (comp == 0 ? -c.y : c.x) * s;
                if (MODE == COL_COMBINE) v = v + bnd[2 * cl] * phim[q] + bnd[2 * cl + 1] * phip[q];
            }
        }
        out[q] = v;
    }
}

template <typename T>
int column_lanes(int nz)
{
    const int bytes_per_lane = 2 * (2 * nz) * (int)sizeof(typename cplx<T>::type);
    int B = 1;
    while (B < 16 && (2 * B) * bytes_per_lane <= 65536) B *= 2;
    return B;
}

template <typename T, typename TIN>
void columns_in(const Dims &d, cudaStream_t st, int mode, const TIN *in, T *out, const T *phim,
                const T *phip, const typename cplx<T>::type *twz2, Probe *pr)
{
    if (pr) pr->begin(PROBE_COLUMNS, st);
    int B = column_lanes<T>(d.nz);
    const long long ncol = (long long)d.nx * d.ny;
    while (B > 1 && ncol % (2 * B) != 0) B /= 2;
    const int logB = ilog2(B);
    const unsigned grid = (unsigned)(ncol / (2 * B));
    const size_t sm = 2 * (size_t)(2 * d.nz) * B * sizeof(typename cplx<T>::type) + 4 * B * sizeof(T);
    switch (mode) {
    case COL_DST:
        k_columns<T, COL_DST, TIN><<<grid, 256, sm, st>>>(in, out, d.nz, d.P, logB, phim, phip, twz2);
        break;
    case COL_DCT:
        k_columns<T, COL_DCT, TIN><<<grid, 256, sm, st>>>(in, out, d.nz, d.P, logB, phim, phip, twz2);
        break;
    case COL_DECOMP:
        k_columns<T, COL_DECOMP, TIN><<<grid, 256, sm, st>>>(in, out, d.nz, d.P, logB, phim, phip, twz2);
        break;
    default:
        k_columns<T, COL_COMBINE, TIN><<<grid, 256, sm, st>>>(in, out, d.nz, d.P, logB, phim, phip, twz2);
        break;
    }
    if (pr) pr->end(PROBE_COLUMNS, st, pass_bytes<T>(d));
}

template <typename T>
void columns(const Dims &d, cudaStream_t st, int mode, const T *in, T *out, const T *phim,
             const T *phip, const typename cplx<T>::type *twz2, Probe *pr)
{
    columns_in<T, T>(d, st, mode, in, out, phim, phip, twz2, pr);
}

size_t lines_smem_bytes(int n, bool fp64)
{
    if (fp64) return 2 * (size_t)n * lines_lanes<double>(n) * sizeof(double2);
    return 2 * (size_t)n * lines_lanes<float>(n) * sizeof(float2);
}

size_t columns_smem_bytes(int nz, bool fp64)
{
    if (fp64) return 2 * (size_t)(2 * nz) * column_lanes<double>(nz) * sizeof(double2) + 4 * 16 * sizeof(double);
    return 2 * (size_t)(2 * nz) * column_lanes<float>(nz) * sizeof(float2) + 4 * 16 * sizeof(float);
}

template <typename T, typename TIN>
static void set_col_attrs()
{
    cudaFuncSetAttribute(k_columns<T, COL_DST, TIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    cudaFuncSetAttribute(k_columns<T, COL_DCT, TIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    cudaFuncSetAttribute(k_columns<T, COL_DECOMP, TIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    cudaFuncSetAttribute(k_columns<T, COL_COMBINE, TIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
}

template <typename T>
static void set_smem_attrs()
{
    cudaFuncSetAttribute(k_lines<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    cudaFuncSetAttribute(k_lines<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    set_col_attrs<T, T>();
}

void transforms_init()
{
    lines32_init();
    set_smem_attrs<double>();
    set_smem_attrs<float>();
    set_col_attrs<float, double>();
}

template void xy_forward<double>(const Dims &, cudaStream_t, const double *, double *, const double2 *,
                                 const double2 *, Probe *, int);
template void xy_forward<float>(const Dims &, cudaStream_t, const float *, float *, const float2 *,
                                const float2 *, Probe *, int);
template void xy_inverse<double>(const Dims &, cudaStream_t, const double *, double *, const double2 *,
                                 const double2 *, Probe *, int);
template void xy_inverse<float>(const Dims &, cudaStream_t, const float *, float *, const float2 *,
                                const float2 *, Probe *, int);
template void x_forward<float>(const Dims &, cudaStream_t, const float *, float *, const float2 *, Probe *, int);
template void x_inverse<float>(const Dims &, cudaStream_t, const float *, float *, const float2 *, Probe *, int);
template void y_inverse<float>(const Dims &, cudaStream_t, const float *, float *, const float2 *, Probe *, int);
template void columns<double>(const Dims &, cudaStream_t, int, const double *, double *, const double *,
                              const double *, const double2 *, Probe *);
template void columns<float>(const Dims &, cudaStream_t, int, const float *, float *, const float *,
                             const float *, const float2 *, Probe *);
template void columns_in<float, double>(const Dims &, cudaStream_t, int, const double *, float *, const float *,
                                       const float *, const float2 *, Probe *);

}  // namespace ps3d
