// Learned sub-grid closure: a four-layer 3x3x3 convolution network on the
// physical grid of a run, trained and evaluated on the device.
//
// No counterpart in the reference (its only sub-grid model is the horizontal
// hyperdiffusion of inversion_utils.f90:124-218, which stays in force).
//
// Layout.  A grid point p = iz + Z*(iy + ny*ix), Z = nz+1 (the reference's
// column-major order without padding).  Activations are channels-last BF16,
// act[p*C + c], with C padded to 16 or 32 channels: the network input has 6
// channels (3 vorticity + 3 velocity components over their rms) padded to 16,
// the hidden layers 32, the output 3 padded to 8 (FP32), its gradient 16.
//
// Convolution = implicit GEMM on the tensor cores (mma.sync m16n8k16, BF16
// in, FP32 accumulate): rows are 16 grid points, the reduction runs over 27
// taps x the input channels, the columns are the output channels.  The
// reduction index inside each 16-wide step is permuted so that a lane's A
// fragment for a row is ONE contiguous 8- or 16-byte load of the input row
// (lane t of a quad holds channels [C/4*t, C/4*(t+1))); the weight image in
// shared memory is stored in the same permuted order, already in B-fragment
// register order (one 8-byte shared load per fragment).  The output columns
// are permuted the same way so that each lane stores a contiguous run of
// C/4 channels per row.
// Backward data = the same kernel with the mirrored, transposed weight image
// (periodic x, y and zero padding in z make the adjoint another convolution
// of the same shape), the GELU derivative fused in its epilogue.
// Weight gradients: per tap, dW = X_tap^T dZ over the points, staged through
// shared memory and read with ldmatrix.trans; per-chunk partial sums are
// reduced by a second kernel (deterministic).  Tap 27 is the bias (a column
// of ones).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ps3d_gpu.h"
#include "kernels.h"

namespace {

using bf16 = __nv_bfloat16;

constexpr int NL = 4;
constexpr int NTAP = 27;
constexpr int CREAL_IN[NL] = {6, 32, 32, 32};
constexpr int CREAL_OUT[NL] = {32, 32, 32, 3};
constexpr int CPAD_IN[NL] = {16, 32, 32, 32};
constexpr int CPAD_OUT[NL] = {32, 32, 32, 8};
constexpr int CPAD_DZ4 = 16;  // output-layer gradient channels (a 16-wide k step)
constexpr int OUTC = 8;       // = CPAD_OUT[NL - 1], usable in device code

constexpr int woff(int l)
{
    int o = 0;
    for (int i = 0; i < l; ++i) o += NTAP * CREAL_IN[i] * CREAL_OUT[i] + CREAL_OUT[i];
    return o;
}
constexpr int NPARAM = woff(NL);
static_assert(NPARAM == PS3D_CLOSURE_NPARAM, "parameter count");

constexpr int CONV_THREADS = 128;  // 4 warps
constexpr int CONV_ROWS = 128;     // grid points per block tile (32 per warp)
constexpr int WG_KW = 32;          // 16-point k steps per warp in the weight gradient
constexpr int WG_CHUNK = 4 * WG_KW * 16;
constexpr int RED_THREADS = 256;
constexpr int RED_BLOCKS = 256;

enum { EPI_GELU = 0, EPI_OUT = 1, EPI_BWD = 2 };

// ------------------------------------------------------------ device helpers
__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float dgelu_f(float x)
{
    // d/dx [x Phi(x)] = Phi(x) + x phi(x)
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}
__device__ __forceinline__ uint32_t pack2(float a, float b)
{
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&h);
}
__device__ __forceinline__ float2 unpack2(uint32_t u)
{
    __nv_bfloat162 h = *reinterpret_cast<__nv_bfloat162 *>(&u);
    return __bfloat1622float2(h);
}
__device__ __forceinline__ void mma16816(float *d, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}
__device__ __forceinline__ void ldsm_x4_trans(uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3,
                                              const void *smem_row)
{
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(smem_row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(a));
}

// A-operand row slice of one lane: C/4 channels (CIN 32: 16 bytes, CIN 16: 8)
template <int CIN> struct RowT;
template <> struct RowT<32> {
    using type = uint4;
    __device__ static uint32_t reg(const uint4 &v, int i) { return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w; }
    __device__ static uint4 zero() { return make_uint4(0u, 0u, 0u, 0u); }
};
template <> struct RowT<16> {
    using type = uint2;
    __device__ static uint32_t reg(const uint2 &v, int i) { return i == 0 ? v.x : v.y; }
    __device__ static uint2 zero() { return make_uint2(0u, 0u); }
};

struct ConvArgs {
    const bf16 *in;      // [npts][CIN]
    const uint2 *wimg;   // fragment-ordered weights, NTAP*(CIN/16)*(COUT/8)*32 entries
    const float *bias;   // [COUT] (EPI_GELU, EPI_OUT)
    bf16 *z;             // EPI_GELU: pre-activation [npts][COUT]
    bf16 *act;           // EPI_GELU: GELU(z); EPI_BWD: gradient of the layer below
    float *outf;         // EPI_OUT: [npts][COUT]
    const bf16 *zprev;   // EPI_BWD: pre-activation of the layer below [npts][COUT]
    int nx, ny, Z;
    long long npts;
};

// One 3x3x3 convolution over all grid points: a persistent grid of 4-warp
// blocks walks tiles of 128 points, each warp 2 row tiles of 16 points x all
// COUT output channels.
template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(CONV_THREADS, 4) k_conv(ConvArgs a)
{
    constexpr int S = CIN / 16, NT = COUT / 8, MT = 2;
    constexpr int WIMG = NTAP * S * NT * 32;
    using R = RowT<CIN>;
    using LT = typename R::type;
    extern __shared__ uint2 sw[];
    for (int i = threadIdx.x; i < WIMG; i += CONV_THREADS) sw[i] = a.wimg[i];
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int nym = a.ny - 1, nxm = a.nx - 1, Z = a.Z;
    const long long ntiles = (a.npts + CONV_ROWS - 1) / CONV_ROWS;
    const LT *in = reinterpret_cast<const LT *>(a.in);

    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        // the lane's four rows: r = 2*mt + half, row = base + 16 mt + 8 half + g
        int iz[4], iy[4], ix[4];
        bool ok[4];
        long long prow[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const long long p = tile * CONV_ROWS + warp * 32 + (r >> 1) * 16 + (r & 1) * 8 + g;
            ok[r] = p < a.npts;
            prow[r] = p;
            const long long pp = ok[r] ? p : 0;
            const long long col = pp / Z;
            iz[r] = (int)(pp - col * Z);
            iy[r] = (int)(col & nym);
            ix[r] = (int)(col / a.ny);
        }
        float acc[MT][NT][4];
#pragma unroll
        for (int m = 0; m < MT; ++m)
#pragma unroll
            for (int n = 0; n < NT; ++n)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[m][n][q] = 0.f;

        // the nine (dx, dy) neighbour columns in a loop that stays rolled (a
        // fully unrolled 27-tap body overflows the instruction cache); the
        // three dz taps of a column issue their loads together
#pragma unroll 1
        for (int dxy = 0; dxy < 9; ++dxy) {
            const int dx = dxy / 3 - 1, dy = dxy % 3 - 1;
            long long cb[4];
#pragma unroll
            for (int r = 0; r < 4; ++r)
                cb[r] = (long long)Z * ((long long)((iy[r] + dy) & nym) + (long long)a.ny * ((ix[r] + dx) & nxm));
            LT v[3][4];
#pragma unroll
            for (int k = 0; k < 3; ++k)
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    const int z2 = iz[r] + k - 1;
                    v[k][r] = (ok[r] && z2 >= 0 && z2 < Z) ? __ldg(in + (cb[r] + z2) * 4 + t) : R::zero();
                }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int tap = dxy * 3 + k;
#pragma unroll
                for (int s = 0; s < S; ++s) {
#pragma unroll
                    for (int n = 0; n < NT; ++n) {
                        const uint2 b = sw[((tap * S + s) * NT + n) * 32 + lane];
#pragma unroll
                        for (int m = 0; m < MT; ++m)
                            mma16816(acc[m][n], R::reg(v[k][2 * m], 2 * s), R::reg(v[k][2 * m + 1], 2 * s),
                                     R::reg(v[k][2 * m], 2 * s + 1), R::reg(v[k][2 * m + 1], 2 * s + 1), b.x, b.y);
                    }
                }
            }
        }

        // epilogue: the lane owns channels [COUT/4*t, COUT/4*(t+1)) of its rows
        constexpr int CL = COUT / 4;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            if (!ok[r]) continue;
            const int m = r >> 1, h = r & 1;
            float v[CL];
#pragma unroll
            for (int n = 0; n < NT; ++n) {
                v[2 * n] = acc[m][n][2 * h];
                v[2 * n + 1] = acc[m][n][2 * h + 1];
            }
            const long long p = prow[r];
            const int c0 = CL * t;
            if (EPI == EPI_GELU) {
                uint32_t zz[CL / 2], aa[CL / 2];
#pragma unroll
                for (int j = 0; j < CL / 2; ++j) {
                    const float z0 = v[2 * j] + a.bias[c0 + 2 * j], z1 = v[2 * j + 1] + a.bias[c0 + 2 * j + 1];
                    // the activation is formed from the rounded pre-activation,
                    // so that the backward pass differentiates what it reads
                    const float2 zr = unpack2(pack2(z0, z1));
                    zz[j] = pack2(z0, z1);
                    aa[j] = pack2(gelu_f(zr.x), gelu_f(zr.y));
                }
                if (CL == 8) {
                    *reinterpret_cast<uint4 *>(a.z + p * COUT + c0) = make_uint4(zz[0], zz[1], zz[2], zz[3]);
                    *reinterpret_cast<uint4 *>(a.act + p * COUT + c0) = make_uint4(aa[0], aa[1], aa[2], aa[3]);
                } else {
#pragma unroll
                    for (int j = 0; j < CL / 2; ++j) {
                        reinterpret_cast<uint32_t *>(a.z + p * COUT + c0)[j] = zz[j];
                        reinterpret_cast<uint32_t *>(a.act + p * COUT + c0)[j] = aa[j];
                    }
                }
            } else if (EPI == EPI_OUT) {
#pragma unroll
                for (int j = 0; j < CL; ++j) a.outf[p * COUT + c0 + j] = v[j] + a.bias[c0 + j];
            } else {
                uint32_t gg[CL / 2];
                const uint32_t *zp = reinterpret_cast<const uint32_t *>(a.zprev + p * COUT + c0);
#pragma unroll
                for (int j = 0; j < CL / 2; ++j) {
                    const float2 zf = unpack2(__ldg(zp + j));
                    gg[j] = pack2(v[2 * j] * dgelu_f(zf.x), v[2 * j + 1] * dgelu_f(zf.y));
                }
#pragma unroll
                for (int j = 0; j < CL / 2; ++j) reinterpret_cast<uint32_t *>(a.act + p * COUT + c0)[j] = gg[j];
            }
        }
    }
}

// Weight gradient of one layer, partial sums per chunk of WG_CHUNK points:
// part[chunk][tap][ci][co] = sum_p X_tap[p][ci] dZ[p][co], tap 27 = bias.
template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_wgrad(const bf16 *__restrict__ act, const bf16 *__restrict__ dz,
                                               float *__restrict__ part, int nx, int ny, int Z, long long npts)
{
    constexpr int XS = CIN * 2 + 16;  // padded row bytes: conflict-free ldmatrix
    constexpr int GS = COUT * 2 + 16;
    constexpr int MT = CIN / 16, NT = COUT / 8;
    __shared__ __align__(16) unsigned char sx[4][16 * XS];
    __shared__ __align__(16) unsigned char sg[4][16 * GS];
    __shared__ float red[4][CIN * COUT];
    const int tap = blockIdx.y;
    const long long chunk = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int dx = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dzz = tap % 3 - 1;
    const int nym = ny - 1, nxm = nx - 1;
    float acc[MT][NT][4];
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
        for (int n = 0; n < NT; ++n)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[m][n][q] = 0.f;

    const long long p0 = (chunk * 4 + warp) * (long long)(WG_KW * 16);
    unsigned char *xs = sx[warp];
    unsigned char *gs = sg[warp];
    for (int k = 0; k < WG_KW; ++k) {
        const long long pb = p0 + k * 16;
        if (pb >= npts) break;  // warp-uniform
        for (int e = lane; e < 16 * (CIN / 8); e += 32) {
            const int row = e / (CIN / 8), q = e % (CIN / 8);
            const long long p = pb + row;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (p < npts) {
                if (tap == NTAP) {
                    if (q == 0) v.x = 0x3F80u;  // BF16 1.0 in channel 0
                } else {
                    const long long col = p / Z;
                    const int iz = (int)(p - col * Z) + dzz;
                    if (iz >= 0 && iz < Z) {
                        const int iy = (int)(col & nym), ix = (int)(col / ny);
                        const long long pn =
                            iz + (long long)Z * ((long long)((iy + dy) & nym) + (long long)ny * ((ix + dx) & nxm));
                        v = __ldg(reinterpret_cast<const uint4 *>(act + pn * CIN) + q);
                    }
                }
            }
            *reinterpret_cast<uint4 *>(xs + row * XS + q * 16) = v;
        }
        for (int e = lane; e < 16 * (COUT / 8); e += 32) {
            const int row = e / (COUT / 8), q = e % (COUT / 8);
            const long long p = pb + row;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (p < npts) v = __ldg(reinterpret_cast<const uint4 *>(dz + p * COUT) + q);
            *reinterpret_cast<uint4 *>(gs + row * GS + q * 16) = v;
        }
        __syncwarp();
        const int mi = lane >> 3, mr = lane & 7;
        uint32_t A[MT][4];
#pragma unroll
        for (int m = 0; m < MT; ++m)
            ldsm_x4_trans(A[m][0], A[m][1], A[m][2], A[m][3],
                          xs + (mr + 8 * (mi >> 1)) * XS + (m * 16 + 8 * (mi & 1)) * 2);
        uint32_t B[NT][2];
#pragma unroll
        for (int n2 = 0; n2 < NT / 2; ++n2)
            ldsm_x4_trans(B[2 * n2][0], B[2 * n2][1], B[2 * n2 + 1][0], B[2 * n2 + 1][1],
                          gs + (mr + 8 * (mi & 1)) * GS + (n2 * 16 + 8 * (mi >> 1)) * 2);
#pragma unroll
        for (int m = 0; m < MT; ++m)
#pragma unroll
            for (int n = 0; n < NT; ++n) mma16816(acc[m][n], A[m][0], A[m][1], A[m][2], A[m][3], B[n][0], B[n][1]);
        __syncwarp();
    }
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
        for (int n = 0; n < NT; ++n)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int ci = m * 16 + g + 8 * (q >> 1), co = n * 8 + 2 * t + (q & 1);
                red[warp][ci * COUT + co] = acc[m][n][q];
            }
    __syncthreads();
    float *dst = part + (chunk * (NTAP + 1) + tap) * (long long)(CIN * COUT);
    for (int e = threadIdx.x; e < CIN * COUT; e += 128) dst[e] = red[0][e] + red[1][e] + red[2][e] + red[3][e];
}

// grad[e] for e < 27*cin*cout + cout (weights then bias of one layer)
__global__ void k_wgrad_reduce(const float *__restrict__ part, long long nchunk, int CIN, int COUT, int cin, int cout,
                               float *__restrict__ grad)
{
    const int n = NTAP * cin * cout + cout;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    long long src;
    if (e < NTAP * cin * cout) {
        const int tap = e / (cin * cout), rem = e % (cin * cout), ci = rem / cout, co = rem % cout;
        src = ((long long)tap * CIN + ci) * COUT + co;
    } else {
        src = (long long)NTAP * CIN * COUT + (e - NTAP * cin * cout);
    }
    const long long stride = (long long)(NTAP + 1) * CIN * COUT;
    float s = 0.f;
    for (long long c = 0; c < nchunk; ++c) s += part[c * stride + src];
    grad[e] = s;
}

// Fragment-ordered BF16 weight image of one layer (and its padded bias).
// Image entry (tap, s, n, lane) holds the B fragment registers {b0b1, b2b3}
// of k step s and n tile n: row k (0..15) of the step is input channel
// CINP/4*(k%8/2) + 4s + 2(k/8) + k%2, column j (0..7) of the tile is output
// channel COUTP/4*(j/2) + 2n + j%2.  transpose != 0 builds the backward-data
// image: input channels of the image = the layer's outputs, outputs = the
// layer's inputs, taps mirrored.
__global__ void k_wimage(const float *__restrict__ W, const float *__restrict__ b, int cin, int cout, int CINP,
                         int COUTP, int transpose, uint2 *__restrict__ img, float *__restrict__ bpad)
{
    const int S = CINP / 16, NT = COUTP / 8;
    const int total = NTAP * S * NT * 32;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (bpad && e < COUTP) bpad[e] = (!transpose && e < cout) ? b[e] : 0.f;
    if (e >= total) return;
    const int lane = e & 31;
    int rest = e >> 5;
    const int n = rest % NT;
    rest /= NT;
    const int s = rest % S;
    const int tap = rest / S;
    const int t = lane & 3, gq = lane >> 2;
    const int co = (COUTP / 4) * (gq >> 1) + 2 * n + (gq & 1);
    float w[4];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int ci = (CINP / 4) * t + 4 * s + 2 * r + j;
            float v = 0.f;
            if (!transpose) {
                if (ci < cin && co < cout) v = W[((long long)tap * cin + ci) * cout + co];
            } else {
                if (ci < cout && co < cin) v = W[((long long)(NTAP - 1 - tap) * cin + co) * cout + ci];
            }
            w[2 * r + j] = v;
        }
    img[e] = make_uint2(pack2(w[0], w[1]), pack2(w[2], w[3]));
}

// network input from 3 vorticity + 3 velocity fields of type T (pitch
// `pitch` per column, component stride cstride): channels 0-2 vor*scal[0],
// 3-5 vel*scal[1], 6-15 zero
template <typename T>
__global__ void k_pack(const T *__restrict__ vor, const T *__restrict__ vel, long long cstride, int pitch, int Z,
                       long long npts, const float *__restrict__ scal, bf16 *__restrict__ a0)
{
    const float sw = scal[0], su = scal[1];
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npts;
         p += (long long)gridDim.x * blockDim.x) {
        const long long col = p / Z;
        const long long src = (p - col * Z) + (long long)pitch * col;
        const float v0 = (float)vor[src] * sw, v1 = (float)vor[src + cstride] * sw, v2 = (float)vor[src + 2 * cstride] * sw;
        const float u0 = (float)vel[src] * su, u1 = (float)vel[src + cstride] * su, u2 = (float)vel[src + 2 * cstride] * su;
        uint4 *dst = reinterpret_cast<uint4 *>(a0 + p * 16);
        dst[0] = make_uint4(pack2(v0, v1), pack2(v2, u0), pack2(u1, u2), 0u);
        dst[1] = make_uint4(0u, 0u, 0u, 0u);
    }
}

// correction fields out[c] (type T, pitch, component stride) = outf[p][c] * scal[2].
// flags (PS3D_CLOSURE_*): CLIP zeroes the correction at points where it
// would raise the local enstrophy (vor . corr > 0, backscatter); WALLS
// zeroes its horizontal components on the walls (free slip: xi = eta = 0)
template <typename T>
__global__ void k_unpack(const float *__restrict__ outf, const float *__restrict__ scal, const T *__restrict__ vor,
                         long long vstride, int Z, long long npts, int pitch, long long ostride, int flags,
                         T *__restrict__ out)
{
    const float s = scal[2];
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npts;
         p += (long long)gridDim.x * blockDim.x) {
        const long long col = p / Z;
        const int iz = (int)(p - col * Z);
        const long long dst = iz + (long long)pitch * col;
        const float *o = outf + p * CPAD_OUT[NL - 1];
        float c0 = o[0] * s, c1 = o[1] * s, c2 = o[2] * s;
        if (flags & PS3D_CLOSURE_WALLS) {
            if (iz == 0 || iz == Z - 1) c0 = c1 = 0.f;
        }
        if (flags & PS3D_CLOSURE_CLIP) {
            // the sign test in the field's precision
            const T w = vor[dst] * (T)c0 + vor[dst + vstride] * (T)c1 + vor[dst + 2 * vstride] * (T)c2;
            if (w > (T)0) c0 = c1 = c2 = 0.f;
        }
        out[dst] = (T)c0;
        out[dst + ostride] = (T)c1;
        out[dst + 2 * ostride] = (T)c2;
    }
}

__device__ __forceinline__ double block_sum(double v, double *sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
    return s;  // valid in thread 0
}

// sums of |vor|^2 and |vel|^2 over the grid points, per block
template <typename T>
__global__ void k_sumsq(const T *__restrict__ vor, const T *__restrict__ vel, long long cstride, int pitch, int Z,
                        long long npts, double *__restrict__ part)
{
    __shared__ double sh[32];
    double sw = 0.0, su = 0.0;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npts;
         p += (long long)gridDim.x * blockDim.x) {
        const long long col = p / Z;
        const long long src = (p - col * Z) + (long long)pitch * col;
        for (int c = 0; c < 3; ++c) {
            const double w = (double)vor[src + c * cstride], u = (double)vel[src + c * cstride];
            sw += w * w;
            su += u * u;
        }
    }
    const double a = block_sum(sw, sh);
    const double b = block_sum(su, sh);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
    }
}

// scal[0] = 1/rms(vor), scal[1] = 1/rms(vel), scal[2] = ct * <|vor|^2>
// (ct read from device memory, so that captured launches follow a change)
__global__ void k_scal_finish(const double *__restrict__ part, int nblocks, long long npts, const double *ctp,
                              float *__restrict__ scal)
{
    __shared__ double sh[32];
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
        a += part[2 * i];
        b += part[2 * i + 1];
    }
    a = block_sum(a, sh);
    b = block_sum(b, sh);
    if (threadIdx.x == 0) {
        const double w2 = a / (double)npts, u2 = b / (double)npts;
        scal[0] = w2 > 0.0 ? (float)(1.0 / sqrt(w2)) : 0.f;
        scal[1] = u2 > 0.0 ? (float)(1.0 / sqrt(u2)) : 0.f;
        scal[2] = (float)(*ctp * w2);
    }
}

// mean squared error against the normalised target and its gradient dz4
// (channels 0-2, the rest zero); per-block partial sums of the squares
__global__ void k_loss(const float *__restrict__ outf, const float *__restrict__ tgt, const float *__restrict__ sscal,
                       long long npts, bf16 *__restrict__ dz4, double *__restrict__ part)
{
    __shared__ double sh[32];
    const float ts = sscal[2];
    const float gs = 2.0f / (3.0f * (float)npts);
    double acc = 0.0;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npts;
         p += (long long)gridDim.x * blockDim.x) {
        const float *o = outf + p * CPAD_OUT[NL - 1];
        const float d0 = o[0] - tgt[p] * ts, d1 = o[1] - tgt[npts + p] * ts, d2 = o[2] - tgt[2 * npts + p] * ts;
        acc += (double)d0 * d0 + (double)d1 * d1 + (double)d2 * d2;
        uint4 *dst = reinterpret_cast<uint4 *>(dz4 + p * CPAD_DZ4);
        dst[0] = make_uint4(pack2(gs * d0, gs * d1), pack2(gs * d2, 0.f), 0u, 0u);
        dst[1] = make_uint4(0u, 0u, 0u, 0u);
    }
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_loss_finish(const double *__restrict__ part, int nblocks, double scale, double *__restrict__ out)
{
    __shared__ double sh[32];
    double a = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) a += part[i];
    a = block_sum(a, sh);
    if (threadIdx.x == 0) *out = a * scale;
}

__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, int n, float lr, float b1, float b2, float c1, float c2, float eps)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

// ===================================================== tcgen05 inference path
// The forward pass on the 5th-generation tensor cores.  Activations live in a
// padded, channel-chunk-planar layout: padded row r = GUARD + (iz+1) +
// ZP*((iy+1) + YP*(ix+1)) (ZP = nz+3, YP = ny+2), chunk plane kc (8 channels,
// 16 bytes) at byte (kc*RTOT + r)*16.  Ghost rows at iz = -1, nz+1 stay zero
// (the z zero padding); ghost rows at iy = -1, ny and ix = -1, nx hold the
// periodic copies, written by the producer of each activation; GUARD rows
// before and after keep every load of a tile in bounds.  Every tap is then a
// uniform shift of the row index, so one tile of 128 output rows needs, per x
// shift dx, one contiguous run of 128 + 2(ZP+1) rows per chunk plane: 3 x KC
// one-dimensional TMA bulk copies.  The 27 taps x CIN/16 k-steps are
// tcgen05.mma (M 128, N = COUT, K 16, BF16 in, FP32 accumulate in TMEM)
// issued by one thread from shared-memory descriptors shifted by
// (ZP*dy + dz) rows (no-swizzle K-major core matrices: 8 rows x 16 bytes,
// SBO 128 bytes between row groups, LBO one chunk plane); the epilogue reads
// the accumulator with tcgen05.ld (one TMEM lane per thread = one output row).

struct TcArgs {
    const unsigned char *in;   // padded chunk-planar input (CIN/8 planes)
    const uint4 *wimg;         // [tap][kc][co] x 16 bytes
    const float *bias;         // [COUT]
    unsigned char *out;        // EPI_GELU: padded chunk-planar activation
    float *outf;               // EPI_OUT: [npts][CPAD_OUT] FP32
    int *err;                  // device error word (bounded waits)
    int nx, ny, Z, ZP, YP;
    long long QN, RTOT, GUARD, npts;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    // sm_100-family shared-memory matrix descriptor, no swizzle
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version
    return d;
}

template <int COUT> __host__ __device__ constexpr uint32_t tc_idesc()
{
    // kind::f16: D F32 (bits 4-5 = 1), A BF16 (7-9 = 1), B BF16 (10-12 = 1),
    // both K-major, N >> 3 at 17-22, M >> 4 at 24-28 (M = 128)
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(COUT >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(a), "r"(bytes) : "memory");
}
// bounded wait for the completion of the phase with the given parity: a
// non-blocking test with a short sleep, at most 2^21 rounds (about a second)
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity)
{
    for (int i = 0; i < (1 << 21); ++i) {
        uint32_t ok;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
        if (i > 64) __nanosleep(256);
    }
    return false;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}
__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void tc_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// 16 / 8 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tc_ld8(uint32_t taddr, float *v)
{
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// padded row of point (ix, iy, iz) with x / y shifts (ghost copies)
__device__ __forceinline__ long long tc_row(long long G, int ZP, int YP, int ixp, int iyp, int iz)
{
    return G + (iz + 1) + (long long)ZP * (iyp + (long long)YP * ixp);
}

// write the 16-byte chunks v[kc] of interior point (ix, iy, iz) to its row
// and to the periodic ghost rows that mirror it
template <int KC>
__device__ __forceinline__ void tc_store_point(unsigned char *base, long long RTOT, long long G, int ZP, int YP, int nx,
                                               int ny, int ix, int iy, int iz, const uint4 *v, int kc0 = 0)
{
    // the point itself, then its ghost copies (x edge, y edge, corner)
    const int xg = ix == 0 ? nx + 1 : (ix == nx - 1 ? 0 : -1);
    const int yg = iy == 0 ? ny + 1 : (iy == ny - 1 ? 0 : -1);
    auto put = [&](int xp, int yp) {
        const long long r = tc_row(G, ZP, YP, xp, yp, iz);
#pragma unroll
        for (int kc = 0; kc < KC; ++kc) *reinterpret_cast<uint4 *>(base + ((long long)(kc0 + kc) * RTOT + r) * 16) = v[kc];
    };
    put(ix + 1, iy + 1);
    if (xg >= 0) put(xg, iy + 1);
    if (yg >= 0) put(ix + 1, yg);
    if (xg >= 0 && yg >= 0) put(xg, yg);
}

// network input in the padded layout (channels 0-2 vor*scal[0], 3-5
// vel*scal[1], 6-15 zero; two chunk planes)
template <typename T>
__global__ void k_pack_pad(const T *__restrict__ vor, const T *__restrict__ vel, long long cstride, int pitch, int nx,
                           int ny, int Z, int ZP, int YP, long long RTOT, long long G, long long npts,
                           const float *__restrict__ scal, unsigned char *__restrict__ a0)
{
    const float sw = scal[0], su = scal[1];
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npts;
         p += (long long)gridDim.x * blockDim.x) {
        const long long col = p / Z;
        const int iz = (int)(p - col * Z), iy = (int)(col % ny), ix = (int)(col / ny);
        const long long src = iz + (long long)pitch * col;
        const float v0 = (float)vor[src] * sw, v1 = (float)vor[src + cstride] * sw, v2 = (float)vor[src + 2 * cstride] * sw;
        const float u0 = (float)vel[src] * su, u1 = (float)vel[src + cstride] * su, u2 = (float)vel[src + 2 * cstride] * su;
        uint4 v[2];
        v[0] = make_uint4(pack2(v0, v1), pack2(v2, u0), pack2(u1, u2), 0u);
        v[1] = make_uint4(0u, 0u, 0u, 0u);
        tc_store_point<2>(a0, RTOT, G, ZP, YP, nx, ny, ix, iy, iz, v);
    }
}

// [tap][kc][co] x 8 BF16 weight image of one layer for the tcgen05 kernel
__global__ void k_wimage_tc(const float *__restrict__ W, int cin, int cout, int CINP, int COUTP, uint4 *__restrict__ img)
{
    const int KC = CINP / 8;
    const int total = NTAP * KC * COUTP;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total) return;
    const int co = e % COUTP, kc = (e / COUTP) % KC, tap = e / (COUTP * KC);
    float w[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int ci = kc * 8 + j;
        w[j] = (ci < cin && co < cout) ? W[((long long)tap * cin + ci) * cout + co] : 0.f;
    }
    img[e] = make_uint4(pack2(w[0], w[1]), pack2(w[2], w[3]), pack2(w[4], w[5]), pack2(w[6], w[7]));
}

template <int CIN, int COUT> __host__ __device__ constexpr int tc_wbytes() { return NTAP * (CIN / 8) * COUT * 16; }
__host__ __device__ inline int tc_seg(int ZP) { return 128 + 2 * (ZP + 1); }
// weights + two tile buffers of 3 x CIN/8 chunk planes
template <int CIN, int COUT> __host__ __device__ inline size_t tc_smem(int ZP)
{
    return (size_t)tc_wbytes<CIN, COUT>() + (size_t)2 * 3 * (CIN / 8) * tc_seg(ZP) * 16;
}

// epilogue of one tile for one output row and one half of the accumulator
// columns (v: COUT/2 values from column half*COUT/2): bias + GELU into the
// padded activation (with its ghost copies), or, for half 0 of the output
// layer, bias only into the FP32 output
template <int COUT, int EPI>
__device__ __forceinline__ void tc_epilogue(const TcArgs &a, const float *bias, unsigned q, int half, const float *v)
{
    if ((long long)q >= a.QN) return;
    const unsigned ZP = (unsigned)a.ZP, YP = (unsigned)a.YP;
    const unsigned t1 = q / ZP;
    const int iz = (int)(q - t1 * ZP) - 1, iy = (int)(t1 % YP) - 1, ix = (int)(t1 / YP) - 1;
    if (iz < 0 || iz >= a.Z || iy < 0 || iy >= a.ny || ix < 0 || ix >= a.nx) return;
    constexpr int H = COUT / 2;
    if (EPI == EPI_GELU) {
        uint4 o[H / 8];
#pragma unroll
        for (int k = 0; k < H / 8; ++k) {
            uint32_t w4[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = half * H + 8 * k + 2 * j;
                const float2 zr = unpack2(pack2(v[8 * k + 2 * j] + bias[c], v[8 * k + 2 * j + 1] + bias[c + 1]));
                w4[j] = pack2(gelu_f(zr.x), gelu_f(zr.y));
            }
            o[k] = make_uint4(w4[0], w4[1], w4[2], w4[3]);
        }
        tc_store_point<H / 8>(a.out, a.RTOT, a.GUARD, a.ZP, a.YP, a.nx, a.ny, ix, iy, iz, o, half * (H / 8));
    } else if (half == 0) {
        const long long p = iz + (long long)a.Z * (iy + (long long)a.ny * ix);
        float *o = a.outf + p * OUTC;
#pragma unroll
        for (int j = 0; j < OUTC; ++j) o[j] = v[j] + bias[j];
    }
}

__device__ __forceinline__ void mbar_arrive(uint32_t a)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(a) : "memory");
}

// One convolution layer over the padded grid, warp-specialised.  Persistent
// CTAs of 9 warps walk tiles of 128 padded rows.  Warp 8 (one elected lane)
// is the producer and issuer: TMA copies of tile k+1 into the shared buffer
// freed by the products of tile k-1, and the 27 x CIN/16 tcgen05.mma of tile
// k into TMEM accumulator k%2 once the epilogue has released it.  Warps 0-7
// are the epilogue: they wait for the products of tile k, read their lane
// quarter (warp % 4) and column half (warp / 4) of the accumulator, release
// it, and apply bias + GELU and the stores.  The roles meet only on
// mbarriers: full[b] (copies landed), done[b] (products complete, tcgen05.
// commit), free[b] (256 epilogue arrivals).  Every wait is bounded; a wait
// that runs out sets a shared flag that stops both roles, raises the error
// word, and the issuer lets its operations in flight finish (bounded) before
// the accumulator is released.
template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(288, 1) k_conv_tc(TcArgs a)
{
    constexpr int KC = CIN / 8, S = CIN / 16;
    constexpr int WB = tc_wbytes<CIN, COUT>();
    constexpr uint32_t IDESC = tc_idesc<COUT>();
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar[6];  // full[0..1], done[2..3], free[4..5]
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int bad;
    __shared__ float sbias[32];
    unsigned char *sW = smem;
    unsigned char *sA = smem + WB;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ZP = a.ZP;
    const uint32_t segb = (uint32_t)tc_seg(ZP) * 16u;
    const uint32_t abuf = (uint32_t)(3 * KC) * segb;
    const long long plane = (long long)ZP * a.YP;

    if (tid < 32) sbias[tid] = tid < COUT ? a.bias[tid] : 0.f;
    if (tid == 0) {
        for (int i = 0; i < 4; ++i) mbar_init(smem_u32(&mbar[i]), 1);
        mbar_init(smem_u32(&mbar[4]), 256);
        mbar_init(smem_u32(&mbar[5]), 256);
        bad = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 8) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;\n" ::"r"(smem_u32(&tmem_slot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    for (int i = tid; i < WB / 16; i += 288) reinterpret_cast<uint4 *>(sW)[i] = __ldg(a.wimg + i);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const long long ntiles = (a.QN + 127) / 128;
    const long long nk = ntiles > (long long)blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    auto tile_q0 = [&](long long k) { return ((long long)blockIdx.x + k * (long long)gridDim.x) * 128; };

    if (warp == 8) {
        if (lane == 0) {
            const uint32_t sAu = smem_u32(sA), sWu = smem_u32(sW);
            const uint64_t bd0 = tc_desc(sWu, COUT * 16u, 128u);
            const int seg = (int)(segb >> 4);
            // phase parities and pending operations as bit masks (bit i:
            // barrier i; pending bits 0-3: copies into buffer 0/1, products
            // into accumulator 0/1), kept in registers
            uint32_t ph = 0u, pend = 0u;
            auto wait_bar = [&](int i) {
                if (mbar_wait(smem_u32(&mbar[i]), (ph >> i) & 1u)) {
                    ph ^= 1u << i;
                    pend &= ~(1u << i);
                    return true;
                }
                bad = 1;
                return false;
            };
            auto issue_load = [&](long long k) {
                const int b = (int)(k & 1);
                const uint32_t mb = smem_u32(&mbar[b]);
                pend |= 1u << b;
                mbar_expect_tx(mb, abuf);
                const long long q0 = tile_q0(k);
                for (int dxi = 0; dxi < 3; ++dxi) {
                    const long long r0 = a.GUARD + q0 + (dxi - 1) * plane - (ZP + 1);
                    for (int kc = 0; kc < KC; ++kc)
                        bulk_g2s(sAu + (uint32_t)b * abuf + (uint32_t)(dxi * KC + kc) * segb,
                                 a.in + ((long long)kc * a.RTOT + r0) * 16, segb, mb);
                }
            };
            if (nk > 0) issue_load(0);
            for (long long k = 0; k < nk && !bad; ++k) {
                const int b = (int)(k & 1);
                if (!wait_bar(b)) break;                          // tile k in shared memory
                if (k >= 2 && !wait_bar(4 + b)) break;            // epilogue of tile k-2 released accumulator b
                tc_fence_after();
                const uint32_t acc = tmem + (uint32_t)(b * 32);
                // descriptors = base descriptor + start offset in 16-byte units
                // (the 14-bit start field cannot carry below 256 KB)
                const uint64_t ad0 = tc_desc(sAu + (uint32_t)b * abuf, segb, 128u);
#pragma unroll
                for (int dxi = 0; dxi < 3; ++dxi)
#pragma unroll
                    for (int dyi = 0; dyi < 3; ++dyi)
#pragma unroll
                        for (int dzi = 0; dzi < 3; ++dzi)
#pragma unroll
                            for (int s2 = 0; s2 < S; ++s2) {
                                const int tap = dxi * 9 + dyi * 3 + dzi;
                                // row offset of the tap in the tile buffer, >= 0
                                const int off = (dxi * KC + 2 * s2) * seg + (ZP + 1) + ZP * (dyi - 1) + (dzi - 1);
                                const uint64_t ad = ad0 + (uint64_t)(uint32_t)off;
                                const uint64_t bd = bd0 + (uint64_t)((tap * KC + 2 * s2) * COUT);
                                tc_mma(acc, ad, bd, IDESC, (tap | s2) != 0 ? 1u : 0u);
                            }
                pend |= 1u << (2 + b);
                tc_commit(smem_u32(&mbar[2 + b]));
                if (k + 1 < nk) {
                    // buffer 1-b is free once the products of tile k-1 are complete
                    if (k >= 1 && !wait_bar(2 + (1 - b))) break;
                    issue_load(k + 1);
                }
            }
            if (bad) {
                atomicOr(a.err, 1);
                for (int i = 0; i < 4; ++i)
                    if ((pend >> i) & 1u) mbar_wait(smem_u32(&mbar[i]), (ph >> i) & 1u);
            } else if (nk > 0) {
                // the last tile's products (the epilogue waits for them too)
                const int b = (int)((nk - 1) & 1);
                if ((pend >> (2 + b)) & 1u) wait_bar(2 + b);
            }
        }
    } else {
        const int quarter = warp & 3, half = warp >> 2;
        uint32_t ph_done = 0u;  // bit b: phase parity of done[b]
        for (long long k = 0; k < nk; ++k) {
            // warp-uniform decisions: the TMEM load below is warp-collective
            if (__any_sync(0xffffffffu, bad != 0)) break;
            const int b = (int)(k & 1);
            const bool ok = mbar_wait(smem_u32(&mbar[2 + b]), (ph_done >> b) & 1u);
            if (!__all_sync(0xffffffffu, ok)) {
                bad = 1;
                break;
            }
            ph_done ^= 1u << b;
            tc_fence_after();
            float v[16];
            const uint32_t taddr = tmem + (uint32_t)(b * 32 + half * (COUT / 2)) + ((uint32_t)(quarter * 32) << 16);
            if (COUT == 32) tc_ld16(taddr, v);
            else tc_ld8(taddr, v);
            tc_fence_before();
            mbar_arrive(smem_u32(&mbar[4 + b]));  // accumulator b may take the products of tile k+2
            tc_epilogue<COUT, EPI>(a, sbias, (unsigned)(tile_q0(k) + quarter * 32 + lane), half, v);
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 8) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;\n" ::"r"(tmem) : "memory");
}

// host-side SplitMix64 (parameter initialisation, sample order)
struct SplitMix {
    unsigned long long s;
    unsigned long long next()
    {
        unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

}  // namespace

// ======================================================================
struct ps3d_closure {
    int nx = 0, ny = 0, nz = 0, Z = 0, device = 0, nsm = 0;
    long long npts = 0, nchunk = 0;
    cudaStream_t st = nullptr;
    std::string err;
    std::vector<void *> allocs;
    const void *owner = nullptr;  // attached context
    // parameters, gradients, Adam moments (FP32, NPARAM)
    float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    uint2 *imgf[NL] = {}, *imgb[NL] = {};  // forward images; backward-data images (layers 1..3)
    float *bpad[NL] = {};
    // activations
    bf16 *a0 = nullptr, *z[3] = {}, *act[3] = {}, *dz4 = nullptr, *dzA = nullptr, *dzB = nullptr;
    float *outf = nullptr, *wpart = nullptr, *scal = nullptr;
    double *rpart = nullptr, *lpart = nullptr, *lossd = nullptr;
    double *ctd = nullptr;   // ct in device memory; lpart[RED_BLOCKS]: one loss value
    // tcgen05 inference path: padded chunk-planar activations (input, two
    // ping-pong hidden buffers), weight images, device error word
    int engine = 0, tc_ok = 0, tc_occ[3] = {1, 1, 1};
    int ZP = 0, YP = 0;
    long long QN = 0, RTOT = 0, GUARD = 0;
    unsigned char *pa0 = nullptr, *pact[2] = {};
    uint4 *imgtc[NL] = {};
    int *derr = nullptr;
    int occ[5] = {1, 1, 1, 1, 1};  // resident conv blocks per SM per instantiation
    int loss_cap = 0;
    double *host_out = nullptr;   // predict staging (device)
    double *host_in = nullptr;    // 6 fields FP64 staging (device)
    // training samples: per sample 9 fields FP32 [vor 3, vel 3, target 3][npts]
    int max_samples = 0, nsamples = 0;
    float *data = nullptr;
    float *sscal = nullptr;  // per sample {1/rms(vor), 1/rms(vel), 1/(ct <|vor|^2>), 0}
    std::vector<double> w2, u2, t2;
    double ct = 0.0;
    long long adam_t = 0;
    SplitMix rng{0};
};

namespace {

int cfail(ps3d_closure *cl, int code, const std::string &msg)
{
    if (cl) cl->err = msg;
    return code;
}
int ccheck(ps3d_closure *cl, const char *where)
{
    const cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return PS3D_OK;
    return cfail(cl, PS3D_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
template <typename P> bool calloc_dev(ps3d_closure *cl, P **p, size_t bytes)
{
    void *q = nullptr;
    if (cudaMalloc(&q, bytes) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaMemset(q, 0, bytes);
    cl->allocs.push_back(q);
    *p = reinterpret_cast<P *>(q);
    return true;
}

template <int CIN, int COUT, int EPI> size_t conv_smem() { return (size_t)NTAP * (CIN / 16) * (COUT / 8) * 32 * 8; }

template <int CIN, int COUT, int EPI> constexpr int conv_slot()
{
    return EPI == EPI_OUT ? 2 : EPI == EPI_BWD ? (CIN == 16 ? 3 : 4) : (CIN == 16 ? 0 : 1);
}

template <int CIN, int COUT, int EPI> void conv_attr(ps3d_closure *cl)
{
    cudaFuncSetAttribute(k_conv<CIN, COUT, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)conv_smem<CIN, COUT, EPI>());
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_conv<CIN, COUT, EPI>, CONV_THREADS,
                                                      conv_smem<CIN, COUT, EPI>()) != cudaSuccess || nb < 1) {
        cudaGetLastError();
        nb = 1;
    }
    cl->occ[conv_slot<CIN, COUT, EPI>()] = nb;
}

// persistent grid: at most one wave of resident blocks, the tiles spread
// evenly over it
template <int CIN, int COUT, int EPI> void conv(ps3d_closure *cl, cudaStream_t st, const ConvArgs &a)
{
    const long long ntiles = (cl->npts + CONV_ROWS - 1) / CONV_ROWS;
    const long long maxb = (long long)cl->nsm * cl->occ[conv_slot<CIN, COUT, EPI>()];
    const long long per = (ntiles + maxb - 1) / maxb;
    const unsigned grid = (unsigned)((ntiles + per - 1) / per);
    k_conv<CIN, COUT, EPI><<<grid, CONV_THREADS, conv_smem<CIN, COUT, EPI>(), st>>>(a);
}

ConvArgs base_args(ps3d_closure *cl)
{
    ConvArgs a{};
    a.nx = cl->nx;
    a.ny = cl->ny;
    a.Z = cl->Z;
    a.npts = cl->npts;
    return a;
}

void forward(ps3d_closure *cl, cudaStream_t st);

TcArgs tc_args(ps3d_closure *cl)
{
    TcArgs a{};
    a.err = cl->derr;
    a.nx = cl->nx;
    a.ny = cl->ny;
    a.Z = cl->Z;
    a.ZP = cl->ZP;
    a.YP = cl->YP;
    a.QN = cl->QN;
    a.RTOT = cl->RTOT;
    a.GUARD = cl->GUARD;
    a.npts = cl->npts;
    return a;
}

template <int CIN, int COUT, int EPI> constexpr int tc_slot() { return EPI == EPI_OUT ? 2 : (CIN == 16 ? 0 : 1); }

template <int CIN, int COUT, int EPI> bool tc_attr(ps3d_closure *cl)
{
    const size_t sm = tc_smem<CIN, COUT>(cl->ZP);
    if (cudaFuncSetAttribute(k_conv_tc<CIN, COUT, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
        cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_conv_tc<CIN, COUT, EPI>, 288, sm) != cudaSuccess ||
        nb < 1) {
        cudaGetLastError();
        return false;
    }
    cl->tc_occ[tc_slot<CIN, COUT, EPI>()] = nb;
    return true;
}

template <int CIN, int COUT, int EPI> void conv_tc(ps3d_closure *cl, cudaStream_t st, const TcArgs &a)
{
    const long long ntiles = (cl->QN + 127) / 128;
    const long long maxb = (long long)cl->nsm * cl->tc_occ[tc_slot<CIN, COUT, EPI>()];
    const long long per = (ntiles + maxb - 1) / maxb;
    const unsigned grid = (unsigned)((ntiles + per - 1) / per);
    k_conv_tc<CIN, COUT, EPI><<<grid, 288, tc_smem<CIN, COUT>(cl->ZP), st>>>(a);
}

// tcgen05 forward pass: pa0 -> pact[0] -> pact[1] -> pact[0] -> outf
void forward_tc(ps3d_closure *cl, cudaStream_t st)
{
    TcArgs a = tc_args(cl);
    a.in = cl->pa0;
    a.wimg = cl->imgtc[0];
    a.bias = cl->bpad[0];
    a.out = cl->pact[0];
    conv_tc<16, 32, EPI_GELU>(cl, st, a);
    a.in = cl->pact[0];
    a.wimg = cl->imgtc[1];
    a.bias = cl->bpad[1];
    a.out = cl->pact[1];
    conv_tc<32, 32, EPI_GELU>(cl, st, a);
    a.in = cl->pact[1];
    a.wimg = cl->imgtc[2];
    a.bias = cl->bpad[2];
    a.out = cl->pact[0];
    conv_tc<32, 32, EPI_GELU>(cl, st, a);
    a.in = cl->pact[0];
    a.wimg = cl->imgtc[3];
    a.bias = cl->bpad[3];
    a.out = nullptr;
    a.outf = cl->outf;
    conv_tc<32, 16, EPI_OUT>(cl, st, a);
}

// input packing and forward pass of the selected engine
template <typename T>
void pack_forward(ps3d_closure *cl, cudaStream_t st, const T *vor, const T *vel, long long cstride, int pitch)
{
    if (cl->engine == 1) {
        k_pack_pad<T><<<RED_BLOCKS * 4, RED_THREADS, 0, st>>>(vor, vel, cstride, pitch, cl->nx, cl->ny, cl->Z, cl->ZP,
                                                            cl->YP, cl->RTOT, cl->GUARD, cl->npts, cl->scal, cl->pa0);
        forward_tc(cl, st);
    } else {
        k_pack<T><<<RED_BLOCKS * 4, RED_THREADS, 0, st>>>(vor, vel, cstride, pitch, cl->Z, cl->npts, cl->scal, cl->a0);
        forward(cl, st);
    }
}

// four layers: a0 -> z1/a1 -> z2/a2 -> z3/a3 -> outf
void forward(ps3d_closure *cl, cudaStream_t st)
{
    ConvArgs a = base_args(cl);
    a.in = cl->a0;
    a.wimg = cl->imgf[0];
    a.bias = cl->bpad[0];
    a.z = cl->z[0];
    a.act = cl->act[0];
    conv<16, 32, EPI_GELU>(cl, st, a);
    for (int l = 1; l < 3; ++l) {
        a.in = cl->act[l - 1];
        a.wimg = cl->imgf[l];
        a.bias = cl->bpad[l];
        a.z = cl->z[l];
        a.act = cl->act[l];
        conv<32, 32, EPI_GELU>(cl, st, a);
    }
    a.in = cl->act[2];
    a.wimg = cl->imgf[3];
    a.bias = cl->bpad[3];
    a.z = nullptr;
    a.act = nullptr;
    a.outf = cl->outf;
    conv<32, 8, EPI_OUT>(cl, st, a);
}

template <int CIN, int COUT> void wgrad(ps3d_closure *cl, cudaStream_t st, const bf16 *act, const bf16 *dz, int l)
{
    dim3 grid((unsigned)cl->nchunk, NTAP + 1);
    k_wgrad<CIN, COUT><<<grid, 128, 0, st>>>(act, dz, cl->wpart, cl->nx, cl->ny, cl->Z, cl->npts);
    const int n = NTAP * CREAL_IN[l] * CREAL_OUT[l] + CREAL_OUT[l];
    k_wgrad_reduce<<<(n + 255) / 256, 256, 0, st>>>(cl->wpart, cl->nchunk, CIN, COUT, CREAL_IN[l], CREAL_OUT[l],
                                                    cl->g + woff(l));
}

// backward pass after forward + k_loss (dz4 holds dL/dout): all parameter
// gradients into cl->g
void backward(ps3d_closure *cl, cudaStream_t st)
{
    wgrad<32, 16>(cl, st, cl->act[2], cl->dz4, 3);
    ConvArgs a = base_args(cl);
    // dz3 = (W4^T * dz4) . gelu'(z3)
    a.in = cl->dz4;
    a.wimg = cl->imgb[3];
    a.zprev = cl->z[2];
    a.act = cl->dzA;
    conv<16, 32, EPI_BWD>(cl, st, a);
    wgrad<32, 32>(cl, st, cl->act[1], cl->dzA, 2);
    // dz2 = (W3^T * dz3) . gelu'(z2)
    a.in = cl->dzA;
    a.wimg = cl->imgb[2];
    a.zprev = cl->z[1];
    a.act = cl->dzB;
    conv<32, 32, EPI_BWD>(cl, st, a);
    wgrad<32, 32>(cl, st, cl->act[0], cl->dzB, 1);
    // dz1 = (W2^T * dz2) . gelu'(z1)
    a.in = cl->dzB;
    a.wimg = cl->imgb[1];
    a.zprev = cl->z[0];
    a.act = cl->dzA;
    conv<32, 32, EPI_BWD>(cl, st, a);
    wgrad<16, 32>(cl, st, cl->a0, cl->dzA, 0);
}

// rebuild the BF16 images from the FP32 master parameters
void images(ps3d_closure *cl, cudaStream_t st)
{
    for (int l = 0; l < NL; ++l) {
        const float *W = cl->w + woff(l);
        const float *b = W + NTAP * CREAL_IN[l] * CREAL_OUT[l];
        const int nf = NTAP * (CPAD_IN[l] / 16) * (CPAD_OUT[l] / 8) * 32;
        k_wimage<<<(nf + 255) / 256, 256, 0, st>>>(W, b, CREAL_IN[l], CREAL_OUT[l], CPAD_IN[l], CPAD_OUT[l], 0,
                                                  cl->imgf[l], cl->bpad[l]);
        if (l > 0) {
            const int cinp = l == NL - 1 ? CPAD_DZ4 : CPAD_OUT[l];
            const int nb = NTAP * (cinp / 16) * (CPAD_IN[l] / 8) * 32;
            k_wimage<<<(nb + 255) / 256, 256, 0, st>>>(W, b, CREAL_IN[l], CREAL_OUT[l], cinp, CPAD_IN[l], 1,
                                                      cl->imgb[l], nullptr);
        }
        if (cl->tc_ok) {
            const int coutp = l == NL - 1 ? 16 : CPAD_OUT[l];
            const int nt = NTAP * (CPAD_IN[l] / 8) * coutp;
            k_wimage_tc<<<(nt + 255) / 256, 256, 0, st>>>(W, CREAL_IN[l], CREAL_OUT[l], CPAD_IN[l], coutp,
                                                         cl->imgtc[l]);
        }
    }
}

// pack stored sample s into a0
void pack_sample(ps3d_closure *cl, cudaStream_t st, int s)
{
    const float *base = cl->data + (size_t)s * 9 * cl->npts;
    k_pack<float><<<RED_BLOCKS * 4, RED_THREADS, 0, st>>>(base, base + 3 * cl->npts, cl->npts, cl->Z, cl->Z,
                                                         cl->npts, cl->sscal + 4 * s, cl->a0);
}

void loss_and_grad(ps3d_closure *cl, cudaStream_t st, int s, double *loss_dst)
{
    const float *tgt = cl->data + (size_t)s * 9 * cl->npts + 6 * cl->npts;
    k_loss<<<RED_BLOCKS, RED_THREADS, 0, st>>>(cl->outf, tgt, cl->sscal + 4 * s, cl->npts, cl->dz4, cl->lpart);
    k_loss_finish<<<1, RED_THREADS, 0, st>>>(cl->lpart, RED_BLOCKS, 1.0 / (3.0 * (double)cl->npts), loss_dst);
}

// per-sample scalars from the current ct
void upload_sample_scalars(ps3d_closure *cl)
{
    std::vector<float> h(4 * (size_t)cl->nsamples);
    for (int s = 0; s < cl->nsamples; ++s) {
        h[4 * s + 0] = cl->w2[s] > 0 ? (float)(1.0 / std::sqrt(cl->w2[s])) : 0.f;
        h[4 * s + 1] = cl->u2[s] > 0 ? (float)(1.0 / std::sqrt(cl->u2[s])) : 0.f;
        h[4 * s + 2] = (cl->ct > 0 && cl->w2[s] > 0) ? (float)(1.0 / (cl->ct * cl->w2[s])) : 0.f;
        h[4 * s + 3] = 0.f;
    }
    if (!h.empty()) cudaMemcpy(cl->sscal, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice);
}

int centre(ps3d_closure *cl)
{
    if (!cl) return PS3D_ERR_INVALID_ARG;
    if (cudaSetDevice(cl->device) != cudaSuccess) return ccheck(cl, "cudaSetDevice");
    return PS3D_OK;
}

// mean squares over the points of 3-component host fields
double mean_sq3(const double *f, long long npts)
{
    double s = 0.0;
    for (long long i = 0; i < 3 * npts; ++i) s += f[i] * f[i];
    return s / (double)npts;
}

}  // namespace

// ---------------------------------------------------- internal interface
namespace ps3d {

int closure_attach(ps3d_closure *cl, const void *owner, int nx, int ny, int nz, int device, std::string *err)
{
    if (cl->owner && cl->owner != owner) {
        *err = "closure already attached to another context";
        return PS3D_ERR_INVALID_ARG;
    }
    if (cl->nx != nx || cl->ny != ny || cl->nz != nz || cl->device != device) {
        *err = "closure grid or device differs from the context's";
        return PS3D_ERR_INVALID_ARG;
    }
    if (!(cl->ct > 0.0)) {
        *err = "closure output scale not set (train or set_scale first)";
        return PS3D_ERR_NOT_READY;
    }
    cl->owner = owner;
    return PS3D_OK;
}

void closure_detach(ps3d_closure *cl, const void *owner)
{
    if (cl && cl->owner == owner) cl->owner = nullptr;
}

template <typename T>
int closure_apply(ps3d_closure *cl, cudaStream_t st, const T *vor, const T *vel, long long cstride, int pitch, T *out,
                  long long ostride, int flags)
{
    k_sumsq<T><<<RED_BLOCKS, RED_THREADS, 0, st>>>(vor, vel, cstride, pitch, cl->Z, cl->npts, cl->rpart);
    k_scal_finish<<<1, RED_THREADS, 0, st>>>(cl->rpart, RED_BLOCKS, cl->npts, cl->ctd, cl->scal);
    pack_forward<T>(cl, st, vor, vel, cstride, pitch);
    k_unpack<T><<<RED_BLOCKS * 4, RED_THREADS, 0, st>>>(cl->outf, cl->scal, vor, cstride, cl->Z, cl->npts, pitch,
                                                       ostride, flags, out);
    return cudaPeekAtLastError() == cudaSuccess ? PS3D_OK : PS3D_ERR_CUDA;
}
template int closure_apply<float>(ps3d_closure *, cudaStream_t, const float *, const float *, long long, int, float *,
                                  long long, int);
template int closure_apply<double>(ps3d_closure *, cudaStream_t, const double *, const double *, long long, int,
                                   double *, long long, int);

}  // namespace ps3d

// ======================================================================
extern "C" {

int ps3d_closure_create(int nx, int ny, int nz, int max_samples, int device, unsigned long long seed,
                        ps3d_closure **out)
{
    if (!out) return PS3D_ERR_INVALID_ARG;
    *out = nullptr;
    auto pow2 = [](int v) { return v >= 8 && (v & (v - 1)) == 0; };
    if (!pow2(nx) || !pow2(ny) || !pow2(nz) || nx > 2048 || ny > 2048 || nz > 2048) return PS3D_ERR_UNSUPPORTED_SIZE;
    if (max_samples < 0) return PS3D_ERR_INVALID_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return PS3D_ERR_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess || prop.major != 10 || prop.minor != 3) {
        cudaGetLastError();
        return PS3D_ERR_NO_DEVICE;
    }
    ps3d_closure *cl = new ps3d_closure();
    cl->nx = nx;
    cl->ny = ny;
    cl->nz = nz;
    cl->Z = nz + 1;
    cl->npts = (long long)nx * ny * (nz + 1);
    cl->device = device;
    cl->nsm = prop.multiProcessorCount;
    cl->max_samples = max_samples;
    cl->nchunk = (cl->npts + WG_CHUNK - 1) / WG_CHUNK;
    cl->rng.s = seed;
    cudaSetDevice(device);
    cudaStreamCreateWithFlags(&cl->st, cudaStreamNonBlocking);
    conv_attr<16, 32, EPI_GELU>(cl);
    conv_attr<32, 32, EPI_GELU>(cl);
    conv_attr<32, 8, EPI_OUT>(cl);
    conv_attr<16, 32, EPI_BWD>(cl);
    conv_attr<32, 32, EPI_BWD>(cl);
    // tcgen05 path: padded geometry; available when a tile's shared memory
    // (weights + 3 x 4 chunk planes of 128 + 2(ZP+1) rows) fits a block
    cl->ZP = nz + 3;
    cl->YP = ny + 2;
    cl->QN = (long long)(nx + 2) * cl->YP * cl->ZP;
    cl->GUARD = (long long)cl->YP * cl->ZP + cl->ZP + 256;
    cl->RTOT = (cl->QN + 2 * cl->GUARD + 7) / 8 * 8;
    cl->tc_ok = tc_smem<32, 32>(cl->ZP) + 2048 <= (size_t)prop.sharedMemPerBlockOptin && tc_attr<16, 32, EPI_GELU>(cl) &&
                tc_attr<32, 32, EPI_GELU>(cl) && tc_attr<32, 16, EPI_OUT>(cl);
    cl->engine = cl->tc_ok ? PS3D_CLOSURE_ENGINE_TCGEN05 : PS3D_CLOSURE_ENGINE_MMA;
    const long long P = cl->npts;
    bool ok = calloc_dev(cl, &cl->w, NPARAM * 4) && calloc_dev(cl, &cl->g, NPARAM * 4) &&
              calloc_dev(cl, &cl->m, NPARAM * 4) && calloc_dev(cl, &cl->v, NPARAM * 4);
    for (int l = 0; l < NL && ok; ++l) {
        ok = calloc_dev(cl, &cl->imgf[l], (size_t)NTAP * (CPAD_IN[l] / 16) * (CPAD_OUT[l] / 8) * 32 * 8) &&
             calloc_dev(cl, &cl->bpad[l], 64 * 4);
        if (ok && l > 0) {
            const int cinp = l == NL - 1 ? CPAD_DZ4 : CPAD_OUT[l];
            ok = calloc_dev(cl, &cl->imgb[l], (size_t)NTAP * (cinp / 16) * (CPAD_IN[l] / 8) * 32 * 8);
        }
    }
    ok = ok && calloc_dev(cl, &cl->a0, P * 16 * 2);
    for (int l = 0; l < 3 && ok; ++l) ok = calloc_dev(cl, &cl->z[l], P * 32 * 2) && calloc_dev(cl, &cl->act[l], P * 32 * 2);
    ok = ok && calloc_dev(cl, &cl->dz4, P * CPAD_DZ4 * 2) && calloc_dev(cl, &cl->dzA, P * 32 * 2) &&
         calloc_dev(cl, &cl->dzB, P * 32 * 2) && calloc_dev(cl, &cl->outf, P * CPAD_OUT[NL - 1] * 4) &&
         calloc_dev(cl, &cl->wpart, (size_t)cl->nchunk * (NTAP + 1) * 32 * 32 * 4) &&
         calloc_dev(cl, &cl->scal, 4 * 4) && calloc_dev(cl, &cl->rpart, 2 * RED_BLOCKS * 8) &&
         calloc_dev(cl, &cl->lpart, (RED_BLOCKS + 1) * 8) && calloc_dev(cl, &cl->ctd, 8) && calloc_dev(cl, &cl->host_out, (size_t)3 * P * 8) &&
         calloc_dev(cl, &cl->host_in, (size_t)6 * P * 8) && calloc_dev(cl, &cl->sscal, (size_t)(max_samples + 1) * 16);
    if (ok && max_samples > 0) ok = calloc_dev(cl, &cl->data, (size_t)max_samples * 9 * P * 4);
    ok = ok && calloc_dev(cl, &cl->derr, 16);
    if (ok && cl->tc_ok) {
        ok = calloc_dev(cl, &cl->pa0, (size_t)2 * cl->RTOT * 16) &&
             calloc_dev(cl, &cl->pact[0], (size_t)4 * cl->RTOT * 16) &&
             calloc_dev(cl, &cl->pact[1], (size_t)4 * cl->RTOT * 16);
        for (int l = 0; l < NL && ok; ++l) {
            const int coutp = l == NL - 1 ? 16 : CPAD_OUT[l];
            ok = calloc_dev(cl, &cl->imgtc[l], (size_t)NTAP * (CPAD_IN[l] / 8) * coutp * 16);
        }
    }
    if (!ok) {
        cudaGetLastError();
        ps3d_closure_destroy(cl);
        return PS3D_ERR_OUT_OF_MEMORY;
    }
    // He-uniform weights (bound sqrt(6 / fan_in)), the output layer scaled by
    // 0.1 so that an untrained closure starts as a small correction; zero bias
    std::vector<float> h(NPARAM, 0.f);
    for (int l = 0; l < NL; ++l) {
        const double bound = std::sqrt(6.0 / (NTAP * CREAL_IN[l])) * (l == NL - 1 ? 0.1 : 1.0);
        const int nw = NTAP * CREAL_IN[l] * CREAL_OUT[l];
        for (int i = 0; i < nw; ++i) h[woff(l) + i] = (float)((2.0 * cl->rng.uniform() - 1.0) * bound);
    }
    cudaMemcpy(cl->w, h.data(), NPARAM * 4, cudaMemcpyHostToDevice);
    images(cl, cl->st);
    cudaStreamSynchronize(cl->st);
    const int rc = ccheck(cl, "closure_create");
    if (rc) {
        ps3d_closure_destroy(cl);
        return rc;
    }
    *out = cl;
    return PS3D_OK;
}

int ps3d_closure_destroy(ps3d_closure *cl)
{
    if (!cl) return PS3D_OK;
    if (cl->owner) return cfail(cl, PS3D_ERR_INVALID_ARG, "closure is attached to a context");
    cudaSetDevice(cl->device);
    if (cl->st) cudaStreamSynchronize(cl->st);
    for (void *p : cl->allocs) cudaFree(p);
    if (cl->st) cudaStreamDestroy(cl->st);
    delete cl;
    return PS3D_OK;
}

const char *ps3d_closure_last_error(const ps3d_closure *cl) { return cl ? cl->err.c_str() : ""; }

int ps3d_closure_get_params(ps3d_closure *cl, float *params)
{
    int rc = centre(cl);
    if (rc) return rc;
    if (!params) return PS3D_ERR_INVALID_ARG;
    cudaStreamSynchronize(cl->st);
    cudaMemcpy(params, cl->w, NPARAM * 4, cudaMemcpyDeviceToHost);
    return ccheck(cl, "get_params");
}

int ps3d_closure_set_params(ps3d_closure *cl, const float *params)
{
    int rc = centre(cl);
    if (rc) return rc;
    if (!params) return PS3D_ERR_INVALID_ARG;
    cudaStreamSynchronize(cl->st);
    cudaMemcpy(cl->w, params, NPARAM * 4, cudaMemcpyHostToDevice);
    images(cl, cl->st);
    cudaStreamSynchronize(cl->st);
    return ccheck(cl, "set_params");
}

int ps3d_closure_get_scale(ps3d_closure *cl, double *ct)
{
    if (!cl || !ct) return PS3D_ERR_INVALID_ARG;
    *ct = cl->ct;
    return PS3D_OK;
}

int ps3d_closure_set_scale(ps3d_closure *cl, double ct)
{
    if (!cl || !(ct > 0.0) || !std::isfinite(ct)) return PS3D_ERR_INVALID_ARG;
    int rc = centre(cl);
    if (rc) return rc;
    cl->ct = ct;
    cudaStreamSynchronize(cl->st);
    cudaMemcpy(cl->ctd, &cl->ct, 8, cudaMemcpyHostToDevice);
    return ccheck(cl, "set_scale");
}

int ps3d_closure_add_sample(ps3d_closure *cl, const double *vor, const double *vel, const double *target)
{
    int rc = centre(cl);
    if (rc) return rc;
    if (!vor || !vel || !target) return PS3D_ERR_INVALID_ARG;
    if (cl->nsamples >= cl->max_samples) return cfail(cl, PS3D_ERR_INVALID_ARG, "sample store full");
    const long long P = cl->npts;
    std::vector<float> h((size_t)9 * P);
    for (long long i = 0; i < 3 * P; ++i) {
        h[i] = (float)vor[i];
        h[3 * P + i] = (float)vel[i];
        h[6 * P + i] = (float)target[i];
    }
    cudaStreamSynchronize(cl->st);
    cudaMemcpy(cl->data + (size_t)cl->nsamples * 9 * P, h.data(), h.size() * 4, cudaMemcpyHostToDevice);
    rc = ccheck(cl, "add_sample");
    if (rc) return rc;
    cl->w2.push_back(mean_sq3(vor, P));
    cl->u2.push_back(mean_sq3(vel, P));
    cl->t2.push_back(mean_sq3(target, P));
    cl->nsamples += 1;
    return PS3D_OK;
}

int ps3d_closure_num_samples(ps3d_closure *cl, int *n)
{
    if (!cl || !n) return PS3D_ERR_INVALID_ARG;
    *n = cl->nsamples;
    return PS3D_OK;
}

int ps3d_closure_train(ps3d_closure *cl, int iters, double lr0, double lr1, unsigned long long seed, double *loss)
{
    int rc = centre(cl);
    if (rc) return rc;
    if (iters < 0 || cl->nsamples == 0) return cfail(cl, PS3D_ERR_NOT_READY, "no training samples");
    if (!(cl->ct > 0.0)) {
        // ct = mean over the samples of rms(target) / <|vor|^2>
        double s = 0.0;
        int n = 0;
        for (int i = 0; i < cl->nsamples; ++i)
            if (cl->w2[i] > 0) {
                s += std::sqrt(cl->t2[i]) / cl->w2[i];
                ++n;
            }
        if (!(s > 0.0)) return cfail(cl, PS3D_ERR_INVALID_ARG, "training targets are zero");
        cl->ct = s / n;
        cudaMemcpy(cl->ctd, &cl->ct, 8, cudaMemcpyHostToDevice);
    }
    upload_sample_scalars(cl);
    if (cl->loss_cap < iters) {
        void *q = nullptr;
        if (cudaMalloc(&q, (size_t)(iters > 0 ? iters : 1) * 8) != cudaSuccess) {
            cudaGetLastError();
            return cfail(cl, PS3D_ERR_OUT_OF_MEMORY, "loss buffer");
        }
        if (cl->lossd) {
            for (auto &p : cl->allocs)
                if (p == cl->lossd) p = q;
            cudaFree(cl->lossd);
        } else {
            cl->allocs.push_back(q);
        }
        cl->lossd = reinterpret_cast<double *>(q);
        cl->loss_cap = iters;
    }
    SplitMix order{seed};
    std::vector<int> perm(cl->nsamples);
    int pos = cl->nsamples;
    const float b1 = 0.9f, b2 = 0.999f;
    for (int it = 0; it < iters; ++it) {
        if (pos == cl->nsamples) {
            for (int i = 0; i < cl->nsamples; ++i) perm[i] = i;
            for (int i = cl->nsamples - 1; i > 0; --i) {
                const int j = (int)(order.next() % (unsigned long long)(i + 1));
                std::swap(perm[i], perm[j]);
            }
            pos = 0;
        }
        const int s = perm[pos++];
        pack_sample(cl, cl->st, s);
        forward(cl, cl->st);
        loss_and_grad(cl, cl->st, s, cl->lossd + it);
        backward(cl, cl->st);
        cl->adam_t += 1;
        const double frac = iters > 1 ? (double)it / (double)(iters - 1) : 0.0;
        const double lr = lr1 + 0.5 * (lr0 - lr1) * (1.0 + std::cos(3.14159265358979323846 * frac));
        const float c1 = (float)(1.0 / (1.0 - std::pow((double)b1, (double)cl->adam_t)));
        const float c2 = (float)(1.0 / (1.0 - std::pow((double)b2, (double)cl->adam_t)));
        k_adam<<<(NPARAM + 255) / 256, 256, 0, cl->st>>>(cl->w, cl->g, cl->m, cl->v, NPARAM, (float)lr, b1, b2, c1, c2,
                                                         1e-8f);
        images(cl, cl->st);
        if ((it & 63) == 63) {
            rc = ccheck(cl, "train");
            if (rc) return rc;
        }
    }
    if (cudaStreamSynchronize(cl->st) != cudaSuccess) return ccheck(cl, "train");
    if (loss && iters > 0) cudaMemcpy(loss, cl->lossd, (size_t)iters * 8, cudaMemcpyDeviceToHost);
    return ccheck(cl, "train");
}

int ps3d_closure_predict(ps3d_closure *cl, const double *vor, const double *vel, double *corr)
{
    int rc = centre(cl);
    if (rc) return rc;
    if (!vor || !vel || !corr) return PS3D_ERR_INVALID_ARG;
    if (!(cl->ct > 0.0)) return cfail(cl, PS3D_ERR_NOT_READY, "closure output scale not set");
    const long long P = cl->npts;
    cudaMemcpyAsync(cl->host_in, vor, (size_t)3 * P * 8, cudaMemcpyHostToDevice, cl->st);
    cudaMemcpyAsync(cl->host_in + 3 * P, vel, (size_t)3 * P * 8, cudaMemcpyHostToDevice, cl->st);
    const double *dv = cl->host_in;
    k_sumsq<double><<<RED_BLOCKS, RED_THREADS, 0, cl->st>>>(dv, dv + 3 * P, P, cl->Z, cl->Z, P, cl->rpart);
    k_scal_finish<<<1, RED_THREADS, 0, cl->st>>>(cl->rpart, RED_BLOCKS, P, cl->ctd, cl->scal);
    pack_forward<double>(cl, cl->st, dv, dv + 3 * P, P, cl->Z);
    k_unpack<double><<<RED_BLOCKS * 4, RED_THREADS, 0, cl->st>>>(cl->outf, cl->scal, dv, P, cl->Z, P, cl->Z, P, 0,
                                                                cl->host_out);
    cudaMemcpyAsync(corr, cl->host_out, (size_t)3 * P * 8, cudaMemcpyDeviceToHost, cl->st);
    if (cudaStreamSynchronize(cl->st) != cudaSuccess) return ccheck(cl, "predict");
    rc = ccheck(cl, "predict");
    return rc ? rc : ps3d_closure_check(cl);
}

int ps3d_closure_set_engine(ps3d_closure *cl, int engine)
{
    if (!cl || (engine != PS3D_CLOSURE_ENGINE_MMA && engine != PS3D_CLOSURE_ENGINE_TCGEN05))
        return PS3D_ERR_INVALID_ARG;
    if (engine == PS3D_CLOSURE_ENGINE_TCGEN05 && !cl->tc_ok)
        return cfail(cl, PS3D_ERR_UNSUPPORTED_SIZE, "tcgen05 tile does not fit shared memory at this nz");
    cl->engine = engine;
    return PS3D_OK;
}

int ps3d_closure_get_engine(ps3d_closure *cl, int *engine)
{
    if (!cl || !engine) return PS3D_ERR_INVALID_ARG;
    *engine = cl->engine;
    return PS3D_OK;
}

int ps3d_closure_check(ps3d_closure *cl)
{
    int rc = centre(cl);
    if (rc) return rc;
    int h = 0;
    cudaStreamSynchronize(cl->st);
    cudaMemcpy(&h, cl->derr, sizeof(int), cudaMemcpyDeviceToHost);
    rc = ccheck(cl, "check");
    if (rc) return rc;
    if (h) {
        cudaMemset(cl->derr, 0, sizeof(int));
        return cfail(cl, PS3D_ERR_DEVICE_LIMIT, "tcgen05 convolution: a bounded wait ran out");
    }
    return PS3D_OK;
}

int ps3d_closure_time_forward(ps3d_closure *cl, int reps, double *ms)
{
    int rc = centre(cl);
    if (rc) return rc;
    if (reps < 1 || !ms) return PS3D_ERR_INVALID_ARG;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto fwd = [cl]() {
        if (cl->engine == 1) forward_tc(cl, cl->st);
        else forward(cl, cl->st);
    };
    fwd();  // warm-up
    cudaEventRecord(e0, cl->st);
    for (int i = 0; i < reps; ++i) fwd();
    cudaEventRecord(e1, cl->st);
    cudaError_t e = cudaEventSynchronize(e1);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cfail(cl, PS3D_ERR_CUDA, std::string("time_forward: ") + cudaGetErrorString(e));
    *ms = (double)t / reps;
    rc = ccheck(cl, "time_forward");
    return rc ? rc : ps3d_closure_check(cl);
}

int ps3d_closure_gradients(ps3d_closure *cl, int sample, float *out, float *grad, double *loss)
{
    int rc = centre(cl);
    if (rc) return rc;
    if (sample < 0 || sample >= cl->nsamples) return PS3D_ERR_INVALID_ARG;
    if (!(cl->ct > 0.0)) return cfail(cl, PS3D_ERR_NOT_READY, "closure output scale not set");
    upload_sample_scalars(cl);
    const long long P = cl->npts;
    pack_sample(cl, cl->st, sample);
    forward(cl, cl->st);
    loss_and_grad(cl, cl->st, sample, cl->lpart + RED_BLOCKS);
    backward(cl, cl->st);
    if (cudaStreamSynchronize(cl->st) != cudaSuccess) return ccheck(cl, "gradients");
    if (grad) cudaMemcpy(grad, cl->g, NPARAM * 4, cudaMemcpyDeviceToHost);
    if (loss) cudaMemcpy(loss, cl->lpart + RED_BLOCKS, 8, cudaMemcpyDeviceToHost);
    if (out) {
        std::vector<float> h((size_t)P * CPAD_OUT[NL - 1]);
        cudaMemcpy(h.data(), cl->outf, h.size() * 4, cudaMemcpyDeviceToHost);
        for (long long p = 0; p < P; ++p)
            for (int c = 0; c < 3; ++c) out[c * P + p] = h[p * CPAD_OUT[NL - 1] + c];
    }
    return ccheck(cl, "gradients");
}

}  // extern "C"
