// FP32 column transforms (the mixed form's DST / DCT along z), one warp per
// pair of columns, held in registers.
//
// The two columns are packed as the real and imaginary parts of one complex
// sequence: their odd (DST) or even (DCT) extension y of length L = 2*nz
// (src/fft/stafft.f90:410-550 restated as one complex FFT).  With L = 32*M,
// lane l holds y[l + 32 m] (m = 0..M-1, a coalesced load), and
//   X[M a + b] = sum_l w32^(l a) [ wL^(l b) sum_m y[l + 32 m] wM^(m b) ]:
// an M-point DFT in registers, a twiddle, and a 32-point DFT across the warp
// by shuffles.  Results go through a padded per-warp shared buffer back to
// coalesced column stores.  The harmonic functions phim/phip of the
// decompose/combine steps (inversion_utils.f90:484-542, 563-647) are
// evaluated in registers instead of being read from N-sized tables, so a
// launch moves one field in and one field out.
#include "kernels.h"

namespace ps3d {

__constant__ float2 c_w32[32];  // exp(-2 pi i j / 32)

template <int M> __device__ __forceinline__ int bitrev(int r)
{
    int o = 0;
#pragma unroll
    for (int b = 1; b < M; b <<= 1) {
        o = (o << 1) | (r & 1);
        r >>= 1;
    }
    return o;
}

__device__ __forceinline__ float2 fmulc(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// harmonic functions of one (kx, ky) column at level iz (FP32):
// ep = exp(-kl zp) = 2^(a iz), em = exp(-kl zm) = 2^(c - a iz) with
// a = -kl dz log2(e), c = -kl Lz log2(e)
struct Harm {
    float a, c, ef, div, dz, Lz;
    bool mean;  // (0,0) column: linear functions
    __device__ static Harm make(float kl, float dz, float Lz, bool mean)
    {
        const float l2e = 1.4426950408889634f;
        Harm h;
        h.a = -kl * dz * l2e;
        h.c = -kl * Lz * l2e;
        h.ef = exp2f(h.c);
        h.div = 1.0f / (1.0f - h.ef * h.ef);
        h.dz = dz;
        h.Lz = Lz;
        h.mean = mean;
        return h;
    }
    __device__ void at(int iz, float &pm, float &pp) const
    {
        if (mean) {
            const float zp = dz * (float)iz, zm = Lz - zp;
            pm = zm / Lz;
            pp = zp / Lz;
        } else {
            const float t = a * (float)iz;
            const float ep = exp2f(t), em = exp2f(c - t);
            pm = div * (ep - ef * em);
            pp = div * (em - ef * ep);
        }
    }
};

// in-register DIF FFT of length M (output in bit-reversed order)
template <int M> __device__ __forceinline__ void dif_regs(float2 *v)
{
#pragma unroll
    for (int h = M / 2; h >= 1; h >>= 1) {
#pragma unroll
        for (int s0 = 0; s0 < M; s0 += 2 * h) {
#pragma unroll
            for (int i = 0; i < h; ++i) {
                const float2 a = v[s0 + i], b = v[s0 + i + h];
                v[s0 + i] = make_float2(a.x + b.x, a.y + b.y);
                const float2 d = make_float2(a.x - b.x, a.y - b.y);
                v[s0 + i + h] = (i == 0) ? d : fmulc(d, c_w32[i * (16 / h)]);
            }
        }
    }
}

template <int MODE, int M, typename TIN>
__global__ void __launch_bounds__(256) k_col32(const TIN *__restrict__ in, float *__restrict__ out, int nz, int P,
                                               long long npairs, const double *__restrict__ k2l2, float dz,
                                               float Lz, const float2 *__restrict__ twL)
{
    constexpr int L = 32 * M;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    extern __shared__ float sm32[];
    const int pad = nz + 1 + (nz + 1) / 32 + 1;
    float *sA = sm32 + (size_t)wib * 2 * pad;
    float *sB = sA + pad;
    const float s = rsqrtf((float)L);
    // per-lane twiddles of the cross-lane DIF network: w_(2h)^(lane & (h-1))
    float2 wl[5];
#pragma unroll
    for (int st = 0; st < 5; ++st) {
        const int h = 16 >> st;
        wl[st] = c_w32[(lane & (h - 1)) * (16 / h)];
    }
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long pr = (long long)blockIdx.x * (blockDim.x >> 5) + wib; pr < npairs; pr += warps) {
        const long long cA = 2 * pr, cB = cA + 1;
        const long long oA = cA * P, oB = cB * P;
        float fA0 = 0.f, fAn = 0.f, fB0 = 0.f, fBn = 0.f;
        Harm hA{}, hB{};
        if (MODE == COL_DECOMP || MODE == COL_COMBINE) {
            fA0 = (float)in[oA];
            fAn = (float)in[oA + nz];
            fB0 = (float)in[oB];
            fBn = (float)in[oB + nz];
            hA = Harm::make(sqrtf((float)k2l2[cA]), dz, Lz, cA == 0);
            hB = Harm::make(sqrtf((float)k2l2[cB]), dz, Lz, cB == 0);
        }
        // ---- load the extension (raw loads first)
        float2 v[M];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            const int j = lane + 32 * m;
            const int jj = j <= nz ? j : L - j;
            float a = 0.f, b = 0.f;
            if (MODE == COL_DCT || (j != 0 && j != nz)) {
                a = (float)in[oA + jj];
                b = (float)in[oB + jj];
            }
            v[m] = make_float2(a, b);
        }
        if (MODE != COL_DCT) {
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const int j = lane + 32 * m;
                const int jj = j <= nz ? j : L - j;
                if (MODE == COL_DECOMP && j != 0 && j != nz) {
                    float pm, pp;
                    hA.at(jj, pm, pp);
                    v[m].x = v[m].x - (fA0 * pm + fAn * pp);
                    hB.at(jj, pm, pp);
                    v[m].y = v[m].y - (fB0 * pm + fBn * pp);
                }
                if (j > nz) v[m] = make_float2(-v[m].x, -v[m].y);
            }
        }
        // ---- M-point DIF FFT in registers (output in bit-reversed order)
        dif_regs<M>(v);
        // ---- twiddle wL^(lane * b), b = bitrev(r)
#pragma unroll
        for (int r = 1; r < M; ++r) {
            const int b = bitrev<M>(r);
            v[r] = fmulc(v[r], __ldg(&twL[(lane * b) & (L - 1)]));
        }
        if constexpr (M == 32) {
            // ---- transpose the 32 x 32 block through shared memory: lane b
            // then holds Z[l][b] for l = 0..31
            float2 *tr = reinterpret_cast<float2 *>(sm32) + (size_t)wib * 32 * 33;
#pragma unroll
            for (int r = 0; r < 32; ++r) tr[lane * 33 + bitrev<32>(r)] = v[r];
            __syncwarp();
#pragma unroll
            for (int l = 0; l < 32; ++l) v[l] = tr[l * 33 + lane];
            __syncwarp();
            // ---- 32-point DIF over l: register r holds X[32 bitrev(r) + lane]
            dif_regs<32>(v);
            // ---- coalesced column stores (k = 32 a + lane)
#pragma unroll
            for (int r = 0; r < 32; ++r) {
                const int a = bitrev<32>(r);
                const int k = 32 * a + lane;
                if (a <= 16 && k <= nz) {
                    float ra, rb;
                    if (MODE == COL_DCT) {
                        ra = v[r].x * s;
                        rb = v[r].y * s;
                    } else if (k == 0) {
                        ra = (MODE == COL_DST) ? (float)in[oA] : fA0;
                        rb = (MODE == COL_DST) ? (float)in[oB] : fB0;
                    } else if (k == nz) {
                        ra = (MODE == COL_DST) ? 0.f : fAn;
                        rb = (MODE == COL_DST) ? 0.f : fBn;
                    } else {
                        ra = -v[r].y * s;
                        rb = v[r].x * s;
                        if (MODE == COL_COMBINE) {
                            float pm, pp;
                            hA.at(k, pm, pp);
                            ra = ra + fA0 * pm + fAn * pp;
                            hB.at(k, pm, pp);
                            rb = rb + fB0 * pm + fBn * pp;
                        }
                    }
                    out[oA + k] = ra;
                    out[oB + k] = rb;
                }
            }
            continue;
        }
        // ---- 32-point DIF across lanes (lane l ends with index bitrev5(l))
#pragma unroll
        for (int st = 0; st < 5; ++st) {
            const int h = 16 >> st;
            const bool hi = (lane & h) != 0;
#pragma unroll
            for (int r = 0; r < M; ++r) {
                float2 u;
                u.x = __shfl_xor_sync(0xffffffffu, v[r].x, h);
                u.y = __shfl_xor_sync(0xffffffffu, v[r].y, h);
                const float2 sum = make_float2(v[r].x + u.x, v[r].y + u.y);
                const float2 dif = fmulc(make_float2(u.x - v[r].x, u.y - v[r].y), wl[st]);
                v[r] = hi ? dif : sum;
            }
        }
        // ---- scatter X[M a + b] to the padded shared buffer
        const int a = bitrev<32>(lane);
#pragma unroll
        for (int r = 0; r < M; ++r) {
            const int k = M * a + bitrev<M>(r);
            if (k <= nz) {
                const int kk = k + (k >> 5);
                if (MODE == COL_DCT) {
                    sA[kk] = v[r].x * s;
                    sB[kk] = v[r].y * s;
                } else {
                    sA[kk] = -v[r].y * s;
                    sB[kk] = v[r].x * s;
                }
            }
        }
        __syncwarp();
        // ---- coalesced column stores with the mode's boundary rows
        for (int iz = lane; iz <= nz; iz += 32) {
            const int kk = iz + (iz >> 5);
            float ra = sA[kk], rb = sB[kk];
            if (MODE != COL_DCT) {
                if (iz == 0) {
                    if (MODE == COL_DST) {
                        ra = (float)in[oA];
                        rb = (float)in[oB];
                    } else {
                        ra = fA0;
                        rb = fB0;
                    }
                } else if (iz == nz) {
                    ra = (MODE == COL_DST) ? 0.f : fAn;
                    rb = (MODE == COL_DST) ? 0.f : fBn;
                } else if (MODE == COL_COMBINE) {
                    float pm, pp;
                    hA.at(iz, pm, pp);
                    ra = ra + fA0 * pm + fAn * pp;
                    hB.at(iz, pm, pp);
                    rb = rb + fB0 * pm + fBn * pp;
                }
            }
            out[oA + iz] = ra;
            out[oB + iz] = rb;
        }
        __syncwarp();
    }
}

template <int MODE, typename TIN>
static void launch_m(int M, const TIN *in, float *out, const Dims &d, cudaStream_t st, const double *k2l2, float dz,
                     float Lz, const float2 *twL)
{
    const long long npairs = d.ncol / 2;
    const int pad = d.nz + 1 + (d.nz + 1) / 32 + 1;
    size_t per_warp = 2 * pad * sizeof(float);
    if (M == 32 && per_warp < 32 * 33 * sizeof(float2)) per_warp = 32 * 33 * sizeof(float2);
    const size_t sm = 8 * per_warp;
    long long nb = (npairs + 7) / 8;
    if (nb > 152 * 16) nb = 152 * 16;
    switch (M) {
    case 2: k_col32<MODE, 2, TIN><<<(unsigned)nb, 256, sm, st>>>(in, out, d.nz, d.P, npairs, k2l2, dz, Lz, twL); break;
    case 4: k_col32<MODE, 4, TIN><<<(unsigned)nb, 256, sm, st>>>(in, out, d.nz, d.P, npairs, k2l2, dz, Lz, twL); break;
    case 8: k_col32<MODE, 8, TIN><<<(unsigned)nb, 256, sm, st>>>(in, out, d.nz, d.P, npairs, k2l2, dz, Lz, twL); break;
    case 16: k_col32<MODE, 16, TIN><<<(unsigned)nb, 256, sm, st>>>(in, out, d.nz, d.P, npairs, k2l2, dz, Lz, twL); break;
    default: k_col32<MODE, 32, TIN><<<(unsigned)nb, 256, sm, st>>>(in, out, d.nz, d.P, npairs, k2l2, dz, Lz, twL); break;
    }
}

// L = 2 nz = 32 M with M a power of two, 2..32
bool col32_supported(int nz) { return nz == 32 || nz == 64 || nz == 128 || nz == 256 || nz == 512; }

template <typename TIN>
void columns32(const Dims &d, cudaStream_t st, int mode, const TIN *in, float *out, const double *k2l2, float dz,
               float Lz, const float2 *twL, Probe *pr)
{
    const int M = (2 * d.nz) / 32;
    if (pr) pr->begin(PROBE_COLUMNS, st);
    switch (mode) {
    case COL_DST: launch_m<COL_DST, TIN>(M, in, out, d, st, k2l2, dz, Lz, twL); break;
    case COL_DCT: launch_m<COL_DCT, TIN>(M, in, out, d, st, k2l2, dz, Lz, twL); break;
    case COL_DECOMP: launch_m<COL_DECOMP, TIN>(M, in, out, d, st, k2l2, dz, Lz, twL); break;
    default: launch_m<COL_COMBINE, TIN>(M, in, out, d, st, k2l2, dz, Lz, twL); break;
    }
    if (pr) pr->end(PROBE_COLUMNS, st, 2.0 * (double)d.ncol * (double)(d.nz + 1) * sizeof(float));
}

template <typename TIN> static void col32_attrs()
{
    const int bytes = 8 * 32 * 33 * (int)sizeof(float2);
    cudaFuncSetAttribute(k_col32<COL_DST, 32, TIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_col32<COL_DCT, 32, TIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_col32<COL_DECOMP, 32, TIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_col32<COL_COMBINE, 32, TIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

void columns32_init()
{
    col32_attrs<float>();
    col32_attrs<double>();
    float2 w[32];
    for (int j = 0; j < 32; ++j) {
        const double a = 2.0 * 3.14159265358979323846 * (double)j / 32.0;
        double c = cos(a), s = sin(a);
        if (j % 8 == 0) {
            const int q = j / 8;
            c = (q == 0) ? 1.0 : (q == 2 ? -1.0 : 0.0);
            s = (q == 1) ? 1.0 : (q == 3 ? -1.0 : 0.0);
        }
        w[j] = make_float2((float)c, (float)(-s));
    }
    cudaMemcpyToSymbol(c_w32, w, sizeof(w));
}

template void columns32<float>(const Dims &, cudaStream_t, int, const float *, float *, const double *, float, float,
                               const float2 *, Probe *);
template void columns32<double>(const Dims &, cudaStream_t, int, const double *, float *, const double *, float,
                                float, const float2 *, Probe *);

}  // namespace ps3d
