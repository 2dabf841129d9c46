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

// harmonic functions of one (kx, ky) column at level iz (FP32)
struct Harm {
    float kl, ef, div, dz, Lz;
    bool mean;  // (0,0) column: linear functions
    __device__ void at(int iz, float &pm, float &pp) const
    {
        const float zp = dz * (float)iz, zm = Lz - zp;
        if (mean) {
            pm = zm / Lz;
            pp = zp / Lz;
        } else {
            const float ep = expf(-kl * zp), em = expf(-kl * zm);
            pm = div * (ep - ef * em);
            pp = div * (em - ef * ep);
        }
    }
};

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
            const float kA = sqrtf((float)k2l2[cA]), kB = sqrtf((float)k2l2[cB]);
            const float eA = expf(-kA * Lz), eB = expf(-kB * Lz);
            hA = Harm{kA, eA, 1.0f / (1.0f - eA * eA), dz, Lz, cA == 0};
            hB = Harm{kB, eB, 1.0f / (1.0f - eB * eB), dz, Lz, cB == 0};
        }
        // ---- load the extension
        float2 v[M];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            const int j = lane + 32 * m;
            float a = 0.f, b = 0.f;
            if (MODE == COL_DCT) {
                const int jj = j <= nz ? j : L - j;
                a = (float)in[oA + jj];
                b = (float)in[oB + jj];
            } else if (j != 0 && j != nz) {
                const int jj = j < nz ? j : L - j;
                a = (float)in[oA + jj];
                b = (float)in[oB + jj];
                if (MODE == COL_DECOMP) {
                    float pm, pp;
                    hA.at(jj, pm, pp);
                    a = a - (fA0 * pm + fAn * pp);
                    hB.at(jj, pm, pp);
                    b = b - (fB0 * pm + fBn * pp);
                }
                if (j > nz) {
                    a = -a;
                    b = -b;
                }
            }
            v[m] = make_float2(a, b);
        }
        // ---- M-point DIF FFT in registers (output in bit-reversed order)
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
        // ---- twiddle wL^(lane * b), b = bitrev(r)
#pragma unroll
        for (int r = 1; r < M; ++r) {
            const int b = bitrev<M>(r);
            v[r] = fmulc(v[r], __ldg(&twL[(lane * b) & (L - 1)]));
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
    const size_t sm = 8 * 2 * pad * sizeof(float);
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

bool col32_supported(int nz) { return nz >= 32 && nz <= 512; }

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

void columns32_init()
{
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
