// FP32 column (z) transforms of the mixed form: one warp per pair of
// columns, half-length algorithm.
//
// The reference computes its sine and cosine transforms (src/fft/stafft.f90:
// 410-550) from one real FFT of length n = nz of a pre-processed sequence
//   dst:  wk(j) = (x(j) - x(n-j))/2 + sin(j pi/n) (x(j) + x(n-j))
//   dct:  wk(j) = (x(j) + x(n-j))/2 - sin(j pi/n) (x(j) - x(n-j))
// followed by a running sum over the cosine (dst) or sine (dct) part of the
// spectrum.  Here the two columns of a pair are packed as the real and
// imaginary parts of one complex sequence, so one n-point complex FFT serves
// both; the running sums become a warp scan.
//
// Warp FFT of n = 32*M points: lane l holds c[l + 32 m] (m < M); an M-point
// DFT in registers, a twiddle, a transpose through the warp's shared buffer,
// an M-point DFT over the other index, and S = 32/M lanes combined by
// shuffles.  Inputs stored as FP64 (the prognostic state) are narrowed with
// integer arithmetic, keeping GB300's FP64 pipe out of the kernel.
#include "kernels.h"

namespace ps3d {

namespace {

__constant__ float2 c_w32z[32];  // exp(-2 pi i j / 32)

__device__ __forceinline__ float2 fm(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

template <int M> __device__ __forceinline__ int brev(int r)
{
    int o = 0;
#pragma unroll
    for (int b = 1; b < M; b <<= 1) {
        o = (o << 1) | (r & 1);
        r >>= 1;
    }
    return o;
}

__device__ __forceinline__ float ld(const float *p, long long i) { return p[i]; }
__device__ __forceinline__ float ld(const double *p, long long i) { return narrow32(p[i]); }

// 2^x on the special-function unit, results below the normal range flushed
__device__ __forceinline__ float ex2(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// harmonic functions of one column (inversion_utils.f90:484-542):
// phim(z) = div (ep - ef em), phip(z) = div (em - ef ep), ep = exp(-kl zp),
// em = exp(-kl zm) = ep at the mirrored level; phip(iz) = phim(nz - iz)
struct Harm {
    float a, c, ef, div, inv_n;
    bool mean;
    __device__ static Harm make(float kl, float dz, float Lz, int nz, bool mean)
    {
        const float l2e = 1.4426950408889634f;
        Harm h;
        h.a = -kl * dz * l2e;
        h.c = -kl * Lz * l2e;
        h.ef = ex2(h.c);
        h.div = 1.0f / (1.0f - h.ef * h.ef);
        h.inv_n = 1.0f / (float)nz;
        h.mean = mean;
        return h;
    }
    __device__ void at(int iz, int nz, float &pm, float &pp) const
    {
        if (mean) {
            pp = (float)iz * inv_n;
            pm = (float)(nz - iz) * inv_n;
        } else {
            const float t = a * (float)iz;
            const float ep = ex2(t), em = ex2(c - t);
            pm = div * (ep - ef * em);
            pp = div * (em - ef * ep);
        }
    }
};

template <int M> __device__ __forceinline__ void dif(float2 *v)
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
                v[s0 + i + h] = (i == 0) ? d : fm(d, c_w32z[i * (16 / h)]);
            }
        }
    }
}

// n = 32 M point forward FFT of the warp's sequence; on entry lane l holds
// v[m] = c[l + 32 m]; on exit X[k] (natural order) is in xs[0..n).
template <int M>
__device__ __forceinline__ void warp_fft(float2 *v, float2 *xs, const float2 *__restrict__ twn, int lane)
{
    constexpr int S = 32 / M;
    constexpr int n = 32 * M;
    dif<M>(v);  // register r: Z_l[b], b = brev(r)
#pragma unroll
    for (int r = 1; r < M; ++r) v[r] = fm(v[r], __ldg(&twn[(lane * brev<M>(r)) & (n - 1)]));
    // transpose: lane (b, h) = (lane / S, lane % S) gathers Z[h + S t][b]
#pragma unroll
    for (int r = 0; r < M; ++r) xs[lane * (M + 1) + brev<M>(r)] = v[r];
    __syncwarp();
    const int b = lane / S, h = lane % S;
#pragma unroll
    for (int t = 0; t < M; ++t) v[t] = xs[(h + S * t) * (M + 1) + b];
    __syncwarp();
    dif<M>(v);  // register r: F_h[a'], a' = brev(r)
    if (S > 1) {
#pragma unroll
        for (int r = 1; r < M; ++r) v[r] = fm(v[r], c_w32z[(h * brev<M>(r)) & 31]);
        // S-point DIF across the S lanes of the group
#pragma unroll
        for (int hs = S / 2; hs >= 1; hs >>= 1) {
            const bool upper = (h & hs) != 0;
            const float2 w = c_w32z[((h & (hs - 1)) * (16 / hs)) & 31];
#pragma unroll
            for (int r = 0; r < M; ++r) {
                float2 u;
                u.x = __shfl_xor_sync(0xffffffffu, v[r].x, hs);
                u.y = __shfl_xor_sync(0xffffffffu, v[r].y, hs);
                const float2 sum = make_float2(v[r].x + u.x, v[r].y + u.y);
                const float2 dif2 = fm(make_float2(u.x - v[r].x, u.y - v[r].y), w);
                v[r] = upper ? dif2 : sum;
            }
        }
    }
    const int e = brev<S>(h);
#pragma unroll
    for (int r = 0; r < M; ++r) xs[b + M * brev<M>(r) + M * M * e] = v[r];
    __syncwarp();
}

__device__ __forceinline__ int zpad(int z) { return z + (z >> 4); }

// inclusive warp scan of one value per lane
__device__ __forceinline__ float warp_incl_scan(float x, int lane)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const float y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    return x;
}


// DST post-processing (stafft.f90:531-549 on the packed spectra in xs):
// interior outputs z = 1..n-1 of both columns into zA / zB
template <int M>
__device__ __forceinline__ void post_dst(const float2 *xs, float *zA, float *zB, int lane, float r2s)
{
    constexpr int n = 32 * M, KPL = n / 64;
    float carryA = 0.f, carryB = 0.f;
#pragma unroll
    for (int i = 0; i < KPL; ++i) {
        const int k = lane + 32 * i;
        const float2 ck = xs[k], cn = xs[(n - k) & (n - 1)];
        const float ReA = 0.5f * (ck.x + cn.x), ImA = 0.5f * (ck.y - cn.y);
        const float ReB = 0.5f * (ck.y + cn.y), ImB = -0.5f * (ck.x - cn.x);
        const float ia = warp_incl_scan((k == 0) ? 0.5f * ReA : ReA, lane) + carryA;
        const float ib = warp_incl_scan((k == 0) ? 0.5f * ReB : ReB, lane) + carryB;
        carryA = __shfl_sync(0xffffffffu, ia, 31);
        carryB = __shfl_sync(0xffffffffu, ib, 31);
        zA[zpad(2 * k + 1)] = r2s * ia;
        zB[zpad(2 * k + 1)] = r2s * ib;
        if (k > 0) {
            zA[zpad(2 * k)] = -r2s * ImA;
            zB[zpad(2 * k)] = -r2s * ImB;
        }
    }
}

// DCT post-processing (stafft.f90:458-482): outputs z = 0..n; x1 = x(1)
// from the direct sum
template <int M>
__device__ __forceinline__ void post_dct(const float2 *xs, float *zA, float *zB, int lane, float r2s, float x1A,
                                         float x1B)
{
    constexpr int n = 32 * M, KPL = n / 64;
    float carryA = 0.f, carryB = 0.f;
#pragma unroll
    for (int i = 0; i < KPL; ++i) {
        const int k = lane + 32 * i;
        const float2 ck = xs[k], cn = xs[(n - k) & (n - 1)];
        const float ReA = 0.5f * (ck.x + cn.x), ImA = 0.5f * (ck.y - cn.y);
        const float ReB = 0.5f * (ck.y + cn.y), ImB = -0.5f * (ck.x - cn.x);
        const float ia = warp_incl_scan((k == 0) ? 0.f : ImA, lane) + carryA;
        const float ib = warp_incl_scan((k == 0) ? 0.f : ImB, lane) + carryB;
        carryA = __shfl_sync(0xffffffffu, ia, 31);
        carryB = __shfl_sync(0xffffffffu, ib, 31);
        zA[zpad(2 * k)] = r2s * ReA;
        zB[zpad(2 * k)] = r2s * ReB;
        zA[zpad(2 * k + 1)] = x1A - r2s * ia;
        zB[zpad(2 * k + 1)] = x1B - r2s * ib;
    }
    if (lane == 0) {
        const float2 cm = xs[n / 2];
        zA[zpad(n)] = r2s * cm.x;
        zB[zpad(n)] = r2s * cm.y;
    }
}

__device__ __forceinline__ float warp_sum(float x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// Theta functions of the vertical-velocity inversion (inversion_utils.f90:
// 484-542, Dritschel & Frey 2023 eqs 3.4, 3.10, 3.11) for one column
struct Theta {
    Harm h;
    float kl, Q, R, k2ifac, dz, Lz;
    bool zero;  // (0,0) column: all theta functions vanish
    __device__ static Theta make(float kl, float k2i, float dz, float Lz, int nz, bool mean)
    {
        Theta t;
        t.h = Harm::make(kl, dz, Lz, nz, mean);
        t.kl = kl;
        t.Q = t.h.div * (1.0f + t.h.ef * t.h.ef);
        t.R = t.h.div * 2.0f * t.h.ef;
        t.k2ifac = 0.5f * k2i;
        t.dz = dz;
        t.Lz = Lz;
        t.zero = mean;
        return t;
    }
    // thetam, thetap (z values of w) and dthetam, dthetap (dw/dz) at level iz
    __device__ void at(int iz, float &tm, float &tp, float &dtm, float &dtp) const
    {
        if (zero) {
            tm = tp = dtm = dtp = 0.f;
            return;
        }
        const float zp = dz * (float)iz, zm = Lz - zp;
        const float Lm = kl * zm, Lp = kl * zp;
        const float t = h.a * (float)iz;
        const float ep = ex2(t), em = ex2(h.c - t);
        const float phm = h.div * (ep - h.ef * em), php = h.div * (em - h.ef * ep);
        const float dphm = -kl * h.div * (ep + h.ef * em), dphp = kl * h.div * (em + h.ef * ep);
        tm = k2ifac * (R * Lm * php - Q * Lp * phm);
        tp = k2ifac * (R * Lp * phm - Q * Lm * php);
        dtm = -k2ifac * ((Q * Lp - 1.0f) * dphm - R * Lm * dphp);
        dtp = -k2ifac * ((Q * Lm - 1.0f) * dphp - R * Lp * dphm);
    }
};

}  // namespace

// MODE: COL_DST, COL_DCT, COL_DECOMP, COL_COMBINE (see kernels.h)
template <int MODE, int M, typename TIN>
__global__ void __launch_bounds__(256, 2) k_colz(const TIN *__restrict__ in, float *__restrict__ out, int P,
                                              long long npairs, const double *__restrict__ k2l2, float dz,
                                              float Lz, const float2 *__restrict__ twn,
                                              const float *__restrict__ sinz, const float *__restrict__ cosz)
{
    constexpr int n = 32 * M;  // = nz
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    extern __shared__ __align__(16) unsigned char smz[];
    constexpr int XS = (32 * (M + 1) > n ? 32 * (M + 1) : n);  // float2 per warp
    constexpr int ZS = n + 1 + (n + 1) / 16 + 2;                // floats per output column
    float2 *xs = reinterpret_cast<float2 *>(smz) + (size_t)wib * (XS + ZS);
    float *zA = reinterpret_cast<float *>(xs + XS);
    float *zB = zA + ZS;
    const float s = rsqrtf((float)n);
    const float r2s = 1.41421356237309505f * s;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long pr = (long long)blockIdx.x * (blockDim.x >> 5) + wib; pr < npairs; pr += warps) {
        const long long cA = 2 * pr, cB = cA + 1;
        const long long oA = cA * P, oB = cB * P;
        float fA0 = 0.f, fAn = 0.f, fB0 = 0.f, fBn = 0.f;
        Harm hA{}, hB{};
        if (MODE == COL_DECOMP || MODE == COL_COMBINE || MODE == COL_DCT) {
            fA0 = ld(in, oA);
            fAn = ld(in, oA + n);
            fB0 = ld(in, oB);
            fBn = ld(in, oB + n);
        }
        if (MODE == COL_DECOMP || MODE == COL_COMBINE) {
            hA = Harm::make(sqrtf((float)k2l2[cA]), dz, Lz, n, cA == 0);
            hB = Harm::make(sqrtf((float)k2l2[cB]), dz, Lz, n, cB == 0);
        }
        // ---- pre-processed sequence wk (both columns), lane l: j = l + 32 m
        float2 v[M];
        float dsumA = 0.f, dsumB = 0.f;  // DCT direct sum for x(1)
#pragma unroll
        for (int m = 0; m < M; ++m) {
            const int j = lane + 32 * m;
            float xa = 0.f, xb = 0.f, ya = 0.f, yb = 0.f;  // x(j), x(n-j)
            if (j > 0) {
                xa = ld(in, oA + j);
                xb = ld(in, oB + j);
                ya = ld(in, oA + n - j);
                yb = ld(in, oB + n - j);
            }
            if (MODE == COL_DECOMP && j > 0) {
                float pm, pp;
                hA.at(j, n, pm, pp);
                xa -= fA0 * pm + fAn * pp;
                ya -= fA0 * pp + fAn * pm;
                hB.at(j, n, pm, pp);
                xb -= fB0 * pm + fBn * pp;
                yb -= fB0 * pp + fBn * pm;
            }
            const float sj = __ldg(&sinz[j]);
            if (MODE == COL_DCT) {
                if (j == 0) {
                    v[m] = make_float2(0.5f * (fA0 + fAn), 0.5f * (fB0 + fBn));
                } else {
                    const float cj = __ldg(&cosz[j]);
                    dsumA += xa * cj;
                    dsumB += xb * cj;
                    v[m] = make_float2(0.5f * (xa + ya) - sj * (xa - ya), 0.5f * (xb + yb) - sj * (xb - yb));
                }
            } else {
                v[m] = (j == 0) ? make_float2(0.f, 0.f)
                                : make_float2(0.5f * (xa - ya) + sj * (xa + ya), 0.5f * (xb - yb) + sj * (xb + yb));
            }
        }
        warp_fft<M>(v, xs, twn, lane);
        // ---- split the packed spectra, running sums as warp scans with a
        // carry, outputs to zA / zB
        if (MODE == COL_DCT) {
            const float x1A = r2s * (0.5f * fA0 + warp_sum(dsumA) - 0.5f * fAn);
            const float x1B = r2s * (0.5f * fB0 + warp_sum(dsumB) - 0.5f * fBn);
            post_dct<M>(xs, zA, zB, lane, r2s, x1A, x1B);
        } else {
            post_dst<M>(xs, zA, zB, lane, r2s);
        }
        __syncwarp();
        // ---- coalesced column stores with the mode's boundary rows
        for (int iz = lane; iz <= n; iz += 32) {
            float ra, rb;
            if (MODE == COL_DCT) {
                ra = zA[zpad(iz)];
                rb = zB[zpad(iz)];
            } else if (iz == 0) {
                ra = (MODE == COL_DST) ? ld(in, oA) : fA0;
                rb = (MODE == COL_DST) ? ld(in, oB) : fB0;
            } else if (iz == n) {
                ra = (MODE == COL_DST) ? 0.f : fAn;
                rb = (MODE == COL_DST) ? 0.f : fBn;
            } else {
                ra = zA[zpad(iz)];
                rb = zB[zpad(iz)];
                if (MODE == COL_COMBINE) {
                    float pm, pp;
                    hA.at(iz, n, pm, pp);
                    ra += fA0 * pm + fAn * pp;
                    hB.at(iz, n, pm, pp);
                    rb += fB0 * pm + fBn * pp;
                }
            }
            out[oA + iz] = ra;
            out[oB + iz] = rb;
        }
        __syncwarp();
    }
}

// Per-column scalars of a column pair spread over the warp (lane i holds
// scalar i): they stay out of the registers while the warp FFT runs and are
// fetched with one shuffle each where needed.
__device__ __forceinline__ float lane_get(float par, int i) { return __shfl_sync(0xffffffffu, par, i); }

// ------------------------------------------------------------------------
// Vertical velocity of vor2vel in one kernel (inversion.f90:94-139):
//   bs = ds(0) thetam + ds(nz) thetap,  es = ds(0) dthetam + ds(nz) dthetap,
//   dsg = green ds (interior), as = rkz dsg,
//   w = [0, dst(dsg) + bs, 0],  dw/dz = es + dct(as),
// with green(kz) = -1/(k^2 + l^2 + rkz^2) and the theta functions evaluated
// in registers: one read of ds (the second transform re-reads it from L2),
// one write each of w and dw/dz.
template <int M>
__global__ void __launch_bounds__(256, 2) k_colz_w(const float *__restrict__ ds, float *__restrict__ w,
                                                   float *__restrict__ es, int P, long long npairs,
                                                   const double *__restrict__ k2l2, const double *__restrict__ k2l2i,
                                                   float dz, float Lz, const float2 *__restrict__ twn,
                                                   const float *__restrict__ sinz, const float *__restrict__ cosz)
{
    constexpr int n = 32 * M;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    extern __shared__ __align__(16) unsigned char smz[];
    constexpr int XS = (32 * (M + 1) > n ? 32 * (M + 1) : n);
    constexpr int ZS = n + 1 + (n + 1) / 16 + 2;
    float2 *xs = reinterpret_cast<float2 *>(smz) + (size_t)wib * (XS + ZS);
    float *zA = reinterpret_cast<float *>(xs + XS);
    float *zB = zA + ZS;
    const float r2s = 1.41421356237309505f * rsqrtf((float)n);
    const float pk = 3.14159265358979324f / Lz;  // rkz(kz) = pk kz
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long pr = (long long)blockIdx.x * (blockDim.x >> 5) + wib; pr < npairs; pr += warps) {
        const long long cA = 2 * pr, cB = cA + 1;
        const long long oA = cA * P, oB = cB * P;
        // lanes 0..3 (column A) and 8..11 (column B): k^2+l^2, 1/(k^2+l^2),
        // ds(0), ds(nz)
        float par = 0.f;
        if (lane < 16 && (lane & 7) < 4) {
            const long long c = lane < 8 ? cA : cB;
            const int f = lane & 3;
            par = f == 0 ? (float)k2l2[c] : f == 1 ? (float)k2l2i[c] : ds[c * P + (f == 2 ? 0 : n)];
        }
        // ---- dst of dsg = green ds
        {
            const float k2A = lane_get(par, 0), k2B = lane_get(par, 8);
            float2 v[M];
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const int j = lane + 32 * m;
                v[m] = make_float2(0.f, 0.f);
                if (j > 0) {
                    const float rj = pk * (float)j, rn = pk * (float)(n - j);
                    const float rj2 = rj * rj, rn2 = rn * rn;
                    const float xa = __fdividef(-ds[oA + j], k2A + rj2), ya = __fdividef(-ds[oA + n - j], k2A + rn2);
                    const float xb = __fdividef(-ds[oB + j], k2B + rj2), yb = __fdividef(-ds[oB + n - j], k2B + rn2);
                    const float sj = __ldg(&sinz[j]);
                    v[m] = make_float2(0.5f * (xa - ya) + sj * (xa + ya), 0.5f * (xb - yb) + sj * (xb + yb));
                }
            }
            warp_fft<M>(v, xs, twn, lane);
        }
        post_dst<M>(xs, zA, zB, lane, r2s);
        __syncwarp();
        {
            const float d0A = lane_get(par, 2), dnA = lane_get(par, 3), d0B = lane_get(par, 10),
                        dnB = lane_get(par, 11);
            const Theta tA = Theta::make(sqrtf(lane_get(par, 0)), lane_get(par, 1), dz, Lz, n, cA == 0);
            const Theta tB = Theta::make(sqrtf(lane_get(par, 8)), lane_get(par, 9), dz, Lz, n, cB == 0);
            for (int iz = lane; iz <= n; iz += 32) {
                float ra = 0.f, rb = 0.f;
                if (iz > 0 && iz < n) {
                    float tm, tp, dtm, dtp;
                    tA.at(iz, tm, tp, dtm, dtp);
                    ra = zA[zpad(iz)] + d0A * tm + dnA * tp;
                    tB.at(iz, tm, tp, dtm, dtp);
                    rb = zB[zpad(iz)] + d0B * tm + dnB * tp;
                }
                w[oA + iz] = ra;
                w[oB + iz] = rb;
            }
        }
        __syncwarp();
        // ---- dct of as = rkz green ds (as(0) = as(nz) = 0)
        {
            const float k2A = lane_get(par, 0), k2B = lane_get(par, 8);
            // opaque copies of the offsets keep the compiler from hoisting
            // this phase's loads above the first transform (register spills)
            long long oA = cA * P, oB = cB * P;
            asm volatile("" : "+l"(oA), "+l"(oB));
            float2 v[M];
            float sA = 0.f, sB = 0.f;
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const int j = lane + 32 * m;
                v[m] = make_float2(0.f, 0.f);
                if (j > 0) {
                    const float rj = pk * (float)j, rn = pk * (float)(n - j);
                    const float rj2 = rj * rj, rn2 = rn * rn;
                    const float xa = __fdividef(-rj * ds[oA + j], k2A + rj2);
                    const float ya = __fdividef(-rn * ds[oA + n - j], k2A + rn2);
                    const float xb = __fdividef(-rj * ds[oB + j], k2B + rj2);
                    const float yb = __fdividef(-rn * ds[oB + n - j], k2B + rn2);
                    const float sj = __ldg(&sinz[j]), cj = __ldg(&cosz[j]);
                    sA += xa * cj;
                    sB += xb * cj;
                    v[m] = make_float2(0.5f * (xa + ya) - sj * (xa - ya), 0.5f * (xb + yb) - sj * (xb - yb));
                }
            }
            const float x1A = r2s * warp_sum(sA), x1B = r2s * warp_sum(sB);
            warp_fft<M>(v, xs, twn, lane);
            post_dct<M>(xs, zA, zB, lane, r2s, x1A, x1B);
        }
        __syncwarp();
        {
            const float d0A = lane_get(par, 2), dnA = lane_get(par, 3), d0B = lane_get(par, 10),
                        dnB = lane_get(par, 11);
            const Theta tA = Theta::make(sqrtf(lane_get(par, 0)), lane_get(par, 1), dz, Lz, n, cA == 0);
            const Theta tB = Theta::make(sqrtf(lane_get(par, 8)), lane_get(par, 9), dz, Lz, n, cB == 0);
            for (int iz = lane; iz <= n; iz += 32) {
                float tm, tp, dtm, dtp;
                tA.at(iz, tm, tp, dtm, dtp);
                const float ra = zA[zpad(iz)] + d0A * dtm + dnA * dtp;
                tB.at(iz, tm, tp, dtm, dtp);
                const float rb = zB[zpad(iz)] + d0B * dtm + dnB * dtp;
                es[oA + iz] = ra;
                es[oB + iz] = rb;
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------------
// es = decompose(central_diffz(combine(f))) in one kernel (the z part of
// the solenoidal projection, inversion.f90:41-47): combine through the
// warp FFT, the two-sided difference on the warp's z buffer, then the
// decomposition; one read of f and one write of es.
template <int M>
__global__ void __launch_bounds__(256, 2) k_colz_proj(const float *__restrict__ f, float *__restrict__ es, int P,
                                                      long long npairs, const double *__restrict__ k2l2, float dz,
                                                      float Lz, const float2 *__restrict__ twn,
                                                      const float *__restrict__ sinz)
{
    constexpr int n = 32 * M;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    extern __shared__ __align__(16) unsigned char smz[];
    constexpr int XS = (32 * (M + 1) > n ? 32 * (M + 1) : n);
    constexpr int ZS = n + 1 + (n + 1) / 16 + 2;
    float2 *xs = reinterpret_cast<float2 *>(smz) + (size_t)wib * (XS + ZS);
    float *zA = reinterpret_cast<float *>(xs + XS);
    float *zB = zA + ZS;
    // the derivative columns reuse the FFT buffer: 2 (n + 1) <= 2 XS floats
    float *gA = reinterpret_cast<float *>(xs), *gB = gA + (n + 1);
    const float r2s = 1.41421356237309505f * rsqrtf((float)n);
    const float dzi = 1.0f / dz, hdzi = 0.5f / dz;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long pr = (long long)blockIdx.x * (blockDim.x >> 5) + wib; pr < npairs; pr += warps) {
        const long long cA = 2 * pr, cB = cA + 1;
        const long long oA = cA * P, oB = cB * P;
        // lanes 0..2 (column A) and 8..10 (column B): k^2+l^2, f(0), f(nz)
        float par = 0.f;
        if (lane < 16 && (lane & 7) < 3) {
            const long long c = lane < 8 ? cA : cB;
            const int q = lane & 7;
            par = q == 0 ? (float)k2l2[c] : f[c * P + (q == 1 ? 0 : n)];
        }
        // ---- combine: dst of the interior, plus the harmonic part
        {
            float2 v[M];
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const int j = lane + 32 * m;
                v[m] = make_float2(0.f, 0.f);
                if (j > 0) {
                    const float xa = f[oA + j], ya = f[oA + n - j], xb = f[oB + j], yb = f[oB + n - j];
                    const float sj = __ldg(&sinz[j]);
                    v[m] = make_float2(0.5f * (xa - ya) + sj * (xa + ya), 0.5f * (xb - yb) + sj * (xb + yb));
                }
            }
            warp_fft<M>(v, xs, twn, lane);
        }
        post_dst<M>(xs, zA, zB, lane, r2s);
        __syncwarp();
        {
            const float f0A = lane_get(par, 1), fnA = lane_get(par, 2), f0B = lane_get(par, 9),
                        fnB = lane_get(par, 10);
            const Harm hA = Harm::make(sqrtf(lane_get(par, 0)), dz, Lz, n, cA == 0);
            const Harm hB = Harm::make(sqrtf(lane_get(par, 8)), dz, Lz, n, cB == 0);
            for (int iz = lane; iz <= n; iz += 32) {
                float ca, cb;
                if (iz == 0) {
                    ca = f0A;
                    cb = f0B;
                } else if (iz == n) {
                    ca = fnA;
                    cb = fnB;
                } else {
                    float pm, pp;
                    hA.at(iz, n, pm, pp);
                    ca = zA[zpad(iz)] + f0A * pm + fnA * pp;
                    hB.at(iz, n, pm, pp);
                    cb = zB[zpad(iz)] + f0B * pm + fnB * pp;
                }
                zA[zpad(iz)] = ca;
                zB[zpad(iz)] = cb;
            }
        }
        __syncwarp();
        // ---- central_diffz (inversion_utils.f90:653-673) into gA / gB
        for (int iz = lane; iz <= n; iz += 32) {
            const int lo = iz == 0 ? 0 : iz - 1, hi = iz == n ? n : iz + 1;
            const float sc = (iz == 0 || iz == n) ? dzi : hdzi;
            gA[iz] = (zA[zpad(hi)] - zA[zpad(lo)]) * sc;
            gB[iz] = (zB[zpad(hi)] - zB[zpad(lo)]) * sc;
        }
        __syncwarp();
        // ---- decompose: subtract the harmonic part, dst
        {
            const float g0A = gA[0], gnA = gA[n], g0B = gB[0], gnB = gB[n];
            const Harm hA = Harm::make(sqrtf(lane_get(par, 0)), dz, Lz, n, cA == 0);
            const Harm hB = Harm::make(sqrtf(lane_get(par, 8)), dz, Lz, n, cB == 0);
            float2 v[M];
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const int j = lane + 32 * m;
                v[m] = make_float2(0.f, 0.f);
                if (j > 0) {
                    float xa = gA[j], ya = gA[n - j], xb = gB[j], yb = gB[n - j];
                    float pm, pp;
                    hA.at(j, n, pm, pp);
                    xa -= g0A * pm + gnA * pp;
                    ya -= g0A * pp + gnA * pm;
                    hB.at(j, n, pm, pp);
                    xb -= g0B * pm + gnB * pp;
                    yb -= g0B * pp + gnB * pm;
                    const float sj = __ldg(&sinz[j]);
                    v[m] = make_float2(0.5f * (xa - ya) + sj * (xa + ya), 0.5f * (xb - yb) + sj * (xb + yb));
                }
            }
            // the boundary rows pass through unchanged
            if (lane == 0) {
                zA[zpad(0)] = g0A;
                zB[zpad(0)] = g0B;
                zA[zpad(n)] = gnA;
                zB[zpad(n)] = gnB;
            }
            __syncwarp();
            warp_fft<M>(v, xs, twn, lane);
        }
        post_dst<M>(xs, zA, zB, lane, r2s);
        __syncwarp();
        for (int iz = lane; iz <= n; iz += 32) {
            es[oA + iz] = zA[zpad(iz)];
            es[oB + iz] = zB[zpad(iz)];
        }
        __syncwarp();
    }
}

namespace {
template <int M> constexpr size_t colz_smem_per_warp()
{
    constexpr int n = 32 * M;
    constexpr int XS = (32 * (M + 1) > n ? 32 * (M + 1) : n);
    constexpr int ZS = n + 1 + (n + 1) / 16 + 2;
    return XS * sizeof(float2) + 2 * ZS * sizeof(float);
}

template <int MODE, int M, typename TIN>
void launch_colz_m(const TIN *in, float *out, const Dims &d, cudaStream_t st, const double *k2l2, float dz, float Lz,
                   const float2 *twn, const float *sinz, const float *cosz)
{
    const long long npairs = d.ncol / 2;
    const size_t sm = 8 * colz_smem_per_warp<M>();
    long long nb = (npairs + 7) / 8;
    if (nb > 152 * 24) nb = 152 * 24;
    k_colz<MODE, M, TIN><<<(unsigned)nb, 256, sm, st>>>(in, out, d.P, npairs, k2l2, dz, Lz, twn, sinz, cosz);
}

template <int MODE, typename TIN>
void launch_colz(const TIN *in, float *out, const Dims &d, cudaStream_t st, const double *k2l2, float dz, float Lz,
                 const float2 *twn, const float *sinz, const float *cosz)
{
    switch (d.nz) {
    case 64: launch_colz_m<MODE, 2, TIN>(in, out, d, st, k2l2, dz, Lz, twn, sinz, cosz); break;
    case 128: launch_colz_m<MODE, 4, TIN>(in, out, d, st, k2l2, dz, Lz, twn, sinz, cosz); break;
    case 256: launch_colz_m<MODE, 8, TIN>(in, out, d, st, k2l2, dz, Lz, twn, sinz, cosz); break;
    case 512: launch_colz_m<MODE, 16, TIN>(in, out, d, st, k2l2, dz, Lz, twn, sinz, cosz); break;
    default: launch_colz_m<MODE, 32, TIN>(in, out, d, st, k2l2, dz, Lz, twn, sinz, cosz); break;
    }
}

template <int MODE, int M, typename TIN> void attr_m()
{
    cudaFuncSetAttribute(k_colz<MODE, M, TIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(8 * colz_smem_per_warp<M>()));
}
template <int MODE, typename TIN> void attr_mode()
{
    attr_m<MODE, 2, TIN>();
    attr_m<MODE, 4, TIN>();
    attr_m<MODE, 8, TIN>();
    attr_m<MODE, 16, TIN>();
    attr_m<MODE, 32, TIN>();
}
template <typename TIN> void attr_all()
{
    attr_mode<COL_DST, TIN>();
    attr_mode<COL_DCT, TIN>();
    attr_mode<COL_DECOMP, TIN>();
    attr_mode<COL_COMBINE, TIN>();
}
}  // namespace

template <int M>
static void launch_w_m(const Dims &d, cudaStream_t st, const float *ds, float *w, float *es, const double *k2l2,
                       const double *k2l2i, float dz, float Lz, const float2 *twn, const float *sinz, const float *cosz)
{
    const long long npairs = d.ncol / 2;
    long long nb = (npairs + 7) / 8;
    if (nb > 152 * 24) nb = 152 * 24;
    k_colz_w<M><<<(unsigned)nb, 256, 8 * colz_smem_per_warp<M>(), st>>>(ds, w, es, d.P, npairs, k2l2, k2l2i, dz, Lz,
                                                                         twn, sinz, cosz);
}
template <int M>
static void launch_proj_m(const Dims &d, cudaStream_t st, const float *f, float *es, const double *k2l2, float dz,
                          float Lz, const float2 *twn, const float *sinz)
{
    const long long npairs = d.ncol / 2;
    long long nb = (npairs + 7) / 8;
    if (nb > 152 * 24) nb = 152 * 24;
    k_colz_proj<M><<<(unsigned)nb, 256, 8 * colz_smem_per_warp<M>(), st>>>(f, es, d.P, npairs, k2l2, dz, Lz, twn,
                                                                            sinz);
}

void columns_w(const Dims &d, cudaStream_t st, const float *ds, float *w, float *es, const double *k2l2,
               const double *k2l2i, float dz, float Lz, const float2 *twn, const float *sinz, const float *cosz,
               Probe *pr)
{
    if (pr) pr->begin(PROBE_COLUMNS, st);
    switch (d.nz) {
    case 64: launch_w_m<2>(d, st, ds, w, es, k2l2, k2l2i, dz, Lz, twn, sinz, cosz); break;
    case 128: launch_w_m<4>(d, st, ds, w, es, k2l2, k2l2i, dz, Lz, twn, sinz, cosz); break;
    case 256: launch_w_m<8>(d, st, ds, w, es, k2l2, k2l2i, dz, Lz, twn, sinz, cosz); break;
    case 512: launch_w_m<16>(d, st, ds, w, es, k2l2, k2l2i, dz, Lz, twn, sinz, cosz); break;
    default: launch_w_m<32>(d, st, ds, w, es, k2l2, k2l2i, dz, Lz, twn, sinz, cosz); break;
    }
    if (pr) pr->end(PROBE_COLUMNS, st, 3.0 * (double)d.ncol * (double)(d.nz + 1) * sizeof(float));
}

void columns_proj(const Dims &d, cudaStream_t st, const float *f, float *es, const double *k2l2, float dz, float Lz,
                  const float2 *twn, const float *sinz, Probe *pr)
{
    if (pr) pr->begin(PROBE_COLUMNS, st);
    switch (d.nz) {
    case 64: launch_proj_m<2>(d, st, f, es, k2l2, dz, Lz, twn, sinz); break;
    case 128: launch_proj_m<4>(d, st, f, es, k2l2, dz, Lz, twn, sinz); break;
    case 256: launch_proj_m<8>(d, st, f, es, k2l2, dz, Lz, twn, sinz); break;
    case 512: launch_proj_m<16>(d, st, f, es, k2l2, dz, Lz, twn, sinz); break;
    default: launch_proj_m<32>(d, st, f, es, k2l2, dz, Lz, twn, sinz); break;
    }
    if (pr) pr->end(PROBE_COLUMNS, st, 2.0 * (double)d.ncol * (double)(d.nz + 1) * sizeof(float));
}

bool colz_supported(int nz) { return nz == 64 || nz == 128 || nz == 256 || nz == 512 || nz == 1024; }

void colz_init()
{
    float2 w[32];
    for (int j = 0; j < 32; ++j) {
        const double a = 2.0 * 3.14159265358979323846 * (double)j / 32.0;
        double c = cos(a), sn = sin(a);
        if (j % 8 == 0) {
            const int q = j / 8;
            c = (q == 0) ? 1.0 : (q == 2 ? -1.0 : 0.0);
            sn = (q == 1) ? 1.0 : (q == 3 ? -1.0 : 0.0);
        }
        w[j] = make_float2((float)c, (float)(-sn));
    }
    cudaMemcpyToSymbol(c_w32z, w, sizeof(w));
    attr_all<float>();
    attr_all<double>();
    cudaFuncSetAttribute(k_colz_w<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(8 * colz_smem_per_warp<16>()));
    cudaFuncSetAttribute(k_colz_w<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(8 * colz_smem_per_warp<32>()));
    cudaFuncSetAttribute(k_colz_proj<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(8 * colz_smem_per_warp<16>()));
    cudaFuncSetAttribute(k_colz_proj<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(8 * colz_smem_per_warp<32>()));
}

template <typename TIN>
void columns_z(const Dims &d, cudaStream_t st, int mode, const TIN *in, float *out, const double *k2l2, float dz,
               float Lz, const float2 *twn, const float *sinz, const float *cosz, Probe *pr)
{
    if (pr) pr->begin(PROBE_COLUMNS, st);
    switch (mode) {
    case COL_DST: launch_colz<COL_DST, TIN>(in, out, d, st, k2l2, dz, Lz, twn, sinz, cosz); break;
    case COL_DCT: launch_colz<COL_DCT, TIN>(in, out, d, st, k2l2, dz, Lz, twn, sinz, cosz); break;
    case COL_DECOMP: launch_colz<COL_DECOMP, TIN>(in, out, d, st, k2l2, dz, Lz, twn, sinz, cosz); break;
    default: launch_colz<COL_COMBINE, TIN>(in, out, d, st, k2l2, dz, Lz, twn, sinz, cosz); break;
    }
    if (pr) pr->end(PROBE_COLUMNS, st, 2.0 * (double)d.ncol * (double)(d.nz + 1) * sizeof(float));
}

template void columns_z<float>(const Dims &, cudaStream_t, int, const float *, float *, const double *, float, float,
                               const float2 *, const float *, const float *, Probe *);
template void columns_z<double>(const Dims &, cudaStream_t, int, const double *, float *, const double *, float,
                                float, const float2 *, const float *, const float *, Probe *);

}  // namespace ps3d
