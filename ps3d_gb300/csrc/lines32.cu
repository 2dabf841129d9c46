// FP32 line FFTs of the mixed form (fftxyp2s / fftxys2p of
// src/fft/sta3dfft.f90:136-260 in the Hermitian storage of
// src/fft/stafft.f90:55-58), tuned for HBM bandwidth.
//
// A block owns 32 consecutive z values (one 128-byte row segment per line
// index) of one line set: 16 complex lanes, each packing two real lines
// (z, z+1).  A thread carries two adjacent lanes as one float4, so every
// global and shared-memory access moves 16 bytes and eight threads cover a
// 128-byte row.  The Stockham passes keep their butterflies in registers:
// the first pass of a forward transform loads its inputs straight from HBM
// (coalesced 128-byte rows), the last pass of an inverse transform stores
// straight to HBM, and the passes in between exchange through one shared
// buffer laid out [line index][lane] so every access is bank-conflict free.
// The first pass of an inverse transform rebuilds the packed spectrum from
// the Hermitian rows k and N - k as it loads them (one lane per thread
// there, to bound the registers).  N (the line length) is a compile-time
// constant: 64..1024.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "kernels.h"

namespace ps3d {

namespace {

constexpr int LANES = 16;  // complex lanes per block
constexpr int PAIRS = 8;   // threads per row (two lanes each)

// Block shape W at N = 512: 0 = 512-thread blocks, two per SM (64
// registers); 1 = 256-thread blocks, three per SM (85 registers).  The
// autotuner picks one per pass; by default the forward transform takes 0
// and the inverse (its Hermitian first pass needs more registers) takes 1.
// N = 1024 always runs one 512-thread block per SM (128 KB of shared
// memory), N <= 256 three 256-thread blocks.
template <int N, bool INV, int W> struct LinePlan {
    static constexpr bool BIG = N >= 1024 || (N == 512 && W == 0);
    static constexpr int T = BIG ? 512 : 256;  // threads per block
    static constexpr int G = T / PAIRS;        // butterfly groups
    static constexpr int MINB = N >= 1024 ? 1 : (BIG ? 2 : 3);
};

__device__ __forceinline__ float2 cm(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float4 f4(float2 a, float2 b) { return make_float4(a.x, a.y, b.x, b.y); }

template <int R, bool INV> __device__ __forceinline__ void dftR(float2 *v) { dft<R, INV, float2>(v); }

// one radix-R Stockham pass with span NS over N points: inputs x[j + r N/R]
// of butterfly j, outputs at (j - k) R + k + r NS, k = j mod NS; each thread
// applies it to its two lanes
template <int N, int R, int NS, bool INV, int W, bool FROM_GLOBAL, bool TO_GLOBAL>
__device__ __forceinline__ void pass(float4 *sm, const float4 *__restrict__ gin, float4 *__restrict__ gout,
                                     long long gstride, bool valid, float scale, const float2 *__restrict__ tw,
                                     int nval = 4)
{
    constexpr int G = LinePlan<N, INV, W>::G;
    constexpr int NB = N / R;              // butterflies per lane
    constexpr int NBT = (NB + G - 1) / G;  // per thread
    const int p = threadIdx.x & (PAIRS - 1), g = threadIdx.x / PAIRS;
    float2 va[NBT][R], vb[NBT][R];
#pragma unroll
    for (int q = 0; q < NBT; ++q) {
        const int j = g + G * q;
        if (NB % G == 0 || j < NB) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int row = j + r * NB;
                float4 x;
                if (FROM_GLOBAL) {
                    x = valid ? gin[row * gstride] : make_float4(0.f, 0.f, 0.f, 0.f);
                    // z rows beyond the top wall (padding) enter as zero: the
                    // paired real line must not pick up leftover content
                    if (nval < 4) {
                        x.w = 0.f;
                        if (nval < 3) x.z = 0.f;
                        if (nval < 2) x.y = 0.f;
                        if (nval < 1) x.x = 0.f;
                    }
                } else {
                    x = sm[row * PAIRS + p];
                }
                va[q][r] = lo2(x);
                vb[q][r] = hi2(x);
            }
        }
    }
    if (!FROM_GLOBAL) __syncthreads();
#pragma unroll
    for (int q = 0; q < NBT; ++q) {
        const int j = g + G * q;
        if (NB % G == 0 || j < NB) {
            const int k = j & (NS - 1);
            if (NS > 1) {
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    float2 w = __ldg(&tw[k * r * (N / (NS * R))]);
                    if (INV) w.y = -w.y;
                    va[q][r] = cm(va[q][r], w);
                    vb[q][r] = cm(vb[q][r], w);
                }
            }
            dftR<R, INV>(va[q]);
            dftR<R, INV>(vb[q]);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int row = (j - k) * R + k + r * NS;
                if (TO_GLOBAL) {
                    if (valid)
                        gout[row * gstride] = make_float4(va[q][r].x * scale, va[q][r].y * scale,
                                                          vb[q][r].x * scale, vb[q][r].y * scale);
                } else {
                    sm[row * PAIRS + p] = f4(va[q][r], vb[q][r]);
                }
            }
        }
    }
    __syncthreads();
}

// C_k = A_k + i B_k of the two packed lines from the Hermitian rows
// lo = H[min(k, N-k)] and hi = H[max(k, N-k)] (stafft.f90:55-58 storage)
__device__ __forceinline__ float2 herm_low(float2 lo, float2 hi) { return make_float2(lo.x - hi.y, hi.x + lo.y); }
__device__ __forceinline__ float2 herm_high(float2 lo, float2 hi) { return make_float2(lo.x + hi.y, lo.y - hi.x); }

// First radix-8 pass (span 1) of an inverse transform straight from the
// Hermitian rows in HBM.  Butterfly j reads rows j + r N/8, whose mirrors
// N - row are the rows of butterfly N/8 - j: one work item is such a pair of
// butterflies (slot s: s and N/8 - s; slot 0: butterflies 0 and N/16, each
// its own mirror) for one lane, so every row is loaded once and used for
// both C_k and C_{N-k}.  Items: slots x 16 lanes over the block's threads.
template <int N, int W>
__device__ __forceinline__ void herm_first_pass(float2 *sm2, const float2 *__restrict__ gin2, long long gs2,
                                                int z0, int P, int zv)
{
    constexpr int T = LinePlan<N, true, W>::T, NB = N / 8, SLOTS = NB / 2;
    constexpr int ITEMS = SLOTS * LANES, IPT = (ITEMS + T - 1) / T;
#pragma unroll 1
    for (int q = 0; q < IPT; ++q) {
        const int it = threadIdx.x + T * q;
        if (!(ITEMS % T == 0 || it < ITEMS)) continue;
        const int lane = it & (LANES - 1), s = it / LANES;
        const bool valid = z0 + 2 * lane < P;
        const float2 *g = gin2 + lane;
        const int j1 = s == 0 ? 0 : s, j2 = s == 0 ? NB / 2 : NB - s;
        float2 h1[8], h2[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            h1[r] = valid ? g[(j1 + r * NB) * gs2] : make_float2(0.f, 0.f);
            h2[r] = valid ? g[(j2 + r * NB) * gs2] : make_float2(0.f, 0.f);
        }
        // padding rows (z >= zv) enter as zero
        const int nv = zv - (z0 + 2 * lane);
        if (nv < 2) {
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                h1[r].y = 0.f;
                h2[r].y = 0.f;
                if (nv < 1) {
                    h1[r].x = 0.f;
                    h2[r].x = 0.f;
                }
            }
        }
        float2 a[8], b[8];
        if (s == 0) {
            // butterfly 0: rows r N/8, mirror index 8 - r; rows 0 and N/2 are
            // their own mirrors (imaginary rows absent)
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int rm = (8 - r) & 7;
                a[r] = (r == 0 || r == 4) ? h1[r] : (r < 4 ? herm_low(h1[r], h1[rm]) : herm_high(h1[rm], h1[r]));
            }
            // butterfly N/16: mirror index 7 - r
#pragma unroll
            for (int r = 0; r < 8; ++r)
                b[r] = r < 4 ? herm_low(h2[r], h2[7 - r]) : herm_high(h2[7 - r], h2[r]);
        } else {
            // row j1 + r N/8 mirrors row j2 + (7 - r) N/8; it is the lower
            // row of the pair for r < 4
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                if (r < 4) {
                    a[r] = herm_low(h1[r], h2[7 - r]);
                    b[7 - r] = herm_high(h1[r], h2[7 - r]);
                } else {
                    a[r] = herm_high(h2[7 - r], h1[r]);
                    b[7 - r] = herm_low(h2[7 - r], h1[r]);
                }
            }
        }
        dftR<8, true>(a);
        dftR<8, true>(b);
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            sm2[(j1 * 8 + r) * LANES + lane] = a[r];
            sm2[(j2 * 8 + r) * LANES + lane] = b[r];
        }
    }
    __syncthreads();
}

// the passes after the first for N = 8^a * {1, 2, 4}
template <int N, bool INV, int W, bool TO_GLOBAL>
__device__ __forceinline__ void later_passes(float4 *sm, float4 *gout, long long gs, bool valid, float scale,
                                             const float2 *tw)
{
    if constexpr (N == 64) {
        pass<N, 8, 8, INV, W, false, TO_GLOBAL>(sm, nullptr, gout, gs, valid, scale, tw);
    } else if constexpr (N == 128) {
        pass<N, 8, 8, INV, W, false, false>(sm, nullptr, gout, gs, valid, scale, tw);
        pass<N, 2, 64, INV, W, false, TO_GLOBAL>(sm, nullptr, gout, gs, valid, scale, tw);
    } else if constexpr (N == 256) {
        pass<N, 8, 8, INV, W, false, false>(sm, nullptr, gout, gs, valid, scale, tw);
        pass<N, 4, 64, INV, W, false, TO_GLOBAL>(sm, nullptr, gout, gs, valid, scale, tw);
    } else if constexpr (N == 512) {
        pass<N, 8, 8, INV, W, false, false>(sm, nullptr, gout, gs, valid, scale, tw);
        pass<N, 8, 64, INV, W, false, TO_GLOBAL>(sm, nullptr, gout, gs, valid, scale, tw);
    } else {  // 1024
        pass<N, 8, 8, INV, W, false, false>(sm, nullptr, gout, gs, valid, scale, tw);
        pass<N, 8, 64, INV, W, false, false>(sm, nullptr, gout, gs, valid, scale, tw);
        pass<N, 2, 512, INV, W, false, TO_GLOBAL>(sm, nullptr, gout, gs, valid, scale, tw);
    }
}

template <int N, bool INV, int W>
__global__ void __launch_bounds__(LinePlan<N, INV, W>::T, LinePlan<N, INV, W>::MINB)
    k_lines32(const float *__restrict__ in, float *__restrict__ out, int P, int zv, long long line_stride,
              long long batch_stride, const float2 *__restrict__ tw, long long fs_in, long long fs_out)
{
    extern __shared__ __align__(16) float4 smL[];
    // several fields per launch: field blockIdx.z at in + z fs_in, out + z fs_out
    in += blockIdx.z * fs_in;
    out += blockIdx.z * fs_out;
    constexpr int T = LinePlan<N, INV, W>::T;
    const int p = threadIdx.x & (PAIRS - 1);
    const int z0 = blockIdx.x * 2 * LANES;
    const bool valid = z0 + 4 * p < P;  // P is a multiple of 8: both lanes or neither
    const long long base = (long long)blockIdx.y * batch_stride + z0;  // floats
    const float s = rsqrtf((float)N);
    constexpr int H = N / 2;
    if (!INV) {
        const long long gs = line_stride >> 2;  // float4 units
        const float4 *gin = reinterpret_cast<const float4 *>(in + base) + p;
        pass<N, 8, 1, false, W, true, false>(smL, gin, nullptr, gs, valid, 1.0f, tw, zv - (z0 + 4 * p));
        later_passes<N, false, W, false>(smL, nullptr, gs, valid, 1.0f, tw);
        // split the two packed real transforms of each lane and store the
        // Hermitian rows k and N - k
        float4 *o = reinterpret_cast<float4 *>(out + base);
        for (int e = threadIdx.x; e < (H + 1) * PAIRS; e += T) {
            const int k = e / PAIRS, q = e & (PAIRS - 1);
            if (z0 + 4 * q >= P) continue;
            const float4 ck = smL[k * PAIRS + q];
            const float4 cn = smL[((N - k) & (N - 1)) * PAIRS + q];
            // lane 0 in (x, y), lane 1 in (z, w); A = real line z, B = z + 1
            const float4 re = make_float4(0.5f * (ck.x + cn.x) * s, 0.5f * (ck.y + cn.y) * s,
                                          0.5f * (ck.z + cn.z) * s, 0.5f * (ck.w + cn.w) * s);
            o[k * gs + q] = re;
            if (k > 0 && k < H)
                o[(N - k) * gs + q] = make_float4(0.5f * (ck.y - cn.y) * s, -0.5f * (ck.x - cn.x) * s,
                                                  0.5f * (ck.w - cn.w) * s, -0.5f * (ck.z - cn.z) * s);
        }
    } else {
        herm_first_pass<N, W>(reinterpret_cast<float2 *>(smL), reinterpret_cast<const float2 *>(in + base),
                              line_stride >> 1, z0, P, zv);
        const long long gs = line_stride >> 2;
        float4 *gout = reinterpret_cast<float4 *>(out + base) + p;
        later_passes<N, true, W, true>(smL, gout, gs, valid, s, tw);
    }
}

template <int N, bool INV, int W>
void launch32w(cudaStream_t st, const float *in, float *out, int P, int zv, long long ls, long long nbatch,
               long long bs, const float2 *tw, int nf, long long fs_in, long long fs_out)
{
    dim3 grid((P + 2 * LANES - 1) / (2 * LANES), (unsigned)nbatch, (unsigned)nf);
    const size_t sm = (size_t)N * LANES * sizeof(float2);
    k_lines32<N, INV, W><<<grid, LinePlan<N, INV, W>::T, sm, st>>>(in, out, P, zv, ls, bs, tw, fs_in, fs_out);
}


// ------------------------------------------------------------------------
// Forward y lines of the five products of vorticity_tendency straight from
// the velocity and vorticity (inversion.f90:298-340, mixed form).  Three
// blocks per 32-level tile of an x column (blockIdx.x = 3 * tile + o):
//   o = 0: r = u eta - v xi,
//   o = 1: q = w xi - u zeta  and dq/dz,
//   o = 2: p = v zeta - w eta and dp/dz
// (central_diffz, inversion_utils.f90:653-673: one-sided at iz = 0 and
// iz = nz, centred in between).  The first radix-8 pass forms the product at
// each of the block's (y, z) points from the physical u, omega there, so the
// products never go to HBM; blocks 1 and 2 also form the z derivative from
// the same values (the z neighbours of a thread's four levels come from the
// adjacent threads of its row by shuffles, the levels just outside the
// block's 32 from scalar loads) and park it in the derivative's output tile,
// which the same threads read back for its own line transform once the
// product's is stored (the tile is still in L2).  The three blocks of a tile
// are consecutive, so the tile's velocity and vorticity come from DRAM
// about once and from L2 after that.  The passes and the Hermitian stores
// are those of k_lines32; out holds r, q, p, dq/dz, dp/dz nfield apart.
struct ProdSrc {
    const float *vel, *vor;  // three components each, nfield apart
    long long nfield;
    float dzi, hdzi;
    int nz;
};

template <int N, int W>
__global__ void __launch_bounds__(LinePlan<N, false, W>::T, LinePlan<N, false, W>::MINB)
    k_lines32_prod(ProdSrc ps, float *__restrict__ out, int P, long long line_stride, long long batch_stride,
                   const float2 *__restrict__ tw)
{
    extern __shared__ __align__(16) float4 smL[];
    constexpr int T = LinePlan<N, false, W>::T, G = LinePlan<N, false, W>::G;
    constexpr int R = 8, NB = N / R, NBT = (NB + G - 1) / G;
    // butterflies j >= NB (N <= 128) leave whole warps idle: a warp's four
    // row groups are g = 4w..4w+3 and NB is a multiple of 4, so the
    // shuffles below always run on full warps
    static_assert(NB % 4 == 0 && PAIRS == 8, "warp-uniform butterfly ranges");
    const int o = blockIdx.x % 3;
    const int z0 = (blockIdx.x / 3) * 2 * LANES;
    const int p = threadIdx.x & (PAIRS - 1), g = threadIdx.x / PAIRS;
    const int zt = z0 + 4 * p;  // first of the thread's four levels
    const bool valid = zt < P;  // P is a multiple of 8: all four or none
    const long long base = (long long)blockIdx.y * batch_stride + z0;
    const long long Nf = ps.nfield;
    const float *u = ps.vel, *v = ps.vel + Nf, *w = ps.vel + 2 * Nf;
    const float *xi = ps.vor, *eta = ps.vor + Nf, *zeta = ps.vor + 2 * Nf;
    const int nz = ps.nz;
    const int nval = nz + 1 - zt;  // levels of the thread's four below the top wall
    float *dout = o ? out + (long long)(o + 2) * Nf : nullptr;  // dq/dz or dp/dz
    // the product of block o at one point
    auto prod = [&](long long i) -> float {
        if (o == 0) return u[i] * eta[i] - v[i] * xi[i];
        if (o == 1) return w[i] * xi[i] - u[i] * zeta[i];
        return v[i] * zeta[i] - w[i] * eta[i];
    };
    auto prod4 = [&](long long i) -> float4 {
        const float4 *U = reinterpret_cast<const float4 *>(u + i), *V = reinterpret_cast<const float4 *>(v + i),
                     *Wv = reinterpret_cast<const float4 *>(w + i);
        const float4 *X = reinterpret_cast<const float4 *>(xi + i), *E = reinterpret_cast<const float4 *>(eta + i),
                     *Z = reinterpret_cast<const float4 *>(zeta + i);
        float4 a, b, c, d;
        if (o == 0) {
            a = *U; b = *E; c = *V; d = *X;
        } else if (o == 1) {
            a = *Wv; b = *X; c = *U; d = *Z;
        } else {
            a = *V; b = *Z; c = *Wv; d = *E;
        }
        return make_float4(a.x * b.x - c.x * d.x, a.y * b.y - c.y * d.y, a.z * b.z - c.z * d.z,
                           a.w * b.w - c.w * d.w);
    };
    // levels above the top wall (padding) enter as zero
    auto mask = [&](float4 f) {
        if (nval < 4) {
            f.w = 0.f;
            if (nval < 3) f.z = 0.f;
            if (nval < 2) f.y = 0.f;
            if (nval < 1) f.x = 0.f;
        }
        return f;
    };
    // the product at (row, levels zt..zt+3); blocks 1, 2 write its z
    // derivative there to their derivative's output tile
    auto load = [&](int row) -> float4 {
        const long long i = base + (long long)row * line_stride + 4 * p;
        const float4 f = valid ? prod4(i) : make_float4(0.f, 0.f, 0.f, 0.f);
        if (o) {
            // neighbours zt - 1 and zt + 4: from the threads beside this one
            // in the row, or loaded at the block's edges
            float fm = __shfl_up_sync(0xffffffffu, f.w, 1);
            float fp = __shfl_down_sync(0xffffffffu, f.x, 1);
            if (p == 0) fm = (valid && zt > 0) ? prod(i - 1) : 0.f;
            if (p == PAIRS - 1) fp = (valid && zt + 4 <= nz) ? prod(i + 4) : 0.f;
            const float lv[6] = {fm, f.x, f.y, f.z, f.w, fp};
            float dv[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int iz = zt + c;
                if (iz == 0) dv[c] = (lv[c + 2] - lv[c + 1]) * ps.dzi;
                else if (iz == nz) dv[c] = (lv[c + 1] - lv[c]) * ps.dzi;
                else dv[c] = (lv[c + 2] - lv[c]) * ps.hdzi;
            }
            if (valid) *reinterpret_cast<float4 *>(dout + i) = mask(make_float4(dv[0], dv[1], dv[2], dv[3]));
        }
        return mask(f);
    };
    const long long gs = line_stride >> 2;
    const float s = rsqrtf((float)N);
    constexpr int H = N / 2;
    // split the two packed real transforms of each lane, store the
    // Hermitian rows k and N - k (as k_lines32)
    auto store = [&](float *dst) {
        float4 *ob = reinterpret_cast<float4 *>(dst + base);
        for (int e = threadIdx.x; e < (H + 1) * PAIRS; e += T) {
            const int k = e / PAIRS, q = e & (PAIRS - 1);
            if (z0 + 4 * q >= P) continue;
            const float4 ck = smL[k * PAIRS + q];
            const float4 cn = smL[((N - k) & (N - 1)) * PAIRS + q];
            const float4 re = make_float4(0.5f * (ck.x + cn.x) * s, 0.5f * (ck.y + cn.y) * s,
                                          0.5f * (ck.z + cn.z) * s, 0.5f * (ck.w + cn.w) * s);
            ob[k * gs + q] = re;
            if (k > 0 && k < H)
                ob[(N - k) * gs + q] = make_float4(0.5f * (ck.y - cn.y) * s, -0.5f * (ck.x - cn.x) * s,
                                                   0.5f * (ck.w - cn.w) * s, -0.5f * (ck.z - cn.z) * s);
        }
    };
    // first radix-8 pass (span 1) of the product: butterfly j reads rows
    // j + r N/8 and writes rows 8 j + r
    {
        float2 va[NBT][R], vb[NBT][R];
#pragma unroll
        for (int q = 0; q < NBT; ++q) {
            const int j = g + G * q;
            if (NB % G == 0 || j < NB) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const float4 x = load(j + r * NB);
                    va[q][r] = lo2(x);
                    vb[q][r] = hi2(x);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < NBT; ++q) {
            const int j = g + G * q;
            if (!(NB % G == 0 || j < NB)) continue;
            dftR<R, false>(va[q]);
            dftR<R, false>(vb[q]);
#pragma unroll
            for (int r = 0; r < R; ++r) smL[(j * R + r) * PAIRS + p] = f4(va[q][r], vb[q][r]);
        }
        __syncthreads();
    }
    later_passes<N, false, W, false>(smL, nullptr, gs, valid, 1.0f, tw);
    store(out + (long long)o * Nf);
    if (!o) return;
    // the derivative: each thread reads back the values it parked (its own
    // rows and levels), then the same transform in place
    __syncthreads();
    const float4 *gin = reinterpret_cast<const float4 *>(dout + base) + p;
    pass<N, 8, 1, false, W, true, false>(smL, gin, nullptr, gs, valid, 1.0f, tw, nval);
    later_passes<N, false, W, false>(smL, nullptr, gs, valid, 1.0f, tw);
    store(dout);
}

template <int N, int W>
void launch_prod(cudaStream_t st, const ProdSrc &ps, float *out, int P, int nx, int ny, const float2 *tw)
{
    const int ztiles = (P + 2 * LANES - 1) / (2 * LANES);
    dim3 grid((unsigned)(3 * ztiles), (unsigned)nx);
    const size_t sm = (size_t)N * LANES * sizeof(float2);
    k_lines32_prod<N, W><<<grid, LinePlan<N, false, W>::T, sm, st>>>(ps, out, P, P, (long long)ny * P, tw);
}

// ------------------------------------------------------------------------
// TMA-fed persistent form (N = 128, 256, 512).  One block per SM owns two
// tile buffers in shared memory; while it transforms the tile in one
// buffer, a cp.async.bulk.tensor copy brings its next tile into the other,
// so the loads of a block overlap its arithmetic.  A tile is the same
// 32-level slab of one line set as above, copied as N rows of 128 bytes by
// 3-D tensor copies (z, y, x) of at most 256 rows each.  The tensor's z
// extent is nz + 1, so the copy fills the padding rows above the top wall
// with zeros.  The butterflies are those of the kernel above, the first
// pass reading the tile from shared memory.  Every mbarrier wait is bounded
// (about a second); one that runs out sets the error word and the block
// stops taking tiles (the host reports PS3D_ERR_DEVICE_LIMIT).
__device__ unsigned int g_lines_err;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool tma_wait(uint32_t bar, uint32_t parity)
{
    for (int i = 0; i < (1 << 21); ++i) {
        uint32_t ok;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        if (i > 32) __nanosleep(128);
    }
    return false;
}

// the inverse transform's first pass from the Hermitian rows of the tile in
// shared memory (the same items as herm_first_pass; every thread holds at
// most one item, read completely before the buffer is overwritten)
template <int N, int W> __device__ __forceinline__ void herm_first_pass_smem(float2 *sm2)
{
    constexpr int T = LinePlan<N, true, W>::T, NB = N / 8, SLOTS = NB / 2;
    constexpr int ITEMS = SLOTS * LANES;
    static_assert(ITEMS <= T, "one item per thread");
    const int it = threadIdx.x;
    const bool act = it < ITEMS;
    const int lane = it & (LANES - 1), s = it / LANES;
    const int j1 = s == 0 ? 0 : s, j2 = s == 0 ? NB / 2 : NB - s;
    float2 h1[8], h2[8];
    if (act) {
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            h1[r] = sm2[(j1 + r * NB) * LANES + lane];
            h2[r] = sm2[(j2 + r * NB) * LANES + lane];
        }
    }
    __syncthreads();
    if (act) {
        float2 a[8], b[8];
        if (s == 0) {
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int rm = (8 - r) & 7;
                a[r] = (r == 0 || r == 4) ? h1[r] : (r < 4 ? herm_low(h1[r], h1[rm]) : herm_high(h1[rm], h1[r]));
            }
#pragma unroll
            for (int r = 0; r < 8; ++r)
                b[r] = r < 4 ? herm_low(h2[r], h2[7 - r]) : herm_high(h2[7 - r], h2[r]);
        } else {
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                if (r < 4) {
                    a[r] = herm_low(h1[r], h2[7 - r]);
                    b[7 - r] = herm_high(h1[r], h2[7 - r]);
                } else {
                    a[r] = herm_high(h2[7 - r], h1[r]);
                    b[7 - r] = herm_low(h2[7 - r], h1[r]);
                }
            }
        }
        dftR<8, true>(a);
        dftR<8, true>(b);
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            sm2[(j1 * 8 + r) * LANES + lane] = a[r];
            sm2[(j2 * 8 + r) * LANES + lane] = b[r];
        }
    }
    __syncthreads();
}

// ylines: the lines run along the tensor's second dimension (y lines; tiles
// are numbered z-tile fastest, then the x index), else along the third
template <int N, bool INV>
__global__ void __launch_bounds__(LinePlan<N, INV, 0>::T, 1)
    k_lines32_tma(const __grid_constant__ CUtensorMap tmap, float *__restrict__ out, int P, long long line_stride,
                  long long batch_stride, int ztiles, long long ntiles, int ylines, const float2 *__restrict__ tw)
{
    constexpr int W = 0;
    constexpr int T = LinePlan<N, INV, W>::T;
    constexpr int BOX = N < 256 ? N : 256;
    constexpr uint32_t TILE_BYTES = N * 128;
    extern __shared__ __align__(128) unsigned char smraw[];
    __shared__ __align__(8) unsigned long long mbar[2];
    __shared__ int stop;
    const uint32_t bar0 = smem_addr(&mbar[0]), bar1 = smem_addr(&mbar[1]);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        stop = 0;
    }
    __syncthreads();
    // thread 0: copy tile `tile` into buffer b
    auto issue = [&](long long tile, int b) {
        const int zt = (int)(tile % ztiles);
        const int batch = (int)(tile / ztiles);
        const uint32_t bar = b ? bar1 : bar0;
        const uint32_t dst = smem_addr(smraw + (size_t)b * TILE_BYTES);
        // the buffer was last read through the generic proxy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(TILE_BYTES) : "memory");
#pragma unroll
        for (int r0 = 0; r0 < N; r0 += BOX) {
            const int c0 = zt * 2 * LANES, c1 = ylines ? r0 : batch, c2 = ylines ? batch : r0;
            asm volatile(
                "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
                    dst + (uint32_t)r0 * 128u),
                "l"(&tmap), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
                : "memory");
        }
    };
    long long tile = blockIdx.x;
    if (threadIdx.x == 0 && tile < ntiles) issue(tile, 0);
    uint32_t ph0 = 0, ph1 = 0;
    const int p = threadIdx.x & (PAIRS - 1);
    const float sc = rsqrtf((float)N);
    constexpr int H = N / 2;
    for (int b = 0; tile < ntiles; tile += gridDim.x, b ^= 1) {
        const long long next = tile + gridDim.x;
        // buffer b ^ 1 was released by the barrier that ended the last tile
        if (threadIdx.x == 0 && next < ntiles) issue(next, b ^ 1);
        if (!tma_wait(b ? bar1 : bar0, b ? ph1 : ph0)) {
            atomicOr(&g_lines_err, 1u);
            stop = 1;
        }
        if (b) ph1 ^= 1u;
        else ph0 ^= 1u;
        __syncthreads();
        if (stop) break;
        float4 *sm = reinterpret_cast<float4 *>(smraw + (size_t)b * TILE_BYTES);
        const int zt = (int)(tile % ztiles);
        const long long batch = tile / ztiles;
        const int z0 = zt * 2 * LANES;
        const bool valid = z0 + 4 * p < P;
        const long long base = batch * batch_stride + z0;
        const long long gs = line_stride >> 2;
        if (!INV) {
            pass<N, 8, 1, false, W, false, false>(sm, nullptr, nullptr, gs, valid, 1.0f, tw);
            later_passes<N, false, W, false>(sm, nullptr, gs, valid, 1.0f, tw);
            float4 *o = reinterpret_cast<float4 *>(out + base);
            for (int e = threadIdx.x; e < (H + 1) * PAIRS; e += T) {
                const int k = e / PAIRS, q = e & (PAIRS - 1);
                if (z0 + 4 * q >= P) continue;
                const float4 ck = sm[k * PAIRS + q];
                const float4 cn = sm[((N - k) & (N - 1)) * PAIRS + q];
                const float4 re = make_float4(0.5f * (ck.x + cn.x) * sc, 0.5f * (ck.y + cn.y) * sc,
                                              0.5f * (ck.z + cn.z) * sc, 0.5f * (ck.w + cn.w) * sc);
                o[k * gs + q] = re;
                if (k > 0 && k < H)
                    o[(N - k) * gs + q] = make_float4(0.5f * (ck.y - cn.y) * sc, -0.5f * (ck.x - cn.x) * sc,
                                                      0.5f * (ck.w - cn.w) * sc, -0.5f * (ck.z - cn.z) * sc);
            }
        } else {
            herm_first_pass_smem<N, W>(reinterpret_cast<float2 *>(sm));
            float4 *gout = reinterpret_cast<float4 *>(out + base) + p;
            later_passes<N, true, W, true>(sm, gout, gs, valid, sc, tw);
        }
        __syncthreads();
    }
    // a copy issued for a tile this block no longer takes (after a stop):
    // wait for it (bounded) before the block's shared memory is released
    if (stop && threadIdx.x == 0) {
        const long long next = tile + gridDim.x;
        if (next < ntiles) tma_wait(bar0, ph0), tma_wait(bar1, ph1);
    }
}

using EncodeTiled = PFN_cuTensorMapEncodeTiled_v12000;

EncodeTiled tensor_encoder()
{
    static EncodeTiled fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(f);
        cudaGetLastError();
    }
    return fn;
}

// false: no tensor map for this field (the caller takes the plain kernel)
template <int N, bool INV>
bool launch32tma(cudaStream_t st, const float *in, float *out, int P, int zv, long long ls, long long nbatch,
                 long long bs, const float2 *tw)
{
    EncodeTiled enc = tensor_encoder();
    if (!enc) return false;
    // y lines: line stride P, batches over x; x lines: line stride ny P,
    // batches over y
    const bool ylines = ls == P;
    const long long ny = ylines ? N : nbatch, nx = ylines ? nbatch : N;
    cuuint64_t dims[3] = {(cuuint64_t)zv, (cuuint64_t)ny, (cuuint64_t)nx};
    cuuint64_t strides[2] = {(cuuint64_t)P * 4, (cuuint64_t)P * 4 * (cuuint64_t)ny};
    constexpr int BOX = N < 256 ? N : 256;
    cuuint32_t box[3] = {32, ylines ? (cuuint32_t)BOX : 1u, ylines ? 1u : (cuuint32_t)BOX};
    cuuint32_t es[3] = {1, 1, 1};
    CUtensorMap map;
    if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(in), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    static int blocks = 0;  // resident blocks (the same on every GB300)
    const size_t sm = 2 * (size_t)N * 128;
    if (!blocks) {
        int dev = 0, sms = 1, per = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_lines32_tma<N, INV>, LinePlan<N, INV, 0>::T, sm);
        blocks = sms * (per > 0 ? per : 1);
    }
    const int ztiles = (P + 2 * LANES - 1) / (2 * LANES);
    const long long ntiles = (long long)ztiles * nbatch;
    const int grid = (int)(ntiles < blocks ? ntiles : blocks);
    k_lines32_tma<N, INV><<<grid, LinePlan<N, INV, 0>::T, sm, st>>>(map, out, P, ls, bs, ztiles, ntiles,
                                                                    ylines ? 1 : 0, tw);
    return true;
}

template <int N>
void launch32(cudaStream_t st, const float *in, float *out, int P, int zv, long long ls, long long nbatch,
              long long bs, bool inverse, const float2 *tw, int shape, int nf, long long fs_in, long long fs_out)
{
    // shape 2: the TMA-fed persistent kernel (N = 128, 256, 512), one launch
    // per field (its tensor map covers one field)
    if constexpr (N >= 128 && N <= 512) {
        if (shape == 2) {
            bool ok = true;
            for (int f = 0; f < nf && ok; ++f) {
                const float *fi = in + f * fs_in;
                float *fo = out + f * fs_out;
                ok = inverse ? launch32tma<N, true>(st, fi, fo, P, zv, ls, nbatch, bs, tw)
                             : launch32tma<N, false>(st, fi, fo, P, zv, ls, nbatch, bs, tw);
                if (!ok && f > 0) {  // the remaining fields with the plain kernel
                    in = fi;
                    out = fo;
                    nf -= f;
                }
            }
            if (ok) return;
            shape = -1;
        }
    }
    if (N == 512) {
        const int w = shape < 0 ? (inverse ? 1 : 0) : shape;
        if (inverse) {
            if (w) launch32w<N, true, 1>(st, in, out, P, zv, ls, nbatch, bs, tw, nf, fs_in, fs_out);
            else launch32w<N, true, 0>(st, in, out, P, zv, ls, nbatch, bs, tw, nf, fs_in, fs_out);
        } else {
            if (w) launch32w<N, false, 1>(st, in, out, P, zv, ls, nbatch, bs, tw, nf, fs_in, fs_out);
            else launch32w<N, false, 0>(st, in, out, P, zv, ls, nbatch, bs, tw, nf, fs_in, fs_out);
        }
        return;
    }
    if (inverse) launch32w<N, true, 0>(st, in, out, P, zv, ls, nbatch, bs, tw, nf, fs_in, fs_out);
    else launch32w<N, false, 0>(st, in, out, P, zv, ls, nbatch, bs, tw, nf, fs_in, fs_out);
}

}  // namespace

bool lines32_supported(int n) { return n == 64 || n == 128 || n == 256 || n == 512 || n == 1024; }

void lines32_init()
{
    tensor_encoder();  // resolve the driver's tensor-map encoder outside any stream capture
    cudaFuncSetAttribute(k_lines32<1024, false, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 1024 * LANES * 8);
    cudaFuncSetAttribute(k_lines32<1024, true, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 1024 * LANES * 8);
    cudaFuncSetAttribute(k_lines32<512, false, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 512 * LANES * 8);
    cudaFuncSetAttribute(k_lines32<512, true, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 512 * LANES * 8);
    cudaFuncSetAttribute(k_lines32<512, false, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 512 * LANES * 8);
    cudaFuncSetAttribute(k_lines32<512, true, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 512 * LANES * 8);
    cudaFuncSetAttribute(k_lines32_prod<1024, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 1024 * LANES * 8);
    cudaFuncSetAttribute(k_lines32_prod<512, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 512 * LANES * 8);
    cudaFuncSetAttribute(k_lines32_tma<512, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * 512 * 128);
    cudaFuncSetAttribute(k_lines32_tma<512, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * 512 * 128);
    cudaFuncSetAttribute(k_lines32_tma<256, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * 256 * 128);
    cudaFuncSetAttribute(k_lines32_tma<256, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * 256 * 128);
    cudaFuncSetAttribute(k_lines32_tma<128, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * 128 * 128);
    cudaFuncSetAttribute(k_lines32_tma<128, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * 128 * 128);
}

// kernel shapes: 0 the default blocks, 1 the 256-thread blocks (N = 512),
// 2 the TMA-fed persistent kernel (N = 128, 256, 512)
bool lines32_has_shape(int n, int w)
{
    if (w == 0) return lines32_supported(n);
    if (w == 1) return n == 512;
    return w == 2 && (n == 128 || n == 256 || n == 512);
}

int lines32_shapes(int n)
{
    int c = 0;
    for (int w = 0; w < 3; ++w) c += lines32_has_shape(n, w) ? 1 : 0;
    return c;
}

int lines32_error()
{
    unsigned int e = 0;
    if (cudaMemcpyFromSymbol(&e, g_lines_err, sizeof(e)) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (e) {
        const unsigned int z = 0;
        cudaMemcpyToSymbol(g_lines_err, &z, sizeof(z));
    }
    return e ? 1 : 0;
}

void launch_lines32(cudaStream_t st, const float *in, float *out, int n, int P, int zv, long long line_stride,
                    long long nbatch, long long batch_stride, bool inverse, const float2 *tw, int shape, int nf,
                    long long fs_in, long long fs_out)
{
    switch (n) {
    case 64: launch32<64>(st, in, out, P, zv, line_stride, nbatch, batch_stride, inverse, tw, shape, nf, fs_in, fs_out); break;
    case 128: launch32<128>(st, in, out, P, zv, line_stride, nbatch, batch_stride, inverse, tw, shape, nf, fs_in, fs_out); break;
    case 256: launch32<256>(st, in, out, P, zv, line_stride, nbatch, batch_stride, inverse, tw, shape, nf, fs_in, fs_out); break;
    case 512: launch32<512>(st, in, out, P, zv, line_stride, nbatch, batch_stride, inverse, tw, shape, nf, fs_in, fs_out); break;
    default: launch32<1024>(st, in, out, P, zv, line_stride, nbatch, batch_stride, inverse, tw, shape, nf, fs_in, fs_out); break;
    }
}

bool lines32_prod_supported(int ny) { return ny == 64 || ny == 128 || ny == 256 || ny == 512 || ny == 1024; }

void lines32_prod_y(cudaStream_t st, const float *vel, const float *vor, float *out, const Dims &d, double dzi,
                    const float2 *twy, Probe *pr)
{
    ProdSrc ps{vel, vor, d.nfield, (float)dzi, (float)(0.5 * dzi), d.nz};
    if (pr) pr->begin(PROBE_PRODUCTS, st);
    switch (d.ny) {
    case 64: launch_prod<64, 0>(st, ps, out, d.P, d.nx, d.ny, twy); break;
    case 128: launch_prod<128, 0>(st, ps, out, d.P, d.nx, d.ny, twy); break;
    case 256: launch_prod<256, 0>(st, ps, out, d.P, d.nx, d.ny, twy); break;
    case 512: launch_prod<512, 0>(st, ps, out, d.P, d.nx, d.ny, twy); break;
    default: launch_prod<1024, 0>(st, ps, out, d.P, d.nx, d.ny, twy); break;
    }
    // algorithmic bytes: six fields read, five written
    if (pr) pr->end(PROBE_PRODUCTS, st, 11.0 * (double)d.ncol * (double)(d.nz + 1) * sizeof(float));
}

}  // namespace ps3d
