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
// shuffles.  Both shared-memory exchanges use XOR-swizzled layouts that keep
// every access free of bank conflicts.  The post-processing produces output
// levels 2k and 2k+1 in the same lane, so results leave as coalesced float2
// stores straight from registers.  Inputs stored as FP64 (the prognostic
// state) are narrowed with integer arithmetic, keeping GB300's FP64 pipe out
// of the kernel.
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

template <int M> constexpr int lg2() { return M <= 1 ? 0 : 1 + lg2<M / 2>(); }

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
// em = exp(-kl zm) = ep at the mirrored level; phip(iz) = phim(nz - iz).
// Both exponents are a times an exact level count (iz or nz - iz), so the
// exponential near either boundary carries one rounding of its argument.
// The (0,0) column uses the linear functions (nz - iz)/nz and iz/nz.
struct Harm {
    float a, ef, div, g, inv_n;
    bool mean;
    __device__ static Harm make(float kl, float dz, float Lz, int nz, bool mean)
    {
        const float l2e = 1.4426950408889634f;
        Harm h;
        h.a = -kl * dz * l2e;
        h.ef = ex2(-kl * Lz * l2e);
        h.div = 1.0f / (1.0f - h.ef * h.ef);
        h.g = ex2(h.a);  // ep(iz + 1) = g ep(iz)
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
            const float ep = ex2(a * (float)iz), em = ex2(a * (float)(nz - iz));
            pm = div * (ep - ef * em);
            pp = div * (em - ef * ep);
        }
    }
    // levels z0 and z0 + 1 from two exponentials
    __device__ void at2(int z0, int nz, float &pm0, float &pp0, float &pm1, float &pp1) const
    {
        if (mean) {
            pp0 = (float)z0 * inv_n;
            pm0 = (float)(nz - z0) * inv_n;
            pp1 = (float)(z0 + 1) * inv_n;
            pm1 = (float)(nz - z0 - 1) * inv_n;
        } else {
            const float ep0 = ex2(a * (float)z0), em1 = ex2(a * (float)(nz - z0 - 1));
            const float ep1 = ep0 * g, em0 = em1 * g;
            pm0 = div * (ep0 - ef * em0);
            pp0 = div * (em0 - ef * ep0);
            pm1 = div * (ep1 - ef * em1);
            pp1 = div * (em1 - ef * ep1);
        }
    }
};

// d exp(-2 pi i j / 32) for a j known at compile time (the loops that call
// it are unrolled): the factors 1, -i, -1, i become moves and sign flips,
// and the eighth turns two adds and two multiplies.  cos(2 pi q / 32) for
// q = 0..8 as decimal literals.
__device__ __forceinline__ float2 tw32(float2 d, int j)
{
    constexpr float C[9] = {1.0f,
                            0.98078528040323044913f,
                            0.92387953251128675613f,
                            0.83146961230254523708f,
                            0.70710678118654752440f,
                            0.55557023301960222474f,
                            0.38268343236508977173f,
                            0.19509032201612826785f,
                            0.0f};
    j &= 31;
    if (j == 0) return d;
    if (j == 8) return make_float2(d.y, -d.x);
    if (j == 16) return make_float2(-d.x, -d.y);
    if (j == 24) return make_float2(-d.y, d.x);
    if ((j & 7) == 4) {
        const float r = C[4];
        // (1 - i) / sqrt 2 rotated by the quadrant of j
        const float2 q = (j == 4) ? make_float2(d.x + d.y, d.y - d.x)
                       : (j == 12) ? make_float2(d.y - d.x, -d.x - d.y)
                       : (j == 20) ? make_float2(-d.x - d.y, d.x - d.y)
                                   : make_float2(d.x - d.y, d.x + d.y);
        return make_float2(q.x * r, q.y * r);
    }
    // w = cos t - i sin t, t = 2 pi j / 32; cos and sin from the octant
    const int o = j & 7, qd = j >> 3;
    const float c0 = C[o], s0 = C[8 - o];  // cos, sin of the in-quadrant angle
    const float c = (qd == 0) ? c0 : (qd == 1) ? -s0 : (qd == 2) ? -c0 : s0;
    const float s = (qd == 0) ? s0 : (qd == 1) ? c0 : (qd == 2) ? -s0 : -c0;
    return make_float2(d.x * c + d.y * s, d.y * c - d.x * s);
}

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
                v[s0 + i + h] = tw32(make_float2(a.x - b.x, a.y - b.y), i * (16 / h));
            }
        }
    }
}

// Swizzles of the warp buffer (float2 slots; a half-warp of 8-byte accesses
// is conflict free when its slots differ modulo 16).
// Transpose slot of (lane l, column b < M): l M + (b ^ tsw(l)).  Writes (fixed
// b, 16 consecutive l) and reads (lanes (b, h) of rows h + S t) both land on
// 16 distinct slots modulo 16.
template <int M> __device__ __forceinline__ int tsw(int l)
{
    if constexpr (M == 32) {
        return l & 31;
    } else {
        constexpr int B = lg2<M>();
        const int x = (l >> (4 - B)) & (M - 1);
        return (x >> 1) | ((x & 1) << (B - 1));
    }
}
// natural-order spectrum slot of X[x]: bit-field XOR with the high bits,
// a bijection (the XOR source lies above its target)
template <int M> __device__ __forceinline__ int nsw(int x)
{
    constexpr int B = lg2<M>(), S = 32 / M;
    if constexpr (S == 1) return x;
    else return x ^ (((x >> (2 * B)) & (S - 1)) << (B - 1));
}

// n = 32 M point forward FFT of the warp's sequence; on entry lane l holds
// v[m] = c[l + 32 m]; on exit X[k] (natural order) is in xs[nsw(k)].
template <int M>
__device__ __forceinline__ void warp_fft(float2 *v, float2 *xs, const float2 *__restrict__ twn, int lane)
{
    constexpr int S = 32 / M;
    constexpr int n = 32 * M;
    dif<M>(v);  // register r: Z_l[b], b = brev(r)
#pragma unroll
    for (int r = 1; r < M; ++r) v[r] = fm(v[r], __ldg(&twn[(lane * brev<M>(r)) & (n - 1)]));
    // transpose: lane (b, h) = (lane / S, lane % S) gathers Z[h + S t][b]
    const int swl = tsw<M>(lane);
#pragma unroll
    for (int r = 0; r < M; ++r) xs[lane * M + (brev<M>(r) ^ swl)] = v[r];
    __syncwarp();
    const int b = lane / S, h = lane % S;
#pragma unroll
    for (int t = 0; t < M; ++t) {
        const int lp = h + S * t;
        v[t] = xs[lp * M + (b ^ tsw<M>(lp))];
    }
    __syncwarp();
    dif<M>(v);  // register r: F_h[a'], a' = brev(r)
    if (S > 1) {
#pragma unroll
        for (int r = 1; r < M; ++r) v[r] = fm(v[r], c_w32z[(h * brev<M>(r)) & 31]);
        // S-point DIF across the S lanes of the group
#pragma unroll
        // the lower lane of a butterfly keeps v + u, the upper one takes
        // (u - v) w: one fused multiply-add with a sign, then a multiply by
        // w or by exactly 1
        for (int hs = S / 2; hs >= 1; hs >>= 1) {
            const bool upper = (h & hs) != 0;
            const float sg = upper ? -1.f : 1.f;
            const float2 w = upper ? c_w32z[((h & (hs - 1)) * (16 / hs)) & 31] : make_float2(1.f, 0.f);
#pragma unroll
            for (int r = 0; r < M; ++r) {
                float2 u;
                u.x = __shfl_xor_sync(0xffffffffu, v[r].x, hs);
                u.y = __shfl_xor_sync(0xffffffffu, v[r].y, hs);
                v[r] = fm(make_float2(fmaf(sg, v[r].x, u.x), fmaf(sg, v[r].y, u.y)), w);
            }
        }
    }
    const int e = brev<S>(h);
#pragma unroll
    for (int r = 0; r < M; ++r) xs[nsw<M>(b + M * brev<M>(r) + M * M * e)] = v[r];
    __syncwarp();
}

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

__device__ __forceinline__ float warp_sum(float x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// Per-column scalars of a column pair spread over the warp (lane i holds
// scalar i): they stay out of the registers while the warp FFT runs and are
// fetched with one shuffle each where needed.
__device__ __forceinline__ float lane_get(float par, int i) { return __shfl_sync(0xffffffffu, par, i); }

__device__ __forceinline__ void st2(float *col, int k, float e, float o)
{
    reinterpret_cast<float2 *>(col)[k] = make_float2(e, o);
}

// Post-processing of the packed spectra in xs (stafft.f90:458-482 cosine,
// :531-549 sine).  At spectral index k both columns get a direct value (level
// 2k) and a running sum (level 2k+1) over the other half of the spectrum;
// split() gives the direct values and the running-sum addends, the running
// sums are warp scans with a carry.  For every k, fix(k, eA, oA, eB, oB) may
// change the two levels of both columns (mode-specific terms), then they are
// stored.  With n >= 128 a lane takes two consecutive k (one scan for both,
// one 16-byte store per column); sine: the value at level 0 is meaningless,
// cosine: x1 is the direct sum that gives level 1's constant.
template <bool COS>
__device__ __forceinline__ void split(int k, float2 ck, float2 cn, float r2s, float &dA, float &aA, float &dB,
                                      float &aB)
{
    const float ReA = 0.5f * (ck.x + cn.x), ImA = 0.5f * (ck.y - cn.y);
    const float ReB = 0.5f * (ck.y + cn.y), ImB = -0.5f * (ck.x - cn.x);
    if (COS) {
        dA = r2s * ReA;
        dB = r2s * ReB;
        aA = (k == 0) ? 0.f : ImA;
        aB = (k == 0) ? 0.f : ImB;
    } else {
        dA = -r2s * ImA;
        dB = -r2s * ImB;
        aA = (k == 0) ? 0.5f * ReA : ReA;
        aB = (k == 0) ? 0.5f * ReB : ReB;
    }
}

template <bool COS> __device__ __forceinline__ float odd_level(float run, float x1, float r2s)
{
    return COS ? x1 - r2s * run : r2s * run;
}

template <int M, bool COS, typename F>
__device__ __forceinline__ void post(const float2 *xs, int lane, float r2s, float x1A, float x1B, float *colA,
                                     float *colB, F &&fix)
{
    constexpr int n = 32 * M, KPL = n / 64;
    if constexpr (KPL == 1) {
        const int k = lane;
        float dA, aA, dB, aB;
        split<COS>(k, xs[nsw<M>(k)], xs[nsw<M>((n - k) & (n - 1))], r2s, dA, aA, dB, aB);
        float eA = dA, oA = odd_level<COS>(warp_incl_scan(aA, lane), x1A, r2s);
        float eB = dB, oB = odd_level<COS>(warp_incl_scan(aB, lane), x1B, r2s);
        fix(k, eA, oA, eB, oB);
        st2(colA, k, eA, oA);
        st2(colB, k, eB, oB);
    } else {
        float carryA = 0.f, carryB = 0.f;
#pragma unroll
        for (int i = 0; i < KPL / 2; ++i) {
            const int k0 = 2 * lane + 64 * i;
            // X[k0], X[k0 + 1] share one aligned 16-byte slot pair
            const float4 c = *reinterpret_cast<const float4 *>(xs + nsw<M>(k0));
            const float2 m0 = xs[nsw<M>((n - k0) & (n - 1))], m1 = xs[nsw<M>(n - k0 - 1)];
            float dA0, aA0, dB0, aB0, dA1, aA1, dB1, aB1;
            split<COS>(k0, make_float2(c.x, c.y), m0, r2s, dA0, aA0, dB0, aB0);
            split<COS>(k0 + 1, make_float2(c.z, c.w), m1, r2s, dA1, aA1, dB1, aB1);
            const float ra1 = warp_incl_scan(aA0 + aA1, lane) + carryA;
            const float rb1 = warp_incl_scan(aB0 + aB1, lane) + carryB;
            carryA = __shfl_sync(0xffffffffu, ra1, 31);
            carryB = __shfl_sync(0xffffffffu, rb1, 31);
            float eA0 = dA0, oA0 = odd_level<COS>(ra1 - aA1, x1A, r2s);
            float eB0 = dB0, oB0 = odd_level<COS>(rb1 - aB1, x1B, r2s);
            float eA1 = dA1, oA1 = odd_level<COS>(ra1, x1A, r2s);
            float eB1 = dB1, oB1 = odd_level<COS>(rb1, x1B, r2s);
            fix(k0, eA0, oA0, eB0, oB0);
            fix(k0 + 1, eA1, oA1, eB1, oB1);
            reinterpret_cast<float4 *>(colA)[lane + 32 * i] = make_float4(eA0, oA0, eA1, oA1);
            reinterpret_cast<float4 *>(colB)[lane + 32 * i] = make_float4(eB0, oB0, eB1, oB1);
        }
    }
}

// dst pre-processing of x(j), x(n-j) of both columns
__device__ __forceinline__ float2 pre_sine(float xa, float ya, float xb, float yb, float sj)
{
    return make_float2(0.5f * (xa - ya) + sj * (xa + ya), 0.5f * (xb - yb) + sj * (xb + yb));
}
// dct pre-processing
__device__ __forceinline__ float2 pre_cosine(float xa, float ya, float xb, float yb, float sj)
{
    return make_float2(0.5f * (xa + ya) - sj * (xa - ya), 0.5f * (xb + yb) - sj * (xb - yb));
}

// ---- staging of a column pair in shared memory
// The two columns of a pair are adjacent (column B = column A + 1), so the
// pair is one contiguous run of 2P floats.  One lane of the warp copies the
// warp's next pair with a bulk copy (cp.async.bulk, completion counted on the
// warp's mbarrier) as soon as the current pair has been read: the copy runs
// while the warp does the FFT and the post-processing, and every read of the
// input comes from shared memory.  Waits are bounded; a wait that runs out
// sets g_colz_err and the warp stops.
__device__ unsigned int g_colz_err;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void stage_init(uint32_t bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// one lane: copy `bytes` (a multiple of 16, both addresses 16-byte aligned)
// from global src to shared dst; the warp's earlier reads of dst are ordered
// before the copy by the __syncwarp the caller issues and the proxy fence
__device__ __forceinline__ void stage_copy(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ bool stage_wait(uint32_t bar, uint32_t parity)
{
    for (int i = 0; i < (1 << 21); ++i) {
        uint32_t ok;
        asm volatile("{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(ok)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (ok) return true;
        if (i > 32) __nanosleep(64);
    }
    return false;
}

// Per-warp stager: the warp's pair buffer zin (2P floats) and its mbarrier.
struct Stager {
    uint32_t bar, dst, bytes, phase;
    bool stopped;
    __device__ void start(int lane, const float *in, long long first, long long npairs, int P)
    {
        phase = 0;
        stopped = false;
        if (lane == 0) {
            stage_init(bar);
            if (first < npairs) stage_copy(dst, in + 2 * first * (long long)P, bytes, bar);
        }
        __syncwarp();
    }
    // wait for the current pair; false (warp-uniform) when the wait ran out
    __device__ bool wait(int lane)
    {
        const bool ok = __all_sync(0xffffffffu, stage_wait(bar, phase));
        phase ^= 1u;
        if (!ok) {
            if (lane == 0) atomicOr(&g_colz_err, 1u);
            stopped = true;
        }
        return ok;
    }
    // the current pair has been read: start the copy of the next one
    __device__ void next(int lane, const float *in, long long pr_next, long long npairs, int P)
    {
        __syncwarp();
        if (lane == 0 && pr_next < npairs) stage_copy(dst, in + 2 * pr_next * (long long)P, bytes, bar);
    }
    // the same with the source address of the pair given (nullptr: none)
    __device__ void start_at(int lane, const float *src)
    {
        phase = 0;
        stopped = false;
        if (lane == 0) {
            stage_init(bar);
            if (src) stage_copy(dst, src, bytes, bar);
        }
        __syncwarp();
    }
    __device__ void next_at(int lane, const float *src)
    {
        __syncwarp();
        if (lane == 0 && src) stage_copy(dst, src, bytes, bar);
    }
    // after a stop the copy that ran out may still land: wait once more
    // (bounded) before the block's shared memory is released
    __device__ void finish(int lane)
    {
        if (stopped && lane == 0) stage_wait(bar, phase ^ 1u);
    }
};

// float inputs up to nz = 512 are staged (at nz = 1024 the buffer would
// halve the resident warps)
template <int M, typename TIN> constexpr bool staged() { return std::is_same<TIN, float>::value && M <= 16; }

// shared memory of a block of 8 warps: 8 mbarriers, then per warp the FFT
// buffer (n float2) and, when staged, the pair buffer (2P floats)
constexpr size_t COLZ_BAR_BYTES = 64;
template <int M> constexpr size_t xs_bytes() { return 32 * M * sizeof(float2); }
__host__ __device__ inline size_t warp_bytes(size_t xsb, bool stage, int P) { return xsb + (stage ? 2 * (size_t)P * sizeof(float) : 0); }

}  // namespace

// resident 256-thread blocks per SM: three up to nz = 512, two at nz = 1024
template <int M> constexpr int col_blocks_per_sm() { return M <= 16 ? 3 : 2; }

// MODE: COL_DST, COL_DCT, COL_DECOMP, COL_COMBINE (see kernels.h).  Safe in
// place: a pair's inputs are all read before its outputs are written, and a
// staged copy only reads the warp's own next pair.
template <int MODE, int M, typename TIN>
__global__ void __launch_bounds__(256, col_blocks_per_sm<M>())
    k_colz(const TIN *__restrict__ in, float *__restrict__ out, int P, long long npairs,
           const double *__restrict__ k2l2, float dz, float Lz, const float2 *__restrict__ twn,
           const float *__restrict__ sinz, const float *__restrict__ cosz)
{
    constexpr int n = 32 * M;  // = nz
    constexpr bool ST = staged<M, TIN>();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    extern __shared__ __align__(16) unsigned char smz[];
    unsigned char *wbase = smz + COLZ_BAR_BYTES + (size_t)wib * warp_bytes(xs_bytes<M>(), ST, P);
    float2 *xs = reinterpret_cast<float2 *>(wbase);
    const float *zin = reinterpret_cast<const float *>(wbase + xs_bytes<M>());
    const float r2s = 1.41421356237309505f * rsqrtf((float)n);
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    const long long first = (long long)blockIdx.x * (blockDim.x >> 5) + wib;
    Stager sg;
    if (ST) {
        sg.bar = smem_addr(smz + 8 * wib);
        sg.dst = smem_addr(zin);
        sg.bytes = 8u * (uint32_t)P;
        sg.start(lane, reinterpret_cast<const float *>(in), first, npairs, P);
    }
    for (long long pr = first; pr < npairs; pr += warps) {
        if (ST && !sg.wait(lane)) break;
        const long long cA = 2 * pr, cB = cA + 1;
        const long long oA = cA * P, oB = cB * P;
        // column values at level z: from the pair buffer or from global memory
        auto xA = [&](int z) { return ST ? zin[z] : ld(in, oA + z); };
        auto xB = [&](int z) { return ST ? zin[P + z] : ld(in, oB + z); };
        // lanes 0..2 (column A) and 8..10 (column B): f(0), f(nz), kl
        float par = 0.f;
        if (lane < 16 && (lane & 7) < 3) {
            const int q = lane & 7;
            if (q == 2) par = sqrtf((float)k2l2[lane < 8 ? cA : cB]);
            else par = lane < 8 ? xA(q == 0 ? 0 : n) : xB(q == 0 ? 0 : n);
        }
        // ---- pre-processed sequence wk (both columns), lane l: j = l + 32 m
        float dsumA = 0.f, dsumB = 0.f;  // DCT direct sum for x(1)
        {
            float2 v[M];
            const float f0A = lane_get(par, 0), fnA = lane_get(par, 1), f0B = lane_get(par, 8),
                        fnB = lane_get(par, 9);
            Harm hA{}, hB{};
            if (MODE == COL_DECOMP) {
                hA = Harm::make(lane_get(par, 2), dz, Lz, n, cA == 0);
                hB = Harm::make(lane_get(par, 10), dz, Lz, n, cB == 0);
            }
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const int j = lane + 32 * m;
                float xa = 0.f, xb = 0.f, ya = 0.f, yb = 0.f;  // x(j), x(n-j)
                if (j > 0) {
                    xa = xA(j);
                    xb = xB(j);
                    ya = xA(n - j);
                    yb = xB(n - j);
                }
                if (MODE == COL_DECOMP && j > 0) {
                    float pm, pp;
                    hA.at(j, n, pm, pp);
                    xa -= f0A * pm + fnA * pp;
                    ya -= f0A * pp + fnA * pm;
                    hB.at(j, n, pm, pp);
                    xb -= f0B * pm + fnB * pp;
                    yb -= f0B * pp + fnB * pm;
                }
                const float sj = __ldg(&sinz[j]);
                if (MODE == COL_DCT) {
                    if (j == 0) {
                        v[m] = make_float2(0.5f * (f0A + fnA), 0.5f * (f0B + fnB));
                    } else {
                        const float cj = __ldg(&cosz[j]);
                        dsumA += xa * cj;
                        dsumB += xb * cj;
                        v[m] = pre_cosine(xa, ya, xb, yb, sj);
                    }
                } else {
                    v[m] = (j == 0) ? make_float2(0.f, 0.f) : pre_sine(xa, ya, xb, yb, sj);
                }
            }
            if (ST) sg.next(lane, reinterpret_cast<const float *>(in), pr + warps, npairs, P);
            warp_fft<M>(v, xs, twn, lane);
        }
        // ---- split the packed spectra, store levels 2k, 2k+1
        float *colA = out + oA, *colB = out + oB;
        const float f0A = lane_get(par, 0), fnA = lane_get(par, 1), f0B = lane_get(par, 8),
                    fnB = lane_get(par, 9);
        if (MODE == COL_DCT) {
            const float x1A = r2s * (0.5f * f0A + warp_sum(dsumA) - 0.5f * fnA);
            const float x1B = r2s * (0.5f * f0B + warp_sum(dsumB) - 0.5f * fnB);
            post<M, true>(xs, lane, r2s, x1A, x1B, colA, colB, [](int, float &, float &, float &, float &) {});
            if (lane == 0) {
                const float2 cm = xs[nsw<M>(n / 2)];
                colA[n] = r2s * cm.x;
                colB[n] = r2s * cm.y;
            }
        } else if (MODE == COL_COMBINE) {
            const Harm hA = Harm::make(lane_get(par, 2), dz, Lz, n, cA == 0);
            const Harm hB = Harm::make(lane_get(par, 10), dz, Lz, n, cB == 0);
            post<M, false>(xs, lane, r2s, 0.f, 0.f, colA, colB,
                           [&](int k, float &eA, float &oA_, float &eB, float &oB_) {
                               float pm0, pp0, pm1, pp1;
                               hA.at2(2 * k, n, pm0, pp0, pm1, pp1);
                               eA = (k == 0) ? f0A : eA + f0A * pm0 + fnA * pp0;
                               oA_ += f0A * pm1 + fnA * pp1;
                               hB.at2(2 * k, n, pm0, pp0, pm1, pp1);
                               eB = (k == 0) ? f0B : eB + f0B * pm0 + fnB * pp0;
                               oB_ += f0B * pm1 + fnB * pp1;
                           });
            if (lane == 0) {
                colA[n] = fnA;
                colB[n] = fnB;
            }
        } else {
            // DST keeps the input's level 0 and zeroes level nz; DECOMP
            // keeps both boundary values
            post<M, false>(xs, lane, r2s, 0.f, 0.f, colA, colB, [&](int k, float &eA, float &, float &eB, float &) {
                if (k == 0) {
                    eA = f0A;
                    eB = f0B;
                }
            });
            if (lane == 0) {
                colA[n] = (MODE == COL_DST) ? 0.f : fnA;
                colB[n] = (MODE == COL_DST) ? 0.f : fnB;
            }
        }
        __syncwarp();
    }
    if (ST) sg.finish(lane);
}

namespace {
// Boundary-driven part of the vertical-velocity inversion for one column
// (inversion.f90:94-139 with the theta functions of inversion_utils.f90:
// 484-542).  With Lp = kl zp, Lm = kl zm, ep = exp(-Lp), em = exp(-Lm),
//   ds(0) thetam + ds(nz) thetap   (w) and
//   ds(0) dthetam + ds(nz) dthetap (dw/dz)
// are both em (c_mm Lm + c_mp Lp + c_mc) + ep (c_pm Lm + c_pp Lp + c_pc):
// expanding thetam, thetap (and their z derivatives) in phim, phip leaves
// terms linear in Lm and Lp times the two exponentials.  Lp and Lm are taken
// as kl dz times the exact level counts iz and nz - iz.
struct ThetaCol {
    float a, g, kdz;
    float c_mm, c_mp, c_mc, c_pm, c_pp, c_pc;
    bool zero;  // (0,0) column: no boundary-driven part
    __device__ static ThetaCol make(bool dwdz, float kl, float k2i, float d0, float dn, float dz, float Lz,
                                    bool zero)
    {
        const float l2e = 1.4426950408889634f;
        ThetaCol t;
        t.zero = zero;
        t.a = -kl * dz * l2e;
        t.g = ex2(t.a);
        t.kdz = kl * dz;
        const float ef = ex2(-kl * Lz * l2e);
        const float div = 1.0f / (1.0f - ef * ef);
        const float Q = div * (1.0f + ef * ef), R = div * 2.0f * ef;
        const float A = d0 * R - dn * Q, B = d0 * Q - dn * R;
        if (!dwdz) {
            const float s = 0.5f * k2i * div;
            t.c_mm = s * A;
            t.c_mp = s * ef * B;
            t.c_mc = 0.f;
            t.c_pm = -s * ef * A;
            t.c_pp = -s * B;
            t.c_pc = 0.f;
        } else {
            const float s = 0.5f * k2i * kl * div;
            t.c_mm = s * A;
            t.c_mp = s * ef * B;
            t.c_mc = s * (dn - d0 * ef);
            t.c_pm = s * ef * A;
            t.c_pp = s * B;
            t.c_pc = s * (dn * ef - d0);
        }
        return t;
    }
    // values at levels z0 and z0 + 1
    __device__ void at2(int z0, int n, float &v0, float &v1) const
    {
        if (zero) {
            v0 = v1 = 0.f;
            return;
        }
        const float ep0 = ex2(a * (float)z0), em1 = ex2(a * (float)(n - z0 - 1));
        const float ep1 = ep0 * g, em0 = em1 * g;
        const float Lp0 = kdz * (float)z0, Lp1 = kdz * (float)(z0 + 1);
        const float Lm0 = kdz * (float)(n - z0), Lm1 = kdz * (float)(n - z0 - 1);
        v0 = em0 * (c_mm * Lm0 + c_mp * Lp0 + c_mc) + ep0 * (c_pm * Lm0 + c_pp * Lp0 + c_pc);
        v1 = em1 * (c_mm * Lm1 + c_mp * Lp1 + c_mc) + ep1 * (c_pm * Lm1 + c_pp * Lp1 + c_pc);
    }
};
}  // namespace

// ------------------------------------------------------------------------
// Vertical velocity of vor2vel (inversion.f90:94-139):
//   bs = ds(0) thetam + ds(nz) thetap,  es = ds(0) dthetam + ds(nz) dthetap,
//   dsg = green ds (interior), as = rkz dsg,
//   w = [0, dst(dsg) + bs, 0],  dw/dz = es + dct(as),
// with green(kz) = -1/(k^2 + l^2 + rkz^2) and the boundary-driven parts
// evaluated in registers.  PART 1 computes w, PART 2 dw/dz, PART 3 both from
// one read of ds.  Two single-part launches, each reading ds, take less time
// than one two-part launch (51.4 against 52.0 ms per 512^3 step), and run
// faster at two blocks per SM with 128 registers than at three with 80 and
// spills (51.4 against 51.7 ms).
template <int PART> constexpr int w_blocks_per_sm() { return 2; }

//
// SRC: the kernel also forms ds itself (the w source of inversion.f90:86-92,
// ds = cy A(kx, -ky) - cx B(-kx, ky) with the state components A, B, the
// partner columns as in k_v2v_wsrc): the x-partner pair of B (two adjacent
// columns) comes by the staged copy, A's y partners are read with one batch
// of loads, and the pair buffer is overwritten with ds.  `ds` is then B.
// Staged lengths only (nz <= 512).
template <int M, int PART, bool SRC = false>
__global__ void __launch_bounds__(256, w_blocks_per_sm<PART>()) k_colz_w(const float *__restrict__ ds, float *__restrict__ w,
                                                   float *__restrict__ es, int P, long long npairs,
                                                   const double *__restrict__ k2l2, const double *__restrict__ k2l2i,
                                                   float dz, float Lz, const float2 *__restrict__ twn,
                                                   const float *__restrict__ sinz, const float *__restrict__ cosz,
                                                   const float *__restrict__ A = nullptr,
                                                   const double *__restrict__ cxv = nullptr,
                                                   const double *__restrict__ cyv = nullptr, int ny = 0)
{
    static_assert(!SRC || staged<M, float>(), "the fused w source needs the staged pair buffer");
    constexpr int n = 32 * M;
    constexpr bool ST = staged<M, float>();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    extern __shared__ __align__(16) unsigned char smz[];
    unsigned char *wbase = smz + COLZ_BAR_BYTES + (size_t)wib * warp_bytes(xs_bytes<M>(), ST, P);
    float2 *xs = reinterpret_cast<float2 *>(wbase);
    const float *zin = reinterpret_cast<const float *>(wbase + xs_bytes<M>());
    const float r2s = 1.41421356237309505f * rsqrtf((float)n);
    const float pk = 3.14159265358979324f / Lz;  // rkz(kz) = pk kz
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    const long long first = (long long)blockIdx.x * (blockDim.x >> 5) + wib;
    // source of the staged pair (SRC: B's x-partner pair)
    auto stage_src = [&](long long pr) -> const float * {
        if (pr >= npairs) return nullptr;
        if (!SRC) return ds + 2 * pr * (long long)P;
        const long long cA = 2 * pr, kx = cA / ny, ky = cA - kx * ny, nx = (2 * npairs) / ny;
        return ds + ((kx == 0 ? 0 : nx - kx) * ny + ky) * (long long)P;
    };
    Stager sg;
    if (ST) {
        sg.bar = smem_addr(smz + 8 * wib);
        sg.dst = smem_addr(zin);
        sg.bytes = 8u * (uint32_t)P;
        sg.start_at(lane, stage_src(first));
    }
    for (long long pr = first; pr < npairs; pr += warps) {
        if (ST && !sg.wait(lane)) break;
        const long long cA = 2 * pr, cB = cA + 1;
        const long long oA = cA * P, oB = cB * P;
        if (SRC) {
            // ds = cy A(y partner) - cx B(x partner), in place over the
            // staged B pair; every load of A issued before the first is used
            float *zw = const_cast<float *>(zin);
            const long long kx = cA / ny;
            const int kyA = (int)(cA - kx * ny), kyB = kyA + 1;
            const long long aA = (kx * ny + (kyA == 0 ? 0 : ny - kyA)) * (long long)P;
            const long long aB = (kx * ny + (ny - kyB)) * (long long)P;
            const float cx = (float)cxv[kx], cyA = (float)cyv[kyA], cyB = (float)cyv[kyB];
            float h[2][M];
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int m = 0; m < M; ++m) h[b][m] = A[(b ? aB : aA) + lane + 32 * m];
#pragma unroll
            for (int b = 0; b < 2; ++b) {
                float *zc = zw + b * P;
                const float cy = b ? cyB : cyA;
#pragma unroll
                for (int m = 0; m < M; ++m) zc[lane + 32 * m] = cy * h[b][m] - cx * zc[lane + 32 * m];
            }
            if (lane < 2) {
                float *zc = zw + lane * P;
                zc[n] = (lane ? cyB : cyA) * A[(lane ? aB : aA) + n] - cx * zc[n];
            }
            __syncwarp();
        }
        // opaque copies of the offsets keep the compiler from hoisting the
        // second transform's global loads above the first (register spills)
        long long qA = oA, qB = oB;
        asm volatile("" : "+l"(qA), "+l"(qB));
        auto dA = [&](int z) { return ST ? zin[z] : ds[oA + z]; };
        auto dB = [&](int z) { return ST ? zin[P + z] : ds[oB + z]; };
        auto dA2 = [&](int z) { return ST ? zin[z] : ds[qA + z]; };
        auto dB2 = [&](int z) { return ST ? zin[P + z] : ds[qB + z]; };
        // lanes 0..3 (column A) and 8..11 (column B): k^2+l^2, 1/(k^2+l^2),
        // ds(0), ds(nz)
        float par = 0.f;
        if (lane < 16 && (lane & 7) < 4) {
            const long long c = lane < 8 ? cA : cB;
            const int f = lane & 3;
            if (f == 0) par = (float)k2l2[c];
            else if (f == 1) par = (float)k2l2i[c];
            else par = lane < 8 ? dA(f == 2 ? 0 : n) : dB(f == 2 ? 0 : n);
        }
        // ---- dst of dsg = green ds
        if (PART & 1) {
            const float k2A = lane_get(par, 0), k2B = lane_get(par, 8);
            float2 v[M];
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const int j = lane + 32 * m;
                v[m] = make_float2(0.f, 0.f);
                if (j > 0) {
                    const float rj = pk * (float)j, rn = pk * (float)(n - j);
                    const float rj2 = rj * rj, rn2 = rn * rn;
                    const float xa = __fdividef(-dA(j), k2A + rj2), ya = __fdividef(-dA(n - j), k2A + rn2);
                    const float xb = __fdividef(-dB(j), k2B + rj2), yb = __fdividef(-dB(n - j), k2B + rn2);
                    v[m] = pre_sine(xa, ya, xb, yb, __ldg(&sinz[j]));
                }
            }
            if (ST && PART == 1) sg.next_at(lane, stage_src(pr + warps));
            warp_fft<M>(v, xs, twn, lane);
        }
        if (PART & 1) {
            const float klA = sqrtf(lane_get(par, 0)), klB = sqrtf(lane_get(par, 8));
            const ThetaCol tA =
                ThetaCol::make(false, klA, lane_get(par, 1), lane_get(par, 2), lane_get(par, 3), dz, Lz, cA == 0);
            const ThetaCol tB =
                ThetaCol::make(false, klB, lane_get(par, 9), lane_get(par, 10), lane_get(par, 11), dz, Lz, cB == 0);
            float *wA = w + oA, *wB = w + oB;
            post<M, false>(xs, lane, r2s, 0.f, 0.f, wA, wB, [&](int k, float &eA, float &oA_, float &eB, float &oB_) {
                float b0, b1;
                tA.at2(2 * k, n, b0, b1);
                eA = (k == 0) ? 0.f : eA + b0;
                oA_ += b1;
                tB.at2(2 * k, n, b0, b1);
                eB = (k == 0) ? 0.f : eB + b0;
                oB_ += b1;
            });
            if (lane == 0) {
                wA[n] = 0.f;
                wB[n] = 0.f;
            }
        }
        __syncwarp();
        // ---- dct of as = rkz green ds (as(0) = as(nz) = 0)
        float x1A = 0.f, x1B = 0.f;
        if (PART & 2) {
            const float k2A = lane_get(par, 0), k2B = lane_get(par, 8);
            float2 v[M];
            float sA = 0.f, sB = 0.f;
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const int j = lane + 32 * m;
                v[m] = make_float2(0.f, 0.f);
                if (j > 0) {
                    const float rj = pk * (float)j, rn = pk * (float)(n - j);
                    const float rj2 = rj * rj, rn2 = rn * rn;
                    const float xa = __fdividef(-rj * dA2(j), k2A + rj2);
                    const float ya = __fdividef(-rn * dA2(n - j), k2A + rn2);
                    const float xb = __fdividef(-rj * dB2(j), k2B + rj2);
                    const float yb = __fdividef(-rn * dB2(n - j), k2B + rn2);
                    const float cj = __ldg(&cosz[j]);
                    sA += xa * cj;
                    sB += xb * cj;
                    v[m] = pre_cosine(xa, ya, xb, yb, __ldg(&sinz[j]));
                }
            }
            if (ST) sg.next_at(lane, stage_src(pr + warps));
            x1A = r2s * warp_sum(sA);
            x1B = r2s * warp_sum(sB);
            warp_fft<M>(v, xs, twn, lane);
        }
        if (PART & 2) {
            const float klA = sqrtf(lane_get(par, 0)), klB = sqrtf(lane_get(par, 8));
            const ThetaCol tA =
                ThetaCol::make(true, klA, lane_get(par, 1), lane_get(par, 2), lane_get(par, 3), dz, Lz, cA == 0);
            const ThetaCol tB =
                ThetaCol::make(true, klB, lane_get(par, 9), lane_get(par, 10), lane_get(par, 11), dz, Lz, cB == 0);
            float *eA_ = es + oA, *eB_ = es + oB;
            post<M, true>(xs, lane, r2s, x1A, x1B, eA_, eB_, [&](int k, float &eA, float &oA_, float &eB, float &oB_) {
                float b0, b1;
                tA.at2(2 * k, n, b0, b1);
                eA += b0;
                oA_ += b1;
                tB.at2(2 * k, n, b0, b1);
                eB += b0;
                oB_ += b1;
            });
            if (lane == 0) {
                const float2 cm = xs[nsw<M>(n / 2)];
                float b0, b1;
                tA.at2(n - 1, n, b0, b1);
                eA_[n] = r2s * cm.x + b1;
                tB.at2(n - 1, n, b0, b1);
                eB_[n] = r2s * cm.y + b1;
            }
        }
        __syncwarp();
    }
    if (ST) sg.finish(lane);
}

// ------------------------------------------------------------------------
// The third tendency component's two decompositions in one kernel (mixed
// form): from the semi-spectral S3 of a column pair,
//   out = decompose(S3)                 (the mixed-spectral tendency), and
//   es  = decompose(central_diffz(S3))  (the z part of its solenoidal
//                                        projection, inversion.f90:41-47),
// one read of S3 into the warp's pair buffer, two warp FFTs, one write each.
// Safe in place (out == f): the pair is read whole before anything is
// written.  Up to nz = 512 the pair arrives by a staged bulk copy (prefetched
// one pair ahead); at nz = 1024 the warp loads it itself.
template <int M>
__global__ void __launch_bounds__(256, M <= 16 ? 3 : 2) k_colz_dec2(const float *__restrict__ f, float *out, float *__restrict__ es,
                                                      int P, long long npairs, const double *__restrict__ k2l2,
                                                      float dz, float Lz, const float2 *__restrict__ twn,
                                                      const float *__restrict__ sinz)
{
    constexpr int n = 32 * M;
    constexpr bool ST = staged<M, float>();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    extern __shared__ __align__(16) unsigned char smz[];
    unsigned char *wbase = smz + COLZ_BAR_BYTES + (size_t)wib * warp_bytes(xs_bytes<M>(), true, P);
    float2 *xs = reinterpret_cast<float2 *>(wbase);
    float *zA = reinterpret_cast<float *>(wbase + xs_bytes<M>());
    float *zB = zA + P;
    float *gA = reinterpret_cast<float *>(xs), *gB = gA + n;
    const float r2s = 1.41421356237309505f * rsqrtf((float)n);
    const float dzi = 1.0f / dz, hdzi = 0.5f / dz;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    const long long first = (long long)blockIdx.x * (blockDim.x >> 5) + wib;
    Stager sg;
    if (ST) {
        sg.bar = smem_addr(smz + 8 * wib);
        sg.dst = smem_addr(zA);
        sg.bytes = 8u * (uint32_t)P;
        sg.start(lane, f, first, npairs, P);
    }
    for (long long pr = first; pr < npairs; pr += warps) {
        const long long cA = 2 * pr, cB = cA + 1;
        const long long oA = cA * P, oB = cB * P;
        if (ST) {
            if (!sg.wait(lane)) break;
        } else {
            for (int iz = lane; iz <= n; iz += 32) {
                zA[iz] = f[oA + iz];
                zB[iz] = f[oB + iz];
            }
            __syncwarp();
        }
        // lanes 0 / 8: kl of columns A / B
        float par = 0.f;
        if (lane == 0 || lane == 8) par = sqrtf((float)k2l2[lane == 0 ? cA : cB]);
        const float f0A = zA[0], fnA = zA[n], f0B = zB[0], fnB = zB[n];
        // ---- decompose S3: subtract the harmonic part, dst
        {
            const Harm hA = Harm::make(lane_get(par, 0), dz, Lz, n, cA == 0);
            const Harm hB = Harm::make(lane_get(par, 8), dz, Lz, n, cB == 0);
            float2 v[M];
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const int j = lane + 32 * m;
                v[m] = make_float2(0.f, 0.f);
                if (j > 0) {
                    float xa = zA[j], ya = zA[n - j], xb = zB[j], yb = zB[n - j];
                    float pm, pp;
                    hA.at(j, n, pm, pp);
                    xa -= f0A * pm + fnA * pp;
                    ya -= f0A * pp + fnA * pm;
                    hB.at(j, n, pm, pp);
                    xb -= f0B * pm + fnB * pp;
                    yb -= f0B * pp + fnB * pm;
                    v[m] = pre_sine(xa, ya, xb, yb, __ldg(&sinz[j]));
                }
            }
            warp_fft<M>(v, xs, twn, lane);
        }
        {
            float *colA = out + oA, *colB = out + oB;
            post<M, false>(xs, lane, r2s, 0.f, 0.f, colA, colB, [&](int k, float &eA, float &, float &eB, float &) {
                if (k == 0) {
                    eA = f0A;
                    eB = f0B;
                }
            });
            if (lane == 0) {
                colA[n] = fnA;
                colB[n] = fnB;
            }
        }
        __syncwarp();
        // ---- central_diffz (inversion_utils.f90:653-673): levels 0..n-1
        // into gA / gB (the FFT buffer), level n in registers
        for (int iz = lane; iz < n; iz += 32) {
            const int lo = iz == 0 ? 0 : iz - 1;
            const float sc = iz == 0 ? dzi : hdzi;
            gA[iz] = (zA[iz + 1] - zA[lo]) * sc;
            gB[iz] = (zB[iz + 1] - zB[lo]) * sc;
        }
        const float gnA = dzi * (fnA - zA[n - 1]);
        const float gnB = dzi * (fnB - zB[n - 1]);
        // the pair buffer is free: start the next pair's copy
        if (ST) sg.next(lane, f, pr + warps, npairs, P);
        else __syncwarp();
        // ---- decompose the derivative
        const float g0A = gA[0], g0B = gB[0];
        {
            const Harm hA = Harm::make(lane_get(par, 0), dz, Lz, n, cA == 0);
            const Harm hB = Harm::make(lane_get(par, 8), dz, Lz, n, cB == 0);
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
                    v[m] = pre_sine(xa, ya, xb, yb, __ldg(&sinz[j]));
                }
            }
            __syncwarp();
            warp_fft<M>(v, xs, twn, lane);
        }
        {
            float *eA_ = es + oA, *eB_ = es + oB;
            post<M, false>(xs, lane, r2s, 0.f, 0.f, eA_, eB_, [&](int k, float &eA, float &, float &eB, float &) {
                if (k == 0) {
                    eA = g0A;
                    eB = g0B;
                }
            });
            if (lane == 0) {
                eA_[n] = gnA;
                eB_[n] = gnB;
            }
        }
        __syncwarp();
    }
    if (ST) sg.finish(lane);
}

// ------------------------------------------------------------------------
// The tail of the mixed source as three column kernels.  Each forms one
// tendency component of a column pair from the transformed products of
// vorticity_tendency (inversion.f90:298-388: spectral x / y derivatives by
// partner columns, as the orbit kernel k_svorts_orbit forms them) and
// decomposes it at once, so the undecomposed tendency never goes to HBM:
//   OUT 1: S1 = cy r(kx, -ky) - gq                 -> decompose(S1)
//   OUT 2: S2 = gp - cx r(-kx, ky)                 -> decompose(S2)
//   OUT 3: S3 = cx q(-kx, ky) - cy p(kx, -ky)      -> decompose(S3) and
//          es = decompose(central_diffz(S3))
// (-k: the partner column of the Hermitian storage).  One operand (gq, gp:
// the pair itself; q: the x-partner pair, also two adjacent columns) comes
// into the warp's pair buffer by the staged bulk copy; the other is read
// from global memory column by column while the buffer is overwritten with
// the combined values (for ky = 0 the y partners of a pair are columns 0 and
// ny - 1).  From there on OUT 1, 2 are the DECOMP column transform and
// OUT 3 is k_colz_dec2.
template <int M, int OUT>
__global__ void __launch_bounds__(256, M <= 16 ? 3 : 2)
    k_colz_src(const float *__restrict__ fs, const float *__restrict__ fh, float *__restrict__ out,
               float *__restrict__ es, int P, int ny, long long npairs, const double *__restrict__ k2l2,
               const double *__restrict__ cxv, const double *__restrict__ cyv, float dz, float Lz,
               const float2 *__restrict__ twn, const float *__restrict__ sinz, const float *__restrict__ corr)
{
    constexpr int n = 32 * M;
    constexpr bool ST = staged<M, float>();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    extern __shared__ __align__(16) unsigned char smz[];
    unsigned char *wbase = smz + COLZ_BAR_BYTES + (size_t)wib * warp_bytes(xs_bytes<M>(), true, P);
    float2 *xs = reinterpret_cast<float2 *>(wbase);
    float *zA = reinterpret_cast<float *>(wbase + xs_bytes<M>());
    float *zB = zA + P;
    float *gA = reinterpret_cast<float *>(xs), *gB = gA + n;
    const float r2s = 1.41421356237309505f * rsqrtf((float)n);
    const float dzi = 1.0f / dz, hdzi = 0.5f / dz;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    const long long first = (long long)blockIdx.x * (blockDim.x >> 5) + wib;
    // first column of the pair whose values the staged operand holds
    auto staged_col = [&](long long pr) -> long long {
        const long long cA = 2 * pr;
        if (OUT != 3) return cA;
        const long long kx = cA / ny;
        const long long ky = cA - kx * ny;
        const long long nx = (2 * npairs) / ny;
        return (kx == 0 ? 0 : nx - kx) * ny + ky;
    };
    Stager sg;
    if (ST) {
        sg.bar = smem_addr(smz + 8 * wib);
        sg.dst = smem_addr(zA);
        sg.bytes = 8u * (uint32_t)P;
        sg.phase = 0;
        sg.stopped = false;
        if (lane == 0) {
            stage_init(sg.bar);
            if (first < npairs) stage_copy(sg.dst, fs + staged_col(first) * (long long)P, sg.bytes, sg.bar);
        }
        __syncwarp();
    }
    for (long long pr = first; pr < npairs; pr += warps) {
        const long long cA = 2 * pr, cB = cA + 1;
        const long long oA = cA * P, oB = cB * P;
        const long long sA = staged_col(pr) * (long long)P;
        if (ST) {
            if (!sg.wait(lane)) break;
        } else {
            for (int iz = lane; iz <= n; iz += 32) {
                zA[iz] = fs[sA + iz];
                zB[iz] = fs[sA + P + iz];
            }
            __syncwarp();
        }
        // ---- the tendency component of both columns, in place
        {
            const long long kx = cA / ny;
            const int kyA = (int)(cA - kx * ny), kyB = kyA + 1;
            const long long nx = (2 * npairs) / ny;
            const long long xp = kx == 0 ? 0 : nx - kx;
            // columns of the operand read from global memory
            long long hA, hB;
            if (OUT == 2) {
                hA = (xp * ny + kyA) * P;
                hB = hA + P;
            } else {
                hA = (kx * ny + (kyA == 0 ? 0 : ny - kyA)) * P;
                hB = (kx * ny + (ny - kyB)) * P;
            }
            const float cx = (float)cxv[kx];
            const float cyA = (float)cyv[kyA], cyB = (float)cyv[kyB];
            auto comb = [&](float sv, float h, float cy) {
                if (OUT == 1) return fmaf(cy, h, -sv);
                if (OUT == 2) return fmaf(-cx, h, sv);
                return fmaf(cx, sv, -(cy * h));
            };
            // levels 0..n-1: every load of a batch issued before the first
            // is used (one memory latency per batch: both columns at once up
            // to nz = 512, one column at a time at nz = 1024); level n by
            // lanes 0 (column A) and 1 (column B)
            constexpr int NB = M <= 16 ? 2 : 1;
#pragma unroll
            for (int b0 = 0; b0 < 2; b0 += NB) {
                float h[NB][M];
#pragma unroll
                for (int b = 0; b < NB; ++b)
#pragma unroll
                    for (int m = 0; m < M; ++m) h[b][m] = fh[(b0 + b ? hB : hA) + lane + 32 * m];
#pragma unroll
                for (int b = 0; b < NB; ++b) {
                    float *zc = b0 + b ? zB : zA;
                    const float cy = b0 + b ? cyB : cyA;
#pragma unroll
                    for (int m = 0; m < M; ++m) zc[lane + 32 * m] = comb(zc[lane + 32 * m], h[b][m], cy);
                }
            }
            if (lane < 2) {
                float *zc = lane ? zB : zA;
                zc[n] = comb(zc[n], fh[(lane ? hB : hA) + n], lane ? cyB : cyA);
            }
            if (corr) {
                // an attached closure's correction of this component (the
                // pair's own columns), added as the separate add would
                __syncwarp();
                for (int i = lane; i < 2 * (n + 1); i += 32) {
                    const bool b = i > n;
                    const int z = b ? i - (n + 1) : i;
                    float *zp = (b ? zB : zA) + z;
                    *zp = *zp + corr[(b ? oB : oA) + z];
                }
            }
            __syncwarp();
        }
        // lanes 0 / 8: kl of columns A / B
        float par = 0.f;
        if (lane == 0 || lane == 8) par = sqrtf((float)k2l2[lane == 0 ? cA : cB]);
        const float f0A = zA[0], fnA = zA[n], f0B = zB[0], fnB = zB[n];
        // ---- decompose: subtract the harmonic part, dst
        {
            const Harm hA = Harm::make(lane_get(par, 0), dz, Lz, n, cA == 0);
            const Harm hB = Harm::make(lane_get(par, 8), dz, Lz, n, cB == 0);
            float2 v[M];
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const int j = lane + 32 * m;
                v[m] = make_float2(0.f, 0.f);
                if (j > 0) {
                    float xa = zA[j], ya = zA[n - j], xb = zB[j], yb = zB[n - j];
                    float pm, pp;
                    hA.at(j, n, pm, pp);
                    xa -= f0A * pm + fnA * pp;
                    ya -= f0A * pp + fnA * pm;
                    hB.at(j, n, pm, pp);
                    xb -= f0B * pm + fnB * pp;
                    yb -= f0B * pp + fnB * pm;
                    v[m] = pre_sine(xa, ya, xb, yb, __ldg(&sinz[j]));
                }
            }
            if (OUT != 3) {
                // the pair buffer is consumed: start the next pair's copy
                if (ST) {
                    __syncwarp();
                    if (lane == 0 && pr + warps < npairs)
                        stage_copy(sg.dst, fs + staged_col(pr + warps) * (long long)P, sg.bytes, sg.bar);
                } else {
                    __syncwarp();
                }
            }
            warp_fft<M>(v, xs, twn, lane);
        }
        {
            float *colA = out + oA, *colB = out + oB;
            post<M, false>(xs, lane, r2s, 0.f, 0.f, colA, colB, [&](int k, float &eA, float &, float &eB, float &) {
                if (k == 0) {
                    eA = f0A;
                    eB = f0B;
                }
            });
            if (lane == 0) {
                colA[n] = fnA;
                colB[n] = fnB;
            }
        }
        __syncwarp();
        if (OUT != 3) continue;
        // ---- central_diffz (inversion_utils.f90:653-673): levels 0..n-1
        // into gA / gB (the FFT buffer), level n in registers
        for (int iz = lane; iz < n; iz += 32) {
            const int lo = iz == 0 ? 0 : iz - 1;
            const float sc = iz == 0 ? dzi : hdzi;
            gA[iz] = (zA[iz + 1] - zA[lo]) * sc;
            gB[iz] = (zB[iz + 1] - zB[lo]) * sc;
        }
        const float gnA = dzi * (fnA - zA[n - 1]);
        const float gnB = dzi * (fnB - zB[n - 1]);
        __syncwarp();
        if (ST && lane == 0 && pr + warps < npairs)
            stage_copy(sg.dst, fs + staged_col(pr + warps) * (long long)P, sg.bytes, sg.bar);
        // ---- decompose the derivative
        const float g0A = gA[0], g0B = gB[0];
        {
            const Harm hA = Harm::make(lane_get(par, 0), dz, Lz, n, cA == 0);
            const Harm hB = Harm::make(lane_get(par, 8), dz, Lz, n, cB == 0);
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
                    v[m] = pre_sine(xa, ya, xb, yb, __ldg(&sinz[j]));
                }
            }
            __syncwarp();
            warp_fft<M>(v, xs, twn, lane);
        }
        {
            float *eA_ = es + oA, *eB_ = es + oB;
            post<M, false>(xs, lane, r2s, 0.f, 0.f, eA_, eB_, [&](int k, float &eA, float &, float &eB, float &) {
                if (k == 0) {
                    eA = g0A;
                    eB = g0B;
                }
            });
            if (lane == 0) {
                eA_[n] = gnA;
                eB_[n] = gnB;
            }
        }
        __syncwarp();
    }
    if (ST) sg.finish(lane);
}

namespace {
template <int M> size_t colz_smem(bool stage, int P) { return COLZ_BAR_BYTES + 8 * warp_bytes(xs_bytes<M>(), stage, P); }

// set by a launch whose pointers or pitch break the 16-byte rules (the
// kernels store 16-byte pairs of levels, the staged copy needs 16-byte
// runs): the launch is skipped and colz_error() reports it
bool g_colz_host_err = false;

bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

// One block of 8 warps per 8 pairs, at most as many blocks as are resident
// at once (the warps then loop over pairs, so each warp's prefetch of its
// next pair overlaps its current one).
template <typename K> unsigned colz_grid(K kern, size_t smem, long long npairs)
{
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const long long nb = (npairs + 7) / 8, cap = (long long)per_sm * sms;
    return (unsigned)(nb < cap ? nb : cap);
}

template <int MODE, int M, typename TIN>
void launch_colz_m(const TIN *in, float *out, const Dims &d, cudaStream_t st, const double *k2l2, float dz, float Lz,
                   const float2 *twn, const float *sinz, const float *cosz)
{
    const long long npairs = d.ncol / 2;
    const size_t smem = colz_smem<M>(staged<M, TIN>(), d.P);
    auto kern = k_colz<MODE, M, TIN>;
    kern<<<colz_grid(kern, smem, npairs), 256, smem, st>>>(in, out, d.P, npairs, k2l2, dz, Lz, twn, sinz, cosz);
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

template <int M>
void launch_w_m(const Dims &d, cudaStream_t st, const float *ds, float *w, float *es, const double *k2l2,
                const double *k2l2i, float dz, float Lz, const float2 *twn, const float *sinz, const float *cosz)
{
    const long long npairs = d.ncol / 2;
    const size_t smem = colz_smem<M>(staged<M, float>(), d.P);
    k_colz_w<M, 1><<<colz_grid(k_colz_w<M, 1>, smem, npairs), 256, smem, st>>>(ds, w, es, d.P, npairs, k2l2, k2l2i,
                                                                               dz, Lz, twn, sinz, cosz);
    k_colz_w<M, 2><<<colz_grid(k_colz_w<M, 2>, smem, npairs), 256, smem, st>>>(ds, w, es, d.P, npairs, k2l2, k2l2i,
                                                                               dz, Lz, twn, sinz, cosz);
}

template <int M>
void launch_w_src_m(const Dims &d, cudaStream_t st, const float *A, const float *B, float *w, float *es,
                    const double *k2l2, const double *k2l2i, const double *cx, const double *cy, float dz, float Lz,
                    const float2 *twn, const float *sinz, const float *cosz)
{
    if constexpr (staged<M, float>()) {
        const long long npairs = d.ncol / 2;
        const size_t smem = colz_smem<M>(true, d.P);
        k_colz_w<M, 1, true><<<colz_grid(k_colz_w<M, 1, true>, smem, npairs), 256, smem, st>>>(
            B, w, es, d.P, npairs, k2l2, k2l2i, dz, Lz, twn, sinz, cosz, A, cx, cy, d.ny);
        k_colz_w<M, 2, true><<<colz_grid(k_colz_w<M, 2, true>, smem, npairs), 256, smem, st>>>(
            B, w, es, d.P, npairs, k2l2, k2l2i, dz, Lz, twn, sinz, cosz, A, cx, cy, d.ny);
    }
}

template <int M>
void launch_dec2_m(const Dims &d, cudaStream_t st, const float *f, float *out, float *es, const double *k2l2,
                   float dz, float Lz, const float2 *twn, const float *sinz)
{
    const long long npairs = d.ncol / 2;
    const size_t smem = colz_smem<M>(true, d.P);
    k_colz_dec2<M><<<colz_grid(k_colz_dec2<M>, smem, npairs), 256, smem, st>>>(f, out, es, d.P, npairs, k2l2, dz, Lz,
                                                                               twn, sinz);
}

template <int M>
void launch_src_m(const Dims &d, cudaStream_t st, const float *r, const float *q, const float *p, const float *gq,
                  const float *gp, float *s1, float *s2, float *s3, float *es, const double *k2l2,
                  const double *cx, const double *cy, float dz, float Lz, const float2 *twn, const float *sinz,
                  const float *corr)
{
    const long long npairs = d.ncol / 2;
    const long long N = d.nfield;
    const size_t smem = colz_smem<M>(true, d.P);
    k_colz_src<M, 1><<<colz_grid(k_colz_src<M, 1>, smem, npairs), 256, smem, st>>>(
        gq, r, s1, nullptr, d.P, d.ny, npairs, k2l2, cx, cy, dz, Lz, twn, sinz, corr);
    k_colz_src<M, 2><<<colz_grid(k_colz_src<M, 2>, smem, npairs), 256, smem, st>>>(
        gp, r, s2, nullptr, d.P, d.ny, npairs, k2l2, cx, cy, dz, Lz, twn, sinz, corr ? corr + N : nullptr);
    k_colz_src<M, 3><<<colz_grid(k_colz_src<M, 3>, smem, npairs), 256, smem, st>>>(
        q, p, s3, es, d.P, d.ny, npairs, k2l2, cx, cy, dz, Lz, twn, sinz, corr ? corr + 2 * N : nullptr);
}

// every column kernel may take up to the device's opt-in shared memory per
// block (the launch asks for what its pitch needs)
template <typename K> void smem_attr(K kern, int optin)
{
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
}
template <int M> void attr_m(int optin)
{
    smem_attr(k_colz<COL_DST, M, float>, optin);
    smem_attr(k_colz<COL_DCT, M, float>, optin);
    smem_attr(k_colz<COL_DECOMP, M, float>, optin);
    smem_attr(k_colz<COL_COMBINE, M, float>, optin);
    smem_attr(k_colz<COL_DST, M, double>, optin);
    smem_attr(k_colz<COL_DCT, M, double>, optin);
    smem_attr(k_colz<COL_DECOMP, M, double>, optin);
    smem_attr(k_colz<COL_COMBINE, M, double>, optin);
    smem_attr(k_colz_w<M, 1>, optin);
    smem_attr(k_colz_w<M, 2>, optin);
    if constexpr (staged<M, float>()) {
        smem_attr(k_colz_w<M, 1, true>, optin);
        smem_attr(k_colz_w<M, 2, true>, optin);
    }
    smem_attr(k_colz_dec2<M>, optin);
    smem_attr(k_colz_src<M, 1>, optin);
    smem_attr(k_colz_src<M, 2>, optin);
    smem_attr(k_colz_src<M, 3>, optin);
}

// the 16-byte rules of the column kernels: pitch a multiple of 4 floats,
// every column pointer 16-byte aligned
bool colz_layout_ok(const Dims &d, const void *a, const void *b, const void *c)
{
    const bool ok = d.P % 4 == 0 && aligned16(a) && aligned16(b) && (!c || aligned16(c));
    if (!ok) g_colz_host_err = true;
    return ok;
}
}  // namespace

int colz_error()
{
    unsigned int e = 0;
    if (cudaMemcpyFromSymbol(&e, g_colz_err, sizeof(e)) != cudaSuccess) {
        cudaGetLastError();
        e = 0;
    }
    if (e) {
        const unsigned int z = 0;
        cudaMemcpyToSymbol(g_colz_err, &z, sizeof(z));
    }
    const bool h = g_colz_host_err;
    g_colz_host_err = false;
    return (e || h) ? 1 : 0;
}

void columns_w(const Dims &d, cudaStream_t st, const float *ds, float *w, float *es, const double *k2l2,
               const double *k2l2i, float dz, float Lz, const float2 *twn, const float *sinz, const float *cosz,
               Probe *pr)
{
    if (!colz_layout_ok(d, ds, w, es)) return;
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

bool columns_w_src_supported(int nz) { return nz == 64 || nz == 128 || nz == 256 || nz == 512; }

void columns_w_src(const Dims &d, cudaStream_t st, const float *A, const float *B, float *w, float *es,
                   const double *k2l2, const double *k2l2i, const double *cx, const double *cy, float dz, float Lz,
                   const float2 *twn, const float *sinz, const float *cosz, Probe *pr)
{
    if (!colz_layout_ok(d, A, B, w) || !colz_layout_ok(d, es, es, nullptr)) return;
    if (pr) pr->begin(PROBE_COLUMNS, st);
    switch (d.nz) {
    case 64: launch_w_src_m<2>(d, st, A, B, w, es, k2l2, k2l2i, cx, cy, dz, Lz, twn, sinz, cosz); break;
    case 128: launch_w_src_m<4>(d, st, A, B, w, es, k2l2, k2l2i, cx, cy, dz, Lz, twn, sinz, cosz); break;
    case 256: launch_w_src_m<8>(d, st, A, B, w, es, k2l2, k2l2i, cx, cy, dz, Lz, twn, sinz, cosz); break;
    default: launch_w_src_m<16>(d, st, A, B, w, es, k2l2, k2l2i, cx, cy, dz, Lz, twn, sinz, cosz); break;
    }
    // two launches, each reading A and B and writing one field
    if (pr) pr->end(PROBE_COLUMNS, st, 6.0 * (double)d.ncol * (double)(d.nz + 1) * sizeof(float));
}

void columns_dec2(const Dims &d, cudaStream_t st, const float *f, float *out, float *es, const double *k2l2,
                  float dz, float Lz, const float2 *twn, const float *sinz, Probe *pr)
{
    if (!colz_layout_ok(d, f, out, es)) return;
    if (pr) pr->begin(PROBE_COLUMNS, st);
    switch (d.nz) {
    case 64: launch_dec2_m<2>(d, st, f, out, es, k2l2, dz, Lz, twn, sinz); break;
    case 128: launch_dec2_m<4>(d, st, f, out, es, k2l2, dz, Lz, twn, sinz); break;
    case 256: launch_dec2_m<8>(d, st, f, out, es, k2l2, dz, Lz, twn, sinz); break;
    case 512: launch_dec2_m<16>(d, st, f, out, es, k2l2, dz, Lz, twn, sinz); break;
    default: launch_dec2_m<32>(d, st, f, out, es, k2l2, dz, Lz, twn, sinz); break;
    }
    if (pr) pr->end(PROBE_COLUMNS, st, 3.0 * (double)d.ncol * (double)(d.nz + 1) * sizeof(float));
}

void columns_src(const Dims &d, cudaStream_t st, const float *r, const float *q, const float *p, const float *gq,
                 const float *gp, float *s1, float *s2, float *s3, float *es, const double *k2l2, const double *cx,
                 const double *cy, float dz, float Lz, const float2 *twn, const float *sinz, Probe *pr,
                 const float *corr)
{
    if (!colz_layout_ok(d, r, q, p) || !colz_layout_ok(d, gq, gp, es) || !colz_layout_ok(d, s1, s2, s3)) return;
    if (pr) pr->begin(PROBE_COLUMNS, st);
    switch (d.nz) {
    case 64: launch_src_m<2>(d, st, r, q, p, gq, gp, s1, s2, s3, es, k2l2, cx, cy, dz, Lz, twn, sinz, corr); break;
    case 128: launch_src_m<4>(d, st, r, q, p, gq, gp, s1, s2, s3, es, k2l2, cx, cy, dz, Lz, twn, sinz, corr); break;
    case 256: launch_src_m<8>(d, st, r, q, p, gq, gp, s1, s2, s3, es, k2l2, cx, cy, dz, Lz, twn, sinz, corr); break;
    case 512: launch_src_m<16>(d, st, r, q, p, gq, gp, s1, s2, s3, es, k2l2, cx, cy, dz, Lz, twn, sinz, corr); break;
    default: launch_src_m<32>(d, st, r, q, p, gq, gp, s1, s2, s3, es, k2l2, cx, cy, dz, Lz, twn, sinz, corr); break;
    }
    // six fields read, four written (three launches)
    if (pr) pr->end(PROBE_COLUMNS, st, 10.0 * (double)d.ncol * (double)(d.nz + 1) * sizeof(float));
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
    int dev = 0, optin = 48 * 1024;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    attr_m<2>(optin);
    attr_m<4>(optin);
    attr_m<8>(optin);
    attr_m<16>(optin);
    attr_m<32>(optin);
}

template <typename TIN>
void columns_z(const Dims &d, cudaStream_t st, int mode, const TIN *in, float *out, const double *k2l2, float dz,
               float Lz, const float2 *twn, const float *sinz, const float *cosz, Probe *pr)
{
    if (!colz_layout_ok(d, in, out, nullptr)) return;
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
