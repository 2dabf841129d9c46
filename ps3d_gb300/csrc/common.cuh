// Shared device helpers for the ps3d GB300 kernels: complex arithmetic,
// radix-2/4/8 butterflies and the shared-memory Stockham FFT used by every
// transform kernel.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace ps3d {

template <typename T> struct cplx;
template <> struct cplx<double> { using type = double2; };
template <> struct cplx<float> { using type = float2; };

template <typename C> __device__ __forceinline__ C mk(decltype(C::x) x, decltype(C::x) y)
{
    C c;
    c.x = x;
    c.y = y;
    return c;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return mk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return mk<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b)
{
    return mk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// multiply by -i (forward) or +i (inverse)
template <bool INV, typename C> __device__ __forceinline__ C mul_mi(C a)
{
    return INV ? mk<C>(-a.y, a.x) : mk<C>(a.y, -a.x);
}

// In-register DFTs with the sign of the forward (e^{-2 pi i/R}) or inverse
// transform.
template <bool INV, typename C> __device__ __forceinline__ void dft2(C &a, C &b)
{
    C t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <bool INV, typename C> __device__ __forceinline__ void dft4(C &a0, C &a1, C &a2, C &a3)
{
    C t0 = cadd(a0, a2), t1 = csub(a0, a2);
    C t2 = cadd(a1, a3), t3 = mul_mi<INV>(csub(a1, a3));
    a0 = cadd(t0, t2);
    a2 = csub(t0, t2);
    a1 = cadd(t1, t3);
    a3 = csub(t1, t3);
}

template <bool INV, typename C> __device__ __forceinline__ void dft8(C *v)
{
    using R = decltype(C::x);
    const R h = (R)0.70710678118654752440084436210484903928483593768847;
    // even / odd halves
    dft4<INV>(v[0], v[2], v[4], v[6]);
    dft4<INV>(v[1], v[3], v[5], v[7]);
    // twiddle the odd half by w8^k, k = 0..3
    C o1 = v[3], o2 = v[5], o3 = v[7];
    if (!INV) {
        o1 = mk<C>((o1.x + o1.y) * h, (o1.y - o1.x) * h);   // (1-i)/sqrt2
        o2 = mk<C>(o2.y, -o2.x);                            // -i
        o3 = mk<C>((o3.y - o3.x) * h, -(o3.x + o3.y) * h);  // (-1-i)/sqrt2
    } else {
        o1 = mk<C>((o1.x - o1.y) * h, (o1.x + o1.y) * h);   // (1+i)/sqrt2
        o2 = mk<C>(-o2.y, o2.x);                            // +i
        o3 = mk<C>(-(o3.x + o3.y) * h, (o3.x - o3.y) * h);  // (-1+i)/sqrt2
    }
    C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6], o0 = v[1];
    v[0] = cadd(e0, o0);
    v[4] = csub(e0, o0);
    v[1] = cadd(e1, o1);
    v[5] = csub(e1, o1);
    v[2] = cadd(e2, o2);
    v[6] = csub(e2, o2);
    v[3] = cadd(e3, o3);
    v[7] = csub(e3, o3);
}

// radix 3: X1, X2 = m -/+ i (sqrt3/2) (a1 - a2), m = a0 - (a1 + a2)/2
// (forward; the inverse swaps the signs of the imaginary terms)
template <bool INV, typename C> __device__ __forceinline__ void dft3(C *v)
{
    using R = decltype(C::x);
    const R h = (R)0.86602540378443864676372317075293618347140262690519;  // sqrt(3)/2
    const C t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
    const C m = mk<C>(v[0].x - (R)0.5 * t1.x, v[0].y - (R)0.5 * t1.y);
    // -i h t2 (forward) or +i h t2 (inverse)
    const C s = INV ? mk<C>(-h * t2.y, h * t2.x) : mk<C>(h * t2.y, -h * t2.x);
    v[0] = cadd(v[0], t1);
    v[1] = cadd(m, s);
    v[2] = csub(m, s);
}

// radix 5 from the real and imaginary parts of w = exp(-2 pi i / 5):
// t1 = a1 + a4, t2 = a2 + a3, t3 = a1 - a4, t4 = a2 - a3,
// X1, X4 = (a0 + c1 t1 + c2 t2) -/+ i (s1 t3 + s2 t4),
// X2, X3 = (a0 + c2 t1 + c1 t2) -/+ i (s2 t3 - s1 t4),
// c1 = cos(2 pi/5), c2 = cos(4 pi/5), s1 = sin(2 pi/5), s2 = sin(4 pi/5)
template <bool INV, typename C> __device__ __forceinline__ void dft5(C *v)
{
    using R = decltype(C::x);
    const R c1 = (R)0.30901699437494742410229341718281905886436448684277;
    const R c2 = (R)-0.80901699437494742410229341718281905886436448684277;
    const R s1 = (R)0.95105651629515357211643933337938214340569863412575;
    const R s2 = (R)0.58778525229247312916870595463907276859765243764314;
    const C t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]), t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
    const C m1 = mk<C>(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
    const C m2 = mk<C>(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
    const C n1 = mk<C>(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
    const C n2 = mk<C>(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
    // -i n (forward) or +i n (inverse)
    const C j1 = INV ? mk<C>(-n1.y, n1.x) : mk<C>(n1.y, -n1.x);
    const C j2 = INV ? mk<C>(-n2.y, n2.x) : mk<C>(n2.y, -n2.x);
    v[0] = cadd(v[0], cadd(t1, t2));
    v[1] = cadd(m1, j1);
    v[4] = csub(m1, j1);
    v[2] = cadd(m2, j2);
    v[3] = csub(m2, j2);
}

template <int R, bool INV, typename C> __device__ __forceinline__ void dft(C *v)
{
    if (R == 2) dft2<INV>(v[0], v[1]);
    else if (R == 3) dft3<INV>(v);
    else if (R == 4) dft4<INV>(v[0], v[1], v[2], v[3]);
    else if (R == 5) dft5<INV>(v);
    else dft8<INV>(v);
}

// One Stockham autosort pass of radix R over B interleaved sequences of
// length n held in shared memory as buf[j*B + b].  Ns is the product of the
// radices already applied (any order of the factors of n).
// tw[k] = exp(-2 pi i k / n).
template <int R, bool INV, typename C>
__device__ __forceinline__ void stockham_pass(const C *__restrict__ src, C *__restrict__ dst, int n,
                                              int logB, int Ns, const C *__restrict__ tw)
{
    const int B = 1 << logB;
    const int nR = n / R;
    const int nbf = nR << logB;
    const int twstride = n / (Ns * R);
    for (int g = threadIdx.x; g < nbf; g += blockDim.x) {
        const int b = g & (B - 1);
        const int j = g >> logB;
        const int k = ((Ns & (Ns - 1)) == 0) ? (j & (Ns - 1)) : (j % Ns);
        C v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = src[((j + r * nR) << logB) + b];
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                C w = tw[k * r * twstride];
                if (INV) w.y = -w.y;
                v[r] = cmul(v[r], w);
            }
        }
        dft<R, INV>(v);
        const int idxD = (j - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) dst[((idxD + r * Ns) << logB) + b] = v[r];
    }
}

// Complex FFT of B = 2^logB interleaved sequences of length n = 2^a 3^b 5^c
// (2..4096) in shared memory: radix-8 passes while 8 divides what is left,
// one radix-4 or radix-2 pass for the rest of the power of two, then the
// radix-3 and radix-5 passes (the factorisation of stafft.f90:128-187, in
// its own order).  buf0 holds the input, the result ends in the returned
// buffer (buf0 or buf1).  All threads of the block take part; the caller
// synchronises before the call.
template <bool INV, typename C>
__device__ C *smem_fft(C *buf0, C *buf1, int n, int logB, const C *__restrict__ tw)
{
    C *s = buf0, *d = buf1;
    int Ns = 1, rem = n;
    auto step = [&](auto radix) {
        constexpr int R = decltype(radix)::value;
        stockham_pass<R, INV>(s, d, n, logB, Ns, tw);
        __syncthreads();
        C *t = s;
        s = d;
        d = t;
        Ns *= R;
        rem /= R;
    };
    while (rem % 8 == 0) step(std::integral_constant<int, 8>());
    if (rem % 4 == 0) step(std::integral_constant<int, 4>());
    else if (rem % 2 == 0) step(std::integral_constant<int, 2>());
    while (rem % 3 == 0) step(std::integral_constant<int, 3>());
    while (rem % 5 == 0) step(std::integral_constant<int, 5>());
    return s;
}

// n = 2^a 3^b 5^c
__host__ __device__ inline bool radix235(int n)
{
    if (n < 1) return false;
    for (int p : {2, 3, 5})
        while (n % p == 0) n /= p;
    return n == 1;
}

__host__ __device__ inline int ilog2(int v)
{
    int r = 0;
    while ((1 << r) < v) ++r;
    return r;
}

}  // namespace ps3d

namespace ps3d {
// FP32 <-> FP64 conversions with integer instructions only (GB300 runs
// F2F to or from FP64 on its narrow FP64 pipe).  narrow32 rounds to nearest
// (ties away from zero) and flushes results below the FP32 normal range to
// zero; widen64 is exact for normal FP32 values and flushes FP32 denormals.
__device__ __forceinline__ float narrow32(double x)
{
    const long long b = __double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ff) - 1023 + 127;
    if (e <= 0) return __uint_as_float(sign);
    if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
    unsigned f = sign | ((unsigned)e << 23);
    f += ((hi & 0xfffffu) << 3) | (lo >> 29);
    f += (lo >> 28) & 1u;
    return __uint_as_float(f);
}

__device__ __forceinline__ double widen64(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned long long s = (unsigned long long)(u & 0x80000000u) << 32;
    if (e == 0) return __longlong_as_double((long long)s);
    const unsigned long long de = (e == 255u) ? 2047ull : (unsigned long long)(e + 896u);
    return __longlong_as_double((long long)(s | (de << 52) | ((unsigned long long)(u & 0x7fffffu) << 29)));
}
}  // namespace ps3d
