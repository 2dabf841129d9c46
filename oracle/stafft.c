/*
 * CPU oracle (test infrastructure, not the product): restatement of the
 * reference's 1-D real transform module, src/fft/stafft.f90 (matt-frey/ps3d,
 * BSD-3-Clause).  FP64 throughout.
 *
 * Conventions kept from the reference:
 *   - forfft: m real sequences of length n, stored x[i + m*j] (i = sequence,
 *     j = sample), transformed in place into "Hermitian" order:
 *       x[0]            = mean mode,
 *       x[1 .. n/2]     = cosine modes k = 1 .. n/2,
 *       x[n-k]          = sine mode k (k = 1 .. (n-1)/2, stored in reverse),
 *     scaled by 1/sqrt(n)                         (stafft.f90:55-58, 277).
 *   - revfft: the inverse (sine part negated, mean/Nyquist halved, radix
 *     passes, scale 2/sqrt(n))                     (stafft.f90:296-403).
 *   - dct: self-inverse cosine transform on x[0..n]  (stafft.f90:410-483).
 *   - dst: self-inverse sine transform on x[1..n-1], x[n] := 0
 *                                                   (stafft.f90:489-550).
 *
 * The radix-4 and radix-2 passes (the only ones a power-of-two length uses)
 * restate forrdx4/forrdx2 (stafft.f90:901-1152) and revrdx4/revrdx2
 * (stafft.f90:1503-1757).  Lengths whose factorisation needs 3, 5 or 6 fall
 * back to a direct O(n^2) evaluation of the same transform definition, which
 * is adequate for the small sizes the tests use on those lengths.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "ps3d_oracle.h"

static const double RTF12 = 0.70710678118654752440084436210484903928483593768847;
static const double RT2 = 1.41421356237309504880168872420969807856967187537695;

/* factorisen (stafft.f90:128-187): counts of 6, 4, 2, 3, 5 in that order. */
int ps3o_factorise(int n, int factors[5])
{
    static const int fac[5] = {6, 4, 2, 3, 5};
    int rem = n;
    for (int i = 0; i < 5; ++i) factors[i] = 0;
    if (n < 2) return 1;
    for (int i = 0; i < 5; ++i) {
        while (rem % fac[i] == 0) {
            factors[i] += 1;
            rem /= fac[i];
            if (rem == 1) return 0;
        }
    }
    return 1;
}

/* initfft (stafft.f90:76-125): the trig table is the concatenation, stage by
 * stage in the order 6,4,2,3,5, of cos/-sin(2*pi*k*l/len) for k=1..R-1 and
 * l=0..rem-1 (l fastest).  trig[0..n-1] holds cosines, trig[n..2n-1] -sines. */
int ps3o_initfft(int n, int factors[5], double *trig)
{
    static const int fac[5] = {6, 4, 2, 3, 5};
    if (ps3o_factorise(n, factors) != 0) return 1;
    const double twopi = 2.0 * acos(-1.0);
    double ftwopin = twopi / (double)n;
    int rem = n, m = 0;
    for (int i = 0; i < 5; ++i) {
        for (int j = 0; j < factors[i]; ++j) {
            rem /= fac[i];
            for (int k = 1; k < fac[i]; ++k)
                for (int l = 0; l < rem; ++l)
                    trig[m++] = ftwopin * (double)(k * l);
            ftwopin *= fac[i];
        }
    }
    for (int i = 0; i < n - 1; ++i) {
        double a = trig[i];
        trig[n + i] = -sin(a);
        trig[i] = cos(a);
    }
    trig[n - 1] = 0.0;
    trig[2 * n - 1] = 0.0;
    return 0;
}

static int needs_generic(const int factors[5])
{
    return factors[0] != 0 || factors[3] != 0 || factors[4] != 0;
}

/* ---------------------------------------------------------------------- */
/* forward radix passes ("decimation in time", physical -> Hermitian)      */
/* a(0:nv-1, 0:R-1, 0:lv-1) -> b(0:nv-1, 0:lv-1, 0:R-1)                    */
/* ---------------------------------------------------------------------- */

#define A3(i, r, k) a[(i) + nv * ((r) + R * (k))]
#define B3(i, k, r) b[(i) + nv * ((k) + lv * (r))]

/* forrdx2, stafft.f90:1101-1152 */
static void forrdx2(const double *a, double *b, int nv, int lv,
                    const double *cosine, const double *sine)
{
    const int R = 2;
    for (int i = 0; i < nv; ++i) {
        B3(i, 0, 0) = A3(i, 0, 0) + A3(i, 1, 0);
        B3(i, 0, 1) = A3(i, 0, 0) - A3(i, 1, 0);
    }
    for (int k = 1; k <= (lv - 1) / 2; ++k) {
        const int kc = lv - k;
        const double c1 = cosine[k], s1 = sine[k];
        for (int i = 0; i < nv; ++i) {
            double x1 = c1 * A3(i, 1, k) - s1 * A3(i, 1, kc);
            double y1 = c1 * A3(i, 1, kc) + s1 * A3(i, 1, k);
            B3(i, k, 0) = A3(i, 0, k) + x1;
            B3(i, kc, 0) = A3(i, 0, k) - x1;
            B3(i, k, 1) = y1 - A3(i, 0, kc);
            B3(i, kc, 1) = A3(i, 0, kc) + y1;
        }
    }
}

/* forrdx4, stafft.f90:901-1013 */
static void forrdx4(const double *a, double *b, int nv, int lv,
                    const double *cosine, const double *sine)
{
    const int R = 4;
#define C4(k, r) cosine[(k) + lv * ((r) - 1)]
#define S4(k, r) sine[(k) + lv * ((r) - 1)]
    for (int i = 0; i < nv; ++i) {
        double t1r = A3(i, 0, 0) + A3(i, 2, 0);
        double t2r = A3(i, 1, 0) + A3(i, 3, 0);
        B3(i, 0, 0) = t1r + t2r;
        B3(i, 0, 1) = A3(i, 0, 0) - A3(i, 2, 0);
        B3(i, 0, 2) = t1r - t2r;
        B3(i, 0, 3) = A3(i, 3, 0) - A3(i, 1, 0);
    }
    for (int k = 1; k <= (lv - 1) / 2; ++k) {
        const int kc = lv - k;
        const double c1 = C4(k, 1), s1 = S4(k, 1);
        const double c2 = C4(k, 2), s2 = S4(k, 2);
        const double c3 = C4(k, 3), s3 = S4(k, 3);
        for (int i = 0; i < nv; ++i) {
            double x1 = c1 * A3(i, 1, k) - s1 * A3(i, 1, kc);
            double y1 = c1 * A3(i, 1, kc) + s1 * A3(i, 1, k);
            double x2 = c2 * A3(i, 2, k) - s2 * A3(i, 2, kc);
            double y2 = c2 * A3(i, 2, kc) + s2 * A3(i, 2, k);
            double x3 = c3 * A3(i, 3, k) - s3 * A3(i, 3, kc);
            double y3 = c3 * A3(i, 3, kc) + s3 * A3(i, 3, k);
            double t1r = A3(i, 0, k) + x2, t1i = A3(i, 0, kc) + y2;
            double t2r = x1 + x3, t2i = y1 + y3;
            double t3r = A3(i, 0, k) - x2, t3i = A3(i, 0, kc) - y2;
            double t4r = x3 - x1, t4i = y1 - y3;
            B3(i, k, 0) = t1r + t2r;
            B3(i, kc, 0) = t3r - t4i;
            B3(i, k, 1) = t3r + t4i;
            B3(i, kc, 1) = t1r - t2r;
            B3(i, k, 2) = t2i - t1i;
            B3(i, kc, 2) = t3i + t4r;
            B3(i, k, 3) = t4r - t3i;
            B3(i, kc, 3) = t1i + t2i;
        }
    }
    if (lv % 2 == 0) {
        const int h = lv / 2;
        for (int i = 0; i < nv; ++i) {
            double q1 = RTF12 * (A3(i, 1, h) - A3(i, 3, h));
            double q2 = RTF12 * (A3(i, 1, h) + A3(i, 3, h));
            B3(i, h, 0) = A3(i, 0, h) + q1;
            B3(i, h, 1) = A3(i, 0, h) - q1;
            B3(i, h, 2) = A3(i, 2, h) - q2;
            B3(i, h, 3) = -A3(i, 2, h) - q2;
        }
    }
#undef C4
#undef S4
}
#undef A3
#undef B3

/* ---------------------------------------------------------------------- */
/* reverse radix passes ("decimation in frequency", Hermitian -> physical) */
/* a(0:nv-1, 0:lv-1, 0:R-1) -> b(0:nv-1, 0:R-1, 0:lv-1)                    */
/* ---------------------------------------------------------------------- */
#define A3(i, k, r) a[(i) + nv * ((k) + lv * (r))]
#define B3(i, r, k) b[(i) + nv * ((r) + R * (k))]

/* revrdx2, stafft.f90:1706-1757 */
static void revrdx2(const double *a, double *b, int nv, int lv,
                    const double *cosine, const double *sine)
{
    const int R = 2;
    for (int i = 0; i < nv; ++i) {
        B3(i, 0, 0) = A3(i, 0, 0) + A3(i, 0, 1);
        B3(i, 1, 0) = A3(i, 0, 0) - A3(i, 0, 1);
    }
    for (int k = 1; k <= (lv - 1) / 2; ++k) {
        const int kc = lv - k;
        const double c1 = cosine[k], s1 = sine[k];
        for (int i = 0; i < nv; ++i) {
            double x1 = A3(i, k, 0) - A3(i, kc, 0);
            double y1 = A3(i, kc, 1) + A3(i, k, 1);
            B3(i, 0, k) = A3(i, k, 0) + A3(i, kc, 0);
            B3(i, 0, kc) = A3(i, kc, 1) - A3(i, k, 1);
            B3(i, 1, k) = c1 * x1 - s1 * y1;
            B3(i, 1, kc) = c1 * y1 + s1 * x1;
        }
    }
}

/* revrdx4, stafft.f90:1503-1616 */
static void revrdx4(const double *a, double *b, int nv, int lv,
                    const double *cosine, const double *sine)
{
    const int R = 4;
#define C4(k, r) cosine[(k) + lv * ((r) - 1)]
#define S4(k, r) sine[(k) + lv * ((r) - 1)]
    for (int i = 0; i < nv; ++i) {
        double t1r = A3(i, 0, 0) + A3(i, 0, 2);
        double t2r = A3(i, 0, 1);
        double t3r = A3(i, 0, 0) - A3(i, 0, 2);
        double t4r = A3(i, 0, 3);
        B3(i, 0, 0) = t1r + t2r;
        B3(i, 1, 0) = t3r + t4r;
        B3(i, 2, 0) = t1r - t2r;
        B3(i, 3, 0) = t3r - t4r;
    }
    for (int k = 1; k <= (lv - 1) / 2; ++k) {
        const int kc = lv - k;
        const double c1 = C4(k, 1), s1 = S4(k, 1);
        const double c2 = C4(k, 2), s2 = S4(k, 2);
        const double c3 = C4(k, 3), s3 = S4(k, 3);
        for (int i = 0; i < nv; ++i) {
            double t1r = A3(i, k, 0) + A3(i, kc, 1);
            double t1i = A3(i, kc, 3) - A3(i, k, 2);
            double t2r = A3(i, k, 1) + A3(i, kc, 0);
            double t2i = A3(i, kc, 2) - A3(i, k, 3);
            double t3r = A3(i, k, 0) - A3(i, kc, 1);
            double t3i = A3(i, kc, 3) + A3(i, k, 2);
            double t4r = A3(i, k, 1) - A3(i, kc, 0);
            double t4i = A3(i, kc, 2) + A3(i, k, 3);
            double x1 = t3r + t4i, y1 = t3i - t4r;
            double x2 = t1r - t2r, y2 = t1i - t2i;
            double x3 = t3r - t4i, y3 = t3i + t4r;
            B3(i, 0, k) = t1r + t2r;
            B3(i, 0, kc) = t1i + t2i;
            B3(i, 1, k) = c1 * x1 - s1 * y1;
            B3(i, 1, kc) = c1 * y1 + s1 * x1;
            B3(i, 2, k) = c2 * x2 - s2 * y2;
            B3(i, 2, kc) = c2 * y2 + s2 * x2;
            B3(i, 3, k) = c3 * x3 - s3 * y3;
            B3(i, 3, kc) = c3 * y3 + s3 * x3;
        }
    }
    if (lv % 2 == 0) {
        const int h = lv / 2;
        for (int i = 0; i < nv; ++i) {
            B3(i, 0, h) = A3(i, h, 0) + A3(i, h, 1);
            B3(i, 2, h) = A3(i, h, 3) - A3(i, h, 2);
            double t3r = A3(i, h, 0) - A3(i, h, 1);
            double t4r = A3(i, h, 3) + A3(i, h, 2);
            B3(i, 1, h) = RTF12 * (t3r + t4r);
            B3(i, 3, h) = RTF12 * (t4r - t3r);
        }
    }
#undef C4
#undef S4
}
#undef A3
#undef B3

/* ---------------------------------------------------------------------- */
/* generic lengths: direct evaluation of the same Hermitian transform      */
/* ---------------------------------------------------------------------- */
static void forfft_direct(int m, int n, double *x, double *wk)
{
    const double twopi = 2.0 * acos(-1.0);
    const double s = 1.0 / sqrt((double)n);
    for (int i = 0; i < m; ++i) {
        for (int k = 0; k <= n / 2; ++k) {
            double re = 0.0, im = 0.0;
            for (int j = 0; j < n; ++j) {
                double ang = twopi * (double)((long)j * k % n) / (double)n;
                re += x[i + m * j] * cos(ang);
                im -= x[i + m * j] * sin(ang);
            }
            wk[i + m * k] = re * s;
            if (k >= 1 && n - k > n / 2) wk[i + m * (n - k)] = im * s;
        }
    }
    memcpy(x, wk, sizeof(double) * (size_t)m * n);
}

static void revfft_direct(int m, int n, double *x, double *wk)
{
    const double twopi = 2.0 * acos(-1.0);
    const double s = 1.0 / sqrt((double)n);
    for (int i = 0; i < m; ++i) {
        for (int j = 0; j < n; ++j) {
            double v = x[i];
            for (int k = 1; k <= (n - 1) / 2; ++k) {
                double ang = twopi * (double)((long)j * k % n) / (double)n;
                v += 2.0 * (x[i + m * k] * cos(ang) - x[i + m * (n - k)] * sin(ang));
            }
            if (n % 2 == 0) v += x[i + m * (n / 2)] * ((j % 2) ? -1.0 : 1.0);
            wk[i + m * j] = v * s;
        }
    }
    memcpy(x, wk, sizeof(double) * (size_t)m * n);
}

/* ---------------------------------------------------------------------- */
/* forfft (stafft.f90:196-287).  wk: m*n doubles of scratch.               */
/* ---------------------------------------------------------------------- */
void ps3o_forfft(int m, int n, double *x, double *wk, const double *trig,
                 const int factors[5])
{
    if (needs_generic(factors)) {
        forfft_direct(m, n, x, wk);
        return;
    }
    int orig = 1, rem = n, cum = 1;
    /* factors of 2 (at most one for a power of two) then factors of 4 */
    for (int i = 0; i < factors[2]; ++i) {
        rem /= 2;
        const int iloc = (rem - 1) * 2 * cum;
        if (orig) forrdx2(x, wk, m * rem, cum, trig + iloc, trig + n + iloc);
        else      forrdx2(wk, x, m * rem, cum, trig + iloc, trig + n + iloc);
        orig = !orig;
        cum *= 2;
    }
    for (int i = 0; i < factors[1]; ++i) {
        rem /= 4;
        const int iloc = (rem - 1) * 4 * cum;
        if (orig) forrdx4(x, wk, m * rem, cum, trig + iloc, trig + n + iloc);
        else      forrdx4(wk, x, m * rem, cum, trig + iloc, trig + n + iloc);
        orig = !orig;
        cum *= 4;
    }
    const double normfac = 1.0 / sqrt((double)n);
    const size_t len = (size_t)m * n;
    if (orig) {
        for (size_t i = 0; i < len; ++i) x[i] *= normfac;
    } else {
        for (size_t i = 0; i < len; ++i) x[i] = wk[i] * normfac;
    }
}

/* revfft (stafft.f90:296-403). */
void ps3o_revfft(int m, int n, double *x, double *wk, const double *trig,
                 const int factors[5])
{
    if (needs_generic(factors)) {
        revfft_direct(m, n, x, wk);
        return;
    }
    /* flip the sign of the sine coefficients, halve mean and Nyquist */
    for (size_t i = (size_t)(n / 2 + 1) * m; i < (size_t)n * m; ++i) x[i] = -x[i];
    for (int i = 0; i < m; ++i) x[i] *= 0.5;
    if (n % 2 == 0) {
        const size_t k = (size_t)m * (n / 2);
        for (int i = 0; i < m; ++i) x[k + i] *= 0.5;
    }
    int orig = 1, cum = 1, rem = n;
    for (int i = 0; i < factors[1]; ++i) {
        rem /= 4;
        const int iloc = (cum - 1) * 4 * rem;
        if (orig) revrdx4(x, wk, m * cum, rem, trig + iloc, trig + n + iloc);
        else      revrdx4(wk, x, m * cum, rem, trig + iloc, trig + n + iloc);
        orig = !orig;
        cum *= 4;
    }
    for (int i = 0; i < factors[2]; ++i) {
        rem /= 2;
        const int iloc = (cum - 1) * 2 * rem;
        if (orig) revrdx2(x, wk, m * cum, rem, trig + iloc, trig + n + iloc);
        else      revrdx2(wk, x, m * cum, rem, trig + iloc, trig + n + iloc);
        orig = !orig;
        cum *= 2;
    }
    const double normfac = 2.0 / sqrt((double)n);
    const size_t len = (size_t)m * n;
    if (orig) {
        for (size_t i = 0; i < len; ++i) x[i] *= normfac;
    } else {
        for (size_t i = 0; i < len; ++i) x[i] = wk[i] * normfac;
    }
}

/* dct (stafft.f90:410-483): x(m, 0:n), self-inverse.
 * wk: m*n doubles, wk2: m*n doubles (scratch for forfft). */
void ps3o_dct(int m, int n, double *x, double *wk, double *wk2,
              const double *trig, const int factors[5])
{
    const double fpin = acos(-1.0) / (double)n;
    const double rtn = sqrt((double)n);
#define X(i, j) x[(i) + (size_t)m * (j)]
#define W(i, j) wk[(i) + (size_t)m * (j)]
    for (int i = 0; i < m; ++i) W(i, 0) = 0.5 * (X(i, 0) + X(i, n));
    for (int j = 1; j < n; ++j) {
        const double sj = sin((double)j * fpin);
        for (int i = 0; i < m; ++i)
            W(i, j) = 0.5 * (X(i, j) + X(i, n - j)) - sj * (X(i, j) - X(i, n - j));
    }
    /* first coefficient by a direct sum, parked in x(:, n) */
    for (int i = 0; i < m; ++i) {
        double rowsum = 0.0;
        rowsum += 0.5 * X(i, 0);
        for (int j = 1; j < n; ++j) rowsum += X(i, j) * cos((double)j * fpin);
        rowsum -= 0.5 * X(i, n);
        X(i, n) = RT2 * rowsum / rtn;
    }
    ps3o_forfft(m, n, wk, wk2, trig, factors);
    for (int i = 0; i < m; ++i) X(i, 0) = RT2 * W(i, 0);
    for (int i = 0; i < m; ++i) X(i, 1) = X(i, n);
    if (n % 2 == 0) {
        const int nd2 = n / 2;
        for (int j = 1; j < nd2; ++j)
            for (int i = 0; i < m; ++i) {
                X(i, 2 * j) = RT2 * W(i, j);
                X(i, 2 * j + 1) = X(i, 2 * j - 1) - RT2 * W(i, n - j);
            }
        for (int i = 0; i < m; ++i) X(i, n) = RT2 * W(i, nd2);
    } else {
        for (int j = 1; j <= (n - 1) / 2; ++j)
            for (int i = 0; i < m; ++i) {
                X(i, 2 * j) = RT2 * W(i, j);
                X(i, 2 * j + 1) = X(i, 2 * j - 1) - RT2 * W(i, n - j);
            }
    }
#undef X
#undef W
}

/* dst (stafft.f90:489-550): x(m, 1:n) passed as a pointer to x(1,1),
 * self-inverse on 1..n-1, x(:, n) := 0. */
void ps3o_dst(int m, int n, double *x1, double *wk, double *wk2,
              const double *trig, const int factors[5])
{
    const double fpin = acos(-1.0) / (double)n;
#define X(i, j) x1[(i) + (size_t)m * ((j) - 1)]
#define W(i, j) wk[(i) + (size_t)m * (j)]
    for (int i = 0; i < m; ++i) W(i, 0) = 0.0;
    for (int j = 1; j < n; ++j) {
        const double sj = sin((double)j * fpin);
        for (int i = 0; i < m; ++i)
            W(i, j) = 0.5 * (X(i, j) - X(i, n - j)) + sj * (X(i, j) + X(i, n - j));
    }
    ps3o_forfft(m, n, wk, wk2, trig, factors);
    for (int i = 0; i < m; ++i) X(i, 1) = W(i, 0) / RT2;
    if (n % 2 == 0) {
        for (int j = 1; j < n / 2; ++j) {
            for (int i = 0; i < m; ++i) X(i, 2 * j) = -RT2 * W(i, n - j);
            for (int i = 0; i < m; ++i) X(i, 2 * j + 1) = RT2 * W(i, j) + X(i, 2 * j - 1);
        }
    } else {
        for (int j = 1; j < (n - 1) / 2; ++j)
            for (int i = 0; i < m; ++i) {
                X(i, 2 * j) = -RT2 * W(i, n - j);
                X(i, 2 * j + 1) = RT2 * W(i, j) + X(i, 2 * j - 1);
            }
        for (int i = 0; i < m; ++i) X(i, n - 1) = -RT2 * W(i, (n + 1) / 2);
    }
    for (int i = 0; i < m; ++i) X(i, n) = 0.0;
#undef X
#undef W
}
