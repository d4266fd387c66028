/*
 * ibdwt_oracle.c -- CPU restatement of the gpuLucas IBDWT Lucas-Lehmer iteration.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, smoke()
 * and the CPU-baseline leg of bench.py use it as the checker.  The product
 * library never links, loads or calls it.
 *
 * It follows the reference algorithm step by step (file:line into the reference
 * project gpuLucas):
 *   - word sizes      gpuLucas.cu:688-694 (computeBitsPerWord), restated with exact
 *                     int64 arithmetic; bitsPerWord8 flags gpuLucas.cu:700-714
 *   - weights         gpuLucas.cu:673-686 (computeWeightVectors, QD dd_real), restated
 *                     with an own double-double type (Dekker/Knuth two-sum/two-product)
 *   - S0 = 4          gpuLucas.cu:718-726 (loadValue4ToFFTarray)
 *   - weighted load   gpuLucas.cu:730-766 (loadIntToDoubleIBDWT): d = A*(digit + hi[j-1])
 *   - real FFT square gpuLucas.cu:647-665, 858-877 (cuFFT D2Z, ComplexPointwiseSqr, Z2D);
 *                     here an own mixed-radix Stockham FFT of N/2 complex points with
 *                     the even/odd real-signal split, no cuFFT
 *   - unweight/-2     gpuLucas.cu:774-805 (invDWTproductMinus2): x = d*Ainv, x -= 2 at
 *                     word 0, round half-even to int64, err = |x - rint(x)|
 *   - dicing          IrrBaseBalanced.cu:52-110 (llintToIrrBal<n>)
 *   - carry depth n   gpuLucas.cu:323-343 (setSliceAndDice), table extended to ratio 21
 *   - final carry     IrrBaseBalanced.cu:117-125 (addPseudoBalanced),
 *                     IrrBaseBalanced.cu:133-169 (rebalanceIrrIntSEQGPU)
 *   - residue         gpuLucas.cu:1288-1352 (print_residue), zero test gpuLucas.cu:1506-1512
 *
 * Build: -O2 -ffp-contract=off (so that double-double and all host arithmetic is the
 * same on x86_64 and aarch64), optionally -fopenmp.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------- */
/* double-double arithmetic (Dekker 1971, Knuth TAOCP 4.2.2; same algorithms  */
/* QD's dd_real implements).                                                  */
/* ------------------------------------------------------------------------- */
typedef struct { double hi, lo; } dd_t;

static dd_t dd_quick_two_sum(double a, double b) {
    double s = a + b;
    dd_t r = { s, b - (s - a) };
    return r;
}
static dd_t dd_two_sum(double a, double b) {
    double s = a + b;
    double bb = s - a;
    dd_t r = { s, (a - (s - bb)) + (b - bb) };
    return r;
}
static dd_t dd_two_prod(double a, double b) {
    double p = a * b;
    dd_t r = { p, fma(a, b, -p) };
    return r;
}
static dd_t dd_from(double a) { dd_t r = { a, 0.0 }; return r; }
static dd_t dd_add(dd_t a, dd_t b) {
    dd_t s = dd_two_sum(a.hi, b.hi);
    dd_t t = dd_two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = dd_quick_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return dd_quick_two_sum(s.hi, s.lo);
}
static dd_t dd_neg(dd_t a) { dd_t r = { -a.hi, -a.lo }; return r; }
static dd_t dd_sub(dd_t a, dd_t b) { return dd_add(a, dd_neg(b)); }
static dd_t dd_mul(dd_t a, dd_t b) {
    dd_t p = dd_two_prod(a.hi, b.hi);
    p.lo += a.hi * b.lo;
    p.lo += a.lo * b.hi;
    return dd_quick_two_sum(p.hi, p.lo);
}
static dd_t dd_mul_d(dd_t a, double b) {
    dd_t p = dd_two_prod(a.hi, b);
    p.lo += a.lo * b;
    return dd_quick_two_sum(p.hi, p.lo);
}
static dd_t dd_div(dd_t a, dd_t b) {
    double q1 = a.hi / b.hi;
    dd_t r = dd_sub(a, dd_mul_d(b, q1));
    double q2 = r.hi / b.hi;
    r = dd_sub(r, dd_mul_d(b, q2));
    double q3 = r.hi / b.hi;
    dd_t q = dd_quick_two_sum(q1, q2);
    return dd_add(q, dd_from(q3));
}
/* exactly representable integers up to 2^53 */
static dd_t dd_from_i64(int64_t v) { return dd_from((double)v); }
/* round a double-double to the nearest double */
static double dd_to_double(dd_t a) { return a.hi + a.lo; }

/* ln 2 and pi/4 to double-double precision (values of the mathematical constants) */
static const dd_t DD_LN2 = { 0x1.62e42fefa39efp-1, 0x1.abc9e3b39803fp-56 };
static const dd_t DD_PI_4 = { 0x1.921fb54442d18p-1, 0x1.1a62633145c07p-55 };

/* exp(x) for 0 <= x < 1 in double-double: x/2^10, Taylor series for expm1, then
 * ten doublings e' = 2e + e^2 on expm1 (keeps relative precision), result 1 + e. */
static dd_t dd_exp_small(dd_t x) {
    dd_t y = { ldexp(x.hi, -10), ldexp(x.lo, -10) };
    dd_t term = y, sum = y;
    for (int k = 2; k <= 14; ++k) {
        term = dd_div(dd_mul(term, y), dd_from((double)k));
        sum = dd_add(sum, term);
    }
    for (int i = 0; i < 10; ++i) {
        dd_t two_s = { 2.0 * sum.hi, 2.0 * sum.lo };
        sum = dd_add(two_s, dd_mul(sum, sum));
    }
    return dd_add(dd_from(1.0), sum);
}

/* sin and cos of (pi/4) * num / den, 0 <= num <= den, by Taylor series in dd. */
static void dd_sincos_octant(int64_t num, int64_t den, dd_t* s, dd_t* c) {
    dd_t x = dd_mul(DD_PI_4, dd_div(dd_from_i64(num), dd_from_i64(den)));
    dd_t x2 = dd_mul(x, x);
    dd_t st = x, ss = x;          /* sin: x - x^3/3! + ... */
    dd_t ct = dd_from(1.0), cs = dd_from(1.0);
    for (int k = 1; k <= 14; ++k) {
        st = dd_neg(dd_div(dd_mul(st, x2), dd_from((double)((2 * k) * (2 * k + 1)))));
        ss = dd_add(ss, st);
        ct = dd_neg(dd_div(dd_mul(ct, x2), dd_from((double)((2 * k - 1) * (2 * k)))));
        cs = dd_add(cs, ct);
    }
    *s = ss;
    *c = cs;
}

/* exp(-2 pi i t / L) rounded to double, by exact octant reduction of t/L. */
static void twiddle(int64_t t, int64_t L, double* re, double* im) {
    t %= L;
    if (t < 0) t += L;
    int64_t u = 8 * t;
    int64_t o = u / L;          /* octant 0..7 */
    int64_t r = u - o * L;      /* angle inside the octant = (pi/4) r/L */
    dd_t s, c;
    if (o & 1) dd_sincos_octant(L - r, L, &s, &c); /* angle (pi/4)(1 - r/L) */
    else dd_sincos_octant(r, L, &s, &c);
    /* cos/sin of the full angle theta = o*pi/4 + phi */
    double cs = dd_to_double(c), sn = dd_to_double(s);
    double C, S;
    switch (o) {
    case 0: C = cs; S = sn; break;            /* phi */
    case 1: C = sn; S = cs; break;            /* pi/2 - psi, psi = pi/4 - phi */
    case 2: C = -sn; S = cs; break;           /* pi/2 + phi */
    case 3: C = -cs; S = sn; break;           /* pi - psi */
    case 4: C = -cs; S = -sn; break;          /* pi + phi */
    case 5: C = -sn; S = -cs; break;          /* 3pi/2 - psi */
    case 6: C = sn; S = -cs; break;           /* 3pi/2 + phi */
    default: C = cs; S = -sn; break;          /* 2pi - psi */
    }
    *re = C;
    *im = -S;
}

/* ------------------------------------------------------------------------- */
/* Parameters: word sizes, flags, weights                                     */
/* ------------------------------------------------------------------------- */

/* setSliceAndDice, gpuLucas.cu:323-343: carry depth from ratio p/N.  The reference
 * exits for ratio >= 21; the table here accepts 21 (three 21-bit slices cover 63 bits,
 * more than the ~49-bit products at N=2048) and returns -1 for ratio >= 22. */
int orc_slice_depth(int p, int N) {
    int ratio = p / N;
    if (ratio >= 22) return -1;
    if (ratio >= 18) return 2;
    if (ratio >= 16) return 3;
    if (ratio >= 14) return 4;
    if (ratio >= 12) return 5;
    return 6;
}

/* ceil(p*j/N) with exact integer arithmetic */
static int64_t ceil_pj_n(int64_t p, int64_t j, int64_t N) {
    int64_t num = p * j;
    return (num + N - 1) / N;
}

/* computeBitsPerWord, gpuLucas.cu:688-694, exact: bits[j] = ceil(p(j+1)/N) - ceil(pj/N).
 * computeBitsPerWordVectors, gpuLucas.cu:700-714: bpw8[j] bit i = word (j-i) mod N is HI. */
void orc_bits(int p, int N, int32_t* bits, uint8_t* bpw8) {
    int LO = p / N;
    for (int j = 0; j < N; ++j)
        bits[j] = (int32_t)(ceil_pj_n(p, j + 1, N) - ceil_pj_n(p, j, N));
    if (bpw8) {
        for (int j = 0; j < N; ++j) {
            uint8_t v = 0;
            for (int b = 0; b < 8; ++b) {
                int k = j - b;
                while (k < 0) k += N;
                v |= (uint8_t)((bits[k] == LO ? 0 : 1) << b);
            }
            bpw8[j] = v;
        }
    }
}

/* The reference's own double-precision formula (gpuLucas.cu:690-692), kept only so a
 * test can show it agrees with the exact integer one on the configured sizes. */
void orc_bits_refdouble(int p, int N, int32_t* bits) {
    double PoverN = p / (double)N;
    for (int j = 1; j <= N; ++j)
        bits[j - 1] = (int32_t)(ceil(PoverN * j) - ceil(PoverN * (j - 1)));
}

/* computeWeightVectors, gpuLucas.cu:673-686.  A[j] = 2^(ceil(jp/N) - jp/N),
 * Ainv[j] = (1/A[j])/N, both in double-double, rounded to double.  The exponent
 * ceil(jp/N) - jp/N equals r/N with the integer r = (-j p) mod N, formed exactly. */
void orc_weights(int p, int N, double* A, double* Ainv) {
    dd_t dN = dd_from((double)N);
    for (int j = 0; j < N; ++j) {
        int64_t r = (int64_t)(ceil_pj_n(p, j, N) * N - (int64_t)p * j);
        dd_t e = dd_exp_small(dd_mul(dd_div(dd_from_i64(r), dN), DD_LN2));
        dd_t inv = dd_div(dd_div(dd_from(1.0), e), dN);
        A[j] = dd_to_double(e);
        Ainv[j] = dd_to_double(inv);
    }
}

/* ------------------------------------------------------------------------- */
/* Mixed-radix Stockham complex FFT (own; no FFTW/cuFFT)                      */
/* ------------------------------------------------------------------------- */
typedef struct { double re, im; } cplx;

typedef struct {
    int M;
    int nstages;
    int radix[40];
    cplx* tw;      /* exp(-2 pi i t / M), t in [0, M) */
} fft_plan;

static int fft_plan_init(fft_plan* f, int M) {
    f->M = M;
    f->nstages = 0;
    int m = M;
    /* radix 4 first, then 2, 3, 5, 7 */
    while (m % 4 == 0) { f->radix[f->nstages++] = 4; m /= 4; }
    while (m % 2 == 0) { f->radix[f->nstages++] = 2; m /= 2; }
    while (m % 3 == 0) { f->radix[f->nstages++] = 3; m /= 3; }
    while (m % 5 == 0) { f->radix[f->nstages++] = 5; m /= 5; }
    while (m % 7 == 0) { f->radix[f->nstages++] = 7; m /= 7; }
    if (m != 1) return -1;
    f->tw = (cplx*)malloc(sizeof(cplx) * (size_t)M);
    if (!f->tw) return -1;
#pragma omp parallel for schedule(static) if (M >= 4096)
    for (int t = 0; t < M; ++t) twiddle(t, M, &f->tw[t].re, &f->tw[t].im);
    return 0;
}
static void fft_plan_free(fft_plan* f) { free(f->tw); f->tw = NULL; }

static inline cplx cmul(cplx a, cplx b) {
    cplx r = { a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re };
    return r;
}
static inline cplx cconj(cplx a) { cplx r = { a.re, -a.im }; return r; }

/* One Stockham stage (Bainville's formulation): butterfly j reads x[j + q*M/R],
 * twiddles by w_{Ns R}^{(j mod Ns) q}, does a radix-R DFT and writes
 * y[(j/Ns)*Ns*R + (j mod Ns) + q*Ns].  sign=-1 forward, +1 inverse (unnormalized). */
static void fft_stage(const fft_plan* f, int R, int Ns, const cplx* x, cplx* y, int sign) {
    const int M = f->M, MR = M / R;
    const int twstep = M / (Ns * R);
#pragma omp parallel for schedule(static) if (M >= 32768)
    for (int j = 0; j < MR; ++j) {
        cplx a[8], b[8];
        int k = j % Ns;
        for (int q = 0; q < R; ++q) {
            cplx v = x[j + q * MR];
            if (q && k) {
                cplx w = f->tw[(int64_t)k * q * twstep];
                if (sign > 0) w = cconj(w);
                v = cmul(v, w);
            }
            a[q] = v;
        }
        if (R == 2) {
            b[0].re = a[0].re + a[1].re; b[0].im = a[0].im + a[1].im;
            b[1].re = a[0].re - a[1].re; b[1].im = a[0].im - a[1].im;
        } else if (R == 4) {
            cplx s02 = { a[0].re + a[2].re, a[0].im + a[2].im };
            cplx d02 = { a[0].re - a[2].re, a[0].im - a[2].im };
            cplx s13 = { a[1].re + a[3].re, a[1].im + a[3].im };
            cplx d13 = { a[1].re - a[3].re, a[1].im - a[3].im };
            /* multiply d13 by -i (forward) or +i (inverse) */
            cplx rd13 = sign < 0 ? (cplx){ d13.im, -d13.re } : (cplx){ -d13.im, d13.re };
            b[0].re = s02.re + s13.re; b[0].im = s02.im + s13.im;
            b[2].re = s02.re - s13.re; b[2].im = s02.im - s13.im;
            b[1].re = d02.re + rd13.re; b[1].im = d02.im + rd13.im;
            b[3].re = d02.re - rd13.re; b[3].im = d02.im - rd13.im;
        } else {
            /* generic O(R^2) DFT with table roots exp(-+2 pi i s/R) */
            int rstep = M / R;
            for (int s = 0; s < R; ++s) {
                cplx acc = a[0];
                for (int q = 1; q < R; ++q) {
                    cplx w = f->tw[(int64_t)((q * s) % R) * rstep];
                    if (sign > 0) w = cconj(w);
                    cplx t = cmul(a[q], w);
                    acc.re += t.re; acc.im += t.im;
                }
                b[s] = acc;
            }
        }
        int base = (j / Ns) * Ns * R + k;
        for (int q = 0; q < R; ++q) y[base + q * Ns] = b[q];
    }
}

/* transform x in place (tmp: scratch of M). */
static void fft_run(const fft_plan* f, cplx* x, cplx* tmp, int sign) {
    cplx* src = x;
    cplx* dst = tmp;
    int Ns = 1;
    for (int s = 0; s < f->nstages; ++s) {
        fft_stage(f, f->radix[s], Ns, src, dst, sign);
        Ns *= f->radix[s];
        cplx* t = src; src = dst; dst = t;
    }
    if (src != x) memcpy(x, src, sizeof(cplx) * (size_t)f->M);
}

/* ------------------------------------------------------------------------- */
/* LL iteration context                                                       */
/* ------------------------------------------------------------------------- */
typedef struct {
    int p, N, M, LO, HI, n;
    int32_t* bits;
    uint8_t* bpw8;
    double* A;
    double* Ainv;      /* reference convention (1/A)/N */
    double* d_signal;  /* weighted FFT input, the loop-carried state (gpuLucas.cu:250) */
    int64_t* ll;       /* rounded products of the last iteration */
    int32_t* digit;    /* i_signal */
    int8_t* hi;        /* i_hiBitArr */
    cplx* z;
    cplx* tmp;
    fft_plan fft;
    int64_t iters_done;
    double maxerr;
    int64_t max_abs_ll;
    int overflow;      /* a product had bits beyond what its n+1 slices cover */
} orc_ctx;

void orc_destroy(orc_ctx* c);

orc_ctx* orc_create(int p, int N, int nthreads) {
    if (N <= 0 || (N & 1) || p <= 2 || (int64_t)N > (int64_t)p) return NULL;
    int n = orc_slice_depth(p, N);
    if (n < 0) return NULL;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    orc_ctx* c = (orc_ctx*)calloc(1, sizeof(orc_ctx));
    if (!c) return NULL;
    c->p = p; c->N = N; c->M = N / 2; c->LO = p / N; c->HI = c->LO + 1; c->n = n;
    c->bits = (int32_t*)malloc(sizeof(int32_t) * N);
    c->bpw8 = (uint8_t*)malloc(N);
    c->A = (double*)malloc(sizeof(double) * N);
    c->Ainv = (double*)malloc(sizeof(double) * N);
    c->d_signal = (double*)malloc(sizeof(double) * N);
    c->ll = (int64_t*)malloc(sizeof(int64_t) * N);
    c->digit = (int32_t*)malloc(sizeof(int32_t) * N);
    c->hi = (int8_t*)malloc(N);
    c->z = (cplx*)malloc(sizeof(cplx) * c->M);
    c->tmp = (cplx*)malloc(sizeof(cplx) * c->M);
    if (!c->bits || !c->bpw8 || !c->A || !c->Ainv || !c->d_signal || !c->ll || !c->digit ||
        !c->hi || !c->z || !c->tmp || fft_plan_init(&c->fft, c->M) != 0) {
        orc_destroy(c);
        return NULL;
    }
    orc_bits(p, N, c->bits, c->bpw8);
    orc_weights(p, N, c->A, c->Ainv);
    return c;
}

void orc_destroy(orc_ctx* c) {
    if (!c) return;
    free(c->bits); free(c->bpw8); free(c->A); free(c->Ainv); free(c->d_signal);
    free(c->ll); free(c->digit); free(c->hi); free(c->z); free(c->tmp);
    fft_plan_free(&c->fft);
    free(c);
}

/* loadValue4ToFFTarray, gpuLucas.cu:718-726: S0 = 4 (A[0] = 1). */
void orc_reset(orc_ctx* c) {
    memset(c->d_signal, 0, sizeof(double) * c->N);
    c->d_signal[0] = 4.0;
    memset(c->ll, 0, sizeof(int64_t) * c->N);
    c->ll[0] = 4;
    memset(c->digit, 0, sizeof(int32_t) * c->N);
    c->digit[0] = 4;
    memset(c->hi, 0, c->N);
    c->iters_done = 0;
    c->maxerr = 0.0;
    c->max_abs_ll = 0;
    c->overflow = 0;
}

/* llintToIrrBal<n>, IrrBaseBalanced.cu:52-110, for every word: sign-magnitude slices
 * of the n+1 products ending at word j summed into one value, split into a balanced
 * digit and an int8 carry.  Also flags products with bits beyond the slices. */
static void dice(int N, int LO, int n, const int64_t* ll, const uint8_t* bpw8,
                 int32_t* digit, int8_t* hi) {
#pragma omp parallel for schedule(static) if (N >= 65536)
    for (int j = 0; j < N; ++j) {
        uint8_t f = bpw8[j];
        int isHi = f & 1;
        int BITS = LO + isHi;
        int64_t base = (int64_t)1 << BITS;
        int64_t mask = base - 1;
        int64_t half = base >> 1;
        int64_t v = ll[j];
        int64_t sgn = v < 0 ? -1 : 1;
        int64_t sum = sgn * ((v * sgn) & mask);
        int shift = 0;
        for (int i = 1; i <= n; ++i) {
            int k = j - i;
            if (k < 0) k += N;
            shift += LO + ((f >> i) & 1);
            if (shift >= 63) break;     /* PTX clamps such shifts: the slice is 0 */
            int64_t w = ll[k];
            int64_t s = w < 0 ? -1 : 1;
            sum += s * (((w * s) >> shift) & mask);
        }
        int64_t h = 0;
        if (sum < -half) h = -((-sum + half) >> BITS);
        else if (sum >= half) h = (sum + half) >> BITS;
        digit[j] = (int32_t)(sum - h * base);
        hi[j] = (int8_t)h;
    }
}

void orc_dice(int p, int N, const int64_t* ll, int32_t* digit, int8_t* hi) {
    uint8_t* bpw8 = (uint8_t*)malloc(N);
    int32_t* bits = (int32_t*)malloc(sizeof(int32_t) * N);
    orc_bits(p, N, bits, bpw8);
    dice(N, p / N, orc_slice_depth(p, N), ll, bpw8, digit, hi);
    free(bpw8);
    free(bits);
}

/* loadIntToDoubleIBDWT, gpuLucas.cu:730-766: d[j] = A[j] * (digit[j] + hi[j-1 mod N]). */
static void load_weighted(orc_ctx* c) {
    const int N = c->N;
#pragma omp parallel for schedule(static) if (N >= 65536)
    for (int j = 0; j < N; ++j) {
        int v = c->digit[j] + c->hi[j == 0 ? N - 1 : j - 1];
        c->d_signal[j] = c->A[j] * (double)v;
    }
}

/* One LL iteration (mersenneIter, gpuLucas.cu:845-942) from d_signal.  The real
 * length-N transform is an M=N/2 complex FFT of u[m] = x[2m] + i x[2m+1]; with
 * Et = U[k] + conj(U[M-k]) = 2E[k] and Ot = -i (U[k] - conj(U[M-k])) = 2O[k] (E, O the
 * DFTs of the even/odd words) the spectrum of the squared signal packs into
 * Vt[k] = Et^2 + w_M^k Ot^2 + 2i Et Ot = 4 DFT_M(z_even + i z_odd), so the
 * unnormalized inverse returns 2N z: the reference's (1/A)/N then needs an extra 1/2. */
static void orc_iter_one(orc_ctx* c) {
    const int N = c->N, M = c->M;
    cplx* z = c->z;
#pragma omp parallel for schedule(static) if (M >= 32768)
    for (int m = 0; m < M; ++m) {
        z[m].re = c->d_signal[2 * m];
        z[m].im = c->d_signal[2 * m + 1];
    }
    fft_run(&c->fft, z, c->tmp, -1);
    cplx* V = c->tmp;
#pragma omp parallel for schedule(static) if (M >= 32768)
    for (int k = 0; k < M; ++k) {
        cplx u = z[k], w = z[k == 0 ? 0 : M - k];
        cplx e = { u.re + w.re, u.im - w.im };
        cplx d = { u.re - w.re, u.im + w.im };
        cplx o = { d.im, -d.re };                /* -i * d */
        cplx e2 = cmul(e, e), o2 = cmul(o, o), eo = cmul(e, o);
        cplx t = cmul(o2, c->fft.tw[k]);
        V[k].re = e2.re + t.re - 2.0 * eo.im;
        V[k].im = e2.im + t.im + 2.0 * eo.re;
    }
    memcpy(z, V, sizeof(cplx) * (size_t)M);
    fft_run(&c->fft, z, c->tmp, +1);
    double maxerr = c->maxerr;
    int64_t maxll = c->max_abs_ll;
#pragma omp parallel for schedule(static) reduction(max : maxerr, maxll) if (N >= 65536)
    for (int j = 0; j < N; ++j) {
        double zz = (j & 1) ? z[j >> 1].im : z[j >> 1].re;
        double x = zz * (c->Ainv[j] * 0.5);
        if (j == 0) x -= 2.0;
        double r = nearbyint(x);                /* round half-even, as __double2ll_rn */
        double e = fabs(x - r);
        if (e > maxerr) maxerr = e;
        int64_t v = (int64_t)r;
        c->ll[j] = v;
        int64_t av = v < 0 ? -v : v;
        if (av > maxll) maxll = av;
    }
    c->maxerr = maxerr;
    c->max_abs_ll = maxll;
    /* overflow check: product j spreads over words j..j+n; the bits it can place there
     * are bits[j] + ... + bits[j+n] */
    int ovf = 0;
#pragma omp parallel for schedule(static) reduction(| : ovf) if (N >= 65536)
    for (int j = 0; j < N; ++j) {
        int tot = 0;
        for (int i = 0; i <= c->n; ++i) tot += c->bits[(j + i) % N];
        int64_t v = c->ll[j];
        uint64_t av = (uint64_t)(v < 0 ? -v : v);
        if (tot < 63 && (av >> tot) != 0) ovf |= 1;
    }
    c->overflow |= ovf;
    dice(N, c->LO, c->n, c->ll, c->bpw8, c->digit, c->hi);
    load_weighted(c);
    c->iters_done++;
}

void orc_iterate(orc_ctx* c, int64_t iters) {
    for (int64_t i = 0; i < iters; ++i) orc_iter_one(c);
}

double orc_maxerr(const orc_ctx* c) { return c->maxerr; }
int64_t orc_max_abs_product(const orc_ctx* c) { return c->max_abs_ll; }
int orc_overflow(const orc_ctx* c) { return c->overflow; }
int64_t orc_iters_done(const orc_ctx* c) { return c->iters_done; }
void orc_get_ll(const orc_ctx* c, int64_t* out) { memcpy(out, c->ll, sizeof(int64_t) * c->N); }
void orc_get_state(const orc_ctx* c, int32_t* digit, int8_t* hi) {
    memcpy(digit, c->digit, sizeof(int32_t) * c->N);
    memcpy(hi, c->hi, c->N);
}
void orc_get_signal(const orc_ctx* c, double* out) { memcpy(out, c->d_signal, sizeof(double) * c->N); }
void orc_get_tables(const orc_ctx* c, int32_t* bits, uint8_t* bpw8, double* A, double* Ainv) {
    if (bits) memcpy(bits, c->bits, sizeof(int32_t) * c->N);
    if (bpw8) memcpy(bpw8, c->bpw8, c->N);
    if (A) memcpy(A, c->A, sizeof(double) * c->N);
    if (Ainv) memcpy(Ainv, c->Ainv, sizeof(double) * c->N);
}

/* Set the carry-save state directly (digits + carries), then reload the signal. */
void orc_set_state(orc_ctx* c, const int32_t* digit, const int8_t* hi, int64_t iters_done) {
    memcpy(c->digit, digit, sizeof(int32_t) * c->N);
    memcpy(c->hi, hi, c->N);
    load_weighted(c);
    c->iters_done = iters_done;
}

/* ------------------------------------------------------------------------- */
/* Final normalisation and residue                                            */
/* ------------------------------------------------------------------------- */

/* addPseudoBalanced (IrrBaseBalanced.cu:117-125) then rebalanceIrrIntSEQGPU
 * (IrrBaseBalanced.cu:133-169): one sequential balanced carry pass, wrap into word 0. */
void orc_rebalance(int p, int N, const int32_t* digit, const int8_t* hi, int32_t* out) {
    int LO = p / N;
    int32_t* bits = (int32_t*)malloc(sizeof(int32_t) * N);
    orc_bits(p, N, bits, NULL);
    for (int j = 0; j < N; ++j) out[j] = digit[j] + hi[j == 0 ? N - 1 : j - 1];
    int carry = 0;
    for (int i = 0; i < N; ++i) {
        int isHi = bits[i] != LO;
        int base = 1 << (LO + isHi);
        int half = base >> 1;
        int total = out[i] + carry;
        if (total >= half) { out[i] = total - base; carry = 1; }
        else if (total < -half) { out[i] = total + base; carry = -1; }
        else { out[i] = total; carry = 0; }
    }
    if (carry != 0) out[0] += carry;
    free(bits);
}

/* print_residue, gpuLucas.cu:1288-1352: borrow-normalise the balanced digits to
 * non-negative ones (the HI/LO rule there is (b*j mod N) >= c with b = p mod N,
 * c = N - b, word 0 HI, word N-1 LO: the same as the bits table), then pack the low
 * 64 bits.  Modifies `digits`.  Returns the 64-bit residue. */
uint64_t orc_res64_normalize(int p, int N, int32_t* h) {
    int LO = p / N;
    int32_t* bits = (int32_t*)malloc(sizeof(int32_t) * N);
    orc_bits(p, N, bits, NULL);
    int sudden_death = 0;
    int64_t guard = 0;
    int j = 0;
    for (;;) {
        if (h[j] < 0) {
            h[(j + 1) % N] -= 1;
            h[j] += 1 << bits[j];
        } else if (sudden_death) {
            break;
        }
        if (++j == N) { sudden_death = 1; j = 0; }
        if (++guard > 4 * (int64_t)N + 16) break;   /* cannot happen for a valid state */
    }
    uint64_t res = 0;
    int bitpos = 0;
    for (int w = 0; w < N && bitpos < 64; ++w) {
        int k = bits[w];
        uint64_t word = (uint64_t)(uint32_t)h[w];
        for (int b = 0; b < k && bitpos < 64; ++b, ++bitpos)
            res |= ((word >> b) & 1u) << bitpos;
    }
    (void)LO;
    free(bits);
    return res;
}

/* Full residue of the current state: rebalance, the reference's zero test
 * (gpuLucas.cu:1506-1512: no digit > 0) and an exact one (the value is 0 mod M_p:
 * all normalised digits 0, or all equal to base-1, i.e. the value M_p itself). */
void orc_residue(const orc_ctx* c, int32_t* digits_out, uint64_t* res64, int* ref_zero, int* exact_zero) {
    const int N = c->N;
    int32_t* d = (int32_t*)malloc(sizeof(int32_t) * N);
    orc_rebalance(c->p, N, c->digit, c->hi, d);
    if (digits_out) memcpy(digits_out, d, sizeof(int32_t) * N);
    int any_pos = 0;
    for (int j = 0; j < N; ++j) if (d[j] > 0) { any_pos = 1; break; }
    *ref_zero = !any_pos;
    *res64 = orc_res64_normalize(c->p, N, d);
    int all0 = 1, allmax = 1;
    for (int j = 0; j < N; ++j) {
        if (d[j] != 0) all0 = 0;
        if (d[j] != (1 << c->bits[j]) - 1) allmax = 0;
    }
    *exact_zero = all0 || allmax;
    if (allmax) *res64 = 0;
    free(d);
}

int orc_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* Twiddle table exp(-2 pi i t / L) for tests of the double-double sin/cos. */
void orc_twiddles(int L, double* re, double* im) {
    for (int t = 0; t < L; ++t) twiddle(t, L, &re[t], &im[t]);
}
