/*
 * exact_oracle.c -- exact Lucas-Lehmer sequence S_{k+1} = S_k^2 - 2 mod 2^p - 1.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  Pure integer arithmetic, independent of any
 * floating point: squaring by a number-theoretic transform over the prime
 * P = 2^64 - 2^32 + 1, then the Mersenne reduction by shift-and-add.  It pins the
 * residues that the IBDWT implementations (the reference gpuLucas.cu mersenneTest,
 * gpuLucas.cu:1358-1551, restated in ibdwt_oracle.c, and the CUDA product) compute.
 *
 * Limbs are 16 bits; with L = ceil(p/16) limbs the convolution terms are below
 * L * 2^32 < 2^54 < P for p < 2^26 * 16, so one prime suffices and no CRT is needed.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;
static const uint64_t GP = 0xFFFFFFFF00000001ull; /* 2^64 - 2^32 + 1 */
static const uint64_t GEPS = 0xFFFFFFFFull;       /* 2^64 mod P = 2^32 - 1 */

/* x mod P for x < 2^128, using 2^64 = 2^32 - 1 and 2^96 = -1 (mod P). */
static inline uint64_t g_reduce(u128 x) {
    uint64_t lo = (uint64_t)x, hi = (uint64_t)(x >> 64);
    uint64_t hh = hi >> 32, hl = hi & 0xFFFFFFFFull;
    uint64_t t0 = lo - hh;
    if (lo < hh) t0 -= GEPS;          /* borrow of 2^64 == EPS */
    uint64_t t1 = hl * GEPS;
    uint64_t r = t0 + t1;
    if (r < t1) r += GEPS;            /* carry of 2^64 == EPS */
    if (r >= GP) r -= GP;
    return r;
}
static inline uint64_t g_mul(uint64_t a, uint64_t b) { return g_reduce((u128)a * b); }
static inline uint64_t g_add(uint64_t a, uint64_t b) {
    uint64_t r = a + b;
    if (r < a || r >= GP) r -= GP;
    return r;
}
static inline uint64_t g_sub(uint64_t a, uint64_t b) {
    uint64_t r = a - b;
    if (a < b) r += GP;
    return r;
}
static uint64_t g_pow(uint64_t a, uint64_t e) {
    uint64_t r = 1;
    while (e) {
        if (e & 1) r = g_mul(r, a);
        a = g_mul(a, a);
        e >>= 1;
    }
    return r;
}

typedef struct {
    int p;
    int W;             /* 64-bit words holding p bits */
    int L;             /* 16-bit limbs */
    int logT;
    int64_t T;         /* transform length, power of two >= 2L */
    uint64_t* s;       /* current S_k, W words, canonical in [0, 2^p - 1) */
    uint64_t* a;       /* transform buffer, T */
    uint64_t* tw;      /* forward roots w^k, k < T/2 */
    uint64_t* twi;     /* inverse roots */
    uint32_t* rev;     /* bit reversal */
    uint64_t* sq;      /* 2W+2 words: S^2 */
    int64_t k;
} ex_ctx;

void ex_destroy(ex_ctx* c) {
    if (!c) return;
    free(c->s); free(c->a); free(c->tw); free(c->twi); free(c->rev); free(c->sq);
    free(c);
}

ex_ctx* ex_create(int p, int nthreads) {
    if (p < 3) return NULL;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    ex_ctx* c = (ex_ctx*)calloc(1, sizeof(ex_ctx));
    if (!c) return NULL;
    c->p = p;
    c->W = (p + 63) / 64;
    c->L = (p + 15) / 16;
    c->logT = 1;
    while (((int64_t)1 << c->logT) < 2 * (int64_t)c->L) c->logT++;
    c->T = (int64_t)1 << c->logT;
    c->s = (uint64_t*)calloc(c->W, 8);
    c->a = (uint64_t*)malloc(8 * c->T);
    c->tw = (uint64_t*)malloc(8 * (c->T / 2));
    c->twi = (uint64_t*)malloc(8 * (c->T / 2));
    c->rev = (uint32_t*)malloc(4 * c->T);
    c->sq = (uint64_t*)calloc(2 * c->W + 4, 8);
    if (!c->s || !c->a || !c->tw || !c->twi || !c->rev || !c->sq) { ex_destroy(c); return NULL; }
    /* 7 generates the multiplicative group of P; w = 7^((P-1)/T) has order T */
    uint64_t w = g_pow(7, (GP - 1) >> c->logT);
    uint64_t wi = g_pow(w, GP - 2);
    c->tw[0] = 1; c->twi[0] = 1;
    for (int64_t i = 1; i < c->T / 2; ++i) {
        c->tw[i] = g_mul(c->tw[i - 1], w);
        c->twi[i] = g_mul(c->twi[i - 1], wi);
    }
    for (int64_t i = 0; i < c->T; ++i) {
        uint32_t r = 0, v = (uint32_t)i;
        for (int b = 0; b < c->logT; ++b) { r = (r << 1) | (v & 1); v >>= 1; }
        c->rev[i] = r;
    }
    c->s[0] = 4;
    c->k = 0;
    return c;
}

/* iterative radix-2 decimation-in-time NTT, bit-reversed input order */
static void ntt(ex_ctx* c, const uint64_t* roots) {
    uint64_t* a = c->a;
    const int64_t T = c->T;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < T; ++i) {
        int64_t j = c->rev[i];
        if (i < j) { uint64_t t = a[i]; a[i] = a[j]; a[j] = t; }
    }
    for (int64_t len = 2; len <= T; len <<= 1) {
        int64_t half = len >> 1, step = T / len;
#pragma omp parallel for schedule(static)
        for (int64_t b = 0; b < T / 2; ++b) {
            int64_t grp = b / half, pos = b % half;
            int64_t i = grp * len + pos;
            uint64_t u = a[i], v = g_mul(a[i + half], roots[pos * step]);
            a[i] = g_add(u, v);
            a[i + half] = g_sub(u, v);
        }
    }
}

static int get_bit_range16(const uint64_t* s, int W, int64_t limb) {
    int64_t bit = limb * 16;
    int64_t w = bit >> 6;
    int sh = (int)(bit & 63);
    if (w >= W) return 0;
    return (int)((s[w] >> sh) & 0xFFFF);
}

/* S <- S^2 - 2 mod 2^p - 1 */
static void ex_step(ex_ctx* c) {
    const int p = c->p, W = c->W, L = c->L;
    const int64_t T = c->T;
    uint64_t* a = c->a;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < T; ++i) a[i] = i < L ? (uint64_t)get_bit_range16(c->s, W, i) : 0;
    ntt(c, c->tw);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < T; ++i) a[i] = g_mul(a[i], a[i]);
    ntt(c, c->twi);
    uint64_t tinv = g_pow((uint64_t)T, GP - 2);
    /* carry the exact convolution terms into 64-bit words of S^2 */
    uint64_t* sq = c->sq;
    const int SW = 2 * W + 4;
    memset(sq, 0, 8 * SW);
    u128 carry = 0;
    int64_t nlimbs = 2 * (int64_t)L + 8;
    for (int64_t i = 0; i < nlimbs; ++i) {
        if (i < T) carry += (u128)g_mul(a[i], tinv);
        uint64_t limb = (uint64_t)(carry & 0xFFFF);
        carry >>= 16;
        int64_t bit = i * 16;
        if ((bit >> 6) < SW) sq[bit >> 6] |= limb << (bit & 63);
    }
    /* reduce: S^2 = hi * 2^p + lo == hi + lo (mod 2^p - 1) */
    uint64_t* lo = (uint64_t*)calloc(W + 1, 8);
    uint64_t* hi = (uint64_t*)calloc(W + 1, 8);
    for (int i = 0; i < W; ++i) lo[i] = sq[i];
    if (p % 64) lo[W - 1] &= (((uint64_t)1) << (p % 64)) - 1;
    int wsh = p / 64, bsh = p % 64;
    for (int i = 0; i < W + 1; ++i) {
        int64_t src = i + wsh;
        uint64_t v = src < SW ? sq[src] >> bsh : 0;
        if (bsh && src + 1 < SW) v |= sq[src + 1] << (64 - bsh);
        hi[i] = v;
    }
    /* r = lo + hi (fits p+1 bits) */
    u128 cy = 0;
    for (int i = 0; i < W + 1; ++i) {
        cy += (u128)lo[i] + hi[i];
        lo[i] = (uint64_t)cy;
        cy >>= 64;
    }
    /* fold bit p and above once more */
    for (int rep = 0; rep < 2; ++rep) {
        uint64_t over;
        if (bsh == 0) { over = lo[W]; lo[W] = 0; }
        else { over = (lo[W - 1] >> bsh) | (lo[W] << (64 - bsh)); lo[W - 1] &= (((uint64_t)1) << bsh) - 1; lo[W] = 0; }
        cy = over;
        for (int i = 0; i < W + 1 && cy; ++i) {
            cy += lo[i];
            lo[i] = (uint64_t)cy;
            cy >>= 64;
        }
    }
    /* canonical: if r == 2^p - 1 then r = 0 */
    int allones = 1;
    for (int i = 0; i < W; ++i) {
        uint64_t m = (i == W - 1 && bsh) ? ((((uint64_t)1) << bsh) - 1) : ~(uint64_t)0;
        if (lo[i] != m) { allones = 0; break; }
    }
    if (allones) memset(lo, 0, 8 * (W + 1));
    /* subtract 2 mod 2^p - 1 */
    int small = 1;
    for (int i = 1; i < W; ++i) if (lo[i]) { small = 0; break; }
    if (small && lo[0] < 2) {
        /* r - 2 + (2^p - 1) */
        uint64_t r0 = lo[0];
        for (int i = 0; i < W; ++i) lo[i] = (i == W - 1 && bsh) ? ((((uint64_t)1) << bsh) - 1) : ~(uint64_t)0;
        lo[0] = lo[0] - (2 - r0);
    } else {
        uint64_t b = 2;
        for (int i = 0; i < W && b; ++i) {
            uint64_t v = lo[i];
            lo[i] = v - b;
            b = v < b ? 1 : 0;
        }
    }
    memcpy(c->s, lo, 8 * W);
    free(lo);
    free(hi);
    c->k++;
}

void ex_iterate(ex_ctx* c, int64_t iters) {
    for (int64_t i = 0; i < iters; ++i) ex_step(c);
}
int64_t ex_iters_done(const ex_ctx* c) { return c->k; }
uint64_t ex_res64(const ex_ctx* c) { return c->s[0]; }
int ex_is_zero(const ex_ctx* c) {
    for (int i = 0; i < c->W; ++i) if (c->s[i]) return 0;
    return 1;
}
int ex_words(const ex_ctx* c) { return c->W; }
void ex_get(const ex_ctx* c, uint64_t* out) { memcpy(out, c->s, 8 * c->W); }
void ex_set(ex_ctx* c, const uint64_t* in, int64_t k) { memcpy(c->s, in, 8 * c->W); c->k = k; }
