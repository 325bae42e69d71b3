/*
 * ORACLE -- test infrastructure only.  Nothing in the product links this file;
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it,
 * and only as the checker.
 *
 * CPU restatement of monofonIC's NGenIC white-noise plugin
 * (src/plugins/random_ngenic.cc:39-154) and of the generator it draws from,
 * GSL's `gsl_rng_ranlxd1` (GSL is a third-party dependency absent from the
 * reference tree; version unpinned: CMakeLists.txt:132, CI installs Debian's
 * libgsl-dev, bitbucket-pipelines.yml:26).
 *
 * The generator is restated from M. Luescher's published RANLUX algorithm
 * (Comput. Phys. Commun. 79 (1994) 100; double-precision "ranlxd" variant):
 *   - a subtract-with-borrow sequence on 48-bit words,
 *       y[n] = y[n-5] - y[n-12] - c[n-1]  (mod 2^48),  c[n] = borrow of that step;
 *   - luxury level 1 ("ranlxd1"): per block 202 words are generated and the
 *     last 12 of them are delivered, in generation order, as y / 2^48;
 *   - seeding: a 31-bit shift register initialised from the low 31 bits of the
 *     seed; each of the 12 initial words is built from 48 successive
 *     complemented register bits, most significant first, the register
 *     advancing as b[i] <- b[i] xor b[i+18 mod 31]; seed 0 means seed 1.
 * All values are exact integers, so this is integer arithmetic end to end.
 *
 * Parity status: no reference test, golden vector or GSL build exists in the
 * reference tree or in this environment, so the stream itself is "parity
 * unpinned" (see the repository's design notes); the GPU kernels are checked
 * bit-exact against this file.
 *
 * This implementation deliberately uses a circular buffer (the product uses a
 * sliding register window) so the two are independent codings of the same
 * algorithm.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MASK48 ((((uint64_t)1) << 48) - 1)

typedef struct {
    uint64_t buf[12]; /* buf[n % 12] = y[n] for the last 12 generated words */
    uint64_t n;       /* index of the next word to generate                 */
    uint64_t carry;   /* borrow of the previous step                        */
    uint64_t out[12]; /* delivered words of the current block               */
    int avail;        /* words of out[] not yet delivered                   */
} oracle_rlx;

static void rlx_seed(oracle_rlx *r, unsigned long s)
{
    int bits[31];
    int32_t v;
    int ib = 0, jb = 18, w, l, q;
    if (s == 0) s = 1;
    v = (int32_t)(uint32_t)(s & 0xffffffffUL);
    for (q = 0; q < 31; ++q) { bits[q] = v % 2; v /= 2; }
    for (w = 0; w < 12; ++w) {
        uint64_t word = 0;
        for (l = 0; l < 48; ++l) {
            word = 2 * word + (uint64_t)((bits[ib] + 1) % 2);
            bits[ib] = (bits[ib] + bits[jb]) % 2;
            ib = (ib + 1) % 31;
            jb = (jb + 1) % 31;
        }
        r->buf[w] = word;
    }
    r->n = 12;
    r->carry = 0;
    r->avail = 0;
}

static void rlx_block(oracle_rlx *r)
{
    int t;
    for (t = 0; t < 202; ++t) {
        uint64_t n = r->n;
        uint64_t a = r->buf[(n - 5) % 12], b = r->buf[(n - 12) % 12];
        uint64_t d;
        if (a >= b + r->carry) { d = a - b - r->carry; r->carry = 0; }
        else { d = a + (((uint64_t)1) << 48) - b - r->carry; r->carry = 1; }
        r->buf[n % 12] = d & MASK48;
        if (t >= 190) r->out[t - 190] = d & MASK48;
        r->n = n + 1;
    }
    r->avail = 12;
}

static uint64_t rlx_next_int(oracle_rlx *r)
{
    if (r->avail == 0) rlx_block(r);
    return r->out[12 - r->avail--];
}

static double rlx_uniform(oracle_rlx *r)
{
    return (double)rlx_next_int(r) * (1.0 / 281474976710656.0);
}

/* First `count` words (48-bit integers) of the stream seeded with `seed`. */
void mfxo_ranlxd1_words(unsigned long seed, size_t count, uint64_t *out)
{
    oracle_rlx r;
    size_t q;
    rlx_seed(&r, seed);
    for (q = 0; q < count; ++q) out[q] = rlx_next_int(&r);
}

/* NGenIC seed table, random_ngenic.cc:42-74 (the spiral fill order). */
void mfxo_ngenic_seed_table(long seed, size_t nres, uint32_t *table)
{
    oracle_rlx r;
    size_t i, j;
    const double m = (double)0x7fffffff;
    rlx_seed(&r, (unsigned long)seed);
    memset(table, 0, nres * nres * sizeof(uint32_t));
    for (i = 0; i < nres / 2; ++i) {
        for (j = 0; j < i; j++) table[i * nres + j] = (uint32_t)(m * rlx_uniform(&r));
        for (j = 0; j < i + 1; j++) table[j * nres + i] = (uint32_t)(m * rlx_uniform(&r));
        for (j = 0; j < i; j++) table[(nres - 1 - i) * nres + j] = (uint32_t)(m * rlx_uniform(&r));
        for (j = 0; j < i + 1; j++) table[(nres - 1 - j) * nres + i] = (uint32_t)(m * rlx_uniform(&r));
        for (j = 0; j < i; j++) table[i * nres + (nres - 1 - j)] = (uint32_t)(m * rlx_uniform(&r));
        for (j = 0; j < i + 1; j++) table[j * nres + (nres - 1 - i)] = (uint32_t)(m * rlx_uniform(&r));
        for (j = 0; j < i; j++) table[(nres - 1 - i) * nres + (nres - 1 - j)] = (uint32_t)(m * rlx_uniform(&r));
        for (j = 0; j < i + 1; j++) table[(nres - 1 - j) * nres + (nres - 1 - i)] = (uint32_t)(m * rlx_uniform(&r));
    }
}

/*
 * RNG_ngenic::Fill_Grid, random_ngenic.cc:84-154, non-distributed branch.
 * `out` is the k-space grid as interleaved (re,im) doubles in the layout
 * kelem(i,j,k) = out[2*((i*N + j)*(N/2+1) + k)] (grid_fft.hh:196-206).
 * If `uniforms` is non-NULL it receives, per column (i,j), the first
 * 2*(N/2+1) delivered uniforms of that column's stream in draw order
 * (phase, amplitude per k; a rejected amplitude draw is not recorded).
 */
void mfxo_ngenic_fill(size_t nres, const uint32_t *table, double *out, double *uniforms)
{
    const size_t nk = nres / 2 + 1;
    size_t i, j, k;
    memset(out, 0, 2 * nres * nres * nk * sizeof(double));
    for (i = 0; i < nres; ++i) {
        size_t ii = (i > 0) ? nres - i : 0;
        for (j = 0; j < nres; ++j) {
            size_t jj = (j > 0) ? nres - j : 0;
            oracle_rlx r;
            rlx_seed(&r, table[i * nres + j]);
            for (k = 0; k < nk; ++k) {
                double uphase = rlx_uniform(&r);
                double phase = uphase * 2 * M_PI;
                double ampl = 0, re, im;
                double *u = uniforms ? uniforms + 2 * ((i * nres + j) * nk + k) : NULL;
                if (u) u[0] = uphase;
                do {
                    ampl = rlx_uniform(&r);
                } while (ampl == 0 || ampl == 1);
                if (u) u[1] = ampl;
                if (i == nres / 2 || j == nres / 2 || k == nres / 2) continue;
                if (i == 0 && j == 0 && k == 0) continue;
                ampl = sqrt(-log(ampl));
                re = ampl * cos(phase);
                im = ampl * sin(phase);
                if (k > 0) {
                    double *e = out + 2 * ((i * nres + j) * nk + k);
                    e[0] = re; e[1] = im;
                } else {
                    if (i == 0) {
                        if (j < nres / 2) {
                            double *e = out + 2 * ((i * nres + j) * nk);
                            double *c = out + 2 * ((i * nres + jj) * nk);
                            e[0] = re; e[1] = im;
                            c[0] = re; c[1] = -im;
                        }
                    } else if (i < nres / 2) {
                        double *e = out + 2 * ((i * nres + j) * nk);
                        double *c = out + 2 * ((ii * nres + jj) * nk);
                        e[0] = re; e[1] = im;
                        c[0] = re; c[1] = -im;
                    }
                }
            }
        }
    }
}
