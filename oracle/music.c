/*
 * ORACLE -- test infrastructure only.  Nothing in the product links this file;
 * only tests/ and bench.py's CPU legs load it, and only as the checker.
 *
 * CPU restatement of monofonIC's MUSIC1 white-noise plugin: the cube fill of
 * one level (src/plugins/random_music.cc:83-130, 236-283 and
 * src/plugins/random_music_wnoise_generator.cc:27-52, 588-626, 684-797); the
 * refinement from coarser seeded levels is in oracle/lpt.py (music_levels).
 *
 *   - the grid of res^3 cells is cut into cubes of cubesize^3 (32 by default;
 *     one cube of res^3 when res < cubesize), cube (ic, jc, kc) numbered
 *     icube = (ic ncubes + jc) ncubes + kc;
 *   - each cube draws its values, cell (ii, jj, kk) with kk fastest, from its
 *     own Mersenne-Twister stream seeded with seed + icube;
 *   - the mean of the cube means is subtracted from every value, then the mean
 *     of all res^3 values once more (the zero-mean pass);
 *   - Fill_Grid copies the cells into the real-space grid, which the IC
 *     generator transforms to k-space (ic_generator.cc:305-383).
 *
 * The generators are GSL's (a third-party dependency absent from the reference
 * tree, version unpinned: CMakeLists.txt:132), restated from their published
 * algorithms:
 *   - gsl_rng_mt19937: M. Matsumoto and T. Nishimura's MT19937 (ACM TOMACS 8
 *     (1998) 3), seeded with their 2002 initialisation (x[0] = s, x[i] =
 *     1812433253 (x[i-1] xor (x[i-1] >> 30)) + i, mod 2^32; seed 0 means
 *     4357), uniform = output / 2^32 -- the same seeding as C++'s std::mt19937,
 *     against which the tests check it;
 *   - gsl_ran_ugaussian_ratio_method: J. L. Leva's ratio-of-uniforms normal
 *     generator (ACM TOMS 18 (1992) 449) with its published bounding constants.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    uint32_t x[624];
    int i;
} oracle_mt;

static void mt_seed(oracle_mt *m, unsigned long s)
{
    int k;
    if (s == 0) s = 4357;
    m->x[0] = (uint32_t)(s & 0xffffffffUL);
    for (k = 1; k < 624; ++k) m->x[k] = (uint32_t)(1812433253UL * (m->x[k - 1] ^ (m->x[k - 1] >> 30)) + (uint32_t)k);
    m->i = 624;
}

static uint32_t mt_next(oracle_mt *m)
{
    uint32_t y;
    if (m->i >= 624) {
        int k;
        for (k = 0; k < 624; ++k) {
            const uint32_t v = (m->x[k] & 0x80000000u) | (m->x[(k + 1) % 624] & 0x7fffffffu);
            m->x[k] = m->x[(k + 397) % 624] ^ (v >> 1) ^ ((v & 1u) ? 0x9908b0dfu : 0u);
        }
        m->i = 0;
    }
    y = m->x[m->i++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

static double mt_uniform(oracle_mt *m) { return (double)mt_next(m) / 4294967296.0; }

/* Leva's ratio-of-uniforms method: u in (0, 1], v in [-1/2, 1/2) scaled by
 * 2 sqrt(2/e); quick acceptance inside the inner quadratic bound, quick
 * rejection outside the outer one, the exact test v^2 <= -4 u^2 ln u between */
static double leva_normal(oracle_mt *m)
{
    const double s = 0.449871, t = -0.386595, a = 0.19600, b = 0.25472, r1 = 0.27597, r2 = 0.27846;
    double u, v, x, y, q;
    do {
        u = 1.0 - mt_uniform(m);
        v = mt_uniform(m) - 0.5;
        v *= 1.7156;
        x = u - s;
        y = fabs(v) - t;
        q = x * x + y * (a * y - b * x);
    } while (q >= r1 && (q > r2 || v * v > -4.0 * u * u * log(u)));
    return v / u;
}

/* First `count` 32-bit outputs of the stream seeded with `seed`. */
void mfxo_mt19937_words(unsigned long seed, size_t count, uint32_t *out)
{
    oracle_mt m;
    size_t q;
    mt_seed(&m, seed);
    for (q = 0; q < count; ++q) out[q] = mt_next(&m);
}

/* First `count` normals of the ratio method on the stream seeded with `seed`. */
void mfxo_leva_normals(unsigned long seed, size_t count, double *out)
{
    oracle_mt m;
    size_t q;
    mt_seed(&m, seed);
    for (q = 0; q < count; ++q) out[q] = leva_normal(&m);
}

/* The cubes of one level without any mean subtraction (the refinement
 * levels' fill, random_music_wnoise_generator.cc:392-406: their mean only
 * moves the k = 0 mode, which the coarse level's replaces). */
void mfxo_music_cubes(size_t res, size_t cubesize, long seed, double *out)
{
    size_t nc, cs, ic, jc, kc, ii, jj, kk;
    if (res < cubesize) {
        nc = 1;
        cs = res;
    } else {
        nc = res / cubesize;
        cs = cubesize;
    }
    for (ic = 0; ic < nc; ++ic)
        for (jc = 0; jc < nc; ++jc)
            for (kc = 0; kc < nc; ++kc) {
                oracle_mt m;
                mt_seed(&m, (unsigned long)(seed + (long)((ic * nc + jc) * nc + kc)));
                for (ii = 0; ii < cs; ++ii)
                    for (jj = 0; jj < cs; ++jj)
                        for (kk = 0; kk < cs; ++kk)
                            out[((ic * cs + ii) * res + (jc * cs + jj)) * res + (kc * cs + kk)] = leva_normal(&m);
            }
}

/* The MUSIC1 single-level white noise in real space, out[(i res + j) res + k]. */
void mfxo_music_noise(size_t res, size_t cubesize, long seed, double *out)
{
    size_t nc, cs, ic, jc, kc, ii, jj, kk, q;
    double msum = 0.0, mean = 0.0;
    if (res < cubesize) {
        nc = 1;
        cs = res;
    } else {
        nc = res / cubesize;
        if (nc < 1) nc = 1;
        cs = cubesize;
    }
    for (ic = 0; ic < nc; ++ic)
        for (jc = 0; jc < nc; ++jc)
            for (kc = 0; kc < nc; ++kc) {
                const size_t icube = (ic * nc + jc) * nc + kc;
                oracle_mt m;
                double cm = 0.0;
                mt_seed(&m, (unsigned long)(seed + (long)icube));
                for (ii = 0; ii < cs; ++ii)
                    for (jj = 0; jj < cs; ++jj)
                        for (kk = 0; kk < cs; ++kk) {
                            const double g = leva_normal(&m);
                            out[((ic * cs + ii) * res + (jc * cs + jj)) * res + (kc * cs + kk)] = g;
                            cm += g;
                        }
                msum += cm / (double)(cs * cs * cs);
            }
    msum /= (double)(nc * nc * nc);
    for (q = 0; q < res * res * res; ++q) out[q] -= msum;
    for (q = 0; q < res * res * res; ++q) mean += out[q];
    mean *= 1.0 / (double)(res * res * res);
    for (q = 0; q < res * res * res; ++q) out[q] -= mean;
}
