"""CPU tests: oracle pinned against golden vectors, host-side plugin logic of
libmfx against the oracle, and the C ABI surface.  No GPU needed."""
import pathlib
import re

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"


# ---------------------------------------------------------------------------
# C ABI surface
# ---------------------------------------------------------------------------
def header_symbols():
    txt = (ROOT / "include" / "mfx.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mfx_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(mfxlib):
    L = mfxlib.load()
    syms = header_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    assert set(syms) == set(mfxlib.EXPORTS), set(syms) ^ set(mfxlib.EXPORTS)


def test_engine_create_fails_loudly_without_gpu(mfxlib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(mfxlib.MfxError) as e:
        mfxlib.Engine(0)
    assert e.value.code == mfxlib.MFX_ECUDA


# ---------------------------------------------------------------------------
# RANLUX / NGenIC
# ---------------------------------------------------------------------------
def _py_ranlxd1(seed, count):
    """Third, pure-Python coding of the ranlxd1 stream (small counts only)."""
    return _py_ranlxd(seed, count, block=202)


def _py_ranlxd(seed, count, block):
    """Pure-Python RANLUX on 48-bit words: `block` words generated per 12
    delivered (202 for ranlxd1, 397 for ranlxd2)."""
    if seed == 0:
        seed = 1
    bits = [(seed >> q) & 1 for q in range(31)]
    ib, jb = 0, 18
    y = []
    for _ in range(12):
        w = 0
        for _ in range(48):
            w = 2 * w + (1 - bits[ib])
            bits[ib] = bits[ib] ^ bits[jb]
            ib, jb = (ib + 1) % 31, (jb + 1) % 31
        y.append(w)
    out, c = [], 0
    while len(out) < count:
        blk = []
        for _ in range(block):
            d = y[-5] - y[-12] - c
            c = 1 if d < 0 else 0
            d %= 1 << 48
            y.append(d)
            y = y[-12:]
            blk.append(d)
        out.extend(blk[-12:])
    return np.array(out[:count], dtype=np.uint64)


# Published known-answer values of GSL's RANLUX generators: GSL's own RNG test
# suite (rng/test.c, `rng_test(gsl_rng_ranlxd1, 1, 10000, 1998227290UL)` and
# `rng_test(gsl_rng_ranlxd2, 1, 10000, 3949287736UL)`) seeds the generator with
# gsl_rng_set(r, 1), draws 10000 values with gsl_rng_get and checks the last
# one.  gsl_rng_get of ranlxd returns floor(u * 2^32) of the 48-bit uniform u,
# i.e. the word's top 32 bits; the suite's comments give u itself,
# 0.465248546261094020 (ranlxd1) and 0.919515205581550532 (ranlxd2).  The
# reference draws its NGenIC noise from gsl_rng_ranlxd1
# (src/plugins/random_ngenic.cc:44-45, 104-114).
GSL_RANLXD1_SEED1_DRAW10000 = 1998227290
GSL_RANLXD2_SEED1_DRAW10000 = 3949287736


def test_ranlxd1_matches_gsl_known_answer(oracle):
    w = int(oracle.ranlxd1_words(1, 10000)[-1])
    assert w >> 16 == GSL_RANLXD1_SEED1_DRAW10000
    assert abs(w / 2.0**48 - 0.465248546261094020) < 1e-16


def test_ranlux_luxury_two_matches_gsl_known_answer():
    """The same restatement with ranlxd2's block length (397 words per 12
    delivered) reproduces GSL's ranlxd2 value: seeding, the subtract-with-borrow
    recursion and the delivery order are pinned independently of the block
    length that ranlxd1 uses."""
    w = int(_py_ranlxd(1, 10000, block=397)[-1])
    assert w >> 16 == GSL_RANLXD2_SEED1_DRAW10000
    assert abs(w / 2.0**48 - 0.919515205581550532) < 1e-16


@pytest.mark.parametrize("seed", [1, 12345, 4242, 2**31 - 2])
def test_ranlux_three_codings_agree(oracle, seed):
    a = oracle.ranlxd1_words(seed, 100)
    b = _py_ranlxd1(seed, 100)
    assert np.array_equal(a, b)
    assert np.all(a < 2**48)


def test_seed_zero_means_one(oracle):
    assert np.array_equal(oracle.ranlxd1_words(0, 30), oracle.ranlxd1_words(1, 30))


@pytest.mark.parametrize("n,seed", [(16, 12345), (64, 12345), (128, 4242), (96, 1)])
def test_host_seed_table_matches_oracle(mfxlib, oracle, n, seed):
    assert np.array_equal(mfxlib.ngenic_seed_table(seed, n), oracle.ngenic_seed_table(seed, n))


def test_golden_ranlux_and_seed_table(oracle):
    g = np.load(GOLDEN / "ngenic_16.npz")
    assert np.array_equal(oracle.ranlxd1_words(int(g["seed"]), g["words"].size), g["words"])
    assert np.array_equal(oracle.ngenic_seed_table(int(g["seed"]), 16), g["seed_table"])
    w = oracle.ngenic_fill(16, g["seed_table"])
    np.testing.assert_allclose(w, g["noise"], rtol=0, atol=1e-15)


def test_noise_hermitian_and_nyquist(oracle):
    n = 32
    w = oracle.ngenic_fill(n, oracle.ngenic_seed_table(7, n))
    nh = n // 2
    assert np.all(w[nh] == 0) and np.all(w[:, nh] == 0) and np.all(w[:, :, nh] == 0)
    assert w[0, 0, 0] == 0
    p = w[:, :, 0]
    idx = (-np.arange(n)) % n
    assert np.array_equal(p[np.ix_(idx, idx)], np.conj(p))
    # unit-variance Gaussian modes: <|z|^2> = 1 (ampl = sqrt(-ln u))
    m = np.abs(w[1:nh, 1:nh, 1:nh]) ** 2
    assert abs(m.mean() - 1.0) < 0.05


# ---------------------------------------------------------------------------
# oracle convolver properties
# ---------------------------------------------------------------------------
def test_orszag_product_is_exact_for_band_limited_fields(oracle):
    """For fields with modes |k_i| < N/3 the 3/2-padded product has no aliasing:
    it equals the exact product truncated to the N-grid."""
    n, L = 24, 1.0
    rng = np.random.default_rng(0)
    r1 = rng.standard_normal((n, n, n))
    r2 = rng.standard_normal((n, n, n))
    k1, k2 = oracle.fft_r2c(r1), oracle.fft_r2c(r2)
    i = np.arange(n)
    si = np.where(i > n // 2, i - n, i)
    keep = (np.abs(si)[:, None, None] < n // 4) & (np.abs(si)[None, :, None] < n // 4) & (np.arange(n // 2 + 1)[None, None, :] < n // 4)
    k1, k2 = k1 * keep, k2 * keep
    C = oracle.OrszagConvolver(n, L)
    got = C.convolve2(k1, k2)
    # with unitary transforms on both grids the padded product equals the
    # product taken directly on the N-grid (no aliasing for these bands)
    ref = oracle.fft_r2c(oracle.fft_c2r(k1, n) * oracle.fft_c2r(k2, n))
    ref[C.nyq] = 0
    np.testing.assert_allclose(got, ref, atol=1e-12)


def test_inverse_laplacian_of_laplacian(oracle):
    n, L = 16, 10.0
    rng = np.random.default_rng(1)
    f = oracle.fft_r2c(rng.standard_normal((n, n, n)))
    f[0, 0, 0] = 0
    lap = -oracle.kmod2(n, L) * f
    np.testing.assert_allclose(oracle.inverse_laplacian(lap, n, L), f, atol=1e-12)


# ---------------------------------------------------------------------------
# host cosmology vs the oracle's independent restatement
# ---------------------------------------------------------------------------
def test_host_cosmology_matches_oracle(mfxlib):
    from oracle import cosmo
    o = cosmo.Cosmology(Om=0.3, Ob=0.045, H0=70.0, n_s=0.965, sigma8=0.81)
    c = mfxlib.Cosmology(mfxlib.ini_text(64, 100.0, 49.0, 2, 12345))
    assert c.get("Omega_DE") == pytest.approx(0.7, abs=1e-15)
    assert c.get("Omega_r") == 0.0
    k = np.logspace(-4, 2.5, 200)
    np.testing.assert_allclose(c.transfer(k), o.transfer(k), rtol=1e-13)
    assert c.get("pnorm") == pytest.approx(o.pnorm, rel=1e-10)
    np.testing.assert_allclose(c.amplitude(k), o.amplitude(k), rtol=1e-10)
    for z in (49.0, 24.0, 0.5):
        a = 1.0 / (1.0 + z)
        # the reference's own Cash-Karp (eps 1e-10) + log-log spline is good to ~1e-8
        assert c.growth(a) == pytest.approx(o.growth(a), rel=5e-8)
    assert c.get("vfact_start") == pytest.approx(o.vfact(1.0 / 50.0), rel=1e-8)


def test_amp_table_definition(mfxlib):
    c = mfxlib.Cosmology(mfxlib.ini_text(32, 100.0, 49.0, 2, 1))
    t = c.amp_table(32, 100.0)
    assert t.size == 3 * 16 * 16 + 1 and t[0] == 0.0
    kf = 2 * np.pi / 100.0
    n = np.arange(1, t.size)
    k = kf * np.sqrt(n)
    np.testing.assert_allclose(t[1:], c.amplitude(k) / (k * k), rtol=1e-14)


def test_config_parser_and_errors(mfxlib):
    with pytest.raises(mfxlib.MfxError):
        mfxlib.Cosmology("[setup]\nzstart=10\n[cosmology]\ntransfer = CLASS\n")
    txt = mfxlib.ini_text(32, 50.0, 24.0, 3, 3).replace("Omega_m = 0.3", "Omega_m = 0.31 # trailing comment")
    c = mfxlib.Cosmology(txt)
    assert c.get("Omega_m") == 0.31


# ---------------------------------------------------------------------------
# MUSIC1 white noise (oracle/music.c): GSL's mt19937 and ratio-method normals
# ---------------------------------------------------------------------------
def test_mt19937_tenthousandth_output_is_the_cpp_standards(oracle):
    """The C++ standard's requirement on std::mt19937 ([rand.predef]): the
    10000th output of a default-seeded engine (seed 5489) is 4123659995."""
    assert int(oracle.mt19937_words(5489, 10000)[-1]) == 4123659995


def test_mt19937_matches_cpp_std_mt19937(oracle, tmp_path):
    """GSL seeds mt19937 like std::mt19937 (the 2002 initialisation): the
    restatement equals the C++ library's engine output for output."""
    import subprocess
    src = tmp_path / "mt.cc"
    src.write_text("""
#include <cstdio>
#include <cstdlib>
#include <random>
int main(int argc, char **argv) {
  std::mt19937 g(std::strtoul(argv[1], nullptr, 10));
  for (int i = 0; i < 2000; ++i) std::printf("%u\\n", unsigned(g()));
}
""")
    exe = tmp_path / "mt"
    subprocess.check_call(["g++", "-O1", "-o", str(exe), str(src)])
    for seed in (1, 4357, 12345, 2**31 + 5, 4294967295):
        out = subprocess.run([str(exe), str(seed)], capture_output=True, text=True, check=True).stdout.split()
        ref = np.array(out, dtype=np.uint64).astype(np.uint32)
        assert np.array_equal(oracle.mt19937_words(seed, 2000), ref), seed


def test_ratio_method_normals_are_standard_normal(oracle):
    from scipy import stats
    x = oracle.leva_normals(20261204, 400000)
    assert abs(x.mean()) < 5e-3 and abs(x.var() - 1.0) < 1e-2
    assert abs(stats.kurtosis(x)) < 3e-2 and abs(stats.skew(x)) < 1e-2
    assert stats.kstest(x, "norm").pvalue > 1e-3


def test_music_noise_cubes_and_means(oracle):
    """Each 32^3 cube is the ratio-method stream of seed + cube index (kk
    fastest), less the two mean subtractions; the field has zero mean."""
    n, seed, cs = 64, 777, 32
    f = oracle.music_noise_real(n, seed, cs)
    assert abs(f.mean()) < 1e-15
    raw = [oracle.leva_normals(seed + q, cs ** 3).reshape(cs, cs, cs) for q in range(8)]
    shift = np.mean([r.mean() for r in raw])
    for q, r in enumerate(raw):
        ic, jc, kc = q // 4, (q // 2) % 2, q % 2
        blk = f[ic * cs:(ic + 1) * cs, jc * cs:(jc + 1) * cs, kc * cs:(kc + 1) * cs]
        d = blk - (r - shift)
        assert np.ptp(d) < 1e-13  # the remaining zero-mean correction is one constant
    small = oracle.music_noise_real(16, 3, 32)  # one cube of the whole grid below the cube size
    r = oracle.leva_normals(3, 16 ** 3).reshape(16, 16, 16)
    assert np.allclose(small, r - r.mean(), rtol=0, atol=1e-13)


def test_music_dummy_seeds(oracle):
    """Levels without a seed[level] key get -|(-2 - l) % 123 + (-2 + 7342523521 l) % 123456789|
    with C's truncating remainder (random_music.cc:176-183)."""
    assert oracle.music_dummy_seed(0) == -4
    assert oracle.music_dummy_seed(1) == -(7342523519 % 123456789 - 3)
    assert oracle.music_dummy_seed(5) == -abs(-7 + (5 * 7342523521 - 2) % 123456789)
    assert all(oracle.music_dummy_seed(level) < 0 for level in range(12))


def test_music_refinement_keeps_the_coarse_modes(oracle):
    """A refined level carries the coarse level's modes (half-cell phase,
    sqrt 8) off the coarse Nyquist indices and its own cubes' modes elsewhere."""
    nc, nf = 8, 16
    coarse = oracle.music_noise_real(nc, 21, 4)
    fine_raw = oracle.music_cubes_raw(nf, 22, 4)
    fine = oracle.music_refine(coarse, fine_raw)
    cf, cr, cc = (np.fft.rfftn(x) for x in (fine, fine_raw, coarse))
    for (i, j, k) in [(1, 2, 3), (7, 6, 1), (0, 5, 2), (3, 0, 0)]:
        ii = i if i <= nc // 2 else i + nf // 2
        jj = j if j <= nc // 2 else j + nf // 2
        kx, ky = (i if i <= nc // 2 else i - nc), (j if j <= nc // 2 else j - nc)
        ph = np.exp(-0.5j * np.pi * (kx + ky + k) / nc)
        assert abs(cf[ii, jj, k] - cc[i, j, k] * ph * np.sqrt(8.0)) < 1e-10
    assert abs(cf[5, 9, 6] - cr[5, 9, 6]) < 1e-10  # not a coarse mode: the fine cubes' own
    assert abs(cf[4, 1, 1] - cr[4, 1, 1]) < 1e-10  # a coarse Nyquist index: kept from the fine level
    lev = oracle.music_levels(16, {3: 21}, 4)
    assert np.allclose(lev, oracle.music_refine(coarse, oracle.music_cubes_raw(16, oracle.music_dummy_seed(4), 4)))


def test_music_restriction_is_the_inverse_embedding(oracle):
    """Restricting a refined level returns the coarse field where the
    refinement copied its modes: k-space averaging undoes the half-cell phase
    and the sqrt(8) of the coarse mode replacement (off the Nyquist indices)."""
    coarse = oracle.music_noise_real(8, 5, 4)
    fine = oracle.music_refine(coarse, oracle.music_cubes_raw(16, 6, 4))
    back = np.fft.rfftn(oracle.music_restrict(fine))
    cc = np.fft.rfftn(coarse)
    keep = np.ones(cc.shape, bool)
    keep[4, :, :] = keep[:, 4, :] = False
    keep[:, :, 4] = False
    assert np.max(np.abs(back[keep] - cc[keep])) < 1e-10


def write_grafic(path, field_xyz, marker=4, dtype=np.float32, sign=-1.0):
    """A MUSIC1 white-noise file holding field_xyz ([x][y][z]) as the reader
    of random_music_wnoise_generator.cc:68-282 expects it (values stored
    negated for the default grafic_sign = false)."""
    n = field_xyz.shape[0]
    mk = (lambda v: np.array([v], np.uint32 if marker == 4 else np.uint64).tobytes())
    with open(path, "wb") as f:
        f.write(mk(16) + np.array([n, n, n, 7], np.int32).tobytes() + mk(16))
        for z in range(n):
            rec = (sign * field_xyz[:, :, z].T).astype(dtype).tobytes()  # [y][x], x fastest
            f.write(mk(len(rec)) + rec + mk(len(rec)))


@pytest.mark.parametrize("marker,dtype", [(4, np.float32), (8, np.float64)])
def test_grafic_noise_reader(oracle, tmp_path, marker, dtype):
    rng = np.random.default_rng(3)
    field = rng.standard_normal((8, 8, 8))
    p = tmp_path / "wn.bin"
    write_grafic(p, field, marker, dtype)
    got = oracle.read_grafic_noise(str(p), 8)
    tol = 1e-6 if dtype == np.float32 else 0.0
    assert np.max(np.abs(got - field)) <= tol
    assert np.allclose(oracle.read_grafic_noise(str(p), 8, grafic_sign=True), -got)
