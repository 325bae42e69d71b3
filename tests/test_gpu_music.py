"""MUSIC1 white noise on the device against the oracle (oracle/music.c).

The cube normals are the sequential generator's values bit for bit (MT19937
words and the ratio method's accept/reject decisions reproduced exactly), so
the FP64 k-space noise matches the oracle's forward transform to FFT rounding;
the mean subtraction of the reference only moves k = 0, which both sides hold
at zero.  The whole pipeline then meets the same bars as with NGenIC's noise:
1e-10 relative for the plain FP64 form, 1e-5 of the interparticle spacing for
the FP32 form.
"""
import numpy as np
import pytest

from test_gpu_parity import TOL_FP64, Case, check_fields, check_particles, rel_l2

pytestmark = pytest.mark.gpu


def music_job(mfxlib, engine, c, seed, cubesize=32, precision=None, **kw):
    precision = mfxlib.FP64 if precision is None else precision
    return mfxlib.Job(engine, c.n, c.L, c.order, None, c.amp, c.coef, lattice=c.lattice, precision=precision,
                      plt_table=c.plt, fixing=c.fixing, inversion=c.inversion, lunit=c.lunit, vunit=c.vunit,
                      noise_generator=mfxlib.NOISE_MUSIC1, music_seed=seed, music_cubesize=cubesize, **kw)


def oracle_noise(oracle, n, seed, cubesize):
    w = oracle.music_fill(n, seed, cubesize)
    w[0, 0, 0] = 0.0  # zero mean up to rounding on the reference's side
    return w


@pytest.mark.parametrize("n,cubesize,seed", [(16, 32, 12345), (32, 8, 7), (64, 32, 4242),
                                             (32, 16, (1 << 32) - 3)])
def test_music_raw_noise_matches_oracle(mfxlib, engine, oracle, n, cubesize, seed):
    """One cube below the cube size, 64 small cubes, the default cubes, and cube
    seeds that cross 2^32 (the low 32 bits of the seed go into the state, and a
    seed of 2^32 is not GSL's zero seed)."""
    c = Case(mfxlib, n, 100.0, 49.0, 1, 1)
    j = music_job(mfxlib, engine, c, seed, cubesize, want_particles=False)
    j.run_noise(raw=True)
    got = j.field(mfxlib.FIELD_NOISE)
    ref = oracle_noise(oracle, n, seed, cubesize)
    assert got[0, 0, 0] == 0
    assert np.max(np.abs(got - ref)) < 1e-12
    # unit variance per mode, Nyquist planes populated (unlike NGenIC)
    assert abs(np.mean(np.abs(got[1:, 1:, 1:-1]) ** 2) - 1.0) < 0.1
    assert np.all(got[:, :, n // 2] != 0)


@pytest.mark.parametrize("fixing,inversion", [(False, False), (True, True)])
def test_music_normalised_noise(mfxlib, engine, oracle, fixing, inversion):
    n, L = 32, 300.0
    c = Case(mfxlib, n, L, 24.0, 1, 1, fixing=fixing, inversion=inversion)
    j = music_job(mfxlib, engine, c, 99, 16, want_particles=False)
    j.run_noise(raw=False)
    ref = oracle.normalise_noise(oracle_noise(oracle, n, 99, 16), n, L, fixing, inversion)
    ref[0, 0, 0] = 0.0
    assert rel_l2(j.field(mfxlib.FIELD_NOISE), ref) < 1e-13


@pytest.mark.parametrize("order,lattice,plt", [(2, 0, False), (3, 1, False), (2, 2, False), (3, 2, True)])
def test_music_pipeline_fp64(mfxlib, engine, oracle, order, lattice, plt):
    """MUSIC1 noise fills the Nyquist planes: with PLT the kz = N/2 plane takes
    the same Hermitian (odd-gradient) treatment as kz = 0, and on FCC the
    sub-lattice phases of the Nyquist modes on both planes follow the
    reference's step-by-step shifts (three c2r projections, not one)."""
    n, seed = 64, 31337
    tab = engine.plt_table(lattice) if plt else None
    c = Case(mfxlib, n, 200.0, 30.0, order, 1, lattice=lattice, plt=tab)
    j = music_job(mfxlib, engine, c, seed)
    j.run()
    grad = None
    if plt:
        from oracle import plt as oplt
        grad = oplt.PLTGradient(n, c.L, tab)
    res = oracle.run_lpt(n, c.L, None, c.amplitude, order, c.dplus, c.vfac, lattice=lattice, lunit=c.lunit,
                         vunit=c.vunit, grad=grad, noise=oracle_noise(oracle, n, seed, 32))
    check_fields(mfxlib, j, res, order, TOL_FP64)
    check_particles(c, j, res, TOL_FP64)


def test_music_pipeline_fp32c_plt(mfxlib, engine, oracle):
    """FP32 form with PLT on FCC: MUSIC1 noise fills the Nyquist planes, so the
    job takes the cuFFT route rather than the pruned transforms."""
    n, seed, lattice = 64, 5, 2
    tab = engine.plt_table(lattice)
    c = Case(mfxlib, n, 1000.0 * 64 / 768, 24.0, 3, 1, lattice=lattice, plt=tab)
    j = music_job(mfxlib, engine, c, seed, precision=mfxlib.FP32C, pos64=True, vel64=False)
    j.run()
    from oracle import plt as oplt
    res = oracle.run_lpt(n, c.L, None, c.amplitude, 3, c.dplus, c.vfac, lattice=lattice, lunit=c.lunit,
                         vunit=c.vunit, grad=oplt.PLTGradient(n, c.L, tab), noise=oracle_noise(oracle, n, seed, 32))
    pos, vel, ids = j.particles()
    delta = c.L / (c.n * 2 ** (lattice / 3.0))
    err = (pos - res["pos"]) / delta
    assert np.sqrt(np.mean(err ** 2)) < 1e-5
    assert np.max(np.abs(err)) < 2e-4
    assert rel_l2(vel.astype(np.float64), res["vel"]) < 1e-5
    assert np.array_equal(ids, res["ids"])


def test_music_reseed_through_captured_graph(mfxlib, engine, oracle):
    """The base seed is read from device memory: a captured pipeline replays
    with the seed uploaded after the capture."""
    n = 32
    c = Case(mfxlib, n, 100.0, 49.0, 2, 1)
    j = music_job(mfxlib, engine, c, 11, 8, want_particles=False)
    j.capture()
    for seed in (11, 12):
        j.upload(music_seed=seed)
        j.run()
        w = oracle.normalise_noise(oracle_noise(oracle, n, seed, 8), n, c.L, False, False)
        phi = oracle.phi1_from_noise(w, n, c.L, c.amplitude)
        assert rel_l2(j.field(mfxlib.FIELD_PHI1) * c.coef["g1"], phi * c.coef["g1"]) < 1e-12


@pytest.mark.parametrize("n,cubesize,why", [(48, 16, "power of two"), (64, 24, "tile"), (64, 1, "tile")])
def test_music_descriptor_checks(mfxlib, engine, n, cubesize, why):
    c = Case(mfxlib, n, 100.0, 49.0, 1, 1)
    with pytest.raises(mfxlib.MfxError, match=why):
        music_job(mfxlib, engine, c, 5, cubesize, want_particles=False)
    with pytest.raises(mfxlib.MfxError, match="positive seed"):
        music_job(mfxlib, engine, Case(mfxlib, 32, 100.0, 49.0, 1, 1), 0, 32, want_particles=False)


def test_run_config_music1(mfxlib, engine, tmp_path):
    """The driver takes [random] generator = MUSIC1 with seed[log2 GridRes]."""
    f = tmp_path / "ics.bin"
    engine.run_config(mfxlib.ini_text(32, 50.0, 24.0, 2, 777, "sc", filename=str(f), generator="MUSIC1",
                                      cubesize=16))
    raw = f.read_bytes()
    np_ = int(np.frombuffer(raw[8:16], np.uint64)[0])
    assert np_ == 32 ** 3
    c = Case(mfxlib, 32, 50.0, 24.0, 2, 1)
    j = music_job(mfxlib, engine, c, 777, 16)
    j.run()
    pos, vel, ids = j.particles()
    off = 8 + 8 + 4 + 4 + 24
    assert np.array_equal(np.frombuffer(raw[off:off + 24 * np_], np.float64).reshape(-1, 3), pos)
    bad = mfxlib.ini_text(32, 50.0, 24.0, 2, 777, filename=str(f), generator="MUSIC1").replace(
        "seed[5] = 777", "seed[9] = 12\nseed[5] = 777")
    with pytest.raises(mfxlib.MfxError):
        engine.run_config(bad)  # a seed more than three levels finer than the grid's


@pytest.mark.parametrize("n,cubesize,seeds", [(32, 8, {3: 4242}), (32, 4, {2: 11, 4: 12}),
                                              (64, 16, {4: 99, 6: 100}), (32, 8, {3: 5, 4: 6, 5: 7}),
                                              (16, 8, {5: 123}), (16, 8, {6: 321, 7: 9})])
def test_music_multilevel_noise_matches_oracle(mfxlib, engine, oracle, n, cubesize, seeds):
    """Seeds at coarser levels: the coarsest seeded level refined up to the
    grid's by coarse mode replacement, unseeded levels with their dummy seeds
    (random_music.cc:222-245, random_music_wnoise_generator.cc:392-547).  Seeds
    only at finer levels: the coarsest of them restricted down by k-space
    averaging (random_music.cc:247-272, random_music_wnoise_generator.cc:288-380)."""
    c = Case(mfxlib, n, 100.0, 49.0, 1, 1)
    j = mfxlib.Job(engine, n, c.L, 1, None, c.amp, c.coef, precision=mfxlib.FP64, want_particles=False,
                   noise_generator=mfxlib.NOISE_MUSIC1, music_cubesize=cubesize, music_seeds=seeds)
    j.run_noise(raw=True)
    got = j.field(mfxlib.FIELD_NOISE)
    ref = oracle.fft_r2c(oracle.music_levels(n, seeds, cubesize))
    ref[0, 0, 0] = 0.0
    assert rel_l2(got, ref) < 1e-12
    # the coarsest level's modes come through to the grid's noise
    lo = min(seeds)
    assert np.abs(got[1, 1, 1]) > 0


def test_run_config_music1_multilevel(mfxlib, engine, tmp_path):
    f = tmp_path / "ics.bin"
    txt = mfxlib.ini_text(32, 50.0, 24.0, 2, 777, "sc", filename=str(f), generator="MUSIC1", cubesize=8)
    engine.run_config(txt.replace("seed[5] = 777", "seed[3] = 31\nseed[5] = 777"))
    raw = f.read_bytes()
    np_ = int(np.frombuffer(raw[8:16], np.uint64)[0])
    c = Case(mfxlib, 32, 50.0, 24.0, 2, 1)
    j = mfxlib.Job(engine, 32, c.L, 2, None, c.amp, c.coef, precision=mfxlib.FP64, lunit=c.lunit, vunit=c.vunit,
                   noise_generator=mfxlib.NOISE_MUSIC1, music_cubesize=8, music_seeds={3: 31, 5: 777})
    j.run()
    pos, vel, ids = j.particles()
    off = 8 + 8 + 4 + 4 + 24
    assert np.array_equal(np.frombuffer(raw[off:off + 24 * np_], np.float64).reshape(-1, 3), pos)


def test_noise_field_matches_oracle(mfxlib, engine, oracle):
    """A white-noise field given in real space (MFX_NOISE_FIELD): its unitary
    forward transform, the mean kept in the raw noise (zeroed in phi(1))."""
    n = 32
    rng = np.random.default_rng(17)
    field = rng.standard_normal((n, n, n)) + 0.01
    c = Case(mfxlib, n, 100.0, 49.0, 2, 1)
    j = mfxlib.Job(engine, n, c.L, 2, None, c.amp, c.coef, precision=mfxlib.FP64, lunit=c.lunit, vunit=c.vunit,
                   noise_field=field)
    j.run_noise(raw=True)
    ref = oracle.fft_r2c(field)
    assert rel_l2(j.field(mfxlib.FIELD_NOISE), ref) < 1e-13
    j.run()
    res = oracle.run_lpt(n, c.L, None, c.amplitude, 2, c.dplus, c.vfac, lunit=c.lunit, vunit=c.vunit, noise=ref)
    check_fields(mfxlib, j, res, 2, TOL_FP64)
    check_particles(c, j, res, TOL_FP64)


def test_run_config_music1_noise_file(mfxlib, engine, tmp_path):
    """[random] seed[log2 GridRes] = <file>: the grafic white noise read by the
    driver (negated unless grafic_sign), the same particles as a job given the
    field."""
    from test_cpu import write_grafic
    n = 32
    rng = np.random.default_rng(5)
    field = rng.standard_normal((n, n, n))
    wn = tmp_path / "wn.bin"
    write_grafic(wn, field)
    f = tmp_path / "ics.bin"
    txt = mfxlib.ini_text(n, 50.0, 24.0, 2, 777, "sc", filename=str(f), generator="MUSIC1")
    engine.run_config(txt.replace("seed[5] = 777", "seed[5] = %s" % wn))
    raw = f.read_bytes()
    np_ = int(np.frombuffer(raw[8:16], np.uint64)[0])
    c = Case(mfxlib, n, 50.0, 24.0, 2, 1)
    j = mfxlib.Job(engine, n, c.L, 2, None, c.amp, c.coef, precision=mfxlib.FP64, lunit=c.lunit, vunit=c.vunit,
                   noise_field=field.astype(np.float32).astype(np.float64))
    j.run()
    pos, vel, ids = j.particles()
    off = 8 + 8 + 4 + 4 + 24
    assert np.array_equal(np.frombuffer(raw[off:off + 24 * np_], np.float64).reshape(-1, 3), pos)


@pytest.mark.parametrize("n,cubesize,res,seeds", [(32, 8, 8, {4: 77}), (32, 8, 16, {}), (16, 4, 2, {3: 5, 4: 6})])
def test_music_noise_file_at_coarser_level(mfxlib, engine, oracle, n, cubesize, res, seeds):
    """A noise file at a level coarser than the grid's starts the refinement
    chain (random_music.cc:216-236): its values as read (mean kept), each
    finer level refining it with its seed or the level's dummy seed."""
    rng = np.random.default_rng(n + res)
    field = rng.standard_normal((res, res, res)) + 0.05
    c = Case(mfxlib, n, 100.0, 49.0, 1, 1)
    j = mfxlib.Job(engine, n, c.L, 1, None, c.amp, c.coef, precision=mfxlib.FP64, want_particles=False,
                   noise_generator=mfxlib.NOISE_MUSIC1, music_cubesize=cubesize, music_seeds=seeds,
                   noise_field=field)
    j.run_noise(raw=True)
    got = j.field(mfxlib.FIELD_NOISE)
    ref = oracle.fft_r2c(oracle.music_levels(n, seeds, cubesize, field=field))
    assert rel_l2(got, ref) < 1e-12
    assert abs(got[0, 0, 0]) > 0  # the file's mean comes through
    j.run_noise(raw=True)  # a second run reads the field again
    assert np.array_equal(j.field(mfxlib.FIELD_NOISE), got)
    j.close()
    with pytest.raises(mfxlib.MfxError, match="noise field"):
        mfxlib.Job(engine, n, c.L, 1, None, c.amp, c.coef, precision=mfxlib.FP64, want_particles=False,
                   noise_generator=mfxlib.NOISE_MUSIC1, music_cubesize=cubesize,
                   music_seeds={**seeds, int(res).bit_length() - 1: 9}, noise_field=field)


def test_run_config_music1_noise_file_at_coarser_level(mfxlib, engine, tmp_path):
    """[random] seed[3] = <file> with seed[5] on a 32^3 grid: the file's noise
    refined up to the grid's level, the same particles as a job given the
    field and the seed."""
    from test_cpu import write_grafic
    rng = np.random.default_rng(9)
    field = rng.standard_normal((8, 8, 8))
    wn = tmp_path / "wn8.bin"
    write_grafic(wn, field)
    f = tmp_path / "ics.bin"
    txt = mfxlib.ini_text(32, 50.0, 24.0, 2, 777, "sc", filename=str(f), generator="MUSIC1", cubesize=8)
    engine.run_config(txt.replace("seed[5] = 777", "seed[3] = %s\nseed[5] = 777" % wn))
    raw = f.read_bytes()
    np_ = int(np.frombuffer(raw[8:16], np.uint64)[0])
    c = Case(mfxlib, 32, 50.0, 24.0, 2, 1)
    j = mfxlib.Job(engine, 32, c.L, 2, None, c.amp, c.coef, precision=mfxlib.FP64, lunit=c.lunit, vunit=c.vunit,
                   noise_generator=mfxlib.NOISE_MUSIC1, music_cubesize=8, music_seeds={5: 777},
                   noise_field=field.astype(np.float32).astype(np.float64))
    j.run()
    pos, vel, ids = j.particles()
    off = 8 + 8 + 4 + 4 + 24
    assert np.array_equal(np.frombuffer(raw[off:off + 24 * np_], np.float64).reshape(-1, 3), pos)
    j.close()
    # a file above a coarser seed is ignored (the reference warns and goes on)
    g = tmp_path / "ics2.bin"
    txt2 = mfxlib.ini_text(32, 50.0, 24.0, 2, 777, "sc", filename=str(g), generator="MUSIC1", cubesize=8)
    engine.run_config(txt2.replace("seed[5] = 777", "seed[3] = 31\nseed[4] = %s\nseed[5] = 777" % wn))
    h = tmp_path / "ics3.bin"
    txt3 = mfxlib.ini_text(32, 50.0, 24.0, 2, 777, "sc", filename=str(h), generator="MUSIC1", cubesize=8)
    engine.run_config(txt3.replace("seed[5] = 777", "seed[3] = 31\nseed[5] = 777"))
    assert g.read_bytes() == h.read_bytes()
