"""GPU parity tests: the CUDA engine (through the C ABI) against the oracle.

FP64 plain form: the white-noise integer stream bit-exact, every field and the
particle displacements / velocities within 1e-10 relative (L2) of the FP64
oracle.  FP32-compensated form: rms displacement error <= 1e-5 of the mean
interparticle spacing.
"""
import pathlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = pathlib.Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"

TOL_FP64 = 1e-10  # L2-relative bar of the plain FP64 form


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


class Case:
    """Scalars and tables of one job, built by the product's host library."""

    def __init__(self, mfx, n, L, z, order, seed, lattice=0, fixing=False, inversion=False, plt=None):
        self.n, self.L, self.z, self.order, self.lattice = n, L, z, order, lattice
        lat = {0: "sc", 1: "bcc", 2: "fcc"}[lattice]
        self.cosmo = mfx.Cosmology(mfx.ini_text(n, L, z, order, seed, lat, fixing=fixing))
        self.dplus = self.cosmo.get("dplus_start")
        self.vfac = self.cosmo.get("vfact_start")
        self.seeds = mfx.ngenic_seed_table(seed, n)
        self.amp = self.cosmo.amp_table(n, L)
        self.coef = mfx.lpt_coefficients(self.dplus, self.vfac, order)
        self.fixing, self.inversion = fixing, inversion
        self.plt = plt
        self.lunit = L
        self.vunit = L / np.sqrt(1.0 / (1.0 + z))

    def job(self, mfx, engine, precision=None, **kw):
        precision = mfx.FP64 if precision is None else precision
        return mfx.Job(engine, self.n, self.L, self.order, self.seeds, self.amp, self.coef, lattice=self.lattice,
                       precision=precision, plt_table=self.plt, fixing=self.fixing, inversion=self.inversion,
                       lunit=self.lunit, vunit=self.vunit, **kw)

    def amplitude(self, kmod):
        out = self.cosmo.amplitude(kmod.ravel())
        return out.reshape(kmod.shape)

    def oracle(self, oracle, want_particles=True):
        grad = None
        if self.plt is not None:
            from oracle import plt as oplt
            grad = oplt.PLTGradient(self.n, self.L, self.plt)
        return oracle.run_lpt(self.n, self.L, self.seeds, self.amplitude, self.order, self.dplus, self.vfac,
                              lattice=self.lattice, lunit=self.lunit, vunit=self.vunit, fixing=self.fixing,
                              inversion=self.inversion, grad=grad, want_particles=want_particles)


def lattice_q(n, lattice, lunit):
    """Unperturbed positions (particle_generator.hh:529-531)."""
    from oracle.lpt import LATTICE_SHIFTS
    out = []
    idx = np.arange(n, dtype=np.float64)
    for s in LATTICE_SHIFTS[lattice]:
        g = [((idx + s[a]) / float(n)) * lunit for a in range(3)]
        X, Y, Z = np.meshgrid(*g, indexing="ij")
        out.append(np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1))
    return np.concatenate(out)


# ---------------------------------------------------------------------------
# white noise
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("seed", [1, 12345, 4242, 0x7ffffffe])
def test_device_ranlux_stream_bit_exact(engine, oracle, seed):
    got = engine.ranlxd1_words(seed, 3000)
    assert np.array_equal(got, oracle.ranlxd1_words(seed, 3000))


def test_device_ranlux_matches_gsl_known_answer(engine):
    """GSL's published ranlxd1 value (rng/test.c: seed 1, 10000th draw of
    gsl_rng_get = 1998227290, i.e. the top 32 bits of the 48-bit word)."""
    w = int(engine.ranlxd1_words(1, 10000)[-1])
    assert w >> 16 == 1998227290


def test_device_ranlux_on_seed_table_entries(mfxlib, engine, oracle):
    t = mfxlib.ngenic_seed_table(12345, 32)
    for s in t[[0, 5, 100, 1023]]:
        assert np.array_equal(engine.ranlxd1_words(int(s), 800), oracle.ranlxd1_words(int(s), 800))


@pytest.mark.parametrize("n", [16, 64])
def test_noise_matches_oracle(mfxlib, engine, oracle, n):
    c = Case(mfxlib, n, 100.0, 49.0, 1, 12345)
    j = c.job(mfxlib, engine, want_particles=False)
    j.run_noise(raw=True)
    got = j.field(mfxlib.FIELD_NOISE)
    ref = oracle.ngenic_fill(n, c.seeds)
    assert np.array_equal(got == 0, ref == 0)  # same zero pattern (Nyquist, DC)
    assert np.max(np.abs(got - ref)) < 1e-13
    p = got[:, :, 0]
    idx = (-np.arange(n)) % n
    assert np.array_equal(p[np.ix_(idx, idx)], np.conj(p))  # exact Hermitian k=0 plane


def test_noise_golden(mfxlib, engine):
    g = np.load(GOLDEN / "ngenic_16.npz")
    c = Case(mfxlib, 16, 100.0, 49.0, 1, int(g["seed"]))
    assert np.array_equal(c.seeds, g["seed_table"])
    j = c.job(mfxlib, engine, want_particles=False)
    j.run_noise(raw=True)
    assert np.max(np.abs(j.field(mfxlib.FIELD_NOISE) - g["noise"])) < 1e-13


@pytest.mark.parametrize("fixing,inversion", [(True, False), (False, True), (True, True)])
def test_noise_normalisation_fixing_inversion(mfxlib, engine, oracle, fixing, inversion):
    n, L = 32, 300.0
    c = Case(mfxlib, n, L, 24.0, 1, 99, fixing=fixing, inversion=inversion)
    j = c.job(mfxlib, engine, want_particles=False)
    j.run_noise(raw=False)
    ref = oracle.normalise_noise(oracle.ngenic_fill(n, c.seeds), n, L, fixing, inversion)
    assert rel_l2(j.field(mfxlib.FIELD_NOISE), ref) < 1e-14


# ---------------------------------------------------------------------------
# LPT potentials and particles, plain FP64 form
# ---------------------------------------------------------------------------
def check_fields(mfxlib, j, res, order, tol=TOL_FP64):
    g = res["coef"]
    assert rel_l2(j.field(mfxlib.FIELD_PHI1) * g["g1"], res["phi"]) < tol
    if order > 1:
        assert rel_l2(j.field(mfxlib.FIELD_PHI2) * g["g2"], res["phi2"]) < tol
    if order > 2:
        assert rel_l2(j.field(mfxlib.FIELD_PHI3) * g["g3"], res["phi3"]) < tol
        for d, fid in enumerate((mfxlib.FIELD_A3X, mfxlib.FIELD_A3Y, mfxlib.FIELD_A3Z)):
            assert rel_l2(j.field(fid) * g["g3c"], res["A3"][d]) < tol


def check_particles(c, j, res, tol=TOL_FP64):
    pos, vel, ids = j.particles()
    q = lattice_q(c.n, c.lattice, c.lunit)
    psi_ref = res["pos"] - q
    assert rel_l2(pos - q, psi_ref) < tol
    assert rel_l2(vel, res["vel"]) < tol
    assert np.array_equal(ids, res["ids"])


def test_config1_2lpt_sc_64(mfxlib, engine, oracle):
    """2LPT, 64^3 SC, L = 100 Mpc/h, z = 49, seed 12345, no PLT, FP64."""
    c = Case(mfxlib, 64, 100.0, 49.0, 2, 12345)
    j = c.job(mfxlib, engine)
    j.run()
    res = c.oracle(oracle)
    check_fields(mfxlib, j, res, 2)
    check_particles(c, j, res)


@pytest.mark.parametrize("lattice", [0, 1, 2])
def test_3lpt_fp64_lattices_32(mfxlib, engine, oracle, lattice):
    c = Case(mfxlib, 32, 300.0, 24.0, 3, 4242, lattice=lattice)
    j = c.job(mfxlib, engine)
    j.run()
    res = c.oracle(oracle)
    check_fields(mfxlib, j, res, 3)
    check_particles(c, j, res)


def test_1lpt_fp64_fixing_48(mfxlib, engine, oracle):
    c = Case(mfxlib, 48, 200.0, 30.0, 1, 77, fixing=True)
    j = c.job(mfxlib, engine)
    j.run()
    res = c.oracle(oracle)
    check_fields(mfxlib, j, res, 1)
    check_particles(c, j, res)


def test_golden_lpt_16(mfxlib, engine):
    """Engine against the committed oracle fixture (16^3 3LPT SC)."""
    from oracle import cosmo
    g = np.load(GOLDEN / "lpt_16.npz")
    n, L = int(g["n"]), float(g["L"])
    o = cosmo.Cosmology(Om=0.3, Ob=0.045, H0=70.0, n_s=0.965, sigma8=0.81)
    kf = 2 * np.pi / L
    nn = np.arange(3 * (n // 2) ** 2 + 1)
    with np.errstate(divide="ignore", invalid="ignore"):
        k = kf * np.sqrt(nn)
        amp = np.where(nn > 0, o.amplitude(k) / (k * k), 0.0)
    seeds = np.load(GOLDEN / "ngenic_16.npz")["seed_table"]
    coef = mfxlib.lpt_coefficients(float(g["dplus"]), float(g["vfac"]), 3)
    j = mfxlib.Job(engine, n, L, 3, seeds, amp, coef, lunit=L, vunit=L)
    j.run()
    assert rel_l2(j.field(mfxlib.FIELD_PHI1), g["phi"]) < 1e-12
    assert rel_l2(j.field(mfxlib.FIELD_PHI2), g["phi2"]) < TOL_FP64
    assert rel_l2(j.field(mfxlib.FIELD_PHI3), g["phi3"]) < TOL_FP64
    pos, vel, ids = j.particles()
    q = lattice_q(n, 0, L)
    assert rel_l2(pos - q, g["pos"] - q) < TOL_FP64
    assert rel_l2(vel, g["vel"]) < TOL_FP64
    assert np.array_equal(ids, g["ids"])


# ---------------------------------------------------------------------------
# PLT
# ---------------------------------------------------------------------------
_PLT_CACHE = {}


def oracle_plt(lattice):
    if lattice not in _PLT_CACHE:
        from oracle import plt as oplt
        _PLT_CACHE[lattice] = oplt.plt_tables(lattice)
    return _PLT_CACHE[lattice]


@pytest.mark.parametrize("lattice", [1, 2])
def test_plt_tables_match_oracle(engine, lattice):
    got = engine.plt_table(lattice)
    ref = oracle_plt(lattice)
    assert np.all(np.isfinite(got))
    assert np.array_equal(got[0], ref[0])
    # eigensolvers differ (Jacobi vs LAPACK): identical up to rounding except at
    # isolated modes with a degenerate leading eigenvalue
    for t in (1, 2, 3):
        d = np.abs(got[t] - ref[t])
        assert np.median(d) < 1e-12
        assert np.mean(d > 1e-9) < 1e-3


@pytest.mark.parametrize("lattice", [1, 2])
def test_3lpt_plt_fp64_32(mfxlib, engine, oracle, lattice):
    tab = engine.plt_table(lattice)
    c = Case(mfxlib, 32, 300.0, 24.0, 3, 4242, lattice=lattice, plt=tab)
    j = c.job(mfxlib, engine)
    j.run()
    res = c.oracle(oracle)
    check_fields(mfxlib, j, res, 3)
    check_particles(c, j, res)


# ---------------------------------------------------------------------------
# FP32-compensated form
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("lattice,fixing,L", [(1, False, 300.0), (2, True, 1000.0 * 64 / 768)])
def test_fp32c_error_in_interparticle_spacing(mfxlib, engine, oracle, lattice, fixing, L):
    """FP32 form (fused transforms and assembly) against the FP64 oracle: the
    256^3 BCC and the amplitude-fixed 768^3 FCC configurations' physics at 64^3."""
    tab = engine.plt_table(lattice)
    c = Case(mfxlib, 64, L, 24.0, 3, 4242, lattice=lattice, fixing=fixing, plt=tab)
    j = c.job(mfxlib, engine, precision=mfxlib.FP32C, pos64=True, vel64=False)
    j.run()
    res = c.oracle(oracle)
    pos, vel, ids = j.particles()
    delta = c.L / (c.n * 2 ** (lattice / 3.0))  # mean interparticle spacing (box units x lunit = Mpc/h)
    err = (pos - res["pos"]) / delta
    rms = np.sqrt(np.mean(err ** 2))
    assert rms < 1e-5, rms
    assert np.max(np.abs(err)) < 2e-4
    assert rel_l2(vel.astype(np.float64), res["vel"]) < 1e-5
    assert np.array_equal(ids, res["ids"])


@pytest.mark.parametrize("lattice", [0, 1])
def test_plt_interpolated_128_fp64_and_fp32(mfxlib, engine, oracle, lattice):
    """N > 64: the PLT tables are CIC-interpolated between nodes, including the
    table's Nyquist node; both forms must agree with the oracle."""
    tab = engine.plt_table(lattice)
    c = Case(mfxlib, 128, 300.0, 24.0, 3, 4242, lattice=lattice, plt=tab)
    res = c.oracle(oracle)
    j = c.job(mfxlib, engine)
    j.run()
    check_particles(c, j, res)
    j.close()
    j = c.job(mfxlib, engine, precision=mfxlib.FP32C)
    j.run()
    pos, vel, _ = j.particles()
    delta = c.L / (c.n * 2 ** (lattice / 3.0))
    assert np.sqrt(np.mean(((pos - res["pos"]) / delta) ** 2)) < 1e-6
    assert rel_l2(vel, res["vel"]) < 2e-6


@pytest.mark.parametrize("n,lattice,order", [(32, 1, 3), (64, 2, 3), (96, 0, 2), (128, 0, 3), (192, 1, 2)])
def test_fused_transforms_match_cufft_path(mfxlib, engine, n, lattice, order, monkeypatch):
    """FP32 form: the pruned, fused padded transforms against the cuFFT path of
    the same form (both FP32), field by field, and the autotuner's choice."""
    tab = engine.plt_table(lattice) if lattice else None
    c = Case(mfxlib, n, 300.0, 24.0, order, 77, lattice=lattice, plt=tab)
    fids = [mfxlib.FIELD_PHI1, mfxlib.FIELD_PHI2] + ([mfxlib.FIELD_PHI3, mfxlib.FIELD_A3X, mfxlib.FIELD_A3Y,
                                                       mfxlib.FIELD_A3Z] if order > 2 else [])
    monkeypatch.setenv("MFX_FUSED", "1")
    j = c.job(mfxlib, engine, precision=mfxlib.FP32C)
    pxy, pz = j.autotune()
    assert pxy in (4, 8, 16, 32) and pz in (1, 2, 3, 4)
    j.run()
    fused = [j.field(f) for f in fids]
    pf = j.particles()
    j.close()
    monkeypatch.setenv("MFX_FUSED", "0")
    j = c.job(mfxlib, engine, precision=mfxlib.FP32C)
    j.run()
    ref = [j.field(f) for f in fids]
    pr = j.particles()
    j.close()
    for a, b in zip(fused, ref):
        assert rel_l2(a, b) < 5e-6
    # particles: fused assembly (own x/y/z passes) against cuFFT's c2r + read-out
    delta = c.L / (c.n * 2 ** (lattice / 3.0))
    assert np.sqrt(np.mean(((pf[0] - pr[0]) / delta) ** 2)) < 1e-6
    assert rel_l2(pf[1].astype(np.float64), pr[1].astype(np.float64)) < 5e-6
    assert np.array_equal(pf[2], pr[2])


@pytest.mark.parametrize("n,lean,plain", [(192, 32, 8), (384, 16, 8), (384, 32, 8)])
def test_lean_xy_tiles_match_plain_tiles(mfxlib, engine, n, lean, plain, monkeypatch):
    """x/y tiles too wide for one butterfly per thread (lean form: a third as
    many threads, in-place transforms) give the fields and particles of the
    plain tiles to rounding; so do tiles whose two stages do not fit (384^3,
    32 pencils: the in-place form, input rows split between a side buffer and
    the tile, transformed in halves of 16 pencils)."""
    monkeypatch.setenv("MFX_FUSED", "1")
    c = Case(mfxlib, n, 300.0, 24.0, 3, 5, lattice=1, plt=engine.plt_table(1))
    fids = [mfxlib.FIELD_PHI2, mfxlib.FIELD_PHI3, mfxlib.FIELD_A3X, mfxlib.FIELD_A3Z]
    out = []
    for p in (lean, plain):
        j = c.job(mfxlib, engine, precision=mfxlib.FP32C)
        j.set_tiles(p, 1)
        j.run()
        out.append(([j.field(f) for f in fids], j.particles()))
        j.close()
    # FP32 rounding of the same sums (the A3 components carry the most cancellation)
    for f, a, b in zip(fids, out[0][0], out[1][0]):
        assert np.all(np.isfinite(a)) and rel_l2(a, b) < 5e-6, (f, rel_l2(a, b))
    delta = c.L / (c.n * 2 ** (1 / 3.0))
    assert np.sqrt(np.mean(((out[0][1][0] - out[1][1][0]) / delta) ** 2)) < 1e-7
    assert rel_l2(out[0][1][1], out[1][1][1]) < 1e-6


@pytest.mark.parametrize("n,lattice,order,plt", [(64, 2, 3, True), (96, 1, 2, False), (48, 2, 2, False)])
def test_fused_assembly_once_for_all_sublattices(mfxlib, engine, n, lattice, order, plt, monkeypatch):
    """Fused assembly: each mode assembled once and all sub-lattices emitted
    from it (tiles of 4 pencils, or of 8 in halves) gives the particles of the
    per-sub-lattice assembly."""
    tab = engine.plt_table(lattice) if plt else None
    c = Case(mfxlib, n, 300.0, 24.0, order, 99, lattice=lattice, plt=tab)
    monkeypatch.setenv("MFX_FUSED", "1")
    out = []
    # all sub-lattices from one assembly (tiles of 4), the same in halves
    # (tiles of 8, each half assembled on its own), one sub-lattice at a time
    for keep, halves in (("1", "0"), ("1", "1"), ("0", "0")):
        monkeypatch.setenv("MFX_FA_KEEP", keep)
        monkeypatch.setenv("MFX_FA_HALVES", halves)
        j = c.job(mfxlib, engine, precision=mfxlib.FP32C)
        j.run()
        out.append(j.particles())
        j.close()
    delta = c.L / (c.n * 2 ** (lattice / 3.0))
    for o in out[1:]:
        assert np.all(np.isfinite(o[0])) and np.all(np.isfinite(o[1]))
        assert np.sqrt(np.mean(((out[0][0] - o[0]) / delta) ** 2)) < 1e-7
        assert rel_l2(out[0][1].astype(np.float64), o[1].astype(np.float64)) < 1e-6
        assert np.array_equal(out[0][2], o[2])


@pytest.mark.parametrize("n,lattice", [(64, 2), (48, 2)])
def test_fused_rerun_is_identical(mfxlib, engine, n, lattice, monkeypatch):
    """A second run of the same job (the particle stage reuses the padded
    transforms' buffers in between) reproduces the first bit for bit, for every
    admissible tile shape."""
    monkeypatch.setenv("MFX_FUSED", "1")
    c = Case(mfxlib, n, 300.0, 24.0, 3, 4242, lattice=lattice, plt=engine.plt_table(lattice))
    fids = [mfxlib.FIELD_PHI2, mfxlib.FIELD_PHI3, mfxlib.FIELD_A3Y]
    first = None
    for pxy in (4, 8, 16, 32):
        for pz in (1, 2, 3, 4):
            j = c.job(mfxlib, engine, precision=mfxlib.FP32C)
            try:
                j.set_tiles(pxy, pz)
            except RuntimeError:
                j.close()
                continue
            j.run()
            a = [j.field(f) for f in fids] + [j.particles()[0]]
            j.run()
            b = [j.field(f) for f in fids] + [j.particles()[0]]
            j.close()
            for x, y in zip(a, b):
                assert np.all(np.isfinite(x)) and np.array_equal(x, y)
            if first is None:
                first = a
            for x, y in zip(a[:-1], first[:-1]):  # tiles change only the summation order
                assert rel_l2(x, y) < 1e-6


@pytest.mark.parametrize("lattice,id64", [(2, True), (1, False)])
def test_fetched_ids_follow_the_lattice_rule(mfxlib, engine, lattice, id64):
    """A fetch writes the ids of host destinations with host threads (a closed
    form of the particle index, particle_generator.hh:229-248) and copies those
    of device destinations from the device's array: both agree with the rule
    for an id offset, for ranges across sub-lattice boundaries and for the
    asynchronous fetch."""
    import torch
    n, off = 32, 5
    c = Case(mfxlib, n, 300.0, 24.0, 1, 4242, lattice=lattice)
    j = c.job(mfxlib, engine, precision=mfxlib.FP32C, id64=id64, id_offset=off)
    j.run()
    npart, n3 = j.num_particles, n ** 3
    ns = npart // n3
    p = np.arange(npart, dtype=np.uint64)
    want = np.uint64(off * ns * n3) + np.uint64(ns) * (p % np.uint64(n3)) + p // np.uint64(n3)
    want = want if id64 else want.astype(np.uint32)
    assert np.array_equal(j.particles()[2], want)
    first = n3 - 1000
    count = min(2 * n3 + 37, npart - first)  # across one (BCC) or two (FCC) sub-lattice boundaries
    assert np.array_equal(j.particles_range(first, count)[2], want[first:first + count])
    tdt = torch.int64 if id64 else torch.int32
    dev = torch.zeros(count, dtype=tdt, device="cuda")
    j.fetch_particles_range_into(first, count, None, None, dev.data_ptr())
    assert np.array_equal(dev.cpu().numpy().view(want.dtype), want[first:first + count])
    pinned = torch.zeros(count, dtype=tdt, pin_memory=True)
    j.fetch_particles_range_async(first, count, None, None, pinned.data_ptr())
    j.wait_fetch()
    assert np.array_equal(pinned.numpy().view(want.dtype), want[first:first + count])
    j.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_assemble_per_order_is_linear(mfxlib, engine, precision):
    """mfx_job_assemble: the displacements and velocities of the orders taken
    one at a time add up to those of the full assembly."""
    prec = mfxlib.FP64 if precision == "fp64" else mfxlib.FP32C
    c = Case(mfxlib, 32, 300.0, 24.0, 3, 4242, lattice=1, plt=engine.plt_table(1))
    j = c.job(mfxlib, engine, precision=prec)
    j.run()
    pos, vel, ids = j.particles()
    q = lattice_q(c.n, c.lattice, c.lunit)
    psi, v = np.zeros_like(pos), np.zeros_like(vel, dtype=np.float64)
    for m in (1, 2, 4):
        j.assemble(m)
        p, vv, ii = j.particles()
        assert np.array_equal(ii, ids)
        psi += p - q
        v += vv
    j.assemble(7)
    p7, v7, _ = j.particles()
    j.close()
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert rel_l2(psi, pos - q) < tol
    assert rel_l2(v, vel.astype(np.float64)) < tol
    assert np.array_equal(p7, pos) and np.array_equal(v7, vel)


# ---------------------------------------------------------------------------
# edge cases and errors
# ---------------------------------------------------------------------------
def test_smallest_grid_and_32bit_outputs(mfxlib, engine, oracle):
    c = Case(mfxlib, 8, 20.0, 49.0, 3, 5, lattice=2)
    j = c.job(mfxlib, engine, pos64=False, vel64=False, id64=False)
    j.run()
    res = c.oracle(oracle)
    pos, vel, ids = j.particles()
    assert pos.dtype == np.float32 and ids.dtype == np.uint32
    np.testing.assert_allclose(pos, res["pos"], rtol=0, atol=1e-5 * c.L)
    assert np.array_equal(ids.astype(np.uint64), res["ids"])


def test_invalid_descriptors_are_errors_not_faults(mfxlib, engine):
    c = Case(mfxlib, 16, 100.0, 49.0, 2, 1)
    for bad in ({"ngrid": 18}, {"lpt_order": 4}, {"lattice": 5}, {"boxlen": -1.0}):
        d = mfxlib.JobDesc()
        ref = c.job(mfxlib, engine).desc
        for f, _ in mfxlib.JobDesc._fields_:
            setattr(d, f, getattr(ref, f))
        for k, v in bad.items():
            setattr(d, k, v)
        import ctypes
        h = ctypes.c_void_p()
        rc = mfxlib.load().mfx_job_create(engine.handle, ctypes.byref(d), ctypes.byref(h))
        assert rc == mfxlib.MFX_EINVAL, (bad, rc)
    # short amplitude table
    with pytest.raises(mfxlib.MfxError):
        mfxlib.Job(engine, 16, 100.0, 2, c.seeds, c.amp[:10], c.coef)


def test_job_outliving_its_engine_is_released_cleanly(mfxlib):
    """Destroying an engine while a job on it is alive only marks it closing:
    the job stays usable and its destruction releases the engine."""
    eng = mfxlib.Engine(0)
    c = Case(mfxlib, 16, 100.0, 49.0, 2, 1)
    j = c.job(mfxlib, eng)
    j.run()
    eng.close()
    pos, vel, ids = j.particles()
    assert np.all(np.isfinite(pos)) and np.all(np.isfinite(vel))
    j.run()
    j.close()


def test_wait_timeout_is_bounded(mfxlib, engine):
    c = Case(mfxlib, 64, 100.0, 49.0, 3, 1)
    j = c.job(mfxlib, engine)
    j.run(wait=False)
    rc = mfxlib.load().mfx_job_wait(j.handle, 0)
    assert rc in (mfxlib.MFX_OK, mfxlib.MFX_ETIMEOUT)
    j.wait()


def test_rerun_is_deterministic(mfxlib, engine):
    c = Case(mfxlib, 32, 100.0, 24.0, 3, 11, lattice=1)
    j = c.job(mfxlib, engine)
    j.run()
    p1 = j.particles()
    j.run()
    p2 = j.particles()
    for a, b in zip(p1, p2):
        assert np.array_equal(a, b)


def test_run_config_end_to_end(mfxlib, engine, tmp_path):
    f = tmp_path / "ics.bin"
    txt = mfxlib.ini_text(16, 50.0, 24.0, 2, 3, "bcc", filename=str(f))
    engine.run_config(txt)
    raw = f.read_bytes()
    assert raw[:8] == b"MFXIC001"
    np_ = int(np.frombuffer(raw[8:16], np.uint64)[0])
    assert np_ == 2 * 16 ** 3
    c = Case(mfxlib, 16, 50.0, 24.0, 2, 3, lattice=1)
    j = c.job(mfxlib, engine)
    j.run()
    pos, vel, ids = j.particles()
    off = 8 + 8 + 4 + 4 + 24
    got_pos = np.frombuffer(raw[off:off + 24 * np_], np.float64).reshape(-1, 3)
    assert np.array_equal(got_pos, pos)
