"""Baryon + CDM runs (ic_generator.cc:706-1064 with DoBaryons and DoBaryonVrel):
both species from the potentials of one run, through mfx_job_set_species and
mfx_job_assemble, against the oracle's two-species restatement
(oracle/lpt.py species_particles).

The E&H transfer function gives delta_bc = theta_bc = 0 (transfer_eisenstein.cc
compute() returns 0 for both), which would leave the masses unperturbed and the
relative-velocity term empty; the tests therefore feed smooth synthetic
delta_bc / theta_bc amplitude tables (5% and 1% of the matter amplitude), as a
transfer-function plugin that provides them (CLASS) would.
"""
import numpy as np
import pytest

from test_gpu_parity import Case, TOL_FP64, lattice_q, rel_l2

pytestmark = pytest.mark.gpu

OM, OB = 0.3, 0.045
FB = OB / OM
# (secondary lattice, IDoffset, C factor, Omega): ic_generator.cc:718-739, 158-166
SPECIES = {"dm": (False, 0, -FB, OM - OB), "baryon": (True, 1, 1.0 - FB, OB)}
SECOND = {0: (0.5, 0.5, 0.5), 1: (0.5, 0.5, 0.0), 2: (0.5, 0.5, 0.5)}


def synthetic_tables(c):
    kf = 2.0 * np.pi / c.L
    q = np.arange(len(c.amp), dtype=np.float64)
    amplitude = c.amp * (kf * kf * q)  # the amplitude table holds amplitude / k^2
    return 0.05 * amplitude, 0.01 * amplitude


@pytest.mark.parametrize("n,lattice,plt,precision,noise", [(32, 1, True, "fp64", "ngenic"), (24, 0, False, "fp64", "ngenic"),
                                                           (32, 2, True, "fp64", "ngenic"), (32, 1, True, "fp32c", "ngenic"),
                                                           (32, 2, True, "fp64", "music"), (32, 1, False, "fp64", "music")])
def test_baryon_and_cdm_species_match_oracle(mfxlib, engine, oracle, n, lattice, plt, precision, noise):
    """With MUSIC1 noise the Nyquist planes carry modes: the secondary
    lattice's global shift is one more shift_field step before the
    sub-lattice steps, whose projections the masses and particles follow."""
    from oracle import lpt, plt as oplt
    tab = engine.plt_table(lattice) if plt else None
    c = Case(mfxlib, n, 300.0, 24.0, 3, 4242, lattice=lattice, plt=tab)
    prec = mfxlib.FP64 if precision == "fp64" else mfxlib.FP32C
    if noise == "music":
        j = mfxlib.Job(engine, n, c.L, 3, None, c.amp, c.coef, lattice=lattice, precision=prec, plt_table=tab,
                       lunit=c.lunit, vunit=c.vunit, noise_generator=mfxlib.NOISE_MUSIC1, music_seed=808,
                       music_cubesize=8)
        j.run()
        w = oracle.music_fill(n, 808, 8)
        w[0, 0, 0] = 0.0
        res = oracle.run_lpt(n, c.L, None, c.amplitude, 3, c.dplus, c.vfac, lattice=lattice, lunit=c.lunit,
                             vunit=c.vunit, want_particles=False, noise=w)
    else:
        j = c.job(mfxlib, engine, precision=prec)
        j.run()
        res = c.oracle(oracle, want_particles=False)
    grad = oplt.PLTGradient(n, c.L, tab) if plt else lpt.FourierGradient(n, c.L)
    fields = (res["phi"], res["phi2"], res["phi3"], res["A3"])
    dbc, tbc = synthetic_tables(c)
    delta = c.L / (n * 2 ** (lattice / 3.0))
    ns = 1 << lattice
    for name, (sec, idoff, cs, om) in SPECIES.items():
        j.set_species(secondary=sec, id_offset=idoff, c_species=cs, mass_factor=om, amp_dbc=dbc, amp_tbc=tbc)
        j.assemble(7)
        pos, vel, ids = j.particles()
        mass = j.masses()
        rp, rv, rid, rm = oracle.species_particles(fields, res["noise"], res["coef"], grad, lattice, n, c.L, c.lunit,
                                                   c.vunit, 3, cs, om, amp_dbc=dbc, amp_tbc=tbc, secondary=sec,
                                                   id_offset=idoff)
        q = lattice_q(n, lattice, c.lunit)
        if sec:
            q = q + np.array(SECOND[lattice]) / n * c.lunit
        m0 = om / (ns * n ** 3)
        assert np.array_equal(ids, rid), name
        if precision == "fp64":
            assert rel_l2(pos - q, rp - q) < TOL_FP64, name
            assert rel_l2(vel, rv) < TOL_FP64, name
            assert rel_l2(mass - m0, rm - m0) < TOL_FP64, name
        else:
            assert np.sqrt(np.mean(((pos - rp) / delta) ** 2)) < 1e-5, name
            assert rel_l2(vel.astype(np.float64), rv) < 1e-5, name
            assert rel_l2(mass.astype(np.float64) - m0, rm - m0) < 1e-5, name
        # the perturbations are there: masses vary, the relative-velocity term moves v
        assert np.std(rm) > 1e-3 * m0
    # back to the descriptor's single species: the plain run's particles again
    j.set_species(reset=True)
    j.assemble(7)
    p1, v1, i1 = j.particles()
    ref = oracle.particles(fields, res["coef"], grad, lattice, n, c.L, c.lunit, c.vunit, 3)
    if precision == "fp64":
        assert rel_l2(p1 - lattice_q(n, lattice, c.lunit), ref[0] - lattice_q(n, lattice, c.lunit)) < TOL_FP64
        assert rel_l2(v1, ref[1]) < TOL_FP64
    assert np.array_equal(i1, ref[2])
    j.close()


def test_species_without_tables_gives_unperturbed_masses(mfxlib, engine, oracle):
    """With E&H (delta_bc = theta_bc = 0): masses Omega_species / (n_s N^3),
    velocities of the plain run, baryons on the secondary lattice."""
    c = Case(mfxlib, 16, 100.0, 24.0, 2, 7, lattice=1)
    j = c.job(mfxlib, engine)
    j.run()
    p0, v0, _ = j.particles()
    sec, idoff, cs, om = SPECIES["baryon"]
    j.set_species(secondary=sec, id_offset=idoff, c_species=cs, mass_factor=om)
    j.assemble(7)
    pos, vel, ids = j.particles()
    m = j.masses()
    assert np.allclose(m, om / (2 * 16 ** 3), rtol=1e-15, atol=0)
    assert rel_l2(vel, v0) > 1e-6  # read out on the shifted lattice
    assert ids.min() == 2 * 16 ** 3  # IDoffset 1: ids start after the first species'
    j.close()


def test_species_errors(mfxlib, engine):
    c = Case(mfxlib, 16, 100.0, 24.0, 1, 7)
    j = c.job(mfxlib, engine)
    with pytest.raises(mfxlib.MfxError):
        j.masses()  # no species with masses yet
    with pytest.raises(mfxlib.MfxError):
        j.set_species(amp_dbc=np.zeros(5))  # table too short
    j.close()


def test_run_config_with_baryons_writes_both_species(mfxlib, engine, tmp_path):
    """[setup] DoBaryons = yes through the C++ driver: one file per species, the
    baryons on the secondary lattice with IDoffset 1, masses Omega_species /
    (n_s N^3) (E&H has no delta_bc), positions of the same displacement field."""
    f = tmp_path / "ics.bin"
    n, L = 16, 50.0
    txt = mfxlib.ini_text(n, L, 24.0, 2, 3, "bcc", filename=str(f)).replace("[setup]", "[setup]\nDoBaryons = yes")
    engine.run_config(txt)
    out = {}
    for name, path in (("dm", f), ("baryon", tmp_path / "ics.bin.baryon")):
        raw = path.read_bytes()
        assert raw[:8] == b"MFXIC002"
        np_ = int(np.frombuffer(raw[8:16], np.uint64)[0])
        assert np_ == 2 * n ** 3
        off = 8 + 8 + 4 + 4 + 24
        pos = np.frombuffer(raw[off:off + 24 * np_], np.float64).reshape(-1, 3)
        ids = np.frombuffer(raw[off + 48 * np_:off + 56 * np_], np.uint64)
        mass = np.frombuffer(raw[off + 56 * np_:off + 64 * np_], np.float64)
        out[name] = (pos, ids, mass)
    assert np.allclose(out["dm"][2], (OM - OB) / (2 * n ** 3), rtol=1e-14, atol=0)
    assert np.allclose(out["baryon"][2], OB / (2 * n ** 3), rtol=1e-14, atol=0)
    assert out["dm"][1].min() == 0 and out["baryon"][1].min() == 2 * n ** 3
    # the baryons sit half a cell along x and y from the CDM particles (BCC secondary shift)
    d = out["baryon"][0] - out["dm"][0]
    d -= L * np.round(d / L)
    assert np.allclose(np.median(d, axis=0), [0.5 * L / n, 0.5 * L / n, 0.0], atol=0.05 * L / n)
