"""Semiclassical (PPT) Eulerian fields (ic_generator.cc:783-901) through
mfx_job_ppt_fields, against the oracle's restatement (oracle/lpt.py
ppt_fields): the density contrast and the three velocity fields within 1e-10
relative (L2) and hbar to rounding for the plain FP64 form; the FP32 form's
potentials give the same fields to its precision."""
import numpy as np
import pytest

from test_gpu_parity import Case, TOL_FP64, rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,order,lattice,species", [(32, 2, 0, False), (48, 1, 0, False), (32, 3, 1, True),
                                                     (64, 2, 0, True)])
def test_ppt_fields_match_oracle(mfxlib, engine, oracle, n, order, lattice, species):
    c = Case(mfxlib, n, 200.0, 49.0, order, 12345, lattice=lattice)
    res = c.oracle(oracle, want_particles=False)
    cs, dbc = 0.0, None
    if species:
        kf = 2.0 * np.pi / c.L
        q = np.arange(len(c.amp), dtype=np.float64)
        dbc = 0.05 * c.amp * (kf * kf * q)
        cs = 1.0 - 0.045 / 0.3
    ref = oracle.ppt_fields(res["phi"], res["phi2"], res["noise"], order, n, c.L, c.dplus, c.coef["vfac1"], c.vunit,
                            c_species=cs, amp_dbc=dbc)
    for prec, tol in ((mfxlib.FP64, TOL_FP64), (mfxlib.FP32C, 2e-4)):
        j = c.job(mfxlib, engine, precision=prec, want_particles=False)
        j.run()
        delta, vel, hbar = j.ppt_fields(c_species=cs, amp_dbc=dbc)
        j.close()
        assert abs(hbar - ref[2]) <= (1e-12 if prec == mfxlib.FP64 else 1e-5) * ref[2]
        assert rel_l2(delta, ref[0]) < tol, (prec, rel_l2(delta, ref[0]))
        for d in range(3):
            assert rel_l2(vel[d], ref[1][d]) < tol, (prec, d, rel_l2(vel[d], ref[1][d]))
    # a density contrast and a flow are there
    assert np.std(ref[0]) > 1e-3 and np.std(ref[1][0]) > 0


def test_ppt_needs_potentials(mfxlib, engine):
    c = Case(mfxlib, 16, 100.0, 49.0, 2, 3)
    j = c.job(mfxlib, engine, want_particles=False)
    with pytest.raises(mfxlib.MfxError):
        j.ppt_fields()
    j.close()


def test_ppt_fields_with_music1_noise(mfxlib, engine, oracle):
    """MUSIC1 noise fills the Nyquist planes the PPT fields' transforms see."""
    n, order = 32, 2
    c = Case(mfxlib, n, 200.0, 49.0, order, 1)
    w = oracle.music_fill(n, 4321, 8)
    w[0, 0, 0] = 0.0
    res = oracle.run_lpt(n, c.L, None, c.amplitude, order, c.dplus, c.vfac, lunit=c.lunit, vunit=c.vunit,
                         want_particles=False, noise=w)
    ref = oracle.ppt_fields(res["phi"], res["phi2"], res["noise"], order, n, c.L, c.dplus, c.coef["vfac1"], c.vunit)
    j = mfxlib.Job(engine, n, c.L, order, None, c.amp, c.coef, precision=mfxlib.FP64, want_particles=False,
                   lunit=c.lunit, vunit=c.vunit, noise_generator=mfxlib.NOISE_MUSIC1, music_seed=4321,
                   music_cubesize=8)
    j.run()
    delta, vel, hbar = j.ppt_fields()
    j.close()
    assert abs(hbar - ref[2]) <= 1e-12 * ref[2]
    assert rel_l2(delta, ref[0]) < TOL_FP64
    for d in range(3):
        assert rel_l2(vel[d], ref[1][d]) < TOL_FP64
