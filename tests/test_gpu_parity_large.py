"""GPU parity at the large configurations.

* 3LPT + PLT on a BCC lattice at 256^3 (box 300 Mpc/h, z = 24, NGenIC seed
  4242), the plain FP64 form against the FP64 oracle: the noise, every
  potential and every particle within 1e-10 relative (L2), the ids exact.
* The same case in the FP32-compensated form against the oracle: rms
  displacement error <= 1e-5 of the mean interparticle spacing, for the full
  displacement and for each LPT order on its own.
* The kz = 0 (and kz = N/2) planes that the final c2r transforms receive: with
  the PLT gradient they are not exactly Hermitian; the relative size of the
  anti-Hermitian part bounds what any FFT pass order could change in the
  displacements and velocities.
* The pruned, fused padded transforms at the long padded lengths M = 768
  (N = 512) and M = 1152 (N = 768, the 768^3 configuration's length) against
  the cuFFT route of the same FP32 form.

The oracle's 256^3 run takes about half a minute on 16 cores and is shared by
the tests of this module.
"""
import numpy as np
import pytest

from test_gpu_parity import Case, TOL_FP64, check_fields, check_particles, lattice_q, rel_l2

pytestmark = pytest.mark.gpu

N2, L2, Z2, SEED2, LAT2 = 256, 300.0, 24.0, 4242, 1


@pytest.fixture(scope="module")
def cfg2(mfxlib, engine, oracle):
    tab = engine.plt_table(LAT2)
    c = Case(mfxlib, N2, L2, Z2, 3, SEED2, lattice=LAT2, plt=tab)
    res = c.oracle(oracle)
    return c, res


def oracle_order_particles(c, res, order):
    """The oracle's particles with only LPT order `order` in the displacement
    and velocity (the other potentials zeroed)."""
    from oracle import lpt, plt as oplt
    grad = oplt.PLTGradient(c.n, c.L, c.plt)
    zero = np.zeros_like(res["phi"])
    fields = {1: (res["phi"], None, None, None),
              2: (zero, res["phi2"], None, None),
              3: (zero, zero, res["phi3"], res["A3"])}[order]
    pos, vel, _ = lpt.particles(fields, res["coef"], grad, c.lattice, c.n, c.L, c.lunit, c.vunit, order)
    return pos, vel


def test_config2_fp64_every_field_and_particle(mfxlib, engine, cfg2):
    c, res = cfg2
    j = c.job(mfxlib, engine)
    j.run_noise(raw=False)
    assert rel_l2(j.field(mfxlib.FIELD_NOISE), res["noise"]) < 1e-13
    j.run()
    check_fields(mfxlib, j, res, 3)
    check_particles(c, j, res)
    j.close()


def test_config2_fp32c_error_in_spacing_units_per_order(mfxlib, engine, cfg2, capsys):
    c, res = cfg2
    delta = c.L / (c.n * 2 ** (c.lattice / 3.0))
    j = c.job(mfxlib, engine, precision=mfxlib.FP32C, pos64=True, vel64=False)
    j.run()
    pos, vel, ids = j.particles()
    assert np.array_equal(ids, res["ids"])
    err = (pos - res["pos"]) / delta
    rms, mx = float(np.sqrt(np.mean(err ** 2))), float(np.max(np.abs(err)))
    vrel = rel_l2(vel.astype(np.float64), res["vel"])
    report = {"all": (rms, mx, vrel)}
    assert rms < 1e-5 and mx < 1e-3 and vrel < 1e-5, report
    q = lattice_q(c.n, c.lattice, c.lunit)
    for order in (1, 2, 3):
        j.assemble(1 << (order - 1))
        p, v, _ = j.particles()
        pr, vr = oracle_order_particles(c, res, order)
        e = (p - pr) / delta
        o_rms, o_max = float(np.sqrt(np.mean(e ** 2))), float(np.max(np.abs(e)))
        o_v = rel_l2(v.astype(np.float64), vr)
        report["psi%d" % order] = (o_rms, o_max, o_v, float(np.sqrt(np.mean(((pr - q) / delta) ** 2))))
        assert o_rms < 1e-5, report
    j.close()
    with capsys.disabled():
        print("\n256^3 BCC FP32 form vs FP64 oracle (rms, max of the spacing; v rel L2; [order rms size]):", report)


def test_config2_kz_planes_antihermitian_share(cfg2, capsys):
    """The displacement and velocity spectra handed to the final c2r: the
    anti-Hermitian part of their kz = 0 and kz = N/2 planes, relative to the
    whole field (Parseval weights), bounds how far any c2r pass order could
    move the real-space result.  FFTW's multi-dimensional c2r runs the complex
    transforms over x and y before the real transform along z, which keeps
    only the Hermitian part -- the engine's and the oracle's choice."""
    from oracle import lpt, plt as oplt
    c, res = cfg2
    grad = oplt.PLTGradient(c.n, c.L, c.plt)
    fields = (res["phi"], res["phi2"], res["phi3"], res["A3"])
    idx = (-np.arange(c.n)) % c.n
    out = {}
    for kind in ("psi", "vel"):
        for d in range(3):
            if kind == "psi":
                f = lpt.assemble_displacement(d, fields, res["coef"], grad, c.lunit, c.L, 3)
            else:
                f = lpt.assemble_velocity(d, fields, res["coef"], grad, c.vunit, c.L, 3)
            w = np.full(f.shape[2], 2.0)
            w[0] = w[-1] = 1.0
            total = float(np.sum(w * np.sum(np.abs(f) ** 2, axis=(0, 1))))
            anti = 0.0
            for kz in (0, f.shape[2] - 1):
                p = f[:, :, kz]
                anti += float(np.sum(np.abs(0.5 * (p - np.conj(p[np.ix_(idx, idx)]))) ** 2))
            out["%s%d" % (kind, d)] = np.sqrt(anti / total)
    with capsys.disabled():
        print("\n256^3 BCC+PLT anti-Hermitian share of the kz planes (relative L2):",
              {k: "%.2e" % v for k, v in out.items()})
    # present (the PLT stencil touches the table's Nyquist node) and small
    assert max(out.values()) > 0.0
    assert max(out.values()) < 1e-2


@pytest.mark.parametrize("n", [512, 768])
def test_fused_long_padded_lengths_match_cufft_route(mfxlib, engine, n, monkeypatch):
    """M = 3N/2 = 768 and 1152: the fused route's potentials and particles
    against the cuFFT route of the same FP32 form (3LPT, SC lattice)."""
    c = Case(mfxlib, n, 300.0 * n / 256, 24.0, 3, 31, lattice=0)
    fids = [mfxlib.FIELD_PHI2, mfxlib.FIELD_PHI3, mfxlib.FIELD_A3Z]
    count = 1 << 22
    first = (n ** 3) // 2 - count // 2
    out = []
    for fused in ("1", "0"):
        monkeypatch.setenv("MFX_FUSED", fused)
        j = c.job(mfxlib, engine, precision=mfxlib.FP32C)
        j.run()
        out.append(([j.field(f) for f in fids], j.particles_range(first, count)))
        j.close()
    for f, a, b in zip(fids, out[0][0], out[1][0]):
        assert np.all(np.isfinite(a)) and rel_l2(a, b) < 5e-6, (f, rel_l2(a, b))
    delta = c.L / c.n
    pf, pr = out[0][1], out[1][1]
    assert np.sqrt(np.mean(((pf[0] - pr[0]) / delta) ** 2)) < 1e-6
    assert rel_l2(pf[1].astype(np.float64), pr[1].astype(np.float64)) < 5e-6
    assert np.array_equal(pf[2], pr[2])
