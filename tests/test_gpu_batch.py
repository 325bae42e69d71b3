"""CUDA-graph replay and ensembles: a job's results do not depend on whether
it runs eagerly, as a replayed graph, or as one branch of an ensemble graph."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def spec(mfx, n, L, z, order, seed, lattice=0, precision=None, sigma8=0.81):
    lat = {0: "sc", 1: "bcc", 2: "fcc"}[lattice]
    c = mfx.Cosmology(mfx.ini_text(n, L, z, order, seed, lat, sigma8=sigma8))
    return dict(ngrid=n, boxlen=L, order=order, seed_table=mfx.ngenic_seed_table(seed, n),
                amp_table=c.amp_table(n, L), coef=mfx.lpt_coefficients(c.get("dplus_start"), c.get("vfact_start"), order),
                lattice=lattice, precision=mfx.FP64 if precision is None else precision, lunit=L,
                vunit=L / np.sqrt(1.0 / (1.0 + z)))


def run_alone(mfx, engine, sp):
    j = mfx.Job(engine, sp["ngrid"], sp["boxlen"], sp["order"], sp["seed_table"], sp["amp_table"], sp["coef"],
                lattice=sp["lattice"], precision=sp["precision"], lunit=sp["lunit"], vunit=sp["vunit"])
    j.run()
    out = j.particles()
    j.close()
    return out


def test_captured_graph_replay_matches_eager(mfxlib, engine):
    sp = spec(mfxlib, 32, 100.0, 24.0, 3, 21, lattice=1)
    ref = run_alone(mfxlib, engine, sp)
    j = mfxlib.Job(engine, 32, 100.0, 3, sp["seed_table"], sp["amp_table"], sp["coef"], lattice=1,
                   lunit=sp["lunit"], vunit=sp["vunit"])
    j.capture()
    for _ in range(2):
        j.run()
        got = j.particles()
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
    j.close()


def test_ensemble_members_match_standalone_runs(mfxlib, engine):
    specs = [spec(mfxlib, 16, 60.0, 49.0, 2, 1, sigma8=0.75),
             spec(mfxlib, 24, 80.0, 49.0, 1, 2, lattice=2, sigma8=0.8),
             spec(mfxlib, 32, 120.0, 24.0, 3, 3, lattice=1, precision=mfxlib.FP32C, sigma8=0.85),
             spec(mfxlib, 16, 60.0, 49.0, 2, 1, sigma8=0.75)]
    b = mfxlib.Batch(engine, specs)
    b.run()
    ms = b.wait()
    assert ms > 0
    for q, sp in enumerate(specs):
        got = b.job(q).particles()
        ref = run_alone(mfxlib, engine, sp)
        for a, r in zip(got, ref):
            assert np.array_equal(a, r), q
    # a second launch of the same graph reproduces the results
    b.run()
    b.wait()
    again = b.job(2).particles()
    ref = run_alone(mfxlib, engine, specs[2])
    assert np.array_equal(again[0], ref[0])
    b.close()
