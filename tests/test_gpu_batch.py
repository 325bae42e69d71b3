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


@pytest.mark.parametrize("ring", [2, 1, 0])
def test_pipelined_downloads_match_runs_one_at_a_time(mfxlib, engine, ring):
    """Asynchronous downloads, with the output ring of two particle sets (runs
    alternate between them and compute while the previous run's particles
    download), of one set (a run's assembly waits for the previous download)
    and without it (the next run waits): three runs of one job, three seeds
    through mfx_job_upload, each run enqueued right after the previous run's
    download, give each seed's particles of a run made alone."""
    import torch
    specs = [spec(mfxlib, 48, 150.0, 24.0, 3, s, lattice=1, precision=mfxlib.FP32C) for s in (31, 32, 33)]
    refs = [run_alone(mfxlib, engine, sp) for sp in specs]
    sp0 = specs[0]
    j = mfxlib.Job(engine, 48, 150.0, 3, sp0["seed_table"], sp0["amp_table"], sp0["coef"], lattice=1,
                   precision=mfxlib.FP32C, lunit=sp0["lunit"], vunit=sp0["vunit"])
    if ring:
        j.set_output_ring(ring)
    npart = j.num_particles
    bufs = []
    for _ in specs:
        bufs.append((torch.empty((npart, 3), dtype=torch.float64 if j.pos64 else torch.float32, pin_memory=True),
                     torch.empty((npart, 3), dtype=torch.float64 if j.vel64 else torch.float32, pin_memory=True),
                     torch.empty(npart, dtype=torch.int64 if j.id64 else torch.int32, pin_memory=True)))
    for sp, (p, v, i) in zip(specs, bufs):
        j.upload(sp["seed_table"], sp["amp_table"])
        j.run(wait=False)
        j.fetch_particles_range_async(0, npart, p.data_ptr(), v.data_ptr(), i.data_ptr())
    j.wait()
    j.wait_fetch()
    for ref, (p, v, i) in zip(refs, bufs):
        assert np.array_equal(p.numpy(), ref[0])
        assert np.array_equal(v.numpy(), ref[1])
        assert np.array_equal(i.numpy().view(ref[2].dtype), ref[2])
    # the synchronous fetch reads the last run's set
    last = j.particles()
    assert np.array_equal(last[0], refs[-1][0])
    j.close()


def test_output_ring_state_errors(mfxlib, engine):
    """The output ring and graph capture exclude each other; asynchronous
    downloads need particles of a run."""
    sp = spec(mfxlib, 32, 100.0, 24.0, 2, 5, lattice=1, precision=mfxlib.FP32C)
    j = mfxlib.Job(engine, 32, 100.0, 2, sp["seed_table"], sp["amp_table"], sp["coef"], lattice=1,
                   precision=mfxlib.FP32C, lunit=sp["lunit"], vunit=sp["vunit"])
    buf = np.zeros(j.num_particles * 3, dtype=np.float64)
    with pytest.raises(RuntimeError):
        j.fetch_particles_range_async(0, 1, buf.ctypes.data, None, None)  # no run yet
    j.set_output_ring(True)
    with pytest.raises(RuntimeError):
        j.capture()
    j.set_output_ring(False)
    j.capture()
    with pytest.raises(RuntimeError):
        j.set_output_ring(True)
    j.run()
    ref = run_alone(mfxlib, engine, sp)
    assert np.array_equal(j.particles()[0], ref[0])
    j.close()
