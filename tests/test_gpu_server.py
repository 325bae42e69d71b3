"""Serving loop: admission by HBM footprint, overlap of concurrent jobs, and
results that are the same alone and in the mix."""
import numpy as np
import pytest

from test_gpu_batch import run_alone, spec

pytestmark = pytest.mark.gpu

_PLT = {}


def mixed_specs(mfx, engine, count, seed=7):
    rng = np.random.default_rng(seed)
    out = []
    for q in range(count):
        n = int(rng.choice([16, 24, 32, 48]))
        order = int(rng.integers(1, 4))
        lat = int(rng.integers(0, 3))
        prec = mfx.FP32C if q % 2 else mfx.FP64
        sp = spec(mfx, n, 50.0 * n / 32, 24.0, order, 100 + q, lattice=lat, precision=prec)
        if lat != 0:
            if lat not in _PLT:
                _PLT[lat] = engine.plt_table(lat)
            sp["plt_table"] = _PLT[lat]
        out.append(sp)
    return out


def alone(mfx, engine, sp):
    j = mfx.Job(engine, sp["ngrid"], sp["boxlen"], sp["order"], sp["seed_table"], sp["amp_table"], sp["coef"],
                lattice=sp["lattice"], precision=sp["precision"], plt_table=sp.get("plt_table"),
                lunit=sp["lunit"], vunit=sp["vunit"])
    j.run()
    out = j.particles()
    j.close()
    return out


def test_server_results_same_alone_and_in_the_mix(mfxlib, engine):
    specs = mixed_specs(mfxlib, engine, 10)
    # two larger jobs in the mix: 3LPT + PLT FCC at 128^3 and 2LPT BCC at 192^3, FP32 form
    for n, lat, order in ((128, 2, 3), (192, 1, 2)):
        sp = spec(mfxlib, n, 300.0 * n / 256, 24.0, order, 500 + n, lattice=lat, precision=mfxlib.FP32C)
        if lat not in _PLT:
            _PLT[lat] = engine.plt_table(lat)
        sp["plt_table"] = _PLT[lat]
        specs.insert(3 + len(specs) % 4, sp)
    srv = mfxlib.Server(engine, max_inflight=4)
    tickets = [srv.submit(sp) for sp in specs]
    for t in tickets:
        srv.wait(t, 60000)
    for t, sp in zip(tickets, specs):
        got = srv.job(t).particles()
        ref = alone(mfxlib, engine, sp)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
        q, lat = srv.times(t)
        assert 0 <= q <= lat
        srv.release(t)
    srv.close()


def test_server_admission_by_footprint(mfxlib):
    import ctypes
    specs = [spec(mfxlib, 32, 60.0, 24.0, 3, 200 + q) for q in range(4)]
    # footprint of one job, measured through the ABI
    probe = mfxlib.Engine(0)
    j = mfxlib.Job(probe, 32, 60.0, 3, specs[0]["seed_table"], specs[0]["amp_table"], specs[0]["coef"])
    fp = ctypes.c_size_t()
    mfxlib.check(mfxlib.load().mfx_job_footprint(probe.handle, ctypes.byref(j.desc), ctypes.byref(fp)))
    j.close()
    probe.close()
    # a budget for about 1.5 jobs: admission must serialise them
    eng = mfxlib.Engine(0, hbm_budget_bytes=int(fp.value * 1.5))
    srv = mfxlib.Server(eng, max_inflight=4)
    tickets = [srv.submit(sp) for sp in specs]
    ends = []
    for t in tickets:
        srv.wait(t, 60000)
        ends.append(srv.times(t))
        srv.release(t)  # frees the arena for the next admission
    # later jobs waited in the queue for memory
    assert ends[-1][0] > 0.0
    ref = run_alone(mfxlib, eng, specs[-1])
    srv.close()
    eng.close()
    assert ref[0].shape[0] == 32 ** 3


def test_server_wait_timeout_is_an_error_not_a_hang(mfxlib, engine):
    sp = spec(mfxlib, 64, 100.0, 24.0, 3, 9)
    srv = mfxlib.Server(engine, max_inflight=1)
    t = srv.submit(sp)
    rc = mfxlib.load().mfx_server_wait(srv._h, t, 0)
    assert rc in (mfxlib.MFX_OK, mfxlib.MFX_ETIMEOUT)
    srv.wait(t, 60000)
    srv.release(t)
    with pytest.raises(mfxlib.MfxError):
        srv.release(t)
    srv.close()


def _footprint(mfx, engine, sp):
    import ctypes
    j = mfx.Job(engine, sp["ngrid"], sp["boxlen"], sp["order"], sp["seed_table"], sp["amp_table"], sp["coef"],
                want_particles=True)
    fp = ctypes.c_size_t()
    mfx.check(mfx.load().mfx_job_footprint(engine.handle, ctypes.byref(j.desc), ctypes.byref(fp)))
    j.close()
    return fp.value


@pytest.mark.parametrize("bypass", [True, False])
def test_server_bounded_bypass_of_a_head_that_does_not_fit(mfxlib, bypass):
    """A budget for one large job and a little more: while the first large job's
    results are held, a second large job cannot be admitted.  With bypass, the
    small jobs queued behind it start and finish anyway; with strict
    first-in first-out admission they wait behind it.  Releasing the first
    large job lets the rest through, in both policies."""
    big = [spec(mfxlib, 64, 100.0, 24.0, 3, 300 + q) for q in range(2)]
    small = [spec(mfxlib, 16, 25.0, 24.0, 1, 400 + q) for q in range(2)]
    probe = mfxlib.Engine(0)
    fb, fs = _footprint(mfxlib, probe, big[0]), _footprint(mfxlib, probe, small[0])
    probe.close()
    eng = mfxlib.Engine(0, hbm_budget_bytes=int(fb * 1.5) + 4 * fs)
    srv = mfxlib.Server(eng, max_inflight=4)
    srv.set_policy(bypass=bypass, bypass_age_ms=60000.0)
    t_big0 = srv.submit(big[0])
    srv.wait(t_big0, 60000)
    t_big1 = srv.submit(big[1])
    t_small = [srv.submit(sp) for sp in small]
    if bypass:
        for t in t_small:
            srv.wait(t, 60000)
    else:
        with pytest.raises(mfxlib.MfxError) as e:
            srv.wait(t_small[0], 500)
        assert e.value.code == mfxlib.MFX_ETIMEOUT
    with pytest.raises(mfxlib.MfxError):
        srv.wait(t_big1, 200)  # the head still does not fit
    srv.release(t_big0)
    srv.wait(t_big1, 60000)
    for t in t_small:
        srv.wait(t, 60000)
    ref = alone(mfxlib, eng, small[1])
    got = srv.job(t_small[1]).particles()
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    for t in [t_big1] + t_small:
        srv.release(t)
    srv.close()
    eng.close()


def test_server_age_limit_stops_bypassing_an_old_head(mfxlib):
    """With an age limit of zero the head is never passed: a small job that
    would fit waits behind a large head that does not."""
    big = [spec(mfxlib, 64, 100.0, 24.0, 3, 310 + q) for q in range(2)]
    small = spec(mfxlib, 16, 25.0, 24.0, 1, 410)
    probe = mfxlib.Engine(0)
    fb, fs = _footprint(mfxlib, probe, big[0]), _footprint(mfxlib, probe, small)
    probe.close()
    eng = mfxlib.Engine(0, hbm_budget_bytes=int(fb * 1.5) + 4 * fs)
    srv = mfxlib.Server(eng, max_inflight=4)
    srv.set_policy(bypass=True, bypass_age_ms=0.0)
    t0 = srv.submit(big[0])
    srv.wait(t0, 60000)
    t1 = srv.submit(big[1])
    import time
    time.sleep(0.01)  # the head is now older than the limit
    ts = srv.submit(small)
    with pytest.raises(mfxlib.MfxError):
        srv.wait(ts, 500)
    srv.release(t0)
    srv.wait(t1, 60000)
    srv.wait(ts, 60000)
    srv.release(t1)
    srv.release(ts)
    srv.close()
    eng.close()


def test_server_largest_first_admission(mfxlib, engine):
    """With largest-first admission (and a head young enough to be passed), a
    large request queued behind small ones is admitted first once a slot
    frees; first-in first-out admits the small ones first.  Results equal the
    jobs run alone."""
    blocker_spec = spec(mfxlib, 128, 300.0, 24.0, 3, 900, precision=mfxlib.FP64)
    small_specs = [spec(mfxlib, 16, 25.0, 24.0, 1, 910 + q) for q in range(2)]
    big_spec = spec(mfxlib, 64, 100.0, 24.0, 2, 920)
    for largest_first in (True, False):
        srv = mfxlib.Server(engine, max_inflight=1)
        srv.set_policy(bypass=True, bypass_age_ms=60000.0, largest_first=largest_first)
        # all three queue behind the blocker (a 128^3 3LPT job in FP64)
        blocker = srv.submit(blocker_spec)
        small = [srv.submit(sp) for sp in small_specs]
        big = srv.submit(big_spec)
        for t in [blocker] + small + [big]:
            srv.wait(t, 60000)
        qb = srv.times(big)[0]
        qs = [srv.times(t)[0] for t in small]
        if largest_first:
            assert all(qb < q for q in qs), (qb, qs)
        else:
            assert all(qb > q for q in qs), (qb, qs)
        got = srv.job(big).particles()
        for a, b in zip(got, alone(mfxlib, engine, big_spec)):
            assert np.array_equal(a, b)
        for t in [blocker] + small + [big]:
            srv.release(t)
        srv.close()


def test_server_small_jobs_beside_the_slots(mfxlib, engine):
    """A small job takes no in-flight slot: with the one slot held and a large
    head waiting for it (too old to be passed), the small job is admitted and
    finishes while the head still waits; without the setting it waits."""
    import time
    blocker_spec = spec(mfxlib, 192, 300.0, 24.0, 3, 930, precision=mfxlib.FP64)
    big_spec = spec(mfxlib, 64, 100.0, 24.0, 3, 931, precision=mfxlib.FP64)
    small_spec = spec(mfxlib, 16, 25.0, 24.0, 1, 932)
    fs = mfxlib.footprint(engine, small_spec)
    assert fs < mfxlib.footprint(engine, big_spec)
    for beside in (True, False):
        srv = mfxlib.Server(engine, max_inflight=1)
        srv.set_policy(bypass=True, bypass_age_ms=0.0)
        if beside:
            srv.set_small_jobs(fs, 4)
        t0 = srv.submit(blocker_spec)
        t1 = srv.submit(big_spec)
        time.sleep(0.01)  # the head is now older than the age limit
        ts = srv.submit(small_spec)
        if beside:
            srv.wait(ts, 60000)
            with pytest.raises(mfxlib.MfxError):
                srv.wait(t1, 0)  # the head still waits for the slot (or runs)
        else:
            with pytest.raises(mfxlib.MfxError):
                srv.wait(ts, 20)
        for t in (t0, t1, ts):
            srv.wait(t, 60000)
        got = srv.job(ts).particles()
        for a, b in zip(got, alone(mfxlib, engine, small_spec)):
            assert np.array_equal(a, b)
        for t in (t0, t1, ts):
            srv.release(t)
        srv.close()
