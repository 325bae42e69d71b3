"""The allocation-free white-noise entry point, mfx_noise_fill_noalloc.

It exists for callers that cannot let a library call cudaMalloc -- a host code
that already owns all of HBM through its own pool allocator, or one running
under a device-memory cap: the caller allocates the output field itself and
the library stages the seed table in a fixed __device__ array.  This test plays
such a caller (its output buffer comes from torch's allocator, not from
libmfx) and checks the result against the regular entry point
(mfx_job_run_noise on a job whose arena libmfx allocated), on two calls in a
row with different sizes, seeds, normalisations and precisions.

Collected last on purpose (file name), so a run that stops at the first
failure has run every other test before this one.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def regular_noise(mfx, engine, n, boxlen, seeds, raw, fixing, inversion, precision):
    cosmo = mfx.Cosmology(mfx.ini_text(n, boxlen, 49.0, 1, 1))
    coef = mfx.lpt_coefficients(cosmo.get("dplus_start"), cosmo.get("vfact_start"), 1)
    job = mfx.Job(engine, n, boxlen, 1, seeds, cosmo.amp_table(n, boxlen), coef, precision=precision,
                  fixing=fixing, inversion=inversion, want_particles=False)
    job.run_noise(raw=raw)
    out = job.field(mfx.FIELD_NOISE)
    job.close()
    return out


def test_noise_fill_without_allocation_matches_regular_entry_point(mfxlib, engine):
    torch = pytest.importorskip("torch")
    L = mfxlib.load()
    calls = [
        # (ngrid, boxlen, seed, raw, fixing, inversion, precision)
        (64, 100.0, 12345, True, False, False, mfxlib.FP64),
        (96, 300.0, 4242, False, True, True, mfxlib.FP32C),
    ]
    for n, boxlen, seed, raw, fixing, inversion, prec in calls:
        seeds = mfxlib.ngenic_seed_table(seed, n)
        dt = torch.float64 if prec == mfxlib.FP64 else torch.float32
        buf = torch.full((n, n, n // 2 + 1, 2), float("nan"), dtype=dt, device="cuda")
        torch.cuda.synchronize()
        rc = L.mfx_noise_fill_noalloc(engine.handle, n, boxlen, seeds.ctypes.data, int(raw), int(fixing),
                                      int(inversion), prec, ctypes.c_void_p(buf.data_ptr()), None)
        assert rc == mfxlib.MFX_OK, mfxlib.last_error()
        torch.cuda.synchronize()
        a = buf.cpu().double().numpy()
        got = a[..., 0] + 1j * a[..., 1]
        ref = regular_noise(mfxlib, engine, n, boxlen, seeds, raw, fixing, inversion, prec)
        assert np.all(np.isfinite(got))
        # same tolerance as the noise parity tests (absolute, unit-variance modes)
        assert np.max(np.abs(got - ref)) < 1e-13


def test_noise_fill_without_allocation_rejects_oversized_grid(mfxlib, engine):
    L = mfxlib.load()
    n = 1028  # above MFX_NOALLOC_MAX_NGRID = 1024
    dummy = np.zeros(1, dtype=np.uint32)
    rc = L.mfx_noise_fill_noalloc(engine.handle, n, 100.0, dummy.ctypes.data, 1, 0, 0, mfxlib.FP64,
                                  ctypes.c_void_p(1), None)
    assert rc == mfxlib.MFX_EINVAL
    assert "1024" in mfxlib.last_error()
