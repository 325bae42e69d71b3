"""The allocation-free white-noise entry point, mfx_noise_fill_noalloc.

It exists for callers that cannot let a library call cudaMalloc -- a host code
that already owns all of HBM through its own pool allocator, or one running
under a device-memory cap: the caller allocates the output field itself and
the library stages the seed table in a fixed __device__ array.  This test plays
such a caller (its output buffer comes from torch's allocator, not from
libmfx) and checks the result against the regular entry point
(mfx_job_run_noise on a job whose arena libmfx allocated), on two calls in a
row with different sizes, seeds, normalisations and precisions.

A second test runs in a fresh process, where nothing else has loaded a CUDA
module yet: after the engine exists, two calls (one on a non-default stream)
must leave the device's free memory exactly as it was -- the property such a
caller relies on -- and must leave the caller's current device unchanged.

Collected last on purpose (file name), so a run that stops at the first
failure has run every other test before this one.
"""
import ctypes
import pathlib
import subprocess
import sys

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


FRESH_PROCESS = r"""
import ctypes, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
from monofonic_gb300 import mfx
L = mfx.load()
eng = mfx.Engine(0)  # loads the allocation-free entry point's scratch array and kernels
n = 128
seeds = mfx.ngenic_seed_table(7, n)
buf = torch.empty((n, n, n // 2 + 1, 2), dtype=torch.float64, device="cuda")
side = torch.cuda.Stream()
outs = [torch.empty_like(buf) for _ in range(2)]  # made before the measurement starts
for o in outs:
    o.copy_(buf)  # torch's copy kernel is loaded before the measurement too
torch.cuda.synchronize()
dev0 = torch.cuda.current_device()
free0 = torch.cuda.mem_get_info()[0]
for q, stream in enumerate((None, side.cuda_stream)):
    rc = L.mfx_noise_fill_noalloc(eng.handle, n, 500.0, seeds.ctypes.data, 0, 0, 0, mfx.FP64,
                                  ctypes.c_void_p(buf.data_ptr()), ctypes.c_void_p(stream) if stream else None)
    assert rc == mfx.MFX_OK, mfx.last_error()
    torch.cuda.synchronize()
    outs[q].copy_(buf)
torch.cuda.synchronize()
free1 = torch.cuda.mem_get_info()[0]
assert torch.equal(outs[0], outs[1]), "the two calls disagree"
assert torch.cuda.current_device() == dev0
# control: an 8 MiB device allocation is visible to the same measurement
x = torch.cuda.caching_allocator_alloc(8 << 20)
free2 = torch.cuda.mem_get_info()[0]
torch.cuda.caching_allocator_delete(x)
print("FREE", free0, free1, free2)
"""


def test_noise_fill_without_allocation_leaves_free_memory_unchanged(mfxlib):
    """Fresh process: device free memory is identical before and after two calls
    (default stream, then a side stream); an 8 MiB allocation made afterwards
    does show up in the same measurement."""
    mfxlib.load()  # built in-tree by the session fixture
    root = pathlib.Path(__file__).resolve().parent.parent
    r = subprocess.run([sys.executable, "-c", FRESH_PROCESS, str(root)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("FREE")][-1]
    free0, free1, free2 = (int(v) for v in line.split()[1:])
    assert free1 == free0, "the allocation-free call changed free device memory by %d bytes" % (free0 - free1)
    assert free2 < free1, "the free-memory measurement did not see a control allocation"
