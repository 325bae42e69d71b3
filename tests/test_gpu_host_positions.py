"""Host-side positions (mfx_job_set_host_positions): the FP32 form keeps float
displacements on the device and the fetch forms q + Psi in FP64 on the host
(fused route: grids whose padded length is instantiated, here 64^3 -> 96).
The particles must equal those of device-side positions bit for bit -- through
the synchronous fetch, ranges across sub-lattice boundaries, and the
asynchronous fetch with output rings of one and two sets over several runs."""
import numpy as np
import pytest

from test_gpu_batch import run_alone, spec

pytestmark = pytest.mark.gpu


def _job(mfx, engine, sp, **kw):
    return mfx.Job(engine, sp["ngrid"], sp["boxlen"], sp["order"], sp["seed_table"], sp["amp_table"], sp["coef"],
                   lattice=sp["lattice"], precision=sp["precision"], plt_table=sp.get("plt_table"),
                   lunit=sp["lunit"], vunit=sp["vunit"], pos64=True, vel64=False, id64=True, **kw)


@pytest.mark.parametrize("n,lattice,plt", [(64, 1, True), (64, 2, False), (128, 2, True)])
def test_host_positions_equal_device_positions(mfxlib, engine, n, lattice, plt):
    """128^3 FCC: 8.4M particles, three staging chunks of 4M taken by
    different host threads; the range crosses a chunk and a sub-lattice
    boundary."""
    sp = spec(mfxlib, n, 200.0 * n / 64, 24.0, 3, 21, lattice=lattice, precision=mfxlib.FP32C)
    if plt:
        sp["plt_table"] = engine.plt_table(lattice)
    j = _job(mfxlib, engine, sp)
    j.run()
    ref = j.particles()
    j.set_host_positions(True)  # re-assembles the last run in the new form
    got = j.particles()
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    n3 = n ** 3
    first, count = n3 - 777, min(n3 + 1555, j.num_particles - (n3 - 777))
    if n == 128:
        count = j.num_particles - first - 5  # across both chunk boundaries
    rng = j.particles_range(first, count)
    for a, b in zip(rng, ref):
        assert np.array_equal(a, b[first:first + count])
    j.run()
    for a, b in zip(j.particles(), ref):
        assert np.array_equal(a, b)
    j.set_host_positions(False)
    for a, b in zip(j.particles(), ref):
        assert np.array_equal(a, b)
    j.close()


@pytest.mark.parametrize("ring", [0, 1, 2])
def test_host_positions_pipelined(mfxlib, engine, ring):
    """Three runs, three seeds, each fetched asynchronously right after its run
    is enqueued: every seed's particles equal a run made alone."""
    import torch
    specs = [spec(mfxlib, 64, 200.0, 24.0, 3, s, lattice=1, precision=mfxlib.FP32C) for s in (41, 42, 43)]
    for sp in specs:
        sp["plt_table"] = None
    refs = []
    for sp in specs:
        j = _job(mfxlib, engine, sp)
        j.run()
        refs.append(j.particles())
        j.close()
    sp0 = specs[0]
    j = _job(mfxlib, engine, sp0)
    j.set_host_positions(True)
    if ring:
        j.set_output_ring(ring)
    npart = j.num_particles
    bufs = [(torch.empty((npart, 3), dtype=torch.float64, pin_memory=True),
             torch.empty((npart, 3), dtype=torch.float32, pin_memory=True),
             torch.empty(npart, dtype=torch.int64, pin_memory=True)) for _ in specs]
    for sp, (p, v, i) in zip(specs, bufs):
        j.upload(sp["seed_table"], sp["amp_table"])
        j.run(wait=False)
        j.fetch_particles_range_async(0, npart, p.data_ptr(), v.data_ptr(), i.data_ptr())
    j.wait()
    j.wait_fetch()
    for ref, (p, v, i) in zip(refs, bufs):
        assert np.array_equal(p.numpy(), ref[0])
        assert np.array_equal(v.numpy(), ref[1])
        assert np.array_equal(i.numpy().view(np.uint64), ref[2])
    j.close()


def test_host_positions_errors(mfxlib, engine):
    import torch
    sp = spec(mfxlib, 32, 100.0, 24.0, 2, 5, lattice=0)  # plain FP64 form
    j = _job(mfxlib, engine, sp)
    with pytest.raises(mfxlib.MfxError):
        j.set_host_positions(True)
    j.close()
    sp = spec(mfxlib, 32, 100.0, 24.0, 2, 5, lattice=0, precision=mfxlib.FP32C)
    j = _job(mfxlib, engine, sp)
    j.set_output_ring(1)
    with pytest.raises(mfxlib.MfxError):
        j.set_host_positions(True)  # after the ring
    j.set_output_ring(0)
    j.set_host_positions(True)
    j.run()
    dev = torch.zeros((j.num_particles, 3), dtype=torch.float64, device="cuda")
    with pytest.raises(RuntimeError):
        j.fetch_particles_range_into(0, j.num_particles, dev.data_ptr(), None, None)
    j.close()


def test_fused_device_ids_on_request(mfxlib, engine):
    """The fused read-out writes no device ids: a device destination gets them
    from the id kernel (the lattice rule), and mfx_job_particles_device fills an
    array of its own on request."""
    import ctypes
    import torch
    sp = spec(mfxlib, 32, 100.0, 24.0, 2, 7, lattice=2, precision=mfxlib.FP32C)
    j = _job(mfxlib, engine, sp, id_offset=3)
    j.run()
    want = j.particles()[2]
    dev = torch.zeros(j.num_particles, dtype=torch.int64, device="cuda")
    j.fetch_particles_range_into(0, j.num_particles, None, None, dev.data_ptr())
    assert np.array_equal(dev.cpu().numpy().view(np.uint64), want)
    L = mfxlib.load()
    pp, vp, ip, n = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_size_t()
    for _ in range(2):
        mfxlib.check(L.mfx_job_particles_device(j.handle, ctypes.byref(pp), ctypes.byref(vp), ctypes.byref(ip),
                                                ctypes.byref(n)))
        assert ip.value and pp.value and n.value == j.num_particles
    j.close()
