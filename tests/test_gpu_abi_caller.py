"""A C++ program (tests/abi_caller.cc) that uses include/mfx.h alone, linked
against libmfx.so: its particles equal those of the same job driven through
the Python ctypes binding, bit for bit, in both arithmetic forms."""
import pathlib
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = pathlib.Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def caller(mfxlib, tmp_path_factory):
    lib = mfxlib.lib_path()
    exe = tmp_path_factory.mktemp("abi") / "abi_caller"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "include"), "-o", str(exe),
                           str(ROOT / "tests" / "abi_caller.cc"), str(lib), "-Wl,-rpath," + str(lib.parent)])
    return exe


@pytest.mark.parametrize("n,lattice,order,precision", [(16, 0, 2, 0), (32, 1, 3, 0), (32, 2, 3, 1)])
def test_cpp_caller_matches_python_binding(mfxlib, engine, caller, tmp_path, n, lattice, order, precision):
    L, z, seed = 100.0, 24.0, 4242
    lat = {0: "sc", 1: "bcc", 2: "fcc"}[lattice]
    ini = mfxlib.ini_text(n, L, z, order, seed, lat)
    cfg = tmp_path / "ics.conf"
    cfg.write_text(ini)
    out = tmp_path / "particles.bin"
    r = subprocess.run([str(caller), str(cfg), str(n), repr(L), repr(z), str(order), str(lattice), str(seed),
                        str(precision), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = out.read_bytes()
    count = int(np.frombuffer(raw[:8], np.uint64)[0])
    assert count == (1 << lattice) * n ** 3
    o = 8
    pos = np.frombuffer(raw[o:o + 24 * count], np.float64).reshape(-1, 3)
    vel = np.frombuffer(raw[o + 24 * count:o + 48 * count], np.float64).reshape(-1, 3)
    ids = np.frombuffer(raw[o + 48 * count:], np.uint64)

    cosmo = mfxlib.Cosmology(ini)
    coef = mfxlib.lpt_coefficients(cosmo.get("dplus_start"), cosmo.get("vfact_start"), order)
    j = mfxlib.Job(engine, n, L, order, mfxlib.ngenic_seed_table(seed, n), cosmo.amp_table(n, L), coef,
                   lattice=lattice, precision=precision, lunit=L, vunit=L / np.sqrt(1.0 / (1.0 + z)),
                   pos64=True, vel64=True, id64=True)
    j.run()
    p, v, i = j.particles()
    j.close()
    assert np.array_equal(pos, p) and np.array_equal(vel, v) and np.array_equal(ids, i)
