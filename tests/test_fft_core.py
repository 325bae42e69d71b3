"""The compile-time pencil FFT of the fused transforms (fused.cuh), built for
the host and run step by step as the CTA runs it, against numpy's FFT for
every padded length the engine supports, in both shared-memory layouts."""
import pathlib
import subprocess

import numpy as np
import pytest

HERE = pathlib.Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe = tmp_path_factory.mktemp("fft") / "fft_core_check"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-o", str(exe), str(HERE / "fft_core_check.cc")])
    return exe


@pytest.mark.parametrize("L", [16, 24, 32, 48, 64, 96, 128, 144, 192, 256, 288, 384, 512, 576, 768, 1024, 1152, 1536])
@pytest.mark.parametrize("inv", [0, 1])
@pytest.mark.parametrize("layout", [0, 1])
def test_stockham_matches_numpy(harness, L, inv, layout):
    P = 3
    rng = np.random.default_rng(L + 7 * inv + 3 * layout)
    x = (rng.standard_normal((P, L)) + 1j * rng.standard_normal((P, L))).astype(np.complex64)
    inp = "\n".join("%r %r" % (float(v.real), float(v.imag)) for v in x.ravel())
    out = subprocess.run([str(harness), str(L), str(P), str(inv), str(layout)], input=inp, capture_output=True,
                         text=True, check=True).stdout.split()
    got = np.array(out, dtype=np.float64).reshape(P, L, 2)
    got = got[..., 0] + 1j * got[..., 1]
    ref = np.fft.ifft(x.astype(np.complex128), axis=1) * L if inv else np.fft.fft(x.astype(np.complex128), axis=1)
    err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    assert err < 5e-7
