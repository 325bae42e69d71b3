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


def test_xy_tile_forms(harness):
    """Every admissible x/y tile's shared memory, and the in-place form's side
    buffer and stage rows, are within bounds (fused.cuh XY)."""
    out = subprocess.run([str(harness), "xy"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout[-2000:]
    last = out.stdout.split()
    assert int(last[last.index("inplace") + 1]) > 0


@pytest.mark.parametrize("L,side", [(96, 0), (96, 37), (576, 314), (768, 768), (1152, 592), (1152, 1)])
@pytest.mark.parametrize("inv", [0, 1])
def test_inplace_halves_match_numpy(harness, L, side, inv):
    """The x/y passes' in-place form run step by step on the host: 16 pencils,
    input rows split between the side buffer and the tile, the first steps of
    both 8-pencil halves before the others (the side buffer is refilled after
    them), the result read back from the tile's rows."""
    P = 16
    rng = np.random.default_rng(L + side + inv)
    x = (rng.standard_normal((P, L)) + 1j * rng.standard_normal((P, L))).astype(np.complex64)
    inp = "\n".join("%r %r" % (float(v.real), float(v.imag)) for v in x.ravel())
    out = subprocess.run([str(harness), "ip", str(L), str(inv), str(side)], input=inp, capture_output=True, text=True,
                         check=True).stdout.split()
    got = np.array(out, dtype=np.float64).reshape(P, L, 2)
    got = got[..., 0] + 1j * got[..., 1]
    ref = np.fft.ifft(x.astype(np.complex128), axis=1) * L if inv else np.fft.fft(x.astype(np.complex128), axis=1)
    err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    assert err < 5e-7
