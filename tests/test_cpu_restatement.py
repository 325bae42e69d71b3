"""The C++/OpenMP restatement of the reference path (oracle/lpt_omp.cc), which
bench.py times as the CPU baseline, checked against numpy: its own FFTs
against numpy's, and the whole path against the numpy oracle (oracle/lpt.py)
field by field.  No GPU needed."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def omp(oracle):
    oracle.build_omp_lib()
    return oracle.omp_lib()


@pytest.mark.parametrize("n", [2, 3, 4, 6, 12, 24, 96, 144, 384, 576])
def test_batched_fft_matches_numpy(omp, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal((19, n)) + 1j * rng.standard_normal((19, n))
    for sign, ref in ((-1, np.fft.fft(x, axis=1)), (+1, np.fft.ifft(x, axis=1) * n)):
        a = np.ascontiguousarray(x.copy())
        omp.mfxo_omp_fft1(n, 19, sign, a.ctypes.data)
        assert np.abs(a - ref).max() <= 1e-14 * np.abs(ref).max()


@pytest.mark.parametrize("n", [8, 12, 48])
def test_grid_fft_layout_and_unitary_norm(omp, n):
    """In-place Grid_FFT layout (rows padded to N+2), 1/sqrt(N^3) both ways."""
    rng = np.random.default_rng(n)
    r = rng.standard_normal((n, n, n))
    a = np.zeros((n, n, n + 2))
    a[:, :, :n] = r
    omp.mfxo_omp_fft3(n, 1, a.ctypes.data)
    got = a.view(np.complex128).reshape(n, n, n // 2 + 1)
    ref = np.fft.rfftn(r, norm="ortho")
    assert np.abs(got - ref).max() < 1e-14 * np.abs(ref).max()
    omp.mfxo_omp_fft3(n, 0, a.ctypes.data)
    assert np.abs(a[:, :, :n] - r).max() < 1e-13


def test_c2r_keeps_the_hermitian_part_of_the_kz0_plane(omp, oracle):
    """A kz = 0 plane that is not Hermitian: the x/y-before-z ordering returns
    the transform of its Hermitian part, as the oracle's c2r does."""
    n = 16
    rng = np.random.default_rng(3)
    c = rng.standard_normal((n, n, n // 2 + 1)) + 1j * rng.standard_normal((n, n, n // 2 + 1))
    a = np.zeros((n, n, n + 2))
    a.view(np.complex128).reshape(n, n, n // 2 + 1)[:] = c
    omp.mfxo_omp_fft3(n, 0, a.ctypes.data)
    ref = oracle.fft_c2r(c, n)
    assert np.abs(a[:, :, :n] - ref).max() < 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("n,lattice,order,plt,fixing", [(16, 0, 2, False, False), (24, 1, 3, True, False),
                                                         (16, 2, 3, True, True), (24, 0, 1, False, False)])
def test_whole_path_matches_numpy_oracle(oracle, n, lattice, order, plt, fixing):
    from oracle import cosmo, plt as oplt
    c = cosmo.Cosmology()
    L, a = 300.0, 1.0 / 25.0
    dplus, vfac = c.growth(a), c.vfact(a)
    seeds = oracle.ngenic_seed_table(77, n)
    kf = 2 * np.pi / L
    q = np.arange(3 * (n // 2) ** 2 + 1)
    with np.errstate(divide="ignore", invalid="ignore"):
        k = kf * np.sqrt(q)
        amp = np.where(q > 0, c.amplitude(k) / (k * k), 0.0)
    tab = oplt.plt_tables(lattice) if plt else None
    grad = oplt.PLTGradient(n, L, tab) if plt else None

    def amplitude(kk):
        return c.amplitude(kk.ravel()).reshape(kk.shape)

    ref = oracle.run_lpt(n, L, seeds, amplitude, order, dplus, vfac, lattice=lattice, lunit=L,
                         vunit=L / np.sqrt(a), fixing=fixing, grad=grad)
    got = oracle.run_lpt_omp(n, L, seeds, amp, order, oracle.lpt_coefficients(dplus, vfac, order), lattice=lattice,
                             lunit=L, vunit=L / np.sqrt(a), fixing=fixing, plt_table=tab, want_fields=True)

    def rel(x, y):
        return np.linalg.norm(x - y) / np.linalg.norm(y)

    assert rel(got["phi"], ref["phi"]) < 1e-13
    if order > 1:
        assert rel(got["phi2"], ref["phi2"]) < 1e-12
    if order > 2:
        assert rel(got["phi3"], ref["phi3"]) < 1e-12
        for d in range(3):
            assert rel(got["A3"][d], ref["A3"][d]) < 1e-12
    assert rel(got["pos"], ref["pos"]) < 1e-13
    assert rel(got["vel"], ref["vel"]) < 1e-12
    assert np.array_equal(got["ids"], ref["ids"])
