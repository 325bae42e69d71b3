"""ORACLE -- test infrastructure only.

A CPU restatement (numpy/scipy, FP64) of monofonIC's LPT initial-condition hot
path, written to follow the reference loop by loop so that the GPU engine can be
checked against it.  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg import this module, and only as the checker;
the product never calls it.

Conventions restated from the reference (file:line within the monofonIC tree):

* k-space layout ``kelem(i,j,k)`` = array[i, j, k] of shape (N, N, N/2+1),
  i -> k_x, j -> k_y (grid_fft.hh:196-206, 281-296; grid_fft.cc:40-112).
* Unitary FFTs: r2c and c2r both scaled by 1/sqrt(N^3) (grid_fft.cc:69,
  199-270) == ``norm="ortho"``.
* ``get_k``: index i > N/2 maps to i-N, index N/2 stays positive
  (grid_fft.hh:281-296); ``gradient`` zeroes the index N/2 (grid_fft.hh:376-385).
* Orszag 3/2 padding, pad factor 1.5^1.5, unpad by sqrt(M^3)/sqrt(N^3) and
  zeroing of every Nyquist index (convolution.hh:552-651).
* ``convolve3`` is two pairwise-dealiased ``convolve2`` (convolution.hh:525-532).

The FFT is pocketfft (scipy), not FFTW; results agree with the reference's
arithmetic to rounding (~1e-15 relative), far inside the 1e-10 parity bar.
"""
from __future__ import annotations

import ctypes
import os
import pathlib

import numpy as np
import scipy.fft as sfft

_HERE = pathlib.Path(__file__).resolve().parent
_BUILD = _HERE / "_build"
WORKERS = os.cpu_count() or 1


# ----------------------------------------------------------------------------
# RANLUX / NGenIC (C restatement in oracle/ranlux.c)
# ----------------------------------------------------------------------------
def build_lib() -> pathlib.Path:
    """Compile oracle/ranlux.c and oracle/music.c into
    oracle/_build/liboracle_rng.so (if stale)."""
    srcs = [_HERE / "ranlux.c", _HERE / "music.c"]
    out = _BUILD / "liboracle_rng.so"
    _BUILD.mkdir(exist_ok=True)
    if not out.exists() or any(out.stat().st_mtime < s.stat().st_mtime for s in srcs):
        import subprocess
        tmp = out.with_suffix(".so.tmp%d" % os.getpid())
        # no FMA contraction: the ratio method's tests round like plain C on every host
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-o", str(tmp)]
                              + [str(x) for x in srcs] + ["-lm"])
        os.replace(tmp, out)
    return out


def build_omp_lib() -> pathlib.Path:
    """Compile the C++/OpenMP restatement (oracle/lpt_omp.cc, with the NGenIC
    fill of oracle/ranlux.c) into oracle/_build/liblpt_omp.so (if stale)."""
    srcs = [_HERE / "lpt_omp.cc", _HERE / "ranlux.c"]
    out = _BUILD / "liblpt_omp.so"
    _BUILD.mkdir(exist_ok=True)
    if not out.exists() or any(out.stat().st_mtime < s.stat().st_mtime for s in srcs):
        import subprocess
        obj = _BUILD / ("ranlux_omp.o.tmp%d" % os.getpid())
        tmp = out.with_suffix(".so.tmp%d" % os.getpid())
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-c", str(srcs[1]), "-o", str(obj)])
        subprocess.check_call(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", str(tmp),
                               str(srcs[0]), str(obj), "-lm"])
        os.replace(tmp, out)
        obj.unlink()
    return out


_lib = None
_omp = None


def omp_lib():
    """The C++/OpenMP restatement (CPU baseline of the hot path)."""
    global _omp
    if _omp is None:
        L = ctypes.CDLL(str(build_omp_lib()))
        L.mfxo_omp_fft1.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.mfxo_omp_fft3.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.mfxo_omp_lpt.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        _omp = L
    return _omp


def run_lpt_omp(n, L, seed_table, amp_table, order, coef, lattice=0, lunit=1.0, vunit=1.0, fixing=False,
                inversion=False, plt_table=None, want_fields=False):
    """The C++/OpenMP restatement of the whole path (oracle/lpt_omp.cc).
    amp_table[q] = amplitude(kf sqrt q) / (kf^2 q); coef as lpt_coefficients.
    Returns dict(pos, vel, ids, times[, phi, phi2, phi3, A3])."""
    ns = 1 << lattice
    npart = ns * n ** 3
    pos = np.empty((npart, 3))
    vel = np.empty((npart, 3))
    ids = np.empty(npart, dtype=np.uint64)
    times = np.zeros(6)
    nk = n // 2 + 1
    fields = np.zeros((6, n, n, nk), dtype=np.complex128) if want_fields else None
    seeds = np.ascontiguousarray(seed_table, dtype=np.uint32)
    amp = np.ascontiguousarray(amp_table, dtype=np.float64)
    cf = np.array([coef["g1"], coef["g2"], coef["g3"], coef["g3c"], coef["vfac1"], coef["vfac2"], coef["vfac3"]])
    tab = None if plt_table is None else np.ascontiguousarray(plt_table, dtype=np.float64)
    rc = omp_lib().mfxo_omp_lpt(n, L, order, lattice, int(fixing), int(inversion), seeds.ctypes.data, amp.ctypes.data,
                                len(amp), None if tab is None else tab.ctypes.data, cf.ctypes.data, lunit, vunit,
                                pos.ctypes.data, vel.ctypes.data, ids.ctypes.data,
                                None if fields is None else fields.ctypes.data, times.ctypes.data)
    if rc != 0:
        raise ValueError("mfxo_omp_lpt rejected the arguments")
    out = dict(pos=pos, vel=vel, ids=ids, times=times)
    if want_fields:
        out.update(phi=fields[0], phi2=fields[1], phi3=fields[2], A3=[fields[3], fields[4], fields[5]])
    return out


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(build_lib()))
        _lib.mfxo_ranlxd1_words.argtypes = [ctypes.c_ulong, ctypes.c_size_t, ctypes.c_void_p]
        _lib.mfxo_ngenic_seed_table.argtypes = [ctypes.c_long, ctypes.c_size_t, ctypes.c_void_p]
        _lib.mfxo_ngenic_fill.argtypes = [ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        _lib.mfxo_mt19937_words.argtypes = [ctypes.c_ulong, ctypes.c_size_t, ctypes.c_void_p]
        _lib.mfxo_leva_normals.argtypes = [ctypes.c_ulong, ctypes.c_size_t, ctypes.c_void_p]
        _lib.mfxo_music_noise.argtypes = [ctypes.c_size_t, ctypes.c_size_t, ctypes.c_long, ctypes.c_void_p]
        _lib.mfxo_music_cubes.argtypes = [ctypes.c_size_t, ctypes.c_size_t, ctypes.c_long, ctypes.c_void_p]
    return _lib


def mt19937_words(seed: int, count: int) -> np.ndarray:
    out = np.zeros(count, dtype=np.uint32)
    lib().mfxo_mt19937_words(seed, count, out.ctypes.data)
    return out


def leva_normals(seed: int, count: int) -> np.ndarray:
    out = np.zeros(count)
    lib().mfxo_leva_normals(seed, count, out.ctypes.data)
    return out


def music_noise_real(n: int, seed: int, cubesize: int = 32) -> np.ndarray:
    """MUSIC1 single-level white noise in real space (oracle/music.c)."""
    out = np.zeros((n, n, n))
    lib().mfxo_music_noise(n, cubesize, seed, out.ctypes.data)
    return out


def music_cubes_raw(n: int, seed: int, cubesize: int = 32) -> np.ndarray:
    """One level's cubes without mean subtraction (oracle/music.c)."""
    out = np.zeros((n, n, n))
    lib().mfxo_music_cubes(n, cubesize, seed, out.ctypes.data)
    return out


def _cmod(a: int, b: int) -> int:
    """C's % (truncating toward zero) on integers."""
    r = abs(a) % abs(b)
    return r if a >= 0 else -r


def music_dummy_seed(level: int) -> int:
    """The seed of a level no [random] seed[level] names (random_music.cc:176-183):
    negative, a function of the level only."""
    ltemp = -2
    return -abs(_cmod(ltemp - level, 123) + _cmod(ltemp + 7342523521 * level, 123456789))


def music_refine(coarse: np.ndarray, fine: np.ndarray) -> np.ndarray:
    """A finer level from a coarser one by coarse mode replacement
    (random_music_wnoise_generator.cc:392-547): the fine level's cubes in
    k-space get the coarse level's modes, phase-shifted by half a coarse cell
    and scaled by sqrt(8), except on the coarse Nyquist indices; FFTW's
    unnormalised transforms, the result scaled by 1/n^3 before the c2r."""
    nc, nf = coarse.shape[0], fine.shape[0]
    cf = sfft.rfftn(fine, workers=WORKERS)
    cc = sfft.rfftn(coarse, workers=WORKERS)
    i = np.arange(nc)
    k = np.arange(nc // 2 + 1)
    kx = np.where(i <= nc // 2, i, i - nc).astype(np.float64)
    kz = k.astype(np.float64)
    idx = np.where(i > nc // 2, i + nf // 2, i)
    phase = (kx[:, None, None] / nc + kx[None, :, None] / nc + kz[None, None, :] / nc) * (-0.5) * np.pi
    val = cc * np.exp(1j * phase) * np.sqrt(8.0)
    keep = (i != nc // 2)[:, None, None] & (i != nc // 2)[None, :, None] & (k != nc // 2)[None, None, :]
    sub = cf[np.ix_(idx, idx, k)]
    cf[np.ix_(idx, idx, k)] = np.where(keep, val, sub)
    cf *= 1.0 / float(nf) ** 3
    return sfft.irfftn(cf, s=(nf, nf, nf), workers=WORKERS) * float(nf) ** 3


def music_restrict(fine: np.ndarray) -> np.ndarray:
    """The next coarser level of a field by k-space averaging
    (random_music_wnoise_generator.cc:288-380): every coarse mode takes the
    fine mode of the same wave vector times exp(+i pi/2 (kx + ky + kz)/nc) /
    sqrt(8), FFTW's unnormalised transforms, 1/nc^3 before the c2r."""
    nf = fine.shape[0]
    nc = nf // 2
    cf = sfft.rfftn(fine, workers=WORKERS)
    i = np.arange(nc)
    k = np.arange(nc // 2 + 1)
    kx = np.where(i <= nc // 2, i, i - nc).astype(np.float64)
    idx = np.where(i > nc // 2, i + nf // 2, i)
    phase = (kx[:, None, None] / nc + kx[None, :, None] / nc + k[None, None, :].astype(np.float64) / nc) * 0.5 * np.pi
    cc = cf[np.ix_(idx, idx, k)] * np.exp(1j * phase) * (1.0 / float(nc) ** 3) / np.sqrt(8.0)
    return sfft.irfftn(cc, s=(nc, nc, nc), workers=WORKERS) * float(nc) ** 3


def music_levels(n: int, seeds: dict, cubesize: int = 32, field=None) -> np.ndarray:
    """MUSIC1's real-space noise at level log2(n) (random_music.cc:222-283):
    with seeds at coarser levels the coarsest seeded level is filled (its mean
    subtracted) and each finer level up to log2(n) refines the one below with
    its own seed or the level's dummy seed; with seeds only at finer levels the
    coarsest of them is filled and restricted down level by level.  field: the
    noise of a coarser level read from a file (random_music.cc:216-236, values
    as read, no mean subtracted), the start of the refinement chain."""
    lmin = int(n).bit_length() - 1
    if field is not None:
        f = np.asarray(field, dtype=np.float64)
        l0 = int(f.shape[0]).bit_length() - 1
        for level in range(l0 + 1, lmin + 1):
            f = music_refine(f, music_cubes_raw(1 << level, seeds.get(level, music_dummy_seed(level)), cubesize))
        return f
    l0 = min(seeds)
    if l0 == lmin:
        return music_noise_real(n, seeds[lmin], cubesize)
    if l0 > lmin:
        f = music_noise_real(1 << l0, seeds[l0], cubesize)
        for level in range(l0 - 1, lmin - 1, -1):
            f = music_restrict(f)
        return f
    f = music_noise_real(1 << l0, seeds[l0], cubesize)
    for level in range(l0 + 1, lmin + 1):
        seed = seeds.get(level, music_dummy_seed(level))
        f = music_refine(f, music_cubes_raw(1 << level, seed, cubesize))
    return f


def read_grafic_noise(path: str, res: int, grafic_sign: bool = False) -> np.ndarray:
    """MUSIC1's white-noise file (random_music_wnoise_generator.cc:68-282):
    a header record (nx ny nz iseed, int32) and nz records of nx*ny float32 or
    float64, framed by 32- or 64-bit byte counts; record z, x fastest, fills
    [x][y][z], negated unless grafic_sign."""
    raw = open(path, "rb").read()
    mw = 4
    if not (int.from_bytes(raw[0:4], "little") == 16 and int.from_bytes(raw[4:8], "little") == res):
        mw = 8
        if not (int.from_bytes(raw[0:8], "little") == 16 and int.from_bytes(raw[8:12], "little") == res):
            raise ValueError("corrupt random number file")
    pos = mw
    nx, ny, nz, _ = np.frombuffer(raw[pos:pos + 16], np.int32)
    pos += 16 + mw
    assert nx == ny == nz == res
    out = np.zeros((res, res, res))
    for z in range(res):
        m = int.from_bytes(raw[pos:pos + mw], "little")
        pos += mw
        dt = np.float32 if m == res * res * 4 else np.float64
        rec = np.frombuffer(raw[pos:pos + m], dt).astype(np.float64).reshape(res, res)  # [y][x]
        pos += m + mw
        out[:, :, z] = rec.T
    return out if grafic_sign else -out


def music_fill(n: int, seed: int, cubesize: int = 32) -> np.ndarray:
    """RNG_music::Fill_Grid followed by the IC generator's forward transform:
    the k-space white noise (random_music.cc:92-116, ic_generator.cc:305-383)."""
    return fft_r2c(music_noise_real(n, seed, cubesize))


def ranlxd1_words(seed: int, count: int) -> np.ndarray:
    out = np.zeros(count, dtype=np.uint64)
    lib().mfxo_ranlxd1_words(seed, count, out.ctypes.data)
    return out


def ngenic_seed_table(seed: int, n: int) -> np.ndarray:
    """random_ngenic.cc:39-75"""
    t = np.zeros(n * n, dtype=np.uint32)
    lib().mfxo_ngenic_seed_table(seed, n, t.ctypes.data)
    return t


def ngenic_fill(n: int, table: np.ndarray, with_uniforms: bool = False):
    """random_ngenic.cc:84-154 (non-distributed).  Returns complex (N,N,N/2+1)."""
    nk = n // 2 + 1
    out = np.zeros((n, n, nk), dtype=np.complex128)
    uni = np.zeros((n, n, nk, 2), dtype=np.float64) if with_uniforms else None
    table = np.ascontiguousarray(table, dtype=np.uint32)
    lib().mfxo_ngenic_fill(n, table.ctypes.data, out.ctypes.data,
                           uni.ctypes.data if uni is not None else None)
    return (out, uni) if with_uniforms else out


# ----------------------------------------------------------------------------
# Grid_FFT helpers
# ----------------------------------------------------------------------------
def fft_r2c(r: np.ndarray) -> np.ndarray:
    """Grid_FFT::FourierTransformForward + ApplyNorm (grid_fft.cc:199-238)."""
    return sfft.rfftn(r, norm="ortho", workers=WORKERS)


def fft_c2r(c: np.ndarray, n: int) -> np.ndarray:
    """Grid_FFT::FourierTransformBackward + ApplyNorm (grid_fft.cc:241-270).

    A c2r transform of a kz = 0 (or kz = N/2) plane that is not exactly
    Hermitian is defined only up to the transform's pass order; with the PLT
    gradient this happens at modes whose CIC stencil touches the PLT table's
    Nyquist node.  The oracle takes the Hermitian part of those planes (what a
    c2c-then-c2r ordering, pocketfft's and FFTW's usual one, computes)."""
    c = hermitian_planes(c, n)
    return sfft.irfftn(c, s=(n, n, n), norm="ortho", workers=WORKERS)


def hermitian_planes(c: np.ndarray, n: int) -> np.ndarray:
    """(X(k) + conj X(-k)) / 2 on the kz = 0 and kz = N/2 planes."""
    idx = (-np.arange(c.shape[0])) % c.shape[0]
    out = c.copy()
    for kz in (0, c.shape[2] - 1) if (n % 2 == 0) else (0,):
        p = c[:, :, kz]
        out[:, :, kz] = 0.5 * (p + np.conj(p[np.ix_(idx, idx)]))
    return out


def _signed(n: int, count: int) -> np.ndarray:
    i = np.arange(count)
    return (i.astype(np.float64) - (i > n // 2).astype(np.float64) * n)


def kvec(n: int, L: float):
    """get_k<real_t>(i,j,k) components as broadcastable arrays (grid_fft.hh:281-296)."""
    kfac = 2.0 * np.pi / L
    kx = (_signed(n, n) * kfac)[:, None, None]
    ky = (_signed(n, n) * kfac)[None, :, None]
    kz = (_signed(n, n // 2 + 1) * kfac)[None, None, :]
    return kx, ky, kz


def grad_factors(n: int, L: float):
    """Imaginary parts of Grid_FFT::gradient for the three axes (grid_fft.hh:376-385):
    (real(i) - (i>N/2)*N)*kfac, zero at i == N/2."""
    kfac = 2.0 * np.pi / L
    g = []
    for axis, cnt in ((0, n), (1, n), (2, n // 2 + 1)):
        i = np.arange(cnt)
        v = np.where(i != n // 2, _signed(n, cnt) * kfac, 0.0)
        shape = [1, 1, 1]
        shape[axis] = cnt
        g.append(v.reshape(shape))
    return g


def kmod2(n: int, L: float):
    kx, ky, kz = kvec(n, L)
    return kx * kx + ky * ky + kz * kz


def inverse_laplacian(f: np.ndarray, n: int, L: float) -> np.ndarray:
    """apply_InverseLaplacian in k-space: -x/|k|^2 then zero_DC_mode (grid_fft.hh:440-449, 844-850)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        out = -f / kmod2(n, L)
    out[0, 0, 0] = 0.0
    return out


# ----------------------------------------------------------------------------
# Orszag 3/2 convolver (convolution.hh:412-652)
# ----------------------------------------------------------------------------
class OrszagConvolver:
    def __init__(self, n: int, L: float):
        assert n % 2 == 0
        self.n, self.L = n, L
        self.m = 3 * n // 2
        nh = n // 2
        i = np.arange(n)
        self.ip = np.where(i > nh, i + nh, i)
        self.g = grad_factors(n, L)
        nyq = np.zeros((n, n, nh + 1), dtype=bool)
        nyq[nh, :, :] = True
        nyq[:, nh, :] = True
        nyq[:, :, nh] = True
        self.nyq = nyq

    # kfunc builders -----------------------------------------------------
    def hessian(self, f, a, b):
        """grad_a * grad_b * f with i*g factors: (i g_a)(i g_b) = -(g_a g_b)."""
        return -(self.g[a] * self.g[b]) * f

    def sum_of_hessians(self, f, ab1, ab2):
        """(grad11*grad12 + grad21*grad22) * f (convolution.hh:208-235)."""
        return (-(self.g[ab1[0]] * self.g[ab1[1]]) + -(self.g[ab2[0]] * self.g[ab2[1]])) * f

    def difference_of_hessians(self, f, ab1, ab2):
        """(grad11*grad12 - grad21*grad22) * f (convolution.hh:248-275)."""
        return (-(self.g[ab1[0]] * self.g[ab1[1]]) - -(self.g[ab2[0]] * self.g[ab2[1]])) * f

    # pad / unpad --------------------------------------------------------
    def pad_insert(self, fk):
        """convolution.hh:552-575."""
        n, m = self.n, self.m
        rfac = np.power(1.5, 1.5)
        out = np.zeros((m, m, m // 2 + 1), dtype=np.complex128)
        out[np.ix_(self.ip, self.ip, np.arange(n // 2 + 1))] = fk * rfac
        return out

    def unpad(self, Fk):
        """convolution.hh:600-636: divide by sqrt(M^3)/sqrt(N^3), zero Nyquist."""
        n, m = self.n, self.m
        rfac = np.sqrt(float(m * m * m)) / np.sqrt(float(n * n * n))
        out = Fk[np.ix_(self.ip, self.ip, np.arange(n // 2 + 1))] / rfac
        out[self.nyq] = 0.0
        return out

    def convolve2(self, k1, k2):
        """convolution.hh:495-518; returns the unpadded N-grid k-space product."""
        m = self.m
        a = fft_c2r(self.pad_insert(k1), m)
        b = fft_c2r(self.pad_insert(k2), m)
        b *= a
        return self.unpad(fft_r2c(b))

    def convolve3(self, k1, k2, k3):
        """convolution.hh:525-532 (pairwise dealiasing)."""
        return self.convolve2(self.convolve2(k1, k2), k3)


# ----------------------------------------------------------------------------
# LPT potentials (ic_generator.cc:378-383, 509-658)
# ----------------------------------------------------------------------------
def normalise_noise(w: np.ndarray, n: int, L: float, fixing: bool, inversion: bool) -> np.ndarray:
    """ic_generator.cc:378-383 with volfac from ic_generator.cc:247."""
    volfac = np.power(L / n / 2.0 / np.pi, 1.5)
    out = w.copy()
    if fixing:
        a = np.abs(out)
        nz = a != 0.0
        out[nz] = out[nz] / a[nz]
    s = -1.0 if inversion else 1.0
    return s * out / volfac


def phi1_from_noise(w: np.ndarray, n: int, L: float, amplitude) -> np.ndarray:
    """ic_generator.cc:509-516: phi = -delta/k^2 with delta = w*amplitude(|k|)."""
    kx, ky, kz = kvec(n, L)
    kmod = np.sqrt(kx * kx + ky * ky + kz * kz)
    with np.errstate(divide="ignore", invalid="ignore"):
        amp = amplitude(kmod)
        phi = -(w * amp) / (kmod * kmod)
    phi[0, 0, 0] = 0.0
    return phi


def lpt_potentials(phi: np.ndarray, n: int, L: float, order: int):
    """ic_generator.cc:523-628.  Returns unscaled (phi2, phi3, [A3x, A3y, A3z])."""
    C = OrszagConvolver(n, L)
    H, S, D = C.hessian, C.sum_of_hessians, C.difference_of_hessians
    phi2 = phi3 = None
    A3 = None
    if order > 1:
        phi2 = C.convolve2(H(phi, 0, 0), S(phi, (1, 1), (2, 2)))
        phi2 = phi2 + C.convolve2(H(phi, 1, 1), H(phi, 2, 2))
        phi2 = phi2 - C.convolve2(H(phi, 0, 1), H(phi, 0, 1))
        phi2 = phi2 - C.convolve2(H(phi, 0, 2), H(phi, 0, 2))
        phi2 = phi2 - C.convolve2(H(phi, 1, 2), H(phi, 1, 2))
        phi2 = inverse_laplacian(phi2, n, L)
    if order > 2:
        phi3 = C.convolve3(H(phi, 0, 0), H(phi, 1, 1), H(phi, 2, 2))
        phi3 = phi3 + C.convolve3(H(phi, 0, 1), H(phi, 0, 2), H(phi, 1, 2)) * 2.0
        phi3 = phi3 - C.convolve3(H(phi, 1, 2), H(phi, 1, 2), H(phi, 0, 0))
        phi3 = phi3 - C.convolve3(H(phi, 0, 2), H(phi, 0, 2), H(phi, 1, 1))
        phi3 = phi3 - C.convolve3(H(phi, 0, 1), H(phi, 0, 1), H(phi, 2, 2))
        c57, c107 = -5.0 / 7.0, +10.0 / 7.0
        phi3 = phi3 + C.convolve2(H(phi, 0, 0), S(phi2, (1, 1), (2, 2))) * c57
        phi3 = phi3 + C.convolve2(H(phi, 1, 1), S(phi2, (2, 2), (0, 0))) * c57
        phi3 = phi3 + C.convolve2(H(phi, 2, 2), S(phi2, (0, 0), (1, 1))) * c57
        phi3 = phi3 + C.convolve2(H(phi, 0, 1), H(phi2, 0, 1)) * c107
        phi3 = phi3 + C.convolve2(H(phi, 0, 2), H(phi2, 0, 2)) * c107
        phi3 = phi3 + C.convolve2(H(phi, 1, 2), H(phi2, 1, 2)) * c107
        phi3 = inverse_laplacian(phi3, n, L)
        A3 = []
        for d in range(3):
            dp, dpp = (d + 1) % 3, (d + 2) % 3
            a = C.convolve2(H(phi2, d, dp), H(phi, d, dpp))
            a = a - C.convolve2(H(phi2, d, dpp), H(phi, d, dp))
            a = a + C.convolve2(H(phi, dp, dpp), D(phi2, (dp, dp), (dpp, dpp)))
            a = a - C.convolve2(H(phi2, dp, dpp), D(phi, (dp, dp), (dpp, dpp)))
            A3.append(inverse_laplacian(a, n, L))
    return phi2, phi3, A3


def lpt_coefficients(dplus: float, vfac: float, order: int):
    """ic_generator.cc:252-269."""
    g1 = -dplus
    g2 = (-3.0 / 7.0 * dplus * dplus) if order > 1 else 0.0
    g3 = (1.0 / 3.0 * dplus * dplus * dplus) if order > 2 else 0.0
    g3c = (1.0 / 7.0 * dplus * dplus * dplus) if order > 2 else 0.0
    return dict(g1=g1, g2=g2, g3=g3, g3c=g3c, vfac1=vfac, vfac2=2 * vfac, vfac3=3 * vfac)


# ----------------------------------------------------------------------------
# Displacement / velocity assembly (ic_generator.cc:916-1060)
# ----------------------------------------------------------------------------
class FourierGradient:
    """op::fourier_gradient (operators.hh:38-61): i*k with the Nyquist index zeroed, vfac_corr = 1."""

    def __init__(self, n: int, L: float):
        self.g = grad_factors(n, L)

    def gradient(self, d):
        return self.g[d]  # imaginary part

    def vfac_corr(self):
        return 1.0


def _times_i(g, f):
    """ccomplex_t(0,g) * f."""
    return 1j * (g * f)


def assemble_displacement(d, fields, coef, grad, lunit, L, order):
    """ic_generator.cc:929-968 for component d; returns the k-space field (DC zeroed)."""
    phi, phi2, phi3, A3 = fields
    dp, dpp = (d + 1) % 3, (d + 2) % 3
    phitot = phi.copy()
    if order > 1:
        phitot = phitot + phi2
    if order > 2:
        phitot = phitot + phi3
    tmp = _times_i(grad.gradient(d), phitot)
    if order > 2:
        tmp = tmp + (_times_i(grad.gradient(dp), A3[dpp]) - _times_i(grad.gradient(dpp), A3[dp]))
    tmp = tmp * (lunit / L)
    tmp[0, 0, 0] = 0.0
    return tmp


def assemble_velocity(d, fields, coef, grad, vunit, L, order):
    """ic_generator.cc:986-1053 for component d (no baryon / neutrino terms)."""
    phi, phi2, phi3, A3 = fields
    dp, dpp = (d + 1) % 3, (d + 2) % 3
    pv = coef["vfac1"] * phi
    if order > 1:
        pv = pv + coef["vfac2"] * phi2
    if order > 2:
        pv = pv + coef["vfac3"] * phi3
    tmp = _times_i(grad.gradient(d), pv)
    if order > 2:
        tmp = tmp + coef["vfac3"] * (_times_i(grad.gradient(dp), A3[dpp]) - _times_i(grad.gradient(dpp), A3[dp]))
    tmp = tmp * grad.vfac_corr()
    tmp = tmp * (vunit / L)
    tmp[0, 0, 0] = 0.0
    return tmp


LATTICE_SHIFTS = {
    # particle_generator.hh:47-54 (SC, BCC, FCC)
    0: [(0.0, 0.0, 0.0)],
    1: [(0.0, 0.0, 0.0), (0.5, 0.5, 0.5)],
    2: [(0.0, 0.0, 0.0), (0.0, 0.5, 0.5), (0.5, 0.0, 0.5), (0.5, 0.5, 0.0)],
}


def shift_field(fr: np.ndarray, s, n: int, L: float) -> np.ndarray:
    """Grid_FFT::shift_field (grid_fft.hh:832-842): r2c, multiply exp(i k.s dx), c2r."""
    kx, ky, kz = kvec(n, L)
    dx = L / n
    fk = fft_r2c(fr)
    shift = s[0] * kx * dx + s[1] * ky * dx + s[2] * kz * dx
    fk = fk * np.exp(1j * shift)
    return fft_c2r(fk, n)


def lattice_read_out(field_r, lattice, n, L, lunit=None):
    """set_positions (lunit given) / set_velocities (lunit None), particle_generator.hh:499-543, 597-639.

    Returns an (n_s*N^3,) array of this component for all particles, ordered
    ishift*N^3 + (i*N + j)*N + k."""
    shifts = LATTICE_SHIFTS[lattice]
    out = []
    f = field_r
    for ish, s in enumerate(shifts):
        if ish > 0:
            prev = shifts[ish - 1]
            f = shift_field(f, (s[0] - prev[0], s[1] - prev[1], s[2] - prev[2]), n, L)
        if lunit is None:
            out.append(f.reshape(-1).copy())
        else:
            idx = np.arange(n, dtype=np.float64)
            comp = []
            for axis in range(3):
                shape = [1, 1, 1]
                shape[axis] = n
                comp.append(((idx + s[axis]) / float(n)).reshape(shape))
            out.append(comp)
    return out


def particles(fields, coef, grad, lattice, n, L, lunit, vunit, order, id_offset=0):
    """Positions, velocities and IDs of all particles as the reference's
    lattice_generator leaves them (particle_generator.hh:212-253, 499-687).

    Returns pos (np_,3), vel (np_,3), ids (np_,) uint64."""
    shifts = LATTICE_SHIFTS[lattice]
    ns = len(shifts)
    n3 = n ** 3
    pos = np.zeros((ns * n3, 3))
    vel = np.zeros((ns * n3, 3))
    for d in range(3):
        fr = fft_c2r(assemble_displacement(d, fields, coef, grad, lunit, L, order), n)
        f = fr
        for ish, s in enumerate(shifts):
            if ish > 0:
                prev = shifts[ish - 1]
                f = shift_field(f, (s[0] - prev[0], s[1] - prev[1], s[2] - prev[2]), n, L)
            idx = np.arange(n, dtype=np.float64)
            shape = [1, 1, 1]
            shape[d] = n
            q = ((idx + s[d]) / float(n)).reshape(shape)
            pos[ish * n3:(ish + 1) * n3, d] = (q * lunit + f).reshape(-1)
    for d in range(3):
        fr = fft_c2r(assemble_velocity(d, fields, coef, grad, vunit, L, order), n)
        f = fr
        for ish, s in enumerate(shifts):
            if ish > 0:
                prev = shifts[ish - 1]
                f = shift_field(f, (s[0] - prev[0], s[1] - prev[1], s[2] - prev[2]), n, L)
            vel[ish * n3:(ish + 1) * n3, d] = f.reshape(-1)
    cell = np.arange(n3, dtype=np.uint64)
    ids = np.zeros(ns * n3, dtype=np.uint64)
    off = np.uint64(id_offset * ns * n3)
    for il in range(ns):
        ids[il * n3:(il + 1) * n3] = off + np.uint64(ns) * cell + np.uint64(il)
    return pos, vel, ids


# particle_generator.hh:56-63: the secondary lattice of a second species
SECOND_LATTICE_SHIFT = {0: (0.5, 0.5, 0.5), 1: (0.5, 0.5, 0.0), 2: (0.5, 0.5, 0.5)}


def amp_of_index(table, n, L):
    """A per-mode array from a table indexed by |k|^2 / kf^2 = i^2 + j^2 + k^2
    over signed mode indices (zero beyond the table)."""
    i = _signed(n, n)
    kk = np.arange(n // 2 + 1, dtype=np.float64)
    q = (i[:, None, None] ** 2 + i[None, :, None] ** 2 + kk[None, None, :] ** 2).astype(np.int64)
    t = np.asarray(table, dtype=np.float64)
    out = np.zeros(q.shape)
    ok = q < len(t)
    out[ok] = t[q[ok]]
    return out


def species_particles(fields, noise, coef, grad, lattice, n, L, lunit, vunit, order, c_species,
                      mass_factor, amp_dbc=None, amp_tbc=None, secondary=False, id_offset=0):
    """One species of a baryon + CDM run (ic_generator.cc:706-1064): positions
    from the shared LPT displacement on the species' lattice (the secondary
    lattice for baryons, shifted by SECOND_LATTICE_SHIFT before the read-out,
    particle_generator.hh:388-395, 510-517), velocities with the linear
    relative-velocity term -vfac1 C A_theta_bc(k) w grad_d / k^2 added before
    vfac_corr (ic_generator.cc:1016-1020), masses (1 + C delta_bc(x)) *
    mass_factor / (n_s N^3) with delta_bc(k) = w A_delta_bc(k)
    (ic_generator.cc:749-780, particle_generator.hh:369-427), ids with the
    species' IDoffset.  amp_dbc / amp_tbc: get_amplitude_delta_bc /
    get_amplitude_theta_bc per |k|^2 index (None: zero).
    Returns pos, vel, ids, masses."""
    phi, phi2, phi3, A3 = fields
    shifts = LATTICE_SHIFTS[lattice]
    ns = len(shifts)
    n3 = n ** 3
    kx, ky, kz = kvec(n, L)
    k2 = kx * kx + ky * ky + kz * kz
    sec = SECOND_LATTICE_SHIFT[lattice] if secondary else (0.0, 0.0, 0.0)

    def read_out(f, d=None, q_unit=None):
        out = np.zeros(ns * n3)
        for ish, s in enumerate(shifts):
            if ish == 0 and secondary:
                f = shift_field(f, sec, n, L)
            if ish > 0:
                prev = shifts[ish - 1]
                f = shift_field(f, (s[0] - prev[0], s[1] - prev[1], s[2] - prev[2]), n, L)
            vals = f.reshape(-1)
            if d is not None:
                idx = np.arange(n, dtype=np.float64)
                shape = [1, 1, 1]
                shape[d] = n
                qd = ((idx + s[d] + sec[d]) / float(n)).reshape(shape)
                vals = (qd * q_unit + f).reshape(-1)
            out[ish * n3:(ish + 1) * n3] = vals
        return out

    pos = np.zeros((ns * n3, 3))
    vel = np.zeros((ns * n3, 3))
    for d in range(3):
        pos[:, d] = read_out(fft_c2r(assemble_displacement(d, fields, coef, grad, lunit, L, order), n), d, lunit)
    tbc = amp_of_index(amp_tbc, n, L) if amp_tbc is not None else None
    for d in range(3):
        dp, dpp = (d + 1) % 3, (d + 2) % 3
        pv = coef["vfac1"] * phi
        if order > 1:
            pv = pv + coef["vfac2"] * phi2
        if order > 2:
            pv = pv + coef["vfac3"] * phi3
        tmp = _times_i(grad.gradient(d), pv)
        if order > 2:
            tmp = tmp + coef["vfac3"] * (_times_i(grad.gradient(dp), A3[dpp]) - _times_i(grad.gradient(dpp), A3[dp]))
        if tbc is not None:
            with np.errstate(divide="ignore", invalid="ignore"):
                term = coef["vfac1"] * c_species * tbc * noise * 1j * grad.gradient(d) / k2
            term[0, 0, 0] = 0.0
            tmp = tmp - term
        tmp = tmp * grad.vfac_corr()
        tmp = tmp * (vunit / L)
        tmp[0, 0, 0] = 0.0
        vel[:, d] = read_out(fft_c2r(tmp, n))
    masses = np.full(ns * n3, mass_factor / (ns * n3))
    if amp_dbc is not None:
        rho = noise * amp_of_index(amp_dbc, n, L)
        rho[0, 0, 0] = 0.0
        r = fft_c2r(rho, n)
        r = (1.0 + c_species * r) * mass_factor
        masses = read_out(r) / (ns * n3)
    cell = np.arange(n3, dtype=np.uint64)
    ids = np.zeros(ns * n3, dtype=np.uint64)
    off = np.uint64(id_offset * ns * n3)
    for il in range(ns):
        ids[il * n3:(il + 1) * n3] = off + np.uint64(ns) * cell + np.uint64(il)
    return pos, vel, ids, masses


def ppt_fields(phi_s, phi2_s, noise, order, n, L, dplus, vfac, vunit, c_species=0.0, amp_dbc=None):
    """Semiclassical (PPT) Eulerian density and velocity fields of one species,
    ic_generator.cc:783-901: rho = sqrt(1 + C delta_bc(x)); hbar from the
    largest nearest-neighbour step of the real-space phi (the x loop stops one
    short of the last plane, ic_generator.cc:813-829) as maxdphi / pi / D+ x
    1.01; psi = rho exp(i (phi [+ phi2]) / (hbar D+)); one drift step
    exp(-i hbar k^2 D+ / 2) in k-space; for 2LPT and above a second kick
    exp(i phi2 / (hbar D+)); delta = |psi|^2 - 1 and
    v_d = vunit' Re[(conj(psi) d_d psi - psi conj(d_d psi)) / (2i / hbar)] / (1 + delta)
    with vunit' = D+ vfac / L * vunit.  phi_s, phi2_s: the growth-scaled
    potentials (k-space).  Returns delta, (vx, vy, vz), hbar."""
    phir = fft_c2r(phi_s, n)
    rho = np.ones((n, n, n))
    if amp_dbc is not None:
        d = noise * amp_of_index(amp_dbc, n, L)
        d[0, 0, 0] = 0.0
        rho = np.sqrt(1.0 + c_species * fft_c2r(d, n))
    dx = np.abs(np.roll(phir, -1, axis=0) - phir)[:n - 1]
    dy = np.abs(np.roll(phir, -1, axis=1) - phir)[:n - 1]
    dz = np.abs(np.roll(phir, -1, axis=2) - phir)[:n - 1]
    maxdphi = max(dx.max(), dy.max(), dz.max())
    hbar = maxdphi / np.pi / dplus * 1.01
    if order == 1:
        psi = rho * np.exp(1j / hbar * (phir / dplus))
    else:
        phi2r = fft_c2r(phi2_s, n)
        psi = rho * np.exp(1j / hbar * (phir + phi2r) / dplus)
    kfac = 2.0 * np.pi / L
    k1 = _signed(n, n) * kfac
    kx, ky, kz = k1[:, None, None], k1[None, :, None], k1[None, None, :]
    k2 = kx * kx + ky * ky + kz * kz
    psi = np.fft.ifftn(np.fft.fftn(psi) * np.exp(-0.5j * hbar * k2 * dplus))
    if order >= 2:
        psi = psi * np.exp(1j / hbar * phi2r / dplus)
    delta = psi.real ** 2 + psi.imag ** 2 - 1.0
    vu = dplus * vfac / L * vunit
    vel = []
    fk = np.fft.fftn(psi)
    for kd in (kx, ky, kz):
        g = np.fft.ifftn(fk * (1j * kd))
        vel.append(vu * np.real((np.conj(psi) * g - psi * np.conj(g)) / (2.0j / hbar)) / (1.0 + delta))
    return delta, vel, hbar


def run_lpt(n, L, seed_table, amplitude, order, dplus, vfac, lattice=0, lunit=1.0, vunit=1.0,
            fixing=False, inversion=False, grad=None, want_particles=True, noise=None):
    """The whole hot path, ic_generator.cc:288-1064, for one species (dm, no baryons).

    noise: the raw k-space white noise of another generator (music_fill, before
    normalisation) in place of NGenIC's from seed_table."""
    w = ngenic_fill(n, seed_table) if noise is None else noise
    w = normalise_noise(w, n, L, fixing, inversion)
    phi = phi1_from_noise(w, n, L, amplitude)
    phi2, phi3, A3 = lpt_potentials(phi, n, L, order)
    c = lpt_coefficients(dplus, vfac, order)
    phi_s = phi * c["g1"]
    phi2_s = phi2 * c["g2"] if order > 1 else None
    phi3_s = phi3 * c["g3"] if order > 2 else None
    A3_s = [a * c["g3c"] for a in A3] if order > 2 else None
    res = dict(noise=w, phi=phi_s, phi2=phi2_s, phi3=phi3_s, A3=A3_s, coef=c)
    if want_particles:
        g = grad if grad is not None else FourierGradient(n, L)
        pos, vel, ids = particles((phi_s, phi2_s, phi3_s, A3_s), c, g, lattice, n, L, lunit, vunit, order)
        res.update(pos=pos, vel=vel, ids=ids)
    return res
