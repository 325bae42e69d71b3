"""ORACLE -- test infrastructure only.

numpy restatement of monofonIC's PLT (particle linear theory) correction,
``particle::lattice_gradient`` (include/particle_plt.hh:50-587):

* ``plt_tables(lattice)``: ``init_D`` (particle_plt.hh:68-515) -- Ewald-summed
  dynamical matrix on the 64^3 mesh (176-273), its FFT (283-288), per-mode
  eigensystem and first-Brillouin-zone fold with first-insert-wins in the
  reference's serial loop order (302-395), neighbour interpolation (405-459)
  and the production tables (461-499).
* ``PLTGradient``: ``gradient`` and ``vfac_corr`` (551-585) with the k-space
  CIC interpolation ``get_cic_kspace`` (grid_fft.hh:347-373).

Parity status: the reference gets the eigensystem from GSL's ``symmv``; this
file uses LAPACK (numpy.linalg.eigh).  Both give the same eigenvalues and the
same eigenvectors up to sign (the sign is fixed by ``align_with_k``) except
where the largest eigenvalue is degenerate.  No reference output exists to
pin the tables ("parity unpinned").
"""
from __future__ import annotations

import numpy as np
from scipy.special import erfc

NG = 64
NK = NG // 2 + 1

_PI = np.pi


def lattice_props(ilat: int):
    pi, twopi, fourpi = _PI, 2 * _PI, 4 * _PI
    if ilat == 0:
        B = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
        R = np.array([[twopi, 0, 0], [0, twopi, 0], [0, 0, twopi]])
        IR = np.array([[2, 0, 0], [0, 2, 0], [0, 0, 2]])
        cf = 1
        normals = [(pi, 0, 0), (-pi, 0, 0), (0, pi, 0), (0, -pi, 0), (0, 0, pi), (0, 0, -pi)]
    elif ilat == 1:
        B = np.array([[1, 0, 0.5], [0, 1, 0.5], [0, 0, 0.5]])
        R = np.array([[twopi, 0, 0], [0, twopi, 0], [-twopi, -twopi, fourpi]])
        IR = np.array([[2, 0, 0], [0, 2, 0], [1, 1, 1]])
        cf = 2
        normals = [(0, pi, pi), (0, -pi, pi), (0, pi, -pi), (0, -pi, -pi), (pi, 0, pi), (-pi, 0, pi),
                   (pi, 0, -pi), (-pi, 0, -pi), (pi, pi, 0), (-pi, pi, 0), (pi, -pi, 0), (-pi, -pi, 0)]
    else:
        B = np.array([[0, 0.5, 0], [0.5, 0, 1], [0.5, 0.5, 0]])
        R = np.array([[-fourpi, fourpi, twopi], [0, 0, twopi], [fourpi, 0, -twopi]])
        IR = np.array([[0, 1, 1], [1, 0, 1], [0, 2, 0]])
        cf = 4
        normals = [(twopi, 0, 0), (-twopi, 0, 0), (0, twopi, 0), (0, -twopi, 0), (0, 0, twopi), (0, 0, -twopi),
                   (pi, pi, pi), (pi, pi, -pi), (pi, -pi, pi), (pi, -pi, -pi), (-pi, pi, pi), (-pi, pi, -pi),
                   (-pi, -pi, pi), (-pi, -pi, -pi)]
    return B, R, IR, cf, np.array(normals, float)


def ewald_real_space(ilat: int) -> np.ndarray:
    """D_ij at every site of the 64^3 mesh (particle_plt.hh:218-281); shape (6, 64, 64, 64)
    in the order xx, xy, xz, yy, yz, zz."""
    B, R, IR, cf, _ = lattice_props(ilat)
    dx = 1.0 / NG
    eta = 4.0
    alpha = 1.0 / np.sqrt(2) / eta
    a2, a3 = alpha * alpha, alpha ** 3
    sqrtpi, pi32, fourpi = np.sqrt(_PI), np.power(_PI, 1.5), 4 * _PI
    charge = 1.0 / np.power(float(NG), 3) / cf
    fft_norm = 1.0 / np.power(float(NG), 3.0)
    idx = np.arange(NG)
    I, J, K = np.meshgrid(idx, idx, idx, indexing="ij")
    x = np.stack([dx * I.ravel(), dx * J.ravel(), dx * K.ravel()], axis=1)  # (S,3)
    ar = x @ B.T
    ar = np.fmod(2.0 + ar, 1.0)
    rng = np.arange(-3, 4)
    n = np.stack(np.meshgrid(rng, rng, rng, indexing="ij"), axis=-1).reshape(-1, 3).astype(float)  # (343,3)
    bn = n @ B.T
    m = n[np.abs(n).sum(axis=1) != 0] / NG
    ak = m @ R.T  # (342,3)
    kmod2 = (ak ** 2).sum(axis=1)
    kfac = np.exp(-kmod2 / (4 * a2)) / kmod2 * fft_norm
    pairs = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    out = np.zeros((6, ar.shape[0]))
    chunk = 8192
    for s0 in range(0, ar.shape[0], chunk):
        a = ar[s0:s0 + chunk]
        d = a[:, None, :] - bn[None, :, :]  # (c,343,3)
        r = np.sqrt((d ** 2).sum(axis=2))
        ok = r >= 1e-14
        rs = np.where(ok, r, 1.0)
        r2, r3 = rs * rs, rs * rs * rs
        r5 = r3 * r2
        ex = np.exp(-a2 * r2)
        K1 = -a3 / pi32 * ex / r2
        K2 = (erfc(alpha * rs) + 2.0 * alpha / sqrtpi * ex * rs) / fourpi
        kr = a @ ak.T  # (c,342)
        term = np.cos(kr) * kfac[None, :]
        for c, (mu, nu) in enumerate(pairs):
            dd = d[:, :, mu] * d[:, :, nu] * K1 + ((1.0 if mu == nu else 0.0) / r3 - 3.0 * (d[:, :, mu] * d[:, :, nu]) / r5) * K2
            sr = np.where(ok, dd, 0.0).sum(axis=1)
            lr = (ak[None, :, mu] * ak[None, :, nu] * term).sum(axis=1)
            out[c, s0:s0 + chunk] = (sr + lr) * charge
    out = out.reshape(6, NG, NG, NG)
    out[:, 0, 0, 0] = [1.0 / 3.0, 0.0, 0.0, 1.0 / 3.0, 0.0, 1.0 / 3.0]
    return out


def _signed(i, n=NG):
    return i.astype(float) - (i > n // 2).astype(float) * n


def tables_from_dk(ilat: int, Dk: np.ndarray) -> np.ndarray:
    """Host half of init_D given the 6 raw-DFT k-space components (6,64,64,33)."""
    B, R, IR, cf, normals = lattice_props(ilat)
    twopi = 2 * _PI
    nm = NG * NG * NK
    Dre = Dk.real.reshape(6, nm)
    i, j, k = np.meshgrid(np.arange(NG), np.arange(NG), np.arange(NK), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    kv = np.stack([_signed(i), _signed(j), _signed(k)], axis=1) * twopi
    Dm = np.zeros((nm, 3, 3))
    Dm[:, 0, 0] = Dre[0]
    Dm[:, 0, 1] = Dm[:, 1, 0] = Dre[1]
    Dm[:, 0, 2] = Dm[:, 2, 0] = Dre[2]
    Dm[:, 1, 1] = Dre[3]
    Dm[:, 1, 2] = Dm[:, 2, 1] = Dre[4]
    Dm[:, 2, 2] = Dre[5]
    ev, V = np.linalg.eigh(Dm)  # ascending
    e3 = V[:, :, 2] / (twopi * NG)
    a = (kv / (twopi * NG)) @ R.T  # (nm,3)
    # candidates in the reference's loop order (l1, l2, l3, isign)
    cands = []
    for l1 in (-1, 0, 1):
        for l2 in (-1, 0, 1):
            for l3 in (-1, 0, 1):
                for isign in (0, 1):
                    cands.append((2.0 * isign - 1.0, np.array([l1, l2, l3], float) @ R.T))
    nn = (normals ** 2).sum(axis=1)
    keys_all, q_all, ord_all = [], [], []
    has = np.zeros(nm, bool)
    for ci, (sign, rv) in enumerate(cands):
        vk = sign * a + rv[None, :]
        ok = np.all(vk @ normals.T <= 1.0001 * nn[None, :], axis=1)
        qs = np.nonzero(ok)[0]
        if qs.size == 0:
            continue
        # std::round: halves away from zero
        key = np.sign(vk[qs] * NG / twopi) * np.floor(np.abs(vk[qs] * NG / twopi) + 0.5)
        keys_all.append(key.astype(np.int64))
        q_all.append(qs)
        ord_all.append(qs * len(cands) + ci)
        has[qs] = True
    keys = np.concatenate(keys_all)
    qv = np.concatenate(q_all)
    order = np.concatenate(ord_all)
    srt = np.argsort(order, kind="stable")
    keys, qv = keys[srt], qv[srt]
    enc = (keys[:, 0] + 512) * 1024 * 1024 + (keys[:, 1] + 512) * 1024 + (keys[:, 2] + 512)
    uenc, first = np.unique(enc, return_index=True)
    uq = qv[first]
    eig = np.concatenate([ev[:, ::-1], e3], axis=1)  # (eval2, eval1, eval0, e3x, e3y, e3z)

    def lookup(ii, jj, kk):
        e = (ii + 512) * 1024 * 1024 + (jj + 512) * 1024 + (kk + 512)
        pos = np.searchsorted(uenc, e)
        pos = np.minimum(pos, uenc.size - 1)
        found = uenc[pos] == e
        return found, uq[pos]

    ii = np.where(i > NG // 2, i - NG, i)
    jj = np.where(j > NG // 2, j - NG, j)
    kk = np.where(k > NG // 2, k - NG, k)
    kvi = np.stack([ii, jj, kk], axis=1).astype(float)

    def align(v):
        dot = (v * kvi).sum(axis=1)
        return np.where((dot < 0.0)[:, None], -v, v)

    vi = np.stack([i, j, k], axis=1)
    inlat = np.all((vi @ IR.T) % 2 == 0, axis=1)
    l = np.zeros((nm, 3))
    v = np.zeros((nm, 3))
    # on-lattice modes
    f, q = lookup(ii, jj, kk)
    sel = inlat & f
    l[sel] = eig[q[sel], :3]
    v[sel] = align(eig[q, 3:])[sel]
    # off-lattice: neighbour average (the reference's order of the six neighbours)
    cnt = np.zeros(nm)
    ls = np.zeros((nm, 3))
    vs = np.zeros((nm, 3))
    for (di, dj, dk) in ((-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)):
        f, q = lookup(ii + di, jj + dj, kk + dk)
        m = (~inlat) & f
        cnt += m
        ls += np.where(m[:, None], eig[q, :3], 0.0)
        vs += np.where(m[:, None], align(eig[q, 3:]), 0.0)
    off = ~inlat
    with np.errstate(invalid="ignore", divide="ignore"):
        l[off] = ls[off] / cnt[off, None]
        v[off] = vs[off] / cnt[off, None]
    # production tables
    mu1 = l[:, 0]
    with np.errstate(invalid="ignore", divide="ignore"):
        e1 = v / np.sqrt((v ** 2).sum(axis=1))[:, None]
    kx, ky, kz = kv[:, 0], kv[:, 1], kv[:, 2]
    kr = np.sqrt(kx * kx + ky * ky + kz * kz)
    with np.errstate(invalid="ignore", divide="ignore"):
        kphi = np.where(kr > 0, np.arctan2(ky, kx), 0.0)
        kth = np.where(kr > 0, np.arccos(np.where(kr > 0, kz / np.where(kr > 0, kr, 1.0), 1.0)), 0.0)
    st, ct, sp, cp = np.sin(kth), np.cos(kth), np.sin(kphi), np.cos(kphi)
    er = np.stack([st * cp, st * sp, ct], 1)
    et = np.stack([ct * cp, ct * sp, -st], 1)
    ep = np.stack([-sp, cp, np.zeros_like(sp)], 1)
    renorm = (e1 * er).sum(axis=1)
    renorm = np.where(renorm < 0.01, 1.0, renorm)
    out = np.zeros((4, nm))
    out[0] = 1.0
    out[1] = (e1 * et).sum(axis=1) / renorm
    out[2] = (e1 * ep).sum(axis=1) / renorm
    with np.errstate(invalid="ignore", divide="ignore"):
        out[3] = 1.0 / (0.25 * (np.sqrt(1.0 + 24 * mu1) - 1.0))
    out[:, 0] = [1.0, 0.0, 0.0, 1.0]
    return out.reshape(4, NG, NG, NK)


def plt_tables(ilat: int) -> np.ndarray:
    """(4, 64, 64, 33): D_r, D_theta, D_phi, alpha^{-1}."""
    Dr = ewald_real_space(ilat)
    Dk = np.fft.rfftn(Dr, axes=(1, 2, 3))
    return tables_from_dk(ilat, Dk)


def cic_kspace(T: np.ndarray, x, y, z):
    """Grid_FFT::get_cic_kspace on a (64,64,33) real table (grid_fft.hh:347-373)."""
    ix, iy, iz = np.floor(x).astype(int), np.floor(y).astype(int), np.floor(z).astype(int)
    dx, dy, dz = x - ix, y - iy, z - iz
    tx, ty, tz = 1.0 - dx, 1.0 - dy, 1.0 - dz
    ix1, iy1, iz1 = (ix + 1) % 64, (iy + 1) % 64, np.minimum(iz + 1, 32)
    v = 0.0
    v = v + T[ix, iy, iz] * tx * ty * tz
    v = v + T[ix, iy, iz1] * tx * ty * dz
    v = v + T[ix, iy1, iz] * tx * dy * tz
    v = v + T[ix, iy1, iz1] * tx * dy * dz
    v = v + T[ix1, iy, iz] * dx * ty * tz
    v = v + T[ix1, iy, iz1] * dx * ty * dz
    v = v + T[ix1, iy1, iz] * dx * dy * tz
    v = v + T[ix1, iy1, iz1] * dx * dy * dz
    return v


class PLTGradient:
    """lattice_gradient::gradient / vfac_corr evaluated on the N-grid k-space modes."""

    def __init__(self, n: int, L: float, tables: np.ndarray):
        mapratio = float(NG) / float(n)
        i, j, k = np.meshgrid(np.arange(n), np.arange(n), np.arange(n // 2 + 1), indexing="ij")
        x, y, z = i * mapratio, j * mapratio, k * mapratio
        twopi = 2.0 * _PI
        kx = (x - (x > 32.0) * 64.0) * twopi
        ky = (y - (y > 32.0) * 64.0) * twopi
        kz = (z - (z > 32.0) * 64.0) * twopi
        kr = np.sqrt(kx * kx + ky * ky + kz * kz)
        kmod = kr / mapratio / L
        Dr = cic_kspace(tables[0], x, y, z)
        Dt = cic_kspace(tables[1], x, y, z)
        Dp = cic_kspace(tables[2], x, y, z)
        with np.errstate(invalid="ignore", divide="ignore"):
            kphi = np.where(kr > 0, np.arctan2(ky, kx), 0.0)
            kth = np.where(kr > 0, np.arccos(np.where(kr > 0, kz / np.where(kr > 0, kr, 1.0), 1.0)), 0.0)
        st, ct, sp, cp = np.sin(kth), np.cos(kth), np.sin(kphi), np.cos(kphi)
        self.g = [kmod * (Dr * st * cp + Dt * ct * cp - Dp * sp),
                  kmod * (Dr * st * sp + Dt * ct * sp + Dp * cp),
                  kmod * (Dr * ct - Dt * st)]
        alpha = 1.0 / cic_kspace(tables[3], x, y, z)
        self.vc = 1.0 / alpha

    def gradient(self, d):
        return self.g[d]

    def vfac_corr(self):
        return self.vc
