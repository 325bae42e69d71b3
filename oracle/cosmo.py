"""ORACLE -- test infrastructure only.

Independent numpy/scipy restatement of the cosmology the hot path consumes:
H(a) (cosmology_calculator.hh:334-342), the linear growth factor D+(a)
(cosmology_calculator.hh:92-152, here by scipy's adaptive integrator rather
than the reference's Cash-Karp stepper), the sigma_8 normalisation
(cosmology_calculator.hh:441-511, here scipy.integrate.quad), vfact
(cosmology_calculator.hh:373-376) and the Eisenstein & Hu transfer function
(src/plugins/transfer_eisenstein.cc:58-243).

Used to check the product's C++ cosmology; the engine parity tests feed both
sides the same scalars.
"""
from __future__ import annotations

import numpy as np
from scipy import integrate


def eisenstein_hu(k_hmpc, H0, Om, Ob, Tcmb):
    """transfer_eisenstein.cc:58-201 at_k(): fb*T_b + fc*T_c at k in h/Mpc."""
    h0 = H0 * 0.01
    omhh = Om * H0 * H0 * 1e-4
    fbar = Ob / Om
    obhh = omhh * fbar
    th = Tcmb / 2.7
    z_eq = 2.50e4 * omhh / th ** 4
    k_eq = 0.0746 * omhh / th ** 2
    b1 = 0.313 * omhh ** -0.419 * (1 + 0.607 * omhh ** 0.674)
    b2 = 0.238 * omhh ** 0.223
    z_d = 1291 * omhh ** 0.251 / (1 + 0.659 * omhh ** 0.828) * (1 + b1 * obhh ** b2)
    R_d = 31.5 * obhh / th ** 4 * (1000 / (1 + z_d))
    R_eq = 31.5 * obhh / th ** 4 * (1000 / z_eq)
    s = 2. / 3. / k_eq * np.sqrt(6. / R_eq) * np.log((np.sqrt(1 + R_d) + np.sqrt(R_d + R_eq)) / (1 + np.sqrt(R_eq)))
    k_silk = 1.6 * obhh ** 0.52 * omhh ** 0.73 * (1 + (10.4 * omhh) ** -0.95)
    a1 = (46.9 * omhh) ** 0.670 * (1 + (32.1 * omhh) ** -0.532)
    a2 = (12.0 * omhh) ** 0.424 * (1 + (45.0 * omhh) ** -0.582)
    a_c = a1 ** -fbar * a2 ** -(fbar ** 3)
    bb1 = 0.944 / (1 + (458 * omhh) ** -0.708)
    bb2 = (0.395 * omhh) ** -0.0266
    b_c = 1.0 / (1 + bb1 * ((1 - fbar) ** bb2 - 1))
    y = z_eq / (1 + z_d)
    G = y * (-6. * np.sqrt(1 + y) + (2. + 3. * y) * np.log((np.sqrt(1 + y) + 1) / (np.sqrt(1 + y) - 1)))
    a_b = 2.07 * k_eq * s * (1 + R_d) ** -0.75 * G
    b_node = 8.41 * omhh ** 0.435
    b_b = 0.5 + fbar + (3. - 2. * fbar) * np.sqrt((17.2 * omhh) ** 2.0 + 1)
    k = np.abs(np.asarray(k_hmpc, dtype=float) * h0)
    with np.errstate(divide="ignore", invalid="ignore"):
        q = k / 13.41 / k_eq
        xx = k * s
        lnb = np.log(2.718282 + 1.8 * b_c * q)
        lnn = np.log(2.718282 + 1.8 * q)
        Ca = 14.2 / a_c + 386.0 / (1 + 69.9 * q ** 1.08)
        Cn = 14.2 + 386.0 / (1 + 69.9 * q ** 1.08)
        f = 1.0 / (1.0 + (xx / 5.4) ** 4)
        Tc = f * lnb / (lnb + Cn * q * q) + (1 - f) * lnb / (lnb + Ca * q * q)
        st = s * (1. + (b_node / xx) ** 3) ** (-1. / 3.)
        xt = k * st
        T0 = lnn / (lnn + Cn * q * q)
        Tb = np.sin(xt) / xt * (T0 / (1. + (xx / 5.2) ** 2) + a_b / (1. + (b_b / xx) ** 3) * np.exp(-(k / k_silk) ** 1.4))
    Tb = np.where(k == 0, 1.0, Tb)
    Tc = np.where(k == 0, 1.0, Tc)
    return fbar * Tb + (Om - Ob) / Om * Tc


class Cosmology:
    """Flat LCDM without radiation (ZeroRadiation, m_nu = 0) as in the benchmark configs."""

    def __init__(self, Om=0.3, Ob=0.045, H0=70.0, n_s=0.965, sigma8=0.81, Tcmb=2.7255, OL=None):
        self.Om, self.Ob, self.H0, self.n_s, self.sigma8, self.Tcmb = Om, Ob, H0, n_s, sigma8, Tcmb
        self.h = H0 / 100.0
        self.OL = 1.0 - Om if OL is None else OL
        self.Dnow = self._D(1.0)
        self.pnorm = sigma8 ** 2 / self._sigma8_unnorm() ** 2
        self.sqrtpnorm = np.sqrt(self.pnorm)

    def H(self, a):
        return self.H0 * np.sqrt(self.Om / a ** 3 + self.OL)

    def _D(self, a):
        # growing mode of D'' + (3/a + dlnH/da) D' - 3/2 Om H0^2/(a^5 H^2) D = 0 in a,
        # started deep in matter domination where D = a
        a0 = 1e-5

        def rhs(a, y):
            D, Dp = y
            H = self.H(a)
            dlnH = -1.5 * self.H0 ** 2 * self.Om / a ** 4 / H ** 2
            return [Dp, -(3.0 / a + dlnH) * Dp + 1.5 * self.Om * self.H0 ** 2 / (a ** 5 * H ** 2) * D]

        sol = integrate.solve_ivp(rhs, (a0, a), [a0, 1.0], rtol=1e-12, atol=1e-18, method="DOP853")
        return sol.y[0, -1], sol.y[1, -1]

    def growth(self, a):
        return self._D(a)[0] / self.Dnow[0]

    def f(self, a):
        D, Dp = self._D(a)
        return a * Dp / D

    def vfact(self, a):
        return self.f(a) * a * self.H(a) / self.h

    def transfer(self, k):
        return eisenstein_hu(k, self.H0, self.Om, self.Ob, self.Tcmb)

    def _sigma8_unnorm(self):
        def integrand(u):
            k = np.exp(u)
            x = 8.0 * k
            w = 1.0 - 0.1 * x * x if x < 0.001 else 3.0 * (np.sin(x) - x * np.cos(x)) / x ** 3
            T = self.transfer(k)
            return k * k * k * w * w * k ** self.n_s * T * T

        val, _ = integrate.quad(integrand, np.log(1e-4), np.log(1e4), epsabs=0, epsrel=1e-13, limit=2000)
        return np.sqrt(4.0 * np.pi * val)

    def amplitude(self, k):
        k = np.asarray(k, dtype=float)
        return np.power(k, 0.5 * self.n_s) * self.transfer(k) * self.sqrtpnorm
