"""Generates the small golden fixtures of tests/golden/ from the oracle.

The reference publishes no golden vectors and cannot be built here (it needs
FFTW3, GSL and HDF5), so these fixtures pin the oracle against regressions
and give the GPU tests fixed expected values:

* ngenic_16.npz: the first 600 ranlxd1 words for seed 12345, the 16^2 NGenIC
  seed table and the 16^3 k-space white noise (random_ngenic.cc:39-154).
* lpt_16.npz: phi(1), phi(2), phi(3), A(3) (unscaled) and the SC particle
  positions / velocities / IDs of a 16^3 3LPT run, with the scalar inputs used.

Run:  python tests/golden/make_golden.py
"""
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from oracle import cosmo, lpt  # noqa: E402


def main():
    seed, n = 12345, 16
    words = lpt.ranlxd1_words(seed, 600)
    table = lpt.ngenic_seed_table(seed, n)
    noise = lpt.ngenic_fill(n, table)
    np.savez_compressed(HERE / "ngenic_16.npz", seed=seed, words=words, seed_table=table, noise=noise)

    L, z, order = 50.0, 24.0, 3
    c = cosmo.Cosmology(Om=0.3, Ob=0.045, H0=70.0, n_s=0.965, sigma8=0.81)
    a = 1.0 / (1.0 + z)
    dplus, vfac = c.growth(a), c.vfact(a)
    res = lpt.run_lpt(n, L, table, c.amplitude, order, dplus, vfac, lattice=0, lunit=L, vunit=L)
    np.savez_compressed(HERE / "lpt_16.npz", n=n, L=L, order=order, dplus=dplus, vfac=vfac,
                        sqrtpnorm=c.sqrtpnorm, n_s=c.n_s,
                        phi=res["phi"] / res["coef"]["g1"], phi2=res["phi2"] / res["coef"]["g2"],
                        phi3=res["phi3"] / res["coef"]["g3"],
                        A3=np.stack(res["A3"]) / res["coef"]["g3c"],
                        pos=res["pos"], vel=res["vel"], ids=res["ids"])


if __name__ == "__main__":
    main()
