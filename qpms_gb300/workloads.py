"""Seeded synthetic workloads with the shapes and value distributions of the
benchmark configurations (there is no public dataset for this path).

Physical constants are scipy.constants' CODATA values, as qpms/constants.py
uses them (eV, hbar, c).
"""
import numpy as np

EV = 1.602176634e-19
HBAR = 1.054571817e-34
C0 = 299792458.0


def eV_to_omega(E_eV):
    return np.asarray(E_eV) * EV / HBAR


def translation_vectors(n, seed=2024, n_medium=1.5, rmin=50e-9, rmax=10e-6, E_lo=1.6, E_hi=2.6,
                        im_frac=1e-3):
    """Config 'batched translation-operator kernel': n separation vectors with
    |r| log-uniform on [rmin, rmax], directions uniform on the sphere, complex k
    with Re k = n_medium * omega / c (hbar omega ~ U[E_lo, E_hi] eV) and
    Im k ~ U[0, im_frac * Re k].  Returns kr (complex128), theta, phi."""
    rng = np.random.default_rng(seed)
    r = np.exp(rng.uniform(np.log(rmin), np.log(rmax), n))
    cth = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2 * np.pi, n)
    omega = eV_to_omega(rng.uniform(E_lo, E_hi, n))
    kre = n_medium * omega / C0
    kim = rng.uniform(0.0, im_frac, n) * kre
    kr = (kre + 1j * kim) * r
    return kr.astype(np.complex128), np.arccos(cth), phi
