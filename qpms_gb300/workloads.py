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


def square_lattice(a=580e-9):
    """Square lattice, one particle at the origin: (b1, b2, positions)."""
    return (a, 0.0), (0.0, a), np.zeros((1, 3))


def honeycomb_lattice(a=580e-9):
    """Hexagonal Bravais lattice of constant a with two particles at
    +-(a/sqrt 3)/2 along x (nearest-neighbour distance a/sqrt 3)."""
    d = a / np.sqrt(3) / 2
    return (a, 0.0), (a / 2, a * np.sqrt(3) / 2), np.array([[-d, 0, 0], [d, 0, 0]])


def kpath(points, n):
    """n points uniform in arc length along the polyline through `points` (2D)."""
    P = np.asarray(points, dtype=np.float64)
    seg = np.linalg.norm(np.diff(P, axis=0), axis=1)
    s = np.concatenate([[0], np.cumsum(seg)])
    t = np.linspace(0, s[-1], n)
    out = np.empty((n, 2))
    for d in range(2):
        out[:, d] = np.interp(t, s, P[:, d])
    return out


def square_path(a=580e-9, n=4096):
    """Gamma - X - M - Gamma of the square lattice."""
    G, X, M = (0, 0), (np.pi / a, 0), (np.pi / a, np.pi / a)
    return kpath([G, X, M, G], n)


def honeycomb_path(a=580e-9, n=4096):
    """Gamma - K - M - Gamma of the hexagonal lattice with b1 = (a, 0), b2 = (a/2, a sqrt3/2)."""
    G, K, M = (0, 0), (4 * np.pi / (3 * a), 0), (np.pi / a, np.pi / (np.sqrt(3) * a))
    return kpath([G, K, M, G], n)


def jittered_square_cluster(nspheres, rng, pitch=400e-9, jitter=0.1):
    """nspheres positions on a square grid (row by row, side ceil(sqrt n)),
    each displaced uniformly by up to +-jitter * pitch in x and y, centred."""
    side = int(np.ceil(np.sqrt(nspheres)))
    idx = np.arange(nspheres)
    xy = np.stack([idx % side, idx // side], 1).astype(float) * pitch
    xy += rng.uniform(-jitter, jitter, size=xy.shape) * pitch
    xy -= xy.mean(axis=0)
    return np.concatenate([xy, np.zeros((nspheres, 1))], axis=1)


def serving_requests(n, seed=0, nmin=16, nmax=400, lmaxes=(2, 3, 4), finite_frac=0.7, a=580e-9):
    """Seeded request mix of the serving workload: finite clusters (N uniform
    in [nmin, nmax] spheres of r = 50 nm on a jittered 400 nm grid, lMax drawn
    from lmaxes, normal incidence) and single (omega, k) solves of the square
    and honeycomb lattices (r = 80 nm, lMax 3, a = 580 nm, k on the
    high-symmetry paths); hbar omega uniform in 1.6-2.6 eV.  Returns specs."""
    rng = np.random.default_rng(seed)
    sq = square_path(a, 64)
    hx = honeycomb_path(a, 64)
    out = []
    for _ in range(n):
        om = rng.uniform(1.6, 2.6) * EV / HBAR
        if rng.uniform() < finite_frac:
            ns = int(rng.integers(nmin, nmax + 1))
            out.append({"kind": "finite", "positions": jittered_square_cluster(ns, rng),
                        "lMax": int(rng.choice(lmaxes)), "omega": om})
        else:
            lat = "square" if rng.uniform() < 0.5 else "honeycomb"
            path = sq if lat == "square" else hx
            out.append({"kind": "lattice", "lattice": lat, "k": tuple(path[rng.integers(len(path))]), "omega": om})
    return out


def poisson_arrivals(n, rate, seed=0):
    """Arrival times (s) of a Poisson stream of n requests at `rate` per second."""
    rng = np.random.default_rng(seed + 7919)
    return np.cumsum(rng.exponential(1.0 / rate, size=n))
