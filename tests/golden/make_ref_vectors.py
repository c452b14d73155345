"""Generates ref_vectors.npz: translation coefficients and lattice-summed
translation coefficients computed by the reference's own translations.c /
ewald.c / ewaldsf.c (compiled into oracle/_ref by oracle/build_oracle.py),
the golden vectors the GPU tests compare the library with on machines where
the reference is absent.

  * A/B arrays, lMax 3 and 6, J = 1 and 3, seeded complex kr, directions;
  * Ewald A/B arrays, lMax 3, the reference's eta-invariance parameter sets
    (unit square lattice, eta 1.6, maxR 20/40, maxK 160) and the 580 nm square
    and honeycomb lattices of the dispersion scan (adjusted eta, the
    reference's cut-offs).

Run where the reference tree is: python tests/golden/make_ref_vectors.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import build_oracle, orc, refpin  # noqa: E402
from qpms_gb300.workloads import honeycomb_lattice, square_lattice  # noqa: E402

NORM = 65536 | 8  # QPMS_NORMALISATION_DEFAULT


def main():
    build_oracle.build_oracle()
    if not build_oracle.build_ref_lib():
        raise SystemExit("reference tree not found")
    rng = np.random.default_rng(20261204)
    out = {}
    for lMax, nkd in ((3, 12), (6, 4)):
        rc = refpin.RefCalculator(lMax, NORM)
        kr = rng.uniform(0.4, 60, nkd) + 1j * rng.uniform(0, 0.05, nkd) * rng.uniform(0.4, 60, nkd)
        th = np.arccos(rng.uniform(-1, 1, nkd))
        ph = rng.uniform(0, 2 * np.pi, nkd)
        for J in (1, 3):
            A = np.zeros((nkd, rc.nelem, rc.nelem), np.complex128)
            B = np.zeros_like(A)
            for i in range(nkd):
                A[i], B[i] = rc.get_AB_arrays(kr[i], th[i], ph[i], J)
            out["AB_l%d_J%d_A" % (lMax, J)] = A
            out["AB_l%d_J%d_B" % (lMax, J)] = B
        out["AB_l%d_kd" % lMax] = np.stack([kr, th + 0j, ph + 0j], 1)
    # lattice sums: rows (eta, k, b1x, b1y, b2x, b2y, beta_x, beta_y, sx, sy, sz, maxR, maxK)
    cases = []
    for k, beta, shift, maxR in [(2.3, (2.7, 1), (0.5, 0.1325), 20), (2.3, (2.7, 1), (0.0, 0.0), 20),
                                 (2.3 + 0.1j, (2.7, 1), (0.5, 0.1325), 20), (2.3 - 0.1j, (2.7, 1), (0.0, 0.0), 20),
                                 (2.3, (0.0, 0.0), (0.5, 0.1325), 40)]:
        cases.append((1.6, k, (1, 0), (0, 1), beta, (shift[0], shift[1], 0.0), maxR, 160))
    for lat in (square_lattice(), honeycomb_lattice()):
        b1, b2, pos = lat
        area = abs(b1[0] * b2[1] - b1[1] * b2[0])
        maxR = 64 * np.sqrt(area)
        maxK = 2048 * 2 * np.pi / maxR
        for k, beta in ((1.6e7, (2e6, 1e6)), (1.9e7 + 2e4j, (5e5, 0.0))):
            eta = orc.adjusted_eta(area, k, np.array([beta[0], beta[1], 0.0]), 3)
            for d in pos:
                cases.append((eta, k, b1, b2, beta, tuple(d - pos[0]), maxR, maxK))
    rc = refpin.RefCalculator(3, NORM)
    par, EA, EB = [], [], []
    for eta, k, b1, b2, beta, sh, maxR, maxK in cases:
        A, _, B, _ = rc.get_AB_arrays_e32(eta, k, b1, b2, beta, sh, maxR, maxK)
        k = complex(k)
        par.append([eta, k.real, k.imag, b1[0], b1[1], b2[0], b2[1], beta[0], beta[1], sh[0], sh[1], sh[2], maxR,
                    maxK])
        EA.append(A)
        EB.append(B)
    out["e32_params"] = np.array(par)
    out["e32_A"] = np.array(EA)
    out["e32_B"] = np.array(EB)
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "ref_vectors.npz"), **out)
    print({k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
