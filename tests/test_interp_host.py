"""Tabulated data on the host (no GPU): the oracle's interpolation against
scipy, and the library's interpolators and SCUFF-EM reader against the oracle.

The reference interpolates with GSL's gsl_interp_cspline (natural cubic
spline) and gsl_interp_linear (materials.c:11-30, tmatrices.c:287-350); scipy's
CubicSpline(bc_type="natural") and numpy.interp are the same published
interpolants.
"""
import ctypes as C

import numpy as np
import pytest

C0 = 299792458.0


def test_oracle_spline_vs_scipy(orc):
    from scipy.interpolate import CubicSpline
    rng = np.random.default_rng(1)
    for n in (3, 4, 17, 60):
        x = np.cumsum(rng.uniform(0.1, 1.0, n))
        y = rng.normal(size=n)
        q = np.concatenate([rng.uniform(x[0], x[-1], 200), x])
        np.testing.assert_allclose(orc.spline_eval(1, x, y, q), CubicSpline(x, y, bc_type="natural")(q),
                                   rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(orc.spline_eval(0, x, y, q), np.interp(q, x, y), rtol=1e-14, atol=1e-14)
        assert np.isnan(orc.spline_eval(1, x, y, [x[0] - 1e-9, x[-1] * 1.0001])).all()


def test_permittivity_interpolator_vs_oracle(orc, tmp_path):
    from qpms_gb300.materials import MaterialInterpolator
    rng = np.random.default_rng(2)
    wl = np.linspace(350e-9, 1000e-9, 40) + rng.uniform(-3e-9, 3e-9, 40)
    n = 0.2 + 0.1 * rng.random(40)
    k = 2 + 3 * rng.random(40)
    for kind, ik in (("cspline", 1), ("linear", 0)):
        mi = MaterialInterpolator.from_arrays(wl, n, k, kind=kind)
        assert mi.freq_interval[0] == pytest.approx(2 * np.pi * C0 / wl[-1], rel=1e-15)
        assert mi.freq_interval[1] == pytest.approx(2 * np.pi * C0 / wl[0], rel=1e-15)
        om = np.linspace(mi.omegamin, mi.omegamax, 57)[1:-1]
        lam = 2 * np.pi * C0 / om
        ref = (orc.spline_eval(ik, wl, n, lam) + 1j * orc.spline_eval(ik, wl, k, lam)) ** 2
        got = np.array([mi(w) for w in om])
        np.testing.assert_allclose(got, ref, rtol=1e-12)
        with pytest.raises(ValueError):
            mi(mi.omegamax * 1.01)
    # refractiveindex.info file: '#' lines skipped, data after "data: |" until the first non-triple
    path = tmp_path / "metal.yml"
    with open(path, "w") as f:
        f.write("# comment\nREFERENCES: x\nDATA:\n  - type: tabulated nk\n    data: |\n")
        for a, b, c in zip(wl * 1e6, n, k):
            f.write("        %.17g %.17g %.17g\n" % (a, b, c))
        f.write("SPECS:\n    thickness: 1\n")
    my = MaterialInterpolator(str(path))
    fa = MaterialInterpolator.from_arrays(wl * 1e6 * 1e-6, n, k)
    for w in np.linspace(my.omegamin, my.omegamax, 11)[1:-1]:
        assert abs(my(w) - fa(w)) <= 1e-14 * abs(fa(w))
    with pytest.raises(IOError):
        MaterialInterpolator(str(tmp_path / "missing.yml"))


def _T_arrays(rng, nf, n):
    T = rng.normal(size=(nf, n, n)) + 1j * rng.normal(size=(nf, n, n))
    T[:, 0, 1] = 0                      # no data at all: the element is left untouched
    T[:, 1, 2] = T[:, 1, 2].real        # real part only
    T[:, 2, 3] = 1j * T[:, 2, 3].imag   # imaginary part only
    return T


def test_tmatrix_interpolator_vs_oracle(orc):
    from qpms_gb300.tmatrices import TMatrixInterpolator
    rng = np.random.default_rng(3)
    lMax, nf = 2, 12
    n = 2 * lMax * (lMax + 2)
    fr = np.cumsum(rng.uniform(0.5, 1.5, nf)) * 1e14
    T = _T_arrays(rng, nf, n)
    for kind, ik in (("cspline", 1), ("linear", 0)):
        ti = TMatrixInterpolator.from_arrays(fr, T, lMax, kind=kind)
        for f in np.concatenate([rng.uniform(fr[0], fr[-1], 5), fr[[0, 4, -1]]]):
            got = ti(f)
            ref = np.empty((n, n), complex)
            for i in range(n):
                for j in range(n):
                    ref[i, j] = orc.spline_eval(ik, fr, T[:, i, j].real, [f])[0] + \
                        1j * orc.spline_eval(ik, fr, T[:, i, j].imag, [f])[0]
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-13)
        # eval_fill semantics (tmatrices.c:339-349): untabulated elements keep
        # their value, imaginary-only elements are incremented
        L = ti._L
        t = L.qpms_tmatrix_init(L.qpms_tmatrix_interpolator_bspec(ti.ptr))
        m = np.ctypeslib.as_array(C.cast(t.contents.m, C.POINTER(C.c_double)), (n * n * 2,)).view(np.complex128)
        m[:] = 7 + 5j
        assert L.qpms_tmatrix_interpolator_eval_fill(t, ti.ptr, float(fr[3])) == 0
        M = m.reshape(n, n).copy()
        L.qpms_tmatrix_free(C.cast(t, C.c_void_p))
        assert M[0, 1] == 7 + 5j
        assert M[1, 2] == pytest.approx(T[3, 1, 2].real, rel=1e-13) and M[1, 2].imag == 0
        assert M[2, 3] == pytest.approx(7 + 5j + 1j * T[3, 2, 3].imag, rel=1e-13)
        np.testing.assert_allclose(M[4:, 4:], T[3, 4:, 4:], rtol=1e-13)
        with pytest.raises(ValueError):
            ti(fr[-1] * 1.01)


def test_scuff_tmatrix_reader(tmp_path):
    """SCUFF-EM lines 'freq_SU a la ma pa b lb mb pb ReT ImT' (pa/pb = 0 magnetic,
    1 electric) into [dest][src] of the default basis, converted from SCUFF's
    convention (magnetic waves times i, electric times -1): T = T_SU g(dest)/g(src)."""
    from qpms_gb300.tmatrices import load_scuff_tmatrix
    lMax = 1
    rng = np.random.default_rng(4)
    # default basis order: electric (l=1, m=-1,0,1), then magnetic
    basis = [(1, 1, m) for m in (-1, 0, 1)] + [(0, 1, m) for m in (-1, 0, 1)]
    g = {1: -1.0, 0: 1j}
    freqs_su = [1.5, 2.25]
    Tsu = rng.normal(size=(2, 6, 6)) + 1j * rng.normal(size=(2, 6, 6))
    path = tmp_path / "t.TMatrix"
    with open(path, "w") as f:
        f.write("# SCUFF T-matrix\n")
        for w in range(2):
            for d, (pb, lb, mb) in enumerate(basis):
                for s_, (pa, la, ma) in enumerate(basis):
                    f.write("%.17g %d %d %d %d %d %d %d %d %.17g %.17g\n" % (
                        freqs_su[w], s_ + 1, la, ma, pa, d + 1, lb, mb, pb, Tsu[w, d, s_].real, Tsu[w, d, s_].imag))
            # an element outside the basis is skipped
            f.write("%.17g 9 2 0 1 9 2 0 1 1.0 1.0\n" % freqs_su[w])
    freqs, T, has_nan = load_scuff_tmatrix(str(path), lMax)
    assert not has_nan
    np.testing.assert_allclose(freqs, np.array(freqs_su) * 3e14, rtol=1e-15)
    for d, (pb, _, _) in enumerate(basis):
        for s_, (pa, _, _) in enumerate(basis):
            np.testing.assert_allclose(T[:, d, s_], Tsu[:, d, s_] * g[pb] / g[pa], rtol=1e-14)
    # a missing element is reported (NaN in the data)
    lines = open(path).read().splitlines()
    with open(path, "w") as f:
        f.write("\n".join(lines[:-3]) + "\n")
    _, T2, has_nan = load_scuff_tmatrix(str(path), lMax)
    assert has_nan and np.isnan(T2[-1]).any()
    with pytest.raises(IOError):
        load_scuff_tmatrix(str(tmp_path / "none.TMatrix"), lMax)
