"""GPU Beyn eigensolver against the oracle (oracle/beyn.py, numpy restatement of beyn.c).

Tolerance (from the path specification): eigenfrequencies within 1e-8
relative of the oracle's.  Both sides use the same probe matrix; the oracle
solves each node with LAPACK zgesv, the library with its GPU LU (plain FP64 or
complex64 + FP64 refinement).  The library returns eigenvalues in the order
of its own Schur form, so sets are matched nearest-to-nearest.  Eigenvectors
are compared up to a complex scale, singular values of the rank test
relatively.
"""
import numpy as np
import pytest

from oracle import beyn as ob
from qpms_gb300.workloads import EV, HBAR

pytestmark = pytest.mark.gpu
EIG_RTOL = 1e-8


@pytest.fixture(scope="module")
def qb():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from qpms_gb300 import beyn
    return beyn


def _match(ref, got, rtol=EIG_RTOL):
    """every ref eigenvalue has a got eigenvalue within rtol |ref|"""
    got = np.asarray(got)
    for e in ref:
        d = np.min(np.abs(got - e)) if got.size else np.inf
        assert d <= rtol * abs(e), (e, d / abs(e))


def _parallel(a, b):
    return abs(np.vdot(a, b)) / (np.linalg.norm(a) * np.linalg.norm(b))


@pytest.mark.parametrize("mode", [0, 1])
def test_quadratic_callback(qb, mode):
    """tests/tbeyn2.c setup through the callback beyn_solve (dim 60: padded LU)."""
    rng = np.random.default_rng(1)
    T0, T1, T2 = (rng.normal(size=(60, 60)) for _ in range(3))
    Mf = lambda z: T0 + z * T1 + z * z * T2
    V = rng.normal(size=(60, 30)) + 1j * rng.normal(size=(60, 30))
    ref = ob.beyn_solve(Mf, 60, 30, ob.ellipse(0, 0.3, 0.3, 150), V, 1e-4, 1, 1e-4)
    got = qb.beyn_solve(Mf, 60, 30, 0, 0.3, 0.3, 150, 1e-4, 1, 1e-4, Vhat=V, mode=mode)
    assert got["eigval"].size == ref["neig"] >= 3
    _match(ref["eigval"], got["eigval"])
    assert np.allclose(got["ranktest_SV"][:ref["neig"]], ref["ranktest_SV"][:ref["neig"]], rtol=1e-8, atol=0)
    assert got["node_residual_max"] <= 1e-12
    for z, v in zip(got["eigval"], got["eigvec"]):
        k = np.argmin(np.abs(ref["eigval"] - z))
        assert _parallel(v, ref["eigvec"][k]) > 1 - 1e-8


def test_loaded_string_dropin(qb):
    """tests/tbeyn.c: the drop-in beyn_solve (default seed, mixed precision)
    with the reference's arguments; the oracle uses the same seeded probe matrix."""
    from test_oracle_beyn import loaded_string
    m = 400
    M, _, _, _ = loaded_string(m)
    got = qb.beyn_solve(M, m, 10, 150 + 2j, 148, 148, 50, 1e-4, 1, 1e-4)
    V = qb.probe_matrix(m, 10, qb.DEFAULT_SEED)
    ref = ob.beyn_solve(M, m, 10, ob.ellipse(150 + 2j, 148, 148, 50), V, 1e-4, 1, 1e-4)
    assert got["eigval"].size == ref["neig"]
    # eigenvalues inside the contour (outside it the quadrature does not resolve them)
    inside = ref["eigval"][ob.inside_ellipse(ref["eigval"], 150 + 2j, 148, 148)]
    assert inside.size == 5
    _match(inside, got["eigval"])
    assert (got["residuals"] <= 1e-4).all()


def _square(nx, pitch):
    xs = (np.arange(nx) - (nx - 1) / 2) * pitch
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), np.zeros(nx * nx)], 1)


def test_finite_cluster_dropin(qb, orc):
    """qpms_scatsys_finite_find_eigenmodes on a 2 x 2 cluster (l = fecv_size = 64,
    the reference's choice), rank tolerance at the singular-value gap."""
    import qpms_gb300
    pos = _square(2, 400e-9)
    ss = qpms_gb300.ScatteringSystem(pos, 60e-9, -12 + 1.2j, 2.25, 2)
    m = ss.fecv_size
    c, rr, ri = (2.52 - 0.3j) * EV / HBAR, 0.1 * EV / HBAR, 0.1 * EV / HBAR
    V = qb.probe_matrix(m, m, qb.DEFAULT_SEED)
    Mf = ob.finite_sphere_M(orc, pos, 60e-9, -12 + 1.2j, 2.25, 2)
    ref0 = ob.beyn_solve(Mf, m, m, ob.ellipse(c, rr, ri, 64), V, 1e300, 1, 0)
    tol = 1e-10 * ref0["ranktest_SV"][0]
    ref = ob.beyn_solve(Mf, m, m, ob.ellipse(c, rr, ri, 64), V, tol, 1, 0)
    got = ss.find_modes(c, rr, ri, contour_points=64, rank_tol=tol)
    assert ref["neig"] == 3 and got["eigval"].size == 3
    _match(ref["eigval"], got["eigval"])
    assert np.allclose(got["ranktest_SV"][:3], ref["ranktest_SV"][:3], rtol=1e-10, atol=0)
    # the simple mode (2.5002 - 0.2201i eV): its vector is unique up to scale
    k_ref = np.argmin(np.abs(ref["eigval"] * HBAR / EV - (2.5002 - 0.2201j)))
    k_got = np.argmin(np.abs(got["eigval"] - ref["eigval"][k_ref]))
    assert _parallel(got["eigvec"][k_got], ref["eigvec"][k_ref]) > 1 - 1e-9
    assert (np.abs(got["eigval_err"]) < 1e-6 * np.abs(got["eigval"])).all()


@pytest.mark.parametrize("mode", [0, 1])
def test_finite_cluster_6x6(qb, orc, mode):
    """6 x 6 cluster (m = 576: several LU blocks), 40 probe columns, both precisions."""
    import qpms_gb300
    pos = _square(6, 400e-9)
    ss = qpms_gb300.ScatteringSystem(pos, 60e-9, -12 + 1.2j, 2.25, 2)
    m, l = ss.fecv_size, 40
    c, rr, ri = (2.1 - 0.05j) * EV / HBAR, 0.1 * EV / HBAR, 0.06 * EV / HBAR
    rng = np.random.default_rng(0)
    V = rng.normal(size=(m, l)) + 1j * rng.normal(size=(m, l))
    Mf = ob.finite_sphere_M(orc, pos, 60e-9, -12 + 1.2j, 2.25, 2)
    ref = ob.beyn_solve(Mf, m, l, ob.ellipse(c, rr, ri, 64), V, 1e-4, 1, 0)
    got = ss.find_modes(c, rr, ri, contour_points=64, rank_tol=1e-4, l=l, Vhat=V, mode=mode)
    # the genuine modes inside the contour: M(z) singular to roundoff
    genuine = [z for z in ref["eigval"][ob.inside_ellipse(ref["eigval"], c, rr, ri)]
               if (lambda s: s[-1] / s[0])(np.linalg.svd(Mf(z), compute_uv=False)) < 1e-12]
    assert len(genuine) >= 1
    _match(genuine, got["eigval"])
    top = ref["ranktest_SV"][:4]
    assert np.allclose(got["ranktest_SV"][:4], top, rtol=1e-9 if mode == 0 else 1e-7, atol=0)


def test_periodic_gamma(qb, orc):
    """qpms_scatsys_periodic_find_eigenmodes, square lattice a = 580 nm, r = 80 nm,
    lMax 3 (30 x 30), at Gamma: one mode near 1.909 - 0.079i eV."""
    import qpms_gb300
    from qpms_gb300.workloads import square_lattice
    b1, b2, pos = square_lattice()
    ss = qpms_gb300.ScatteringSystem(pos, 80e-9, -12 + 1.2j, 2.25, 3, lattice=(b1, b2))
    m = ss.fecv_size
    c, rr, ri = (1.72 - 0.1j) * EV / HBAR, 0.2 * EV / HBAR, 0.15 * EV / HBAR
    kv = np.zeros(3)
    V = qb.probe_matrix(m, m, qb.DEFAULT_SEED)
    Mf = ob.periodic_sphere_M(orc, pos, 80e-9, -12 + 1.2j, 2.25, 3, b1, b2, kv)
    ref0 = ob.beyn_solve(Mf, m, m, ob.ellipse(c, rr, ri, 48), V, 1e300, 1, 0)
    tol = 1e-6 * ref0["ranktest_SV"][0]
    ref = ob.beyn_solve(Mf, m, m, ob.ellipse(c, rr, ri, 48), V, tol, 1, 0)
    got = ss.find_modes(c, rr, ri, blochvector=kv, contour_points=48, rank_tol=tol)
    assert ref["neig"] == 1 and got["eigval"].size == 1
    _match(ref["eigval"], got["eigval"])
    assert abs(got["eigval"][0] * HBAR / EV - (1.909063 - 0.078786j)) < 1e-5


def test_split_quadrature_matches_whole(qb):
    """The contour split in two node ranges (as sharded ranks would) and summed
    gives the eigenvalues of the whole quadrature (6 x 6 cluster, l = 40; rank
    tolerance at the singular-value gap, where the eigenvalues are well
    conditioned)."""
    import qpms_gb300
    pos = _square(6, 400e-9)
    ss = qpms_gb300.ScatteringSystem(pos, 60e-9, -12 + 1.2j, 2.25, 2)
    c, rr, ri = (2.1 - 0.05j) * EV / HBAR, 0.1 * EV / HBAR, 0.06 * EV / HBAR
    whole = qb.scatsys_quadrature(ss.s, ss.fecv_size, c, rr, ri, 64, 0, 64, 40, seed=77, mode=1)
    p1 = qb.scatsys_quadrature(ss.s, ss.fecv_size, c, rr, ri, 64, 0, 29, 40, seed=77, mode=1)
    p2 = qb.scatsys_quadrature(ss.s, ss.fecv_size, c, rr, ri, 64, 29, 64, 40, seed=77, mode=1)
    for a, b, w in zip(p1, p2, whole):
        assert np.linalg.norm(a + b - w) <= 1e-13 * np.linalg.norm(w)
    sv = qb.process(*whole, c, 1e300, 1)["ranktest_SV"]
    tol = 1e-4 * sv[0]
    r_whole = qb.process(*whole, c, tol, 1)
    r_split = qb.process(*[a + b for a, b in zip(p1, p2)], c, tol, 1)
    assert r_split["eigval"].size == r_whole["eigval"].size >= 1
    _match(r_whole["eigval"], r_split["eigval"], rtol=1e-10)


def test_graph_replay_matches_eager(qb, monkeypatch):
    """The Beyn node loop captures the dense solver's factorisation and solve
    launch sequences as CUDA graphs at the second node and replays them from
    the third: the four quadrature sums equal those of eager execution (the
    same kernels in the same order) to 1e-13, with replays counted."""
    import qpms_gb300
    L = qpms_gb300.lib()
    pos = _square(6, 400e-9)
    ss = qpms_gb300.ScatteringSystem(pos, 60e-9, -12 + 1.2j, 2.25, 2)
    c, rr, ri = (2.1 - 0.05j) * EV / HBAR, 0.1 * EV / HBAR, 0.06 * EV / HBAR
    args = (ss.s, ss.fecv_size, c, rr, ri, 16, 0, 16, 40)
    monkeypatch.setenv("QPMS_GB300_GRAPHS", "0")
    r0 = L.qpms_gpu_graph_replay_count()
    eager = qb.scatsys_quadrature(*args, seed=77, mode=1)
    assert L.qpms_gpu_graph_replay_count() == r0
    monkeypatch.delenv("QPMS_GB300_GRAPHS")
    graph = qb.scatsys_quadrature(*args, seed=77, mode=1)
    assert L.qpms_gpu_graph_replay_count() - r0 >= 14  # factorisations of nodes 3..16 at least
    for a, b in zip(eager, graph):
        assert np.linalg.norm(a - b) <= 1e-13 * np.linalg.norm(a)
