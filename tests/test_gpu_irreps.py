"""Irrep decomposition (symmetry-adapted basis) of finite systems on the GPU,
against the oracle's full matrices.

The packed basis is the library's own (the reference's orbit bases differ by a
unitary change of basis inside each irrep), so the checks are basis-free or
made in the library's basis: U is unitary, the oracle's M = I - T S and S are
block-diagonal in it (off-irrep blocks below 1e-12 of |M|), the packed mode
problem equals U M_oracle U^H (1e-10 Frobenius), and the solution assembled
from the per-irrep packed solves equals the oracle's full solve (1e-9).
"""
import numpy as np
import pytest

from qpms_gb300.workloads import EV, HBAR, C0

pytestmark = pytest.mark.gpu

EPS_I = -12 + 1.2j
EPS_E = 2.25


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import qpms_gb300
    return qpms_gb300


def rect_array(nx, ny, px, py):
    xs = (np.arange(nx) - (nx - 1) / 2) * px
    ys = (np.arange(ny) - (ny - 1) / 2) * py
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), np.zeros(nx * ny)], axis=1)


REF_NAMES = {"D2h": ["A1'", "A1''", "A2'", "A2''", "B1'", "B1''", "B2'", "B2''"],
             "C2v": ["A1", "A2", "B1", "B2"], "C2": ["A", "B"], "trivial": ["A"],
             "C4": ["1E", "2E", "A", "B"], "C4v": ["A1", "A2", "B1", "B2", "E"],
             "D4h": ["A1'", "A1''", "A2'", "A2''", "B1'", "B1''", "B2'", "B2''", "E'", "E''"],
             "D3h": ["A1'", "A1''", "A2'", "A2''", "E'", "E''"], "trivial_g": ["A"],
             "x_and_z_flip": ["P'", "P''", "R'", "R''"], "y_and_z_flip": ["P'", "P''", "R'", "R''"]}


def hexagon_cluster(r):
    """A centre particle and a hexagonal ring (D3h, D6h symmetric)."""
    ang = np.arange(6) * np.pi / 3
    ring = np.stack([r * np.cos(ang), r * np.sin(ang), np.zeros(6)], axis=1)
    return np.vstack([np.zeros((1, 3)), ring])


@pytest.mark.parametrize("group,nx,ny,lMax", [("D2h", 4, 3, 2), ("D2h", 3, 3, 3), ("C2v", 3, 2, 2),
                                              ("C2", 4, 4, 1), ("trivial", 2, 2, 2),
                                              ("D4h", 4, 4, 2), ("D4h", 3, 3, 3), ("C4v", 3, 3, 2),
                                              ("C4", 4, 4, 2), ("D3h", 0, 0, 3), ("D3h", 0, 0, 2),
                                              ("x_and_z_flip", 3, 2, 2), ("y_and_z_flip", 2, 3, 2),
                                              ("trivial_g", 2, 1, 2)])
def test_bases_and_block_diagonal_oracle_matrix(gpu, orc, group, nx, ny, lMax):
    """Square groups (C4, C4v, D4h: rotations by pi/2, two-dimensional E
    irreps with d x multiplicity packed vectors, complex bases) on square
    arrays, D3h (rotation by 2 pi/3) on a hexagonal cluster; the mirror groups
    on rectangular ones."""
    py = 400e-9 if group in ("C4", "C4v", "D4h") else 330e-9
    pos = hexagon_cluster(420e-9) if group == "D3h" else rect_array(nx, ny, 400e-9, py)
    ss = gpu.ScatteringSystem(pos, 50e-9, EPS_I, EPS_E, lMax, sym=group)
    assert ss.irrep_names == REF_NAMES[group]
    assert sum(ss.saecv_sizes) == ss.fecv_size
    U = np.vstack([ss.irrep_transform_matrix(i) for i in range(ss.nirreps)])
    assert np.abs(U @ U.conj().T - np.eye(ss.fecv_size)).max() <= 1e-14
    om = 2.05 * EV / HBAR
    k = np.sqrt(EPS_E) * om / C0
    calc = orc.TransCalculator(lMax)
    Td = orc.tmatrix_sphere_diag(lMax, 50e-9, om, EPS_I, EPS_E)
    T = np.ascontiguousarray(np.broadcast_to(np.diag(Td), (pos.shape[0], Td.size, Td.size)))
    M = orc.finite_modeproblem(calc, pos, T, k)
    B = U @ M @ U.conj().T
    off = 0
    nrm = np.linalg.norm(M)
    ssw = ss(om)
    for i, n in enumerate(ss.saecv_sizes):
        blk = B[off:off + n, off:off + n]
        rest = np.delete(B[off:off + n], np.s_[off:off + n], axis=1)
        assert np.abs(rest).max(initial=0) <= 1e-12 * nrm, (group, i)
        P = ssw.modeproblem_matrix_packed(i)
        assert np.linalg.norm(P - blk) <= 1e-10 * np.linalg.norm(blk)
        np.testing.assert_allclose(ss.pack_matrix(M, i), blk, rtol=0, atol=1e-12 * nrm)
        off += n
    # packed translation matrix
    S = orc.finite_translation_matrix(calc, pos, k, 3)
    U0 = ss.irrep_transform_matrix(0)
    Sp = ss.translation_matrix_packed(k, 0)
    ref = U0 @ S @ U0.conj().T
    assert np.linalg.norm(Sp - ref) <= 1e-10 * np.linalg.norm(ref)


@pytest.mark.parametrize("group", ["D2h", "D4h", "C4", "D3h"])
def test_vectors_and_packed_solves_vs_oracle(gpu, orc, group):
    lMax = 2
    pos = hexagon_cluster(420e-9) if group == "D3h" else rect_array(4, 4, 400e-9, 400e-9)
    ss = gpu.ScatteringSystem(pos, 50e-9, EPS_I, EPS_E, lMax, sym=group)
    rng = np.random.default_rng(3)
    v = rng.normal(size=ss.fecv_size) + 1j * rng.normal(size=ss.fecv_size)
    back = sum(ss.unpack_vector(ss.pack_vector(v, i), i) for i in range(ss.nirreps))
    assert np.abs(back - v).max() <= 1e-14 * np.abs(v).max()
    om = 2.25 * EV / HBAR
    k = np.sqrt(EPS_E) * om / C0
    calc = orc.TransCalculator(lMax)
    f_ref, a_inc, sig = orc.finite_sphere_scatter(calc, pos, 50e-9, EPS_I, EPS_E, om)
    ssw = ss(om)
    rhs = ssw.apply_Tmatrices_full(a_inc)
    f = np.zeros(ss.fecv_size, complex)
    for i in range(ss.nirreps):
        sol = ssw.scatter_solver(iri=i)
        f += ss.unpack_vector(sol(ss.pack_vector(rhs, i)), i)
    assert np.linalg.norm(f - f_ref) <= 1e-9 * np.linalg.norm(f_ref)
    # packed M = I + U A U^H blocks: eigenvalues of the blocks are those of M
    M = ssw.modeproblem_matrix_full()
    ev_full = np.sort_complex(np.linalg.eigvals(M))
    ev_blk = np.sort_complex(np.concatenate([np.linalg.eigvals(ssw.modeproblem_matrix_packed(i))
                                            for i in range(ss.nirreps)]))
    assert np.abs(ev_full - ev_blk).max() <= 1e-9 * np.abs(ev_full).max()


def test_errors(gpu):
    from qpms_gb300 import QpmsGpuError
    from qpms_gb300.workloads import jittered_square_cluster, square_lattice
    pos = jittered_square_cluster(9, np.random.default_rng(1))
    with pytest.raises(QpmsGpuError):            # not symmetric
        gpu.ScatteringSystem(pos, 50e-9, EPS_I, EPS_E, 2, sym="D2h")
    with pytest.raises(QpmsGpuError):            # unknown group
        gpu.ScatteringSystem(rect_array(2, 2, 4e-7, 4e-7), 50e-9, EPS_I, EPS_E, 2, sym="D6h")
    with pytest.raises(QpmsGpuError):            # a rectangle has no rotation by pi/2
        gpu.ScatteringSystem(rect_array(2, 2, 4e-7, 3e-7), 50e-9, EPS_I, EPS_E, 2, sym="D4h")
    b1, b2, p1 = square_lattice()
    with pytest.raises(QpmsGpuError):            # lattices: full matrices only
        gpu.ScatteringSystem(p1, 80e-9, EPS_I, EPS_E, 2, lattice=(b1, b2), sym="D2h")
    # kinds must map onto their own kind
    pos = rect_array(2, 1, 4e-7, 4e-7)
    with pytest.raises(QpmsGpuError):
        gpu.ScatteringSystem(pos, [50e-9, 60e-9], [EPS_I, EPS_I], EPS_E, 2, kinds=[0, 1], sym="C2v")


@pytest.mark.parametrize("group,nx,ny,py,lMax,N", [("D2h", 6, 4, 350e-9, 3, 720), ("D4h", 6, 6, 400e-9, 2, 576)])
def test_symmetric_large_scatter_vs_full(gpu, orc, group, nx, ny, py, lMax, N):
    """Above 512 unknowns with D2h (8 systems of about N/8) or D4h (8 of
    about N/16 and two two-dimensional irreps of about N/8): each frequency is
    solved per irrep and unpacked; the same as the system without symmetry and
    as the oracle's full solve."""
    pos = rect_array(nx, ny, 400e-9, py)
    om = np.array([1.95, 2.35]) * EV / HBAR
    sym = gpu.ScatteringSystem(pos, 50e-9, EPS_I, EPS_E, lMax, sym=group)
    full = gpu.ScatteringSystem(pos, 50e-9, EPS_I, EPS_E, lMax)
    assert sym.fecv_size == N
    a = sym.planewave_scatter_batch(om, mode=1, want_f=True, want_scat=True)
    b = full.planewave_scatter_batch(om, mode=1, want_f=True, want_scat=True)
    calc = orc.TransCalculator(lMax)
    for i, w in enumerate(om):
        assert a["residual"][i] <= 1e-12
        assert np.linalg.norm(a["f"][i] - b["f"][i]) <= 1e-9 * np.linalg.norm(b["f"][i])
        f, _, sig = orc.finite_sphere_scatter(calc, pos, 50e-9, EPS_I, EPS_E, w)
        assert np.linalg.norm(a["f"][i] - f) <= 1e-9 * np.linalg.norm(f)
        assert abs(a["sigma_ext"][i] - sig) <= 1e-9 * abs(sig)
        assert abs(a["sigma_scat"][i] - b["sigma_scat"][i]) <= 1e-9 * abs(b["sigma_scat"][i])


@pytest.mark.parametrize("group", ["D2h", "D4h"])
def test_beyn_per_irrep(gpu, group):
    """Eigenmodes of a symmetric 2 x 2 cluster searched irrep by irrep: every
    mode of the full search is found in one of the irreps (packed problems of
    8 unknowns or fewer instead of 64)."""
    pos = rect_array(2, 2, 400e-9, 400e-9)
    ss = gpu.ScatteringSystem(pos, 60e-9, EPS_I, EPS_E, 2, sym=group)
    c, rr, ri = (2.52 - 0.3j) * EV / HBAR, 0.1 * EV / HBAR, 0.1 * EV / HBAR
    full0 = ss.find_modes(c, rr, ri, contour_points=64, rank_tol=1e300)
    full = ss.find_modes(c, rr, ri, contour_points=64, rank_tol=1e-10 * full0["ranktest_SV"][0])
    assert full["eigval"].size == 3
    found = []
    for i in range(ss.nirreps):
        r0 = ss.find_modes(c, rr, ri, iri=i, contour_points=64, rank_tol=1e300)
        r = ss.find_modes(c, rr, ri, iri=i, contour_points=64, rank_tol=1e-10 * r0["ranktest_SV"][0])
        assert r["eigvec"].shape[1] == ss.saecv_sizes[i]
        found.extend(r["eigval"][r["residuals"] < 1e-6 * np.abs(r["eigval"])] if r["eigval"].size else [])
    found = np.array(found)
    for e in full["eigval"]:
        assert np.min(np.abs(found - e)) <= 1e-8 * abs(e), e
