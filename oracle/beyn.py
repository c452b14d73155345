"""Oracle (test infrastructure only): numpy restatement of the reference's Beyn
contour-integral eigensolver, qpms/beyn.c, and of its two scattering-system
callers, qpms/scatsystem.c:2280-2372.

Only tests and the CPU leg of the benchmark use this module, to check results;
the library never calls it.

The linear algebra is the reference's own LAPACK drivers through numpy:
numpy.linalg.solve is zgesv (= zgetrf + zgetrs, beyn.c:552-564),
numpy.linalg.svd(full_matrices=False) is zgesdd (beyn.c:321-333),
numpy.linalg.eig is zgeev (beyn.c:404-416).

The probe matrix V-hat is an argument: the reference seeds random() with
time(NULL) (beyn.c:292, 306-316), so its V-hat is not reproducible; callers
pass the same V-hat to the oracle and to the library under test, or compare
eigenvalues only (they do not depend on V-hat once the rank is captured).
"""
import numpy as np


def contour_ellipse(centre, rRe, rIm, n):
    """Nodes z_i and weights dz_i of the elliptic trapezoid contour (beyn.c:69-86)."""
    z = np.empty(n, dtype=np.complex128)
    dz = np.empty(n, dtype=np.complex128)
    for i in range(n):
        t = i * 2 * np.pi / n
        st, ct = np.sin(t), np.cos(t)
        z[i] = centre + ct * rRe + 1j * st * rIm
        dz[i] = (-rRe * st + 1j * rIm * ct) * (2 * np.pi / n)
    return z, dz


def inside_ellipse(z, centre, rRe, rIm):
    """beyn_contour_ellipse_inside_test (beyn.c:61-67)."""
    zn = np.asarray(z) - centre
    return (zn.real / rRe) ** 2 + (zn.imag / rIm) ** 2 < 1


def _process_matrices(A0, A1, z0, rank_tol, rank_sel_min, res_tol, M_function, want_vectors):
    """Beyn steps 3-6 (beyn_process_matrices, beyn.c:302-468)."""
    m, l = A0.shape
    U, sigma, Vh = np.linalg.svd(A0, full_matrices=False)       # zgesdd, jobz 'O'
    K = sum(1 for k in range(l) if k < rank_sel_min or sigma[k] > rank_tol)
    eigval = np.zeros(l, dtype=np.complex128)
    eigvec = np.zeros((l, m), dtype=np.complex128) if want_vectors else None
    residuals = np.zeros(l)
    if K == 0:
        return 0, eigval, eigvec, residuals, sigma
    V0 = U[:, :K]
    W0T = Vh[:K, :]
    TM2 = V0.conj().T @ A1                                      # beyn.c:377-378
    B = TM2 @ W0T.conj().T                                      # beyn.c:382-383
    B = B * (1.0 / sigma[:K])[None, :]                          # B <- B Sigma^-1 (beyn.c:389-395)
    lam, S = np.linalg.eig(B)                                   # zgeev, right vectors
    V0S = V0 @ S
    kept = 0
    for k in range(K):
        z = z0 + lam[k]
        vk = V0S[:, k]
        residual = 0.0
        if res_tol > 0:
            residual = np.linalg.norm(M_function(z) @ vk)
            if residual > res_tol:
                continue
        eigval[kept] = z
        if want_vectors:
            eigvec[kept] = vk
            residuals[kept] = residual
        kept += 1
    return kept, eigval, eigvec, residuals, sigma


def beyn_solve(M_function, m, l, contour, Vhat, rank_tol=1e-4, rank_sel_min=1, res_tol=0.0):
    """beyn_solve_gsl (beyn.c:471-584) with an explicit probe matrix Vhat (m x l).

    contour = (z, dz, centre), e.g. from ellipse().
    M_function(z) returns the m x m complex128 matrix M(z).  Returns a dict with
    the fields of beyn_result_t (beyn.h:82-94): neig, eigval, eigval_err,
    residuals, eigvec (rows), ranktest_SV.
    """
    z, dz, z0 = contour
    Vhat = np.asarray(Vhat, dtype=np.complex128)
    assert Vhat.shape == (m, l) and l <= m
    if rank_tol < 0:  # the library's relative rank test (the reference's is absolute)
        rank_tol = -rank_tol * rank_scale(dz, Vhat)
    A0, A1, A0c, A1c = quadrature(M_function, contour, Vhat, 0, len(z))
    _, err, _, _, _ = _process_matrices(A0c, A1c, z0, rank_tol, rank_sel_min, res_tol, M_function, False)
    K, ev, vec, res, sigma = _process_matrices(A0, A1, z0, rank_tol, rank_sel_min, res_tol, M_function, True)
    return {"neig": K, "eigval": ev[:K], "eigval_err": (err - ev)[:K], "residuals": res[:K],
            "eigvec": vec[:K], "ranktest_SV": sigma, "A0": A0, "A1": A1}


def quadrature(M_function, contour, Vhat, node_begin, node_end):
    """Beyn step 2 over nodes [node_begin, node_end) (beyn.c:524-581): the
    sums A0, A1 and the coarse A0c, A1c (even global node indices, twice)."""
    z, dz, z0 = contour
    A0 = np.zeros(Vhat.shape, dtype=np.complex128)
    A1 = np.zeros_like(A0)
    A0c = np.zeros_like(A0)
    A1c = np.zeros_like(A0)
    for i in range(node_begin, node_end):
        X = np.linalg.solve(M_function(z[i]), Vhat)             # zgetrf + zgetrs
        X *= dz[i]
        A0 += X
        if i % 2 == 0:
            A0c += X
            A0c += X
        X *= (z[i] - z0)                                        # Beyn's Remark 3.2(b) scaling
        A1 += X
        if i % 2 == 0:
            A1c += X
            A1c += X
    return A0, A1, A0c, A1c


def probe_matrix(m, l, seed):
    """The library's seeded complex-Gaussian probe matrix (m x l, row-major):
    splitmix64 draws u in (0, 1], Box-Muller sqrt(-2 log u1) cos(2 pi u2), the
    real then the imaginary part of each entry.  The reference seeds random()
    with the time instead (beyn.c:306-316), so its probe is not reproducible;
    this restatement lets fixtures be regenerated from the seed alone."""
    n = 4 * m * l
    with np.errstate(over="ignore"):
        st = np.uint64(seed) + np.arange(1, n + 1, dtype=np.uint64) * np.uint64(0x9e3779b97f4a7c15)
        z = st
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xbf58476d1ce4e5b9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94d049bb133111eb)
        z = z ^ (z >> np.uint64(31))
    u = ((z >> np.uint64(11)) + np.uint64(1)).astype(np.float64) * (1.0 / 9007199254740992.0)
    u = u.reshape(-1, 4)
    re = np.sqrt(-2 * np.log(u[:, 0])) * np.cos(2 * np.pi * u[:, 1])
    im = np.sqrt(-2 * np.log(u[:, 2])) * np.cos(2 * np.pi * u[:, 3])
    return (re + 1j * im).reshape(m, l)


def rank_scale(dz, Vhat):
    """Scale of the quadrature sums against which the library's relative rank
    tolerance (rank_tol < 0) is taken: sum_i |dz_i| times the RMS column norm
    ||Vhat||_F / sqrt(l), the size of A0 without cancellation when M^-1 is of
    order one along the contour.  With no eigenvalue inside, A0 is
    cancellation noise of about 1e-16 of it; each enclosed eigenvalue adds a
    singular value of the order of its residue."""
    Vhat = np.asarray(Vhat)
    return float(np.sum(np.abs(dz)) * np.linalg.norm(Vhat) / np.sqrt(Vhat.shape[1]))


def ellipse(centre, rRe, rIm, n):
    """Contour tuple (z, dz, centre) as beyn_contour_ellipse stores it."""
    z, dz = contour_ellipse(centre, rRe, rIm, n)
    return (z, dz, complex(centre))


def _orientation(orient, rRe, rIm):
    """(rotation, l, h) of a half-ellipse orientation (beyn.c:134-152)."""
    return {3: (-1j, rIm, rRe), 1: (1j, rIm, rRe), 0: (1.0, rRe, rIm), 2: (-1.0, rRe, rIm)}[orient]


def halfellipse(centre, rRe, rIm, n, orient):
    """Contour tuple of beyn_contour_halfellipse (beyn.c:117-167): narc = n - n//2
    midpoint nodes on the half-ellipse, n//2 equal steps along its straight side."""
    fk, l, h = _orientation(orient, rRe, rIm)
    nline = n // 2
    narc = n - nline
    t = (np.arange(narc) + 0.5) * np.pi / narc
    za = centre + fk * (np.cos(t) * l + 1j * np.sin(t) * h)
    dza = fk * (-l * np.sin(t) + 1j * h * np.cos(t)) * (np.pi / narc)
    s = 0.5 * (1 - nline) + np.arange(nline)
    zl = centre + fk * s * 2 * l / nline
    dzl = np.full(nline, fk * 2 * l / nline, dtype=complex)
    return (np.concatenate([za, zl]), np.concatenate([dza, dzl]), complex(centre))


def kidney(centre, rRe, rIm, rounding, n, orient):
    """Contour tuple of beyn_contour_kidney (beyn.c:169-226): the half-ellipse
    with its two corners rounded by circles of radius rounding * h, nodes at
    equal steps of the arc-length-like parameter."""
    fk, l, h = _orientation(orient, rRe, rIm)
    y = rounding * h
    x = np.sqrt((h - y) ** 2 - y ** 2)
    al = np.arcsin(y / (h - y))
    ar = l / h
    tmax = 2 * (x + (np.pi / 2 + al) * y + (np.pi / 2 - al) * h)
    dt = tmax / n
    b1 = x
    b2 = b1 + (np.pi / 2 + al) * y
    b3 = b2 + (np.pi - 2 * al) * h
    b4 = b3 + (np.pi / 2 + al) * y
    z, dz = np.empty(n, complex), np.empty(n, complex)
    for i in range(n):
        t = i * dt
        if t <= b1:
            z[i], dz[i] = centre + t * ar * fk, dt * ar * fk
            continue
        if t < b2:
            ph, cx, cy, r = (t - b1) / y - np.pi / 2, x, y, y
        elif t < b3:
            ph, cx, cy, r = (t - b2) / h + al, 0.0, 0.0, h
        elif t < b4:
            ph, cx, cy, r = (t - b3) / y + np.pi - al, -x, y, y
        else:
            z[i], dz[i] = centre + (t - b4 - x) * ar * fk, dt * ar * fk
            continue
        z[i] = centre + (ar * (cx + r * np.cos(ph)) + 1j * (cy + r * np.sin(ph))) * fk
        dz[i] = dt * (-ar * np.sin(ph) + 1j * np.cos(ph)) * fk
    return (z, dz, complex(centre))


def finite_sphere_M(orc, positions, radius, eps_inside, eps_medium, lMax):
    """M(omega) = I - T S of a finite cluster of identical spheres, as the
    reference's qpms_scatsys_finite_eval_Beyn_ImTS builds it
    (scatsystem.c:2280-2299 with QPMS_NO_IRREP)."""
    C0 = 299792458.0
    calc = orc.TransCalculator(lMax)
    pos = np.ascontiguousarray(positions, dtype=np.float64)

    def M(omega):
        Td = orc.tmatrix_sphere_diag(lMax, radius, omega, eps_inside, eps_medium)
        T = np.broadcast_to(np.diag(Td), (pos.shape[0],) + (Td.size, Td.size))
        k = np.sqrt(complex(eps_medium)) * omega / C0
        return orc.finite_modeproblem(calc, pos, np.ascontiguousarray(T), k)
    M.calc = calc
    return M


def finite_find_eigenmodes(orc, positions, radius, eps_inside, eps_medium, lMax, omega_centre, omega_rr,
                           omega_ri, contour_points, Vhat, rank_tol=1e-4, rank_sel_min=1, res_tol=0.0):
    """qpms_scatsys_finite_find_eigenmodes (scatsystem.c:2301-2324), full
    (no irrep) system, with an explicit probe matrix of l columns."""
    Mf = finite_sphere_M(orc, positions, radius, eps_inside, eps_medium, lMax)
    m = Vhat.shape[0]
    return beyn_solve(Mf, m, Vhat.shape[1], ellipse(omega_centre, omega_rr, omega_ri, contour_points), Vhat,
                      rank_tol, rank_sel_min, res_tol)


def periodic_sphere_M(orc, positions, radius, eps_inside, eps_medium, lMax, b1, b2, kvec):
    """M(omega) = I - T W(omega, k) of a 2D lattice of identical spheres with
    the adjusted Ewald parameter, as qpms_scatsys_periodic_eval_Beyn_ImTW
    builds it (scatsystem.c:2332-2349)."""
    C0 = 299792458.0
    calc = orc.TransCalculator(lMax)
    pos = np.ascontiguousarray(positions, dtype=np.float64)
    area = abs(b1[0] * b2[1] - b1[1] * b2[0])

    def M(omega):
        Td = orc.tmatrix_sphere_diag(lMax, radius, omega, eps_inside, eps_medium)
        T = np.ascontiguousarray(np.broadcast_to(np.diag(Td), (pos.shape[0],) + (Td.size, Td.size)))
        k = np.sqrt(complex(eps_medium)) * omega / C0
        eta = orc.adjusted_eta(area, k, kvec, lMax)
        return orc.periodic_modeproblem(calc, pos, T, k, b1, b2, kvec, eta)
    M.calc = calc
    return M
