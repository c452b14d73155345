"""Host-side checks of the dense solver's scheduling claims (numpy restatements
of the launch order, no GPU):

* the LU by groups of blocks (qg_dense.cu, lu_nopiv_tc) forms the same
  Schur-complement factors as taking the blocks one at a time, for every
  group size 1-4 and ragged last blocks;
* the one-launch substitution sweeps (sweep_fwd_kernel, sweep_bwd_kernel,
  sweep_diag_kernel) solve the system from those factors when their tiles
  run in ticket order under arbitrary interleavings of the warps; a tile only
  waits for tiles with earlier tickets (so every wait ends however many warps
  are resident), and a tile past its wait for block k sees every block on the
  near side of k final (the skipped waits are safe).
"""
import random

import numpy as np
import pytest


def _schur_lu(M, nb, group):
    """Schur-form block LU without pivoting: per block, D -> I - D^-1 in its
    slot, the rest of its column block multiplied by D^-1, and the trailing
    matrix updated; `group` blocks share one trailing update."""
    A = M.astype(np.complex128).copy()
    N = A.shape[0]
    k = 0

    def invert_and_scale(ki, kbi):
        Di = np.linalg.inv(A[ki:ki + kbi, ki:ki + kbi])
        A[:, ki:ki + kbi] = A[:, ki:ki + kbi] @ Di
        A[ki:ki + kbi, ki:ki + kbi] = np.eye(kbi) - Di

    while k < N:
        ge = min(k + group * nb, N)
        ki = k
        while ki < ge:
            kbi = min(nb, N - ki)
            ke = ki + kbi
            invert_and_scale(ki, kbi)
            if ke >= N:
                return A
            if ke == ge:  # the group's combined update, K = ge - k
                A[ge:, ge:] -= A[ge:, k:ge] @ A[k:ge, ge:]
                break
            wi = ge - ke
            P = A[ke:, ki:ke].copy()   # the operand planes are cut before the products
            A12 = A[ki:ke, ke:].copy()
            A[ke:, ke:ke + wi] -= P @ A12[:, :wi]           # the group's later block columns
            A[ke:ke + wi, ke + wi:] -= P[:wi] @ A12[:, wi:]  # its later block rows, past the group
            ki = ke
        k = ge
    return A


def _sweeps(A, nb, B, rows=4, nwarps=7, seed=0):
    """Forward and backward sweeps over tiles of `rows` rows taken by ticket,
    warps interleaved at random at every step, then the diagonal pass."""
    N = A.shape[0]
    B = B.copy()
    nblk = (N + nb - 1) // nb
    ntiles = (N + rows - 1) // rows

    def need(k):
        return (min(nb, N - k * nb) + rows - 1) // rows

    rnd = random.Random(seed)
    for forward in (True, False):
        cnt = [0] * nblk
        ticket = [0]
        owner = {}

        def warp(wid):
            known = -1 if forward else nblk
            while True:
                tk = ticket[0]
                ticket[0] += 1
                if tk >= ntiles:
                    return
                t = tk if forward else ntiles - 1 - tk
                owner[t] = tk
                row0 = t * rows
                j = row0 // nb
                acc = np.zeros((rows, B.shape[1]), complex)
                for k in (range(j) if forward else range(nblk - 1, j, -1)):
                    if (forward and k > known) or (not forward and k < known):
                        while cnt[k] < need(k):
                            # every tile of block k holds an earlier ticket
                            tiles_k = range(k * nb // rows, (k * nb + min(nb, N - k * nb) + rows - 1) // rows)
                            assert all(ntiles - 1 - tt < tk if not forward else tt < tk for tt in tiles_k)
                            yield
                        known = k
                    near = range(k) if forward else range(k + 1, nblk)
                    assert all(cnt[x] >= need(x) for x in near)
                    k0 = k * nb
                    kb = min(nb, N - k0)
                    r1 = min(row0 + rows, N)
                    acc[:r1 - row0] += A[row0:r1, k0:k0 + kb] @ B[k0:k0 + kb]
                    yield
                r1 = min(row0 + rows, N)
                B[row0:r1] -= acc[:r1 - row0]
                cnt[j] += 1

        ws = [warp(w) for w in range(nwarps)]
        while ws:
            w = rnd.choice(ws)
            try:
                next(w)
            except StopIteration:
                ws.remove(w)
    X = np.empty_like(B)
    for j0 in range(0, N, nb):
        kb = min(nb, N - j0)
        X[j0:j0 + kb] = B[j0:j0 + kb] - A[j0:j0 + kb, j0:j0 + kb] @ B[j0:j0 + kb]
    return X


def _system(N, seed):
    rng = np.random.default_rng(seed)
    M = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N)) + 3 * np.sqrt(N) * np.eye(N)
    return M, rng


@pytest.mark.parametrize("N,nb", [(100, 16), (128, 32), (96, 32), (200, 64), (36, 64), (68, 32), (300, 16)])
def test_grouped_lu_equals_single_steps(N, nb):
    M, _ = _system(N, N + nb)
    ref = _schur_lu(M, nb, 1)
    for g in (2, 3, 4):
        assert np.max(np.abs(_schur_lu(M, nb, g) - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("N,nb,nrhs", [(100, 64, 1), (260, 128, 3), (196, 64, 8), (36, 64, 2), (4, 128, 1),
                                       (132, 32, 2)])
def test_ticket_sweeps_solve(N, nb, nrhs):
    M, rng = _system(N, 7 * N + nrhs)
    b = rng.standard_normal((N, nrhs)) + 1j * rng.standard_normal((N, nrhs))
    A = _schur_lu(M, nb, 2)
    ref = np.linalg.solve(M, b)
    for seed in range(3):
        x = _sweeps(A, nb, b, seed=seed)
        assert np.max(np.abs(x - ref)) <= 1e-10 * np.max(np.abs(ref))
