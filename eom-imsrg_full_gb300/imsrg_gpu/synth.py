"""Seeded synthetic operators in the flat layout.

Two families:

* ``random_operator`` restates ``construct_random_rank0`` of the reference's
  own test harness (n-parzuchowski/EOM-IMSRG_FULL,
  im-SRG/brute_force_testing.f90:15-120): uniform values in [-5, 5] on every
  (l, j, tz)-allowed one-body element and every two-body element, with the
  chosen Hermiticity and the Pauli rule (identical-orbit pairs vanish at odd
  J, :102-109).
* ``synth_hamiltonian`` / ``synth_omega`` build the benchmark inputs: a
  harmonic-oscillator one-body spectrum eps_a = hw (2n + l + 3/2) with
  N(0, sigma1) Hermitian off-diagonals between orbits of equal (l, j, tz), and
  N(0, sigma2) J-coupled two-body elements, Hermitian within each
  (2J, Tz, parity) block; Omega is anti-Hermitian with N(0, sigma) two-body
  elements and N(0, sigma) allowed particle-hole one-body elements.

Random numbers come from numpy's counter-based Philox generator keyed by
(seed, stream), so the same call gives the same operator on any machine.
"""
from __future__ import annotations

import numpy as np

from .layout import SQUARE, GAM_ROWCAT, GAM_COLCAT, Layout


def _rng(seed: int, stream: int = 0):
    return np.random.Generator(np.random.Philox(key=[int(seed) & (2**64 - 1), int(stream) & (2**64 - 1)]))


def _pauli_mask(pairs: np.ndarray, J2: int) -> np.ndarray:
    """1.0 for allowed pairs, 0.0 for (a, a) pairs at odd J."""
    if len(pairs) == 0:
        return np.ones(0)
    same = pairs[:, 0] == pairs[:, 1]
    bad = same & ((J2 // 2) % 2 == 1)
    return np.where(bad, 0.0, 1.0)


def _fill_two_body(lay: Layout, op, herm, draw):
    for q, b in enumerate(lay.blocks, 1):
        for g in range(1, 7):
            X = lay.gam(op, q, g)
            n1, n2 = X.shape
            if n1 * n2 == 0:
                continue
            mr = _pauli_mask(b.qn[GAM_ROWCAT[g - 1]], b.J2)
            mc = _pauli_mask(b.qn[GAM_COLCAT[g - 1]], b.J2)
            if SQUARE[g - 1]:
                R = draw((n1, n1))
                U = np.triu(R, 1)
                M = U + herm * U.T
                if herm == 1:
                    M[np.diag_indices(n1)] = np.diag(R)
                X[...] = M * mr[:, None] * mc[None, :]
            else:
                X[...] = draw((n1, n2)) * mr[:, None] * mc[None, :]


def _ljt_mask(lay: Layout, rows, cols):
    m = np.zeros((len(rows), len(cols)))
    for i, a in enumerate(rows):
        for j, c in enumerate(cols):
            if lay.same_ljt(int(a), int(c)):
                m[i, j] = 1.0
    return m


def random_operator(lay: Layout, herm: int, seed: int, stream: int = 0):
    """Uniform [-5, 5] operator as in brute_force_testing.f90:15-120."""
    rng = _rng(seed, stream)

    def draw(shape):
        return 10.0 * rng.random(shape) - 5.0

    op = np.zeros(lay.nfull)
    for M, rows, cols, square in ((lay.fhh(op), lay.holes, lay.holes, True),
                                  (lay.fph(op), lay.parts, lay.holes, False),
                                  (lay.fpp(op), lay.parts, lay.parts, True)):
        mask = _ljt_mask(lay, rows, cols)
        R = draw(M.shape)
        if square:
            U = np.triu(R, 1)
            S = U + herm * U.T
            S[np.diag_indices(len(rows))] = np.diag(R) * (herm + 1) / 2.0
            M[...] = S * mask
        else:
            M[...] = R * mask
    _fill_two_body(lay, op, herm, draw)
    return op


def synth_hamiltonian(lay: Layout, seed: int, hw: float = 20.0, sigma1: float = 0.5, sigma2: float = 1.0,
                      stream: int = 1):
    """Hermitian H: HO single-particle energies + N(0,sigma1) off-diagonals +
    N(0,sigma2) two-body elements (herm = +1)."""
    rng = _rng(seed, stream)
    op = np.zeros(lay.nfull)
    eps = hw * (2 * lay.nn + lay.ll + 1.5)
    for M, rows, cols, square in ((lay.fhh(op), lay.holes, lay.holes, True),
                                  (lay.fph(op), lay.parts, lay.holes, False),
                                  (lay.fpp(op), lay.parts, lay.parts, True)):
        mask = _ljt_mask(lay, rows, cols)
        R = rng.normal(0.0, sigma1, M.shape)
        if square:
            U = np.triu(R, 1)
            S = U + U.T
            S[np.diag_indices(len(rows))] = eps[np.asarray(rows) - 1]
            M[...] = S * mask
        else:
            M[...] = R * mask
    _fill_two_body(lay, op, 1, lambda shape: rng.normal(0.0, sigma2, shape))
    return op


def synth_omega(lay: Layout, seed: int, sigma: float = 0.05, stream: int = 2):
    """Anti-Hermitian Omega (herm = -1): N(0,sigma) two-body elements and
    N(0,sigma) on (l,j,tz)-allowed particle-hole one-body elements."""
    rng = _rng(seed, stream)
    op = np.zeros(lay.nfull)
    M = lay.fph(op)
    M[...] = rng.normal(0.0, sigma, M.shape) * _ljt_mask(lay, lay.parts, lay.holes)
    _fill_two_body(lay, op, -1, lambda shape: rng.normal(0.0, sigma, shape))
    return op
