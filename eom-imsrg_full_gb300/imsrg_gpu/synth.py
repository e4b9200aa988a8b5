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


def write_vrenorm(lay: Layout, op, path: str, seed: int | None = None) -> int:
    """Write the two-body part of a Hermitian operator as the ASCII file that
    read_interaction reads (n-parzuchowski/EOM-IMSRG_FULL,
    im-SRG/interaction_IO.f90:8-107): eight header lines, then one line
    "Tz Par 2J a b c d V" per stored element (orbits 1-based; square arrays
    upper triangles only, the reader stores both orders).  With a seed, pair
    orders and bra/ket are swapped at random with the value carrying the pair
    phases the reader undoes, so every branch of the reader is exercised.
    Returns the number of element lines."""
    rng = _rng(seed, 7) if seed is not None else None

    def ph(a, b, J2):  # the reader's phase of a reversed pair
        return -1.0 if (1 + (lay.jj[a - 1] + lay.jj[b - 1] - J2) // 2) % 2 else 1.0

    n = 0
    with open(path, "w") as f:
        f.write("# two-body matrix elements, J-coupled, normalised kets\n")
        for k in range(6):
            f.write(f"# header line {k + 2}\n")
        f.write("# Tz Par 2J a b c d V\n")
        for b in lay.blocks:
            for g in range(6):
                n1, n2 = b.shape[g]
                if n1 * n2 == 0:
                    continue
                X = op[b.off[g]:b.off[g] + n1 * n2].reshape(n2, n1).T
                rows, cols = b.qn[GAM_ROWCAT[g]], b.qn[GAM_COLCAT[g]]
                for JX in range(n2):
                    for IX in range(n1):
                        if SQUARE[g] and IX > JX:
                            continue
                        v = float(X[IX, JX])
                        if v == 0.0:
                            continue
                        a, bb = (int(x) for x in rows[IX])
                        c, d = (int(x) for x in cols[JX])
                        if rng is not None:
                            if rng.random() < 0.5 and a != bb:
                                a, bb = bb, a
                                v *= ph(a, bb, b.J2)
                            if rng.random() < 0.5 and c != d:
                                c, d = d, c
                                v *= ph(c, d, b.J2)
                            if rng.random() < 0.5:
                                a, bb, c, d = c, d, a, bb
                        f.write(f"{b.tz} {b.par} {b.J2} {a} {bb} {c} {d} {v!r}\n")
                        n += 1
    return n


def adjoint_terms(lay: Layout):
    """The derivative workload H(c) = T + sum_k c_k V_k: T is the E0 and
    one-body part of the seed-300 synthetic Hamiltonian, V_1..V_4 the two-body
    parts of the seed-301..304 ones (independent N(0, 1) MeV elements)."""
    one = lay.off_fpp + lay.P * lay.P
    T = synth_hamiltonian(lay, 300)
    T[one:] = 0.0
    V = []
    for k in range(4):
        v = synth_hamiltonian(lay, 301 + k)
        v[:one] = 0.0
        V.append(v)
    return T, V
