"""Single-particle bases and the ``sq_op`` block layout, on the host.

Restates, in numpy, the parts of the reference that fix *where* every matrix
element of a scalar operator lives (n-parzuchowski/EOM-IMSRG_FULL, paths
relative to im-SRG/):

* orbit list, holes/particles, ``hb4``/``pb4``   basic_IMSRG.f90:217-238, 380-398
* (2J, Tz, parity) blocks and their pair lists     basic_IMSRG.f90:477-641
* ``vectorize`` / ``repackage`` packing order       basic_IMSRG.f90:3794-3918

The GPU library computes the same layout in C++ (``csrc/basis.cpp``); the
tests check that both agree with the oracle.  This module is used by the
benchmark and the tests to build synthetic operators in the flat layout:

    [E0 | fhh (A,A) | fph (P,A) | fpp (P,P) | per block q, gam 1..6 ]

with every matrix in Fortran (column-major) order and gam 1..6 =
pppp, ppph, pphh, phph, hhhh, phhh (basic_IMSRG.f90:579-584).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# sqs / jst of basic_IMSRG.f90:127-133 (first six entries)
SQUARE = (True, False, False, True, True, False)
GAM_ROWCAT = (0, 0, 0, 1, 2, 1)  # sea1-1: 0 pp, 1 ph, 2 hh
GAM_COLCAT = (0, 1, 2, 1, 2, 2)  # sea2-1


def ho_basis(emax: int, nucleus: str | None = None):
    """Harmonic-oscillator j-orbits with 2n+l <= emax.

    Order: for e = 0..emax, l = e, e-2, ..; j = l-1/2 then l+1/2; proton
    (2tz = -1) then neutron (+1).  Holes: the 0s shell per isospin for
    4He, 0s+0p for 16O (the default is 4He at emax < 4, else 16O).

    Returns dict of int32 arrays nn, ll, jj (2j), itzp (2tz), con (1 = hole).
    """
    if nucleus is None:
        nucleus = "4He" if emax < 4 else "16O"
    nn, ll, jj, tz = [], [], [], []
    for e in range(emax + 1):
        for l in range(e, -1, -2):
            n = (e - l) // 2
            for j2 in (2 * l - 1, 2 * l + 1):
                if j2 < 0:
                    continue
                for t in (-1, 1):
                    nn.append(n)
                    ll.append(l)
                    jj.append(j2)
                    tz.append(t)
    nn = np.array(nn, np.int32)
    ll = np.array(ll, np.int32)
    jj = np.array(jj, np.int32)
    tz = np.array(tz, np.int32)
    shell = 2 * nn + ll
    if nucleus == "4He":
        con = (shell == 0).astype(np.int32)
    elif nucleus == "16O":
        con = (shell <= 1).astype(np.int32)
    else:
        raise ValueError(f"unknown nucleus {nucleus!r}")
    return dict(nn=nn, ll=ll, jj=jj, itzp=tz, con=con)


@dataclass
class Block:
    J2: int
    par: int
    tz: int
    qn: list  # three (n,2) int arrays of 1-based orbit pairs: pp, ph, hh
    off: list = field(default_factory=list)  # flat offsets of gam 1..6
    shape: list = field(default_factory=list)  # (n1, n2) of gam 1..6

    @property
    def npp(self):
        return len(self.qn[0])

    @property
    def nph(self):
        return len(self.qn[1])

    @property
    def nhh(self):
        return len(self.qn[2])


class Layout:
    """Block layout of a scalar operator over a given orbit list."""

    def __init__(self, nn, ll, jj, itzp, con):
        self.nn = np.asarray(nn, np.int32)
        self.ll = np.asarray(ll, np.int32)
        self.jj = np.asarray(jj, np.int32)
        self.itzp = np.asarray(itzp, np.int32)
        self.con = np.asarray(con, np.int32)
        N = self.norb = len(self.jj)
        self.A = int(self.con.sum())
        self.P = N - self.A
        self.holes = np.array([i + 1 for i in range(N) if self.con[i] == 1], np.int32)
        self.parts = np.array([i + 1 for i in range(N) if self.con[i] == 0], np.int32)
        self.Jtotal_max = int(self.jj.max())
        self.lmax = int(self.ll.max())
        self.off_fhh = 1
        self.off_fph = 1 + self.A * self.A
        self.off_fpp = self.off_fph + self.P * self.A
        off = self.off_fpp + self.P * self.P
        neq = 1 + self.A * self.A + self.P * self.P + self.P * self.A
        self.blocks: list[Block] = []
        for J2 in range(0, 2 * self.Jtotal_max + 1, 2):
            for tz in (-1, 0, 1):
                for par in (0, 1):
                    cats = ([], [], [])
                    for i in range(N):
                        for j in range(i, N):
                            if tz != (self.itzp[i] + self.itzp[j]) // 2:
                                continue
                            if par != (self.ll[i] + self.ll[j]) % 2:
                                continue
                            if not (abs(self.jj[i] - self.jj[j]) <= J2 <= self.jj[i] + self.jj[j]):
                                continue
                            cats[self.con[i] + self.con[j]].append((i + 1, j + 1))
                    qn = [np.array(c, np.int32).reshape(-1, 2) for c in cats]
                    blk = Block(J2, par, tz, qn)
                    n = (len(qn[0]), len(qn[1]), len(qn[2]))
                    for g in range(6):
                        n1, n2 = n[GAM_ROWCAT[g]], n[GAM_COLCAT[g]]
                        blk.off.append(off)
                        blk.shape.append((n1, n2))
                        off += n1 * n2
                        neq += n1 * (n1 + 1) // 2 if SQUARE[g] else n1 * n2
                    self.blocks.append(blk)
        self.nblocks = len(self.blocks)
        self.nfull = off
        self.neq = neq

    # ------------------------------------------------------------------
    def block_dims(self):
        """(nblocks, 6) int array: J2, par, tz, npp, nph, nhh."""
        return np.array([[b.J2, b.par, b.tz, b.npp, b.nph, b.nhh] for b in self.blocks], np.int32)

    def gam(self, op, q, g):
        """View of gam(g) (1-based) of block q (1-based) as a (n1, n2) array."""
        b = self.blocks[q - 1]
        n1, n2 = b.shape[g - 1]
        o = b.off[g - 1]
        return op[o:o + n1 * n2].reshape((n1, n2), order="F")

    def fhh(self, op):
        return op[self.off_fhh:self.off_fhh + self.A * self.A].reshape((self.A, self.A), order="F")

    def fph(self, op):
        return op[self.off_fph:self.off_fph + self.P * self.A].reshape((self.P, self.A), order="F")

    def fpp(self, op):
        return op[self.off_fpp:self.off_fpp + self.P * self.P].reshape((self.P, self.P), order="F")

    def same_ljt(self, a, b):
        """True when 1-based orbits a, b share (l, j, tz)."""
        return (self.ll[a - 1] == self.ll[b - 1] and self.jj[a - 1] == self.jj[b - 1]
                and self.itzp[a - 1] == self.itzp[b - 1])

    # ------------------------------------------------------------------
    def vectorize(self, op):
        """Packed vector of basic_IMSRG.f90:3794-3854 (length neq)."""
        out = [op[:1], self.fhh(op).T.ravel(), self.fpp(op).T.ravel(), self.fph(op).T.ravel()]
        for q, b in enumerate(self.blocks, 1):
            for g in range(1, 7):
                X = self.gam(op, q, g)
                if SQUARE[g - 1]:
                    n = X.shape[0]
                    r, c = np.tril_indices(n)
                    order = np.lexsort((r, c))
                    out.append(X[r[order], c[order]])
                else:
                    out.append(X.T.ravel())
        return np.concatenate(out)

    def repackage(self, vec, herm):
        """Inverse of vectorize (basic_IMSRG.f90:3857-3918)."""
        op = np.zeros(self.nfull)
        op[0] = vec[0]
        k = 1
        for M, n1, n2 in ((self.fhh(op), self.A, self.A), (self.fpp(op), self.P, self.P),
                          (self.fph(op), self.P, self.A)):
            M[...] = vec[k:k + n1 * n2].reshape((n2, n1)).T
            k += n1 * n2
        for q, b in enumerate(self.blocks, 1):
            for g in range(1, 7):
                X = self.gam(op, q, g)
                n1, n2 = X.shape
                if SQUARE[g - 1]:
                    r, c = np.tril_indices(n1)
                    order = np.lexsort((r, c))
                    r, c = r[order], c[order]
                    m = len(r)
                    X[r, c] = vec[k:k + m]
                    X[c, r] = herm * vec[k:k + m]  # the diagonal ends as herm * v
                    k += m
                else:
                    X[...] = vec[k:k + n1 * n2].reshape((n2, n1)).T
                    k += n1 * n2
        return op
