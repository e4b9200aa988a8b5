"""The setup steps before the flow, restated on the CPU (test infrastructure only).

* read_interaction (n-parzuchowski/EOM-IMSRG_FULL, im-SRG/interaction_IO.f90:
  8-107) with the centre-of-mass terms r1_r2 / p1_p2 and their reduced matrix
  elements (im-SRG/basic_IMSRG.f90:4310-4530);
* calculate_h0_harm_osc (basic_IMSRG.f90:2049-2147), including the
  single-precision square roots its default-REAL literals produce;
* calc_HF without a three-body force (im-SRG/HF_mod.f90:14-106) with
  write_kin_matrix (:138-166), gamma_matrix (:169-232), density_matrix
  (:346-373), e_HF (:376-405), transform_1b_to_HF (:408-491) and
  transform_2b_to_HF (:494-619, its four products as written).  The block
  eigen-decompositions use LAPACK through numpy (the reference calls dsyev).

Orbits are 1-based as in the reference; operators are numpy arrays in the
flat layout of the oracle (oracle.py).  Parity here is unpinned by the
reference (it ships no known answer for these routines); the tests check the
restatement against identities instead: HF stationarity, E_HF against normal
ordering in the HF basis, the non-interacting case, file round trips.
"""
from __future__ import annotations

import numpy as np


def _pm1(n: int) -> float:
    return -1.0 if n % 2 else 1.0


def _fdiv(a: int, b: int) -> int:
    """Fortran integer division (truncates toward zero)."""
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b > 0) else -q


class Setup:
    """Layout tables of one oracle basis for the setup routines."""

    def __init__(self, orc, nn, ll, jj, itzp, con):
        self.orc = orc
        self.nn, self.ll, self.jj = [np.asarray(x, int) for x in (nn, ll, jj)]
        self.itzp, self.con = np.asarray(itzp, int), np.asarray(con, int)
        self.N = len(self.jj)
        self.A, self.P = int(self.con.sum()), self.N - int(self.con.sum())
        # hb4 / pb4 positions (find_holes, basic_IMSRG.f90:380-398), 0-based
        self.pos = np.zeros(self.N + 1, int)
        nh = npar = 0
        for i in range(1, self.N + 1):
            if self.con[i - 1]:
                self.pos[i] = nh
                nh += 1
            else:
                self.pos[i] = npar
                npar += 1
        self.off_fhh, self.off_fph = 1, 1 + self.A * self.A
        self.off_fpp = self.off_fph + self.P * self.A
        dims = orc.block_dims()
        self.nblocks = len(dims)
        self.qn, self.goff, self.gshape, self.row = [], [], [], {}
        off = self.off_fpp + self.P * self.P
        for q in range(1, self.nblocks + 1):
            npp, nph, nhh = (int(x) for x in dims[q - 1][3:6])
            n = {1: npp, 2: nph, 3: nhh}
            qn = {c: orc.block_qn(q, c) for c in (1, 2, 3)}
            self.qn.append(qn)
            for c in (1, 2, 3):
                for r, (a, b) in enumerate(qn[c]):
                    self.row[(int(a), int(b), int(dims[q - 1][0]))] = r
            # gam 1..6: (pp,pp) (pp,ph) (pp,hh) (ph,ph) (hh,hh) (ph,hh)
            shp = [(n[1], n[1]), (n[1], n[2]), (n[1], n[3]), (n[2], n[2]), (n[3], n[3]), (n[2], n[3])]
            offs = []
            for n1, n2 in shp:
                offs.append(off)
                off += n1 * n2
            self.goff.append(offs)
            self.gshape.append(shp)
        self.nfull = off
        assert self.nfull == orc.nfull
        self.jtm = int(self.jj.max())
        self.lmax = int(self.ll.max())

    def gx(self, q, g, i, j):
        """flat index of gam(g)%X(i, j) of block q (1-based q, g; 0-based i, j)."""
        return self.goff[q - 1][g - 1] + i + j * self.gshape[q - 1][g - 1][0]

    def f_index(self, a, b):
        """flat index of the stored one-body element read by f_elem(a, b)."""
        ca, cb = self.con[a - 1], self.con[b - 1]
        if ca + cb == 0:
            return self.off_fpp + self.pos[a] + self.pos[b] * self.P
        if ca + cb == 2:
            return self.off_fhh + self.pos[a] + self.pos[b] * self.A
        if ca > cb:
            return self.off_fph + self.pos[b] + self.pos[a] * self.P
        return self.off_fph + self.pos[a] + self.pos[b] * self.P

    # ----------------------------------------------------------------- COM
    def _reduced(self, a, b, p):
        la, lb, na, nb = self.ll[a - 1], self.ll[b - 1], self.nn[a - 1], self.nn[b - 1]
        c1 = p1 = 0.0
        if la == lb + 1:
            c1 = np.sqrt(lb + 1.0)
            if na == nb:
                p1 = (-1.0 if p else 1.0) * np.sqrt(nb + lb + 1.5)
            elif na == nb - 1:
                p1 = -np.sqrt(nb * 1.0)
        elif la == lb - 1:
            c1 = -np.sqrt(1.0 * lb)
            if na == nb:
                p1 = np.sqrt(nb + lb + 0.5)
            elif na == nb + 1:
                p1 = (1.0 if p else -1.0) * np.sqrt(nb + 1.0)
        return p1 * c1

    def _jx(self, x, y, p):
        if self.itzp[x - 1] != self.itzp[y - 1]:
            return 0.0
        jx, jy, lx, ly = self.jj[x - 1], self.jj[y - 1], self.ll[x - 1], self.ll[y - 1]
        return (np.sqrt((jx + 1.0) * (jy + 1.0)) * _pm1(_fdiv(3 + 2 * lx + jy, 2)) *
                self.orc.d6ji(int(jx), 2, int(jy), int(2 * ly), 1, int(2 * lx)) * self._reduced(x, y, p))

    def r1_r2_p1_p2(self, a, b, c, d, J, p):
        """r1_r2 (p False) or p1_p2 (p True) of basic_IMSRG.f90:4310-4420."""
        ja, jb, jc, jd = (int(self.jj[x - 1]) for x in (a, b, c, d))
        j_ac, j_ad = self._jx(a, c, p), self._jx(a, d, p)
        j_bc, j_bd = self._jx(b, c, p), self._jx(b, d, p)
        s1 = _fdiv(jb - jc - J, 2) if p else _fdiv(jb + jc - J, 2)
        s2 = _fdiv(jb - jd - J, 2) if p else _fdiv(jb + jd - J, 2)
        v = (_pm1(s1) * self.orc.d6ji(ja, jb, J, jd, jc, 2) * j_ac * j_bd -
             _pm1(_fdiv(jc + jd - J, 2)) * _pm1(s2) * self.orc.d6ji(ja, jb, J, jc, jd, 2) * j_ad * j_bc)
        return v / np.sqrt((1.0 + (a == b)) * (1.0 + (c == d)))

    # --------------------------------------------------------------- reader
    def read_interaction(self, path, htype=1, hw=20.0, com_hw=None, lawson_beta=0.0, mass=16):
        """interaction_IO.f90:8-107 into a zero operator."""
        com_hw = hw if com_hw is None else com_hw
        H = np.zeros(self.nfull)
        com = 1.0 if htype == 1 else 0.0
        with open(path) as f:
            lines = f.read().splitlines()[8:]
        for line in lines:
            if not line.strip():
                continue
            t = line.split()
            Tz, Par, J, a, b, c, d = (int(x) for x in t[:7])
            V = float(t[7])
            g2 = self.r1_r2_p1_p2(a, b, c, d, J, False)
            g3 = self.r1_r2_p1_p2(a, b, c, d, J, True)
            g1 = (g3 + com_hw ** 2 / hw ** 2 * g2) * lawson_beta
            V = V + (g1 - g3 * com) * hw / mass
            q = 3 * J + 2 * (Tz + 1) + Par + 1
            C1 = self.con[a - 1] + self.con[b - 1] + 1
            C2 = self.con[c - 1] + self.con[d - 1] + 1
            qx = C1 * C2
            if qx == 9:
                qx = 5
            pre = 1.0
            if a > b:
                i1 = self.row[(b, a, J)]
                pre = _pm1(1 + _fdiv(self.jj[a - 1] + self.jj[b - 1] - J, 2))
            else:
                i1 = self.row[(a, b, J)]
            if c > d:
                i2 = self.row[(d, c, J)]
                pre *= _pm1(1 + _fdiv(self.jj[c - 1] + self.jj[d - 1] - J, 2))
            else:
                i2 = self.row[(c, d, J)]
            if qx in (1, 5, 4):
                H[self.gx(q, qx, i2, i1)] = V * pre
                H[self.gx(q, qx, i1, i2)] = V * pre
            elif C1 > C2:
                H[self.gx(q, qx, i2, i1)] = V * pre
            else:
                H[self.gx(q, qx, i1, i2)] = V * pre
        return H

    # -------------------------------------------------------------- h0 (HO)
    def h0_harm_osc(self, H, htype=1, hw=20.0, com_hw=None, lawson_beta=0.0, mass=16):
        """basic_IMSRG.f90:2049-2147 into the one-body part of a copy of H."""
        com_hw = hw if com_hw is None else com_hw
        out = H.copy()
        out[self.off_fhh:self.off_fpp + self.P * self.P] = 0.0
        kd = lambda x, y: 1.0 if x == y else 0.0  # noqa: E731
        f32 = np.float32
        for i in range(1, self.N + 1):
            ni, li, ji, ti = self.nn[i - 1], self.ll[i - 1], self.jj[i - 1], self.itzp[i - 1]
            for j in range(i, self.N + 1):
                nj, lj = self.nn[j - 1], self.ll[j - 1]
                if li != lj or ji != self.jj[j - 1] or ti != self.itzp[j - 1] or abs(ni - nj) > 1:
                    continue
                if ni == nj:
                    kij = 0.5 * hw * float(f32(2 * nj + lj) + f32(1.5))
                elif ni == nj - 1:
                    kij = 0.5 * hw * float(np.sqrt(f32(nj) * (f32(nj + lj) + f32(0.5))))
                else:
                    kij = 0.5 * hw * float(np.sqrt(f32(nj + 1) * (f32(nj + lj) + f32(1.5))))
                hcm = kij * (kd(ni, nj) - kd(ni, nj + 1) - kd(ni, nj - 1)) / mass
                if htype == 1:
                    if abs(lawson_beta) < 1e-5:
                        T = kij * (1.0 - 1.0 / mass)
                    else:
                        T = (kij * (1.0 + (lawson_beta - 1.0) / mass) + lawson_beta * com_hw * com_hw / (hw * hw) * kij
                             * (kd(ni, nj) - kd(ni, nj + 1) - kd(ni, nj - 1)) / mass)
                elif htype == 2:
                    T = 2 * kij * kd(ni, nj)
                elif htype == 3:
                    T = kij
                elif htype == 4:
                    T = kij / mass
                else:
                    T = hcm
                out[self.f_index(i, j)] = T
                if self.con[i - 1] == self.con[j - 1]:
                    out[self.f_index(j, i)] = T
        return out

    # ------------------------------------------------------------ Hartree-Fock
    def sp_blocks(self):
        """(l, j, tz) blocks in allocate_sp_mat order (basic_IMSRG.f90:2600-2660)."""
        out = []
        for tz in (-1, 1):
            for l in range(self.lmax + 1):
                for j in range(1, self.jtm + 1, 2):
                    st = [i for i in range(1, self.N + 1)
                          if self.ll[i - 1] == l and self.jj[i - 1] == j and self.itzp[i - 1] == tz]
                    out.append((j, st))
        return out

    def hartree_fock(self, H, tol=1e-6, max_iter=1000):
        """calc_HF: returns (H in the normal-ordered HF basis, E_HF, D, iterations)."""
        orc, blocks = self.orc, self.sp_blocks()
        T = []
        for j, st in blocks:  # write_kin_matrix
            n = len(st)
            M = np.zeros((n, n))
            for a in range(n):
                for b in range(a, n):
                    M[a, b] = M[b, a] = orc.f_elem(st[a], st[b], H, 1)
            T.append(M)
        # gamma_matrix's v_elem sums, which do not change between iterations
        W = []
        for jf, st in blocks:
            n = len(st)
            Wq = []
            for a in range(n):
                row = []
                for b in range(a, n):
                    per = []
                    for jr, sr in blocks:
                        m = len(sr)
                        X = np.zeros((m, m))  # X[h, g]
                        for g in range(m):
                            for h in range(m):
                                s = 0.0
                                for JJ in range(abs(jr - jf), jr + jf + 1, 2):
                                    s += orc.v_elem(st[a], sr[g], st[b], sr[h], JJ, H, 1) * (JJ + 1.0) / (jr + 1.0)
                                X[h, g] = s
                        per.append(X)
                    row.append(per)
                Wq.append(row)
            W.append(Wq)
        D = [np.eye(len(st)) for _, st in blocks]
        eig = [np.zeros(len(st)) for _, st in blocks]
        crit, it = 10.0, 0
        while crit > tol:
            if it == max_iter:
                raise RuntimeError("Hartree-Fock did not converge")
            rho = []
            for q, (j, st) in enumerate(blocks):  # density_matrix
                Dx = D[q] * np.array([self.con[s - 1] for s in st], float)[None, :]
                rho.append(Dx @ Dx.T * (j + 1))
            gam = []
            for q, (jf, st) in enumerate(blocks):  # gamma_matrix
                n = len(st)
                G = np.zeros((n, n))
                for a in range(n):
                    for b in range(a, n):
                        sm = sum(float(np.sum(rho[r] * W[q][a][b - a][r])) for r in range(len(blocks)))
                        G[a, b] = G[b, a] = sm / (jf + 1.0)
                gam.append(G)
            crit = 0.0
            for q in range(len(blocks)):
                e, v = np.linalg.eigh(T[q] + gam[q]) if len(blocks[q][1]) else (np.zeros(0), np.zeros((0, 0)))
                crit += np.sqrt(np.sum((eig[q] - e) ** 2))
                D[q], eig[q] = v, e
            it += 1
        out = H.copy()
        out[self.off_fhh:self.off_fpp + self.P * self.P] = 0.0
        ehf = 0.0
        Dsm = np.zeros((self.N + 1, self.N + 1))
        for q, (j, st) in enumerate(blocks):
            n = len(st)
            if n == 0:
                continue
            for i in range(n):  # sign convention (:74-81)
                if D[q][i, i] < 0.0:
                    D[q][:, i] *= -1
            F = T[q] + gam[q]
            F1, T1, G1 = (D[q].T @ X @ D[q] for X in (F, T[q], gam[q]))  # transform_1b_to_HF
            for i in range(n):  # e_HF
                ehf += (T1[i, i] + 0.5 * G1[i, i]) * self.con[st[i] - 1] * (j + 1.0)
            for a in range(n):
                for c in range(n):
                    Dsm[st[a], st[c]] = D[q][a, c]
                for c in range(a, n):
                    i, k = st[a], st[c]
                    ci, ck = self.con[i - 1], self.con[k - 1]
                    if ci + ck in (0, 2):
                        out[self.f_index(i, k)] = F1[a, c]
                        out[self.f_index(k, i)] = F1[a, c]
                    elif ck > ci:
                        out[self.f_index(i, k)] = F1[a, c]
                    else:
                        out[self.f_index(k, i)] = F1[c, a]
        out[0] = ehf
        self._transform_2b(out, Dsm)
        return out, ehf, Dsm[1:, 1:], it

    def transform_to_hf(self, Op, D):
        """sqop_to_HF (HF_mod.f90:108-136) of a Hermitian scalar operator with
        the coefficients D (norb x norb): one-body and two-body parts to the
        HF basis, then normal ordering (the oracle's normal_order)."""
        out = Op.copy()
        out[self.off_fhh:self.off_fpp + self.P * self.P] = 0.0
        for j, st in self.sp_blocks():
            if not st:
                continue
            idx = np.array(st) - 1
            X = np.array([[self.orc.f_elem(a, c, Op, 1) for c in st] for a in st])
            Dq = D[np.ix_(idx, idx)]
            X1 = Dq.T @ X @ Dq
            for a in range(len(st)):
                for c in range(a, len(st)):
                    i, k = st[a], st[c]
                    ci, ck = self.con[i - 1], self.con[k - 1]
                    if ci == ck:
                        out[self.f_index(i, k)] = X1[a, c]
                        out[self.f_index(k, i)] = X1[a, c]
                    elif ck > ci:
                        out[self.f_index(i, k)] = X1[a, c]
                    else:
                        out[self.f_index(k, i)] = X1[c, a]
        Dsm = np.zeros((self.N + 1, self.N + 1))
        Dsm[1:, 1:] = D
        self._transform_2b(out, Dsm)
        return self.orc.normal_order(out, 1)

    def _transform_2b(self, H, Dsm):
        """transform_2b_to_HF (HF_mod.f90:494-619) in place."""
        jj = self.jj
        for q in range(1, self.nblocks + 1):
            qn = self.qn[q - 1]
            nh, nb, npp = len(qn[3]), len(qn[2]), len(qn[1])
            nt = nh + nb + npp
            if nt == 0:
                continue
            G = lambda g: H[self.goff[q - 1][g - 1]:self.goff[q - 1][g - 1] + int(np.prod(  # noqa: E731
                self.gshape[q - 1][g - 1]))].reshape(self.gshape[q - 1][g - 1][::-1]).T
            V = np.zeros((nt, nt))
            h, p = slice(0, nh), slice(nh, nh + nb)
            pp = slice(nh + nb, nt)
            V[h, h] = G(5)
            V[p, h] = G(6)
            V[h, p] = G(6).T
            V[pp, h] = G(3)
            V[h, pp] = G(3).T
            V[p, p] = G(4)
            V[pp, p] = G(2)
            V[p, pp] = G(2).T
            V[pp, pp] = G(1)
            big = np.concatenate([qn[3], qn[2], qn[1]]).reshape(-1, 2)
            Cf = np.zeros((nt, nt))
            Cr = np.zeros((nt, nt))
            for II in range(nt):
                i, j = (int(x) for x in big[II])
                for JJ in range(nt):
                    a, b = (int(x) for x in big[JJ])
                    nrm = np.sqrt(1.0 + (a == b)) / np.sqrt(1.0 + (i == j))
                    Cf[JJ, II] = Dsm[a, i] * Dsm[b, j] * nrm
                    Cr[JJ, II] = Dsm[b, i] * Dsm[a, j] * (1 - (a == b)) * _pm1((jj[a - 1] + jj[b - 1]) // 2) * nrm
            V1 = Cf.T @ (V @ Cf)
            V2 = Cf.T @ (V @ Cr)
            V3 = Cr.T @ (V @ Cf)
            V4 = Cr.T @ (V @ Cr)
            J2 = int(self.orc.block_dims()[q - 1][0])
            V = V1 - _pm1(J2 // 2) * (V2 + V3) + V4
            for g, (rs, cs) in {5: (h, h), 6: (p, h), 3: (pp, h), 4: (p, p), 2: (pp, p), 1: (pp, pp)}.items():
                n1, n2 = self.gshape[q - 1][g - 1]
                if n1 * n2:
                    o = self.goff[q - 1][g - 1]
                    H[o:o + n1 * n2] = V[rs, cs].T.reshape(-1)
