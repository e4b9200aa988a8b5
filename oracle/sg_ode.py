"""Shampine-Gordon ODE solver and the IMSRG ODE flow (test infrastructure only).

A numpy restatement of the solver the reference hands its flow equations to
(im-SRG/adams_ode.f90: ODE :33-247, DE :249-595, STEP :597-1230, INTRP
:1232-1357), the published variable-order (1-12), variable-step Adams PECE
method with local extrapolation of L. F. Shampine and M. K. Gordon, "Computer
Solution of Ordinary Differential Equations" (Freeman, 1975), and of the
single-operator flow driver decouple_hamiltonian (im-SRG/IMSRG_ODE.f90:9-178)
with its derivative dHds (:416-463).  Only the tests use this module; the GPU
library restates the same algorithm on the device.

The state vector is the reference's packed operator (vectorize order); the
error norms of STEP are sums over it, as in the reference.
"""
from __future__ import annotations

import math

import numpy as np

# STEP's error-constant and power-of-two tables (adams_ode.f90:772-780), the
# published method's constants
GSTR = (0.50, 0.0833, 0.0417, 0.0264, 0.0188, 0.0143, 0.0114, 0.00936, 0.00789, 0.00679, 0.00592,
        0.00524, 0.00468)
TWO = tuple(2.0 ** i for i in range(1, 14))
EPSILON = np.finfo(np.float64).eps
MAXNUM = 500  # DE's step budget per call (adams_ode.f90:404)


class ShampineGordon:
    """Integrates dy/dt = f(t, y) from call to call like ODE with a positive
    IFLAG: the first call starts (iflag 1), later calls continue (iflag 2..5
    as returned).  Arrays use 1-based column numbers of the reference through
    phi[i - 1]."""

    def __init__(self, f, neqn):
        self.f = f
        self.n = neqn
        self.nfev = 0
        self.yy = np.zeros(neqn)
        self.wt = np.zeros(neqn)
        self.p = np.zeros(neqn)
        self.yp = np.zeros(neqn)
        self.ypout = np.zeros(neqn)
        self.phi = np.zeros((16, neqn))
        self.alpha = np.zeros(12)
        self.beta = np.zeros(12)
        self.sig = np.zeros(13)
        self.v = np.zeros(12)
        self.w = np.zeros(12)
        self.g = np.zeros(13)
        self.psi = np.zeros(12)
        self.x = self.h = self.hold = self.told = self.delsgn = 0.0
        self.start = self.phase1 = self.nornd = False
        self.ns = self.k = self.kold = 0
        self.isnold = 0

    def _f(self, t, y):
        self.nfev += 1
        return self.f(t, y)

    # DE (adams_ode.f90:249-595), positive IFLAG only (the flow driver's use)
    def ode(self, y, t, tout, relerr, abserr, iflag):
        """Returns (y, t, relerr, abserr, iflag) like ODE."""
        fouru = 4.0 * EPSILON
        if t == tout or relerr < 0.0 or abserr < 0.0:
            return y, t, relerr, abserr, 6
        eps = max(relerr, abserr)
        if eps <= 0.0 or iflag <= 0:
            return y, t, relerr, abserr, 6
        isn = 1
        if iflag != 1:
            if t != self.told or not 2 <= iflag <= 5:
                return y, t, relerr, abserr, 6
        dl = tout - t
        absdel = abs(dl)
        tend = t + 10.0 * dl
        nostep = 0
        kle4 = 0
        stiff = False
        releps = relerr / eps
        abseps = abserr / eps
        if iflag == 1 or self.isnold < 0 or self.delsgn * dl <= 0.0:
            self.start = True
            self.x = t
            self.yy = y.copy()
            self.delsgn = math.copysign(1.0, dl)
            self.h = math.copysign(max(abs(tout - self.x), fouru * abs(self.x)), tout - self.x)
        while True:
            if absdel <= abs(self.x - t):
                y = self.intrp(tout)
                self.told = t = tout
                self.isnold = isn
                return y, t, relerr, abserr, 2
            if MAXNUM <= nostep:
                y = self.yy.copy()
                self.told = t = self.x
                self.isnold = 1
                return y, t, relerr, abserr, 5 if stiff else 4
            self.h = math.copysign(min(abs(self.h), abs(tend - self.x)), self.h)
            self.wt = releps * np.abs(self.yy) + abseps
            crash, eps = self.step(eps)
            if crash:
                relerr, abserr = eps * releps, eps * abseps
                y = self.yy.copy()
                self.told = t = self.x
                self.isnold = 1
                return y, t, relerr, abserr, 3
            nostep += 1
            kle4 += 1
            if self.kold > 4:
                kle4 = 0
            if kle4 >= 50:
                stiff = True

    # STEP (adams_ode.f90:597-1230); returns (crash, eps)
    def step(self, eps):
        twou = 2.0 * EPSILON
        fouru = 2.0 * twou
        phi, g, sig = self.phi, self.g, self.sig
        alpha, beta, psi, v, w = self.alpha, self.beta, self.psi, self.v, self.w
        if abs(self.h) < fouru * abs(self.x):
            self.h = math.copysign(fouru * abs(self.x), self.h)
            return True, eps
        p5eps = 0.5 * eps
        rnd = twou * math.sqrt(np.sum((self.yy / self.wt) ** 2))
        if p5eps < rnd:
            return True, 2.0 * rnd * (1.0 + fouru)
        g[0], g[1], sig[0] = 1.0, 0.5, 1.0
        if self.start:
            self.yp = self._f(self.x, self.yy)
            phi[0] = self.yp
            phi[1] = 0.0
            total = math.sqrt(np.sum((self.yp / self.wt) ** 2))
            absh = abs(self.h)
            if eps < 16.0 * total * self.h * self.h:
                absh = 0.25 * math.sqrt(eps / total)
            self.h = math.copysign(max(absh, fouru * abs(self.x)), self.h)
            self.hold = 0.0
            self.k, self.kold = 1, 0
            self.start = False
            self.phase1 = True
            self.nornd = True
            if p5eps <= 100.0 * rnd:
                self.nornd = False
                phi[14] = 0.0
        ifail = 0
        while True:
            k, h = self.k, self.h
            kp1, kp2, km1, km2 = k + 1, k + 2, k - 1, k - 2
            if h != self.hold:
                self.ns = 0
            if self.ns <= self.kold:
                self.ns += 1
            ns = self.ns
            nsp1 = ns + 1
            if ns <= k:
                beta[ns - 1] = 1.0
                alpha[ns - 1] = 1.0 / ns
                temp1 = h * ns
                sig[nsp1 - 1] = 1.0
                for i in range(nsp1, k + 1):
                    temp2 = psi[i - 2]
                    psi[i - 2] = temp1
                    beta[i - 1] = beta[i - 2] * psi[i - 2] / temp2
                    temp1 = temp2 + h
                    alpha[i - 1] = h / temp1
                    sig[i] = i * alpha[i - 1] * sig[i - 1]
                psi[k - 1] = temp1
                if ns <= 1:
                    for iq in range(1, k + 1):
                        v[iq - 1] = 1.0 / (iq * (iq + 1))
                        w[iq - 1] = v[iq - 1]
                else:
                    if self.kold < k:
                        v[k - 1] = 1.0 / (k * kp1)
                        for j in range(1, ns - 1):
                            i = k - j
                            v[i - 1] = v[i - 1] - alpha[j] * v[i]
                    for iq in range(1, kp1 - ns + 1):
                        v[iq - 1] = v[iq - 1] - alpha[ns - 1] * v[iq]
                        w[iq - 1] = v[iq - 1]
                    g[nsp1 - 1] = w[0]
                for i in range(ns + 2, kp1 + 1):
                    for iq in range(1, kp2 - i + 1):
                        w[iq - 1] = w[iq - 1] - alpha[i - 2] * w[iq]
                    g[i - 1] = w[0]
            # predict (element-wise; the same operations in the same order as
            # the reference's column loops)
            for i in range(nsp1, k + 1):
                phi[i - 1] = beta[i - 1] * phi[i - 1]
            phi[kp2 - 1] = phi[kp1 - 1]
            phi[kp1 - 1] = 0.0
            pp = np.zeros(self.n)
            for j in range(1, k + 1):
                i = kp1 - j
                pp = pp + phi[i - 1] * g[i - 1]
                phi[i - 1] = phi[i - 1] + phi[i]
            if not self.nornd:
                tau = h * pp - phi[14]
                self.p = self.yy + tau
                phi[15] = (self.p - self.yy) - tau
            else:
                self.p = self.yy + h * pp
            xold = self.x
            self.x = self.x + h
            absh = abs(h)
            self.yp = self._f(self.x, self.p)
            d1 = (self.yp - phi[0]) / self.wt
            erkm2 = erkm1 = 0.0
            if km2 > 0:
                erkm2 = absh * sig[km1 - 1] * GSTR[km2 - 1] * math.sqrt(
                    np.sum(((phi[km1 - 1] + self.yp - phi[0]) / self.wt) ** 2))
            if km2 >= 0:
                erkm1 = absh * sig[k - 1] * GSTR[km1 - 1] * math.sqrt(
                    np.sum(((phi[k - 1] + self.yp - phi[0]) / self.wt) ** 2))
            serk = math.sqrt(np.sum(d1 ** 2))
            err = absh * serk * (g[k - 1] - g[kp1 - 1])
            erk = absh * serk * sig[kp1 - 1] * GSTR[k - 1]
            knew = k
            if km2 > 0:
                if max(erkm1, erkm2) <= erk:
                    knew = km1
            elif km2 == 0:
                if erkm1 <= 0.5 * erk:
                    knew = km1
            if err <= eps:
                break
            # failed step: restore, shrink h, maybe lower the order
            self.phase1 = False
            self.x = xold
            for i in range(1, k + 1):
                phi[i - 1] = (phi[i - 1] - phi[i]) / beta[i - 1]
            for i in range(2, k + 1):
                psi[i - 2] = psi[i - 1] - h
            ifail += 1
            temp2 = 0.5
            if ifail > 3 and p5eps < 0.25 * erk:
                temp2 = math.sqrt(p5eps / erk)
            if ifail >= 3:
                knew = 1
            self.h = temp2 * h
            self.k = knew
            if abs(self.h) < fouru * abs(self.x):
                self.h = math.copysign(fouru * abs(self.x), self.h)
                return True, eps + eps
        # correct, evaluate, update the differences
        self.kold = k
        self.hold = h
        if not self.nornd:
            rho = h * g[kp1 - 1] * (self.yp - phi[0]) - phi[15]
            self.yy = self.p + rho
            phi[14] = (self.yy - self.p) - rho
        else:
            self.yy = self.p + h * g[kp1 - 1] * (self.yp - phi[0])
        self.yp = self._f(self.x, self.yy)
        phi[kp1 - 1] = self.yp - phi[0]
        phi[kp2 - 1] = phi[kp1 - 1] - phi[kp2 - 1]
        for i in range(1, k + 1):
            phi[i - 1] = phi[i - 1] + phi[kp1 - 1]
        erkp1 = 0.0
        if knew == km1 or k == 12:
            self.phase1 = False
        if self.phase1:
            self.k = kp1
            erk = erkp1
        elif knew == km1:
            self.k = km1
            erk = erkm1
        elif kp1 <= self.ns:
            erkp1 = absh * GSTR[kp1 - 1] * math.sqrt(np.sum((phi[kp2 - 1] / self.wt) ** 2))
            if k == 1:
                if erkp1 < 0.5 * erk:
                    self.k = kp1
                    erk = erkp1
            elif erkm1 <= min(erk, erkp1):
                self.k = km1
                erk = erkm1
            elif erkp1 < erk and k < 12:
                self.k = kp1
                erk = erkp1
        hnew = h + h
        if not self.phase1:
            if p5eps < erk * TWO[self.k]:
                hnew = h
                if p5eps < erk:
                    r = (p5eps / erk) ** (1.0 / (self.k + 1))
                    hnew = absh * max(0.5, min(0.9, r))
                    hnew = math.copysign(max(hnew, fouru * abs(self.x)), h)
        self.h = hnew
        return False, eps

    # INTRP (adams_ode.f90:1232-1357)
    def intrp(self, xout):
        hi = xout - self.x
        ki = self.kold + 1
        w = [1.0 / i for i in range(1, ki + 1)] + [0.0]
        g = [0.0] * (ki + 1)
        rho = [0.0] * (ki + 1)
        g[0] = rho[0] = 1.0
        term = 0.0
        for j in range(2, ki + 1):
            psijm1 = self.psi[j - 2]
            gamma = (hi + term) / psijm1
            eta = hi / psijm1
            for i in range(1, ki + 2 - j):
                w[i - 1] = gamma * w[i - 1] - eta * w[i]
            g[j - 1] = w[0]
            rho[j - 1] = gamma * rho[j - 2]
            term = psijm1
        yout = np.zeros(self.n)
        ypout = np.zeros(self.n)
        for j in range(1, ki + 1):
            i = ki + 1 - j
            yout = yout + g[i - 1] * self.phi[i - 1]
            ypout = ypout + rho[i - 1] * self.phi[i - 1]
        self.ypout = ypout
        return self.yy + hi * yout


def decouple_hamiltonian(orc, H, generator="white", ds=0.1, max_steps=10000, conv=1e-6, relerr=1e-6,
                         abserr=1e-6, s_max=0.0):
    """decouple_hamiltonian (IMSRG_ODE.f90:9-178), one operator: integrate
    dH/ds = [eta(H), H] with the Shampine-Gordon solver in output steps of ds
    until |E_mbpt2| < conv (or s_max > 0 is reached, or max_steps).  Returns H
    (flat layout), the trace rows (step, s, E0, E0 + E_mbpt2, |E_mbpt2|) and
    the number of derivative evaluations."""
    gen = {"white": orc.white, "atan": orc.atan_gen, "w2": orc.w2_gen}[generator]

    def dhds(t, y):  # IMSRG_ODE.f90:416-463
        hs = orc.repackage(y, 1)
        return orc.vectorize(orc.commutator(gen(hs), -1, hs, 1))

    hs = H.copy()
    solver = ShampineGordon(dhds, orc.neq)
    s, steps, iflag = 0.0, 0, 1
    emp2 = orc.mbpt2(hs)
    trace = [(0, s, hs[0], hs[0] + emp2, abs(emp2))]
    while steps < max_steps:
        y = orc.vectorize(hs)
        y, s, relerr, abserr, iflag = solver.ode(y, s, s + ds, relerr, abserr, iflag)
        if iflag == 6:
            raise ValueError("invalid solver input")
        hs = orc.repackage(y, 1)
        steps += 1
        emp2 = orc.mbpt2(hs)
        trace.append((steps, s, hs[0], hs[0] + emp2, abs(emp2)))
        if abs(emp2) < conv or (s_max > 0.0 and s >= s_max - 1e-12):
            break
    return dict(H=hs, trace=np.array(trace), steps=steps, nfev=solver.nfev)
