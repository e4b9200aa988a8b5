"""The oracle's Shampine-Gordon restatement (adams_ode.f90 ODE/DE/STEP/INTRP)
against known answers: analytic solutions of small systems at the solver's
tolerances, and a fine fixed-step RK4 integration of the IMSRG flow."""
import math

import numpy as np
import pytest

from conftest import make_case


def _solve(f, y0, t_out, relerr=1e-6, abserr=1e-6):
    from oracle.sg_ode import ShampineGordon
    sg = ShampineGordon(f, len(y0))
    y, t, iflag = np.array(y0, float), 0.0, 1
    out = []
    for t1 in t_out:
        y, t, relerr, abserr, iflag = sg.ode(y, t, t1, relerr, abserr, iflag)
        assert iflag == 2
        out.append(y.copy())
    return np.array(out), sg


def test_exponential_decay():
    t_out = np.arange(1, 21) * 0.25
    ys, sg = _solve(lambda t, y: -y, [1.0, 2.0], t_out)
    exact = np.exp(-t_out)[:, None] * np.array([1.0, 2.0])
    assert np.max(np.abs(ys - exact)) < 1e-5
    assert sg.nfev < 200


def test_harmonic_oscillator_keeps_order_and_accuracy():
    # y'' = -y as a system; the solver raises its order on a smooth problem
    t_out = np.arange(1, 41) * 0.5
    ys, sg = _solve(lambda t, y: np.array([y[1], -y[0]]), [0.0, 1.0], t_out, 1e-9, 1e-9)
    assert np.max(np.abs(ys[:, 0] - np.sin(t_out))) < 1e-7
    assert sg.kold >= 6


def test_tolerance_too_small_reports_iflag_3():
    from oracle.sg_ode import ShampineGordon
    sg = ShampineGordon(lambda t, y: -y, 1)
    y, t, relerr, abserr, iflag = sg.ode(np.array([1.0]), 0.0, 1.0, 1e-20, 0.0, 1)
    assert iflag == 3 and relerr > 1e-20


def test_imsrg_flow_matches_rk4():
    from imsrg_gpu.synth import synth_hamiltonian
    from oracle import oracle as om
    from oracle.sg_ode import decouple_hamiltonian
    bas, lay = make_case(2)
    orc = om.Oracle(**bas)
    H = orc.normal_order(synth_hamiltonian(lay, 21))
    out = decouple_hamiltonian(orc, H, s_max=0.5)

    def f(y):
        hs = orc.repackage(y, 1)
        return orc.vectorize(orc.commutator(orc.white(hs), -1, hs, 1))

    y, h = orc.vectorize(H), 0.0025
    for _ in range(200):
        k1 = f(y)
        k2 = f(y + 0.5 * h * k1)
        k3 = f(y + 0.5 * h * k2)
        k4 = f(y + h * k3)
        y = y + h / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
    assert out["trace"][-1, 1] == pytest.approx(0.5)
    assert abs(out["trace"][-1, 2] - y[0]) < 1e-5
    assert np.max(np.abs(orc.vectorize(out["H"]) - y)) < 1e-4
