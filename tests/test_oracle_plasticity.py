"""Analytic checks of the p122 oracle's Mohr-Coulomb routines (CPU).

INVAR, MOCOUF, MOCOUQ and FORMM (new_library.f90:1813-1916, 2364-2417,
2423-2490, 85-198) restated in oracle/p122_oracle.c, checked against the
mathematics they implement rather than against a recorded run:
  * MOCOUF in invariant form equals the principal-stress Mohr-Coulomb
    function (s1 - s3)/2 + (s1 + s3)/2 sin(phi) - c cos(phi), tension
    positive, s1 >= s2 >= s3, and does not change when the stress is rotated;
  * the viscoplastic flow direction p122 forms, (dq1 m1 + dq2 m2 + dq3 m3)
    stress with dq from MOCOUQ and m from FORMM, is the gradient of the
    plastic potential Q = MOCOUF(psi, c = 0) with respect to the six stress
    components, away from the corners |sin(theta)| > 0.49, where MOCOUQ
    rounds the potential off.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

_D = ctypes.c_double


def _invar(s):
    a, b, c = _D(), _D(), _D()
    O.lib().orc_invar(np.ascontiguousarray(s, dtype=np.float64), ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
    return a.value, b.value, c.value


def _voigt(t):
    """(sx, sy, sz, txy, tyz, tzx), the stress order of INVAR and FORMM."""
    return np.array([t[0, 0], t[1, 1], t[2, 2], t[0, 1], t[1, 2], t[2, 0]])


def test_mocouf_is_the_principal_stress_mohr_coulomb_function():
    rng = np.random.default_rng(2)
    for _ in range(300):
        p = rng.normal(size=3) * 10.0
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        t = q @ np.diag(p) @ q.T
        phi, c = rng.uniform(5.0, 40.0), rng.uniform(0.0, 20.0)
        f = O.lib().orc_mocouf(phi, c, *_invar(_voigt(t)))
        s1, s3, pr = p.max(), p.min(), np.radians(phi)
        expect = 0.5 * (s1 - s3) + 0.5 * (s1 + s3) * np.sin(pr) - c * np.cos(pr)
        assert abs(f - expect) <= 1e-12 * (abs(expect) + 1.0)
        unrotated = O.lib().orc_mocouf(phi, c, *_invar(_voigt(np.diag(p))))
        assert abs(f - unrotated) <= 1e-12 * (abs(f) + 1.0)


@pytest.mark.parametrize("psi", [0.0, 20.0])
def test_flow_direction_is_the_gradient_of_the_plastic_potential(psi):
    L = O.lib()
    rng = np.random.default_rng(1)
    checked = 0
    for _ in range(200):
        s = rng.normal(size=6) * 10.0
        sigm, dsbar, theta = _invar(s)
        if abs(np.sin(theta)) > 0.45 or abs(sigm) < 0.5:
            continue   # the rounded corners, and FORMM's 1/sigm
        dq1, dq2, dq3 = _D(), _D(), _D()
        L.orc_mocouq(psi, dsbar, theta, ctypes.byref(dq1), ctypes.byref(dq2), ctypes.byref(dq3))
        m1, m2, m3 = np.zeros(36), np.zeros(36), np.zeros(36)
        L.orc_formm(np.ascontiguousarray(s), m1, m2, m3)
        m = (dq1.value * m1 + dq2.value * m2 + dq3.value * m3).reshape(6, 6).T   # column-major m(6,6)
        flow = m @ s
        h = 1e-6
        grad = np.array([(L.orc_mocouf(psi, 0.0, *_invar(s + h * e)) - L.orc_mocouf(psi, 0.0, *_invar(s - h * e)))
                         / (2 * h) for e in np.eye(6)])
        assert np.abs(flow - grad).max() <= 1e-6 * np.abs(grad).max()
        checked += 1
    assert checked > 50
