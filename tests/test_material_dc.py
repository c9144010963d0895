"""The material derivative behind the single-component DV gradients
(asend_material_dC, host code): dC/dD of C = S^-1 for the reference's
compliance form (element_properties.rs:648-764), against a central
difference of numpy's inverse of that compliance with the one component
perturbed.  Tolerance 1e-7 relative to max |dC| (step 1e-6 relative)."""
import ctypes as C

import numpy as np
import pytest

from asend3d_gb300 import _lib


def compliance(e, nu, g):
    """e = (E1, E2, E3), nu = (nu12, nu13, nu23), g = (G12, G13, G23)."""
    S = np.zeros((6, 6))
    S[0, 0], S[1, 1], S[2, 2] = 1 / e[0], 1 / e[1], 1 / e[2]
    S[0, 1] = S[1, 0] = -nu[0] / e[0]
    S[0, 2] = S[2, 0] = -nu[1] / e[0]
    S[1, 2] = S[2, 1] = -nu[2] / e[1]
    S[3, 3], S[4, 4], S[5, 5] = 1 / g[0], 1 / g[1], 1 / g[2]
    return S


@pytest.mark.parametrize("category", [_lib.DV_MODULUS, _lib.DV_SHEAR_MODULUS, _lib.DV_POISSON_RATIO])
@pytest.mark.parametrize("component", [1, 2, 3])
@pytest.mark.parametrize("E,nu", [(70e9, 0.33), (1e6, 0.0), (200e9, 0.45)])
def test_material_dC_matches_finite_difference(category, component, E, nu):
    lib = _lib.load()
    out = np.zeros(36)
    assert lib.asend_material_dC(category, component, E, nu, out.ctypes.data_as(C.POINTER(C.c_double))) == 0
    G = E / (2 * (1 + nu))
    which = {_lib.DV_MODULUS: 0, _lib.DV_POISSON_RATIO: 1, _lib.DV_SHEAR_MODULUS: 2}[category]
    base = [E, nu, G][which]
    h = 1e-6 * (abs(base) if base != 0 else 1.0)

    def C_of(delta):
        p = [[E] * 3, [nu] * 3, [G] * 3]  # (E1..3), (nu12, nu13, nu23), (G12, G13, G23)
        p[which][component - 1] += delta
        return np.linalg.inv(compliance(p[0], p[1], p[2]))

    fd = (C_of(h) - C_of(-h)) / (2 * h)
    dC = out.reshape(6, 6)
    assert np.abs(dC - fd).max() <= 1e-7 * np.abs(fd).max()


def test_material_dC_rejects_bad_input():
    lib = _lib.load()
    out = np.zeros(36)
    p = out.ctypes.data_as(C.POINTER(C.c_double))
    assert lib.asend_material_dC(3, 1, 1e9, 0.3, p) == _lib.ASEND_EINVAL
    assert lib.asend_material_dC(0, 4, 1e9, 0.3, p) == _lib.ASEND_EINVAL
    assert lib.asend_material_dC(0, 1, 1e9, 0.5, p) == _lib.ASEND_EINVAL
