"""diaq_expm_negative_pade against the reference's Pade routine (src/spME.cpp:298-445) run on its
own CPU build (tests/golden/pade.npz): one-diagonal inputs give the fixture's exponential (to
1e-12; the device's exp/sin/cos against the host's libm), every other input the reference's
exception message with the library's status."""
import ctypes

import numpy as np
import pytest

from conftest import golden, maxrel

pytestmark = pytest.mark.gpu


def _cases():
    g = golden("pade.npz")
    names = sorted({k[: -len("_shape")] for k in g.files if k.endswith("_shape")})
    return g, names


@pytest.mark.parametrize("name", _cases()[1])
def test_pade_matches_reference(native, name):
    capi, _ = native
    g, _ = _cases()
    rows, cols = (int(v) for v in g[f"{name}_shape"])
    A = capi.Matrix.create(rows, cols, g[f"{name}_off"], g[f"{name}_re"], g[f"{name}_im"])
    t = float(g[f"{name}_t"])
    U = ctypes.c_void_p()
    st = capi.lib().diaq_expm_negative_pade(A.h, t, 100, 1.0, 1e-12, None, ctypes.byref(U))
    if f"{name}_error" in g.files:
        assert st != 0
        assert capi.lib().diaq_last_error().decode() == str(g[f"{name}_error"])
        assert st == (1 if "shapes" in str(g[f"{name}_error"]) else 4)
        assert not U.value
        return
    assert st == 0, capi.lib().diaq_last_error().decode()
    U = capi.Matrix(U)
    off, re, im = U.download()
    assert np.array_equal(off, g[f"{name}_U_off"])
    assert U.info()[:2] == (rows, rows)
    assert maxrel(re + 1j * im, g[f"{name}_U_re"] + 1j * g[f"{name}_U_im"]) < 1e-12


def test_pade_empty_matrix_is_an_error(native):
    """No diagonals: the reference's process ends (its inverse throws inside an OpenMP loop); here
    the same message comes back as a status."""
    capi, _ = native
    A = capi.Matrix.create(4, 4, np.zeros(0, dtype=np.int32), np.zeros(0), np.zeros(0))
    U = ctypes.c_void_p()
    assert capi.lib().diaq_expm_negative_pade(A.h, 0.5, 100, 1.0, 1e-12, None, ctypes.byref(U)) == 4
    assert "singular" in capi.lib().diaq_last_error().decode()
