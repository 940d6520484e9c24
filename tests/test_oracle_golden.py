"""Pin the NumPy oracle against fixtures recorded from the PtyLab.py reference.

The ``reg_*`` and ``prop_*`` fixtures equal the reference's own committed
goldens (tests/regression/data/*.npz) exactly -- ``tests/golden/make_golden.py``
refuses to write them otherwise -- and the ``scan_*`` fixtures are further runs
of the unmodified reference.  The oracle must reproduce all of them to the
reference's own CPU tolerance (rtol=1e-5, atol=1e-7,
tests/regression/test_engine_regression.py:150-154); in practice it is
bit-exact.
"""

import numpy as np
import pytest

from conftest import fixture_names, load_fixture, platform_reproduces_order
from oracle import ptyoracle as O

ENGINE_FIXTURES = fixture_names("reg_") + fixture_names("scan_")


@pytest.mark.parametrize("name", ENGINE_FIXTURES)
def test_oracle_reproduces_reference(name):
    fx = load_fixture(name)
    if not platform_reproduces_order(fx):
        pytest.skip("this platform's np.argsort breaks 'NA'-order ties differently from the recording platform")
    st = O.run_fixture(fx)
    for key in ("object", "probe", "error"):
        np.testing.assert_allclose(
            getattr(st, key), fx[f"out_{key}"], rtol=1e-5, atol=1e-7, err_msg=f"{name}: {key}"
        )
    np.testing.assert_allclose(st.errorAtPos, fx["out_errorAtPos"], rtol=1e-5, atol=1e-7)
    if "out_detectorError" in fx:
        np.testing.assert_allclose(st.detectorError, fx["out_detectorError"], rtol=1e-5, atol=1e-7)
    if "out_objectMomentum" in fx:
        np.testing.assert_allclose(st.objectMomentum, fx["out_objectMomentum"], rtol=1e-5, atol=1e-7)
        np.testing.assert_allclose(st.probeMomentum, fx["out_probeMomentum"], rtol=1e-5, atol=1e-7)
    for key in ("objectBuffer", "probeBuffer", "objectMomentum_v", "probeMomentum_v", "background", "intensityScaling",
                "reference"):
        if f"out_{key}" in fx:
            np.testing.assert_allclose(getattr(st, key), fx[f"out_{key}"], rtol=1e-5, atol=1e-7, err_msg=key)


@pytest.mark.parametrize("name", fixture_names("prop_"))
def test_oracle_propagators(name):
    fx = load_fixture(name)
    prop = str(fx["meta_propagator"])
    g = O.Geometry(
        Np=int(fx["in_Np"]), No=int(fx["in_Np"]), dxp=float(fx["in_dxp"]),
        wavelength=float(fx["in_wavelength"]), zo=float(fx["in_zo"]), dxd=float(fx["in_dxd"]),
        nlambda=int(fx["in_nlambda"]), spectralDensity=tuple(fx["in_spectralDensity"]),
    )
    fwd = O.object2detector(fx["in_field"], prop, False, g)
    back = O.detector2object(fwd, prop, False, g)
    np.testing.assert_allclose(fwd, fx["out_forward"], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(back, fx["out_back"], rtol=1e-5, atol=1e-7)
    # in practice the restatement is bit-exact
    np.testing.assert_array_equal(fwd, fx["out_forward"])
    np.testing.assert_array_equal(back, fx["out_back"])


def test_centred_fft_is_checkerboard_modulated_fft():
    """fft2c(x) == M * fft2(M * x) / N with M = (-1)^(i+j) for N divisible by 4
    (the identity the CUDA kernels use instead of fftshift copies)."""
    rng = np.random.default_rng(0)
    for n in (32, 64, 128, 256):
        x = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        i = np.arange(n)
        M = (-1.0) ** (i[:, None] + i[None, :])
        np.testing.assert_allclose(O.fft2c(x), M * np.fft.fft2(M * x) / n, rtol=1e-10, atol=1e-10)
        np.testing.assert_allclose(O.ifft2c(x), M * np.fft.ifft2(M * x) * n, rtol=1e-10, atol=1e-10)
