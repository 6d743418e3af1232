"""RF pulses and the single-spin Bloch integrator (dmipy_sim_gb300.rf) against dmipy-sim's own
rf.py on the same constructors (tests/golden/rf_kat.npz), plus the closed forms: a hard pulse's
flip, adiabatic inversion across B1+ scales, a slice profile's width."""
from pathlib import Path

import numpy as np
import pytest

from dmipy_sim_gb300 import rf
from golden.make_golden import rf_pulses


@pytest.fixture(scope="module")
def z():
    return np.load(Path(__file__).parent / "golden" / "rf_kat.npz")


@pytest.mark.parametrize("name", ["hard", "sinc", "sinc_rect", "hs", "ahp", "bir4", "comp",
                                  "samples"])
def test_pulses_and_bloch_integration_match_reference(z, name):
    p = rf_pulses(rf)[name]
    # the envelopes are the reference's to rounding (the amplitude scale is formed in another
    # order, so a sample may differ in its last bit)
    np.testing.assert_allclose(p.b1, z[f"{name}_b1"], rtol=1e-13, atol=1e-22)
    np.testing.assert_allclose([p.duration, p.peak_b1, p.b1_rms, p.sar_proxy,
                                p.nominal_flip_deg, p.max_slew_b1], z[f"{name}_props"],
                               rtol=1e-14)
    mxy, mz = rf.bloch_simulate(p, df_hz=np.linspace(-2000.0, 2000.0, 9),
                                b1_scale=np.linspace(0.8, 1.2, 9), T1=0.9, T2=0.05)
    np.testing.assert_allclose(mxy, z[f"{name}_mxy"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(mz, z[f"{name}_mz"], rtol=1e-12, atol=1e-14)


def test_history_and_slice_profile_match_reference(z):
    p = rf_pulses(rf)["hard"]
    mxy, mz, hist = rf.bloch_simulate(p, df_hz=[0.0, 300.0], M0=[0.0, 1.0, 0.0],
                                      return_history=True)
    np.testing.assert_allclose(hist, z["hist"], rtol=1e-12, atol=1e-14)
    _, smxy, smz = rf.slice_profile(rf_pulses(rf)["sinc"], 0.01, np.linspace(-5e-3, 5e-3, 21))
    np.testing.assert_allclose(smxy, z["slice_mxy"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(smz, z["slice_mz"], rtol=1e-12, atol=1e-14)


def test_closed_forms():
    mxy, mz = rf.bloch_simulate(rf.B1Pulse.hard(90.0, 1e-3, 1e-5))
    assert abs(mz[0]) < 1e-12 and abs(mxy[0]) == pytest.approx(1.0, abs=1e-12)
    hs = rf.B1Pulse.adiabatic_hs(10e-3, 1e-5, peak_b1=20e-6)
    _, mz = rf.bloch_simulate(hs, b1_scale=np.array([0.8, 1.0, 1.5, 2.0]))
    assert np.all(mz < -0.95)                     # inversion held over a 2.5 x B1+ range
    with pytest.raises(NotImplementedError):
        hs.deliverability("any")
