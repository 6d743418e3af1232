"""Susceptibility fields (dmipy_sim_gb300.susceptibility) against dmipy-sim's own providers, k-space
dipole solver and grid sampler (tests/golden/susceptibility_kat.npz)."""
from pathlib import Path

import numpy as np
import pytest

from dmipy_sim_gb300 import susceptibility as su
from golden.make_golden import susceptibility_inputs


@pytest.fixture(scope="module")
def z():
    return np.load(Path(__file__).parent / "golden" / "susceptibility_kat.npz")


def test_sphere_sources_match_reference(z):
    x = susceptibility_inputs()
    f = su.SusceptibilitySources(x["sph_c"], x["sph_a"], x["sph_chi"], B0=3.0).delta_bz_fn()
    np.testing.assert_allclose(f(x["pts"]), z["sph"], rtol=2e-5, atol=1e-12)
    np.testing.assert_allclose(f(x["pts"][3]), z["sph"][3], rtol=2e-5, atol=1e-12)


@pytest.mark.parametrize("k,th,al,per", [(0, 0.7, 0.3, True), (1, np.pi / 2, 1.1, True),
                                         (2, 1.2, 0.0, False)])
def test_myelin_cylinders_match_reference(z, k, th, al, per):
    x = susceptibility_inputs()
    g = su.MyelinSusceptibility(x["my_c"], x["my_a"], x["my_b"], 8e-6, delta_chi_a=-0.1e-6,
                                B0=3.0, theta=th, alpha=al, periodic=per).delta_bz_fn()
    ref = z[f"my{k}"]
    np.testing.assert_allclose(g(x["pts"]), ref, rtol=1e-4, atol=1e-6 * np.abs(ref).max())


def test_dipole_solver_tensor_and_sampler_match_reference(z):
    x = susceptibility_inputs()
    chi6 = su.myelin_susceptibility_tensor(x["mask"], x["rad"], chi_iso=-0.05e-6,
                                           chi_aniso=-0.1e-6)
    np.testing.assert_allclose(chi6, z["chi6"], rtol=1e-13, atol=1e-22)
    dB = su.dipole_field(chi6, [0.2e-6, 0.25e-6, 0.3e-6], [0.3, 0.2, 1.0], B0=3.0)
    np.testing.assert_allclose(dB, z["dB"], rtol=1e-10, atol=1e-12 * np.abs(z["dB"]).max())
    sdf = np.linalg.norm(np.stack(np.meshgrid(*[np.arange(n) - n / 2 for n in (12, 10, 8)],
                                              indexing="ij"), -1), axis=-1) - 3.0
    np.testing.assert_allclose(su.radial_from_sdf(sdf, 0.2e-6), z["radial"], rtol=1e-12,
                               atol=1e-12)
    org = np.array([-1e-6, -0.5e-6, 0.2e-6])
    for per, key in ((False, "samp_clamp"), (True, "samp_wrap")):
        np.testing.assert_allclose(su.sample_grid(x["grid"], z["samp_q"], org, 0.4e-6,
                                                  periodic=per), z[key], rtol=1e-10, atol=1e-12)
        prov = su.GridSusceptibility(x["grid"], org, 0.4e-6, periodic=per).delta_bz_fn()
        np.testing.assert_allclose(prov(z["samp_q"]), z[key], rtol=1e-5, atol=1e-6)
