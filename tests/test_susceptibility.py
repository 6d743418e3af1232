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


def _device_formula(b, tab, r):
    """The kernel's field_dbz restated over the packed table (walk-frame positions r (M, 3))."""
    R = np.asarray(b.field_rot[:], np.float64).reshape(3, 3)
    p = r @ R.T
    par = np.asarray(b.field_par[:], np.float64)
    if b.field_kind == 1:
        t = tab.reshape(-1, 5)
        dd = p[:, None, :] - t[None, :, :3]
        q = np.maximum(np.sum(dd * dd, -1), t[:, 4])
        return np.sum(t[:, 3] * (3 * dd[..., 2] ** 2 / q - 1) / q ** 1.5, -1)
    if b.field_kind == 2:
        t = tab.reshape(-1, 8)
        L, ni = par[0], int(par[4])
        x, y = p[:, 0], p[:, 1]
        if par[5]:
            x = np.mod(x + 0.5 * L, L) - 0.5 * L
            y = np.mod(y + 0.5 * L, L) - 0.5 * L
        p0 = pc = ps = 0.0
        for cx, cy, a2, b2, a4, lba, _, _ in t:
            for jy in range(-ni, ni + 1):
                for jx in range(-ni, ni + 1):
                    dx, dy = x - (cx + jx * L), y - (cy + jy * L)
                    r2 = dx * dx + dy * dy
                    r4 = r2 * r2
                    f = np.where(r2 > b2, (b2 - a2) / r4,
                                 np.where(r2 > a2, (r4 - a4) / (r4 * (b2 + a2)), 0.0))
                    p0 = p0 + np.where((r2 > a2) & (r2 <= b2), -0.5 * np.log(r2 / b2), 0.0)
                    p0 = p0 + np.where(r2 < a2, lba, 0.0)
                    pc = pc + f * (dx * dx - dy * dy)
                    ps = ps + f * 2 * dx * dy
        return par[1] * p0 + par[1] * (par[2] * pc + par[3] * ps)
    dims = np.asarray(b.field_dims[:])
    idx = (p - par[:3]) / par[3:6] - 0.5
    return su._trilinear(tab.reshape(tuple(dims)), np.mod(idx, dims) if par[6] else idx,
                         (bool(par[6]),) * 3)


@pytest.mark.parametrize("kind", ["spheres", "myelin", "grid"])
def test_device_tables_reproduce_the_providers(kind):
    """The tables and parameters simulate_bloch hands the kernel (bloch._field_params), read
    with the kernel's formulas, give the provider's field, in a rotated cylinder's walk frame."""
    import dmipy_sim_gb300 as d
    from dmipy_sim_gb300 import _lib
    from dmipy_sim_gb300.bloch import _field_params
    x = susceptibility_inputs()
    if kind == "spheres":
        prov = su.SusceptibilitySources(x["sph_c"], x["sph_a"], x["sph_chi"], B0=3.0)
    elif kind == "myelin":
        prov = su.MyelinSusceptibility(x["my_c"], x["my_a"], x["my_b"], 8e-6, theta=0.9,
                                       alpha=0.2)
    else:
        prov = su.GridSusceptibility(x["grid"], [-1e-6, -0.5e-6, 0.2e-6], 0.4e-6, periodic=True)
    g = d.Cylinder(4e-6, (0.3, 0.2, 1.0))
    b, keep = _lib.BlochParams(), []
    _field_params(prov, g, 1e-4, b, "cpu", keep)
    r_lab = x["pts"]
    r_walk = d.core._to_frame(g, r_lab.astype(np.float32)).astype(np.float64)
    got = _device_formula(b, keep[0].numpy().astype(np.float64), r_walk)
    want = prov.delta_bz_fn()(r_lab)
    np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-6 * np.abs(want).max())
