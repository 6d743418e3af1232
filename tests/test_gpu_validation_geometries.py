"""The validation slabs and shell and the ellipsoid on the GPU (Box1D, PermeableSlab1D,
PermeableShell, Ellipsoid): the device
steps against the reference's own plug-in calls (kat.npz), walks against the CPU oracle, and the
closed-form limits these geometries exist for (two-compartment exchange across a planar membrane,
Brownstein-Tarr relaxation between two walls)."""
import numpy as np
import pytest

import dmipy_sim_gb300 as d
from dmipy_sim_gb300 import core
from parity_cases import oracle_walk

pytestmark = pytest.mark.gpu
D = 2e-9
L = 6e-6
CASES = [("box", "reflect"), ("box", "relax"), ("slab", "reflect"), ("slab", "relax"),
         ("slab", "perm"), ("shs", "reflect"), ("shs", "perm"), ("shc", "reflect"),
         ("shc", "perm"), ("ell", "reflect"), ("ell", "relax"), ("ell", "perm")]


def _geom(tag, rho=None, kappa=None):
    if tag == "ell":
        return d.Ellipsoid([2e-6, 3e-6, 4.5e-6], surface_relaxivity_t2=rho, permeability=kappa)
    if tag == "box":
        return d.Box1D(L, surface_relaxivity_t2=rho)
    if tag == "slab":
        return d.PermeableSlab1D(L, permeability=1e-5, surface_relaxivity_t2=rho)
    return d.PermeableShell(2e-6, 4e-6, permeability=1e-5,
                            kind="cylinder" if tag == "shc" else "sphere",
                            surface_relaxivity_t2=rho)


@pytest.mark.parametrize("tag,mode", CASES)
def test_device_step_matches_reference_plugin(cuda, kat, tag, mode):
    g = _geom(tag)
    wall = {"reflect": 0, "relax": 1, "perm": 2}[mode]
    k = f"pl_{tag}_{mode}"
    out, dl = core.step_kat(g, kat[k + "_r"], kat[k + "_step"], kat[k + "_u"], wall=wall)
    ref = kat[k + "_out"]
    scale = np.maximum(np.max(np.abs(ref), axis=1), 1e-6)
    bad = np.max(np.abs(out - ref), axis=1) > 2e-6 * scale
    assert bad.mean() <= 0.01, f"{bad.sum()} of {len(ref)} steps differ"
    if mode != "reflect":
        dref = kat[k + "_dlog"]
        ok = np.abs(dl * 500.0 - dref) <= 1e-4 * np.abs(dref) + 1e-9
        assert ok.mean() >= 0.99


def _plan(g, wf):
    gap = core._replay_gap(g, return_positions=False, return_compartments=False,
                           return_walker_signals=False, diffusivity=D)
    if gap is None and core._replay_auto_allowed(g):
        return core.replay_sub_steps(g, D, wf.dt), False
    return core.fused_sub_steps(g, D, wf.dt), True


@pytest.mark.parametrize("tag", ["box", "slab", "shs", "shc", "ell"])
def test_walks_match_oracle(cuda, tag):
    """Walker by walker over ~100 sub-steps and whole echoes on the same stream, with surface
    relaxivity on (the weighted walls) and T2."""
    g = _geom(tag, rho=2e-6)
    rng = np.random.default_rng(0)
    bv = rng.normal(size=(4, 3))
    bv /= np.linalg.norm(bv, axis=1, keepdims=True)
    wf = d.set_b(d.pgse(0.005, 0.015, 0.05, bv, 60), 1e9)
    G, _ = core._waveform_arrays(wf, g)
    S, ps = _plan(g, wf)
    r0 = g.init_positions(4096, 3)
    if hasattr(g, "_R") and not g._is_identity_rotation:
        r0 = core._to_frame(g, r0)
    n_t = max(2, min(60, 100 // S))
    gpu = core.run_walk(g, n_walkers=4096, diffusivity=D, G=G[:, :n_t], dt=wf.dt, sub_steps=S,
                        phase_per_substep=ps, seed=5, T2=0.07, r0=r0, want_positions=True,
                        want_walker_signals=True)
    ora = oracle_walk(g, G[:, :n_t], wf.dt, S, ps, 4096, seed=5, T2=0.07, r0=r0)
    same = np.max(np.abs(gpu.extras["pos"].cpu().numpy() - ora["pos"]), axis=1) < 1e-4 * 2e-6
    assert same.mean() >= 0.97, f"only {same.mean():.3f} of walkers follow the oracle's walk"
    np.testing.assert_allclose(gpu.extras["phi"].cpu().numpy()[same], ora["phi"][same],
                               atol=1e-3, rtol=1e-4)
    np.testing.assert_allclose(gpu.extras["log_w"].cpu().numpy()[same], ora["log_w"][same],
                               rtol=1e-4, atol=1e-6)
    n = 16384
    r0 = g.init_positions(n, 4)
    if hasattr(g, "_R") and not g._is_identity_rotation:
        r0 = core._to_frame(g, r0)
    gpu = core.run_walk(g, n_walkers=n, diffusivity=D, G=G, dt=wf.dt, sub_steps=S,
                        phase_per_substep=ps, seed=8, T2=0.07, r0=r0)
    ora = oracle_walk(g, G, wf.dt, S, ps, n, seed=8, T2=0.07, r0=r0, want_walkers=False)
    z = (gpu.signal[0] - ora["signal"][0]) / np.maximum(np.sqrt(2.0) * gpu.stderr[0], 1e-9)
    assert np.max(np.abs(z)) < 4.0, z


def test_planar_membrane_exchange(cuda):
    """Every walker starts in A (x < L/2); the fraction still in A after t is
    1/2 + 1/2 exp(-4 kappa t / L) for the closed two-compartment slab (geometries.py:3222-3230)."""
    Ls, kappa = 10e-6, 1e-5
    g = d.PermeableSlab1D(Ls, permeability=kappa)
    wf = d.set_b(d.pgse(0.01, 0.05, 0.05, [[1, 0, 0]], 101), 0.0)
    n = 100_000
    _, c0, c1 = d.simulate(n, D, wf, g, seed=1, return_compartments="final")
    assert np.all(c0 == 0)
    t = (wf.G.shape[1]) * wf.dt
    expect = 0.5 + 0.5 * np.exp(-4.0 * kappa * t / Ls)
    assert abs(np.mean(c1 == 0) - expect) < 0.01, (np.mean(c1 == 0), expect)


def test_two_wall_surface_relaxation_fast_limit(cuda):
    """Box1D with surface relaxivity in the fast-diffusion limit (rho L / D << 1): the b = 0
    signal decays as exp(-rho (S/V) t) with S/V = 2/L."""
    Lb, rho = 5e-6, 1e-6
    g = d.Box1D(Lb, surface_relaxivity_t2=rho)
    wf = d.set_b(d.pgse(0.01, 0.05, 0.05, [[1, 0, 0]], 101), 0.0)
    s = d.simulate(50_000, D, wf, g, seed=2)
    t = (wf.G.shape[1]) * wf.dt
    np.testing.assert_allclose(s, np.exp(-rho * 2.0 / Lb * t), atol=3e-3)


def test_round_ellipsoid_is_the_sphere(cuda):
    """a = b = c = R walks the sphere: the two step rules agree on the ensemble signal."""
    R = 4e-6
    rng = np.random.default_rng(2)
    bv = rng.normal(size=(4, 3))
    bv /= np.linalg.norm(bv, axis=1, keepdims=True)
    wf = d.set_b(d.pgse(0.006, 0.02, 0.05, bv, 80), 1.5e9)
    s_e = d.simulate(200_000, D, wf, d.Ellipsoid([R, R, R]), seed=3)
    s_s = d.simulate(200_000, D, wf, d.Sphere(R), seed=3)
    np.testing.assert_allclose(s_e, s_s, atol=6e-3)
