"""Generate the golden fixtures of the parity tests from the dmipy-sim reference itself.

Runs the reference's own ``waveforms.py``, ``geometries.py``, ``physics.py``, ``trajectories.py``
and ``core.py`` unmodified, under the numpy stand-in for JAX in ``jaxstub.py`` (JAX is not
installed where the fixtures are made), and writes:

  kat.npz  known-answer vectors: waveform constructors / calc_b / set_b, the sub-step rules, the
           RSA packers, every geometry plug-in call (reflect / reflect_with_log_weight / permeate)
           on seeded inputs with the Powles uniform injected, and the replay operator.
  mc.json  the reference's own Monte-Carlo signals (core.simulate / simulate_cpmg, numpy random
           numbers in place of threefry) on small configurations, with their standard errors,
           for the 3-standard-error statistical parity tests.

Usage:  python tests/golden/make_golden.py [--kat] [--mc] [--ref /path/to/dmipy-sim]
"""
import argparse
import json
import multiprocessing as mp
import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import jaxstub  # noqa: E402

D = 2e-9


def _ref(root):
    return jaxstub.load_reference(root)


# ------------------------------------------------------------------------------------------------
# Known-answer vectors
# ------------------------------------------------------------------------------------------------
def _unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _plugin_cases(m, rng, out):
    geo = m["geometries"]
    R = 5e-6
    n = 256

    def run(tag, g, mode, rs, steps, rho=0.0, kappa=0.0, us=None):
        ro = np.zeros((len(rs), 3), np.float64)
        dl = np.zeros(len(rs), np.float64)
        for i, (r, s) in enumerate(zip(rs, steps)):
            r32 = np.asarray(r, np.float32)
            s32 = np.asarray(s, np.float32)
            if mode == 0:
                o, d = g.reflect(r32, s32), 0.0
            elif mode == 1:
                o, d = g.reflect_with_log_weight(r32, s32, np.float32(rho))
            else:
                o, d = g.permeate(r32, s32, np.float32(kappa), np.float32(rho),
                                  jaxstub.Injected(us[i]))
            ro[i] = np.asarray(o, np.float64)
            dl[i] = float(d)
        out[f"pl_{tag}_r"] = np.asarray(rs, np.float32)
        out[f"pl_{tag}_step"] = np.asarray(steps, np.float32)
        out[f"pl_{tag}_out"] = ro
        out[f"pl_{tag}_dlog"] = dl
        out[f"pl_{tag}_mode"] = np.array(mode)
        out[f"pl_{tag}_rho"] = np.array(rho)
        out[f"pl_{tag}_kappa"] = np.array(kappa)
        if us is not None:
            out[f"pl_{tag}_u"] = np.asarray(us, np.float32)

    # single cylinder: identity and tilted frames
    for tag, ori in (("cyl", (0, 0, 1)), ("cyltilt", (1.0, 1.0, 0.3))):
        c = geo.Cylinder(R, ori)
        Rm = np.asarray(c._R, np.float64)
        rad = R * np.sqrt(rng.uniform(0.2, 0.9999, n))
        ang = rng.uniform(0, 2 * np.pi, n)
        rc = np.stack([rad * np.cos(ang), rad * np.sin(ang), rng.uniform(-R, R, n)], 1)
        rl = rc @ Rm                                   # lab = R^T r_c
        st = _unit(rng, n) * (R * rng.uniform(0.02, 1.5, n))[:, None]
        out[f"geo_{tag}_R"] = np.array(R)
        out[f"geo_{tag}_ori"] = np.array(ori, np.float64)
        run(tag + "_reflect", c, 0, rl, st)
        run(tag + "_relax", c, 1, rl, st, rho=500.0)
        cp = geo.Cylinder(R, ori, permeability=1e-5)
        rad2 = R * rng.uniform(0.6, 1.4, n)
        rc2 = np.stack([rad2 * np.cos(ang), rad2 * np.sin(ang), rng.uniform(-R, R, n)], 1)
        st2 = _unit(rng, n) * (R * rng.uniform(0.01, 0.5, n))[:, None]
        run(tag + "_perm", cp, 2, rc2 @ Rm, st2, rho=500.0, kappa=5000.0,
            us=rng.uniform(0, 1, n))
    # single sphere
    s = geo.Sphere(R)
    dirs = _unit(rng, n)
    rs = dirs * (R * rng.uniform(0.2, 0.9999, n) ** (1 / 3))[:, None]
    st = _unit(rng, n) * (R * rng.uniform(0.02, 1.5, n))[:, None]
    out["geo_sph_R"] = np.array(R)
    run("sph_reflect", s, 0, rs, st)
    run("sph_relax", s, 1, rs, st, rho=500.0)
    sp = geo.Sphere(R, permeability=1e-5)
    rs2 = dirs * (R * rng.uniform(0.6, 1.4, n))[:, None]
    st2 = _unit(rng, n) * (R * rng.uniform(0.01, 0.5, n))[:, None]
    run("sph_perm", sp, 2, rs2, st2, rho=500.0, kappa=5000.0, us=rng.uniform(0, 1, n))

    # packed cylinders / spheres (RSA), unfolded positions several boxes away
    radii = np.clip(rng.lognormal(np.log(2e-6), 0.25, 16), 0.9e-6, 3.5e-6)
    cen, L, vf = geo.pack_cylinders(radii, target_vf=0.45, seed=11)
    pc = geo.PackedCylinders(radii, cen, L)
    pts = []
    while len(pts) < n:
        p = rng.uniform(-L / 2, L / 2, 2)
        d = p - cen
        d -= L * np.round(d / L)
        if np.all(np.sum(d * d, 1) > (radii * 1.0001) ** 2):
            pts.append(p)
    pts = np.array(pts)
    # walkers start next to a wall half of the time
    k = rng.integers(0, len(radii), n)
    near = rng.uniform(size=n) < 0.5
    a2 = rng.uniform(0, 2 * np.pi, n)
    pn = cen[k] + (radii[k] * rng.uniform(1.0005, 1.2, n))[:, None] * np.stack(
        [np.cos(a2), np.sin(a2)], 1)
    pts = np.where(near[:, None], pn, pts)
    img = rng.integers(-3, 4, (n, 2)) * L
    rl = np.concatenate([pts + img, rng.uniform(-R, R, (n, 1))], 1)
    st = _unit(rng, n) * (radii.min() * rng.uniform(0.05, 0.6, n))[:, None]
    out["geo_pcyl_radii"] = radii
    out["geo_pcyl_centers"] = cen
    out["geo_pcyl_L"] = np.array(L)
    run("pcyl_reflect", pc, 0, rl, st)
    run("pcyl_relax", pc, 1, rl, st, rho=500.0)
    pcp = geo.PackedCylinders(radii, cen, L, permeability=2e-5)
    inside = rng.uniform(size=n) < 0.5
    pin = cen[k] + (radii[k] * rng.uniform(0.7, 0.9995, n))[:, None] * np.stack(
        [np.cos(a2), np.sin(a2)], 1)
    rl2 = np.concatenate([np.where(inside[:, None], pin, pts) + img, rl[:, 2:]], 1)
    run("pcyl_perm", pcp, 2, rl2, st, rho=500.0, kappa=10000.0, us=rng.uniform(0, 1, n))

    sr = np.clip(rng.lognormal(np.log(1.5e-6), 0.2, 12), 0.8e-6, 2.5e-6)
    scen, sL, svf = geo.pack_spheres(sr, target_vf=0.25, seed=5)
    ps = geo.PackedSpheres(sr, scen, sL)
    pts = []
    while len(pts) < n:
        p = rng.uniform(-sL / 2, sL / 2, 3)
        d = p - scen
        d -= sL * np.round(d / sL)
        if np.all(np.sum(d * d, 1) > (sr * 1.0001) ** 2):
            pts.append(p)
    pts = np.array(pts)
    k = rng.integers(0, len(sr), n)
    dd = _unit(rng, n)
    pn = scen[k] + (sr[k] * rng.uniform(1.0005, 1.2, n))[:, None] * dd
    near = rng.uniform(size=n) < 0.5
    pts = np.where(near[:, None], pn, pts)
    img = rng.integers(-3, 4, (n, 3)) * sL
    st = _unit(rng, n) * (sr.min() * rng.uniform(0.05, 0.6, n))[:, None]
    out["geo_psph_radii"] = sr
    out["geo_psph_centers"] = scen
    out["geo_psph_L"] = np.array(sL)
    run("psph_reflect", ps, 0, pts + img, st)
    run("psph_relax", ps, 1, pts + img, st, rho=500.0)
    psp = geo.PackedSpheres(sr, scen, sL, permeability=2e-5)
    pin = scen[k] + (sr[k] * rng.uniform(0.7, 0.9995, n))[:, None] * dd
    inside = rng.uniform(size=n) < 0.5
    run("psph_perm", psp, 2, np.where(inside[:, None], pin, pts) + img, st, rho=500.0,
        kappa=10000.0, us=rng.uniform(0, 1, n))


def _waveform_cases(m, out):
    wf = m["waveforms"]
    bv3 = [[1, 0, 0]] * 3
    w = wf.pgse(0.01, 0.04, 0.05, bv3, 300)
    w = wf.set_b(w, [0, 1e9, 2e9])
    out["wf_pgse_G"] = np.asarray(w.G)
    out["wf_pgse_dt"] = np.array(w.dt)
    out["wf_pgse_b"] = wf.calc_b(w)
    rng = np.random.default_rng(0)
    bv = rng.normal(size=(30, 3))
    bv /= np.linalg.norm(bv, axis=1, keepdims=True)
    w = wf.set_b(wf.pgse(0.01, 0.04, 0.05, bv, 300), 1e9)
    out["wf_pgse30_G"] = np.asarray(w.G)
    out["wf_pgse30_bvecs"] = bv
    w = wf.pgse(0.008, 0.03, 0.1, [[0, 1, 0], [0, 0, 1]], 101, slew_rate=np.inf)
    out["wf_square_G"] = np.asarray(w.G)
    out["wf_square_btensor"] = wf.calc_btensor(w)
    w = wf.pgste(0.005, 0.02, 0.08, [[1, 0, 0]], 121)
    out["wf_pgste_G"] = np.asarray(w.G)
    out["wf_pgste_chi"] = np.asarray(w.chi_perp, np.float32)
    out["wf_pgste_dt"] = np.array(w.dt)
    for f in (10.0, 50.0, 100.0):
        w = wf.ogse(f, 0.05, 0.06, [[1, 0, 0], [0.6, 0.8, 0]], 1000)
        out[f"wf_ogse{int(f)}_G"] = np.asarray(w.G)
    w = wf.cpmg(16, 5e-3, 0.02, [[1, 0, 0], [0, 0, 1]], n_t_per_echo=100)
    out["wf_cpmg_G"] = np.asarray(w.G)
    out["wf_cpmg_echo"] = np.asarray(w.echo_indices)
    out["wf_cpmg_dt"] = np.array(w.dt)


def _substep_cases(m, out):
    geo, ph, core = m["geometries"], m["physics"], m["core"]
    rows = []
    for R in (0.8e-6, 2e-6, 5e-6):
        for dt in (1.6722408e-4, 5.005e-5, 1e-3):
            s = geo.Sphere(R, permeability=1e-5)
            c = geo.Cylinder(R, (0, 0, 1), surface_relaxivity_t2=1e-6)
            rows.append([R, dt, ph.permeable_sub_steps(s, D, dt), ph.surface_sub_steps(c, D, dt)])
    out["sub_perm_surf"] = np.array(rows, np.float64)

    class _Grid:
        def __init__(self, cs):
            self.cell_size = cs
    rows = []
    for cs in (0.1e-6, 0.5e-6, 2e-6):
        for dt in (5e-5, 1.6722408e-4, 1e-3):
            rows.append([cs, dt, ph.collision_sub_steps(_Grid(cs), D, dt)])
    out["sub_collision"] = np.array(rows, np.float64)
    # the replay producer's rule, read back from simulate_trajectories itself on a tiny walk
    rows = []
    for name, g in (("cyl", geo.Cylinder(5e-6, (0, 0, 1))),
                    ("sphk", geo.Sphere(3e-6, permeability=1e-5)),
                    ("pcyl", geo.PackedCylinders([1.1e-6, 2e-6], [[-2e-6, -2e-6], [2.5e-6, 2.5e-6]],
                                                 9e-6))):
        for dt in (1.6722408e-4, 5e-5):
            out_ = core.simulate_trajectories(2, D, g, dt * 2, dt, seed=1, require_gpu=False)
            rows.append([dt, out_[2]])
        out[f"sub_replay_{name}"] = np.array(rows[-2:], np.float64)


def _pack_cases(m, out):
    geo = m["geometries"]
    rng = np.random.default_rng(7)
    radii = np.clip(rng.lognormal(np.log(2e-6), 0.25, 40), 0.8e-6, 4e-6)
    c, L, vf = geo.pack_cylinders(radii, target_vf=0.5, seed=3)
    out["pack_cyl_radii"], out["pack_cyl_centers"], out["pack_cyl_L"] = radii, c, np.array(L)
    sr = rng.uniform(1e-6, 2e-6, 25)
    c, L, vf = geo.pack_spheres(sr, target_vf=0.3, seed=4)
    out["pack_sph_radii"], out["pack_sph_centers"], out["pack_sph_L"] = sr, c, np.array(L)


def _replay_cases(m, out):
    tr, wf = m["trajectories"], m["waveforms"]
    rng = np.random.default_rng(3)
    n, n_t = 400, 121
    traj = np.cumsum(rng.normal(scale=0.3e-6, size=(n, n_t, 3)), axis=1).astype(np.float16)
    w = wf.set_b(wf.pgste(0.005, 0.02, 0.08, [[1, 0, 0], [0, 1, 0], [0.6, 0, 0.8]], n_t), 1e9)
    dlog = -np.abs(rng.normal(scale=1e-9, size=(n, n_t))).astype(np.float16)
    sig = tr.replay(traj, w.dt, np.asarray(w.G), w.dt, chi_perp=w.chi_perp,
                    dlog_boundary_unit=dlog, T2=0.08, T1=0.9, surface_relaxivity=1e-5, D=D,
                    stimulated_echo=True)
    out["rep_traj"], out["rep_G"], out["rep_chi"] = traj, np.asarray(w.G), np.asarray(
        w.chi_perp, np.float32)
    out["rep_dt"], out["rep_dlog"], out["rep_signal"] = np.array(w.dt), dlog, np.asarray(sig)
    sig2 = tr.replay(traj, w.dt, np.asarray(w.G), w.dt)
    out["rep_signal_plain"] = np.asarray(sig2)


def _mesh_cases(m, rng, out):
    """Mesh.reflect / reflect_with_log_weight / permeate of the reference on a closed icosphere
    and on a periodic box whose sphere crosses a face (ghost triangles)."""
    import importlib
    import warnings
    shapes = importlib.import_module("dmipy_sim.mesh_shapes")
    mesh_mod = importlib.import_module("dmipy_sim.mesh")
    R = 5e-6
    V, F = shapes.icosphere(R, 2)
    out["mesh_V"], out["mesh_F"] = np.asarray(V, np.float64), np.asarray(F, np.int64)
    n = 192
    cases = {}
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        cases["msh"] = (mesh_mod.Mesh(V, F), mesh_mod.Mesh(V, F, intra={"surface_relaxivity_t2": 1e-6}),
                        mesh_mod.Mesh(V, F, permeability=1e-5,
                                      intra={"surface_relaxivity_t2": 1e-6}), np.zeros(3), None)
        Vp = V * 0.6 + np.array([3.5e-6, 0.0, 0.0])
        kw = dict(periodic=True, voxel_min=[-5e-6] * 3, voxel_max=[5e-6] * 3, feature_radius=3e-6)
        cases["mshp"] = (mesh_mod.Mesh(Vp, F, **kw),
                         mesh_mod.Mesh(Vp, F, intra={"surface_relaxivity_t2": 1e-6}, **kw),
                         mesh_mod.Mesh(Vp, F, permeability=1e-5, **kw), np.array([3.5e-6, 0, 0]),
                         kw)
    out["mesh_Vp"] = np.asarray(V * 0.6 + np.array([3.5e-6, 0.0, 0.0]), np.float64)
    for tag, (g0, g1, g2, c0, kw) in cases.items():
        rr = (R if tag == "msh" else 0.6 * R)
        d = _unit(rng, n)
        rad = rr * rng.uniform(0.6, 1.3, n)
        rs = (c0 + d * rad[:, None]).astype(np.float32)
        if tag == "mshp":
            rs = rs + (rng.integers(-2, 3, (n, 3)) * 10e-6).astype(np.float32)
        st = (_unit(rng, n) * (rr * rng.uniform(0.02, 0.3, n))[:, None]).astype(np.float32)
        us = rng.uniform(0, 1, n).astype(np.float32)
        for mode, g in (("reflect", g0), ("relax", g1), ("perm", g2)):
            ro = np.zeros((n, 3))
            dl = np.zeros(n)
            for i in range(n):
                if mode == "reflect":
                    o, dd = g.reflect(rs[i], st[i]), 0.0
                elif mode == "relax":
                    o, dd = g.reflect_with_log_weight(rs[i], st[i], np.float32(500.0))
                else:
                    o, dd = g.permeate(rs[i], st[i], np.float32(5000.0), np.float32(500.0),
                                       jaxstub.Injected(us[i]))
                ro[i] = np.asarray(o, np.float64)
                dl[i] = float(dd)
            key = f"pl_{tag}_{mode}"
            out[key + "_r"], out[key + "_step"], out[key + "_out"] = rs, st, ro
            out[key + "_dlog"], out[key + "_u"] = dl, us


def _waveform_cases_tensor(m, out):
    """Trapezoidal OGSE, its closed-form b, spherical/planar tensor encodings and the b-tensor
    invariants (waveforms.py:353-720)."""
    w = m["waveforms"]
    t = w.trapezoidal_ogse(3, 0.02, 0.03, 0.05, [[1, 0, 0], [0, 0.6, 0.8]], 500)
    out["wf_trap_G"] = np.asarray(t.G, np.float32)
    out["wf_trap_dt"] = np.float64(t.dt)
    t1 = w.trapezoidal_ogse(1, 0.01, 0.03, 0.08, [[0, 1, 0]], 301, rise_time=5e-4)
    out["wf_trap1_G"] = np.asarray(t1.G, np.float32)
    out["wf_trap_bformula"] = np.array([w.b_trapezoidal_ogse(n, 0.02, 0.03, 0.05, 2.5e-4)
                                        for n in (1, 2, 3, 4)])
    s = w.ste(0.01, 0.03, 0.05, 300)
    out["wf_ste_G"] = np.asarray(s.G, np.float32)
    p = w.pte(0.01, 0.03, 0.05, [0.3, 0.4, 0.866], 301)
    out["wf_pte_G"] = np.asarray(p.G, np.float32)
    p2 = w.pte(0.01, 0.03, 0.05, [1.0, 0.1, 0.0], 200, slew_rate=np.inf)
    out["wf_pte2_G"] = np.asarray(p2.G, np.float32)
    B = np.concatenate([w.calc_btensor(s), w.calc_btensor(p), w.calc_btensor(t)])
    out["wf_inv_B"] = B
    out["wf_inv_b"], out["wf_inv_bdelta"], out["wf_inv_beta"] = (
        np.asarray(x) for x in w.btensor_invariants(B))


def _myelin_cases(m, rng, out):
    """make_myelin_step_fn (physics.py:420-680) of the reference, one step per case, with the
    direction and the two Powles uniforms the step drew recorded: a sheath thin enough that most
    cases cross a wall, every compartment, permeable and impermeable walls."""
    geo, phys = m["geometries"], m["physics"]
    rnd = sys.modules["jax.random"]
    drawn = {}
    real_normal, real_uniform = rnd.normal, rnd.uniform

    def normal(key, shape=(), dtype=np.float32):
        v = real_normal(key, shape, dtype)
        drawn["noise"] = np.asarray(v, np.float32)
        return v

    def uniform(key, shape=(), dtype=np.float32, minval=0.0, maxval=1.0):
        v = real_uniform(key, shape, dtype, minval, maxval)
        drawn.setdefault("u", []).append(np.float32(v))
        return v
    rnd.normal, rnd.uniform = normal, uniform
    try:
        n = 256
        dt = 1e-4
        # permeabilities high enough that about half the crossings transmit
        for tag, kw in (("perm", dict(kappa_inner=2e-3, kappa_outer=1e-3)), ("refl", {})):
            g = geo.MyelinatedCylinder(2e-6, 2.6e-6, (0, 0, 1), D_intra=2e-9, D_extra=2.5e-9,
                                       D_myelin=0.8e-9, T2_intra=0.08, T2_myelin=0.012,
                                       T2_extra=0.07, water_fractions=(1.0, 0.4, 1.0), **kw)
            step = phys.make_myelin_step_fn(g, dt, T1=0.9)
            ang = rng.uniform(0, 2 * np.pi, n)
            rad = rng.uniform(0.0, 3.4e-6, n)
            r = np.stack([rad * np.cos(ang), rad * np.sin(ang),
                          rng.uniform(-1e-6, 1e-6, n)], 1).astype(np.float32)
            comp = np.where(rad < 2e-6, 0, np.where(rad < 2.6e-6, 1, 2)).astype(np.int32)
            chi = (rng.uniform(size=n) < 0.7).astype(np.float32)
            ro, co, dl, units, us = [], [], [], [], []
            for i in range(n):
                drawn.clear()
                key = rnd.PRNGKey(1000 + i)
                carry = (r[i], np.zeros(1, np.float32), np.float32(0.0), np.int32(comp[i]), key)
                new, _ = step(carry, (np.zeros((1, 3), np.float32), np.float32(chi[i])))
                nz = drawn["noise"]
                units.append(nz / np.linalg.norm(nz))
                us.append(drawn["u"][:2])
                ro.append(np.asarray(new[0], np.float64))
                co.append(int(new[3]))
                dl.append(float(new[2]))
            key = f"my_{tag}"
            out[key + "_r"], out[key + "_comp"], out[key + "_chi"] = r, comp, chi
            out[key + "_unit"] = np.asarray(units, np.float32)
            out[key + "_u"] = np.asarray(us, np.float32)
            out[key + "_out"], out[key + "_comp_out"] = np.asarray(ro), np.asarray(co, np.int32)
            out[key + "_dlog"] = np.asarray(dl)
    finally:
        rnd.normal, rnd.uniform = real_normal, real_uniform


def pmyelin_substrate(geo, perm):
    """Five myelinated axons packed in a periodic cell (the same packing for the reference and
    this package: pack_myelinated_cylinders draws the same numbers)."""
    ri = np.array([1.0e-6, 1.3e-6, 0.8e-6, 1.1e-6, 0.9e-6])
    ri, g, c = geo.pack_myelinated_cylinders(ri, 0.7, 0.5, seed=4)
    L = float(np.sqrt(np.pi * np.sum((ri / g) ** 2) / 0.5))
    kw = dict(kappa_inner=2e-3, kappa_outer=1e-3) if perm else {}
    return geo.PackedMyelinatedCylinders(ri, g, c, L, N_max=8, D_intra=2e-9, D_myelin=0.5e-9,
                                         D_extra=2.5e-9, T2_intra=0.07, T2_myelin=0.015,
                                         T2_extra=0.06, **kw)


def _pmyelin_cases(m, rng, out):
    """make_packed_myelin_traj_step_fn (physics.py:682-976) of the reference, one sub-step per
    case with the direction and Powles uniforms it drew: walkers of every compartment anywhere in
    the cell (walls across the cell edge, extra-axonal walkers entering a sheath)."""
    geo, phys = m["geometries"], m["physics"]
    rnd = sys.modules["jax.random"]
    drawn = {}
    real_normal, real_uniform = rnd.normal, rnd.uniform

    def normal(key, shape=(), dtype=np.float32):
        v = real_normal(key, shape, dtype)
        drawn["noise"] = np.asarray(v, np.float32)
        return v

    def uniform(key, shape=(), dtype=np.float32, minval=0.0, maxval=1.0):
        v = real_uniform(key, shape, dtype, minval, maxval)
        drawn.setdefault("u", []).append(np.float32(v))
        return v
    rnd.normal, rnd.uniform = normal, uniform
    try:
        n = 384
        for tag, perm in (("perm", True), ("refl", False)):
            g = pmyelin_substrate(geo, perm)
            step = phys.make_packed_myelin_traj_step_fn(g, 1e-4)
            L = g._L_float
            r = np.concatenate([rng.uniform(-L / 2, L / 2, (n, 2)),
                                rng.uniform(-1e-6, 1e-6, (n, 1))], 1).astype(np.float32)
            comp = np.zeros(n, np.int32)
            for k in range(g.N_actual - 1, -1, -1):
                q = r[:, :2] - g._centers_np[k].astype(np.float32)
                q = q - np.float32(L) * np.floor(q / np.float32(L) + np.float32(0.5))
                d2 = np.sum(q * q, 1)
                comp = np.where(d2 < np.float32(g._outer_radii_np[k]) ** 2, g.N_max + 1 + k, comp)
            for k in range(g.N_actual - 1, -1, -1):
                q = r[:, :2] - g._centers_np[k].astype(np.float32)
                q = q - np.float32(L) * np.floor(q / np.float32(L) + np.float32(0.5))
                d2 = np.sum(q * q, 1)
                comp = np.where(d2 < np.float32(g._inner_radii_np[k]) ** 2, 1 + k, comp)
            ro, co, dl, units, us = [], [], [], [], []
            for i in range(n):
                drawn.clear()
                new, _ = step((r[i], rnd.PRNGKey(5000 + i), np.float32(0.0), np.int32(comp[i])),
                              None)
                nz = drawn["noise"]
                units.append(nz / np.linalg.norm(nz))
                us.append(drawn["u"][:2])
                ro.append(np.asarray(new[0], np.float64))
                dl.append(float(new[2]))
                co.append(int(new[3]))
            key = f"pmy_{tag}"
            out[key + "_r"], out[key + "_comp"] = r, comp
            out[key + "_unit"] = np.asarray(units, np.float32)
            out[key + "_u"] = np.asarray(us, np.float32)
            out[key + "_out"], out[key + "_comp_out"] = np.asarray(ro), np.asarray(co, np.int32)
            out[key + "_dlog"] = np.asarray(dl)
    finally:
        rnd.normal, rnd.uniform = real_normal, real_uniform


def _validation_geom_cases(m, rng, out):
    """Box1D, PermeableSlab1D and PermeableShell (sphere and cylinder) plug-in calls of the
    reference (geometries.py:48-140, 3221-3431): reflect, reflect_with_log_weight where defined,
    permeate with recorded uniforms."""
    geo = m["geometries"]
    n = 256
    L = 6e-6
    rho, kappa = 500.0, 5000.0

    def run(tag, g, mode, rs, st, us):
        ro = np.zeros((n, 3))
        dl = np.zeros(n)
        for i in range(n):
            if mode == "reflect":
                o, dd = g.reflect(rs[i], st[i]), 0.0
            elif mode == "relax":
                o, dd = g.reflect_with_log_weight(rs[i], st[i], np.float32(rho))
            else:
                o, dd = g.permeate(rs[i], st[i], np.float32(kappa), np.float32(rho),
                                   jaxstub.Injected(us[i]))
            ro[i] = np.asarray(o, np.float64)
            dl[i] = float(dd)
        key = f"pl_{tag}_{mode}"
        out[key + "_r"], out[key + "_step"], out[key + "_u"] = rs, st, us
        out[key + "_out"], out[key + "_dlog"] = ro, dl

    us = rng.uniform(0, 1, n).astype(np.float32)
    # slabs: x spread over the slab and a little beyond each wall's reach, steps up to 0.4 L
    rs = np.stack([rng.uniform(0, L, n), rng.normal(0, 1e-6, n), rng.normal(0, 1e-6, n)],
                  1).astype(np.float32)
    st = (_unit(rng, n) * rng.uniform(0.02, 0.4, (n, 1)) * L).astype(np.float32)
    box = geo.Box1D(L)
    run("box", box, "reflect", rs, st, us)
    run("box", box, "relax", rs, st, us)
    slab = geo.PermeableSlab1D(L, permeability=1e-5)
    for mode in ("reflect", "relax", "perm"):
        run("slab", slab, mode, rs, st, us)
    ell = geo.Ellipsoid([2e-6, 3e-6, 4.5e-6])
    d = _unit(rng, n)
    rs = (d * rng.uniform(0.3, 1.15, (n, 1)) * np.array([2e-6, 3e-6, 4.5e-6])).astype(np.float32)
    st = (_unit(rng, n) * rng.uniform(0.05, 0.5, (n, 1)) * 2e-6).astype(np.float32)
    run("ell", ell, "reflect", rs, st, us)
    run("ell", ell, "relax", rs, st, us)
    run("ell", geo.Ellipsoid([2e-6, 3e-6, 4.5e-6], permeability=1e-5), "perm", rs, st, us)
    for kind, tag in (("sphere", "shs"), ("cylinder", "shc")):
        sh = geo.PermeableShell(2e-6, 4e-6, permeability=1e-5, kind=kind)
        d = _unit(rng, n)
        rad = rng.uniform(0.2, 1.0, n) * 4e-6
        rs = (d * rad[:, None]).astype(np.float32)
        if kind == "cylinder":
            rs[:, 2] = rng.uniform(-3e-6, 3e-6, n)
        st = (_unit(rng, n) * rng.uniform(0.05, 0.6, (n, 1)) * 2e-6).astype(np.float32)
        run(tag, sh, "reflect", rs, st, us)
        run(tag, sh, "perm", rs, st, us)


def make_myelin_kat(root):
    """Add the myelinated-cylinder step known answers to kat.npz."""
    m = _ref(root)
    path = HERE / "kat.npz"
    out = {k: v for k, v in np.load(path).items()
           if not k.startswith(("my_", "pmy_", "pl_box_", "pl_slab_", "pl_shs_", "pl_shc_",
                                "pl_ell_"))}
    _myelin_cases(m, np.random.default_rng(17), out)
    _pmyelin_cases(m, np.random.default_rng(23), out)
    _validation_geom_cases(m, np.random.default_rng(29), out)
    np.savez_compressed(path, **out)
    print(f"kat.npz: {len(out)} arrays")


def make_replay_kat(root):
    """Known answers of the reference's compression.py / replay.py codecs and mode-space replay
    and of trajectories.replay on a compressed master, on a seeded synthetic walk
    (replay_kat.npz)."""
    import importlib
    m = _ref(root)
    cx = importlib.import_module("dmipy_sim.compression")
    rp = importlib.import_module("dmipy_sim.replay")
    wfm, tr = m["waveforms"], m["trajectories"]
    rng = np.random.default_rng(11)
    n_w, n_t, dt = 200, 100, 2.5e-4
    X = np.cumsum(rng.normal(scale=0.25e-6, size=(n_w, n_t, 3)), axis=1)
    out = {"traj": X, "dt": np.float64(dt)}
    a, mm, nb = cx.encode_temporal_dct(X, 16)
    for k, v in a.items():
        out[f"tdct_{k}"] = v
    out["tdct_decoded"] = cx.decode(a, mm).astype(np.float32)
    a, mm, nb = cx.encode_lowrank(X, 8)
    out["lowrank_decoded"] = cx.decode(a, mm).astype(np.float32)
    # boundary local time: spiky, mostly zero, <= 0
    dlog = -np.abs(rng.normal(scale=1e-7, size=(n_w, n_t))) * (rng.uniform(size=(n_w, n_t)) < 0.1)
    out["blt_raw"] = dlog
    a, mm = cx.encode_boundary_dct(dlog, K=8)
    out["blt_dct_coeffs"], out["blt_endpoint"] = a["blt_dct_coeffs"], a["blt_endpoint"]
    out["blt_dct_decoded"] = cx.decode_boundary_dct(a, mm)
    a, mm = cx.encode_boundary_local_time(dlog)
    out["blt_sparse_mode"] = np.array(mm["mode"] == "sparse")
    for k, v in a.items():
        out[f"bltq_{k}"] = v
    out["bltq_decoded"] = cx.decode_boundary_local_time(a, mm)
    dense = -np.abs(rng.normal(scale=1e-7, size=(40, n_t)))
    a, mm = cx.encode_boundary_local_time(dense)
    out["bltd_raw"] = dense
    out["bltd_q"], out["bltd_decoded"] = a["blt_dense_q"], cx.decode_boundary_local_time(a, mm)
    comp = (rng.uniform(size=(n_w, 1)) < 0.4).astype(np.int32) * np.ones((1, n_t), np.int32)
    comp[:50, 60:] = 2
    a, mm = cx.encode_compartment(comp)
    for k, v in a.items():
        out[f"comp_{k}"] = v
    fr = np.clip(np.cumsum(rng.normal(scale=0.05, size=(30, n_t)), axis=1) * 0.3 + 0.5, 0, 1)
    a, mm = cx.encode_compartment(fr)
    out["compf_decoded"] = cx.decode_compartment(a, mm)
    a, mm = cx.encode_bound_fraction(fr)
    out["bfrac_decoded"] = cx.decode_bound_fraction(a, mm)
    out["comp_frac"] = fr
    out["comp_int"] = comp
    out["relax_lw"] = cx.relaxation_logweight(comp.clip(0, 1), [0.06, 0.08], [0.9, 1.2], dt,
                                              chi=(np.arange(n_t) < 80).astype(float))
    out["relax_lw_frac"] = cx.relaxation_logweight(fr, [0.06, 0.08], [0.9, 1.2], dt)
    out["surf_lw"] = cx.surface_logweight(dlog, 500.0, chi=(np.arange(n_t) % 3 == 0).astype(float))
    # acquisition battery, mode-space replay and fidelity
    env = cx.default_envelope()
    G, meta = cx.acquisition_battery(n_t, dt, env)
    out["battery_G"] = G
    out["battery_b"] = np.array([q["b"] for q in meta])
    out["battery_Gpeak"] = np.array([q["Gpeak"] for q in meta])
    out["battery_fam"] = np.array([q["fam"] for q in meta])
    a16, m16, _ = cx.encode_temporal_dct(X, 16)
    out["ms_phi"] = cx.mode_space_phi(a16, m16, G[:12], dt)
    lw = -np.abs(rng.normal(scale=0.05, size=n_w))
    w = rng.uniform(0.5, 1.5, n_w)
    out["ms_logw"], out["ms_w"] = lw, w
    out["ms_signal"] = cx.mode_space_signal(a16, m16, G[:12], dt, logw=lw, weights=w)
    a8, m8, _ = cx.encode_temporal_dct(X, 8)
    fid = cx.measure_fidelity(X, dt, cx.decode(a8, m8), env)
    out["fid_err_max"], out["fid_floor_max"] = fid["err_max"], fid["floor_max"]
    out["fid_fams"] = np.array(sorted(fid["per_family"]))
    out["fid_fam_err"] = np.array([fid["per_family"][f]["err_max"] for f in out["fid_fams"]])
    out["fid_fam_floor"] = np.array([fid["per_family"][f]["floor_max"]
                                     for f in out["fid_fams"]])
    Kbest, fbest = cx.auto_select_modes(X, X, dt, env=env, K_grid=(4, 8, 16, 32))
    out["auto_K"] = np.array(Kbest)
    # compiled-scheme forward of a pack with spin weights and boundary bands
    W = rp.compile_scheme(G[:12], dt, 16)
    out["scheme_W"] = W
    blt_pack = rng.normal(scale=1e-8, size=(n_w, 6))
    pack = dict(a16, spin_weights=w.astype(np.float32), blt_dct=blt_pack)
    out["pack_blt_dct"] = blt_pack
    out["rs_plain"] = rp.replay_signal(dict(a16), W)
    out["rs_complex"] = rp.replay_signal(pack, W, complex_signal=True)
    out["rs_surface"] = rp.replay_signal(rp.ReplayPack(pack, {"n_t": n_t}), W, rho_over_D=500.0)
    chi_hat = rng.normal(size=4)
    out["rs_chi_hat"] = chi_hat
    out["rs_gated"] = rp.replay_signal(rp.ReplayPack(pack, {"n_t": n_t}), W, rho_over_D=500.0,
                                       chi_hat=chi_hat)
    # trajectories.replay on a compressed master (mode space, no reconstruction)
    C = cx.read_position_coeffs(a16, dtype=np.float32)
    ab, _ = cx.encode_boundary_dct(dlog, K=16)
    master = {"compressed": True, "method": "temporal_dct", "K": 16, "n_t": n_t, "dt_traj": dt,
              "pos_modes": C, "blt_endpoint": ab["blt_endpoint"],
              "blt_modes": ab["blt_dct_coeffs"], "comp_traj": comp.clip(0, 1)}
    out["master_blt_modes"], out["master_blt_endpoint"] = ab["blt_dct_coeffs"], ab["blt_endpoint"]
    w1 = wfm.set_b(wfm.pgse(0.006, 0.015, 0.1, [[1, 0, 0], [0, 0.6, 0.8]], 61), [1e9, 2e9])
    out["rc_G"], out["rc_dt"] = np.asarray(w1.G), np.float64(w1.dt)
    out["rc_plain"] = np.asarray(tr.replay(master, None, np.asarray(w1.G), w1.dt))
    out["rc_relax"] = np.asarray(tr.replay(master, None, np.asarray(w1.G), w1.dt, T2=0.07,
                                           T1=0.9, surface_relaxivity=1e-5, D=2e-9))
    w2 = wfm.pgste(0.005, 0.012, 0.02, [[1, 0, 0]], 101)
    out["rc2_G"], out["rc2_dt"] = np.asarray(w2.G), np.float64(w2.dt)
    out["rc2_chi"] = np.asarray(w2.chi_perp, np.float64)
    out["rc_gated"] = np.asarray(tr.replay(master, None, np.asarray(w2.G), w2.dt,
                                           chi_perp=w2.chi_perp, T2_per_comp=[0.05, 0.08],
                                           T1_per_comp=[0.8, 1.1], surface_relaxivity=2e-5, D=2e-9,
                                           stimulated_echo=True))
    path = HERE / "replay_kat.npz"
    np.savez_compressed(path, **out)
    print(f"replay_kat.npz: {len(out)} arrays")


def make_kat_extra(root):
    """Add the tensor-encoding waveform vectors to an existing kat.npz."""
    m = _ref(root)
    path = HERE / "kat.npz"
    out = dict(np.load(path))
    _waveform_cases_tensor(m, out)
    np.savez_compressed(path, **out)
    print(f"kat.npz: {len(out)} arrays")


def make_kat(root):
    m = _ref(root)
    out = {}
    rng = np.random.default_rng(2024)
    _waveform_cases(m, out)
    _waveform_cases_tensor(m, out)
    _substep_cases(m, out)
    _pack_cases(m, out)
    _replay_cases(m, out)
    _plugin_cases(m, rng, out)
    _mesh_cases(m, np.random.default_rng(77), out)
    np.savez_compressed(HERE / "kat.npz", **out)
    print(f"kat.npz: {len(out)} arrays")


# ------------------------------------------------------------------------------------------------
# Reference Monte-Carlo signals (statistical fixtures)
# ------------------------------------------------------------------------------------------------
def _mc_configs():
    """name -> (kind, kwargs).  Small enough for the reference's per-walker Python walk."""
    return {
        "free_pgse": dict(geom=("free",), wf=("pgse3",), n=8000, api="simulate"),
        "free_pgse_fused": dict(geom=("free",), wf=("pgse3",), n=6000, api="simulate",
                                engine="fused"),
        "cyl_rho": dict(geom=("cyl", 5e-6, 1e-6, None), wf=("pgse6",), n=3200, api="simulate"),
        "cyl_rho_fused": dict(geom=("cyl", 5e-6, 1e-6, None), wf=("pgse6",), n=1600,
                              api="simulate", engine="fused"),
        "sph_kappa": dict(geom=("sph", 5e-6, None, 1e-5), wf=("pgse_short",), n=960,
                          api="simulate"),
        "cyl_kappa": dict(geom=("cyl", 5e-6, None, 1e-5), wf=("pgse_short",), n=960,
                          api="simulate"),
        "sph_t2": dict(geom=("sph", 5e-6, None, None), wf=("pgse6",), n=4000, api="simulate",
                       T2=0.06),
        "lattice_fused": dict(geom=("lattice", 0.6), wf=("pgse_lat",), n=6400, api="simulate",
                              engine="fused"),
        "rsa_fused": dict(geom=("rsa",), wf=("pgse_lat",), n=4000, api="simulate",
                          engine="fused"),
        "psph_fused": dict(geom=("psph",), wf=("pgse_lat",), n=4000, api="simulate",
                           engine="fused"),
        "cpmg_sph": dict(geom=("sph", 5e-6, None, None), wf=("cpmg",), n=4000, api="cpmg",
                         T2=0.06),
        "cpmg_free": dict(geom=("free",), wf=("cpmg_g",), n=4000, api="cpmg", T2=0.08),
        # a closed icosphere mesh (4 um, 320 triangles); walkers start uniformly inside it from
        # explicit positions (mesh_r0), since the reference seeds meshes through trimesh
        "mesh_reflect": dict(geom=("mesh", None), wf=("pgse_mesh",), n=1600, api="simulate",
                             r0="mesh"),
        "mesh_perm": dict(geom=("mesh", 1e-5), wf=("pgse_mesh",), n=640, api="simulate",
                          r0="mesh"),
        # the myelinated cylinder's own step rule, one step per sample, diffusivity None
        "myelin_refl": dict(geom=("myelin", None, None, 0.0), wf=("pgse_my",), n=8000,
                            api="simulate", D=None),
        "myelin_perm": dict(geom=("myelin", 5e-5, 3e-5, 0.5e-9), wf=("pgse_my",), n=8000,
                            api="simulate", D=None),
        "pmyelin_refl": dict(geom=("pmyelin", False), wf=("pgse_my",), n=8000, api="simulate",
                             D=None),
        "pmyelin_perm": dict(geom=("pmyelin", True), wf=("pgse_my",), n=8000, api="simulate",
                             D=None),
    }


def mesh_surface():
    """The closed icosphere of the mesh fixtures (vertices, faces), from this package."""
    sys.path.insert(0, str(HERE.parent.parent))
    from dmipy_sim_gb300.mesh import icosphere
    return icosphere(4e-6, 2)


def mesh_r0(n, seed):
    """n positions uniform inside the fixture mesh (rejection by ray-crossing parity)."""
    sys.path.insert(0, str(HERE.parent.parent))
    from dmipy_sim_gb300.mesh import mesh_contains
    V, F = mesh_surface()
    rng = np.random.default_rng(int(seed))
    out = []
    while sum(len(o) for o in out) < n:
        p = rng.uniform(-4e-6, 4e-6, size=(2 * n, 3))
        out.append(p[mesh_contains(V, F, p)])
    return np.concatenate(out)[:n].astype(np.float32)


def build_waveform(wfm, spec):
    name = spec[0]
    if name == "pgse3":
        return wfm.set_b(wfm.pgse(0.01, 0.04, 0.05, [[1, 0, 0]] * 3, 300), [0, 1e9, 2e9])
    rng = np.random.default_rng(0)
    bv = rng.normal(size=(6, 3))
    bv /= np.linalg.norm(bv, axis=1, keepdims=True)
    if name == "pgse6":
        return wfm.set_b(wfm.pgse(0.01, 0.04, 0.05, bv, 300), 1e9)
    if name == "pgse_short":
        return wfm.set_b(wfm.pgse(0.003, 0.008, 0.2, bv[:4], 60), 1e9)
    if name == "pgse_lat":
        return wfm.set_b(wfm.pgse(0.005, 0.02, 0.1, [[1, 0, 0], [0, 1, 0], [0, 0, 1],
                                                     [0.6, 0.8, 0]], 200), 1.5e9)
    if name == "cpmg":
        return wfm.cpmg(8, 12e-3, 0.0, [[1, 0, 0]], n_t_per_echo=60)
    if name == "cpmg_g":
        return wfm.cpmg(6, 10e-3, 0.02, [[1, 0, 0], [0, 0, 1]], n_t_per_echo=50)
    if name == "pgse_my":
        return wfm.set_b(wfm.pgse(0.006, 0.02, 0.1, [[1, 0, 0], [0, 0, 1], [0.6, 0.8, 0]], 120),
                         [5e8, 1e9, 2e9])
    if name == "pgse_mesh":
        return wfm.set_b(wfm.pgse(0.003, 0.008, 0.2, [[1, 0, 0], [0, 0, 1], [0.6, 0.8, 0]], 60),
                         [5e8, 1e9, 2e9])
    raise KeyError(name)


def build_geometry(geo, spec):
    kind = spec[0]
    if kind == "free":
        return geo.FreeDiffusion()
    if kind == "cyl":
        return geo.Cylinder(spec[1], (0, 0, 1), surface_relaxivity_t2=spec[2], permeability=spec[3])
    if kind == "sph":
        return geo.Sphere(spec[1], surface_relaxivity_t2=spec[2], permeability=spec[3])
    if kind == "lattice":
        a = 4e-6
        r = a * np.sqrt(spec[1] / np.pi)
        cen = np.array([[(i + 0.5) * a - a, (j + 0.5) * a - a] for i in range(2) for j in range(2)])
        return geo.PackedCylinders(np.full(4, r), cen, 2 * a)
    if kind == "rsa":
        rng = np.random.default_rng(1)
        radii = np.clip(rng.lognormal(np.log(1.5e-6), 0.25, 20), 0.8e-6, 3e-6)
        cen, L, _ = geo.pack_cylinders(radii, target_vf=0.45, seed=2)
        return geo.PackedCylinders(radii, cen, L)
    if kind == "psph":
        sr = np.full(10, 1.5e-6)
        cen, L, _ = geo.pack_spheres(sr, target_vf=0.25, seed=3)
        return geo.PackedSpheres(sr, cen, L)
    if kind == "mesh":
        V, F = mesh_surface()
        return geo.Mesh(V, F, permeability=spec[1])
    if kind == "pmyelin":
        return pmyelin_substrate(geo, spec[1])
    if kind == "myelin":
        # an axon of 2 um in a 0.8 um sheath, T2 per compartment, myelin water density 0.4
        return geo.MyelinatedCylinder(2e-6, 2.8e-6, (0.2, 0.3, 1.0), D_intra=2e-9, D_extra=2.2e-9,
                                      D_myelin=spec[3], kappa_inner=spec[1], kappa_outer=spec[2],
                                      T2_intra=0.07, T2_myelin=0.015, T2_extra=0.06,
                                      water_fractions=(1.0, 0.4, 1.0))
    raise KeyError(kind)


def _mc_worker(args):
    root, name, cfg, seed, n = args
    m = _ref(root)
    import contextlib
    import io
    wf = build_waveform(m["waveforms"], cfg["wf"])
    if cfg["geom"][0] == "mesh":
        import importlib
        g = build_geometry(importlib.import_module("dmipy_sim.mesh"), cfg["geom"])
    else:
        g = build_geometry(m["geometries"], cfg["geom"])
    r0 = mesh_r0(n, seed) if cfg.get("r0") == "mesh" else None
    with contextlib.redirect_stdout(io.StringIO()):
        if cfg["api"] == "cpmg":
            s = m["core"].simulate_cpmg(n, D, wf, g, T2=cfg.get("T2"), seed=seed,
                                        require_gpu=False)
        else:
            s = m["core"].simulate(n, cfg.get("D", D), wf, g, seed=seed, T2=cfg.get("T2"),
                                   require_gpu=False, engine=cfg.get("engine", "auto"), r0=r0)
    return name, n, np.asarray(s, np.float64)


def make_mc(root, procs, only=None):
    cfgs = _mc_configs()
    jobs = []
    for name, cfg in cfgs.items():
        if only and name not in only:
            continue
        per = cfg["n"] // procs
        for k in range(procs):
            jobs.append((root, name, cfg, 1000 + 17 * k, per))
    t0 = time.time()
    res = {}
    with mp.get_context("spawn").Pool(procs) as pool:
        for name, n, s in pool.imap_unordered(_mc_worker, jobs):
            res.setdefault(name, []).append((n, s))
            print(f"  {name}: chunk of {n} done ({time.time() - t0:.0f}s)", flush=True)
    path = HERE / "mc.json"
    out = json.loads(path.read_text()) if path.exists() else {}
    for name, chunks in res.items():
        arr = np.stack([s for _, s in chunks])                 # (procs, ...)
        ns = np.array([n for n, _ in chunks], float)
        mean = np.tensordot(ns, arr, axes=1) / ns.sum()
        # standard error from the spread of the independent chunks
        se = np.sqrt(np.sum(ns[:, None] * (arr.reshape(len(ns), -1) - mean.reshape(1, -1)) ** 2,
                            axis=0) / ns.sum() / (len(ns) - 1)).reshape(mean.shape)
        out[name] = dict(config=_jsonable(cfgs[name]), n_walkers=int(ns.sum()),
                         chunks=len(ns), signal=mean.tolist(), stderr=se.tolist())
    path.write_text(json.dumps(out, indent=1))
    print(f"mc.json: {sorted(out)}")


def _bloch_worker(args):
    root, name, seed, n = args
    m = _ref(root)
    import importlib
    sys.path.insert(0, str(HERE.parent))
    import bloch_cases as bc
    ps = importlib.import_module("dmipy_sim.pulse_sequence")
    case = bc.CASES[name]
    seq = bc.sequence(ps, case["seq"])
    g = bc.geometry(m["geometries"], case["geom"])
    out = ps.run_bloch_sequence(seq, n, bc.D, g, seed=seed, require_gpu=False, **case["kw"])
    return name, n, bc.flatten(out, case["kw"].get("return_mz", False))


def make_mc_bloch(root, procs, only=None):
    """mc_bloch.json: dmipy-sim's own simulate_bloch on the scenarios of bloch_cases.py, mean and
    standard error over independent chunks (Re S, Im S, and Mz where returned)."""
    sys.path.insert(0, str(HERE.parent))
    import bloch_cases as bc
    jobs = []
    for name, case in bc.CASES.items():
        if only and name not in only:
            continue
        per = max(1, case["n"] // procs)
        for k in range(procs):
            jobs.append((root, name, 3000 + 29 * k, per))
    t0 = time.time()
    res = {}
    with mp.get_context("spawn").Pool(procs) as pool:
        for name, n, s in pool.imap_unordered(_bloch_worker, jobs):
            res.setdefault(name, []).append((n, s))
            print(f"  {name}: chunk of {n} done ({time.time() - t0:.0f}s)", flush=True)
    path = HERE / "mc_bloch.json"
    out = json.loads(path.read_text()) if path.exists() else {}
    for name, chunks in res.items():
        arr = np.stack([s for _, s in chunks])
        ns = np.array([n for n, _ in chunks], float)
        mean = np.tensordot(ns, arr, axes=1) / ns.sum()
        se = np.sqrt(np.sum(ns[:, None] * (arr - mean[None]) ** 2, axis=0) / ns.sum()
                     / (len(ns) - 1))
        out[name] = dict(n_walkers=int(ns.sum()), chunks=len(ns), value=mean.tolist(),
                         stderr=se.tolist())
    path.write_text(json.dumps(out, indent=1))
    print(f"mc_bloch.json: {sorted(out)}")


def make_bloch_kat(root):
    """bloch_kat.npz: dmipy-sim's own RF rasterisation, crusher schedule and sequence builders
    (bloch.py:60-89, 208-225; pulse_sequence.py:47-213) on fixed inputs."""
    m = _ref(root)
    import importlib
    b = importlib.import_module("dmipy_sim.bloch")
    ps = importlib.import_module("dmipy_sim.pulse_sequence")
    out = {}
    events = [
        [{'t_s': 0.0, 'flip_deg': 90.0, 'axis_deg': 90.0}],
        [{'t_s': 0.0, 'flip_deg': 90.0}, {'t_s': 2.05e-3, 'flip_deg': 180.0, 'axis_deg': 0.0,
                                           'duration_s': 1e-3, 'offset_hz': 120.0}],
        [{'t_s': 1e-3, 'flip_deg': 45.0, 'axis_deg': 30.0, 'duration_s': 2.4e-3,
          'offset_hz': -80.0}, {'t_s': 9.99e-3, 'flip_deg': 33.0, 'duration_s': 5e-4}],
    ]
    for i, ev in enumerate(events):
        fl, ax, ca = b._build_rf_schedule(ev, 1e-4, 100)
        out[f"rf{i}_flip"], out[f"rf{i}_axis"], out[f"rf{i}_carrier"] = fl, ax, ca
    for i, cr in enumerate([None, {'windows_s': [(1e-3, 3e-3)], 'n_cycles': 8.0},
                            {'windows_s': [(-1e-3, 2e-3), (8e-3, 20e-3)]}]):
        rate, has = b._build_crusher(cr, 1e-4, 100)
        out[f"crush{i}_rate"], out[f"crush{i}_has"] = rate, np.array(has)
    seqs = {
        "gre": ps.gradient_echo(5e-3, 1e-4, n_meas=2),
        "se": ps.spin_echo(6e-3, 1e-4, exc_axis_deg=45.0),
        "fexi": ps.fexi(2e-3, 5e-3, 1e-4, g_filter=0.2, g_detect=[0.0, 0.1, 0.2], Delta=4e-3,
                        direction=(1.0, 1.0, 0.0), crush_cycles=16.0),
        "fexi2": ps.fexi(2e-3, 3e-3, 2e-4, g_filter=0.1, g_detect=0.05),
        "mt": ps.prepend_mt_prep(ps.spin_echo(6e-3, 1e-4),
                                 {'offset_hz': 2000.0, 'duration_s': 3e-3, 'b1_hz': 100.0}),
        "mt2": ps.prepend_mt_prep(
            ps.BlochSequence(G=np.zeros((1, 30, 3)), dt=1e-4, rf_events=[
                {'t_s': 0.0, 'flip_deg': 90.0}], echo_steps=[10, 29]),
            {'offset_hz': -500.0, 'duration_s': 1e-3, 'flip_deg': 400.0, 'spoiler_s': 0.0}),
    }
    for k, q in seqs.items():
        out[f"seq_{k}_G"] = np.asarray(q.G)
        out[f"seq_{k}_dt"] = np.float64(q.dt)
        out[f"seq_{k}_rf"] = np.array(json.dumps(q.rf_events))
        out[f"seq_{k}_echo"] = np.array(json.dumps(q.echo_steps))
        out[f"seq_{k}_crusher"] = np.array(json.dumps(q.crusher))
        out[f"seq_{k}_meta"] = np.array(json.dumps([q.complex_signal, q.family]))
        if hasattr(q, "b_detect"):
            out[f"seq_{k}_b_detect"] = np.asarray(q.b_detect)
    np.savez_compressed(HERE / "bloch_kat.npz", **out)
    print(f"bloch_kat.npz: {len(out)} arrays")


def replay_bloch_inputs():
    """The seeded walk and per-step inputs of the replay_bloch known answers (also rebuilt by
    the tests): 96 walkers x 150 samples in a 4 um cylinder, two compartments."""
    rng = np.random.default_rng(21)
    n_w, n_t, dt = 96, 150, 1e-4
    r = np.zeros((n_w, n_t, 3))
    r[:, 0, :2] = rng.uniform(-2e-6, 2e-6, (n_w, 2))
    for t in range(1, n_t):
        r[:, t] = r[:, t - 1] + rng.normal(0, 0.6e-6, (n_w, 3))
        rad = np.linalg.norm(r[:, t, :2], axis=1)
        out = rad > 4e-6
        r[out, t, :2] *= (8e-6 / rad[out] - 1.0)[:, None]
    traj = r.astype(np.float32)
    comp = (np.linalg.norm(traj[..., :2], axis=-1) > 2.5e-6).astype(np.int64)
    G = np.zeros((3, 301, 3))
    G[0, 20:80, 0] = G[0, 160:220, 0] = 0.06
    G[1, 20:80, 1] = G[1, 160:220, 1] = 0.06
    G[2, 30:250, 2] = 0.02 * np.sin(np.linspace(0, 6 * np.pi, 220))
    rf = [{'t_s': 0.0, 'flip_deg': 90.0, 'axis_deg': 90.0},
          {'t_s': 7.5e-3, 'flip_deg': 180.0, 'axis_deg': 0.0, 'duration_s': 8e-4,
           'offset_hz': 250.0},
          {'t_s': 11e-3, 'flip_deg': 60.0, 'axis_deg': 30.0, 'duration_s': 1.2e-3,
           'b1_envelope': [0.2, 1.0, 0.6, 0.1]}]
    dlog = -np.abs(rng.normal(0, 2e-8, (n_w, n_t))).astype(np.float32)
    dlog[rng.random((n_w, n_t)) < 0.7] = 0.0
    bf = np.clip(rng.random((n_w, n_t)) * 1.5 - 0.7, 0.0, 1.0).astype(np.float32)
    xph = rng.normal(0, 0.02, (n_w, n_t))
    wts = rng.uniform(0.5, 1.5, n_w)
    b1s = rng.uniform(0.85, 1.1, n_w)
    sl = rng.uniform(-1e-3, 1e-3, n_w)
    return dict(traj=traj, dt_traj=dt, G=G, dt_wf=0.5e-4, rf=rf, comp=comp, dlog=dlog, bf=bf,
                xph=xph, wts=wts, b1s=b1s, slice=sl)


def replay_bloch_cases(x):
    """name -> keyword arguments of the replay_bloch known answers."""
    return {
        "plain": dict(T2=0.07),
        "relax": dict(T2=0.07, T1=0.9, echo_steps=[40, 75, 149, 75]),
        "comp": dict(comp_traj=x["comp"], T2_per_comp=[0.06, 0.09], T1_per_comp=[0.8, 1.2],
                     dlog_boundary_unit=x["dlog"], surface_relaxivity=3e-5, D=2e-9,
                     weights=x["wts"]),
        "mt": dict(T2=0.07, T1=1.0, bound_frac=x["bf"], T2_bound=1e-4, T1_bound=0.6,
                   off_resonance_bound=-600.0, echo_steps=[60, 120], echo_per_walker=True),
        "susc": dict(T2=0.08, extra_phase_per_step=x["xph"], b1_scale=x["b1s"],
                     slice_offsets=x["slice"], slice_gradient=0.01, return_walker_signals=True),
    }


def make_replay_bloch_kat(root):
    """replay_bloch_kat.npz: dmipy-sim's own trajectories.replay_bloch (numpy, FP64) on the
    seeded walk of replay_bloch_inputs(), one case per option group."""
    m = _ref(root)
    x = replay_bloch_inputs()
    out = {}
    for name, kw in replay_bloch_cases(x).items():
        res = m["trajectories"].replay_bloch(x["traj"], x["dt_traj"], x["G"], x["dt_wf"],
                                             x["rf"], **kw)
        if isinstance(res, tuple):
            out[f"{name}_mlast"] = np.asarray(res[0])
            res = res[1]
        out[name] = np.asarray(res)
    tr = m["trajectories"]
    out["sign_se"] = tr.pathway_sign_se(37, 1e-4, 2.2e-3, te_frac=0.45)
    rng = np.random.default_rng(8)
    walk = np.cumsum(rng.normal(0, 0.7e-6, (5, 60, 3)), axis=1)
    out["wrapped"] = (walk - 6e-6 * np.floor(walk / 6e-6 + 0.5)).astype(np.float32)
    out["unwrapped"] = tr.unwrap_periodic(out["wrapped"], 6e-6)
    out["unwrapped_xyz"] = tr.unwrap_periodic(out["wrapped"], 6e-6, periodic_axes=(0, 1, 2))
    out["dwell180"] = tr.finite_180_longitudinal_dwell(np.linspace(-3, 3, 11), 2e-3, 0.3)
    out["phi_pre"] = tr.pre_pulse_gradient_phase(x["traj"], x["dt_traj"], x["G"], x["dt_wf"], 150)
    np.savez_compressed(HERE / "replay_bloch_kat.npz", **out)
    print(f"replay_bloch_kat.npz: {sorted(out)}")


def rf_pulses(rf):
    """The pulses of the RF known answers, from an rf module (the reference's or this
    package's, same constructors)."""
    return {
        "hard": rf.B1Pulse.hard(90.0, 1e-3, 1e-5, phase_deg=30.0),
        "sinc": rf.B1Pulse.windowed_sinc(90.0, 2e-3, 1e-5, time_bw=6.0),
        "sinc_rect": rf.B1Pulse.windowed_sinc(30.0, 1.5e-3, 1e-5, n_zeros=2, window=None),
        "hs": rf.B1Pulse.adiabatic_hs(8e-3, 1e-5, peak_b1=15e-6),
        "ahp": rf.B1Pulse.adiabatic_half_passage(4e-3, 1e-5, peak_b1=12e-6),
        "bir4": rf.B1Pulse.bir4(60.0, 8e-3, 1e-5, peak_b1=15e-6),
        "comp": rf.B1Pulse.composite([(90, 0), (180, 90), (90, 0)], 1e-5, peak_b1=10e-6),
        "samples": rf.B1Pulse.from_magnitude_phase(np.linspace(0, 5e-6, 50),
                                                   np.linspace(0, 1, 50), 2e-5),
    }


def make_rf_kat(root):
    """rf_kat.npz: dmipy-sim's own RF pulse constructors and Bloch integrator (rf.py)."""
    _ref(root)
    import importlib
    rf = importlib.import_module("dmipy_sim.rf")
    out = {}
    df = np.linspace(-2000.0, 2000.0, 9)
    for k, p in rf_pulses(rf).items():
        out[f"{k}_b1"] = p.b1
        out[f"{k}_props"] = np.array([p.duration, p.peak_b1, p.b1_rms, p.sar_proxy,
                                      p.nominal_flip_deg, p.max_slew_b1])
        mxy, mz = rf.bloch_simulate(p, df_hz=df, b1_scale=np.linspace(0.8, 1.2, 9), T1=0.9,
                                    T2=0.05)
        out[f"{k}_mxy"], out[f"{k}_mz"] = mxy, mz
    p = rf_pulses(rf)["hard"]
    mxy, mz, hist = rf.bloch_simulate(p, df_hz=[0.0, 300.0], M0=[0.0, 1.0, 0.0],
                                      return_history=True)
    out["hist"], out["hist_mxy"], out["hist_mz"] = hist, mxy, mz
    z, mxy, mz = rf.slice_profile(rf_pulses(rf)["sinc"], 0.01, np.linspace(-5e-3, 5e-3, 21))
    out["slice_mxy"], out["slice_mz"] = mxy, mz
    np.savez_compressed(HERE / "rf_kat.npz", **out)
    print(f"rf_kat.npz: {len(out)} arrays")


def susceptibility_inputs():
    """Sources, sample points and a small chi grid of the susceptibility known answers."""
    rng = np.random.default_rng(31)
    return dict(
        sph_c=rng.uniform(-6e-6, 6e-6, (7, 3)), sph_a=rng.uniform(0.5e-6, 1.5e-6, 7),
        sph_chi=rng.uniform(-1e-6, 2e-6, 7),
        my_c=np.array([[-2e-6, -2e-6], [2e-6, 1.5e-6], [1.8e-6, -2.2e-6]]),
        my_a=np.array([0.9e-6, 0.7e-6, 0.8e-6]), my_b=np.array([1.3e-6, 1.1e-6, 1.2e-6]),
        pts=rng.uniform(-5e-6, 5e-6, (64, 3)),
        mask=(rng.random((12, 10, 8)) > 0.6).astype(float), rad=rng.normal(size=(12, 10, 8, 3)),
        grid=rng.normal(size=(9, 7, 6)))


def make_susceptibility_kat(root):
    """susceptibility_kat.npz: dmipy-sim's own susceptibility fields (susceptibility.py)."""
    _ref(root)
    import importlib
    su = importlib.import_module("dmipy_sim.susceptibility")
    x = susceptibility_inputs()
    out = {}
    f = su.SusceptibilitySources(x["sph_c"], x["sph_a"], x["sph_chi"], B0=3.0).delta_bz_fn()
    out["sph"] = np.array([float(f(p)) for p in x["pts"]])
    for k, (th, al, per) in enumerate(((0.7, 0.3, True), (np.pi / 2, 1.1, True),
                                       (1.2, 0.0, False))):
        g = su.MyelinSusceptibility(x["my_c"], x["my_a"], x["my_b"], 8e-6, delta_chi_a=-0.1e-6,
                                    B0=3.0, theta=th, alpha=al, periodic=per).delta_bz_fn()
        out[f"my{k}"] = np.array([float(g(p)) for p in x["pts"]])
    chi6 = su.myelin_susceptibility_tensor(x["mask"], x["rad"], chi_iso=-0.05e-6,
                                           chi_aniso=-0.1e-6)
    out["chi6"] = chi6
    out["dB"] = su.dipole_field(chi6, [0.2e-6, 0.25e-6, 0.3e-6], [0.3, 0.2, 1.0], B0=3.0)
    sdf = np.linalg.norm(np.stack(np.meshgrid(*[np.arange(n) - n / 2 for n in (12, 10, 8)],
                                              indexing="ij"), -1), axis=-1) - 3.0
    out["radial"] = su.radial_from_sdf(sdf, 0.2e-6)
    org = np.array([-1e-6, -0.5e-6, 0.2e-6])
    q = np.random.default_rng(5).uniform(-2e-6, 3e-6, (50, 3))
    out["samp_clamp"] = su.sample_grid(x["grid"], q, org, 0.4e-6, periodic=False)
    out["samp_wrap"] = su.sample_grid(x["grid"], q, org, 0.4e-6, periodic=True)
    out["samp_q"] = q
    np.savez_compressed(HERE / "susceptibility_kat.npz", **out)
    print(f"susceptibility_kat.npz: {sorted(out)}")


def make_mt_kat(root):
    """mt_kat.npz: dmipy-sim's own two-pool Bloch-McConnell model and binding bookkeeping
    (mt.py) on fixed inputs."""
    m = _ref(root)
    import importlib
    mt = importlib.import_module("dmipy_sim.mt")
    out = {}
    out["gen"] = mt.two_pool_generator(R1a=1.1, R2a=12.5, R1b=0.9, R2b=1e5, k_f=40.0, k_r=80.0,
                                       dw_a=300.0, dw_b=-50.0, w1=700.0, rf_phase=0.4)
    out["gen_m0b"] = mt.two_pool_generator(R1a=1.0, R2a=10.0, R1b=1.0, R2b=1e4, k_f=30.0,
                                           k_r=100.0, M0a=0.8, M0b=0.1)
    t = np.array([0.0, 1e-3, 5e-3, 0.02, 0.08])
    out["bmt"] = mt.bloch_mcconnell_transverse(t, T2a=80e-3, T2b=1e-5, k_f=30.0, k_r=100.0)
    out["bmt_dw"] = mt.bloch_mcconnell_transverse(t, T2a=60e-3, T2b=2e-3, k_f=20.0, k_r=50.0,
                                                  dw_a=100.0, dw_b=400.0, T1a=0.9, T1b=0.5)
    out["bml"] = mt.bloch_mcconnell_longitudinal(t * 10, T1a=1.0, T1b=0.7, k_f=30.0, k_r=90.0)
    out["bml_sat"] = mt.bloch_mcconnell_longitudinal(t * 10, T1a=1.2, T1b=1.0, k_f=30.0,
                                                     k_r=90.0, Mza0=1.0, Mzb0=0.0)
    off = np.array([-5000.0, -500.0, 0.0, 200.0, 2000.0, 20000.0])
    kw = dict(w1_hz=200.0, t_sat=0.025, T1a=1.0, T2a=80e-3, T1b=1.0, T2b=1e-5, k_f=40.0,
              k_r=80.0)
    out["z_a"] = mt.mt_z_spectrum(off, **kw)
    out["z_b"] = mt.mt_z_spectrum(off, read_pool="b", **kw)
    out["misc"] = np.array([
        mt.forward_rate(2e-6, 3e5), mt.backward_rate(0.0125), mt.bound_fraction(2e-6, 0.0125, 3e5),
        mt.kappa_MT_from_forward_rate(40.0, 1.5e6), mt.dwell_time_from_fraction(0.3, 40.0)])
    out["stick"] = mt.stick_probability(np.array([0.0, 1e-9, 1e-8, 1e-6]), 2e-5, 2e-9)
    geo, phys = m["geometries"], m["physics"]
    out["mt_sub"] = np.array([
        phys.mt_sub_steps(geo.Sphere(2e-6), 2e-9, 2e-5, 1.0 / 80.0),
        phys.mt_sub_steps(geo.Sphere(5e-6), 1e-9, 1e-3, 0.01),
        phys.mt_sub_steps(geo.Cylinder(3e-6, (0, 0, 1)), 2e-9, 1e-4, 1e-5),
        phys.mt_sub_steps(geo.Box1D(4e-6), 2e-9, 1e-4, 0.02),
        phys.mt_sub_steps(geo.Box1D(4e-6), 2e-9, 1e-4, 0.0)])
    np.savez_compressed(HERE / "mt_kat.npz", **out)
    print(f"mt_kat.npz: {len(out)} arrays")


def _jsonable(cfg):
    return {k: (list(v) if isinstance(v, tuple) else v) for k, v in cfg.items()}


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("DMIPY_SIM_SRC", "/root/reference"))
    ap.add_argument("--kat", action="store_true")
    ap.add_argument("--kat-extra", action="store_true",
                    help="add the tensor-encoding waveform vectors to an existing kat.npz")
    ap.add_argument("--myelin-kat", action="store_true",
                    help="add the myelinated-cylinder step vectors to an existing kat.npz")
    ap.add_argument("--replay-kat", action="store_true",
                    help="write replay_kat.npz (compression / replay-pack known answers)")
    ap.add_argument("--mc", action="store_true")
    ap.add_argument("--susceptibility-kat", action="store_true",
                    help="write susceptibility_kat.npz (field providers, dipole solver)")
    ap.add_argument("--rf-kat", action="store_true",
                    help="write rf_kat.npz (RF pulse constructors, Bloch integrator)")
    ap.add_argument("--replay-bloch-kat", action="store_true",
                    help="write replay_bloch_kat.npz (the Bloch replay on a stored walk)")
    ap.add_argument("--mt-kat", action="store_true",
                    help="write mt_kat.npz (the two-pool model and binding bookkeeping)")
    ap.add_argument("--mc-bloch", action="store_true",
                    help="write mc_bloch.json (the reference's simulate_bloch on bloch_cases.py)")
    ap.add_argument("--bloch-kat", action="store_true",
                    help="write bloch_kat.npz (RF schedule, crusher, sequence builders)")
    ap.add_argument("--only", nargs="*")
    ap.add_argument("--procs", type=int, default=os.cpu_count() or 4)
    a = ap.parse_args()
    if a.kat:
        make_kat(a.ref)
    if a.kat_extra:
        make_kat_extra(a.ref)
    if a.replay_kat:
        make_replay_kat(a.ref)
    if a.myelin_kat:
        make_myelin_kat(a.ref)
    if a.mc:
        make_mc(a.ref, a.procs, a.only)
    if a.susceptibility_kat:
        make_susceptibility_kat(a.ref)
    if a.rf_kat:
        make_rf_kat(a.ref)
    if a.replay_bloch_kat:
        make_replay_bloch_kat(a.ref)
    if a.mt_kat:
        make_mt_kat(a.ref)
    if a.mc_bloch:
        make_mc_bloch(a.ref, a.procs, a.only)
    if a.bloch_kat:
        make_bloch_kat(a.ref)
