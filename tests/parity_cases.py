"""Shared walk configurations of the GPU-vs-oracle parity tests."""
import numpy as np

import dmipy_sim_gb300 as d
from dmipy_sim_gb300 import core
from oracle import oracle as O

D = 2e-9


def waveform(n_dirs=4, n_t=100, b=1e9, delta=0.008, DELTA=0.03):
    rng = np.random.default_rng(0)
    bv = rng.normal(size=(n_dirs, 3))
    bv /= np.linalg.norm(bv, axis=1, keepdims=True)
    return d.set_b(d.pgse(delta, DELTA, 0.05, bv, n_t), b)


def packed_cylinders(**kw):
    rng = np.random.default_rng(1)
    radii = np.clip(rng.lognormal(np.log(1.5e-6), 0.25, 20), 0.8e-6, 3e-6)
    c, L, _ = d.pack_cylinders(radii, target_vf=0.5, seed=2)
    return d.PackedCylinders(radii, c, L, **kw)


def packed_spheres(**kw):
    sr = np.clip(np.random.default_rng(3).normal(1.5e-6, 0.2e-6, 12), 1e-6, 2e-6)
    c, L, _ = d.pack_spheres(sr, target_vf=0.25, seed=3)
    return d.PackedSpheres(sr, c, L, **kw)


def geometries():
    R = 5e-6
    return {
        "free": d.FreeDiffusion(),
        "cyl": d.Cylinder(R, (0, 0, 1)),
        "cyl_rho": d.Cylinder(R, (0, 0, 1), surface_relaxivity_t2=2e-5),
        "cyl_tilt": d.Cylinder(R, (1.0, 1.0, 0.3)),
        "cyl_kappa": d.Cylinder(R, (0, 0, 1), permeability=1e-5),
        "sph": d.Sphere(R),
        "sph_rho": d.Sphere(R, surface_relaxivity_t2=2e-5),
        "sph_kappa": d.Sphere(R, permeability=1e-5),
        "pcyl": packed_cylinders(),
        "pcyl_rho": packed_cylinders(surface_relaxivity_t2=2e-5),
        "pcyl_kappa": packed_cylinders(permeability=2e-5),
        "psph": packed_spheres(),
        "psph_rho": packed_spheres(surface_relaxivity_t2=2e-5),
        "psph_kappa": packed_spheres(permeability=2e-5),
    }


def plan(geom, wf, engine):
    """(sub_steps, phase_per_substep) as simulate() picks them."""
    gap = core._replay_gap(geom, return_positions=False, return_compartments=False,
                           return_walker_signals=False, diffusivity=D)
    use_replay = engine == "replay" or (engine == "auto" and gap is None)
    if use_replay:
        return core.replay_sub_steps(geom, D, wf.dt), False
    return core.fused_sub_steps(geom, D, wf.dt), True


def oracle_walk(geom, G, dt, S, phase_sub, n, seed, T2=None, echo_idx=None, fp64=False,
                walker_offset=0, want_walkers=True, r0=None, T1=None):
    if getattr(geom, "_is_packed_myelinated", False):
        wall = O.PERMEATE if (np.any(geom._kappa_inner > 0) or np.any(geom._kappa_outer > 0)) \
            else O.REFLECT
        return O.walk(O.geom_from(geom, dt / S), n_walkers=n, G=G, dt=dt, sub_steps=S,
                      phase_per_substep=phase_sub, seed=seed, wall=wall, T1=T1,
                      has_weight=geom._has_weight() or T1 is not None, step_length=1.0,
                      echo_idx=echo_idx, fp64=fp64, walker_offset=walker_offset,
                      want_walkers=want_walkers, r0=r0)
    if getattr(geom, "_is_myelinated", False):
        # unit steps, per-compartment T2 in the geometry, simulate's T2 unused
        wall = O.PERMEATE if (geom.kappa_inner is not None or geom.kappa_outer is not None) \
            else O.REFLECT
        return O.walk(O.geom_from(geom, dt / S), n_walkers=n, G=G, dt=dt, sub_steps=S,
                      phase_per_substep=phase_sub, seed=seed, wall=wall, T1=T1,
                      has_weight=geom._has_weight() or T1 is not None, step_length=1.0,
                      echo_idx=echo_idx, fp64=fp64, walker_offset=walker_offset,
                      want_walkers=want_walkers, r0=r0)
    rho = geom.surface_relaxivity_t2
    kappa = geom.permeability
    wall = O.PERMEATE if kappa is not None else (O.RELAX if rho is not None else O.REFLECT)
    return O.walk(O.geom_from(geom), n_walkers=n, G=G, dt=dt, sub_steps=S,
                  phase_per_substep=phase_sub, seed=seed, wall=wall, T2=T2,
                  rho_over_D=0.0 if rho is None else rho / D,
                  kappa_over_D=0.0 if kappa is None else kappa / D, D=D, echo_idx=echo_idx,
                  fp64=fp64, walker_offset=walker_offset, want_walkers=want_walkers, r0=r0)
