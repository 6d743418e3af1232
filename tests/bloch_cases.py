"""Vector-Bloch scenarios shared by the fixture generator (run there against dmipy-sim's own
bloch.simulate_bloch / pulse_sequence builders) and the GPU tests (run against this package).
Each scenario builds its sequence with the pulse_sequence module it is given, so the two sides
differ only in the engine (and in the sequence builders, which the known-answer tests pin)."""
import numpy as np

D = 2e-9

# name -> geometry spec, sequence, walkers for the reference run, simulate_bloch keywords
CASES = {
    # diffusion-weighted spin echo (physical same-sign lobes, the 180 refocuses) across and
    # along a reflecting cylinder, with surface relaxivity on the Bloch walk
    "bloch_se_cyl": dict(geom=("cyl", 4e-6, None), seq="se_dw", n=2000,
                         kw=dict(T2=0.08, T1=1.0, surface_relaxivity=2e-5)),
    # a 180 train refocusing a static off-resonance under a constant gradient in a sphere
    "bloch_cpmg_sph": dict(geom=("sph", 4e-6, None), seq="cpmg", n=2000,
                           kw=dict(T2=0.06, off_resonance_hz=30.0)),
    # filter-exchange stimulated echo: three 90s, longitudinal storage, voxel crusher
    "bloch_fexi_sph": dict(geom=("sph", 5e-6, None), seq="fexi", n=2000, kw=dict(T2=0.08, T1=0.8)),
    # a finite off-resonant tilted pulse, no gradient: every walker carries the same M
    "bloch_finite_free": dict(geom=("free",), seq="finite", n=16,
                              kw=dict(T2=0.05, T1=0.3, off_resonance_hz=40.0, return_mz=True)),
    # spin echo in a square lattice of reflecting cylinders (packed single-reflection rule)
    "bloch_se_pcyl": dict(geom=("lattice", 0.6), seq="se_dw", n=2000, kw=dict(T2=0.08)),
    # magnetisation transfer: a gradient echo from the equilibrium bound occupancy ('fast'
    # start), and an off-resonance CW saturation from an all-free start; few explicit sub-steps
    # keep the reference's per-walker walk tractable
    "bloch_mt_gre_fast": dict(geom=("sph", 2e-6, None), seq="gre3", n=1600, kw=dict(
        T2=0.08, T1=1.0, kappa_MT=40.0 * 2e-6 / 3.0, dwell_time=1.0 / 80.0, T2_bound=1e-5,
        T1_bound=1.0, sub_steps=4, equilibrate_binding='fast', return_mz=True,
        return_bound_frac=True)),
    "bloch_mt_sat_off": dict(geom=("sph", 2e-6, None), seq="cw_sat", n=800, kw=dict(
        T2=0.08, T1=1.0, kappa_MT=40.0 * 2e-6 / 3.0, dwell_time=1.0 / 80.0, T2_bound=1e-5,
        T1_bound=1.0, sub_steps=3, equilibrate_binding='off', return_mz=True)),
}


def sequence(ps, name):
    """The scenario's BlochSequence, built with the pulse_sequence module ``ps``."""
    if name == "se_dw":
        TE, dt, g, delta = 20e-3, 1e-4, 0.1, 4e-3
        dirs = np.array([[1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
        seq = ps.spin_echo(TE, dt, n_meas=2)
        nd = int(round(delta / dt))
        i1 = int(round(2e-3 / dt))
        i2 = int(round((TE / 2 + 1e-3) / dt))
        for m in range(2):
            seq.G[m, i1:i1 + nd] = g * dirs[m]
            seq.G[m, i2:i2 + nd] = g * dirs[m]
        return seq
    if name == "cpmg":
        dt, TE, n_echo = 1e-4, 8e-3, 4
        n_t = n_echo * int(round(TE / dt)) + 1
        G = np.zeros((2, n_t, 3))
        G[0, :, 0] = 0.02
        rf = [{'t_s': 0.0, 'flip_deg': 90.0, 'axis_deg': 90.0}] + [
            {'t_s': (2 * k + 1) * TE / 2, 'flip_deg': 180.0, 'axis_deg': 0.0}
            for k in range(n_echo)]
        echo = [int(round((k + 1) * TE / dt)) for k in range(n_echo)]
        return ps.BlochSequence(G=G, dt=dt, rf_events=rf, echo_steps=echo, family="cpmg")
    if name == "fexi":
        return ps.fexi(3e-3, 6e-3, 1e-4, g_filter=0.15, g_detect=[0.0, 0.15], Delta=6e-3)
    if name == "gre3":
        return ps.gradient_echo(3e-3, 1e-4)
    if name == "cw_sat":
        dt, t_sat = 5e-5, 5e-3
        rf = [{'t_s': t_sat / 2, 'flip_deg': 360.0 * 200.0 * t_sat, 'axis_deg': 0.0,
               'duration_s': t_sat, 'offset_hz': 1000.0}]
        return ps.BlochSequence(G=np.zeros((1, int(round(t_sat / dt)) + 1, 3)), dt=dt,
                                rf_events=rf, family="cw")
    if name == "finite":
        dt, n_t = 1e-4, 100
        rf = [{'t_s': 1e-3, 'flip_deg': 90.0, 'axis_deg': 30.0, 'duration_s': 2e-3,
               'offset_hz': 150.0},
              {'t_s': 6e-3, 'flip_deg': 120.0, 'axis_deg': 100.0, 'duration_s': 0.0}]
        return ps.BlochSequence(G=np.zeros((1, n_t, 3)), dt=dt, rf_events=rf, family="finite")
    raise KeyError(name)


def geometry(geo, spec):
    """The scenario's geometry from the geometry module ``geo`` (same constructors)."""
    kind = spec[0]
    if kind == "free":
        return geo.FreeDiffusion()
    if kind == "cyl":
        return geo.Cylinder(spec[1], (0, 0, 1), permeability=spec[2])
    if kind == "sph":
        return geo.Sphere(spec[1], permeability=spec[2])
    if kind == "lattice":
        a = 4e-6
        r = a * np.sqrt(spec[1] / np.pi)
        cen = np.array([[(i + 0.5) * a - a, (j + 0.5) * a - a] for i in range(2) for j in range(2)])
        return geo.PackedCylinders(np.full(4, r), cen, 2 * a)
    raise KeyError(kind)


def flatten(out, return_mz=False):
    """simulate_bloch's return as one real vector: Re S, Im S, then whatever follows (the final
    Mz, the bound-fraction series)."""
    items = list(out) if isinstance(out, tuple) else [out]
    s = np.asarray(items[0])
    parts = [s.real.ravel(), s.imag.ravel()]
    parts += [np.asarray(x, np.float64).ravel() for x in items[1:]]
    return np.concatenate(parts).astype(np.float64)
