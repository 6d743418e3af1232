"""The vector-Bloch walk on the GPU (dmsim_bloch through simulate_bloch).

  * the closed forms dmipy-sim pins its own engine with (tests/test_bloch_forward.py,
    tests/test_bloch_permeation.py there): T2 decay, inversion recovery, off-resonance
    precession, PGSE parity with the scalar walk on the identical walk, emergent CPMG
    refocusing, permeability raising the attenuation toward free diffusion;
  * the CPU oracle's eager restatement on the same walk (same draws, steps, sub-steps): the
    ensemble sums of Mx, My, Mz, across reflecting, relaxing, permeable and packed walls, finite
    pulses, carriers, the crusher, echo trains and more measurements than one pass holds;
  * dmipy-sim's own simulate_bloch results (tests/golden/mc_bloch.json) within 4 standard errors.
"""
import json
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

import dmipy_sim_gb300 as d
from dmipy_sim_gb300 import bloch as B
from dmipy_sim_gb300 import pulse_sequence as ps
from oracle import oracle as O
import bloch_cases as bc

pytestmark = pytest.mark.gpu
D = 2e-9
EXC_Y = [{'t_s': 0.0, 'flip_deg': 90.0, 'axis_deg': 90.0}]


def _zero(n_t, dt, n_meas=1):
    return SimpleNamespace(G=np.zeros((n_meas, n_t, 3)), dt=dt)


# ---- closed forms (dmipy-sim tests/test_bloch_forward.py) -----------------------------------
def test_transverse_decays_at_T2(cuda):
    n_t, dt, T2 = 200, 2e-4, 0.05
    s = d.simulate_bloch(2000, D, _zero(n_t, dt), d.FreeDiffusion(), EXC_Y, T2=T2, seed=0)
    assert abs(s[0]) == pytest.approx(np.exp(-n_t * dt / T2), rel=1e-4)
    assert abs(np.angle(s[0])) < 1e-5


def test_inversion_recovery_T1(cuda):
    n_t, dt, T1 = 300, 5e-4, 0.8
    _, mz = d.simulate_bloch(2000, D, _zero(n_t, dt), d.FreeDiffusion(),
                             [{'t_s': 0.0, 'flip_deg': 180.0, 'axis_deg': 0.0}], T1=T1, M0=1.0,
                             seed=0, return_mz=True)
    assert mz[0] == pytest.approx(1.0 - 2.0 * np.exp(-n_t * dt / T1), abs=1e-4)


def test_off_resonance_precession(cuda):
    n_t, dt, f = 200, 1e-5, 200.0
    s = d.simulate_bloch(2000, D, _zero(n_t, dt), d.FreeDiffusion(), EXC_Y, off_resonance_hz=f,
                         seed=0)
    assert abs(s[0]) == pytest.approx(1.0, rel=1e-5)
    assert np.angle(s[0]) == pytest.approx(2.0 * np.pi * f * n_t * dt, rel=1e-4)


def test_pgse_parity_with_scalar_engine(cuda):
    """Same seed, same walk, same phase: Re S of the Bloch walk is simulate()'s signal to FP32
    rounding, and exp(-bD) within the sampling error."""
    b = 1.0e9
    wf = d.set_b(d.pgse(0.01, 0.03, 0.05, [[1., 0., 0.]], 300), b)
    N = 16000
    scalar = d.simulate(N, D, wf, d.FreeDiffusion(), seed=7)
    vec = d.simulate_bloch(N, D, wf, d.FreeDiffusion(), EXC_Y, seed=7)
    assert np.real(vec[0]) == pytest.approx(float(scalar[0]), abs=2e-5)
    assert np.real(vec[0]) == pytest.approx(np.exp(-b * D), abs=0.02)


def test_cpmg_refocuses_static_offset(cuda):
    dt, TE, n_echo, T2, f = 1e-4, 4e-3, 4, 0.06, 100.0
    n_t = n_echo * int(round(TE / dt)) + 1
    echo = [int(round((k + 1) * TE / dt)) for k in range(n_echo)]
    refocus = [{'t_s': (2 * k + 1) * (TE / 2), 'flip_deg': 180.0, 'axis_deg': 0.0}
               for k in range(n_echo)]
    ec = d.simulate_bloch(4000, D, _zero(n_t, dt), d.FreeDiffusion(), EXC_Y + refocus, T2=T2,
                          off_resonance_hz=f, seed=0, echo_steps=echo)[0]
    for k in range(n_echo):
        # an echo is read after its sample's relaxation: samples 0 .. echo[k] each decay
        assert abs(ec[k]) == pytest.approx(np.exp(-(echo[k] + 1) * dt / T2), rel=1e-4)
        assert abs(np.angle(ec[k])) < 0.15
    free = d.simulate_bloch(4000, D, _zero(n_t, dt), d.FreeDiffusion(), EXC_Y, T2=T2,
                            off_resonance_hz=f, seed=0, echo_steps=echo)[0]
    assert abs(np.angle(free[-1])) > 1.0


# ---- permeability (dmipy-sim tests/test_bloch_permeation.py) --------------------------------
def _dw_spin_echo(g=0.20, TE=30e-3, dt=1e-4, delta=5e-3):
    seq = ps.spin_echo(TE, dt)
    nd = int(round(delta / dt))
    i1, i2 = int(round(4e-3 / dt)), int(round((TE / 2 + 1e-3) / dt))
    seq.G[0, i1:i1 + nd, 0] = g
    seq.G[0, i2:i2 + nd, 0] = g
    return seq


def _S(kappa, seq, n=20000, seed=0):
    geom = d.Cylinder(3e-6, (0, 0, 1), permeability=None if kappa == 0 else kappa)
    return abs(complex(d.run_bloch_sequence(seq, n, D, geom, seed=seed)[0]))


def test_permeability_increases_attenuation_monotonically(cuda):
    seq = _dw_spin_echo()
    S = [_S(k, seq) for k in (0.0, 3e-5, 3e-3)]
    assert S[0] > S[1] > S[2]
    assert S[0] - S[2] > 0.1


def test_high_permeability_approaches_free_diffusion(cuda):
    seq = _dw_spin_echo()
    s_free = abs(complex(d.run_bloch_sequence(seq, 20000, D, d.FreeDiffusion(), seed=0)[0]))
    assert abs(_S(1e-2, seq) - s_free) < 0.12


def test_walk_is_deterministic(cuda):
    seq = _dw_spin_echo()
    assert _S(0.0, seq, seed=7) == _S(0.0, seq, seed=7)


# ---- the oracle's eager restatement on the same walk ------------------------------------------
def _cases():
    rng = np.random.default_rng(4)
    dirs = rng.normal(size=(20, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    Gm = np.zeros((20, 100, 3))
    Gm[:, 10:40] = 0.08 * dirs[:, None, :]
    Gm[:, 60:90] = -0.08 * dirs[:, None, :]
    lat = bc.geometry(d, ("lattice", 0.6))
    return {
        "free_pgse": (d.FreeDiffusion(), d.set_b(d.pgse(0.01, 0.03, 0.05, [[1, 0, 0], [0, 1, 0]],
                                                        300), [1e9, 2e9]),
                      EXC_Y, dict(T2=0.05), 4096),
        "cyl_se_rho": (d.Cylinder(4e-6, (0, 0, 1)), bc.sequence(ps, "se_dw"), None,
                       dict(T2=0.08, T1=1.0, surface_relaxivity=2e-5), 4096),
        "sph_perm_offres": (d.Sphere(4e-6, permeability=2e-5), bc.sequence(ps, "se_dw"), None,
                            dict(T2=0.08, T1=0.7, off_resonance_hz=50.0, echo_steps=[100, 200],
                                 return_mz=True, surface_relaxivity=1e-5), 1024),
        "pcyl_fexi": (lat, bc.sequence(ps, "fexi"), None, dict(T2=0.08, T1=0.8), 4096),
        "ell_finite": (d.Ellipsoid([2e-6, 3e-6, 4.5e-6]), bc.sequence(ps, "finite"), None,
                       dict(T2=0.05, T1=0.3, off_resonance_hz=40.0, return_mz=True), 2048),
        "sph_20_meas": (d.Sphere(5e-6), SimpleNamespace(G=Gm, dt=1e-4),
                        [{'t_s': 0.0, 'flip_deg': 90.0, 'axis_deg': 90.0},
                         {'t_s': 5e-3, 'flip_deg': 180.0}], dict(T2=0.06), 2048),
    }


@pytest.mark.parametrize("name", ["free_pgse", "cyl_se_rho", "sph_perm_offres", "pcyl_fexi",
                                  "ell_finite", "sph_20_meas"])
def test_matches_oracle_on_the_same_walk(cuda, name):
    g, wf, rf, kw, n = _cases()[name]
    if isinstance(wf, ps.BlochSequence):
        rf, kw = wf.rf_events, dict(kw, echo_steps=kw.get("echo_steps", wf.echo_steps),
                                    crusher=wf.crusher)
        wf = SimpleNamespace(G=np.asarray(wf.G), dt=float(wf.dt))
    r0 = None
    if isinstance(g, d.Ellipsoid):
        r0 = g.init_positions(n, 11)
    kw = dict(kw, seed=5)
    w, uniq, idx = B._prepare(n, D, wf, g, rf, r0=r0, want_positions=True,
                              **{k: kw.get(k, dflt) for k, dflt in (
                                  ("T2", None), ("T1", None), ("M0", 1.0),
                                  ("off_resonance_hz", 0.0), ("seed", 0), ("echo_steps", None),
                                  ("return_mz", False), ("crusher", None),
                                  ("surface_relaxivity", 0.0))})
    w.launch()
    sums = w.result()
    assert np.all(np.isfinite(w.pos.cpu().numpy()))
    G, _ = B._waveform_arrays(wf, g)
    fl, ax, ca = B._build_rf_schedule(rf, wf.dt, G.shape[1])
    car = ca + 2.0 * np.pi * kw.get("off_resonance_hz", 0.0) * wf.dt
    rate, has = B._build_crusher(kw.get("crusher"), wf.dt, G.shape[1])
    og = O.geom_from(g)
    ora = O.bloch(og, n_walkers=n, G=G, dt=wf.dt, sub_steps=w.sub_steps, seed=5,
                  rf_flip=fl, rf_axis=ax, carrier=car if np.any(car) else None,
                  crush=rate if has else None, wall=int(w.gdesc.wall_mode), T2=kw.get("T2"),
                  T1=kw.get("T1"), rho_over_D=float(w.gdesc.rho_over_D),
                  kappa_over_D=float(w.gdesc.kappa_over_D), D=D, echo_idx=uniq, r0=r0)
    # walker by walker the two agree to FP32 rounding until a reflecting walk, a chaotic
    # billiard, parts between the device's arithmetic and the oracle's; such walkers (each
    # worth at most 2 / n) bound the difference of the means
    diff = np.abs(sums - ora) / n
    assert diff.max() < 0.02, (name, diff.max())
    assert np.median(diff) < 2e-3, (name, np.median(diff))


# ---- dmipy-sim's own simulate_bloch (statistical) -----------------------------------------
@pytest.fixture(scope="module")
def mc_bloch():
    return json.loads((Path(__file__).parent / "golden" / "mc_bloch.json").read_text())


@pytest.mark.parametrize("name", sorted(bc.CASES))
def test_within_4_standard_errors_of_reference(cuda, mc_bloch, name):
    case = bc.CASES[name]
    ref = mc_bloch[name]
    seq = bc.sequence(ps, case["seq"])
    g = bc.geometry(d, case["geom"])
    n_rep, n_each = 16, 12_500
    vals = np.stack([bc.flatten(d.run_bloch_sequence(seq, n_each, D, g, seed=100 + k,
                                                     **case["kw"]),
                                case["kw"].get("return_mz", False)) for k in range(n_rep)])
    mean = vals.mean(axis=0)
    sd_walker = vals.std(axis=0, ddof=1) * np.sqrt(n_each)
    se = sd_walker * np.sqrt(1.0 / ref["n_walkers"] + 1.0 / (n_rep * n_each))
    se = np.maximum(se, np.asarray(ref["stderr"]))
    # a value without walker spread (no gradient: every walker carries the same M) is compared
    # to FP32 rounding
    se = np.maximum(se, 2e-6 + 2e-5 * np.abs(np.asarray(ref["value"])))
    z = (mean - np.asarray(ref["value"])) / se
    assert np.max(np.abs(z)) < 4.0, (name, z)


# ---- susceptibility fields on the device ---------------------------------------------------------
def _provider(kind):
    rng = np.random.default_rng(12)
    if kind == "spheres":
        return d.SusceptibilitySources(rng.uniform(-5e-6, 5e-6, (6, 3)),
                                       rng.uniform(0.6e-6, 1.2e-6, 6), 5e-6, B0=3.0)
    if kind == "myelin":
        return d.MyelinSusceptibility([[-2e-6, -2e-6], [2e-6, 1.5e-6]], [0.9e-6, 0.7e-6],
                                      [1.4e-6, 1.1e-6], 8e-6, delta_chi_a=-1e-6, B0=3.0,
                                      theta=1.3, alpha=0.4)
    x, y, z = np.meshgrid(*[np.linspace(0, 1, 24)] * 3, indexing="ij")
    dB = 1e-6 * (np.sin(5 * x) * np.cos(3 * y) + 0.5 * z)
    return d.GridSusceptibility(dB, np.array([-6e-6, -6e-6, -6e-6]), 0.5e-6, periodic=False)


@pytest.mark.parametrize("kind", ["spheres", "myelin", "grid"])
def test_static_field_dephases_the_gradient_echo_and_the_180_refocuses_it(cuda, kind):
    """Walkers held still (D ~ 0): the gradient echo is the mean of exp(i n_t gamma dt dBz(r0))
    with dBz from the host provider, and a 180 at the middle refocuses the static field."""
    n, n_t, dt = 4096, 101, 1e-4
    g = d.Sphere(6e-6)
    r0 = g.init_positions(n, 3).astype(np.float32)
    prov = _provider(kind)
    wf = _zero(n_t, dt)
    gre = B._bloch_walk(n, 1e-20, wf, g, EXC_Y, r0=r0, susceptibility=prov)[0]
    phase = n_t * np.float64(np.float32(d.GAMMA * dt)) * prov.delta_bz_fn()(r0).astype(np.float64)
    expect = np.mean(np.exp(1j * phase))
    assert abs(complex(gre[0]) - expect) < 2e-3, (gre[0], expect)
    assert abs(expect) < 0.9
    se = B._bloch_walk(n, 1e-20, wf, g, EXC_Y + [{'t_s': 50 * dt, 'flip_deg': 180.0}], r0=r0,
                       susceptibility=prov)[0]
    one = np.mean(np.exp(-1j * phase / n_t))      # one sample's phase is left after the echo
    assert abs(abs(complex(se[0])) - abs(one)) < 2e-3
