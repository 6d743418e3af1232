"""Statistical parity with the reference's own Monte-Carlo results on the benchmark
configurations (tests/golden/mc_configs.json, made by running dmipy-sim's core.simulate /
simulate_cpmg unmodified, tens of thousands of walkers each): free diffusion with PGSE; a
cylinder with surface relaxivity and a permeable sphere, 30 directions; the 16 x 16 lognormal
lattice at f = 0.6 under the default engine (walk once + replay, 27 sub-steps per sample) with
all 64 benchmark measurements, with permeable walls (kappa = 2e-5, 460 sub-steps per sample)
and as a 16-echo CPMG train.

The GPU walks 1,000,000 walkers through the same plan as simulate() / simulate_cpmg(), so its
own error is small; every signal must lie within 3 standard errors of the difference, the
standard error being the per-walker spread (measured on the GPU walk, the same distribution when
the two walks are the same process) over both walker counts."""
import json
from pathlib import Path

import numpy as np
import pytest

import dmipy_sim_gb300 as d
from dmipy_sim_gb300 import core
from golden import mc_configs as MC

pytestmark = pytest.mark.gpu
D = 2e-9
N_GPU = 1_000_000
FIXTURE = Path(__file__).parent / "golden" / "mc_configs.json"


def _fixtures():
    if not FIXTURE.exists():
        return {}
    return json.loads(FIXTURE.read_text())


def _gpu(cfg, n, seed):
    wf = MC.waveform(d, tuple(cfg["wf"]))
    g = MC.geometry(d, tuple(cfg["geom"]))
    G, chi = core._waveform_arrays(wf, g)
    if cfg["api"] == "cpmg":
        S, fused, echo = core.fused_sub_steps(g, D, wf.dt), True, np.unique(wf.echo_indices)
    else:
        gap = core._replay_gap(g, return_positions=False, return_compartments=False,
                               return_walker_signals=False, diffusivity=D)
        rep = gap is None and core._replay_auto_allowed(g)
        S = core.replay_sub_steps(g, D, wf.dt) if rep else core.fused_sub_steps(g, D, wf.dt)
        fused, echo = not rep, None
    res = core.run_walk(g, n_walkers=n, diffusivity=D, G=G, dt=wf.dt, sub_steps=S,
                        phase_per_substep=fused, seed=seed, chi=chi, T2=cfg.get("T2"),
                        echo_idx=echo)
    if cfg["api"] == "cpmg":
        return res.signal, res.stderr * np.sqrt(n)
    return res.signal[0], res.stderr[0] * np.sqrt(n)


@pytest.mark.parametrize("name", sorted(MC.CONFIGS))
def test_benchmark_configuration_within_3_standard_errors_of_reference(cuda, name):
    fx = _fixtures()
    if name not in fx:
        pytest.skip(f"{name} is not in tests/golden/mc_configs.json")
    ref = fx[name]
    sig, sd = _gpu(ref["config"], N_GPU, seed=31337)
    s_ref = np.asarray(ref["signal"]).reshape(sig.shape)
    se = sd * np.sqrt(1.0 / ref["n_walkers"] + 1.0 / N_GPU)
    # a signal with no spread across walkers (no gradient: every walker carries the same
    # weight) is compared to the FP32 rounding of that weight
    se = np.maximum(se, 1e-6 + 1e-5 * np.abs(s_ref))
    z = (sig - s_ref) / se
    worst = int(np.argmax(np.abs(z)))
    assert np.max(np.abs(z)) < 3.0, (f"{name}: signal {worst} GPU {sig.ravel()[worst]:.5f} "
                                     f"reference {s_ref.ravel()[worst]:.5f} "
                                     f"z {z.ravel()[worst]:.2f}")
