"""Error of the FP32 GPU walk against an FP64 rerun of the same walks (the oracle's FP64 twin on
the same Philox stream).

* Free diffusion has no walls, so GPU and FP64 walkers stay identical and the difference is pure
  FP32 rounding: per-walker phase error and the resulting signal error are bounded tightly.
* With walls, FP32 and FP64 trajectories part ways after enough reflections (chaotic billiards),
  so the signals are compared against the Monte-Carlo standard error: the FP32 error must be
  invisible under the MC noise.
"""
import numpy as np
import pytest

from dmipy_sim_gb300 import core
from parity_cases import D, geometries, oracle_walk, plan, waveform

pytestmark = pytest.mark.gpu


def test_free_diffusion_phase_error_vs_fp64(cuda):
    geom = geometries()["free"]
    wf = waveform(n_dirs=16, n_t=1000, b=3e9)
    G, _ = core._waveform_arrays(wf, geom)
    n = 20000
    for use_basis in (True, False):
        gpu = core.run_walk(geom, n_walkers=n, diffusivity=D, G=G, dt=wf.dt, sub_steps=1,
                            phase_per_substep=False, seed=4, want_walker_signals=True,
                            use_basis=use_basis)
        ref = oracle_walk(geom, G, wf.dt, 1, False, n, seed=4, fp64=True)
        dphi = np.abs(gpu.extras["phi"].cpu().numpy() - ref["phi"])
        assert np.max(dphi) < 5e-4, np.max(dphi)
        np.testing.assert_allclose(gpu.signal[0], ref["signal"][0], atol=2e-5)


@pytest.mark.parametrize("name", ["cyl_rho", "sph", "pcyl", "psph", "sph_kappa"])
def test_walls_signal_error_vs_fp64_below_mc_noise(cuda, name):
    geom = geometries()[name]
    wf = waveform(n_dirs=5, n_t=60)
    G, _ = core._waveform_arrays(wf, geom)
    S, ps = plan(geom, wf, "auto")
    n = 8192
    gpu = core.run_walk(geom, n_walkers=n, diffusivity=D, G=G, dt=wf.dt, sub_steps=S,
                        phase_per_substep=ps, seed=6, T2=0.07)
    ref = oracle_walk(geom, G, wf.dt, S, ps, n, seed=6, T2=0.07, fp64=True, want_walkers=False)
    z = (gpu.signal[0] - ref["signal"][0]) / np.maximum(np.sqrt(2.0) * gpu.stderr[0], 1e-9)
    assert np.max(np.abs(z)) < 4.0, z
