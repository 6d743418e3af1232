"""Compressed walks and replay packs on the GPU: the temporal projections (dmsim_project_modes)
and mode-space replays (dmsim_replay over DCT bands) against the reference's own compression.py,
replay.py and trajectories.replay outputs (tests/golden/replay_kat.npz); the compressed trajectory
export against the raw one; a pack built, written, read and replayed end to end."""
from pathlib import Path

import numpy as np
import pytest

import dmipy_sim_gb300 as d
from dmipy_sim_gb300.trajectories import replay as tr_replay
from dmipy_sim_gb300 import compression as cx
from dmipy_sim_gb300 import core
from dmipy_sim_gb300 import replay as rp

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def z():
    return np.load(Path(__file__).parent / "golden" / "replay_kat.npz")


def _scale(x):
    return float(np.max(np.abs(x)))


def test_temporal_projection_matches_reference(cuda, z):
    a, meta, _ = cx.encode_temporal_dct(z["traj"], 16)
    assert meta == {"method": "temporal_dct", "K": 16, "n_t": z["traj"].shape[1]}
    for k in cx.POSITION_AXES:
        ref = z[f"tdct_{k}"]
        # FP32 input and Kahan-compensated FP32 sums against an FP64 DCT rounded to FP32
        np.testing.assert_allclose(a[k], ref, rtol=0, atol=2e-6 * _scale(ref))
    a8, m8 = cx.encode_boundary_dct(z["blt_raw"], K=8)
    np.testing.assert_allclose(a8["blt_endpoint"], z["blt_endpoint"], rtol=1e-5,
                               atol=1e-6 * _scale(z["blt_endpoint"]))
    np.testing.assert_allclose(a8["blt_dct_coeffs"], z["blt_dct_coeffs"], rtol=0,
                               atol=1e-5 * _scale(z["blt_dct_coeffs"]))


def test_projection_of_float16_series_and_ragged_sizes(cuda):
    """Odd walker counts (partial tiles), n_t not a multiple of the staging chunk, K not a
    multiple of the register tile, float16 input, K > n_t (clamped to n_t)."""
    import torch
    from scipy.fft import dct
    rng = np.random.default_rng(3)
    for n_w, n_t, K in ((1, 1, 1), (129, 37, 11), (300, 16, 40)):
        x = rng.normal(size=(n_w, n_t, 3)).astype(np.float16)
        got = cx.project_modes(torch.from_numpy(x).cuda(), K).cpu().numpy()
        ref = dct(x.astype(np.float64), type=2, norm="ortho", axis=1)[:, :K, :]
        assert got.shape == ref.shape
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-5 * max(_scale(ref), 1.0))
        e, m = cx.project_modes(x[..., 0].astype(np.float32), K, cumulative=True)
        B = np.cumsum(x[..., 0].astype(np.float64), axis=1)
        resid = B - B[:, -1:] * np.linspace(0, 1, n_t)[None, :]
        np.testing.assert_allclose(e.cpu().numpy(), B[:, -1], rtol=1e-5, atol=1e-5)
        np.testing.assert_allclose(m.cpu().numpy(),
                                   dct(resid, type=2, norm="ortho", axis=1)[:, :K],
                                   rtol=0, atol=2e-5 * max(_scale(B), 1.0))


def test_mode_space_replay_matches_reference(cuda, z):
    a = {k: z[f"tdct_{k}"] for k in cx.POSITION_AXES}
    meta = {"method": "temporal_dct", "K": 16, "n_t": z["traj"].shape[1]}
    G = z["battery_G"][:12]
    phi = cx.mode_space_phi(a, meta, G, float(z["dt"]))
    np.testing.assert_allclose(phi, z["ms_phi"], rtol=0, atol=2e-5 * max(_scale(z["ms_phi"]), 1))
    S = cx.mode_space_signal(a, meta, G, float(z["dt"]), logw=z["ms_logw"], weights=z["ms_w"])
    np.testing.assert_allclose(S, z["ms_signal"], atol=2e-6)


def test_pack_replay_signal_matches_reference(cuda, z):
    a = {k: z[f"tdct_{k}"] for k in cx.POSITION_AXES}
    W = z["scheme_W"]
    np.testing.assert_allclose(rp.replay_signal(dict(a), W), z["rs_plain"], atol=2e-6)
    pack = dict(a, spin_weights=z["ms_w"].astype(np.float32), blt_dct=z["pack_blt_dct"])
    np.testing.assert_allclose(rp.replay_signal(pack, W, complex_signal=True), z["rs_complex"],
                               atol=2e-6)
    n_t = z["traj"].shape[1]
    P = rp.ReplayPack(pack, {"n_t": n_t})
    np.testing.assert_allclose(rp.replay_signal(P, W, rho_over_D=500.0), z["rs_surface"],
                               atol=2e-6)
    np.testing.assert_allclose(rp.replay_signal(P, W, rho_over_D=500.0, chi_hat=z["rs_chi_hat"]),
                               z["rs_gated"], atol=2e-6)


def test_fidelity_and_mode_selection_match_reference(cuda, z):
    X, dt = z["traj"], float(z["dt"])
    a8, m8, _ = cx.encode_temporal_dct(X, 8)
    fid = cx.measure_fidelity(X, dt, cx.decode(a8, m8), cx.default_envelope())
    np.testing.assert_allclose(fid["err_max"], z["fid_err_max"], rtol=1e-4)
    np.testing.assert_allclose(fid["floor_max"], z["fid_floor_max"], rtol=1e-4)
    assert sorted(fid["per_family"]) == list(z["fid_fams"])
    np.testing.assert_allclose([fid["per_family"][f]["err_max"] for f in z["fid_fams"]],
                               z["fid_fam_err"], rtol=1e-3, atol=1e-6)
    K, _ = cx.auto_select_modes(X, X, dt, K_grid=(4, 8, 16, 32))
    assert K == int(z["auto_K"])


def test_replay_of_compressed_master_matches_reference(cuda, z):
    C = cx.read_position_coeffs({k: z[f"tdct_{k}"] for k in cx.POSITION_AXES}, dtype=np.float32)
    n_t = z["traj"].shape[1]
    master = {"compressed": True, "method": "temporal_dct", "K": 16, "n_t": n_t,
              "dt_traj": float(z["dt"]), "pos_modes": C,
              "blt_endpoint": z["master_blt_endpoint"], "blt_modes": z["master_blt_modes"],
              "comp_traj": z["comp_int"].clip(0, 1)}
    G, dtw = z["rc_G"], float(z["rc_dt"])
    np.testing.assert_allclose(tr_replay(master, None, G, dtw), z["rc_plain"], atol=2e-6)
    np.testing.assert_allclose(tr_replay(master, None, G, dtw, T2=0.07, T1=0.9,
                                        surface_relaxivity=1e-5, D=2e-9), z["rc_relax"],
                               atol=2e-6)
    got = tr_replay(master, None, z["rc2_G"], float(z["rc2_dt"]), chi_perp=z["rc2_chi"],
                   T2_per_comp=[0.05, 0.08], T1_per_comp=[0.8, 1.1], surface_relaxivity=2e-5,
                   D=2e-9, stimulated_echo=True)
    np.testing.assert_allclose(got, z["rc_gated"], atol=2e-6)


@pytest.mark.parametrize("geom", ["cyl_rho", "sph_kappa"])
def test_compressed_export_is_the_projection_of_the_raw_walk(cuda, geom):
    """simulate_trajectories(compress=K) walks the same walkers as the raw export (walkers are
    keyed by their global index, whatever the batch split) and keeps their DCT-II bands; a
    waveform mostly inside the band replays the same from both."""
    from scipy.fft import dct
    g = (d.Cylinder(4e-6, (0.3, 0.2, 1.0), surface_relaxivity_t2=1e-5) if geom == "cyl_rho"
         else d.Sphere(4e-6, permeability=1e-5))
    D, n, T, dts, K = 2e-9, 3000, 0.03, 3e-4, 24
    m = d.simulate_trajectories(n, D, g, T, dts, seed=5, compress=K, walker_batch_size=1100,
                                save_relaxation_data=True)
    raw = d.simulate_trajectories(n, D, g, T, dts, seed=5, save_relaxation_data=True)
    traj, dt_act = raw[0], raw[1]
    assert m["n_t"] == traj.shape[1] and m["K"] == K and abs(m["dt_traj"] - dt_act) < 1e-15
    # the bands of the (float16) raw export, against the float32 walk's bands
    ref = dct(traj.astype(np.float64), type=2, norm="ortho", axis=1)[:, :K, :]
    err = np.abs(m["pos_modes"] - ref).max(axis=(1, 2))
    assert np.mean(err < 4e-3 * _scale(ref[:, 0])) > 0.99
    dl = raw[4].astype(np.float32)
    e_ref = dl.astype(np.float64).sum(1)
    np.testing.assert_allclose(m["blt_endpoint"], e_ref, rtol=2e-2, atol=1e-3 * _scale(e_ref))
    if geom == "sph_kappa":
        np.testing.assert_array_equal(m["comp_traj"], raw[5])
    # replay from the bands vs replay from the raw trajectory: a PGSE mostly inside the band.
    # The gate is passed explicitly: without one the raw replay relaxes only inside the
    # waveform's window and the compressed replay over the whole walk, as in the reference
    # (trajectories.py:500-501, 289-291).
    wf = d.set_b(d.pgse(0.008, 0.016, 0.03, [[1, 0, 0], [0, 0, 1]], 101), [1e9, 2e9])
    chi = np.ones(wf.G.shape[1])
    s_c = tr_replay(m, None, wf.G, wf.dt, chi_perp=chi, T2=0.08)
    s_r = tr_replay(traj, dt_act, wf.G, wf.dt, chi_perp=chi, T2=0.08)
    np.testing.assert_allclose(s_c, s_r, atol=5e-3)


def test_pack_built_written_read_and_replayed(cuda, tmp_path):
    g = d.Cylinder(3e-6, (0, 0, 1), surface_relaxivity_t2=1e-5)
    D = 2e-9
    t, dt_act, S, _, dlog, comp = d.simulate_trajectories(2000, D, g, 0.02, 2e-4, seed=9,
                                                          save_relaxation_data=True)
    master = {"traj": t, "dt_traj": dt_act, "T_max": 0.02, "dlog_b": dlog.astype(np.float32),
              "D_intra": D, "seed": 9, "walkers_shuffled": True}
    path = tmp_path / "cyl.rpk"
    pack = d.build_replay_pack(master, id="cyl3um", K=32, license="CC-BY-4.0", citation="test",
                               surface_relaxivity=True, blt_temporal_K=16, out_path=str(path))
    back = d.read_rpk(path)
    assert back.K == 32 and back.n_walkers == 2000 and back.n_t == t.shape[1]
    assert back.meta["replay_envelope"]["surface_relaxivity"]
    assert back.meta["compression"]["precision_tiers"]["usable"]
    for k in cx.POSITION_AXES:
        np.testing.assert_array_equal(back.arrays[k], pack.arrays[k])
    wf = d.set_b(d.pgse(0.005, 0.012, 0.02, [[1, 0, 0], [0, 1, 0], [0, 0, 1]], 101),
                 [1.5e9, 1.5e9, 1.5e9])
    from dmipy_sim_gb300.trajectories import _resample
    Gt, _ = _resample(np.asarray(wf.G, np.float64), np.ones(101), back.n_t, back.dt, wf.dt)
    W = rp.compile_scheme(Gt, back.dt, back.K)
    # the real part of the pack's complex signal against the raw replay's mean cosine (the
    # magnitude carries the imaginary part's sampling noise, ~1/sqrt(2N), at low signal)
    s_pack = rp.replay_signal(back, W, complex_signal=True).real
    s_raw = tr_replay(t, dt_act, wf.G, wf.dt)
    np.testing.assert_allclose(s_pack, s_raw, atol=4e-3)
    assert back.fidelity["floor_max"] > 0 and np.isfinite(back.fidelity["err_max"])
