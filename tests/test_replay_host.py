"""Replay packs and compressed walks, host side: the codecs, decoders, acquisition battery,
compiled scheme and log-weights against the reference's own compression.py / replay.py outputs
(tests/golden/replay_kat.npz), and the .rpk container round trip."""
import json
import struct

import numpy as np
import pytest

from dmipy_sim_gb300 import compression as cx
from dmipy_sim_gb300 import replay as rp


@pytest.fixture(scope="module")
def z():
    from pathlib import Path
    return np.load(Path(__file__).parent / "golden" / "replay_kat.npz")


def test_rle_rows_round_trip_and_match_reference(z):
    comp = z["comp_int"]
    a, meta = cx.encode_compartment(comp)
    for k in ("comp_rle_vals", "comp_rle_lens", "comp_rle_counts"):
        np.testing.assert_array_equal(a[k], z[f"comp_{k}"])
        assert a[k].dtype == z[f"comp_{k}"].dtype
    np.testing.assert_array_equal(cx.decode_compartment(a, meta), comp)
    rng = np.random.default_rng(2)
    A = rng.integers(-3, 4, (17, 9))
    v, l, c, n = cx.rle_encode_rows(A)
    np.testing.assert_array_equal(cx.rle_decode_rows(v, l, c, n), A)


def test_fractional_channels_match_reference(z):
    fr = z["comp_frac"]
    a, meta = cx.encode_compartment(fr)
    np.testing.assert_array_equal(cx.decode_compartment(a, meta), z["compf_decoded"])
    a, meta = cx.encode_bound_fraction(fr)
    np.testing.assert_array_equal(cx.decode_bound_fraction(a, meta), z["bfrac_decoded"])


def test_boundary_local_time_codecs_match_reference(z):
    raw = z["blt_raw"]
    a, meta = cx.encode_boundary_local_time(raw)
    assert (meta["mode"] == "sparse") == bool(z["blt_sparse_mode"])
    for k, v in a.items():
        np.testing.assert_array_equal(v, z[f"bltq_{k}"])
    np.testing.assert_array_equal(cx.decode_boundary_local_time(a, meta), z["bltq_decoded"])
    a, meta = cx.encode_boundary_local_time(z["bltd_raw"])
    assert meta["mode"] == "dense"
    np.testing.assert_array_equal(a["blt_dense_q"], z["bltd_q"])
    np.testing.assert_array_equal(cx.decode_boundary_local_time(a, meta), z["bltd_decoded"])


def test_decoders_match_reference(z):
    arrays = {k: z[f"tdct_{k}"] for k in cx.POSITION_AXES}
    n_t = z["traj"].shape[1]
    dec = cx.decode(arrays, {"method": "temporal_dct", "K": 16, "n_t": n_t})
    np.testing.assert_allclose(dec, z["tdct_decoded"], rtol=1e-6, atol=1e-13)
    meta = {"n_t": n_t, "K": 8}
    ell = cx.decode_boundary_dct({"blt_dct_coeffs": z["blt_dct_coeffs"],
                                  "blt_endpoint": z["blt_endpoint"]}, meta)
    np.testing.assert_allclose(ell, z["blt_dct_decoded"], rtol=1e-6, atol=1e-14)
    # low rank: the reconstruction does not depend on the SVD's sign convention
    a, m, _ = cx.encode_lowrank(z["traj"], 8)
    np.testing.assert_allclose(cx.decode(a, m), z["lowrank_decoded"], atol=2e-3 * np.abs(
        z["traj"]).max())


def test_acquisition_battery_matches_reference(z):
    n_t = z["traj"].shape[1]
    G, meta = cx.acquisition_battery(n_t, float(z["dt"]), cx.default_envelope())
    np.testing.assert_array_equal(G, z["battery_G"])
    np.testing.assert_allclose([q["b"] for q in meta], z["battery_b"])
    np.testing.assert_allclose([q["Gpeak"] for q in meta], z["battery_Gpeak"], rtol=1e-14)
    assert [q["fam"] for q in meta] == list(z["battery_fam"])


def test_compiled_scheme_and_log_weights_match_reference(z):
    W = rp.compile_scheme(z["battery_G"][:12], float(z["dt"]), 16)
    np.testing.assert_allclose(W, z["scheme_W"], rtol=1e-12, atol=1e-9)
    comp, fr = z["comp_int"], z["comp_frac"]
    n_t = comp.shape[1]
    dt = float(z["dt"])
    np.testing.assert_allclose(
        cx.relaxation_logweight(comp.clip(0, 1), [0.06, 0.08], [0.9, 1.2], dt,
                                chi=(np.arange(n_t) < 80).astype(float)), z["relax_lw"])
    np.testing.assert_allclose(cx.relaxation_logweight(fr, [0.06, 0.08], [0.9, 1.2], dt),
                               z["relax_lw_frac"])
    np.testing.assert_allclose(
        cx.surface_logweight(z["blt_raw"], 500.0, chi=(np.arange(n_t) % 3 == 0).astype(float)),
        z["surf_lw"])
    blt = z["pack_blt_dct"]
    np.testing.assert_allclose(rp.surface_logweight(blt, 500.0, n_t),
                               500.0 * np.sqrt(n_t) * blt[:, 0])
    np.testing.assert_allclose(rp.surface_logweight(blt, 500.0, n_t, z["rs_chi_hat"]),
                               500.0 * blt[:, :4] @ z["rs_chi_hat"])


def test_rpk_container_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    arrays = {"pos_x": rng.normal(size=(7, 5)).astype(np.float32),
              "pos_y": rng.normal(size=(7, 5)).astype(np.float32),
              "pos_z": rng.normal(size=(7, 5)).astype(np.float32),
              "spin_weights": rng.uniform(size=7).astype(np.float32),
              "comp_rle_vals": np.arange(11, dtype=np.int16), "blt_dense_q": np.ones((7, 3), np.int8),
              "empty": np.zeros((0, 4), np.float64), "flags": np.array([True, False])}
    meta = {"id": "t", "walk_params": {"n_t": 40, "dt_traj": 1e-4}, "compression": {
        "method": "temporal_dct"}, "license": "CC-BY-4.0"}
    path = tmp_path / "t.rpk"
    rp.write_rpk(path, arrays, meta)
    raw = path.read_bytes()
    (n,) = struct.unpack("<Q", raw[:8])
    assert n % 8 == 0
    hdr = json.loads(raw[8:8 + n])
    assert json.loads(hdr["__metadata__"]["rpk"]) == meta
    ends = sorted(v["data_offsets"] for k, v in hdr.items() if k != "__metadata__")
    assert ends[0][0] == 0 and all(a[1] == b[0] for a, b in zip(ends, ends[1:]))
    assert ends[-1][1] == len(raw) - 8 - n
    p = rp.read_rpk(path)
    assert set(p.arrays) == set(arrays)
    for k, v in arrays.items():
        assert p.arrays[k].dtype == v.dtype and np.array_equal(p.arrays[k], v)
    assert (p.n_t, p.dt, p.K, p.n_walkers, p.method, p.license) == (40, 1e-4, 5, 7,
                                                                     "temporal_dct", "CC-BY-4.0")
    assert p.dct_coeffs.shape == (7, 5, 3)


def test_position_layout_is_strict():
    with pytest.raises(KeyError):
        cx.read_position_coeffs({"dct_coeffs": np.zeros((2, 3, 3))})
    with pytest.raises(KeyError):
        cx.read_position_coeffs({"pos_x": np.zeros((2, 3))}, axes=(0, 2))
    C = np.arange(24, dtype=np.float32).reshape(2, 4, 3)
    a = cx.pack_position_arrays(C)
    np.testing.assert_array_equal(cx.read_position_coeffs(a, dtype=np.float32), C)
    np.testing.assert_array_equal(cx.read_position_coeffs(a, axes=(2,))[..., 0], C[..., 2])


def test_dct_basis_is_scipys_orthonormal_dct():
    from scipy.fft import dct
    x = np.random.default_rng(0).normal(size=(37, 2))
    B = cx.dct_basis(37, 9)
    np.testing.assert_allclose(B @ x, dct(x, type=2, norm="ortho", axis=0)[:9], atol=1e-12)
    np.testing.assert_allclose(B @ B.T, np.eye(9), atol=1e-12)
