"""Replay-pack producer (bank.py of dmipy-sim): compress a master walk and assemble a
self-certifying ``.rpk``.

``build_replay_pack`` takes a master walk (``traj`` (n, n_t, 3), ``dt_traj``, ``T_max`` and the
optional tier channels: ``comp``/``T2_per_comp``/``T1_per_comp`` bulk relaxation, ``dlog_b`` surface
relaxivity, ``bfrac`` magnetisation transfer, ``w`` spin weights), picks the mode count that keeps
the measured replay error within ``tol`` x the split-half Monte-Carlo floor over an acquisition
envelope (or takes ``K``), encodes the positions and channels (compression.py) and records the
fidelity, precision tiers and provenance in the metadata.  The fidelity replays and the temporal
projections run on the GPU.  The susceptibility tiers are not assembled (their field grids and
off-resonance replay are outside this package).
"""
import numpy as np

from . import compression as _cx
from .replay import ReplayPack, write_rpk

RPK_SCHEMA_VERSION = "1.1"

__all__ = ["build_replay_pack", "build_to_floor", "frame_from_axis", "RPK_SCHEMA_VERSION"]


def _master_arrays(src):
    """The master dict of a raw walk dict / ``.npz`` (bank.py:35-65)."""
    if not (isinstance(src, dict) or hasattr(src, "files")):
        raise TypeError("build_replay_pack expects a master-walk dict / .npz with keys "
                        "traj/dt_traj/T_max[/comp/T2_per_comp/T1_per_comp/dlog_b/bfrac/w]; got "
                        f"{type(src).__name__}.")
    keys = src.files if hasattr(src, "files") else src.keys()
    m = {k: src[k] for k in keys}

    def g(k):
        return np.asarray(m[k]) if k in m and m[k] is not None else None

    def scal(k):
        return float(np.asarray(m[k])) if m.get(k) is not None else None
    traj = np.asarray(m["traj"])
    return dict(traj=traj, dt_traj=float(np.asarray(m["dt_traj"])),
                T_max=float(np.asarray(m["T_max"])), comp=g("comp"), comp0=g("comp0"), w=g("w"),
                dlog_b=g("dlog_b"), bfrac=g("bfrac"),
                susc_field_basis=m.get("susc_field_basis") if isinstance(m, dict) else None,
                PhiC=g("PhiC"), susc_basis=g("susc_basis"),
                mt_params=m.get("mt_params") if isinstance(m, dict) else None,
                cell_size=scal("cell_size"), R=g("R"), D_intra=scal("D_intra"),
                T2_per_comp=g("T2_per_comp"), T1_per_comp=g("T1_per_comp"),
                substrate_frame=g("substrate_frame"),
                walkers_shuffled=bool(m.get("walkers_shuffled", False)),
                n_walkers=int(traj.shape[0]), seed=int(np.asarray(m.get("seed", 0))))


def frame_from_axis(axis):
    """Orthonormal substrate frame (columns x, y, z) with z along ``axis`` and x from the global
    axis least aligned with it (bank.py:69-80)."""
    z = np.asarray(axis, float)
    z = z / np.linalg.norm(z)
    seed = np.eye(3)[int(np.argmin(np.abs(z)))]
    x = seed - z * float(seed @ z)
    x /= np.linalg.norm(x)
    return np.column_stack([x, np.cross(z, x), z])


def _envelope_summary(env):
    return dict(b_max=float(max(env["bvals"])), ogse_periods=list(env.get("ogse_periods", [])),
                B0_list=list(env.get("B0_list", [])),
                note="temporal band set by max OGSE period / min delta")


def _measure_floor(m, env):
    """Split-half Monte-Carlo floor of the raw walk over the envelope (bank.py:113-117)."""
    traj = np.asarray(m["traj"])
    return float(_cx.measure_fidelity(traj, float(m["dt_traj"]), traj, env)["floor_max"])


def _surface_fidelity(m, arrays, chan_meta, env):
    """Surface-tier check: the attenuation from the stored boundary channel against the raw one
    over a rho battery, with the raw channel's split-half floor (bank.py:120-146)."""
    raw = m.get("dlog_b")
    if raw is None or not any(k in arrays for k in ("blt_dct_coeffs", "blt_dense_q",
                                                   "blt_counts")):
        return None
    raw = np.asarray(raw, np.float64)
    n_w = raw.shape[0]
    w = np.asarray(m["w"], np.float64) if m.get("w") is not None else np.ones(n_w)
    D = float(m.get("D_intra") or 0.0) or 1.0
    dec = (_cx.decode_boundary_dct(arrays, chan_meta) if "blt_dct_coeffs" in arrays
           else _cx.decode_boundary_local_time(arrays, chan_meta))
    perm = np.random.RandomState(0).permutation(n_w)
    A, B = perm[:n_w // 2], perm[n_w // 2:]

    def fac(sl, idx):
        return float(np.sum(w[idx] * np.exp(sl[idx])) / np.sum(w[idx]))
    err = floor = 0.0
    for rho in (env.get("rho_list") or [1e-5, 3e-5, 1e-4]):
        rd = float(rho) / D
        s_raw = _cx.surface_logweight(raw, rd)
        s_dec = _cx.surface_logweight(dec, rd)
        err = max(err, abs(fac(s_raw, slice(None)) - fac(s_dec, slice(None))))
        floor = max(floor, abs(fac(s_raw, A) - fac(s_raw, B)))
    return dict(err=float(err), floor=float(floor))


def _select_boundary_codec(m, dlog, env, tol, dtype, verbose=False):
    """Cheapest boundary codec that passes the surface gate: the detrended cumulative DCT at
    K = 8, 16, 32, 64, else the exact sparse/dense codec (bank.py:560-589)."""
    cands = []
    for K in (8, 16, 32, 64):
        a, mm = _cx.encode_boundary_dct(dlog, K=K, dtype=dtype)
        cf = _surface_fidelity(m, a, mm, env)
        cands.append((K, cf))
        if cf is not None and cf["err"] <= tol * cf["floor"]:
            if verbose:
                print(f"boundary channel: {K} cumulative DCT bands ({np.dtype(dtype).name}), "
                      f"surface error {cf['err']:.2e} / floor {cf['floor']:.2e}", flush=True)
            return a, mm
    a, mm = _cx.encode_boundary_local_time(dlog)
    if verbose:
        print(f"boundary channel: no band count met the surface gate, stored {mm['mode']} "
              "(quantised per step)", flush=True)
    return a, mm


_TIER_FLOORS = (1e-2, 3e-3, 1e-3)


def _prefix_layout(arrays, n_walkers):
    """(bytes per walker of the walker-leading tensors, bytes of the rest, names of the rest).

    A tensor whose first axis is the walker axis can be read for a walker prefix as one
    contiguous range; the others (run-length rows, modes, tables) must be read whole."""
    per_walker, whole = 0, {}
    for name, v in arrays.items():
        a = np.asarray(v)
        if a.ndim and a.shape[0] == n_walkers:
            per_walker += a.nbytes // max(n_walkers, 1)
        else:
            whole[name] = a.nbytes
    return int(per_walker), int(sum(whole.values())), sorted(whole)


def _precision_tiers(arrays, n_walkers, floor_max, walkers_shuffled):
    """Walker-prefix reads for the statistical floors 1e-2, 3e-3 and 1e-3 (the metadata block of
    bank.py:526-557): the Monte-Carlo floor falls as n^-1/2, so a floor eps needs the first
    n = N (floor_max / eps)^2 walkers (at least 1, at most N).  A prefix is an unbiased
    sub-ensemble only when the producer declares the walker order shuffled."""
    per_walker, fixed, whole = _prefix_layout(arrays, n_walkers)

    def tier(eps):
        n = int(np.clip(np.ceil(n_walkers * (floor_max / eps) ** 2), 1, n_walkers))
        return dict(eps=float(eps), n_walkers=n, bytes=int(n * per_walker + fixed),
                    reachable=bool(n < n_walkers or floor_max <= eps))

    shuffled = bool(walkers_shuffled)
    return dict(bytes_per_walker=per_walker, fixed_bytes=fixed, not_prefix_sliceable=whole,
                floor_at_full_n=float(floor_max), walkers_shuffled=shuffled, usable=shuffled,
                tiers=[tier(e) for e in _TIER_FLOORS] if floor_max > 0 else [],
                note=("walker prefixes are exchangeable samples of the ensemble" if shuffled
                      else "walker order not declared shuffled: a prefix can be a biased "
                           "sub-ensemble"))


def _refresh(fid, err, floor, sigma_star):
    fid["err_max"] = max(float(fid.get("err_max", 0.0)), err)
    fid["floor_max"] = max(float(fid.get("floor_max", 0.0)), floor)
    fid["within_2x_floor"] = bool(fid["err_max"] <= 2.0 * fid["floor_max"])
    if sigma_star is not None:
        fid["meets_target"] = bool(fid["err_max"] <= sigma_star and fid["floor_max"] <= sigma_star)
    return fid


def build_replay_pack(src, *, id, method="temporal_dct", envelope=None, tol=2.0, K=None,
                      err_target=None, sigma_star=None, license, citation, provenance=None,
                      surface_relaxivity=False, blt_temporal_K=None, blt_dtype=np.float16,
                      susc_path_K=None, mt=False, out_path=None, verbose=False):
    """Compress a master walk into a replay pack (bank.py:592-787); returns a ReplayPack and
    writes it to ``out_path`` when given."""
    m = _master_arrays(src)
    if (m.get("PhiC") is not None or m.get("susc_basis") is not None
            or m.get("susc_field_basis") is not None or susc_path_K):
        raise NotImplementedError("the susceptibility (field) tiers are not assembled by this "
                                  "package")
    env = envelope or _cx.default_envelope()
    X = np.asarray(m["traj"])
    dt = float(m["dt_traj"])
    wp = _cx.is_walker_preserving(method)
    if K is None:
        K, fid = _cx.auto_select_modes(X, X, dt, method=method, env=env, tol=tol,
                                       err_target=err_target, verbose=verbose)
    else:
        a0, m0, _ = _cx.encode(X, method, K)
        fid = _cx.measure_fidelity(X, dt, _cx.decode(a0, m0, n_walkers=(X.shape[0] if wp
                                                                         else None)), env)
    fid = dict(fid)
    if sigma_star is not None:
        fid.update(target_floor=float(sigma_star),
                   meets_target=bool(fid["err_max"] <= sigma_star
                                     and fid["floor_max"] <= sigma_star))
    pos_arrays, pos_meta, _ = _cx.encode(X, method, K)
    arrays = dict(pos_arrays)
    chan_meta = {}
    channels = {"gradient": True, "susceptibility": False, "T1T2": False, "rho": False,
                "mt": (m.get("bfrac") is not None) or (m.get("mt_params") is not None)}
    if wp:
        if m.get("comp") is not None and m.get("T2_per_comp") is not None:
            a, cm = _cx.encode_compartment(np.asarray(m["comp"]))
            arrays.update(a)
            chan_meta["compartment"] = cm
            if m.get("w") is not None:
                arrays["spin_weights"] = np.asarray(m["w"], np.float32)
            channels["T1T2"] = True
        if surface_relaxivity and m.get("dlog_b") is not None:
            if blt_temporal_K:
                a, mm = _cx.encode_boundary_dct(np.asarray(m["dlog_b"]), K=int(blt_temporal_K),
                                                dtype=blt_dtype)
            else:
                a, mm = _select_boundary_codec(m, np.asarray(m["dlog_b"]), env, tol, blt_dtype,
                                               verbose)
            arrays.update(a)
            chan_meta["boundary_local_time"] = mm
            channels["rho"] = True
        if mt and m.get("bfrac") is not None:
            a, mm = _cx.encode_bound_fraction(np.asarray(m["bfrac"]), Q=256)
            arrays.update(a)
            chan_meta["bound_fraction"] = mm
            channels["mt"] = True
    if channels["rho"]:
        cf = _surface_fidelity(m, arrays, chan_meta["boundary_local_time"], env)
        if cf is not None:
            fid.update(err_surface=cf["err"], floor_surface=cf["floor"])
            fid = _refresh(fid, cf["err"], cf["floor"], sigma_star)
    n_t = X.shape[1]
    meta = _pack_metadata(m, id=id, method=method, K=K, walker_preserving=wp, n_t=n_t, dt=dt,
                          arrays=arrays, chan_meta=chan_meta, channels=channels, env=env,
                          fidelity=fid, provenance=provenance, license=license,
                          citation=citation)
    pack = ReplayPack(arrays, meta, source=out_path)
    if out_path is not None:
        write_rpk(out_path, {k: v for k, v in arrays.items() if v is not None}, meta)
    if verbose:
        verdict = "within" if fid["within_2x_floor"] else "beyond"
        print(f"pack {id}: {method} with {K} modes, replay error {fid['err_max']:.4f} "
              f"({verdict} 2 x the floor {fid['floor_max']:.4f})", flush=True)
    return pack


def _as_list(m, key):
    v = m.get(key)
    return None if v is None else np.asarray(v).tolist()


def _pack_metadata(m, *, id, method, K, walker_preserving, n_t, dt, arrays, chan_meta, channels,
                   env, fidelity, provenance, license, citation):
    """The .rpk metadata of a pack (the key layout of bank.py:741-781, which readers of the
    format rely on): compression block (method, modes, precision tiers, channel codecs), walk
    parameters, per-compartment constants, the replay envelope, fidelity and provenance."""
    compression = dict(method=method, K=int(K), walker_preserving=bool(walker_preserving),
                       n_t=int(n_t))
    if walker_preserving:
        compression["precision_tiers"] = _precision_tiers(
            arrays, int(m["n_walkers"]), float(fidelity.get("floor_max") or 0.0),
            bool(m.get("walkers_shuffled")))
    if chan_meta:
        compression["channels"] = chan_meta
    walk = dict(n_walkers=int(m["n_walkers"]), n_t=int(n_t), dt_traj=dt, T_max=float(m["T_max"]),
                diffusivity=m.get("D_intra"), seed=int(m["seed"]), cell_size=m.get("cell_size"),
                substrate_frame=_as_list(m, "substrate_frame"))
    envelope = dict(gradient=True, bulk_relaxation=channels["T1T2"],
                    surface_relaxivity=channels["rho"], field=False,
                    magnetization_transfer=channels["mt"], diffusivity_fixed=True,
                    acquisition=_envelope_summary(env))
    meta = dict(rpk_schema_version=RPK_SCHEMA_VERSION, id=id, compression=compression,
                walk_params=walk,
                per_comp=dict(T2=_as_list(m, "T2_per_comp"), T1=_as_list(m, "T1_per_comp"),
                              R=_as_list(m, "R")),
                replay_envelope=envelope, fidelity=fidelity, provenance=provenance or {},
                license=license, citation=citation)
    if m.get("mt_params") is not None:
        meta["mt"] = {k: (float(v) if isinstance(v, (int, float, np.floating)) else v)
                      for k, v in m["mt_params"].items()}
    return meta


def build_to_floor(make_model, *, id, envelope=None, sigma_star=1e-3, pilot_n=8000, safety=1.4,
                   max_n=400000, walk=None, method="temporal_dct", verbose=True, **bp):
    """A pack whose split-half floor reaches ``sigma_star`` (the contract of bank.py:790-808).

    The floor of a walk falls as n^-1/2, so a pilot of ``pilot_n`` walkers predicts the walker
    count, inflated by ``safety`` and capped at ``max_n``; when the walk at that count still
    misses the target, the count is predicted once more from it.  ``make_model(n)`` returns the
    master walk of n walkers on a fixed substrate (``walk`` maps it to the master dict)."""
    env = envelope or _cx.default_envelope()
    master_of = walk or _master_arrays

    def walk_floor(n):
        model = make_model(n)
        return model, _measure_floor(master_of(model), env)

    def predicted(n, floor):
        return int(min(max_n, round(n * (floor / sigma_star) ** 2 * safety)))

    _, f_pilot = walk_floor(pilot_n)
    n = max(pilot_n, predicted(pilot_n, f_pilot)) if pilot_n < max_n else max_n
    model, f = walk_floor(n)
    history = [(pilot_n, f_pilot), (n, f)]
    if f > sigma_star and n < max_n:
        n = predicted(n, f)
        model, f = walk_floor(n)
        history.append((n, f))
    if verbose:
        steps = ", ".join(f"{k} walkers -> {v:.3g}" for k, v in history)
        print(f"walker count for floor {sigma_star:.3g}: {steps}", flush=True)
    return build_replay_pack(model, id=id, envelope=env, method=method, err_target=sigma_star,
                             sigma_star=sigma_star, verbose=verbose, **bp)
