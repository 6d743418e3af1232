"""Pins the CPU oracle to the reference: every geometry plug-in call of dmipy-sim (reflect,
reflect_with_log_weight, permeate — recorded from the reference itself in tests/golden/kat.npz,
for the cylinder, sphere, packed substrates and triangle meshes) is reproduced by the oracle's FP32
restatement, and by its FP64 twin to FP32 rounding."""
import numpy as np
import pytest

from oracle import oracle as O

TAGS = ["cyl", "cyltilt", "sph", "pcyl", "psph"]
MODES = ["reflect", "relax", "perm"]


def _geom(kat, tag):
    if tag in ("cyl", "cyltilt"):
        from dmipy_sim_gb300.geometries import _rotation_to_z
        R = _rotation_to_z(kat[f"geo_{tag}_ori"]).astype(np.float32)
        return O.geom(O.CYLINDER, radius=float(kat[f"geo_{tag}_R"]), rot=R), float(kat[f"geo_{tag}_R"])
    if tag == "sph":
        return O.geom(O.SPHERE, radius=float(kat["geo_sph_R"])), float(kat["geo_sph_R"])
    radii = kat[f"geo_{tag}_radii"]
    c = kat[f"geo_{tag}_centers"]
    objs = np.zeros((len(radii), 4))
    objs[:, :c.shape[1]] = c.astype(np.float32)
    objs[:, 3] = radii.astype(np.float32)
    kind = O.PACKED_CYLINDERS if tag == "pcyl" else O.PACKED_SPHERES
    return O.geom(kind, L=np.float32(kat[f"geo_{tag}_L"]), objects=objs), float(radii.min())


def _run(kat, tag, mode, fp64):
    g, scale = _geom(kat, tag)
    key = f"pl_{tag}_{mode}"
    rs, st, ref, dref = (kat[key + "_r"], kat[key + "_step"], kat[key + "_out"], kat[key + "_dlog"])
    us = kat.get(key + "_u", np.zeros(len(rs)))
    m = int(kat[key + "_mode"])
    outs = np.zeros_like(ref)
    dl = np.zeros(len(rs))
    for i in range(len(rs)):
        outs[i], dl[i] = O.plugin(g, m, rs[i], st[i], float(kat[key + "_rho"]),
                                  float(kat[key + "_kappa"]), float(us[i]), fp64=fp64)
    return outs, dl, ref, dref, scale


@pytest.mark.parametrize("tag", TAGS)
@pytest.mark.parametrize("mode", MODES)
def test_oracle_fp32_matches_reference_plugins(kat, tag, mode):
    outs, dl, ref, dref, scale = _run(kat, tag, mode, fp64=False)
    err = np.max(np.abs(outs - ref), axis=1)
    # positions: FP32 restatement of FP32 code -> agreement at the rounding level of |r|
    tol = 1e-6 * np.maximum(np.max(np.abs(ref), axis=1), scale)
    bad = np.nonzero(err > tol)[0]
    assert len(bad) <= max(1, len(ref) // 100), (
        f"{len(bad)}/{len(ref)} cases differ; worst {err.max():.3e} m at case {int(np.argmax(err))}")
    np.testing.assert_allclose(dl, dref, rtol=1e-4, atol=1e-9)


@pytest.mark.parametrize("tag", TAGS)
@pytest.mark.parametrize("mode", MODES)
def test_oracle_fp64_close_to_reference_plugins(kat, tag, mode):
    outs, dl, ref, dref, scale = _run(kat, tag, mode, fp64=True)
    err = np.max(np.abs(outs - ref), axis=1)
    tol = 1e-4 * scale
    bad = np.nonzero(err > tol)[0]
    assert len(bad) <= max(2, len(ref) // 50), f"{len(bad)} cases beyond FP32 rounding"
    ok = np.abs(dl - dref) <= 1e-3 * np.abs(dref) + 1e-8
    assert ok.mean() > 0.97


def _mesh_geom(kat, tag, mode):
    """The oracle's own build of the meshes the reference recorded its calls on: a closed
    icosphere (5 um, 320 triangles) and a periodic 10 um box whose sphere crosses a face."""
    kw = {}
    if tag == "mshp":
        kw = dict(periodic=True, voxel_min=[-5e-6] * 3, voxel_max=[5e-6] * 3, feature_radius=3e-6)
    if mode == "reflect":
        sides = O.mesh_sides()
    elif mode == "relax":
        sides = O.mesh_sides(rho_intra=1e-6)
    else:
        sides = O.mesh_sides(rho_intra=1e-6 if tag == "msh" else None, kappa_out=1e-5,
                             kappa_in=1e-5)
    V = kat["mesh_V"] if tag == "msh" else kat["mesh_Vp"]
    return O.mesh_geom(V, kat["mesh_F"], rho_mult=sides[0], kappa_mult=sides[1],
                       permeable=sides[2], **kw)


@pytest.mark.parametrize("tag", ["msh", "mshp"])
@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("fp64", [False, True])
def test_oracle_mesh_matches_reference_plugins(kat, tag, mode, fp64):
    """Mesh.reflect / reflect_with_log_weight / permeate (rho/D = 500, kappa/D = 5000, the recorded
    Bernoulli uniform): FP32 agrees to the last bit but for rounding-order cases, FP64 to FP32
    rounding."""
    g = _mesh_geom(kat, tag, mode)
    wall = {"reflect": O.REFLECT, "relax": O.RELAX, "perm": O.PERMEATE}[mode]
    key = f"pl_{tag}_{mode}"
    rs, st, us = kat[key + "_r"], kat[key + "_step"], kat[key + "_u"]
    ref, dref = kat[key + "_out"], kat[key + "_dlog"]
    outs = np.zeros_like(ref)
    dl = np.zeros(len(rs))
    for i in range(len(rs)):
        outs[i], dl[i] = O.plugin(g, wall, rs[i], st[i], float(np.float32(500.0)),
                                  float(np.float32(5000.0)), float(us[i]), fp64=fp64)
    err = np.max(np.abs(outs - ref), axis=1)
    if not fp64:
        assert np.mean(np.all(outs == ref, axis=1)) >= 0.95
        assert err.max() <= 1e-7 * 5e-6 * 10      # a few ulp of the coordinates
        np.testing.assert_allclose(dl, dref, rtol=1e-5, atol=1e-9)
    else:
        assert np.mean(err <= 1e-4 * 5e-6) >= 0.98
        assert np.mean(np.abs(dl - dref) <= 1e-3 * np.abs(dref) + 1e-8) > 0.97


def test_oracle_mesh_walk_stays_inside_a_closed_surface():
    """A short reflecting walk of the oracle inside the closed icosphere: no walker leaves it (the
    bounce, nudge and leak guard of the restatement keep every walker in), and the walk is
    deterministic walker by walker."""
    from dmipy_sim_gb300.mesh import icosphere
    V, F = icosphere(4e-6, 2)
    g = O.mesh_geom(V, F)
    rng = np.random.default_rng(4)
    d = rng.normal(size=(256, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r0 = (d * 3.2e-6 * rng.uniform(0, 1, (256, 1)) ** (1 / 3)).astype(np.float32)
    G = np.zeros((2, 40, 3), np.float32)
    G[0, :20, 0], G[0, 20:, 0] = 0.05, -0.05
    G[1, :20, 2], G[1, 20:, 2] = 0.05, -0.05
    kw = dict(n_walkers=256, G=G, dt=1e-4, sub_steps=4, phase_per_substep=True, seed=3, r0=r0,
              want_walkers=True, n_threads=2)
    a = O.walk(g, **kw)
    b = O.walk(g, **kw)
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["phi"], b["phi"])
    rad = np.linalg.norm(a["pos"].astype(np.float64), axis=1)
    assert rad.max() < 4e-6 and np.all(np.isfinite(a["phi"]))
    assert np.max(np.abs(a["pos"] - r0)) > 1e-7           # the walkers moved


@pytest.mark.parametrize("tag", ["perm", "refl"])
@pytest.mark.parametrize("fp64", [False, True])
def test_oracle_myelin_step_matches_reference(kat, tag, fp64):
    """make_myelin_step_fn (physics.py:420-680), one step per case with the direction and Powles
    uniforms the reference drew: FP32 restatement bit for bit (end point, compartment, weight),
    FP64 twin to FP32 rounding."""
    kw = (2e-3, 1e-3) if tag == "perm" else (None, None)
    g = O.myelin_geom(2e-6, 2.6e-6, (2e-9, 0.8e-9, 2.5e-9), 1e-4, kw[0], kw[1],
                      (0.08, 0.012, 0.07), (1.0, 0.4, 1.0))
    k = f"my_{tag}"
    r, comp, unit, u = kat[k + "_r"], kat[k + "_comp"], kat[k + "_unit"], kat[k + "_u"]
    ref, cref, dref, chi = kat[k + "_out"], kat[k + "_comp_out"], kat[k + "_dlog"], kat[k + "_chi"]
    out = np.zeros_like(ref)
    co = np.zeros(len(r), int)
    dl = np.zeros(len(r))
    t1 = np.float32(1e-4) * np.float32(1 / 0.9)
    for i in range(len(r)):
        out[i], co[i], t2 = O.myelin_plugin(g, r[i], unit[i], comp[i], u[i][0], u[i][1],
                                            permeate=tag == "perm", fp64=fp64)
        dl[i] = np.float32(-(np.float32(t2) * chi[i])) - t1 * (1 - chi[i])
    if tag == "perm":
        assert np.sum(comp != cref) > 20        # the cases exercise transmission
    if fp64:
        assert np.mean(co == cref) > 0.99
        ok = co == cref
        assert np.max(np.abs(out[ok] - ref[ok])) < 1e-12
    else:
        np.testing.assert_array_equal(out, ref)
        np.testing.assert_array_equal(co, cref)
        np.testing.assert_array_equal(dl, dref)


@pytest.mark.parametrize("tag", ["perm", "refl"])
@pytest.mark.parametrize("fp64", [False, True])
def test_oracle_packed_myelin_step_matches_reference(kat, tag, fp64):
    """make_packed_myelin_traj_step_fn (physics.py:682-976), one sub-step per case with the
    direction and uniforms the reference drew, on five axons packed by this package's
    pack_myelinated_cylinders (the reference's packer gave the same cell): FP32 bit for bit
    (in-cell end point, compartment, boundary log-weight), FP64 to FP32 rounding."""
    import dmipy_sim_gb300 as d
    from golden.make_golden import pmyelin_substrate
    g = O.geom_from(pmyelin_substrate(d, tag == "perm"), 1e-4)
    k = f"pmy_{tag}"
    r, comp, unit, u = kat[k + "_r"], kat[k + "_comp"], kat[k + "_unit"], kat[k + "_u"]
    ref, cref, dref = kat[k + "_out"], kat[k + "_comp_out"], kat[k + "_dlog"]
    out = np.zeros_like(ref)
    co = np.zeros(len(r), int)
    dl = np.zeros(len(r))
    for i in range(len(r)):
        out[i], co[i], dl[i] = O.pmyelin_plugin(g, r[i], unit[i], comp[i], u[i][0], u[i][1],
                                                permeate=tag == "perm", fp64=fp64)
    if tag == "perm":
        assert np.sum(comp != cref) > 40            # transmissions are exercised
    assert np.sum(comp == 0) > 100 and np.sum(dref != 0) > 50
    if fp64:
        ok = co == cref
        assert ok.mean() > 0.98
        assert np.mean(np.max(np.abs(out[ok] - ref[ok]), axis=1) < 1e-12) > 0.98
    else:
        np.testing.assert_array_equal(out, ref)
        np.testing.assert_array_equal(co, cref)
        np.testing.assert_array_equal(dl, dref)


VALIDATION_CASES = [("box", "reflect"), ("box", "relax"), ("slab", "reflect"), ("slab", "relax"),
                    ("slab", "perm"), ("shs", "reflect"), ("shs", "perm"), ("shc", "reflect"),
                    ("shc", "perm"), ("ell", "reflect"), ("ell", "relax"), ("ell", "perm")]


def _validation_geom(tag):
    L = 6e-6
    if tag == "ell":
        return O.ellipsoid_geom([2e-6, 3e-6, 4.5e-6])
    if tag == "box":
        return O.slab_geom(O.BOX1D, L)
    if tag == "slab":
        return O.slab_geom(O.SLAB, L)
    return O.shell_geom(2e-6, 4e-6, cylinder=tag == "shc")


@pytest.mark.parametrize("tag,mode", VALIDATION_CASES)
def test_oracle_validation_geometries_match_reference(kat, tag, mode):
    """Box1D, PermeableSlab1D, PermeableShell (sphere, cylinder), Ellipsoid plug-in calls of the
    reference:
    end points to the last bit or a few ulps (the reflected point of a sphere shell can differ by
    2-3 ulps where the reference's compiled graph orders the FP32 sums differently), log-weights of
    the weighted modes to FP32 rounding."""
    g = _validation_geom(tag)
    wall = {"reflect": O.REFLECT, "relax": O.RELAX, "perm": O.PERMEATE}[mode]
    k = f"pl_{tag}_{mode}"
    r, st, u, ref, dref = kat[k + "_r"], kat[k + "_step"], kat[k + "_u"], kat[k + "_out"], \
        kat[k + "_dlog"]
    out = np.zeros_like(ref)
    dl = np.zeros(len(r))
    for i in range(len(r)):
        out[i], dl[i] = O.plugin(g, wall, r[i], st[i], float(np.float32(500.0)),
                                 float(np.float32(5000.0)), float(u[i]))
    scale = np.maximum(np.max(np.abs(ref), axis=1), 1e-6)
    assert np.all(np.max(np.abs(out - ref), axis=1) <= 4e-7 * scale)
    assert np.mean(np.all(out == ref, axis=1)) > 0.9
    if mode != "reflect":
        assert np.mean(dref != 0) > 0.05
        np.testing.assert_allclose(dl, dref, rtol=1e-5, atol=1e-9)


def _philox_py(seed, walker, stream, j):
    """Philox4x32-10 round function written out from the published description (Salmon et al.,
    SC'11), independent of the C and CUDA implementations."""
    c = [j, walker & 0xFFFFFFFF, walker >> 32, stream]
    k = [seed & 0xFFFFFFFF, seed >> 32]
    for _ in range(10):
        p0 = 0xD2511F53 * c[0]
        p1 = 0xCD9E8D57 * c[2]
        c = [((p1 >> 32) ^ c[1] ^ k[0]) & 0xFFFFFFFF, p1 & 0xFFFFFFFF,
             ((p0 >> 32) ^ c[3] ^ k[1]) & 0xFFFFFFFF, p0 & 0xFFFFFFFF]
        k = [(k[0] + 0x9E3779B9) & 0xFFFFFFFF, (k[1] + 0xBB67AE85) & 0xFFFFFFFF]
    return c


def test_philox_stream_contract():
    rng = np.random.default_rng(5)
    for _ in range(200):
        seed = int(rng.integers(0, 2**63))
        w = int(rng.integers(0, 2**40))
        st = int(rng.integers(0, 4))
        j = int(rng.integers(0, 2**32))
        assert O.philox(seed, w, st, j) == _philox_py(seed, w, st, j)


def test_philox_uniforms_are_uniform():
    u = np.array([O.philox(7, w, 0, j) for w in range(64) for j in range(64)], np.uint64).ravel()
    x = (u >> 8).astype(np.float64) / 2**24
    counts, _ = np.histogram(x, bins=16, range=(0, 1))
    chi2 = np.sum((counts - len(x) / 16) ** 2 / (len(x) / 16))
    assert chi2 < 45.0        # 15 dof, p ~ 1e-4
    assert abs(np.corrcoef(x[:-1], x[1:])[0, 1]) < 0.03
