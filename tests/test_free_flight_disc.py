"""The free-flight rule of the packed-cylinder walk (csrc/walk_ff.cuh), restated in numpy on the CPU.

After a wall scan that meets no wall, the kernel lets the walker step without scanning while its
displacement stays inside a disc about the scanned step's end point, of radius
    min(end point's distance to each wall the start cell lists,
        start point's distance to the cell's edge + the list's reach - the step) - 16 nudges.
Two properties make the skipped steps exact, and both are checked here on the benchmark lattice
(reflecting, at the benchmark's sub-step; with the much longer steps of one sub-step per sample;
and permeable with its 36 nm sub-steps, walkers inside cylinders included):
  * the radius never exceeds the true distance to the nearest wall of any periodic image of any
    cylinder (float64, brute force over every object);
  * a walk of random steps that stays inside the disc never makes the FP32 wall test of a scan
    (root and end-point containment, as packed_cyl_step computes them from the cell list of the
    step's own start point) report a wall, so the scan would have returned x + step.
"""
import numpy as np
import pytest

import dmipy_sim_gb300 as d
from dmipy_sim_gb300 import core
from dmipy_sim_gb300.geometries import build_cell_list

f32 = np.float32
D = 2e-9


def _setup(S_from, permeable):
    radii, centers, L = d.lattice_cylinders(16, 0.6, 2e-6, 0.5e-6, seed=0)
    geom = d.PackedCylinders(radii, centers, L, permeability=2e-5 if permeable else None)
    dt = 0.05 / 999
    if S_from == "one":
        S = 1
    else:
        S = {"replay": core.replay_sub_steps, "fused": core.fused_sub_steps}[S_from](geom, D, dt)
    step = float(f32(np.sqrt(6 * D * dt / S)))
    reach = step * 1.05 + 8 * float(geom._nudge)
    n, start, cand, _ = build_cell_list(geom._centers_np, geom._radii_np, geom._L_float, reach)
    c0 = centers - L * np.floor(centers / L + 0.5)
    shifts = np.array([(i, j) for i in (-1, 0, 1) for j in (-1, 0, 1)], np.float64)
    imgs = (c0[None] + L * shifts[:, None]).reshape(-1, 2)
    return dict(L=L, halfL=f32(L / 2), h=f32(L / n), inv_h=f32(n / L), n=n, start=start,
                cand=cand, reach=f32(reach), step=step, tol=f32(16 * float(geom._nudge)),
                eps=f32(geom._eps_detect), imgs=imgs, rimg=np.tile(radii, 9),
                permeable=permeable)


def _cell(g, v):
    return np.clip(np.floor((v + g["halfL"]) * g["inv_h"]).astype(np.int64), 0, g["n"] - 1)


def _fold(g, v):
    v = v.copy()
    v[v >= g["halfL"]] -= f32(g["L"])
    v[v < -g["halfL"]] += f32(g["L"])
    return v


def _cands(g, x, y):
    c = _cell(g, y) * g["n"] + _cell(g, x)
    kb, ke = g["start"][c].astype(np.int64), g["start"][c + 1].astype(np.int64)
    kmax = int((ke - kb).max())
    ks = kb[:, None] + np.arange(kmax)[None]
    ok = ks < ke[:, None]
    C = g["cand"][np.minimum(ks, len(g["cand"]) - 1)]
    return C, ok


def _wall_hit(g, x, y, sx, sy):
    """The scan's FP32 verdict (any valid root, any contained end point) for each step."""
    C, ok = _cands(g, x, y)
    lxy = np.sqrt(sx * sx + sy * sy).astype(f32)
    dx = (sx / np.maximum(lxy, f32(1e-30))).astype(f32)
    dy = (sy / np.maximum(lxy, f32(1e-30))).astype(f32)
    ex, ey = (x + sx).astype(f32), (y + sy).astype(f32)
    R2 = C[..., 3] * C[..., 3]
    fx, fy = ex[:, None] - C[..., 0], ey[:, None] - C[..., 1]
    end_in = ok & (fx * fx + fy * fy < R2) & (not g["permeable"])
    qx, qy = x[:, None] - C[..., 0], y[:, None] - C[..., 1]
    dp = dx[:, None] * qx + dy[:, None] * qy
    q2 = qx * qx + qy * qy
    disc = dp * dp - (q2 - R2)
    ins = g["permeable"] & (q2 < R2)
    sq = np.sqrt(np.maximum(disc, 0)).astype(f32)
    t = np.where(ins, -dp + sq, -dp - sq)
    valid = ok & (ins | (dp < 0)) & (disc > 0) & (t > g["eps"]) & (t < lxy[:, None]) & \
        (lxy[:, None] > 0)
    return np.any(valid | end_in, axis=1)


def _disc(g, x, y, sx, sy):
    """The kernel's disc radius about the end point of the (wall-free) step from (x, y)."""
    C, ok = _cands(g, x, y)
    ex, ey = (x + sx).astype(f32), (y + sy).astype(f32)
    fx, fy = ex[:, None] - C[..., 0], ey[:, None] - C[..., 1]
    f2 = fx * fx + fy * fy
    dmin = np.min(np.where(ok, np.abs(np.sqrt(f2).astype(f32) - C[..., 3]), np.inf), axis=1)
    inside = np.any(ok & (f2 < C[..., 3] ** 2), axis=1)
    cx, cy = _cell(g, x), _cell(g, y)
    xlo = -g["halfL"] + cx.astype(f32) * g["h"]
    ylo = -g["halfL"] + cy.astype(f32) * g["h"]
    dbox = np.minimum(np.minimum(x - xlo, xlo + g["h"] - x), np.minimum(y - ylo, ylo + g["h"] - y))
    lxy = np.sqrt(sx * sx + sy * sy).astype(f32)
    rs = (np.minimum(dmin, dbox + g["reach"] - lxy) - g["tol"]).astype(f32)
    if not g["permeable"]:
        rs = np.where(inside, f32(-1), rs)
    return rs


def _steps(g, rng, n):
    cz = f32(1) - f32(2) * rng.random(n).astype(f32)
    st = np.sqrt(np.maximum(f32(0), f32(1) - cz * cz)).astype(f32)
    ph = f32(np.pi) * (f32(2) * rng.random(n).astype(f32) - f32(1))
    return (f32(g["step"]) * st * np.cos(ph)).astype(f32), \
        (f32(g["step"]) * st * np.sin(ph)).astype(f32)


def _true_wall_distance(g, x, y):
    q = np.stack([x, y], 1).astype(np.float64)[:, None, :] - g["imgs"][None]
    return np.min(np.abs(np.sqrt((q ** 2).sum(-1)) - g["rimg"][None]), axis=1)


@pytest.mark.parametrize("S_from,permeable", [("replay", False), ("one", False),
                                              ("fused", True)])
def test_free_flight_disc_is_wall_free(S_from, permeable):
    g = _setup(S_from, permeable)
    rng = np.random.default_rng(3)
    n = 20_000
    x = ((rng.random(n) - 0.5) * g["L"]).astype(f32)
    y = ((rng.random(n) - 0.5) * g["L"]).astype(f32)
    if not permeable:   # reflecting walkers live outside the cylinders
        keep = _true_wall_distance(g, x, y) > 0
        q = np.stack([x, y], 1).astype(np.float64)[:, None, :] - g["imgs"][None]
        keep &= np.all(np.sqrt((q ** 2).sum(-1)) > g["rimg"][None], axis=1)
        x, y = x[keep], y[keep]
    sx, sy = _steps(g, rng, len(x))
    free = ~_wall_hit(g, x, y, sx, sy)
    x, y, sx, sy = x[free], y[free], sx[free], sy[free]
    rs = _disc(g, x, y, sx, sy)
    ex, ey = _fold(g, (x + sx).astype(f32)), _fold(g, (y + sy).astype(f32))
    # 1. the disc never reaches past the nearest wall of any object image
    has = rs > 0
    assert has.mean() > 0.3
    dtrue = _true_wall_distance(g, ex[has], ey[has])
    assert np.all(rs[has] <= dtrue), float(np.max(rs[has] - dtrue))
    # 2. steps that keep the walker inside the disc never meet a wall in the FP32 scan
    px, py, r = ex[has], ey[has], rs[has]
    adx = np.zeros_like(px)
    ady = np.zeros_like(py)
    checked = 0
    for _ in range(12):
        tx, ty = _steps(g, rng, len(px))
        nx, ny = (adx + tx).astype(f32), (ady + ty).astype(f32)
        inside = nx * nx + ny * ny < r * r
        if not inside.any():
            break
        hit = _wall_hit(g, px[inside], py[inside], tx[inside], ty[inside])
        assert not hit.any(), int(hit.sum())
        checked += int(inside.sum())
        px = np.where(inside, _fold(g, (px + tx).astype(f32)), px)
        py = np.where(inside, _fold(g, (py + ty).astype(f32)), py)
        adx, ady = np.where(inside, nx, adx), np.where(inside, ny, ady)
    assert checked > 1000
