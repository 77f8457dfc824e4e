"""Vectorised NumPy mirror of a baked hair mesh, for the baker's quality tests.

* ``styled_positions``: HairMesh::styled_position (src/mesh.rs:98-175), the
  reference's CPU mirror of the rasterizer's strand generation, for many
  (bundle, u, v, w) at once in float32 (tests/test_styled_position.py holds
  the one-point restatement it is checked against);
* ``resample``: equal-arc-length resampling of source strands to 16 points
  (what the reference's baker tests compare reconstructions with,
  src/bake.rs:683-714);
* the three quality measures of the reference's baker tests
  (src/bake.rs:1495-1527, with the helpers at :1553-1789), restated:
  ``max_styled_stray`` (how far a bundle's uniform uv fill strays from the
  source strands), ``uncovered_roots`` (roots outside every root quad) and
  ``max_reconstruction_error`` (how well the cage of the bundle holding a
  root reproduces that strand).  Distances to the source strands are taken to
  points sampled along them at most 0.5 units apart, which overestimates the
  distance to the polyline by at most 0.25 units.
"""
from __future__ import annotations

import numpy as np

F = np.float32
LAYERS, SU, SV, SW = 16, 8, 8, 16


def _cage(mesh):
    off = mesh.bundles["layer_offset"].astype(np.int64)
    idx = off[:, None] + np.arange(LAYERS * 4)[None, :]
    return mesh.layers["pos_ao"][idx, :3].astype(F).reshape(-1, LAYERS, 4, 3)


def _style(mesh):
    off = mesh.bundles["style_offset"].astype(np.int64)
    idx = off[:, None] + np.arange(SW * SV * SU)[None, :]
    return mesh.style[idx, :3].astype(F).reshape(-1, SW, SV, SU, 3)


def _bilinear(q, u, v):
    one = F(1.0)
    u, v = u[:, None], v[:, None]
    return (((q[:, 0] * (one - u)) * (one - v) + (q[:, 1] * u) * (one - v)) + (q[:, 2] * (one - u)) * v) + (q[:, 3] * u) * v


def styled_positions(mesh, bundle, u, v, w, cage=None, style=None) -> np.ndarray:
    """styled_position for arrays of bundle indices and (u, v, w) -> float32 [n, 3]."""
    cage = _cage(mesh) if cage is None else cage
    style = _style(mesh) if style is None else style
    b = np.asarray(bundle, np.int64)
    u, v, w = (np.asarray(x, F) for x in (u, v, w))
    lf = np.clip(w, F(0), F(1)) * F(LAYERS - 1)
    i0 = np.minimum(np.floor(lf).astype(np.int64), LAYERS - 1)
    i1 = np.minimum(i0 + 1, LAYERS - 1)
    t = (lf - i0.astype(F))[:, None]

    def point(layer):
        return _bilinear(cage[b, np.clip(layer, 0, LAYERS - 1)], u, v)

    def tangent(layer):
        first, last = layer == 0, layer >= LAYERS - 1
        nxt, prv, cur = point(layer + 1), point(layer - 1), point(layer)
        d = np.where(first[:, None], nxt - cur, np.where(last[:, None], cur - prv, nxt - prv))
        n = np.sqrt(np.sum(d * d, axis=1, dtype=F)).astype(F)
        scale = np.where(first | last, n, n * F(0.5))
        ok = n > F(0)
        dirn = np.where(ok[:, None], d / np.where(ok, n, F(1))[:, None], np.array([0, 1, 0], F))
        return dirn * np.maximum(scale, F(1e-4))[:, None]

    p0, p1, m0, m1 = point(i0), point(i1), tangent(i0), tangent(i1)
    t2 = t * t
    t3 = t2 * t
    base = ((p0 * ((F(2) * t3 - F(3) * t2) + F(1)) + m0 * ((t3 - F(2) * t2) + t)) + p1 * (F(-2) * t3 + F(3) * t2)) \
        + m1 * (t3 - t2)
    # trilinear style (glam lerp: a + (b - a) t)
    uu = np.clip(u, F(0), F(1)) * F(SU - 1)
    vv = np.clip(v, F(0), F(1)) * F(SV - 1)
    ww = np.clip(w, F(0), F(1)) * F(SW - 1)
    u0 = np.floor(uu).astype(np.int64)
    v0 = np.floor(vv).astype(np.int64)
    w0 = np.floor(ww).astype(np.int64)
    u1, v1, w1 = np.minimum(u0 + 1, SU - 1), np.minimum(v0 + 1, SV - 1), np.minimum(w0 + 1, SW - 1)
    tu, tv, tw = ((uu - u0.astype(F))[:, None], (vv - v0.astype(F))[:, None], (ww - w0.astype(F))[:, None])

    def at(iu, iv, iw):
        return style[b, iw, iv, iu]

    def lerp(a, c, s):
        return a + (c - a) * s

    c00 = lerp(at(u0, v0, w0), at(u1, v0, w0), tu)
    c01 = lerp(at(u0, v1, w0), at(u1, v1, w0), tu)
    c10 = lerp(at(u0, v0, w1), at(u1, v0, w1), tu)
    c11 = lerp(at(u0, v1, w1), at(u1, v1, w1), tu)
    return base + lerp(lerp(c00, c01, tv), lerp(c10, c11, tv), tw)


def resample(points, first, count) -> tuple[np.ndarray, np.ndarray]:
    """16 points at equal arc length of every strand with >= 2 points and
    length >= 1e-5 (src/bake.rs:683-714 semantics).  Returns (strand indices,
    float32 [n, 16, 3])."""
    pts = np.asarray(points, F)
    first = np.asarray(first, np.int64)
    count = np.asarray(count, np.int64)
    keep = np.flatnonzero(count >= 2)
    out_idx, out = [], []
    for s in keep:
        p = pts[first[s]:first[s] + count[s]]
        seg = np.sqrt(np.sum((p[1:] - p[:-1]) ** 2, axis=1, dtype=F)).astype(F)
        cum = np.concatenate([[F(0)], np.cumsum(seg, dtype=F)]).astype(F)
        length = cum[-1]
        if length < 1e-5:
            continue
        target = (length * np.arange(LAYERS, dtype=F) / F(LAYERS - 1)).astype(F)
        idx = np.clip(np.searchsorted(cum, target, side="left"), 1, len(p) - 1)
        span = np.maximum(cum[idx] - cum[idx - 1], F(1e-6))
        t = np.clip((target - cum[idx - 1]) / span, F(0), F(1))[:, None]
        out.append(p[idx - 1] + (p[idx] - p[idx - 1]) * t)
        out_idx.append(s)
    return np.asarray(out_idx, np.int64), np.asarray(out, F).reshape(-1, LAYERS, 3)


def _source_tree(points, first, count, spacing=0.5):
    from scipy.spatial import cKDTree

    pts = np.asarray(points, np.float64)
    first = np.asarray(first, np.int64)
    count = np.asarray(count, np.int64)
    # segments i -> i + 1 inside each strand
    starts = np.concatenate([np.arange(f, f + c - 1) for f, c in zip(first, count) if c >= 2]) \
        if np.any(count >= 2) else np.zeros(0, np.int64)
    p0, p1 = pts[starts], pts[starts + 1]
    d = np.sqrt(np.sum((p1 - p0) ** 2, axis=1))
    k = np.maximum(1, np.ceil(d / spacing).astype(np.int64))
    seg = np.repeat(np.arange(len(starts)), k)
    t = np.arange(len(seg)) - np.repeat(np.cumsum(k) - k, k)
    samples = p0[seg] + (p1[seg] - p0[seg]) * (t / np.repeat(k, k))[:, None]
    ends = pts[first[count >= 1] + np.maximum(count[count >= 1] - 1, 0)]
    return cKDTree(np.concatenate([samples, ends]))


def max_styled_stray(mesh, points, first, count) -> float:
    """Largest distance from a bundle's uv fill (5 x 5 grid, 31 heights) to
    the source strands (src/bake.rs:1553-1594)."""
    tree = _source_tree(points, first, count)
    g = np.array([0.0, 0.25, 0.5, 0.75, 1.0], F)
    uu, vv, ww = np.meshgrid(g, g, np.arange(2 * LAYERS - 1, dtype=F) / F(2 * LAYERS - 2), indexing="ij")
    nb = mesh.bundle_count
    b = np.repeat(np.arange(nb), uu.size)
    pos = styled_positions(mesh, b, np.tile(uu.ravel(), nb), np.tile(vv.ravel(), nb), np.tile(ww.ravel(), nb))
    d, _ = tree.query(pos.astype(np.float64))
    return float(d.max()) if len(d) else 0.0


def _quad_uv(q, p):
    """HairMesh::quad_uv for parallelogram quads q [n, 4, 3] and points p [n, 3]."""
    eu, ev, rel = q[:, 1] - q[:, 0], q[:, 2] - q[:, 0], p - q[:, 0]
    nrm = np.cross(eu, ev)
    den = np.sum(nrm * nrm, axis=1)
    ok = den >= 1e-12
    den = np.where(ok, den, 1.0)
    u = np.sum(np.cross(rel, ev) * nrm, axis=1) / den
    v = np.sum(np.cross(eu, rel) * nrm, axis=1) / den
    return np.where(ok, u, 0.5), np.where(ok, v, 0.5)


def _plane_distance(q, p):
    nrm = np.cross(q[:, 1] - q[:, 0], q[:, 2] - q[:, 0])
    ln = np.sqrt(np.sum(nrm * nrm, axis=1))
    far = np.sqrt(np.sum((p - q[:, 0]) ** 2, axis=1))
    return np.where(ln < 1e-8, far, np.sum((p - q[:, 0]) * nrm, axis=1) / np.where(ln < 1e-8, 1.0, ln))


def _root_candidates(mesh, roots):
    """(strand, bundle) pairs whose root quad may hold the root: bundles whose
    root-quad box, widened by 8, contains it."""
    from scipy.spatial import cKDTree

    q0 = _cage(mesh)[:, 0].astype(np.float64)
    centre = q0.mean(axis=1)
    reach = np.sqrt(np.max(np.sum((q0 - centre[:, None]) ** 2, axis=2), axis=1)) + 8.0
    tree = cKDTree(centre)
    lists = tree.query_ball_point(roots, r=float(reach.max()) + 1e-3)
    s = np.repeat(np.arange(len(roots)), [len(x) for x in lists])
    b = np.concatenate([np.asarray(x, np.int64) for x in lists]) if len(lists) else np.zeros(0, np.int64)
    keep = np.sqrt(np.sum((roots[s] - centre[b]) ** 2, axis=1)) <= reach[b]
    return s[keep], b[keep], q0


def uncovered_roots(mesh, roots) -> np.ndarray:
    """Roots outside every root quad: uv outside [0, 1]^2 or more than 8 from
    the quad's plane (src/bake.rs:1596-1614)."""
    roots = np.asarray(roots, np.float64)
    s, b, q0 = _root_candidates(mesh, roots)
    u, v = _quad_uv(q0[b], roots[s])
    inside = (u >= 0) & (u <= 1) & (v >= 0) & (v <= 1) & (np.abs(_plane_distance(q0[b], roots[s])) < 8.0)
    covered = np.zeros(len(roots), bool)
    covered[s[inside]] = True
    return np.flatnonzero(~covered)


def max_reconstruction_error(mesh, resampled) -> float:
    """For every resampled strand, the best over the bundles whose root quad
    holds its root of the largest distance between styled_position at the
    root's uv and its 16 points; the worst of these (src/bake.rs:1616-1660)."""
    roots = resampled[:, 0].astype(np.float64)
    s, b, q0 = _root_candidates(mesh, roots)
    u, v = _quad_uv(q0[b], roots[s])
    ok = (u >= 0) & (u <= 1) & (v >= 0) & (v <= 1) & (np.abs(_plane_distance(q0[b], roots[s])) <= 8.0)
    s, b, u, v = s[ok], b[ok], u[ok].astype(F), v[ok].astype(F)
    cage, style = _cage(mesh), _style(mesh)
    worst = np.zeros(len(s), np.float64)
    for layer in range(LAYERS):
        w = np.full(len(s), F(layer) / F(LAYERS - 1), F)
        p = styled_positions(mesh, b, u, v, w, cage, style)
        worst = np.maximum(worst, np.sqrt(np.sum((p - resampled[s, layer]) ** 2, axis=1)))
    best = np.full(len(roots), 1.0e6)
    np.minimum.at(best, s, worst)
    return float(best.max()) if len(best) else 0.0
