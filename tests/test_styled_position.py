"""Strand generation pinned to the reference's own CPU mirror of it.

HairMesh::styled_position (src/mesh.rs:98-175, documented there as "matching
the rasterizer") evaluates a strand at (uv, w) from the bundle cage: bilinear
layer points, finite-difference layer tangents, a Hermite segment between
layers, plus the trilinear style residual.  It is restated below in NumPy
float32, in the operation order of mesh.rs, independently of the oracle's C
restatement of raster.wgsl.  The control points the oracle generates
(oracle_strand_points) and the GPU strand cache (hg_generate,
HG_GBUF_STRAND_CACHE) must agree with it at every control point, within a
tolerance of 2e-6 of the largest coordinate: mesh.rs and raster.wgsl round
the same formulas in a slightly different order (e.g. bilinear weights
multiplied in sequence, not as products), so the two differ by a few ulps
(at most 2.8e-7 of the largest coordinate on these grooms).
"""
import numpy as np
import pytest

import oracle
from bevy_hair_gb300 import abi, configs

F = np.float32
LAYERS, SU, SV, SW = 16, 8, 8, 16


def pcg(v: int) -> int:
    """common.wgsl's pcg hash on u32 (wrapping arithmetic)."""
    state = (v * 747796405 + 2891336453) & 0xFFFFFFFF
    word = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & 0xFFFFFFFF
    return ((word >> 22) ^ word) & 0xFFFFFFFF


def strand_uv(bundle: int, strand: int) -> tuple[np.float32, np.float32]:
    """The uv the raster gives strand `strand` of `bundle` (raster.wgsl:233)."""
    seed = (strand ^ ((bundle * 0x85EBCA6B) & 0xFFFFFFFF)) & 0xFFFFFFFF
    a = pcg(seed)
    b = pcg(a ^ 0x9E3779B9)
    s = F(1.0 / 4294967296.0)
    return F(a) * s, F(b) * s


def _corners(mesh, bundle, layer):
    off = int(mesh.bundles["layer_offset"][bundle]) + layer * 4
    return mesh.layers["pos_ao"][off:off + 4, :3].astype(F)


def _bilinear(q, u, v):
    # mesh.rs bilinear: quad[0] * (1 - u) * (1 - v) + quad[1] * u * (1 - v) + ...
    one = F(1.0)
    return (((q[0] * (one - u)) * (one - v) + (q[1] * u) * (one - v)) + (q[2] * (one - u)) * v) + (q[3] * u) * v


def _normalize_or_y(d):
    n = np.sqrt(F(np.dot(d, d)))
    if not np.isfinite(n) or n <= F(0.0) or not np.isfinite(F(1.0) / n):
        return np.array([0.0, 1.0, 0.0], F)
    return d * (F(1.0) / n)


def _layer_tangent(mesh, bundle, layer, u, v):
    curr = _bilinear(_corners(mesh, bundle, layer), u, v)
    prev = _bilinear(_corners(mesh, bundle, max(layer - 1, 0)), u, v)
    nxt = _bilinear(_corners(mesh, bundle, min(layer + 1, LAYERS - 1)), u, v)
    if layer == 0:
        delta, scale = nxt - curr, None
        scale = np.sqrt(F(np.dot(delta, delta)))
    elif layer + 1 >= LAYERS:
        delta = curr - prev
        scale = np.sqrt(F(np.dot(delta, delta)))
    else:
        delta = nxt - prev
        scale = np.sqrt(F(np.dot(delta, delta))) * F(0.5)
    return _normalize_or_y(delta) * max(scale, F(1e-4))


def _hermite(p0, p1, m0, m1, t):
    t2 = t * t
    t3 = t2 * t
    return ((p0 * ((F(2.0) * t3 - F(3.0) * t2) + F(1.0)) + m0 * ((t3 - F(2.0) * t2) + t))
            + p1 * (F(-2.0) * t3 + F(3.0) * t2)) + m1 * (t3 - t2)


def _sample_style(mesh, bundle, u, v, w):
    off = int(mesh.bundles["style_offset"][bundle])
    style = mesh.style

    def clamp01(x):
        return min(max(x, F(0.0)), F(1.0))

    uu, vv, ww = clamp01(u) * F(SU - 1), clamp01(v) * F(SV - 1), clamp01(w) * F(SW - 1)
    u0, v0, w0 = int(np.floor(uu)), int(np.floor(vv)), int(np.floor(ww))
    u1, v1, w1 = min(u0 + 1, SU - 1), min(v0 + 1, SV - 1), min(w0 + 1, SW - 1)
    tu, tv, tw = uu - F(u0), vv - F(v0), ww - F(w0)

    def at(iu, iv, iw):
        return style[off + (iw * SV + iv) * SU + iu, :3].astype(F)

    def lerp(a, b, t):  # glam Vec3::lerp: a + (b - a) * t
        return a + (b - a) * t

    c00 = lerp(at(u0, v0, w0), at(u1, v0, w0), tu)
    c01 = lerp(at(u0, v1, w0), at(u1, v1, w0), tu)
    c10 = lerp(at(u0, v0, w1), at(u1, v0, w1), tu)
    c11 = lerp(at(u0, v1, w1), at(u1, v1, w1), tu)
    return lerp(lerp(c00, c01, tv), lerp(c10, c11, tv), tw)


def styled_position(mesh, bundle: int, u, v, w) -> np.ndarray:
    """HairMesh::styled_position (src/mesh.rs:98-110) in float32."""
    layers_f = min(max(w, F(0.0)), F(1.0)) * F(LAYERS - 1)
    i0 = min(int(np.floor(layers_f)), LAYERS - 1)
    i1 = min(i0 + 1, LAYERS - 1)
    t = layers_f - F(i0)
    p0 = _bilinear(_corners(mesh, bundle, i0), u, v)
    p1 = _bilinear(_corners(mesh, bundle, i1), u, v)
    m0 = _layer_tangent(mesh, bundle, i0, u, v)
    m1 = _layer_tangent(mesh, bundle, i1, u, v)
    return _hermite(p0, p1, m0, m1, t) + _sample_style(mesh, bundle, u, v, w)


def _oracle_points(mesh, bundle, strand, ncp):
    ref = np.zeros(1, abi.STRAND_REF)
    ref[0] = (bundle, strand, int(mesh.bundles["strand_count"][bundle]), ncp)
    pos = np.zeros((128, 4), F)
    tan = np.zeros((128, 4), F)
    uvw = np.zeros((128, 4), F)
    n = oracle.lib().oracle_strand_points(abi.ptr(np.ascontiguousarray(mesh.bundles)),
                                          abi.ptr(np.ascontiguousarray(mesh.layers)),
                                          abi.ptr(np.ascontiguousarray(mesh.style, dtype=F)), abi.ptr(ref),
                                          abi.ptr(pos), abi.ptr(tan), abi.ptr(uvw))
    assert n == ncp
    return pos[:ncp, :3]


def _mirror(mesh, bundle, strand, ncp):
    u, v = strand_uv(bundle, strand)
    den = F(max(ncp - 1, 1))
    return np.stack([styled_position(mesh, bundle, u, v, F(i) / den) for i in range(ncp)])


def _sample(mesh, k, seed):
    rng = np.random.default_rng(seed)
    bundles = rng.choice(mesh.bundle_count, size=min(k, mesh.bundle_count), replace=False)
    out = []
    for b in bundles:
        n = int(mesh.bundles["strand_count"][b])
        if n:
            out.append((int(b), int(rng.integers(n))))
    return out


def _tol(p):
    # observed: at most 2.8e-7 of the largest coordinate (a few ulps)
    return 2e-6 * float(np.abs(p).max()) + 1e-6


@pytest.mark.parametrize("name", ["config1", "config2", "config3"])
@pytest.mark.parametrize("ncp", [9, 17, 33, 65, 127])
def test_oracle_strand_points_follow_styled_position(name, ncp):
    sc = getattr(configs, name)(scale=0.01)
    for b, s in _sample(sc.mesh, 12, 7 + ncp):
        want = _mirror(sc.mesh, b, s, ncp)
        got = _oracle_points(sc.mesh, b, s, ncp)
        np.testing.assert_allclose(got, want, rtol=0, atol=_tol(want), err_msg=f"bundle {b} strand {s}")


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["config1", "config2", "config3"])
def test_gpu_strand_cache_follows_styled_position(name):
    """hg_generate's world-space control points (65 per strand) against
    styled_position mapped through world_from_model."""
    from bevy_hair_gb300.pipeline import HairRenderer

    sc = getattr(configs, name)(scale=0.02)
    cam, _ = sc.params()
    wfm = np.asarray(cam["world_from_model"], np.float64).reshape(4, 4).T  # column-major
    with HairRenderer(0) as r:
        g = r.upload(sc.mesh)
        r.generate(g, cam)
        assert r.synchronize() == 0
        cache = g.read(abi.SLOT_CAMERA, abi.GBUF_STRAND_CACHE)
        g.close()
    base = np.concatenate([[0], np.cumsum(sc.mesh.bundles["strand_count"].astype(np.int64))])
    assert cache.shape == (base[-1], 130, 4)
    for b, s in _sample(sc.mesh, 16, 11):
        model = _mirror(sc.mesh, b, s, 65).astype(np.float64)
        world = (np.c_[model, np.ones(65)] @ wfm.T)[:, :3]
        got = cache[base[b] + s, :65, :3]
        np.testing.assert_allclose(got, world, rtol=0, atol=_tol(world), err_msg=f"bundle {b} strand {s}")
