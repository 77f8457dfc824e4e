"""Groom data: baked hair meshes and seeded synthetic strand grooms.

``HairMesh`` holds the three buffers ``GpuGroom::upload`` sends to the GPU
(``src/render/pass.rs:98-167``; layout ``src/mesh.rs:16-41``): bundles
(GpuBundle), cage corners (GpuLayer, 64 per bundle, layer-major, corner order
c00 c10 c01 c11) and the 8x8x16 style volume per bundle.

Synthetic grooms are generated in millimetres (1 unit = 1 mm) so the baker's
absolute thresholds (``src/bake.rs:17-31``) mean what they mean for the
reference's real grooms, whose extent is about 120 units.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi

F = np.float32


@dataclass
class HairMesh:
    bundles: np.ndarray  # GPU_BUNDLE
    layers: np.ndarray   # GPU_LAYER
    style: np.ndarray    # float32 [n, 4]
    bounds_min: np.ndarray
    bounds_max: np.ndarray

    @property
    def bundle_count(self) -> int:
        return int(len(self.bundles))

    def strand_count(self) -> int:
        return int(self.bundles["strand_count"].sum(dtype=np.uint64)) if len(self.bundles) else 0


@dataclass
class Strands:
    """Explicit strands: points float32 [n, 3]; strand i spans first[i] .. first[i]+count[i]."""
    points: np.ndarray
    first: np.ndarray
    count: np.ndarray

    @property
    def strand_count(self) -> int:
        return int(len(self.first))


@dataclass
class Scalp:
    """Triangle mesh the strands grow from: vertices float32 [n, 3], triangles uint32 [m, 3]."""
    vertices: np.ndarray
    triangles: np.ndarray


def parse_obj(text: str) -> Scalp:
    """Positions and faces of a Wavefront OBJ file (``v`` and ``f`` records;
    face corners ``i``, ``i/t`` or ``i/t/n`` with 1-based or negative indices;
    polygons split into triangle fans), the head mesh the reference's example
    bakes against (src/obj.rs:12-44)."""
    verts: list[tuple[float, float, float]] = []
    tris: list[tuple[int, int, int]] = []
    for raw in text.splitlines():
        line = raw.strip()
        if line.startswith("v "):
            parts = line[2:].split()
            xyz = []
            for k in range(3):
                try:
                    xyz.append(float(parts[k]))
                except (IndexError, ValueError):
                    xyz.append(0.0)
            verts.append((xyz[0], xyz[1], xyz[2]))
        elif line.startswith("f "):
            corners = []
            for c in line[2:].split():
                try:
                    i = int(c.split("/")[0])
                except ValueError:
                    continue
                if i > 0:
                    corners.append(i - 1)
                elif i < 0:
                    corners.append(len(verts) + i)
            for k in range(1, len(corners) - 1):
                tris.append((corners[0], corners[k], corners[k + 1]))
    return Scalp(np.asarray(verts, dtype=F).reshape(-1, 3), np.asarray(tris, dtype=np.uint32).reshape(-1, 3))


def bake(strands: Strands, ambient_occlusion: bool = True, scalp: Scalp | None = None) -> HairMesh:
    """Bake explicit strands (and optionally the scalp mesh they grow from)
    into bundle cages with the native baker (the interface of
    bake_hair_mesh_with_scalp, src/bake.rs:89-213; include/hairgb_bake.h)."""
    lib = abi.load_bake()
    pts = np.ascontiguousarray(strands.points, dtype=F)
    first = np.ascontiguousarray(strands.first, dtype=np.uint32)
    count = np.ascontiguousarray(strands.count, dtype=np.uint32)
    flags = 1 if ambient_occlusion else 0
    if scalp is not None and len(scalp.triangles):
        sv = np.ascontiguousarray(scalp.vertices, dtype=F)
        si = np.ascontiguousarray(scalp.triangles, dtype=np.uint32)
        r = lib.hg_bake_scalp(pts.ctypes.data, len(pts), first.ctypes.data, count.ctypes.data, len(first),
                              sv.ctypes.data, len(sv), si.ctypes.data, si.size, flags)
    else:
        r = lib.hg_bake(pts.ctypes.data, len(pts), first.ctypes.data, count.ctypes.data, len(first), flags)
    if not r:
        raise ValueError("the baker rejected the input (a strand outside the point array or a scalp index "
                         "outside the vertex array)")
    try:
        nb, nl, ns = lib.hg_bake_bundle_count(r), lib.hg_bake_layer_count(r), lib.hg_bake_style_count(r)
        bundles = np.zeros(nb, dtype=abi.GPU_BUNDLE)
        layers = np.zeros(nl, dtype=abi.GPU_LAYER)
        style = np.zeros((ns, 4), dtype=F)
        bounds = np.zeros(6, dtype=F)
        lib.hg_bake_copy(r, bundles.ctypes.data, layers.ctypes.data, style.ctypes.data, bounds.ctypes.data)
    finally:
        lib.hg_bake_free(r)
    return HairMesh(bundles, layers, style, bounds[:3].copy(), bounds[3:].copy())


# ----------------------------------------------------------------- synthetic grooms


def _roots_upper_hemisphere(rng: np.random.Generator, n: int, radius: float) -> np.ndarray:
    """Uniform by area on the upper (+Y) hemisphere: height uniform, azimuth uniform."""
    h = rng.random(n)
    phi = 2.0 * np.pi * rng.random(n)
    r = np.sqrt(np.maximum(1.0 - h * h, 0.0))
    return np.stack([r * np.cos(phi), h, r * np.sin(phi)], axis=1) * radius


def _centerlines(roots: np.ndarray, segments: int, length: float, droop: float) -> np.ndarray:
    """Strand centre lines leaving the sphere along its normal and bending
    toward -Y (gravity): direction(s) = normalize(n + droop * s * (-Y))."""
    n = roots / np.linalg.norm(roots, axis=1, keepdims=True)
    step = length / segments
    pts = np.empty((len(roots), segments + 1, 3))
    pts[:, 0] = roots
    down = np.array([0.0, -1.0, 0.0])
    for k in range(segments):
        s = (k + 0.5) / segments
        d = n + droop * s * down
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        pts[:, k + 1] = pts[:, k] + d * step
    return pts


def _frames(center: np.ndarray):
    """Per-point unit tangent and two normals of the centre lines."""
    t = np.gradient(center, axis=1)
    t /= np.maximum(np.linalg.norm(t, axis=2, keepdims=True), 1e-12)
    ref = np.broadcast_to(np.array([0.0, 0.0, 1.0]), t.shape).copy()
    near = np.abs(np.sum(t * ref, axis=2)) > 0.9
    ref[near] = (1.0, 0.0, 0.0)
    b1 = np.cross(t, ref)
    b1 /= np.maximum(np.linalg.norm(b1, axis=2, keepdims=True), 1e-12)
    b2 = np.cross(t, b1)
    return t, b1, b2


def synthetic_strands(n_strands: int, segments: int, style: str, seed: int, *, radius: float = 100.0,
                      length: float = 300.0, droop: float = 3.0, wave_amp: float = 2.0, wave_period: float = 20.0,
                      helix_radius: float = 4.0, helix_pitch: float = 10.0, helix_jitter: float = 0.2) -> Strands:
    """Seeded groom: roots on the upper hemisphere of a sphere, strands of
    ``length`` mm in ``segments`` segments drooping under gravity.
    style: "straight", "wavy" (lateral sinusoid, per-strand phase) or "curly"
    (helix around the centre line, per-strand radius jitter and phase)."""
    rng = np.random.default_rng(seed)
    roots = _roots_upper_hemisphere(rng, n_strands, radius)
    center = _centerlines(roots, segments, length, droop)
    arc = np.linspace(0.0, length, segments + 1)[None, :]
    phase = 2.0 * np.pi * rng.random((n_strands, 1))
    if style == "straight":
        pts = center
    elif style == "wavy":
        _, b1, _ = _frames(center)
        off = wave_amp * np.sin(2.0 * np.pi * arc / wave_period + phase)
        pts = center + b1 * off[..., None]
    elif style == "curly":
        _, b1, b2 = _frames(center)
        r = helix_radius * (1.0 + helix_jitter * (2.0 * rng.random((n_strands, 1)) - 1.0))
        ang = 2.0 * np.pi * arc / helix_pitch + phase
        # fade the helix in over the first 5 mm so the roots stay on the sphere
        fade = np.clip(arc / 5.0, 0.0, 1.0)
        pts = center + (b1 * (r * np.cos(ang) * fade)[..., None] + b2 * (r * np.sin(ang) * fade)[..., None])
    else:
        raise ValueError(f"unknown groom style {style!r}")
    pts = pts.astype(F).reshape(-1, 3)
    count = np.full(n_strands, segments + 1, dtype=np.uint32)
    first = (np.arange(n_strands, dtype=np.uint64) * (segments + 1)).astype(np.uint32)
    return Strands(np.ascontiguousarray(pts), first, count)


def parse_hair(data: bytes) -> Strands:
    """Cem Yuksel's binary HAIR format; restates parse_hair (src/hair_file.rs:49-120).
    Optional thickness/transparency/colour arrays are ignored as the reference does."""
    if len(data) < 128 or data[:4] != b"HAIR":
        raise ValueError("not a HAIR file")
    hdr = np.frombuffer(data[:40], dtype="<u4")
    strand_count, point_count, flags, default_segments = int(hdr[1]), int(hdr[2]), int(hdr[3]), int(hdr[4])
    if not flags & 2:
        raise ValueError("HAIR file has no point array")
    cursor = 128
    if flags & 1:
        need = strand_count * 2
        if cursor + need > len(data):
            raise ValueError("HAIR file ended early")
        segs = np.frombuffer(data[cursor:cursor + need], dtype="<u2").astype(np.uint32)
        cursor += need
    else:
        segs = np.full(strand_count, default_segments, dtype=np.uint32)
    need = point_count * 12
    if cursor + need > len(data):
        raise ValueError("HAIR file ended early")
    points = np.frombuffer(data[cursor:cursor + need], dtype="<f4").reshape(-1, 3).copy()
    count = np.minimum(segs.astype(np.uint64) + 1, 0xFFFFFFFF).astype(np.uint32)
    first = np.zeros(strand_count, dtype=np.uint64)
    if strand_count > 1:
        first[1:] = np.cumsum(count[:-1], dtype=np.uint64)
    if strand_count and int(first[-1]) + int(count[-1]) > point_count:
        raise ValueError("HAIR file ended early")
    return Strands(points, first.astype(np.uint32), count)
