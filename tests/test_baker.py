"""The native baker against the reference's baker tests (src/bake.rs:1391-1527:
cage residuals, root AO, locks not bridged, bent locks, and the real grooms'
quality bounds), the scalp path, the OBJ reader and the HAIR reader
(src/hair_file.rs:144-165)."""
import math
import os
import struct
from pathlib import Path

import numpy as np
import pytest

import hair_mirror as H
from bevy_hair_gb300 import groom


def straight_bundle() -> groom.Strands:
    # src/bake.rs:1529-1552: 3 copies of 4 corner strands, 8 points up +Y
    corners = [(-1, 0, -1), (1, 0, -1), (-1, 0, 1), (1, 0, 1)]
    pts = []
    for _ in range(3):
        for c in corners:
            for layer in range(8):
                pts.append((c[0], c[1] + layer, c[2]))
    pts = np.array(pts, np.float32)
    n = 12
    return groom.Strands(pts, np.arange(n, dtype=np.uint32) * 8, np.full(n, 8, np.uint32))


def test_straight_cage_residuals_are_near_zero():
    mesh = groom.bake(straight_bundle(), ambient_occlusion=False)
    assert mesh.bundle_count == 1
    assert np.isfinite(mesh.layers["pos_ao"]).all() and np.isfinite(mesh.layers["tangent"]).all()
    assert np.linalg.norm(mesh.style[:, :3], axis=1).max() < 1e-2


def test_isolated_bundle_ao_does_not_darken_toward_the_root():
    mesh = groom.bake(straight_bundle(), ambient_occlusion=True)
    ao = mesh.layers["pos_ao"][:, 3]
    root, tip = ao[0:4].mean(), ao[60:64].mean()
    assert root + 0.15 >= tip


def test_diverging_strands_are_not_bridged():
    pts, first = [], []
    for side in (-1.0, 1.0):
        for i in range(16):
            first.append(len(pts))
            tip = np.array([side * 30.0, (i - 7.5) * 0.15, -40.0])
            for layer in range(16):
                pts.append(tip * (layer / 15.0))
    s = groom.Strands(np.array(pts, np.float32), np.array(first, np.uint32), np.full(32, 16, np.uint32))
    mesh = groom.bake(s, ambient_occlusion=False)
    assert mesh.bundle_count > 1
    assert mesh.strand_count() == 32
    assert H.max_styled_stray(mesh, s.points, s.first, s.count) < 8.0


def test_bent_bundle_keeps_its_cross_section():
    # src/bake.rs:1465-1493: a 4 x 4 lock bending through a quarter circle
    pts, first = [], []
    for i in range(4):
        for j in range(4):
            first.append(len(pts))
            root = np.array([i * 0.4, j * 0.4, 0.0])
            for layer in range(16):
                a = layer / 15.0 * math.pi / 2
                pts.append(root + np.array([20.0 * (1.0 - math.cos(a)), 0.0, 20.0 * math.sin(a)]))
    s = groom.Strands(np.array(pts, np.float32), np.array(first, np.uint32), np.full(16, 16, np.uint32))
    mesh = groom.bake(s, ambient_occlusion=False)
    assert H.max_styled_stray(mesh, s.points, s.first, s.count) < 8.0


def _quality(mesh, s):
    idx, rs = H.resample(s.points, s.first, s.count)
    return (mesh.strand_count(), int((s.count >= 2).sum()), len(H.uncovered_roots(mesh, rs[:, 0])),
            H.max_styled_stray(mesh, s.points, s.first, s.count), H.max_reconstruction_error(mesh, rs))


@pytest.mark.parametrize("style", ["straight", "wavy", "curly"])
def test_synthetic_grooms_meet_the_quality_bounds(style):
    """The bounds of the reference's real-groom test (src/bake.rs:1495-1527) on
    seeded grooms: no strand dropped, every root inside a root quad, the uv
    fill within 8 of the strands, every strand reconstructed within 6."""
    s = groom.synthetic_strands(3000, 48, style, 17)
    kept, usable, uncovered, stray, error = _quality(groom.bake(s), s)
    assert kept == usable and uncovered == 0, (kept, usable, uncovered)
    assert stray < 8.0 and error < 6.0, (stray, error)


def _sphere_scalp(radius: float, n: int = 24) -> groom.Scalp:
    verts, tris = [], []
    for i in range(n + 1):
        th = math.pi * i / n
        for j in range(2 * n):
            ph = math.pi * j / n
            verts.append((radius * math.sin(th) * math.cos(ph), radius * math.cos(th), radius * math.sin(th) * math.sin(ph)))
    for i in range(n):
        for j in range(2 * n):
            a, b = i * 2 * n + j, i * 2 * n + (j + 1) % (2 * n)
            c, d = a + 2 * n, b + 2 * n
            tris += [(a, c, b), (b, c, d)]
    return groom.Scalp(np.array(verts, np.float32), np.array(tris, np.uint32))


def test_scalp_roots_lie_in_root_quads_across_the_scalp_normal():
    """With the scalp (bake_hair_mesh_with_scalp): the quality bounds hold, the
    root quads lie across the scalp normal (flush with the scalp) and the
    scalp occludes the roots (darker than the tips)."""
    s = groom.synthetic_strands(2000, 32, "straight", 5, radius=100.0)
    scalp = _sphere_scalp(100.0)
    mesh = groom.bake(s, ambient_occlusion=True, scalp=scalp)
    kept, usable, uncovered, stray, error = _quality(mesh, s)
    assert kept == usable and uncovered == 0 and stray < 8.0 and error < 6.0, (kept, usable, uncovered, stray, error)
    q0 = H._cage(mesh)[:, 0].astype(np.float64)
    nrm = np.cross(q0[:, 1] - q0[:, 0], q0[:, 2] - q0[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    centre = q0.mean(axis=1)
    radial = centre / np.linalg.norm(centre, axis=1, keepdims=True)
    assert np.median(np.abs(np.sum(nrm * radial, axis=1))) > 0.97
    ao = mesh.layers["pos_ao"][:, 3].reshape(-1, 16, 4)
    assert ao[:, 0].mean() < ao[:, -1].mean() - 0.05


def test_scalp_indices_are_checked():
    s = groom.synthetic_strands(50, 8, "straight", 1)
    bad = groom.Scalp(np.zeros((3, 3), np.float32), np.array([[0, 1, 7]], np.uint32))
    with pytest.raises(ValueError):
        groom.bake(s, scalp=bad)


def test_obj_reader_triangulates_polygons_and_resolves_negative_indices():
    text = "# a quad and a triangle\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1/1/1 2/2/2 3/3/3 4/4/4\nv 0 0 1\nf -1 1 2\n"
    sc = groom.parse_obj(text)
    assert sc.vertices.shape == (5, 3)
    np.testing.assert_array_equal(sc.triangles, [[0, 1, 2], [0, 2, 3], [4, 0, 1]])


REFERENCE = os.environ.get("BEVY_HAIR_REFERENCE")


@pytest.mark.skipif(not REFERENCE or not (Path(REFERENCE) / "assets" / "hair" / "woman.obj").exists(),
                    reason="the reference's grooms are not present (set BEVY_HAIR_REFERENCE)")
@pytest.mark.parametrize("name", ["wStraight.hair", "wWavy.hair", "wCurly.hair"])
def test_reference_grooms_with_the_scalp_meet_the_quality_bounds(name):
    """src/bake.rs:1495-1527 on the reference's own assets: the Yuksel grooms
    baked against woman.obj keep every usable strand, cover every root, stray
    less than 8 and reconstruct every strand within 6."""
    hair = Path(REFERENCE) / "assets" / "hair"
    scalp = groom.parse_obj((hair / "woman.obj").read_text())
    s = groom.parse_hair((hair / name).read_bytes())
    kept, usable, uncovered, stray, error = _quality(groom.bake(s, scalp=scalp), s)
    assert kept == usable, (name, kept, usable)
    assert uncovered == 0, (name, uncovered)
    assert stray < 8.0, (name, stray)
    assert error < 6.0, (name, error)


def test_every_strand_lands_in_a_bundle():
    s = groom.synthetic_strands(2000, 16, "wavy", 7)
    mesh = groom.bake(s, ambient_occlusion=False)
    assert mesh.strand_count() == 2000
    assert (mesh.bundles["layer_offset"] % 64 == 0).all()
    assert (mesh.bundles["style_offset"] % 1024 == 0).all()
    assert len(mesh.layers) == 64 * mesh.bundle_count and len(mesh.style) == 1024 * mesh.bundle_count


def test_bake_is_deterministic():
    s = groom.synthetic_strands(1500, 16, "curly", 3)
    a, b = groom.bake(s), groom.bake(s)
    assert np.array_equal(a.bundles, b.bundles)
    assert np.array_equal(a.layers.view(np.uint8), b.layers.view(np.uint8))
    assert np.array_equal(a.style, b.style)


def test_parses_header_and_default_segments():
    # src/hair_file.rs:144-165: one strand, default segment count 2, no segment array
    header = bytearray(128)
    header[0:4] = b"HAIR"
    struct.pack_into("<IIII", header, 4, 1, 3, 0x2, 2)
    body = struct.pack("<9f", 0, 0, 0, 0, 1, 0, 0, 2, 0)
    s = groom.parse_hair(bytes(header) + body)
    assert s.strand_count == 1 and int(s.count[0]) == 3
    assert np.allclose(s.points[2], [0, 2, 0])


def test_hair_reader_rejects_bad_files():
    import pytest

    with pytest.raises(ValueError):
        groom.parse_hair(b"NOPE" + bytes(200))
    header = bytearray(128)
    header[0:4] = b"HAIR"
    struct.pack_into("<IIII", header, 4, 2, 10, 0x2, 4)
    with pytest.raises(ValueError):
        groom.parse_hair(bytes(header) + bytes(12))
