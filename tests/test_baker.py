"""The native baker against the reference's baker tests (src/bake.rs:1391-1493)
and the HAIR reader (src/hair_file.rs:144-165)."""
import struct

import numpy as np

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
