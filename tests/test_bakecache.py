"""HAIRBAK1 bake caches (examples/bake.rs:91-241): byte layout, round trip and
the rejection rules (magic, fingerprint, both stamps, exact payload length)."""
import struct

import numpy as np
import pytest

from bevy_hair_gb300 import bakecache as BC
from bevy_hair_gb300 import groom


@pytest.fixture(scope="module")
def mesh():
    return groom.bake(groom.synthetic_strands(300, 24, "wavy", 11), ambient_occlusion=True)


STAMP = BC.SourceStamp(123456, 1_700_000_000, 987_654_321, 42, 1_600_000_000, 5)


def test_header_and_payload_follow_the_reference_encoder(mesh):
    fp = 0x0123456789ABCDEF
    data = BC.encode(mesh, STAMP, fp)
    nb, nc, ns = len(mesh.bundles), len(mesh.layers), len(mesh.style)
    # examples/bake.rs:157-193, field by field
    head = struct.pack("<8sQQQIQQIIII", b"HAIRBAK1", fp, STAMP.len, STAMP.secs, STAMP.nanos, STAMP.scalp_len,
                       STAMP.scalp_secs, STAMP.scalp_nanos, nb, nc, ns)
    head += struct.pack("<3f3f", *mesh.bounds_min[:3], *mesh.bounds_max[:3])
    assert data[:len(head)] == head and len(head) == 92
    assert len(data) == 92 + 12 * nb + 28 * nc + 16 * ns
    b0 = mesh.bundles[0]
    assert data[92:104] == struct.pack("<III", b0["layer_offset"], b0["style_offset"], b0["strand_count"])
    c0 = mesh.layers[0]
    at = 92 + 12 * nb
    assert data[at:at + 28] == struct.pack("<7f", *c0["pos_ao"][:3], *c0["tangent"][:3], c0["pos_ao"][3])
    at += 28 * nc
    assert data[at:at + 16] == struct.pack("<4f", *mesh.style[0])


def test_round_trip(mesh, tmp_path):
    p = tmp_path / "g.bake"
    BC.write(p, mesh, STAMP)
    got = BC.read(p, STAMP)
    assert got is not None
    np.testing.assert_array_equal(got.bundles, mesh.bundles)
    np.testing.assert_array_equal(got.layers["pos_ao"], mesh.layers["pos_ao"])
    np.testing.assert_array_equal(got.layers["tangent"][:, :3], mesh.layers["tangent"][:, :3])
    assert (got.layers["tangent"][:, 3] == 0).all()
    np.testing.assert_array_equal(got.style, mesh.style)
    np.testing.assert_array_equal(got.bounds_min, mesh.bounds_min[:3])
    assert not (tmp_path / "g.bake.tmp").exists()


@pytest.mark.parametrize("field", ["len", "secs", "nanos", "scalp_len", "scalp_secs", "scalp_nanos"])
def test_any_stamp_change_invalidates(mesh, field):
    data = BC.encode(mesh, STAMP)
    other = BC.SourceStamp(**{**STAMP.__dict__, field: getattr(STAMP, field) + 1})
    assert BC.decode(data, other) is None
    assert BC.decode(data, STAMP) is not None


def test_fingerprint_magic_and_length_checks(mesh):
    data = BC.encode(mesh, STAMP)
    assert BC.decode(data, STAMP, fp=BC.fingerprint() ^ 1) is None
    assert BC.decode(b"HAIRBAK2" + data[8:], STAMP) is None
    assert BC.decode(data[:-1], STAMP) is None
    assert BC.decode(data + b"\0", STAMP) is None
    assert BC.decode(data[:50], STAMP) is None
    assert BC.read("/nonexistent/path.bake", STAMP) is None


def test_fingerprint_is_fnv1a_of_the_baker_source():
    # FNV-1a 64 known answers (Fowler/Noll/Vo reference values)
    assert BC.fnv1a_64(b"") == 0xCBF29CE484222325
    assert BC.fnv1a_64(b"a") == 0xAF63DC4C8601EC8C
    assert BC.fnv1a_64(b"foobar") == 0x85944171F73967E8
    src = b"fn bake() {}"
    assert BC.baker_fingerprint(src) == BC.fnv1a_64(src) ^ (16 << 32) ^ 1024


def test_cached_bake_uses_and_refreshes_the_cache(tmp_path):
    strands = groom.synthetic_strands(64, 12, "straight", 3)
    # a HAIR file with explicit segment counts (src/hair_file.rs:49-120)
    n, pts = strands.strand_count, strands.points
    header = bytearray(128)
    struct.pack_into("<4sIII", header, 0, b"HAIR", n, len(pts), 1 | 2)
    body = (strands.count - 1).astype("<u2").tobytes()  # segments per strand
    hair = tmp_path / "tiny.hair"
    hair.write_bytes(bytes(header) + body + pts.astype("<f4").tobytes())
    cache_dir = tmp_path / "cache"
    m1 = BC.cached_bake(hair, cache_dir)
    cache = cache_dir / "tiny.bake"
    assert cache.exists()
    stamp = BC.source_stamp(hair)
    assert BC.read(cache, stamp) is not None
    m2 = BC.cached_bake(hair, cache_dir)  # from the cache
    np.testing.assert_array_equal(m1.layers["pos_ao"], m2.layers["pos_ao"])
    np.testing.assert_array_equal(m1.bundles, m2.bundles)
