"""HAIRBAK1 bake caches: the on-disk groom cache of the reference's bake
example (examples/bake.rs:91-241), read and written byte for byte.

Layout (little-endian, packed):

    "HAIRBAK1"                                   8 B  magic
    fingerprint                                  u64  identity of the baker that wrote it
    source len, mtime secs, mtime nanos          u64 u64 u32  stamp of the .hair file
    scalp len, mtime secs, mtime nanos           u64 u64 u32  stamp of the scalp mesh (0 without one)
    bundle count, corner count, style count      u32 u32 u32
    bounds_min, bounds_max                       3 x f32 each
    bundles  [layer_offset, style_offset, strand_count]   u32 x 3 each     (12 B)
    corners  [position xyz, tangent xyz, ao]              f32 x 7 each     (28 B)
    style    [x, y, z, w]                                 f32 x 4 each     (16 B)

A cache is used only when the magic, fingerprint and both stamps match and
the payload has exactly the announced length (examples/bake.rs:196-219);
anything else reads as "no cache".  The fingerprint is FNV-1a 64 of the
baker's source text xor (layer count << 32) xor style texels
(src/bake.rs:34-47); this package's baker is csrc/bake.cpp, so its caches
carry that file's fingerprint and caches of the reference's baker are read
by passing the reference's fingerprint.
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import abi
from .groom import HairMesh

MAGIC = b"HAIRBAK1"
HEADER = np.dtype([
    ("magic", "S8"), ("fingerprint", "<u8"),
    ("len", "<u8"), ("secs", "<u8"), ("nanos", "<u4"),
    ("scalp_len", "<u8"), ("scalp_secs", "<u8"), ("scalp_nanos", "<u4"),
    ("bundles", "<u4"), ("corners", "<u4"), ("style", "<u4"),
    ("bounds_min", "<f4", 3), ("bounds_max", "<f4", 3),
])
assert HEADER.itemsize == 92
BUNDLE = np.dtype([("layer_offset", "<u4"), ("style_offset", "<u4"), ("strand_count", "<u4")])
CORNER = np.dtype([("position", "<f4", 3), ("tangent", "<f4", 3), ("ao", "<f4")])
assert BUNDLE.itemsize == 12 and CORNER.itemsize == 28


@dataclass(frozen=True)
class SourceStamp:
    """Size and modification time of the source .hair file and of the scalp mesh."""
    len: int
    secs: int
    nanos: int
    scalp_len: int = 0
    scalp_secs: int = 0
    scalp_nanos: int = 0


def file_stamp(path) -> tuple[int, int, int]:
    """(size, mtime seconds, mtime nanoseconds) of a file (examples/bake.rs:113-118)."""
    st = os.stat(path)
    ns = int(st.st_mtime_ns)
    return int(st.st_size), ns // 1_000_000_000, ns % 1_000_000_000


def source_stamp(hair_path, scalp_path=None) -> SourceStamp:
    a = file_stamp(hair_path)
    b = file_stamp(scalp_path) if scalp_path is not None else (0, 0, 0)
    return SourceStamp(*a, *b)


def fnv1a_64(data: bytes) -> int:
    h = 0xCBF29CE484222325
    for byte in data:
        h = ((h ^ byte) * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
    return h


def baker_fingerprint(source: bytes, layer_count: int = abi.LAYER_COUNT, style_texels: int = abi.STYLE_TEXELS) -> int:
    return (fnv1a_64(source) ^ ((layer_count << 32) & 0xFFFFFFFFFFFFFFFF) ^ style_texels) & 0xFFFFFFFFFFFFFFFF


_FINGERPRINT: int | None = None


def fingerprint() -> int:
    """Identity of this package's baker (csrc/bake.cpp)."""
    global _FINGERPRINT
    if _FINGERPRINT is None:
        _FINGERPRINT = baker_fingerprint((Path(__file__).resolve().parent / "csrc" / "bake.cpp").read_bytes())
    return _FINGERPRINT


def encode(mesh: HairMesh, stamp: SourceStamp, fp: int | None = None) -> bytes:
    fp = fingerprint() if fp is None else fp
    h = np.zeros(1, dtype=HEADER)
    h["magic"] = MAGIC
    h["fingerprint"] = fp
    h["len"], h["secs"], h["nanos"] = stamp.len, stamp.secs, stamp.nanos
    h["scalp_len"], h["scalp_secs"], h["scalp_nanos"] = stamp.scalp_len, stamp.scalp_secs, stamp.scalp_nanos
    h["bundles"], h["corners"], h["style"] = len(mesh.bundles), len(mesh.layers), len(mesh.style)
    h["bounds_min"] = np.asarray(mesh.bounds_min, dtype=np.float32)[:3]
    h["bounds_max"] = np.asarray(mesh.bounds_max, dtype=np.float32)[:3]
    b = np.zeros(len(mesh.bundles), dtype=BUNDLE)
    for f in BUNDLE.names:
        b[f] = mesh.bundles[f]
    c = np.zeros(len(mesh.layers), dtype=CORNER)
    c["position"] = mesh.layers["pos_ao"][:, :3]
    c["ao"] = mesh.layers["pos_ao"][:, 3]
    c["tangent"] = mesh.layers["tangent"][:, :3]
    s = np.ascontiguousarray(mesh.style, dtype="<f4").reshape(-1, 4)
    return h.tobytes() + b.tobytes() + c.tobytes() + s.tobytes()


def decode(data: bytes, stamp: SourceStamp | None = None, fp: int | None = None) -> HairMesh | None:
    """The mesh in `data`, or None when it is not a valid cache for this
    stamp and fingerprint (stamp None: any stamp)."""
    fp = fingerprint() if fp is None else fp
    if len(data) < HEADER.itemsize:
        return None
    h = np.frombuffer(data, dtype=HEADER, count=1)[0]
    if bytes(h["magic"]) != MAGIC or int(h["fingerprint"]) != fp:
        return None
    if stamp is not None and (int(h["len"]), int(h["secs"]), int(h["nanos"]), int(h["scalp_len"]),
                              int(h["scalp_secs"]), int(h["scalp_nanos"])) != (
            stamp.len, stamp.secs, stamp.nanos, stamp.scalp_len, stamp.scalp_secs, stamp.scalp_nanos):
        return None
    nb, nc, ns = int(h["bundles"]), int(h["corners"]), int(h["style"])
    at = HEADER.itemsize
    if len(data) - at != nb * 12 + nc * 28 + ns * 16:
        return None
    b = np.frombuffer(data, dtype=BUNDLE, count=nb, offset=at)
    at += nb * 12
    c = np.frombuffer(data, dtype=CORNER, count=nc, offset=at)
    at += nc * 28
    s = np.frombuffer(data, dtype="<f4", count=ns * 4, offset=at).reshape(ns, 4)
    bundles = np.zeros(nb, dtype=abi.GPU_BUNDLE)
    for f in BUNDLE.names:
        bundles[f] = b[f]
    layers = np.zeros(nc, dtype=abi.GPU_LAYER)
    layers["pos_ao"][:, :3] = c["position"]
    layers["pos_ao"][:, 3] = c["ao"]
    layers["tangent"][:, :3] = c["tangent"]  # GpuLayer.tangent.w = 0 (src/render/pass.rs:100-106)
    return HairMesh(bundles=bundles, layers=layers, style=np.array(s, dtype=np.float32),
                    bounds_min=np.array(h["bounds_min"], dtype=np.float32),
                    bounds_max=np.array(h["bounds_max"], dtype=np.float32))


def write(path, mesh: HairMesh, stamp: SourceStamp, fp: int | None = None) -> None:
    """Write through a temporary file and rename (examples/bake.rs:139-155)."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    tmp = path.with_suffix(path.suffix + ".tmp")
    tmp.write_bytes(encode(mesh, stamp, fp))
    os.replace(tmp, path)


def read(path, stamp: SourceStamp | None = None, fp: int | None = None) -> HairMesh | None:
    try:
        data = Path(path).read_bytes()
    except OSError:
        return None
    return decode(data, stamp, fp)


def cached_bake(hair_path, cache_dir, ambient_occlusion: bool = True) -> HairMesh:
    """The baked mesh of a .hair file through a HAIRBAK1 cache in cache_dir
    (examples/bake.rs:60-89 without a scalp): read it when valid, else parse,
    bake and write it."""
    from . import groom

    hair_path = Path(hair_path)
    stamp = source_stamp(hair_path)
    cache = Path(cache_dir) / (hair_path.stem + ".bake")
    mesh = read(cache, stamp)
    if mesh is not None:
        return mesh
    mesh = groom.bake(groom.parse_hair(hair_path.read_bytes()), ambient_occlusion=ambient_occlusion)
    write(cache, mesh, stamp)
    return mesh
