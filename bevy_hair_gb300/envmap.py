"""Environment maps for the shade pass's light-probe term (shade.wesl:330-427).

The reference's probes are KTX2 cubemaps in VK_FORMAT_E5B9G9R9_UFLOAT_PACK32
with Zstandard supercompression (assets/env/*.ktx2: a 512^2 x 9-level
specular map and a 32^2 diffuse irradiance map).  This module reads and
writes that container (KTX 2.0 specification: 80-byte header + index, one
level-index entry per mip, each level compressed on its own), decodes and
encodes the shared-exponent texels (EXT_texture_shared_exponent), builds a
seeded procedural sky in the same format for runs without the asset, and
hands the texels to the library (hg_env_set).

Zstandard comes from the system's libzstd.so.1 through ctypes.
"""
from __future__ import annotations

import ctypes as C
import math
import struct
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import abi

KTX2_ID = b"\xabKTX 20\xbb\r\n\x1a\n"
VK_FORMAT_E5B9G9R9_UFLOAT_PACK32 = 123
SUPERCOMPRESSION_NONE, SUPERCOMPRESSION_ZSTD = 0, 2

_ZSTD = None


def _zstd() -> C.CDLL:
    global _ZSTD
    if _ZSTD is None:
        lib = C.CDLL("libzstd.so.1")
        lib.ZSTD_decompress.restype = C.c_size_t
        lib.ZSTD_decompress.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t]
        lib.ZSTD_compress.restype = C.c_size_t
        lib.ZSTD_compress.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_int]
        lib.ZSTD_compressBound.restype = C.c_size_t
        lib.ZSTD_compressBound.argtypes = [C.c_size_t]
        lib.ZSTD_isError.restype = C.c_uint
        lib.ZSTD_isError.argtypes = [C.c_size_t]
        _ZSTD = lib
    return _ZSTD


def zstd_decompress(data: bytes, size: int) -> bytes:
    lib = _zstd()
    out = C.create_string_buffer(size)
    n = lib.ZSTD_decompress(out, size, data, len(data))
    if lib.ZSTD_isError(n) or n != size:
        raise ValueError("zstd: corrupt level data")
    return out.raw


def zstd_compress(data: bytes, level: int = 3) -> bytes:
    lib = _zstd()
    cap = lib.ZSTD_compressBound(len(data))
    out = C.create_string_buffer(cap)
    n = lib.ZSTD_compress(out, cap, data, len(data), level)
    if lib.ZSTD_isError(n):
        raise ValueError("zstd: compression failed")
    return out.raw[:n]


# ---------------------------------------------------------------- RGB9E5


def rgb9e5_decode(words: np.ndarray) -> np.ndarray:
    """u32 texels -> float32 (..., 3): m * 2^(e - 24)."""
    w = np.asarray(words, dtype=np.uint32)
    e = (w >> 27).astype(np.int32) - 24
    m = np.stack([w & 0x1FF, (w >> 9) & 0x1FF, (w >> 18) & 0x1FF], axis=-1).astype(np.float32)
    return np.ldexp(m, e[..., None]).astype(np.float32)


def rgb9e5_encode(rgb: np.ndarray) -> np.ndarray:
    """float (..., 3) -> u32 texels (shared exponent, 9-bit mantissas, bias 15;
    EXT_texture_shared_exponent, section 3.8.x)."""
    c = np.clip(np.nan_to_num(np.asarray(rgb, dtype=np.float64), nan=0.0), 0.0, 65408.0)
    mx = c.max(axis=-1)
    e = np.maximum(-16, np.floor(np.log2(np.maximum(mx, 1e-300)))).astype(np.int64) + 1 + 15
    maxm = np.floor(mx / np.ldexp(1.0, e - 24) + 0.5)
    e = np.where(maxm >= 512, e + 1, e)
    m = np.floor(c / np.ldexp(1.0, e - 24)[..., None] + 0.5).astype(np.uint64)
    m = np.minimum(m, 511)
    return (m[..., 0] | (m[..., 1] << 9) | (m[..., 2] << 18) | (e.astype(np.uint64) << 27)).astype(np.uint32)


# ---------------------------------------------------------------- cubemaps


@dataclass
class Cube:
    """A cubemap mip chain: levels[l] is u32 RGB9E5 [6, size_l, size_l], faces +X -X +Y -Y +Z -Z."""
    size: int
    levels: list[np.ndarray] = field(default_factory=list)

    def packed(self) -> np.ndarray:
        return np.concatenate([np.ascontiguousarray(l, dtype=np.uint32).ravel() for l in self.levels])


@dataclass
class Environment:
    specular: Cube
    diffuse: Cube
    rotation: tuple = (0.0, 0.0, 0.0, 1.0)  # light_probes.view_rotation (x, y, z, w)
    intensity: float = 1.0                   # light_probes.intensity_for_view


def read_ktx2(data: bytes) -> Cube:
    """A KTX2 cubemap in E5B9G9R9 (optionally zstd-supercompressed)."""
    if len(data) < 80 or data[:12] != KTX2_ID:
        raise ValueError("not a KTX2 file")
    (vk, type_size, w, h, depth, layers, faces, levels, scheme) = struct.unpack_from("<9I", data, 12)
    if vk != VK_FORMAT_E5B9G9R9_UFLOAT_PACK32 or type_size != 4:
        raise ValueError(f"unsupported vkFormat {vk}")
    if faces != 6 or w != h or depth not in (0, 1) or layers not in (0, 1):
        raise ValueError("expected a square, non-array cubemap")
    if scheme not in (SUPERCOMPRESSION_NONE, SUPERCOMPRESSION_ZSTD):
        raise ValueError(f"unsupported supercompression {scheme}")
    levels = max(levels, 1)
    cube = Cube(size=w)
    for l in range(levels):
        off, length, raw = struct.unpack_from("<3Q", data, 80 + 24 * l)
        blob = data[off:off + length]
        if len(blob) != length:
            raise ValueError("KTX2 level data ends early")
        sz = max(w >> l, 1)
        need = 6 * sz * sz * 4
        if raw != need:
            raise ValueError("KTX2 level has an unexpected size")
        level = zstd_decompress(blob, raw) if scheme == SUPERCOMPRESSION_ZSTD else blob
        cube.levels.append(np.frombuffer(level, dtype="<u4").reshape(6, sz, sz).copy())
    return cube


def write_ktx2(cube: Cube, zstd_level: int = 3) -> bytes:
    """A minimal KTX2 file (no DFD or key/value data) with zstd-compressed levels."""
    n = len(cube.levels)
    blobs = [zstd_compress(np.ascontiguousarray(l, dtype="<u4").tobytes(), zstd_level) for l in cube.levels]
    head = KTX2_ID + struct.pack("<9I", VK_FORMAT_E5B9G9R9_UFLOAT_PACK32, 4, cube.size, cube.size, 0, 0, 6, n,
                                 SUPERCOMPRESSION_ZSTD)
    head += struct.pack("<4I2Q", 0, 0, 0, 0, 0, 0)
    off = 80 + 24 * n
    index, body = b"", b""
    for l, b in enumerate(blobs):
        sz = max(cube.size >> l, 1)
        index += struct.pack("<3Q", off + len(body), len(b), 6 * sz * sz * 4)
        body += b
    return head + index + body


def load_ktx2(path) -> Cube:
    return read_ktx2(Path(path).read_bytes())


def _face_dirs(size: int) -> np.ndarray:
    """Unit directions through texel centres of every face [6, size, size, 3] (the
    face/axis convention the sampler uses, hg_device.cuh cube_face_uv)."""
    s = (np.arange(size) + 0.5) / size * 2.0 - 1.0
    sc, tc = np.meshgrid(s, s, indexing="xy")
    one = np.ones_like(sc)
    faces = [
        np.stack([one, -tc, -sc], -1),    # +X: sc = -z, tc = -y
        np.stack([-one, -tc, sc], -1),    # -X: sc = +z, tc = -y
        np.stack([sc, one, tc], -1),      # +Y: sc = +x, tc = +z
        np.stack([sc, -one, -tc], -1),    # -Y: sc = +x, tc = -z
        np.stack([sc, -tc, one], -1),     # +Z: sc = +x, tc = -y
        np.stack([-sc, -tc, -one], -1),   # -Z: sc = -x, tc = -y
    ]
    d = np.stack(faces)
    return d / np.linalg.norm(d, axis=-1, keepdims=True)


def procedural(seed: int = 0x5EED0006, size: int = 512, levels: int = 9, diffuse_size: int = 32) -> Environment:
    """A seeded sky: horizon gradient, a warm sun disc and a few soft blobs,
    with box-filtered mips standing in for prefiltered specular levels and a
    coarse average for the diffuse irradiance map."""
    rng = np.random.default_rng(seed)
    sun = rng.normal(size=3)
    sun[1] = abs(sun[1]) + 0.5
    sun /= np.linalg.norm(sun)
    blobs = rng.normal(size=(6, 3))
    blobs /= np.linalg.norm(blobs, axis=1, keepdims=True)
    tints = rng.uniform(0.2, 1.0, size=(6, 3))

    def radiance(d):
        up = d[..., 1:2]
        sky = np.where(up > 0, np.array([0.35, 0.55, 0.95]) * (0.4 + 0.6 * up), np.array([0.25, 0.2, 0.15]) * 0.6)
        c = sky + 40.0 * np.array([1.0, 0.85, 0.6]) * np.maximum(d @ sun, 0.0)[..., None] ** 400
        for b, t in zip(blobs, tints):
            c = c + 0.6 * t * np.maximum(d @ b, 0.0)[..., None] ** 16
        return c

    base = radiance(_face_dirs(size))
    spec_levels, cur = [], base
    for l in range(levels):
        spec_levels.append(rgb9e5_encode(cur))
        if cur.shape[1] > 1:
            cur = 0.25 * (cur[:, 0::2, 0::2] + cur[:, 1::2, 0::2] + cur[:, 0::2, 1::2] + cur[:, 1::2, 1::2])
    f = size // diffuse_size
    diff = base.reshape(6, diffuse_size, f, diffuse_size, f, 3).mean(axis=(2, 4))
    glow = diff.reshape(-1, 3).mean(axis=0)
    diff = 0.5 * diff + 0.5 * glow
    return Environment(Cube(size, spec_levels), Cube(diffuse_size, [rgb9e5_encode(diff)]))


def env_desc(env: Environment | None):
    """(hg_env_desc, keep-alive arrays) for hg_env_set."""
    if env is None:
        return None, ()
    spec, diff = env.specular.packed(), env.diffuse.packed()
    d = abi.EnvDesc()
    d.specular = spec.ctypes.data
    d.specular_size = env.specular.size
    d.specular_levels = len(env.specular.levels)
    d.diffuse = diff.ctypes.data
    d.diffuse_size = env.diffuse.size
    d.diffuse_levels = len(env.diffuse.levels)
    for i in range(4):
        d.rotation[i] = float(env.rotation[i])
    d.intensity = float(env.intensity)
    return d, (spec, diff)


def oracle_arrays(env: Environment | None):
    """The flat arrays the oracle's sampler takes (test infrastructure helper)."""
    if env is None:
        return None
    return (env.specular.packed(), env.specular.size, len(env.specular.levels), env.diffuse.packed(),
            env.diffuse.size, len(env.diffuse.levels), np.asarray(env.rotation, dtype=np.float32),
            float(env.intensity))
