"""Benchmark and test scenes: seeded synthetic grooms with the shapes and
sizes of the reference workloads (1 unit = 1 mm).

Config 1: 10,000 straight strands x 32 segments, 512x512 camera, DOM 256^2,
          one key directional light, LOD off, roughness 0.3, albedo 0.3.
Config 2: 100,000 wavy strands x 64 segments, 1920x1080, DOM 1024^2, key
          directional light plus 8 ranged point lights, LOD on (lambda 3).
Config 3: 200,000 curly strands x 128 segments, 3840x2160, DOM 2048^2, LOD on
          with the camera far enough that bundles take several LOD levels,
          16 lights.
Config 4: a batch of 64 independent grooms of uneven size (1k-50k strands,
          16-128 segments, log-uniform from the seed, mixed straight / wavy /
          curly), each with its own square camera view of side 256-1024
          (log-uniform) and its own 512^2 deep opacity map; key directional
          light plus 2 point lights shared by all.

``scale`` shrinks the strand count and the image/DOM sides for quick tests
(the scene geometry stays the same).
"""
from __future__ import annotations

import functools
import math
from dataclasses import dataclass, field

import numpy as np

from . import abi, groom, host
from .pipeline import Light, pack_lights

F = np.float32
SEED_BASE = 0x5EED0000


@dataclass
class Scene:
    name: str
    mesh: groom.HairMesh
    groom: host.HairGroom
    view: host.View
    dom_size: tuple[int, int]
    lights: list[Light]
    directionals: list[host.Directional] = field(default_factory=list)
    exposure: float = 1.0

    def params(self, native: bool = True) -> tuple[np.ndarray, np.ndarray]:
        """Camera and DOM uniforms: through the library's native host code, or
        (native=False) through the NumPy restatement, which loads no library."""
        fn = host.groom_params if native else host.groom_params_numpy
        return fn(self.view, self.groom, self.mesh.bounds_min, self.mesh.bounds_max, self.mesh.bundle_count,
                  self.directionals, self.dom_size)

    def light_array(self) -> np.ndarray:
        return pack_lights(self.lights)


KEY_DIR = tuple(host.normalize_or(host.v3(0.35, 0.82, 0.45), (0, 1, 0)).tolist())


def _camera(width: int, height: int, distance: float, target=(0.0, -10.0, 0.0), elevation: float = 0.12,
            azimuth: float = 0.3) -> host.View:
    t = np.asarray(target, dtype=F)
    d = np.array([math.sin(azimuth) * math.cos(elevation), math.sin(elevation),
                  math.cos(azimuth) * math.cos(elevation)], dtype=F)
    eye = t + d * F(distance)
    wfv = host.looking_at(eye, t)
    proj = host.perspective_infinite_reverse_rh(math.pi / 4.0, width / height, 0.1)
    return host.View(wfv, proj, width, height)


def _ring_lights(n: int, radius: float, height: float, intensity: float, rng_seed: int) -> list[Light]:
    rng = np.random.default_rng(rng_seed)
    out = []
    for i in range(n):
        a = 2.0 * math.pi * (i + 0.5) / n
        col = 0.6 + 0.4 * rng.random(3)
        out.append(Light(kind=abi.LIGHT_POINT, color=tuple((col * intensity).tolist()),
                         position=(radius * math.cos(a), height + 60.0 * math.sin(3 * a), radius * math.sin(a)),
                         range=2.5 * radius))
    return out


@functools.lru_cache(maxsize=160)
def _mesh(n_strands: int, segments: int, style: str, seed: int) -> groom.HairMesh:
    return groom.bake(groom.synthetic_strands(n_strands, segments, style, seed), ambient_occlusion=True)


def _scaled(n: int, scale: float, minimum: int) -> int:
    return max(minimum, int(round(n * scale)))


def config1(scale: float = 1.0) -> Scene:
    n = _scaled(10_000, scale, 16)
    side = _scaled(512, math.sqrt(scale), 32)
    dom = _scaled(256, math.sqrt(scale), 16)
    mesh = _mesh(n, 32, "straight", SEED_BASE + 1)
    g = host.HairGroom(lam=3.0, albedo=(0.3, 0.3, 0.3), roughness=0.3, tilt=0.08, lod=False, filter=True,
                       ambient_occlusion=True, deep_opacity=True, center_diameter=1.0)
    key = Light(kind=abi.LIGHT_DIRECTIONAL, color=(3.0, 3.0, 3.0), direction=KEY_DIR, casts_shadows=True)
    return Scene("config1", mesh, g, _camera(side, side, 1000.0), (dom, dom), [key],
                 [host.Directional(np.asarray(KEY_DIR, dtype=F), True)])


def config2(scale: float = 1.0) -> Scene:
    n = _scaled(100_000, scale, 16)
    w, h = _scaled(1920, math.sqrt(scale), 32), _scaled(1080, math.sqrt(scale), 18)
    dom = _scaled(1024, math.sqrt(scale), 16)
    mesh = _mesh(n, 64, "wavy", SEED_BASE + 2)
    g = host.HairGroom(lam=3.0, albedo=(0.16, 0.07, 0.035), roughness=0.3, tilt=0.08, lod=True, filter=True,
                       ambient_occlusion=True, deep_opacity=True, center_diameter=1.0)
    key = Light(kind=abi.LIGHT_DIRECTIONAL, color=(3.0, 2.9, 2.7), direction=KEY_DIR, casts_shadows=True)
    lights = [key] + _ring_lights(8, 500.0, 50.0, 6.0e4, SEED_BASE + 2)
    return Scene("config2", mesh, g, _camera(w, h, 900.0), (dom, dom), lights,
                 [host.Directional(np.asarray(KEY_DIR, dtype=F), True)])


def config3(scale: float = 1.0) -> Scene:
    n = _scaled(200_000, scale, 16)
    w, h = _scaled(3840, math.sqrt(scale), 32), _scaled(2160, math.sqrt(scale), 18)
    dom = _scaled(2048, math.sqrt(scale), 16)
    mesh = _mesh(n, 128, "curly", SEED_BASE + 3)
    g = host.HairGroom(lam=1.5, albedo=(0.3, 0.15, 0.08), roughness=0.35, tilt=0.08, lod=True, filter=True,
                       ambient_occlusion=True, deep_opacity=True, center_diameter=1.0)
    key = Light(kind=abi.LIGHT_DIRECTIONAL, color=(3.0, 3.0, 3.0), direction=KEY_DIR, casts_shadows=True)
    fill = Light(kind=abi.LIGHT_DIRECTIONAL, color=(0.4, 0.45, 0.6), direction=(-0.5, 0.3, -0.8))
    lights = [key, fill] + _ring_lights(14, 600.0, 0.0, 8.0e4, SEED_BASE + 3)
    return Scene("config3", mesh, g, _camera(w, h, 1400.0), (dom, dom), lights,
                 [host.Directional(np.asarray(KEY_DIR, dtype=F), True)])


def real_groom(hair_path, scalp_path=None, width: int = 1920, height: int = 1080, dom: int = 1024) -> Scene:
    """A groom from a HAIR file (e.g. the Cem Yuksel grooms the reference ships
    in assets/hair, 50,000 strands each), baked against its scalp mesh when an
    OBJ is given, framed by a camera on the mesh's bounds, with config 2's
    material and lights."""
    from pathlib import Path

    strands = groom.parse_hair(Path(hair_path).read_bytes())
    scalp = groom.parse_obj(Path(scalp_path).read_text()) if scalp_path else None
    mesh = groom.bake(strands, ambient_occlusion=True, scalp=scalp)
    centre = 0.5 * (mesh.bounds_min + mesh.bounds_max)
    radius = float(np.linalg.norm(mesh.bounds_max - mesh.bounds_min)) * 0.5
    g = host.HairGroom(lam=3.0, albedo=(0.16, 0.07, 0.035), roughness=0.3, tilt=0.08, lod=True, filter=True,
                       ambient_occlusion=True, deep_opacity=True, center_diameter=1.0)
    key = Light(kind=abi.LIGHT_DIRECTIONAL, color=(3.0, 2.9, 2.7), direction=KEY_DIR, casts_shadows=True)
    lights = [key] + _ring_lights(8, 4.0 * radius, 0.3 * radius, 6.0e4 * (radius / 500.0) ** 2, SEED_BASE + 6)
    return Scene(Path(hair_path).stem, mesh, g, _camera(width, height, 2.6 * radius, target=tuple(centre.tolist())),
                 (dom, dom), lights, [host.Directional(np.asarray(KEY_DIR, dtype=F), True)])


@dataclass
class BatchScene:
    name: str
    scenes: list[Scene]
    lights: list[Light]

    def light_array(self) -> np.ndarray:
        return pack_lights(self.lights)

    def sizes(self) -> list[tuple[int, int, int, int]]:
        return [(s.view.width, s.view.height, *s.dom_size) for s in self.scenes]


def config4(scale: float = 1.0, items: int = 64) -> BatchScene:
    rng = np.random.default_rng(SEED_BASE + 4)
    styles = ("straight", "wavy", "curly")
    key = Light(kind=abi.LIGHT_DIRECTIONAL, color=(3.0, 2.9, 2.7), direction=KEY_DIR, casts_shadows=True)
    lights = [key] + _ring_lights(2, 500.0, 50.0, 6.0e4, SEED_BASE + 4)
    dom = _scaled(512, math.sqrt(scale), 16)
    scenes = []
    for k in range(items):
        n = _scaled(int(round(math.exp(rng.uniform(math.log(1_000), math.log(50_000))))), scale, 16)
        segments = int(round(math.exp(rng.uniform(math.log(16), math.log(128)))))
        style = styles[int(rng.integers(0, 3))]
        side = _scaled(int(round(math.exp(rng.uniform(math.log(256), math.log(1024))))), math.sqrt(scale), 32)
        azimuth = float(rng.uniform(0.0, 2.0 * math.pi))
        distance = float(rng.uniform(700.0, 1100.0))
        mesh = _mesh(n, segments, style, SEED_BASE + 400 + k)
        g = host.HairGroom(lam=3.0, albedo=tuple(float(v) for v in rng.uniform(0.05, 0.4, 3)), roughness=0.3,
                           tilt=0.08, lod=True, filter=True, ambient_occlusion=True, deep_opacity=True,
                           center_diameter=1.0)
        scenes.append(Scene(f"config4[{k}]", mesh, g, _camera(side, side, distance, azimuth=azimuth), (dom, dom),
                            lights, [host.Directional(np.asarray(KEY_DIR, dtype=F), True)]))
    return BatchScene("config4", scenes, lights)


CONFIGS = {1: config1, 2: config2, 3: config3}


def segments_of(refs: np.ndarray, total: int) -> int:
    """Segments a raster pass draws: sum over refs of (control_points - 1)."""
    cps = refs["control_points"][:total].astype(np.int64)
    return int(np.clip(cps, 2, 127).sum() - total)
