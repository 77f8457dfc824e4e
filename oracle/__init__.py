"""Python binding of the CPU oracle.  TEST INFRASTRUCTURE ONLY.

The oracle (hair_oracle.c) restates the reference's per-frame passes on the
CPU.  Only the tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline
leg use it, as the checker; the product never imports it.  See
hair_oracle.h for what is pinned by the reference's known-answer tests and
for the float semantics it defines.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

from bevy_hair_gb300 import abi

HERE = Path(__file__).resolve().parent
SO = HERE / "_build" / "libhair_oracle.so"


class Env(C.Structure):
    _fields_ = [("spec", C.c_void_p), ("spec_size", C.c_uint32), ("spec_levels", C.c_uint32),
                ("diff", C.c_void_p), ("diff_size", C.c_uint32), ("diff_levels", C.c_uint32),
                ("rot", C.c_float * 4), ("intensity", C.c_float)]


def _env(env):
    """An oracle_env for a bevy_hair_gb300.envmap.Environment (or None), plus keep-alive arrays."""
    if env is None:
        return None, ()
    spec, diff = env.specular.packed(), env.diffuse.packed()
    e = Env(spec.ctypes.data, env.specular.size, len(env.specular.levels), diff.ctypes.data, env.diffuse.size,
            len(env.diffuse.levels), (C.c_float * 4)(*[float(v) for v in env.rotation]), float(env.intensity))
    return e, (spec, diff)


class Counts(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("samples", "cons_min", "center_min", "beta_min", "dom_min", "dom_add",
                                          "segments")]

    def as_dict(self) -> dict:
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


_LIB = None
_VP, _U32, _U64, _F, _I = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_int

_SIGS = {
    "oracle_set_threads": (None, [_I]),
    "oracle_get_threads": (_I, []),
    "oracle_pcg": (_U32, [_U32]),
    "oracle_pack_gb": (_U64, [_U32] * 7),
    "oracle_unpack_gb": (None, [_U64, _VP]),
    "oracle_pack_beta": (_U32, [_U32, _F]),
    "oracle_quantize_depth": (_U32, [_F, _F, _F]),
    "oracle_dequantize_depth": (_F, [_U32, _F, _F]),
    "oracle_control_points_for_lod": (_U32, [_F]),
    "oracle_lod_selection": (_F, [_F, _F, _F]),
    "oracle_strand_count_lod": (_U32, [_F, _U32, _F, _I]),
    "oracle_dom_optical_depth": (_F, [_VP, _U32, _F]),
    "oracle_depth_correction": (_F, [_F]),
    "oracle_oct_encode": (None, [_VP, _VP]),
    "oracle_oct_decode": (None, [_U32, _U32, _VP]),
    "oracle_clear": (None, [_VP, _VP, _VP, _U64]),
    "oracle_clear_dom": (None, [_VP, _U64]),
    "oracle_lod": (None, [_VP, _VP, _VP, _VP]),
    "oracle_scan": (None, [_VP, _VP, _VP, _U32, _VP]),
    "oracle_strand_points": (_U32, [_VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "oracle_raster": (None, [_VP, _VP, _VP, _VP, _VP, _U32, _VP, _VP, _VP, _VP, _VP, C.POINTER(Counts)]),
    "oracle_shade": (None, [_VP, _VP, _VP, _VP, _VP, _U32, _U32, _F, _VP, _U32, _VP, _VP, _VP]),
    "oracle_sample_cube": (None, [_VP, _U32, _U32, _VP, _F, _VP]),
    "oracle_mlp_forward": (None, [_VP, _VP, _U32, _VP]),
    "oracle_mlp_forward_arch": (None, [_VP, _U32, _VP, _U32, _VP]),
    "oracle_filter": (None, [_VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "oracle_composite": (None, [_VP, _VP, _VP, _VP, _VP]),
    "oracle_hair_visibility": (None, [_VP, _VP, _U32, _U32, _VP, _U32, _VP]),
    "oracle_lobes_batch": (None, [_I, _VP, _U32, C.c_double, _VP]),
}


def build() -> Path:
    src = [HERE / "hair_oracle.c", HERE / "marschner.c", HERE / "hair_oracle.h", HERE.parent / "include" / "hairgb.h"]
    if not SO.exists() or any(s.stat().st_mtime > SO.stat().st_mtime for s in src):
        res = subprocess.run(["make", "-C", str(HERE)], capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"building the oracle failed:\n{res.stdout}\n{res.stderr}")
    return SO


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        build()
        l = C.CDLL(str(SO))
        for name, (res, args) in _SIGS.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = l
    return _LIB


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def _p(a):
    return None if a is None else a.ctypes.data


# ------------------------------------------------------------------ passes


def lod(params: np.ndarray, mesh) -> np.ndarray:
    count = int(params["pass_mode"][1])
    count = min(count, mesh.bundle_count)
    out = np.zeros(max(count, 1), dtype=abi.LOD_RECORD)
    p = params.copy()
    p["pass_mode"][1] = count
    if count:
        lib().oracle_lod(_p(p), _p(mesh.bundles), _p(mesh.layers), _p(out))
    return out[:count]


def scan(params: np.ndarray, lod_records: np.ndarray, capacity: int) -> tuple[np.ndarray, int]:
    p = params.copy()
    p["pass_mode"][1] = len(lod_records)
    refs = np.zeros(max(capacity, 1), dtype=abi.STRAND_REF)
    ind = np.zeros(4, dtype=np.uint32)
    recs = np.ascontiguousarray(lod_records) if len(lod_records) else np.zeros(1, dtype=abi.LOD_RECORD)
    lib().oracle_scan(_p(p), _p(recs), _p(refs), max(capacity, 1), _p(ind))
    return refs, int(ind[0])


def clear_targets(width: int, height: int):
    n = width * height
    center = np.empty(n, dtype=np.uint64)
    cons = np.empty(n, dtype=np.uint64)
    beta = np.empty(n, dtype=np.uint32)
    lib().oracle_clear(_p(center), _p(cons), _p(beta), n)
    return center, cons, beta


def clear_dom(dom_w: int, dom_h: int) -> np.ndarray:
    texels = dom_w * dom_h
    dom = np.empty(texels * (1 + abi.DOM_LAYERS), dtype=np.uint32)
    lib().oracle_clear_dom(_p(dom), texels)
    return dom


def raster(params, mesh, refs, total, center, cons, beta, dom, scene_depth=None) -> dict:
    counts = Counts()
    style = np.ascontiguousarray(mesh.style, dtype=np.float32)
    lib().oracle_raster(_p(params), _p(mesh.bundles), _p(mesh.layers), _p(style), _p(refs), int(total), _p(center),
                        _p(cons), _p(beta), _p(dom), _p(scene_depth), C.byref(counts))
    return counts.as_dict()


def shade(params, center, beta, dom, lights, exposure=1.0, ortho=False, mlp=None, env=None, mlp_arch=0):
    """Shade model 0 (Karis fit), or the surrogate when `mlp` holds its parameters
    (mlp_arch 0: the 4 x 64 network of models 1 and 2; 1: the compact network of model 3);
    env: a bevy_hair_gb300.envmap.Environment for the light-probe term."""
    w, h = int(params["screen"][0]), int(params["screen"][1])
    shaded = np.empty(w * h * 4, dtype=np.float32)
    sdepth = np.empty(w * h, dtype=np.float32)
    lights = np.ascontiguousarray(lights, dtype=abi.LIGHT)
    dom_arr = dom if dom is not None else np.zeros(16, dtype=np.uint32)
    mlp_arr = None if mlp is None else np.ascontiguousarray(mlp, dtype=np.float32)
    e, keep = _env(env)
    lib().oracle_shade(_p(params), _p(center), _p(beta), _p(dom_arr), _p(lights) if len(lights) else None,
                       len(lights), int(ortho), float(exposure), _p(mlp_arr), int(mlp_arch), C.byref(e) if e else None,
                       _p(shaded), _p(sdepth))
    return shaded, sdepth


def sample_cube(texels: np.ndarray, size: int, levels: int, direction, lod: float) -> np.ndarray:
    out = np.zeros(3, dtype=np.float32)
    d = np.asarray(direction, dtype=np.float32)
    t = np.ascontiguousarray(texels, dtype=np.uint32)
    lib().oracle_sample_cube(_p(t), size, levels, _p(d), float(lod), _p(out))
    return out


def mlp_forward(params: np.ndarray, raw: np.ndarray, arch: int = 0) -> np.ndarray:
    """The surrogate network on raw inputs (n, 10) -> raw outputs, FP16 rounding emulated
    (arch 0: 4 x 64, (n, 12) lobes; 1: the compact 2 x 32, (n, 3) BSDF channels)."""
    p = np.ascontiguousarray(params, dtype=np.float32)
    x = np.ascontiguousarray(raw, dtype=np.float32).reshape(-1, 10)
    out = np.empty((len(x), 3 if arch == 1 else 12), dtype=np.float32)
    lib().oracle_mlp_forward_arch(_p(p), int(arch), _p(x), len(x), _p(out))
    return out


def filter_(params, center, cons, shaded, shaded_depth):
    w, h = int(params["screen"][0]), int(params["screen"][1])
    filt = np.empty(w * h * 4, dtype=np.float32)
    fdepth = np.empty(w * h, dtype=np.float32)
    lib().oracle_filter(_p(params), _p(center), _p(cons), _p(np.ascontiguousarray(shaded, dtype=np.float32)),
                        _p(np.ascontiguousarray(shaded_depth, dtype=np.float32)), _p(filt), _p(fdepth))
    return filt, fdepth


def composite(params, color_src, depth_src, color_dst, depth_dst) -> None:
    lib().oracle_composite(_p(params), _p(np.ascontiguousarray(color_src, dtype=np.float32)),
                           _p(np.ascontiguousarray(depth_src, dtype=np.float32)), _p(color_dst), _p(depth_dst))


def frame(mesh, camera, dom_params, lights, exposure=1.0, ortho=False, scene_depth=None, mlp=None, env=None,
          mlp_arch=0) -> dict:
    """The per-groom sequence of hair_pass (src/render/pass.rs:375-643) on the CPU."""
    w, h = int(camera["screen"][0]), int(camera["screen"][1])
    out: dict = {}
    capacity = max(mesh.strand_count(), 1)
    center, cons, beta = clear_targets(w, h)
    lod_c = lod(camera, mesh)
    refs_c, total_c = scan(camera, lod_c, capacity)
    out["lod_camera"], out["refs_camera"], out["total_camera"] = lod_c, refs_c, total_c
    out["counts_camera"] = raster(camera, mesh, refs_c, total_c, center, cons, beta, None, scene_depth)
    dom = None
    if int(camera["flags"][3]):
        dw, dh = int(dom_params["screen"][0]), int(dom_params["screen"][1])
        dom = clear_dom(dw, dh)
        lod_d = lod(dom_params, mesh)
        refs_d, total_d = scan(dom_params, lod_d, capacity)
        out["lod_dom"], out["refs_dom"], out["total_dom"] = lod_d, refs_d, total_d
        out["counts_dom_depth"] = raster(dom_params, mesh, refs_d, total_d, center, cons, beta, dom)
        layers = dom_params.copy()
        layers["pass_mode"][0] = 2
        out["counts_dom_layers"] = raster(layers, mesh, refs_d, total_d, center, cons, beta, dom)
    shaded, sdepth = shade(camera, center, beta, dom, lights, exposure, ortho, mlp, env, mlp_arch)
    out.update(center=center, cons=cons, beta=beta, dom=dom, shaded=shaded, shaded_depth=sdepth)
    if int(camera["flags"][1]):
        filt, fdepth = filter_(camera, center, cons, shaded, sdepth)
        out.update(filtered=filt, filtered_depth=fdepth)
        src, srcd = filt, fdepth
    else:
        src, srcd = shaded, sdepth
    color = np.zeros(w * h * 4, dtype=np.float32)
    depth = np.full(w * h, 0.0 if int(camera["pass_mode"][2]) == 1 else 1.0, dtype=np.float32)
    composite(camera, src, srcd, color, depth)
    out.update(color=color, depth=depth)
    return out


def hair_visibility(light: np.ndarray, dom: np.ndarray, dom_w: int, dom_h: int, points: np.ndarray) -> np.ndarray:
    """hair_shadow.wesl:52-75 for float4 points against a deep opacity map."""
    pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 4)
    out = np.empty(len(pts), dtype=np.float32)
    lib().oracle_hair_visibility(_p(np.ascontiguousarray(light)), _p(np.ascontiguousarray(dom)), dom_w, dom_h,
                                 _p(pts), len(pts), _p(out))
    return out


def lobes(inputs: np.ndarray, model: str = "marschner", tilt: float = 0.08) -> np.ndarray:
    """FP64 hair lobes for inputs (n, 10): sin_i, sin_o, cos_phi, sin_phi, sigma_a rgb,
    beta_m, beta_n, eta.  Returns (n, 12): R, TT, TRT, B (rgb each).  model
    "marschner": exact azimuthal integrals (the FP64 reference); "karis": shade.wesl's fits."""
    x = np.ascontiguousarray(inputs, dtype=np.float64).reshape(-1, 10)
    out = np.empty((len(x), 12), dtype=np.float64)
    lib().oracle_lobes_batch(0 if model == "marschner" else 1, _p(x), len(x), float(tilt), _p(out))
    return out
