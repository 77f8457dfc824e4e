"""Pass orchestration over the C ABI: the per-view, per-groom body of
``hair_pass`` (src/render/pass.rs:259-657).

``HairRenderer`` owns one hairgb context (device memory, one CUDA stream).
Each pass of the reference has a method with the same role; ``render_groom``
runs the whole per-groom sequence in one native call (``hg_groom_frame``).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi
from .groom import HairMesh


def _check(lib, ctx, status: int) -> None:
    if status != abi.HG_OK:
        msg = lib.hg_last_error(ctx) if ctx else b""
        raise abi.HairGbError(status, (msg or b"").decode())


@dataclass
class Light:
    """One light of the shade pass (see hg_light in include/hairgb.h)."""
    kind: int
    color: tuple
    position: tuple = (0.0, 0.0, 0.0)
    direction: tuple = (0.0, 1.0, 0.0)
    range: float = 1000.0
    casts_shadows: bool = False
    spot_scale: float = 1.0
    spot_offset: float = 0.0
    right: tuple = (1.0, 0.0, 0.0)
    up: tuple = (0.0, 1.0, 0.0)
    width: float = 1.0
    height: float = 1.0


def pack_lights(lights: list[Light]) -> np.ndarray:
    out = np.zeros(len(lights), dtype=abi.LIGHT)
    for i, l in enumerate(lights):
        out[i]["kind"] = l.kind
        out[i]["flags"] = abi.LIGHT_CASTS_SHADOWS if l.casts_shadows else 0
        out[i]["range"] = l.range
        out[i]["position"][:3] = l.position
        out[i]["color"][:3] = l.color
        out[i]["direction"][:3] = l.direction
        if l.kind == abi.LIGHT_RECT:
            out[i]["spot"][:2] = (l.width, l.height)
        else:
            out[i]["spot"][:2] = (l.spot_scale, l.spot_offset)
        out[i]["right"][:3] = l.right
        out[i]["up"][:3] = l.up
    return out


class GpuGroom:
    """A groom uploaded to the device (GpuGroom::upload, src/render/pass.rs:98-167)."""

    def __init__(self, renderer: "HairRenderer", mesh: HairMesh):
        self.renderer = renderer
        self.mesh = mesh
        lib = renderer.lib
        out = C.c_void_p()
        bundles = np.ascontiguousarray(mesh.bundles)
        layers = np.ascontiguousarray(mesh.layers)
        style = np.ascontiguousarray(mesh.style, dtype=np.float32)
        _check(lib, renderer.ctx, lib.hg_groom_upload(renderer.ctx, abi.ptr(bundles), len(bundles), abi.ptr(layers),
                                                      len(layers), abi.ptr(style), len(style), C.byref(out)))
        self.handle = out

    @property
    def bundle_count(self) -> int:
        return self.mesh.bundle_count

    def buffer(self, slot: int, which: int) -> tuple[int, int]:
        p, n = C.c_void_p(), C.c_size_t()
        lib = self.renderer.lib
        _check(lib, self.renderer.ctx,
               lib.hg_groom_buffer(self.renderer.ctx, self.handle, slot, which, C.byref(p), C.byref(n)))
        return p.value or 0, n.value

    def read(self, slot: int, which: int) -> np.ndarray:
        """Copy the slot's LodRecords, StrandRefs or indirect words (or the
        strand cache, as float32 [strands, 130, 4]) to the host."""
        _, nbytes = self.buffer(slot, which)
        host = np.empty(nbytes, dtype=np.uint8)
        lib = self.renderer.lib
        _check(lib, self.renderer.ctx, lib.hg_groom_copy_out(self.renderer.ctx, self.handle, slot, which,
                                                             abi.ptr(host), nbytes))
        if which == abi.GBUF_STRAND_CACHE:
            return host.view(np.float32).reshape(-1, 130, 4)
        dt = {abi.GBUF_LOD: abi.LOD_RECORD, abi.GBUF_REFS: abi.STRAND_REF, abi.GBUF_INDIRECT: np.uint32}[which]
        return host.view(dt)

    def close(self) -> None:
        if self.handle:
            self.renderer.lib.hg_groom_destroy(self.renderer.ctx, self.handle)
            self.handle = None


class HairBatch:
    """hg_batch: many grooms with their own camera views and deep opacity maps,
    one launch per pass, replayed as a CUDA graph."""

    def __init__(self, renderer: "HairRenderer", grooms: list["GpuGroom"], sizes: list[tuple[int, int, int, int]]):
        self.renderer, self.lib = renderer, renderer.lib
        items = (abi.BatchItem * len(grooms))()
        for k, (g, (w, h, dw, dh)) in enumerate(zip(grooms, sizes)):
            items[k] = abi.BatchItem(g.handle.value, w, h, dw, dh)
        handle = C.c_void_p()
        _check(self.lib, renderer.ctx, self.lib.hg_batch_create(renderer.ctx, items, len(grooms), C.byref(handle)))
        self.handle, self.sizes, self.grooms = handle, list(sizes), list(grooms)
        if not hasattr(renderer, "_batches"):
            renderer._batches = []
        renderer._batches.append(self)

    def _check(self, status: int) -> None:
        _check(self.lib, self.renderer.ctx, status)

    def set_params(self, item: int, camera: np.ndarray, dom: np.ndarray | None) -> None:
        self._check(self.lib.hg_batch_set_params(self.handle, item, camera.ctypes.data,
                                                 dom.ctypes.data if dom is not None else None))

    @staticmethod
    def _desc(lights: np.ndarray, exposure: float, ortho: bool) -> tuple[abi.ShadeDesc, np.ndarray]:
        lights = np.ascontiguousarray(lights, dtype=abi.LIGHT)
        return abi.ShadeDesc(abi.ptr(lights) if len(lights) else None, len(lights), int(ortho), exposure, 0), lights

    def frame(self, lights: np.ndarray, mode: int = abi.BATCH_GRAPH, exposure: float = 1.0,
              ortho: bool = False) -> None:
        d, keep = self._desc(lights, exposure, ortho)
        self._check(self.lib.hg_batch_frame(self.handle, C.byref(d), mode))

    def profile(self, lights: np.ndarray, exposure: float = 1.0) -> dict:
        """Per-phase milliseconds of one directly launched batched frame."""
        d, keep = self._desc(lights, exposure, False)
        ms = np.zeros(4, dtype=np.float32)
        self._check(self.lib.hg_batch_profile(self.handle, C.byref(d), ms.ctypes.data))
        return dict(zip(("setup", "raster", "shade", "filter_composite"), (round(float(v), 4) for v in ms)))

    def launches(self, mode: int) -> int:
        n = C.c_uint32()
        self._check(self.lib.hg_batch_launches(self.handle, mode, C.byref(n)))
        return int(n.value)

    def tune(self, lights: np.ndarray, exposure: float = 1.0) -> list[dict]:
        d, keep = self._desc(lights, exposure, False)
        res = (abi.BatchTuning * 64)()
        n = C.c_uint32()
        self._check(self.lib.hg_batch_tune(self.handle, C.byref(d), res, 64, C.byref(n)))
        return [res[k].as_dict() for k in range(min(int(n.value), 64))]

    def tuning(self) -> dict:
        t = abi.BatchTuning()
        self._check(self.lib.hg_batch_get_tuning(self.handle, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, **kw) -> None:
        t = abi.BatchTuning()
        self._check(self.lib.hg_batch_get_tuning(self.handle, C.byref(t)))
        for k, v in kw.items():
            setattr(t, k, v)
        self._check(self.lib.hg_batch_set_tuning(self.handle, C.byref(t)))

    def buffer(self, item: int, which: int) -> tuple[int, int]:
        p, n = C.c_void_p(), C.c_size_t()
        self._check(self.lib.hg_batch_buffer(self.handle, item, which, C.byref(p), C.byref(n)))
        return p.value or 0, n.value

    def read(self, item: int, which: int) -> np.ndarray:
        _, nbytes = self.buffer(item, which)
        dt = HairRenderer._DTYPES[which]
        out = np.empty(nbytes // np.dtype(dt).itemsize, dtype=dt)
        if nbytes:
            self._check(self.lib.hg_batch_copy_out(self.handle, item, which, abi.ptr(out), out.nbytes))
        return out

    def close(self) -> None:
        if self.handle:
            self.lib.hg_batch_destroy(self.handle)
            self.handle = None
            if self in getattr(self.renderer, "_batches", []):
                self.renderer._batches.remove(self)


class HairRenderer:
    """One hairgb context: targets, grooms and the passes of hair_pass."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self.lib = abi.load()
        ctx = C.c_void_p()
        st = self.lib.hg_create(device, stream, C.byref(ctx))
        if st != abi.HG_OK:
            raise abi.HairGbError(st, "hg_create failed (is a CUDA device visible?)")
        self.ctx = ctx
        self.size = (0, 0, 0, 0)

    # -- resources ----------------------------------------------------------
    def ensure_targets(self, width: int, height: int, dom_w: int, dom_h: int) -> None:
        _check(self.lib, self.ctx, self.lib.hg_ensure_targets(self.ctx, width, height, dom_w, dom_h))
        self.size = (width, height, dom_w, dom_h)

    def upload(self, mesh: HairMesh) -> GpuGroom:
        return GpuGroom(self, mesh)

    def buffer(self, which: int) -> tuple[int, int]:
        p, n = C.c_void_p(), C.c_size_t()
        _check(self.lib, self.ctx, self.lib.hg_buffer(self.ctx, which, C.byref(p), C.byref(n)))
        return p.value or 0, n.value

    _DTYPES = {
        abi.BUF_CENTER: np.uint64, abi.BUF_CONSERVATIVE: np.uint64, abi.BUF_BETA: np.uint32,
        abi.BUF_DOM: np.uint32, abi.BUF_SHADED: np.float32, abi.BUF_SHADED_DEPTH: np.float32,
        abi.BUF_FILTERED: np.float32, abi.BUF_FILTERED_DEPTH: np.float32, abi.BUF_COLOR: np.float32,
        abi.BUF_DEPTH: np.float32,
    }

    def read(self, which: int, out: np.ndarray | None = None) -> np.ndarray:
        _, nbytes = self.buffer(which)
        dt = self._DTYPES[which]
        if out is None:
            out = np.empty(nbytes // np.dtype(dt).itemsize, dtype=dt)
        _check(self.lib, self.ctx, self.lib.hg_copy_out(self.ctx, which, abi.ptr(out), out.nbytes))
        return out

    def read_async(self, which: int, host_ptr: int, nbytes: int) -> None:
        """hg_copy_out_async: enqueue a copy of buffer `which` into host memory at
        `host_ptr` (page-locked for overlap) and return; the data is final after
        copy_wait()."""
        _check(self.lib, self.ctx, self.lib.hg_copy_out_async(self.ctx, which, host_ptr, nbytes))

    def copy_wait(self) -> None:
        _check(self.lib, self.ctx, self.lib.hg_copy_wait(self.ctx))

    def write(self, which: int, host: np.ndarray) -> None:
        host = np.ascontiguousarray(host)
        _check(self.lib, self.ctx, self.lib.hg_copy_in(self.ctx, which, abi.ptr(host), host.nbytes))

    def synchronize(self) -> int:
        word = C.c_uint32()
        st = self.lib.hg_synchronize(self.ctx, C.byref(word))
        _check(self.lib, self.ctx, st)
        return word.value

    # -- passes -------------------------------------------------------------
    def clear(self) -> None:
        _check(self.lib, self.ctx, self.lib.hg_clear(self.ctx))

    def clear_dom(self) -> None:
        _check(self.lib, self.ctx, self.lib.hg_clear_dom(self.ctx))

    def lod(self, groom: GpuGroom, params: np.ndarray, slot: int) -> None:
        _check(self.lib, self.ctx, self.lib.hg_lod(self.ctx, groom.handle, params.ctypes.data, slot))

    def scan(self, groom: GpuGroom, params: np.ndarray, slot: int) -> None:
        _check(self.lib, self.ctx, self.lib.hg_scan(self.ctx, groom.handle, params.ctypes.data, slot))

    def generate(self, groom: GpuGroom, params: np.ndarray) -> None:
        _check(self.lib, self.ctx, self.lib.hg_generate(self.ctx, groom.handle, params.ctypes.data))

    def raster(self, groom: GpuGroom, params: np.ndarray, slot: int, scene_depth_ptr: int | None = None) -> None:
        _check(self.lib, self.ctx,
               self.lib.hg_raster(self.ctx, groom.handle, params.ctypes.data, slot, scene_depth_ptr))

    def set_camera_raster(self, mode: int) -> None:
        """abi.CAMERA_RASTER_DIRECT (global atomics per sample, the default) or
        abi.CAMERA_RASTER_BINNED (32x32 tiles resolved in shared memory); the
        G-buffer words are the same."""
        _check(self.lib, self.ctx, self.lib.hg_set_camera_raster(self.ctx, int(mode)))

    def shade(self, params: np.ndarray, lights: np.ndarray, exposure: float = 1.0, ortho: bool = False,
              model: int = abi.SHADE_KARIS) -> None:
        lights = np.ascontiguousarray(lights, dtype=abi.LIGHT)
        d = abi.ShadeDesc(abi.ptr(lights) if len(lights) else None, len(lights), int(ortho), exposure, int(model))
        _check(self.lib, self.ctx, self.lib.hg_shade(self.ctx, params.ctypes.data, C.byref(d)))

    def filter(self, params: np.ndarray) -> None:
        _check(self.lib, self.ctx, self.lib.hg_filter(self.ctx, params.ctypes.data))

    def composite(self, params: np.ndarray, source_filtered: bool) -> None:
        _check(self.lib, self.ctx, self.lib.hg_composite(self.ctx, params.ctypes.data, int(source_filtered)))

    def clear_color(self, depth_clear: float) -> None:
        _check(self.lib, self.ctx, self.lib.hg_clear_color(self.ctx, depth_clear))

    def render_groom(self, groom: GpuGroom, camera: np.ndarray, dom: np.ndarray | None, lights: np.ndarray,
                     exposure: float = 1.0, ortho: bool = False, scene_depth_ptr: int | None = None,
                     composite: bool = True, clear_color: bool = True, model: int = abi.SHADE_KARIS) -> None:
        """hg_groom_frame: clear, lod, scan, raster, [DOM], shade, [filter], composite."""
        lights = np.ascontiguousarray(lights, dtype=abi.LIGHT)
        d = abi.FrameDesc()
        d.camera = camera.ctypes.data
        d.dom = dom.ctypes.data if dom is not None else None
        d.scene_depth = scene_depth_ptr
        d.shade = abi.ShadeDesc(abi.ptr(lights) if len(lights) else None, len(lights), int(ortho), exposure,
                                int(model))
        d.composite = int(composite)
        d.clear_color = int(clear_color)
        self._frame_keepalive = (lights, camera, dom)
        _check(self.lib, self.ctx, self.lib.hg_groom_frame(self.ctx, groom.handle, C.byref(d)))

    def set_environment(self, env) -> None:
        """Upload a light probe (a bevy_hair_gb300.envmap.Environment), or drop it with None."""
        from . import envmap

        d, keep = envmap.env_desc(env)
        _check(self.lib, self.ctx, self.lib.hg_env_set(self.ctx, C.byref(d) if d is not None else None))

    def bind_surrogate(self, surrogate) -> None:
        """Make `surrogate` (a bevy_hair_gb300.surrogate.Surrogate, or None) the
        network that shade model 1 evaluates."""
        handle = surrogate.handle if surrogate is not None else None
        _check(self.lib, self.ctx, self.lib.hg_mlp_bind(self.ctx, handle))

    def close(self) -> None:
        if self.ctx:
            for s in list(getattr(self, "_surrogates", ())) + list(getattr(self, "_batches", ())):
                s.close()
            self.lib.hg_destroy(self.ctx)
            self.ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
