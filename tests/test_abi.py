"""The C-ABI libraries load and export every function include/*.h declares;
struct layouts match the header.  No GPU work is done here."""
import ctypes as C
import re
from pathlib import Path

import numpy as np

from bevy_hair_gb300 import abi

INCLUDE = Path(__file__).resolve().parents[1] / "include"


def declared(header: str) -> list[str]:
    text = (INCLUDE / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*[A-Za-z_][\w\s\*]*?\b(hg_\w+)\s*\(", text, flags=re.M)))


def test_hairgb_exports_every_declared_symbol():
    lib = abi.load()
    names = declared("hairgb.h")
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(abi.exported_symbols())


def test_bake_exports_every_declared_symbol():
    lib = abi.load_bake()
    names = declared("hairgb_bake.h")
    assert names
    assert all(hasattr(lib, n) for n in names)


def test_struct_sizes_match_the_reference_layouts():
    assert abi.HAIR_PARAMS.itemsize == 432
    assert abi.GPU_BUNDLE.itemsize == 16
    assert abi.GPU_LAYER.itemsize == 32
    assert abi.LOD_RECORD.itemsize == 16
    assert abi.STRAND_REF.itemsize == 16
    assert abi.LIGHT.itemsize == 112
    # field offsets of HairParams (common.wgsl:10-28)
    offs = {n: abi.HAIR_PARAMS.fields[n][1] for n in abi.HAIR_PARAMS.names}
    assert offs["camera_pos"] == 256 and offs["flags"] == 352 and offs["pass_mode"] == 368 and offs["dom_info"] == 416


def test_status_strings_and_version():
    lib = abi.load()
    assert lib.hg_abi_version() == 1
    for s, text in abi.STATUS.items():
        assert lib.hg_status_string(s).decode() == text


def test_null_arguments_are_rejected_without_a_device():
    lib = abi.load()
    assert lib.hg_destroy(None) == abi.HG_INVALID_ARG
    assert lib.hg_clear(None) == abi.HG_INVALID_ARG
    assert lib.hg_create(0, None, None) == abi.HG_INVALID_ARG
    out = C.c_void_p()
    # an out-of-range device ordinal is an argument error, never a crash
    assert lib.hg_create(10_000, None, C.byref(out)) == abi.HG_INVALID_ARG
    assert lib.hg_last_error(None) == b"null context"
