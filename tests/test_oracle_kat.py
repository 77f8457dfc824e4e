"""The oracle against every known-answer test the reference holds for the
hot path (tests/golden/reference_kat.json, extracted from src/gbuffer.rs:65-104
and src/lod.rs:76-134 by tests/golden/make_reference_kat.py)."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

import oracle

KAT = json.loads((Path(__file__).parent / "golden" / "reference_kat.json").read_text())
L = oracle.lib()
EMPTY = (1 << 64) - 1


def unpack(word):
    out = np.zeros(7, dtype=np.uint32)
    L.oracle_unpack_gb(word, out.ctypes.data)
    return [int(x) for x in out]


def pack(s):
    return L.oracle_pack_gb(s["depth"], s["tx"], s["ty"], *s["uvw"], s["ao"])


def test_gbuffer_roundtrip_preserves_fields():
    s = KAT["gbuffer_roundtrip"]
    word = pack(s)
    assert word != EMPTY
    d, tx, ty, u, v, w, ao = unpack(word)
    assert (d, tx, ty, [u, v, w], ao) == (s["depth"], s["tx"], s["ty"], s["uvw"], s["ao"])


def test_gbuffer_closer_depth_is_numerically_smaller():
    far, near = pack(KAT["gbuffer_order"]["far"]), pack(KAT["gbuffer_order"]["near"])
    assert near < far < EMPTY


def test_gbuffer_layout_is_depth24_oct16_uvw18_ao6():
    # field positions of src/gbuffer.rs:19-28
    assert L.oracle_pack_gb(1, 0, 0, 0, 0, 0, 0) == 1 << 40
    assert L.oracle_pack_gb(0, 1, 0, 0, 0, 0, 0) == 1 << 32
    assert L.oracle_pack_gb(0, 0, 1, 0, 0, 0, 0) == 1 << 24
    assert L.oracle_pack_gb(0, 0, 0, 1, 0, 0, 0) == 1 << 18
    assert L.oracle_pack_gb(0, 0, 0, 0, 1, 0, 0) == 1 << 12
    assert L.oracle_pack_gb(0, 0, 0, 0, 0, 1, 0) == 1 << 6
    assert L.oracle_pack_gb(0, 0, 0, 0, 0, 0, 1) == 1
    assert L.oracle_pack_gb(0xFFFFFE, 255, 255, 63, 63, 63, 63) < EMPTY


def test_beta_word_orders_by_depth():
    b = KAT["beta_word"]
    far = L.oracle_pack_beta(*b["far"])
    near = L.oracle_pack_beta(*b["near"])
    assert near < far
    word = L.oracle_pack_beta(*b["roundtrip"])
    assert word >> 8 == b["roundtrip"][0]
    assert abs((word & 0xFF) / 255.0 - b["roundtrip"][1]) < b["beta_tolerance"]


@pytest.mark.parametrize("case", KAT["lod_selection"])
def test_lod_selection(case):
    got = L.oracle_lod_selection(case["extent"], case["screen_h"], case["lambda"])
    assert abs(got - case["expected"]) <= max(case["tol"], 1e-7)


@pytest.mark.parametrize("case", KAT["strand_count_lod"])
def test_strand_count_respects_cull_and_bounds(case):
    got = L.oracle_strand_count_lod(case["l"], case["n"], case["delta"], int(case["culled"]))
    assert got == case["expected"]


def test_control_points_snap_to_power_of_two_plus_one():
    rule = KAT["control_points"]
    for case in rule["cases"]:
        c = L.oracle_control_points_for_lod(case["l"])
        assert rule["min"] <= c <= rule["max"]
        assert bin(c - 1).count("1") == 1
    # the full sweep of L gives exactly the four LOD levels of Eqs. 4-5
    levels = {L.oracle_control_points_for_lod(float(l)) for l in np.linspace(0, 1, 2001)}
    assert levels == {9, 17, 33, 65}
    assert L.oracle_control_points_for_lod(1.0) == 65


@pytest.mark.parametrize("case", KAT["viewport_cull"])
def test_viewport_cull(case):
    mnx, mny, mxx, mxy, w, h = case["args"]
    outside = mxx < 0 or mxy < 0 or mnx > w or mny > h  # lod.wgsl:312-313
    assert outside == case["outside"]


def test_depth_correction_grows_as_strands_are_removed():
    dc = KAT["depth_correction"]
    assert abs(L.oracle_depth_correction(dc["zero_at"])) < dc["tol"]
    pairs = dc["increasing_as_beta_falls"]
    for lo_beta, hi_beta in zip(pairs[0::2], pairs[1::2]):
        assert L.oracle_depth_correction(lo_beta) > L.oracle_depth_correction(hi_beta)


@pytest.mark.parametrize("case", KAT["dom_optical_depth"]["cases"])
def test_deep_opacity_ignores_hair_at_or_behind_the_sample(case):
    layers = np.array(KAT["dom_optical_depth"]["layers"], dtype=np.uint32)
    got = L.oracle_dom_optical_depth(layers.ctypes.data, len(layers), case["t"])
    if case["tol"] == 0.0:
        assert got == case["expected"]
    else:
        assert abs(got - case["expected"]) < case["tol"]


def test_shader_constants_match_the_buffer_layout():
    from bevy_hair_gb300 import abi

    c = KAT["constants"]
    assert abi.DOM_LAYERS == c["DOM_LAYERS"]
    assert abi.LAYER_COUNT == c["LAYER_COUNT"]
    assert abi.HAIR_PARAMS.itemsize == c["HAIR_PARAMS_SIZE"]
    from bevy_hair_gb300 import host

    assert float(host.DOM_SIGMA) == pytest.approx(c["DOM_SIGMA"])


def test_quantize_depth_range_and_sentinel():
    assert L.oracle_quantize_depth(0.0, 1.0, 2.0) == 0
    assert L.oracle_quantize_depth(5.0, 1.0, 2.0) == 0xFFFFFE  # never the empty sentinel
    assert L.oracle_quantize_depth(float("nan"), 1.0, 2.0) == 0
    q = L.oracle_quantize_depth(1.5, 1.0, 2.0)
    assert abs(L.oracle_dequantize_depth(q, 1.0, 2.0) - 1.5) < 1e-6


def test_oct_roundtrip_is_close():
    rng = np.random.default_rng(1)
    for _ in range(200):
        n = rng.normal(size=3).astype(np.float32)
        n /= np.linalg.norm(n)
        o = np.zeros(2, dtype=np.uint32)
        L.oracle_oct_encode(n.ctypes.data, o.ctypes.data)
        back = np.zeros(3, dtype=np.float32)
        L.oracle_oct_decode(int(o[0]), int(o[1]), back.ctypes.data)
        assert np.dot(back, n) > 0.999 - 1e-3


def test_pcg_matches_the_wgsl_hash():
    # common.wgsl:56-60 evaluated with Python integers modulo 2^32
    def pcg(x):
        state = (x * 747796405 + 2891336453) & 0xFFFFFFFF
        word = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & 0xFFFFFFFF
        return ((word >> 22) ^ word) & 0xFFFFFFFF

    for x in [0, 1, 2, 0x9E3779B9, 0xFFFFFFFF, 123456789]:
        assert L.oracle_pcg(x) == pcg(x)
