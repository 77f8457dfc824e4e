"""Extract the reference's known-answer tests for the hot path into
reference_kat.json.

Reads the Rust unit tests of the reference as text (they cannot run here:
there is no Rust toolchain) and records every literal input/expected pair:

* src/gbuffer.rs:65-104  -- G-buffer pack/unpack and beta side-channel word
* src/lod.rs:76-134      -- LOD selection, Eq. 1 strand counts, Eqs. 4-5
                            control points, viewport cull, Eq. 8, DOM slices
* src/render/pass.rs:1066-1090 and the shaders -- DOM_SIZE / DOM_LAYERS

Usage: python tests/golden/make_reference_kat.py [reference_root]
(default: the checkout named by the BEVY_HAIR_REFERENCE environment variable).
The JSON is committed; tests never read the reference tree.
"""
from __future__ import annotations

import json
import os
import re
import sys
from pathlib import Path

NUM = r"(-?[0-9_]+(?:\.[0-9_]+)?(?:e-?[0-9]+)?)"


def num(s: str) -> float:
    return float(s.replace("_", ""))


def intval(s: str) -> int:
    s = s.replace("_", "")
    return int(s, 16) if s.lower().startswith("0x") else int(s)


def extract(root: Path) -> dict:
    gb = (root / "src/gbuffer.rs").read_text()
    lod = (root / "src/lod.rs").read_text()
    out: dict = {"source": {}}

    # gbuffer: roundtrip sample
    m = re.search(r"depth:\s*(0x[0-9a-fA-F_]+),\s*tangent_oct:\s*\[(\d+),\s*(\d+)\],\s*uvw:\s*\[(\d+),\s*(\d+),\s*(\d+)\],"
                  r"\s*ao:\s*(\d+)", gb)
    out["gbuffer_roundtrip"] = {"depth": intval(m.group(1)), "tx": int(m.group(2)), "ty": int(m.group(3)),
                                "uvw": [int(m.group(4)), int(m.group(5)), int(m.group(6))], "ao": int(m.group(7))}
    samples = re.findall(r"depth:\s*(\d+),\s*tangent_oct:\s*\[(\d+),\s*(\d+)\],\s*uvw:\s*\[(\d+),\s*(\d+),\s*(\d+)\],"
                         r"\s*ao:\s*(\d+)", gb)
    far, near = samples[0], samples[1]
    out["gbuffer_order"] = {
        "far": {"depth": int(far[0]), "tx": int(far[1]), "ty": int(far[2]), "uvw": [int(x) for x in far[3:6]],
                "ao": int(far[6])},
        "near": {"depth": int(near[0]), "tx": int(near[1]), "ty": int(near[2]), "uvw": [int(x) for x in near[3:6]],
                 "ao": int(near[6])},
    }
    bw = re.findall(r"pack_beta_word\((\d+),\s*" + NUM + r"\)", gb)
    out["beta_word"] = {"far": [int(bw[0][0]), num(bw[0][1])], "near": [int(bw[1][0]), num(bw[1][1])],
                        "roundtrip": [int(bw[2][0]), num(bw[2][1])], "beta_tolerance": 1.0 / 255.0}
    out["source"]["gbuffer"] = "src/gbuffer.rs:65-104"

    # lod selection
    sel = []
    for a, b, c, rhs in re.findall(r"lod_selection\(" + NUM + r",\s*" + NUM + r",\s*" + NUM + r"\)\s*-\s*\(?([^)]+?)\)?\)\.abs\(\)",
                                   lod):
        expr = rhs.strip()
        if "/" in expr:
            n_, d_ = expr.split("/")
            expected = num(n_.strip()) / num(d_.strip())
        else:
            expected = num(expr)
        sel.append({"extent": num(a), "screen_h": num(b), "lambda": num(c), "expected": expected, "tol": 1e-5})
    for a, b, c, e in re.findall(r"assert_eq!\(lod_selection\(" + NUM + r",\s*" + NUM + r",\s*" + NUM + r"\),\s*" + NUM + r"\)",
                                 lod):
        sel.append({"extent": num(a), "screen_h": num(b), "lambda": num(c), "expected": num(e), "tol": 0.0})
    out["lod_selection"] = sel

    counts = []
    for l, n, d, culled, e in re.findall(r"assert_eq!\(strand_count_lod\(" + NUM + r",\s*(\d+),\s*" + NUM +
                                         r",\s*(true|false)\),\s*(\d+)\)", lod):
        counts.append({"l": num(l), "n": int(n), "delta": num(d), "culled": culled == "true", "expected": int(e)})
    m = re.search(r"let mid = strand_count_lod\(" + NUM + r",\s*(\d+),\s*" + NUM + r",\s*(true|false)\);\s*"
                  r"assert_eq!\(mid,\s*(\d+)\)", lod)
    counts.append({"l": num(m.group(1)), "n": int(m.group(2)), "delta": num(m.group(3)),
                   "culled": m.group(4) == "true", "expected": int(m.group(5))})
    out["strand_count_lod"] = counts

    cps = re.findall(r"control_point_count\(" + NUM + r",\s*(\d+)\)", lod)
    out["control_points"] = {"cases": [{"l": num(l), "layers": int(k)} for l, k in cps], "min": 3, "max": 127,
                             "rule": "C - 1 is a power of two"}

    cull = re.findall(r"(!?)aabb_outside_viewport\(\s*" + r",\s*".join([NUM] * 6) + r"\s*\)", lod)
    out["viewport_cull"] = [{"args": [num(x) for x in c[1:]], "outside": c[0] != "!"} for c in cull]

    dc = re.findall(r"depth_correction\(" + NUM + r"\)", lod)
    out["depth_correction"] = {"zero_at": num(dc[0]), "tol": 1e-4, "increasing_as_beta_falls": [num(x) for x in dc[1:]]}

    layers = re.search(r"let layers = \[([0-9,\s]+)\];", lod).group(1)
    slices = [int(x) for x in layers.split(",") if x.strip()]
    kat = []
    for t, e in re.findall(r"assert_eq!\(dom_optical_depth\(&layers,\s*" + NUM + r"\),\s*" + NUM + r"\)", lod):
        kat.append({"t": num(t), "expected": num(e), "tol": 0.0})
    for t, e in re.findall(r"\(dom_optical_depth\(&layers,\s*" + NUM + r"\)\s*-\s*" + NUM + r"\)\.abs\(\)", lod):
        kat.append({"t": num(t), "expected": num(e), "tol": 1e-4})
    out["dom_optical_depth"] = {"layers": slices, "cases": kat}
    out["source"]["lod"] = "src/lod.rs:76-134"

    pass_rs = (root / "src/render/pass.rs").read_text()
    out["constants"] = {
        "DOM_SIZE": int(re.search(r"pub const DOM_SIZE: u32 = (\d+);", pass_rs).group(1)),
        "DOM_LAYERS": int(re.search(r"pub const DOM_LAYERS: u32 = (\d+);", pass_rs).group(1)),
        "DOM_SIGMA": num(re.search(r"const DOM_SIGMA: f32 = " + NUM + ";", pass_rs).group(1)),
        "HAIR_PARAMS_SIZE": int(re.search(r"HAIR_PARAMS_SIZE: u64 = (\d+);",
                                          (root / "src/render/pipeline.rs").read_text()).group(1)),
        "LAYER_COUNT": int(re.search(r"pub const LAYER_COUNT: u32 = (\d+);", (root / "src/mesh.rs").read_text()).group(1)),
    }
    out["source"]["constants"] = "src/render/pass.rs:22-28, src/render/pipeline.rs:12, src/mesh.rs:10"
    return out


def main() -> None:
    if len(sys.argv) > 1:
        root = Path(sys.argv[1])
    elif os.environ.get("BEVY_HAIR_REFERENCE"):
        root = Path(os.environ["BEVY_HAIR_REFERENCE"])
    else:
        sys.exit("usage: make_reference_kat.py REFERENCE_ROOT (or set BEVY_HAIR_REFERENCE)")
    data = extract(root)
    dst = Path(__file__).with_name("reference_kat.json")
    dst.write_text(json.dumps(data, indent=1) + "\n")
    print("wrote", dst)


if __name__ == "__main__":
    main()
