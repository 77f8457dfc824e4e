"""The shade pass's light probe (shade.wesl:330-427): KTX2 + zstd + RGB9E5
decoding, the cubemap sampler, and probe_radiance on the GPU against the
oracle."""
import os
from pathlib import Path

import numpy as np
import pytest

import oracle
from bevy_hair_gb300 import abi, configs
from bevy_hair_gb300 import envmap as E

# The reference's own probes, when a checkout of it is named by
# BEVY_HAIR_REFERENCE (its assets/env/*.ktx2 are not part of this repository).
REF_ROOT = os.environ.get("BEVY_HAIR_REFERENCE")
REF_ENV = Path(REF_ROOT) / "assets" / "env" if REF_ROOT else None


@pytest.fixture(scope="module")
def env():
    return E.procedural(size=64, levels=7, diffuse_size=8)


# ------------------------------------------------------------------ CPU


def test_rgb9e5_known_values_and_round_trip():
    w = E.rgb9e5_encode(np.array([[1.0, 1.0, 1.0], [0.0, 0.0, 0.0], [0.5, 0.25, 0.125]]))
    # 1.0: exponent 16 (2^(16-24) * 256), mantissas 256
    assert int(w[0]) == 256 | (256 << 9) | (256 << 18) | (16 << 27)
    assert int(w[1]) == 0
    np.testing.assert_array_equal(E.rgb9e5_decode(w), [[1, 1, 1], [0, 0, 0], [0.5, 0.25, 0.125]])
    rng = np.random.default_rng(1)
    c = np.exp(rng.uniform(-8, 8, size=(5000, 3)))
    d = E.rgb9e5_decode(E.rgb9e5_encode(c))
    # each channel within half a mantissa step of the shared exponent (which
    # rounding of the largest channel can push up by one)
    step = np.ldexp(1.0, (np.floor(np.log2(c.max(axis=1))) - 8).astype(np.int64))
    assert (np.abs(d - c) <= step[:, None] * 1.0001).all()


def test_ktx2_round_trip(env):
    data = E.write_ktx2(env.specular)
    assert data[:12] == E.KTX2_ID
    back = E.read_ktx2(data)
    assert back.size == env.specular.size and len(back.levels) == len(env.specular.levels)
    for a, b in zip(back.levels, env.specular.levels):
        np.testing.assert_array_equal(a, b)
    with pytest.raises(ValueError):
        E.read_ktx2(b"not a ktx2 file" * 8)
    with pytest.raises(ValueError):
        E.read_ktx2(data[:-10])


@pytest.mark.skipif(REF_ENV is None or not REF_ENV.exists(),
                    reason="the reference's environment maps are not present (set BEVY_HAIR_REFERENCE)")
def test_reference_probe_files_decode():
    spec = E.load_ktx2(REF_ENV / "little_paris_eiffel_tower_2k_specular.ktx2")
    diff = E.load_ktx2(REF_ENV / "little_paris_eiffel_tower_2k_diffuse.ktx2")
    assert spec.size == 512 and len(spec.levels) == 9
    assert [l.shape for l in spec.levels] == [(6, 512 >> k, 512 >> k) for k in range(9)]
    assert diff.size == 32 and len(diff.levels) == 1
    for cube in (spec, diff):
        for l in cube.levels:
            v = E.rgb9e5_decode(l)
            assert np.isfinite(v).all() and (v >= 0).all()
    # prefiltered mips keep the mean radiance roughly
    m0 = E.rgb9e5_decode(spec.levels[0]).mean()
    m4 = E.rgb9e5_decode(spec.levels[4]).mean()
    assert 0.5 < m4 / m0 < 2.0


def test_sampler_reads_face_centres_and_interpolates_mips():
    # a map whose level l is the constant (l + 1) on face f times (f + 1)
    size, levels = 8, 4
    lv = []
    for l in range(levels):
        n = max(size >> l, 1)
        vals = np.array([(l + 1) * (f + 1) for f in range(6)], dtype=np.float64)
        lv.append(E.rgb9e5_encode(np.repeat(vals[:, None, None, None], 3, axis=3) * np.ones((6, n, n, 3))))
    tex = E.Cube(size, lv).packed()
    dirs = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
    for f, d in enumerate(dirs):
        np.testing.assert_allclose(oracle.sample_cube(tex, size, levels, d, 0.0), f + 1, rtol=1e-6)
        np.testing.assert_allclose(oracle.sample_cube(tex, size, levels, d, 1.25), (f + 1) * 2.25, rtol=1e-6)
        np.testing.assert_allclose(oracle.sample_cube(tex, size, levels, d, 99.0), (f + 1) * levels, rtol=1e-6)


def test_face_convention_matches_the_procedural_generator(env):
    # the generator bakes radiance(direction through each texel centre); the
    # sampler at that direction returns that texel exactly
    size, levels = env.specular.size, len(env.specular.levels)
    d = E._face_dirs(size)
    lvl0 = E.rgb9e5_decode(env.specular.levels[0])
    rng = np.random.default_rng(3)
    for _ in range(50):
        f, i, j = int(rng.integers(6)), int(rng.integers(size)), int(rng.integers(size))
        got = oracle.sample_cube(env.specular.packed(), size, levels, d[f, i, j], 0.0)
        np.testing.assert_allclose(got, lvl0[f, i, j], rtol=1e-5, atol=1e-7)


# ------------------------------------------------------------------ GPU


@pytest.fixture(scope="module")
def renderer():
    from bevy_hair_gb300.pipeline import HairRenderer

    r = HairRenderer(0)
    yield r
    r.close()


@pytest.mark.gpu
@pytest.mark.parametrize("model", [abi.SHADE_KARIS, abi.SHADE_SURROGATE, abi.SHADE_SURROGATE_COMPACT])
def test_probe_radiance_matches_the_oracle(renderer, env, model):
    from bevy_hair_gb300 import surrogate as S

    sc = configs.config2(scale=0.02)
    cam, dom = sc.params()
    lights = sc.light_array()
    renderer.ensure_targets(sc.view.width, sc.view.height, *sc.dom_size)
    g = renderer.upload(sc.mesh)
    renderer.render_groom(g, cam, dom, lights)
    assert renderer.synchronize() == 0
    center, beta, dmap = renderer.read(abi.BUF_CENTER), renderer.read(abi.BUF_BETA), renderer.read(abi.BUF_DOM)
    mlp = None
    s = None
    arch = abi.MLP_ARCH_COMPACT if model == abi.SHADE_SURROGATE_COMPACT else abi.MLP_ARCH_DEEP
    if model != abi.SHADE_KARIS:
        mlp = S.load_params(arch)
        s = S.Surrogate(renderer, mlp, arch)
        renderer.bind_surrogate(s)
    renderer.shade(cam, lights, model=model)
    renderer.synchronize()
    without = renderer.read(abi.BUF_SHADED).copy()
    e = E.Environment(env.specular, env.diffuse, rotation=(0.0, 0.38268343, 0.0, 0.92387953), intensity=1.7)
    renderer.set_environment(e)
    renderer.shade(cam, lights, model=model)
    assert renderer.synchronize() == 0
    got = renderer.read(abi.BUF_SHADED)
    want, _ = oracle.shade(cam, center, beta, dmap, lights, mlp=mlp, env=e, mlp_arch=arch)
    hit = center != np.uint64(0xFFFFFFFFFFFFFFFF)
    assert hit.sum() > 50
    g4, w4, n4 = got.reshape(-1, 4)[hit, :3], want.reshape(-1, 4)[hit, :3], without.reshape(-1, 4)[hit, :3]
    assert np.abs(g4 - n4).mean() > 1e-3  # the probe adds light
    err = np.abs(g4 - w4).sum() / np.abs(w4).sum()
    assert err < (2e-4 if model == abi.SHADE_KARIS else 2e-3), err
    np.testing.assert_allclose(g4, w4, rtol=3e-2, atol=1e-3 * np.abs(w4).max())
    renderer.set_environment(None)
    renderer.shade(cam, lights, model=model)
    renderer.synchronize()
    np.testing.assert_array_equal(renderer.read(abi.BUF_SHADED), without)
    if s is not None:
        renderer.bind_surrogate(None)
        s.close()
    g.close()


@pytest.mark.gpu
def test_env_argument_errors(renderer, env):
    bad = E.Environment(E.Cube(0, env.specular.levels), env.diffuse)
    with pytest.raises(abi.HairGbError):
        renderer.set_environment(bad)
    too_many = E.Environment(E.Cube(4, [np.zeros((6, 4, 4), np.uint32)] * 5), env.diffuse)
    with pytest.raises(abi.HairGbError):
        renderer.set_environment(too_many)
