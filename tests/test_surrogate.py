"""The learned shading surrogate: its FP64 reference lobes, the FP16 tensor-core network
(inference, gradients, training) and shade model 1.

CPU tests pin the FP64 lobe integrator against an independent brute-force
integration and the FP64 network reference against finite differences.  GPU
tests call libhairgb.so through the C ABI: the GPU sample generator against
the CPU integrator, the network's forward pass against the oracle's FP16
emulation, its gradients against the FP64 reference, a short training run,
shade model 1 against the oracle, and the shipped weights' error against the
Karis fit's.
"""
import math

import numpy as np
import pytest

import oracle
from oracle import mlp_ref
from bevy_hair_gb300 import abi, configs, surrogate as S

TILT = float(np.float32(S.TILT))
EMPTY = np.uint64(0xFFFFFFFFFFFFFFFF)


def _inputs(n: int, seed: int) -> np.ndarray:
    """Raw inputs drawn from the training distribution, as float32 values."""
    rng = np.random.default_rng(seed)
    x = np.zeros((n, 10))
    x[:, 0] = rng.uniform(-1, 1, n)
    x[:, 1] = rng.uniform(-1, 1, n)
    phi = rng.uniform(0, np.pi, n)
    x[:, 2], x[:, 3] = np.cos(phi), np.sin(phi)
    x[:, 4:7] = np.exp(rng.uniform(np.log(0.02), np.log(8.0), (n, 3)))
    x[:, 7] = rng.uniform(0.03, 0.3, n)
    x[:, 8] = rng.uniform(0.2, 0.8, n)
    x[:, 9] = 1.55
    return x.astype(np.float32)


# ------------------------------------------------------------------ CPU


def _brute_lobes(x: np.ndarray, tilt: float, m: int = 20001) -> np.ndarray:
    """The 12 lobes by composite Simpson over h = sin(u) on a fine grid and the
    wrapped Gaussian summed over 7 periods: an independent check of the
    oracle's Gauss-Legendre integrator."""
    from scipy.special import erf

    def wrapped(d, s):
        d = np.remainder(d + np.pi, 2 * np.pi) - np.pi
        return sum(np.exp(-0.5 * ((d + 2 * np.pi * k) / s) ** 2) for k in range(-3, 4)) / (math.sqrt(2 * np.pi) * s)

    def mass(a, b, c, s):
        r = 1.0 / (s * math.sqrt(2.0))
        return sum(0.5 * (erf((b - c - 2 * np.pi * k) * r) - erf((a - c - 2 * np.pi * k) * r)) for k in range(-4, 5))

    def fresnel(c, eta):
        c = np.clip(c, 0.0, 1.0)
        st2 = (1 - c * c) / eta ** 2
        ct = np.sqrt(np.maximum(1 - st2, 0.0))
        rs, rp = (c - eta * ct) / (c + eta * ct), (eta * c - ct) / (eta * c + ct)
        return np.where(st2 >= 1, 1.0, 0.5 * (rs * rs + rp * rp))

    def gauss(b, v):
        b = max(b, 1e-3)
        return math.exp(-0.5 * v * v / (b * b)) / (math.sqrt(2 * np.pi) * b)

    u = np.linspace(-np.pi / 2, np.pi / 2, m)
    h = np.sin(u)
    w = np.ones(m)
    w[1:-1:2], w[2:-1:2] = 4.0, 2.0
    w *= (u[1] - u[0]) / 3.0 * np.cos(u)

    def terms(cos_td, sin_td, sa, eta):
        eta_p = math.sqrt(eta * eta - sin_td ** 2) / cos_td
        stt = sin_td / eta
        ctt = math.sqrt(1 - stt * stt)
        gt = np.arcsin(h / eta_p)
        f = fresnel(cos_td * np.cos(u), eta)
        a = np.zeros((3, 3, m))
        for c in range(3):
            t = np.exp(-sa[c] * 2 * np.cos(gt) / ctt)
            a[0, c], a[1, c], a[2, c] = f, (1 - f) ** 2 * t, (1 - f) ** 2 * f * t * t
        return a, [2 * p * gt - 2 * u + p * np.pi for p in range(3)]

    x = x.astype(np.float64)
    si, so = float(np.clip(x[0], -1, 1)), float(np.clip(x[1], -1, 1))
    phi = math.atan2(x[3], x[2])
    sa, bm, bn, eta = x[4:7], x[7], x[8], x[9]
    ti, to = math.asin(si), math.asin(so)
    th = ti + to
    al, be = [tilt, -0.5 * tilt, -1.5 * tilt], [bm, 0.5 * bm, 2 * bm]
    out = np.zeros(12)
    td = 0.5 * (to - ti)
    a, ph = terms(max(math.cos(td), 1e-3), math.sin(td), sa, eta)
    for p in range(3):
        d = wrapped(phi - ph[p], bn)
        for c in range(3):
            out[3 * p + c] = gauss(be[p], th - al[p]) * 0.5 * np.sum(w * a[p, c] * d)
    cto = max(math.sqrt(max(1 - so * so, 1e-6)), 1e-3)
    a, ph = terms(cto, math.sqrt(max(0.0, 1 - cto * cto)), sa, eta)
    fwd, back = np.zeros((3, 3)), np.zeros((3, 3))
    for p in range(3):
        mb, mf = mass(-np.pi / 2, np.pi / 2, ph[p], bn), mass(np.pi / 2, 1.5 * np.pi, ph[p], bn)
        for c in range(3):
            back[p, c] = 0.5 * np.sum(w * a[p, c] * mb)
            fwd[p, c] = 0.5 * np.sum(w * a[p, c] * mf)
    b2 = np.array(be) ** 2
    for c in range(3):
        f, b = fwd[:, c], back[:, c]
        af, ab = min(f.sum(), 0.95), b.sum()
        bf2 = (f * b2).sum() / max(af, 1e-5)
        alb = (b * np.array(al)).sum() / max(ab, 1e-5)
        bb2 = (b * b2).sum() / max(ab, 1e-5)
        af2, ab2 = af * af, ab * ab
        rest, ab3 = 1 - af2, ab2 * ab
        a_back = ab * af2 / rest + ab3 * af2 / rest ** 3
        db = alb * (1 - 2 * ab2 / rest ** 2) + alb * (2 * rest * rest + 4 * af2 * ab2) / rest ** 3
        sb = (1 + 0.7 * af2) * (ab * math.sqrt(2 * bf2 + bb2) + ab3 * math.sqrt(2 * bf2 + 3 * bb2)) / max(
            ab + ab3 * (2 * math.sqrt(bf2) + 3 * math.sqrt(bb2)), 1e-5)
        out[9 + c] = 2 * a_back * gauss(sb, th - db) / np.pi
    return out


def test_fp64_lobes_match_brute_force_integration():
    x = _inputs(24, 5)
    got = oracle.lobes(x, tilt=TILT)
    want = np.array([_brute_lobes(v, TILT) for v in x])
    assert np.isfinite(got).all() and (got >= 0).all()
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-300)


def test_fp64_lobes_are_even_in_phi():
    x = _inputs(64, 6)
    y = x.copy()
    y[:, 3] = -y[:, 3]
    np.testing.assert_allclose(oracle.lobes(x, tilt=TILT), oracle.lobes(y, tilt=TILT), rtol=1e-12, atol=0)


def test_karis_fit_is_far_from_the_fp64_lobes():
    """The reason for the surrogate: the Karis fits miss the exact lobes by
    tens of percent on the training distribution."""
    x = _inputs(4000, 7)
    exact = oracle.lobes(x, tilt=TILT)
    karis = oracle.lobes(x, model="karis", tilt=TILT)
    assert S.relative_l1(S.bsdf(karis), S.bsdf(exact)) > 0.2


def test_fp64_network_reference_matches_finite_differences():
    p = S.init_params(3).astype(np.float64)
    x = _inputs(48, 8)
    t = np.random.default_rng(9).normal(size=(48, 12))
    g, _ = mlp_ref.gradients(p, x, t, half=False)
    for idx in (3, 700, 1100, 3000, 5300, 9000, 13600, 14595, 14600):
        e = 1e-6
        a, b = p.copy(), p.copy()
        a[idx] += e
        b[idx] -= e
        fd = (mlp_ref.gradients(a, x, t, half=False)[1] - mlp_ref.gradients(b, x, t, half=False)[1]) / (2 * e)
        assert abs(fd - g[idx]) <= 1e-6 * max(1.0, abs(fd)), (idx, fd, g[idx])


def test_oracle_network_emulation_matches_fp64_reference():
    p = S.init_params(4)
    x = _inputs(256, 10)
    got = oracle.mlp_forward(p, x)
    want, _, _ = mlp_ref.forward(p, x)
    np.testing.assert_allclose(got, want[:, :12], rtol=0, atol=3e-3)


def test_init_params_keep_padding_zero():
    p = S.init_params(0)
    layers = S.split(p)
    assert (layers[0][0][:, 10:] == 0).all()
    assert (layers[4][0][12:, :] == 0).all() and (layers[4][1] == 0).all()


def test_shipped_weights_have_the_parameter_layout():
    p = S.load_params()
    assert p.shape == (abi.MLP_PARAMS,) and np.isfinite(p).all()
    layers = S.split(p)
    assert (layers[0][0][:, 10:] == 0).all() and (layers[4][0][12:, :] == 0).all()


# ------------------------------------------------------------------ GPU

gpu = pytest.mark.gpu


@pytest.fixture(scope="module")
def renderer():
    from bevy_hair_gb300.pipeline import HairRenderer

    r = HairRenderer(0)
    yield r
    r.close()


def _torch():
    torch = pytest.importorskip("torch")
    return torch, torch.device("cuda", 0)


@gpu
def test_gpu_samples_match_the_fp64_integrator(renderer):
    torch, dev = _torch()
    n = 4096
    x = torch.empty((n, 10), dtype=torch.float32, device=dev)
    t = torch.empty((n, 12), dtype=torch.float32, device=dev)
    lob = torch.empty((n, 12), dtype=torch.float64, device=dev)
    S.samples(renderer, 1234, 0, n, x, t, lob)
    renderer.synchronize()
    xs, ts, ls = x.cpu().numpy(), t.cpu().numpy(), lob.cpu().numpy()
    assert (np.abs(xs[:, :2]) <= 1).all() and (xs[:, 3] >= 0).all()
    assert (xs[:, 4:7] >= 0.0199).all() and (xs[:, 4:7] <= 8.01).all()
    assert (xs[:, 7] >= 0.03).all() and (xs[:, 7] <= 0.3).all() and (xs[:, 9] == np.float32(1.55)).all()
    want = oracle.lobes(xs, tilt=TILT)
    np.testing.assert_allclose(ls, want, rtol=1e-10, atol=1e-14)
    scale = float(np.float32(1e-3))  # the kernel divides by the float constant, widened
    np.testing.assert_allclose(ts, np.log1p(ls / scale).astype(np.float32), rtol=1e-6, atol=1e-44)
    # sample k depends on (seed, first + k) only
    x2 = torch.empty((16, 10), dtype=torch.float32, device=dev)
    S.samples(renderer, 1234, 100, 16, x2)
    renderer.synchronize()
    np.testing.assert_array_equal(x2.cpu().numpy(), xs[100:116])


@gpu
def test_karis_lobes_kernel_matches_the_fp64_karis_fit(renderer):
    torch, dev = _torch()
    xs = _inputs(4096, 11)
    x = torch.from_numpy(xs).to(dev)
    out = torch.empty((len(xs), 12), dtype=torch.float32, device=dev)
    S.karis_lobes(renderer, x, len(xs), out)
    renderer.synchronize()
    want = oracle.lobes(xs, model="karis", tilt=TILT)
    got = out.cpu().numpy()
    assert S.relative_l1(got, want) < 1e-4
    np.testing.assert_allclose(got, want, rtol=5e-3, atol=1e-6 * np.abs(want).max())


@gpu
@pytest.mark.parametrize("which", ["init", "shipped"])
def test_network_forward_matches_the_oracle_emulation(renderer, which):
    torch, dev = _torch()
    p = S.init_params(5) if which == "init" else S.load_params()
    s = S.Surrogate(renderer, p)
    xs = _inputs(5000, 12)
    x = torch.from_numpy(xs).to(dev)
    net = torch.empty((len(xs), 12), dtype=torch.float32, device=dev)
    lob = torch.empty((len(xs), 12), dtype=torch.float32, device=dev)
    s.infer(x, len(xs), lob, net)
    renderer.synchronize()
    got, want = net.cpu().numpy(), oracle.mlp_forward(p, xs)
    # One FP16 step (2^-11 relative) in an activation moves an output by ~1e-3.
    assert np.abs(got - want).mean() < 2e-3
    np.testing.assert_allclose(got, want, rtol=0, atol=5e-2)
    np.testing.assert_allclose(lob.cpu().numpy(), 1e-3 * np.expm1(np.maximum(got, 0)), rtol=1e-5, atol=1e-9)
    s.close()


@gpu
@pytest.mark.parametrize("n", [5000, 128, 77])
def test_tcgen05_inference_matches_mma_sync_and_the_oracle(renderer, n):
    torch, dev = _torch()
    p = S.load_params()
    s = S.Surrogate(renderer, p)
    xs = _inputs(n, 13)
    x = torch.from_numpy(xs).to(dev)
    net_tc = torch.full((n, 12), float("nan"), dtype=torch.float32, device=dev)
    lob_tc = torch.empty((n, 12), dtype=torch.float32, device=dev)
    net_ms = torch.empty((n, 12), dtype=torch.float32, device=dev)
    s.infer_tc(x, n, lob_tc, net_tc)
    s.infer(x, n, None, net_ms)
    assert renderer.synchronize() == 0
    tc, ms = net_tc.cpu().numpy(), net_ms.cpu().numpy()
    assert np.isfinite(tc).all()
    want = oracle.mlp_forward(p, xs)
    assert np.abs(tc - ms).mean() < 2e-3 and np.abs(tc - want).mean() < 2e-3
    np.testing.assert_allclose(tc, ms, rtol=0, atol=5e-2)
    np.testing.assert_allclose(lob_tc.cpu().numpy(), 1e-3 * np.expm1(np.maximum(tc, 0)), rtol=1e-5, atol=1e-9)
    s.close()


@gpu
def test_gradients_match_the_fp64_reference(renderer):
    torch, dev = _torch()
    n = 3000  # not a multiple of 32: the ragged last warp must contribute nothing extra
    x = torch.empty((n, 10), dtype=torch.float32, device=dev)
    t = torch.empty((n, 12), dtype=torch.float32, device=dev)
    S.samples(renderer, 77, 0, n, x, t)
    p = S.init_params(6)
    s = S.Surrogate(renderer, p)
    g, loss = s.gradients(x, t, n)
    xs, ts = x.cpu().numpy(), t.cpu().numpy()
    want, want_loss = mlp_ref.gradients(p, xs, ts)
    assert loss == pytest.approx(want_loss, rel=2e-3)
    err = np.linalg.norm(g - want) / np.linalg.norm(want)
    cos = float(g @ want / (np.linalg.norm(g) * np.linalg.norm(want)))
    assert err < 2e-2 and cos > 0.9995, (err, cos)
    for k, ((gw, gb), (ww, wb)) in enumerate(zip(S.split(g), S.split(want.astype(np.float32)))):
        assert np.linalg.norm(gw - ww) <= 3e-2 * np.linalg.norm(ww) + 1e-6, k
        assert np.linalg.norm(gb - wb) <= 3e-2 * np.linalg.norm(wb) + 1e-6, k
    # padding stays exactly zero
    assert (S.split(g)[0][0][:, 10:] == 0).all() and (S.split(g)[4][0][12:, :] == 0).all()
    # the parameters did not move
    np.testing.assert_array_equal(s.get_params(), p)
    s.close()


@gpu
def test_training_reduces_the_loss(renderer):
    torch, dev = _torch()
    n, batch = 1 << 18, 8192
    x = torch.empty((n, 10), dtype=torch.float32, device=dev)
    t = torch.empty((n, 12), dtype=torch.float32, device=dev)
    S.samples(renderer, 99, 0, n, x, t)
    s = S.Surrogate(renderer, S.init_params(7))
    steps = 300
    losses = torch.zeros(steps, dtype=torch.float32, device=dev)
    for k in range(steps):
        lo = (k % (n // batch)) * batch
        s.train_step(x[lo:lo + batch], t[lo:lo + batch], batch, 2e-3, losses[k:k + 1])
    renderer.synchronize()
    l = losses.cpu().numpy() / (batch * 12)
    assert np.isfinite(l).all()
    assert l[-20:].mean() < 0.2 * l[:5].mean(), (l[:5], l[-20:])
    p = s.get_params()
    assert (S.split(p)[0][0][:, 10:] == 0).all() and (S.split(p)[4][0][12:, :] == 0).all()
    s.close()


@gpu
@pytest.mark.parametrize("model", [abi.SHADE_SURROGATE, abi.SHADE_SURROGATE_MMA])
def test_shade_model_one_matches_the_oracle(renderer, model):
    sc = configs.config2(scale=0.02)
    cam, dom = sc.params()
    lights = sc.light_array()
    w, h = sc.view.width, sc.view.height
    renderer.ensure_targets(w, h, *sc.dom_size)
    g = renderer.upload(sc.mesh)
    renderer.render_groom(g, cam, dom, lights)  # G-buffer and map
    assert renderer.synchronize() == 0
    with pytest.raises(abi.HairGbError):
        renderer.shade(cam, lights, model=model)  # nothing bound
    p = S.load_params()
    s = S.Surrogate(renderer, p)
    renderer.bind_surrogate(s)
    renderer.shade(cam, lights, model=model)
    assert renderer.synchronize() == 0
    center, beta, dmap = renderer.read(abi.BUF_CENTER), renderer.read(abi.BUF_BETA), renderer.read(abi.BUF_DOM)
    shaded, sdepth = renderer.read(abi.BUF_SHADED), renderer.read(abi.BUF_SHADED_DEPTH)
    o_shaded, o_sdepth = oracle.shade(cam, center, beta, dmap, lights, mlp=p)
    hit = center != EMPTY
    assert hit.sum() > 50
    np.testing.assert_array_equal(sdepth, o_sdepth)
    assert np.isfinite(shaded).all()
    got, want = shaded.reshape(-1, 4)[hit, :3], o_shaded.reshape(-1, 4)[hit, :3]
    assert S.relative_l1(got, want) < 2e-3
    np.testing.assert_allclose(got, want, rtol=3e-2, atol=1e-3 * np.abs(want).max())
    # the frame entry point takes the same model
    renderer.render_groom(g, cam, dom, lights, model=model)
    assert renderer.synchronize() == 0
    np.testing.assert_array_equal(renderer.read(abi.BUF_SHADED), shaded)
    renderer.bind_surrogate(None)
    s.close()
    g.close()


@gpu
def test_shipped_surrogate_beats_the_karis_fit(renderer):
    s = S.Surrogate(renderer, S.load_params())
    ev = S.evaluate(renderer, s, n=1 << 15)
    s.close()
    assert ev["karis_bsdf"] > 0.2
    assert ev["surrogate_bsdf"] < 0.25 * ev["karis_bsdf"], ev


# ------------------------------------------------------------------ compact network (shade model 3)

COMPACT = abi.MLP_ARCH_COMPACT


def test_compact_fp64_reference_matches_finite_differences():
    p = S.init_params(13, COMPACT).astype(np.float64)
    x = _inputs(48, 14)
    t = np.random.default_rng(15).uniform(0.0, 3.0, size=(48, 12))  # transformed lobes
    g, _ = mlp_ref.gradients(p, x, t, half=False, arch=COMPACT)
    assert g.shape == (abi.MLP_COMPACT_PARAMS,)
    for idx in (5, 300, 520, 700, 1500, 1570, 1700, 2100, 2115):
        e = 1e-6
        a, b = p.copy(), p.copy()
        a[idx] += e
        b[idx] -= e
        fd = (mlp_ref.gradients(a, x, t, half=False, arch=COMPACT)[1]
              - mlp_ref.gradients(b, x, t, half=False, arch=COMPACT)[1]) / (2 * e)
        assert abs(fd - g[idx]) <= 1e-6 * max(1.0, abs(fd)), (idx, fd, g[idx])


def test_compact_oracle_emulation_matches_fp64_reference():
    p = S.init_params(16, COMPACT)
    x = _inputs(256, 17)
    got = oracle.mlp_forward(p, x, arch=COMPACT)
    want, _, _ = mlp_ref.forward(p, x, arch=COMPACT)
    assert got.shape == (256, abi.MLP_COMPACT_OUTPUTS)
    np.testing.assert_allclose(got, want[:, :3], rtol=0, atol=3e-3)


def test_compact_targets_are_the_per_light_bsdf():
    rng = np.random.default_rng(23)
    lobes = rng.uniform(0.0, 2.0, size=(64, 12))
    t12 = np.log1p(lobes / 1e-3)
    want = np.log1p(S.bsdf(lobes) / 1e-3)
    np.testing.assert_allclose(mlp_ref.bsdf_targets(t12), want, rtol=1e-12)


def test_compact_init_params_keep_padding_zero():
    p = S.init_params(0, COMPACT)
    layers = S.split(p, COMPACT)
    assert [w.shape for w, _ in layers] == [(32, 16), (32, 32), (16, 32)]
    assert (layers[0][0][:, 10:] == 0).all()
    assert (layers[2][0][abi.MLP_COMPACT_OUTPUTS:, :] == 0).all() and (layers[2][1] == 0).all()


def test_shipped_compact_weights_have_the_parameter_layout():
    p = S.load_params(COMPACT)
    assert p.shape == (abi.MLP_COMPACT_PARAMS,) and np.isfinite(p).all()
    layers = S.split(p, COMPACT)
    assert (layers[0][0][:, 10:] == 0).all() and (layers[2][0][abi.MLP_COMPACT_OUTPUTS:, :] == 0).all()


@gpu
def test_compact_surrogate_entry_points_check_the_architecture(renderer):
    s = S.Surrogate(renderer, None, COMPACT)
    assert s.n_params == abi.MLP_COMPACT_PARAMS and s.n_out == abi.MLP_COMPACT_OUTPUTS
    with pytest.raises(abi.HairGbError):
        s.set_params(S.init_params(0))  # 4 x 64 parameter count
    torch, dev = _torch()
    x = torch.from_numpy(_inputs(64, 18)).to(dev)
    out = torch.empty((64, 3), dtype=torch.float32, device=dev)
    with pytest.raises(abi.HairGbError):
        s.infer_tc(x, 64, out)  # tcgen05 inference is for the 4 x 64 network
    s.close()
    with pytest.raises(abi.HairGbError):
        S.Surrogate(renderer, None, 7)


@gpu
@pytest.mark.parametrize("which", ["init", "shipped"])
def test_compact_forward_matches_the_oracle_emulation(renderer, which):
    torch, dev = _torch()
    p = S.init_params(19, COMPACT) if which == "init" else S.load_params(COMPACT)
    s = S.Surrogate(renderer, p, COMPACT)
    for n in (5000, 77):
        xs = _inputs(n, 20)
        x = torch.from_numpy(xs).to(dev)
        # one extra row each: the kernel writes n rows of 3, nothing past them
        net = torch.full((n + 1, 3), float("nan"), dtype=torch.float32, device=dev)
        lob = torch.full((n + 1, 3), -7.0, dtype=torch.float32, device=dev)
        s.infer(x, n, lob, net)
        assert renderer.synchronize() == 0
        got_all, lob_all = net.cpu().numpy(), lob.cpu().numpy()
        assert np.isnan(got_all[n]).all() and (lob_all[n] == -7.0).all()
        got, want = got_all[:n], oracle.mlp_forward(p, xs, arch=COMPACT)
        assert np.isfinite(got).all()
        assert np.abs(got - want).mean() < 1e-3
        np.testing.assert_allclose(got, want, rtol=0, atol=3e-2)
        np.testing.assert_allclose(lob_all[:n], 1e-3 * np.expm1(np.maximum(got, 0)), rtol=1e-5, atol=1e-9)
    s.close()


@gpu
def test_compact_gradients_match_the_fp64_reference(renderer):
    torch, dev = _torch()
    n = 3000  # not a multiple of 32: the ragged last block must contribute nothing extra
    x = torch.empty((n, 10), dtype=torch.float32, device=dev)
    t = torch.empty((n, 12), dtype=torch.float32, device=dev)
    S.samples(renderer, 78, 0, n, x, t)
    p = S.init_params(21, COMPACT)
    s = S.Surrogate(renderer, p, COMPACT)
    g, loss = s.gradients(x, t, n)
    xs, ts = x.cpu().numpy(), t.cpu().numpy()
    want, want_loss = mlp_ref.gradients(p, xs, ts, arch=COMPACT)
    assert loss == pytest.approx(want_loss, rel=1e-3)
    # the backward pass runs on the tensor cores from the FP16-rounded forward activations, with FP16 deltas
    err = np.linalg.norm(g - want) / np.linalg.norm(want)
    cos = float(g @ want / (np.linalg.norm(g) * np.linalg.norm(want)))
    assert err < 5e-3 and cos > 0.99999, (err, cos)
    for k, ((gw, gb), (ww, wb)) in enumerate(zip(S.split(g, COMPACT), S.split(want.astype(np.float32), COMPACT))):
        assert np.linalg.norm(gw - ww) <= 1e-2 * np.linalg.norm(ww) + 1e-6, k
        assert np.linalg.norm(gb - wb) <= 1e-2 * np.linalg.norm(wb) + 1e-6, k
    assert (S.split(g, COMPACT)[0][0][:, 10:] == 0).all() and (S.split(g, COMPACT)[2][0][3:, :] == 0).all()
    np.testing.assert_array_equal(s.get_params(), p)
    s.close()


@gpu
def test_compact_training_reduces_the_loss(renderer):
    torch, dev = _torch()
    n, batch = 1 << 18, 8192
    x = torch.empty((n, 10), dtype=torch.float32, device=dev)
    t = torch.empty((n, 12), dtype=torch.float32, device=dev)
    S.samples(renderer, 98, 0, n, x, t)
    s = S.Surrogate(renderer, S.init_params(22, COMPACT), COMPACT)
    steps = 300
    losses = torch.zeros(steps, dtype=torch.float32, device=dev)
    for k in range(steps):
        lo = (k % (n // batch)) * batch
        s.train_step(x[lo:lo + batch], t[lo:lo + batch], batch, 3e-3, losses[k:k + 1])
    renderer.synchronize()
    l = losses.cpu().numpy() / (batch * 12)
    assert np.isfinite(l).all()
    assert l[-20:].mean() < 0.25 * l[:5].mean(), (l[:5], l[-20:])
    p = s.get_params()
    assert (S.split(p, COMPACT)[0][0][:, 10:] == 0).all() and (S.split(p, COMPACT)[2][0][3:, :] == 0).all()
    s.close()


@gpu
def test_shade_model_three_matches_the_oracle(renderer):
    sc = configs.config2(scale=0.02)
    cam, dom = sc.params()
    lights = sc.light_array()
    w, h = sc.view.width, sc.view.height
    renderer.ensure_targets(w, h, *sc.dom_size)
    g = renderer.upload(sc.mesh)
    renderer.render_groom(g, cam, dom, lights)
    assert renderer.synchronize() == 0
    deep = S.Surrogate(renderer, S.load_params())
    renderer.bind_surrogate(deep)
    with pytest.raises(abi.HairGbError):
        renderer.shade(cam, lights, model=abi.SHADE_SURROGATE_COMPACT)  # model 3 takes the compact network
    p = S.load_params(COMPACT)
    s = S.Surrogate(renderer, p, COMPACT)
    renderer.bind_surrogate(s)
    with pytest.raises(abi.HairGbError):
        renderer.shade(cam, lights, model=abi.SHADE_SURROGATE_MMA)  # models 1 and 2 take the 4 x 64 one
    renderer.shade(cam, lights, model=abi.SHADE_SURROGATE_COMPACT)
    assert renderer.synchronize() == 0
    center, beta, dmap = renderer.read(abi.BUF_CENTER), renderer.read(abi.BUF_BETA), renderer.read(abi.BUF_DOM)
    shaded, sdepth = renderer.read(abi.BUF_SHADED), renderer.read(abi.BUF_SHADED_DEPTH)
    o_shaded, o_sdepth = oracle.shade(cam, center, beta, dmap, lights, mlp=p, mlp_arch=COMPACT)
    hit = center != EMPTY
    assert hit.sum() > 50
    np.testing.assert_array_equal(sdepth, o_sdepth)
    assert np.isfinite(shaded).all()
    got, want = shaded.reshape(-1, 4)[hit, :3], o_shaded.reshape(-1, 4)[hit, :3]
    assert S.relative_l1(got, want) < 2e-3
    np.testing.assert_allclose(got, want, rtol=3e-2, atol=1e-3 * np.abs(want).max())
    renderer.render_groom(g, cam, dom, lights, model=abi.SHADE_SURROGATE_COMPACT)
    assert renderer.synchronize() == 0
    np.testing.assert_array_equal(renderer.read(abi.BUF_SHADED), shaded)
    renderer.bind_surrogate(None)
    s.close()
    deep.close()
    g.close()


@gpu
def test_shipped_compact_surrogate_beats_the_karis_fit(renderer):
    s = S.Surrogate(renderer, S.load_params(COMPACT), COMPACT)
    ev = S.evaluate(renderer, s, n=1 << 15)
    s.close()
    assert ev["surrogate_bsdf"] < 0.75 * ev["karis_bsdf"], ev


@gpu
def test_shade_model_three_on_an_empty_g_buffer_and_without_lights(renderer):
    """No hair pixel (empty list) and no light: the pass writes the empty outputs and nothing else."""
    sc = configs.config2(scale=0.02)
    cam, dom = sc.params()
    lights = sc.light_array()
    renderer.ensure_targets(sc.view.width, sc.view.height, *sc.dom_size)
    s = S.Surrogate(renderer, S.load_params(COMPACT), COMPACT)
    renderer.bind_surrogate(s)
    renderer.clear()
    renderer.shade(cam, lights, model=abi.SHADE_SURROGATE_COMPACT)
    assert renderer.synchronize() == 0
    assert (renderer.read(abi.BUF_SHADED) == 0).all() and (renderer.read(abi.BUF_SHADED_DEPTH) == 0).all()
    g = renderer.upload(sc.mesh)
    renderer.render_groom(g, cam, dom, lights)
    assert renderer.synchronize() == 0
    renderer.shade(cam, lights[:0], model=abi.SHADE_SURROGATE_COMPACT)
    assert renderer.synchronize() == 0
    center = renderer.read(abi.BUF_CENTER)
    shaded = renderer.read(abi.BUF_SHADED).reshape(-1, 4)
    hit = center != EMPTY
    want, _ = oracle.shade(cam, center, renderer.read(abi.BUF_BETA), renderer.read(abi.BUF_DOM), lights[:0],
                           mlp=S.load_params(COMPACT), mlp_arch=COMPACT)
    np.testing.assert_array_equal(shaded[:, 3], hit.astype(np.float32))
    np.testing.assert_allclose(shaded[hit, :3], want.reshape(-1, 4)[hit, :3], rtol=1e-5, atol=1e-7)
    renderer.bind_surrogate(None)
    s.close()
    g.close()
