"""The guiding network on the tensor cores against its CPU oracle (forward and
gradient), unbiasedness of the guided estimator, and its gain over plain sampling at
equal device time on the indirect-lit room."""
import numpy as np
import pytest

from oracle import guide_oracle as go
from parity import zscores
from spica_gb300 import GpuBVHAccel, GpuGuide, scenes
from spica_gb300.gpu import GUIDE_COLLECT, GUIDE_GUIDED, GUIDE_MEGAKERNEL

pytestmark = pytest.mark.gpu


def _room(n_boxes=200, **kw):
    return scenes.guiding_room(n_boxes=n_boxes, **kw)


def _random_params(seed):
    rng = np.random.default_rng(seed)
    p = go.init_params(seed)
    p[go.N_PARAMS - 40:] = (rng.normal(size=40) * 0.5).astype(np.float32)
    for off, n in ((576, 64), (4736, 64), (8896, 64)):
        p[off:off + n] = (rng.normal(size=n) * 0.1).astype(np.float32)
    return p


def _blocks():
    """(name, slice) of each weight matrix and bias vector in the parameter layout."""
    out, off = [], 0
    for li, (o, i) in enumerate(go.SHAPES):
        out.append((f"W{li + 1}", slice(off, off + o * i)))
        off += o * i
        out.append((f"b{li + 1}", slice(off, off + o)))
        off += o
    return out


def _gather_indices(seed, step, n, avail):
    """The training batch of Adam step `step`: ring entries chosen by Philox4x32-10 keyed
    by (seed, 0), counter (sample, step, 0x47415448, 0), index = (word 0 * avail) >> 32."""
    from oracle import philox as P
    s = np.arange(n, dtype=np.uint64)
    ctr = np.stack([s, np.full(n, step), np.full(n, 0x47415448), np.zeros(n)], 1).astype(np.uint32)
    key = np.tile(np.array([seed, 0], np.uint32), (n, 1))
    r = P.philox4x32_10(ctr, key)[:, 0].astype(np.uint64)
    return ((r * np.uint64(avail)) >> np.uint64(32)).astype(np.int64)


def test_adam_steps_match_oracle(gpulib):
    """Three training steps (batch gather, gradient, Adam, weight packing) against a numpy
    restatement of the same steps (Kingma and Ba, ICLR 2015: beta1 0.9, beta2 0.999,
    eps 1e-8, bias-corrected moments) applied to the device's own gradient of the same
    gathered batch, and the batch gather against the oracle's Philox indices."""
    import torch
    sc = _room(30)
    W, H = 48, 32
    acc = GpuBVHAccel(sc).construct()
    lr, seed = 2e-3, 13
    g = GpuGuide(acc, seed=seed, lr=lr, batch=4096)
    f = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    for k in range(64):   # collection passes until the ring holds a few thousand entries
        g.render(sc.camera, {"width": W, "height": H, "sampleCount": 16, "maxDepth": sc.max_depth}, f,
                 GUIDE_GUIDED | GUIDE_COLLECT, seed=5, sample_offset=16 * k)
        if g.samples() >= 4096:
            break
    torch.cuda.synchronize()
    ring = g.ring(1 << 20)
    avail = ring.shape[0]
    assert avail > 1000
    n = min(4096, avail)
    m = np.zeros(go.N_PARAMS)
    v = np.zeros(go.N_PARAMS)
    p = g.params().astype(np.float64)
    for step in range(3):
        batch = ring[_gather_indices(seed, step, n, avail)]
        grad = torch.zeros(go.N_PARAMS, dtype=torch.float32, device="cuda")
        g.grad(torch.from_numpy(np.ascontiguousarray(batch)).cuda(), grad)
        gd = grad.cpu().numpy().astype(np.float64)
        want = go.grad(p.astype(np.float32), batch[:, :9], batch[:, 9:12], batch[:, 12], emulate_bf16=True)
        assert np.linalg.norm(gd - want) < 1e-2 * np.linalg.norm(want)
        m = 0.9 * m + 0.1 * gd
        v = 0.999 * v + 0.001 * gd * gd
        vhat = v / (1 - 0.999 ** (step + 1))
        p_next = p - lr * (m / (1 - 0.9 ** (step + 1))) / (np.sqrt(vhat) + 1e-8)
        g.train(1)
        got = g.params().astype(np.float64)
        # The training step sums the same per-CTA partial gradients in the same order as
        # the gradient entry point, so where sqrt(v_hat) is well above eps the update is
        # the same up to float32 rounding: within 1 % of a step (lr).  Parameters whose
        # gradients sit at the level of float32 rounding (dead units, cancelling terms)
        # still move by at most one step.
        firm = np.sqrt(vhat) > 1e-5
        assert firm.mean() > 0.5
        err = np.abs(got - p_next)
        assert err[firm].max() <= 1e-2 * lr + 1e-6, (step, err[firm].max(), int(np.argmax(np.where(firm, err, 0))))
        assert np.abs(got - p).max() <= 1.1 * lr, (step, np.abs(got - p).max())
        assert np.abs(got - p).max() > 0.5 * lr
        p = got


def test_gradient_matches_finite_differences(gpulib):
    """The device gradient against central differences of the device's own loss along
    directions of the parameters (steps of 3e-3 of the parameter norm, wide against the
    weights' BF16 rounding; the oracle's own central differences agree within 2 %)."""
    import torch
    acc = GpuBVHAccel(_room(10)).construct()
    g = GpuGuide(acc, seed=3)
    p = _random_params(11).astype(np.float64)
    rng = np.random.default_rng(4)
    n = 2048
    S = np.zeros((n, 16), np.float32)
    S[:, :9] = rng.random((n, 9))
    S[:, 3:9] = S[:, 3:9] * 2 - 1
    w = rng.normal(size=(n, 3))
    S[:, 9:12] = w / np.linalg.norm(w, axis=1, keepdims=True)
    S[:, 12] = rng.random(n) + 0.05
    Sd = torch.from_numpy(S).cuda()
    grad = torch.zeros(go.N_PARAMS, dtype=torch.float32, device="cuda")

    def loss_at(q):
        g.set_params(q.astype(np.float32))
        return g.grad(Sd, grad)

    g.set_params(p.astype(np.float32))
    g.grad(Sd, grad)
    gd = grad.cpu().numpy().astype(np.float64)
    for k in range(4):
        # half along the gradient, half random, so that the derivative is well above the
        # loss's BF16 rounding noise
        r = rng.normal(size=go.N_PARAMS)
        d = gd / np.linalg.norm(gd) + r / np.linalg.norm(r)
        d *= 3e-3 * np.linalg.norm(p) / np.linalg.norm(d)
        fd = (loss_at(p + d) - loss_at(p - d)) / 2.0
        assert abs(fd - gd @ d) <= 0.05 * abs(gd @ d), (k, fd, gd @ d)


def test_mlp_forward_matches_oracle(gpulib):
    import torch
    acc = GpuBVHAccel(_room(10)).construct()
    g = GpuGuide(acc, seed=3)
    p = _random_params(5)
    g.set_params(p)
    assert np.array_equal(g.params(), p)
    rng = np.random.default_rng(2)
    n = 1000   # not a multiple of the 128-sample tile
    x = rng.random((n, 9)).astype(np.float32)
    x[:, 3:] = x[:, 3:] * 2 - 1
    out = torch.zeros((n, 40), dtype=torch.float32, device="cuda")
    g.mlp(torch.from_numpy(x).cuda(), out)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    want, _ = go.forward(p, x, emulate_bf16=True)
    scale = np.abs(want).max()
    assert np.abs(got - want).max() <= 2e-2 * scale, np.abs(got - want).max() / scale


def test_gradient_matches_oracle(gpulib):
    import torch
    acc = GpuBVHAccel(_room(10)).construct()
    g = GpuGuide(acc, seed=3)
    p = _random_params(7)
    g.set_params(p)
    rng = np.random.default_rng(3)
    n = 700
    S = np.zeros((n, 16), np.float32)
    S[:, :9] = rng.random((n, 9))
    S[:, 3:9] = S[:, 3:9] * 2 - 1
    w = rng.normal(size=(n, 3))
    S[:, 9:12] = w / np.linalg.norm(w, axis=1, keepdims=True)
    S[:, 12] = rng.random(n) + 0.05
    grad = torch.zeros(go.N_PARAMS, dtype=torch.float32, device="cuda")
    loss = g.grad(torch.from_numpy(S).cuda(), grad)
    gg = grad.cpu().numpy().astype(np.float64)
    want = go.grad(p, S[:, :9], S[:, 9:12], S[:, 12], emulate_bf16=True)
    cos = gg @ want / (np.linalg.norm(gg) * np.linalg.norm(want))
    assert cos > 0.995, cos
    assert abs(np.linalg.norm(gg) / np.linalg.norm(want) - 1) < 0.03
    # every parameter block on its own: W1, b1, ..., W4, b4 within 1e-2 relative
    for name, sl in _blocks():
        err = np.linalg.norm(gg[sl] - want[sl]) / max(np.linalg.norm(want[sl]), 1e-30)
        assert err < 1e-2, (name, err)
    ref_loss = go.loss(p, S[:, :9], S[:, 9:12], S[:, 12], emulate_bf16=True)
    assert abs(loss - ref_loss) <= 0.02 * abs(ref_loss) + 1e-3, (loss, ref_loss)


def test_training_reduces_loss_and_guided_render_is_unbiased(gpulib):
    import torch
    sc = _room(60)
    W, H = 64, 36
    acc = GpuBVHAccel(sc).construct()
    g = GpuGuide(acc, seed=1, batch=8192)
    p = {"width": W, "height": H, "maxDepth": sc.max_depth}
    scratch = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    losses = []
    for k in range(12):
        g.render(sc.camera, dict(p, sampleCount=4), scratch, GUIDE_GUIDED | GUIDE_COLLECT, seed=50, sample_offset=4 * k)
        losses.append(g.train(10))
    assert g.samples() > 0
    assert np.mean(losses[-3:]) < np.mean(losses[:3]), losses
    # guided and plain estimates agree per pixel (batch means, 16 x 128 spp each)
    means = {}
    for flags in (0, GUIDE_GUIDED):
        ms = []
        for b in range(16):
            f = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
            g.render(sc.camera, dict(p, sampleCount=128), f, flags, seed=9 + flags, sample_offset=128 * b)
            fh = f.cpu().numpy()
            ms.append(fh[..., :3] / fh[..., 3:])
        m = np.stack(ms)
        means[flags] = (m.mean(0), m.var(0, ddof=1) / 16)
    z = zscores(means[0][0], means[0][1], means[GUIDE_GUIDED][0], means[GUIDE_GUIDED][1])
    assert (np.abs(z) > 3).mean() < 0.02, ((np.abs(z) > 3).mean(), np.abs(z).max())


def test_plain_megakernel_matches_wavefront(gpulib):
    """The plain megakernel is the same estimator as spgpu_render: same film from the
    same streams."""
    import torch
    from spica_gb300 import GpuPathIntegrator
    sc = _room(20)
    W, H = 48, 32
    acc = GpuBVHAccel(sc).construct()
    g = GpuGuide(acc, seed=1)
    f = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    g.render(sc.camera, {"width": W, "height": H, "sampleCount": 16, "maxDepth": sc.max_depth}, f, GUIDE_MEGAKERNEL,
             seed=4)
    ref = GpuPathIntegrator(seed=4).render(sc.camera, acc, {"width": W, "height": H, "sampleCount": 16,
                                                            "maxDepth": sc.max_depth})
    got = f.cpu().numpy()
    assert np.array_equal(got[..., 3], ref[..., 3])
    np.testing.assert_allclose(got[..., :3], ref[..., :3], rtol=2e-3, atol=2e-3)


def test_guided_wavefront_matches_guided_megakernel(gpulib):
    """Guided rendering in the wavefront (network run per bounce over the queue of diffuse
    hits) and in the megakernel (network run per CTA at each bounce) are the same
    estimator: the same inputs reach the network, a row's outputs do not depend on the
    other rows of its tile, and both shade with the same code and sampler streams, so
    the films agree up to the order of the film's atomic additions."""
    import torch
    sc = _room(40)
    W, H = 64, 40
    acc = GpuBVHAccel(sc).construct()
    g = GpuGuide(acc, seed=5)
    p = {"width": W, "height": H, "maxDepth": sc.max_depth}
    scratch = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    for k in range(6):
        g.render(sc.camera, dict(p, sampleCount=4), scratch, GUIDE_GUIDED | GUIDE_COLLECT, seed=70, sample_offset=4 * k)
        g.train(16)
    films = []
    for flags in (GUIDE_GUIDED, GUIDE_GUIDED | GUIDE_MEGAKERNEL):
        f = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
        st = g.render(sc.camera, dict(p, sampleCount=16), f, flags, seed=8, sample_offset=0)
        assert st.paths == W * H * 16
        films.append(f.cpu().numpy())
    a, b = films
    assert np.array_equal(a[..., 3], b[..., 3])
    assert a[..., :3].sum() > 0
    np.testing.assert_allclose(a[..., :3], b[..., :3], rtol=2e-3, atol=2e-3)


@pytest.mark.parametrize("guided_bounces", [0, 2])
def test_streaming_guided_matches_pass_by_pass(gpulib, guided_bounces):
    """Guided passes on the streaming wavefront (the default: one guided shading launch
    per iteration over a Lambert queue that mixes depths) and on the pass-by-pass
    wavefront (one guided launch per bounce) draw the same numbers for every (pixel,
    sample, depth) and give the network the same inputs, so with the same weights the
    films agree up to the order of the film's atomic additions; likewise plain passes.
    With guided_bounces = 2 the deeper rows of the streaming queue take plain BSDF
    sampling inside the guided kernel, as the pass-by-pass wavefront's later bounces do."""
    import torch
    from spica_gb300 import Context
    sc = _room(40)
    W, H = 96, 56
    p = {"width": W, "height": H, "maxDepth": sc.max_depth}
    acc = GpuBVHAccel(sc).construct()
    g = GpuGuide(acc, seed=5, guided_bounces=guided_bounces)
    scratch = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    for k in range(6):
        g.render(sc.camera, dict(p, sampleCount=4), scratch, GUIDE_GUIDED | GUIDE_COLLECT, seed=70, sample_offset=4 * k)
        g.train(16)
    acc1 = GpuBVHAccel(sc, ctx=Context(0, wavefront=1)).construct()
    g1 = GpuGuide(acc1, seed=5, guided_bounces=guided_bounces)
    g1.set_params(g.params())
    for flags in (GUIDE_GUIDED, 0):
        films = []
        for guide in (g, g1):
            f = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
            st = guide.render(sc.camera, dict(p, sampleCount=24), f, flags, seed=8, sample_offset=3)
            assert st.paths == W * H * 24 and st.kernel_launches > 0
            films.append(f.cpu().numpy())
        a, b = films
        assert np.array_equal(a[..., 3], b[..., 3])
        assert a[..., :3].sum() > 0
        np.testing.assert_allclose(a[..., :3], b[..., :3], rtol=2e-3, atol=2e-3)


def test_wavefront_collection_matches_megakernel(gpulib):
    """Training records collected in the wavefront (per-path records closed when their
    continuation ray finds its hit, turned into ring entries at the end of the pass)
    are the megakernel's: the same entries, with the same weights c up to the order in
    which a path's radiance was summed."""
    import torch
    sc = _room(30)
    W, H = 128, 96
    acc = GpuBVHAccel(sc).construct()
    p = {"width": W, "height": H, "maxDepth": sc.max_depth}
    rings = []
    for flags in (GUIDE_GUIDED | GUIDE_COLLECT, GUIDE_GUIDED | GUIDE_COLLECT | GUIDE_MEGAKERNEL):
        g = GpuGuide(acc, seed=6)   # the same initial weights
        f = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
        g.render(sc.camera, dict(p, sampleCount=16), f, flags, seed=21, sample_offset=0)
        rings.append(g.ring(1 << 20))
    a, b = rings
    assert len(a) > 500, len(a)
    assert abs(len(a) - len(b)) <= 0.002 * len(b) + 2, (len(a), len(b))
    ka = {r[:12].tobytes(): r for r in a}
    kb = {r[:12].tobytes(): r for r in b}
    common = ka.keys() & kb.keys()
    assert len(common) >= 0.998 * min(len(ka), len(kb)), (len(common), len(ka), len(kb))
    ca = np.array([ka[k][12] for k in common])
    cb = np.array([kb[k][12] for k in common])
    qa = np.array([ka[k][13] for k in common])
    qb = np.array([kb[k][13] for k in common])
    np.testing.assert_array_equal(qa, qb)
    assert np.mean(np.abs(ca - cb) <= 1e-4 * np.abs(cb) + 1e-12) > 0.999


def test_trained_guide_lowers_error_per_sample(gpulib):
    """What the trained network gains over plain BSDF sampling on the indirect-lit room:
    after online training (collection passes + Adam steps on the device), a guided
    render has a clearly lower relMSE than a plain render with the same samples per
    pixel (measured 1.7-2.2x; asserted >= 1.4x).  The equal-time comparison, which
    also charges inference and training time, is reported by the benchmark."""
    import torch
    from spica_gb300 import guiding
    sc = _room()
    W, H = 320, 180
    acc = GpuBVHAccel(sc).construct()
    g = GpuGuide(acc, seed=2)
    ref = guiding.render_reference(torch, acc, g, sc, W, H, spp=4096)
    p = {"width": W, "height": H, "maxDepth": sc.max_depth}
    scratch = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    for k in range(48):
        g.render(sc.camera, dict(p, sampleCount=2), scratch, GUIDE_GUIDED | GUIDE_COLLECT, seed=1011,
                 sample_offset=2 * k)
        g.train(32)
    imgs = {}
    for flags in (0, GUIDE_GUIDED):
        f = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
        for k in range(0, 256, 16):
            g.render(sc.camera, dict(p, sampleCount=16), f, flags, seed=11, sample_offset=k)
        torch.cuda.synchronize()
        f = f.cpu().numpy()
        imgs[flags] = f[..., :3] / f[..., 3:4]
    e_plain, e_guided = guiding.relmse(imgs[0], ref), guiding.relmse(imgs[GUIDE_GUIDED], ref)
    print({"relmse_plain": e_plain, "relmse_guided": e_guided, "gain": e_plain / e_guided})
    assert e_guided * 1.4 <= e_plain, (e_plain, e_guided)
