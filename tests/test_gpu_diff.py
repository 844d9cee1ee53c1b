"""Differentiable render: gradients of an L2 image loss w.r.t. means,
log-scales, quaternions, opacity logits and SH, from the CUDA backward,
against FP64 central differences (h = 1e-4) of the same loss computed end
to end in double by the oracle (oracle/gsr_oracle.c ora_image_fp64), on 64
randomly sampled parameters of Gaussians that reach the image.

Bar (written here): a sampled gradient agrees when
|g_gpu - g_fd| <= 0.05 |g_fd| + 0.01 max|g_fd|; at least 60 of 64 agree (a
few may sit where the FP32 and FP64 tile lists or saturation exits differ).
The float image itself is within 2/255 of the FP64 image."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from polysplat_gb300 import Camera, scenes
from polysplat_gb300 import diff
from polysplat_gb300.diff import render, render_views

pytestmark = pytest.mark.gpu


def _setup(seed=4, n=1500, W=160, H=120):
    raw = scenes.scene_plain_small(n, seed=seed, mean_sigma=1.5)
    rng = np.random.default_rng(seed)
    cams = [scenes.orbit_camera(6.0, 0.3 + 1.1 * k, 0.1, W, H, scenes.focal_for(W)) for k in range(2)]
    tmeans = raw.means + rng.normal(0, 0.05, raw.means.shape).astype(np.float32)
    tshs = raw.shs.copy()
    tshs[:, 0, :] += rng.normal(0, 0.1, tshs[:, 0, :].shape).astype(np.float32)
    targets = [O.image_fp64(tmeans, raw.log_scales, raw.quats, raw.opacity_logits, tshs, c)[1] for c in cams]
    return raw, cams, targets


def _loss_fp64(theta, raw, cams, targets):
    m, ls, q, lg, sh = theta
    return sum(O.image_fp64(m, ls, q, lg, sh, c, target=t)[0] for c, t in zip(cams, targets))


def test_gradients_match_fp64_finite_differences(cuda_device):
    raw, cams, targets = _setup()
    dev = cuda_device
    params = [torch.tensor(a, dtype=torch.float32, device=dev, requires_grad=True)
              for a in (raw.means, raw.log_scales, raw.quats, raw.opacity_logits, raw.shs.reshape(-1, 48))]
    loss = 0.0
    for c, t in zip(cams, targets):
        img = render(*params, Camera.from_spec(c))
        img64 = O.image_fp64(raw.means, raw.log_scales, raw.quats, raw.opacity_logits, raw.shs, c)[1]
        assert np.abs(img.detach().cpu().numpy() - img64).max() <= 2.0 / 255.0
        loss = loss + ((img - torch.tensor(t, dtype=torch.float32, device=dev)) ** 2).sum()
    loss.backward()
    grads = [p.grad.detach().cpu().numpy().astype(np.float64) for p in params]
    theta = [np.asarray(a, np.float64).copy() for a in (raw.means, raw.log_scales, raw.quats, raw.opacity_logits,
                                                        raw.shs.reshape(-1, 48))]
    # sample 64 parameters among Gaussians with a visible gradient
    rng = np.random.default_rng(11)
    active = np.flatnonzero(np.abs(grads[0]).sum(1) > 1e-3 * np.abs(grads[0]).sum(1).max())
    picks = []
    while len(picks) < 64:
        g = int(rng.choice(active))
        t = int(rng.choice(5, p=[0.25, 0.2, 0.2, 0.15, 0.2]))
        k = int(rng.integers(0, theta[t].shape[1])) if theta[t].ndim == 2 else 0
        picks.append((t, g, k))
    h = 1e-4
    ok, rows = 0, []
    fd = []
    for t, g, k in picks:
        idx = (g, k) if theta[t].ndim == 2 else (g,)
        old = theta[t][idx]
        theta[t][idx] = old + h
        lp = _loss_fp64(theta, raw, cams, targets)
        theta[t][idx] = old - h
        lm = _loss_fp64(theta, raw, cams, targets)
        theta[t][idx] = old
        fd.append((lp - lm) / (2 * h))
        rows.append(grads[t][idx])
    fd, gg = np.array(fd), np.array(rows)
    scale = np.abs(fd).max()
    good = np.abs(gg - fd) <= 0.05 * np.abs(fd) + 0.01 * scale
    print("\nagree %d/64; worst rel %s" % (good.sum(), np.sort(np.abs(gg - fd) / (np.abs(fd) + 1e-12))[-5:]))
    assert good.sum() >= 60, list(zip(picks, gg, fd))


def test_gradients_1m_8cam_distribution(cuda_device):
    """The diff_1m_8cam distribution (means ~ N(0, 3^2 I), 8 cameras on a
    radius-10 orbit), subsampled to 4000 Gaussians at 256x144 so the FP64
    oracle evaluates the loss quickly; same bar as above."""
    import math

    full = scenes.scene_plain_small(1_000_000, seed=4, mean_sigma=3.0)
    raw = scenes.subsample(full, 4000, seed=1)
    cams = [scenes.orbit_camera(10.0, 2 * math.pi * k / 8, 0.0, 256, 144, 180.0) for k in range(8)]
    rng = np.random.default_rng(4)
    tmeans = raw.means + rng.normal(0, 0.05, raw.means.shape).astype(np.float32)
    tshs = raw.shs.copy()
    tshs[:, 0, :] += rng.normal(0, 0.1, tshs[:, 0, :].shape).astype(np.float32)
    targets = [O.image_fp64(tmeans, raw.log_scales, raw.quats, raw.opacity_logits, tshs, c)[1] for c in cams]
    dev = cuda_device
    tt = [torch.tensor(t, dtype=torch.float32, device=dev) for t in targets]

    def grads_of(multi):
        params = [torch.tensor(a, dtype=torch.float32, device=dev, requires_grad=True)
                  for a in (raw.means, raw.log_scales, raw.quats, raw.opacity_logits, raw.shs.reshape(-1, 48))]
        cs = [Camera.from_spec(c) for c in cams]
        imgs = render_views(*params, cs) if multi else [render(*params, c) for c in cs]
        sum(((img - t) ** 2).sum() for img, t in zip(imgs, tt)).backward()
        return [p.grad.detach().cpu().numpy().astype(np.float64) for p in params]

    # the per-view passes and the one pass over all views, against the same differences
    grads, grads_multi = grads_of(False), grads_of(True)
    theta = [np.asarray(a, np.float64).copy() for a in (raw.means, raw.log_scales, raw.quats, raw.opacity_logits,
                                                        raw.shs.reshape(-1, 48))]
    rng = np.random.default_rng(12)
    active = np.flatnonzero(np.abs(grads[0]).sum(1) > 1e-3 * np.abs(grads[0]).sum(1).max())
    picks = [(int(rng.choice(5, p=[0.25, 0.2, 0.2, 0.15, 0.2])), int(rng.choice(active))) for _ in range(64)]
    picks = [(t, g, int(rng.integers(0, theta[t].shape[1])) if theta[t].ndim == 2 else 0) for t, g in picks]
    h = 1e-4
    fd, gg = [], []
    for t, g, k in picks:
        idx = (g, k) if theta[t].ndim == 2 else (g,)
        old = theta[t][idx]
        theta[t][idx] = old + h
        lp = _loss_fp64(theta, raw, cams, targets)
        theta[t][idx] = old - h
        lm = _loss_fp64(theta, raw, cams, targets)
        theta[t][idx] = old
        fd.append((lp - lm) / (2 * h))
        gg.append((grads[t][idx], grads_multi[t][idx]))
    fd, gg = np.array(fd), np.array(gg)
    for col, name in ((0, "per view"), (1, "all views in one pass")):
        good = np.abs(gg[:, col] - fd) <= 0.05 * np.abs(fd) + 0.01 * np.abs(fd).max()
        print("\ndiff_1m_8cam distribution, %s: agree %d/64" % (name, good.sum()))
        assert good.sum() >= 60, name


def test_gradients_1m_8cam_full_scene_tile_sampled(cuda_device):
    """diff_1m_8cam at full size: 1 M Gaussians (means ~ N(0, 3^2 I)), 8 cameras
    at 1280x720 on a radius-10 orbit, L2 loss against renders of the scene
    with means perturbed by N(0, 0.05^2) and SH DC by N(0, 0.1^2).  The GPU
    gradients are checked against FP64 central differences (h = 1e-4) of
    the same loss on 64 sampled parameters.  A parameter of Gaussian g only
    changes the tiles of g's rectangle, so each difference is evaluated by
    the FP64 oracle on those tiles (grown by one tile) of every view that
    sees g, which equals the whole image's difference
    (tests/test_oracle.py::test_masked_fp64_loss_gives_the_whole_image_differences).
    Same bar as above; every miss is printed and listed on failure."""
    import math

    raw = scenes.scene_plain_small(1_000_000, seed=4, mean_sigma=3.0)
    specs = [scenes.orbit_camera(10.0, 2 * math.pi * k / 8, 0.0, 1280, 720, 900.0, id=k) for k in range(8)]
    dev = cuda_device
    rng = np.random.default_rng(4)
    t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float32, device=dev)
    tm = raw.means + rng.normal(0, 0.05, raw.means.shape).astype(np.float32)
    tsh = raw.shs.copy()
    tsh[:, 0, :] += rng.normal(0, 0.1, tsh[:, 0, :].shape).astype(np.float32)
    with torch.no_grad():
        targets = [render(t(tm), t(raw.log_scales), t(raw.quats), t(raw.opacity_logits), t(tsh.reshape(-1, 48)),
                          Camera.from_spec(c), key_capacity=1 << 24) for c in specs]

    def grads_of(multi):
        params = [t(a).requires_grad_(True) for a in (raw.means, raw.log_scales, raw.quats, raw.opacity_logits,
                                                      raw.shs.reshape(-1, 48))]
        cs = [Camera.from_spec(c) for c in specs]
        imgs = (render_views(*params, cs, key_capacity=1 << 24) if multi
                else [render(*params, c, key_capacity=1 << 24) for c in cs])
        sum(((img - tg) ** 2).sum() for img, tg in zip(imgs, targets)).backward()
        return [p.grad.detach().cpu().numpy().astype(np.float64) for p in params]

    # the per-view passes and the one pass over all views (the diff_1m_8cam
    # bench's path), against the same differences
    grads, grads_multi = grads_of(False), grads_of(True)
    tnp = [tg.cpu().numpy().astype(np.float64) for tg in targets]
    theta = [np.asarray(a, np.float64).copy() for a in (raw.means, raw.log_scales, raw.quats, raw.opacity_logits,
                                                        raw.shs.reshape(-1, 48))]
    # every Gaussian's tile rectangle in every view (FP64 projection)
    rects = [O.image_fp64_masked(*theta, c, np.zeros(((720 + 15) // 16) * ((1280 + 15) // 16), np.uint8))[2]
             for c in specs]
    sel = np.random.default_rng(13)
    gmag = np.abs(grads[0]).sum(1)
    active = np.flatnonzero(gmag > 1e-3 * gmag.max())
    picks = [(int(sel.choice(5, p=[0.25, 0.2, 0.2, 0.15, 0.2])), int(sel.choice(active))) for _ in range(64)]
    picks = [(k, g, int(sel.integers(0, theta[k].shape[1])) if theta[k].ndim == 2 else 0) for k, g in picks]
    gx, gy = (1280 + 15) // 16, (720 + 15) // 16
    h = 1e-4
    fd, gg = [], []
    for k, g, j in picks:
        idx = (g, j) if theta[k].ndim == 2 else (g,)
        views = []
        for v, r in enumerate(rects):
            x0, y0, x1, y1 = (int(z) for z in r[g])
            if x1 > x0 and y1 > y0:
                m = np.zeros((gy, gx), np.uint8)
                m[max(0, y0 - 1):min(gy, y1 + 1), max(0, x0 - 1):min(gx, x1 + 1)] = 1
                views.append((v, m.reshape(-1)))
        old = theta[k][idx]
        lv = []
        for sgn in (1.0, -1.0):
            theta[k][idx] = old + sgn * h
            lv.append(sum(O.image_fp64_masked(*theta, specs[v], m, target=tnp[v])[0] for v, m in views))
        theta[k][idx] = old
        fd.append((lv[0] - lv[1]) / (2 * h))
        gg.append((grads[k][idx], grads_multi[k][idx]))
    fd, gg = np.array(fd), np.array(gg)
    names = ["mean", "log_scale", "quat", "logit", "sh"]
    for col, path in ((0, "per view"), (1, "all views in one pass")):
        good = np.abs(gg[:, col] - fd) <= 0.05 * np.abs(fd) + 0.01 * np.abs(fd).max()
        misses = [(names[k], g, j, float(a), float(b))
                  for (k, g, j), a, b, ok in zip(picks, gg[:, col], fd, good) if not ok]
        rel = np.abs(gg[:, col] - fd) / (np.abs(fd) + 1e-12)
        print("\ndiff_1m_8cam, 1 M Gaussians, 8 x 1280x720, %s: agree %d/64, median rel err %.2e; misses (param, "
              "gaussian, index, gpu, fp64): %s" % (path, good.sum(), float(np.median(rel)), misses))
        assert good.sum() >= 60, (path, misses)


def _views_case(dev, n, views, W, H, seed=5):
    import math

    raw = scenes.subsample(scenes.scene_plain_small(1_000_000, seed=4, mean_sigma=3.0), n, seed=seed)
    cams = [Camera.from_spec(scenes.orbit_camera(10.0, 2 * math.pi * k / views, 0.05 * k, W, H,
                                                 0.7 * W, id=k)) for k in range(views)]
    params = [torch.tensor(a, dtype=torch.float32, device=dev) for a in
              (raw.means, raw.log_scales, raw.quats, raw.opacity_logits, raw.shs.reshape(-1, 48))]
    return params, cams


def _grads(params, cams, weights, multi, key_capacity=1 << 22, quad=True):
    ps = [p.clone().requires_grad_(True) for p in params]
    imgs = (render_views(*ps, cams, key_capacity=key_capacity, quad_keys=quad) if multi
            else [render(*ps, c, key_capacity=key_capacity) for c in cams])
    sum((img * w).sum() for img, w in zip(imgs, weights)).backward()
    return [img.detach() for img in imgs], [p.grad.detach() for p in ps]


@pytest.mark.parametrize("quad", [True, False])
@pytest.mark.parametrize("n,views,W,H", [(200_000, 8, 640, 360), (20_000, 18, 96, 64)])
def test_render_views_matches_per_view_passes(cuda_device, n, views, W, H, quad):
    """One pass over all views (one preprocess, sort, render and render
    backward over every view's tiles, and a per-Gaussian adjoint summed over
    views, 16 views per launch), with per-tile and with quad keys, against
    one pass per view (per-tile keys) on the same scene and cameras.  With
    per-tile keys the key count is the sum of the views' counts exactly.
    Bar: images within 1e-5 except where equal keys blend in another order
    (at most 1e-4 of the pixels, and within 2/255); every parameter's
    gradient within a relative L2 error of 1e-4 of the per-view sum (float
    atomics add in another order)."""
    dev = cuda_device
    params, cams = _views_case(dev, n, views, W, H)
    gen = torch.Generator(device=dev).manual_seed(3)
    weights = [torch.rand((H, W, 3), device=dev, generator=gen) - 0.5 for _ in cams]
    imgs_m, g_m = _grads(params, cams, weights, True, quad=quad)
    imgs_s, g_s = _grads(params, cams, weights, False)
    # the per-view key counts, from the single-view function
    counts = []
    for c in cams:
        ps = [p.clone().requires_grad_(True) for p in params]
        counts.append(diff._RenderFn.apply(*ps, c, [0.0, 0.0, 0.0], 1 << 22).grad_fn.num_rendered)
    ps = [p.clone().requires_grad_(True) for p in params]
    total = diff._RenderViewsFn.apply(*ps, cams, [0.0, 0.0, 0.0], (1 << 22) * views, quad).grad_fn.num_rendered
    if quad:
        assert 0 < total < sum(counts)  # one key per quad a Gaussian touches
    else:
        assert total == sum(counts) > 0
    for a, b in zip(imgs_m, imgs_s):
        d = (a - b).abs()
        assert float(d.max()) <= 2.0 / 255.0
        assert int((d > 1e-5).sum()) <= 1e-4 * d.numel()
    names = ["means", "log_scales", "quats", "logits", "shs"]
    for name, a, b in zip(names, g_m, g_s):
        err = float((a - b).norm() / b.norm().clamp_min(1e-30))
        assert err <= 1e-4, (name, err)


def test_render_views_grows_the_key_buffers(cuda_device):
    """A key capacity far below the views' keys: the forward reports the
    overflow, grows the buffers and runs again, with the same images."""
    dev = cuda_device
    params, cams = _views_case(dev, 50_000, 4, 320, 180)
    with torch.no_grad():
        small = render_views(*params, cams, key_capacity=1 << 10)
        big = render_views(*params, cams, key_capacity=1 << 22)
    for a, b in zip(small, big):
        d = (a - b).abs()
        assert float(d.max()) <= 2.0 / 255.0
        assert int((d > 1e-5).sum()) <= 1e-4 * d.numel()


def test_render_views_of_mixed_sizes_runs_per_view(cuda_device):
    """Cameras of different sizes go through one pass each."""
    dev = cuda_device
    params, cams = _views_case(dev, 20_000, 2, 160, 96)
    odd = Camera.from_spec(scenes.orbit_camera(10.0, 1.0, 0.0, 128, 80, 90.0, id=9))
    with torch.no_grad():
        imgs = render_views(*params, cams + [odd])
        ref = render(*params, odd)
    assert [tuple(i.shape) for i in imgs] == [(96, 160, 3), (96, 160, 3), (80, 128, 3)]
    d = (imgs[2] - ref).abs()
    assert float(d.max()) <= 2.0 / 255.0 and int((d > 1e-5).sum()) <= 1e-4 * d.numel()


def test_training_view_entries_reject_bad_arguments(cuda_device):
    """The multi-view entries check their arguments before any launch: no
    views, a parameter scratch smaller than gsr_train_views_scratch_bytes, a
    gradient record buffer off a 16-byte boundary (the record atomics are 16
    bytes wide) and unknown flag bits return GSR_INVALID_ARG."""
    import ctypes

    from polysplat_gb300._lib import GSR_INVALID_ARG, lib

    dev = cuda_device
    L = lib()
    assert L.gsr_train_views_scratch_bytes(0) == 0
    assert L.gsr_train_views_scratch_bytes(8) >= 8 * 64
    P, V, W, H = 16, 2, 32, 32
    buf = torch.zeros(1 << 20, dtype=torch.float32, device=dev)
    p = ctypes.c_void_p(buf.data_ptr())
    pos = (ctypes.c_float * (3 * V))()
    rot = (ctypes.c_float * (9 * V))()
    intr = (ctypes.c_float * (4 * V))(*([100.0, 100.0, 100.0, 0.01] * V))
    bg = (ctypes.c_float * 3)()
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    ws = L.gsr_workspace_size(1 << 10)

    def fwd(n_views, scratch_bytes):
        return L.gsr_train_forward_views(P, p, p, p, p, p, n_views, W, H, pos, rot, intr, bg, p, p, p,
                                         scratch_bytes, p, p, ws, p, p, p, p, 1 << 10, p, p, p, p, p, p, p, 0, stream)

    assert fwd(0, 1 << 20) == GSR_INVALID_ARG
    assert fwd(V, L.gsr_train_views_scratch_bytes(V) - 1) == GSR_INVALID_ARG

    def bwd(grad_feat):
        return L.gsr_train_backward_views(P, p, p, p, p, p, V, W, H, pos, rot, intr, bg, p, 1 << 10, p, p, p, p,
                                          p, p, p, p, grad_feat, p, p, p, p, p, 0, 0, stream)

    assert bwd(ctypes.c_void_p(buf.data_ptr() + 4)) == GSR_INVALID_ARG
    assert bwd(None) == GSR_INVALID_ARG
    # unknown flag bits
    assert L.gsr_train_forward_views(P, p, p, p, p, p, V, W, H, pos, rot, intr, bg, p, p, p, 1 << 20, p, p, ws, p, p,
                                     p, p, 1 << 10, p, p, p, p, p, p, p, 1, stream) == GSR_INVALID_ARG
    torch.cuda.synchronize()


def test_render_views_stacked_equals_the_list(cuda_device):
    """render_views(stacked=True) returns the views as one [views, H, W, 3]
    tensor, the same images as the list form, with the same gradients."""
    dev = cuda_device
    params, cams = _views_case(dev, 50_000, 4, 320, 180)
    gen = torch.Generator(device=dev).manual_seed(5)
    w = torch.rand((4, 180, 320, 3), device=dev, generator=gen)
    ps_a = [p.clone().requires_grad_(True) for p in params]
    ps_b = [p.clone().requires_grad_(True) for p in params]
    out = render_views(*ps_a, cams, stacked=True)
    lst = render_views(*ps_b, cams)
    assert tuple(out.shape) == (4, 180, 320, 3)
    for a, b in zip(out.detach().unbind(0), lst):
        d = (a - b.detach()).abs()
        assert float(d.max()) <= 2.0 / 255.0 and int((d > 1e-5).sum()) <= 1e-4 * d.numel()
    (out * w).sum().backward()
    sum((img * wv).sum() for img, wv in zip(lst, w.unbind(0))).backward()
    for a, b in zip(ps_a, ps_b):
        assert float((a.grad - b.grad).norm() / b.grad.norm().clamp_min(1e-30)) <= 1e-4
    odd = Camera.from_spec(scenes.orbit_camera(10.0, 1.0, 0.0, 128, 80, 90.0, id=9))
    with pytest.raises(ValueError):
        render_views(*params, cams + [odd], stacked=True)
