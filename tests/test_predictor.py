"""The bin-capacity model.

CPU: the float64 oracle's gradient (oracle/mlp_oracle.py) against central
finite differences, so it can check the GPU kernels.
GPU: the training kernels' forward and loss + gradient (BF16 parameters,
FP32 accumulation) against the oracle; predicted-capacity binning gives bin
lists and images identical to exact binning, both when the capacities hold
and when a bin overflows and the frame is re-binned on the device.
"""
import ctypes as C

import numpy as np
import pytest

import scenes
from oracle import mlp_oracle


def random_problem(n=96, seed=0, scale=0.3):
    rng = np.random.default_rng(seed)
    w = mlp_oracle.f32_to_bf16(rng.normal(0, scale, mlp_oracle.NUM_PARAMS))
    X = rng.normal(0.5, 1.0, (n, mlp_oracle.F)).astype(np.float32)
    y = rng.integers(0, 400, n).astype(np.float32)
    return w, X, y


def test_oracle_gradient_matches_finite_differences():
    w16, X, y = random_problem(16, seed=1)
    w = mlp_oracle.bf16_to_f64(w16)
    _, g = mlp_oracle.loss_grad(w16, X, y)

    def loss_at(wv):
        W1, b1, W2, b2, W3, b3 = mlp_oracle.unpack(wv)
        h1 = np.maximum(X @ W1 + b1, 0)
        h2 = np.maximum(h1 @ W2 + b2, 0)
        lam = mlp_oracle.softplus(h2 @ W3 + b3)
        return float(((np.log1p(lam) - np.log1p(y)) ** 2).sum())

    rng = np.random.default_rng(2)
    for i in rng.choice(mlp_oracle.NUM_PARAMS, 60, replace=False).tolist() + [mlp_oracle.OFF_B3]:
        e = np.zeros_like(w)
        e[i] = 1e-6
        fd = (loss_at(w + e) - loss_at(w - e)) / 2e-6
        assert abs(fd - g[i]) <= 1e-4 * max(1.0, abs(fd)), (i, fd, g[i])


@pytest.mark.gpu
def test_gpu_loss_gradient_and_forward_match_oracle(gbr_lib, cuda_device):
    import torch
    L = gbr_lib.lib()
    assert L.gbr_mlp_num_params() == mlp_oracle.NUM_PARAMS
    w16, X, y = random_problem(200, seed=3)
    dw = torch.from_numpy(w16.view(np.int16)).to(cuda_device)
    dX = torch.from_numpy(X).to(cuda_device)
    dy = torch.from_numpy(y).to(cuda_device)
    grad = torch.zeros(mlp_oracle.NUM_PARAMS, device=cuda_device)
    loss = torch.zeros(1, device=cuda_device)
    out = torch.empty(len(y), device=cuda_device)
    p = lambda t: C.c_void_p(t.data_ptr())
    gbr_lib.check(L.gbr_mlp_loss_grad(p(dw), p(dX), p(dy), len(y), p(grad), p(loss), None))
    gbr_lib.check(L.gbr_mlp_predict(p(dw), p(dX), len(y), p(out), None))
    torch.cuda.synchronize()
    ref_loss, ref_grad = mlp_oracle.loss_grad(w16, X, y)
    g = grad.cpu().numpy().astype(np.float64)
    assert abs(float(loss.item()) - ref_loss) <= 1e-4 * abs(ref_loss)
    scale = np.abs(ref_grad).max()
    assert np.abs(g - ref_grad).max() <= 2e-4 * scale, np.abs(g - ref_grad).max() / scale
    lam = out.cpu().numpy().astype(np.float64)
    ref_lam = mlp_oracle.predict(w16, X)
    assert np.allclose(lam, ref_lam, rtol=1e-4, atol=1e-5)


def _frame(gbr, scene, predictor=None):
    r = gbr.Renderer(scene.width, scene.height)
    r.load_scene(scene)
    if predictor is not None:
        w, a, b, g = predictor
        gbr.check(r._lib.gbr_set_predictor(r.h, w.ctypes.data_as(C.c_void_p), len(w), C.c_float(a), C.c_float(b),
                                           C.c_float(g)))
        r.set_binning(gbr.BINNING_PREDICTED)
        # a first frame sizes the bin storage for the predicted capacities
        r.render_scene(scene)
        r.stats()
    r.render_scene(scene)
    colour, depth = r.readback()
    ids = r.readback_ids()
    offsets, bins = r.get_bins()
    st = r.stats()
    r.close()
    return colour, depth, ids, offsets, bins, st


def _constant_model(count: float) -> np.ndarray:
    """A model that predicts `count` for every bin (all weights zero, output
    bias softplus^-1(count))."""
    w = np.zeros(mlp_oracle.NUM_PARAMS, np.float32)
    w[mlp_oracle.OFF_B3] = count + np.log(-np.expm1(-count))
    return mlp_oracle.f32_to_bf16(w)


@pytest.mark.gpu
@pytest.mark.parametrize("count,expect_overflow", [(4000.0, False), (2.0, True), (5.0e6, True)])
def test_predicted_binning_is_identical_to_exact(gbr_lib, cuda_device, count, expect_overflow):
    """Capacities that hold, capacities that overflow a bin, and predictions
    whose capacities add up to far more than the bin storage (5e6 per bin,
    6e9 before clamping to the triangle count): the frame is re-binned
    exactly on the device and matches exact binning."""
    s = scenes.soup_scene(60000, 640, 480, seed=41)
    exact = _frame(gbr_lib, s)
    pred = _frame(gbr_lib, s, (_constant_model(count), 0.0, 0.0, 0.0))
    assert pred[5]["predicted_overflow"] == (1 if expect_overflow else 0)
    for a, b in zip(exact[:5], pred[:5]):
        assert np.array_equal(a, b)
    assert pred[5]["num_pairs"] == exact[5]["num_pairs"] and pred[5]["num_visible"] == exact[5]["num_visible"]


def bf16_round(a):
    """float32 -> nearest-even BF16 -> float32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


@pytest.mark.gpu
def test_tensor_core_capacities_match_the_model(gbr_lib, cuda_device):
    """The capacity kernel runs the 12-64-64-1 model on the tensor cores
    (tcgen05.mma, BF16 operands -- features and hidden layer rounded to
    BF16 -- FP32 accumulation in tensor memory).  Its capacities match the
    same model evaluated on the CPU with those roundings to within the
    accumulation order (1% + 2 entries), on every bin."""
    import predictor
    s = scenes.soup_scene(150_000, 960, 540, 16, seed=9)
    nb = s.num_bins_x * s.num_bins_y
    feats = np.empty((nb, mlp_oracle.F), np.float32)
    counts = np.empty(nb, np.uint32)
    with gbr_lib.Renderer(s.width, s.height) as r:
        r.load_scene(s)
        cam = gbr_lib.make_camera(s.camera)
        gbr_lib.check(r._lib.gbr_collect_bin_features(r.h, C.byref(cam), s.cull, s.sample, s.vis,
                                                      feats.ctypes.data_as(C.c_void_p),
                                                      counts.ctypes.data_as(C.c_void_p), None))
        predictor.install(r)
        r.render_scene(s)
        r.stats()
        caps = r.predicted_capacities().astype(np.float64)
    w16, a, b, g, _ = predictor.load()
    W1, b1, W2, b2, W3, b3 = (np.asarray(x, np.float32) for x in mlp_oracle.unpack(mlp_oracle.bf16_to_f64(w16)))
    h1 = np.maximum(bf16_round(feats) @ W1 + b1, 0).astype(np.float32)
    h2 = np.maximum(bf16_round(h1) @ W2 + b2, 0).astype(np.float32)
    lam = mlp_oracle.softplus((h2 @ W3 + b3).astype(np.float64))
    want = np.clip(np.ceil(lam * (1 + a) + b * np.sqrt(lam + 1) + g), 0, s.num_triangles)
    assert caps.shape == want.shape
    assert np.all(np.abs(caps - want) <= 0.01 * want + 2), float(np.max(np.abs(caps - want) - 0.01 * want))


def _predicted_frames(gbr, s, mode):
    """Two frames of `s` (the first sizes the storage) with exact binning,
    the committed model ("mlp") or the plain sampled-count rule ("sampled");
    returns the outputs of the second and its statistics."""
    import predictor
    with gbr.Renderer(s.width, s.height) as r:
        r.load_scene(s)
        if mode != "exact":
            predictor.install(r, sampled=(mode == "sampled"))
        for _ in range(2):
            r.render_scene(s)
            st = r.stats()
        colour, depth = r.readback()
        ids = r.readback_ids()
        offsets, bins = r.get_bins()
    return (colour, depth, ids, offsets, bins), st


@pytest.mark.gpu
def test_full_size_predicted_binning_with_the_committed_model(gbr_lib, cuda_device):
    """The 1M-triangle 1920x1080 soup of the benchmark (seed 0) and a
    held-out one (seed 77), binned with the committed capacity model: bin
    lists, winning ids, depth and colour identical to exact binning, without
    a capacity overflow (the predicted pass, not its exact fallback, binned
    them)."""
    for seed in (0, 77):
        s = scenes.soup_scene(1_000_000, 1920, 1080, 16, seed=seed)
        e, est = _predicted_frames(gbr_lib, s, "exact")
        p, pst = _predicted_frames(gbr_lib, s, "mlp")
        assert pst["predicted_overflow"] == 0
        assert pst["num_pairs"] == est["num_pairs"]
        for a, b in zip(e, p):
            assert np.array_equal(a, b)


@pytest.mark.gpu
def test_the_network_allocates_less_than_the_sampled_count_rule(gbr_lib, cuda_device):
    """What the trained network gains over the method without it, on
    held-out 1M-triangle 1080p soups (seeds the training never drew): both
    estimators' capacity rules were fitted the same way (least total
    capacity with at most 1e-6 of ~1M held-out bins overflowing); both give
    bin lists and images identical to exact binning and no overflow here,
    and the network's capacities over-allocate the list far less than
    (sampled pairs x 8) does."""
    over = {"mlp": [], "sampled": []}
    for seed in (1001, 1002, 1003):
        s = scenes.soup_scene(1_000_000, 1920, 1080, 16, seed=seed)
        e, est = _predicted_frames(gbr_lib, s, "exact")
        for mode in ("mlp", "sampled"):
            p, pst = _predicted_frames(gbr_lib, s, mode)
            assert pst["predicted_overflow"] == 0, mode
            for a, b in zip(e, p):
                assert np.array_equal(a, b), mode
            over[mode].append(pst["predicted_capacity"] / est["num_pairs"] - 1.0)
    mlp, sampled = float(np.mean(over["mlp"])), float(np.mean(over["sampled"]))
    print(f"over-allocation: network {mlp:.3f}, sampled-count rule {sampled:.3f}")
    assert mlp < 0.5 * sampled, (mlp, sampled)
