"""Bin-capacity model: training data, training and capacity rule, all on the
GPU through the library's own kernels (gbr_collect_bin_features,
gbr_mlp_loss_grad, gbr_mlp_adam, gbr_mlp_predict).

    python predictor.py train [--pairs 2000000] [--out predictor_weights.npz]

Training pairs are (12 features of a bin from the 1/8-sample coarse
pre-pass, exact triangle count of the bin from exact two-pass binning) over
seeded scenes drawn like the 1M-triangle soup (varied count, blob, area
range) and like the displaced icosphere (varied subdivision, distance,
resolution), all with 16x16 bins.  The capacity rule
ceil(l*(1+alpha) + beta*sqrt(l+1) + gamma) is fitted on about a million
held-out bins so that none of them overflows, with the least
over-allocation; `evaluate` then measures frame overflow rate,
over-allocation, bit-identity and time against exact binning on held-out
1M-triangle 1080p soups.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import gbr  # noqa: E402
import scenes  # noqa: E402

WEIGHTS = os.path.join(HERE, "predictor_weights.npz")
NUM_FEATURES = 12
SAMPLED_SCALE = 256.0   # feature 0 = (8 x sampled pairs of the bin) / 256 (gbr_predict.cu: bin_features)


def num_params() -> int:
    return int(gbr.lib().gbr_mlp_num_params())


def training_scene(i: int, rng: np.random.Generator):
    """Scene i of the training distribution (16x16 bins)."""
    if i % 5 == 4:
        subdiv = int(rng.integers(5, 8))
        w, h = ((1920, 1080), (3840, 2160), (1280, 720))[int(rng.integers(0, 3))]
        s = scenes.icosphere_scene(w, h, 16, subdiv, tex_size=64, distance=float(rng.uniform(2.5, 12.0)))
        s.meshes[0].textures = [None] * 4
        s.cull = int(rng.integers(0, 3))
        return s
    n = int(math.exp(rng.uniform(math.log(1e5), math.log(2e6))))
    v = scenes.soup_vertices(n, 1920, 1080, seed=int(rng.integers(1 << 30)), blob_frac=float(rng.uniform(0, 0.4)),
                             blob_sigma=float(rng.uniform(40, 300)), area_max=float(math.exp(rng.uniform(math.log(256),
                                                                                                          math.log(8192)))))
    return scenes.Scene(f"soup{n}", 1920, 1080, 16, 16, scenes.identity_camera(), [scenes.Mesh(vertices=v)],
                        cull=scenes.CULL_NONE)


def collect(scene_list, log=print):
    """(features [N, 12] float32, exact counts [N] float32) over the scenes."""
    feats, counts = [], []
    for k, s in enumerate(scene_list):
        with gbr.Renderer(s.width, s.height) as r:
            r.load_scene(s)
            nb = s.num_bins_x * s.num_bins_y
            f = np.empty((nb, NUM_FEATURES), np.float32)
            c = np.empty(nb, np.uint32)
            cam = gbr.make_camera(s.camera)
            gbr.check(r._lib.gbr_collect_bin_features(r.h, C.byref(cam), s.cull, s.sample, s.vis,
                                                      f.ctypes.data_as(C.c_void_p), c.ctypes.data_as(C.c_void_p),
                                                      None))
        feats.append(f)
        counts.append(c.astype(np.float32))
        if log and (k + 1) % 25 == 0:
            log(f"collected {k + 1} frames, {sum(len(x) for x in counts)} pairs")
    return np.concatenate(feats), np.concatenate(counts)


def _init_master(seed: int) -> np.ndarray:
    """He-initialised FP32 master parameters in the kernel's layout."""
    rng = np.random.default_rng(seed)
    F, H = NUM_FEATURES, 64
    parts = [rng.normal(0, math.sqrt(2 / F), F * H), np.zeros(H), rng.normal(0, math.sqrt(2 / H), H * H), np.zeros(H),
             rng.normal(0, math.sqrt(1 / H), H), np.array([1.0])]
    w = np.concatenate(parts).astype(np.float32)
    assert len(w) == num_params()
    return w


def to_bf16(w: np.ndarray) -> np.ndarray:
    u = np.asarray(w, np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def train(X: np.ndarray, y: np.ndarray, epochs: int = 10, batch: int = 8192, lr: float = 3e-3, seed: int = 0,
          log=print):
    """Adam on the GPU kernels; returns (BF16 parameters, per-epoch mean loss)."""
    import torch
    dev = torch.device("cuda", 0)
    L = gbr.lib()
    P = num_params()
    master = torch.from_numpy(_init_master(seed)).to(dev)
    wq = torch.from_numpy(to_bf16(master.cpu().numpy()).view(np.int16)).to(dev)
    m = torch.zeros(P, device=dev)
    v = torch.zeros(P, device=dev)
    grad = torch.zeros(P, device=dev)
    loss = torch.zeros(1, device=dev)
    dX = torch.from_numpy(np.ascontiguousarray(X, np.float32)).to(dev)
    dy = torch.from_numpy(np.ascontiguousarray(y, np.float32)).to(dev)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    step = 0
    history = []
    n = len(y)
    p = lambda t: C.c_void_p(t.data_ptr())
    for ep in range(epochs):
        perm = torch.randperm(n, device=dev, generator=g)
        Xs, ys = dX[perm].contiguous(), dy[perm].contiguous()
        tot = 0.0
        for b0 in range(0, n, batch):
            nb = min(batch, n - b0)
            grad.zero_()
            loss.zero_()
            gbr.check(L.gbr_mlp_loss_grad(p(wq), C.c_void_p(Xs.data_ptr() + b0 * NUM_FEATURES * 4),
                                          C.c_void_p(ys.data_ptr() + b0 * 4), nb, p(grad), p(loss), None))
            step += 1
            lr_t = lr * 0.5 * (1 + math.cos(math.pi * step / (epochs * math.ceil(n / batch))))
            gbr.check(L.gbr_mlp_adam(p(master), p(wq), p(grad), p(m), p(v), step, C.c_float(lr_t),
                                     C.c_float(1.0 / nb), None))
            tot += float(loss.item())
        history.append(tot / n)
        if log:
            log(f"epoch {ep + 1}/{epochs}: mean loss {history[-1]:.5f}")
    return wq.cpu().numpy().view(np.uint16).copy(), history


def predict(w_bf16: np.ndarray, X: np.ndarray) -> np.ndarray:
    import torch
    dev = torch.device("cuda", 0)
    dw = torch.from_numpy(w_bf16.view(np.int16)).to(dev)
    dX = torch.from_numpy(np.ascontiguousarray(X, np.float32)).to(dev)
    out = torch.empty(len(X), device=dev)
    gbr.check(gbr.lib().gbr_mlp_predict(C.c_void_p(dw.data_ptr()), C.c_void_p(dX.data_ptr()), len(X),
                                        C.c_void_p(out.data_ptr()), None))
    return out.cpu().numpy()


def capacity(lam, alpha, beta, gamma):
    return np.ceil(lam * (1 + alpha) + beta * np.sqrt(lam + 1.0) + gamma)


def fit_rule(lam: np.ndarray, y: np.ndarray, margin: float = 1.0, rate: float = 1e-6):
    """The (alpha, beta, gamma) of least over-allocation under which at most
    floor(rate * bins) held-out bins overflow: for each (alpha, gamma) on a
    grid, beta is the smallest value that covers all other bins,
    (y - l*(1+alpha) - gamma) / sqrt(l+1), plus `margin`.  The sampled
    pre-pass count of a bin with n triangles has a binomial spread of about
    sqrt(7n) at stride 8, so the sqrt term carries most of the allowance;
    gamma covers bins whose sampled count is 0 although they hold a few dozen
    triangles."""
    lam = np.maximum(np.nan_to_num(np.asarray(lam, np.float64), nan=0.0), 0.0)
    y = np.asarray(y, np.float64)
    root = np.sqrt(lam + 1.0)
    allowed = int(rate * len(y))
    best = None
    for alpha in (0.0, 0.05, 0.1, 0.2, 0.3, 0.5):
        for gamma in (16.0, 32.0, 64.0, 128.0, 256.0, 512.0):
            need = (y - lam * (1 + alpha) - gamma) / root
            worst = np.partition(need, len(need) - 1 - allowed)[len(need) - 1 - allowed] if len(need) > allowed else 0.0
            beta = max(float(worst), 0.0) + margin
            cap = capacity(lam, alpha, beta, gamma)
            alloc = float(cap.sum() / max(y.sum(), 1.0))
            if best is None or alloc < best[0]:
                best = (alloc, alpha, beta, gamma)
    return best[1], best[2], best[3]


def evaluate(w_bf16, rule, frames: int = 12, seed0: int = 10_000, log=print) -> dict:
    """Held-out 1M-triangle 1080p soups rendered with exact and with predicted
    binning: frame overflow rate, over-allocation of the predicted capacities,
    bit-identity of bin lists and images, and per-frame times (CUDA events,
    L2 flushed between frames)."""
    import torch
    dev = torch.device("cuda", 0)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    alpha, beta, gamma = rule
    over = 0
    identical = True
    alloc, t_exact, t_pred, bin_exact, bin_pred = [], [], [], [], []
    for k in range(frames):
        s = scenes.soup_scene(1_000_000, 1920, 1080, 16, seed=seed0 + k)
        out = {}
        for mode in ("exact", "predicted"):
            with gbr.Renderer(s.width, s.height) as r:
                r.load_scene(s)
                if mode == "predicted":
                    gbr.check(r._lib.gbr_set_predictor(r.h, w_bf16.ctypes.data_as(C.c_void_p), len(w_bf16),
                                                       C.c_float(alpha), C.c_float(beta), C.c_float(gamma)))
                    r.set_binning(gbr.BINNING_PREDICTED)
                r.set_timing(True)
                for _ in range(2):
                    r.render_scene(s)
                    r.stats()
                ts, tb = [], []
                for _ in range(5):
                    flush.zero_()
                    r.render_scene(s)
                    st = r.stats()
                    ts.append(st["ms_total"])
                    tb.append(st["ms_setup"] + st["ms_bin"])
                colour, depth = r.readback()
                offsets, bins = r.get_bins()
                out[mode] = (colour, depth, offsets, bins, st, float(np.median(ts)), float(np.median(tb)))
        e, p = out["exact"], out["predicted"]
        identical &= all(np.array_equal(a, b) for a, b in zip(e[:4], p[:4]))
        over += int(p[4]["predicted_overflow"])
        alloc.append(p[4]["predicted_capacity"] / max(e[4]["num_pairs"], 1) - 1.0)
        t_exact.append(e[5]); t_pred.append(p[5]); bin_exact.append(e[6]); bin_pred.append(p[6])
        if log:
            log(f"eval frame {k}: exact {e[5]:.3f} ms, predicted {p[5]:.3f} ms, overflow {p[4]['predicted_overflow']}")
    return {"frames": frames, "frame_overflow_rate": over / frames, "over_allocation": float(np.mean(alloc)),
            "bit_identical": bool(identical), "ms_frame_exact": float(np.mean(t_exact)),
            "ms_frame_predicted": float(np.mean(t_pred)), "ms_binning_exact": float(np.mean(bin_exact)),
            "ms_binning_predicted": float(np.mean(bin_pred)),
            "frame_speedup": float(np.mean(t_exact) / np.mean(t_pred)),
            "binning_speedup": float(np.mean(bin_exact) / np.mean(bin_pred))}


def save(path, w_bf16, alpha, beta, gamma, meta):
    np.savez(path, weights_bf16=w_bf16, rule=np.array([alpha, beta, gamma], np.float32), meta=json.dumps(meta))


def load(path=WEIGHTS):
    d = np.load(path)
    a, b, g = (float(x) for x in d["rule"])
    return d["weights_bf16"].astype(np.uint16), a, b, g, json.loads(str(d["meta"]))


def install(renderer, path=WEIGHTS, sampled: bool = False):
    """Loads the committed model into a renderer and switches it to predicted
    binning.  With `sampled`, the method without the network instead: the
    predicted count of a bin is its sampled pair count times the sampling
    stride, under the capacity rule fitted for it on the same held-out bins
    (meta "sampled_count_rule")."""
    w, a, b, g, meta = load(path)
    if sampled:
        a, b, g = (float(x) for x in meta["sampled_count_rule"])
        gbr.check(renderer._lib.gbr_set_predictor(renderer.h, None, 0, C.c_float(a), C.c_float(b), C.c_float(g)))
    else:
        gbr.check(renderer._lib.gbr_set_predictor(renderer.h, w.ctypes.data_as(C.c_void_p), len(w), C.c_float(a),
                                                  C.c_float(b), C.c_float(g)))
    renderer.set_binning(gbr.BINNING_PREDICTED)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train"])
    ap.add_argument("--pairs", type=int, default=2_000_000)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--val-frames", type=int, default=120)
    ap.add_argument("--eval-frames", type=int, default=12)
    args = ap.parse_args()
    rng = np.random.default_rng(args.seed)
    t0 = time.time()
    frames, total = [], 0
    while total < args.pairs:
        s = training_scene(len(frames), rng)
        frames.append(s)
        total += s.num_bins_x * s.num_bins_y
    val = [training_scene(i, rng) for i in range(args.val_frames)]
    X, y = collect(frames)
    Xv, yv = collect(val, log=None)
    print(f"collected {len(y)} training pairs from {len(frames)} frames, {len(yv)} validation pairs "
          f"({time.time() - t0:.1f}s)", flush=True)
    w, hist = train(X, y, epochs=args.epochs, seed=args.seed)
    lam = predict(w, Xv)
    alpha, beta, gamma = fit_rule(lam, yv)
    cap = capacity(lam, alpha, beta, gamma)
    # the same rule on the plain sampled estimate (8 x sampled pairs) for
    # comparison, in float64 (a float32 sum of a million capacities overflows)
    lam0 = Xv[:, 0].astype(np.float64) * SAMPLED_SCALE
    yv = yv.astype(np.float64)
    lam = lam.astype(np.float64)
    a0, b0, g0 = fit_rule(lam0, yv)
    cap0 = capacity(lam0, a0, b0, g0)
    meta = {"pairs": int(len(y)), "frames": len(frames), "epochs": args.epochs, "loss": hist,
            "val_pairs": int(len(yv)), "val_bin_overflow": float((yv > cap).mean()),
            "val_over_allocation": float(cap.sum() / yv.sum() - 1),
            "val_mean_abs_log_err": float(np.abs(np.log1p(lam) - np.log1p(yv)).mean()),
            "sampled_count_rule": [a0, b0, g0], "sampled_count_over_allocation": float(cap0.sum() / yv.sum() - 1),
            "sampled_count_mean_abs_log_err": float(np.abs(np.log1p(lam0) - np.log1p(yv)).mean()),
            "seed": args.seed}
    print(json.dumps({"rule": [alpha, beta, gamma], **meta}), flush=True)
    if args.eval_frames:
        meta["eval_1m_1080p"] = evaluate(w, (alpha, beta, gamma), frames=args.eval_frames)
        print(json.dumps(meta["eval_1m_1080p"]), flush=True)
    save(args.out, w, alpha, beta, gamma, meta)


if __name__ == "__main__":
    main()
