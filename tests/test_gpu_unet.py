"""The learned warm start's U-Net: forward and backward of the library's own BF16
kernels against a float64 PyTorch restatement of the same network on the CPU, a
short capture / train / solve cycle on a small case, and the sweeps the trained
network in the package saves on a held-out run."""
from __future__ import annotations

import pathlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KN = [16, 16, 32, 32, 64, 64, 32, 32, 16, 16]
KK = [16, 16, 16, 32, 32, 64, 96, 32, 48, 16]


def layout():
    """Offsets of each layer's weights [N][27][K] and biases in the parameter vector."""
    off, out = 0, []
    for n, k in zip(KN, KK):
        w = off
        b = w + n * 27 * k
        off = b + n
        off = (off + 7) & ~7
        out.append((w, b, n, k))
    return out, off


def torch_forward(params: np.ndarray, x: np.ndarray, bf16: bool = False):
    """The network in float64 PyTorch. With bf16, every tensor the library stores in
    BF16 (input, weights, activations, pooled and upsampled maps, and in the backward
    pass the gradient of each of them) is rounded to BF16 at the same place."""
    import torch
    import torch.nn.functional as F

    def rb(t):
        return t.to(torch.bfloat16).to(torch.float64) if bf16 else t

    class Stored(torch.autograd.Function):
        @staticmethod
        def forward(ctx, t):
            return rb(t)

        @staticmethod
        def backward(ctx, g):
            return rb(g)

    st = Stored.apply
    lay, head = layout()
    p = torch.tensor(params.astype(np.float64), requires_grad=True)
    xt = torch.tensor(x.astype(np.float64)).permute(0, 4, 1, 2, 3)        # B,4,S,S,S
    xt = rb(torch.cat([xt, torch.zeros(xt.shape[0], 16 - xt.shape[1], *xt.shape[2:], dtype=xt.dtype)], 1))

    def conv(t, l):
        w, b, n, k = lay[l]
        wt = rb(p[w:w + n * 27 * k]).reshape(n, 27, k).permute(0, 2, 1).reshape(n, k, 3, 3, 3)
        return st(F.relu(F.conv3d(t, wt, p[b:b + n], padding=1)))

    up = lambda t: st(F.interpolate(t, scale_factor=2, mode="nearest"))
    pool = lambda t: st(F.avg_pool3d(t, 2))
    a1 = conv(xt, 0); e1 = conv(a1, 1)
    a2 = conv(pool(e1), 2); e2 = conv(a2, 3)
    a3 = conv(pool(e2), 4); b = conv(a3, 5)
    a4 = conv(torch.cat([up(b), st(e2)], 1), 6); d2 = conv(a4, 7)
    a5 = conv(torch.cat([up(d2), st(e1)], 1), 8); d1 = conv(a5, 9)
    out = torch.einsum("bcdhw,c->bdhw", d1, p[head:head + 16]) + p[head + 16]
    return p, out


def reference_grad(params, x, t, bf16):
    import torch
    p, out = torch_forward(params, x, bf16)
    loss = ((out - torch.tensor(t.astype(np.float64))) ** 2).mean()
    loss.backward()
    return loss.item(), p.grad.numpy(), out.detach().numpy()


def compare(grad, ref, rel_max, cos_min, label):
    lay, head = layout()
    blocks = [(l, what, lo, hi) for l, (w, b, n, k) in enumerate(lay)
              for lo, hi, what in ((w, b, "weights"), (b, b + n, "bias"))]
    blocks.append((10, "head", head, head + 17))
    for l, what, lo, hi in blocks:
        g, r = grad[lo:hi], ref[lo:hi]
        if np.linalg.norm(r) == 0:
            continue
        rel = np.linalg.norm(g - r) / np.linalg.norm(r)
        cos = float(np.dot(g, r) / (np.linalg.norm(g) * np.linalg.norm(r)))
        print(f"{label} layer {l} {what}: rel {rel:.3e} cos {cos:.6f}")
        assert rel < rel_max and cos > cos_min, (label, l, what, rel, cos)


def test_tensor_core_weight_gradients_match_the_cuda_core_reduction(ib3d):
    """The weight gradients of the implicit-GEMM tcgen05 kernel (k_wgrad_tc) against
    the FP32 CUDA-core reduction on the same batch: both sum the same BF16 products in
    FP32, in different orders, so every weight block must agree to accumulation
    rounding (relative norm 1e-4); the loss, bias and head gradients do not depend on
    the kernel (their atomic sums may still round differently: 1e-6)."""
    net = ib3d.Net(seed=3)
    lay, head = layout()
    rng = np.random.default_rng(4)
    B, S = 2, 16
    x = rng.standard_normal((B, S, S, S, 4)).astype(np.float32)
    t = rng.standard_normal((B, S, S, S)).astype(np.float32)
    params = net.get_params()
    params[head:head + 16] = rng.standard_normal(16) * 0.3
    net.set_params(params)
    loss_tc, g_tc, _ = net.loss_grad(x, t)
    net.set_wgrad_tensor_cores(False)
    loss_cc, g_cc, _ = net.loss_grad(x, t)
    net.set_wgrad_tensor_cores(True)
    assert abs(loss_tc - loss_cc) <= 1e-6 * loss_cc
    close = lambda a, c: np.linalg.norm(a - c) <= 1e-6 * np.linalg.norm(c) + 1e-30
    for l, (w, b, n, k) in enumerate(lay):
        gt, gc = g_tc[w:b], g_cc[w:b]
        rel = np.linalg.norm(gt - gc) / np.linalg.norm(gc)
        print(f"layer {l} ({n}x{k}): weight gradient rel {rel:.2e}")
        assert rel < 1e-4, (l, rel)
        assert close(g_tc[b:b + n], g_cc[b:b + n]), l
    assert close(g_tc[head:head + 17], g_cc[head:head + 17])
    net.close()


def test_net_loss_and_gradients_match_float64_reference(ib3d):
    """Loss and every parameter gradient of one batch. Against the float64 network
    with the library's BF16 roundings the differences come only from FP32 against
    float64 accumulation; against the plain float64 network they are the BF16
    storage error itself (up to ~11 % on some layers of a random network)."""
    pytest.importorskip("torch")
    net = ib3d.Net(seed=5)
    lay, head = layout()
    assert net.nparams == head + 17
    rng = np.random.default_rng(1)
    B, S = 2, 8
    x = rng.standard_normal((B, S, S, S, 4)).astype(np.float32)
    t = rng.standard_normal((B, S, S, S)).astype(np.float32)
    params = net.get_params()
    params[head:head + 16] = rng.standard_normal(16) * 0.3   # a head large enough to carry gradient
    net.set_params(params)
    loss, grad, out = net.loss_grad(x, t)
    l16, g16, o16 = reference_grad(params, x, t, True)
    l64, g64, o64 = reference_grad(params, x, t, False)
    assert np.linalg.norm(out - o16) <= 1e-2 * np.linalg.norm(o16)
    assert abs(loss - l16) <= 5e-3 * l16
    compare(grad, g16, 4e-2, 0.999, "bf16-rounded float64")
    assert np.linalg.norm(out - o64) <= 3e-2 * np.linalg.norm(o64)
    assert abs(loss - l64) <= 2e-2 * l64
    compare(grad, g64, 0.25, 0.97, "float64")
    net.close()


def test_capture_train_and_learned_warm_start(ib3d, grids):
    """Patches captured from a small run train the network: on the same batches
    (chosen by seed; lr = 0 evaluates without moving the weights) the loss falls.
    Steps warm-started by it still stop at the same FP64 residual, with drag/lift
    within 1e-4 of the FP64 path."""
    cs = grids.case("small")
    common = dict(precision=ib3d.PREC_FP32DC, criterion=ib3d.CRIT_RESIDUAL, eps=1e-6, inner_sweeps=64)
    src = ib3d.setup_case(cs, warm_start=ib3d.WARM_PREV, **common)
    src.enable_history()
    net = ib3d.Net(seed=0)
    net.reserve(16, 256)         # 16^3 voxels of 2x2x2 cells: 32^3 cells of the 64x48x48 grid
    for step in range(1, 9):
        src.step(step == 1)
        if step >= 3:
            net.capture(src, 16, seed=step)
    assert net.dataset_size() == 96

    def fit():
        return float(np.mean([net.train(1, batch=8, lr=0.0, seed=1000 + q) for q in range(8)]))

    before = fit()
    net.train(300, batch=4, lr=1e-3, seed=2)
    after = fit()
    print(f"training-set loss {before:.4f} -> {after:.4f}")
    assert after < 0.8 * before, (before, after)
    ref = ib3d.setup_case(cs, precision=ib3d.PREC_FP64, criterion=ib3d.CRIT_RESIDUAL, eps=1e-6, check_every=1)
    lrn = ib3d.setup_case(cs, warm_start=ib3d.WARM_LEARNED, **common)
    lrn.attach_net(net)
    for step in range(1, 6):
        _, c64 = ref.step(step == 1)
        st, cl = lrn.step(step == 1)
        print(f"step {step}: learned warm start {st['sweeps']} sweeps")
        assert st["final_err"] < 1e-6
    assert abs((cl[0] + cl[1]) - (c64[0] + c64[1])) <= 1e-4 * abs(c64[0] + c64[1])
    for s in (src, ref, lrn):
        s.close()
    net.close()


WEIGHTS_DIR = pathlib.Path(__file__).resolve().parent.parent / "ib3d-gpu_gb300" / "weights"


def _networks():
    import json
    manifest = WEIGHTS_DIR / "networks.json"
    return json.loads(manifest.read_text())["networks"] if manifest.exists() else {}


@pytest.mark.parametrize("name", sorted(_networks()))
def test_trained_network_saves_sweeps(ib3d, grids, name):
    """What a trained network of the package gains: on a held-out Reynolds number
    (275; trained at 200/250/300/350) of the 256x192x192 sphere, the learned warm
    start needs fewer SOR sweeps than the previous-correction warm start over steps
    3-8 (the network acts from step 3), both stopping at the same FP64 residual 1e-6
    (pass lengths adaptive so that the counts resolve small differences); drag and
    lift agree within 1e-4."""
    import dataclasses
    import importlib
    learned = importlib.import_module("ib3d_gpu_gb300.learned")
    net = ib3d.Net(seed=0)
    net.set_coarsening(int(_networks()[name]["coarsen"]))
    net.set_params(np.fromfile(WEIGHTS_DIR / name, dtype="<f4"))
    cs = dataclasses.replace(grids.case("sphere256"), omega=1.99, eps=1e-6)
    ev = learned.evaluate(net, cs, 275.0, 8, inner_schedule=1)
    prev, lrn = ev["prev"], ev["learned"]
    saved = 1.0 - sum(lrn["sweeps"][2:]) / sum(prev["sweeps"][2:])
    print(f"{name}: sweeps previous-correction {prev['sweeps']}, learned {lrn['sweeps']}: {100 * saved:.1f} % saved")
    assert saved > 0.0
    c0, c1 = np.array(prev["coef"][-1]), np.array(lrn["coef"][-1])
    assert abs((c1[0] + c1[1]) - (c0[0] + c0[1])) <= 1e-4 * abs(c0[0] + c0[1])
    net.close()


def test_smoothing_sweeps_cut_the_sweeps_after_a_coarse_guess(ib3d, grids):
    """The default network's guess is a 4x4x4-voxel field taken back by trilinear
    interpolation; Gauss-Seidel sweeps at the start of the solve (smooth_sweeps) damp
    the rough error it leaves, which over-relaxed sweeps barely touch. On the
    256x192x192 sphere, steps 3-6 (the network acts from step 3) need fewer sweeps
    with six smoothing sweeps than with none, at the same FP64 residual, with drag
    and lift within 1e-4."""
    import dataclasses
    import json
    info = json.loads((WEIGHTS_DIR / "networks.json").read_text())
    name = info["default"]
    cs = dataclasses.replace(grids.case("sphere256"), omega=1.99, eps=1e-6)
    runs = {}
    for smooth in (0, 6):
        net = ib3d.Net(seed=0)
        net.set_coarsening(int(info["networks"][name]["coarsen"]))
        net.set_params(np.fromfile(WEIGHTS_DIR / name, dtype="<f4"))
        s = ib3d.setup_case(cs, precision=ib3d.PREC_FP32DC, criterion=ib3d.CRIT_RESIDUAL, warm_start=ib3d.WARM_LEARNED,
                            inner_sweeps=512, inner_schedule=ib3d.INNER_TAIL, omega_inner=1.9937,
                            smooth_sweeps=smooth, max_sweeps=400000)
        s.attach_net(net)
        sweeps = []
        for step in range(1, 7):
            st, coef = s.step(step == 1)
            assert st["final_err"] < 1e-6
            sweeps.append(st["sweeps"])
        runs[smooth] = (sweeps, np.asarray(coef))
        s.close()
        net.close()
    print(f"sweeps without smoothing {runs[0][0]}, with six smoothing sweeps {runs[6][0]}")
    assert sum(runs[6][0][2:]) < sum(runs[0][0][2:])
    c0, c6 = runs[0][1], runs[6][1]
    assert abs((c6[0] + c6[1]) - (c0[0] + c0[1])) <= 1e-4 * abs(c0[0] + c0[1])
