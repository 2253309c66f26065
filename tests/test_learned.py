"""The learned Newton starting pressure: hand-written training kernels checked
against a CPU autograd reference (torch, FP32, same BF16 rounding of weights,
inputs and activations, straight-through gradients), tensor-core inference
against the FP32 forward pass, training convergence, and what the trained
network gains over the reference's starting pressure inside the FP32 scheme."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _torch_forward(p, X):
    """FP32 reference of the network with BF16 rounding (straight-through)."""
    def q(t):
        return t + (t.to(torch.bfloat16).to(torch.float32) - t).detach()
    W1 = p[0:384].view(64, 6); b1 = p[384:448]; W2 = p[448:4544].view(64, 64); b2 = p[4544:4608]
    w3 = p[4608:4672]; b3 = p[4672]
    x = q(X)
    h1 = q(torch.relu(x @ q(W1).T + b1))
    h2 = q(torch.relu(h1 @ q(W2).T + b2))
    return h2 @ q(w3) + b3


@pytest.mark.gpu
def test_gradient_matches_cpu_autograd(gpu_lib):
    hg = gpu_lib
    net = hg.Mlp(seed=3)
    rng = np.random.default_rng(0)
    X = rng.uniform(-1, 1, (300, 6)).astype(np.float32)
    Y = rng.normal(0, 1, 300).astype(np.float32)
    g_gpu, loss_gpu = net.gradient(X, Y)
    p = torch.tensor(net.params(), requires_grad=True)
    y = _torch_forward(p, torch.tensor(X))
    loss = ((y - torch.tensor(Y)) ** 2).mean()
    loss.backward()
    g_cpu = p.grad.numpy()
    assert abs(loss_gpu - loss.item()) <= 1e-4 * max(1.0, loss.item())
    for name, sl in (("W1", slice(0, 384)), ("b1", slice(384, 448)), ("W2", slice(448, 4544)),
                     ("b2", slice(4544, 4608)), ("w3", slice(4608, 4672)), ("b3", slice(4672, 4673))):
        a, b = g_gpu[sl], g_cpu[sl]
        assert np.linalg.norm(a - b) <= 1e-3 * np.linalg.norm(b) + 1e-7, name


@pytest.mark.gpu
def test_tensor_core_inference_matches_fp32_forward(gpu_lib):
    hg = gpu_lib
    net = hg.Mlp(seed=5)
    rng = np.random.default_rng(1)
    X = rng.uniform(-1, 1, (1000, 6)).astype(np.float32)
    y_tc = net.predict(X)
    with torch.no_grad():
        y_ref = _torch_forward(torch.tensor(net.params()), torch.tensor(X)).numpy()
    d = np.abs(y_tc - y_ref)
    assert d.mean() <= 2e-3 * (np.abs(y_ref).mean() + 1.0)
    assert d.max() <= 5e-2 * (np.abs(y_ref).max() + 1.0)


@pytest.mark.gpu
def test_training_reduces_loss(gpu_lib):
    hg = gpu_lib
    net = hg.Mlp(seed=11)
    net.generate(300_000, seed=5)
    X, Y = net.data(300_000)
    hold = slice(250_000, 300_000)
    before = float(np.mean((net.predict(X[hold]) - Y[hold]) ** 2))
    losses = net.train(4, batch=4096, lr=3e-3, holdout=50_000)
    after = float(np.mean((net.predict(X[hold]) - Y[hold]) ** 2))
    assert losses[-1] < losses[0]
    assert after < 0.2 * before, (before, after)


@pytest.mark.gpu
def test_learned_form_on_weak_waves(gpu_lib):
    """Newton-heavy data (periodic shear layer, most faces exact, every jump
    weak): the learned form leaves the weak jumps to the FP32 form's own
    starting pressure, so it takes no more Newton iterations per exact solve
    than the plain FP32 form, and stays within 1e-5 (relative L1) of the FP64
    form.  (What the network saves against the reference's starting pressure
    is test_learned_start_cost_parts.)"""
    hg = gpu_lib
    from hydro_gb300 import cases

    net = hg.Mlp(seed=2)
    net.generate(1_000_000, seed=9)
    net.train(6, batch=8192, lr=3e-3)
    w = net.params()
    m = n = 256
    rho, u, v, p = cases.shear_layer(m, n, seed=1)
    cfg = hg.config_2d(t_all=-1, steps=20, hx=1.0 / m, hy=1.0 / n, bx=-7, by=-7)
    ref, _ = hg.run_2d(rho, u, v, p, cfg, form=hg.FORM_FP64)
    plain, ip = hg.run_2d(rho, u, v, p, cfg, form=hg.FORM_FP32, stats=True)
    learned, il = hg.run_2d(rho, u, v, p, cfg, form=hg.FORM_FP32_LEARNED, stats=True, mlp=w)
    it_plain = ip.newton_iters / ip.newton_faces
    it_learned = il.newton_iters / il.newton_faces
    assert ip.newton_faces > 0.5 * 2 * m * n * 20  # most faces run the exact solver here
    assert it_learned <= it_plain, (it_plain, it_learned)
    # v is a small perturbation field here (|v| ~ 1e-2): FP32 rounding alone
    # gives it a relative L1 of order 1e-4, so v is held to the plain FP32
    # form's own error; the O(1) fields to 1e-5
    for f in ("rho", "u", "v", "p"):
        rel = np.abs(learned[f] - ref[f]).sum() / np.abs(ref[f]).sum()
        rel_plain = np.abs(plain[f] - ref[f]).sum() / np.abs(ref[f]).sum()
        bound = 1.25 * rel_plain + 1e-7 if f == "v" else 1e-5
        assert rel <= bound, (f, rel, rel_plain)


@pytest.mark.gpu
def test_learned_start_cost_parts(gpu_lib):
    """hydro_learned_costs on 64 K seeded exact-path faces with the shipped
    weights: every part takes time, the network's start needs fewer Newton
    iterations than the reference's (half the tangent intersection), the FP32
    form's own start (the tangent intersection) fewer still, and the
    per-iteration cost derived is positive (the parts the learned-start
    analysis is built on)."""
    hg = gpu_lib
    c = hg.learned_costs(nfaces=65536, seed=3)
    for k in ("network_ns_per_face", "solve_ns_per_face_reference_start", "solve_ns_per_face_learned_start",
              "grp_derivatives_ns_per_face", "exact_face_ns_per_face", "solve_ns_per_face_fp32_start"):
        assert c[k] > 0, (k, c)
    assert 1.0 <= c["iters_learned_start"] < c["iters_reference_start"], c
    assert c["iters_fp32_start"] < c["iters_reference_start"], c
    assert c["ns_per_newton_iteration"] > 0, c
    with pytest.raises(RuntimeError):
        hg.learned_costs(nfaces=16)
