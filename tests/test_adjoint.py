"""Hand-written adjoint of the recurrent LIF network.

GPU: gradients of the CUDA forward + adjoint (FP32) against
  * FP64 torch autograd of the same discretised dynamics (reference_forward):
    spiking mode with the fast-sigmoid surrogate, slope 10 (tolerance 1e-3 of
    the largest gradient entry; FP32 autograd itself sits at ~7e-5), and
    sigmoid-smoothed mode (tolerance 1e-4);
  * central finite differences, eps = 1e-3, of the FP64 loss in smoothed mode
    (2e-3 relative per checked entry plus 1e-5 of the largest entry).
The smoothed mode uses sigmoid slope 0.5: at slope 10 the smooth recurrence
is chaotic over 60 steps (gradient norms 1e3-1e7; FP32 and FP64 autograd
themselves disagree by 1e-1 and more), so no finite-difference or
cross-precision check is meaningful there.
CPU: torch.autograd.gradcheck of reference_forward itself in FP64.
"""
import math

import numpy as np
import pytest
import torch

from neuronbridge_gb300.adjoint import reference_forward

KW = dict(n_in=16, n_rec=32, n_out=5, checkpoint=20, seed=11)
T, B = 60, 4
SPIKING = dict(weight_scale=20.0, slope=10.0)
SMOOTH = dict(weight_scale=10.0, slope=0.5)


def _setup(smooth, device="cuda"):
    from neuronbridge_gb300.adjoint import RecurrentLIF, poisson_inputs

    torch.manual_seed(0)
    model = RecurrentLIF(smooth=smooth, device=device, **KW, **(SMOOTH if smooth else SPIKING))
    rates = torch.linspace(5.0, 50.0, KW["n_in"]) * 8.0
    x = poisson_inputs(rates, T, B, dt=1.0, seed=3)
    labels = torch.randint(0, KW["n_out"], (B,), generator=torch.Generator().manual_seed(6)).to(device)
    return model, x, labels


def _params(model):
    return [model.w_in, model.w_rec, model.w_out, model.alpha, model.theta]


def _ref_loss(model, x, labels, params, smooth):
    """FP64 loss of the same dynamics (slope and refractoriness from the model)."""
    y = reference_forward(x, *params, smooth=smooth, t_ref=model.params.t_ref, slope=model.params.slope)
    return torch.nn.functional.cross_entropy(y, labels)


@pytest.mark.gpu
@pytest.mark.parametrize("smooth", [True, False])
def test_adjoint_matches_fp64_autograd(smooth):
    model, x, labels = _setup(smooth)
    loss = torch.nn.functional.cross_entropy(model(x), labels)
    loss.backward()
    ours = [p.grad.detach().double().cpu() for p in _params(model)]
    ref_params = [p.detach().double().cpu().requires_grad_(True) for p in _params(model)]
    ref_loss = _ref_loss(model, x.double().cpu(), labels.cpu(), ref_params, smooth)
    ref_loss.backward()
    assert abs(loss.item() - ref_loss.item()) < 1e-4 * max(1.0, abs(ref_loss.item()))
    tol = 1e-4 if smooth else 1e-3
    for name, g, r in zip(("w_in", "w_rec", "w_out", "alpha", "theta"), ours, ref_params):
        scale = r.grad.abs().max().item()
        assert scale > 0, name
        err = (g - r.grad).abs().max().item()
        assert err <= tol * scale, (name, err, scale)


@pytest.mark.gpu
def test_adjoint_matches_central_differences_smoothed():
    model, x, labels = _setup(True)
    torch.nn.functional.cross_entropy(model(x), labels).backward()
    xd, ld = x.double().cpu(), labels.cpu()
    base = [p.detach().double().cpu() for p in _params(model)]
    rng = np.random.default_rng(1)
    eps = 1e-3
    for pi, p in enumerate(_params(model)):
        g = p.grad.detach().double().cpu().reshape(-1)
        gmax = g.abs().max().item()
        for idx in rng.choice(g.numel(), size=min(6, g.numel()), replace=False):
            vals = []
            for sgn in (1, -1):
                ps = [b.clone() for b in base]
                ps[pi].view(-1)[idx] += sgn * eps
                vals.append(_ref_loss(model, xd, ld, ps, True).item())
            fd = (vals[0] - vals[1]) / (2 * eps)
            assert abs(fd - g[idx].item()) <= 2e-3 * abs(fd) + 1e-5 * gmax, (pi, int(idx), fd, g[idx].item())


@pytest.mark.gpu
def test_full_size_step_runs():
    from neuronbridge_gb300.adjoint import RecurrentLIF, poisson_inputs

    model = RecurrentLIF()  # 256 -> 1024 -> 10, T = 1000, checkpoints every 100
    rates = torch.empty(256).uniform_(5.0, 50.0, generator=torch.Generator().manual_seed(5))
    x = poisson_inputs(rates, 1000, 128, dt=1.0, seed=5)
    labels = torch.randint(0, 10, (128,), generator=torch.Generator().manual_seed(6)).cuda()
    loss = torch.nn.functional.cross_entropy(model(x), labels)
    loss.backward()
    for p in _params(model):
        assert torch.isfinite(p.grad).all()


def _grads(model, x, labels):
    model.zero_grad(set_to_none=True)
    loss = torch.nn.functional.cross_entropy(model(x), labels)
    loss.backward()
    return loss.item(), [p.grad.detach().clone() for p in _params(model)]


def _close(a, b, rel=1e-5):
    for g, r in zip(a, b):
        assert (g - r).abs().max().item() <= rel * max(1e-30, r.abs().max().item())


@pytest.mark.gpu
def test_graph_replay_matches_eager_with_ragged_segment_and_sgd_steps():
    """The captured-graph path (default) against eager launches of the same
    kernels: T = 70 with checkpoints every 20 leaves a 10-step last segment;
    three SGD steps in place reuse one captured plan."""
    from neuronbridge_gb300.adjoint import RecurrentLIF, poisson_inputs

    models = [RecurrentLIF(use_graphs=g, **KW, **SPIKING) for g in (False, True)]
    x = poisson_inputs(torch.linspace(40.0, 400.0, KW["n_in"]), 70, B, dt=1.0, seed=4)
    labels = torch.randint(0, KW["n_out"], (B,), generator=torch.Generator().manual_seed(2)).cuda()
    for _ in range(3):
        (la, ga), (lb, gb) = (_grads(m, x, labels) for m in models)
        assert abs(la - lb) <= 1e-6 * max(1.0, abs(la))
        _close(gb, ga)
        for m in models:  # a small normalised step keeps the dynamics in range
            with torch.no_grad():
                for q in _params(m):
                    q -= 1e-3 * q.grad / q.grad.abs().max().clamp(min=1e-30)
    assert len(models[1]._plans) == 1


@pytest.mark.gpu
@pytest.mark.parametrize("record", [False, True])
def test_graph_plan_backward_after_interleaved_forwards(record):
    """Two forwards before either backward: each backward restores its own
    inputs and checkpoints into the plan's static buffers (replay mode) or
    runs its forward again to rebuild the record (record mode)."""
    from neuronbridge_gb300.adjoint import RecurrentLIF, poisson_inputs

    model = RecurrentLIF(record=record, **KW, **SPIKING)
    xs = [poisson_inputs(torch.linspace(40.0, 400.0, KW["n_in"]), T, B, dt=1.0, seed=s) for s in (5, 6)]
    labels = torch.randint(0, KW["n_out"], (B,), generator=torch.Generator().manual_seed(2)).cuda()
    alone = [_grads(model, x, labels)[1] for x in xs]
    model.zero_grad(set_to_none=True)
    losses = [torch.nn.functional.cross_entropy(model(x), labels) for x in xs]
    for loss, want in zip(losses, alone):
        model.zero_grad(set_to_none=True)
        loss.backward()
        _close([p.grad for p in _params(model)], want)


@pytest.mark.gpu
@pytest.mark.parametrize("graphs", [False, True])
def test_recorded_state_gradients_equal_replayed(graphs):
    """Recording every step's state in the forward and replaying segments
    from checkpoints in the backward run the same kernels on the same values:
    the loss and the W_out, alpha and theta gradients are bitwise equal, and
    W_in and W_rec (one product over the whole run with the record, one per
    segment with the replay: other split-K sums) agree to FP32 rounding.
    T = 70 with segments of 20 leaves a ragged last segment; N = 512 takes
    the fused tensor-core adjoint step."""
    from neuronbridge_gb300.adjoint import RecurrentLIF, poisson_inputs

    kw = dict(n_in=64, n_rec=512, n_out=5, checkpoint=20, seed=11)
    x = poisson_inputs(torch.linspace(5.0, 50.0, kw["n_in"]) * 8.0, 70, 128, dt=1.0, seed=3)
    labels = torch.randint(0, kw["n_out"], (128,), generator=torch.Generator().manual_seed(6)).cuda()
    out = [_grads(RecurrentLIF(record=r, use_graphs=graphs, **kw, **SPIKING), x, labels) for r in (False, True)]
    assert out[0][0] == out[1][0]
    for name, a, b in zip(("w_in", "w_rec", "w_out", "alpha", "theta"), out[0][1], out[1][1]):
        if name in ("w_in", "w_rec"):
            assert (a - b).abs().max().item() <= 1e-5 * a.abs().max().item(), name
        else:
            assert torch.equal(a, b), name


def test_record_mode_default_follows_budget():
    from neuronbridge_gb300 import adjoint

    assert adjoint.record_bytes(1000, 128, 1024) == 1000 * 128 * 1024 * 9 + 1001 * 128 * 1024 * 4
    assert adjoint.record_bytes(1000, 128, 1024) <= adjoint.RECORD_BUDGET_BYTES  # the benchmark's size records
    assert adjoint.record_bytes(10000, 512, 4096) > adjoint.RECORD_BUDGET_BYTES  # this one replays


def test_reference_dynamics_gradcheck_cpu():
    torch.manual_seed(0)
    Tn, Bn, C, N, O = 8, 2, 3, 4, 2
    x = (torch.rand(Tn, Bn, C, dtype=torch.float64) < 0.3).double()
    params = [torch.randn(C, N, dtype=torch.float64) * 8, torch.randn(N, N, dtype=torch.float64) * 5,
              torch.randn(N, O, dtype=torch.float64), torch.full((N,), 0.05, dtype=torch.float64),
              torch.full((N,), -50.0, dtype=torch.float64)]
    params = [p.requires_grad_(True) for p in params]
    f = lambda *ps: reference_forward(x, *ps, smooth=True, slope=1.0)
    assert torch.autograd.gradcheck(f, params, eps=1e-6, atol=1e-6, rtol=1e-4)
    assert math.isfinite(f(*params).sum().item())


@pytest.mark.gpu
def test_tensor_core_recurrent_product(monkeypatch):
    """B = 128 rows, N and C multiples of 256, spiking mode: dI_{t+1} W_rec^T
    and the segments' weight gradients S^T dI and X^T dI run on tcgen05 in
    split BF16.  Gradients stay within the FP64 tolerance of the spiking test
    and agree with the cuBLAS FP32 path."""
    from neuronbridge_gb300 import adjoint
    from neuronbridge_gb300.adjoint import RecurrentLIF, poisson_inputs

    kw = dict(n_in=256, n_rec=256, n_out=5, checkpoint=20, seed=11)  # W_in gradient on the tensor cores too
    torch.manual_seed(0)
    model = RecurrentLIF(smooth=False, device="cuda", use_graphs=False, **kw, **SPIKING)
    rates = torch.linspace(5.0, 50.0, kw["n_in"]) * 8.0
    x = poisson_inputs(rates, T, 128, dt=1.0, seed=3)
    labels = torch.randint(0, kw["n_out"], (128,), generator=torch.Generator().manual_seed(6)).cuda()
    assert adjoint._tc_ok(model.params, 128, 256)
    loss_tc, tc = _grads(model, x, labels)
    monkeypatch.setattr(adjoint, "_tc_ok", lambda p, B, N: False)
    loss_fp32, fp32 = _grads(model, x, labels)
    assert loss_tc == loss_fp32  # same forward
    ref_params = [p.detach().double().cpu().requires_grad_(True) for p in _params(model)]
    ref_loss = _ref_loss(model, x.double().cpu(), labels.cpu(), ref_params, False)
    ref_loss.backward()
    for name, g, h, r in zip(("w_in", "w_rec", "w_out", "alpha", "theta"), tc, fp32, ref_params):
        scale = r.grad.abs().max().item()
        assert (g.double().cpu() - r.grad).abs().max().item() <= 1e-3 * scale, name
        assert (g - h).abs().max().item() <= 1e-3 * h.abs().max().item(), name


@pytest.mark.gpu
def test_segment_forward_equals_per_step_launches():
    """nbg_lif_forward_segment_sparse (a checkpoint segment in one launch, each
    CTA running its row through every step) gives bit for bit what one
    nbg_lif_forward_step_sparse launch per step gives."""
    from neuronbridge_gb300.adjoint import GradParams, _bind, _SpikeLists, _stream

    lib = _bind()
    g = torch.Generator(device="cuda").manual_seed(1)
    B, N, L = 48, 640, 37
    w = torch.randn(N, N, device="cuda", generator=g) * 0.3
    xi = torch.rand(L, B, N, device="cuda", generator=g) * 0.3
    alpha = torch.full((N,), 0.05, device="cuda")
    theta = torch.rand(N, device="cuda", generator=g) * 0.5 + 0.5
    p = GradParams(0.0, 0.0, 10.0, 3, 0)
    c = torch.linspace(0.1, 1.0, L, device="cuda")
    s0 = (torch.rand(B, N, device="cuda", generator=g) < 0.05).float()
    v0 = torch.rand(B, N, device="cuda", generator=g)
    ref0 = torch.randint(0, 4, (B, N), device="cuda", dtype=torch.int32, generator=g)
    st = _stream()
    out = []
    for segment in (False, True):
        lists = _SpikeLists(B, N, "cuda")
        v, ref = v0.clone(), ref0.clone()
        S = torch.zeros((L + 1, B, N), device="cuda")
        U = torch.zeros((L, B, N), device="cuda")
        M = torch.zeros((L, B, N), device="cuda", dtype=torch.uint8)
        VP = torch.zeros((L, B, N), device="cuda")
        z = torch.zeros((B, N), device="cuda")
        lists.load(lib, s0, B, N, st)
        if segment:
            lists.segment(lib, xi, w, v, ref, S[1], None, U, M, VP, z, c, alpha, theta, p, L, B, N, st)
        else:
            for k in range(L):
                lists.step(lib, xi[k], w, v, ref, S[k + 1], U[k], M[k], VP[k], z, float(c[k]), alpha, theta, p, B,
                           N, st)
        torch.cuda.synchronize()
        cnt = lists.cnt[lists.cur].clone()
        idx = torch.cat([lists.idx[lists.cur][b][:int(cnt[b])] for b in range(B)])
        out.append((v, ref, S, U, M, VP, z, cnt, idx))
    assert out[0][2].sum() > 0  # the rows spike
    for a, b in zip(out[0], out[1]):
        assert torch.equal(a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("binary", [True, False])
def test_segment_gather_equals_ascending_input_sum(binary):
    """nbg_lif_forward_segment_gather (the input term gathered over each row's
    nonzero inputs inside the segment launch) equals the precomputed-input
    segment fed xi_t = sum over c, ascending, of x_t[:, c] * W_in[c] in FP32,
    bit for bit: spike inputs (exact products) and sparse real-valued ones,
    with more channels than the CTA has threads."""
    from neuronbridge_gb300.adjoint import GradParams, _bind, _SpikeLists, _stream

    lib = _bind()
    g = torch.Generator(device="cuda").manual_seed(2)
    B, N, L, C = 32, 512, 25, 300
    w_rec = torch.randn(N, N, device="cuda", generator=g) * 0.3
    w_in = torch.randn(C, N, device="cuda", generator=g) * 0.5
    x = (torch.rand(L, B, C, device="cuda", generator=g) < 0.05).float()
    if not binary:
        x = x * torch.rand(L, B, C, device="cuda", generator=g) * 2.0
    xi = torch.zeros(L, B, N, device="cuda")
    for ch in range(C):  # elementwise adds: ascending channel order, one rounding each
        xi = xi + x[:, :, ch:ch + 1] * w_in[ch]
    alpha = torch.full((N,), 0.05, device="cuda")
    theta = torch.rand(N, device="cuda", generator=g) * 0.5 + 0.5
    p = GradParams(0.0, 0.0, 10.0, 3, 0)
    c = torch.linspace(0.1, 1.0, L, device="cuda")
    st = _stream()
    out = []
    for gather in (False, True):
        lists = _SpikeLists(B, N, "cuda")
        v, ref = torch.zeros(B, N, device="cuda"), torch.zeros(B, N, device="cuda", dtype=torch.int32)
        S = torch.zeros((L + 1, B, N), device="cuda")
        U = torch.zeros((L, B, N), device="cuda")
        z = torch.zeros((B, N), device="cuda")
        lists.load(lib, S[0], B, N, st)
        if gather:
            lists.segment_gather(lib, x, w_in, w_rec, v, ref, S[1], None, U, None, None, z, c, alpha, theta, p, L,
                                 B, N, st)
        else:
            lists.segment(lib, xi, w_rec, v, ref, S[1], None, U, None, None, z, c, alpha, theta, p, L, B, N, st)
        torch.cuda.synchronize()
        out.append((v, ref, S, U, z))
    assert out[0][2].sum() > 0
    for a, b in zip(out[0], out[1]):
        assert torch.equal(a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("n_rec", [512, 1024])
def test_fused_adjoint_step_equals_two_launch_form(monkeypatch, n_rec):
    """N = 512 and 1024, B = 128, spiking mode: each backward step as one launch
    (nbg_lif_adjoint_step_fused, split-K partials reduced through distributed
    shared memory) gives the same gradients, bit for bit, as the product and
    the step as two launches, and stays within the FP64 tolerance."""
    from neuronbridge_gb300 import adjoint
    from neuronbridge_gb300.adjoint import RecurrentLIF, poisson_inputs

    kw = dict(n_in=64, n_rec=n_rec, n_out=5, checkpoint=20, seed=11)
    torch.manual_seed(0)  # replay mode: both forms take the weight gradients per segment
    model = RecurrentLIF(smooth=False, device="cuda", use_graphs=False, record=False, **kw, **SPIKING)
    rates = torch.linspace(5.0, 50.0, kw["n_in"]) * 8.0
    x = poisson_inputs(rates, T, 128, dt=1.0, seed=3)
    labels = torch.randint(0, kw["n_out"], (128,), generator=torch.Generator().manual_seed(6)).cuda()
    assert adjoint._fused_ok(model.params, 128, n_rec)
    loss_f, fused = _grads(model, x, labels)
    monkeypatch.setattr(adjoint, "FUSED_STEP", False)
    loss_u, unfused = _grads(model, x, labels)
    assert loss_f == loss_u
    for g, h in zip(fused, unfused):
        assert torch.equal(g, h)
    ref_params = [p.detach().double().cpu().requires_grad_(True) for p in _params(model)]
    ref_loss = _ref_loss(model, x.double().cpu(), labels.cpu(), ref_params, False)
    ref_loss.backward()
    for name, g, r in zip(("w_in", "w_rec", "w_out", "alpha", "theta"), fused, ref_params):
        scale = r.grad.abs().max().item()
        assert (g.double().cpu() - r.grad).abs().max().item() <= 1e-3 * scale, name


@pytest.mark.gpu
def test_tensor_core_weight_gradients_padded_shapes(monkeypatch):
    """N = 384 and C = 100 (not multiples of the weight-gradient tile of 256):
    the tensor-core weight gradients pad S^T and X^T with zero rows, and the
    gradients stay within the FP64 tolerance and agree with the cuBLAS FP32
    path."""
    from neuronbridge_gb300 import adjoint
    from neuronbridge_gb300.adjoint import RecurrentLIF, poisson_inputs

    kw = dict(n_in=100, n_rec=384, n_out=5, checkpoint=20, seed=11)
    torch.manual_seed(0)
    model = RecurrentLIF(smooth=False, device="cuda", use_graphs=False, **kw, **SPIKING)
    rates = torch.linspace(5.0, 50.0, kw["n_in"]) * 8.0
    x = poisson_inputs(rates, T, 128, dt=1.0, seed=3)
    labels = torch.randint(0, kw["n_out"], (128,), generator=torch.Generator().manual_seed(6)).cuda()
    assert adjoint._tc_ok(model.params, 128, 384)
    loss_tc, tc = _grads(model, x, labels)
    monkeypatch.setattr(adjoint, "_tc_ok", lambda p, B, N: False)
    loss_fp32, fp32 = _grads(model, x, labels)
    assert loss_tc == loss_fp32
    ref_params = [p.detach().double().cpu().requires_grad_(True) for p in _params(model)]
    ref_loss = _ref_loss(model, x.double().cpu(), labels.cpu(), ref_params, False)
    ref_loss.backward()
    for name, g, h, r in zip(("w_in", "w_rec", "w_out", "alpha", "theta"), tc, fp32, ref_params):
        scale = r.grad.abs().max().item()
        assert (g.double().cpu() - r.grad).abs().max().item() <= 1e-3 * scale, name
        assert (g - h).abs().max().item() <= 1e-3 * h.abs().max().item(), name
