"""Differentiable recurrent LIF network with a hand-written adjoint.

``RecurrentLIF`` runs T steps of the voltage-jump LIF recurrence of
``include/nbg_adjoint.h`` for a batch of B input sequences and returns the
time-averaged leaky readout.  Its backward is not autograd: the forward either records the state
the adjoint reads (u_t, s_t, m_t, v_{t-1}) at every step, or saves the network
state every ``checkpoint`` steps and lets the backward replay each segment from
its checkpoint; the backward then runs the fused adjoint kernel in reverse
time.  Recording is the default while the records fit in
RECORD_BUDGET_BYTES (13 bytes per neuron, row and step: 1.7 GB at
T = 1000, B = 128, N = 1024), which takes the replay, a third of the
backward, off the training step.

* Spiking mode: the forward (and the backward's replay) runs each
  segment in one launch per row block: the input current of a step is the
  sum of the W_in rows of the row's nonzero inputs (x_t times the row) and
  the W_rec rows of its previous spikes, each in ascending order, so there
  is no GEMM in the forward at all.  The adjoint's recurrent term
  dI_{t+1} W_rec^T and the weight gradients run on tcgen05 in split BF16
  (nbg_adjoint_tc.cu) where the shapes allow (B = 128, N a multiple of
  128), else as the engine's FP32 CUDA-core product (nbg_small_gemm).
* Smoothed (sigmoid) mode, the finite-difference test mode: x W_in and
  s_{t-1} W_rec are that FP32 product too, followed by the fused elementwise
  step.  No cuBLAS kernel runs in either mode.
* All elementwise work of an adjoint step is one fused kernel.

Readout: y_t = a_out y_{t-1} + s_t W_out, a_out = exp(-dt / tau_out), and
mean_t y_t = (sum_t c_t s_t) W_out with c_t = (1 - a_out^(T-t)) / ((1 - a_out) T),
so the forward only accumulates z = sum_t c_t s_t.

Trainable: W_in, W_rec, W_out, and per-neuron alpha = dt / tau and threshold.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib


class GradParams(ctypes.Structure):
    _fields_ = [("v_rest", ctypes.c_float), ("v_reset", ctypes.c_float), ("slope", ctypes.c_float),
                ("t_ref", ctypes.c_int), ("smooth", ctypes.c_int)]


_vp = ctypes.c_void_p
_SIG = {
    "nbg_lif_forward_step": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_float, _vp, _vp,
                                            ctypes.POINTER(GradParams), ctypes.c_int, ctypes.c_int, _vp]),
    "nbg_lif_adjoint_step": (ctypes.c_int, [_vp, _vp, ctypes.c_float, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                            _vp, ctypes.POINTER(GradParams), ctypes.c_int, ctypes.c_int, _vp]),
    "nbg_poisson_inputs": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                          ctypes.c_int, _vp]),
    "nbg_lif_forward_step_sparse": (ctypes.c_int, [_vp] * 13 + [ctypes.c_float, _vp, _vp, ctypes.POINTER(GradParams),
                                                                ctypes.c_int, ctypes.c_int, _vp]),
    "nbg_spike_lists": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp]),
    "nbg_lif_forward_segment_gather": (ctypes.c_int, [_vp, _vp, ctypes.c_int] + [_vp] * 14 +
                                       [ctypes.POINTER(GradParams), ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp]),
    "nbg_lif_forward_segment_sparse": (ctypes.c_int, [_vp] * 15 + [ctypes.POINTER(GradParams), ctypes.c_int,
                                                                  ctypes.c_int, ctypes.c_int, _vp]),
    "nbg_adjoint_rec_prepare": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, _vp]),
    "nbg_lif_adjoint_step_split": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_float] + [_vp] * 12 +
                                   [ctypes.POINTER(GradParams), ctypes.c_int, ctypes.c_int, _vp]),
    "nbg_adjoint_rec_grad": (ctypes.c_int, [_vp] * 5 + [ctypes.c_int] * 3 + [_vp, _vp]),
    "nbg_lif_adjoint_step_fused": (ctypes.c_int, [_vp] * 7 + [ctypes.c_float] + [_vp] * 10 +
                                   [ctypes.POINTER(GradParams), ctypes.c_int, ctypes.c_int, _vp, _vp,
                                    ctypes.c_int64, ctypes.c_int64, _vp, _vp]),
    "nbg_adjoint_blocked_t": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp,
                                             _vp]),
    "nbg_small_gemm": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _vp, ctypes.c_int, ctypes.c_int, _vp,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp]),
    "nbg_adjoint_wgrad": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp,
                                         ctypes.c_int, _vp, _vp]),
    "nbg_adjoint_reduce_add": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int64, ctypes.c_int64, _vp]),
}
_LIB = None


def _bind():
    global _LIB
    if _LIB is None:
        lib = _lib.load()
        for name, (res, args) in _SIG.items():
            fn = getattr(lib, name)
            fn.restype, fn.argtypes = res, args
        _LIB = lib
    return _LIB


def _ptr(t: torch.Tensor | None):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def poisson_inputs(rates_hz: torch.Tensor, T: int, B: int, dt: float = 1.0, seed: int = 0) -> torch.Tensor:
    """Seeded Poisson input spikes x[t, b, c] (device float32 0/1)."""
    lib = _bind()
    rates = rates_hz.to(device="cuda", dtype=torch.float32).contiguous()
    C = rates.numel()
    x = torch.empty((T, B, C), device=rates.device, dtype=torch.float32)
    _lib.check(lib.nbg_poisson_inputs(_ptr(x), _ptr(rates), T, B, C, float(dt), int(seed), _stream()))
    return x


def readout_coefficients(T: int, a_out: float) -> np.ndarray:
    t = np.arange(T, dtype=np.float64)
    return ((1.0 - a_out ** (T - t)) / ((1.0 - a_out) * T)).astype(np.float32)


class _SpikeLists:
    """Double-buffered ascending spike lists of the B rows (spiking mode): the
    recurrent input s_{t-1} W_rec is a gather-sum over them."""

    def __init__(self, B: int, N: int, device):
        self.idx = torch.empty((2, B, N), device=device, dtype=torch.int32)
        self.cnt = torch.zeros((2, B), device=device, dtype=torch.int32)
        self.cur = 0

    def load(self, lib, s, B, N, st):
        _lib.check(lib.nbg_spike_lists(_ptr(s), _ptr(self.idx[self.cur]), _ptr(self.cnt[self.cur]), B, N, st))

    def segment(self, lib, xi, w_rec, v, ref, s_out, s_last, u_rec, m_rec, vp_rec, z, c, alpha, theta, p, L, B, N,
                st):
        """L steps in one launch (nbg_lif_forward_segment_sparse); the lists
        are updated in place."""
        _lib.check(lib.nbg_lif_forward_segment_sparse(
            _ptr(xi), _ptr(w_rec), _ptr(self.idx[self.cur]), _ptr(self.cnt[self.cur]), _ptr(v), _ptr(ref),
            _ptr(s_out), _ptr(s_last), _ptr(u_rec), _ptr(m_rec), _ptr(vp_rec), _ptr(z), _ptr(c), _ptr(alpha),
            _ptr(theta), ctypes.byref(p), L, B, N, st))

    def segment_gather(self, lib, x, w_in, w_rec, v, ref, s_out, s_last, u_rec, m_rec, vp_rec, z, c, alpha, theta,
                       p, L, B, N, st):
        """As segment, with the input term x_t W_in gathered over each row's
        nonzero inputs inside the same launch (nbg_lif_forward_segment_gather)."""
        C = x.shape[-1]
        _lib.check(lib.nbg_lif_forward_segment_gather(
            _ptr(x), _ptr(w_in), C, _ptr(w_rec), _ptr(self.idx[self.cur]), _ptr(self.cnt[self.cur]), _ptr(v),
            _ptr(ref), _ptr(s_out), _ptr(s_last), _ptr(u_rec), _ptr(m_rec), _ptr(vp_rec), _ptr(z), _ptr(c),
            _ptr(alpha), _ptr(theta), ctypes.byref(p), L, B, N, st))

    def step(self, lib, xi, w_rec, v, ref, s_out, u_rec, m_rec, vp_rec, z, c, alpha, theta, p, B, N, st):
        a, b = self.cur, self.cur ^ 1
        _lib.check(lib.nbg_lif_forward_step_sparse(
            _ptr(xi), _ptr(w_rec), _ptr(self.idx[a]), _ptr(self.cnt[a]), _ptr(self.idx[b]), _ptr(self.cnt[b]),
            _ptr(v), _ptr(ref), _ptr(s_out), _ptr(u_rec), _ptr(m_rec), _ptr(vp_rec), _ptr(z), float(c), _ptr(alpha),
            _ptr(theta), ctypes.byref(p), B, N, st))
        self.cur = b


def _sparse_ok(p, N: int) -> bool:
    return not p.smooth and N <= 2048


_COEF = {}


def _coef_device(coef, device) -> torch.Tensor:
    """The readout coefficients on the device, made once per (values, device)
    so that a CUDA graph capture finds them already there."""
    key = (np.asarray(coef, np.float32).tobytes(), str(device))
    t = _COEF.get(key)
    if t is None:
        t = torch.tensor(np.asarray(coef, np.float32), device=device)
        _COEF[key] = t
    return t


# The recurrent product dI_{t+1} W_rec^T of the adjoint runs on the tensor
# cores (split BF16, nbg_adjoint_rec_grad) for B = 128 rows and N a multiple
# of 128 in spiking mode; its split-K partials are added by the next step.
TC_SPLIT = 8
# The segment's weight gradients S^T dI (spikes exact in BF16) and X^T dI
# (inputs split like dI) on the tensor cores as well when N (and C) are
# multiples of 256; split-K partials.
WGRAD_SPLIT = 4
WGRAD_IN_SPLIT = 16


def _tc_ok(p, B: int, N: int) -> bool:
    return not p.smooth and B == 128 and N % 128 == 0


# With N >= 512 the product and the adjoint step that consumes it are one
# launch per step (nbg_lif_adjoint_step_fused: an 8-CTA cluster per 128-row
# tile reduces its split-K partials through distributed shared memory); the
# same sums in the same order as the two-launch form.
FUSED_STEP = True


def _fused_ok(p, B: int, N: int) -> bool:
    return FUSED_STEP and _tc_ok(p, B, N) and N >= 512


# Largest state record (u, s, m, v_{t-1} of every step) a forward keeps by
# default instead of checkpoints.
RECORD_BUDGET_BYTES = 8 << 30


def record_bytes(T: int, B: int, N: int) -> int:
    """Bytes of the per-step record: u, v_{t-1} (FP32), m (uint8) for T steps
    and s (FP32) for T + 1 (s_{-1} = 0 first)."""
    return T * B * N * 9 + (T + 1) * B * N * 4


def _record_buffers(T, B, N, dev):
    """(U, S, M, VP): U[t] = u_t, S[t + 1] = s_t (S[0] = 0), M[t] = m_t,
    VP[t] = v_{t-1}."""
    S = torch.empty((T + 1, B, N), device=dev, dtype=torch.float32)
    S[0].zero_()
    return (torch.empty((T, B, N), device=dev, dtype=torch.float32), S,
            torch.empty((T, B, N), device=dev, dtype=torch.uint8),
            torch.empty((T, B, N), device=dev, dtype=torch.float32))


def _forward_body(lib, x, w_in, w_rec, w_out, alpha, theta, p, K, coef, ck_v, ck_ref, ck_s, z, out, rec=None):
    """Forward recurrence into caller-owned buffers: the checkpoints
    ck_*[segment] (state entering each K-step segment) or, with rec = (U, S,
    M, VP) from _record_buffers, every step's state the adjoint reads; the
    readout accumulator z and the output z W_out.  Launches only (no host
    sync), so it runs eagerly or under CUDA graph capture alike.  With binary
    spikes the recurrent product is the spike-driven gather-sum (one fused
    kernel per segment); with sigmoid spikes it is a GEMM."""
    T, B, C = x.shape
    N = w_rec.shape[0]
    st = _stream()
    v = torch.full((B, N), p.v_reset, device=x.device, dtype=torch.float32)
    ref = torch.zeros((B, N), device=x.device, dtype=torch.int32)
    sbuf = [torch.empty((B, N), device=x.device, dtype=torch.float32) for _ in range(2)]
    s_prev = sbuf[1]
    s_prev.zero_()
    z.zero_()
    sparse = _sparse_ok(p, N)
    lists = _SpikeLists(B, N, x.device) if sparse else None  # no spikes before step 0
    coef_dev = _coef_device(coef, x.device) if sparse else None
    I = torch.empty((B, N), device=x.device, dtype=torch.float32)
    for seg, t0 in enumerate(range(0, T, K)):
        t1 = min(T, t0 + K)
        if rec is None:
            ck_v[seg].copy_(v)
            ck_ref[seg].copy_(ref)
            ck_s[seg].copy_(s_prev)
        if sparse:  # the whole segment in one launch, inputs gathered in it
            if rec is None:
                s_prev = sbuf[seg & 1]
                lists.segment_gather(lib, x[t0:t1], w_in, w_rec, v, ref, None, s_prev, None, None, None, z,
                                     coef_dev[t0:t1], alpha, theta, p, t1 - t0, B, N, st)
            else:
                U, S, M, VP = rec
                lists.segment_gather(lib, x[t0:t1], w_in, w_rec, v, ref, S[t0 + 1], None, U[t0], M[t0], VP[t0], z,
                                     coef_dev[t0:t1], alpha, theta, p, t1 - t0, B, N, st)
            continue
        xi = torch.empty((t1 - t0, B, N), device=x.device, dtype=torch.float32)
        _gemm(lib, x[t0:t1], C, 1, w_in, N, 1, xi, (t1 - t0) * B, N, C, st)  # x W_in of the segment
        for t in range(t0, t1):
            if rec is None:
                s, u_t, m_t, vp_t = sbuf[t & 1], None, None, None
            else:
                s, u_t, m_t, vp_t = rec[1][t + 1], _ptr(rec[0][t]), _ptr(rec[2][t]), _ptr(rec[3][t])
            _gemm(lib, s_prev, N, 1, w_rec, N, 1, I, B, N, N, st)  # s_{t-1} W_rec, then + x_t W_in
            I.add_(xi[t - t0])
            _lib.check(lib.nbg_lif_forward_step(_ptr(I), _ptr(v), _ptr(ref), _ptr(s), u_t, m_t, vp_t, _ptr(z),
                                                float(coef[t]), _ptr(alpha), _ptr(theta), ctypes.byref(p), B, N, st))
            s_prev = s
    _readout(lib, z, w_out, out, st)


def _gemm(lib, a, a_rs, a_cs, b, b_rs, b_cs, out, M, N, K, st) -> None:
    """out (M x N, row-major) = A B with the engine's small deterministic
    product; element (r, c) of A at a[r * a_rs + c * a_cs], likewise B."""
    _lib.check(lib.nbg_small_gemm(_ptr(a), a_rs, a_cs, _ptr(b), b_rs, b_cs, _ptr(out), M, N, K, st))


def _readout(lib, z, w_out, out, st) -> None:
    """out = z W_out (B x N by N x O) with the engine's small deterministic
    product."""
    B, N = z.shape
    O = w_out.shape[1]
    _lib.check(lib.nbg_small_gemm(_ptr(z), N, 1, _ptr(w_out), O, 1, _ptr(out), B, O, N, st))


def _backward_body(lib, gy, x, w_in, w_rec, w_out, alpha, theta, z, ck_v, ck_ref, ck_s, p, K, coef, rec=None):
    """Adjoint sweep over the K-step segments in reverse: each segment's
    u_t, s_t, m_t, v_{t-1} from the forward's record (rec) or from a replay of
    the segment from its checkpoint, then the adjoint step in reverse time and
    the weight gradients (per segment, or once over the whole run when the
    state is recorded).  Returns the gradients of (W_in, W_rec, W_out, alpha,
    theta).  Launches only, like the forward body."""
    T, B, C = x.shape
    N = w_rec.shape[0]
    dev = x.device
    st = _stream()
    O = w_out.shape[1]
    g_read = torch.empty((B, N), device=dev, dtype=torch.float32)  # gy W_out^T
    g_w_out = torch.empty((N, O), device=dev, dtype=torch.float32)  # z^T gy
    _lib.check(lib.nbg_small_gemm(_ptr(gy), O, 1, _ptr(w_out), 1, O, _ptr(g_read), B, N, O, st))
    _lib.check(lib.nbg_small_gemm(_ptr(z), 1, N, _ptr(gy), O, 1, _ptr(g_w_out), N, O, B, st))
    g_w_in = torch.zeros_like(w_in)
    g_w_rec = torch.zeros_like(w_rec)
    lam_v = torch.zeros((B, N), device=dev, dtype=torch.float32)
    g_theta = torch.zeros((B, N), device=dev, dtype=torch.float32)
    g_alpha = torch.zeros((B, N), device=dev, dtype=torch.float32)
    g_ext = torch.empty((B, N), device=dev, dtype=torch.float32)
    I = torch.empty((B, N), device=dev, dtype=torch.float32)
    L_max = min(K, T)
    if rec is None:  # one segment's replay
        U = torch.empty((L_max, B, N), device=dev, dtype=torch.float32)
        S = torch.empty((L_max + 1, B, N), device=dev, dtype=torch.float32)  # S[0] = s_{t0-1}
        M = torch.empty((L_max, B, N), device=dev, dtype=torch.uint8)
        VP = torch.empty((L_max, B, N), device=dev, dtype=torch.float32)
    have_next = False
    sparse = _sparse_ok(p, N)
    lists = _SpikeLists(B, N, dev) if sparse and rec is None else None
    tc = _tc_ok(p, B, N)
    fused = _fused_ok(p, B, N)
    # the fused step writes dI^T for the weight gradients itself (no FP32 dI,
    # no transpose); the other forms keep dI in FP32
    dI = None if fused else torch.empty((L_max, B, N), device=dev, dtype=torch.float32)
    dI_next = None if fused else torch.empty((B, N), device=dev, dtype=torch.float32)
    if not tc:  # the weight-gradient products of a segment (CUDA cores)
        tmp_rec = torch.empty((N, N), device=dev, dtype=torch.float32)
        tmp_in = torch.empty((C, N), device=dev, dtype=torch.float32)
    if tc:
        w_hi = torch.empty(N * N, device=dev, dtype=torch.bfloat16)
        w_lo = torch.empty(N * N, device=dev, dtype=torch.bfloat16)
        # the split BF16 operand dI: two buffers in the fused form (a step
        # reads one while writing the other; the run's last step reads zeros),
        # else one
        d_hi = [torch.zeros(B * N, device=dev, dtype=torch.bfloat16) for _ in range(2 if fused else 1)]
        d_lo = [torch.zeros(B * N, device=dev, dtype=torch.bfloat16) for _ in range(2 if fused else 1)]
        split = min(TC_SPLIT, N // 64)
        g_parts = None if fused else torch.empty((split, B, N), device=dev, dtype=torch.float32)
        tc_err = torch.zeros(1, device=dev, dtype=torch.int32)
        _lib.check(lib.nbg_adjoint_rec_prepare(_ptr(w_rec), _ptr(w_hi), _ptr(w_lo), N, st))
    # weight gradients on the tensor cores: the product's column operand (S^T,
    # X^T) is padded with zero rows to a multiple of 256; with the state
    # recorded they run once, over every (step, row) pair of the run
    whole = fused and rec is not None
    if tc:
        kk_max = (T if whole else L_max) * B
        N256, C256 = -(-N // 256) * 256, -(-C // 256) * 256
        dT_hi = torch.empty(N * kk_max, device=dev, dtype=torch.bfloat16)
        dT_lo = torch.empty(N * kk_max, device=dev, dtype=torch.bfloat16)
        sT = torch.empty(N256 * kk_max, device=dev, dtype=torch.bfloat16)
        w_part = torch.empty(max(WGRAD_SPLIT * N256 * N, WGRAD_IN_SPLIT * C256 * N), device=dev,
                             dtype=torch.float32)
        xT_hi = torch.empty(C256 * kk_max, device=dev, dtype=torch.bfloat16)
        xT_lo = torch.empty(C256 * kk_max, device=dev, dtype=torch.bfloat16)

    def transposes(s_rows, x_rows, L):
        """S^T and X^T of L steps in the products' blocked BF16 layout."""
        _lib.check(lib.nbg_adjoint_blocked_t(_ptr(s_rows), L, B, N, N256, _ptr(sT), None, st))
        _lib.check(lib.nbg_adjoint_blocked_t(_ptr(x_rows), L, B, C, C256, _ptr(xT_hi), _ptr(xT_lo), st))

    def wgrad(L):
        """dW_rec += S^T dI and dW_in += X^T dI over L steps, dI^T in dT."""
        kk = L * B
        ws = min(WGRAD_SPLIT, kk // 64)
        _lib.check(lib.nbg_adjoint_wgrad(_ptr(dT_hi), _ptr(dT_lo), _ptr(sT), None, N, N256, kk, _ptr(w_part), ws,
                                         _ptr(tc_err), st))
        _lib.check(lib.nbg_adjoint_reduce_add(_ptr(g_w_rec), _ptr(w_part), ws, N * N, N256 * N, st))
        ws = min(WGRAD_IN_SPLIT, kk // 64)
        _lib.check(lib.nbg_adjoint_wgrad(_ptr(dT_hi), _ptr(dT_lo), _ptr(xT_hi), _ptr(xT_lo), N, C256, kk,
                                         _ptr(w_part), ws, _ptr(tc_err), st))
        _lib.check(lib.nbg_adjoint_reduce_add(_ptr(g_w_in), _ptr(w_part), ws, C * N, C256 * N, st))


    segments = list(enumerate(range(0, T, K)))
    for seg, t0 in reversed(segments):
        t1 = min(T, t0 + K)
        L = t1 - t0
        if rec is not None:  # the forward's record of the segment
            U, S, M, VP = rec[0][t0:t1], rec[1][t0:t1 + 1], rec[2][t0:t1], rec[3][t0:t1]
        else:  # replay the segment from its checkpoint, recording u, m, v_{t-1} and s
            v, ref = ck_v[seg].clone(), ck_ref[seg].clone()
            S[0].copy_(ck_s[seg])
            if sparse:  # in one launch
                lists.load(lib, S[0], B, N, st)
                lists.segment_gather(lib, x[t0:t1], w_in, w_rec, v, ref, S[1], None, U, M, VP, None, None, alpha,
                                     theta, p, L, B, N, st)
            else:
                xi = torch.empty((L, B, N), device=dev, dtype=torch.float32)
                _gemm(lib, x[t0:t1], C, 1, w_in, N, 1, xi, L * B, N, C, st)
                for k in range(L):
                    _gemm(lib, S[k], N, 1, w_rec, N, 1, I, B, N, N, st)
                    I.add_(xi[k])
                    _lib.check(lib.nbg_lif_forward_step(_ptr(I), _ptr(v), _ptr(ref), _ptr(S[k + 1]), _ptr(U[k]),
                                                        _ptr(M[k]), _ptr(VP[k]), None, 0.0, _ptr(alpha),
                                                        _ptr(theta), ctypes.byref(p), B, N, st))
        for k in reversed(range(L)):
            t = t0 + k
            if fused:  # dI_{t+1} W_rec^T (zero at the run's last step) and step t, one launch
                cur, nxt = t & 1, (t + 1) & 1
                k_off, k_cols = (t * B, T * B) if whole else (k * B, L * B)
                _lib.check(lib.nbg_lif_adjoint_step_fused(
                    _ptr(w_hi), _ptr(w_lo), _ptr(d_hi[nxt]), _ptr(d_lo[nxt]), _ptr(d_hi[cur]), _ptr(d_lo[cur]),
                    _ptr(g_read), float(coef[t]), _ptr(U[k]), _ptr(S[k + 1]), _ptr(M[k]), _ptr(VP[k]),
                    _ptr(lam_v), None, _ptr(g_theta), _ptr(g_alpha), _ptr(alpha), _ptr(theta), ctypes.byref(p), B,
                    N, _ptr(dT_hi), _ptr(dT_lo), k_off, k_cols, _ptr(tc_err), st))
                continue
            if tc:  # g_parts holds dI_{t+1} W_rec^T from the previous iteration
                _lib.check(lib.nbg_lif_adjoint_step_split(
                    _ptr(g_parts) if have_next else None, split, _ptr(g_read), float(coef[t]), _ptr(U[k]),
                    _ptr(S[k + 1]), _ptr(M[k]), _ptr(VP[k]), _ptr(lam_v), _ptr(dI[k]), _ptr(d_hi[0]), _ptr(d_lo[0]),
                    _ptr(g_theta), _ptr(g_alpha), _ptr(alpha), _ptr(theta), ctypes.byref(p), B, N, st))
                _lib.check(lib.nbg_adjoint_rec_grad(_ptr(w_hi), _ptr(w_lo), _ptr(d_hi[0]), _ptr(d_lo[0]),
                                                    _ptr(g_parts), split, B, N, _ptr(tc_err), st))
                have_next = True
                continue
            ge = None
            if have_next:  # dL/ds_t from the recurrent path: dI_{t+1} W_rec^T
                _gemm(lib, dI_next if k == L - 1 else dI[k + 1], N, 1, w_rec, 1, N, g_ext, B, N, N, st)
                ge = g_ext
            _lib.check(lib.nbg_lif_adjoint_step(_ptr(ge), _ptr(g_read), float(coef[t]), _ptr(U[k]),
                                                _ptr(S[k + 1]), _ptr(M[k]), _ptr(VP[k]), _ptr(lam_v),
                                                _ptr(dI[k]), _ptr(g_theta), _ptr(g_alpha), _ptr(alpha),
                                                _ptr(theta), ctypes.byref(p), B, N, st))
            have_next = True
        if whole:
            continue
        if tc:
            if not fused:  # dI^T from the FP32 dI
                _lib.check(lib.nbg_adjoint_blocked_t(_ptr(dI), L, B, N, N, _ptr(dT_hi), _ptr(dT_lo), st))
            transposes(S, x[t0:t1], L)
            wgrad(L)
        else:
            # S^T dI and X^T dI over the segment's (step, row) pairs
            _gemm(lib, S, 1, N, dI, N, 1, tmp_rec, N, N, L * B, st)
            g_w_rec.add_(tmp_rec)
            _gemm(lib, x[t0:t1], 1, C, dI, N, 1, tmp_in, C, N, L * B, st)
            g_w_in.add_(tmp_in)
        if dI_next is not None:
            dI_next.copy_(dI[0])
    if whole:  # the whole run's weight gradients at once
        transposes(rec[1], x, T)
        wgrad(T)
    return g_w_in, g_w_rec, g_w_out, g_alpha.sum(0), g_theta.sum(0), (tc_err if tc else None)


def _check_tc(err) -> None:
    """Raise if a bounded wait of the tensor-core recurrent product gave up."""
    if err is not None and int(err.item()) != 0:
        raise RuntimeError("nbg_adjoint_rec_grad: a tensor-core wait timed out; the gradients are invalid")


class _GraphPlan:
    """The forward and the backward of one shape, each captured once as a CUDA
    graph over static buffers and replayed on later calls (the recurrence is
    thousands of small launches; replay removes their host cost).  Inputs are
    copied into the static buffers before a replay and results cloned out, so
    callers never alias graph memory.  Keyed by shape, checkpoint interval,
    record mode, readout coefficients, LIF parameters and the parameters'
    storage; in-place optimiser updates keep the storage, so one plan serves a
    training run."""

    def __init__(self, x, w_in, w_rec, w_out, alpha, theta, p, K, coef, record):
        T, B, C = x.shape
        N = w_rec.shape[0]
        nseg = (T + K - 1) // K
        dev = x.device
        self.params = (w_in, w_rec, w_out, alpha, theta)
        self.p, self.K, self.coef = p, K, coef
        self.x = torch.empty_like(x)
        self.rec = _record_buffers(T, B, N, dev) if record else None
        ck = 0 if record else nseg
        self.ck_v = torch.empty((ck, B, N), device=dev, dtype=torch.float32)
        self.ck_ref = torch.empty((ck, B, N), device=dev, dtype=torch.int32)
        self.ck_s = torch.empty((ck, B, N), device=dev, dtype=torch.float32)
        self.z = torch.empty((B, N), device=dev, dtype=torch.float32)
        self.out = torch.empty((B, w_out.shape[1]), device=dev, dtype=torch.float32)
        self.gy = torch.empty((B, w_out.shape[1]), device=dev, dtype=torch.float32)
        self.fwd = self.bwd = None
        self.grads = None
        self.owner = None  # the forward whose x and checkpoints (or record) the buffers hold

    @staticmethod
    def _capture(fn):
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):  # warm-up: allocations and library state exist before capture
            out = fn()
        torch.cuda.current_stream().wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            out = fn()
        return g, out

    def forward(self, x):
        lib = _bind()
        self.x.copy_(x)
        if self.fwd is None:
            w_in, w_rec, w_out, alpha, theta = self.params
            self.fwd, _ = self._capture(lambda: _forward_body(
                lib, self.x, w_in, w_rec, w_out, alpha, theta, self.p, self.K, self.coef, self.ck_v, self.ck_ref,
                self.ck_s, self.z, self.out, self.rec))
        self.fwd.replay()
        self.owner = object()
        return self.owner

    def backward(self, owner, gy, x, saved):
        lib = _bind()
        if owner is not self.owner:  # another forward ran since: restore this one's inputs
            self.x.copy_(x)
            if self.rec is not None:  # run its forward again: the same launches give the same record
                self.fwd.replay()
            else:
                self.ck_v.copy_(saved[0])
                self.ck_ref.copy_(saved[1])
                self.ck_s.copy_(saved[2])
                self.z.copy_(saved[3])
            self.owner = owner
        self.gy.copy_(gy)
        if self.bwd is None:
            w_in, w_rec, w_out, alpha, theta = self.params
            self.bwd, self.grads = self._capture(lambda: _backward_body(
                lib, self.gy, self.x, w_in, w_rec, w_out, alpha, theta, self.z, self.ck_v, self.ck_ref, self.ck_s,
                self.p, self.K, self.coef, self.rec))
        self.bwd.replay()
        _check_tc(self.grads[5])
        return tuple(g.clone() for g in self.grads[:5])


class _Recurrence(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, w_in, w_rec, w_out, alpha, theta, cfg):
        lib = _bind()
        T, B, C = x.shape
        N = w_rec.shape[0]
        K = cfg["checkpoint"]
        nseg = (T + K - 1) // K
        plan = cfg.get("plan")
        ctx.cfg = cfg
        if plan is not None:
            ctx.owner = plan.forward(x)
            z = plan.z.clone()
            keep = cfg["needs_grad"] and plan.rec is None
            ctx.ck = (plan.ck_v.clone(), plan.ck_ref.clone(), plan.ck_s.clone()) if keep else ()
            ctx.rec = None
            ctx.save_for_backward(x, w_in, w_rec, w_out, alpha, theta, z)
            return plan.out.clone()
        record = cfg["record"]
        ck = 0 if record else nseg
        ck_v = torch.empty((ck, B, N), device=x.device, dtype=torch.float32)
        ck_ref = torch.empty((ck, B, N), device=x.device, dtype=torch.int32)
        ck_s = torch.empty((ck, B, N), device=x.device, dtype=torch.float32)
        rec = _record_buffers(T, B, N, x.device) if record else None
        z = torch.empty((B, N), device=x.device, dtype=torch.float32)
        out = torch.empty((B, w_out.shape[1]), device=x.device, dtype=torch.float32)
        _forward_body(lib, x, w_in, w_rec, w_out, alpha, theta, cfg["params"], K, cfg["coef"], ck_v, ck_ref, ck_s,
                      z, out, rec)
        ctx.ck = (ck_v, ck_ref, ck_s)
        ctx.rec = rec if cfg["needs_grad"] else None
        ctx.save_for_backward(x, w_in, w_rec, w_out, alpha, theta, z)
        return out

    @staticmethod
    def backward(ctx, gy):
        x, w_in, w_rec, w_out, alpha, theta, z = ctx.saved_tensors
        cfg = ctx.cfg
        gy = gy.contiguous()
        plan = cfg.get("plan")
        if plan is not None:
            grads = plan.backward(ctx.owner, gy, x, ctx.ck + (z,))
        else:
            *grads, err = _backward_body(_bind(), gy, x, w_in, w_rec, w_out, alpha, theta, z, *ctx.ck, cfg["params"],
                                         cfg["checkpoint"], cfg["coef"], ctx.rec)
            _check_tc(err)
        return (None, *grads, None)


class RecurrentLIF(torch.nn.Module):
    """n_in Poisson channels -> n_rec recurrent voltage-jump LIF -> n_out leaky
    readout; ``forward(x)`` returns the time-averaged readout (B x n_out).

    ``checkpoint``: the segment length of the launches (and of the replay);
    ``record``: keep every step's state for the backward (True), replay
    segments from checkpoints (False), or record while ``record_bytes`` fits
    in RECORD_BUDGET_BYTES (None)."""

    def __init__(self, n_in: int = 256, n_rec: int = 1024, n_out: int = 10, *, dt: float = 1.0, tau: float = 20.0,
                 v_rest: float = -65.0, v_reset: float = -65.0, v_th: float = -50.0, t_ref_ms: float = 2.0,
                 tau_out: float = 20.0, slope: float = 10.0, smooth: bool = False, checkpoint: int = 100,
                 record: bool | None = None, weight_scale: float = 1.0, seed: int = 5, device: str = "cuda",
                 use_graphs: bool = True):
        super().__init__()
        g = torch.Generator().manual_seed(seed)
        init = lambda *shape: (torch.randn(*shape, generator=g, dtype=torch.float64) * weight_scale /
                               math.sqrt(shape[0])).float()
        self.w_in = torch.nn.Parameter(init(n_in, n_rec).to(device))
        self.w_rec = torch.nn.Parameter(init(n_rec, n_rec).to(device))
        self.w_out = torch.nn.Parameter(init(n_rec, n_out).to(device))
        self.alpha = torch.nn.Parameter(torch.full((n_rec,), dt / tau, device=device))
        self.theta = torch.nn.Parameter(torch.full((n_rec,), v_th, device=device))
        self.params = GradParams(v_rest, v_reset, slope, int(round(t_ref_ms / dt)), int(bool(smooth)))
        self.dt, self.tau_out, self.checkpoint = dt, tau_out, int(checkpoint)
        self.record = record
        self.use_graphs = bool(use_graphs)
        self._plans = {}

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        T = x.shape[0]
        a_out = math.exp(-self.dt / self.tau_out)
        coef = readout_coefficients(T, a_out)
        x = x.contiguous()
        record = self.record
        if record is None:
            record = record_bytes(T, x.shape[1], self.w_rec.shape[0]) <= RECORD_BUDGET_BYTES
        cfg = {"params": self.params, "checkpoint": self.checkpoint, "coef": coef, "record": bool(record),
               "needs_grad": torch.is_grad_enabled() and any(q.requires_grad for q in self.parameters())}
        if self.use_graphs:
            key = (tuple(x.shape), str(x.device), self.checkpoint, bool(record), coef.tobytes(), bytes(self.params),
                   tuple(q.data_ptr() for q in self.parameters()))
            plan = self._plans.get(key)
            if plan is None:
                self._plans.clear()
                plan = self._plans[key] = _GraphPlan(x, self.w_in, self.w_rec, self.w_out, self.alpha, self.theta,
                                                     self.params, self.checkpoint, coef, bool(record))
            cfg["plan"] = plan
        return _Recurrence.apply(x, self.w_in, self.w_rec, self.w_out, self.alpha, self.theta, cfg)


def reference_forward(x, w_in, w_rec, w_out, alpha, theta, *, v_rest=-65.0, v_reset=-65.0, slope=10.0, t_ref=2,
                      smooth=False, dt=1.0, tau_out=20.0):
    """The same discretised dynamics in plain torch ops (any dtype/device),
    differentiated by autograd; the spiking mode's Heaviside uses the same
    fast-sigmoid surrogate in its backward."""

    class Spike(torch.autograd.Function):
        @staticmethod
        def forward(ctx, d):
            ctx.save_for_backward(d)
            return (d > 0).to(d.dtype)

        @staticmethod
        def backward(ctx, g):
            (d,) = ctx.saved_tensors
            return g / (1.0 + slope * d.abs()) ** 2

    T, B, _ = x.shape
    N = w_rec.shape[0]
    v = torch.full((B, N), v_reset, dtype=x.dtype, device=x.device)
    ref = torch.zeros((B, N), dtype=torch.int64, device=x.device)
    s = torch.zeros((B, N), dtype=x.dtype, device=x.device)
    a_out = math.exp(-dt / tau_out)
    coef = torch.as_tensor(readout_coefficients(T, a_out).astype(np.float64), dtype=x.dtype, device=x.device)
    z = torch.zeros((B, N), dtype=x.dtype, device=x.device)
    for t in range(T):
        I = x[t] @ w_in + s @ w_rec
        m = ref == 0 if not smooth else torch.ones_like(ref, dtype=torch.bool)
        u = torch.where(m, v + alpha * (v_rest - v) + I, torch.full_like(v, v_reset))
        s = torch.sigmoid(slope * (u - theta)) if smooth else Spike.apply(u - theta)
        v = u - s * (u - v_reset)
        if not smooth:
            ref = torch.where(s > 0, torch.full_like(ref, t_ref), (ref - 1).clamp(min=0))
        z = z + coef[t] * s
    return z @ w_out
