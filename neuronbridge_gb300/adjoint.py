"""Differentiable recurrent LIF network with a hand-written adjoint.

``RecurrentLIF`` runs T steps of the voltage-jump LIF recurrence of
``include/nbg_adjoint.h`` for a batch of B input sequences and returns the
time-averaged leaky readout.  Its backward is not autograd: the forward saves
the network state every ``checkpoint`` steps, and the backward replays each
segment from its checkpoint (recording u_t, s_t, m_t, v_{t-1}) and runs the
fused adjoint kernel in reverse time.  Dense products go to cuBLAS through
torch (x W_in for a whole segment at once, s W_rec and dI W_rec^T per step,
and the weight gradients as one GEMM per segment); all elementwise work of a
step is one CUDA kernel each way.

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


class _Recurrence(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, w_in, w_rec, w_out, alpha, theta, cfg):
        lib = _bind()
        T, B, C = x.shape
        N = w_rec.shape[0]
        p = cfg["params"]
        K = cfg["checkpoint"]
        coef = cfg["coef"]
        st = _stream()
        v = torch.full((B, N), p.v_reset, device=x.device, dtype=torch.float32)
        ref = torch.zeros((B, N), device=x.device, dtype=torch.int32)
        s_prev = torch.zeros((B, N), device=x.device, dtype=torch.float32)
        z = torch.zeros((B, N), device=x.device, dtype=torch.float32)
        ckpts = []
        sbuf = [torch.empty((B, N), device=x.device, dtype=torch.float32) for _ in range(2)]
        I = torch.empty((B, N), device=x.device, dtype=torch.float32)
        for t0 in range(0, T, K):
            t1 = min(T, t0 + K)
            ckpts.append((t0, t1, v.clone(), ref.clone(), s_prev.clone()))
            xi = (x[t0:t1].reshape(-1, C) @ w_in).reshape(t1 - t0, B, N)
            for t in range(t0, t1):
                torch.addmm(xi[t - t0], s_prev, w_rec, out=I)
                s = sbuf[t & 1]
                _lib.check(lib.nbg_lif_forward_step(_ptr(I), _ptr(v), _ptr(ref), _ptr(s), None, None, None, _ptr(z),
                                                    float(coef[t]), _ptr(alpha), _ptr(theta), ctypes.byref(p), B, N,
                                                    st))
                s_prev = s
        ctx.save_for_backward(x, w_in, w_rec, w_out, alpha, theta, z)
        ctx.cfg = cfg
        ctx.ckpts = ckpts
        return z @ w_out

    @staticmethod
    def backward(ctx, gy):
        lib = _bind()
        x, w_in, w_rec, w_out, alpha, theta, z = ctx.saved_tensors
        cfg = ctx.cfg
        p = cfg["params"]
        coef = cfg["coef"]
        T, B, C = x.shape
        N = w_rec.shape[0]
        st = _stream()
        gy = gy.contiguous()
        g_read = (gy @ w_out.t()).contiguous()
        g_w_out = z.t() @ gy
        g_w_in = torch.zeros_like(w_in)
        g_w_rec = torch.zeros_like(w_rec)
        lam_v = torch.zeros((B, N), device=x.device, dtype=torch.float32)
        g_theta = torch.zeros((B, N), device=x.device, dtype=torch.float32)
        g_alpha = torch.zeros((B, N), device=x.device, dtype=torch.float32)
        g_ext = torch.empty((B, N), device=x.device, dtype=torch.float32)
        I = torch.empty((B, N), device=x.device, dtype=torch.float32)
        dI_next = None
        for (t0, t1, v0, ref0, s0) in reversed(ctx.ckpts):
            L = t1 - t0
            v, ref = v0.clone(), ref0.clone()
            U = torch.empty((L, B, N), device=x.device, dtype=torch.float32)
            S = torch.empty((L + 1, B, N), device=x.device, dtype=torch.float32)  # S[0] = s_{t0-1}
            M = torch.empty((L, B, N), device=x.device, dtype=torch.uint8)
            VP = torch.empty((L, B, N), device=x.device, dtype=torch.float32)
            S[0].copy_(s0)
            xi = (x[t0:t1].reshape(-1, C) @ w_in).reshape(L, B, N)
            for k in range(L):  # recompute the segment, recording what the adjoint needs
                torch.addmm(xi[k], S[k], w_rec, out=I)
                _lib.check(lib.nbg_lif_forward_step(_ptr(I), _ptr(v), _ptr(ref), _ptr(S[k + 1]), _ptr(U[k]),
                                                    _ptr(M[k]), _ptr(VP[k]), None, 0.0, _ptr(alpha), _ptr(theta),
                                                    ctypes.byref(p), B, N, st))
            dI = torch.empty((L, B, N), device=x.device, dtype=torch.float32)
            for k in reversed(range(L)):
                t = t0 + k
                ge = None
                if dI_next is not None:
                    torch.mm(dI_next, w_rec.t(), out=g_ext)
                    ge = g_ext
                _lib.check(lib.nbg_lif_adjoint_step(_ptr(ge), _ptr(g_read), float(coef[t]), _ptr(U[k]),
                                                    _ptr(S[k + 1]), _ptr(M[k]), _ptr(VP[k]), _ptr(lam_v),
                                                    _ptr(dI[k]), _ptr(g_theta), _ptr(g_alpha), _ptr(alpha),
                                                    _ptr(theta), ctypes.byref(p), B, N, st))
                dI_next = dI[k]
            g_w_rec += S[:L].reshape(-1, N).t() @ dI.reshape(-1, N)
            g_w_in += x[t0:t1].reshape(-1, C).t() @ dI.reshape(-1, N)
            dI_next = dI[0].clone()
        return None, g_w_in, g_w_rec, g_w_out, g_alpha.sum(0), g_theta.sum(0), None


class RecurrentLIF(torch.nn.Module):
    """n_in Poisson channels -> n_rec recurrent voltage-jump LIF -> n_out leaky
    readout; ``forward(x)`` returns the time-averaged readout (B x n_out)."""

    def __init__(self, n_in: int = 256, n_rec: int = 1024, n_out: int = 10, *, dt: float = 1.0, tau: float = 20.0,
                 v_rest: float = -65.0, v_reset: float = -65.0, v_th: float = -50.0, t_ref_ms: float = 2.0,
                 tau_out: float = 20.0, slope: float = 10.0, smooth: bool = False, checkpoint: int = 100,
                 weight_scale: float = 1.0, seed: int = 5, device: str = "cuda"):
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

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        T = x.shape[0]
        a_out = math.exp(-self.dt / self.tau_out)
        cfg = {"params": self.params, "checkpoint": self.checkpoint, "coef": readout_coefficients(T, a_out)}
        return _Recurrence.apply(x.contiguous(), self.w_in, self.w_rec, self.w_out, self.alpha, self.theta, cfg)


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
