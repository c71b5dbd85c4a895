"""The delivery entry point that allocates nothing, for callers that cannot
call cudaMalloc (a host that owns all device memory, a real-time control
loop, code inside a global-mode stream capture).

It is checked through the C ABI against the allocating entry point
(nbg_dense_deliver of an engine on the mma.sync split-BF16 path) on the same
weights and spikes, on two calls in a row, within the split-BF16 tolerance the
dense tests use (2e-5 absolute; both run the same kernel and summation order,
so they agree exactly).  This
file is collected last, and the test also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPLIT_ABS_TOL = 2e-5


def _bind(lib):
    fn = lib.nbg_dense_deliver_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int, ctypes.c_void_p]
    return fn


def test_noalloc_delivery_matches_allocating_entry_point():
    import torch

    import neuronbridge_gb300 as nb
    from neuronbridge_gb300 import NeuronLayer
    from neuronbridge_gb300.dense import DensePopulations, dense_weights
    from neuronbridge_gb300.workloads import LIF_PARAMS

    lib = nb.load()
    noalloc = _bind(lib)
    n = 1024
    w = dense_weights(n, seed=4)
    eng = DensePopulations(w, NeuronLayer("TimeDrivenLIF_Voltage_jump", 1, parameters=dict(LIF_PARAMS)),
                           precision="split_bf16_sync")
    wt = torch.from_numpy(w).cuda()
    w_hi = wt.to(torch.bfloat16)
    w_lo = (wt - w_hi.float()).to(torch.bfloat16)
    w_hi_t, w_lo_t = w_hi.t().contiguous(), w_lo.t().contiguous()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(7)
    for _ in range(2):  # two calls in a row share the scratch array
        s = (rng.random((64, n)) < 0.03).astype(np.uint8)
        expected = eng.deliver(s)
        s_dev = torch.from_numpy(s).cuda().to(torch.bfloat16)
        out = torch.full((64, n), float("nan"), device="cuda")
        st = noalloc(w_hi_t.data_ptr(), w_lo_t.data_ptr(), s_dev.data_ptr(), out.data_ptr(), n, stream)
        assert st == 0, lib.nbg_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.abs(got - expected).max() <= SPLIT_ABS_TOL

    # sizes beyond the stated maximum are refused, nothing is launched
    big = 8192 + 128
    st = noalloc(w_hi_t.data_ptr(), w_lo_t.data_ptr(), s_dev.data_ptr(), out.data_ptr(), big, stream)
    assert st == 1 and b"no-allocation limit" in lib.nbg_last_error()

    # an input that does not start on a 16-byte boundary (an offset view) is
    # refused before any launch
    st = noalloc(w_hi_t.data_ptr() + 2, w_lo_t.data_ptr(), s_dev.data_ptr(), out.data_ptr(), n, stream)
    assert st == 1 and b"16-byte aligned" in lib.nbg_last_error()
    st = noalloc(w_hi_t.data_ptr(), w_lo_t.data_ptr(), s_dev.data_ptr() + 8, out.data_ptr(), n, stream)
    assert st == 1 and b"16-byte aligned" in lib.nbg_last_error()
