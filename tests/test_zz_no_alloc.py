"""The allocation-free loss entry point (gbnde_loss_noalloc) against the
context-based one (gbnde_loss_device), through the C ABI, on two calls in a
row with different targets. The file name sorts last so that a run stopping
at its first failure has already run every other test; it also passes alone
in a fresh process."""
import ctypes as C

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA GPU")]


def test_loss_noalloc_matches_loss_device_twice():
    import torch

    import gbnde
    from gbnde import _lib

    lib = gbnde.load(build_if_missing=True)
    S, H, B = 8, 32, 300
    rng = np.random.default_rng(11)
    model = gbnde.Chain(gbnde.Dense(S, H, "tanh"), gbnde.Dense(H, S))
    p = model.init_params(rng)
    ts = np.linspace(0.0, 1.0, 5)
    node = gbnde.NeuralODE(model, (0.0, 1.0), gbnde.Tsit5(), saveat=ts, abstol=1e-6, reltol=1e-4)
    s = node.solver
    dev = torch.device("cuda", 0)
    u0 = torch.from_numpy(np.ascontiguousarray(rng.standard_normal((B, S)).astype(np.float32))).to(dev)
    us = torch.empty((len(ts), B, S), dtype=torch.float32, device=dev)
    s.set_params(p)
    torch.cuda.synchronize()
    st = s.forward_device(u0, us, node.desc(), S, B)
    assert st.retcode == 0
    n = us.numel()
    stream = torch.cuda.current_stream(dev).cuda_stream
    for call in range(2):
        for kind in (0, 1):
            tg = torch.from_numpy(rng.standard_normal((len(ts), B, S)).astype(np.float32)).to(dev)
            dl_ref = torch.empty_like(us)
            dl_new = torch.full_like(us, float("nan"))
            torch.cuda.synchronize()
            ref = s.loss_device(us, tg, kind, dl_ref)
            out = C.c_double(float("nan"))
            rc = lib.gbnde_loss_noalloc(us.data_ptr(), tg.data_ptr(), n, kind, dl_new.data_ptr(),
                                        C.byref(out), stream)
            assert rc == 0, (call, kind, rc)
            torch.cuda.synchronize()
            # the allocation-free kernel sums every square in FP64, loss_device in
            # compensated FP32 partial sums: about 1e-9 relative apart
            assert abs(out.value - ref) <= 1e-8 * abs(ref), (call, kind, out.value, ref)
            assert torch.equal(dl_new, dl_ref)
    # sizes beyond the fixed scratch are refused, not truncated -- also those
    # that a signed comparison would see as negative
    out = C.c_double()
    for big in (4096 * 65536 + 1, 2**63 + 5, 2**64 - 1):
        assert lib.gbnde_loss_noalloc(us.data_ptr(), us.data_ptr(), C.c_size_t(big), 0, us.data_ptr(),
                                      C.byref(out), stream) == _lib.ERR_UNSUPPORTED, big
