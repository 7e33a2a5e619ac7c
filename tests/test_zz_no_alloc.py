"""kura_integrate_volcano_noalloc: the integration entry point that allocates nothing.

It serves callers that cannot call cudaMalloc, for example code inside a framework
that owns the device allocator.  They pass their own device buffers, and every scratch
buffer comes from a static device array inside libkura.  This test calls it twice in
a row through the C ABI, with buffers the test allocates through torch as such a
caller would hold them.  Both calls must agree with the handle API (kura_create /
kura_run) within the parity tolerances of the other tests: 1e-4 on r, and 1e-4 rad
plus one float32 ulp on the phases.  The file sorts last, so a run that stops at the
first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from helpers import normal_inputs

pytestmark = pytest.mark.gpu


def _entry(native):
    f = native.lib().kura_integrate_volcano_noalloc
    f.restype = ctypes.c_int32
    f.argtypes = [ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_float),
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                  ctypes.c_double, ctypes.c_double, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]
    return f


# (batch, k, side stream): the batch-1 and batch-8 kernels, the rank-8 and rank-32 factor
# caches, and a caller's own stream next to the legacy default stream
CASES = [(3, 5, False), (1, 5, True), (2, 20, True)]


@pytest.mark.parametrize("batch,k,side_stream", CASES)
def test_noalloc_matches_handle_api_twice(native, batch, k, side_stream):
    import torch

    n, seed, t1, dt, h0 = 3000, 7, 6.0, 0.5, 0.005
    cs = [1.5, 3.0, 4.5][:batch]
    B = len(cs)
    th, om = normal_inputs(n, 19)
    thetas = [th, (th + 0.3).astype(np.float32), (th * 0.5).astype(np.float32)][:B]

    net = native.Network(n, k=k, coupling=native.COUPLING_VOLCANO, batch=B, seed=seed, dense_level=0)
    net.set_frequencies(om)
    for b in range(B):
        net.set_coupling(b, cs[b])
        net.set_state(b, thetas[b], 0.0, h0)
    net.set_horizon(t1, dt, True)
    net.run()
    ref_r = [net.order(b) for b in range(B)]
    ref_th = [net.state(b)[0] for b in range(B)]
    ref_acc = net.stats()["accepted"]
    # the final phases read into a caller's pinned buffer are the same values
    buf = torch.empty(n, dtype=torch.float32).pin_memory().numpy()
    got = net.state(B - 1, out=buf)[0]
    assert got is buf and np.array_equal(buf, ref_th[B - 1])
    net.close()

    f = _entry(native)
    cap = 64
    c_arr = (ctypes.c_float * B)(*cs)
    om_d = torch.from_numpy(om).cuda()
    stream = torch.cuda.Stream() if side_stream else None
    for call in range(2):
        th_d = torch.from_numpy(np.stack(thetas)).cuda().contiguous()
        r_d = torch.full((B, cap), -1.0, dtype=torch.float32, device="cuda")
        acc = ctypes.c_int64(0)
        torch.cuda.synchronize()
        rc = f(n, k, B, seed, c_arr, om_d.data_ptr(), th_d.data_ptr(), t1, dt, h0, 1e-6, 0.0, 0,
               ctypes.c_void_p(stream.cuda_stream) if stream is not None else None,
               r_d.data_ptr(), cap, ctypes.byref(acc))
        assert rc == 0, native.lib().kura_last_error().decode()
        assert torch.cuda.current_device() == 0
        r = r_d.cpu().numpy()
        fin = th_d.cpu().numpy()
        assert acc.value == ref_acc
        for b in range(B):
            m = ref_r[b].size
            assert m == int(t1 / dt) + 1
            assert np.max(np.abs(r[b, :m] - ref_r[b])) < 1e-4, (call, b)
            assert np.all(r[b, m:] == -1.0)
            ulp = np.spacing(np.abs(ref_th[b])).astype(np.float64)
            assert np.all(np.abs(fin[b].astype(np.float64) - ref_th[b]) <= 1e-4 + ulp), (call, b)


def test_noalloc_rejects_sizes_beyond_its_scratch(native):
    import torch

    f = _entry(native)
    om_d = torch.zeros(70000, device="cuda")
    th_d = torch.zeros(70000, device="cuda")
    r_d = torch.zeros(16, device="cuda")
    c_arr = (ctypes.c_float * 1)(1.0)
    rc = f(70000, 5, 1, 1, c_arr, om_d.data_ptr(), th_d.data_ptr(), 1.0, 1.0, 0.01, 1e-6, 0.0, 0, None,
           r_d.data_ptr(), 16, None)
    assert rc == -1 and "65536" in native.lib().kura_last_error().decode()
    rc = f(1000, 5, 1, 1, c_arr, om_d.data_ptr(), th_d.data_ptr(), 100.0, 1.0, 0.01, 1e-6, 0.0, 0, None,
           r_d.data_ptr(), 16, None)
    assert rc == -1 and "order_cap" in native.lib().kura_last_error().decode()


def test_noalloc_rejects_non_finite_or_oversized_horizons(native):
    """Each of these returns before any device work: the checks are on the host."""
    import torch

    f = _entry(native)
    om_d = torch.zeros(100, device="cuda")
    th_d = torch.zeros(100, device="cuda")
    r_d = torch.zeros(16, device="cuda")
    c_arr = (ctypes.c_float * 1)(1.0)
    nan, inf = float("nan"), float("inf")
    bad = [(nan, 1.0, 0.01, 1e-6, 0.0), (inf, 1.0, 0.01, 1e-6, 0.0), (1e30, 1e-30, 0.01, 1e-6, 0.0),
           (1e12, 1.0, 0.01, 1e-6, 0.0), (1.0, 1.0, nan, 1e-6, 0.0), (1.0, 1.0, 0.01, 1e-6, nan),
           (1.0, nan, 0.01, 1e-6, 0.0), (-1.0, 1.0, 0.01, 1e-6, 0.0)]
    for t1, dt, h0, atol, rtol in bad:
        rc = f(100, 5, 1, 1, c_arr, om_d.data_ptr(), th_d.data_ptr(), t1, dt, h0, atol, rtol, 0, None,
               r_d.data_ptr(), 16, None)
        assert rc == -1, (t1, dt, h0, atol, rtol)
