"""pd_compute_velocity_noalloc: the entry point for callers that cannot call
cudaMalloc (a host application whose own pool owns all device memory, or a
latency-critical loop where an allocation would synchronise the device).

The caller owns every buffer; the test allocates them with torch (the caller's
pool here) and checks, over two calls in a row, that the results equal the
existing host-buffer entry point pd_compute_velocity on the same inputs --
bit for bit, the tolerance of every FP64 test here.  This file is collected
last on purpose, and also passes when run alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest


def _noalloc(pdg, n, bufs, params, stream=None):
    L = pdg.native.lib()
    err = ctypes.create_string_buffer(256)
    rc = L.pd_compute_velocity_noalloc(
        n, *(ctypes.c_void_p(b.data_ptr() if b is not None else 0) for b in bufs), ctypes.byref(params),
        stream, err, 256)
    return rc, err.value.decode()


def test_noalloc_rejects_sizes_beyond_the_maximum(pdg):
    L = pdg.native.lib()
    err = ctypes.create_string_buffer(256)
    p = pdg.default_params()
    big = pdg.native.lib().pd_compute_velocity_noalloc  # checked before any device work
    rc = big(70000, None, None, None, None, None, None, None, None, ctypes.byref(p), None, err, 256)
    assert rc == -4 and b"PD_NOALLOC_MAX_PARTICLES" in err.value
    assert L.pd_compute_velocity_noalloc(-1, None, None, None, None, None, None, None, None, ctypes.byref(p), None,
                                         None, 0) == -4


@pytest.mark.gpu
def test_noalloc_matches_compute_velocity_on_two_calls(pdg):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    plate = pdg.plates.make_plate(60, seed=21, crack="centre-half")
    n = plate.n
    ctx = plate.context(s_c=0.0)  # the existing entry point's context (FP64, no breaking)
    rp, col = ctx.families()
    ctx.step(4)  # start from a loaded state
    u, v, f = ctx.state()
    acc = f * (1.0 / plate.material.rho)
    params = plate.params(s_c=0.0)
    dev = torch.device("cuda", 0)
    t = lambda a, dt=torch.float64: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dt)
    dx, dvol, drp, dcol = t(plate.x), t(plate.vol), t(rp, torch.int64), t(col, torch.int32)
    dv, dacc, df = t(v), t(acc), torch.zeros((n, 2), dtype=torch.float64, device=dev)
    hv, hacc = v.copy(), acc.copy()
    for call in range(2):
        du = t(u)
        rc, msg = _noalloc(pdg, n, (dx, dvol, drp, dcol, du, dv, dacc, df), params)
        assert rc == 0, msg
        torch.cuda.synchronize()
        hf = ctx.compute_velocity(u, hv, hacc)  # existing entry point, host buffers
        assert np.array_equal(dv.cpu().numpy(), hv), f"call {call}: velocity differs"
        assert np.array_equal(dacc.cpu().numpy(), hacc), f"call {call}: acce differs"
        assert np.array_equal(df.cpu().numpy(), hf), f"call {call}: netF differs"
        assert np.abs(hf).max() > 0
        # next call: a drifted displacement, as the caller's host loop would make
        u = u + hv * plate.dt + (0.5 * plate.dt * plate.dt) * hacc
