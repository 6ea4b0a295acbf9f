"""pd_compute_velocity_noalloc: the entry point for callers that cannot call
cudaMalloc (a host application whose own pool owns all device memory, or a
latency-critical loop where an allocation would synchronise the device).

The caller owns every buffer; the tests allocate them with torch (the
caller's pool here) and check the results against the existing host-buffer
entry point pd_compute_velocity on the same inputs -- bit for bit, the
tolerance of every FP64 test here -- over two calls in a row, with an
isolated particle (an empty family), on a non-default stream, and with a
smaller problem after a larger one (the shared scratch then still holds the
larger call's entries).  This file is collected last on purpose, and also
passes when run alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

PD_ERR_ARG, PD_ERR_CAPACITY = -1, -4


def _noalloc(pdg, n, bufs, params, stream=None):
    L = pdg.native.lib()
    err = ctypes.create_string_buffer(256)
    rc = L.pd_compute_velocity_noalloc(
        n, *(ctypes.c_void_p(b.data_ptr() if b is not None else 0) for b in bufs), ctypes.byref(params),
        ctypes.c_void_p(stream), err, 256)
    return rc, err.value.decode()


def test_noalloc_rejects_sizes_beyond_the_maximum(pdg):
    L = pdg.native.lib()
    err = ctypes.create_string_buffer(256)
    p = pdg.default_params()
    rc = L.pd_compute_velocity_noalloc(70000, None, None, None, None, None, None, None, None, ctypes.byref(p), None,
                                       err, 256)  # checked before any device work
    assert rc == PD_ERR_CAPACITY and b"PD_NOALLOC_MAX_PARTICLES" in err.value
    assert L.pd_compute_velocity_noalloc(-1, None, None, None, None, None, None, None, None, ctypes.byref(p), None,
                                         None, 0) == PD_ERR_CAPACITY


@pytest.mark.parametrize("field,value,words", [("precision", 1, b"FP64 only"), ("n1", 10.0, b"classic weights"),
                                               ("n2", 2.0, b"classic weights"), ("s_c", 5e-4, b"no bond breaking")])
def test_noalloc_refuses_what_it_does_not_implement(pdg, field, value, words):
    """Parameters this path would ignore are refused (before any device work)."""
    L = pdg.native.lib()
    err = ctypes.create_string_buffer(256)
    p = pdg.default_params(rho=2440.0, dt=1e-7)
    setattr(p, field, value)
    rc = L.pd_compute_velocity_noalloc(10, None, None, None, None, None, None, None, None, ctypes.byref(p), None,
                                       err, 256)
    assert rc == PD_ERR_ARG and words in err.value, err.value


def _problem(pdg, side, seed, isolated=False):
    """A plate context (FP64, no breaking) loaded by 4 steps, optionally with
    one extra particle far from the plate (an empty family)."""
    plate = pdg.plates.make_plate(side, seed=seed, crack="centre-half")
    x, vol = plate.x, plate.vol
    if isolated:
        x = np.vstack([x, [[1.0, 1.0]]])
        vol = np.append(vol, vol[0])
    ctx = pdg.native.Context(plate.params(s_c=0.0))
    ctx.set_particles(x, vol)
    ctx.build_families(plate.cutoff, plate.cracks)
    g = np.append(plate.group_of, 0) if isolated else plate.group_of
    ctx.set_bc(plate.group_kind, plate.group_val, g)
    ctx.step(4)
    u, v, f = ctx.state()
    return plate, ctx, x, vol, u, v, f * (1.0 / plate.material.rho)


def _run_and_compare(pdg, torch, plate, ctx, x, vol, u, v, acc, calls=2, stream=None):
    n = x.shape[0]
    rp, col = ctx.families()
    params = plate.params(s_c=0.0)
    dev = torch.device("cuda", 0)
    t = lambda a, dt=torch.float64: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dt)
    dx, dvol, drp, dcol = t(x), t(vol), t(rp, torch.int64), t(col, torch.int32)
    dv, dacc, df = t(v), t(acc), torch.zeros((n, 2), dtype=torch.float64, device=dev)
    hv, hacc = v.copy(), acc.copy()
    for call in range(calls):
        du = t(u)
        if stream is not None:
            stream.wait_stream(torch.cuda.current_stream())
        rc, msg = _noalloc(pdg, n, (dx, dvol, drp, dcol, du, dv, dacc, df), params,
                           None if stream is None else stream.cuda_stream)
        assert rc == 0, msg
        (stream if stream is not None else torch.cuda).synchronize()
        hf = ctx.compute_velocity(u, hv, hacc)  # existing entry point, host buffers
        assert np.array_equal(dv.cpu().numpy(), hv), f"call {call}: velocity differs"
        assert np.array_equal(dacc.cpu().numpy(), hacc), f"call {call}: acce differs"
        assert np.array_equal(df.cpu().numpy(), hf), f"call {call}: netF differs"
        assert np.abs(hf).max() > 0 and np.isfinite(hf).all()
        # next call: a drifted displacement, as the caller's host loop would make
        u = u + hv * plate.dt + (0.5 * plate.dt * plate.dt) * hacc
    return hf


@pytest.mark.gpu
def test_noalloc_matches_compute_velocity_on_two_calls(pdg):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    plate, ctx, x, vol, u, v, acc = _problem(pdg, 60, 21)
    _run_and_compare(pdg, torch, plate, ctx, x, vol, u, v, acc)
    ctx.close()


@pytest.mark.gpu
def test_noalloc_isolated_particle_on_a_stream_after_a_larger_call(pdg):
    """A 3,600-particle call, then a 1,601-particle call whose last particle has
    no family, on a non-default stream: the second call reads only entries it
    wrote itself, whatever the larger call left in the shared scratch."""
    torch = pytest.importorskip("torch")
    plate, ctx, x, vol, u, v, acc = _problem(pdg, 60, 22)
    _run_and_compare(pdg, torch, plate, ctx, x, vol, u, v, acc, calls=1)
    ctx.close()
    plate, ctx, x, vol, u, v, acc = _problem(pdg, 40, 23, isolated=True)
    rp, _ = ctx.families()
    assert rp[-1] == rp[-2]  # the extra particle's family is empty
    s = torch.cuda.Stream()
    hf = _run_and_compare(pdg, torch, plate, ctx, x, vol, u, v, acc, calls=2, stream=s)
    assert np.array_equal(hf[-1], [0.0, 0.0])
    ctx.close()


@pytest.mark.gpu
def test_noalloc_bad_family_index_poisons_instead_of_reading(pdg):
    """A family index outside [0, n) is caught by the kernels' own check (no
    read through it): that particle's outputs are NaN, every particle whose
    family does not reach it keeps the result of the valid families."""
    torch = pytest.importorskip("torch")
    plate, ctx, x, vol, u, v, acc = _problem(pdg, 40, 24)
    n = x.shape[0]
    rp, col = ctx.families()
    bad = n // 2
    col_bad = col.copy()
    col_bad[rp[bad]] = n + 5  # out of range
    dev = torch.device("cuda", 0)
    t = lambda a, dt=torch.float64: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dt)
    outs = []
    for c in (col, col_bad):
        dv, dacc, df = t(v), t(acc), torch.zeros((n, 2), dtype=torch.float64, device=dev)
        rc, msg = _noalloc(pdg, n, (t(x), t(vol), t(rp, torch.int64), t(c, torch.int32), t(u), dv, dacc, df),
                           plate.params(s_c=0.0))
        assert rc == 0, msg
        torch.cuda.synchronize()
        outs.append((dv.cpu().numpy(), df.cpu().numpy()))
    (v_ok, f_ok), (v_bad, f_bad) = outs
    assert np.isnan(f_bad[bad]).all() and np.isnan(v_bad[bad]).all()
    reach = {bad} | {i for i in range(n) if bad in col[rp[i]:rp[i + 1]]}
    keep = np.array([i not in reach for i in range(n)])
    assert np.array_equal(f_bad[keep], f_ok[keep]) and np.array_equal(v_bad[keep], v_ok[keep])
    ctx.close()
