"""ctypes binding of the C ABI in include/pd_gb300.h (libpd_gb300.so).

The library is the product: there is no CPU fallback.  If it is missing or a
CUDA device is unavailable, every call fails loudly.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libpd_gb300.so")

PD_OK = 0
PD_FP64, PD_MIXED = 0, 1
PD_BC_NONE, PD_BC_VELOCITY, PD_BC_FIXED = 0, 1, 2
PD_SINGULAR_ZERO, PD_SINGULAR_ERROR = 0, 1
PD_KERNEL_NAMES = ("drift", "pass_a", "pass_b")
PD_ERRORS = {-1: "PD_ERR_ARG", -2: "PD_ERR_CUDA", -3: "PD_ERR_ORDER", -4: "PD_ERR_CAPACITY",
             -5: "PD_ERR_SINGULAR", -6: "PD_ERR_DEVICE", -7: "PD_ERR_TIMEOUT"}


class PdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{PD_ERRORS.get(code, code)}: {msg}")
        self.code = code


class MazarsParams(ctypes.Structure):
    """pd_mazars_params (include/pd_gb300.h)."""
    _fields_ = [("kappa0", ctypes.c_double), ("a_t", ctypes.c_double), ("b_t", ctypes.c_double),
                ("a_c", ctypes.c_double), ("b_c", ctypes.c_double)]


def mazars_default_params(**kw):
    p = MazarsParams()
    lib().pd_mazars_default_params(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class Params(ctypes.Structure):
    _fields_ = [
        ("precision", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("E", ctypes.c_double),
        ("nu", ctypes.c_double),
        ("rho", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("s_c", ctypes.c_double),
        ("det_guard", ctypes.c_double),
        ("k_hg", ctypes.c_double),
        ("damage_fail", ctypes.c_double),
        ("n1", ctypes.c_double),
        ("n2", ctypes.c_double),
        ("weight_len", ctypes.c_double),
        ("singular_policy", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class Counters(ctypes.Structure):
    _fields_ = [
        ("bonds_broken", ctypes.c_int64),
        ("singular_events", ctypes.c_int64),
        ("steps", ctypes.c_int64),
        ("device_error", ctypes.c_int32),
        ("unstaged_blocks", ctypes.c_int32),
    ]


class BatchConfig(ctypes.Structure):
    _fields_ = [
        ("block", ctypes.c_int32),
        ("blocks_per_sm", ctypes.c_int32),
        ("persistent", ctypes.c_int32),
        ("tile", ctypes.c_int32),
    ]


_vp = ctypes.c_void_p
_lib = None

# name -> argtypes (restype int unless listed in _RESTYPES)
_SIGS = {
    "pd_abi_version": [],
    "pd_default_params": [ctypes.POINTER(Params)],
    "pd_create": [ctypes.POINTER(Params), ctypes.POINTER(_vp)],
    "pd_destroy": [_vp],
    "pd_last_error": [_vp],
    "pd_set_params": [_vp, ctypes.POINTER(Params)],
    "pd_get_params": [_vp, ctypes.POINTER(Params)],
    "pd_set_stiffness": [_vp, _vp],
    "pd_set_particles": [_vp, ctypes.c_int64, _vp, _vp],
    "pd_build_families": [_vp, ctypes.c_double, ctypes.c_int32, _vp],
    "pd_set_families": [_vp, _vp, _vp],
    "pd_num_bonds": [_vp, ctypes.POINTER(ctypes.c_int64)],
    "pd_get_families": [_vp, _vp, _vp],
    "pd_set_bc": [_vp, ctypes.c_int32, _vp, _vp, _vp],
    "pd_reset": [_vp],
    "pd_set_state": [_vp, _vp, _vp, _vp],
    "pd_get_state": [_vp, _vp, _vp, _vp],
    "pd_get_damage": [_vp, _vp],
    "pd_get_bond_mask": [_vp, _vp],
    "pd_get_counters": [_vp, ctypes.POINTER(Counters)],
    "pd_mazars_default_params": [_vp],
    "pd_mazars_init": [_vp, _vp],
    "pd_mazars_update": [_vp],
    "pd_mazars_get": [_vp, _vp, _vp, _vp],
    "pd_mazars_set": [_vp, _vp, _vp],
    "pd_checkpoint_size": [_vp, ctypes.POINTER(ctypes.c_int64)],
    "pd_checkpoint_save": [_vp, _vp, ctypes.c_int64],
    "pd_checkpoint_load": [_vp, _vp, ctypes.c_int64],
    "pd_step": [_vp, ctypes.c_int32],
    "pd_step_host": [_vp, ctypes.c_int32, _vp, _vp, _vp, _vp, _vp, _vp],
    "pd_synchronize": [_vp],
    "pd_compute_velocity": [_vp, _vp, _vp, _vp, _vp],
    "pd_step_timed": [_vp, ctypes.c_int32, ctypes.POINTER(ctypes.c_float)],
    "pd_profile_steps": [_vp, ctypes.c_int32, _vp, _vp],
    "pd_model_bytes": [_vp, ctypes.POINTER(ctypes.c_double)],
    "pd_compute_velocity_noalloc": [ctypes.c_int64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                    ctypes.POINTER(Params), _vp, ctypes.c_char_p, ctypes.c_int],
    "pd_batch_create": [ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(_vp)],
    "pd_batch_destroy": [_vp],
    "pd_batch_last_error": [_vp],
    "pd_batch_add": [_vp, _vp],
    "pd_batch_remove": [_vp, _vp],
    "pd_batch_info": [_vp, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int64),
                      ctypes.POINTER(ctypes.c_int64)],
    "pd_batch_set_config": [_vp, ctypes.POINTER(BatchConfig)],
    "pd_batch_get_config": [_vp, ctypes.POINTER(BatchConfig)],
    "pd_batch_step": [_vp, ctypes.c_int32],
    "pd_batch_synchronize": [_vp],
    "pd_batch_step_timed": [_vp, ctypes.c_int32, ctypes.POINTER(ctypes.c_float)],
    "pd_batch_set_barrier_limits": [_vp, ctypes.c_uint64, ctypes.c_uint32],
    "pd_batch_last_step_ms": [_vp, ctypes.POINTER(ctypes.c_float)],
    "pd_probe_fma_rates": [ctypes.c_int32, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)],
    "pd_probe_link_rates": [ctypes.c_int32, ctypes.c_int64, ctypes.POINTER(ctypes.c_double),
                            ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)],
    "pd_host_alloc": [ctypes.c_int64, ctypes.POINTER(_vp)],
    "pd_host_free": [_vp],
}
_RESTYPES = {"pd_default_params": None, "pd_mazars_default_params": None, "pd_last_error": ctypes.c_char_p,
             "pd_batch_last_error": ctypes.c_char_p}

EXPORTED = tuple(_SIGS)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() "
                               "(the CUDA extension is required; there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        _lib = L
    return _lib


def ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


class PinnedArray:
    """numpy view of a page-locked host buffer (pd_host_alloc)."""

    def __init__(self, shape, dtype=np.float64):
        self.nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self._p = _vp()
        rc = lib().pd_host_alloc(self.nbytes, ctypes.byref(self._p))
        if rc != PD_OK:
            raise PdError(rc, "pd_host_alloc failed")
        buf = (ctypes.c_char * max(self.nbytes, 1)).from_address(self._p.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def free(self):
        if self._p:
            self.array = None
            lib().pd_host_free(self._p)
            self._p = _vp()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def default_params(**kw):
    p = Params()
    lib().pd_default_params(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def probe_fma_rates(device=0):
    """Measured (fp64, fp32) FMA lane-operations per second of the device."""
    a, b = ctypes.c_double(), ctypes.c_double()
    rc = lib().pd_probe_fma_rates(device, ctypes.byref(a), ctypes.byref(b))
    if rc != PD_OK:
        raise PdError(rc, "pd_probe_fma_rates failed")
    return a.value, b.value


def probe_link_rates(nbytes, device=0):
    """Measured copy-engine GB/s of nbytes between page-locked host memory and
    the device: (host to device, device to host, each while both run)."""
    a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    rc = lib().pd_probe_link_rates(device, int(nbytes), ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
    if rc != PD_OK:
        raise PdError(rc, "pd_probe_link_rates failed")
    return a.value, b.value, c.value


class Context:
    """One device-resident plate (a pd_ctx)."""

    def __init__(self, params: Params):
        self._h = _vp()
        self._params = params
        rc = lib().pd_create(ctypes.byref(params), ctypes.byref(self._h))
        if rc != PD_OK:
            raise PdError(rc, lib().pd_last_error(None).decode())
        self.n = 0
        self.nnz = 0

    # -- plumbing
    def _ck(self, rc):
        if rc != PD_OK:
            raise PdError(rc, lib().pd_last_error(self._h).decode())
        return rc

    def close(self):
        if self._h:
            lib().pd_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    # -- set-up
    def set_params(self, **kw):
        p = Params()
        self._ck(lib().pd_get_params(self._h, ctypes.byref(p)))
        for k, v in kw.items():
            setattr(p, k, v)
        self._ck(lib().pd_set_params(self._h, ctypes.byref(p)))

    def set_particles(self, x, vol):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 2)
        vol = np.ascontiguousarray(vol, dtype=np.float64).reshape(-1)
        self._ck(lib().pd_set_particles(self._h, x.shape[0], ptr(x), ptr(vol)))
        self.n = x.shape[0]

    def build_families(self, cutoff, cracks=None):
        cr = np.ascontiguousarray(np.zeros((0, 4)) if cracks is None else cracks, dtype=np.float64).reshape(-1, 4)
        self._ck(lib().pd_build_families(self._h, float(cutoff), cr.shape[0], ptr(cr) if cr.size else None))
        self._refresh_nnz()

    def set_families(self, row_ptr, col):
        rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
        cl = np.ascontiguousarray(col, dtype=np.int32)
        self._ck(lib().pd_set_families(self._h, ptr(rp), ptr(cl) if cl.size else None))
        self._refresh_nnz()

    def _refresh_nnz(self):
        v = ctypes.c_int64(0)
        self._ck(lib().pd_num_bonds(self._h, ctypes.byref(v)))
        self.nnz = v.value

    def families(self):
        rp = np.zeros(self.n + 1, dtype=np.int64)
        col = np.zeros(max(self.nnz, 1), dtype=np.int32)
        self._ck(lib().pd_get_families(self._h, ptr(rp), ptr(col)))
        return rp, col[: self.nnz]

    def set_bc(self, kinds, values, group_of):
        k = np.ascontiguousarray(kinds, dtype=np.int32)
        v = np.ascontiguousarray(values, dtype=np.float64).reshape(-1, 2)
        g = np.ascontiguousarray(group_of, dtype=np.uint8)
        self._ck(lib().pd_set_bc(self._h, k.size, ptr(k), ptr(v), ptr(g)))

    # -- state
    def reset(self):
        self._ck(lib().pd_reset(self._h))

    def set_state(self, u=None, v=None, f=None):
        c = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(-1, 2)
        u, v, f = c(u), c(v), c(f)
        self._ck(lib().pd_set_state(self._h, ptr(u), ptr(v), ptr(f)))

    def state(self):
        u = np.zeros((self.n, 2))
        v = np.zeros((self.n, 2))
        f = np.zeros((self.n, 2))
        self._ck(lib().pd_get_state(self._h, ptr(u), ptr(v), ptr(f)))
        return u, v, f

    def damage(self):
        d = np.zeros(self.n)
        self._ck(lib().pd_get_damage(self._h, ptr(d)))
        return d

    def bond_mask(self):
        m = np.zeros(max(self.nnz, 1), dtype=np.uint8)
        self._ck(lib().pd_get_bond_mask(self._h, ptr(m)))
        return m[: self.nnz]

    def counters(self):
        c = Counters()
        self._ck(lib().pd_get_counters(self._h, ctypes.byref(c)))
        return {"bonds_broken": c.bonds_broken, "singular_events": c.singular_events, "steps": c.steps,
                "device_error": c.device_error, "unstaged_blocks": c.unstaged_blocks}

    # -- Mazars damage (pd_mazars_*)
    def mazars_init(self, params=None, **kw):
        p = params if params is not None else mazars_default_params(**kw)
        self._ck(lib().pd_mazars_init(self._h, ctypes.byref(p)))

    def mazars_update(self):
        self._ck(lib().pd_mazars_update(self._h))

    def mazars(self):
        """(threshold[nnz], bond_damage[nnz]) in family order and status[n]."""
        thr, bd, st = np.empty(self.nnz), np.empty(self.nnz), np.empty(self.n)
        self._ck(lib().pd_mazars_get(self._h, ptr(thr), ptr(bd), ptr(st)))
        return thr, bd, st

    def mazars_set(self, threshold=None, bond_damage=None):
        t = None if threshold is None else np.ascontiguousarray(threshold, dtype=np.float64)
        b = None if bond_damage is None else np.ascontiguousarray(bond_damage, dtype=np.float64)
        self._ck(lib().pd_mazars_set(self._h, ptr(t) if t is not None else None, ptr(b) if b is not None else None))

    # -- checkpoint / restore (pd_checkpoint_*)
    def checkpoint(self) -> bytes:
        """The dynamic state as an opaque blob (restore into a context built from the same inputs)."""
        nb = ctypes.c_int64()
        self._ck(lib().pd_checkpoint_size(self._h, ctypes.byref(nb)))
        buf = ctypes.create_string_buffer(nb.value)
        self._ck(lib().pd_checkpoint_save(self._h, buf, nb.value))
        return buf.raw

    def restore(self, blob: bytes):
        buf = ctypes.create_string_buffer(blob, len(blob))
        self._ck(lib().pd_checkpoint_load(self._h, buf, len(blob)))

    # -- stepping
    def step_host(self, nsteps, u, v, f, u_out=None, v_out=None, f_out=None):
        """pd_step_host: u, v, f ([n][2], page-locked: PinnedArray.array) in,
        the new state written to the *_out buffers (default: in place)."""
        u_out = u if u_out is None else u_out
        v_out = v if v_out is None else v_out
        f_out = f if f_out is None else f_out
        self._ck(lib().pd_step_host(self._h, int(nsteps), ptr(u), ptr(v), ptr(f), ptr(u_out), ptr(v_out),
                                    ptr(f_out)))

    def step(self, nsteps=1):
        self._ck(lib().pd_step(self._h, int(nsteps)))

    def synchronize(self):
        self._ck(lib().pd_synchronize(self._h))

    def compute_velocity(self, u, velocity, acce, netf=None):
        """The reference GPU wrapper's one-call contract on host arrays (velocity
        and acce in place; the force into netf, a new array when None).  With
        every buffer page-locked (PinnedArray.array) the call is pipelined."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        if netf is None:
            netf = np.zeros_like(velocity)
        self._ck(lib().pd_compute_velocity(self._h, ptr(u), ptr(velocity), ptr(acce), ptr(netf)))
        return netf

    def step_timed(self, nsteps):
        ms = ctypes.c_float(0.0)
        self._ck(lib().pd_step_timed(self._h, int(nsteps), ctypes.byref(ms)))
        return ms.value

    def profile_steps(self, nsteps):
        ms = np.zeros(3)
        launches = np.zeros(3, dtype=np.int64)
        self._ck(lib().pd_profile_steps(self._h, int(nsteps), ptr(ms), ptr(launches)))
        return {k: (float(ms[i]), int(launches[i])) for i, k in enumerate(PD_KERNEL_NAMES)}

    def model_bytes(self):
        b = ctypes.c_double(0.0)
        self._ck(lib().pd_model_bytes(self._h, ctypes.byref(b)))
        return b.value


class Batch:
    """Many contexts stepped together (pd_batch): every member's own step graph
    on its own stream (the default), one persistent kernel, or one graph of
    phase kernels advances every member; results equal solo runs."""

    def __init__(self, precision=PD_FP64, device=0):
        self._h = _vp()
        rc = lib().pd_batch_create(device, precision, ctypes.byref(self._h))
        if rc != PD_OK:
            raise PdError(rc, lib().pd_batch_last_error(None).decode())
        self.precision = precision
        self.members = []

    def _ck(self, rc):
        if rc != PD_OK:
            raise PdError(rc, lib().pd_batch_last_error(self._h).decode())
        return rc

    def add(self, ctx):
        self._ck(lib().pd_batch_add(self._h, ctx.handle))
        self.members.append(ctx)

    def remove(self, ctx):
        self._ck(lib().pd_batch_remove(self._h, ctx.handle))
        self.members.remove(ctx)

    def info(self):
        n, p, b = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int64()
        self._ck(lib().pd_batch_info(self._h, ctypes.byref(n), ctypes.byref(p), ctypes.byref(b)))
        return {"plates": n.value, "particles": p.value, "bonds": b.value}

    def config(self):
        c = BatchConfig()
        self._ck(lib().pd_batch_get_config(self._h, ctypes.byref(c)))
        return {"block": c.block, "blocks_per_sm": c.blocks_per_sm, "persistent": c.persistent, "tile": c.tile}

    def set_config(self, block=None, blocks_per_sm=None, persistent=None, tile=None):
        cur = self.config()
        for k, v in (("block", block), ("blocks_per_sm", blocks_per_sm), ("persistent", persistent), ("tile", tile)):
            if v is not None:
                cur[k] = int(v)
        c = BatchConfig(cur["block"], cur["blocks_per_sm"], cur["persistent"], cur["tile"])
        self._ck(lib().pd_batch_set_config(self._h, ctypes.byref(c)))

    def step(self, nsteps=1):
        self._ck(lib().pd_batch_step(self._h, int(nsteps)))

    def synchronize(self):
        self._ck(lib().pd_batch_synchronize(self._h))

    def set_barrier_limits(self, spin_limit=0, hold_ns=0):
        """Persistent-kernel barrier controls (0, 0: the defaults); see pd_gb300.h."""
        self._ck(lib().pd_batch_set_barrier_limits(self._h, int(spin_limit), int(hold_ns)))

    def step_timed(self, nsteps):
        ms = ctypes.c_float(0.0)
        self._ck(lib().pd_batch_step_timed(self._h, int(nsteps), ctypes.byref(ms)))
        return ms.value

    def last_step_ms(self):
        """GPU time of the last step() call's kernels."""
        ms = ctypes.c_float(0.0)
        self._ck(lib().pd_batch_last_step_ms(self._h, ctypes.byref(ms)))
        return ms.value

    def close(self):
        if self._h:
            lib().pd_batch_destroy(self._h)
            self._h = _vp()
            self.members = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
