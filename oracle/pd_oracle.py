"""TEST ORACLE -- not part of the product.

ctypes wrapper over the C restatement (oracle/pd_oracle.c, built by
``make -C oracle oracle`` into oracle/_build/libpd_oracle.so) and a runner for
the reference's own sequential build (oracle/_ref/pd_ref_harness, see
oracle/ref_harness.cpp).  Only tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline / reference leg import this module, and only as the
checker or the CPU baseline; the product path never touches it.
"""
from __future__ import annotations

import ctypes
import os
import struct
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpd_oracle.so")
REF_HARNESS = os.path.join(HERE, "_ref", "pd_ref_harness")

BC_NONE, BC_VELOCITY, BC_FIXED = 0, 1, 2

_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_f64p = ctypes.POINTER(ctypes.c_double)


class _Problem(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64),
        ("x", _f64p),
        ("vol", _f64p),
        ("row_ptr", _i64p),
        ("col", _i32p),
        ("bc", _u8p),
        ("n_groups", ctypes.c_int32),
        ("group_kind", _i32p),
        ("group_val", _f64p),
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
        ("wlen", ctypes.c_double),
        ("nthreads", ctypes.c_int32),
    ]


class _Mazars(ctypes.Structure):
    _fields_ = [("kappa0", ctypes.c_double), ("a_t", ctypes.c_double), ("b_t", ctypes.c_double),
                ("a_c", ctypes.c_double), ("b_c", ctypes.c_double)]


class _State(ctypes.Structure):
    _fields_ = [
        ("u", _f64p),
        ("v", _f64p),
        ("f", _f64p),
        ("alive", _u8p),
        ("broken", _i32p),
        ("damage", _f64p),
        ("kinv", _f64p),
        ("mt", _f64p),
        ("w", _f64p),
        ("hg", _f64p),
        ("singular", _u8p),
        ("tb", _f64p),
        ("rev", _i64p),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"oracle library missing: build it with `make -C {HERE} oracle`")
        L = ctypes.CDLL(LIB_PATH)
        L.pdo_build_families.restype = ctypes.c_int
        L.pdo_build_families.argtypes = [ctypes.c_int64, _f64p, ctypes.c_double, ctypes.c_int32, _f64p,
                                         _i64p, _i32p, ctypes.c_int64, _i64p, ctypes.c_int32]
        L.pdo_init.restype = ctypes.c_int
        L.pdo_init.argtypes = [ctypes.POINTER(_Problem), ctypes.POINTER(_State)]
        L.pdo_step.restype = ctypes.c_int64
        L.pdo_step.argtypes = [ctypes.POINTER(_Problem), ctypes.POINTER(_State), ctypes.c_int32]
        L.pdo_reverse_bonds.restype = ctypes.c_int
        L.pdo_reverse_bonds.argtypes = [ctypes.c_int64, _i64p, _i32p, _i64p]
        L.pdo_mazars_update.restype = ctypes.c_int
        L.pdo_mazars_update.argtypes = [ctypes.POINTER(_Problem), ctypes.POINTER(_State), ctypes.POINTER(_Mazars),
                                        _f64p, _f64p, _f64p]
        L.pdo_stiffness.restype = None
        L.pdo_stiffness.argtypes = [ctypes.c_double, ctypes.c_double, _f64p]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def build_families(x, cutoff, cracks=None, nthreads=0):
    """CSR families (row_ptr int64[n+1], col int32[nnz]) -- restated findNeighbor."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    n = x.shape[0]
    cr = np.ascontiguousarray(np.zeros((0, 4)) if cracks is None else cracks, dtype=np.float64).reshape(-1, 4)
    rp = np.zeros(n + 1, dtype=np.int64)
    nnz = ctypes.c_int64(0)
    L = lib()
    rc = L.pdo_build_families(n, _p(x, _f64p), cutoff, cr.shape[0], _p(cr, _f64p), _p(rp, _i64p), None, 0,
                              ctypes.byref(nnz), nthreads)
    if rc != 0:
        raise RuntimeError(f"pdo_build_families count rc={rc}")
    col = np.zeros(max(nnz.value, 1), dtype=np.int32)
    rc = L.pdo_build_families(n, _p(x, _f64p), cutoff, cr.shape[0], _p(cr, _f64p), _p(rp, _i64p),
                              _p(col, _i32p), col.size, ctypes.byref(nnz), nthreads)
    if rc != 0:
        raise RuntimeError(f"pdo_build_families fill rc={rc}")
    return rp, col[: nnz.value]


def stiffness(E, nu):
    c = np.zeros(3)
    lib().pdo_stiffness(E, nu, _p(c, _f64p))
    return c


@dataclass
class OracleSim:
    """The C restatement stepping one problem (FP64)."""

    x: np.ndarray
    vol: np.ndarray
    row_ptr: np.ndarray
    col: np.ndarray
    E: float
    nu: float
    rho: float
    dt: float
    s_c: float = 0.0
    det_guard: float = 1e-10
    k_hg: float = 0.0
    damage_fail: float = 1.0
    n1: float = 0.0
    n2: float = 0.0
    wlen: float = 1.0
    bc: np.ndarray | None = None
    group_kind: np.ndarray | None = None
    group_val: np.ndarray | None = None
    nthreads: int = 0
    _keep: list = field(default_factory=list, repr=False)

    def __post_init__(self):
        n = self.x.shape[0]
        self.x = np.ascontiguousarray(self.x, dtype=np.float64)
        self.vol = np.ascontiguousarray(self.vol, dtype=np.float64)
        self.row_ptr = np.ascontiguousarray(self.row_ptr, dtype=np.int64)
        self.col = np.ascontiguousarray(self.col, dtype=np.int32)
        nnz = int(self.row_ptr[-1])
        if self.bc is None:
            self.bc = np.zeros(n, dtype=np.uint8)
            self.group_kind = np.zeros(1, dtype=np.int32)
            self.group_val = np.zeros((1, 2))
        self.bc = np.ascontiguousarray(self.bc, dtype=np.uint8)
        self.group_kind = np.ascontiguousarray(self.group_kind, dtype=np.int32)
        self.group_val = np.ascontiguousarray(self.group_val, dtype=np.float64).reshape(-1, 2)
        self.u = np.zeros((n, 2))
        self.v = np.zeros((n, 2))
        self.f = np.zeros((n, 2))
        self.alive = np.zeros(max(nnz, 1), dtype=np.uint8)
        self.broken = np.zeros(n, dtype=np.int32)
        self.damage = np.zeros(n)
        self.kinv = np.zeros((n, 3))
        self.mt = np.zeros((n, 2))
        self.w = np.zeros((n, 4))
        self.singular = np.zeros(n, dtype=np.uint8)
        self.hg = np.zeros((n, 2))
        self.tb = np.zeros((max(nnz, 1), 2))
        self.rev = np.zeros(max(nnz, 1), dtype=np.int64)
        if self.n1 != 0.0 or self.n2 != 0.0:
            if lib().pdo_reverse_bonds(n, _p(self.row_ptr, _i64p), _p(self.col, _i32p), _p(self.rev, _i64p)) != 0:
                raise ValueError("bond-associated mode needs symmetric families")
        self._pb = _Problem(n, _p(self.x, _f64p), _p(self.vol, _f64p), _p(self.row_ptr, _i64p),
                            _p(self.col, _i32p), _p(self.bc, _u8p), self.group_kind.size,
                            _p(self.group_kind, _i32p), _p(self.group_val, _f64p), self.E, self.nu, self.rho,
                            self.dt, self.s_c, self.det_guard, self.k_hg, self.damage_fail, self.n1, self.n2,
                            self.wlen, self.nthreads)
        self._st = _State(_p(self.u, _f64p), _p(self.v, _f64p), _p(self.f, _f64p), _p(self.alive, _u8p),
                          _p(self.broken, _i32p), _p(self.damage, _f64p), _p(self.kinv, _f64p),
                          _p(self.mt, _f64p), _p(self.w, _f64p), _p(self.hg, _f64p), _p(self.singular, _u8p),
                          _p(self.tb, _f64p), _p(self.rev, _i64p))
        lib().pdo_init(ctypes.byref(self._pb), ctypes.byref(self._st))

    def step(self, nsteps=1):
        return int(lib().pdo_step(ctypes.byref(self._pb), ctypes.byref(self._st), int(nsteps)))

    @property
    def mask(self):
        return self.alive[: int(self.row_ptr[-1])]

    def mazars(self, thr, bd, kappa0, a_t=0.87, b_t=20000.0, a_c=0.65, b_c=2150.0):
        """One computeDamageStatus (src/main_seq.cpp:473-598) from the current
        displacements: thr / bd (per bond, family order, float64) are updated in
        place; returns the per-particle damage status."""
        assert thr.dtype == np.float64 and bd.dtype == np.float64 and thr.flags.c_contiguous and bd.flags.c_contiguous
        status = np.zeros(self.x.shape[0])
        mp = _Mazars(kappa0, a_t, b_t, a_c, b_c)
        if lib().pdo_mazars_update(ctypes.byref(self._pb), ctypes.byref(self._st), ctypes.byref(mp),
                                   _p(thr, _f64p), _p(bd, _f64p), _p(status, _f64p)) != 0:
            raise ValueError("bond-associated Mazars damage: a family has more than 256 bonds")
        return status


# ------------------------------------------------------------ reference build

def ref_available():
    return os.path.exists(REF_HARNESS)


def reference_dir():
    """The reference checkout: PD_REFERENCE_DIR, else the one oracle/_ref was
    built from (recorded by oracle/Makefile), else None."""
    d = os.environ.get("PD_REFERENCE_DIR")
    if d:
        return d
    rec = os.path.join(HERE, "_ref", "REFERENCE_DIR")
    if os.path.exists(rec):
        d = open(rec).read().strip()
        return d or None
    return None


def run_ref_mazars(mesh_dir, n1, n2, out):
    """The reference's computeDamageStatus on the Hassa mesh at two imposed
    displacement levels (oracle/ref_harness.cpp, mode `mazars`)."""
    subprocess.run([REF_HARNESS, "mazars", mesh_dir, str(n1), str(n2), out], check=True, capture_output=True)
    b = open(out, "rb").read()
    o = 0
    n = struct.unpack_from("<i", b, o)[0]
    o += 4
    nnz = struct.unpack_from("<q", b, o)[0]
    o += 8
    res = {"n": n, "row_ptr": np.frombuffer(b, "<i8", n + 1, o).copy()}
    o += 8 * (n + 1)
    res["col"] = np.frombuffer(b, "<i4", nnz, o).copy()
    o += 4 * nnz
    for _ in range(2):
        lv = struct.unpack_from("<i", b, o)[0]
        o += 4
        d = {"u": np.frombuffer(b, "<f8", 2 * n, o).reshape(n, 2).copy()}
        o += 16 * n
        d["thr"] = np.frombuffer(b, "<f8", nnz, o).copy()
        o += 8 * nnz
        d["bd"] = np.frombuffer(b, "<f8", nnz, o).copy()
        o += 8 * nnz
        d["status"] = np.frombuffer(b, "<f8", n, o).copy()
        o += 8 * n
        res[lv] = d
    return res


def read_ref_output(path, n_hint=None, hassa=False):
    """Parse pd_ref_harness output (see oracle/ref_harness.cpp)."""
    b = open(path, "rb").read()
    o = 0
    n = struct.unpack_from("<i", b, o)[0]
    o += 4
    out = {"n": n}
    if hassa:
        xv = np.frombuffer(b, "<f8", 3 * n, o).reshape(n, 3).copy()
        o += 24 * n
        out["x"], out["vol"] = xv[:, :2].copy(), xv[:, 2].copy()
        sets = []
        for _ in range(4):
            c = struct.unpack_from("<i", b, o)[0]
            o += 4
            sets.append(np.frombuffer(b, "<i4", c, o).copy())
            o += 4 * c
        out["boundary_sets"] = sets
    nnz = struct.unpack_from("<q", b, o)[0]
    o += 8
    out["row_ptr"] = np.frombuffer(b, "<i8", n + 1, o).copy()
    o += 8 * (n + 1)
    out["col"] = np.frombuffer(b, "<i4", nnz, o).copy()
    o += 4 * nnz
    steps = {}
    while o < len(b):
        s = struct.unpack_from("<i", b, o)[0]
        o += 4
        arr = np.frombuffer(b, "<f8", 8 * n, o).reshape(4, n, 2).copy()
        o += 64 * n
        steps[s] = {"u": arr[0], "v": arr[1], "f": arr[2], "a": arr[3]}
    out["steps"] = steps
    return out


def write_ref_input(path, x, vol, params, nsteps, dump_every=1, families=None, vbc=(), fixed=(), state=None):
    """Write the plate-mode input of pd_ref_harness.  vbc: [(idx, (vx, vy))];
    state: None (start at rest) or (u0, v0), the initial displacement and
    velocity, [n][2] each (input format version 2)."""
    n = x.shape[0]
    with open(path, "wb") as fh:
        fh.write(b"PDRF")
        fh.write(struct.pack("<iii", 1 if state is None else 2, n, 1 if families is not None else 0))
        fh.write(struct.pack("<8d", params["dx"], params["horizon"], params.get("n1", 0.0), params.get("n2", 0.0),
                             params["E"], params["nu"], params["rho"], params["dt"]))
        fh.write(struct.pack("<ii", nsteps, dump_every))
        fh.write(np.ascontiguousarray(x, dtype="<f8").tobytes())
        fh.write(np.ascontiguousarray(vol, dtype="<f8").tobytes())
        if state is not None:
            fh.write(struct.pack("<i", 1))
            fh.write(np.ascontiguousarray(state[0], dtype="<f8").tobytes())
            fh.write(np.ascontiguousarray(state[1], dtype="<f8").tobytes())
        if families is not None:
            fh.write(np.ascontiguousarray(families[0], dtype="<i8").tobytes())
            fh.write(np.ascontiguousarray(families[1], dtype="<i4").tobytes())
        fh.write(struct.pack("<i", len(vbc)))
        for idx, val in vbc:
            idx = np.ascontiguousarray(idx, dtype="<i4")
            fh.write(struct.pack("<idd", idx.size, float(val[0]), float(val[1])))
            fh.write(idx.tobytes())
        fixed = np.ascontiguousarray(fixed, dtype="<i4")
        fh.write(struct.pack("<i", fixed.size))
        fh.write(fixed.tobytes())


def read_grid_dump(path):
    """The `grid` dump of computeInitialPositions (oracle/ref_harness.cpp; the
    drop-in's tests/grid_main.cpp writes the same format): each long double
    as the pair (hi, lo) of doubles."""
    b = open(path, "rb").read()
    n, nd = struct.unpack_from("<ii", b, 0)
    o = 8
    box = np.frombuffer(b, "<f8", 4 * nd, o).reshape(2 * nd, 2).copy()
    o += 8 * 4 * nd
    rec = np.dtype([("gid", "<i4"), ("part", "<i4"), ("x0", "<f8", (nd, 2)), ("x", "<f8", (nd, 2)),
                    ("vol", "<f8", (2,))])
    r = np.frombuffer(b, rec, n, o)
    return {"n": n, "ndim": nd, "boxlimit": box, "gid": r["gid"].copy(), "part": r["part"].copy(),
            "x0": r["x0"].copy(), "x": r["x"].copy(), "vol": r["vol"].copy()}


def run_ref_grid(rows, dx, ndim, out_path):
    """The reference's computeInitialPositions (oracle/ref_harness.cpp, mode `grid`)."""
    subprocess.run([REF_HARNESS, "grid", str(rows), repr(dx), str(ndim), out_path], check=True,
                   capture_output=True)
    return read_grid_dump(out_path)


def run_ref_plate(in_path, out_path, timeout=3600):
    subprocess.run([REF_HARNESS, "plate", in_path, out_path], check=True, timeout=timeout,
                   stdout=subprocess.DEVNULL)
    return read_ref_output(out_path)


def run_ref_hassa(mesh_dir, work_dir, n1, n2, nsteps, out_path, timeout=3600):
    subprocess.run([REF_HARNESS, "hassa", mesh_dir, work_dir, str(n1), str(n2), str(nsteps), out_path],
                   check=True, timeout=timeout, stdout=subprocess.DEVNULL)
    return read_ref_output(out_path, hassa=True)
