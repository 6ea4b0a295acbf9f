"""Seeded synthetic plates (the workloads the step is measured on).

A plate is a uniform grid of n_x * n_y particles in row-major order, x
fastest, centred as the reference's computeInitialPositions
(src/SetupParticleSystem.cpp:62-98: box minimum -floor(n/2)*dx), each
coordinate jittered by a seeded uniform +-jitter*dx, volume dx^2 * thickness.
Families use the reference's findNeighbor cutoff 1.01 * dx * horizon
(src/SetupParticleSystem.cpp:113) with horizon = 3.015 (28 neighbours in the
interior); bonds crossing the pre-crack segment are removed.  The top and
bottom `bc_rows` rows carry prescribed +-y velocity (the reference selects one
row per face with defineBoundarySet, src/SetupParticleSystem.cpp:513-529; the
plate workloads ask for three).  Random numbers come from a counter-based
splitmix64 stream, so every consumer regenerates identical inputs.

The plates run with a zero-energy-mode penalty (G_s = 0.25) and material-
point failure at damage 0.5: the classic correspondence model alone lets the
velocity loading grow hourglass modes until bonds fail spuriously, and
particles held by a few bonds outgrow the time step once cracks run; both
make the run diverge (hourglass=0, damage_fail=1 give the reference's model).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import native

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(z):
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def uniform(seed, stream, idx):
    """Uniform [0, 1) doubles for counters idx of (seed, stream)."""
    with np.errstate(over="ignore"):
        key = splitmix64(np.uint64(seed) * np.uint64(0x9E3779B1) + np.uint64(stream) * np.uint64(0x632BE59BD9B4E019))
        r = splitmix64(key + np.asarray(idx, dtype=np.uint64))
    return (r >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


@dataclass
class Material:
    E: float = 72e9
    nu: float = 0.33
    rho: float = 2440.0
    s_c: float = 5e-4


@dataclass
class Plate:
    nx: int
    ny: int
    dx: float
    thickness: float
    x: np.ndarray            # [n][2]
    vol: np.ndarray          # [n]
    cutoff: float
    cracks: np.ndarray       # [k][4]
    group_of: np.ndarray     # [n] uint8, 0 free, 1 top, 2 bottom
    group_kind: np.ndarray   # [2]
    group_val: np.ndarray    # [2][2]
    material: Material
    dt: float
    steps: int
    name: str = ""
    meta: dict = field(default_factory=dict)
    hourglass: float = 0.25  # G_s of the zero-energy-mode penalty (0: the reference's model)
    damage_fail: float = 0.5  # material-point failure threshold (>= 1: never)

    @property
    def n(self):
        return self.x.shape[0]

    @property
    def k_hg(self):
        """Zero-energy-mode penalty coefficient k = G_s C11 / (mean V * cutoff^2)."""
        m = self.material
        c11 = m.E / (1.0 - m.nu * m.nu)
        return self.hourglass * c11 / (float(self.vol.mean()) * self.cutoff * self.cutoff)

    def params(self, precision=native.PD_FP64, device=0, s_c=None, det_guard=1e-10, k_hg=None, damage_fail=None):
        m = self.material
        return native.default_params(precision=precision, device=device, E=m.E, nu=m.nu, rho=m.rho, dt=self.dt,
                                     s_c=m.s_c if s_c is None else s_c, det_guard=det_guard,
                                     k_hg=self.k_hg if k_hg is None else k_hg,
                                     damage_fail=self.damage_fail if damage_fail is None else damage_fail)

    def context(self, precision=native.PD_FP64, device=0, s_c=None, k_hg=None):
        """A device context with particles, GPU-built families and BCs set."""
        ctx = native.Context(self.params(precision, device, s_c, k_hg=k_hg))
        ctx.set_particles(self.x, self.vol)
        ctx.build_families(self.cutoff, self.cracks)
        ctx.set_bc(self.group_kind, self.group_val, self.group_of)
        return ctx


def cfl_dt(dx, E, rho, factor=0.8):
    """dt = factor * dx / sqrt(E/rho) (the reference fixes stepSize by hand, src/main_seq.cpp:657)."""
    return factor * dx / math.sqrt(E / rho)


def make_plate(nx, ny=None, *, dx=1e-3, thickness=1e-3, jitter=0.01, seed=0, horizon=3.015, bc_rows=3,
               v_load=1.0, material=None, crack=None, steps=100, dt=None, name="") -> Plate:
    """crack: None, or (cx, cy, length, angle_rad) in metres/radians, or 'centre-half'."""
    ny = nx if ny is None else ny
    material = material or Material()
    n = nx * ny
    idx = np.arange(n, dtype=np.int64)
    col, row = idx % nx, idx // nx
    x0 = -math.floor(nx / 2) * dx
    y0 = -math.floor(ny / 2) * dx
    jit = (2.0 * uniform(seed, 1, np.arange(2 * n)) - 1.0).reshape(n, 2) * (jitter * dx)
    x = np.empty((n, 2))
    x[:, 0] = x0 + col * dx + jit[:, 0]
    x[:, 1] = y0 + row * dx + jit[:, 1]
    vol = np.full(n, dx * dx * thickness)
    cracks = np.zeros((0, 4))
    if crack == "centre-half":
        # horizontal, centred, half the width long, between two particle rows
        yc = y0 + (ny // 2 - 0.5) * dx
        xc = x0 + 0.5 * (nx - 1) * dx
        half = 0.25 * (nx - 1) * dx
        cracks = np.array([[xc - half, yc, xc + half, yc]])
    elif crack is not None:
        cx, cy, length, ang = crack
        h = 0.5 * length
        cracks = np.array([[cx - h * math.cos(ang), cy - h * math.sin(ang), cx + h * math.cos(ang),
                            cy + h * math.sin(ang)]])
    group_of = np.zeros(n, dtype=np.uint8)
    group_of[row >= ny - bc_rows] = 1
    group_of[row < bc_rows] = 2
    group_kind = np.array([native.PD_BC_VELOCITY, native.PD_BC_VELOCITY], dtype=np.int32)
    group_val = np.array([[0.0, v_load], [0.0, -v_load]])
    if dt is None:
        dt = cfl_dt(dx, material.E, material.rho)
    return Plate(nx, ny, dx, thickness, x, vol, 1.01 * dx * horizon, cracks, group_of, group_kind, group_val,
                 material, dt, steps, name, {"seed": seed, "x0": x0, "y0": y0})


def hassa_mesh_text():
    """The reference's only input mesh, 2D_Hassa_test_mesh.dat, written by its
    rule: a 70 x 60 grid of unit cells, centres x in [-34.5, 34.5], y in
    [-29.5, 29.5], area 1, x the outer loop, six decimals, one header line.
    (tests/golden/make_golden.py checks it equals the reference's file.)"""
    rows = ["Center_X Center_Y Area"]
    for ix in range(70):
        for iy in range(60):
            rows.append(f"{ix - 34.5:.6f} {iy - 29.5:.6f} {1.0:.6f}")
    return "\n".join(rows) + "\n"


def config_plate_100(seed=0):
    """100 x 100 FP64 plate, centred half-width horizontal pre-crack, 100 steps."""
    return make_plate(100, seed=seed, crack="centre-half", steps=100, name="plate100x100-fp64")


def config_plate_scale(side=1000, seed=0, steps=1000):
    """side x side plate, crack of seeded length in [0.2, 0.5] width at a seeded
    height (middle half of the plate), 1000 steps with bond breaking."""
    dx = 1e-3
    r = uniform(seed, 7, np.arange(2))
    length = (0.2 + 0.3 * r[0]) * (side - 1) * dx
    x0 = -math.floor(side / 2) * dx
    row = int(side * 0.25 + r[1] * side * 0.5)
    cy = x0 + (row - 0.5) * dx
    cx = x0 + 0.5 * (side - 1) * dx
    return make_plate(side, seed=seed, crack=(cx, cy, length, 0.0), steps=steps,
                      name=f"plate{side}x{side}")


def batch_plate_specs(count=256, seed=0, side_lo=50, side_hi=400):
    """Per-plate specs of the ragged batch: side U[50,400], crack length 0.1-0.5
    width at angle +-30 deg, E U[50,100] GPa, nu U[0.2,0.35], load U[0.5,2] m/s."""
    r = uniform(seed, 11, np.arange(8 * count)).reshape(count, 8)
    specs = []
    for b in range(count):
        side = int(side_lo + r[b, 0] * (side_hi - side_lo + 1))
        side = min(side, side_hi)
        mat = Material(E=50e9 + 50e9 * r[b, 1], nu=0.2 + 0.15 * r[b, 2], rho=2440.0, s_c=5e-4)
        specs.append({"side": side, "material": mat, "v_load": 0.5 + 1.5 * r[b, 3],
                      "crack_len": 0.1 + 0.4 * r[b, 4], "crack_ang": math.radians(-30.0 + 60.0 * r[b, 5]),
                      "crack_cx": 0.3 + 0.4 * r[b, 6], "crack_cy": 0.3 + 0.4 * r[b, 7], "seed": seed * 1000 + b})
    return specs


def plate_from_spec(spec, steps=500):
    side = spec["side"]
    dx = 1e-3
    x0 = -math.floor(side / 2) * dx
    w = (side - 1) * dx
    crack = (x0 + spec["crack_cx"] * w, x0 + spec["crack_cy"] * w, spec["crack_len"] * w, spec["crack_ang"])
    return make_plate(side, seed=spec["seed"], crack=crack, steps=steps, material=spec["material"],
                      v_load=spec["v_load"], name=f"batch-plate-{side}")
