"""Generate the golden fixtures in tests/golden/ from the reference's OWN code.

Run here, where the reference checkout exists (it does not exist on the GPU
machine, which only reads the committed .npz files):

    make -C oracle ref oracle REF=<reference checkout>
    python tests/golden/make_golden.py [--reference <checkout>] [--only mazars|plates]

(--reference defaults to PD_REFERENCE_DIR, else the checkout oracle/_ref was
built from.)

Steps, each recorded in manifest.json:
 1. Hassa mesh (the reference's only input, 2D_Hassa_test_mesh.dat): the
    fixture regenerates it from its rule (70 x 60 unit grid, x in
    [-34.5, 34.5], y in [-29.5, 29.5], unit area) and checks it equals the
    reference file, so the mesh itself is not copied.
 2. oracle/_ref/pd_ref_harness (reference main_seq.cpp + SetupParticleSystem.cpp
    + matrix.cpp) runs the reference main with n1 = n2 = 10; its 6-digit
    outputs must equal the reference's shipped goldens
    output/velocity_step_0_after_seq_ref.txt and
    output/LocalParticlesPositions_rank_0step_0.txt byte for byte.  This pins
    the harness.
 3. The pinned harness runs the classic case n1 = n2 = 0 for 3 steps and the
    bond-associated case n1 = n2 = 10 for 1 step at full precision -> hassa_ref.npz.
 4. A seeded 30 x 30 SI plate (jitter, centre crack, 3-row +-1 m/s BCs):
    the reference's findNeighbor families (no crack) and 4 reference steps
    with the crack-cut families -> plate30_ref.npz.
 5. The reference's Mazars damage (computeDamageStatus) on the Hassa mesh,
    classic and n1 = n2 = 10 weights, at two imposed displacement fields in
    turn -> mazars_ref.npz.  `--only mazars` regenerates just this one.
 7. The reference's computeInitialPositions (src/SetupParticleSystem.cpp:62-98)
    on grids of 1, 2 and 3 dimensions, odd and even rows (`--only grid`)
    -> grid_ref.npz: every particle's ids, positions and volume and the box
    limits, long doubles as (hi, lo) double pairs.
 6. The reference's own step with its own model (no zero-energy-mode
    penalty, no bond breaking) on the benchmark plates (`--only plates`):
    the config-1 100 x 100 plate (plates.config_plate_100(seed=0)) for 3
    steps from rest, and again from a seeded preloaded state (preload_state
    below: every particle displaced and moving, so the crack and the whole
    interior carry load from the first step); and the 200 x 200 cut of the
    1M-particle workload (plates.config_plate_scale(side=200, seed=0)) for 2
    steps from rest -> config1_ref.npz, plate200_ref.npz.  Families are the
    crack-cut restatement families (the reference's findNeighbor has no crack
    rule for plates); their sha256 is stored so a test can check its own.
"""
from __future__ import annotations

import argparse
import filecmp
import hashlib
import importlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pd_oracle as po  # noqa: E402

plates = importlib.import_module("2d_pd_gpu_gb300.plates")


def sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def families_sha(row_ptr, col):
    """sha256 of the CSR families as little-endian int64 row_ptr then int32 col."""
    h = hashlib.sha256(np.ascontiguousarray(row_ptr, dtype="<i8").tobytes())
    h.update(np.ascontiguousarray(col, dtype="<i4").tobytes())
    return h.hexdigest()


def preload_state(p, seed=5):
    """A seeded initial displacement and velocity for plate p ([n][2] each).

    Polynomials of the reference coordinates plus splitmix64 noise: plain
    IEEE additions and multiplications (no transcendental functions), so every
    machine regenerates the same bits.  Displacement: a stretch-shear of
    strain 2e-4, a quadratic bend and +-2e-7 m noise; velocity: a linear
    field of up to ~0.5 m/s and +-0.05 m/s noise."""
    x = p.x
    cx = p.meta["x0"] + 0.5 * (p.nx - 1) * p.dx
    cy = p.meta["y0"] + 0.5 * (p.ny - 1) * p.dx
    X = (x[:, 0] - cx) / p.dx
    Y = (x[:, 1] - cy) / p.dx
    r = plates.uniform(seed, 3, np.arange(4 * p.n)).reshape(p.n, 4) * 2.0 - 1.0
    u0 = np.empty((p.n, 2))
    u0[:, 0] = p.dx * (2e-4 * (X + 0.3 * Y) + 1e-6 * X * Y) + 2e-7 * r[:, 0]
    u0[:, 1] = p.dx * (-0.8e-4 * Y + 1.5e-6 * X * X) + 2e-7 * r[:, 1]
    v0 = np.empty((p.n, 2))
    v0[:, 0] = 0.01 * X + 0.05 * r[:, 2]
    v0[:, 1] = -0.005 * Y + 0.05 * r[:, 3]
    return u0, v0


def state_sha(u0, v0):
    h = hashlib.sha256(np.ascontiguousarray(u0, dtype="<f8").tobytes())
    h.update(np.ascontiguousarray(v0, dtype="<f8").tobytes())
    return h.hexdigest()


def _ref_plate_run(p, td, tag, nsteps, state=None):
    """The reference's own step (k_hg = 0, no breaking) on plate p with the
    crack-cut restatement families; returns (row_ptr, col, harness output)."""
    rp, col = po.build_families(p.x, p.cutoff, p.cracks)
    prm = {"dx": p.dx, "horizon": 3.015, "E": p.material.E, "nu": p.material.nu, "rho": p.material.rho,
           "dt": p.dt}
    vbc = [(np.nonzero(p.group_of == 1)[0], p.group_val[0]), (np.nonzero(p.group_of == 2)[0], p.group_val[1])]
    fin = os.path.join(td, f"{tag}.bin")
    po.write_ref_input(fin, p.x, p.vol, prm, nsteps, families=(rp, col), vbc=vbc, state=state)
    return rp, col, po.run_ref_plate(fin, os.path.join(td, f"{tag}.out"), timeout=4 * 3600)


def fixtures_plates(td, man):
    import time
    p = plates.config_plate_100(seed=0)
    t0 = time.time()
    rp, col, rest = _ref_plate_run(p, td, "c1_rest", 3)
    t_rest = time.time() - t0
    u0, v0 = preload_state(p)
    _, _, pre = _ref_plate_run(p, td, "c1_pre", 3, state=(u0, v0))
    out = {"families_sha": np.array(families_sha(rp, col)), "state_sha": np.array(state_sha(u0, v0))}
    for s in (1, 3):
        for k in ("u", "v", "f"):
            out[f"rest_{k}{s}"] = rest["steps"][s][k]
    for k in ("u", "v", "f"):
        out[f"pre_{k}3"] = pre["steps"][3][k]
    np.savez_compressed(os.path.join(HERE, "config1_ref.npz"), **out)
    man["config1"] = {"generator": "plates.config_plate_100(seed=0)", "n": int(p.n), "bonds": int(rp[-1]),
                      "model": "reference (k_hg=0, s_c=0, damage_fail=1)", "steps": {"rest": [1, 3], "preloaded": [3]},
                      "preload": "make_golden.preload_state(plate, seed=5)",
                      "reference_seconds_per_step": round(t_rest / 3, 1)}
    p2 = plates.config_plate_scale(side=200, seed=0)
    t0 = time.time()
    rp2, col2, r2 = _ref_plate_run(p2, td, "p200_rest", 2)
    t2 = time.time() - t0
    out2 = {"families_sha": np.array(families_sha(rp2, col2))}
    for s in (1, 2):
        for k in ("u", "v", "f"):
            out2[f"rest_{k}{s}"] = r2["steps"][s][k]
    np.savez_compressed(os.path.join(HERE, "plate200_ref.npz"), **out2)
    man["plate200"] = {"generator": "plates.config_plate_scale(side=200, seed=0)", "n": int(p2.n),
                       "bonds": int(rp2[-1]), "model": "reference (k_hg=0, s_c=0, damage_fail=1)",
                       "steps": {"rest": [1, 2]}, "reference_seconds_per_step": round(t2 / 2, 1)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=po.reference_dir())
    ap.add_argument("--only", choices=["mazars", "plates", "grid"], default=None)
    args = ap.parse_args()
    ref = args.reference
    if not po.ref_available() or not ref:
        sys.exit("build the reference oracle first: make -C oracle ref REF=<reference checkout>")
    man_path = os.path.join(HERE, "manifest.json")
    man = json.load(open(man_path)) if args.only and os.path.exists(man_path) else {}
    with tempfile.TemporaryDirectory() as td:
        # 1. mesh by rule
        mesh_dir = os.path.join(td, "mesh")
        os.makedirs(mesh_dir)
        mesh = os.path.join(mesh_dir, "2D_Hassa_test_mesh.dat")
        open(mesh, "w").write(plates.hassa_mesh_text())
        if args.only is None:
            fixtures_1_to_4(ref, td, mesh_dir, mesh, man)
        if args.only in (None, "plates"):
            fixtures_plates(td, man)
        if args.only in (None, "mazars"):
            fixtures_mazars(td, mesh_dir, man)
        if args.only in (None, "grid"):
            fixtures_grid(td, man)
    json.dump(man, open(man_path, "w"), indent=1, sort_keys=True)
    print(json.dumps(man, indent=1, sort_keys=True))
    bad = [k for k, v in man.items() if v is False]
    if bad:
        sys.exit(f"pinning failed: {bad}")


# (numParticlesRow, dx, ndim): the config-1 plate's 100 x 100 at 1e-3, odd
# and even rows, dx not a power of two, and the 1D and 3D branches
GRID_CASES = [(100, 1e-3, 2), (7, 0.5, 2), (8, 0.3, 2), (5, 1.0, 1), (5, 0.1, 3), (4, 2.5e-4, 3)]


def fixtures_grid(td, man):
    out = {}
    for k, (rows, dx, nd) in enumerate(GRID_CASES):
        r = po.run_ref_grid(rows, dx, nd, os.path.join(td, f"grid{k}.bin"))
        for key in ("boxlimit", "gid", "part", "x0", "x", "vol"):
            out[f"c{k}_{key}"] = r[key]
    out["cases"] = np.array(GRID_CASES, dtype=object).astype(str)
    np.savez_compressed(os.path.join(HERE, "grid_ref.npz"), **out)
    man["grid"] = {"function": "computeInitialPositions (src/SetupParticleSystem.cpp:62-98)",
                   "cases": [list(c) for c in GRID_CASES], "long_double": "(hi, lo) double pairs"}


def fixtures_mazars(td, mesh_dir, man):
    if True:
        # 5. Mazars damage, classic and bond-associated weights
        out = {"kappa0": np.float64(np.longdouble(3.0) / np.longdouble(3.5e4))}
        for tag, w in (("c", 0), ("b", 10)):
            r = po.run_ref_mazars(mesh_dir, w, w, os.path.join(td, f"mz{w}.bin"))
            for lv in (1, 2):
                out[f"u{lv}"] = r[lv]["u"]
                out[f"{tag}_st{lv}"] = r[lv]["status"]
            # per-bond history after both calls (level 1 enters through the statuses)
            out[f"{tag}_thr2"], out[f"{tag}_bd2"] = r[2]["thr"], r[2]["bd"]
            out[f"{tag}_updated1"] = int((r[1]["thr"] > out["kappa0"]).sum())
        np.savez_compressed(os.path.join(HERE, "mazars_ref.npz"), **out)
        man["mazars"] = {"mesh": "hassa", "weights": ["n1=n2=0", "n1=n2=10"], "levels": [1, 2],
                         "kappa0": "3.0L / 3.5e4L (tensileStrength / E, src/main_seq.cpp:659)",
                         "law": "a_t=0.87 b_t=20000 a_c=0.65 b_c=2150 (src/main_seq.cpp:481)",
                         "bonds_updated_level1": {"classic": out["c_updated1"], "bond_associated": out["b_updated1"]}}


def fixtures_1_to_4(ref, td, mesh_dir, mesh, man):
    if True:
        ref_mesh = os.path.join(ref, "2D_Hassa_test_mesh.dat")
        man["hassa_mesh_rule_matches_reference"] = filecmp.cmp(mesh, ref_mesh, shallow=False) or bool(
            np.array_equal(np.loadtxt(mesh, skiprows=1), np.loadtxt(ref_mesh, skiprows=1)))
        # 2. + 3. reference main, n1 = n2 = 10, then pin against shipped goldens
        w10 = os.path.join(td, "run10")
        os.makedirs(w10)
        r10 = po.run_ref_hassa(mesh_dir, w10, 10, 10, 1, os.path.join(td, "h10.bin"))
        for name in ("velocity_step_0_after_seq_ref.txt", "LocalParticlesPositions_rank_0step_0.txt"):
            mine = os.path.join(w10, "output", name)
            theirs = os.path.join(ref, "output", name)
            man[f"reference_golden_identical:{name}"] = filecmp.cmp(mine, theirs, shallow=False)
            man[f"sha256:{name}"] = sha(theirs)
        w0 = os.path.join(td, "run0")
        os.makedirs(w0)
        r0 = po.run_ref_hassa(mesh_dir, w0, 0, 0, 3, os.path.join(td, "h0.bin"))
        sets = r0["boundary_sets"]
        np.savez_compressed(
            os.path.join(HERE, "hassa_ref.npz"),
            x=r0["x"], vol=r0["vol"], row_ptr=r0["row_ptr"], col=r0["col"],
            left=sets[0], right=sets[1], bottom=sets[2], top=sets[3],
            c_u1=r0["steps"][1]["u"], c_v1=r0["steps"][1]["v"], c_f1=r0["steps"][1]["f"],
            c_u3=r0["steps"][3]["u"], c_v3=r0["steps"][3]["v"], c_f3=r0["steps"][3]["f"],
            b_v1=r10["steps"][1]["v"], b_f1=r10["steps"][1]["f"],
            params=np.array([1.0, 3.0, 3.5e4, 0.2, 2.5e-6, 1e-9]))  # dx, horizon, E, nu, rho, dt
        man["hassa"] = {"n": int(r0["n"]), "bonds": int(r0["row_ptr"][-1]), "classic_steps": [1, 3],
                        "bond_associated_steps": [1],
                        "params": "dx=1 horizon=3 E=3.5e4 nu=0.2 rho=2.5e-6 dt=1e-9 top v=(0,5) bottom fixed"}
        # 4. seeded 30 x 30 plate
        p = plates.make_plate(30, seed=3, crack="centre-half")
        rp_c, col_c = po.build_families(p.x, p.cutoff, p.cracks)
        prm = {"dx": p.dx, "horizon": 3.015, "E": p.material.E, "nu": p.material.nu, "rho": p.material.rho,
               "dt": p.dt}
        vbc = [(np.nonzero(p.group_of == 1)[0], p.group_val[0]), (np.nonzero(p.group_of == 2)[0], p.group_val[1])]
        # reference findNeighbor families (no crack), 1 step
        fin = os.path.join(td, "p_nocrack.bin")
        po.write_ref_input(fin, p.x, p.vol, prm, 1, families=None, vbc=vbc)
        rn = po.run_ref_plate(fin, os.path.join(td, "p_nocrack.out"))
        # crack-cut families from the restatement, 4 steps
        fin2 = os.path.join(td, "p_crack.bin")
        po.write_ref_input(fin2, p.x, p.vol, prm, 4, families=(rp_c, col_c), vbc=vbc)
        rc = po.run_ref_plate(fin2, os.path.join(td, "p_crack.out"))
        np.savez_compressed(
            os.path.join(HERE, "plate30_ref.npz"),
            nocrack_row_ptr=rn["row_ptr"], nocrack_col=rn["col"],
            row_ptr=rp_c, col=col_c,
            u1=rc["steps"][1]["u"], v1=rc["steps"][1]["v"], f1=rc["steps"][1]["f"],
            u4=rc["steps"][4]["u"], v4=rc["steps"][4]["v"], f4=rc["steps"][4]["f"])
        man["plate30"] = {"generator": "plates.make_plate(30, seed=3, crack='centre-half')", "n": int(p.n),
                          "bonds_with_crack": int(rp_c[-1]), "bonds_reference_findNeighbor": int(rn["row_ptr"][-1]),
                          "steps": [1, 4]}


if __name__ == "__main__":
    main()
