"""Generate the golden fixtures in tests/golden/ from the reference's OWN code.

Run here, where the reference checkout exists (it does not exist on the GPU
machine, which only reads the committed .npz files):

    make -C oracle ref oracle
    python tests/golden/make_golden.py [--reference /root/reference]

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


def hassa_mesh_lines():
    """The Hassa mesh file content by rule (x outer loop, y inner)."""
    lines = ["Center_X Center_Y Area"]
    for ix in range(70):
        for iy in range(60):
            lines.append(f"{ix - 34.5:.6f} {iy - 29.5:.6f} {1.0:.6f}")
    return "\n".join(lines) + "\n"


def sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    ap.add_argument("--only", choices=["mazars"], default=None)
    args = ap.parse_args()
    ref = args.reference
    if not po.ref_available():
        sys.exit("build the reference oracle first: make -C oracle ref")
    man_path = os.path.join(HERE, "manifest.json")
    man = json.load(open(man_path)) if args.only and os.path.exists(man_path) else {}
    with tempfile.TemporaryDirectory() as td:
        # 1. mesh by rule
        mesh_dir = os.path.join(td, "mesh")
        os.makedirs(mesh_dir)
        mesh = os.path.join(mesh_dir, "2D_Hassa_test_mesh.dat")
        open(mesh, "w").write(hassa_mesh_lines())
        if args.only != "mazars":
            fixtures_1_to_4(ref, td, mesh_dir, mesh, man)
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
    json.dump(man, open(man_path, "w"), indent=1, sort_keys=True)
    print(json.dumps(man, indent=1, sort_keys=True))
    bad = [k for k, v in man.items() if v is False]
    if bad:
        sys.exit(f"pinning failed: {bad}")


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
