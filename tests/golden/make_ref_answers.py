"""Answers of the reference engine itself (oracle/_ref, compiled from the reference
sources) on the committed engine fixture (tests/golden/engine/receptor.json and
ligand.json), so that hosts without the reference checkout still pin the FP64 port to
the reference: tests/test_oracle_golden.py replays every input below on the port.

Run where oracle/_ref exists:  python tests/golden/make_ref_answers.py
Writes tests/golden/ref_answers.npz: the inputs (coordinates, torsions, rotations,
RNG draw kinds) and the reference's outputs for
  - ligand and receptor forward kinematics   (free_ligand / torsional_receptor::apply_parameters)
  - brute-force and grid score + gradient     (binding_system_interactions::put_gradients)
  - two maps of the grid build               (receptor_cache::populate)
  - L-BFGS trajectories, reference constants  (lbfgs_step::apply)
  - pose-selection and affinity scores        (root_scorer::combine)
  - Monte-Carlo walker 0                      (monte_carlo_searcher)
  - mt19937 draw streams                      (random_generator)
"""
import json
import math
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(REPO, "protenix-dock_gb300"), os.path.join(REPO, "oracle")]

import ctypes as C  # noqa: E402

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from pxdock_gb300 import abi, model, synth  # noqa: E402

ENGINE = os.path.join(HERE, "engine")
OUT = os.path.join(HERE, "ref_answers.npz")
GRID = dict(center=(0.0, 0.0, 0.0), size=(8.0, 8.0, 8.0), spacing=1.0)
RNG_SEEDS = (0, 7, 12345)
RNG_DRAWS = 300


def padded_sf_path(tmp):
    """The scoring function with the affinity vdW scale list padded to 99 types (the
    reference reads past the shipped 38 entries)."""
    sf = json.load(open(os.path.join(HERE, "scoring_function.json")))
    for sec in sf.values():
        types = sec.get("interaction_vdw_energy", {}).get("types")
        if types is not None:
            types.extend({"sigma_scale": 1.0, "epsilon_scale": 1.0} for _ in range(99 - len(types)))
    path = os.path.join(tmp, "sf.json")
    json.dump(sf, open(path, "w"))
    return path


def rng_draws_ref(seed):
    """RNG_DRAWS mixed draws (int, torsion, orientation, in-sphere, real) from the
    reference generator, flattened."""
    rl = oracle.ref_lib()
    h = rl.ref_rng_create(seed)
    out = []
    for k in range(RNG_DRAWS):
        op = k % 5
        if op == 0:
            out.append(float(rl.ref_rng_uniform_int(h, 0, 6)))
        elif op == 1:
            out.append(rl.ref_rng_torsion(h))
        elif op == 2:
            y = np.zeros(4)
            rl.ref_rng_orientation(h, y.ctypes.data_as(abi.f64p))
            out.extend(y.tolist())
        elif op == 3:
            y = np.zeros(3)
            rl.ref_rng_in_sphere(h, y.ctypes.data_as(abi.f64p))
            out.extend(y.tolist())
        else:
            out.append(rl.ref_rng_uniform_real(h, -2.0, 5.0))
    rl.ref_rng_destroy(h)
    return np.array(out)


def main():
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref is not built: run make -C oracle ref first")
    rp, lp = os.path.join(ENGINE, "receptor.json"), os.path.join(ENGINE, "ligand.json")
    rec, lig = model.Receptor.from_file(rp), model.Ligand.from_file(lp)
    ref = oracle.RefSystem(rp, lp)
    x0 = lig.poses[0]
    R = rec.n_rotors
    out = {}
    rng = np.random.default_rng(21)
    # kinematics
    q = synth.random_quaternions(rng, 5)
    out["kin_rot"] = synth.quaternion_matrix(q)
    out["kin_center"] = rng.normal(size=(5, 3))
    out["kin_tors"] = rng.uniform(-math.pi, math.pi, size=(5, lig.n_torsions))
    out["kin_xyz"] = np.stack([ref.ligand_apply(x0, c, m, t) for c, m, t in
                               zip(out["kin_center"], out["kin_rot"], out["kin_tors"])])
    out["rec_tors"] = rng.uniform(-3, 3, size=(2, R))
    out["rec_xyz"] = np.stack([ref.receptor_apply(t) for t in out["rec_tors"]])
    # brute-force score + gradient
    ref.drop_grid()
    bx = np.stack([x0 + rng.normal(scale=0.2, size=x0.shape) for _ in range(3)])
    bt = rng.uniform(-3, 3, size=(3, R))
    res = [ref.score_grad(t, x) for t, x in zip(bt, bx)]
    out["bf_xyz"], out["bf_tors"] = bx, bt
    out["bf_e"] = np.array([r[0] for r in res])
    out["bf_tg"] = np.stack([r[1] for r in res])
    out["bf_lg"] = np.stack([r[2] for r in res])
    # grid build and grid score + gradient (slope 0 and 1e6)
    ref.build_grid(GRID["center"], GRID["size"], GRID["spacing"])
    types = sorted(set(int(t) for t in lig.vdw_type))
    out["map_ids"] = np.array([abi.COULOMB_MAP, types[0]], np.int32)
    out["maps"] = np.stack([ref.grid_map(int(m)) for m in out["map_ids"]])
    gx = np.stack([x0 + rng.normal(scale=1.5, size=x0.shape) for _ in range(4)])
    gt = rng.uniform(-3, 3, size=(4, R))
    out["grid_xyz"], out["grid_tors"] = gx, gt
    for name, slope in (("s0", 0.0), ("s6", 1e6)):
        ref.set_slope(slope)
        res = [ref.score_grad(t, x) for t, x in zip(gt, gx)]
        out["grid_e_" + name] = np.array([r[0] for r in res])
        out["grid_tg_" + name] = np.stack([r[1] for r in res])
        out["grid_lg_" + name] = np.stack([r[2] for r in res])
    # L-BFGS at the reference constants (m = 100, tol_grad 0.5), 60 iterations, slope 1e6
    ref.set_slope(1e6)
    lx = np.stack([x0 + rng.normal(scale=0.3, size=x0.shape) for _ in range(3)])
    lt = rng.uniform(-1, 1, size=(3, R))
    res = [ref.lbfgs(60, 0, t, x) for t, x in zip(lt, lx)]
    out["lbfgs_xyz0"], out["lbfgs_tors0"] = lx, lt
    out["lbfgs_nevals"] = np.array([r["nevals"] for r in res], np.int32)
    out["lbfgs_converged"] = np.array([r["converged"] for r in res], np.int32)
    out["lbfgs_e"] = np.array([r["energy"] for r in res])
    out["lbfgs_xyz"] = np.stack([r["xyz"] for r in res])
    out["lbfgs_tors"] = np.stack([r["torsions"] for r in res])
    # scores, then walker 0 of a short search
    with tempfile.TemporaryDirectory() as tmp:
        ref.load_sf(padded_sf_path(tmp))
    sx = np.stack([x0 + rng.normal(scale=0.5, size=x0.shape) for _ in range(4)])
    st = rng.uniform(-2, 2, size=(4, R))
    out["score_xyz"], out["score_tors"] = sx, st
    vals, terms = [], []
    for x, t in zip(sx, st):
        rx = ref.receptor_apply(t)
        for which in (0, 1):
            v, tr = ref.score(which, rx, x)
            vals.append(v)
            terms.append(tr)
    out["score_v"] = np.array(vals).reshape(4, 2)
    out["score_terms"] = np.stack(terms).reshape(4, 2, -1)
    w = ref.mc_walker(7, 0, 12, 15)
    out["mc_xyz"], out["mc_pscore"] = w["xyz"], np.array(w["pscore"])
    out["mc_nevals"], out["mc_energy"] = np.array(w["nevals"]), np.array(w["energy"])
    # generator streams
    out["rng_seeds"] = np.array(RNG_SEEDS, np.int64)
    out["rng_draws"] = np.stack([rng_draws_ref(s) for s in RNG_SEEDS])
    ref.close()
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
