"""Answers of the reference engine itself (oracle/_ref, compiled from the reference
sources) on a small seeded docking system, for the engine-level tests on hosts that
have no reference checkout.

Run where oracle/_ref exists:  python tests/golden/make_ref_golden.py
Writes tests/golden/engine/: the inputs (receptor.json, ligand.json, index.txt,
scoring_function.json) and
the reference's outputs of ReusableEngine.evaluate (ref_evaluate.csv),
ReusableEngine.optimize (ref_optimize/ligand_out.json) and ReusableEngine.search
(ref_search/ligand_out.json), with the calls' arguments in calls.json.
"""
import json
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(REPO, "protenix-dock_gb300"), os.path.join(REPO, "oracle")]

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from pxdock_gb300 import synth  # noqa: E402

OUT = os.path.join(HERE, "engine")
CALLS = {
    "box": [0.0, 0.0, 0.0, 12.0, 12.0, 12.0],
    "spacing": 0.5,
    "optimize": {"max_niters": 30, "slope": 1e6},
    "search": {"seed": 5, "exhaustiveness": 6, "max_nsteps": 3, "relax_nsteps": 5, "num_modes": 4,
               "min_rmsd": 0.5, "mc_mmenergy_threshold": -1.0, "slope": 1e6},
}


def inputs():
    rec = synth.make_receptor(seed=0, n_heavy=300, cube=18.0, cavity=6.0, n_rotors=2)
    lig = synth.make_ligand(seed=1)
    rng = np.random.default_rng(4)
    x0 = np.array(lig["xyz"][0])
    lig["xyz"] = [x0.round(4).tolist()] + [(x0 + rng.normal(scale=0.3, size=x0.shape)).round(4).tolist()
                                           for _ in range(2)]
    return rec, lig


def main():
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref is not built: run make -C oracle ref first")
    if os.path.isdir(OUT):
        shutil.rmtree(OUT)
    os.makedirs(OUT)
    rec, lig = inputs()
    rp, lp = os.path.join(OUT, "receptor.json"), os.path.join(OUT, "ligand.json")
    json.dump(rec, open(rp, "w"))
    json.dump(lig, open(lp, "w"))
    with open(os.path.join(OUT, "index.txt"), "w") as f:
        f.write("ligand.json\n")
    json.dump(CALLS, open(os.path.join(OUT, "calls.json"), "w"), indent=1)
    # the shipped affinity function lists vdW scales for 38 ligand types; the reference
    # reads past that list for higher types, so the engine fixture pads it with scale 1
    sfd = json.load(open(os.path.join(HERE, "scoring_function.json")))
    for sec in sfd.values():
        types = sec.get("interaction_vdw_energy", {}).get("types")
        if types is not None:
            types.extend({"sigma_scale": 1.0, "epsilon_scale": 1.0} for _ in range(99 - len(types)))
    sf = os.path.join(OUT, "scoring_function.json")
    json.dump(sfd, open(sf, "w"))
    lib = oracle.ref_lib()
    cwd = os.getcwd()
    os.chdir(OUT)  # the index file names ligand.json relative to here
    try:
        h = lib.ref_engine_create(b"receptor.json", sf.encode(), 1)
        lib.ref_engine_set_box(h, *CALLS["box"])
        assert lib.ref_engine_evaluate(h, b"index.txt", b"ref_evaluate.csv") == 0
        assert lib.ref_engine_generate_maps(h, CALLS["spacing"], 0.0) == 0
        o = CALLS["optimize"]
        assert lib.ref_engine_optimize(h, b"index.txt", b"ref_optimize", o["max_niters"], o["slope"]) == 0
        s = CALLS["search"]
        assert lib.ref_engine_search(h, b"index.txt", b"ref_search", s["seed"], s["exhaustiveness"],
                                     s["max_nsteps"], s["relax_nsteps"], s["num_modes"], s["min_rmsd"],
                                     s["mc_mmenergy_threshold"], s["slope"]) == 0
        lib.ref_engine_destroy(h)
    finally:
        os.chdir(cwd)


if __name__ == "__main__":
    main()
