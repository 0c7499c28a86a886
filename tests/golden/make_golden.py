"""Regenerates the golden fixtures in this folder from the reference checkout.

Run here, where the reference exists:  python tests/golden/make_golden.py
It writes
  utest_*.json         the receptor / ligand JSON fixtures that the reference's gtest
                       files embed as raw strings (engine/utest/test_interaction.cpp,
                       test_optimizer.cpp, test_conformer.cpp), unchanged;
  ref_*.npz            answers of the reference engine itself (oracle/_ref, compiled
                       from the reference sources) on seeded synthetic systems, so that
                       the GPU host -- which has no reference checkout -- can pin the
                       port and the CUDA path against the reference's own numbers.
The gtest expected values themselves are restated, with citations, in the tests.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
UTEST = "/root/reference/engine/utest"


def extract(path, tag):
    text = open(os.path.join(UTEST, path)).read()
    blocks = re.findall(r'R"%s\((.*?)\)%s"' % (tag, tag), text, re.S)
    return [json.loads(b) for b in blocks]


def write(name, obj):
    with open(os.path.join(HERE, name), "w") as f:
        json.dump(obj, f, indent=1)
        f.write("\n")


SF_KEYS = ["ligand_ff", "interaction_coulomb_energy_coef", "interaction_vdw_energy_coef",
           "ionic_energy_coef", "pi_cationic_energy_coef", "f2f_pi_stacking_energy_coef",
           "e2f_pi_stacking_energy_coef", "hbond_energy_coef", "hydrophobic_energy_coef",
           "torsion_strain_penalty_coef", "rotatable_energy_coef",
           "molecular_weight_reward_coef", "gbsa_energy_delta_coef",
           "interaction_vdw_energy", "ionic_energy", "pi_cationic_energy",
           "f2f_pi_stacking_energy", "e2f_pi_stacking_energy", "hbond_energy",
           "hydrophobic_energy"]


def scoring_function():
    """The fields of the default scoring-function file that the engine reads
    (factory.cpp:144-202): term weights and term parameters."""
    src = json.load(open("/root/reference/pxdock/data/pscore-v7_and_bscore-fake.json"))
    out = {}
    for section in ("pose_selection", "affinity_ranking"):
        out[section] = {k: v for k, v in src[section].items() if k in SF_KEYS}
        # terms whose parameter blocks the engine reads but ignores (factory.cpp:136-142)
        for k in ("interaction_coulomb_energy", "torsion_strain_penalty", "rotatable_energy",
                  "molecular_weight_reward", "gbsa_energy_delta"):
            if k in src[section]:
                out[section][k] = {}
    write("scoring_function.json", out)


def fixtures():
    rec_int = extract("test_interaction.cpp", "receptor_json")[0]
    lig_int = extract("test_interaction.cpp", "ligand_json")[0]
    rec_opt = extract("test_optimizer.cpp", "receptor_json")[0]
    lig_opt = extract("test_optimizer.cpp", "ligand_json")[0]
    lig_conf = extract("test_conformer.cpp", "ligand_json")[0]
    rec_conf = extract("test_conformer.cpp", "receptor_json")[0]
    write("utest_interaction_receptor.json", rec_int)
    write("utest_interaction_ligand.json", lig_int)
    write("utest_optimizer_receptor.json", rec_opt)
    write("utest_optimizer_ligand.json", lig_opt)
    write("utest_conformer_ligand.json", lig_conf)
    write("utest_conformer_receptor.json", rec_conf)
    scoring_function()


if __name__ == "__main__":
    fixtures()
    if "--fixtures-only" not in sys.argv:
        sys.path.insert(0, HERE)
        import make_ref_golden  # noqa: E402

        make_ref_golden.main()
