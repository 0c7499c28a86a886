"""The C++ engine's host logic (csrc/engine.cpp: writer and clustering, callable
without a GPU) against the reference engine's own output files (tests/golden/engine,
written by oracle/_ref through ReusableEngine; see tests/golden/make_ref_golden.py).

- The writer reproduces the reference's output text byte for byte from the values
  (pose_writer::consume, writer.cpp:40-81; report_writer, writer.cpp:210-230).
- The pose clustering follows pose_cluster::preprocess (writer.cpp:115-160).
- The FP64 port reproduces the reference's optimize energies (6 printed digits), which
  pins the fixture the GPU engine test compares against.
"""
import csv
import json
import os

import numpy as np
import pytest

import oracle as O
from pxdock_gb300 import abi, model

import _protenix_dock as E

ENG = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "engine")


def leaf_order(aligned, receptor):
    return [aligned[m] for m in receptor.bond_mappings]


@pytest.mark.parametrize("which", ["ref_optimize", "ref_search"])
def test_writer_reproduces_reference_text(tmp_path, which):
    rec = model.Receptor.from_file(os.path.join(ENG, "receptor.json"))
    src = os.path.join(ENG, which, "ligand_out.json")
    d = json.load(open(src))
    poses = [dict(offset=p["offset"], energy=p["energy"], pscore=p["pscore"], nevals=p["nevals"],
                  torsions=leaf_order(p["receptor"]["torsions"], rec), xyz=np.array(p["ligand"]["xyz"]))
             for p in d["poses"]]
    out = E._write_poses(str(tmp_path / "ligand_out.json"), d.get("mapped_smiles", ""),
                         d["best_pose"]["index"], d["best_pose"]["bscore"], poses, rec.bond_mappings,
                         rec.num_rotatable_bonds)
    assert open(out).read() == open(src).read()


def test_evaluate_csv_text():
    src = os.path.join(ENG, "ref_evaluate.csv")
    rows = list(csv.reader(open(src)))
    assert rows[0] == ["ligand_file", "pose_id", "pscore", "bscore"]
    text = "ligand_file,pose_id,pscore,bscore\n" + "".join(
        "%s,%d,%.16g,%.16g\n" % (r[0], int(r[1]), float(r[2]), float(r[3])) for r in rows[1:])
    assert text == open(src).read()


@pytest.mark.parametrize("n_rot", [0, 2, 10, 11])
def test_torsion_rows_and_numbers(tmp_path, n_rot):
    """Receptor torsions in rows of ten, every row but the last ending in ", " (printer.h);
    numbers as std::ostream prints doubles by default."""
    vals = [float(k) + 0.5 for k in range(n_rot)]
    vals[:1] = [-0.0] if n_rot else []
    pose = dict(offset=3, energy=1e-5, pscore=123456789.0, nevals=7, torsions=vals,
                xyz=np.array([[1.0, 2.25, -3.0]]))
    path = E._write_poses(str(tmp_path / "o.json"), "C\\C", 0, -2.5, [pose], list(range(n_rot)), n_rot)
    text = open(path).read()
    assert '"mapped_smiles": "C\\\\C"' in text
    assert '"energy": 1e-05,' in text and '"pscore": 1.23457e+08,' in text
    fmt = ["%g" % v for v in vals]
    rows = [fmt[i:i + 10] for i in range(0, len(fmt), 10)]
    expect = "".join("            " + ", ".join(r) + (",\n" if k < len(rows) - 1 else "\n")
                     for k, r in enumerate(rows))
    # the full rows end with ", " before the newline
    expect = expect.replace(",\n", ", \n")
    assert '"torsions": [\n' + expect + "        ]" in text
    assert '"xyz": [\n          [1, 2.25, -3]\n        ]' in text


def cand(ps, x, nevals=1, off=0):
    return dict(pscore=ps, xyz=np.array(x, float), nevals=nevals, offset=off)


def test_cluster_rules():
    a = [[0, 0, 0]]
    far = lambda k: [[10.0 * k, 0, 0]]
    # failed walkers are skipped; a close pose replaces a worse one; kept sorted
    kept = E._cluster([cand(-1, a, 0), cand(-2, a), cand(-3, [[0.1, 0, 0]]), cand(-5, far(1))], 4, 0.5)
    assert [k["pscore"] for k in kept] == [-5, -3]
    # at num_modes, a better distinct pose replaces the worst
    kept = E._cluster([cand(-1, far(1)), cand(-2, far(2)), cand(-3, far(3))], 2, 0.5)
    assert [k["pscore"] for k in kept] == [-3, -2]
    assert E._cluster([cand(-1, a, 0)], 4, 0.5) == []


def test_port_reproduces_reference_optimize():
    calls = json.load(open(os.path.join(ENG, "calls.json")))
    rec = model.Receptor.from_file(os.path.join(ENG, "receptor.json"))
    lig = model.Ligand.from_file(os.path.join(ENG, "ligand.json"), geometry=False)
    ref = json.load(open(os.path.join(ENG, "ref_optimize", "ligand_out.json")))
    box = model.make_box(calls["box"][:3], calls["box"][3:], calls["spacing"])
    port = O.PortSystem(rec, lig)
    port.build_grid(box, sorted(set(int(t) for t in lig.vdw_type)), nthreads=os.cpu_count() or 1)
    port.set_slope(calls["optimize"]["slope"])
    p = abi.lbfgs_params(max_iter=calls["optimize"]["max_niters"])
    for pose in ref["poses"]:
        r = port.lbfgs(p, np.zeros(rec.n_rotors), lig.poses[pose["offset"]])
        assert "%g" % r["energy"] == "%g" % pose["energy"]
        assert r["nevals"] == pose["nevals"]
