"""The FP64 port against the reference engine's own answers, committed as a fixture.

tests/golden/ref_answers.npz holds the inputs and outputs of the reference engine
(compiled from its sources as oracle/_ref) on the committed engine fixture system; it is
written by tests/golden/make_ref_answers.py. This test replays the same inputs on the
port, so the port stays pinned to the reference on hosts without the reference
checkout. Where the checkout exists, test_oracle_vs_ref.py compares the two live.
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

import oracle as O
from pxdock_gb300 import abi, model


@pytest.fixture(scope="module")
def fixture(golden):
    ans = np.load(os.path.join(golden, "ref_answers.npz"))
    eng = os.path.join(golden, "engine")
    rec = model.Receptor.from_file(os.path.join(eng, "receptor.json"))
    lig = model.Ligand.from_file(os.path.join(eng, "ligand.json"))
    return ans, rec, lig, O.PortSystem(rec, lig)


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / max(1.0, np.max(np.abs(b)))


def grid_box():
    return model.make_box((0.0, 0.0, 0.0), (8.0, 8.0, 8.0), 1.0)


def test_kinematics(fixture):
    ans, rec, lig, port = fixture
    for c, m, t, want in zip(ans["kin_center"], ans["kin_rot"], ans["kin_tors"], ans["kin_xyz"]):
        assert rel(port.ligand_apply(lig.poses[0], c, m, t), want) < 1e-13
    for t, want in zip(ans["rec_tors"], ans["rec_xyz"]):
        assert rel(port.receptor_apply(t), want) < 1e-13


def test_score_grad_brute_force(fixture):
    ans, rec, lig, port = fixture
    port.drop_grid()
    for i in range(len(ans["bf_e"])):
        e, tg, lg = port.score_grad(ans["bf_tors"][i], ans["bf_xyz"][i])
        assert abs(e - ans["bf_e"][i]) <= 1e-12 * max(1.0, abs(ans["bf_e"][i]))
        assert rel(lg, ans["bf_lg"][i]) < 1e-12 and rel(tg, ans["bf_tg"][i]) < 1e-12


def test_grid_maps_and_score(fixture):
    ans, rec, lig, port = fixture
    box = grid_box()
    port.build_grid(box, sorted(set(int(t) for t in lig.vdw_type)))
    for m, want in zip(ans["map_ids"], ans["maps"]):
        assert rel(port.grid_map(int(m), box), want) < 1e-13, m
    for name, slope in (("s0", 0.0), ("s6", 1e6)):
        port.set_slope(slope)
        for i in range(len(ans["grid_xyz"])):
            e, tg, lg = port.score_grad(ans["grid_tors"][i], ans["grid_xyz"][i])
            want = ans["grid_e_" + name][i]
            assert abs(e - want) <= 1e-12 * max(1.0, abs(want))
            assert rel(lg, ans["grid_lg_" + name][i]) < 1e-12
            assert rel(tg, ans["grid_tg_" + name][i]) < 1e-12


def test_lbfgs_trajectories(fixture):
    ans, rec, lig, port = fixture
    port.build_grid(grid_box(), sorted(set(int(t) for t in lig.vdw_type)))
    port.set_slope(1e6)
    for i in range(len(ans["lbfgs_e"])):
        a = port.lbfgs(abi.lbfgs_params(max_iter=60), ans["lbfgs_tors0"][i], ans["lbfgs_xyz0"][i])
        assert a["nevals"] == ans["lbfgs_nevals"][i]
        assert (a["status"] == abi.POSE_CONVERGED) == bool(ans["lbfgs_converged"][i])
        assert abs(a["energy"] - ans["lbfgs_e"][i]) <= 1e-9 * max(1.0, abs(ans["lbfgs_e"][i]))
        assert rel(a["xyz"], ans["lbfgs_xyz"][i]) < 1e-9
        assert rel(a["torsions"], ans["lbfgs_tors"][i]) < 1e-9


def padded_sf(golden, tmp_path):
    sf = json.load(open(os.path.join(golden, "scoring_function.json")))
    for sec in sf.values():
        types = sec.get("interaction_vdw_energy", {}).get("types")
        if types is not None:
            types.extend({"sigma_scale": 1.0, "epsilon_scale": 1.0} for _ in range(99 - len(types)))
    path = str(tmp_path / "sf.json")
    json.dump(sf, open(path, "w"))
    return model.load_scoring_function(path)


def test_scores_and_walker(fixture, golden, tmp_path):
    ans, rec, lig, port = fixture
    pose_sf, aff_sf = padded_sf(golden, tmp_path)
    for i in range(len(ans["score_xyz"])):
        rx = port.receptor_apply(ans["score_tors"][i])
        for which, sf in ((0, pose_sf), (1, aff_sf)):
            v, terms = port.score(sf, rx, ans["score_xyz"][i])
            want = ans["score_v"][i, which]
            assert abs(v - want) <= 1e-10 * max(1.0, abs(want)), (i, which, v, want)
            for k in (0, 1, 2, 3, 4, 5, 6, 7, 8, 10):
                w = ans["score_terms"][i, which, k]
                if w != 0.0:
                    assert abs(terms[k] - w) <= 1e-10 * max(1.0, abs(w)), (i, which, k)
    box = grid_box()
    port.build_grid(box, sorted(set(int(t) for t in lig.vdw_type)))
    port.set_slope(1e6)
    lo = np.array(box.init_xyz)
    hi = lo + (np.array(box.npoints) - 1) * box.spacing
    w = port.mc_walker(pose_sf, lo, hi, 7, 0, lig.poses[0], True, 12, 15)
    assert w["nevals"] == int(ans["mc_nevals"])
    assert rel(w["xyz"], ans["mc_xyz"]) < 1e-6
    assert abs(w["pscore"] - float(ans["mc_pscore"])) <= 1e-6 * max(1.0, abs(float(ans["mc_pscore"])))


def test_rng_streams(fixture):
    ans = fixture[0]
    lib = O.port_lib()

    class Rng(C.Structure):
        _fields_ = [("mt", C.c_uint32 * 624), ("idx", C.c_int)]

    for seed, want in zip(ans["rng_seeds"], ans["rng_draws"]):
        r = Rng()
        lib.po_rng_seed(C.byref(r), int(seed))
        got = []
        for k in range(300):
            op = k % 5
            if op == 0:
                got.append(float(lib.po_rng_uniform_int(C.byref(r), 0, 6)))
            elif op == 1:
                got.append(lib.po_rng_torsion(C.byref(r)))
            elif op == 2:
                x = np.zeros(4)
                lib.po_rng_orientation(C.byref(r), x.ctypes.data_as(abi.f64p))
                got.extend(x.tolist())
            elif op == 3:
                x = np.zeros(3)
                lib.po_rng_in_sphere(C.byref(r), x.ctypes.data_as(abi.f64p))
                got.extend(x.tolist())
            else:
                got.append(lib.po_rng_uniform_real(C.byref(r), -2.0, 5.0))
        np.testing.assert_array_equal(np.array(got), want)
