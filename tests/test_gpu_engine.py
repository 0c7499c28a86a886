"""The GB300 `_protenix_dock.ReusableEngine` on the reference engine's own inputs and
outputs (tests/golden/engine, written by oracle/_ref).

- evaluate: every pose's pscore / bscore within 1e-3 + 1e-5 |s| of the reference's;
- optimize: the reference's schema and pose order; every energy and score is the FP64
  value at the returned pose (|dE| <= 1e-3); the final energies of the 30-iteration runs
  from the same starts differ from the reference's by no more than the FP64 port's own
  final energies do when its starts move by FP32 rounding (+ 1e-3 kcal/mol);
- search: schema, at most num_modes poses sorted by pose score, poses inside the box,
  every energy / score the FP64 value at the pose; the best pose score no worse than the
  FP64 port's walkers (from the same and from FP32-rounded starts) by more than 1 kcal/mol;
- dump_maps / load_maps round trip through the reference's cache files (.bdg + meta.dat)
  and restore's errors; the reference's precondition errors.
"""
import csv
import json
import os
import shutil

import numpy as np
import pytest

import oracle as O
from pxdock_gb300 import abi, mapcache, model

import _protenix_dock as E

pytestmark = pytest.mark.gpu

ENG = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "engine")
SF = os.path.join(ENG, "scoring_function.json")


@pytest.fixture(scope="module")
def setup(tmp_path_factory):
    d = tmp_path_factory.mktemp("engine")
    for f in ("receptor.json", "ligand.json"):
        shutil.copy(os.path.join(ENG, f), d / f)
    (d / "index.txt").write_text(str(d / "ligand.json") + "\n")
    calls = json.load(open(os.path.join(ENG, "calls.json")))
    rec = model.Receptor.from_file(os.path.join(ENG, "receptor.json"))
    lig = model.Ligand.from_file(os.path.join(ENG, "ligand.json"))
    pose_sf, aff_sf = model.load_scoring_function(SF)
    port = O.PortSystem(rec, lig)
    box = model.make_box(calls["box"][:3], calls["box"][3:], calls["spacing"])
    port.build_grid(box, sorted(set(int(t) for t in lig.vdw_type)), nthreads=os.cpu_count() or 1)
    port.set_slope(1e6)
    eng = E.ReusableEngine(str(d / "receptor.json"), SF)
    eng.set_box(*calls["box"])
    return dict(dir=d, calls=calls, rec=rec, lig=lig, port=port, sf=(pose_sf, aff_sf), eng=eng, box=box)


def consistent(s, p):
    t = np.asarray([p["receptor"]["torsions"][m] for m in s["rec"].bond_mappings])
    x = np.asarray(p["ligand"]["xyz"])
    e, _, _ = s["port"].score_grad(t, x)
    assert abs(p["energy"] - e) <= 1e-3 + 1e-5 * abs(e), (p["energy"], e)
    ps, _ = s["port"].score(s["sf"][0], s["port"].receptor_apply(t), x)
    assert abs(p["pscore"] - ps) <= 1e-3 + 1e-5 * abs(ps) + 5e-6 * abs(p["pscore"])
    return t, x


def test_evaluate_matches_reference(setup):
    s = setup
    out = str(s["dir"] / "eval.csv")
    s["eng"].evaluate(str(s["dir"] / "index.txt"), out)
    ours = list(csv.reader(open(out)))
    ref = list(csv.reader(open(os.path.join(ENG, "ref_evaluate.csv"))))
    assert ours[0] == ref[0] and len(ours) == len(ref)
    for a, b in zip(ours[1:], ref[1:]):
        assert a[:2] == b[:2]
        for k in (2, 3):
            assert abs(float(a[k]) - float(b[k])) <= 1e-3 + 1e-5 * abs(float(b[k])), (a, b)


def test_optimize_matches_reference(setup):
    s = setup
    s["eng"].generate_maps(s["calls"]["spacing"])
    out = s["dir"] / "opt"
    s["eng"].optimize(str(s["dir"] / "index.txt"), str(out), **s["calls"]["optimize"])
    ours = json.load(open(out / "ligand_out.json"))
    ref = json.load(open(os.path.join(ENG, "ref_optimize", "ligand_out.json")))
    assert list(ours) == list(ref)
    assert [p["offset"] for p in ours["poses"]] == [p["offset"] for p in ref["poses"]]
    # the FP64 port reproduces the reference's runs from the same starts; the control is the
    # port from the starts moved by FP32 rounding and 1e-6 A (four draws): the spread of
    # final energies that input precision alone causes after these iterations
    pp = abi.lbfgs_params(max_iter=s["calls"]["optimize"]["max_niters"])
    R = s["rec"].n_rotors
    rng = np.random.default_rng(3)
    for a, b in zip(ours["poses"], ref["poses"]):
        assert list(a) == list(b)
        consistent(s, a)
        assert a["nevals"] > 0
        x0 = s["lig"].poses[a["offset"]]
        same = s["port"].lbfgs(pp, np.zeros(R), x0)["energy"]
        # (the fixture's numbers carry six significant digits)
        assert abs(same - b["energy"]) <= 1e-5 * max(1.0, abs(b["energy"])), (same, b["energy"])
        spread = max(abs(s["port"].lbfgs(pp, np.zeros(R), x0.astype(np.float32).astype(np.float64) +
                                         rng.normal(scale=1e-6, size=x0.shape))["energy"] - b["energy"])
                     for _ in range(4))
        print("optimize pose %d: gpu %.6f ref %.6f control spread %.6f" % (a["offset"], a["energy"], b["energy"],
                                                                           spread))
        assert abs(a["energy"] - b["energy"]) <= spread + 1e-3 + 1e-5 * abs(b["energy"]), \
            (a["energy"], b["energy"], spread)
    best = ours["poses"][ours["best_pose"]["index"]]
    assert best["pscore"] == min(p["pscore"] for p in ours["poses"])


def test_search_outputs(setup):
    s = setup
    out = s["dir"] / "search"
    args = s["calls"]["search"]
    s["eng"].search(str(s["dir"] / "index.txt"), str(out), **args)
    ours = json.load(open(out / "ligand_out.json"))
    ref = json.load(open(os.path.join(ENG, "ref_search", "ligand_out.json")))
    assert list(ours) == list(ref)
    assert 1 <= len(ours["poses"]) <= args["num_modes"]
    ps = [p["pscore"] for p in ours["poses"]]
    assert ps == sorted(ps) and ours["best_pose"]["index"] == 0
    lo = np.array(s["box"].init_xyz)
    hi = lo + (np.array(s["box"].npoints) - 1) * s["box"].spacing
    for p in ours["poses"]:
        t, x = consistent(s, p)
        assert np.all(x > lo) and np.all(x < hi)
    t, x = consistent(s, ours["poses"][0])
    bs, _ = s["port"].score(s["sf"][1], s["port"].receptor_apply(t), x)
    assert abs(ours["best_pose"]["bscore"] - bs) <= 1e-3 + 1e-5 * abs(bs)
    # best pose score: the FP64 port's walkers reproduce the reference's best; the GPU's best
    # is no worse than both that and the port's walkers from FP32-rounded starts by more
    # than 1 kcal/mol (Monte-Carlo trajectories diverge at the first different acceptance,
    # so the bar is on the search's outcome, not on equality)
    x0 = s["lig"].poses[0]
    walk = lambda start: min(
        r["pscore"] for r in (s["port"].mc_walker(s["sf"][0], lo, hi, args["seed"], w, start, True, args["max_nsteps"],
                                                  args["relax_nsteps"], args["mc_mmenergy_threshold"])
                              for w in range(args["exhaustiveness"])) if r["nevals"] > 0)
    ref_best = ref["poses"][0]["pscore"]
    port_best = walk(x0)
    ctl_best = walk(x0.astype(np.float32).astype(np.float64))
    print("search best pscore: gpu %.4f ref %.4f port %.4f control %.4f" % (ps[0], ref_best, port_best, ctl_best))
    assert abs(port_best - ref_best) <= 1e-5 * max(1.0, abs(ref_best)), (port_best, ref_best)
    assert ps[0] <= max(ref_best, ctl_best) + 1.0, (ps[0], ref_best, ctl_best)


def test_optimize_rigid_body_torsion_mode(setup):
    """optimize(..., dof_mode=1): the reference's schema; every energy the FP64 value at its
    pose; each pose keeps its input bond lengths (to FP32 precision) and lowers its energy;
    the next default call is the reference's Cartesian mode again."""
    s = setup
    idx = str(s["dir"] / "index.txt")
    out = s["dir"] / "opt_dof"
    s["eng"].optimize(idx, str(out), max_niters=60, dof_mode=1)
    ours = json.load(open(out / "ligand_out.json"))
    ref = json.load(open(os.path.join(ENG, "ref_optimize", "ligand_out.json")))
    assert list(ours) == list(ref)
    b = s["lig"].ff.bonds
    R = s["rec"].n_rotors
    for p in ours["poses"]:
        t, x = consistent(s, p)
        x0 = s["lig"].poses[p["offset"]]
        d0 = np.linalg.norm(x0[b[:, 0]] - x0[b[:, 1]], axis=-1)
        d1 = np.linalg.norm(x[b[:, 0]] - x[b[:, 1]], axis=-1)
        assert np.max(np.abs(d1 - d0)) <= 1e-4
        e0, _, _ = s["port"].score_grad(np.zeros(R), x0)
        assert p["energy"] < e0
    with pytest.raises(RuntimeError, match="dof_mode"):
        s["eng"].optimize(idx, str(s["dir"] / "opt_bad"), max_niters=5, dof_mode=2)
    cart = s["dir"] / "opt_cart"
    s["eng"].optimize(idx, str(cart), max_niters=5)
    moved = []
    for p in json.load(open(cart / "ligand_out.json"))["poses"]:
        x, x0 = np.asarray(p["ligand"]["xyz"]), s["lig"].poses[p["offset"]]
        moved.append(np.max(np.abs(np.linalg.norm(x[b[:, 0]] - x[b[:, 1]], axis=-1) -
                                   np.linalg.norm(x0[b[:, 0]] - x0[b[:, 1]], axis=-1))))
    assert max(moved) > 1e-3  # Cartesian steps stretch bonds


def test_maps_round_trip(setup):
    """dump_maps writes the reference's cache (a <tag>.bdg per ligand type, coul.bdg,
    meta.dat); a second engine loads it and optimises to the same file."""
    s = setup
    cache = s["dir"] / "maps"
    s["eng"].dump_maps(str(cache))
    names = os.listdir(cache)
    assert "meta.dat" in names and "coul.bdg" in names and "c.bdg" in names
    assert len([n for n in names if n.endswith(".bdg")]) == 100
    meta = mapcache.decode_meta((cache / "meta.dat").read_text())
    assert meta["version"] == mapcache.FORMAT_VERSION and meta["spacing"] == s["calls"]["spacing"]
    movable = {a for (_, axis), g in zip(s["rec"].rotor_axis, s["rec"].rotor_groups) for a in g if a != axis}
    assert sorted(meta["excluded"]) == sorted(movable) and movable
    rec, vb = mapcache.decode_bdg((cache / "coul.bdg").read_bytes())
    assert vb == 8 and rec.shape[0] == int(np.prod(meta["npoints"]))
    a = s["dir"] / "opt_a"
    s["eng"].optimize(str(s["dir"] / "index.txt"), str(a), max_niters=10)
    other = E.ReusableEngine(str(s["dir"] / "receptor.json"), SF)
    other.load_maps(str(cache))
    b = s["dir"] / "opt_b"
    other.optimize(str(s["dir"] / "index.txt"), str(b), max_niters=10)
    assert (a / "ligand_out.json").read_text() == (b / "ligand_out.json").read_text()
    # dumped again from the loaded maps: the same bytes
    again = s["dir"] / "maps_again"
    other.dump_maps(str(again))
    for n in ("coul.bdg", "c.bdg", "sq.bdg", "meta.dat"):
        assert (again / n).read_bytes() == (cache / n).read_bytes(), n


def test_map_cache_errors(setup):
    """receptor_cache::restore's messages (grid.cpp:347-431)."""
    s = setup
    src = s["dir"] / "maps_err_src"
    s["eng"].dump_maps(str(src))
    eng = E.ReusableEngine(str(s["dir"] / "receptor.json"), SF)
    bad = s["dir"] / "maps_err"
    shutil.copytree(src, bad)
    (bad / "meta.dat").write_text((src / "meta.dat").read_text().replace(" 20241030 ", " 20240101 "))
    with pytest.raises(RuntimeError, match=r"Format version of map files are not compatible! "
                                           r"Expected \[20241030\] vs. Got \[20240101\]"):
        eng.load_maps(str(bad))
    shutil.copy(src / "meta.dat", bad / "meta.dat")
    os.remove(bad / "cl.bdg")
    with pytest.raises(RuntimeError, match=r"Map file for atom type \[cl\] is missing!"):
        eng.load_maps(str(bad))
    os.remove(bad / "meta.dat")
    with pytest.raises(RuntimeError, match="The metadata file of maps is missing!"):
        eng.load_maps(str(bad))


def test_precondition_errors(setup):
    s = setup
    eng = E.ReusableEngine(str(s["dir"] / "receptor.json"), SF)
    with pytest.raises(RuntimeError, match="set_box"):
        eng.generate_maps(0.5)
    with pytest.raises(RuntimeError, match="set_box"):
        eng.search(str(s["dir"] / "index.txt"), str(s["dir"] / "x"))
    with pytest.raises(RuntimeError):
        eng.dump_maps(str(s["dir"] / "y"))
    with pytest.raises(RuntimeError):
        E.ReusableEngine(str(s["dir"] / "missing.json"), SF)
    assert E.version()
