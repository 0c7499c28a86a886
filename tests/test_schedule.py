"""Host scheduling of the force-field terms into conflict-free rounds of 32 lanes
(protenix-dock_gb300/csrc/schedule.h), compiled here with g++ and checked on the
synthetic ligands: every term exactly once, per round and term position no atom
twice, reversed terms listed reversed, and the round counts the device relies on."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from pxdock_gb300 import model, synth

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "protenix-dock_gb300", "csrc")
REV = 1 << 30


@pytest.fixture(scope="module")
def scheduler(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("sched") / "schedule")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "native", "schedule_main.cpp"),
                    "-o", exe], check=True)

    def run(terms, n_atoms, K=None):
        terms = np.asarray(terms, np.int64).reshape(len(terms), K or -1)
        K = terms.shape[1]
        text = "%d %d %d\n" % (K, n_atoms, len(terms)) + "\n".join(" ".join(map(str, t)) for t in terms)
        out = subprocess.run([exe], input=text, capture_output=True, text=True, check=True).stdout
        return [int(v) for v in out.split()]

    return run


def check(schedule, terms, n_atoms):
    terms = np.asarray(terms).reshape(len(terms), -1)
    assert len(schedule) % 32 == 0
    seen = np.zeros(len(terms), int)
    for r in range(0, len(schedule), 32):
        used = set()
        for s in schedule[r:r + 32]:
            if s < 0:
                continue
            t = s & ~REV
            seen[t] += 1
            atoms = terms[t][::-1] if s & REV else terms[t]
            for k, a in enumerate(atoms):
                assert (k, int(a)) not in used, (r // 32, k, a)
                used.add((k, int(a)))
    assert np.all(seen == 1)
    return len(schedule) // 32


def ligand_terms(lig):
    f = lig.ff
    dih = np.concatenate([np.asarray(f.propers[0]).reshape(-1, 4), np.asarray(f.impropers[0]).reshape(-1, 4)])
    pairs = np.concatenate([f.pairs14.reshape(-1, 2), f.pairs.reshape(-1, 2)])
    return dict(bonds=f.bonds, angles=f.angles, dih=dih, pairs=pairs)


def test_config0_ligand_rounds(scheduler):
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    t = ligand_terms(lig)
    rounds = {k: check(scheduler(v, lig.n_atoms), v, lig.n_atoms) for k, v in t.items()}
    # 748 pairs pack into the minimum ceil(748 / 32) = 24 rounds
    assert rounds["pairs"] == -(-len(t["pairs"]) // 32)
    assert rounds["bonds"] <= 3 and rounds["angles"] <= 7 and rounds["dih"] <= 10
    # against 92 rounds when no atom may occur twice in a round
    assert sum(rounds.values()) <= 44


@pytest.mark.parametrize("seed,heavy,rot", [(3, 12, 2), (5, 30, 6), (7, 48, 10)])
def test_other_ligands_conflict_free(scheduler, seed, heavy, rot):
    lig = model.Ligand.from_json(synth.make_ligand(seed=seed, n_heavy=heavy, n_rot=rot, n_n=2, n_o=3))
    for k, v in ligand_terms(lig).items():
        if len(v):
            check(scheduler(v, lig.n_atoms), v, lig.n_atoms)


def test_repeated_atoms_and_tiny_lists(scheduler):
    # a term naming one atom twice (different positions) and lists shorter than a round
    terms = [[0, 1, 0, 2], [2, 1, 0, 3], [3, 2, 1, 0]]
    check(scheduler(terms, 4), terms, 4)
    assert scheduler([], 4, K=2) == []
