"""GPU empirical scores (pose selection, affinity incl. GB/SA) against the FP64 port.

Tolerance: |d score| <= 1e-3 absolute + 1e-5 relative per pose; each term likewise.
"""
import os

import numpy as np
import pytest

import oracle as O
from pxdock_gb300 import abi, model, native, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scored(golden):
    native.load(auto_build=True)
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=700, cube=20.0, cavity=6.0,
                                                       n_rotors=3))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    pose_sf, aff_sf = model.load_scoring_function(os.path.join(golden, "scoring_function.json"))
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    ctx.set_scoring_function(0, pose_sf)
    ctx.set_scoring_function(1, aff_sf)
    lid = ctx.add_ligand(lig)
    port = O.PortSystem(rec, lig)
    yield dict(ctx=ctx, lid=lid, port=port, rec=rec, lig=lig, sf=(pose_sf, aff_sf))
    ctx.close()


def test_pose_selection_score(scored):
    c = scored
    rng = np.random.default_rng(3)
    poses = c["lig"].poses[0][None] + rng.normal(scale=0.6, size=(16,) + c["lig"].poses[0].shape)
    tors = rng.uniform(-3, 3, size=(16, 3))
    s, terms = c["ctx"].score(0, c["lid"], poses, tors)
    for i in range(16):
        rx = c["port"].receptor_apply(tors[i])
        ref, tref = c["port"].score(c["sf"][0], rx, poses[i])
        assert abs(s[i] - ref) <= 1e-3 + 1e-5 * abs(ref), (i, s[i], ref)
        np.testing.assert_allclose(terms[i], tref, atol=2e-3, rtol=1e-5)
    # the synthetic complex exercises at least six term families
    assert np.count_nonzero(np.abs(terms).sum(axis=0)[:9]) >= 6


def test_affinity_score_with_gbsa(scored):
    c = scored
    x = c["lig"].poses[0]
    t = np.array([0.3, -0.2, 1.0])
    s, terms = c["ctx"].score(1, c["lid"], x[None], t[None])
    ref, tref = c["port"].score(c["sf"][1], c["port"].receptor_apply(t), x)
    assert abs(terms[0][abi.TERM_NAMES.index("Gbsa_Com_Energy-Gbsa_Lig_Energy-Gbsa_Pro_Energy")] -
               tref[10]) <= 1e-6 * max(1.0, abs(tref[10]))
    assert abs(s[0] - ref) <= 1e-3 + 1e-5 * abs(ref)


def test_score_requires_function(golden):
    native.load(auto_build=True)
    rec = model.Receptor.from_json(synth.make_receptor(seed=2, n_heavy=200, cube=14.0, cavity=4.0))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    lid = ctx.add_ligand(lig)
    with pytest.raises(native.NativeError):
        ctx.score(0, lid, lig.poses[0][None])
    ctx.close()
