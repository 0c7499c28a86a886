"""L2 residency of the maps (pxd_set_l2_residency): the access-policy window changes what
L2 keeps, not what the kernels compute, so a batched optimisation and a Monte-Carlo search
end bit for bit where they end without it; the persisting set-aside is returned when the
context turns it off, and fractions outside [0, 1] are refused."""
import numpy as np
import pytest

from pxdock_gb300 import model, native, synth

pytestmark = pytest.mark.gpu


def test_residency_window_leaves_results_unchanged():
    native.load(auto_build=True)
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=400, cube=18.0, cavity=5.0))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    box = model.make_box((0.0, 0.0, 0.0), (12.0, 12.0, 12.0), 0.375)
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    ctx.build_grid(box)  # every ligand type: 100 maps, beyond L2
    ctx.set_slope(1e6)
    lid = ctx.add_ligand(lig)
    lo = np.array(box.init_xyz)
    hi = lo + (np.array(box.npoints) - 1) * box.spacing
    poses = synth.random_poses(lig, lo + 1.0, hi - 1.0, 1024, seed=4)
    p = native.lbfgs_params(max_iter=60, history=8, tolerance_grad=1e-3)
    off = ctx.lbfgs(p, lid, poses)
    with pytest.raises(native.NativeError):
        ctx.set_l2_residency(1.5)
    ctx.set_l2_residency(0.75)
    on = ctx.lbfgs(p, lid, poses)
    for k in ("xyz", "energy", "nevals", "status"):
        assert np.array_equal(on[k], off[k]), k
    ctx.set_l2_residency(0.0)
    again = ctx.lbfgs(p, lid, poses)
    assert np.array_equal(again["energy"], off["energy"])
    ctx.set_l2_residency(0.5)  # left on: destroying the context returns the set-aside
    ctx.close()
