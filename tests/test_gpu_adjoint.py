"""The differentiable empirical score on the GPU (pxd_score_adjoint) and its
torch.autograd bindings, against the FP64 port (po_score_diff, whose adjoint is pinned
to finite differences in test_oracle_diff.py) and against central FP64 finite
differences with h = 1e-4.

Tolerances (FP32 on the GPU): score 1e-3 + 1e-5 relative; features 2e-3 + 1e-5
relative; coordinate and DOF gradients 1e-4 of the pose's largest component; weight and
table gradients 1e-4 relative (of the largest entry for the table).

The score is piecewise smooth (ramps, LJ clamp, pair-table bins 0.03125 A wide). Where
the FP32 rounding of a distance can move it across a kink, the FP64 gradient itself
jumps; components whose FP64 gradient changes under 1e-5 A perturbations of the pose
are left out of the coordinate comparison (at most 5 % of them)."""
import os

import numpy as np
import pytest

import oracle as O
from pxdock_gb300 import abi, model, native, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def adj(golden):
    native.load(auto_build=True)
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=700, cube=20.0, cavity=6.0, n_rotors=3))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    pose_sf, _ = model.load_scoring_function(os.path.join(golden, "scoring_function.json"))
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    ctx.set_scoring_function(0, pose_sf)
    lid = ctx.add_ligand(lig)
    port = O.PortSystem(rec, lig)
    rng = np.random.default_rng(0)
    w = abi.sf_weights(pose_sf) * rng.uniform(0.5, 1.5, size=abi.NUM_SF_WEIGHTS)
    yield dict(ctx=ctx, lid=lid, port=port, rec=rec, lig=lig, sf=pose_sf, w=w, tab=abi.smooth_pair_tables(1))
    ctx.close()


def poses(adj, n, seed, scale=0.5):
    rng = np.random.default_rng(seed)
    x0 = adj["lig"].poses[0]
    x = x0[None] + rng.normal(scale=scale, size=(n,) + x0.shape)
    return x.astype(np.float32).astype(np.float64), rng.uniform(-3, 3, size=(n, 3))


def port_diff(adj, x, t, w, tab, g=1.0, grads=True):
    rx = adj["port"].receptor_apply(t)
    return O.port_score_diff(adj["sf"], adj["rec"], adj["lig"], rx, x, w, tab, g=g, grads=grads)


def stable_mask(adj, x, t, w, tab, g, gx, tol):
    """Components whose FP64 gradient holds within tol under 1e-5 A perturbations."""
    ok = np.ones(gx.shape, bool)
    rng = np.random.default_rng(99)
    for _ in range(3):
        _, _, g2, _, _ = port_diff(adj, x + rng.normal(scale=1e-5, size=x.shape), t, w, tab, g=g)
        ok &= np.abs(g2 - gx) <= tol
    return ok


def test_weights_layout_matches_the_library(adj):
    w = np.zeros(abi.NUM_SF_WEIGHTS)
    native.load().pxd_sf_weights(adj["sf"], native._p(w))
    np.testing.assert_array_equal(w, abi.sf_weights(adj["sf"]))


def test_value_equals_the_score_kernel(adj):
    """With the scoring function's own weights and no table, S is root_scorer's score."""
    x, t = poses(adj, 16, 1)
    s, f = adj["ctx"].score_adjoint(0, adj["lid"], x, abi.sf_weights(adj["sf"]), tors=t, grads=False)
    ref, _ = adj["ctx"].score(0, adj["lid"], x, t)
    np.testing.assert_allclose(s, ref, atol=1e-3, rtol=1e-5)
    assert np.all(f[:, 27] == 0.0)


def test_adjoint_matches_the_port(adj):
    x, t = poses(adj, 24, 2)
    g = np.random.default_rng(5).normal(size=len(x))
    s, f, dx, dw, dt = adj["ctx"].score_adjoint(0, adj["lid"], x, adj["w"], adj["tab"], grad_out=g, tors=t)
    rw = np.zeros(abi.NUM_SF_WEIGHTS)
    rt = np.zeros(abi.PAIR_TYPES * abi.PAIR_BINS)
    checked = total = 0
    for p in range(len(x)):
        v, fr, gx, gw, gt = port_diff(adj, x[p], t[p], adj["w"], adj["tab"], g=g[p])
        rw += gw
        rt += gt
        assert abs(s[p] - v) <= 1e-3 + 1e-5 * abs(v), (p, s[p], v)
        np.testing.assert_allclose(f[p], fr, atol=2e-3, rtol=1e-5)
        tol = 1e-4 * max(np.max(np.abs(gx)), 1e-6)
        m = stable_mask(adj, x[p], t[p], adj["w"], adj["tab"], g[p], gx, tol)
        total += m.size
        checked += m.sum()
        assert np.max(np.abs(dx[p] - gx)[m]) <= tol, (p, np.max(np.abs(dx[p] - gx)[m]), tol)
    assert checked >= 0.95 * total
    np.testing.assert_allclose(dw, rw, rtol=1e-4, atol=1e-4 * np.max(np.abs(rw)))
    np.testing.assert_allclose(dt.reshape(-1), rt, rtol=1e-4, atol=1e-4 * np.max(np.abs(rt)))
    assert np.count_nonzero(rt) > 500


def test_repeated_adjoint_is_reproducible(adj):
    """Scores, features, coordinate and weight gradients repeat bit for bit (per-warp
    weight accumulators, per-block partials summed in a fixed order); the table gradient's
    shared-memory atomics leave only its last bits to the order of arrival."""
    x, t = poses(adj, 64, 3)
    a = adj["ctx"].score_adjoint(0, adj["lid"], x, adj["w"], adj["tab"], tors=t)
    b = adj["ctx"].score_adjoint(0, adj["lid"], x, adj["w"], adj["tab"], tors=t)
    for u, v in zip(a[:4], b[:4]):
        np.testing.assert_array_equal(u, v)
    np.testing.assert_allclose(a[4], b[4], rtol=1e-6, atol=1e-6 * np.max(np.abs(a[4])))


def test_autograd_parameters_match_finite_differences(adj):
    """torch.autograd through the adjoint kernel: d(sum_p S_p)/dw and /dT against central
    FP64 differences (h = 1e-4) of the port; S is linear in each, so they are exact."""
    torch = pytest.importorskip("torch")
    from pxdock_gb300 import autograd as AG
    x, t = poses(adj, 8, 4)
    dev = torch.device("cuda", 0)
    N = adj["lig"].n_atoms
    xt = torch.tensor(x, dtype=torch.float32, device=dev, requires_grad=True)
    wt = torch.tensor(adj["w"], dtype=torch.float64, device=dev, requires_grad=True)
    tt = torch.tensor(adj["tab"], dtype=torch.float64, device=dev, requires_grad=True)
    ids = torch.full((len(x),), adj["lid"], dtype=torch.int32, device=dev)
    rt = torch.tensor(t, dtype=torch.float32, device=dev)
    total = AG.empirical_score(adj["ctx"], ids, xt, wt, tt, rec_tors=rt).sum()
    total.backward()
    gw = wt.grad.cpu().numpy()
    gtab = tt.grad.cpu().numpy().reshape(-1)
    h = 1e-4

    def S(w, tab):
        return sum(port_diff(adj, x[p], t[p], w, tab, grads=False)[0] for p in range(len(x)))

    ref = S(adj["w"], adj["tab"])
    assert abs(total.item() - ref) <= 1e-3 * len(x) + 1e-5 * abs(ref)
    for k in range(abi.NUM_SF_WEIGHTS):
        wp, wm = adj["w"].copy(), adj["w"].copy()
        wp[k] += h
        wm[k] -= h
        fd = (S(wp, adj["tab"]) - S(wm, adj["tab"])) / (2 * h)
        assert abs(gw[k] - fd) <= 1e-4 * max(1.0, abs(fd)), (k, gw[k], fd)
    nz = np.flatnonzero(gtab)
    scale = np.max(np.abs(gtab))
    for k in np.random.default_rng(2).choice(nz, size=16, replace=False):
        tp, tm = adj["tab"].reshape(-1).copy(), adj["tab"].reshape(-1).copy()
        tp[k] += h
        tm[k] -= h
        fd = (S(adj["w"], tp) - S(adj["w"], tm)) / (2 * h)
        assert abs(gtab[k] - fd) <= 1e-4 * max(scale, 1e-3), (k, gtab[k], fd)
    assert xt.grad is not None and xt.grad.shape == (len(x), N, 3)


def quat_rot(q):
    q = np.asarray(q, float) / np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (a * c + b * d)],
                     [2 * (a * d + b * c), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (a * b + c * d), a * a - b * b - c * c + d * d]])


def test_autograd_dofs_match_finite_differences(adj):
    """Centre, quaternion and torsion gradients of sum_p S_p through ligand_pose (no pair
    table: the remaining kinks are few) against central FP64 differences, h = 1e-4, of
    the port's forward kinematics and score."""
    torch = pytest.importorskip("torch")
    from pxdock_gb300 import autograd as AG
    lig, port = adj["lig"], adj["port"]
    dev = torch.device("cuda", 0)
    x0 = lig.poses[0]
    T = lig.n_torsions
    P = 4
    rng = np.random.default_rng(7)
    c = x0.mean(axis=0)[None] + rng.normal(scale=0.3, size=(P, 3))
    q = rng.normal(size=(P, 4)) * 0.1 + np.array([1.0, 0, 0, 0])
    q *= rng.uniform(0.8, 1.2, size=(P, 1))  # not unit: the normalisation is differentiated
    tor = rng.uniform(-0.5, 0.5, size=(P, T))
    rt = np.zeros((P, 3))
    ref = torch.tensor(x0, dtype=torch.float32, device=dev)
    ct = torch.tensor(c, dtype=torch.float64, device=dev, requires_grad=True)
    qt = torch.tensor(q, dtype=torch.float64, device=dev, requires_grad=True)
    tt = torch.tensor(tor, dtype=torch.float64, device=dev, requires_grad=True)
    ids = torch.full((P,), adj["lid"], dtype=torch.int32, device=dev)
    xyz = AG.ligand_pose(adj["ctx"], adj["lid"], ref, ct, qt, tt)
    wt = torch.tensor(adj["w"], dtype=torch.float64, device=dev)
    total = AG.empirical_score(adj["ctx"], ids, xyz, wt, None,
                               rec_tors=torch.zeros((P, 3), dtype=torch.float32, device=dev)).sum()
    total.backward()
    got = [ct.grad.cpu().numpy(), qt.grad.cpu().numpy(), tt.grad.cpu().numpy()]
    h = 1e-4

    def S(p, cc, qq, tq):
        xp = port.ligand_apply(x0, cc, quat_rot(qq), tq)
        return port_diff(adj, xp, rt[p], adj["w"], None, grads=False)[0]

    def fd(p, k, step):
        """Central difference of S in DOF k (centre 0-2, quaternion 3-6, torsions)."""
        def at(sgn):
            cc, qq, tq = c[p].copy(), q[p].copy(), tor[p].copy()
            if k < 3:
                cc[k] += sgn * step
            elif k < 7:
                qq[k - 3] += sgn * step
            else:
                tq[k - 7] += sgn * step
            return S(p, cc, qq, tq)
        return (at(1) - at(-1)) / (2 * step)

    checked = total = 0
    for p in range(P):
        g = np.concatenate([got[0][p], got[1][p], got[2][p]])
        want = np.array([fd(p, k, h) for k in range(7 + T)])
        # a kink (ramp end, LJ clamp) inside the step shows as a difference from h / 4
        quarter = np.array([fd(p, k, h / 4) for k in range(7 + T)])
        scale = max(1.0, np.max(np.abs(want)))
        smooth = np.abs(want - quarter) <= 1e-5 * scale
        total += smooth.size
        checked += smooth.sum()
        assert np.max(np.abs(g - want)[smooth]) <= 1e-4 * scale, (p, g, want, smooth)
    assert checked >= 0.75 * total  # a DOF step moves every atom: kinks are common at h = 1e-4


def test_multi_context_launches_match_single_context(adj, golden):
    """Poses of two receptors in one launch (pose kinematics forward and backward, docking
    energy, score adjoint) equal the per-context launches bit for bit."""
    torch = pytest.importorskip("torch")
    from pxdock_gb300 import autograd as AG
    dev = torch.device("cuda", 0)
    rec2 = model.Receptor.from_json(synth.make_receptor(seed=5, n_heavy=500, cube=18.0, cavity=6.0))
    lig2 = model.Ligand.from_json(synth.make_ligand(seed=7, n_heavy=18, n_rot=3))
    c2 = native.Context(0)
    c2.set_receptor(rec2)
    c2.build_grid(model.make_box((0.0, 0.0, 0.0), (16.0,) * 3, 0.375), sorted(set(int(t) for t in lig2.vdw_type)))
    c2.set_scoring_function(0, adj["sf"])
    l2 = c2.add_ligand(lig2)
    c1 = adj["ctx"]
    c1.build_grid(model.make_box((0.0, 0.0, 0.0), (16.0,) * 3, 0.375),
                  sorted(set(int(t) for t in adj["lig"].vdw_type)))
    ligs = [adj["lig"], lig2]
    A = max(l.n_atoms for l in ligs)
    D = 7 + max(l.n_torsions for l in ligs)
    P = 6
    rng = np.random.default_rng(11)
    order = np.array([0, 1, 1, 0, 1, 0])  # interleaved contexts
    ref = np.zeros((P, A, 3), np.float32)
    q = np.zeros((P, D), np.float32)
    for p, c in enumerate(order):
        l = ligs[c]
        ref[p, : l.n_atoms] = l.poses[0] - l.poses[0].mean(axis=0)
        qq = rng.normal(size=4)
        q[p, :3] = rng.uniform(-2, 2, 3)
        q[p, 3:7] = qq / np.linalg.norm(qq)
        q[p, 7:7 + l.n_torsions] = rng.uniform(-1, 1, l.n_torsions)
    t = lambda a, dt=torch.float32: torch.tensor(a, dtype=dt, device=dev)
    ctx_ids = t(order, torch.int32)
    lig_ids = t([adj["lid"] if c == 0 else l2 for c in order], torch.int32)
    qt = t(q).requires_grad_(True)
    xyz = AG.ligand_pose_multi([c1, c2], ctx_ids, lig_ids, t(ref), qt)
    e = AG.docking_energy([c1, c2], lig_ids, xyz, ctx_ids=ctx_ids,
                          rec_tors=torch.zeros((P, 3), dtype=torch.float32, device=dev))
    wt = t(adj["w"], torch.float64)
    tab = t(adj["tab"])
    s = AG.empirical_score([c1, c2], lig_ids, xyz, wt, tab, ctx_ids=ctx_ids,
                           rec_tors=torch.zeros((P, 3), dtype=torch.float32, device=dev))
    (e + s).sum().backward()
    for p, c in enumerate(order):
        l, ctx, lid = ligs[c], [c1, c2][c], lig_ids[p:p + 1]
        n, T = l.n_atoms, l.n_torsions
        qp = qt.detach()[p:p + 1]
        one = AG.ligand_pose(ctx, int(lid.item()), t(ref[p, :n]), qp[:, :3].clone().requires_grad_(True),
                             qp[:, 3:7].clone().requires_grad_(True), qp[:, 7:7 + T].clone().requires_grad_(True))
        torch.testing.assert_close(one, xyz.detach()[p:p + 1, :n], rtol=0, atol=0)
        rt = torch.zeros((1, 3), dtype=torch.float32, device=dev) if ctx.n_rotors else None
        e1 = AG.docking_energy(ctx, lid, one.detach(), rec_tors=rt)
        assert e1.item() == e.detach()[p].item()
        s1 = AG.empirical_score(ctx, lid, one.detach(), wt, tab, rec_tors=rt)
        assert s1.item() == s.detach()[p].item()
    c2.close()


def test_hessian_vector_products_match_differences(adj):
    """pxd_score_hvp_multi_dev (the adjoint run on dual numbers) against central FP64
    differences (h = 1e-5) of the port's analytic adjoint along the same directions:
    H v per pose, the features' derivatives, and the mixed weight / table derivatives.
    Components whose differences change between h and h/4 (a kink inside the step) are
    left out, at most 5 % of them."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    x, t = poses(adj, 8, 21)
    rng = np.random.default_rng(22)
    v = rng.normal(size=x.shape)
    v /= np.linalg.norm(v.reshape(len(x), -1), axis=1)[:, None, None]
    g = rng.normal(size=len(x))
    N = adj["lig"].n_atoms
    T = lambda a, dt=torch.float32: torch.tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    xt, vt, tt = T(x), T(v), T(t)
    ids = torch.full((len(x),), adj["lid"], dtype=torch.int32, device=dev)
    w, tab = T(adj["w"], torch.float64), T(adj["tab"])
    hv = torch.zeros_like(xt)
    fd_ = torch.zeros((len(x), abi.NUM_SCORE_FEATURES), dtype=torch.float64, device=dev)
    dw = torch.zeros(abi.NUM_SF_WEIGHTS, dtype=torch.float64, device=dev)
    dt = torch.zeros(abi.PAIR_TYPES * abi.PAIR_BINS, dtype=torch.float64, device=dev)
    native.score_hvp_multi_dev([adj["ctx"]], 0, len(x), N, None, ids.data_ptr(), xt.data_ptr(), vt.data_ptr(),
                               tt.data_ptr(), w.data_ptr(), tab.data_ptr(), T(g, torch.float64).data_ptr(),
                               fd_.data_ptr(), hv.data_ptr(), dw.data_ptr(), dt.data_ptr(), 1)
    torch.cuda.synchronize()
    hv, fd_, dw, dt = hv.cpu().numpy(), fd_.cpu().numpy(), dw.cpu().numpy(), dt.cpu().numpy()

    def diff(p, h):
        a = port_diff(adj, x[p] + h * v[p], t[p], adj["w"], adj["tab"], g=g[p])
        b = port_diff(adj, x[p] - h * v[p], t[p], adj["w"], adj["tab"], g=g[p])
        return [(u - w_) / (2 * h) for u, w_ in zip(a[1:], b[1:])]

    rw, rt, rt4 = np.zeros_like(dw), np.zeros_like(dt), np.zeros_like(dt)
    checked = total = 0
    for p in range(len(x)):
        f1, gx1, gw1, gt1 = diff(p, 1e-5)
        f4, gx4, _, gt4 = diff(p, 2.5e-6)
        rw += gw1
        rt += gt1
        rt4 += gt4
        scale = max(np.max(np.abs(gx1)), 1e-6)
        smooth = np.abs(gx1 - gx4) <= 1e-5 * scale
        total += smooth.size
        checked += smooth.sum()
        assert np.max(np.abs(hv[p] - gx1)[smooth]) <= 1e-4 * scale, (p, np.max(np.abs(hv[p] - gx1)[smooth]), scale)
        fsmooth = np.abs(f1 - f4) <= 1e-5 * np.maximum(np.abs(f1), 1.0)
        np.testing.assert_allclose(fd_[p][fsmooth], f1[fsmooth], rtol=1e-4, atol=1e-3)
    assert checked >= 0.95 * total
    np.testing.assert_allclose(dw, rw, rtol=1e-3, atol=1e-4 * np.max(np.abs(rw)))
    # a pair crossing a bin edge inside the step moves its hat-weight derivative to the
    # next bins: such bins differ between h and h/4 and are left out
    tol = 1e-4 * np.max(np.abs(rt))
    bins = np.abs(rt - rt4) <= tol
    assert np.mean(bins[rt != 0]) >= 0.98
    np.testing.assert_allclose(dt[bins], rt[bins], rtol=1e-3, atol=tol)


def test_adjoint_edge_cases(adj):
    """Empty batch, a bad ligand id (NaN score, zero gradient rows), an oversize row stride
    (refused), and a rigid ligand (no torsions) through the multi-context kinematics."""
    torch = pytest.importorskip("torch")
    from pxdock_gb300 import autograd as AG
    dev = torch.device("cuda", 0)
    N = adj["lig"].n_atoms
    w = torch.tensor(adj["w"], dtype=torch.float64, device=dev)
    x = torch.tensor(np.tile(adj["lig"].poses[0], (2, 1, 1)), dtype=torch.float32, device=dev)
    ids = torch.tensor([adj["lid"], 99], dtype=torch.int32, device=dev)
    rt = torch.zeros((2, 3), dtype=torch.float32, device=dev)
    s = torch.zeros(2, dtype=torch.float64, device=dev)
    g = torch.ones(2, dtype=torch.float64, device=dev)
    dx = torch.full_like(x, 7.0)
    dw = torch.zeros(abi.NUM_SF_WEIGHTS, dtype=torch.float64, device=dev)
    args = lambda n, a: (0, n, a, ids.data_ptr(), x.data_ptr(), rt.data_ptr(), w.data_ptr(), None, g.data_ptr(),
                         s.data_ptr(), None, dx.data_ptr(), dw.data_ptr(), None, 1)
    adj["ctx"].score_adjoint_dev(*args(0, N))
    adj["ctx"].score_adjoint_dev(*args(2, N))
    torch.cuda.synchronize()
    assert np.isfinite(s[0].item()) and np.isnan(s[1].item())
    assert torch.all(dx[1] == 0) and torch.any(dx[0] != 0)
    with pytest.raises(native.NativeError):
        adj["ctx"].score_adjoint_dev(*args(2, abi_max_atoms_plus_one()))
    # a rigid ligand: DOF rows of 7, no torsion columns
    rigid = model.Ligand.from_json(synth.make_ligand(seed=3, n_heavy=12, n_rot=0))
    assert rigid.n_torsions == 0
    lid = adj["ctx"].add_ligand(rigid)
    ref = torch.tensor((rigid.poses[0] - rigid.poses[0].mean(axis=0))[None], dtype=torch.float32, device=dev)
    q = torch.tensor([[0.5, -0.2, 0.1, 0.9, 0.1, -0.3, 0.2]], dtype=torch.float64, device=dev, requires_grad=True)
    xyz = AG.ligand_pose_multi([adj["ctx"]], torch.zeros(1, dtype=torch.int32, device=dev),
                               torch.tensor([lid], dtype=torch.int32, device=dev), ref, q)
    xyz.sum().backward()
    assert torch.allclose(q.grad[0, :3], torch.full((3,), float(rigid.n_atoms), dtype=torch.float64, device=dev))
    adj["ctx"].clear_ligands()
    adj["lid"] = adj["ctx"].add_ligand(adj["lig"])


def abi_max_atoms_plus_one():
    return 257
