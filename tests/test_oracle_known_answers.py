"""Pins the FP64 port (oracle/port) against the reference's own unit-test answers.

Every expected number below is a known answer from the reference gtest suite
(engine/utest/*.cpp, cited per test) with that test's tolerance. The fixtures are the
test's own inputs (the JSON ones are extracted to tests/golden by make_golden.py).
"""
import math
import os

import numpy as np
import pytest

import oracle as O
from pxdock_gb300 import abi, model

PI = math.pi


def rad(deg):
    return (deg / 180.0) * PI


def topo(xyz, **kw):
    n = len(xyz)
    return model.Topology(n, kw.pop("charge", np.zeros(n)), kw.pop("sigma", np.zeros(n)),
                          kw.pop("epsilon", np.zeros(n)), **kw)


def intra(which, top, xyz):
    lib = O.port_lib()
    keep = []
    t = top.to_c(keep)
    x = np.ascontiguousarray(np.asarray(xyz, np.float64).reshape(-1))
    g = np.zeros_like(x)
    e = lib.po_intra_energy(which, t, x.ctypes.data_as(abi.f64p), g.ctypes.data_as(abi.f64p))
    return e, g.reshape(-1, 3)


XYZ10 = [[7.908, 27.763, 9.369], [8.890, 26.662, 8.959], [8.190, 25.303, 9.005],
         [9.472, 26.977, 7.565], [8.806, 26.234, 6.393], [9.781, 25.678, 5.445],
         [10.482, 24.527, 5.659], [10.255, 23.716, 6.568], [11.714, 24.349, 4.739],
         [11.305, 23.973, 3.332]]


def test_vdw_table_matches_reference_header():
    path = os.path.join(O.REF_ENGINE, "include", "bytedock", "core", "constant.h")
    if not os.path.exists(path):
        pytest.skip("reference checkout not present on this host")
    import re

    src = open(path).read()
    db = re.search(r"kVdwTypeDatabase\[\] = \{(.*?)\};", src, re.S).group(1)
    pairs = np.array(re.findall(r"\{([0-9.]+),\s*([0-9.]+)\}", db), dtype=float)
    sig, eps = model.vdw_table()
    assert np.array_equal(pairs[:, 0], sig) and np.array_equal(pairs[:, 1], eps)


def test_dihedral_angle_and_gradient():
    """test_math.cpp:39-62"""
    lib = O.port_lib()
    p = [np.array(v, float) for v in ([7.908, 27.763, 9.369], [8.890, 26.662, 8.959],
                                       [9.472, 26.977, 7.565], [8.806, 26.234, 6.393])]
    ptr = [v.ctypes.data_as(abi.f64p) for v in p]
    theta = lib.po_dihedral(*ptr)
    assert abs(theta - -1.7239) < 3e-5
    g = [np.zeros(3) for _ in range(4)]
    theta2 = lib.po_dihedral_and_gradient(*ptr, *[x.ctypes.data_as(abi.f64p) for x in g])
    assert abs(theta2 - -1.7239) < 3e-5
    ref = [[-0.5188, -0.3524, -0.2962], [0.4927, 0.6991, 0.3637],
           [0.4956, -0.8849, 0.0070], [-0.4695, 0.5383, -0.0744]]
    for a, b in zip(g, ref):
        np.testing.assert_allclose(a, b, atol=1e-4)


def test_rotation_matrix_and_gradient():
    """test_math.cpp:64-97"""
    lib = O.port_lib()
    axis = np.array([0.26726124, 0.5345225, 0.8017837])
    rot, jac = np.zeros(9), np.zeros(9)
    lib.po_rotation_axis_angle(axis.ctypes.data_as(abi.f64p), O.C.c_double(PI / 4),
                               rot.ctypes.data_as(abi.f64p), jac.ctypes.data_as(abi.f64p))
    v = np.ones(3)
    np.testing.assert_allclose(rot.reshape(3, 3) @ v, [0.6437, 1.3361, 0.8947], atol=5e-5)
    np.testing.assert_allclose(jac.reshape(3, 3) @ v, [-0.5930, 0.2769, 0.0130], atol=5e-5)


def test_harmonic_bond():
    """test_interaction.cpp:25-62"""
    xyz = XYZ10[:6]
    t = topo(xyz, bonds=[[0, 1], [1, 2], [1, 3], [3, 4], [4, 5]],
             bond_k=[520.7307] * 4 + [697.9920], bond_length=[1.5364] * 4 + [1.4652])
    e, g = intra(0, t, xyz)
    assert abs(e - 0.039156) < 1e-4
    ref = [[1.7266, -1.9359, -0.7209], [-4.7169, -2.0213, 3.9922], [1.6703, 3.2427, -0.1098],
           [1.9575, 1.4257, -2.0395], [-2.4871, 0.3434, 0.6763], [1.8495, -1.0547, -1.7983]]
    np.testing.assert_allclose(g, ref, atol=2e-2)


def test_harmonic_angle():
    """test_interaction.cpp:64-104"""
    xyz = XYZ10[:7]
    t = topo(xyz, angles=[[0, 1, 2], [0, 1, 3], [1, 3, 4], [2, 1, 3], [3, 4, 5], [4, 5, 6]],
             angle_k=[81.2141] * 5 + [109.2473],
             angle_radian=[rad(109.8749)] * 5 + [rad(118.8684)])
    e, g = intra(1, t, xyz)
    assert abs(e - 0.971852) < 2e-5
    ref = [[-0.0771, -0.0219, -0.1260], [3.2393, 0.5275, -0.9226], [-0.6397, 0.4076, 2.3082],
           [-7.9720, -2.5917, 2.9012], [6.3865, 7.7524, -6.7594], [-4.1822, -6.8758, 8.9158],
           [3.2451, 0.8019, -6.3172]]
    np.testing.assert_allclose(g, ref, atol=2e-4)


def _dihedral_block(rows):
    ids = np.array([r[0] for r in rows], np.int32)
    per = np.array([r[1] for r in rows], np.int32)
    phase = np.array([r[2] for r in rows], float)
    k = np.array([r[3] for r in rows], float)
    return ids, per, phase, k


def test_fourier_dihedral():
    """test_interaction.cpp:106-159"""
    P4 = [1, 2, 3, 4, 0, 0]
    PH = [0.0, PI, 0.0, PI, 0.0, 0.0]
    propers = [
        ([0, 1, 3, 4], P4, PH, [-0.0237973, 0.0580221, 0.0825244, 0.0666989, 0, 0]),
        ([1, 3, 4, 5], P4, PH, [0.1194276, -0.0281046, 0.1573266, 0.1047968, 0, 0]),
        ([2, 1, 3, 4], P4, PH, [-0.0237973, 0.0580221, 0.0825244, 0.0666989, 0, 0]),
        ([3, 4, 5, 6], P4, PH, [-0.2879912, -0.0000743, -0.0120200, -0.0986383, 0, 0]),
        ([4, 5, 6, 7], P4, PH, [-0.5587948, 2.5157614, -0.2466097, 0.1436590, 0, 0]),
        ([4, 5, 6, 8], P4, PH, [-0.0613361, 1.6208833, 0.1640346, 0.1171070, 0, 0]),
        ([5, 6, 8, 9], P4, PH, [0.0861966, -0.0945933, -0.2458158, -0.0589235, 0, 0]),
        ([7, 6, 8, 9], P4, PH, [0.0312411, 0.3406516, -0.2255443, -0.0649818, 0, 0]),
    ]
    IP = [2, 0, 0, 0, 0, 0]
    IPH = [PI, 0, 0, 0, 0, 0]
    IK = [3.5, 0, 0, 0, 0, 0]
    impropers = [([6, 5, 7, 8], IP, IPH, IK), ([6, 7, 8, 5], IP, IPH, IK),
                 ([6, 8, 5, 7], IP, IPH, IK)]
    t = topo(XYZ10, impropers=_dihedral_block(impropers), propers=_dihedral_block(propers))
    e, g = intra(2, t, XYZ10)
    assert abs(e - -0.445926) < 2e-6
    ref = [[0.1888, 0.1282, 0.1078], [-0.1391, -0.3687, -0.1414], [0.0773, -0.0390, 0.0235],
           [-0.3187, 0.7261, -0.1640], [3.1714, 1.8067, 1.9171], [-4.4598, -3.2939, -2.4912],
           [1.6537, 1.0094, 0.7008], [-1.4417, -1.1764, -1.4134], [1.2504, 1.6017, 1.3607],
           [0.0178, -0.3940, 0.1001]]
    np.testing.assert_allclose(g, ref, atol=1e-4)


def test_self_nonbonded():
    """test_interaction.cpp:161-225"""
    xyz = XYZ10[:8]
    t = topo(xyz,
             charge=[-0.0861, -0.0617, -0.0861, -0.0604, 0.0017, -0.5409, 0.6301, -0.6651],
             sigma=[3.3795] * 5 + [3.2069, 3.4806, 3.0398],
             epsilon=[0.1088] * 5 + [0.1677, 0.0869, 0.2102],
             pairs14=[[0, 4], [1, 5], [2, 4], [3, 6], [4, 7]],
             pairs=[[0, 5], [0, 6], [0, 7], [1, 6], [1, 7], [2, 5], [2, 6], [2, 7], [3, 7]])
    e, g = intra(3, t, xyz)
    assert abs(e - 12.38822) < 1e-3
    ref = [[0.2816, -0.4702, -0.6080], [0.1016, -0.3013, -0.4143], [1.9576, 1.6140, -6.5721],
           [0.2167, -0.9959, -0.2429], [0.0525, -4.3827, 5.9701], [-0.7626, 0.3425, 1.9301],
           [1.2506, -1.0887, -2.0243], [-3.0981, 5.2822, 1.9613]]
    np.testing.assert_allclose(g, ref, atol=3e-3)


def _system(golden, rec_name, lig_name):
    rec = model.Receptor.from_file(os.path.join(golden, rec_name))
    lig = model.Ligand.from_file(os.path.join(golden, lig_name))
    return rec, lig, O.PortSystem(rec, lig)


def test_inter_molecular_brute_force(golden):
    """test_interaction.cpp:227-278: two receptor atoms, three ligand atoms, no maps."""
    rxyz = [[28.80, 40.38, 5.30], [28.08, 40.41, 4.60]]
    rtop = topo(rxyz, charge=[-0.2020, 0.3120], sigma=[3.25, 1.0691], epsilon=[0.17, 0.0157])
    rec = model.Receptor(rxyz, rtop)
    lxyz = [[9.781, 25.678, 5.445], [10.482, 24.527, 5.659], [10.255, 23.716, 6.568]]
    sig, eps = model.vdw_table()
    types = [19, 13, 16]
    ltop = topo(lxyz, charge=[-0.5409, 0.6301, -0.6651], sigma=sig[types], epsilon=eps[types])
    lig = model.Ligand(ltop, types, None, [lxyz])
    s = O.PortSystem(rec, lig)
    e, _, lg = s.score_grad([], lxyz)
    assert abs(e - -0.8934) < 2e-5
    ref = [[-0.0293, -0.0252, 0.0033], [0.0315, 0.0305, -0.0041], [-0.0303, -0.0304, 0.0056]]
    np.testing.assert_allclose(lg, ref, atol=1e-4)


def test_binding_system_receptor_torsion_chain_rule(golden):
    """test_interaction.cpp:280-454: 3 receptor rotors, brute-force inter terms."""
    rec, lig, s = _system(golden, "utest_interaction_receptor.json",
                          "utest_interaction_ligand.json")
    assert rec.n_rotors == 3
    x = lig.poses[0]
    e, tg, _ = s.score_grad(np.zeros(3), x)
    assert abs(e - -24.8695) < 4e-5
    np.testing.assert_allclose(tg, [-1.6258, 0.1114, -0.0144], atol=3e-5)
    t = [rad(i * 360.0 / 3) for i in range(3)]
    e, tg, _ = s.score_grad(t, x)
    assert abs(e - -25.51645) < 5e-5
    np.testing.assert_allclose(tg, [-1.6258, -0.5845, -0.0027], atol=4e-5)


def test_lbfgs_one_iteration(golden):
    """test_optimizer.cpp:177-198: lbfgs_step(1, 8) from zero torsions."""
    rec, lig, s = _system(golden, "utest_optimizer_receptor.json", "utest_optimizer_ligand.json")
    r = s.lbfgs(abi.lbfgs_params(max_iter=1, max_eval=8), np.zeros(3), lig.poses[0])
    assert abs(r["energy"] - -65.1168) < 1e-4
    np.testing.assert_allclose(r["torsions"], [1.7078, -0.1169, 0.0151], atol=1e-4)
    ref = [[12.3282, 26.6937, 6.1659], [7.2854, 22.2396, 5.1075], [12.6085, 26.1862, 6.4895]]
    np.testing.assert_allclose(r["xyz"], ref, atol=1e-4)


def test_lbfgs_two_iterations(golden):
    """test_optimizer.cpp:200-221: lbfgs_step(2, 12) from torsions (1, 2, 3)."""
    rec, lig, s = _system(golden, "utest_optimizer_receptor.json", "utest_optimizer_ligand.json")
    r = s.lbfgs(abi.lbfgs_params(max_iter=2, max_eval=12), [1.0, 2.0, 3.0], lig.poses[0])
    assert abs(r["energy"] - -75.4551) < 1e-4
    np.testing.assert_allclose(r["torsions"], [0.3757, 2.6070, 2.9846], atol=2e-4)
    ref = [[12.6585, 27.4573, 6.1878], [7.5778, 21.4340, 5.0107], [12.3453, 26.6342, 6.5759]]
    np.testing.assert_allclose(r["xyz"], ref, atol=2e-4)


def test_receptor_rotor_kinematics(golden):
    """test_conformer.cpp:267-293"""
    rec, lig, s = _system(golden, "utest_conformer_receptor.json", "utest_conformer_ligand.json")
    out = s.receptor_apply([PI / 2, PI, -PI / 3])
    ref = [[28.800000, 40.380000, 5.300000], [15.410000, 27.400000, 6.380000],
           [15.100000, 27.430000, 5.060000], [14.245493, 27.873225, 4.951510],
           [16.630000, 31.420000, 1.350000], [17.020000, 30.230000, 0.680000],
           [16.646023, 29.472904, 1.127602], [2.680000, 30.610000, 11.500000],
           [1.600000, 31.410000, 10.900000], [0.894953, 31.602039, 11.597803],
           [1.975777, 32.290713, 10.570551], [1.187745, 30.907720, 10.133019]]
    np.testing.assert_allclose(out, ref, atol=5e-7)


def test_ligand_translate_and_rotate(golden):
    """test_conformer.cpp:295-326"""
    rec, lig, s = _system(golden, "utest_conformer_receptor.json", "utest_conformer_ligand.json")
    x = lig.poses[0]
    c0 = x.mean(axis=0)
    t = np.zeros(lig.n_torsions)
    out = s.ligand_apply(x, [10.0, 11.0, 12.0], np.eye(3), t)
    np.testing.assert_allclose(x - c0, out - np.array([10.0, 11.0, 12.0]), atol=1e-7)
    out = s.ligand_apply(x, [0.0, 0.0, 0.0], np.diag([-1.0, -1.0, 1.0]), t)
    ref = np.stack([c0[0] - x[:, 0], c0[1] - x[:, 1], x[:, 2] - c0[2]], axis=1)
    np.testing.assert_allclose(out, ref, atol=1e-7)


def test_ligand_torsion_tree_kinematics(golden):
    """test_conformer.cpp:328-378: 27 atoms, 5 torsions, Euler ZYX orientation."""
    rec, lig, s = _system(golden, "utest_conformer_receptor.json", "utest_conformer_ligand.json")
    r2, r3, r6, r18 = math.sqrt(2), math.sqrt(3), math.sqrt(6), math.sqrt(18)
    rot = [[r2 / 4, -r6 / 8 - r3 / 4, r2 / 8 - 0.75],
           [r6 / 4, 0.25 - r18 / 8, r6 / 8 + r3 / 4],
           [-r2 / 2, -r6 / 4, r2 / 4]]
    tors = [PI / 2, -PI, 0.0, PI, -PI / 2]
    out = s.ligand_apply(lig.poses[0], [-1.0, -2.0, -3.0], rot, tors)
    ref = [[-2.154209, -1.958485, -4.511250], [-1.261266, -2.335375, -3.494563],
           [-1.685584, -3.366784, -2.464486], [-1.049737, -3.142559, -1.170300],
           [-3.177796, -3.359105, -2.268266], [-3.890403, -4.602241, -1.789304],
           [-4.079913, -4.130074, -3.202317], [0.010293, -1.735018, -3.468816],
           [0.379463, -0.784787, -4.432720], [1.735818, -0.192449, -4.348892],
           [2.459659, -0.683096, -3.326595], [2.193265, 0.649541, -5.098981],
           [-0.527274, -0.426520, -5.435662], [-1.791783, -1.013204, -5.472913],
           [-3.146909, -2.401913, -4.560062], [-1.372945, -4.361594, -2.806240],
           [-1.776214, -3.091916, -0.457779], [-0.475629, -3.947074, -0.928210],
           [-3.552369, -2.413113, -1.889015], [-4.709986, -4.474396, -1.091418],
           [-3.302540, -5.498038, -1.620227], [-5.032260, -3.684236, -3.467175],
           [-3.629927, -4.714830, -3.997214], [0.723404, -2.002182, -2.690264],
           [2.918414, -1.457612, -3.715306], [-0.258596, 0.308153, -6.191015],
           [-2.496645, -0.733824, -6.252317]]
    np.testing.assert_allclose(out, ref, atol=5e-7)


def test_rng_distributions():
    """test_random.cpp:24-77 properties, seed 59."""
    lib = O.port_lib()
    import ctypes as C

    class Rng(C.Structure):
        _fields_ = [("mt", C.c_uint32 * 624), ("idx", C.c_int)]

    r = Rng()
    lib.po_rng_seed(C.byref(r), 59)
    for i in range(5):
        lo = np.zeros(3)
        lib.po_rng_in_sphere(C.byref(r), lo.ctypes.data_as(abi.f64p))
        lo *= i + 1
        hi = lo + np.array([lib.po_rng_uniform_int(C.byref(r), 1, 10) for _ in range(3)])
        out = np.zeros(3)
        lib.po_rng_in_box(C.byref(r), lo.ctypes.data_as(abi.f64p), hi.ctypes.data_as(abi.f64p),
                          out.ctypes.data_as(abi.f64p))
        assert np.all(out > lo) and np.all(out < hi)
    for _ in range(5):
        q = np.zeros(4)
        lib.po_rng_orientation(C.byref(r), q.ctypes.data_as(abi.f64p))
        assert abs(q @ q - 1.0) < 1e-7
    prev = -1.0
    for _ in range(5):
        v = np.zeros(3)
        lib.po_rng_in_sphere(C.byref(r), v.ctypes.data_as(abi.f64p))
        n = np.linalg.norm(v)
        assert n < 1.0 and n != prev
        prev = n


def _lists(**kw):
    ff = {}
    ff.update(kw)
    return model.ScoreLists(ff, kw.pop("_n", 0), ligand=True)


def test_torsion_strain_penalty():
    """test_scorer.cpp:25-94"""
    xyz = np.array([
        [-19.492, 19.720, -7.201], [-19.063, 18.558, -7.938], [-18.960, 18.607, -9.386],
        [-20.077, 17.159, -7.527], [-21.147, 17.375, -6.637], [-21.982, 16.325, -6.257],
        [-21.750, 15.047, -6.749], [-20.675, 14.819, -7.609], [-19.827, 15.867, -7.998],
        [-18.539, 15.433, -9.053], [-17.500, 18.112, -7.433], [-16.455, 17.929, -8.463],
        [-15.587, 19.154, -8.657], [-14.229, 19.120, -8.308], [-13.422, 20.244, -8.487],
        [-13.959, 21.408, -9.034], [-15.298, 21.443, -9.417], [-16.107, 20.321, -9.239],
        [-17.198, 18.289, -5.976], [-16.256, 17.156, -5.513], [-15.287, 17.773, -4.563],
        [-15.163, 19.208, -4.949], [-16.534, 19.601, -5.524], [-17.337, 20.458, -4.579],
        [-17.723, 20.058, -3.207], [-20.147, 19.632, -3.822], [-17.359, 22.127, -4.945],
        [-16.891, 22.222, -6.310], [-18.666, 22.636, -4.594], [-16.156, 22.842, -3.870],
        [-16.567, 23.231, -2.585]])
    ff = {"tstrain_atomidx_pose_selection": [[[4, 3, 1, 10]], [[30, 29, 26, 23]],
                                              [[3, 1, 10, 11], [3, 1, 10, 18]],
                                              [[29, 26, 23, 22], [29, 26, 23, 24]]],
          "tstrain_params_pose_selection": [[0.1, 0.2, 0.3, 0.4], [0.4, 0.3, 0.2, 0.1],
                                             [0.2, 0.1, 0.4, 0.3], [0.3, 0.4, 0.1, 0.2]]}
    lists = model.ScoreLists(ff, len(xyz), ligand=True)
    keep = []
    c = lists.to_c(keep)
    x = np.ascontiguousarray(xyz.reshape(-1))
    v = O.port_lib().po_torsion_strain(O.C.byref(c), x.ctypes.data_as(abi.f64p))
    assert abs(v - 5.07775) < 1e-5


def test_rotatable_energy_term():
    """test_scorer.cpp:96-105: -1 / (2.620643 + 3)"""
    sf = abi.SfParams()
    sf.coef[abi.TERM_NAMES.index("rotatable_energy")] = 1.0
    from types import SimpleNamespace as NS

    empty = model.Topology(0, [], [], [])
    rec = NS(n_atoms=0, ff=empty, lists=model.ScoreLists({}, 0, ligand=False))
    lig = NS(n_atoms=0, ff=empty, vdw_type=np.zeros(0, np.int32),
             lists=model.ScoreLists({"rotatable_bond_index": [[0, 1], [1, 2], [2, 3]]}, 0,
                                    ligand=True))
    v, terms = O.port_score(sf, rec, lig, np.zeros((0, 3)), np.zeros((0, 3)))
    assert abs(v - -0.1779) < 1e-4


def test_gbsa_ligand_only():
    """test_scorer.cpp:107-169: ligand-only GB/SA, empty receptor."""
    xyz = np.array([[7.9080, 27.7630, 9.3690], [8.8900, 26.6620, 8.9590], [8.1900, 25.3030, 9.0050],
                    [9.4720, 26.9770, 7.5650], [8.8060, 26.2340, 6.3930], [9.7810, 25.6780, 5.4450],
                    [10.4820, 24.5270, 5.6590], [10.2550, 23.7160, 6.5680], [7.8577, 27.8194, 10.4664],
                    [8.2507, 28.7281, 8.9676], [6.9102, 27.5324, 8.9676], [9.7322, 26.6217, 9.6655],
                    [8.0365, 25.0049, 10.0527], [7.2166, 25.3746, 8.4977], [8.8135, 24.5520, 8.4977],
                    [9.3648, 28.0573, 7.3878], [10.5178, 26.6366, 7.5871], [8.2962, 25.3296, 6.7565],
                    [9.8020, 26.0140, 4.4710]])
    q = np.array([-0.0861, -0.0617, -0.0861, -0.0604, 0.0017, -0.5409, 0.6301, -0.6651, 0.0304,
                  0.0304, 0.0304, 0.0117, 0.0304, 0.0304, 0.0304, 0.0442, 0.0442, 0.0477, 0.3655])
    ff = {"atomic_numbers": [6, 6, 6, 6, 6, 7, 6, 8, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1],
          "bond_index": [[0, 1], [1, 2], [1, 3], [3, 4], [4, 5], [5, 6], [6, 7], [0, 8], [0, 9],
                         [0, 10], [1, 11], [2, 12], [2, 13], [2, 14], [3, 15], [3, 16], [4, 17],
                         [5, 18]]}
    ll = model.ScoreLists(ff, 19, ligand=True)
    rl = model.ScoreLists({}, 0, ligand=False)
    keep = []
    lc, rc = ll.to_c(keep), rl.to_c(keep)
    parts = np.zeros(3)
    x = np.ascontiguousarray(xyz.reshape(-1))
    d = O.port_lib().po_gbsa_parts(0, np.zeros(3).ctypes.data_as(abi.f64p),
                                   np.zeros(1).ctypes.data_as(abi.f64p), O.C.byref(rc), 19,
                                   x.ctypes.data_as(abi.f64p), q.ctypes.data_as(abi.f64p),
                                   O.C.byref(lc), parts.ctypes.data_as(abi.f64p))
    assert abs(parts[1] - -14.4667) < 1e-4  # Gbsa_Lig_Energy
    assert abs(parts[2]) < 1e-4             # Gbsa_Pro_Energy
    assert abs(parts[0] - -14.4667) < 1e-4  # Gbsa_Com_Energy
    assert abs(d) < 1e-4
