"""ctypes mirrors of the C ABI structs declared in include/pxdock_gb300.h.

The layouts must match the header field for field; tests/test_capi.py checks the
sizes against the compiled library.
"""
import ctypes as C

i32p = C.POINTER(C.c_int32)
f64p = C.POINTER(C.c_double)
f32p = C.POINTER(C.c_float)


class Topology(C.Structure):
    """pxd_topology: force-field terms of one molecule (system.h:85-109)."""

    _fields_ = [
        ("n_atoms", C.c_int32),
        ("charge", f64p),
        ("sigma", f64p),
        ("epsilon", f64p),
        ("n_bonds", C.c_int32),
        ("bond_atoms", i32p),
        ("bond_k", f64p),
        ("bond_length", f64p),
        ("n_angles", C.c_int32),
        ("angle_atoms", i32p),
        ("angle_k", f64p),
        ("angle_radian", f64p),
        ("n_impropers", C.c_int32),
        ("improper_atoms", i32p),
        ("improper_periodicity", i32p),
        ("improper_phase", f64p),
        ("improper_k", f64p),
        ("n_propers", C.c_int32),
        ("proper_atoms", i32p),
        ("proper_periodicity", i32p),
        ("proper_phase", f64p),
        ("proper_k", f64p),
        ("n_pairs14", C.c_int32),
        ("pairs14", i32p),
        ("n_pairs", C.c_int32),
        ("pairs", i32p),
    ]


class TorsionTree(C.Structure):
    """pxd_torsion_tree: flat fragment tree (system.h:135-154)."""

    _fields_ = [
        ("n_frags", C.c_int32),
        ("frag_start", i32p),
        ("frag_end", i32p),
        ("perm", i32p),
        ("n_roots", C.c_int32),
        ("roots", i32p),
        ("n_torsions", C.c_int32),
        ("tors_frag", i32p),
        ("tors_parent", i32p),
        ("tors_parent_atom", i32p),
        ("tors_mine_atom", i32p),
    ]


class ScoreLists(C.Structure):
    """pxd_score_lists: interaction atom lists of one molecule."""

    _fields_ = [
        ("n_hydrophobic", C.c_int32), ("hydrophobic", i32p),
        ("n_cation", C.c_int32), ("cation", i32p),
        ("n_anion", C.c_int32), ("anion", i32p),
        ("n_ring5", C.c_int32), ("ring5", i32p),
        ("n_ring6", C.c_int32), ("ring6", i32p),
        ("n_don_charged", C.c_int32), ("don_charged", i32p),
        ("n_don_neutral", C.c_int32), ("don_neutral", i32p),
        ("n_acc_charged", C.c_int32), ("acc_charged", i32p),
        ("n_acc_neutral", C.c_int32), ("acc_neutral", i32p),
        ("n_tstrain", C.c_int32), ("tstrain_coefs", f64p), ("tstrain_offsets", i32p),
        ("tstrain_quads", i32p),
        ("n_rotatable", C.c_int32),
        ("atomic_numbers", i32p),
        ("n_all_bonds", C.c_int32), ("all_bonds", i32p),
    ]


class LigandDesc(C.Structure):
    _fields_ = [("ff", Topology), ("vdw_type", i32p), ("tree", TorsionTree),
                ("lists", C.POINTER(ScoreLists))]


class ReceptorDesc(C.Structure):
    _fields_ = [
        ("n_atoms", C.c_int32),
        ("xyz", f64p),
        ("ff", Topology),
        ("n_rotors", C.c_int32),
        ("rotor_axis", i32p),
        ("rotor_offsets", i32p),
        ("rotor_atoms", i32p),
        ("lists", C.POINTER(ScoreLists)),
    ]


class Box(C.Structure):
    """pxd_box (box_config, grid.h:31-40)."""

    _fields_ = [
        ("init_xyz", C.c_double * 3),
        ("npoints", C.c_int32 * 3),
        ("spacing", C.c_double),
    ]


class LbfgsParams(C.Structure):
    """pxd_lbfgs_params (optimizer.h:52-66, optimizer.cpp:235-246)."""

    _fields_ = [
        ("max_iter", C.c_int32),
        ("max_eval", C.c_int32),
        ("history", C.c_int32),
        ("ls_max", C.c_int32),
        ("lr", C.c_double),
        ("tolerance_grad", C.c_double),
        ("tolerance_change", C.c_double),
        ("ls_c1", C.c_double),
        ("ls_c2", C.c_double),
        ("ls_tolerance_change", C.c_double),
        ("ls_gtd_threshold", C.c_double),
        ("reset_threshold", C.c_double),
        ("dof_mode", C.c_int32),
        ("reserved", C.c_int32),
    ]


class McParams(C.Structure):
    """pxd_mc_params (monte_carlo_searcher, searcher.h:29-41; search() arguments)."""

    _fields_ = [
        ("seed", C.c_uint32),
        ("max_nsteps", C.c_int32),
        ("relax_nsteps", C.c_int32),
        ("full_nsteps", C.c_int32),
        ("mc_mmenergy_threshold", C.c_double),
        ("amplitude", C.c_double),
        ("temperature", C.c_double),
        ("box_lo", C.c_double * 3),
        ("box_hi", C.c_double * 3),
        ("lbfgs", LbfgsParams),
    ]


DOF_CARTESIAN = 0
DOF_RIGID_TORSION = 1


def lbfgs_params(max_iter=240, max_eval=0, history=100, tolerance_grad=0.5,
                 tolerance_change=1e-4, lr=1.0, dof_mode=DOF_CARTESIAN):
    """Reference constants by default (lbfgs_step, optimizer.h:50-67)."""
    p = LbfgsParams()
    p.max_iter = max_iter
    p.max_eval = max_eval
    p.history = history
    p.ls_max = 25
    p.lr = lr
    p.tolerance_grad = tolerance_grad
    p.tolerance_change = tolerance_change
    p.ls_c1 = 1e-4
    p.ls_c2 = 0.9
    p.ls_tolerance_change = 1e-9
    p.ls_gtd_threshold = 1e5
    p.reset_threshold = 1e8
    p.dof_mode = dof_mode
    return p


POSE_CONVERGED = 0
POSE_NOT_CONVERGED = 1
POSE_NAN = 2
POSE_BAD_INPUT = 3
NUM_VDW_TYPES = 99
COULOMB_MAP = 99


class SfParams(C.Structure):
    """pxd_sf_params: one scoring function (ScoringFunctionParams, conf.h:122-150)."""

    _fields_ = [
        ("coef", C.c_double * 11),
        ("vdw_scale", C.c_double), ("vdw_cutoff", C.c_double),
        ("vdw_sigma_scale", C.c_double * 99), ("vdw_epsilon_scale", C.c_double * 99),
        ("ionic_coef", C.c_double * 2), ("ionic", (C.c_double * 2) * 2),
        ("picat_coef", C.c_double * 4), ("picat", (C.c_double * 2) * 4),
        ("stack_coef", (C.c_double * 4) * 2), ("stack", ((C.c_double * 6) * 4) * 2),
        ("hbond_scale", C.c_double), ("hbond_coef", C.c_double * 8),
        ("hbond", (C.c_double * 6) * 8),
        ("hydro_scale", C.c_double), ("hydro_dist_min", C.c_double),
        ("hydro_dist_max", C.c_double), ("hydro_scale_factor", C.c_double),
    ]


TERM_NAMES = ["InteractionCoulomb_oriEnergy", "InteractionVDW_Energy", "Ionic_Energy",
              "Pi_Cationic_Energy", "F2FPiStacking_Energy", "E2FPiStacking_Energy",
              "Hbond_Energy", "Hydrophobic_Energy", "TorsionStrain_Penalty", "rotatable_energy",
              "Gbsa_Com_Energy-Gbsa_Lig_Energy-Gbsa_Pro_Energy"]

# Differentiable empirical score (pxd_score_adjoint): weight vector layout, feature
# count and pair-table shape, as in include/pxdock_gb300.h.
NUM_SF_WEIGHTS = 36
NUM_SCORE_FEATURES = 28
PAIR_TYPES, PAIR_BINS, PAIR_BIN_WIDTH = 32, 256, 0.03125
W_COEF, W_VDW_SCALE, W_HYDRO_SCALE, W_HBOND_SCALE = 0, 11, 12, 13
W_IONIC, W_PICAT, W_STACK, W_HBOND = 14, 16, 20, 28


def sf_weights(sf):
    """The 36 weights of a scoring function in pxd_sf_weight order (pxd_sf_weights)."""
    import numpy as np
    w = np.zeros(NUM_SF_WEIGHTS)
    w[W_COEF:W_COEF + 11] = list(sf.coef)
    w[W_VDW_SCALE], w[W_HYDRO_SCALE], w[W_HBOND_SCALE] = sf.vdw_scale, sf.hydro_scale, sf.hbond_scale
    w[W_IONIC:W_IONIC + 2] = list(sf.ionic_coef)
    w[W_PICAT:W_PICAT + 4] = list(sf.picat_coef)
    w[W_STACK:W_STACK + 8] = [sf.stack_coef[q][k] for q in range(2) for k in range(4)]
    w[W_HBOND:W_HBOND + 8] = list(sf.hbond_coef)
    return w


def smooth_pair_tables(seed=0):
    """Seeded smooth pair tables [32][256] (FP32 values): a soft wall plus one well per
    atom-type pair, zero at the cut-off."""
    import numpy as np
    rng = np.random.default_rng(seed)
    r = np.arange(PAIR_BINS) * PAIR_BIN_WIDTH
    t = np.zeros((PAIR_TYPES, PAIR_BINS))
    for p in range(PAIR_TYPES):
        r0 = rng.uniform(3.2, 4.4)
        depth = rng.uniform(0.05, 0.4)
        width = rng.uniform(0.4, 0.9)
        wall = 2.0 * np.exp(-(r - 1.0) / 0.35)
        t[p] = wall - depth * np.exp(-((r - r0) / width) ** 2)
        t[p] *= np.clip((r[-1] - r) / 1.0, 0.0, 1.0)  # taper to zero at the cut-off
    return t.astype(np.float32).astype(np.float64)


def weights_grad(w, f):
    """d(sum_p g_p S_p)/dw from the weights w [36] and the g-weighted feature sum
    f = sum_p g_p features_p [28]: the derivative of pxd's feature combination (S is
    linear in each weight group), in the layout of pxd_sf_weights. Works on numpy arrays
    and torch tensors."""
    C = W_COEF
    hb = sum(w[W_HBOND + k] * f[16 + k] for k in range(8))
    pc = sum(w[W_PICAT + k] * f[4 + k] for k in range(4))
    st = [sum(w[W_STACK + 4 * q + k] * f[8 + 4 * q + k] for k in range(4)) for q in range(2)]
    d = [0.0] * NUM_SF_WEIGHTS
    d[C + 0] = f[0]
    d[C + 1] = w[W_VDW_SCALE] * f[1]
    d[C + 2] = w[W_IONIC] * f[2] + w[W_IONIC + 1] * f[3]
    d[C + 3] = pc
    d[C + 4], d[C + 5] = st[0], st[1]
    d[C + 6] = w[W_HBOND_SCALE] * hb
    d[C + 7] = w[W_HYDRO_SCALE] * f[24]
    d[C + 8] = f[25]
    d[C + 9] = f[26]
    d[C + 10] = 0.0 * f[0]  # GB/SA is not part of the differentiable score
    d[W_VDW_SCALE] = w[C + 1] * f[1]
    d[W_HYDRO_SCALE] = w[C + 7] * f[24]
    d[W_HBOND_SCALE] = w[C + 6] * hb
    for k in range(2):
        d[W_IONIC + k] = w[C + 2] * f[2 + k]
    for k in range(4):
        d[W_PICAT + k] = w[C + 3] * f[4 + k]
    for q in range(2):
        for k in range(4):
            d[W_STACK + 4 * q + k] = w[C + 4 + q] * f[8 + 4 * q + k]
    for k in range(8):
        d[W_HBOND + k] = w[C + 6] * w[W_HBOND_SCALE] * f[16 + k]
    try:
        import torch
        if isinstance(f, torch.Tensor):
            return torch.stack([x if isinstance(x, torch.Tensor) else torch.as_tensor(x, dtype=f.dtype,
                                                                                     device=f.device) for x in d])
    except ImportError:
        pass
    import numpy as np
    return np.array(d, dtype=float)
