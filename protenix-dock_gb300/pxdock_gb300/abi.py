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


class LigandDesc(C.Structure):
    _fields_ = [("ff", Topology), ("vdw_type", i32p), ("tree", TorsionTree)]


class ReceptorDesc(C.Structure):
    _fields_ = [
        ("n_atoms", C.c_int32),
        ("xyz", f64p),
        ("ff", Topology),
        ("n_rotors", C.c_int32),
        ("rotor_axis", i32p),
        ("rotor_offsets", i32p),
        ("rotor_atoms", i32p),
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
    ]


def lbfgs_params(max_iter=240, max_eval=0, history=100, tolerance_grad=0.5,
                 tolerance_change=1e-4, lr=1.0):
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
    return p


POSE_CONVERGED = 0
POSE_NOT_CONVERGED = 1
POSE_NAN = 2
POSE_BAD_INPUT = 3
NUM_VDW_TYPES = 99
COULOMB_MAP = 99
