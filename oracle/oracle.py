"""TEST INFRASTRUCTURE: Python access to the two oracles.

  Port      oracle/lib/libpxd_oracle.so  -- FP64 C restatement (oracle/port), builds
            anywhere gcc exists; the checker on the GPU host and the CPU baseline.
  Reference oracle/_ref/liboracle_ref.so -- the reference engine compiled from its own
            sources (oracle/Makefile target `ref`); only where the checkout exists.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module, and only to check or time the reference algorithm -- never as the product.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "protenix-dock_gb300"))

from pxdock_gb300 import abi  # noqa: E402

PORT_LIB = os.path.join(HERE, "lib", "libpxd_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "liboracle_ref.so")
# the reference engine's source tree (engine/ of the reference checkout); the Makefile
# reads the same variable
REF_ENGINE = os.environ.get("REF_ENGINE", "/root/reference/engine")

f64p = abi.f64p
i32p = abi.i32p


def build(ref=None):
    """Builds the port (always) and the reference library (when its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    if ref is None:
        ref = os.path.isdir(REF_ENGINE)
    if ref:
        subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref"], check=True)


def _p(a, ctype=C.c_double):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


def _d(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


_port = None


def port_lib():
    global _port
    if _port is None:
        if not os.path.exists(PORT_LIB):
            build(ref=False)
        lib = C.CDLL(PORT_LIB)
        lib.po_dihedral.restype = C.c_double
        lib.po_dihedral_and_gradient.restype = C.c_double
        lib.po_angle_and_gradient.restype = C.c_double
        lib.po_intra_energy.restype = C.c_double
        lib.po_intra_energy.argtypes = [C.c_int, C.POINTER(abi.Topology), f64p, f64p]
        lib.po_system_create.restype = C.c_void_p
        lib.po_system_create.argtypes = [C.POINTER(abi.ReceptorDesc), C.POINTER(abi.LigandDesc)]
        lib.po_system_destroy.argtypes = [C.c_void_p]
        lib.po_build_grid.argtypes = [C.c_void_p, C.POINTER(abi.Box), i32p, C.c_int32, C.c_int]
        lib.po_set_slope.argtypes = [C.c_void_p, C.c_double]
        lib.po_drop_grid.argtypes = [C.c_void_p]
        lib.po_grid_copy.argtypes = [C.c_void_p, C.c_int, f64p]
        lib.po_grid_get.argtypes = [C.c_void_p, C.c_int, C.c_double, f64p, f64p, f64p]
        lib.po_score_grad.restype = C.c_double
        lib.po_score_grad.argtypes = [C.c_void_p, f64p, f64p, f64p, f64p]
        lib.po_lbfgs.argtypes = [C.c_void_p, C.POINTER(abi.LbfgsParams), f64p, f64p, f64p, i32p]
        lib.po_lbfgs_batch.argtypes = [C.c_void_p, C.POINTER(abi.LbfgsParams), C.c_int32, f64p,
                                       f64p, f64p, i32p, i32p, C.c_int]
        lib.po_ligand_apply.argtypes = [C.c_void_p, f64p, f64p, f64p, f64p, f64p]
        lib.po_receptor_apply.argtypes = [C.c_void_p, f64p, f64p]
        lib.po_score.restype = C.c_double
        lib.po_score.argtypes = [C.POINTER(abi.SfParams), C.c_int, f64p, f64p, f64p, f64p,
                                 C.POINTER(abi.ScoreLists), C.c_int, f64p, f64p, i32p,
                                 C.POINTER(abi.ScoreLists), f64p]
        lib.po_score_diff.restype = C.c_double
        lib.po_score_diff.argtypes = [C.POINTER(abi.SfParams), C.c_int, f64p, f64p, f64p, f64p,
                                      C.POINTER(abi.ScoreLists), C.c_int, f64p, f64p, i32p,
                                      C.POINTER(abi.ScoreLists), f64p, f64p, C.c_double, f64p, f64p, f64p,
                                      f64p]
        lib.po_combine_features.restype = C.c_double
        lib.po_combine_features.argtypes = [f64p, f64p]
        lib.po_combine_grad.restype = None
        lib.po_combine_grad.argtypes = [f64p, f64p, C.c_double, f64p]
        lib.po_vdw_check.restype = C.c_double
        lib.po_vdw_check.argtypes = [C.POINTER(abi.SfParams), C.c_int, f64p, f64p, f64p, C.c_int,
                                     f64p, i32p]
        lib.po_torsion_strain.restype = C.c_double
        lib.po_torsion_strain.argtypes = [C.POINTER(abi.ScoreLists), f64p]
        lib.po_gbsa_parts.restype = C.c_double
        lib.po_gbsa_parts.argtypes = [C.c_int, f64p, f64p, C.POINTER(abi.ScoreLists), C.c_int,
                                      f64p, f64p, C.POINTER(abi.ScoreLists), f64p]
        lib.po_mc_walker.argtypes = [C.c_void_p, C.POINTER(abi.SfParams), C.POINTER(abi.ScoreLists),
                                     C.POINTER(abi.ScoreLists), f64p, f64p, C.c_uint32, C.c_int,
                                     f64p, C.c_int, C.c_int, C.c_int, C.c_double, f64p, f64p, f64p,
                                     f64p, f64p, C.POINTER(C.c_long)]
        lib.po_mc_randomize.argtypes = [C.c_void_p, C.POINTER(abi.SfParams), f64p, f64p, C.c_uint32,
                                        C.c_int, f64p, C.c_int, f64p]
        lib.po_rng_uniform_int.restype = C.c_int
        lib.po_rng_uniform_real.restype = C.c_double
        lib.po_rng_uniform_real.argtypes = [C.c_void_p, C.c_double, C.c_double]
        lib.po_rng_torsion.restype = C.c_double
        lib.po_rng_next.restype = C.c_uint32
        _port = lib
    return _port


def ref_available():
    return os.path.exists(REF_LIB)


_ref = None


def ref_lib():
    global _ref
    if _ref is None:
        lib = C.CDLL(REF_LIB)
        for name in ("ref_dihedral_and_gradient", "ref_dihedral", "ref_angle_and_gradient",
                     "ref_intra_energy", "ref_system_score_grad", "ref_rng_uniform_real",
                     "ref_rng_torsion", "ref_system_score"):
            getattr(lib, name).restype = C.c_double
        lib.ref_last_error.restype = C.c_char_p
        lib.ref_system_create.restype = C.c_void_p
        lib.ref_system_create.argtypes = [C.c_char_p, C.c_char_p]
        lib.ref_system_destroy.argtypes = [C.c_void_p]
        lib.ref_system_counts.argtypes = [C.c_void_p, i32p]
        lib.ref_system_get_pose.argtypes = [C.c_void_p, C.c_int, f64p]
        lib.ref_system_build_grid.argtypes = [C.c_void_p] + [C.c_double] * 7 + [C.c_int, i32p]
        lib.ref_system_grid_info.argtypes = [C.c_void_p, f64p, i32p, f64p]
        lib.ref_system_grid_copy.argtypes = [C.c_void_p, C.c_int, f64p]
        lib.ref_system_set_slope.argtypes = [C.c_void_p, C.c_double]
        lib.ref_system_drop_grid.argtypes = [C.c_void_p]
        lib.ref_system_grid_get.argtypes = [C.c_void_p, C.c_int, C.c_double, f64p, f64p, f64p]
        lib.ref_system_score_grad.argtypes = [C.c_void_p, f64p, f64p, f64p, f64p]
        lib.ref_system_lbfgs.argtypes = [C.c_void_p, C.c_int, C.c_int, f64p, f64p, f64p, i32p]
        lib.ref_system_ligand_apply.argtypes = [C.c_void_p, f64p, f64p, f64p, f64p, f64p]
        lib.ref_system_receptor_apply.argtypes = [C.c_void_p, f64p, f64p]
        lib.ref_system_load_sf.argtypes = [C.c_void_p, C.c_char_p]
        lib.ref_system_score.argtypes = [C.c_void_p, C.c_int, f64p, f64p, f64p]
        lib.ref_system_mc_walker.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                             C.c_double, f64p, f64p, f64p, f64p,
                                             C.POINTER(C.c_long)]
        lib.ref_rng_create.restype = C.c_void_p
        lib.ref_rng_create.argtypes = [C.c_uint]
        lib.ref_rng_destroy.argtypes = [C.c_void_p]
        lib.ref_rng_uniform_int.argtypes = [C.c_void_p, C.c_int, C.c_int]
        lib.ref_rng_uniform_real.argtypes = [C.c_void_p, C.c_double, C.c_double]
        lib.ref_rng_torsion.argtypes = [C.c_void_p]
        lib.ref_rng_in_box.argtypes = [C.c_void_p, f64p, f64p, f64p]
        lib.ref_rng_orientation.argtypes = [C.c_void_p, f64p]
        lib.ref_rng_in_sphere.argtypes = [C.c_void_p, f64p]
        lib.ref_engine_create.restype = C.c_void_p
        lib.ref_engine_create.argtypes = [C.c_char_p, C.c_char_p, C.c_int]
        lib.ref_engine_destroy.argtypes = [C.c_void_p]
        lib.ref_engine_set_box.argtypes = [C.c_void_p] + [C.c_double] * 6
        lib.ref_engine_generate_maps.argtypes = [C.c_void_p, C.c_double, C.c_double]
        lib.ref_engine_optimize.argtypes = [C.c_void_p, C.c_char_p, C.c_char_p, C.c_int,
                                            C.c_double]
        lib.ref_engine_search.argtypes = [C.c_void_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int,
                                          C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                          C.c_double]
        lib.ref_engine_evaluate.argtypes = [C.c_void_p, C.c_char_p, C.c_char_p]
        _ref = lib
    return _ref


class PortSystem:
    """FP64 port of one receptor + ligand system."""

    def __init__(self, receptor, ligand):
        self._keep = []
        self.receptor, self.ligand = receptor, ligand
        self.rec_c = receptor.to_c(self._keep)
        self.lig_c = ligand.to_c(self._keep)
        self.lib = port_lib()
        self.h = self.lib.po_system_create(C.byref(self.rec_c), C.byref(self.lig_c))
        self.n_lig = ligand.n_atoms
        self.n_tors = receptor.n_rotors

    def close(self):
        if self.h:
            self.lib.po_system_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def build_grid(self, box, types=None, nthreads=8):
        t = np.ascontiguousarray(np.asarray([] if types is None else types, np.int32))
        n = -1 if types is None else len(t)
        self.lib.po_build_grid(self.h, C.byref(box), _p(t, C.c_int32) if t.size else None, n,
                               nthreads)

    def set_slope(self, slope):
        self.lib.po_set_slope(self.h, slope)

    def drop_grid(self):
        self.lib.po_drop_grid(self.h)

    def grid_map(self, m, box):
        P = box.npoints[0] * box.npoints[1] * box.npoints[2]
        out = np.zeros((P, 4))
        if self.lib.po_grid_copy(self.h, m, _p(out)) != 0:
            return None
        return out

    def grid_get(self, atom_type, q, xyz):
        e = np.zeros(1)
        g = np.zeros(3)
        hit = self.lib.po_grid_get(self.h, atom_type, q, _p(_d(xyz)), _p(e), _p(g))
        return e[0], g, bool(hit)

    def score_grad(self, tors, xyz):
        tors = _d(tors).reshape(-1)
        xyz = _d(xyz).reshape(-1)
        tg = np.zeros(max(self.n_tors, 1))
        lg = np.zeros(self.n_lig * 3)
        e = self.lib.po_score_grad(self.h, _p(tors) if tors.size else None, _p(xyz), _p(tg), _p(lg))
        return e, tg[: self.n_tors], lg.reshape(-1, 3)

    def lbfgs(self, params, tors, xyz):
        tors = _d(tors).reshape(-1).copy()
        xyz = _d(xyz).reshape(-1).copy()
        e = np.zeros(1)
        nev = np.zeros(1, np.int32)
        st = self.lib.po_lbfgs(self.h, C.byref(params), _p(tors) if tors.size else _p(np.zeros(1)),
                               _p(xyz), _p(e), _p(nev, C.c_int32))
        return dict(status=st, energy=e[0], nevals=int(nev[0]), torsions=tors,
                    xyz=xyz.reshape(-1, 3))

    def lbfgs_batch(self, params, tors, xyz, nthreads):
        n = xyz.shape[0]
        tors = np.ascontiguousarray(np.asarray(tors, np.float64).reshape(n, -1)).copy()
        xyz = np.ascontiguousarray(np.asarray(xyz, np.float64).reshape(n, -1)).copy()
        e = np.zeros(n)
        nev = np.zeros(n, np.int32)
        st = np.zeros(n, np.int32)
        tp = _p(tors) if tors.size else _p(np.zeros(1))
        self.lib.po_lbfgs_batch(self.h, C.byref(params), n, tp, _p(xyz), _p(e),
                                _p(nev, C.c_int32), _p(st, C.c_int32), nthreads)
        return dict(status=st, energy=e, nevals=nev, torsions=tors, xyz=xyz.reshape(n, -1, 3))

    def ligand_apply(self, xyz, center, rot, torsions):
        out = np.zeros(self.n_lig * 3)
        t = _d(torsions).reshape(-1)
        self.lib.po_ligand_apply(self.h, _p(_d(xyz).reshape(-1)), _p(_d(center)),
                                 _p(_d(rot).reshape(-1)), _p(t) if t.size else _p(np.zeros(1)),
                                 _p(out))
        return out.reshape(-1, 3)

    def receptor_apply(self, torsions):
        out = np.zeros(self.receptor.n_atoms * 3)
        t = _d(torsions).reshape(-1)
        self.lib.po_receptor_apply(self.h, _p(t) if t.size else _p(np.zeros(1)), _p(out))
        return out.reshape(-1, 3)

    def score(self, sf, rec_xyz, lig_xyz):
        """root_scorer::combine with the scoring function sf; returns (score, terms[11])."""
        return port_score(sf, self.receptor, self.ligand, rec_xyz, lig_xyz)

    def mc_walker(self, sf, lo, hi, seed, walker, start, first_pose, max_nsteps, relax_nsteps,
                  threshold=-1.0, global_min=None):
        keep = []
        rl = self.receptor.lists.to_c(keep)
        ll = self.ligand.lists.to_c(keep)
        xyz = np.zeros(self.n_lig * 3)
        tors = np.zeros(max(self.n_tors, 1))
        e, ps = np.zeros(1), np.zeros(1)
        nev = C.c_long(0)
        gm = np.array([1e8 if global_min is None else global_min])
        st = self.lib.po_mc_walker(self.h, C.byref(sf), C.byref(rl), C.byref(ll), _p(_d(lo)), _p(_d(hi)),
                                   seed, walker, _p(_d(start).reshape(-1)), int(first_pose), max_nsteps,
                                   relax_nsteps, threshold, _p(gm), _p(xyz), _p(tors), _p(e), _p(ps),
                                   C.byref(nev))
        return dict(status=st, xyz=xyz.reshape(-1, 3), torsions=tors[: self.n_tors], energy=e[0],
                    pscore=ps[0], nevals=nev.value, global_min=gm[0])

    def mc_randomize(self, sf, lo, hi, seed, walker, start, first_pose=True):
        out = np.zeros(self.n_lig * 3)
        self.lib.po_mc_randomize(self.h, C.byref(sf), _p(_d(lo)), _p(_d(hi)), seed, walker,
                                 _p(_d(start).reshape(-1)), int(first_pose), _p(out))
        return out.reshape(-1, 3)


def port_rng_draws(seed, kinds, ints):
    """The draw sequence pxd_rng_draws makes, from the port's generator."""
    lib = port_lib()

    class Rng(C.Structure):
        _fields_ = [("mt", C.c_uint32 * 624), ("idx", C.c_int)]

    r = Rng()
    lib.po_rng_seed(C.byref(r), seed)
    out = []
    for k, n in zip(kinds, ints):
        if k == 0:
            out.append(lib.po_rng_uniform_int(C.byref(r), 0, int(n)))
        elif k == 1:
            out.append(lib.po_rng_torsion(C.byref(r)))
        elif k == 2:
            out.append(lib.po_rng_uniform_real(C.byref(r), 0.0, 1.0))
        else:
            v = np.zeros(3 if k == 3 else 4)
            (lib.po_rng_in_sphere if k == 3 else lib.po_rng_orientation)(C.byref(r), _p(v))
            out.extend(v.tolist())
    return np.array(out, np.float64)


def port_score(sf, receptor, ligand, rec_xyz, lig_xyz):
    lib = port_lib()
    keep = []
    rl = receptor.lists.to_c(keep)
    ll = ligand.lists.to_c(keep)
    rx = _d(rec_xyz).reshape(-1)
    lx = _d(lig_xyz).reshape(-1)
    terms = np.zeros(11)
    v = lib.po_score(C.byref(sf), receptor.n_atoms, _p(rx), _p(receptor.ff.charge),
                     _p(receptor.ff.sigma), _p(receptor.ff.epsilon), C.byref(rl), ligand.n_atoms,
                     _p(lx), _p(ligand.ff.charge), _p(ligand.vdw_type, C.c_int32), C.byref(ll),
                     _p(terms))
    return v, terms


def port_score_diff(sf, receptor, ligand, rec_xyz, lig_xyz, weights, table=None, g=1.0, grads=True):
    """FP64 differentiable empirical score of one pose: (score, features[28], and with
    grads: g dS/dx [N][3], g dS/dw [36], g dS/dT [32*256])."""
    lib = port_lib()
    keep = []
    rl = receptor.lists.to_c(keep)
    ll = ligand.lists.to_c(keep)
    rx = _d(rec_xyz).reshape(-1)
    lx = _d(lig_xyz).reshape(-1)
    w = _d(weights)
    tab = None if table is None else _d(table).reshape(-1)
    f = np.zeros(28)
    gx = np.zeros(ligand.n_atoms * 3) if grads else None
    gw = np.zeros(36) if grads else None
    gt = np.zeros(32 * 256) if grads and tab is not None else None
    v = lib.po_score_diff(C.byref(sf), receptor.n_atoms, _p(rx), _p(receptor.ff.charge), _p(receptor.ff.sigma),
                          _p(receptor.ff.epsilon), C.byref(rl), ligand.n_atoms, _p(lx), _p(ligand.ff.charge),
                          _p(ligand.vdw_type, C.c_int32), C.byref(ll), _p(w), _p(tab), g, _p(f), _p(gx), _p(gw),
                          _p(gt))
    if not grads:
        return v, f
    return v, f, gx.reshape(-1, 3), gw, gt


class RefSystem:
    """The reference engine's own classes on one receptor + ligand JSON pair."""

    def __init__(self, receptor_json, ligand_json):
        self.lib = ref_lib()
        self.h = self.lib.ref_system_create(receptor_json.encode(), ligand_json.encode())
        if not self.h:
            raise RuntimeError(self.lib.ref_last_error().decode())
        c = np.zeros(6, np.int32)
        self.lib.ref_system_counts(self.h, _p(c, C.c_int32))
        self.n_lig, self.n_rec, self.n_tors, self.n_lig_tors, self.n_poses, self.n_mov = map(int, c)

    def close(self):
        if self.h:
            self.lib.ref_system_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def pose(self, i):
        out = np.zeros(self.n_lig * 3)
        self.lib.ref_system_get_pose(self.h, i, _p(out))
        return out.reshape(-1, 3)

    def build_grid(self, center, size, spacing, nthreads=8):
        npts = np.zeros(3, np.int32)
        self.lib.ref_system_build_grid(self.h, *center, *size, spacing, nthreads,
                                       _p(npts, C.c_int32))
        return npts

    def grid_map(self, m):
        init = np.zeros(3)
        npts = np.zeros(3, np.int32)
        sp = np.zeros(1)
        self.lib.ref_system_grid_info(self.h, _p(init), _p(npts, C.c_int32), _p(sp))
        out = np.zeros((int(np.prod(npts)), 4))
        self.lib.ref_system_grid_copy(self.h, m, _p(out))
        return out

    def set_slope(self, s):
        self.lib.ref_system_set_slope(self.h, s)

    def drop_grid(self):
        self.lib.ref_system_drop_grid(self.h)

    def grid_get(self, atom_type, q, xyz):
        e = np.zeros(1)
        g = np.zeros(3)
        hit = self.lib.ref_system_grid_get(self.h, atom_type, q, _p(_d(xyz)), _p(e), _p(g))
        return e[0], g, bool(hit)

    def score_grad(self, tors, xyz):
        tors = _d(tors).reshape(-1)
        tg = np.zeros(max(self.n_tors, 1))
        lg = np.zeros(self.n_lig * 3)
        e = self.lib.ref_system_score_grad(self.h, _p(tors) if tors.size else _p(np.zeros(1)),
                                           _p(_d(xyz).reshape(-1)), _p(tg), _p(lg))
        return e, tg[: self.n_tors], lg.reshape(-1, 3)

    def lbfgs(self, max_iter, max_eval, tors, xyz):
        tors = _d(tors).reshape(-1).copy()
        xyz = _d(xyz).reshape(-1).copy()
        e = np.zeros(1)
        nev = np.zeros(1, np.int32)
        conv = self.lib.ref_system_lbfgs(self.h, max_iter, max_eval,
                                         _p(tors) if tors.size else _p(np.zeros(1)), _p(xyz),
                                         _p(e), _p(nev, C.c_int32))
        return dict(converged=bool(conv), energy=e[0], nevals=int(nev[0]), torsions=tors,
                    xyz=xyz.reshape(-1, 3))

    def ligand_apply(self, xyz, center, rot, torsions):
        out = np.zeros(self.n_lig * 3 if self.n_lig else _d(xyz).size)
        t = _d(torsions).reshape(-1)
        self.lib.ref_system_ligand_apply(self.h, _p(_d(xyz).reshape(-1)), _p(_d(center)),
                                         _p(_d(rot).reshape(-1)),
                                         _p(t) if t.size else _p(np.zeros(1)), _p(out))
        return out.reshape(-1, 3)

    def receptor_apply(self, torsions):
        out = np.zeros(self.n_rec * 3)
        t = _d(torsions).reshape(-1)
        self.lib.ref_system_receptor_apply(self.h, _p(t) if t.size else _p(np.zeros(1)), _p(out))
        return out.reshape(-1, 3)

    def load_sf(self, path):
        if self.lib.ref_system_load_sf(self.h, path.encode()) != 0:
            raise RuntimeError(self.lib.ref_last_error().decode())

    def score(self, which, rec_xyz, lig_xyz):
        terms = np.zeros(11)
        v = self.lib.ref_system_score(self.h, which, _p(_d(rec_xyz).reshape(-1)),
                                      _p(_d(lig_xyz).reshape(-1)), _p(terms))
        return v, terms

    def mc_walker(self, seed, pose_id, max_nsteps, relax_nsteps, threshold=-1.0):
        xyz = np.zeros(self.n_lig * 3)
        tors = np.zeros(max(self.n_tors, 1))
        e = np.zeros(1)
        ps = np.zeros(1)
        nev = C.c_long(0)
        rc = self.lib.ref_system_mc_walker(self.h, seed, pose_id, max_nsteps, relax_nsteps,
                                           threshold, _p(xyz), _p(tors), _p(e), _p(ps),
                                           C.byref(nev))
        if rc != 0:
            raise RuntimeError(self.lib.ref_last_error().decode())
        return dict(xyz=xyz.reshape(-1, 3), torsions=tors[: self.n_tors], energy=e[0],
                    pscore=ps[0], nevals=nev.value)


# ------------------------------------------------------------------ optimiser outcomes
# Optimiser outcomes of two runs over the same starting poses, for
# tests/test_gpu_headline.py and bench.py's CPU-baseline leg: evaluations per pose,
# status counts, final-energy quartiles and the fraction of poses that end within
# 0.05 A RMSD (lbfgs_step::apply, optimizer.cpp:429-560, on both sides).

OUTCOME_STATUS = ("converged", "not_converged", "nan", "bad_input")


def pose_rmsd(a, b):
    """Per-pose RMSD of [P][N][3] coordinate arrays."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.sqrt(np.mean(np.sum((a - b) ** 2, axis=-1), axis=-1))


def outcome_summary(run):
    """Population figures of one run (dict with energy, nevals, status)."""
    st = np.asarray(run["status"])
    e = np.asarray(run["energy"], np.float64)
    return {
        "evals_per_pose": float(np.mean(run["nevals"])),
        "status": {n: int((st == k).sum()) for k, n in enumerate(OUTCOME_STATUS)},
        "energy_quartiles": [float(v) for v in np.percentile(e, [25, 50, 75])],
    }


def compare_outcomes(run, ref, tol_rmsd=0.05):
    """Figures of `run` against `ref` over the same starts (both dicts with xyz, energy,
    nevals, status)."""
    d = pose_rmsd(run["xyz"], ref["xyz"])
    return {
        "poses": int(len(d)),
        "within_rmsd": float(np.mean(d <= tol_rmsd)),
        "tol_rmsd": tol_rmsd,
        "run": outcome_summary(run),
        "ref": outcome_summary(ref),
    }

