"""ctypes binding of libpxdock_gb300.so (the C ABI in include/pxdock_gb300.h).

The library is required: importing this module without a built library raises, and
every call that reports an error status raises NativeError with the library's message.
There is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

from . import abi, build

_lib = None


class NativeError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("pxdock_gb300 error %d: %s" % (code, msg))
        self.code = code


def load(auto_build=False):
    """Loads the native library (building it first when auto_build is set)."""
    global _lib
    if _lib is not None:
        return _lib
    path = build.lib_path()
    if auto_build:
        path = build.build()
    if not os.path.exists(path):
        raise RuntimeError("native library %s is missing: run build() first" % path)
    lib = C.CDLL(path)
    vp = C.c_void_p
    lib.pxd_abi_version.restype = C.c_int32
    lib.pxd_version.restype = C.c_char_p
    lib.pxd_context_create.argtypes = [C.c_int32, C.POINTER(vp)]
    lib.pxd_context_destroy.argtypes = [vp]
    lib.pxd_last_error.argtypes = [vp]
    lib.pxd_last_error.restype = C.c_char_p
    lib.pxd_context_stream.argtypes = [vp]
    lib.pxd_context_stream.restype = vp
    lib.pxd_lbfgs_defaults.argtypes = [C.POINTER(abi.LbfgsParams)]
    lib.pxd_set_receptor.argtypes = [vp, C.POINTER(abi.ReceptorDesc)]
    lib.pxd_decide_grid_dims.argtypes = [C.c_double] * 7 + [C.POINTER(abi.Box)]
    lib.pxd_grid_build.argtypes = [vp, C.POINTER(abi.Box), abi.i32p, C.c_int32]
    lib.pxd_grid_set_slope.argtypes = [vp, C.c_double]
    lib.pxd_grid_drop.argtypes = [vp]
    lib.pxd_grid_info.argtypes = [vp, C.POINTER(abi.Box), abi.i32p]
    lib.pxd_grid_read_map.argtypes = [vp, C.c_int32, abi.f32p]
    lib.pxd_grid_write_map.argtypes = [vp, C.POINTER(abi.Box), C.c_int32, abi.f32p]
    lib.pxd_grid_read_map64.argtypes = [vp, C.c_int32, abi.f64p]
    lib.pxd_grid_write_map64.argtypes = [vp, C.POINTER(abi.Box), C.c_int32, abi.f64p]
    lib.pxd_bdg_encode.argtypes = [abi.f64p, C.c_int64, C.c_int32, C.c_char_p, C.c_int64]
    lib.pxd_bdg_encode.restype = C.c_int64
    lib.pxd_bdg_decode.argtypes = [C.c_char_p, C.c_int64, abi.f64p, C.c_int64, abi.i32p]
    lib.pxd_bdg_decode.restype = C.c_int64
    lib.pxd_meta_encode.argtypes = [C.POINTER(abi.Box), C.POINTER(C.c_int64), C.c_int64, C.c_char_p, C.c_int64]
    lib.pxd_meta_encode.restype = C.c_int64
    lib.pxd_meta_decode.argtypes = [C.c_char_p, C.c_int64, C.POINTER(abi.Box), C.POINTER(C.c_uint64),
                                    C.POINTER(C.c_int64), C.c_int64]
    lib.pxd_meta_decode.restype = C.c_int64
    lib.pxd_add_ligand.argtypes = [vp, C.POINTER(abi.LigandDesc), abi.i32p]
    lib.pxd_clear_ligands.argtypes = [vp]
    lib.pxd_score_grad_dev.argtypes = [vp, C.c_int32, C.c_int32, vp, vp, vp, vp, vp, vp, vp]
    lib.pxd_score_grad.argtypes = [vp, C.c_int32, C.c_int32, abi.f64p, abi.f64p, abi.f64p,
                                   abi.f64p, abi.f64p]
    lib.pxd_lbfgs_dev.argtypes = [vp, C.POINTER(abi.LbfgsParams), C.c_int32, C.c_int32, vp, vp, vp,
                                  vp, vp, vp, vp]
    lib.pxd_lbfgs_dev_noalloc.argtypes = lib.pxd_lbfgs_dev.argtypes
    lib.pxd_lbfgs.argtypes = [vp, C.POINTER(abi.LbfgsParams), C.c_int32, C.c_int32, abi.f64p,
                              abi.f64p, abi.f64p, abi.i32p, abi.i32p]
    lib.pxd_ligand_kinematics.argtypes = [vp, C.c_int32, C.c_int32, abi.f64p, abi.f64p, abi.f64p,
                                          abi.f64p, abi.f64p]
    lib.pxd_ligand_backward.argtypes = [vp, C.c_int32, C.c_int32] + [abi.f64p] * 6
    lib.pxd_receptor_kinematics.argtypes = [vp, C.c_int32, abi.f64p, abi.f64p]
    lib.pxd_set_scoring_function.argtypes = [vp, C.c_int32, C.POINTER(abi.SfParams)]
    lib.pxd_score_dev.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, vp, vp, vp, vp, vp, vp]
    lib.pxd_score.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, abi.f64p, abi.f64p, abi.f64p,
                              abi.f64p]
    lib.pxd_score_gbsa.argtypes = [vp, C.c_int32, abi.f64p, abi.f64p, abi.f64p, abi.f64p]
    lib.pxd_mc_defaults.argtypes = [C.POINTER(abi.McParams)]
    lib.pxd_mc_search_dev.argtypes = [vp, C.POINTER(abi.McParams), C.c_int32, C.c_int32] + [vp] * 12
    lib.pxd_mc_search.argtypes = [vp, C.POINTER(abi.McParams), C.c_int32, C.c_int32, abi.i32p,
                                  abi.i32p, abi.f64p, abi.f64p, abi.f64p, abi.f64p, abi.f64p,
                                  abi.i32p, abi.i32p]
    lib.pxd_lbfgs_multi.argtypes = [vp, C.POINTER(abi.LbfgsParams), C.c_int32, C.c_int32, abi.i32p,
                                    abi.f64p, abi.f64p, abi.f64p, abi.i32p, abi.i32p]
    lib.pxd_mc_search_multi.argtypes = [vp, C.POINTER(abi.McParams), C.c_int32, C.c_int32, abi.i32p,
                                        abi.i32p, abi.i32p, abi.f64p, abi.f64p, abi.f64p, abi.f64p,
                                        abi.f64p, abi.i32p, abi.i32p, abi.f64p]
    lib.pxd_rng_draws.argtypes = [vp, C.c_uint32, C.c_int32, abi.i32p, abi.i32p, abi.f64p]
    lib.pxd_gather_bandwidth.argtypes = [C.c_int32, C.c_int64, C.c_int32, abi.f64p]
    lib.pxd_set_l2_residency.argtypes = [vp, C.c_double]
    lib.pxd_sf_weights.argtypes = [C.POINTER(abi.SfParams), abi.f64p]
    lib.pxd_sf_weights.restype = None
    lib.pxd_score_adjoint_dev.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32] + [vp] * 12
    lib.pxd_score_adjoint.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32] + [abi.f64p] * 10
    lib.pxd_score_adjoint_multi_dev.argtypes = [C.POINTER(vp), C.c_int32, C.c_int32, C.c_int32, C.c_int32] + [vp] * 13
    lib.pxd_ligand_pose_multi_dev.argtypes = [C.POINTER(vp), C.c_int32, C.c_int32, C.c_int32, C.c_int32] + [vp] * 8
    lib.pxd_score_grad_multi_dev.argtypes = [C.POINTER(vp), C.c_int32, C.c_int32, C.c_int32] + [vp] * 8
    lib.pxd_score_hvp_multi_dev.argtypes = [C.POINTER(vp), C.c_int32, C.c_int32, C.c_int32, C.c_int32] + [vp] * 13
    lib.pxd_lbfgs_autotune_dev.argtypes = [vp, C.POINTER(abi.LbfgsParams), C.c_int32, C.c_int32, vp, vp, vp,
                                           C.c_int32, C.c_int32, abi.i32p, vp]
    lib.pxd_lbfgs_set_variant.argtypes = [vp, C.c_int32, C.c_int32]
    lib.pxd_ligand_pose_dir_multi_dev.argtypes = [C.POINTER(vp), C.c_int32, C.c_int32, C.c_int32, C.c_int32] + [vp] * 10
    lib.pxd_ligand_pose_dev.argtypes = [vp, C.c_int32, C.c_int32] + [vp] * 6
    lib.pxd_ligand_pose_backward_dev.argtypes = [vp, C.c_int32, C.c_int32] + [vp] * 8
    _lib = lib
    return lib


LBFGS_HIST_SMEM = 256  # PXD_LBFGS_HIST_SMEM: a variant's history-in-shared-memory flag


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def ligand_pose_multi_dev(contexts, n_poses, max_atoms, dof, ctx_ids_ptr, lig_ids_ptr, xyz_ref_ptr, dofs_ptr,
                          xyz_ptr, atom_grad_ptr, dofs_grad_ptr, stream=None):
    """pxd_ligand_pose_multi_dev over a list of Contexts (forward, or backward with atom_grad)."""
    lib = load()
    arr = (C.c_void_p * len(contexts))(*[c.h.value for c in contexts])
    rc = lib.pxd_ligand_pose_multi_dev(arr, len(contexts), n_poses, max_atoms, dof, ctx_ids_ptr, lig_ids_ptr,
                                       xyz_ref_ptr, dofs_ptr, xyz_ptr, atom_grad_ptr, dofs_grad_ptr, stream)
    if rc != 0:
        raise NativeError(rc, lib.pxd_last_error(contexts[0].h).decode())


def score_grad_multi_dev(contexts, n_poses, max_atoms, ctx_ids_ptr, ids_ptr, xyz_ptr, tors_ptr, energy_ptr,
                         lig_grad_ptr, tors_grad_ptr, stream=None):
    """pxd_score_grad_multi_dev over a list of Contexts (integer device addresses)."""
    lib = load()
    arr = (C.c_void_p * len(contexts))(*[c.h.value for c in contexts])
    rc = lib.pxd_score_grad_multi_dev(arr, len(contexts), n_poses, max_atoms, ctx_ids_ptr, ids_ptr, xyz_ptr, tors_ptr,
                                      energy_ptr, lig_grad_ptr, tors_grad_ptr, stream)
    if rc != 0:
        raise NativeError(rc, lib.pxd_last_error(contexts[0].h).decode())


def ligand_pose_dir_multi_dev(contexts, n_poses, max_atoms, dof, ctx_ids_ptr, lig_ids_ptr, xyz_ptr, dofs_ptr,
                              dofs_dir_ptr, xyz_dir_ptr, atom_grad_ptr, atom_grad_dir_ptr, out_dir_ptr, stream=None):
    """pxd_ligand_pose_dir_multi_dev: kinematics JVP, or the derivative of the pose backward."""
    lib = load()
    arr = (C.c_void_p * len(contexts))(*[c.h.value for c in contexts])
    rc = lib.pxd_ligand_pose_dir_multi_dev(arr, len(contexts), n_poses, max_atoms, dof, ctx_ids_ptr, lig_ids_ptr,
                                           xyz_ptr, dofs_ptr, dofs_dir_ptr, xyz_dir_ptr, atom_grad_ptr,
                                           atom_grad_dir_ptr, out_dir_ptr, stream)
    if rc != 0:
        raise NativeError(rc, lib.pxd_last_error(contexts[0].h).decode())


def score_hvp_multi_dev(contexts, which, n_poses, max_atoms, ctx_ids_ptr, ids_ptr, xyz_ptr, xyz_dir_ptr, tors_ptr,
                        weights_ptr, tables_ptr, grad_out_ptr, features_dir_ptr, dxyz_dir_ptr, dweights_dir_ptr,
                        dtables_dir_ptr, stream=None):
    """pxd_score_hvp_multi_dev over a list of Contexts (integer device addresses)."""
    lib = load()
    arr = (C.c_void_p * len(contexts))(*[c.h.value for c in contexts])
    rc = lib.pxd_score_hvp_multi_dev(arr, len(contexts), which, n_poses, max_atoms, ctx_ids_ptr, ids_ptr, xyz_ptr,
                                     xyz_dir_ptr, tors_ptr, weights_ptr, tables_ptr, grad_out_ptr, features_dir_ptr,
                                     dxyz_dir_ptr, dweights_dir_ptr, dtables_dir_ptr, stream)
    if rc != 0:
        raise NativeError(rc, lib.pxd_last_error(contexts[0].h).decode())


def score_adjoint_multi_dev(contexts, which, n_poses, max_atoms, ctx_ids_ptr, ids_ptr, xyz_ptr, tors_ptr,
                            weights_ptr, tables_ptr, grad_out_ptr, score_ptr, features_ptr, dxyz_ptr, dweights_ptr,
                            dtables_ptr, stream=None):
    """pxd_score_adjoint_multi_dev over a list of Contexts (integer device addresses)."""
    lib = load()
    arr = (C.c_void_p * len(contexts))(*[c.h.value for c in contexts])
    rc = lib.pxd_score_adjoint_multi_dev(arr, len(contexts), which, n_poses, max_atoms, ctx_ids_ptr, ids_ptr, xyz_ptr,
                                         tors_ptr, weights_ptr, tables_ptr, grad_out_ptr, score_ptr, features_ptr,
                                         dxyz_ptr, dweights_ptr, dtables_ptr, stream)
    if rc != 0:
        raise NativeError(rc, lib.pxd_last_error(contexts[0].h).decode())


class Context:
    """One receptor on one GPU (pxd_context)."""

    def __init__(self, device=0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.pxd_context_create(device, C.byref(h))
        if rc != 0:
            raise NativeError(rc, "cannot create a context on CUDA device %d" % device)
        self.h = h
        self._keep = []
        self.ligands = []
        self.n_rotors = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.pxd_context_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        if rc != 0:
            raise NativeError(rc, self.lib.pxd_last_error(self.h).decode())

    @property
    def stream(self):
        return self.lib.pxd_context_stream(self.h)

    def set_receptor(self, receptor):
        keep = []
        desc = receptor.to_c(keep)
        self._check(self.lib.pxd_set_receptor(self.h, C.byref(desc)))
        self.n_rotors = receptor.n_rotors
        self.receptor = receptor

    def build_grid(self, box, types=None):
        if types is None:
            self._check(self.lib.pxd_grid_build(self.h, C.byref(box), None, -1))
        else:
            t = np.ascontiguousarray(np.asarray(sorted(set(int(x) for x in types)), np.int32))
            self._check(self.lib.pxd_grid_build(self.h, C.byref(box), _p(t, C.c_int32), len(t)))
        self.box = box

    def set_slope(self, slope):
        self._check(self.lib.pxd_grid_set_slope(self.h, slope))

    def drop_grid(self):
        self._check(self.lib.pxd_grid_drop(self.h))

    def read_map(self, m):
        box = abi.Box()
        n = C.c_int32()
        self._check(self.lib.pxd_grid_info(self.h, C.byref(box), C.byref(n)))
        P = box.npoints[0] * box.npoints[1] * box.npoints[2]
        out = np.zeros((P, 4), np.float32)
        self._check(self.lib.pxd_grid_read_map(self.h, m, _p(out, C.c_float)))
        return out

    def write_map(self, box, m, records):
        r = np.ascontiguousarray(np.asarray(records, np.float32))
        self._check(self.lib.pxd_grid_write_map(self.h, C.byref(box), m, _p(r, C.c_float)))

    def add_ligand(self, ligand):
        keep = []
        desc = ligand.to_c(keep)
        lid = C.c_int32()
        self._check(self.lib.pxd_add_ligand(self.h, C.byref(desc), C.byref(lid)))
        self.ligands.append(ligand)
        return lid.value

    def clear_ligands(self):
        self._check(self.lib.pxd_clear_ligands(self.h))
        self.ligands = []

    def score_grad(self, lig, xyz, tors=None):
        xyz = _f64(xyz)
        n = xyz.shape[0] if xyz.ndim == 3 else 1
        N = self.ligands[lig].n_atoms
        xyz = xyz.reshape(n, N, 3)
        tors = _f64(np.zeros((n, self.n_rotors)) if tors is None else tors).reshape(n, self.n_rotors)
        e = np.zeros(n)
        g = np.zeros((n, N, 3))
        tg = np.zeros((n, self.n_rotors))
        dummy = np.zeros(1)
        self._check(self.lib.pxd_score_grad(self.h, lig, n, _p(xyz), _p(tors if tors.size else dummy),
                                            _p(e), _p(g), _p(tg if tg.size else dummy)))
        return e, g, tg

    def lbfgs(self, params, lig, xyz, tors=None):
        xyz = _f64(xyz)
        n = xyz.shape[0] if xyz.ndim == 3 else 1
        N = self.ligands[lig].n_atoms
        xyz = xyz.reshape(n, N, 3).copy()
        tors = _f64(np.zeros((n, self.n_rotors)) if tors is None else tors).reshape(n, self.n_rotors).copy()
        e = np.zeros(n)
        nev = np.zeros(n, np.int32)
        st = np.zeros(n, np.int32)
        dummy = np.zeros(1)
        self._check(self.lib.pxd_lbfgs(self.h, C.byref(params), lig, n, _p(xyz),
                                       _p(tors if tors.size else dummy), _p(e), _p(nev, C.c_int32),
                                       _p(st, C.c_int32)))
        return dict(xyz=xyz, torsions=tors, energy=e, nevals=nev, status=st)

    def lbfgs_inplace(self, params, lig, xyz, tors, energy, nevals, status):
        """pxd_lbfgs on the caller's arrays, in place as the C call works (no copies):
        xyz [n][N][3] float64 C-contiguous (the starts in, the optimised poses out), tors
        [n][R] float64, energy [n] float64, nevals / status [n] int32."""
        n = xyz.shape[0]
        for a, t in ((xyz, np.float64), (tors, np.float64), (energy, np.float64), (nevals, np.int32),
                     (status, np.int32)):
            if a.dtype != t or not a.flags["C_CONTIGUOUS"]:
                raise ValueError("lbfgs_inplace needs C-contiguous %s arrays" % np.dtype(t).name)
        dummy = np.zeros(1)
        self._check(self.lib.pxd_lbfgs(self.h, C.byref(params), lig, n, _p(xyz),
                                       _p(tors if tors.size else dummy), _p(energy), _p(nevals, C.c_int32),
                                       _p(status, C.c_int32)))

    def score_grad_dev(self, n_poses, max_atoms, ids_ptr, xyz_ptr, tors_ptr, energy_ptr,
                       lig_grad_ptr, tors_grad_ptr, stream=None):
        """Device-pointer call; pointers are integer device addresses."""
        self._check(self.lib.pxd_score_grad_dev(self.h, n_poses, max_atoms, ids_ptr, xyz_ptr,
                                                tors_ptr, energy_ptr, lig_grad_ptr, tors_grad_ptr,
                                                stream))

    def set_l2_residency(self, fraction):
        """pxd_set_l2_residency: keep `fraction` of the persisting L2 for this context's
        maps on its optimiser and search launches (0 turns it off)."""
        self._check(self.lib.pxd_set_l2_residency(self.h, float(fraction)))

    def lbfgs_dev(self, params, n_poses, max_atoms, ids_ptr, xyz_ptr, tors_ptr, energy_ptr,
                  nevals_ptr, status_ptr, stream=None):
        self._check(self.lib.pxd_lbfgs_dev(self.h, C.byref(params), n_poses, max_atoms, ids_ptr,
                                           xyz_ptr, tors_ptr, energy_ptr, nevals_ptr, status_ptr,
                                           stream))

    def lbfgs_autotune_dev(self, params, n_poses, max_atoms, ids_ptr, xyz_ptr, tors_ptr, sample=2048, probe_iters=40,
                           stream=None):
        """pxd_lbfgs_autotune_dev: times the optimiser's variants per size class on a sample of
        the batch and keeps the fastest; returns {class bound: chosen variant}."""
        rep = np.zeros(16, np.int32)
        self._check(self.lib.pxd_lbfgs_autotune_dev(self.h, C.byref(params), n_poses, max_atoms, ids_ptr, xyz_ptr,
                                                    tors_ptr, sample, probe_iters, _p(rep, C.c_int32), stream))
        return {int(rep[2 * k]): int(rep[2 * k + 1]) for k in range(8) if rep[2 * k] >= 0}

    def lbfgs_set_variant(self, class_bound, variant):
        """pxd_lbfgs_set_variant: pins the optimiser variant of one size class (-1: default)."""
        self._check(self.lib.pxd_lbfgs_set_variant(self.h, class_bound, variant))

    def lbfgs_dev_noalloc(self, params, n_poses, max_atoms, ids_ptr, xyz_ptr, tors_ptr, energy_ptr,
                          nevals_ptr, status_ptr, stream=None):
        """pxd_lbfgs_dev_noalloc: the batched optimiser without device allocations."""
        self._check(self.lib.pxd_lbfgs_dev_noalloc(self.h, C.byref(params), n_poses, max_atoms, ids_ptr,
                                                   xyz_ptr, tors_ptr, energy_ptr, nevals_ptr,
                                                   status_ptr, stream))

    def ligand_kinematics(self, lig, xyz, centers, rots, torsions):
        centers = _f64(centers).reshape(-1, 3)
        n = centers.shape[0]
        N = self.ligands[lig].n_atoms
        T = self.ligands[lig].n_torsions
        rots = _f64(rots).reshape(n, 9)
        tors = _f64(torsions).reshape(n, T) if T else np.zeros((n, 1))
        out = np.zeros((n, N, 3))
        self._check(self.lib.pxd_ligand_kinematics(self.h, lig, n, _p(_f64(xyz).reshape(-1)),
                                                   _p(centers), _p(rots), _p(tors), _p(out)))
        return out

    def ligand_backward(self, lig, xyz, centers, atom_grad):
        """(dE/dcentre [P][3], torque [P][3], dE/dtorsion [P][T]) from dE/dx at poses xyz."""
        N = self.ligands[lig].n_atoms
        T = self.ligands[lig].n_torsions
        xyz = _f64(xyz).reshape(-1, N, 3)
        n = xyz.shape[0]
        g = _f64(atom_grad).reshape(n, N, 3)
        c = _f64(centers).reshape(n, 3)
        oc, oq = np.zeros((n, 3)), np.zeros((n, 3))
        ot = np.zeros((n, max(T, 1)))
        self._check(self.lib.pxd_ligand_backward(self.h, lig, n, _p(xyz), _p(c), _p(g), _p(oc), _p(oq), _p(ot)))
        return oc, oq, ot[:, :T]

    def set_scoring_function(self, which, params):
        self._check(self.lib.pxd_set_scoring_function(self.h, which, C.byref(params)))

    def score(self, which, lig, xyz, tors=None):
        """Empirical score (0: pose selection, 1: affinity) of poses; returns (score, terms)."""
        xyz = _f64(xyz)
        N = self.ligands[lig].n_atoms
        xyz = xyz.reshape(-1, N, 3)
        n = xyz.shape[0]
        tors = _f64(np.zeros((n, self.n_rotors)) if tors is None else tors).reshape(n, self.n_rotors)
        s = np.zeros(n)
        terms = np.zeros((n, 11))
        dummy = np.zeros(1)
        self._check(self.lib.pxd_score(self.h, which, lig, n, _p(xyz),
                                       _p(tors if tors.size else dummy), _p(s), _p(terms)))
        return s, terms

    def score_adjoint(self, which, lig, xyz, weights, tables=None, grad_out=None, tors=None, grads=True):
        """Differentiable empirical score of poses of one ligand (pxd_score_adjoint):
        returns (score [P], features [P][28]) and, with grads, (dxyz [P][N][3], dweights [36],
        dtables [32][256]) of sum_p grad_out_p * S_p (grad_out defaults to ones)."""
        N = self.ligands[lig].n_atoms
        xyz = _f64(xyz).reshape(-1, N, 3)
        n = xyz.shape[0]
        tors = _f64(np.zeros((n, self.n_rotors)) if tors is None else tors).reshape(n, self.n_rotors)
        dummy = np.zeros(1)
        w = _f64(weights).reshape(abi.NUM_SF_WEIGHTS)
        tab = None if tables is None else _f64(tables).reshape(-1)
        g = None if grad_out is None else _f64(grad_out).reshape(n)
        s = np.zeros(n)
        f = np.zeros((n, abi.NUM_SCORE_FEATURES))
        dx = np.zeros((n, N, 3)) if grads else None
        dw = np.zeros(abi.NUM_SF_WEIGHTS) if grads else None
        dt = np.zeros(abi.PAIR_TYPES * abi.PAIR_BINS) if grads else None
        opt = lambda a: None if a is None else _p(a)
        self._check(self.lib.pxd_score_adjoint(self.h, which, lig, n, _p(xyz), _p(tors if tors.size else dummy),
                                               _p(w), opt(tab), opt(g), _p(s), _p(f), opt(dx), opt(dw), opt(dt)))
        if not grads:
            return s, f
        return s, f, dx, dw, dt.reshape(abi.PAIR_TYPES, abi.PAIR_BINS)

    def score_adjoint_dev(self, which, n_poses, max_atoms, ids_ptr, xyz_ptr, tors_ptr, weights_ptr, tables_ptr,
                          grad_out_ptr, score_ptr, features_ptr, dxyz_ptr, dweights_ptr, dtables_ptr, stream=None):
        """pxd_score_adjoint_dev on integer device addresses (None for NULL)."""
        self._check(self.lib.pxd_score_adjoint_dev(self.h, which, n_poses, max_atoms, ids_ptr, xyz_ptr, tors_ptr,
                                                   weights_ptr, tables_ptr, grad_out_ptr, score_ptr, features_ptr,
                                                   dxyz_ptr, dweights_ptr, dtables_ptr, stream))

    def ligand_pose_dev(self, lig, n_poses, xyz_in_ptr, centers_ptr, quats_ptr, tors_ptr, out_ptr, stream=None):
        self._check(self.lib.pxd_ligand_pose_dev(self.h, lig, n_poses, xyz_in_ptr, centers_ptr, quats_ptr, tors_ptr,
                                                 out_ptr, stream))

    def ligand_pose_backward_dev(self, lig, n_poses, xyz_ptr, centers_ptr, quats_ptr, grad_ptr, out_center_ptr,
                                 out_quat_ptr, out_tors_ptr, stream=None):
        self._check(self.lib.pxd_ligand_pose_backward_dev(self.h, lig, n_poses, xyz_ptr, centers_ptr, quats_ptr,
                                                          grad_ptr, out_center_ptr, out_quat_ptr, out_tors_ptr,
                                                          stream))

    def gbsa(self, lig, xyz, tors=None):
        xyz = _f64(xyz).reshape(-1)
        tors = _f64(np.zeros(self.n_rotors) if tors is None else tors).reshape(-1)
        d = np.zeros(1)
        parts = np.zeros(3)
        self._check(self.lib.pxd_score_gbsa(self.h, lig, _p(xyz), _p(tors if tors.size else np.zeros(1)),
                                            _p(d), _p(parts)))
        return d[0], parts

    def mc_search(self, params, lig, starts, walker_ids, first_pose=None):
        """Monte-Carlo walkers of one ligand: starts [W][N][3] (the pose each walker starts
        from), walker_ids [W] (seed offsets; walker 0 only relaxes)."""
        N = self.ligands[lig].n_atoms
        starts = _f64(starts).reshape(-1, N, 3)
        W = starts.shape[0]
        wid = np.ascontiguousarray(np.asarray(walker_ids, np.int32).reshape(W))
        fp = np.ascontiguousarray(np.ones(W, np.int32) if first_pose is None
                                  else np.asarray(first_pose, np.int32).reshape(W))
        out = np.zeros((W, N, 3))
        tors = np.zeros((W, max(self.n_rotors, 1)))
        e, ps = np.zeros(W), np.zeros(W)
        nev, st = np.zeros(W, np.int32), np.zeros(W, np.int32)
        self._check(self.lib.pxd_mc_search(self.h, C.byref(params), lig, W, _p(wid, C.c_int32),
                                           _p(fp, C.c_int32), _p(starts), _p(out), _p(tors), _p(e),
                                           _p(ps), _p(nev, C.c_int32), _p(st, C.c_int32)))
        return dict(xyz=out, torsions=tors[:, : self.n_rotors], energy=e, pscore=ps, nevals=nev,
                    status=st)

    def lbfgs_multi(self, params, lig_ids, xyz, tors=None):
        """Poses of several ligands in one launch: lig_ids [n], xyz [n][max_atoms][3]
        (each pose padded to max_atoms), tors [n][R]."""
        xyz = _f64(xyz).copy()
        n, max_atoms = xyz.shape[0], xyz.shape[1]
        ids = np.ascontiguousarray(np.asarray(lig_ids, np.int32).reshape(n))
        R = self.n_rotors
        tors = _f64(np.zeros((n, R)) if tors is None else tors).reshape(n, R).copy()
        e = np.zeros(n)
        nev = np.zeros(n, np.int32)
        st = np.zeros(n, np.int32)
        dummy = np.zeros(1)
        self._check(self.lib.pxd_lbfgs_multi(self.h, C.byref(params), n, max_atoms, _p(ids, C.c_int32), _p(xyz),
                                             _p(tors if tors.size else dummy), _p(e), _p(nev, C.c_int32),
                                             _p(st, C.c_int32)))
        return dict(xyz=xyz, torsions=tors, energy=e, nevals=nev, status=st)

    def mc_search_multi(self, params, lig_ids, starts, walker_ids, first_pose, global_min=None):
        """Walkers of several ligands in one launch; starts [n][max_atoms][3]."""
        starts = _f64(starts)
        n, max_atoms = starts.shape[0], starts.shape[1]
        i32 = lambda a: np.ascontiguousarray(np.asarray(a, np.int32).reshape(n))
        ids, wid, fp = i32(lig_ids), i32(walker_ids), i32(first_pose)
        out = np.zeros_like(starts)
        tors = np.zeros((n, max(self.n_rotors, 1)))
        e, ps = np.zeros(n), np.zeros(n)
        nev, st = np.zeros(n, np.int32), np.zeros(n, np.int32)
        gm = None if global_min is None else np.ascontiguousarray(global_min, np.float64)
        self._check(self.lib.pxd_mc_search_multi(self.h, C.byref(params), n, max_atoms, _p(ids, C.c_int32),
                                                 _p(wid, C.c_int32), _p(fp, C.c_int32), _p(starts), _p(out),
                                                 _p(tors), _p(e), _p(ps), _p(nev, C.c_int32), _p(st, C.c_int32),
                                                 None if gm is None else _p(gm)))
        return dict(xyz=out, torsions=tors[:, : self.n_rotors], energy=e, pscore=ps, nevals=nev,
                    status=st, global_min=gm)

    def mc_search_dev(self, params, n_walkers, max_atoms, ids_ptr, walker_ptr, first_ptr, start_ptr,
                      out_xyz_ptr, out_tors_ptr, energy_ptr, pscore_ptr, nevals_ptr, status_ptr,
                      global_min_ptr=None, stream=None):
        self._check(self.lib.pxd_mc_search_dev(self.h, C.byref(params), n_walkers, max_atoms, ids_ptr,
                                               walker_ptr, first_ptr, start_ptr, out_xyz_ptr,
                                               out_tors_ptr, energy_ptr, pscore_ptr, nevals_ptr,
                                               status_ptr, global_min_ptr, stream))

    def rng_draws(self, seed, kinds, ints):
        """Values of the device walker generator (see pxd_rng_draws)."""
        kinds = np.ascontiguousarray(np.asarray(kinds, np.int32))
        ints = np.ascontiguousarray(np.asarray(ints, np.int32))
        width = {3: 3, 4: 4}
        out = np.zeros(sum(width.get(int(k), 1) for k in kinds) or 1)
        self._check(self.lib.pxd_rng_draws(self.h, seed, len(kinds), _p(kinds, C.c_int32),
                                           _p(ints, C.c_int32), _p(out)))
        return out[: sum(width.get(int(k), 1) for k in kinds)]

    def receptor_kinematics(self, torsions):
        t = _f64(torsions).reshape(-1, self.n_rotors)
        n = t.shape[0]
        out = np.zeros((n, self.receptor.n_atoms, 3))
        self._check(self.lib.pxd_receptor_kinematics(self.h, n, _p(t if t.size else np.zeros(1)),
                                                     _p(out)))
        return out


def lbfgs_params(**kw):
    """pxd_lbfgs_params with the reference defaults (pxd_lbfgs_defaults) overridden by kw."""
    p = abi.LbfgsParams()
    load().pxd_lbfgs_defaults(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def mc_params(box_lo, box_hi, **kw):
    """pxd_mc_params with the reference defaults (pxd_mc_defaults) and the search box;
    keyword arguments override fields, lbfgs=dict(...) the optimiser constants."""
    p = abi.McParams()
    load().pxd_mc_defaults(C.byref(p))
    for d in range(3):
        p.box_lo[d] = float(box_lo[d])
        p.box_hi[d] = float(box_hi[d])
    for k, v in kw.items():
        if k == "lbfgs":
            for kk, vv in v.items():
                setattr(p.lbfgs, kk, vv)
        else:
            setattr(p, k, v)
    return p


def gather_bandwidth(device=0, working_set_bytes=64 << 20, reps=10):
    """pxd_gather_bandwidth: GB/s of random 16-byte gathers over a working set on `device`
    (below the L2 size: the L2 gather roofline of the batched kernels)."""
    lib = load()
    out = np.zeros(1)
    rc = lib.pxd_gather_bandwidth(device, working_set_bytes, reps, _p(out))
    if rc != 0:
        raise NativeError(rc, "gather bandwidth probe failed")
    return float(out[0])
