"""GB300 drop-in for the reference's Python module `_protenix_dock`.

Same module functions, class, method names, keyword names and defaults as the
reference binding (engine/src/pyb/api.cpp:34-63) over bytedock::ReusableEngine
(engine/src/core/entrance.cpp:69-438). This module is a thin ctypes binding of the
library's C++ engine (csrc/engine.cpp, the pxd_engine_* C ABI): files in, files out,
in the reference's output formats (engine/src/core/writer.cpp:40-230). Errors surface as
RuntimeError with the reference's messages, as its C++ exceptions do through its binding.

Each workflow call runs one batched device launch over every pose (optimize) or every
walker (search) of every ligand in the index. Differences a caller can see:
  - dump_maps / load_maps write and read the reference's cache files (<tag>.bdg Boost
    binary archives of FP64 records and the meta.dat text archive, grid.cpp:305-431);
    load_maps also reads this library's earlier layout (grid.json + map_NNN.f32), and
    refuses a cache whose excluded receptor atoms are not this receptor's movable ones;
  - output files are written in index-file order;
  - the extra keyword `device` (default 0) picks the CUDA device;
  - optimize and search take the extra keywords `rank` and `world` (default 0 and 1, the
    reference's single process): with world > 1, the call processes only this rank's
    cost-balanced share of the index (pxdock_gb300.shard), so that one process per GPU
    covers the index with every output file written once.
"""
import os
import tempfile

import ctypes as C

import numpy as np

from pxdock_gb300 import native

_bound = None


def _lib():
    global _bound
    if _bound is None:
        lib = native.load()
        vp, cp, d, i32 = C.c_void_p, C.c_char_p, C.c_double, C.c_int32
        lib.pxd_engine_create.argtypes = [cp, cp, i32, i32, C.POINTER(vp)]
        lib.pxd_engine_destroy.argtypes = [vp]
        lib.pxd_engine_last_error.argtypes = [vp]
        lib.pxd_engine_last_error.restype = cp
        lib.pxd_engine_set_box.argtypes = [vp] + [d] * 6
        lib.pxd_engine_generate_maps.argtypes = [vp, d, d]
        lib.pxd_engine_dump_maps.argtypes = [vp, cp]
        lib.pxd_engine_load_maps.argtypes = [vp, cp]
        lib.pxd_engine_drop_maps.argtypes = [vp]
        lib.pxd_engine_evaluate.argtypes = [vp, cp, cp]
        lib.pxd_engine_optimize.argtypes = [vp, cp, cp, i32, d]
        lib.pxd_engine_set_dof_mode.argtypes = [vp, i32]
        lib.pxd_engine_search.argtypes = [vp, cp, cp, i32, i32, i32, i32, i32, d, d, d]
        lib.pxd_engine_log2file.argtypes = [cp, i32]
        f64p, i32p, i64p = C.POINTER(d), C.POINTER(i32), C.POINTER(C.c_int64)
        lib.pxd_write_poses.argtypes = [cp, cp, i32, d, i32, i32, i32p, f64p, f64p, i64p, i32, f64p, f64p, i32p,
                                        i32]
        lib.pxd_cluster_poses.argtypes = [i32, i32, f64p, f64p, i64p, i32, d, i32p, i32p]
        _bound = lib
    return _bound


def _b(s):
    return s.encode() if isinstance(s, str) else s


def version():
    """Library version string (api.cpp:24-27)."""
    return _lib().pxd_version().decode()


def log2file(log_file="-", verbosity=1):
    """Routes the engine log to a file ("-": standard error), as setup_global_logging
    (entrance.cpp:51-54) does; verbosity 0 warnings, 1 info, 2 debug."""
    lib = _lib()
    if lib.pxd_engine_log2file(_b(log_file), verbosity):
        raise RuntimeError(lib.pxd_engine_last_error(None).decode())


class ReusableEngine:
    """bytedock::ReusableEngine (entrance.h:30-74) on one GB300."""

    def __init__(self, receptor_file, sf_file="", cpu_nthreads=0, device=0):
        lib = _lib()
        h = C.c_void_p()
        if lib.pxd_engine_create(_b(receptor_file), _b(sf_file or ""), cpu_nthreads, device, C.byref(h)):
            raise RuntimeError(lib.pxd_engine_last_error(None).decode())
        self._h = h
        self._lib = lib

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pxd_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def _call(self, fn, *args):
        if fn(self._h, *args):
            raise RuntimeError(self._lib.pxd_engine_last_error(self._h).decode())

    def set_box(self, center_x, center_y, center_z, size_x, size_y, size_z):
        self._call(self._lib.pxd_engine_set_box, center_x, center_y, center_z, size_x, size_y, size_z)

    def generate_maps(self, grid_spacing, max_size=0.):
        self._call(self._lib.pxd_engine_generate_maps, grid_spacing, max_size)

    def dump_maps(self, cache_dir):
        self._call(self._lib.pxd_engine_dump_maps, _b(cache_dir))

    def load_maps(self, cache_dir):
        self._call(self._lib.pxd_engine_load_maps, _b(cache_dir))

    def drop_maps(self):
        self._call(self._lib.pxd_engine_drop_maps)

    def evaluate(self, ligand_index_file, output_dir):
        """The reference names this argument output_dir; it is the CSV file written."""
        self._call(self._lib.pxd_engine_evaluate, _b(ligand_index_file), _b(output_dir))

    def _sharded(self, ligand_index_file, rank, world, walkers, run):
        """Runs run(index_file) on this rank's share of the index (world > 1) or on the
        whole index (world == 1, the reference's behaviour)."""
        if world == 1 and rank == 0:
            return run(ligand_index_file)
        if world < 1 or not 0 <= rank < world:
            raise RuntimeError("rank %d outside a world of %d" % (rank, world))
        from pxdock_gb300 import shard

        fd, path = tempfile.mkstemp(prefix="pxd_rank%d_" % rank, suffix=".txt")
        os.close(fd)
        try:
            if shard.rank_index(ligand_index_file, rank, world, path, walkers) > 0:
                run(path)
        finally:
            os.unlink(path)

    def optimize(self, ligand_index_file, output_dir, max_niters=240, slope=1e6, rank=0, world=1, dof_mode=0):
        """dof_mode 0: L-BFGS over ligand coordinates and receptor torsions (the reference);
        1: over rigid body + ligand torsions + receptor torsions (bond lengths and angles
        keep their input values)."""
        self._call(self._lib.pxd_engine_set_dof_mode, dof_mode)
        self._sharded(ligand_index_file, rank, world, None,
                      lambda idx: self._call(self._lib.pxd_engine_optimize, _b(idx), _b(output_dir),
                                             max_niters, slope))

    def search(self, ligand_index_file, output_dir, seed=0, exhaustiveness=256, max_nsteps=200,
               relax_nsteps=40, num_modes=8, min_rmsd=0.5, mc_mmenergy_threshold=-1., slope=1e6, rank=0,
               world=1):
        self._sharded(ligand_index_file, rank, world, exhaustiveness,
                      lambda idx: self._call(self._lib.pxd_engine_search, _b(idx), _b(output_dir), seed,
                                             exhaustiveness, max_nsteps, relax_nsteps, num_modes, min_rmsd,
                                             mc_mmenergy_threshold, slope))


# ----------------------------------------------------- the engine's host-only parts
def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def _write_poses(path, smiles, best_id, bscore, poses, bond_mappings, num_rotatable_bonds):
    """The engine's writer (pxd_write_poses) on a list of dicts with offset, energy,
    pscore, nevals, torsions (leaf order) and xyz."""
    n = len(poses)
    N = len(poses[0]["xyz"]) if n else 0
    R = len(bond_mappings)
    off = np.array([p["offset"] for p in poses], np.int32)
    e = np.array([p["energy"] for p in poses], np.float64)
    ps = np.array([p["pscore"] for p in poses], np.float64)
    nev = np.array([p["nevals"] for p in poses], np.int64)
    tors = np.ascontiguousarray(np.array([p["torsions"] for p in poses], np.float64).reshape(n, R)) if R else \
        np.zeros(1)
    xyz = np.ascontiguousarray(np.array([p["xyz"] for p in poses], np.float64).reshape(n, N, 3))
    maps = np.array(bond_mappings if R else [0], np.int32)
    lib = _lib()
    if lib.pxd_write_poses(_b(path), _b(smiles or ""), best_id, bscore, n, N, _p(off, C.c_int32), _p(e, C.c_double),
                           _p(ps, C.c_double), _p(nev, C.c_int64), R, _p(tors, C.c_double), _p(xyz, C.c_double),
                           _p(maps, C.c_int32), num_rotatable_bonds):
        raise RuntimeError(lib.pxd_engine_last_error(None).decode())
    return path


def _cluster(candidates, num_modes, min_rmsd):
    """The engine's pose clustering (pxd_cluster_poses): the kept candidates, best first."""
    n = len(candidates)
    if n == 0:
        return []
    xyz = np.ascontiguousarray(np.array([c["xyz"] for c in candidates], np.float64))
    N = xyz.shape[1]
    ps = np.array([c["pscore"] for c in candidates], np.float64)
    nev = np.array([c["nevals"] for c in candidates], np.int64)
    kept = np.zeros(n, np.int32)
    nk = C.c_int32()
    _lib().pxd_cluster_poses(n, N, _p(xyz, C.c_double), _p(ps, C.c_double), _p(nev, C.c_int64), num_modes, min_rmsd,
                             _p(kept, C.c_int32), C.byref(nk))
    return [candidates[k] for k in kept[: nk.value]]
