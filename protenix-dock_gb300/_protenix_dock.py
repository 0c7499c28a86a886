"""GB300 drop-in for the reference's Python module `_protenix_dock`.

Same module functions, class, method names, keyword names and defaults as the
reference binding (engine/src/pyb/api.cpp:34-63) over bytedock::ReusableEngine
(engine/src/core/entrance.cpp:69-438): files in, files out, with the reference's
output schema (engine/src/core/writer.cpp:40-230). Errors surface as RuntimeError,
as the reference's C++ exceptions do through its binding.

Behind the class is the GB300 C ABI (include/pxdock_gb300.h): maps built on the
device, and each call runs ONE batched launch over every pose (optimize) or every
walker (search) of every ligand in the index, instead of one CPU task per pose.
Differences from the reference that a caller can see:
  - dump_maps / load_maps use this library's own cache format (a JSON header and one
    FP32 {E, dE/dx, dE/dy, dE/dz} file per map); the reference's Boost archives are
    not readable here;
  - output files are written in index-file order (the reference's writer threads
    finish in any order);
  - the extra keyword `device` (default 0) picks the CUDA device.
"""
import json
import logging
import os

import numpy as np

from pxdock_gb300 import model, native

_log = logging.getLogger("protenix_dock")
_DEFAULT_SF = os.path.join(os.path.dirname(os.path.abspath(__file__)), "pxdock_gb300", "data",
                           "scoring_function.json")
_MAP_FORMAT = "pxdock-gb300 maps 1"
_COULOMB = 99


def version():
    """Library version string (api.cpp:24-27)."""
    return native.load().pxd_version().decode()


def log2file(log_file="-", verbosity=1):
    """Routes the engine log to a file ("-": standard error), as setup_global_logging
    (entrance.cpp:51-54) does; verbosity 0 warnings, 1 info, 2 debug."""
    for h in list(_log.handlers):
        _log.removeHandler(h)
    h = logging.StreamHandler() if log_file == "-" else logging.FileHandler(log_file)
    h.setFormatter(logging.Formatter("[%(asctime)s] %(levelname)s %(message)s"))
    _log.addHandler(h)
    _log.setLevel({0: logging.WARNING, 1: logging.INFO}.get(verbosity, logging.DEBUG))


# --------------------------------------------------------------------------- output
def _g(v):
    """A double as std::ostream prints it by default (precision 6, %g)."""
    return "%g" % v


def _format_rows(values, prefix, ncols):
    """printer.h format<T, NCOLS>: rows of NCOLS values, the last row without the
    trailing comma; nothing for an empty list."""
    indent = prefix + "  "
    n = len(values)
    nrows, remained = divmod(n, ncols)
    if remained == 0 and nrows > 0:
        nrows -= 1
        remained = ncols
    out = []
    for i in range(nrows):
        out.append(indent + "".join(_g(values[i * ncols + j]) + ", " for j in range(ncols)) + "\n")
    if remained > 0:
        off = nrows * ncols
        out.append(indent + ", ".join(_g(v) for v in values[off:off + remained]) + "\n")
    return "".join(out)


def _pose_string(xyz, prefix):
    """to_string(molecule_pose, prefix) (system.cpp:319-336)."""
    if len(xyz) == 0:
        return "[]"
    rows = [prefix + "  [" + ", ".join(_g(c) for c in a) + "]" for a in xyz]
    return "[\n" + ",\n".join(rows) + "\n" + prefix + "]"


def _write_poses(path, smiles, best_id, bscore, poses, receptor):
    """pose_writer::consume (writer.cpp:40-81)."""
    out = ["{\n"]
    if smiles:
        out.append('  "mapped_smiles": "' + smiles.replace("\\", "\\\\") + '",\n')
    out.append('  "best_pose": {\n')
    out.append('    "index": %d,\n' % best_id)
    out.append('    "bscore": ' + _g(bscore) + "\n")
    out.append("  },\n")
    out.append('  "poses": [\n')
    for i, p in enumerate(poses):
        aligned = [0.0] * receptor.num_rotatable_bonds
        for k, t in enumerate(p["torsions"]):
            aligned[receptor.bond_mappings[k]] = float(t)
        out.append("    {\n")
        out.append('      "offset": %d,\n' % p["offset"])
        out.append('      "energy": ' + _g(p["energy"]) + ",\n")
        out.append('      "pscore": ' + _g(p["pscore"]) + ",\n")
        out.append('      "nevals": %d,\n' % p["nevals"])
        out.append('      "receptor": {\n')
        out.append('        "torsions": [\n' + _format_rows(aligned, "          ", 10) + "        ]\n")
        out.append("      },\n")
        out.append('      "ligand": {\n')
        out.append('        "xyz": ' + _pose_string(p["xyz"], "        ") + "\n")
        out.append("      }\n")
        out.append("    }" + ("," if i < len(poses) - 1 else "") + "\n")
    out.append("  ]\n")
    out.append("}\n")
    with open(path, "w") as f:
        f.write("".join(out))
    return path


def _rmsd(a, b):
    """calculate_rmsd_upper_bound (writer.cpp:86-93): plain RMSD in atom order."""
    return float(np.sqrt(np.sum((a - b) ** 2) / len(a)))


def _cluster(candidates, num_modes, min_rmsd):
    """pose_cluster::preprocess (writer.cpp:115-160): greedy RMSD clustering of the
    walkers' best poses, kept sorted by pose score; failed walkers (nevals == 0) skipped."""
    kept = []
    for c in candidates:
        if c["nevals"] == 0:
            continue
        if not kept:
            kept.append(c)
            continue
        d = [_rmsd(k["xyz"], c["xyz"]) for k in kept]
        off = int(np.argmin(d))
        updated = False
        if d[off] < min_rmsd:
            if c["pscore"] < kept[off]["pscore"]:
                kept[off] = c
                updated = True
        elif len(kept) < num_modes:
            kept.append(c)
            updated = True
        elif c["pscore"] < kept[-1]["pscore"]:
            kept[-1] = c
            updated = True
        if updated:
            kept.sort(key=lambda k: k["pscore"])
    return kept


def _read_index(path):
    """index_file_source::fill (source.cpp:26-44): one ligand file per line; empty
    lines and missing files are skipped with a warning."""
    files = []
    with open(path) as f:
        for no, line in enumerate(f, 1):
            line = line.rstrip("\n")
            if not line:
                _log.warning("Skip illegal line#%d with empty text.", no)
            elif not os.path.isfile(line):
                _log.warning("Skip illegal line#%d with ghost file: %s", no, line)
            else:
                files.append(line)
    return files


def _stem(path):
    return os.path.splitext(os.path.basename(path))[0]


class ReusableEngine:
    """bytedock::ReusableEngine (entrance.h:30-74) on one GB300."""

    def __init__(self, receptor_file, sf_file="", cpu_nthreads=0, device=0):
        try:
            self._receptor = model.Receptor.from_file(receptor_file)
        except (OSError, ValueError, KeyError) as e:
            raise RuntimeError("Failed to parse receptor file %s: %s" % (receptor_file, e)) from None
        if not sf_file:
            if not os.path.exists(_DEFAULT_SF):
                raise RuntimeError("Failed to find the default parameter file of scoring function. "
                                   "Please explicitly provide its location!.")
            _log.info("Since no scoring function parameter file provided, the default one is "
                      "enabled at: %s", _DEFAULT_SF)
            sf_file = _DEFAULT_SF
        try:
            self._pose_sf, self._affinity_sf = model.load_scoring_function(sf_file)
        except (OSError, ValueError, KeyError) as e:
            raise RuntimeError("Failed to parse scoring function file %s: %s" % (sf_file, e)) from None
        self._nthreads = cpu_nthreads if cpu_nthreads >= 1 else (os.cpu_count() or 1)
        native.load()
        self._ctx = native.Context(device)
        self._ctx.set_receptor(self._receptor)
        self._ctx.set_scoring_function(0, self._pose_sf)
        self._ctx.set_scoring_function(1, self._affinity_sf)
        self._box = []      # set_box appends, as the reference's box_ vector does
        self._grid = None   # pxd_box of the maps on the device

    # ----------------------------------------------------------------- box and maps
    def _require_box(self):
        if len(self._box) == 0:
            raise RuntimeError("Please call `set_box(...)` first!")

    def _require_maps(self):
        if self._grid is None:
            raise RuntimeError("Please call either `generate_cache_maps(...)` or `load_maps(...)` first!")

    def set_box(self, center_x, center_y, center_z, size_x, size_y, size_z):
        # the reference pushes the six values onto its box vector and reads the first
        # six afterwards, so the first call's box stays in force
        self._box.extend(float(v) for v in (center_x, center_y, center_z, size_x, size_y, size_z))

    def generate_maps(self, grid_spacing, max_size=0.):
        self._require_box()
        b = self._box
        size = [max(b[3 + d], max_size) for d in range(3)]
        box = model.make_box(b[:3], size, grid_spacing)
        _log.info("Generating receptor cache with grid settings: init [%.3f, %.3f, %.3f], points "
                  "[%d, %d, %d]", *box.init_xyz, *box.npoints)
        self._ctx.build_grid(box)  # every ligand vdW type, as receptor_cache::populate
        self._grid = box

    def drop_maps(self):
        if self._grid is not None:
            self._ctx.drop_grid()
        self._grid = None

    def dump_maps(self, cache_dir):
        self._require_maps()
        os.makedirs(cache_dir, exist_ok=True)
        g = self._grid
        head = {"format": _MAP_FORMAT, "init_xyz": list(g.init_xyz), "npoints": list(g.npoints),
                "spacing": g.spacing, "maps": list(range(100))}
        for m in range(100):
            self._ctx.read_map(m).tofile(os.path.join(cache_dir, "map_%03d.f32" % m))
        with open(os.path.join(cache_dir, "grid.json"), "w") as f:
            json.dump(head, f)

    def load_maps(self, cache_dir):
        try:
            with open(os.path.join(cache_dir, "grid.json")) as f:
                head = json.load(f)
        except (OSError, ValueError) as e:
            raise RuntimeError("Failed to read maps from %s: %s" % (cache_dir, e)) from None
        if head.get("format") != _MAP_FORMAT:
            raise RuntimeError("Unknown map cache format in %s" % cache_dir)
        box = model.make_box((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), 1.0)
        for d in range(3):
            box.init_xyz[d] = head["init_xyz"][d]
            box.npoints[d] = head["npoints"][d]
        box.spacing = head["spacing"]
        P = box.npoints[0] * box.npoints[1] * box.npoints[2]
        for m in head["maps"]:
            rec = np.fromfile(os.path.join(cache_dir, "map_%03d.f32" % m), np.float32).reshape(P, 4)
            self._ctx.write_map(box, m, rec)
        self._grid = box
        _log.info("Previous grid settings: init [%.3f, %.3f, %.3f], spacing %g, points [%d, %d, %d]",
                  box.init_xyz[0], box.init_xyz[1], box.init_xyz[2], box.spacing, *box.npoints)

    # ------------------------------------------------------------------- ligands
    def _load(self, files, geometry):
        """Parses the ligand files; a file that fails is skipped with a warning
        (reader.cpp:27-35)."""
        out = []
        for path in files:
            try:
                lig = model.Ligand.from_file(path, geometry=geometry)
            except (OSError, ValueError, KeyError, IndexError) as e:
                _log.warning("Due to invalid format or content, skip ligand: %s with reason: %s", path, e)
                continue
            out.append((path, lig))
        return out

    def _register(self, ligands):
        self._ctx.clear_ligands()
        return [self._ctx.add_ligand(lig) for _, lig in ligands]

    # ------------------------------------------------------------------ workflows
    def evaluate(self, ligand_index_file, output_dir):
        """scoring_evaluator over every pose of every ligand (evaluator.cpp:22-46); the
        CSV goes to `output_dir`, which is a file path, as in the reference."""
        ligands = self._load(_read_index(ligand_index_file), geometry=False)
        ids = self._register(ligands)
        lines = ["ligand_file,pose_id,pscore,bscore\n"]
        for (path, lig), lid in zip(ligands, ids):
            ps, _ = self._ctx.score(0, lid, lig.poses)
            bs, _ = self._ctx.score(1, lid, lig.poses)
            for k in range(len(lig.poses)):
                lines.append("%s,%d,%.16g,%.16g\n" % (_stem(path), k, ps[k], bs[k]))
        with open(output_dir, "w") as f:
            f.write("".join(lines))
        _log.info("Number of successful evaluations is: %d", len(lines) - 1)

    def optimize(self, ligand_index_file, output_dir, max_niters=240, slope=1e6):
        """serial_optimizer over every pose (optimizer.cpp:28-36), then pose_ranker
        (writer.cpp:162-189): one batched L-BFGS launch over all poses."""
        if self._grid is None:
            _log.info("Receptor cache is disabled in this run.")
        else:
            self._ctx.set_slope(slope)
        ligands = self._load(_read_index(ligand_index_file), geometry=False)  # multi_pose_reader
        ids = self._register(ligands)
        os.makedirs(output_dir, exist_ok=True)
        if not ligands:
            return
        max_atoms = max(lig.n_atoms for _, lig in ligands)
        rows, owner = [], []
        for k, ((path, lig), lid) in enumerate(zip(ligands, ids)):
            for p in range(len(lig.poses)):
                x = np.zeros((max_atoms, 3))
                x[: lig.n_atoms] = lig.poses[p]
                rows.append(x)
                owner.append((k, p, lid))
        params = native.lbfgs_params(max_iter=max_niters)
        res = self._ctx.lbfgs_multi(params, [o[2] for o in owner], np.stack(rows))
        written = 0
        for k, ((path, lig), lid) in enumerate(zip(ligands, ids)):
            sel = [i for i, o in enumerate(owner) if o[0] == k]
            xyz = res["xyz"][sel, : lig.n_atoms]
            tors = res["torsions"][sel]
            ps, _ = self._ctx.score(0, lid, xyz, tors)
            best = int(np.argmin(ps))  # first minimum, as `cdd.pscore < best` keeps it
            bs, _ = self._ctx.score(1, lid, xyz[best][None], tors[best][None])
            poses = [dict(offset=owner[i][1], energy=res["energy"][i], pscore=ps[j],
                          nevals=int(res["nevals"][i]), torsions=tors[j], xyz=xyz[j])
                     for j, i in enumerate(sel)]
            _write_poses(os.path.join(output_dir, _stem(path) + "_out.json"), lig.smiles, best,
                         bs[0], poses, self._receptor)
            written += 1
        _log.info("Number of successful optimizations is: %d", written)

    def search(self, ligand_index_file, output_dir, seed=0, exhaustiveness=256, max_nsteps=200,
               relax_nsteps=40, num_modes=8, min_rmsd=0.5, mc_mmenergy_threshold=-1., slope=1e6):
        """monte_carlo_searcher over `exhaustiveness` walkers per ligand
        (searcher.cpp:98-187, reader.cpp:27-52), then pose_cluster (writer.cpp:115-160):
        one persistent launch over every walker of every ligand."""
        if self._grid is None:
            self._require_box()
            b = self._box
            lo = [b[d] - b[3 + d] * 0.5 for d in range(3)]  # describe_boundary, grid.cpp:42-55
            hi = [b[d] + b[3 + d] * 0.5 for d in range(3)]
            _log.info("Receptor cache is disabled in this run.")
        else:
            self._ctx.set_slope(slope)
            g = self._grid
            lo = [g.init_xyz[d] for d in range(3)]
            hi = [g.init_xyz[d] + (g.npoints[d] - 1) * g.spacing for d in range(3)]
        ligands = self._load(_read_index(ligand_index_file), geometry=True)
        ids = self._register(ligands)
        os.makedirs(output_dir, exist_ok=True)
        if not ligands:
            return
        max_atoms = max(lig.n_atoms for _, lig in ligands)
        starts, lig_ids, walkers, first, owner = [], [], [], [], []
        for k, ((path, lig), lid) in enumerate(zip(ligands, ids)):
            for w in range(exhaustiveness):
                src = w if len(lig.poses) > w else 0
                x = np.zeros((max_atoms, 3))
                x[: lig.n_atoms] = lig.poses[src if w else 0]
                starts.append(x)
                lig_ids.append(lid)
                walkers.append(w)
                first.append(1 if src == 0 else 0)
                owner.append(k)
        params = native.mc_params(lo, hi, seed=seed, max_nsteps=max_nsteps, relax_nsteps=relax_nsteps,
                                  mc_mmenergy_threshold=mc_mmenergy_threshold)
        gmin = np.full(len(ligands), 1e8)
        res = self._ctx.mc_search_multi(params, lig_ids, np.stack(starts), walkers, first, gmin)
        written = 0
        owner = np.array(owner)
        for k, ((path, lig), lid) in enumerate(zip(ligands, ids)):
            sel = np.nonzero(owner == k)[0]
            cands = [dict(offset=walkers[i], energy=res["energy"][i], pscore=res["pscore"][i],
                          nevals=int(res["nevals"][i]), torsions=res["torsions"][i],
                          xyz=res["xyz"][i, : lig.n_atoms]) for i in sel]
            kept = _cluster(cands, num_modes, min_rmsd)
            if not kept:
                _log.debug("Tasks with prefix [%s] has failed.", _stem(path))
                continue
            bs, _ = self._ctx.score(1, lid, kept[0]["xyz"][None], np.asarray(kept[0]["torsions"])[None])
            _write_poses(os.path.join(output_dir, _stem(path) + "_out.json"), lig.smiles, 0, bs[0], kept,
                         self._receptor)
            written += 1
        _log.info("Number of successful dockings is: %d", written)
