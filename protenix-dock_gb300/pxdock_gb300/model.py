"""Receptor / ligand data model: engine JSON -> flat arrays -> C ABI structs.

The parsing rules restate the reference parser (engine/src/core/data.cpp):
  - force-field terms                 data.cpp:31-296  (fill(..., force_field_params))
  - receptor rotor leaves             data.cpp:310-364 (fill(rotable_geometry), parse)
  - ligand fragment tree              data.cpp:410-482 (fill(fragment_tree))
  - ligand vdW type offset 1000       data.cpp:234-244
Degrees are turned into radians as (x / 180) * pi, the reference's MATH_TO_RADIAN
(math.h:228), so that FP64 inputs match the reference bit for bit.
"""
import ctypes as C
import json
import math

import numpy as np

from . import abi

VDW_OFFSET = 1000
COUL14_SCALE = 0.833333333
VDW14_SCALE = 0.5
COULOMB_FACTOR = 332.0637141491396

# Ligand vdW type table (sigma, epsilon); the same numbers as include/pxdock_gb300_vdw.h.
_VDW_TABLE = None


def vdw_table():
    """(sigma[99], epsilon[99]) read from include/pxdock_gb300_vdw.h."""
    global _VDW_TABLE
    if _VDW_TABLE is None:
        import os
        import re

        here = os.path.dirname(os.path.abspath(__file__))
        path = os.path.join(here, "..", "..", "include", "pxdock_gb300_vdw.h")
        text = open(path).read()

        def arr(name):
            body = re.search(name + r"\[99\] = \{(.*?)\};", text, re.S).group(1)
            return np.array([float(v) for v in body.replace("\n", " ").split(",") if v.strip()])

        _VDW_TABLE = (arr("PXD_VDW_SIGMA"), arr("PXD_VDW_EPSILON"))
    return _VDW_TABLE


def _radian(deg):
    return (float(deg) / 180.0) * math.pi


def _i32(a, shape=None):
    out = np.ascontiguousarray(np.asarray(a, dtype=np.int32))
    if shape is not None:
        out = out.reshape(shape)
    return out


def _f64(a, shape=None):
    out = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if shape is not None:
        out = out.reshape(shape)
    return out


def _per_atom(values, n):
    """Per-atom list, zero-filled when a fixture leaves it empty."""
    if len(values) == n:
        return values
    if len(values) == 0:
        return [0.0] * n
    raise ValueError("per-atom list has %d entries for %d atoms" % (len(values), n))


def _dihedrals(ff, prefix):
    atoms = ff.get(prefix + "_atomidx", [])
    n = len(atoms)
    ids = np.zeros((n, 4), np.int32)
    per = np.zeros((n, 6), np.int32)
    phase = np.zeros((n, 6), np.float64)
    k = np.zeros((n, 6), np.float64)
    for d in range(n):
        ids[d] = atoms[d]
        for t, v in enumerate(ff[prefix + "_periodicity"][d]):
            per[d, t] = int(v)
        for t, v in enumerate(ff[prefix + "_k"][d]):
            k[d, t] = float(v)
        for t, v in enumerate(ff[prefix + "_phase"][d]):
            phase[d, t] = _radian(v)
    return ids, per, phase, k


class Topology:
    """Flat force-field arrays of one molecule (force_field_params, system.h:85-109)."""

    def __init__(self, n_atoms, charge, sigma, epsilon, bonds=(), bond_k=(), bond_length=(),
                 angles=(), angle_k=(), angle_radian=(), impropers=None, propers=None,
                 pairs14=(), pairs=()):
        self.n_atoms = int(n_atoms)
        self.charge = _f64(charge)
        self.sigma = _f64(sigma)
        self.epsilon = _f64(epsilon)
        self.bonds = _i32(bonds).reshape(-1, 2)
        self.bond_k = _f64(bond_k).reshape(-1)
        self.bond_length = _f64(bond_length).reshape(-1)
        self.angles = _i32(angles).reshape(-1, 3)
        self.angle_k = _f64(angle_k).reshape(-1)
        self.angle_radian = _f64(angle_radian).reshape(-1)
        empty = (np.zeros((0, 4), np.int32), np.zeros((0, 6), np.int32),
                 np.zeros((0, 6)), np.zeros((0, 6)))
        self.impropers = tuple(np.ascontiguousarray(a) for a in (impropers or empty))
        self.propers = tuple(np.ascontiguousarray(a) for a in (propers or empty))
        self.pairs14 = _i32(pairs14).reshape(-1, 2)
        self.pairs = _i32(pairs).reshape(-1, 2)

    @classmethod
    def from_ffdata(cls, ff, n_atoms, sigma, epsilon):
        bonds = ff.get("FF_Bonds_atomidx", [])
        angles = ff.get("FF_Angles_atomidx", [])
        return cls(
            n_atoms,
            _per_atom([float(q) for q in ff["partial_charges"]], n_atoms),
            sigma,
            epsilon,
            bonds=bonds,
            bond_k=[float(v) for v in ff.get("FF_Bonds_k", [])],
            bond_length=[float(v) for v in ff.get("FF_Bonds_length", [])],
            angles=angles,
            angle_k=[float(v) for v in ff.get("FF_Angles_k", [])],
            angle_radian=[_radian(v) for v in ff.get("FF_Angles_angle", [])],
            impropers=_dihedrals(ff, "FF_ImproperTorsions"),
            propers=_dihedrals(ff, "FF_ProperTorsions"),
            pairs14=ff.get("FF_Nonbonded14_atomidx", []),
            pairs=ff.get("FF_NonbondedAll_atomidx", []),
        )

    def to_c(self, keep):
        """pxd_topology pointing into these arrays; `keep` collects the arrays."""
        t = abi.Topology()
        t.n_atoms = self.n_atoms

        def p(arr, ctype):
            keep.append(arr)
            if arr.size == 0:
                return C.cast(None, C.POINTER(ctype))
            return arr.ctypes.data_as(C.POINTER(ctype))

        t.charge = p(self.charge, C.c_double)
        t.sigma = p(self.sigma, C.c_double)
        t.epsilon = p(self.epsilon, C.c_double)
        t.n_bonds = len(self.bonds)
        t.bond_atoms = p(self.bonds, C.c_int32)
        t.bond_k = p(self.bond_k, C.c_double)
        t.bond_length = p(self.bond_length, C.c_double)
        t.n_angles = len(self.angles)
        t.angle_atoms = p(self.angles, C.c_int32)
        t.angle_k = p(self.angle_k, C.c_double)
        t.angle_radian = p(self.angle_radian, C.c_double)
        t.n_impropers = len(self.impropers[0])
        t.improper_atoms = p(self.impropers[0], C.c_int32)
        t.improper_periodicity = p(self.impropers[1], C.c_int32)
        t.improper_phase = p(self.impropers[2], C.c_double)
        t.improper_k = p(self.impropers[3], C.c_double)
        t.n_propers = len(self.propers[0])
        t.proper_atoms = p(self.propers[0], C.c_int32)
        t.proper_periodicity = p(self.propers[1], C.c_int32)
        t.proper_phase = p(self.propers[2], C.c_double)
        t.proper_k = p(self.propers[3], C.c_double)
        t.n_pairs14 = len(self.pairs14)
        t.pairs14 = p(self.pairs14, C.c_int32)
        t.n_pairs = len(self.pairs)
        t.pairs = p(self.pairs, C.c_int32)
        return t


class Receptor:
    """torsional_receptor (data.h:34-67) as flat arrays."""

    def __init__(self, xyz, topology, rotor_axis=(), rotor_atoms=(), raw=None):
        self.xyz = _f64(xyz).reshape(-1, 3)
        self.n_atoms = len(self.xyz)
        self.ff = topology
        self.rotor_axis = _i32(rotor_axis).reshape(-1, 2)
        self.rotor_groups = [list(map(int, g)) for g in rotor_atoms]
        offs = [0]
        for g in self.rotor_groups:
            offs.append(offs[-1] + len(g))
        self.rotor_offsets = _i32(offs)
        flat = [a for g in self.rotor_groups for a in g]
        self.rotor_atoms = _i32(flat if flat else np.zeros(0))
        self.n_rotors = len(self.rotor_axis)
        self.raw = raw  # the parsed JSON dict (scoring terms read it)

    @classmethod
    def from_json(cls, d):
        geo = d["geometry"]
        ff = d["ffdata"]
        xyz = d["xyz"]
        n = len(xyz)
        if int(geo["num_atoms"]) != n:
            raise ValueError("Atom count mismatches! Wanted [%s] vs. Parsed [%d]"
                             % (geo["num_atoms"], n))
        axes, groups, order = [], [], []
        for batch in geo.get("data", {}).values():  # data.cpp:314-336, JSON key order
            a0 = batch["rot_bond_1"]
            a1 = batch["rot_bond_2"]
            for i in range(len(a0)):
                axes.append((int(a0[i]), int(a1[i])))
            for frag in batch["fragments"]:
                groups.append([int(a) for a in frag])
            order.extend(int(v) for v in batch.get("rot_bond_order", []))
        sigma = _per_atom([float(v) for v in ff["FF_vdW_sigma"]], n)
        eps = _per_atom([float(v) for v in ff["FF_vdW_epsilon"]], n)
        top = Topology.from_ffdata(ff, n, sigma, eps)
        r = cls(xyz, top, axes, groups, raw=d)
        r.lists = ScoreLists(ff, n, ligand=False)
        # leaf -> position among the rotatable bonds (data.cpp:337-348), used to write
        # receptor torsions in bond order (restore_bond_orders, data.h:53-61)
        r.bond_mappings = order if len(order) == len(axes) else list(range(len(axes)))
        r.num_rotatable_bonds = max([int(geo.get("num_rotatable_bonds", 0))] +
                                    [m + 1 for m in r.bond_mappings])
        return r

    @classmethod
    def from_file(cls, path):
        with open(path) as f:
            return cls.from_json(json.load(f))

    def to_c(self, keep):
        r = abi.ReceptorDesc()
        r.n_atoms = self.n_atoms
        keep.append(self.xyz)
        r.xyz = self.xyz.ctypes.data_as(abi.f64p)
        r.ff = self.ff.to_c(keep)
        r.n_rotors = self.n_rotors
        for name in ("rotor_axis", "rotor_offsets", "rotor_atoms"):
            arr = getattr(self, name)
            keep.append(arr)
            setattr(r, name, arr.ctypes.data_as(abi.i32p) if arr.size else C.cast(None, abi.i32p))
        lists = getattr(self, "lists", None)
        if lists is not None:
            lc = lists.to_c(keep)
            keep.append(lc)
            r.lists = C.pointer(lc)
        return r

    def movable_atoms(self):
        """Rotor atoms except the axis atom, leaf by leaf (data.cpp:358-361)."""
        out = []
        for (a0, a1), g in zip(self.rotor_axis, self.rotor_groups):
            out.extend(a for a in g if a != a1)
        return out


class TorsionTree:
    """Flat fragment tree (fill(fragment_tree), data.cpp:410-482)."""

    def __init__(self, n_atoms, frag_start, frag_end, perm, roots, tors_frag, tors_parent,
                 tors_parent_atom, tors_mine_atom):
        self.n_atoms = n_atoms
        self.frag_start = _i32(frag_start)
        self.frag_end = _i32(frag_end)
        self.perm = _i32(perm)
        self.roots = _i32(roots)
        self.tors_frag = _i32(tors_frag)
        self.tors_parent = _i32(tors_parent)
        self.tors_parent_atom = _i32(tors_parent_atom)
        self.tors_mine_atom = _i32(tors_mine_atom)

    @property
    def n_frags(self):
        return len(self.frag_start)

    @property
    def n_torsions(self):
        return len(self.tors_frag)

    @classmethod
    def from_json(cls, geo):
        n = int(geo["num_atoms"])
        split = [int(v) for v in geo["frag_split_index"]]
        F = len(split) + 1
        children = {}
        roots = []
        for level in geo["frag_traverse_levels"]:
            for key, node in level.items():
                f = int(key)
                if len(node["parent"]) == 0:
                    roots.append(f)
                children[f] = [int(c) for c in node["children"]]
        bounds = [0] + split + [n]
        frag_start = [bounds[f] for f in range(F)]
        frag_end = [bounds[f + 1] for f in range(F)]
        perm = [int(v) for v in geo["permute_index"]]
        rev = [0] * len(perm)
        for p, a in enumerate(perm):
            rev[a] = p
        bonds = {k: (rev[int(v[0])], rev[int(v[1])]) for k, v in geo["edge_to_bond"].items()}
        tf, tp, tpa, tma = [], [], [], []

        def walk(node):  # pre-order, children in listed order (data.cpp:562-590)
            for c in children.get(node, []):
                pa, ma = bonds["%d->%d" % (node, c)]
                tf.append(c)
                tp.append(node)
                tpa.append(pa)
                tma.append(ma)
                walk(c)

        for r in roots:
            walk(r)
        return cls(n, frag_start, frag_end, perm, roots, tf, tp, tpa, tma)

    def to_c(self, keep):
        t = abi.TorsionTree()
        t.n_frags = self.n_frags
        t.n_roots = len(self.roots)
        t.n_torsions = self.n_torsions
        for name in ("frag_start", "frag_end", "perm", "roots", "tors_frag", "tors_parent",
                     "tors_parent_atom", "tors_mine_atom"):
            arr = getattr(self, name)
            keep.append(arr)
            setattr(t, name, arr.ctypes.data_as(abi.i32p) if arr.size else C.cast(None, abi.i32p))
        return t


class Ligand:
    """free_ligand (data.h:70-99) as flat arrays, with its poses."""

    def __init__(self, topology, vdw_type, tree, poses, smiles="", raw=None):
        self.ff = topology
        self.vdw_type = _i32(vdw_type)
        self.tree = tree
        self.poses = _f64(poses).reshape(-1, topology.n_atoms, 3)
        self.smiles = smiles
        self.raw = raw

    @property
    def n_atoms(self):
        return self.ff.n_atoms

    @property
    def n_torsions(self):
        return 0 if self.tree is None else self.tree.n_torsions

    @classmethod
    def from_json(cls, d, geometry=True):
        ff = d["ffdata"]
        types = [int(v) - VDW_OFFSET for v in ff["FF_vdW_paraidx"]]
        for i, t in enumerate(types):
            if t > 98 or t < 0:
                raise ValueError("VDW type [%d] of atom#%dis illegal!" % (t, i))
        sig, eps = vdw_table()
        n = len(types)
        if n == 0 and len(d["xyz"]) > 0:
            # kinematics-only fixtures carry coordinates but no force field
            n = len(d["xyz"][0])
            types = [0] * n
        top = Topology.from_ffdata(ff, n, sig[types] if n else [], eps[types] if n else [])
        tree = TorsionTree.from_json(d["geometry"]) if geometry and "geometry" in d else None
        poses = np.array(d["xyz"], dtype=np.float64).reshape(-1, n, 3)
        lig = cls(top, types, tree, poses, d.get("mapped_smiles", ""), raw=d)
        lig.lists = ScoreLists(ff, n, ligand=True)
        return lig

    @classmethod
    def from_file(cls, path, geometry=True):
        with open(path) as f:
            return cls.from_json(json.load(f), geometry)

    def to_c(self, keep):
        lig = abi.LigandDesc()
        lig.ff = self.ff.to_c(keep)
        keep.append(self.vdw_type)
        lig.vdw_type = self.vdw_type.ctypes.data_as(abi.i32p)
        if self.tree is not None:
            lig.tree = self.tree.to_c(keep)
        lists = getattr(self, "lists", None)
        if lists is not None:
            lc = lists.to_c(keep)
            keep.append(lc)
            lig.lists = C.pointer(lc)
        return lig


def decide_grid_dims(center, size, spacing):
    """decide_grid_dims (grid.cpp:65-86) -> (init_xyz, npoints)."""
    init, npts = [], []
    for c, s in zip(center, size):
        nv = int(math.ceil(s / spacing))
        if nv % 2 == 1:
            nv += 1
        length = nv * spacing
        npts.append(nv + 1)
        init.append(c - length * 0.5)
    return init, npts


def make_box(center, size, spacing):
    init, npts = decide_grid_dims(center, size, spacing)
    b = abi.Box()
    for d in range(3):
        b.init_xyz[d] = init[d]
        b.npoints[d] = npts[d]
    b.spacing = spacing
    return b


# ---------------------------------------------------------------- empirical scores
class ScoreLists:
    """Interaction atom lists of one molecule (the pscore / bscore fields of the engine
    JSON, parsed as data.cpp:271-295 does)."""

    def __init__(self, ff, n_atoms, ligand):
        def idx(key):
            return _i32(ff.get(key, [])).reshape(-1)

        def pairs(key):
            return _i32(ff.get(key, [])).reshape(-1, 2)

        def rings(key):
            rs = ff.get(key, [])
            out = -np.ones((len(rs), 6), np.int32)
            for k, r in enumerate(rs):
                out[k, : len(r)] = r
            return out

        self.hydrophobic = idx("hydrophobic_atomidx")
        self.cation = idx("cation_atomidx")
        self.anion = idx("anion_atomidx")
        self.ring5 = rings("piring5_atomidx")
        self.ring6 = rings("piring6_atomidx")
        self.don_charged = pairs("hbonddon_charged_atomidx")
        self.don_neutral = pairs("hbonddon_neut_atomidx")
        self.acc_charged = idx("hbondacc_charged_atomidx")
        self.acc_neutral = idx("hbondacc_neut_atomidx")
        coefs, offs, quads = [], [0], []
        if ligand:  # data.cpp:201-219
            for entry, params in zip(ff.get("tstrain_atomidx_pose_selection", []),
                                     ff.get("tstrain_params_pose_selection", [])):
                coefs.append([float(v) for v in params])
                for q in entry:
                    quads.append([int(v) for v in q])
                offs.append(len(quads))
        self.tstrain_coefs = _f64(coefs).reshape(-1, 4)
        self.tstrain_offsets = _i32(offs)
        self.tstrain_quads = _i32(quads).reshape(-1, 4)
        self.n_rotatable = len(ff.get("rotatable_bond_index", [])) if ligand else 0
        an = ff.get("atomic_numbers", [])
        self.atomic_numbers = _i32(an if len(an) == n_atoms else [0] * n_atoms)
        self.all_bonds = pairs("bond_index")

    def to_c(self, keep):
        s = abi.ScoreLists()

        def p(name, arr, ctype=C.c_int32):
            keep.append(arr)
            setattr(s, name, arr.ctypes.data_as(C.POINTER(ctype)) if arr.size else
                    C.cast(None, C.POINTER(ctype)))

        for name in ("hydrophobic", "cation", "anion", "ring5", "ring6", "don_charged",
                     "don_neutral", "acc_charged", "acc_neutral"):
            arr = getattr(self, name)
            setattr(s, "n_" + name, len(arr))
            p(name, arr)
        s.n_tstrain = len(self.tstrain_coefs)
        p("tstrain_coefs", self.tstrain_coefs, C.c_double)
        p("tstrain_offsets", self.tstrain_offsets)
        p("tstrain_quads", self.tstrain_quads)
        s.n_rotatable = self.n_rotatable
        p("atomic_numbers", self.atomic_numbers)
        s.n_all_bonds = len(self.all_bonds)
        p("all_bonds", self.all_bonds)
        return s


def _sf_active(x):
    return x > 1e-5 or x < -1e-5  # CHECK_PARAMETER_NON_ZERO, utility.h:26


def scoring_function_params(node):
    """pxd_sf_params from one section ("pose_selection" / "affinity_ranking") of a
    scoring-function JSON, as fill(ScoringFunctionParams) and the root_scorer constructor
    read it (factory.cpp:144-202, scorer.cpp:53-115). The reference registers the
    rotatable-energy weight under the name "TorsionStrain_Penalty" (scorer.cpp:103-106),
    so a non-zero rotatable weight replaces the torsion-strain weight and the
    rotatable term itself is never summed; the effective weights here say exactly that."""
    p = abi.SfParams()
    keys = ["interaction_coulomb_energy_coef", "interaction_vdw_energy_coef", "ionic_energy_coef",
            "pi_cationic_energy_coef", "f2f_pi_stacking_energy_coef",
            "e2f_pi_stacking_energy_coef", "hbond_energy_coef", "hydrophobic_energy_coef",
            "torsion_strain_penalty_coef", "rotatable_energy_coef", "gbsa_energy_delta_coef"]
    raw = [float(node.get(k, 0.0)) for k in keys]
    eff = list(raw)
    eff[9] = 0.0
    if _sf_active(raw[9]):
        eff[8] = raw[9] if _sf_active(raw[8]) else 0.0
    for k in range(11):
        p.coef[k] = eff[k] if _sf_active(raw[k]) or k == 8 else 0.0
    if _sf_active(raw[1]):
        v = node["interaction_vdw_energy"]
        p.vdw_scale = float(v["scale"])
        p.vdw_cutoff = float(v["cutoff"])
        # types beyond the file's list keep the neutral scale 1 (the reference reads
        # past its list there: scorer.cpp indexes the scales by ligand type)
        for t in range(99):
            p.vdw_sigma_scale[t] = 1.0
            p.vdw_epsilon_scale[t] = 1.0
        for t, ty in enumerate(v["types"][:99]):
            p.vdw_sigma_scale[t] = float(ty["sigma_scale"])
            p.vdw_epsilon_scale[t] = float(ty["epsilon_scale"])
    if _sf_active(raw[2]):
        v = node["ionic_energy"]
        p.ionic_coef[0], p.ionic_coef[1] = float(v["lc_coef"]), float(v["pc_coef"])
        for k, name in enumerate(("lc_inter", "pc_inter")):
            p.ionic[k][0] = float(v[name]["dist_min"])
            p.ionic[k][1] = float(v[name]["dist_max"])
    if _sf_active(raw[3]):
        v = node["pi_cationic_energy"]
        for k, name in enumerate(("lc5", "lc6", "pc5", "pc6")):
            p.picat_coef[k] = float(v[name + "_coef"])
            p.picat[k][0] = float(v[name + "_inter"]["dist_min"])
            p.picat[k][1] = float(v[name + "_inter"]["dist_max"])
    for w, key in ((0, "f2f_pi_stacking_energy"), (1, "e2f_pi_stacking_energy")):
        if not _sf_active(raw[4 + w]):
            continue
        v = node[key]
        for k, name in enumerate(("l5r5", "l5r6", "l6r5", "l6r6")):
            p.stack_coef[w][k] = float(v[name + "_coef"])
            it = v[name + "_inter"]
            for u, f in enumerate(("dist_min", "dist_max", "angle_min", "angle_max", "sigma_min",
                                   "sigma_max")):
                p.stack[w][k][u] = float(it[f])
    if _sf_active(raw[6]):
        v = node["hbond_energy"]
        p.hbond_scale = float(v["scale"])
        for k, name in enumerate(("hldcc", "hldcn", "hldnc", "hldnn", "hpdcc", "hpdcn", "hpdnc",
                                  "hpdnn")):
            p.hbond_coef[k] = float(v[name + "_coef"])
            it = v[name + "_inter"]
            for u, f in enumerate(("dist_min", "dist_max", "angle_min", "angle_max", "dist_center",
                                   "angle_center")):
                p.hbond[k][u] = float(it[f])
    if _sf_active(raw[7]):
        v = node["hydrophobic_energy"]
        p.hydro_scale = float(v["scale"])
        p.hydro_dist_min = float(v["dist_min"])
        p.hydro_dist_max = float(v["dist_max"])
        p.hydro_scale_factor = float(v["scale_factor"])
    if not _sf_active(raw[8]):
        p.coef[8] = 0.0
    return p


def load_scoring_function(path):
    """(pose_selection, affinity_ranking) pxd_sf_params of a scoring-function file."""
    with open(path) as f:
        d = json.load(f)
    return scoring_function_params(d["pose_selection"]), scoring_function_params(d["affinity_ranking"])
