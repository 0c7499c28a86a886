"""Seeded synthetic complexes in the engine's JSON schema.

The public benchmark sets are not available here, so seeded synthetic inputs of the
named shapes stand in for them:
  receptor  heavy atoms drawn uniformly in a cube with a minimum spacing, element mix
            C 62 / N 17 / O 19 / S 2 %, a polar H on every N and on 40 % of O, FF14SB-like
            per-element sigma/epsilon, charges ~N(0, 0.25) clipped to +-0.8 and shifted
            to net zero. A spherical cavity is kept free of atoms around the box centre so
            that the pocket can hold a ligand. Optional polar-H rotors (O-H about C-O).
  ligand    rigid fragments (aromatic 6- and 5-rings, sp3 linkers, amide / carbonyl /
            ether units) joined by exactly n_rot rotatable single bonds, decorated with
            N / O / halogen substituents, hydrogens to valence, built with ideal geometry
            and clash rejection. GAFF2-style type indices (type + 1000), bonded terms in
            GAFF2 ranges, pair lists by the rule of calc_nonbonded_atomidx
            (pxdock/parser/ffdata.py:179-226), the fragment tree by the rules of
            RigidFragmentTree (pxdock/geometry/tree.py:93-260).
The JSON written here is read by the same parsers as real prepared inputs.
"""
import math
import os

import numpy as np

# GAFF2 type indices in the ligand vdW table order (kVdwTypeTags)
T_C, T_C2, T_C3, T_CA = 0, 3, 4, 5
T_HA, T_HC, T_HN, T_HO = 26, 27, 28, 29
T_F, T_CL, T_BR = 34, 35, 36
T_N, T_N3, T_NA, T_NB = 38, 41, 43, 44
T_O, T_OH, T_OS = 72, 73, 76
T_SS = 94

ATOMIC_NUMBER = {"C": 6, "N": 7, "O": 8, "S": 16, "F": 9, "Cl": 17, "Br": 35, "H": 1}
MASS = {"C": 12.011, "N": 14.007, "O": 15.999, "S": 32.06, "F": 18.998, "Cl": 35.45,
        "Br": 79.904, "H": 1.008}
BOND_LEN = {("C", "C"): 1.53, ("C", "N"): 1.47, ("C", "O"): 1.43, ("C", "S"): 1.81,
            ("C", "F"): 1.35, ("C", "Cl"): 1.76, ("C", "Br"): 1.93, ("C", "H"): 1.09,
            ("N", "H"): 1.01, ("O", "H"): 0.96, ("N", "N"): 1.45, ("N", "O"): 1.40,
            ("O", "O"): 1.45, ("N", "S"): 1.70, ("O", "S"): 1.60, ("S", "S"): 2.05}


def _blen(a, b):
    return BOND_LEN.get((a, b)) or BOND_LEN.get((b, a)) or 1.5


# 3-vector cross product and norm with the values numpy's cross / linalg.norm give (the
# same IEEE products and the same sqrt of the dot product), without their per-call
# overhead, which dominated ligand generation.
def _cross3(a, b):
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]])


def _norm3(v):
    return math.sqrt(v.dot(v))


def _unit(v):
    return v / _norm3(v)


def _perp(v, rng):
    while True:
        w = _cross3(v, rng.normal(size=3))
        n = _norm3(w)
        if n > 1e-3:
            return w / n


def _rot(axis, ang):
    axis = _unit(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + math.sin(ang) * K + (1 - math.cos(ang)) * (K @ K)


# --------------------------------------------------------------------- receptor
def make_receptor(seed=0, n_heavy=1500, cube=26.0, min_dist=1.4, center=(0.0, 0.0, 0.0),
                  cavity=7.0, n_rotors=0, n_rings=(4, 8)):
    rng = np.random.default_rng(seed)
    center = np.asarray(center, float)
    half = cube / 2.0
    cell = min_dist
    ncell = int(math.ceil(cube / cell)) + 2
    grid = {}
    pts = []
    tries = 0
    while len(pts) < n_heavy:
        tries += 1
        if tries > n_heavy * 200:
            raise RuntimeError("cannot place receptor atoms")
        p = center + rng.uniform(-half, half, size=3)
        if np.linalg.norm(p - center) < cavity:
            continue
        key = tuple(((p - center + half) // cell).astype(int))
        ok = True
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for q in grid.get((key[0] + dx, key[1] + dy, key[2] + dz), ()):
                        if np.sum((q - p) ** 2) < min_dist * min_dist:
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if not ok:
                break
        if ok:
            grid.setdefault(key, []).append(p)
            pts.append(p)
    del ncell
    elems = rng.choice(["C", "N", "O", "S"], size=n_heavy, p=[0.62, 0.17, 0.19, 0.02])
    xyz = [list(p) for p in pts]
    el = list(elems)
    parent = [-1] * n_heavy
    for i in range(n_heavy):
        if el[i] == "N" or (el[i] == "O" and rng.random() < 0.4):
            d = _unit(rng.normal(size=3))
            xyz.append(list(np.asarray(pts[i]) + d * 1.0))
            el.append("H")
            parent.append(i)
    n = len(xyz)
    sig_eps = {"C": (3.3997, 0.0860), "N": (3.2500, 0.1700), "O": (3.0665, 0.2104),
               "S": (3.5636, 0.2500)}
    sigma, eps = [], []
    for i in range(n):
        if el[i] == "H":
            if el[parent[i]] == "N":
                sigma.append(1.0691), eps.append(0.0157)
            else:
                sigma.append(0.0), eps.append(0.0)
        else:
            s, e = sig_eps[el[i]]
            sigma.append(s), eps.append(e)
    q = np.clip(rng.normal(0.0, 0.25, size=n), -0.8, 0.8)
    q -= q.mean()
    xyz_a = np.asarray(xyz)
    heavy = np.arange(n_heavy)
    # interaction atom lists used by the pose-selection score
    hydrophobic = [i for i in heavy if el[i] in ("C", "S")]
    nitro = [i for i in heavy if el[i] == "N"]
    oxy = [i for i in heavy if el[i] == "O"]
    cations = [i for i in nitro if rng.random() < 0.1]
    anions = [i for i in oxy if rng.random() < 0.1]
    don_c, don_n = [], []
    for h in range(n_heavy, n):
        pair = [parent[h], h]
        (don_c if parent[h] in cations else don_n).append(pair)
    acc_c = list(anions)
    acc_n = [i for i in oxy if i not in anions]
    bond_index = [[parent[h], h] for h in range(n_heavy, n)]
    # aromatic-ring stand-ins: a carbon near the pocket and its nearest carbons
    rings5, rings6 = [], []
    carbons = np.array([i for i in heavy if el[i] == "C"])
    used = set()
    if len(carbons) > 12:
        cx = xyz_a[carbons]
        order = carbons[np.argsort(np.linalg.norm(cx - center, axis=1))]
        for size, out, count in ((5, rings5, n_rings[0]), (6, rings6, n_rings[1])):
            for c0 in order:
                if len(out) >= count:
                    break
                if c0 in used:
                    continue
                d = np.linalg.norm(cx - xyz_a[c0], axis=1)
                near = [int(carbons[k]) for k in np.argsort(d) if int(carbons[k]) not in used][:size]
                if len(near) < size or c0 not in near:
                    continue
                used.update(near)
                out.append(near)
    ff = {
        "FF_Bonds_atomidx": [], "FF_Bonds_k": [], "FF_Bonds_length": [],
        "FF_Angles_atomidx": [], "FF_Angles_k": [], "FF_Angles_angle": [],
        "FF_ProperTorsions_atomidx": [], "FF_ProperTorsions_periodicity": [],
        "FF_ProperTorsions_k": [], "FF_ProperTorsions_phase": [],
        "FF_ImproperTorsions_atomidx": [], "FF_ImproperTorsions_periodicity": [],
        "FF_ImproperTorsions_k": [], "FF_ImproperTorsions_phase": [],
        "FF_Nonbonded14_atomidx": [], "FF_NonbondedAll_atomidx": [],
        "hydrophobic_atomidx": [int(i) for i in hydrophobic],
        "cation_atomidx": [int(i) for i in cations],
        "anion_atomidx": [int(i) for i in anions],
        "piring5_atomidx": rings5, "piring6_atomidx": rings6,
        "hbonddon_charged_atomidx": [[int(a), int(b)] for a, b in don_c],
        "hbonddon_neut_atomidx": [[int(a), int(b)] for a, b in don_n],
        "hbondacc_charged_atomidx": [int(i) for i in acc_c],
        "hbondacc_neut_atomidx": [int(i) for i in acc_n],
        "partial_charges": [round(float(v), 6) for v in q],
        "FF_vdW_sigma": sigma, "FF_vdW_epsilon": eps,
        "rotatable_bond_index": [], "bond_index": bond_index,
        "atomic_numbers": [ATOMIC_NUMBER[e] for e in el],
    }
    geometry = {"num_atoms": n, "num_rotatable_bonds": 0, "data": {}}
    if n_rotors > 0:
        _add_receptor_rotors(rng, xyz_a, el, parent, n_heavy, ff, geometry, n_rotors, center)
    return {"xyz": [[round(float(c), 4) for c in p] for p in xyz_a], "ffdata": ff,
            "geometry": geometry}


def _add_receptor_rotors(rng, xyz, el, parent, n_heavy, ff, geometry, n_rotors, center):
    """Hydroxyl rotors: H turns about the (nearest C) -> O axis; bonded terms touch H."""
    cands = [h for h in range(n_heavy, len(el)) if el[parent[h]] == "O"]
    cands.sort(key=lambda h: np.linalg.norm(xyz[h] - center))
    carbons = [i for i in range(n_heavy) if el[i] == "C"]
    cxyz = xyz[carbons]
    chosen = cands[:n_rotors]
    frags, b1, b2, order = [], [], [], []
    for r, h in enumerate(chosen):
        o = parent[h]
        c = carbons[int(np.argmin(np.sum((cxyz - xyz[o]) ** 2, axis=1)))]
        frags.append([o, h])
        b1.append(c)
        b2.append(o)
        order.append(r)
        ff["FF_Bonds_atomidx"].append([o, h])
        ff["FF_Bonds_k"].append(1106.0)
        ff["FF_Bonds_length"].append(0.96)
        ang = math.degrees(math.acos(np.clip(np.dot(_unit(xyz[c] - xyz[o]), _unit(xyz[h] - xyz[o])),
                                             -1, 1)))
        ff["FF_Angles_atomidx"].append([c, o, h])
        ff["FF_Angles_k"].append(94.0)
        ff["FF_Angles_angle"].append(round(0.5 * ang + 0.5 * 108.5, 4))
        # a proper on X-C-O-H with the nearest other heavy atom as X
        d2 = np.sum((xyz[:n_heavy] - xyz[c]) ** 2, axis=1)
        d2[[c, o]] = 1e9
        x = int(np.argmin(d2))
        ff["FF_ProperTorsions_atomidx"].append([x, c, o, h])
        ff["FF_ProperTorsions_periodicity"].append([3])
        ff["FF_ProperTorsions_k"].append([0.1667])
        ff["FF_ProperTorsions_phase"].append([0.0])
        ff["FF_Nonbonded14_atomidx"].append(sorted([x, h]))
        near = np.where(np.sum((xyz - xyz[h]) ** 2, axis=1) < 16.0)[0]
        for j in near:
            j = int(j)
            if j in (h, o, c, x):
                continue
            ff["FF_NonbondedAll_atomidx"].append(sorted([j, h]))
    geometry["num_rotatable_bonds"] = len(chosen)
    geometry["data"] = {"1": {"fragments": frags, "rot_bond_1": b1, "rot_bond_2": b2,
                              "rot_bond_order": order}}


# ----------------------------------------------------------------------- ligand
class _Mol:
    def __init__(self):
        self.el, self.ty, self.hyb, self.xyz = [], [], [], []
        self.bonds = {}          # (i, j) sorted -> dict(rot=bool, order=1|2|1.5)
        self.nbr = []
        self.ring = []           # ring id or -1
        self.rings = []          # list of (atom list, aromatic)
        self.frag = []           # rigid fragment id (before rotatable bonds)

    def add(self, el, ty, hyb, pos, frag, ring=-1):
        self.el.append(el)
        self.ty.append(ty)
        self.hyb.append(hyb)
        self.xyz.append(np.asarray(pos, float))
        self.nbr.append([])
        self.ring.append(ring)
        self.frag.append(frag)
        return len(self.el) - 1

    def bond(self, i, j, rot=False, order=1):
        self.bonds[tuple(sorted((i, j)))] = dict(rot=rot, order=order)
        self.nbr[i].append(j)
        self.nbr[j].append(i)


MAX_VALENCE = {"C": 4, "N": 3, "O": 2, "S": 2, "F": 1, "Cl": 1, "Br": 1, "H": 1}


def _free_dirs(m, i, rng, count):
    """Unit directions for `count` new neighbours of atom i (sp3 / sp2 geometry)."""
    nb = [_unit(m.xyz[j] - m.xyz[i]) for j in m.nbr[i]]
    hyb = m.hyb[i]
    if m.ring[i] >= 0:
        atoms = m.rings[m.ring[i]][0]
        cen = np.mean([m.xyz[a] for a in atoms], axis=0)
        out = _unit(m.xyz[i] - cen)
        if hyb == "ar" or count == 1:
            return [out] * count
        nrm = _unit(_cross3(m.xyz[atoms[1]] - m.xyz[atoms[0]], m.xyz[atoms[2]] - m.xyz[atoms[0]]))
        return [_unit(out * 0.58 + nrm * 0.81), _unit(out * 0.58 - nrm * 0.81)][:count]
    if hyb == "sp2":
        if len(nb) == 0:
            a = _unit(rng.normal(size=3))
            b = _perp(a, rng)
            return [a, _unit(-0.5 * a + 0.866 * b), _unit(-0.5 * a - 0.866 * b)][:count]
        if len(nb) == 1:
            a = -nb[0]
            b = _perp(a, rng)
            return [_unit(0.5 * a + 0.866 * b), _unit(0.5 * a - 0.866 * b)][:count]
        return [_unit(-(nb[0] + nb[1]))][:count]
    # sp3
    if len(nb) == 0:
        t = [np.array([1, 1, 1.0]), np.array([1, -1, -1.0]), np.array([-1, 1, -1.0]),
             np.array([-1, -1, 1.0])]
        R = _rot(rng.normal(size=3), rng.uniform(0, 2 * math.pi))
        return [_unit(R @ v) for v in t][:count]
    if len(nb) == 1:
        a = -nb[0]
        b = _perp(a, rng)
        c = _cross3(a, b)
        ca, sa = math.cos(math.radians(70.5)), math.sin(math.radians(70.5))
        out = []
        for k in range(3):
            phi = 2 * math.pi * k / 3
            out.append(_unit(ca * a + sa * (math.cos(phi) * b + math.sin(phi) * c)))
        return out[:count]
    if len(nb) == 2:
        bis = _unit(-(nb[0] + nb[1]))
        nrm = _unit(_cross3(nb[0], nb[1]))
        return [_unit(bis * 0.58 + nrm * 0.81), _unit(bis * 0.58 - nrm * 0.81)][:count]
    return [_unit(-(nb[0] + nb[1] + nb[2]))][:count]


def _ring(m, rng, size, frag, hetero=None):
    """Planar aromatic ring of `size` atoms in its own frame (placed later)."""
    rid = len(m.rings)
    atoms = []
    radius = 1.39 / (2 * math.sin(math.pi / size))
    for k in range(size):
        ang = 2 * math.pi * k / size
        pos = np.array([radius * math.cos(ang), radius * math.sin(ang), 0.0])
        el, ty = "C", T_CA
        if hetero is not None and k == hetero[0]:
            el, ty = hetero[1], hetero[2]
        atoms.append(m.add(el, ty, "ar", pos, frag, ring=rid))
    for k in range(size):
        m.bond(atoms[k], atoms[(k + 1) % size], order=1.5)
    m.rings.append((atoms, True))
    return atoms


def _frag_atoms(m, f):
    return [i for i in range(len(m.el)) if m.frag[i] == f]


def _place_fragment(m, f, anchor, new_atom, rng):
    """Moves fragment f rigidly so that new_atom sits bonded to anchor."""
    atoms = _frag_atoms(m, f)
    d_out = _free_dirs(m, anchor, rng, 1)[0]
    pos_new = m.xyz[anchor] + d_out * _blen(m.el[anchor], m.el[new_atom])
    # fragment's own outward direction at new_atom
    if m.ring[new_atom] >= 0:
        ring_atoms = m.rings[m.ring[new_atom]][0]
        own = _unit(m.xyz[new_atom] - np.mean([m.xyz[a] for a in ring_atoms], axis=0))
    elif len(m.nbr[new_atom]) > 0:
        own = _unit(-np.sum([_unit(m.xyz[j] - m.xyz[new_atom]) for j in m.nbr[new_atom]], axis=0))
    else:
        own = np.array([1.0, 0.0, 0.0])
    target = -d_out
    v = _cross3(own, target)
    s, c = _norm3(v), float(np.dot(own, target))
    if s < 1e-8:
        R = np.eye(3) if c > 0 else _rot(_perp(own, rng), math.pi)
    else:
        R = _rot(v, math.atan2(s, c))
    R = _rot(target, rng.uniform(0, 2 * math.pi)) @ R
    origin = m.xyz[new_atom].copy()
    for a in atoms:
        m.xyz[a] = pos_new + R @ (m.xyz[a] - origin)


def _clash_free(m, min_heavy=2.2, min_h=1.6):
    n = len(m.el)
    X = np.asarray(m.xyz)
    topo = _topo_dist(m, 3)
    for i in range(n):
        d = np.sqrt(np.sum((X[i + 1:] - X[i]) ** 2, axis=1))
        for k, dist in enumerate(d):
            j = i + 1 + k
            if topo.get((i, j), 99) <= 3:
                continue
            lim = min_h if (m.el[i] == "H" or m.el[j] == "H") else min_heavy
            if dist < lim:
                return False
    return True


def _topo_dist(m, maxd):
    out = {}
    for s in range(len(m.el)):
        seen = {s: 0}
        frontier = [s]
        for d in range(1, maxd + 1):
            nxt = []
            for a in frontier:
                for b in m.nbr[a]:
                    if b not in seen:
                        seen[b] = d
                        nxt.append(b)
            frontier = nxt
        for b, d in seen.items():
            if b > s:
                out[(s, b)] = d
    return out


def _build_skeleton(rng, n_heavy, n_rot, n_n, n_o, n_other):
    """Rigid fragments joined by n_rot rotatable bonds; returns the molecule or None."""
    m = _Mol()
    frags = []
    budget = n_heavy - n_n - n_o - n_other
    n_frags = n_rot + 1
    # choose fragment kinds so that carbon count fits the budget
    kinds = []
    remaining = budget
    for f in range(n_frags):
        left = n_frags - f - 1
        opts = []
        if remaining - 6 >= left:
            opts += ["ar6", "ar6"]
        if remaining - 5 >= left:
            opts += ["ar5"]
        if remaining - 1 >= left:
            opts += ["sp3", "sp3", "sp2c"]
        if not opts:
            return None
        k = rng.choice(opts)
        kinds.append(k)
        remaining -= {"ar6": 6, "ar5": 5, "sp3": 1, "sp2c": 1}[k]
    if remaining < 0:
        return None
    for f, k in enumerate(kinds):
        if k == "ar6":
            frags.append(_ring(m, rng, 6, f))
        elif k == "ar5":
            frags.append(_ring(m, rng, 5, f))
        elif k == "sp3":
            frags.append([m.add("C", T_C3, "sp3", [0, 0, 0], f)])
        else:
            frags.append([m.add("C", T_C2, "sp2", [0, 0, 0], f)])
    # random tree over fragments with rotatable bonds, placed in order
    placed = [0]
    for f in range(1, n_frags):
        for _ in range(50):
            pf = int(rng.choice(placed))
            a = int(rng.choice(frags[pf]))
            if len(m.nbr[a]) >= _cap(m, a) - 0:
                continue
            b = int(rng.choice(frags[f]))
            if len(m.nbr[b]) >= _cap(m, b):
                continue
            break
        else:
            return None
        _place_fragment(m, f, a, b, rng)
        m.bond(a, b, rot=True)
        placed.append(f)
    # extra carbons as methyl/chain substituents inside fragments (non-rotatable)
    return m, remaining


def _cap(m, i):
    """Heavy-neighbour capacity of atom i."""
    if m.hyb[i] == "ar":
        return 3
    if m.el[i] == "C":
        return 4 if m.hyb[i] == "sp3" else 3
    return MAX_VALENCE[m.el[i]]


def _attach(m, i, el, ty, hyb, rng, rot=False, order=1):
    d = _free_dirs(m, i, rng, 1)[0]
    blen = _blen(m.el[i], el) - (0.2 if order == 2 else 0.0)
    j = m.add(el, ty, hyb, m.xyz[i] + d * blen, m.frag[i])
    m.bond(i, j, rot=rot, order=order)
    return j


def make_ligand(seed=1, n_heavy=24, n_rot=5, n_n=2, n_o=3, n_other=0, other="Cl",
                max_tries=400):
    """A drug-like ligand in the engine's ligand JSON schema (one pose)."""
    rng = np.random.default_rng(seed)
    for _ in range(max_tries):
        res = _build_skeleton(rng, n_heavy, n_rot, n_n, n_o, n_other)
        if res is None:
            continue
        m, extra_c = res
        ok = True
        # extra carbons: methyl groups on free ring / sp3 atoms
        for _ in range(extra_c):
            cands = [i for i in range(len(m.el)) if m.el[i] == "C" and len(m.nbr[i]) < _cap(m, i)]
            if not cands:
                ok = False
                break
            _attach(m, int(rng.choice(cands)), "C", T_C3, "sp3", rng)
        if not ok:
            continue
        # heteroatom substituents
        subs = ["N"] * n_n + ["O"] * n_o + [other] * n_other
        rng.shuffle(subs)
        for el in subs:
            cands = [i for i in range(len(m.el)) if m.el[i] == "C" and len(m.nbr[i]) < _cap(m, i)]
            if not cands:
                ok = False
                break
            i = int(rng.choice(cands))
            if el == "O":
                if m.hyb[i] == "sp2" and len(m.nbr[i]) <= 2 and not any(
                        m.bonds[tuple(sorted((i, j)))]["order"] == 2 for j in m.nbr[i]):
                    _attach(m, i, "O", T_O, "sp2", rng, order=2)
                    m.ty[i] = T_C
                else:
                    _attach(m, i, "O", T_OH, "sp3", rng)
            elif el == "N":
                _attach(m, i, "N", T_N3, "sp3", rng)
            elif el == "S":
                s = _attach(m, i, "S", T_SS, "sp3", rng)
                del s
            else:
                _attach(m, i, el, {"F": T_F, "Cl": T_CL, "Br": T_BR}[el], "sp3", rng)
        if not ok:
            continue
        _add_hydrogens(m, rng)
        if not _clash_free(m):
            continue
        return _ligand_json(m, rng)
    raise RuntimeError("ligand generation failed")


def _add_hydrogens(m, rng):
    n0 = len(m.el)
    for i in range(n0):
        el = m.el[i]
        if el in ("F", "Cl", "Br"):
            continue
        if m.hyb[i] == "ar":
            need = 3 - len(m.nbr[i]) if el == "C" else 0
        elif el == "C":
            order = sum(1 if m.bonds[tuple(sorted((i, j)))]["order"] != 2 else 2 for j in m.nbr[i])
            need = (4 if m.hyb[i] == "sp3" else 4) - order
            if m.hyb[i] == "sp2":
                need = 3 - len(m.nbr[i]) - (1 if order > len(m.nbr[i]) else 0)
                need = max(need, 0)
        elif el == "N":
            need = 3 - len(m.nbr[i])
        elif el == "O":
            need = 0 if any(m.bonds[tuple(sorted((i, j)))]["order"] == 2 for j in m.nbr[i]) \
                else 2 - len(m.nbr[i])
        elif el == "S":
            need = 2 - len(m.nbr[i])
        else:
            need = 0
        if need <= 0:
            continue
        dirs = _free_dirs(m, i, rng, need)
        hty = {"C": T_HA if m.hyb[i] == "ar" else T_HC, "N": T_HN, "O": T_HO, "S": T_HC}[el]
        for d in dirs[:need]:
            j = m.add("H", hty, "h", m.xyz[i] + d * _blen(el, "H"), m.frag[i])
            m.bond(i, j)


def _angle(a, b, c):
    u, v = _unit(a - b), _unit(c - b)
    return math.degrees(math.acos(np.clip(np.dot(u, v), -1.0, 1.0)))


def _ligand_json(m, rng):
    n = len(m.el)
    X = np.asarray(m.xyz)
    X -= X.mean(axis=0)
    bonds = sorted(m.bonds.keys())
    # bonded terms at the built geometry (so the input pose is near equilibrium)
    bk, bl = [], []
    for i, j in bonds:
        o = m.bonds[(i, j)]["order"]
        hydrogen = "H" in (m.el[i], m.el[j])
        bk.append(float(rng.uniform(650, 760) if hydrogen else (950 if o == 1.5 else
                                                                (1300 if o == 2 else rng.uniform(520, 700)))))
        bl.append(round(float(np.linalg.norm(X[i] - X[j])), 4))
    angles = []
    for j in range(n):
        nb = sorted(m.nbr[j])
        for a in range(len(nb)):
            for c in range(a + 1, len(nb)):
                angles.append((nb[a], j, nb[c]))
    ak = [float(rng.uniform(85, 105) if "H" in (m.el[i], m.el[k]) else rng.uniform(120, 145))
          for i, j, k in angles]
    aa = [round(_angle(X[i], X[j], X[k]), 3) for i, j, k in angles]
    propers = []
    for (j, k) in bonds:
        for i in m.nbr[j]:
            if i == k:
                continue
            for l in m.nbr[k]:
                if l == j or l == i:
                    continue
                propers.append((i, j, k, l))
    pper, pk, pph = [], [], []
    for (i, j, k, l) in propers:
        b = m.bonds[tuple(sorted((j, k)))]
        if b["order"] == 1.5:
            pper.append([2]), pk.append([3.625]), pph.append([180.0])
        elif b["order"] == 2:
            pper.append([2]), pk.append([2.5]), pph.append([180.0])
        elif b["rot"]:
            pper.append([1, 2, 3])
            pk.append([round(float(v), 4) for v in rng.uniform(0.0, 0.5, size=3)])
            pph.append([0.0, 180.0, 0.0])
        else:
            pper.append([3]), pk.append([0.15]), pph.append([0.0])
    impropers = []
    for j in range(n):
        if (m.hyb[j] in ("ar", "sp2")) and len(m.nbr[j]) == 3:
            a, b, c = m.nbr[j]
            impropers.append((j, a, b, c))
    # pair lists (calc_nonbonded_atomidx rule)
    nb12 = set(bonds)
    nb13 = {tuple(sorted((i, k))) for i, j, k in angles}
    nb14 = {tuple(sorted((i, l))) for i, j, k, l in propers} - nb12 - nb13
    allp = {(i, j) for i in range(n) for j in range(i + 1, n)} - nb14 - nb13 - nb12
    # charges
    base = {T_CA: -0.12, T_C3: -0.06, T_C2: -0.1, T_C: 0.55, T_HA: 0.13, T_HC: 0.04,
            T_HN: 0.36, T_HO: 0.41, T_N3: -0.85, T_NA: -0.3, T_NB: -0.6, T_O: -0.55,
            T_OH: -0.6, T_OS: -0.35, T_SS: -0.25, T_F: -0.2, T_CL: -0.1, T_BR: -0.08}
    q = np.array([base.get(t, 0.0) for t in m.ty]) + rng.normal(0, 0.03, size=n)
    q -= q.mean()
    # fragment tree from rotatable bonds
    rot = [b for b in bonds if m.bonds[b]["rot"]]
    geometry = fragment_tree_geometry(n, bonds, rot)
    hydro = [i for i in range(n) if m.el[i] == "C" and not any(m.el[j] in ("N", "O") for j in m.nbr[i])]
    hydro += [i for i in range(n) if m.el[i] in ("Cl", "Br", "F")]
    don = [[m.nbr[h][0], h] for h in range(n) if m.el[h] == "H" and m.el[m.nbr[h][0]] in ("N", "O")]
    acc = [i for i in range(n) if m.el[i] == "O" or (m.el[i] == "N" and m.hyb[i] == "ar")]
    ring5 = [a for a, aro in m.rings if aro and len(a) == 5]
    ring6 = [a for a, aro in m.rings if aro and len(a) == 6]
    tstrain_idx, tstrain_par = [], []
    for (j, k) in rot:
        i = next((a for a in m.nbr[j] if a != k), None)
        l = next((a for a in m.nbr[k] if a != j), None)
        if i is None or l is None:
            continue
        tstrain_idx.append([[i, j, k, l]])
        tstrain_par.append([round(float(v), 4) for v in rng.uniform(0.0, 0.6, size=4)])
    mw = float(sum(MASS[e] for e in m.el))
    ff = {
        "FF_Bonds_atomidx": [list(b) for b in bonds], "FF_Bonds_k": bk, "FF_Bonds_length": bl,
        "FF_Angles_atomidx": [list(a) for a in angles], "FF_Angles_k": ak, "FF_Angles_angle": aa,
        "FF_ProperTorsions_atomidx": [list(p) for p in propers],
        "FF_ProperTorsions_periodicity": pper, "FF_ProperTorsions_k": pk,
        "FF_ProperTorsions_phase": pph,
        "FF_ImproperTorsions_atomidx": [list(p) for p in impropers],
        "FF_ImproperTorsions_periodicity": [[2]] * len(impropers),
        "FF_ImproperTorsions_k": [[1.1]] * len(impropers),
        "FF_ImproperTorsions_phase": [[180.0]] * len(impropers),
        "FF_Nonbonded14_atomidx": [list(p) for p in sorted(nb14)],
        "FF_NonbondedAll_atomidx": [list(p) for p in sorted(allp)],
        "hydrophobic_atomidx": hydro,
        "cation_atomidx": [i for i in range(n) if m.ty[i] == T_N3],
        "anion_atomidx": [i for i in range(n) if m.ty[i] == T_O],
        "piring5_atomidx": ring5, "piring6_atomidx": ring6,
        "tstrain_atomidx_pose_selection": tstrain_idx,
        "tstrain_params_pose_selection": tstrain_par,
        "hbonddon_charged_atomidx": [], "hbonddon_neut_atomidx": don,
        "hbondacc_charged_atomidx": [], "hbondacc_neut_atomidx": acc,
        "partial_charges": [round(float(v), 6) for v in q],
        "FF_vdW_paraidx": [int(t) + 1000 for t in m.ty],
        "rotatable_bond_index": [list(b) for b in rot],
        "bond_index": [list(b) for b in bonds],
        "atomic_numbers": [ATOMIC_NUMBER[e] for e in m.el],
        "molecular_weight": round(mw, 3),
    }
    return {"mapped_smiles": "", "xyz": [[[round(float(c), 4) for c in p] for p in X]],
            "ffdata": ff, "geometry": geometry}


def fragment_tree_geometry(n, bonds, rot_bonds):
    """Fragment tree fields of the ligand JSON, by the rules of RigidFragmentTree and
    LigandGeometry (pxdock/geometry/tree.py:23-260, geometry.py:168-192)."""
    rot = {tuple(sorted(b)) for b in rot_bonds}
    adj = [[] for _ in range(n)]
    for b in bonds:
        if tuple(sorted(b)) in rot:
            continue
        adj[b[0]].append(b[1])
        adj[b[1]].append(b[0])
    comp = [-1] * n
    frags = []
    for s in range(n):  # components in order of their first atom
        if comp[s] >= 0:
            continue
        stack, members = [s], []
        comp[s] = len(frags)
        while stack:
            a = stack.pop()
            members.append(a)
            for b in adj[a]:
                if comp[b] < 0:
                    comp[b] = comp[s]
                    stack.append(b)
        frags.append(sorted(members))
    F = len(frags)
    qadj = [[] for _ in range(F)]
    edge = {}
    for i in range(F):
        for j in range(i + 1, F):
            rb = None
            for a, b in sorted(rot):
                if comp[a] == i and comp[b] == j:
                    rb = (a, b)
                elif comp[b] == i and comp[a] == j:
                    rb = (b, a)
                if rb is not None:
                    break
            if rb is not None:
                qadj[i].append(j)
                qadj[j].append(i)
                edge["%d->%d" % (i, j)] = [rb[0], rb[1]]
                edge["%d->%d" % (j, i)] = [rb[1], rb[0]]

    def bfs_order(src):
        seen, order, q = {src}, [src], [src]
        while q:
            nq = []
            for a in q:
                for b in qadj[a]:
                    if b not in seen:
                        seen.add(b)
                        order.append(b)
                        nq.append(b)
            q = nq
        return order

    def path(a, b):
        prev = {a: None}
        q = [a]
        while q:
            nq = []
            for x in q:
                for y in qadj[x]:
                    if y not in prev:
                        prev[y] = x
                        nq.append(y)
            q = nq
        out = [b]
        while out[-1] != a:
            out.append(prev[out[-1]])
        return out[::-1]

    if F <= 2:
        root = max(range(F), key=lambda f: (len(frags[f]), -f))
    else:
        f1 = bfs_order(0)[-1]
        f2 = bfs_order(f1)[-1]
        p = path(f1, f2)
        root = p[len(p) // 2]
    levels = []
    visited = set()
    current = [root]
    parent_of = {root: []}
    while current:
        visited.update(current)
        level = {}
        nxt = []
        for node in sorted(current):
            ch = sorted(set(qadj[node]) - visited)
            level[str(node)] = {"children": ch, "parent": parent_of[node]}
            for c in ch:
                parent_of[c] = [node]
            nxt += ch
        levels.append(level)
        current = nxt
    split = []
    acc = 0
    for f in frags:
        acc += len(f)
        split.append(acc)
    split.pop()
    return {"num_atoms": n, "permute_index": [a for f in frags for a in f],
            "frag_split_index": split, "frag_traverse_levels": levels, "edge_to_bond": edge}


# ------------------------------------------------------------------------ poses
def quaternion_matrix(q):
    """get_rotation_matrix(vector_4d) (math.cpp:22-42), vectorised over rows of q."""
    a, b, c, d = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    m = np.empty(q.shape[:-1] + (9,))
    m[..., 0] = a * a + b * b - c * c - d * d
    m[..., 1] = 2 * (b * c - a * d)
    m[..., 2] = 2 * (a * c + b * d)
    m[..., 3] = 2 * (a * d + b * c)
    m[..., 4] = a * a - b * b + c * c - d * d
    m[..., 5] = 2 * (c * d - a * b)
    m[..., 6] = 2 * (b * d - a * c)
    m[..., 7] = 2 * (a * b + c * d)
    m[..., 8] = a * a - b * b - c * c + d * d
    return m.reshape(q.shape[:-1] + (3, 3))


def random_quaternions(rng, n):
    """Uniform unit quaternions as random_orientation draws them (random.cpp:29-40)."""
    u1, u2, u3 = rng.random(n), rng.random(n) * 2 * math.pi, rng.random(n) * 2 * math.pi
    return np.stack([np.sqrt(1 - u1) * np.sin(u2), np.sqrt(1 - u1) * np.cos(u2),
                     np.sqrt(u1) * np.sin(u3), np.sqrt(u1) * np.cos(u3)], axis=1)


def _rodrigues(axis, theta):
    """get_rotation_matrix(axis, theta) (math.cpp:44-60), vectorised."""
    kx, ky, kz = axis[..., 0], axis[..., 1], axis[..., 2]
    st, ct = np.sin(theta), np.cos(theta)
    omc = 1 - ct
    m = np.empty(axis.shape[:-1] + (9,))
    m[..., 0] = ct + kx * kx * omc
    m[..., 1] = kx * ky * omc - kz * st
    m[..., 2] = ky * st + kx * kz * omc
    m[..., 3] = kz * st + kx * ky * omc
    m[..., 4] = ct + ky * ky * omc
    m[..., 5] = ky * kz * omc - kx * st
    m[..., 6] = kx * kz * omc - ky * st
    m[..., 7] = kx * st + ky * kz * omc
    m[..., 8] = ct + kz * kz * omc
    return m.reshape(axis.shape[:-1] + (3, 3))


def apply_parameters(tree, xyz, centers, rots, torsions):
    """free_ligand::apply_parameters (data.cpp:592-641) vectorised over poses.
    xyz [N,3] reference pose; centers [P,3]; rots [P,3,3]; torsions [P,T] -> [P,N,3]."""
    P = centers.shape[0]
    perm = tree.perm
    c = np.broadcast_to(xyz[perm], (P,) + xyz.shape).copy()
    F = tree.n_frags
    mine = -np.ones(F, int)
    axes = np.zeros((P, F, 3))
    for k in range(tree.n_torsions):
        f = tree.tors_frag[k]
        mine[f] = tree.tors_mine_atom[k]
        v = c[:, tree.tors_mine_atom[k]] - c[:, tree.tors_parent_atom[k]]
        axes[:, f] = v / np.linalg.norm(v, axis=1, keepdims=True)
    old_center = c.sum(axis=1) * (1.0 / c.shape[1])
    is_root = np.zeros(F, bool)
    is_root[tree.roots] = True
    for k in range(tree.n_torsions):
        f = tree.tors_frag[k]
        idx = [i for i in range(tree.frag_start[f], tree.frag_end[f]) if i != mine[f]]
        c[:, idx] -= c[:, mine[f]][:, None, :]
    for k in range(tree.n_torsions - 1, -1, -1):
        f, pf = tree.tors_frag[k], tree.tors_parent[k]
        c[:, mine[f]] -= old_center if is_root[pf] else c[:, mine[pf]]
    for r in tree.roots:
        c[:, tree.frag_start[r]:tree.frag_end[r]] -= old_center[:, None, :]
    fused = np.zeros((P, F, 3, 3))
    origin = np.zeros((P, F, 3))
    for r in tree.roots:
        fused[:, r] = rots
        origin[:, r] = centers
        sl = slice(tree.frag_start[r], tree.frag_end[r])
        c[:, sl] = np.einsum("pij,pnj->pni", rots, c[:, sl]) + centers[:, None, :]
    for k in range(tree.n_torsions):
        f, pf = tree.tors_frag[k], tree.tors_parent[k]
        axes[:, f] = np.einsum("pij,pj->pi", fused[:, pf], axes[:, f])
        c[:, mine[f]] = np.einsum("pij,pj->pi", fused[:, pf], c[:, mine[f]]) + origin[:, pf]
        fused[:, f] = np.einsum("pij,pjk->pik", _rodrigues(axes[:, f], torsions[:, k]), fused[:, pf])
        origin[:, f] = c[:, mine[f]]
        idx = [i for i in range(tree.frag_start[f], tree.frag_end[f]) if i != mine[f]]
        c[:, idx] = np.einsum("pij,pnj->pni", fused[:, f], c[:, idx]) + origin[:, f][:, None, :]
    out = np.empty_like(c)
    out[:, perm] = c
    return out


def random_poses(ligand, box_lo, box_hi, n, seed):
    """n poses: centre uniform in the box, uniform orientation, torsions U[-pi, pi),
    applied to the ligand's first pose by forward kinematics."""
    rng = np.random.default_rng(seed)
    lo, hi = np.asarray(box_lo, float), np.asarray(box_hi, float)
    centers = lo + (hi - lo) * rng.random((n, 3))
    rots = quaternion_matrix(random_quaternions(rng, n))
    T = ligand.n_torsions
    tors = rng.uniform(-math.pi, math.pi, size=(n, T))
    return apply_parameters(ligand.tree, ligand.poses[0], centers, rots, tors)


# ------------------------------------------------------------ screening ligand sets
def _screening_spec_ligand(spec):
    """One draw of screening_set: (k, heavy atoms, rotors) -> (k, ligand JSON or None)."""
    k, h, r = spec
    try:
        return k, make_ligand(seed=1000 + k, n_heavy=h, n_rot=min(r, h // 3), n_n=max(1, round(0.12 * h)),
                              n_o=max(1, round(0.15 * h)), n_other=round(0.03 * h))
    except RuntimeError:
        return k, None


def screening_set(n, seed=3, processes=None, accept=None):
    """n seeded ligands of uneven size: heavy atoms U{10..60}, rotatable bonds U{0..15},
    C 70 % / N 12 % / O 15 % / Cl 3 %. Draw k (k = 1, 2, ...) takes (heavy, rotors) from one
    seeded stream and builds ligand seed 1000 + k; a draw the generator cannot embed, or
    that accept(json) refuses, is skipped, and the first n accepted draws are returned in
    draw order. The draws are built by a process pool (started with spawn) in batches, so
    the set is the same for any number of processes."""
    import multiprocessing as mp

    rng = np.random.default_rng(seed)
    specs = [(k, int(rng.integers(10, 61)), int(rng.integers(0, 16))) for k in range(1, 20 * n + 1)]
    processes = processes or os.cpu_count() or 1
    out, pos = [], 0
    pool = mp.get_context("spawn").Pool(processes) if processes > 1 and n > 8 else None
    try:
        while len(out) < n and pos < len(specs):
            batch = specs[pos:pos + max(2 * (n - len(out)), 16)]
            pos += len(batch)
            done = (pool.map(_screening_spec_ligand, batch, chunksize=1) if pool
                    else [_screening_spec_ligand(s) for s in batch])
            for _, lj in sorted(done, key=lambda kv: kv[0]):
                if lj is not None and (accept is None or accept(lj)) and len(out) < n:
                    out.append(lj)
    finally:
        if pool:
            pool.close()
            pool.join()
    return out
