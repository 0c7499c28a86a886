// Input readers (see inputs.h). The rules restate the reference parser:
//   force-field terms            data.cpp:31-296  (fill(..., force_field_params))
//   receptor rotor leaves        data.cpp:310-364 (fill(rotable_geometry), parse)
//   ligand fragment tree         data.cpp:410-482 (fill(fragment_tree))
//   ligand vdW type offset 1000  data.cpp:234-244
//   scoring-function sections    factory.cpp:144-202, scorer.cpp:53-115
// Degrees become radians as (x / 180) * pi, the reference's MATH_TO_RADIAN (math.h:228).
#include "inputs.h"

#include <cmath>
#include <map>
#include <stdexcept>

#include "../../include/pxdock_gb300_vdw.h"

namespace pxd {

namespace {

constexpr int kVdwOffset = 1000;
constexpr double kPi = 3.141592653589793;

double radian(double deg) { return (deg / 180.0) * kPi; }

const json::Value kEmpty;

const json::Value& get(const json::Value& o, const char* key) {
    const json::Value* v = o.find(key);
    return v ? *v : kEmpty;
}

std::vector<double> doubles(const json::Value& a) {
    std::vector<double> out;
    for (auto& v : a.items) out.push_back(v.as_double());
    return out;
}

std::vector<int32_t> ints(const json::Value& a) {
    std::vector<int32_t> out;
    for (auto& v : a.items) out.push_back(static_cast<int32_t>(v.as_long()));
    return out;
}

// rows of K integers (nested arrays), flattened
template <int K>
std::vector<int32_t> rows(const json::Value& a) {
    std::vector<int32_t> out;
    for (auto& r : a.items) {
        if (static_cast<int>(r.items.size()) != K) throw std::runtime_error("index row of wrong length");
        for (auto& v : r.items) out.push_back(static_cast<int32_t>(v.as_long()));
    }
    return out;
}

// a per-atom list, zero-filled when the file leaves it empty
std::vector<double> per_atom(const json::Value& a, int n) {
    std::vector<double> v = doubles(a);
    if (static_cast<int>(v.size()) == n) return v;
    if (v.empty()) return std::vector<double>(n, 0.0);
    throw std::runtime_error("per-atom list has " + std::to_string(v.size()) + " entries for " +
                             std::to_string(n) + " atoms");
}

void dihedrals(const json::Value& ff, const std::string& prefix, std::vector<int32_t>& atoms,
               std::vector<int32_t>& per, std::vector<double>& phase, std::vector<double>& k) {
    const json::Value& ids = get(ff, (prefix + "_atomidx").c_str());
    const json::Value& pv = get(ff, (prefix + "_periodicity").c_str());
    const json::Value& kv = get(ff, (prefix + "_k").c_str());
    const json::Value& fv = get(ff, (prefix + "_phase").c_str());
    const size_t n = ids.size();
    atoms = rows<4>(ids);
    per.assign(n * 6, 0);
    phase.assign(n * 6, 0.0);
    k.assign(n * 6, 0.0);
    for (size_t d = 0; d < n; ++d) {
        for (size_t t = 0; t < pv.items[d].items.size() && t < 6; ++t)
            per[d * 6 + t] = static_cast<int32_t>(pv.items[d].items[t].as_long());
        for (size_t t = 0; t < kv.items[d].items.size() && t < 6; ++t) k[d * 6 + t] = kv.items[d].items[t].as_double();
        for (size_t t = 0; t < fv.items[d].items.size() && t < 6; ++t)
            phase[d * 6 + t] = radian(fv.items[d].items[t].as_double());
    }
}

TopologyData topology(const json::Value& ff, int n, std::vector<double> sigma, std::vector<double> eps) {
    TopologyData t;
    t.n_atoms = n;
    t.charge = per_atom(get(ff, "partial_charges"), n);
    t.sigma = std::move(sigma);
    t.epsilon = std::move(eps);
    t.bonds = rows<2>(get(ff, "FF_Bonds_atomidx"));
    t.bond_k = doubles(get(ff, "FF_Bonds_k"));
    t.bond_length = doubles(get(ff, "FF_Bonds_length"));
    t.angles = rows<3>(get(ff, "FF_Angles_atomidx"));
    t.angle_k = doubles(get(ff, "FF_Angles_k"));
    for (auto& v : get(ff, "FF_Angles_angle").items) t.angle_radian.push_back(radian(v.as_double()));
    dihedrals(ff, "FF_ImproperTorsions", t.imp_atoms, t.imp_per, t.imp_phase, t.imp_k);
    dihedrals(ff, "FF_ProperTorsions", t.prop_atoms, t.prop_per, t.prop_phase, t.prop_k);
    t.pairs14 = rows<2>(get(ff, "FF_Nonbonded14_atomidx"));
    t.pairs = rows<2>(get(ff, "FF_NonbondedAll_atomidx"));
    if (t.bond_k.size() * 2 != t.bonds.size() || t.angle_k.size() * 3 != t.angles.size())
        throw std::runtime_error("force-field term lists of different lengths");
    return t;
}

ScoreListData score_lists(const json::Value& ff, int n, bool ligand) {
    ScoreListData s;
    s.hydrophobic = ints(get(ff, "hydrophobic_atomidx"));
    s.cation = ints(get(ff, "cation_atomidx"));
    s.anion = ints(get(ff, "anion_atomidx"));
    auto rings = [&](const char* key) {
        std::vector<int32_t> out;
        for (auto& r : get(ff, key).items) {
            std::vector<int32_t> row(6, -1);
            for (size_t k = 0; k < r.items.size() && k < 6; ++k) row[k] = static_cast<int32_t>(r.items[k].as_long());
            out.insert(out.end(), row.begin(), row.end());
        }
        return out;
    };
    s.ring5 = rings("piring5_atomidx");
    s.ring6 = rings("piring6_atomidx");
    s.don_c = rows<2>(get(ff, "hbonddon_charged_atomidx"));
    s.don_n = rows<2>(get(ff, "hbonddon_neut_atomidx"));
    s.acc_c = ints(get(ff, "hbondacc_charged_atomidx"));
    s.acc_n = ints(get(ff, "hbondacc_neut_atomidx"));
    s.ts_offsets.push_back(0);
    if (ligand) {
        const json::Value& idx = get(ff, "tstrain_atomidx_pose_selection");
        const json::Value& prm = get(ff, "tstrain_params_pose_selection");
        for (size_t e = 0; e < idx.size() && e < prm.size(); ++e) {
            for (auto& v : prm.items[e].items) s.ts_coefs.push_back(v.as_double());
            for (auto& q : idx.items[e].items)
                for (auto& v : q.items) s.ts_quads.push_back(static_cast<int32_t>(v.as_long()));
            s.ts_offsets.push_back(static_cast<int32_t>(s.ts_quads.size() / 4));
        }
        s.n_rotatable = static_cast<int>(get(ff, "rotatable_bond_index").size());
    }
    std::vector<int32_t> an = ints(get(ff, "atomic_numbers"));
    s.atomic_numbers = static_cast<int>(an.size()) == n ? an : std::vector<int32_t>(n, 0);
    s.all_bonds = rows<2>(get(ff, "bond_index"));
    return s;
}

template <class T>
const T* ptr(const std::vector<T>& v) {
    return v.empty() ? nullptr : v.data();
}

}  // namespace

pxd_topology TopologyData::desc() const {
    pxd_topology t{};
    t.n_atoms = n_atoms;
    t.charge = ptr(charge);
    t.sigma = ptr(sigma);
    t.epsilon = ptr(epsilon);
    t.n_bonds = static_cast<int32_t>(bonds.size() / 2);
    t.bond_atoms = ptr(bonds);
    t.bond_k = ptr(bond_k);
    t.bond_length = ptr(bond_length);
    t.n_angles = static_cast<int32_t>(angles.size() / 3);
    t.angle_atoms = ptr(angles);
    t.angle_k = ptr(angle_k);
    t.angle_radian = ptr(angle_radian);
    t.n_impropers = static_cast<int32_t>(imp_atoms.size() / 4);
    t.improper_atoms = ptr(imp_atoms);
    t.improper_periodicity = ptr(imp_per);
    t.improper_phase = ptr(imp_phase);
    t.improper_k = ptr(imp_k);
    t.n_propers = static_cast<int32_t>(prop_atoms.size() / 4);
    t.proper_atoms = ptr(prop_atoms);
    t.proper_periodicity = ptr(prop_per);
    t.proper_phase = ptr(prop_phase);
    t.proper_k = ptr(prop_k);
    t.n_pairs14 = static_cast<int32_t>(pairs14.size() / 2);
    t.pairs14 = ptr(pairs14);
    t.n_pairs = static_cast<int32_t>(pairs.size() / 2);
    t.pairs = ptr(pairs);
    return t;
}

pxd_score_lists ScoreListData::desc() const {
    pxd_score_lists s{};
    s.n_hydrophobic = static_cast<int32_t>(hydrophobic.size());
    s.hydrophobic = ptr(hydrophobic);
    s.n_cation = static_cast<int32_t>(cation.size());
    s.cation = ptr(cation);
    s.n_anion = static_cast<int32_t>(anion.size());
    s.anion = ptr(anion);
    s.n_ring5 = static_cast<int32_t>(ring5.size() / 6);
    s.ring5 = ptr(ring5);
    s.n_ring6 = static_cast<int32_t>(ring6.size() / 6);
    s.ring6 = ptr(ring6);
    s.n_don_charged = static_cast<int32_t>(don_c.size() / 2);
    s.don_charged = ptr(don_c);
    s.n_don_neutral = static_cast<int32_t>(don_n.size() / 2);
    s.don_neutral = ptr(don_n);
    s.n_acc_charged = static_cast<int32_t>(acc_c.size());
    s.acc_charged = ptr(acc_c);
    s.n_acc_neutral = static_cast<int32_t>(acc_n.size());
    s.acc_neutral = ptr(acc_n);
    s.n_tstrain = static_cast<int32_t>(ts_coefs.size() / 4);
    s.tstrain_coefs = ptr(ts_coefs);
    s.tstrain_offsets = ptr(ts_offsets);
    s.tstrain_quads = ptr(ts_quads);
    s.n_rotatable = n_rotatable;
    s.atomic_numbers = ptr(atomic_numbers);
    s.n_all_bonds = static_cast<int32_t>(all_bonds.size() / 2);
    s.all_bonds = ptr(all_bonds);
    return s;
}

pxd_receptor_desc ReceptorData::desc() {
    lists_c = lists.desc();
    pxd_receptor_desc r{};
    r.n_atoms = n_atoms;
    r.xyz = ptr(xyz);
    r.ff = ff.desc();
    r.n_rotors = static_cast<int32_t>(rotor_axis.size() / 2);
    r.rotor_axis = ptr(rotor_axis);
    r.rotor_offsets = ptr(rotor_offsets);
    r.rotor_atoms = ptr(rotor_atoms);
    r.lists = &lists_c;
    return r;
}

pxd_ligand_desc LigandData::desc() {
    lists_c = lists.desc();
    pxd_ligand_desc l{};
    l.ff = ff.desc();
    l.vdw_type = ptr(vdw_type);
    if (has_tree) {
        l.tree.n_frags = static_cast<int32_t>(frag_start.size());
        l.tree.frag_start = ptr(frag_start);
        l.tree.frag_end = ptr(frag_end);
        l.tree.perm = ptr(perm);
        l.tree.n_roots = static_cast<int32_t>(roots.size());
        l.tree.roots = ptr(roots);
        l.tree.n_torsions = static_cast<int32_t>(tors_frag.size());
        l.tree.tors_frag = ptr(tors_frag);
        l.tree.tors_parent = ptr(tors_parent);
        l.tree.tors_parent_atom = ptr(tors_parent_atom);
        l.tree.tors_mine_atom = ptr(tors_mine_atom);
    }
    l.lists = &lists_c;
    return l;
}

ReceptorData read_receptor(const json::Value& d) {
    const json::Value& geo = d.at("geometry");
    const json::Value& ff = d.at("ffdata");
    const json::Value& xyz = d.at("xyz");
    ReceptorData r;
    r.n_atoms = static_cast<int>(xyz.size());
    const long wanted = geo.at("num_atoms").as_long();
    if (wanted != r.n_atoms)
        throw std::runtime_error("Atom count mismatches! Wanted [" + std::to_string(wanted) + "] vs. Parsed [" +
                                 std::to_string(r.n_atoms) + "]");
    for (auto& a : xyz.items)
        for (auto& c : a.items) r.xyz.push_back(c.as_double());
    if (r.xyz.size() != 3 * static_cast<size_t>(r.n_atoms)) throw std::runtime_error("receptor xyz rows of wrong length");
    std::vector<int> order;
    r.rotor_offsets.push_back(0);
    for (auto& kv : get(geo, "data").fields) {  // JSON key order, as data.cpp:314-336 walks it
        const json::Value& b = kv.second;
        std::vector<int32_t> a0 = ints(b.at("rot_bond_1")), a1 = ints(b.at("rot_bond_2"));
        for (size_t i = 0; i < a0.size() && i < a1.size(); ++i) {
            r.rotor_axis.push_back(a0[i]);
            r.rotor_axis.push_back(a1[i]);
        }
        for (auto& frag : b.at("fragments").items) {
            for (auto& v : frag.items) r.rotor_atoms.push_back(static_cast<int32_t>(v.as_long()));
            r.rotor_offsets.push_back(static_cast<int32_t>(r.rotor_atoms.size()));
        }
        for (auto& v : get(b, "rot_bond_order").items) order.push_back(static_cast<int>(v.as_long()));
    }
    const size_t n_rot = r.rotor_axis.size() / 2;
    if (r.rotor_offsets.size() != n_rot + 1) throw std::runtime_error("rotor axes and fragments differ in number");
    r.bond_mappings.resize(n_rot);
    for (size_t k = 0; k < n_rot; ++k) r.bond_mappings[k] = order.size() == n_rot ? order[k] : static_cast<int>(k);
    r.num_rotatable_bonds = static_cast<int>(get(geo, "num_rotatable_bonds").is_null()
                                                 ? 0
                                                 : get(geo, "num_rotatable_bonds").as_long());
    for (int m : r.bond_mappings) r.num_rotatable_bonds = std::max(r.num_rotatable_bonds, m + 1);
    r.ff = topology(ff, r.n_atoms, per_atom(get(ff, "FF_vdW_sigma"), r.n_atoms),
                    per_atom(get(ff, "FF_vdW_epsilon"), r.n_atoms));
    r.lists = score_lists(ff, r.n_atoms, false);
    return r;
}

LigandData read_ligand(const json::Value& d, bool geometry) {
    const json::Value& ff = d.at("ffdata");
    LigandData l;
    const json::Value& xyz = d.at("xyz");
    for (auto& v : get(ff, "FF_vdW_paraidx").items) {
        const long t = v.as_long() - kVdwOffset;
        if (t > 98 || t < 0)
            throw std::runtime_error("VDW type [" + std::to_string(t) + "] of atom#" + std::to_string(l.vdw_type.size()) +
                                     "is illegal!");
        l.vdw_type.push_back(static_cast<int32_t>(t));
    }
    int n = static_cast<int>(l.vdw_type.size());
    if (n == 0 && xyz.size() > 0) {  // kinematics-only files carry coordinates but no force field
        n = static_cast<int>(xyz.items[0].size());
        l.vdw_type.assign(n, 0);
    }
    std::vector<double> sig(n), eps(n);
    for (int a = 0; a < n; ++a) {
        sig[a] = PXD_VDW_SIGMA[l.vdw_type[a]];
        eps[a] = PXD_VDW_EPSILON[l.vdw_type[a]];
    }
    l.ff = topology(ff, n, sig, eps);
    for (auto& pose : xyz.items) {
        std::vector<double> p;
        for (auto& a : pose.items)
            for (auto& c : a.items) p.push_back(c.as_double());
        if (p.size() != 3 * static_cast<size_t>(n)) throw std::runtime_error("ligand pose of wrong size");
        l.poses.push_back(std::move(p));
    }
    if (const json::Value* s = d.find("mapped_smiles")) l.smiles = s->kind == json::Value::String ? s->str : "";
    l.lists = score_lists(ff, n, true);
    if (geometry && d.has("geometry")) {
        const json::Value& geo = d.at("geometry");
        const int na = static_cast<int>(geo.at("num_atoms").as_long());
        std::vector<int32_t> split = ints(geo.at("frag_split_index"));
        const int F = static_cast<int>(split.size()) + 1;
        std::map<int, std::vector<int>> children;
        for (auto& level : geo.at("frag_traverse_levels").items)
            for (auto& kv : level.fields) {
                const int f = std::stoi(kv.first);
                if (kv.second.at("parent").size() == 0) l.roots.push_back(f);
                std::vector<int> ch;
                for (auto& c : kv.second.at("children").items) ch.push_back(static_cast<int>(c.as_long()));
                children[f] = ch;
            }
        std::vector<int32_t> bounds;
        bounds.push_back(0);
        bounds.insert(bounds.end(), split.begin(), split.end());
        bounds.push_back(na);
        for (int f = 0; f < F; ++f) {
            l.frag_start.push_back(bounds[f]);
            l.frag_end.push_back(bounds[f + 1]);
        }
        l.perm = ints(geo.at("permute_index"));
        std::vector<int> rev(l.perm.size(), 0);
        for (size_t p = 0; p < l.perm.size(); ++p) {
            if (l.perm[p] < 0 || l.perm[p] >= static_cast<int>(rev.size())) throw std::runtime_error("bad permute_index");
            rev[l.perm[p]] = static_cast<int>(p);
        }
        std::map<std::string, std::pair<int, int>> bonds;
        for (auto& kv : geo.at("edge_to_bond").fields)
            bonds[kv.first] = {rev.at(kv.second.items.at(0).as_long()), rev.at(kv.second.items.at(1).as_long())};
        // pre-order walk, children in listed order (data.cpp:562-590)
        std::vector<int> stack(l.roots.rbegin(), l.roots.rend());
        std::vector<std::pair<int, int>> work;  // (node, next child index)
        for (int root : l.roots) {
            work.assign(1, {root, 0});
            while (!work.empty()) {
                auto& top = work.back();
                const auto& ch = children[top.first];
                if (top.second >= static_cast<int>(ch.size())) {
                    work.pop_back();
                    continue;
                }
                const int node = top.first, c = ch[top.second++];
                auto it = bonds.find(std::to_string(node) + "->" + std::to_string(c));
                if (it == bonds.end()) throw std::runtime_error("fragment edge without a bond");
                l.tors_frag.push_back(c);
                l.tors_parent.push_back(node);
                l.tors_parent_atom.push_back(it->second.first);
                l.tors_mine_atom.push_back(it->second.second);
                work.push_back({c, 0});
            }
        }
        l.has_tree = true;
    }
    return l;
}

namespace {

bool active(double x) { return x > 1e-5 || x < -1e-5; }  // CHECK_PARAMETER_NON_ZERO, utility.h:26

pxd_sf_params sf_section(const json::Value& node) {
    pxd_sf_params p{};
    static const char* keys[PXD_NUM_TERMS] = {
        "interaction_coulomb_energy_coef", "interaction_vdw_energy_coef", "ionic_energy_coef",
        "pi_cationic_energy_coef", "f2f_pi_stacking_energy_coef", "e2f_pi_stacking_energy_coef",
        "hbond_energy_coef", "hydrophobic_energy_coef", "torsion_strain_penalty_coef", "rotatable_energy_coef",
        "gbsa_energy_delta_coef"};
    double raw[PXD_NUM_TERMS], eff[PXD_NUM_TERMS];
    for (int k = 0; k < PXD_NUM_TERMS; ++k) {
        const json::Value& v = get(node, keys[k]);
        raw[k] = v.is_null() ? 0.0 : v.as_double();
        eff[k] = raw[k];
    }
    // the reference registers the rotatable weight under the torsion-strain name
    // (scorer.cpp:103-106): a non-zero rotatable weight replaces the torsion-strain
    // weight and the rotatable term itself is never summed
    eff[9] = 0.0;
    if (active(raw[9])) eff[8] = active(raw[8]) ? raw[9] : 0.0;
    for (int k = 0; k < PXD_NUM_TERMS; ++k) p.coef[k] = (active(raw[k]) || k == 8) ? eff[k] : 0.0;
    if (active(raw[1])) {
        const json::Value& v = node.at("interaction_vdw_energy");
        p.vdw_scale = v.at("scale").as_double();
        p.vdw_cutoff = v.at("cutoff").as_double();
        // types beyond the file's list keep the neutral scale 1 (the reference reads past
        // its list there)
        for (int t = 0; t < PXD_NUM_VDW_TYPES; ++t) p.vdw_sigma_scale[t] = p.vdw_epsilon_scale[t] = 1.0;
        const json::Value& types = v.at("types");
        for (size_t t = 0; t < types.size() && t < PXD_NUM_VDW_TYPES; ++t) {
            p.vdw_sigma_scale[t] = types.items[t].at("sigma_scale").as_double();
            p.vdw_epsilon_scale[t] = types.items[t].at("epsilon_scale").as_double();
        }
    }
    if (active(raw[2])) {
        const json::Value& v = node.at("ionic_energy");
        p.ionic_coef[0] = v.at("lc_coef").as_double();
        p.ionic_coef[1] = v.at("pc_coef").as_double();
        const char* names[2] = {"lc_inter", "pc_inter"};
        for (int k = 0; k < 2; ++k) {
            p.ionic[k][0] = v.at(names[k]).at("dist_min").as_double();
            p.ionic[k][1] = v.at(names[k]).at("dist_max").as_double();
        }
    }
    if (active(raw[3])) {
        const json::Value& v = node.at("pi_cationic_energy");
        const char* names[4] = {"lc5", "lc6", "pc5", "pc6"};
        for (int k = 0; k < 4; ++k) {
            const std::string n = names[k];
            p.picat_coef[k] = v.at(n + "_coef").as_double();
            p.picat[k][0] = v.at(n + "_inter").at("dist_min").as_double();
            p.picat[k][1] = v.at(n + "_inter").at("dist_max").as_double();
        }
    }
    const char* stack_keys[2] = {"f2f_pi_stacking_energy", "e2f_pi_stacking_energy"};
    for (int w = 0; w < 2; ++w) {
        if (!active(raw[4 + w])) continue;
        const json::Value& v = node.at(stack_keys[w]);
        const char* names[4] = {"l5r5", "l5r6", "l6r5", "l6r6"};
        const char* fields[6] = {"dist_min", "dist_max", "angle_min", "angle_max", "sigma_min", "sigma_max"};
        for (int k = 0; k < 4; ++k) {
            const std::string n = names[k];
            p.stack_coef[w][k] = v.at(n + "_coef").as_double();
            for (int u = 0; u < 6; ++u) p.stack[w][k][u] = v.at(n + "_inter").at(fields[u]).as_double();
        }
    }
    if (active(raw[6])) {
        const json::Value& v = node.at("hbond_energy");
        p.hbond_scale = v.at("scale").as_double();
        const char* names[8] = {"hldcc", "hldcn", "hldnc", "hldnn", "hpdcc", "hpdcn", "hpdnc", "hpdnn"};
        const char* fields[6] = {"dist_min", "dist_max", "angle_min", "angle_max", "dist_center", "angle_center"};
        for (int k = 0; k < 8; ++k) {
            const std::string n = names[k];
            p.hbond_coef[k] = v.at(n + "_coef").as_double();
            for (int u = 0; u < 6; ++u) p.hbond[k][u] = v.at(n + "_inter").at(fields[u]).as_double();
        }
    }
    if (active(raw[7])) {
        const json::Value& v = node.at("hydrophobic_energy");
        p.hydro_scale = v.at("scale").as_double();
        p.hydro_dist_min = v.at("dist_min").as_double();
        p.hydro_dist_max = v.at("dist_max").as_double();
        p.hydro_scale_factor = v.at("scale_factor").as_double();
    }
    if (!active(raw[8])) p.coef[8] = 0.0;
    return p;
}

}  // namespace

std::array<pxd_sf_params, 2> read_scoring_function(const json::Value& doc) {
    return {sf_section(doc.at("pose_selection")), sf_section(doc.at("affinity_ranking"))};
}

}  // namespace pxd
