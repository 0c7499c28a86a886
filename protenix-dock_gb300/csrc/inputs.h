// Readers of the engine's input files: receptor JSON, ligand JSON and the scoring-function
// JSON, restating the reference parser (engine/src/core/data.cpp, factory.cpp). Each
// parsed object owns its arrays and hands out the C ABI descriptors that point into
// them. Host code only.
#ifndef PXD_INPUTS_H_
#define PXD_INPUTS_H_

#include <array>
#include <string>
#include <vector>

#include "../../include/pxdock_gb300.h"
#include "json.h"

namespace pxd {

// force_field_params (system.h:85-109) of one molecule
struct TopologyData {
    int n_atoms = 0;
    std::vector<double> charge, sigma, epsilon;
    std::vector<int32_t> bonds, angles;
    std::vector<double> bond_k, bond_length, angle_k, angle_radian;
    std::vector<int32_t> imp_atoms, imp_per, prop_atoms, prop_per;
    std::vector<double> imp_phase, imp_k, prop_phase, prop_k;
    std::vector<int32_t> pairs14, pairs;
    pxd_topology desc() const;
};

// the pscore / bscore atom lists of one molecule (data.cpp:201-295)
struct ScoreListData {
    std::vector<int32_t> hydrophobic, cation, anion, ring5, ring6, don_c, don_n, acc_c, acc_n;
    std::vector<double> ts_coefs;
    std::vector<int32_t> ts_offsets, ts_quads, atomic_numbers, all_bonds;
    int n_rotatable = 0;
    pxd_score_lists desc() const;
};

struct ReceptorData {
    int n_atoms = 0;
    std::vector<double> xyz;
    TopologyData ff;
    std::vector<int32_t> rotor_axis, rotor_offsets, rotor_atoms;
    std::vector<int> bond_mappings;  // leaf -> position among the rotatable bonds
    int num_rotatable_bonds = 0;
    ScoreListData lists;
    pxd_score_lists lists_c{};
    pxd_receptor_desc desc();
};

struct LigandData {
    TopologyData ff;
    std::vector<int32_t> vdw_type;
    // fragment tree (data.cpp:410-482)
    std::vector<int32_t> frag_start, frag_end, perm, roots, tors_frag, tors_parent, tors_parent_atom,
        tors_mine_atom;
    bool has_tree = false;
    std::vector<std::vector<double>> poses;  // [n_poses][n_atoms * 3]
    std::string smiles;
    ScoreListData lists;
    pxd_score_lists lists_c{};
    int n_atoms() const { return ff.n_atoms; }
    int n_torsions() const { return static_cast<int>(tors_frag.size()); }
    pxd_ligand_desc desc();
};

// throw std::runtime_error with the reference's messages where it has one
ReceptorData read_receptor(const json::Value& doc);
LigandData read_ligand(const json::Value& doc, bool geometry);
// (pose_selection, affinity_ranking)
std::array<pxd_sf_params, 2> read_scoring_function(const json::Value& doc);

}  // namespace pxd

#endif  // PXD_INPUTS_H_
