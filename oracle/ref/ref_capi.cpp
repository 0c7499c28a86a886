// Test infrastructure (oracle): a C-ABI wrapper over the reference engine's own
// classes, compiled together with the reference sources in place
// (engine/src/{lib,core,ext}) into oracle/_ref/liboracle_ref.so. It is a checker
// only: the parity tests and the golden-fixture script call it to obtain the
// reference engine's FP64 answers. Nothing in the product links or loads it.
//
// Wrapped reference entry points (engine/ paths):
//   binding_system_interactions::put_gradients   src/core/interaction.cpp:271-298
//   receptor_cache::{populate,get}               src/core/grid.cpp:115-262
//   lbfgs_step::apply                            src/core/optimizer.cpp:429-560
//   free_ligand / torsional_receptor kinematics  src/core/data.cpp:366-385, 592-641
//   root_scorer::combine / summary               include/bytedock/core/scorer.h:92-136
//   monte_carlo_searcher::fill                   src/core/searcher.cpp:30-44
//   random_generator                             include/bytedock/lib/random.h:33-63
//   ReusableEngine                               src/core/entrance.cpp:68-436
#include <cstring>
#include <memory>
#include <string>
#include <vector>

// Map arrays of receptor_cache are private in the reference; the checker reads them
// directly to compare map records point by point.
#define private public
#include "bytedock/core/grid.h"
#undef private
#include "bytedock/core/constant.h"
#include "bytedock/core/entrance.h"
#include "bytedock/core/factory.h"
#include "bytedock/core/interaction.h"
#include "bytedock/core/optimizer.h"
#include "bytedock/core/scorer.h"
#include "bytedock/core/searcher.h"
#include "bytedock/ext/pfile.h"
#include "bytedock/lib/math.h"
#include "bytedock/lib/random.h"
#include "bytedock/version.h"

using namespace bytedock;

namespace {

struct ref_system {
    std::shared_ptr<torsional_receptor> receptor;
    std::shared_ptr<free_ligand> ligand;
    std::shared_ptr<receptor_cache> cache;
    std::unique_ptr<scoring_function_factory> sf;
    box_config bc;
    bool has_box = false;
};

thread_local std::string g_error;

molecule_pose to_pose(const double* xyz, size_t n) {
    molecule_pose p(n);
    for (size_t i = 0; i < n; ++i) {
        p[i].xyz[0] = xyz[3 * i];
        p[i].xyz[1] = xyz[3 * i + 1];
        p[i].xyz[2] = xyz[3 * i + 2];
    }
    return p;
}

void from_pose(const molecule_pose& p, double* xyz) {
    for (size_t i = 0; i < p.size(); ++i) {
        xyz[3 * i] = p[i].xyz[0];
        xyz[3 * i + 1] = p[i].xyz[1];
        xyz[3 * i + 2] = p[i].xyz[2];
    }
}

force_field_params to_ff(int n_atoms, const double* charge, const double* sigma,
                         const double* epsilon, int nb, const int* bij, const double* bk,
                         const double* br0, int na, const int* aijk, const double* ak,
                         const double* at0, int ni, const int* iijkl, const int* iper,
                         const double* iphase, const double* ik, int np, const int* pijkl,
                         const int* pper, const double* pphase, const double* pk, int n14,
                         const int* p14, int nall, const int* pall) {
    force_field_params ff;
    ff.partial_charges.assign(charge, charge + n_atoms);
    ff.vdw_params.resize(n_atoms);
    for (int i = 0; i < n_atoms; ++i) {
        ff.vdw_params[i].sigma = sigma[i];
        ff.vdw_params[i].epsilon = epsilon[i];
    }
    ff.bonds.resize(nb);
    for (int i = 0; i < nb; ++i) {
        ff.bonds[i].ids[0] = bij[2 * i];
        ff.bonds[i].ids[1] = bij[2 * i + 1];
        ff.bonds[i].k = bk[i];
        ff.bonds[i].length = br0[i];
    }
    ff.angles.resize(na);
    for (int i = 0; i < na; ++i) {
        for (int d = 0; d < 3; ++d) ff.angles[i].ids[d] = aijk[3 * i + d];
        ff.angles[i].k = ak[i];
        ff.angles[i].radian = at0[i];
    }
    auto fill_dih = [](std::vector<fourier_dihedral>& dst, int n, const int* ijkl,
                       const int* per, const double* phase, const double* k) {
        dst.resize(n);
        for (int i = 0; i < n; ++i) {
            for (int d = 0; d < 4; ++d) dst[i].ids[d] = ijkl[4 * i + d];
            for (int d = 0; d < FF_DIHEDRAL_NDIMS; ++d) {
                dst[i].periodicity[d] = per[6 * i + d];
                dst[i].phase[d] = phase[6 * i + d];
                dst[i].k[d] = k[6 * i + d];
            }
        }
    };
    fill_dih(ff.impropers, ni, iijkl, iper, iphase, ik);
    fill_dih(ff.propers, np, pijkl, pper, pphase, pk);
    ff.pairs.resize(n14);
    for (int i = 0; i < n14; ++i) {
        ff.pairs[i].ids[0] = p14[2 * i];
        ff.pairs[i].ids[1] = p14[2 * i + 1];
    }
    ff.others.resize(nall);
    for (int i = 0; i < nall; ++i) {
        ff.others[i].ids[0] = pall[2 * i];
        ff.others[i].ids[1] = pall[2 * i + 1];
    }
    return ff;
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_error.c_str(); }

const char* ref_version() { return VERSION_STR; }

// ---------------------------------------------------------------- math (math.cpp)
double ref_dihedral_and_gradient(const double* i, const double* j, const double* k,
                                 const double* l, double* gi, double* gj, double* gk,
                                 double* gl) {
    return get_dihedral_angle_and_gradient_3d(i, j, k, l, gi, gj, gk, gl);
}

double ref_dihedral(const double* i, const double* j, const double* k, const double* l) {
    return get_dihedral_angle_3d(i, j, k, l);
}

double ref_angle_and_gradient(const double* i, const double* j, const double* k,
                              double* gi, double* gk) {
    return get_angle_and_gradient_3d(i, j, k, gi, gk);
}

void ref_rotation_axis_angle(const double* axis, double theta, double* rot9, double* jac9) {
    vector_3d ax = {{axis[0], axis[1], axis[2]}};
    matrix_3x3 r, j;
    get_rotation_matrix_and_gradient(ax, theta, r, j);
    std::memcpy(rot9, r.data, sizeof(r.data));
    std::memcpy(jac9, j.data, sizeof(j.data));
}

void ref_rotation_quaternion(const double* q, double* rot9) {
    vector_4d qt = {{q[0], q[1], q[2], q[3]}};
    matrix_3x3 r;
    get_rotation_matrix(qt, r);
    std::memcpy(rot9, r.data, sizeof(r.data));
}

// ------------------------------------------------- intra terms on flat FF arrays
// which: 0 bonds, 1 angles, 2 dihedrals, 3 nonbonded (1-4 + all), 4 total intra.
double ref_intra_energy(int which, int n_atoms, const double* xyz, const double* charge,
                        const double* sigma, const double* epsilon, int nb, const int* bij,
                        const double* bk, const double* br0, int na, const int* aijk,
                        const double* ak, const double* at0, int ni, const int* iijkl,
                        const int* iper, const double* iphase, const double* ik, int np,
                        const int* pijkl, const int* pper, const double* pphase,
                        const double* pk, int n14, const int* p14, int nall, const int* pall,
                        double* grad) {
    auto ff = to_ff(n_atoms, charge, sigma, epsilon, nb, bij, bk, br0, na, aijk, ak, at0, ni,
                    iijkl, iper, iphase, ik, np, pijkl, pper, pphase, pk, n14, p14, nall, pall);
    auto pose = to_pose(xyz, n_atoms);
    molecule_pose g(n_atoms, {{0., 0., 0.}});
    double e = 0.;
    switch (which) {
        case 0: { harmonic_bond_interaction t; e = t.put_gradients(pose, ff, g); break; }
        case 1: { harmonic_angle_interaction t; e = t.put_gradients(pose, ff, g); break; }
        case 2: { fourier_dihedral_interaction t; e = t.put_gradients(pose, ff, g); break; }
        case 3: { self_nonbonded_interactions t; e = t.put_gradients(pose, ff, g); break; }
        default: { intra_molecular_interactions t; e = t.put_gradients(pose, ff, g); break; }
    }
    from_pose(g, grad);
    return e;
}

// ------------------------------------------------------------ systems from JSON
void* ref_system_create(const char* receptor_json, const char* ligand_json) {
    try {
        auto* s = new ref_system;
        s->receptor = std::make_shared<torsional_receptor>();
        s->receptor->parse(open_for_read(receptor_json));
        s->ligand = std::make_shared<free_ligand>();
        s->ligand->parse(open_for_read(ligand_json));
        return s;
    } catch (std::exception& e) {
        g_error = e.what();
        return nullptr;
    }
}

void ref_system_destroy(void* h) { delete static_cast<ref_system*>(h); }

void ref_system_counts(void* h, int* out) {
    auto* s = static_cast<ref_system*>(h);
    out[0] = static_cast<int>(s->ligand->get_ffdata().vdw_types.size());
    out[1] = static_cast<int>(s->receptor->get_positions().size());
    out[2] = static_cast<int>(s->receptor->num_torsions());
    out[3] = static_cast<int>(s->ligand->num_torsions());
    out[4] = static_cast<int>(s->ligand->get_nposes());
    out[5] = static_cast<int>(s->receptor->num_movable_atoms());
}

void ref_system_get_pose(void* h, int pose_id, double* xyz) {
    from_pose(static_cast<ref_system*>(h)->ligand->get_pose(pose_id), xyz);
}

int ref_system_build_grid(void* h, double cx, double cy, double cz, double sx, double sy,
                          double sz, double spacing, int nthreads, int* npoints) {
    auto* s = static_cast<ref_system*>(h);
    s->bc = decide_grid_dims(cx, cy, cz, sx, sy, sz, spacing);
    s->has_box = true;
    s->cache = std::make_shared<receptor_cache>(s->bc);
    s->cache->populate(*s->receptor, nthreads);
    for (int d = 0; d < 3; ++d) npoints[d] = static_cast<int>(s->bc.npoints[d]);
    return 0;
}

void ref_system_grid_info(void* h, double* init_xyz, int* npoints, double* spacing) {
    auto* s = static_cast<ref_system*>(h);
    for (int d = 0; d < 3; ++d) {
        init_xyz[d] = s->bc.init_xyz[d];
        npoints[d] = static_cast<int>(s->bc.npoints[d]);
    }
    *spacing = s->bc.spacing;
}

// map 0..98: vdW map of that ligand type; 99: Coulomb map. out: [P][4] = E, dE/dx,y,z
void ref_system_grid_copy(void* h, int map, double* out) {
    auto* s = static_cast<ref_system*>(h);
    const auto& g = map == static_cast<int>(kNumVdwTypes) ? s->cache->coul_grid_
                                                          : s->cache->vdw_grids_[map];
    for (size_t p = 0; p < g.size(); ++p) {
        out[4 * p] = g[p].first;
        out[4 * p + 1] = g[p].second.xyz[0];
        out[4 * p + 2] = g[p].second.xyz[1];
        out[4 * p + 3] = g[p].second.xyz[2];
    }
}

void ref_system_set_slope(void* h, double slope) {
    auto* s = static_cast<ref_system*>(h);
    if (s->cache) s->cache->set_slope(slope);
}

void ref_system_drop_grid(void* h) { static_cast<ref_system*>(h)->cache.reset(); }

int ref_system_grid_get(void* h, int type, double q, const double* xyz, double* energy,
                        double* grad) {
    auto* s = static_cast<ref_system*>(h);
    atom_position p = {{xyz[0], xyz[1], xyz[2]}};
    atom_position g = {{grad[0], grad[1], grad[2]}};
    double e = *energy;
    bool hit = s->cache->get(type, q, p, e, g);
    *energy = e;
    grad[0] = g.xyz[0];
    grad[1] = g.xyz[1];
    grad[2] = g.xyz[2];
    return hit ? 1 : 0;
}

double ref_system_score_grad(void* h, const double* torsions, const double* lig_xyz,
                             double* tgrad, double* lgrad) {
    auto* s = static_cast<ref_system*>(h);
    binding_system_interactions model(s->receptor, s->ligand, s->cache);
    std::vector<param_t> tg;
    molecule_pose lg;
    model.init_gradients(tg, lg);
    std::vector<param_t> t(torsions, torsions + s->receptor->num_torsions());
    auto x = to_pose(lig_xyz, lg.size());
    double e = model.put_gradients(t, x, tg, lg);
    for (size_t i = 0; i < tg.size(); ++i) tgrad[i] = tg[i];
    from_pose(lg, lgrad);
    return e;
}

int ref_system_lbfgs(void* h, int max_iter, int max_eval, double* torsions, double* lig_xyz,
                     double* energy, int* nevals) {
    auto* s = static_cast<ref_system*>(h);
    binding_system_interactions model(s->receptor, s->ligand, s->cache);
    optimized_result out;
    size_t n = s->ligand->get_ffdata().vdw_types.size();
    out.ligand_xyz = to_pose(lig_xyz, n);
    out.torsions.assign(torsions, torsions + s->receptor->num_torsions());
    lbfgs_step step(max_iter, max_eval);
    bool converged = step.apply(model, out);
    from_pose(out.ligand_xyz, lig_xyz);
    for (size_t i = 0; i < out.torsions.size(); ++i) torsions[i] = out.torsions[i];
    *energy = out.energy;
    *nevals = static_cast<int>(out.nevals);
    return converged ? 1 : 0;
}

void ref_system_ligand_apply(void* h, const double* xyz, const double* center,
                             const double* rot9, const double* torsions, double* out) {
    auto* s = static_cast<ref_system*>(h);
    size_t n = s->ligand->get_ffdata().vdw_types.size();
    if (n == 0) n = s->ligand->get_pose(0).size();
    auto pose = to_pose(xyz, n);
    atom_position c = {{center[0], center[1], center[2]}};
    matrix_3x3 r;
    std::memcpy(r.data, rot9, sizeof(r.data));
    std::vector<param_t> t(torsions, torsions + s->ligand->num_torsions());
    from_pose(s->ligand->apply_parameters(pose, c, r, t), out);
}

void ref_system_receptor_apply(void* h, const double* torsions, double* out) {
    auto* s = static_cast<ref_system*>(h);
    std::vector<param_t> t(torsions, torsions + s->receptor->num_torsions());
    from_pose(s->receptor->apply_parameters(t), out);
}

int ref_system_load_sf(void* h, const char* sf_json) {
    try {
        static_cast<ref_system*>(h)->sf.reset(new scoring_function_factory(sf_json));
        return 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

// Term names in the order the checker reports them.
static const char* kTermNames[] = {
    "InteractionCoulomb_oriEnergy", "InteractionVDW_Energy", "Ionic_Energy",
    "Pi_Cationic_Energy", "F2FPiStacking_Energy", "E2FPiStacking_Energy", "Hbond_Energy",
    "Hydrophobic_Energy", "TorsionStrain_Penalty", "rotatable_energy",
    "Gbsa_Com_Energy-Gbsa_Lig_Energy-Gbsa_Pro_Energy"};
static const int kNumTerms = 11;

// which: 0 pose-selection (pscore), 1 affinity (bscore). terms[11] gets each leaf value
// (0 where the term is inactive). Returns the combined score.
double ref_system_score(void* h, int which, const double* rec_xyz, const double* lig_xyz,
                        double* terms) {
    auto* s = static_cast<ref_system*>(h);
    const root_scorer& sc =
        which == 0 ? s->sf->get_pose_selection() : s->sf->get_affinity_ranking();
    auto r = to_pose(rec_xyz, s->receptor->get_positions().size());
    auto l = to_pose(lig_xyz, s->ligand->get_ffdata().vdw_types.size());
    auto memo = sc.precalculate(r, s->receptor->get_ffdata(), l, s->ligand->get_ffdata());
    auto scores = sc.summary(r, s->receptor->get_ffdata(), l, s->ligand->get_ffdata(), &memo);
    for (int i = 0; i < kNumTerms; ++i) {
        auto it = scores.find(kTermNames[i]);
        terms[i] = it == scores.end() ? 0. : it->second;
    }
    return sc.combine(scores);
}

// One Monte-Carlo walker exactly as the reference searcher runs it.
int ref_system_mc_walker(void* h, int seed, int pose_id, int max_nsteps, int relax_nsteps,
                         double mc_mmenergy_threshold, double* out_xyz, double* out_torsions,
                         double* energy, double* pscore, long* nevals) {
    auto* s = static_cast<ref_system*>(h);
    if (!s->has_box || !s->sf) {
        g_error = "box and scoring function are required";
        return -1;
    }
    const name_and_task eoq("", {});
    blocking_queue<name_and_task> in_queue(4, eoq, 1);
    blocking_queue<name_and_task> out_queue(4, eoq, 1);
    docking_task task;
    task.feed.receptor = s->receptor;
    task.feed.cache = s->cache;
    task.feed.ligand = s->ligand;
    task.feed.pose_id = pose_id;
    std::string name = "oracle/pose-" + std::to_string(pose_id);
    global_energy_info["oracle"] = {{"minimum_pre_opt_energy", 1e8},
                                    {"minimum_accepted_energy", 1e8}};
    in_queue.push({name, std::move(task)});
    in_queue.close();
    monte_carlo_searcher searcher(*s->sf, s->bc, seed, max_nsteps, relax_nsteps,
                                  mc_mmenergy_threshold, in_queue);
    searcher.fill(out_queue);
    auto res = out_queue.pop();
    auto& f = res.second.fetch;
    from_pose(f.ligand_xyz, out_xyz);
    for (size_t i = 0; i < f.torsions.size(); ++i) out_torsions[i] = f.torsions[i];
    *energy = f.energy;
    *pscore = f.pscore;
    *nevals = static_cast<long>(f.nevals);
    return 0;
}

// ----------------------------------------------------------------- RNG (random.h)
void* ref_rng_create(unsigned seed) { return new random_generator(seed); }
void ref_rng_destroy(void* h) { delete static_cast<random_generator*>(h); }
int ref_rng_uniform_int(void* h, int a, int b) {
    return static_cast<random_generator*>(h)->uniform_int(a, b);
}
double ref_rng_uniform_real(void* h, double a, double b) {
    return static_cast<random_generator*>(h)->uniform_real(a, b);
}
double ref_rng_torsion(void* h) { return static_cast<random_generator*>(h)->uniform_torsion(); }
void ref_rng_in_box(void* h, const double* lo, const double* hi, double* out) {
    static_cast<random_generator*>(h)->random_in_box(lo, hi, out);
}
void ref_rng_orientation(void* h, double* q) {
    static_cast<random_generator*>(h)->random_orientation(q);
}
void ref_rng_in_sphere(void* h, double* out) {
    static_cast<random_generator*>(h)->random_in_sphere(out);
}

// ---------------------------------------------------- whole engine (entrance.cpp)
void* ref_engine_create(const char* receptor_file, const char* sf_file, int nthreads) {
    try {
        return new ReusableEngine(receptor_file, sf_file, nthreads);
    } catch (std::exception& e) {
        g_error = e.what();
        return nullptr;
    }
}
void ref_engine_destroy(void* h) { delete static_cast<ReusableEngine*>(h); }
void ref_engine_set_box(void* h, double cx, double cy, double cz, double sx, double sy,
                        double sz) {
    static_cast<ReusableEngine*>(h)->set_box(cx, cy, cz, sx, sy, sz);
}
int ref_engine_generate_maps(void* h, double spacing, double max_size) {
    try {
        static_cast<ReusableEngine*>(h)->generate_maps(spacing, max_size);
        return 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}
int ref_engine_optimize(void* h, const char* index_file, const char* out_dir, int max_niters,
                        double slope) {
    try {
        static_cast<ReusableEngine*>(h)->optimize(index_file, out_dir, max_niters, slope);
        return 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}
int ref_engine_search(void* h, const char* index_file, const char* out_dir, int seed,
                      int exhaustiveness, int max_nsteps, int relax_nsteps, int num_modes,
                      double min_rmsd, double mc_mmenergy_threshold, double slope) {
    try {
        static_cast<ReusableEngine*>(h)->search(index_file, out_dir, seed, exhaustiveness,
                                                max_nsteps, relax_nsteps, num_modes, min_rmsd,
                                                mc_mmenergy_threshold, slope);
        return 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}
int ref_engine_evaluate(void* h, const char* index_file, const char* out_file) {
    try {
        static_cast<ReusableEngine*>(h)->evaluate(index_file, out_file);
        return 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

}  // extern "C"
