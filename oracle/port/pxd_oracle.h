/*
 * pxd_oracle.h -- TEST INFRASTRUCTURE. FP64 C restatement of the Protenix-Dock
 * reference hot path, used only as the checker in tests/, by __graft_entry__.smoke()
 * and as the CPU baseline leg of bench.py. The product (the CUDA library) never
 * links, loads or calls it.
 *
 * Each function follows the reference file:line given beside it and keeps the
 * reference's FP64 operation order, so that results agree with the reference engine
 * compiled from its own sources (oracle/_ref) to rounding level. Parity of this port
 * is pinned by the oracle tests under tests/ against the reference unit-test golden values
 * (the gtest files under engine/utest) and against oracle/_ref where that library can be built.
 */
#ifndef PXD_ORACLE_H_
#define PXD_ORACLE_H_

#include <stdint.h>

#include "../../include/pxdock_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- math (engine/src/lib/math.cpp) ---- */
double po_dihedral(const double* pi, const double* pj, const double* pk, const double* pl);
double po_dihedral_and_gradient(const double* pi, const double* pj, const double* pk,
                                const double* pl, double* gi, double* gj, double* gk,
                                double* gl);
double po_angle_and_gradient(const double* pi, const double* pj, const double* pk,
                             double* gi, double* gk);
void po_rotation_axis_angle(const double* axis, double theta, double* rot9, double* jac9);
void po_rotation_quaternion(const double* q, double* rot9);
void po_vdw_type_table(double* sigma99, double* epsilon99);

/* ---- intra-molecular terms (engine/src/core/interaction.cpp:27-196) ----
 * which: 0 bonds, 1 angles, 2 dihedrals, 3 non-bonded, 4 total. grad accumulates. */
double po_intra_energy(int which, const pxd_topology* ff, const double* xyz, double* grad);

/* ---- a receptor + ligand system ---- */
typedef struct po_system po_system;
po_system* po_system_create(const pxd_receptor_desc* rec, const pxd_ligand_desc* lig);
void po_system_destroy(po_system* s);
int po_build_grid(po_system* s, const pxd_box* box, const int32_t* types, int32_t n_types,
                  int nthreads);
void po_set_slope(po_system* s, double slope);
void po_drop_grid(po_system* s);
/* map: ligand type 0..98, or 99 for Coulomb; out [P][4]; returns -1 if not built */
int po_grid_copy(const po_system* s, int map, double* out);
int po_grid_get(const po_system* s, int type, double q, const double* xyz, double* energy,
                double* grad);
/* binding_system_interactions::put_gradients; gradients are overwritten */
double po_score_grad(po_system* s, const double* rec_tors, const double* lig_xyz,
                     double* tors_grad, double* lig_grad);
/* lbfgs_step::apply on one pose (in/out), returns enum pxd_pose_status */
int po_lbfgs(po_system* s, const pxd_lbfgs_params* p, double* rec_tors, double* lig_xyz,
             double* energy, int32_t* nevals);
/* The same over a batch with nthreads host threads (the CPU baseline). */
int po_lbfgs_batch(po_system* s, const pxd_lbfgs_params* p, int32_t n_poses, double* rec_tors,
                   double* lig_xyz, double* energy, int32_t* nevals, int32_t* status,
                   int nthreads);
/* free_ligand::apply_parameters and torsional_receptor::apply_parameters */
void po_ligand_apply(const po_system* s, const double* xyz, const double* center,
                     const double* rot9, const double* torsions, double* out);
void po_receptor_apply(const po_system* s, const double* torsions, double* out);

/* ---- empirical scores (engine/src/core/scorer.cpp:53-866) ---- */
double po_score(const pxd_sf_params* sf, int n_rec, const double* rec_xyz, const double* rec_q,
                const double* rec_sigma, const double* rec_eps, const pxd_score_lists* rec_l,
                int n_lig, const double* lig_xyz, const double* lig_q, const int32_t* lig_type,
                const pxd_score_lists* lig_l, double* terms);
double po_vdw_check(const pxd_sf_params* sf, int n_rec, const double* rec_xyz,
                    const double* rec_sigma, const double* rec_eps, int n_lig,
                    const double* lig_xyz, const int32_t* lig_type);
double po_torsion_strain(const pxd_score_lists* l, const double* x);
double po_gbsa_parts(int n_rec, const double* rec_xyz, const double* rec_q,
                     const pxd_score_lists* rec_l, int n_lig, const double* lig_xyz,
                     const double* lig_q, const pxd_score_lists* lig_l, double* parts);

/* ---- differentiable empirical score (no reference counterpart; see pxd_score_adjoint) ----
 * Features [PXD_NUM_SCORE_FEATURES], S = po_combine_features(w, f), and, with g = dL/dS:
 * G [n_lig][3] += g dS/dx, dw [36] += g dS/dw, dtab [32*256] += g dS/dT (each may be NULL;
 * table NULL: no pair-table term; the table needs atomic_numbers in both lists). */
double po_score_diff(const pxd_sf_params* sf, int n_rec, const double* rec_xyz, const double* rec_q,
                     const double* rec_sigma, const double* rec_eps, const pxd_score_lists* rec_l,
                     int n_lig, const double* lig_xyz, const double* lig_q, const int32_t* lig_type,
                     const pxd_score_lists* lig_l, const double* weights, const double* table, double g,
                     double* features, double* dxyz, double* dweights, double* dtable);
double po_combine_features(const double* weights, const double* features);
void po_combine_grad(const double* weights, const double* features, double g, double* dweights);

/* ---- Monte-Carlo walker (engine/src/core/searcher.cpp:46-223) ---- */
int po_mc_walker(po_system* s, const pxd_sf_params* sf, const pxd_score_lists* rl,
                 const pxd_score_lists* ll, const double* lo, const double* hi, uint32_t seed,
                 int walker, const double* start, int first_pose, int max_nsteps,
                 int relax_nsteps, double threshold, double* global_min, double* out_xyz,
                 double* out_tors, double* out_energy, double* out_pscore, long* out_nevals);
void po_mc_randomize(po_system* s, const pxd_sf_params* sf, const double* lo, const double* hi,
                     uint32_t seed, int walker, const double* start, int first_pose, double* out);

/* ---- mt19937 + libstdc++ distributions as random_generator uses them
 *      (engine/include/bytedock/lib/random.h:33-63, engine/src/lib/random.cpp) ---- */
typedef struct po_rng {
    uint32_t mt[624];
    int idx;
} po_rng;
void po_rng_seed(po_rng* r, uint32_t seed);
uint32_t po_rng_next(po_rng* r);
int po_rng_uniform_int(po_rng* r, int a, int b);
double po_rng_uniform_real(po_rng* r, double a, double b);
double po_rng_torsion(po_rng* r);
void po_rng_in_box(po_rng* r, const double* lo, const double* hi, double* out);
void po_rng_orientation(po_rng* r, double* q);
void po_rng_in_sphere(po_rng* r, double* out);

#ifdef __cplusplus
}
#endif

#endif /* PXD_ORACLE_H_ */
