/*
 * pxdock_gb300.h -- C ABI of the GB300 docking hot path.
 *
 * The library replaces the CPU hot path of Protenix-Dock's C++ engine
 * (engine/src/core/{interaction,grid,optimizer,searcher,scorer,data}.cpp) with
 * hand-written sm_103a kernels. All entry points are plain C: opaque handles,
 * plain pointers and sizes, an int status (PXD_OK == 0) and a per-context error
 * string. Two levels are exported:
 *
 *   1. The engine facade (pxd_engine_*): file in / file out, the same methods,
 *      argument meanings and defaults as bytedock::ReusableEngine
 *      (engine/include/bytedock/core/entrance.h:30-74) and its Python binding
 *      _protenix_dock.ReusableEngine (engine/src/pyb/api.cpp:34-63).
 *
 *   2. The batch kernels (pxd_*): arrays of poses in, arrays of results out,
 *      each replacing one reference interface named in its comment.
 *
 * Conventions
 *   - Host-facing coordinates, torsions and energies are double (the reference's
 *     param_t in its default FP64 build). Device-facing buffers ("_dev") are float
 *     for coordinates/gradients and double for energies.
 *   - Ligand coordinates are [n_atoms][3] in the ligand file's atom order.
 *   - Receptor torsions are in receptor-leaf order (torsional_receptor::get_leaf).
 *   - A stream argument of NULL means the context's own stream.
 *   - Every call is synchronous with respect to the host unless it takes device
 *     pointers ("_dev"), in which case it is ordered on the given stream.
 */
#ifndef PXDOCK_GB300_H_
#define PXDOCK_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PXD_ABI_VERSION 2

/* ------------------------------------------------------------------ status */
enum pxd_status_code {
    PXD_OK = 0,
    PXD_ERR_INVALID = 1,      /* bad argument, size or index (the call did nothing) */
    PXD_ERR_STATE = 2,        /* precondition missing, e.g. no box or no maps */
    PXD_ERR_CUDA = 3,         /* CUDA runtime error */
    PXD_ERR_IO = 4,           /* file missing, unreadable or malformed */
    PXD_ERR_NOMEM = 5,        /* device or host allocation failed */
    PXD_ERR_DEVICE_FLAG = 6   /* a kernel reported an error flag (see pxd_last_error) */
};

/* Per-pose outcome of an optimisation (pxd_lbfgs_*), one int32 per pose. */
enum pxd_pose_status {
    PXD_POSE_CONVERGED = 0,     /* a tolerance test ended the run (lbfgs_step returns true) */
    PXD_POSE_NOT_CONVERGED = 1, /* iteration or evaluation cap reached */
    PXD_POSE_NAN = 2,           /* loss became NaN, run stopped (optimizer.cpp:532) */
    PXD_POSE_BAD_INPUT = 3      /* pose rejected before optimisation (bad ligand id) */
};

/* ------------------------------------------------------------------ limits */
#define PXD_NUM_VDW_TYPES 99          /* ligand vdW types (kNumVdwTypes, constant.h:26) */
#define PXD_MAX_LIGAND_ATOMS 256
#define PXD_MAX_RECEPTOR_TORSIONS 64

/* --------------------------------------------------------------- data model */

/* Force-field terms of one molecule; the layout follows force_field_params
 * (engine/include/bytedock/core/system.h:85-109). Atom indices are 0-based into
 * the molecule. Dihedral terms keep the reference's 6 periodic slots; a slot with
 * periodicity 0 ends the list for that dihedral (interaction.cpp:90). */
typedef struct pxd_topology {
    int32_t n_atoms;
    const double* charge;        /* [n_atoms] partial charges */
    const double* sigma;         /* [n_atoms] LJ sigma, Angstrom */
    const double* epsilon;       /* [n_atoms] LJ epsilon, kcal/mol */

    int32_t n_bonds;
    const int32_t* bond_atoms;   /* [n_bonds][2] */
    const double* bond_k;        /* [n_bonds] */
    const double* bond_length;   /* [n_bonds] */

    int32_t n_angles;
    const int32_t* angle_atoms;  /* [n_angles][3], vertex in the middle */
    const double* angle_k;       /* [n_angles] */
    const double* angle_radian;  /* [n_angles] */

    int32_t n_impropers;
    const int32_t* improper_atoms;       /* [n][4] */
    const int32_t* improper_periodicity; /* [n][6] */
    const double* improper_phase;        /* [n][6] radian */
    const double* improper_k;            /* [n][6] */

    int32_t n_propers;
    const int32_t* proper_atoms;         /* [n][4] */
    const int32_t* proper_periodicity;   /* [n][6] */
    const double* proper_phase;          /* [n][6] radian */
    const double* proper_k;              /* [n][6] */

    int32_t n_pairs14;
    const int32_t* pairs14;      /* [n][2]  1-4 pairs: Coulomb x 0.833333333, LJ x 0.5 */
    int32_t n_pairs;
    const int32_t* pairs;        /* [n][2]  all other non-bonded pairs, scale 1 */
} pxd_topology;

/* Interaction atom lists of one molecule used by the empirical scores (the pscore /
 * bscore fields of force_field_params, system.h:95-108). Rings are [n][6] atom ids,
 * padded with -1 after the ring's last atom. Donors are (heavy atom, hydrogen). The
 * torsion-strain lists are ligand-only: entry e has coefficients tstrain_coefs[e][4] and
 * the matched quadruples tstrain_quads[tstrain_offsets[e] .. tstrain_offsets[e+1]). */
typedef struct pxd_score_lists {
    int32_t n_hydrophobic; const int32_t* hydrophobic;
    int32_t n_cation; const int32_t* cation;
    int32_t n_anion; const int32_t* anion;
    int32_t n_ring5; const int32_t* ring5;
    int32_t n_ring6; const int32_t* ring6;
    int32_t n_don_charged; const int32_t* don_charged;
    int32_t n_don_neutral; const int32_t* don_neutral;
    int32_t n_acc_charged; const int32_t* acc_charged;
    int32_t n_acc_neutral; const int32_t* acc_neutral;
    int32_t n_tstrain; const double* tstrain_coefs; const int32_t* tstrain_offsets;
    const int32_t* tstrain_quads;
    int32_t n_rotatable;
    const int32_t* atomic_numbers;   /* [n_atoms], may be NULL when GBSA is off */
    int32_t n_all_bonds; const int32_t* all_bonds;
} pxd_score_lists;

/* Empirical score terms, in the order of their coefficients in pxd_sf_params. */
enum pxd_score_term {
    PXD_TERM_COULOMB = 0,     /* InteractionCoulomb_oriEnergy */
    PXD_TERM_VDW = 1,         /* InteractionVDW_Energy */
    PXD_TERM_IONIC = 2,       /* Ionic_Energy */
    PXD_TERM_PI_CATION = 3,   /* Pi_Cationic_Energy */
    PXD_TERM_F2F = 4,         /* F2FPiStacking_Energy */
    PXD_TERM_E2F = 5,         /* E2FPiStacking_Energy */
    PXD_TERM_HBOND = 6,       /* Hbond_Energy */
    PXD_TERM_HYDROPHOBIC = 7, /* Hydrophobic_Energy */
    PXD_TERM_TSTRAIN = 8,     /* TorsionStrain_Penalty */
    PXD_TERM_ROTATABLE = 9,   /* rotatable_energy */
    PXD_TERM_GBSA = 10,       /* Gbsa_Com_Energy-Gbsa_Lig_Energy-Gbsa_Pro_Energy */
    PXD_NUM_TERMS = 11
};

/* One scoring function (ScoringFunctionParams, conf.h:122-150) with the parameters of
 * its active terms. coef[t] is the weight of term t as root_scorer::combine applies it
 * (scorer.cpp:117-126); a term is active when |coef| > 1e-5 (utility.h:26). */
typedef struct pxd_sf_params {
    double coef[PXD_NUM_TERMS];
    double vdw_scale, vdw_cutoff;
    double vdw_sigma_scale[PXD_NUM_VDW_TYPES], vdw_epsilon_scale[PXD_NUM_VDW_TYPES];
    double ionic_coef[2];              /* lc, pc */
    double ionic[2][2];                /* dist_min, dist_max */
    double picat_coef[4];              /* lc5, lc6, pc5, pc6 */
    double picat[4][2];                /* dist_min, dist_max */
    double stack_coef[2][4];           /* [f2f, e2f][l5r5, l5r6, l6r5, l6r6] */
    double stack[2][4][6];             /* dist_min, dist_max, angle_min, angle_max, sigma_min, sigma_max */
    double hbond_scale;
    double hbond_coef[8];              /* hldcc hldcn hldnc hldnn hpdcc hpdcn hpdnc hpdnn */
    double hbond[8][6];                /* dist_min, dist_max, angle_min, angle_max, dist_center, angle_center */
    double hydro_scale, hydro_dist_min, hydro_dist_max, hydro_scale_factor;
} pxd_sf_params;

/* Ligand torsion tree (fragment_tree, system.h:135-154) in a flat form. Fragments
 * are numbered as in the ligand file. Atom positions are "permuted" positions:
 * position p holds atom perm[p], and fragment f owns positions
 * [frag_start[f], frag_end[f]). Non-root fragments are listed in torsion order,
 * i.e. the reference's pre-order walk (data.cpp:555-590), so entry k of
 * tors_* belongs to torsion k. */
typedef struct pxd_torsion_tree {
    int32_t n_frags;
    const int32_t* frag_start;    /* [n_frags] */
    const int32_t* frag_end;      /* [n_frags] */
    const int32_t* perm;          /* [n_atoms] permuted position -> atom index */
    int32_t n_roots;
    const int32_t* roots;         /* [n_roots] root fragment ids (no torsion) */
    int32_t n_torsions;           /* n_frags - n_roots */
    const int32_t* tors_frag;     /* [n_torsions] fragment rotated by torsion k */
    const int32_t* tors_parent;   /* [n_torsions] parent fragment id */
    const int32_t* tors_parent_atom; /* [n_torsions] bond atom in parent (permuted position) */
    const int32_t* tors_mine_atom;   /* [n_torsions] bond atom in fragment (permuted position) */
} pxd_torsion_tree;

/* A ligand as parsed from its JSON file (free_ligand, data.h:70-99). */
typedef struct pxd_ligand_desc {
    pxd_topology ff;             /* sigma/epsilon taken from the ligand vdW type table */
    const int32_t* vdw_type;     /* [n_atoms] ligand vdW type 0..98 (kVdwTypeTags order) */
    pxd_torsion_tree tree;       /* may have n_frags == 0 for optimisation-only use */
    const pxd_score_lists* lists;/* NULL: the ligand cannot be scored by pxd_score_* */
} pxd_ligand_desc;

/* The receptor (torsional_receptor, data.h:34-67). Rotor r turns the atoms
 * rotor_atoms[rotor_offsets[r] .. rotor_offsets[r+1]) -- the terminal fragment --
 * about the axis from atom rotor_axis[r][0] to atom rotor_axis[r][1]; the axis atom
 * itself does not move (data.cpp:352-363). */
typedef struct pxd_receptor_desc {
    int32_t n_atoms;
    const double* xyz;           /* [n_atoms][3] */
    pxd_topology ff;             /* charge/sigma/epsilon for every atom + intra terms */
    int32_t n_rotors;
    const int32_t* rotor_axis;   /* [n_rotors][2] */
    const int32_t* rotor_offsets;/* [n_rotors+1] */
    const int32_t* rotor_atoms;  /* [rotor_offsets[n_rotors]] */
    const pxd_score_lists* lists;/* NULL: no empirical scores for this receptor */
} pxd_receptor_desc;

/* Grid box (box_config, grid.h:31-40). */
typedef struct pxd_box {
    double init_xyz[3];          /* front-left-bottom grid point */
    int32_t npoints[3];          /* points per axis (N_vox + 1) */
    double spacing;              /* Angstrom */
} pxd_box;

/* L-BFGS + strong-Wolfe constants. pxd_lbfgs_defaults() gives the reference's
 * values (optimizer.h:52-66, optimizer.cpp:235-246). */
typedef struct pxd_lbfgs_params {
    int32_t max_iter;            /* reference: max_niters argument (240) */
    int32_t max_eval;            /* 0 -> max_iter * 5 / 4 (optimizer.h:54) */
    int32_t history;             /* memory size m; reference 100; at most PXD_MAX_HISTORY */
    int32_t ls_max;              /* strong-Wolfe evaluations per iteration, 25 */
    double lr;                   /* 1.0 */
    double tolerance_grad;       /* 0.5, max-norm of the gradient */
    double tolerance_change;     /* 1e-4 */
    double ls_c1;                /* 1e-4 */
    double ls_c2;                /* 0.9 */
    double ls_tolerance_change;  /* 1e-9 */
    double ls_gtd_threshold;     /* 1e5 */
    double reset_threshold;      /* 1e8: history is dropped when max|y| exceeds it */
    int32_t dof_mode;            /* PXD_DOF_CARTESIAN (0, the reference) or PXD_DOF_RIGID_TORSION */
    int32_t reserved;            /* 0 */
} pxd_lbfgs_params;

/* Variables of the batched optimiser (pxd_lbfgs_params.dof_mode).
 *   PXD_DOF_CARTESIAN       [ligand xyz (3N) | receptor torsions (R)], the reference's
 *                           flat closure (optimizer.cpp:155-167);
 *   PXD_DOF_RIGID_TORSION   [centre (3) | quaternion (4) | ligand torsions (T) | receptor
 *                           torsions (R)], D = 7 + T + R (no reference counterpart). The
 *                           ligand is placed from the pose's own input coordinates by the
 *                           torsion-tree forward map (free_ligand::apply_parameters,
 *                           data.cpp:592-641) starting at centre = the input's geometric
 *                           centre, identity orientation and zero torsion changes, so bond
 *                           lengths and angles keep their input values; the gradient is
 *                           the Cartesian one pulled back through the tree. The returned
 *                           pose is the placed Cartesian pose. Ligands need <= 32 torsions
 *                           and <= 64 fragments (else the pose's status is
 *                           PXD_POSE_BAD_INPUT). Applies to pxd_lbfgs*, not to the
 *                           Monte-Carlo search (PXD_ERR_INVALID there). */
#define PXD_DOF_CARTESIAN 0
#define PXD_DOF_RIGID_TORSION 1

#define PXD_MAX_HISTORY 128

/* ------------------------------------------------------------------ context */
typedef struct pxd_context pxd_context;

int32_t pxd_abi_version(void);
const char* pxd_version(void);

/* One context per receptor, bound to one CUDA device. */
int pxd_context_create(int32_t device, pxd_context** out);
void pxd_context_destroy(pxd_context* ctx);
/* Message of the last failed call on this context (empty string if none). */
const char* pxd_last_error(const pxd_context* ctx);
/* Stream the context orders its own work on (a cudaStream_t). */
void* pxd_context_stream(pxd_context* ctx);

void pxd_lbfgs_defaults(pxd_lbfgs_params* out);

/* Copies the receptor to the device and prepares the rotor tables
 * (torsional_receptor::parse post-processing, data.cpp:366-385). Drops any maps. */
int pxd_set_receptor(pxd_context* ctx, const pxd_receptor_desc* receptor);

/* decide_grid_dims (grid.cpp:65-86): N_vox = ceil(size/spacing) rounded up to
 * even, N_vox + 1 points per axis, box centred on the centre. */
int pxd_decide_grid_dims(double center_x, double center_y, double center_z, double size_x,
                         double size_y, double size_z, double spacing, pxd_box* out);

/* Builds the Coulomb map and the vdW maps of the listed ligand types (0..98) on the
 * device; replaces receptor_cache::populate (grid.cpp:115-195). n_types == -1 builds
 * all 99 types, as the reference does. Receptor rotor atoms are excluded from the
 * maps and handled as explicit pairs (grid.cpp:119-123). */
int pxd_grid_build(pxd_context* ctx, const pxd_box* box, const int32_t* types,
                   int32_t n_types);
/* Out-of-box penalty slope (receptor_cache::set_slope, grid.h:78). */
int pxd_grid_set_slope(pxd_context* ctx, double slope);
int pxd_grid_drop(pxd_context* ctx);
int pxd_grid_info(pxd_context* ctx, pxd_box* box, int32_t* n_maps);
/* Copies one map to the host as float records {E, dE/dx, dE/dy, dE/dz} per point,
 * k fastest (grid.h:120-122). map = ligand type 0..98, or 99 for Coulomb.
 * Returns PXD_ERR_INVALID if the map was not built. */
int pxd_grid_read_map(pxd_context* ctx, int32_t map, float* host_out);
/* Installs a map from host records (used by load_maps). */
int pxd_grid_write_map(pxd_context* ctx, const pxd_box* box, int32_t map,
                       const float* host_records);
/* The same in FP64, as the reference's val_and_grad records (grid.h:54-57) hold them:
 * read gives E = FP32 record + the map's FP64 energy remainder and the gradient
 * widened; write rounds E to the FP32 record and keeps the remainder, so a read after a
 * write returns the energies it was given (to ~2^-48 relative) and reading, writing and
 * reading again is exact. Used by dump_maps / load_maps with the reference's files. */
int pxd_grid_read_map64(pxd_context* ctx, int32_t map, double* host_out);
int pxd_grid_write_map64(pxd_context* ctx, const pxd_box* box, int32_t map,
                         const double* host_records);

/* ------------------------------------------------ the reference's map cache files */

/* Codec of receptor_cache::save / restore's files (grid.cpp:305-431), host only (no
 * device is touched): a <tag>.bdg Boost binary archive of one map's
 * std::vector<val_and_grad> and the meta.dat Boost text archive (format version
 * 20241030, box origin, points per axis, spacing, excluded receptor atoms).
 * pxd_bdg_encode: records = n_points x {E, dE/dx, dE/dy, dE/dz}; value_bytes 8 (the
 * reference's default double build) or 4 (its float build). Returns the archive's
 * length; the bytes are written only when out_capacity holds them (out may be NULL).
 * pxd_bdg_decode: returns the point count and sets value_bytes; records are written
 * only when capacity_points holds them. pxd_meta_encode returns the text length and
 * writes it NUL-terminated when out_capacity > length. pxd_meta_decode returns the
 * number of excluded atoms (written when capacity holds them) and sets version; when
 * version is not 20241030 nothing after it is read. Errors are negative PXD_ERR_* codes
 * (PXD_ERR_IO: malformed input). */
int64_t pxd_bdg_encode(const double* records, int64_t n_points, int32_t value_bytes,
                       uint8_t* out, int64_t out_capacity);
int64_t pxd_bdg_decode(const uint8_t* data, int64_t size, double* records,
                       int64_t capacity_points, int32_t* value_bytes);
int64_t pxd_meta_encode(const pxd_box* box, const int64_t* excluded, int64_t n_excluded,
                        char* out, int64_t out_capacity);
int64_t pxd_meta_decode(const char* text, int64_t size, pxd_box* box, uint64_t* version,
                        int64_t* excluded, int64_t capacity);

/* Registers a ligand's topology and torsion tree on the device. */
int pxd_add_ligand(pxd_context* ctx, const pxd_ligand_desc* ligand, int32_t* ligand_id);
int pxd_clear_ligands(pxd_context* ctx);

/* ------------------------------------------------------------ batch kernels */

/* Energy and gradient of n_poses poses: replaces
 * binding_system_interactions::put_gradients (interaction.cpp:271-298) -- intra
 * receptor + intra ligand + grid or brute-force inter terms, chain rule onto
 * receptor torsions. Gradients are written, not accumulated.
 *   ligand_ids_dev [n_poses]             int32
 *   lig_xyz_dev    [n_poses][max_atoms][3] float, pose p in row p
 *   rec_tors_dev   [n_poses][n_rec_torsions] float (NULL when no rotors)
 *   energy_dev     [n_poses]             double
 *   lig_grad_dev   [n_poses][max_atoms][3] float
 *   tors_grad_dev  [n_poses][n_rec_torsions] float (NULL when no rotors)
 * max_atoms is the row stride in atoms (>= every ligand's n_atoms). */
int pxd_score_grad_dev(pxd_context* ctx, int32_t n_poses, int32_t max_atoms,
                       const int32_t* ligand_ids_dev, const float* lig_xyz_dev,
                       const float* rec_tors_dev, double* energy_dev, float* lig_grad_dev,
                       float* tors_grad_dev, void* stream);

/* pxd_score_grad_dev over poses of several contexts (one receptor and map set each, all
 * on one device) in one launch: contexts [n_contexts] is a host array, ctx_ids_dev [P]
 * picks each pose's context and ligand_ids_dev the ligand in it; rec_tors / tors_grad
 * rows have the largest receptor-torsion count of the contexts. lig_grad padding rows
 * are zero. Errors are reported on contexts[0]. */
int pxd_score_grad_multi_dev(pxd_context* const* contexts, int32_t n_contexts, int32_t n_poses,
                             int32_t max_atoms, const int32_t* ctx_ids_dev,
                             const int32_t* ligand_ids_dev, const float* lig_xyz_dev,
                             const float* rec_tors_dev, double* energy_dev, float* lig_grad_dev,
                             float* tors_grad_dev, void* stream);

/* Host-buffer version of pxd_score_grad_dev for one ligand (double in/out). */
int pxd_score_grad(pxd_context* ctx, int32_t ligand_id, int32_t n_poses,
                   const double* lig_xyz, const double* rec_tors, double* energy,
                   double* lig_grad, double* tors_grad);

/* L-BFGS with strong-Wolfe line search over [ligand xyz | receptor torsions] for
 * every pose, all in one persistent launch; replaces lbfgs_step::apply
 * (optimizer.cpp:429-560) as driven by serial_optimizer (optimizer.cpp:28-54).
 * lig_xyz_dev / rec_tors_dev hold the start state and receive the final state.
 *   energy_dev [n_poses] double  final energy (re-evaluated, optimizer.cpp:554-558)
 *   nevals_dev [n_poses] int32   score+gradient evaluations used
 *   status_dev [n_poses] int32   enum pxd_pose_status */
int pxd_lbfgs_dev(pxd_context* ctx, const pxd_lbfgs_params* params, int32_t n_poses,
                  int32_t max_atoms, const int32_t* ligand_ids_dev, float* lig_xyz_dev,
                  float* rec_tors_dev, double* energy_dev, int32_t* nevals_dev,
                  int32_t* status_dev, void* stream);

/* pxd_lbfgs_dev without any device allocation (no counterpart in the reference: it
 * serves callers that must not allocate, e.g. inside a memory-pool budget). The
 * L-BFGS history and the pose-queue counter live in a 32 MiB file-scope device array;
 * the persistent grid shrinks to the warps whose history fits, and a request where not
 * even one block fits is rejected with PXD_ERR_INVALID. The counter is cleared by a
 * memset on `stream` at every call. Overlapping calls (other streams or threads) share
 * the array and race. The first call on a device resolves the array's address: make
 * it before any stream capture. Ligands added since the last launch must fit the
 * existing device ligand table (else PXD_ERR_STATE: one pxd_lbfgs_dev call grows it). */
int pxd_lbfgs_dev_noalloc(pxd_context* ctx, const pxd_lbfgs_params* params, int32_t n_poses,
                          int32_t max_atoms, const int32_t* ligand_ids_dev, float* xyz_dev,
                          float* receptor_torsions_dev, double* energy_dev, int32_t* nevals_dev,
                          int32_t* status_dev, void* stream);

/* Host-buffer version for one ligand: copies in, runs, copies out (double). */
int pxd_lbfgs(pxd_context* ctx, const pxd_lbfgs_params* params, int32_t ligand_id,
              int32_t n_poses, double* lig_xyz, double* rec_tors, double* energy,
              int32_t* nevals, int32_t* status);

/* Autotuner of the batched optimiser (no reference counterpart). For every size class
 * (ligands of <= 32, 64, ... 256 atoms) present in the batch, runs each variant of the
 * optimiser kernel -- resident blocks per SM 3, 4, 5, 6 or unbounded (the register
 * budget), each with the L-BFGS history in global memory or, where it fits, in shared
 * memory (+ PXD_LBFGS_HIST_SMEM) -- on up to `sample` of the class's poses with max_iter
 * capped at probe_iters, times them with CUDA events, and keeps the variant with the most
 * score+gradient evaluations per second for this context's later pxd_lbfgs* calls.
 * Probes run on copies: the caller's poses are not modified. report [8][2] (may be NULL)
 * receives (class bound, chosen variant), -1 after the last class. Synchronous. */
int pxd_lbfgs_autotune_dev(pxd_context* ctx, const pxd_lbfgs_params* params, int32_t n_poses,
                           int32_t max_atoms, const int32_t* ligand_ids_dev, const float* xyz_dev,
                           const float* tors_dev, int32_t sample, int32_t probe_iters,
                           int32_t* report, void* stream);

/* Sets the optimiser variant of one size class (class_bound 32, 64, ... 256) for this
 * context's later pxd_lbfgs* calls, as the autotuner would: variant = resident blocks per
 * SM (3, 4, 5, 6, or 0 for unbounded registers), + PXD_LBFGS_HIST_SMEM for the history in
 * shared memory (ignored for launches whose slices would not fit it); -1 restores the
 * default. Lets a caller reuse a saved tuning. Every variant computes the same arithmetic;
 * register budgets may contract it differently. */
#define PXD_LBFGS_HIST_SMEM 256
int pxd_lbfgs_set_variant(pxd_context* ctx, int32_t class_bound, int32_t variant);

/* Host-buffer version over poses of several ligands in one launch (the engine's
 * optimize over a whole ligand index): ligand_ids [n], xyz [n][max_atoms][3] and
 * torsions [n][R] (in/out, double), energy [n], nevals [n], status [n]. */
int pxd_lbfgs_multi(pxd_context* ctx, const pxd_lbfgs_params* params, int32_t n_poses,
                    int32_t max_atoms, const int32_t* ligand_ids, double* xyz, double* torsions,
                    double* energy, int32_t* nevals, int32_t* status);

/* Forward torsion-tree kinematics of a batch: replaces free_ligand::apply_parameters
 * (data.cpp:592-641). For pose p: centre [3], rotation matrix rot [9] row-major,
 * torsions [n_torsions] (pre-order), applied to the reference pose xyz_in. */
int pxd_ligand_kinematics(pxd_context* ctx, int32_t ligand_id, int32_t n_poses,
                          const double* xyz_in, const double* centers, const double* rots,
                          const double* torsions, double* xyz_out);

/* Backward torsion-tree kinematics (no reference counterpart: the reference optimises
 * ligand atoms in Cartesian space and only runs the tree forward). For poses produced by
 * pxd_ligand_kinematics with centre c, and dE/dx of some E at those coordinates:
 *   center_grad [P][3] = sum_i dE/dx_i,
 *   torque      [P][3] = sum_i (x_i - c) x dE/dx_i   (rotation applied left of the root
 *                        orientation, rotation-vector coordinates at zero),
 *   torsion_grad [P][T] = dE/dtheta_k: u_k . sum over the torsion's subtree of
 *                        (x_i - x_bond) x dE/dx_i, u_k the unit parent->bond-atom axis.
 * xyz and atom_grad are [P][N][3] in the ligand's atom order. */
int pxd_ligand_backward(pxd_context* ctx, int32_t ligand_id, int32_t n_poses, const double* xyz,
                        const double* centers, const double* atom_grad, double* center_grad,
                        double* torque, double* torsion_grad);

/* Receptor rotor kinematics: replaces torsional_receptor::apply_parameters
 * (data.cpp:366-385). out: [n_poses][n_atoms][3]. */
int pxd_receptor_kinematics(pxd_context* ctx, int32_t n_poses, const double* torsions,
                            double* xyz_out);

/* ------------------------------------------------------- empirical scores */

/* Installs a scoring function: which = 0 pose selection (pscore), 1 affinity (bscore).
 * Replaces scoring_function_factory (factory.cpp:213-238) for the device scorers. */
int pxd_set_scoring_function(pxd_context* ctx, int32_t which, const pxd_sf_params* params);

/* Empirical score of a batch (root_scorer::combine with precalculate,
 * scorer.h:92-136), one warp per pose. terms_dev [n_poses][PXD_NUM_TERMS] receives the
 * unweighted term values (may be NULL). The GB/SA term is evaluated by
 * pxd_score_gbsa and contributes 0 here. */
int pxd_score_dev(pxd_context* ctx, int32_t which, int32_t n_poses, int32_t max_atoms,
                  const int32_t* ligand_ids_dev, const float* lig_xyz_dev,
                  const float* rec_tors_dev, double* score_dev, double* terms_dev, void* stream);

/* Host-buffer version for one ligand; the GB/SA term is included when its weight is
 * non-zero. */
int pxd_score(pxd_context* ctx, int32_t which, int32_t ligand_id, int32_t n_poses,
              const double* lig_xyz, const double* rec_tors, double* score, double* terms);

/* Generalised-Born / surface-area energy difference complex - ligand - receptor
 * (gbsa_total_energy::summary, scorer.cpp:737-866) of one pose, FP64 on the device.
 * parts[3] (may be NULL) receives the complex, ligand and receptor energies. */
int pxd_score_gbsa(pxd_context* ctx, int32_t ligand_id, const double* lig_xyz,
                   const double* rec_tors, double* delta, double* parts);

/* ------------------------------------------- differentiable empirical score */
/* No reference counterpart: the reference's scorers return values only
 * (root_scorer::combine, scorer.cpp:53-126). Here the empirical score is a function
 *   S(x; w, T) = sum over the terms of scorer.cpp:207-613 with the 36 weights w in place
 *                of the scoring function's coefficients and term scales (GB/SA
 *                excluded; every term is evaluated whatever its weight)
 *              + sum over ligand x receptor heavy-atom pairs closer than
 *                (PXD_PAIR_BINS - 1) * PXD_PAIR_BIN_WIDTH of T[type][r / width],
 *                linearly interpolated between bins,
 * and the adjoint returns dS/dx (ligand atoms), dS/dw and dS/dT. The ramps, cut-offs
 * and sigma / epsilon scales stay those of the installed scoring function. */
#define PXD_NUM_SF_WEIGHTS 36
enum pxd_sf_weight {
    PXD_W_COEF = 0,          /* coef[PXD_TERM_*], 11 entries */
    PXD_W_VDW_SCALE = 11,
    PXD_W_HYDRO_SCALE = 12,
    PXD_W_HBOND_SCALE = 13,
    PXD_W_IONIC = 14,        /* ionic_coef[2] */
    PXD_W_PICAT = 16,        /* picat_coef[4] */
    PXD_W_STACK = 20,        /* stack_coef[2][4] */
    PXD_W_HBOND = 28         /* hbond_coef[8] */
};
/* Unweighted sums the score is linear in, per pose (features[PXD_NUM_SCORE_FEATURES]):
 * 0 Coulomb, 1 clamped LJ, 2-3 ionic (ligand cation, receptor cation), 4-7 cation-pi
 * (l-cation x r-ring5, x r-ring6, l-ring5 x r-cation, l-ring6 x r-cation), 8-15
 * pi stacking [f2f, e2f][l5r5, l5r6, l6r5, l6r6], 16-23 hydrogen-bond classes, 24
 * hydrophobic, 25 torsion strain, 26 rotatable, 27 pair table. */
#define PXD_NUM_SCORE_FEATURES 28
/* Pair-table typing: ligand heavy atoms C N O S P F Cl other (8 classes) x receptor
 * heavy atoms C N O other (4 classes); hydrogens take no table term. Needs
 * atomic_numbers in both molecules' pxd_score_lists. */
#define PXD_PAIR_TYPES 32
#define PXD_PAIR_BINS 256
#define PXD_PAIR_BIN_WIDTH 0.03125

/* The 36 weights of a scoring function, in pxd_sf_weight order. */
void pxd_sf_weights(const pxd_sf_params* params, double* weights);

/* Score and adjoint of a batch, one warp per pose (device buffers, stream-ordered).
 * weights [36] (double) and tables [PXD_PAIR_TYPES][PXD_PAIR_BINS] (float, NULL: no
 * table term). grad_out [n_poses] is dL/dS per pose; NULL computes scores and features
 * only. Outputs (each may be NULL): score [n_poses], features [n_poses][28],
 * dxyz [n_poses][max_atoms][3] = grad_out * dS/dx (overwritten, padding rows zero),
 * dweights [36] and dtables [32][256] (double) ACCUMULATE sum_p grad_out_p * dS_p/d...
 * (callers zero them first, as the reference's gradient callers do). Receptor atoms are
 * fixed (rotor atoms placed by rec_tors). */
int pxd_score_adjoint_dev(pxd_context* ctx, int32_t which, int32_t n_poses, int32_t max_atoms,
                          const int32_t* ligand_ids_dev, const float* lig_xyz_dev,
                          const float* rec_tors_dev, const double* weights_dev,
                          const float* tables_dev, const double* grad_out_dev, double* score_dev,
                          double* features_dev, float* dxyz_dev, double* dweights_dev,
                          double* dtables_dev, void* stream);

/* pxd_score_adjoint_dev over poses of several contexts (one receptor and its grid each,
 * all on one device) in one launch: contexts [n_contexts] is a host array,
 * context_ids_dev [n_poses] picks each pose's context and ligand_ids_dev the ligand in it;
 * rec_tors_dev rows have the largest receptor-torsion count of the contexts. Every
 * context needs scoring function `which`. Errors are reported on contexts[0]. */
int pxd_score_adjoint_multi_dev(pxd_context* const* contexts, int32_t n_contexts, int32_t which,
                                int32_t n_poses, int32_t max_atoms, const int32_t* context_ids_dev,
                                const int32_t* ligand_ids_dev, const float* lig_xyz_dev,
                                const float* rec_tors_dev, const double* weights_dev,
                                const float* tables_dev, const double* grad_out_dev,
                                double* score_dev, double* features_dev, float* dxyz_dev,
                                double* dweights_dev, double* dtables_dev, void* stream);

/* Second-order products of the same score along a direction of the ligand coordinates
 * (forward-mode over the adjoint, derivatives almost everywhere): for each pose p with
 * direction xyz_dir [P][max_atoms][3] and output weight grad_out[p],
 *   dxyz_dir [P][max_atoms][3] = grad_out_p * H_p xyz_dir_p   (H_p = d2 S_p / dx2),
 *   features_dir [P][28]       = the features' derivatives along xyz_dir_p,
 *   dweights_dir [36], dtables_dir [32][256] += sum_p grad_out_p * d/dw, d/dT of
 *                                (xyz_dir_p . dS_p/dx)  (the mixed derivatives).
 * Outputs may be NULL; the same context rules as pxd_score_adjoint_multi_dev. */
int pxd_score_hvp_multi_dev(pxd_context* const* contexts, int32_t n_contexts, int32_t which,
                            int32_t n_poses, int32_t max_atoms, const int32_t* context_ids_dev,
                            const int32_t* ligand_ids_dev, const float* lig_xyz_dev,
                            const float* xyz_dir_dev, const float* rec_tors_dev,
                            const double* weights_dev, const float* tables_dev,
                            const double* grad_out_dev, double* features_dir_dev,
                            float* dxyz_dir_dev, double* dweights_dir_dev,
                            double* dtables_dir_dev, void* stream);

/* Host-buffer version for one ligand (double in/out; tables may be NULL, grad_out NULL
 * means 1 for every pose). */
int pxd_score_adjoint(pxd_context* ctx, int32_t which, int32_t ligand_id, int32_t n_poses,
                      const double* lig_xyz, const double* rec_tors, const double* weights,
                      const double* tables, const double* grad_out, double* score,
                      double* features, double* dxyz, double* dweights, double* dtables);

/* Device-buffer pose kinematics for gradient pipelines (no reference counterpart beyond
 * free_ligand::apply_parameters, data.cpp:592-641). Pose p: centre [3], orientation as a
 * quaternion (w, x, y, z) [4], normalised on use and turned into a matrix as
 * get_rotation_matrix does (math.cpp:22-42), torsions [T]. xyz_in [N][3] is the
 * ligand's reference pose; xyz_out [P][N][3]. */
int pxd_ligand_pose_dev(pxd_context* ctx, int32_t ligand_id, int32_t n_poses, const float* xyz_in_dev,
                        const float* centers_dev, const float* quats_dev, const float* torsions_dev,
                        float* xyz_out_dev, void* stream);

/* Pose kinematics over poses of several contexts (no reference counterpart beyond
 * free_ligand::apply_parameters, data.cpp:592-641): pose p is ligand lig_ids[p] of
 * contexts[ctx_ids[p]]; dofs [P][dof] (centre, quaternion w x y z, torsions padded to
 * dof); xyz_ref [P][max_atoms][3] each pose's reference coordinates. With atom_grad NULL,
 * writes xyz_out [P][max_atoms][3] (padding rows zero). With atom_grad [P][max_atoms][3]
 * (dE/dx at xyz_out), writes dofs_grad [P][dof] instead (backward; xyz_out is read). A
 * pose whose ligand does not fit its row (atoms > max_atoms or 7 + torsions > dof) gets
 * NaN outputs. */
int pxd_ligand_pose_multi_dev(pxd_context* const* contexts, int32_t n_contexts, int32_t n_poses,
                              int32_t max_atoms, int32_t dof, const int32_t* ctx_ids_dev,
                              const int32_t* lig_ids_dev, const float* xyz_ref_dev,
                              const float* dofs_dev, float* xyz_out_dev, const float* atom_grad_dev,
                              float* dofs_grad_dev, void* stream);

/* Directional derivatives of the multi-context pose kinematics along a DOF direction
 * dofs_dir [P][dof] at the poses xyz [P][max_atoms][3] = placed from dofs:
 *   atom_grad NULL:  out_dir [P][max_atoms][3] = dx along dofs_dir (forward mode);
 *   atom_grad set:   out_dir [P][dof] = derivative along dofs_dir of the backward map
 *                    (dofs, x, dE/dx) -> dE/dq, with xyz_dir = dx along dofs_dir and
 *                    atom_grad_dir = d(dE/dx) along it (H_x xyz_dir). This is the
 *                    DOF-space Hessian-vector product of E. */
int pxd_ligand_pose_dir_multi_dev(pxd_context* const* contexts, int32_t n_contexts, int32_t n_poses,
                                  int32_t max_atoms, int32_t dof, const int32_t* ctx_ids_dev,
                                  const int32_t* lig_ids_dev, const float* xyz_dev, const float* dofs_dev,
                                  const float* dofs_dir_dev, const float* xyz_dir_dev,
                                  const float* atom_grad_dev, const float* atom_grad_dir_dev,
                                  float* out_dir_dev, void* stream);

/* Backward of pxd_ligand_pose_dev: from dL/dx [P][N][3] at xyz [P][N][3], writes
 * dL/dcentre [P][3], dL/dquaternion [P][4] (through the normalisation) and
 * dL/dtorsions [P][T]. */
int pxd_ligand_pose_backward_dev(pxd_context* ctx, int32_t ligand_id, int32_t n_poses,
                                 const float* xyz_dev, const float* centers_dev, const float* quats_dev,
                                 const float* atom_grad_dev, float* center_grad_dev, float* quat_grad_dev,
                                 float* torsion_grad_dev, void* stream);

/* ------------------------------------------------------- Monte-Carlo search */

/* Constants of one Monte-Carlo search (monte_carlo_searcher, searcher.h:29-41 and the
 * search() arguments, entrance.cpp:318-330). pxd_mc_defaults() gives the reference's. */
typedef struct pxd_mc_params {
    uint32_t seed;                 /* walker w draws from mt19937(seed + w) */
    int32_t max_nsteps;            /* 200 */
    int32_t relax_nsteps;          /* 40: L-BFGS iterations after each move */
    int32_t full_nsteps;           /* 240: L-BFGS iterations of a full relaxation */
    double mc_mmenergy_threshold;  /* -1: no pruning on the pre-relaxation energy */
    double amplitude;              /* 2 A: translation radius and rotation scale */
    double temperature;            /* 1.2: Metropolis temperature on the pose score */
    double box_lo[3], box_hi[3];   /* search box (grid box, or the set_box box) */
    pxd_lbfgs_params lbfgs;        /* optimiser constants (history, tolerances, ...) */
} pxd_mc_params;

void pxd_mc_defaults(pxd_mc_params* out);

/* Runs n_walkers Monte-Carlo walkers in one persistent launch, one warp per walker:
 * random start (walker != 0), full relaxation, then max_nsteps moves of translation /
 * rotation / one torsion, each relaxed, scored by the pose-selection score and accepted
 * by Metropolis; a new best is fully relaxed again (searcher.cpp:46-223).
 *   ligand_ids_dev [W] int32, walker_ids_dev [W] int32 (the reference's pose_id: seeds
 *   the walker's generator; walker 0 only relaxes its start pose),
 *   first_pose_dev [W] int32 (1: the start is the ligand file's first pose, so torsions
 *   are randomised too), start_xyz_dev [W][max_atoms][3] float.
 *   Outputs: best pose xyz [W][max_atoms][3], receptor torsions [W][R], MM energy,
 *   pose score (double), evaluations and a status (0 ok, 1 crashed: coordinates beyond
 *   1e8 after the first relaxation, 2 relaxed start outside the box: no moves).
 *   global_min_dev [n_ligands] double (in/out) holds the pruning minimum per ligand;
 *   may be NULL when mc_mmenergy_threshold <= 0. */
int pxd_mc_search_dev(pxd_context* ctx, const pxd_mc_params* params, int32_t n_walkers,
                      int32_t max_atoms, const int32_t* ligand_ids_dev,
                      const int32_t* walker_ids_dev, const int32_t* first_pose_dev,
                      const float* start_xyz_dev, float* out_xyz_dev, float* out_tors_dev,
                      double* out_energy_dev, double* out_pscore_dev, int32_t* out_nevals_dev,
                      int32_t* out_status_dev, double* global_min_dev, void* stream);

/* Host-buffer version for the walkers of one ligand (double in / out). */
int pxd_mc_search(pxd_context* ctx, const pxd_mc_params* params, int32_t ligand_id,
                  int32_t n_walkers, const int32_t* walker_ids, const int32_t* first_pose,
                  const double* start_xyz, double* out_xyz, double* out_tors, double* out_energy,
                  double* out_pscore, int32_t* out_nevals, int32_t* out_status);

/* Host-buffer version over walkers of several ligands in one launch (the engine's
 * search over a whole ligand index). start / out xyz [n][max_atoms][3]; out_tors
 * [n][R]; global_min [n_ligands] (in/out, may be NULL: every ligand starts at 1e8,
 * the reference's minimum_pre_opt_energy). */
int pxd_mc_search_multi(pxd_context* ctx, const pxd_mc_params* params, int32_t n_walkers,
                        int32_t max_atoms, const int32_t* ligand_ids, const int32_t* walker_ids,
                        const int32_t* first_pose, const double* start_xyz, double* out_xyz,
                        double* out_tors, double* out_energy, double* out_pscore,
                        int32_t* out_nevals, int32_t* out_status, double* global_min);

/* Draws of the walker generator as the reference's random_generator makes them
 * (mt19937 + libstdc++ distributions, random.h:33-63), for checking the device stream:
 * kinds[i] = 0 uniform_int(0, ints[i]), 1 uniform_torsion, 2 uniform_real(0, 1),
 * 3 random_in_sphere (3 values), 4 random_orientation (4 values). out gets the values
 * in order. */
int pxd_rng_draws(pxd_context* ctx, uint32_t seed, int32_t n, const int32_t* kinds,
                  const int32_t* ints, double* out);

/* L2 residency of the maps (no reference counterpart; the loop it serves is
 * receptor_cache::get, grid.cpp:197-303). Sets aside `fraction` (0..1) of the device's
 * persisting-L2 capacity for this process and marks the context's map records as a
 * persisting access-policy window on its optimiser and search launches; 0 turns it off.
 * The set-aside is restored when the last context holding one turns it off or is
 * destroyed, and ends with the process. Results are unchanged: only caching differs. */
int pxd_set_l2_residency(pxd_context* ctx, double fraction);

/* Measurement probe (no reference counterpart): the bandwidth of random 16-byte gathers
 * -- the access pattern of the map lookups inside receptor_cache::get (grid.cpp:273-303)
 * as the kernels make it -- over a working set of working_set_bytes (rounded down to a
 * power of two) on `device`, in GB/s of bytes loaded, median of `reps` timed launches.
 * Below the L2 size it gives the L2 gather roofline of the batched kernels whose maps
 * stay L2-resident. Allocates and frees its own buffers. */
int pxd_gather_bandwidth(int32_t device, int64_t working_set_bytes, int32_t reps, double* gbs);

/* ------------------------------------------------------------ engine facade */

/* bytedock::ReusableEngine (engine/include/bytedock/core/entrance.h:30-74) over this
 * library: the same methods, argument meanings and defaults, files in and files out
 * in the reference's formats (engine/src/core/writer.cpp:40-230). Every call returns
 * PXD_OK or an error whose message pxd_engine_last_error gives (the reference's
 * exception texts: "Please call `set_box(...)` first!", ...). pxd_engine_create's own
 * failure is reported by pxd_engine_last_error(NULL). An empty sf_file selects the
 * default scoring function shipped beside the library (data/scoring_function.json). */
typedef struct pxd_engine pxd_engine;

int pxd_engine_create(const char* receptor_file, const char* sf_file, int32_t cpu_nthreads,
                      int32_t device, pxd_engine** out);
void pxd_engine_destroy(pxd_engine* engine);
const char* pxd_engine_last_error(const pxd_engine* engine);
int pxd_engine_set_box(pxd_engine* engine, double center_x, double center_y, double center_z,
                       double size_x, double size_y, double size_z);
int pxd_engine_generate_maps(pxd_engine* engine, double grid_spacing, double max_size);
/* map cache in this library's format: grid.json + one FP32 record file per map */
int pxd_engine_dump_maps(pxd_engine* engine, const char* cache_dir);
int pxd_engine_load_maps(pxd_engine* engine, const char* cache_dir);
int pxd_engine_drop_maps(pxd_engine* engine);
/* evaluate: pscore / bscore of every pose of every ligand in the index -> CSV file */
int pxd_engine_evaluate(pxd_engine* engine, const char* ligand_index_file, const char* output_file);
/* optimize: L-BFGS of every pose (max_niters, slope), pose_ranker output per ligand */
int pxd_engine_optimize(pxd_engine* engine, const char* ligand_index_file, const char* output_dir,
                        int32_t max_niters, double slope);
/* Variables of optimize's L-BFGS for this engine's later optimize calls (no reference
 * counterpart): PXD_DOF_CARTESIAN (default, the reference's) or PXD_DOF_RIGID_TORSION. */
int pxd_engine_set_dof_mode(pxd_engine* engine, int32_t dof_mode);
/* search: exhaustiveness Monte-Carlo walkers per ligand, pose_cluster output per ligand */
int pxd_engine_search(pxd_engine* engine, const char* ligand_index_file, const char* output_dir,
                      int32_t seed, int32_t exhaustiveness, int32_t max_nsteps, int32_t relax_nsteps,
                      int32_t num_modes, double min_rmsd, double mc_mmenergy_threshold, double slope);
/* setup_global_logging (entrance.cpp:51-54): "-" = standard error; verbosity 0..2 */
int pxd_engine_log2file(const char* log_file, int32_t verbosity);

/* The engine's writer and clustering alone (host only, no device needed):
 * pose_writer::consume for n_poses poses (torsions [n][n_rotors] in receptor-leaf order,
 * written in rotatable-bond order through bond_mappings), and pose_cluster::preprocess
 * (kept receives the indices of the kept poses, best first). */
int pxd_write_poses(const char* path, const char* smiles, int32_t best_id, double bscore,
                    int32_t n_poses, int32_t n_atoms, const int32_t* offsets, const double* energy,
                    const double* pscore, const int64_t* nevals, int32_t n_rotors,
                    const double* torsions, const double* xyz, const int32_t* bond_mappings,
                    int32_t num_rotatable_bonds);
/* pose_cluster::preprocess (writer.cpp:99-177) for many ligands in one launch, one warp per
 * ligand: group g's candidates are poses group_start[g] .. group_start[g + 1] - 1 of xyz
 * ([poses][stride_atoms][3]), of which the first group_atoms[g] atoms count. kept
 * ([n_groups][num_modes]) receives each group's kept pose indices, best pose score first,
 * -1 past n_kept[g]; num_modes at most 32. The kept lists are those of pxd_cluster_poses.
 * The _dev form takes device buffers on `stream`; the _batch form host buffers (xyz as
 * double, FP32-representable as search outputs are). */
int pxd_cluster_poses_dev(pxd_context* ctx, int32_t n_groups, const int32_t* group_start,
                          const int32_t* group_atoms, int32_t stride_atoms, const float* xyz,
                          const double* pscore, const int32_t* nevals, int32_t num_modes, double min_rmsd,
                          int32_t* kept, int32_t* n_kept, void* stream);
int pxd_cluster_poses_batch(pxd_context* ctx, int32_t n_groups, const int32_t* group_start,
                            const int32_t* group_atoms, int32_t stride_atoms, const double* xyz,
                            const double* pscore, const int32_t* nevals, int32_t num_modes, double min_rmsd,
                            int32_t* kept, int32_t* n_kept);
int pxd_cluster_poses(int32_t n_poses, int32_t n_atoms, const double* xyz, const double* pscore,
                      const int64_t* nevals, int32_t num_modes, double min_rmsd, int32_t* kept,
                      int32_t* n_kept);

#ifdef __cplusplus
}
#endif

#endif /* PXDOCK_GB300_H_ */
