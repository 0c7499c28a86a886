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

#define PXD_ABI_VERSION 1

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
} pxd_lbfgs_params;

#define PXD_MAX_HISTORY 128
#define PXD_NUM_VDW_TYPES 99
#define PXD_MAX_LIGAND_ATOMS 256
#define PXD_MAX_RECEPTOR_TORSIONS 64

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

/* Host-buffer version for one ligand: copies in, runs, copies out (double). */
int pxd_lbfgs(pxd_context* ctx, const pxd_lbfgs_params* params, int32_t ligand_id,
              int32_t n_poses, double* lig_xyz, double* rec_tors, double* energy,
              int32_t* nevals, int32_t* status);

/* Forward torsion-tree kinematics of a batch: replaces free_ligand::apply_parameters
 * (data.cpp:592-641). For pose p: centre [3], rotation matrix rot [9] row-major,
 * torsions [n_torsions] (pre-order), applied to the reference pose xyz_in. */
int pxd_ligand_kinematics(pxd_context* ctx, int32_t ligand_id, int32_t n_poses,
                          const double* xyz_in, const double* centers, const double* rots,
                          const double* torsions, double* xyz_out);

/* Receptor rotor kinematics: replaces torsional_receptor::apply_parameters
 * (data.cpp:366-385). out: [n_poses][n_atoms][3]. */
int pxd_receptor_kinematics(pxd_context* ctx, int32_t n_poses, const double* torsions,
                            double* xyz_out);

#ifdef __cplusplus
}
#endif

#endif /* PXDOCK_GB300_H_ */
