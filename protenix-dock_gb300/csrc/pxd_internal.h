// Internal host/device declarations of the GB300 docking library.
//
// Device layout (all FP32 unless noted; one allocation per ligand / receptor):
//   maps      float4 [n_slots][P]   {E, dE/dx, dE/dy, dE/dz}, k fastest; slot 0 = Coulomb
//   ligand    term lists reordered into "rounds" of 32 slots in which no atom occurs
//             twice, so that the 32 lanes of a warp add gradients to distinct atoms;
//             unused slots carry atom index -1 and are skipped.
//   receptor  explicit-pair atoms (rotor atoms when maps exist, every atom otherwise),
//             rotor tables, and the receptor intra terms that touch a rotor atom over a
//             compact local atom space [rotor atoms | fixed atoms they reference].
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/pxdock_gb300.h"

namespace pxd {

constexpr int kWarp = 32;
constexpr int kMaxDihTerms = 6;

// Molecule terms on the device (ligand, or the receptor's rotor-touching terms).
struct DevTopo {
    int n_atoms;
    int n_bond_slots, n_angle_slots, n_dih_slots, n_pair_slots;  // multiples of 32
    const int2* bond_ij;      // -1 = empty slot
    const float2* bond_p;     // k, r0
    const int4* angle_ijk;    // i, j (vertex), k, -
    const float2* angle_p;    // k, theta0
    const int4* dih_ijkl;
    const int2* dih_terms;    // first term, number of terms
    const float4* dih_term;   // k, periodicity, phase, -
    const int2* pair_ij;
    const float4* pair_p;     // A = 332.06 qi qj s_c, C = 4 sqrt(ei ej) s_v, S2 = ((si+sj)/2)^2
    // the same parameters in FP64, slot for slot, for the final FP64 energy (energy64.cuh)
    const double2* bond_p64;
    const double2* angle_p64;
    const double4* dih_term64;
    const double4* pair_p64;
};

struct DevSf {
    float coef[PXD_NUM_TERMS];
    float vdw_scale, vdw_cutoff;
    float2 vdw_type[PXD_NUM_VDW_TYPES];  // scaled sigma, epsilon per ligand type
    float vdw_sigma_raw[PXD_NUM_VDW_TYPES];  // unscaled sigma (hydrophobic thresholds)
    float ionic_coef[2], ionic[2][2];
    float picat_coef[4], picat[4][2];
    float stack_coef[2][4], stack[2][4][6];
    float hbond_scale, hbond_coef[8], hbond[8][6];
    float hydro_scale, hydro_min, hydro_max, hydro_factor;
};

struct DevRecScore {
    int has;
    int n_all;
    const float4* all_xyzq;    // every receptor atom: position, charge
    const float2* all_se;      // sigma, epsilon
    const int* all_local;      // rotor-atom local index or -1
    int n_hyd, n_cat, n_an, n_r5, n_r6, n_donc, n_donn, n_accc, n_accn;
    const int* hyd;
    const int* cat;
    const int* an;
    const float4* r5c;         // ring centroid
    const float4* r5n;         // ring normal
    const float4* r6c;
    const float4* r6n;
    const int2* donc;
    const int2* donn;
    const int* accc;
    const int* accn;
    const int* pclass;         // [n_all] pair-table class (C N O other: 0-3), -1 none; NULL: no table term
    const float4* pair_rec;    // [n_all] sigma, sqrt(epsilon), pair-table class, rotor local index (int bits)
};

struct DevLigScore {
    int has;
    int n_hyd, n_cat, n_an, n_r5, n_r6, n_donc, n_donn, n_accc, n_accn, n_ts, n_rot;
    const int* hyd;
    const int* cat;
    const int* an;
    const int* r5;             // [n][6], -1 padded
    const int* r6;
    const int2* donc;
    const int2* donn;
    const int* accc;
    const int* accn;
    const float4* ts_coef;     // torsion-strain coefficients
    const int2* ts_range;      // quads [first, first + count)
    const int4* ts_quad;
    const int* pclass;         // [N] 4 * pair-table class (C N O S P F Cl other), -1 none; NULL: no table term
};

struct DevLigand {
    DevTopo topo;
    DevLigScore score;        // interaction lists (score.has == 0: not scorable)
    int n_atoms;
    const float* charge;      // [N]
    const int* map_slot;      // [N] vdW map slot of the atom's type (-1: no map)
    const float2* se;         // [N] sigma, epsilon (explicit inter pairs)
    const double* charge64;   // [N] FP64 copies for the final FP64 energy
    const double2* se64;      // [N]
    const int* type;          // [N] ligand vdW type
    // torsion tree (forward kinematics, data.cpp:592-641)
    int n_frags, n_tors;
    const int* perm;          // [N]
    const int* frag_range;    // [2*F]
    const int4* tors;         // [T] frag, parent frag, parent atom, mine atom (positions)
    const int* is_root;       // [F]
    const int* frag_of;       // [N] fragment of each permuted position
    const int* frag_mine;     // [F] bond atom of the fragment (-1 for roots)
    const int* frag_parent;   // [F] parent fragment (-1 for roots)
};

struct DevReceptor {
    int n_explicit;           // atoms paired explicitly with every ligand atom
    const float4* ex_xyzq;    // fixed position, charge
    const float2* ex_se;      // sigma, epsilon
    const int* ex_local;      // local index of a rotor atom (< n_mov) or -1 if fixed
    int n_rotors, n_mov, n_local;
    const float4* rotor_origin;   // [R]
    const float4* rotor_axis;     // [R] unit
    const int* rotor_mov;         // [R+1] rotor atoms are local [rotor_mov[r], rotor_mov[r+1])
    const float4* local_xyz0;     // [n_local] input coordinates (rotor atoms: x0 - origin)
    // FP64 copies for the final FP64 energy
    const double4* ex_xyzq64;
    const double2* ex_se64;
    const double4* rotor_origin64;
    const double4* rotor_axis64;
    const double4* local_xyz064;  // w: rotor id as a double (rotor atoms)
    DevTopo intra;                // rotor-touching receptor terms over local atoms
    double e_const;               // energy of the receptor terms that touch no rotor atom
};

struct DevGrid {
    int has_grid;
    float3 init;
    // box faces as FP32 hi + lo pairs (init and init + (npoints - 1) * spacing), so
    // that the distance of an atom beyond a face is formed exactly near the face
    float3 lo_h, lo_l, hi_h, hi_l;
    int3 npts;                // points per axis
    float spacing, spacing_inv;
    float slope;
    int P;
    const float4* maps;
    // the final FP64 energy: box geometry and slope in FP64, and per map point the FP64
    // energy's residual below its FP32 record, E = maps[.].x + e_lo[.]
    double3 init64;
    double spacing64, slope64;
    const float* e_lo;        // [n_slots][P]
};

// Flat DOF layout of a pose: [ligand xyz (3N) | receptor torsions (T_r)] (optimizer.cpp:56-76)
struct HostTopoBuffers;

struct LigandEntry {
    DevLigand dev;
    void* mem = nullptr;      // single device allocation
    int n_atoms = 0;
    int n_tors = 0;
    std::vector<int32_t> types;
    void* score_mem = nullptr;                // interaction lists allocation
    std::vector<double> charge;               // FP64 copies for the GB/SA term
    std::vector<double> gb_radius, gb_screen;
};

}  // namespace pxd

struct pxd_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    // side streams and events for the concurrent size-class launches of the batched
    // optimiser (created on first use)
    cudaStream_t class_streams[8] = {};
    cudaEvent_t class_events[9] = {};
    std::string error;
    int n_sm = 0;
    // receptor
    bool has_receptor = false;
    int n_rec = 0;
    std::vector<double> rec_xyz;          // [M][3]
    std::vector<double> rec_charge, rec_sigma, rec_epsilon;
    std::vector<int> mov_atoms;           // rotor atoms (axis atom removed), grouped by rotor
    std::vector<int> mov_rotor;
    std::vector<int> rotor_mov_off;       // [R+1]
    std::vector<double> rotor_origin, rotor_axis;
    std::vector<uint8_t> is_mov;
    pxd::DevReceptor rec{};
    void* rec_mem = nullptr;
    void* rec_ex_all = nullptr;           // explicit list with every receptor atom (no maps)
    void* rec_ex_mov = nullptr;           // explicit list with rotor atoms (maps present)
    int n_ex_all = 0, n_ex_mov = 0;
    size_t ex_all_off[5] = {0, 0, 0, 0, 0}, ex_mov_off[5] = {0, 0, 0, 0, 0};
    // maps
    pxd::DevGrid grid{};
    pxd_box box{};
    double slope = 0.0;
    float4* maps = nullptr;
    int type_slot[PXD_NUM_VDW_TYPES];
    int n_slots = 0;
    // ligands
    std::vector<pxd::LigandEntry> ligands;
    pxd::DevLigand* d_ligands = nullptr;  // device copy of every entry's DevLigand
    int d_ligands_cap = 0;
    bool ligands_dirty = true;
    // empirical scores
    pxd::DevRecScore rec_score{};
    void* rec_score_mem = nullptr;
    std::vector<double> rec_gb_radius, rec_gb_screen;
    pxd::DevSf* d_sf[2] = {nullptr, nullptr};
    pxd_sf_params sf_host[2];
    bool sf_set[2] = {false, false};
    // autotuned L-BFGS variant (minimum resident blocks per SM) per size-class bound
    std::map<int, int> lbfgs_tuned;
    // L2 residency of the maps (pxd_set_l2_residency): persisting set-aside this context
    // holds (0: off) and the device's largest access-policy window
    size_t l2_setaside = 0;
    size_t l2_max_window = 0;
    // scratch
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    int* d_counter = nullptr;
};

namespace pxd {

int set_error(pxd_context* ctx, int code, const std::string& msg);
int cuda_check(pxd_context* ctx, cudaError_t e, const char* what);
// Raises kernel fn's dynamic shared-memory limit on the context's device to at least
// `bytes`, never lowering it. The limit is a process-wide property of the kernel: a
// launcher on another thread that set a larger limit for its own launch must not see it
// lowered between its attribute call and its launch.
int raise_smem_limit(pxd_context* ctx, const void* fn, size_t bytes, const char* what);
int ensure_scratch(pxd_context* ctx, size_t bytes);
int sync_ligand_table(pxd_context* ctx);
int refresh_ligand_slots(pxd_context* ctx);

// Size classes of a batch (lbfgs.cu): poses are sorted on the device by the atom count of
// their ligand into classes of capacity 32, 64, ..., 256 atoms, and each class runs its own
// persistent launch, with per-warp slices sized for its capacity, concurrently on the
// context's class streams.
constexpr int kSizeClasses = 8;
// Capacities (ascending, the last = max_atoms) of the classes that the context's ligands
// fall in; one class when there is only one or the batch is smaller than 1,024 items.
std::vector<int> size_class_caps(const pxd_context* ctx, int max_atoms, int n_items);
// Ints of class scratch for n_cls classes over n_items: counters [n_cls], counts [n_cls],
// lists [n_cls][n_items].
size_t size_class_ints(size_t n_cls, int n_items);
// Zeroes the counters and counts and lists every item under its class, on stream s.
int launch_size_classes(pxd_context* ctx, int n_items, const int* lig_ids, const std::vector<int>& caps,
                        int* scratch, cudaStream_t s);
// Fork: the class streams wait for what s has queued. Join: s waits for class k's stream.
int class_fork(pxd_context* ctx, size_t n_cls, cudaStream_t s);
int class_join(pxd_context* ctx, size_t k, cudaStream_t s);

// L2 residency (residency.cu): the access-policy window over the context's map records
// when residency control is on (*on false otherwise), and the release of its set-aside.
cudaLaunchAttribute map_window(const pxd_context* ctx, bool* on);
int release_l2_residency(pxd_context* ctx);

// Launches kern<<<grid, block, smem, s>>>(args) with the map window attached when the
// context has residency control on; a plain launch otherwise.
template <class... KArgs, class... Args>
cudaError_t launch_with_map_window(const pxd_context* ctx, void (*kern)(KArgs...), dim3 grid, dim3 block,
                                   size_t smem, cudaStream_t s, Args&&... args) {
    bool on = false;
    cudaLaunchAttribute attr = map_window(ctx, &on);
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = on ? &attr : nullptr;
    cfg.numAttrs = on ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

// kernels (launchers), one per translation unit
int launch_grid_build(pxd_context* ctx, const float4* atoms_xyzq, const float4* atoms_lo,
                      const float2* atoms_se, const double2* atoms_se64, int n_atoms, const int* slot_types,
                      int n_slots, float4* maps, float* e_lo);
int launch_score(pxd_context* ctx, int n_poses, int max_atoms, const int* lig_ids,
                 const float* xyz, const float* tors, double* energy, float* lig_grad,
                 float* tors_grad, cudaStream_t s);
int launch_lbfgs(pxd_context* ctx, const pxd_lbfgs_params& p, int n_poses, int max_atoms,
                 const int* lig_ids, float* xyz, float* tors, double* energy, int* nevals,
                 int* status, cudaStream_t s);
int launch_lbfgs_noalloc(pxd_context* ctx, const pxd_lbfgs_params& p, int n_poses, int max_atoms,
                         const int* lig_ids, float* xyz, float* tors, double* energy, int* nevals,
                         int* status, cudaStream_t s);
int launch_ligand_kinematics(pxd_context* ctx, int lig, int n_poses, const float* xyz_in,
                             const float* centers, const float* rots, const float* tors,
                             float* xyz_out, cudaStream_t s);
int launch_ligand_backward(pxd_context* ctx, int lig, int n_poses, const float* xyz, const float* centers,
                           const float* grad, float* out_center, float* out_torque, float* out_tors,
                           cudaStream_t s);
int launch_receptor_kinematics(pxd_context* ctx, int n_poses, const float* tors, float* out,
                               cudaStream_t s);
int launch_ligand_pose(pxd_context* ctx, int lig, int n_poses, const float* xyz_in, const float* centers,
                       const float* quats, const float* tors, float* xyz_out, cudaStream_t s);
int launch_ligand_pose_backward(pxd_context* ctx, int lig, int n_poses, const float* xyz, const float* centers,
                                const float* quats, const float* grad, float* out_center, float* out_quat,
                                float* out_tors, cudaStream_t s);
int pair_class(int is_receptor, int z);
int upload_receptor_scoring(pxd_context* ctx, const pxd_score_lists* l, const std::vector<int>& local_of);
int upload_ligand_scoring(pxd_context* ctx, LigandEntry& e, const pxd_score_lists* l);
void gbsa_properties(const pxd_score_lists* l, int n, std::vector<double>& radius,
                     std::vector<double>& screen);

// Host-buffer wrappers stage their arrays in stream-ordered device allocations.
// Queues one asynchronous copy unless an earlier step failed (*rc != 0), keeping the first
// failure in *rc and in the context's error string. Zero-byte copies are skipped.
inline void queue_copy(pxd_context* ctx, int* rc, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind,
                       cudaStream_t s, const char* what = "copy") {
    if (*rc || bytes == 0) return;
    *rc = cuda_check(ctx, cudaMemcpyAsync(dst, src, bytes, kind, s), what);
}

// Waits for the work queued on s, so that no host buffer is released while a copy into it
// is in flight, and returns the first failure: rc (a copy that failed to queue) before the
// stream's own.
inline int sync_copies(pxd_context* ctx, int rc, cudaStream_t s, const char* what) {
    const cudaError_t e = cudaStreamSynchronize(s);
    if (rc) return rc;
    return cuda_check(ctx, e, what);
}

struct Staging {
    pxd_context* ctx;
    std::vector<void*> dev;
    ~Staging() {
        for (void* p : dev) cudaFreeAsync(p, ctx->stream);
    }
    template <class T>
    T* alloc(size_t n, int* rc) {
        void* p = nullptr;
        *rc = cuda_check(ctx, cudaMallocAsync(&p, std::max<size_t>(n, 1) * sizeof(T), ctx->stream), "staging");
        if (!*rc) dev.push_back(p);
        return static_cast<T*>(p);
    }
};

}  // namespace pxd
