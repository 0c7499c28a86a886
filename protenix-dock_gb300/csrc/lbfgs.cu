// Persistent batched L-BFGS kernel (one warp per pose, dynamic pose queue) and the
// score+gradient kernel, with their launchers.
#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <type_traits>

#include "device_dof.cuh"
#include "device_lbfgs.cuh"

namespace pxd {

struct LbfgsArgs {
    EvalEnv env;
    const DevLigand* ligands;
    const int* lig_ids;
    int n_ligands;
    float* xyz;        // [P][stride_atoms][3]
    float* tors;       // [P][R]
    int max_atoms;     // shared-memory capacity of a warp (atoms)
    int stride_atoms;  // pose stride of xyz
    const int* order;     // optional: queue position -> pose (a size class)
    const int* count_dev; // optional: number of queue positions, on the device
    double* energy;
    int* nevals;
    int* status;
    int n_poses;
    int* counter;
    LbfgsConsts c;
    int n_local;       // receptor local atoms (smem sizing)
    int D_pad;         // padded vector length
    float* hist;       // per warp: S [m][D_pad], Y [m][D_pad]
    size_t hist_stride;
    int hist_smem;     // 1: the history lives in the warp's shared memory instead
    int X_pad;         // rigid-body + torsion variables: padded 3 * max_atoms + R (0: Cartesian)
};

constexpr int kWarpsPerBlock = 4;
constexpr int kDefaultMinBlocks = 5;  // measured best on GB300 for the 42-atom bench ligand (296.7k poses/s against 293.3k for 4)

// Floats of one warp's shared-memory slice: the evaluation buffers, the optimiser
// vectors and scalars, the history when it is held there, and for rigid-body + torsion
// variables (xp > 0) the forward-map frames, the input-frame relative coordinates and
// torsion axes, the placed pose, its Cartesian gradient and the evaluated variables.
__host__ __device__ inline int lbfgs_warp_floats(int cap, int n_local, int dp, int m, int hist_smem, int xp) {
    return pose_bufs_floats(cap, n_local) + kOptVecs * dp + opt_scalar_floats(m) +
           (hist_smem ? 2 * hist_slots(m) * dp : 0) + (xp > 0 ? kKinFloats + 4 * cap + 4 * kWarp + 2 * xp + dp : 0);
}

// kMinBlocks > 0 asks the compiler to fit that many blocks per SM (register cap);
// variants are chosen per launch (lbfgs_variant). kDof: the variables are rigid body +
// torsions (DofClosure) instead of Cartesian coordinates (Closure).
template <int kMinBlocks, bool kDof>
__global__ void __launch_bounds__(kWarpsPerBlock * kWarp, kMinBlocks > 0 ? kMinBlocks : 1)
    lbfgs_kernel(const __grid_constant__ LbfgsArgs a) {
    extern __shared__ __align__(16) float smem[];
    const int lane = threadIdx.x & (kWarp - 1);
    const int wib = threadIdx.x / kWarp;
    const int Dp = a.D_pad;
    const int per_warp = lbfgs_warp_floats(a.max_atoms, a.n_local, Dp, a.c.m, a.hist_smem, kDof ? a.X_pad : 0);
    float* base = smem + wib * per_warp;
    const PoseBufs b = carve_pose_bufs(base, a.max_atoms, a.n_local);
    float* vb = base + pose_bufs_floats(a.max_atoms, a.n_local);
    Vecs v = carve_vecs(vb, Dp, a.c.m);
    const size_t gw = static_cast<size_t>(blockIdx.x) * kWarpsPerBlock + wib;
    v.S = a.hist_smem ? vb + kOptVecs * Dp + opt_scalar_floats(a.c.m) : a.hist + gw * a.hist_stride;
    v.Y = v.S + static_cast<size_t>(hist_slots(a.c.m)) * Dp;
    const int R = a.env.rec.n_rotors;
    using Cl = typename std::conditional<kDof, DofClosure, Closure>::type;
    Cl c;
    c.env = &a.env;
    c.b = &b;
    c.lane = lane;
    if constexpr (kDof) {
        float* xb = vb + kOptVecs * Dp + opt_scalar_floats(a.c.m) + (a.hist_smem ? 2 * hist_slots(a.c.m) * Dp : 0);
        c.ks = reinterpret_cast<KinShared*>(xb);
        c.rel = reinterpret_cast<float4*>(xb + kKinFloats);
        c.axes = c.rel + a.max_atoms;
        c.xc = reinterpret_cast<float*>(c.axes + kWarp);
        c.gc = c.xc + a.X_pad;
        c.q = c.gc + a.X_pad;
    }
    const int n_queue = a.count_dev ? *a.count_dev : a.n_poses;
    while (true) {
        int k = 0;
        if (lane == 0) k = atomicAdd(a.counter, 1);
        k = __shfl_sync(kFull, k, 0);
        if (k >= n_queue) break;
        const int pose = a.order ? a.order[k] : k;
        const int lid = a.lig_ids[pose];
        if (lid < 0 || lid >= a.n_ligands || a.ligands[lid].n_atoms > a.max_atoms) {
            if (lane == 0) {
                a.status[pose] = PXD_POSE_BAD_INPUT;
                a.nevals[pose] = 0;
                a.energy[pose] = 0.0;
            }
            continue;
        }
        const DevLigand& L = a.ligands[lid];
        const int N = L.n_atoms;
        float* px = a.xyz + static_cast<size_t>(pose) * a.stride_atoms * 3;
        float* pt = a.tors + static_cast<size_t>(pose) * R;
        c.L = &L;
        double energy = 0.0;
        int st;
        if constexpr (kDof) {
            const int T = L.n_tors;
            if (T > kWarp || L.n_frags < 1 || L.n_frags > kMaxFrags || 7 + T + R > Dp || 3 * N + R > a.X_pad) {
                if (lane == 0) {
                    a.status[pose] = PXD_POSE_BAD_INPUT;
                    a.nevals[pose] = 0;
                    a.energy[pose] = 0.0;
                }
                continue;
            }
            // q0: the input's centre, the identity quaternion, no torsion change
            const int D = 7 + T + R;
            const float3 c0 = dof_prepare(c, px);
            for (int e = lane; e < D; e += kWarp)
                v.x[e] = e == 0 ? c0.x : e == 1 ? c0.y : e == 2 ? c0.z : e == 3 ? 1.f : e < 7 + T ? 0.f : pt[e - 7 - T];
            __syncwarp();
            st = lbfgs_pose<false, true>(c, a.c, v, D, Dp, lane, energy);
            // the final energy placed the returned variables: c.xc is the returned pose
            for (int e = lane; e < 3 * N; e += kWarp) px[e] = c.xc[e];
            for (int r = lane; r < R; r += kWarp) pt[r] = c.xc[3 * N + r];
        } else {
            const int D = 3 * N + R;
            for (int e = lane; e < 3 * N; e += kWarp) v.x[e] = px[e];
            for (int r = lane; r < R; r += kWarp) v.x[3 * N + r] = pt[r];
            __syncwarp();
            st = lbfgs_pose<false, true>(c, a.c, v, D, Dp, lane, energy);
            for (int e = lane; e < 3 * N; e += kWarp) px[e] = v.x[e];
            for (int r = lane; r < R; r += kWarp) pt[r] = v.x[3 * N + r];
        }
        if (lane == 0) {
            a.energy[pose] = energy;
            a.nevals[pose] = c.nevals;
            a.status[pose] = st;
        }
        __syncwarp();
    }
}

struct ScoreArgs {
    EvalEnv env;
    const DevLigand* ligands;
    const int* lig_ids;
    int n_ligands;
    const float* xyz;
    const float* tors;
    int max_atoms;
    double* energy;
    float* lig_grad;
    float* tors_grad;
    int n_poses;
    int n_local;
    int D_pad;
};

__global__ void __launch_bounds__(kWarpsPerBlock * kWarp) score_kernel(const __grid_constant__ ScoreArgs a) {
    extern __shared__ __align__(16) float smem[];
    const int lane = threadIdx.x & (kWarp - 1);
    const int wib = threadIdx.x / kWarp;
    const int per_warp = pose_bufs_floats(a.max_atoms, a.n_local) + 2 * a.D_pad;
    float* base = smem + wib * per_warp;
    const PoseBufs b = carve_pose_bufs(base, a.max_atoms, a.n_local);
    float* x = base + pose_bufs_floats(a.max_atoms, a.n_local);
    float* g = x + a.D_pad;
    const int R = a.env.rec.n_rotors;
    const int nw = gridDim.x * kWarpsPerBlock;
    for (int pose = blockIdx.x * kWarpsPerBlock + wib; pose < a.n_poses; pose += nw) {
        const int lid = a.lig_ids[pose];
        if (lid < 0 || lid >= a.n_ligands || a.ligands[lid].n_atoms > a.max_atoms) {
            if (lane == 0) a.energy[pose] = nan("");
            continue;
        }
        const DevLigand L = a.ligands[lid];
        const int N = L.n_atoms;
        const float* px = a.xyz + static_cast<size_t>(pose) * a.max_atoms * 3;
        for (int e = lane; e < 3 * N; e += kWarp) x[e] = px[e];
        for (int r = lane; r < R; r += kWarp) x[3 * N + r] = a.tors[static_cast<size_t>(pose) * R + r];
        __syncwarp();
        eval_pose_body(a.env, L, x, nullptr, 0.f, g, b, lane);
        float* og = a.lig_grad + static_cast<size_t>(pose) * a.max_atoms * 3;
        for (int k = lane; k < 3 * N; k += kWarp) og[k] = g[k];
        for (int r = lane; r < R; r += kWarp)
            a.tors_grad[static_cast<size_t>(pose) * R + r] = g[3 * N + r];
        // the energy is the FP64 objective, the gradient the FP32 one
        const double e = energy64(a.env, a.ligands[lid], x, b, lane);
        if (lane == 0) a.energy[pose] = e;
        __syncwarp();
    }
}

static EvalEnv make_env(pxd_context* ctx) {
    EvalEnv env;
    env.rec = ctx->rec;
    env.grid = ctx->grid;
    return env;
}

static int padded(int D) { return (D + kWarp - 1) / kWarp * kWarp; }

using LbfgsKernelFn = void (*)(LbfgsArgs);

// Variant of lbfgs_kernel: the low byte is the minimum resident blocks per SM (register
// cap; 0 = unconstrained), kHistSmem marks the history in shared memory.
constexpr int kHistSmem = PXD_LBFGS_HIST_SMEM;
static LbfgsKernelFn variant_fn(int variant) {
    switch (variant & 255) {
        case 3: return lbfgs_kernel<3, false>;
        case 4: return lbfgs_kernel<4, false>;
        case 5: return lbfgs_kernel<5, false>;
        case 6: return lbfgs_kernel<6, false>;
        default: return lbfgs_kernel<0, false>;
    }
}

// Rigid-body + torsion variables run one register budget, the default's, whatever the
// class's variant (its shared-memory history flag still applies).
static LbfgsKernelFn dof_kernel() { return lbfgs_kernel<kDefaultMinBlocks, true>; }

// Size class of a per-warp atom capacity: the smallest bound of 32, 64, ..., 256 it fits.
static int class_bound(int cap) { return std::min(256, (cap + 31) / 32 * 32); }

// The variant of a size class: the autotuner's choice for the class (pxd_lbfgs_autotune_dev),
// else PXD_LBFGS_MIN_BLOCKS (| kHistSmem when PXD_LBFGS_HIST_SMEM=1), else the default.
static int lbfgs_variant_id(const pxd_context* ctx, int cap) {
    auto it = ctx->lbfgs_tuned.find(class_bound(cap));
    if (it != ctx->lbfgs_tuned.end()) return it->second;
    static int choice = [] {
        const char* v = std::getenv("PXD_LBFGS_MIN_BLOCKS");
        const char* h = std::getenv("PXD_LBFGS_HIST_SMEM");
        return (v ? std::atoi(v) : kDefaultMinBlocks) | (h && std::atoi(h) ? kHistSmem : 0);
    }();
    return choice;
}
static LbfgsKernelFn lbfgs_variant(const pxd_context* ctx, int cap, bool dof) {
    return dof ? dof_kernel() : variant_fn(lbfgs_variant_id(ctx, cap));
}

// Padded length of the optimiser's vectors for ligands of up to `cap` atoms: 3 cap + R
// Cartesian, or 7 + T + R with T the most torsions of the context's ligands (at most 32;
// a ligand with more is a bad input of that mode).
static int vec_pad(const pxd_context* ctx, int cap, bool dof) {
    if (!dof) return padded(3 * cap + ctx->rec.n_rotors);
    int t = 0;
    for (auto& e : ctx->ligands) t = std::max(t, std::min(e.n_tors, kWarp));
    return padded(7 + t + ctx->rec.n_rotors);
}
static int dof_xpad(const pxd_context* ctx, int cap, bool dof) { return dof ? padded(3 * cap + ctx->rec.n_rotors) : 0; }

// Dynamic shared memory of one lbfgs_kernel block for ligands of up to `cap` atoms.
static size_t lbfgs_block_smem(const pxd_context* ctx, int cap, int history, bool hist_smem, bool dof) {
    return sizeof(float) * kWarpsPerBlock *
           lbfgs_warp_floats(cap, ctx->rec.n_local, vec_pad(ctx, cap, dof), history, hist_smem ? 1 : 0,
                             dof_xpad(ctx, cap, dof));
}

int launch_score(pxd_context* ctx, int n_poses, int max_atoms, const int* lig_ids,
                 const float* xyz, const float* tors, double* energy, float* lig_grad,
                 float* tors_grad, cudaStream_t s) {
    if (n_poses <= 0) return PXD_OK;
    int rc = sync_ligand_table(ctx);
    if (rc) return rc;
    ScoreArgs a{};
    a.env = make_env(ctx);
    a.ligands = ctx->d_ligands;
    a.lig_ids = lig_ids;
    a.n_ligands = static_cast<int>(ctx->ligands.size());
    a.xyz = xyz;
    a.tors = tors;
    a.max_atoms = max_atoms;
    a.energy = energy;
    a.lig_grad = lig_grad;
    a.tors_grad = tors_grad;
    a.n_poses = n_poses;
    a.n_local = ctx->rec.n_local;
    a.D_pad = padded(3 * max_atoms + ctx->rec.n_rotors);
    const size_t smem =
        sizeof(float) * kWarpsPerBlock * (pose_bufs_floats(max_atoms, a.n_local) + 2 * a.D_pad);
    if (smem > 48 * 1024) {
        rc = raise_smem_limit(ctx, reinterpret_cast<const void*>(score_kernel), smem, "score smem attribute");
        if (rc) return rc;
    }
    const int warps = (n_poses + 0);
    int blocks = (warps + kWarpsPerBlock - 1) / kWarpsPerBlock;
    const int cap = ctx->n_sm * 16;
    if (blocks > cap) blocks = cap;
    score_kernel<<<blocks, kWarpsPerBlock * kWarp, smem, s>>>(a);
    return cuda_check(ctx, cudaGetLastError(), "score_kernel launch");
}

// score_kernel over poses of several contexts (one receptor and map set each): pose p
// is ligand lig_ids[p] of context ctx_ids[p]; the per-warp buffers are sized for the
// largest ligand and rotor-atom set of the batch.
struct ScoreMultiArgs {
    const EvalEnv* envs;           // [n_ctx]
    const DevLigand* const* tabs;  // [n_ctx] device ligand tables
    const int* n_ligs;             // [n_ctx]
    const int* ctx_ids;
    const int* lig_ids;
    const float* xyz;
    const float* tors;             // [P][tors_stride]
    int tors_stride;
    int max_atoms;
    double* energy;
    float* lig_grad;
    float* tors_grad;
    int n_poses;
    int n_local;
    int D_pad;
};

__global__ void __launch_bounds__(kWarpsPerBlock * kWarp) score_multi_kernel(const __grid_constant__ ScoreMultiArgs a) {
    extern __shared__ __align__(16) float smem[];
    const int lane = threadIdx.x & (kWarp - 1);
    const int wib = threadIdx.x / kWarp;
    const int per_warp = pose_bufs_floats(a.max_atoms, a.n_local) + 2 * a.D_pad;
    float* base = smem + wib * per_warp;
    const PoseBufs b = carve_pose_bufs(base, a.max_atoms, a.n_local);
    float* x = base + pose_bufs_floats(a.max_atoms, a.n_local);
    float* g = x + a.D_pad;
    const int nw = gridDim.x * kWarpsPerBlock;
    for (int pose = blockIdx.x * kWarpsPerBlock + wib; pose < a.n_poses; pose += nw) {
        const int c = a.ctx_ids[pose];
        const int lid = a.lig_ids[pose];
        if (lid < 0 || lid >= a.n_ligs[c] || a.tabs[c][lid].n_atoms > a.max_atoms) {
            if (lane == 0) a.energy[pose] = nan("");
            continue;
        }
        const EvalEnv& env = a.envs[c];
        const DevLigand L = a.tabs[c][lid];
        const int N = L.n_atoms;
        const int R = env.rec.n_rotors;
        const float* px = a.xyz + static_cast<size_t>(pose) * a.max_atoms * 3;
        for (int e = lane; e < 3 * N; e += kWarp) x[e] = px[e];
        for (int r = lane; r < R; r += kWarp) x[3 * N + r] = a.tors[static_cast<size_t>(pose) * a.tors_stride + r];
        __syncwarp();
        eval_pose_body(env, L, x, nullptr, 0.f, g, b, lane);
        float* og = a.lig_grad + static_cast<size_t>(pose) * a.max_atoms * 3;
        for (int k = lane; k < 3 * a.max_atoms; k += kWarp) og[k] = k < 3 * N ? g[k] : 0.f;
        for (int r = lane; r < R; r += kWarp)
            a.tors_grad[static_cast<size_t>(pose) * a.tors_stride + r] = g[3 * N + r];
        // the energy is the FP64 objective, the gradient the FP32 one (as score_kernel)
        const double e = energy64(env, a.tabs[c][lid], x, b, lane);
        if (lane == 0) a.energy[pose] = e;
        __syncwarp();
    }
}

// Size classes of the batched launch: poses are grouped by their ligand's atom count so
// that each persistent launch sizes its per-warp shared memory (and so its residency)
// for its own class instead of the largest ligand of the batch.
constexpr int kClassBound[kSizeClasses] = {32, 64, 96, 128, 160, 192, 224, 256};

struct ClassArgs {
    const int* lig_ids;
    const DevLigand* ligands;
    int n_ligands, n_poses, n_classes;
    int bound[kSizeClasses];  // atom capacity of each class, ascending
    int* counts;              // [n_classes]
    int* lists;               // [n_classes][n_poses]
};

// One thread per pose: appends the pose to the first class that holds its ligand (an
// invalid ligand id or an oversize ligand goes to the last class, whose launch flags it).
__global__ void size_class_kernel(const ClassArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n_poses) return;
    const int lid = a.lig_ids[i];
    int c = a.n_classes - 1;
    if (lid >= 0 && lid < a.n_ligands) {
        const int n = a.ligands[lid].n_atoms;
        for (int k = 0; k < a.n_classes; ++k)
            if (n <= a.bound[k]) {
                c = k;
                break;
            }
    }
    const int pos = atomicAdd(&a.counts[c], 1);
    a.lists[static_cast<size_t>(c) * a.n_poses + pos] = i;
}

std::vector<int> size_class_caps(const pxd_context* ctx, int max_atoms, int n_items) {
    std::vector<int> caps;
    for (int k = 0; k < kSizeClasses; ++k) {
        const int cap = std::min(kClassBound[k], max_atoms);
        bool used = false;
        for (auto& e : ctx->ligands) used = used || (e.n_atoms <= cap && (k == 0 || e.n_atoms > kClassBound[k - 1]));
        if (used && (caps.empty() || caps.back() != cap)) caps.push_back(cap);
        if (cap == max_atoms) break;
    }
    if (caps.empty() || caps.back() != max_atoms) caps.push_back(max_atoms);  // oversize / invalid ids
    if (caps.size() > 1 && n_items < 1024) caps.assign(1, max_atoms);
    return caps;
}

size_t size_class_ints(size_t n_cls, int n_items) { return 2 * n_cls + n_cls * static_cast<size_t>(n_items); }

int launch_size_classes(pxd_context* ctx, int n_items, const int* lig_ids, const std::vector<int>& caps,
                        int* scratch, cudaStream_t s) {
    const size_t n_cls = caps.size();
    ClassArgs ca{};
    ca.lig_ids = lig_ids;
    ca.ligands = ctx->d_ligands;
    ca.n_ligands = static_cast<int>(ctx->ligands.size());
    ca.n_poses = n_items;
    ca.n_classes = static_cast<int>(n_cls);
    for (size_t k = 0; k < n_cls; ++k) ca.bound[k] = caps[k];
    ca.counts = scratch + n_cls;
    ca.lists = scratch + 2 * n_cls;
    int rc = cuda_check(ctx, cudaMemsetAsync(scratch, 0, sizeof(int) * 2 * n_cls, s), "class counters");
    if (rc) return rc;
    size_class_kernel<<<(n_items + 255) / 256, 256, 0, s>>>(ca);
    return cuda_check(ctx, cudaGetLastError(), "size_class_kernel launch");
}

int class_fork(pxd_context* ctx, size_t n_cls, cudaStream_t s) {
    for (size_t k = 0; k <= n_cls; ++k) {
        if (k < n_cls && !ctx->class_streams[k]) {
            int rc = cuda_check(ctx, cudaStreamCreateWithFlags(&ctx->class_streams[k], cudaStreamNonBlocking),
                                "class stream");
            if (rc) return rc;
        }
        if (!ctx->class_events[k]) {
            int rc = cuda_check(ctx, cudaEventCreateWithFlags(&ctx->class_events[k], cudaEventDisableTiming),
                                "class event");
            if (rc) return rc;
        }
    }
    int rc = cuda_check(ctx, cudaEventRecord(ctx->class_events[n_cls], s), "fork");
    for (size_t k = 0; k < n_cls && !rc; ++k)
        rc = cuda_check(ctx, cudaStreamWaitEvent(ctx->class_streams[k], ctx->class_events[n_cls], 0), "fork wait");
    return rc;
}

int class_join(pxd_context* ctx, size_t k, cudaStream_t s) {
    int rc = cuda_check(ctx, cudaEventRecord(ctx->class_events[k], ctx->class_streams[k]), "join record");
    if (!rc) rc = cuda_check(ctx, cudaStreamWaitEvent(s, ctx->class_events[k], 0), "join wait");
    return rc;
}

static void fill_consts(LbfgsArgs& a, const pxd_lbfgs_params& p) {
    a.c.max_iter = p.max_iter;
    a.c.max_eval = p.max_eval;
    a.c.m = p.history;
    a.c.ls_max = p.ls_max;
    a.c.lr = p.lr;
    a.c.tol_grad = p.tolerance_grad;
    a.c.tol_change = p.tolerance_change;
    a.c.c1 = p.ls_c1;
    a.c.c2 = p.ls_c2;
    a.c.ls_tol_change = p.ls_tolerance_change;
    a.c.gtd_threshold = p.ls_gtd_threshold;
    a.c.reset = p.reset_threshold;
}

int launch_lbfgs(pxd_context* ctx, const pxd_lbfgs_params& p, int n_poses, int max_atoms,
                 const int* lig_ids, float* xyz, float* tors, double* energy, int* nevals,
                 int* status, cudaStream_t s) {
    if (n_poses <= 0) return PXD_OK;
    int rc = sync_ligand_table(ctx);
    if (rc) return rc;
    LbfgsArgs base{};
    base.env = make_env(ctx);
    base.ligands = ctx->d_ligands;
    base.lig_ids = lig_ids;
    base.n_ligands = static_cast<int>(ctx->ligands.size());
    base.xyz = xyz;
    base.tors = tors;
    base.stride_atoms = max_atoms;
    base.energy = energy;
    base.nevals = nevals;
    base.status = status;
    base.n_poses = n_poses;
    base.order = nullptr;
    base.count_dev = nullptr;
    base.hist_smem = 0;
    fill_consts(base, p);
    base.n_local = ctx->rec.n_local;
    const std::vector<int> caps = size_class_caps(ctx, max_atoms, n_poses);
    const bool classes = caps.size() > 1;
    struct Plan {
        int cap, dp, xp, blocks, hist_smem;
        size_t smem, stride;
        LbfgsKernelFn kern;
    };
    std::vector<Plan> plan;
    size_t hist_floats = 0;
    int smem_limit = 0;
    rc = cuda_check(ctx, cudaDeviceGetAttribute(&smem_limit, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device),
                    "shared memory limit");
    if (rc) return rc;
    const bool dof = p.dof_mode == PXD_DOF_RIGID_TORSION;
    for (int cap : caps) {
        Plan q;
        q.cap = cap;
        q.kern = lbfgs_variant(ctx, cap, dof);
        q.hist_smem = (lbfgs_variant_id(ctx, cap) & kHistSmem) ? 1 : 0;
        // a pinned shared-memory history that does not fit this class falls back to the slab
        if (q.hist_smem && lbfgs_block_smem(ctx, cap, p.history, true, dof) > static_cast<size_t>(smem_limit))
            q.hist_smem = 0;
        q.dp = vec_pad(ctx, cap, dof);
        q.xp = dof_xpad(ctx, cap, dof);
        q.smem = lbfgs_block_smem(ctx, cap, p.history, q.hist_smem, dof);
        q.stride = q.hist_smem ? 0 : static_cast<size_t>(2) * hist_slots(p.history) * q.dp;
        plan.push_back(q);
    }
    // classes may share a kernel variant with different slices: its dynamic shared-memory
    // limit is the largest of theirs, set before any occupancy query or launch
    std::map<LbfgsKernelFn, size_t> smem_of;
    for (const Plan& q : plan) smem_of[q.kern] = std::max(smem_of[q.kern], q.smem);
    for (const auto& [kern, bytes] : smem_of) {
        rc = raise_smem_limit(ctx, reinterpret_cast<const void*>(kern), bytes, "lbfgs smem attribute");
        if (rc) return rc;
    }
    for (Plan& q : plan) {
        int per_sm = 0;
        rc = cuda_check(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, q.kern, kWarpsPerBlock * kWarp,
                                                                          q.smem),
                        "lbfgs occupancy");
        if (rc) return rc;
        if (per_sm < 1) return set_error(ctx, PXD_ERR_INVALID, "ligand too large for shared memory");
        q.blocks = per_sm * ctx->n_sm;
        const int need = (n_poses + kWarpsPerBlock - 1) / kWarpsPerBlock;
        if (q.blocks > need) q.blocks = need;
    }
    // the class launches run concurrently, each on its own history slab
    std::vector<size_t> hist_off(plan.size());
    for (size_t k = 0; k < plan.size(); ++k) {
        hist_off[k] = hist_floats;
        hist_floats += (plan[k].stride * plan[k].blocks * kWarpsPerBlock + 63) / 64 * 64;
    }
    const size_t hist_bytes = (sizeof(float) * hist_floats + 255) / 256 * 256;
    const size_t n_cls = plan.size();
    const size_t class_bytes = classes ? sizeof(int) * size_class_ints(n_cls, n_poses) : 0;
    rc = ensure_scratch(ctx, hist_bytes + class_bytes);
    if (rc) return rc;
    float* hist = static_cast<float*>(ctx->scratch);
    int* counters = classes ? reinterpret_cast<int*>(static_cast<char*>(ctx->scratch) + hist_bytes) : ctx->d_counter;
    if (classes) {
        // class k runs on class stream k after the classification; s waits for all of them
        rc = launch_size_classes(ctx, n_poses, lig_ids, caps, counters, s);
        if (!rc) rc = class_fork(ctx, n_cls, s);
    } else {
        rc = cuda_check(ctx, cudaMemsetAsync(ctx->d_counter, 0, sizeof(int), s), "counter reset");
    }
    if (rc) return rc;
    for (size_t k = 0; k < n_cls; ++k) {
        LbfgsArgs a = base;
        a.max_atoms = plan[k].cap;
        a.D_pad = plan[k].dp;
        a.X_pad = plan[k].xp;
        a.hist = hist + hist_off[k];
        a.hist_stride = plan[k].stride;
        a.hist_smem = plan[k].hist_smem;
        a.counter = counters + k;
        cudaStream_t ks = s;
        if (classes) {
            a.count_dev = counters + n_cls + k;
            a.order = counters + 2 * n_cls + k * static_cast<size_t>(n_poses);
            ks = ctx->class_streams[k];
        }
        // A launch of at most one block per SM (a few poses, the plain per-pose calls) asks for
        // the smallest shared-memory carve-out that holds its block, so the rest of the SM's
        // memory serves as L1 for the map gathers, the history and the topology records; larger
        // launches keep the driver's choice. The preference is a property of the kernel, set
        // before each launch (a concurrent launch of the same variant can only see a different
        // preference, never an invalid one: the driver still fits the dynamic shared memory).
        int carveout = cudaSharedmemCarveoutDefault;
        if (plan[k].blocks <= ctx->n_sm) {
            int sm_smem = 0;
            rc = cuda_check(ctx, cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor,
                                                        ctx->device),
                            "shared memory per SM");
            if (rc) return rc;
            carveout = static_cast<int>(std::min<size_t>(100, (100 * (plan[k].smem + 1024) + sm_smem - 1) / sm_smem + 1));
        }
        rc = cuda_check(ctx, cudaFuncSetAttribute(plan[k].kern, cudaFuncAttributePreferredSharedMemoryCarveout, carveout),
                        "lbfgs carve-out");
        if (!rc)
            rc = cuda_check(ctx, launch_with_map_window(ctx, plan[k].kern, plan[k].blocks, kWarpsPerBlock * kWarp,
                                                        plan[k].smem, ks, a),
                            "lbfgs_kernel launch");
        if (!rc && classes) rc = class_join(ctx, k, s);
        if (rc) return rc;
    }
    return PXD_OK;
}

// ------------------------------------------------------- allocation-free variant
// The same kernel with its per-warp L-BFGS history and its pose-queue counter in a
// file-scope device array instead of the context's growable slab, so a launch makes
// no device allocation. The array holds 32 MiB: 256 bytes for the counter, then the
// history slabs of as many warps as fit; the persistent grid is trimmed to that many
// warps (at history 8 and 42 atoms: 4,096 warps, more than one launch's ~1,800).
// The counter must be zero when the kernel starts: each launch clears it with a
// memset on the caller's stream. Calls that overlap in time (other streams, other
// threads) share the array and race; the first call on a device resolves the array's
// address (cudaGetSymbolAddress), so make it before any stream capture.
constexpr size_t kStaticScratchBytes = size_t(32) << 20;
constexpr size_t kStaticCounterBytes = 256;
constexpr int kStaticMaxDevices = 64;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

static std::mutex g_static_mu;
static unsigned char* g_static_base[kStaticMaxDevices] = {};

static int static_scratch(pxd_context* ctx, unsigned char** out) {
    if (ctx->device < 0 || ctx->device >= kStaticMaxDevices)
        return set_error(ctx, PXD_ERR_INVALID, "device ordinal beyond the static scratch table");
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_base[ctx->device]) {
        void* p = nullptr;
        int rc = cuda_check(ctx, cudaGetSymbolAddress(&p, g_static_scratch), "static scratch address");
        if (rc) return rc;
        g_static_base[ctx->device] = static_cast<unsigned char*>(p);
    }
    *out = g_static_base[ctx->device];
    return PXD_OK;
}

int launch_lbfgs_noalloc(pxd_context* ctx, const pxd_lbfgs_params& p, int n_poses, int max_atoms,
                         const int* lig_ids, float* xyz, float* tors, double* energy, int* nevals,
                         int* status, cudaStream_t s) {
    if (n_poses <= 0) return PXD_OK;
    if (ctx->ligands_dirty && static_cast<int>(ctx->ligands.size()) > ctx->d_ligands_cap)
        return set_error(ctx, PXD_ERR_STATE,
                         "the device ligand table must grow, which allocates: make one "
                         "pxd_lbfgs_dev or pxd_score_grad_dev call after adding ligands");
    int rc = sync_ligand_table(ctx);  // a copy into the existing table
    if (rc) return rc;
    unsigned char* base = nullptr;
    rc = static_scratch(ctx, &base);
    if (rc) return rc;
    LbfgsArgs a{};
    a.env = make_env(ctx);
    a.ligands = ctx->d_ligands;
    a.lig_ids = lig_ids;
    a.n_ligands = static_cast<int>(ctx->ligands.size());
    a.xyz = xyz;
    a.tors = tors;
    a.max_atoms = max_atoms;
    a.energy = energy;
    a.nevals = nevals;
    a.status = status;
    a.n_poses = n_poses;
    a.stride_atoms = max_atoms;
    a.order = nullptr;
    a.count_dev = nullptr;
    fill_consts(a, p);
    a.n_local = ctx->rec.n_local;
    const bool dof = p.dof_mode == PXD_DOF_RIGID_TORSION;
    a.D_pad = vec_pad(ctx, max_atoms, dof);
    a.X_pad = dof_xpad(ctx, max_atoms, dof);
    const size_t smem = lbfgs_block_smem(ctx, max_atoms, p.history, false, dof);
    const LbfgsKernelFn kern = lbfgs_variant(ctx, max_atoms, dof);
    rc = raise_smem_limit(ctx, reinterpret_cast<const void*>(kern), smem, "lbfgs smem attribute");
    if (rc) return rc;
    int per_sm = 0;
    rc = cuda_check(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern,
                                                                      kWarpsPerBlock * kWarp, smem),
                    "lbfgs occupancy");
    if (rc) return rc;
    if (per_sm < 1) return set_error(ctx, PXD_ERR_INVALID, "ligand too large for shared memory");
    a.hist_stride = static_cast<size_t>(2) * hist_slots(p.history) * a.D_pad;
    const size_t block_bytes = sizeof(float) * a.hist_stride * kWarpsPerBlock;
    const size_t fit = (kStaticScratchBytes - kStaticCounterBytes) / block_bytes;
    if (fit < 1)
        return set_error(ctx, PXD_ERR_INVALID,
                         "one block's L-BFGS history (" + std::to_string(block_bytes) +
                             " bytes) exceeds the 32 MiB static scratch: lower history or max_atoms");
    int blocks = per_sm * ctx->n_sm;
    const int need = (n_poses + kWarpsPerBlock - 1) / kWarpsPerBlock;
    if (blocks > need) blocks = need;
    if (static_cast<size_t>(blocks) > fit) blocks = static_cast<int>(fit);
    a.counter = reinterpret_cast<int*>(base);
    a.hist = reinterpret_cast<float*>(base + kStaticCounterBytes);
    rc = cuda_check(ctx, cudaMemsetAsync(a.counter, 0, sizeof(int), s), "counter reset");
    if (rc) return rc;
    kern<<<blocks, kWarpsPerBlock * kWarp, smem, s>>>(a);
    return cuda_check(ctx, cudaGetLastError(), "lbfgs_kernel launch");
}

}  // namespace pxd

using namespace pxd;

extern "C" int pxd_score_grad_multi_dev(pxd_context* const* ctxs, int32_t n_ctx, int32_t n_poses, int32_t max_atoms,
                                        const int32_t* ctx_ids, const int32_t* lig_ids, const float* xyz,
                                        const float* tors, double* energy, float* lig_grad, float* tors_grad,
                                        void* stream) {
    if (!ctxs || n_ctx < 1 || !ctxs[0]) return PXD_ERR_INVALID;
    pxd_context* ctx = ctxs[0];  // errors are reported here
    if (n_poses < 0 || max_atoms <= 0 || max_atoms > PXD_MAX_LIGAND_ATOMS || !ctx_ids || !lig_ids || !xyz ||
        !energy || !lig_grad)
        return set_error(ctx, PXD_ERR_INVALID, "bad pose batch shape");
    cudaSetDevice(ctx->device);
    std::vector<EvalEnv> envs(n_ctx);
    std::vector<const DevLigand*> tabs(n_ctx);
    std::vector<int> n_ligs(n_ctx);
    int max_local = 0, max_rot = 0;
    for (int c = 0; c < n_ctx; ++c) {
        pxd_context* k = ctxs[c];
        if (!k || k->device != ctx->device) return set_error(ctx, PXD_ERR_INVALID, "contexts must be on one device");
        if (!k->has_receptor) return set_error(ctx, PXD_ERR_STATE, "set a receptor first");
        int rc = sync_ligand_table(k);
        if (rc) return set_error(ctx, rc, k->error);
        envs[c] = make_env(k);
        tabs[c] = k->d_ligands;
        n_ligs[c] = static_cast<int>(k->ligands.size());
        max_local = std::max(max_local, k->rec.n_local);
        max_rot = std::max(max_rot, k->rec.n_rotors);
    }
    if (max_rot > 0 && (!tors || !tors_grad))
        return set_error(ctx, PXD_ERR_INVALID, "receptor torsion buffers required");
    if (n_poses == 0) return PXD_OK;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    const size_t e_bytes = (sizeof(EvalEnv) * n_ctx + 255) / 256 * 256;
    const size_t t_bytes = (sizeof(void*) * n_ctx + 255) / 256 * 256;
    void* mem = nullptr;
    int rc = cuda_check(ctx, cudaMallocAsync(&mem, e_bytes + t_bytes + sizeof(int) * n_ctx, s), "context tables");
    if (rc) return rc;
    char* base = static_cast<char*>(mem);
    rc = cuda_check(ctx, cudaMemcpyAsync(base, envs.data(), sizeof(EvalEnv) * n_ctx, cudaMemcpyHostToDevice, s),
                    "context table copy");
    if (!rc)
        rc = cuda_check(ctx, cudaMemcpyAsync(base + e_bytes, tabs.data(), sizeof(void*) * n_ctx,
                                             cudaMemcpyHostToDevice, s),
                        "ligand table pointer copy");
    if (!rc)
        rc = cuda_check(ctx, cudaMemcpyAsync(base + e_bytes + t_bytes, n_ligs.data(), sizeof(int) * n_ctx,
                                             cudaMemcpyHostToDevice, s),
                        "ligand count copy");
    if (rc) {
        cudaFreeAsync(mem, s);
        return rc;
    }
    ScoreMultiArgs a{};
    a.envs = reinterpret_cast<const EvalEnv*>(base);
    a.tabs = reinterpret_cast<const DevLigand* const*>(base + e_bytes);
    a.n_ligs = reinterpret_cast<const int*>(base + e_bytes + t_bytes);
    a.ctx_ids = ctx_ids;
    a.lig_ids = lig_ids;
    a.xyz = xyz;
    a.tors = tors;
    a.tors_stride = max_rot;
    a.max_atoms = max_atoms;
    a.energy = energy;
    a.lig_grad = lig_grad;
    a.tors_grad = tors_grad;
    a.n_poses = n_poses;
    a.n_local = max_local;
    a.D_pad = padded(3 * max_atoms + max_rot);
    const size_t smem = sizeof(float) * kWarpsPerBlock * (pose_bufs_floats(max_atoms, a.n_local) + 2 * a.D_pad);
    rc = raise_smem_limit(ctx, reinterpret_cast<const void*>(score_multi_kernel), smem, "score smem attribute");
    if (!rc) {
        int blocks = (n_poses + kWarpsPerBlock - 1) / kWarpsPerBlock;
        if (blocks > ctx->n_sm * 16) blocks = ctx->n_sm * 16;
        score_multi_kernel<<<blocks, kWarpsPerBlock * kWarp, smem, s>>>(a);
        rc = cuda_check(ctx, cudaGetLastError(), "score_multi_kernel launch");
    }
    cudaFreeAsync(mem, s);
    return rc;
}

// ------------------------------------------------------------------ autotuner
extern "C" int pxd_lbfgs_set_variant(pxd_context* ctx, int32_t class_bound, int32_t variant) {
    if (!ctx) return PXD_ERR_INVALID;
    if (class_bound < 32 || class_bound > 256 || class_bound % 32)
        return set_error(ctx, PXD_ERR_INVALID, "class bound must be 32, 64, ... 256");
    if (variant == -1) {
        ctx->lbfgs_tuned.erase(class_bound);
        return PXD_OK;
    }
    const int blocks = variant & ~kHistSmem;
    if (variant < 0 || !(blocks == 0 || (blocks >= 3 && blocks <= 6)))
        return set_error(ctx, PXD_ERR_INVALID, "variant: 0 or 3..6 resident blocks, + PXD_LBFGS_HIST_SMEM");
    ctx->lbfgs_tuned[class_bound] = variant;
    return PXD_OK;
}

extern "C" int pxd_lbfgs_autotune_dev(pxd_context* ctx, const pxd_lbfgs_params* params, int32_t n_poses,
                                      int32_t max_atoms, const int32_t* ids, const float* xyz, const float* tors,
                                      int32_t sample, int32_t probe_iters, int32_t* report, void* stream) {
    if (!ctx) return PXD_ERR_INVALID;
    if (!ctx->has_receptor) return set_error(ctx, PXD_ERR_STATE, "set a receptor first");
    if (!params || n_poses < 0 || max_atoms <= 0 || max_atoms > PXD_MAX_LIGAND_ATOMS || sample < 1 ||
        probe_iters < 1 || !ids || !xyz || (ctx->rec.n_rotors > 0 && !tors))
        return set_error(ctx, PXD_ERR_INVALID, "bad autotune batch");
    cudaSetDevice(ctx->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    const int R = ctx->rec.n_rotors;
    std::vector<int32_t> h_ids(n_poses);
    int rc = cuda_check(ctx, cudaMemcpyAsync(h_ids.data(), ids, sizeof(int32_t) * n_poses, cudaMemcpyDeviceToHost, s),
                        "autotune ids");
    if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(s), "autotune ids");
    if (rc) return rc;
    // poses per size class (class of the pose's ligand), at most `sample` each
    std::map<int, std::vector<int>> by_class;
    for (int i = 0; i < n_poses; ++i) {
        const int lid = h_ids[i];
        if (lid < 0 || lid >= static_cast<int>(ctx->ligands.size())) continue;
        const int n = ctx->ligands[lid].n_atoms;
        if (n > max_atoms) continue;
        std::vector<int>& v = by_class[class_bound(n)];
        if (static_cast<int>(v.size()) < sample) v.push_back(i);
    }
    pxd_lbfgs_params p = *params;
    p.max_iter = std::min(p.max_iter, probe_iters);
    static const int kVariants[10] = {4, 5, 6, 3, 0, 4 | kHistSmem, 5 | kHistSmem, 6 | kHistSmem, 3 | kHistSmem,
                                      0 | kHistSmem};
    int n_report = 0;
    for (auto& [bound, rows] : by_class) {
        const int m = static_cast<int>(rows.size());
        const int cap = std::min(bound, max_atoms);
        std::vector<int> rid(m);
        for (int k = 0; k < m; ++k) rid[k] = h_ids[rows[k]];
        Staging st{ctx, {}};
        int* d_ids = st.alloc<int>(m, &rc);
        float* d_x0 = rc ? nullptr : st.alloc<float>(static_cast<size_t>(m) * cap * 3, &rc);
        float* d_x = rc ? nullptr : st.alloc<float>(static_cast<size_t>(m) * cap * 3, &rc);
        float* d_t0 = rc ? nullptr : st.alloc<float>(static_cast<size_t>(m) * std::max(R, 1), &rc);
        float* d_t = rc ? nullptr : st.alloc<float>(static_cast<size_t>(m) * std::max(R, 1), &rc);
        double* d_e = rc ? nullptr : st.alloc<double>(m, &rc);
        int* d_n = rc ? nullptr : st.alloc<int>(m, &rc);
        int* d_s = rc ? nullptr : st.alloc<int>(m, &rc);
        if (rc) return rc;
        queue_copy(ctx, &rc, d_ids, rid.data(), sizeof(int) * m, cudaMemcpyHostToDevice, s, "autotune ids");
        for (int k = 0; k < m && !rc; ++k) {  // gather the sampled rows at the class's stride
            rc = cuda_check(ctx, cudaMemcpy2DAsync(d_x0 + static_cast<size_t>(k) * cap * 3, sizeof(float) * cap * 3,
                                                   xyz + static_cast<size_t>(rows[k]) * max_atoms * 3,
                                                   sizeof(float) * max_atoms * 3, sizeof(float) * cap * 3, 1,
                                                   cudaMemcpyDeviceToDevice, s),
                            "autotune pose gather");
            if (R > 0)
                queue_copy(ctx, &rc, d_t0 + static_cast<size_t>(k) * R, tors + static_cast<size_t>(rows[k]) * R,
                           sizeof(float) * R, cudaMemcpyDeviceToDevice, s, "autotune torsion gather");
        }
        if (rc) return rc;
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        double best_rate = -1.0;
        int best = kDefaultMinBlocks;
        std::vector<int> nev(m);
        int smem_limit = 0;
        cudaDeviceGetAttribute(&smem_limit, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
        for (int v : kVariants) {
            if ((v & kHistSmem) && lbfgs_block_smem(ctx, cap, p.history, true, p.dof_mode == PXD_DOF_RIGID_TORSION) >
                                        static_cast<size_t>(smem_limit))
                continue;  // the history does not fit beside the pose buffers
            ctx->lbfgs_tuned[bound] = v;
            queue_copy(ctx, &rc, d_x, d_x0, sizeof(float) * m * cap * 3, cudaMemcpyDeviceToDevice, s,
                       "autotune pose restore");
            queue_copy(ctx, &rc, d_t, d_t0, sizeof(float) * m * std::max(R, 1), cudaMemcpyDeviceToDevice, s,
                       "autotune torsion restore");
            if (rc) break;
            cudaEventRecord(a, s);
            rc = launch_lbfgs(ctx, p, m, cap, d_ids, d_x, d_t, d_e, d_n, d_s, s);
            cudaEventRecord(b, s);
            if (!rc) rc = cuda_check(ctx, cudaMemcpyAsync(nev.data(), d_n, sizeof(int) * m, cudaMemcpyDeviceToHost, s),
                                     "autotune evaluations");
            if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(s), "autotune probe");
            if (rc) break;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, a, b);
            double evals = 0.0;
            for (int x : nev) evals += x;
            const double rate = ms > 0.f ? evals / ms : 0.0;
            if (rate > best_rate) {
                best_rate = rate;
                best = v;
            }
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        ctx->lbfgs_tuned[bound] = best;
        if (rc) return rc;
        if (report && n_report < kSizeClasses) {
            report[2 * n_report] = bound;
            report[2 * n_report + 1] = best;
        }
        ++n_report;
    }
    if (report)
        for (int k = n_report; k < kSizeClasses; ++k) report[2 * k] = report[2 * k + 1] = -1;
    return PXD_OK;
}
