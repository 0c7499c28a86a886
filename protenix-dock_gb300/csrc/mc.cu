// Monte-Carlo docking search on the GPU: one warp per walker in a persistent launch
// (monte_carlo_searcher::mutate_and_optimize, searcher.cpp:46-223).
//
// Each walker owns the reference's generator, std::mt19937 seeded seed + walker, and
// draws from it exactly as random_generator does (random.h:33-63, random.cpp:22-49):
// lane 0 advances the state (kept in a per-warp global slab) and broadcasts the values,
// so every random start, move and Metropolis test consumes the reference's stream.
// Relaxations reuse the batched L-BFGS device code, scores the device pose scorer.
#include <cstdlib>
#include <cstring>
#include <vector>

#include "device_kin.cuh"
#include "device_lbfgs.cuh"
#include "device_score.cuh"

namespace pxd {

// ----------------------------------------------------------------- mt19937
struct MtState {
    uint32_t mt[624];
    int idx;
};

__device__ void mt_seed(MtState* s, uint32_t seed) {
    s->mt[0] = seed;
    for (int i = 1; i < 624; ++i) s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + i;
    s->idx = 624;
}

// MT19937 (Matsumoto & Nishimura 1998), generated 624 words at a time.
__device__ uint32_t mt_next(MtState* s) {
    if (s->idx >= 624) {
        for (int i = 0; i < 624; ++i) {
            const uint32_t y = (s->mt[i] & 0x80000000u) | (s->mt[i + 1 < 624 ? i + 1 : 0] & 0x7fffffffu);
            const int k = i + 397 < 624 ? i + 397 : i + 397 - 624;
            s->mt[i] = s->mt[k] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        s->idx = 0;
    }
    uint32_t y = s->mt[s->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

// std::generate_canonical<double, 53> over mt19937: two words, (lo + hi 2^32) / 2^64
__device__ double mt_canonical(MtState* s) {
    double v = static_cast<double>(mt_next(s));
    v += static_cast<double>(mt_next(s)) * 4294967296.0;
    v = v / 18446744073709551616.0;
    if (v >= 1.0) v = nextafter(1.0, 0.0);
    return v;
}

// std::uniform_int_distribution<int>: Lemire's multiply-and-reject (arXiv:1805.10941)
__device__ int mt_uniform_int(MtState* s, int a, int b) {
    const uint32_t range = static_cast<uint32_t>(b) - static_cast<uint32_t>(a) + 1u;
    uint64_t prod = static_cast<uint64_t>(mt_next(s)) * range;
    uint32_t low = static_cast<uint32_t>(prod);
    if (low < range) {
        const uint32_t threshold = (0u - range) % range;
        for (int guard = 0; low < threshold && guard < 64; ++guard) {
            prod = static_cast<uint64_t>(mt_next(s)) * range;
            low = static_cast<uint32_t>(prod);
        }
    }
    return static_cast<int>(static_cast<uint32_t>(a) + static_cast<uint32_t>(prod >> 32));
}

// The distributions below round every product and sum separately (no fused
// multiply-add), as the host library computes them, so the device draws are bit-identical.
__device__ double mt_uniform_real(MtState* s, double a, double b) {
    return __dadd_rn(__dmul_rn(mt_canonical(s), __dsub_rn(b, a)), a);
}

__device__ double mt_torsion(MtState* s) {
    const double pi = 3.141592653589793;
    return mt_uniform_real(s, -pi, pi);
}

// random_in_sphere: rejection in [-1, 1)^3 (acceptance pi/6; bounded)
__device__ void mt_in_sphere(MtState* s, double* o) {
    for (int guard = 0; guard < 4096; ++guard) {
        o[0] = mt_uniform_real(s, -1.0, 1.0);
        o[1] = mt_uniform_real(s, -1.0, 1.0);
        o[2] = mt_uniform_real(s, -1.0, 1.0);
        double t = __dmul_rn(o[0], o[0]);
        t = __dadd_rn(t, __dmul_rn(o[1], o[1]));
        t = __dadd_rn(t, __dmul_rn(o[2], o[2]));
        if (t < 1.0) return;
    }
}

// random_orientation: Shoemake's uniform quaternion
__device__ void mt_orientation(MtState* s, double* q) {
    const double two_pi = 2 * 3.141592653589793;
    const double u1 = mt_uniform_real(s, 0.0, 1.0);
    const double u2 = __dmul_rn(mt_uniform_real(s, 0.0, 1.0), two_pi);
    const double u3 = __dmul_rn(mt_uniform_real(s, 0.0, 1.0), two_pi);
    const double a = sqrt(1.0 - u1), b = sqrt(u1);
    q[0] = a * sin(u2);
    q[1] = a * cos(u2);
    q[2] = b * sin(u3);
    q[3] = b * cos(u3);
}

// ------------------------------------------------------------------ kernel
constexpr int kMcWarps = 4;
constexpr int kMaxTries = 20000;

struct McArgs {
    EvalEnv env;
    ScoreEnv senv;
    const DevLigand* ligands;
    int n_ligands;
    const int* lig_ids;
    const int* walker_ids;
    const int* first_pose;
    const float* start;
    int max_atoms;
    float* out_xyz;
    float* out_tors;
    double* out_e;
    double* out_ps;
    int* out_nev;
    int* out_st;
    double* gmin;
    int n_walkers;
    int* counter;
    int* error;
    LbfgsConsts full, fast;
    int max_nsteps;
    double threshold, amp, temp;
    float lo[3], hi[3];
    double blo[3], bhi[3];  // the box as given, for the random centre draws
    uint32_t seed;
    int n_local, D_pad;
    int warps_per_block;  // kMcWarps
    int team;             // kMcWarps: the block's warps search one walker together; 1: a walker per warp
    int drop_member;      // test of the bounded team barriers: the last member leaves at once
    float* hist;
    size_t hist_stride;
    MtState* rng;
};

__host__ __device__ inline int mc_warp_floats(int max_atoms, int n_local, int Dp, int m) {
    return pose_bufs_floats(max_atoms, n_local) + kOptVecs * Dp + opt_scalar_floats(m) + 2 * Dp + 4 * max_atoms +
           static_cast<int>(sizeof(KinShared) / sizeof(float)) + 64 + 16;
}

__device__ bool all_in_box(const float* x, int N, const McArgs& a, int lane) {
    bool ok = true;
    for (int i = lane; i < N; i += kWarp) {
        ok = ok && x[3 * i] > a.lo[0] && x[3 * i] < a.hi[0] && x[3 * i + 1] > a.lo[1] &&
             x[3 * i + 1] < a.hi[1] && x[3 * i + 2] > a.lo[2] && x[3 * i + 2] < a.hi[2];
    }
    return __all_sync(kFull, ok);
}

__device__ float3 mean_xyz(const float* x, int N, int lane) {
    float sx = 0.f, sy = 0.f, sz = 0.f;
    for (int i = lane; i < N; i += kWarp) {
        sx += x[3 * i];
        sy += x[3 * i + 1];
        sz += x[3 * i + 2];
    }
    return mul3(make_float3(warp_sum_f(sx), warp_sum_f(sy), warp_sum_f(sz)), 1.f / N);
}

// free_ligand::apply_parameters on the atom-ordered pose x (in place)
__device__ void apply_tree(const DevLigand& L, float* x, float4* c, KinShared& ks, float3 center,
                           const Mat3& R, const float* tors, int lane) {
    const int N = L.n_atoms;
    for (int p = lane; p < N; p += kWarp) {
        const int atom = __ldg(&L.perm[p]);
        c[p] = make_float4(x[3 * atom], x[3 * atom + 1], x[3 * atom + 2], 0.f);
    }
    __syncwarp();
    ligand_forward(L, c, L.frag_of, L.frag_mine, L.frag_parent, center, R, tors, ks, lane);
    for (int p = lane; p < N; p += kWarp) {
        const int atom = __ldg(&L.perm[p]);
        x[3 * atom] = c[p].x;
        x[3 * atom + 1] = c[p].y;
        x[3 * atom + 2] = c[p].z;
    }
    __syncwarp();
}

// mm_interaction_vdw_energy::report with the receptor's input coordinates (the
// randomize() clash test, searcher.cpp:76-79)
__device__ double vdw_check(const ScoreEnv& se, const DevLigand& L, const float* x, int lane) {
    const DevSf& sf = *se.sf;
    DS acc{0.f, 0.f};
    for (int i = 0; i < L.n_atoms; ++i) {
        const float3 xi = make_float3(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
        const float2 ti = sf.vdw_type[__ldg(&L.type[i])];
        float ev = 0.f;
        for (int j = lane; j < se.rs.n_all; j += kWarp) {
            const float4 rj = __ldg(&se.rs.all_xyzq[j]);
            const float2 sej = __ldg(&se.rs.all_se[j]);
            const float d = dist3(xi, xyz(rj));
            const float s = (ti.x + sej.x) * 0.5f / (d + kEpsF);
            const float s2 = s * s;
            const float u6 = s2 * s2 * s2;
            const float v = (u6 * u6 - u6) * (sqrtf(ti.y * sej.y) * 4.f);
            ev += fminf(fmaxf(v, -sf.vdw_cutoff), sf.vdw_cutoff);
        }
        ds_add(acc, ev);
    }
    return ds_warp_sum(acc) * sf.vdw_scale;
}

// Pose score of the state [xyz | torsions] in x (root_scorer::combine).
__device__ double mc_pscore(const McArgs& a, const DevLigand& L, const float* x, const PoseBufs& b,
                            const Team& tm, int lane) {
    const int N = L.n_atoms;
    const DevReceptor& R = a.env.rec;
    for (int i = lane; i < N; i += kWarp) b.lig_xyz[i] = make_float4(x[3 * i], x[3 * i + 1], x[3 * i + 2], 0.f);
    for (int l = lane; l < R.n_mov; l += kWarp) {
        const float4 v = __ldg(&R.local_xyz0[l]);
        const int r = __float_as_int(v.w);
        Mat3 Rm, Jm;
        rotation_and_jacobian(xyz(__ldg(&R.rotor_axis[r])), x[3 * N + r], Rm, Jm);
        const float3 p = add3(mat_apply(Rm, xyz(v)), xyz(__ldg(&R.rotor_origin[r])));
        b.loc_xyz[l] = make_float4(p.x, p.y, p.z, 0.f);
    }
    __syncwarp();
    return score_pose<true>(a.senv, L, L.score, b.lig_xyz, b.loc_xyz, lane, nullptr, tm.w, tm.n, tm.ts);
}

__device__ void atomic_min_double(double* p, double v) {
    unsigned long long* u = reinterpret_cast<unsigned long long*>(p);
    unsigned long long old = *u;
    for (int guard = 0; guard < 1024; ++guard) {
        if (__longlong_as_double(static_cast<long long>(old)) <= v) return;
        const unsigned long long seen = atomicCAS(u, old, static_cast<unsigned long long>(__double_as_longlong(v)));
        if (seen == old) return;
        old = seen;
    }
}

// The relaxations form the two-loop coefficients in FP32 (lbfgs_pose<true>): a walker's warp
// is usually alone on its SM, where the FP64 operations on each pass's dependent chain are
// what it waits on.
//
// Team mode (a.team = kMcWarps, at most one walker per SM): the block's warps search one
// walker together. Every member runs the walker's whole search on its own slice
// with its own copy of the generator, seeded alike, so all members draw the same numbers and
// take the same branches; the evaluations split their terms, lookups and explicit pairs
// among the members and sum the members' parts in member order (eval_pose_team_body), so every
// member holds the same energy and gradient. The history slab is the team's: members write
// the same values to it. Only member 0 takes walkers from the queue, updates the global
// minimum and writes the outputs, and its queue slot and minimum reach the others through
// the team's shared state. Team barriers spin a bounded number of times; a team that gives
// up raises the launch's second error flag (a.error[1], reported by the host) and leaves
// its walker with status 3.
__global__ void __launch_bounds__(kMcWarps * kWarp) mc_kernel(const __grid_constant__ McArgs a) {
    extern __shared__ __align__(16) float smem[];
    const int lane = threadIdx.x & (kWarp - 1);
    const int wib = threadIdx.x / kWarp;
    const int Dp = a.D_pad;
    const int m = a.full.m;
    const int slice = mc_warp_floats(a.max_atoms, a.n_local, Dp, m);
    const bool team = a.team > 1;
    const bool lead = !team || wib == 0;  // the member that takes walkers and writes results
    float* base = smem + static_cast<size_t>(wib) * slice;
    const PoseBufs b = carve_pose_bufs(base, a.max_atoms, a.n_local);
    Team tm{0, 1, 0, nullptr};
    if (team) {
        tm.w = wib;
        tm.n = a.team;
        tm.f4 = slice / 4;
        tm.ts = reinterpret_cast<TeamShared*>(smem + static_cast<size_t>(a.warps_per_block) * slice);
        if (threadIdx.x == 0) {
            tm.ts->count = 0;
            tm.ts->gen = 0;
            tm.ts->abort = 0;
            tm.ts->slot = 0;
        }
        __syncthreads();
        // failure test (PXD_TEST_TEAM_DROPOUT): a member that never arrives, so that the
        // others' waits run out and the launch reports it
        if (a.drop_member && wib == a.team - 1) return;
    }
    float* vb = base + pose_bufs_floats(a.max_atoms, a.n_local);
    Vecs v = carve_vecs(vb, Dp, m);
    float* best_x = vb + kOptVecs * Dp + opt_scalar_floats(m);
    float* tmp_x = best_x + Dp;
    float4* kc = reinterpret_cast<float4*>(tmp_x + Dp);
    KinShared& ks = *reinterpret_cast<KinShared*>(kc + a.max_atoms);
    float* tq = reinterpret_cast<float*>(&ks + 1);          // [64] torsions of a move
    double* bc = reinterpret_cast<double*>(tq + 64);         // [8] broadcast slots
    const size_t gw = static_cast<size_t>(blockIdx.x) * a.warps_per_block + wib;
    v.S = a.hist + (team ? static_cast<size_t>(blockIdx.x) : gw) * a.hist_stride;
    v.Y = v.S + static_cast<size_t>(hist_slots(m)) * Dp;
    MtState* rng = a.rng + gw;
    const int R = a.env.rec.n_rotors;
    TeamClosure c;
    c.env = &a.env;
    c.b = &b;
    c.team = &tm;
    c.lane = lane;
    while (true) {
        int w = 0;
        if (team) {
            if (threadIdx.x == 0) tm.ts->slot = atomicAdd(a.counter, 1);
            bool ok = team_sync(tm.ts, a.team, lane);
            w = *reinterpret_cast<volatile int*>(&tm.ts->slot);
            ok = ok && team_sync(tm.ts, a.team, lane);  // read by all before the next take
            if (!ok) {  // the team gave up waiting: its walker is not searched
                if (lead && lane == 0) atomicExch(a.error + 1, 1);
                break;
            }
        } else {
            if (lane == 0) w = atomicAdd(a.counter, 1);
            w = __shfl_sync(kFull, w, 0);
        }
        if (w >= a.n_walkers) break;
        const int lid = a.lig_ids[w];
        if (lid < 0 || lid >= a.n_ligands || a.ligands[lid].n_atoms > a.max_atoms || !a.ligands[lid].score.has ||
            a.ligands[lid].n_frags == 0) {
            if (lead && lane == 0) {
                a.out_st[w] = 3;
                a.out_nev[w] = 0;
            }
            continue;
        }
        const DevLigand& L = a.ligands[lid];
        const int N = L.n_atoms, T = L.n_tors, D = 3 * N + R;
        const int walker = a.walker_ids[w];
        const float* start = a.start + static_cast<size_t>(w) * a.max_atoms * 3;
        if (lane == 0) mt_seed(rng, a.seed + static_cast<uint32_t>(walker));
        __syncwarp();
        c.L = &L;
        // ---- start pose: the input (walker 0) or randomize() (searcher.cpp:46-87)
        for (int e = lane; e < 3 * N; e += kWarp) v.x[e] = start[e];
        for (int r = lane; r < R; r += kWarp) v.x[3 * N + r] = 0.f;
        __syncwarp();
        if (walker != 0) {
            const bool first = a.first_pose[w] != 0;
            bool placed = false;
            // the reference loops until the centroid lands in the box; this loop is
            // bounded and reports a walker that never placed its ligand
            for (int tries = 1; tries <= kMaxTries && !placed; ++tries) {
                if (lane == 0) {
                    double q[4];
                    for (int d = 0; d < 3; ++d) bc[d] = mt_uniform_real(rng, a.blo[d], a.bhi[d]);
                    mt_orientation(rng, q);
                    const double aa = q[0] * q[0], ab = q[0] * q[1], ac = q[0] * q[2], ad = q[0] * q[3];
                    const double bb = q[1] * q[1], bcq = q[1] * q[2], bd = q[1] * q[3];
                    const double cc = q[2] * q[2], cd = q[2] * q[3], dd = q[3] * q[3];
                    const float rm[9] = {static_cast<float>(aa + bb - cc - dd), static_cast<float>(2 * (bcq - ad)),
                                         static_cast<float>(2 * (ac + bd)),     static_cast<float>(2 * (ad + bcq)),
                                         static_cast<float>(aa - bb + cc - dd), static_cast<float>(2 * (cd - ab)),
                                         static_cast<float>(2 * (bd - ac)),     static_cast<float>(2 * (ab + cd)),
                                         static_cast<float>(aa - bb - cc + dd)};
                    for (int k = 0; k < 9; ++k) tq[32 + k] = rm[k];
                    for (int k = 0; k < T; ++k) tq[k] = first ? static_cast<float>(mt_torsion(rng)) : 0.f;
                }
                __syncwarp();
                for (int e = lane; e < 3 * N; e += kWarp) v.x[e] = start[e];
                __syncwarp();
                Mat3 Rq;
                Rq.r0 = make_float3(tq[32], tq[33], tq[34]);
                Rq.r1 = make_float3(tq[35], tq[36], tq[37]);
                Rq.r2 = make_float3(tq[38], tq[39], tq[40]);
                const float3 ctr = make_float3(static_cast<float>(bc[0]), static_cast<float>(bc[1]),
                                               static_cast<float>(bc[2]));
                __syncwarp();
                apply_tree(L, v.x, kc, ks, ctr, Rq, tq, lane);
                if (tries < 2000 && !all_in_box(v.x, N, a, lane)) continue;
                const float3 g = mean_xyz(v.x, N, lane);
                if (!(g.x > a.lo[0] && g.x < a.hi[0] && g.y > a.lo[1] && g.y < a.hi[1] && g.z > a.lo[2] &&
                      g.z < a.hi[2]))
                    continue;
                placed = tries > 1999 || vdw_check(a.senv, L, v.x, lane) < 100.0;
            }
            if (!placed && lead && lane == 0) atomicAdd(a.error, 1);
        }
        // ---- full relaxation and score of the start (searcher.cpp:120-126)
        double best_e = 0.0;
        lbfgs_pose<true>(c, a.full, v, D, Dp, lane, best_e);
        long total = c.nevals;
        double best_ps = mc_pscore(a, L, v.x, b, tm, lane);
        vcopy(best_x, v.x, D, lane);
        int status = 0;
        if (walker != 0) {
            if (all_in_box(best_x, N, a, lane)) {
                vcopy(tmp_x, best_x, D, lane);
                double tmp_ps = best_ps;
                for (int step = 0; step < a.max_nsteps; ++step) {
                    vcopy(v.x, tmp_x, D, lane);
                    // mutate_inplace (searcher.cpp:189-223)
                    if (lane == 0) {
                        const int which = mt_uniform_int(rng, 0, T + 1);
                        reinterpret_cast<int*>(bc)[14] = which;
                    }
                    __syncwarp();
                    const int which = reinterpret_cast<int*>(bc)[14];
                    float3 ctr = mean_xyz(v.x, N, lane);
                    bool moved = true;
                    Mat3 Rm;
                    Rm.r0 = make_float3(1.f, 0.f, 0.f);
                    Rm.r1 = make_float3(0.f, 1.f, 0.f);
                    Rm.r2 = make_float3(0.f, 0.f, 1.f);
                    if (which == 0) {
                        if (lane == 0) mt_in_sphere(rng, bc);
                        __syncwarp();
                        ctr = add3(ctr, make_float3(static_cast<float>(bc[0] * a.amp), static_cast<float>(bc[1] * a.amp),
                                                    static_cast<float>(bc[2] * a.amp)));
                    } else if (which == 1) {
                        float acc = 0.f;
                        for (int i = lane; i < N; i += kWarp) {
                            const float3 dx = make_float3(v.x[3 * i] - ctr.x, v.x[3 * i + 1] - ctr.y, v.x[3 * i + 2] - ctr.z);
                            acc += dot3(dx, dx);
                        }
                        const float gr = sqrtf(warp_sum_f(acc) / N);
                        if (gr < 1e-6f) {
                            moved = false;
                        } else {
                            if (lane == 0) mt_in_sphere(rng, bc);
                            __syncwarp();
                            float3 dl = make_float3(static_cast<float>(bc[0] * (a.amp / gr)),
                                                    static_cast<float>(bc[1] * (a.amp / gr)),
                                                    static_cast<float>(bc[2] * (a.amp / gr)));
                            const float ang = sqrtf(dot3(dl, dl));
                            dl = mul3(dl, 1.f / ang);
                            Rm = rodrigues(dl, ang);
                        }
                    }
                    if (lane == 0) {
                        for (int k = 0; k < T; ++k) tq[k] = 0.f;
                        if (which > 1) tq[which - 2] = static_cast<float>(mt_torsion(rng));
                    }
                    __syncwarp();
                    if (moved) apply_tree(L, v.x, kc, ks, ctr, Rm, tq, lane);
                    // optional pruning on the pre-relaxation energy (searcher.cpp:141-157)
                    if (a.threshold > 0.0 && a.gmin) {
                        c.x0 = v.x;
                        const double pre = eval_pose<true>(a.env, L, v.x, nullptr, 0.f, v.gnew, b, lane, nullptr, &tm);
                        double gm;
                        if (team) {
                            // the leader's view of the shared minimum, so that every member
                            // takes the same branch
                            if (threadIdx.x == 0) {
                                atomic_min_double(&a.gmin[lid], pre);
                                tm.ts->gmin = *reinterpret_cast<volatile double*>(&a.gmin[lid]);
                            }
                            team_sync(tm.ts, a.team, lane);
                            gm = *reinterpret_cast<volatile double*>(&tm.ts->gmin);
                            team_sync(tm.ts, a.team, lane);
                        } else {
                            if (lane == 0) atomic_min_double(&a.gmin[lid], pre);
                            __syncwarp();
                            gm = *reinterpret_cast<volatile double*>(&a.gmin[lid]);
                        }
                        if (pre > gm + a.threshold) continue;
                    }
                    double cdd_e = 0.0;  // unused: the step is judged by its pose score
                    lbfgs_pose<true>(c, a.fast, v, D, Dp, lane, cdd_e, false);
                    total += c.nevals;
                    const double cdd_ps = mc_pscore(a, L, v.x, b, tm, lane);
                    bool accept = step == 0 || cdd_ps < tmp_ps;
                    if (!accept) {
                        if (lane == 0) bc[4] = mt_uniform_real(rng, 0.0, 1.0);
                        __syncwarp();
                        accept = bc[4] < exp((tmp_ps - cdd_ps) / a.temp);
                    }
                    if (accept && all_in_box(v.x, N, a, lane)) {
                        tmp_ps = cdd_ps;
                        if (tmp_ps < best_ps) {
                            double e2 = 0.0;
                            lbfgs_pose<true>(c, a.full, v, D, Dp, lane, e2);
                            total += c.nevals;
                            tmp_ps = mc_pscore(a, L, v.x, b, tm, lane);
                            if (tmp_ps < best_ps) {
                                best_ps = tmp_ps;
                                best_e = e2;
                                vcopy(best_x, v.x, D, lane);
                            }
                        }
                        vcopy(tmp_x, v.x, D, lane);
                    }
                }
            } else {
                bool big = false;
                for (int e = lane; e < 3 * N; e += kWarp) big = big || fabsf(best_x[e]) > 1e8f;
                status = __any_sync(kFull, big) ? 1 : 2;
                if (status == 1) total = 0;
            }
        }
        if (lead) {
            float* ox = a.out_xyz + static_cast<size_t>(w) * a.max_atoms * 3;
            for (int e = lane; e < 3 * N; e += kWarp) ox[e] = best_x[e];
            for (int r = lane; r < R; r += kWarp) a.out_tors[static_cast<size_t>(w) * R + r] = best_x[3 * N + r];
            if (lane == 0) {
                const bool aborted = team && *reinterpret_cast<volatile int*>(&tm.ts->abort);
                a.out_e[w] = best_e;
                a.out_ps[w] = best_ps;
                a.out_nev[w] = static_cast<int>(total);
                a.out_st[w] = aborted ? 3 : status;
                if (aborted) atomicExch(a.error + 1, 1);
            }
        }
        __syncwarp();
    }
}

// Device generator checks: draws in the order the caller lists them.
__global__ void rng_draws_kernel(uint32_t seed, int n, const int* kinds, const int* ints, double* out, MtState* s) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    mt_seed(s, seed);
    int o = 0;
    for (int i = 0; i < n; ++i) {
        double v[4];
        switch (kinds[i]) {
            case 0: out[o++] = mt_uniform_int(s, 0, ints[i]); break;
            case 1: out[o++] = mt_torsion(s); break;
            case 2: out[o++] = mt_uniform_real(s, 0.0, 1.0); break;
            case 3:
                mt_in_sphere(s, v);
                for (int k = 0; k < 3; ++k) out[o++] = v[k];
                break;
            default:
                mt_orientation(s, v);
                for (int k = 0; k < 4; ++k) out[o++] = v[k];
        }
    }
}

static LbfgsConsts consts(const pxd_lbfgs_params& p, int max_iter) {
    LbfgsConsts c;
    c.max_iter = max_iter;
    c.max_eval = 0;
    c.m = p.history;
    c.ls_max = p.ls_max;
    c.lr = p.lr;
    c.tol_grad = p.tolerance_grad;
    c.tol_change = p.tolerance_change;
    c.c1 = p.ls_c1;
    c.c2 = p.ls_c2;
    c.ls_tol_change = p.ls_tolerance_change;
    c.gtd_threshold = p.ls_gtd_threshold;
    c.reset = p.reset_threshold;
    return c;
}

}  // namespace pxd

using namespace pxd;

extern "C" {

void pxd_mc_defaults(pxd_mc_params* p) {
    std::memset(p, 0, sizeof(*p));
    p->seed = 0;
    p->max_nsteps = 200;
    p->relax_nsteps = 40;
    p->full_nsteps = 240;
    p->mc_mmenergy_threshold = -1.0;
    p->amplitude = 2.0;
    p->temperature = 1.2;
    pxd_lbfgs_defaults(&p->lbfgs);
}

int pxd_mc_search_dev(pxd_context* ctx, const pxd_mc_params* p, int32_t n_walkers, int32_t max_atoms,
                      const int32_t* lig_ids, const int32_t* walker_ids, const int32_t* first_pose,
                      const float* start, float* out_xyz, float* out_tors, double* out_e, double* out_ps,
                      int32_t* out_nev, int32_t* out_st, double* gmin, void* stream) {
    if (!ctx || !p) return PXD_ERR_INVALID;
    if (p->lbfgs.dof_mode != PXD_DOF_CARTESIAN)
        return set_error(ctx, PXD_ERR_INVALID, "the search relaxes in Cartesian variables (dof_mode 0)");
    if (!ctx->has_receptor) return set_error(ctx, PXD_ERR_STATE, "set a receptor first");
    if (!ctx->sf_set[0] || !ctx->rec_score.has)
        return set_error(ctx, PXD_ERR_STATE, "the search needs the pose-selection scoring function and receptor lists");
    if (n_walkers < 0 || max_atoms <= 0 || max_atoms > PXD_MAX_LIGAND_ATOMS || p->max_nsteps < 0 ||
        p->relax_nsteps < 0 || p->full_nsteps < 0 || p->lbfgs.history < 1 || p->lbfgs.history > PXD_MAX_HISTORY ||
        p->lbfgs.ls_max < 1 || !(p->temperature > 0))
        return set_error(ctx, PXD_ERR_INVALID, "bad search parameters");
    for (int d = 0; d < 3; ++d)
        if (!(p->box_hi[d] > p->box_lo[d])) return set_error(ctx, PXD_ERR_INVALID, "empty search box");
    if (p->mc_mmenergy_threshold > 0 && !gmin)
        return set_error(ctx, PXD_ERR_INVALID, "pruning needs the per-ligand minimum buffer");
    for (auto& e : ctx->ligands)
        if (e.dev.n_frags > kMaxFrags || e.n_tors > kWarp)
            return set_error(ctx, PXD_ERR_INVALID, "a ligand exceeds 64 fragments / 32 torsions");
    cudaSetDevice(ctx->device);
    if (n_walkers == 0) return PXD_OK;
    int rc = sync_ligand_table(ctx);
    if (rc) return rc;
    McArgs a{};
    a.env.rec = ctx->rec;
    a.env.grid = ctx->grid;
    a.senv.rs = ctx->rec_score;
    a.senv.sf = ctx->d_sf[0];
    a.ligands = ctx->d_ligands;
    a.n_ligands = static_cast<int>(ctx->ligands.size());
    a.lig_ids = lig_ids;
    a.walker_ids = walker_ids;
    a.first_pose = first_pose;
    a.start = start;
    a.max_atoms = max_atoms;
    a.out_xyz = out_xyz;
    a.out_tors = out_tors;
    a.out_e = out_e;
    a.out_ps = out_ps;
    a.out_nev = out_nev;
    a.out_st = out_st;
    a.gmin = gmin;
    a.n_walkers = n_walkers;
    a.full = consts(p->lbfgs, p->full_nsteps);
    a.fast = consts(p->lbfgs, p->relax_nsteps);
    a.max_nsteps = p->max_nsteps;
    a.threshold = p->mc_mmenergy_threshold;
    a.amp = p->amplitude;
    a.temp = p->temperature;
    for (int d = 0; d < 3; ++d) {
        a.lo[d] = static_cast<float>(p->box_lo[d]);
        a.hi[d] = static_cast<float>(p->box_hi[d]);
        a.blo[d] = p->box_lo[d];
        a.bhi[d] = p->box_hi[d];
    }
    a.seed = p->seed;
    a.n_local = ctx->rec.n_local;
    a.D_pad = (3 * max_atoms + ctx->rec.n_rotors + kWarp - 1) / kWarp * kWarp;
    // At most one walker per SM (a single docking search): a block of kMcWarps warps per
    // walker searching as a team, so each walker has an SM's L1, shared-memory pipe and issue
    // slots, and its four schedulers share the evaluations. Fewer walkers than 4 per SM: one
    // warp per block, so each walker has an SM to itself or shares it with few others.
    a.team = n_walkers <= ctx->n_sm ? kMcWarps : 1;
    {
        const char* drop = std::getenv("PXD_TEST_TEAM_DROPOUT");
        a.drop_member = drop && drop[0] == '1' && a.team > 1 ? 1 : 0;
    }
    a.warps_per_block = a.team > 1 || n_walkers >= kMcWarps * ctx->n_sm ? kMcWarps : 1;
    const int wpb = a.warps_per_block;
    const size_t smem = sizeof(float) * wpb * mc_warp_floats(max_atoms, a.n_local, a.D_pad, p->lbfgs.history) +
                        (a.team > 1 ? (sizeof(TeamShared) + 15) / 16 * 16 : 0);
    rc = raise_smem_limit(ctx, reinterpret_cast<const void*>(mc_kernel), smem, "mc smem attribute");
    if (rc) return rc;
    // One walker per block leaves the SMs nearly empty: ask for the smallest shared-memory carve-out
    // (percent of the SM's shared memory) that still holds the blocks each SM must run at
    // once for every walker to start together, so the rest serves as L1; full launches keep
    // the driver's choice.
    int carveout = cudaSharedmemCarveoutDefault;
    if (a.team > 1 || wpb == 1) {
        int sm_smem = 0;
        rc = cuda_check(ctx, cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device),
                        "shared memory per SM");
        if (rc) return rc;
        const size_t per_sm_blocks = (static_cast<size_t>(n_walkers) + ctx->n_sm - 1) / ctx->n_sm;
        const size_t need = per_sm_blocks * (smem + 1024);  // each block plus the driver's reserved kilobyte
        carveout = static_cast<int>(std::min<size_t>(100, (100 * need + sm_smem - 1) / sm_smem + 1));
    }
    rc = cuda_check(ctx, cudaFuncSetAttribute(mc_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, carveout),
                    "mc carve-out");
    if (rc) return rc;
    int per_sm = 0;
    rc = cuda_check(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mc_kernel, wpb * kWarp, smem),
                    "mc occupancy");
    if (rc) return rc;
    if (per_sm < 1) return set_error(ctx, PXD_ERR_INVALID, "ligand too large for shared memory");
    int blocks = per_sm * ctx->n_sm;
    const int walkers_per_block = a.team > 1 ? 1 : wpb;
    const int need = (n_walkers + walkers_per_block - 1) / walkers_per_block;
    if (blocks > need) blocks = need;
    const size_t warps = static_cast<size_t>(blocks) * wpb;
    a.hist_stride = static_cast<size_t>(2) * hist_slots(p->lbfgs.history) * a.D_pad;
    const size_t hist_bytes = sizeof(float) * a.hist_stride * warps;  // a slab per warp, or per team
    const size_t rng_off = (hist_bytes + 255) / 256 * 256;
    rc = ensure_scratch(ctx, rng_off + sizeof(MtState) * warps);
    if (rc) return rc;
    a.hist = static_cast<float*>(ctx->scratch);
    a.rng = reinterpret_cast<MtState*>(static_cast<char*>(ctx->scratch) + rng_off);
    a.counter = ctx->d_counter;
    a.error = ctx->d_counter + 1;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    rc = cuda_check(ctx, cudaMemsetAsync(ctx->d_counter, 0, 3 * sizeof(int), s), "counter reset");
    if (rc) return rc;
    return cuda_check(ctx, launch_with_map_window(ctx, mc_kernel, blocks, wpb * kWarp, smem, s, a),
                      "mc_kernel launch");
}

int pxd_mc_search(pxd_context* ctx, const pxd_mc_params* p, int32_t lig, int32_t n, const int32_t* walker_ids,
                  const int32_t* first_pose, const double* start, double* out_xyz, double* out_tors,
                  double* out_e, double* out_ps, int32_t* out_nev, int32_t* out_st) {
    if (!ctx) return PXD_ERR_INVALID;
    if (lig < 0 || lig >= static_cast<int>(ctx->ligands.size()) || n < 0)
        return set_error(ctx, PXD_ERR_INVALID, "ligand id / walker count");
    cudaSetDevice(ctx->device);
    const int N = ctx->ligands[lig].n_atoms, R = ctx->rec.n_rotors;
    const size_t nx = static_cast<size_t>(n) * N * 3, nt = static_cast<size_t>(n) * R;
    std::vector<float> hx(nx);
    for (size_t i = 0; i < nx; ++i) hx[i] = static_cast<float>(start[i]);
    std::vector<int> ids(n, lig);
    std::vector<double> gm(ctx->ligands.size(), 1e8);
    const size_t bytes = 8 * (2 * static_cast<size_t>(n) + gm.size()) + 4 * (2 * nx + nt + 5 * static_cast<size_t>(n)) + 256;
    void* mem = nullptr;
    int rc = cuda_check(ctx, cudaMallocAsync(&mem, bytes, ctx->stream), "search staging");
    if (rc) return rc;
    double* d_e = static_cast<double*>(mem);
    double* d_ps = d_e + n;
    double* d_gm = d_ps + n;
    float* d_start = reinterpret_cast<float*>(d_gm + gm.size());
    float* d_out = d_start + nx;
    float* d_tors = d_out + nx;
    int* d_ids = reinterpret_cast<int*>(d_tors + nt);
    int* d_w = d_ids + n;
    int* d_first = d_w + n;
    int* d_nev = d_first + n;
    int* d_st = d_nev + n;
    queue_copy(ctx, &rc, d_start, hx.data(), 4 * nx, cudaMemcpyHostToDevice, ctx->stream, "search starts");
    queue_copy(ctx, &rc, d_ids, ids.data(), 4 * static_cast<size_t>(n), cudaMemcpyHostToDevice, ctx->stream,
               "search ligand ids");
    queue_copy(ctx, &rc, d_w, walker_ids, 4 * static_cast<size_t>(n), cudaMemcpyHostToDevice, ctx->stream,
               "search walker ids");
    queue_copy(ctx, &rc, d_first, first_pose, 4 * static_cast<size_t>(n), cudaMemcpyHostToDevice, ctx->stream,
               "search first-pose flags");
    queue_copy(ctx, &rc, d_gm, gm.data(), 8 * gm.size(), cudaMemcpyHostToDevice, ctx->stream, "search radii");
    if (!rc) rc = pxd_mc_search_dev(ctx, p, n, N, d_ids, d_w, d_first, d_start, d_out, d_tors, d_e, d_ps, d_nev, d_st, d_gm,
                           ctx->stream);
    std::vector<float> ho(nx), ht(nt);
    if (!rc) {
        queue_copy(ctx, &rc, ho.data(), d_out, 4 * nx, cudaMemcpyDeviceToHost, ctx->stream, "search poses");
        if (nt) queue_copy(ctx, &rc, ht.data(), d_tors, 4 * nt, cudaMemcpyDeviceToHost, ctx->stream, "search torsions");
        queue_copy(ctx, &rc, out_e, d_e, 8 * static_cast<size_t>(n), cudaMemcpyDeviceToHost, ctx->stream,
                   "search energies");
        queue_copy(ctx, &rc, out_ps, d_ps, 8 * static_cast<size_t>(n), cudaMemcpyDeviceToHost, ctx->stream,
                   "search pose scores");
        queue_copy(ctx, &rc, out_nev, d_nev, 4 * static_cast<size_t>(n), cudaMemcpyDeviceToHost, ctx->stream,
                   "search evaluations");
        queue_copy(ctx, &rc, out_st, d_st, 4 * static_cast<size_t>(n), cudaMemcpyDeviceToHost, ctx->stream,
                   "search status");
    }
    cudaFreeAsync(mem, ctx->stream);
    rc = sync_copies(ctx, rc, ctx->stream, "search");
    if (rc) return rc;
    int err[2] = {0, 0};
    rc = cuda_check(ctx, cudaMemcpy(err, ctx->d_counter + 1, 2 * sizeof(int), cudaMemcpyDeviceToHost),
                    "search flags");
    if (rc) return rc;
    for (size_t i = 0; i < nx; ++i) out_xyz[i] = ho[i];
    for (size_t i = 0; i < nt; ++i) out_tors[i] = ht[i];
    if (err[1])
        return set_error(ctx, PXD_ERR_DEVICE_FLAG, "a search team stopped waiting at a barrier (walkers with status 3)");
    if (err[0]) return set_error(ctx, PXD_ERR_DEVICE_FLAG, "a random start found no pose inside the box");
    return PXD_OK;
}

int pxd_mc_search_multi(pxd_context* ctx, const pxd_mc_params* p, int32_t n, int32_t max_atoms,
                        const int32_t* ligand_ids, const int32_t* walker_ids, const int32_t* first_pose,
                        const double* start, double* out_xyz, double* out_tors, double* out_e, double* out_ps,
                        int32_t* out_nev, int32_t* out_st, double* global_min) {
    if (!ctx) return PXD_ERR_INVALID;
    if (n < 0 || max_atoms <= 0 || max_atoms > PXD_MAX_LIGAND_ATOMS ||
        (n > 0 && (!ligand_ids || !walker_ids || !first_pose || !start)))
        return set_error(ctx, PXD_ERR_INVALID, "bad walker batch");
    if (n == 0) return PXD_OK;
    cudaSetDevice(ctx->device);
    const int R = ctx->rec.n_rotors;
    const size_t nl = ctx->ligands.size();
    const size_t nx = static_cast<size_t>(n) * max_atoms * 3, nt = static_cast<size_t>(n) * R;
    std::vector<float> hx(nx);
    for (size_t i = 0; i < nx; ++i) hx[i] = static_cast<float>(start[i]);
    std::vector<double> gm(nl ? nl : 1, 1e8);
    if (global_min)
        for (size_t i = 0; i < nl; ++i) gm[i] = global_min[i];
    const size_t bytes =
        8 * (2 * static_cast<size_t>(n) + gm.size()) + 4 * (2 * nx + nt + 5 * static_cast<size_t>(n)) + 256;
    void* mem = nullptr;
    int rc = cuda_check(ctx, cudaMallocAsync(&mem, bytes, ctx->stream), "search staging");
    if (rc) return rc;
    double* d_e = static_cast<double*>(mem);
    double* d_ps = d_e + n;
    double* d_gm = d_ps + n;
    float* d_start = reinterpret_cast<float*>(d_gm + gm.size());
    float* d_out = d_start + nx;
    float* d_tors = d_out + nx;
    int* d_ids = reinterpret_cast<int*>(d_tors + nt);
    int* d_w = d_ids + n;
    int* d_first = d_w + n;
    int* d_nev = d_first + n;
    int* d_st = d_nev + n;
    queue_copy(ctx, &rc, d_start, hx.data(), 4 * nx, cudaMemcpyHostToDevice, ctx->stream, "search starts");
    queue_copy(ctx, &rc, d_ids, ligand_ids, 4 * static_cast<size_t>(n), cudaMemcpyHostToDevice, ctx->stream,
               "search ligand ids");
    queue_copy(ctx, &rc, d_w, walker_ids, 4 * static_cast<size_t>(n), cudaMemcpyHostToDevice, ctx->stream,
               "search walker ids");
    queue_copy(ctx, &rc, d_first, first_pose, 4 * static_cast<size_t>(n), cudaMemcpyHostToDevice, ctx->stream,
               "search first-pose flags");
    queue_copy(ctx, &rc, d_gm, gm.data(), 8 * gm.size(), cudaMemcpyHostToDevice, ctx->stream, "search minima");
    if (!rc) rc = pxd_mc_search_dev(ctx, p, n, max_atoms, d_ids, d_w, d_first, d_start, d_out, d_tors, d_e, d_ps, d_nev,
                           d_st, d_gm, ctx->stream);
    std::vector<float> ho(nx), ht(nt);
    if (!rc) {
        queue_copy(ctx, &rc, ho.data(), d_out, 4 * nx, cudaMemcpyDeviceToHost, ctx->stream, "search poses");
        if (nt) queue_copy(ctx, &rc, ht.data(), d_tors, 4 * nt, cudaMemcpyDeviceToHost, ctx->stream, "search torsions");
        queue_copy(ctx, &rc, out_e, d_e, 8 * static_cast<size_t>(n), cudaMemcpyDeviceToHost, ctx->stream,
                   "search energies");
        queue_copy(ctx, &rc, out_ps, d_ps, 8 * static_cast<size_t>(n), cudaMemcpyDeviceToHost, ctx->stream,
                   "search pose scores");
        queue_copy(ctx, &rc, out_nev, d_nev, 4 * static_cast<size_t>(n), cudaMemcpyDeviceToHost, ctx->stream,
                   "search evaluations");
        queue_copy(ctx, &rc, out_st, d_st, 4 * static_cast<size_t>(n), cudaMemcpyDeviceToHost, ctx->stream,
                   "search status");
        queue_copy(ctx, &rc, gm.data(), d_gm, 8 * gm.size(), cudaMemcpyDeviceToHost, ctx->stream, "search minima");
    }
    cudaFreeAsync(mem, ctx->stream);
    rc = sync_copies(ctx, rc, ctx->stream, "search");
    if (rc) return rc;
    int err[2] = {0, 0};
    rc = cuda_check(ctx, cudaMemcpy(err, ctx->d_counter + 1, 2 * sizeof(int), cudaMemcpyDeviceToHost),
                    "search flags");
    if (rc) return rc;
    for (size_t i = 0; i < nx; ++i) out_xyz[i] = ho[i];
    for (size_t i = 0; i < nt; ++i) out_tors[i] = ht[i];
    if (global_min)
        for (size_t i = 0; i < nl; ++i) global_min[i] = gm[i];
    if (err[1])
        return set_error(ctx, PXD_ERR_DEVICE_FLAG, "a search team stopped waiting at a barrier (walkers with status 3)");
    if (err[0]) return set_error(ctx, PXD_ERR_DEVICE_FLAG, "a random start found no pose inside the box");
    return PXD_OK;
}

int pxd_rng_draws(pxd_context* ctx, uint32_t seed, int32_t n, const int32_t* kinds, const int32_t* ints, double* out) {
    if (!ctx || n < 0 || (n > 0 && (!kinds || !ints || !out))) return PXD_ERR_INVALID;
    cudaSetDevice(ctx->device);
    int total = 0;
    for (int i = 0; i < n; ++i) {
        if (kinds[i] < 0 || kinds[i] > 4) return set_error(ctx, PXD_ERR_INVALID, "draw kind");
        if (kinds[i] == 0 && ints[i] < 0) return set_error(ctx, PXD_ERR_INVALID, "draw range");
        total += kinds[i] == 3 ? 3 : kinds[i] == 4 ? 4 : 1;
    }
    void* mem = nullptr;
    const size_t bytes = 8 * static_cast<size_t>(total) + 8 * static_cast<size_t>(n) + sizeof(MtState) + 64;
    int rc = cuda_check(ctx, cudaMallocAsync(&mem, bytes, ctx->stream), "rng staging");
    if (rc) return rc;
    double* d_out = static_cast<double*>(mem);
    int* d_k = reinterpret_cast<int*>(d_out + total);
    int* d_i = d_k + n;
    MtState* d_s = reinterpret_cast<MtState*>(reinterpret_cast<char*>(d_i + n) + (16 - ((8 * total + 8 * n) % 16)) % 16);
    queue_copy(ctx, &rc, d_k, kinds, 4 * static_cast<size_t>(n), cudaMemcpyHostToDevice, ctx->stream, "draw kinds");
    queue_copy(ctx, &rc, d_i, ints, 4 * static_cast<size_t>(n), cudaMemcpyHostToDevice, ctx->stream, "draw bounds");
    if (!rc) {
        rng_draws_kernel<<<1, 32, 0, ctx->stream>>>(seed, n, d_k, d_i, d_out, d_s);
        rc = cuda_check(ctx, cudaGetLastError(), "rng_draws_kernel launch");
    }
    queue_copy(ctx, &rc, out, d_out, 8 * static_cast<size_t>(total), cudaMemcpyDeviceToHost, ctx->stream, "draws");
    cudaFreeAsync(mem, ctx->stream);
    return sync_copies(ctx, rc, ctx->stream, "rng draws");
}

}  // extern "C"
