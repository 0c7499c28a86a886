// C ABI of the GB300 docking library: context, receptor, maps, ligands and the batch
// entry points declared in include/pxdock_gb300.h.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pxdock_gb300_vdw.h"
#include "pxd_internal.h"
#include "schedule.h"

namespace pxd {

static float bits_as_float(int v) {
    float f;
    std::memcpy(&f, &v, sizeof(f));
    return f;
}

constexpr double kCoulomb = 332.0637141491396;  // kCoulombFactor (system.h:83)
constexpr double kCoul14 = 0.833333333;         // interaction.h:52
constexpr double kVdw14 = 0.5;                  // interaction.h:53

int set_error(pxd_context* ctx, int code, const std::string& msg) {
    if (ctx) ctx->error = msg;
    return code;
}

int cuda_check(pxd_context* ctx, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return PXD_OK;
    return set_error(ctx, e == cudaErrorMemoryAllocation ? PXD_ERR_NOMEM : PXD_ERR_CUDA,
                     std::string(what) + ": " + cudaGetErrorString(e));
}

int raise_smem_limit(pxd_context* ctx, const void* fn, size_t bytes, const char* what) {
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> limit;
    std::lock_guard<std::mutex> lock(mu);
    size_t& cur = limit[{ctx->device, fn}];
    if (bytes <= cur) return PXD_OK;
    const int rc = cuda_check(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        static_cast<int>(bytes)),
                              what);
    if (!rc) cur = bytes;
    return rc;
}

template <class From, class To>
__global__ void convert_kernel(const From* __restrict__ in, To* __restrict__ out, size_t n) {
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x)
        out[i] = static_cast<To>(in[i]);
}

__global__ void fill_kernel(int* out, int v, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = v;
}

// Element-wise type conversion of n values on stream s (grid-stride, at most 8 blocks per SM).
template <class From, class To>
void convert_on_device(const From* in, To* out, size_t n, int n_sm, cudaStream_t s) {
    if (n == 0) return;
    const size_t blocks = std::min<size_t>((n + 255) / 256, static_cast<size_t>(n_sm) * 8);
    convert_kernel<From, To><<<static_cast<unsigned>(blocks), 256, 0, s>>>(in, out, n);
}

void fill_on_device(int* out, int v, int n, int n_sm, cudaStream_t s) {
    if (n <= 0) return;
    const int blocks = std::min((n + 255) / 256, n_sm * 8);
    fill_kernel<<<blocks, 256, 0, s>>>(out, v, n);
}

int ensure_scratch(pxd_context* ctx, size_t bytes) {
    if (bytes <= ctx->scratch_bytes) return PXD_OK;
    if (ctx->scratch) {
        // a launch on any stream may still read the old slab
        cudaDeviceSynchronize();
        cudaFree(ctx->scratch);
        ctx->scratch = nullptr;
        ctx->scratch_bytes = 0;
    }
    int rc = cuda_check(ctx, cudaMalloc(&ctx->scratch, bytes), "scratch allocation");
    if (rc) return rc;
    ctx->scratch_bytes = bytes;
    return PXD_OK;
}

// --------------------------------------------------------- device packing
// A growing host image of one device allocation; every block is 16-byte aligned.
struct Packer {
    std::vector<unsigned char> bytes;
    template <class T>
    size_t put(const std::vector<T>& v) {
        size_t off = (bytes.size() + 15) / 16 * 16;
        bytes.resize(off + v.size() * sizeof(T) + 16);
        if (!v.empty()) std::memcpy(bytes.data() + off, v.data(), v.size() * sizeof(T));
        return off;
    }
};

template <class T>
const T* at(void* base, size_t off) {
    return reinterpret_cast<const T*>(static_cast<const unsigned char*>(base) + off);
}

struct TopoIn {
    int n_atoms;
    std::vector<double> q, sigma, eps;
    std::vector<std::array<int, 2>> bonds;
    std::vector<double> bond_k, bond_r0;
    std::vector<std::array<int, 3>> angles;
    std::vector<double> angle_k, angle_t0;
    std::vector<std::array<int, 4>> dih;             // impropers then propers
    std::vector<std::vector<std::array<double, 3>>> dih_terms;  // (k, n, phase) until n == 0
    std::vector<std::array<int, 2>> pairs;           // 1-4 then all
    std::vector<double> pair_sc, pair_sv;            // Coulomb / LJ scales
};

void append_dihedrals(TopoIn& t, int n, const int32_t* ids, const int32_t* per,
                      const double* phase, const double* k) {
    for (int d = 0; d < n; ++d) {
        t.dih.push_back({ids[4 * d], ids[4 * d + 1], ids[4 * d + 2], ids[4 * d + 3]});
        std::vector<std::array<double, 3>> terms;
        for (int u = 0; u < kMaxDihTerms; ++u) {
            if (per[6 * d + u] == 0) break;  // interaction.cpp:90
            terms.push_back({k[6 * d + u], static_cast<double>(per[6 * d + u]), phase[6 * d + u]});
        }
        t.dih_terms.push_back(terms);
    }
}

TopoIn topo_from_desc(const pxd_topology& f) {
    TopoIn t;
    t.n_atoms = f.n_atoms;
    t.q.assign(f.charge, f.charge + f.n_atoms);
    t.sigma.assign(f.sigma, f.sigma + f.n_atoms);
    t.eps.assign(f.epsilon, f.epsilon + f.n_atoms);
    for (int b = 0; b < f.n_bonds; ++b) {
        t.bonds.push_back({f.bond_atoms[2 * b], f.bond_atoms[2 * b + 1]});
        t.bond_k.push_back(f.bond_k[b]);
        t.bond_r0.push_back(f.bond_length[b]);
    }
    for (int a = 0; a < f.n_angles; ++a) {
        t.angles.push_back({f.angle_atoms[3 * a], f.angle_atoms[3 * a + 1], f.angle_atoms[3 * a + 2]});
        t.angle_k.push_back(f.angle_k[a]);
        t.angle_t0.push_back(f.angle_radian[a]);
    }
    append_dihedrals(t, f.n_impropers, f.improper_atoms, f.improper_periodicity, f.improper_phase,
                     f.improper_k);
    append_dihedrals(t, f.n_propers, f.proper_atoms, f.proper_periodicity, f.proper_phase,
                     f.proper_k);
    for (int p = 0; p < f.n_pairs14; ++p) {
        t.pairs.push_back({f.pairs14[2 * p], f.pairs14[2 * p + 1]});
        t.pair_sc.push_back(kCoul14);
        t.pair_sv.push_back(kVdw14);
    }
    for (int p = 0; p < f.n_pairs; ++p) {
        t.pairs.push_back({f.pairs[2 * p], f.pairs[2 * p + 1]});
        t.pair_sc.push_back(1.0);
        t.pair_sv.push_back(1.0);
    }
    return t;
}

bool topo_indices_ok(const TopoIn& t) {
    auto ok = [&](int a) { return a >= 0 && a < t.n_atoms; };
    for (auto& b : t.bonds) if (!ok(b[0]) || !ok(b[1]) || b[0] == b[1]) return false;
    for (auto& a : t.angles) if (!ok(a[0]) || !ok(a[1]) || !ok(a[2])) return false;
    for (auto& d : t.dih) if (!ok(d[0]) || !ok(d[1]) || !ok(d[2]) || !ok(d[3])) return false;
    for (auto& p : t.pairs) if (!ok(p[0]) || !ok(p[1]) || p[0] == p[1]) return false;
    return true;
}

struct TopoOffsets {
    int n_bond_slots, n_angle_slots, n_dih_slots, n_pair_slots;
    size_t bond_ij, bond_p, angle_ijk, angle_p, dih_ijkl, dih_terms, dih_term, pair_ij, pair_p;
    size_t bond_p64, angle_p64, dih_term64, pair_p64;
};

TopoOffsets pack_topo(Packer& pk, const TopoIn& t) {
    TopoOffsets o{};
    {
        auto order = schedule_rounds<2>(t.bonds, t.n_atoms);
        std::vector<int2> ij;
        std::vector<float2> p;
        std::vector<double2> p64;
        for (int s : order) {
            if (s < 0) {
                ij.push_back(make_int2(-1, -1));
                p.push_back(make_float2(0.f, 0.f));
                p64.push_back(make_double2(0.0, 0.0));
            } else {
                const auto a = slot_atoms<2>(t.bonds, s);
                const int b = s & ~kReversed;
                ij.push_back(make_int2(a[0], a[1]));
                p.push_back(make_float2(static_cast<float>(t.bond_k[b]), static_cast<float>(t.bond_r0[b])));
                p64.push_back(make_double2(t.bond_k[b], t.bond_r0[b]));
            }
        }
        o.n_bond_slots = static_cast<int>(order.size());
        o.bond_ij = pk.put(ij);
        o.bond_p = pk.put(p);
        o.bond_p64 = pk.put(p64);
    }
    {
        auto order = schedule_rounds<3>(t.angles, t.n_atoms);
        std::vector<int4> ijk;
        std::vector<float2> p;
        std::vector<double2> p64;
        for (int s : order) {
            if (s < 0) {
                ijk.push_back(make_int4(-1, -1, -1, -1));
                p.push_back(make_float2(0.f, 0.f));
                p64.push_back(make_double2(0.0, 0.0));
            } else {
                const auto a = slot_atoms<3>(t.angles, s);
                const int b = s & ~kReversed;
                ijk.push_back(make_int4(a[0], a[1], a[2], 0));
                p.push_back(make_float2(static_cast<float>(t.angle_k[b]), static_cast<float>(t.angle_t0[b])));
                p64.push_back(make_double2(t.angle_k[b], t.angle_t0[b]));
            }
        }
        o.n_angle_slots = static_cast<int>(order.size());
        o.angle_ijk = pk.put(ijk);
        o.angle_p = pk.put(p);
        o.angle_p64 = pk.put(p64);
    }
    {
        auto order = schedule_rounds<4>(t.dih, t.n_atoms);
        std::vector<int4> ijkl;
        std::vector<int2> tr;
        std::vector<float4> terms;
        std::vector<double4> terms64;
        for (int s : order) {
            if (s < 0) {
                ijkl.push_back(make_int4(-1, -1, -1, -1));
                tr.push_back(make_int2(0, 0));
            } else {
                const auto a = slot_atoms<4>(t.dih, s);
                const int b = s & ~kReversed;
                ijkl.push_back(make_int4(a[0], a[1], a[2], a[3]));
                tr.push_back(make_int2(static_cast<int>(terms.size()), static_cast<int>(t.dih_terms[b].size())));
                for (auto& u : t.dih_terms[b]) {
                    terms.push_back(make_float4(static_cast<float>(u[0]), static_cast<float>(u[1]),
                                                static_cast<float>(u[2]), 0.f));
                    terms64.push_back(make_double4(u[0], u[1], u[2], 0.0));
                }
            }
        }
        o.n_dih_slots = static_cast<int>(order.size());
        o.dih_ijkl = pk.put(ijkl);
        o.dih_terms = pk.put(tr);
        o.dih_term = pk.put(terms);
        o.dih_term64 = pk.put(terms64);
    }
    {
        auto order = schedule_rounds<2>(t.pairs, t.n_atoms);
        std::vector<int2> ij;
        std::vector<float4> p;
        std::vector<double4> p64;
        for (int s : order) {
            if (s < 0) {
                ij.push_back(make_int2(-1, -1));
                p.push_back(make_float4(0.f, 0.f, 0.f, 0.f));
                p64.push_back(make_double4(0.0, 0.0, 0.0, 0.0));
                continue;
            }
            const auto a = slot_atoms<2>(t.pairs, s);
            const int i = a[0], j = a[1], b = s & ~kReversed;
            // pair.h:25-60: qq = qi qj scale; fused eps = sqrt(ei ej) scale 4; sigma mean
            const double A = t.q[i] * t.q[j] * t.pair_sc[b] * kCoulomb;
            const double C = std::sqrt(t.eps[i] * t.eps[j]) * t.pair_sv[b] * 4.0;
            const double sm = (t.sigma[i] + t.sigma[j]) * 0.5;
            ij.push_back(make_int2(i, j));
            p.push_back(make_float4(static_cast<float>(A), static_cast<float>(C),
                                    static_cast<float>(sm * sm), 0.f));
            p64.push_back(make_double4(A, C, sm * sm, 0.0));
        }
        o.n_pair_slots = static_cast<int>(order.size());
        o.pair_ij = pk.put(ij);
        o.pair_p = pk.put(p);
        o.pair_p64 = pk.put(p64);
    }
    return o;
}

DevTopo topo_pointers(void* base, int n_atoms, const TopoOffsets& o) {
    DevTopo d;
    d.n_atoms = n_atoms;
    d.n_bond_slots = o.n_bond_slots;
    d.n_angle_slots = o.n_angle_slots;
    d.n_dih_slots = o.n_dih_slots;
    d.n_pair_slots = o.n_pair_slots;
    d.bond_ij = at<int2>(base, o.bond_ij);
    d.bond_p = at<float2>(base, o.bond_p);
    d.angle_ijk = at<int4>(base, o.angle_ijk);
    d.angle_p = at<float2>(base, o.angle_p);
    d.dih_ijkl = at<int4>(base, o.dih_ijkl);
    d.dih_terms = at<int2>(base, o.dih_terms);
    d.dih_term = at<float4>(base, o.dih_term);
    d.pair_ij = at<int2>(base, o.pair_ij);
    d.pair_p = at<float4>(base, o.pair_p);
    d.bond_p64 = at<double2>(base, o.bond_p64);
    d.angle_p64 = at<double2>(base, o.angle_p64);
    d.dih_term64 = at<double4>(base, o.dih_term64);
    d.pair_p64 = at<double4>(base, o.pair_p64);
    return d;
}

// FP64 energy of the receptor terms that touch no rotor atom; they are constant for
// the whole run (the reference recomputes them every evaluation, interaction.cpp:286).
double constant_intra_energy(const TopoIn& t, const std::vector<double>& x,
                             const std::vector<uint8_t>& mov) {
    auto P = [&](int a) { return &x[3 * static_cast<size_t>(a)]; };
    auto touches = [&](std::initializer_list<int> ids) {
        for (int a : ids) if (mov[a]) return true;
        return false;
    };
    double e_b = 0, e_a = 0, e_d = 0, e1 = 0, e2 = 0;
    for (size_t b = 0; b < t.bonds.size(); ++b) {
        const int i = t.bonds[b][0], j = t.bonds[b][1];
        if (touches({i, j})) continue;
        const double dx = P(j)[0] - P(i)[0], dy = P(j)[1] - P(i)[1], dz = P(j)[2] - P(i)[2];
        const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
        e_b += 0.5 * t.bond_k[b] * (r - t.bond_r0[b]) * (r - t.bond_r0[b]);
    }
    for (size_t a = 0; a < t.angles.size(); ++a) {
        const int i = t.angles[a][0], j = t.angles[a][1], k = t.angles[a][2];
        if (touches({i, j, k})) continue;
        double v0[3], v1[3], c[3];
        for (int d = 0; d < 3; ++d) {
            v0[d] = P(j)[d] - P(i)[d];
            v1[d] = P(j)[d] - P(k)[d];
        }
        c[0] = v0[1] * v1[2] - v0[2] * v1[1];
        c[1] = v0[2] * v1[0] - v0[0] * v1[2];
        c[2] = v0[0] * v1[1] - v0[1] * v1[0];
        const double th = std::atan2(std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]),
                                     v0[0] * v1[0] + v0[1] * v1[1] + v0[2] * v1[2] + 1e-20);
        e_a += 0.5 * t.angle_k[a] * (th - t.angle_t0[a]) * (th - t.angle_t0[a]);
    }
    for (size_t d = 0; d < t.dih.size(); ++d) {
        const auto& q = t.dih[d];
        if (touches({q[0], q[1], q[2], q[3]})) continue;
        double rij[3], rkj[3], rkl[3], m[3], n[3], w[3];
        for (int u = 0; u < 3; ++u) {
            rij[u] = P(q[1])[u] - P(q[0])[u];
            rkj[u] = P(q[1])[u] - P(q[2])[u];
            rkl[u] = P(q[3])[u] - P(q[2])[u];
        }
        auto cross = [](const double* a, const double* b, double* c) {
            c[0] = a[1] * b[2] - a[2] * b[1];
            c[1] = a[2] * b[0] - a[0] * b[2];
            c[2] = a[0] * b[1] - a[1] * b[0];
        };
        cross(rij, rkj, m);
        cross(rkj, rkl, n);
        cross(m, n, w);
        const double phi = std::atan2(std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]),
                                      m[0] * n[0] + m[1] * n[1] + m[2] * n[2] + 1e-20);
        const double th = (rij[0] * n[0] + rij[1] * n[1] + rij[2] * n[2]) < 0 ? phi : -phi;
        for (auto& u : t.dih_terms[d]) e_d += u[0] * (1 + std::cos(th * u[1] - u[2]));
    }
    for (size_t p = 0; p < t.pairs.size(); ++p) {
        const int i = t.pairs[p][0], j = t.pairs[p][1];
        if (touches({i, j})) continue;
        const double dx = P(j)[0] - P(i)[0], dy = P(j)[1] - P(i)[1], dz = P(j)[2] - P(i)[2];
        const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
        e1 += t.q[i] * t.q[j] * t.pair_sc[p] / (r + 1e-20) * kCoulomb;
        const double s = (t.sigma[i] + t.sigma[j]) * 0.5;
        const double u6 = std::pow(s / (r + 1e-20), 6.0);
        e2 += (u6 * u6 - u6) * std::sqrt(t.eps[i] * t.eps[j]) * t.pair_sv[p] * 4.0;
    }
    return e_b + e_a + e_d + (e1 + e2);
}

void free_receptor(pxd_context* ctx) {
    if (ctx->rec_mem) cudaFree(ctx->rec_mem);
    if (ctx->rec_ex_all) cudaFree(ctx->rec_ex_all);
    if (ctx->rec_ex_mov) cudaFree(ctx->rec_ex_mov);
    if (ctx->rec_score_mem) cudaFree(ctx->rec_score_mem);
    ctx->rec_mem = ctx->rec_ex_all = ctx->rec_ex_mov = ctx->rec_score_mem = nullptr;
    ctx->rec_score = DevRecScore{};
    ctx->rec = DevReceptor{};
    ctx->has_receptor = false;
}

// Explicit-pair atom list: (position, charge), (sigma, epsilon), local rotor index.
int upload_explicit(pxd_context* ctx, const std::vector<int>& atoms, const std::vector<int>& local_of,
                    void** mem, size_t* offs) {
    Packer pk;
    std::vector<float4> xq;
    std::vector<float2> se;
    std::vector<int> loc;
    std::vector<double4> xq64;
    std::vector<double2> se64;
    for (int a : atoms) {
        xq64.push_back(make_double4(ctx->rec_xyz[3 * a], ctx->rec_xyz[3 * a + 1], ctx->rec_xyz[3 * a + 2],
                                    ctx->rec_charge[a]));
        se64.push_back(make_double2(ctx->rec_sigma[a], ctx->rec_epsilon[a]));
        xq.push_back(make_float4(static_cast<float>(ctx->rec_xyz[3 * a]),
                                 static_cast<float>(ctx->rec_xyz[3 * a + 1]),
                                 static_cast<float>(ctx->rec_xyz[3 * a + 2]),
                                 static_cast<float>(ctx->rec_charge[a])));
        se.push_back(make_float2(static_cast<float>(ctx->rec_sigma[a]), static_cast<float>(ctx->rec_epsilon[a])));
        // only rotor atoms move; every other atom keeps its stored position
        loc.push_back(ctx->is_mov[a] ? local_of[a] : -1);
    }
    offs[0] = pk.put(xq);
    offs[1] = pk.put(se);
    offs[2] = pk.put(loc);
    offs[3] = pk.put(xq64);
    offs[4] = pk.put(se64);
    int rc = cuda_check(ctx, cudaMalloc(mem, pk.bytes.size()), "receptor explicit list");
    if (rc) return rc;
    return cuda_check(ctx, cudaMemcpy(*mem, pk.bytes.data(), pk.bytes.size(), cudaMemcpyHostToDevice),
                      "receptor explicit copy");
}

void point_explicit(pxd_context* ctx, bool with_maps) {
    const int n = with_maps ? ctx->n_ex_mov : ctx->n_ex_all;
    void* mem = with_maps ? ctx->rec_ex_mov : ctx->rec_ex_all;
    const size_t* o = with_maps ? ctx->ex_mov_off : ctx->ex_all_off;
    ctx->rec.n_explicit = n;
    ctx->rec.ex_xyzq = at<float4>(mem, o[0]);
    ctx->rec.ex_se = at<float2>(mem, o[1]);
    ctx->rec.ex_local = at<int>(mem, o[2]);
    ctx->rec.ex_xyzq64 = at<double4>(mem, o[3]);
    ctx->rec.ex_se64 = at<double2>(mem, o[4]);
}

int sync_ligand_table(pxd_context* ctx) {
    if (!ctx->ligands_dirty) return PXD_OK;
    const int n = static_cast<int>(ctx->ligands.size());
    if (n > ctx->d_ligands_cap) {
        if (ctx->d_ligands) cudaFree(ctx->d_ligands);
        ctx->d_ligands = nullptr;
        ctx->d_ligands_cap = 0;
        const int cap = std::max(16, n * 2);
        int rc = cuda_check(ctx, cudaMalloc(&ctx->d_ligands, sizeof(DevLigand) * cap), "ligand table");
        if (rc) return rc;
        ctx->d_ligands_cap = cap;
    }
    std::vector<DevLigand> host(n);
    for (int i = 0; i < n; ++i) host[i] = ctx->ligands[i].dev;
    if (n > 0) {
        int rc = cuda_check(ctx, cudaMemcpyAsync(ctx->d_ligands, host.data(), sizeof(DevLigand) * n,
                                                 cudaMemcpyHostToDevice, ctx->stream),
                            "ligand table copy");
        if (rc) return rc;
        rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "ligand table sync");
        if (rc) return rc;
    }
    ctx->ligands_dirty = false;
    return PXD_OK;
}

// Rewrites every ligand's per-atom map slots after the maps changed.
int refresh_ligand_slots(pxd_context* ctx) {
    for (auto& e : ctx->ligands) {
        std::vector<int> slots(e.n_atoms, -1);
        for (int a = 0; a < e.n_atoms; ++a) {
            if (ctx->grid.has_grid) {
                const int s = ctx->type_slot[e.types[a]];
                if (s < 0)
                    return set_error(ctx, PXD_ERR_STATE,
                                     "no map for ligand vdW type " + std::to_string(e.types[a]) + " (" +
                                         PXD_VDW_TAGS[e.types[a]] + ")");
                slots[a] = s;
            }
        }
        int rc = cuda_check(ctx, cudaMemcpy(const_cast<int*>(e.dev.map_slot), slots.data(),
                                            sizeof(int) * e.n_atoms, cudaMemcpyHostToDevice),
                            "map slot refresh");
        if (rc) return rc;
    }
    return PXD_OK;
}

}  // namespace pxd

using namespace pxd;



extern "C" {

int32_t pxd_abi_version(void) { return PXD_ABI_VERSION; }

const char* pxd_version(void) { return "pxdock-gb300 1.0 (sm_103a)"; }

int pxd_context_create(int32_t device, pxd_context** out) {
    if (!out) return PXD_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return PXD_ERR_CUDA;
    if (cudaSetDevice(device) != cudaSuccess) return PXD_ERR_CUDA;
    auto* ctx = new pxd_context;
    ctx->device = device;
    for (int t = 0; t < PXD_NUM_VDW_TYPES; ++t) ctx->type_slot[t] = -1;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaDeviceGetAttribute(&ctx->n_sm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaMalloc(&ctx->d_counter, sizeof(int) * 4) != cudaSuccess) {
        delete ctx;
        return PXD_ERR_CUDA;
    }
    *out = ctx;
    return PXD_OK;
}

void pxd_context_destroy(pxd_context* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    release_l2_residency(ctx);
    pxd_clear_ligands(ctx);
    pxd_grid_drop(ctx);
    free_receptor(ctx);
    if (ctx->d_ligands) cudaFree(ctx->d_ligands);
    for (int k = 0; k < 2; ++k)
        if (ctx->d_sf[k]) cudaFree(ctx->d_sf[k]);
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->d_counter) cudaFree(ctx->d_counter);
    for (auto& cs : ctx->class_streams)
        if (cs) {
            cudaStreamSynchronize(cs);
            cudaStreamDestroy(cs);
        }
    for (auto& ev : ctx->class_events)
        if (ev) cudaEventDestroy(ev);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* pxd_last_error(const pxd_context* ctx) { return ctx ? ctx->error.c_str() : ""; }

void* pxd_context_stream(pxd_context* ctx) { return ctx ? ctx->stream : nullptr; }

void pxd_lbfgs_defaults(pxd_lbfgs_params* p) {
    p->max_iter = 240;
    p->max_eval = 0;
    p->history = 100;
    p->ls_max = 25;
    p->lr = 1.0;
    p->tolerance_grad = 0.5;
    p->tolerance_change = 1e-4;
    p->ls_c1 = 1e-4;
    p->ls_c2 = 0.9;
    p->ls_tolerance_change = 1e-9;
    p->ls_gtd_threshold = 1e5;
    p->reset_threshold = 1e8;
    p->dof_mode = PXD_DOF_CARTESIAN;
    p->reserved = 0;
}

int pxd_set_receptor(pxd_context* ctx, const pxd_receptor_desc* r) {
    if (!ctx || !r || r->n_atoms < 0 || (r->n_atoms > 0 && !r->xyz))
        return set_error(ctx, PXD_ERR_INVALID, "invalid receptor");
    if (r->ff.n_atoms != r->n_atoms) return set_error(ctx, PXD_ERR_INVALID, "receptor force field size");
    if (r->n_rotors > PXD_MAX_RECEPTOR_TORSIONS)
        return set_error(ctx, PXD_ERR_INVALID, "too many receptor rotors");
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    pxd_grid_drop(ctx);
    free_receptor(ctx);
    const int M = r->n_atoms;
    ctx->n_rec = M;
    ctx->rec_xyz.assign(r->xyz, r->xyz + 3 * static_cast<size_t>(M));
    ctx->rec_charge.assign(r->ff.charge, r->ff.charge + M);
    ctx->rec_sigma.assign(r->ff.sigma, r->ff.sigma + M);
    ctx->rec_epsilon.assign(r->ff.epsilon, r->ff.epsilon + M);
    // rotor leaves (torsional_receptor::parse, data.cpp:349-363)
    ctx->mov_atoms.clear();
    ctx->mov_rotor.clear();
    ctx->rotor_mov_off.assign(1, 0);
    ctx->rotor_origin.clear();
    ctx->rotor_axis.clear();
    ctx->is_mov.assign(M, 0);
    for (int k = 0; k < r->n_rotors; ++k) {
        const int a0 = r->rotor_axis[2 * k], a1 = r->rotor_axis[2 * k + 1];
        if (a0 < 0 || a0 >= M || a1 < 0 || a1 >= M)
            return set_error(ctx, PXD_ERR_INVALID, "rotor axis atom out of range");
        double ax[3];
        for (int d = 0; d < 3; ++d) {
            ctx->rotor_origin.push_back(r->xyz[3 * a0 + d]);
            ax[d] = r->xyz[3 * a1 + d] - r->xyz[3 * a0 + d];
        }
        const double n = std::sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
        for (int d = 0; d < 3; ++d) ctx->rotor_axis.push_back(ax[d] / n);
        for (int u = r->rotor_offsets[k]; u < r->rotor_offsets[k + 1]; ++u) {
            const int j = r->rotor_atoms[u];
            if (j < 0 || j >= M) return set_error(ctx, PXD_ERR_INVALID, "rotor atom out of range");
            if (j == a1) continue;
            ctx->mov_atoms.push_back(j);
            ctx->mov_rotor.push_back(k);
            ctx->is_mov[j] = 1;
        }
        ctx->rotor_mov_off.push_back(static_cast<int>(ctx->mov_atoms.size()));
    }
    const int n_mov = static_cast<int>(ctx->mov_atoms.size());
    // receptor intra terms: the rotor-touching ones go to the device over a compact
    // local atom space, the rest is a constant
    TopoIn full = topo_from_desc(r->ff);
    if (!topo_indices_ok(full)) return set_error(ctx, PXD_ERR_INVALID, "receptor term atom out of range");
    std::vector<int> local_of(M, -1);
    std::vector<int> locals;
    for (int k = 0; k < n_mov; ++k) {
        local_of[ctx->mov_atoms[k]] = static_cast<int>(locals.size());
        locals.push_back(ctx->mov_atoms[k]);
    }
    auto loc = [&](int a) {
        if (local_of[a] < 0) {
            local_of[a] = static_cast<int>(locals.size());
            locals.push_back(a);
        }
        return local_of[a];
    };
    TopoIn sub;
    auto mv = [&](std::initializer_list<int> ids) {
        for (int a : ids) if (ctx->is_mov[a]) return true;
        return false;
    };
    for (size_t b = 0; b < full.bonds.size(); ++b) {
        auto& q = full.bonds[b];
        if (!mv({q[0], q[1]})) continue;
        sub.bonds.push_back({loc(q[0]), loc(q[1])});
        sub.bond_k.push_back(full.bond_k[b]);
        sub.bond_r0.push_back(full.bond_r0[b]);
    }
    for (size_t a = 0; a < full.angles.size(); ++a) {
        auto& q = full.angles[a];
        if (!mv({q[0], q[1], q[2]})) continue;
        sub.angles.push_back({loc(q[0]), loc(q[1]), loc(q[2])});
        sub.angle_k.push_back(full.angle_k[a]);
        sub.angle_t0.push_back(full.angle_t0[a]);
    }
    for (size_t d = 0; d < full.dih.size(); ++d) {
        auto& q = full.dih[d];
        if (!mv({q[0], q[1], q[2], q[3]})) continue;
        sub.dih.push_back({loc(q[0]), loc(q[1]), loc(q[2]), loc(q[3])});
        sub.dih_terms.push_back(full.dih_terms[d]);
    }
    for (size_t p = 0; p < full.pairs.size(); ++p) {
        auto& q = full.pairs[p];
        if (!mv({q[0], q[1]})) continue;
        sub.pairs.push_back({loc(q[0]), loc(q[1])});
        sub.pair_sc.push_back(full.pair_sc[p]);
        sub.pair_sv.push_back(full.pair_sv[p]);
    }
    const int n_local = static_cast<int>(locals.size());
    sub.n_atoms = n_local;
    for (int a : locals) {
        sub.q.push_back(ctx->rec_charge[a]);
        sub.sigma.push_back(ctx->rec_sigma[a]);
        sub.eps.push_back(ctx->rec_epsilon[a]);
    }
    const double e_const = constant_intra_energy(full, ctx->rec_xyz, ctx->is_mov);
    Packer pk;
    std::vector<float4> origin, axis, local_xyz0;
    std::vector<double4> origin64, axis64, local64;
    for (int k = 0; k < r->n_rotors; ++k) {
        origin64.push_back(make_double4(ctx->rotor_origin[3 * k], ctx->rotor_origin[3 * k + 1],
                                        ctx->rotor_origin[3 * k + 2], 0.0));
        axis64.push_back(make_double4(ctx->rotor_axis[3 * k], ctx->rotor_axis[3 * k + 1], ctx->rotor_axis[3 * k + 2],
                                      0.0));
        origin.push_back(make_float4(static_cast<float>(ctx->rotor_origin[3 * k]),
                                     static_cast<float>(ctx->rotor_origin[3 * k + 1]),
                                     static_cast<float>(ctx->rotor_origin[3 * k + 2]), 0.f));
        axis.push_back(make_float4(static_cast<float>(ctx->rotor_axis[3 * k]),
                                   static_cast<float>(ctx->rotor_axis[3 * k + 1]),
                                   static_cast<float>(ctx->rotor_axis[3 * k + 2]), 0.f));
    }
    for (int l = 0; l < n_local; ++l) {
        const int a = locals[l];
        if (l < n_mov) {
            const int k = ctx->mov_rotor[l];
            local64.push_back(make_double4(ctx->rec_xyz[3 * a] - ctx->rotor_origin[3 * k],
                                           ctx->rec_xyz[3 * a + 1] - ctx->rotor_origin[3 * k + 1],
                                           ctx->rec_xyz[3 * a + 2] - ctx->rotor_origin[3 * k + 2], k));
            local_xyz0.push_back(make_float4(
                static_cast<float>(ctx->rec_xyz[3 * a] - ctx->rotor_origin[3 * k]),
                static_cast<float>(ctx->rec_xyz[3 * a + 1] - ctx->rotor_origin[3 * k + 1]),
                static_cast<float>(ctx->rec_xyz[3 * a + 2] - ctx->rotor_origin[3 * k + 2]),
                bits_as_float(k)));
        } else {
            local64.push_back(make_double4(ctx->rec_xyz[3 * a], ctx->rec_xyz[3 * a + 1], ctx->rec_xyz[3 * a + 2],
                                           -1.0));
            local_xyz0.push_back(make_float4(static_cast<float>(ctx->rec_xyz[3 * a]),
                                             static_cast<float>(ctx->rec_xyz[3 * a + 1]),
                                             static_cast<float>(ctx->rec_xyz[3 * a + 2]), 0.f));
        }
    }
    const size_t o_origin = pk.put(origin);
    const size_t o_axis = pk.put(axis);
    const size_t o_rmov = pk.put(ctx->rotor_mov_off);
    const size_t o_local = pk.put(local_xyz0);
    const size_t o_origin64 = pk.put(origin64), o_axis64 = pk.put(axis64), o_local64 = pk.put(local64);
    TopoOffsets to = pack_topo(pk, sub);
    int rc = cuda_check(ctx, cudaMalloc(&ctx->rec_mem, pk.bytes.size()), "receptor allocation");
    if (rc) return rc;
    rc = cuda_check(ctx, cudaMemcpy(ctx->rec_mem, pk.bytes.data(), pk.bytes.size(), cudaMemcpyHostToDevice),
                    "receptor copy");
    if (rc) return rc;
    DevReceptor& d = ctx->rec;
    d.n_rotors = r->n_rotors;
    d.n_mov = n_mov;
    d.n_local = n_local;
    d.rotor_origin = at<float4>(ctx->rec_mem, o_origin);
    d.rotor_axis = at<float4>(ctx->rec_mem, o_axis);
    d.rotor_mov = at<int>(ctx->rec_mem, o_rmov);
    d.local_xyz0 = at<float4>(ctx->rec_mem, o_local);
    d.rotor_origin64 = at<double4>(ctx->rec_mem, o_origin64);
    d.rotor_axis64 = at<double4>(ctx->rec_mem, o_axis64);
    d.local_xyz064 = at<double4>(ctx->rec_mem, o_local64);
    d.intra = topo_pointers(ctx->rec_mem, n_local, to);
    d.e_const = e_const;
    // explicit pair lists: every atom (no maps) and the rotor atoms (maps present)
    std::vector<int> all(M);
    for (int a = 0; a < M; ++a) all[a] = a;
    rc = upload_explicit(ctx, all, local_of, &ctx->rec_ex_all, ctx->ex_all_off);
    if (rc) return rc;
    std::vector<int> movs(ctx->mov_atoms.begin(), ctx->mov_atoms.end());
    std::sort(movs.begin(), movs.end());  // grid.cpp:118-123 keeps them in a set
    rc = upload_explicit(ctx, movs, local_of, &ctx->rec_ex_mov, ctx->ex_mov_off);
    if (rc) return rc;
    ctx->n_ex_all = M;
    ctx->n_ex_mov = static_cast<int>(movs.size());
    point_explicit(ctx, false);
    rc = upload_receptor_scoring(ctx, r->lists, local_of);
    if (rc) return rc;
    ctx->has_receptor = true;
    ctx->ligands_dirty = true;
    return PXD_OK;
}

int pxd_decide_grid_dims(double cx, double cy, double cz, double sx, double sy, double sz,
                         double spacing, pxd_box* out) {
    if (!out || !(spacing > 0)) return PXD_ERR_INVALID;
    const double c[3] = {cx, cy, cz}, s[3] = {sx, sy, sz};
    for (int d = 0; d < 3; ++d) {
        long nv = static_cast<long>(std::ceil(s[d] / spacing));
        if (nv % 2 == 1) nv += 1;
        const double length = nv * spacing;
        out->npoints[d] = static_cast<int32_t>(nv + 1);
        out->init_xyz[d] = c[d] - length * 0.5;
    }
    out->spacing = spacing;
    return PXD_OK;
}

static int alloc_maps(pxd_context* ctx, const pxd_box* box, const std::vector<int>& types) {
    pxd_grid_drop(ctx);
    for (int d = 0; d < 3; ++d)
        if (box->npoints[d] < 2) return set_error(ctx, PXD_ERR_INVALID, "box needs >= 2 points per axis");
    const long long P = static_cast<long long>(box->npoints[0]) * box->npoints[1] * box->npoints[2];
    if (P > (1LL << 31) / 128) return set_error(ctx, PXD_ERR_INVALID, "box too large");
    ctx->box = *box;
    ctx->n_slots = 1 + static_cast<int>(types.size());
    for (int t = 0; t < PXD_NUM_VDW_TYPES; ++t) ctx->type_slot[t] = -1;
    for (size_t k = 0; k < types.size(); ++k) ctx->type_slot[types[k]] = 1 + static_cast<int>(k);
    // float4 records of every slot, then the FP32 residuals of their FP64 energies
    int rc = cuda_check(ctx, cudaMalloc(&ctx->maps, (sizeof(float4) + sizeof(float)) * P * ctx->n_slots),
                        "map allocation");
    if (rc) return rc;
    DevGrid& g = ctx->grid;
    g.has_grid = 1;
    g.init = make_float3(static_cast<float>(box->init_xyz[0]), static_cast<float>(box->init_xyz[1]),
                         static_cast<float>(box->init_xyz[2]));
    g.npts = make_int3(box->npoints[0], box->npoints[1], box->npoints[2]);
    float fl[3][4];
    for (int d = 0; d < 3; ++d) {
        const double lo = box->init_xyz[d], hi = box->init_xyz[d] + (box->npoints[d] - 1) * box->spacing;
        fl[d][0] = static_cast<float>(lo);
        fl[d][1] = static_cast<float>(lo - fl[d][0]);
        fl[d][2] = static_cast<float>(hi);
        fl[d][3] = static_cast<float>(hi - fl[d][2]);
    }
    g.lo_h = make_float3(fl[0][0], fl[1][0], fl[2][0]);
    g.lo_l = make_float3(fl[0][1], fl[1][1], fl[2][1]);
    g.hi_h = make_float3(fl[0][2], fl[1][2], fl[2][2]);
    g.hi_l = make_float3(fl[0][3], fl[1][3], fl[2][3]);
    g.spacing = static_cast<float>(box->spacing);
    g.spacing_inv = static_cast<float>(1.0 / box->spacing);
    g.slope = static_cast<float>(ctx->slope);
    g.P = static_cast<int>(P);
    g.maps = ctx->maps;
    g.e_lo = reinterpret_cast<const float*>(ctx->maps + P * ctx->n_slots);
    g.init64 = make_double3(box->init_xyz[0], box->init_xyz[1], box->init_xyz[2]);
    g.spacing64 = box->spacing;
    g.slope64 = ctx->slope;
    return PXD_OK;
}

static std::vector<int> type_list(const int32_t* types, int32_t n_types, int* rc) {
    std::vector<int> out;
    *rc = PXD_OK;
    if (n_types < 0) {
        for (int t = 0; t < PXD_NUM_VDW_TYPES; ++t) out.push_back(t);
        return out;
    }
    for (int k = 0; k < n_types; ++k) {
        if (types[k] < 0 || types[k] >= PXD_NUM_VDW_TYPES) {
            *rc = PXD_ERR_INVALID;
            return out;
        }
        if (std::find(out.begin(), out.end(), types[k]) == out.end()) out.push_back(types[k]);
    }
    return out;
}

int pxd_grid_build(pxd_context* ctx, const pxd_box* box, const int32_t* types, int32_t n_types) {
    if (!ctx || !box) return PXD_ERR_INVALID;
    if (!ctx->has_receptor) return set_error(ctx, PXD_ERR_STATE, "set a receptor first");
    cudaSetDevice(ctx->device);
    int rc;
    std::vector<int> tl = type_list(types, n_types, &rc);
    if (rc) return set_error(ctx, rc, "vdW type out of range");
    rc = alloc_maps(ctx, box, tl);
    if (rc) return rc;
    // non-rotor receptor atoms (grid.cpp:119-123, 173)
    std::vector<float4> xq, xl;
    std::vector<float2> se;
    std::vector<double2> se64;
    for (int a = 0; a < ctx->n_rec; ++a) {
        if (ctx->is_mov[a]) continue;
        se64.push_back(make_double2(ctx->rec_sigma[a], ctx->rec_epsilon[a]));
        const double* x = &ctx->rec_xyz[3 * a];
        const float4 hi = make_float4(static_cast<float>(x[0]), static_cast<float>(x[1]), static_cast<float>(x[2]),
                                      static_cast<float>(ctx->rec_charge[a]));
        xq.push_back(hi);
        xl.push_back(make_float4(static_cast<float>(x[0] - hi.x), static_cast<float>(x[1] - hi.y),
                                 static_cast<float>(x[2] - hi.z), static_cast<float>(ctx->rec_charge[a] - hi.w)));
        se.push_back(make_float2(static_cast<float>(ctx->rec_sigma[a]), static_cast<float>(ctx->rec_epsilon[a])));
    }
    std::vector<int> slot_type(ctx->n_slots, -1);
    for (size_t k = 0; k < tl.size(); ++k) slot_type[1 + k] = tl[k];
    Packer pk;
    const size_t o_xq = pk.put(xq), o_xl = pk.put(xl), o_se = pk.put(se), o_st = pk.put(slot_type);
    const size_t o_se64 = pk.put(se64);
    void* mem = nullptr;
    rc = cuda_check(ctx, cudaMalloc(&mem, pk.bytes.size()), "grid atom upload");
    if (rc) return rc;
    rc = cuda_check(ctx, cudaMemcpy(mem, pk.bytes.data(), pk.bytes.size(), cudaMemcpyHostToDevice), "grid atom copy");
    if (!rc)
        rc = launch_grid_build(ctx, at<float4>(mem, o_xq), at<float4>(mem, o_xl), at<float2>(mem, o_se),
                               at<double2>(mem, o_se64), static_cast<int>(xq.size()), at<int>(mem, o_st),
                               ctx->n_slots, ctx->maps, const_cast<float*>(ctx->grid.e_lo));
    cudaFree(mem);
    if (rc) {
        pxd_grid_drop(ctx);
        return rc;
    }
    point_explicit(ctx, true);
    rc = refresh_ligand_slots(ctx);
    ctx->ligands_dirty = true;
    if (rc) {
        const std::string msg = ctx->error;
        pxd_grid_drop(ctx);
        return set_error(ctx, rc, msg + " (maps dropped)");
    }
    return PXD_OK;
}

int pxd_grid_set_slope(pxd_context* ctx, double slope) {
    if (!ctx) return PXD_ERR_INVALID;
    ctx->slope = slope;
    ctx->grid.slope = static_cast<float>(slope);
    ctx->grid.slope64 = slope;
    return PXD_OK;
}

int pxd_grid_drop(pxd_context* ctx) {
    if (!ctx) return PXD_ERR_INVALID;
    if (ctx->maps) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(ctx->maps);
    }
    ctx->maps = nullptr;
    ctx->grid.has_grid = 0;
    ctx->grid.maps = nullptr;
    ctx->n_slots = 0;
    for (int t = 0; t < PXD_NUM_VDW_TYPES; ++t) ctx->type_slot[t] = -1;
    if (ctx->has_receptor) {
        point_explicit(ctx, false);
        refresh_ligand_slots(ctx);
    }
    return PXD_OK;
}

int pxd_grid_info(pxd_context* ctx, pxd_box* box, int32_t* n_maps) {
    if (!ctx) return PXD_ERR_INVALID;
    if (!ctx->grid.has_grid) return set_error(ctx, PXD_ERR_STATE, "no maps");
    if (box) *box = ctx->box;
    if (n_maps) *n_maps = ctx->n_slots;
    return PXD_OK;
}

static int map_slot(pxd_context* ctx, int32_t map) {
    if (map == PXD_NUM_VDW_TYPES) return 0;
    if (map >= 0 && map < PXD_NUM_VDW_TYPES) return ctx->type_slot[map];
    return -1;
}

int pxd_grid_read_map(pxd_context* ctx, int32_t map, float* host_out) {
    if (!ctx || !host_out) return PXD_ERR_INVALID;
    if (!ctx->grid.has_grid) return set_error(ctx, PXD_ERR_STATE, "no maps");
    const int slot = map_slot(ctx, map);
    if (slot < 0) return set_error(ctx, PXD_ERR_INVALID, "map not built");
    cudaSetDevice(ctx->device);
    return cuda_check(ctx, cudaMemcpy(host_out, ctx->maps + static_cast<size_t>(slot) * ctx->grid.P,
                                      sizeof(float4) * ctx->grid.P, cudaMemcpyDeviceToHost),
                      "map read");
}

int pxd_grid_read_map64(pxd_context* ctx, int32_t map, double* host_out) {
    if (!ctx || !host_out) return PXD_ERR_INVALID;
    if (!ctx->grid.has_grid) return set_error(ctx, PXD_ERR_STATE, "no maps");
    const int slot = map_slot(ctx, map);
    if (slot < 0) return set_error(ctx, PXD_ERR_INVALID, "map not built");
    const size_t P = ctx->grid.P;
    std::vector<float4> rec(P);
    std::vector<float> lo(P);
    cudaSetDevice(ctx->device);
    int rc = cuda_check(ctx, cudaMemcpy(rec.data(), ctx->maps + static_cast<size_t>(slot) * P, sizeof(float4) * P,
                                        cudaMemcpyDeviceToHost),
                        "map read");
    if (!rc)
        rc = cuda_check(ctx, cudaMemcpy(lo.data(), ctx->grid.e_lo + static_cast<size_t>(slot) * P, sizeof(float) * P,
                                        cudaMemcpyDeviceToHost),
                        "map remainder read");
    if (rc) return rc;
    for (size_t p = 0; p < P; ++p) {
        host_out[4 * p] = static_cast<double>(rec[p].x) + static_cast<double>(lo[p]);
        host_out[4 * p + 1] = rec[p].y;
        host_out[4 * p + 2] = rec[p].z;
        host_out[4 * p + 3] = rec[p].w;
    }
    return PXD_OK;
}

// Installs one map's FP32 records and FP64 energy remainders (e_lo_host, or zeros).
static int install_map(pxd_context* ctx, const pxd_box* box, int32_t map, const float* host_records,
                       const float* e_lo_host) {
    if (map < 0 || map > PXD_NUM_VDW_TYPES) return set_error(ctx, PXD_ERR_INVALID, "map index");
    cudaSetDevice(ctx->device);
    const bool same = ctx->grid.has_grid && std::memcmp(&ctx->box, box, sizeof(pxd_box)) == 0;
    if (!same || (map < PXD_NUM_VDW_TYPES && ctx->type_slot[map] < 0)) {
        // (re)allocate with every vdW type so that maps can be installed one by one
        std::vector<int> all;
        for (int t = 0; t < PXD_NUM_VDW_TYPES; ++t) all.push_back(t);
        int rc = alloc_maps(ctx, box, all);
        if (rc) return rc;
        rc = cuda_check(ctx, cudaMemset(ctx->maps, 0, (sizeof(float4) + sizeof(float)) * ctx->grid.P * ctx->n_slots),
                        "map clear");
        if (rc) return rc;
    }
    const int slot = map == PXD_NUM_VDW_TYPES ? 0 : ctx->type_slot[map];
    int rc = cuda_check(ctx, cudaMemcpy(ctx->maps + static_cast<size_t>(slot) * ctx->grid.P, host_records,
                                        sizeof(float4) * ctx->grid.P, cudaMemcpyHostToDevice),
                        "map write");
    if (rc) return rc;
    float* lo = const_cast<float*>(ctx->grid.e_lo) + static_cast<size_t>(slot) * ctx->grid.P;
    if (e_lo_host)
        rc = cuda_check(ctx, cudaMemcpy(lo, e_lo_host, sizeof(float) * ctx->grid.P, cudaMemcpyHostToDevice),
                        "map remainder write");
    else  // an installed FP32 record set carries no FP64 remainder: its energies are the records'
        rc = cuda_check(ctx, cudaMemset(lo, 0, sizeof(float) * ctx->grid.P), "map remainder clear");
    if (rc) return rc;
    if (ctx->has_receptor) point_explicit(ctx, true);
    rc = refresh_ligand_slots(ctx);
    ctx->ligands_dirty = true;
    if (rc) {
        const std::string msg = ctx->error;
        pxd_grid_drop(ctx);
        return set_error(ctx, rc, msg + " (maps dropped)");
    }
    return PXD_OK;
}

int pxd_grid_write_map(pxd_context* ctx, const pxd_box* box, int32_t map, const float* host_records) {
    if (!ctx || !box || !host_records) return PXD_ERR_INVALID;
    return install_map(ctx, box, map, host_records, nullptr);
}

int pxd_grid_write_map64(pxd_context* ctx, const pxd_box* box, int32_t map, const double* host_records) {
    if (!ctx || !box || !host_records) return PXD_ERR_INVALID;
    const size_t P = static_cast<size_t>(box->npoints[0]) * box->npoints[1] * box->npoints[2];
    if (box->npoints[0] < 2 || box->npoints[1] < 2 || box->npoints[2] < 2)
        return set_error(ctx, PXD_ERR_INVALID, "points per axis");
    std::vector<float> rec(4 * P), lo(P);
    for (size_t p = 0; p < P; ++p) {
        const double e = host_records[4 * p];
        // the grid build's record rule: clamp to +-1e30, E rounded to FP32, remainder kept
        const double ec = std::fmin(std::fmax(e, -1e30), 1e30);
        const float hi = static_cast<float>(ec);
        rec[4 * p] = hi;
        lo[p] = std::fabs(e) < 1e30 ? static_cast<float>(e - static_cast<double>(hi)) : 0.f;
        for (int c = 1; c < 4; ++c)
            rec[4 * p + c] = static_cast<float>(std::fmin(std::fmax(host_records[4 * p + c], -1e30), 1e30));
    }
    return install_map(ctx, box, map, rec.data(), lo.data());
}

int pxd_add_ligand(pxd_context* ctx, const pxd_ligand_desc* lig, int32_t* ligand_id) {
    if (!ctx || !lig || !ligand_id) return PXD_ERR_INVALID;
    const int N = lig->ff.n_atoms;
    if (N <= 0 || N > PXD_MAX_LIGAND_ATOMS)
        return set_error(ctx, PXD_ERR_INVALID, "ligand atom count out of range (1.." +
                                                   std::to_string(PXD_MAX_LIGAND_ATOMS) + ")");
    for (int a = 0; a < N; ++a)
        if (lig->vdw_type[a] < 0 || lig->vdw_type[a] >= PXD_NUM_VDW_TYPES)
            return set_error(ctx, PXD_ERR_INVALID, "VDW type of atom#" + std::to_string(a) + " is illegal");
    cudaSetDevice(ctx->device);
    TopoIn t = topo_from_desc(lig->ff);
    if (!topo_indices_ok(t)) return set_error(ctx, PXD_ERR_INVALID, "ligand term atom out of range");
    Packer pk;
    const TopoOffsets to = pack_topo(pk, t);
    std::vector<float> q(N);
    std::vector<int> slots(N, -1), types(lig->vdw_type, lig->vdw_type + N);
    std::vector<float2> se(N);
    std::vector<double> q64(N);
    std::vector<double2> se64(N);
    for (int a = 0; a < N; ++a) {
        q64[a] = lig->ff.charge[a];
        se64[a] = make_double2(PXD_VDW_SIGMA[types[a]], PXD_VDW_EPSILON[types[a]]);
        q[a] = static_cast<float>(lig->ff.charge[a]);
        se[a] = make_float2(static_cast<float>(PXD_VDW_SIGMA[types[a]]), static_cast<float>(PXD_VDW_EPSILON[types[a]]));
        if (ctx->grid.has_grid) {
            slots[a] = ctx->type_slot[types[a]];
            if (slots[a] < 0)
                return set_error(ctx, PXD_ERR_STATE, std::string("no map for ligand vdW type ") + PXD_VDW_TAGS[types[a]]);
        }
    }
    const size_t o_q = pk.put(q), o_slot = pk.put(slots), o_se = pk.put(se), o_type = pk.put(types);
    const size_t o_q64 = pk.put(q64), o_se64 = pk.put(se64);
    // torsion tree
    const pxd_torsion_tree& tr = lig->tree;
    if (tr.n_frags > 0) {
        bool ok = tr.n_roots >= 1 && tr.n_torsions == tr.n_frags - tr.n_roots && tr.n_torsions <= kWarp &&
                  tr.n_frags <= 64;
        std::vector<int> seen(N, 0);
        for (int p = 0; ok && p < N; ++p) {
            ok = tr.perm[p] >= 0 && tr.perm[p] < N && !seen[tr.perm[p]];
            if (ok) seen[tr.perm[p]] = 1;
        }
        for (int f = 0; ok && f < tr.n_frags; ++f)
            ok = tr.frag_start[f] >= 0 && tr.frag_start[f] <= tr.frag_end[f] && tr.frag_end[f] <= N;
        for (int r = 0; ok && r < tr.n_roots; ++r) ok = tr.roots[r] >= 0 && tr.roots[r] < tr.n_frags;
        for (int k = 0; ok && k < tr.n_torsions; ++k)
            ok = tr.tors_frag[k] >= 0 && tr.tors_frag[k] < tr.n_frags && tr.tors_parent[k] >= 0 &&
                 tr.tors_parent[k] < tr.n_frags && tr.tors_parent_atom[k] >= 0 && tr.tors_parent_atom[k] < N &&
                 tr.tors_mine_atom[k] >= 0 && tr.tors_mine_atom[k] < N;
        if (!ok) return set_error(ctx, PXD_ERR_INVALID, "invalid torsion tree (at most 64 fragments, 32 torsions)");
    }
    std::vector<int> perm, frange, isroot;
    std::vector<int4> tors;
    if (tr.n_frags > 0) {
        perm.assign(tr.perm, tr.perm + N);
        for (int f = 0; f < tr.n_frags; ++f) {
            frange.push_back(tr.frag_start[f]);
            frange.push_back(tr.frag_end[f]);
        }
        isroot.assign(tr.n_frags, 0);
        for (int r = 0; r < tr.n_roots; ++r) isroot[tr.roots[r]] = 1;
        for (int k = 0; k < tr.n_torsions; ++k)
            tors.push_back(make_int4(tr.tors_frag[k], tr.tors_parent[k], tr.tors_parent_atom[k], tr.tors_mine_atom[k]));
    }
    std::vector<int> frag_of(N, 0), frag_mine(tr.n_frags, -1), frag_parent(tr.n_frags, -1);
    for (int f = 0; f < tr.n_frags; ++f)
        for (int p = tr.frag_start[f]; p < tr.frag_end[f]; ++p) frag_of[p] = f;
    for (int k = 0; k < tr.n_torsions; ++k) {
        frag_mine[tr.tors_frag[k]] = tr.tors_mine_atom[k];
        frag_parent[tr.tors_frag[k]] = tr.tors_parent[k];
    }
    const size_t o_perm = pk.put(perm), o_fr = pk.put(frange), o_tors = pk.put(tors), o_root = pk.put(isroot);
    const size_t o_fof = pk.put(frag_of), o_fmine = pk.put(frag_mine), o_fpar = pk.put(frag_parent);
    LigandEntry e;
    int rc = cuda_check(ctx, cudaMalloc(&e.mem, pk.bytes.size()), "ligand allocation");
    if (rc) return rc;
    rc = cuda_check(ctx, cudaMemcpy(e.mem, pk.bytes.data(), pk.bytes.size(), cudaMemcpyHostToDevice), "ligand copy");
    if (rc) {
        cudaFree(e.mem);
        return rc;
    }
    e.n_atoms = N;
    e.n_tors = tr.n_torsions;
    e.types = types;
    DevLigand& d = e.dev;
    d.topo = topo_pointers(e.mem, N, to);
    d.n_atoms = N;
    d.charge = at<float>(e.mem, o_q);
    d.map_slot = at<int>(e.mem, o_slot);
    d.se = at<float2>(e.mem, o_se);
    d.charge64 = at<double>(e.mem, o_q64);
    d.se64 = at<double2>(e.mem, o_se64);
    d.type = at<int>(e.mem, o_type);
    d.n_frags = tr.n_frags;
    d.n_tors = tr.n_torsions;
    d.perm = at<int>(e.mem, o_perm);
    d.frag_range = at<int>(e.mem, o_fr);
    d.tors = at<int4>(e.mem, o_tors);
    d.is_root = at<int>(e.mem, o_root);
    d.frag_of = at<int>(e.mem, o_fof);
    d.frag_mine = at<int>(e.mem, o_fmine);
    d.frag_parent = at<int>(e.mem, o_fpar);
    e.charge.assign(lig->ff.charge, lig->ff.charge + N);
    rc = upload_ligand_scoring(ctx, e, lig->lists);
    if (rc) {
        cudaFree(e.mem);
        return rc;
    }
    *ligand_id = static_cast<int32_t>(ctx->ligands.size());
    ctx->ligands.push_back(e);
    ctx->ligands_dirty = true;
    return PXD_OK;
}

int pxd_clear_ligands(pxd_context* ctx) {
    if (!ctx) return PXD_ERR_INVALID;
    cudaStreamSynchronize(ctx->stream);
    for (auto& e : ctx->ligands) {
        if (e.mem) cudaFree(e.mem);
        if (e.score_mem) cudaFree(e.score_mem);
    }
    ctx->ligands.clear();
    ctx->ligands_dirty = true;
    return PXD_OK;
}

static int check_ready(pxd_context* ctx) {
    if (!ctx) return PXD_ERR_INVALID;
    if (!ctx->has_receptor) return set_error(ctx, PXD_ERR_STATE, "set a receptor first");
    cudaSetDevice(ctx->device);
    return PXD_OK;
}

static cudaStream_t pick(pxd_context* ctx, void* s) {
    return s ? static_cast<cudaStream_t>(s) : ctx->stream;
}

int pxd_score_grad_dev(pxd_context* ctx, int32_t n_poses, int32_t max_atoms, const int32_t* ids,
                       const float* xyz, const float* tors, double* energy, float* lig_grad,
                       float* tors_grad, void* stream) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (n_poses < 0 || max_atoms <= 0 || max_atoms > PXD_MAX_LIGAND_ATOMS)
        return set_error(ctx, PXD_ERR_INVALID, "bad pose batch shape");
    if (ctx->rec.n_rotors > 0 && (!tors || !tors_grad))
        return set_error(ctx, PXD_ERR_INVALID, "receptor torsion buffers required");
    return launch_score(ctx, n_poses, max_atoms, ids, xyz, tors, energy, lig_grad, tors_grad, pick(ctx, stream));
}

int pxd_lbfgs_dev(pxd_context* ctx, const pxd_lbfgs_params* p, int32_t n_poses, int32_t max_atoms,
                  const int32_t* ids, float* xyz, float* tors, double* energy, int32_t* nevals,
                  int32_t* status, void* stream) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (!p || p->history < 1 || p->history > PXD_MAX_HISTORY || p->max_iter < 0 || p->ls_max < 1 ||
        (p->dof_mode != PXD_DOF_CARTESIAN && p->dof_mode != PXD_DOF_RIGID_TORSION))
        return set_error(ctx, PXD_ERR_INVALID, "bad L-BFGS parameters");
    if (n_poses < 0 || max_atoms <= 0 || max_atoms > PXD_MAX_LIGAND_ATOMS)
        return set_error(ctx, PXD_ERR_INVALID, "bad pose batch shape");
    if (ctx->rec.n_rotors > 0 && !tors) return set_error(ctx, PXD_ERR_INVALID, "receptor torsion buffer required");
    return launch_lbfgs(ctx, *p, n_poses, max_atoms, ids, xyz, tors, energy, nevals, status, pick(ctx, stream));
}

int pxd_lbfgs_dev_noalloc(pxd_context* ctx, const pxd_lbfgs_params* p, int32_t n_poses, int32_t max_atoms,
                          const int32_t* ids, float* xyz, float* tors, double* energy, int32_t* nevals,
                          int32_t* status, void* stream) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (!p || p->history < 1 || p->history > PXD_MAX_HISTORY || p->max_iter < 0 || p->ls_max < 1 ||
        (p->dof_mode != PXD_DOF_CARTESIAN && p->dof_mode != PXD_DOF_RIGID_TORSION))
        return set_error(ctx, PXD_ERR_INVALID, "bad L-BFGS parameters");
    if (n_poses < 0 || max_atoms <= 0 || max_atoms > PXD_MAX_LIGAND_ATOMS)
        return set_error(ctx, PXD_ERR_INVALID, "bad pose batch shape");
    if (ctx->rec.n_rotors > 0 && !tors) return set_error(ctx, PXD_ERR_INVALID, "receptor torsion buffer required");
    return launch_lbfgs_noalloc(ctx, *p, n_poses, max_atoms, ids, xyz, tors, energy, nevals, status,
                                pick(ctx, stream));
}

int pxd_score_grad(pxd_context* ctx, int32_t lig, int32_t n_poses, const double* xyz, const double* tors,
                   double* energy, double* lig_grad, double* tors_grad) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (lig < 0 || lig >= static_cast<int>(ctx->ligands.size()) || n_poses < 0)
        return set_error(ctx, PXD_ERR_INVALID, "ligand id");
    const int N = ctx->ligands[lig].n_atoms, R = ctx->rec.n_rotors;
    const size_t nx = static_cast<size_t>(n_poses) * N * 3, nt = static_cast<size_t>(n_poses) * R;
    std::vector<float> hx(nx), ht(nt);
    for (size_t i = 0; i < nx; ++i) hx[i] = static_cast<float>(xyz[i]);
    for (size_t i = 0; i < nt; ++i) ht[i] = static_cast<float>(tors[i]);
    std::vector<int> ids(n_poses, lig);
    Staging st{ctx, {}};
    float* dx = st.alloc<float>(nx, &rc);
    if (rc) return rc;
    float* dt = st.alloc<float>(nt, &rc);
    if (rc) return rc;
    float* dg = st.alloc<float>(nx, &rc);
    if (rc) return rc;
    float* dtg = st.alloc<float>(nt, &rc);
    if (rc) return rc;
    double* de = st.alloc<double>(n_poses, &rc);
    if (rc) return rc;
    int* di = st.alloc<int>(n_poses, &rc);
    if (rc) return rc;
    queue_copy(ctx, &rc, dx, hx.data(), nx * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
    if (nt) queue_copy(ctx, &rc, dt, ht.data(), nt * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
    queue_copy(ctx, &rc, di, ids.data(), n_poses * sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
    if (rc) return rc;
    rc = pxd_score_grad_dev(ctx, n_poses, N, di, dx, dt, de, dg, dtg, ctx->stream);
    if (rc) return rc;
    std::vector<float> hg(nx), htg(nt);
    queue_copy(ctx, &rc, energy, de, n_poses * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    queue_copy(ctx, &rc, hg.data(), dg, nx * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    if (nt) queue_copy(ctx, &rc, htg.data(), dtg, nt * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    rc = sync_copies(ctx, rc, ctx->stream, "score_grad");
    if (rc) return rc;
    for (size_t i = 0; i < nx; ++i) lig_grad[i] = hg[i];
    for (size_t i = 0; i < nt; ++i) tors_grad[i] = htg[i];
    return PXD_OK;
}

// The host-buffer optimiser calls: the caller's FP64 arrays are copied as they are and
// narrowed to FP32 (widened back) on the device, next to the kernel, instead of in loops
// over the whole batch on one host core. static_cast rounds to nearest on both sides, so the
// values are those of a host conversion.
static int lbfgs_host(pxd_context* ctx, const pxd_lbfgs_params* p, int32_t n_poses, int32_t max_atoms, int32_t lig,
                      const int32_t* ligand_ids, double* xyz, double* tors, double* energy, int32_t* nevals,
                      int32_t* status) {
    const int R = ctx->rec.n_rotors;
    const size_t nx = static_cast<size_t>(n_poses) * max_atoms * 3, nt = static_cast<size_t>(n_poses) * R;
    int rc = PXD_OK;
    Staging st{ctx, {}};
    double* dx64 = st.alloc<double>(nx, &rc);
    double* dt64 = rc ? nullptr : st.alloc<double>(nt, &rc);
    float* dx = rc ? nullptr : st.alloc<float>(nx, &rc);
    float* dt = rc ? nullptr : st.alloc<float>(nt, &rc);
    double* de = rc ? nullptr : st.alloc<double>(n_poses, &rc);
    int* dn = rc ? nullptr : st.alloc<int>(n_poses, &rc);
    int* ds = rc ? nullptr : st.alloc<int>(n_poses, &rc);
    int* di = rc ? nullptr : st.alloc<int>(n_poses, &rc);
    if (rc) return rc;
    cudaStream_t s = ctx->stream;
    rc = cuda_check(ctx, cudaMemcpyAsync(dx64, xyz, nx * sizeof(double), cudaMemcpyHostToDevice, s), "poses in");
    if (!rc && nt)
        rc = cuda_check(ctx, cudaMemcpyAsync(dt64, tors, nt * sizeof(double), cudaMemcpyHostToDevice, s), "torsions in");
    if (!rc && ligand_ids)
        rc = cuda_check(ctx, cudaMemcpyAsync(di, ligand_ids, n_poses * sizeof(int), cudaMemcpyHostToDevice, s), "ids in");
    if (rc) return rc;
    convert_on_device(dx64, dx, nx, ctx->n_sm, s);
    convert_on_device(dt64, dt, nt, ctx->n_sm, s);
    if (!ligand_ids) fill_on_device(di, lig, n_poses, ctx->n_sm, s);
    rc = cuda_check(ctx, cudaGetLastError(), "conversion kernels");
    if (!rc) rc = pxd_lbfgs_dev(ctx, p, n_poses, max_atoms, di, dx, dt, de, dn, ds, s);
    if (rc) return rc;
    convert_on_device(dx, dx64, nx, ctx->n_sm, s);
    convert_on_device(dt, dt64, nt, ctx->n_sm, s);
    rc = cuda_check(ctx, cudaGetLastError(), "conversion kernels");
    if (!rc) rc = cuda_check(ctx, cudaMemcpyAsync(xyz, dx64, nx * sizeof(double), cudaMemcpyDeviceToHost, s), "poses out");
    if (!rc && nt)
        rc = cuda_check(ctx, cudaMemcpyAsync(tors, dt64, nt * sizeof(double), cudaMemcpyDeviceToHost, s), "torsions out");
    if (!rc) rc = cuda_check(ctx, cudaMemcpyAsync(energy, de, n_poses * sizeof(double), cudaMemcpyDeviceToHost, s), "energies out");
    if (!rc) rc = cuda_check(ctx, cudaMemcpyAsync(nevals, dn, n_poses * sizeof(int), cudaMemcpyDeviceToHost, s), "evaluations out");
    if (!rc) rc = cuda_check(ctx, cudaMemcpyAsync(status, ds, n_poses * sizeof(int), cudaMemcpyDeviceToHost, s), "status out");
    if (!rc) rc = cuda_check(ctx, cudaStreamSynchronize(s), "lbfgs");
    return rc;
}

int pxd_lbfgs(pxd_context* ctx, const pxd_lbfgs_params* p, int32_t lig, int32_t n_poses, double* xyz,
              double* tors, double* energy, int32_t* nevals, int32_t* status) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (lig < 0 || lig >= static_cast<int>(ctx->ligands.size()) || n_poses < 0)
        return set_error(ctx, PXD_ERR_INVALID, "ligand id");
    if (n_poses == 0) return PXD_OK;
    return lbfgs_host(ctx, p, n_poses, ctx->ligands[lig].n_atoms, lig, nullptr, xyz, tors, energy, nevals, status);
}

int pxd_lbfgs_multi(pxd_context* ctx, const pxd_lbfgs_params* p, int32_t n_poses, int32_t max_atoms,
                    const int32_t* ligand_ids, double* xyz, double* tors, double* energy, int32_t* nevals,
                    int32_t* status) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (n_poses < 0 || max_atoms <= 0 || max_atoms > PXD_MAX_LIGAND_ATOMS || (n_poses > 0 && !ligand_ids))
        return set_error(ctx, PXD_ERR_INVALID, "bad pose batch shape");
    if (n_poses == 0) return PXD_OK;
    return lbfgs_host(ctx, p, n_poses, max_atoms, -1, ligand_ids, xyz, tors, energy, nevals, status);
}

int pxd_ligand_kinematics(pxd_context* ctx, int32_t lig, int32_t n_poses, const double* xyz_in,
                          const double* centers, const double* rots, const double* torsions, double* xyz_out) {
    if (!ctx) return PXD_ERR_INVALID;
    cudaSetDevice(ctx->device);
    if (lig < 0 || lig >= static_cast<int>(ctx->ligands.size()) || n_poses < 0)
        return set_error(ctx, PXD_ERR_INVALID, "ligand id");
    const LigandEntry& e = ctx->ligands[lig];
    if (e.dev.n_frags == 0) return set_error(ctx, PXD_ERR_STATE, "ligand has no torsion tree");
    const int N = e.n_atoms, T = e.n_tors;
    std::vector<float> hx(3 * N), hc(3 * static_cast<size_t>(n_poses)), hr(9 * static_cast<size_t>(n_poses)),
        ht(static_cast<size_t>(n_poses) * T), ho(static_cast<size_t>(n_poses) * N * 3);
    for (int i = 0; i < 3 * N; ++i) hx[i] = static_cast<float>(xyz_in[i]);
    for (size_t i = 0; i < hc.size(); ++i) hc[i] = static_cast<float>(centers[i]);
    for (size_t i = 0; i < hr.size(); ++i) hr[i] = static_cast<float>(rots[i]);
    for (size_t i = 0; i < ht.size(); ++i) ht[i] = static_cast<float>(torsions[i]);
    int rc;
    Staging st{ctx, {}};
    float* dx = st.alloc<float>(hx.size(), &rc);
    if (rc) return rc;
    float* dc = st.alloc<float>(hc.size(), &rc);
    if (rc) return rc;
    float* dr = st.alloc<float>(hr.size(), &rc);
    if (rc) return rc;
    float* dt = st.alloc<float>(ht.size(), &rc);
    if (rc) return rc;
    float* dout = st.alloc<float>(ho.size(), &rc);
    if (rc) return rc;
    rc = cuda_check(ctx, cudaMemcpyAsync(dx, hx.data(), hx.size() * 4, cudaMemcpyHostToDevice, ctx->stream),
                    "ligand kinematics: coordinates to the device");
    if (!rc)
        rc = cuda_check(ctx, cudaMemcpyAsync(dc, hc.data(), hc.size() * 4, cudaMemcpyHostToDevice, ctx->stream),
                        "ligand kinematics: centres to the device");
    if (!rc)
        rc = cuda_check(ctx, cudaMemcpyAsync(dr, hr.data(), hr.size() * 4, cudaMemcpyHostToDevice, ctx->stream),
                        "ligand kinematics: rotations to the device");
    if (!rc && !ht.empty())
        rc = cuda_check(ctx, cudaMemcpyAsync(dt, ht.data(), ht.size() * 4, cudaMemcpyHostToDevice, ctx->stream),
                        "ligand kinematics: torsions to the device");
    if (rc) return rc;
    rc = launch_ligand_kinematics(ctx, lig, n_poses, dx, dc, dr, dt, dout, ctx->stream);
    if (rc) return rc;
    rc = cuda_check(ctx, cudaMemcpyAsync(ho.data(), dout, ho.size() * 4, cudaMemcpyDeviceToHost, ctx->stream),
                    "ligand kinematics: coordinates to the host");
    if (rc) return rc;
    rc = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "ligand kinematics");
    if (rc) return rc;
    for (size_t i = 0; i < ho.size(); ++i) xyz_out[i] = ho[i];
    return PXD_OK;
}

int pxd_ligand_backward(pxd_context* ctx, int32_t lig, int32_t n_poses, const double* xyz, const double* centers,
                        const double* atom_grad, double* center_grad, double* torque, double* torsion_grad) {
    if (!ctx) return PXD_ERR_INVALID;
    cudaSetDevice(ctx->device);
    if (lig < 0 || lig >= static_cast<int>(ctx->ligands.size()) || n_poses < 0)
        return set_error(ctx, PXD_ERR_INVALID, "ligand id");
    const LigandEntry& e = ctx->ligands[lig];
    if (e.dev.n_frags == 0) return set_error(ctx, PXD_ERR_STATE, "ligand has no torsion tree");
    if (n_poses == 0) return PXD_OK;
    const int N = e.n_atoms, T = e.n_tors;
    const size_t nx = static_cast<size_t>(n_poses) * N * 3;
    std::vector<float> hx(nx), hg(nx), hc(3 * static_cast<size_t>(n_poses));
    for (size_t i = 0; i < nx; ++i) {
        hx[i] = static_cast<float>(xyz[i]);
        hg[i] = static_cast<float>(atom_grad[i]);
    }
    for (size_t i = 0; i < hc.size(); ++i) hc[i] = static_cast<float>(centers[i]);
    int rc;
    Staging st{ctx, {}};
    float* dx = st.alloc<float>(nx, &rc);
    if (rc) return rc;
    float* dg = st.alloc<float>(nx, &rc);
    if (rc) return rc;
    float* dc = st.alloc<float>(hc.size(), &rc);
    if (rc) return rc;
    float* doc = st.alloc<float>(hc.size(), &rc);
    if (rc) return rc;
    float* dot = st.alloc<float>(hc.size(), &rc);
    if (rc) return rc;
    float* dtt = st.alloc<float>(static_cast<size_t>(n_poses) * T, &rc);
    if (rc) return rc;
    queue_copy(ctx, &rc, dx, hx.data(), nx * 4, cudaMemcpyHostToDevice, ctx->stream);
    queue_copy(ctx, &rc, dg, hg.data(), nx * 4, cudaMemcpyHostToDevice, ctx->stream);
    queue_copy(ctx, &rc, dc, hc.data(), hc.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (rc) return rc;
    rc = launch_ligand_backward(ctx, lig, n_poses, dx, dc, dg, doc, dot, dtt, ctx->stream);
    if (rc) return rc;
    std::vector<float> oc(hc.size()), oq(hc.size()), ot(static_cast<size_t>(n_poses) * T);
    queue_copy(ctx, &rc, oc.data(), doc, oc.size() * 4, cudaMemcpyDeviceToHost, ctx->stream);
    queue_copy(ctx, &rc, oq.data(), dot, oq.size() * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (!ot.empty()) queue_copy(ctx, &rc, ot.data(), dtt, ot.size() * 4, cudaMemcpyDeviceToHost, ctx->stream);
    rc = sync_copies(ctx, rc, ctx->stream, "ligand backward");
    if (rc) return rc;
    for (size_t i = 0; i < oc.size(); ++i) {
        center_grad[i] = oc[i];
        torque[i] = oq[i];
    }
    for (size_t i = 0; i < ot.size(); ++i) torsion_grad[i] = ot[i];
    return PXD_OK;
}

int pxd_receptor_kinematics(pxd_context* ctx, int32_t n_poses, const double* torsions, double* xyz_out) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    const int M = ctx->n_rec, R = ctx->rec.n_rotors;
    std::vector<float> ht(static_cast<size_t>(n_poses) * R), ho(static_cast<size_t>(n_poses) * M * 3);
    for (size_t i = 0; i < ht.size(); ++i) ht[i] = static_cast<float>(torsions[i]);
    Staging st{ctx, {}};
    float* dt = st.alloc<float>(ht.size(), &rc);
    if (rc) return rc;
    float* dout = st.alloc<float>(ho.size(), &rc);
    if (rc) return rc;
    if (!ht.empty()) queue_copy(ctx, &rc, dt, ht.data(), ht.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (rc) return rc;
    rc = launch_receptor_kinematics(ctx, n_poses, dt, dout, ctx->stream);
    if (rc) return rc;
    queue_copy(ctx, &rc, ho.data(), dout, ho.size() * 4, cudaMemcpyDeviceToHost, ctx->stream);
    rc = sync_copies(ctx, rc, ctx->stream, "receptor kinematics");
    if (rc) return rc;
    for (size_t i = 0; i < ho.size(); ++i) xyz_out[i] = ho[i];
    return PXD_OK;
}

}  // extern "C"
