// Engine facade (see engine.h) and its C ABI (pxd_engine_*).
#include "engine.h"

#include <dlfcn.h>
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <mutex>
#include <sstream>
#include <stdexcept>

#include "../../include/pxdock_gb300_vdw.h"
#include "inputs.h"
#include "json.h"
#include "mapcache.h"

namespace pxd {

// ---------------------------------------------------------------------- logging
namespace {

std::mutex g_log_mu;
std::ofstream g_log_file;
bool g_log_to_file = false;
int g_verbosity = 1;

void log(int level, const std::string& msg) {  // level 0 warning, 1 info, 2 debug
    std::lock_guard<std::mutex> lock(g_log_mu);
    if (level > g_verbosity) return;
    static const char* names[3] = {"WARNING", "INFO", "DEBUG"};
    std::ostream& out = g_log_to_file ? static_cast<std::ostream&>(g_log_file) : std::cerr;
    out << "[pxdock-gb300] " << names[level] << " " << msg << std::endl;
}

void check(pxd_context* ctx, int rc) {
    if (rc != PXD_OK) throw std::runtime_error(ctx ? pxd_last_error(ctx) : "invalid context");
}

bool is_file(const std::string& p) {
    struct stat st;
    return stat(p.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

void make_dirs(const std::string& dir) {
    std::string acc;
    for (size_t i = 0; i <= dir.size(); ++i) {
        if (i == dir.size() || dir[i] == '/') {
            if (!acc.empty()) {
                struct stat st;
                if (stat(acc.c_str(), &st) != 0 && mkdir(acc.c_str(), 0755) != 0)
                    throw std::runtime_error("Failed to create directory: " + acc);
            }
        }
        if (i < dir.size()) acc += dir[i];
    }
}

std::string join(const std::string& dir, const std::string& name) {
    return dir.empty() || dir.back() == '/' ? dir + name : dir + "/" + name;
}

// boost::filesystem::path::stem: the file name without its last extension
std::string stem(const std::string& path) {
    const size_t slash = path.find_last_of('/');
    std::string name = slash == std::string::npos ? path : path.substr(slash + 1);
    const size_t dot = name.find_last_of('.');
    if (dot != std::string::npos && dot > 0) name.resize(dot);
    return name;
}

// index_file_source::fill (source.cpp:26-44)
std::vector<std::string> read_index(const std::string& path) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("Failed to open file: " + path);
    std::vector<std::string> out;
    std::string line;
    size_t no = 0;
    while (std::getline(in, line)) {
        ++no;
        if (line.empty())
            log(0, "Skip illegal line#" + std::to_string(no) + " with empty text.");
        else if (!is_file(line))
            log(0, "Skip illegal line#" + std::to_string(no) + " with ghost file: " + line);
        else
            out.push_back(line);
    }
    return out;
}

// the default scoring-function file shipped beside the library (data/ next to _native/)
std::string default_sf_path() {
    Dl_info info;
    if (dladdr(reinterpret_cast<void*>(&default_sf_path), &info) && info.dli_fname) {
        std::string lib = info.dli_fname;
        const size_t slash = lib.find_last_of('/');
        const std::string dir = slash == std::string::npos ? "." : lib.substr(0, slash);
        return join(dir, "../data/scoring_function.json");
    }
    return "";
}

struct Loaded {
    std::string path;
    LigandData lig;
    int id = -1;
};

// multi_pose_reader / single_pose_reader parsing: a file that fails is skipped
std::vector<Loaded> load_ligands(const std::vector<std::string>& files, bool geometry) {
    std::vector<Loaded> out;
    for (auto& f : files) {
        try {
            Loaded l;
            l.path = f;
            l.lig = read_ligand(json::parse_file(f), geometry);
            out.push_back(std::move(l));
        } catch (std::exception& e) {
            log(0, "Due to invalid format or content, skip ligand: " + f + " with reason: " + e.what());
        }
    }
    return out;
}

void register_ligands(pxd_context* ctx, std::vector<Loaded>& ligs) {
    check(ctx, pxd_clear_ligands(ctx));
    for (auto& l : ligs) {
        pxd_ligand_desc d = l.lig.desc();
        int32_t id = -1;
        check(ctx, pxd_add_ligand(ctx, &d, &id));
        l.id = id;
    }
}

double rmsd(const std::vector<double>& a, const std::vector<double>& b) {
    double s = 0.0;
    for (size_t i = 0; i < a.size(); i += 3) {
        const double dx = a[i] - b[i], dy = a[i + 1] - b[i + 1], dz = a[i + 2] - b[i + 2];
        s += dx * dx + dy * dy + dz * dz;
    }
    return std::sqrt(s / static_cast<double>(a.size() / 3));
}

}  // namespace

void set_log(const std::string& path, int verbosity) {
    std::lock_guard<std::mutex> lock(g_log_mu);
    g_verbosity = verbosity;
    if (g_log_file.is_open()) g_log_file.close();
    g_log_to_file = path != "-";
    if (g_log_to_file) {
        g_log_file.open(path, std::ios::app);
        if (!g_log_file) {
            g_log_to_file = false;
            throw std::runtime_error("Failed to open log file: " + path);
        }
    }
}

// ------------------------------------------------------------------- writers
void write_poses(const std::string& path, const std::string& smiles, int best_id, double bscore,
                 const std::vector<PoseResult>& poses, const std::vector<int>& bond_mappings, int num_rotatable_bonds) {
    std::ofstream out(path);
    if (!out) throw std::runtime_error("Failed to open file for writing: " + path);
    out << "{" << std::endl;
    if (!smiles.empty()) {
        out << "  \"mapped_smiles\": \"";
        for (char c : smiles) {
            out << c;
            if (c == '\\') out << c;  // backslashes doubled (writer.cpp:27-38)
        }
        out << "\"," << std::endl;
    }
    out << "  \"best_pose\": {" << std::endl;
    out << "    \"index\": " << best_id << "," << std::endl;
    out << "    \"bscore\": " << bscore << std::endl;
    out << "  }," << std::endl;
    out << "  \"poses\": [" << std::endl;
    for (size_t i = 0; i < poses.size(); ++i) {
        const PoseResult& p = poses[i];
        // receptor torsions in rotatable-bond order (restore_bond_orders, data.h:53-61)
        std::vector<double> aligned(num_rotatable_bonds, 0.0);
        for (size_t k = 0; k < p.torsions.size() && k < bond_mappings.size(); ++k)
            aligned[bond_mappings[k]] = p.torsions[k];
        out << "    {" << std::endl;
        out << "      \"offset\": " << p.offset << "," << std::endl;
        out << "      \"energy\": " << p.energy << "," << std::endl;
        out << "      \"pscore\": " << p.pscore << "," << std::endl;
        out << "      \"nevals\": " << p.nevals << "," << std::endl;
        out << "      \"receptor\": {" << std::endl;
        out << "        \"torsions\": [" << std::endl;
        // rows of 10 values; every row but the last ends with ", " (printer.h format)
        const std::string indent = "            ";
        size_t nrows = aligned.size() / 10, rem = aligned.size() % 10;
        if (rem == 0 && nrows > 0) {
            --nrows;
            rem = 10;
        }
        for (size_t r = 0; r < nrows; ++r) {
            out << indent;
            for (size_t j = 0; j < 10; ++j) out << aligned[r * 10 + j] << ", ";
            out << std::endl;
        }
        if (rem > 0) {
            out << indent << aligned[nrows * 10];
            for (size_t j = 1; j < rem; ++j) out << ", " << aligned[nrows * 10 + j];
            out << std::endl;
        }
        out << "        ]" << std::endl;
        out << "      }," << std::endl;
        out << "      \"ligand\": {" << std::endl;
        out << "        \"xyz\": ";
        // to_string(molecule_pose, prefix) (system.cpp:319-336)
        const size_t na = p.xyz.size() / 3;
        if (na == 0) {
            out << "[]";
        } else {
            out << "[" << std::endl;
            for (size_t a = 0; a < na; ++a) {
                out << "          [" << p.xyz[3 * a] << ", " << p.xyz[3 * a + 1] << ", " << p.xyz[3 * a + 2] << "]";
                if (a + 1 < na) out << ",";
                out << std::endl;
            }
            out << "        ]";
        }
        out << std::endl;
        out << "      }" << std::endl;
        out << "    }";
        if (i + 1 < poses.size()) out << ",";
        out << std::endl;
    }
    out << "  ]" << std::endl;
    out << "}" << std::endl;
}

std::vector<PoseResult> cluster_poses(const std::vector<PoseResult>& candidates, int num_modes, double min_rmsd) {
    std::vector<PoseResult> kept;
    for (const PoseResult& c : candidates) {
        if (c.nevals == 0) continue;  // failure mark from the searcher
        if (kept.empty()) {
            kept.push_back(c);
            continue;
        }
        size_t off = 0;
        double best = std::numeric_limits<double>::infinity();
        for (size_t k = 0; k < kept.size(); ++k) {
            const double r = rmsd(kept[k].xyz, c.xyz);
            if (k == 0 || r < best) {
                off = k;
                best = r;
            }
        }
        bool updated = false;
        if (best < min_rmsd) {
            if (c.pscore < kept[off].pscore) {
                kept[off] = c;
                updated = true;
            }
        } else if (static_cast<int>(kept.size()) < num_modes) {
            kept.push_back(c);
            updated = true;
        } else if (c.pscore < kept.back().pscore) {
            kept.back() = c;
            updated = true;
        }
        if (updated)
            std::sort(kept.begin(), kept.end(), [](const PoseResult& a, const PoseResult& b) { return a.pscore < b.pscore; });
    }
    return kept;
}

// -------------------------------------------------------------------- engine
Engine::Engine(const std::string& receptor_file, const std::string& sf_file, int cpu_nthreads, int device) {
    receptor_.reset(new ReceptorData(read_receptor(json::parse_file(receptor_file))));
    std::string sf = sf_file;
    if (sf.empty()) {
        sf = default_sf_path();
        if (sf.empty() || !is_file(sf))
            throw std::runtime_error("Failed to find the default parameter file of scoring function. Please "
                                     "explicitly provide its location!.");
        log(1, "Since no scoring function parameter file provided, the default one is enabled at: " + sf);
    }
    const auto params = read_scoring_function(json::parse_file(sf));
    nthreads_ = cpu_nthreads >= 1 ? cpu_nthreads : 1;
    check(nullptr, pxd_context_create(device, &ctx_));
    try {
        pxd_receptor_desc rd = receptor_->desc();
        check(ctx_, pxd_set_receptor(ctx_, &rd));
        check(ctx_, pxd_set_scoring_function(ctx_, 0, &params[0]));
        check(ctx_, pxd_set_scoring_function(ctx_, 1, &params[1]));
    } catch (...) {
        pxd_context_destroy(ctx_);
        ctx_ = nullptr;
        throw;
    }
}

Engine::~Engine() {
    if (ctx_) pxd_context_destroy(ctx_);
}

void Engine::require_box() const {
    if (box_.size() < 6) throw std::runtime_error("Please call `set_box(...)` first!");
}

void Engine::require_maps() const {
    if (!has_maps_) throw std::runtime_error("Please call either `generate_cache_maps(...)` or `load_maps(...)` first!");
}

void Engine::set_box(double cx, double cy, double cz, double sx, double sy, double sz) {
    // appended, as the reference's box vector is: the first call's box stays in force
    for (double v : {cx, cy, cz, sx, sy, sz}) box_.push_back(v);
}

void Engine::generate_maps(double grid_spacing, double max_size) {
    require_box();
    pxd_box b{};
    check(ctx_, pxd_decide_grid_dims(box_[0], box_[1], box_[2], std::max(box_[3], max_size), std::max(box_[4], max_size),
                                     std::max(box_[5], max_size), grid_spacing, &b));
    std::ostringstream oss;
    oss << std::fixed << std::setprecision(3) << "Generating receptor cache with grid settings: init [" << b.init_xyz[0]
        << ", " << b.init_xyz[1] << ", " << b.init_xyz[2] << "], points [" << b.npoints[0] << ", " << b.npoints[1]
        << ", " << b.npoints[2] << "]";
    log(1, oss.str());
    check(ctx_, pxd_grid_build(ctx_, &b, nullptr, -1));  // every ligand type, as populate()
    grid_ = b;
    has_maps_ = true;
}

void Engine::drop_maps() {
    if (has_maps_) check(ctx_, pxd_grid_drop(ctx_));
    has_maps_ = false;
}

// This library's earlier cache layout (grid.json + map_NNN.f32), still read by load_maps.
static const char* kMapFormat = "pxdock-gb300 maps 1";

// The receptor atoms the maps leave out (receptor_cache::populate's excluded_, grid.cpp:118-123):
// every rotor leaf's atoms but the axis atom they turn about (data.cpp:349-363), ascending.
static std::vector<int64_t> excluded_atoms(const ReceptorData& r) {
    std::vector<int64_t> out;
    const size_t n_rot = r.rotor_axis.size() / 2;
    for (size_t k = 0; k < n_rot && k + 1 < r.rotor_offsets.size(); ++k)
        for (int u = r.rotor_offsets[k]; u < r.rotor_offsets[k + 1]; ++u)
            if (r.rotor_atoms[u] != r.rotor_axis[2 * k + 1]) out.push_back(r.rotor_atoms[u]);
    std::sort(out.begin(), out.end());
    out.erase(std::unique(out.begin(), out.end()), out.end());
    return out;
}

static std::vector<uint8_t> read_bytes(const std::string& path) {
    std::ifstream in(path, std::ios::binary | std::ios::ate);
    if (!in) throw std::runtime_error("Failed to open file for reading: " + path);
    const std::streamsize n = in.tellg();
    std::vector<uint8_t> b(static_cast<size_t>(n));
    in.seekg(0);
    if (n > 0 && !in.read(reinterpret_cast<char*>(b.data()), n)) throw std::runtime_error("Failed to read " + path);
    return b;
}

// receptor_cache::save (grid.cpp:309-345): <tag>.bdg per ligand type and coul.bdg, FP64
// records, then meta.dat last as the completion flag.
void Engine::dump_maps(const std::string& cache_dir) {
    require_maps();
    make_dirs(cache_dir);
    const size_t P = static_cast<size_t>(grid_.npoints[0]) * grid_.npoints[1] * grid_.npoints[2];
    std::vector<double> rec(P * 4);
    for (int m = 0; m <= PXD_NUM_VDW_TYPES; ++m) {
        check(ctx_, pxd_grid_read_map64(ctx_, m, rec.data()));
        const std::vector<uint8_t> bytes = mapcache::encode_bdg(rec.data(), P, 8);
        const std::string path = join(cache_dir, std::string(PXD_VDW_TAGS[m]) + ".bdg");
        std::ofstream out(path, std::ios::binary);
        out.write(reinterpret_cast<const char*>(bytes.data()), static_cast<std::streamsize>(bytes.size()));
        if (!out) throw std::runtime_error("Failed to write map file: " + path);
    }
    mapcache::Meta meta;
    meta.box = grid_;
    meta.excluded = excluded_atoms(*receptor_);
    std::ofstream out(join(cache_dir, "meta.dat"));
    out << mapcache::encode_meta(meta);
    if (!out) throw std::runtime_error("Failed to write the map metadata in " + cache_dir);
}

// receptor_cache::restore (grid.cpp:347-391, 408-431), with its messages; a cache in this
// library's earlier layout (grid.json) is read as well.
void Engine::load_maps(const std::string& cache_dir) {
    const std::string meta_path = join(cache_dir, "meta.dat");
    if (!is_file(meta_path)) {
        if (is_file(join(cache_dir, "grid.json"))) return load_own_maps(cache_dir);
        throw std::runtime_error("The metadata file of maps is missing!");
    }
    std::ifstream in(meta_path);
    std::stringstream text;
    text << in.rdbuf();
    const mapcache::Meta meta = mapcache::decode_meta(text.str());
    if (meta.version != mapcache::kFormatVersion) {
        std::ostringstream oss;
        oss << "Format version of map files are not compatible! Expected [" << mapcache::kFormatVersion << "] vs. Got ["
            << meta.version << "]";
        throw std::runtime_error(oss.str());
    }
    std::vector<int64_t> excl = meta.excluded;
    std::sort(excl.begin(), excl.end());
    excl.erase(std::unique(excl.begin(), excl.end()), excl.end());
    if (excl != excluded_atoms(*receptor_))
        throw std::runtime_error("The maps in " + cache_dir +
                                 " leave out other receptor atoms than this receptor's movable ones");
    const pxd_box b = meta.box;
    const size_t P = static_cast<size_t>(b.npoints[0]) * b.npoints[1] * b.npoints[2];
    for (int m = 0; m <= PXD_NUM_VDW_TYPES; ++m) {
        const std::string path = join(cache_dir, std::string(PXD_VDW_TAGS[m]) + ".bdg");
        if (!is_file(path))
            throw std::runtime_error(std::string("Map file for atom type [") + PXD_VDW_TAGS[m] + "] is missing!");
        const std::vector<uint8_t> bytes = read_bytes(path);
        std::vector<double> rec;
        try {
            rec = mapcache::decode_bdg(bytes.data(), bytes.size(), nullptr);
        } catch (const std::exception& e) {
            throw std::runtime_error(path + ": " + e.what());
        }
        if (rec.size() != 4 * P) throw std::runtime_error(path + ": point count does not match meta.dat's box");
        check(ctx_, pxd_grid_write_map64(ctx_, &b, m, rec.data()));
    }
    grid_ = b;
    has_maps_ = true;
}

void Engine::load_own_maps(const std::string& cache_dir) {
    const std::string meta = join(cache_dir, "grid.json");
    const json::Value head = json::parse_file(meta);
    if (head.at("format").str != kMapFormat) throw std::runtime_error("Unknown map cache format in " + cache_dir);
    pxd_box b{};
    for (int d = 0; d < 3; ++d) {
        b.init_xyz[d] = head.at("init_xyz").items.at(d).as_double();
        b.npoints[d] = static_cast<int32_t>(head.at("npoints").items.at(d).as_long());
    }
    b.spacing = head.at("spacing").as_double();
    const size_t P = static_cast<size_t>(b.npoints[0]) * b.npoints[1] * b.npoints[2];
    std::vector<float> rec(P * 4);
    for (auto& mv : head.at("maps").items) {
        const int m = static_cast<int>(mv.as_long());
        char name[32];
        std::snprintf(name, sizeof(name), "map_%03d.f32", m);
        std::ifstream in(join(cache_dir, name), std::ios::binary);
        in.read(reinterpret_cast<char*>(rec.data()), static_cast<std::streamsize>(rec.size() * sizeof(float)));
        if (!in) throw std::runtime_error(std::string("Map file ") + name + " is missing or short!");
        check(ctx_, pxd_grid_write_map(ctx_, &b, m, rec.data()));
    }
    grid_ = b;
    has_maps_ = true;
}

void Engine::evaluate(const std::string& ligand_index_file, const std::string& output_file) {
    auto ligs = load_ligands(read_index(ligand_index_file), false);
    register_ligands(ctx_, ligs);
    std::ofstream out(output_file);
    if (!out) throw std::runtime_error("Failed to open file for writing: " + output_file);
    out << "ligand_file,pose_id,pscore,bscore" << std::endl;
    size_t n_out = 0;
    for (auto& l : ligs) {
        const int n = static_cast<int>(l.lig.poses.size());
        if (n == 0) continue;
        std::vector<double> xyz;
        for (auto& p : l.lig.poses) xyz.insert(xyz.end(), p.begin(), p.end());
        std::vector<double> tors(static_cast<size_t>(n) * receptor_->rotor_axis.size() / 2 + 1, 0.0);
        std::vector<double> ps(n), bs(n);
        check(ctx_, pxd_score(ctx_, 0, l.id, n, xyz.data(), tors.data(), ps.data(), nullptr));
        check(ctx_, pxd_score(ctx_, 1, l.id, n, xyz.data(), tors.data(), bs.data(), nullptr));
        for (int k = 0; k < n; ++k) {
            out << stem(l.path) << "," << k << "," << std::setprecision(16) << ps[k] << "," << std::setprecision(16) << bs[k]
                << std::endl;
            ++n_out;
        }
    }
    log(1, "Number of successful evaluations is: " + std::to_string(n_out));
}

void Engine::set_dof_mode(int mode) {
    if (mode != PXD_DOF_CARTESIAN && mode != PXD_DOF_RIGID_TORSION)
        throw std::runtime_error("dof_mode must be 0 (Cartesian) or 1 (rigid body + torsions)");
    dof_mode_ = mode;
}

void Engine::optimize(const std::string& ligand_index_file, const std::string& output_dir, int max_niters, double slope) {
    if (has_maps_)
        check(ctx_, pxd_grid_set_slope(ctx_, slope));
    else
        log(1, "Receptor cache is disabled in this run.");
    // multi_pose_reader; the rigid-body + torsion mode also reads each ligand's torsion tree
    auto ligs = load_ligands(read_index(ligand_index_file), dof_mode_ == PXD_DOF_RIGID_TORSION);
    if (dof_mode_ == PXD_DOF_RIGID_TORSION)
        for (auto& l : ligs)
            if (!l.lig.has_tree)
                throw std::runtime_error("dof_mode 1 needs the torsion tree of ligand " + l.path +
                                         " (its \"geometry\" block)");
    register_ligands(ctx_, ligs);
    make_dirs(output_dir);
    if (ligs.empty()) return;
    const int R = static_cast<int>(receptor_->rotor_axis.size() / 2);
    int max_atoms = 0;
    size_t n_total = 0;
    for (auto& l : ligs) {
        max_atoms = std::max(max_atoms, l.lig.n_atoms());
        n_total += l.lig.poses.size();
    }
    std::vector<double> xyz(n_total * max_atoms * 3, 0.0), tors(n_total * R + 1, 0.0), energy(n_total);
    std::vector<int32_t> ids(n_total), nev(n_total), st(n_total);
    size_t row = 0;
    for (auto& l : ligs)
        for (auto& p : l.lig.poses) {
            std::copy(p.begin(), p.end(), xyz.begin() + row * max_atoms * 3);
            ids[row++] = l.id;
        }
    pxd_lbfgs_params prm;
    pxd_lbfgs_defaults(&prm);
    prm.max_iter = max_niters;
    prm.dof_mode = dof_mode_;
    if (n_total) check(ctx_, pxd_lbfgs_multi(ctx_, &prm, static_cast<int32_t>(n_total), max_atoms, ids.data(), xyz.data(),
                                              tors.data(), energy.data(), nev.data(), st.data()));
    row = 0;
    int written = 0;
    for (auto& l : ligs) {
        const int N = l.lig.n_atoms(), n = static_cast<int>(l.lig.poses.size());
        if (n == 0) continue;
        std::vector<PoseResult> poses(n);
        std::vector<double> lx, lt;
        for (int k = 0; k < n; ++k, ++row) {
            PoseResult& p = poses[k];
            p.offset = k;
            p.energy = energy[row];
            p.nevals = nev[row];
            p.xyz.assign(xyz.begin() + row * max_atoms * 3, xyz.begin() + row * max_atoms * 3 + N * 3);
            p.torsions.assign(tors.begin() + row * R, tors.begin() + row * R + R);
            lx.insert(lx.end(), p.xyz.begin(), p.xyz.end());
            lt.insert(lt.end(), p.torsions.begin(), p.torsions.end());
        }
        lt.push_back(0.0);
        std::vector<double> ps(n), bs(1);
        check(ctx_, pxd_score(ctx_, 0, l.id, n, lx.data(), lt.data(), ps.data(), nullptr));
        int best = 0;  // pose_ranker: the first minimum (writer.cpp:179-208)
        for (int k = 0; k < n; ++k) {
            poses[k].pscore = ps[k];
            if (ps[k] < ps[best]) best = k;
        }
        std::vector<double> bt = poses[best].torsions;
        bt.push_back(0.0);
        check(ctx_, pxd_score(ctx_, 1, l.id, 1, poses[best].xyz.data(), bt.data(), bs.data(), nullptr));
        write_poses(join(output_dir, stem(l.path) + "_out.json"), l.lig.smiles, best, bs[0], poses,
                    receptor_->bond_mappings, receptor_->num_rotatable_bonds);
        ++written;
    }
    log(1, "Number of successful optimizations is: " + std::to_string(written));
}

void Engine::search(const std::string& ligand_index_file, const std::string& output_dir, int seed, int exhaustiveness,
                    int max_nsteps, int relax_nsteps, int num_modes, double min_rmsd, double mc_mmenergy_threshold,
                    double slope) {
    double lo[3], hi[3];
    if (!has_maps_) {
        require_box();
        for (int d = 0; d < 3; ++d) {  // describe_boundary (grid.cpp:42-55)
            const double half = box_[3 + d] * 0.5;
            lo[d] = box_[d] - half;
            hi[d] = box_[d] + half;
        }
        log(1, "Receptor cache is disabled in this run.");
    } else {
        check(ctx_, pxd_grid_set_slope(ctx_, slope));
        for (int d = 0; d < 3; ++d) {
            lo[d] = grid_.init_xyz[d];
            hi[d] = grid_.init_xyz[d] + (grid_.npoints[d] - 1) * grid_.spacing;
        }
    }
    auto ligs = load_ligands(read_index(ligand_index_file), true);  // single_pose_reader
    register_ligands(ctx_, ligs);
    make_dirs(output_dir);
    if (ligs.empty() || exhaustiveness <= 0) return;
    const int R = static_cast<int>(receptor_->rotor_axis.size() / 2);
    int max_atoms = 0;
    for (auto& l : ligs) max_atoms = std::max(max_atoms, l.lig.n_atoms());
    const size_t W = ligs.size() * static_cast<size_t>(exhaustiveness);
    std::vector<double> start(W * max_atoms * 3, 0.0), out(W * max_atoms * 3), tors(W * R + 1), energy(W), ps(W);
    std::vector<int32_t> ids(W), walker(W), first(W), nev(W), st(W);
    size_t row = 0;
    for (auto& l : ligs)
        for (int w = 0; w < exhaustiveness; ++w, ++row) {
            // walker w starts from pose w when the file has it (searcher.cpp:105-114)
            const int src = static_cast<int>(l.lig.poses.size()) > w ? w : 0;
            const auto& p = l.lig.poses.at(src);
            std::copy(p.begin(), p.end(), start.begin() + row * max_atoms * 3);
            ids[row] = l.id;
            walker[row] = w;
            first[row] = src == 0 ? 1 : 0;
        }
    pxd_mc_params prm;
    pxd_mc_defaults(&prm);
    prm.seed = static_cast<uint32_t>(seed);
    prm.max_nsteps = max_nsteps;
    prm.relax_nsteps = relax_nsteps;
    prm.mc_mmenergy_threshold = mc_mmenergy_threshold;
    for (int d = 0; d < 3; ++d) {
        prm.box_lo[d] = lo[d];
        prm.box_hi[d] = hi[d];
    }
    std::vector<double> gmin(ligs.size() + 1, 1e8);
    check(ctx_, pxd_mc_search_multi(ctx_, &prm, static_cast<int32_t>(W), max_atoms, ids.data(), walker.data(),
                                    first.data(), start.data(), out.data(), tors.data(), energy.data(), ps.data(),
                                    nev.data(), st.data(), gmin.data()));
    // clustering of every ligand's walkers in one launch (num_modes <= 32; beyond, the same
    // rule runs on the host per ligand)
    const int n_l = static_cast<int>(ligs.size());
    std::vector<int32_t> g_start(n_l + 1), g_atoms(n_l), kept_rows, kept_n(n_l);
    const bool on_device = num_modes >= 1 && num_modes <= 32;
    if (on_device) {
        for (int g = 0; g < n_l; ++g) {
            g_start[g] = g * exhaustiveness;
            g_atoms[g] = ligs[g].lig.n_atoms();
        }
        g_start[n_l] = n_l * exhaustiveness;
        kept_rows.assign(static_cast<size_t>(n_l) * num_modes, -1);
        check(ctx_, pxd_cluster_poses_batch(ctx_, n_l, g_start.data(), g_atoms.data(), max_atoms, out.data(),
                                            ps.data(), nev.data(), num_modes, min_rmsd, kept_rows.data(),
                                            kept_n.data()));
    }
    row = 0;
    int written = 0;
    for (int gi = 0; gi < n_l; ++gi) {
        auto& l = ligs[gi];
        const int N = l.lig.n_atoms();
        std::vector<PoseResult> cands(exhaustiveness);
        for (int w = 0; w < exhaustiveness; ++w, ++row) {
            PoseResult& p = cands[w];
            p.offset = walker[row];
            p.energy = energy[row];
            p.pscore = ps[row];
            p.nevals = nev[row];
            p.xyz.assign(out.begin() + row * max_atoms * 3, out.begin() + row * max_atoms * 3 + N * 3);
            p.torsions.assign(tors.begin() + row * R, tors.begin() + row * R + R);
        }
        std::vector<PoseResult> kept;
        if (on_device) {
            for (int k = 0; k < kept_n[gi]; ++k)
                kept.push_back(cands[kept_rows[static_cast<size_t>(gi) * num_modes + k] - g_start[gi]]);
        } else {
            kept = cluster_poses(cands, num_modes, min_rmsd);
        }
        if (kept.empty()) {
            log(2, "Tasks with prefix [" + stem(l.path) + "] has failed.");
            continue;
        }
        std::vector<double> bt = kept[0].torsions, bs(1);
        bt.push_back(0.0);
        check(ctx_, pxd_score(ctx_, 1, l.id, 1, kept[0].xyz.data(), bt.data(), bs.data(), nullptr));
        write_poses(join(output_dir, stem(l.path) + "_out.json"), l.lig.smiles, 0, bs[0], kept,
                    receptor_->bond_mappings, receptor_->num_rotatable_bonds);
        ++written;
    }
    log(1, "Number of successful dockings is: " + std::to_string(written));
}

}  // namespace pxd

// ------------------------------------------------------------------------ C ABI
using pxd::Engine;

struct pxd_engine {
    std::unique_ptr<Engine> e;
    std::string error;
};

namespace {
thread_local std::string g_create_error;

template <class F>
int guarded(pxd_engine* h, F&& f) {
    if (!h || !h->e) return PXD_ERR_INVALID;
    try {
        f(*h->e);
        h->error.clear();
        return PXD_OK;
    } catch (std::exception& ex) {
        h->error = ex.what();
        return PXD_ERR_STATE;
    }
}
}  // namespace

extern "C" {

int pxd_engine_create(const char* receptor_file, const char* sf_file, int32_t cpu_nthreads, int32_t device,
                      pxd_engine** out) {
    if (!out || !receptor_file) return PXD_ERR_INVALID;
    *out = nullptr;
    try {
        auto* h = new pxd_engine;
        h->e.reset(new Engine(receptor_file, sf_file ? sf_file : "", cpu_nthreads, device));
        *out = h;
        return PXD_OK;
    } catch (std::exception& ex) {
        g_create_error = ex.what();
        return PXD_ERR_STATE;
    }
}

void pxd_engine_destroy(pxd_engine* h) { delete h; }

const char* pxd_engine_last_error(const pxd_engine* h) { return h ? h->error.c_str() : g_create_error.c_str(); }

int pxd_engine_set_box(pxd_engine* h, double cx, double cy, double cz, double sx, double sy, double sz) {
    return guarded(h, [&](Engine& e) { e.set_box(cx, cy, cz, sx, sy, sz); });
}
int pxd_engine_generate_maps(pxd_engine* h, double grid_spacing, double max_size) {
    return guarded(h, [&](Engine& e) { e.generate_maps(grid_spacing, max_size); });
}
int pxd_engine_dump_maps(pxd_engine* h, const char* dir) {
    return guarded(h, [&](Engine& e) { e.dump_maps(dir ? dir : ""); });
}
int pxd_engine_load_maps(pxd_engine* h, const char* dir) {
    return guarded(h, [&](Engine& e) { e.load_maps(dir ? dir : ""); });
}
int pxd_engine_drop_maps(pxd_engine* h) {
    return guarded(h, [&](Engine& e) { e.drop_maps(); });
}
int pxd_engine_evaluate(pxd_engine* h, const char* index_file, const char* output_file) {
    return guarded(h, [&](Engine& e) { e.evaluate(index_file ? index_file : "", output_file ? output_file : ""); });
}
int pxd_engine_optimize(pxd_engine* h, const char* index_file, const char* output_dir, int32_t max_niters,
                        double slope) {
    return guarded(h, [&](Engine& e) {
        e.optimize(index_file ? index_file : "", output_dir ? output_dir : "", max_niters, slope);
    });
}
int pxd_engine_set_dof_mode(pxd_engine* h, int32_t dof_mode) {
    return guarded(h, [&](Engine& e) { e.set_dof_mode(dof_mode); });
}
int pxd_engine_search(pxd_engine* h, const char* index_file, const char* output_dir, int32_t seed,
                      int32_t exhaustiveness, int32_t max_nsteps, int32_t relax_nsteps, int32_t num_modes,
                      double min_rmsd, double mc_mmenergy_threshold, double slope) {
    return guarded(h, [&](Engine& e) {
        e.search(index_file ? index_file : "", output_dir ? output_dir : "", seed, exhaustiveness, max_nsteps,
                 relax_nsteps, num_modes, min_rmsd, mc_mmenergy_threshold, slope);
    });
}

int pxd_engine_log2file(const char* path, int32_t verbosity) {
    try {
        pxd::set_log(path ? path : "-", verbosity);
        return PXD_OK;
    } catch (std::exception& ex) {
        g_create_error = ex.what();
        return PXD_ERR_INVALID;
    }
}

int pxd_write_poses(const char* path, const char* smiles, int32_t best_id, double bscore, int32_t n_poses,
                    int32_t n_atoms, const int32_t* offsets, const double* energy, const double* pscore,
                    const int64_t* nevals, int32_t n_rotors, const double* torsions, const double* xyz,
                    const int32_t* bond_mappings, int32_t num_rotatable_bonds) {
    if (!path || n_poses < 0 || n_atoms < 0 || n_rotors < 0) return PXD_ERR_INVALID;
    try {
        std::vector<pxd::PoseResult> poses(n_poses);
        for (int k = 0; k < n_poses; ++k) {
            poses[k].offset = offsets[k];
            poses[k].energy = energy[k];
            poses[k].pscore = pscore[k];
            poses[k].nevals = static_cast<long>(nevals[k]);
            poses[k].torsions.assign(torsions + static_cast<size_t>(k) * n_rotors,
                                     torsions + static_cast<size_t>(k + 1) * n_rotors);
            poses[k].xyz.assign(xyz + static_cast<size_t>(k) * n_atoms * 3, xyz + static_cast<size_t>(k + 1) * n_atoms * 3);
        }
        std::vector<int> maps(bond_mappings, bond_mappings + n_rotors);
        pxd::write_poses(path, smiles ? smiles : "", best_id, bscore, poses, maps, num_rotatable_bonds);
        return PXD_OK;
    } catch (std::exception& ex) {
        g_create_error = ex.what();
        return PXD_ERR_INVALID;
    }
}

int pxd_cluster_poses(int32_t n_poses, int32_t n_atoms, const double* xyz, const double* pscore, const int64_t* nevals,
                      int32_t num_modes, double min_rmsd, int32_t* kept, int32_t* n_kept) {
    if (n_poses < 0 || n_atoms <= 0 || !kept || !n_kept) return PXD_ERR_INVALID;
    std::vector<pxd::PoseResult> c(n_poses);
    for (int k = 0; k < n_poses; ++k) {
        c[k].offset = k;
        c[k].pscore = pscore[k];
        c[k].nevals = static_cast<long>(nevals[k]);
        c[k].xyz.assign(xyz + static_cast<size_t>(k) * n_atoms * 3, xyz + static_cast<size_t>(k + 1) * n_atoms * 3);
    }
    std::vector<pxd::PoseResult> out = pxd::cluster_poses(c, num_modes, min_rmsd);
    *n_kept = static_cast<int32_t>(out.size());
    for (size_t k = 0; k < out.size(); ++k) kept[k] = out[k].offset;
    return PXD_OK;
}

}  // extern "C"
