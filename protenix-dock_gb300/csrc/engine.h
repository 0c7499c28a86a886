// The engine facade: bytedock::ReusableEngine (engine/include/bytedock/core/entrance.h:30-74)
// on the GB300 C ABI. Files in, files out: receptor / ligand / scoring-function JSON in,
// <ligand>_out.json and the evaluation CSV out, in the reference's formats
// (engine/src/core/writer.cpp:40-230). Each workflow call runs one batched device launch
// over every pose (optimize) or walker (search) of every ligand in the index file.
// Host code only; errors are std::runtime_error with the reference's messages.
#ifndef PXD_ENGINE_H_
#define PXD_ENGINE_H_

#include <memory>
#include <string>
#include <vector>

#include "../../include/pxdock_gb300.h"

namespace pxd {

struct ReceptorData;

// One optimised pose as the writer prints it (optimized_result, task.h:32-41).
struct PoseResult {
    int offset = 0;
    double energy = 0.0, pscore = 0.0;
    long nevals = 0;
    std::vector<double> torsions;  // receptor torsions in leaf order
    std::vector<double> xyz;       // ligand [N][3]
};

class Engine {
public:
    Engine(const std::string& receptor_file, const std::string& sf_file, int cpu_nthreads, int device);
    ~Engine();
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;

    void set_box(double cx, double cy, double cz, double sx, double sy, double sz);
    void generate_maps(double grid_spacing, double max_size);
    void dump_maps(const std::string& cache_dir);
    void load_maps(const std::string& cache_dir);
    void drop_maps();
    void evaluate(const std::string& ligand_index_file, const std::string& output_file);
    void optimize(const std::string& ligand_index_file, const std::string& output_dir, int max_niters, double slope);
    // variables of optimize's L-BFGS: PXD_DOF_CARTESIAN (the reference) or PXD_DOF_RIGID_TORSION
    void set_dof_mode(int mode);
    void search(const std::string& ligand_index_file, const std::string& output_dir, int seed, int exhaustiveness,
                int max_nsteps, int relax_nsteps, int num_modes, double min_rmsd, double mc_mmenergy_threshold,
                double slope);

private:
    void require_box() const;
    void require_maps() const;
    void load_own_maps(const std::string& cache_dir);
    pxd_context* ctx_ = nullptr;
    std::unique_ptr<ReceptorData> receptor_;
    std::vector<double> box_;  // set_box appends, as the reference's box_ vector does
    bool has_maps_ = false;
    pxd_box grid_{};
    int nthreads_ = 1;
    int dof_mode_ = PXD_DOF_CARTESIAN;
};

// pose_writer::consume (writer.cpp:40-81): the <ligand>_out.json text
void write_poses(const std::string& path, const std::string& smiles, int best_id, double bscore,
                 const std::vector<PoseResult>& poses, const std::vector<int>& bond_mappings, int num_rotatable_bonds);
// pose_cluster::preprocess (writer.cpp:115-160): greedy RMSD clustering, sorted by pose score
std::vector<PoseResult> cluster_poses(const std::vector<PoseResult>& candidates, int num_modes, double min_rmsd);

// engine log ("-" = standard error), verbosity 0 warnings, 1 info, 2 debug
void set_log(const std::string& path, int verbosity);

}  // namespace pxd

#endif  // PXD_ENGINE_H_
