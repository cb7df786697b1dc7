// Host-side model of a FasterCap extraction: the panel hierarchy and the
// interaction links, built from a FastCap-format input file and flattened
// into the structure-of-arrays layout the device kernels consume.
#ifndef FCG_HOST_MODEL_HPP
#define FCG_HOST_MODEL_HPP

#include <stdint.h>
#include <memory>
#include <string>
#include <vector>

namespace fcg {

// Build options: the subset of the reference's CAutoRefGlobalVars
// (Solver/SolverGlobal.h:162-183) that shapes the mesh and the links.
struct BuildOptions {
    double mesh_eps = 0.1;        // -m   (m_dMeshEps)
    double eps_ratio = 1.0;       // -d   (m_dEpsRatio); link eps = d * m
    double mesh_curv = 3.0;       // -mc  (m_dMeshCurvCoeff)
    bool verbose = false;
    // device builds only: leave the link sources in device memory
    // (Model::d_link_src) instead of copying them to link_src
    bool links_on_device = false;
};

// One element of the hierarchy: an input panel, a refined sub-panel or a
// super node. Geometry is single precision like the reference's panels.
struct Element {
    float v[9];
    float c[3];
    float n[3];
    double area = 0.0;
    double maxside = 0.0;
    int32_t left = -1, right = -1;
    uint8_t type = 1;       // FCG_IS_LEAF until subdivided or made a super node
    uint8_t maxside_idx = 0;
    uint8_t diel = 0;       // index into the owning conductor's outer permittivities
};

struct Conductor {
    std::string name;
    bool is_diel = false;
    double outperm = 1.0, inperm = 0.0;
    double ref[3] = {0, 0, 0};         // dielectric reference point (outperm side)
    std::vector<double> surf_outperm;  // distinct outer permittivities around a conductor
    std::vector<int32_t> panels;       // input panels (element ids), in creation order
    int32_t top = -1;                  // root element after the super hierarchy
    int64_t leaf_count = 0;
};

// Flattened model (post-order node array, CSR links by destination node).
struct Model {
    // nodes
    int64_t n_nodes = 0, n_panels = 0, n_links = 0;
    std::vector<uint8_t> type;
    std::vector<int32_t> left, right, cond;
    std::vector<int64_t> leaf_first, leaf_count;   // contiguous leaf range of every node
    std::vector<int64_t> link_ptr;                 // n_nodes + 1
    std::vector<float> vert, cent, norm;           // 9, 3, 3 per node
    std::vector<double> area, maxside;
    std::vector<uint8_t> maxside_idx;
    // links
    std::vector<int32_t> link_src;
    // the link sources in device memory when the build left them there
    // (BuildOptions::links_on_device); link_src is then empty
    std::shared_ptr<int32_t> d_link_src;
    // leaves
    std::vector<int32_t> leaf_node;                // node of every leaf
    std::vector<uint8_t> leaf_diel;
    // conductors, in solver order (dielectric interfaces first)
    std::vector<Conductor> conductors;
    std::vector<int64_t> cond_leaf_first;
    // statistics, mirroring the reference's solve statistics
    int64_t input_panels = 0, raw_cond_panels = 0, raw_diel_panels = 0;
    double max_mesh_eps = 0.0, max_area = 0.0, max_side = 0.0, total_area = 0.0;
    double eps = 0.0, mesh_eps = 0.0;
    int max_level = 0;
    std::vector<std::string> warnings;
};

// Status codes, same values as the reference's FC_* codes (Solver/SolverGlobal.h:39-49).
enum Status {
    FC_NORMAL_END = 0,
    FC_GENERIC_ERROR = 1,
    FC_COMMAND_LINE_ERROR = 64,
    FC_CANNOT_OPEN_FILE = 66,
    FC_OUT_OF_MEMORY = 71,
    FC_FILE_ERROR = 74,
    FC_USER_BREAK = 125,
};

struct DeviceContext;

// Parse, build the super hierarchy, refine the mesh, construct the links and
// flatten. Returns an FC_* status; on error `err` holds a message. With a
// device context the link construction runs on that GPU (same arrays).
int build_model(const std::string &path, const BuildOptions &opt, Model &out, std::string &err, DeviceContext *dev = nullptr);

}  // namespace fcg

#endif
