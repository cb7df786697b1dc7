// Test infrastructure: the integration glue of INTEGRATION.md, compiled
// against the reference's own objects (oracle/Makefile) and run on its
// models, so that the flattening a FasterCap maintainer would add is real
// code, not prose.
//
// flatten_for_gpu() walks CMultHier's post-order node array m_pNodes
// (Solver/Autorefine.cpp:1173-1220), its link chunks m_pdPanelPtrLinks
// (Solver/Autorefine.h:271-272) and its conductor deque after the link-store
// pass of CAutoRefine::AutoRefineLinks (Solver/Autorefine.cpp:481-728) and
// fills the C-ABI arrays of include/fastercap_gb300.h. SolveOnGpu() is the
// replacement of CSolveCap::SolveForCapacitance -> Solve
// (Solver/SolveCapacitance.cpp:1138-1425) through the C ABI.
//
// Usage: fcref_glue <outdir> <input file> [FasterCap switches] [--gpu]
// Runs the reference's manual branch (Solver/SolveCapacitance.cpp:479-531) up
// to the link pass, flattens the model, checks it with
// fcg_model_arrays_check (host only) and writes the arrays as .npy files into
// <outdir>; with --gpu it also solves through SolveOnGpu and writes cap.npy.
#define protected public
#define private public
#include "Solver/SolveCapacitance.h"
#include "FasterCapConsole.h"
#undef protected
#undef private

#include <map>
#include <string>
#include <vector>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include "fastercap_gb300.h"

volatile bool g_bFCContinue = true;
int LogMsg(const char *, ...) { return 0; }
int ErrMsg(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    int r = vfprintf(stderr, fmt, ap);
    va_end(ap);
    return r;
}
int DebugMsg(const char *, ...) { return 0; }

// ---------------------------------------------------------------- the glue

// The model in the C-ABI layout; the vectors own what `arrays` points to.
struct GpuModel {
    std::vector<uint8_t> type, leaf_diel, is_diel;
    std::vector<int32_t> left, right, src, surf_ptr;
    std::vector<int64_t> leaf_first, leaf_count, link_ptr, cond_first, cond_count;
    std::vector<float> vert, cent, norm;
    std::vector<double> area, maxside, outperm, inperm, surf;
    fcg_model_arrays arrays;
};

static void flatten_for_gpu(CMultHier &mh, GpuModel &g) {
    const unsigned long Nn = mh.GetNodeNum(0), Np = mh.GetPanelNum(0), L = mh.GetLinksNum(0);
    std::map<CAutoElement *, int32_t> index;  // node pointer -> post-order index
    for (unsigned long i = 0; i < Nn; i++) index[mh.m_pNodes[i]] = (int32_t)i;

    g.type.resize(Nn); g.left.resize(Nn); g.right.resize(Nn); g.src.resize(L);
    g.leaf_first.resize(Nn); g.leaf_count.resize(Nn); g.link_ptr.resize(Nn + 1);
    g.vert.resize(9 * Nn); g.cent.resize(3 * Nn); g.norm.resize(3 * Nn);
    g.area.resize(Nn); g.maxside.resize(Nn); g.leaf_diel.assign(Np, 0);
    for (unsigned long i = 0; i < Nn; i++) {
        CAutoPanel *p = (CAutoPanel *)mh.m_pNodes[i];
        g.type[i] = p->m_ucType;
        g.left[i] = p->m_pLeft ? index[p->m_pLeft] : -1;
        g.right[i] = p->m_pRight ? index[p->m_pRight] : -1;
        g.leaf_count[i] = (int64_t)p->m_lNumOfChildren;
        g.leaf_first[i] = p->IsLeaf() ? (int64_t)p->m_lIndex[0] : g.leaf_first[g.left[i]];
        for (int k = 0; k < 3; k++) {
            g.vert[9 * i + 3 * k] = p->m_clsVertex[k].x;
            g.vert[9 * i + 3 * k + 1] = p->m_clsVertex[k].y;
            g.vert[9 * i + 3 * k + 2] = p->m_clsVertex[k].z;
        }
        g.cent[3 * i] = p->m_clsCentroid.x; g.cent[3 * i + 1] = p->m_clsCentroid.y; g.cent[3 * i + 2] = p->m_clsCentroid.z;
        g.norm[3 * i] = p->m_clsNormal.x; g.norm[3 * i + 1] = p->m_clsNormal.y; g.norm[3 * i + 2] = p->m_clsNormal.z;
        g.area[i] = p->m_dDimension;
        g.maxside[i] = p->m_dMaxSideLen;
        g.link_ptr[i] = (int64_t)p->m_ulLinkIndexStart[0];
        // a conductor leaf's permittivity index (the reference copies it to
        // m_pucDielIndex only in its coefficient loop, which the GPU replaces)
        if (p->IsLeaf() && !(p->m_ucType & AUTOPANEL_IS_DIEL)) g.leaf_diel[p->m_lIndex[0]] = p->m_ucDielIndex;
    }
    g.link_ptr[Nn] = (int64_t)L;
    for (unsigned long l = 0; l < L; l++)
        g.src[l] = index[mh.m_pdPanelPtrLinks[0][l / AUTOREFINE_LINK_CHUNK_SIZE][l % AUTOREFINE_LINK_CHUNK_SIZE]];
    // conductors in deque order: leaf ranges, permittivities, dielectric flags
    g.surf_ptr.assign(1, 0);
    int64_t first = 0;
    for (StlAutoCondDeque::iterator it = mh.m_stlConductors.begin(); it != mh.m_stlConductors.end(); it++) {
        g.is_diel.push_back((*it)->m_bIsDiel ? 1 : 0);
        g.cond_first.push_back(first);
        g.cond_count.push_back((int64_t)(*it)->m_ulLeafPanelNum);
        first += (int64_t)(*it)->m_ulLeafPanelNum;
        g.outperm.push_back((*it)->m_dOutperm[0]);
        g.inperm.push_back((*it)->m_dInperm[0]);
        for (int k = 0; k < (*it)->m_ucMaxSurfOutperm; k++) g.surf.push_back((*it)->m_dSurfOutperm[k][0]);
        g.surf_ptr.push_back((int32_t)g.surf.size());
    }
    if (g.surf.empty()) g.surf.push_back(0.0);
    fcg_model_arrays a = {(int64_t)Nn, (int64_t)Np, (int64_t)L, (int32_t)g.is_diel.size(),
                          g.type.data(), g.left.data(), g.right.data(), g.leaf_first.data(), g.leaf_count.data(),
                          g.vert.data(), g.cent.data(), g.norm.data(), g.area.data(), g.maxside.data(),
                          g.link_ptr.data(), g.src.data(), g.leaf_diel.data(), g.is_diel.data(), g.cond_first.data(),
                          g.cond_count.data(), g.outperm.data(), g.inperm.data(), g.surf_ptr.data(), g.surf.data()};
    g.arrays = a;
}

// replaces SolveForCapacitance -> Solve -> gmresPrecondSFastAll
static int SolveOnGpu(CSolveCap &solve, CLin_Matrix *cRe) {
    GpuModel g;
    flatten_for_gpu(solve.m_clsMulthier, g);
    fcg_context *ctx = NULL;
    fcg_problem *prob = NULL;
    int ret = fcg_context_create(0, &ctx);
    if (ret == FCG_NORMAL_END) ret = fcg_problem_create(ctx, &g.arrays, FCG_PREC_MIXED, &prob);
    if (ret == FCG_NORMAL_END) ret = fcg_problem_fill(prob);  // replaces the PotEstimateOpt loop
    if (ret == FCG_NORMAL_END) {
        int nc = 0;
        for (size_t c = 0; c < g.is_diel.size(); c++) nc += g.is_diel[c] ? 0 : 1;
        cRe->newsize(nc, nc);
        std::vector<double> cap((size_t)nc * nc);
        fcg_solve_options so = {solve.m_clsGlobalVars.m_dGmresTol, FCG_PRECOND_JACOBI, 0, 0, 0, 0, FCG_KRYLOV_PAIR};
        if (solve.m_clsGlobalVars.m_ucPrecondType & AUTOREFINE_PRECOND_SUPER) {
            so.precond = FCG_PRECOND_TWO_LEVEL;
            so.precond_dim = (int)solve.m_clsGlobalVars.m_uiSuperPreDim;
        } else if (!(solve.m_clsGlobalVars.m_ucPrecondType & AUTOREFINE_PRECOND_JACOBI)) {
            so.precond = FCG_PRECOND_NONE;
        }
        ret = fcg_problem_solve(prob, &so, cap.data(), NULL);  // replaces Solve()
        for (int r = 0; r < nc; r++)
            for (int c = 0; c < nc; c++) (*cRe)[r][c] = cap[(size_t)r * nc + c];
    }
    if (prob) fcg_problem_destroy(prob);
    if (ctx) fcg_context_destroy(ctx);
    if (ret != FCG_NORMAL_END && ret != FCG_NOT_CONVERGED) ErrMsg("GPU solve failed: %s\n", fcg_last_error());
    return ret == FCG_NOT_CONVERGED ? FC_NORMAL_END : ret;  // the reference reports, then continues
}

// ---------------------------------------------------------------- driver

static std::string g_out;

template <class T> static void npy(const char *name, const char *descr, const std::vector<T> &v, long cols = 0) {
    std::string path = g_out + "/" + name + ".npy";
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", path.c_str()); exit(2); }
    char shape[64];
    if (cols > 0) snprintf(shape, sizeof shape, "(%ld, %ld)", (long)(v.size() / cols), cols);
    else snprintf(shape, sizeof shape, "(%ld,)", (long)v.size());
    std::string h = std::string("{'descr': '") + descr + "', 'fortran_order': False, 'shape': " + shape + ", }";
    size_t total = 10 + h.size() + 1;
    h.append((64 - total % 64) % 64, ' ');
    h += "\n";
    unsigned char pre[10] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0, (unsigned char)(h.size() & 0xff), (unsigned char)(h.size() >> 8)};
    fwrite(pre, 1, 10, f);
    fwrite(h.data(), 1, h.size(), f);
    if (!v.empty()) fwrite(v.data(), sizeof(T), v.size(), f);
    fclose(f);
}

int main(int argc, char **argv) {
    if (argc < 3) { fprintf(stderr, "usage: fcref_glue <outdir> <input> [switches] [--gpu]\n"); return 64; }
    g_out = argv[1];
    mkdir(g_out.c_str(), 0755);
    // ReadFastCapFile changes the working directory: keep an absolute path
    if (g_out[0] != '/') { char cwd[4096]; if (getcwd(cwd, sizeof cwd)) g_out = std::string(cwd) + "/" + g_out; }
    bool gpu = false;
    std::string cmd;
    for (int i = 2; i < argc; i++) {
        if (!strcmp(argv[i], "--gpu")) { gpu = true; continue; }
        cmd += argv[i];
        cmd += " ";
    }
    FasterCapConsole console;
    CAutoRefGlobalVars gv;
    wxString err;
    if (console.ParseCmdLine(cmd.c_str(), gv, err)) { fprintf(stderr, "%s\n", (const char *)err); return 64; }
    gv.m_dEps = gv.m_dEpsRatio * gv.m_dMeshEps;
    if (gv.m_dEps == 0.0) gv.m_dEps = 0.01;
    CSolveCap *solve = new CSolveCap();
    CMultHier &mh = solve->m_clsMulthier;
    int ret = mh.AllocateMemory();
    if (ret == FC_NORMAL_END) { mh.Clean(AUTOREFINE_DEALLMEM_AT_START, gv); ret = solve->InputFile(&gv); }
    if (ret != FC_NORMAL_END) { fprintf(stderr, "input failed %d\n", ret); return ret; }
    solve->m_clsGlobalVars = gv;
    ret = solve->RefineGeoAndCountLinks();
    if (ret == FC_NORMAL_END) ret = solve->SolveComputeLinks();
    if (ret != FC_NORMAL_END) { fprintf(stderr, "links failed %d\n", ret); return ret; }

    GpuModel g;
    flatten_for_gpu(mh, g);
    int check = fcg_model_arrays_check(&g.arrays);
    if (check != FCG_NORMAL_END) { fprintf(stderr, "fcg_model_arrays_check: %s\n", fcg_last_error()); return 3; }
    npy("node_type", "|u1", g.type); npy("node_left", "<i4", g.left); npy("node_right", "<i4", g.right);
    npy("node_leaf_first", "<i8", g.leaf_first); npy("node_leaf_count", "<i8", g.leaf_count);
    npy("node_vertices", "<f4", g.vert, 9); npy("node_centroid", "<f4", g.cent, 3); npy("node_normal", "<f4", g.norm, 3);
    npy("node_area", "<f8", g.area); npy("node_maxside", "<f8", g.maxside); npy("link_ptr", "<i8", g.link_ptr);
    npy("link_src", "<i4", g.src); npy("leaf_diel", "|u1", g.leaf_diel); npy("cond_is_diel", "|u1", g.is_diel);
    npy("cond_leaf_first", "<i8", g.cond_first); npy("cond_leaf_count", "<i8", g.cond_count);
    npy("cond_outperm", "<f8", g.outperm); npy("cond_inperm", "<f8", g.inperm); npy("cond_surf_ptr", "<i4", g.surf_ptr);
    npy("cond_surf_outperm", "<f8", g.surf);
    if (gpu) {
        CLin_Matrix cRe;
        ret = SolveOnGpu(*solve, &cRe);
        if (ret != FC_NORMAL_END) return ret;
        std::vector<double> cap(cRe.m_a.begin(), cRe.m_a.end());
        npy("cap", "<f8", cap, cRe.num_cols());
    }
    fprintf(stderr, "flattened %lu nodes, %lu links\n", mh.GetNodeNum(0), mh.GetLinksNum(0));
    return 0;
}
