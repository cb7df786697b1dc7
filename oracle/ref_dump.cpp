// Test infrastructure (oracle only): drives the reference FasterCap solver,
// compiled from its own Solver/*.cpp against the shim headers in oracle/shim,
// step by step and dumps its internal model and results as .npy files.
//
// It follows the manual (non "-a") branch of CSolveCap::SolveMain
// (Solver/SolveCapacitance.cpp:479-531): InputFile -> RefineGeoAndCountLinks
// -> SolveComputeLinks -> SolveForCapacitance, with the tolerance derivation
// of CSolveCap::Run (Solver/SolveCapacitance.cpp:108). Output (directory
// argv[1]):
//   node_*.npy     post-order node array m_pNodes (Solver/Autorefine.cpp:1173-1220)
//   link_src.npy   source node index of every stored link (pointer -> index)
//   link_coef.npy  FP64 coefficient of every link (Solver/Autorefine.cpp:799-826)
//   self_coef.npy, leaf_diel.npy   m_clsSelfPotCoeff and m_pucDielIndex
//   cap.npy        the capacitance matrix of CSolveCap::Solve
//   mv_q.npy/mv_v.npy   seeded q and v = MultiplyMatByVec_fast(q)
//   meta.json      counts, per-conductor data, GMRES iteration counts
// Usage: fcref_dump <outdir> <input file> [FasterCap switches] [--mv N]
#define protected public
#define private public
#include "Solver/SolveCapacitance.h"
#include "FasterCapConsole.h"
#undef protected
#undef private

#include <map>
#include <vector>
#include <string>
#include <sstream>
#include <random>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>

// The dump driver provides the globals of FasterCapGlobal.cpp itself so that it
// can record the solver's log (GMRES iteration lists) as well as echo it.
volatile bool g_bFCContinue = true;
static std::string g_log;

int LogMsg(const char *fmt, ...) {
    char buf[8192];
    va_list ap;
    va_start(ap, fmt);
    int r = vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_log += buf;
    fputs(buf, stderr);
    return r;
}
int ErrMsg(const char *fmt, ...) {
    char buf[8192];
    va_list ap;
    va_start(ap, fmt);
    int r = vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    fputs(buf, stderr);
    return r;
}
int DebugMsg(const char *, ...) { return 0; }

static std::string g_out;

static void write_npy(const char *name, const char *descr, const std::vector<long> &shape, const void *data, size_t elem) {
    std::string path = g_out + "/" + name + ".npy";
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", path.c_str()); exit(2); }
    std::ostringstream h;
    h << "{'descr': '" << descr << "', 'fortran_order': False, 'shape': (";
    size_t n = 1;
    for (size_t i = 0; i < shape.size(); i++) { h << shape[i] << ","; if (i + 1 < shape.size()) h << " "; n *= (size_t)shape[i]; }
    h << "), }";
    std::string hs = h.str();
    size_t total = 10 + hs.size() + 1;
    size_t pad = (64 - total % 64) % 64;
    hs.append(pad, ' ');
    hs += "\n";
    unsigned char pre[10] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0, 0, 0};
    unsigned short hl = (unsigned short)hs.size();
    pre[8] = (unsigned char)(hl & 0xff);
    pre[9] = (unsigned char)(hl >> 8);
    fwrite(pre, 1, 10, f);
    fwrite(hs.data(), 1, hs.size(), f);
    if (n) fwrite(data, elem, n, f);
    fclose(f);
}

template <class T> static void npy(const char *name, const char *descr, const std::vector<T> &v, long cols = 0) {
    std::vector<long> shape;
    if (cols > 0) { shape.push_back((long)v.size() / cols); shape.push_back(cols); }
    else shape.push_back((long)v.size());
    write_npy(name, descr, shape, v.data(), sizeof(T));
}

int main(int argc, char **argv) {
    if (argc < 3) { fprintf(stderr, "usage: fcref_dump <outdir> <input> [switches] [--mv N]\n"); return 64; }
    g_out = argv[1];
    mkdir(g_out.c_str(), 0755);
    // keep an absolute output path: ReadFastCapFile changes the working directory
    if (g_out[0] != '/') { char cwd[4096]; if (getcwd(cwd, sizeof cwd)) g_out = std::string(cwd) + "/" + g_out; }

    int nmv = 2;
    std::string cmd;
    for (int i = 2; i < argc; i++) {
        if (!strcmp(argv[i], "--mv") && i + 1 < argc) { nmv = atoi(argv[++i]); continue; }
        cmd += argv[i];
        cmd += " ";
    }
    FasterCapConsole console;
    CAutoRefGlobalVars gv;
    wxString err;
    if (console.ParseCmdLine(cmd.c_str(), gv, err)) { fprintf(stderr, "%s\n", (const char *)err); return 64; }
    gv.m_dEps = gv.m_dEpsRatio * gv.m_dMeshEps;
    if (gv.m_dEps == 0.0) gv.m_dEps = 0.01;
    // the option checks CSolveCap::Run applies before solving
    // (Solver/SolveCapacitance.cpp:122-147): two-level wins over Jacobi, and
    // its dimension is clamped
    if ((gv.m_ucPrecondType & AUTOREFINE_PRECOND_SUPER) && (gv.m_ucPrecondType & AUTOREFINE_PRECOND_JACOBI))
        gv.m_ucPrecondType = AUTOREFINE_PRECOND_SUPER;
    if (gv.m_ucPrecondType & AUTOREFINE_PRECOND_SUPER) {
        if (gv.m_uiSuperPreDim > SOLVE_MAX_SUPER_PRECOND_NUM) gv.m_uiSuperPreDim = SOLVE_MAX_SUPER_PRECOND_NUM;
        else if (gv.m_uiSuperPreDim < SOLVE_MIN_SUPER_PRECOND_NUM) gv.m_uiSuperPreDim = SOLVE_MIN_SUPER_PRECOND_NUM;
    }

    CSolveCap *solve = new CSolveCap();
    CMultHier &mh = solve->m_clsMulthier;
    int ret = mh.AllocateMemory();
    if (ret == FC_NORMAL_END) { mh.Clean(AUTOREFINE_DEALLMEM_AT_START, gv); ret = solve->InputFile(&gv); }
    if (ret != FC_NORMAL_END) { fprintf(stderr, "input failed %d\n", ret); return ret; }
    solve->m_clsGlobalVars = gv;
    ret = solve->RefineGeoAndCountLinks();
    if (ret == FC_NORMAL_END) ret = solve->SolveComputeLinks();
    if (ret != FC_NORMAL_END) { fprintf(stderr, "links failed %d\n", ret); return ret; }

    unsigned long Nn = mh.GetNodeNum(0), Np = mh.GetPanelNum(0), L = mh.GetLinksNum(0);
    std::map<CAutoElement *, int> idx;
    for (unsigned long i = 0; i < Nn; i++) idx[mh.m_pNodes[i]] = (int)i;

    std::vector<unsigned char> type(Nn), diel(Nn), maxsidei(Nn);
    std::vector<int> left(Nn), right(Nn), cond(Nn);
    std::vector<long long> leaf(Nn), nch(Nn);
    std::vector<unsigned long long> ls(Nn), le(Nn);
    std::vector<float> vert(Nn * 9), cen(Nn * 3), nrm(Nn * 3);
    std::vector<double> dim(Nn), maxside(Nn);
    {
        // conductor of each node: the post-order array is laid out conductor by
        // conductor and each conductor's top element closes its block
        unsigned long n = 0;
        int c = 0;
        for (StlAutoCondDeque::iterator it = mh.m_stlConductors.begin(); it != mh.m_stlConductors.end(); it++, c++) {
            unsigned long top = (unsigned long)idx[(*it)->m_uTopElement.m_pTopElement];
            for (; n <= top; n++) cond[n] = c;
        }
    }
    for (unsigned long i = 0; i < Nn; i++) {
        CAutoPanel *p = (CAutoPanel *)mh.m_pNodes[i];
        type[i] = p->m_ucType;
        left[i] = p->m_pLeft ? idx[p->m_pLeft] : -1;
        right[i] = p->m_pRight ? idx[p->m_pRight] : -1;
        leaf[i] = p->IsLeaf() ? p->m_lIndex[0] : -1;
        nch[i] = (long long)p->m_lNumOfChildren;
        ls[i] = p->m_ulLinkIndexStart[0];
        le[i] = p->m_ulLinkIndexEnd[0];
        for (int k = 0; k < 3; k++) {
            vert[i * 9 + k * 3 + 0] = p->m_clsVertex[k].x;
            vert[i * 9 + k * 3 + 1] = p->m_clsVertex[k].y;
            vert[i * 9 + k * 3 + 2] = p->m_clsVertex[k].z;
        }
        cen[i * 3 + 0] = p->m_clsCentroid.x; cen[i * 3 + 1] = p->m_clsCentroid.y; cen[i * 3 + 2] = p->m_clsCentroid.z;
        nrm[i * 3 + 0] = p->m_clsNormal.x; nrm[i * 3 + 1] = p->m_clsNormal.y; nrm[i * 3 + 2] = p->m_clsNormal.z;
        dim[i] = p->m_dDimension;
        maxside[i] = p->m_dMaxSideLen;
        maxsidei[i] = p->m_ucMaxSide;
        // the permittivity index is defined on conductor leaves only
        diel[i] = (p->IsLeaf() && !(p->m_ucType & AUTOPANEL_IS_DIEL)) ? p->m_ucDielIndex : 0;
    }
    std::vector<int> src(L);
    std::vector<double> coef(L);
    for (unsigned long l = 0; l < L; l++) {
        unsigned long ch = l / AUTOREFINE_LINK_CHUNK_SIZE, pos = l % AUTOREFINE_LINK_CHUNK_SIZE;
        src[l] = idx[mh.m_pdPanelPtrLinks[0][ch][pos]];
        coef[l] = mh.m_dPotCoeffLinks[0][ch][pos];
    }
    std::vector<double> selfc(Np);
    std::vector<unsigned char> leafdiel(Np);
    for (unsigned long i = 0; i < Np; i++) { selfc[i] = mh.m_clsSelfPotCoeff[i]; leafdiel[i] = mh.m_pucDielIndex[i]; }

    npy("node_type", "|u1", type); npy("node_left", "<i4", left); npy("node_right", "<i4", right);
    npy("node_leaf", "<i8", leaf); npy("node_nchildren", "<i8", nch); npy("node_link_start", "<u8", ls);
    npy("node_link_end", "<u8", le); npy("node_vertices", "<f4", vert, 9); npy("node_centroid", "<f4", cen, 3);
    npy("node_normal", "<f4", nrm, 3); npy("node_area", "<f8", dim); npy("node_maxside", "<f8", maxside);
    npy("node_maxside_index", "|u1", maxsidei); npy("node_diel", "|u1", diel); npy("node_cond", "<i4", cond);
    npy("link_src", "<i4", src); npy("link_coef", "<f8", coef);
    npy("self_coef", "<f8", selfc); npy("leaf_diel", "|u1", leafdiel);

    // seeded matrix-vector products through the reference's own operator
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    std::vector<double> mq, mv;
    for (int t = 0; t < nmv; t++) {
        CLin_Vector q(Np), v(Np);
        for (unsigned long i = 0; i < Np; i++) q[i] = U(rng);
        mh.MultiplyMatByVec_fast(&v, &q);
        for (unsigned long i = 0; i < Np; i++) { mq.push_back(q[i]); mv.push_back(v[i]); }
    }
    if (nmv > 0) { npy("mv_q", "<f8", mq, (long)Np); npy("mv_v", "<f8", mv, (long)Np); }

    size_t logmark = g_log.size();
    CLin_Matrix cRe, cIm;
    ret = solve->SolveForCapacitance(&cRe, &cIm);
    if (ret != FC_NORMAL_END) { fprintf(stderr, "solve failed %d\n", ret); return ret; }
    std::vector<double> cap(cRe.m_a.begin(), cRe.m_a.end());
    npy("cap", "<f8", cap, cRe.num_cols());
    // two-level preconditioner as the reference built it
    if ((solve->m_clsGlobalVars.m_ucPrecondType & AUTOREFINE_PRECOND_SUPER) && solve->m_uiSupPreNum > 0) {
        unsigned int msup = solve->m_uiSupPreNum;
        std::vector<int> sn(msup), si(Np);
        std::vector<float> sa(Np);
        std::vector<double> minv((size_t)msup * msup);
        for (unsigned int i = 0; i < msup; i++) sn[i] = idx[solve->m_clsSupPrecondElements[i].m_pclsHiLevLeaf];
        for (unsigned long i = 0; i < Np; i++) { si[i] = (int)solve->m_puiSupPrecondIndex[i]; sa[i] = solve->m_pfSupPrecondAreae[i]; }
        for (unsigned int i = 0; i < msup; i++)
            for (unsigned int j = 0; j < msup; j++) minv[(size_t)i * msup + j] = solve->m_pclsSupPrecondMtx[i][j];
        npy("sup_nodes", "<i4", sn); npy("sup_index", "<i4", si); npy("sup_area", "<f4", sa);
        npy("sup_minv", "<f8", minv, (long)msup);
    }

    // GMRES iteration lists "GMRES Iteration: 0 1 2 ... k" -> k+1 Arnoldi steps
    std::vector<int> iters;
    {
        std::string s = g_log.substr(logmark);
        size_t p = 0;
        while ((p = s.find("GMRES Iteration:", p)) != std::string::npos) {
            size_t e = s.find('\n', p);
            std::istringstream ss(s.substr(p + 16, e - p - 16));
            int x, cnt = 0;
            while (ss >> x) cnt++;
            iters.push_back(cnt);
            p = e;
        }
    }

    FILE *mf = fopen((g_out + "/meta.json").c_str(), "w");
    fprintf(mf, "{\n  \"panels\": %lu, \"nodes\": %lu, \"links\": %lu,\n", Np, Nn, L);
    fprintf(mf, "  \"input_panels\": %lu, \"max_mesh_eps\": %.17g, \"max_level\": %d,\n", mh.m_ulInputPanelNum, mh.m_dMaxMeshEps, mh.m_iMaxLevel);
    fprintf(mf, "  \"max_area\": %.17g, \"max_side\": %.17g, \"eps\": %.17g, \"mesh_eps\": %.17g,\n", mh.m_dMaxArea, mh.m_dMaxSide, gv.m_dEps, gv.m_dMeshEps);
    fprintf(mf, "  \"gmres_tol\": %.17g, \"precond\": %d, \"mesh_curv\": %.17g,\n", gv.m_dGmresTol, (int)gv.m_ucPrecondType, gv.m_dMeshCurvCoeff);
    fprintf(mf, "  \"gmres_iterations\": [");
    for (size_t i = 0; i < iters.size(); i++) fprintf(mf, "%s%d", i ? ", " : "", iters[i]);
    fprintf(mf, "],\n  \"conductors\": [\n");
    int c = 0;
    for (StlAutoCondDeque::iterator it = mh.m_stlConductors.begin(); it != mh.m_stlConductors.end(); it++, c++) {
        CAutoConductor *cd = *it;
        fprintf(mf, "    {\"name\": \"%s\", \"is_diel\": %s, \"leaf_panels\": %lu, \"input_panels\": %lu, \"outperm\": %.17g, \"inperm\": %.17g, \"top\": %d, \"surf_outperm\": [",
                cd->m_sName, cd->m_bIsDiel ? "true" : "false", cd->m_ulLeafPanelNum, cd->m_ulInputPanelNum, cd->m_dOutperm[0], cd->m_dInperm[0],
                idx[cd->m_uTopElement.m_pTopElement]);
        for (int k = 0; k < cd->m_ucMaxSurfOutperm; k++) fprintf(mf, "%s%.17g", k ? ", " : "", cd->m_dSurfOutperm[k][0]);
        fprintf(mf, "]}%s\n", (it + 1) == mh.m_stlConductors.end() ? "" : ",");
    }
    fprintf(mf, "  ]\n}\n");
    fclose(mf);
    fprintf(stderr, "dumped %lu panels, %lu nodes, %lu links to %s\n", Np, Nn, L, g_out.c_str());
    return 0;
}
