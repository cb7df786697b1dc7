// C ABI of fastercap_gb300 (include/fastercap_gb300.h): model construction,
// device problems and the reference-compatible command-line driver.
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <chrono>
#include <string>
#include <vector>
#include <algorithm>
#include <new>

#include "../../include/fastercap_gb300.h"
#include "../csrc/fcg_internal.hpp"
#include "handles.hpp"
#include "model.hpp"

namespace fcg {
static thread_local std::string g_err;
void set_error(const std::string &msg) { g_err = msg; }
const char *get_error() { return g_err.c_str(); }
}  // namespace fcg

struct fcg_model {
    fcg::Model m;
    // flattened conductor arrays for the C view
    std::vector<uint8_t> cond_is_diel;
    std::vector<int64_t> cond_first, cond_count;
    std::vector<double> cond_out, cond_in, surf;
    std::vector<int32_t> surf_ptr;
};


static void finish_model(fcg_model *fm) {
    fcg::Model &m = fm->m;
    fm->surf_ptr.assign(1, 0);
    for (size_t c = 0; c < m.conductors.size(); c++) {
        const fcg::Conductor &C = m.conductors[c];
        fm->cond_is_diel.push_back(C.is_diel ? 1 : 0);
        fm->cond_first.push_back(m.cond_leaf_first[c]);
        fm->cond_count.push_back(C.leaf_count);
        fm->cond_out.push_back(C.outperm);
        fm->cond_in.push_back(C.inperm);
        fm->surf.insert(fm->surf.end(), C.surf_outperm.begin(), C.surf_outperm.end());
        fm->surf_ptr.push_back((int32_t)fm->surf.size());
    }
    if (fm->surf.empty()) fm->surf.push_back(0.0);
}

extern "C" {

int fcg_model_build(const char *path, const fcg_build_options *opt, fcg_model **out, char *err, size_t err_len) {
    return fcg_model_build_on(NULL, path, opt, out, err, err_len);
}

}  // extern "C"

static int build_on(fcg::DeviceContext *dev, const char *path, const fcg_build_options *opt, bool links_on_device,
                    fcg_model **out, char *err, size_t err_len);

namespace fcg {
// a server job's model: built on the server's GPU with the link sources left
// in device memory (problem creation copies them device to device)
int model_build_device_links(DeviceContext *dev, const char *path, const fcg_build_options *opt, fcg_model **out, char *err,
                             size_t err_len) {
    return build_on(dev, path, opt, true, out, err, err_len);
}
}  // namespace fcg

extern "C" int fcg_model_build_on(fcg_context *ctx, const char *path, const fcg_build_options *opt, fcg_model **out,
                                  char *err, size_t err_len) {
    return build_on(ctx ? ctx->dev : nullptr, path, opt, false, out, err, err_len);
}

static int build_on(fcg::DeviceContext *dev, const char *path, const fcg_build_options *opt, bool links_on_device,
                    fcg_model **out, char *err, size_t err_len) {
    if (!path || !out) return FCG_GENERIC_ERROR;
    *out = NULL;
    fcg::BuildOptions o;
    if (opt) {
        o.mesh_eps = opt->mesh_eps;
        o.eps_ratio = opt->eps_ratio;
        o.mesh_curv = opt->mesh_curv;
        o.verbose = opt->verbose != 0;
    }
    o.links_on_device = links_on_device && dev;
    fcg_model *fm = new (std::nothrow) fcg_model();
    if (!fm) return FCG_OUT_OF_MEMORY;
    std::string e;
    int r;
    try {
        r = fcg::build_model(path, o, fm->m, e, dev);
    } catch (std::bad_alloc &) {
        r = FCG_OUT_OF_MEMORY;
        e = "out of host memory while building the model";
    }
    if (r != FCG_NORMAL_END) {
        fcg::set_error(e);
        if (err && err_len) snprintf(err, err_len, "%s", e.c_str());
        delete fm;
        return r;
    }
    finish_model(fm);
    *out = fm;
    return FCG_NORMAL_END;
}

extern "C" {

int fcg_model_info_get(const fcg_model *fm, fcg_model_info *info) {
    if (!fm || !info) return FCG_GENERIC_ERROR;
    const fcg::Model &m = fm->m;
    info->n_nodes = m.n_nodes;
    info->n_panels = m.n_panels;
    info->n_links = m.n_links;
    info->input_panels = m.input_panels;
    info->n_conductors = (int32_t)m.conductors.size();
    int nd = 0;
    for (size_t c = 0; c < m.conductors.size(); c++) nd += m.conductors[c].is_diel ? 1 : 0;
    info->n_dielectrics = nd;
    info->max_level = m.max_level;
    info->max_mesh_eps = m.max_mesh_eps;
    info->eps = m.eps;
    info->mesh_eps = m.mesh_eps;
    return FCG_NORMAL_END;
}

int fcg_model_arrays_get(const fcg_model *fm, fcg_model_arrays *a) {
    if (!fm || !a) return FCG_GENERIC_ERROR;
    const fcg::Model &m = fm->m;
    a->n_nodes = m.n_nodes;
    a->n_panels = m.n_panels;
    a->n_links = m.n_links;
    a->n_conductors = (int32_t)m.conductors.size();
    a->node_type = m.type.data();
    a->node_left = m.left.data();
    a->node_right = m.right.data();
    a->node_leaf_first = m.leaf_first.data();
    a->node_leaf_count = m.leaf_count.data();
    a->node_vertices = m.vert.data();
    a->node_centroid = m.cent.data();
    a->node_normal = m.norm.data();
    a->node_area = m.area.data();
    a->node_maxside = m.maxside.data();
    a->link_ptr = m.link_ptr.data();
    a->link_src = m.d_link_src ? m.d_link_src.get() : m.link_src.data();
    a->leaf_diel = m.leaf_diel.data();
    a->cond_is_diel = fm->cond_is_diel.data();
    a->cond_leaf_first = fm->cond_first.data();
    a->cond_leaf_count = fm->cond_count.data();
    a->cond_outperm = fm->cond_out.data();
    a->cond_inperm = fm->cond_in.data();
    a->cond_surf_ptr = fm->surf_ptr.data();
    a->cond_surf_outperm = fm->surf.data();
    return FCG_NORMAL_END;
}

const char *fcg_model_conductor_name(const fcg_model *fm, int32_t i) {
    if (!fm || i < 0 || i >= (int32_t)fm->m.conductors.size()) return NULL;
    return fm->m.conductors[i].name.c_str();
}

void fcg_model_free(fcg_model *fm) { delete fm; }

int fcg_model_concat(const fcg_model *const *models, int32_t n, fcg_model **out, int32_t *geom_of_cond) {
    if (!models || n <= 0 || !out) return FCG_GENERIC_ERROR;
    *out = NULL;
    fcg_model *fm = new (std::nothrow) fcg_model();
    if (!fm) return FCG_OUT_OF_MEMORY;
    fcg::Model &M = fm->m;
    try {
        int64_t node_off = 0, leaf_off = 0, link_off = 0;
        int32_t ci = 0;
        M.link_ptr.push_back(0);
        for (int32_t g = 0; g < n; g++) {
            if (!models[g]) { delete fm; return FCG_GENERIC_ERROR; }
            const fcg::Model &A = models[g]->m;
            for (int64_t i = 0; i < A.n_nodes; i++) {
                M.type.push_back(A.type[i]);
                M.left.push_back(A.left[i] >= 0 ? (int32_t)(A.left[i] + node_off) : -1);
                M.right.push_back(A.right[i] >= 0 ? (int32_t)(A.right[i] + node_off) : -1);
                M.cond.push_back(A.cond[i] + ci);
                M.leaf_first.push_back(A.leaf_first[i] + leaf_off);
                M.leaf_count.push_back(A.leaf_count[i]);
                M.link_ptr.push_back(A.link_ptr[i + 1] + link_off);
                M.area.push_back(A.area[i]);
                M.maxside.push_back(A.maxside[i]);
                M.maxside_idx.push_back(A.maxside_idx[i]);
            }
            M.vert.insert(M.vert.end(), A.vert.begin(), A.vert.end());
            M.cent.insert(M.cent.end(), A.cent.begin(), A.cent.end());
            M.norm.insert(M.norm.end(), A.norm.begin(), A.norm.end());
            for (int64_t l = 0; l < A.n_links; l++) M.link_src.push_back((int32_t)(A.link_src[l] + node_off));
            for (int64_t j = 0; j < A.n_panels; j++) {
                M.leaf_node.push_back((int32_t)(A.leaf_node[j] + node_off));
                M.leaf_diel.push_back(A.leaf_diel[j]);
            }
            for (size_t c = 0; c < A.conductors.size(); c++) {
                M.conductors.push_back(A.conductors[c]);
                M.cond_leaf_first.push_back(A.cond_leaf_first[c] + leaf_off);
                if (geom_of_cond) geom_of_cond[ci] = g;
                ci++;
            }
            node_off += A.n_nodes;
            leaf_off += A.n_panels;
            link_off += A.n_links;
            M.input_panels += A.input_panels;
            M.max_level = std::max(M.max_level, A.max_level);
            M.max_mesh_eps = std::max(M.max_mesh_eps, A.max_mesh_eps);
        }
        if (node_off > 0x1FFFFFFF || link_off > 0x7fffffff) {
            delete fm;
            fcg::set_error("concatenated model too large");
            return FCG_OUT_OF_MEMORY;
        }
        M.n_nodes = node_off;
        M.n_panels = leaf_off;
        M.n_links = link_off;
    } catch (std::bad_alloc &) {
        delete fm;
        return FCG_OUT_OF_MEMORY;
    }
    finish_model(fm);
    *out = fm;
    return FCG_NORMAL_END;
}

const char *fcg_last_error(void) { return fcg::get_error(); }

int fcg_context_create(int device, fcg_context **out) {
    if (!out) return FCG_GENERIC_ERROR;
    *out = NULL;
    fcg_context *c = new fcg_context();
    c->dev = new fcg::DeviceContext();
    int r = fcg::context_init(*c->dev, device);
    if (r != FCG_NORMAL_END) { fcg::context_unref(c->dev); delete c; return r; }
    *out = c;
    return FCG_NORMAL_END;
}

void fcg_context_destroy(fcg_context *ctx) {
    if (!ctx) return;
    fcg::context_unref(ctx->dev);
    delete ctx;
}

void *fcg_context_stream(fcg_context *ctx) { return ctx ? ctx->dev->stream : NULL; }

int fcg_problem_create(fcg_context *ctx, const fcg_model_arrays *a, int precision, fcg_problem **out) {
    return fcg_problem_create_on_stream(ctx, a, precision, ctx ? ctx->dev->stream : NULL, out);
}

int fcg_problem_create_on_stream(fcg_context *ctx, const fcg_model_arrays *a, int precision, void *stream, fcg_problem **out) {
    if (!ctx || !a || !out) return FCG_GENERIC_ERROR;
    *out = NULL;
    fcg::DeviceProblem *p = NULL;
    int r = fcg::problem_create(*ctx->dev, *a, precision, stream, &p);
    if (r != FCG_NORMAL_END) return r;
    *out = new fcg_problem();
    (*out)->p = p;
    return FCG_NORMAL_END;
}

void fcg_problem_destroy(fcg_problem *p) {
    if (!p) return;
    fcg::problem_destroy(p->p);
    delete p;
}

int64_t fcg_problem_device_bytes(const fcg_problem *p) { return p ? fcg::problem_device_bytes(p->p) : 0; }
int fcg_problem_fill(fcg_problem *p) { return p ? fcg::problem_fill(p->p) : FCG_GENERIC_ERROR; }
int fcg_problem_get_coefficients(fcg_problem *p, double *lc, double *sc) {
    return p ? fcg::problem_get_coefficients(p->p, lc, sc) : FCG_GENERIC_ERROR;
}
int fcg_problem_matvec(fcg_problem *p, const double *q, double *v, int k) {
    return (p && q && v && k > 0) ? fcg::problem_matvec_host(p->p, q, v, k) : FCG_GENERIC_ERROR;
}
int fcg_problem_matvec_device(fcg_problem *p, const double *q, double *v, int k) {
    return (p && q && v && k > 0) ? fcg::problem_matvec_device(p->p, q, v, k) : FCG_GENERIC_ERROR;
}
int fcg_problem_matvec_device_noalloc(fcg_problem *p, const double *q, double *v, int k) {
    return (p && q && v && k > 0) ? fcg::problem_matvec_noalloc(p->p, q, v, k) : FCG_GENERIC_ERROR;
}
int fcg_problem_solve(fcg_problem *p, const fcg_solve_options *opt, double *cap, int *iterations) {
    if (!p) return FCG_GENERIC_ERROR;
    fcg_solve_options o;
    o.tol = 0.01;
    o.precond = FCG_PRECOND_JACOBI;
    o.max_iter = 0;
    o.rhs_width = 0;
    o.precond_dim = 0;
    o.refine = 0;
    o.krylov = FCG_KRYLOV_PAIR;
    if (opt) o = *opt;
    return fcg::problem_solve(p->p, o, cap, iterations);
}
int fcg_problem_get_charges(fcg_problem *p, double *charges) {
    return (p && charges) ? fcg::problem_get_charges(p->p, charges) : FCG_GENERIC_ERROR;
}

int fcg_model_arrays_check(const fcg_model_arrays *a) {
    if (!a) return FCG_GENERIC_ERROR;
    std::string bad = fcg::model_check(*a);
    if (bad.empty()) return FCG_NORMAL_END;
    fcg::set_error("invalid model: " + bad);
    return FCG_GENERIC_ERROR;
}

int fcg_problem_cancel(fcg_problem *p) {
    if (!p) return FCG_GENERIC_ERROR;
    fcg::problem_cancel(p->p);
    return FCG_NORMAL_END;
}

int64_t fcg_problem_estimate_bytes(const fcg_model_arrays *a, int precision, int rhs, int iterations) {
    return a ? fcg::problem_estimate_bytes(*a, precision, rhs, iterations) : -1;
}

int fcg_problem_set_geometries(fcg_problem *p, int32_t n, const int32_t *geom) {
    return p ? fcg::problem_set_geometries(p->p, n, geom) : FCG_GENERIC_ERROR;
}

int fcg_problem_set_profiling(fcg_problem *p, int enable) {
    return p ? fcg::problem_set_profiling(p->p, enable != 0) : FCG_GENERIC_ERROR;
}

int fcg_problem_set_tuning(fcg_problem *p, int enable) {
    return p ? fcg::problem_set_tuning(p->p, enable != 0) : FCG_GENERIC_ERROR;
}

int fcg_problem_get_stats(fcg_problem *p, fcg_problem_stats *st) {
    if (!p || !st) return FCG_GENERIC_ERROR;
    fcg::SolveTimings t = fcg::problem_timings(p->p);
    st->kernel_launches = t.launches;
    st->link_launches = t.link_launches;
    st->link_ms = t.link_ms;
    st->link_bytes = t.link_bytes;
    st->fill_ms = t.fill_ms;
    st->solve_ms = t.solve_ms;
    st->refine_checks = t.refine_checks;
    st->refine_cycles = t.refine_cycles;
    st->fill_fp64 = t.fill_fp64;
    st->rhs_width = t.rhs_width;
    return FCG_NORMAL_END;
}

int fcg_problem_reset_stats(fcg_problem *p) {
    if (!p) return FCG_GENERIC_ERROR;
    fcg::problem_reset_stats(p->p);
    return FCG_NORMAL_END;
}

}  // extern "C"

// ------------------------------------------------------------------ driver

namespace {

struct CmdOptions {
    std::string file;
    double mesh_eps = 0.1, eps_ratio = 1.0, mesh_curv = 3.0, gmres_tol = 0.01, out_of_core = 5.0, max_disc_side = 0.1;
    double auto_err = 0.01;
    int precond = FCG_PRECOND_JACOBI;
    unsigned super_dim = 128, block_size = 32;
    bool automatic = false, auto_precond = false, galerkin = false, dump_residual = false, dump_time = false, verbose = false;
    bool out_geo = false, dump_input = false, out_cap = false, out_charge = false, keep_charge = false;
    int precision = FCG_PREC_MIXED;
};

// Same grammar as FasterCapConsole::ParseCmdLine (FasterCapConsole.cpp:136-357):
// options are matched on their first letters; returns true on error.
bool parse_cmd(const char *cmd, CmdOptions &o, std::string &err) {
    std::vector<std::string> args;
    const char *p = cmd;
    while (*p) {
        while (*p == ' ' || *p == '\t' || *p == '\n') p++;
        if (!*p) break;
        std::string tok;
        if (*p == '"') {
            p++;
            while (*p && *p != '"') tok += *p++;
            if (*p == '"') p++;
        } else {
            while (*p && *p != ' ' && *p != '\t' && *p != '\n') {
                if (*p == '"') { p++; continue; }
                tok += *p++;
            }
        }
        args.push_back(tok);
    }
    if (args.empty()) { err = "FasterCap launched without enough arguments! You must specify at least the input file name"; return true; }
    for (size_t i = 0; i < args.size(); i++) {
        const std::string &a = args[i];
        if (a.size() && a[0] == '-') {
            char c1 = a.size() > 1 ? a[1] : 0, c2 = a.size() > 2 ? a[2] : 0;
            const char *rest2 = a.c_str() + (a.size() > 2 ? 2 : a.size());
            const char *rest3 = a.c_str() + (a.size() > 3 ? 3 : a.size());
            if (c1 == 's') {
                if (sscanf(rest2, "%lf", &o.max_disc_side) != 1) { err = "unsupported parameter '" + a + "'"; return true; }
            } else if (c1 == 'm') {
                if (c2 == 'c') {
                    if (sscanf(rest3, "%lf", &o.mesh_curv) != 1) { err = "bad mesh curvature coefficient '" + a + "'"; return true; }
                } else if (sscanf(rest2, "%lf", &o.mesh_eps) != 1) { err = "bad mesh relative refinement value '" + a + "'"; return true; }
            } else if (c1 == 'd') {
                if (sscanf(rest2, "%lf", &o.eps_ratio) != 1) { err = "bad direct potential interaction coefficient '" + a + "'"; return true; }
            } else if (c1 == 'f') {
                if (sscanf(rest2, "%lf", &o.out_of_core) != 1) { err = "bad out-of-core ratio '" + a + "'"; return true; }
            } else if (c1 == 'p') {
                if (c2 == 'N' || c2 == 'n') o.precond = FCG_PRECOND_NONE;
                else if (c2 == 'J' || c2 == 'j') o.precond |= FCG_PRECOND_JACOBI;
                else if (c2 == 'S' || c2 == 's') {
                    if (sscanf(rest3, "%u", &o.super_dim) != 1) { err = "bad preconditioner dimension '" + a + "'"; return true; }
                    o.precond |= 4;
                } else if (c2 == 'B' || c2 == 'b') {
                    if (sscanf(rest3, "%u", &o.block_size) != 1) { err = "bad preconditioner dimension '" + a + "'"; return true; }
                    o.precond |= 2;
                } else if (c2 == 'H' || c2 == 'h') {
                    o.precond |= 8;
                } else { err = "bad preconditioner type '" + a + "'"; return true; }
            } else if (c1 == 'c') o.out_charge = true;
            else if (c1 == 'k') { if (c2 == 'c') o.keep_charge = true; }
            else if (c1 == 'r') o.dump_residual = true;
            else if (c1 == 'i') o.dump_time = true;
            else if (c1 == 'v') o.verbose = true;
            else if (c1 == 't') {
                if (sscanf(rest2, "%lf", &o.gmres_tol) != 1) { err = "bad GMRES iteration tolerance '" + a + "'"; return true; }
            } else if (c1 == 'o') { if (c2 == 'i') o.dump_input = true; else o.out_geo = true; }
            else if (c1 == 'e') o.out_cap = true;
            else if (c1 == 'g') o.galerkin = true;
            else if (c1 == 'a') {
                if (c2 == 'p' || c2 == 'P') o.auto_precond = true;
                else {
                    o.automatic = true;
                    if (sscanf(rest2, "%lf", &o.auto_err) != 1) { err = "bad max error value for auto option '" + a + "'"; return true; }
                }
            } else if (c1 == 'x') {
                // -x64 / -xm: arithmetic of the GPU link product (this library only)
                if (a == "-x64") o.precision = FCG_PREC_FP64;
                else if (a == "-xm") o.precision = FCG_PREC_MIXED;
                else { err = "illegal option -- '" + a.substr(1) + "'"; return true; }
            } else if (c1 != 'b') { err = "illegal option -- '" + a.substr(1) + "'"; return true; }
        } else {
            o.file = a;
        }
    }
    return false;
}

}  // namespace

// One build + fill + solve at a given refinement, printing the reference's
// report blocks; the C matrix and the model counts are returned.
struct SolveRun {
    std::vector<double> cap;
    std::vector<int> iters;
    std::vector<double> charges;  // -c: every conductor's panel charges, [conductor][panel]
    fcg_model_info info;
    int nc = 0;
    double build_s = 0, fill_s = 0, solve_s = 0;
    int64_t device_bytes = 0;
};

// the mesh refinement and the link construction run on the console's GPU,
// and the links stay in device memory for the problem built from them (the
// automatic refinement builds a model per pass: none of them goes through
// host memory and back)
static int build_model_at(fcg_context *ctx, const CmdOptions &o, double mesh_eps, fcg_model **m, fcg_model_info &info) {
    fcg_build_options bo = {mesh_eps, o.eps_ratio, o.mesh_curv, o.verbose ? 1 : 0};
    char ebuf[512] = {0};
    int r = fcg::model_build_device_links(ctx->dev, o.file.c_str(), &bo, m, ebuf, sizeof ebuf);
    if (r != FCG_NORMAL_END) { printf("Error: %s\n", ebuf); return r; }
    fcg_model_info_get(*m, &info);
    return FCG_NORMAL_END;
}

// CSolveCap::AutoSetPrecondType (Solver/SolveCapacitance.cpp:580-608)
static void auto_precond(int64_t links, int cond_num, int &kind, unsigned &dim) {
    long lx = (long)(links / 1000) * cond_num;
    if (lx <= 500) { kind = FCG_PRECOND_JACOBI; return; }
    kind = FCG_PRECOND_TWO_LEVEL;
    dim = lx <= 5000 ? 128 : (lx <= 10000 ? 512 : 1024);
}

static int solve_model(fcg_context *ctx, fcg_model *m, const CmdOptions &o, double gmres_tol, int kind, unsigned dim, SolveRun &out) {
    fcg_model_info &info = out.info;
    fcg_model_info_get(m, &info);
    if (kind == FCG_PRECOND_TWO_LEVEL) printf("Precond Type(s) (-p): Two-levels, dimension %u\n", dim);
    else printf("Precond Type(s) (-p): %s\n", kind == FCG_PRECOND_JACOBI ? "Jacobi" : "None");
    printf("Number of input panels to solver engine: %lld\n", (long long)info.input_panels);
    printf("Number of panels after refinement: %lld\n", (long long)info.n_panels);
    printf("Number of links to be computed: %lld\n", (long long)info.n_links);
    fcg_problem *p = NULL;
    fcg_model_arrays arr;
    fcg_model_arrays_get(m, &arr);
    int r = fcg_problem_create(ctx, &arr, o.precision, &p);
    if (r == FCG_NORMAL_END) r = fcg_problem_fill(p);
    out.nc = info.n_conductors - info.n_dielectrics;
    if (r == FCG_NORMAL_END) {
        out.cap.assign((size_t)out.nc * out.nc, 0.0);
        out.iters.assign(out.nc, 0);
        fcg_solve_options so = {gmres_tol, kind, 0, 0, (int)dim, 0};
        if (o.out_charge) {
            // the charge vectors of every conductor's solve (the reference's
            // m_pCondCharges) for the charge-density files
            out.charges.assign((size_t)out.nc * (size_t)info.n_panels, 0.0);
            r = fcg::problem_solve(p->p, so, out.cap.data(), out.iters.data(), out.charges.data());
        } else {
            r = fcg_problem_solve(p, &so, out.cap.data(), out.iters.data());
        }
    }
    if (r != FCG_NORMAL_END && r != FCG_NOT_CONVERGED) {
        printf("Error: %s\n", fcg_last_error());
        fcg_problem_destroy(p);
        return r;
    }
    if (r == FCG_NOT_CONVERGED) printf("Error: GMRES not converging within the iteration cap\n");
    printf("GMRES iterations per conductor:");
    for (int i = 0; i < out.nc; i++) printf(" %d", out.iters[i]);
    printf("\nCapacitance matrix is:\nDimension %d x %d\n", out.nc, out.nc);
    int row = 0;
    for (int32_t c = 0; c < info.n_conductors; c++) {
        if (arr.cond_is_diel[c]) continue;
        printf("%s  ", fcg_model_conductor_name(m, c));
        for (int j = 0; j < out.nc; j++) printf("%g ", out.cap[(size_t)row * out.nc + j]);
        printf("\n");
        row++;
    }
    for (int i = 0; i < out.nc; i++)
        for (int j = 0; j < out.nc; j++)
            if (i != j && out.cap[(size_t)i * out.nc + j] >= 0.0)
                printf("Warning: capacitance matrix has a non-negative off-diagonal element at row %d col %d\n", i + 1, j + 1);
    fcg_problem_stats st;
    fcg_problem_get_stats(p, &st);
    out.fill_s = st.fill_ms / 1000.0;
    out.solve_s = st.solve_ms / 1000.0;
    out.device_bytes = fcg_problem_device_bytes(p);
    fcg_problem_destroy(p);
    return FCG_NORMAL_END;
}

static void print_stats(const CmdOptions &o, const SolveRun &run) {
    printf("\nSolve statistics:\n");
    printf("Number of panels after refinement: %lld\n", (long long)run.info.n_panels);
    printf("Number of links: %lld\n", (long long)(run.info.n_links + run.info.n_panels));
    printf("Max recursion level: %d\n", run.info.max_level);
    printf("Max Mesh relative refinement value: %g\n", run.info.max_mesh_eps);
    if (o.dump_time) {
        printf("Time for building the model (host): %fs\n", run.build_s);
        printf("Time for building potential matrix (GPU): %fs\n", run.fill_s);
        printf("Time for gmres solving (GPU): %fs\n", run.solve_s);
        printf("Device memory for the problem: %lld bytes\n", (long long)run.device_bytes);
    }
}

// CSolveCap::OutputCapMtxToFile (Solver/SolveCapacitance.cpp:835-911): the
// matrix as <input without extension>.csv
static void write_csv(const CmdOptions &o, const SolveRun &run) {
    std::string name = o.file;
    size_t dot = name.rfind('.');
    if (dot != std::string::npos) name.resize(dot);
    name += ".csv";
    FILE *f = fopen(name.c_str(), "w");
    if (!f) { printf("Warning: cannot open \"%s\" for writing, skipping\n", name.c_str()); return; }
    printf("Generating capacitance matrix file \"%s\"\n", name.c_str());
    for (int i = 0; i < run.nc; i++) {
        for (int j = 0; j < run.nc; j++) {
            fprintf(f, "%g", run.cap[(size_t)i * run.nc + j]);
            if (j < run.nc - 1) fprintf(f, ", ");
        }
        fprintf(f, "\n");
    }
    fclose(f);
}

// CAutoRefine::OutputFastCapFile / OutputPanelFile / OutputPanel
// (Solver/Autorefine.cpp:1230-1565): a list file <input without
// extension>_<suffix>.lst naming one panel file per conductor surface
// (conductors: one per distinct outer permittivity, dielectric interfaces:
// one), each holding the conductor's refined panels in leaf order; with
// charges, every panel line ends with its charge density (charge / area).
// Names, line formats and the path handling (only a backslash separates a
// directory in the list file's names) follow the reference, so the files
// read back as FastCap input.
// node type bits (include/fastercap_gb300.h): outer permittivity on the
// normal's side; the side given by the panel's own reference point
static const uint8_t kOutpermNormalDir = 4, kOutpermElementLevel = 8;

static void write_panel_file(const fcg::Model &M, size_t c, int diel_index, const std::string &name, const std::string &filein,
                             const std::string &fileout, const double *charges) {
    FILE *f = fopen(name.c_str(), "w");
    if (!f) {
        printf("  Warning: cannot open \"%s\" for writing, skipping\n", name.c_str());
        return;
    }
    fprintf(f, "0 Refined FastCap file derived from %s, referenced in list file %s\n", filein.c_str(), fileout.c_str());
    fprintf(f, "*\n");
    const fcg::Conductor &C = M.conductors[c];
    const int64_t first = M.cond_leaf_first[c];
    for (int64_t j = first; j < first + C.leaf_count; j++) {
        if (diel_index >= 0 && M.leaf_diel[(size_t)j] != diel_index) continue;
        const size_t n = (size_t)M.leaf_node[(size_t)j];
        const float *v = &M.vert[n * 9];
        fprintf(f, "T %s  %g %g %g  %g %g %g  %g %g %g", C.name.c_str(), v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8]);
        const uint8_t t = M.type[n];
        if (t & kOutpermElementLevel) {
            // the panel's local dielectric reference point: centroid + the
            // unit normal toward the outer permittivity
            double nx = M.norm[n * 3], ny = M.norm[n * 3 + 1], nz = M.norm[n * 3 + 2];
            if (!(t & kOutpermNormalDir)) { nx = -nx; ny = -ny; nz = -nz; }
            fprintf(f, "  %g %g %g", (double)M.cent[n * 3] + nx, (double)M.cent[n * 3 + 1] + ny, (double)M.cent[n * 3 + 2] + nz);
        }
        if (charges) fprintf(f, "  %e\n", charges[j] / M.area[n]);
        else fprintf(f, "\n");
    }
    fclose(f);
}

static void write_fastcap_files(const fcg::Model &M, const std::string &path, const std::string &suffix, const double *charges) {
    // the reference runs in the input's directory: the files go there and
    // name the input by its bare file name
    std::string dir, filein = path;
    size_t sl = filein.rfind('/');
    if (sl != std::string::npos) {
        dir = filein.substr(0, sl + 1);
        filein = filein.substr(sl + 1);
    }
    std::string base = filein;
    size_t pos = base.rfind('.');
    if (pos != std::string::npos) base.resize(pos);
    const std::string fileout = base + "_" + suffix + ".lst";
    FILE *f = fopen((dir + fileout).c_str(), "w");
    if (!f) {
        printf("  Warning: cannot open \"%s\" for writing, skipping\n", fileout.c_str());
        return;
    }
    printf("  generating list file \"%s\"\n", fileout.c_str());
    fprintf(f, "* Refined FastCap file derived from %s\n", filein.c_str());
    fprintf(f, "*\n");
    fprintf(f, "* Total number of panels %lu\n", (unsigned long)M.n_panels);
    fprintf(f, "*\n");
    for (size_t c = 0; c < M.conductors.size(); c++) {
        const fcg::Conductor &C = M.conductors[c];
        std::string cname = base + "_" + C.name + "_" + suffix, nopath = cname;
        size_t bs = cname.rfind('\\');
        if (bs != std::string::npos) nopath = cname.substr(bs + 1);
        if (!C.is_diel) {
            const size_t ns = C.surf_outperm.size();
            for (size_t i = 0; i < ns; i++) {
                const std::string ext = "_" + std::to_string(i) + ".txt";
                fprintf(f, "C %s  %g  0.0 0.0 0.0%s\n", (nopath + ext).c_str(), C.surf_outperm[i], i + 1 == ns ? "" : " +");
                write_panel_file(M, c, (int)i, dir + cname + ext, filein, fileout, charges);
            }
        } else {
            fprintf(f, "D %s  %g %g  0.0 0.0 0.0  %g %g %g\n", (nopath + ".txt").c_str(), C.outperm, C.inperm, C.ref[0], C.ref[1],
                    C.ref[2]);
            write_panel_file(M, c, -1, dir + cname + ".txt", filein, fileout, charges);
        }
    }
    fclose(f);
}

static double fnorm(const std::vector<double> &a) {
    double s = 0.0;
    for (double v : a) s += v * v;
    return sqrt(s);
}

static int run_command_line_impl(const char *command_line) {
    CmdOptions o;
    std::string err;
    if (!command_line || parse_cmd(command_line, o, err)) {
        printf("%s\n", err.c_str());
        printf("Usage: fastercap_gb300 <input file> [-a<max err>] [-ap] [-m<mesh>] [-mc<mesh curvature>] [-t<tolerance>]\n");
        printf("                       [-d<interaction coeff>] [-pj|-pn|-ps<dim>] [-e] [-i] [-v] [-x64|-xm]\n");
        return FCG_COMMAND_LINE_ERROR;
    }
    if (o.galerkin) { printf("Error: the Galerkin scheme (-g) is not supported by the GPU solver\n"); return FCG_COMMAND_LINE_ERROR; }
    // the input-geometry dump and the kept global charges (-oi, -kc) are not
    // written by this solver: refuse the switches rather than drop the files
    if (o.dump_input || o.keep_charge) {
        printf("Error: the input-geometry dump and kept-charge files (-oi, -kc) are not written by the GPU solver\n");
        return FCG_COMMAND_LINE_ERROR;
    }
    if (o.precond & (2 | 8)) {
        printf("Error: the block (-pb) and hierarchical (-ph) preconditioners are not supported by the GPU solver\n");
        return FCG_COMMAND_LINE_ERROR;
    }
    // CSolveCap::Run's option checks (Solver/SolveCapacitance.cpp:122-147)
    if ((o.precond & 4) && (o.precond & FCG_PRECOND_JACOBI)) {
        o.precond = 4;
        printf("Warning: both two-levels preconditioner and Jacobi preconditioner specified, keeping only the two-levels preconditioner\n");
    }
    if (o.precond & 4) {
        if (o.super_dim > 4096) {
            o.super_dim = 4096;
            printf("Warning: maximum two-levels preconditioner dimension is 4096, using 4096\n");
        } else if (o.super_dim < 16) {
            o.super_dim = 16;
            printf("Warning: minimum two-levels preconditioner dimension is 16, using 16\n");
        }
    }
    int kind = (o.precond & 4) ? FCG_PRECOND_TWO_LEVEL : (o.precond & FCG_PRECOND_JACOBI) ? FCG_PRECOND_JACOBI : FCG_PRECOND_NONE;
    unsigned dim = o.super_dim;
    printf("Running fastercap_gb300 (GB300 solve path for FasterCap input files)\n");
    printf("Input file: %s\n", o.file.c_str());
    auto t0 = std::chrono::steady_clock::now();
    fcg_context *ctx = NULL;
    fcg_model *m = NULL;
    SolveRun run;
    int r;
    // an unreadable input is reported before the device is touched
    if (FILE *f = fopen(o.file.c_str(), "rb")) {
        fclose(f);
    } else {
        printf("Error: cannot open file '%s'\n", o.file.c_str());
        return FCG_CANNOT_OPEN_FILE;
    }
    if (!o.automatic) {
        // manual settings (CSolveCap::Run, Solver/SolveCapacitance.cpp:479-531)
        r = fcg_context_create(0, &ctx);
        if (r != FCG_NORMAL_END) { printf("Error: %s\n", fcg_last_error()); return r; }
        auto tb = std::chrono::steady_clock::now();
        r = build_model_at(ctx, o, o.mesh_eps, &m, run.info);
        if (r != FCG_NORMAL_END) { fcg_context_destroy(ctx); return r; }
        run.build_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - tb).count();
        printf("Mesh refinement (-m): %g\nGMRES tolerance (-t): %g\n", o.mesh_eps, o.gmres_tol);
        r = solve_model(ctx, m, o, o.gmres_tol, kind, dim, run);
    } else {
        // automatic refinement (CSolveCap::Run auto branch,
        // Solver/SolveCapacitance.cpp:294-477): start unrefined, then divide
        // the mesh parameter by sqrt(2) (from the achieved refinement) until
        // panels and links grow by 10 %, solve, and stop when the relative
        // Frobenius norm of the change of C is within the error
        const double tol = o.auto_err / 2.0;
        printf("Auto calculation with max error: %g\n", o.auto_err);
        printf("GMRES tolerance (-t): %g\n", tol);
        r = fcg_context_create(0, &ctx);
        if (r != FCG_NORMAL_END) { printf("Error: %s\n", fcg_last_error()); return r; }
        printf("\nIteration number #0 ***************************\n\n");
        r = build_model_at(ctx, o, 1e32, &m, run.info);
        if (r == FCG_NORMAL_END) {
            printf("Mesh refinement (-m): %g\n", 1e32);
            if (o.auto_precond) auto_precond(run.info.n_links, (int)(run.info.n_conductors - run.info.n_dielectrics), kind, dim);
            r = solve_model(ctx, m, o, tol, kind, dim, run);
        }
        int64_t old_panels = run.info.n_panels, old_links = run.info.n_links;
        for (int it = 1; r == FCG_NORMAL_END && it < 128; it++) {
            printf("\nIteration number #%d ***************************\n\n", it);
            bool enough = false;
            double meps = 0.0;
            for (int j = 0; !enough && j < 128; j++) {
                meps = run.info.max_mesh_eps / sqrt(2.0);
                fcg_model_free(m);
                m = NULL;
                r = build_model_at(ctx, o, meps, &m, run.info);
                if (r != FCG_NORMAL_END) break;
                enough = run.info.n_links > old_links * 1.1 && run.info.n_panels > old_panels * 1.1;
                if (!enough)
                    printf("Delta in refined panel and link count w.r.t. previous iteration less than 10%%\n(Panels # %lld, Links # %lld)\n",
                           (long long)run.info.n_panels, (long long)run.info.n_links);
            }
            if (r != FCG_NORMAL_END) break;
            printf("Mesh refinement (-m): %g\n", meps);
            if (o.auto_precond) auto_precond(run.info.n_links, (int)(run.info.n_conductors - run.info.n_dielectrics), kind, dim);
            std::vector<double> prev = run.cap;
            r = solve_model(ctx, m, o, tol, kind, dim, run);
            if (r != FCG_NORMAL_END) break;
            std::vector<double> d(run.cap.size());
            for (size_t q = 0; q < d.size(); q++) d[q] = run.cap[q] - (q < prev.size() ? prev[q] : 0.0);
            double diff = fnorm(d) / fnorm(run.cap);
            printf("Weighted Frobenius norm of the difference between capacitance (auto option): %g\n", diff);
            if (diff <= o.auto_err) break;
            old_panels = run.info.n_panels;
            old_links = run.info.n_links;
        }
    }
    auto t2 = std::chrono::steady_clock::now();
    if (r == FCG_NORMAL_END) {
        print_stats(o, run);
        if (o.out_cap) write_csv(o, run);
        // CSolveCap::Run (Solver/SolveCapacitance.cpp:538-568): charge
        // densities per conductor solve, then the refined geometry
        if (o.out_charge && m) {
            printf("\n");
            const fcg::Model &M = m->m;
            int capnum = 0;
            for (size_t c = 0; c < M.conductors.size() && capnum < run.nc; c++) {
                if (M.conductors[c].is_diel) continue;
                printf("Outputting charge densities for conductor %s..\n", M.conductors[c].name.c_str());
                write_fastcap_files(M, o.file, M.conductors[c].name, run.charges.data() + (size_t)capnum * (size_t)M.n_panels);
                printf("Done\n");
                capnum++;
            }
        }
        if (o.out_geo && m) {
            printf("\nOutputting refined geometry in FastCap compatible format..\n");
            write_fastcap_files(m->m, o.file, "ref", NULL);
            printf("Done\n");
        }
        printf("Total time: %fs\n", std::chrono::duration<double>(t2 - t0).count());
    }
    if (ctx) fcg_context_destroy(ctx);
    if (m) fcg_model_free(m);
    return r;
}

extern "C" int fcg_run_command_line(const char *command_line) {
    int r = run_command_line_impl(command_line);
    fflush(stdout);  // the report is complete when the call returns
    return r;
}
