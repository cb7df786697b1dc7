// Host model builder: FastCap-format input -> panel hierarchy -> adaptive mesh
// -> interaction links -> flattened SoA model.
//
// The steps restate the reference's model construction so that the panel,
// node and link sets (and the order of links inside every node's row) are the
// same as the reference's:
//   parse_file          CAutoRefine::Parse3DInputFile   Solver/Autorefine.cpp:4746-5568
//   create_panel        CAutoRefine::CreatePanel        Solver/Autorefine.cpp:5990-6083
//                       CAutoPanel::CalcPanelGeomPar    Solver/AutoPanel.cpp:51-104
//   get_conductor       CAutoRefine::GetConductor       Solver/Autorefine.cpp:6279-6365
//   build_super         CAutoRefine::BuildSuperHierarchy / RecurBuild3DSuperHier
//                                                       Solver/Autorefine.cpp:6410-6629
//   make_super          CAutoPanel::MakeSuperPanel      Solver/AutoPanel.cpp:209-379
//   subdivide           CAutoPanel::Subdivide           Solver/AutoPanel.cpp:382-523
//   discretize_*        CAutoRefine::DiscretizeMutual/Self Solver/Autorefine.cpp:2638-2795
//   refine_criteria     CAutoRefine::RefineCriteria     Solver/Autorefine.cpp:2928-3003
//   refine_mutual/self  CAutoRefine::RefineMutual/RefineSelf Solver/Autorefine.cpp:3096-3235, 2115-2229
//   flatten             CAutoRefine::RecurseIndex       Solver/Autorefine.cpp:1173-1220
// Elements live in one index-addressed array instead of a pointer tree; the
// links are emitted once as (node, node) pairs in traversal order and bucketed
// by destination with a stable counting sort, which yields the reference's row
// order without its separate counting pass.
//
// Floating-point rules (kept identical everywhere): panel geometry is float; a
// difference or sum of two float vectors is formed in float; an operation that
// meets a double operand, and every modulus / dot / cross product, is done in
// double; a double result stored into panel geometry is rounded to float.
#include "model.hpp"

#include <deque>
#include <errno.h>
#include <map>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <unistd.h>
#include <chrono>
#include <atomic>
#include <thread>

#include "../csrc/fc_potential.h"
#include "../csrc/fcg_internal.hpp"

namespace fcg {
namespace {

const double kCosMin = 0.99619469809174553229501040247389;  // 5 degrees
const double kQuadSideTol = 0.2;
const double kQuadAngleTol = 0.1;
const double kRelDielTol = 0.001;
const double k2DivFourthRoot27 = 0.87738267530166164054614593453133;
const double k2DivFourthRoot3 = 1.5196713713031850946623755013091;
const double kMinus05PlusSqr2Div4 = -0.14644660940672623779957781894758;
const double k05PlusSqr2Div4 = 0.85355339059327376220042218105242;
const double kSqr2 = 1.4142135623730950488016887242097;
const int kMaxParseLevel = 128;
const int kMaxDepth = 4096;
const int kMaxLineLen = 512;

struct D3 {
    double x, y, z;
    double &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline D3 d3(double x, double y, double z) { D3 r = {x, y, z}; return r; }
inline D3 widen(const float *v) { return d3(v[0], v[1], v[2]); }
inline D3 fsub(const float *a, const float *b) {
    float x = a[0] - b[0], y = a[1] - b[1], z = a[2] - b[2];
    return d3(x, y, z);
}
inline D3 sub(D3 a, D3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline D3 add(D3 a, D3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline D3 scale(D3 a, double s) { return d3(a.x * s, a.y * s, a.z * s); }
inline D3 divs(D3 a, double s) { return d3(a.x / s, a.y / s, a.z / s); }
inline double mod(D3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 cross(D3 a, D3 b) { return d3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline void store(float *dst, D3 a) { dst[0] = (float)a.x; dst[1] = (float)a.y; dst[2] = (float)a.z; }
inline void normalize(D3 &a) { double m = mod(a); a.x /= m; a.y /= m; a.z /= m; }

// The fields of a 'T' or 'Q' panel line as the reference's sscanf sequence
// reads them (Parse3DInputFile, Solver/Autorefine.cpp:5030-5110): the
// conductor name, the raw vertex coordinates and the optional reference
// point. A pure function of the line's text, so large files are read on all
// host threads before the (sequential) parse.
struct PanelLine {
    bool ok = false;
    std::string name;
    float v[12];
    float ref[3];
    bool uselocal = false;
    // a triangle's element geometry for a zero file offset (pre-read only)
    bool geo = false;
    Element e;
    double cosmin = 0;
};

static inline bool c_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }

// One "%f" conversion as sscanf makes it, for a plain decimal token: C-locale
// whitespace, [+-]digits[.digits][(e|E)[+-]digits] with at least one
// mantissa digit, then whitespace or the end of the text. strtof rounds such
// a token to the nearest float exactly as the %f conversion does (glibc's
// %f hands the same characters to the same conversion). Anything else - hex,
// inf, nan, an exponent without digits, a token glued to other text, a
// value out of float range - returns false, and the caller runs sscanf
// itself. `used` counts the characters consumed from p, as %n would.
static bool scan_plain_float(const char *p, float &x, int &used) {
    const char *s = p;
    while (c_space(*s)) s++;
    const char *t = s;
    if (*t == '+' || *t == '-') t++;
    int digits = 0;
    while (*t >= '0' && *t <= '9') { t++; digits++; }
    if (*t == '.') {
        t++;
        while (*t >= '0' && *t <= '9') { t++; digits++; }
    }
    if (digits == 0) return false;
    if (*t == 'e' || *t == 'E') {
        const char *u = t + 1;
        if (*u == '+' || *u == '-') u++;
        if (!(*u >= '0' && *u <= '9')) return false;
        while (*u >= '0' && *u <= '9') u++;
        t = u;
    }
    if (*t != 0 && !c_space(*t)) return false;
    char *end = NULL;
    errno = 0;
    const float v = strtof(s, &end);
    if (end != t || errno != 0) return false;
    x = v;
    used = (int)(t - p);
    return true;
}

// sscanf(p, "%f%f%f%n", ...) for three plain tokens: true with the values and
// the characters used; false leaves everything to sscanf
static bool scan_plain_float3(const char *p, float &x, float &y, float &z, int &used) {
    int a, b, c;
    if (!scan_plain_float(p, x, a) || !scan_plain_float(p + a, y, b) || !scan_plain_float(p + a + b, z, c)) return false;
    used = a + b + c;
    return true;
}

static void parse_panel_fields(const char *line, PanelLine &o) {
    const int nv = line[0] == 'T' ? 3 : 4;
    char tmpname[kMaxLineLen];
    tmpname[0] = 0;
    int skip = 0;
    const char *point = line + 1;
    {
        // "%s%n": the conductor name (sscanf for a line with none)
        const char *s = point;
        while (c_space(*s)) s++;
        const char *t = s;
        while (*t && !c_space(*t)) t++;
        if (t > s) {
            memcpy(tmpname, s, (size_t)(t - s));
            tmpname[t - s] = 0;
            skip = (int)(t - point);
        } else {
            sscanf(point, "%s%n", tmpname, &skip);
        }
    }
    point += skip;
    for (int i = 0; i < nv; i++) {
        float x = 0, y = 0, z = 0;
        if (!scan_plain_float3(point, x, y, z, skip)) {
            x = y = z = 0;
            sscanf(point, "%f%f%f%n", &x, &y, &z, &skip);
        }
        o.v[3 * i] = x;
        o.v[3 * i + 1] = y;
        o.v[3 * i + 2] = z;
        point += skip;
    }
    float x, y, z;
    const char *rest = point;
    while (c_space(*rest)) rest++;
    if (*rest == 0) o.uselocal = false;  // sscanf would find no input (EOF)
    else if (scan_plain_float3(point, x, y, z, skip)) o.uselocal = true;
    else o.uselocal = sscanf(point, "%f%f%f%n", &x, &y, &z, &skip) == 3;
    if (o.uselocal) { o.ref[0] = x; o.ref[1] = y; o.ref[2] = z; }
    o.name = tmpname;
    o.ok = true;
}

// One physical input file, split the way fgets() with a 512-byte buffer splits
// it; `eof` marks a final chunk without a newline (the reference's read loop
// stops before processing such a chunk).
// fn(0..n-1) on up to 16 host threads (inline when par is false;
// FCG_HOST_THREADS caps the threads, 1 runs everything inline)
static const size_t kParallelNodes = 50000;
template <class F> static void host_parallel(int64_t n, bool par, F fn) {
    int nt = (int)std::min<size_t>(std::max(1u, std::thread::hardware_concurrency()), 16);
    if (const char *ht = getenv("FCG_HOST_THREADS")) nt = std::max(1, std::min(nt, atoi(ht)));
    if (!par || nt <= 1 || n <= 1) {
        for (int64_t i = 0; i < n; i++) fn(i);
        return;
    }
    nt = (int)std::min<int64_t>(nt, n);
    std::atomic<int64_t> next(0);
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++)
        th.emplace_back([&]() {
            for (int64_t i; (i = next.fetch_add(1)) < n;) fn(i);
        });
    for (std::thread &t : th) t.join();
}

struct InFile {
    std::vector<std::string> lines;
    std::vector<bool> eof;
    std::map<std::string, size_t> sub;  // "File <name>" sections -> first line index
    std::vector<PanelLine> panels;      // pre-read panel lines (large files), by line index
};

struct Builder {
    BuildOptions opt;
    std::vector<Element> el;
    std::vector<Conductor> conds;
    std::deque<int> order;  // solver order of conductors
    std::deque<InFile> files;
    int parse_level = -1;
    int group_num[kMaxParseLevel + 2];
    long group_diel_num = 0;
    int64_t input_panels = 0, raw_cond = 0, raw_diel = 0;
    double max_area = 0, max_side = 0, total_area = 0, max_mesh_eps = 0;
    double eps = 0, mesh_eps = 0, mesh_curv = 3.0;
    int level = 0, max_level = 0;
    bool warned_thin = false, warned_skew = false, warned_tri = false;
    std::string err;
    std::vector<std::string> warnings;
    std::vector<std::pair<int32_t, int32_t>> pairs;

    void warn(const std::string &w) {
        warnings.push_back(w);
        if (opt.verbose) fprintf(stderr, "%s\n", w.c_str());
    }

    // ---------------------------------------------------------------- files
    // directory relative names resolve against (the input file's); the
    // process working directory is never changed, so builds may run on
    // several threads at once
    std::string base_dir;

    int load_file(const std::string &name, InFile *&out) {
        std::string full = (!name.empty() && name[0] != '/') ? base_dir + name : name;
        FILE *f = fopen(full.c_str(), "rb");
        if (!f) { err = "cannot open file '" + name + "'"; return FC_CANNOT_OPEN_FILE; }
        files.push_back(InFile());
        InFile &F = files.back();
        char buf[kMaxLineLen];
        while (fgets(buf, kMaxLineLen, f)) {
            F.lines.push_back(buf);
            size_t n = strlen(buf);
            bool nl = n > 0 && buf[n - 1] == '\n';
            F.eof.push_back(!nl && feof(f));
        }
        fclose(f);
        // a large file's panel lines are read on all host threads
        // (FCG_PARSE_THREADS caps the threads; 1 reads them during the parse)
        const size_t kParallelLines = 20000;
        int nt = (int)std::min<size_t>(std::max(1u, std::thread::hardware_concurrency()), 16);
        if (const char *pt = getenv("FCG_PARSE_THREADS")) nt = std::max(1, std::min(nt, atoi(pt)));
        if (F.lines.size() >= kParallelLines && nt > 1) {
            F.panels.resize(F.lines.size());
            std::vector<std::thread> th;
            size_t per = (F.lines.size() + nt - 1) / nt;
            for (int t = 0; t < nt; t++) {
                size_t b = t * per, e = std::min(F.lines.size(), b + per);
                if (b >= e) break;
                th.emplace_back([&F, b, e]() {
                    for (size_t i = b; i < e; i++) {
                        char c = F.lines[i][0];
                        if ((c == 'T' || c == 'Q') && !F.eof[i]) {
                            PanelLine &pl = F.panels[i];
                            parse_panel_fields(F.lines[i].c_str(), pl);
                            if (c == 'T') {
                                // the vertices exactly as a zero offset leaves them
                                for (int k = 0; k < 9; k++) pl.e.v[k] = (float)((double)pl.v[k] + 0.0);
                                pl.cosmin = geom_par(pl.e);
                                pl.geo = true;
                            }
                        }
                    }
                });
            }
            for (auto &x : th) x.join();
        }
        for (size_t i = 0; i < F.lines.size(); i++) {
            if (F.lines[i][0] == 'F') {
                char t1[kMaxLineLen], t2[kMaxLineLen];
                if (sscanf(F.lines[i].c_str(), "%s %s", t1, t2) == 2) F.sub.insert(std::make_pair(std::string(t2), i + 1));
            }
        }
        out = &F;
        return FC_NORMAL_END;
    }

    // ----------------------------------------------------------- conductors
    int find_cond(const std::string &name) {
        for (size_t i = 0; i < order.size(); i++)
            if (conds[order[i]].name == name) return (int)i;
        return -1;
    }

    int get_conductor(const std::string &name, bool isdiel, double outperm, double inperm, const double *ref, uint8_t *diel_index) {
        int pos = find_cond(name);
        int id;
        if (pos < 0) {
            Conductor c;
            c.name = name;
            c.is_diel = isdiel;
            c.outperm = outperm;
            if (isdiel) {
                c.inperm = inperm;
                c.ref[0] = ref[0]; c.ref[1] = ref[1]; c.ref[2] = ref[2];
            }
            conds.push_back(c);
            id = (int)conds.size() - 1;
            if (isdiel) order.push_front(id);
            else order.push_back(id);
        } else {
            id = order[pos];
        }
        if (!isdiel) {
            Conductor &c = conds[id];
            size_t k;
            for (k = 0; k < c.surf_outperm.size(); k++)
                if (c.surf_outperm[k] == outperm) break;
            if (k == c.surf_outperm.size()) {
                if (c.surf_outperm.size() < 255) c.surf_outperm.push_back(outperm);
                else { k--; warn("maximum number of permittivities around conductor " + c.name + " reached"); }
            }
            *diel_index = (uint8_t)k;
        }
        return id;
    }

    // -------------------------------------------------------------- panels
    static uint8_t max_side3(Element &e, double l0, double l1, double l2) { return (uint8_t)fcg_max_side3(e, l0, l1, l2); }

    static double newell_normal(const float *v, float *n) { return fcg_newell_normal(v, n); }

    static void centroid3(Element &e) { fcg_centroid3(e); }

    // returns the cosine of the smallest angle
    static double geom_par(Element &e) {
        double sl[3];
        sl[0] = mod(fsub(e.v + 3, e.v + 0));
        sl[1] = mod(fsub(e.v + 6, e.v + 3));
        sl[2] = mod(fsub(e.v + 0, e.v + 6));
        double nm = newell_normal(e.v, e.n);
        e.area = nm / 2.0;
        centroid3(e);
        uint8_t b;
        double l0 = sl[0], l1 = sl[1], l2 = sl[2];
        uint8_t minside;
        if (l0 >= l1 && l0 >= l2) { e.maxside_idx = 0; e.maxside = l0; minside = (l1 >= l2) ? 2 : 1; }
        else if (l1 >= l0 && l1 >= l2) { e.maxside_idx = 1; e.maxside = l1; minside = (l0 >= l2) ? 2 : 0; }
        else { e.maxside_idx = 2; e.maxside = l2; minside = (l0 >= l1) ? 1 : 0; }
        b = minside;
        int a, c;
        if (b == 0) { a = 2; c = 1; }
        else if (b == 1) { a = 0; c = 2; }
        else { a = 1; c = 0; }
        return (sl[a] * sl[a] + sl[c] * sl[c] - sl[b] * sl[b]) / (2.0 * sl[a] * sl[c]);
    }

    // pre: the element's geometry computed ahead from the same vertices
    int create_panel(const float *vtx, int cond, uint8_t diel_index, bool uselocal, const double *localref, bool triangulated,
                     const Element *pre = NULL, double pre_cosmin = 0.0) {
        Element e;
        double cosmin;
        if (pre) {
            e = *pre;
            cosmin = pre_cosmin;
        } else {
            memcpy(e.v, vtx, sizeof(e.v));
            cosmin = geom_par(e);
        }
        Conductor &C = conds[cond];
        if (C.is_diel) {
            const double *ref = uselocal ? localref : C.ref;
            D3 r = d3(ref[0] - (double)e.v[0], ref[1] - (double)e.v[1], ref[2] - (double)e.v[2]);
            float tmpref = (float)dot(r, widen(e.n));
            if (uselocal) e.type |= FCG_OUTPERM_ELEMENT_LEVEL;
            if (tmpref > 0) e.type |= (FCG_IS_DIEL | FCG_OUTPERM_NORMAL_DIR);
            else e.type |= FCG_IS_DIEL;
        } else {
            e.diel = diel_index;
        }
        if (cosmin >= kCosMin && !warned_thin) {
            warned_thin = true;
            warn(std::string("thin triangles (min angle less than 5 degrees) ") +
                 (triangulated ? "created in the triangulation of a quadrilateral panel" : "found in the input file"));
        }
        el.push_back(e);
        input_panels++;
        C.panels.push_back((int32_t)el.size() - 1);
        return FC_NORMAL_END;
    }

    int create_tri(const D3 &a, const D3 &b, const D3 &c, int cond, uint8_t di, bool ul, const double *lr) {
        float v[9];
        store(v, a); store(v + 3, b); store(v + 6, c);
        return create_panel(v, cond, di, ul, lr, true);
    }

    // Quadrilateral handling: plane, planarity test, split into triangles.
    int quad_panel(D3 q[4], int cond, uint8_t di, bool ul, const double *lr) {
        D3 nrm = d3(0, 0, 0), avg = d3(0, 0, 0);
        for (int i = 0; i < 4; i++) {
            int j = (i + 1) % 4;
            nrm.x += (q[i].y - q[j].y) * (q[i].z + q[j].z);
            nrm.y += (q[i].z - q[j].z) * (q[i].x + q[j].x);
            nrm.z += (q[i].x - q[j].x) * (q[i].y + q[j].y);
            avg = add(avg, q[i]);
        }
        double m = mod(nrm);
        nrm = divs(nrm, m);
        avg = divs(avg, 4.0);
        double pd = -dot(nrm, avg);
        bool planar = true;
        for (int i = 0; i < 4; i++) {
            double dist = dot(nrm, q[i]) + pd;
            if (fabs(dist) > FCG_PANEL_EPS) {
                if (!warned_skew) {
                    warned_skew = true;
                    warn("non-planar quadrilateral panels found in the input file; splitting into two triangles along the smaller diagonal");
                }
                if (opt.verbose) { planar = false; break; }
            }
        }
        if (!planar) return split_diag(q, cond, di, ul, lr);

        D3 sides[4];
        double ds[4];
        for (int i = 0; i < 4; i++) { sides[i] = sub(q[(i + 1) % 4], q[i]); ds[i] = mod(sides[i]); }
        double cosangle = dot(sides[0], sides[1]) / (ds[0] * ds[1]);
        if (fabs(ds[2] - ds[0]) < ds[0] * kQuadSideTol && fabs(ds[3] - ds[1]) < ds[1] * kQuadSideTol && fabs(cosangle) < kQuadAngleTol) {
            if (ds[0] < ds[1]) {
                D3 t = q[0]; q[0] = q[1]; q[1] = q[2]; q[2] = q[3]; q[3] = t;
                t = sides[0]; sides[0] = sides[1]; sides[1] = sides[2]; sides[2] = sides[3]; sides[3] = t;
                double tm = ds[0]; ds[0] = ds[1]; ds[1] = ds[2]; ds[2] = ds[3]; ds[3] = tm;
            }
            long numsegs = (long)(ds[0] / (ds[1] * 5.0) + 0.5);
            if (numsegs == 0) numsegs = 1;
            D3 nodes[4];
            nodes[0] = q[0];
            nodes[3] = q[3];
            D3 span01 = divs(sides[0], (double)numsegs);
            D3 span32 = divs(d3(-sides[2].x, -sides[2].y, -sides[2].z), (double)numsegs);
            int ret;
            for (long i = 0; i < numsegs - 1; i++) {
                nodes[1] = add(nodes[0], span01);
                nodes[2] = add(nodes[3], span32);
                if ((ret = create_tri(nodes[0], nodes[1], nodes[2], cond, di, ul, lr)) != FC_NORMAL_END) return ret;
                if ((ret = create_tri(nodes[0], nodes[2], nodes[3], cond, di, ul, lr)) != FC_NORMAL_END) return ret;
                nodes[0] = nodes[1];
                nodes[3] = nodes[2];
            }
            nodes[1] = q[1];
            nodes[2] = q[2];
            if ((ret = create_tri(nodes[0], nodes[1], nodes[2], cond, di, ul, lr)) != FC_NORMAL_END) return ret;
            return create_tri(nodes[0], nodes[2], nodes[3], cond, di, ul, lr);
        }
        // The reference runs a constrained quality Delaunay triangulation here;
        // this builder splits the quadrilateral along its shorter diagonal.
        if (!warned_tri) {
            warned_tri = true;
            warn("quadrilateral far from a rectangle: split along the shorter diagonal (no quality triangulation)");
        }
        return split_diag(q, cond, di, ul, lr);
    }

    int split_diag(D3 q[4], int cond, uint8_t di, bool ul, const double *lr) {
        double diag1 = mod(sub(q[2], q[0])), diag2 = mod(sub(q[3], q[1]));
        int ret;
        if (diag1 <= diag2) {
            if ((ret = create_tri(q[0], q[1], q[2], cond, di, ul, lr)) != FC_NORMAL_END) return ret;
            return create_tri(q[2], q[3], q[0], cond, di, ul, lr);
        }
        if ((ret = create_tri(q[0], q[1], q[3], cond, di, ul, lr)) != FC_NORMAL_END) return ret;
        return create_tri(q[1], q[2], q[3], cond, di, ul, lr);
    }

    // ---------------------------------------------------------------- parser
    // reads a permittivity "re[-jim|+jim]"; complex values are rejected
    bool read_perm(const char *&point, float &re) {
        int skip = 0;
        sscanf(point, "%f%n", &re, &skip);
        point += skip;
        float im;
        if (sscanf(point, " - j %f%n", &im, &skip) == 1 || sscanf(point, " + j %f%n", &im, &skip) == 1) {
            err = "complex permittivities are not supported by this solver";
            return false;
        }
        return true;
    }

    int parse_file(const std::string &fname, InFile *parent, bool isdiel, D3 offset, double outperm,
                   const std::string &groupname, double inperm, D3 dielref) {
        parse_level++;
        if (parse_level >= kMaxParseLevel) { err = "input file nesting too deep"; return FC_FILE_ERROR; }
        InFile *F = NULL;
        size_t li = 0;
        if (parent && parent->sub.count(fname)) {
            F = parent;
            li = parent->sub[fname];
        } else {
            int r = load_file(fname, F);
            if (r != FC_NORMAL_END) return r;
        }
        int ret = FC_NORMAL_END;
        for (; li < F->lines.size(); li++) {
            if (F->eof[li]) break;
            const char *line = F->lines[li].c_str();
            char c0 = line[0];
            if (c0 == 'E' || c0 == 'e' || c0 == 'F' || c0 == 'f') break;
            char name[kMaxLineLen], tmpname[kMaxLineLen];
            int skip = 0;
            if (c0 == 'C') {
                const char *point = line + 1;
                sscanf(point, "%s%n", name, &skip);
                point += skip;
                float perm;
                if (!read_perm(point, perm)) { ret = FC_FILE_ERROR; break; }
                float x = 0, y = 0, z = 0;
                sscanf(point, "%f%f%f%n", &x, &y, &z, &skip);
                D3 loff = add(d3(x, y, z), offset);
                point += skip;
                std::string lgroup = (parse_level == 0) ? std::string("g") : groupname;
                char num[32];
                snprintf(num, sizeof num, "%d_", group_num[parse_level]);
                lgroup += num;
                tmpname[0] = '\0';
                sscanf(point, "%s%n", tmpname, &skip);
                if (tmpname[0] != '+') group_num[parse_level]++;
                group_num[parse_level + 1] = 1;
                InFile *mapsrc = F;
                ret = parse_file(name, mapsrc, false, loff, (double)perm, lgroup, 0.0, d3(0, 0, 0));
                if (ret != FC_NORMAL_END) break;
            } else if (c0 == 'D') {
                const char *point = line + 1;
                sscanf(point, "%s%n", name, &skip);
                point += skip;
                float out, in;
                if (!read_perm(point, out) || !read_perm(point, in)) { ret = FC_FILE_ERROR; break; }
                float x = 0, y = 0, z = 0;
                sscanf(point, "%f%f%f%n", &x, &y, &z, &skip);
                D3 loff = add(d3(x, y, z), offset);
                point += skip;
                sscanf(point, "%f%f%f%n", &x, &y, &z, &skip);
                D3 lref = add(d3(x, y, z), offset);
                point += skip;
                tmpname[0] = '\0';
                sscanf(point, "%s%n", tmpname, &skip);
                if (tmpname[0] == '-') { float t = out; out = in; in = t; }
                bool dummy = (in <= 0.0 || out <= 0.0) || (fabs(in - out) / in < kRelDielTol);
                if (dummy) {
                    warn("dummy dielectric-dielectric interface found in the input file, skipping");
                } else {
                    char g[64];
                    snprintf(g, sizeof g, "diel%ld", group_diel_num);
                    group_diel_num++;
                    ret = parse_file(name, F, true, loff, (double)out, g, (double)in, lref);
                    if (ret != FC_NORMAL_END) break;
                }
            } else if (c0 == 'T' || c0 == 'Q') {
                int nv = (c0 == 'T') ? 3 : 4;
                PanelLine own;
                const PanelLine *pl = (li < F->panels.size() && F->panels[li].ok) ? &F->panels[li] : NULL;
                if (!pl) {
                    parse_panel_fields(line, own);
                    pl = &own;
                }
                float fv[12];
                D3 qv[4];
                for (int i = 0; i < nv; i++) {
                    float x = pl->v[3 * i], y = pl->v[3 * i + 1], z = pl->v[3 * i + 2];
                    if (nv == 3) {
                        fv[3 * i] = (float)((double)x + offset.x);
                        fv[3 * i + 1] = (float)((double)y + offset.y);
                        fv[3 * i + 2] = (float)((double)z + offset.z);
                    } else {
                        qv[i] = add(d3(x, y, z), offset);
                    }
                }
                double lref[3] = {0, 0, 0};
                bool uselocal = pl->uselocal;
                if (uselocal) {
                    lref[0] = (double)pl->ref[0] + offset.x; lref[1] = (double)pl->ref[1] + offset.y; lref[2] = (double)pl->ref[2] + offset.z;
                }
                std::string cname = groupname;
                if (!isdiel) cname += pl->name;
                double refp[3] = {dielref.x, dielref.y, dielref.z};
                if (nv == 4) {
                    // degenerate (collinear) quadrilaterals are skipped before any conductor is created
                    D3 nrm = d3(0, 0, 0);
                    for (int i = 0; i < 4; i++) {
                        int j = (i + 1) % 4;
                        nrm.x += (qv[i].y - qv[j].y) * (qv[i].z + qv[j].z);
                        nrm.y += (qv[i].z - qv[j].z) * (qv[i].x + qv[j].x);
                        nrm.z += (qv[i].x - qv[j].x) * (qv[i].y + qv[j].y);
                    }
                    if (mod(nrm) < 1e-300) {
                        warn("degenerate quadrilateral panel 'Q' found (co-linear vertexes), skipping");
                        if (isdiel) raw_diel++; else raw_cond++;
                        continue;
                    }
                }
                uint8_t di = 0;
                int cond = get_conductor(cname, isdiel, outperm, inperm, refp, &di);
                const bool zero_off = offset.x == 0.0 && offset.y == 0.0 && offset.z == 0.0;
                if (nv == 3) ret = create_panel(fv, cond, di, uselocal, lref, false, (pl->geo && zero_off) ? &pl->e : NULL, pl->cosmin);
                else ret = quad_panel(qv, cond, di, uselocal, lref);
                if (ret != FC_NORMAL_END) break;
                if (isdiel) raw_diel++; else raw_cond++;
            } else if (c0 == 'N') {
                if (!isdiel) {
                    const char *point = line + 1;
                    char condname[kMaxLineLen];
                    sscanf(point, "%s%n", condname, &skip);
                    point += skip;
                    sscanf(point, "%s%n", tmpname, &skip);
                    std::string oldn = groupname + condname, newn = groupname + tmpname;
                    if (oldn != newn) {
                        int po = find_cond(oldn);
                        if (po >= 0) {
                            int pn = find_cond(newn);
                            if (pn >= 0) {
                                // merge the old conductor's panels into the new one
                                int ido = order[po], idn = order[pn];
                                conds[idn].panels.insert(conds[idn].panels.end(), conds[ido].panels.begin(), conds[ido].panels.end());
                                order.erase(order.begin() + po);
                            } else {
                                conds[order[po]].name = newn;
                            }
                        }
                    }
                }
            }
        }
        parse_level--;
        return ret;
    }

    // ------------------------------------------------------ super hierarchy
    D3 geo_normal(int id) {
        fcg_d3 n = fcg_geo_normal(el[id]);
        return d3(n.x, n.y, n.z);
    }

    int make_super(int lid, int rid) {
        const bool ld = el[lid].type & FCG_IS_DIEL, rd = el[rid].type & FCG_IS_DIEL;
        if (ld != rd) warn("internal: dielectric sub-panels not coherent in type");
        Element e;
        fcg_make_super(el[lid], el[rid], lid, rid, e);
        el.push_back(e);
        return (int)el.size() - 1;
    }

    struct BBox {
        D3 mn, mx;
        bool empty = true;
        void add(const float *p) {
            D3 q = widen(p);
            if (empty) { mn = q; mx = q; empty = false; return; }
            for (int i = 0; i < 3; i++) {
                if (q[i] < mn[i]) mn[i] = q[i];
                if (q[i] > mx[i]) mx[i] = q[i];
            }
        }
        int max_side() const {
            double dx = mx.x - mn.x, dy = mx.y - mn.y, dz = mx.z - mn.z;
            if (dx >= dy && dx >= dz) return 0;
            if (dy >= dz) return 1;
            return 2;
        }
    };

    std::vector<int32_t> arr1, arr2;

    int rec_super(size_t first, size_t n, const BBox &bb, int depth) {
        if (n == 1) return arr1[first];
        if (depth > kMaxDepth) { err = "super hierarchy too deep (coincident panel centroids?)"; return -1; }
        int mc = bb.max_side();
        double mid = (bb.mx[mc] + bb.mn[mc]) / 2.0;
        size_t lo = first, hi = first + n - 1;
        for (size_t i = first; i < first + n; i++) {
            if ((double)el[arr1[i]].c[mc] <= mid) arr2[lo++] = arr1[i];
            else arr2[hi--] = arr1[i];
        }
        if (lo == first || lo == first + n) {
            err = "panels with coincident centroids cannot be split into a hierarchy";
            return -1;
        }
        BBox lb, rb;
        for (size_t i = first; i < lo; i++) { arr1[i] = arr2[i]; lb.add(el[arr1[i]].c); }
        for (size_t i = lo; i < first + n; i++) { arr1[i] = arr2[i]; rb.add(el[arr1[i]].c); }
        int l = rec_super(first, lo - first, lb, depth + 1);
        if (l < 0) return -1;
        int r = rec_super(lo, first + n - lo, rb, depth + 1);
        if (r < 0) return -1;
        return make_super(l, r);
    }

    // panel sets of at least this size build their super hierarchy on the
    // device when there is one (the same tree and elements)
    static const size_t kDeviceSuperPanels = 20000;

    int build_super(DeviceContext *dev) {
        max_area = max_side = total_area = 0.0;
        size_t total = 0;
        for (size_t k = 0; k < order.size(); k++) total += conds[order[k]].panels.size();
        if (dev && total >= kDeviceSuperPanels) {
            std::vector<std::vector<int32_t>> sets(order.size());
            for (size_t k = 0; k < order.size(); k++) {
                Conductor &C = conds[order[k]];
                if (C.panels.empty()) { err = "conductor " + C.name + " has no panels"; return FC_FILE_ERROR; }
                sets[k] = C.panels;
            }
            std::vector<int32_t> tops;
            int r = super_build_device(*dev, el, sets, tops, kMaxDepth, err);
            if (r != FC_NORMAL_END) return r;
            for (size_t k = 0; k < order.size(); k++) {
                Conductor &C = conds[order[k]];
                C.top = tops[k];
                if (el[C.top].maxside > max_side) max_side = el[C.top].maxside;
                if (el[C.top].area > max_area) max_area = el[C.top].area;
                total_area += el[C.top].area;
            }
            return FC_NORMAL_END;
        }
        for (size_t k = 0; k < order.size(); k++) {
            Conductor &C = conds[order[k]];
            if (C.panels.empty()) { err = "conductor " + C.name + " has no panels"; return FC_FILE_ERROR; }
            BBox bb;
            arr1.assign(C.panels.begin(), C.panels.end());
            arr2.assign(C.panels.size(), 0);
            for (size_t i = 0; i < arr1.size(); i++) bb.add(el[arr1[i]].c);
            int top = rec_super(0, arr1.size(), bb, 0);
            if (top < 0) return FC_FILE_ERROR;
            C.top = top;
            if (el[top].maxside > max_side) max_side = el[top].maxside;
            if (el[top].area > max_area) max_area = el[top].area;
            total_area += el[top].area;
        }
        return FC_NORMAL_END;
    }

    // ------------------------------------------------------------ refinement
    int subdivide(int id) {
        if (!(el[id].type & FCG_IS_LEAF)) return FC_NORMAL_END;
        Element Lc, Rc;
        fcg_subdivide(el[id], Lc, Rc);
        el.push_back(Lc);
        el.push_back(Rc);
        int l = (int)el.size() - 2, r = (int)el.size() - 1;
        el[id].left = l;
        el[id].right = r;
        el[id].type &= ~FCG_IS_LEAF;
        return FC_NORMAL_END;
    }

    bool refine_criteria(double *c1, double *c2, int p1, int p2, D3 dist, double rdist, double rmax, double e, double ccoeff) {
        return fcg_refine_criteria(el[p1], el[p2], fcg_mk(dist.x, dist.y, dist.z), rdist, rmax, e, ccoeff, max_side, max_area, c1, c2);
    }

    int discretize_mutual(int p1, int p2, bool selfc) {
        level++;
        if (level > max_level) max_level = level;
        if (level > kMaxDepth) { err = "mesh refinement recursion too deep (touching or overlapping panels?)"; return FC_GENERIC_ERROR; }
        double c1, c2;
        int ret = FC_NORMAL_END;
        int which = fcg_mesh_decision(el[p1], el[p2], selfc, mesh_eps, mesh_curv, max_side, max_area, &c1, &c2);
        if (which == 1) {
            subdivide(p1);
            if ((ret = discretize_mutual(el[p1].left, p2, selfc)) == FC_NORMAL_END) ret = discretize_mutual(el[p1].right, p2, selfc);
        } else if (which == 2) {
            subdivide(p2);
            if ((ret = discretize_mutual(p1, el[p2].left, selfc)) == FC_NORMAL_END) ret = discretize_mutual(p1, el[p2].right, selfc);
        } else {
            if (!(el[p1].type & FCG_IS_SUPER_NODE) && c1 > max_mesh_eps) max_mesh_eps = c1;
            if (!(el[p2].type & FCG_IS_SUPER_NODE) && c2 > max_mesh_eps) max_mesh_eps = c2;
        }
        level--;
        return ret;
    }

    int discretize_self(int id, int64_t &panels, int64_t &nodes) {
        level++;
        if (level > max_level) max_level = level;
        int ret = FC_NORMAL_END;
        if ((el[id].type & FCG_IS_LEAF) && level == 1) subdivide(id);
        if (!(el[id].type & FCG_IS_LEAF)) {
            int l = el[id].left, r = el[id].right;
            if ((ret = discretize_mutual(l, r, true)) != FC_NORMAL_END) return ret;
            if ((ret = discretize_self(l, panels, nodes)) != FC_NORMAL_END) return ret;
            if ((ret = discretize_self(r, panels, nodes)) != FC_NORMAL_END) return ret;
        } else {
            panels++;
        }
        nodes++;
        level--;
        return ret;
    }

    void refine_mutual(int p1, int p2) {
        level++;
        if (level > max_level) max_level = level;
        int which = fcg_link_decision(el[p1], el[p2], eps, max_side, max_area);
        if (which == 1) { refine_mutual(el[p1].left, p2); refine_mutual(el[p1].right, p2); }
        else if (which == 2) { refine_mutual(p1, el[p2].left); refine_mutual(p1, el[p2].right); }
        else pairs.push_back(std::make_pair(p1, p2));
        level--;
    }

    void refine_self(int id) {
        level++;
        if (level > max_level) max_level = level;
        if (!(el[id].type & FCG_IS_LEAF)) {
            refine_mutual(el[id].left, el[id].right);
            refine_self(el[id].left);
            refine_self(el[id].right);
        }
        level--;
    }

    // ---------------------------------------------------------------- device mesh
    // The refinement closure runs on the device (mesh_refine_device) from the
    // host order's root pairs: every conductor pair at level 1, then the
    // children pair of every internal element at its depth + 2, flagged as
    // self pairs. A conductor that is a single panel is bisected first, as the
    // host self pass does at its top level.
    int device_mesh(DeviceContext &dev) {
        for (size_t i = 0; i < order.size(); i++) {
            int32_t t = conds[order[i]].top;
            if (el[t].type & FCG_IS_LEAF) subdivide(t);
        }
        std::vector<int32_t> depth(el.size(), 0), ra, rb;
        std::vector<uint16_t> rm;
        for (size_t i = 0; i < order.size(); i++)
            for (size_t j = i + 1; j < order.size(); j++) {
                ra.push_back(conds[order[i]].top);
                rb.push_back(conds[order[j]].top);
                rm.push_back(1);
            }
        std::vector<std::pair<int32_t, int>> st;
        for (size_t i = 0; i < order.size(); i++) {
            st.push_back(std::make_pair(conds[order[i]].top, 0));
            while (!st.empty()) {
                int32_t id = st.back().first;
                int s = st.back().second;
                st.pop_back();
                depth[id] = s;
                if (el[id].type & FCG_IS_LEAF) continue;
                ra.push_back(el[id].left);
                rb.push_back(el[id].right);
                rm.push_back((uint16_t)(kMeshSelfPair | std::min(s + 2, 0x7fff)));
                st.push_back(std::make_pair(el[id].right, s + 1));
                st.push_back(std::make_pair(el[id].left, s + 1));
            }
        }
        double meps = 0.0;
        int lvl = 0;
        int r = mesh_refine_device(dev, el, depth, ra, rb, rm, mesh_eps, mesh_curv, max_side, max_area, meps, lvl, err);
        if (r != FC_NORMAL_END) return r;
        if (meps > max_mesh_eps) max_mesh_eps = meps;
        if (lvl > max_level) max_level = lvl;
        return FC_NORMAL_END;
    }

    // ---------------------------------------------------------------- device links
    // The root pairs of the link traversal in the host order (per conductor:
    // its mutual pairs with the later conductors, then the self pairs of its
    // internal elements in pre-order), each with the recursion level at which
    // refine_mutual visits it; the traversal itself runs on the device
    // (link_build_device) and yields the same rows as the host traversal.
    int device_links(Model &M, const std::vector<int32_t> &node_of, DeviceContext &dev) {
        std::vector<int32_t> ra, rb;
        std::vector<uint16_t> rl;
        int self_level = 0;
        std::vector<std::pair<int32_t, int>> st;
        for (size_t i = 0; i < order.size(); i++) {
            int32_t ti = conds[order[i]].top;
            for (size_t j = i + 1; j < order.size(); j++) {
                ra.push_back(ti);
                rb.push_back(conds[order[j]].top);
                rl.push_back(1);
            }
            st.push_back(std::make_pair(ti, 0));
            while (!st.empty()) {
                int32_t id = st.back().first;
                int s = st.back().second;
                st.pop_back();
                if (s + 1 > self_level) self_level = s + 1;  // refine_self's own level
                if (el[id].type & FCG_IS_LEAF) continue;
                if (s + 2 > 0xffff) { err = "element hierarchy too deep for the device link construction"; return FC_GENERIC_ERROR; }
                ra.push_back(el[id].left);
                rb.push_back(el[id].right);
                rl.push_back((uint16_t)(s + 2));
                st.push_back(std::make_pair(el[id].right, s + 1));
                st.push_back(std::make_pair(el[id].left, s + 1));
            }
        }
        int lvl = 0;
        int r = link_build_device(dev, el.data(), (int64_t)el.size(), ra.data(), rb.data(), rl.data(), (int64_t)ra.size(),
                                  node_of.data(), M.n_nodes, eps, max_side, max_area, M.link_ptr, M.link_src, lvl, err,
                                  opt.links_on_device ? &M.d_link_src : nullptr);
        if (r != FC_NORMAL_END) return r;
        M.n_links = M.link_ptr[(size_t)M.n_nodes];
        if (self_level > max_level) max_level = self_level;
        if (lvl > max_level) max_level = lvl;
        return FC_NORMAL_END;
    }

    // ---------------------------------------------------------------- flatten
    // The conductors' trees are walked in post-order side by side (each
    // conductor's nodes and leaves are one contiguous range, placed by prefix
    // sums), then the node arrays are written in parallel: the same arrays as
    // one sequential walk over the conductors in solver order.
    int flatten(Model &M, DeviceContext *dev) {
        const auto t_flat = std::chrono::steady_clock::now();
        size_t ne = el.size();
        const size_t nc = order.size();
        std::vector<std::vector<int32_t>> cpost(nc);
        std::vector<int64_t> cleaves(nc, 0);
        host_parallel((int64_t)nc, ne >= kParallelNodes, [&](int64_t k) {
            std::vector<int32_t> &out = cpost[(size_t)k];
            // iterative post-order traversal
            std::vector<std::pair<int32_t, int>> st;
            st.push_back(std::make_pair(conds[order[(size_t)k]].top, 0));
            while (!st.empty()) {
                std::pair<int32_t, int> &t = st.back();
                int32_t id = t.first;
                if (el[id].type & FCG_IS_LEAF) {
                    cleaves[(size_t)k]++;
                    out.push_back(id);
                    st.pop_back();
                } else if (t.second == 0) {
                    t.second = 1;
                    st.push_back(std::make_pair(el[id].left, 0));
                } else if (t.second == 1) {
                    t.second = 2;
                    st.push_back(std::make_pair(el[id].right, 0));
                } else {
                    out.push_back(id);
                    st.pop_back();
                }
            }
        });
        std::vector<int64_t> node_off(nc + 1, 0), leaf_off(nc + 1, 0);
        for (size_t k = 0; k < nc; k++) {
            node_off[k + 1] = node_off[k] + (int64_t)cpost[k].size();
            leaf_off[k + 1] = leaf_off[k] + cleaves[k];
        }
        M.conductors.clear();
        M.cond_leaf_first.clear();
        for (size_t k = 0; k < nc; k++) {
            Conductor &C = conds[order[k]];
            C.leaf_count = cleaves[k];
            M.cond_leaf_first.push_back(leaf_off[k]);
            M.conductors.push_back(C);
        }
        int64_t Nn = node_off[nc], Np = leaf_off[nc], L = 2 * (int64_t)pairs.size();
        if (L > 0x7fffffffLL || Nn > 0x7fffffffLL) { err = "model too large for 32-bit link indices"; return FC_OUT_OF_MEMORY; }
        std::vector<int32_t> node_of(ne, -1), post((size_t)Nn), cond_of((size_t)Nn);
        std::vector<int64_t> leaf_first_of(ne, 0), leaf_count_of(ne, 0);
        host_parallel((int64_t)nc, ne >= kParallelNodes, [&](int64_t k) {
            int64_t n0 = node_off[(size_t)k], leaf = leaf_off[(size_t)k];
            const std::vector<int32_t> &cp = cpost[(size_t)k];
            for (size_t t = 0; t < cp.size(); t++) {
                const int32_t id = cp[t];
                post[(size_t)n0 + t] = id;
                node_of[id] = (int32_t)(n0 + (int64_t)t);
                cond_of[(size_t)n0 + t] = (int32_t)k;
                if (el[id].type & FCG_IS_LEAF) {
                    leaf_first_of[id] = leaf++;
                    leaf_count_of[id] = 1;
                } else {  // post-order: both children are done
                    leaf_first_of[id] = leaf_first_of[el[id].left];
                    leaf_count_of[id] = leaf_count_of[el[id].left] + leaf_count_of[el[id].right];
                }
            }
        });
        M.n_nodes = Nn; M.n_panels = Np; M.n_links = L;
        M.type.resize(Nn); M.left.resize(Nn); M.right.resize(Nn); M.cond.resize(Nn);
        M.leaf_first.resize(Nn); M.leaf_count.resize(Nn); M.link_ptr.assign(Nn + 1, 0);
        M.vert.resize(Nn * 9); M.cent.resize(Nn * 3); M.norm.resize(Nn * 3);
        M.area.resize(Nn); M.maxside.resize(Nn); M.maxside_idx.resize(Nn);
        M.leaf_node.resize(Np); M.leaf_diel.resize(Np);
        const int64_t kChunk = 4096;
        host_parallel((Nn + kChunk - 1) / kChunk, Nn >= (int64_t)kParallelNodes, [&](int64_t c) {
            for (int64_t i = c * kChunk; i < std::min(Nn, (c + 1) * kChunk); i++) {
                const Element &e = el[post[i]];
                M.cond[i] = cond_of[i];
                M.type[i] = e.type;
                M.left[i] = e.left >= 0 ? node_of[e.left] : -1;
                M.right[i] = e.right >= 0 ? node_of[e.right] : -1;
                M.leaf_first[i] = leaf_first_of[post[i]];
                M.leaf_count[i] = leaf_count_of[post[i]];
                memcpy(&M.vert[i * 9], e.v, 36);
                memcpy(&M.cent[i * 3], e.c, 12);
                memcpy(&M.norm[i * 3], e.n, 12);
                M.area[i] = e.area;
                M.maxside[i] = e.maxside;
                M.maxside_idx[i] = e.maxside_idx;
                if (e.type & FCG_IS_LEAF) {
                    M.leaf_node[M.leaf_first[i]] = (int32_t)i;
                    M.leaf_diel[M.leaf_first[i]] = (e.type & FCG_IS_DIEL) ? 0 : e.diel;
                }
            }
        });
        if (dev) {
            if (getenv("FCG_TRACE"))
                fprintf(stderr, "[fcg build]   flatten on the host %9.3f ms\n",
                        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_flat).count());
            return device_links(M, node_of, *dev);
        }
        // links: stable counting sort of the emitted pairs by destination node
        std::vector<int64_t> cnt(Nn + 1, 0);
        for (size_t k = 0; k < pairs.size(); k++) { cnt[node_of[pairs[k].first]]++; cnt[node_of[pairs[k].second]]++; }
        for (int64_t i = 0; i < Nn; i++) M.link_ptr[i + 1] = M.link_ptr[i] + cnt[i];
        std::vector<int64_t> fill(M.link_ptr.begin(), M.link_ptr.end() - 1);
        M.link_src.resize(L);
        for (size_t k = 0; k < pairs.size(); k++) {
            int32_t a = node_of[pairs[k].first], b = node_of[pairs[k].second];
            M.link_src[fill[a]++] = b;
            M.link_src[fill[b]++] = a;
        }
        std::vector<std::pair<int32_t, int32_t>>().swap(pairs);
        return FC_NORMAL_END;
    }
};

}  // namespace

int build_model(const std::string &path, const BuildOptions &opt, Model &M, std::string &err, DeviceContext *dev) {
    Builder B;
    B.opt = opt;
    for (int i = 0; i < kMaxParseLevel + 2; i++) B.group_num[i] = 1;
    B.mesh_eps = opt.mesh_eps;
    B.eps = opt.eps_ratio * opt.mesh_eps;
    if (B.eps == 0.0) B.eps = 0.01;
    B.mesh_curv = opt.mesh_curv < 1.0 ? 1.0 : opt.mesh_curv;

    // sub-file names and external files resolve relative to the input's directory
    std::string dir, base = path;
    size_t slash = path.rfind('/');
    if (slash != std::string::npos) { dir = path.substr(0, slash + 1); base = path.substr(slash + 1); }
    {
        // the first line (as the first fgets() chunk) decides 2D versus 3D;
        // the parse below reads the file itself
        FILE *f = fopen(path.c_str(), "rb");
        if (!f) { err = "cannot open file '" + path + "'"; return FC_CANNOT_OPEN_FILE; }
        char first[kMaxLineLen];
        const bool have = fgets(first, kMaxLineLen, f) != NULL;
        fclose(f);
        if (have && (strstr(first, "2D") || strstr(first, "2d"))) {
            err = "2D input files are not supported by this solver";
            return FC_FILE_ERROR;
        }
    }
    B.base_dir = dir;
    // FCG_TRACE=1 prints the builder's phases to stderr
    const bool trace = getenv("FCG_TRACE") != NULL;
    auto t_last = std::chrono::steady_clock::now();
    auto mark = [&](const char *what) {
        if (!trace) return;
        auto now = std::chrono::steady_clock::now();
        fprintf(stderr, "[fcg build] %-22s %9.3f ms\n", what, std::chrono::duration<double, std::milli>(now - t_last).count());
        t_last = now;
    };
    int ret = B.parse_file(base, NULL, false, d3(0, 0, 0), 1.0, "", 0.0, d3(0, 0, 0));
    mark("parse");
    if (ret != FC_NORMAL_END) { err = B.err; return ret; }
    if (B.order.empty()) { err = "no panels found in the input file"; return FC_FILE_ERROR; }

    if ((ret = B.build_super(dev)) != FC_NORMAL_END) { err = B.err; return ret; }
    mark("super hierarchy");

    // adaptive mesh: mutual refinement of all conductor pairs, then self
    B.level = 0;
    B.max_level = 0;
    B.max_mesh_eps = 0.0;
    size_t nc = B.order.size();
    if (dev) {
        if ((ret = B.device_mesh(*dev)) != FC_NORMAL_END) { err = B.err; return ret; }
    } else {
        for (size_t i = 0; i < nc; i++)
            for (size_t j = i + 1; j < nc; j++) {
                ret = B.discretize_mutual(B.conds[B.order[i]].top, B.conds[B.order[j]].top, false);
                if (ret != FC_NORMAL_END) { err = B.err; return ret; }
            }
        int64_t panels = 0, nodes = 0;
        for (size_t i = 0; i < nc; i++) {
            B.level = 0;
            ret = B.discretize_self(B.conds[B.order[i]].top, panels, nodes);
            if (ret != FC_NORMAL_END) { err = B.err; return ret; }
        }
    }
    mark("mesh refinement");
    // links: mutual interactions of all conductor pairs, then self, conductor
    // by conductor (on the device, inside flatten, when a context is given)
    if (!dev) {
        for (size_t i = 0; i < nc; i++) {
            for (size_t j = i + 1; j < nc; j++) B.refine_mutual(B.conds[B.order[i]].top, B.conds[B.order[j]].top);
            B.refine_self(B.conds[B.order[i]].top);
        }
        mark("link traversal");
    }
    if ((ret = B.flatten(M, dev)) != FC_NORMAL_END) { err = B.err; return ret; }
    mark("flatten");
    M.input_panels = B.input_panels;
    M.raw_cond_panels = B.raw_cond;
    M.raw_diel_panels = B.raw_diel;
    M.max_mesh_eps = B.max_mesh_eps;
    M.max_area = B.max_area;
    M.max_side = B.max_side;
    M.total_area = B.total_area;
    M.eps = B.eps;
    M.mesh_eps = B.mesh_eps;
    M.max_level = B.max_level;
    M.warnings = B.warnings;
    return FC_NORMAL_END;
}

}  // namespace fcg
