// pf_host.cpp -- host-side driver layer of libpfgpu.so (no device work).
//
// Deck I/O in the text formats of ParaFEM's p121 tools, the structured cube
// generator and its restraint/load sets, equation numbering, and the p121
// job driver that calls the solve layer.  The formats and numbering schemes
// are fixed by the reference decks, so they follow:
//   p12meshgen.f90:118-323 (src/tools/preprocessing/p12meshgen) .mg -> .dat/.d/.bnd/.lds
//   geometry.f90:172-290 GEOMETRY_20BXZ node numbering, :425-504 cube_bc20
//   loading.f90:386-480 load_p121 patch pattern
//   input.f90:3336 READ_P121, :1037-1060 READ_G_NUM_PP, :893-896 READ_G_COORD_PP,
//     :2622 READ_REST, :2399 READ_LOADS
//   new_library.f90:3059-3212 REARRANGE + find_g3, :3569-3597 ABAQUS2SG
//   p121.f90:70-141 .res lines and the Ensight displacement file
#include "pfgpu.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <fstream>
#include <new>
#include <sstream>
#include <string>
#include <vector>

namespace pf {
void set_error(const char *fmt, ...);
int host_exception(const char *name);   // pf_abi.cu: an exception -> PF_FAILURE
}
using pf::set_error;

namespace {

// Rows reserved up front when a deck is read; beyond this the arrays grow
// with the lines actually present, whatever counts the .dat record claims.
constexpr int kReserveRows = 1 << 20;

// ---------------------------------------------------------------------------
// Fortran edit descriptors used by the decks and result files
std::string fmt_E(double v, int w, int d)
{
    const bool neg = std::signbit(v);
    const double a = std::fabs(v);
    std::string digits;
    int ex = 0;
    if (a == 0.0) {
        digits.assign(d, '0');
    } else {
        char buf[64];
        snprintf(buf, sizeof buf, "%.*e", d - 1, a);   // m.mmmme+XX
        digits.push_back(buf[0]);
        if (d > 1) digits.append(buf + 2, d - 1);
        ex = atoi(strchr(buf, 'e') + 1) + 1;
    }
    char eb[16];
    snprintf(eb, sizeof eb, "E%c%02d", ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
    std::string s = std::string(neg ? "-" : "") + "0." + digits + eb;
    if ((int)s.size() < w) s.insert(0, w - s.size(), ' ');
    return s;
}

std::string fmt_I(long long v, int w)
{
    char buf[64];
    snprintf(buf, sizeof buf, "%*lld", w, v);
    return buf;
}

std::string fmt_F(double v, int w, int d)
{
    char buf[64];
    snprintf(buf, sizeof buf, "%*.*f", w, d, v);
    return buf;
}

bool read_tokens(const std::string &path, std::vector<std::string> &tok)
{
    std::ifstream f(path);
    if (!f) return false;
    std::string t;
    while (f >> t) {
        // list-directed input: quotes delimit strings, commas separate values
        std::string u;
        for (char ch : t)
            if (ch != '\'' && ch != '"') u.push_back(ch == ',' ? ' ' : ch);
        std::istringstream ss(u);
        std::string w;
        while (ss >> w) tok.push_back(w);
    }
    return true;
}

double to_d(const std::string &s)
{
    std::string t = s;
    for (char &ch : t)
        if (ch == 'd' || ch == 'D') ch = 'E';
    return strtod(t.c_str(), nullptr);
}

// ---------------------------------------------------------------------------
// Structured 20-node cube in GEOMETRY_20BXZ numbering.  Each y-layer holds a
// "face" plane of F1 nodes (z-levels of 2*nxe+1 nodes alternating with
// rows of nxe+1 z-midside nodes, top level first) followed by a "mid" plane
// of F2 = (nxe+1)(nze+1) y-midside nodes.
struct CubeNumbering {
    long long nxe, nze, F1, F2, L, pitch;
    CubeNumbering(int nx, int nz)
        : nxe(nx), nze(nz), F1((2LL * nx + 1) * (nz + 1) + (nx + 1LL) * nz), F2((nx + 1LL) * (nz + 1)),
          L(F1 + F2), pitch(3LL * nx + 2)
    {
    }
    long long face(long long j, long long lev, long long xh) const { return 1 + j * L + lev * pitch + xh; }
    long long half(long long j, long long lev, long long xc) const
    {
        return 1 + j * L + lev * pitch + (2 * nxe + 1) + xc;
    }
    long long mid(long long j, long long lev, long long xc) const { return 1 + j * L + F1 + lev * (nxe + 1) + xc; }
};

// Nodes and coordinates of element iel (1-based), Smith-Griffiths order.
void cube_element(int iel, int nxe, int nze, double aa, double bb, double cc, int num[20], double co[60])
{
    const CubeNumbering N(nxe, nze);
    const long long e = iel - 1;
    const long long j = e / ((long long)nxe * nze);           // y layer
    const long long rem = e % ((long long)nxe * nze);
    const long long k = rem / nxe, i = rem % nxe;             // z layer (0 = top), x column
    const long long nodes[20] = {
        N.face(j, k + 1, 2 * i), N.half(j, k, i), N.face(j, k, 2 * i), N.face(j, k, 2 * i + 1),
        N.face(j, k, 2 * i + 2), N.half(j, k, i + 1), N.face(j, k + 1, 2 * i + 2), N.face(j, k + 1, 2 * i + 1),
        N.mid(j, k + 1, i), N.mid(j, k, i), N.mid(j, k, i + 1), N.mid(j, k + 1, i + 1),
        N.face(j + 1, k + 1, 2 * i), N.half(j + 1, k, i), N.face(j + 1, k, 2 * i), N.face(j + 1, k, 2 * i + 1),
        N.face(j + 1, k, 2 * i + 2), N.half(j + 1, k, i + 1), N.face(j + 1, k + 1, 2 * i + 2),
        N.face(j + 1, k + 1, 2 * i + 1)};
    for (int a = 0; a < 20; ++a) num[a] = (int)nodes[a];
    // x: 0 = left, 1 = mid, 2 = right; y: 0 front, 1 mid, 2 back; z: 0 bottom, 1 mid, 2 top
    static const int xs[20] = {0, 0, 0, 1, 2, 2, 2, 1, 0, 0, 2, 2, 0, 0, 0, 1, 2, 2, 2, 1};
    static const int ys[20] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2, 2, 2};
    static const int zs[20] = {0, 1, 2, 2, 2, 1, 0, 0, 0, 2, 2, 0, 0, 1, 2, 2, 2, 1, 0, 0};
    const double x0 = (double)i * aa, x1 = (double)(i + 1) * aa;
    const double y0 = (double)j * bb, y1 = (double)(j + 1) * bb;
    const double zt = -(double)k * cc, zb = -(double)(k + 1) * cc;
    const double xv[3] = {x0, .5 * (x0 + x1), x1};
    const double yv[3] = {y0, .5 * (y0 + y1), y1};
    const double zv[3] = {zb, .5 * (zb + zt), zt};
    for (int a = 0; a < 20; ++a) {
        co[a] = xv[xs[a]];
        co[20 + a] = yv[ys[a]];
        co[40 + a] = zv[zs[a]];
    }
}

long long cube_nn(long long nxe, long long nye, long long nze)
{
    return ((2 * nxe + 1) * (nze + 1) + (nxe + 1) * nze) * (nye + 1) + (nxe + 1) * (nze + 1) * nye;
}

// Restraints per node (1 free, 0 fixed), bc 0 = cube_bc20, bc 1 = fixed base.
void cube_fix(int nxe, int nye, int nze, int bc, std::vector<int> &fix)
{
    const CubeNumbering N(nxe, nze);
    const long long nn = cube_nn(nxe, nye, nze);
    fix.assign((size_t)nn * 3, 1);
    auto set = [&](long long node, int fx, int fy, int fz) {
        int *f = &fix[(size_t)(node - 1) * 3];
        f[0] &= fx;
        f[1] &= fy;
        f[2] &= fz;
    };
    for (long long j = 0; j <= nye; ++j) {
        const bool yface = (j == 0 || j == nye);
        for (long long lev = 0; lev <= nze; ++lev) {
            const bool base = lev == nze;
            for (long long xh = 0; xh <= 2 * nxe; ++xh) {
                const long long nd = N.face(j, lev, xh);
                const bool xface = (xh == 0 || xh == 2 * nxe);
                if (base) set(nd, 0, 0, 0);
                else if (bc == 0) set(nd, xface ? 0 : 1, yface ? 0 : 1, 1);
            }
            if (lev < nze)
                for (long long xc = 0; xc <= nxe; ++xc) {
                    const long long nd = N.half(j, lev, xc);
                    const bool xface = (xc == 0 || xc == nxe);
                    if (bc == 0) set(nd, xface ? 0 : 1, yface ? 0 : 1, 1);
                }
        }
        if (j < nye)
            for (long long lev = 0; lev <= nze; ++lev)
                for (long long xc = 0; xc <= nxe; ++xc) {
                    const long long nd = N.mid(j, lev, xc);
                    const bool xface = (xc == 0 || xc == nxe);
                    if (lev == nze) set(nd, 0, 0, 0);
                    else if (bc == 0) set(nd, xface ? 0 : 1, 1, 1);
                }
    }
}

// Sequential equation numbering over nodes and dofs, skipping fixed dofs:
// the numbering REARRANGE + find_g3 produce for a restraint list sorted by
// node (new_library.f90:3059-3212).
int number_nodes(int nn, const int *fix, std::vector<int> &node_eq)
{
    node_eq.assign((size_t)nn * 3, 0);
    long long q = 0;
    for (size_t s = 0; s < (size_t)nn * 3; ++s)
        if (fix[s]) node_eq[s] = (int)++q;
    return (int)q;
}

// load_p121 patch pattern for 20-node meshes (loading.f90:386-480): node and
// multiplier in the order the reference lists them.
void load_p121_pattern(int nle, int nxe, int nze, std::vector<int> &node, std::vector<double> &mult)
{
    const CubeNumbering N(nxe, nze);
    node.clear();
    mult.clear();
    auto row = [&](long long j, bool outer) {
        for (int xh = 0; xh <= 2 * nle; ++xh) {
            node.push_back((int)N.face(j, 0, xh));
            const bool end = (xh == 0 || xh == 2 * nle);
            mult.push_back(outer ? (end ? -1.0 : (xh % 2 ? 4.0 : -2.0)) : (end ? -2.0 : (xh % 2 ? 8.0 : -4.0)));
        }
    };
    row(0, true);
    for (int j = 0; j < nle; ++j) {
        for (int xc = 0; xc <= nle; ++xc) {
            node.push_back((int)N.mid(j, 0, xc));
            mult.push_back((xc == 0 || xc == nle) ? 4.0 : 8.0);
        }
        row(j + 1, j == nle - 1);
    }
}

struct Deck {
    std::string element;
    int meshgen = 0, partitioner = 0, nels = 0, nn = 0, nr = 0, nip = 0, nod = 0, loaded = 0, limit = 0;
    double e = 0, v = 0, tol = 0;
    std::vector<double> coords;   // (3, nn)
    std::vector<int> g_num;       // (nod, nels)
    std::vector<int> rest;        // (4, nr) row-major per node
    std::vector<int> lnode;
    std::vector<double> lval;     // (3, loaded)
};

int read_mesh_files(const std::string &job, Deck &D);

int read_deck(const std::string &job, Deck &D)
{
    std::vector<std::string> t;
    if (!read_tokens(job + ".dat", t) || t.size() < 13) {
        set_error("cannot read %s.dat", job.c_str());
        return 1;
    }
    D.element = t[0];
    D.meshgen = atoi(t[1].c_str());
    D.partitioner = atoi(t[2].c_str());
    D.nels = atoi(t[3].c_str());
    D.nn = atoi(t[4].c_str());
    D.nr = atoi(t[5].c_str());
    D.nip = atoi(t[6].c_str());
    D.nod = atoi(t[7].c_str());
    D.loaded = atoi(t[8].c_str());
    D.e = to_d(t[9]);
    D.v = to_d(t[10]);
    D.tol = to_d(t[11]);
    D.limit = atoi(t[12].c_str());
    if (D.element != "hexahedron" || D.nod != 20) {
        set_error("%s.dat: only 20-node hexahedra are supported (got %s, nod=%d)", job.c_str(),
                  D.element.c_str(), D.nod);
        return 1;
    }
    return read_mesh_files(job, D);
}

// job.d (nodes, elements of D.nod = 20 or 8 nodes), job.bnd and job.lds of a
// deck whose .dat record is already in D (READ_G_NUM_PP, READ_G_COORD_PP,
// READ_REST, READ_LOADS of src/modules/mpi/input.f90)
int read_mesh_files(const std::string &job, Deck &D)
{
    std::ifstream f(job + ".d");
    if (!f) {
        set_error("cannot read %s.d", job.c_str());
        return 1;
    }
    if (D.nn < 1 || D.nels < 1) {
        set_error("%s.dat: %d elements and %d nodes", job.c_str(), D.nels, D.nn);
        return 1;
    }
    std::string line;
    std::getline(f, line);
    std::getline(f, line);
    // the arrays grow with the lines actually read, not with the counts the
    // .dat record claims
    D.coords.clear();
    D.coords.reserve((size_t)3 * std::min(D.nn, kReserveRows));
    for (int i = 0; i < D.nn; ++i) {
        if (!std::getline(f, line)) { set_error("%s.d: short node list", job.c_str()); return 1; }
        std::istringstream ss(line);
        std::string id, a, b, c;
        ss >> id >> a >> b >> c;
        D.coords.push_back(to_d(a));
        D.coords.push_back(to_d(b));
        D.coords.push_back(to_d(c));
    }
    std::getline(f, line);   // *ELEMENTS
    const int nod = D.nod;
    if (nod != 20 && nod != 8) { set_error("%s: %d-node elements are not supported", job.c_str(), nod); return 1; }
    D.g_num.clear();
    D.g_num.reserve((size_t)nod * std::min(D.nels, kReserveRows));
    for (int e = 0; e < D.nels; ++e) {
        if (!std::getline(f, line)) { set_error("%s.d: short element list", job.c_str()); return 1; }
        std::istringstream ss(line);
        long long k;
        int nd[20];
        ss >> k >> k >> k >> k;
        for (int a = 0; a < nod; ++a) ss >> nd[a];
        if (!ss) { set_error("%s.d: bad element line %d", job.c_str(), e + 1); return 1; }
        D.g_num.insert(D.g_num.end(), nd, nd + nod);
    }
    if (D.meshgen == 2) {   // ABAQUS2SG (new_library.f90:3569-3627): node i takes file node from[i]
        static const int from20[20] = {4, 12, 1, 9, 2, 10, 3, 11, 20, 17, 18, 19, 8, 16, 5, 13, 6, 14, 7, 15};
        static const int from8[8] = {1, 5, 6, 2, 4, 8, 7, 3};
        const int *from = nod == 20 ? from20 : from8;
        int tmp[20];
        for (int e = 0; e < D.nels; ++e) {
            int *g = &D.g_num[nod * (size_t)e];
            std::copy(g, g + nod, tmp);
            for (int a = 0; a < nod; ++a) g[a] = tmp[from[a] - 1];
        }
    }
    std::vector<std::string> tb;
    if (!read_tokens(job + ".bnd", tb) || tb.size() < (size_t)4 * D.nr) {
        set_error("cannot read %d restraints from %s.bnd", D.nr, job.c_str());
        return 1;
    }
    D.rest.resize((size_t)4 * D.nr);
    for (size_t i = 0; i < (size_t)4 * D.nr; ++i) D.rest[i] = atoi(tb[i].c_str());
    if (D.loaded > 0) {
        std::vector<std::string> tl;
        if (!read_tokens(job + ".lds", tl) || tl.size() < (size_t)4 * D.loaded) {
            set_error("cannot read %d loads from %s.lds", D.loaded, job.c_str());
            return 1;
        }
        D.lnode.resize(D.loaded);
        D.lval.resize((size_t)3 * D.loaded);
        for (int i = 0; i < D.loaded; ++i) {
            D.lnode[i] = atoi(tl[4 * (size_t)i].c_str());
            for (int d = 0; d < 3; ++d) D.lval[3 * (size_t)i + d] = to_d(tl[4 * (size_t)i + 1 + d]);
        }
    }
    return 0;
}

// rest -> per-node fixity (rest rows: node, then 0 = fixed / nonzero = free)
int rest_to_fix(int nn, int nr, const int *rest, std::vector<int> &fix)
{
    fix.assign((size_t)nn * 3, 1);
    int last = 0;
    for (int i = 0; i < nr; ++i) {
        const int nd = rest[4 * (size_t)i];
        if (nd < 1 || nd > nn) {
            set_error("restraint row %d names node %d outside 1..%d", i + 1, nd, nn);
            return 1;
        }
        if (nd <= last) {
            set_error("restraint rows must be sorted by node (row %d: node %d after %d)", i + 1, nd, last);
            return 1;
        }
        last = nd;
        for (int d = 0; d < 3; ++d) fix[(size_t)(nd - 1) * 3 + d] = rest[4 * (size_t)i + 1 + d] != 0 ? 1 : 0;
    }
    return 0;
}

}  // namespace

// ===========================================================================
extern "C" int pf_mesh_cube(const int *nxe, const int *nye, const int *nze, const double *aa, const double *bb,
                            const double *cc, int *nels, int *nn, int *g_num, double *g_coord)
try {
    if (!nxe || !nye || !nze || !aa || !bb || !cc || !nels || !nn || *nxe < 1 || *nye < 1 || *nze < 1) {
        set_error("pf_mesh_cube: invalid arguments");
        return PF_FAILURE;
    }
    const long long ne = (long long)*nxe * *nye * *nze;
    const long long nnl = cube_nn(*nxe, *nye, *nze);
    if (ne * 60 > 0x7fffffffLL * 4 || nnl * 3 > 0x7fffffffLL) {
        set_error("pf_mesh_cube: mesh too large");
        return PF_FAILURE;
    }
    *nels = (int)ne;
    *nn = (int)nnl;
    if (!g_num) return PF_SUCCESS;
    for (long long e = 0; e < ne; ++e) {
        double co[60];
        cube_element((int)(e + 1), *nxe, *nze, *aa, *bb, *cc, g_num + 20 * e, co);
        if (g_coord) std::copy(co, co + 60, g_coord + 60 * e);
    }
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_mesh_cube");
}

extern "C" int pf_cube_restraints(const int *nxe, const int *nye, const int *nze, const int *bc, int *node_fix)
try {
    if (!nxe || !nye || !nze || !bc || !node_fix || (*bc != 0 && *bc != 1) || *nxe < 1 || *nye < 1 || *nze < 1 ||
        cube_nn(*nxe, *nye, *nze) * 3 > 0x7fffffffLL) {
        set_error("pf_cube_restraints: invalid arguments");
        return PF_FAILURE;
    }
    std::vector<int> fix;
    cube_fix(*nxe, *nye, *nze, *bc, fix);
    std::copy(fix.begin(), fix.end(), node_fix);
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_cube_restraints");
}

extern "C" int pf_number_equations(const int *nels, const int *nn, const int *g_num, const int *node_fix, int *g_g,
                                   int *neq)
try {
    if (!nels || !nn || !g_num || !node_fix || !g_g || !neq) {
        set_error("pf_number_equations: null argument");
        return PF_FAILURE;
    }
    if (*nels < 0 || *nn < 1) {
        set_error("pf_number_equations: %d elements and %d nodes", *nels, *nn);
        return PF_FAILURE;
    }
    std::vector<int> node_eq;
    *neq = number_nodes(*nn, node_fix, node_eq);
    for (size_t e = 0; e < (size_t)*nels; ++e)
        for (int a = 0; a < 20; ++a) {
            const int nd = g_num[20 * e + a];
            if (nd < 1 || nd > *nn) {
                set_error("pf_number_equations: node %d outside 1..%d", nd, *nn);
                return PF_FAILURE;
            }
            for (int d = 0; d < 3; ++d) g_g[60 * e + 3 * a + d] = node_eq[(size_t)(nd - 1) * 3 + d];
        }
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_number_equations");
}

extern "C" int pf_cube_top_pressure(const int *nxe, const int *nze, const int *nels, const double *aa,
                                    const double *bb, const double *p, const int *g_g, const int *neq, double *r)
try {
    if (!nxe || !nze || !nels || !aa || !bb || !p || !g_g || !neq || !r) {
        set_error("pf_cube_top_pressure: null argument");
        return PF_FAILURE;
    }
    if (*nxe < 1 || *nze < 1 || *nels < 0) {
        set_error("pf_cube_top_pressure: nxe=%d nze=%d nels=%d", *nxe, *nze, *nels);
        return PF_FAILURE;
    }
    const double A = *aa * *bb;
    const double corner = *p * A / 12.0, midside = -*p * A / 3.0;
    // top-face nodes of an element: corners 3,5,15,17 and mid-sides 4,10,11,16
    static const int cn[4] = {3, 5, 15, 17}, ms[4] = {4, 10, 11, 16};
    const long long per_layer = (long long)*nxe * *nze;
    for (long long e = 0; e < *nels; ++e) {
        const long long k = (e % per_layer) / *nxe;
        if (k != 0) continue;
        for (int t = 0; t < 4; ++t) {
            const int qc = g_g[60 * e + 3 * (cn[t] - 1) + 2];
            if (qc > 0 && qc <= *neq) r[qc - 1] += corner;
            const int qm = g_g[60 * e + 3 * (ms[t] - 1) + 2];
            if (qm > 0 && qm <= *neq) r[qm - 1] += midside;
        }
    }
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_cube_top_pressure");
}

namespace {
inline uint32_t mulhilo(uint32_t a, uint32_t b, uint32_t *hi)
{
    const uint64_t pr = (uint64_t)a * b;
    *hi = (uint32_t)(pr >> 32);
    return (uint32_t)pr;
}
// Philox4x32-10 (Salmon et al., SC'11)
void philox4x32(uint32_t ctr[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, hi1;
        const uint32_t lo0 = mulhilo(0xD2511F53u, ctr[0], &hi0);
        const uint32_t lo1 = mulhilo(0xCD9E8D57u, ctr[2], &hi1);
        const uint32_t c0 = hi1 ^ ctr[1] ^ k0, c2 = hi0 ^ ctr[3] ^ k1;
        ctr[0] = c0;
        ctr[1] = lo1;
        ctr[2] = c2;
        ctr[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}
}  // namespace

extern "C" int pf_random_material(const int *nels, const long long *seed, const double *e_lo, const double *e_hi,
                                  const double *v_lo, const double *v_hi, double *e, double *v)
try {
    if (!nels || !seed || !e_lo || !e_hi || !v_lo || !v_hi || !e || !v || *nels < 0 || !(*e_lo > 0) ||
        !(*e_hi >= *e_lo)) {
        set_error("pf_random_material: invalid arguments");
        return PF_FAILURE;
    }
    const uint32_t k0 = (uint32_t)((unsigned long long)*seed & 0xffffffffu);
    const uint32_t k1 = (uint32_t)((unsigned long long)*seed >> 32);
    const double l0 = std::log(*e_lo), l1 = std::log(*e_hi);
    for (long long i = 0; i < *nels; ++i) {
        uint32_t c[4] = {(uint32_t)i, (uint32_t)((unsigned long long)i >> 32), 0u, 0u};
        philox4x32(c, k0, k1);
        // 53-bit uniforms in [0,1)
        const double u1 = (double)((((uint64_t)c[0]) << 21) ^ (c[1] >> 11)) / 9007199254740992.0;
        const double u2 = (double)((((uint64_t)c[2]) << 21) ^ (c[3] >> 11)) / 9007199254740992.0;
        e[i] = std::exp(l0 + u1 * (l1 - l0));
        v[i] = *v_lo + u2 * (*v_hi - *v_lo);
    }
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_random_material");
}

// ---------------------------------------------------------------------------
static int p12meshgen_p123(const std::string &job, const std::vector<std::string> &t);
static int p12meshgen_p122(const std::string &job, const std::vector<std::string> &t);

extern "C" int pf_p12meshgen(const char *job_c)
try {
    if (!job_c) { set_error("pf_p12meshgen: null job name"); return PF_FAILURE; }
    const std::string job(job_c);
    std::vector<std::string> t;
    if (!read_tokens(job + ".mg", t) || t.size() < 14) {
        set_error("cannot read %s.mg", job.c_str());
        return PF_FAILURE;
    }
    if (t[0] == "p123") return p12meshgen_p123(job, t);
    if (t[0] == "p122") return p12meshgen_p122(job, t);
    if (t[0] != "p121") {
        set_error("%s.mg: the p121, p122 and p123 cases are supported (got %s)", job.c_str(), t[0].c_str());
        return PF_FAILURE;
    }
    const std::string iotype = t[1];
    const int nels = atoi(t[2].c_str()), nxe = atoi(t[3].c_str()), nze = atoi(t[4].c_str());
    const int nod = atoi(t[5].c_str()), nip = atoi(t[6].c_str());
    const double aa = to_d(t[7]), bb = to_d(t[8]), cc = to_d(t[9]), e = to_d(t[10]), v = to_d(t[11]);
    const double tol = to_d(t[12]);
    const int limit = atoi(t[13].c_str());
    if (nod != 20 || iotype != "parafem" || nxe < 1 || nze < 1 || nels < 1 || (long long)nxe * nze > nels || nels % (nxe * nze) != 0) {
        set_error("%s.mg: supported: 'parafem' decks of 20-node cubes (nels divisible by nxe*nze)", job.c_str());
        return PF_FAILURE;
    }
    const int nye = nels / nxe / nze;
    const long long nn = cube_nn(nxe, nye, nze);
    const int nle = nxe / 5;
    // node coordinates (every node is written by some element)
    std::vector<double> gc((size_t)3 * nn, 0.0);
    std::vector<int> gnum((size_t)20 * nels);
    for (int iel = 1; iel <= nels; ++iel) {
        double co[60];
        int *num = &gnum[20 * (size_t)(iel - 1)];
        cube_element(iel, nxe, nze, aa, bb, cc, num, co);
        for (int a = 0; a < 20; ++a)
            for (int d = 0; d < 3; ++d) gc[3 * (size_t)(num[a] - 1) + d] = co[a + 20 * d];
    }
    std::vector<int> fix;
    cube_fix(nxe, nye, nze, 0, fix);
    std::vector<int> lnode;
    std::vector<double> mult;
    load_p121_pattern(nle, nxe, nze, lnode, mult);

    FILE *fd = fopen((job + ".d").c_str(), "w");
    if (!fd) { set_error("cannot write %s.d", job.c_str()); return PF_FAILURE; }
    fprintf(fd, "*THREE_DIMENSIONAL\n*NODES\n");
    for (long long i = 0; i < nn; ++i)
        fprintf(fd, "%s%s%s%s\n", fmt_I(i + 1, 12).c_str(), fmt_E(gc[3 * i], 14, 6).c_str(),
                fmt_E(gc[3 * i + 1], 14, 6).c_str(), fmt_E(gc[3 * i + 2], 14, 6).c_str());
    fprintf(fd, "*ELEMENTS\n");
    static const int abq[20] = {3, 5, 7, 1, 15, 17, 19, 13, 4, 6, 8, 2, 16, 18, 20, 14, 10, 11, 12, 9};
    for (int iel = 0; iel < nels; ++iel) {
        std::string s = fmt_I(iel + 1, 12) + " 3 20 1 ";
        for (int a = 0; a < 20; ++a) s += fmt_I(gnum[20 * (size_t)iel + abq[a] - 1], 12);
        fprintf(fd, "%s 1\n", s.c_str());
    }
    fclose(fd);

    FILE *fb = fopen((job + ".bnd").c_str(), "w");
    if (!fb) { set_error("cannot write %s.bnd", job.c_str()); return PF_FAILURE; }
    long long nr = 0;
    for (long long i = 0; i < nn; ++i) {
        const int *f = &fix[3 * (size_t)i];
        if (f[0] && f[1] && f[2]) continue;
        fprintf(fb, "%s%s%s%s\n", fmt_I(i + 1, 15).c_str(), fmt_I(f[0], 6).c_str(), fmt_I(f[1], 6).c_str(),
                fmt_I(f[2], 6).c_str());
        ++nr;
    }
    fclose(fb);

    FILE *fl = fopen((job + ".lds").c_str(), "w");
    if (!fl) { set_error("cannot write %s.lds", job.c_str()); return PF_FAILURE; }
    for (size_t i = 0; i < lnode.size(); ++i) {
        const double val = -mult[i] * aa * bb * (25.0 / 12.0);
        fprintf(fl, "%s  0.00000000E+00  0.00000000E+00%s\n", fmt_I(lnode[i], 12).c_str(),
                fmt_E(val, 16, 8).c_str());
    }
    fclose(fl);

    FILE *ft = fopen((job + ".dat").c_str(), "w");
    if (!ft) { set_error("cannot write %s.dat", job.c_str()); return PF_FAILURE; }
    fprintf(ft, "'hexahedron'\n2\n1\n%s%s%s%s%s%s\n", fmt_I(nels, 12).c_str(), fmt_I(nn, 12).c_str(),
            fmt_I(nr, 12).c_str(), fmt_I(nip, 5).c_str(), fmt_I(nod, 5).c_str(),
            fmt_I((long long)lnode.size(), 9).c_str());
    fprintf(ft, "%s%s%s%s\n", fmt_E(e, 12, 4).c_str(), fmt_E(v, 12, 4).c_str(), fmt_E(tol, 12, 4).c_str(),
            fmt_I(limit, 8).c_str());
    fclose(ft);
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_p12meshgen");
}

// ---------------------------------------------------------------------------
// The p121 job (p121.f90:1-141) with the solve on the GPU.
extern "C" int pf_p121_run(const char *job_c, const int *device, const int *mode, int *iters_out,
                           double *central_out)
try {
    if (!job_c || !device || !mode) { set_error("pf_p121_run: null argument"); return PF_FAILURE; }
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    auto secs = [&](clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); };
    const std::string job(job_c);
    Deck D;
    if (read_deck(job, D)) return PF_FAILURE;
    std::vector<int> fix;
    if (rest_to_fix(D.nn, D.nr, D.rest.data(), fix)) return PF_FAILURE;
    const double t_read = secs(t0);
    std::vector<int> g_g((size_t)60 * D.nels);
    int neq = 0;
    if (pf_number_equations(&D.nels, &D.nn, D.g_num.data(), fix.data(), g_g.data(), &neq)) return PF_FAILURE;
    std::vector<double> gcoord((size_t)60 * D.nels);
    for (size_t e = 0; e < (size_t)D.nels; ++e)
        for (int a = 0; a < 20; ++a)
            for (int d = 0; d < 3; ++d)
                gcoord[60 * e + a + 20 * d] = D.coords[3 * (size_t)(D.g_num[20 * e + a] - 1) + d];
    void *ctx = nullptr;
    int rc = PF_FAILURE;
    std::vector<double> r(neq > 0 ? neq : 1, 0.0), x(neq > 0 ? neq : 1, 0.0);
    double q = 0.0, sigma[6] = {0}, relres = 0.0;
    int iters = 0, one = 1, flags = 0;
    double t_setup = 0, t_solve = 0;
    do {
        if (pf_ctx_create(device, &ctx)) break;
        if (pf_setup(&ctx, &D.nels, &D.nn, &neq, D.g_num.data(), g_g.data(), gcoord.data())) break;
        if (pf_set_material(&ctx, &one, &D.e, &D.v)) break;
        if (pf_form_storkm(&ctx, &D.nip, &flags)) break;
        t_setup = secs(t0);
        // LOAD + SCATTER_NOADD (loading.f90:36-146): r(eq) = value, last node entry wins
        std::vector<int> node_slot((size_t)D.nn + 1, -1);
        for (int i = 0; i < D.loaded; ++i)
            if (D.lnode[i] >= 1 && D.lnode[i] <= D.nn) node_slot[D.lnode[i]] = i;
        // equation of (node, dof) from the numbering
        std::vector<int> node_eq;
        number_nodes(D.nn, fix.data(), node_eq);
        for (int nd = 1; nd <= D.nn; ++nd) {
            const int i = node_slot[nd];
            if (i < 0) continue;
            for (int d = 0; d < 3; ++d) {
                const int eq = node_eq[(size_t)(nd - 1) * 3 + d];
                if (eq > 0) r[eq - 1] = D.lval[3 * (size_t)i + d];
            }
        }
        for (int i = 0; i < neq; ++i) q += r[i];
        const auto ts = clk::now();
        if (pf_solve(&ctx, r.data(), &D.tol, &D.limit, mode, x.data(), &iters, &relres)) break;
        t_solve = secs(ts);
        int iel = 1;
        if (pf_centroid_stress(&ctx, &iel, x.data(), sigma)) break;
        rc = PF_SUCCESS;
    } while (0);
    if (ctx) pf_ctx_destroy(&ctx);
    if (rc) return PF_FAILURE;

    FILE *fr = fopen((job + ".res").c_str(), "w");
    if (!fr) { set_error("cannot write %s.res", job.c_str()); return PF_FAILURE; }
    fprintf(fr, "This job ran on %s processes\n", fmt_I(1, 7).c_str());
    fprintf(fr, "There are %s nodes%s restrained and %s equations\n", fmt_I(D.nn, 12).c_str(),
            fmt_I(D.nr, 12).c_str(), fmt_I(neq, 12).c_str());
    fprintf(fr, "Time to read input is:%s\n", fmt_F(t_read, 10, 4).c_str());
    fprintf(fr, "Time after setup is:%s\n", fmt_F(t_setup, 10, 4).c_str());
    if (D.loaded > 0) fprintf(fr, "The total load is:%s\n", fmt_E(q, 12, 4).c_str());
    fprintf(fr, "The number of iterations to convergence was %s\n", fmt_I(iters, 6).c_str());
    fprintf(fr, "Time to solve equations was  :%s\n", fmt_F(t_solve, 10, 4).c_str());
    fprintf(fr, "The central nodal displacement is :%s\n", fmt_E(neq > 0 ? x[0] : 0.0, 12, 4).c_str());
    fprintf(fr, "The Centroid point stresses for element 1 are\n");
    fprintf(fr, "Point %s\n", fmt_I(1, 5).c_str());
    std::string sl;
    for (int k = 0; k < 6; ++k) sl += fmt_E(sigma[k], 12, 4);
    fprintf(fr, "%s\n", sl.c_str());

    // Ensight Gold per-node vector file (p121.f90:124-138, output.f90:2983-3117)
    FILE *fe = fopen((job + ".ensi.DISPL-000001").c_str(), "w");
    if (!fe) { fclose(fr); set_error("cannot write the displacement file"); return PF_FAILURE; }
    fprintf(fe, "Alya Ensight Gold --- Vector per-node variable file\npart\n     1\ncoordinates\n");
    std::vector<int> node_eq;
    number_nodes(D.nn, fix.data(), node_eq);
    for (int d = 0; d < 3; ++d)
        for (int nd = 0; nd < D.nn; ++nd) {
            const int eq = node_eq[(size_t)nd * 3 + d];
            fprintf(fe, "%s\n", fmt_E(eq > 0 ? x[eq - 1] : 0.0, 12, 5).c_str());
        }
    fclose(fe);
    fprintf(fr, "This analysis took  :%s\n", fmt_F(secs(t0), 10, 4).c_str());
    fclose(fr);
    if (iters_out) *iters_out = iters;
    if (central_out) *central_out = neq > 0 ? x[0] : 0.0;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_p121_run");
}

// load_p121's patch on the top face (loading.f90:386-480) as a load vector:
// r(z-equation of each listed node) = factor * multiplier, by LOAD +
// SCATTER_NOADD (loading.f90:36-146): assignment, the last entry wins.
extern "C" int pf_patch_loads(const int *nxe, const int *nze, const double *factor, const int *nels,
                              const int *g_num, const int *g_g, const int *neq, double *r)
try {
    if (!nxe || !nze || !factor || !nels || !g_num || !g_g || !neq || !r || *nxe < 5 || *nze < 1 || *nels < 0) {
        set_error("pf_patch_loads: invalid arguments (nxe >= 5)");
        return PF_FAILURE;
    }
    std::vector<int> node;
    std::vector<double> mult;
    load_p121_pattern(*nxe / 5, *nxe, *nze, node, mult);
    int maxnode = 0;
    for (int nd : node) maxnode = nd > maxnode ? nd : maxnode;
    std::vector<int> which((size_t)maxnode + 1, -1);
    for (size_t i = 0; i < node.size(); ++i) which[node[i]] = (int)i;
    for (size_t e = 0; e < (size_t)*nels; ++e)
        for (int a = 0; a < 20; ++a) {
            const int nd = g_num[20 * e + a];
            if (nd < 1 || nd > maxnode || which[nd] < 0) continue;
            const int q = g_g[60 * e + 3 * a + 2];
            if (q > 0 && q <= *neq) r[q - 1] = *factor * mult[which[nd]];
        }
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_patch_loads");
}

// ===========================================================================
// p123: 3-D Laplace with 8-node bricks (src/programs/5th_ed/p123/p123.f90).
namespace {

// Nodes (Smith-Griffiths order) and coordinates coord(8,3) of element iel
// (1-based) of an nxe x nye x nze box of bricks numbered in x-z planes
// marching in y (GEOMETRY_8BXZ, src/modules/shared/geometry.f90:70-166).
void box8_element(int iel, int nxe, int nze, double aa, double bb, double cc, int num[8], double co[24])
{
    const int per_plane = nxe * nze;
    const int iq = (iel - 1) / per_plane;          // y layer (0-based)
    const int in = (iel - 1) % per_plane;
    const int is = in / nxe;                       // z row from the top (0-based)
    const int ip = in % nxe;                       // x column (0-based)
    const long long plane = (long long)(nxe + 1) * (nze + 1);
    // node (x column cx, z level lz from the top, y plane py), 1-based
    auto node = [&](int cx, int lz, int py) { return (int)(py * plane + (long long)lz * (nxe + 1) + cx + 1); };
    // corner signs of the Smith-Griffiths brick: (x: 0 left / 1 right, z: 0 bottom / 1 top, y: 0 front / 1 back)
    static const int sx[8] = {0, 0, 1, 1, 0, 0, 1, 1}, sz[8] = {0, 1, 1, 0, 0, 1, 1, 0},
                     sy[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    for (int a = 0; a < 8; ++a) {
        const int lz = is + 1 - sz[a];             // top of the element is level is, bottom is + 1
        num[a] = node(ip + sx[a], lz, iq + sy[a]);
        co[a] = (ip + sx[a]) * aa;
        co[a + 8] = (iq + sy[a]) * bb;
        co[a + 16] = -(double)lz * cc;
    }
}

// box_bc8 (src/modules/shared/geometry.f90:655-696): node_fix[n] = 1 for a
// free node, 0 for a restrained one.  Restrained: in every x-z plane but
// the last, the last x column (x = nxe*aa) and the top level (z = 0); the
// whole last plane.
void box8_fix(int nxe, int nye, int nze, std::vector<int> &fix)
{
    const long long plane = (long long)(nxe + 1) * (nze + 1);
    fix.assign((size_t)plane * (nye + 1), 1);
    for (long long py = 0; py <= nye; ++py)
        for (long long k = 0; k < plane; ++k) {
            const long long lz = k / (nxe + 1), cx = k % (nxe + 1);
            if (py == nye || cx == nxe || lz == 0) fix[(size_t)(py * plane + k)] = 0;
        }
}

struct Deck8 {
    int meshgen = 0, partitioner = 0, nels = 0, nn = 0, nr = 0, nip = 0, nod = 0, loaded = 0, fixed = 0;
    int limit = 0, nres = 0;
    double kx = 0, ky = 0, kz = 0, tol = 0;
    std::vector<double> coords;   // (3, nn)
    std::vector<int> g_num;       // (8, nels), Smith-Griffiths order
    std::vector<int> rest;        // (2, nr): node, flag
    std::vector<int> lno;         // loaded freedoms (used as equation numbers, p123.f90:98-103)
    std::vector<double> lval;
    std::vector<int> fnode, fsense;
    std::vector<double> fval;
};

int read_deck8(const std::string &job, Deck8 &D)
{
    std::vector<std::string> t;
    if (!read_tokens(job + ".dat", t) || t.size() < 16) {
        set_error("cannot read %s.dat", job.c_str());
        return 1;
    }
    // READ_P123 (src/modules/mpi/input.f90:3620-3806): element, mesh, partition,
    // nels, nn, nr, nip, nod, loaded, fixed, kx, ky, kz, tol, limit, nres
    D.meshgen = atoi(t[1].c_str());
    D.partitioner = atoi(t[2].c_str());
    D.nels = atoi(t[3].c_str());
    D.nn = atoi(t[4].c_str());
    D.nr = atoi(t[5].c_str());
    D.nip = atoi(t[6].c_str());
    D.nod = atoi(t[7].c_str());
    D.loaded = atoi(t[8].c_str());
    D.fixed = atoi(t[9].c_str());
    D.kx = to_d(t[10]);
    D.ky = to_d(t[11]);
    D.kz = to_d(t[12]);
    D.tol = to_d(t[13]);
    D.limit = atoi(t[14].c_str());
    D.nres = atoi(t[15].c_str());
    if (t[0] != "hexahedron" || D.nod != 8 || D.nels < 1 || D.nn < 1) {
        set_error("%s.dat: p123 decks of 8-node hexahedra only (got %s, nod=%d)", job.c_str(), t[0].c_str(), D.nod);
        return 1;
    }
    std::ifstream f(job + ".d");
    if (!f) {
        set_error("cannot read %s.d", job.c_str());
        return 1;
    }
    std::string line;
    std::getline(f, line);
    std::getline(f, line);
    D.coords.clear();   // grown with the lines read, as in read_mesh_files
    D.coords.reserve((size_t)3 * std::min(D.nn, kReserveRows));
    for (int i = 0; i < D.nn; ++i) {
        if (!std::getline(f, line)) { set_error("%s.d: short node list", job.c_str()); return 1; }
        std::istringstream ss(line);
        std::string id, a, b, c;
        ss >> id >> a >> b >> c;
        D.coords.push_back(to_d(a));
        D.coords.push_back(to_d(b));
        D.coords.push_back(to_d(c));
    }
    std::getline(f, line);   // *ELEMENTS
    D.g_num.clear();
    D.g_num.reserve((size_t)8 * std::min(D.nels, kReserveRows));
    for (int e = 0; e < D.nels; ++e) {
        if (!std::getline(f, line)) { set_error("%s.d: short element list", job.c_str()); return 1; }
        std::istringstream ss(line);
        long long k;
        int nd[8];
        ss >> k >> k >> k >> k;
        for (int a = 0; a < 8; ++a) ss >> nd[a];
        if (!ss) { set_error("%s.d: bad element line %d", job.c_str(), e + 1); return 1; }
        D.g_num.insert(D.g_num.end(), nd, nd + 8);
    }
    if (D.meshgen == 2) {   // ABAQUS2SG, 8-node (new_library.f90:3604-3618)
        static const int from[8] = {1, 5, 6, 2, 4, 8, 7, 3};
        int tmp[8];
        for (int e = 0; e < D.nels; ++e) {
            int *g = &D.g_num[8 * (size_t)e];
            std::copy(g, g + 8, tmp);
            for (int a = 0; a < 8; ++a) g[a] = tmp[from[a] - 1];
        }
    }
    std::vector<std::string> tb;
    if (!read_tokens(job + ".bnd", tb) || tb.size() < (size_t)2 * D.nr) {
        set_error("cannot read %d restraints from %s.bnd", D.nr, job.c_str());
        return 1;
    }
    D.rest.resize((size_t)2 * D.nr);
    for (size_t i = 0; i < (size_t)2 * D.nr; ++i) D.rest[i] = atoi(tb[i].c_str());
    if (D.loaded > 0) {   // READ_LOADS (input.f90:2350-2411), one value per freedom
        std::vector<std::string> tl;
        if (!read_tokens(job + ".lds", tl) || tl.size() < (size_t)2 * D.loaded) {
            set_error("cannot read %d loads from %s.lds", D.loaded, job.c_str());
            return 1;
        }
        for (int i = 0; i < D.loaded; ++i) {
            D.lno.push_back(atoi(tl[2 * (size_t)i].c_str()));
            D.lval.push_back(to_d(tl[2 * (size_t)i + 1]));
        }
    }
    if (D.fixed > 0) {   // READ_FIXED (input.f90:2483-2564): node, sense, value
        std::vector<std::string> tf;
        if (!read_tokens(job + ".fix", tf) || tf.size() < (size_t)3 * D.fixed) {
            set_error("cannot read %d fixed freedoms (node sense value) from %s.fix", D.fixed, job.c_str());
            return 1;
        }
        for (int i = 0; i < D.fixed; ++i) {
            D.fnode.push_back(atoi(tf[3 * (size_t)i].c_str()));
            D.fsense.push_back(atoi(tf[3 * (size_t)i + 1].c_str()));
            D.fval.push_back(to_d(tf[3 * (size_t)i + 2]));
        }
    }
    return 0;
}

}  // namespace

extern "C" int pf_mesh_box8(const int *nxe, const int *nye, const int *nze, const double *aa, const double *bb,
                            const double *cc, int *g_num, double *g_coord)
try {
    if (!nxe || !nye || !nze || !aa || !bb || !cc || !g_num || !g_coord || *nxe < 1 || *nye < 1 || *nze < 1) {
        set_error("pf_mesh_box8: invalid arguments");
        return PF_FAILURE;
    }
    const long long nels = (long long)*nxe * *nye * *nze;
    for (long long iel = 1; iel <= nels; ++iel)
        box8_element((int)iel, *nxe, *nze, *aa, *bb, *cc, g_num + 8 * (iel - 1), g_coord + 24 * (iel - 1));
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_mesh_box8");
}

extern "C" int pf_box8_restraints(const int *nxe, const int *nye, const int *nze, int *node_fix)
try {
    if (!nxe || !nye || !nze || !node_fix || *nxe < 1 || *nye < 1 || *nze < 1) {
        set_error("pf_box8_restraints: invalid arguments");
        return PF_FAILURE;
    }
    std::vector<int> fix;
    box8_fix(*nxe, *nye, *nze, fix);
    std::copy(fix.begin(), fix.end(), node_fix);
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_box8_restraints");
}

extern "C" int pf_number_equations1(const int *nels, const int *nn, const int *nod, const int *g_num,
                                    const int *node_fix, int *g_g, int *neq)
try {
    if (!nels || !nn || !nod || !g_num || !node_fix || !g_g || !neq || *nels < 0 || *nn < 1 || *nod < 1) {
        set_error("pf_number_equations1: invalid arguments");
        return PF_FAILURE;
    }
    // equation of a free node = free nodes up to it (rearrange_2 + find_g4,
    // new_library.f90:3118-3124, 3249-3271, for a restraint list sorted by node)
    std::vector<int> eq((size_t)*nn, 0);
    int q = 0;
    for (int n = 0; n < *nn; ++n)
        if (node_fix[n]) eq[n] = ++q;
    for (size_t k = 0; k < (size_t)*nels * *nod; ++k) {
        const int nd = g_num[k];
        if (nd < 1 || nd > *nn) {
            set_error("pf_number_equations1: node %d outside 1..%d", nd, *nn);
            return PF_FAILURE;
        }
        g_g[k] = eq[nd - 1];
    }
    *neq = q;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_number_equations1");
}

// p12meshgen's p123 case (src/tools/preprocessing/p12meshgen/p12meshgen.f90:
// 658-801).  The .fix file is written as READ_FIXED reads it (node, sense,
// value); the reference's generator writes node and value only.
static int p12meshgen_p123(const std::string &job, const std::vector<std::string> &t)
{
    if (t.size() < 15) {
        set_error("%s.mg: the p123 case needs 14 values", job.c_str());
        return PF_FAILURE;
    }
    const std::string iotype = t[1];
    const int nels = atoi(t[2].c_str()), nxe = atoi(t[3].c_str()), nze = atoi(t[4].c_str());
    const int nip = atoi(t[5].c_str());
    const double aa = to_d(t[6]), bb = to_d(t[7]), cc = to_d(t[8]), kx = to_d(t[9]), ky = to_d(t[10]),
                 kz = to_d(t[11]), tol = to_d(t[12]);
    const int limit = atoi(t[13].c_str()), loaded = atoi(t[14].c_str());
    const int fixed = t.size() > 15 ? atoi(t[15].c_str()) : 0;
    if (iotype != "parafem" || nxe < 1 || nze < 1 || nels < 1 || (long long)nxe * nze > nels || nels % (nxe * nze) != 0) {
        set_error("%s.mg: supported: 'parafem' decks (nels divisible by nxe*nze)", job.c_str());
        return PF_FAILURE;
    }
    const int nye = nels / nxe / nze;
    const long long nn = (long long)(nxe + 1) * (nye + 1) * (nze + 1);
    const long long nr = (long long)(nxe + 1) * (nye + 1) + (long long)(nxe + 1) * nze + (long long)nye * nze;
    const int nres = nxe * (nze - 1) + 1;
    std::vector<double> gc((size_t)3 * nn, 0.0);
    std::vector<int> gnum((size_t)8 * nels);
    for (int iel = 1; iel <= nels; ++iel) {
        double co[24];
        int *num = &gnum[8 * (size_t)(iel - 1)];
        box8_element(iel, nxe, nze, aa, bb, cc, num, co);
        for (int a = 0; a < 8; ++a)
            for (int d = 0; d < 3; ++d) gc[3 * (size_t)(num[a] - 1) + d] = co[a + 8 * d];
    }
    FILE *fd = fopen((job + ".d").c_str(), "w");
    if (!fd) { set_error("cannot write %s.d", job.c_str()); return PF_FAILURE; }
    fprintf(fd, "*THREE_DIMENSIONAL\n*NODES\n");
    for (long long i = 0; i < nn; ++i)
        fprintf(fd, "%s%s%s%s\n", fmt_I(i + 1, 12).c_str(), fmt_E(gc[3 * i], 14, 6).c_str(),
                fmt_E(gc[3 * i + 1], 14, 6).c_str(), fmt_E(gc[3 * i + 2], 14, 6).c_str());
    fprintf(fd, "*ELEMENTS\n");
    static const int abq[8] = {1, 4, 8, 5, 2, 3, 7, 6};   // Abaqus order of the written nodes
    for (int iel = 0; iel < nels; ++iel) {
        std::string s = fmt_I(iel + 1, 12) + " 3 8 1 ";
        for (int a = 0; a < 8; ++a) s += fmt_I(gnum[8 * (size_t)iel + abq[a] - 1], 10);
        fprintf(fd, "%s 1\n", s.c_str());
    }
    fclose(fd);
    std::vector<int> fix;
    box8_fix(nxe, nye, nze, fix);
    FILE *fb = fopen((job + ".bnd").c_str(), "w");
    if (!fb) { set_error("cannot write %s.bnd", job.c_str()); return PF_FAILURE; }
    long long written = 0;
    for (long long i = 0; i < nn; ++i)
        if (!fix[(size_t)i]) {
            fprintf(fb, "%s%s\n", fmt_I(i + 1, 8).c_str(), fmt_I(0, 6).c_str());
            ++written;
        }
    fclose(fb);
    if (written != nr) {
        set_error("p12meshgen p123: %lld restrained nodes, expected %lld", written, nr);
        return PF_FAILURE;
    }
    if (loaded > 0) {
        FILE *fl = fopen((job + ".lds").c_str(), "w");
        if (!fl) { set_error("cannot write %s.lds", job.c_str()); return PF_FAILURE; }
        for (int i = 0; i < loaded; ++i) fprintf(fl, "%s%s\n", fmt_I(nres, 10).c_str(), fmt_E(10.0, 16, 8).c_str());
        fclose(fl);
    }
    if (fixed > 0) {
        FILE *ff = fopen((job + ".fix").c_str(), "w");
        if (!ff) { set_error("cannot write %s.fix", job.c_str()); return PF_FAILURE; }
        for (int i = 0; i < fixed; ++i)
            fprintf(ff, "%s%s%s\n", fmt_I(nres, 10).c_str(), fmt_I(1, 6).c_str(), fmt_E(100.0, 16, 8).c_str());
        fclose(ff);
    }
    FILE *ft = fopen((job + ".dat").c_str(), "w");
    if (!ft) { set_error("cannot write %s.dat", job.c_str()); return PF_FAILURE; }
    fprintf(ft, "'hexahedron'\n2\n1\n%s%s%s%s%s%s%s\n", fmt_I(nels, 12).c_str(), fmt_I(nn, 12).c_str(),
            fmt_I(nr, 12).c_str(), fmt_I(nip, 6).c_str(), fmt_I(8, 6).c_str(), fmt_I(loaded, 6).c_str(),
            fmt_I(fixed, 6).c_str());
    fprintf(ft, "%s%s%s%s%s%s\n", fmt_E(kx, 12, 4).c_str(), fmt_E(ky, 12, 4).c_str(), fmt_E(kz, 12, 4).c_str(),
            fmt_E(tol, 12, 4).c_str(), fmt_I(limit, 8).c_str(), fmt_I(nres, 8).c_str());
    fclose(ft);
    return PF_SUCCESS;
}

// The p123 job (p123.f90:1-182) with the solve on the GPU.
extern "C" int pf_p123_run(const char *job_c, const int *device, int *iters_out, double *potentials_out)
try {
    if (!job_c || !device) { set_error("pf_p123_run: null argument"); return PF_FAILURE; }
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    auto secs = [&](clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); };
    const std::string job(job_c);
    Deck8 D;
    if (read_deck8(job, D)) return PF_FAILURE;
    std::vector<int> fix((size_t)D.nn, 1);
    int last = 0;
    for (int i = 0; i < D.nr; ++i) {
        const int nd = D.rest[2 * (size_t)i];
        if (nd < 1 || nd > D.nn || nd <= last) {
            set_error("%s.bnd: restraint row %d (node %d) out of range or not sorted", job.c_str(), i + 1, nd);
            return PF_FAILURE;
        }
        last = nd;
        fix[(size_t)nd - 1] = D.rest[2 * (size_t)i + 1] != 0 ? 1 : 0;
    }
    std::vector<int> g_g((size_t)8 * D.nels);
    int neq = 0, nod = 8;
    if (pf_number_equations1(&D.nels, &D.nn, &nod, D.g_num.data(), fix.data(), g_g.data(), &neq)) return PF_FAILURE;
    std::vector<double> gcoord((size_t)24 * D.nels);
    for (size_t e = 0; e < (size_t)D.nels; ++e)
        for (int a = 0; a < 8; ++a)
            for (int d = 0; d < 3; ++d)
                gcoord[24 * e + a + 8 * d] = D.coords[3 * (size_t)(D.g_num[8 * e + a] - 1) + d];
    void *ctx = nullptr;
    int rc = PF_FAILURE;
    std::vector<double> r(neq > 0 ? neq : 1, 0.0), x(neq > 0 ? neq : 1, 0.0), dg(neq > 0 ? neq : 1, 0.0);
    double q = 0.0, relres = 0.0, t_setup = 0, t_solve = 0;
    int iters = 0, mode = PF_MODE_P121;
    do {
        if (pf_ctx_create(device, &ctx)) break;
        if (pf_setup_scalar8(&ctx, &D.nels, &D.nn, &neq, D.g_num.data(), g_g.data(), gcoord.data())) break;
        if (pf_form_storkc(&ctx, &D.nip, &D.kx, &D.ky, &D.kz)) break;
        // loads: the listed numbers are equations (p123.f90:98-103)
        bool bad = false;
        for (int i = 0; i < D.loaded; ++i) {
            if (D.lno[i] < 1 || D.lno[i] > neq) { bad = true; break; }
            r[D.lno[i] - 1] = D.lval[i];
        }
        if (bad) { set_error("%s.lds: a loaded freedom is outside 1..%d", job.c_str(), neq); break; }
        for (int i = 0; i < neq; ++i) q += r[i];
        // fixed freedoms by the penalty method (p123.f90:104-118; FIND_NO2, loading.f90:742-828)
        std::vector<int> feq;
        for (int i = 0; i < D.fixed; ++i) {
            const int nd = D.fnode[i];
            if (nd < 1 || nd > D.nn || D.fsense[i] != 1 || !fix[(size_t)nd - 1]) { bad = true; break; }
            int e = 0;
            for (int n = 0; n < nd; ++n) e += fix[(size_t)n];
            feq.push_back(e);
        }
        if (bad) { set_error("%s.fix: a fixed freedom is not a free node with sense 1", job.c_str()); break; }
        const double penalty = 1.0e20;
        int nfix = (int)feq.size();
        if (pf_set_fixed(&ctx, &nfix, feq.data(), &penalty)) break;
        if (nfix > 0) {
            if (pf_get_diag(&ctx, dg.data())) break;
            for (int i = 0; i < nfix; ++i) r[feq[i] - 1] = dg[feq[i] - 1] * D.fval[i];
        }
        t_setup = secs(t0);
        const auto ts = clk::now();
        if (pf_solve(&ctx, r.data(), &D.tol, &D.limit, &mode, x.data(), &iters, &relres)) break;
        t_solve = secs(ts);
        rc = PF_SUCCESS;
    } while (0);
    if (ctx) pf_ctx_destroy(&ctx);
    if (rc) return PF_FAILURE;

    FILE *fr = fopen((job + ".res").c_str(), "w");
    if (!fr) { set_error("cannot write %s.res", job.c_str()); return PF_FAILURE; }
    fprintf(fr, "This job ran on %s  processes\n", fmt_I(1, 5).c_str());
    fprintf(fr, "There are %s nodes%s restrained and   %s equations\n", fmt_I(D.nn, 12).c_str(),
            fmt_I(D.nr, 12).c_str(), fmt_I(neq, 12).c_str());
    fprintf(fr, "Time after setup is %s\n", fmt_F(t_setup, 10, 4).c_str());
    fprintf(fr, "The number of iterations to convergence was %s\n", fmt_I(iters, 5).c_str());
    fprintf(fr, "The total load is %s\n", fmt_E(q, 12, 4).c_str());
    fprintf(fr, "The potentials are:\n Freedom       Potential\n");
    for (int i = 0; i < 4; ++i) {
        const int fq = D.nres + i;
        const double v = (fq >= 1 && fq <= neq) ? x[fq - 1] : 0.0;
        fprintf(fr, "%s     %s\n", fmt_I(fq, 8).c_str(), fmt_E(v, 12, 4).c_str());
        if (potentials_out) potentials_out[i] = v;
    }
    fprintf(fr, "Integration, preconditioning and loading took %s\n", fmt_F(t_setup, 10, 4).c_str());
    fprintf(fr, "Time spent in the solver was %s\n", fmt_F(t_solve, 10, 4).c_str());
    // Ensight Gold per-node scalar file (p123.f90:160-173)
    FILE *fe = fopen((job + ".ensi.NDPTL-000001").c_str(), "w");
    if (!fe) { fclose(fr); set_error("cannot write the potential file"); return PF_FAILURE; }
    fprintf(fe, "Alya Ensight Gold --- Scalar per-node variable file\npart\n    1\ncoordinates\n");
    int e = 0;
    for (int nd = 0; nd < D.nn; ++nd) {
        const int eq = fix[(size_t)nd] ? ++e : 0;
        fprintf(fe, "%s\n", fmt_E(eq > 0 ? x[eq - 1] : 0.0, 12, 5).c_str());
    }
    fclose(fe);
    fprintf(fr, "This analysis took %s\n", fmt_F(secs(t0), 10, 4).c_str());
    fclose(fr);
    if (iters_out) *iters_out = iters;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_p123_run");
}

// ===========================================================================
// p122: elastic-plastic (Mohr-Coulomb) solid, 20-node bricks, load control
// (src/programs/5th_ed/p122/p122.f90).

// p12meshgen's p122 case for 20-node bricks (p12meshgen.f90:372-590).
static int p12meshgen_p122(const std::string &job, const std::vector<std::string> &t)
{
    if (t.size() < 20) {
        set_error("%s.mg: the p122 case needs at least 19 values", job.c_str());
        return PF_FAILURE;
    }
    const std::string iotype = t[1];
    const int nels = atoi(t[2].c_str()), nxe = atoi(t[3].c_str()), nze = atoi(t[4].c_str());
    const int nod = atoi(t[5].c_str()), nip = atoi(t[6].c_str());
    const double aa = to_d(t[7]), bb = to_d(t[8]), cc = to_d(t[9]);
    const int incs = atoi(t[10].c_str());
    const double phi = to_d(t[11]), c = to_d(t[12]), psi = to_d(t[13]), e = to_d(t[14]), v = to_d(t[15]);
    const int plasits = atoi(t[16].c_str()), cjits = atoi(t[17].c_str());
    const double plastol = to_d(t[18]), cjtol = to_d(t[19]);
    if (nod != 20 || iotype != "parafem" || nxe < 5 || nze < 1 || nels < 1 || (long long)nxe * nze > nels || nels % (nxe * nze) != 0 || incs < 1 ||
        t.size() < (size_t)20 + incs) {
        set_error("%s.mg: supported: 'parafem' p122 decks of 20-node cubes (nxe >= 5) with incs qinc values",
                  job.c_str());
        return PF_FAILURE;
    }
    const int nye = nels / nxe / nze;
    const long long nn = cube_nn(nxe, nye, nze);
    std::vector<double> gc((size_t)3 * nn, 0.0);
    std::vector<int> gnum((size_t)20 * nels);
    for (int iel = 1; iel <= nels; ++iel) {
        double co[60];
        int *num = &gnum[20 * (size_t)(iel - 1)];
        cube_element(iel, nxe, nze, aa, bb, cc, num, co);
        for (int a = 0; a < 20; ++a)
            for (int d = 0; d < 3; ++d) gc[3 * (size_t)(num[a] - 1) + d] = co[a + 20 * d];
    }
    std::vector<int> fix;
    cube_fix(nxe, nye, nze, 0, fix);
    std::vector<int> lnode;
    std::vector<double> mult;
    load_p121_pattern(nxe / 5, nxe, nze, lnode, mult);
    FILE *fd = fopen((job + ".d").c_str(), "w");
    if (!fd) { set_error("cannot write %s.d", job.c_str()); return PF_FAILURE; }
    fprintf(fd, "*THREE_DIMENSIONAL\n*NODES\n");
    for (long long i = 0; i < nn; ++i)
        fprintf(fd, "%s%s%s%s\n", fmt_I(i + 1, 12).c_str(), fmt_E(gc[3 * i], 14, 6).c_str(),
                fmt_E(gc[3 * i + 1], 14, 6).c_str(), fmt_E(gc[3 * i + 2], 14, 6).c_str());
    fprintf(fd, "*ELEMENTS\n");
    static const int abq[20] = {3, 5, 7, 1, 15, 17, 19, 13, 4, 6, 8, 2, 16, 18, 20, 14, 10, 11, 12, 9};
    for (int iel = 0; iel < nels; ++iel) {
        std::string s = fmt_I(iel + 1, 12) + " 3 20 1 ";
        for (int a = 0; a < 20; ++a) s += fmt_I(gnum[20 * (size_t)iel + abq[a] - 1], 12);
        fprintf(fd, "%s 1\n", s.c_str());
    }
    fclose(fd);
    FILE *fb = fopen((job + ".bnd").c_str(), "w");
    if (!fb) { set_error("cannot write %s.bnd", job.c_str()); return PF_FAILURE; }
    long long nr = 0;
    for (long long i = 0; i < nn; ++i) {
        const int *f = &fix[3 * (size_t)i];
        if (f[0] && f[1] && f[2]) continue;
        fprintf(fb, "%s%s%s%s\n", fmt_I(i + 1, 8).c_str(), fmt_I(f[0], 6).c_str(), fmt_I(f[1], 6).c_str(),
                fmt_I(f[2], 6).c_str());
        ++nr;
    }
    fclose(fb);
    FILE *fl = fopen((job + ".lds").c_str(), "w");
    if (!fl) { set_error("cannot write %s.lds", job.c_str()); return PF_FAILURE; }
    for (size_t i = 0; i < lnode.size(); ++i)
        fprintf(fl, "%s  0.00000000E+00  0.00000000E+00%s\n", fmt_I(lnode[i], 12).c_str(),
                fmt_E(-mult[i] * aa * bb / 12.0, 16, 8).c_str());
    fclose(fl);
    FILE *ft = fopen((job + ".dat").c_str(), "w");
    if (!ft) { set_error("cannot write %s.dat", job.c_str()); return PF_FAILURE; }
    fprintf(ft, "'hexahedron'\n2\n1\n%s%s%s%s%s  0  %s\n", fmt_I(nels, 9).c_str(), fmt_I(nn, 9).c_str(),
            fmt_I(nr, 9).c_str(), fmt_I(nip, 9).c_str(), fmt_I(nod, 9).c_str(),
            fmt_I((long long)lnode.size(), 9).c_str());
    fprintf(ft, "%s%s%s%s%s\n", fmt_E(phi, 12, 4).c_str(), fmt_E(c, 12, 4).c_str(), fmt_E(psi, 12, 4).c_str(),
            fmt_E(e, 12, 4).c_str(), fmt_E(v, 12, 4).c_str());
    fprintf(ft, "%s%s%s%s%s\n", fmt_I(incs, 6).c_str(), fmt_I(plasits, 6).c_str(), fmt_I(cjits, 6).c_str(),
            fmt_E(plastol, 12, 4).c_str(), fmt_E(cjtol, 12, 4).c_str());
    for (int i = 0; i < incs; ++i) fprintf(ft, "%s\n", fmt_E(to_d(t[20 + i]), 12, 4).c_str());
    fclose(ft);
    return PF_SUCCESS;
}

// The p122 job (p122.f90:1-233) with the solve on the GPU: reads job.dat
// (READ_P122, input.f90, and the qinc values that follow), .d (20-node or
// 8-node hexahedra), .bnd, .lds (loaded nodes) and .fix (fixed freedoms:
// node, sense, value; READ_FIXED, input.f90:2483-2564); writes job.res and
// job.ensi.DISPL-0000nn for every increment.
extern "C" int pf_p122_run(const char *job_c, const int *device, int *incs_out)
try {
    if (!job_c || !device) { set_error("pf_p122_run: null argument"); return PF_FAILURE; }
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    auto secs = [&](clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); };
    const std::string job(job_c);
    std::vector<std::string> t;
    if (!read_tokens(job + ".dat", t) || t.size() < 21) {
        set_error("cannot read %s.dat", job.c_str());
        return PF_FAILURE;
    }
    // element, mesh, partition, nels, nn, nr, nip, nod, fixed, loaded, phi, c, psi, e, v,
    // incs, plasits, cjits, plastol, cjtol, qinc(incs)
    Deck D;
    D.element = t[0];
    D.meshgen = atoi(t[1].c_str());
    D.partitioner = atoi(t[2].c_str());
    D.nels = atoi(t[3].c_str());
    D.nn = atoi(t[4].c_str());
    D.nr = atoi(t[5].c_str());
    D.nip = atoi(t[6].c_str());
    D.nod = atoi(t[7].c_str());
    const int fixed = atoi(t[8].c_str());
    D.loaded = atoi(t[9].c_str());
    const double phi = to_d(t[10]), coh = to_d(t[11]), psi = to_d(t[12]);
    D.e = to_d(t[13]);
    D.v = to_d(t[14]);
    const int incs = atoi(t[15].c_str()), plasits = atoi(t[16].c_str()), cjits = atoi(t[17].c_str());
    const double plastol = to_d(t[18]), cjtol = to_d(t[19]);
    if (D.element != "hexahedron" || (D.nod != 20 && D.nod != 8) || fixed < 0 || (fixed > 0 && D.nod != 8) ||
        (fixed == 0 && D.loaded <= 0) || incs < 1 || t.size() < (size_t)20 + incs) {
        set_error("%s.dat: p122 decks of 20-node hexahedra under load control or 8-node hexahedra under load or "
                  "displacement control (nod=%d, fixed freedoms %d, loaded nodes %d)",
                  job.c_str(), D.nod, fixed, D.loaded);
        return PF_FAILURE;
    }
    std::vector<double> qinc(incs);
    for (int i = 0; i < incs; ++i) qinc[i] = to_d(t[20 + i]);
    if (read_mesh_files(job, D)) return PF_FAILURE;
    std::vector<int> fix;
    if (rest_to_fix(D.nn, D.nr, D.rest.data(), fix)) return PF_FAILURE;
    // equations in node order over the free freedoms (find_g, new_library.f90:3218-3243)
    std::vector<int> node_eq;
    const int neq = number_nodes(D.nn, fix.data(), node_eq);
    const int nod = D.nod, ne = 3 * nod;
    std::vector<int> g_g((size_t)ne * D.nels);
    std::vector<double> gcoord((size_t)ne * D.nels);
    for (size_t e = 0; e < (size_t)D.nels; ++e)
        for (int a = 0; a < nod; ++a) {
            const int nd = D.g_num[nod * e + a];
            if (nd < 1 || nd > D.nn) {
                set_error("%s.d: element %zu names node %d outside 1..%d", job.c_str(), e + 1, nd, D.nn);
                return PF_FAILURE;
            }
            for (int d = 0; d < 3; ++d) {
                g_g[ne * e + 3 * a + d] = node_eq[(size_t)(nd - 1) * 3 + d];
                gcoord[ne * e + a + nod * d] = D.coords[3 * (size_t)(nd - 1) + d];
            }
        }
    // fixed freedoms: the equation of freedom `sense` of each node (find_no)
    std::vector<int> fix_eq(fixed > 0 ? fixed : 1);
    std::vector<double> fix_val(fixed > 0 ? fixed : 1);
    if (fixed > 0) {
        std::vector<std::string> tf;
        if (!read_tokens(job + ".fix", tf) || tf.size() < (size_t)3 * fixed) {
            set_error("cannot read %d fixed freedoms from %s.fix", fixed, job.c_str());
            return PF_FAILURE;
        }
        for (int i = 0; i < fixed; ++i) {
            const int nd = atoi(tf[3 * (size_t)i].c_str()), sense = atoi(tf[3 * (size_t)i + 1].c_str());
            if (nd < 1 || nd > D.nn || sense < 1 || sense > 3 || node_eq[(size_t)(nd - 1) * 3 + sense - 1] == 0) {
                set_error("%s.fix: line %d: node %d freedom %d is not a free freedom", job.c_str(), i + 1, nd,
                          sense);
                return PF_FAILURE;
            }
            fix_eq[i] = node_eq[(size_t)(nd - 1) * 3 + sense - 1];
            fix_val[i] = to_d(tf[3 * (size_t)i + 2]);
        }
    }
    std::vector<double> ld0(neq > 0 ? neq : 1, 0.0);
    {   // LOAD + SCATTER_NOADD (loading.f90:36-146): assignment, the last node entry wins
        std::vector<int> node_slot((size_t)D.nn + 1, -1);
        for (int i = 0; i < D.loaded; ++i)
            if (D.lnode[i] >= 1 && D.lnode[i] <= D.nn) node_slot[D.lnode[i]] = i;
        for (int nd = 1; nd <= D.nn; ++nd) {
            const int i = node_slot[nd];
            if (i < 0) continue;
            for (int d = 0; d < 3; ++d) {
                const int eq = node_eq[(size_t)(nd - 1) * 3 + d];
                if (eq > 0) ld0[eq - 1] = D.lval[3 * (size_t)i + d];
            }
        }
    }
    void *ctx = nullptr;
    int rc = PF_FAILURE, done = 0, one = 1, flags = 0;
    std::vector<double> res((size_t)6 * incs, 0.0), totd((size_t)(neq > 0 ? neq : 1) * incs, 0.0);
    double t_setup = 0.0;
    do {
        if (pf_ctx_create(device, &ctx)) break;
        int nq = neq;
        if (nod == 8 ? pf_setup_solid8(&ctx, &D.nels, &D.nn, &nq, D.g_num.data(), g_g.data(), gcoord.data())
                     : pf_setup(&ctx, &D.nels, &D.nn, &nq, D.g_num.data(), g_g.data(), gcoord.data()))
            break;
        if (pf_set_material(&ctx, &one, &D.e, &D.v)) break;
        if (pf_form_storkm(&ctx, &D.nip, &flags)) break;
        t_setup = secs(t0);
        int incs_i = incs;
        if (pf_p122_solve_fixed(&ctx, &D.nip, &phi, &coh, &psi, &incs_i, qinc.data(), &plasits, &cjits, &plastol,
                                &cjtol, D.loaded > 0 ? ld0.data() : nullptr, &fixed, fix_eq.data(), fix_val.data(),
                                res.data(), totd.data(), &done))
            break;
        rc = PF_SUCCESS;
    } while (0);
    if (ctx) pf_ctx_destroy(&ctx);
    if (rc) return PF_FAILURE;
    const double pi = std::acos(-1.0), snph = std::sin(phi * pi / 180.0);
    const double dt = 4.0 * (1.0 + D.v) * (1.0 - 2.0 * D.v) / (D.e * (1.0 - 2.0 * D.v + snph * snph));
    FILE *fr = fopen((job + ".res").c_str(), "w");
    if (!fr) { set_error("cannot write %s.res", job.c_str()); return PF_FAILURE; }
    fprintf(fr, "This job ran on %s  processes\n", fmt_I(1, 5).c_str());
    fprintf(fr, "There are %s nodes%s restrained and   %s equations\n", fmt_I(D.nn, 7).c_str(),
            fmt_I(D.nr, 7).c_str(), fmt_I(neq, 7).c_str());
    fprintf(fr, "Time after setup is:%s\n", fmt_F(t_setup, 10, 4).c_str());
    fprintf(fr, "The critical timestep is   %s\n", fmt_E(dt, 12, 4).c_str());
    for (int iy = 1; iy <= done; ++iy) {
        const double *o = &res[6 * (size_t)(iy - 1)];
        fprintf(fr, "\nLoad Increment   %s\n", fmt_I(iy, 5).c_str());
        fprintf(fr, "The displacement is  %s\n", fmt_E(o[0], 12, 4).c_str());
        fprintf(fr, "  sigma z    sigma x     sigma y\n%s%s%s\n", fmt_E(o[1], 12, 4).c_str(),
                fmt_E(o[2], 12, 4).c_str(), fmt_E(o[3], 12, 4).c_str());
        fprintf(fr, "The total number of cj iterations was  %s\n", fmt_I((long long)o[4], 12).c_str());
        fprintf(fr, "The number of plastic iterations was  %s\n", fmt_I((long long)o[5], 12).c_str());
        fprintf(fr, "cj iterations per plastic iteration were %s\n", fmt_F(o[4] / o[5], 11, 2).c_str());
        char name[64];
        snprintf(name, sizeof name, ".ensi.DISPL-%06d", iy);
        FILE *fe = fopen((job + name).c_str(), "w");
        if (!fe) { fclose(fr); set_error("cannot write the displacement file"); return PF_FAILURE; }
        fprintf(fe, "Alya Ensight Gold --- Vector per-node variable file\npart\n    1\ncoordinates\n");
        const double *x = &totd[(size_t)neq * (iy - 1)];
        for (int d = 0; d < 3; ++d)
            for (int nd = 0; nd < D.nn; ++nd) {
                const int eq = node_eq[(size_t)nd * 3 + d];
                fprintf(fe, "%s\n", fmt_E(eq > 0 ? x[eq - 1] : 0.0, 12, 5).c_str());
            }
        fclose(fe);
    }
    fprintf(fr, "This analysis took: %s\n", fmt_F(secs(t0), 10, 4).c_str());
    fclose(fr);
    if (incs_out) *incs_out = done;
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_p122_run");
}
