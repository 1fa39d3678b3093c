/*
 * slvof_oracle.cpp — TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
 *
 * CPU restatement of Mist.jl's semi-Lagrangian geometric VOF transport path, written from
 * the reference's Julia source: ELVIRA normals, PLIC plane-distance solve, PLIC->VF clip,
 * band gate, single-rank ghost fill, backward RK tracing of cell vertices, the recursive
 * mesh/PLIC tet clip and the SL cell update.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load this library, and only as the checker.
 *
 * Pinning.  The PLIC distance solve and the PLIC->VF clip are pinned to the reference's own
 * tests: the known answers of test/test_PLIC_dist.jl:41-51 and the 1e-12 round trip of
 * test/runtests.jl:32-45 + test/test_PLIC_dist_cutting.jl:35-49.  ELVIRA, the RK
 * projection, cutTet and the full step have no reference fixture (the reference is Julia and
 * Julia is not installed), so for those this restatement is "parity unpinned" by the
 * reference and is checked against analytic invariants in tests/ instead (exact
 * reconstruction of planar interfaces, exact transport of a plane by a uniform velocity,
 * pre-image volume of divergence-free linear flows).
 *
 * Arithmetic.  Every expression keeps the reference's operation order (Julia evaluates
 * a+b+c as (a+b)+c, x^2 as x*x, x^3 as x*x*x, and never contracts to FMA).  Build with
 * -ffp-contract=off.  cbrt/acos/sin/cos come from the package's deterministic math header
 * (csrc/detmath.h) so that this file and the FP64 CUDA path round identically.
 *
 * Indices are the reference's Julia indices: interior cells 1..N, ghost cells 1-g..0 and
 * N+1..N+g (g = mesh.nghost), and VF carries three more ghost layers (src/Tools.jl:144).
 * Arrays are the OffsetArray parents, column-major with i fastest.
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>

#include "detmath.h"

extern "C" {
typedef struct orc_mesh {
    int32_t Nx, Ny, Nz;      /* global = local interior cells (single rank) */
    int32_t nghost;          /* src/Mesh.jl:66 */
    int32_t nband;           /* src/Parameters.jl:70 */
    int32_t projection;      /* 0 Euler, 1 Midpoint, 2 RK4 (src/Tools.jl:392-418) */
    int32_t xper, yper, zper;
    double Lx, Ly, Lz, dx, dy, dz;
    double VFlo, VFhi, rho_liq, rho_gas;
    const double *x, *y, *z;    /* faces, index 1-g .. N+g+1 */
    const double *xm, *ym, *zm; /* centres, index 1-g .. N+g */
    int32_t tesselation;        /* 5, 6 or 24 (0 means 5): param.tesselation, src/Parameters.jl:77 */
    int32_t pressure_scheme;    /* 0 "semi-lagrangian", 1 "finite-difference": param.pressure_scheme */
} orc_mesh;
}

namespace {

const double EPS = 2.220446049250313e-16; /* Julia eps() */

/* Forward-mode dual numbers for the derivative checks: the SL path, ELVIRA and the plane-
 * constant solve below are written for a generic scalar, instantiated with double (the
 * restatement), with Dual (value plus K directional derivatives, the CPU analogue of
 * ForwardDiff.jl's Dual; orc_sl_forward, orc_rollout_forward) and with Cnt (the operation
 * count, orc_count_ops).  Branches and comparisons use the value; the double instantiation is
 * the plain restatement. */
constexpr int NDUAL = 16;
struct Dual {
    double v = 0.0;
    double d[NDUAL] = {};
    Dual() = default;
    Dual(double x) : v(x) {}
};
inline Dual operator+(const Dual& a, const Dual& b) { Dual r(a.v + b.v); for (int q = 0; q < NDUAL; ++q) r.d[q] = a.d[q] + b.d[q]; return r; }
inline Dual operator-(const Dual& a, const Dual& b) { Dual r(a.v - b.v); for (int q = 0; q < NDUAL; ++q) r.d[q] = a.d[q] - b.d[q]; return r; }
inline Dual operator-(const Dual& a) { Dual r(-a.v); for (int q = 0; q < NDUAL; ++q) r.d[q] = -a.d[q]; return r; }
inline Dual operator*(const Dual& a, const Dual& b)
{
    Dual r(a.v * b.v);
    for (int q = 0; q < NDUAL; ++q) r.d[q] = a.d[q] * b.v + a.v * b.d[q];
    return r;
}
inline Dual operator/(const Dual& a, const Dual& b)
{
    Dual r(a.v / b.v);
    for (int q = 0; q < NDUAL; ++q) r.d[q] = (a.d[q] * b.v - a.v * b.d[q]) / (b.v * b.v);
    return r;
}
inline Dual& operator+=(Dual& a, const Dual& b) { a = a + b; return a; }
inline double val(double x) { return x; }
inline double val(const Dual& x) { return x.v; }

/* Operation counter for the algorithmic FLOP count of a step: the ELVIRA, plane-constant and
 * SL paths below are also instantiated with Cnt, a double that counts each +, -, *, / and
 * each sqrt, cbrt, acos, sin, cos it takes part in.  Negation, comparisons, min/max and fabs
 * are not counted, nor are expressions of mesh constants alone (they stay double).  The
 * counter is global: count on one thread. */
unsigned long long g_nops = 0;
struct Cnt {
    double v;
    Cnt() : v(0.0) {}
    Cnt(double x) : v(x) {}
};
inline Cnt operator+(const Cnt& a, const Cnt& b) { ++g_nops; return Cnt(a.v + b.v); }
inline Cnt operator-(const Cnt& a, const Cnt& b) { ++g_nops; return Cnt(a.v - b.v); }
inline Cnt operator*(const Cnt& a, const Cnt& b) { ++g_nops; return Cnt(a.v * b.v); }
inline Cnt operator/(const Cnt& a, const Cnt& b) { ++g_nops; return Cnt(a.v / b.v); }
inline Cnt operator-(const Cnt& a) { return Cnt(-a.v); }
inline Cnt& operator+=(Cnt& a, const Cnt& b) { a = a + b; return a; }
inline Cnt& operator-=(Cnt& a, const Cnt& b) { a = a - b; return a; }
inline bool operator<(const Cnt& a, const Cnt& b) { return a.v < b.v; }
inline bool operator>(const Cnt& a, const Cnt& b) { return a.v > b.v; }
inline bool operator<=(const Cnt& a, const Cnt& b) { return a.v <= b.v; }
inline bool operator>=(const Cnt& a, const Cnt& b) { return a.v >= b.v; }
inline double val(const Cnt& x) { return x.v; }

/* Math functions of the generic paths: the restatement's own for double, counted for Cnt. */
inline double f_sqrt(double x) { return std::sqrt(x); }
inline double f_cbrt(double x) { return detm_cbrt(x); }
inline double f_acos(double x) { return detm_acos(x); }
inline double f_sin(double x) { return detm_sin(x); }
inline double f_cos(double x) { return detm_cos(x); }
inline double f_abs(double x) { return std::fabs(x); }
inline Cnt f_sqrt(const Cnt& x) { ++g_nops; return Cnt(std::sqrt(x.v)); }
inline Cnt f_cbrt(const Cnt& x) { ++g_nops; return Cnt(detm_cbrt(x.v)); }
inline Cnt f_acos(const Cnt& x) { ++g_nops; return Cnt(detm_acos(x.v)); }
inline Cnt f_sin(const Cnt& x) { ++g_nops; return Cnt(detm_sin(x.v)); }
inline Cnt f_cos(const Cnt& x) { ++g_nops; return Cnt(detm_cos(x.v)); }
inline Cnt f_abs(const Cnt& x) { return Cnt(std::fabs(x.v)); }

/* The same for Dual: comparisons on the value, derivatives of the math functions. */
inline Dual& operator-=(Dual& a, const Dual& b) { a = a - b; return a; }
inline bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
inline bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
inline bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
inline bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
inline Dual dual_chain(double v, const Dual& a, double dv)
{
    Dual r(v);
    for (int q = 0; q < NDUAL; ++q) r.d[q] = a.d[q] * dv;
    return r;
}
inline Dual f_sqrt(const Dual& x) { const double v = std::sqrt(x.v); return dual_chain(v, x, 0.5 / v); }
inline Dual f_cbrt(const Dual& x) { const double v = detm_cbrt(x.v); return dual_chain(v, x, 1.0 / (3.0 * v * v)); }
inline Dual f_acos(const Dual& x) { return dual_chain(detm_acos(x.v), x, -1.0 / std::sqrt(1.0 - x.v * x.v)); }
inline Dual f_sin(const Dual& x) { return dual_chain(detm_sin(x.v), x, detm_cos(x.v)); }
inline Dual f_cos(const Dual& x) { return dual_chain(detm_cos(x.v), x, -detm_sin(x.v)); }
inline Dual f_abs(const Dual& x) { return x.v < 0.0 ? -x : x; }

/* Result stores of the generic paths. */
inline void store(double& o, double x) { o = x; }
inline void store(double& o, const Cnt& x) { o = x.v; }
inline void store(Dual& o, const Dual& x) { o = x; }

/* Julia min/max on Float64: NaN-propagating. */
template <class R>
inline R jmax(const R& a, const R& b)
{
    const double x = val(a), y = val(b);
    return (x != x || y != y) ? R(NAN) : (x > y ? a : (y > x ? b : (std::signbit(x) ? b : a)));
}
template <class R>
inline R jmin(const R& a, const R& b)
{
    const double x = val(a), y = val(b);
    return (x != x || y != y) ? R(NAN) : (x < y ? a : (y < x ? b : (std::signbit(x) ? a : b)));
}

/* /̂  (src/Tools.jl:375-377) */
template <class R>
inline R sdiv(const R& a, const R& b) { return std::fabs(val(b)) <= EPS ? R(INFINITY) : a / b; }

struct Grid {
    const orc_mesh* m;
    int g, N[3];
    int lo[3], hi[3];   /* cell arrays imino_..imaxo_ */
    int vlo[3], vhi[3]; /* VF array */
    long n[3], vn[3];
    int tess;
    explicit Grid(const orc_mesh* mm) : m(mm)
    {
        tess = mm->tesselation == 0 ? 5 : mm->tesselation;
        g = mm->nghost;
        N[0] = mm->Nx; N[1] = mm->Ny; N[2] = mm->Nz;
        for (int d = 0; d < 3; ++d) {
            lo[d] = 1 - g; hi[d] = N[d] + g; n[d] = hi[d] - lo[d] + 1;
            vlo[d] = lo[d] - 3; vhi[d] = hi[d] + 3; vn[d] = vhi[d] - vlo[d] + 1;
        }
    }
    long c(int i, int j, int k) const { return (i - lo[0]) + n[0] * ((j - lo[1]) + n[1] * (long)(k - lo[2])); }
    long v(int i, int j, int k) const { return (i - vlo[0]) + vn[0] * ((j - vlo[1]) + vn[1] * (long)(k - vlo[2])); }
    double x(int i) const { return m->x[i - lo[0]]; }
    double y(int j) const { return m->y[j - lo[1]]; }
    double z(int k) const { return m->z[k - lo[2]]; }
    double xm(int i) const { return m->xm[i - lo[0]]; }
    double ym(int j) const { return m->ym[j - lo[1]]; }
    double zm(int k) const { return m->zm[k - lo[2]]; }
    double fc(int d, int i) const { return d == 0 ? x(i) : (d == 1 ? y(i) : z(i)); }
};

/* ---------------------------------------------------------------------------------------
 * Cut tables, src/VFgeom.jl:55-165, kept in the reference's 1-based layout:
 * T_V1[case-1][n-1] == cut_v1[n,case], T_VTET[case-1][n-1][t-1] == cut_vtet[t,n,case],
 * T_SIDE[case-1][n-1] == cut_side[n,case].
 * ------------------------------------------------------------------------------------- */
const int T_NVERT[16] = {0, 3, 3, 4, 3, 4, 4, 3, 3, 4, 4, 3, 4, 3, 3, 0};
const int T_NTETS[16] = {1, 4, 4, 6, 4, 6, 6, 4, 4, 6, 6, 4, 6, 4, 4, 1};
const int T_NNTET[16] = {1, 2, 2, 4, 2, 4, 4, 4, 2, 4, 4, 4, 4, 4, 4, 2};
const int T_V1[16][4] = {
    {-1, -1, -1, -1}, {1, 1, 1, -1}, {2, 2, 2, -1}, {1, 2, 1, 2}, {3, 3, 3, -1}, {1, 3, 1, 3},
    {2, 3, 2, 3},     {4, 4, 4, -1}, {4, 4, 4, -1}, {1, 4, 1, 4}, {2, 4, 2, 4}, {3, 3, 3, -1},
    {3, 4, 3, 4},     {2, 2, 2, -1}, {1, 1, 1, -1}, {-1, -1, -1, -1}};
const int T_V2[16][4] = {
    {-1, -1, -1, -1}, {2, 3, 4, -1}, {3, 4, 1, -1}, {4, 4, 3, 3}, {4, 1, 2, -1}, {4, 4, 2, 2},
    {4, 4, 1, 1},     {1, 2, 3, -1}, {1, 2, 3, -1}, {3, 3, 2, 2}, {3, 3, 1, 1}, {4, 1, 2, -1},
    {2, 2, 1, 1},     {3, 4, 1, -1}, {2, 3, 4, -1}, {-1, -1, -1, -1}};
const int T_VTET[16][6][4] = {
    {{1, 2, 3, 4}, {-1, -1, -1, -1}, {-1, -1, -1, -1}, {-1, -1, -1, -1}, {-1, -1, -1, -1}, {-1, -1, -1, -1}},
    {{5, 7, 6, 1}, {6, 2, 3, 4}, {4, 2, 5, 6}, {5, 6, 7, 4}, {-1, -1, -1, -1}, {-1, -1, -1, -1}},
    {{7, 5, 6, 2}, {1, 3, 4, 6}, {1, 5, 3, 6}, {5, 7, 6, 1}, {-1, -1, -1, -1}, {-1, -1, -1, -1}},
    {{5, 8, 6, 2}, {5, 7, 8, 1}, {5, 1, 8, 2}, {5, 6, 8, 4}, {5, 8, 7, 3}, {5, 8, 3, 4}},
    {{6, 5, 7, 3}, {2, 1, 4, 6}, {6, 5, 4, 2}, {6, 7, 5, 2}, {-1, -1, -1, -1}, {-1, -1, -1, -1}},
    {{5, 6, 8, 3}, {5, 8, 7, 1}, {5, 8, 1, 3}, {5, 8, 6, 4}, {5, 7, 8, 2}, {5, 8, 4, 2}},
    {{8, 6, 5, 3}, {5, 7, 8, 2}, {8, 5, 2, 3}, {8, 5, 6, 4}, {5, 8, 7, 1}, {5, 8, 1, 4}},
    {{1, 2, 3, 7}, {1, 2, 7, 6}, {5, 7, 6, 1}, {5, 6, 7, 4}, {-1, -1, -1, -1}, {-1, -1, -1, -1}},
    {{5, 6, 7, 4}, {1, 2, 3, 6}, {5, 1, 3, 6}, {5, 7, 6, 3}, {-1, -1, -1, -1}, {-1, -1, -1, -1}},
    {{5, 8, 6, 4}, {5, 7, 8, 1}, {5, 8, 4, 1}, {5, 6, 8, 3}, {5, 8, 7, 2}, {5, 8, 2, 3}},
    {{8, 5, 6, 4}, {5, 8, 7, 2}, {8, 2, 5, 4}, {8, 6, 5, 3}, {5, 7, 8, 1}, {5, 8, 3, 1}},
    {{1, 4, 2, 7}, {4, 1, 6, 7}, {6, 7, 5, 4}, {6, 5, 7, 3}, {-1, -1, -1, -1}, {-1, -1, -1, -1}},
    {{8, 6, 5, 4}, {5, 7, 8, 3}, {8, 4, 5, 3}, {8, 5, 6, 2}, {5, 8, 7, 1}, {5, 8, 1, 2}},
    {{3, 4, 1, 7}, {7, 6, 3, 4}, {7, 6, 5, 3}, {7, 5, 6, 2}, {-1, -1, -1, -1}, {-1, -1, -1, -1}},
    {{7, 4, 2, 3}, {2, 3, 6, 7}, {5, 6, 7, 2}, {5, 7, 6, 1}, {-1, -1, -1, -1}, {-1, -1, -1, -1}},
    {{1, 2, 3, 4}, {-1, -1, -1, -1}, {-1, -1, -1, -1}, {-1, -1, -1, -1}, {-1, -1, -1, -1}, {-1, -1, -1, -1}}};
const int T_SIDE[16][6] = {
    {1, -1, -1, -1, -1, -1}, {2, 1, 1, 1, -1, -1}, {2, 1, 1, 1, -1, -1}, {2, 2, 2, 1, 1, 1},
    {2, 1, 1, 1, -1, -1},    {2, 2, 2, 1, 1, 1},   {2, 2, 2, 1, 1, 1},   {2, 2, 2, 1, -1, -1},
    {2, 1, 1, 1, -1, -1},    {2, 2, 2, 1, 1, 1},   {2, 2, 2, 1, 1, 1},   {2, 2, 2, 1, -1, -1},
    {2, 2, 2, 1, 1, 1},      {2, 2, 2, 1, -1, -1}, {2, 2, 2, 1, -1, -1}, {2, -1, -1, -1, -1, -1}};

/* 5-tet decomposition of the 8 cell vertices, src/VFgeom.jl:235-256 (1-based vertex ids). */
const int TET5[5][4] = {{1, 2, 4, 6}, {1, 4, 3, 7}, {1, 5, 6, 7}, {4, 7, 6, 8}, {1, 4, 7, 6}};
/* 6_tets, src/VFgeom.jl:257-282 (1-based vertex ids). */
const int TET6[6][4] = {{5, 6, 4, 8}, {5, 6, 2, 4}, {5, 2, 1, 4}, {7, 8, 5, 4}, {3, 4, 7, 5}, {1, 4, 3, 5}};
/* 24_tets, src/VFgeom.jl:283-330: per face (vertex ids in the order of `vts`, 1-based), four
 * tets (v4, v1, f, m), (v1, v2, f, m), (v2, v3, f, m), (v3, v4, f, m) with f the face's mean
 * point and m the cell's mean point. */
const int FACE24[6][4] = {{1, 3, 7, 5}, {2, 6, 8, 4}, {1, 5, 6, 2}, {3, 4, 8, 7}, {1, 2, 4, 3}, {5, 7, 8, 6}};

/* Points of a cell's tessellation, 0-based: 0..7 the vertices (cell2verts! order), 8 the mean
 * of the vertices, 9..14 the means of the six faces (24_tets only).  Tet t of a tessellation
 * as four point ids. */
inline int tess_ntets(int tess) { return tess == 6 ? 6 : (tess == 24 ? 24 : 5); }
inline void tess_tet(int tess, int t, int out[4])
{
    if (tess == 6) {
        for (int n = 0; n < 4; ++n) out[n] = TET6[t][n] - 1;
    } else if (tess == 24) {
        const int f = t / 4, q = t % 4;
        const int* v = FACE24[f];
        const int a = q == 0 ? v[3] : v[q - 1], b = q == 0 ? v[0] : v[q];
        out[0] = a - 1; out[1] = b - 1; out[2] = 9 + f; out[3] = 8;
    } else {
        for (int n = 0; n < 4; ++n) out[n] = TET5[t][n] - 1;
    }
}
/* mean(eachcol(p)) as Julia's Statistics.mean computes it: the vectors summed in order, then
 * divided by their count. */
template <class R>
inline void tess_points(int tess, R pts[15][3])
{
    if (tess != 24) return;
    for (int p = 0; p < 3; ++p) {
        R s = pts[0][p];
        for (int n = 1; n < 8; ++n) s = s + pts[n][p];
        pts[8][p] = s / 8.0;
    }
    for (int f = 0; f < 6; ++f)
        for (int p = 0; p < 3; ++p) {
            R s = pts[FACE24[f][0] - 1][p];
            for (int n = 1; n < 4; ++n) s = s + pts[FACE24[f][n] - 1][p];
            pts[9 + f][p] = s / 4.0;
        }
}
inline int tess_npoints(int tess) { return tess == 24 ? 15 : 8; }

struct Err { int flags = 0; };
enum { E_INDEX = 1, E_DEPTH = 2, E_NAN = 4, E_VOLUME = 8 };

/* tet_vol, src/VFgeom.jl:669-681.  v[vertex][coord]. */
template <class R>
inline R tet_vol(const R v[4][3])
{
    const R a1 = v[0][0] - v[3][0], a2 = v[0][1] - v[3][1], a3 = v[0][2] - v[3][2];
    const R b1 = v[1][0] - v[3][0], b2 = v[1][1] - v[3][1], b3 = v[1][2] - v[3][2];
    const R c1 = v[2][0] - v[3][0], c2 = v[2][1] - v[3][1], c3 = v[2][2] - v[3][2];
    return R(-1.0 / 6.0) * ((a1 * (b2 * c3 - c2 * b3) - a2 * (b1 * c3 - c1 * b3)) + a3 * (b1 * c2 - c1 * b2));
}

/* d2case, src/VFgeom.jl:693-708.  Modifies d (callers pass a copy where the reference does). */
inline int d2case(double d[4], Err* err)
{
    int npos = 0, nneg = 0;
    for (int n = 0; n < 4; ++n) { npos += d[n] > 0.0; nneg += d[n] < 0.0; }
    for (int n = 0; n < 4; ++n)
        if (std::fabs(d[n]) < EPS) d[n] = npos > nneg ? EPS : -EPS;
    int c = 1;
    for (int n = 0; n < 4; ++n) {
        if (d[n] != d[n]) { if (err) err->flags |= E_NAN; continue; }
        c += (1 << n) * (d[n] > 0.0 ? 1 : 0);
    }
    return c;
}

template <class R>
inline R clamp_mu(const R& q) { return jmin(R(1.0), jmax(R(0.0), q)); }

/* oddEvenCell + cell2verts!, src/VFgeom.jl:171-216: only 5_tets mirrors odd cells.
 * verts[vertex][coord]. */
double cell2verts(const Grid& G, int i, int j, int k, double verts[][3])
{
    const bool even = G.tess != 5 || ((i + j + k) % 2) == 0;
    const int ia = even ? i : i + 1, ib = even ? i + 1 : i;
    const double xs[2] = {G.x(ia), G.x(ib)};
    const double ys[2] = {G.y(j), G.y(j + 1)};
    const double zs[2] = {G.z(k), G.z(k + 1)};
    for (int c = 0; c < 2; ++c)
        for (int b = 0; b < 2; ++b)
            for (int a = 0; a < 2; ++a) {
                double* p = verts[a + 2 * b + 4 * c];
                p[0] = xs[a]; p[1] = ys[b]; p[2] = zs[c];
            }
    return even ? 1.0 : -1.0;
}

/* computeAlpha, src/VF.jl:164-214. */
template <class R>
R compute_alpha(const R min[3], R VF)
{
    R m[3] = {min[0], min[1], min[2]};
    std::sort(m, m + 3, [](const R& a, const R& b) { return val(a) < val(b); });
    const R m1 = m[0], m2 = m[1], m3 = m[2];
    const R m12 = m[0] + m[1];
    const R V1 = m[0] * m[0] / jmax(R(6.0) * m[1] * m[2], R(EPS));
    const R V2 = V1 + sdiv(R(0.5) * (m[1] - m[0]), m3);
    R V3;
    if (m12 <= m[2]) V3 = sdiv(R(0.5) * m12, m3);
    else V3 = sdiv((m3 * m3 * (R(3.0) * m12 - m3) + m1 * m1 * (m1 - R(3.0) * m3)) + m2 * m2 * (m2 - R(3.0) * m3),
                   R(6.0) * m1 * m2 * m3);
    R alpha;
    if (R(0.0) <= VF && VF < V1) {
        alpha = f_cbrt(R(6.0) * m1 * m2 * m3 * VF);
    } else if (V1 <= VF && VF < V2) {
        alpha = R(0.5) * (m1 + f_sqrt(m1 * m1 + R(8.0) * m2 * m3 * (VF - V1)));
    } else if (V2 <= VF && VF < V3) {
        R a0 = (m1 * m1 * m1 + m2 * m2 * m2) - R(6.0) * m1 * m2 * m3 * VF;
        R a1 = R(-3.0) * (m1 * m1 + m2 * m2);
        R a2 = R(3.0) * m12;
        R a3 = R(-1.0);
        a0 = a0 / a3; a1 = a1 / a3; a2 = a2 / a3; a3 = a3 / a3;
        const R p0 = a1 / R(3.0) - a2 * a2 / R(9.0);
        const R q0 = (a1 * a2 - R(3.0) * a0) / R(6.0) - a2 * a2 * a2 / R(27.0);
        const R theta = f_acos(jmin(R(1.0), jmax(R(-1.0), q0 / f_sqrt(R(-1.0) * (p0 * p0 * p0))))) / R(3.0);
        alpha = f_sqrt(-p0) * (R(std::sqrt(3.0)) * f_sin(theta) - f_cos(theta)) - a2 / R(3.0);
    } else {
        if (m12 <= m3) {
            alpha = m3 * VF + R(0.5) * m12;
        } else {
            R a0 = ((m1 * m1 * m1 + m2 * m2 * m2) + m3 * m3 * m3) - R(6.0) * m1 * m2 * m3 * VF;
            R a1 = R(-3.0) * ((m1 * m1 + m2 * m2) + m3 * m3);
            R a2 = R(3.0);
            R a3 = R(-2.0);
            a0 = a0 / a3; a1 = a1 / a3; a2 = a2 / a3; a3 = a3 / a3;
            const R p0 = a1 / R(3.0) - a2 * a2 / R(9.0);
            const R q0 = (a1 * a2 - R(3.0) * a0) / R(6.0) - a2 * a2 * a2 / R(27.0);
            const R theta = f_acos(jmin(R(1.0), jmax(R(-1.0), q0 / f_sqrt(-(p0 * p0 * p0))))) / R(3.0);
            alpha = f_sqrt(-p0) * (R(std::sqrt(3.0)) * f_sin(theta) - f_cos(theta)) - a2 / R(3.0);
        }
    }
    return alpha;
}

/* computeDist, src/VF.jl:109-156. */
template <class R>
R compute_dist(const Grid& G, int i, int j, int k, R nx, R ny, R nz, R VF)
{
    const orc_mesh* M = G.m;
    if (VF < M->VFlo) return R(-((M->Lx + M->Ly) + M->Lz));
    if (VF > M->VFhi) return R(+((M->Lx + M->Ly) + M->Lz));
    R mm[3] = {nx * M->dx, ny * M->dy, nz * M->dz};
    const R norm = ((f_abs(mm[0]) + f_abs(mm[1])) + f_abs(mm[2])) + R(EPS);
    mm[0] = mm[0] / norm; mm[1] = mm[1] / norm; mm[2] = mm[2] / norm;
    R factor(0.0);
    if (mm[0] < 0.0) factor += mm[0];
    if (mm[1] < 0.0) factor += mm[1];
    if (mm[2] < 0.0) factor += mm[2];
    const R VFo = VF > 0.5 ? R(1.0) - VF : VF;
    const R am[3] = {f_abs(mm[0]), f_abs(mm[1]), f_abs(mm[2])};
    R alpha = compute_alpha(am, VFo);
    alpha = VF > 0.5 ? R(1.0) - alpha : alpha;
    alpha += factor;
    alpha -= R(0.5) * ((mm[0] + mm[1]) + mm[2]);
    R dist = alpha * norm;
    dist += (nx * G.xm(i) + ny * G.ym(j)) + nz * G.zm(k);
    return dist;
}

/* computePLIC2VF, src/VF.jl:219-278 (5_tets).  d2case modifies d in place here. */
template <class R>
R compute_plic2vf(const Grid& G, int i, int j, int k, R nx, R ny, R nz, R dist, Err* err)
{
    const orc_mesh* M = G.m;
    double verts[15][3];
    const double tetsign = cell2verts(G, i, j, k, verts);
    tess_points(G.tess, verts);
    R VF(0.0);
    for (int t = 0; t < tess_ntets(G.tess); ++t) {
        R vert[8][3];
        int tv[4];
        tess_tet(G.tess, t, tv);
        for (int n = 0; n < 4; ++n)
            for (int p = 0; p < 3; ++p) vert[n][p] = verts[tv[n]][p];
        R d[4];
        for (int n = 0; n < 4; ++n) d[n] = ((nx * vert[n][0] + ny * vert[n][1]) + nz * vert[n][2]) - dist;
        double dc[4] = {val(d[0]), val(d[1]), val(d[2]), val(d[3])};
        const int cs = d2case(dc, err) - 1;
        for (int n = 0; n < 4; ++n)
            if (!(dc[n] == val(d[n]))) d[n] = R(dc[n]);
        for (int n = 0; n < T_NVERT[cs]; ++n) {
            const int v1 = T_V1[cs][n] - 1, v2 = T_V2[cs][n] - 1;
            const R mu = clamp_mu(sdiv<R>(-d[v1], d[v2] - d[v1]));
            for (int p = 0; p < 3; ++p) vert[4 + n][p] = (R(1.0) - mu) * vert[v1][p] + mu * vert[v2][p];
        }
        for (int n = T_NTETS[cs]; n >= T_NNTET[cs]; --n) {
            R tet[4][3];
            for (int tt = 0; tt < 4; ++tt)
                for (int p = 0; p < 3; ++p) tet[tt][p] = vert[T_VTET[cs][n - 1][tt] - 1][p];
            VF += R(tetsign) * tet_vol(tet) / R(M->dx * M->dy * M->dz);
        }
    }
    return VF;
}

/* ---------------------------------------------------------------------------------------
 * Ghost fill, single rank (src/Tools.jl:4-18 Neumann!, src/Parallel.jl:63-143
 * update_borders!).  Each statement reads the state before it (Julia slices copy).
 * ------------------------------------------------------------------------------------- */
template <class T>
struct Arr3 {
    T* a; int lo[3], hi[3]; long n[3];
    Arr3(T* p, const int l[3], const int h[3]) : a(p)
    {
        for (int d = 0; d < 3; ++d) { lo[d] = l[d]; hi[d] = h[d]; n[d] = h[d] - l[d] + 1; }
    }
    T& at(int i, int j, int k) const { return a[(i - lo[0]) + n[0] * ((j - lo[1]) + n[1] * (long)(k - lo[2]))]; }
};

/* Copy A[dst range along dim] = A[src range along dim] (full extent in the other dims),
 * reading the pre-statement state. */
template <class T>
void slab_copy(Arr3<T>& A, int dim, int dlo, int dhi, int slo)
{
    const int cnt = dhi - dlo + 1;
    int r0[3] = {A.lo[0], A.lo[1], A.lo[2]}, r1[3] = {A.hi[0], A.hi[1], A.hi[2]};
    r0[dim] = 0; r1[dim] = cnt - 1;
    std::vector<T> tmp;
    tmp.reserve((size_t)(r1[0] - r0[0] + 1) * (r1[1] - r0[1] + 1) * (r1[2] - r0[2] + 1));
    for (int k = r0[2]; k <= r1[2]; ++k)
        for (int j = r0[1]; j <= r1[1]; ++j)
            for (int i = r0[0]; i <= r1[0]; ++i) {
                int s[3] = {i, j, k}; s[dim] += slo;
                tmp.push_back(A.at(s[0], s[1], s[2]));
            }
    size_t q = 0;
    for (int k = r0[2]; k <= r1[2]; ++k)
        for (int j = r0[1]; j <= r1[1]; ++j)
            for (int i = r0[0]; i <= r1[0]; ++i) {
                int d[3] = {i, j, k}; d[dim] += dlo;
                A.at(d[0], d[1], d[2]) = tmp[q++];
            }
}

template <class T>
void neumann(const Grid& G, Arr3<T>& A)
{
    for (int d = 0; d < 3; ++d) {
        slab_copy(A, d, 0, 0, 1);                  /* A[min_-1] = A[min_] */
        slab_copy(A, d, G.N[d] + 1, G.N[d] + 1, G.N[d]); /* A[max_+1] = A[max_] */
    }
}

template <class T>
void update_borders(const Grid& G, Arr3<T>& A)
{
    const int per[3] = {G.m->xper, G.m->yper, G.m->zper};
    const int g = G.g;
    for (int d = 0; d < 3; ++d) {
        if (!per[d]) continue; /* MPI.PROC_NULL neighbours: receive buffer unchanged */
        const int mn = 1, mx = G.N[d];
        slab_copy(A, d, mx + 1, mx + g, mn);             /* [max_+1:maxo_] <- [min_:min_+g-1] */
        slab_copy(A, d, mn - g, mn - 1, mx - g + 1);     /* [mino_:min_-1] <- [max_-g+1:max_] */
    }
}

/* ---------------------------------------------------------------------------------------
 * ELVIRA, src/ELVIRA.jl:6-137.
 * ------------------------------------------------------------------------------------- */
template <class T>
struct FieldsT {
    const Grid* G;
    const T* VF;
    T VFat(int i, int j, int k) const { return VF[G->v(i, j, k)]; }
};
using Fields = FieldsT<double>;

template <class R, class FT, class OT>
void check_normal(const Grid& G, const FT& F, R& err, R nx_, R ny_, R nz_, OT* nx, OT* ny, OT* nz, int i, int j,
                  int k, Err* e)
{
    R err_(0.0);
    const R norm = f_sqrt((nx_ * nx_ + ny_ * ny_) + nz_ * nz_);
    nx_ = nx_ / norm; ny_ = ny_ / norm; nz_ = nz_ / norm;
    const R dist = compute_dist<R>(G, i, j, k, nx_, ny_, nz_, R(F.VFat(i, j, k)));
    for (int kk = k - 1; kk <= k + 1; ++kk)
        for (int jj = j - 1; jj <= j + 1; ++jj)
            for (int ii = i - 1; ii <= i + 1; ++ii) {
                const R VF_ = compute_plic2vf<R>(G, ii, jj, kk, nx_, ny_, nz_, dist, e);
                const R r = R(F.VFat(ii, jj, kk)) - VF_;
                err_ += r * r;
            }
    if (val(err_) < val(err)) {
        err = err_;
        const long c = G.c(i, j, k);
        store(nx[c], nx_); store(ny[c], ny_); store(nz[c], nz_);
    }
}

template <class R = double, class FT = Fields, class OT = double>
void elvira_calc(const Grid& G, const FT& F, OT* nx, OT* ny, OT* nz, int i, int j, int k, Err* e)
{
    const orc_mesh* M = G.m;
    R err(INFINITY);
    auto V = [&](int a, int b, int c) { return R(F.VFat(a, b, c)); };
    const int P[3][2] = {{-1, 0}, {-1, 1}, {0, 1}};
    if (M->Nz > 1) {
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                const int jj1 = j + P[a][0], jj2 = j + P[a][1], ii1 = i + P[b][0], ii2 = i + P[b][1];
                const R s2x = (V(ii2, j, k - 1) * M->dz + V(ii2, j, k) * M->dz) + V(ii2, j, k + 1) * M->dz;
                const R s1x = (V(ii1, j, k - 1) * M->dz + V(ii1, j, k) * M->dz) + V(ii1, j, k + 1) * M->dz;
                const R nx_ = -(s2x - s1x) / (G.xm(ii2) - G.xm(ii1));
                const R s2y = (V(i, jj2, k - 1) * M->dz + V(i, jj2, k) * M->dz) + V(i, jj2, k + 1) * M->dz;
                const R s1y = (V(i, jj1, k - 1) * M->dz + V(i, jj1, k) * M->dz) + V(i, jj1, k + 1) * M->dz;
                const R ny_ = -(s2y - s1y) / (G.ym(jj2) - G.ym(jj1));
                const R nz_ = val(V(i, j, k + 1)) > val(V(i, j, k - 1)) ? R(-1.0) : R(1.0);
                check_normal<R, FT, OT>(G, F, err, nx_, ny_, nz_, nx, ny, nz, i, j, k, e);
            }
    }
    if (M->Ny > 1) {
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                const int kk1 = k + P[a][0], kk2 = k + P[a][1], ii1 = i + P[b][0], ii2 = i + P[b][1];
                const R s2x = (V(ii2, j - 1, k) * M->dy + V(ii2, j, k) * M->dy) + V(ii2, j + 1, k) * M->dy;
                const R s1x = (V(ii1, j - 1, k) * M->dy + V(ii1, j, k) * M->dy) + V(ii1, j + 1, k) * M->dy;
                const R nx_ = -(s2x - s1x) / (G.xm(ii2) - G.xm(ii1));
                const R ny_ = val(V(i, j + 1, k)) > val(V(i, j - 1, k)) ? R(-1.0) : R(1.0);
                const R s2z = (V(i, j - 1, kk2) * M->dy + V(i, j, kk2) * M->dy) + V(i, j + 1, kk2) * M->dy;
                const R s1z = (V(i, j - 1, kk1) * M->dy + V(i, j, kk1) * M->dy) + V(i, j + 1, kk1) * M->dy;
                const R nz_ = -(s2z - s1z) / (G.zm(kk2) - G.zm(kk1));
                check_normal<R, FT, OT>(G, F, err, nx_, ny_, nz_, nx, ny, nz, i, j, k, e);
            }
    }
    if (M->Nx > 1) {
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                const int kk1 = k + P[a][0], kk2 = k + P[a][1], jj1 = j + P[b][0], jj2 = j + P[b][1];
                const R nx_ = val(V(i + 1, j, k)) > val(V(i - 1, j, k)) ? R(-1.0) : R(1.0);
                const R s2y = (V(i - 1, jj2, k) * M->dx + V(i, jj2, k) * M->dx) + V(i + 1, jj2, k) * M->dx;
                const R s1y = (V(i - 1, jj1, k) * M->dx + V(i, jj1, k) * M->dx) + V(i + 1, jj1, k) * M->dx;
                const R ny_ = -(s2y - s1y) / (G.ym(jj2) - G.ym(jj1));
                const R s2z = (V(i - 1, j, kk2) * M->dx + V(i, j, kk2) * M->dx) + V(i + 1, j, kk2) * M->dx;
                const R s1z = (V(i - 1, j, kk1) * M->dx + V(i, j, kk1) * M->dx) + V(i + 1, j, kk1) * M->dx;
                const R nz_ = -(s2z - s1z) / (G.zm(kk2) - G.zm(kk1));
                check_normal<R, FT, OT>(G, F, err, nx_, ny_, nz_, nx, ny, nz, i, j, k, e);
            }
    }
}

template <class R = double, class FT = Fields, class OT = double>
void elvira_cell(const Grid& G, const FT& F, OT* nx, OT* ny, OT* nz, int i, int j, int k, Err* e)
{
    const orc_mesh* M = G.m;
    const double lo = M->VFlo, hi = M->VFhi;
    auto V = [&](int a, int b, int c) { return val(F.VFat(a, b, c)); };
    const double v = V(i, j, k);
    const long c = G.c(i, j, k);
    if (v >= lo && v <= hi) {
        elvira_calc<R, FT, OT>(G, F, nx, ny, nz, i, j, k, e);
    } else if (v < lo) {
        if (V(i - 1, j, k) > hi) nx[c] = 1;
        else if (V(i + 1, j, k) > hi) nx[c] = -1;
        else if (V(i, j - 1, k) > hi) ny[c] = 1;
        else if (V(i, j + 1, k) > hi) ny[c] = -1;
        else if (V(i, j, k - 1) > hi) nz[c] = 1;
        else if (V(i, j, k + 1) > hi) nz[c] = -1;
    } else if (v > hi) {
        if (V(i - 1, j, k) < lo) nx[c] = -1;
        else if (V(i + 1, j, k) < lo) nx[c] = 1;
        else if (V(i, j - 1, k) < lo) ny[c] = -1;
        else if (V(i, j + 1, k) < lo) ny[c] = 1;
        else if (V(i, j, k - 1) < lo) nz[c] = -1;
        else if (V(i, j, k + 1) < lo) nz[c] = 1;
    }
}

/* ---------------------------------------------------------------------------------------
 * Velocity interpolation and projection, src/Tools.jl:392-641.
 * ------------------------------------------------------------------------------------- */
struct Vel {
    const double *uf, *vf, *wf;
    const int *su = nullptr, *sv = nullptr, *sw = nullptr; /* Dual: derivative slot of each face value, -1 none */
};

template <class R>
inline R fetch(const double* f, const int* seed, long t);
template <>
inline double fetch<double>(const double* f, const int*, long t) { return f[t]; }
template <>
inline Cnt fetch<Cnt>(const double* f, const int*, long t) { return Cnt(f[t]); }
template <>
inline Dual fetch<Dual>(const double* f, const int* seed, long t)
{
    Dual r(f[t]);
    if (seed && seed[t] >= 0) r.d[seed[t]] = 1.0;
    return r;
}

/* get_velocity_{u,v,w}face: stag = which direction uses face coordinates. */
template <class R>
R interp_face(const Grid& G, const double* f, const int* seed, int stag, const R pt[3], int i, int j, int k)
{
    int I[3] = {i, j, k};
    for (int d = 0; d < 3; ++d) {
        auto co = [&](int q) { return d == stag ? G.fc(d, q) : (d == 0 ? G.xm(q) : (d == 1 ? G.ym(q) : G.zm(q))); };
        while (val(pt[d]) - co(I[d]) < 0.0 && I[d] > G.lo[d]) I[d] = I[d] - 1;
        while (val(pt[d]) - co(I[d] + 1) >= 0.0 && I[d] + 1 < G.hi[d]) I[d] = I[d] + 1;
    }
    R w1[3], w2[3];
    for (int d = 0; d < 3; ++d) {
        auto co = [&](int q) { return d == stag ? G.fc(d, q) : (d == 0 ? G.xm(q) : (d == 1 ? G.ym(q) : G.zm(q))); };
        w1[d] = sdiv<R>(pt[d] - co(I[d]), R(co(I[d] + 1) - co(I[d])));
        w2[d] = R(1.0) - w1[d];
    }
    const int a = I[0], b = I[1], c = I[2];
    auto F = [&](int ii, int jj, int kk) { return fetch<R>(f, seed, G.c(ii, jj, kk)); };
    return w1[2] * (w1[1] * (w1[0] * F(a + 1, b + 1, c + 1) + w2[0] * F(a, b + 1, c + 1)) +
                    w2[1] * (w1[0] * F(a + 1, b, c + 1) + w2[0] * F(a, b, c + 1))) +
           w2[2] * (w1[1] * (w1[0] * F(a + 1, b + 1, c) + w2[0] * F(a, b + 1, c)) +
                    w2[1] * (w1[0] * F(a + 1, b, c) + w2[0] * F(a, b, c)));
}

template <class R>
void velocity(const Grid& G, const Vel& V, const R pt[3], int i, int j, int k, R out[3])
{
    out[0] = interp_face<R>(G, V.uf, V.su, 0, pt, i, j, k);
    out[1] = interp_face<R>(G, V.vf, V.sv, 1, pt, i, j, k);
    out[2] = interp_face<R>(G, V.wf, V.sw, 2, pt, i, j, k);
}

template <class R>
void project(const Grid& G, const Vel& V, R pt[3], int i, int j, int k, double dt)
{
    const int method = G.m->projection;
    if (method == 3) {
        /* test_case == "Zalesak": exact rotation about (0.5, 0.5), src/Tools.jl:396-399;
         * 2*pi in Float64 is 2.0*pi exactly */
        const double a = 6.283185307179586 * dt;
        const double c = detm_cos(a), s = detm_sin(a);
        const R x0 = pt[0], y0 = pt[1];
        pt[0] = (0.5 + c * (x0 - 0.5)) + s * (y0 - 0.5);
        pt[1] = (0.5 - s * (x0 - 0.5)) + c * (y0 - 0.5);
        return;
    }
    if (method == 2) {
        R v1[3], v2[3], v3[3], v4[3], p[3];
        velocity(G, V, pt, i, j, k, v1);
        for (int d = 0; d < 3; ++d) p[d] = pt[d] - 0.5 * dt * v1[d];
        velocity(G, V, p, i, j, k, v2);
        for (int d = 0; d < 3; ++d) p[d] = pt[d] - 0.5 * dt * v2[d];
        velocity(G, V, p, i, j, k, v3);
        for (int d = 0; d < 3; ++d) p[d] = pt[d] - dt * v3[d];
        velocity(G, V, p, i, j, k, v4);
        for (int d = 0; d < 3; ++d) pt[d] = pt[d] + (-dt) / 6.0 * (((v1[d] + 2.0 * v2[d]) + 2.0 * v3[d]) + v4[d]);
    } else if (method == 0) {
        R v1[3];
        velocity(G, V, pt, i, j, k, v1);
        for (int d = 0; d < 3; ++d) pt[d] = pt[d] + (-dt) * v1[d];
    } else {
        R v1[3], v2[3], p[3];
        velocity(G, V, pt, i, j, k, v1);
        for (int d = 0; d < 3; ++d) p[d] = pt[d] - 0.5 * dt * v1[d];
        velocity(G, V, p, i, j, k, v2);
        for (int d = 0; d < 3; ++d) pt[d] = pt[d] + (-dt) * v2[d];
    }
}

/* pt2index!, src/Tools.jl:424-434.  The reference's loops are unbounded; here leaving the
 * coordinate arrays raises E_INDEX and clamps. */
void pt2index(const Grid& G, int I[3], const double pt[3], int i, int j, int k, Err* e)
{
    I[0] = i; I[1] = j; I[2] = k;
    for (int d = 0; d < 3; ++d) {
        while (pt[d] > G.fc(d, I[d] + 1) + EPS) {
            if (I[d] >= G.hi[d]) { e->flags |= E_INDEX; break; }
            I[d] += 1;
        }
        while (pt[d] < G.fc(d, I[d]) - EPS) {
            if (I[d] <= G.lo[d]) { e->flags |= E_INDEX; break; }
            I[d] -= 1;
        }
    }
}

inline void pt2index(const Grid& G, int I[3], const Cnt pt[3], int i, int j, int k, Err* e)
{
    const double p[3] = {pt[0].v, pt[1].v, pt[2].v};
    pt2index(G, I, p, i, j, k, e);
}

inline void pt2index(const Grid& G, int I[3], const Dual pt[3], int i, int j, int k, Err* e)
{
    const double p[3] = {pt[0].v, pt[1].v, pt[2].v};
    pt2index(G, I, p, i, j, k, e);
}

/* ---------------------------------------------------------------------------------------
 * cutTet, src/VFgeom.jl:713-900, kept recursive as in the reference.
 * ------------------------------------------------------------------------------------- */
template <class T>
struct PlicT { const T *nx, *ny, *nz, *D; };
using Plic = PlicT<double>;
/* cell-centred velocities and densities for the momentum sums of transport! (may be absent) */
struct Mom { const double *u, *v, *w; double rho_liq, rho_gas; };

template <class R>
struct CutOutT { R vol, vLiq, vrhoU, vrhoV, vrhoW, vrho; };
using CutOut = CutOutT<double>;

template <class R, class PT = Plic>
CutOutT<R> cut_tet(const Grid& G, const PT& P, const Mom* M, R tet[4][3], int ind[4][3], bool xdone, bool ydone,
               bool zdone, int lvl, Err* e)
{
    if (lvl > 64) { e->flags |= E_DEPTH; return {R(0.0), R(0.0), R(0.0), R(0.0), R(0.0), R(0.0)}; }
    int dir = -1, cut_ind = 0;
    R d[4];
    for (;;) {
        bool* done[3] = {&xdone, &ydone, &zdone};
        int q = -1;
        for (int dd = 0; dd < 3; ++dd)
            if (!*done[dd]) { q = dd; break; }
        if (q < 0) break; /* PLIC leaf */
        int mx = ind[0][q], mn = ind[0][q];
        for (int n = 1; n < 4; ++n) { mx = std::max(mx, ind[n][q]); mn = std::min(mn, ind[n][q]); }
        if (mx > mn) {
            dir = q; cut_ind = mx;
            for (int n = 0; n < 4; ++n) d[n] = tet[n][q] - G.fc(q, cut_ind);
            break;
        }
        *done[q] = true; /* tail call cutTet(..., xdone=true, ...) at the same level */
    }
    if (dir < 0) {
        /* Leaf: clip by the donor cell's PLIC plane (src/VFgeom.jl:757-830). */
        R vert[8][3];
        for (int n = 0; n < 4; ++n)
            for (int p = 0; p < 3; ++p) vert[n][p] = tet[n][p];
        const int i = ind[0][0], j = ind[0][1], k = ind[0][2];
        const long c = G.c(i, j, k);
        for (int n = 0; n < 4; ++n) d[n] = ((P.nx[c] * vert[n][0] + P.ny[c] * vert[n][1]) + P.nz[c] * vert[n][2]) - P.D[c];
        double dc[4] = {val(d[0]), val(d[1]), val(d[2]), val(d[3])};
        const int cs = d2case(dc, e) - 1;
        for (int n = 0; n < T_NVERT[cs]; ++n) {
            const int v1 = T_V1[cs][n] - 1, v2 = T_V2[cs][n] - 1;
            const R mu = clamp_mu(sdiv<R>(-d[v1], d[v2] - d[v1]));
            for (int p = 0; p < 3; ++p) vert[4 + n][p] = (R(1.0) - mu) * vert[v1][p] + mu * vert[v2][p];
        }
        CutOutT<R> r{R(0.0), R(0.0), R(0.0), R(0.0), R(0.0), R(0.0)};
        const double uc = M ? M->u[c] : 0.0, vc = M ? M->v[c] : 0.0, wc = M ? M->w[c] : 0.0;
        for (int n = T_NTETS[cs]; n >= T_NNTET[cs]; --n) {
            R nt[4][3];
            for (int t = 0; t < 4; ++t)
                for (int p = 0; p < 3; ++p) nt[t][p] = vert[T_VTET[cs][n - 1][t] - 1][p];
            const R tv = tet_vol(nt);
            r.vol += tv;
            r.vLiq += tv;
            if (M) {
                r.vrhoU += tv * uc * M->rho_liq;
                r.vrhoV += tv * vc * M->rho_liq;
                r.vrhoW += tv * wc * M->rho_liq;
                r.vrho += tv * M->rho_liq;
            }
        }
        for (int n = 1; n <= T_NNTET[cs] - 1; ++n) {
            R nt[4][3];
            for (int t = 0; t < 4; ++t)
                for (int p = 0; p < 3; ++p) nt[t][p] = vert[T_VTET[cs][n - 1][t] - 1][p];
            const R tv = tet_vol(nt);
            r.vol += tv;
            if (M) {
                r.vrhoU += tv * uc * M->rho_gas;
                r.vrhoV += tv * vc * M->rho_gas;
                r.vrhoW += tv * wc * M->rho_gas;
                r.vrho += tv * M->rho_gas;
            }
        }
        return r;
    }
    /* Cut by the mesh plane (src/VFgeom.jl:832-899). */
    double dc[4] = {val(d[0]), val(d[1]), val(d[2]), val(d[3])};
    const int cs = d2case(dc, e) - 1;
    R vert[8][3];
    int vind[8][3][2];
    for (int n = 0; n < 4; ++n) {
        for (int p = 0; p < 3; ++p) {
            vert[n][p] = tet[n][p];
            vind[n][p][0] = ind[n][p];
            vind[n][p][1] = ind[n][p];
        }
        vind[n][dir][0] = std::min(vind[n][dir][0], cut_ind - 1);
        vind[n][dir][1] = std::max(vind[n][dir][0], cut_ind);
    }
    for (int n = 0; n < T_NVERT[cs]; ++n) {
        const int v1 = T_V1[cs][n] - 1, v2 = T_V2[cs][n] - 1;
        const R mu = clamp_mu(sdiv<R>(-d[v1], d[v2] - d[v1]));
        for (int p = 0; p < 3; ++p) vert[4 + n][p] = (R(1.0) - mu) * vert[v1][p] + mu * vert[v2][p];
        /* seed: side-1 index of vertex n (src/VFgeom.jl:854-857) */
        int I[3];
        pt2index(G, I, vert[4 + n], vind[n][0][0], vind[n][1][0], vind[n][2][0], e);
        for (int p = 0; p < 3; ++p) {
            int val = I[p];
            val = std::max(val, std::min(vind[v1][p][0], vind[v2][p][0]));
            val = std::min(val, std::max(vind[v1][p][0], vind[v2][p][0]));
            vind[4 + n][p][0] = val;
            vind[4 + n][p][1] = val;
        }
        vind[4 + n][dir][0] = cut_ind - 1;
        vind[4 + n][dir][1] = cut_ind;
    }
    CutOutT<R> acc{R(0.0), R(0.0), R(0.0), R(0.0), R(0.0), R(0.0)};
    for (int n = 0; n < T_NTETS[cs]; ++n) {
        R ct[4][3];
        int ci[4][3];
        const int side = T_SIDE[cs][n] - 1;
        for (int nn = 0; nn < 4; ++nn) {
            const int vt = T_VTET[cs][n][nn] - 1;
            for (int p = 0; p < 3; ++p) {
                ct[nn][p] = vert[vt][p];
                ci[nn][p] = vind[vt][p][side];
            }
        }
        const CutOutT<R> r = cut_tet<R, PT>(G, P, M, ct, ci, xdone, ydone, zdone, lvl + 1, e);
        acc.vol += r.vol;
        acc.vLiq += r.vLiq;
        acc.vrhoU += r.vrhoU;
        acc.vrhoV += r.vrhoV;
        acc.vrhoW += r.vrhoW;
        acc.vrho += r.vrho;
    }
    return acc;
}

template <class R>
void correction_tets(const Grid& G, const Vel& V, int i, int j, int k, double dt, R tets[12][4][3]);

/* SL update of one cell, src/Transport.jl:111-148 with cell2tets!(project_verts=true,
 * compute_indices=true) (src/VFgeom.jl:345-420). Returns VFnew. */
template <class R = double, class PT = Plic>
R sl_cell(const Grid& G, const Vel& V, const PT& P, double dt, int i, int j, int k, Err* e, double* vol_out,
          const Mom* M = nullptr, double* mom_out = nullptr)
{
    double v0[15][3];
    const double tetsign = cell2verts(G, i, j, k, v0);
    R verts[15][3];
    for (int n = 0; n < 8; ++n)
        for (int p = 0; p < 3; ++p) verts[n][p] = v0[n][p];
    for (int n = 0; n < 8; ++n) project(G, V, verts[n], i, j, k, dt);
    /* 24_tets: mean points of the projected vertices, their cells seeded at the cell
     * (verts2tets! inside cell2tets!, src/VFgeom.jl:283-330,402-406) */
    tess_points(G.tess, verts);
    int vInds[15][3];
    for (int n = 0; n < tess_npoints(G.tess); ++n) pt2index(G, vInds[n], verts[n], i, j, k, e);
    R vol(0.0), vLiq(0.0), vrhoU(0.0), vrhoV(0.0), vrhoW(0.0), vrho(0.0);
    for (int t = 0; t < tess_ntets(G.tess); ++t) {
        R tet[4][3];
        int ind[4][3];
        int tv[4];
        tess_tet(G.tess, t, tv);
        for (int n = 0; n < 4; ++n)
            for (int p = 0; p < 3; ++p) {
                tet[n][p] = verts[tv[n]][p];
                ind[n][p] = vInds[tv[n]][p];
            }
        const CutOutT<R> r = cut_tet<R, PT>(G, P, M, tet, ind, false, false, false, 1, e);
        vol += tetsign * r.vol;
        vLiq += tetsign * r.vLiq;
        vrhoU += tetsign * r.vrhoU;
        vrhoV += tetsign * r.vrhoV;
        vrhoW += tetsign * r.vrhoW;
        vrho += tetsign * r.vrho;
    }
    if (G.m->pressure_scheme == 1) {
        /* pressure_scheme "finite-difference": the flux-correction tets, their vertices' cells
         * by pt2index! seeded at the cell (src/Transport.jl:121-124, src/VFgeom.jl:654-661) */
        R ct[12][4][3];
        correction_tets<R>(G, V, i, j, k, dt, ct);
        for (int t = 0; t < 12; ++t) {
            int ind[4][3];
            for (int n = 0; n < 4; ++n) pt2index(G, ind[n], ct[t][n], i, j, k, e);
            const CutOutT<R> r = cut_tet<R, PT>(G, P, M, ct[t], ind, false, false, false, 1, e);
            vol += tetsign * r.vol;
            vLiq += tetsign * r.vLiq;
            vrhoU += tetsign * r.vrhoU;
            vrhoV += tetsign * r.vrhoV;
            vrhoW += tetsign * r.vrhoW;
            vrho += tetsign * r.vrho;
        }
    }
    if (!(val(vol) > 0.0) || !std::isfinite(val(vol))) e->flags |= E_VOLUME;
    if (vol_out) *vol_out = val(vol);
    /* us, vs, ws of the cell (src/Transport.jl:146-148) */
    if (mom_out) {
        mom_out[0] = val(vrhoU / vrho);
        mom_out[1] = val(vrhoV / vrho);
        mom_out[2] = val(vrhoW / vrho);
    }
    return vLiq / vol;
}

/* ---------------------------------------------------------------------------------------
 * Momentum of transport! (src/Transport.jl:34-104,146-166): face fluxes, SLfluxVol.
 * ------------------------------------------------------------------------------------- */
/* Vertices of the flux volume of face `dir` of cell (i,j,k) (src/VFgeom.jl:428-509): index
 * offsets (di, dj, dk) and whether the point is projected, for even and odd cells. */
const int FLUXV[3][2][8][4] = {
    {{{0, 0, 0, 1}, {0, 0, 0, 0}, {0, 1, 0, 1}, {0, 1, 0, 0}, {0, 0, 1, 1}, {0, 0, 1, 0}, {0, 1, 1, 1}, {0, 1, 1, 0}},
     {{0, 0, 0, 0}, {0, 0, 0, 1}, {0, 1, 0, 0}, {0, 1, 0, 1}, {0, 0, 1, 0}, {0, 0, 1, 1}, {0, 1, 1, 0}, {0, 1, 1, 1}}},
    {{{0, 0, 0, 1}, {1, 0, 0, 1}, {0, 0, 0, 0}, {1, 0, 0, 0}, {0, 0, 1, 1}, {1, 0, 1, 1}, {0, 0, 1, 0}, {1, 0, 1, 0}},
     {{1, 0, 0, 1}, {0, 0, 0, 1}, {1, 0, 0, 0}, {0, 0, 0, 0}, {1, 0, 1, 1}, {0, 0, 1, 1}, {1, 0, 1, 0}, {0, 0, 1, 0}}},
    {{{0, 0, 0, 1}, {1, 0, 0, 1}, {0, 1, 0, 1}, {1, 1, 0, 1}, {0, 0, 0, 0}, {1, 0, 0, 0}, {0, 1, 0, 0}, {1, 1, 0, 0}},
     {{1, 0, 0, 1}, {0, 0, 0, 1}, {1, 1, 0, 1}, {0, 1, 0, 1}, {1, 0, 0, 0}, {0, 0, 0, 0}, {1, 1, 0, 0}, {0, 1, 0, 0}}}};

/* SLfluxVol's vertices (tessellation order, mean points for 24_tets) and signed volume. */
template <class R>
R sl_flux_verts(const Grid& G, const Vel& V, int dir, int i, int j, int k, double dt, R verts[15][3])
{
    const bool even = G.tess != 5 || ((i + j + k) % 2) == 0;
    const double tetsign = even ? 1.0 : -1.0;
    for (int n = 0; n < 8; ++n) {
        const int* f = FLUXV[dir][even ? 0 : 1][n];
        verts[n][0] = G.x(i + f[0]);
        verts[n][1] = G.y(j + f[1]);
        verts[n][2] = G.z(k + f[2]);
        if (f[3]) project<R>(G, V, verts[n], i, j, k, dt);
    }
    tess_points(G.tess, verts);
    R vol(0.0); /* tets_vol, src/VFgeom.jl:683-689 */
    for (int t = 0; t < tess_ntets(G.tess); ++t) {
        int tv[4];
        tess_tet(G.tess, t, tv);
        R tet[4][3];
        for (int n = 0; n < 4; ++n)
            for (int p = 0; p < 3; ++p) tet[n][p] = verts[tv[n]][p];
        vol += tet_vol(tet);
    }
    return vol * R(tetsign);
}

double sl_flux_vol(const Grid& G, const Vel& V, int dir, int i, int j, int k, double dt)
{
    double verts[15][3];
    return sl_flux_verts<double>(G, V, dir, i, j, k, dt, verts);
}

/* Apex of add_correction_tets' tets (a,b,d,e) and (b,c,d,e) over a face quad a,b,c,d
 * (src/VFgeom.jl:590-646): e starts at the quad's mean 0.25*(a+b+c+d) and its `axis`
 * coordinate moves until V(a,b,d,e) + V(b,c,d,e) = vol.  Both volumes are affine in e with
 * gradient (a x b + d x a + b x c + c x d)/6, so the coordinate moves by
 * 6 (vol - V(mean)) / that gradient's component.  (The reference writes the same solution as
 * one expanded polynomial, which rounds differently.) */
template <class R>
void correction_apex(int axis, const R* a, const R* b, const R* c, const R* d, const R& vol, R e[3])
{
    for (int p = 0; p < 3; ++p) e[p] = R(0.25) * (((a[p] + b[p]) + c[p]) + d[p]);
    R t1[4][3], t2[4][3];
    for (int p = 0; p < 3; ++p) {
        t1[0][p] = a[p]; t1[1][p] = b[p]; t1[2][p] = d[p]; t1[3][p] = e[p];
        t2[0][p] = b[p]; t2[1][p] = c[p]; t2[2][p] = d[p]; t2[3][p] = e[p];
    }
    const R v0 = tet_vol(t1) + tet_vol(t2);
    const int p = (axis + 1) % 3, q = (axis + 2) % 3; /* (u x w)_axis = u_p w_q - u_q w_p */
    auto cr = [&](const R* u, const R* w) { return u[p] * w[q] - u[q] * w[p]; };
    const R N = ((cr(a, b) + cr(d, a)) + cr(b, c)) + cr(c, d);
    e[axis] = e[axis] + R(6.0) * (vol - v0) / N;
}

/* add_correction_tets (src/VFgeom.jl:514-664), 5_tets: two tets on each face of cell (i,j,k),
 * faces x-, x+, y-, y+, z-, z+, built on the face's SLfluxVol vertices so that the face's flux
 * volume becomes the finite-difference one, dt * area * face velocity. */
template <class R>
void correction_tets(const Grid& G, const Vel& V, int i, int j, int k, double dt, R tets[12][4][3])
{
    const orc_mesh* M = G.m;
    static const int QUAD[3][2][4] = {{{4, 6, 2, 0}, {7, 5, 1, 3}}, {{1, 5, 4, 0}, {1, 5, 4, 0}}, {{1, 0, 2, 3}, {1, 0, 2, 3}}};
    for (int f = 0; f < 6; ++f) {
        const int dir = f / 2, up = f & 1;
        const int fi = i + (dir == 0 ? up : 0), fj = j + (dir == 1 ? up : 0), fk = k + (dir == 2 ? up : 0);
        R fv[15][3];
        const R flux_vol = sl_flux_verts<R>(G, V, dir, fi, fj, fk, dt, fv);
        const long t = G.c(fi, fj, fk);
        const R divg_vol = dir == 0 ? R((dt * M->dy) * M->dz) * fetch<R>(V.uf, V.su, t)
                                    : (dir == 1 ? R((dt * M->dx) * M->dz) * fetch<R>(V.vf, V.sv, t)
                                                : R((dt * M->dx) * M->dy) * fetch<R>(V.wf, V.sw, t));
        const bool even = G.tess != 5 || ((fi + fj + fk) % 2) == 0; /* oddEvenCell of the face's cell */
        const R vol = even ? (divg_vol - flux_vol) : -(divg_vol - flux_vol);
        const int* qd = QUAD[dir][even ? 0 : 1];
        const R *a = fv[qd[0]], *b = fv[qd[1]], *c = fv[qd[2]], *d = fv[qd[3]];
        R e[3];
        correction_apex<R>(dir, a, b, c, d, vol, e);
        for (int p = 0; p < 3; ++p) {
            tets[2 * f][0][p] = a[p]; tets[2 * f][1][p] = b[p]; tets[2 * f][2][p] = d[p]; tets[2 * f][3][p] = e[p];
            tets[2 * f + 1][0][p] = b[p]; tets[2 * f + 1][1][p] = c[p]; tets[2 * f + 1][2][p] = d[p];
            tets[2 * f + 1][3][p] = e[p];
        }
    }
}

/* Convective fluxes through face `dir` (0 x, 1 y, 2 z) at the low side of cell (i,j,k),
 * src/Transport.jl:34-104 with pressure_scheme "semi-lagrangian". */
void face_flux(const Grid& G, const Vel& V, const Mom& M, const int16_t* band, int dir, int i, int j, int k, double dt,
               double F[3])
{
    const int li = i - (dir == 0), lj = j - (dir == 1), lk = k - (dir == 2);
    const long c = G.c(i, j, k), l = G.c(li, lj, lk);
    const double uface = 0.5 * (M.u[l] + M.u[c]);
    const double vface = 0.5 * (M.v[l] + M.v[c]);
    const double wface = 0.5 * (M.w[l] + M.w[c]);
    const int nb = G.m->nband;
    const bool bl = std::abs((int)band[l]) <= nb, bc = std::abs((int)band[c]) <= nb;
    if (bl && bc) {
        F[0] = 0.0; F[1] = 0.0; F[2] = 0.0;
    } else if ((bl || bc) && G.m->pressure_scheme == 0) {
        const double vol = sl_flux_vol(G, V, dir, i, j, k, dt) / dt;
        F[0] = -uface * vol; F[1] = -vface * vol; F[2] = -wface * vol;
    } else {
        const orc_mesh* Mm = G.m;
        const double a = dir == 0 ? Mm->dy : Mm->dx, b = dir == 2 ? Mm->dy : Mm->dz;
        const double q = dir == 0 ? V.uf[c] : (dir == 1 ? V.vf[c] : V.wf[c]);
        F[0] = -uface * a * b * q; F[1] = -vface * a * b * q; F[2] = -wface * a * b * q;
    }
}

/* ---------------------------------------------------------------------------------------
 * Divergence and the pressure operator (src/Velocity.jl:59-122, src/Pressure.jl:83-115).
 * ------------------------------------------------------------------------------------- */
/* divg_cell, src/Velocity.jl:71-122.  sl: pressure_scheme == "semi-lagrangian".  A band cell
 * gives (v2 - v1)/v2/dt with v1 the volume of its projected cell (cell2tets! with
 * project_verts, tets_vol) and v2 = dx*dy*dz; any other cell the face fluxes, SLfluxVol/dt
 * through a face whose neighbour is a band cell, the finite-difference flux otherwise. */
double divg_cell(const Grid& G, const Vel& V, const int16_t* band, bool sl, int i, int j, int k, double dt)
{
    const orc_mesh* M = G.m;
    auto inband = [&](int a, int b, int c) { return sl && std::abs((int)band[G.c(a, b, c)]) <= M->nband; };
    if (inband(i, j, k)) {
        double verts[15][3];
        const double tetsign = cell2verts(G, i, j, k, verts);
        for (int n = 0; n < 8; ++n) project(G, V, verts[n], i, j, k, dt);
        tess_points(G.tess, verts);
        double vol = 0.0; /* tets_vol, src/VFgeom.jl:683-689 */
        for (int t = 0; t < tess_ntets(G.tess); ++t) {
            int tv[4];
            tess_tet(G.tess, t, tv);
            double tet[4][3];
            for (int n = 0; n < 4; ++n)
                for (int p = 0; p < 3; ++p) tet[n][p] = verts[tv[n]][p];
            vol += tet_vol(tet);
        }
        const double v2 = (M->dx * M->dy) * M->dz;
        const double v1 = tetsign * vol;
        return (v2 - v1) / v2 / dt;
    }
    auto flux = [&](int dir, int a, int b, int c, int na, int nb, int nc) {
        if (inband(na, nb, nc)) return sl_flux_vol(G, V, dir, a, b, c, dt) / dt;
        const long t = G.c(a, b, c);
        if (dir == 0) return (M->dy * M->dz) * V.uf[t];
        if (dir == 1) return (M->dx * M->dz) * V.vf[t];
        return (M->dx * M->dy) * V.wf[t];
    };
    const double Fxm = flux(0, i, j, k, i - 1, j, k), Fxp = flux(0, i + 1, j, k, i + 1, j, k);
    const double Fym = flux(1, i, j, k, i, j - 1, k), Fyp = flux(1, i, j + 1, k, i, j + 1, k);
    const double Fzm = flux(2, i, j, k, i, j, k - 1), Fzp = flux(2, i, j, k + 1, i, j, k + 1);
    return (((((Fxp - Fxm) + Fyp) - Fym) + Fzp) - Fzm) / ((M->dx * M->dy) * M->dz);
}

/* ---------------------------------------------------------------------------------------
 * Height-function curvature (src/ELVIRA.jl:141-184) and the face properties
 * (compute_props!, src/Tools.jl:1186-1210).
 * ------------------------------------------------------------------------------------- */
/* x^(3/2) as x*sqrt(x): IEEE sqrt and one rounded product, within two ulp of a correctly
 * rounded power (the reference's Julia ^ is not vendored). */
inline double pow32(double x) { return x * std::sqrt(x); }

/* compute_curvature!: heights of 7 cells along the normal's dominant axis (strictly larger
 * component) in the 3x3 columns around the cell, scaled by the spacing; central differences of
 * the heights; the curvature of the height function.  A cell without a strictly dominant
 * component keeps Curve = 0. */
double curvature_cell(const Grid& G, const double* VF, double nx, double ny, double nz, int i, int j, int k)
{
    const orc_mesh* M = G.m;
    const double ax = std::fabs(nx), ay = std::fabs(ny), az = std::fabs(nz);
    double h[3][3]; /* h[a][b]: a, b the two tangential offsets + 1 in the branch's hf order */
    if (ax > ay && ax > az) {
        for (int kk = -1; kk <= 1; ++kk)
            for (int jj = -1; jj <= 1; ++jj) {
                double s = 0.0;
                for (int ii = -3; ii <= 3; ++ii) s += VF[G.v(i + ii, j + jj, k + kk)];
                h[jj + 1][kk + 1] = s;
            }
        for (auto& r : h) for (double& x : r) x *= M->dx;
        const double dy = M->dy, dz = M->dz;
        const double hfy = (h[2][1] - h[0][1]) / (2 * dy), hfz = (h[1][2] - h[1][0]) / (2 * dz);
        const double hfyy = ((h[2][1] - 2 * h[1][1]) + h[0][1]) / (dy * dy);
        const double hfzz = ((h[1][2] - 2 * h[1][1]) + h[1][0]) / (dz * dz);
        const double hfyz = (((h[2][2] - h[0][2]) - h[2][0]) + h[0][0]) / ((4 * dy) * dz);
        return ((((hfyy + hfzz) + hfyy * (hfz * hfz)) + hfzz * (hfy * hfy)) - ((2 * hfyz) * hfy) * hfz) /
               pow32((1 + hfy * hfy) + hfz * hfz);
    }
    if (ay > ax && ay > az) {
        for (int ii = -1; ii <= 1; ++ii)
            for (int kk = -1; kk <= 1; ++kk) {
                double s = 0.0;
                for (int jj = -3; jj <= 3; ++jj) s += VF[G.v(i + ii, j + jj, k + kk)];
                h[kk + 1][ii + 1] = s;
            }
        for (auto& r : h) for (double& x : r) x *= M->dy;
        const double dx = M->dx, dz = M->dz;
        const double hfz = (h[2][1] - h[0][1]) / (2 * dz), hfx = (h[1][2] - h[1][0]) / (2 * dx);
        const double hfzz = ((h[2][1] - 2 * h[1][1]) + h[0][1]) / (dz * dz);
        const double hfxx = ((h[1][2] - 2 * h[1][1]) + h[1][0]) / (dx * dx);
        const double hfxz = (((h[2][2] - h[2][0]) - h[0][2]) + h[0][0]) / ((4 * dz) * dx);
        return ((((hfzz + hfxx) + hfzz * (hfx * hfx)) + hfxx * (hfz * hfz)) - ((2 * hfxz) * hfz) * hfx) /
               pow32((1 + hfz * hfz) + hfx * hfx);
    }
    if (az > ay && az > ax) {
        for (int jj = -1; jj <= 1; ++jj)
            for (int ii = -1; ii <= 1; ++ii) {
                double s = 0.0;
                for (int kk = -3; kk <= 3; ++kk) s += VF[G.v(i + ii, j + jj, k + kk)];
                h[ii + 1][jj + 1] = s;
            }
        for (auto& r : h) for (double& x : r) x *= M->dz;
        const double dx = M->dx, dy = M->dy;
        const double hfx = (h[2][1] - h[0][1]) / (2 * dx), hfy = (h[1][2] - h[1][0]) / (2 * dy);
        const double hfxx = ((h[2][1] - 2 * h[1][1]) + h[0][1]) / (dx * dx);
        const double hfyy = ((h[1][2] - 2 * h[1][1]) + h[1][0]) / (dy * dy);
        const double hfxy = (((h[2][2] - h[2][0]) - h[0][2]) + h[0][0]) / ((4 * dy) * dx);
        return ((((hfxx + hfyy) + hfxx * (hfy * hfy)) + hfyy * (hfx * hfx)) - ((2 * hfxy) * hfx) * hfy) /
               pow32((1 + hfx * hfx) + hfy * hfy);
    }
    return 0.0;
}

} // namespace

/* =========================================================================================
 * C API (ctypes).  All arrays are OffsetArray parents: cell arrays (N+2g)^3, VF (N+2g+6)^3.
 * ======================================================================================= */
extern "C" {

double orc_detm_cbrt(double x) { return detm_cbrt(x); }
double orc_detm_acos(double x) { return detm_acos(x); }
double orc_detm_sin(double x) { return detm_sin(x); }
double orc_detm_cos(double x) { return detm_cos(x); }

double orc_compute_alpha(const double m[3], double VF) { return compute_alpha(m, VF); }

double orc_compute_dist(const orc_mesh* M, int i, int j, int k, double nx, double ny, double nz, double VF)
{
    Grid G(M);
    return compute_dist(G, i, j, k, nx, ny, nz, VF);
}

double orc_compute_plic2vf(const orc_mesh* M, int i, int j, int k, double nx, double ny, double nz, double dist)
{
    Grid G(M);
    Err e;
    return compute_plic2vf(G, i, j, k, nx, ny, nz, dist, &e);
}

double orc_tet_vol(const double v[12])
{
    double t[4][3];
    for (int n = 0; n < 4; ++n)
        for (int p = 0; p < 3; ++p) t[n][p] = v[3 * n + p];
    return tet_vol(t);
}

/* ELVIRA! (src/ELVIRA.jl:6-55): zero the whole normal arrays, compute the interior, then
 * update_borders! on each.  Cells k in [klo, khi] only when klo <= khi (bench sample). */
int orc_elvira(const orc_mesh* M, const double* VF, double* nx, double* ny, double* nz, int klo, int khi)
{
    Grid G(M);
    const long ncell = G.n[0] * G.n[1] * G.n[2];
    if (klo > khi) {
        klo = 1;
        khi = G.N[2];
        std::fill(nx, nx + ncell, 0.0);
        std::fill(ny, ny + ncell, 0.0);
        std::fill(nz, nz + ncell, 0.0);
    } else {
        /* sample: the slab's own layers are zeroed, as the whole arrays are for the full grid */
        const long a = G.c(G.lo[0], G.lo[1], klo), b = G.c(G.lo[0], G.lo[1], khi + 1);
        std::fill(nx + a, nx + b, 0.0);
        std::fill(ny + a, ny + b, 0.0);
        std::fill(nz + a, nz + b, 0.0);
    }
    Fields F{&G, VF};
    int flags = 0;
#pragma omp parallel for collapse(2) schedule(dynamic, 1) reduction(| : flags)
    for (int k = klo; k <= khi; ++k)
        for (int j = 1; j <= G.N[1]; ++j) {
            Err e;
            for (int i = 1; i <= G.N[0]; ++i) elvira_cell(G, F, nx, ny, nz, i, j, k, &e);
            flags |= e.flags;
        }
    Arr3<double> A(nx, G.lo, G.hi), B(ny, G.lo, G.hi), C(nz, G.lo, G.hi);
    update_borders(G, A); update_borders(G, B); update_borders(G, C);
    return flags;
}

/* computePLIC! (src/VF.jl:94-103): D at every cell including ghosts, then update_borders!. */
int orc_compute_plic(const orc_mesh* M, double* D, const double* nx, const double* ny, const double* nz, const double* VF)
{
    Grid G(M);
#pragma omp parallel for collapse(2)
    for (int k = G.lo[2]; k <= G.hi[2]; ++k)
        for (int j = G.lo[1]; j <= G.hi[1]; ++j)
            for (int i = G.lo[0]; i <= G.hi[0]; ++i) {
                const long c = G.c(i, j, k);
                D[c] = compute_dist(G, i, j, k, nx[c], ny[c], nz[c], VF[G.v(i, j, k)]);
            }
    Arr3<double> A(D, G.lo, G.hi);
    update_borders(G, A);
    return 0;
}

/* computePLIC!'s per-cell work on the cells k in [klo, khi] only (CPU baseline sample). */
int orc_compute_plic_slab(const orc_mesh* M, double* D, const double* nx, const double* ny, const double* nz,
                          const double* VF, int klo, int khi)
{
    Grid G(M);
#pragma omp parallel for collapse(2)
    for (int k = klo; k <= khi; ++k)
        for (int j = G.lo[1]; j <= G.hi[1]; ++j)
            for (int i = G.lo[0]; i <= G.hi[0]; ++i) {
                const long c = G.c(i, j, k);
                D[c] = compute_dist(G, i, j, k, nx[c], ny[c], nz[c], VF[G.v(i, j, k)]);
            }
    return 0;
}

/* computeBand! (src/VF.jl:16-74) on the cells k in [klo, khi]; the ghost updates only for
 * the whole grid (the CPU baseline's sample times the per-cell passes of a slab).  Julia's
 * combined for-loop "break" leaves all three loops. */
static void compute_band_k(const orc_mesh* M, int16_t* band, const double* VF, int klo, int khi, bool borders)
{
    Grid G(M);
    const int nb = M->nband;
    Arr3<int16_t> B(band, G.lo, G.hi);
    /* the first pass reads VF only: cells are independent; the sweeps update in place */
#pragma omp parallel for collapse(2)
    for (int k = klo; k <= khi; ++k)
        for (int j = 1; j <= G.N[1]; ++j)
            for (int i = 1; i <= G.N[0]; ++i) {
                const double v = VF[G.v(i, j, k)];
                int16_t& b = B.at(i, j, k);
                if (v < M->VFlo) {
                    bool hit = false;
                    for (int kk = k - 1; kk <= k + 1 && !hit; ++kk)
                        for (int jj = j - 1; jj <= j + 1 && !hit; ++jj)
                            for (int ii = i - 1; ii <= i + 1 && !hit; ++ii)
                                if (VF[G.v(ii, jj, kk)] >= M->VFhi) hit = true;
                    b = hit ? 0 : (int16_t)(-nb - 1);
                } else if (v > M->VFhi) {
                    bool hit = false;
                    for (int kk = k - 1; kk <= k + 1 && !hit; ++kk)
                        for (int jj = j - 1; jj <= j + 1 && !hit; ++jj)
                            for (int ii = i - 1; ii <= i + 1 && !hit; ++ii)
                                if (VF[G.v(ii, jj, kk)] <= M->VFlo) hit = true;
                    b = hit ? 0 : (int16_t)(nb + 1);
                } else {
                    b = 0;
                }
            }
    if (borders) {
        neumann(G, B);
        update_borders(G, B);
    }
    for (int n = 1; n <= nb; ++n) {
        for (int k = klo; k <= khi; ++k)
            for (int j = 1; j <= G.N[1]; ++j)
                for (int i = 1; i <= G.N[0]; ++i) {
                    int16_t& b = B.at(i, j, k);
                    if (std::abs((int)b) > n) {
                        for (int kk = k - 1; kk <= k + 1; ++kk)
                            for (int jj = j - 1; jj <= j + 1; ++jj)
                                for (int ii = i - 1; ii <= i + 1; ++ii)
                                    if (std::abs((int)B.at(ii, jj, kk)) == n - 1) b = (int16_t)(n * (b > 0 ? 1 : (b < 0 ? -1 : 0)));
                    }
                }
        if (borders) update_borders(G, B);
    }
}

int orc_compute_band(const orc_mesh* M, int16_t* band, const double* VF)
{
    compute_band_k(M, band, VF, 1, M->Nz, true);
    return 0;
}

/* computeBand!'s per-cell passes on the cells k in [klo, khi] only (CPU baseline sample). */
int orc_compute_band_slab(const orc_mesh* M, int16_t* band, const double* VF, int klo, int khi)
{
    compute_band_k(M, band, VF, klo, khi, false);
    return 0;
}

/* Neumann!(VF) + update_VF_borders!(VF) (src/Transport.jl:180-181). */
int orc_vf_ghost_fill(const orc_mesh* M, double* VF)
{
    Grid G(M);
    Arr3<double> A(VF, G.vlo, G.vhi);
    neumann(G, A);
    update_borders(G, A);
    return 0;
}

/* The SL cell loop + VF copy + ghost fill (src/Transport.jl:108-151,179-181).
 * VF is updated in place.  If klo <= khi only cells k in [klo,khi] are advanced and the VF
 * copy/ghost fill is skipped (bench sample mode); VFnew then receives the sample. */
int orc_transport(const orc_mesh* M, double dt, double* VF, double* VFnew, const double* uf, const double* vf,
                  const double* wf, const double* nx, const double* ny, const double* nz, const double* D,
                  const int16_t* band, int klo, int khi)
{
    Grid G(M);
    const bool sample = klo <= khi;
    if (!sample) { klo = 1; khi = G.N[2]; }
    Vel V{uf, vf, wf};
    Plic P{nx, ny, nz, D};
    int flags = 0;
#pragma omp parallel for collapse(2) schedule(dynamic, 1) reduction(| : flags)
    for (int k = klo; k <= khi; ++k)
        for (int j = 1; j <= G.N[1]; ++j) {
            Err e;
            for (int i = 1; i <= G.N[0]; ++i) {
                const long c = G.c(i, j, k);
                const long v = G.v(i, j, k);
                if (std::abs((int)band[c]) <= M->nband) VFnew[v] = sl_cell(G, V, P, dt, i, j, k, &e, nullptr);
                else VFnew[v] = VF[v];
            }
            flags |= e.flags;
        }
    if (sample) return flags;
    for (int k = 1; k <= G.N[2]; ++k)
        for (int j = 1; j <= G.N[1]; ++j)
            for (int i = 1; i <= G.N[0]; ++i) VF[G.v(i, j, k)] = VFnew[G.v(i, j, k)];
    orc_vf_ghost_fill(M, VF);
    return flags;
}

/* transport!'s SL cell loop with its momentum (src/Transport.jl:34-166, pressure_scheme
 * "semi-lagrangian"): VFnew as orc_transport, and us, vs, ws for every interior cell -- band
 * cells from the clipped pre-image (vrhoU/vrho, ...), the others from the face fluxes.  VF is
 * updated in place and its ghosts filled, as orc_transport does. */
int orc_transport_mom(const orc_mesh* M, double dt, double* VF, double* VFnew, const double* uf, const double* vf,
                      const double* wf, const double* nx, const double* ny, const double* nz, const double* D,
                      const int16_t* band, const double* u, const double* v, const double* w, double* us, double* vs,
                      double* ws)
{
    Grid G(M);
    Vel V{uf, vf, wf};
    Plic P{nx, ny, nz, D};
    Mom Mo{u, v, w, M->rho_liq, M->rho_gas};
    int flags = 0;
    const double cv = (M->dx * M->dy) * M->dz;
#pragma omp parallel for collapse(2) schedule(dynamic, 1) reduction(| : flags)
    for (int k = 1; k <= G.N[2]; ++k)
        for (int j = 1; j <= G.N[1]; ++j) {
            Err e;
            for (int i = 1; i <= G.N[0]; ++i) {
                const long c = G.c(i, j, k);
                const long vv = G.v(i, j, k);
                if (std::abs((int)band[c]) <= M->nband) {
                    double mom[3];
                    VFnew[vv] = sl_cell(G, V, P, dt, i, j, k, &e, nullptr, &Mo, mom);
                    us[c] = mom[0]; vs[c] = mom[1]; ws[c] = mom[2];
                } else {
                    VFnew[vv] = VF[vv];
                    double Fx0[3], Fx1[3], Fy0[3], Fy1[3], Fz0[3], Fz1[3];
                    face_flux(G, V, Mo, band, 0, i, j, k, dt, Fx0);
                    face_flux(G, V, Mo, band, 0, i + 1, j, k, dt, Fx1);
                    face_flux(G, V, Mo, band, 1, i, j, k, dt, Fy0);
                    face_flux(G, V, Mo, band, 1, i, j + 1, k, dt, Fy1);
                    face_flux(G, V, Mo, band, 2, i, j, k, dt, Fz0);
                    face_flux(G, V, Mo, band, 2, i, j, k + 1, dt, Fz1);
                    const double f = dt / cv;
                    us[c] = u[c] + f * (((((Fx1[0] - Fx0[0]) + Fy1[0]) - Fy0[0]) + Fz1[0]) - Fz0[0]);
                    vs[c] = v[c] + f * (((((Fx1[1] - Fx0[1]) + Fy1[1]) - Fy0[1]) + Fz1[1]) - Fz0[1]);
                    ws[c] = w[c] + f * (((((Fx1[2] - Fx0[2]) + Fy1[2]) - Fy0[2]) + Fz1[2]) - Fz0[2]);
                }
            }
            flags |= e.flags;
        }
    for (int k = 1; k <= G.N[2]; ++k)
        for (int j = 1; j <= G.N[1]; ++j)
            for (int i = 1; i <= G.N[0]; ++i) VF[G.v(i, j, k)] = VFnew[G.v(i, j, k)];
    orc_vf_ghost_fill(M, VF);
    return flags;
}

/* divergence!, src/Velocity.jl:59-68: divg = 0 on every cell, divg_cell on the interior.
 * scheme 0 "semi-lagrangian", 1 "finite-difference". */
int orc_divergence(const orc_mesh* M, double dt, int scheme, double* divg, const double* uf, const double* vf,
                   const double* wf, const int16_t* band)
{
    Grid G(M);
    Vel V{uf, vf, wf};
    const long nc = G.n[0] * G.n[1] * G.n[2];
    for (long t = 0; t < nc; ++t) divg[t] = 0.0;
#pragma omp parallel for collapse(2) schedule(dynamic, 1)
    for (int k = 1; k <= G.N[2]; ++k)
        for (int j = 1; j <= G.N[1]; ++j)
            for (int i = 1; i <= G.N[0]; ++i) divg[G.c(i, j, k)] = divg_cell(G, V, band, scheme == 0, i, j, k, dt);
    return 0;
}

/* A!, src/Pressure.jl:83-115: Neumann!(P) + update_borders!(P) in place; the pressure-corrected
 * face velocities gradx = uf - dt/denx*(P - P[i-1])/dx (grady, gradz with the safe divide)
 * over the reference's index ranges, 0 elsewhere; LHS = 0 on every cell and divg_cell of the
 * corrected velocities on the interior. */
int orc_A(const orc_mesh* M, double dt, int scheme, double* LHS, double* P, const double* uf, const double* vf,
          const double* wf, const double* denx, const double* deny, const double* denz, const int16_t* band,
          double* gradx, double* grady, double* gradz)
{
    Grid G(M);
    Arr3<double> A(P, G.lo, G.hi);
    neumann(G, A);
    update_borders(G, A);
    const long nc = G.n[0] * G.n[1] * G.n[2];
    for (long t = 0; t < nc; ++t) { gradx[t] = 0.0; grady[t] = 0.0; gradz[t] = 0.0; LHS[t] = 0.0; }
    const int* N = G.N;
    for (int kk = 0; kk <= N[2] + 1; ++kk)
        for (int jj = 0; jj <= N[1] + 1; ++jj)
            for (int ii = 0; ii <= N[0] + 2; ++ii) {
                const long t = G.c(ii, jj, kk);
                gradx[t] = uf[t] - dt / denx[t] * (P[t] - P[G.c(ii - 1, jj, kk)]) / M->dx;
            }
    for (int kk = 0; kk <= N[2] + 1; ++kk)
        for (int jj = 0; jj <= N[1] + 2; ++jj)
            for (int ii = 0; ii <= N[0] + 1; ++ii) {
                const long t = G.c(ii, jj, kk);
                grady[t] = vf[t] - sdiv(sdiv(dt, deny[t]) * (P[t] - P[G.c(ii, jj - 1, kk)]), M->dy);
            }
    for (int kk = 0; kk <= N[2] + 2; ++kk)
        for (int jj = 0; jj <= N[1] + 1; ++jj)
            for (int ii = 0; ii <= N[0] + 1; ++ii) {
                const long t = G.c(ii, jj, kk);
                gradz[t] = wf[t] - sdiv(sdiv(dt, denz[t]) * (P[t] - P[G.c(ii, jj, kk - 1)]), M->dz);
            }
    Vel V{gradx, grady, gradz};
#pragma omp parallel for collapse(2) schedule(dynamic, 1)
    for (int k = 1; k <= N[2]; ++k)
        for (int j = 1; j <= N[1]; ++j)
            for (int i = 1; i <= N[0]; ++i) LHS[G.c(i, j, k)] = divg_cell(G, V, band, scheme == 0, i, j, k, dt);
    return 0;
}

/* The curvature section of transport! (src/Transport.jl:187-191): Curve = 0, then
 * compute_curvature! on the interior. */
int orc_curvature(const orc_mesh* M, double* Curve, const double* VF, const double* nx, const double* ny,
                  const double* nz)
{
    Grid G(M);
    const long nc = G.n[0] * G.n[1] * G.n[2];
    for (long t = 0; t < nc; ++t) Curve[t] = 0.0;
#pragma omp parallel for collapse(2)
    for (int k = 1; k <= G.N[2]; ++k)
        for (int j = 1; j <= G.N[1]; ++j)
            for (int i = 1; i <= G.N[0]; ++i) {
                const long c = G.c(i, j, k);
                Curve[c] = curvature_cell(G, VF, nx[c], ny[c], nz[c], i, j, k);
            }
    return 0;
}

/* compute_props! (src/Tools.jl:1186-1210) on every cell of the cell arrays: face VF
 * clamp((VF + VF[-1])/2, 0, 1), density rho_liq*vf + rho_gas*(1 - vf), viscosity
 * vf*mu_liq + (1 - vf)*mu_gas.  Null viscosity arrays give compute_dens! (:1212-1231). */
int orc_props(const orc_mesh* M, const double* VF, double rho_liq, double rho_gas, double mu_liq, double mu_gas,
              double* denx, double* deny, double* denz, double* viscx, double* viscy, double* viscz)
{
    Grid G(M);
    double* den[3] = {denx, deny, denz};
    double* visc[3] = {viscx, viscy, viscz};
    for (int d = 0; d < 3; ++d)
        for (int k = G.lo[2]; k <= G.hi[2]; ++k)
            for (int j = G.lo[1]; j <= G.hi[1]; ++j)
                for (int i = G.lo[0]; i <= G.hi[0]; ++i) {
                    const int a = i - (d == 0), b = j - (d == 1), c = k - (d == 2);
                    const double vf = jmin(1.0, jmax(0.0, (VF[G.v(i, j, k)] + VF[G.v(a, b, c)]) / 2));
                    const long t = G.c(i, j, k);
                    den[d][t] = rho_liq * vf + rho_gas * (1 - vf);
                    if (visc[d]) visc[d][t] = vf * mu_liq + (1 - vf) * mu_gas;
                }
    return 0;
}

/* Forward-mode derivatives of transport!'s SL update (the CPU analogue of ForwardDiff.jl's
 * Dual numbers): for each listed cell (i, j, k triples), VFnew and its derivatives with respect
 * to up to orc_ndual() face velocities, selected by the slot arrays su, sv, sw (cell-array
 * shaped: the derivative slot of each face value, -1 for none).  grad is ncells x orc_ndual(). */
int orc_ndual() { return NDUAL; }

/* Forward-mode derivatives of a rollout, the CPU analogue of a ForwardDiff.jl gradient of
 * run_solver's transport loop: from VF0, the initial state (Neumann + VF borders,
 * computeBand!, computeNormal!, computePLIC!), then `steps` steps (SL update of the band cells,
 * VF copy and ghost fill, normals, PLIC and band again), every value a Dual.  Up to NDUAL
 * directions are seeded: face values of the velocities (su/sv/sw: the slot of each parent entry,
 * -1 none; the same entry of every step's velocities, as for a perturbation added to every
 * step) and entries of VF0 (sVF, same convention, VF layout).  uf, vf, wf hold vel_steps
 * consecutive cell arrays: step s uses array min(s, vel_steps - 1) (1: frozen velocities).
 * The band is recomputed from the values, as it switches discretely.  L = sum of w * VF_T over
 * the interior (w: Nx*Ny*Nz, i fastest); dL[q] its derivative along direction q.  Cells are
 * processed in parallel (OpenMP); each cell's arithmetic is the restatement's. */
int orc_rollout_forward(const orc_mesh* M, double dt, int steps, int vel_steps, const double* VF0, const double* uf,
                        const double* vf, const double* wf, const int* su, const int* sv, const int* sw,
                        const int* sVF, const double* w, double* L, double* dL)
{
    Grid G(M);
    const long nvf = (long)G.vn[0] * G.vn[1] * G.vn[2], ncell = (long)G.n[0] * G.n[1] * G.n[2];
    std::vector<Dual> VF(nvf), VFn(nvf), nx(ncell), ny(ncell), nz(ncell), D(ncell);
    std::vector<double> vfv(nvf);
    std::vector<int16_t> band(ncell);
    for (long t = 0; t < nvf; ++t) {
        VF[t] = Dual(VF0[t]);
        if (sVF && sVF[t] >= 0) VF[t].d[sVF[t]] = 1.0;
    }
    int flags = 0;
    auto ghost = [&]() {
        Arr3<Dual> A(VF.data(), G.vlo, G.vhi);
        neumann(G, A);
        update_borders(G, A);
    };
    auto geometry = [&](bool do_band) {
        for (long t = 0; t < nvf; ++t) vfv[t] = VF[t].v;
        if (do_band) orc_compute_band(M, band.data(), vfv.data());
        std::fill(nx.begin(), nx.end(), Dual(0.0));
        std::fill(ny.begin(), ny.end(), Dual(0.0));
        std::fill(nz.begin(), nz.end(), Dual(0.0));
        FieldsT<Dual> F{&G, VF.data()};
        int fl = 0;
#pragma omp parallel for collapse(2) schedule(dynamic, 1) reduction(| : fl)
        for (int k = 1; k <= G.N[2]; ++k)
            for (int j = 1; j <= G.N[1]; ++j) {
                Err e;
                for (int i = 1; i <= G.N[0]; ++i)
                    elvira_cell<Dual, FieldsT<Dual>, Dual>(G, F, nx.data(), ny.data(), nz.data(), i, j, k, &e);
                fl |= e.flags;
            }
        flags |= fl;
        Arr3<Dual> A(nx.data(), G.lo, G.hi), B(ny.data(), G.lo, G.hi), C(nz.data(), G.lo, G.hi);
        update_borders(G, A); update_borders(G, B); update_borders(G, C);
#pragma omp parallel for collapse(2)
        for (int k = G.lo[2]; k <= G.hi[2]; ++k)
            for (int j = G.lo[1]; j <= G.hi[1]; ++j)
                for (int i = G.lo[0]; i <= G.hi[0]; ++i) {
                    const long c = G.c(i, j, k);
                    D[c] = compute_dist<Dual>(G, i, j, k, nx[c], ny[c], nz[c], VF[G.v(i, j, k)]);
                }
        Arr3<Dual> Dd(D.data(), G.lo, G.hi);
        update_borders(G, Dd);
    };
    ghost();
    geometry(true);
    for (int s = 0; s < steps; ++s) {
        const long off = (long)std::min(s, std::max(vel_steps, 1) - 1) * ncell;
        Vel V{uf + off, vf + off, wf + off, su, sv, sw};
        PlicT<Dual> P{nx.data(), ny.data(), nz.data(), D.data()};
        int fl = 0;
#pragma omp parallel for collapse(2) schedule(dynamic, 1) reduction(| : fl)
        for (int k = 1; k <= G.N[2]; ++k)
            for (int j = 1; j <= G.N[1]; ++j) {
                Err e;
                for (int i = 1; i <= G.N[0]; ++i) {
                    const long c = G.c(i, j, k), v = G.v(i, j, k);
                    if (std::abs((int)band[c]) <= M->nband)
                        VFn[v] = sl_cell<Dual, PlicT<Dual>>(G, V, P, dt, i, j, k, &e, nullptr);
                    else
                        VFn[v] = VF[v];
                }
                fl |= e.flags;
            }
        flags |= fl;
        for (int k = 1; k <= G.N[2]; ++k)
            for (int j = 1; j <= G.N[1]; ++j)
                for (int i = 1; i <= G.N[0]; ++i) VF[G.v(i, j, k)] = VFn[G.v(i, j, k)];
        ghost();
        geometry(true);
    }
    Dual acc(0.0);
    long q = 0;
    for (int k = 1; k <= G.N[2]; ++k)
        for (int j = 1; j <= G.N[1]; ++j)
            for (int i = 1; i <= G.N[0]; ++i, ++q) acc = acc + Dual(w[q]) * VF[G.v(i, j, k)];
    *L = acc.v;
    for (int d = 0; d < NDUAL; ++d) dL[d] = acc.d[d];
    return flags;
}

/* Algorithmic operation counts (see Cnt) of one step's per-cell parts, summed over the given
 * cells (interior cells as linear indices (i-1) + Nx*((j-1) + Ny*(k-1))), on one thread:
 *   out[0]  ELVIRA at the interface cells: elvira_calc, 27 (2D: 18) candidates, each
 *           normalised, computeDist, and computePLIC2VF of the 27 neighbours;
 *   out[1]  the plane constant at the interface cells (computeDist with the given normals);
 *   out[2]  the SL update at the band cells (sl_cell: the projected vertices and the clip).
 * vals, when given, receives the values the counted paths compute (3 normal components per
 * interface cell, then D per interface cell, then VFnew per band cell), which equal the
 * double paths' bit for bit. */
int orc_count_ops(const orc_mesh* M, double dt, const double* VF, const double* nx, const double* ny,
                  const double* nz, const double* D, const double* uf, const double* vf, const double* wf, int n_if,
                  const int* if_cells, int n_band, const int* band_cells, unsigned long long out[3], double* vals)
{
    Grid G(M);
    Fields F{&G, VF};
    Err e;
    const long ncell = (long)G.n[0] * G.n[1] * G.n[2];
    std::vector<double> sx(ncell, 0.0), sy(ncell, 0.0), sz(ncell, 0.0);
    auto ijk = [&](int L, int& i, int& j, int& k) {
        i = 1 + L % M->Nx;
        j = 1 + (L / M->Nx) % M->Ny;
        k = 1 + L / (M->Nx * M->Ny);
    };
    g_nops = 0;
    for (int q = 0; q < n_if; ++q) {
        int i, j, k;
        ijk(if_cells[q], i, j, k);
        elvira_calc<Cnt>(G, F, sx.data(), sy.data(), sz.data(), i, j, k, &e);
        if (vals) {
            const long c = G.c(i, j, k);
            vals[3 * q] = sx[c]; vals[3 * q + 1] = sy[c]; vals[3 * q + 2] = sz[c];
        }
    }
    out[0] = g_nops;
    g_nops = 0;
    for (int q = 0; q < n_if; ++q) {
        int i, j, k;
        ijk(if_cells[q], i, j, k);
        const long c = G.c(i, j, k);
        const Cnt d = compute_dist<Cnt>(G, i, j, k, Cnt(nx[c]), Cnt(ny[c]), Cnt(nz[c]), Cnt(VF[G.v(i, j, k)]));
        if (vals) vals[3 * n_if + q] = d.v;
    }
    out[1] = g_nops;
    g_nops = 0;
    Vel V{uf, vf, wf};
    Plic P{nx, ny, nz, D};
    for (int q = 0; q < n_band; ++q) {
        int i, j, k;
        ijk(band_cells[q], i, j, k);
        const Cnt r = sl_cell<Cnt>(G, V, P, dt, i, j, k, &e, nullptr);
        if (vals) vals[4 * n_if + q] = r.v;
    }
    out[2] = g_nops;
    g_nops = 0;
    return e.flags;
}

int orc_sl_forward(const orc_mesh* M, double dt, int ncells, const int* cells, const double* uf, const double* vf,
                   const double* wf, const int* su, const int* sv, const int* sw, const double* nx, const double* ny,
                   const double* nz, const double* D, double* vf_out, double* grad)
{
    Grid G(M);
    Vel V{uf, vf, wf, su, sv, sw};
    Plic P{nx, ny, nz, D};
    int flags = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : flags)
    for (int q = 0; q < ncells; ++q) {
        Err e;
        const Dual r = sl_cell<Dual>(G, V, P, dt, cells[3 * q], cells[3 * q + 1], cells[3 * q + 2], &e, nullptr);
        vf_out[q] = r.v;
        for (int s = 0; s < NDUAL; ++s) grad[(long)q * NDUAL + s] = r.d[s];
        flags |= e.flags;
    }
    return flags;
}

double orc_sl_flux_vol(const orc_mesh* M, int dir, int i, int j, int k, const double* uf, const double* vf,
                       const double* wf, double dt)
{
    Grid G(M);
    Vel V{uf, vf, wf};
    return sl_flux_vol(G, V, dir, i, j, k, dt);
}

/* Pre-image of one cell: projected vertices and indices + the SL result, for unit tests. */
double orc_sl_cell(const orc_mesh* M, double dt, int i, int j, int k, const double* uf, const double* vf,
                   const double* wf, const double* nx, const double* ny, const double* nz, const double* D,
                   double* vol_out, int* flags)
{
    Grid G(M);
    Vel V{uf, vf, wf};
    Plic P{nx, ny, nz, D};
    Err e;
    const double r = sl_cell(G, V, P, dt, i, j, k, &e, vol_out);
    if (flags) *flags = e.flags;
    return r;
}

int orc_project(const orc_mesh* M, double pt[3], int i, int j, int k, const double* uf, const double* vf,
                const double* wf, double dt)
{
    Grid G(M);
    Vel V{uf, vf, wf};
    project(G, V, pt, i, j, k, dt);
    return 0;
}

/* VFsphere's rule (src/Tools.jl:907-922) for a union of spheres (dims 3) or circles in x-y
 * (dims 2), over every cell of the cell-array extent (ghosts included): nF points per direction
 * at xmin + i/(nF+1)*(xmax-xmin); a point is liquid when rad^2 - ((xh-xo)^2 + (yh-yo)^2 +
 * (zh-zo)^2) > 0 for some sphere; VF is the sequential sum of count copies of 1/nF^dims.  Cells
 * whose box is entirely inside a sphere take the full sum without sampling.  The workload
 * generator of the CPU baseline (the GPU library generates the same field on the device); the
 * caller fills the VF ghost layers afterwards.  VF must be zeroed by the caller. */
int orc_vf_spheres(const orc_mesh* M, const double* cen, const double* rad, int ns, int nF, int dims, double* VF)
{
    Grid G(M);
    const int npts = dims == 3 ? nF * nF * nF : nF * nF;
    std::vector<double> table(npts + 1);
    const double sub = 1.0 / (double)npts;
    double acc = 0.0;
    table[0] = 0.0;
    for (int q = 1; q <= npts; ++q) { acc = acc + sub; table[q] = acc; }
#pragma omp parallel for collapse(2) schedule(dynamic, 4)
    for (int k = G.lo[2]; k <= G.hi[2]; ++k)
        for (int j = G.lo[1]; j <= G.hi[1]; ++j) {
            std::vector<int> cand;
            for (int i = G.lo[0]; i <= G.hi[0]; ++i) {
                const double x0 = G.x(i), x1 = G.x(i + 1), y0 = G.y(j), y1 = G.y(j + 1), z0 = G.z(k), z1 = G.z(k + 1);
                cand.clear();
                bool full = false;
                for (int s = 0; s < ns; ++s) {
                    const double cx = cen[3 * s], cy = cen[3 * s + 1], cz = cen[3 * s + 2], r = rad[s];
                    if (x1 < cx - r || x0 > cx + r || y1 < cy - r || y0 > cy + r) continue;
                    if (dims == 3 && (z1 < cz - r || z0 > cz + r)) continue;
                    const double fx = std::fmax(std::fabs(x0 - cx), std::fabs(x1 - cx));
                    const double fy = std::fmax(std::fabs(y0 - cy), std::fabs(y1 - cy));
                    const double fz = dims == 3 ? std::fmax(std::fabs(z0 - cz), std::fabs(z1 - cz)) : 0.0;
                    if (fx * fx + fy * fy + fz * fz < r * r * (1.0 - 1e-12)) { full = true; break; }
                    cand.push_back(s);
                }
                int cnt = 0;
                if (full) {
                    cnt = npts;
                } else if (!cand.empty()) {
                    const int nzp = dims == 3 ? nF : 1;
                    for (int c = 1; c <= nzp; ++c) {
                        const double zh = z0 + (double)c / (double)(nF + 1) * (z1 - z0);
                        for (int b = 1; b <= nF; ++b) {
                            const double yh = y0 + (double)b / (double)(nF + 1) * (y1 - y0);
                            for (int a = 1; a <= nF; ++a) {
                                const double xh = x0 + (double)a / (double)(nF + 1) * (x1 - x0);
                                bool hit = false;
                                for (size_t q = 0; q < cand.size() && !hit; ++q) {
                                    const int s = cand[q];
                                    const double r = rad[s];
                                    const double ex = xh - cen[3 * s], ey = yh - cen[3 * s + 1];
                                    double Gv;
                                    if (dims == 3) {
                                        const double ez = zh - cen[3 * s + 2];
                                        Gv = r * r - ((ex * ex + ey * ey) + ez * ez);
                                    } else {
                                        Gv = r * r - (ex * ex + ey * ey);
                                    }
                                    hit = Gv > 0.0;
                                }
                                cnt += hit;
                            }
                        }
                    }
                }
                VF[G.v(i, j, k)] = table[cnt];
            }
        }
    return 0;
}

/* Sum of interior VF * dx*dy*dz (src/WriteData.jl:33), Neumaier-compensated. */
double orc_mass(const orc_mesh* M, const double* VF)
{
    Grid G(M);
    const double cv = (M->dx * M->dy) * M->dz;
    double s = 0.0, comp = 0.0;
    for (int k = 1; k <= G.N[2]; ++k)
        for (int j = 1; j <= G.N[1]; ++j)
            for (int i = 1; i <= G.N[0]; ++i) {
                const double x = VF[G.v(i, j, k)] * cv;
                const double t = s + x;
                comp += std::fabs(s) >= std::fabs(x) ? (s - t) + x : (x - t) + s;
                s = t;
            }
    return s + comp;
}

/* One full step as the reference's transport! leaves the state (SL section):
 * SL update + VF ghosts (Transport.jl:108-181), ELVIRA (:184), computePLIC! (:260);
 * then, if do_band, computeBand! as run_solver does next (NavierStokes_Parallel.jl:143). */
int orc_step(const orc_mesh* M, double dt, double* VF, double* VFnew, const double* uf, const double* vf,
             const double* wf, double* nx, double* ny, double* nz, double* D, int16_t* band, int do_band)
{
    int f = orc_transport(M, dt, VF, VFnew, uf, vf, wf, nx, ny, nz, D, band, 1, 0);
    f |= orc_elvira(M, VF, nx, ny, nz, 1, 0);
    f |= orc_compute_plic(M, D, nx, ny, nz, VF);
    if (do_band) f |= orc_compute_band(M, band, VF);
    return f;
}

} // extern "C"
