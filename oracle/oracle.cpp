// CPU oracle for the curvedSpaceSim per-timestep hot path.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library, its C ABI or the host classes) links,
// loads or calls this file; only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / --impl reference
// legs use it, as the checker and as the timed CPU baseline.
//
// Parity status: UNPINNED against the reference itself.  The reference computes geodesics with CGAL's
// Surface_mesh_shortest_path (CGAL 5.6 / 5.6.1 requested by Installation.md:7-16, not vendored, no lockfile), and
// neither CGAL nor Boost/GMP/MPFR is available here, so the reference cannot be built; it also ships no tests or
// golden vectors.  This oracle is pinned instead against closed-form known answers (planar, developable prism and
// cone, cube unfoldings) and against an independent brute-force edge-sequence unfolding solver (below).
//
// Contents, each restating the cited reference code:
//   * mesh helpers   - barycentric_coordinates / construct_point / compute_face_normal formulas used through CGAL PMP
//   * walk           - triangulatedMeshSpace::transportParticleAndVectors + helpers
//                      (src/models/triangulatedMeshSpace.cpp:247-407, 448-658; src/utility/meshUtilities.cpp:138-331;
//                       src/utility/functionUtilities.cpp:8-45)
//   * patch          - submesher::constructSubmeshFromSourceAndTargets (src/utility/submesher.cpp:55-147)
//   * geodesics      - exact polyhedral distances by continuous-Dijkstra window propagation (the Chen-Han /
//                      Xin-Wang family named in Citations.md:9-21), written from the published method, replacing the
//                      CGAL calls of triangulatedMeshSpace::distance / distanceWithSubmeshing (:155-238) and
//                      computePathDistanceAndTangents (meshUtilities.cpp:360-380)
//   * brute force    - independent exact solver by enumerating unfoldings along face sequences (checker of the above)
//   * candidates     - cellListNeighborStructure::constructCandidateNeighborList + hyperRectangularCellList
//                      (src/utility/cellListNeighborStructure.cpp:45-84, hyperRectangularCellList.cpp:9-159) and the
//                      all-to-all baseNeighborStructure (baseNeighborStructure.cpp:17-36)
//   * forces         - force::computeForces / computeEnergy (src/forces/baseForce.cpp:12-44), harmonicRepulsion
//                      (harmonicRepulsion.cpp:3-34), gaussianRepulsion (gaussianRepulsion.cpp:3-12)
//   * integrators    - velocityVerletNVE (src/updaters/velocityVerletNVE.cpp:3-29), noseHooverNVT
//                      (src/updaters/noseHooverNVT.cpp:3-150), simpleModel::moveParticles / findNeighbors
//                      (src/models/simpleModel.cpp:44-112)
//   * open meshes    - the walk's border branches of openMeshSpace / tangentialOpenMeshSpace / absorbingOpenMeshSpace
//                      (src/models/openMeshSpace.cpp:114-238, tangentialOpenMeshSpace.cpp:3-64,
//                       absorbingOpenMeshSpace.cpp:2-50)
//   * minimisers     - fireMinimization::minimizeByFire / fireStep (src/updaters/fireMinimization.cpp:3-96); the
//                      gradient-descent updater (gradientDescent.cpp:6-18) is composed in oracle/__init__.py from the
//                      forces and the walk
//   * analysis       - simulation::computeMonodisperseStress (src/simulation/simulation.cpp:104-173)
//
// Build: see oracle/build.sh (g++ -O2 -ffp-contract=off -fopenmp, no -ffast-math).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <queue>
#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double kInf = std::numeric_limits<double>::infinity();
const double kPi = 3.14159265358979323846;

// status codes shared with the CUDA library (see include/cssg.h)
enum {
    ST_OK = 0,
    ST_BORDER = 1,
    ST_NAN = 2,
    ST_VERTEX = 3,
    ST_ITER = 4,
    ST_NO_INTERSECTION = 5,
    ST_CAPACITY = 6,
};

inline void sub3(const double* a, const double* b, double* o) { o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2]; }
inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline void cross3(const double* a, const double* b, double* o)
{
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
inline double norm3(const double* a) { return std::sqrt(dot3(a, a)); }
inline double len2(double x, double y) { return std::sqrt(x * x + y * y); }

// ------------------------------------------------------------------------------------------------------------------
// Mesh
// ------------------------------------------------------------------------------------------------------------------
struct Mesh {
    int nV = 0, nF = 0;
    std::vector<double> V;      // 3 nV
    std::vector<int> F;         // 3 nF, vertex order defines barycentric order
    std::vector<int> twin;      // 3 nF: neighbour across local edge k (F[k] -> F[k+1]) as face*3 + local edge, -1 border
    std::vector<double> N;      // 3 nF unit normals
    std::vector<double> EL;     // 3 nF edge length of local edge k
    std::vector<double> CX, CY; // 3 nF third vertex F[k+2] in the frame (origin F[k], x to F[k+1], y into the face)
    std::vector<int> vfStart, vfList;  // vertex -> incident faces (CSR)
    std::vector<int> ringStart, ringV, ringF;  // closed vertices only: clockwise neighbour ring and spanned faces
    std::vector<char> ringOk;
    std::vector<double> angleSum;
    std::vector<char> borderV;
    double bbMin[3], bbMax[3];
    double area = 0;
};

inline const double* vp(const Mesh& M, int v) { return &M.V[3 * v]; }

void build_mesh(Mesh& M, const double* V, int nV, const int* F, int nF)
{
    M.nV = nV;
    M.nF = nF;
    M.V.assign(V, V + 3 * nV);
    M.F.assign(F, F + 3 * nF);
    M.twin.assign(3 * nF, -1);
    std::unordered_map<uint64_t, int> edge;
    edge.reserve(3 * nF);
    for (int f = 0; f < nF; ++f)
        for (int k = 0; k < 3; ++k) {
            uint64_t a = (uint64_t)F[3 * f + k], b = (uint64_t)F[3 * f + (k + 1) % 3];
            edge[(a << 32) | b] = 3 * f + k;
        }
    for (int f = 0; f < nF; ++f)
        for (int k = 0; k < 3; ++k) {
            uint64_t a = (uint64_t)F[3 * f + k], b = (uint64_t)F[3 * f + (k + 1) % 3];
            auto it = edge.find((b << 32) | a);
            if (it != edge.end()) M.twin[3 * f + k] = it->second;
        }
    M.N.assign(3 * nF, 0.0);
    M.EL.assign(3 * nF, 0.0);
    M.CX.assign(3 * nF, 0.0);
    M.CY.assign(3 * nF, 0.0);
    M.area = 0;
    for (int f = 0; f < nF; ++f) {
        const double *p0 = vp(M, F[3 * f]), *p1 = vp(M, F[3 * f + 1]), *p2 = vp(M, F[3 * f + 2]);
        double e1[3], e2[3], n[3];
        sub3(p1, p0, e1);
        sub3(p2, p0, e2);
        cross3(e1, e2, n);
        double nn = norm3(n);
        M.area += 0.5 * nn;
        for (int c = 0; c < 3; ++c) M.N[3 * f + c] = n[c] / nn;
        for (int k = 0; k < 3; ++k) {
            const double* A = vp(M, F[3 * f + k]);
            const double* B = vp(M, F[3 * f + (k + 1) % 3]);
            const double* C = vp(M, F[3 * f + (k + 2) % 3]);
            double ab[3], ac[3], cr[3];
            sub3(B, A, ab);
            sub3(C, A, ac);
            double L = norm3(ab);
            cross3(ab, ac, cr);
            M.EL[3 * f + k] = L;
            M.CX[3 * f + k] = dot3(ac, ab) / L;
            M.CY[3 * f + k] = norm3(cr) / L;
        }
    }
    // vertex -> faces
    M.vfStart.assign(nV + 1, 0);
    for (int i = 0; i < 3 * nF; ++i) M.vfStart[F[i] + 1]++;
    for (int v = 0; v < nV; ++v) M.vfStart[v + 1] += M.vfStart[v];
    M.vfList.assign(3 * nF, 0);
    std::vector<int> fill(M.vfStart.begin(), M.vfStart.end() - 1);
    for (int f = 0; f < nF; ++f)
        for (int k = 0; k < 3; ++k) M.vfList[fill[F[3 * f + k]]++] = f;
    // angle sums and border flags
    M.angleSum.assign(nV, 0.0);
    M.borderV.assign(nV, 0);
    for (int f = 0; f < nF; ++f)
        for (int k = 0; k < 3; ++k) {
            if (M.twin[3 * f + k] < 0) {
                M.borderV[F[3 * f + k]] = 1;
                M.borderV[F[3 * f + (k + 1) % 3]] = 1;
            }
            const double* A = vp(M, F[3 * f + k]);
            const double* B = vp(M, F[3 * f + (k + 1) % 3]);
            const double* C = vp(M, F[3 * f + (k + 2) % 3]);
            double ab[3], ac[3];
            sub3(B, A, ab);
            sub3(C, A, ac);
            double c = dot3(ab, ac) / (norm3(ab) * norm3(ac));
            c = std::max(-1.0, std::min(1.0, c));
            M.angleSum[F[3 * f + k]] += std::acos(c);
        }
    // clockwise rings (the order CGAL's Vertex_around_target_circulator visits, used by throughVertex)
    M.ringStart.assign(nV + 1, 0);
    M.ringOk.assign(nV, 0);
    std::vector<std::vector<int>> rv(nV), rf(nV);
    for (int v = 0; v < nV; ++v) {
        if (M.borderV[v] || M.vfStart[v + 1] == M.vfStart[v]) continue;
        int f0 = M.vfList[M.vfStart[v]];
        int f = f0;
        int k = 0;
        while (F[3 * f + k] != v) ++k;
        rv[v].push_back(F[3 * f + (k + 2) % 3]);
        int guard = 0;
        bool ok = true;
        while (true) {
            int nxt = F[3 * f + (k + 1) % 3];
            rv[v].push_back(nxt);
            rf[v].push_back(f);
            int t = M.twin[3 * f + k];
            if (t < 0) { ok = false; break; }
            f = t / 3;
            k = 0;
            while (F[3 * f + k] != v) ++k;
            if (f == f0) break;
            if (++guard > 1000) { ok = false; break; }
        }
        if (ok) {
            rv[v].pop_back();  // last pushed neighbour repeats the first
            M.ringOk[v] = 1;
        }
    }
    for (int v = 0; v < nV; ++v) M.ringStart[v + 1] = M.ringStart[v] + (M.ringOk[v] ? (int)rv[v].size() : 0);
    M.ringV.resize(M.ringStart[nV]);
    M.ringF.resize(M.ringStart[nV]);
    for (int v = 0; v < nV; ++v)
        if (M.ringOk[v])
            for (size_t i = 0; i < rv[v].size(); ++i) {
                M.ringV[M.ringStart[v] + i] = rv[v][i];
                M.ringF[M.ringStart[v] + i] = rf[v][i];
            }
    // the reference's cell-list domain starts from the origin and grows to the vertex span
    // (triangulatedMeshSpace::updateMeshSpanAndTree, triangulatedMeshSpace.cpp:6-30)
    for (int c = 0; c < 3; ++c) { M.bbMin[c] = 0; M.bbMax[c] = 0; }
    for (int v = 0; v < nV; ++v)
        for (int c = 0; c < 3; ++c) {
            M.bbMin[c] = std::min(M.bbMin[c], V[3 * v + c]);
            M.bbMax[c] = std::max(M.bbMax[c], V[3 * v + c]);
        }
}

// ------------------------------------------------------------------------------------------------------------------
// CGAL PMP formulas restated (barycentric_coordinates, construct_point/barycenter)
// ------------------------------------------------------------------------------------------------------------------
void bary_of(const double* p, const double* q, const double* r, const double* x, double* out)
{
    double v0[3], v1[3], v2[3];
    sub3(q, p, v0);
    sub3(r, p, v1);
    sub3(x, p, v2);
    double d00 = dot3(v0, v0), d01 = dot3(v0, v1), d11 = dot3(v1, v1);
    double d20 = dot3(v2, v0), d21 = dot3(v2, v1);
    double denom = d00 * d11 - d01 * d01;
    double v = (d11 * d20 - d01 * d21) / denom;
    double w = (d00 * d21 - d01 * d20) / denom;
    out[0] = 1.0 - v - w;
    out[1] = v;
    out[2] = w;
}

void construct_pt(const double* p0, const double* p1, const double* p2, const double* b, double* out)
{
    double s = b[0] + b[1] + b[2];
    for (int c = 0; c < 3; ++c) out[c] = (b[0] * p0[c] + b[1] * p1[c] + b[2] * p2[c]) / s;
}

void face_pts(const Mesh& M, int f, const double** p)
{
    p[0] = vp(M, M.F[3 * f]);
    p[1] = vp(M, M.F[3 * f + 1]);
    p[2] = vp(M, M.F[3 * f + 2]);
}

// meshUtilities.cpp:138-168
void below_zero_clamp(double* b, double tol = 1e-11)
{
    double s = 0;
    for (int i = 0; i < 3; ++i) {
        b[i] = std::max(b[i], tol);
        s += b[i];
    }
    for (int i = 0; i < 3; ++i) b[i] = b[i] / s;
}

void near_zero_clamp(double* b, double tol = 1e-13)
{
    double s = 0;
    for (int i = 0; i < 3; ++i) {
        if (b[i] > -tol && b[i] < tol) b[i] = tol;
        s += b[i];
    }
    for (int i = 0; i < 3; ++i) b[i] = b[i] / s;
}

// ------------------------------------------------------------------------------------------------------------------
// Walk: restatement of transportParticleAndVectors and helpers
// ------------------------------------------------------------------------------------------------------------------
// meshUtilities.cpp:229-281: the segment start->end against the three edges in barycentric form
bool hit_v1v2(const double* s, const double* e, double* ip)
{
    double den = s[0] + s[1] - e[0] - e[1];
    if (den == 0) return false;
    double t1 = (-e[1] + e[1] * s[0] + s[1] - e[0] * s[1]) / den;
    double t2 = (-1 + s[0] + s[1]) / den;
    for (int c = 0; c < 3; ++c) ip[c] = s[c] + t2 * (e[c] - s[c]);
    return t1 >= 0 && t1 <= 1 && t2 >= 0 && t2 <= 1;
}
bool hit_v2v3(const double* s, const double* e, double* ip)
{
    double den = -e[0] + s[0];
    if (den == 0) return false;
    double t1 = -(e[0] - s[0] + e[1] * s[0] - e[0] * s[1]) / den;
    double t2 = s[0] / den;
    for (int c = 0; c < 3; ++c) ip[c] = s[c] + t2 * (e[c] - s[c]);
    return t1 >= 0 && t1 <= 1 && t2 >= 0 && t2 <= 1;
}
bool hit_v3v1(const double* s, const double* e, double* ip)
{
    double den = s[1] - e[1];
    if (den == 0) return false;
    double t1 = (e[0] * s[1] - e[1] * s[0]) / den;
    double t2 = s[1] / den;
    for (int c = 0; c < 3; ++c) ip[c] = s[c] + t2 * (e[c] - s[c]);
    return t1 >= 0 && t1 <= 1 && t2 >= 0 && t2 <= 1;
}

// Rodrigues rotation of point p about the axis through o with unit direction a (functionUtilities.cpp:8-32).
// cos/sin of the angle are passed directly: for the edge and vertex crossings they are n_s.n_t and |n_s x n_t|,
// the cosine and sine of acos(n_s.n_t) that the reference evaluates.
void rotate_about(const double* p, const double* o, const double* a, double c, double s, double* out)
{
    double sh[3];
    sub3(p, o, sh);
    double d = a[0] * sh[0] + a[1] * sh[1] + a[2] * sh[2];
    double r0 = a[0] * d * (1. - c) + sh[0] * c + (a[1] * sh[2] - a[2] * sh[1]) * s;
    double r1 = a[1] * d * (1. - c) + sh[1] * c + (a[2] * sh[0] - a[0] * sh[2]) * s;
    double r2 = a[2] * d * (1. - c) + sh[2] * c + (a[0] * sh[1] - a[1] * sh[0]) * s;
    out[0] = r0 + o[0];
    out[1] = r1 + o[1];
    out[2] = r2 + o[2];
}

double angle_between(const double* u, const double* v)
{
    double a[3] = {u[0], u[1], u[2]}, b[3] = {v[0], v[1], v[2]};
    double na = norm3(a), nb = norm3(b);
    for (int c = 0; c < 3; ++c) { a[c] /= na; b[c] /= nb; }
    double d = dot3(a, b);
    if (d >= 1) return 0;
    if (d <= -1) return kPi;
    return std::acos(d);
}

int face_across(const Mesh& M, int f, int va, int vb)
{
    for (int k = 0; k < 3; ++k) {
        int a = M.F[3 * f + k], b = M.F[3 * f + (k + 1) % 3];
        if ((a == va && b == vb) || (a == vb && b == va)) {
            int t = M.twin[3 * f + k];
            return t < 0 ? -1 : t / 3;
        }
    }
    return -1;
}

// triangulatedMeshSpace::throughVertex (triangulatedMeshSpace.cpp:247-407)
int through_vertex(const Mesh& M, int v, const double* toInter, int srcFace, int* outFace, double* heading)
{
    if (!M.ringOk[v]) return ST_BORDER;
    const double* vi = vp(M, v);
    int startV = -1;
    for (int k = 0; k < 3; ++k)
        if (M.F[3 * srcFace + k] == v) startV = M.F[3 * srcFace + (k + 1) % 3];
    int b = M.ringStart[v], n = M.ringStart[v + 1] - b;
    int s0 = -1;
    for (int i = 0; i < n; ++i)
        if (M.ringV[b + i] == startV) s0 = i;
    if (s0 < 0) return ST_VERTEX;
    std::vector<int> nb(n);
    std::vector<double> ev(3 * n);
    for (int i = 0; i < n; ++i) {
        nb[i] = M.ringV[b + (s0 + i) % n];
        double e[3];
        sub3(vp(M, nb[i]), vi, e);
        double l = norm3(e);
        for (int c = 0; c < 3; ++c) ev[3 * i + c] = e[c] / l;
    }
    double total = 0;
    for (int i = 0; i < n; ++i) total += angle_between(&ev[3 * i], &ev[3 * ((i + 1) % n)]);
    double half = total / 2.0;
    double qh[3] = {-toInter[0], -toInter[1], -toInter[2]};
    double ql = norm3(qh);
    for (int c = 0; c < 3; ++c) qh[c] /= ql;
    double traveled = angle_between(qh, &ev[0]);
    int counter = 0;
    while (traveled < half) {
        traveled += angle_between(&ev[3 * counter], &ev[3 * ((counter + 1) % n)]);
        counter++;
        if (counter >= n) return ST_VERTEX;  // the reference prints and then reads past the ring
    }
    if (counter == 0) return ST_VERTEX;      // the reference reads edgeVectors[-1] here
    double diff = half - traveled;
    double ax[3];
    cross3(&ev[3 * (counter - 1)], &ev[3 * counter], ax);
    double al = norm3(ax);
    for (int c = 0; c < 3; ++c) ax[c] /= al;
    double rt[3] = {vi[0] + ev[3 * counter], vi[1] + ev[3 * counter + 1], vi[2] + ev[3 * counter + 2]};
    double pr[3];
    rotate_about(rt, vi, ax, std::cos(diff), std::sin(diff), pr);
    double h[3];
    sub3(pr, vi, h);
    double hl = norm3(h);
    for (int c = 0; c < 3; ++c) heading[c] = h[c] / hl;
    int want1 = nb[counter - 1], want2 = nb[counter];
    int tf = srcFace;
    for (int i = M.vfStart[v]; i < M.vfStart[v + 1]; ++i) {
        int f = M.vfList[i];
        if (f == srcFace) continue;
        bool h1 = false, h2 = false;
        for (int k = 0; k < 3; ++k) {
            h1 |= M.F[3 * f + k] == want1;
            h2 |= M.F[3 * f + k] == want2;
        }
        if (h1 && h2) { tf = f; break; }
    }
    if (tf == srcFace) return ST_VERTEX;
    *outFace = tf;
    return ST_OK;
}

// Open-mesh boundary conditions (src/models/openMeshSpace.cpp, tangentialOpenMeshSpace.cpp,
// absorbingOpenMeshSpace.cpp).  0: closed mesh (a border is an error), 1: tangential, 2: absorbing.
enum { BC_CLOSED = 0, BC_TANGENTIAL = 1, BC_ABSORBING = 2 };

inline void normalize3(double* v)
{
    const double l = norm3(v);
    for (int c = 0; c < 3; ++c) v[c] = v[c] / l;
}

// triangulatedMeshSpace::projectVectorsIfOverBoundary (triangulatedMeshSpace.cpp:411-426) with
// projectVectorOrthogonalToDirection (meshUtilities.cpp:125-129)
void project_if_over_boundary(double* tv, int ntv, const double* orthogonal, const double* inward)
{
    const bool pointsOut = dot3(orthogonal, inward) < 0;
    double dh[3] = {orthogonal[0], orthogonal[1], orthogonal[2]};
    normalize3(dh);
    for (int i = 0; i < ntv; ++i) {
        double* v = &tv[3 * i];
        const bool alongPerp = dot3(v, orthogonal) > 0;
        if ((pointsOut && alongPerp) || (!pointsOut && !alongPerp)) {
            const double d = dot3(v, dh);
            for (int c = 0; c < 3; ++c) v[c] = v[c] - d * dh[c];
        }
    }
}

// openMeshSpace::getBoundaryVertexHeading (openMeshSpace.cpp:3-75), by its stated rule: the next heading runs along
// the edge from v that overlaps most with the displacement, among the edges of v's faces other than the current one.
// The reference collects its (neighbour, face) candidates with a vertex circulator that advances once per face
// compared, so which pairs it sees depends on CGAL's per-vertex halfedge choice; here every (neighbour, face) pair
// around v is a candidate, faces in increasing index order, the first maximum kept.  Returns the new face and the
// neighbour, or -1 (the reference's "New face not found").
int boundary_vertex_heading(const Mesh& M, int v, int f, const double* disp, double* heading, int* neighbour)
{
    double dn[3] = {disp[0], disp[1], disp[2]};
    normalize3(dn);
    double best = -1;
    int bestFace = -1;
    for (int i = M.vfStart[v]; i < M.vfStart[v + 1]; ++i) {
        const int g = M.vfList[i];
        if (g == f) continue;
        for (int k = 0; k < 3; ++k) {
            const int w = M.F[3 * g + k];
            if (w == v) continue;
            double out[3];
            sub3(vp(M, w), vp(M, v), out);
            normalize3(out);
            const double ov = dot3(out, dn);
            if (ov > best) {
                best = ov;
                bestFace = g;
                *neighbour = w;
                for (int c = 0; c < 3; ++c) heading[c] = out[c];
            }
        }
    }
    return bestFace;
}

// openMeshSpace::projectVectorsForBoundaryVertex (openMeshSpace.cpp:77-99)
void project_for_boundary_vertex(const Mesh& M, const double* heading, int v, int w, const double* fNormal, int g,
                                 double* tv, int ntv)
{
    double orth[3];
    cross3(fNormal, heading, orth);
    normalize3(orth);
    int inside = -1;
    for (int k = 0; k < 3; ++k) {
        const int u = M.F[3 * g + k];
        if (u == v || u == w) continue;
        inside = u;
    }
    double inward[3] = {0, 0, 0};
    if (inside >= 0) sub3(vp(M, inside), vp(M, v), inward);
    else for (int c = 0; c < 3; ++c) inward[c] = -vp(M, v)[c];  // the reference's insideVertex stays (0,0,0)
    project_if_over_boundary(tv, ntv, orth, inward);
}

int g_bc = BC_CLOSED;  // boundary condition used by the oracle's API entry points (oracle_set_boundary)

// triangulatedMeshSpace::transportParticleAndVectors (triangulatedMeshSpace.cpp:448-564); with bc != 0 the loop of
// openMeshSpace::transportParticleAndVectors (openMeshSpace.cpp:101-238), which differs only at border edges and
// vertices
int transport_one(const Mesh& M, int& face, double* bary, double* disp, double* tv, int ntv, int maxIter, int* crossings,
                  int bc = BC_CLOSED)
{
    int f = face;
    const double* p[3];
    face_pts(M, f, p);
    double sb[3] = {bary[0], bary[1], bary[2]};
    double sp[3];
    construct_pt(p[0], p[1], p[2], sb, sp);
    double ns[3] = {M.N[3 * f], M.N[3 * f + 1], M.N[3 * f + 2]};
    double nd = dot3(ns, disp);
    if (std::fabs(nd) > 1e-14)
        for (int c = 0; c < 3; ++c) disp[c] -= nd * ns[c];
    double target[3] = {sp[0] + disp[0], sp[1] + disp[1], sp[2] + disp[2]};
    int lastA = -1, lastB = -1;
    double tb[3];
    int iter = 0;
    int cross = 0;
    // qf: the face whose vertex positions the target's weights are computed against.  The reference keeps them in
    // vertexPositions, which updateForEdgeIntersection refreshes (by reference, :614-658) but
    // updateForVertexIntersection (:566-611) and getBoundaryVertexHeading (openMeshSpace.cpp:3-66) receive by value:
    // after a vertex crossing the next passes weigh the target against the triangle of the face before the vertex
    // (the weights are then read in the new face by clampAndUpdatePosition, meshUtilities.cpp:170-182).
    int qf = f;
    while (true) {
        if (++iter > maxIter) return ST_ITER;
        {
            const double* q[3];
            face_pts(M, qf, q);
            bary_of(q[0], q[1], q[2], target, tb);
        }
        near_zero_clamp(tb);
        construct_pt(p[0], p[1], p[2], tb, target);
        below_zero_clamp(sb);
        construct_pt(p[0], p[1], p[2], sb, sp);
        sub3(target, sp, disp);
        if (tb[0] != tb[0]) return ST_NAN;
        if (tb[0] >= 0 && tb[1] >= 0 && tb[2] >= 0) break;
        const int* vl = &M.F[3 * f];
        double ip[3], ic[3];
        int nhit = 0;
        int inv0 = -1, inv1 = -1;
        auto isLast = [&](int a, int b) { return (a == lastA && b == lastB) || (a == lastB && b == lastA); };
        if (!isLast(vl[0], vl[1]) && hit_v1v2(sb, tb, ic)) {
            for (int c = 0; c < 3; ++c) ip[c] = ic[c];
            if (nhit == 0) { inv0 = vl[0]; inv1 = vl[1]; }
            nhit++;
        }
        if (!isLast(vl[1], vl[2]) && hit_v2v3(sb, tb, ic)) {
            for (int c = 0; c < 3; ++c) ip[c] = ic[c];
            if (nhit == 0) { inv0 = vl[1]; inv1 = vl[2]; }
            nhit++;
        }
        if (!isLast(vl[2], vl[0]) && hit_v3v1(sb, tb, ic)) {
            for (int c = 0; c < 3; ++c) ip[c] = ic[c];
            if (nhit == 0) { inv0 = vl[2]; inv1 = vl[0]; }
            nhit++;
        }
        if (nhit == 0) return ST_NO_INTERSECTION;
        below_zero_clamp(ip);
        double ep[3];
        construct_pt(p[0], p[1], p[2], ip, ep);
        double toI[3];
        sub3(ep, sp, toI);
        for (int c = 0; c < 3; ++c) { sb[c] = ip[c]; sp[c] = ep[c]; }
        cross++;
        if (nhit == 2) {
            // vertex crossing (triangulatedMeshSpace.cpp:520-532, 566-611); like the reference, the vertex passed on
            // is the first vertex of the first edge that reported a hit
            int v = inv0;
            if (!M.borderV[v]) cross += (1 << 16) - 1;  // crossings of interior vertices are counted in the high half
            if (M.borderV[v]) {
                if (bc == BC_CLOSED) return ST_BORDER;
                // updateAtBoundaryVertex (tangentialOpenMeshSpace.cpp:41-64, absorbingOpenMeshSpace.cpp:28-50)
                double heading[3];
                int w = -1;
                const int g = boundary_vertex_heading(M, v, f, disp, heading, &w);
                if (g < 0) return ST_VERTEX;
                f = g;
                face_pts(M, f, p);
                bary_of(p[0], p[1], p[2], vp(M, v), sb);
                if (ntv > 0) project_for_boundary_vertex(M, heading, v, w, ns, f, tv, ntv);
                // getBoundaryVertexHeading receives vertexPositions and sourceNormal by value, so the caller keeps the
                // previous face's: qf and ns are not updated here
                lastA = lastB = -1;
                if (bc == BC_ABSORBING) {
                    for (int c = 0; c < 3; ++c) tb[c] = sb[c];
                    break;
                }
                // projectVectorOntoDirection (meshUtilities.cpp:119-123)
                double hh[3] = {heading[0], heading[1], heading[2]};
                normalize3(hh);
                const double d2 = dot3(disp, hh);
                construct_pt(p[0], p[1], p[2], sb, sp);
                for (int c = 0; c < 3; ++c) {
                    disp[c] = d2 * hh[c];
                    target[c] = sp[c] + disp[c];
                }
                continue;
            }
            int g;
            double heading[3];
            int st = through_vertex(M, v, toI, f, &g, heading);
            if (st) return st;
            double len = norm3(disp);  // remaining length measured before moving to the vertex, as the reference does
            double nt[3] = {M.N[3 * g], M.N[3 * g + 1], M.N[3 * g + 2]};
            for (int c = 0; c < 3; ++c) {
                disp[c] = heading[c] * len;
                target[c] = sp[c] + disp[c];
            }
            if (ntv > 0) {
                double ndt = dot3(ns, nt);
                if (ndt < 0) {
                    double ax[3];
                    cross3(ns, nt, ax);
                    double al = norm3(ax);
                    for (int c = 0; c < 3; ++c) ax[c] /= al;
                    for (int i = 0; i < ntv; ++i) {
                        double q[3] = {sp[0] + tv[3 * i], sp[1] + tv[3 * i + 1], sp[2] + tv[3 * i + 2]};
                        double r[3];
                        rotate_about(q, sp, ax, ndt, al, r);
                        sub3(r, sp, &tv[3 * i]);
                    }
                }
            }
            f = g;
            face_pts(M, f, p);
            bary_of(p[0], p[1], p[2], sp, sb);
            for (int c = 0; c < 3; ++c) ns[c] = nt[c];
            lastA = lastB = -1;
            continue;
        }
        if (nhit != 1) return ST_NO_INTERSECTION;
        // edge crossing (triangulatedMeshSpace.cpp:543-557, 614-658)
        int g = face_across(M, f, inv0, inv1);
        if (g < 0) {
            if (bc == BC_CLOSED) return ST_BORDER;
            // updateAtBoundaryEdge (tangentialOpenMeshSpace.cpp:3-39, absorbingOpenMeshSpace.cpp:2-26)
            int inner = -1;
            for (int k = 0; k < 3; ++k)
                if (M.F[3 * f + k] != inv0 && M.F[3 * f + k] != inv1) inner = M.F[3 * f + k];
            double edge[3], orth[3], inward[3], here[3];
            sub3(vp(M, inv1), vp(M, inv0), edge);
            // the absorbing rule recomputes the face normal (absorbingOpenMeshSpace.cpp:14), the tangential rule uses
            // the loop's sourceNormal (tangentialOpenMeshSpace.cpp:22)
            cross3(bc == BC_ABSORBING ? &M.N[3 * f] : ns, edge, orth);
            normalize3(orth);
            construct_pt(p[0], p[1], p[2], sb, here);
            sub3(vp(M, inner), here, inward);
            if (bc == BC_ABSORBING) {
                if (ntv > 0) project_if_over_boundary(tv, ntv, orth, inward);
                for (int c = 0; c < 3; ++c) tb[c] = sb[c];
                break;
            }
            double fwd[3] = {edge[0], edge[1], edge[2]}, bwd[3];
            sub3(vp(M, inv0), vp(M, inv1), bwd);
            normalize3(fwd);
            normalize3(bwd);
            double dn[3] = {disp[0], disp[1], disp[2]};
            normalize3(dn);
            const double fd = dot3(dn, fwd), bd = dot3(dn, bwd);
            const double len = norm3(disp);  // the whole remaining displacement, measured before the edge was reached
            project_if_over_boundary(tv, ntv, orth, inward);
            const bool stop = fd <= 0 && bd <= 0;
            for (int c = 0; c < 3; ++c) {
                disp[c] = fd > bd ? fd * len * fwd[c] : bd * len * bwd[c];
                target[c] = here[c] + disp[c];
            }
            lastA = lastB = -1;
            if (stop) break;  // the reference then writes the target weights found at the top of this pass
            continue;
        }
        construct_pt(p[0], p[1], p[2], ip, sp);
        double nt[3] = {M.N[3 * g], M.N[3 * g + 1], M.N[3 * g + 2]};
        double ndt = dot3(ns, nt);
        // the reference also divides by |n_s x n_t| here; for coplanar faces whose normals' dot product rounds
        // below 1 that length is exactly zero (NaN there); the rotation is then the identity and is skipped
        if (ndt < 1 && (ns[0] * nt[1] - ns[1] * nt[0] != 0 || ns[1] * nt[2] - ns[2] * nt[1] != 0 ||
                        ns[2] * nt[0] - ns[0] * nt[2] != 0)) {
            double ax[3];
            cross3(ns, nt, ax);
            double al = norm3(ax);
            for (int c = 0; c < 3; ++c) ax[c] /= al;
            double r[3];
            rotate_about(target, sp, ax, ndt, al, r);
            for (int c = 0; c < 3; ++c) target[c] = r[c];
            sub3(target, sp, disp);
            for (int i = 0; i < ntv; ++i) {
                double q[3] = {sp[0] + tv[3 * i], sp[1] + tv[3 * i + 1], sp[2] + tv[3 * i + 2]};
                rotate_about(q, sp, ax, ndt, al, r);
                sub3(r, sp, &tv[3 * i]);
            }
        }
        lastA = inv0;
        lastB = inv1;
        f = g;
        qf = g;
        face_pts(M, f, p);
        bary_of(p[0], p[1], p[2], sp, sb);
        for (int c = 0; c < 3; ++c) ns[c] = nt[c];
    }
    face = f;
    bary[0] = tb[0];
    bary[1] = tb[1];
    bary[2] = tb[2];
    if (crossings) *crossings = cross;
    return ST_OK;
}

// ------------------------------------------------------------------------------------------------------------------
// Patch: submesher::constructSubmeshFromSourceAndTargets (submesher.cpp:55-147)
// ------------------------------------------------------------------------------------------------------------------
void build_patch(const Mesh& M, int f0, const double* b0, const int* tFace, int nT, double r, std::vector<int>& out)
{
    out.clear();
    const double* p[3];
    face_pts(M, f0, p);
    double sp[3];
    construct_pt(p[0], p[1], p[2], b0, sp);
    double r2 = r * r;
    std::unordered_set<int> visited, goal;
    visited.insert(f0);
    std::vector<int> order;
    order.push_back(f0);
    for (int i = 0; i < nT; ++i)
        if (tFace[i] != f0) goal.insert(tFace[i]);
    auto finish = [&]() {
        for (int g : goal)
            if (!visited.count(g)) { visited.insert(g); order.push_back(g); }
        out = order;
    };
    if (goal.empty()) { out = order; return; }
    std::vector<int> stack;
    for (int k = 0; k < 3; ++k) {
        int t = M.twin[3 * f0 + k];
        if (t < 0) continue;
        int nbf = t / 3;
        if (visited.insert(nbf).second) order.push_back(nbf);
        stack.push_back(nbf);
        goal.erase(nbf);
    }
    if (goal.empty()) { out = order; return; }
    while (!stack.empty()) {
        int cur = stack.back();
        stack.pop_back();
        for (int k = 0; k < 3; ++k) {
            int t = M.twin[3 * cur + k];
            if (t < 0) continue;
            int nbf = t / 3;
            if (visited.count(nbf)) continue;
            bool far = true;
            for (int c = 0; c < 3; ++c) {
                const double* q = vp(M, M.F[3 * nbf + c]);
                double d[3];
                sub3(sp, q, d);
                if (!(dot3(d, d) > r2)) far = false;
            }
            if (far) continue;
            visited.insert(nbf);
            order.push_back(nbf);
            goal.erase(nbf);
            stack.push_back(nbf);
        }
    }
    finish();
}

// ------------------------------------------------------------------------------------------------------------------
// Exact geodesics by window propagation
// ------------------------------------------------------------------------------------------------------------------
// A window lives on the edge through which it enters face g (local edge j: F[g][j] -> F[g][j+1]).  Frame: origin
// F[g][j], x along the edge, y into g.  The pseudo-source I = (sx, sy) lies behind the edge (sy < 0) at path
// length sigma from the source.  For sigma == 0 windows (c, s) rotate directions of this frame into the source
// face frame; for sigma > 0 they hold the (source-frame) start direction of the pseudo-source's own path.
struct Win {
    int g, j, src;
    double b0, b1, sx, sy, sigma, c, s;
};

struct Target {
    int face;
    double b[3];
    double p[3];
    double best;
    double ts2[2];  // start direction in the source frame
    double te[3];   // end direction (3D)
};

struct GeoStats {
    long long windowsCreated = 0;
    long long windowsProcessed = 0;
    long long vertexLaunches = 0;
    long long rounds = 0;
    long long frontier = 0;
};

struct GeoWork {
    std::vector<double> lab, vtx, vty;
    std::vector<char> launched;
    std::vector<int> touchedV;
    std::vector<int> faceHead;  // per face: first target index
    std::vector<int> tNext;
    std::vector<char> inD;
    std::vector<int> touchedF;
    void ensure(const Mesh& M)
    {
        if ((int)lab.size() != M.nV) {
            lab.assign(M.nV, kInf);
            vtx.assign(M.nV, 0);
            vty.assign(M.nV, 0);
            launched.assign(M.nV, 0);
        }
        if ((int)faceHead.size() != M.nF) {
            faceHead.assign(M.nF, -1);
            inD.assign(M.nF, 0);
        }
    }
    void reset()
    {
        for (int v : touchedV) {
            lab[v] = kInf;
            launched[v] = 0;
        }
        touchedV.clear();
        for (int f : touchedF) {
            faceHead[f] = -1;
            inD[f] = 0;
        }
        touchedF.clear();
    }
};

// processing order: 0 = exact priority queue (Dijkstra order); 1 = distance-banded rounds of width g_delta
// (the order the CUDA kernel uses; results are identical, only the work differs)
int g_order = 0;
double g_delta = 0.0;
double g_bfs = 0;  // 1: plain breadth-first rounds (no banding, launches immediately)

struct PQItem {
    double key;
    int kind;  // 0 window, 1 vertex
    int idx;
    bool operator<(const PQItem& o) const { return key > o.key; }
};

struct Geo {
    const Mesh& M;
    GeoWork& W;
    bool full;
    double cutoff;
    int f0;
    double S[3];
    double e1[3], e2[3];  // source frame axes in 3D
    std::vector<Win> wins;
    std::priority_queue<PQItem> pq;
    std::vector<Target>& T;
    GeoStats st;

    Geo(const Mesh& m, GeoWork& w, std::vector<Target>& t) : M(m), W(w), T(t) {}

    bool in_domain(int f) const { return f >= 0 && (full || W.inD[f]); }

    bool launchable(int v) const
    {
        if (M.borderV[v]) return true;
        if (M.angleSum[v] > 2.0 * kPi + 1e-9) return true;
        if (!full)
            for (int i = M.vfStart[v]; i < M.vfStart[v + 1]; ++i)
                if (!W.inD[M.vfList[i]]) return true;
        return false;
    }

    void touchV(int v)
    {
        if (W.lab[v] == kInf && !W.launched[v]) W.touchedV.push_back(v);
    }

    void propose(int v, double d, double dx, double dy)
    {
        if (!(d < W.lab[v])) return;
        touchV(v);
        W.lab[v] = d;
        W.vtx[v] = dx;
        W.vty[v] = dy;
        if (d <= cutoff && launchable(v)) pq.push({d, 1, v});
    }

    static double key_of(const Win& w)
    {
        double m;
        if (w.sx < w.b0) m = len2(w.sx - w.b0, w.sy);
        else if (w.sx > w.b1) m = len2(w.sx - w.b1, w.sy);
        else m = std::fabs(w.sy);
        return w.sigma + m;
    }

    // Remove the parts of the window that a path through an endpoint vertex of its edge beats (exact: the excess
    // of the window's path over the vertex path is monotone along the edge).
    bool trim(Win& w)
    {
        double L = M.EL[3 * w.g + w.j];
        int A = M.F[3 * w.g + w.j], B = M.F[3 * w.g + (w.j + 1) % 3];
        double dA = W.lab[A], dB = W.lab[B];
        if (dA < kInf) {
            double a = dA - w.sigma;
            double fb0 = len2(w.b0 - w.sx, w.sy) - a - w.b0;
            if (fb0 > 0) {
                if (a + w.sx <= 0) return false;
                double xs = (w.sx * w.sx + w.sy * w.sy - a * a) / (2.0 * (a + w.sx));
                if (xs >= w.b1) return false;
                w.b0 = std::max(w.b0, xs);
            }
        }
        if (dB < kInf) {
            double a = dB - w.sigma;
            double sxm = L - w.sx;
            double xm = L - w.b1;
            double fb1 = len2(xm - sxm, w.sy) - a - xm;
            if (fb1 > 0) {
                if (a + sxm <= 0) return false;
                double xs = (sxm * sxm + w.sy * w.sy - a * a) / (2.0 * (a + sxm));
                if (L - xs <= w.b0) return false;
                w.b1 = std::min(w.b1, L - xs);
            }
        }
        // third vertex: whole-window test
        int C = M.F[3 * w.g + (w.j + 2) % 3];
        double dC = W.lab[C];
        if (dC < kInf) {
            double cx = M.CX[3 * w.g + w.j], cy = M.CY[3 * w.g + w.j];
            double m0 = len2(cx - w.b0, cy), m1 = len2(cx - w.b1, cy);
            double key = key_of(w);
            if (dC + std::max(m0, m1) < key) return false;
        }
        return w.b1 - w.b0 > 1e-14 * L;
    }

    void push_win(Win w)
    {
        if (!in_domain(w.g) || w.g == f0) return;
        w.b0 = std::max(0.0, w.b0);
        w.b1 = std::min(M.EL[3 * w.g + w.j], w.b1);
        if (!trim(w)) return;
        double k = key_of(w);
        if (k > cutoff) return;
        wins.push_back(w);
        st.windowsCreated++;
        pq.push({k, 0, (int)wins.size() - 1});
    }

    void start_dir(const Win& w, double px, double py, double& dx, double& dy) const
    {
        if (w.sigma == 0) {
            double ux = px - w.sx, uy = py - w.sy;
            double l = len2(ux, uy);
            ux /= l;
            uy /= l;
            dx = w.c * ux - w.s * uy;
            dy = w.s * ux + w.c * uy;
        } else {
            dx = w.c;
            dy = w.s;
        }
    }

    void update_target(Target& t, double d, double dx, double dy, const double* te)
    {
        if (d < t.best) {
            t.best = d;
            t.ts2[0] = dx;
            t.ts2[1] = dy;
            t.te[0] = te[0];
            t.te[1] = te[1];
            t.te[2] = te[2];
        }
    }

    void process(const Win& w0)
    {
        Win w = w0;
        if (!trim(w)) return;
        st.windowsProcessed++;
        const int g = w.g, j = w.j;
        const double L = M.EL[3 * g + j], cx = M.CX[3 * g + j], cy = M.CY[3 * g + j];
        const int A = M.F[3 * g + j], B = M.F[3 * g + (j + 1) % 3], C = M.F[3 * g + (j + 2) % 3];
        const double tol = 1e-12 * L;
        // targets in g
        if (W.faceHead[g] >= 0) {
            const double* PA = vp(M, A);
            const double* PB = vp(M, B);
            const double* PC = vp(M, C);
            double ex[3], ey[3];
            sub3(PB, PA, ex);
            for (int c = 0; c < 3; ++c) ex[c] /= L;
            for (int c = 0; c < 3; ++c) ey[c] = (PC[c] - PA[c] - cx * ex[c]) / cy;
            for (int ti = W.faceHead[g]; ti >= 0; ti = W.tNext[ti]) {
                Target& t = T[ti];
                double px = t.b[(j + 1) % 3] * L + t.b[(j + 2) % 3] * cx;
                double py = t.b[(j + 2) % 3] * cy;
                double xp = w.sx + (px - w.sx) * (-w.sy) / (py - w.sy);
                if (xp >= w.b0 - tol && xp <= w.b1 + tol) {
                    double d = w.sigma + len2(px - w.sx, py - w.sy);
                    if (d < t.best) {
                        double dx, dy;
                        start_dir(w, px, py, dx, dy);
                        double ux = px - w.sx, uy = py - w.sy;
                        double ul = len2(ux, uy);
                        double te[3];
                        for (int c = 0; c < 3; ++c) te[c] = (ux * ex[c] + uy * ey[c]) / ul;
                        update_target(t, d, dx, dy, te);
                    }
                }
            }
        }
        // vertex labels
        double xC = w.sx + (cx - w.sx) * (-w.sy) / (cy - w.sy);
        if (xC >= w.b0 - tol && xC <= w.b1 + tol) {
            double dx, dy;
            start_dir(w, cx, cy, dx, dy);
            propose(C, w.sigma + len2(cx - w.sx, cy - w.sy), dx, dy);
        }
        if (w.b0 <= tol) {
            double dx, dy;
            start_dir(w, 0, 0, dx, dy);
            propose(A, w.sigma + len2(w.sx, w.sy), dx, dy);
        }
        if (w.b1 >= L - tol) {
            double dx, dy;
            start_dir(w, L, 0, dx, dy);
            propose(B, w.sigma + len2(L - w.sx, w.sy), dx, dy);
        }
        // children
        if (w.b0 < xC) {  // left: exit edge C->A (local j+2), new frame origin A, x toward C
            double n = len2(cx, cy);
            double ux = cx / n, uy = cy / n;
            double isx = ux * w.sx + uy * w.sy, isy = -uy * w.sx + ux * w.sy;
            auto proj = [&](double x) {
                double X = ux * x, Y = -uy * x;
                return isx + (X - isx) * (-isy) / (Y - isy);
            };
            int t = M.twin[3 * g + (j + 2) % 3];
            if (t >= 0) {
                Win c;
                c.g = t / 3;
                c.j = t % 3;
                c.src = w.src;
                c.sigma = w.sigma;
                c.sx = isx;
                c.sy = isy;
                c.b0 = proj(w.b0);
                c.b1 = (w.b1 >= xC) ? M.EL[t] : proj(w.b1);
                if (w.sigma == 0) {
                    c.c = w.c * ux - w.s * uy;
                    c.s = w.s * ux + w.c * uy;
                } else {
                    c.c = w.c;
                    c.s = w.s;
                }
                push_win(c);
            }
        }
        if (w.b1 > xC) {  // right: exit edge B->C (local j+1), new frame origin C, x toward B
            double bx = L - cx, by = -cy;
            double n = len2(bx, by);
            double ux = bx / n, uy = by / n;
            double rx = w.sx - cx, ry = w.sy - cy;
            double isx = ux * rx + uy * ry, isy = -uy * rx + ux * ry;
            auto proj = [&](double x) {
                double X = ux * (x - cx) + uy * (-cy), Y = -uy * (x - cx) + ux * (-cy);
                return isx + (X - isx) * (-isy) / (Y - isy);
            };
            int t = M.twin[3 * g + (j + 1) % 3];
            if (t >= 0) {
                Win c;
                c.g = t / 3;
                c.j = t % 3;
                c.src = w.src;
                c.sigma = w.sigma;
                c.sx = isx;
                c.sy = isy;
                c.b0 = (w.b0 <= xC) ? 0.0 : proj(w.b0);
                c.b1 = proj(w.b1);
                if (w.sigma == 0) {
                    c.c = w.c * ux - w.s * uy;
                    c.s = w.s * ux + w.c * uy;
                } else {
                    c.c = w.c;
                    c.s = w.s;
                }
                push_win(c);
            }
        }
    }

    void launch(int v)
    {
        st.vertexLaunches++;
        double d = W.lab[v];
        W.launched[v] = 1;
        for (int i = M.vfStart[v]; i < M.vfStart[v + 1]; ++i) {
            int f = M.vfList[i];
            if (!in_domain(f)) continue;
            int k = 0;
            while (M.F[3 * f + k] != v) ++k;
            int e = (k + 1) % 3;  // opposite edge F[k+1] -> F[k+2]
            // edge paths from v to the other two vertices of f
            propose(M.F[3 * f + e], d + M.EL[3 * f + k], W.vtx[v], W.vty[v]);
            propose(M.F[3 * f + (k + 2) % 3], d + M.EL[3 * f + (k + 2) % 3], W.vtx[v], W.vty[v]);
            int t = M.twin[3 * f + e];
            if (t < 0) continue;
            Win c;
            c.g = t / 3;
            c.j = t % 3;
            c.src = v;
            c.sigma = d;
            double L = M.EL[3 * f + e];
            c.sx = L - M.CX[3 * f + e];
            c.sy = -M.CY[3 * f + e];
            c.b0 = 0;
            c.b1 = L;
            c.c = W.vtx[v];
            c.s = W.vty[v];
            push_win(c);
        }
    }

    void run(int face0, const double* b, bool earlyExit)
    {
        f0 = face0;
        const double* p[3];
        face_pts(M, f0, p);
        construct_pt(p[0], p[1], p[2], b, S);
        // source frame = edge-0 frame of f0
        double L0 = M.EL[3 * f0], cx0 = M.CX[3 * f0], cy0 = M.CY[3 * f0];
        sub3(p[1], p[0], e1);
        for (int c = 0; c < 3; ++c) e1[c] /= L0;
        for (int c = 0; c < 3; ++c) e2[c] = (p[2][c] - p[0][c] - cx0 * e1[c]) / cy0;
        double P2[3][2] = {{0, 0}, {L0, 0}, {cx0, cy0}};
        double S2[2] = {b[1] * L0 + b[2] * cx0, b[2] * cy0};
        for (int k = 0; k < 3; ++k) {
            int v = M.F[3 * f0 + k];
            double dx = P2[k][0] - S2[0], dy = P2[k][1] - S2[1];
            double l = len2(dx, dy);
            double d3[3];
            sub3(vp(M, v), S, d3);
            propose(v, norm3(d3), dx / l, dy / l);
        }
        for (int k = 0; k < 3; ++k) {
            int t = M.twin[3 * f0 + k];
            if (t < 0) continue;
            double L = M.EL[3 * f0 + k];
            double skx = b[(k + 1) % 3] * L + b[(k + 2) % 3] * M.CX[3 * f0 + k];
            double sky = b[(k + 2) % 3] * M.CY[3 * f0 + k];
            Win w;
            w.g = t / 3;
            w.j = t % 3;
            w.src = -1;
            w.sigma = 0;
            w.sx = L - skx;
            w.sy = std::min(-sky, -1e-15 * L);
            w.b0 = 0;
            w.b1 = L;
            double ddx = P2[(k + 1) % 3][0] - P2[k][0], ddy = P2[(k + 1) % 3][1] - P2[k][1];
            double dl = len2(ddx, ddy);
            w.c = -ddx / dl;
            w.s = -ddy / dl;
            push_win(w);
        }
        if (g_order == 1) {
            run_rounds(earlyExit);
            return;
        }
        long long pops = 0;
        while (!pq.empty()) {
            PQItem it = pq.top();
            pq.pop();
            if (it.key > cutoff) break;
            if (it.kind == 1) {
                if (W.lab[it.idx] != it.key || W.launched[it.idx] == 2) continue;
                launch(it.idx);
            } else {
                process(wins[it.idx]);
            }
            if (earlyExit && ((++pops) & 63) == 0 && !pq.empty()) {
                double top = pq.top().key;
                bool done = true;
                for (auto& t : T) {
                    double b2 = final_candidate(t);
                    if (!(b2 <= top)) { done = false; break; }
                }
                if (done) break;
            }
        }
    }

    // distance-banded rounds over the same window / launch events (drains the priority queue into lists)
    void run_rounds(bool earlyExit)
    {
        std::vector<int> front, pend;
        std::vector<char> launchedWith;  // unused: launched label tracked in lastLaunch
        std::unordered_map<int, double> lastLaunch;
        auto drain = [&](std::vector<int>& fr, std::vector<int>& pe) {
            while (!pq.empty()) {
                PQItem it = pq.top();
                pq.pop();
                if (it.kind == 0) fr.push_back(it.idx);
                else pe.push_back(it.idx);
            }
        };
        drain(front, pend);
        long long rounds = 0;
        while (!front.empty() || !pend.empty()) {
            if (++rounds > 100000) break;
            double mk = kInf;
            for (int w : front) mk = std::min(mk, key_of(wins[w]));
            for (int v : pend) mk = std::min(mk, W.lab[v]);
            if (mk > cutoff) break;
            if (earlyExit) {
                bool done = true;
                for (auto& t : T)
                    if (!(final_candidate(t) <= mk)) { done = false; break; }
                if (done) break;
            }
            double thr = g_bfs ? kInf : mk + g_delta;
            for (int w : front) frontierSum += key_of(wins[w]) <= thr ? 1 : 0;
            std::vector<int> nf, np;
            for (int v : pend) {
                double d = W.lab[v];
                if (d > thr) { np.push_back(v); continue; }
                auto itl = lastLaunch.find(v);
                if (itl != lastLaunch.end() && itl->second == d) continue;
                lastLaunch[v] = d;
                launch(v);
            }
            drain(nf, np);
            for (int w : front) {
                if (key_of(wins[w]) > thr) { nf.push_back(w); continue; }
                process(wins[w]);
                drain(nf, np);
            }
            front.swap(nf);
            pend.swap(np);
        }
        roundsUsed = rounds;
    }

    long long roundsUsed = 0;
    long long frontierSum = 0;

    double final_candidate(const Target& t) const
    {
        if (t.face == f0) return 0;
        double b = t.best;
        for (int c = 0; c < 3; ++c) {
            int v = M.F[3 * t.face + c];
            if (W.lab[v] < kInf) {
                double d3[3];
                sub3(t.p, vp(M, v), d3);
                b = std::min(b, W.lab[v] + norm3(d3));
            }
        }
        return b;
    }

    void finish(double* dOut, double* tsOut, double* teOut)
    {
        for (size_t i = 0; i < T.size(); ++i) {
            Target& t = T[i];
            double d, ts[3] = {0, 0, 0}, te[3] = {0, 0, 0};
            if (t.face == f0) {
                double u[3];
                sub3(t.p, S, u);
                d = norm3(u);
                if (d > 0)
                    for (int c = 0; c < 3; ++c) ts[c] = te[c] = u[c] / d;
            } else {
                double dx = t.ts2[0], dy = t.ts2[1];
                d = t.best;
                for (int c = 0; c < 3; ++c) te[c] = t.te[c];
                for (int c = 0; c < 3; ++c) {
                    int v = M.F[3 * t.face + c];
                    if (W.lab[v] < kInf) {
                        double u[3];
                        sub3(t.p, vp(M, v), u);
                        double l = norm3(u);
                        double dv = W.lab[v] + l;
                        if (dv < d) {
                            d = dv;
                            dx = W.vtx[v];
                            dy = W.vty[v];
                            for (int q = 0; q < 3; ++q) te[q] = l > 0 ? u[q] / l : 0;
                        }
                    }
                }
                if (d < kInf)
                    for (int c = 0; c < 3; ++c) ts[c] = dx * e1[c] + dy * e2[c];
            }
            if (d > cutoff) d = kInf;
            dOut[i] = d;
            if (tsOut)
                for (int c = 0; c < 3; ++c) tsOut[3 * i + c] = d < kInf ? ts[c] : 0;
            if (teOut)
                for (int c = 0; c < 3; ++c) teOut[3 * i + c] = d < kInf ? te[c] : 0;
        }
    }
};

// One source against nT targets.  faceSet (nSet entries) restricts the domain (patch mode); nullptr = whole mesh.
void geodesic_one(const Mesh& M, GeoWork& W, int f0, const double* b0, int nT, const int* tFace, const double* tBary,
                  const int* faceSet, int nSet, double cutoff, bool earlyExit, double* dOut, double* tsOut,
                  double* teOut, GeoStats* stats)
{
    W.ensure(M);
    std::vector<Target> T(nT);
    W.tNext.assign(nT, -1);
    for (int i = 0; i < nT; ++i) {
        Target& t = T[i];
        t.face = tFace[i];
        for (int c = 0; c < 3; ++c) t.b[c] = tBary[3 * i + c];
        const double* p[3];
        face_pts(M, t.face, p);
        construct_pt(p[0], p[1], p[2], t.b, t.p);
        t.best = kInf;
        t.ts2[0] = t.ts2[1] = 0;
        t.te[0] = t.te[1] = t.te[2] = 0;
        if (W.faceHead[t.face] < 0 && !W.inD[t.face]) W.touchedF.push_back(t.face);
        W.tNext[i] = W.faceHead[t.face];
        W.faceHead[t.face] = i;
    }
    Geo G(M, W, T);
    G.full = (faceSet == nullptr);
    G.cutoff = cutoff;
    if (!G.full)
        for (int i = 0; i < nSet; ++i) {
            int f = faceSet[i];
            if (W.faceHead[f] < 0 && !W.inD[f]) W.touchedF.push_back(f);
            W.inD[f] = 1;
        }
    G.run(f0, b0, earlyExit);
    G.finish(dOut, tsOut, teOut);
    if (stats) {
        stats->windowsCreated += G.st.windowsCreated;
        stats->windowsProcessed += G.st.windowsProcessed;
        stats->vertexLaunches += G.st.vertexLaunches;
        stats->rounds += G.roundsUsed;
        stats->frontier += G.frontierSum;
    }
    W.reset();
}

// ------------------------------------------------------------------------------------------------------------------
// Brute force: shortest path as a chain of straight unfolded segments between {source, saddle/border vertices,
// target}; each straight segment found by enumerating simple face sequences (depth-limited, pruned by length).
// ------------------------------------------------------------------------------------------------------------------
struct BF {
    const Mesh& M;
    const std::vector<char>& inD;
    int maxDepth;
    BF(const Mesh& m, const std::vector<char>& d, int depth) : M(m), inD(d), maxDepth(depth) {}

    // layout of face f in 2D given the 2D positions of two of its vertices (va at a, vb at b) and the side sign
    static void place_third(const double* a, const double* b, double la, double lb, double side, double* out)
    {
        // third point at distance la from a and lb from b, on the given side of a->b (side=+1 left)
        double dx = b[0] - a[0], dy = b[1] - a[1];
        double L = len2(dx, dy);
        double x = (la * la - lb * lb + L * L) / (2 * L);
        double y = std::sqrt(std::max(0.0, la * la - x * x));
        double ux = dx / L, uy = dy / L;
        out[0] = a[0] + x * ux - side * y * uy;
        out[1] = a[1] + x * uy + side * y * ux;
    }

    double len(int u, int v) const
    {
        double d[3];
        sub3(vp(M, u), vp(M, v), d);
        return norm3(d);
    }

    // DFS over face sequences.  cur: face, P[3][2]: its 2D layout (vertex order as M.F), X: start point (2D),
    // crossings so far validated.  dest: target face + 2D point computed from barycentrics on arrival.
    void dfs(int f, double P[3][2], const double* X, int depth, std::vector<char>& onPath, int destFace,
             const double* destBary, int destVertex, double& best, int enterEdge)
    {
        bool atDest = (destVertex < 0) ? (f == destFace) : false;
        if (destVertex >= 0)
            for (int k = 0; k < 3; ++k)
                if (M.F[3 * f + k] == destVertex) atDest = true;
        if (atDest) {
            double Y[2];
            if (destVertex < 0) {
                Y[0] = destBary[0] * P[0][0] + destBary[1] * P[1][0] + destBary[2] * P[2][0];
                Y[1] = destBary[0] * P[0][1] + destBary[1] * P[1][1] + destBary[2] * P[2][1];
            } else {
                int k = 0;
                while (M.F[3 * f + k] != destVertex) ++k;
                Y[0] = P[k][0];
                Y[1] = P[k][1];
            }
            double d = len2(Y[0] - X[0], Y[1] - X[1]);
            if (d < best && valid_segment(X, Y)) best = d;
        }
        if (depth >= maxDepth) return;
        for (int k = 0; k < 3; ++k) {
            if (k == enterEdge) continue;
            int t = M.twin[3 * f + k];
            if (t < 0) continue;
            int g = t / 3;
            if (!inD[g] || onPath[g]) continue;
            // the segment must be able to leave through edge k: distance from X to edge k segment < best
            double* a = P[k];
            double* bpt = P[(k + 1) % 3];
            double ex = bpt[0] - a[0], ey = bpt[1] - a[1];
            double tt = ((X[0] - a[0]) * ex + (X[1] - a[1]) * ey) / (ex * ex + ey * ey);
            tt = std::max(0.0, std::min(1.0, tt));
            double md = len2(a[0] + tt * ex - X[0], a[1] + tt * ey - X[1]);
            if (md >= best) continue;
            int j = t % 3;  // g: F[g][j] = F[f][k+1], F[g][j+1] = F[f][k]
            double Q[3][2];
            Q[j][0] = bpt[0];
            Q[j][1] = bpt[1];
            Q[(j + 1) % 3][0] = a[0];
            Q[(j + 1) % 3][1] = a[1];
            int vc = M.F[3 * g + (j + 2) % 3];
            double la = len(M.F[3 * g + j], vc), lb = len(M.F[3 * g + (j + 1) % 3], vc);
            // third vertex of g goes on the opposite side of edge from f's third vertex
            double* fc = P[(k + 2) % 3];
            double side0 = ((bpt[0] - a[0]) * (fc[1] - a[1]) - (bpt[1] - a[1]) * (fc[0] - a[0])) > 0 ? 1.0 : -1.0;
            // edge a->b in f; in g the same points are Q[j]=b, Q[j+1]=a; place relative to b->a: f's third vertex is
            // on side side0 of a->b, i.e. on side -side0 of b->a; g's vertex goes on side +side0 of b->a
            place_third(Q[j], Q[(j + 1) % 3], la, lb, side0, Q[(j + 2) % 3]);
            path.push_back({a[0], a[1], bpt[0], bpt[1]});
            onPath[g] = 1;
            dfs(g, Q, X, depth + 1, onPath, destFace, destBary, destVertex, best, j);
            onPath[g] = 0;
            path.pop_back();
        }
    }

    struct Seg { double ax, ay, bx, by; };
    std::vector<Seg> path;

    bool valid_segment(const double* X, const double* Y) const
    {
        const double tol = 1e-9;
        double tprev = -tol;
        for (const Seg& s : path) {
            double dx = Y[0] - X[0], dy = Y[1] - X[1];
            double ex = s.bx - s.ax, ey = s.by - s.ay;
            double den = dx * ey - dy * ex;
            if (std::fabs(den) < 1e-300) return false;
            double t = ((s.ax - X[0]) * ey - (s.ay - X[1]) * ex) / den;
            double u = ((s.ax - X[0]) * dy - (s.ay - X[1]) * dx) / den;
            if (t < -tol || t > 1 + tol || u < -tol || u > 1 + tol) return false;
            if (t < tprev - tol) return false;  // edges must be crossed in sequence order
            tprev = t;
        }
        return true;
    }

    void layout(int f, double P[3][2]) const
    {
        P[0][0] = 0;
        P[0][1] = 0;
        P[1][0] = M.EL[3 * f];
        P[1][1] = 0;
        P[2][0] = M.CX[3 * f];
        P[2][1] = M.CY[3 * f];
    }

    // straight (vertex-free) distance from a point (face fa, bary ba) or a vertex va to a point or a vertex
    double direct(int fa, const double* ba, int va, int fb, const double* bb, int vb)
    {
        double best = kInf;
        std::vector<char> onPath(M.nF, 0);
        std::vector<int> starts;
        if (va < 0) starts.push_back(fa);
        else
            for (int i = M.vfStart[va]; i < M.vfStart[va + 1]; ++i)
                if (inD[M.vfList[i]]) starts.push_back(M.vfList[i]);
        for (int f : starts) {
            double P[3][2];
            layout(f, P);
            double X[2];
            if (va < 0) {
                X[0] = ba[0] * P[0][0] + ba[1] * P[1][0] + ba[2] * P[2][0];
                X[1] = ba[0] * P[0][1] + ba[1] * P[1][1] + ba[2] * P[2][1];
            } else {
                int k = 0;
                while (M.F[3 * f + k] != va) ++k;
                X[0] = P[k][0];
                X[1] = P[k][1];
            }
            onPath[f] = 1;
            path.clear();
            dfs(f, P, X, 0, onPath, fb, bb, vb, best, -1);
            onPath[f] = 0;
        }
        return best;
    }
};

}  // namespace

// ======================================================================================================================
// C API (ctypes)
// ======================================================================================================================
extern "C" {

void oracle_set_order(int order, double delta, int bfs)
{
    g_order = order;
    g_delta = delta;
    g_bfs = bfs;
}

void* oracle_mesh_create(const double* V, int nV, const int* F, int nF)
{
    Mesh* M = new Mesh();
    build_mesh(*M, V, nV, F, nF);
    return M;
}

void oracle_mesh_destroy(void* m) { delete (Mesh*)m; }

double oracle_mesh_area(void* m) { return ((Mesh*)m)->area; }

void oracle_mesh_bbox(void* m, double* out)
{
    Mesh* M = (Mesh*)m;
    for (int c = 0; c < 3; ++c) {
        out[c] = M->bbMin[c];
        out[3 + c] = M->bbMax[c];
    }
}

void oracle_angle_sums(void* m, double* out)
{
    Mesh* M = (Mesh*)m;
    for (int v = 0; v < M->nV; ++v) out[v] = M->angleSum[v];
}

void oracle_positions_r3(void* m, int n, const int* face, const double* bary, double* out)
{
    Mesh* M = (Mesh*)m;
    for (int i = 0; i < n; ++i) {
        const double* p[3];
        face_pts(*M, face[i], p);
        construct_pt(p[0], p[1], p[2], &bary[3 * i], &out[3 * i]);
    }
}

// batched transportParticleAndVectors; transport: n x ntv x 3; crossings may be null
void oracle_transport(void* m, int n, int* face, double* bary, double* disp, double* transport, int ntv, int maxIter,
                      int* status, int* crossings)
{
    Mesh* M = (Mesh*)m;
    for (int i = 0; i < n; ++i) {
        int cr = 0;
        int st = transport_one(*M, face[i], &bary[3 * i], &disp[3 * i], transport ? &transport[3 * ntv * i] : nullptr,
                               ntv, maxIter, &cr, g_bc);
        if (status) status[i] = st;
        if (crossings) crossings[i] = cr;
    }
}

// submesher face set for one source; returns the face count (faces written to out, capacity cap)
int oracle_patch(void* m, int f0, const double* b0, int nT, const int* tFace, double r, int* out, int cap)
{
    Mesh* M = (Mesh*)m;
    std::vector<int> faces;
    build_patch(*M, f0, b0, tFace, nT, r, faces);
    int n = (int)faces.size();
    for (int i = 0; i < n && i < cap; ++i) out[i] = faces[i];
    return n;
}

// triangulatedMeshSpace::distance / distanceWithSubmeshing for one source.
//   submesh: 0 = whole mesh, 1 = reference patch with radius min(maxDist, threshold)
//   cutoff : prune paths longer than this (inf for the exact reference semantics)
// Unreached targets: patch mode -> 2*maxDist and tangent (0,0,1) (triangulatedMeshSpace.cpp:197-203);
// beyond the cutoff -> +inf and zero tangents.
void oracle_distance(void* m, int f0, const double* b0, int nT, const int* tFace, const double* tBary, int submesh,
                     double maxDist, double threshold, double cutoff, double* dOut, double* tsOut, double* teOut,
                     long long* statsOut)
{
    Mesh* M = (Mesh*)m;
    GeoWork W;
    GeoStats st;
    std::vector<int> faces;
    const int* fs = nullptr;
    int nfs = 0;
    if (submesh) {
        double r = maxDist;
        if (threshold < maxDist) r = threshold;
        build_patch(*M, f0, b0, tFace, nT, r, faces);
        fs = faces.data();
        nfs = (int)faces.size();
    }
    geodesic_one(*M, W, f0, b0, nT, tFace, tBary, fs, nfs, cutoff, false, dOut, tsOut, teOut, &st);
    if (submesh && !(cutoff < kInf))
        for (int i = 0; i < nT; ++i)
            if (!(dOut[i] < kInf)) {
                dOut[i] = 2.0 * maxDist;
                if (tsOut) { tsOut[3 * i] = 0; tsOut[3 * i + 1] = 0; tsOut[3 * i + 2] = 1; }
                if (teOut) { teOut[3 * i] = 0; teOut[3 * i + 1] = 0; teOut[3 * i + 2] = 1; }
            }
    if (statsOut) {
        statsOut[0] = st.windowsCreated;
        statsOut[1] = st.windowsProcessed;
        statsOut[2] = st.vertexLaunches;
        statsOut[3] = nfs;
    }
}

// brute-force exact distance between two surface points on a face set (nullptr faceSet = whole mesh)
double oracle_distance_bruteforce(void* m, int fa, const double* ba, int fb, const double* bb, const int* faceSet,
                                  int nSet, int maxDepth)
{
    Mesh* M = (Mesh*)m;
    std::vector<char> inD(M->nF, faceSet ? 0 : 1);
    if (faceSet)
        for (int i = 0; i < nSet; ++i) inD[faceSet[i]] = 1;
    if (fa == fb) {
        double pa[3], pb[3];
        const double* p[3];
        face_pts(*M, fa, p);
        construct_pt(p[0], p[1], p[2], ba, pa);
        construct_pt(p[0], p[1], p[2], bb, pb);
        double d[3];
        sub3(pa, pb, d);
        return norm3(d);
    }
    BF bf(*M, inD, maxDepth);
    // pseudo-source vertices: saddles and border vertices of the face set
    std::vector<int> ps;
    for (int v = 0; v < M->nV; ++v) {
        bool touches = false, border = M->borderV[v];
        for (int i = M->vfStart[v]; i < M->vfStart[v + 1]; ++i) {
            if (inD[M->vfList[i]]) touches = true;
            else border = true;
        }
        if (!touches) continue;
        if (border || M->angleSum[v] > 2.0 * kPi + 1e-9) ps.push_back(v);
    }
    int n = (int)ps.size();
    // Dijkstra over {source, ps..., target}
    std::vector<double> dist(n + 1, kInf);
    std::vector<char> done(n + 1, 0);
    for (int i = 0; i < n; ++i) dist[i] = bf.direct(fa, ba, -1, -1, nullptr, ps[i]);
    dist[n] = bf.direct(fa, ba, -1, fb, bb, -1);
    while (true) {
        int u = -1;
        for (int i = 0; i <= n; ++i)
            if (!done[i] && dist[i] < kInf && (u < 0 || dist[i] < dist[u])) u = i;
        if (u < 0 || u == n) break;
        done[u] = 1;
        for (int i = 0; i < n; ++i)
            if (!done[i]) {
                double d = bf.direct(-1, nullptr, ps[u], -1, nullptr, ps[i]);
                if (dist[u] + d < dist[i]) dist[i] = dist[u] + d;
            }
        double d = bf.direct(-1, nullptr, ps[u], fb, bb, -1);
        if (dist[u] + d < dist[n]) dist[n] = dist[u] + d;
    }
    return dist[n];
}

// candidate neighbours (hyperRectangularCellList + cellListNeighborStructure): returns CSR (offsets n+1, indices)
// into caller buffers; idx capacity cap; returns total candidates (or -needed if cap too small).  maxChord[i] is
// the value constructCandidateNeighborList returns.  range <= 0 selects the all-to-all structure.
long long oracle_candidates(void* m, int n, const int* face, const double* bary, double range, int* offsets, int* idx,
                            long long cap, double* maxChord)
{
    Mesh* M = (Mesh*)m;
    std::vector<double> P(3 * n);
    for (int i = 0; i < n; ++i) {
        const double* p[3];
        face_pts(*M, face[i], p);
        construct_pt(p[0], p[1], p[2], &bary[3 * i], &P[3 * i]);
    }
    long long total = 0;
    offsets[0] = 0;
    if (range <= 0) {
        for (int i = 0; i < n; ++i) {
            for (int j = 0; j < n; ++j)
                if (j != i) {
                    if (total < cap) idx[total] = j;
                    total++;
                }
            offsets[i + 1] = (int)total;
            maxChord[i] = 1e20;
        }
        return total <= cap ? total : -total;
    }
    int nc[3];
    double cs[3];
    for (int c = 0; c < 3; ++c) {
        double ext = M->bbMax[c] - M->bbMin[c];
        nc[c] = std::max(1, (int)std::floor(ext / range));
        cs[c] = ext / nc[c];
    }
    auto cellOf = [&](const double* p, int* ci) {
        for (int c = 0; c < 3; ++c)
            ci[c] = std::max(0, std::min(nc[c] - 1, (int)std::floor((p[c] - M->bbMin[c]) / cs[c])));
    };
    // Index3D(x,y,z) = x + nx*(y + ny*z) (indexer.h); particles appended in index order
    int totalCells = nc[0] * nc[1] * nc[2];
    std::vector<std::vector<int>> cells(totalCells);
    for (int i = 0; i < n; ++i) {
        int ci[3];
        cellOf(&P[3 * i], ci);
        cells[ci[0] + nc[0] * (ci[1] + nc[1] * ci[2])].push_back(i);
    }
    double r2 = range * range;
    for (int i = 0; i < n; ++i) {
        int ci[3];
        cellOf(&P[3 * i], ci);
        double mx = 0;
        for (int xx = std::max(0, ci[0] - 1); xx <= std::min(nc[0] - 1, ci[0] + 1); ++xx)
            for (int yy = std::max(0, ci[1] - 1); yy <= std::min(nc[1] - 1, ci[1] + 1); ++yy)
                for (int zz = std::max(0, ci[2] - 1); zz <= std::min(nc[2] - 1, ci[2] + 1); ++zz)
                    for (int j : cells[xx + nc[0] * (yy + nc[1] * zz)]) {
                        if (j == i) continue;
                        double d[3];
                        sub3(&P[3 * i], &P[3 * j], d);
                        double d2 = dot3(d, d);
                        if (d2 < r2) {
                            if (total < cap) idx[total] = j;
                            total++;
                            if (d2 > mx) mx = d2;
                        }
                    }
        offsets[i + 1] = (int)total;
        maxChord[i] = std::sqrt(mx);
    }
    return total <= cap ? total : -total;
}

}  // extern "C"

// ======================================================================================================================
// Model: neighbours + forces + integrators over a whole system (used for multi-step parity and the CPU baseline)
// ======================================================================================================================
namespace {

struct SysParams {
    int forceKind;     // 0 harmonic, 1 gaussian
    double k, sigma;   // harmonic stiffness and range; gaussian: k = alpha, sigma = sigma
    double range;      // candidate range (force maximumInteractionRange); <= 0: all-to-all
    int submesh;       // 1 = reference patches
    double maxDist;    // useSubmeshingRoutines radius
    double cutoff;     // geodesic pruning radius (>= the largest distance any force reads)
};

double pair_force_mag(const SysParams& P, double d)
{
    if (P.forceKind == 0) return (d <= P.sigma) ? -P.k * (P.sigma - d) : 0.0;
    const double sqrtTwoPi = 2.50662827463100050241576528481104525300698674061;
    double s2 = 2.0 * P.sigma * P.sigma;
    double pref = d * P.k * std::exp(-d * d / s2) / ((sqrtTwoPi * P.sigma) * std::sqrt(P.sigma));
    return -pref;
}

double pair_energy(const SysParams& P, double d)
{
    if (P.forceKind == 0) return (d < P.sigma) ? 0.5 * P.k * (P.sigma - d) * (P.sigma - d) : 0.0;
    const double sqrtTwoPi = 2.50662827463100050241576528481104525300698674061;
    return P.k * std::exp(-d * d / (2.0 * P.sigma * P.sigma)) / (sqrtTwoPi * P.sigma);
}

// simpleModel::findNeighbors + force::computeForces; returns energy via *energy if requested
void compute_forces(const Mesh& M, const SysParams& P, int n, const int* face, const double* bary, double* force,
                    double* energy, int nThreads, long long* pairsInRange, GeoStats* stats)
{
    std::vector<int> off(n + 1);
    long long cap = (long long)n * 64 + 1024;
    std::vector<int> idx;
    std::vector<double> mc(n);
    long long tot;
    while (true) {
        idx.resize(cap);
        tot = oracle_candidates((void*)&M, n, face, bary, P.range, off.data(), idx.data(), cap, mc.data());
        if (tot >= 0) break;
        cap = -tot;
    }
    double e = 0;
    long long inr = 0;
#ifdef _OPENMP
    if (nThreads > 0) omp_set_num_threads(nThreads);
#endif
    std::vector<GeoStats> sts;
#pragma omp parallel reduction(+ : e, inr)
    {
        GeoWork W;
        GeoStats st;
        std::vector<int> tf;
        std::vector<double> tb, d, ts;
        std::vector<int> faces;
#pragma omp for schedule(dynamic, 4)
        for (int i = 0; i < n; ++i) {
            int a = off[i], b = off[i + 1], nt = b - a;
            force[3 * i] = force[3 * i + 1] = force[3 * i + 2] = 0;
            if (nt == 0) continue;
            tf.resize(nt);
            tb.resize(3 * nt);
            d.resize(nt);
            ts.resize(3 * nt);
            for (int q = 0; q < nt; ++q) {
                int jj = idx[a + q];
                tf[q] = face[jj];
                for (int c = 0; c < 3; ++c) tb[3 * q + c] = bary[3 * jj + c];
            }
            const int* fs = nullptr;
            int nfs = 0;
            if (P.submesh) {
                double r = P.maxDist;
                if (mc[i] < P.maxDist) r = mc[i];
                build_patch(M, face[i], &bary[3 * i], tf.data(), nt, r, faces);
                fs = faces.data();
                nfs = (int)faces.size();
            }
            geodesic_one(M, W, face[i], &bary[3 * i], nt, tf.data(), tb.data(), fs, nfs, P.cutoff, true, d.data(),
                         ts.data(), nullptr, &st);
            for (int q = 0; q < nt; ++q) {
                if (!(d[q] < kInf)) continue;
                double fm = pair_force_mag(P, d[q]);
                if (P.forceKind != 0 || d[q] <= P.sigma) {
                    for (int c = 0; c < 3; ++c) force[3 * i + c] += fm * ts[3 * q + c];
                }
                if (energy) e += pair_energy(P, d[q]);
                if (d[q] <= P.sigma) inr++;
            }
        }
#pragma omp critical
        sts.push_back(st);
    }
    if (energy) *energy = e;
    if (pairsInRange) *pairsInRange = inr;
    if (stats)
        for (auto& s : sts) {
            stats->windowsCreated += s.windowsCreated;
            stats->windowsProcessed += s.windowsProcessed;
            stats->vertexLaunches += s.vertexLaunches;
        }
}

int move_all(const Mesh& M, int n, int* face, double* bary, double* disp, double* vel, int nThreads)
{
    int err = 0;
#pragma omp parallel for schedule(static) reduction(| : err)
    for (int i = 0; i < n; ++i) {
        int st = transport_one(M, face[i], &bary[3 * i], &disp[3 * i], vel ? &vel[3 * i] : nullptr, vel ? 1 : 0,
                               100000, nullptr, g_bc);
        if (st) err |= (1 << st);
    }
    (void)nThreads;
    return err;
}

}  // namespace

extern "C" {

// Per-source distances for an explicit candidate CSR (the model's neighbour pass), used by parity tests.
// dOut/tsOut sized to the candidate count.
void oracle_neighbor_distances(void* m, int n, const int* face, const double* bary, const int* off, const int* idx,
                               const double* maxChord, int submesh, double maxDist, double cutoff, double* dOut,
                               double* tsOut, long long* statsOut, int nThreads)
{
    Mesh* M = (Mesh*)m;
#ifdef _OPENMP
    if (nThreads > 0) omp_set_num_threads(nThreads);
#endif
    long long w0 = 0, w1 = 0, w2 = 0, w3 = 0, w4 = 0;
#pragma omp parallel reduction(+ : w0, w1, w2, w3, w4)
    {
        GeoWork W;
        GeoStats st;
        std::vector<int> tf, faces;
        std::vector<double> tb;
#pragma omp for schedule(dynamic, 4)
        for (int i = 0; i < n; ++i) {
            int a = off[i], nt = off[i + 1] - a;
            if (nt == 0) continue;
            tf.resize(nt);
            tb.resize(3 * nt);
            for (int q = 0; q < nt; ++q) {
                tf[q] = face[idx[a + q]];
                for (int c = 0; c < 3; ++c) tb[3 * q + c] = bary[3 * idx[a + q] + c];
            }
            const int* fs = nullptr;
            int nfs = 0;
            if (submesh) {
                double r = maxDist;
                if (maxChord[i] < maxDist) r = maxChord[i];
                build_patch(*M, face[i], &bary[3 * i], tf.data(), nt, r, faces);
                fs = faces.data();
                nfs = (int)faces.size();
            }
            geodesic_one(*M, W, face[i], &bary[3 * i], nt, tf.data(), tb.data(), fs, nfs, cutoff, true, &dOut[a],
                         &tsOut[3 * a], nullptr, &st);
        }
        w0 += st.windowsCreated;
        w1 += st.windowsProcessed;
        w2 += st.vertexLaunches;
        w3 += st.rounds;
        w4 += st.frontier;
    }
    if (statsOut) {
        statsOut[0] = w0;
        statsOut[1] = w1;
        statsOut[2] = w2;
        statsOut[3] = w3;
        statsOut[4] = w4;
    }
}

// force::computeForces over the system; returns the pair energy (computeEnergy) in energy[0] if non-null
void oracle_forces(void* m, int n, const int* face, const double* bary, const double* params, double* force,
                   double* energy, int nThreads, long long* statsOut)
{
    Mesh* M = (Mesh*)m;
    SysParams P{(int)params[0], params[1], params[2], params[3], (int)params[4], params[5], params[6]};
    GeoStats st;
    long long inr = 0;
    compute_forces(*M, P, n, face, bary, force, energy, nThreads, &inr, &st);
    if (statsOut) {
        statsOut[0] = st.windowsCreated;
        statsOut[1] = st.windowsProcessed;
        statsOut[2] = st.vertexLaunches;
        statsOut[3] = inr;
    }
}

// Run `steps` timesteps of NVE (kind 0) or Nose-Hoover NVT (kind 1) in place.
//   params: forceKind, k, sigma, range, submesh, maxDist, cutoff, dt, T, tau, chainLength
//   chain : (chainLength+1) x 4 bath variables (pos, vel, accel, mass) + [kineticEnergy, scale] - in/out (NVT)
// NVE follows velocityVerletNVE::performUpdate; the forces array carries over between calls like
// simpleModel::forces (zero before the first call, velocityVerletNVE.cpp:14-21).
int oracle_simulate(void* m, int kind, int steps, int n, int* face, double* bary, double* vel, double* force,
                    const double* params, double* chain, int nThreads, long long* statsOut)
{
    Mesh* M = (Mesh*)m;
    SysParams P{(int)params[0], params[1], params[2], params[3], (int)params[4], params[5], params[6]};
    double dt = params[7], T = params[8];
    int Mc = (int)params[10];
    std::vector<double> disp(3 * n);
    int err = 0;
    GeoStats st;
    long long inr = 0;
#ifdef _OPENMP
    if (nThreads > 0) omp_set_num_threads(nThreads);
#endif
    for (int s = 0; s < steps; ++s) {
        if (kind == 0) {
            for (int i = 0; i < 3 * n; ++i) {
                disp[i] = dt * vel[i] + 0.5 * dt * dt * force[i];
                vel[i] += 0.5 * dt * force[i];
            }
            err |= move_all(*M, n, face, bary, disp.data(), vel, nThreads);
            compute_forces(*M, P, n, face, bary, force, nullptr, nThreads, &inr, &st);
            for (int i = 0; i < 3 * n; ++i) vel[i] += 0.5 * dt * force[i];
        } else {
            // noseHooverNVT::performUpdate (noseHooverNVT.cpp:42-59, 65-139)
            double* bv = chain;  // (Mc+1) x 4
            double& KE = chain[4 * (Mc + 1)];
            double& scale = chain[4 * (Mc + 1) + 1];
            double dt2 = 0.5 * dt, dt4 = 0.25 * dt, dt8 = 0.125 * dt;
            auto propagateChain = [&]() {
                double ef = 0;
                for (int ii = Mc - 1; ii > 0; --ii) {
                    bv[4 * ii + 2] = (bv[4 * (ii - 1) + 3] * bv[4 * (ii - 1) + 1] * bv[4 * (ii - 1) + 1] - T) / bv[4 * ii + 3];
                    ef = std::exp(-dt8 * bv[4 * (ii + 1) + 1]);
                    bv[4 * ii + 1] *= ef;
                    bv[4 * ii + 1] += bv[4 * ii + 2] * dt4;
                    bv[4 * ii + 1] *= ef;
                }
                bv[2] = (2.0 * KE / bv[3] - 1.0);
                ef = std::exp(-dt8 * bv[4 + 1]);
                bv[1] *= ef;
                bv[1] += bv[2] * dt4;
                bv[1] *= ef;
                for (int ii = 0; ii < Mc; ++ii) bv[4 * ii] += dt2 * bv[4 * ii + 1];
                scale = std::exp(-dt2 * bv[1]);
                KE = scale * scale * KE;
                bv[2] = (2.0 * KE / bv[3] - 1.0);
                ef = std::exp(-dt8 * bv[4 + 1]);
                bv[1] *= ef;
                bv[1] += bv[2] * dt4;
                bv[1] *= ef;
                for (int ii = 1; ii < Mc; ++ii) {
                    bv[4 * ii + 2] = (bv[4 * (ii - 1) + 3] * bv[4 * (ii - 1) + 1] * bv[4 * (ii - 1) + 1] - T) / bv[4 * ii + 3];
                    ef = std::exp(-dt8 * bv[4 * (ii + 1) + 1]);
                    bv[4 * ii + 1] *= ef;
                    bv[4 * ii + 1] += bv[4 * ii + 2] * dt4;
                    bv[4 * ii + 1] *= ef;
                }
            };
            propagateChain();
            for (int i = 0; i < 3 * n; ++i) vel[i] = scale * vel[i];
            KE = 0.0;
            for (int i = 0; i < 3 * n; ++i) disp[i] = dt2 * vel[i];
            err |= move_all(*M, n, face, bary, disp.data(), vel, nThreads);
            compute_forces(*M, P, n, face, bary, force, nullptr, nThreads, &inr, &st);
            for (int i = 0; i < n; ++i) {
                double vv = 0;
                for (int c = 0; c < 3; ++c) {
                    vel[3 * i + c] = vel[3 * i + c] + (dt / 1.0) * force[3 * i + c];
                    disp[3 * i + c] = dt2 * vel[3 * i + c];
                }
                vv = vel[3 * i] * vel[3 * i] + vel[3 * i + 1] * vel[3 * i + 1] + vel[3 * i + 2] * vel[3 * i + 2];
                KE += 0.5 * 1.0 * vv;
            }
            err |= move_all(*M, n, face, bary, disp.data(), vel, nThreads);
            propagateChain();
            for (int i = 0; i < 3 * n; ++i) vel[i] = scale * vel[i];
        }
    }
    if (statsOut) {
        statsOut[0] = st.windowsCreated;
        statsOut[1] = st.windowsProcessed;
        statsOut[2] = st.vertexLaunches;
        statsOut[3] = inr;
    }
    return err;
}

// fireMinimization::minimizeByFire (src/updaters/fireMinimization.cpp:3-21): forces, then velocity-Verlet half
// steps (velocityVerletNVE.cpp:14-29) with the force and the velocity transported by the walk (simpleModel.cpp:44-66:
// force first, then velocity, because fireMinimization::setModel sets both transport flags), fireStep (:38-77) and
// getMaxForce (src/updaters/baseUpdater.cpp:39-54) until forceMax <= forceCutoff or maximumIterations.
//   fire : maximumIterations, alphaStart, deltaTMax, deltaTMin, deltaTInc, deltaTDec, alphaDec, nMin, forceCutoff,
//          alphaMin
//   state: deltaT, alpha, nSinceNegativePower (in/out: the reference keeps them as members between calls)
//   out  : iterations, forceMax
int oracle_fire(void* m, int n, int* face, double* bary, double* vel, double* force, const double* params,
                const double* fire, double* state, int nThreads, double* out)
{
    Mesh* M = (Mesh*)m;
    SysParams P{(int)params[0], params[1], params[2], params[3], (int)params[4], params[5], params[6]};
    const int maxIt = (int)fire[0];
    const double alphaStart = fire[1], dtMax = fire[2], dtMin = fire[3], dtInc = fire[4], dtDec = fire[5];
    const double alphaDec = fire[6], cutoff = fire[8], alphaMin = fire[9];
    const int nMin = (int)fire[7];
    double dt = state[0], alpha = state[1];
    int nSince = (int)state[2];
    std::vector<double> disp(3 * n), tv(6 * (size_t)n);
    long long inr = 0;
    GeoStats st;
    int err = 0;
    auto maxForce = [&]() {
        double mx = 0;
        for (int i = 0; i < n; ++i) {
            double q = force[3 * i] * force[3 * i] + force[3 * i + 1] * force[3 * i + 1] + force[3 * i + 2] * force[3 * i + 2];
            if (q > mx) mx = q;
        }
        return std::sqrt(mx);
    };
    auto dot = [&](const double* a, const double* b) {
        double acc = 0;
        for (int i = 0; i < n; ++i) acc += a[3 * i] * b[3 * i] + a[3 * i + 1] * b[3 * i + 1] + a[3 * i + 2] * b[3 * i + 2];
        return acc;
    };
    compute_forces(*M, P, n, face, bary, force, nullptr, nThreads, &inr, &st);
    double fmax = maxForce();
    int it = 0;
    while (it < maxIt && fmax > cutoff) {
        it += 1;
        for (int i = 0; i < 3 * n; ++i) {
            disp[i] = dt * vel[i] + 0.5 * dt * dt * force[i];
            vel[i] += 0.5 * dt * force[i];
        }
        for (int i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c) {
                tv[6 * i + c] = force[3 * i + c];
                tv[6 * i + 3 + c] = vel[3 * i + c];
            }
#pragma omp parallel for schedule(static) reduction(| : err)
        for (int i = 0; i < n; ++i) {
            int s2 = transport_one(*M, face[i], &bary[3 * i], &disp[3 * i], &tv[6 * i], 2, 100000, nullptr, g_bc);
            if (s2) err |= (1 << s2);
        }
        for (int i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c) {
                force[3 * i + c] = tv[6 * i + c];
                vel[3 * i + c] = tv[6 * i + 3 + c];
            }
        compute_forces(*M, P, n, face, bary, force, nullptr, nThreads, &inr, &st);
        for (int i = 0; i < 3 * n; ++i) vel[i] += 0.5 * dt * force[i];
        // fireStep
        const double forceNorm = dot(force, force), velocityNorm = dot(vel, vel), power = dot(force, vel);
        double scaling = 0.0;
        if (forceNorm > 0) scaling = std::sqrt(velocityNorm / forceNorm);
        for (int i = 0; i < 3 * n; ++i) vel[i] = (1 - alpha) * vel[i] + alpha * scaling * force[i];
        if (power > 0) {
            if (nSince > nMin) {
                dt = std::min(dt * dtInc, dtMax);
                alpha = alpha * alphaDec;
                alpha = std::max(alpha, alphaMin);
            }
            nSince += 1;
        } else {
            nSince = 0;
            dt = dt * dtDec;
            dt = std::max(dt, dtMin);
            alpha = alphaStart;
            for (int i = 0; i < 3 * n; ++i) vel[i] = 0.0;
        }
        fmax = maxForce();
    }
    state[0] = dt;
    state[1] = alpha;
    state[2] = nSince;
    out[0] = it;
    out[1] = fmax;
    return err;
}

// simulation::computeMonodisperseStress (src/simulation/simulation.cpp:104-173) for one force computer: sums
// f(t_ij, d_ij) (x) t_ij over every neighbour pair and, as the reference does inside the same pair loop, v_i (x) v_i
// once per neighbour pair; stress = rho v(x)v / (2N) + f(x)t / (2 * 2 * area * N) with rho = N / area, kB = 1.
void oracle_stress(void* m, int n, const int* face, const double* bary, const double* vel, const double* params,
                   double* stress)
{
    Mesh* M = (Mesh*)m;
    SysParams P{(int)params[0], params[1], params[2], params[3], (int)params[4], params[5], params[6]};
    std::vector<int> off(n + 1);
    long long cap = (long long)n * 64 + 1024;
    std::vector<int> idx;
    std::vector<double> mc(n);
    long long tot;
    while (true) {
        idx.resize(cap);
        tot = oracle_candidates((void*)M, n, face, bary, P.range, off.data(), idx.data(), cap, mc.data());
        if (tot >= 0) break;
        cap = -tot;
    }
    double fdr[9] = {0}, vv[9] = {0};
    GeoWork W;
    GeoStats st;
    std::vector<int> tf, faces;
    std::vector<double> tb, d, ts;
    for (int i = 0; i < n; ++i) {
        int a = off[i], b = off[i + 1], nt = b - a;
        if (nt == 0) continue;
        tf.resize(nt);
        tb.resize(3 * nt);
        d.resize(nt);
        ts.resize(3 * nt);
        for (int q = 0; q < nt; ++q) {
            int jj = idx[a + q];
            tf[q] = face[jj];
            for (int c = 0; c < 3; ++c) tb[3 * q + c] = bary[3 * jj + c];
        }
        const int* fs = nullptr;
        int nfs = 0;
        if (P.submesh) {
            double r = P.maxDist;
            if (mc[i] < P.maxDist) r = mc[i];
            build_patch(*M, face[i], &bary[3 * i], tf.data(), nt, r, faces);
            fs = faces.data();
            nfs = (int)faces.size();
        }
        geodesic_one(*M, W, face[i], &bary[3 * i], nt, tf.data(), tb.data(), fs, nfs, P.cutoff, true, d.data(),
                     ts.data(), nullptr, &st);
        for (int q = 0; q < nt; ++q) {
            double f3[3] = {0, 0, 0};
            if (d[q] < kInf && (P.forceKind != 0 || d[q] <= P.sigma)) {
                double fm = pair_force_mag(P, d[q]);
                for (int c = 0; c < 3; ++c) f3[c] = fm * ts[3 * q + c];
            }
            for (int al = 0; al < 3; ++al)
                for (int be = 0; be < 3; ++be) {
                    fdr[3 * al + be] += f3[al] * ts[3 * q + be];
                    vv[3 * al + be] += vel[3 * i + al] * vel[3 * i + be];
                }
        }
    }
    const double area = M->area;
    const double density = n / area;
    for (int k = 0; k < 9; ++k) stress[k] = density * 1.0 * vv[k] / (2 * n) + fdr[k] / (2 * 2 * area * n);
}

// Boundary condition of every later walk: 0 closed (triangulatedMeshSpace), 1 tangentialOpenMeshSpace,
// 2 absorbingOpenMeshSpace.
void oracle_set_boundary(int bc) { g_bc = bc; }

// noseHooverNVT::setBathVariables (noseHooverNVT.cpp:28-36): fills chain as used by oracle_simulate
void oracle_nvt_init(int n, double T, double tau, int Mc, double* chain)
{
    for (int i = 0; i < 4 * (Mc + 1) + 2; ++i) chain[i] = 0;
    chain[3] = 2.0 * (n - 1) * T * tau * tau;
    for (int ii = 1; ii < Mc + 1; ++ii) chain[4 * ii + 3] = T * tau * tau;
    chain[4 * (Mc + 1)] = chain[3];
    chain[4 * (Mc + 1) + 1] = 1.0;
}

}  // extern "C"
