// Geodesic face walk with parallel transport: one thread per particle, FP64.
//
// Restates triangulatedMeshSpace::transportParticleAndVectors (src/models/triangulatedMeshSpace.cpp:448-564) with
// updateForEdgeIntersection (:614-658), updateForVertexIntersection (:566-611), throughVertex (:247-407) and the
// barycentric helpers of src/utility/meshUtilities.cpp:138-331 (clamps, line/edge intersections) and
// src/utility/functionUtilities.cpp:8-45 (Rodrigues rotation, angleBetween).  Same tolerances (1e-14 normal
// projection, 1e-13 near-zero clamp, 1e-11 below-zero clamp), same edge order and last-edge exclusion, same
// vertex-crossing rules (transport rotation only when n_s.n_t < 0, remaining length measured before the vertex).
// Edge and vertex crossings rotate by cos = n_s.n_t and sin = |n_s x n_t| instead of evaluating acos and then
// cos/sin of it, so no transcendental function is involved in an edge crossing.
//
// This translation unit is compiled with -fmad=false so an edge-crossing walk performs exactly the IEEE operations
// of the CPU restatement (no fused multiply-add contraction).
//
// Memory: per particle-step it reads face (4 B), bary (24 B), disp (24 B; the force instead in the NVE kick mode),
// transported vectors (24 B each) and writes them back; each crossing reads the next face's 3 vertex indices,
// 3 neighbours, 3 vertex positions and normal.  The face arrays are gathered with ordinary loads: particles address
// faces at random, so a bulk tensor copy (TMA) of a fixed tile has nothing to stage.
//
// The kernel also carries two pieces of the step around it, to save launches: the velocity-Verlet first half
// (kick + drift, velocityVerletNVE.cpp:14-21) when given the forces, and the reduction of its warps' failure codes
// into the system's status bits.
#include "cssg_internal.cuh"

namespace {

#define WALK_MAX_TRANSPORT 4

__device__ __forceinline__ void ld3(const double* p, double* o)
{
    o[0] = p[0];
    o[1] = p[1];
    o[2] = p[2];
}
__device__ __forceinline__ double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
__device__ __forceinline__ void cross3(const double* a, const double* b, double* o)
{
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

struct FacePts {
    double p[3][3];
};

__device__ __forceinline__ void load_face(const DevMesh& M, int f, FacePts& P)
{
    for (int k = 0; k < 3; ++k) ld3(&M.V[3 * M.F[3 * f + k]], P.p[k]);
}

// PMP::barycentric_coordinates formula
__device__ void bary_of(const FacePts& P, const double* x, double* out)
{
    double v0[3], v1[3], v2[3];
    for (int c = 0; c < 3; ++c) {
        v0[c] = P.p[1][c] - P.p[0][c];
        v1[c] = P.p[2][c] - P.p[0][c];
        v2[c] = x[c] - P.p[0][c];
    }
    double d00 = dot3(v0, v0), d01 = dot3(v0, v1), d11 = dot3(v1, v1);
    double d20 = dot3(v2, v0), d21 = dot3(v2, v1);
    double denom = d00 * d11 - d01 * d01;
    double v = (d11 * d20 - d01 * d21) / denom;
    double w = (d00 * d21 - d01 * d20) / denom;
    out[0] = 1.0 - v - w;
    out[1] = v;
    out[2] = w;
}

// Divisions by a weight sum below: normalised weights usually sum to exactly 1 (about 80-97% of the sums in a walk
// step), and x / 1 == x exactly, so the division (the costliest FP64 operation of the walk, ~10 FP64-pipe
// instructions) is skipped then.  The results are the same bits either way.

// barycenter of three weighted points (PMP::construct_point)
__device__ __forceinline__ void construct_pt(const FacePts& P, const double* b, double* out)
{
    const double s = b[0] + b[1] + b[2];
    for (int c = 0; c < 3; ++c) {
        const double x = b[0] * P.p[0][c] + b[1] * P.p[1][c] + b[2] * P.p[2][c];
        out[c] = s == 1.0 ? x : x / s;
    }
}

__device__ __forceinline__ void below_zero_clamp(double* b)
{
    const double tol = 1e-11;
    double s = 0;
    for (int i = 0; i < 3; ++i) {
        b[i] = fmax(b[i], tol);
        s += b[i];
    }
    if (s != 1.0)
        for (int i = 0; i < 3; ++i) b[i] = b[i] / s;
}

__device__ __forceinline__ void near_zero_clamp(double* b)
{
    const double tol = 1e-13;
    double s = 0;
    for (int i = 0; i < 3; ++i) {
        if (b[i] > -tol && b[i] < tol) b[i] = tol;
        s += b[i];
    }
    if (s != 1.0)
        for (int i = 0; i < 3; ++i) b[i] = b[i] / s;
}

__device__ bool hit_v1v2(const double* s, const double* e, double* ip)
{
    double den = s[0] + s[1] - e[0] - e[1];
    if (den == 0) return false;
    double t1 = (-e[1] + e[1] * s[0] + s[1] - e[0] * s[1]) / den;
    double t2 = (-1 + s[0] + s[1]) / den;
    for (int c = 0; c < 3; ++c) ip[c] = s[c] + t2 * (e[c] - s[c]);
    return t1 >= 0 && t1 <= 1 && t2 >= 0 && t2 <= 1;
}
__device__ bool hit_v2v3(const double* s, const double* e, double* ip)
{
    double den = -e[0] + s[0];
    if (den == 0) return false;
    double t1 = -(e[0] - s[0] + e[1] * s[0] - e[0] * s[1]) / den;
    double t2 = s[0] / den;
    for (int c = 0; c < 3; ++c) ip[c] = s[c] + t2 * (e[c] - s[c]);
    return t1 >= 0 && t1 <= 1 && t2 >= 0 && t2 <= 1;
}
__device__ bool hit_v3v1(const double* s, const double* e, double* ip)
{
    double den = s[1] - e[1];
    if (den == 0) return false;
    double t1 = (e[0] * s[1] - e[1] * s[0]) / den;
    double t2 = s[1] / den;
    for (int c = 0; c < 3; ++c) ip[c] = s[c] + t2 * (e[c] - s[c]);
    return t1 >= 0 && t1 <= 1 && t2 >= 0 && t2 <= 1;
}

__device__ void rotate_about(const double* p, const double* o, const double* a, double c, double s, double* out)
{
    double sh[3] = {p[0] - o[0], p[1] - o[1], p[2] - o[2]};
    double d = a[0] * sh[0] + a[1] * sh[1] + a[2] * sh[2];
    double r0 = a[0] * d * (1. - c) + sh[0] * c + (a[1] * sh[2] - a[2] * sh[1]) * s;
    double r1 = a[1] * d * (1. - c) + sh[1] * c + (a[2] * sh[0] - a[0] * sh[2]) * s;
    double r2 = a[2] * d * (1. - c) + sh[2] * c + (a[0] * sh[1] - a[1] * sh[0]) * s;
    out[0] = r0 + o[0];
    out[1] = r1 + o[1];
    out[2] = r2 + o[2];
}

__device__ double angle_between(const double* u, const double* v)
{
    double nu = sqrt(dot3(u, u)), nv = sqrt(dot3(v, v));
    double a[3] = {u[0] / nu, u[1] / nu, u[2] / nu}, b[3] = {v[0] / nv, v[1] / nv, v[2] / nv};
    double d = dot3(a, b);
    if (d >= 1) return 0;
    if (d <= -1) return 3.14159265358979323846;
    return acos(d);
}

__device__ __forceinline__ void ring_edge(const DevMesh& M, int v, int rb, int n, int s0, int i, double* e)
{
    int w = M.ringV[rb + (s0 + i) % n];
    double l2 = 0;
    for (int c = 0; c < 3; ++c) {
        e[c] = M.V[3 * w + c] - M.V[3 * v + c];
        l2 += e[c] * e[c];
    }
    double l = sqrt(l2);
    for (int c = 0; c < 3; ++c) e[c] /= l;
}

// throughVertex: straightest continuation through vertex v, half the total vertex angle on each side
__device__ int through_vertex(const DevMesh& M, int v, const double* toInter, int srcFace, int* outFace, double* heading)
{
    if (!(M.vflag[v] & VF_RING)) return CSSG_ST_BORDER;
    int startV = -1;
    for (int k = 0; k < 3; ++k)
        if (M.F[3 * srcFace + k] == v) startV = M.F[3 * srcFace + (k + 1) % 3];
    int rb = M.ringStart[v], n = M.ringStart[v + 1] - rb;
    int s0 = -1;
    for (int i = 0; i < n; ++i)
        if (M.ringV[rb + i] == startV) s0 = i;
    if (s0 < 0 || n < 3) return CSSG_ST_VERTEX;
    double ea[3], eb[3];
    double total = 0;
    for (int i = 0; i < n; ++i) {
        ring_edge(M, v, rb, n, s0, i, ea);
        ring_edge(M, v, rb, n, s0, (i + 1) % n, eb);
        total += angle_between(ea, eb);
    }
    double half = total / 2.0;
    double qh[3] = {-toInter[0], -toInter[1], -toInter[2]};
    double ql = sqrt(dot3(qh, qh));
    for (int c = 0; c < 3; ++c) qh[c] /= ql;
    ring_edge(M, v, rb, n, s0, 0, ea);
    double traveled = angle_between(qh, ea);
    int counter = 0;
    while (traveled < half) {
        ring_edge(M, v, rb, n, s0, counter, ea);
        ring_edge(M, v, rb, n, s0, (counter + 1) % n, eb);
        traveled += angle_between(ea, eb);
        counter++;
        if (counter >= n) return CSSG_ST_VERTEX;
    }
    if (counter == 0) return CSSG_ST_VERTEX;
    double diff = half - traveled;
    ring_edge(M, v, rb, n, s0, counter - 1, ea);
    ring_edge(M, v, rb, n, s0, counter, eb);
    double ax[3];
    cross3(ea, eb, ax);
    double al = sqrt(dot3(ax, ax));
    for (int c = 0; c < 3; ++c) ax[c] /= al;
    const double* vi = &M.V[3 * v];
    double rt[3] = {vi[0] + eb[0], vi[1] + eb[1], vi[2] + eb[2]};
    double pr[3];
    rotate_about(rt, vi, ax, cos(diff), sin(diff), pr);
    double h[3] = {pr[0] - vi[0], pr[1] - vi[1], pr[2] - vi[2]};
    double hl = sqrt(dot3(h, h));
    for (int c = 0; c < 3; ++c) heading[c] = h[c] / hl;
    int want1 = M.ringV[rb + (s0 + counter - 1) % n], want2 = M.ringV[rb + (s0 + counter) % n];
    for (int i = M.vfStart[v]; i < M.vfStart[v + 1]; ++i) {
        int f = M.vfList[i];
        if (f == srcFace) continue;
        bool h1 = false, h2 = false;
        for (int k = 0; k < 3; ++k) {
            h1 |= M.F[3 * f + k] == want1;
            h2 |= M.F[3 * f + k] == want2;
        }
        if (h1 && h2) {
            *outFace = f;
            return CSSG_ST_OK;
        }
    }
    return CSSG_ST_VERTEX;
}

__device__ int face_across(const DevMesh& M, int f, int va, int vb)
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

__device__ __forceinline__ void normalize3(double* v)
{
    const double l = sqrt(dot3(v, v));
    for (int c = 0; c < 3; ++c) v[c] = v[c] / l;
}

// triangulatedMeshSpace::projectVectorsIfOverBoundary (triangulatedMeshSpace.cpp:411-426) with
// projectVectorOrthogonalToDirection (meshUtilities.cpp:125-129)
__device__ void project_if_over_boundary(double (*tv)[3], int ntv, const double* orthogonal, const double* inward)
{
    const bool pointsOut = dot3(orthogonal, inward) < 0;
    double dh[3] = {orthogonal[0], orthogonal[1], orthogonal[2]};
    normalize3(dh);
    for (int i = 0; i < ntv; ++i) {
        const bool alongPerp = dot3(tv[i], orthogonal) > 0;
        if ((pointsOut && alongPerp) || (!pointsOut && !alongPerp)) {
            const double d = dot3(tv[i], dh);
            for (int c = 0; c < 3; ++c) tv[i][c] = tv[i][c] - d * dh[c];
        }
    }
}

// openMeshSpace::getBoundaryVertexHeading (openMeshSpace.cpp:3-75) by its stated rule: the next heading runs along
// the edge from v that overlaps most with the displacement, among the edges of v's faces other than the current one
// (every (neighbour, face) pair, faces in increasing index order, first maximum kept; the reference's circulator
// loop sees a subset that depends on CGAL's per-vertex halfedge).  Returns the new face or -1.
__device__ int boundary_vertex_heading(const DevMesh& M, int v, int f, const double* disp, double* heading,
                                       int* neighbour)
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
            double out[3] = {M.V[3 * w] - M.V[3 * v], M.V[3 * w + 1] - M.V[3 * v + 1], M.V[3 * w + 2] - M.V[3 * v + 2]};
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
__device__ void project_for_boundary_vertex(const DevMesh& M, const double* heading, int v, int w,
                                            const double* fNormal, int g, double (*tv)[3], int ntv)
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
    double inward[3];
    for (int c = 0; c < 3; ++c) inward[c] = (inside >= 0 ? M.V[3 * inside + c] : 0.0) - M.V[3 * v + c];
    project_if_over_boundary(tv, ntv, orth, inward);
}

// With M.bc != BC_CLOSED, the loop of openMeshSpace::transportParticleAndVectors (openMeshSpace.cpp:101-238), which
// differs only at border edges (updateAtBoundaryEdge) and border vertices (updateAtBoundaryVertex) of the
// tangential (tangentialOpenMeshSpace.cpp) and absorbing (absorbingOpenMeshSpace.cpp) conditions.
__device__ int transport_one(const DevMesh& M, int& face, double* bary, double* disp, double (*tv)[3], int ntv,
                             int maxIter, int* crossings, double* finalPos)
{
    int f = face;
    FacePts P;
    load_face(M, f, P);
    double sb[3] = {bary[0], bary[1], bary[2]};
    double sp[3];
    construct_pt(P, sb, sp);
    double ns[3];
    ld3(&M.N[3 * f], ns);
    double nd = dot3(ns, disp);
    if (fabs(nd) > 1e-14)
        for (int c = 0; c < 3; ++c) disp[c] -= nd * ns[c];
    double target[3] = {sp[0] + disp[0], sp[1] + disp[1], sp[2] + disp[2]};
    int lastA = -1, lastB = -1;
    double tb[3];
    int iter = 0, cross = 0;
    // qf: the face whose triangle the target's weights are computed against.  The reference keeps its vertex
    // positions in vertexPositions, which updateForEdgeIntersection refreshes (by reference) but
    // updateForVertexIntersection and getBoundaryVertexHeading receive by value: after a vertex crossing the target
    // is weighed against the triangle of the face before the vertex, and the weights are read in the new face.
    int qf = f;
    while (true) {
        if (++iter > maxIter) return CSSG_ST_ITER;
        if (qf == f) {
            bary_of(P, target, tb);
        } else {
            FacePts Q;
            load_face(M, qf, Q);
            bary_of(Q, target, tb);
        }
        near_zero_clamp(tb);
        construct_pt(P, tb, target);
        below_zero_clamp(sb);
        construct_pt(P, sb, sp);
        for (int c = 0; c < 3; ++c) disp[c] = target[c] - sp[c];
        if (tb[0] != tb[0]) return CSSG_ST_NAN;
        if (tb[0] >= 0 && tb[1] >= 0 && tb[2] >= 0) break;
        int vl[3] = {M.F[3 * f], M.F[3 * f + 1], M.F[3 * f + 2]};
        double ip[3], ic[3];
        int nhit = 0, inv0 = -1, inv1 = -1;
#define IS_LAST(a, b) (((a) == lastA && (b) == lastB) || ((a) == lastB && (b) == lastA))
        if (!IS_LAST(vl[0], vl[1]) && hit_v1v2(sb, tb, ic)) {
            for (int c = 0; c < 3; ++c) ip[c] = ic[c];
            if (nhit == 0) { inv0 = vl[0]; inv1 = vl[1]; }
            nhit++;
        }
        if (!IS_LAST(vl[1], vl[2]) && hit_v2v3(sb, tb, ic)) {
            for (int c = 0; c < 3; ++c) ip[c] = ic[c];
            if (nhit == 0) { inv0 = vl[1]; inv1 = vl[2]; }
            nhit++;
        }
        if (!IS_LAST(vl[2], vl[0]) && hit_v3v1(sb, tb, ic)) {
            for (int c = 0; c < 3; ++c) ip[c] = ic[c];
            if (nhit == 0) { inv0 = vl[2]; inv1 = vl[0]; }
            nhit++;
        }
#undef IS_LAST
        if (nhit == 0) return CSSG_ST_NO_INTERSECTION;
        below_zero_clamp(ip);
        double ep[3];
        construct_pt(P, ip, ep);
        double toI[3] = {ep[0] - sp[0], ep[1] - sp[1], ep[2] - sp[2]};
        for (int c = 0; c < 3; ++c) {
            sb[c] = ip[c];
            sp[c] = ep[c];
        }
        cross++;
        if (nhit == 2) {
            int v = inv0;  // the reference passes involvedVertex[0], the first vertex of the first edge hit
            if (M.vflag[v] & VF_BORDER) {
                if (M.bc == BC_CLOSED) return CSSG_ST_BORDER;
                double heading[3];
                int w = -1;
                const int g = boundary_vertex_heading(M, v, f, disp, heading, &w);
                if (g < 0) return CSSG_ST_VERTEX;
                f = g;
                load_face(M, f, P);
                bary_of(P, &M.V[3 * v], sb);
                if (ntv > 0) project_for_boundary_vertex(M, heading, v, w, ns, f, tv, ntv);
                // getBoundaryVertexHeading receives vertexPositions and sourceNormal by value, so the caller keeps the
                // previous face's: qf and ns are not updated here
                lastA = lastB = -1;
                if (M.bc == BC_ABSORBING) {
                    for (int c = 0; c < 3; ++c) tb[c] = sb[c];
                    break;
                }
                double hh[3] = {heading[0], heading[1], heading[2]};  // projectVectorOntoDirection
                normalize3(hh);
                const double d2 = dot3(disp, hh);
                construct_pt(P, sb, sp);
                for (int c = 0; c < 3; ++c) {
                    disp[c] = d2 * hh[c];
                    target[c] = sp[c] + disp[c];
                }
                continue;
            }
            int g = -1;
            double heading[3];
            int st = through_vertex(M, v, toI, f, &g, heading);
            if (st) return st;
            double len = sqrt(dot3(disp, disp));
            double nt[3];
            ld3(&M.N[3 * g], nt);
            for (int c = 0; c < 3; ++c) {
                disp[c] = heading[c] * len;
                target[c] = sp[c] + disp[c];
            }
            if (ntv > 0) {
                double ndt = dot3(ns, nt);
                if (ndt < 0) {
                    double ax[3];
                    cross3(ns, nt, ax);
                    double al = sqrt(dot3(ax, ax));
                    for (int c = 0; c < 3; ++c) ax[c] /= al;
                    for (int i = 0; i < ntv; ++i) {
                        double q[3] = {sp[0] + tv[i][0], sp[1] + tv[i][1], sp[2] + tv[i][2]};
                        double r[3];
                        rotate_about(q, sp, ax, ndt, al, r);
                        for (int c = 0; c < 3; ++c) tv[i][c] = r[c] - sp[c];
                    }
                }
            }
            f = g;
            load_face(M, f, P);
            bary_of(P, sp, sb);
            for (int c = 0; c < 3; ++c) ns[c] = nt[c];
            lastA = lastB = -1;
            continue;
        }
        if (nhit != 1) return CSSG_ST_NO_INTERSECTION;
        int g = face_across(M, f, inv0, inv1);
        if (g < 0) {
            if (M.bc == BC_CLOSED) return CSSG_ST_BORDER;
            // updateAtBoundaryEdge (tangentialOpenMeshSpace.cpp:3-39, absorbingOpenMeshSpace.cpp:2-26)
            int inner = -1;
            for (int k = 0; k < 3; ++k)
                if (M.F[3 * f + k] != inv0 && M.F[3 * f + k] != inv1) inner = M.F[3 * f + k];
            double edge[3], orth[3], inward[3], here[3];
            for (int c = 0; c < 3; ++c) edge[c] = M.V[3 * inv1 + c] - M.V[3 * inv0 + c];
            // the absorbing rule recomputes the face normal, the tangential rule uses the loop's sourceNormal
            double nf[3];
            if (M.bc == BC_ABSORBING) ld3(&M.N[3 * f], nf);
            else ld3(ns, nf);
            cross3(nf, edge, orth);
            normalize3(orth);
            construct_pt(P, sb, here);
            for (int c = 0; c < 3; ++c) inward[c] = M.V[3 * inner + c] - here[c];
            if (M.bc == BC_ABSORBING) {
                if (ntv > 0) project_if_over_boundary(tv, ntv, orth, inward);
                for (int c = 0; c < 3; ++c) tb[c] = sb[c];
                break;
            }
            double fwd[3] = {edge[0], edge[1], edge[2]}, bwd[3];
            for (int c = 0; c < 3; ++c) bwd[c] = M.V[3 * inv0 + c] - M.V[3 * inv1 + c];
            normalize3(fwd);
            normalize3(bwd);
            double dn[3] = {disp[0], disp[1], disp[2]};
            normalize3(dn);
            const double fd = dot3(dn, fwd), bd = dot3(dn, bwd);
            const double len = sqrt(dot3(disp, disp));  // the whole remaining displacement, measured before the edge
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
        construct_pt(P, ip, sp);
        double nt[3];
        ld3(&M.N[3 * g], nt);
        double ndt = dot3(ns, nt);
        // the reference also divides by |n_s x n_t| here; for coplanar faces whose normals' dot product rounds
        // below 1 that length is exactly zero (NaN there); the rotation is then the identity and is skipped
        if (ndt < 1 && (ns[0] * nt[1] - ns[1] * nt[0] != 0 || ns[1] * nt[2] - ns[2] * nt[1] != 0 ||
                        ns[2] * nt[0] - ns[0] * nt[2] != 0)) {
            double ax[3];
            cross3(ns, nt, ax);
            double al = sqrt(dot3(ax, ax));
            for (int c = 0; c < 3; ++c) ax[c] /= al;
            double r[3];
            rotate_about(target, sp, ax, ndt, al, r);
            for (int c = 0; c < 3; ++c) {
                target[c] = r[c];
                disp[c] = target[c] - sp[c];
            }
            for (int i = 0; i < ntv; ++i) {
                double q[3] = {sp[0] + tv[i][0], sp[1] + tv[i][1], sp[2] + tv[i][2]};
                rotate_about(q, sp, ax, ndt, al, r);
                for (int c = 0; c < 3; ++c) tv[i][c] = r[c] - sp[c];
            }
        }
        lastA = inv0;
        lastB = inv1;
        f = g;
        qf = g;
        load_face(M, f, P);
        bary_of(P, sp, sb);
        for (int c = 0; c < 3; ++c) ns[c] = nt[c];
    }
    face = f;
    for (int c = 0; c < 3; ++c) bary[c] = tb[c];
    if (finalPos) construct_pt(P, tb, finalPos);
    *crossings = cross;
    return CSSG_ST_OK;
}

__global__ void __launch_bounds__(128) transport_kernel(const DevMesh* __restrict__ meshes, const int* __restrict__ meshOf,
                                                        int n, int* __restrict__ face,
                                                        double* __restrict__ bary, double* __restrict__ disp,
                                                        double* __restrict__ transport, int ntv, int* __restrict__ status,
                                                        unsigned long long* crossings, double* __restrict__ posOut,
                                                        const int* __restrict__ skip, int* __restrict__ statusBits,
                                                        const double* __restrict__ kickForce, double kickDt,
                                                        const int* __restrict__ skipSys)
{
    if (skip && *skip) return;  // a device-side stop flag (FIRE after convergence): nothing moves
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int cr = 0, bits = 0;
    // skipSys: per-system stop flags (batched FIRE), the particles of a stopped system stay where they are
    if (i < n && !(skipSys && skipSys[meshOf ? meshOf[i] : 0])) {
        const DevMesh& M = meshes[meshOf ? meshOf[i] : 0];
        int f = face[i];
        double b[3] = {bary[3 * i], bary[3 * i + 1], bary[3 * i + 2]};
        double d[3];
        double tv[WALK_MAX_TRANSPORT][3];
        for (int t = 0; t < ntv; ++t)
            for (int c = 0; c < 3; ++c) tv[t][c] = transport[3 * (ntv * (size_t)i + t) + c];
        if (kickForce) {
            // velocityVerletNVE first half (the velocity is transported vector 0)
            for (int c = 0; c < 3; ++c) {
                const double fc = kickForce[3 * i + c];
                d[c] = kickDt * tv[0][c] + 0.5 * kickDt * kickDt * fc;
                tv[0][c] += 0.5 * kickDt * fc;
            }
        } else {
            for (int c = 0; c < 3; ++c) d[c] = disp[3 * i + c];
        }
        double kicked[3] = {tv[0][0], tv[0][1], tv[0][2]};
        double pos[3];
        int st = transport_one(M, f, b, d, tv, ntv, 100000, &cr, posOut ? pos : nullptr);
        status[i] = st;
        if (st == CSSG_ST_OK) {
            face[i] = f;
            for (int c = 0; c < 3; ++c) bary[3 * i + c] = b[c];
            for (int t = 0; t < ntv; ++t)
                for (int c = 0; c < 3; ++c) transport[3 * (ntv * (size_t)i + t) + c] = tv[t][c];
            if (posOut)
                for (int c = 0; c < 3; ++c) posOut[3 * i + c] = pos[c];
        } else {
            bits = 1 << st;
            if (kickForce)  // the kick stands even where the walk failed
                for (int c = 0; c < 3; ++c) transport[3 * (ntv * (size_t)i) + c] = kicked[c];
        }
        for (int c = 0; c < 3; ++c) disp[3 * i + c] = d[c];
    }
    // warp-aggregated crossing count and failure bits
    const unsigned mask = 0xffffffffu;
    for (int o = 16; o > 0; o >>= 1) {
        cr += __shfl_xor_sync(mask, cr, o);
        bits |= __shfl_xor_sync(mask, bits, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (crossings && cr) atomicAdd(crossings, (unsigned long long)cr);
        if (statusBits && bits) atomicOr(statusBits, bits);
    }
}

__global__ void positions_kernel(const DevMesh* __restrict__ meshes, const int* __restrict__ meshOf, int n,
                                 const int* __restrict__ face, const double* __restrict__ bary, double* __restrict__ pos)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DevMesh& M = meshes[meshOf ? meshOf[i] : 0];
    FacePts P;
    load_face(M, face[i], P);
    double b[3] = {bary[3 * i], bary[3 * i + 1], bary[3 * i + 2]};
    double o[3];
    construct_pt(P, b, o);
    for (int c = 0; c < 3; ++c) pos[3 * i + c] = o[c];
}

}  // namespace

void cssg_launch_transport(const DevMesh* meshes, const int* meshOf, int n, int* face, double* bary, double* disp,
                           double* transport, int nT, int* status, unsigned long long* crossings, double* pos_out,
                           cudaStream_t s, const int* skip, int* status_bits, const double* kick_force, double kick_dt,
                           const int* skip_sys)
{
    if (n <= 0) return;
    // A warp's FP64 instructions share its SM sub-partition's FP64 pipe with the other warps there.  While the
    // particles fit one warp per SM, blocks of one warp spread them over the SMs; beyond that, blocks of four warps.
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int threads = (n <= 32 * sms) ? 32 : 128;
    if (nT < 1) kick_force = nullptr;  // the kick needs the velocity as transported vector 0
    transport_kernel<<<(n + threads - 1) / threads, threads, 0, s>>>(meshes, meshOf, n, face, bary, disp, transport, nT,
                                                                     status, crossings, pos_out, skip, status_bits,
                                                                     kick_force, kick_dt, skip_sys);
}

void cssg_launch_positions(const DevMesh* meshes, const int* meshOf, int n, const int* face, const double* bary,
                           double* pos, cudaStream_t s)
{
    if (n <= 0) return;
    positions_kernel<<<(n + 127) / 128, 128, 0, s>>>(meshes, meshOf, n, face, bary, pos);
}

extern "C" int cssg_transport_batch(cssg_ctx* ctx, const cssg_mesh* mesh, int n, int* face, double* bary, double* disp,
                                    double* transport, int nTransport, int* status, unsigned long long* crossings)
{
    if (!ctx || !mesh || n < 0 || (n > 0 && (!face || !bary || !disp || !status)) || nTransport < 0 ||
        nTransport > WALK_MAX_TRANSPORT || (nTransport > 0 && !transport)) {
        cssg_set_error("cssg_transport_batch: bad arguments (at most 4 transported vectors)");
        return CSSG_ERR_ARG;
    }
    DeviceScope scope(ctx->device);
    CSSG_CUDA(scope.err);
    cssg_launch_transport(mesh->dself, nullptr, n, face, bary, disp, transport, nTransport, status, crossings, nullptr,
                          ctx->stream);
    CSSG_CUDA(cudaGetLastError());
    return CSSG_OK;
}
