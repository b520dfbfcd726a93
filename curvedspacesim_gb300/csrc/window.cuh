// Window geometry of the exact geodesic propagation, shared by the source-group kernel (geodesic.cu) and the
// one-source-per-lane kernel (lanes.cu).
//
// Continuous-Dijkstra window propagation (the Chen-Han / Xin-Wang family of exact algorithms that CGAL's
// Surface_mesh_shortest_path implements), restated from the published method:
//   * a window lives on the edge through which it enters face g; its frame has the origin at the edge's first
//     vertex, x along the edge and y into g; the pseudo-source I = (sx, sy) lies behind the edge at path length
//     sigma from the source; [b0, b1] is the part of the edge it covers;
//   * propagating through g splits the window at the ray through g's opposite vertex C into children on the two
//     other edges (rigid 2D frame changes, no trigonometry);
//   * vertex labels (best known path lengths) trim windows exactly against the two endpoint vertices of their edge
//     (the excess of the window path over an endpoint-vertex path is monotone along the edge) and discard windows
//     that the opposite vertex dominates everywhere;
//   * start tangents ride along: windows from the source carry the rotation of their frame into the source face
//     frame (c, s), windows from a vertex pseudo-source carry that vertex's start direction.
#pragma once
#include <math_constants.h>

#include "cssg_internal.cuh"

namespace {

constexpr unsigned long long INF_BITS = 0x7FF0000000000000ull;
constexpr unsigned FULL = 0xffffffffu;

// FP64 arithmetic of one processed window on its usual path, counted from the functions below (add, subtract and
// multiply 1 flop, fused multiply-add 2, square root 1; rcp_nr = its four fused multiply-adds, 8; comparisons, min/max
// and FP32 work not counted): trim_window 7 (label differences, the trimmed ends, the emptiness test); the opposite
// vertex's proposal 36 (CrossC 5, two interval tests 6, path length 7, start direction through rcp_nr 18); two
// children 98 (per child CrossC 9 with its two tests, make_child 37-39, the interval clamp of the push 2).  A
// window that also proposes an end vertex of its edge adds 7-25 per end.  The propagation roofline counts
// windows processed (the kernels' counters) times this figure; cssg_diag_flops_per_window exports it.
constexpr int kFlopsPerWindow = 141;

struct __align__(16) Win {
    double b0, b1, sx, sy, sigma, c, s;
    int he;     // entered face * 4 + local edge
    float key;  // smallest path length over the interval when queued (ordering and banding only)
};

__device__ __forceinline__ double len2(double x, double y) { return sqrt(x * x + y * y); }

__device__ __forceinline__ unsigned long long dbits(double x) { return (unsigned long long)__double_as_longlong(x); }
__device__ __forceinline__ double bitsd(unsigned long long b)
{
    return b >= INF_BITS ? CUDART_INF : __longlong_as_double((long long)b);
}

// Does the ray from the window's pseudo-source through (px, py) meet the edge line inside [b0 - tol, b1 + tol]?
// The crossing is xp = sx + (px - sx) * (-sy) / D with D = py - sy; for D > 0 (the usual case: the point lies above
// the edge and the pseudo-source below it) the test is done on xp * D, without a division.
__device__ __forceinline__ bool ray_hits(const Win& w, double px, double py, double tol)
{
    const double D = py - w.sy;
    const double num = w.sx * D + (px - w.sx) * (-w.sy);
    if (D > 0) return num >= (w.b0 - tol) * D && num <= (w.b1 + tol) * D;
    const double xp = num / D;
    return xp >= w.b0 - tol && xp <= w.b1 + tol;
}

// Lower bound (FP32, rounded down) of the window's distances: sigma + the distance from the pseudo-source to the
// interval.  The float evaluation's error is far below the 1e-6 * scale subtracted, so the bound stays below the
// exact value: the banding and the early exit only need a lower bound.
__device__ __forceinline__ float key_lo(const Win& w)
{
    const float sx = (float)w.sx, sy = (float)w.sy, b0 = (float)w.b0, b1 = (float)w.b1;
    float m;
    if (sx < b0) m = sqrtf((sx - b0) * (sx - b0) + sy * sy);
    else if (sx > b1) m = sqrtf((sx - b1) * (sx - b1) + sy * sy);
    else m = fabsf(sy);
    const float scale = fabsf(sx) + fabsf(sy) + fabsf(b0) + fabsf(b1);
    return __fsub_rd(__fadd_rd(__double2float_rd(w.sigma), m), 1e-6f * scale + 1e-6f * m);
}

// Remove the parts of the window that a path through an endpoint vertex of its edge beats.  The excess of the
// window's path over the vertex path is monotone along the edge, so the dominated part is an interval at that end,
// bounded by the root of a linear equation.  This is a pruning test, so it runs in FP32 with margins that make it
// conservative: inputs are rounded from FP64 (relative error 6e-8), and every decision below holds with a margin of
// 1e-5 * scale^2 (squared lengths) or 1e-6 * scale (lengths), at least 10x the worst float error, where scale bounds
// the magnitudes involved.  An undecided case keeps the window; a trimmed end is moved back by the root's error
// bound.  The interval itself (and every distance) stays FP64.
__device__ __forceinline__ bool trim_end(float a, float sx, float sy2, float b, float bfar, float scale, float& xs)
{
    // end at b (distance b from the vertex along the edge), pseudo-source at (sx, sy) in the frame with the vertex at
    // the origin; a = vertex label - sigma.  Returns false when the whole window is dominated; xs = new end (>= b)
    // when the end is dominated, else xs = b.
    xs = b;
    const float eps = 1e-6f * scale, eps2 = 1e-5f * scale * scale;
    const float r = a + b, dx = b - sx;
    const bool dominated = (r < -eps) || (r >= -eps && dx * dx + sy2 > r * r + eps2);
    if (!dominated) return true;
    const float den = a + sx;  // > 0: the dominated part ends inside the edge line
    if (den < -eps) return false;
    if (den <= eps) return true;  // undecided: keep
    const float num = (sx - a) * (sx + a) + sy2;
    float root = num / (2.0f * den);
    root -= 1e-5f * scale * (scale + fabsf(root)) / den;  // error bound of the float root
    if (root >= bfar) return false;
    if (root > b) xs = root;
    return true;
}

// Trim a window against the labels of its edge's endpoint vertices (A at the frame origin, B at x = L) and test it
// against the opposite vertex C; returns false when the window is dominated everywhere.  lab(v) returns vertex v's
// label (+inf when it has none); it is called lazily, A first.
template <class Lab>
__device__ __forceinline__ bool trim_window(const DevMesh& M, Win& w, Lab lab)
{
    const int g = w.he >> 2, j = w.he & 3;
    const double L = M.geom[9 * g + 3 * j];
    const int A = M.F[3 * g + j], B = M.F[3 * g + (j + 1) % 3], Cv = M.F[3 * g + (j + 2) % 3];
    const float sx = (float)w.sx, sy = (float)w.sy, Lf = (float)L;
    const float sy2 = sy * sy;
    const float b0 = (float)w.b0, b1 = (float)w.b1;
    const double dA = lab(A);
    if (dA < CUDART_INF) {
        const float a = (float)(dA - w.sigma);
        const float scale = fabsf(sx) + fabsf(sy) + Lf + fabsf(a);
        float xs;
        if (!trim_end(a, sx, sy2, b0, b1, scale, xs)) return false;
        if (xs > b0) w.b0 = fmax(w.b0, (double)xs);
    }
    const double dB = lab(B);
    if (dB < CUDART_INF) {
        // mirrored frame: origin at B, x toward A
        const float a = (float)(dB - w.sigma);
        const float scale = fabsf(sx) + fabsf(sy) + Lf + fabsf(a);
        const float m0 = (float)(L - w.b1), m1 = (float)(L - w.b0);
        float xs;
        if (!trim_end(a, Lf - sx, sy2, m0, m1, scale, xs)) return false;
        if (xs > m0) w.b1 = fmin(w.b1, L - (double)xs);
    }
    if (!(w.b1 - w.b0 > 1e-14 * L)) return false;
    const double dC = lab(Cv);
    if (dC < CUDART_INF) {
        float cx = (float)M.geom[9 * g + 3 * j + 1], cy = (float)M.geom[9 * g + 3 * j + 2];
        float e0 = (float)w.b0, e1 = (float)w.b1;
        float m = fmaxf(sqrtf((cx - e0) * (cx - e0) + cy * cy), sqrtf((cx - e1) * (cx - e1) + cy * cy));
        float near = (sx < e0) ? sqrtf((sx - e0) * (sx - e0) + sy2)
                                : (sx > e1 ? sqrtf((sx - e1) * (sx - e1) + sy2) : fabsf(sy));
        if ((float)dC + m < ((float)w.sigma + near) * (1.0f - 1e-5f)) return false;
    }
    return true;
}

// unit start direction (source frame) of the path through (px, py); l = |(px, py) - (sx, sy)| when sigma == 0
__device__ __forceinline__ void start_dir_l(const Win& w, double px, double py, double l, double& dx, double& dy)
{
    if (w.sigma == 0) {
        const double inv = rcp_nr(l);
        double ux = (px - w.sx) * inv, uy = (py - w.sy) * inv;
        dx = w.c * ux - w.s * uy;
        dy = w.s * ux + w.c * uy;
    } else {
        dx = w.c;
        dy = w.s;
    }
}

__device__ __forceinline__ void start_dir(const Win& w, double px, double py, double& dx, double& dy)
{
    start_dir_l(w, px, py, w.sigma == 0 ? len2(px - w.sx, py - w.sy) : 1.0, dx, dy);
}

// Where b lies relative to xC, the crossing of the edge line by the ray from the pseudo-source through the opposite
// vertex C = (cx, cy): the sign of (b - xC), scaled by DC = cy - sy when DC > 0 (no division).
struct CrossC {
    double DC, nC, xC;
    bool pos;
    __device__ __forceinline__ CrossC(const Win& w, double cx, double cy)
    {
        DC = cy - w.sy;
        nC = w.sx * DC + (cx - w.sx) * (-w.sy);  // xC * DC
        pos = DC > 0;
        xC = pos ? 0.0 : nC / DC;
    }
    __device__ __forceinline__ double rel(double b) const { return pos ? b * DC - nC : b - xC; }
};

// The child of window w that leaves its face through one of the two other edges, expressed in the frame of that
// edge's twin: exitBC = false, edge C->A (flag: the interval reaches past C); exitBC = true, edge B->C (flag: the
// interval starts before C).  The caller has checked that the exit edge has a twin.
__device__ __forceinline__ void make_child(const DevMesh& M, const Win& w, bool exitBC, bool flag, Win& c)
{
    const int g = w.he >> 2, j = w.he & 3;
    const double cx = M.geom[9 * g + 3 * j + 1], cy = M.geom[9 * g + 3 * j + 2];
    c.sigma = w.sigma;
    double ux, uy;
    if (!exitBC) {  // exit through edge C->A (local j+2); child frame: origin A, x toward C
        const int t = M.twin[3 * g + (j + 2) % 3];
        ux = M.exitu[12 * g + 4 * j];
        uy = M.exitu[12 * g + 4 * j + 1];
        const double isx = ux * w.sx + uy * w.sy, isy = -uy * w.sx + ux * w.sy;
        c.he = (t / 3) * 4 + t % 3;
        c.sx = isx;
        c.sy = isy;
        // interval ends: rays from the pseudo-source through (b0, 0) and (b1, 0), in the child frame
        const double X0 = ux * w.b0, D0 = -uy * w.b0 - isy;
        if (flag) {
            c.b0 = isx + (X0 - isx) * (-isy) * rcp_nr(D0);
            c.b1 = M.geom[9 * (t / 3) + 3 * (t % 3)];
        } else {
            const double X1 = ux * w.b1, D1 = -uy * w.b1 - isy;
            const double R = rcp_nr(D0 * D1);
            c.b0 = isx + (X0 - isx) * (-isy) * (R * D1);
            c.b1 = isx + (X1 - isx) * (-isy) * (R * D0);
        }
    } else {  // exit through edge B->C (local j+1); child frame: origin C, x toward B
        const int t = M.twin[3 * g + (j + 1) % 3];
        ux = M.exitu[12 * g + 4 * j + 2];
        uy = M.exitu[12 * g + 4 * j + 3];
        const double rx = w.sx - cx, ry = w.sy - cy;
        const double isx = ux * rx + uy * ry, isy = -uy * rx + ux * ry;
        c.he = (t / 3) * 4 + t % 3;
        c.sx = isx;
        c.sy = isy;
        const double X1 = ux * (w.b1 - cx) + uy * (-cy), D1 = -uy * (w.b1 - cx) + ux * (-cy) - isy;
        if (flag) {
            c.b0 = 0.0;
            c.b1 = isx + (X1 - isx) * (-isy) * rcp_nr(D1);
        } else {
            const double X0 = ux * (w.b0 - cx) + uy * (-cy), D0 = -uy * (w.b0 - cx) + ux * (-cy) - isy;
            const double R = rcp_nr(D0 * D1);
            c.b0 = isx + (X0 - isx) * (-isy) * (R * D1);
            c.b1 = isx + (X1 - isx) * (-isy) * (R * D0);
        }
    }
    if (w.sigma == 0) {
        c.c = w.c * ux - w.s * uy;
        c.s = w.s * ux + w.c * uy;
    } else {
        c.c = w.c;
        c.s = w.s;
    }
}

__device__ __forceinline__ void load_pt(const DevMesh& M, int f, const double* b, double* out)
{
    const double* p0 = &M.V[3 * M.F[3 * f]];
    const double* p1 = &M.V[3 * M.F[3 * f + 1]];
    const double* p2 = &M.V[3 * M.F[3 * f + 2]];
    const double s = b[0] + b[1] + b[2];
    for (int c = 0; c < 3; ++c) {
        const double x = b[0] * p0[c] + b[1] * p1[c] + b[2] * p2[c];
        out[c] = s == 1.0 ? x : x / s;  // normalised weights usually sum to exactly 1: skip the FP64 division
    }
}


}  // namespace
