// Exact geodesic distances + start tangents + pair forces with one source per lane.
//
// The same per-source work as the source-group kernel (geodesic.cu): the reference's per-source loop of
// simpleModel::findNeighbors (src/models/simpleModel.cpp:68-112) with the patch of
// submesher::constructSubmeshFromSourceAndTargets (src/utility/submesher.cpp:55-147), the exact window propagation of
// window.cuh in place of CGAL's Surface_mesh_shortest_path (triangulatedMeshSpace.cpp:155-238, path tangents as in
// meshUtilities.cpp:360-380) and the force sum of force::computeForces (src/forces/baseForce.cpp:12-28).
//
// Why one source per lane: on GB300 an FP64 warp instruction occupies its sub-partition's FP64 pipe for the same
// ~64 cycles whether 1 or 32 lanes are active.  Small patches (tens of faces, a few dozen windows per source) give a
// source group only a handful of windows at a time, so most FP64 instructions there run with a few lanes.  Here each
// lane solves its own source serially, in the order of a bucket queue (Dial's algorithm on the windows' FP32 lower
// bounds), and every FP64 instruction of the window step serves up to 32 sources at once.  Lanes take new sources in
// bulk as old ones finish (lane_kernel).  Every data-dependent loop (hash probes, list walks, the bucket scan) has one
// exit and re-converges the lanes that entered it, so a warp's lanes stay one instruction stream.
//
// Memory: each lane has its own tables in global memory (L2- and L1-resident at these sizes), interleaved by lane
// (element k of lane l at [k * 32 + l]) so that the lanes' accesses to the same element coalesce:
//   targets (96 B records), face table (patch membership + per-face target lists), vertex table (dense keys; labels,
//   start directions, launch state and queue links in 40 B records), a window slab with a free list (64 B records),
//   the bucket heads and a breadth-first queue for the patch.  Tables are cleared at the start of every source
//   (coalesced stores).
// A source whose tables or work cap overflow is handed to the medium-table source-group pass (failList), so
// results never depend on the capacities chosen here.
#include <algorithm>
#include <cstring>

#include "cssg_internal.cuh"
#include "window.cuh"

namespace {

constexpr int kW = 32;        // lanes of a warp (interleave stride)
constexpr int kBuckets = 32;  // bucket queue: key range [0, reach] in 32 bands, the last one open-ended
constexpr int kNotQueued = -2;

// element k of this lane's array
template <class T>
struct LaneArr {
    T* p;
    __device__ __forceinline__ T& operator[](int k) const { return p[(size_t)k * kW]; }
};

struct TRec {         // a target (candidate pair) of the lane's source
    double b[3];      // barycentric weights on its face
    double P[3];      // R3 position
    double best;      // shortest path through a processed window so far
    double dx, dy;    // start direction of that path (source frame)
    int face;
    int idx;          // output index (distance API) or particle index j; -(j + 1): screened out (not queried)
    int next;         // next target on the same face (-1: none)
    int pad;
};

struct VRec {         // a vertex of the lane's table (its key, the vertex index, is in a separate dense array)
    double lab;       // best known path length
    double dx, dy;    // start direction of that path
    double launched;  // label of its last pseudo-source launch (-1: never)
    int qnext;        // next item of its bucket list; kNotQueued: not queued
    int pad;          // can it become a pseudo-source: -1 not evaluated yet, 0 no, 1 yes
};

struct FRec {         // a face of the lane's table
    int key;          // face index, -1: empty entry
    int val;          // bit 30: in the domain (patch); low 30 bits: first target on the face + 1 (0: none)
};

constexpr int kInDomain = 1 << 30;

struct LaneSlot {
    LaneArr<TRec> T;
    LaneArr<double> te;  // 3 per target: end tangents (distance API)
    LaneArr<FRec> F;
    LaneArr<int> bfs;
    LaneArr<int> vkey;  // vertex index of each vertex-table entry, -1: empty
    LaneArr<VRec> V;
    LaneArr<Win> W;
    LaneArr<int> wnext;
    LaneArr<int> wfree;
    LaneArr<int> bucket;
};

__host__ __device__ inline size_t lane_align(size_t x) { return (x + 255) & ~(size_t)255; }

// byte offsets of the arrays in one warp's scratch (each array holds cap x 32 elements)
__host__ __device__ inline size_t lane_carve(const LaneCaps& c, char* base, int lane, LaneSlot* S)
{
    size_t o = 0;
#define LCARVE(field, type, count)                                        \
    if (S) S->field.p = (type*)(base + o) + lane;                         \
    o = lane_align(o + sizeof(type) * (size_t)(count) * kW);
    LCARVE(T, TRec, c.CT);
    LCARVE(te, double, 3 * c.CT);
    LCARVE(F, FRec, c.CF);
    LCARVE(bfs, int, c.CF);
    LCARVE(vkey, int, c.CV);
    LCARVE(V, VRec, c.CV);
    LCARVE(W, Win, c.CW);
    LCARVE(wnext, int, c.CW);
    LCARVE(wfree, int, c.CW);
    LCARVE(bucket, int, kBuckets);
#undef LCARVE
    return o;
}

__device__ __forceinline__ unsigned lhash(int k) { return (unsigned)k * 2654435761u; }

// Lanes that enter a data-dependent loop together (a hash probe, a list walk) leave it at different steps, and nothing
// makes them converge again on their own: the code after the loop would then be issued once per exit step, and with
// nested probes the warp ends up running its lanes one after another.  Functions with such loops therefore have one
// exit and re-converge the lanes that entered them before returning.
#define LANES_ENTER const unsigned lanesIn = __activemask()
#define LANES_LEAVE __syncwarp(lanesIn)
// The same for one iteration of a loop whose body branches: the lanes that start an iteration together finish it
// together (loop bodies have no `continue`, so every lane that starts an iteration reaches its end).
#define ITER_BEGIN const unsigned iterLanes = __activemask()
#define ITER_END __syncwarp(iterLanes)

// Per-lane solver state (registers).
struct Lane {
    int si;           // source index
    int f0;
    bool full;        // whole mesh (no patch)
    bool wantTe;
    double S[3], e1[3], e2[3];
    double cutoff;
    int nT;
    int err;
    int freeTop, wTop;  // free list depth, slab high-water mark
    int cur;            // current bucket
    float invBw;        // buckets per unit key
    float bw;           // bucket width
    int processed, launches, pops;
    long long popCap;
    double b0[3];       // the source's barycentric weights
    double rmax;        // patch radius
    bool handedOff;     // passed to the medium-table source-group pass
};

struct LaneCtx {
    const DevMesh& M;
    const LaneCaps& C;
    LaneSlot& S;
    Lane& st;
};

// ---- face table --------------------------------------------------------------------------------------------------
__device__ int lf_find(const LaneCtx& x, int f)
{
    LANES_ENTER;
    const int CF = x.C.CF;
    unsigned h = lhash(f) & (CF - 1);
    int found = -1;
    for (int p = 0; p < CF; ++p) {
        const int k = x.S.F[h].key;
        if (k == f) found = (int)h;
        if (k == f || k == -1) break;
        h = (h + 1) & (CF - 1);
    }
    LANES_LEAVE;
    return found;
}

// returns the entry of f (inserted if absent); *fresh = 1 when inserted here
__device__ int lf_insert(const LaneCtx& x, int f, bool* fresh)
{
    LANES_ENTER;
    const int CF = x.C.CF;
    *fresh = false;
    unsigned h = lhash(f) & (CF - 1);
    int found = -1;
    for (int p = 0; p < CF; ++p) {
        const int k = x.S.F[h].key;
        if (k == -1) {
            x.S.F[h].key = f;
            x.S.F[h].val = 0;
            *fresh = true;
        }
        if (k == f || k == -1) {
            found = (int)h;
            break;
        }
        h = (h + 1) & (CF - 1);
    }
    if (found < 0) x.st.err = CSSG_ST_CAPACITY;
    LANES_LEAVE;
    return found;
}

__device__ __forceinline__ bool lane_in_domain(const LaneCtx& x, int g)
{
    LANES_ENTER;
    bool in = g >= 0 && x.st.full;
    if (g >= 0 && !x.st.full) {
        const int h = lf_find(x, g);
        in = h >= 0 && (x.S.F[h].val & kInDomain);
    }
    LANES_LEAVE;
    return in;
}

// ---- vertex table ------------------------------------------------------------------------------------------------
__device__ int lv_find(const LaneCtx& x, int v)
{
    LANES_ENTER;
    const int CV = x.C.CV;
    unsigned h = lhash(v) & (CV - 1);
    int found = -1;
    for (int p = 0; p < CV; ++p) {
        const int k = x.S.vkey[h];
        if (k == v) found = (int)h;
        if (k == v || k == -1) break;
        h = (h + 1) & (CV - 1);
    }
    LANES_LEAVE;
    return found;
}

__device__ int lv_insert(const LaneCtx& x, int v)
{
    LANES_ENTER;
    const int CV = x.C.CV;
    unsigned h = lhash(v) & (CV - 1);
    int found = -1;
    for (int p = 0; p < CV; ++p) {
        const int k = x.S.vkey[h];
        if (k == -1) {
            x.S.vkey[h] = v;
            VRec& r = x.S.V[h];
            r.lab = CUDART_INF;
            r.launched = -1.0;
            r.qnext = kNotQueued;
            r.pad = -1;  // launchable: not evaluated yet
        }
        if (k == v || k == -1) {
            found = (int)h;
            break;
        }
        h = (h + 1) & (CV - 1);
    }
    if (found < 0) x.st.err = CSSG_ST_CAPACITY;
    LANES_LEAVE;
    return found;
}

__device__ __forceinline__ double lv_label(const LaneCtx& x, int v)
{
    const int h = lv_find(x, v);
    return h < 0 ? CUDART_INF : x.S.V[h].lab;
}

// ---- bucket queue: items are window slots (< CW) or vertex entries (CW + entry) ------------------------------------
__device__ __forceinline__ int bucket_of(const Lane& st, float key)
{
    const float q = key * st.invBw;
    int b = q >= (float)kBuckets ? kBuckets - 1 : (int)q;
    return max(b, st.cur);
}

__device__ __forceinline__ void queue_window(const LaneCtx& x, int slot, float key)
{
    const int b = bucket_of(x.st, key);
    x.S.wnext[slot] = x.S.bucket[b];
    x.S.bucket[b] = slot;
}

__device__ __forceinline__ void queue_vertex(const LaneCtx& x, int h, double d)
{
    VRec& r = x.S.V[h];
    if (r.qnext != kNotQueued) return;  // already queued (it is launched with its label when popped)
    const int b = bucket_of(x.st, __double2float_rd(d));
    r.qnext = x.S.bucket[b];
    x.S.bucket[b] = x.C.CW + h;
}

__device__ __forceinline__ int alloc_slot(const LaneCtx& x)
{
    Lane& st = x.st;
    if (st.freeTop > 0) return x.S.wfree[--st.freeTop];
    if (st.wTop < x.C.CW) return st.wTop++;
    st.err = CSSG_ST_CAPACITY;
    return -1;
}

__device__ __forceinline__ void free_slot(const LaneCtx& x, int s) { x.S.wfree[x.st.freeTop++] = s; }

// Queue a new window (a child, or a launch's opposite-edge window) unless it leaves the domain, is empty or starts
// beyond the cutoff.  reuse >= 0: the slot to write it to (the processed parent's).  Returns true if a slot was used.
__device__ bool lane_push(const LaneCtx& x, Win& c, int reuse)
{
    LANES_ENTER;
    const DevMesh& M = x.M;
    const int g = c.he >> 2, j = c.he & 3;
    bool used = false;
    if (g != x.st.f0 && lane_in_domain(x, g)) {
        const double L = M.geom[9 * g + 3 * j];
        c.b0 = fmax(0.0, c.b0);
        c.b1 = fmin(L, c.b1);
        const float key = key_lo(c);
        if (c.b1 - c.b0 > 1e-14 * L && (double)key <= x.st.cutoff) {
            c.key = key;
            const int s = reuse >= 0 ? reuse : alloc_slot(x);
            if (s >= 0) {
                x.S.W[s] = c;
                queue_window(x, s, key);
                used = true;
            }
        }
    }
    LANES_LEAVE;
    return used;
}

// can vertex v (entry h) become a pseudo-source: a saddle or border vertex of the mesh, or (patch) a vertex on the
// patch's border; evaluated once per source and kept in the entry (the domain does not change during propagation)
__device__ bool lane_launchable(const LaneCtx& x, int h, int v)
{
    LANES_ENTER;
    const DevMesh& M = x.M;
    VRec& r = x.S.V[h];
    if (r.pad < 0) {
        bool yes = (M.vflag[v] & (VF_BORDER | VF_SADDLE)) != 0;
        if (!yes && !x.st.full)
            for (int i = M.vfStart[v]; i < M.vfStart[v + 1]; ++i)
                if (!lane_in_domain(x, M.vfList[i])) {
                    yes = true;
                    break;
                }
        r.pad = yes ? 1 : 0;
    }
    const bool yes = r.pad == 1;
    LANES_LEAVE;
    return yes;
}

// a path of length d with start direction (dx, dy) to vertex v
__device__ void lane_propose(const LaneCtx& x, int v, double d, double dx, double dy)
{
    LANES_ENTER;
    const int h = lv_insert(x, v);
    if (h >= 0 && d < x.S.V[h].lab) {
        VRec& r = x.S.V[h];
        r.lab = d;
        r.dx = dx;
        r.dy = dy;
        if (d <= x.st.cutoff && lane_launchable(x, h, v)) queue_vertex(x, h, d);
    }
    LANES_LEAVE;
}

// a window's proposal for its face's vertex at (px, py) of its frame; the start direction only when it wins
__device__ void lane_propose_from(const LaneCtx& x, const Win& w, int v, double px, double py)
{
    LANES_ENTER;
    const int h = lv_insert(x, v);
    const double l = len2(px - w.sx, py - w.sy);
    const double d = w.sigma + l;
    if (h >= 0 && d < x.S.V[h].lab) {
        VRec& r = x.S.V[h];
        r.lab = d;
        double dx, dy;
        start_dir_l(w, px, py, l, dx, dy);
        r.dx = dx;
        r.dy = dy;
        if (d <= x.st.cutoff && lane_launchable(x, h, v)) queue_vertex(x, h, d);
    }
    LANES_LEAVE;
}

// ---- one window, in stages (the kernel reconverges the warp between stages) ------------------------------------------
// The window's frame on its face.
struct WinGeo {
    int g, j;
    double L, cx, cy, tol;
};

__device__ __forceinline__ WinGeo win_geo(const DevMesh& M, const Win& w)
{
    WinGeo q;
    q.g = w.he >> 2;
    q.j = w.he & 3;
    q.L = M.geom[9 * q.g + 3 * q.j];
    q.cx = M.geom[9 * q.g + 3 * q.j + 1];
    q.cy = M.geom[9 * q.g + 3 * q.j + 2];
    q.tol = 1e-12 * q.L;
    return q;
}

// Stage 1: load and trim the window in slot s; a dominated window frees its slot.  Returns true if it survives.
__device__ bool lane_trim(const LaneCtx& x, int s, Win& w)
{
    LANES_ENTER;
    const DevMesh& M = x.M;
    w = x.S.W[s];
    // the three labels first (each probe re-converges), then the trim arithmetic on all lanes together
    const int g = w.he >> 2, j = w.he & 3;
    const int A = M.F[3 * g + j], B = M.F[3 * g + (j + 1) % 3];
    const double dA = lv_label(x, A), dB = lv_label(x, B), dC = lv_label(x, M.F[3 * g + (j + 2) % 3]);
    __syncwarp(lanesIn);
    const bool keep = trim_window(M, w, [&](int v) { return v == A ? dA : (v == B ? dB : dC); });
    __syncwarp(lanesIn);
    if (keep) x.st.processed++;
    else free_slot(x, s);
    LANES_LEAVE;
    return keep;
}

// Stage 2: targets on the window's face: the path through this window
__device__ void lane_targets(const LaneCtx& x, const Win& w)
{
    LANES_ENTER;
    const DevMesh& M = x.M;
    const WinGeo q = win_geo(M, w);
    const int fh = lf_find(x, q.g);
    const int head = fh >= 0 ? (x.S.F[fh].val & (kInDomain - 1)) - 1 : -1;
    for (int t = head; t >= 0; t = x.S.T[t].next) {
        ITER_BEGIN;
        TRec& tr = x.S.T[t];
        const double b1 = tr.b[(q.j + 1) % 3], b2 = tr.b[(q.j + 2) % 3];
        const double px = b1 * q.L + b2 * q.cx, py = b2 * q.cy;
        const double l = len2(px - w.sx, py - w.sy);
        const double d = w.sigma + l;
        // screened-out targets (idx < 0) are not queried
        if (tr.idx >= 0 && ray_hits(w, px, py, q.tol) && d < tr.best) {
            tr.best = d;
            double dx, dy;
            start_dir_l(w, px, py, l, dx, dy);
            tr.dx = dx;
            tr.dy = dy;
            if (x.st.wantTe) {
                // direction of arrival in R3: the ray in g's edge frame
                const double* PA = &M.V[3 * M.F[3 * q.g + q.j]];
                const double* PB = &M.V[3 * M.F[3 * q.g + (q.j + 1) % 3]];
                const double* PC = &M.V[3 * M.F[3 * q.g + (q.j + 2) % 3]];
                const double ux = px - w.sx, uy = py - w.sy;
                for (int c = 0; c < 3; ++c) {
                    const double ex = (PB[c] - PA[c]) / q.L;
                    const double ey = (PC[c] - PA[c] - q.cx * ex) / q.cy;
                    x.S.te[3 * t + c] = (ux * ex + uy * ey) / l;
                }
            }
        }
        ITER_END;
    }
    LANES_LEAVE;
}

// Stage 3: vertex proposals: the opposite vertex C when the window's rays reach it, the edge's ends when it covers
// them.  k selects one of the three (the kernel runs them as three sub-stages).
__device__ void lane_proposal(const LaneCtx& x, const Win& w, int k)
{
    LANES_ENTER;
    const DevMesh& M = x.M;
    const WinGeo q = win_geo(M, w);
    if (k == 0) {
        const CrossC xc(w, q.cx, q.cy);
        if (xc.rel(w.b0 - q.tol) <= 0 && xc.rel(w.b1 + q.tol) >= 0)
            lane_propose_from(x, w, M.F[3 * q.g + (q.j + 2) % 3], q.cx, q.cy);
    } else if (k == 1) {
        if (w.b0 <= q.tol) lane_propose_from(x, w, M.F[3 * q.g + q.j], 0.0, 0.0);
    } else {
        if (w.b1 >= q.L - q.tol) lane_propose_from(x, w, M.F[3 * q.g + (q.j + 1) % 3], q.L, 0.0);
    }
    LANES_LEAVE;
}

// Stage 4: the child through exit edge C->A (exitBC = false) or B->C (true); *reuse is the processed window's slot
// while it is free to hold a child (-1 once used).  After the last child the caller frees an unused slot.
__device__ void lane_child(const LaneCtx& x, const Win& w, bool exitBC, int* reuse)
{
    LANES_ENTER;
    const DevMesh& M = x.M;
    const WinGeo q = win_geo(M, w);
    const CrossC xc(w, q.cx, q.cy);
    const double r0 = xc.rel(w.b0), r1 = xc.rel(w.b1);
    const bool want = exitBC ? (r1 > 0 && M.twin[3 * q.g + (q.j + 1) % 3] >= 0)
                             : (r0 < 0 && M.twin[3 * q.g + (q.j + 2) % 3] >= 0);
    if (want) {
        const unsigned lanesWant = __activemask();
        Win c;
        make_child(M, w, exitBC, exitBC ? r0 <= 0 : r1 >= 0, c);
        __syncwarp(lanesWant);
        if (lane_push(x, c, *reuse)) *reuse = -1;
    }
    LANES_LEAVE;
}

// ---- one pseudo-source launch ----------------------------------------------------------------------------------------
__device__ void lane_launch(const LaneCtx& x, int h)
{
    LANES_ENTER;
    const DevMesh& M = x.M;
    VRec& r = x.S.V[h];
    r.qnext = kNotQueued;
    const double d = r.lab;
    if (d != r.launched) {  // not yet launched with this label
        r.launched = d;
        x.st.launches++;
        const int v = x.S.vkey[h];
        const double tx = r.dx, ty = r.dy;
        for (int i = M.vfStart[v]; i < M.vfStart[v + 1]; ++i) {
            ITER_BEGIN;
            const int f = M.vfList[i];
            if (lane_in_domain(x, f)) {
                int k = 0;
                while (M.F[3 * f + k] != v) ++k;
                const int e = (k + 1) % 3;
                // edge paths to the face's two other vertices, then the window on the opposite edge
                lane_propose(x, M.F[3 * f + e], d + M.geom[9 * f + 3 * k], tx, ty);
                lane_propose(x, M.F[3 * f + (k + 2) % 3], d + M.geom[9 * f + 3 * ((k + 2) % 3)], tx, ty);
                const int t = M.twin[3 * f + e];
                if (t >= 0) {
                    Win c;
                    c.he = (t / 3) * 4 + t % 3;
                    c.sigma = d;
                    const double L = M.geom[9 * f + 3 * e];
                    c.sx = L - M.geom[9 * f + 3 * e + 1];
                    c.sy = -M.geom[9 * f + 3 * e + 2];
                    c.b0 = 0;
                    c.b1 = L;
                    c.c = tx;
                    c.s = ty;
                    lane_push(x, c, -1);
                }
            }
            ITER_END;
        }
    }
    LANES_LEAVE;
}

// Early exit: every queried target's best known path (through a window or a labelled vertex of its face) is no
// longer than `bound`, a lower bound of every queued item's distances.  The vertex paths are FP32 upper bounds.
__device__ bool lane_settled(const LaneCtx& x, double bound)
{
    LANES_ENTER;
    const DevMesh& M = x.M;
    bool done = true;
    for (int t = 0; t < x.st.nT && done; ++t) {
        ITER_BEGIN;
        const TRec& tr = x.S.T[t];
        if (tr.face != x.st.f0 && tr.idx >= 0) {  // targets on the source face and screened-out ones do not count
            double b = tr.best;
            for (int c = 0; c < 3; ++c) {
                const int v = M.F[3 * tr.face + c];
                const double lab = lv_label(x, v);
                const double* pv = &M.V[3 * v];
                const float ux = (float)(tr.P[0] - pv[0]), uy = (float)(tr.P[1] - pv[1]), uz = (float)(tr.P[2] - pv[2]);
                const float l = sqrtf(ux * ux + uy * uy + uz * uz) * 1.000001f + 1e-30f;
                if (lab < CUDART_INF) b = fmin(b, lab + (double)l);
            }
            if (!(b <= bound)) done = false;
        }
        ITER_END;
    }
    LANES_LEAVE;
    return done;
}

// next item in key order, or -1 when the source is done
__device__ int lane_pop(const LaneCtx& x)
{
    LANES_ENTER;
    Lane& st = x.st;
    int item = -1;
    while (st.cur < kBuckets) {
        const int h = x.S.bucket[st.cur];
        if (h >= 0) {
            x.S.bucket[st.cur] = h < x.C.CW ? x.S.wnext[h] : x.S.V[h - x.C.CW].qnext;
            item = h;
            break;
        }
        ++st.cur;
        // every queued key is >= cur * bw up to the float rounding of the bucket index
        if (st.cur < kBuckets && lane_settled(x, (double)st.cur * (double)st.bw * (1.0 - 1e-5))) st.cur = kBuckets;
    }
    LANES_LEAVE;
    return item;
}

// ---- the per-source solve: set-up, propagation steps, results ----------------------------------------------------
// Targets, patch, source frame and the initial windows.  Returns true when the source has propagation to do.
__device__ bool lane_setup_body(const GeoLaunch& Lp, const LaneCaps& C, LaneSlot& S, Lane& st)
{
    const int si = st.si;
    const SysDesc& D = Lp.sys[Lp.sysOf ? Lp.sysOf[si] : 0];
    const DevMesh& M = D.mesh;
    LaneCtx x{M, C, S, st};
    st.err = 0;
    st.processed = st.launches = st.pops = 0;
    st.freeTop = st.wTop = 0;
    st.cur = 0;
    st.nT = 0;
    st.handedOff = false;
    st.f0 = Lp.srcFace[si];
    st.cutoff = D.cutoff;
    st.full = !D.submesh;
    st.wantTe = D.searchMode == 0 && Lp.teOut != nullptr;
    st.popCap = 4LL * Lp.maxWindows + 1024;
    if (D.bigBin && Lp.routeBig && Lp.failList) {
        st.handedOff = true;
        return false;
    }
    double* b0 = st.b0;
    for (int c = 0; c < 3; ++c) b0[c] = Lp.srcBary[3 * si + c];
    load_pt(M, st.f0, b0, st.S);
    // empty tables
    for (int k = 0; k < C.CF; ++k) S.F[k].key = -1;
    for (int k = 0; k < C.CV; ++k) S.vkey[k] = -1;
    for (int k = 0; k < kBuckets; ++k) S.bucket[k] = -1;
    // ---- targets --------------------------------------------------------------------------------------------------
    int nT = 0;
    double rmax = D.maxDist;
    if (D.searchMode == 0 || D.searchMode == 3) {
        const int beg = Lp.candOff[si];
        nT = Lp.candOff[si + 1] - beg;
        if (nT > C.CT) {
            st.err = CSSG_ST_CAPACITY;
            nT = 0;
        }
        for (int t = 0; t < nT; ++t) {
            TRec& tr = S.T[t];
            int jj, fidx;
            const double* bb;
            if (D.searchMode == 0) {
                fidx = Lp.candFace[beg + t];
                bb = &Lp.candBary[3 * (beg + t)];
                jj = beg + t;
            } else {
                const int pj = Lp.candJ[beg + t];
                fidx = Lp.partFace[pj];
                bb = &Lp.partBary[3 * pj];
                jj = Lp.candSkip[beg + t] ? -(pj + 1) : pj;
            }
            tr.face = fidx;
            tr.idx = jj;
            for (int c = 0; c < 3; ++c) tr.b[c] = bb[c];
        }
        if (Lp.threshold && Lp.threshold[si] < rmax) rmax = Lp.threshold[si];
        if (D.searchMode == 3 && Lp.pairCount) Lp.pairCount[si] = nT;
    } else {
        // padded candidate rows (cell-list search done by the candidates kernel)
        nT = Lp.rowCount[si];
        if (nT > C.CT || nT > Lp.rowCap) {  // the row was truncated or the targets do not fit: medium pass
            st.err = CSSG_ST_CAPACITY;
            nT = 0;
        }
        for (int t = 0; t < nT; ++t) {
            TRec& tr = S.T[t];
            const int pj = Lp.rowJ[(size_t)si * Lp.rowCap + t];
            tr.face = Lp.partFace[pj];
            tr.idx = pj;
            for (int c = 0; c < 3; ++c) tr.b[c] = Lp.partBary[3 * pj + c];
        }
        if (Lp.rowChord[si] < rmax) rmax = Lp.rowChord[si];
        if (Lp.pairCount) Lp.pairCount[si] = nT;
    }
    st.nT = nT;
    st.rmax = rmax;
    if (st.err == CSSG_ST_CAPACITY && Lp.failList) {
        st.handedOff = true;
        return false;
    }
    if (!isfinite(st.S[0] + st.S[1] + st.S[2])) st.err = CSSG_ST_NAN;
    if (nT == 0 || st.err) return false;
    for (int t = 0; t < nT; ++t) {
        TRec& tr = S.T[t];
        load_pt(M, tr.face, tr.b, tr.P);
        tr.best = CUDART_INF;
        tr.next = -1;
    }
    // ---- domain: the reference patch (faces with a vertex within rmax of the source, from the source face's
    // neighbours outward; target faces complete it) or the whole mesh ------------------------------------------------
    bool fresh;
    if (D.submesh) {
        const int h0 = lf_insert(x, st.f0, &fresh);
        if (h0 >= 0) S.F[h0].val |= kInDomain;
        bool notInF0 = false, notInSeeds = false;
        int nb[3];
        for (int k = 0; k < 3; ++k) {
            const int t = M.twin[3 * st.f0 + k];
            nb[k] = t < 0 ? -1 : t / 3;
        }
        for (int t = 0; t < nT; ++t) {
            const int f = S.T[t].face;
            if (f != st.f0) {
                notInF0 = true;
                if (f != nb[0] && f != nb[1] && f != nb[2]) notInSeeds = true;
            }
        }
        if (notInF0) {
            int nq = 0;
            for (int k = 0; k < 3; ++k) {
                if (nb[k] < 0) continue;
                const int h = lf_insert(x, nb[k], &fresh);
                if (h < 0) break;
                S.F[h].val |= kInDomain;
                if (fresh && notInSeeds) S.bfs[nq++] = nb[k];
            }
            if (notInSeeds) {
                const double r2 = rmax * rmax;
                for (int q = 0; q < nq && !st.err; ++q) {
                    ITER_BEGIN;
                    const int f = S.bfs[q];
                    for (int k = 0; k < 3 && !st.err; ++k) {
                        const int tw = M.twin[3 * f + k];
                        const int g = tw < 0 ? -1 : tw / 3;
                        bool add = g >= 0 && lf_find(x, g) < 0;
                        if (add) {
                            bool near = false;
                            for (int c = 0; c < 3; ++c) {
                                const double* pv = &M.V[3 * M.F[3 * g + c]];
                                const double dx = st.S[0] - pv[0], dy = st.S[1] - pv[1], dz = st.S[2] - pv[2];
                                if (!(dx * dx + dy * dy + dz * dz > r2)) near = true;
                            }
                            add = near;
                        }
                        if (add) {
                            const int h = lf_insert(x, g, &fresh);
                            if (h >= 0) {
                                S.F[h].val |= kInDomain;
                                if (nq < C.CF) S.bfs[nq++] = g;
                                else st.err = CSSG_ST_CAPACITY;
                            }
                        }
                    }
                    ITER_END;
                }
            }
        }
    }
    // target lists per face (in patch mode the target faces complete the patch)
    for (int t = nT - 1; t >= 0 && !st.err; --t) {
        const int h = lf_insert(x, S.T[t].face, &fresh);
        if (h < 0) break;
        if (D.submesh) S.F[h].val |= kInDomain;
        S.T[t].next = (S.F[h].val & (kInDomain - 1)) - 1;
        S.F[h].val = (S.F[h].val & kInDomain) | (t + 1);
    }
    // ---- source: frame, face-vertex labels, the three initial windows -------------------------------------------------
    const int f0 = st.f0;
    const double L0 = M.geom[9 * f0], cx0 = M.geom[9 * f0 + 1], cy0 = M.geom[9 * f0 + 2];
    {
        const double* p0 = &M.V[3 * M.F[3 * f0]];
        const double* p1 = &M.V[3 * M.F[3 * f0 + 1]];
        const double* p2 = &M.V[3 * M.F[3 * f0 + 2]];
        for (int c = 0; c < 3; ++c) st.e1[c] = (p1[c] - p0[c]) / L0;
        for (int c = 0; c < 3; ++c) st.e2[c] = (p2[c] - p0[c] - cx0 * st.e1[c]) / cy0;
    }
    // bucket width: the key range is [0, min(cutoff, 2 x patch radius + 2 mean edges)]
    {
        double reach = st.cutoff;
        const double cap = D.submesh ? 2.0 * rmax + 2.0 * D.delta : reach;
        if (!(reach < cap)) reach = cap;
        if (!(reach > 0) || !(reach < 1e300)) reach = 64.0 * (D.delta > 0 ? D.delta : 1.0);
        st.bw = (float)(reach / kBuckets);
        st.invBw = (float)(kBuckets / reach);
    }
    const double P2[3][2] = {{0, 0}, {L0, 0}, {cx0, cy0}};
    const double S2x = b0[1] * L0 + b0[2] * cx0, S2y = b0[2] * cy0;
    for (int k = 0; k < 3 && !st.err; ++k) {
        const int v = M.F[3 * f0 + k];
        const double dx = P2[k][0] - S2x, dy = P2[k][1] - S2y;
        const double l = len2(dx, dy);
        const double* pv = &M.V[3 * v];
        const double u[3] = {pv[0] - st.S[0], pv[1] - st.S[1], pv[2] - st.S[2]};
        lane_propose(x, v, sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]), dx / l, dy / l);
    }
    for (int k = 0; k < 3 && !st.err; ++k) {
        const int t = M.twin[3 * f0 + k];
        if (t < 0) continue;
        const double L = M.geom[9 * f0 + 3 * k];
        const double skx = b0[(k + 1) % 3] * L + b0[(k + 2) % 3] * M.geom[9 * f0 + 3 * k + 1];
        const double sky = b0[(k + 2) % 3] * M.geom[9 * f0 + 3 * k + 2];
        Win w;
        w.he = (t / 3) * 4 + t % 3;
        w.sigma = 0;
        w.sx = L - skx;
        w.sy = fmin(-sky, -1e-15 * L);
        w.b0 = 0;
        w.b1 = L;
        const double ddx = P2[(k + 1) % 3][0] - P2[k][0], ddy = P2[(k + 1) % 3][1] - P2[k][1];
        const double dl = len2(ddx, ddy);
        w.c = -ddx / dl;
        w.s = -ddy / dl;
        lane_push(x, w, -1);
    }
    return !st.err;
}

__device__ bool lane_setup(const GeoLaunch& Lp, const LaneCaps& C, LaneSlot& S, Lane& st)
{
    LANES_ENTER;
    const bool live = lane_setup_body(Lp, C, S, st);
    LANES_LEAVE;
    return live;
}

// The next item of the propagation in key order (-1: the source is done or failed).
__device__ __forceinline__ int lane_next(const GeoLaunch& Lp, const LaneCaps& C, LaneSlot& S, Lane& st)
{
    const SysDesc& D = Lp.sys[Lp.sysOf ? Lp.sysOf[st.si] : 0];
    LaneCtx x{D.mesh, C, S, st};
    const int it = lane_pop(x);
    if (it < 0) return -1;
    if (++st.pops > st.popCap || st.processed > Lp.maxWindows) {
        st.err = CSSG_ST_CAPACITY;
        return -1;
    }
    return it;
}

// Distances, tangents, pair records and the force of the source (or its hand-off to the medium pass).
__device__ void lane_finish_body(const GeoLaunch& Lp, const LaneCaps& C, LaneSlot& S, Lane& st,
                                 unsigned long long* cnt)
{
    const int si = st.si;
    if (st.err == CSSG_ST_CAPACITY && Lp.failList) st.handedOff = true;
    if (st.handedOff) {
        Lp.status[si] = 0;
        Lp.failList[atomicAdd(Lp.failCount, 1)] = si;
        return;
    }
    const SysDesc& D = Lp.sys[Lp.sysOf ? Lp.sysOf[si] : 0];
    const DevMesh& M = D.mesh;
    LaneCtx x{M, C, S, st};
    const int nT = st.nT;
    // ---- results ---------------------------------------------------------------------------------------------------
    const int err = st.err;
    double fx = 0, fy = 0, fz = 0;
    int inRange = 0;
    for (int t = 0; t < nT; ++t) {
        const TRec& tr = S.T[t];
        const bool screened = tr.idx < 0;
        double d = CUDART_INF, ts[3] = {0, 0, 0}, te[3] = {0, 0, 0};
        if (!err && !screened) {
            if (tr.face == st.f0) {
                const double u[3] = {tr.P[0] - st.S[0], tr.P[1] - st.S[1], tr.P[2] - st.S[2]};
                d = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
                if (d > 0)
                    for (int c = 0; c < 3; ++c) ts[c] = te[c] = u[c] / d;
            } else {
                d = tr.best;
                double dx = tr.dx, dy = tr.dy;
                if (st.wantTe && d < CUDART_INF)
                    for (int c = 0; c < 3; ++c) te[c] = S.te[3 * t + c];
                for (int c = 0; c < 3; ++c) {
                    const int v = M.F[3 * tr.face + c];
                    const int h = lv_find(x, v);
                    const double lab = h < 0 ? CUDART_INF : S.V[h].lab;
                    if (!(lab < CUDART_INF)) continue;
                    const double* pv = &M.V[3 * v];
                    const double u[3] = {tr.P[0] - pv[0], tr.P[1] - pv[1], tr.P[2] - pv[2]};
                    const double l = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
                    if (lab + l < d) {
                        d = lab + l;
                        dx = S.V[h].dx;
                        dy = S.V[h].dy;
                        if (st.wantTe)
                            for (int q = 0; q < 3; ++q) te[q] = l > 0 ? u[q] / l : 0;
                    }
                }
                if (d < CUDART_INF)
                    for (int c = 0; c < 3; ++c) ts[c] = dx * st.e1[c] + dy * st.e2[c];
            }
        }
        if (d > st.cutoff) {
            d = CUDART_INF;
            ts[0] = ts[1] = ts[2] = te[0] = te[1] = te[2] = 0;
        }
        if (D.searchMode == 0) {
            const int o = tr.idx;
            if (!(d < CUDART_INF) && Lp.patchDisconnected && !err) {
                d = 2.0 * D.maxDist;
                ts[0] = ts[1] = te[0] = te[1] = 0;
                ts[2] = te[2] = 1;
            }
            Lp.dOut[o] = d;
            if (Lp.tsOut)
                for (int c = 0; c < 3; ++c) Lp.tsOut[3 * o + c] = ts[c];
            if (Lp.teOut)
                for (int c = 0; c < 3; ++c) Lp.teOut[3 * o + c] = te[c];
        } else {
            if (Lp.dOut && t < Lp.pairCap) {
                const size_t o = (size_t)si * Lp.pairCap + t;
                Lp.dOut[o] = d;
                Lp.pairJ[o] = tr.idx;  // -(j + 1) for a screened-out pair
                for (int c = 0; c < 3; ++c) Lp.tsOut[3 * o + c] = ts[c];
            }
            if (d < CUDART_INF) {
                double fm = 0;
                if (D.forceKind == 0) {
                    if (d <= D.sigma) fm = -D.k * (D.sigma - d);
                } else {
                    const double sqrtTwoPi = 2.50662827463100050241576528481104525300698674061;
                    fm = -(d * D.k * exp(-d * d / (2.0 * D.sigma * D.sigma)) / ((sqrtTwoPi * D.sigma) * sqrt(D.sigma)));
                }
                fx += fm * ts[0];
                fy += fm * ts[1];
                fz += fm * ts[2];
                if (d <= D.sigma) inRange++;
            }
        }
    }
    if (Lp.force) {
        Lp.force[3 * si] = fx;
        Lp.force[3 * si + 1] = fy;
        Lp.force[3 * si + 2] = fz;
        if (Lp.kickVel) {  // velocityVerletNVE second half (velocityVerletNVE.cpp:23-29) for this particle
            Lp.kickVel[3 * si] += 0.5 * Lp.kickDt * fx;
            Lp.kickVel[3 * si + 1] += 0.5 * Lp.kickDt * fy;
            Lp.kickVel[3 * si + 2] += 0.5 * Lp.kickDt * fz;
        }
    }
    if (Lp.inRangeOut) Lp.inRangeOut[si] = inRange;
    if (Lp.srcCost) Lp.srcCost[si] = st.processed + st.launches + 1;
    if (Lp.stats) {
        Lp.stats[4 * si] = st.processed;
        Lp.stats[4 * si + 1] = st.launches;
        Lp.stats[4 * si + 2] = 1;
        Lp.stats[4 * si + 3] = nT;
    }
    Lp.status[si] = err;
    if (err && Lp.statusBits) atomicOr(Lp.statusBits, 1 << err);
    cnt[0] += st.processed;
    cnt[1] += st.launches;
    cnt[2] += inRange;
    cnt[3] += err ? 1 : 0;
}

__device__ void lane_finish(const GeoLaunch& Lp, const LaneCaps& C, LaneSlot& S, Lane& st, unsigned long long* cnt)
{
    LANES_ENTER;
    lane_finish_body(Lp, C, S, st, cnt);
    LANES_LEAVE;
}

// A warp keeps up to `lanes` sources in flight, one per lane.  Lanes whose source is done wait until half of them
// are idle (or none is live); then the idle lanes write their sources' results and take the next consecutive sources
// from the work counter together, so set-up and results run on many lanes at once and no lane waits for the slowest
// source of a fixed batch.  The propagation loop is warp-synchronous: every live lane takes one item per iteration,
// and every stage sits at the top level of the loop body and ends with a warp-wide reconvergence, so the lanes' window
// steps issue as shared instructions rather than one lane's path after another's.
__global__ void __launch_bounds__(128) lane_kernel(GeoLaunch L, LaneCaps C, size_t warpBytes, int lanes)
{
    const int lane = threadIdx.x & 31;
    const int warp = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (warp >= L.nSlots) return;
    LaneSlot S;
    lane_carve(C, (char*)L.scratch + (size_t)warp * warpBytes, lane, &S);
    unsigned long long cnt[4] = {0, 0, 0, 0};
    int nItems = L.nSrc;
    if (L.itemCountDev) nItems = min(nItems, *(volatile const int*)L.itemCountDev);
    const int refillAt = max(1, lanes / 2);
    Lane st;
    st.si = 0;
    bool live = false, pending = false, more = true;
    while (true) {
        const bool idle = lane < lanes && !live;
        const unsigned idleMask = __ballot_sync(0xffffffffu, idle);
        const int nLive = __popc(__ballot_sync(0xffffffffu, live));
        if (!more && nLive == 0) break;
        if (more && (nLive == 0 || __popc(idleMask) >= refillAt)) {
            if (idle && pending) {
                lane_finish(L, C, S, st, cnt);
                pending = false;
            }
            __syncwarp();
            const int want = __popc(idleMask);
            int base = 0;
            if (lane == 0) base = atomicAdd(L.workCounter, want);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base + want >= nItems) more = false;
            if (idle) {
                const int item = base + __popc(idleMask & ((1u << lane) - 1));
                if (item < nItems) {
                    st.si = L.order ? L.order[item] : item;
                    live = lane_setup(L, C, S, st);
                    pending = true;
                }
            }
            __syncwarp();
            continue;
        }
        const DevMesh& M = L.sys[L.sysOf ? L.sysOf[st.si] : 0].mesh;
        const LaneCtx x{M, C, S, st};
        int it = -1;
        if (live) {
            it = lane_next(L, C, S, st);
            if (it < 0) live = false;
        }
        __syncwarp();
        const bool isWin = live && it < C.CW, isVtx = live && it >= C.CW;
        Win w;
        bool on = false;
        if (isWin) on = lane_trim(x, it, w);
        __syncwarp();
        if (on) lane_targets(x, w);
        __syncwarp();
        for (int k = 0; k < 3; ++k) {
            if (on) lane_proposal(x, w, k);
            __syncwarp();
        }
        int reuse = on ? it : -1;
        if (on) lane_child(x, w, false, &reuse);
        __syncwarp();
        if (on) lane_child(x, w, true, &reuse);
        __syncwarp();
        if (on && reuse >= 0) free_slot(x, reuse);
        if (isVtx) lane_launch(x, it - C.CW);
        __syncwarp();
        if (live && st.err) live = false;
    }
    if (pending) lane_finish(L, C, S, st, cnt);
    __syncwarp();
    for (int k = 0; k < 4; ++k) {
        unsigned long long v = cnt[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0 && v && L.counters) atomicAdd(&L.counters[k], v);
    }
}

}  // namespace

size_t cssg_lane_warp_bytes(const LaneCaps& c) { return lane_align(lane_carve(c, nullptr, 0, nullptr)); }

void cssg_launch_lanes(const GeoLaunch& L, const LaneCaps& C, int lanes, cudaStream_t s)
{
    if (L.nSrc <= 0 || L.nSlots <= 0) return;
    const size_t warpBytes = cssg_lane_warp_bytes(C);
    const int threads = 128;
    const int blocks = (L.nSlots * 32 + threads - 1) / threads;
    lane_kernel<<<blocks, threads, 0, s>>>(L, C, warpBytes, lanes == 16 ? 16 : 32);
}
