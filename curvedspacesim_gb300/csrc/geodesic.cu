// Exact geodesic distances + start tangents + pair forces: one source group (1, 2, 4 or 8 warps) per source
// particle, persistent groups.
//
// Replaces, per timestep, the reference's per-source loop in simpleModel::findNeighbors
// (src/models/simpleModel.cpp:68-112): candidate search (cellListNeighborStructure::constructCandidateNeighborList,
// src/utility/cellListNeighborStructure.cpp:45-84, or the all-to-all baseNeighborStructure), the patch
// (submesher::constructSubmeshFromSourceAndTargets, src/utility/submesher.cpp:55-147), the CGAL
// Surface_mesh_shortest_path solve and path tangents (triangulatedMeshSpace.cpp:155-238,
// meshUtilities.cpp:360-380) and the force sum of force::computeForces (src/forces/baseForce.cpp:12-28) with
// harmonicRepulsion / gaussianRepulsion::pairwiseForce.
//
// Geodesics: the exact window propagation of window.cuh.  Saddle vertices (angle sum > 2 pi) and border vertices of
// the domain become pseudo-sources when their label improves; windows never re-enter the source face (the chord
// inside it is optimal).
// Order: distance-banded rounds.  A round processes every window and pseudo-source launch whose key (a lower bound of
// its distances) lies within a band above the smallest queued key, including those created inside the band, then
// moves to the next band.  The threads of a group process batches of windows in parallel; vertex labels are
// updated with 64-bit atomicMin on the bit patterns of non-negative doubles and the start direction of a label is
// written, after a group barrier, by the thread whose proposal survived.  Processing order only affects how much
// gets pruned, not the result.
//
// Where each source's force is written, the kernel can also apply the velocity-Verlet second half kick of that
// particle (velocityVerletNVE.cpp:23-29) and records final per-source failures in the system's status bits, so an
// NVE step needs no separate integrator or status launches.
//
// Roofline: this kernel is bound by the FP64 pipe and latency (scalar double arithmetic on irregular,
// data-dependent work); its per-source footprint is a few KB of scratch plus mesh reads, mostly L2-resident.
#include <math_constants.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "cssg_internal.cuh"
#include "window.cuh"

namespace {

// loads of table entries other lanes may be writing (shared-memory tables: plain volatile loads)
__device__ __forceinline__ int ldv(const int* p) { return *(const volatile int*)p; }
__device__ __forceinline__ unsigned long long ldv(const unsigned long long* p)
{
    return *(const volatile unsigned long long*)p;
}

struct WarpCtl {
    int nA, nB, nLA, nLB, nLog, nV, nF, nT, err, nBA, nBB, nProc;
    int nPT, nCT;       // task counts of the current batch of windows
    int qHead, qTail;   // band queue: a ring over S.wA (absolute counts; slot = count % CW)
    double thr;         // upper edge of the current distance band (-inf outside the rounds)
    double maxChord2;   // largest squared chord to a candidate (cell / all-to-all search)
    int item;           // the work item the group is on
};

// Task lists of one batch of up to 32 windows (per warp, shared memory): vertex proposals (window << 2 | vertex:
// 0 opposite vertex C, 1 = A, 2 = B) and child windows (window << 1 | exit: 0 through edge C->A, 1 through B->C).
constexpr int kTaskP = 96, kTaskC = 64;

struct Slot {
    int* taskP;  // shared memory, kTaskP entries
    int* taskC;  // shared memory, kTaskC entries
    int* tface;
    int* tidx;
    int* tnext;
    double* tb;
    double* tp;
    unsigned long long* tbest;
    int* vkey;
    unsigned long long* vlab;
    double* vtx;
    double* vty;
    unsigned long long* vtok;
    unsigned long long* vlaunched;  // label bits a vertex was last launched with
    signed char* vcan;              // can the vertex become a pseudo-source: -1 not evaluated yet, 0 no, 1 yes
    int* vlist;
    int* fkey;
    int* fhead;
    int* flist;
    Win* wA;
    Win* wB;
    Win* wlog;
    int* lognext;  // per log entry: next entry of the same face
    int* flog;     // per face-table slot: first log entry of that face
    int* lA;
    int* lB;
    double* ld;  // per launch entry: label, start direction (x, y) it launched with
    int* lpre;   // per launch entry: exclusive prefix of the launched vertices' face counts
    int* bA;
    int* bB;
};

__host__ __device__ inline size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

__host__ __device__ inline size_t carve(const GeoCaps& c, char* base, Slot* S)
{
    size_t o = 0;
#define CARVE(field, type, count)                                  \
    if (S) S->field = (type*)(base + o);                           \
    o = align_up(o + sizeof(type) * (size_t)(count));
    CARVE(tface, int, c.CT);
    CARVE(tidx, int, c.CT);
    CARVE(tnext, int, c.CT);
    CARVE(tb, double, 3 * c.CT);
    CARVE(tp, double, 3 * c.CT);
    CARVE(tbest, unsigned long long, c.CT);
    CARVE(vkey, int, c.CV);
    CARVE(vlab, unsigned long long, c.CV);
    CARVE(fkey, int, c.CF);
    CARVE(fhead, int, c.CF);
    CARVE(vtx, double, c.CV);
    CARVE(vty, double, c.CV);
    CARVE(vtok, unsigned long long, c.CV);
    CARVE(vlaunched, unsigned long long, c.CV);
    CARVE(vcan, signed char, c.CV);
    CARVE(vlist, int, c.CV);
    CARVE(flist, int, c.CF);
    CARVE(wA, Win, c.CW);
    CARVE(wB, Win, c.CW);
    CARVE(wlog, Win, c.CLOG);
    CARVE(lognext, int, c.CLOG);
    CARVE(flog, int, c.CF);
    CARVE(lA, int, c.CL);
    CARVE(lB, int, c.CL);
    CARVE(ld, double, 3 * c.CL);
    CARVE(lpre, int, c.CL + 1);
    CARVE(bA, int, c.CF);
    CARVE(bB, int, c.CF);
#undef CARVE
    return o;
}

// the probed hash tables live in shared memory when they fit (else in the global slot): vertex labels (key, label
// bits, launchability) and faces (key, target-list head)
__host__ __device__ inline size_t smem_per_warp(const GeoCaps& c)
{
    return (size_t)c.CV * 8 + (size_t)c.CV * 4 + (size_t)c.CF * 8 + (size_t)c.CV;
}

__device__ inline void carve_smem(const GeoCaps& c, char* base, Slot* S)
{
    S->vlab = (unsigned long long*)base;
    S->vkey = (int*)(base + (size_t)c.CV * 8);
    S->fkey = (int*)(base + (size_t)c.CV * 12);
    S->fhead = (int*)(base + (size_t)c.CV * 12 + (size_t)c.CF * 4);
    S->vcan = (signed char*)(base + (size_t)c.CV * 12 + (size_t)c.CF * 8);
}

__device__ __forceinline__ unsigned hash_int(int k) { return (unsigned)k * 2654435761u; }

// ---- hash tables ----------------------------------------------------------------------------------------------
// CSSG_GEO_OUTLINE (geodesic_outlined.cu) compiles the probes out of line: one copy of each instead of one per call
// site, a smaller kernel with fewer instruction-cache misses where sources are small and every phase is hot.
#ifdef CSSG_GEO_OUTLINE
#define CSSG_PROBE __noinline__
#else
#define CSSG_PROBE
#endif
__device__ CSSG_PROBE int vfind(const Slot& S, int CV, int v)
{
    unsigned h = hash_int(v) & (CV - 1);
    for (int p = 0; p < CV; ++p) {
        int k = ldv(&S.vkey[h]);
        if (k == v) return (int)h;
        if (k == -1) return -1;
        h = (h + 1) & (CV - 1);
    }
    return -1;
}

__device__ CSSG_PROBE int vinsert(const Slot& S, int CV, int v, WarpCtl* ctl)
{
    unsigned h = hash_int(v) & (CV - 1);
    for (int p = 0; p < CV; ++p) {
        int k = ldv(&S.vkey[h]);
        if (k == v) return (int)h;
        if (k == -1) {
            int old = atomicCAS(&S.vkey[h], -1, v);
            if (old == -1) {
                int pos = atomicAdd(&ctl->nV, 1);
                if (pos < CV) S.vlist[pos] = (int)h;
                return (int)h;
            }
            if (old == v) return (int)h;
        }
        h = (h + 1) & (CV - 1);
    }
    atomicExch(&ctl->err, CSSG_ST_CAPACITY);
    return -1;
}

__device__ CSSG_PROBE int ffind(const Slot& S, int CF, int f)
{
    unsigned h = hash_int(f) & (CF - 1);
    for (int p = 0; p < CF; ++p) {
        int k = ldv(&S.fkey[h]);
        if (k == f) return (int)h;
        if (k == -1) return -1;
        h = (h + 1) & (CF - 1);
    }
    return -1;
}

// returns slot; *fresh = 1 when this call inserted the key
__device__ CSSG_PROBE int finsert(const Slot& S, int CF, int f, WarpCtl* ctl, int* fresh)
{
    *fresh = 0;
    unsigned h = hash_int(f) & (CF - 1);
    for (int p = 0; p < CF; ++p) {
        int k = ldv(&S.fkey[h]);
        if (k == f) return (int)h;
        if (k == -1) {
            int old = atomicCAS(&S.fkey[h], -1, f);
            if (old == -1) {
                int pos = atomicAdd(&ctl->nF, 1);
                if (pos < CF) S.flist[pos] = (int)h;
                else atomicExch(&ctl->err, CSSG_ST_CAPACITY);
                *fresh = 1;
                return (int)h;
            }
            if (old == f) return (int)h;
        }
        h = (h + 1) & (CF - 1);
    }
    atomicExch(&ctl->err, CSSG_ST_CAPACITY);
    return -1;
}

__device__ __forceinline__ double vlabel(const Slot& S, int CV, int v)
{
    int h = vfind(S, CV, v);
    return h < 0 ? CUDART_INF : bitsd(ldv(&S.vlab[h]));
}

// ---- per-source solver state ----------------------------------------------------------------------------------
struct Src {
    int f0;
    double S[3];
    double e1[3], e2[3];
    bool full;
    double cutoff;
};

struct VRec {
    int slot, v;
    double d, dx, dy;
};

__device__ __forceinline__ bool in_domain(const DevMesh& M, const Slot& S, const GeoCaps& C, const Src& src, int g)
{
    if (g < 0) return false;
    if (src.full) return true;
    return ffind(S, C.CF, g) >= 0;
}

__device__ __noinline__ bool trim(const DevMesh& M, const Slot& S, const GeoCaps& C, Win& w)
{
    return trim_window(M, w, [&](int v) { return vlabel(S, C.CV, v); });
}

// Where a new window goes: 0 nowhere (outside the domain, empty, beyond the cutoff), 1 the current band queue,
// 2 the next frontier.  Clamps its interval to the edge and sets its key.  No trim here: windows are trimmed when
// they are processed, against the labels of that round.
__device__ __forceinline__ int window_dest(const DevMesh& M, const Slot& S, const GeoCaps& C, const Src& src,
                                           const WarpCtl* ctl, Win& w)
{
    const int g = w.he >> 2, j = w.he & 3;
    if (g == src.f0 || !in_domain(M, S, C, src, g)) return 0;
    const double L = M.geom[9 * g + 3 * j];
    w.b0 = fmax(0.0, w.b0);
    w.b1 = fmin(L, w.b1);
    if (!(w.b1 - w.b0 > 1e-14 * L)) return 0;
    const float key = key_lo(w);
    if ((double)key > src.cutoff) return 0;
    w.key = key;
    return (double)key <= ctl->thr ? 1 : 2;
}

__device__ __forceinline__ void push_win(const DevMesh& M, const Slot& S, const GeoCaps& C, const Src& src, WarpCtl* ctl, Win w)
{
    const int dest = window_dest(M, S, C, src, ctl, w);
    if (dest == 0) return;
    if (dest == 1) {
        // inside the current band: queue it for this round
        const int pos = atomicAdd(&ctl->qTail, 1);
        if (pos - ctl->qHead >= C.CW) {
            atomicExch(&ctl->err, CSSG_ST_CAPACITY);
            return;
        }
        S.wA[pos % C.CW] = w;
        return;
    }
    int pos = atomicAdd(&ctl->nB, 1);
    if (pos >= C.CW) {
        atomicExch(&ctl->err, CSSG_ST_CAPACITY);
        return;
    }
    S.wB[pos] = w;
}

__device__ __forceinline__ void propose(const Slot& S, const GeoCaps& C, WarpCtl* ctl, int v, double d, double dx,
                                        double dy, VRec& rec)
{
    rec.slot = -1;
    int h = vinsert(S, C.CV, v, ctl);
    if (h < 0) return;
    unsigned long long b = dbits(d);
    unsigned long long old = atomicMin(&S.vlab[h], b);
    if (b < old) {
        rec.slot = h;
        rec.v = v;
        rec.d = d;
        rec.dx = dx;
        rec.dy = dy;
    }
}

// a window's proposal for the vertex at (px, py) of its frame; the start direction is computed only if it wins
__device__ __forceinline__ void propose_from(const Slot& S, const GeoCaps& C, WarpCtl* ctl, const Win& w, int v,
                                             double px, double py, VRec& rec)
{
    const double l = len2(px - w.sx, py - w.sy);
    propose(S, C, ctl, v, w.sigma + l, 0.0, 0.0, rec);
    if (rec.slot >= 0) start_dir_l(w, px, py, l, rec.dx, rec.dy);
}

// Can vertex v (vertex-table slot h) become a pseudo-source: a border or saddle vertex of the mesh, or on a patch, a
// vertex with an incident face outside the patch.  The patch is complete before the first call, so the answer is
// cached per slot (lanes that evaluate the same vertex at once store the same value).
__device__ __noinline__ bool launchable(const DevMesh& M, const Slot& S, const GeoCaps& C, const Src& src, int v, int h)
{
    if (M.vflag[v] & (VF_BORDER | VF_SADDLE)) return true;
    if (src.full) return false;
    const signed char known = *(volatile signed char*)&S.vcan[h];
    if (known >= 0) return known != 0;
    bool out = false;
    for (int i = M.vfStart[v]; i < M.vfStart[v + 1] && !out; ++i) out = ffind(S, C.CF, M.vfList[i]) < 0;
    S.vcan[h] = out ? 1 : 0;
    return out;
}

// after __syncwarp: the surviving proposal writes the start direction and queues a pseudo-source launch
__device__ void resolve(const DevMesh& M, const Slot& S, const GeoCaps& C, const Src& src, WarpCtl* ctl,
                        const VRec& r)
{
    if (r.slot < 0) return;
    unsigned long long b = dbits(r.d);
    if (ldv(&S.vlab[r.slot]) != b) return;
    S.vtx[r.slot] = r.dx;
    S.vty[r.slot] = r.dy;
    if (r.d <= src.cutoff && launchable(M, S, C, src, r.v, r.slot)) {
        if (atomicExch(&S.vtok[r.slot], b) != b) {
            int pos = atomicAdd(&ctl->nLA, 1);
            if (pos < C.CL) S.lA[pos] = r.v;
            else atomicExch(&ctl->err, CSSG_ST_CAPACITY);
        }
    }
}

// Phase A of one window (one lane): trim, log it for the target queries and update the targets' running bests,
// then queue the vertex proposals and the child windows it makes.  The trimmed interval is written back to wA[q],
// where the tasks read it.
// Returns the tasks the window makes as a mask: bits 0-2 vertex proposals (opposite vertex, A, B), bits 3-4 child
// windows (through C->A, through B->C); bit 5 = processed (it survived the trim).  The caller appends them with
// warp-aggregated offsets.
__device__ int classify(const DevMesh& M, const Slot& S, const GeoCaps& C, WarpCtl* ctl, Win w, int q)
{
    if (!trim(M, S, C, w)) return 0;
    const int g = w.he >> 2, j = w.he & 3;
    const double L = M.geom[9 * g + 3 * j], cx = M.geom[9 * g + 3 * j + 1], cy = M.geom[9 * g + 3 * j + 2];
    const double tol = 1e-12 * L;
    int fh = ffind(S, C.CF, g);
    if (fh >= 0) {
        int head = ldv(&S.fhead[fh]);
        if (head >= 0) {
            int pos = atomicAdd(&ctl->nLog, 1);
            if (pos < C.CLOG) {
                S.wlog[pos] = w;
                S.lognext[pos] = atomicExch(&S.flog[fh], pos);
            } else {
                atomicExch(&ctl->err, CSSG_ST_CAPACITY);
            }
            for (int t = head; t >= 0; t = S.tnext[t]) {
                if (S.tidx[t] < 0) continue;
                double b1 = S.tb[3 * t + (j + 1) % 3], b2 = S.tb[3 * t + (j + 2) % 3];
                double px = b1 * L + b2 * cx, py = b2 * cy;
                if (ray_hits(w, px, py, tol)) {
                    double d = w.sigma + len2(px - w.sx, py - w.sy);
                    atomicMin(&S.tbest[t], dbits(d));
                }
            }
        }
    }
    S.wA[q].b0 = w.b0;
    S.wA[q].b1 = w.b1;
    const CrossC xc(w, cx, cy);
    int mask = 32;
    if (xc.rel(w.b0 - tol) <= 0 && xc.rel(w.b1 + tol) >= 0) mask |= 1;
    if (w.b0 <= tol) mask |= 2;
    if (w.b1 >= L - tol) mask |= 4;
    const double r0 = xc.rel(w.b0), r1 = xc.rel(w.b1);
    if (r0 < 0 && M.twin[3 * g + (j + 2) % 3] >= 0) mask |= 8;
    if (r1 > 0 && M.twin[3 * g + (j + 1) % 3] >= 0) mask |= 16;
    if (r1 >= 0) mask |= 64;   // the C->A child reaches C
    if (r0 <= 0) mask |= 128;  // the B->C child starts at C
    return mask;
}

// warp-aggregated append: lanes with `take` get consecutive slots starting at *counter (shared); returns the lane's
// slot (or -1).  Every lane of the warp must call it.
__device__ __forceinline__ int warp_append(int* counter, bool take, int lane)
{
    const unsigned m = __ballot_sync(FULL, take);
    int base = 0;
    if (lane == 0 && m) base = atomicAdd(counter, __popc(m));
    base = __shfl_sync(FULL, base, 0);
    return take ? base + __popc(m & ((1u << lane) - 1)) : -1;
}

// a queued vertex proposal: path length through the window to one of its face's vertices
__device__ void proposal_task(const DevMesh& M, const Slot& S, const GeoCaps& C, WarpCtl* ctl, int task, VRec& rec)
{
    const Win w = S.wA[task >> 2];
    const int k = task & 3;
    const int g = w.he >> 2, j = w.he & 3;
    double px = 0, py = 0;
    int v;
    if (k == 0) {
        px = M.geom[9 * g + 3 * j + 1];
        py = M.geom[9 * g + 3 * j + 2];
        v = M.F[3 * g + (j + 2) % 3];
    } else if (k == 1) {
        v = M.F[3 * g + j];
    } else {
        px = M.geom[9 * g + 3 * j];
        v = M.F[3 * g + (j + 1) % 3];
    }
    propose_from(S, C, ctl, w, v, px, py, rec);
}

// a queued child window: the part of the window's rays that leaves its face through one of the two other edges,
// expressed in the frame of that edge's twin
__device__ void child_task(const DevMesh& M, const Slot& S, const GeoCaps& C, const Src& src, int task, Win& c)
{
    // task = window << 2 | exit << 1 | flag: exit 0 (C->A) with flag "the interval reaches past C", exit 1 (B->C)
    // with flag "the interval starts before C" (both decided by classify)
    make_child(M, S.wA[task >> 2], (task & 2) != 0, (task & 1) != 0, c);
}

__device__ __forceinline__ double warp_max(double x)
{
    for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(FULL, x, o));
    return x;
}

// final distance of target t: source face, logged windows and face-vertex labels.  te (the direction of arrival) is
// filled only when wantTe: the force path uses the start direction alone.
__device__ __noinline__ double target_query(const DevMesh& M, const Slot& S, const GeoCaps& C, const Src& src, int t, int nLog,
                               double* ts, double* te, bool wantTe)
{
    const int f = S.tface[t];
    const double* P = &S.tp[3 * t];
    ts[0] = ts[1] = ts[2] = 0;
    te[0] = te[1] = te[2] = 0;
    if (f == src.f0) {
        double u[3] = {P[0] - src.S[0], P[1] - src.S[1], P[2] - src.S[2]};
        double d = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        if (d > 0)
            for (int c = 0; c < 3; ++c) ts[c] = te[c] = u[c] / d;  // one division serves both
        return d;
    }
    double best = CUDART_INF, bdx = 0, bdy = 0;
    int bw = -1;
    double bux = 0, buy = 0;
    const int fh = ffind(S, C.CF, f);
    for (int e = fh >= 0 ? __ldcg(&S.flog[fh]) : -1; e >= 0; e = S.lognext[e]) {
        if (e >= nLog) break;
        const Win w = S.wlog[e];
        const int g = w.he >> 2;
        const int j = w.he & 3;
        const double L = M.geom[9 * g + 3 * j], cx = M.geom[9 * g + 3 * j + 1], cy = M.geom[9 * g + 3 * j + 2];
        double b1 = S.tb[3 * t + (j + 1) % 3], b2 = S.tb[3 * t + (j + 2) % 3];
        double px = b1 * L + b2 * cx, py = b2 * cy;
        const double tol = 1e-12 * L;
        if (ray_hits(w, px, py, tol)) {
            double d = w.sigma + len2(px - w.sx, py - w.sy);
            if (d < best) {
                best = d;
                start_dir(w, px, py, bdx, bdy);
                bw = e;
                bux = px - w.sx;
                buy = py - w.sy;
            }
        }
    }
    if (bw >= 0 && wantTe) {
        const Win w = S.wlog[bw];
        const int g = w.he >> 2, j = w.he & 3;
        const double L = M.geom[9 * g + 3 * j], cx = M.geom[9 * g + 3 * j + 1], cy = M.geom[9 * g + 3 * j + 2];
        const double* PA = &M.V[3 * M.F[3 * g + j]];
        const double* PB = &M.V[3 * M.F[3 * g + (j + 1) % 3]];
        const double* PC = &M.V[3 * M.F[3 * g + (j + 2) % 3]];
        double ul = len2(bux, buy);
        for (int c = 0; c < 3; ++c) {
            double ex = (PB[c] - PA[c]) / L;
            double ey = (PC[c] - PA[c] - cx * ex) / cy;
            te[c] = (bux * ex + buy * ey) / ul;
        }
    }
    for (int c = 0; c < 3; ++c) {
        int v = M.F[3 * f + c];
        int h = vfind(S, C.CV, v);
        if (h < 0) continue;
        double lab = bitsd(ldv(&S.vlab[h]));
        if (!(lab < CUDART_INF)) continue;
        const double* pv = &M.V[3 * v];
        double u[3] = {P[0] - pv[0], P[1] - pv[1], P[2] - pv[2]};
        double l = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        double d = lab + l;
        if (d < best) {
            best = d;
            bdx = S.vtx[h];
            bdy = S.vty[h];
            if (wantTe)
                for (int q = 0; q < 3; ++q) te[q] = l > 0 ? u[q] / l : 0;
        }
    }
    if (best < CUDART_INF)
        for (int c = 0; c < 3; ++c) ts[c] = bdx * src.e1[c] + bdy * src.e2[c];
    return best;
}

// A source group: the G warps that solve one source together (G = 1, 2, 4 or 8).  With G = 1 the group is a warp and
// synchronises with __syncwarp; otherwise with a named barrier of 32 G threads (ids 1..8, one per group of the block).
// The barrier is the non-aligned form (barrier.sync): the groups of one block run different sources and so reach
// their barriers at different instructions, which the aligned form (bar.sync) does not allow.  Every thread of a
// group executes the same sequence of group barriers: all loops and early exits around them test values that the
// group read from its shared control block after the previous barrier.
template <int G>
struct Grp {
    static constexpr int NT = 32 * G;
    int t;        // thread in the group
    int lane;     // lane in its warp
    int wig;      // warp in the group
    int bar;      // named barrier id
    double* redD; // G doubles of shared scratch for reductions
    int* redI;    // G ints
    __device__ __forceinline__ void sync() const
    {
        if (G == 1) {
            __syncwarp();
        } else {
            __syncwarp();
            asm volatile("barrier.sync %0, %1;" ::"r"(bar), "r"(NT) : "memory");
        }
    }
    __device__ __forceinline__ double min(double x) const
    {
        for (int o = 16; o > 0; o >>= 1) x = fmin(x, __shfl_xor_sync(FULL, x, o));
        if (G == 1) return x;
        if (lane == 0) redD[wig] = x;
        sync();
        double r = redD[0];
        for (int k = 1; k < G; ++k) r = fmin(r, redD[k]);
        sync();
        return r;
    }
    __device__ __forceinline__ double sum(double x) const
    {
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
        if (G == 1) return x;
        if (lane == 0) redD[wig] = x;
        sync();
        double r = redD[0];
        for (int k = 1; k < G; ++k) r += redD[k];
        sync();
        return r;
    }
    __device__ __forceinline__ int sumi(int x) const
    {
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
        if (G == 1) return x;
        if (lane == 0) redI[wig] = x;
        sync();
        int r = redI[0];
        for (int k = 1; k < G; ++k) r += redI[k];
        sync();
        return r;
    }
    __device__ __forceinline__ bool any(bool p) const
    {
        if (G == 1) return __any_sync(FULL, p);
        return sumi(__any_sync(FULL, p) && lane == 0 ? 1 : 0) > 0;
    }
    __device__ __forceinline__ bool all(bool p) const
    {
        if (G == 1) return __all_sync(FULL, p);
        return sumi(__all_sync(FULL, p) || lane != 0 ? 0 : 1) == 0;
    }
};

// candidate-based early exit: no queued window can improve any target any more
template <int G>
__device__ __noinline__ bool settled(const DevMesh& M, const Slot& S, const GeoCaps& C, const Src& src, int nT,
                                    double minKey, const Grp<G>& gp)
{
    bool ok = true;
    for (int t = gp.t; t < nT; t += Grp<G>::NT) {
        if (S.tface[t] == src.f0 || S.tidx[t] < 0) continue;
        double b = bitsd(__ldcg(&S.tbest[t]));
        const double* P = &S.tp[3 * t];
        for (int c = 0; c < 3; ++c) {
            int v = M.F[3 * S.tface[t] + c];
            int h = vfind(S, C.CV, v);
            if (h < 0) continue;
            double lab = bitsd(ldv(&S.vlab[h]));
            if (!(lab < CUDART_INF)) continue;
            const double* pv = &M.V[3 * v];
            // upper bound of the path through v (FP32 length rounded up with a 1e-6 margin): the early exit only
            // needs upper bounds of the targets' distances
            const float ux = (float)(P[0] - pv[0]), uy = (float)(P[1] - pv[1]), uz = (float)(P[2] - pv[2]);
            const float l = sqrtf(ux * ux + uy * uy + uz * uz) * 1.000001f + 1e-30f;
            b = fmin(b, lab + (double)l);
        }
        if (!(b <= minKey || minKey > src.cutoff)) ok = false;
    }
    return gp.all(ok);
}

// The per-source solve (one source group).  Leaves results in the slot and the outputs.
// MODE 1: every system takes reference patches with cell-list (search mode 1) or screened-CSR (3) candidates, so the
// code of the other modes is compiled out (a smaller kernel); MODE 0 reads the mode of each system.
template <int G, int MODE>
__device__ void solve_source(const GeoLaunch& Lp, Slot S, WarpCtl* ctl, int si, const Grp<G>& gp,
                             unsigned long long* cnt)
{
    constexpr int NT = Grp<G>::NT;
    const int lane = gp.lane;
    const int t0 = gp.t;
    const GeoCaps& C = Lp.caps;
    const SysDesc& D = Lp.sys[Lp.sysOf ? Lp.sysOf[si] : 0];
    const DevMesh& M = D.mesh;
    const int searchMode = MODE == 1 ? (D.searchMode == 3 ? 3 : 1) : D.searchMode;
    const bool submesh = MODE == 1 ? true : D.submesh != 0;
    if (D.bigBin && Lp.routeBig && Lp.failList) {
        // binned to the large-table pass
        if (t0 == 0) {
            Lp.status[si] = 0;
            Lp.failList[atomicAdd(Lp.failCount, 1)] = si;
        }
        return;
    }
    Src src;
    src.f0 = Lp.srcFace[si];
    src.cutoff = D.cutoff;
    double b0[3] = {Lp.srcBary[3 * si], Lp.srcBary[3 * si + 1], Lp.srcBary[3 * si + 2]};
    load_pt(M, src.f0, b0, src.S);
    if (!isfinite(src.S[0] + src.S[1] + src.S[2])) {
        // a source whose position is not finite (a NaN barycentric weight): no geodesics, zero force
        if (t0 == 0) {
            Lp.status[si] = CSSG_ST_NAN;
            if (Lp.statusBits) atomicOr(Lp.statusBits, 1 << CSSG_ST_NAN);
            if (Lp.force) Lp.force[3 * si] = Lp.force[3 * si + 1] = Lp.force[3 * si + 2] = 0;
            if (Lp.pairCount) Lp.pairCount[si] = 0;
            if (Lp.inRangeOut) Lp.inRangeOut[si] = 0;
            if (Lp.srcCost) Lp.srcCost[si] = 1;
        }
        if (searchMode == 0)
            for (int o = Lp.candOff[si] + t0; o < Lp.candOff[si + 1]; o += Grp<G>::NT) {
                Lp.dOut[o] = CUDART_INF;
                for (int c = 0; c < 3; ++c) {
                    if (Lp.tsOut) Lp.tsOut[3 * o + c] = 0;
                    if (Lp.teOut) Lp.teOut[3 * o + c] = 0;
                }
            }
        return;
    }
    if (t0 == 0) {
        ctl->nA = ctl->nB = ctl->nLA = ctl->nLB = ctl->nLog = ctl->nV = ctl->nF = ctl->nT = ctl->err = 0;
        ctl->nBA = ctl->nBB = ctl->nProc = 0;
        ctl->qHead = ctl->qTail = 0;
        ctl->maxChord2 = 0;
        ctl->thr = -CUDART_INF;
    }
    gp.sync();
    // ---- targets ---------------------------------------------------------------------------------------------
    double maxChord2 = 0;
    if (searchMode == 0 || searchMode == 3) {
        int beg = Lp.candOff[si], nT = Lp.candOff[si + 1] - beg;
        if (nT > C.CT) {
            if (t0 == 0) ctl->err = CSSG_ST_CAPACITY;
            nT = 0;
        }
        for (int t = t0; t < nT; t += NT) {
            if (searchMode == 0) {
                S.tface[t] = Lp.candFace[beg + t];
                S.tidx[t] = beg + t;
                for (int c = 0; c < 3; ++c) S.tb[3 * t + c] = Lp.candBary[3 * (beg + t) + c];
            } else {
                // screened-out candidates keep their face in the patch but are not queried: index stored as -(j+1)
                int jj = Lp.candJ[beg + t];
                S.tface[t] = Lp.partFace[jj];
                S.tidx[t] = Lp.candSkip[beg + t] ? -(jj + 1) : jj;
                for (int c = 0; c < 3; ++c) S.tb[3 * t + c] = Lp.partBary[3 * jj + c];
            }
        }
        if (t0 == 0) ctl->nT = nT;
        if (searchMode == 3 && Lp.pairCount && t0 == 0) Lp.pairCount[si] = nT;
    } else if (gp.wig == 0) {
        // candidates j != i with chord^2 < range2 (cell list: 27 cells in (x, y, z) loop order; or all particles);
        // the first warp of the group searches, in the reference's order
        const double* Pi = &Lp.srcPos[3 * si];
        int count = 0;
        auto consider = [&](int jj, bool valid) {
            bool take = false;
            double d2 = 0;
            if (valid && jj != si) {
                const double* Pj = &Lp.partPos[3 * jj];
                double dx = Pi[0] - Pj[0], dy = Pi[1] - Pj[1], dz = Pi[2] - Pj[2];
                d2 = dx * dx + dy * dy + dz * dz;
                take = (searchMode == 2) || (d2 < D.range2);
            }
            unsigned m = __ballot_sync(FULL, take);
            if (take) {
                int pos = count + __popc(m & ((1u << lane) - 1));
                if (pos < C.CT) {
                    S.tface[pos] = Lp.partFace[jj];
                    S.tidx[pos] = jj;
                    for (int c = 0; c < 3; ++c) S.tb[3 * pos + c] = Lp.partBary[3 * jj + c];
                }
                maxChord2 = fmax(maxChord2, d2);
            }
            count += __popc(m);
        };
        if (searchMode == 2) {
            for (int base = 0; base < D.nPart; base += 32) consider(D.partBase + base + lane, base + lane < D.nPart);
        } else {
            int ci[3];
            for (int c = 0; c < 3; ++c) {
                int q = (int)floor((Pi[c] - D.lo[c]) / D.cs[c]);
                ci[c] = max(0, min(D.nc[c] - 1, q));
            }
            for (int xx = max(0, ci[0] - 1); xx <= min(D.nc[0] - 1, ci[0] + 1); ++xx)
                for (int yy = max(0, ci[1] - 1); yy <= min(D.nc[1] - 1, ci[1] + 1); ++yy)
                    for (int zz = max(0, ci[2] - 1); zz <= min(D.nc[2] - 1, ci[2] + 1); ++zz) {
                        int cell = D.cellBase + xx + D.nc[0] * (yy + D.nc[1] * zz);
                        int a = Lp.cellStart[cell], b = Lp.cellStart[cell + 1];
                        for (int base = a; base < b; base += 32) {
                            int q = base + lane;
                            consider(q < b ? Lp.cellList[q] : 0, q < b);
                        }
                    }
        }
        maxChord2 = warp_max(maxChord2);
        if (count > C.CT) {
            if (lane == 0) ctl->err = CSSG_ST_CAPACITY;
            count = 0;
        }
        if (lane == 0) {
            ctl->nT = count;
            ctl->maxChord2 = maxChord2;
        }
        if (Lp.pairCount && lane == 0) Lp.pairCount[si] = count;
    }
    gp.sync();
    maxChord2 = ctl->maxChord2;
    const int nT = ctl->nT;
    if (ctl->err == CSSG_ST_CAPACITY && Lp.failList) {
        if (t0 == 0) {
            Lp.status[si] = 0;
            Lp.failList[atomicAdd(Lp.failCount, 1)] = si;
        }
        return;
    }
    if (nT == 0) {
        if (Lp.srcCost && t0 == 0) Lp.srcCost[si] = 1;
        if (Lp.inRangeOut && t0 == 0) Lp.inRangeOut[si] = 0;
        if (Lp.force && t0 == 0) {
            Lp.force[3 * si] = Lp.force[3 * si + 1] = Lp.force[3 * si + 2] = 0;  // no kick: zero force
        }
        if (t0 == 0) {
            Lp.status[si] = ctl->err;
            if (ctl->err && Lp.statusBits) atomicOr(Lp.statusBits, 1 << ctl->err);
        }
        return;
    }
    for (int t = t0; t < nT; t += NT) {
        load_pt(M, S.tface[t], &S.tb[3 * t], &S.tp[3 * t]);
        S.tbest[t] = INF_BITS;
        S.tnext[t] = -1;
    }
    gp.sync();
    // ---- domain: whole mesh or the reference patch ---------------------------------------------------------------
    src.full = !submesh;
    double r = D.maxDist;
    if (searchMode == 0 || searchMode == 3) {
        if (Lp.threshold && Lp.threshold[si] < r) r = Lp.threshold[si];
    } else {
        double mc = sqrt(maxChord2);
        if (searchMode == 2) mc = 1e20;
        if (mc < r) r = mc;
    }
    if (submesh) {
        int fresh;
        bool notInF0 = false, notInSeeds = false;
        int nb[3];
        for (int k = 0; k < 3; ++k) {
            int t = M.twin[3 * src.f0 + k];
            nb[k] = t < 0 ? -1 : t / 3;
        }
        for (int t = t0; t < nT; t += NT) {
            int f = S.tface[t];
            if (f != src.f0) {
                notInF0 = true;
                if (f != nb[0] && f != nb[1] && f != nb[2]) notInSeeds = true;
            }
        }
        notInF0 = gp.any(notInF0);
        notInSeeds = gp.any(notInSeeds);
        if (t0 == 0) finsert(S, C.CF, src.f0, ctl, &fresh);
        gp.sync();
        if (notInF0) {
            if (t0 < 3 && nb[t0] >= 0) {
                int h = finsert(S, C.CF, nb[t0], ctl, &fresh);
                if (fresh && notInSeeds) {
                    int pos = atomicAdd(&ctl->nBA, 1);
                    S.bA[pos] = nb[t0];
                }
            }
            gp.sync();
            if (notInSeeds) {
                const double r2 = r * r;
                int* cur = S.bA;
                int* nxt = S.bB;
                int nCur = ctl->nBA;
                int guard = 0;
                while (nCur > 0 && guard++ < 100000) {
                    gp.sync();  // every lane has read nCur / err before lane 0 resets the counter
                    if (t0 == 0) ctl->nBB = 0;
                    gp.sync();
                    for (int q = t0; q < 3 * nCur; q += NT) {
                        int f = cur[q / 3], k = q % 3;
                        int t = M.twin[3 * f + k];
                        if (t < 0) continue;
                        int g = t / 3;
                        if (ffind(S, C.CF, g) >= 0) continue;
                        bool near = false;
                        for (int c = 0; c < 3; ++c) {
                            const double* pv = &M.V[3 * M.F[3 * g + c]];
                            double dx = src.S[0] - pv[0], dy = src.S[1] - pv[1], dz = src.S[2] - pv[2];
                            if (!(dx * dx + dy * dy + dz * dz > r2)) near = true;
                        }
                        if (!near) continue;
                        finsert(S, C.CF, g, ctl, &fresh);
                        if (fresh) {
                            int pos = atomicAdd(&ctl->nBB, 1);
                            if (pos < C.CF) nxt[pos] = g;
                            else atomicExch(&ctl->err, CSSG_ST_CAPACITY);
                        }
                    }
                    gp.sync();
                    nCur = ctl->err ? 0 : min(ctl->nBB, C.CF);
                    int* tmp = cur;
                    cur = nxt;
                    nxt = tmp;
                }
            }
        }
        // goal faces (targets) complete the patch
        for (int t = t0; t < nT; t += NT) finsert(S, C.CF, S.tface[t], ctl, &fresh);
        gp.sync();
    }
    // target lists per face (full mode: the face table holds only target faces)
    for (int t = t0; t < nT; t += NT) {
        int fresh;
        int h = finsert(S, C.CF, S.tface[t], ctl, &fresh);
        if (h >= 0) S.tnext[t] = atomicExch(&S.fhead[h], t);
    }
    gp.sync();
    // ---- source: frame, face-vertex labels, initial windows -------------------------------------------------------
    const int f0 = src.f0;
    const double L0 = M.geom[9 * f0], cx0 = M.geom[9 * f0 + 1], cy0 = M.geom[9 * f0 + 2];
    {
        const double* p0 = &M.V[3 * M.F[3 * f0]];
        const double* p1 = &M.V[3 * M.F[3 * f0 + 1]];
        const double* p2 = &M.V[3 * M.F[3 * f0 + 2]];
        for (int c = 0; c < 3; ++c) src.e1[c] = (p1[c] - p0[c]) / L0;
        for (int c = 0; c < 3; ++c) src.e2[c] = (p2[c] - p0[c] - cx0 * src.e1[c]) / cy0;
    }
    const double P2[3][2] = {{0, 0}, {L0, 0}, {cx0, cy0}};
    const double S2x = b0[1] * L0 + b0[2] * cx0, S2y = b0[2] * cy0;
    VRec rec[3];
    rec[0].slot = rec[1].slot = rec[2].slot = -1;
    if (t0 < 3) {
        int k = t0;
        int v = M.F[3 * f0 + k];
        double dx = P2[k][0] - S2x, dy = P2[k][1] - S2y;
        double l = len2(dx, dy);
        const double* pv = &M.V[3 * v];
        double u[3] = {pv[0] - src.S[0], pv[1] - src.S[1], pv[2] - src.S[2]};
        propose(S, C, ctl, v, sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]), dx / l, dy / l, rec[0]);
    }
    gp.sync();
    resolve(M, S, C, src, ctl, rec[0]);
    gp.sync();
    if (t0 < 3) {
        int k = t0;
        int t = M.twin[3 * f0 + k];
        if (t >= 0) {
            double L = M.geom[9 * f0 + 3 * k];
            double skx = b0[(k + 1) % 3] * L + b0[(k + 2) % 3] * M.geom[9 * f0 + 3 * k + 1];
            double sky = b0[(k + 2) % 3] * M.geom[9 * f0 + 3 * k + 2];
            Win w;
            w.he = (t / 3) * 4 + t % 3;
            w.sigma = 0;
            w.sx = L - skx;
            w.sy = fmin(-sky, -1e-15 * L);
            w.b0 = 0;
            w.b1 = L;
            double ddx = P2[(k + 1) % 3][0] - P2[k][0], ddy = P2[(k + 1) % 3][1] - P2[k][1];
            double dl = len2(ddx, ddy);
            w.c = -ddx / dl;
            w.s = -ddy / dl;
            push_win(M, S, C, src, ctl, w);
        }
    }
    gp.sync();
    // ---- rounds ---------------------------------------------------------------------------------------------------
    // Distance-banded rounds: each round takes the smallest key among queued windows and queued pseudo-source
    // launches (mk) and handles only what lies within mk + delta, deferring the rest, so labels are close to final
    // when they are used (a breadth-first order would relaunch border and saddle vertices in cascades).  The initial
    // windows sit in S.wB (ctl->nB); each round swaps the buffers and processes S.wA into S.wB.
    int processed = 0, launches = 0;
    int round = 0;
    while (true) {
        gp.sync();
        const int nA = min(ctl->nB, C.CW);
        const int nP = min(ctl->nLA, C.CL);
        if (ctl->err || (nA == 0 && nP == 0)) break;
        if (++round > Lp.maxRounds || ctl->nProc > Lp.maxWindows) {
            if (t0 == 0) ctl->err = CSSG_ST_CAPACITY;
            break;
        }
        {
            Win* t = S.wA;
            S.wA = S.wB;
            S.wB = t;
        }
        for (int q = t0; q < nP; q += NT) S.lB[q] = S.lA[q];
        gp.sync();
        if (t0 == 0) {
            ctl->nB = 0;
            ctl->nLA = 0;
        }
        double mk = CUDART_INF;
        for (int q = t0; q < nA; q += NT) mk = fmin(mk, (double)S.wA[q].key);
        for (int q = t0; q < nP; q += NT) mk = fmin(mk, vlabel(S, C.CV, S.lB[q]));
        mk = gp.min(mk);
        gp.sync();
        if (settled<G>(M, S, C, src, nT, mk, gp)) break;
        const double thr = mk + (Lp.deltaScale > 0 ? Lp.deltaScale : 1.0) * (D.delta > 0 ? D.delta : Lp.delta);
        // the band queue starts with this round's frontier; windows created inside the band join it
        if (t0 == 0) {
            ctl->qHead = 0;
            ctl->qTail = nA;
            ctl->thr = thr;
        }
        gp.sync();
        // The band: pseudo-source launches within it, then its window queue until empty; launches queued meanwhile
        // whose labels fall inside the band are launched in the same round, then the queue runs again.
        int nPc = nP;
        while (true) {
            if (nPc > 0) {
                const int nP = nPc;
                // pseudo-source launches within the band; the rest stay queued.  Decide per queued vertex, then
                // spread the (vertex, incident face) pairs over the lanes.
                for (int q = t0; q < nP; q += NT) {
                    int v = S.lB[q];
                    int h = vfind(S, C.CV, v);
                    S.ld[3 * q] = -1.0;
                    int deg = 0;
                    if (h >= 0) {
                        unsigned long long lb = ldv(&S.vlab[h]);
                        double d = bitsd(lb);
                        if (d > thr) {
                            int pos = atomicAdd(&ctl->nLA, 1);
                            if (pos < C.CL) S.lA[pos] = v;
                            else atomicExch(&ctl->err, CSSG_ST_CAPACITY);
                        } else if (atomicExch(&S.vlaunched[h], lb) != lb) {  // not yet launched with this label
                            S.ld[3 * q] = d;
                            S.ld[3 * q + 1] = S.vtx[h];
                            S.ld[3 * q + 2] = S.vty[h];
                            deg = M.vfStart[v + 1] - M.vfStart[v];
                            launches++;
                        }
                    }
                    S.lpre[q] = deg;
                }
                gp.sync();
                // exclusive prefix of the face counts (warp scan over chunks of 32 entries)
                if (gp.wig == 0) {
                    int run = 0;
                    for (int base = 0; base < nP; base += 32) {
                        int q = base + lane;
                        int x = q < nP ? S.lpre[q] : 0;
                        int incl = x;
                        for (int o = 1; o < 32; o <<= 1) {
                            int y = __shfl_up_sync(FULL, incl, o);
                            if (lane >= o) incl += y;
                        }
                        __syncwarp();  // the first warp alone: a warp barrier, not the group's
                        if (q < nP) S.lpre[q] = run + incl - x;
                        run += __shfl_sync(FULL, incl, 31);
                    }
                    if (t0 == 0) S.lpre[nP] = run;
                }
                gp.sync();
                const int pairs = S.lpre[nP];
                // pass 1: windows on the opposite edges + edge-path proposals, one (vertex, face) pair per lane
                for (int p = t0; p < pairs; p += NT) {
                    int lo = 0, hi = nP - 1;  // last entry with lpre <= p
                    while (lo < hi) {
                        int mid = (lo + hi + 1) >> 1;
                        if (S.lpre[mid] <= p) lo = mid;
                        else hi = mid - 1;
                    }
                    const int q = lo;
                    const int v = S.lB[q];
                    const double d = S.ld[3 * q], tx = S.ld[3 * q + 1], ty = S.ld[3 * q + 2];
                    const int f = M.vfList[M.vfStart[v] + (p - S.lpre[q])];
                    if (!in_domain(M, S, C, src, f)) continue;
                    int k = 0;
                    while (M.F[3 * f + k] != v) ++k;
                    int e = (k + 1) % 3;
                    VRec r1, r2;
                    propose(S, C, ctl, M.F[3 * f + e], d + M.geom[9 * f + 3 * k], tx, ty, r1);
                    propose(S, C, ctl, M.F[3 * f + (k + 2) % 3], d + M.geom[9 * f + 3 * ((k + 2) % 3)], tx, ty, r2);
                    int t = M.twin[3 * f + e];
                    if (t < 0) continue;
                    Win c;
                    c.he = (t / 3) * 4 + t % 3;
                    c.sigma = d;
                    double L = M.geom[9 * f + 3 * e];
                    c.sx = L - M.geom[9 * f + 3 * e + 1];
                    c.sy = -M.geom[9 * f + 3 * e + 2];
                    c.b0 = 0;
                    c.b1 = L;
                    c.c = tx;
                    c.s = ty;
                    push_win(M, S, C, src, ctl, c);
                }
                gp.sync();
                // pass 2: surviving edge-path proposals take the start direction their launcher had
                for (int p = t0; p < pairs; p += NT) {
                    int lo = 0, hi = nP - 1;
                    while (lo < hi) {
                        int mid = (lo + hi + 1) >> 1;
                        if (S.lpre[mid] <= p) lo = mid;
                        else hi = mid - 1;
                    }
                    const int q = lo;
                    const int v = S.lB[q];
                    const double d = S.ld[3 * q], tx = S.ld[3 * q + 1], ty = S.ld[3 * q + 2];
                    const int f = M.vfList[M.vfStart[v] + (p - S.lpre[q])];
                    if (!in_domain(M, S, C, src, f)) continue;
                    int k = 0;
                    while (M.F[3 * f + k] != v) ++k;
                    VRec r;
                    r.dx = tx;
                    r.dy = ty;
                    r.v = M.F[3 * f + (k + 1) % 3];
                    r.d = d + M.geom[9 * f + 3 * k];
                    r.slot = vfind(S, C.CV, r.v);
                    resolve(M, S, C, src, ctl, r);
                    r.v = M.F[3 * f + (k + 2) % 3];
                    r.d = d + M.geom[9 * f + 3 * ((k + 2) % 3)];
                    r.slot = vfind(S, C.CV, r.v);
                    resolve(M, S, C, src, ctl, r);
                }
                gp.sync();
            }
            // the band queue, 32 windows at a time: each lane classifies one window, then the vertex proposals and
            // the child windows of the batch are spread over all lanes (FP64 instructions cost the same with 1 or
            // 32 lanes); children inside the band join the queue, so the queue runs until the band is empty
            while (true) {
                gp.sync();
                const int head = ctl->qHead;
                const int tail = min(ctl->qTail, head + C.CW);
                if (head >= tail || ctl->err) break;
                if (ctl->nProc > Lp.maxWindows) {
                    if (t0 == 0) ctl->err = CSSG_ST_CAPACITY;
                    break;
                }
                const int cnt = min(NT, tail - head);
                const int q = (head + t0) % C.CW;
                gp.sync();
                if (t0 == 0) {
                    ctl->nPT = 0;
                    ctl->nCT = 0;
                }
                gp.sync();
                int tmask = 0;
                bool defer = false;
                Win w;
                if (t0 < cnt) {
                    w = S.wA[q];
                    defer = (double)w.key > thr;
                    if (!defer) tmask = classify(M, S, C, ctl, w, q);
                }
                {
                    const int pos = warp_append(&ctl->nB, defer, lane);  // beyond the band: next frontier
                    if (defer) {
                        if (pos < C.CW) S.wB[pos] = w;
                        else atomicExch(&ctl->err, CSSG_ST_CAPACITY);
                    }
                }
                {
                    const unsigned pm = __ballot_sync(FULL, tmask & 32);
                    processed += (tmask & 32) ? 1 : 0;
                    if (lane == 0 && pm) atomicAdd(&ctl->nProc, __popc(pm));  // every warp of the group
                }
                for (int k = 0; k < 3; ++k) {
                    const int pos = warp_append(&ctl->nPT, (tmask >> k) & 1, lane);
                    if (pos >= 0) S.taskP[pos] = (q << 2) | k;
                }
                for (int k = 0; k < 2; ++k) {
                    const int pos = warp_append(&ctl->nCT, (tmask >> (3 + k)) & 1, lane);
                    if (pos >= 0) S.taskC[pos] = (q << 2) | (k << 1) | ((tmask >> (6 + k)) & 1);
                }
                gp.sync();
                const int nPT = ctl->nPT, nCT = ctl->nCT;
                for (int p0 = 0; p0 < nPT; p0 += NT) {
                    VRec r;
                    r.slot = -1;
                    if (p0 + t0 < nPT) proposal_task(M, S, C, ctl, S.taskP[p0 + t0], r);
                    gp.sync();
                    resolve(M, S, C, src, ctl, r);
                    gp.sync();
                }
                for (int p0 = 0; p0 < nCT; p0 += NT) {
                    Win c;
                    int dest = 0;
                    if (p0 + t0 < nCT) {
                        child_task(M, S, C, src, S.taskC[p0 + t0], c);
                        dest = window_dest(M, S, C, src, ctl, c);
                    }
                    const int pr = warp_append(&ctl->qTail, dest == 1, lane);
                    const int pb = warp_append(&ctl->nB, dest == 2, lane);
                    if (dest == 1) {
                        if (pr - head >= C.CW) atomicExch(&ctl->err, CSSG_ST_CAPACITY);
                        else S.wA[pr % C.CW] = c;
                    } else if (dest == 2) {
                        if (pb < C.CW) S.wB[pb] = c;
                        else atomicExch(&ctl->err, CSSG_ST_CAPACITY);
                    }
                }
                gp.sync();
                if (t0 == 0) ctl->qHead = head + cnt;
            }
            gp.sync();
            if (ctl->err) break;
            const int nL = min(ctl->nLA, C.CL);
            bool inBand = false;
            for (int q = t0; q < nL; q += NT) inBand |= vlabel(S, C.CV, S.lA[q]) <= thr;
            if (!gp.any(inBand)) break;
            for (int q = t0; q < nL; q += NT) S.lB[q] = S.lA[q];
            gp.sync();
            if (t0 == 0) ctl->nLA = 0;
            gp.sync();
            nPc = nL;
        }
        if (t0 == 0) ctl->thr = -CUDART_INF;
    }
    gp.sync();
    // ---- results -------------------------------------------------------------------------------------------------
    const int nLog = min(ctl->nLog, C.CLOG);
    const int err = ctl->err;
    if (err == CSSG_ST_CAPACITY && Lp.failList) {
        // tables too small for this source: queue it for the large-table pass, which writes all its outputs
        if (t0 == 0) {
            Lp.status[si] = 0;
            Lp.failList[atomicAdd(Lp.failCount, 1)] = si;
        }
        return;
    }
    double fx = 0, fy = 0, fz = 0;
    int inRange = 0;
    const bool wantTe = searchMode == 0 && Lp.teOut;
    for (int t = t0; t < nT; t += NT) {
        double ts[3], te[3] = {0, 0, 0};
        const bool screened = S.tidx[t] < 0;
        double d = (err || screened) ? CUDART_INF : target_query(M, S, C, src, t, nLog, ts, te, wantTe);
        if (screened) ts[0] = ts[1] = ts[2] = te[0] = te[1] = te[2] = 0;
        if (d > src.cutoff) {
            d = CUDART_INF;
            ts[0] = ts[1] = ts[2] = te[0] = te[1] = te[2] = 0;
        }
        if (searchMode == 0) {
            int o = S.tidx[t];
            if (!(d < CUDART_INF) && Lp.patchDisconnected) {
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
                size_t o = (size_t)si * Lp.pairCap + t;
                Lp.dOut[o] = d;
                Lp.pairJ[o] = S.tidx[t];  // -(j + 1) for a screened-out pair
                for (int c = 0; c < 3; ++c) Lp.tsOut[3 * o + c] = ts[c];
            }
            if (d < CUDART_INF) {
                double fm = 0;
                if (D.forceKind == 0) {
                    if (d <= D.sigma) fm = -D.k * (D.sigma - d);
                } else {
                    const double sqrtTwoPi = 2.50662827463100050241576528481104525300698674061;
                    fm = -(d * D.k * exp(-d * d / (2.0 * D.sigma * D.sigma)) /
                           ((sqrtTwoPi * D.sigma) * sqrt(D.sigma)));
                }
                fx += fm * ts[0];
                fy += fm * ts[1];
                fz += fm * ts[2];
                if (d <= D.sigma) inRange++;
            }
        }
    }
    if (Lp.force) {
        fx = gp.sum(fx);
        fy = gp.sum(fy);
        fz = gp.sum(fz);
        if (t0 == 0) {
            Lp.force[3 * si] = fx;
            Lp.force[3 * si + 1] = fy;
            Lp.force[3 * si + 2] = fz;
            if (Lp.kickVel) {  // velocityVerletNVE second half (velocityVerletNVE.cpp:23-29) for this particle
                Lp.kickVel[3 * si] += 0.5 * Lp.kickDt * fx;
                Lp.kickVel[3 * si + 1] += 0.5 * Lp.kickDt * fy;
                Lp.kickVel[3 * si + 2] += 0.5 * Lp.kickDt * fz;
            }
        }
    }
    inRange = gp.sumi(inRange);
    if (t0 == 0 && Lp.inRangeOut) Lp.inRangeOut[si] = inRange;
    processed = gp.sumi(processed);
    launches = gp.sumi(launches);
    if (t0 == 0 && Lp.srcCost) Lp.srcCost[si] = processed + launches + 8 * round + 1;
    if (t0 == 0 && Lp.stats) {
        Lp.stats[4 * si] = processed;
        Lp.stats[4 * si + 1] = launches;
        Lp.stats[4 * si + 2] = round;
        Lp.stats[4 * si + 3] = nT;
    }
    if (t0 == 0) {
        Lp.status[si] = err;
        if (err && Lp.statusBits) atomicOr(Lp.statusBits, 1 << err);
        cnt[0] += processed;
        cnt[1] += launches;
        cnt[2] += inRange;
        cnt[3] += err ? 1 : 0;
    }
}

template <int G>
__device__ void reset_slot(const Slot& S, const GeoCaps& C, WarpCtl* ctl, const Grp<G>& gp)
{
    constexpr int NT = Grp<G>::NT;
    const int lane = gp.t;
    gp.sync();
    int nV = min(ctl->nV, C.CV), nF = min(ctl->nF, C.CF);
    for (int q = lane; q < nV; q += NT) {
        int h = S.vlist[q];
        S.vkey[h] = -1;
        S.vlab[h] = INF_BITS;
        S.vtok[h] = ~0ull;
        S.vlaunched[h] = ~0ull;
        S.vcan[h] = -1;
    }
    for (int q = lane; q < nF; q += NT) {
        int h = S.flist[q];
        S.fkey[h] = -1;
        S.fhead[h] = -1;
        S.flog[h] = -1;
    }
    if (ctl->nV > C.CV || ctl->nF > C.CF) {
        // a table overflowed its touched list: clear it whole
        for (int q = lane; q < C.CV; q += NT) {
            S.vkey[q] = -1;
            S.vlab[q] = INF_BITS;
            S.vtok[q] = ~0ull;
            S.vlaunched[q] = ~0ull;
            S.vcan[q] = -1;
        }
        for (int q = lane; q < C.CF; q += NT) {
            S.fkey[q] = -1;
            S.fhead[q] = -1;
            S.flog[q] = -1;
        }
    }
    gp.sync();
}

// One source group (G warps) per slot; groups pull sources from the work counter until none are left.
// MINB = 2 lets ptxas use up to 128 registers per thread (two full blocks per SM); MINB = 1 up to 255 (no spills,
// at most 8 warps per SM).  The autotuner picks.
template <int G, int MINB, int MODE>
__global__ void __launch_bounds__(256, MINB) geodesic_kernel(GeoLaunch L)
{
    constexpr int NT = 32 * G;
    __shared__ WarpCtl ctls[8];
    __shared__ int tasks[8 * (kTaskP + kTaskC)];
    __shared__ double redD[8][8];
    __shared__ int redI[8][8];
    extern __shared__ __align__(16) char dyn[];
    const int gib = threadIdx.x / NT;
    const int group = blockIdx.x * (blockDim.x / NT) + gib;
    if (group >= L.nSlots) return;
    Grp<G> gp;
    gp.t = threadIdx.x % NT;
    gp.lane = threadIdx.x & 31;
    gp.wig = gp.t >> 5;
    gp.bar = 1 + gib;
    gp.redD = redD[gib];
    gp.redI = redI[gib];
    WarpCtl* ctl = &ctls[gib];
    Slot S;
    carve(L.caps, (char*)L.scratch + (size_t)group * L.slotBytes, &S);
    S.taskP = &tasks[gib * G * (kTaskP + kTaskC)];
    S.taskC = S.taskP + G * kTaskP;
    if (L.smemTables) {
        carve_smem(L.caps, dyn + (size_t)gib * smem_per_warp(L.caps), &S);
        for (int q = gp.t; q < L.caps.CV; q += NT) {
            S.vkey[q] = -1;
            S.vlab[q] = INF_BITS;
            S.vcan[q] = -1;
        }
        for (int q = gp.t; q < L.caps.CF; q += NT) {
            S.fkey[q] = -1;
            S.fhead[q] = -1;
        }
    }
    gp.sync();
    unsigned long long cnt[4] = {0, 0, 0, 0};
    while (true) {
        if (gp.t == 0) ctl->item = atomicAdd(L.workCounter, 1);
        gp.sync();
        const int item = ctl->item;
        gp.sync();
        int nItems = L.nSrc;
        if (L.itemCountDev) nItems = min(nItems, *(volatile const int*)L.itemCountDev);
        if (item >= nItems) break;
        int si = L.order ? L.order[item] : item;
        solve_source<G, MODE>(L, S, ctl, si, gp, cnt);
        reset_slot<G>(S, L.caps, ctl, gp);
    }
    if (gp.t == 0 && L.counters) {
        for (int k = 0; k < 4; ++k)
            if (cnt[k]) atomicAdd(&L.counters[k], cnt[k]);
    }
}

__global__ void init_scratch_kernel(char* scratch, size_t slotBytes, int nSlots, GeoCaps C)
{
    int warp = blockIdx.x;
    if (warp >= nSlots) return;
    Slot S;
    carve(C, scratch + (size_t)warp * slotBytes, &S);
    for (int q = threadIdx.x; q < C.CV; q += blockDim.x) {
        S.vtok[q] = ~0ull;
        S.vlaunched[q] = ~0ull;
        S.vcan[q] = -1;
        S.vkey[q] = -1;
        S.vlab[q] = INF_BITS;
    }
    for (int q = threadIdx.x; q < C.CF; q += blockDim.x) {
        S.fkey[q] = -1;
        S.fhead[q] = -1;
        S.flog[q] = -1;
    }
}

__global__ void max_count_kernel(int n, const int* off, int* out)
{
    int m = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) m = max(m, off[i + 1] - off[i]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(FULL, m, o));
    __shared__ int s[32];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        int r = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) r = max(r, s[k]);
        *out = r;
    }
}

#ifndef CSSG_GEO_OUTLINE
int next_pow2(long long x)
{
    int p = 1;
    while (p < x && p < (1 << 30)) p <<= 1;
    return p;
}

#endif
}  // namespace

#ifndef CSSG_GEO_OUTLINE
// warp per source: the same candidate search as the fused kernel's cell-list mode, written out as padded rows
__global__ void __launch_bounds__(256) candidates_kernel(GeoLaunch L, int n, int cap, int* __restrict__ candJ,
                                                         int* __restrict__ count, double* __restrict__ maxChord)
{
    const int lane = threadIdx.x & 31;
    for (int si = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; si < n; si += (gridDim.x * blockDim.x) >> 5) {
        const SysDesc& D = L.sys[L.sysOf ? L.sysOf[si] : 0];
        const double* Pi = &L.srcPos[3 * si];
        int cnt = 0;
        double mx = 0;
        auto consider = [&](int jj, bool valid) {
            bool take = false;
            double d2 = 0;
            if (valid && jj != si) {
                const double* Pj = &L.partPos[3 * jj];
                double dx = Pi[0] - Pj[0], dy = Pi[1] - Pj[1], dz = Pi[2] - Pj[2];
                d2 = dx * dx + dy * dy + dz * dz;
                take = d2 < D.range2;
            }
            unsigned m = __ballot_sync(FULL, take);
            if (take) {
                int pos = cnt + __popc(m & ((1u << lane) - 1));
                if (pos < cap) candJ[(size_t)si * cap + pos] = jj;
                mx = fmax(mx, d2);
            }
            cnt += __popc(m);
        };
        int ci[3];
        for (int c = 0; c < 3; ++c) {
            int q = (int)floor((Pi[c] - D.lo[c]) / D.cs[c]);
            ci[c] = max(0, min(D.nc[c] - 1, q));
        }
        for (int xx = max(0, ci[0] - 1); xx <= min(D.nc[0] - 1, ci[0] + 1); ++xx)
            for (int yy = max(0, ci[1] - 1); yy <= min(D.nc[1] - 1, ci[1] + 1); ++yy)
                for (int zz = max(0, ci[2] - 1); zz <= min(D.nc[2] - 1, ci[2] + 1); ++zz) {
                    int cell = D.cellBase + xx + D.nc[0] * (yy + D.nc[1] * zz);
                    int a = L.cellStart[cell], b = L.cellStart[cell + 1];
                    for (int base = a; base < b; base += 32) {
                        int q = base + lane;
                        consider(q < b ? L.cellList[q] : 0, q < b);
                    }
                }
        mx = warp_max(mx);
        if (lane == 0) {
            count[si] = cnt;
            maxChord[si] = sqrt(mx);
        }
    }
}

size_t cssg_geo_slot_bytes(const GeoCaps& c) { return align_up(carve(c, nullptr, nullptr)); }

void cssg_launch_candidates(const GeoLaunch& L, int n, int cap, int* candJ, int* count, double* maxChord,
                            cudaStream_t s)
{
    if (n <= 0) return;
    int blocks = (n + 7) / 8;
    candidates_kernel<<<blocks, 256, 0, s>>>(L, n, cap, candJ, count, maxChord);
}

void cssg_geo_init_scratch(void* scratch, size_t slotBytes, int nSlots, const GeoCaps& c, cudaStream_t s)
{
    if (nSlots > 0) init_scratch_kernel<<<nSlots, 256, 0, s>>>((char*)scratch, slotBytes, nSlots, c);
}

size_t cssg_geo_smem_per_warp(const GeoCaps& c) { return smem_per_warp(c); }
#endif

namespace {
template <int G, int MINB, int MODE = 0>
void launch_groups(GeoLaunch L, cudaStream_t s)
{
    // groups of G warps, each solving one source at a time in its own slot; a block holds gpb groups
    const size_t per = smem_per_warp(L.caps);  // tables of one group
    const size_t budget = 200 * 1024;
    const int wmax = (L.wpbMax > 0 && L.wpbMax < 8) ? L.wpbMax : 8;
    int gpb = std::max(1, wmax / G);
    size_t smem = 0;
    const int dev = L.device;
    L.smemTables = per <= budget ? 1 : 0;
    if (L.smemTables) {
        gpb = (int)std::max<size_t>(1, std::min<size_t>(gpb, budget / per));
        smem = per * gpb;
        static std::atomic<unsigned long long> configured{0};
        // the 48 KB default covers static + dynamic shared memory together, so raise the limit whenever the tables
        // are in shared memory (once per device)
        cssg_raise_smem_once(configured, geodesic_kernel<G, MINB, MODE>, (int)budget, dev);
    }
    // spread the groups evenly over the SMs: sources are FP64-pipe bound per SM, so an SM holding two blocks while
    // another holds one would take twice as long.  Full occupancy = sms * bps blocks; fewer slots than that get
    // fewer groups per block, not fewer blocks.
    int sms = 1, bps = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (L.warpsPerSM > 0) L.nSlots = (int)std::min<long long>(L.nSlots, std::max<long long>(1, (long long)sms * L.warpsPerSM / G));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, geodesic_kernel<G, MINB, MODE>, 32 * G * gpb, smem);
    bps = std::max(bps, 1);
    const long long full = (long long)sms * bps;
    int blocks;
    if ((long long)L.nSlots >= full * gpb) {
        blocks = (L.nSlots + gpb - 1) / gpb;
    } else {
        gpb = (int)((L.nSlots + full - 1) / full);  // groups per block; groups past nSlots return at once
        if (L.smemTables) smem = per * gpb;
        blocks = (int)full;
    }
    geodesic_kernel<G, MINB, MODE><<<blocks, 32 * G * gpb, smem, s>>>(L);
}

}  // namespace

#ifdef CSSG_GEO_OUTLINE
void cssg_launch_geodesic_outlined(GeoLaunch L, cudaStream_t s)
#else
void cssg_launch_geodesic(GeoLaunch L, cudaStream_t s)
#endif
{
#ifndef CSSG_GEO_OUTLINE
    if (L.hashOutline) {
        cssg_launch_geodesic_outlined(L, s);
        return;
    }
#endif
    // patch systems with 1 or 2 warps per source: the version with the search mode fixed
    if (L.patchSystems && L.groupWarps <= 2) {
        if (L.wideRegs) {
            if (L.groupWarps == 2) launch_groups<2, 1, 1>(L, s);
            else launch_groups<1, 1, 1>(L, s);
        } else {
            if (L.groupWarps == 2) launch_groups<2, 2, 1>(L, s);
            else launch_groups<1, 2, 1>(L, s);
        }
        return;
    }
    if (L.wideRegs) {
        if (L.groupWarps == 8) launch_groups<8, 1>(L, s);
        else if (L.groupWarps == 4) launch_groups<4, 1>(L, s);
        else if (L.groupWarps == 2) launch_groups<2, 1>(L, s);
        else launch_groups<1, 1>(L, s);
    } else {
        if (L.groupWarps == 8) launch_groups<8, 2>(L, s);
        else if (L.groupWarps == 4) launch_groups<4, 2>(L, s);
        else if (L.groupWarps == 2) launch_groups<2, 2>(L, s);
        else launch_groups<1, 2>(L, s);
    }
}

#ifndef CSSG_GEO_OUTLINE
GeoSizing cssg_geo_sizing(const cssg_mesh* mesh, int maxTargets, int submesh, double max_dist, double cutoff)
{
    GeoSizing z;
    long long est;
    double reach = cutoff;
    if (submesh && max_dist < reach) reach = max_dist;
    if (reach < 1e30) {
        double r = reach + mesh->meanEdge;
        est = (long long)(1.3 * 3.14159265 * r * r / mesh->meanFaceArea) + 32;
    } else {
        est = mesh->d.nF;
    }
    if (est > mesh->d.nF) est = mesh->d.nF;
    long long estV = std::min<long long>(mesh->d.nV, est / 2 + 4 * (long long)std::sqrt((double)est) + 16);
    GeoCaps& caps = z.caps;
    caps.CT = std::max(32, maxTargets);
    // whole mesh: the face table holds only target faces; patch: the patch plus the goal faces
    caps.CF = submesh ? next_pow2(2 * (est + caps.CT) + 64) : next_pow2(2 * caps.CT + 64);
    caps.CV = next_pow2(2 * estV + 64);
    caps.CW = (int)std::min<long long>(1 << 22, 16 * est + 1024);
    caps.CL = (int)std::min<long long>(1 << 20, 2 * estV + 256);
    caps.CLOG = (int)std::min<long long>(1 << 22, 32 * (long long)caps.CT + 16 * est + 1024);
    z.est = est;
    z.maxWindows = (int)std::min<long long>(1 << 30, 400 * est + 100000);
    return z;
}

// --------------------------------------------------------------------------------------------------------------------
// C ABI: batched distance queries (per-source API of triangulatedMeshSpace::distance)
// --------------------------------------------------------------------------------------------------------------------
extern "C" int cssg_distance_batch(cssg_ctx* ctx, const cssg_mesh* mesh, int nSrc, const int* src_face,
                                   const double* src_bary, const int* cand_offsets, const int* cand_face,
                                   const double* cand_bary, int submesh, double max_dist, const double* threshold,
                                   double cutoff, double* d_out, double* tstart_out, double* tend_out, int* status,
                                   long long* stats)
{
    if (!ctx || !mesh || nSrc < 0 || (nSrc > 0 && (!src_face || !src_bary || !cand_offsets || !d_out || !status))) {
        cssg_set_error("cssg_distance_batch: bad arguments");
        return CSSG_ERR_ARG;
    }
    if (nSrc == 0) return CSSG_OK;
    DeviceScope scope(ctx->device);
    CSSG_CUDA(scope.err);
    cudaStream_t s = ctx->stream;
    // size the per-warp tables: targets = the largest candidate list, the rest from the domain size
    int* dmax = nullptr;
    CSSG_CUDA(cudaMallocAsync((void**)&dmax, sizeof(int), s));
    max_count_kernel<<<1, 1024, 0, s>>>(nSrc, cand_offsets, dmax);
    int hmax = 0;
    CSSG_CUDA(cudaMemcpyAsync(&hmax, dmax, sizeof(int), cudaMemcpyDeviceToHost, s));
    CSSG_CUDA(cudaStreamSynchronize(s));
    CSSG_CUDA(cudaFreeAsync(dmax, s));
    const GeoSizing z = cssg_geo_sizing(mesh, hmax, submesh, max_dist, cutoff);
    size_t slotBytes = cssg_geo_slot_bytes(z.caps);
    int dev = ctx->device;
    int sms = 0;
    CSSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    size_t freeB = 0, totalB = 0;
    CSSG_CUDA(cudaMemGetInfo(&freeB, &totalB));
    long long nSlots = std::min<long long>((long long)sms * 16, nSrc);
    long long fit = (long long)(freeB / 4 / slotBytes);
    if (nSlots > fit) nSlots = std::max<long long>(1, fit);
    void* scratch = nullptr;
    int* work = nullptr;
    CSSG_CUDA(cudaMallocAsync(&scratch, slotBytes * nSlots, s));
    CSSG_CUDA(cudaMallocAsync((void**)&work, sizeof(int), s));
    CSSG_CUDA(cudaMemsetAsync(work, 0, sizeof(int), s));
    cssg_geo_init_scratch(scratch, slotBytes, (int)nSlots, z.caps, s);
    SysDesc hd;
    memset(&hd, 0, sizeof(hd));
    hd.mesh = mesh->d;
    hd.searchMode = 0;
    hd.submesh = submesh;
    hd.maxDist = max_dist;
    hd.cutoff = cutoff;
    SysDesc* dsys = nullptr;
    CSSG_CUDA(cudaMallocAsync((void**)&dsys, sizeof(SysDesc), s));
    CSSG_CUDA(cudaMemcpyAsync(dsys, &hd, sizeof(SysDesc), cudaMemcpyHostToDevice, s));
    GeoLaunch L;
    memset(&L, 0, sizeof(L));
    L.sys = dsys;
    L.nSrc = nSrc;
    L.srcFace = src_face;
    L.srcBary = src_bary;
    L.candOff = cand_offsets;
    L.candFace = cand_face;
    L.candBary = cand_bary;
    L.threshold = threshold;
    L.stats = stats;
    L.dOut = d_out;
    L.tsOut = tstart_out;
    L.teOut = tend_out;
    L.status = status;
    L.patchDisconnected = (submesh && !(cutoff < 1e300)) ? 1 : 0;
    L.delta = mesh->meanEdge;
    L.maxRounds = 1 << 16;
    L.maxWindows = z.maxWindows;
    L.caps = z.caps;
    L.scratch = scratch;
    L.slotBytes = slotBytes;
    L.nSlots = (int)nSlots;
    L.workCounter = work;
    L.device = dev;
    cssg_launch_geodesic(L, s);
    CSSG_CUDA(cudaGetLastError());
    CSSG_CUDA(cudaFreeAsync(dsys, s));
    CSSG_CUDA(cudaFreeAsync(scratch, s));
    CSSG_CUDA(cudaFreeAsync(work, s));
    return CSSG_OK;
}
#endif  // CSSG_GEO_OUTLINE
