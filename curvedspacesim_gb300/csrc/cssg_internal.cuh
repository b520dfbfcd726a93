// Internal declarations shared by the translation units of libcssg.so.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>

#include "../../include/cssg.h"

// Device-resident mesh (structure of arrays).  Local edge k of face f runs F[3f+k] -> F[3f+(k+1)%3].
struct DevMesh {
    int nV, nF;
    const double* V;            // 3 nV vertex positions
    const int* F;               // 3 nF vertex indices (counter-clockwise)
    const int* twin;            // 3 nF: face*3 + local edge of the neighbour across local edge k, -1 on a border
    const double* N;            // 3 nF unit face normals
    const double* geom;         // 9 nF: [9f + 3k + 0] edge length, [+1],[+2] third vertex in the edge frame
    const double* exitu;        // 12 nF: entering through edge k, unit directions of the exit edges C->A and B->C in
                                //        the edge-k frame: [12f + 4k + 0..1] (C - A)/|C - A|, [+2..3] (B - C)/|B - C|
    const int* vfStart;         // nV + 1: vertex -> incident faces (CSR)
    const int* vfList;
    const int* ringStart;       // nV + 1: clockwise neighbour ring of closed vertices (throughVertex order)
    const int* ringV;
    const unsigned char* vflag; // bit0 closed ring available, bit1 border vertex, bit2 saddle (angle sum > 2 pi)
    const float* fcurv;         // 3 nF: per face mean curvature, Gaussian curvature, mean edge length (screen features)
    double bbMin[3], bbMax[3];
    int bc;                     // walk boundary condition: 0 closed, 1 tangential, 2 absorbing (open meshes)
};

enum { VF_RING = 1, VF_BORDER = 2, VF_SADDLE = 4 };
enum { BC_CLOSED = 0, BC_TANGENTIAL = 1, BC_ABSORBING = 2 };

struct cssg_mesh {
    DevMesh d;
    DevMesh* dself;  // device copy of d (kernels that serve several meshes index arrays of DevMesh)
    int device;
    double area;
    double meanEdge;
    double meanFaceArea;
    void* buffers[14];
};

struct cssg_ctx {
    int device;
    cudaStream_t stream;
    bool ownStream;
};

// Reciprocal by Newton-Raphson iteration r <- r (2 - d r) (two fused multiply-adds per step) seeded with the
// single-precision reciprocal: the relative error squares each step (2^-23 -> 2^-46 -> below double rounding), so
// two steps give 1/d within a few ulps (not correctly rounded).  Cheaper on the FP64 pipe than an IEEE double
// division; used for geometric denominators.  Outside the float range it falls back to the division.
__device__ __forceinline__ double rcp_nr(double d)
{
    const double a = fabs(d);
    if (!(a > 1e-30 && a < 1e30)) return 1.0 / d;
    double r = (double)__frcp_rn((float)d);
    double e = fma(-d, r, 1.0);
    r = fma(r, e, r);
    e = fma(-d, r, 1.0);
    return fma(r, e, r);
}

// Makes `device` current for the lifetime of the object and restores the caller's device afterwards, so an entry
// point that receives a context works on the context's device whatever device the calling thread had selected.
struct DeviceScope {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceScope(int device)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != device) err = cudaSetDevice(device);
    }
    ~DeviceScope()
    {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;
};

// Raises a kernel's dynamic shared-memory limit to `bytes` once on each device: the limit is a per-device attribute
// of the function, so a process that uses several devices must set it on each.  Bit d of `mask` records device d
// (devices past 63 set it on every call).
template <class Kernel>
inline cudaError_t cssg_raise_smem_once(std::atomic<unsigned long long>& mask, Kernel* kernel, int bytes, int device)
{
    const unsigned long long bit = device >= 0 && device < 64 ? 1ull << device : 0ull;
    if (bit && (mask.load() & bit)) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) mask.fetch_or(bit);
    return e;
}

// error plumbing
void cssg_set_error(const std::string& msg);
int cssg_cuda_fail(cudaError_t e, const char* what);
// records "<fn>: bad arguments" as the last error and returns CSSG_ERR_ARG
int cssg_bad_args(const char* fn);
#define CSSG_CUDA(call)                                      \
    do {                                                     \
        cudaError_t e__ = (call);                            \
        if (e__ != cudaSuccess) return cssg_cuda_fail(e__, #call); \
    } while (0)

// ---- walk (walk.cu) ----------------------------------------------------------------------------------------------
// Launches the batched transport kernel; pos_out (nullable) receives the final R3 positions, crossings (nullable)
// accumulates the launch's crossings.
// meshes: device array of meshes; meshOf (nullable): per-particle index into it (null: all on meshes[0])
// kick_force (nullable): velocity-Verlet first half folded into the walk, from the velocity in transport vector 0:
// disp = dt v + dt^2 f / 2, v += dt f / 2 (velocityVerletNVE.cpp:14-21).  status_bits (nullable): OR of
// (1 << status) over the walks that failed.
void cssg_launch_transport(const DevMesh* meshes, const int* meshOf, int n, int* face, double* bary, double* disp,
                           double* transport, int nT, int* status, unsigned long long* crossings, double* pos_out,
                           cudaStream_t s, const int* skip = nullptr, int* status_bits = nullptr,
                           const double* kick_force = nullptr, double kick_dt = 0.0, const int* skip_sys = nullptr);
void cssg_launch_positions(const DevMesh* meshes, const int* meshOf, int n, const int* face, const double* bary,
                           double* pos, cudaStream_t s);

// ---- geodesics (geodesic.cu) -------------------------------------------------------------------------------------
struct GeoCaps {
    int CT;    // targets per source
    int CV;    // vertex hash capacity (power of two)
    int CF;    // face hash capacity (power of two)
    int CW;    // windows per frontier buffer
    int CL;    // launch list entries per buffer
    int CLOG;  // target-face window log entries
};

// One independent system (mesh + interaction parameters + its slice of the particle and cell arrays).  A launch
// serves any number of them: sources carry their system index.
struct SysDesc {
    DevMesh mesh;
    int searchMode;   // 0 CSR candidate lists (distance API), 1 cell list, 2 all-to-all,
                      // 3 CSR of candidate particle indices with screen flags (learned-screen path)
    int bigBin;       // patches too large for the regular tables: sources go straight to the large-table pass
    int submesh;      // reference patches
    int forceKind;    // 0 harmonic, 1 gaussian
    int partBase;     // first particle of this system
    int nPart;
    int cellBase;     // first cell of this system's grid in the shared cell arrays
    int nc[3];
    double cs[3];
    double lo[3];
    double range2;    // candidate test: chord^2 < range2
    double maxDist;   // patch radius cap
    double cutoff;    // paths longer than this are not followed
    double k, sigma;  // force parameters
    double delta;     // band width of the propagation rounds for this system's mesh (0: the launch's value)
};

// Per-launch configuration of the fused neighbour / geodesic / force kernel.
struct GeoLaunch {
    const SysDesc* sys;          // device array of systems
    const int* sysOf;            // nullable: system of each particle (null: all in sys[0])
    // sources
    int nSrc;
    const int* srcFace;
    const double* srcBary;
    const double* srcPos;        // nullable: R3 positions of the sources (system mode)
    const int* order;            // nullable: processing order of the sources (cell order)
    // targets: CSR mode (distance API) ...
    const int* candOff;
    const int* candFace;
    const double* candBary;
    const double* threshold;     // nullable (CSR modes): per-source patch radius
    const int* candJ;            // mode 3: candidate particle index per CSR entry
    const unsigned char* candSkip;  // mode 3: 1 = screened out (its face still completes the patch, not queried)
    // padded candidate rows of the cell-list search (one-source-per-lane kernel, mode 1): row si holds rowCount[si]
    // particle indices at rowJ[si * rowCap], rowChord[si] = the largest candidate chord
    const int* rowJ;
    const int* rowCount;
    const double* rowChord;
    int rowCap;
    // ... or neighbour search (system mode): all particles + the shared cell arrays
    const int* partFace;
    const double* partBary;
    const double* partPos;
    const int* cellStart;        // totalCells + 1
    const int* cellList;         // particle indices sorted by cell (stable)
    // outputs
    double* dOut;                // per candidate (CSR mode) or per pair slot (system mode, nullable)
    double* tsOut;
    double* teOut;
    int* pairJ;                  // system mode pair output: target particle index (nullable)
    int* pairCount;              // system mode: candidates per source (nullable)
    int* inRangeOut;             // nullable: per source, pairs with d <= sigma (the screen's audit compares them)
    int pairCap;                 // system mode: pair slots per source
    double* force;               // system mode: force per source (nullable)
    int* status;                 // per source
    int* statusBits;             // nullable: OR of (1 << status) over the sources whose final status is an error
    double* kickVel;             // nullable: velocity-Verlet second half kick v += 0.5 dt f where the force is written
    double kickDt;
    long long* stats;            // nullable: per source {windows processed, launches, rounds, targets}
    unsigned long long* counters;  // [0] windows processed, [1] vertex launches, [2] in-range pairs, [3] capacity hits
    int patchDisconnected;       // CSR mode with cutoff = inf: unreached -> 2*maxDist, tangent (0,0,1)
    double delta;                // band width of the distance-ordered rounds
    int maxRounds;               // per-source caps: exceeding either reports CSSG_ST_CAPACITY
    int maxWindows;
    // scratch
    GeoCaps caps;
    void* scratch;
    size_t slotBytes;
    int nSlots;                  // warps with a slot
    int* workCounter;            // persistent-warp work queue
    const int* itemCountDev;     // nullable: number of work items read from the device (retry pass)
    int* failList;               // nullable: sources whose tables overflowed are queued here for a retry pass
    int* failCount;
    int routeBig;                // 1: sources of systems marked bigBin go straight to failList (first pass only)
    double deltaScale;           // band width = deltaScale * the system's delta (<= 0: 1)
    int wpbMax;                  // largest warps per block (CTA size / 32; <= 0: 8)
    int warpsPerSM;              // > 0: at most this many source warps per SM (the rest of the slots stay idle)
    int groupWarps;              // warps that solve one source together: 1 (default), 2, 4 or 8
    int wideRegs;                // 1: the kernel build with up to 255 registers per thread (fewer warps per SM)
    int hashOutline;             // 1: the kernel build with out-of-line hash-table probes (geodesic_outlined.cu)
    int patchSystems;            // 1: every system takes reference patches and cell-list or screened candidates
    int* srcCost;                // nullable: work of each source (windows + launches + rounds), for the next order
    int smemTables;              // set by cssg_launch_geodesic: hash tables in shared memory
    int device;                  // the CUDA device the launch runs on (SM count, occupancy, attributes)
};

// Table capacities and the per-source work cap of a batched distance call (cssg_distance_batch and
// cssg_distance_batch_noalloc share this rule, so both run the same kernels with the same tables): targets = the
// largest candidate list, the rest from the number of faces within reach of a source (patch radius or cutoff), or the
// whole mesh.  est receives that face estimate.
struct GeoSizing {
    GeoCaps caps;
    long long est;
    int maxWindows;
};
GeoSizing cssg_geo_sizing(const cssg_mesh* mesh, int maxTargets, int submesh, double max_dist, double cutoff);

size_t cssg_geo_slot_bytes(const GeoCaps& c);
// shared memory one warp's hash tables need (tables go to global scratch when this exceeds the block budget)
size_t cssg_geo_smem_per_warp(const GeoCaps& c);
// Fills slots with their initial (empty) state; call once after allocating the scratch.
void cssg_geo_init_scratch(void* scratch, size_t slotBytes, int nSlots, const GeoCaps& c, cudaStream_t s);
void cssg_launch_geodesic(GeoLaunch L, cudaStream_t s);
// the same kernels built with out-of-line hash-table probes (geodesic_outlined.cu); cssg_launch_geodesic calls it
// when L.hashOutline is set
void cssg_launch_geodesic_outlined(GeoLaunch L, cudaStream_t s);
// ---- one source per lane (lanes.cu) ----------------------------------------------------------------------------------
// Per-lane table capacities: targets, face table and vertex table (powers of two), window slab.
struct LaneCaps {
    int CT, CF, CV, CW;
};
size_t cssg_lane_warp_bytes(const LaneCaps& c);
// The regular propagation pass with one source per lane: L.nSlots warps, each with cssg_lane_warp_bytes(C) of
// scratch at L.scratch; a warp takes `lanes` (16 or 32) sources at a time.  Sources that overflow go to L.failList.
void cssg_launch_lanes(const GeoLaunch& L, const LaneCaps& C, int lanes, cudaStream_t s);

// candidate lists for the learned-screen path: per source (warp) the cell-list candidates in reference order,
// padded rows of `cap` entries; count[i] (> cap: overflow) and the largest candidate chord maxChord[i]
void cssg_launch_candidates(const GeoLaunch& L, int n, int cap, int* candJ, int* count, double* maxChord,
                            cudaStream_t s);

// ---- learned screen (mlp.cu) ---------------------------------------------------------------------------------------
// features + tensor-core MLP + decision for nPairs CSR pairs (pi -> pj): skip[p] = 1 when the predicted distance
// |chord| + sigma * yhat exceeds sigma * (1 + margin).  X (nPairs x 16 BF16), chord, yhat are caller scratch.
// maxPairs bounds the launch; the actual count is read from nPairsDev on the device
// disable (nullable, device int): when set, every pair is kept (the audit's fallback to the exact path)
void cssg_launch_screen(const SysDesc* sys, const int* sysOf, int maxPairs, const int* nPairsDev, const int* pi,
                        const int* pj, const int* face, const double* pos, void* X, float* chord, const float* params,
                        float* yhat, unsigned char* skip, double margin, int* errFlag, int sms, cudaStream_t s,
                        const int* disable = nullptr);
